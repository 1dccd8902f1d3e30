"""GPU parity of the tangent kernels beyond the basic cases, through the C ABI.

- The fused FP32 tangent (geometry and law recomputed per node in FP32, no integration-point records) against the
  records + row-gather tangent and against the FP64 tangent, including states whose integration points sit on the
  law's branch thresholds (eeq = kappa_h, eeq = kappa0): the loading/unloading and damage branches of the FP32
  kernel must be the FP64 kernels' at every point, otherwise whole coupling blocks differ.
- GradientDamage with NonlocalInteraction::Decreasing and with UNILATERAL damage application
  (nuto/mechanics/integrands/GradientDamage.h:153-184, nuto/mechanics/constitutive/LinearElasticDamage.h:58-100)
  against the oracle: FP64 residual and tangent <= 1e-12, FP32 tangent <= 2e-6 relative to the largest entry, and
  load steps into the damaged range.
- The benchmark beam (64^3 Hex8 gradient damage) at its full size: DOF numbering and CSR pattern bit-exact and the
  FP64 residual <= 1e-12 against the oracle at the benchmark's seeded state; tangent values at 32^3.
"""

import numpy as np
import pytest

import bench
from oracle import setups as osetups
from oracle.quasistatic import QuasistaticOracle

pytestmark = pytest.mark.gpu

FP64_REL = 1e-12
FP32_REL = 2e-6


def _torch():
    import torch

    assert torch.cuda.is_available(), "these tests need a CUDA GPU"
    return torch


def _setup(kind, n, law=None):
    from nuto_gb300 import configs

    if kind == "hex8gd":
        s = configs.hex8_gradient_damage(n)
        o = osetups.hex8_gradient_damage(n, law=law)
    elif kind == "quad4gd":
        s = configs.notched_plate(n, 0.4)
        o = osetups.notched_plate(n, 0.4, law=law)
    else:
        s = configs.quad4_elastic(n)
        o = osetups.quad4_elastic(n)
    if law:
        s.integrand.update(law)
    return s, o


def _damage_state(kind, s, P, rng):
    u = rng.uniform(-2e-4, 2e-4, P.n_dofs)
    if kind == "quad4":
        return u * 5.0, None
    nd = s.mesh.layers[s.layers[0]].num_dofs
    u[nd:] = rng.uniform(0.0, 4e-4, P.n_dofs - nd)
    kappa = rng.uniform(0.0, 3e-4, (P.n_el, P.n_ip))
    return u, kappa


def _csr(P, u):
    K = P.build_matrix_scipy(u).tocsr()
    K.sort_indices()
    return K


@pytest.mark.parametrize("kind,n", [("hex8gd", 4), ("quad4gd", 8), ("quad4", 5)])
def test_fused_tangent_matches_records_and_oracle(kind, n, monkeypatch):
    _torch()
    import nuto_gb300

    rng = np.random.default_rng(21)
    s, (om, layers, P, cons) = _setup(kind, n)
    u, kappa = _damage_state(kind, s, P, rng)
    g = s.build_gpu()
    if kappa is not None:
        g.history = kappa
        P.kappa = kappa
    fused = g.build_matrix(u, nuto_gb300.FP32).double().cpu().numpy()
    monkeypatch.setenv("NUTO_GPU_TANGENT", "records")
    g2 = s.build_gpu()
    if kappa is not None:
        g2.history = kappa
    rec = g2.build_matrix(u, nuto_gb300.FP32).double().cpu().numpy()
    K = _csr(P, u)
    scale = np.abs(K.data).max()
    assert np.abs(fused - K.data).max() <= FP32_REL * scale
    assert np.abs(fused - rec).max() <= FP32_REL * scale


def test_fused_tangent_branches_follow_fp64_at_the_thresholds():
    """Integration points placed exactly on the thresholds: history kappa equal to the point's eeq (as after a
    history update at a loading point), slightly above and below it, and nodal eeq equal to kappa0. The FP32 tangent
    stays within FP32 rounding of the FP64 tangent, which decides these branches in FP64."""
    _torch()
    import nuto_gb300
    from nuto_gb300._lib import IP_EEQ

    n = 4
    s, (om, layers, P, cons) = _setup("hex8gd", n)
    g = s.build_gpu()
    rng = np.random.default_rng(5)
    nd = s.mesh.layers[s.layers[0]].num_dofs
    u = rng.uniform(-1e-4, 1e-4, P.n_dofs)
    u[nd:] = rng.uniform(0.5e-4, 2e-4, P.n_dofs - nd)
    # a third of the eeq nodes exactly at kappa0
    e_idx = np.arange(nd, P.n_dofs)
    u[e_idx[::3]] = 1e-4
    g.history = 0.0
    eeq = g.eval_ip(u, IP_EEQ).cpu().numpy()[..., 0]  # FP64 eeq at every point
    choice = rng.integers(0, 4, eeq.shape)
    kappa = np.where(choice == 0, eeq, np.where(choice == 1, np.nextafter(eeq, np.inf),
                                                np.where(choice == 2, np.nextafter(eeq, -np.inf), 1e-4)))
    g.history = kappa
    k32 = g.build_matrix(u, nuto_gb300.FP32).double().cpu().numpy()
    k64 = g.build_matrix(u, nuto_gb300.FP64).cpu().numpy()
    assert np.abs(k32 - k64).max() <= FP32_REL * np.abs(k64).max()


VARIANTS = {"decreasing": dict(interaction=1, R=0.005, eta=5.0),
            "unilateral": dict(damage_application=1),
            "decreasing_unilateral": dict(interaction=1, R=0.05, eta=3.0, damage_application=1)}


@pytest.mark.parametrize("variant", sorted(VARIANTS))
@pytest.mark.parametrize("kind,n", [("hex8gd", 3), ("quad4gd", 8)])
def test_gradient_damage_variants_against_oracle(kind, n, variant):
    _torch()
    import nuto_gb300

    law = VARIANTS[variant]
    s, (om, layers, P, cons) = _setup(kind, n, law)
    g = s.build_gpu()
    rng = np.random.default_rng(31)
    u, kappa = _damage_state(kind, s, P, rng)
    g.history = kappa
    P.kappa = kappa
    f_ref = P.build_vector(u)
    f = g.build_vector(u).cpu().numpy()
    assert np.abs(f - f_ref).max() <= FP64_REL * np.abs(f_ref).max()
    K = _csr(P, u)
    scale = np.abs(K.data).max()
    k64 = g.build_matrix(u, nuto_gb300.FP64).cpu().numpy()
    assert np.abs(k64 - K.data).max() <= FP64_REL * scale
    k32 = g.build_matrix(u, nuto_gb300.FP32).double().cpu().numpy()
    assert np.abs(k32 - K.data).max() <= FP32_REL * scale


@pytest.mark.parametrize("precision", [64, 32])
@pytest.mark.parametrize("variant", ["decreasing", "unilateral"])
def test_gradient_damage_variant_load_steps(variant, precision):
    """Eight load steps of the notched plate into the damaged range with the variant's law; displacements, eeq and
    kappa against the oracle's direct-solve Newton (FP64 path <= 1e-7, FP32 tangent <= 1e-6 relative; the Newton
    tolerance 1e-12 on |C^T r| bounds the eeq unknowns only to about 1e-10 absolute)."""
    _torch()
    law = VARIANTS[variant]
    s, (om, layers, P, cons) = _setup("quad4gd", 8, law)
    g = s.build_gpu()
    tol = 1e-12
    Q = QuasistaticOracle(P, cons[0], cons[1], cons[2], tolerance=tol, max_iterations=30)
    g.set_state(None, 0.0, True)
    opts = g.default_options(precision=precision, newton_rtol=0.0, newton_atol=tol,
                             krylov_rtol=1e-12 if precision == 64 else 1e-5, max_newton=30, max_krylov=50000)
    rel = 1e-7 if precision == 64 else 1e-6
    steps = 8
    for k in range(1, steps + 1):
        t = 0.8 * k / steps  # the schedule of the plain notched-plate test: damage from step 4 on
        Q.do_step(t)
        g.do_step(t, opts)
        x, _ = g.get_state()
        assert np.abs(x - Q.x).max() <= rel * np.abs(Q.x).max(), k
        kap = g.history
        assert np.abs(kap - Q.P.kappa).max() <= rel * max(np.abs(Q.P.kappa).max(), 1e-4), k
    assert Q.P.kappa.max() > 1e-4  # the steps reached the damaged range


def test_benchmark_beam_full_size_pattern_and_residual():
    """The 64^3 beam of the benchmark (1,098,500 DOFs): numbering and CSR pattern bit for bit, FP64 residual at the
    benchmark's seeded state within 1e-12 of the oracle's."""
    _torch()
    from nuto_gb300 import configs

    n = 64
    s = configs.hex8_gradient_damage(n)
    g = s.build_gpu()
    Ld, Le = s.mesh.layers[s.layers[0]], s.mesh.layers[s.layers[1]]
    x, kappa = bench.beam_state(Ld.node_coords, Ld.dof_numbers, Le.dof_numbers, g.n_dofs, s.mesh.num_cells, g.n_ip,
                                n)
    P, xo = bench.oracle_beam(n)
    assert np.array_equal(x, xo) and g.n_dofs == P.n_dofs == 1098500
    rp, ci = g.pattern()
    cp, ri, _ = P.build_matrix_csc(np.zeros(P.n_dofs))
    assert np.array_equal(rp, cp) and np.array_equal(ci, ri)
    del cp, ri
    g.history = kappa
    f = g.build_vector(x).cpu().numpy()
    f_ref = P.build_vector(x)
    assert np.abs(f - f_ref).max() <= FP64_REL * np.abs(f_ref).max()


def test_beam_32_tangent_against_oracle():
    """The beam at 32^3 (143,748 DOFs, 13.6 M nonzeros) at the benchmark's kind of seeded state: FP64 tangent <= 1e-12
    and the FP32 (fused) tangent <= 2e-6 relative to the largest entry."""
    _torch()
    import nuto_gb300
    from nuto_gb300 import configs

    n = 32
    s = configs.hex8_gradient_damage(n)
    g = s.build_gpu()
    P, x = bench.oracle_beam(n)
    g.history = P.kappa
    K = _csr(P, x)
    scale = np.abs(K.data).max()
    k64 = g.build_matrix(x, nuto_gb300.FP64).cpu().numpy()
    assert np.abs(k64 - K.data).max() <= FP64_REL * scale
    k32 = g.build_matrix(x, nuto_gb300.FP32).double().cpu().numpy()
    assert np.abs(k32 - K.data).max() <= FP32_REL * scale


@pytest.mark.parametrize("kind,n", [("hex8gd", 6), ("quad4gd", 12)])
def test_fp64_residual_is_bitwise_reproducible(kind, n):
    """The FP64 residual sums the cell vectors per DOF in a fixed cell order: repeated evaluations of the same state
    are equal bit for bit (and equal the oracle's to 1e-12)."""
    _torch()
    s, (om, layers, P, cons) = _setup(kind, n)
    g = s.build_gpu()
    rng = np.random.default_rng(41)
    u, kappa = _damage_state(kind, s, P, rng)
    g.history = kappa
    first = g.build_vector(u).cpu().numpy()
    for _ in range(3):
        assert np.array_equal(g.build_vector(u).cpu().numpy(), first)
    P.kappa = kappa
    f_ref = P.build_vector(u)
    assert np.abs(first - f_ref).max() <= FP64_REL * np.abs(f_ref).max()


def test_fused_fp32_tangent_is_bitwise_reproducible():
    """The fused tangent adds the cells around a node in a fixed order (no atomics): repeated assemblies of the same
    state are equal bit for bit."""
    _torch()
    import nuto_gb300

    s, (om, layers, P, cons) = _setup("hex8gd", 6)
    g = s.build_gpu()
    rng = np.random.default_rng(43)
    u, kappa = _damage_state("hex8gd", s, P, rng)
    g.history = kappa
    first = g.build_matrix(u, nuto_gb300.FP32).cpu().numpy()
    for _ in range(3):
        assert np.array_equal(g.build_matrix(u, nuto_gb300.FP32).cpu().numpy(), first)


@pytest.mark.parametrize("kind,n", [("hex8gd", 5), ("quad4gd", 8), ("quad4", 5)])
def test_staged_and_fused_tangents_agree(kind, n, monkeypatch):
    """The default FP32 tangent (per-point records computed once, staged per node warp) and the fused variant
    (NUTO_GPU_TANGENT=fused: geometry and law recomputed in every node warp) evaluate the same FP32 expressions: the
    values agree to FP32 rounding."""
    _torch()
    import nuto_gb300

    rng = np.random.default_rng(51)
    s, (om, layers, P, cons) = _setup(kind, n)
    u, kappa = _damage_state(kind, s, P, rng)
    g = s.build_gpu()
    if kappa is not None:
        g.history = kappa
    staged = g.build_matrix(u, nuto_gb300.FP32).double().cpu().numpy()
    monkeypatch.setenv("NUTO_GPU_TANGENT", "fused")
    g2 = s.build_gpu()
    if kappa is not None:
        g2.history = kappa
    fused = g2.build_matrix(u, nuto_gb300.FP32).double().cpu().numpy()
    assert np.abs(staged - fused).max() <= 1e-6 * np.abs(fused).max()


def test_autotuner_picks_measured_shapes_without_changing_results(monkeypatch):
    """The autotuner times the tangent's node-row kernel with 2, 4 and 8 warps per block and the fine-level product
    with 4, 8 and 16 lanes per node and keeps the fastest; the tangent is bitwise the same for every block shape (each
    node's rows are summed by one warp in a fixed order), and a solve with the tuned product matches the default's."""
    _torch()
    import nuto_gb300

    s, (om, layers, P, cons) = _setup("hex8gd", 6)
    rng = np.random.default_rng(61)
    u, kappa = _damage_state("hex8gd", s, P, rng)
    b = rng.uniform(-1.0, 1.0, P.n_dofs)
    res = {}
    for tune in ("1", "0"):
        monkeypatch.setenv("NUTO_GPU_AUTOTUNE", tune)
        g = s.build_gpu()
        g.history = kappa
        k32 = g.build_matrix(u, nuto_gb300.FP32).cpu().numpy()  # damaged state: every branch of the law
        # the solve on the undamaged tangent (a damaged random state need not be solvable)
        g.history = 0.0
        k_el = g.build_matrix(np.zeros(P.n_dofs), nuto_gb300.FP32)
        x, it, rel, ok = g.solve(k_el, b, precision=nuto_gb300.FP32, method=3, rtol=1e-6, max_iterations=5000)
        assert ok, (tune, it, rel)
        res[tune] = (k32, x.cpu().numpy(), g.autotune_info())
    info = res["1"][2]
    assert info["tangent_warps"] in (2, 4, 8) and min(info["tangent_ms"]) > 0
    assert info["spmv_lanes"]["f32/f32"] in (4, 8, 16)
    assert res["0"][2]["tangent_warps"] == 4 and res["0"][2]["spmv_lanes"]["f32/f32"] == 0
    assert np.array_equal(res["1"][0], res["0"][0])
    xs = res["0"][1]
    assert np.abs(res["1"][1] - xs).max() <= 1e-4 * np.abs(xs).max()


@pytest.mark.parametrize("kind,n", [("hex8gd", 6), ("quad4gd", 12)])
def test_pipelined_node_rows_bitwise_equal(kind, n, monkeypatch):
    """The double-buffered node-row kernel (NUTO_GPU_TANGENT=pipelined: a grid of resident blocks walking the nodes,
    the next pass's records copied while the current one is integrated) adds the same blocks in the same order as the
    one-node-per-warp kernel: the tangents are equal bit for bit."""
    _torch()
    import nuto_gb300

    rng = np.random.default_rng(71)
    s, (om, layers, P, cons) = _setup(kind, n)
    u, kappa = _damage_state(kind, s, P, rng)
    monkeypatch.setenv("NUTO_GPU_AUTOTUNE", "0")
    g = s.build_gpu()
    g.history = kappa
    plain = g.build_matrix(u, nuto_gb300.FP32).cpu().numpy()
    monkeypatch.setenv("NUTO_GPU_TANGENT", "pipelined")
    g2 = s.build_gpu()
    g2.history = kappa
    piped = g2.build_matrix(u, nuto_gb300.FP32).cpu().numpy()
    assert g2.autotune_info()["tangent_pipelined"]
    assert np.array_equal(piped, plain)


@pytest.mark.parametrize("kind,n", [("hex8gd", 6), ("quad4gd", 12), ("quad4", 10)])
@pytest.mark.parametrize("records", ["0", "1"])
def test_cell_matrix_tangent_bitwise_equal(kind, n, records, monkeypatch):
    """The element-matrix form (NUTO_GPU_TANGENT=cells: every node-pair block integrated once into the cell's element
    matrix, then one warp per node adds the slabs of its cells in ascending cell order) forms each block with the
    node-row kernel's expressions and adds the blocks in the same order: the tangents are equal bit for bit, and both
    match the oracle at the FP32 tolerance. With the law evaluated in the cell kernel (default) and from the point
    records (NUTO_GPU_CELLS_RECORDS=1)."""
    _torch()
    import nuto_gb300

    monkeypatch.setenv("NUTO_GPU_CELLS_RECORDS", records)
    rng = np.random.default_rng(72)
    s, (om, layers, P, cons) = _setup(kind, n)
    u, kappa = _damage_state(kind, s, P, rng)
    monkeypatch.setenv("NUTO_GPU_AUTOTUNE", "0")
    g = s.build_gpu()
    if kappa is not None:
        g.history = kappa
        P.kappa = kappa
    plain = g.build_matrix(u, nuto_gb300.FP32).cpu().numpy()
    monkeypatch.setenv("NUTO_GPU_TANGENT", "cells")
    g2 = s.build_gpu()
    if kappa is not None:
        g2.history = kappa
    cells = g2.build_matrix(u, nuto_gb300.FP32).cpu().numpy()
    assert g2.autotune_info()["tangent_form"] == "cell_matrices"
    K = _csr(P, u)
    assert np.abs(cells - K.data).max() <= FP32_REL * np.abs(K.data).max()
    assert np.array_equal(cells, plain)


@pytest.mark.parametrize("kind,n", [("hex8gd", 8), ("quad4gd", 16), ("quad4", 12)])
@pytest.mark.parametrize("precision", [32, 64])
@pytest.mark.parametrize("res_blocks", ["2", "1"])
def test_build_system_equals_separate_calls(kind, n, precision, res_blocks, monkeypatch):
    """nuto_gpu_build_system (the residual on a second stream, a persistent grid of a few blocks per SM beside the
    tangent) gives the values of nuto_gpu_build_matrix and nuto_gpu_build_vector: on its first call (run in
    sequence) and on the later, concurrent ones, on two states in turn. Bitwise, except the FP64 tangent, whose
    element kernel adds with FP64 atomics (order-dependent rounding)."""
    torch = _torch()
    monkeypatch.setenv("NUTO_GPU_SYSTEM_RES_BLOCKS", res_blocks)
    s, o = _setup(kind, n)
    g = s.build_gpu()
    P = o[2]
    rng = np.random.default_rng(4)
    states = [_damage_state(kind, s, P, rng) for _ in range(2)]
    for k in range(4):
        u, kappa = states[k % 2]
        if kappa is not None:
            g.history = kappa
        v, f = g.build_system(u, precision)
        v2 = g.build_matrix(u, precision)
        f2 = g.build_vector(u)
        torch.cuda.synchronize()
        if precision == 32:
            assert torch.equal(v, v2), k
        else:
            assert float((v - v2).abs().max()) <= 1e-13 * float(v2.abs().max()), k
        assert torch.equal(f, f2), k


@pytest.mark.parametrize("pinned", [True, False])
def test_build_system_host_equals_device_call(pinned):
    """nuto_gpu_build_system_host (state in from host memory, values and residual back to host memory, the values'
    copy overlapping the residual) returns bitwise what nuto_gpu_build_system leaves on the device, on its first
    (sequential) call and later ones, from page-locked and from pageable host buffers."""
    torch = _torch()
    import nuto_gb300

    s, o = _setup("hex8gd", 8)
    g = s.build_gpu()
    P = o[2]
    rng = np.random.default_rng(5)
    for k in range(3):
        u, kappa = _damage_state("hex8gd", s, P, rng)
        g.history = kappa
        v_dev, f_dev = g.build_system(u, nuto_gb300.FP32)
        uh = torch.as_tensor(u).pin_memory() if pinned else torch.as_tensor(u)
        vh = torch.empty(g.nnz, dtype=torch.float32, pin_memory=pinned)
        fh = torch.empty(g.n_dofs, dtype=torch.float64, pin_memory=pinned)
        g.build_system_host(uh, vh, fh, nuto_gb300.FP32)
        assert torch.equal(vh, v_dev.cpu()), k
        assert torch.equal(fh, f_dev.cpu()), k
