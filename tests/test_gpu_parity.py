"""GPU parity of the CUDA path against the oracle (CPU restatement of NuTo), through the C ABI.

Tolerances: CSR pattern and DOF numbering bit-exact; FP64 residual and FP64 tangent values <= 1e-12 relative to
the largest entry; FP32 tangent values <= 2e-6 relative to the largest entry; displacements of converged
load steps <= 1e-8 (FP64 path) and <= 1e-6 (FP32 tangent / FP32 Krylov path) relative to the largest
displacement.
"""

import json
import os

import numpy as np
import pytest
import scipy.sparse as sp

import oracle
from oracle import setups as osetups
from oracle.quasistatic import QuasistaticOracle

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
FP64_REL = 1e-12
FP32_REL = 2e-6


def _torch():
    import torch

    assert torch.cuda.is_available(), "these tests need a CUDA GPU"
    return torch


def _build(kind, n):
    from nuto_gb300 import configs

    if kind == "quad4":
        s = configs.quad4_elastic(n)
        o = osetups.quad4_elastic(n)
    elif kind == "hex8gd":
        s = configs.hex8_gradient_damage(n)
        o = osetups.hex8_gradient_damage(n)
    elif kind == "quad4gd":
        s = configs.notched_plate(n, 0.4)
        o = osetups.notched_plate(n, 0.4)
    else:
        s = configs.hex20_local_damage(n)
        o = osetups.hex20_local_damage(n)
    g = s.build_gpu()
    return s, g, o


def _state(P, rng, scale):
    u = rng.uniform(-1.0, 1.0, P.n_dofs) * scale
    return u


def _oracle_csr(P, u):
    K = P.build_matrix_scipy(u).tocsr()
    K.sort_indices()
    return K


CASES = [("quad4", 5), ("hex8gd", 3), ("hex20", 2), ("quad4gd", 8)]


@pytest.mark.parametrize("kind,n", CASES)
def test_pattern_bit_exact(kind, n):
    _torch()
    s, g, (om, layers, P, cons) = _build(kind, n)
    rp, ci = g.pattern()
    cp, ri, _ = P.build_matrix_csc(np.zeros(P.n_dofs))
    assert g.n_dofs == P.n_dofs
    assert np.array_equal(rp, cp)
    assert np.array_equal(ci, ri)


def _damage_state(kind, P, rng):
    if kind in ("hex8gd", "quad4gd"):
        u = _state(P, rng, 2e-4)
        nd = (3 if kind == "hex8gd" else 2) * P.mesh.layer_num_nodes(0)
        u[nd:] = rng.uniform(0.0, 4e-4, P.n_dofs - nd)  # eeq around and above kappa0
        kappa = rng.uniform(0.0, 3e-4, (P.n_el, P.n_ip))
    elif kind == "hex20":
        u = _state(P, rng, 3e-4)
        kappa = rng.uniform(0.0, 3e-4, (P.n_el, P.n_ip))
    else:
        u = _state(P, rng, 1e-3)
        kappa = None
    return u, kappa


@pytest.mark.parametrize("kind,n", CASES)
def test_build_vector_fp64(kind, n):
    torch = _torch()
    s, g, (om, layers, P, cons) = _build(kind, n)
    rng = np.random.default_rng(7)
    u, kappa = _damage_state(kind, P, rng)
    if kappa is not None:
        P.kappa = kappa
        g.history = kappa
    f_ref = P.build_vector(u)
    f = g.build_vector(u).cpu().numpy()
    assert np.abs(f - f_ref).max() <= FP64_REL * np.abs(f_ref).max()
    torch.cuda.synchronize()


@pytest.mark.parametrize("kind,n", CASES)
@pytest.mark.parametrize("precision", [64, 32])
def test_build_matrix(kind, n, precision):
    torch = _torch()
    s, g, (om, layers, P, cons) = _build(kind, n)
    rng = np.random.default_rng(11)
    u, kappa = _damage_state(kind, P, rng)
    if kappa is not None:
        P.kappa = kappa
        g.history = kappa
    K = _oracle_csr(P, u)
    v = g.build_matrix(u, precision).double().cpu().numpy()
    rp, ci = g.pattern()
    assert np.array_equal(rp, K.indptr) and np.array_equal(ci, K.indices)
    tol = FP64_REL if precision == 64 else FP32_REL
    assert np.abs(v - K.data).max() <= tol * np.abs(K.data).max()
    torch.cuda.synchronize()


def test_brick8n_golden_on_gpu():
    """applications/integrationtests/mechanics/results/Brick8N*.txt through the GPU kernels."""
    _torch()
    from nuto_gb300 import mesh as M
    from nuto_gb300._lib import MB_LINEAR_ELASTIC

    gold = json.load(open(os.path.join(HERE, "golden", "brick8n.json")))
    st = gold["setup"]
    m = M.MeshFem(3, M.HEX8, np.array(st["coords"], float), np.arange(8)[None, :])
    d = M.add_dof_interpolation(m, 3)
    from nuto_gb300 import GpuCellGroup

    g = GpuCellGroup(m, [d], 2)
    g.build_pattern()
    g.set_integrand(kind=MB_LINEAR_ELASTIC, dim=3, E=st["E"], nu=st["nu"])
    u = np.zeros(24)
    for nd in st["displaced_nodes"]:
        u[3 * nd:3 * nd + 3] = st["displacement"]
    f = g.build_vector(u).cpu().numpy()
    v = g.build_matrix(u, 64).cpu().numpy()
    rp, ci = g.pattern()
    K = sp.csr_matrix((v, ci, rp), shape=(24, 24)).toarray()
    Kg = np.array(gold["K_e"])
    fg = np.array(gold["f_e"])
    assert np.abs(K - Kg).max() <= 1e-11 * np.abs(Kg).max()
    assert np.abs(f - fg).max() <= 1e-11 * np.abs(fg).max()


def test_cell_scatter_known_answer():
    """test/mechanics/cell/SimpleAssembler.cpp:57-114 idea: two cells sharing DOFs, caller-given cell results."""
    _torch()
    from nuto_gb300 import GpuCellGroup
    from nuto_gb300 import mesh as M

    m = M.create_quads(2, 1)
    d = M.add_dof_interpolation(m, 1)
    g = GpuCellGroup(m, [d], 2)
    n, nnz = g.build_pattern()
    conn = m.layers[d].conn
    fe = np.array([[11.0, 22.0, 33.0, 44.0], [11.0, 22.0, 33.0, 44.0]])
    f = g.assemble_cell_vectors(fe).cpu().numpy()
    ref = np.zeros(n)
    for c in range(2):
        np.add.at(ref, conn[c], fe[c])
    assert np.array_equal(f, ref)
    ke = np.array([[[10 * i + j for j in range(1, 5)] for i in range(1, 5)]] * 2, dtype=float)
    v = g.assemble_cell_matrices(ke).cpu().numpy()
    rp, ci = g.pattern()
    K = sp.csr_matrix((v, ci, rp), shape=(n, n)).toarray()
    Kref = np.zeros((n, n))
    for c in range(2):
        Kref[np.ix_(conn[c], conn[c])] += ke[c]
    assert np.array_equal(K, Kref)
    assert nnz == 4 * 4 * 2 - 4  # shared edge: 2 x 2 entries counted once


@pytest.mark.parametrize("kind,n", [("hex8gd", 3), ("hex20", 2), ("quad4gd", 8)])
def test_update_history(kind, n):
    _torch()
    s, g, (om, layers, P, cons) = _build(kind, n)
    rng = np.random.default_rng(5)
    u, kappa = _damage_state(kind, P, rng)
    P.kappa = kappa
    g.history = kappa
    P.update_history(u)
    g.update_history(u)
    assert np.abs(g.history - P.kappa).max() <= 1e-15 + 1e-13 * np.abs(P.kappa).max()


@pytest.mark.parametrize("method,precond", [(1, 1), (1, 2), (2, 1), (3, 1), (3, 2)])
@pytest.mark.parametrize("precision", [64, 32])
def test_linear_solve_quad4(precision, method, precond):
    """PCG (1), BiCGStab (2) and GMRES (3) with the Jacobi (1) or multigrid (2) preconditioner against a direct
    solve of the reduced system C^T K C."""
    _torch()
    s, g, (om, layers, P, cons) = _build("quad4", 12)
    g.set_preconditioner(precond)
    u0 = np.zeros(P.n_dofs)
    K = _oracle_csr(P, u0)
    vals = g.build_matrix(u0, precision)
    rng = np.random.default_rng(3)
    b = rng.uniform(-1, 1, P.n_dofs)
    dep = cons[0]
    indep = np.setdiff1d(np.arange(P.n_dofs), dep)
    x, it, rel, ok = g.solve(vals, b, precision=precision, method=method, rtol=1e-10)
    assert ok, (it, rel)
    import scipy.sparse.linalg as spla

    # FP32 values: the FP64 refinement converges to the solution of the FP32 operator the GPU assembled (removing
    # the rounding of the tangent itself is the job of Newton with the FP64 residual)
    rp, ci = g.pattern()
    Kp = sp.csr_matrix((vals.double().cpu().numpy(), ci, rp), shape=K.shape) if precision == 32 else K
    y = spla.spsolve(Kp[indep][:, indep].tocsc(), b[indep])
    xr = np.zeros(P.n_dofs)
    xr[indep] = y
    xg = x.cpu().numpy()
    assert np.abs(xg[dep]).max() == 0.0
    assert np.abs(xg - xr).max() <= 1e-8 * np.abs(xr).max()


def _run_steps(kind, n, precision, steps, t_end, tol=1e-10):
    s, g, (om, layers, P, cons) = _build(kind, n)
    Q = QuasistaticOracle(P, cons[0], cons[1], cons[2], tolerance=tol, max_iterations=20)
    g.set_state(None, 0.0, True)
    opts = g.default_options(precision=precision, newton_rtol=0.0, newton_atol=tol,
                             krylov_rtol=1e-12 if precision == 64 else 1e-5, max_newton=30, max_krylov=50000)
    out = []
    for k in range(1, steps + 1):
        t = t_end * k / steps
        Q.do_step(t)
        g.do_step(t, opts)
        x, tg = g.get_state()
        out.append((Q.x.copy(), x.copy(), Q.P.kappa.copy(), g.history.copy(), g.stats()))
        assert tg == t
    return out


@pytest.mark.parametrize("precision", [64, 32])
def test_quasistatic_quad4_elastic(precision):
    _torch()
    res = _run_steps("quad4", 10, precision, 1, 1.0, tol=1e-11)
    xo, xg, _, _, st = res[-1]
    rel = np.abs(xg - xo).max() / np.abs(xo).max()
    assert rel <= (1e-8 if precision == 64 else 1e-6), (rel, st)


def test_gmres_nonsymmetric_gradient_damage_tangent():
    """Multigrid-preconditioned GMRES on the non-symmetric gradient-damage tangent in the damaged regime, FP64 and
    FP32 values (Jacobi-preconditioned GMRES stagnates on this matrix: the eeq rows depend on the strain about 15
    times more strongly than on their own diagonal)."""
    _torch()
    s, g, (om, layers, P, cons) = _build("hex8gd", 3)
    g.set_preconditioner(2)
    rng = np.random.default_rng(2)
    # a consistent damaged state: eight load steps of the oracle's Newton (damage grows from step 4)
    Q = QuasistaticOracle(P, cons[0], cons[1], cons[2], tolerance=1e-10, max_iterations=20)
    for k in range(1, 9):
        Q.do_step(0.05 * k)
    u = Q.x.copy()
    kappa = P.kappa.copy()
    assert kappa.max() > 2e-4
    g.history = kappa
    K = _oracle_csr(P, u)
    b = rng.uniform(-1, 1, P.n_dofs)
    dep = cons[0]
    indep = np.setdiff1d(np.arange(P.n_dofs), dep)
    import scipy.sparse.linalg as spla

    for precision in (64, 32):
        vals = g.build_matrix(u, precision)
        x, it, rel, ok = g.solve(vals, b, precision=precision, method=3, rtol=1e-9, max_iterations=5000)
        assert ok, (precision, it, rel)
        rp, ci = g.pattern()
        Kp = sp.csr_matrix((vals.double().cpu().numpy(), ci, rp), shape=K.shape)
        y = spla.spsolve(Kp[indep][:, indep].tocsc(), b[indep])
        xg = x.cpu().numpy()
        assert np.abs(xg[indep] - y).max() <= 1e-6 * np.abs(y).max(), precision


@pytest.mark.parametrize("precision", [64, 32])
def test_quasistatic_hex8_gradient_damage(precision):
    """Eight load steps of the gradient-damage beam (damage starts after step 4); displacement, eeq and the
    kappa history follow the oracle's direct-solve Newton."""
    _torch()
    res = _run_steps("hex8gd", 3, precision, 8, 0.4, tol=1e-12)
    for k, (xo, xg, ko, kg, st) in enumerate(res):
        rel = np.abs(xg - xo).max() / np.abs(xo).max()
        # the Newton tolerance (1e-12 on |C^T r|) bounds the eeq components only to ~1e-10 absolute, because the
        # eeq rows scale with the cell volume; hence 1e-7 relative for the FP64 path
        assert rel <= (1e-7 if precision == 64 else 1e-6), (k, rel, st)
        assert np.abs(kg - ko).max() <= (1e-7 if precision == 64 else 1e-6) * max(np.abs(ko).max(), 1e-4)
    assert res[-1][2].max() > 1e-4  # the last steps are in the damaged regime


@pytest.mark.parametrize("precision", [64, 32])
def test_quasistatic_notched_plate(precision):
    """Eight load steps of one notched plate (2D plane-strain gradient damage, damage from step 4): displacement,
    eeq and kappa follow the oracle's direct-solve Newton."""
    _torch()
    res = _run_steps("quad4gd", 8, precision, 8, 0.8, tol=1e-12)
    for k, (xo, xg, ko, kg, st) in enumerate(res):
        rel = np.abs(xg - xo).max() / np.abs(xo).max()
        assert rel <= (1e-7 if precision == 64 else 1e-6), (k, rel, st)
        assert np.abs(kg - ko).max() <= (1e-7 if precision == 64 else 1e-6) * max(np.abs(ko).max(), 1e-4)
    assert res[-1][2].max() > 1e-4


@pytest.mark.parametrize("precision", [64, 32])
def test_batched_plates_match_separate_oracle_solves(precision):
    """Three notched plates of different sizes solved as one batch on the GPU (one cell group, block-diagonal
    system, absolute Newton tolerance on the combined |C^T r|) against the oracle solving each plate alone: every
    plate's displacement, eeq and kappa within 1e-7 (FP64) / 1e-6 (FP32 tangent) after six load steps."""
    _torch()
    from nuto_gb300 import batch, configs

    specs = [(6, 0.25), (10, 0.5), (8, 0.4)]
    b = batch.concatenate([configs.notched_plate(n, d) for n, d in specs])
    g = b.build_gpu()
    g.set_state(None, 0.0, True)
    opts = g.default_options(precision=precision, newton_rtol=0.0, newton_atol=1e-12,
                             krylov_rtol=1e-12 if precision == 64 else 1e-5, max_newton=30, max_krylov=50000)
    alone = []
    for n, d in specs:
        _, _, Pi, ci = osetups.notched_plate(n, d)
        alone.append((Pi, QuasistaticOracle(Pi, ci[0], ci[1], ci[2], tolerance=1e-12, max_iterations=20)))
    for k in range(1, 7):
        g.do_step(0.1 * k, opts)
        for Pi, Qi in alone:
            Qi.do_step(0.1 * k)
    x, _ = g.get_state()
    tol = 1e-7 if precision == 64 else 1e-6
    for (Pi, Qi), xs, ks in zip(alone, b.split_state(x), b.split_history(g.history)):
        assert np.abs(xs - Qi.x).max() <= tol * np.abs(Qi.x).max()
        assert np.abs(ks - Pi.kappa).max() <= tol * np.abs(Pi.kappa).max()
        assert Pi.kappa.max() > 1e-4


def test_exact_final_phase_within_1e6_of_converged_solution():
    """FP32 tangent with the exact final phase (exact_tangent_below = 1e4, the default): at the benchmark's relative
    Newton tolerance 1e-8, eight load steps into the damaged regime end within 1e-6 (relative, max norm) of the
    oracle's direct-solve Newton converged to 1e-12, as the FP64 path does."""
    _torch()
    res = {}
    for name, prec, ex in (("fp64", 64, 0.0), ("exact", 32, 1.0e4)):
        s, g, (om, layers, P, cons) = _build("hex8gd", 6)
        Q = QuasistaticOracle(P, cons[0], cons[1], cons[2], tolerance=1e-12, max_iterations=30)
        g.set_state(None, 0.0, True)
        opts = g.default_options(precision=prec, newton_rtol=1e-8, krylov_rtol=1e-3, max_newton=30,
                                 max_krylov=50000, exact_tangent_below=ex)
        for k in range(1, 9):
            t = 0.05 * k
            Q.do_step(t)
            g.do_step(t, opts)
        x, _ = g.get_state()
        res[name] = np.abs(x - Q.x).max() / np.abs(Q.x).max()
        assert P.kappa.max() > 1e-4  # damaged regime
    assert res["fp64"] <= 1e-6, res
    assert res["exact"] <= 1e-6, res


@pytest.mark.parametrize("kind,n,steps", [("hex8gd", 8, 0), ("hex8gd", 8, 6), ("hex20", 4, 0), ("quad4", 40, 0)])
def test_multigrid_levels_solve(kind, n, steps):
    """Multigrid-preconditioned solves on meshes large enough for several levels: GMRES (FP64 and FP32 values)
    on the gradient-damage tangent, undamaged and after damaging load steps of the oracle, and PCG on the
    symmetric Hex20 and Quad4 tangents, each against a direct solve; the multigrid solve needs fewer iterations
    than the Jacobi one."""
    _torch()
    import scipy.sparse.linalg as spla

    s, g, (om, layers, P, cons) = _build(kind, n)
    u = np.zeros(P.n_dofs)
    if steps:
        Q = QuasistaticOracle(P, cons[0], cons[1], cons[2], tolerance=1e-10, max_iterations=20)
        for k in range(1, steps + 1):
            Q.do_step(0.05 * k)
        u = Q.x.copy()
        g.history = P.kappa.copy()
    dep = cons[0]
    indep = np.setdiff1d(np.arange(P.n_dofs), dep)
    b = np.random.default_rng(5).uniform(-1, 1, P.n_dofs)
    rp, ci = g.pattern()
    for precision in (64, 32):
        vals = g.build_matrix(u, precision)
        its = {}
        for precond in (2, 1):
            g.set_preconditioner(precond)
            x, it, rel, ok = g.solve(vals, b, precision=precision, method=0, rtol=1e-9, max_iterations=20000)
            if precond == 1 and not ok:
                its[1] = np.inf  # Jacobi may stall on the damaged tangent; the multigrid solve must not
                continue
            assert ok, (precision, precond, it, rel)
            its[precond] = it
            Kp = sp.csr_matrix((vals.double().cpu().numpy(), ci, rp), shape=(P.n_dofs, P.n_dofs))
            y = spla.spsolve(Kp[indep][:, indep].tocsc(), b[indep])
            xg = x.cpu().numpy()
            assert np.abs(xg[indep] - y).max() <= 1e-6 * np.abs(y).max(), (precision, precond)
        assert its[2] < its[1], its


@pytest.mark.parametrize("kind,n", [("quad4", 5), ("hex8gd", 3), ("hex20", 2), ("quad4gd", 8)])
@pytest.mark.parametrize("precision", [32])
def test_tangent_row_gather_matches_element_atomics(kind, n, precision, monkeypatch):
    """The FP32 row-gather tangent (records + one warp per node row) and the element-wise atomic tangent give the
    same CSR values on a damaged state (rounding-level differences only: the summation order differs). FP64 always
    uses the element kernel."""
    _torch()
    rng = np.random.default_rng(11)
    s, g, (om, layers, P, cons) = _build(kind, n)
    u, kappa = _damage_state(kind, P, rng)
    if kappa is not None:
        g.history = kappa
    rows = g.build_matrix(u, precision).double().cpu().numpy()
    monkeypatch.setenv("NUTO_GPU_TANGENT", "atomic")
    s2, g2, _ = _build(kind, n)
    if kappa is not None:
        g2.history = kappa
    atom = g2.build_matrix(u, precision).double().cpu().numpy()
    tol = 1e-13 if precision == 64 else 2e-6
    assert np.abs(rows - atom).max() <= tol * np.abs(atom).max()


@pytest.mark.parametrize("precision", [64, 32])
def test_multigrid_sweep_graph_matches_kernel_launches(precision, monkeypatch):
    """The multigrid sweep replayed as a CUDA graph and launched kernel by kernel (NUTO_GPU_GRAPHS=0) give the same
    GMRES solution (up to the order of the atomic restriction sums) and iteration count within one restart; the
    context reports which form ran (the graph must run on the stream the tests use, the legacy default stream)."""
    _torch()
    from nuto_gb300 import configs

    rng = np.random.default_rng(12)
    b = None
    out = {}
    for graphs in ("1", "0"):
        monkeypatch.setenv("NUTO_GPU_GRAPHS", graphs)
        s, g, (om, layers, P, cons) = _build("hex8gd", 8)
        if b is None:
            # a well-posed damaged tangent: elastic displacements and the two pre-damaged middle layers
            u = _state(P, rng, 1e-6)
            u[3 * P.mesh.layer_num_nodes(0):] = 0.0
            kappa = configs.gradient_damage_imperfection(8, g.n_ip)
            b = rng.uniform(-1, 1, P.n_dofs)
        g.history = kappa
        vals = g.build_matrix(u, precision)
        x, it, rel, ok = g.solve(vals, b, precision=precision, method=3, rtol=1e-8, max_iterations=5000)
        assert ok, (graphs, it, rel)
        levels, graph_active = g.multigrid_info()
        assert levels >= 2 and graph_active == int(graphs), (levels, graph_active)
        out[graphs] = (x.cpu().numpy(), it)
    (x1, it1), (x0, it0) = out["1"], out["0"]
    assert np.abs(x1 - x0).max() <= 1e-5 * np.abs(x0).max()
    assert abs(it1 - it0) <= 40


@pytest.mark.parametrize("kind,n", CASES + [("hex8gd", 8)])
def test_fp64x_tangent_matches_fp64(kind, n):
    """The exact final phase's tangent (FP64 law, node-pair products in double-float FP32 arithmetic) against the
    plain FP64 tangent, in a damaged state: <= 1e-13 relative to max |K| (Hex20 uses the FP64 products: equal)."""
    torch = _torch()
    s, g, (om, layers, P, cons) = _build(kind, n)
    rng = np.random.default_rng(41)
    u = _state(P, rng, 2e-3)
    if g.kind != 0:  # damage laws: a history above kappa0 so that the damage terms are active
        g.history = np.full((g.mesh.num_cells, g.n_ip), 1.5e-4)
    k64 = g.build_matrix(u, 64).cpu().numpy()
    k65 = g.build_matrix(u, 65).cpu().numpy()
    assert np.abs(k65 - k64).max() <= 1e-13 * np.abs(k64).max(), np.abs(k65 - k64).max() / np.abs(k64).max()
    torch.cuda.synchronize()


@pytest.mark.parametrize("kind,n", CASES + [("hex8gd", 8)])
def test_spmv_padded_layout(kind, n):
    """y = K x through nuto_gpu_spmv (the padded-pair-layout product of the solvers) against the CSR product on the
    host: FP64 values 1e-13, FP32 values with FP64 accumulation 1e-13 and with compensated FP32 sums 1e-12, relative
    to max |K| |x|."""
    torch = _torch()
    s, g, (om, layers, P, cons) = _build(kind, n)
    rng = np.random.default_rng(31)
    u = _state(P, rng, 1e-4)
    x = rng.uniform(-1, 1, P.n_dofs)
    rp, ci = g.pattern()
    for precision, comp, tol in ((64, False, 1e-13), (32, False, 1e-13), (32, True, 1e-12)):
        vals = g.build_matrix(u, precision)
        K = sp.csr_matrix((vals.double().cpu().numpy(), ci, rp), shape=(P.n_dofs, P.n_dofs))
        y = g.spmv(vals, x, precision=precision, compensated=comp).cpu().numpy()
        ref = K @ x
        scale = (abs(K) @ np.abs(x)).max()
        assert np.abs(y - ref).max() <= tol * scale, (precision, comp, np.abs(y - ref).max() / scale)
    torch.cuda.synchronize()


@pytest.mark.parametrize("kind,n", CASES)
def test_lumped_mass(kind, n):
    """BuildDiagonallyLumpedMatrix of DynamicMomentumBalance::Hessian2 on the GPU against the oracle (FP64)."""
    _torch()
    s, g, (om, layers, P, cons) = _build(kind, n)
    ref = P.lumped_mass(2.5)
    m = g.lumped_mass(2.5).cpu().numpy()
    assert np.abs(m - ref).max() <= FP64_REL * np.abs(ref).max()


@pytest.mark.parametrize("kind,n", [("quad4", 5), ("hex8gd", 3), ("hex20", 2), ("quad4gd", 8)])
def test_eval_ip(kind, n):
    """Cell::Eval post-processing values (kappa, damage, strain, stress, equivalent strain) against the oracle."""
    _torch()
    from oracle import core

    rng = np.random.default_rng(17)
    s, g, (om, layers, P, cons) = _build(kind, n)
    u, kappa = _damage_state(kind, P, rng)
    if kappa is not None:
        P.kappa = kappa
        g.history = kappa
    for q in (core.IP_KAPPA, core.IP_DAMAGE, core.IP_STRAIN, core.IP_STRESS, core.IP_EEQ):
        ref = P.eval_ip(u, q)
        got = g.eval_ip(u, q).cpu().numpy()
        assert got.shape == ref.shape, q
        assert np.abs(got - ref).max() <= FP64_REL * max(np.abs(ref).max(), 1e-300), q


@pytest.mark.parametrize("kind", ["quad4", "hex8gd"])
def test_external_load(kind):
    """NeumannBc::ExternalLoad over boundary cells (Line2 edges / Quad4 faces) on the GPU against the oracle."""
    _torch()
    from nuto_gb300 import mesh as M
    from oracle import core

    s, g, (om, layers, P, cons) = _build(kind, 4 if kind == "quad4" else 3)
    m = s.mesh
    d = s.layers[0]
    if kind == "quad4":
        fc, fd = M.boundary_faces(m, d, 0, 1.0)
        p = np.array([0.7, -0.2])
    else:
        fc, fd = M.boundary_faces(m, d, 2, 4.0)
        p = np.array([0.1, 0.2, -1.3])
    grp = g.add_boundary_cells(fc, fd, gauss=2)
    f = g.external_load(grp, p).cpu().numpy()
    L = m.layers[d]
    omesh = core.Mesh.from_arrays(m.dim, m.geo_interp, m.coords, m.conn)
    ref = omesh.external_load(g.n_dofs, fc, L.dof_numbers[fd], p, gauss=2)
    assert np.abs(f - ref).max() <= FP64_REL * np.abs(ref).max()


def test_force_driven_patch():
    """Force-driven patch test (PatchTest.cpp:93-327 in spirit): a plane-strain square pulled by a uniform traction
    p on its right edge, x fixed on the left edge and y at the origin; the bilinear cells reproduce the analytic
    field u_x = (1 - nu^2) p x / E, u_y = -nu (1 + nu) p y / E exactly. The load enters nuto_gpu_do_step as the
    constant gradient -f_ext."""
    _torch()
    import nuto_gb300
    from nuto_gb300 import configs
    from nuto_gb300 import mesh as M

    m = M.create_quads(4, 4)
    d = M.add_dof_interpolation(m, 2)
    left = M.nodes_at_axis(m, d, 0, 0.0)
    origin = [n for n in left if abs(m.layers[d].node_coords[n, 1]) < 1e-12]
    cons = configs._merge(M.component_constraints(m, d, left, [0]), M.component_constraints(m, d, origin, [1]))
    E, nu, p = 30000.0, 0.2, 3.0
    integ = dict(kind=nuto_gb300.MB_LINEAR_ELASTIC, dim=2, E=E, nu=nu, plane_state=nuto_gb300._lib.PLANE_STRAIN,
                 disp_slot=0)
    s = configs.Setup("patch", m, [d], 2, integ, [cons])
    g = s.build_gpu()
    fc, fd = M.boundary_faces(m, d, 0, 1.0)
    grp = g.add_boundary_cells(fc, fd, gauss=2)
    fext = g.external_load(grp, [p, 0.0])
    g.set_constant_gradient(-fext)
    g.set_state(None, 0.0, True)
    g.do_step(1.0, g.default_options(precision=64, newton_rtol=0.0, newton_atol=1e-12, krylov_rtol=1e-13))
    x, _ = g.get_state()
    X = m.layers[d].node_coords
    ux = (1 - nu ** 2) * p * X[:, 0] / E
    uy = -nu * (1 + nu) * p * X[:, 1] / E
    u = x.reshape(-1, 2)
    assert np.abs(u[:, 0] - ux).max() <= 1e-9 * np.abs(ux).max()
    assert np.abs(u[:, 1] - uy).max() <= 1e-9 * np.abs(ux).max()
