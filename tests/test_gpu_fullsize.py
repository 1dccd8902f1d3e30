"""The path at the configurations' full sizes.

C0 (Quad4 200 x 200, plane-strain elasticity, 80,802 DOFs) is compared with the oracle entry by entry: CSR pattern
bit-exact, FP64 tangent and residual <= 1e-12 relative to the largest entry, FP32 tangent <= 2e-6, and the
displacements of the load step <= 1e-8 relative to the oracle's direct solve.

C4 (Hex20 on 80^3 cells, 6,318,243 DOFs, 1,086,410,889 nonzeros) is too large for the oracle, so it is checked
through size-independent properties of the elastic state: the DOF and nonzero counts of the structured mesh, a
symmetric tangent (y.Kx = x.Ky), rigid translations in the null space of the unconstrained tangent and residual,
linearity of the residual, f_int(u) = K u, and FP32 values within 2e-6 of the FP64 ones.
"""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _torch():
    import torch

    assert torch.cuda.is_available(), "these tests need a CUDA GPU"
    return torch


def test_c0_quad4_200_full_size_against_oracle():
    torch = _torch()
    import nuto_gb300
    from nuto_gb300 import configs
    from oracle import setups
    from oracle.quasistatic import QuasistaticOracle

    n = 200
    s = configs.quad4_elastic(n)
    g = s.build_gpu()
    om, layers, P, cons = setups.quad4_elastic(n)
    assert g.n_dofs == 80802 and g.nnz == 4 * 601 ** 2
    rng = np.random.default_rng(20)
    u = rng.uniform(-1e-3, 1e-3, P.n_dofs)
    K = P.build_matrix_scipy(u).tocsr()
    K.sort_indices()
    rp, ci = g.pattern()
    assert np.array_equal(rp, K.indptr) and np.array_equal(ci, K.indices)
    k64 = g.build_matrix(u, nuto_gb300.FP64).cpu().numpy()
    assert np.abs(k64 - K.data).max() <= 1e-12 * np.abs(K.data).max()
    k32 = g.build_matrix(u, nuto_gb300.FP32).double().cpu().numpy()
    assert np.abs(k32 - K.data).max() <= 2e-6 * np.abs(K.data).max()
    f_ref = P.build_vector(u)
    f = g.build_vector(u).cpu().numpy()
    assert np.abs(f - f_ref).max() <= 1e-12 * np.abs(f_ref).max()
    # the load step of C0: one BuildMatrix + BuildVector + solve (the trial state of QuasistaticSolver::DoStep)
    Q = QuasistaticOracle(P, cons[0], cons[1], cons[2], tolerance=1e-11, max_iterations=6)
    Q.do_step(1.0)
    g.set_state(None, 0.0, True)
    g.do_step(1.0, g.default_options(precision=nuto_gb300.FP64, newton_rtol=0.0, newton_atol=1e-11,
                                     krylov_rtol=1e-12, max_krylov=50000))
    x, _ = g.get_state()
    assert np.abs(x - Q.x).max() <= 1e-8 * np.abs(Q.x).max()
    torch.cuda.synchronize()


def test_c4_hex20_80_full_size_properties():
    torch = _torch()
    import nuto_gb300
    from nuto_gb300 import configs

    n = 80
    s = configs.hex20_local_damage(n)
    g = s.build_gpu()
    assert g.n_dofs == 6318243
    assert g.nnz == 9 * (234 * n ** 3 + 141 * n ** 2 + 24 * n + 1)
    dev = torch.device("cuda")
    rp, ci = g.pattern()
    crow = torch.as_tensor(rp, device=dev)
    col = torch.as_tensor(ci, device=dev).to(torch.int64)
    del rp, ci
    rng = np.random.default_rng(21)
    nd = g.n_dofs

    def csr(vals):
        return torch.sparse_csr_tensor(crow, col, vals, size=(nd, nd))

    u0 = torch.zeros(nd, dtype=torch.float64, device=dev)
    k64 = g.build_matrix(u0, nuto_gb300.FP64)
    A = csr(k64)
    absrow = torch.sparse_csr_tensor(crow, col, k64.abs(), size=(nd, nd)) @ torch.ones(nd, dtype=torch.float64,
                                                                                          device=dev)
    scale = float(absrow.max())
    # symmetry of the elastic tangent
    x = torch.as_tensor(rng.uniform(-1, 1, nd), device=dev)
    y = torch.as_tensor(rng.uniform(-1, 1, nd), device=dev)
    yKx = float(torch.dot(y, A @ x))
    xKy = float(torch.dot(x, A @ y))
    assert abs(yKx - xKy) <= 1e-12 * scale * nd
    # rigid translations: no force, in the null space of the unconstrained tangent
    for comp in range(3):
        t = torch.zeros(nd, dtype=torch.float64, device=dev)
        t[comp::3] = 1.0
        assert float((A @ t).abs().max()) <= 1e-11 * scale
        assert float(g.build_vector(t * 1e-3).abs().max()) <= 1e-11 * scale * 1e-3
    # elastic state (strains ~1e-7, far below the damage threshold kappa0 = 1e-4 on cells of edge 1/80):
    # f_int linear in u and equal to K u
    u = torch.as_tensor(rng.uniform(-1e-9, 1e-9, nd), device=dev)
    f1 = g.build_vector(u)
    f2 = g.build_vector(2.0 * u)
    fs = float(f1.abs().max())
    assert float((f2 - 2.0 * f1).abs().max()) <= 1e-12 * fs * 100
    assert float((A @ u - f1).abs().max()) <= 1e-11 * fs
    # FP32 values
    del A
    k32 = g.build_matrix(u0, nuto_gb300.FP32)
    assert float((k32.double() - k64).abs().max()) <= 2e-6 * float(k64.abs().max())
    torch.cuda.synchronize()
