"""The FP32 tangent of Hex20 cells on the tensor cores (k_tangent_tc20: tcgen05.mma kind::tf32 into tensor memory),
through the C ABI.

SimpleAssembler::BuildMatrix (nuto/mechanics/cell/SimpleAssembler.cpp:100-156) of MomentumBalance::Hessian0
(nuto/mechanics/integrands/MomentumBalance.h:36-46) with LocalIsotropicDamage (nuto/mechanics/constitutive/
LocalIsotropicDamage.h:59-68, 115-122) and LinearElastic on InterpolationBrickQuadratic cells:

- the default three-product split (hi.hi + hi.lo + lo.hi) against the oracle at the FP32 tangent's tolerance,
  2e-6 of the largest entry, on meshes where every block handles one cell (2^3) and several cells (6^3);
- against the records + row-gather FP32 tangent (NUTO_GPU_TC20=off) and bitwise equal between two calls;
- the one-product variant (NUTO_GPU_TC20=tf32): its error against the oracle is measured and stays far above the
  FP32 kernels' (which is why it is not the default) but below 2e-3;
- the bounded wait on the MMA completion barrier: with the spin limit at 0 every wait gives up, the kernel drains
  its MMAs and returns, synchronize() raises NUTO_GPU_ETIMEOUT, and the next call (default limit) is correct.
"""

import numpy as np
import pytest

from oracle import core as ocore
from oracle import setups as osetups

pytestmark = pytest.mark.gpu

FP32_REL = 2e-6


def _torch():
    import torch

    assert torch.cuda.is_available(), "these tests need a CUDA GPU"
    return torch


def _case(n, kind, seed=11):
    from nuto_gb300 import _lib, configs

    s = configs.hex20_local_damage(n)
    m, layers, P, cons = osetups.hex20_local_damage(n)
    rng = np.random.default_rng(seed)
    u = rng.uniform(-3e-4, 3e-4, P.n_dofs)
    kappa = None
    if kind == "elastic":
        s.integrand = dict(kind=_lib.MB_LINEAR_ELASTIC, dim=3, E=30000.0, nu=0.2, disp_slot=0)
        P = ocore.Problem(m, 3, layers, ocore.Integrand.make(ocore.MB_LINEAR_ELASTIC, 3, E=30000.0, nu=0.2))
    else:
        kappa = rng.uniform(0.0, 3e-4, (P.n_el, P.n_ip))
        P.kappa = kappa
    return s, P, u, kappa


def _gpu(s, kappa):
    g = s.build_gpu()
    if kappa is not None:
        g.history = kappa
    return g


def _oracle(P, u):
    K = P.build_matrix_scipy(u).tocsr()
    K.sort_indices()
    return K


@pytest.mark.parametrize("n", [2, 6])
@pytest.mark.parametrize("kind", ["local_damage", "elastic"])
def test_tc20_tangent_against_oracle(n, kind):
    _torch()
    import nuto_gb300

    s, P, u, kappa = _case(n, kind)
    g = _gpu(s, kappa)
    K = _oracle(P, u)
    v = g.build_matrix(u, nuto_gb300.FP32).double().cpu().numpy()
    rp, ci = g.pattern()
    assert np.array_equal(rp, K.indptr) and np.array_equal(ci, K.indices)
    assert np.abs(v - K.data).max() <= FP32_REL * np.abs(K.data).max()


def test_tc20_matches_record_tangent_and_is_reproducible(monkeypatch):
    torch = _torch()
    import nuto_gb300

    s, P, u, kappa = _case(6, "local_damage", seed=5)
    g = _gpu(s, kappa)
    a = g.build_matrix(u, nuto_gb300.FP32)
    b = g.build_matrix(u, nuto_gb300.FP32)
    assert torch.equal(a, b)  # fixed MMA order, ordered row sums: bitwise reproducible
    monkeypatch.setenv("NUTO_GPU_TC20", "off")
    s2, _, _, _ = _case(6, "local_damage", seed=5)
    g2 = _gpu(s2, kappa)
    r = g2.build_matrix(u, nuto_gb300.FP32)
    scale = float(r.abs().max())
    # each is within FP32_REL of the FP64 values: their difference within twice that
    assert float((a - r).abs().max()) <= 2 * FP32_REL * scale


def test_tc20_single_tf32_product_error(monkeypatch):
    _torch()
    import nuto_gb300

    monkeypatch.setenv("NUTO_GPU_TC20", "tf32")
    s, P, u, kappa = _case(6, "local_damage", seed=3)
    g = _gpu(s, kappa)
    K = _oracle(P, u)
    v = g.build_matrix(u, nuto_gb300.FP32).double().cpu().numpy()
    err = np.abs(v - K.data).max() / np.abs(K.data).max()
    # TF32 keeps 10 explicit mantissa bits: the products carry about 2^-11 relative error
    assert 2e-6 < err <= 2e-3, err


def test_tc20_wait_gives_up_with_etimeout_and_context_stays_usable():
    _torch()
    import nuto_gb300

    s, P, u, kappa = _case(6, "local_damage", seed=9)
    g = _gpu(s, kappa)
    ref = g.build_matrix(u, nuto_gb300.FP32).double().cpu().numpy()
    g.synchronize()
    g.set_spin_limit(0)  # every wait on the MMA barrier runs out at once
    g.build_matrix(u, nuto_gb300.FP32)
    with pytest.raises(nuto_gb300.NutoGpuError) as e:
        g.synchronize()
    assert e.value.code == nuto_gb300._lib.ETIMEOUT
    g.synchronize()  # the status word was cleared by the failed synchronisation
    g.set_spin_limit(1 << 22)
    v = g.build_matrix(u, nuto_gb300.FP32).double().cpu().numpy()
    g.synchronize()
    assert np.array_equal(v, ref)


def test_tc20_at_converged_damaged_states():
    """After FP64 load steps into the damaged range every loading point has eq = kappa_h (the history update wrote
    it at that state): the tensor-core tangent must treat those points as loading like the FP64 tangent does, or it
    loses their rank-1 softening term. 8^3 cells, u_z = 1.5e-4 at t = 1, steps t = 0.2 and 0.4 (damage at the fixed
    face); the FP32 tangent within 2e-6 of the FP64 tangent after each step."""
    torch = _torch()
    import nuto_gb300
    from nuto_gb300 import configs

    s = configs.hex20_local_damage(8, u_end=1.5e-4, load_steps=5)
    g = s.build_gpu()
    o = g.default_options(precision=nuto_gb300.FP64, newton_rtol=1e-10, krylov_rtol=1e-10, forcing=0,
                          max_newton=40, max_krylov=20000)
    g.set_state(None, 0.0, True)
    for t in (0.2, 0.4):
        g.do_step(t, o)
        x = torch.as_tensor(g.get_state()[0], device="cuda")
        k64 = g.build_matrix(x, nuto_gb300.FP64)
        k32 = g.build_matrix(x, nuto_gb300.FP32).double()
        assert float((k32 - k64).abs().max()) <= FP32_REL * float(k64.abs().max()), t
    assert float(np.max(g.history)) > 1e-4  # damaged points present
