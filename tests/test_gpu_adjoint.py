"""The GPU discrete adjoint of the gradient-damage load path (nuto_gb300.adjoint over the C ABI) on the adjoint
workload (hex8_adjoint: unit cube, lognormal per-cell modulus, 10 load steps into the damaged range, squared misfit
at observed surface nodes against the response of a second modulus field):

- dL/dE_e, dL/dkappa0, dL/dbeta against the oracle's adjoint (oracle/adjoint.py, pinned by central differences of
  direct-solve forward runs in tests/test_oracle_adjoint.py): <= 1e-6 relative;
- against central differences of the GPU's own forward solves, h = 1e-6 relative;
- checkpointing every third load step (states recomputed on the backward pass) gives the gradient of checkpointing
  every step;
- the torch.autograd.Function gives the same gradient through torch's backward.
"""

import numpy as np
import pytest

from oracle import setups as osetups
from oracle.adjoint import AdjointOracle

pytestmark = pytest.mark.gpu

E0 = 30000.0


def _torch():
    import torch

    assert torch.cuda.is_available(), "these tests need a CUDA GPU"
    return torch


def _times(steps):
    t, out = 0.0, []
    for _ in range(steps):
        t += 1.0 / steps
        out.append(t)
    return out


def _case(n=2, seed=5, n_obs=6):
    from nuto_gb300 import configs

    case = configs.hex8_adjoint(n, seed=seed, n_obs=n_obs)
    t_values = _times(case.setup.load_steps)

    def oracle_build(law):
        return osetups.hex8_gradient_damage(n, length=1.0, u_end=5e-4, law=law)

    _, _, Pt, ct = oracle_build(None)
    Pt.set_e_scale(case.true_scale)
    target = AdjointOracle(Pt, ct[0], ct[1], ct[2]).forward(t_values)[case.obs_dofs]
    return case, t_values, oracle_build, target


def _path(case, t_values, every=1):
    from nuto_gb300.adjoint import AdjointLoadPath

    g = case.setup.build_gpu()
    return AdjointLoadPath(g, case.setup.integrand, t_values, checkpoint_every=every)


def _gpu_loss_grad(path, scale, k0, beta, obs, target, grad=True):
    torch = _torch()
    x = path.forward(scale, k0, beta)
    idx = torch.as_tensor(obs, device=x.device)
    r = torch.zeros_like(x)
    r[idx] = x[idx] - torch.as_tensor(target, device=x.device)
    L = float((r[idx] ** 2).sum())
    if not grad:
        return L
    gE, gk, gb = path.backward(2.0 * r)
    return L, gE.cpu().numpy(), gk, gb


def test_gpu_adjoint_matches_oracle_adjoint():
    case, t_values, oracle_build, target = _case()
    obs = case.obs_dofs
    path = _path(case, t_values)
    L, gE, gk, gb = _gpu_loss_grad(path, case.scale, 1e-4, 100.0, obs, target)
    _, _, P, cons = oracle_build(None)
    P.set_e_scale(case.scale)
    A = AdjointOracle(P, cons[0], cons[1], cons[2])
    u = A.forward(t_values)
    r = np.zeros_like(u)
    r[obs] = u[obs] - target
    Lo = float(r[obs] @ r[obs])
    go = A.gradient(2.0 * r, E0 * case.scale)
    assert P.kappa.max() > 2e-4 and Lo > 0  # the load path reached the damaged range
    assert abs(L - Lo) <= 1e-8 * Lo
    assert abs(gk - go["kappa0"]) <= 1e-6 * abs(go["kappa0"])
    assert abs(gb - go["beta"]) <= 1e-6 * abs(go["beta"])
    assert np.abs(gE - go["E"]).max() <= 1e-6 * np.abs(go["E"]).max()


def test_gpu_adjoint_matches_central_differences():
    case, t_values, _, target = _case()
    obs = case.obs_dofs
    path = _path(case, t_values)
    base = (1e-4, 100.0)
    L, gE, gk, gb = _gpu_loss_grad(path, case.scale, *base, obs, target)
    for i, g in enumerate((gk, gb)):
        h = 1e-6 * base[i]
        up, dn = list(base), list(base)
        up[i] += h
        dn[i] -= h
        ref = (_gpu_loss_grad(path, case.scale, *up, obs, target, grad=False)
               - _gpu_loss_grad(path, case.scale, *dn, obs, target, grad=False)) / (2 * h)
        assert abs(g - ref) <= 1e-4 * abs(ref), (i, g, ref)
    for c in (0, 5):
        h = 1e-6
        sp, sm = case.scale.copy(), case.scale.copy()
        sp[c] += h
        sm[c] -= h
        ref = (_gpu_loss_grad(path, sp, *base, obs, target, grad=False)
               - _gpu_loss_grad(path, sm, *base, obs, target, grad=False)) / (2 * h) / E0
        assert abs(gE[c] - ref) <= 1e-4 * max(abs(ref), 1e-3 * np.abs(gE).max()), (c, gE[c], ref)


def test_gpu_adjoint_checkpoints_and_autograd():
    torch = _torch()
    from nuto_gb300.adjoint import load_path_function

    case, t_values, _, target = _case()
    obs = case.obs_dofs
    every1 = _path(case, t_values, every=1)
    _, gE1, gk1, gb1 = _gpu_loss_grad(every1, case.scale, 1e-4, 100.0, obs, target)
    every3 = _path(case, t_values, every=3)
    _, gE3, gk3, gb3 = _gpu_loss_grad(every3, case.scale, 1e-4, 100.0, obs, target)
    assert len(every3.checkpoints) == 4 and every3.recomputed_steps == len(t_values)
    assert np.abs(gE3 - gE1).max() <= 1e-8 * np.abs(gE1).max()
    assert abs(gk3 - gk1) <= 1e-8 * abs(gk1) and abs(gb3 - gb1) <= 1e-8 * abs(gb1)
    # through torch.autograd
    dev = torch.device("cuda", 0)
    young = torch.tensor(E0 * case.scale, dtype=torch.float64, device=dev, requires_grad=True)
    k0 = torch.tensor(1e-4, dtype=torch.float64, device=dev, requires_grad=True)
    beta = torch.tensor(100.0, dtype=torch.float64, device=dev, requires_grad=True)
    fn = load_path_function()
    u = fn.apply(young, k0, beta, _path(case, t_values, every=2))
    loss = ((u[torch.as_tensor(obs, device=dev)] - torch.as_tensor(target, device=dev)) ** 2).sum()
    loss.backward()
    assert np.abs(young.grad.cpu().numpy() - gE1).max() <= 1e-8 * np.abs(gE1).max()
    assert abs(float(k0.grad) - gk1) <= 1e-8 * abs(gk1)
    assert abs(float(beta.grad) - gb1) <= 1e-8 * abs(gb1)
