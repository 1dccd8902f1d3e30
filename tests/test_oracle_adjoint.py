"""The oracle's discrete adjoint of the gradient-damage load path (oracle/adjoint.py) against central finite
differences of complete forward solves: dL/dE_e (per-cell Young's modulus), dL/dkappa0 and dL/dbeta of a
displacement misfit after load steps into the damaged regime, on a notched plate (Quad4) and a beam (Hex8). The
reference has no adjoint; this pins the oracle that a GPU adjoint is compared with."""

import numpy as np
import pytest

from oracle import setups as osetups
from oracle.adjoint import AdjointOracle

E0 = 30000.0


def _case(kind):
    if kind == "plate":
        return (lambda law: osetups.notched_plate(6, 0.4, law=law)), [0.1 * k for k in range(1, 7)]
    return (lambda law: osetups.hex8_gradient_damage(2, law=law)), [0.05 * k for k in range(1, 9)]


def _loss(build, t_values, law, scale, obs, target, adjoint=False):
    m, layers, P, cons = build(law)
    P.set_e_scale(scale)
    A = AdjointOracle(P, cons[0], cons[1], cons[2])
    u = A.forward(t_values)
    r = np.zeros_like(u)
    r[obs] = u[obs] - target
    L = 0.5 * float(r[obs] @ r[obs])
    if not adjoint:
        return L, P
    return L, A.gradient(r, E0 * scale), P


def test_adjoint_workload_small_case_matches_central_differences():
    """The adjoint workload's set-up (hex8_adjoint: unit cube, lognormal modulus field, truth field of the next
    seed, observed surface nodes, 10 load steps) at 2^3 cells: the oracle's adjoint against central differences in
    kappa0, beta and the modulus of two cells, for the summed squared misfit against the truth's response."""
    from nuto_gb300 import configs

    case = configs.hex8_adjoint(2, seed=5, n_obs=6)
    t_values = []
    t = 0.0
    for _ in range(case.setup.load_steps):
        t += 1.0 / case.setup.load_steps
        t_values.append(t)

    def build(law):
        return osetups.hex8_gradient_damage(2, length=1.0, u_end=5e-4, law=law)

    obs = case.obs_dofs
    _, _, Pt, ct = build(None)
    Pt.set_e_scale(case.true_scale)
    target = AdjointOracle(Pt, ct[0], ct[1], ct[2]).forward(t_values)[obs]

    def loss(law, scale, adjoint=False):
        _, _, P, cons = build(law)
        P.set_e_scale(scale)
        A = AdjointOracle(P, cons[0], cons[1], cons[2])
        u = A.forward(t_values)
        r = np.zeros_like(u)
        r[obs] = u[obs] - target
        L = float(r[obs] @ r[obs])  # sum of squared misfits
        return (L, A.gradient(2.0 * r, E0 * scale), P) if adjoint else L

    base = {"kappa0": 1e-4, "beta": 100.0}
    L, g, P = loss(base, case.scale, adjoint=True)
    assert P.kappa.max() > 2e-4 and L > 0
    for name in ("kappa0", "beta"):
        h = 1e-4 * base[name]
        up, dn = dict(base), dict(base)
        up[name] += h
        dn[name] -= h
        ref = (loss(up, case.scale) - loss(dn, case.scale)) / (2 * h)
        assert abs(g[name] - ref) <= 1e-5 * abs(ref), (name, g[name], ref)
    for c in (0, 5):
        sp, sm = case.scale.copy(), case.scale.copy()
        sp[c] += 1e-6
        sm[c] -= 1e-6
        ref = (loss(base, sp) - loss(base, sm)) / 2e-6 / E0
        assert abs(g["E"][c] - ref) <= 1e-5 * abs(ref), (c, g["E"][c], ref)


@pytest.mark.parametrize("kind", ["plate", "beam"])
def test_adjoint_matches_central_differences(kind):
    build, t_values = _case(kind)
    rng = np.random.default_rng(3)
    m, layers, P0, cons = build(None)
    n_el = P0.n_el
    scale = 1.0 + 0.2 * rng.uniform(-1.0, 1.0, n_el)
    nu_dofs = m.layer_num_nodes(layers[0]) * (2 if kind == "plate" else 3)
    indep_u = np.setdiff1d(np.arange(nu_dofs), cons[0])
    obs = np.sort(rng.choice(indep_u, size=min(12, indep_u.size), replace=False))
    base = {"kappa0": 1e-4, "beta": 100.0}
    # target: 1.05 times the response of the uniform modulus (so that the misfit and its gradient are not zero)
    _, _, Pt, ct = build(base)
    target = AdjointOracle(Pt, ct[0], ct[1], ct[2]).forward(t_values)[obs] * 1.05
    L, g, P = _loss(build, t_values, base, scale, obs, target, adjoint=True)
    assert P.kappa.max() > 1.5e-4  # the last steps are damaged
    assert L > 0

    def fd(law, sc, h):
        lp, _ = _loss(build, t_values, law[0], sc[0], obs, target)
        lm, _ = _loss(build, t_values, law[1], sc[1], obs, target)
        return (lp - lm) / (2 * h)

    for name in ("kappa0", "beta"):
        h = 1e-4 * base[name]  # the misfit changes by ~1e-11 of itself for h = 1e-6: above the solve noise
        up, dn = dict(base), dict(base)
        up[name] += h
        dn[name] -= h
        ref = fd((up, dn), (scale, scale), h)
        assert abs(g[name] - ref) <= 1e-5 * abs(ref) + 1e-12 * L, (name, g[name], ref)
    cells = rng.choice(n_el, size=3, replace=False)
    for c in cells:
        h = 1e-6
        sp, sm = scale.copy(), scale.copy()
        sp[c] += h
        sm[c] -= h
        ref = fd((base, base), (sp, sm), h) / E0  # d/dE_e = d/d(scale_e) / E
        assert abs(g["E"][c] - ref) <= 1e-5 * max(abs(ref), np.abs(g["E"]).max() * 1e-3), (c, g["E"][c], ref)
