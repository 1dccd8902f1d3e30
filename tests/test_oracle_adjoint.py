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
