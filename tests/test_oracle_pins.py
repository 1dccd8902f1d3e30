"""Pins the oracle (CPU restatement) against the reference's own golden vectors and known answers.

Every test names the reference test or fixture it restates. None of these needs a GPU.
"""

import json
import math
import os

import numpy as np
import pytest

import oracle
from oracle import core

HERE = os.path.dirname(os.path.abspath(__file__))


def _single_element_problem(dim, geo, coords, integrand, ips=2, extra_layers=()):
    conn = np.arange(len(coords), dtype=np.int32)[None, :]
    mesh = oracle.Mesh.from_arrays(dim, geo, np.asarray(coords, float).ravel(), conn)
    d = mesh.add_dof(dim)
    slots = [d] + [mesh.add_dof(nc) for nc in extra_layers]
    return mesh, oracle.Problem(mesh, ips, slots, integrand)


def test_brick8n_golden_stiffness_and_internal_force(oracle_lib):
    """applications/integrationtests/mechanics/results/Brick8N*.txt via Brick8N.py:18-82."""
    g = json.load(open(os.path.join(HERE, "golden", "brick8n.json")))
    s = g["setup"]
    integ = oracle.Integrand.make(oracle.MB_LINEAR_ELASTIC, 3, E=s["E"], nu=s["nu"])
    mesh, P = _single_element_problem(3, oracle.HEX8, s["coords"], integ)
    u = np.zeros(P.n_dofs)
    for n in s["displaced_nodes"]:
        u[3 * n:3 * n + 3] = s["displacement"]
    fe, Ke = P.cell_integrate(0, u)
    K_ref = np.array(g["K_e"])
    f_ref = np.array(g["f_e"])
    assert np.abs(Ke - K_ref).max() <= 1e-11 * np.abs(K_ref).max()
    assert np.abs(fe - f_ref).max() <= 1e-11 * np.abs(f_ref).max()
    # internal force equals K_e u for the linear law
    assert np.allclose(Ke @ u, fe, rtol=0, atol=1e-13)


def test_cell_quad4_known_forces(oracle_lib):
    """test/mechanics/cell/Cell.cpp:17-101 (42 x 12 rectangle, E = 6174, nu = 0, plane strain)."""
    lx, ly, E = 42.0, 12.0, 6174.0
    integ = oracle.Integrand.make(oracle.MB_LINEAR_ELASTIC, 2, E=E, nu=0.0, plane_state=oracle.PLANE_STRAIN)
    mesh, P = _single_element_problem(2, oracle.QUAD4, [[0, 0], [lx, 0], [lx, ly], [0, ly]], integ)
    u = np.zeros(8)
    fe, _ = P.cell_integrate(0, u)
    assert np.abs(fe).max() < 1e-12
    ux = 0.4
    u[2] = u[4] = ux
    fe, _ = P.cell_integrate(0, u)
    F = E * ux / lx * ly / 2.0
    assert np.allclose(fe, [-F, 0, F, 0, F, 0, -F, 0], rtol=1e-12, atol=1e-9)
    u[:] = 0
    uy = 0.2
    u[5] = u[7] = uy
    fe, Ke = P.cell_integrate(0, u)
    F = E * uy / ly * lx / 2.0
    assert np.allclose(fe, [0, -F, 0, -F, 0, F, 0, F], rtol=1e-12, atol=1e-9)
    assert np.allclose(Ke @ u, fe, rtol=1e-12, atol=1e-9)
    assert abs(P.cell_volume(0) - lx * ly) < 1e-10 * lx * ly


@pytest.mark.parametrize("n", [1, 2, 3, 4])
def test_gauss_points_and_weights(oracle_lib, n):
    """test/mechanics/integrationtypes/IntegrationTypeTensorProduct.cpp:6-60 (Gauss)."""
    nodes = {1: [0.0], 2: [-math.sqrt(1 / 3), math.sqrt(1 / 3)], 3: [-math.sqrt(3 / 5), 0, math.sqrt(3 / 5)],
             4: [-math.sqrt(3 / 7 + 2 / 7 * math.sqrt(6 / 5)), -math.sqrt(3 / 7 - 2 / 7 * math.sqrt(6 / 5)),
                 math.sqrt(3 / 7 - 2 / 7 * math.sqrt(6 / 5)), math.sqrt(3 / 7 + 2 / 7 * math.sqrt(6 / 5))]}[n]
    weights = {1: [2.0], 2: [1.0, 1.0], 3: [5 / 9, 8 / 9, 5 / 9],
               4: [(18 - math.sqrt(30)) / 36, (18 + math.sqrt(30)) / 36, (18 + math.sqrt(30)) / 36,
                   (18 - math.sqrt(30)) / 36]}[n]
    pts, w = core.quadrature(1, n)
    assert np.allclose(pts[:, 0], nodes, rtol=1e-10, atol=1e-14)
    assert np.allclose(w, weights, rtol=1e-10)


@pytest.mark.parametrize("dim,n", [(2, 2), (3, 2), (3, 3)])
def test_tensor_product_exactness_and_order(oracle_lib, dim, n):
    """IntegrationTypeTensorProduct.cpp:15-39: first coordinate fastest; polynomial exactness (test :60-194)."""
    pts, w = core.quadrature(dim, n)
    assert abs(w.sum() - 2.0 ** dim) < 1e-13
    a = pts[:, 0] if dim >= 1 else None
    # first coordinate runs fastest
    assert pts[0, 0] < pts[1, 0]
    for deg in range(2 * n):
        val = (w * a ** deg * pts[:, 1] ** 2).sum()
        exact = (0 if deg % 2 else 2.0 / (deg + 1)) * (2.0 / 3.0) * (2.0 ** (dim - 2))
        assert abs(val - exact) < 1e-13


def test_linear_elastic_closed_forms(oracle_lib):
    """test/mechanics/constitutive/LinearElastic.cpp:9-77."""
    E, nu = 6174.0, 0.36
    C = core.linear_elastic_C(2, E, nu, oracle.PLANE_STRESS)
    exp = np.array([[1, nu, 0], [nu, 1, 0], [0, 0, (1 - nu) / 2]]) * E / (1 - nu * nu)
    assert np.allclose(C, exp, rtol=1e-14)
    C = core.linear_elastic_C(2, E, nu, oracle.PLANE_STRAIN)
    exp = np.array([[1 - nu, nu, 0], [nu, 1 - nu, 0], [0, 0, (1 - 2 * nu) / 2]]) * E / ((1 + nu) * (1 - 2 * nu))
    assert np.allclose(C, exp, rtol=1e-14)
    C = core.linear_elastic_C(3, E, nu, oracle.PLANE_STRAIN)
    exp = np.zeros((6, 6))
    exp[:3, :3] = nu
    np.fill_diagonal(exp[:3, :3], 1 - nu)
    for i in range(3, 6):
        exp[i, i] = (1 - 2 * nu) / 2
    exp *= E / ((1 + nu) * (1 - 2 * nu))
    assert np.allclose(C, exp, rtol=1e-14)
    assert np.allclose(core.linear_elastic_C(1, E, nu, 0), [[E]])


@pytest.mark.parametrize("dim,ps", [(1, 1), (2, oracle.PLANE_STRAIN), (2, oracle.PLANE_STRESS), (3, 1)])
def test_linear_elastic_damage_vs_linear_elastic(oracle_lib, dim, ps):
    """test/mechanics/constitutive/LinearElasticDamage.cpp:11-35 (FULL: (1 - omega) C eps)."""
    E, nu, omega = 6174.0, 0.36, 0.4
    vd = {1: 1, 2: 3, 3: 6}[dim]
    strain = np.full(vd, 0.1)
    C = core.linear_elastic_C(dim, E, nu, ps)
    s, dsde, dsdw = core.linear_elastic_damage(dim, E, nu, oracle.FULL, ps, strain, omega)
    assert np.allclose(s, (1 - omega) * C @ strain, rtol=1e-12)
    assert np.allclose(dsde, (1 - omega) * C, rtol=1e-12, atol=1e-9)
    assert np.allclose(dsdw, -C @ strain, rtol=1e-12)


@pytest.mark.parametrize("ps", [oracle.PLANE_STRAIN, oracle.PLANE_STRESS])
@pytest.mark.parametrize("omega", [0.0, 0.5, 0.8])
def test_linear_elastic_damage_unilateral_fd(oracle_lib, ps, omega):
    """test/mechanics/constitutive/LinearElasticDamage.cpp:37-98 (UNILATERAL, forward differences)."""
    for strain in ([0, 0, 0], [2, 0, 0], [-2, 0, 0], [0, 2, 0], [0, -2, 0], [2, 2, 0], [-2, -2, 0], [1, -2, 3]):
        strain = np.array(strain, float)
        s0, dsde, dsdw = core.linear_elastic_damage(2, 20000, 0.2, oracle.UNILATERAL, ps, strain, omega)
        delta = 1e-8
        fd = np.zeros((3, 3))
        for i in range(3):
            e = strain.copy()
            e[i] += delta
            fd[:, i] = (core.linear_elastic_damage(2, 20000, 0.2, oracle.UNILATERAL, ps, e, omega)[0] - s0) / delta
        assert np.allclose(dsde, fd, atol=max(dsde.max(), 1) * 1e-3)
        fdw = (core.linear_elastic_damage(2, 20000, 0.2, oracle.UNILATERAL, ps, strain, omega + delta)[0] - s0) / delta
        assert np.allclose(dsdw, fdw, atol=max(np.abs(dsdw).max() * 1e-6, 1e-6))


@pytest.mark.parametrize("dim,ps", [(1, 0), (2, oracle.PLANE_STRAIN), (2, oracle.PLANE_STRESS), (3, 1)])
def test_modified_mises_derivative_fd(oracle_lib, dim, ps):
    """test/mechanics/constitutive/ModifiedMisesStrainNorm.cpp:28-70 (forward differences, 1e-6)."""
    nu, k = 0.25, 9.81
    vd = {1: 1, 2: 3, 3: 6}[dim]
    cases = []
    for i in range(vd):
        e = np.zeros(vd)
        e[i] = math.pi
        cases.append(e)
        cases.append(-e)
    rng = np.random.default_rng(0)
    cases += [rng.uniform(-1, 1, vd) for _ in range(10)]
    for strain in cases:
        v0, d = core.mises(dim, nu, k, ps, strain)
        fd = np.zeros(vd)
        for i in range(vd):
            e = strain.copy()
            e[i] += 1e-8
            fd[i] = (core.mises(dim, nu, k, ps, e)[0] - v0) / 1e-8
        assert np.allclose(d, fd, atol=1e-6)


def test_modified_mises_known_values(oracle_lib):
    """test/mechanics/constitutive/ModifiedMisesStrainNorm.cpp:72-96."""
    k, nu = 10.0, 0.0
    for dim in (1, 2, 3):
        vd = {1: 1, 2: 3, 3: 6}[dim]
        assert abs(core.mises(dim, nu, k, oracle.PLANE_STRAIN, np.zeros(vd))[0]) < 1e-6
    e = np.zeros(6)
    e[0] = 2.0
    assert abs(core.mises(3, nu, k, 1, e)[0] - 2.0) < 2e-8
    e[:] = 0
    e[2] = -2 * k
    assert abs(core.mises(3, nu, k, 1, e)[0] - 2.0) < 2e-8


def test_damage_law_exponential(oracle_lib):
    """test/mechanics/constitutive/damageLaws/DamageLawExponential.cpp:4-31 + DamageLawHelper.h:12-40."""
    # ExponentialDerivative: central differences of omega(kappa), kappa0 = 1e-4, beta = 350, alpha = 0.9
    k0, beta, alpha = 1e-4, 350.0, 0.9
    delta = 1e-8
    kappa = delta
    while kappa < 0.5:
        w, dw = core.damage_exponential(k0, beta, alpha, kappa)
        if kappa < k0:
            assert abs(w) < 1e-10 and abs(dw) < 1e-10
        cdf = (core.damage_exponential(k0, beta, alpha, kappa + 0.5 * delta)[0]
               - core.damage_exponential(k0, beta, alpha, kappa - 0.5 * delta)[0]) / delta
        assert abs(dw - cdf) < 1e-4
        kappa += k0 / 5
    # ExponentialResLoad: residual pseudo stress E kappa0 (1 - alpha), 1e-3 %
    E = 1e6
    for kappa in (1.0, 2.0, 10.0, 100.0, 1000.0):
        ps = (1 - core.damage_exponential(k0, beta, alpha, kappa)[0]) * E * kappa
        assert abs(ps - E * k0 * (1 - alpha)) <= 1e-5 * E * k0 * (1 - alpha)
    # ExponentialMaterial: DefaultConcrete with fMin = 0, fracture energy integral 1e-5 %
    E, ft, gf = 30000.0, 4.0, 0.1
    k0, beta, alpha = ft / E, ft / gf, 1.0
    dk = k0 / 10
    g = 0.0
    k = k0
    while k < 10000 * k0:
        sa = (1 - core.damage_exponential(k0, beta, alpha, k)[0]) * E * k
        sb = (1 - core.damage_exponential(k0, beta, alpha, k + dk)[0]) * E * (k + dk)
        g += 0.5 * dk * (sa + sb)
        k += dk
    assert abs(g - gf) <= 1e-7 * gf


def test_local_isotropic_damage_1d_analytic(oracle_lib):
    """test/mechanics/constitutive/LocalIsotropicDamage.cpp:12-55 (1D softening branch, 1e-10 %)."""
    E, nu, ft, fc, gf = 30000.0, 0.2, 4.0, 40.0, 0.1
    k0, beta, alpha, k = ft / E, ft / gf, 1.0, fc / ft

    def analytic(strain):
        return E * strain if strain < k0 else ft * math.exp(ft / gf * (k0 - strain))

    kappa_h = 0.0
    strain = k0
    kappa_h = max(kappa_h, core.mises(1, nu, k, 1, np.array([strain]))[0])
    stress = ft * 0.99
    while stress > 0:
        for _ in range(100):
            s, t = core.local_damage(1, E, nu, oracle.FULL, 1, k0, beta, alpha, k, kappa_h, np.array([strain]))
            r = s[0] - stress
            if abs(r) < 1e-12:
                break
            strain -= r / t[0, 0]
        kappa_h = max(kappa_h, core.mises(1, nu, k, 1, np.array([strain]))[0])
        assert abs(stress - analytic(strain)) <= 1e-12 * stress
        stress -= ft * 0.1


def test_local_isotropic_damage_tangent_fd(oracle_lib):
    """test/mechanics/constitutive/LocalIsotropicDamage.cpp:57-114 (central differences, 1e-5)."""
    E, nu, ft, fc, gf = 30000.0, 0.2, 4.0, 40.0, 0.1
    k0, beta, alpha, k = ft / E, ft / gf, 1 - 0.04 / ft, fc / ft
    cases = []
    kappa = k0 / 3
    for v in ([0, 0, 0], [1e-5, 0, 0], [-1e-5, 0, 0], [1e-5, 1e-5, 0], [2e-5, 1e-5, 0], [2e-5, -1e-5, 0],
              [0, 0, 2e-5], [1e-5, 1e-5, 2e-5], [1e-5, -2e-5, 2e-5]):
        cases.append((v, kappa))
    kappa = 2 * k0
    eps = 1e-6
    for v in ([kappa + eps, 0, 0], [kappa, eps, 0], [kappa, 0, eps], [kappa + eps, eps, 0], [kappa, eps, eps],
              [kappa + eps, 0, eps], [kappa - eps, 0, 0], [kappa, -eps, 0], [kappa, 0, -eps],
              [kappa - eps, -eps, 0], [kappa, -eps, -eps], [kappa - eps, 0, -eps]):
        cases.append((v, kappa))
    for v, kh in cases:
        strain = np.zeros(6)
        strain[:3] = v
        _, t = core.local_damage(3, E, nu, oracle.FULL, 1, k0, beta, alpha, k, kh, strain)
        cdf = np.zeros((6, 6))
        d = 1e-8
        for i in range(6):
            e0 = strain.copy()
            e0[i] -= d / 2
            e1 = strain.copy()
            e1[i] += d / 2
            s0, _ = core.local_damage(3, E, nu, oracle.FULL, 1, k0, beta, alpha, k, kh, e0)
            s1, _ = core.local_damage(3, E, nu, oracle.FULL, 1, k0, beta, alpha, k, kh, e1)
            cdf[:, i] = (s1 - s0) / d
        assert np.abs(cdf - t).max() < 1e-5 * max(1.0, np.abs(t).max() / E * 1e3)


@pytest.mark.parametrize("dim", [2, 3])
@pytest.mark.parametrize("app", [oracle.FULL, oracle.UNILATERAL])
@pytest.mark.parametrize("inter", [0, 1])
def test_gradient_damage_hessian0_fd(oracle_lib, dim, app, inter):
    """test/mechanics/integrands/GradientDamage.cpp:11-122: FD check of all four Hessian0 blocks, three states."""
    if dim == 2:
        coords = [[0, 0], [1.1, 0.1], [1.0, 0.9], [-0.1, 1.2]]
        geo = oracle.QUAD4
    else:
        coords = [[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0], [0, 0, 1], [1, 0, 1.1], [1.1, 1, 1], [0, 1, 1]]
        geo = oracle.HEX8
    E, nu = 20000.0, 0.2
    k0 = 4.0 / E
    integ = oracle.Integrand.make(oracle.GRADIENT_DAMAGE, dim, E=E, nu=nu, damage_application=app, kappa0=k0,
                                  beta=360.0 * 0.0 + 4.0 / (4.0 / 360), alpha=0.96, k=10.0, c=0.5,
                                  interaction=inter)
    mesh, P = _single_element_problem(dim, geo, coords, integ, extra_layers=(1,))
    nd = len(coords) * dim
    rng = np.random.default_rng(1)
    for eeq_level, kh in ((0.0, 0.0), (1.0, 2.0), (9.5, 9.0)):
        u = np.zeros(P.n_dofs)
        u[:nd] = rng.uniform(-1, 1, nd) * 0.01
        u[nd:] = k0 * (eeq_level + 0.5 * rng.uniform(-1, 1, len(coords)))
        P.kappa = kh * k0
        f0, K = P.cell_integrate(0, u)
        fd = np.zeros_like(K)
        for j in range(P.n_local):
            delta = k0 / 10000
            up = u.copy()
            up[j] += delta
            fd[:, j] = (P.cell_integrate(0, up)[0] - f0) / delta
        blocks = [(slice(0, nd), slice(0, nd), 1e-4), (slice(0, nd), slice(nd, None), 1e-4),
                  (slice(nd, None), slice(0, nd), 1e-2), (slice(nd, None), slice(nd, None), 1e-4)]
        for r, c, tol in blocks:
            a = K[r, c]
            atol = max(tol, tol * np.abs(a).max())
            assert np.abs(a - fd[r, c]).max() <= atol


def test_first_touch_numbering_and_counts(oracle_lib):
    """MeshFemDofConvert.cpp:164-210 + DofNumbering.cpp:7-58 + test/mechanics/mesh/UnitMeshFem.cpp:47-125."""
    m = oracle.Mesh.bricks(3, 2, 4)
    d = m.add_dof(3)
    assert m.num_elements == 24
    assert m.layer_num_nodes(d) == 4 * 3 * 5
    conn = m.layer_conn(d)
    # first touch: the first element owns nodes 0..7, every later element introduces increasing new ids
    assert conn[0].tolist() == list(range(8))
    seen = -1
    for row in conn:
        for n in row:
            if n > seen:
                assert n == seen + 1
                seen = n
    dn = m.layer_dof_numbers(d, 3)
    assert np.array_equal(dn.ravel(), np.arange(dn.size))
    # Hex20 displacement layer on the Hex8 coordinate mesh (SURVEY config C4 layout)
    m2 = oracle.Mesh.bricks(2, 2, 2)
    q = m2.add_dof(3, oracle.HEX20)
    n = 2
    assert m2.layer_num_nodes(q) == (n + 1) ** 3 + 3 * n * (n + 1) ** 2
    # positive det J on a transformed mesh
    m3 = oracle.Mesh.bricks(2, 2, 2).scale(1, 1, 4)
    l3 = m3.add_dof(3)
    P = oracle.Problem(m3, 2, [l3], oracle.Integrand.make(oracle.MB_LINEAR_ELASTIC, 3))
    assert all(P.cell_volume(e) > 0 for e in range(8))
    assert abs(sum(P.cell_volume(e) for e in range(8)) - 4.0) < 1e-12


def test_assembled_pattern_counts(oracle_lib):
    """nnz(K) of the structural pattern incl. explicit zeros (SimpleAssembler.cpp:118-154)."""
    for n in (2, 3):
        m = oracle.Mesh.bricks(n, n, n)
        d = m.add_dof(3)
        e = m.add_dof(1)
        P = oracle.Problem(m, 2, [d, e], oracle.Integrand.make(oracle.GRADIENT_DAMAGE, 3))
        cp, ri, v = P.build_matrix_csc(np.zeros(P.n_dofs))
        assert len(v) == 16 * (3 * n + 1) ** 3
        # row indices sorted inside every column, pattern structurally symmetric
        import scipy.sparse as sp

        A = sp.csc_matrix((np.ones_like(v), ri, cp), shape=(P.n_dofs, P.n_dofs))
        assert (A != A.T).nnz == 0
        for c in range(P.n_dofs):
            col = ri[cp[c]:cp[c + 1]]
            assert np.all(np.diff(col) > 0)
    m = oracle.Mesh.quads(4, 3)
    d = m.add_dof(2)
    P = oracle.Problem(m, 2, [d], oracle.Integrand.make(oracle.MB_LINEAR_ELASTIC, 2))
    cp, ri, v = P.build_matrix_csc(np.zeros(P.n_dofs))
    # 2D Quad4 node pairs: sum over nodes of (neighbours) * 4
    assert len(v) == 4 * (3 * 4 + 1) * (3 * 3 + 1)


def test_build_vector_matches_cellwise_scatter(oracle_lib):
    """SimpleAssembler::BuildVector scatter (SimpleAssembler.cpp:38-65, test SimpleAssembler.cpp:57-78)."""
    m = oracle.Mesh.quads(3, 2)
    d = m.add_dof(2)
    e = m.add_dof(1)
    P = oracle.Problem(m, 2, [d, e], oracle.Integrand.make(oracle.GRADIENT_DAMAGE, 2))
    rng = np.random.default_rng(3)
    u = rng.uniform(-1e-4, 1e-4, P.n_dofs)
    f = P.build_vector(u)
    ref = np.zeros(P.n_dofs)
    for c in range(P.n_el):
        fe, _ = P.cell_integrate(c, u)
        np.add.at(ref, P.cell_dofs(c), fe)
    # thread-order summation (SimpleAssembler.cpp:61-62): compare relative to the largest entry
    assert np.abs(f - ref).max() <= 1e-13 * np.abs(ref).max()
    K = P.build_matrix_scipy(u).toarray()
    Kref = np.zeros((P.n_dofs, P.n_dofs))
    for c in range(P.n_el):
        _, Ke = P.cell_integrate(c, u)
        idx = P.cell_dofs(c)
        Kref[np.ix_(idx, idx)] += Ke
    assert np.abs(K - Kref).max() <= 1e-13 * np.abs(Kref).max()


def test_lumped_mass_hrz_known_answer():
    """test/mechanics/cell/SimpleAssembler.cpp:116-150: two cells [0,1,2] and [2,3,4] with the local matrix
    11..33 on a one-component DOF type: diagonal scaled by total / diagonal sum, summed at the shared DOF."""
    from oracle import core

    M = np.array([[11, 12, 13], [21, 22, 23], [31, 32, 33]], dtype=float)
    lump = core.lump_hrz(M, 1)
    total = M.sum()
    expect = np.array([11.0, 22.0, 33.0]) * (total / (11.0 + 22.0 + 33.0))
    assert np.allclose(lump, expect, rtol=1e-15)
    glob = np.zeros(5)
    glob[[0, 1, 2]] += lump
    glob[[2, 3, 4]] += lump
    assert np.allclose(glob, [expect[0], expect[1], expect[2] + expect[0], expect[1], expect[2]], rtol=1e-15)
    # the DofType::GetNum division: a block with ncomp components sharing the scalar pattern
    assert np.allclose(core.lump_hrz(np.kron(M, np.eye(3)), 3), np.repeat(expect, 3) / 3, rtol=1e-14)


@pytest.mark.parametrize("kind,n", [("quad4", 4), ("hex8gd", 2), ("hex20", 2)])
def test_lumped_mass_total_is_rho_volume_over_components(kind, n):
    from oracle import setups

    om, layers, P, cons = {"quad4": setups.quad4_elastic, "hex8gd": setups.hex8_gradient_damage,
                           "hex20": setups.hex20_local_damage}[kind](n)
    rho = 2.5
    m = P.lumped_mass(rho)
    volume = {"quad4": 1.0, "hex8gd": 4.0, "hex20": 1.0}[kind]
    ncomp = 2 if kind == "quad4" else 3
    n_disp = ncomp * om.layer_num_nodes(layers[0])
    assert abs(m[:n_disp].sum() - rho * volume) <= 1e-12 * rho * volume
    for c in range(ncomp):
        assert abs(m[c:n_disp:ncomp].sum() - rho * volume / ncomp) <= 1e-12 * rho * volume
    assert np.all(m[n_disp:] == 0.0)
    assert np.all(m[:n_disp] > 0)  # HRZ scales the positive diagonal (unlike row-sum lumping of Hex20)


def test_eval_ip_consistency():
    """Cell::Eval values: kappa after UpdateHistory equals the history, elastic stress is C eps, damage is
    omega(kappa)."""
    from oracle import core, setups

    om, layers, P, cons = setups.hex8_gradient_damage(2)
    rng = np.random.default_rng(3)
    u = rng.uniform(-2e-4, 2e-4, P.n_dofs)
    nd = 3 * om.layer_num_nodes(layers[0])
    u[nd:] = rng.uniform(0, 4e-4, P.n_dofs - nd)
    P.kappa = rng.uniform(0, 3e-4, (P.n_el, P.n_ip))
    kap = P.eval_ip(u, core.IP_KAPPA)[..., 0]
    P.update_history(u)
    assert np.array_equal(kap, P.kappa)
    om_ = P.eval_ip(u, core.IP_DAMAGE)[..., 0]
    k0, beta, alpha = 1e-4, 100.0, 0.99
    ref = np.where(kap < k0, 0.0, 1 - k0 / kap * (1 - alpha + alpha * np.exp(beta * (k0 - kap))))
    assert np.allclose(om_, ref, rtol=1e-13, atol=1e-16)
    omq, layq, Pq, _ = setups.quad4_elastic(3)
    uq = rng.uniform(-1e-3, 1e-3, Pq.n_dofs)
    eps = Pq.eval_ip(uq, core.IP_STRAIN)
    sig = Pq.eval_ip(uq, core.IP_STRESS)
    C = core.linear_elastic_C(2, 30000.0, 0.2, core.PLANE_STRAIN)
    assert np.allclose(sig, eps @ C.T, rtol=1e-13, atol=1e-12)


def test_neumann_known_answers():
    """test/mechanics/integrands/NeumannBc.cpp:17-76: ExternalLoad = N^T p of a Line2 boundary cell in 2D at the
    natural points -1, 0, +1 (all of p at the first node, half at each node, all at the second node)."""
    from oracle import core

    p = np.array([4.0, 42.0])
    assert np.allclose(core.neumann_ip(2, 2, [-1.0], p), [4, 42, 0, 0], atol=1e-15)
    assert np.allclose(core.neumann_ip(2, 2, [1.0], p), [0, 0, 4, 42], atol=1e-15)
    assert np.allclose(core.neumann_ip(2, 2, [0.0], p), [2, 21, 2, 21], atol=1e-15)


@pytest.mark.parametrize("kind", ["quad4", "hex8"])
def test_external_load_total_force(kind):
    """The boundary load of a uniform traction sums to traction x boundary measure (codimension-1 det J)."""
    from oracle import core
    from nuto_gb300 import mesh as M

    if kind == "quad4":
        m = M.create_quads(5, 3).scale(2.0, 1.5)
        d = M.add_dof_interpolation(m, 2)
        fc, fd = M.boundary_faces(m, d, 0, 2.0)
        om = core.Mesh.from_arrays(2, core.QUAD4, m.coords, m.conn)
        p, measure = np.array([0.3, -1.2]), 1.5
    else:
        m = M.create_bricks(3, 2, 4).scale(1.0, 2.0, 3.0)
        d = M.add_dof_interpolation(m, 3)
        fc, fd = M.boundary_faces(m, d, 2, 3.0)
        om = core.Mesh.from_arrays(3, core.HEX8, m.coords, m.conn)
        p, measure = np.array([0.3, -1.2, 2.0]), 2.0
    L = m.layers[d]
    dim = m.dim
    dofs = L.dof_numbers[fd]  # faces x nodes x dim
    f = om.external_load(L.num_dofs, fc, dofs, p, gauss=2)
    for c in range(dim):
        assert abs(f[c::dim].sum() - p[c] * measure) <= 1e-13 * abs(p[c] * measure)
    assert np.count_nonzero(f) == dim * np.unique(fd).size
