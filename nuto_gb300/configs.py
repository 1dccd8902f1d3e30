"""Problem set-ups of the benchmark workloads, at any mesh size (the tests use small sizes).

quad4_elastic      2D plane-strain linear elasticity on the unit square, n x n Quad4 (2x2 Gauss), E = 30000,
                   nu = 0.2; left edge fixed in x and y, right edge u_x = RhsRamp(1, 0.01): one load step to
                   t = 1 is one BuildMatrix + BuildVector + one linear solve (QuasistaticSolver applies only the
                   change of the constraint values between two times, so a constant value would never act).
hex8_gradient_damage
                   3D implicit gradient-enhanced damage: n x n x n Hex8 (2x2x2 Gauss) on a 1 x 1 x 4 beam (z
                   long), u (3 DOF) + nonlocal equivalent strain (1 DOF); LinearElasticDamage(30000, 0.2, FULL),
                   DamageLawExponential(kappa0 = 1e-4, beta = 100, alpha = 0.99), ModifiedMisesStrainNorm(0.2,
                   k = 10), c = 0.01; z = 0 face fixed, z = 4 face u_z = RhsRamp(1, 2e-3) (20 load steps to
                   t = 1). E and nu are NuTo's DefaultConcrete values.
hex20_local_damage 3D Hex20 displacements (3x3x3 Gauss) on an n^3 Hex8 coordinate mesh of the unit cube,
                   MomentumBalance + LocalIsotropicDamage (E = 30000, nu = 0.2, kappa0 = 1e-4, beta = 100,
                   alpha = 0.99, k = 10); z = 0 face fixed, z = 1 face u_z = RhsRamp(1, 5e-5) (5 load steps;
                   mean strain 0.5 kappa0: the fixed face's edges, where the restrained lateral contraction
                   concentrates the strain, damage from the first steps on and the damage stays confined there.
                   Larger loads localise the softening into one cell layer, and Newton then finds no equilibrium
                   within 50 iterations on either path once the mesh is fine enough: 1.5e-4 from 16^3 on,
                   8e-5 from 32^3 on).
hex8_adjoint       the adjoint workload: hex8_gradient_damage on the unit cube (n^3 cells, z = 1 face u_z =
                   RhsRamp(1, 5e-4), the beam's mean strain, 10 load steps), a per-cell lognormal Young's modulus
                   (mean 30000, CoV 0.3, Gaussian correlation exp(-r^2 / (2 l^2)) with l = 0.1 between cell
                   centroids, seeded), a second field of the next seed as the synthetic truth, and 256 seeded
                   observed surface nodes (all three displacement components; the fixed z = 0 face excluded).
notched_plate      2D plane-strain gradient-enhanced damage on the unit square, n x n Quad4 (2x2 Gauss), u (2 DOF)
                   + eeq (1 DOF), the law of hex8_gradient_damage in 2D; a notch one cell high from the left edge
                   at mid height (cells of row n/2 with x index below round(depth n) removed); bottom edge u_y = 0,
                   the corner (0, 0) also u_x = 0, top edge u_y = RhsRamp(1, u_end) (10 load steps). One specimen of
                   the batched workload (nuto_gb300.batch).
"""

from dataclasses import dataclass, field

import numpy as np

from . import mesh as M
from ._lib import (DAMAGE_FULL, GRADIENT_DAMAGE, HEX20, MB_LINEAR_ELASTIC, MB_LOCAL_DAMAGE, PLANE_STRAIN)


@dataclass
class Setup:
    name: str
    mesh: M.MeshFem
    layers: list
    gauss: int
    integrand: dict
    # per layer: (dependent dofs, rhs_const, rhs_slope)
    constraints: list = field(default_factory=list)
    load_steps: int = 1
    t_end: float = 1.0
    # initial history kappa [cell, ip] (None: zero), e.g. an imperfection
    history0: object = None

    def dependent_counts(self):
        return [len(c[0]) for c in self.constraints]

    @property
    def n_dofs(self):
        return sum(self.mesh.layers[l].num_dofs for l in self.layers)

    def build_gpu(self, device=0):
        from .assembly import GpuCellGroup

        g = GpuCellGroup(self.mesh, self.layers, self.gauss, device=device,
                         dependent_counts=self.dependent_counts())
        for slot, (dofs, a, b) in enumerate(self.constraints):
            if len(dofs):
                g.set_dirichlet(slot, dofs, a, b)
        g.build_pattern()
        g.set_integrand(**self.integrand)
        return g


def _merge(*cons):
    dofs = np.concatenate([c[0] for c in cons]).astype(np.int32)
    a = np.concatenate([c[1] for c in cons])
    b = np.concatenate([c[2] for c in cons])
    return dofs, a, b


def _empty():
    return np.zeros(0, np.int32), np.zeros(0), np.zeros(0)


def quad4_elastic(n=200, u_right=0.01):
    m = M.create_quads(n, n)
    d = M.add_dof_interpolation(m, 2)
    left = M.nodes_at_axis(m, d, 0, 0.0)
    right = M.nodes_at_axis(m, d, 0, 1.0)
    cons = _merge(M.component_constraints(m, d, left, [0, 1], 0.0),
                  M.component_constraints(m, d, right, [0], 0.0, u_right))
    integ = dict(kind=MB_LINEAR_ELASTIC, dim=2, E=30000.0, nu=0.2, plane_state=PLANE_STRAIN, disp_slot=0)
    return Setup("quad4_elastic_%dx%d" % (n, n), m, [d], 2, integ, [cons], 1, 1.0)


def gradient_damage_imperfection(n, n_ip, kappa0=1e-4):
    """kappa = 3 kappa0 at every integration point of the two cell layers n/2 and n/2 + 1 along the beam axis: the
    imperfection of StructuralGradientDamage.cpp:66-68 (there: two cells of a 1D bar), which makes the damage
    localise there instead of at a round-off-dependent place."""
    iz = np.arange(n * n * n) // (n * n)
    k = np.zeros((n * n * n, n_ip))
    k[(iz == n // 2) | (iz == n // 2 + 1)] = 3.0 * kappa0
    return k


def hex8_gradient_damage(n=64, length=4.0, u_end=2e-3, load_steps=20, imperfection=False):
    m = M.create_bricks(n, n, n).scale(1.0, 1.0, length)
    d = M.add_dof_interpolation(m, 3)
    e = M.add_dof_interpolation(m, 1)
    bottom = M.nodes_at_axis(m, d, 2, 0.0)
    top = M.nodes_at_axis(m, d, 2, length)
    cons_d = _merge(M.component_constraints(m, d, bottom, [0, 1, 2], 0.0),
                    M.component_constraints(m, d, top, [2], 0.0, u_end))
    integ = dict(kind=GRADIENT_DAMAGE, dim=3, E=30000.0, nu=0.2, plane_state=PLANE_STRAIN,
                 damage_application=DAMAGE_FULL, kappa0=1e-4, beta=100.0, alpha=0.99, k=10.0, c=0.01, disp_slot=0,
                 eeq_slot=1)
    h0 = gradient_damage_imperfection(n, 8, integ["kappa0"]) if imperfection else None
    return Setup("hex8_gradient_damage_%d^3" % n, m, [d, e], 2, integ, [cons_d, _empty()], load_steps, 1.0, h0)


def hex20_local_damage(n=80, u_end=5e-5, load_steps=5):
    m = M.create_bricks(n, n, n)
    d = M.add_dof_interpolation(m, 3, HEX20)
    bottom = M.nodes_at_axis(m, d, 2, 0.0)
    top = M.nodes_at_axis(m, d, 2, 1.0)
    cons = _merge(M.component_constraints(m, d, bottom, [0, 1, 2], 0.0),
                  M.component_constraints(m, d, top, [2], 0.0, u_end))
    integ = dict(kind=MB_LOCAL_DAMAGE, dim=3, E=30000.0, nu=0.2, plane_state=PLANE_STRAIN,
                 damage_application=DAMAGE_FULL, kappa0=1e-4, beta=100.0, alpha=0.99, k=10.0, disp_slot=0)
    return Setup("hex20_local_damage_%d^3" % n, m, [d], 3, integ, [cons], load_steps, 1.0)


def notched_plate_mesh(n, depth=0.3):
    """Unit square, n x n Quad4 cells (UnitMeshFem::CreateQuads order) without the notch cells: row n // 2, x index
    below round(depth n) (at least 1, at most n - 2). Coordinate nodes that no remaining cell uses are dropped; the
    others keep their relative order."""
    full = M.create_quads(n, n)
    cut = notch_cells(n, depth)
    conn = full.conn[~cut]
    used = np.unique(conn)
    remap = np.full(full.coords.shape[0], -1, dtype=np.int64)
    remap[used] = np.arange(used.size)
    return M.MeshFem(2, full.geo_interp, full.coords[used], remap[conn])


def notch_cells(n, depth):
    """Mask over the n x n cells (lattice order, x fastest) of the notch."""
    if n < 4:
        raise ValueError("a notched plate needs n >= 4")
    iy, ix = np.divmod(np.arange(n * n), n)
    d = min(max(int(round(depth * n)), 1), n - 2)
    return (iy == n // 2) & (ix < d)


def notched_plate(n=40, depth=0.3, u_end=2e-4, load_steps=10):
    m = notched_plate_mesh(n, depth)
    d = M.add_dof_interpolation(m, 2)
    e = M.add_dof_interpolation(m, 1)
    bottom = M.nodes_at_axis(m, d, 1, 0.0)
    top = M.nodes_at_axis(m, d, 1, 1.0)
    xy = m.layers[d].node_coords[bottom]
    corner = bottom[np.abs(xy[:, 0]) < 1e-10]
    cons_d = _merge(M.component_constraints(m, d, bottom, [1], 0.0),
                    M.component_constraints(m, d, corner, [0], 0.0),
                    M.component_constraints(m, d, top, [1], 0.0, u_end))
    integ = dict(kind=GRADIENT_DAMAGE, dim=2, E=30000.0, nu=0.2, plane_state=PLANE_STRAIN,
                 damage_application=DAMAGE_FULL, kappa0=1e-4, beta=100.0, alpha=0.99, k=10.0, c=0.01, disp_slot=0,
                 eeq_slot=1)
    return Setup("notched_plate_%dx%d_depth%.3f" % (n, n, depth), m, [d, e], 2, integ, [cons_d, _empty()],
                 load_steps, 1.0)


def lognormal_cell_field(n, rng, mean=30000.0, cov=0.3, corr_length=0.1):
    """Per-cell values exp(mu + sigma g) on the n^3 cells of the unit cube (lattice order, x fastest), g a standard
    Gaussian random field at the cell centroids with correlation exp(-|x - y|^2 / (2 l^2)); sigma^2 = ln(1 + cov^2)
    and mu = ln(mean) - sigma^2 / 2 give the field the prescribed mean and coefficient of variation. The Gaussian
    correlation factorises over the axes, so g = (L_z x L_y x L_x) w with L L^T the 1D correlation matrix of the
    centroid coordinates (symmetric square root through its eigen-decomposition: the matrix is numerically
    singular for l >> 1/n) and w white noise."""
    g = gaussian_cell_field(n, rng, corr_length)
    s2 = np.log1p(cov * cov)
    return np.exp(np.log(mean) - 0.5 * s2 + np.sqrt(s2) * g).reshape(-1)


def gaussian_cell_field(n, rng, corr_length=0.1):
    """The standard Gaussian random field g of lognormal_cell_field, shape [z][y][x]."""
    x = (np.arange(n) + 0.5) / n
    C = np.exp(-((x[:, None] - x[None, :]) ** 2) / (2.0 * corr_length ** 2))
    lam, V = np.linalg.eigh(C)
    L = (V * np.sqrt(np.clip(lam, 0.0, None))) @ V.T
    w = rng.standard_normal((n, n, n))  # [z][y][x]
    return np.einsum("ck,bj,ai,kji->cba", L, L, L, w, optimize=True)


@dataclass
class AdjointCase:
    setup: Setup
    scale: np.ndarray       # per-cell E / 30000 of the field the gradient is taken at
    true_scale: np.ndarray  # per-cell E / 30000 of the synthetic truth (the target is its response)
    obs_nodes: np.ndarray   # observed displacement DOF nodes
    obs_dofs: np.ndarray    # their combined DOF indices, three per node


def hex8_adjoint(n=32, seed=0, n_obs=256, load_steps=10, u_end=5e-4):
    s = hex8_gradient_damage(n, length=1.0, u_end=u_end, load_steps=load_steps)
    s.name = "hex8_adjoint_%d^3_seed%d" % (n, seed)
    rng = np.random.default_rng(seed)
    E0 = s.integrand["E"]
    scale = lognormal_cell_field(n, rng) / E0
    true_scale = lognormal_cell_field(n, np.random.default_rng(seed + 1)) / E0
    L = s.mesh.layers[s.layers[0]]
    xyz = L.node_coords
    on_surface = np.any((np.abs(xyz) < 1e-10) | (np.abs(xyz - 1.0) < 1e-10), axis=1)
    candidates = np.flatnonzero(on_surface & (np.abs(xyz[:, 2]) >= 1e-10))
    if n_obs > candidates.size:
        raise ValueError("only %d observable surface nodes" % candidates.size)
    nodes = np.sort(rng.choice(candidates, size=n_obs, replace=False))
    dofs = L.dof_numbers[nodes].reshape(-1).astype(np.int64)
    return AdjointCase(s, scale, true_scale, nodes, dofs)
