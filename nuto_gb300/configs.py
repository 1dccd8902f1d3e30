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
                   alpha = 0.99, k = 10); z = 0 face fixed, z = 1 face u_z = RhsRamp(1, 3e-4) (5 load steps).
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


def hex20_local_damage(n=80, u_end=3e-4, load_steps=5):
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
