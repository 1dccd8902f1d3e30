"""TEST INFRASTRUCTURE ONLY — the benchmark set-ups rebuilt with the oracle's restatement of NuTo's mesh code.

Mirrors nuto_gb300.configs but takes every array from the C++ restatement (UnitMeshFem generators,
AddDofInterpolation with the SubBoxes coordinate search, MeshFem::NodesAtAxis, DofNumbering::Build), so that
the tests can compare numbering and patterns bit for bit.
"""

import numpy as np

from . import core


def _component(mesh, layer, ncomp, nodes, directions, const, slope):
    dn = mesh.layer_dof_numbers(layer, ncomp)
    dofs = dn[np.asarray(nodes)[:, None], np.asarray(directions)[None, :]].ravel()
    return dofs, np.full(dofs.size, float(const)), np.full(dofs.size, float(slope))


def _cat(*parts):
    return (np.concatenate([p[0] for p in parts]), np.concatenate([p[1] for p in parts]),
            np.concatenate([p[2] for p in parts]))


def quad4_elastic(n, u_right=0.01):
    m = core.Mesh.quads(n, n)
    d = m.add_dof(2)
    integ = core.Integrand.make(core.MB_LINEAR_ELASTIC, 2, E=30000.0, nu=0.2, plane_state=core.PLANE_STRAIN)
    P = core.Problem(m, 2, [d], integ)
    cons = _cat(_component(m, d, 2, m.nodes_at_axis(d, 0, 0.0), [0, 1], 0.0, 0.0),
                _component(m, d, 2, m.nodes_at_axis(d, 0, 1.0), [0], 0.0, u_right))
    return m, [d], P, cons


def hex8_gradient_damage(n, length=4.0, u_end=2e-3, law=None):
    m = core.Mesh.bricks(n, n, n).scale(1.0, 1.0, length)
    d = m.add_dof(3)
    e = m.add_dof(1)
    params = dict(E=30000.0, nu=0.2, damage_application=core.FULL, kappa0=1e-4, beta=100.0, alpha=0.99, k=10.0,
                  c=0.01)
    params.update(law or {})
    integ = core.Integrand.make(core.GRADIENT_DAMAGE, 3, **params)
    P = core.Problem(m, 2, [d, e], integ)
    cons = _cat(_component(m, d, 3, m.nodes_at_axis(d, 2, 0.0), [0, 1, 2], 0.0, 0.0),
                _component(m, d, 3, m.nodes_at_axis(d, 2, length), [2], 0.0, u_end))
    return m, [d, e], P, cons


def hex20_local_damage(n, u_end=5e-5):
    m = core.Mesh.bricks(n, n, n)
    d = m.add_dof(3, core.HEX20)
    integ = core.Integrand.make(core.MB_LOCAL_DAMAGE, 3, E=30000.0, nu=0.2, damage_application=core.FULL,
                                kappa0=1e-4, beta=100.0, alpha=0.99, k=10.0)
    P = core.Problem(m, 3, [d], integ)
    cons = _cat(_component(m, d, 3, m.nodes_at_axis(d, 2, 0.0), [0, 1, 2], 0.0, 0.0),
                _component(m, d, 3, m.nodes_at_axis(d, 2, 1.0), [2], 0.0, u_end))
    return m, [d], P, cons


def notched_plate(n, depth=0.3, u_end=2e-4, law=None):
    """The batched workload's specimen: UnitMeshFem::CreateQuads(n, n) without the notch cells (row n // 2, the
    first round(depth n) cells of it, clamped to 1 .. n - 2), unused coordinate nodes dropped in order; 2D
    plane-strain gradient damage; bottom edge u_y = 0, corner (0, 0) u_x = 0, top edge u_y = RhsRamp(1, u_end)."""
    full = core.Mesh.quads(n, n)
    coords, conn = full.coords(2), full.conn(4)
    cells = np.arange(n * n)
    cut = (cells // n == n // 2) & (cells % n < min(max(int(round(depth * n)), 1), n - 2))
    conn = conn[~cut]
    used = np.unique(conn)
    remap = np.full(coords.shape[0], -1, dtype=np.int64)
    remap[used] = np.arange(used.size)
    m = core.Mesh.from_arrays(2, core.QUAD4, coords[used], remap[conn].astype(np.int32))
    d = m.add_dof(2)
    e = m.add_dof(1)
    params = dict(E=30000.0, nu=0.2, plane_state=core.PLANE_STRAIN, damage_application=core.FULL, kappa0=1e-4,
                  beta=100.0, alpha=0.99, k=10.0, c=0.01)
    params.update(law or {})
    integ = core.Integrand.make(core.GRADIENT_DAMAGE, 2, **params)
    P = core.Problem(m, 2, [d, e], integ)
    bottom = m.nodes_at_axis(d, 1, 0.0)
    corner = bottom[np.abs(m.layer_node_coords(d)[bottom, 0]) < 1e-10]
    cons = _cat(_component(m, d, 2, bottom, [1], 0.0, 0.0), _component(m, d, 2, corner, [0], 0.0, 0.0),
                _component(m, d, 2, m.nodes_at_axis(d, 1, 1.0), [1], 0.0, u_end))
    return m, [d, e], P, cons
