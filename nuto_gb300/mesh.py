"""Structured meshes, DOF layers and Dirichlet selections with NuTo's numbering, vectorised with numpy.

This is the input side of the hot path: it produces exactly the arrays NuTo's own classes would hand to the
GPU path (coordinate connectivity of the cells, DOF-node connectivity and DOF numbers):

- UnitMeshFem::CreateQuads / CreateBricks / Transform (nuto/mechanics/mesh/UnitMeshFem.cpp:36-125): lattice
  node order with x fastest, cells in lattice order.
- AddDofInterpolation (nuto/mechanics/mesh/MeshFemDofConvert.cpp:164-218): DOF nodes are created in
  first-touch order of the cells and their local nodes; coincident nodes are shared. The reference finds
  coincident nodes by coordinates; here they are identified by the coordinate nodes they sit on (a corner) or
  between (a Hex20 edge node), which is the same relation on a conforming mesh.
- DofNumbering::Build over MeshFem::NodesTotal(dof) (nuto/mechanics/dofs/DofNumbering.cpp:7-58): consecutive
  numbers per node and component in first-touch order.
- MeshFem::NodesAtAxis (nuto/mechanics/mesh/MeshFem.cpp:72-93) and Constraint::Component
  (nuto/mechanics/constraints/ConstraintCompanion.cpp:20-42): first-touch node order, one equation per node and
  direction.
"""

import numpy as np

from ._lib import HEX8, HEX20, QUAD4

NUM_NODES = {QUAD4: 4, HEX8: 8, HEX20: 20}
INTERP_DIM = {QUAD4: 2, HEX8: 3, HEX20: 3}

# local corner pairs of the 12 edge nodes of InterpolationBrickQuadratic (local nodes 8..19)
HEX20_EDGES = np.array([[0, 1], [1, 2], [3, 2], [0, 3], [0, 4], [1, 5], [2, 6], [3, 7], [4, 5], [5, 6], [7, 6],
                        [4, 7]], dtype=np.int64)


class MeshFem:
    """Coordinate nodes + cells (coordinate elements) + DOF layers."""

    def __init__(self, dim, geo_interp, coords, conn):
        self.dim = dim
        self.geo_interp = geo_interp
        self.coords = np.ascontiguousarray(coords, dtype=np.float64).reshape(-1, dim)
        self.conn = np.ascontiguousarray(conn, dtype=np.int32).reshape(-1, NUM_NODES[geo_interp])
        self.layers = []

    @property
    def num_cells(self):
        return self.conn.shape[0]

    def transform(self, f):
        """UnitMeshFem::Transform with a vectorised map coords[n, dim] -> coords[n, dim]."""
        self.coords = np.ascontiguousarray(f(self.coords.copy()), dtype=np.float64)
        return self

    def scale(self, *factors):
        return self.transform(lambda x: x * np.asarray(factors[: self.dim], dtype=np.float64))


class DofLayer:
    def __init__(self, ncomp, interp, conn, node_coords):
        self.ncomp = ncomp
        self.interp = interp
        self.conn = np.ascontiguousarray(conn, dtype=np.int32)
        self.node_coords = node_coords
        self.num_nodes = node_coords.shape[0]
        self.dof_numbers = np.arange(self.num_nodes * ncomp, dtype=np.int32).reshape(self.num_nodes, ncomp)
        self.num_dofs = self.num_nodes * ncomp


def create_quads(nx, ny):
    iy, ix = np.meshgrid(np.arange(ny + 1), np.arange(nx + 1), indexing="ij")
    coords = np.stack([ix.ravel() / nx, iy.ravel() / ny], axis=1)
    ey, ex = np.meshgrid(np.arange(ny), np.arange(nx), indexing="ij")
    b = (ex + ey * (nx + 1)).ravel()
    conn = np.stack([b, b + 1, b + 1 + (nx + 1), b + (nx + 1)], axis=1)
    return MeshFem(2, QUAD4, coords, conn)


def create_bricks(nx, ny, nz):
    X, Y = nx + 1, ny + 1
    iz, iy, ix = np.meshgrid(np.arange(nz + 1), np.arange(ny + 1), np.arange(nx + 1), indexing="ij")
    coords = np.stack([ix.ravel() / nx, iy.ravel() / ny, iz.ravel() / nz], axis=1)
    ez, ey, ex = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    b = (ex + ey * X + ez * X * Y).ravel()
    u = b + X * Y
    conn = np.stack([b, b + 1, b + 1 + X, b + X, u, u + 1, u + 1 + X, u + X], axis=1)
    return MeshFem(3, HEX8, coords, conn)


def add_dof_interpolation(mesh, ncomp, interp=None):
    """Adds a DOF layer; returns its index in mesh.layers."""
    if interp is None:
        interp = mesh.geo_interp
    if INTERP_DIM[interp] != mesh.dim:
        raise ValueError("Shape of interpolation and coordinate element don't match.")
    ng = mesh.coords.shape[0]
    geo = mesh.conn.astype(np.int64)
    if interp == mesh.geo_interp:
        keys = geo
    elif interp == HEX20 and mesh.geo_interp == HEX8:
        a = geo[:, HEX20_EDGES[:, 0]]
        b = geo[:, HEX20_EDGES[:, 1]]
        edge = ng + np.minimum(a, b) * ng + np.maximum(a, b)
        keys = np.concatenate([geo, edge], axis=1)
    else:
        raise ValueError("unsupported interpolation on this coordinate mesh")
    flat = keys.ravel()
    uniq, first, inverse = np.unique(flat, return_index=True, return_inverse=True)
    order = np.argsort(first, kind="stable")
    rank = np.empty_like(order)
    rank[order] = np.arange(order.size)
    conn = rank[inverse.ravel()].reshape(keys.shape)
    # coordinates of the DOF nodes (Interpolate(coordinateElement, localCoords))
    ukeys = uniq[order]
    coords3 = np.zeros((ukeys.size, 3))
    corner = ukeys < ng
    coords3[corner, : mesh.dim] = mesh.coords[ukeys[corner]]
    if (~corner).any():
        e = ukeys[~corner] - ng
        lo, hi = e // ng, e % ng
        coords3[~corner, : mesh.dim] = 0.5 * (mesh.coords[lo] + mesh.coords[hi])
    mesh.layers.append(DofLayer(ncomp, interp, conn, coords3))
    return len(mesh.layers) - 1


def nodes_at_axis(mesh, layer, direction, offset=0.0, tol=1e-10):
    """MeshFem::NodesAtAxis(direction, dof, offset): DOF nodes with |x_dir - offset| < tol in first-touch order."""
    L = mesh.layers[layer]
    flat = L.conn.ravel()
    hit = np.abs(L.node_coords[flat, direction] - offset) < tol
    cand = flat[hit]
    _, first = np.unique(cand, return_index=True)
    return cand[np.sort(first)]


def component_constraints(mesh, layer, nodes, directions, rhs_const=0.0, rhs_slope=0.0):
    """Constraint::Component(nodes, directions, rhs): (dependent DOF numbers, rhs_const, rhs_slope) per equation.

    rhs(t) = rhs_const + rhs_slope * t covers RhsConstant (slope 0) and RhsRamp(1, value) (slope = value).
    """
    L = mesh.layers[layer]
    dofs = L.dof_numbers[np.asarray(nodes)[:, None], np.asarray(directions)[None, :]].ravel()
    n = dofs.size
    return (dofs.astype(np.int32), np.full(n, float(rhs_const)), np.full(n, float(rhs_slope)))


# local node lists of the faces of the linear cells, each a valid Line2 / Quad4 order
QUAD4_EDGES = np.array([[0, 1], [1, 2], [3, 2], [0, 3]], dtype=np.int64)
HEX8_FACES = np.array([[0, 1, 2, 3], [4, 5, 6, 7], [0, 3, 7, 4], [1, 2, 6, 5], [0, 1, 5, 4], [3, 2, 6, 7]],
                      dtype=np.int64)


def boundary_faces(mesh, layer, direction, offset, tol=1e-10):
    """Boundary cells on the plane x_direction = offset (edges of Quad4 meshes, faces of Hex8 meshes) in cell order:
    (coordinate connectivity, DOF-node connectivity of the layer), both n_faces x nodes-per-face. The layer must use
    the coordinate interpolation (the DOF nodes of a face are the face's coordinate nodes)."""
    L = mesh.layers[layer]
    faces = QUAD4_EDGES if mesh.geo_interp == QUAD4 else HEX8_FACES
    geo = mesh.conn[:, faces]   # cells x faces x nodes-per-face
    dof = L.conn[:, faces]
    on = np.all(np.abs(mesh.coords[geo, direction] - offset) < tol, axis=2)
    cells, which = np.nonzero(on)
    return (np.ascontiguousarray(geo[cells, which], dtype=np.int32),
            np.ascontiguousarray(dof[cells, which], dtype=np.int32))

