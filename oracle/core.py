"""TEST INFRASTRUCTURE ONLY — ctypes wrapper around the oracle's C entry points (oracle_capi.cpp).

The C++ restatement follows the reference file:line citations given in nuto_oracle.hpp.
"""

import ctypes
import os
import subprocess
import threading

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
LIB_PATH = os.path.join(BUILD_DIR, "liboracle.so")

QUAD4, HEX8, HEX20 = 0, 1, 2
PLANE_STRESS, PLANE_STRAIN = 0, 1
FULL, UNILATERAL = 0, 1
MB_LINEAR_ELASTIC, MB_LOCAL_DAMAGE, GRADIENT_DAMAGE = 0, 1, 2

_lock = threading.Lock()
_lib = None


def build(force=False):
    """Compile the oracle restatement with g++ (OpenMP, no architecture-specific flags)."""
    os.makedirs(BUILD_DIR, exist_ok=True)
    src = [os.path.join(HERE, "oracle_capi.cpp"), os.path.join(HERE, "nuto_oracle.hpp")]
    if not force and os.path.exists(LIB_PATH):
        if os.path.getmtime(LIB_PATH) >= max(os.path.getmtime(s) for s in src):
            return LIB_PATH
    tmp = LIB_PATH + ".tmp.%d" % os.getpid()
    cmd = ["g++", "-O2", "-std=c++17", "-fopenmp", "-fPIC", "-shared", src[0], "-o", tmp]
    subprocess.check_call(cmd)
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


class Integrand(ctypes.Structure):
    """IntegrandParams (nuto_oracle.hpp): integrand kind plus law parameters."""

    _fields_ = [
        ("kind", ctypes.c_int),
        ("dim", ctypes.c_int),
        ("E", ctypes.c_double),
        ("nu", ctypes.c_double),
        ("plane_state", ctypes.c_int),
        ("damage_application", ctypes.c_int),
        ("kappa0", ctypes.c_double),
        ("beta", ctypes.c_double),
        ("alpha", ctypes.c_double),
        ("k", ctypes.c_double),
        ("c", ctypes.c_double),
        ("interaction", ctypes.c_int),
        ("R", ctypes.c_double),
        ("eta", ctypes.c_double),
    ]

    @classmethod
    def make(cls, kind, dim, E=30000.0, nu=0.2, plane_state=PLANE_STRAIN, damage_application=FULL,
             kappa0=1e-4, beta=100.0, alpha=0.99, k=10.0, c=0.01, interaction=0, R=0.005, eta=5.0):
        return cls(kind, dim, E, nu, plane_state, damage_application, kappa0, beta, alpha, k, c,
                   interaction, R, eta)


def lib():
    global _lib
    with _lock:
        if _lib is None:
            build()
            L = ctypes.CDLL(LIB_PATH)
            vp, i, d, ll = ctypes.c_void_p, ctypes.c_int, ctypes.c_double, ctypes.c_longlong
            P = ctypes.POINTER
            sig = {
                "oracle_mesh_quads": (vp, [i, i]),
                "oracle_mesh_bricks": (vp, [i, i, i]),
                "oracle_mesh_from_arrays": (vp, [i, i, i, P(d), i, P(i)]),
                "oracle_mesh_scale": (None, [vp, d, d, d]),
                "oracle_mesh_free": (None, [vp]),
                "oracle_mesh_num_elements": (i, [vp]),
                "oracle_mesh_num_coord_nodes": (i, [vp]),
                "oracle_mesh_coords": (None, [vp, P(d)]),
                "oracle_mesh_conn": (None, [vp, P(i)]),
                "oracle_mesh_add_dof": (i, [vp, i, i]),
                "oracle_layer_num_nodes": (i, [vp, i]),
                "oracle_layer_nen": (i, [vp, i]),
                "oracle_layer_conn": (None, [vp, i, P(i)]),
                "oracle_layer_node_coords": (None, [vp, i, P(d)]),
                "oracle_layer_dof_numbers": (None, [vp, i, P(i)]),
                "oracle_nodes_at_axis": (i, [vp, i, i, d, P(i)]),
                "oracle_problem_create": (vp, [vp, i, i, P(i), P(Integrand)]),
                "oracle_problem_free": (None, [vp]),
                "oracle_problem_num_dofs": (ll, [vp]),
                "oracle_problem_num_ips": (i, [vp]),
                "oracle_problem_set_kappa": (None, [vp, P(d)]),
                "oracle_problem_get_kappa": (None, [vp, P(d)]),
                "oracle_build_vector": (None, [vp, P(d), P(d)]),
                "oracle_build_matrix": (ll, [vp, P(d)]),
                "oracle_matrix_copy": (None, [vp, P(ll), P(i), P(d)]),
                "oracle_matrix_release": (None, [vp]),
                "oracle_update_history": (None, [vp, P(d)]),
                "oracle_lumped_mass": (None, [vp, d, P(d)]),
                "oracle_lump_hrz": (None, [P(d), i, i, P(d)]),
                "oracle_ip_width": (i, [vp, i]),
                "oracle_eval_ip": (None, [vp, P(d), i, P(d)]),
                "oracle_external_load": (None, [vp, i, i, P(i), P(ll), P(d), i, P(d)]),
                "oracle_neumann_ip": (None, [i, i, P(d), P(d), P(d)]),
                "oracle_cell_nlocal": (i, [vp]),
                "oracle_cell_dofs": (None, [vp, i, P(ll)]),
                "oracle_cell_integrate": (None, [vp, i, P(d), P(d), P(d)]),
                "oracle_cell_volume": (d, [vp, i]),
                "oracle_problem_set_e_scale": (None, [vp, P(d)]),
                "oracle_cell_adjoint": (i, [vp, i, P(d), P(d), P(d), P(d)]),
                "oracle_quadrature": (None, [i, i, P(d), P(d)]),
                "oracle_shape": (None, [i, P(d), P(d), P(d)]),
                "oracle_set_threads": (None, [i]),
                "oracle_max_threads": (i, []),
                "oracle_linear_elastic_C": (None, [i, d, d, i, P(d)]),
                "oracle_led": (None, [i, d, d, i, i, P(d), d, P(d), P(d), P(d)]),
                "oracle_mises": (d, [i, d, d, i, P(d), P(d)]),
                "oracle_damage_exp": (None, [d, d, d, d, P(d), P(d)]),
                "oracle_local_damage": (None, [i, d, d, i, i, d, d, d, d, d, P(d), P(d), P(d)]),
            }
            for name, (res, args) in sig.items():
                fn = getattr(L, name)
                fn.restype = res
                fn.argtypes = args
            _lib = L
    return _lib


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _ip(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int))


def _llp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_longlong))


class Mesh:
    """MeshFem restatement: UnitMeshFem generators, Transform, AddDofInterpolation, NodesAtAxis."""

    def __init__(self, handle):
        self.h = handle
        self.L = lib()

    @classmethod
    def quads(cls, nx, ny):
        return cls(lib().oracle_mesh_quads(nx, ny))

    @classmethod
    def bricks(cls, nx, ny, nz):
        return cls(lib().oracle_mesh_bricks(nx, ny, nz))

    @classmethod
    def from_arrays(cls, dim, geo_interp, coords, conn):
        coords = np.ascontiguousarray(coords, dtype=np.float64)
        conn = np.ascontiguousarray(conn, dtype=np.int32)
        n_nodes = coords.size // dim
        return cls(lib().oracle_mesh_from_arrays(dim, geo_interp, n_nodes, _dp(coords), conn.shape[0], _ip(conn)))

    def scale(self, sx, sy, sz=1.0):
        self.L.oracle_mesh_scale(self.h, sx, sy, sz)
        return self

    def external_load(self, n_dofs, face_coord_conn, face_dofs, traction, gauss=2):
        """SimpleAssembler::BuildVector of NeumannBc::ExternalLoad over boundary cells (Line2 in 2D, Quad4 in 3D):
        face_coord_conn (n_faces, nfe) coordinate nodes, face_dofs (n_faces, nfe, dim) combined DOF indices."""
        fc = np.ascontiguousarray(face_coord_conn, dtype=np.int32)
        fd = np.ascontiguousarray(face_dofs, dtype=np.int64)
        p = np.ascontiguousarray(traction, dtype=np.float64)
        f = np.zeros(n_dofs)
        self.L.oracle_external_load(self.h, fc.shape[1], fc.shape[0], _ip(fc), _llp(fd), _dp(p), gauss, _dp(f))
        return f

    def __del__(self):
        try:
            if self.h:
                self.L.oracle_mesh_free(self.h)
                self.h = None
        except Exception:
            pass

    @property
    def num_elements(self):
        return self.L.oracle_mesh_num_elements(self.h)

    def coords(self, dim):
        n = self.L.oracle_mesh_num_coord_nodes(self.h)
        out = np.empty(n * dim)
        self.L.oracle_mesh_coords(self.h, _dp(out))
        return out.reshape(n, dim)

    def conn(self, nen):
        out = np.empty(self.num_elements * nen, dtype=np.int32)
        self.L.oracle_mesh_conn(self.h, _ip(out))
        return out.reshape(-1, nen)

    def add_dof(self, ncomp, interp=-1):
        layer = self.L.oracle_mesh_add_dof(self.h, ncomp, interp)
        if layer < 0:
            raise ValueError("AddDofInterpolation failed")
        return layer

    def layer_num_nodes(self, layer):
        return self.L.oracle_layer_num_nodes(self.h, layer)

    def layer_conn(self, layer):
        nen = self.L.oracle_layer_nen(self.h, layer)
        out = np.empty(self.num_elements * nen, dtype=np.int32)
        self.L.oracle_layer_conn(self.h, layer, _ip(out))
        return out.reshape(-1, nen)

    def layer_nen(self, layer):
        return self.L.oracle_layer_nen(self.h, layer)

    def layer_node_coords(self, layer):
        n = self.layer_num_nodes(layer)
        out = np.empty(n * 3)
        self.L.oracle_layer_node_coords(self.h, layer, _dp(out))
        return out.reshape(n, 3)

    def layer_dof_numbers(self, layer, ncomp):
        n = self.layer_num_nodes(layer)
        out = np.empty(n * ncomp, dtype=np.int32)
        self.L.oracle_layer_dof_numbers(self.h, layer, _ip(out))
        return out.reshape(n, ncomp)

    def nodes_at_axis(self, layer, direction, offset=0.0):
        n = self.L.oracle_nodes_at_axis(self.h, layer, direction, offset, None)
        out = np.empty(max(n, 1), dtype=np.int32)
        self.L.oracle_nodes_at_axis(self.h, layer, direction, offset, _ip(out))
        return out[:n]


class Problem:
    """Cells + integrand + history; BuildVector/BuildMatrix/UpdateHistory restated."""

    def __init__(self, mesh, ips_per_dir, slots, integrand):
        self.mesh = mesh  # keep alive
        self.L = lib()
        self.slots = [int(x) for x in slots]
        slots = np.ascontiguousarray(slots, dtype=np.int32)
        self.integrand = integrand
        self.h = self.L.oracle_problem_create(mesh.h, ips_per_dir, len(slots), _ip(slots), ctypes.byref(integrand))
        self.n_dofs = int(self.L.oracle_problem_num_dofs(self.h))
        self.n_ip = self.L.oracle_problem_num_ips(self.h)
        self.n_el = mesh.num_elements
        self.n_local = self.L.oracle_cell_nlocal(self.h)

    def __del__(self):
        try:
            if self.h:
                self.L.oracle_problem_free(self.h)
                self.h = None
        except Exception:
            pass

    @property
    def kappa(self):
        out = np.empty(self.n_el * self.n_ip)
        self.L.oracle_problem_get_kappa(self.h, _dp(out))
        return out.reshape(self.n_el, self.n_ip)

    @kappa.setter
    def kappa(self, value):
        v = np.ascontiguousarray(np.broadcast_to(value, (self.n_el, self.n_ip)), dtype=np.float64)
        self.L.oracle_problem_set_kappa(self.h, _dp(v))

    def build_vector(self, u):
        u = np.ascontiguousarray(u, dtype=np.float64)
        f = np.empty(self.n_dofs)
        self.L.oracle_build_vector(self.h, _dp(u), _dp(f))
        return f

    def build_matrix(self):
        raise NotImplementedError

    def build_matrix_csc(self, u):
        """Returns (col_ptr int64, row_idx int32, values float64) of the combined matrix."""
        u = np.ascontiguousarray(u, dtype=np.float64)
        nnz = int(self.L.oracle_build_matrix(self.h, _dp(u)))
        col_ptr = np.empty(self.n_dofs + 1, dtype=np.int64)
        row_idx = np.empty(nnz, dtype=np.int32)
        vals = np.empty(nnz)
        self.L.oracle_matrix_copy(self.h, _llp(col_ptr), _ip(row_idx), _dp(vals))
        self.L.oracle_matrix_release(self.h)
        return col_ptr, row_idx, vals

    def build_matrix_scipy(self, u):
        import scipy.sparse as sp

        col_ptr, row_idx, vals = self.build_matrix_csc(u)
        return sp.csc_matrix((vals, row_idx, col_ptr), shape=(self.n_dofs, self.n_dofs))

    def update_history(self, u):
        u = np.ascontiguousarray(u, dtype=np.float64)
        self.L.oracle_update_history(self.h, _dp(u))

    def lumped_mass(self, rho):
        """BuildDiagonallyLumpedMatrix of DynamicMomentumBalance::Hessian2 (combined layout)."""
        m = np.empty(self.n_dofs)
        self.L.oracle_lumped_mass(self.h, float(rho), _dp(m))
        return m

    def eval_ip(self, u, quantity):
        """Cell::Eval of IP_KAPPA / IP_DAMAGE / IP_STRAIN / IP_STRESS / IP_EEQ: (n_el, n_ip, width)."""
        u = np.ascontiguousarray(u, dtype=np.float64)
        w = int(self.L.oracle_ip_width(self.h, quantity))
        out = np.empty((self.n_el, self.n_ip, w))
        self.L.oracle_eval_ip(self.h, _dp(u), quantity, _dp(out))
        return out

    def cell_dofs(self, cell):
        out = np.empty(self.n_local, dtype=np.int64)
        self.L.oracle_cell_dofs(self.h, cell, _llp(out))
        return out

    def cell_integrate(self, cell, u):
        u = np.ascontiguousarray(u, dtype=np.float64)
        fe = np.empty(self.n_local)
        Ke = np.empty(self.n_local * self.n_local)
        self.L.oracle_cell_integrate(self.h, cell, _dp(u), _dp(fe), _dp(Ke))
        return fe, Ke.reshape(self.n_local, self.n_local)

    def set_e_scale(self, scale):
        """Per-cell Young's modulus as multiples of the integrand's E (None: 1 everywhere)."""
        if scale is None:
            self.L.oracle_problem_set_e_scale(self.h, None)
            return
        self._e_scale = np.ascontiguousarray(scale, dtype=np.float64).reshape(self.n_el)
        self.L.oracle_problem_set_e_scale(self.h, _dp(self._e_scale))

    def cell_adjoint(self, cell, u):
        """Gradient damage: (D [n_local, n_ip] = d f_cell / d omega_ip, ipd [n_ip, 5] = kappa_trial, loading flag,
        d omega/d kappa, d omega/d kappa0, d omega/d beta; N [n_ip, n_eeq_nodes] eeq shape values)."""
        if self.integrand.kind != GRADIENT_DAMAGE:
            raise ValueError("adjoint data exist for gradient damage only")
        u = np.ascontiguousarray(u, dtype=np.float64)
        ne = self.mesh.layer_nen(self.slots[1])
        D = np.empty(self.n_local * self.n_ip)
        ipd = np.empty(self.n_ip * 5)
        N = np.empty(self.n_ip * ne)
        self.L.oracle_cell_adjoint(self.h, cell, _dp(u), _dp(D), _dp(ipd), _dp(N))
        return D.reshape(self.n_local, self.n_ip), ipd.reshape(self.n_ip, 5), N.reshape(self.n_ip, ne)

    def cell_volume(self, cell):
        return self.L.oracle_cell_volume(self.h, cell)


def quadrature(dim, n):
    num = n ** dim
    pts = np.empty(num * dim)
    w = np.empty(num)
    lib().oracle_quadrature(dim, n, _dp(pts), _dp(w))
    return pts.reshape(num, dim), w


def shape(interp, xi):
    nn = {QUAD4: 4, HEX8: 8, HEX20: 20}[interp]
    x = np.zeros(3)
    x[: len(xi)] = xi
    N = np.empty(20)
    dN = np.empty(60)
    lib().oracle_shape(interp, _dp(x), _dp(N), _dp(dN))
    return N[:nn], dN.reshape(20, 3)[:nn]


def linear_elastic_C(dim, E, nu, plane_state):
    vd = {1: 1, 2: 3, 3: 6}[dim]
    out = np.empty(vd * vd)
    lib().oracle_linear_elastic_C(dim, E, nu, plane_state, _dp(out))
    return out.reshape(vd, vd)


def linear_elastic_damage(dim, E, nu, app, plane_state, strain, omega):
    vd = {1: 1, 2: 3, 3: 6}[dim]
    strain = np.ascontiguousarray(strain, dtype=np.float64)
    s = np.empty(vd)
    dsde = np.empty(vd * vd)
    dsdw = np.empty(vd)
    lib().oracle_led(dim, E, nu, app, plane_state, _dp(strain), omega, _dp(s), _dp(dsde), _dp(dsdw))
    return s, dsde.reshape(vd, vd), dsdw


def mises(dim, nu, k, plane_state, strain):
    vd = {1: 1, 2: 3, 3: 6}[dim]
    strain = np.ascontiguousarray(strain, dtype=np.float64)
    d = np.empty(vd)
    v = lib().oracle_mises(dim, nu, k, plane_state, _dp(strain), _dp(d))
    return v, d


def damage_exponential(kappa0, beta, alpha, kappa):
    o = ctypes.c_double()
    do = ctypes.c_double()
    lib().oracle_damage_exp(kappa0, beta, alpha, kappa, ctypes.byref(o), ctypes.byref(do))
    return o.value, do.value


def local_damage(dim, E, nu, app, plane_state, kappa0, beta, alpha, k, kappa_hist, strain):
    vd = {1: 1, 2: 3, 3: 6}[dim]
    strain = np.ascontiguousarray(strain, dtype=np.float64)
    s = np.empty(vd)
    t = np.empty(vd * vd)
    lib().oracle_local_damage(dim, E, nu, app, plane_state, kappa0, beta, alpha, k, kappa_hist, _dp(strain), _dp(s),
                              _dp(t))
    return s, t.reshape(vd, vd)


IP_KAPPA, IP_DAMAGE, IP_STRAIN, IP_STRESS, IP_EEQ = 0, 1, 2, 3, 4


def lump_hrz(M, ncomp):
    """SimpleAssembler::BuildDiagonallyLumpedMatrix of one local block (SimpleAssembler.cpp:83-87)."""
    M = np.ascontiguousarray(M, dtype=np.float64)
    nl = M.shape[0]
    out = np.empty(nl)
    lib().oracle_lump_hrz(_dp(M), nl, ncomp, _dp(out))
    return out


def neumann_ip(nfe, dim, xi, traction):
    """NeumannBc::ExternalLoad at one natural point of a boundary cell: N^T p, node-major."""
    x = np.ascontiguousarray(np.atleast_1d(xi), dtype=np.float64)
    p = np.ascontiguousarray(traction, dtype=np.float64)
    out = np.empty(nfe * dim)
    lib().oracle_neumann_ip(nfe, dim, _dp(x), _dp(p), _dp(out))
    return out

