"""Python face of the GB300 path: one cell group on one GPU behind the C ABI.

`GpuCellGroup` plays the roles of NuTo's CellStorage + SimpleAssembler + QuasistaticSolver for the supported
integrands (see include/nuto_gpu.h for the reference interface each call replaces). Device buffers are torch
CUDA tensors (plumbing only); all arithmetic runs in the library's CUDA kernels.
"""

import ctypes

import numpy as np

from . import _lib
from ._lib import (FP32, FP64, GRADIENT_DAMAGE, Integrand, MB_LINEAR_ELASTIC, MB_LOCAL_DAMAGE, Stats, StepOptions,
                   check, load)


def _ptr(a):
    if a is None:
        return None
    if isinstance(a, np.ndarray):
        return ctypes.c_void_p(a.ctypes.data)
    return ctypes.c_void_p(a.data_ptr())


def _torch():
    import torch

    return torch


class GpuCellGroup:
    def __init__(self, mesh, layers, gauss_points_per_direction=2, device=0, stream=None, dependent_counts=None):
        self.L = load()
        self.mesh = mesh
        self.device = device
        h = ctypes.c_void_p()
        if stream is None:
            # run on torch's current stream so that tensors produced by torch are ordered before our kernels
            # (handle 0 is the legacy default stream, passed as cudaStreamLegacy == 1)
            torch = _torch()
            stream = torch.cuda.current_stream(device).cuda_stream or 1
        rc = self.L.nuto_gpu_create(ctypes.byref(h), device, ctypes.c_void_p(stream))
        if rc != _lib.OK:
            msg = self.L.nuto_gpu_last_error(None)
            raise _lib.NutoGpuError(rc, "nuto_gpu_create: " + (msg.decode() if msg else ""))
        self.h = h
        self._call("nuto_gpu_set_cells", mesh.dim, mesh.geo_interp, mesh.coords.shape[0], _ptr(mesh.coords),
                   mesh.num_cells, _ptr(mesh.conn), gauss_points_per_direction)
        self.slots = []
        for k, layer in enumerate(layers):
            L = mesh.layers[layer]
            dep = 0 if dependent_counts is None else int(dependent_counts[k])
            slot = ctypes.c_int()
            dn = np.ascontiguousarray(L.dof_numbers, dtype=np.int32)
            self._call("nuto_gpu_add_dof_type", L.ncomp, L.interp, L.num_nodes, _ptr(L.conn), _ptr(dn),
                       L.num_dofs - dep, dep, ctypes.byref(slot))
            self.slots.append(slot.value)
        self.layers = list(layers)
        self.n_dofs = None
        self.nnz = None
        self.n_ip = None
        self.kind = None

    def _call(self, name, *args):
        check(self.h, getattr(self.L, name)(self.h, *args))

    def close(self):
        if getattr(self, "h", None):
            self.L.nuto_gpu_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ---- set-up --------------------------------------------------------------------------------------------
    def set_dirichlet(self, slot, dofs, rhs_const=None, rhs_slope=None):
        dofs = np.ascontiguousarray(dofs, dtype=np.int32)
        a = None if rhs_const is None else np.ascontiguousarray(rhs_const, dtype=np.float64)
        b = None if rhs_slope is None else np.ascontiguousarray(rhs_slope, dtype=np.float64)
        self._call("nuto_gpu_set_dirichlet", slot, dofs.size, _ptr(dofs), _ptr(a), _ptr(b))

    def build_pattern(self):
        n = ctypes.c_int64()
        nnz = ctypes.c_int64()
        self._call("nuto_gpu_build_pattern", ctypes.byref(n), ctypes.byref(nnz))
        self.n_dofs, self.nnz = n.value, nnz.value
        return self.n_dofs, self.nnz

    def neighbour_list_bytes(self):
        """Bytes of the per-node neighbour lists (int64 pointers, int32 neighbour columns) of every slot pair, for
        meshes whose DOF types share one node graph (every set-up here): node pairs P = nnz / (sum of components)^2."""
        layers = [self.mesh.layers[l] for l in self.layers]
        ncomp = sum(L.ncomp for L in layers)
        pairs = self.nnz // (ncomp * ncomp)
        return sum(pairs * 4 + (L.num_nodes + 1) * 8 for L in layers) * len(layers)

    def spmv(self, values, x, precision=FP64, compensated=False, out=None):
        """y = K x (FP64 vectors on the device) through nuto_gpu_spmv"""
        torch = _torch()
        x = self._dev(x, torch.float64)
        y = out if out is not None else torch.empty(self.n_dofs, dtype=torch.float64, device=x.device)
        self._call("nuto_gpu_spmv", precision, _ptr(values), _ptr(x), _ptr(y), int(bool(compensated)))
        return y

    def multigrid_info(self):
        """(levels of the first slot's hierarchy, 1 when the last sweeps ran as a CUDA graph)"""
        lv = ctypes.c_int()
        ga = ctypes.c_int()
        self._call("nuto_gpu_multigrid_info", ctypes.byref(lv), ctypes.byref(ga))
        return lv.value, ga.value

    def autotune_info(self):
        """Launch shapes the autotuner chose and the times it measured: {"tangent_warps": W, "tangent_form":
        "node_rows" | "pipelined" | "cell_matrices", "tangent_pipelined": bool, "tangent_ms": [2, 4, 8 warps],
        "tangent_pipelined_ms": [2, 4 warps], "tangent_cells_ms": [2, 4 warps], "spmv_lanes": {"f32/f32": G, ...},
        "spmv_ms": {"f32/f32": [4, 8, 16 lanes], ...}} (0: not tuned)."""
        ch = np.zeros(6, dtype=np.int32)
        ms = np.zeros(19, dtype=np.float32)
        self._call("nuto_gpu_autotune_info", _ptr(ch), _ptr(ms))
        names = ["f32/f32", "f32/f64", "f64/f32", "f64/f64"]
        forms = ["node_rows", "pipelined", "cell_matrices"]
        return {"tangent_warps": int(ch[0]), "tangent_form": forms[int(ch[1])], "tangent_pipelined": int(ch[1]) == 1,
                "tangent_ms": [float(v) for v in ms[:3]], "tangent_pipelined_ms": [float(v) for v in ms[3:5]],
                "tangent_cells_ms": [float(v) for v in ms[17:19]],
                "spmv_lanes": {k: int(ch[2 + i]) for i, k in enumerate(names)},
                "spmv_ms": {k: [float(v) for v in ms[5 + 3 * i:8 + 3 * i]] for i, k in enumerate(names)}}

    def solver_layout(self):
        """(padded values, neighbour-list entries) of the solver's copy of the tangent"""
        v = ctypes.c_int64()
        e = ctypes.c_int64()
        self._call("nuto_gpu_solver_layout", ctypes.byref(v), ctypes.byref(e))
        return v.value, e.value

    def pattern(self):
        rp = np.empty(self.n_dofs + 1, dtype=np.int64)
        ci = np.empty(self.nnz, dtype=np.int32)
        self._call("nuto_gpu_copy_pattern", _ptr(rp), _ptr(ci))
        return rp, ci

    def set_integrand(self, kind, dim, E=30000.0, nu=0.2, plane_state=_lib.PLANE_STRAIN,
                      damage_application=_lib.DAMAGE_FULL, kappa0=1e-4, beta=100.0, alpha=0.99, k=10.0, c=0.01,
                      interaction=_lib.INTERACTION_CONSTANT, R=0.005, eta=5.0, disp_slot=0, eeq_slot=-1):
        p = Integrand(kind, dim, E, nu, plane_state, damage_application, kappa0, beta, alpha, k, c, interaction, R,
                      eta, disp_slot, eeq_slot)
        self._call("nuto_gpu_set_integrand", ctypes.byref(p))
        self.kind = kind
        self.n_ip = self.L.nuto_gpu_num_integration_points(self.h)

    @property
    def history(self):
        out = np.empty((self.mesh.num_cells, self.n_ip))
        self._call("nuto_gpu_get_history", _ptr(out))
        return out

    @history.setter
    def history(self, kappa):
        k = np.ascontiguousarray(np.broadcast_to(kappa, (self.mesh.num_cells, self.n_ip)), dtype=np.float64)
        self._call("nuto_gpu_set_history", _ptr(k))

    def set_spin_limit(self, iterations):
        """Iteration limit of the bounded device waits (a wait that runs out makes synchronize() and do_step() raise
        with NUTO_GPU_ETIMEOUT)."""
        self._call("nuto_gpu_set_spin_limit", int(iterations))

    def synchronize(self):
        """Wait for the context's stream; raises with NUTO_GPU_ETIMEOUT if a bounded device wait gave up."""
        self._call("nuto_gpu_synchronize")

    def set_cell_scale(self, scale):
        """Per-cell factor of the integrand's Young's modulus (None: 1 everywhere)."""
        if scale is None:
            self._call("nuto_gpu_set_cell_scale", None)
            return
        sc = np.ascontiguousarray(scale, dtype=np.float64)
        if sc.shape != (self.mesh.num_cells,):
            raise ValueError("one factor per cell")
        self._call("nuto_gpu_set_cell_scale", _ptr(sc))

    # ---- hot path (device tensors) ---------------------------------------------------------------------------
    def _dev(self, x, dtype):
        torch = _torch()
        t = torch.as_tensor(x, dtype=dtype, device="cuda:%d" % self.device)
        return t.contiguous()

    def build_vector(self, u, out=None):
        torch = _torch()
        u = self._dev(u, torch.float64)
        f = out if out is not None else torch.empty(self.n_dofs, dtype=torch.float64, device=u.device)
        self._call("nuto_gpu_build_vector", _ptr(u), _ptr(f))
        return f

    def build_matrix(self, u, precision=FP64, out=None):
        torch = _torch()
        u = self._dev(u, torch.float64)
        dt = torch.float32 if precision == FP32 else torch.float64  # FP64 and FP64X: FP64 values
        v = out if out is not None else torch.empty(self.nnz, dtype=dt, device=u.device)
        self._call("nuto_gpu_build_matrix", _ptr(u), precision, _ptr(v))
        return v

    def build_system(self, u, precision=FP64, out=None, f_out=None):
        """(tangent CSR values, residual) at one state through nuto_gpu_build_system: the same values as
        build_matrix and build_vector, with the FP64 residual running beside the tangent on a second stream."""
        torch = _torch()
        u = self._dev(u, torch.float64)
        dt = torch.float32 if precision == FP32 else torch.float64
        v = out if out is not None else torch.empty(self.nnz, dtype=dt, device=u.device)
        f = f_out if f_out is not None else torch.empty(self.n_dofs, dtype=torch.float64, device=u.device)
        self._call("nuto_gpu_build_system", _ptr(u), precision, _ptr(v), _ptr(f))
        return v, f

    def build_system_host(self, u, values, f, precision=FP64):
        """nuto_gpu_build_system_host: u (host, n_dofs float64), values (host, nnz float32 or float64) and f (host,
        n_dofs float64) as CPU tensors or numpy arrays, page-locked for asynchronous copies (torch
        pin_memory=True). Returns when values and f hold the tangent and the residual."""
        self._call("nuto_gpu_build_system_host", _ptr(u), precision, _ptr(values), _ptr(f))
        return values, f

    def build_matrix_noalloc(self, u, out=None):
        """FP32 tangent through nuto_gpu_build_matrix_noalloc (records in the library's static device array; the
        library allocates nothing). build_matrix(u, FP32) must have run once on this group."""
        torch = _torch()
        u = self._dev(u, torch.float64)
        v = out if out is not None else torch.empty(self.nnz, dtype=torch.float32, device=u.device)
        self._call("nuto_gpu_build_matrix_noalloc", _ptr(u), _ptr(v))
        return v

    def lumped_mass(self, rho, out=None):
        """BuildDiagonallyLumpedMatrix of DynamicMomentumBalance::Hessian2 with density rho (combined layout)."""
        torch = _torch()
        dev = torch.device("cuda", self.device)
        m = out if out is not None else torch.empty(self.n_dofs, dtype=torch.float64, device=dev)
        self._call("nuto_gpu_build_lumped_mass", float(rho), _ptr(m))
        return m

    def add_boundary_cells(self, face_coord_conn, face_dof_conn, gauss=2, slot=0):
        """Boundary cells (Line2 in 2D, Quad4 in 3D) for NeumannBc loads; returns the group index."""
        fc = np.ascontiguousarray(face_coord_conn, dtype=np.int32)
        fd = np.ascontiguousarray(face_dof_conn, dtype=np.int32)
        grp = ctypes.c_int()
        self._call("nuto_gpu_add_boundary_cells", int(slot), fc.shape[0], fc.shape[1], _ptr(fc), _ptr(fd), int(gauss),
                   ctypes.byref(grp))
        return grp.value

    def external_load(self, group, traction, out=None):
        """Sum of NeumannBc::ExternalLoad over a boundary cell group (combined layout, on the device)."""
        torch = _torch()
        p = np.ascontiguousarray(traction, dtype=np.float64)
        f = out if out is not None else torch.empty(self.n_dofs, dtype=torch.float64,
                                                    device=torch.device("cuda", self.device))
        self._call("nuto_gpu_build_external_load", int(group), _ptr(p), _ptr(f))
        return f

    def set_constant_gradient(self, g):
        """A constant vector added to the residual of do_step (None removes it)."""
        torch = _torch()
        if g is None:
            self._call("nuto_gpu_set_constant_gradient", None)
            return
        g = self._dev(g, torch.float64)
        self._call("nuto_gpu_set_constant_gradient", _ptr(g))
        torch.cuda.synchronize()

    def eval_ip(self, u, quantity):
        """Cell::Eval of an IP_* quantity at every integration point: (n_cells, n_ip, width) on the device."""
        torch = _torch()
        u = self._dev(u, torch.float64)
        w = (3 if self.mesh.dim == 2 else 6) if quantity in (_lib.IP_STRAIN, _lib.IP_STRESS) else 1
        out = torch.empty((self.mesh.num_cells, self.n_ip, w), dtype=torch.float64, device=u.device)
        self._call("nuto_gpu_eval_ip", _ptr(u), int(quantity), _ptr(out))
        return out

    def update_history(self, u):
        torch = _torch()
        u = self._dev(u, torch.float64)
        self._call("nuto_gpu_update_history", _ptr(u))

    def assemble_cell_vectors(self, fe):
        torch = _torch()
        fe = self._dev(fe, torch.float64)
        f = torch.empty(self.n_dofs, dtype=torch.float64, device=fe.device)
        self._call("nuto_gpu_assemble_cell_vectors", _ptr(fe), _ptr(f))
        return f

    def assemble_cell_matrices(self, ke, precision=FP64):
        torch = _torch()
        ke = self._dev(ke, torch.float64)
        dt = torch.float32 if precision == FP32 else torch.float64
        v = torch.empty(self.nnz, dtype=dt, device=ke.device)
        self._call("nuto_gpu_assemble_cell_matrices", _ptr(ke), precision, _ptr(v))
        return v

    def solve(self, values, b, precision=FP64, method=_lib.SOLVER_AUTO, rtol=1e-10, max_iterations=100000):
        torch = _torch()
        b = self._dev(b, torch.float64)
        x = torch.empty_like(b)
        it = ctypes.c_int()
        rel = ctypes.c_double()
        rc = self.L.nuto_gpu_solve(self.h, precision, method, _ptr(values), _ptr(b), _ptr(x), rtol, max_iterations,
                                   ctypes.byref(it), ctypes.byref(rel))
        if rc not in (_lib.OK, _lib.ENOCONV):
            check(self.h, rc)
        return x, it.value, rel.value, rc == _lib.OK

    def set_preconditioner(self, kind):
        """PRECOND_JACOBI or PRECOND_AMG (default) for the PCG and GMRES solves of solve() and do_step()."""
        self._call("nuto_gpu_set_preconditioner", int(kind))

    # ---- quasistatic driver --------------------------------------------------------------------------------
    @staticmethod
    def default_options(**kw):
        o = StepOptions()
        load().nuto_gpu_default_step_options(ctypes.byref(o))
        for k, v in kw.items():
            setattr(o, k, v)
        return o

    def set_state(self, x=None, time=0.0, reset_history=True):
        xa = None if x is None else np.ascontiguousarray(x, dtype=np.float64)
        self._call("nuto_gpu_set_state", _ptr(xa), float(time), int(bool(reset_history)))

    def get_state(self):
        x = np.empty(self.n_dofs)
        t = ctypes.c_double()
        self._call("nuto_gpu_get_state", _ptr(x), ctypes.byref(t))
        return x, t.value

    def state_device(self):
        p = ctypes.c_void_p()
        self._call("nuto_gpu_state_device", ctypes.byref(p))
        return p.value

    def do_step(self, t_new, options=None):
        o = options if options is not None else self.default_options()
        it = ctypes.c_int()
        self._call("nuto_gpu_do_step", float(t_new), ctypes.byref(o), ctypes.byref(it))
        return it.value

    def do_step_host(self, t_new, x_in, kappa_in, x_out, kappa_out, options=None):
        o = options if options is not None else self.default_options()
        it = ctypes.c_int()
        self._call("nuto_gpu_do_step_host", float(t_new), ctypes.byref(o), _ptr(x_in), _ptr(kappa_in), _ptr(x_out),
                   _ptr(kappa_out), ctypes.byref(it))
        return it.value

    def stats(self):
        s = Stats()
        check(self.h, self.L.nuto_gpu_get_stats(self.h, ctypes.byref(s)))
        return s.as_dict()

