"""ctypes binding of the C ABI in include/nuto_gpu.h (libnuto_gb300.so, built in-tree by nuto_gb300/build.py).

There is no fallback: if the CUDA library cannot be built or loaded, every call raises.
"""

import ctypes
import os
import threading

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "lib", "libnuto_gb300.so")

OK, EINVAL, ENOMEM, ENOCONV, ENAN, ETIMEOUT, ECUDA, ESTATE = range(8)
QUAD4, HEX8, HEX20 = 0, 1, 2
MB_LINEAR_ELASTIC, MB_LOCAL_DAMAGE, GRADIENT_DAMAGE = 0, 1, 2
PLANE_STRESS, PLANE_STRAIN = 0, 1
DAMAGE_FULL, DAMAGE_UNILATERAL = 0, 1
INTERACTION_CONSTANT, INTERACTION_DECREASING = 0, 1
FP32, FP64, MIXED, FP64X = 32, 64, 48, 65
SOLVER_AUTO, SOLVER_PCG, SOLVER_BICGSTAB, SOLVER_GMRES = 0, 1, 2, 3
PRECOND_JACOBI, PRECOND_AMG = 1, 2
IP_KAPPA, IP_DAMAGE, IP_STRAIN, IP_STRESS, IP_EEQ = 0, 1, 2, 3, 4

_ERRNAMES = {EINVAL: "EINVAL", ENOMEM: "ENOMEM", ENOCONV: "ENOCONV", ENAN: "ENAN", ETIMEOUT: "ETIMEOUT",
             ECUDA: "ECUDA", ESTATE: "ESTATE"}


class NutoGpuError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("%s: %s" % (_ERRNAMES.get(code, str(code)), msg))
        self.code = code


class NoConvergence(NutoGpuError):
    """NewtonRaphson::NoConvergence (nuto/math/NewtonRaphson.h:13-20)."""


class Integrand(ctypes.Structure):
    _fields_ = [
        ("kind", ctypes.c_int), ("dim", ctypes.c_int), ("E", ctypes.c_double), ("nu", ctypes.c_double),
        ("plane_state", ctypes.c_int), ("damage_application", ctypes.c_int), ("kappa0", ctypes.c_double),
        ("beta", ctypes.c_double), ("alpha", ctypes.c_double), ("k", ctypes.c_double), ("c", ctypes.c_double),
        ("interaction", ctypes.c_int), ("R", ctypes.c_double), ("eta", ctypes.c_double),
        ("disp_slot", ctypes.c_int), ("eeq_slot", ctypes.c_int),
    ]


class StepOptions(ctypes.Structure):
    _fields_ = [
        ("precision", ctypes.c_int), ("method", ctypes.c_int), ("newton_rtol", ctypes.c_double),
        ("newton_atol", ctypes.c_double), ("max_newton", ctypes.c_int), ("line_search", ctypes.c_int),
        ("krylov_rtol", ctypes.c_double), ("max_krylov", ctypes.c_int), ("forcing", ctypes.c_int),
        ("exact_tangent_below", ctypes.c_double), ("forcing_floor", ctypes.c_double),
    ]


class Stats(ctypes.Structure):
    _fields_ = [
        ("newton_iterations", ctypes.c_int), ("krylov_iterations", ctypes.c_int),
        ("residual_evaluations", ctypes.c_int), ("matrix_assemblies", ctypes.c_int),
        ("final_residual", ctypes.c_double), ("reference_residual", ctypes.c_double),
        ("ms_assemble_matrix", ctypes.c_double), ("ms_assemble_vector", ctypes.c_double),
        ("ms_krylov", ctypes.c_double), ("ms_total", ctypes.c_double), ("ms_spmv", ctypes.c_double),
        ("spmv_launches", ctypes.c_int64), ("kernel_launches", ctypes.c_int64),
    ]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}


# every exported symbol of include/nuto_gpu.h with its ctypes signature
_vp, _i, _d, _i64 = ctypes.c_void_p, ctypes.c_int, ctypes.c_double, ctypes.c_int64
_P = ctypes.POINTER
SIGNATURES = {
    "nuto_gpu_version": (_i, []),
    "nuto_gpu_create": (_i, [_P(_vp), _i, _vp]),
    "nuto_gpu_destroy": (_i, [_vp]),
    "nuto_gpu_last_error": (ctypes.c_char_p, [_vp]),
    "nuto_gpu_synchronize": (_i, [_vp]),
    "nuto_gpu_set_cells": (_i, [_vp, _i, _i, _i64, _vp, _i64, _vp, _i]),
    "nuto_gpu_add_dof_type": (_i, [_vp, _i, _i, _i64, _vp, _vp, _i64, _i64, _P(_i)]),
    "nuto_gpu_set_dirichlet": (_i, [_vp, _i, _i64, _vp, _vp, _vp]),
    "nuto_gpu_build_pattern": (_i, [_vp, _P(_i64), _P(_i64)]),
    "nuto_gpu_copy_pattern": (_i, [_vp, _vp, _vp]),
    "nuto_gpu_pattern_device": (_i, [_vp, _P(_vp), _P(_vp)]),
    "nuto_gpu_set_integrand": (_i, [_vp, _P(Integrand)]),
    "nuto_gpu_num_integration_points": (_i, [_vp]),
    "nuto_gpu_solver_layout": (_i, [_vp, _vp, _vp]),
    "nuto_gpu_multigrid_info": (_i, [_vp, _vp, _vp]),
    "nuto_gpu_autotune_info": (_i, [_vp, _vp, _vp]),
    "nuto_gpu_spmv": (_i, [_vp, _i, _vp, _vp, _vp, _i]),
    "nuto_gpu_set_history": (_i, [_vp, _vp]),
    "nuto_gpu_get_history": (_i, [_vp, _vp]),
    "nuto_gpu_set_cell_scale": (_i, [_vp, _vp]),
    "nuto_gpu_set_spin_limit": (_i, [_vp, ctypes.c_longlong]),
    "nuto_gpu_history_device": (_i, [_vp, _P(_vp)]),
    "nuto_gpu_transpose_values": (_i, [_vp, _i, _vp, _vp]),
    "nuto_gpu_adjoint_history_load": (_i, [_vp, _vp, _vp, _vp]),
    "nuto_gpu_adjoint_step": (_i, [_vp, _vp, _vp, _vp, _vp, _vp, _vp]),
    "nuto_gpu_build_vector": (_i, [_vp, _vp, _vp]),
    "nuto_gpu_build_matrix": (_i, [_vp, _vp, _i, _vp]),
    "nuto_gpu_build_system": (_i, [_vp, _vp, _i, _vp, _vp]),
    "nuto_gpu_build_system_host": (_i, [_vp, _vp, _i, _vp, _vp]),
    "nuto_gpu_build_matrix_noalloc": (_i, [_vp, _vp, _vp]),
    "nuto_gpu_build_lumped_mass": (_i, [_vp, _d, _vp]),
    "nuto_gpu_eval_ip": (_i, [_vp, _vp, _i, _vp]),
    "nuto_gpu_add_boundary_cells": (_i, [_vp, _i, _i64, _i, _vp, _vp, _i, _P(_i)]),
    "nuto_gpu_build_external_load": (_i, [_vp, _i, _vp, _vp]),
    "nuto_gpu_set_constant_gradient": (_i, [_vp, _vp]),
    "nuto_gpu_update_history": (_i, [_vp, _vp]),
    "nuto_gpu_assemble_cell_vectors": (_i, [_vp, _vp, _vp]),
    "nuto_gpu_assemble_cell_matrices": (_i, [_vp, _vp, _i, _vp]),
    "nuto_gpu_solve": (_i, [_vp, _i, _i, _vp, _vp, _vp, _d, _i, _P(_i), _P(_d)]),
    "nuto_gpu_set_preconditioner": (_i, [_vp, _i]),
    "nuto_gpu_default_step_options": (_i, [_P(StepOptions)]),
    "nuto_gpu_set_state": (_i, [_vp, _vp, _d, _i]),
    "nuto_gpu_get_state": (_i, [_vp, _vp, _P(_d)]),
    "nuto_gpu_state_device": (_i, [_vp, _P(_vp)]),
    "nuto_gpu_do_step": (_i, [_vp, _d, _P(StepOptions), _P(_i)]),
    "nuto_gpu_do_step_host": (_i, [_vp, _d, _P(StepOptions), _vp, _vp, _vp, _vp, _P(_i)]),
    "nuto_gpu_get_stats": (_i, [_vp, _P(Stats)]),
}

_lock = threading.Lock()
_lib = None


def variant():
    """NUTO_GPU_VARIANT=checked selects the range-checked debugging build of the same library."""
    return os.environ.get("NUTO_GPU_VARIANT", "release")


def load(build_if_missing=True):
    """Loads libnuto_gb300.so (building it with nvcc first if it is missing or stale)."""
    global _lib
    with _lock:
        if _lib is None:
            from . import build as _build

            path = _build.lib_path(variant())
            if build_if_missing:
                _build.build(variant=variant())
            if not os.path.exists(path):
                raise RuntimeError("%s is missing: run nuto_gb300/build.py" % os.path.basename(path))
            L = ctypes.CDLL(path)
            for name, (res, args) in SIGNATURES.items():
                fn = getattr(L, name)
                fn.restype = res
                fn.argtypes = args
            _lib = L
    return _lib


def check(ctx_handle, rc):
    if rc == OK:
        return
    msg = load().nuto_gpu_last_error(ctx_handle)
    msg = msg.decode() if msg else ""
    if rc == ENOCONV:
        raise NoConvergence(rc, msg)
    raise NutoGpuError(rc, msg)
