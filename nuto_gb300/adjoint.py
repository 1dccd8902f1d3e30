"""Gradient of a displacement loss through the gradient-damage load path on the GPU (discrete adjoint).

The forward is the quasistatic load path (QuasistaticSolver::DoStep per load step, nuto/mechanics/tools/
QuasistaticSolver.cpp:116-147) on a `GpuCellGroup` with the gradient-damage integrand; the parameters are the
per-cell Young's modulus E_e, kappa0 and beta of DamageLawExponential. The reverse sweep runs the library's adjoint
entry points (include/nuto_gpu.h, "discrete adjoint of the load path") step by step from the last load step back:
history adjoint into ubar, transposed tangent solve, per-point parameter derivatives. The reference has no adjoint;
`LoadPathFunction` exposes it as a torch.autograd.Function.

Checkpointing: the forward keeps the state and history before every `checkpoint_every`-th load step (device
tensors); the reverse sweep recomputes the load steps of a segment from its checkpoint and then walks the segment
backwards, so the memory is (N / checkpoint_every + checkpoint_every) states instead of N.
"""

import ctypes

import numpy as np

from . import _lib
from ._lib import FP64, GRADIENT_DAMAGE, SOLVER_GMRES
from .assembly import _ptr


def _torch():
    import torch

    return torch


class AdjointLoadPath:
    """Forward load steps with checkpoints and the reverse sweep for dL/dE_e, dL/dkappa0, dL/dbeta.

    group        GpuCellGroup with the gradient-damage integrand set (integrand parameters in `integrand`)
    integrand    the set-up's integrand dict (kappa0 and beta are overridden per forward)
    t_values     end times of the load steps
    history0     initial history kappa (cells x points) or None
    """

    def __init__(self, group, integrand, t_values, history0=None, checkpoint_every=1, newton_tol=1e-12,
                 solve_rtol=1e-13, max_krylov=50000):
        if integrand["kind"] != GRADIENT_DAMAGE:
            raise ValueError("the adjoint needs the gradient-damage integrand")
        self.g = group
        self.integrand = dict(integrand)
        self.t_values = list(t_values)
        self.history0 = history0
        self.every = max(1, int(checkpoint_every))
        self.options = group.default_options(precision=FP64, newton_rtol=0.0, newton_atol=newton_tol,
                                             krylov_rtol=1e-12, max_newton=40, max_krylov=max_krylov)
        self.solve_rtol = solve_rtol
        self.max_krylov = max_krylov
        self.checkpoints = []
        self.scale = None
        self.params = None
        self.forward_steps = 0
        self.recomputed_steps = 0

    # ---- device views of the context's state and history --------------------------------------------------
    def _state(self):
        torch = _torch()
        p = self.g.state_device()
        return _wrap(p, self.g.n_dofs, torch.device("cuda", self.g.device))

    def _history(self):
        torch = _torch()
        p = ctypes.c_void_p()
        self.g._call("nuto_gpu_history_device", ctypes.byref(p))
        return _wrap(p.value, self.g.mesh.num_cells * self.g.n_ip, torch.device("cuda", self.g.device))

    # ---- forward ----------------------------------------------------------------------------------------------
    def forward(self, scale, kappa0, beta):
        """Runs the load steps with E_e = scale[e] * E, kappa0 and beta; returns u_N (device tensor, a copy)."""
        torch = _torch()
        g = self.g
        integ = dict(self.integrand)
        integ["kappa0"], integ["beta"] = float(kappa0), float(beta)
        g.set_integrand(**integ)
        g.set_cell_scale(np.asarray(scale, dtype=np.float64))
        g.set_state(None, 0.0, True)
        if self.history0 is not None:
            g.history = self.history0
        self.scale = np.asarray(scale, dtype=np.float64).copy()
        self.params = (float(kappa0), float(beta))
        self.checkpoints = []
        t = 0.0
        for n, tn in enumerate(self.t_values):
            if n % self.every == 0:
                self.checkpoints.append((n, t, self._state().clone(), self._history().clone()))
            g.do_step(tn, self.options)
            t = tn
        self.forward_steps += len(self.t_values)
        self.x_final = self._state().clone()
        self.k_final = self._history().clone()
        return self.x_final.clone()

    def _restore(self, x, kappa, t):
        self.g.set_state(None, t, False)  # the time; the state and history follow as device copies
        self._state().copy_(x)
        self._history().copy_(kappa)

    # ---- reverse sweep ----------------------------------------------------------------------------------------
    def backward(self, ubar_final):
        """dL/dE_e (per cell), dL/dkappa0, dL/dbeta for dL/du_N = ubar_final (device or host vector)."""
        torch = _torch()
        g = self.g
        dev = torch.device("cuda", g.device)
        n_dofs, n_cells, n_ip = g.n_dofs, g.mesh.num_cells, g.n_ip
        ubar_final = torch.as_tensor(ubar_final, dtype=torch.float64, device=dev)
        grad_e = torch.zeros(n_cells, dtype=torch.float64, device=dev)
        grad_p = torch.zeros(2, dtype=torch.float64, device=dev)
        kbar = torch.zeros(n_cells * n_ip, dtype=torch.float64, device=dev)
        kbar_prev = torch.empty_like(kbar)
        ubar = torch.empty(n_dofs, dtype=torch.float64, device=dev)
        K = torch.empty(g.nnz, dtype=torch.float64, device=dev)
        Kt = torch.empty_like(K)
        N = len(self.t_values)
        for ci in range(len(self.checkpoints) - 1, -1, -1):
            n0, t0, x0, k0 = self.checkpoints[ci]
            n1 = self.checkpoints[ci + 1][0] if ci + 1 < len(self.checkpoints) else N
            # recompute the segment's states (u_n, kappa_{n-1}) from its checkpoint
            self._restore(x0, k0, t0)
            seg = []
            for n in range(n0, n1):
                k_prev = self._history().clone()
                g.do_step(self.t_values[n], self.options)
                seg.append((self._state().clone(), k_prev))
            self.recomputed_steps += n1 - n0
            for n in range(n1 - 1, n0 - 1, -1):
                u_n, k_prev = seg[n - n0]
                self._history().copy_(k_prev)
                if n == N - 1:
                    ubar.copy_(ubar_final)
                else:
                    ubar.zero_()
                g._call("nuto_gpu_adjoint_history_load", _ptr(u_n), _ptr(kbar), _ptr(ubar))
                g.build_matrix(u_n, FP64, out=K)
                g._call("nuto_gpu_transpose_values", FP64, _ptr(K), _ptr(Kt))
                lam, it, rel, ok = g.solve(Kt, ubar, precision=FP64, method=SOLVER_GMRES, rtol=self.solve_rtol,
                                           max_iterations=self.max_krylov)
                if not ok:
                    raise _lib.NoConvergence(_lib.ENOCONV, "adjoint solve: %d iterations, relative residual %.2e"
                                             % (it, rel))
                g._call("nuto_gpu_adjoint_step", _ptr(u_n), _ptr(lam), _ptr(kbar), _ptr(kbar_prev), _ptr(grad_e),
                        _ptr(grad_p))
                kbar, kbar_prev = kbar_prev, kbar
        # leave the group at the end of the forward
        self._restore(self.x_final, self.k_final, self.t_values[-1] if self.t_values else 0.0)
        gp = grad_p.cpu().numpy()
        return grad_e, float(gp[0]), float(gp[1])


def _wrap(ptr, n, device):
    """A torch view of n doubles at a device pointer owned by the library (valid while the context lives)."""
    torch = _torch()

    class _Cai:
        __cuda_array_interface__ = {"shape": (n,), "typestr": "<f8", "data": (int(ptr), False), "version": 2,
                                    "strides": None}

    return torch.as_tensor(_Cai(), device=device)


def _make_function():
    torch = _torch()

    class LoadPathFunction(torch.autograd.Function):
        """u_N = LoadPathFunction.apply(young, kappa0, beta, path): the displacements after the load path of
        `path` (an AdjointLoadPath) for the per-cell Young's modulus `young` (tensor, n_cells) and the damage law's
        kappa0, beta (0-d tensors); backward runs the GPU reverse sweep."""

        @staticmethod
        def forward(ctx, young, kappa0, beta, path):
            E = path.integrand["E"]
            scale = (young.detach().double().cpu().numpy() / E)
            x = path.forward(scale, float(kappa0), float(beta))
            ctx.path = path
            return x

        @staticmethod
        def backward(ctx, grad_x):
            ge, gk, gb = ctx.path.backward(grad_x.contiguous())
            dev = grad_x.device
            return (ge, torch.tensor(gk, dtype=torch.float64, device=dev),
                    torch.tensor(gb, dtype=torch.float64, device=dev), None)

    return LoadPathFunction


_FN = None


def load_path_function():
    """The torch.autograd.Function over AdjointLoadPath (built on first use: torch is imported lazily)."""
    global _FN
    if _FN is None:
        _FN = _make_function()
    return _FN
