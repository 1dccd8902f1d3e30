"""Runs each hot kernel of the gradient-damage workload a few times, for ncu captures of single kernels.

    python -m nuto_gb300.profile_kernels --size 64 [--gmres-iterations 20]

Launch order: geometry cache, residual (x3), FP32 tangent (x3; records + row gather), FP64 tangent (x1), then one
Jacobi-preconditioned FP32 GMRES solve of --gmres-iterations iterations (every k_spmv_node launch is a product with
the whole tangent), then one multigrid-preconditioned solve of the same length. With --load-steps the state is the
one reached by that many load steps of the benchmark schedule, so the damage branches of the kernels are exercised.
"""

import argparse
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def main():
    p = argparse.ArgumentParser()
    p.add_argument("--size", type=int, default=64)
    p.add_argument("--gmres-iterations", type=int, default=20)
    p.add_argument("--load-steps", type=int, default=0)
    a = p.parse_args()
    import numpy as np
    import torch

    import nuto_gb300
    from nuto_gb300 import configs

    s = configs.hex8_gradient_damage(a.size)
    g = s.build_gpu()
    if a.load_steps:
        g.set_state(None, 0.0, True)
        o = g.default_options(precision=nuto_gb300.FP32)
        for k in range(1, a.load_steps + 1):
            g.do_step(0.05 * k, o)
        x, _ = g.get_state()
    else:
        x = np.zeros(g.n_dofs)
    u = torch.as_tensor(x, device="cuda")
    f = torch.empty(g.n_dofs, dtype=torch.float64, device="cuda")
    k32 = torch.empty(g.nnz, dtype=torch.float32, device="cuda")
    k64 = torch.empty(g.nnz, dtype=torch.float64, device="cuda")
    for _ in range(3):
        g.build_vector(u, out=f)
    for _ in range(3):
        g.build_matrix(u, nuto_gb300.FP32, out=k32)
    g.build_matrix(u, nuto_gb300.FP64, out=k64)
    b = torch.ones(g.n_dofs, dtype=torch.float64, device="cuda")
    g.set_preconditioner(nuto_gb300.PRECOND_JACOBI)
    x, it, rel, ok = g.solve(k32, b, precision=nuto_gb300.FP32, method=3, rtol=1e-12,
                             max_iterations=a.gmres_iterations)
    g.set_preconditioner(nuto_gb300.PRECOND_AMG)
    x, it2, rel, ok = g.solve(k32, b, precision=nuto_gb300.FP32, method=3, rtol=1e-12,
                              max_iterations=a.gmres_iterations)
    torch.cuda.synchronize()
    print("size %d: n_dofs %d nnz %d, gmres iterations %d (Jacobi) + %d (multigrid)" % (a.size, g.n_dofs, g.nnz, it,
                                                                                        it2))


if __name__ == "__main__":
    main()
