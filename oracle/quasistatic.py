"""TEST INFRASTRUCTURE ONLY — restatement of NuTo's quasistatic driver for small meshes.

QuasistaticSolver::DoStep / TrialState / Norm (nuto/mechanics/tools/QuasistaticSolver.cpp:51-147),
NewtonRaphson::Solve (nuto/math/NewtonRaphson.h:62-94), LineSearch (nuto/math/LineSearch.h:38-63),
Solve / SolveTrialState with the unit constraint matrix (nuto/mechanics/solver/Solve.cpp:8-81,
nuto/mechanics/constraints/Constraints.cpp:37-137). The assembly is the C++ restatement (oracle.Problem); the
sparse direct solve uses scipy's SuperLU as the stand-in for Eigen::SparseLU / MUMPS (parity of the direct
solve itself is unpinned: the reference's solver libraries are not available here).
"""

import numpy as np
import scipy.sparse.linalg as spla


class NoConvergence(RuntimeError):
    pass


class QuasistaticOracle:
    def __init__(self, problem, dependent, rhs_const, rhs_slope, tolerance=1e-10, max_iterations=6):
        """dependent: combined indices of the Dirichlet DOFs; rhs(t) = rhs_const + rhs_slope * t."""
        self.P = problem
        self.n = problem.n_dofs
        self.dep = np.asarray(dependent, dtype=np.int64)
        self.a = np.asarray(rhs_const, dtype=np.float64)
        self.b = np.asarray(rhs_slope, dtype=np.float64)
        self.indep = np.setdiff1d(np.arange(self.n), self.dep)
        self.x = np.zeros(self.n)
        self.t = 0.0
        self.tol = tolerance
        self.max_iterations = max_iterations
        self.iterations = 0

    # Constraints::GetSparseGlobalRhs stores the right-hand sides as float (Constraints.cpp:37-50)
    def global_rhs(self, t):
        v = np.zeros(self.n)
        v[self.dep] = (self.a + self.b * t).astype(np.float32).astype(np.float64)
        return v

    def norm(self, r):
        return float(np.linalg.norm(r[self.indep]))

    def residual(self, x):
        return self.P.build_vector(x)

    def derivative(self, x):
        return self.P.build_matrix_scipy(x).tocsr()

    def _solve_reduced(self, K, f):
        Kr = K[self.indep][:, self.indep].tocsc()
        y = spla.spsolve(Kr, f[self.indep])
        u = np.zeros(self.n)
        u[self.indep] = y
        return u

    def solve(self, K, f):
        return self._solve_reduced(K, f)

    def solve_trial(self, K, f, t_old, t_new):
        db = self.global_rhs(t_new) - self.global_rhs(t_old)
        u = self._solve_reduced(K, f + K @ db)
        return u - db

    def do_step(self, t_new, line_search=True):
        K = self.derivative(self.x)
        g = self.residual(self.x)
        x = self.x - self.solve_trial(K, g, self.t, t_new)
        r = self.residual(x)
        it = 0
        if self.norm(r) >= self.tol:
            converged = False
            while it < self.max_iterations:
                dr = self.derivative(x)
                dx = self.solve(dr, r)
                it += 1
                if line_search:
                    alpha = 1.0
                    x0 = x.copy()
                    previous = self.norm(self.residual(x))
                    done = False
                    for _ in range(6):
                        x = x0 - alpha * dx
                        r = self.residual(x)
                        trial = self.norm(r)
                        if trial < self.tol:
                            done = True
                            break
                        alpha *= 0.5
                        if trial < (1.0 - alpha) * previous:
                            break
                    if done:
                        converged = True
                        break
                else:
                    x = x - dx
                    r = self.residual(x)
                    if self.norm(r) < self.tol:
                        converged = True
                        break
            if not converged:
                raise NoConvergence("No convergence after %d iterations." % it)
        if self.norm(x) > 1e10:
            raise NoConvergence("floating point exception")
        self.P.update_history(x)
        self.t = t_new
        self.x = x
        self.iterations = it
        return it
