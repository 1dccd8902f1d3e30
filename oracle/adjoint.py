"""TEST INFRASTRUCTURE ONLY — discrete adjoint of the quasistatic gradient-damage load path on the oracle.

The reference has no adjoint (no counterpart in NuTo: parity unpinned); this is the oracle for one, verified by
central finite differences of complete oracle forward solves (tests/test_oracle_adjoint.py).

Forward (QuasistaticSolver::DoStep per load step, nuto/mechanics/tools/QuasistaticSolver.cpp:116-147): step n
solves R_n(u_n; kappa_{n-1}, p) = 0 on the independent DOFs (Dirichlet values fixed by the load time), and the
history becomes kappa_n = max(kappa_{n-1}, eeq_ip(u_n)) (GradientDamage::Update, GradientDamage.h:122-125). The
residual depends on the history through kappa_trial = max(kappa_{n-1}, eeq_ip(u_n)) and omega(kappa_trial).

Loss: L = 1/2 |u_N[obs] - target|^2 after the last load step N. Parameters p: the per-cell Young's modulus E_e
(the laws are linear in E: the displacement rows of f_e scale with E_e, the eeq rows do not depend on it) and the
damage law's kappa0 and beta (through omega(kappa_trial; kappa0, beta)).

Reverse sweep, n = N .. 1, from the checkpointed (u_n, kappa_{n-1}); ubar_N = dL/du_N, kbar_N = 0:
    ubar_n  += sum over loading points (eeq >= kappa_{n-1}) of kbar_n[ip] N_ip      (kappa_n = eeq_ip there)
    K_n^T lam = ubar_n on the independent DOFs (K_n: the consistent tangent at (u_n, kappa_{n-1}); lam_dep = 0)
    s_ip     = lam_e . d f_e / d omega_ip                                              (per integration point)
    dL/dkappa0 -= sum s_ip d omega/d kappa0,   dL/dbeta -= sum s_ip d omega/d beta        (at kappa_trial)
    dL/dE_e    -= lam_e . f_e,u / E_e
    kbar_{n-1}[ip] = kbar_n[ip] - s_ip d omega/d kappa (kappa_{n-1})  at unloading points, 0 at loading points
"""

import numpy as np
import scipy.sparse.linalg as spla

from .quasistatic import QuasistaticOracle


class AdjointOracle:
    def __init__(self, problem, dependent, rhs_const, rhs_slope, tolerance=1e-12, max_iterations=30):
        self.P = problem
        self.Q = QuasistaticOracle(problem, dependent, rhs_const, rhs_slope, tolerance=tolerance,
                                   max_iterations=max_iterations)
        self.checkpoints = []

    def forward(self, t_values):
        """Load steps to every t in t_values, checkpointing (u_n, kappa_{n-1}) of each; returns u_N."""
        self.checkpoints = []
        for t in t_values:
            k_prev = self.P.kappa.copy()
            self.Q.do_step(t)
            self.checkpoints.append((self.Q.x.copy(), k_prev))
        return self.Q.x.copy()

    def gradient(self, ubar_final, young):
        """dL/d(E_e, kappa0, beta) for dL/du_N = ubar_final; `young` is the per-cell Young's modulus E_e used in
        the forward run. Restores the problem's history to kappa_N afterwards."""
        P, Q = self.P, self.Q
        n_el, n_ip = P.n_el, P.n_ip
        kappa_final = P.kappa.copy()
        indep = Q.indep
        ne = P.mesh.layer_nen(P.slots[1])
        nl = P.n_local
        n_u = nl - ne  # displacement entries of a cell vector come first (slot-major)
        g_e = np.zeros(n_el)
        g_k0 = 0.0
        g_beta = 0.0
        kbar = np.zeros((n_el, n_ip))
        for n in range(len(self.checkpoints) - 1, -1, -1):
            u_n, k_prev = self.checkpoints[n]
            P.kappa = k_prev
            data = [P.cell_adjoint(e, u_n) for e in range(n_el)]
            dofs = [P.cell_dofs(e) for e in range(n_el)]
            ubar = ubar_final.copy() if n == len(self.checkpoints) - 1 else np.zeros(P.n_dofs)
            for e in range(n_el):
                D, ipd, N = data[e]
                load = ipd[:, 1] > 0.5
                if load.any():
                    np.add.at(ubar, dofs[e][n_u:], (kbar[e, load][:, None] * N[load]).sum(axis=0))
            K = P.build_matrix_scipy(u_n).tocsr()
            Kii = K[indep][:, indep]
            lam = np.zeros(P.n_dofs)
            lam[indep] = spla.spsolve(Kii.T.tocsc(), ubar[indep])
            new_kbar = np.zeros_like(kbar)
            for e in range(n_el):
                D, ipd, N = data[e]
                le = lam[dofs[e]]
                s = le @ D
                g_k0 -= float(s @ ipd[:, 3])
                g_beta -= float(s @ ipd[:, 4])
                fe, _ = P.cell_integrate(e, u_n)
                g_e[e] -= float(le[:n_u] @ fe[:n_u]) / young[e]
                unload = ipd[:, 1] < 0.5
                new_kbar[e, unload] = kbar[e, unload] - s[unload] * ipd[unload, 2]
            kbar = new_kbar
        P.kappa = kappa_final
        return {"E": g_e, "kappa0": g_k0, "beta": g_beta}
