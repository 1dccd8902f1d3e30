// Quasistatic load step on the GPU: QuasistaticSolver::DoStep (nuto/mechanics/tools/QuasistaticSolver.cpp:116-147)
// with the trial state of QuasistaticSolver::TrialState / SolveTrialState (QuasistaticSolver.cpp:51-66,
// nuto/mechanics/solver/Solve.cpp:36-81), NewtonRaphson::Solve (nuto/math/NewtonRaphson.h:62-94) and
// LineSearch (nuto/math/LineSearch.h:38-63). The state vector, history, tangent and every residual stay in HBM;
// the host only sees one norm per residual evaluation to steer the iteration.
//
// Precision: with NUTO_GPU_FP32 the tangent is assembled and the Krylov iteration runs in FP32, while the
// residual, the history, the constraint values and the convergence test stay FP64, so Newton acts as
// iterative refinement of the FP32 linear solves. NUTO_GPU_MIXED keeps the FP32 tangent and preconditioner but runs
// the Krylov vectors and the products' accumulation in FP64. NUTO_GPU_FP64 runs everything in FP64.
#include "solver.cuh"

#include <chrono>
#include <cstdlib>

namespace nuto_gpu
{

// db = float(rhs(tNew)) - float(rhs(tOld)) at the dependent DOFs: Constraints::GetSparseGlobalRhs stores the
// right-hand sides in an Eigen::SparseVector<float> (Constraints.cpp:37-50).
__global__ void k_delta_bc(int64_t nDep, const int64_t* __restrict__ idx, const double* __restrict__ a,
                           const double* __restrict__ b, double tOld, double tNew, double* __restrict__ db)
{
    const int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
    if (i >= nDep)
        return;
    const float vNew = static_cast<float>(a[i] + b[i] * tNew);
    const float vOld = static_cast<float>(a[i] + b[i] * tOld);
    db[idx[i]] = static_cast<double>(vNew) - static_cast<double>(vOld);
}

// out = mask0(f + kdb) (C^T (f + K db) of SolveTrialState; kdb may be null)
__global__ void k_masked_sum(int64_t n, const uint8_t* __restrict__ mask, const double* __restrict__ f,
                             const double* __restrict__ kdb, double* __restrict__ out)
{
    const int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
    if (i >= n)
        return;
    out[i] = mask[i] ? 0. : f[i] + (kdb ? kdb[i] : 0.);
}

// out = x0 - alpha * dx (+ db)
__global__ void k_update(int64_t n, const double* __restrict__ x0, const double* __restrict__ dx, double alpha,
                         const double* __restrict__ db, double* __restrict__ out)
{
    const int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
    if (i >= n)
        return;
    out[i] = x0[i] - alpha * dx[i] + (db ? db[i] : 0.);
}

// f += g: a constant gradient contribution (e.g. NeumannBc::ExternalLoad of boundary cells registered with
// TimeDependentProblem::AddGradientFunction, TimeDependentProblem.cpp:56-66)
__global__ void k_add(int64_t n, const double* __restrict__ g, double* __restrict__ f)
{
    const int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
    if (i < n)
        f[i] += g[i];
}

// FP32 rounding of the FP64 tangent (the preconditioned FP32 operator of the exact final phase)
__global__ void k_round(int64_t n, const double* __restrict__ a, float* __restrict__ b)
{
    const int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
    if (i < n)
        b[i] = static_cast<float>(a[i]);
}

namespace
{
struct Timers
{
    Ctx& c;
    std::vector<std::pair<cudaEvent_t, cudaEvent_t>> pool;
    std::vector<std::pair<int, double*>> pending; // pool index, accumulator
    size_t next = 0;
    explicit Timers(Ctx& ctx)
        : c(ctx)
    {
    }
    ~Timers()
    {
        for (auto& p : pool)
        {
            cudaEventDestroy(p.first);
            cudaEventDestroy(p.second);
        }
    }
    int Begin()
    {
        if (next == pool.size())
        {
            std::pair<cudaEvent_t, cudaEvent_t> p;
            NG_CUDA(cudaEventCreate(&p.first));
            NG_CUDA(cudaEventCreate(&p.second));
            pool.push_back(p);
        }
        NG_CUDA(cudaEventRecord(pool[next].first, c.stream));
        return static_cast<int>(next++);
    }
    void End(int k, double* acc)
    {
        NG_CUDA(cudaEventRecord(pool[k].second, c.stream));
        pending.push_back({k, acc});
    }
    // after a stream synchronisation: fold the finished pairs into their accumulators
    void Collect()
    {
        for (auto& p : pending)
        {
            float ms = 0;
            NG_CUDA(cudaEventElapsedTime(&ms, pool[p.first].first, pool[p.first].second));
            *p.second += ms;
        }
        pending.clear();
        next = 0;
    }
};
} // namespace

int DoStep(Ctx& c, double tNew, const nuto_gpu_step_options& o, int* itersOut)
{
    const auto t0 = std::chrono::steady_clock::now();
    NG_CHECK(o.precision == NUTO_GPU_FP32 || o.precision == NUTO_GPU_FP64 || o.precision == NUTO_GPU_MIXED,
             NUTO_GPU_EINVAL, "precision NUTO_GPU_FP32, NUTO_GPU_FP64 or NUTO_GPU_MIXED");
    NG_CHECK(o.forcing != 1 || (o.forcing_floor > 0. && o.forcing_floor <= 1.), NUTO_GPU_EINVAL,
             "forcing_floor in (0, 1]");
    SolverWork& w = Work(c);
    const int64_t n = c.nDofs;
    for (DBuf<double>* b : {&w.f, &w.rhs, &w.dx, &w.db, &w.x0, &w.xs, &w.tmp, &w.refR, &w.refKx})
        if (b->n != static_cast<size_t>(n))
            b->alloc(n);
    const bool mixed = o.precision == NUTO_GPU_MIXED;
    const bool fp32 = o.precision == NUTO_GPU_FP32 || mixed; // FP32 tangent values
    const int valPrec = fp32 ? NUTO_GPU_FP32 : NUTO_GPU_FP64;
    // FP32 tangent with an exact final phase: the last Newton iterations assemble the FP64 tangent, solve with
    // FP32 Krylov sweeps on its FP32 rounding and refine against the FP64 tangent itself
    const bool exactPhase = o.precision == NUTO_GPU_FP32 && o.exact_tangent_below > 0.;
    bool exactNow = false;
    if (fp32 && w.K32.n != static_cast<size_t>(c.nnz))
        w.K32.alloc(c.nnz);
    if ((!fp32 || exactPhase) && w.K64.n != static_cast<size_t>(c.nnz))
        w.K64.alloc(c.nnz);
    void* K = fp32 ? static_cast<void*>(w.K32.p) : static_cast<void*>(w.K64.p);
    const int method = ResolveMethod(c, o.method);
    c.stats = nuto_gpu_stats{};
    for (double& h : c.hostMs)
        h = 0.;
    nuto_gpu_stats& S = c.stats;
    Timers T(c);
    int lastKrylov = 0;
    double lastRel = 0;
    const unsigned gb = static_cast<unsigned>((n + 255) / 256);

    auto assembleK = [&](const double* x) {
        HostClock hc(&c.hostMs[HP_TANGENT]);
        const int k = T.Begin();
        if (exactNow)
        {
            LaunchTangentExact(c, x, w.K64.p);
            k_round<<<static_cast<unsigned>((c.nnz + 255) / 256), 256, 0, c.stream>>>(c.nnz, w.K64.p, w.K32.p);
            c.valsVersion++;
            S.kernel_launches += 1;
        }
        else
            LaunchTangent(c, x, valPrec, K);
        T.End(k, &S.ms_assemble_matrix);
        S.matrix_assemblies++;
    };
    auto residual = [&](const double* x) {
        HostClock hc(&c.hostMs[HP_RESIDUAL]);
        const int k = T.Begin();
        LaunchResidual(c, x, w.f.p);
        if (c.dConstGrad.p)
        {
            k_add<<<gb, 256, 0, c.stream>>>(n, c.dConstGrad.p, w.f.p);
            S.kernel_launches += 1;
        }
        T.End(k, &S.ms_assemble_vector);
        S.residual_evaluations++;
        const double r = MaskedNorm(c, w.f.p);
        T.Collect();
        if (!std::isfinite(r))
            throw Error{NUTO_GPU_ENAN, "non-finite residual"};
        return r;
    };
    // FP64: one Krylov solve to krylov_rtol. FP32: FP32 Krylov sweeps inside an FP64 refinement on the FP32
    // tangent (r = rhs - K32 dx accumulated in FP64) until the true relative residual reaches krylov_rtol: the
    // FP32 iteration's own residual estimate is not trusted for the Newton direction.
    double eta = o.krylov_rtol; // forcing term of the current linear solve
    // NUTO_GPU_VERBOSE=1: one line per Newton iteration on stderr, like QuasistaticSolver::Info (2: also the FP32
    // refinement sweeps)
    const char* vb = std::getenv("NUTO_GPU_VERBOSE");
    const bool verbose = vb && (vb[0] == '1' || vb[0] == '2');
    const bool verboseSweeps = vb && vb[0] == '2';
    auto solve = [&](const double* rhs, double* out) {
        HostClock hc(&c.hostMs[HP_SOLVE]);
        const auto k0 = std::chrono::steady_clock::now();
        int it = 0;
        double* relp = &lastRel;
        if (mixed)
            KrylovSolveExport<double, float>(c, method, w.K32.p, rhs, out, false, eta, o.max_krylov, &it, relp);
        else if (fp32)
        {
            const double bn = MaskedNorm(c, rhs);
            NG_CUDA(cudaMemsetAsync(out, 0, n * sizeof(double), c.stream));
            NG_CUDA(cudaMemcpyAsync(w.refR.p, rhs, n * sizeof(double), cudaMemcpyDeviceToDevice, c.stream));
            double rel = bn > 0. ? 1. : 0.;
            const int sweeps = exactNow ? 8 : 4;
            for (int sweep = 0; sweep < sweeps && rel > eta && it < o.max_krylov; ++sweep)
            {
                const double inner = std::min(0.5, std::max(eta / rel, 1e-5));
                int its = 0;
                KrylovSolveExport<float, float>(c, method, w.K32.p, w.refR.p, out, true, inner, o.max_krylov - it,
                                                &its, nullptr);
                it += its;
                if (exactNow)
                    SpmvFull64(c, NUTO_GPU_FP64, w.K64.p, out, w.refKx.p);
                else
                    SpmvFull64Comp(c, w.K32.p, out, w.refKx.p);
                Residual64(c, rhs, w.refKx.p, w.refR.p);
                rel = bn > 0. ? MaskedNorm(c, w.refR.p) / bn : 0.;
                if (verboseSweeps)
                    std::fprintf(stderr, "[nuto_gpu]   sweep %d: inner %.1e, krylov %d, true rel %.2e\n", sweep, inner,
                                 its, rel);
            }
            lastRel = rel;
        }
        else
            KrylovSolveExport<double, double>(c, method, w.K64.p, rhs, out, false, eta, o.max_krylov, &it, relp);
        lastKrylov = it;
        T.Collect();
        S.ms_krylov += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - k0).count();
    };

    const double tOld = c.time;
    double* x = c.dX.p;

    // trial state: K(x_old), R(x_old, t_new), x_trial = x - C (C^T K C)^-1 C^T (R + K db) + db
    assembleK(x);
    {
        const int k = T.Begin();
        LaunchResidual(c, x, w.f.p);
        if (c.dConstGrad.p)
        {
            k_add<<<gb, 256, 0, c.stream>>>(n, c.dConstGrad.p, w.f.p);
            S.kernel_launches += 1;
        }
        T.End(k, &S.ms_assemble_vector);
        S.residual_evaluations++;
    }
    NG_CUDA(cudaMemsetAsync(w.db.p, 0, n * sizeof(double), c.stream));
    if (c.nDep > 0)
        k_delta_bc<<<static_cast<unsigned>((c.nDep + 255) / 256), 256, 0, c.stream>>>(
                c.nDep, c.dDepIdx.p, c.dDepA.p, c.dDepB.p, tOld, tNew, w.db.p);
    SpmvFull64(c, valPrec, K, w.db.p, w.tmp.p);
    k_masked_sum<<<gb, 256, 0, c.stream>>>(n, c.dMask.p, w.f.p, w.tmp.p, w.rhs.p);
    AfterLaunch(c, "newton vector kernels");
    S.kernel_launches += c.nDep > 0 ? 2 : 1;
    const double refNorm = MaskedNorm(c, w.rhs.p);
    S.reference_residual = refNorm;
    const double tol = std::max(o.newton_atol, o.newton_rtol * refNorm);
    solve(w.rhs.p, w.dx.p);
    k_update<<<gb, 256, 0, c.stream>>>(n, x, w.dx.p, 1.0, w.db.p, w.xs.p);
    AfterLaunch(c, "newton vector kernels");
    S.kernel_launches += 1;

    // Newton-Raphson with line search on the trial state
    double nr = residual(w.xs.p);
    int it = 0;
    bool conv = nr < tol || refNorm == 0.;
    if (verbose)
        std::fprintf(stderr, "[nuto_gpu] t = %g: trial |C^T r| = %.3e (ref %.3e, tol %.3e), krylov %d (rel %.2e)\n", tNew,
                     nr, refNorm, tol, lastKrylov, lastRel);
    // Forcing terms (forcing = 1): Eisenstat-Walker choice 1, eta_k = | |F_k| - |F_k-1 + a J s_k-1| | / |F_k-1|,
    // the disagreement between the residual and its linear model; with the safeguard eta_k >= eta_k-1^1.618 when
    // that exceeds 0.1, clamped to [krylov_rtol, 0.5] and to no less than forcing_floor tol / |F_k| (no
    // over-solving of the last iteration beyond what the caller asks for). An inaccurate (FP32) tangent gives loose solves, an accurate one tight solves.
    double prevNr = nr, stepAlpha = 1., stepRel = lastRel;
    while (!conv && it < o.max_newton)
    {
        exactNow = exactPhase && nr < o.exact_tangent_below * tol;
        assembleK(w.xs.p);
        k_masked_sum<<<gb, 256, 0, c.stream>>>(n, c.dMask.p, w.f.p, nullptr, w.rhs.p);
        S.kernel_launches += 1;
        if (o.forcing == 1)
        {
            double e = 0.1;
            if (it > 0)
            {
                const double model = ((1. - stepAlpha) + stepAlpha * stepRel) * prevNr;
                e = std::fabs(nr - model) / prevNr;
                const double sg = std::pow(eta, 1.618);
                if (sg > 0.1)
                    e = std::max(e, sg);
            }
            e = std::max(e, o.forcing_floor * tol / nr);
            eta = std::min(0.5, std::max(o.krylov_rtol, e));
        }
        solve(w.rhs.p, w.dx.p);
        stepRel = lastRel;
        prevNr = nr;
        ++it;
        if (o.line_search)
        {
            NG_CUDA(cudaMemcpyAsync(w.x0.p, w.xs.p, n * sizeof(double), cudaMemcpyDeviceToDevice, c.stream));
            const double prev = nr;
            double alpha = 1.;
            for (int step = 0; step < 6; ++step)
            {
                k_update<<<gb, 256, 0, c.stream>>>(n, w.x0.p, w.dx.p, alpha, nullptr, w.xs.p);
                S.kernel_launches += 1;
                const double trial = residual(w.xs.p);
                nr = trial;
                stepAlpha = alpha;
                if (trial < tol)
                {
                    conv = true;
                    break;
                }
                alpha *= 0.5;
                if (trial < (1. - alpha) * prev)
                    break;
            }
            if (verbose)
                std::fprintf(stderr, "[nuto_gpu] iteration %d: |C^T r| = %.3e, krylov %d (rel %.2e, eta %.1e), alpha %g\n",
                             it, nr, lastKrylov, lastRel, eta, stepAlpha);
        }
        else
        {
            k_update<<<gb, 256, 0, c.stream>>>(n, w.xs.p, w.dx.p, 1.0, nullptr, w.xs.p);
            S.kernel_launches += 1;
            nr = residual(w.xs.p);
            conv = nr < tol;
        }
    }
    S.newton_iterations = it;
    S.final_residual = nr;
    if (itersOut)
        *itersOut = it;
    auto finish = [&]() {
        T.Collect();
        S.ms_total = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
        if (verbose)
            std::fprintf(stderr,
                         "[nuto_gpu] host ms: step %.1f, tangent %.1f, residual %.1f, solve %.1f (multigrid set-up "
                         "%.1f, graph capture %.1f, waits %.1f); %s\n",
                         S.ms_total, c.hostMs[HP_TANGENT], c.hostMs[HP_RESIDUAL], c.hostMs[HP_SOLVE],
                         c.hostMs[HP_AMG_SETUP], c.hostMs[HP_GRAPH], c.hostMs[HP_SYNC], AmgGraphStatus(c));
    };
    if (!conv)
    {
        finish();
        c.err = "No convergence after " + std::to_string(it) + " iterations.";
        return NUTO_GPU_ENOCONV;
    }
    if (MaskedNorm(c, w.xs.p) > 1.e10)
    {
        finish();
        c.err = "floating point exception";
        return NUTO_GPU_ENOCONV;
    }
    LaunchHistory(c, w.xs.p);
    NG_CUDA(cudaMemcpyAsync(x, w.xs.p, n * sizeof(double), cudaMemcpyDeviceToDevice, c.stream));
    NG_CUDA(cudaStreamSynchronize(c.stream));
    if (ReadDeviceStatus(c) != 0)
    {
        finish();
        c.err = "a bounded device wait gave up";
        return NUTO_GPU_ETIMEOUT;
    }
    c.time = tNew;
    finish();
    return NUTO_GPU_OK;
}

} // namespace nuto_gpu
