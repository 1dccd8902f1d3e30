// Preconditioned Krylov solvers (PCG for SPD tangents; GMRES and BiCGStab for the non-symmetric damage tangents;
// Jacobi or the aggregation multigrid cycle of amg.cu) on the CSR tangent, replacing the sparse direct solve of the reference (Solve.cpp:8-34 with
// EigenSparseSolve.cpp:22-73). The constrained system C^T K C y = C^T b of unit (Dirichlet) constraints is
// solved in place: dependent rows act as identity and the iterates stay zero there, so the dependent columns
// never contribute.
//
// Every reduction is fused into the kernel that produces its operands; the last block of the grid (atomic
// ticket, no waiting) turns the sums into the iteration scalars (alpha, beta, omega) kept in device memory, so a
// whole chunk of iterations runs without a host round trip. Dot products accumulate in FP64.
#include "spmv.cuh"

namespace nuto_gpu
{

SolverWork::~SolverWork()
{
    for (auto& p : spmvEv)
    {
        cudaEventDestroy(p.first);
        cudaEventDestroy(p.second);
    }
    if (hG)
        cudaFreeHost(hG);
    if (hScal)
        cudaFreeHost(hScal);
    if (hStat)
        cudaFreeHost(hStat);
    for (cudaEvent_t& e : ev)
        if (e)
            cudaEventDestroy(e);
}

SolverWork& Work(Ctx& c)
{
    if (!c.work)
    {
        auto* w = new SolverWork();
        c.work = w;
        w->scal.alloc(SC_COUNT);
        w->stat.alloc(ST_COUNT);
        NG_CUDA(cudaMallocHost(&w->hScal, SC_COUNT * sizeof(double)));
        NG_CUDA(cudaMallocHost(&w->hStat, ST_COUNT * sizeof(int)));
        for (cudaEvent_t& e : w->ev)
            NG_CUDA(cudaEventCreate(&e));
    }
    return *c.work;
}

void FreeSolverWork(Ctx& c)
{
    delete c.work;
    c.work = nullptr;
}

// ---- right-hand side preparation ---------------------------------------------------------------------------
// bb = |mask0(b)|^2; last block: scale = 1/|b| (FP32) or 1, tol2 = rtol^2 |b scale|^2
__global__ void __launch_bounds__(kBS) k_rhs_norm(int64_t n, const uint8_t* __restrict__ mask,
                                                   const double* __restrict__ b, double* sc, int* st, double rtol,
                                                   int scaleToUnit)
{
    __shared__ double sh[kBS / 32];
    double v = 0;
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x)
        if (!mask[i])
            v += b[i] * b[i];
    BlockAccumulate(v, sc + SC_ACC0, sh);
    if (LastBlock(st + ST_COUNTER) && threadIdx.x == 0)
    {
        st[ST_COUNTER] = 0;
        const double bb = VRead(sc + SC_ACC0);
        sc[SC_ACC0] = 0.;
        sc[SC_BB] = bb;
        const double scale = (scaleToUnit && bb > 0.) ? 1. / sqrt(bb) : 1.;
        sc[SC_SCALE] = scale;
        sc[SC_TOL2] = rtol * rtol * bb * scale * scale;
        st[ST_ITERS] = 0;
        st[ST_HALF] = 0;
        st[ST_STATE] = (bb == 0.) ? CONVERGED : (isfinite(bb) ? RUN : NONFINITE);
        sc[SC_RR] = bb * scale * scale;
    }
}

// x = 0, r = mask0(b) * scale, z = dinv r, p = z (PCG) / rh = r, p = v = 0 (BiCGStab); acc0 += r.z (PCG) or
// r.r (BiCGStab); last block: rho
template <typename T, bool PCG>
__global__ void __launch_bounds__(kBS) k_krylov_init(int64_t n, const uint8_t* __restrict__ mask,
                                                      const double* __restrict__ b, T* x, T* r, T* rh, T* p, T* v,
                                                      T* z, const T* __restrict__ dinv, double* sc, int* st)
{
    __shared__ double sh[kBS / 32];
    const double scale = sc[SC_SCALE];
    double acc = 0;
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x)
    {
        const T ri = mask[i] ? T(0) : static_cast<T>(b[i] * scale);
        x[i] = T(0);
        r[i] = ri;
        if (PCG)
        {
            const T zi = dinv[i] * ri;
            z[i] = zi;
            p[i] = zi;
            acc += static_cast<double>(ri) * static_cast<double>(zi);
        }
        else
        {
            rh[i] = ri;
            p[i] = T(0);
            v[i] = T(0);
            acc += static_cast<double>(ri) * static_cast<double>(ri);
        }
    }
    BlockAccumulate(acc, sc + SC_ACC0, sh);
    if (LastBlock(st + ST_COUNTER) && threadIdx.x == 0)
    {
        st[ST_COUNTER] = 0;
        const double a = VRead(sc + SC_ACC0);
        sc[SC_ACC0] = 0.;
        sc[SC_RHO] = a;
        sc[SC_RHO_OLD] = 1.;
        sc[SC_ALPHA] = 1.;
        sc[SC_OMEGA] = 1.;
        sc[SC_BETA] = 0.;
    }
}

// Jacobi: dinv = 1 / K_ii for independent rows, 1 for dependent rows
template <typename TV, typename T>
__global__ void k_diag_inv(int64_t n, const int64_t* __restrict__ rowPtr, const int32_t* __restrict__ col,
                           const TV* __restrict__ val, const uint8_t* __restrict__ mask, T* __restrict__ dinv)
{
    const int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
    if (i >= n)
        return;
    if (mask[i])
    {
        dinv[i] = T(1);
        return;
    }
    int64_t lo = rowPtr[i], hi = rowPtr[i + 1] - 1;
    while (lo < hi)
    {
        const int64_t mid = (lo + hi) / 2;
        if (col[mid] < i)
            lo = mid + 1;
        else
            hi = mid;
    }
    const double d = (lo < rowPtr[i + 1] && col[lo] == i) ? static_cast<double>(val[lo]) : 0.;
    dinv[i] = d != 0. ? static_cast<T>(1. / d) : T(1);
}

// ---- PCG ------------------------------------------------------------------------------------------------------
// x += alpha p; r -= alpha q; z = dinv r; acc0 += r.z; acc1 += r.r; last block: convergence test, beta, rho.
// With dinv == nullptr (multigrid) z, beta and rho are left to k_pcg_rz after the cycle.
template <typename T>
__global__ void __launch_bounds__(kBS) k_pcg_update(int64_t n, T* x, T* r, const T* __restrict__ p,
                                                     const T* __restrict__ q, T* z, const T* __restrict__ dinv,
                                                     double* sc, int* st)
{
    __shared__ double sh[kBS / 32];
    if (st[ST_STATE] != RUN)
        return;
    const T alpha = static_cast<T>(sc[SC_ALPHA]);
    double rz = 0, rr = 0;
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x)
    {
        x[i] += alpha * p[i];
        const T ri = r[i] - alpha * q[i];
        r[i] = ri;
        if (dinv)
        {
            const T zi = dinv[i] * ri;
            z[i] = zi;
            rz += static_cast<double>(ri) * static_cast<double>(zi);
        }
        rr += static_cast<double>(ri) * static_cast<double>(ri);
    }
    BlockAccumulate(rz, sc + SC_ACC0, sh);
    BlockAccumulate(rr, sc + SC_ACC1, sh);
    if (LastBlock(st + ST_COUNTER) && threadIdx.x == 0)
    {
        st[ST_COUNTER] = 0;
        const double a0 = VRead(sc + SC_ACC0), a1 = VRead(sc + SC_ACC1);
        sc[SC_ACC0] = 0.;
        sc[SC_ACC1] = 0.;
        st[ST_ITERS] += 1;
        sc[SC_RR] = a1;
        if (!Finite(a0) || !Finite(a1))
            st[ST_STATE] = NONFINITE;
        else if (a1 <= sc[SC_TOL2])
            st[ST_STATE] = CONVERGED;
        else if (dinv)
        {
            sc[SC_BETA] = a0 / sc[SC_RHO];
            sc[SC_RHO] = a0;
        }
    }
}

// acc0 += r.z for z = M^-1 r of the multigrid cycle; last block: rho (init) or beta and rho
template <typename T>
__global__ void __launch_bounds__(kBS) k_pcg_rz(int64_t n, const T* __restrict__ r, const T* __restrict__ z,
                                                 double* sc, int* st, int init)
{
    __shared__ double sh[kBS / 32];
    if (st[ST_STATE] != RUN)
        return;
    double rz = 0;
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x)
        rz += static_cast<double>(r[i]) * static_cast<double>(z[i]);
    BlockAccumulate(rz, sc + SC_ACC0, sh);
    if (LastBlock(st + ST_COUNTER) && threadIdx.x == 0)
    {
        st[ST_COUNTER] = 0;
        const double a0 = VRead(sc + SC_ACC0);
        sc[SC_ACC0] = 0.;
        if (!Finite(a0))
            st[ST_STATE] = NONFINITE;
        else if (!(a0 > 0.))
            st[ST_STATE] = BREAKDOWN; // the preconditioner is not positive definite for this matrix
        else
        {
            sc[SC_BETA] = init ? 0. : a0 / sc[SC_RHO];
            sc[SC_RHO] = a0;
        }
    }
}

template <typename T>
__global__ void __launch_bounds__(kBS) k_pcg_dir(int64_t n, T* p, const T* __restrict__ z, const double* sc,
                                                  const int* st)
{
    if (st[ST_STATE] != RUN)
        return;
    const T beta = static_cast<T>(sc[SC_BETA]);
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x)
        p[i] = z[i] + beta * p[i];
}

// ---- BiCGStab (right-preconditioned with dinv) ---------------------------------------------------------------
// beta = (rho / rho_old)(alpha / omega) computed by the previous iteration; p = r + beta (p - omega v); ph = dinv p
template <typename T>
__global__ void __launch_bounds__(kBS) k_bicg_p(int64_t n, T* p, const T* __restrict__ r, const T* __restrict__ v,
                                                 T* ph, const T* __restrict__ dinv, const double* sc, const int* st)
{
    if (st[ST_STATE] != RUN)
        return;
    const T beta = static_cast<T>(sc[SC_BETA]);
    const T omega = static_cast<T>(sc[SC_OMEGA]);
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x)
    {
        const T pi = r[i] + beta * (p[i] - omega * v[i]);
        p[i] = pi;
        ph[i] = dinv[i] * pi;
    }
}

// s = r - alpha v; sh = dinv s; acc0 += s.s; last block: converged on s -> half step
template <typename T>
__global__ void __launch_bounds__(kBS) k_bicg_s(int64_t n, T* s, const T* __restrict__ r, const T* __restrict__ v,
                                                 T* sh_, const T* __restrict__ dinv, double* sc, int* st)
{
    __shared__ double sh[kBS / 32];
    if (st[ST_STATE] != RUN)
        return;
    const T alpha = static_cast<T>(sc[SC_ALPHA]);
    double ss = 0;
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x)
    {
        const T si = r[i] - alpha * v[i];
        s[i] = si;
        sh_[i] = dinv[i] * si;
        ss += static_cast<double>(si) * static_cast<double>(si);
    }
    BlockAccumulate(ss, sc + SC_ACC2, sh);
    if (LastBlock(st + ST_COUNTER) && threadIdx.x == 0)
    {
        st[ST_COUNTER] = 0;
        const double a = VRead(sc + SC_ACC2);
        sc[SC_ACC2] = 0.;
        if (!Finite(a))
            st[ST_STATE] = NONFINITE;
        else if (a <= sc[SC_TOL2])
            st[ST_HALF] = 1;
    }
}

// x += alpha ph + omega sh; r = s - omega t; acc0 += rh.r; acc1 += r.r; last block: convergence, beta
template <typename T>
__global__ void __launch_bounds__(kBS) k_bicg_x(int64_t n, T* x, T* r, const T* __restrict__ rh,
                                                 const T* __restrict__ ph, const T* __restrict__ s,
                                                 const T* __restrict__ shv, const T* __restrict__ t, double* sc,
                                                 int* st)
{
    __shared__ double sh[kBS / 32];
    if (st[ST_STATE] != RUN)
        return;
    const bool half = st[ST_HALF] != 0;
    const T alpha = static_cast<T>(sc[SC_ALPHA]);
    const T omega = half ? T(0) : static_cast<T>(sc[SC_OMEGA]);
    double rhr = 0, rr = 0;
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x)
    {
        x[i] += alpha * ph[i] + omega * shv[i];
        const T ri = half ? s[i] : s[i] - omega * t[i];
        r[i] = ri;
        rhr += static_cast<double>(rh[i]) * static_cast<double>(ri);
        rr += static_cast<double>(ri) * static_cast<double>(ri);
    }
    BlockAccumulate(rhr, sc + SC_ACC0, sh);
    BlockAccumulate(rr, sc + SC_ACC1, sh);
    if (LastBlock(st + ST_COUNTER) && threadIdx.x == 0)
    {
        st[ST_COUNTER] = 0;
        const double a0 = VRead(sc + SC_ACC0), a1 = VRead(sc + SC_ACC1);
        sc[SC_ACC0] = 0.;
        sc[SC_ACC1] = 0.;
        st[ST_ITERS] += 1;
        sc[SC_RR] = a1;
        const double om = sc[SC_OMEGA];
        if (!Finite(a0) || !Finite(a1))
            st[ST_STATE] = NONFINITE;
        else if (half || a1 <= sc[SC_TOL2])
            st[ST_STATE] = CONVERGED;
        else if (a0 == 0. || om == 0.)
            st[ST_STATE] = BREAKDOWN;
        else
        {
            sc[SC_BETA] = (a0 / sc[SC_RHO]) * (sc[SC_ALPHA] / om);
            sc[SC_RHO_OLD] = sc[SC_RHO];
            sc[SC_RHO] = a0;
        }
    }
}

// out = x * (1/scale) (converts the Krylov solution back to FP64)
template <typename T>
__global__ void k_unscale(int64_t n, const T* __restrict__ x, const double* sc, double* __restrict__ out, int add)
{
    const int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
    if (i >= n)
        return;
    const double s = sc[SC_SCALE];
    const double v = static_cast<double>(x[i]) / s;
    out[i] = add ? out[i] + v : v;
}

__global__ void k_masked_sq(int64_t n, const uint8_t* __restrict__ mask, const double* __restrict__ v, double* acc)
{
    __shared__ double sh[kBS / 32];
    double s = 0;
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x)
        if (!mask[i])
            s += v[i] * v[i];
    BlockAccumulate(s, acc, sh);
}

// ---- host side -----------------------------------------------------------------------------------------------
// host wait for the context's stream (its time is reported as HP_SYNC)
static void WaitStream(Ctx& c)
{
    HostClock hc(&c.hostMs[HP_SYNC]);
    NG_CUDA(cudaStreamSynchronize(c.stream));
}

static int GridFor(const Ctx& c, int64_t n)
{
    const int64_t want = (n + kBS - 1) / kBS;
    const int64_t cap = static_cast<int64_t>(c.smCount) * 8;
    return static_cast<int>(want < cap ? want : cap);
}

NodeSpmv MakeNodeSpmv(const Ctx& c)
{
    NodeSpmv A{};
    A.ns = static_cast<int>(c.slots.size());
    int64_t w = 0;
    for (int I = 0; I < A.ns; ++I)
    {
        A.ncomp[I] = c.slots[I].ncomp;
        A.nNodes[I] = c.slots[I].nNodes;
        A.firstWarp[I] = w;
        A.gdof[I] = c.slots[I].dGdof.p;
        w += c.slots[I].nNodes;
    }
    A.totalWarps = w;
    for (int p = 0; p < A.ns * A.ns; ++p)
    {
        A.nbrPtr[p] = c.pairs[p].dNbrPtr.p;
        A.nbrIdx[p] = c.pairs[p].dNbrIdx.p;
        A.nbrCol[p] = c.pairs[p].dNbrCol.p;
        A.blk[p] = c.pairs[p].dBlk.p;
        A.nbrTotal[p] = static_cast<int64_t>(c.pairs[p].dNbrIdx.n);
    }
    A.rowPtr = c.dRowPtr.p;
    A.nnz = c.nnz;
    A.nRows = c.nDofs;
    if (c.nb.total > 0)
    {
        for (int p = 0; p < A.ns * A.ns; ++p)
        {
            A.nbBase[p] = c.nb.pair[p].base.p;
            A.nbOff[p] = c.nb.pair[p].off;
        }
        // per group the padded segments of every column slot of one row slot side by side
        A.nbSeg4 = 0;
        A.ncMaxRows = 0;
        for (int I = 0; I < A.ns; ++I)
            A.ncMaxRows = std::max(A.ncMaxRows, c.slots[I].ncomp);
        for (int I = 0; I < A.ns; ++I)
        {
            int sum = 0;
            for (int J = 0; J < A.ns; ++J)
                sum += c.nb.pair[I * A.ns + J].maxSeg4;
            A.nbSeg4 = std::max(A.nbSeg4, sum);
        }
        A.nb32 = c.nb.v32.p;
        A.nb64 = c.nb.v64.p;
        A.nbSrc32 = c.nb.src32;
        A.nbSrc64 = c.nb.src64;
    }
    return A;
}

bool PdlEnabled()
{
    static const bool on = [] {
        const char* e = std::getenv("NUTO_GPU_PDL");
        return !(e && e[0] == '0');
    }();
    return on;
}

template <typename TV>
void EnsureNb(Ctx& c, const TV* vals)
{
    NbLayout& L = c.nb;
    if (L.total <= 0 || !vals)
        return;
    const void*& src = sizeof(TV) == 4 ? L.src32 : L.src64;
    uint64_t& ver = sizeof(TV) == 4 ? L.ver32 : L.ver64;
    if (src == static_cast<const void*>(vals) && ver == c.valsVersion)
        return;
    TV* dst;
    if constexpr (sizeof(TV) == 4)
    {
        if (L.v32.n != static_cast<size_t>(L.total))
            L.v32.alloc(L.total);
        dst = L.v32.p;
    }
    else
    {
        if (L.v64.n != static_cast<size_t>(L.total))
            L.v64.alloc(L.total);
        dst = L.v64.p;
    }
    src = vals; // before MakeNodeSpmv: the view carries the source pointer
    ver = c.valsVersion;
    const NodeSpmv A = MakeNodeSpmv(c);
    k_nb_pack<TV><<<static_cast<unsigned>((A.totalWarps * 32 + kBS - 1) / kBS), kBS, 0, c.stream>>>(A, vals, dst);
    c.stats.kernel_launches += 1;
    AfterLaunch(c, "padded pair layout");
}
template void EnsureNb<float>(Ctx&, const float*);
template void EnsureNb<double>(Ctx&, const double*);

// Autotuner of the fine-level product: the first product of a context with a given value and vector type (outside
// any stream capture) times the padded-layout kernel with 4, 8 and 16 lanes per node (one warm-up and one timed
// launch each, y = K x without dot products, so the tuning launches only write the y the real call writes again)
// and keeps the fastest; NUTO_GPU_AUTOTUNE=0 keeps the default.
template <typename TV, typename TX>
static int SpmvGroup(Ctx& c, const NodeSpmv& A, const TV* vals, const TX* x, TX* y, const uint8_t* mask)
{
    const int key = (sizeof(TV) == 4 ? 0 : 2) + (sizeof(TX) == 4 ? 0 : 1);
    Tuning& T = c.tuning;
    if (T.spmvGroup[key] > 0)
        return T.spmvGroup[key];
    if (!T.enabled || !SpmvPadded(A, vals))
        return 0;
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    NG_CUDA(cudaStreamIsCapturing(c.stream, &cs));
    if (cs != cudaStreamCaptureStatusNone)
        return 0;
    const int cand[3] = {4, 8, 16};
    cudaEvent_t e0, e1;
    NG_CUDA(cudaEventCreate(&e0));
    NG_CUDA(cudaEventCreate(&e1));
    float best = 0.f;
    int pick = kNbG;
    for (int k = 0; k < 3; ++k)
    {
        SpmvNode<TV, TX, 0>(c.stream, A, vals, x, y, nullptr, nullptr, nullptr, FIN_NONE, mask, cand[k]);
        NG_CUDA(cudaEventRecord(e0, c.stream));
        SpmvNode<TV, TX, 0>(c.stream, A, vals, x, y, nullptr, nullptr, nullptr, FIN_NONE, mask, cand[k]);
        NG_CUDA(cudaEventRecord(e1, c.stream));
        NG_CUDA(cudaEventSynchronize(e1));
        float ms = 0.f;
        NG_CUDA(cudaEventElapsedTime(&ms, e0, e1));
        T.spmvMs[key][k] = ms;
        if (k == 0 || ms < best)
        {
            best = ms;
            pick = cand[k];
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    c.stats.kernel_launches += 6;
    T.spmvGroup[key] = pick;
    return pick;
}

template <typename TV, typename TX, int NDOT>
static void SpmvLaunch(Ctx& c, const TV* vals, const TX* x, TX* y, const TX* w0, double* sc, int* st, int fin,
                       const uint8_t* mask)
{
    const NodeSpmv A = MakeNodeSpmv(c);
    const int g = SpmvGroup<TV, TX>(c, A, vals, x, y, mask);
    SpmvNode<TV, TX, NDOT>(c.stream, A, vals, x, y, w0, sc, st, fin, mask, g);
}

// Krylov SpMV with a CUDA-event pair around it (device time of the dominant kernel, collected by SpmvCollect)
template <typename TV, typename TX, int NDOT>
static void SpmvTimed(Ctx& c, const TV* vals, const TX* x, TX* y, const TX* w0, double* sc, int* st, int fin,
                      const uint8_t* mask)
{
    SolverWork& w = Work(c);
    if (w.spmvNext == w.spmvEv.size())
    {
        std::pair<cudaEvent_t, cudaEvent_t> p;
        NG_CUDA(cudaEventCreate(&p.first));
        NG_CUDA(cudaEventCreate(&p.second));
        w.spmvEv.push_back(p);
    }
    auto& ev = w.spmvEv[w.spmvNext++];
    NG_CUDA(cudaEventRecord(ev.first, c.stream));
    SpmvLaunch<TV, TX, NDOT>(c, vals, x, y, w0, sc, st, fin, mask);
    NG_CUDA(cudaEventRecord(ev.second, c.stream));
    c.stats.kernel_launches += 1;
}

// after a stream synchronisation: add the recorded SpMV times to the statistics
static void SpmvCollect(Ctx& c)
{
    SolverWork& w = Work(c);
    for (size_t i = 0; i < w.spmvNext; ++i)
    {
        float ms = 0;
        NG_CUDA(cudaEventElapsedTime(&ms, w.spmvEv[i].first, w.spmvEv[i].second));
        c.stats.ms_spmv += ms;
    }
    c.stats.spmv_launches += static_cast<int64_t>(w.spmvNext);
    w.spmvNext = 0;
}

double MaskedNorm(Ctx& c, const double* v)
{
    SolverWork& w = Work(c);
    NG_CUDA(cudaMemsetAsync(w.scal.p + SC_ACC2, 0, sizeof(double), c.stream));
    k_masked_sq<<<GridFor(c, c.nDofs), kBS, 0, c.stream>>>(c.nDofs, c.dMask.p, v, w.scal.p + SC_ACC2);
    c.stats.kernel_launches += 1;
    NG_CUDA(cudaMemcpyAsync(w.hScal + SC_ACC2, w.scal.p + SC_ACC2, sizeof(double), cudaMemcpyDeviceToHost, c.stream));
    WaitStream(c);
    const double r = w.hScal[SC_ACC2];
    NG_CUDA(cudaMemsetAsync(w.scal.p + SC_ACC2, 0, sizeof(double), c.stream));
    return std::sqrt(r);
}

// ---- FP32 values times FP64 vectors on the FP32 pipe --------------------------------------------------------------
// y = K x with FP32 values and an FP64 x given as hi + lo floats (xs[i] = (hi, lo)): v * hi is formed exactly
// (product and its FMA error term) and summed with TwoSum compensation, v * lo in plain FP32; each lane's row sums
// go to FP64 only for the final 8-lane butterfly. About 48 bits of the sum survive (relative error ~1e-14 of
// sum |v x|), enough for the residual of an FP32 iterative refinement, with no FP64 arithmetic per nonzero: the
// FP64-vector form of this product is limited by the FP64 pipe on this part.
__device__ __forceinline__ void TwoSumAcc(float& s, float& err, float p)
{
    const float t = s + p;
    const float bp = t - s;
    err += (s - (t - bp)) + (p - bp);
    s = t;
}

__global__ void __launch_bounds__(kBS) k_spmv_nb_comp(NodeSpmv A, const uint8_t* __restrict__ mask,
                                                       const float2* __restrict__ xs2, const double* __restrict__ x,
                                                       double* __restrict__ y)
{
    extern __shared__ __align__(16) unsigned char nbSmem[];
    const float* __restrict__ vals = A.nb32;
    const int gl = threadIdx.x & (kNbG - 1);
    const int L = A.nbSeg4;
    float2* xs = reinterpret_cast<float2*>(nbSmem) + (threadIdx.x / kNbG) * L;
    const int64_t u = (blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x) / kNbG;
    int I = 0;
    int64_t a = 0;
    bool valid = u < A.totalWarps;
    if (valid)
    {
        I = (A.ns > 1 && u >= A.firstWarp[1]) ? 1 : 0;
        a = u - A.firstWarp[I];
        valid = a < A.nNodes[I];
    }
    const int ncI = valid ? A.ncomp[I] : 0;
    int64_t q0[kMaxSlots], vbase[kMaxSlots];
    int nn[kMaxSlots], seg4[kMaxSlots], xoff[kMaxSlots];
    int tot = 0, xo = 0;
#pragma unroll
    for (int J = 0; J < kMaxSlots; ++J)
    {
        q0[J] = 0;
        nn[J] = 0;
        vbase[J] = 0;
        if (valid && J < A.ns)
        {
            const int p = I * A.ns + J;
            q0[J] = A.nbrPtr[p][a];
            nn[J] = static_cast<int>(A.nbrPtr[p][a + 1] - q0[J]);
            vbase[J] = A.nbOff[p] + A.nbBase[p][a];
        }
        seg4[J] = (A.ncomp[J < A.ns ? J : 0] * nn[J] + 3) & ~3;
        xoff[J] = xo;
        xo += seg4[J];
        tot += nn[J];
    }
    const int nc0 = A.ncomp[0], nc1 = A.ns > 1 ? A.ncomp[1] : 0;
#pragma unroll 4
    for (int t = gl; t < tot; t += kNbG)
    {
        const int J = t >= nn[0] ? 1 : 0;
        const int kk = t - (J ? nn[0] : 0);
        const int ncJ = J ? nc1 : nc0;
        const int p = I * A.ns + J;
        const int64_t col = A.nbrCol[p][NG_IDX((J ? q0[1] : q0[0]) + kk, A.nbrTotal[p], 60)];
        const int xb = (J ? xoff[1] : 0) + kk * ncJ;
        for (int d = 0; d < ncJ; ++d)
            xs[NG_IDX(xb + d, L, 61)] = xs2[NG_IDX(col + d, A.nRows, 62)];
    }
#pragma unroll
    for (int J = 0; J < kMaxSlots; ++J)
    {
        const int seg = (J ? nc1 : nc0) * nn[J];
        for (int t = seg + gl; t < seg4[J]; t += kNbG)
            xs[NG_IDX(xoff[J] + t, L, 63)] = make_float2(0.f, 0.f);
    }
    __syncwarp();
    float sh[kMaxComp], se[kMaxComp], sl[kMaxComp];
#pragma unroll
    for (int c = 0; c < kMaxComp; ++c)
        sh[c] = se[c] = sl[c] = 0.f;
#pragma unroll
    for (int J = 0; J < kMaxSlots; ++J)
    {
        const float* vp = vals + vbase[J];
        const float2* xj = xs + xoff[J];
        const int sg = seg4[J];
        for (int f = 4 * gl; f < sg; f += 4 * kNbG)
        {
            const float4 x01 = *reinterpret_cast<const float4*>(xj + f);
            const float4 x23 = *reinterpret_cast<const float4*>(xj + f + 2);
            const float xh[4] = {x01.x, x01.z, x23.x, x23.z}, xl[4] = {x01.y, x01.w, x23.y, x23.w};
#pragma unroll
            for (int c = 0; c < kMaxComp; ++c)
                if (c < ncI)
                {
                    const float4 v4 = *reinterpret_cast<const float4*>(vp + c * sg + f);
                    const float v[4] = {v4.x, v4.y, v4.z, v4.w};
#pragma unroll
                    for (int k = 0; k < 4; ++k)
                    {
                        const float p = v[k] * xh[k];
                        se[c] += fmaf(v[k], xh[k], -p);
                        TwoSumAcc(sh[c], se[c], p);
                        sl[c] = fmaf(v[k], xl[k], sl[c]);
                    }
                }
        }
    }
    double s[kMaxComp];
#pragma unroll
    for (int c = 0; c < kMaxComp; ++c)
        s[c] = static_cast<double>(sh[c]) + (static_cast<double>(se[c]) + static_cast<double>(sl[c]));
#pragma unroll
    for (int o = kNbG / 2; o > 0; o >>= 1)
#pragma unroll
        for (int c = 0; c < kMaxComp; ++c)
            s[c] += __shfl_xor_sync(0xffffffffu, s[c], o);
    if (valid && gl == 0)
    {
        const int64_t g0 = A.gdof[I][a];
        for (int c = 0; c < ncI; ++c)
        {
            const int64_t r = NG_IDX(g0 + c, A.nRows, 64);
            y[r] = mask[r] ? x[r] : s[c];
        }
    }
}

// x (FP64) -> (hi, lo) floats for k_spmv_nb_comp
__global__ void k_split_hilo(int64_t n, const double* __restrict__ x, float2* __restrict__ xs)
{
    const int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
    if (i >= n)
        return;
    const float h = static_cast<float>(x[i]);
    xs[i] = make_float2(h, static_cast<float>(x[i] - static_cast<double>(h)));
}

void SpmvFull64Comp(Ctx& c, const float* vals, const double* x, double* y)
{
    SolverWork& w = Work(c);
    const int64_t n = c.nDofs;
    EnsureNb(c, vals);
    const NodeSpmv A = MakeNodeSpmv(c);
    if (!A.nbBase[0] || A.nbSrc32 != static_cast<const void*>(vals) || A.nbSeg4 <= 0)
    {
        SpmvFull64(c, NUTO_GPU_FP32, vals, x, y); // no padded layout: exact FP64 accumulation
        return;
    }
    if (w.zeroMask.n != static_cast<size_t>(n))
    {
        w.zeroMask.alloc(n);
        NG_CUDA(cudaMemsetAsync(w.zeroMask.p, 0, n, c.stream));
    }
    if (w.xsplit.n != static_cast<size_t>(2 * n))
        w.xsplit.alloc(2 * n);
    float2* xs = reinterpret_cast<float2*>(w.xsplit.p);
    k_split_hilo<<<static_cast<unsigned>((n + 255) / 256), 256, 0, c.stream>>>(n, x, xs);
    const size_t perGroup = static_cast<size_t>(A.nbSeg4) * sizeof(float2);
    int threads = kBS;
    while (threads > 32 && (threads / kNbG) * perGroup > 48 * 1024)
        threads -= 32;
    const unsigned blocks = static_cast<unsigned>((A.totalWarps * kNbG + threads - 1) / threads);
    k_spmv_nb_comp<<<blocks, threads, (threads / kNbG) * perGroup, c.stream>>>(A, w.zeroMask.p, xs, x, y);
    c.stats.kernel_launches += 2;
    AfterLaunch(c, "krylov");
}

void SpmvFull64(Ctx& c, int precision, const void* vals, const double* x, double* y)
{
    SolverWork& w = Work(c);
    if (w.zeroMask.n != static_cast<size_t>(c.nDofs))
    {
        w.zeroMask.alloc(c.nDofs);
        NG_CUDA(cudaMemsetAsync(w.zeroMask.p, 0, c.nDofs, c.stream));
    }
    c.stats.kernel_launches += 1;
    if (precision == NUTO_GPU_FP32)
        EnsureNb(c, static_cast<const float*>(vals));
    else
        EnsureNb(c, static_cast<const double*>(vals));
    if (precision == NUTO_GPU_FP32)
        SpmvLaunch<float, double, 0>(c, static_cast<const float*>(vals), x, y, nullptr, nullptr, nullptr, FIN_NONE,
                                     w.zeroMask.p);
    else
        SpmvLaunch<double, double, 0>(c, static_cast<const double*>(vals), x, y, nullptr, nullptr, nullptr, FIN_NONE,
                                      w.zeroMask.p);
    AfterLaunch(c, "krylov");
}


// ---- restarted GMRES(m), right Jacobi preconditioning ----------------------------------------------------------
// Arnoldi with classical Gram-Schmidt and one re-orthogonalisation (CGS2) in three passes over the basis
// (projection; update fused with the second projection; second update with the norm). The FP64 Hessenberg column,
// its Givens rotation and the residual estimate are formed by the last block of the second update, so a whole cycle
// is enqueued without a host round trip. The basis is stored in T (FP32 or FP64).
using GL = GmresLayout;

// Projections on the basis in warp units: a unit is 32 x kUnitRows consecutive rows, lane l reading rows
// base + l + 32 k, so every basis vector is streamed once per pass with coalesced loads. Per basis vector and unit
// the lanes' products are summed by a warp butterfly in T; lane i % 32 keeps the running sum of vector i in a
// register, and at the end of the block the warps' sums are added in T and each block adds one FP64 value per
// vector to the accumulator. No FP64 arithmetic per row or per unit (the FP64 pipe is narrow on this part).
constexpr int kUnitRows = 4;
constexpr int kGmresFirstChunk = 4; // iterations enqueued before the first look at the residual estimate
constexpr int kGmresMaxChunk = 16;
constexpr int kProjChunks = (GL::m + 1 + 31) / 32;

template <typename T>
__device__ __forceinline__ T WarpAllSum(T v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
        v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// adds the block's per-vector sums (lane registers acc[c] hold vector lane + 32 c of each warp) to out[0, nv)
template <typename T>
__device__ __forceinline__ void ProjFlush(const T (&acc)[kProjChunks], int nv, double* out)
{
    __shared__ T red[kBS / 32][kProjChunks * 32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int c = 0; c < kProjChunks; ++c)
        red[wid][c * 32 + lane] = acc[c];
    __syncthreads();
    for (int i = threadIdx.x; i < nv; i += blockDim.x)
    {
        T t = T(0);
#pragma unroll
        for (int q = 0; q < kBS / 32; ++q)
            t += red[q][i];
        atomicAdd(out + i, static_cast<double>(t));
    }
}

// products of the unit's rows (held in r[]) with basis vectors 0 .. nv-1, summed into acc
template <typename T>
__device__ __forceinline__ void ProjUnit(const T* __restrict__ V, int64_t n, int nv, int64_t base, bool full,
                                         const T (&r)[kUnitRows], T (&acc)[kProjChunks])
{
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int c = 0; c < kProjChunks; ++c)
    {
        if (c * 32 >= nv)
            break;
        const int iend = min(32, nv - c * 32);
#pragma unroll 4
        for (int ii = 0; ii < iend; ++ii)
        {
            const T* Vi = V + static_cast<int64_t>(c * 32 + ii) * n;
            T p = T(0);
            if (full)
            {
#pragma unroll
                for (int k = 0; k < kUnitRows; ++k)
                    p += Vi[base + 32 * k] * r[k];
            }
            else
            {
#pragma unroll
                for (int k = 0; k < kUnitRows; ++k)
                    if (base + 32 * k < n)
                        p += Vi[base + 32 * k] * r[k];
            }
            p = WarpAllSum(p);
            if (lane == ii)
                acc[c] += p;
        }
    }
}

// acc[i] += V_i . w for i < nv
template <typename T>
__global__ void __launch_bounds__(kBS) k_gm_proj(int64_t n, const T* __restrict__ V, int nv, const T* __restrict__ w,
                                                  double* acc, const int* st)
{
    PdlWait();
    PdlTrigger();
    if (st[ST_STATE] != RUN)
        return;
    const int lane = threadIdx.x & 31;
    T sums[kProjChunks];
#pragma unroll
    for (int c = 0; c < kProjChunks; ++c)
        sums[c] = T(0);
    const int64_t units = (n + 32 * kUnitRows - 1) / (32 * kUnitRows);
    const int64_t warps = static_cast<int64_t>(gridDim.x) * (kBS / 32);
    for (int64_t u = blockIdx.x * static_cast<int64_t>(kBS / 32) + (threadIdx.x >> 5); u < units; u += warps)
    {
        const int64_t base = u * 32 * kUnitRows + lane;
        const bool full = (u + 1) * 32 * kUnitRows <= n;
        T r[kUnitRows];
#pragma unroll
        for (int k = 0; k < kUnitRows; ++k)
            r[k] = base + 32 * k < n ? w[base + 32 * k] : T(0);
        ProjUnit(V, n, nv, base, full, r, sums);
    }
    ProjFlush(sums, nv, acc);
}

// w -= sum_i h_i V_i with h the first projection (gs + H1), then acc2[i] += V_i . w: the update of classical
// Gram-Schmidt and the re-orthogonalisation's projection in one pass (the unit's V values are re-read from cache)
template <typename T>
__global__ void __launch_bounds__(kBS) k_gm_update_proj(int64_t n, const T* __restrict__ V, int nv, const double* h,
                                                         T* __restrict__ w, double* acc2, const int* st)
{
    PdlWait();
    PdlTrigger();
    __shared__ T hs[GL::m + 1];
    if (st[ST_STATE] != RUN)
        return;
    for (int i = threadIdx.x; i < nv; i += blockDim.x)
        hs[i] = static_cast<T>(h[i]);
    __syncthreads();
    const int lane = threadIdx.x & 31;
    T sums[kProjChunks];
#pragma unroll
    for (int c = 0; c < kProjChunks; ++c)
        sums[c] = T(0);
    const int64_t units = (n + 32 * kUnitRows - 1) / (32 * kUnitRows);
    const int64_t warps = static_cast<int64_t>(gridDim.x) * (kBS / 32);
    for (int64_t u = blockIdx.x * static_cast<int64_t>(kBS / 32) + (threadIdx.x >> 5); u < units; u += warps)
    {
        const int64_t base = u * 32 * kUnitRows + lane;
        const bool full = (u + 1) * 32 * kUnitRows <= n;
        T r[kUnitRows];
#pragma unroll
        for (int k = 0; k < kUnitRows; ++k)
            r[k] = base + 32 * k < n ? w[base + 32 * k] : T(0);
#pragma unroll 4
        for (int i = 0; i < nv; ++i)
        {
            const T hi = hs[i];
            const T* Vi = V + static_cast<int64_t>(i) * n;
#pragma unroll
            for (int k = 0; k < kUnitRows; ++k)
                if (base + 32 * k < n)
                    r[k] -= hi * Vi[base + 32 * k];
        }
#pragma unroll
        for (int k = 0; k < kUnitRows; ++k)
            if (base + 32 * k < n)
                w[base + 32 * k] = r[k];
        ProjUnit(V, n, nv, base, full, r, sums);
    }
    ProjFlush(sums, nv, acc2);
}

// w -= sum_i h_i V_i with h the second projection (gs + H2), |w|^2; the last block completes Arnoldi column j:
// H(:, j) = h1 + h2, H(j+1, j) = |w|, earlier rotations applied, new rotation formed, residual estimate |g(j+1)|
// tested. Row sums of |w|^2 are formed in T per thread and block, one FP64 atomic per block.
template <typename T>
__global__ void __launch_bounds__(kBS) k_gm_update(int64_t n, const T* __restrict__ V, int nv, double* gs, T* w,
                                                    int* st, int j)
{
    PdlWait();
    PdlTrigger();
    __shared__ T sh[kBS / 32];
    __shared__ T hs[GL::m + 1];
    if (st[ST_STATE] != RUN)
        return;
    const double* h = gs + GL::H2;
    for (int i = threadIdx.x; i < nv; i += blockDim.x)
        hs[i] = static_cast<T>(h[i]);
    __syncthreads();
    T nrm = T(0);
    for (int64_t r = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; r < n;
         r += static_cast<int64_t>(gridDim.x) * blockDim.x)
    {
        T a = w[r];
        for (int i = 0; i < nv; ++i)
            a -= hs[i] * V[static_cast<int64_t>(i) * n + r];
        w[r] = a;
        nrm += a * a;
    }
    nrm = WarpAllSum(nrm);
    if ((threadIdx.x & 31) == 0)
        sh[threadIdx.x >> 5] = nrm;
    __syncthreads();
    if (threadIdx.x == 0)
    {
        T t = T(0);
        for (int q = 0; q < static_cast<int>(blockDim.x >> 5); ++q)
            t += sh[q];
        atomicAdd(gs + GL::ACC, static_cast<double>(t));
    }
    if (LastBlock(st + ST_COUNTER) && threadIdx.x == 0)
    {
        st[ST_COUNTER] = 0;
        double* H = gs + GL::H + static_cast<int64_t>(j) * (GL::m + 1);
        for (int i = 0; i <= j; ++i)
        {
            H[i] = VRead(gs + GL::H1 + i) + VRead(gs + GL::H2 + i);
            gs[GL::H1 + i] = 0.;
            gs[GL::H2 + i] = 0.;
        }
        const double hn = sqrt(VRead(gs + GL::ACC));
        gs[GL::ACC] = 0.;
        // earlier rotations
        for (int i = 0; i < j; ++i)
        {
            const double c = gs[GL::CS + i], s = gs[GL::SN + i];
            const double a = H[i], b = H[i + 1];
            H[i] = c * a + s * b;
            H[i + 1] = -s * a + c * b;
        }
        const double a = H[j], b = hn;
        const double r = hypot(a, b);
        const double c = r > 0. ? a / r : 1., s = r > 0. ? b / r : 0.;
        gs[GL::CS + j] = c;
        gs[GL::SN + j] = s;
        H[j] = r;
        H[j + 1] = 0.;
        const double gj = gs[GL::G + j];
        gs[GL::G + j] = c * gj;
        gs[GL::G + j + 1] = -s * gj;
        gs[GL::NRM] = hn;
        st[ST_ITERS] += 1;
        st[ST_JDONE] = j + 1;
        const double res = fabs(gs[GL::G + j + 1]);
        if (!isfinite(res) || !isfinite(hn))
            st[ST_STATE] = NONFINITE;
        else if (res * res <= gs[GL::TOL2] || hn == 0.)
            st[ST_STATE] = CONVERGED;
    }
}

// v_j = w / nrm; z = dinv v_j (Jacobi; z == nullptr when the multigrid cycle computes z)
template <typename T>
__global__ void __launch_bounds__(kBS) k_gm_normalize(int64_t n, const T* __restrict__ w, T* vj, T* z,
                                                       const T* __restrict__ dinv, const double* gs, const int* st)
{
    PdlWait();
    PdlTrigger();
    if (st[ST_STATE] != RUN)
        return;
    const T inv = static_cast<T>(1. / gs[GL::NRM]);
    for (int64_t r = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; r < n;
         r += static_cast<int64_t>(gridDim.x) * blockDim.x)
    {
        const T v = w[r] * inv;
        vj[r] = v;
        if (z)
            z[r] = dinv[r] * v;
    }
}

// w = rhs - w (w holds A x) or w = rhs (first cycle); |w|^2; last block: beta, g, state
template <typename T>
__global__ void __launch_bounds__(kBS) k_gm_start(int64_t n, const T* __restrict__ rhs, T* w, int subtract, double* gs,
                                                   int* st)
{
    __shared__ double sh[kBS / 32];
    double nrm = 0;
    for (int64_t r = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; r < n;
         r += static_cast<int64_t>(gridDim.x) * blockDim.x)
    {
        const T a = subtract ? rhs[r] - w[r] : rhs[r];
        w[r] = a;
        nrm += static_cast<double>(a) * static_cast<double>(a);
    }
    BlockAccumulate(nrm, gs + GL::ACC, sh);
    if (LastBlock(st + ST_COUNTER) && threadIdx.x == 0)
    {
        st[ST_COUNTER] = 0;
        const double beta = sqrt(VRead(gs + GL::ACC));
        gs[GL::ACC] = 0.;
        gs[GL::BETA] = beta;
        gs[GL::NRM] = beta;
        gs[GL::G] = beta;
        for (int i = 1; i <= GL::m; ++i)
            gs[GL::G + i] = 0.;
        st[ST_JDONE] = 0;
        if (!isfinite(beta))
            st[ST_STATE] = NONFINITE;
        else if (beta * beta <= gs[GL::TOL2])
            st[ST_STATE] = CONVERGED;
        else
            st[ST_STATE] = RUN;
    }
}

// x += dinv (sum_i y_i V_i) (Jacobi) or x += sum_i y_i Z_i (flexible form, dinv == nullptr)
template <typename T>
__global__ void __launch_bounds__(kBS) k_gm_solution(int64_t n, const T* __restrict__ V, int k, const double* gs,
                                                      const T* __restrict__ dinv, T* x)
{
    __shared__ T ys[GL::m];
    for (int i = threadIdx.x; i < k; i += blockDim.x)
        ys[i] = static_cast<T>(gs[GL::Y + i]);
    __syncthreads();
    for (int64_t r = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; r < n;
         r += static_cast<int64_t>(gridDim.x) * blockDim.x)
    {
        T a = T(0);
        for (int i = 0; i < k; ++i)
            a += ys[i] * V[static_cast<int64_t>(i) * n + r];
        x[r] += dinv ? dinv[r] * a : a;
    }
}

// rhs in T: mask0(b) * scale (scale from k_rhs_norm)
template <typename T>
__global__ void k_gm_rhs(int64_t n, const uint8_t* __restrict__ mask, const double* __restrict__ b, const double* sc,
                         T* rhs, T* x)
{
    const int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
    if (i >= n)
        return;
    rhs[i] = mask[i] ? T(0) : static_cast<T>(b[i] * sc[SC_SCALE]);
    x[i] = T(0);
}

template <typename T, typename TV>
static int GmresSolve(Ctx& c, const TV* vals, const double* b, double* x64, bool addToX, double rtol, int maxit,
                      int* iters, double* relres)
{
    SolverWork& w = Work(c);
    KVecs<T>* kp;
    GVecs<T>* gp;
    if constexpr (sizeof(T) == 4)
    {
        kp = &w.v32;
        gp = &w.g32;
    }
    else
    {
        kp = &w.v64;
        gp = &w.g64;
    }
    KVecs<T>& K = *kp;
    GVecs<T>& G = *gp;
    const int64_t n = c.nDofs;
    K.ensure(n);
    const int m = c.gmresRestart > 1 ? std::min(c.gmresRestart, static_cast<int>(GL::m)) : kGmresRestart;
    G.ensure(n, m);
    if (w.gsc.n != static_cast<size_t>(GL::SIZE))
    {
        w.gsc.alloc(GL::SIZE);
        if (!w.hG)
            NG_CUDA(cudaMallocHost(&w.hG, GL::SIZE * sizeof(double)));
    }
    double* sc = w.scal.p;
    int* st = w.stat.p;
    double* gs = w.gsc.p;
    NG_CUDA(cudaMemsetAsync(sc, 0, SC_COUNT * sizeof(double), c.stream));
    NG_CUDA(cudaMemsetAsync(st, 0, ST_COUNT * sizeof(int), c.stream));
    NG_CUDA(cudaMemsetAsync(gs, 0, GL::SIZE * sizeof(double), c.stream));
    const int grid = GridFor(c, n);
    // projection kernels: warp units of 32 kUnitRows rows, four blocks per SM
    const int64_t units = (n + 32 * kUnitRows - 1) / (32 * kUnitRows);
    const int gridP = static_cast<int>(std::max<int64_t>(1, std::min<int64_t>((units + kBS / 32 - 1) / (kBS / 32),
                                                                             static_cast<int64_t>(c.smCount) * 4)));
    const unsigned g256 = static_cast<unsigned>((n + 255) / 256);
    const bool amg = c.precond == NUTO_GPU_PRECOND_AMG;
    EnsureNb(c, vals);
    if (amg)
    {
        AmgSetup<TV>(c, vals);
        G.ensureZ();
    }
    else
        k_diag_inv<TV, T><<<g256, 256, 0, c.stream>>>(n, c.dRowPtr.p, c.dColIdx.p, vals, c.dMask.p, K.dinv.p);
    k_rhs_norm<<<grid, kBS, 0, c.stream>>>(n, c.dMask.p, b, sc, st, rtol, sizeof(T) == 4 ? 1 : 0);
    // rhs (scaled) in K.r, solution in K.x; tolerance (rtol relative to the scaled rhs) to the GMRES block
    k_gm_rhs<T><<<g256, 256, 0, c.stream>>>(n, c.dMask.p, b, sc, K.r.p, K.x.p);
    AfterLaunch(c, "gmres set-up");
    c.stats.kernel_launches += 3;
    NG_CUDA(cudaMemcpyAsync(gs + GL::TOL2, sc + SC_TOL2, sizeof(double), cudaMemcpyDeviceToDevice, c.stream));
    int total = 0;
    int state = RUN;
    double relEst = 1.;
    std::vector<double> history;
    double beta0 = -1.;
    bool first = true;
    while (total < maxit)
    {
        // r = rhs - A x, v_0 = r / |r|
        if (!first)
            SpmvTimed<TV, T, 0>(c, vals, K.x.p, G.w.p, nullptr, nullptr, nullptr, FIN_NONE, c.dMask.p);
        c.stats.kernel_launches += 2;
        k_gm_start<T><<<grid, kBS, 0, c.stream>>>(n, K.r.p, G.w.p, first ? 0 : 1, gs, st);
        first = false;
        NG_CUDA(LaunchPdl(k_gm_normalize<T>, grid, kBS, 0, c.stream, n, G.w.p, G.V.p, amg ? nullptr : G.z.p, K.dinv.p,
                          gs, st));
        const int cols = std::min(m, maxit - total);
        // The cycle is enqueued in chunks: after each chunk the host reads the state and the residual estimate and
        // sizes the next chunk from the observed convergence rate (the iterations still needed, 1 .. 16). Kernels
        // of iterations enqueued after convergence return at once but still cost a launch each (about 140 per
        // iteration with the multigrid sweep), so a cycle is never enqueued far past the expected convergence.
        int j = 0, chunk = kGmresFirstChunk, jCheck = 0;
        double resCheck = -1.;
        while (j < cols)
        {
            const int jEnd = std::min(cols, j + chunk);
            for (; j < jEnd; ++j)
            {
                T* vj1 = G.V.p + static_cast<int64_t>(j + 1) * n;
                T* zj = amg ? G.Z.p + static_cast<int64_t>(j) * n : G.z.p;
                if (amg)
                    AmgApply<T>(c, G.V.p + static_cast<int64_t>(j) * n, zj, st, false);
                SpmvTimed<TV, T, 0>(c, vals, zj, G.w.p, nullptr, nullptr, st, FIN_NONE, c.dMask.p);
                c.stats.kernel_launches += 3 + (j + 1 < cols ? 1 : 0);
                NG_CUDA(LaunchPdl(k_gm_proj<T>, gridP, kBS, 0, c.stream, n, G.V.p, j + 1, G.w.p, gs + GL::H1, st));
                NG_CUDA(LaunchPdl(k_gm_update_proj<T>, gridP, kBS, 0, c.stream, n, G.V.p, j + 1, gs + GL::H1, G.w.p,
                                  gs + GL::H2, st));
                NG_CUDA(LaunchPdl(k_gm_update<T>, grid, kBS, 0, c.stream, n, G.V.p, j + 1, gs, G.w.p, st, j));
                if (j + 1 < cols)
                    NG_CUDA(LaunchPdl(k_gm_normalize<T>, grid, kBS, 0, c.stream, n, G.w.p, vj1, amg ? nullptr : G.z.p,
                                      K.dinv.p, gs, st));
            }
            if (j >= cols)
                break;
            NG_CUDA(cudaMemcpyAsync(w.hStat, st, ST_COUNT * sizeof(int), cudaMemcpyDeviceToHost, c.stream));
            NG_CUDA(cudaMemcpyAsync(w.hG + GL::G, gs + GL::G, (GL::SIZE - GL::G) * sizeof(double),
                                    cudaMemcpyDeviceToHost, c.stream));
            WaitStream(c);
            if (w.hStat[ST_STATE] != RUN)
                break;
            const int jd = w.hStat[ST_JDONE];
            const double res = std::fabs(w.hG[GL::G + jd]);
            const double tol = std::sqrt(std::max(w.hG[GL::TOL2], 0.));
            const double ref = resCheck > 0. ? resCheck : w.hG[GL::BETA];
            const int span = jd - (resCheck > 0. ? jCheck : 0);
            chunk = kGmresMaxChunk;
            if (span > 0 && ref > 0. && res > 0. && res < ref && tol > 0.)
            {
                const double rate = std::log(res / ref) / span; // log of the mean reduction per iteration
                const double need = std::log(tol / res) / rate;
                chunk = static_cast<int>(std::min<double>(kGmresMaxChunk, std::max(1., std::ceil(need))));
            }
            resCheck = res;
            jCheck = jd;
        }
        AfterLaunch(c, "gmres cycle");
        NG_CUDA(cudaMemcpyAsync(w.hG, gs, GL::SIZE * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
        NG_CUDA(cudaMemcpyAsync(w.hStat, st, ST_COUNT * sizeof(int), cudaMemcpyDeviceToHost, c.stream));
        WaitStream(c);
        SpmvCollect(c);
        state = w.hStat[ST_STATE];
        const int k = w.hStat[ST_JDONE];
        total = w.hStat[ST_ITERS];
        if (beta0 < 0.)
            beta0 = w.hG[GL::BETA];
        if (state == NONFINITE)
            break;
        if (k > 0)
        {
            // back substitution R y = g on the host (k <= m)
            double* y = w.hG + GL::Y;
            for (int i = k - 1; i >= 0; --i)
            {
                double s = w.hG[GL::G + i];
                for (int l = i + 1; l < k; ++l)
                    s -= w.hG[GL::H + l * (GL::m + 1) + i] * y[l];
                const double d = w.hG[GL::H + i * (GL::m + 1) + i];
                y[i] = d != 0. ? s / d : 0.;
            }
            NG_CUDA(cudaMemcpyAsync(gs + GL::Y, y, k * sizeof(double), cudaMemcpyHostToDevice, c.stream));
            k_gm_solution<T><<<grid, kBS, 0, c.stream>>>(n, amg ? G.Z.p : G.V.p, k, gs, amg ? nullptr : K.dinv.p,
                                                         K.x.p);
            AfterLaunch(c, "gmres solution");
            c.stats.kernel_launches += 1;
            relEst = beta0 > 0. ? std::fabs(w.hG[GL::G + k]) / beta0 : 0.;
        }
        if (state != RUN)
            break;
        // stagnation: eight full cycles that together reduced the residual estimate by less than 10 % end the solve
        // (restarted GMRES can stall on indefinite systems); the caller gets the iterate and a non-converged status
        history.push_back(relEst);
        if (k == cols && history.size() > 8 && relEst > 0.9 * history[history.size() - 9])
        {
            state = BREAKDOWN;
            break;
        }
        // restart: the state flag is reset by k_gm_start
    }
    if (state == CONVERGED && beta0 == 0.)
        relEst = 0.;
    if (iters)
        *iters = total;
    if (relres)
        *relres = relEst;
    c.stats.krylov_iterations += total;
    if (state == NONFINITE)
        throw Error{NUTO_GPU_ENAN, "non-finite value in the GMRES iteration (iteration " + std::to_string(total) + ")"};
    k_unscale<T><<<g256, 256, 0, c.stream>>>(n, K.x.p, sc, x64, addToX ? 1 : 0);
    AfterLaunch(c, "gmres unscale");
    c.stats.kernel_launches += 1;
    return state == CONVERGED ? CONVERGED : (state == RUN ? RUN : state);
}

// Runs one Krylov solve of the constrained system with values `vals` (type TV) in arithmetic T, right-hand side
// b (FP64, combined layout), solution written (or added) to x64. Returns the status.
template <typename T, typename TV>
static int KrylovSolve(Ctx& c, int method, const TV* vals, const double* b, double* x64, bool addToX, double rtol,
                       int maxit, int* iters, double* relres)
{
    if (method == NUTO_GPU_SOLVER_GMRES)
        return GmresSolve<T, TV>(c, vals, b, x64, addToX, rtol, maxit, iters, relres);
    const bool pcg = method == NUTO_GPU_SOLVER_PCG;
    SolverWork& w = Work(c);
    KVecs<T>* vp;
    if constexpr (sizeof(T) == 4)
        vp = &w.v32;
    else
        vp = &w.v64;
    KVecs<T>& V = *vp;
    const int64_t n = c.nDofs;
    V.ensure(n);
    double* sc = w.scal.p;
    int* st = w.stat.p;
    NG_CUDA(cudaMemsetAsync(sc, 0, SC_COUNT * sizeof(double), c.stream));
    NG_CUDA(cudaMemsetAsync(st, 0, ST_COUNT * sizeof(int), c.stream));
    const int grid = GridFor(c, n);
    const bool amg = pcg && c.precond == NUTO_GPU_PRECOND_AMG;
    EnsureNb(c, vals);
    if (amg)
        AmgSetup<TV>(c, vals);
    else
        k_diag_inv<TV, T><<<static_cast<unsigned>((n + 255) / 256), 256, 0, c.stream>>>(
                n, c.dRowPtr.p, c.dColIdx.p, vals, c.dMask.p, V.dinv.p);
    k_rhs_norm<<<grid, kBS, 0, c.stream>>>(n, c.dMask.p, b, sc, st, rtol, sizeof(T) == 4 ? 1 : 0);
    if (amg)
    {
        // x = 0, r = b, p = 0; z = M^-1 r; rho = r.z; p = z
        k_krylov_init<T, false><<<grid, kBS, 0, c.stream>>>(n, c.dMask.p, b, V.x.p, V.r.p, V.rh.p, V.p.p, V.v.p,
                                                             V.z.p, V.dinv.p, sc, st);
        AmgApply<T>(c, V.r.p, V.z.p, st, true);
        k_pcg_rz<T><<<grid, kBS, 0, c.stream>>>(n, V.r.p, V.z.p, sc, st, 1);
        k_pcg_dir<T><<<grid, kBS, 0, c.stream>>>(n, V.p.p, V.z.p, sc, st);
        c.stats.kernel_launches += 2;
    }
    else if (pcg)
        k_krylov_init<T, true><<<grid, kBS, 0, c.stream>>>(n, c.dMask.p, b, V.x.p, V.r.p, V.rh.p, V.p.p, V.v.p,
                                                            V.z.p, V.dinv.p, sc, st);
    else
        k_krylov_init<T, false><<<grid, kBS, 0, c.stream>>>(n, c.dMask.p, b, V.x.p, V.r.p, V.rh.p, V.p.p, V.v.p,
                                                             V.z.p, V.dinv.p, sc, st);
    AfterLaunch(c, "krylov");
    // Iterations are enqueued in chunks with a look at the state in between; with the multigrid cycle (about 70
    // launches per iteration even when they return at once after convergence) the next chunk is sized from the
    // observed reduction of |r|^2, as in the GMRES cycle.
    int chunk = amg ? kGmresFirstChunk : 16;
    int done = 0, itCheck = 0;
    double rrCheck = -1.;
    int state = RUN;
    while (done < maxit)
    {
        const int nIt = std::min(chunk, maxit - done);
        for (int k = 0; k < nIt; ++k)
        {
            if (pcg)
            {
                SpmvTimed<TV, T, 1>(c, vals, V.p.p, V.q.p, V.p.p, sc, st, FIN_PCG_ALPHA, c.dMask.p);
                c.stats.kernel_launches += 2;
                k_pcg_update<T><<<grid, kBS, 0, c.stream>>>(n, V.x.p, V.r.p, V.p.p, V.q.p, V.z.p,
                                                            amg ? nullptr : V.dinv.p, sc, st);
                if (amg)
                {
                    AmgApply<T>(c, V.r.p, V.z.p, st, true);
                    k_pcg_rz<T><<<grid, kBS, 0, c.stream>>>(n, V.r.p, V.z.p, sc, st, 0);
                    c.stats.kernel_launches += 1;
                }
                k_pcg_dir<T><<<grid, kBS, 0, c.stream>>>(n, V.p.p, V.z.p, sc, st);
            }
            else
            {
                k_bicg_p<T><<<grid, kBS, 0, c.stream>>>(n, V.p.p, V.r.p, V.v.p, V.ph.p, V.dinv.p, sc, st);
                SpmvTimed<TV, T, 1>(c, vals, V.ph.p, V.v.p, V.rh.p, sc, st, FIN_BICG_ALPHA, c.dMask.p);
                c.stats.kernel_launches += 3;
                k_bicg_s<T><<<grid, kBS, 0, c.stream>>>(n, V.s.p, V.r.p, V.v.p, V.sh.p, V.dinv.p, sc, st);
                SpmvTimed<TV, T, 2>(c, vals, V.sh.p, V.t.p, V.s.p, sc, st, FIN_BICG_OMEGA, c.dMask.p);
                k_bicg_x<T><<<grid, kBS, 0, c.stream>>>(n, V.x.p, V.r.p, V.rh.p, V.ph.p, V.s.p, V.sh.p, V.t.p, sc, st);
            }
        }
        AfterLaunch(c, "krylov");
        done += nIt;
        NG_CUDA(cudaMemcpyAsync(w.hStat, st, ST_COUNT * sizeof(int), cudaMemcpyDeviceToHost, c.stream));
        NG_CUDA(cudaMemcpyAsync(w.hScal, sc, SC_COUNT * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
        WaitStream(c);
        SpmvCollect(c);
        state = w.hStat[ST_STATE];
        if (state != RUN)
            break;
        if (amg)
        {
            const int itNow = w.hStat[ST_ITERS];
            const double rr = w.hScal[SC_RR], tol2 = w.hScal[SC_TOL2];
            const double ref = rrCheck > 0. ? rrCheck : w.hScal[SC_BB] * w.hScal[SC_SCALE] * w.hScal[SC_SCALE];
            const int span = itNow - itCheck;
            chunk = kGmresMaxChunk;
            if (span > 0 && ref > 0. && rr > 0. && rr < ref && tol2 > 0.)
            {
                const double need = std::log(tol2 / rr) / (std::log(rr / ref) / span);
                chunk = static_cast<int>(std::min<double>(kGmresMaxChunk, std::max(1., std::ceil(need))));
            }
            rrCheck = rr;
            itCheck = itNow;
        }
    }
    const int it = w.hStat[ST_ITERS];
    const double bb = w.hScal[SC_BB] * w.hScal[SC_SCALE] * w.hScal[SC_SCALE];
    const double rel = bb > 0 ? std::sqrt(w.hScal[SC_RR] / bb) : 0.;
    if (iters)
        *iters = it;
    if (relres)
        *relres = rel;
    c.stats.krylov_iterations += it;
    if (state == NONFINITE)
    {
        char buf[256];
        std::snprintf(buf, sizeof(buf),
                      "non-finite value in the Krylov iteration (%s, iteration %d, rho %.3e, alpha %.3e, omega %.3e, "
                      "beta %.3e, |r|^2 %.3e)",
                      pcg ? "PCG" : "BiCGStab", it, w.hScal[SC_RHO], w.hScal[SC_ALPHA], w.hScal[SC_OMEGA],
                      w.hScal[SC_BETA], w.hScal[SC_RR]);
        throw Error{NUTO_GPU_ENAN, buf};
    }
    // breakdown or iteration cap: keep the iterate (Newton refines it) but report non-convergence by the rel value
    k_unscale<T><<<static_cast<unsigned>((n + 255) / 256), 256, 0, c.stream>>>(n, V.x.p, sc, x64, addToX ? 1 : 0);
    c.stats.kernel_launches += 4; // diagonal, rhs norm, init, unscale
    AfterLaunch(c, "krylov");
    return state;
}

template <typename T, typename TV>
int KrylovSolveExport(Ctx& c, int method, const TV* vals, const double* b, double* x64, bool add, double rtol,
                      int maxit, int* iters, double* relres)
{
    return KrylovSolve<T, TV>(c, ResolveMethod(c, method), vals, b, x64, add, rtol, maxit, iters, relres);
}
template int KrylovSolveExport<float, float>(Ctx&, int, const float*, const double*, double*, bool, double, int,
                                             int*, double*);
template int KrylovSolveExport<double, double>(Ctx&, int, const double*, const double*, double*, bool, double, int,
                                               int*, double*);
template int KrylovSolveExport<double, float>(Ctx&, int, const float*, const double*, double*, bool, double, int,
                                              int*, double*);

__global__ void k_residual64(int64_t n, const uint8_t* __restrict__ mask, const double* __restrict__ b,
                             const double* __restrict__ kx, double* __restrict__ r)
{
    const int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
    if (i < n)
        r[i] = mask[i] ? 0. : b[i] - kx[i];
}

void Residual64(Ctx& c, const double* b, const double* kx, double* r)
{
    k_residual64<<<static_cast<unsigned>((c.nDofs + 255) / 256), 256, 0, c.stream>>>(c.nDofs, c.dMask.p, b, kx, r);
    AfterLaunch(c, "krylov");
}

int ResolveMethod(const Ctx& c, int method)
{
    if (method == NUTO_GPU_SOLVER_PCG || method == NUTO_GPU_SOLVER_BICGSTAB || method == NUTO_GPU_SOLVER_GMRES)
        return method;
    return c.prm.kind == NUTO_GPU_MB_LINEAR_ELASTIC ? NUTO_GPU_SOLVER_PCG : NUTO_GPU_SOLVER_GMRES;
}

// nuto_gpu_solve: FP64 solve, or FP32 Krylov inside an FP64 iterative refinement (r = b - K x in FP64 with the
// FP32 values) until |r| <= rtol |b|.
int SolveLinear(Ctx& c, int precision, int method, const void* values, const double* b, double* x, double rtol,
                int maxit, int* iters, double* relres)
{
    SolverWork& w = Work(c);
    const int meth = ResolveMethod(c, method);
    c.stats.krylov_iterations = 0;
    if (precision == NUTO_GPU_FP64)
    {
        int it = 0;
        double rel = 0;
        const int st = KrylovSolve<double, double>(c, meth, static_cast<const double*>(values), b, x, false, rtol,
                                                   maxit, &it, &rel);
        if (iters)
            *iters = it;
        if (relres)
            *relres = rel;
        return st == CONVERGED ? NUTO_GPU_OK : NUTO_GPU_ENOCONV;
    }
    const int64_t n = c.nDofs;
    w.tmp.alloc(n);
    w.rhs.alloc(n);
    const double bnorm = MaskedNorm(c, b);
    NG_CUDA(cudaMemsetAsync(x, 0, n * sizeof(double), c.stream));
    NG_CUDA(cudaMemcpyAsync(w.rhs.p, b, n * sizeof(double), cudaMemcpyDeviceToDevice, c.stream));
    int total = 0;
    double rel = bnorm > 0 ? 1. : 0.;
    for (int sweep = 0; sweep < 30 && rel > rtol && total < maxit; ++sweep)
    {
        const double inner = std::max(rtol / std::max(rel, 1e-300), 1e-5);
        int it = 0;
        KrylovSolve<float, float>(c, meth, static_cast<const float*>(values), w.rhs.p, x, true,
                                  std::min(inner, 0.5), maxit - total, &it, nullptr);
        total += it;
        // r = b - K x (FP64 vectors, FP32 values), constrained rows zero
        SpmvFull64(c, NUTO_GPU_FP32, values, x, w.tmp.p);
        Residual64(c, b, w.tmp.p, w.rhs.p);
        rel = bnorm > 0 ? MaskedNorm(c, w.rhs.p) / bnorm : 0.;
    }
    if (iters)
        *iters = total;
    if (relres)
        *relres = rel;
    return rel <= rtol ? NUTO_GPU_OK : NUTO_GPU_ENOCONV;
}

} // namespace nuto_gpu
