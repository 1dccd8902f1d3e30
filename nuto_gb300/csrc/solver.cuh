// Solver workspace shared by the Krylov kernels and the quasistatic Newton driver.
#pragma once

#include "internal.cuh"

namespace nuto_gpu
{

// device scalar slots (doubles)
enum Scal
{
    SC_BB = 0,   // |b|^2
    SC_TOL2,     // rtol^2 |b|^2
    SC_SCALE,    // 1 / |b| (FP32 right-hand side scaling)
    SC_RHO,      // PCG: r.z ; BiCGStab: rhat.r
    SC_RHO_OLD,
    SC_ALPHA,
    SC_BETA,
    SC_OMEGA,
    SC_ACC0,     // accumulators
    SC_ACC1,
    SC_ACC2,
    SC_RR,       // last |r|^2
    SC_COUNT
};

// device status slots (ints)
enum Stat
{
    ST_STATE = 0, // 0 running, 1 converged, 2 breakdown, 3 non-finite
    ST_ITERS,
    ST_COUNTER,   // last-block counter of the fused reductions
    ST_HALF,      // BiCGStab: converged on s
    ST_JDONE,     // GMRES: Arnoldi columns completed in the current cycle
    ST_COUNT
};

enum SolverState
{
    RUN = 0,
    CONVERGED = 1,
    BREAKDOWN = 2,
    NONFINITE = 3
};

template <typename T>
struct KVecs
{
    DBuf<T> x, r, rh, p, v, s, t, ph, sh, z, q, dinv;
    int64_t n = 0;
    void ensure(int64_t count)
    {
        if (n == count)
            return;
        for (DBuf<T>* b : {&x, &r, &rh, &p, &v, &s, &t, &ph, &sh, &z, &q, &dinv})
            b->alloc(count);
        n = count;
    }
};

// GMRES restart length: default, and the largest the scalar block holds (NUTO_GPU_GMRES_RESTART picks another)
constexpr int kGmresRestart = 80;
constexpr int kGmresMax = 160;

// GMRES workspace: Krylov basis V (m + 1 vectors of n), work vectors and the FP64 Arnoldi scalars.
template <typename T>
struct GVecs
{
    DBuf<T> V, w, z;
    DBuf<T> Z; // preconditioned basis of the flexible form (m vectors), allocated on first use
    int64_t n = 0;
    int m = 0;
    void ensure(int64_t count, int restart)
    {
        if (n == count && m == restart)
            return;
        V.alloc(static_cast<size_t>(count) * (restart + 1));
        w.alloc(count);
        z.alloc(count);
        Z.free();
        n = count;
        m = restart;
    }
    void ensureZ()
    {
        if (Z.n != static_cast<size_t>(n) * m)
            Z.alloc(static_cast<size_t>(n) * m);
    }
};

// offsets into the GMRES scalar block (doubles)
struct GmresLayout
{
    static constexpr int m = kGmresMax;          // capacity; a cycle uses the first restart columns
    static constexpr int H = 0;                  // (m + 1) x m, column-major
    static constexpr int G = H + (m + 1) * m;    // m + 1: rotated right-hand side
    static constexpr int CS = G + m + 1;         // m: Givens cosines
    static constexpr int SN = CS + m;            // m: Givens sines
    static constexpr int H1 = SN + m;            // m + 1: first projection accumulators
    static constexpr int H2 = H1 + m + 1;        // m + 1: second projection accumulators
    static constexpr int Y = H2 + m + 1;         // m: least-squares solution
    static constexpr int ACC = Y + m;            // norm accumulator
    static constexpr int NRM = ACC + 1;          // normalisation of the next basis vector
    static constexpr int BETA = NRM + 1;         // |r| at the start of the cycle
    static constexpr int TOL2 = BETA + 1;        // rtol^2 (right-hand side scaled to unit norm)
    static constexpr int SIZE = TOL2 + 1;
};

struct SolverWork
{
    DBuf<double> scal;
    DBuf<int> stat;
    double* hScal = nullptr; // pinned
    int* hStat = nullptr;    // pinned
    KVecs<float> v32;
    KVecs<double> v64;
    GVecs<float> g32;
    GVecs<double> g64;
    DBuf<double> gsc; // GmresLayout
    double* hG = nullptr; // pinned copy of the GMRES scalars
    // Newton buffers
    DBuf<float> K32;
    DBuf<double> K64;
    DBuf<double> f, rhs, dx, db, x0, xs, tmp;
    DBuf<double> refR, refKx; // FP64 refinement of the FP32 Newton solves
    DBuf<float> xsplit;       // 2n: x as (hi, lo) floats for the compensated FP32 product
    DBuf<uint8_t> zeroMask;
    cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
    // CUDA-event pairs around the Krylov SpMV launches, folded into stats at synchronisation points
    std::vector<std::pair<cudaEvent_t, cudaEvent_t>> spmvEv;
    size_t spmvNext = 0;
    ~SolverWork();
};

SolverWork& Work(Ctx& c);

// |mask0(v)|_2 on the device, result copied to the host (synchronises the stream)
double MaskedNorm(Ctx& c, const double* v);
// y = K x for CSR values of the given precision, all rows (no constraint masking), FP64 vectors
void SpmvFull64(Ctx& c, int precision, const void* vals, const double* x, double* y);
// y = K x for FP32 values and FP64 vectors in compensated FP32 arithmetic (about 1e-14 relative to sum |K x|): the
// residual of the FP32 Newton refinement
void SpmvFull64Comp(Ctx& c, const float* vals, const double* x, double* y);
// r = mask0(b - kx)
void Residual64(Ctx& c, const double* b, const double* kx, double* r);
// NUTO_GPU_SOLVER_AUTO resolves to PCG for the symmetric integrands and GMRES otherwise
int ResolveMethod(const Ctx& c, int method);
// one Krylov solve in arithmetic T on values of type TV; adds to (add) or overwrites x64; returns SolverState
template <typename T, typename TV>
int KrylovSolveExport(Ctx& c, int method, const TV* vals, const double* b, double* x64, bool add, double rtol,
                      int maxit, int* iters, double* relres);

} // namespace nuto_gpu
