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

struct SolverWork
{
    DBuf<double> scal;
    DBuf<int> stat;
    double* hScal = nullptr; // pinned
    int* hStat = nullptr;    // pinned
    KVecs<float> v32;
    KVecs<double> v64;
    // Newton buffers
    DBuf<float> K32;
    DBuf<double> K64;
    DBuf<double> f, rhs, dx, db, x0, xs, tmp;
    DBuf<uint8_t> zeroMask;
    cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
    ~SolverWork();
};

SolverWork& Work(Ctx& c);

// |mask0(v)|_2 on the device, result copied to the host (synchronises the stream)
double MaskedNorm(Ctx& c, const double* v);
// y = K x for CSR values of the given precision, all rows (no constraint masking), FP64 vectors
void SpmvFull64(Ctx& c, int precision, const void* vals, const double* x, double* y);
// r = mask0(b - kx)
void Residual64(Ctx& c, const double* b, const double* kx, double* r);
// PCG for the symmetric integrands (or when asked), BiCGStab otherwise
bool UsePcg(const Ctx& c, int method);
// one Krylov solve in arithmetic T on values of type TV; adds to (add) or overwrites x64; returns SolverState
template <typename T, typename TV>
int KrylovSolveExport(Ctx& c, bool pcg, const TV* vals, const double* b, double* x64, bool add, double rtol,
                      int maxit, int* iters, double* relres);

} // namespace nuto_gpu
