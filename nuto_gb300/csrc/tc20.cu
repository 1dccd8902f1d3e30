// FP32 tangent of Hex20 cells on the tensor cores: SimpleAssembler::BuildMatrix
// (nuto/mechanics/cell/SimpleAssembler.cpp:100-156) of MomentumBalance::Hessian0
// (nuto/mechanics/integrands/MomentumBalance.h:36-46) with LinearElastic or LocalIsotropicDamage::Tangent
// (nuto/mechanics/constitutive/LocalIsotropicDamage.h:59-68, 115-122) for InterpolationBrickQuadratic cells
// (nuto/mechanics/interpolation/InterpolationBrickQuadratic.cpp:37-262) on a Hex8 coordinate mesh, 3x3x3 Gauss points.
//
// Three kernels per assembly:
//   k_tc20_points   one thread per (cell, point): FP32 geometry from the coordinates relative to the cell's first
//                   node, strain, law, and a record of 6 float4: J^-1, lambda w, mu w, the Voigt vectors
//                   s = dsigma/domega domega/dkappa w and t = deps_eq/deps (loading points only). The loading and
//                   damage branches are the FP64 kernels' (decided in FP32 where an error bound separates the
//                   operands, else from the FP64 strain formed exactly as k_residual forms it).
//   k_tangent_tc20  one block per SM walks the cells. Per cell it forms in shared memory the TF32 operands
//                       A = [ lambda_q w_q g_qa,i | P_q(a,i) ]    rows (i, a)        q = 0..26 | 32 + q
//                           [ mu_q w_q g_qa,i     | 0        ]    rows 64 + (i, a)
//                       B = [ g_qb,j              | Q_q(b,j) ]    rows (j, b)
//                   (g the node gradients, P_q(a) = B_a^T s_q, Q_q(b) = B_b^T t_q) and one thread issues
//                   tcgen05.mma kind::tf32, D = A B^T (M = 128, N = 64, K = 64) into tensor memory. D's top half is
//                   the lambda Gram matrix plus the rank-1 part sum_q P_q Q_q^T, its bottom half the mu Gram matrix
//                   G; the epilogue forms K(a,i; b,j) = D(a,i; b,j) + G(a,j; b,i) + delta_ij sum_k G(a,k; b,k), which
//                   is B_a^T C B_b for C = lambda m m^T + mu diag(2,2,2,1,1,1) plus P_a Q_b^T, and writes the
//                   element matrix [a][i][b][j]. With split 3 every operand is the sum of two TF32 numbers
//                   (hi = round(x), lo = round(x - hi)) and D accumulates lo.hi + hi.lo + hi.hi: about FP32
//                   accuracy (the dropped lo.lo term is 2^-22 relative); split 1 keeps hi.hi only.
//   k_tc20_rows     one warp per displacement node adds its rows of the element matrices over the node's cells in
//                   ascending order into shared rows at the ranks of b and stores the CSR rows once (no atomics:
//                   bitwise reproducible).
// The tensor-memory accumulator is double-buffered (2 x 64 columns): the MMAs of one cell run while the epilogue of
// the previous cell reads its accumulator. The only wait is on the MMA completion barrier; it is bounded by the
// context's spin limit and, when it gives up, sets NUTO_GPU_ETIMEOUT in the status word, waits once more (bounded)
// for the MMAs in flight, frees the tensor memory and returns.
#include "internal.cuh"

#include <algorithm>
#include <cfloat>

namespace nuto_gpu
{

void BuildRelativeCoordinates(Ctx& c);

namespace
{

constexpr int kNd = 20, kNg = 8, kNip = 27;
constexpr int kRecF4 = 6;          // float4 per point record
constexpr int kTcThreads = 512;    // 16 warps: 4 per tensor-memory lane quarter
constexpr int kRowCapTc = 256;     // values per CSR row buffer (81 neighbour nodes x 3 in the interior)
// shared memory of k_tangent_tc20 (bytes)
constexpr int kOpAHi = 0, kOpALo = 32768, kOpBHi = 65536, kOpBLo = 81920, kOpEnd = 98304;
constexpr int kRecOff = kOpEnd;                                // 2 x 27 x 6 float4: this cell's records, the next's
constexpr int kMuOff = kRecOff + 2 * kNip * kRecF4 * 16;       // G rows 0..59, 61 floats each
constexpr int kMuStride = 61;
constexpr int kOutOff = kMuOff + 60 * kMuStride * 4;           // element matrix staging [a][181]
constexpr int kOutStride = 181;
constexpr int kTabOff = kOutOff + kNd * kOutStride * 4;        // dN/dxi of the 20 nodes at the 27 points
constexpr int kBarOff = kTabOff + kNip * kNd * 3 * 4;          // 2 mbarriers, the tensor-memory address
constexpr int kSmemTc = kBarOff + 32;
static_assert(kRecOff % 16 == 0 && kMuOff % 16 == 0 && kOutOff % 16 == 0 && kTabOff % 16 == 0 && kBarOff % 16 == 0,
              "16-byte aligned regions");
static_assert(kSmemTc <= 227 * 1024, "fits one block per SM");
constexpr uint32_t kTmemCols = 128; // two 64-column accumulators
constexpr long long kDrainLimit = 1LL << 22; // the final wait for MMAs in flight after a wait gave up

struct Tc20Args
{
    int64_t nCells, nDofs, nNodesD, geoSize;
    const int32_t* connD;  // planar [node][cell]
    const int64_t* gdofD;
    const float* relX;     // planar [(n * 3 + d)][cell]
    const double* kappa;   // [cell][ip]
    const double* escale;  // per-cell Young's modulus factor (nullptr: 1)
    const double* geo64;   // FP64 geometry cache (the fallback strain)
    int geoStride;
    const double* tabDNg;  // [q][8][3]
    const double* tabDNd;  // [q][20][3]
    const double* tabW;    // [q]
};

struct Tc20RowArgs
{
    int64_t nNodes, nCells, nnz, nRows;
    const int64_t* gdofD;
    const int64_t* cellPtr;
    const int32_t* cellIdx;
    const uint8_t* cellLoc;
    const int64_t* rowPtr;
    const uint8_t* rank; // UU ranks, [(loc * 20 + b)][cell]
    const int32_t* blk;
};

// ---- tcgen05 / mbarrier wrappers (inline PTX, sm_100-class tensor cores) --------------------------------------

// Shared-memory matrix descriptor of a K-major operand without swizzle: 8-row x 16-byte core matrices, the core
// matrices of one row group side by side along K (leading byte offset 128 B), row groups 2048 B apart (stride byte
// offset); bits 46-48 hold the fixed value 0b001 of this descriptor version; layout type 0 (no swizzle).
__device__ __forceinline__ uint64_t SmemDesc(uint32_t addr)
{
    return static_cast<uint64_t>((addr & 0x3FFFFu) >> 4) | (static_cast<uint64_t>(128u >> 4) << 16) |
           (static_cast<uint64_t>(2048u >> 4) << 32) | (1ull << 46);
}
// Instruction descriptor, kind::tf32: D F32 (bits 4-5 = 1), A and B TF32 (bits 7-9, 10-12 = 2), both K-major,
// N >> 3 at bits 17-22, M >> 4 at bits 24-28
constexpr uint32_t kIdesc = (1u << 4) | (2u << 7) | (2u << 10) | ((64u >> 3) << 17) | ((128u >> 4) << 24);

// byte offset of element (r, k) in an operand of the layout above (64 K-columns per row group)
__device__ __forceinline__ int OpOff(int r, int k)
{
    return (r >> 3) * 2048 + (k >> 2) * 128 + (r & 7) * 16 + (k & 3) * 4;
}

__device__ __forceinline__ void TmemAlloc(uint32_t dst, uint32_t cols)
{
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(dst), "r"(cols)
                 : "memory");
}
__device__ __forceinline__ void TmemRelinquish()
{
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void TmemDealloc(uint32_t taddr, uint32_t cols)
{
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(cols) : "memory");
}
__device__ __forceinline__ void TcFenceBefore()
{
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void TcFenceAfter()
{
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void FenceProxyAsync()
{
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void MmaTf32(uint32_t d, uint64_t a, uint64_t b, uint32_t accumulate)
{
    asm volatile("{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
                 "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}" ::"r"(d),
                 "l"(a), "l"(b), "r"(kIdesc), "r"(accumulate)
                 : "memory");
}
__device__ __forceinline__ void MmaCommit(uint32_t bar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar)
                 : "memory");
}
__device__ __forceinline__ void BarInit(uint32_t bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ bool BarTryWait(uint32_t bar, uint32_t parity)
{
    uint32_t ok;
    asm volatile("{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                 "selp.u32 %0, 1, 0, p;\n\t}"
                 : "=r"(ok)
                 : "r"(bar), "r"(parity)
                 : "memory");
    return ok != 0;
}
// bounded wait for the completion of the barrier phase with the given parity
__device__ __forceinline__ bool BarWait(uint32_t bar, uint32_t parity, long long limit)
{
    for (long long i = 0; i < limit; ++i)
        if (BarTryWait(bar, parity))
            return true;
    return false;
}
// 16 consecutive 32-bit columns of this warp's 32 tensor-memory lanes (lane quarter set by taddr's lane field)
__device__ __forceinline__ void TmemLoad16(uint32_t taddr, float (&v)[16])
{
    uint32_t r[16];
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, "
                 "%14, %15}, [%16];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
                   "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]),
                   "=r"(r[15])
                 : "r"(taddr)
                 : "memory");
    // the registers are read only after the load has completed (they are operands of the wait)
    asm volatile("tcgen05.wait::ld.sync.aligned;"
                 : "+r"(r[0]), "+r"(r[1]), "+r"(r[2]), "+r"(r[3]), "+r"(r[4]), "+r"(r[5]), "+r"(r[6]), "+r"(r[7]),
                   "+r"(r[8]), "+r"(r[9]), "+r"(r[10]), "+r"(r[11]), "+r"(r[12]), "+r"(r[13]), "+r"(r[14]),
                   "+r"(r[15])
                 :
                 : "memory");
#pragma unroll
    for (int i = 0; i < 16; ++i)
        v[i] = __uint_as_float(r[i]);
}
// round to the nearest TF32 value (10 explicit mantissa bits), kept in an FP32 container
__device__ __forceinline__ float Tf32Round(float x)
{
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
    return __uint_as_float(r);
}

// ---- records: geometry and law per (cell, point) ------------------------------------------------------------

template <int KIND>
__global__ void __launch_bounds__(128) k_tc20_points(Tc20Args A, LawParams L, const double* __restrict__ u,
                                                      float4* __restrict__ recs, int lawFp64)
{
    constexpr bool LD = KIND == NUTO_GPU_MB_LOCAL_DAMAGE;
    constexpr int CPB = 4; // cells per block: 108 of 128 threads evaluate a point
    __shared__ float sDNg[kNip * kNg * 3];
    __shared__ float sDNd[kNip * kNd * 3];
    __shared__ float sW[kNip];
    __shared__ float sX[CPB][kNg][3];
    __shared__ double sU[CPB][kNd][3];
    const int64_t n = A.nCells;
    const int64_t cell0 = static_cast<int64_t>(blockIdx.x) * CPB;
    for (int i = threadIdx.x; i < kNip * kNg * 3; i += blockDim.x)
        sDNg[i] = static_cast<float>(A.tabDNg[i]);
    for (int i = threadIdx.x; i < kNip * kNd * 3; i += blockDim.x)
        sDNd[i] = static_cast<float>(A.tabDNd[i]);
    for (int i = threadIdx.x; i < kNip; i += blockDim.x)
        sW[i] = static_cast<float>(A.tabW[i]);
    for (int it = threadIdx.x; it < CPB * kNg * 3; it += blockDim.x)
    {
        const int cl = it % CPB, r = it / CPB; // r = node * 3 + d
        const int64_t e = cell0 + cl;
        if (e < n)
            sX[cl][r / 3][r % 3] = A.relX[static_cast<int64_t>(r) * n + e];
    }
    for (int it = threadIdx.x; it < CPB * kNd; it += blockDim.x)
    {
        const int cl = it % CPB, nd = it / CPB;
        const int64_t e = cell0 + cl;
        if (e >= n)
            continue;
        const int64_t g = A.gdofD[NG_IDX(A.connD[static_cast<int64_t>(nd) * n + e], A.nNodesD, 60)];
#pragma unroll
        for (int c = 0; c < 3; ++c)
            sU[cl][nd][c] = u[NG_IDX(g + c, A.nDofs, 61)];
    }
    __syncthreads();
    const int t = threadIdx.x;
    if (t >= CPB * kNip)
        return;
    const int cl = t / kNip, q = t % kNip;
    const int64_t e = cell0 + cl;
    if (e >= n)
        return;
    // Jacobian J[i][j] = dx_i / dxi_j from the relative coordinates (k_geometry's formulas in FP32)
    float J[3][3];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j)
        {
            float s = 0.f;
#pragma unroll
            for (int nd = 1; nd < kNg; ++nd) // node 0 sits at the origin of the relative coordinates
                s += sX[cl][nd][i] * sDNg[(q * kNg + nd) * 3 + j];
            J[i][j] = s;
        }
    const float c00 = J[1][1] * J[2][2] - J[1][2] * J[2][1];
    const float c10 = J[1][2] * J[2][0] - J[1][0] * J[2][2];
    const float c20 = J[1][0] * J[2][1] - J[1][1] * J[2][0];
    const float det = J[0][0] * c00 + J[0][1] * c10 + J[0][2] * c20;
    const float id = 1.f / det;
    float inv[3][3];
    inv[0][0] = c00 * id;
    inv[1][0] = c10 * id;
    inv[2][0] = c20 * id;
    inv[0][1] = (J[0][2] * J[2][1] - J[0][1] * J[2][2]) * id;
    inv[1][1] = (J[0][0] * J[2][2] - J[0][2] * J[2][0]) * id;
    inv[2][1] = (J[0][1] * J[2][0] - J[0][0] * J[2][1]) * id;
    inv[0][2] = (J[0][1] * J[1][2] - J[0][2] * J[1][1]) * id;
    inv[1][2] = (J[0][2] * J[1][0] - J[0][0] * J[1][2]) * id;
    inv[2][2] = (J[0][0] * J[1][1] - J[0][1] * J[1][0]) * id;
    const float wdj = sW[q] * det;
    const float wdjE = A.escale ? wdj * static_cast<float>(A.escale[e]) : wdj;
    float lamw, muw, sv[6], tv[6];
#pragma unroll
    for (int v = 0; v < 6; ++v)
        sv[v] = tv[v] = 0.f;
    if (!LD)
    {
        lamw = static_cast<float>(L.C12) * wdjE;
        muw = static_cast<float>(L.C33) * wdjE;
    }
    else
    {
        // displacement gradient H = (sum_a u_a (x) dN_a/dxi) J^-1, and the same sums of magnitudes for the bound
        float Hx[3][3], Ha[3][3];
#pragma unroll
        for (int c = 0; c < 3; ++c)
#pragma unroll
            for (int j = 0; j < 3; ++j)
                Hx[c][j] = Ha[c][j] = 0.f;
        for (int nd = 0; nd < kNd; ++nd)
        {
            const float* dn = sDNd + (q * kNd + nd) * 3;
#pragma unroll
            for (int c = 0; c < 3; ++c)
            {
                const float uc = static_cast<float>(sU[cl][nd][c]);
#pragma unroll
                for (int j = 0; j < 3; ++j)
                {
                    Hx[c][j] += uc * dn[j];
                    Ha[c][j] += fabsf(uc) * fabsf(dn[j]);
                }
            }
        }
        float H[3][3], S = 0.f;
#pragma unroll
        for (int c = 0; c < 3; ++c)
#pragma unroll
            for (int k = 0; k < 3; ++k)
            {
                float h = 0.f, ha = 0.f;
#pragma unroll
                for (int j = 0; j < 3; ++j)
                {
                    h += Hx[c][j] * inv[j][k];
                    ha += Ha[c][j] * fabsf(inv[j][k]);
                }
                H[c][k] = h;
                S += ha;
            }
        float eps[6];
        StrainFromH<float, 3>(H, eps);
        const double kh = A.kappa[NG_IDX(e * kNip + q, n * kNip, 62)];
        const float khf = static_cast<float>(kh), k0f = static_cast<float>(L.kappa0);
        const float eqs = MisesValue<float, 3>(L, eps);
        // the FP32 strain differs from k_residual's FP64 strain by well below 1e-5 S (S bounds the magnitudes that
        // enter H); eq. strain's slope in the strain is below 10, so a margin of 1e-4 S separates both decisions
        const float bound = 1.0e-4f * S + 1.0e-30f;
        const float kapf = eqs > khf ? eqs : khf;
        const bool near = lawFp64 || fabsf(eqs - khf) <= bound + 1.0e-6f * khf ||
                          fabsf(kapf - k0f) <= bound + 1.0e-6f * k0f;
        if (!near)
        {
            const float omega = DamageOmega<float>(L, kapf);
            float lam, mu;
            LedTangentLameParams<float, 3>(L, eps, omega, lam, mu);
            lamw = lam * wdjE;
            muw = mu * wdjE;
            float dsdw[6];
            LedDstressDomega<float, 3>(L, eps, dsdw);
            const float dOdK = DamageDerivative<float>(L, kapf);
            if (eqs >= khf)
                MisesDerivative<float, 3>(L, eps, tv);
#pragma unroll
            for (int v = 0; v < 6; ++v)
                sv[v] = dsdw[v] * dOdK * wdjE;
        }
        else
        {
            // the FP64 strain of k_residual (geometry cache, same order of the sums) and the law in FP64
            const double* G = A.geo64 + NG_IDX(static_cast<int64_t>(q) * A.geoStride * n + e, A.geoSize, 63);
            double H64[3][3];
#pragma unroll
            for (int i = 0; i < 3; ++i)
#pragma unroll
                for (int j = 0; j < 3; ++j)
                    H64[i][j] = 0.;
            for (int nd = 0; nd < kNd; ++nd)
            {
                double g[3];
#pragma unroll
                for (int d = 0; d < 3; ++d)
                    g[d] = G[(1 + nd * 3 + d) * n];
#pragma unroll
                for (int c = 0; c < 3; ++c)
#pragma unroll
                    for (int d = 0; d < 3; ++d)
                        H64[c][d] += sU[cl][nd][c] * g[d];
            }
            double e64[6];
            StrainFromH<double, 3>(H64, e64);
            const double eq64 = MisesValue<double, 3>(L, e64);
            const double kap = eq64 > kh ? eq64 : kh;
            const double omega = DamageOmega<double>(L, kap);
            double lam, mu, dsdw[6], dk[6];
            LedTangentLameParams<double, 3>(L, e64, omega, lam, mu);
            lamw = static_cast<float>(lam) * wdjE;
            muw = static_cast<float>(mu) * wdjE;
            LedDstressDomega<double, 3>(L, e64, dsdw);
            const double dOdK = DamageDerivative<double>(L, kap);
            // loading (EvolutionImplicit: eq >= kappa_h). At a converged state kappa_h is eq itself, written by
            // k_history; this kernel's FP64 eq equals it mathematically but may differ in the last bits (the compiler
            // contracts the sums of squares of the Mises norm into FMAs differently per kernel), so a point within 4
            // ulps below kappa_h is loading, as it is in the kernels whose arithmetic matches k_history's bit for bit
            if (eq64 >= kh - 4.0 * DBL_EPSILON * kh)
                MisesDerivative<double, 3>(L, e64, dk);
            else
#pragma unroll
                for (int v = 0; v < 6; ++v)
                    dk[v] = 0.;
#pragma unroll
            for (int v = 0; v < 6; ++v)
            {
                sv[v] = static_cast<float>(dsdw[v] * dOdK) * wdjE;
                tv[v] = static_cast<float>(dk[v]);
            }
        }
    }
    float4* R = recs + (e * kNip + q) * kRecF4;
    R[0] = make_float4(inv[0][0], inv[0][1], inv[0][2], inv[1][0]);
    R[1] = make_float4(inv[1][1], inv[1][2], inv[2][0], inv[2][1]);
    R[2] = make_float4(inv[2][2], lamw, muw, 0.f);
    R[3] = make_float4(sv[0], sv[1], sv[2], sv[3]);
    R[4] = make_float4(sv[4], sv[5], tv[0], tv[1]);
    R[5] = make_float4(tv[2], tv[3], tv[4], tv[5]);
}

// ---- element matrices on the tensor cores ----------------------------------------------------------------------

__device__ __forceinline__ void AsyncCopy16(void* dst, const void* src)
{
    const unsigned sa = static_cast<unsigned>(__cvta_generic_to_shared(dst));
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(sa), "l"(src) : "memory");
}

// one operand value x at byte offset off: hi = round(x) into the hi buffer, lo = round(x - hi) into the lo buffer
// (split 3 only)
template <int SPLIT>
__device__ __forceinline__ void PutOp(unsigned char* hi, unsigned char* lo, int off, float x)
{
    const float h = Tf32Round(x);
    *reinterpret_cast<float*>(hi + off) = h;
    if (SPLIT == 3)
        *reinterpret_cast<float*>(lo + off) = Tf32Round(x - h);
}

template <bool RANK1, int SPLIT>
__global__ void __launch_bounds__(kTcThreads, 1) k_tangent_tc20(int64_t nCells, const double* __restrict__ tabDNd,
                                                               const float4* __restrict__ recs,
                                                               float* __restrict__ em, int* __restrict__ status,
                                                               long long spin)
{
    extern __shared__ __align__(1024) unsigned char sm[];
    __shared__ int sFail;
    const int tid = threadIdx.x, wid = tid >> 5, lane = tid & 31;
    float4* sRec = reinterpret_cast<float4*>(sm + kRecOff);
    float* sMu = reinterpret_cast<float*>(sm + kMuOff);
    float* sOut = reinterpret_cast<float*>(sm + kOutOff);
    float* sDN = reinterpret_cast<float*>(sm + kTabOff);
    const uint32_t smBase = static_cast<uint32_t>(__cvta_generic_to_shared(sm));
    const uint32_t bar0 = smBase + kBarOff;
    const int64_t n = nCells;
    if (static_cast<int64_t>(blockIdx.x) >= n)
        return; // the grid has at most one block per cell; a block without a cell allocates nothing

    // zero the operands once (padding rows and K columns stay zero), tables, barriers, tensor memory
    for (int i = tid; i < kOpEnd / 16; i += kTcThreads)
        reinterpret_cast<float4*>(sm)[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    for (int i = tid; i < kNip * kNd * 3; i += kTcThreads)
        sDN[i] = static_cast<float>(tabDNd[i]);
    if (tid == 0)
    {
        BarInit(bar0, 1);
        BarInit(bar0 + 8, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        sFail = 0;
    }
    if (wid == 0)
    {
        TmemAlloc(smBase + kBarOff + 16, kTmemCols);
        TmemRelinquish();
    }
    TcFenceBefore();
    __syncthreads();
    TcFenceAfter();
    const uint32_t tmem = *reinterpret_cast<volatile uint32_t*>(sm + kBarOff + 16);

    const int64_t stride = gridDim.x;
    auto issueRecs = [&](int64_t cell, int buf) {
        const float4* src = recs + cell * (kNip * kRecF4);
        float4* dst = sRec + buf * (kNip * kRecF4);
        for (int i = tid; i < kNip * kRecF4; i += kTcThreads)
            AsyncCopy16(dst + i, src + i);
    };
    // epilogue of the cell whose MMAs committed to accumulator acc (their completion has been observed)
    auto epilogue = [&](int64_t cell, int acc) {
        TcFenceAfter();
        const int quarter = wid & 3, chunk = wid >> 2; // lanes 32 quarter.., columns 16 chunk..
        const int row = quarter * 32 + lane;
        float v[16];
        TmemLoad16(tmem + (static_cast<uint32_t>(quarter * 32) << 16) + static_cast<uint32_t>(acc * 64 + chunk * 16),
                   v);
        TcFenceBefore();
        if (row >= 64 && row < 124)
#pragma unroll
            for (int t = 0; t < 16; ++t)
            {
                const int col = chunk * 16 + t;
                if (col < 60)
                    sMu[(row - 64) * kMuStride + col] = v[t];
            }
        __syncthreads();
        if (row < 60)
        {
            const int i = row / 20, a = row % 20;
#pragma unroll
            for (int t = 0; t < 16; ++t)
            {
                const int col = chunk * 16 + t;
                if (col >= 60)
                    continue;
                const int j = col / 20, b = col % 20;
                float x = v[t] + sMu[(j * 20 + a) * kMuStride + i * 20 + b];
                if (i == j)
                    x += sMu[a * kMuStride + b] + sMu[(20 + a) * kMuStride + 20 + b] +
                         sMu[(40 + a) * kMuStride + 40 + b];
                sOut[a * kOutStride + i * 60 + b * 3 + j] = x;
            }
        }
        __syncthreads();
        float* dst = em + cell * (kNd * 180);
        for (int t = tid; t < kNd * 180; t += kTcThreads)
            dst[t] = sOut[(t / 180) * kOutStride + t % 180];
    };

    int64_t e = blockIdx.x;
    int k = 0;
    issueRecs(e, 0);
    asm volatile("cp.async.commit_group;\n" ::: "memory");
    for (; e < n; e += stride, ++k)
    {
        const int b = k & 1;
        if (e + stride < n)
            issueRecs(e + stride, b ^ 1);
        asm volatile("cp.async.commit_group;\n" ::: "memory");
        asm volatile("cp.async.wait_group 1;\n" ::: "memory");
        // the operand buffer is free once the MMAs of the previous cell have completed
        if (k > 0 && !BarWait(bar0 + 8 * (b ^ 1), ((k - 1) >> 1) & 1, spin))
            sFail = 1;
        __syncthreads();
        if (sFail)
            break;
        // operands: item (node a, point q); a warp covers 8 nodes x 4 points, which puts its 32 stores of one
        // value on 32 distinct banks
        const float4* R = sRec + b * (kNip * kRecF4);
        unsigned char* aHi = sm + kOpAHi;
        unsigned char* aLo = sm + kOpALo;
        unsigned char* bHi = sm + kOpBHi;
        unsigned char* bLo = sm + kOpBLo;
        for (int it = tid; it < 21 * 32; it += kTcThreads)
        {
            const int grp = it >> 5, l = it & 31;
            const int a = (grp / 7) * 8 + (l >> 2), q = (grp % 7) * 4 + (l & 3);
            if (a >= kNd || q >= kNip)
                continue;
            const float4* Rq = R + q * kRecF4;
            const float4 r0 = Rq[0], r1 = Rq[1], r2 = Rq[2];
            const float inv[3][3] = {{r0.x, r0.y, r0.z}, {r0.w, r1.x, r1.y}, {r1.z, r1.w, r2.x}};
            const float lamw = r2.y, muw = r2.z;
            const float* dn = sDN + (q * kNd + a) * 3;
            float g[3];
#pragma unroll
            for (int kk = 0; kk < 3; ++kk)
                g[kk] = dn[0] * inv[0][kk] + dn[1] * inv[1][kk] + dn[2] * inv[2][kk];
            float P[3] = {0.f, 0.f, 0.f}, Q[3] = {0.f, 0.f, 0.f};
            if (RANK1)
            {
                const float4 r3 = Rq[3], r4 = Rq[4], r5 = Rq[5];
                const float s[6] = {r3.x, r3.y, r3.z, r3.w, r4.x, r4.y};
                const float tt[6] = {r4.z, r4.w, r5.x, r5.y, r5.z, r5.w};
                BtS<float, 3>(g, s, P);
                BtS<float, 3>(g, tt, Q);
            }
#pragma unroll
            for (int i = 0; i < 3; ++i)
            {
                const int r = i * 20 + a;
                PutOp<SPLIT>(aHi, aLo, OpOff(r, q), lamw * g[i]);
                PutOp<SPLIT>(aHi, aLo, OpOff(64 + r, q), muw * g[i]);
                PutOp<SPLIT>(bHi, bLo, OpOff(r, q), g[i]);
                if (RANK1)
                {
                    PutOp<SPLIT>(aHi, aLo, OpOff(r, 32 + q), P[i]);
                    PutOp<SPLIT>(bHi, bLo, OpOff(r, 32 + q), Q[i]);
                }
            }
        }
        FenceProxyAsync();
        __syncthreads();
        if (tid == 0)
        {
            TcFenceAfter();
            const uint32_t d = tmem + static_cast<uint32_t>(b * 64);
            constexpr int KS = RANK1 ? 8 : 4; // K = 8 per instruction
#pragma unroll
            for (int s = 0; s < KS; ++s)
            {
                const uint32_t off = static_cast<uint32_t>(s * 256);
                if (SPLIT == 3)
                {
                    MmaTf32(d, SmemDesc(smBase + kOpALo + off), SmemDesc(smBase + kOpBHi + off), s > 0 ? 1u : 0u);
                    MmaTf32(d, SmemDesc(smBase + kOpAHi + off), SmemDesc(smBase + kOpBLo + off), 1u);
                    MmaTf32(d, SmemDesc(smBase + kOpAHi + off), SmemDesc(smBase + kOpBHi + off), 1u);
                }
                else
                    MmaTf32(d, SmemDesc(smBase + kOpAHi + off), SmemDesc(smBase + kOpBHi + off), s > 0 ? 1u : 0u);
            }
            MmaCommit(bar0 + 8 * b);
        }
        if (k > 0)
            epilogue(e - stride, b ^ 1);
        __syncthreads();
    }
    if (!sFail && k > 0)
    {
        // the last cell
        const int b = (k - 1) & 1;
        if (!BarWait(bar0 + 8 * b, ((k - 1) >> 1) & 1, spin))
            sFail = 1;
        __syncthreads();
        if (!sFail)
            epilogue(e - stride, b);
    }
    asm volatile("cp.async.wait_group 0;\n" ::: "memory");
    __syncthreads();
    if (sFail)
    {
        // the MMAs of cells 0 .. issued - 1 were committed, alternately to barrier 0 and 1; wait (bounded by a fixed
        // limit, independent of the caller's spin limit) for the last phase of each barrier before the tensor memory
        // is released
        if (tid == 0)
        {
            atomicExch(status, NUTO_GPU_ETIMEOUT);
            const int issued = k;
            for (int bb = 0; bb < 2; ++bb)
            {
                const int commits = (issued + 1 - bb) / 2;
                if (commits > 0)
                    BarWait(bar0 + 8 * bb, static_cast<uint32_t>(commits - 1) & 1u, kDrainLimit);
            }
        }
        __syncthreads();
    }
    TcFenceBefore();
    __syncthreads();
    if (wid == 0)
    {
        TcFenceAfter();
        TmemDealloc(tmem, kTmemCols);
    }
}

// ---- CSR rows from the element matrices ------------------------------------------------------------------------

__global__ void __launch_bounds__(128) k_tc20_rows(Tc20RowArgs r, const float* __restrict__ em,
                                                   float* __restrict__ vals)
{
    __shared__ float sRow[4][3][kRowCapTc];
    const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t a = static_cast<int64_t>(blockIdx.x) * 4 + wid;
    if (a >= r.nNodes)
        return; // the whole warp leaves; only warp-level synchronisation follows
    float(*row)[kRowCapTc] = sRow[wid];
    int64_t rs[3];
    int len[3];
    const int64_t g = r.gdofD[a];
#pragma unroll
    for (int k = 0; k < 3; ++k)
    {
        rs[k] = r.rowPtr[NG_IDX(g + k, r.nRows, 64)];
        len[k] = static_cast<int>(r.rowPtr[g + k + 1] - rs[k]);
        for (int i = lane; i < len[k]; i += 32)
            row[k][i] = 0.f;
    }
    const int32_t bUU = r.blk[a];
    __syncwarp();
    const int64_t k0 = r.cellPtr[a], k1 = r.cellPtr[a + 1];
    for (int64_t kc = k0; kc < k1; ++kc)
    {
        const int64_t e = r.cellIdx[kc];
        const int ia = r.cellLoc[kc];
        const int rk = lane < kNd ? r.rank[(static_cast<int64_t>(ia) * kNd + lane) * r.nCells + e] : 0;
        const float* src = em + NG_IDX((e * kNd + ia) * 180, r.nCells * kNd * 180, 65);
#pragma unroll
        for (int m = 0; m < 6; ++m)
        {
            const int t = lane + 32 * m; // item (row i, neighbour b, column j) of a's 180 values in this cell
            const int tc = t < 180 ? t : 179;
            const int i = tc / 60, b = (tc % 60) / 3, j = tc % 3;
            const int rb = __shfl_sync(0xffffffffu, rk, b);
            if (t < 180)
                row[i][NG_IDX(bUU + 3 * rb + j, kRowCapTc, 66)] += src[t];
        }
        __syncwarp();
    }
#pragma unroll
    for (int k = 0; k < 3; ++k)
        for (int i = lane; i < len[k]; i += 32)
            vals[NG_IDX(rs[k] + i, r.nnz, 67)] = row[k][i];
}

} // namespace

// Hex20 displacement cells on a Hex8 coordinate mesh with 3x3x3 Gauss points, LinearElastic or LocalIsotropicDamage
// with FULL damage application (UNILATERAL switches on the sign of the volumetric strain, a branch FP32 cannot
// decide like FP64 near zero), every CSR row within the row buffer.
bool Tc20TangentSupported(Ctx& c)
{
    if (c.tc20Mode >= 0)
        return c.tc20Mode == 1;
    c.tc20Mode = 0;
    if (c.forceTc20Off || c.slots.size() != 1)
        return false;
    const Slot& D = c.slots[c.prm.disp_slot];
    const bool cells = c.dim == 3 && c.nge == 8 && D.nen == kNd && D.ncomp == 3 && c.ip.nIp == kNip;
    const bool law = c.prm.kind == NUTO_GPU_MB_LINEAR_ELASTIC ||
                     (c.prm.kind == NUTO_GPU_MB_LOCAL_DAMAGE && c.prm.damage_application == NUTO_GPU_DAMAGE_FULL);
    if (!cells || !law)
        return false;
    for (int64_t i = 0; i < D.nNodes; ++i)
        for (int k = 0; k < 3; ++k)
        {
            const int64_t rr = D.offset + D.dof0[i] + k;
            if (c.hRowPtr[rr + 1] - c.hRowPtr[rr] > kRowCapTc)
                return false;
        }
    c.tc20Mode = 1;
    return true;
}

void LaunchTangentTc20(Ctx& c, const double* u, float* vals)
{
    if (c.dRelX.n == 0)
        BuildRelativeCoordinates(c);
    if (!c.haveGeo)
        BuildGeometryCache(c);
    if (c.dStatus.n == 0)
    {
        c.dStatus.alloc(1);
        NG_CUDA(cudaMemset(c.dStatus.p, 0, sizeof(int)));
    }
    const Slot& D = c.slots[c.prm.disp_slot];
    const bool ld = c.prm.kind == NUTO_GPU_MB_LOCAL_DAMAGE;
    const int64_t n = c.nCells;
    const size_t recBytes = static_cast<size_t>(n) * kNip * kRecF4 * 16;
    if (c.dRecords.n < recBytes)
        c.dRecords.alloc(recBytes);
    if (c.dElemMats.n < static_cast<size_t>(n) * kNd * 180)
        c.dElemMats.alloc(static_cast<size_t>(n) * kNd * 180);
    float4* recs = reinterpret_cast<float4*>(c.dRecords.p);

    Tc20Args A{};
    A.nCells = n;
    A.nDofs = c.nDofs;
    A.nNodesD = D.nNodes;
    A.geoSize = static_cast<int64_t>(c.dGeo64.n);
    A.connD = D.dConnT.p;
    A.gdofD = D.dGdof.p;
    A.relX = c.dRelX.p;
    A.kappa = c.dKappa.p;
    A.escale = c.dEScale.n ? c.dEScale.p : nullptr;
    A.geo64 = c.dGeo64.p;
    A.geoStride = c.geoStride;
    A.tabDNg = c.dTables.p + c.tabDN[c.geoInterp];
    A.tabDNd = c.dTables.p + c.tabDN[D.interp];
    A.tabW = c.dTables.p + c.tabW;
    const unsigned pb = static_cast<unsigned>((n + 3) / 4);
    if (ld)
        k_tc20_points<NUTO_GPU_MB_LOCAL_DAMAGE><<<pb, 128, 0, c.stream>>>(A, c.law, u, recs, c.tc20LawFp64);
    else
        k_tc20_points<NUTO_GPU_MB_LINEAR_ELASTIC><<<pb, 128, 0, c.stream>>>(A, c.law, u, recs, 0);
    AfterLaunch(c, "k_tc20_points");

    const unsigned grid = static_cast<unsigned>(std::min<int64_t>(n, c.smCount > 0 ? c.smCount : 1));
    auto tc = [&](auto kern) {
        NG_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemTc));
        kern<<<grid, kTcThreads, kSmemTc, c.stream>>>(n, A.tabDNd, recs, c.dElemMats.p, c.dStatus.p, c.spinLimit);
    };
    if (ld)
    {
        if (c.tc20Split == 1)
            tc(k_tangent_tc20<true, 1>);
        else
            tc(k_tangent_tc20<true, 3>);
    }
    else
    {
        if (c.tc20Split == 1)
            tc(k_tangent_tc20<false, 1>);
        else
            tc(k_tangent_tc20<false, 3>);
    }
    AfterLaunch(c, "k_tangent_tc20");

    Tc20RowArgs r{};
    r.nNodes = D.nNodes;
    r.nCells = n;
    r.nnz = c.nnz;
    r.nRows = c.nDofs;
    r.gdofD = D.dGdof.p;
    r.cellPtr = D.dCellPtr.p;
    r.cellIdx = D.dCellIdx.p;
    r.cellLoc = D.dCellLoc.p;
    r.rowPtr = c.dRowPtr.p;
    const int p = c.prm.disp_slot * static_cast<int>(c.slots.size()) + c.prm.disp_slot;
    r.rank = c.pairs[p].rank;
    r.blk = c.pairs[p].dBlk.p;
    k_tc20_rows<<<static_cast<unsigned>((D.nNodes + 3) / 4), 128, 0, c.stream>>>(r, c.dElemMats.p, vals);
    AfterLaunch(c, "k_tc20_rows");
    c.stats.kernel_launches += 3;
}

int ReadDeviceStatus(Ctx& c)
{
    if (c.dStatus.n == 0)
        return 0;
    int s = 0;
    NG_CUDA(cudaMemcpy(&s, c.dStatus.p, sizeof(int), cudaMemcpyDeviceToHost));
    if (s != 0)
        NG_CUDA(cudaMemset(c.dStatus.p, 0, sizeof(int)));
    return s;
}

} // namespace nuto_gpu
