// Shared device pieces of the solver kernels: block reductions, the last-block ticket and the node-block SpMV.
#pragma once

#include "solver.cuh"

namespace nuto_gpu
{

constexpr int kBS = 256;

__device__ __forceinline__ double WarpSum(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
        v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

// Sums v over the block and adds the block total to *acc (thread 0).
__device__ __forceinline__ void BlockAccumulate(double v, double* acc, double* sh)
{
    v = WarpSum(v);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0)
        sh[wid] = v;
    __syncthreads();
    if (wid == 0)
    {
        v = lane < (blockDim.x >> 5) ? sh[lane] : 0.;
        v = WarpSum(v);
        if (lane == 0)
            atomicAdd(acc, v);
    }
    __syncthreads();
}

// True in exactly one block: the last one to arrive (threadFenceReduction pattern, no spinning).
__device__ __forceinline__ bool LastBlock(int* counter)
{
    __shared__ bool last;
    __threadfence();
    if (threadIdx.x == 0)
    {
        const unsigned prev = atomicAdd(reinterpret_cast<unsigned*>(counter), 1u);
        last = prev == gridDim.x - 1;
    }
    __syncthreads();
    return last;
}

__device__ __forceinline__ double VRead(const double* p)
{
    return *reinterpret_cast<const volatile double*>(p);
}

__device__ __forceinline__ bool Finite(double v)
{
    return isfinite(v);
}

// finalize actions of the SpMV kernel
enum Fin
{
    FIN_NONE = 0,
    FIN_PCG_ALPHA = 1,  // alpha = rho / (p.Ap)
    FIN_BICG_ALPHA = 2, // alpha = rho / (rhat.v)
    FIN_BICG_OMEGA = 3  // omega = (t.s) / (t.t)
};

// Node-block SpMV: one warp per DOF node (of every slot) computes all rows of that node. DofNumbering numbers the
// components of a node consecutively, so every row of node a lists, per slot J, the J-neighbours of a in the
// same order with ncomp_J consecutive values each; the lanes run over the neighbours, load the neighbour's x
// values once for all rows of the node and read the values at rowPtr[row] + blk_IJ(a) + ncomp_J * k + d. The
// column indices are never read: the CSR values plus the per-node neighbour lists are the whole traffic.
// The row segment of node a starts at rowPtr[row] + blk[I * ns][a]: zero for the whole operator; a diagonal-block
// view (ns = 1, the lists and block offsets of the pair (I, I)) covers only the I-columns of the I-rows.
struct NodeSpmv
{
    int ns;
    int ncomp[kMaxSlots];
    int64_t nNodes[kMaxSlots];
    int64_t firstWarp[kMaxSlots];
    int64_t totalWarps;
    const int64_t* gdof[kMaxSlots];
    const int64_t* nbrPtr[kMaxSlots * kMaxSlots];
    const int32_t* nbrIdx[kMaxSlots * kMaxSlots];
    const int32_t* nbrCol[kMaxSlots * kMaxSlots]; // combined row of component 0 of every neighbour entry
    const int32_t* blk[kMaxSlots * kMaxSlots];
    const int64_t* rowPtr;
    int64_t nnz, nRows, nbrTotal[kMaxSlots * kMaxSlots];
    // padded pair layout (nbBase[0] == nullptr: CSR only): per view pair the node blocks and the pair's offset, the
    // longest padded segment, and the layout buffers with the CSR values each was filled from
    const int64_t* nbBase[kMaxSlots * kMaxSlots];
    int64_t nbOff[kMaxSlots * kMaxSlots];
    int nbSeg4;
    int ncMaxRows; // most components of a row node of the view
    const float* nb32;
    const double* nb64;
    const void* nbSrc32;
    const void* nbSrc64;
};

// block sums of the SpMV's dot products and, in the last block, the Krylov scalar they finish
template <int NDOT>
__device__ __forceinline__ void SpmvFinish(double d0, double d1, double* sc, int* st, int fin, double* sh)
{
    BlockAccumulate(d0, sc + SC_ACC0, sh);
    if (NDOT >= 2)
        BlockAccumulate(d1, sc + SC_ACC1, sh);
    if (LastBlock(st + ST_COUNTER) && threadIdx.x == 0)
    {
        st[ST_COUNTER] = 0;
        const double a0 = VRead(sc + SC_ACC0), a1 = VRead(sc + SC_ACC1);
        sc[SC_ACC0] = 0.;
        sc[SC_ACC1] = 0.;
        if (fin == FIN_PCG_ALPHA)
        {
            if (!Finite(a0))
                st[ST_STATE] = NONFINITE;
            else if (!(a0 > 0.))
                st[ST_STATE] = BREAKDOWN;
            else
                sc[SC_ALPHA] = sc[SC_RHO] / a0;
        }
        else if (fin == FIN_BICG_ALPHA)
        {
            if (!Finite(a0))
                st[ST_STATE] = NONFINITE;
            else if (a0 == 0.)
                st[ST_STATE] = BREAKDOWN;
            else
                sc[SC_ALPHA] = sc[SC_RHO] / a0;
        }
        else if (fin == FIN_BICG_OMEGA)
        {
            if (!Finite(a0) || !Finite(a1))
                st[ST_STATE] = NONFINITE;
            else
                sc[SC_OMEGA] = a1 > 0. ? a0 / a1 : 0.;
        }
    }
}

constexpr int kMaxRowLen = 256; // longest row of a node (Hex20 displacements: 3 x 81)
constexpr int kMaxComp = 3;     // components per DOF node
constexpr int kPre = 4;         // row chunks of 32 values prefetched into registers (rows up to 128 entries)

template <typename TV, typename TX, int NDOT>
__global__ void __launch_bounds__(kBS, 5) k_spmv_node(NodeSpmv A, const TV* __restrict__ val,
                                                    const uint8_t* __restrict__ mask, const TX* __restrict__ x,
                                                    TX* __restrict__ y, const TX* __restrict__ w0, double* sc, int* st,
                                                    int fin)
{
    PdlWait();
    PdlTrigger();
    __shared__ double sh[kBS / 32];
    __shared__ TX xs[kBS / 32][kMaxRowLen];
    if (st && st[ST_STATE] != RUN)
        return;
    const int64_t warp = (blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int I = (A.ns > 1 && warp >= A.firstWarp[1]) ? 1 : 0;
    const int64_t a = warp - A.firstWarp[I];
    const bool valid = warp < A.totalWarps && a < A.nNodes[I];
    const int ncI = A.ncomp[I];
    double d0 = 0., d1 = 0.;
    if (valid)
    {
        // independent loads first: neighbour ranges of every slot pair, the node's rows and block offset
        int64_t q0[kMaxSlots];
        int nn[kMaxSlots];
#pragma unroll
        for (int J = 0; J < kMaxSlots; ++J)
        {
            q0[J] = 0;
            nn[J] = 0;
            if (J < A.ns)
            {
                const int p = I * A.ns + J;
                q0[J] = A.nbrPtr[p][a];
                nn[J] = static_cast<int>(A.nbrPtr[p][a + 1] - q0[J]);
            }
        }
        const int64_t g0 = A.gdof[I][a];
        const int32_t seg = A.blk[I * A.ns][a]; // 0 for a whole-row operator, the block start for a block view
        int64_t rs[kMaxComp];
        TX s[kMaxComp];
#pragma unroll
        for (int c = 0; c < kMaxComp; ++c)
        {
            rs[c] = c < ncI ? A.rowPtr[NG_IDX(g0 + c, A.nRows, 16)] + seg : 0;
            s[c] = TX(0);
        }
        const int nc0 = A.ncomp[0], nc1 = A.ns > 1 ? A.ncomp[1] : 0;
        const int len = nc0 * nn[0] + nc1 * nn[1];
        // the first kPre chunks of every row go to registers before the gather, so that the value stream and the
        // gather's dependent loads are in flight together
        TV v[kMaxComp][kPre];
#pragma unroll
        for (int c = 0; c < kMaxComp; ++c)
#pragma unroll
            for (int k = 0; k < kPre; ++k)
            {
                const int q = lane + 32 * k;
                v[c][k] = (c < ncI && q < len) ? val[NG_IDX(rs[c] + q, A.nnz, 19)] : TV(0);
            }
        // x of the node's neighbours in the column order of its rows (both slot pairs in one pass)
        const int tot = nn[0] + nn[1];
#pragma unroll 2
        for (int t = lane; t < tot; t += 32)
        {
            const int J = t >= nn[0] ? 1 : 0;
            const int kk = t - (J ? nn[0] : 0);
            const int ncJ = J ? nc1 : nc0;
            const int p = I * A.ns + J;
            const int64_t qJ = J ? q0[1] : q0[0];
            const int64_t gb = A.nbrCol[p][NG_IDX(qJ + kk, A.nbrTotal[p], 17)];
            const int base = J ? nc0 * nn[0] + nc1 * kk : nc0 * kk;
            for (int d = 0; d < ncJ; ++d)
                xs[wid][NG_IDX(base + d, kMaxRowLen, 20)] = x[NG_IDX(gb + d, A.nRows, 18)];
        }
        __syncwarp();
#pragma unroll
        for (int k = 0; k < kPre; ++k)
        {
            const int q = lane + 32 * k;
            if (q < len)
            {
                const TX xv = xs[wid][q];
#pragma unroll
                for (int c = 0; c < kMaxComp; ++c)
                    s[c] += static_cast<TX>(v[c][k]) * xv;
            }
        }
        for (int q = lane + 32 * kPre; q < len; q += 32) // rows longer than 32 kPre entries (Hex20)
        {
            const TX xv = xs[wid][q];
#pragma unroll
            for (int c = 0; c < kMaxComp; ++c)
                if (c < ncI)
                    s[c] += static_cast<TX>(val[NG_IDX(rs[c] + q, A.nnz, 19)]) * xv;
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1)
#pragma unroll
            for (int c = 0; c < kMaxComp; ++c)
                s[c] += __shfl_down_sync(0xffffffffu, s[c], o);
        if (lane == 0)
        {
#pragma unroll
            for (int c = 0; c < kMaxComp; ++c)
            {
                if (c >= ncI)
                    break;
                const int64_t r = g0 + c;
                const TX yv = mask[r] ? x[r] : s[c];
                y[r] = yv;
                if (NDOT >= 1)
                    d0 += static_cast<double>(w0[r]) * static_cast<double>(yv);
                if (NDOT >= 2)
                    d1 += static_cast<double>(yv) * static_cast<double>(yv);
            }
        }
    }
    if (NDOT == 0)
        return;
    SpmvFinish<NDOT>(d0, d1, sc, st, fin, sh);
}

// NodeSpmv of the context's fine-level pattern
NodeSpmv MakeNodeSpmv(const Ctx& c);

// ---- node SpMV on the padded pair layout -------------------------------------------------------------------------
// kNbG lanes per node (four nodes per warp). For every column slot J of the view the group gathers the x of the
// node's J-neighbours into its shared segment buffer (zero-padded to a multiple of 4), then streams the node's
// padded row segments of pair (I, J) in 16-byte vectors, one lane per 4 columns, accumulating the ncomp_I row sums;
// a 3-step butterfly inside the group finishes the rows. Per value: a quarter of a 16-byte load and one FMA.
constexpr int kNbG = 8;

template <typename T>
__device__ __forceinline__ void Load4(const T* p, T (&o)[4])
{
    if constexpr (sizeof(T) == 4)
    {
        const float4 f = *reinterpret_cast<const float4*>(p);
        o[0] = f.x;
        o[1] = f.y;
        o[2] = f.z;
        o[3] = f.w;
    }
    else
    {
        const double2 f0 = reinterpret_cast<const double2*>(p)[0];
        const double2 f1 = reinterpret_cast<const double2*>(p)[1];
        o[0] = f0.x;
        o[1] = f0.y;
        o[2] = f1.x;
        o[3] = f1.y;
    }
}

template <typename TV>
__device__ __forceinline__ const TV* NbValues(const NodeSpmv& A)
{
    if constexpr (sizeof(TV) == 4)
        return A.nb32;
    else
        return A.nb64;
}

// FP32 values: at most 40 registers (6 blocks of 256 threads per SM: more nodes in flight, measured 10 % faster per
// GMRES iteration despite a few spilled bytes); FP64 values: at most 64 registers (4 blocks; without a cap the
// compiler takes 90 and the FP64 path slowed by 25 %)
template <typename TV>
constexpr int NbMinBlocks()
{
    return sizeof(TV) == 4 ? 6 : 4;
}

template <typename TV, typename TX, int NDOT, int G>
__global__ void __launch_bounds__(kBS, NbMinBlocks<TV>()) k_spmv_nb(NodeSpmv A, const uint8_t* __restrict__ mask,
                                                  const TX* __restrict__ x, TX* __restrict__ y,
                                                  const TX* __restrict__ w0, double* sc, int* st, int fin)
{
    PdlWait();
    PdlTrigger();
    extern __shared__ __align__(16) unsigned char nbSmem[];
    __shared__ double sh[kBS / 32];
    if (st && st[ST_STATE] != RUN)
        return;
    const TV* __restrict__ vals = NbValues<TV>(A);
    const int gl = threadIdx.x & (G - 1);
    const int L = A.nbSeg4;
    TX* xs = reinterpret_cast<TX*>(nbSmem) + (threadIdx.x / G) * L;
    const int64_t u = (blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x) / G;
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
    // neighbour ranges and value blocks of every column slot first (independent loads)
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
    // x of all neighbours of all column slots into the group's segment buffers (unrolled: several neighbour ->
    // x chains in flight per lane)
    const int nc0 = A.ncomp[0], nc1 = A.ns > 1 ? A.ncomp[1] : 0;
#pragma unroll 4
    for (int t = gl; t < tot; t += G)
    {
        const int J = t >= nn[0] ? 1 : 0;
        const int kk = t - (J ? nn[0] : 0);
        const int ncJ = J ? nc1 : nc0;
        const int p = I * A.ns + J;
        const int64_t col = A.nbrCol[p][NG_IDX((J ? q0[1] : q0[0]) + kk, A.nbrTotal[p], 60)];
        const int xb = (J ? xoff[1] : 0) + kk * ncJ;
        for (int d = 0; d < ncJ; ++d)
            xs[NG_IDX(xb + d, L, 61)] = x[NG_IDX(col + d, A.nRows, 62)];
    }
#pragma unroll
    for (int J = 0; J < kMaxSlots; ++J)
    {
        const int seg = (J ? nc1 : nc0) * nn[J];
        for (int t = seg + gl; t < seg4[J]; t += G)
            xs[NG_IDX(xoff[J] + t, L, 63)] = TX(0);
    }
    __syncwarp();
    TX s[kMaxComp];
#pragma unroll
    for (int c = 0; c < kMaxComp; ++c)
        s[c] = TX(0);
#pragma unroll
    for (int J = 0; J < kMaxSlots; ++J)
    {
        const TV* vp = vals + vbase[J];
        const TX* xj = xs + xoff[J];
        const int sg = seg4[J];
#pragma unroll 2
        for (int f = 4 * gl; f < sg; f += 4 * G)
        {
            TX xv[4];
            Load4(xj + f, xv);
#pragma unroll
            for (int c = 0; c < kMaxComp; ++c)
                if (c < ncI)
                {
                    TV v[4];
                    Load4(vp + c * sg + f, v);
                    s[c] += static_cast<TX>(v[0]) * xv[0] + static_cast<TX>(v[1]) * xv[1] +
                            static_cast<TX>(v[2]) * xv[2] + static_cast<TX>(v[3]) * xv[3];
                }
        }
    }
#pragma unroll
    for (int o = G / 2; o > 0; o >>= 1)
#pragma unroll
        for (int c = 0; c < kMaxComp; ++c)
            s[c] += __shfl_xor_sync(0xffffffffu, s[c], o);
    double d0 = 0., d1 = 0.;
    if (valid && gl == 0)
    {
        const int64_t g0 = A.gdof[I][a];
#pragma unroll
        for (int c = 0; c < kMaxComp; ++c)
        {
            if (c >= ncI)
                break;
            const int64_t r = NG_IDX(g0 + c, A.nRows, 64);
            const TX yv = mask[r] ? x[r] : s[c];
            y[r] = yv;
            if (NDOT >= 1)
                d0 += static_cast<double>(w0[r]) * static_cast<double>(yv);
            if (NDOT >= 2)
                d1 += static_cast<double>(yv) * static_cast<double>(yv);
        }
    }
    if (NDOT == 0)
        return;
    SpmvFinish<NDOT>(d0, d1, sc, st, fin, sh);
}

// CSR values -> padded pair layout: one warp per node of the view, lanes over the segment
template <typename TV>
__global__ void __launch_bounds__(kBS) k_nb_pack(NodeSpmv A, const TV* __restrict__ csr, TV* __restrict__ nb)
{
    const int64_t u = (blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (u >= A.totalWarps)
        return;
    const int I = (A.ns > 1 && u >= A.firstWarp[1]) ? 1 : 0;
    const int64_t a = u - A.firstWarp[I];
    if (a >= A.nNodes[I])
        return;
    const int ncI = A.ncomp[I];
    const int64_t g0 = A.gdof[I][a];
    for (int J = 0; J < A.ns; ++J)
    {
        const int p = I * A.ns + J;
        const int nn = static_cast<int>(A.nbrPtr[p][a + 1] - A.nbrPtr[p][a]);
        const int seg = A.ncomp[J] * nn, seg4 = (seg + 3) & ~3;
        const int32_t blk = A.blk[p][a];
        TV* dst = nb + A.nbOff[p] + A.nbBase[p][a];
        for (int c = 0; c < ncI; ++c)
        {
            const TV* src = csr + A.rowPtr[NG_IDX(g0 + c, A.nRows, 65)] + blk;
            for (int q = lane; q < seg4; q += 32)
                dst[c * seg4 + q] = q < seg ? src[NG_IDX(q, A.nnz, 66)] : TV(0);
        }
    }
}

// Launches the padded-layout kernel when the view has the layout and it holds `vals` (the CSR values the caller
// passes), the CSR kernel otherwise.
// true when the view has the padded layout and it holds `vals` (the lanes-per-node choice applies)
template <typename TV>
inline bool SpmvPadded(const NodeSpmv& A, const TV* vals)
{
    const void* src = sizeof(TV) == 4 ? A.nbSrc32 : A.nbSrc64;
    return A.nbBase[0] && src == static_cast<const void*>(vals) && A.nbSeg4 > 0;
}

// group: lanes per node of the padded-layout kernel (4, 8 or 16; 0 = the default: 8, or 4 for views of
// single-component rows and columns)
template <typename TV, typename TX, int NDOT>
void SpmvNode(cudaStream_t stream, const NodeSpmv& A, const TV* vals, const TX* x, TX* y, const TX* w0, double* sc,
              int* st, int fin, const uint8_t* mask, int group = 0)
{
    if (SpmvPadded(A, vals))
    {
        // 8 lanes per node; 4 for views of single-component rows and columns (one short segment per node)
        const bool narrow = A.ns == 1 && A.ncMaxRows == 1;
        const int G = group ? group : (narrow ? 4 : kNbG);
        const size_t perGroup = static_cast<size_t>(A.nbSeg4) * sizeof(TX);
        int threads = kBS;
        while (threads > 32 && (threads / G) * perGroup > 48 * 1024)
            threads -= 32;
        const int64_t total = A.totalWarps * G;
        const unsigned blocks = static_cast<unsigned>((total + threads - 1) / threads);
        const size_t smem = (threads / G) * perGroup;
        if (G == 4)
            NG_CUDA(LaunchPdl(k_spmv_nb<TV, TX, NDOT, 4>, blocks, threads, smem, stream, A, mask, x, y, w0, sc, st,
                              fin));
        else if (G == 16)
            NG_CUDA(LaunchPdl(k_spmv_nb<TV, TX, NDOT, 16>, blocks, threads, smem, stream, A, mask, x, y, w0, sc, st,
                              fin));
        else
            NG_CUDA(LaunchPdl(k_spmv_nb<TV, TX, NDOT, kNbG>, blocks, threads, smem, stream, A, mask, x, y, w0, sc, st,
                              fin));
        return;
    }
    const int64_t threads = A.totalWarps * 32;
    const unsigned blocks = static_cast<unsigned>((threads + kBS - 1) / kBS);
    NG_CUDA(LaunchPdl(k_spmv_node<TV, TX, NDOT>, blocks, kBS, 0, stream, A, vals, mask, x, y, w0, sc, st, fin));
}

} // namespace nuto_gpu
