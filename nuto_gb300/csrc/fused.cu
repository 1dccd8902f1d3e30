// FP32 tangent of linear cells: SimpleAssembler::BuildMatrix (nuto/mechanics/cell/SimpleAssembler.cpp:100-156) of
// MomentumBalance::Hessian0 (nuto/mechanics/integrands/MomentumBalance.h:36-46) and GradientDamage::Hessian0
// (nuto/mechanics/integrands/GradientDamage.h:92-120) for Quad4 and Hex8 cells, written straight into the CSR values
// without atomics in global memory.
//
// Two forms, chosen by the autotuner on a context's first FP32 tangent (the values are bitwise the same):
//
// Element matrices (k_cell_matrices_law + k_rows_from_cells32 / k_rows_from_cells; the faster form on the 64^3
// beam): a warp evaluates the law of 4 cells' points into shared memory and integrates every node-pair block of each
// cell once (two blocks per lane in packed FP32 pairs), writing the cell's element matrix; then one warp per
// displacement node adds the matrix slabs of its cells in ascending cell order into its rows and stores them once.
//
// Node rows: one warp per displacement node a assembles the complete CSR rows of a (and of its eeq node). The cells
// around a are taken a pass of CPP = 32 / NIP at a time; per pass the warp needs, for every point of the pass's
// cells, the node gradients dN/dX and the law's scalars and vectors (PointData):
//   staged: k_point_records evaluates PointData once per (cell, point) into per-cell contiguous records
//       (13 float4 per point for Hex8 gradient damage); the node warp copies a pass's records into shared memory
//       with 16-byte asynchronous copies;
//   fused (NUTO_GPU_TANGENT=fused): (0) lane (cell, node) loads the node's coordinates relative to the cell's first
//       node, displacements and eeq; (A) lane (cell, point) evaluates PointData in the warp (each cell's points are
//       then evaluated by every warp whose node the cell holds, up to 8 times).
// Then (B) lane (cell, neighbour b) integrates the node-pair block (a, b) over the points in registers and adds it
// into the warp's shared copy of a's rows at the rank of b, one cell slot after the other (fixed order: the values
// are bitwise reproducible). At the end the rows are stored once, coalesced. Both forms integrate a block with the
// same explicitly rounded operations (PairPoint, PairPoint2).
//
// Branch decisions of the law are the FP64 kernels' (k_residual, k_tangent<double>): the nonlocal equivalent
// strain at a point is formed in FP32 with an error bound, and where the bound does not separate it from the
// history kappa or from kappa0 it is recomputed in FP64 exactly as the FP64 kernels form it. The loading/unloading
// and damage-threshold branches therefore agree with the FP64 residual at every point; everything else is FP32.
#include "internal.cuh"

#include <algorithm>
#include <type_traits>

namespace nuto_gpu
{

namespace
{

constexpr int kFusedRowCap = 128; // values per row buffer: 32 neighbour nodes of [u | eeq] in 3D

struct FusedArgs
{
    int64_t nNodes, nCells, nnz, nRows, nDofs, nNodesD, nNodesE;
    int64_t nodeBase; // the element-matrix row gathers take nodes nodeBase .. nNodes - 1
    const int32_t* connD; // planar [n][cell]
    const int32_t* connE;
    const int64_t* gdofD; // per node: combined index of component 0
    const int64_t* gdofE;
    const int32_t* eOf;   // displacement node -> its eeq node
    const float* relX;    // planar [(n * DIM + d)][cell]: X_n - X_0
    const double* kappa;  // [cell][ip]
    const double* escale; // per-cell Young's modulus factor (nullptr: 1)
    const double* tabN;   // nIp x nd
    const double* tabDN;  // nIp x nd x 3
    const double* tabW;   // nIp
    const int64_t* cellPtr;
    const int32_t* cellIdx;
    const uint8_t* cellLoc;
    const int64_t* rowPtr;
    const uint8_t* rank[4]; // UU, UE, EU, EE
    const int32_t* blk[4];
};

template <int DIM, int ND, int NIP, int KIND>
struct FCfg
{
    static constexpr int dim = DIM, nd = ND, nip = NIP, kind = KIND;
};

// STAGED: the per-point data come from the records of k_point_records instead of being computed in the warp;
// W: warps (displacement nodes) per block, chosen by the autotuner among 2, 4 and 8
template <int DIM, int ND, int NIP, int KIND, bool STAGED = false, int W = 4>
struct FusedShape
{
    static constexpr bool GD = KIND == NUTO_GPU_GRADIENT_DAMAGE;
    static constexpr int recF4 = ND + (GD ? 5 : 1); // float4 per record: ND gradients, the scalars
    static constexpr int cpp = 32 / NIP;             // cells per pass
    static constexpr int nr = DIM + (GD ? 1 : 0);     // rows per node
    // per warp, in floats: node data (2 float4 per (cell, node)), eeq values in FP64 (2 floats each), per point
    // the node gradients with N (float4 per node) and four float4 of scalars (lambda w, mu w, w, c g w | P_a, the
    // eeq-gradient coupling | the Voigt vector t of the (eeq, disp) block); the row buffer
    // rows of float4 indexed by the integration point are padded to ND + 1 (and the scalars to 5) float4 entries:
    // the 8 lanes of a cell, one per point, then touch 8 distinct bank groups instead of one (a stride of 128 bytes
    // would serialise them 8-fold)
    // staged: the records of a pass in their global layout, [cell][point][recF4] float4 (an odd row length of
    // ND + 5 = 13 float4 keeps the 8 lanes of a cell on distinct bank groups); fused: gradients and scalars apart
    static constexpr int nodeF = STAGED ? 0 : cpp * ND * 8;
    static constexpr int eF = GD && !STAGED ? cpp * ND * 2 : 0;
    static constexpr int gF = STAGED ? cpp * NIP * recF4 * 4 : cpp * NIP * (ND + 1) * 4;
    static constexpr int qF = 0;
    static constexpr int sF = STAGED ? 0 : cpp * NIP * 20; // 5 float4 per point: 4 used (scalars, P_a, t), 1 pad
    static constexpr int rowF = nr * kFusedRowCap;
    static constexpr int perWarp = nodeF + eF + gF + qF + sF + rowF;
    static constexpr int tabF = NIP * (ND + 1) * 4 + NIP; // (dN/dxi, N) per point and node, weights
    static constexpr int tabOff = (tabF + 3) / 4 * 4; // per-warp regions start 16-byte aligned
    static constexpr size_t smem = (static_cast<size_t>(W) * perWarp + tabOff) * sizeof(float);
    static_assert(cpp * NIP == 32 && cpp * ND == 32, "one lane per (cell, point) and per (cell, node)");
};

__device__ __forceinline__ float4 F4(float x, float y, float z, float w)
{
    return make_float4(x, y, z, w);
}

// B_n^T v for the node gradient g (Voigt columns; 2D xx yy xy, 3D xx yy zz yz zx xy). Every product and sum of
// the node-pair arithmetic is rounded explicitly (no contraction left to the compiler), so that every kernel and
// both the scalar and the packed forms below give bitwise the same blocks.
template <int DIM>
__device__ __forceinline__ float3 BtV(float gx, float gy, float gz, const float* v)
{
    if (DIM == 2)
        return make_float3(__fmaf_rn(gy, v[2], __fmul_rn(gx, v[0])), __fmaf_rn(gx, v[2], __fmul_rn(gy, v[1])), 0.f);
    return make_float3(__fmaf_rn(gy, v[5], __fmaf_rn(gz, v[4], __fmul_rn(gx, v[0]))),
                       __fmaf_rn(gx, v[5], __fmaf_rn(gz, v[3], __fmul_rn(gy, v[1]))),
                       __fmaf_rn(gx, v[4], __fmaf_rn(gy, v[3], __fmul_rn(gz, v[2]))));
}

// g . s over DIM components, explicitly rounded
template <int DIM>
__device__ __forceinline__ float DotG(float gx, float gy, float gz, float sx, float sy, float sz)
{
    float r = __fmaf_rn(gy, sy, __fmul_rn(gx, sx));
    if (DIM == 3)
        r = __fmaf_rn(gz, sz, r);
    return r;
}

// ---- node-pair block of one integration point --------------------------------------------------------------------
// lambda w g_a g_b^T + mu w (g_b g_a^T + (g_a . g_b) I), and for gradient damage P_a N_b (disp, eeq), -N_a Q_b^T
// (eeq, disp) and (w N_a + gs_a) N_b + c g w (g_a . g_b) (eeq, eeq). g: (dN/dX, N) float4; s0 = (lambda w, mu w, w,
// c g w); pa = (P_a, gs_a); qb = (Q_b, -).
template <int DIM>
struct PairAcc
{
    float uu[DIM][DIM], ue[DIM], eu[DIM], ee, dg;
    __device__ __forceinline__ void zero()
    {
#pragma unroll
        for (int k = 0; k < DIM; ++k)
        {
            ue[k] = eu[k] = 0.f;
#pragma unroll
            for (int l = 0; l < DIM; ++l)
                uu[k][l] = 0.f;
        }
        ee = dg = 0.f;
    }
};

template <int DIM, bool GD>
__device__ __forceinline__ void PairPoint(const float4& ga, const float4& gb, const float4& s0, const float4& pa,
                                          const float4& qb, PairAcc<DIM>& c)
{
    const float av[3] = {ga.x, ga.y, ga.z}, bv[3] = {gb.x, gb.y, gb.z};
    const float gab = DotG<DIM>(av[0], av[1], av[2], bv[0], bv[1], bv[2]);
#pragma unroll
    for (int k = 0; k < DIM; ++k)
    {
        const float lk = __fmul_rn(s0.x, av[k]), mk = __fmul_rn(s0.y, bv[k]);
#pragma unroll
        for (int l = 0; l < DIM; ++l)
            c.uu[k][l] = __fmaf_rn(mk, av[l], __fmaf_rn(lk, bv[l], c.uu[k][l]));
    }
    c.dg = __fmaf_rn(s0.y, gab, c.dg);
    if (GD)
    {
        const float pv[3] = {pa.x, pa.y, pa.z}, qv[3] = {qb.x, qb.y, qb.z};
#pragma unroll
        for (int k = 0; k < DIM; ++k)
        {
            c.ue[k] = __fmaf_rn(pv[k], gb.w, c.ue[k]);
            c.eu[k] = __fmaf_rn(-ga.w, qv[k], c.eu[k]);
        }
        c.ee = __fmaf_rn(s0.w, gab, __fmaf_rn(__fmaf_rn(s0.z, ga.w, pa.w), gb.w, c.ee));
    }
}

// The same for two blocks (a0, b) and (a1, b) at once in packed FP32 pairs (fma.rn.f32x2 / mul.rn.f32x2: each half
// rounded as the scalar operation, so the results are bitwise those of PairPoint).
using F2 = unsigned long long;
__device__ __forceinline__ F2 Pk(float a, float b)
{
    F2 r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a), "f"(b));
    return r;
}
__device__ __forceinline__ void Unpk(F2 r, float& a, float& b)
{
    asm("mov.b64 {%0, %1}, %2;" : "=f"(a), "=f"(b) : "l"(r));
}
__device__ __forceinline__ F2 Fma2(F2 a, F2 b, F2 c)
{
    F2 d;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
    return d;
}
__device__ __forceinline__ F2 Mul2(F2 a, F2 b)
{
    F2 d;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}

template <int DIM>
struct PairAcc2
{
    F2 uu[DIM][DIM], ue[DIM], eu[DIM], ee, dg;
    __device__ __forceinline__ void zero()
    {
        const F2 z = Pk(0.f, 0.f);
#pragma unroll
        for (int k = 0; k < DIM; ++k)
        {
            ue[k] = eu[k] = z;
#pragma unroll
            for (int l = 0; l < DIM; ++l)
                uu[k][l] = z;
        }
        ee = dg = z;
    }
    // the two blocks' accumulators as scalars
    __device__ __forceinline__ void split(PairAcc<DIM>& c0, PairAcc<DIM>& c1) const
    {
#pragma unroll
        for (int k = 0; k < DIM; ++k)
        {
            Unpk(ue[k], c0.ue[k], c1.ue[k]);
            Unpk(eu[k], c0.eu[k], c1.eu[k]);
#pragma unroll
            for (int l = 0; l < DIM; ++l)
                Unpk(uu[k][l], c0.uu[k][l], c1.uu[k][l]);
        }
        Unpk(ee, c0.ee, c1.ee);
        Unpk(dg, c0.dg, c1.dg);
    }
};

template <int DIM, bool GD>
__device__ __forceinline__ void PairPoint2(const float4& ga0, const float4& ga1, const float4& gb, const float4& s0,
                                           const float4& pa0, const float4& pa1, const float4& qb, PairAcc2<DIM>& c)
{
    const F2 A[3] = {Pk(ga0.x, ga1.x), Pk(ga0.y, ga1.y), Pk(ga0.z, ga1.z)};
    const F2 B[3] = {Pk(gb.x, gb.x), Pk(gb.y, gb.y), Pk(gb.z, gb.z)};
    const float bv[3] = {gb.x, gb.y, gb.z};
    F2 gab = Fma2(A[1], B[1], Mul2(A[0], B[0]));
    if (DIM == 3)
        gab = Fma2(A[2], B[2], gab);
    const F2 sx = Pk(s0.x, s0.x);
#pragma unroll
    for (int k = 0; k < DIM; ++k)
    {
        const F2 lk = Mul2(sx, A[k]);
        const float m = __fmul_rn(s0.y, bv[k]);
        const F2 mk = Pk(m, m);
#pragma unroll
        for (int l = 0; l < DIM; ++l)
            c.uu[k][l] = Fma2(mk, A[l], Fma2(lk, B[l], c.uu[k][l]));
    }
    c.dg = Fma2(Pk(s0.y, s0.y), gab, c.dg);
    if (GD)
    {
        const F2 P[3] = {Pk(pa0.x, pa1.x), Pk(pa0.y, pa1.y), Pk(pa0.z, pa1.z)};
        const F2 Q[3] = {Pk(qb.x, qb.x), Pk(qb.y, qb.y), Pk(qb.z, qb.z)};
        const F2 gbw = Pk(gb.w, gb.w), nga = Pk(-ga0.w, -ga1.w);
#pragma unroll
        for (int k = 0; k < DIM; ++k)
        {
            c.ue[k] = Fma2(P[k], gbw, c.ue[k]);
            c.eu[k] = Fma2(nga, Q[k], c.eu[k]);
        }
        const F2 t = Fma2(Pk(s0.z, s0.z), Pk(ga0.w, ga1.w), Pk(pa0.w, pa1.w));
        c.ee = Fma2(Pk(s0.w, s0.w), gab, Fma2(t, gbw, c.ee));
    }
}

// Everything the node-pair blocks of one integration point need, in FP32: the node gradients dN/dX, the scalars
// (lambda w, mu w, w, c g w for gradient damage; lambda w, mu w for LinearElastic, both with the cell's modulus
// factor), and for gradient damage the Voigt vectors sv (disp, eeq block: dsigma/domega omega' kappa' w) and tv
// (eeq, disp block: deps_eq/deps w) and the eeq-gradient coupling vector c g' omega' kappa' w grad eeq.
template <int DIM, int ND>
struct PointOut
{
    float g[ND][DIM];
    float s0[4];
    float sv[6], tv[6], scge[DIM];
};

// Geometry, strain and law at integration point q of cell e from the cell's node data: X (coordinates relative to
// the first node, eeq value in .w), U (displacements), E64 (eeq values in FP64, for the branch decisions); T the
// (dN/dxi, N) table row of q and w its weight. The loading/unloading and damage branches are the FP64 kernels'
// (decided in FP32 where the error bound of eeq separates the operands, else in FP64 as k_tangent<double> forms
// eeq: same order, FP64 shape values tabN).
template <int DIM, int ND, int NIP, int KIND>
__device__ __forceinline__ void PointData(const FusedArgs& A, const LawParams& L, const float4* T, float w,
                                          const float4* X, const float4* U, const double* E64, int q, int64_t e,
                                          PointOut<DIM, ND>& o)
{
    constexpr bool GD = KIND == NUTO_GPU_GRADIENT_DAMAGE;
    constexpr int VD = DIM == 2 ? 3 : 6;
    const int64_t n = A.nCells;
    float J[DIM][DIM];
#pragma unroll
    for (int i = 0; i < DIM; ++i)
#pragma unroll
        for (int j = 0; j < DIM; ++j)
            J[i][j] = 0.f;
#pragma unroll
    for (int nd = 0; nd < ND; ++nd)
    {
        const float4 x = X[nd], t = T[nd];
        const float xv[3] = {x.x, x.y, x.z}, tv[3] = {t.x, t.y, t.z};
#pragma unroll
        for (int i = 0; i < DIM; ++i)
#pragma unroll
            for (int j = 0; j < DIM; ++j)
                J[i][j] += xv[i] * tv[j];
    }
    float det, inv[DIM][DIM];
    if (DIM == 2)
    {
        det = J[0][0] * J[1][1] - J[0][1] * J[1][0];
        const float id = 1.f / det;
        inv[0][0] = J[1][1] * id;
        inv[0][1] = -J[0][1] * id;
        inv[1][0] = -J[1][0] * id;
        inv[1][1] = J[0][0] * id;
    }
    else
    {
        const float c00 = J[1][1] * J[2 % DIM][2 % DIM] - J[1][2 % DIM] * J[2 % DIM][1];
        const float c10 = J[1][2 % DIM] * J[2 % DIM][0] - J[1][0] * J[2 % DIM][2 % DIM];
        const float c20 = J[1][0] * J[2 % DIM][1] - J[1][1] * J[2 % DIM][0];
        det = J[0][0] * c00 + J[0][1] * c10 + J[0][2 % DIM] * c20;
        const float id = 1.f / det;
        inv[0][0] = c00 * id;
        inv[1][0] = c10 * id;
        inv[2 % DIM][0] = c20 * id;
        inv[0][1] = (J[0][2 % DIM] * J[2 % DIM][1] - J[0][1] * J[2 % DIM][2 % DIM]) * id;
        inv[1][1] = (J[0][0] * J[2 % DIM][2 % DIM] - J[0][2 % DIM] * J[2 % DIM][0]) * id;
        inv[2 % DIM][1] = (J[0][1] * J[2 % DIM][0] - J[0][0] * J[2 % DIM][1]) * id;
        inv[0][2 % DIM] = (J[0][1] * J[1][2 % DIM] - J[0][2 % DIM] * J[1][1]) * id;
        inv[1][2 % DIM] = (J[0][2 % DIM] * J[1][0] - J[0][0] * J[1][2 % DIM]) * id;
        inv[2 % DIM][2 % DIM] = (J[0][0] * J[1][1] - J[0][1] * J[1][0]) * id;
    }
    const float wdj = w * det;
    // per-cell Young's modulus factor: scales the material tangent and dsigma/domega
    const float wdjE = A.escale ? wdj * static_cast<float>(A.escale[e]) : wdj;
    float H[DIM][DIM], ge[DIM];
    float eeq = 0.f, eabs = 0.f;
#pragma unroll
    for (int i = 0; i < DIM; ++i)
    {
        ge[i] = 0.f;
#pragma unroll
        for (int j = 0; j < DIM; ++j)
            H[i][j] = 0.f;
    }
#pragma unroll
    for (int nd = 0; nd < ND; ++nd)
    {
        const float4 t = T[nd];
        const float tv[3] = {t.x, t.y, t.z};
#pragma unroll
        for (int k = 0; k < DIM; ++k)
        {
            float s = 0.f;
#pragma unroll
            for (int j = 0; j < DIM; ++j)
                s += tv[j] * inv[j][k];
            o.g[nd][k] = s;
        }
        const float4 uv = U[nd];
        const float uc[3] = {uv.x, uv.y, uv.z};
#pragma unroll
        for (int c = 0; c < DIM; ++c)
#pragma unroll
            for (int d = 0; d < DIM; ++d)
                H[c][d] += uc[c] * o.g[nd][d];
        if (GD)
        {
            const float ev = X[nd].w;
            eeq += t.w * ev;
            eabs += fabsf(t.w * ev);
#pragma unroll
            for (int d = 0; d < DIM; ++d)
                ge[d] += ev * o.g[nd][d];
        }
    }
    float eps[VD];
    if (DIM == 2)
    {
        eps[0] = H[0][0];
        eps[1] = H[1][1];
        eps[2 % VD] = H[0][1] + H[1][0];
    }
    else
    {
        eps[0] = H[0][0];
        eps[1] = H[1][1];
        eps[2] = H[DIM - 1][DIM - 1];
        eps[3 % VD] = H[1][DIM - 1] + H[DIM - 1][1];
        eps[4 % VD] = H[0][DIM - 1] + H[DIM - 1][0];
        eps[5 % VD] = H[0][1] + H[1][0];
    }
    if (!GD)
    {
        // LinearElastic: C11 = lambda + 2 mu, C12 = lambda, C33 = mu
        o.s0[0] = static_cast<float>(L.C12) * wdjE;
        o.s0[1] = static_cast<float>(L.C33) * wdjE;
        o.s0[2] = o.s0[3] = 0.f;
        return;
    }
    const double kh64 = A.kappa[NG_IDX(e * NIP + q, n * NIP, 55)];
    const float kh = static_cast<float>(kh64);
    const float bound = 1.0e-6f * eabs + 1.0e-30f;
    double e64 = 0.;
    bool have64 = false;
    auto eeq64 = [&]() {
        if (!have64)
        {
            double s = 0.;
            for (int nd = 0; nd < ND; ++nd)
                s += A.tabN[q * ND + nd] * E64[nd];
            e64 = s;
            have64 = true;
        }
        return e64;
    };
    bool loading;
    if (fabsf(eeq - kh) > bound + 1.0e-7f * fabsf(kh))
        loading = eeq >= kh;
    else
        loading = eeq64() >= kh64;
    bool damaged;
    const float k0f = static_cast<float>(L.kappa0);
    if (!loading)
        damaged = kh64 >= L.kappa0;
    else if (fabsf(eeq - k0f) > bound + 1.0e-7f * k0f)
        damaged = eeq >= k0f;
    else
        damaged = eeq64() >= L.kappa0;
    const float kap = loading ? (have64 ? static_cast<float>(e64) : eeq) : kh;
    float omega = 0.f, dOdK = 0.f;
    if (damaged)
    {
        // DamageLawExponential (DamageLawExponential.h:40-52) above kappa0
        const float al = static_cast<float>(L.alpha), be = static_cast<float>(L.beta);
        const float ex = expf(be * (k0f - kap));
        const float r = k0f / kap;
        omega = 1.f - r * (1.f - al + al * ex);
        dOdK = r * ((1.f / kap + be) * al * ex + (1.f - al) / kap);
    }
    const float dKdE = loading ? 1.f : 0.f;
    const float gI = InteractionFactor<float>(L, omega);
    const float dgdw = InteractionDerivative<float>(L, omega);
    float lam, mu;
    LedTangentLameParams<float, DIM>(L, eps, omega, lam, mu);
    float dsdw[VD], dn[VD];
    LedDstressDomega<float, DIM>(L, eps, dsdw);
    MisesDerivative<float, DIM>(L, eps, dn);
    const float f1 = dOdK * dKdE * wdj, f1E = dOdK * dKdE * wdjE;
#pragma unroll
    for (int v = 0; v < 6; ++v)
    {
        o.sv[v] = v < VD ? dsdw[v < VD ? v : 0] * f1E : 0.f; // (disp, eeq): B^T (dsigma/domega w' k') N
        o.tv[v] = v < VD ? dn[v < VD ? v : 0] * wdj : 0.f;   // (eeq, disp): -N^T (deps_eq/deps)^T B
    }
    const float c = static_cast<float>(L.c);
    const float sc = c * dgdw * f1;
#pragma unroll
    for (int d = 0; d < DIM; ++d)
        o.scge[d] = sc * ge[d];
    o.s0[0] = lam * wdjE;
    o.s0[1] = mu * wdjE;
    o.s0[2] = wdj;
    o.s0[3] = c * gI * wdj;
}

// Copies the records of the pass's cells (cells kp .. min(kp + CPP, k1) of the node's list) into the warp's buffer
// with 16-byte asynchronous copies, one contiguous block per cell, and commits them as one group.
template <int DIM, int ND, int NIP, int KIND>
__device__ __forceinline__ void StageRecords(const FusedArgs& A, const float4* __restrict__ recs, float4* sBuf,
                                             int64_t kp, int64_t k1, int lane)
{
    using Sh = FusedShape<DIM, ND, NIP, KIND, true>;
    constexpr int CPP = Sh::cpp;
    const int64_t n = A.nCells; // the records' extent in checked builds
    (void)n;
    float4* sG = sBuf;
    constexpr int R4 = Sh::recF4;
    constexpr int PER_CELL = NIP * R4; // float4 of one cell's records, contiguous in both places
#pragma unroll
    for (int cs = 0; cs < CPP; ++cs)
    {
        const int64_t kc = kp + cs;
        if (kc >= k1)
            break;
        const int64_t e = A.cellIdx[kc];
        const float4* src = recs + NG_IDX(e, n, 58) * PER_CELL;
        float4* dst = sG + cs * PER_CELL;
        for (int i = lane; i < PER_CELL; i += 32)
        {
            const unsigned sa = static_cast<unsigned>(__cvta_generic_to_shared(dst + i));
            asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(sa), "l"(src + i) : "memory");
        }
    }
    asm volatile("cp.async.commit_group;\n" ::: "memory");
}

// Per point of the staged pass, the node-a quantities P_a = B_a^T sv and (c g' omega' kappa' w grad eeq) . g_a in
// place of the record's coupling vector, so that PassBlocks reads what the fused variant computes.
template <int DIM, int ND, int NIP, int KIND>
__device__ __forceinline__ void PrepRecords(const FusedArgs& A, float4* sG, int64_t kp, int64_t k1, int lane)
{
    constexpr bool GD = KIND == NUTO_GPU_GRADIENT_DAMAGE;
    constexpr int R4 = FusedShape<DIM, ND, NIP, KIND, true>::recF4;
    if (GD)
    {
        const int cs = lane / NIP, q = lane % NIP;
        const int64_t kc = kp + cs;
        if (kc < k1)
        {
            const int ia = A.cellLoc[kc];
            const float4* row = sG + (cs * NIP + q) * R4;
            const float4 ga = row[ia];
            float4* S = sG + (cs * NIP + q) * R4 + ND;
            const float4 s1 = S[1], s2 = S[2], s4 = S[4];
            const float sv[6] = {s4.x, s4.y, s4.z, s4.w, s1.w, s2.w};
            const float3 pa = BtV<DIM>(ga.x, ga.y, ga.z, sv);
            const float gs = DotG<DIM>(ga.x, ga.y, ga.z, s1.x, s1.y, s1.z);
            S[1] = F4(pa.x, pa.y, pa.z, gs);
        }
    }
}

// (B) of one pass: lane (cell slot, neighbour b) integrates the node-pair block (a, b) over the points and adds it
// into a's rows (sRow) at the ranks of b, one cell slot after the other. sG / sS: the pass's per-point data in the
// staged (record rows) or fused (padded arrays) layout.
template <int DIM, int ND, int NIP, int KIND, bool STAGED>
__device__ __forceinline__ void PassBlocks(const FusedArgs& A, const float4* sG, const float4* sS, float* sRow,
                                           int64_t kp, int64_t k1, int lane, int32_t bUU, int32_t bUE, int32_t bEU,
                                           int32_t bEE)
{
    using Sh = FusedShape<DIM, ND, NIP, KIND, STAGED>;
    constexpr bool GD = Sh::GD;
    constexpr int CPP = Sh::cpp, NDP = ND + 1;
    const int64_t n = A.nCells;
    // (B) lane (cell slot, neighbour b): the node-pair block (a, b) integrated over the points, added into a's
    // rows at the ranks of b
    {
        const int cs = lane / ND, b = lane % ND;
        const int64_t kc = kp + cs;
        PairAcc<DIM> acc;
        acc.zero();
        int r0 = 0, r1 = 0, r2 = 0, r3 = 0;
        bool active = false;
        if (kc < k1)
        {
            const int64_t e = A.cellIdx[kc];
            const int ia = A.cellLoc[kc];
            // ranks of b in a's neighbour lists (loaded first: their latency overlaps the integration)
            const int64_t ridx = static_cast<int64_t>(ia * ND + b) * n + e;
            r0 = A.rank[0][ridx];
            if (GD)
            {
                r1 = A.rank[1][ridx];
                r2 = A.rank[2][ridx];
                r3 = A.rank[3][ridx];
            }
#pragma unroll 2
            for (int q = 0; q < NIP; ++q)
            {
                // gradients and scalars of point q: one record row (staged) or the padded arrays (fused)
                const float4* G = STAGED ? sG + (cs * NIP + q) * Sh::recF4 : sG + (cs * NIP + q) * NDP;
                const float4* SR = STAGED ? G + ND : sS + (cs * NIP + q) * 5;
                const float4 ga = G[ia], gb = G[b];
                const float4 s0 = SR[0];
                float4 s1 = F4(0.f, 0.f, 0.f, 0.f), qb4 = s1;
                if (GD)
                {
                    s1 = SR[1]; // (P_a, gs_a)
                    const float4 t0 = SR[2], t1 = SR[3];
                    const float tv[6] = {t0.x, t0.y, t0.z, t1.x, t1.y, t1.z};
                    const float3 qb = BtV<DIM>(gb.x, gb.y, gb.z, tv); // B_b^T t
                    qb4 = F4(qb.x, qb.y, qb.z, 0.f);
                }
                PairPoint<DIM, GD>(ga, gb, s0, s1, qb4, acc);
            }
            active = true;
        }
        float(&uu)[DIM][DIM] = acc.uu;
        float(&ue)[DIM] = acc.ue;
        float(&eu)[DIM] = acc.eu;
        const float ee = acc.ee, dg = acc.dg;
        // the cells of a pass can share b: their blocks are added one cell slot after the other (the b of one
        // cell are distinct nodes, so the 8 lanes of a slot write distinct positions); fixed order, no atomics
#pragma unroll
        for (int r = 0; r < CPP; ++r)
        {
            if (active && cs == r)
            {
#pragma unroll
                for (int k = 0; k < DIM; ++k)
                {
                    float* row = sRow + k * kFusedRowCap;
#pragma unroll
                    for (int l = 0; l < DIM; ++l)
                        row[NG_IDX(bUU + DIM * r0 + l, kFusedRowCap, 56)] += uu[k][l] + (k == l ? dg : 0.f);
                    if (GD)
                        row[NG_IDX(bUE + r1, kFusedRowCap, 56)] += ue[k];
                }
                if (GD)
                {
                    float* row = sRow + DIM * kFusedRowCap;
#pragma unroll
                    for (int l = 0; l < DIM; ++l)
                        row[NG_IDX(bEU + DIM * r2 + l, kFusedRowCap, 56)] += eu[l];
                    row[NG_IDX(bEE + r3, kFusedRowCap, 56)] += ee;
                }
            }
            __syncwarp();
        }
    }
}

template <int DIM, int ND, int NIP, int KIND, bool STAGED, int W>
__global__ void __launch_bounds__(W * 32, 20 / W)
        k_tangent_fused(FusedArgs A, LawParams L, const double* __restrict__ u, const float4* __restrict__ recs,
                        float* __restrict__ vals)
{
    using Sh = FusedShape<DIM, ND, NIP, KIND, STAGED, W>;
    constexpr bool GD = Sh::GD;
    constexpr int CPP = Sh::cpp, NR = Sh::nr;
    extern __shared__ __align__(16) float smF[];
    const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
    constexpr int NDP = ND + 1;                     // padded row length (float4)
    float4* sTab = reinterpret_cast<float4*>(smF); // [NIP][NDP]: dN/dxi, N
    float* sW = smF + NIP * NDP * 4;               // [NIP]
    float* base = smF + Sh::tabOff + wid * Sh::perWarp;
    float4* sNodeX = reinterpret_cast<float4*>(base);                   // [CPP][ND]: X - X0, eeq
    float4* sNodeU = sNodeX + CPP * ND;                                 // [CPP][ND]: u
    double* sE64 = reinterpret_cast<double*>(base + Sh::nodeF);         // [CPP][ND]: eeq (gradient damage)
    float4* sG = reinterpret_cast<float4*>(base + Sh::nodeF + Sh::eF);  // [CPP][NIP][NDP]: dN/dX, N
    float4* sS = reinterpret_cast<float4*>(base + Sh::nodeF + Sh::eF + Sh::gF + Sh::qF); // [CPP][NIP][5]
    float* sRow = base + Sh::nodeF + Sh::eF + Sh::gF + Sh::qF + Sh::sF; // [NR][kFusedRowCap]
    for (int i = threadIdx.x; i < NIP * ND; i += blockDim.x)
    {
        const int q = i / ND, nd = i % ND;
        const double* d = A.tabDN + (q * ND + nd) * 3;
        sTab[q * NDP + nd] = F4(static_cast<float>(d[0]), static_cast<float>(d[1]), DIM == 3 ? static_cast<float>(d[2]) : 0.f,
                     static_cast<float>(A.tabN[q * ND + nd]));
    }
    for (int i = threadIdx.x; i < NIP; i += blockDim.x)
        sW[i] = static_cast<float>(A.tabW[i]);
    __syncthreads();

    const int64_t a = static_cast<int64_t>(blockIdx.x) * W + wid;
    if (a >= A.nNodes)
        return; // the whole warp leaves; only warp-level synchronisation follows
    int64_t rs[NR];
    int len[NR];
    const int64_t g0 = A.gdofD[a];
#pragma unroll
    for (int k = 0; k < DIM; ++k)
    {
        rs[k] = A.rowPtr[NG_IDX(g0 + k, A.nRows, 50)];
        len[k] = static_cast<int>(A.rowPtr[g0 + k + 1] - rs[k]);
    }
    int32_t ae = 0;
    if (GD)
    {
        ae = A.eOf[a];
        const int64_t ge = A.gdofE[ae];
        rs[DIM] = A.rowPtr[NG_IDX(ge, A.nRows, 50)];
        len[DIM] = static_cast<int>(A.rowPtr[ge + 1] - rs[DIM]);
    }
    const int32_t bUU = A.blk[0][a];
    const int32_t bUE = GD ? A.blk[1][a] : 0;
    const int32_t bEU = GD ? A.blk[2][ae] : 0;
    const int32_t bEE = GD ? A.blk[3][ae] : 0;
#pragma unroll
    for (int k = 0; k < NR; ++k)
        for (int i = lane; i < kFusedRowCap; i += 32)
            sRow[k * kFusedRowCap + i] = 0.f;

    const int64_t k0 = A.cellPtr[a], k1 = A.cellPtr[a + 1];
    const int64_t n = A.nCells;
    for (int64_t kp = k0; kp < k1; kp += CPP)
    {
        __syncwarp();
        if constexpr (STAGED)
        {
            StageRecords<DIM, ND, NIP, KIND>(A, recs, sG, kp, k1, lane);
            asm volatile("cp.async.wait_group 0;\n" ::: "memory");
            __syncwarp();
            PrepRecords<DIM, ND, NIP, KIND>(A, sG, kp, k1, lane);
            __syncwarp();
        }
        else
        {
        // (0) lane (cell slot, node): the node's data of the cell
        {
            const int cs = lane / ND, nd = lane % ND;
            const int64_t kc = kp + cs;
            if (kc < k1)
            {
                const int64_t e = A.cellIdx[kc];
                const int32_t nD =
                        static_cast<int32_t>(NG_IDX(A.connD[static_cast<int64_t>(nd) * n + e], A.nNodesD, 51));
                const int64_t gd = A.gdofD[nD];
                float x[3] = {0.f, 0.f, 0.f}, v[3] = {0.f, 0.f, 0.f};
#pragma unroll
                for (int d = 0; d < DIM; ++d)
                {
                    x[d] = A.relX[(static_cast<int64_t>(nd) * DIM + d) * n + e];
                    v[d] = static_cast<float>(u[NG_IDX(gd + d, A.nDofs, 52)]);
                }
                float ev = 0.f;
                if (GD)
                {
                    const int32_t nE =
                            static_cast<int32_t>(NG_IDX(A.connE[static_cast<int64_t>(nd) * n + e], A.nNodesE, 53));
                    const double e64 = u[NG_IDX(A.gdofE[nE], A.nDofs, 54)];
                    sE64[cs * ND + nd] = e64;
                    ev = static_cast<float>(e64);
                }
                sNodeX[cs * ND + nd] = F4(x[0], x[1], x[2], ev);
                sNodeU[cs * ND + nd] = F4(v[0], v[1], v[2], 0.f);
            }
        }
        __syncwarp();
        // (A) lane (cell slot, integration point): geometry, strain and law in FP32
        {
            const int cs = lane / NIP, q = lane % NIP;
            const int64_t kc = kp + cs;
            if (kc < k1)
            {
                const int64_t e = A.cellIdx[kc];
                const int ia = A.cellLoc[kc];
                PointOut<DIM, ND> o;
                PointData<DIM, ND, NIP, KIND>(A, L, sTab + q * NDP, sW[q], sNodeX + cs * ND, sNodeU + cs * ND,
                                              sE64 + cs * ND, q, e, o);
                float4* G = sG + (cs * NIP + q) * NDP;
                const float4* T = sTab + q * NDP;
#pragma unroll
                for (int nd = 0; nd < ND; ++nd)
                    G[nd] = F4(o.g[nd][0], o.g[nd][1], DIM == 3 ? o.g[nd][DIM - 1] : 0.f, T[nd].w);
                float4* S = sS + (cs * NIP + q) * 5;
                S[0] = F4(o.s0[0], o.s0[1], o.s0[2], o.s0[3]);
                if (GD)
                {
                    float gA[DIM]; // node a's gradient (local index ia)
#pragma unroll
                    for (int d = 0; d < DIM; ++d)
                    {
                        gA[d] = o.g[0][d];
#pragma unroll
                        for (int nd = 1; nd < ND; ++nd)
                            gA[d] = nd == ia ? o.g[nd][d] : gA[d];
                    }
                    const float gs = DotG<DIM>(gA[0], gA[1], DIM == 3 ? gA[DIM - 1] : 0.f, o.scge[0], o.scge[1],
                                               DIM == 3 ? o.scge[DIM - 1] : 0.f);
                    const float3 pa = BtV<DIM>(gA[0], gA[1], DIM == 3 ? gA[DIM - 1] : 0.f, o.sv);
                    S[1] = F4(pa.x, pa.y, pa.z, gs);
                    S[2] = F4(o.tv[0], o.tv[1], o.tv[2], 0.f);
                    S[3] = F4(o.tv[3], o.tv[4], o.tv[5], 0.f);
                }
            }
        }
        __syncwarp();
        }
        PassBlocks<DIM, ND, NIP, KIND, STAGED>(A, sG, sS, sRow, kp, k1, lane, bUU, bUE, bEU, bEE);
    }
    __syncwarp();
#pragma unroll
    for (int k = 0; k < NR; ++k)
        for (int i = lane; i < len[k]; i += 32)
            vals[NG_IDX(rs[k] + i, A.nnz, 57)] = sRow[k * kFusedRowCap + i];
}

// The staged node rows with the record copies double-buffered: a grid of resident blocks walks the displacement
// nodes (warp w takes nodes w, w + number of warps, ...), and while a warp integrates one pass of cells the copies
// of its next pass (of the same node, or the first pass of its next node) are already in flight into the other
// buffer. Same arithmetic and order per node as k_tangent_fused<STAGED>, so the values are bitwise the same.
template <int DIM, int ND, int NIP, int KIND, int W>
__global__ void __launch_bounds__(W * 32) k_tangent_rows_pipe(FusedArgs A, const float4* __restrict__ recs,
                                                            float* __restrict__ vals)
{
    using Sh = FusedShape<DIM, ND, NIP, KIND, true, W>;
    constexpr bool GD = Sh::GD;
    constexpr int CPP = Sh::cpp, NR = Sh::nr;
    constexpr int BUF = CPP * NIP * Sh::recF4; // float4 of one pass's records
    extern __shared__ __align__(16) float smF[];
    const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
    float4* buf0 = reinterpret_cast<float4*>(smF) + static_cast<size_t>(wid) * (2 * BUF + NR * kFusedRowCap / 4);
    float4* buf1 = buf0 + BUF;
    float* sRow = reinterpret_cast<float*>(buf1 + BUF);
    const int64_t nw = static_cast<int64_t>(gridDim.x) * W;
    int64_t a = static_cast<int64_t>(blockIdx.x) * W + wid;
    if (a >= A.nNodes)
        return; // the whole warp leaves; only warp-level synchronisation follows
    // per-node set-up: row starts and lengths, block offsets, cleared rows
    int64_t rs[NR];
    int len[NR];
    int32_t bUU = 0, bUE = 0, bEU = 0, bEE = 0;
    int64_t k0 = 0, k1 = 0;
    auto enterNode = [&](int64_t node) {
        const int64_t g0 = A.gdofD[node];
#pragma unroll
        for (int k = 0; k < DIM; ++k)
        {
            rs[k] = A.rowPtr[NG_IDX(g0 + k, A.nRows, 50)];
            len[k] = static_cast<int>(A.rowPtr[g0 + k + 1] - rs[k]);
        }
        int32_t ae = 0;
        if (GD)
        {
            ae = A.eOf[node];
            const int64_t ge = A.gdofE[ae];
            rs[DIM] = A.rowPtr[NG_IDX(ge, A.nRows, 50)];
            len[DIM] = static_cast<int>(A.rowPtr[ge + 1] - rs[DIM]);
        }
        bUU = A.blk[0][node];
        bUE = GD ? A.blk[1][node] : 0;
        bEU = GD ? A.blk[2][ae] : 0;
        bEE = GD ? A.blk[3][ae] : 0;
        k0 = A.cellPtr[node];
        k1 = A.cellPtr[node + 1];
#pragma unroll
        for (int k = 0; k < NR; ++k)
            for (int i = lane; i < kFusedRowCap; i += 32)
                sRow[k * kFusedRowCap + i] = 0.f;
    };
    enterNode(a);
    int64_t kp = k0;
    StageRecords<DIM, ND, NIP, KIND>(A, recs, buf0, kp, k1, lane);
    int cur = 0;
    while (true)
    {
        // the next pass: the node's next cells, or the first pass of the warp's next node (every node has at least
        // one pass, possibly empty)
        int64_t nextNode = a, nextKp = kp + CPP, nextK1 = k1;
        if (nextKp >= k1)
        {
            nextNode = a + nw;
            if (nextNode < A.nNodes)
            {
                nextKp = A.cellPtr[nextNode];
                nextK1 = A.cellPtr[nextNode + 1];
            }
        }
        float4* now = cur ? buf1 : buf0;
        float4* next = cur ? buf0 : buf1;
        if (nextNode < A.nNodes)
            StageRecords<DIM, ND, NIP, KIND>(A, recs, next, nextKp, nextK1, lane);
        else
            asm volatile("cp.async.commit_group;\n" ::: "memory"); // an empty group keeps the count uniform
        asm volatile("cp.async.wait_group 1;\n" ::: "memory");  // this pass's copies (all but the newest group)
        __syncwarp();
        PrepRecords<DIM, ND, NIP, KIND>(A, now, kp, k1, lane);
        __syncwarp();
        PassBlocks<DIM, ND, NIP, KIND, true>(A, now, nullptr, sRow, kp, k1, lane, bUU, bUE, bEU, bEE);
        __syncwarp();
        if (nextNode != a)
        {
            // the node's rows are complete
#pragma unroll
            for (int k = 0; k < NR; ++k)
                for (int i = lane; i < len[k]; i += 32)
                    vals[NG_IDX(rs[k] + i, A.nnz, 57)] = sRow[k * kFusedRowCap + i];
            __syncwarp();
            if (nextNode >= A.nNodes)
                break;
            a = nextNode;
            enterNode(a);
            __syncwarp();
        }
        kp = nextKp;
        cur ^= 1;
    }
    asm volatile("cp.async.wait_group 0;\n" ::: "memory");
}

// Per-point records of the staged tangent: one thread per (cell, integration point) evaluates PointData once and
// writes ND float4 (dN/dX, N) and the scalars (gradient damage: lambda w, mu w, w, c g w | c g' w' k' w grad eeq,
// sv4 | tv0..2, sv5 | tv3..5 | sv0..3) contiguously per cell. The node data of a block's cells are loaded once into
// shared memory by one thread per (cell, node).
template <int DIM, int ND, int NIP, int KIND>
__global__ void __launch_bounds__(128) k_point_records(FusedArgs A, LawParams L, const double* __restrict__ u,
                                                      float4* __restrict__ recs)
{
    constexpr bool GD = KIND == NUTO_GPU_GRADIENT_DAMAGE;
    constexpr int CPB = 128 / NIP; // cells per block
    constexpr int R4 = FusedShape<DIM, ND, NIP, KIND, true>::recF4;
    static_assert(CPB * ND <= 128, "one thread per (cell, node)");
    __shared__ float4 sX[CPB][ND], sU[CPB][ND];
    __shared__ double sE[GD ? CPB : 1][ND];
    __shared__ float4 sT[NIP][ND];
    __shared__ float sWq[NIP];
    const int64_t n = A.nCells;
    const int64_t cell0 = static_cast<int64_t>(blockIdx.x) * CPB;
    for (int i = threadIdx.x; i < NIP * ND; i += blockDim.x)
    {
        const int q = i / ND, nd = i % ND;
        const double* d = A.tabDN + (q * ND + nd) * 3;
        sT[q][nd] = F4(static_cast<float>(d[0]), static_cast<float>(d[1]), DIM == 3 ? static_cast<float>(d[2]) : 0.f,
                       static_cast<float>(A.tabN[q * ND + nd]));
    }
    for (int i = threadIdx.x; i < NIP; i += blockDim.x)
        sWq[i] = static_cast<float>(A.tabW[i]);
    if (threadIdx.x < CPB * ND)
    {
        const int cl = threadIdx.x / ND, nd = threadIdx.x % ND;
        const int64_t e = cell0 + cl;
        if (e < n)
        {
            const int32_t nD = static_cast<int32_t>(NG_IDX(A.connD[static_cast<int64_t>(nd) * n + e], A.nNodesD, 51));
            const int64_t gd = A.gdofD[nD];
            float x[3] = {0.f, 0.f, 0.f}, v[3] = {0.f, 0.f, 0.f};
#pragma unroll
            for (int d = 0; d < DIM; ++d)
            {
                x[d] = A.relX[(static_cast<int64_t>(nd) * DIM + d) * n + e];
                v[d] = static_cast<float>(u[NG_IDX(gd + d, A.nDofs, 52)]);
            }
            float ev = 0.f;
            if (GD)
            {
                const int32_t nE =
                        static_cast<int32_t>(NG_IDX(A.connE[static_cast<int64_t>(nd) * n + e], A.nNodesE, 53));
                const double e64 = u[NG_IDX(A.gdofE[nE], A.nDofs, 54)];
                sE[cl][nd] = e64;
                ev = static_cast<float>(e64);
            }
            sX[cl][nd] = F4(x[0], x[1], x[2], ev);
            sU[cl][nd] = F4(v[0], v[1], v[2], 0.f);
        }
    }
    __syncthreads();
    const int cl = threadIdx.x / NIP, q = threadIdx.x % NIP;
    const int64_t e = cell0 + cl;
    if (cl >= CPB || e >= n)
        return;
    PointOut<DIM, ND> o;
    PointData<DIM, ND, NIP, KIND>(A, L, sT[q], sWq[q], sX[cl], sU[cl], GD ? sE[cl] : nullptr, q, e, o);
    float4* r = recs + (e * NIP + q) * R4;
#pragma unroll
    for (int nd = 0; nd < ND; ++nd)
        r[nd] = F4(o.g[nd][0], o.g[nd][1], DIM == 3 ? o.g[nd][DIM - 1] : 0.f, sT[q][nd].w);
    r[ND] = F4(o.s0[0], o.s0[1], o.s0[2], o.s0[3]);
    if (GD)
    {
        r[ND + 1] = F4(o.scge[0], o.scge[1], DIM == 3 ? o.scge[DIM - 1] : 0.f, o.sv[4]);
        r[ND + 2] = F4(o.tv[0], o.tv[1], o.tv[2], o.sv[5]);
        r[ND + 3] = F4(o.tv[3], o.tv[4], o.tv[5], 0.f);
        r[ND + 4] = F4(o.sv[0], o.sv[1], o.sv[2], o.sv[3]);
    }
}

// ---- element-matrix form (NUTO_GPU_TANGENT=cells, an autotuner candidate) ------------------------------------
// k_point_records as for the staged node rows, then
//   k_cell_matrices  one warp per cell: the cell's records staged into shared memory; per (point, node) the vectors
//                    P = B^T sv, gs = (c g' w' k' w grad eeq) . g and Q = B^T tv once; lane (a, b) integrates the
//                    node-pair blocks (a, b) and (a + ND/2, b) over the points with the node-row kernel's
//                    expressions, and the cell's element matrix goes to global memory as ND slabs, one per local
//                    node a: NR rows (a's displacement components, then its eeq row) x NC columns (the
//                    displacement components of b = 0..ND-1, b-major, then the eeq of b = 0..ND-1);
//   k_rows_from_cells one warp per displacement node: the slabs of its cells added in ascending cell order into
//                    shared rows at the ranks of b (a cell's b are distinct nodes: no conflicts), rows stored once.
// Every node-pair block is integrated once (the node rows form it once per row node) and the per-block sums and their
// order over the cells are those of the node-row kernel: the values are bitwise the same.
template <int DIM, int ND, int KIND>
struct CellSlab
{
    static constexpr bool GD = KIND == NUTO_GPU_GRADIENT_DAMAGE;
    static constexpr int nr = DIM + (GD ? 1 : 0);            // rows per local node
    static constexpr int nc = ND * DIM + (GD ? ND : 0);       // columns per row
    static constexpr int size = nr * nc;                      // floats per slab (global)
    static constexpr int pad = (size + 4 + 3) / 4 * 4;        // floats per slab in shared memory (16-byte rows, banks)
};

// All node-pair blocks of one cell integrated over its points from the cell's records (rec: NIP rows of R4 float4,
// the node gradients with N, then the scalars) and the per-(point, node) (P, gs) and Q (sPQ, gradient damage).
// 8-node cells: lane (a, b) and (a + 4, b) in packed FP32 pairs; otherwise one block per lane. write(a, b, acc) takes
// each finished block.
template <int DIM, int ND, int NIP, bool GD, typename Wr>
__device__ __forceinline__ void CellPairs(const float4* rec, int R4, const float4* sPQ, int lane, Wr&& write)
{
    const float4 z4 = F4(0.f, 0.f, 0.f, 0.f);
    if constexpr (ND == 8)
    {
        const int ia0 = lane / ND, ia1 = ia0 + 4, b = lane % ND;
        PairAcc2<DIM> c2;
        c2.zero();
#pragma unroll 2
        for (int q = 0; q < NIP; ++q)
        {
            const float4* G = rec + q * R4;
            const float4 ga0 = G[ia0], ga1 = G[ia1], gb = G[b], s0 = G[ND];
            float4 pa0 = z4, pa1 = z4, qb = z4;
            if (GD)
            {
                pa0 = sPQ[(q * ND + ia0) * 2];
                pa1 = sPQ[(q * ND + ia1) * 2];
                qb = sPQ[(q * ND + b) * 2 + 1];
            }
            PairPoint2<DIM, GD>(ga0, ga1, gb, s0, pa0, pa1, qb, c2);
        }
        PairAcc<DIM> c0, c1;
        c2.split(c0, c1);
        write(ia0, b, c0);
        write(ia1, b, c1);
    }
    else
    {
        for (int p = lane; p < ND * ND; p += 32)
        {
            const int ia = p / ND, b = p % ND;
            PairAcc<DIM> c;
            c.zero();
#pragma unroll 2
            for (int q = 0; q < NIP; ++q)
            {
                const float4* G = rec + q * R4;
                const float4 ga = G[ia], gb = G[b], s0 = G[ND];
                float4 pa = z4, qb = z4;
                if (GD)
                {
                    pa = sPQ[(q * ND + ia) * 2];
                    qb = sPQ[(q * ND + b) * 2 + 1];
                }
                PairPoint<DIM, GD>(ga, gb, s0, pa, qb, c);
            }
            write(ia, b, c);
        }
    }
}

// One finished block into slab a of an element matrix (slab rows of NC columns: the displacement components of b,
// b-major, then the eeq of b)
template <int DIM, int ND, bool GD, int NC>
__device__ __forceinline__ void PutBlock(float* slab, int b, const PairAcc<DIM>& c)
{
#pragma unroll
    for (int k = 0; k < DIM; ++k)
    {
#pragma unroll
        for (int l = 0; l < DIM; ++l)
            slab[k * NC + b * DIM + l] = c.uu[k][l] + (k == l ? c.dg : 0.f);
        if (GD)
            slab[k * NC + ND * DIM + b] = c.ue[k];
    }
    if (GD)
    {
#pragma unroll
        for (int l = 0; l < DIM; ++l)
            slab[DIM * NC + b * DIM + l] = c.eu[l];
        slab[DIM * NC + ND * DIM + b] = c.ee;
    }
}

template <int DIM, int ND, int NIP, int KIND, int W>
__global__ void __launch_bounds__(W * 32) k_cell_matrices(int64_t nCells, const float4* __restrict__ recs,
                                                          float* __restrict__ em)
{
    using Sh = FusedShape<DIM, ND, NIP, KIND, true>;
    using CS = CellSlab<DIM, ND, KIND>;
    constexpr bool GD = Sh::GD;
    constexpr int R4 = Sh::recF4;
    constexpr int PER_CELL = NIP * R4;
    extern __shared__ __align__(16) float smC[];
    const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
    constexpr int recF = PER_CELL * 4, pqF = GD ? NIP * ND * 8 : 0, emF = ND * CS::pad;
    float4* sR = reinterpret_cast<float4*>(smC + wid * (recF + pqF + emF));
    float4* sPQ = sR + PER_CELL;                                   // [NIP][ND][2]: (P, gs), (Q, 0)
    float* sEM = smC + wid * (recF + pqF + emF) + recF + pqF;      // [ND][pad]
    const int64_t e = static_cast<int64_t>(blockIdx.x) * W + wid;
    if (e >= nCells)
        return; // the whole warp leaves; only warp-level synchronisation follows
    const float4* src = recs + NG_IDX(e, nCells, 70) * PER_CELL;
    for (int i = lane; i < PER_CELL; i += 32)
    {
        const unsigned sa = static_cast<unsigned>(__cvta_generic_to_shared(sR + i));
        asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(sa), "l"(src + i) : "memory");
    }
    asm volatile("cp.async.commit_group;\n" ::: "memory");
    asm volatile("cp.async.wait_group 0;\n" ::: "memory");
    __syncwarp();
    if (GD)
    {
        // per (point, node): P = B^T sv and gs as PrepRecords forms them for the row node, Q = B^T tv as PassBlocks
        for (int it = lane; it < NIP * ND; it += 32)
        {
            const int q = it / ND, nd = it % ND;
            const float4* row = sR + q * R4;
            const float4 g = row[nd];
            const float4* S = row + ND;
            const float4 s1 = S[1], s2 = S[2], s3 = S[3], s4 = S[4];
            const float sv[6] = {s4.x, s4.y, s4.z, s4.w, s1.w, s2.w};
            const float tv[6] = {s2.x, s2.y, s2.z, s3.x, s3.y, s3.z};
            const float3 pa = BtV<DIM>(g.x, g.y, g.z, sv);
            const float gs = DotG<DIM>(g.x, g.y, g.z, s1.x, s1.y, s1.z);
            const float3 qb = BtV<DIM>(g.x, g.y, g.z, tv);
            sPQ[(q * ND + nd) * 2] = F4(pa.x, pa.y, pa.z, gs);
            sPQ[(q * ND + nd) * 2 + 1] = F4(qb.x, qb.y, qb.z, 0.f);
        }
        __syncwarp();
    }
    CellPairs<DIM, ND, NIP, GD>(sR, R4, sPQ, lane, [&](int ia, int b, const PairAcc<DIM>& c) {
        PutBlock<DIM, ND, GD, CS::nc>(sEM + ia * CS::pad, b, c);
    });
    __syncwarp();
    // the element matrix, slab after slab, with 16-byte stores (slab sizes are multiples of 4 floats)
    static_assert(CS::size % 4 == 0, "slabs of whole float4");
    float4* dst = reinterpret_cast<float4*>(em + NG_IDX(e, nCells, 71) * (ND * CS::size));
    for (int i = lane; i < ND * CS::size / 4; i += 32)
    {
        const int a = i / (CS::size / 4), j = i % (CS::size / 4);
        dst[i] = *reinterpret_cast<const float4*>(sEM + a * CS::pad + 4 * j);
    }
}

template <int DIM, int ND, int NIP, int KIND, int W>
__global__ void __launch_bounds__(W * 32) k_rows_from_cells(FusedArgs A, const float* __restrict__ em,
                                                            float* __restrict__ vals)
{
    using CS = CellSlab<DIM, ND, KIND>;
    constexpr bool GD = CS::GD;
    constexpr int NR = CS::nr, NC = CS::nc, SL = CS::size;
    constexpr int PER = (SL + 31) / 32; // slab values per lane
    __shared__ float sRowAll[W][NR * kFusedRowCap];
    const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t a = A.nodeBase + static_cast<int64_t>(blockIdx.x) * W + wid;
    if (a >= A.nNodes)
        return; // the whole warp leaves; only warp-level synchronisation follows
    float* sRow = sRowAll[wid];
    int64_t rs[NR];
    int len[NR];
    const int64_t g0 = A.gdofD[a];
#pragma unroll
    for (int k = 0; k < DIM; ++k)
    {
        rs[k] = A.rowPtr[NG_IDX(g0 + k, A.nRows, 72)];
        len[k] = static_cast<int>(A.rowPtr[g0 + k + 1] - rs[k]);
    }
    int32_t ae = 0;
    if (GD)
    {
        ae = A.eOf[a];
        const int64_t ge = A.gdofE[ae];
        rs[DIM] = A.rowPtr[NG_IDX(ge, A.nRows, 72)];
        len[DIM] = static_cast<int>(A.rowPtr[ge + 1] - rs[DIM]);
    }
    const int32_t bUU = A.blk[0][a];
    const int32_t bUE = GD ? A.blk[1][a] : 0;
    const int32_t bEU = GD ? A.blk[2][ae] : 0;
    const int32_t bEE = GD ? A.blk[3][ae] : 0;
#pragma unroll
    for (int k = 0; k < NR; ++k)
        for (int i = lane; i < kFusedRowCap; i += 32)
            sRow[k * kFusedRowCap + i] = 0.f;
    const int64_t n = A.nCells;
    const int64_t k0 = A.cellPtr[a], k1 = A.cellPtr[a + 1];
    // the slab values of the next cell are loaded while the current one is added
    float nxt[PER];
    auto load = [&](int64_t kc, float (&v)[PER]) {
        const int64_t e = A.cellIdx[kc];
        const int ia = A.cellLoc[kc];
        const float* slab = em + (NG_IDX(e, n, 73) * ND + ia) * SL;
#pragma unroll
        for (int m = 0; m < PER; ++m)
        {
            const int i = lane + 32 * m;
            v[m] = i < SL ? slab[i] : 0.f;
        }
    };
    if (k0 < k1)
        load(k0, nxt);
    for (int64_t kc = k0; kc < k1; ++kc)
    {
        float cur[PER];
#pragma unroll
        for (int m = 0; m < PER; ++m)
            cur[m] = nxt[m];
        const int64_t e = A.cellIdx[kc];
        const int ia = A.cellLoc[kc];
        // ranks of b in a's neighbour lists: lane b loads them, the others read them by shuffles
        int r0 = 0, r1 = 0, r2 = 0, r3 = 0;
        if (lane < ND)
        {
            const int64_t ridx = static_cast<int64_t>(ia * ND + lane) * n + e;
            r0 = A.rank[0][ridx];
            if (GD)
            {
                r1 = A.rank[1][ridx];
                r2 = A.rank[2][ridx];
                r3 = A.rank[3][ridx];
            }
        }
        if (kc + 1 < k1)
            load(kc + 1, nxt);
#pragma unroll
        for (int m = 0; m < PER; ++m)
        {
            const int i = lane + 32 * m;
            const int ic = i < SL ? i : 0;
            const int row = ic / NC, col = ic % NC;
            const bool ucol = col < ND * DIM;
            const int b = ucol ? col / DIM : col - ND * DIM;
            const int l = ucol ? col % DIM : 0;
            const int rk0 = __shfl_sync(0xffffffffu, r0, b);
            int pos;
            if (GD)
            {
                const int rk1 = __shfl_sync(0xffffffffu, r1, b);
                const int rk2 = __shfl_sync(0xffffffffu, r2, b);
                const int rk3 = __shfl_sync(0xffffffffu, r3, b);
                if (row < DIM)
                    pos = ucol ? bUU + DIM * rk0 + l : bUE + rk1;
                else
                    pos = ucol ? bEU + DIM * rk2 + l : bEE + rk3;
            }
            else
                pos = bUU + DIM * rk0 + l;
            if (i < SL)
                sRow[row * kFusedRowCap + NG_IDX(pos, kFusedRowCap, 74)] += cur[m];
        }
        __syncwarp();
    }
#pragma unroll
    for (int k = 0; k < NR; ++k)
        for (int i = lane; i < len[k]; i += 32)
            vals[NG_IDX(rs[k] + i, A.nnz, 75)] = sRow[k * kFusedRowCap + i];
}

// The element matrices with the law evaluated in the same kernel (no records in global memory): a warp takes
// CPW = 32 / NIP cells; (0) lane (cell, node) stages the node data, (A) lane (cell, point) evaluates PointData into
// the record layout in shared memory (the values k_point_records writes), (B) the cells one after the other as in
// k_cell_matrices. Bitwise the same element matrices as k_point_records + k_cell_matrices.
template <int DIM, int ND, int NIP, int KIND>
struct CellLawShape
{
    using Sh = FusedShape<DIM, ND, NIP, KIND, true>;
    using CS = CellSlab<DIM, ND, KIND>;
    static constexpr bool GD = Sh::GD;
    static constexpr int cpw = 32 / NIP;
    static constexpr int R4 = Sh::recF4;
    static constexpr int perCell = NIP * R4; // float4
    // per warp, in floats: node coordinates and displacements (2 float4 per (cell, node)), eeq in FP64 (2 floats),
    // the records of the warp's cells, P/Q per (point, node) of one cell, one element matrix
    static constexpr int nodeF = cpw * ND * 8;
    static constexpr int eF = GD ? cpw * ND * 2 : 0;
    static constexpr int recF = cpw * perCell * 4;
    static constexpr int pqF = GD ? NIP * ND * 8 : 0;
    static constexpr int emF = 0; // the element matrix is stored from registers
    static constexpr int perWarp = nodeF + eF + recF + pqF + emF;
    static constexpr int tabF = NIP * ND * 4 + (NIP + 3) / 4 * 4; // (dN/dxi, N) per point and node, weights
    static constexpr size_t smem(int W)
    {
        return (static_cast<size_t>(W) * perWarp + tabF) * sizeof(float);
    }
    static_assert(cpw * ND == 32 && cpw * NIP == 32, "one lane per (cell, node) and per (cell, point)");
    static_assert(nodeF % 4 == 0 && eF % 4 == 0 && recF % 4 == 0 && pqF % 4 == 0 && emF % 4 == 0, "16-byte regions");
};

template <int DIM, int ND, int NIP, int KIND, int W>
__global__ void __launch_bounds__(W * 32) k_cell_matrices_law(FusedArgs A, LawParams L, const double* __restrict__ u,
                                                              float* __restrict__ em)
{
    using LS = CellLawShape<DIM, ND, NIP, KIND>;
    using CS = CellSlab<DIM, ND, KIND>;
    constexpr bool GD = LS::GD;
    constexpr int CPW = LS::cpw, R4 = LS::R4, PER_CELL = LS::perCell;
    extern __shared__ __align__(16) float smL[];
    const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
    float4* sT = reinterpret_cast<float4*>(smL); // [NIP][ND]
    float* sWq = smL + NIP * ND * 4;             // [NIP]
    float* base = smL + LS::tabF + wid * LS::perWarp;
    float4* sX = reinterpret_cast<float4*>(base);                  // [CPW][ND]
    float4* sU = sX + CPW * ND;                                    // [CPW][ND]
    double* sE = reinterpret_cast<double*>(base + LS::nodeF);      // [CPW][ND]
    float4* sR = reinterpret_cast<float4*>(base + LS::nodeF + LS::eF); // [CPW][NIP][R4]
    float4* sPQ = reinterpret_cast<float4*>(base + LS::nodeF + LS::eF + LS::recF); // [NIP][ND][2]
    for (int i = threadIdx.x; i < NIP * ND; i += blockDim.x)
    {
        const int q = i / ND, nd = i % ND;
        const double* d = A.tabDN + (q * ND + nd) * 3;
        sT[i] = F4(static_cast<float>(d[0]), static_cast<float>(d[1]), DIM == 3 ? static_cast<float>(d[2]) : 0.f,
                   static_cast<float>(A.tabN[q * ND + nd]));
    }
    for (int i = threadIdx.x; i < NIP; i += blockDim.x)
        sWq[i] = static_cast<float>(A.tabW[i]);
    __syncthreads();
    const int64_t n = A.nCells;
    const int64_t c0 = (static_cast<int64_t>(blockIdx.x) * W + wid) * CPW;
    if (c0 >= n)
        return; // the whole warp leaves; only warp-level synchronisation follows
    // (0) lane (cell slot, node): the node data, as k_point_records loads them
    {
        const int cl = lane / ND, nd = lane % ND;
        const int64_t e = c0 + cl;
        if (e < n)
        {
            const int32_t nD = static_cast<int32_t>(NG_IDX(A.connD[static_cast<int64_t>(nd) * n + e], A.nNodesD, 80));
            const int64_t gd = A.gdofD[nD];
            float x[3] = {0.f, 0.f, 0.f}, v[3] = {0.f, 0.f, 0.f};
#pragma unroll
            for (int d = 0; d < DIM; ++d)
            {
                x[d] = A.relX[(static_cast<int64_t>(nd) * DIM + d) * n + e];
                v[d] = static_cast<float>(u[NG_IDX(gd + d, A.nDofs, 81)]);
            }
            float ev = 0.f;
            if (GD)
            {
                const int32_t nE =
                        static_cast<int32_t>(NG_IDX(A.connE[static_cast<int64_t>(nd) * n + e], A.nNodesE, 82));
                const double e64 = u[NG_IDX(A.gdofE[nE], A.nDofs, 83)];
                sE[cl * ND + nd] = e64;
                ev = static_cast<float>(e64);
            }
            sX[cl * ND + nd] = F4(x[0], x[1], x[2], ev);
            sU[cl * ND + nd] = F4(v[0], v[1], v[2], 0.f);
        }
    }
    __syncwarp();
    // (A) lane (cell slot, point): the law, written in the record layout
    {
        const int cl = lane / NIP, q = lane % NIP;
        const int64_t e = c0 + cl;
        if (e < n)
        {
            PointOut<DIM, ND> o;
            PointData<DIM, ND, NIP, KIND>(A, L, sT + q * ND, sWq[q], sX + cl * ND, sU + cl * ND,
                                          GD ? sE + cl * ND : nullptr, q, e, o);
            float4* r = sR + cl * PER_CELL + q * R4;
#pragma unroll
            for (int nd = 0; nd < ND; ++nd)
                r[nd] = F4(o.g[nd][0], o.g[nd][1], DIM == 3 ? o.g[nd][DIM - 1] : 0.f, sT[q * ND + nd].w);
            r[ND] = F4(o.s0[0], o.s0[1], o.s0[2], o.s0[3]);
            if (GD)
            {
                r[ND + 1] = F4(o.scge[0], o.scge[1], DIM == 3 ? o.scge[DIM - 1] : 0.f, o.sv[4]);
                r[ND + 2] = F4(o.tv[0], o.tv[1], o.tv[2], o.sv[5]);
                r[ND + 3] = F4(o.tv[3], o.tv[4], o.tv[5], 0.f);
                r[ND + 4] = F4(o.sv[0], o.sv[1], o.sv[2], o.sv[3]);
            }
        }
    }
    __syncwarp();
    // (B) the element matrices of the warp's cells, one after the other
    for (int cl = 0; cl < CPW; ++cl)
    {
        const int64_t e = c0 + cl;
        if (e >= n)
            break;
        const float4* rec = sR + cl * PER_CELL;
        if (GD)
        {
            for (int it = lane; it < NIP * ND; it += 32)
            {
                const int q = it / ND, nd = it % ND;
                const float4* row = rec + q * R4;
                const float4 g = row[nd];
                const float4* S = row + ND;
                const float4 s1 = S[1], s2 = S[2], s3 = S[3], s4 = S[4];
                const float sv[6] = {s4.x, s4.y, s4.z, s4.w, s1.w, s2.w};
                const float tv[6] = {s2.x, s2.y, s2.z, s3.x, s3.y, s3.z};
                const float3 pa = BtV<DIM>(g.x, g.y, g.z, sv);
                const float gs = DotG<DIM>(g.x, g.y, g.z, s1.x, s1.y, s1.z);
                const float3 qb = BtV<DIM>(g.x, g.y, g.z, tv);
                sPQ[(q * ND + nd) * 2] = F4(pa.x, pa.y, pa.z, gs);
                sPQ[(q * ND + nd) * 2 + 1] = F4(qb.x, qb.y, qb.z, 0.f);
            }
            __syncwarp();
        }
        // straight from registers to the cell's slab in global memory (a warp's stores of one (k, l) land in four
        // slab rows of the cell's matrix; L2 merges them into whole sectors before writing back)
        float* cellEm = em + NG_IDX(e, n, 84) * (ND * CS::size);
        CellPairs<DIM, ND, NIP, GD>(rec, R4, sPQ, lane, [&](int ia, int b, const PairAcc<DIM>& c) {
            PutBlock<DIM, ND, GD, CS::nc>(cellEm + ia * CS::size, b, c);
        });
        __syncwarp(); // sPQ is rewritten for the next cell
    }
}

// The ranks of one (cell entry of a node, neighbour b) packed into one word (UU | UE << 8 | EU << 16 | EE << 24), in
// the order of the nodes' cell lists: the row gather of a node then reads the ranks of its cells with contiguous
// loads instead of byte loads from the planar rank tables. Built once per mesh.
template <int ND>
__global__ void k_pack_ranks(FusedArgs A, int64_t nEntries, uint32_t* __restrict__ packed)
{
    const int64_t it = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
    if (it >= nEntries * ND)
        return;
    const int64_t kc = it / ND;
    const int b = static_cast<int>(it % ND);
    const int64_t e = A.cellIdx[kc];
    const int ia = A.cellLoc[kc];
    const int64_t ridx = static_cast<int64_t>(ia * ND + b) * A.nCells + e;
    packed[it] = static_cast<uint32_t>(A.rank[0][ridx]) | static_cast<uint32_t>(A.rank[1][ridx]) << 8 |
                 static_cast<uint32_t>(A.rank[2][ridx]) << 16 | static_cast<uint32_t>(A.rank[3][ridx]) << 24;
}

// Row gather of the element-matrix form for slabs of exactly 32 columns (Hex8 gradient damage: 24 displacement
// columns, 8 eeq columns): lane l owns column l of every slab row, so its neighbour b = l / 3 (or l - 24), and the
// positions in the displacement rows and in the eeq row are fixed per cell. The slab values and packed ranks of a
// batch of CB cells are loaded before any is added (all loads in flight at once); cells are added in ascending
// order.
template <int DIM, int ND, int NIP, int KIND, int W, int CB>
__global__ void __launch_bounds__(W * 32) k_rows_from_cells32(FusedArgs A, const uint32_t* __restrict__ packed,
                                                              const float* __restrict__ em, float* __restrict__ vals)
{
    using CS = CellSlab<DIM, ND, KIND>;
    constexpr bool GD = CS::GD;
    constexpr int NR = CS::nr, SL = CS::size;
    static_assert(CS::nc == 32 && ND == 8, "one slab column per lane, 8 nodes per cell");
    static_assert(CB == 2 || CB == 4 || CB == 8, "cells per batch");
    __shared__ float sRowAll[W][NR * kFusedRowCap];
    const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t a = A.nodeBase + static_cast<int64_t>(blockIdx.x) * W + wid;
    if (a >= A.nNodes)
        return; // the whole warp leaves; only warp-level synchronisation follows
    float* sRow = sRowAll[wid];
    int64_t rs[NR];
    int len[NR];
    const int64_t g0 = A.gdofD[a];
#pragma unroll
    for (int k = 0; k < DIM; ++k)
    {
        rs[k] = A.rowPtr[NG_IDX(g0 + k, A.nRows, 76)];
        len[k] = static_cast<int>(A.rowPtr[g0 + k + 1] - rs[k]);
    }
    int32_t ae = 0;
    if (GD)
    {
        ae = A.eOf[a];
        const int64_t ge = A.gdofE[ae];
        rs[DIM] = A.rowPtr[NG_IDX(ge, A.nRows, 76)];
        len[DIM] = static_cast<int>(A.rowPtr[ge + 1] - rs[DIM]);
    }
    const int32_t bUU = A.blk[0][a];
    const int32_t bUE = GD ? A.blk[1][a] : 0;
    const int32_t bEU = GD ? A.blk[2][ae] : 0;
    const int32_t bEE = GD ? A.blk[3][ae] : 0;
#pragma unroll
    for (int k = 0; k < NR; ++k)
        for (int i = lane; i < kFusedRowCap; i += 32)
            sRow[k * kFusedRowCap + i] = 0.f;
    const bool ucol = lane < ND * DIM;
    const int myB = ucol ? lane / DIM : lane - ND * DIM;
    const int myL = ucol ? lane % DIM : 0;
    const int64_t n = A.nCells; // extent of the checked indices
    (void)n;
    const int64_t k0 = A.cellPtr[a], k1 = A.cellPtr[a + 1];
    for (int64_t kb = k0; kb < k1; kb += CB)
    {
        const int nc = static_cast<int>(k1 - kb < CB ? k1 - kb : CB);
        // packed ranks of the batch: lane l holds (cell slot l / 8, b = l % 8) and (cell slot 4 + l / 8, b)
        uint32_t pk0 = 0, pk1 = 0;
        if (lane / ND < nc)
            pk0 = packed[NG_IDX((kb + lane / ND) * ND + lane % ND, n * ND * ND, 77)];
        if (CB == 8 && 4 + lane / ND < nc)
            pk1 = packed[NG_IDX((kb + 4 + lane / ND) * ND + lane % ND, n * ND * ND, 77)];
        float v[CB][NR];
#pragma unroll
        for (int c = 0; c < CB; ++c)
        {
            if (c < nc)
            {
                const int64_t kc = kb + c;
                const float* slab = em + (NG_IDX(A.cellIdx[kc], n, 78) * ND + A.cellLoc[kc]) * SL;
#pragma unroll
                for (int r = 0; r < NR; ++r)
                    v[c][r] = slab[r * 32 + lane];
            }
        }
#pragma unroll
        for (int c = 0; c < CB; ++c)
        {
            // all lanes take part in the shuffle; cells beyond the batch add nothing
            const uint32_t w = __shfl_sync(0xffffffffu, c < 4 ? pk0 : pk1, (c & 3) * ND + myB);
            if (c < nc)
            {
                const int r0 = w & 0xff, r1 = (w >> 8) & 0xff, r2 = (w >> 16) & 0xff, r3 = w >> 24;
                const int posU = ucol ? bUU + DIM * r0 + myL : bUE + r1;
#pragma unroll
                for (int k = 0; k < DIM; ++k)
                    sRow[k * kFusedRowCap + NG_IDX(posU, kFusedRowCap, 79)] += v[c][k];
                if (GD)
                {
                    const int posE = ucol ? bEU + DIM * r2 + myL : bEE + r3;
                    sRow[DIM * kFusedRowCap + NG_IDX(posE, kFusedRowCap, 79)] += v[c][DIM];
                }
            }
            __syncwarp();
        }
    }
#pragma unroll
    for (int k = 0; k < NR; ++k)
        for (int i = lane; i < len[k]; i += 32)
            vals[NG_IDX(rs[k] + i, A.nnz, 75)] = sRow[k * kFusedRowCap + i];
}

} // namespace

// FP32 coordinates of every cell's nodes relative to its first node (planar [(n * dim + d)][cell]), formed in FP64
// on the host once per mesh: the Jacobian of the fused tangent then sees differences of the size of the cell
// instead of FP32 absolute coordinates
void BuildRelativeCoordinates(Ctx& c)
{
    const int nge = c.nge, dim = c.dim;
    std::vector<float> rel(static_cast<size_t>(nge) * dim * c.nCells);
    for (int64_t e = 0; e < c.nCells; ++e)
    {
        const int32_t* cn = &c.hGeoConn[static_cast<size_t>(e) * nge];
        for (int nd = 0; nd < nge; ++nd)
            for (int d = 0; d < dim; ++d)
                rel[(static_cast<size_t>(nd) * dim + d) * c.nCells + e] = static_cast<float>(
                        c.hCoords[static_cast<size_t>(cn[nd]) * dim + d] - c.hCoords[static_cast<size_t>(cn[0]) * dim + d]);
    }
    c.dRelX.alloc(rel.size());
    NG_CUDA(cudaMemcpy(c.dRelX.p, rel.data(), rel.size() * sizeof(float), cudaMemcpyHostToDevice));
}

bool FusedTangentSupported(Ctx& c)
{
    if (c.fusedMode >= 0)
        return c.fusedMode == 1;
    c.fusedMode = 0;
    const Slot& D = c.slots[c.prm.disp_slot];
    const bool gd = c.prm.kind == NUTO_GPU_GRADIENT_DAMAGE;
    // linear cells whose coordinate and displacement elements coincide, LinearElastic or GradientDamage with FULL
    // damage application (UNILATERAL switches the volumetric damage on the sign of the volumetric strain, a branch
    // that FP32 cannot decide like FP64 near zero), 2x2 / 2x2x2 Gauss points
    const bool cells = (c.dim == 2 && c.nge == 4 && D.nen == 4 && c.ip.nIp == 4) ||
                       (c.dim == 3 && c.nge == 8 && D.nen == 8 && c.ip.nIp == 8);
    const bool law = c.prm.kind == NUTO_GPU_MB_LINEAR_ELASTIC ||
                     (gd && c.prm.damage_application == NUTO_GPU_DAMAGE_FULL);
    if (!cells || !law)
        return false;
    // every row of a displacement node (and of its eeq node) fits the row buffer
    const int eS = gd ? c.prm.eeq_slot : c.prm.disp_slot;
    for (int s : {c.prm.disp_slot, eS})
    {
        const Slot& S = c.slots[s];
        for (int64_t i = 0; i < S.nNodes; ++i)
            for (int k = 0; k < S.ncomp; ++k)
            {
                const int64_t r = S.offset + S.dof0[i] + k;
                if (c.hRowPtr[r + 1] - c.hRowPtr[r] > kFusedRowCap)
                    return false;
            }
    }
    c.fusedMode = 1;
    return true;
}

void LaunchTangentFused(Ctx& c, const double* u, float* vals)
{
    if (c.dRelX.n == 0)
        BuildRelativeCoordinates(c);
    const int ns = static_cast<int>(c.slots.size());
    const int dS = c.prm.disp_slot;
    const bool gd = c.prm.kind == NUTO_GPU_GRADIENT_DAMAGE;
    const int eS = gd ? c.prm.eeq_slot : dS;
    const Slot& D = c.slots[dS];
    FusedArgs A{};
    A.nNodes = D.nNodes;
    A.nCells = c.nCells;
    A.nnz = c.nnz;
    A.nRows = c.nDofs;
    A.nDofs = c.nDofs;
    A.nNodesD = D.nNodes;
    A.nNodesE = c.slots[eS].nNodes;
    A.connD = D.dConnT.p;
    A.connE = c.slots[eS].dConnT.p;
    A.gdofD = D.dGdof.p;
    A.gdofE = c.slots[eS].dGdof.p;
    A.eOf = gd ? c.dEOf.p : nullptr;
    A.relX = c.dRelX.p;
    A.kappa = c.dKappa.p;
    A.escale = c.dEScale.n ? c.dEScale.p : nullptr;
    A.tabN = c.dTables.p + c.tabN[D.interp];
    A.tabDN = c.dTables.p + c.tabDN[D.interp];
    A.tabW = c.dTables.p + c.tabW;
    A.cellPtr = D.dCellPtr.p;
    A.cellIdx = D.dCellIdx.p;
    A.cellLoc = D.dCellLoc.p;
    A.rowPtr = c.dRowPtr.p;
    const int pr[4] = {dS * ns + dS, dS * ns + eS, eS * ns + dS, eS * ns + eS};
    for (int k = 0; k < 4; ++k)
    {
        A.rank[k] = c.pairs[pr[k]].rank;
        A.blk[k] = c.pairs[pr[k]].dBlk.p;
    }
    const bool staged = c.tangentStaged;
    // one assembly with W warps per block; form 0: the node-row kernel, 1: the double-buffered node-row kernel on a
    // grid of resident blocks, 2: element matrices + row gather (1 and 2 with staged records only)
    auto assemble = [&](int W, int form) {
        auto run = [&](auto cfg) {
            using C = decltype(cfg);
            constexpr int DIM = C::dim, ND = C::nd, NIP = C::nip, KIND = C::kind;
            float4* recs = nullptr;
            if (staged && !(form == 2 && c.cellsLawFused))
            {
                const size_t bytes =
                        static_cast<size_t>(c.nCells) * NIP * FusedShape<DIM, ND, NIP, KIND, true>::recF4 * 16;
                if (c.dRecords.n < bytes)
                    c.dRecords.alloc(bytes);
                recs = reinterpret_cast<float4*>(c.dRecords.p);
                k_point_records<DIM, ND, NIP, KIND>
                        <<<static_cast<unsigned>((c.nCells + 128 / NIP - 1) / (128 / NIP)), 128, 0, c.stream>>>(
                                A, c.law, u, recs);
                AfterLaunch(c, "k_point_records");
                c.stats.kernel_launches += 1;
            }
            auto rows = [&](auto w) {
                constexpr int WW = decltype(w)::value;
                if (staged && form == 2)
                {
                    using CS = CellSlab<DIM, ND, KIND>;
                    const size_t emFloats = static_cast<size_t>(c.nCells) * ND * CS::size;
                    if (c.dElemMats.n < emFloats)
                        c.dElemMats.alloc(emFloats);
                    if (c.cellsLawFused)
                    {
                        using LS = CellLawShape<DIM, ND, NIP, KIND>;
                        const size_t smem = LS::smem(WW);
                        auto kern = k_cell_matrices_law<DIM, ND, NIP, KIND, WW>;
                        if (smem > 48 * 1024)
                            NG_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                         static_cast<int>(smem)));
                        const int64_t cellsPerBlock = static_cast<int64_t>(WW) * LS::cpw;
                        kern<<<static_cast<unsigned>((c.nCells + cellsPerBlock - 1) / cellsPerBlock), WW * 32, smem,
                               c.stream>>>(A, c.law, u, c.dElemMats.p);
                        AfterLaunch(c, "k_cell_matrices_law");
                    }
                    else
                    {
                        constexpr int recF = NIP * FusedShape<DIM, ND, NIP, KIND, true>::recF4 * 4;
                        constexpr int pqF = CS::GD ? NIP * ND * 8 : 0;
                        constexpr size_t smem = static_cast<size_t>(WW) * (recF + pqF + ND * CS::pad) * sizeof(float);
                        auto kern = k_cell_matrices<DIM, ND, NIP, KIND, WW>;
                        if (smem > 48 * 1024)
                            NG_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                         static_cast<int>(smem)));
                        kern<<<static_cast<unsigned>((c.nCells + WW - 1) / WW), WW * 32, smem, c.stream>>>(
                                c.nCells, recs, c.dElemMats.p);
                        AfterLaunch(c, "k_cell_matrices");
                    }
                    if constexpr (CS::nc == 32 && ND == 8)
                    {
                        // packed ranks in cell-list order, once per mesh
                        const int64_t entries = static_cast<int64_t>(c.nCells) * ND;
                        if (c.dPackedRanks.n != static_cast<size_t>(entries * ND))
                        {
                            c.dPackedRanks.alloc(static_cast<size_t>(entries * ND));
                            k_pack_ranks<ND><<<static_cast<unsigned>((entries * ND + 255) / 256), 256, 0, c.stream>>>(
                                    A, entries, c.dPackedRanks.p);
                            AfterLaunch(c, "k_pack_ranks");
                        }
                    }
                    // the row gather, in node chunks when a caller hooks into them (each chunk's rows are complete
                    // when its launch is)
                    const int chunks = c.rowChunks > 1 && c.onRowChunk ? c.rowChunks : 1;
                    for (int ch = 0; ch < chunks; ++ch)
                    {
                        FusedArgs Ac = A;
                        Ac.nodeBase = A.nNodes * ch / chunks;
                        Ac.nNodes = A.nNodes * (ch + 1) / chunks;
                        const int64_t nodes = Ac.nNodes - Ac.nodeBase;
                        const unsigned rowBlocks = static_cast<unsigned>((nodes + WW - 1) / WW);
                        if (rowBlocks > 0)
                        {
                            if constexpr (CS::nc == 32 && ND == 8)
                            {
                                // 4 cells per batch: 64 registers, 32 resident warps per SM (8 cells: 86 registers,
                                // 1.14x slower; 2 cells: 1.02x slower, measured at 64^3)
                                k_rows_from_cells32<DIM, ND, NIP, KIND, WW, 4><<<rowBlocks, WW * 32, 0, c.stream>>>(
                                        Ac, c.dPackedRanks.p, c.dElemMats.p, vals);
                                AfterLaunch(c, "k_rows_from_cells32");
                            }
                            else
                            {
                                k_rows_from_cells<DIM, ND, NIP, KIND, WW><<<rowBlocks, WW * 32, 0, c.stream>>>(
                                        Ac, c.dElemMats.p, vals);
                                AfterLaunch(c, "k_rows_from_cells");
                            }
                            c.stats.kernel_launches += 1;
                        }
                        if (chunks > 1)
                        {
                            c.onRowChunk(Ac.nodeBase, Ac.nNodes);
                            c.rowChunksDone++;
                        }
                    }
                    c.stats.kernel_launches += 1;
                    return;
                }
                if (staged && form == 1)
                {
                    auto kern = k_tangent_rows_pipe<DIM, ND, NIP, KIND, WW>;
                    using Sh = FusedShape<DIM, ND, NIP, KIND, true, WW>;
                    constexpr size_t smem =
                            static_cast<size_t>(WW) * (2 * Sh::cpp * NIP * Sh::recF4 * 16 + Sh::nr * kFusedRowCap * 4);
                    if (smem > 48 * 1024)
                        NG_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                     static_cast<int>(smem)));
                    int perSm = 0;
                    NG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSm, kern, WW * 32, smem));
                    const int64_t need = (A.nNodes + WW - 1) / WW;
                    const unsigned blocks = static_cast<unsigned>(
                            std::max<int64_t>(1, std::min<int64_t>(need, static_cast<int64_t>(perSm) * c.smCount)));
                    kern<<<blocks, WW * 32, smem, c.stream>>>(A, recs, vals);
                    AfterLaunch(c, "k_tangent_rows_pipe");
                    c.stats.kernel_launches += 1;
                    return;
                }
                const unsigned blocks = static_cast<unsigned>((A.nNodes + WW - 1) / WW);
                auto launch = [&](auto kern, size_t smem) {
                    if (smem > 48 * 1024)
                        NG_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                     static_cast<int>(smem)));
                    kern<<<blocks, WW * 32, smem, c.stream>>>(A, c.law, u, recs, vals);
                };
                if (staged)
                    launch(k_tangent_fused<DIM, ND, NIP, KIND, true, WW>,
                           FusedShape<DIM, ND, NIP, KIND, true, WW>::smem);
                else
                    launch(k_tangent_fused<DIM, ND, NIP, KIND, false, WW>,
                           FusedShape<DIM, ND, NIP, KIND, false, WW>::smem);
                AfterLaunch(c, "k_tangent_fused");
                c.stats.kernel_launches += 1;
            };
            if (W == 2)
                rows(std::integral_constant<int, 2>{});
            else if (W == 8)
                rows(std::integral_constant<int, 8>{});
            else
                rows(std::integral_constant<int, 4>{});
        };
        if (c.dim == 3 && gd)
            run(FCfg<3, 8, 8, NUTO_GPU_GRADIENT_DAMAGE>{});
        else if (c.dim == 3)
            run(FCfg<3, 8, 8, NUTO_GPU_MB_LINEAR_ELASTIC>{});
        else if (gd)
            run(FCfg<2, 4, 4, NUTO_GPU_GRADIENT_DAMAGE>{});
        else
            run(FCfg<2, 4, 4, NUTO_GPU_MB_LINEAR_ELASTIC>{});
    };
    // autotuner: the first FP32 tangent of a context (outside any stream capture) assembles once with each candidate
    // shape — 2, 4 and 8 warps per block, and with staged records also the double-buffered kernel and the
    // element-matrix form with 2 and 4 warps per block — (a warm-up and a timed assembly each; every one writes the
    // same values) and keeps the fastest
    Tuning& T = c.tuning;
    if (T.tangentWarps == 0)
    {
        cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
        NG_CUDA(cudaStreamIsCapturing(c.stream, &cs));
        if (!T.enabled)
            T.tangentWarps = 4;
        else if (cs == cudaStreamCaptureStatusNone)
        {
            const int candW[7] = {2, 4, 8, 2, 4, 2, 4};
            const int candForm[7] = {0, 0, 0, 1, 1, 2, 2};
            const int nCand = staged ? 7 : 3;
            cudaEvent_t e0, e1;
            NG_CUDA(cudaEventCreate(&e0));
            NG_CUDA(cudaEventCreate(&e1));
            float best = 0.f;
            int pick = 1;
            for (int k = 0; k < nCand; ++k)
            {
                assemble(candW[k], candForm[k]);
                NG_CUDA(cudaEventRecord(e0, c.stream));
                assemble(candW[k], candForm[k]);
                NG_CUDA(cudaEventRecord(e1, c.stream));
                NG_CUDA(cudaEventSynchronize(e1));
                float ms = 0.f;
                NG_CUDA(cudaEventElapsedTime(&ms, e0, e1));
                T.tangentMs[k] = ms;
                if (k == 0 || ms < best)
                {
                    best = ms;
                    pick = k;
                }
            }
            cudaEventDestroy(e0);
            cudaEventDestroy(e1);
            T.tangentWarps = candW[pick];
            T.tangentForm = candForm[pick];
        }
    }
    assemble(T.tangentWarps ? T.tangentWarps : 4, staged ? T.tangentForm : 0);
}

} // namespace nuto_gpu
