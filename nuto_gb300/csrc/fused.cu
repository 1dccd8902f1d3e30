// Fused FP32 tangent: SimpleAssembler::BuildMatrix (nuto/mechanics/cell/SimpleAssembler.cpp:100-156) of
// MomentumBalance::Hessian0 (nuto/mechanics/integrands/MomentumBalance.h:36-46) and GradientDamage::Hessian0
// (nuto/mechanics/integrands/GradientDamage.h:92-120) for linear cells (Quad4, Hex8), written straight into the CSR
// values without integration-point records in HBM and without atomics in global memory.
//
// One warp per displacement node a assembles the complete CSR rows of a (and of its eeq node). The cells around a
// are taken a pass of CPP = 32 / NIP at a time:
//   (0) lane (cell, node) loads that node's data of the cell: FP32 coordinates relative to the cell's first node,
//       displacements, eeq value;
//   (A) lane (cell, integration point) computes J, J^-1, dN/dX, the strain, the law in FP32 and the products
//       B_n^T t of every node of the cell, into the warp's shared memory;
//   (B) lane (cell, neighbour b) integrates the node-pair block (a, b) over the points in registers and adds it into
//       the warp's shared copy of a's rows at the rank of b.
// At the end the rows are stored once, coalesced. Geometry and law are recomputed by each of the (up to) 8 warps
// that share a cell instead of being streamed from HBM: the kernel reads the connectivity, the relative
// coordinates, the state and the history and writes the values.
//
// Branch decisions of the law are the FP64 kernels' (k_residual, k_tangent<double>): the nonlocal equivalent
// strain at a point is formed in FP32 with an error bound, and where the bound does not separate it from the
// history kappa or from kappa0 it is recomputed in FP64 exactly as the FP64 kernels form it. The loading/unloading
// and damage-threshold branches therefore agree with the FP64 residual at every point; everything else is FP32.
#include "internal.cuh"

namespace nuto_gpu
{

namespace
{

constexpr int kFusedRowCap = 128; // values per row buffer: 32 neighbour nodes of [u | eeq] in 3D
constexpr int kFusedWarps = 4;

struct FusedArgs
{
    int64_t nNodes, nCells, nnz, nRows, nDofs, nNodesD, nNodesE;
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
struct FusedShape
{
    static constexpr bool GD = KIND == NUTO_GPU_GRADIENT_DAMAGE;
    static constexpr int cpp = 32 / NIP;             // cells per pass
    static constexpr int nr = DIM + (GD ? 1 : 0);     // rows per node
    // per warp, in floats: node data (2 float4 per (cell, node)), eeq values in FP64 (2 floats each), per point
    // the node gradients with N (float4 per node) and four float4 of scalars (lambda w, mu w, w, c g w | P_a, the
    // eeq-gradient coupling | the Voigt vector t of the (eeq, disp) block); the row buffer
    // rows of float4 indexed by the integration point are padded to ND + 1 (and the scalars to 5) float4 entries:
    // the 8 lanes of a cell, one per point, then touch 8 distinct bank groups instead of one (a stride of 128 bytes
    // would serialise them 8-fold)
    static constexpr int nodeF = cpp * ND * 8;
    static constexpr int eF = GD ? cpp * ND * 2 : 0;
    static constexpr int gF = cpp * NIP * (ND + 1) * 4;
    static constexpr int qF = 0;
    static constexpr int sF = cpp * NIP * 20; // 5 float4 per point: 4 used (scalars, P_a, t), 1 of padding
    static constexpr int rowF = nr * kFusedRowCap;
    static constexpr int perWarp = nodeF + eF + gF + qF + sF + rowF;
    static constexpr int tabF = NIP * (ND + 1) * 4 + NIP; // (dN/dxi, N) per point and node, weights
    static constexpr int tabOff = (tabF + 3) / 4 * 4; // per-warp regions start 16-byte aligned
    static constexpr size_t smem = (static_cast<size_t>(kFusedWarps) * perWarp + tabOff) * sizeof(float);
    static_assert(cpp * NIP == 32 && cpp * ND == 32, "one lane per (cell, point) and per (cell, node)");
};

__device__ __forceinline__ float4 F4(float x, float y, float z, float w)
{
    return make_float4(x, y, z, w);
}

// B_n^T v for the node gradient g (Voigt columns; 2D xx yy xy, 3D xx yy zz yz zx xy)
template <int DIM>
__device__ __forceinline__ float3 BtV(float gx, float gy, float gz, const float* v)
{
    if (DIM == 2)
        return make_float3(gx * v[0] + gy * v[2], gy * v[1] + gx * v[2], 0.f);
    return make_float3(gx * v[0] + gz * v[4] + gy * v[5], gy * v[1] + gz * v[3] + gx * v[5],
                       gz * v[2] + gy * v[3] + gx * v[4]);
}

template <int DIM, int ND, int NIP, int KIND>
__global__ void __launch_bounds__(kFusedWarps * 32)
        k_tangent_fused(FusedArgs A, LawParams L, const double* __restrict__ u, float* __restrict__ vals)
{
    using Sh = FusedShape<DIM, ND, NIP, KIND>;
    constexpr bool GD = Sh::GD;
    constexpr int CPP = Sh::cpp, NR = Sh::nr, VD = DIM == 2 ? 3 : 6;
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

    const int64_t a = static_cast<int64_t>(blockIdx.x) * kFusedWarps + wid;
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
                const float4* T = sTab + q * NDP;
                const float4* X = sNodeX + cs * ND;
                const float4* U = sNodeU + cs * ND;
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
                    const float c00 = J[1][1] * J[2][2] - J[1][2] * J[2][1];
                    const float c10 = J[1][2] * J[2][0] - J[1][0] * J[2][2];
                    const float c20 = J[1][0] * J[2][1] - J[1][1] * J[2][0];
                    det = J[0][0] * c00 + J[0][1] * c10 + J[0][2] * c20;
                    const float id = 1.f / det;
                    inv[0][0] = c00 * id;
                    inv[1][0] = c10 * id;
                    inv[2][0] = c20 * id;
                    inv[0][1] = (J[0][2] * J[2][1] - J[0][1] * J[2][2]) * id;
                    inv[1][1] = (J[0][0] * J[2][2] - J[0][2] * J[2][0]) * id;
                    inv[2][1] = (J[0][1] * J[2][0] - J[0][0] * J[2][1]) * id;
                    inv[0][2] = (J[0][1] * J[1][2] - J[0][2] * J[1][1]) * id;
                    inv[1][2] = (J[0][2] * J[1][0] - J[0][0] * J[1][2]) * id;
                    inv[2][2] = (J[0][0] * J[1][1] - J[0][1] * J[1][0]) * id;
                }
                const float wdj = sW[q] * det;
                // per-cell Young's modulus factor: scales the material tangent and dsigma/domega
                const float wdjE = A.escale ? wdj * static_cast<float>(A.escale[e]) : wdj;
                // node gradients dN/dX = J^-T dN/dxi, displacement gradient, eeq and its gradient
                float g[ND][DIM], H[DIM][DIM], ge[DIM];
                float eeq = 0.f, eabs = 0.f;
#pragma unroll
                for (int i = 0; i < DIM; ++i)
                {
                    ge[i] = 0.f;
#pragma unroll
                    for (int j = 0; j < DIM; ++j)
                        H[i][j] = 0.f;
                }
                float4* G = sG + (cs * NIP + q) * NDP;
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
                        g[nd][k] = s;
                    }
                    G[nd] = F4(g[nd][0], g[nd][1], DIM == 3 ? g[nd][DIM - 1] : 0.f, t.w);
                    const float4 uv = U[nd];
                    const float uc[3] = {uv.x, uv.y, uv.z};
#pragma unroll
                    for (int c = 0; c < DIM; ++c)
#pragma unroll
                        for (int d = 0; d < DIM; ++d)
                            H[c][d] += uc[c] * g[nd][d];
                    if (GD)
                    {
                        const float ev = X[nd].w;
                        eeq += t.w * ev;
                        eabs += fabsf(t.w * ev);
#pragma unroll
                        for (int d = 0; d < DIM; ++d)
                            ge[d] += ev * g[nd][d];
                    }
                }
                float eps[VD];
                if (DIM == 2)
                {
                    eps[0] = H[0][0];
                    eps[1] = H[1][1];
                    eps[2] = H[0][1] + H[1][0];
                }
                else
                {
                    eps[0] = H[0][0];
                    eps[1] = H[1][1];
                    eps[2] = H[DIM - 1][DIM - 1];
                    eps[3] = H[1][DIM - 1] + H[DIM - 1][1];
                    eps[4] = H[0][DIM - 1] + H[DIM - 1][0];
                    eps[5] = H[0][1] + H[1][0];
                }
                float gA[DIM]; // node a's gradient (local index ia)
#pragma unroll
                for (int d = 0; d < DIM; ++d)
                {
                    gA[d] = g[0][d];
#pragma unroll
                    for (int nd = 1; nd < ND; ++nd)
                        gA[d] = nd == ia ? g[nd][d] : gA[d];
                }
                float4* S = sS + (cs * NIP + q) * 5;
                if (!GD)
                {
                    // LinearElastic: C11 = lambda + 2 mu, C12 = lambda, C33 = mu
                    S[0] = F4(static_cast<float>(L.C12) * wdjE, static_cast<float>(L.C33) * wdjE, 0.f, 0.f);
                    S[1] = F4(0.f, 0.f, 0.f, 0.f);
                }
                else
                {
                    // branch decisions of the FP64 kernels: loading (eeq >= kappa_h) and damage (kappa >= kappa0),
                    // decided in FP32 where the error bound of eeq separates the operands, else in FP64 formed
                    // as k_tangent<double> forms eeq (same order, FP64 shape values)
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
                                s += A.tabN[q * ND + nd] * sE64[cs * ND + nd];
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
                    float dsdw[VD], dn[VD], sv[VD], tvv[VD];
                    LedDstressDomega<float, DIM>(L, eps, dsdw);
                    MisesDerivative<float, DIM>(L, eps, dn);
                    const float f1 = dOdK * dKdE * wdj;
                    const float f1E = dOdK * dKdE * wdjE;
#pragma unroll
                    for (int v = 0; v < VD; ++v)
                    {
                        sv[v] = dsdw[v] * f1E; // (disp, eeq): B^T (dsigma/domega w' k') N
                        tvv[v] = dn[v] * wdj; // (eeq, disp): -N^T (deps_eq/deps)^T B
                    }
                    const float c = static_cast<float>(L.c);
                    const float sc = c * dgdw * f1;
                    float gs = 0.f;
#pragma unroll
                    for (int d = 0; d < DIM; ++d)
                        gs += gA[d] * ge[d];
                    const float3 pa = BtV<DIM>(gA[0], gA[1], DIM == 3 ? gA[DIM - 1] : 0.f, sv);
                    S[0] = F4(lam * wdjE, mu * wdjE, wdj, c * gI * wdj);
                    S[1] = F4(pa.x, pa.y, pa.z, sc * gs);
                    S[2] = F4(tvv[0], tvv[1], tvv[2], 0.f);
                    S[3] = F4(VD > 3 ? tvv[VD > 3 ? 3 : 0] : 0.f, VD > 4 ? tvv[VD > 4 ? 4 : 0] : 0.f,
                              VD > 5 ? tvv[VD > 5 ? 5 : 0] : 0.f, 0.f);
                }
            }
        }
        __syncwarp();
        // (B) lane (cell slot, neighbour b): the node-pair block (a, b) integrated over the points, added into a's
        // rows at the ranks of b
        {
            const int cs = lane / ND, b = lane % ND;
            const int64_t kc = kp + cs;
            float uu[DIM][DIM], ue[DIM], eu[DIM], ee = 0.f, dg = 0.f;
#pragma unroll
            for (int k = 0; k < DIM; ++k)
            {
                ue[k] = eu[k] = 0.f;
#pragma unroll
                for (int l = 0; l < DIM; ++l)
                    uu[k][l] = 0.f;
            }
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
                    const float4* G = sG + (cs * NIP + q) * NDP;
                    const float4 ga = G[ia], gb = G[b];
                    const float4 s0 = sS[(cs * NIP + q) * 5];
                    const float av[3] = {ga.x, ga.y, ga.z}, bv[3] = {gb.x, gb.y, gb.z};
                    float gab = 0.f;
#pragma unroll
                    for (int d = 0; d < DIM; ++d)
                        gab += av[d] * bv[d];
                    // lambda w g_a g_b^T + mu w (g_b g_a^T + (g_a . g_b) I)
#pragma unroll
                    for (int k = 0; k < DIM; ++k)
                    {
                        const float lk = s0.x * av[k], mk = s0.y * bv[k];
#pragma unroll
                        for (int l = 0; l < DIM; ++l)
                            uu[k][l] += lk * bv[l] + mk * av[l];
                    }
                    dg += s0.y * gab;
                    if (GD)
                    {
                        const float4 s1 = sS[(cs * NIP + q) * 5 + 1];
                        const float4 t0 = sS[(cs * NIP + q) * 5 + 2], t1 = sS[(cs * NIP + q) * 5 + 3];
                        const float tv[6] = {t0.x, t0.y, t0.z, t1.x, t1.y, t1.z};
                        const float3 qb = BtV<DIM>(gb.x, gb.y, gb.z, tv); // B_b^T t
                        const float pv[3] = {s1.x, s1.y, s1.z}, qv[3] = {qb.x, qb.y, qb.z};
#pragma unroll
                        for (int k = 0; k < DIM; ++k)
                        {
                            ue[k] += pv[k] * gb.w;
                            eu[k] -= ga.w * qv[k];
                        }
                        ee += (s0.z * ga.w + s1.w) * gb.w + s0.w * gab;
                    }
                }
                active = true;
            }
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
    __syncwarp();
#pragma unroll
    for (int k = 0; k < NR; ++k)
        for (int i = lane; i < len[k]; i += 32)
            vals[NG_IDX(rs[k] + i, A.nnz, 57)] = sRow[k * kFusedRowCap + i];
}

} // namespace

// FP32 coordinates of every cell's nodes relative to its first node (planar [(n * dim + d)][cell]), formed in FP64
// on the host once per mesh: the Jacobian of the fused tangent then sees differences of the size of the cell
// instead of FP32 absolute coordinates
static void BuildRelativeCoordinates(Ctx& c)
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
    const unsigned blocks = static_cast<unsigned>((A.nNodes + kFusedWarps - 1) / kFusedWarps);
    auto launch = [&](auto kern, size_t smem) {
        if (smem > 48 * 1024)
            NG_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem)));
        kern<<<blocks, kFusedWarps * 32, smem, c.stream>>>(A, c.law, u, vals);
    };
    if (c.dim == 3 && gd)
        launch(k_tangent_fused<3, 8, 8, NUTO_GPU_GRADIENT_DAMAGE>, FusedShape<3, 8, 8, NUTO_GPU_GRADIENT_DAMAGE>::smem);
    else if (c.dim == 3)
        launch(k_tangent_fused<3, 8, 8, NUTO_GPU_MB_LINEAR_ELASTIC>, FusedShape<3, 8, 8, NUTO_GPU_MB_LINEAR_ELASTIC>::smem);
    else if (gd)
        launch(k_tangent_fused<2, 4, 4, NUTO_GPU_GRADIENT_DAMAGE>, FusedShape<2, 4, 4, NUTO_GPU_GRADIENT_DAMAGE>::smem);
    else
        launch(k_tangent_fused<2, 4, 4, NUTO_GPU_MB_LINEAR_ELASTIC>, FusedShape<2, 4, 4, NUTO_GPU_MB_LINEAR_ELASTIC>::smem);
    AfterLaunch(c, "k_tangent_fused");
    c.stats.kernel_launches += 1;
}

} // namespace nuto_gpu
