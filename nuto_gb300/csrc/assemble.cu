// Element kernels of the GB300 assembly path: integration-point geometry cache, FP64 internal-force residual,
// FP32/FP64 tangent scattered into CSR through the rank maps, history update, and the scatter of caller-given
// cell vectors/matrices.
//
// Work decomposition (all kernels): a CTA owns CPB consecutive cells and runs in phases separated by
// __syncthreads(): (0) gather the cells' DOF values into shared memory, (A) one thread per (cell, integration
// point) evaluates strain, law and integrand data, (B) one thread per (cell, node) or (cell, node pair)
// integrates over the points and scatters. Geometry (w * det J and dN/dX per integration point) is computed once
// per mesh and cached planar ([field][cell]) so that every per-cell load is coalesced.
#include "internal.cuh"

#include <algorithm>
#include <mutex>

namespace nuto_gpu
{

template <int DIM, int NG, int ND, int NIP, int KIND>
struct Cfg
{
    static constexpr int dim = DIM, ng = NG, nd = ND, nip = NIP, kind = KIND;
};

// Calls f(Cfg<...>{}) for the context's configuration (cell dimension, coordinate and displacement
// interpolation, integration points, integrand kind).
template <typename F>
static void DispatchCfg(const Ctx& c, F&& f)
{
    const int nd = c.slots[c.prm.disp_slot].nen;
    const int nip = c.ip.nIp;
    const int kind = c.prm.kind;
#define NG_CASE(D, G, N, Q, K)                                                                                   \
    if (c.dim == D && c.nge == G && nd == N && nip == Q && kind == K)                                            \
    {                                                                                                            \
        f(Cfg<D, G, N, Q, K>{});                                                                                 \
        return;                                                                                                  \
    }
#define NG_KINDS3(D, G, N, Q) NG_CASE(D, G, N, Q, 0) NG_CASE(D, G, N, Q, 1) NG_CASE(D, G, N, Q, 2)
#define NG_KINDS2(D, G, N, Q) NG_CASE(D, G, N, Q, 0) NG_CASE(D, G, N, Q, 1)
    NG_KINDS3(2, 4, 4, 4)
    NG_KINDS3(2, 4, 4, 9)
    NG_KINDS3(3, 8, 8, 8)
    NG_KINDS3(3, 8, 8, 27)
    NG_KINDS2(3, 8, 20, 8)
    NG_KINDS2(3, 8, 20, 27)
#undef NG_KINDS2
#undef NG_KINDS3
#undef NG_CASE
    throw Error{NUTO_GPU_EINVAL, "unsupported cell configuration (interpolation / integration points / integrand)"};
}

// ---- small device helpers -------------------------------------------------------------------------------

// LinearElastic stress sigma = C eps (LinearElastic.h:21-24, CalculateC :47-121)
template <typename T, int DIM>
__device__ __forceinline__ void ElasticStress(const LawParams& L, const T* e, T* s)
{
    const T c11 = T(L.C11), c12 = T(L.C12), c33 = T(L.C33);
    if (DIM == 2)
    {
        s[0] = c11 * e[0] + c12 * e[1];
        s[1] = c12 * e[0] + c11 * e[1];
        s[2] = c33 * e[2];
    }
    else
    {
        s[0] = c11 * e[0] + c12 * (e[1] + e[2]);
        s[1] = c11 * e[1] + c12 * (e[0] + e[2]);
        s[2] = c11 * e[2] + c12 * (e[0] + e[1]);
        s[3] = c33 * e[3];
        s[4] = c33 * e[4];
        s[5] = c33 * e[5];
    }
}

template <int A, int B>
struct MaxI
{
    static constexpr int v = A > B ? A : B;
};

// ---- integration-point geometry cache (Jacobian.h:16-48, CellIpData.h:108-113) -------------------------------
template <int DIM, int NG, int ND, int NIP>
__global__ void __launch_bounds__(128) k_geometry(int64_t nCells, int64_t nCoordValues, const double* __restrict__ coords,
                                                  const int32_t* __restrict__ geoConnT,
                                                  const double* __restrict__ tables, int tabW, int tabDNg,
                                                  int tabDNd, int stride, double* __restrict__ geo64,
                                                  float* __restrict__ geo32)
{
    const int64_t it = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
    if (it >= nCells * NIP)
        return;
    const int64_t e = it % nCells;
    const int q = static_cast<int>(it / nCells);
    double X[NG][DIM];
#pragma unroll
    for (int n = 0; n < NG; ++n)
    {
        const int32_t node = geoConnT[static_cast<int64_t>(n) * nCells + e];
#pragma unroll
        for (int d = 0; d < DIM; ++d)
            X[n][d] = coords[NG_IDX(static_cast<int64_t>(node) * DIM + d, nCoordValues, 1)];
    }
    const double* dNg = tables + tabDNg + q * NG * 3;
    double J[DIM][DIM];
#pragma unroll
    for (int i = 0; i < DIM; ++i)
#pragma unroll
        for (int j = 0; j < DIM; ++j)
        {
            double s = 0;
#pragma unroll
            for (int n = 0; n < NG; ++n)
                s += X[n][i] * dNg[n * 3 + j];
            J[i][j] = s;
        }
    double det, inv[DIM][DIM];
    if (DIM == 2)
    {
        det = J[0][0] * J[1][1] - J[0][1] * J[1][0];
        inv[0][0] = J[1][1] / det;
        inv[0][1] = -J[0][1] / det;
        inv[1][0] = -J[1][0] / det;
        inv[1][1] = J[0][0] / det;
    }
    else
    {
        const double c00 = J[1][1] * J[2][2] - J[1][2] * J[2][1];
        const double c10 = J[1][2] * J[2][0] - J[1][0] * J[2][2];
        const double c20 = J[1][0] * J[2][1] - J[1][1] * J[2][0];
        det = J[0][0] * c00 + J[0][1] * c10 + J[0][2] * c20;
        const double id = 1. / det;
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
    const int64_t base = static_cast<int64_t>(q) * stride;
    const double wdj = tables[tabW + q] * det;
    geo64[base * nCells + e] = wdj;
    geo32[base * nCells + e] = static_cast<float>(wdj);
    const double* dNd = tables + tabDNd + q * ND * 3;
    for (int n = 0; n < ND; ++n)
#pragma unroll
        for (int k = 0; k < DIM; ++k)
        {
            double s = 0;
#pragma unroll
            for (int j = 0; j < DIM; ++j)
                s += dNd[n * 3 + j] * inv[j][k];
            const int64_t idx = (base + 1 + n * DIM + k) * nCells + e;
            geo64[idx] = s;
            geo32[idx] = static_cast<float>(s);
        }
}

void BuildGeometryCache(Ctx& c)
{
    const Slot& D = c.slots[c.prm.disp_slot];
    c.geoStride = 1 + D.nen * c.dim;
    const size_t total = static_cast<size_t>(c.geoStride) * c.ip.nIp * c.nCells;
    c.dGeo64.alloc(total);
    c.dGeo32.alloc(total);
    const int64_t items = c.nCells * c.ip.nIp;
    const int blocks = static_cast<int>((items + 127) / 128);
    DispatchCfg(c, [&](auto cfg) {
        using C = decltype(cfg);
        k_geometry<C::dim, C::ng, C::nd, C::nip><<<blocks, 128, 0, c.stream>>>(
                c.nCells, static_cast<int64_t>(c.dCoords.n), c.dCoords.p, c.dGeoConnT.p, c.dTables.p, c.tabW, c.tabDN[c.geoInterp], c.tabDN[D.interp],
                c.geoStride, c.dGeo64.p, c.dGeo32.p);
    });
    AfterLaunch(c, "k_geometry");
    c.haveGeo = true;
}

static CellArgs MakeCellArgs(Ctx& c);

CellArgs CellArgsOf(Ctx& c)
{
    if (!c.haveGeo)
        BuildGeometryCache(c);
    return MakeCellArgs(c);
}

static CellArgs MakeCellArgs(Ctx& c)
{
    CellArgs a{};
    const Slot& D = c.slots[c.prm.disp_slot];
    a.nCells = c.nCells;
    a.nNodesD = D.nNodes;
    a.nDofs = c.nDofs;
    a.geoSize = static_cast<int64_t>(c.dGeo64.n);
    a.connD = D.dConnT.p;
    a.gdofD = D.dGdof.p;
    a.tabN_D = c.dTables.p + c.tabN[D.interp];
    if (c.prm.kind == NUTO_GPU_GRADIENT_DAMAGE)
    {
        const Slot& E = c.slots[c.prm.eeq_slot];
        a.nNodesE = E.nNodes;
        a.connE = E.dConnT.p;
        a.gdofE = E.dGdof.p;
        a.tabN_E = c.dTables.p + c.tabN[E.interp];
    }
    a.geo64 = c.dGeo64.p;
    a.geo32 = c.dGeo32.p;
    a.geoStride = c.geoStride;
    a.kappa = c.dKappa.p;
    a.escale = c.dEScale.n ? c.dEScale.p : nullptr;
    return a;
}

// ---- FP64 internal-force residual --------------------------------------------------------------------------
// MomentumBalance::Gradient (MomentumBalance.h:26-35) and GradientDamage::Gradient (GradientDamage.h:70-90)
// integrated as in Cell::IntegrateGeneric (Cell.h:105-119) and scattered like SimpleAssembler::BuildVector
// (SimpleAssembler.cpp:38-65).
// The cell vectors are written planar ([local entry][cell]: the displacement entries node-major, then the eeq
// entries) and k_gather_cell_vectors sums them per DOF in ascending cell order: the residual is bitwise the same on
// every run (SimpleAssembler::BuildVector sums thread-local vectors and merges them in a critical section).
// A block integrates CPB cells per pass and walks the cells with the grid's stride: one pass per block when the grid
// covers the mesh, or a persistent grid of a few blocks per SM beside the tangent (nuto_gpu_build_system).
template <int DIM, int ND, int NIP, int KIND>
__global__ void __launch_bounds__(128) k_residual(CellArgs a, LawParams L, const double* __restrict__ u,
                                                  double* __restrict__ fcell)
{
    constexpr int VD = DIM == 2 ? 3 : 6;
    constexpr bool GD = KIND == NUTO_GPU_GRADIENT_DAMAGE;
    constexpr int CPB = MaxI<1, 128 / MaxI<NIP, ND>::v>::v;
    constexpr int REC = VD + (GD ? 1 + DIM : 0);
    __shared__ double sU[CPB][ND][DIM];
    __shared__ double sE[GD ? CPB : 1][GD ? ND : 1];
    __shared__ double sIp[CPB][NIP][REC];
    const int64_t n = a.nCells;
    for (int64_t cell0 = static_cast<int64_t>(blockIdx.x) * CPB; cell0 < n;
         cell0 += static_cast<int64_t>(gridDim.x) * CPB)
    {
        for (int it = threadIdx.x; it < CPB * ND; it += blockDim.x)
        {
            const int cl = it % CPB, nd = it / CPB;
            const int64_t e = cell0 + cl;
            if (e >= n)
                continue;
            const int64_t g = a.gdofD[NG_IDX(a.connD[static_cast<int64_t>(nd) * n + e], a.nNodesD, 2)];
#pragma unroll
            for (int c = 0; c < DIM; ++c)
                sU[cl][nd][c] = u[NG_IDX(g + c, a.nDofs, 3)];
            if (GD)
                sE[cl][nd] = u[NG_IDX(a.gdofE[NG_IDX(a.connE[static_cast<int64_t>(nd) * n + e], a.nNodesE, 4)], a.nDofs, 5)];
        }
        __syncthreads();

        for (int it = threadIdx.x; it < CPB * NIP; it += blockDim.x)
        {
            const int cl = it % CPB, q = it / CPB;
            const int64_t e = cell0 + cl;
            if (e >= n)
                continue;
            const int64_t G0 = static_cast<int64_t>(q) * a.geoStride * n + e;
            const double* G = a.geo64 + NG_IDX(G0, a.geoSize, 6);
            const double wdj = G[0];
            // per-cell Young's modulus factor: scales the stress, i.e. the displacement rows
            const double wdjE = a.escale ? wdj * a.escale[e] : wdj;
            double H[DIM][DIM];
#pragma unroll
            for (int i = 0; i < DIM; ++i)
#pragma unroll
                for (int j = 0; j < DIM; ++j)
                    H[i][j] = 0;
            double eeq = 0, ge[DIM];
#pragma unroll
            for (int d = 0; d < DIM; ++d)
                ge[d] = 0;
#pragma unroll
            for (int nd = 0; nd < ND; ++nd)
            {
                double g[DIM];
#pragma unroll
                for (int d = 0; d < DIM; ++d)
                    g[d] = G[(1 + nd * DIM + d) * n];
#pragma unroll
                for (int c = 0; c < DIM; ++c)
#pragma unroll
                    for (int d = 0; d < DIM; ++d)
                        H[c][d] += sU[cl][nd][c] * g[d];
                if (GD)
                {
                    const double ev = sE[cl][nd];
                    eeq += a.tabN_D[q * ND + nd] * ev;
#pragma unroll
                    for (int d = 0; d < DIM; ++d)
                        ge[d] += ev * g[d];
                }
            }
            double eps[VD], sig[VD];
            StrainFromH<double, DIM>(H, eps);
            const double kh = a.kappa[NG_IDX(e * NIP + q, n * NIP, 7)];
            if (KIND == NUTO_GPU_MB_LINEAR_ELASTIC)
                ElasticStress<double, DIM>(L, eps, sig);
            else if (KIND == NUTO_GPU_MB_LOCAL_DAMAGE)
            {
                // LocalIsotropicDamage::Stress with EvolutionImplicit::Kappa (LocalIsotropicDamage.h:52-57, 110-113)
                const double kap = fmax(MisesValue<double, DIM>(L, eps), kh);
                LedStress<double, DIM>(L, eps, DamageOmega<double>(L, kap), sig);
            }
            else
            {
                const double kap = fmax(kh, eeq); // GradientDamage::Kappa (GradientDamage.h:127-130)
                const double omega = DamageOmega<double>(L, kap);
                LedStress<double, DIM>(L, eps, omega, sig);
                const double cg = L.c * InteractionFactor<double>(L, omega) * wdj;
                sIp[cl][q][VD] = (eeq - MisesValue<double, DIM>(L, eps)) * wdj;
#pragma unroll
                for (int d = 0; d < DIM; ++d)
                    sIp[cl][q][VD + 1 + d] = cg * ge[d];
            }
#pragma unroll
            for (int v = 0; v < VD; ++v)
                sIp[cl][q][v] = sig[v] * wdjE;
        }
        __syncthreads();

        for (int it = threadIdx.x; it < CPB * ND; it += blockDim.x)
        {
            const int cl = it % CPB, nd = it / CPB;
            const int64_t e = cell0 + cl;
            if (e >= n)
                continue;
            double fu[DIM], fe = 0;
#pragma unroll
            for (int c = 0; c < DIM; ++c)
                fu[c] = 0;
#pragma unroll 4
            for (int q = 0; q < NIP; ++q)
            {
                const double* G = a.geo64 + NG_IDX(static_cast<int64_t>(q) * a.geoStride * n + e, a.geoSize, 6);
                double g[DIM], b[DIM];
#pragma unroll
                for (int d = 0; d < DIM; ++d)
                    g[d] = G[(1 + nd * DIM + d) * n];
                BtS<double, DIM>(g, sIp[cl][q], b);
#pragma unroll
                for (int c = 0; c < DIM; ++c)
                    fu[c] += b[c];
                if (GD)
                {
                    double s = a.tabN_D[q * ND + nd] * sIp[cl][q][VD];
#pragma unroll
                    for (int d = 0; d < DIM; ++d)
                        s += g[d] * sIp[cl][q][VD + 1 + d];
                    fe += s;
                }
            }
            const int64_t nLocal = static_cast<int64_t>(ND) * (DIM + (GD ? 1 : 0));
            (void)nLocal; // buffer extent for checked builds
#pragma unroll
            for (int c = 0; c < DIM; ++c)
                fcell[NG_IDX((static_cast<int64_t>(nd) * DIM + c) * n + e, nLocal * n, 8)] = fu[c];
            if (GD)
                fcell[NG_IDX((static_cast<int64_t>(ND) * DIM + nd) * n + e, nLocal * n, 8)] = fe;
        }
        __syncthreads(); // the next pass overwrites the shared arrays
    }
}

// f[dof] (+)= sum of the cell vectors' entries of that DOF over the node's cells in ascending cell order: one thread
// per (node, component) of a slot; entry (off + loc * ncomp + comp) of the planar cell vectors
__global__ void k_gather_cell_vectors(int64_t nNodes, int ncomp, int off, int64_t nCells, int64_t nLocal,
                                      const int64_t* __restrict__ cellPtr, const int32_t* __restrict__ cellIdx,
                                      const uint8_t* __restrict__ cellLoc, const int64_t* __restrict__ gdof,
                                      const double* __restrict__ fcell, int64_t nDofs, double* __restrict__ f,
                                      int add)
{
    const int64_t it = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
    if (it >= nNodes * ncomp)
        return;
    const int64_t i = it / ncomp;
    const int comp = static_cast<int>(it % ncomp);
    double s = 0.;
    for (int64_t k = cellPtr[i]; k < cellPtr[i + 1]; ++k)
    {
        const int64_t e = cellIdx[k];
        const int64_t entry = off + static_cast<int64_t>(cellLoc[k]) * ncomp + comp;
        s += fcell[NG_IDX(entry * nCells + e, nLocal * nCells, 9)];
    }
    double* o = f + NG_IDX(gdof[i] + comp, nDofs, 9);
    *o = add ? *o + s : s;
}

void GatherCellVectors(Ctx& c, const Slot& S, int ncomp, int off, int64_t nLocal, double* f, bool add)
{
    const int64_t items = S.nNodes * ncomp;
    k_gather_cell_vectors<<<static_cast<unsigned>((items + 255) / 256), 256, 0, c.stream>>>(
            S.nNodes, ncomp, off, c.nCells, nLocal, S.dCellPtr.p, S.dCellIdx.p, S.dCellLoc.p, S.dGdof.p, c.dCellVec.p,
            c.nDofs, f, add ? 1 : 0);
    AfterLaunch(c, "k_gather_cell_vectors");
}

void LaunchResidual(Ctx& c, const double* u, double* f, int blocksPerSm)
{
    const Slot& D = c.slots[c.prm.disp_slot];
    const bool gd = c.prm.kind == NUTO_GPU_GRADIENT_DAMAGE;
    const int64_t nLocal = static_cast<int64_t>(D.nen) * (c.dim + (gd ? 1 : 0));
    if (c.dCellVec.n != static_cast<size_t>(nLocal * c.nCells))
        c.dCellVec.alloc(static_cast<size_t>(nLocal * c.nCells));
    // DOFs of slots that the integrand does not touch stay zero
    if (c.slots.size() > static_cast<size_t>(gd ? 2 : 1))
        NG_CUDA(cudaMemsetAsync(f, 0, c.nDofs * sizeof(double), c.stream));
    CellArgs a = MakeCellArgs(c);
    DispatchCfg(c, [&](auto cfg) {
        using C = decltype(cfg);
        constexpr int CPB = MaxI<1, 128 / MaxI<C::nip, C::nd>::v>::v;
        int64_t blocks = (c.nCells + CPB - 1) / CPB;
        if (blocksPerSm > 0)
            blocks = std::min<int64_t>(blocks, static_cast<int64_t>(blocksPerSm) * std::max(c.smCount, 1));
        k_residual<C::dim, C::nd, C::nip, C::kind><<<static_cast<unsigned>(blocks), 128, 0, c.stream>>>(
                a, c.law, u, c.dCellVec.p);
    });
    AfterLaunch(c, "k_residual");
    GatherCellVectors(c, D, c.dim, 0, nLocal, f, false);
    if (gd)
        GatherCellVectors(c, c.slots[c.prm.eeq_slot], 1, D.nen * c.dim, nLocal, f, false);
    c.stats.kernel_launches += gd ? 3 : 2;
}

// ---- tangent: FP32 or FP64 values scattered into CSR ---------------------------------------------------------
// MomentumBalance::Hessian0 (MomentumBalance.h:37-46) with LinearElastic / LocalIsotropicDamage::Tangent
// (LocalIsotropicDamage.h:59-68) and GradientDamage::Hessian0 (GradientDamage.h:92-120). The isotropic part of
// every tangent is lambda m m^T + mu diag(2..2, 1..1); for a node pair (a, b) with global gradients g_a, g_b
// this gives K_ab(k, l) = lambda g_a[k] g_b[l] + mu (g_a[l] g_b[k] + delta_kl g_a.g_b), the same values
// as B_a^T C B_b. Non-isotropic rank-1 parts (local damage, gradient-damage coupling) enter through
// P_a = B_a^T s and Q_b = B_b^T t.
template <int A, int B>
struct MinI
{
    static constexpr int v = A < B ? A : B;
};

// cells per block of the tangent kernel: bounded by the node pairs (512 per block) and by the shared-memory
// records per (cell, integration point, node) (256 per block keeps the static shared memory below 48 KB)
template <int ND, int NIP>
struct TangentShape
{
    static constexpr int threads = 256;
    static constexpr int cpb = MaxI<1, MinI<512 / (ND * ND), 256 / (NIP * ND)>::v>::v;
};

// Integration-point record of the row-gather tangent (per cell and point, contiguous): the node gradients
// G[ND][DIM], the integrand scalars (lambda w, mu w; gradient damage: w, c g w, c g' w' k' w grad eeq) and the
// two Voigt vectors of the rank-1 parts (local / gradient damage).
template <int DIM, int ND, int KIND>
struct IpRecord
{
    static constexpr bool GD = KIND == NUTO_GPU_GRADIENT_DAMAGE;
    static constexpr bool RANK1 = GD || KIND == NUTO_GPU_MB_LOCAL_DAMAGE;
    static constexpr int VD = DIM == 2 ? 3 : 6;
    static constexpr int nrec = 2 + (GD ? 2 + DIM : 0);
    static constexpr int g = 0;
    static constexpr int rec = ND * DIM;
    static constexpr int st = rec + nrec;
    static constexpr int size = st + (RANK1 ? 2 * VD : 0);
};

// ---- double-float arithmetic on the FP32 pipe -----------------------------------------------------------------
// A value is an unevaluated sum hi + lo of two floats (about 48 significant bits). Products use the FMA-exact error
// term, sums TwoSum; the _rn intrinsics keep the compiler from contracting the error-free transforms into FMAs.
struct Df
{
    float hi, lo;
};
__device__ __forceinline__ Df DfSplit(double x)
{
    const float h = __double2float_rn(x);
    return {h, __double2float_rn(x - static_cast<double>(h))};
}
__device__ __forceinline__ Df DfNorm(float s, float e)
{
    const float h = __fadd_rn(s, e);
    return {h, __fadd_rn(e, -__fadd_rn(h, -s))};
}
__device__ __forceinline__ Df DfAdd(Df x, Df y)
{
    const float s = __fadd_rn(x.hi, y.hi);
    const float bb = __fadd_rn(s, -x.hi);
    float e = __fadd_rn(__fadd_rn(x.hi, -__fadd_rn(s, -bb)), __fadd_rn(y.hi, -bb));
    e = __fadd_rn(e, __fadd_rn(x.lo, y.lo));
    return DfNorm(s, e);
}
__device__ __forceinline__ Df DfMul(Df x, Df y)
{
    const float p = __fmul_rn(x.hi, y.hi);
    float e = __fmaf_rn(x.hi, y.hi, -p);
    e = __fmaf_rn(x.hi, y.lo, e);
    e = __fmaf_rn(x.lo, y.hi, e);
    return DfNorm(p, e);
}
__device__ __forceinline__ Df DfNeg(Df x)
{
    return {-x.hi, -x.lo};
}
__device__ __forceinline__ double DfToDouble(Df x)
{
    return static_cast<double>(x.hi) + static_cast<double>(x.lo);
}

// REC = false: element-wise tangent, node-pair blocks added into the CSR values with atomics.
// REC = true: phases 0 and A only; the integration-point records are written for k_tangent_rows.
// T is the arithmetic of the geometry, strain and law evaluation; TO the type of the written values or records.
// DF = true (FP64 T, element-wise): the node-pair products of phase B in double-float FP32 arithmetic instead of
// FP64 (the FP64 pipe is narrow on this part); the law stays FP64 and the result is added with FP64 atomics.
template <typename T, int DIM, int ND, int NIP, int KIND, bool REC, typename TO = T, bool DF = false>
__global__ void __launch_bounds__(256) k_tangent(CellArgs a, LawParams L, ScatterArgs S, int pUU, int pUE, int pEU,
                                                 int pEE, const double* __restrict__ u, TO* __restrict__ vals)
{
    constexpr int VD = DIM == 2 ? 3 : 6;
    constexpr bool GD = KIND == NUTO_GPU_GRADIENT_DAMAGE;
    constexpr bool LD = KIND == NUTO_GPU_MB_LOCAL_DAMAGE;
    constexpr bool RANK1 = GD || LD;
    constexpr int CPB = TangentShape<ND, NIP>::cpb;
    constexpr int NREC = 2 + (GD ? 2 + DIM : 0);
    __shared__ double sU[CPB][ND][DIM];
    __shared__ double sE[GD ? CPB : 1][GD ? ND : 1];
    __shared__ T sG[CPB][NIP][ND][DIM];
    __shared__ T sRec[CPB][NIP][NREC];
    __shared__ T sST[RANK1 ? CPB : 1][RANK1 ? NIP : 1][2][VD];
    __shared__ T sPQ[RANK1 ? CPB : 1][RANK1 ? NIP : 1][RANK1 ? ND : 1][2][DIM];
    __shared__ int64_t sBaseU[CPB][ND][DIM]; // row start + block offset of the (disp, disp) block
    __shared__ int64_t sBaseUE[GD ? CPB : 1][GD ? ND : 1][DIM];
    __shared__ int64_t sBaseEU[GD ? CPB : 1][GD ? ND : 1];
    __shared__ int64_t sBaseEE[GD ? CPB : 1][GD ? ND : 1];
    constexpr bool USE_DF = DF && sizeof(T) == 8 && !REC;
    __shared__ Df sGd[USE_DF ? CPB : 1][USE_DF ? NIP : 1][USE_DF ? ND : 1][DIM];
    __shared__ Df sRecd[USE_DF ? CPB : 1][USE_DF ? NIP : 1][NREC];
    __shared__ Df sPQd[USE_DF && RANK1 ? CPB : 1][USE_DF && RANK1 ? NIP : 1][USE_DF && RANK1 ? ND : 1][2][DIM];
    __shared__ Df sNd[USE_DF && GD ? NIP : 1][USE_DF && GD ? ND : 1];
    const int64_t n = a.nCells;
    const int64_t cell0 = static_cast<int64_t>(blockIdx.x) * CPB;

    // phase 0: DOF values, row bases, geometry
    for (int it = threadIdx.x; it < CPB * ND; it += blockDim.x)
    {
        const int cl = it % CPB, nd = it / CPB;
        const int64_t e = cell0 + cl;
        if (e >= n)
            continue;
        const int32_t aD = static_cast<int32_t>(NG_IDX(a.connD[static_cast<int64_t>(nd) * n + e], a.nNodesD, 2));
        const int64_t g = a.gdofD[aD];
#pragma unroll
        for (int c = 0; c < DIM; ++c)
        {
            sU[cl][nd][c] = u[NG_IDX(g + c, a.nDofs, 3)];
            if (!REC)
            {
                const int64_t rs = S.rowPtr[NG_IDX(g + c, S.nRows, 9)];
                sBaseU[cl][nd][c] = rs + S.blk[pUU][aD];
                if (GD)
                    sBaseUE[cl][nd][c] = rs + S.blk[pUE][aD];
            }
        }
        if (GD)
        {
            const int32_t aE = static_cast<int32_t>(NG_IDX(a.connE[static_cast<int64_t>(nd) * n + e], a.nNodesE, 4));
            const int64_t ge = a.gdofE[aE];
            sE[cl][nd] = u[NG_IDX(ge, a.nDofs, 5)];
            if (!REC)
            {
                const int64_t rs = S.rowPtr[NG_IDX(ge, S.nRows, 9)];
                sBaseEU[cl][nd] = rs + S.blk[pEU][aE];
                sBaseEE[cl][nd] = rs + S.blk[pEE][aE];
            }
        }
    }
    for (int it = threadIdx.x; it < CPB * NIP * ND * DIM; it += blockDim.x)
    {
        const int cl = it % CPB;
        int r = it / CPB;
        const int d = r % DIM;
        r /= DIM;
        const int nd = r % ND;
        const int q = r / ND;
        const int64_t e = cell0 + cl;
        if (e >= n)
            continue;
        const int64_t idx = NG_IDX((static_cast<int64_t>(q) * a.geoStride + 1 + nd * DIM + d) * n + e, a.geoSize, 6);
        if (sizeof(T) == 4)
            sG[cl][q][nd][d] = static_cast<T>(a.geo32[idx]);
        else
            sG[cl][q][nd][d] = static_cast<T>(a.geo64[idx]);
    }
    __syncthreads();

    // phase A: material data per (cell, integration point)
    for (int it = threadIdx.x; it < CPB * NIP; it += blockDim.x)
    {
        const int cl = it % CPB, q = it / CPB;
        const int64_t e = cell0 + cl;
        if (e >= n)
            continue;
        const int64_t widx = NG_IDX(static_cast<int64_t>(q) * a.geoStride * n + e, a.geoSize, 6);
        const T wdj = sizeof(T) == 4 ? static_cast<T>(a.geo32[widx]) : static_cast<T>(a.geo64[widx]);
        // per-cell Young's modulus factor: scales the material tangent and dsigma/domega (displacement rows)
        const T wdjE = a.escale ? wdj * static_cast<T>(a.escale[e]) : wdj;
        T H[DIM][DIM];
#pragma unroll
        for (int i = 0; i < DIM; ++i)
#pragma unroll
            for (int j = 0; j < DIM; ++j)
                H[i][j] = T(0);
        T eeq = T(0), ge[DIM];
#pragma unroll
        for (int d = 0; d < DIM; ++d)
            ge[d] = T(0);
        for (int nd = 0; nd < ND; ++nd)
        {
#pragma unroll
            for (int c = 0; c < DIM; ++c)
#pragma unroll
                for (int d = 0; d < DIM; ++d)
                    H[c][d] += static_cast<T>(sU[cl][nd][c]) * sG[cl][q][nd][d];
            if (GD)
            {
                const T ev = static_cast<T>(sE[cl][nd]);
                eeq += static_cast<T>(a.tabN_D[q * ND + nd]) * ev;
#pragma unroll
                for (int d = 0; d < DIM; ++d)
                    ge[d] += ev * sG[cl][q][nd][d];
            }
        }
        T eps[VD];
        StrainFromH<T, DIM>(H, eps);
        const T kh = static_cast<T>(a.kappa[NG_IDX(e * NIP + q, n * NIP, 7)]);
        T lam, mu;
        if (KIND == NUTO_GPU_MB_LINEAR_ELASTIC)
        {
            // C11 = lambda + 2 mu, C12 = lambda, C33 = mu for every LinearElastic::CalculateC variant
            lam = T(L.C12);
            mu = T(L.C33);
        }
        else if (LD)
        {
            const T eqs = MisesValue<T, DIM>(L, eps);
            const T kap = eqs > kh ? eqs : kh;
            const T omega = DamageOmega<T>(L, kap);
            LedTangentLameParams<T, DIM>(L, eps, omega, lam, mu);
            // rank-1 part dsigma/domega * domega/dkappa * dkappa/deps (LocalIsotropicDamage.h:59-68, 115-122)
            T dsdw[VD], dk[VD];
            LedDstressDomega<T, DIM>(L, eps, dsdw);
            const T dOdK = DamageDerivative<T>(L, kap);
            if (eqs >= kh)
                MisesDerivative<T, DIM>(L, eps, dk);
            else
#pragma unroll
                for (int v = 0; v < VD; ++v)
                    dk[v] = T(0);
#pragma unroll
            for (int v = 0; v < VD; ++v)
            {
                sST[cl][q][0][v] = dsdw[v] * dOdK * wdjE;
                sST[cl][q][1][v] = dk[v];
            }
        }
        else
        {
            const T kap = kh > eeq ? kh : eeq;
            const T omega = DamageOmega<T>(L, kap);
            const T dKdE = eeq >= kh ? T(1) : T(0);
            const T dOdK = DamageDerivative<T>(L, kap);
            const T g = InteractionFactor<T>(L, omega);
            const T dgdw = InteractionDerivative<T>(L, omega);
            LedTangentLameParams<T, DIM>(L, eps, omega, lam, mu);
            T dsdw[VD], dn[VD];
            LedDstressDomega<T, DIM>(L, eps, dsdw);
            MisesDerivative<T, DIM>(L, eps, dn);
#pragma unroll
            for (int v = 0; v < VD; ++v)
            {
                sST[cl][q][0][v] = dsdw[v] * dOdK * dKdE * wdjE; // (disp, eeq): B^T (dsigma/domega w' k') N
                sST[cl][q][1][v] = dn[v] * wdj;                 // (eeq, disp): -N^T (deps_eq/deps)^T B
            }
            sRec[cl][q][2] = wdj;
            sRec[cl][q][3] = T(L.c) * g * wdj;
            const T sc = T(L.c) * dgdw * dOdK * dKdE * wdj;
#pragma unroll
            for (int d = 0; d < DIM; ++d)
                sRec[cl][q][4 + d] = sc * ge[d];
        }
        sRec[cl][q][0] = lam * wdjE;
        sRec[cl][q][1] = mu * wdjE;
    }
    __syncthreads();

    if (REC)
    {
        // records of the block's cells are one contiguous range: coalesced stores
        using R = IpRecord<DIM, ND, KIND>;
        const int cells = static_cast<int>(n - cell0 < CPB ? n - cell0 : CPB);
        TO* out = vals + cell0 * NIP * R::size;
        for (int it = threadIdx.x; it < cells * NIP * R::size; it += blockDim.x)
        {
            const int f = it % R::size;
            const int r = it / R::size;
            const int q = r % NIP, cl = r / NIP;
            T v;
            if (f < R::rec)
                v = sG[cl][q][f / DIM][f % DIM];
            else if (f < R::st)
                v = sRec[cl][q][f - R::rec];
            else
                v = sST[cl][q][(f - R::st) / VD][(f - R::st) % VD];
            out[it] = static_cast<TO>(v);
        }
        return;
    }

    if (RANK1)
    {
        for (int it = threadIdx.x; it < CPB * NIP * ND; it += blockDim.x)
        {
            const int cl = it % CPB;
            const int r = it / CPB;
            const int nd = r % ND, q = r / ND;
            if (cell0 + cl >= n)
                continue;
            BtS<T, DIM>(sG[cl][q][nd], sST[cl][q][0], sPQ[cl][q][nd][0]);
            BtS<T, DIM>(sG[cl][q][nd], sST[cl][q][1], sPQ[cl][q][nd][1]);
        }
        __syncthreads();
    }

    if constexpr (USE_DF)
    {
        // split the FP64 inputs of phase B once per (cell, point, node)
        for (int it = threadIdx.x; it < CPB * NIP * ND; it += blockDim.x)
        {
            const int cl = it % CPB;
            const int r = it / CPB;
            const int nd = r % ND, q = r / ND;
#pragma unroll
            for (int d = 0; d < DIM; ++d)
            {
                sGd[cl][q][nd][d] = DfSplit(static_cast<double>(sG[cl][q][nd][d]));
                if constexpr (RANK1)
                {
                    sPQd[cl][q][nd][0][d] = DfSplit(static_cast<double>(sPQ[cl][q][nd][0][d]));
                    sPQd[cl][q][nd][1][d] = DfSplit(static_cast<double>(sPQ[cl][q][nd][1][d]));
                }
            }
            if (nd == 0)
                for (int k = 0; k < NREC; ++k)
                    sRecd[cl][q][k] = DfSplit(static_cast<double>(sRec[cl][q][k]));
            if constexpr (GD)
                if (cl == 0)
                    sNd[q][nd] = DfSplit(a.tabN_D[q * ND + nd]);
        }
        __syncthreads();
        for (int it = threadIdx.x; it < CPB * ND * ND; it += blockDim.x)
        {
            const int cl = it % CPB;
            const int pr = it / CPB;
            const int ia = pr / ND, ib = pr % ND;
            const int64_t e = cell0 + cl;
            if (e >= n)
                continue;
            const Df z{0.f, 0.f};
            Df kuu[DIM][DIM], kue[DIM], keu[DIM], kee = z;
#pragma unroll
            for (int k = 0; k < DIM; ++k)
            {
                kue[k] = keu[k] = z;
#pragma unroll
                for (int l = 0; l < DIM; ++l)
                    kuu[k][l] = z;
            }
            for (int q = 0; q < NIP; ++q)
            {
                const Df* ga = sGd[cl][q][ia];
                const Df* gb = sGd[cl][q][ib];
                const Df lam = sRecd[cl][q][0], mu = sRecd[cl][q][1];
                Df gab = DfMul(ga[0], gb[0]);
#pragma unroll
                for (int d = 1; d < DIM; ++d)
                    gab = DfAdd(gab, DfMul(ga[d], gb[d]));
                Df la[DIM], ma[DIM];
#pragma unroll
                for (int k = 0; k < DIM; ++k)
                {
                    la[k] = DfMul(lam, ga[k]);
                    ma[k] = DfMul(mu, ga[k]);
                }
                const Df mg = DfMul(mu, gab);
#pragma unroll
                for (int k = 0; k < DIM; ++k)
                {
#pragma unroll
                    for (int l = 0; l < DIM; ++l)
                        kuu[k][l] = DfAdd(kuu[k][l], DfAdd(DfMul(la[k], gb[l]), DfMul(ma[l], gb[k])));
                    kuu[k][k] = DfAdd(kuu[k][k], mg);
                }
                if constexpr (LD)
                {
#pragma unroll
                    for (int k = 0; k < DIM; ++k)
#pragma unroll
                        for (int l = 0; l < DIM; ++l)
                            kuu[k][l] = DfAdd(kuu[k][l], DfMul(sPQd[cl][q][ia][0][k], sPQd[cl][q][ib][1][l]));
                }
                if constexpr (GD)
                {
                    const Df Na = sNd[q][ia], Nb = sNd[q][ib];
                    Df gs = DfMul(ga[0], sRecd[cl][q][4]);
#pragma unroll
                    for (int d = 1; d < DIM; ++d)
                        gs = DfAdd(gs, DfMul(ga[d], sRecd[cl][q][4 + d]));
#pragma unroll
                    for (int k = 0; k < DIM; ++k)
                    {
                        kue[k] = DfAdd(kue[k], DfMul(sPQd[cl][q][ia][0][k], Nb));
                        keu[k] = DfAdd(keu[k], DfNeg(DfMul(Na, sPQd[cl][q][ib][1][k])));
                    }
                    kee = DfAdd(kee, DfAdd(DfMul(DfMul(sRecd[cl][q][2], Na), Nb),
                                           DfAdd(DfMul(sRecd[cl][q][3], gab), DfMul(gs, Nb))));
                }
            }
            const int64_t ridx = static_cast<int64_t>(ia * ND + ib) * n + e;
            const int rUU = S.rank[pUU][ridx];
#pragma unroll
            for (int k = 0; k < DIM; ++k)
            {
                const int64_t row = sBaseU[cl][ia][k] + DIM * rUU;
#pragma unroll
                for (int l = 0; l < DIM; ++l)
                    atomicAdd(vals + NG_IDX(row + l, S.nnz, 10), static_cast<TO>(DfToDouble(kuu[k][l])));
            }
            if constexpr (GD)
            {
                const int rUE = S.rank[pUE][ridx];
                const int rEU = S.rank[pEU][ridx];
                const int rEE = S.rank[pEE][ridx];
#pragma unroll
                for (int k = 0; k < DIM; ++k)
                    atomicAdd(vals + NG_IDX(sBaseUE[cl][ia][k] + rUE, S.nnz, 10), static_cast<TO>(DfToDouble(kue[k])));
                const int64_t rowE = sBaseEU[cl][ia] + DIM * rEU;
#pragma unroll
                for (int l = 0; l < DIM; ++l)
                    atomicAdd(vals + NG_IDX(rowE + l, S.nnz, 10), static_cast<TO>(DfToDouble(keu[l])));
                atomicAdd(vals + NG_IDX(sBaseEE[cl][ia] + rEE, S.nnz, 10), static_cast<TO>(DfToDouble(kee)));
            }
        }
        return;
    }

    // phase B: one thread per (cell, node pair)
    for (int it = threadIdx.x; it < CPB * ND * ND; it += blockDim.x)
    {
        const int cl = it % CPB;
        const int pr = it / CPB;
        const int ia = pr / ND, ib = pr % ND;
        const int64_t e = cell0 + cl;
        if (e >= n)
            continue;
        T kuu[DIM][DIM], kue[DIM], keu[DIM], kee = T(0);
#pragma unroll
        for (int k = 0; k < DIM; ++k)
        {
            kue[k] = keu[k] = T(0);
#pragma unroll
            for (int l = 0; l < DIM; ++l)
                kuu[k][l] = T(0);
        }
        for (int q = 0; q < NIP; ++q)
        {
            const T* ga = sG[cl][q][ia];
            const T* gb = sG[cl][q][ib];
            const T lam = sRec[cl][q][0], mu = sRec[cl][q][1];
            T gab = T(0);
#pragma unroll
            for (int d = 0; d < DIM; ++d)
                gab += ga[d] * gb[d];
#pragma unroll
            for (int k = 0; k < DIM; ++k)
            {
#pragma unroll
                for (int l = 0; l < DIM; ++l)
                    kuu[k][l] += lam * ga[k] * gb[l] + mu * ga[l] * gb[k];
                kuu[k][k] += mu * gab;
            }
            if (LD)
            {
#pragma unroll
                for (int k = 0; k < DIM; ++k)
#pragma unroll
                    for (int l = 0; l < DIM; ++l)
                        kuu[k][l] += sPQ[cl][q][ia][0][k] * sPQ[cl][q][ib][1][l];
            }
            if (GD)
            {
                const T Na = static_cast<T>(a.tabN_D[q * ND + ia]);
                const T Nb = static_cast<T>(a.tabN_D[q * ND + ib]);
                T gs = T(0);
#pragma unroll
                for (int d = 0; d < DIM; ++d)
                    gs += ga[d] * sRec[cl][q][4 + d];
#pragma unroll
                for (int k = 0; k < DIM; ++k)
                {
                    kue[k] += sPQ[cl][q][ia][0][k] * Nb;
                    keu[k] -= Na * sPQ[cl][q][ib][1][k];
                }
                kee += sRec[cl][q][2] * Na * Nb + sRec[cl][q][3] * gab + gs * Nb;
            }
        }
        const int64_t ridx = static_cast<int64_t>(ia * ND + ib) * n + e;
        const int rUU = S.rank[pUU][ridx];
#pragma unroll
        for (int k = 0; k < DIM; ++k)
        {
            const int64_t row = sBaseU[cl][ia][k] + DIM * rUU;
#pragma unroll
            for (int l = 0; l < DIM; ++l)
                atomicAdd(vals + NG_IDX(row + l, S.nnz, 10), kuu[k][l]);
        }
        if (GD)
        {
            const int rUE = S.rank[pUE][ridx];
            const int rEU = S.rank[pEU][ridx];
            const int rEE = S.rank[pEE][ridx];
#pragma unroll
            for (int k = 0; k < DIM; ++k)
                atomicAdd(vals + NG_IDX(sBaseUE[cl][ia][k] + rUE, S.nnz, 10), kue[k]);
            const int64_t rowE = sBaseEU[cl][ia] + DIM * rEU;
#pragma unroll
            for (int l = 0; l < DIM; ++l)
                atomicAdd(vals + NG_IDX(rowE + l, S.nnz, 10), keu[l]);
            atomicAdd(vals + NG_IDX(sBaseEE[cl][ia] + rEE, S.nnz, 10), kee);
        }
    }
}

static ScatterArgs MakeScatterArgs(Ctx& c)
{
    ScatterArgs s{};
    s.nnz = c.nnz;
    s.nRows = c.nDofs;
    s.rowPtr = c.dRowPtr.p;
    const int ns = static_cast<int>(c.slots.size());
    for (int p = 0; p < ns * ns; ++p)
    {
        s.rank[p] = c.pairs[p].rank;
        s.blk[p] = c.pairs[p].dBlk.p;
    }
    return s;
}

// ---- row-gather tangent ------------------------------------------------------------------------------------
// One warp per displacement node a assembles the complete CSR rows of a (and, for gradient damage, of its eeq
// node): for every cell around a it reads the cell's integration-point records once (contiguous), each lane
// integrates one (neighbour b, row) item of the node-pair block over the points, and the sums are added into a
// shared-memory copy of the rows at the ranks of b. Cells are visited one after another, so the row buffer
// needs no atomics; at the end the rows are stored once, coalesced, and no value array reset is needed.
struct RowArgs
{
    int64_t nNodes, nCells, nnz, nRows;
    const int64_t* gdofD;
    const int64_t* gdofE;
    const int32_t* eOf;
    const int64_t* cellPtr;
    const int32_t* cellIdx;
    const uint8_t* cellLoc;
    const int64_t* rowPtr;
    const uint8_t* rank[4]; // UU, UE, EU, EE
    const int32_t* blk[4];
    const double* tabN; // nIp x nd
};

constexpr int kRowCap = 256;

template <typename T, int DIM, int ND, int NIP, int KIND>
struct RowShape
{
    using R = IpRecord<DIM, ND, KIND>;
    static constexpr int nrows = DIM + (R::GD ? 1 : 0);
    static constexpr int warps = sizeof(T) == 4 ? 4 : 2;
    static constexpr int recs = NIP * R::size;                         // one cell's records
    static constexpr int perWarp = 2 * recs + nrows * kRowCap;          // double-buffered records + rows (T)
    static constexpr size_t smem = static_cast<size_t>(warps) * perWarp * sizeof(T);
};

// asynchronous global -> shared copies (cp.async, 4 or 8 bytes), committed and awaited in groups
template <typename T>
__device__ __forceinline__ void AsyncCopy(T* dst, const T* src)
{
    const unsigned sa = static_cast<unsigned>(__cvta_generic_to_shared(dst));
    if constexpr (sizeof(T) == 4)
        asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(sa), "l"(src) : "memory");
    else
        asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(sa), "l"(src) : "memory");
}
__device__ __forceinline__ void AsyncCommit()
{
    asm volatile("cp.async.commit_group;\n" ::: "memory");
}
template <int N>
__device__ __forceinline__ void AsyncWait()
{
    asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

template <typename T, int DIM, int ND, int NIP, int KIND>
__global__ void __launch_bounds__(RowShape<T, DIM, ND, NIP, KIND>::warps * 32)
        k_tangent_rows(RowArgs r, const T* __restrict__ recs, T* __restrict__ vals)
{
    using R = IpRecord<DIM, ND, KIND>;
    using Sh = RowShape<T, DIM, ND, NIP, KIND>;
    constexpr bool GD = R::GD;
    constexpr bool LD = KIND == NUTO_GPU_MB_LOCAL_DAMAGE;
    constexpr int VD = R::VD;
    constexpr int NJ = DIM + (GD ? 1 : 0); // items per neighbour: the DIM displacement rows (+ the eeq row)
    constexpr int NITEM = ND * NJ;
    constexpr int MAXIT = (NITEM + 31) / 32;
    constexpr int NROWS = Sh::nrows;
    extern __shared__ __align__(16) unsigned char smRaw[];
    const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
    T* recBuf = reinterpret_cast<T*>(smRaw) + wid * Sh::perWarp;
    T* row = recBuf + 2 * Sh::recs;
    __shared__ T sN[GD ? NIP * ND : 1]; // shape values N(q, node), gradient damage only
    if (GD)
    {
        for (int i = threadIdx.x; i < NIP * ND; i += blockDim.x)
            sN[i] = static_cast<T>(r.tabN[i]);
        __syncthreads();
    }
    const int64_t a = static_cast<int64_t>(blockIdx.x) * Sh::warps + wid;
    if (a >= r.nNodes)
        return; // the whole warp leaves; only warp-level synchronisation follows
    int64_t rs[NROWS];
    int len[NROWS];
    const int64_t g = r.gdofD[a];
#pragma unroll
    for (int k = 0; k < DIM; ++k)
    {
        rs[k] = r.rowPtr[NG_IDX(g + k, r.nRows, 40)];
        len[k] = static_cast<int>(r.rowPtr[g + k + 1] - rs[k]);
    }
    int32_t ae = 0;
    if (GD)
    {
        ae = r.eOf[a];
        const int64_t ge = r.gdofE[ae];
        rs[DIM] = r.rowPtr[NG_IDX(ge, r.nRows, 40)];
        len[DIM] = static_cast<int>(r.rowPtr[ge + 1] - rs[DIM]);
    }
    const int32_t bUU = r.blk[0][a];
    const int32_t bUE = GD ? r.blk[1][a] : 0;
    const int32_t bEU = GD ? r.blk[2][ae] : 0;
    const int32_t bEE = GD ? r.blk[3][ae] : 0;
#pragma unroll
    for (int k = 0; k < NROWS; ++k)
        for (int q = lane; q < len[k]; q += 32)
            row[k * kRowCap + q] = T(0);
    __syncwarp();

    // the next cell's records stream into the other buffer while the current cell is integrated
    const int64_t k0 = r.cellPtr[a], k1 = r.cellPtr[a + 1];
    auto issue = [&](int64_t kc, T* buf) {
        const T* src = recs + NG_IDX(r.cellIdx[kc], r.nCells, 41) * Sh::recs;
        for (int i = lane; i < Sh::recs; i += 32)
            AsyncCopy(buf + i, src + i);
    };
    if (k0 < k1)
        issue(k0, recBuf);
    AsyncCommit();
    for (int64_t kc = k0; kc < k1; ++kc)
    {
        const int64_t e = r.cellIdx[kc];
        const int ia = r.cellLoc[kc];
        T* rec = recBuf + ((kc - k0) & 1) * Sh::recs;
        if (kc + 1 < k1)
            issue(kc + 1, recBuf + ((kc + 1 - k0) & 1) * Sh::recs);
        AsyncCommit();
        // ranks of this lane's neighbours (independent of the records: loaded while the copies complete)
        int rk0[MAXIT], rk1[MAXIT];
#pragma unroll
        for (int m = 0; m < MAXIT; ++m)
        {
            const int item = lane + 32 * m;
            rk0[m] = rk1[m] = 0;
            if (item >= NITEM)
                continue;
            const int ib = item / NJ, j = item % NJ;
            const int64_t ridx = static_cast<int64_t>(ia * ND + ib) * r.nCells + e;
            if (j < DIM)
            {
                rk0[m] = r.rank[0][ridx];
                if (GD)
                    rk1[m] = r.rank[1][ridx];
            }
            else
            {
                rk0[m] = r.rank[2][ridx];
                rk1[m] = r.rank[3][ridx];
            }
        }
        AsyncWait<1>();
        __syncwarp();
        // Every item (neighbour b, row j) uses one branch-free form; j < DIM is displacement row j, j == DIM the
        // eeq row:  v[l] += c1 gb[l] + c2 ga[l] + c3 Qb[l],  v[DIM] += d1 Nb + d2 (ga . gb),  plus mu (ga . gb)
        // on the diagonal of displacement rows (kept apart and added once per cell).
        T acc[MAXIT][DIM + 1], accd[MAXIT];
#pragma unroll
        for (int m = 0; m < MAXIT; ++m)
        {
            accd[m] = T(0);
#pragma unroll
            for (int l = 0; l <= DIM; ++l)
                acc[m][l] = T(0);
        }
        for (int q = 0; q < NIP; ++q)
        {
            const T* Rq = rec + q * R::size;
            const T* ga = Rq + R::g + ia * DIM;
            const T lamw = Rq[R::rec + 0], muw = Rq[R::rec + 1];
            const T Na = GD ? sN[q * ND + ia] : T(0);
            T gs = T(0); // (c g' w' k' w grad eeq) . g_a, gradient damage only
            if (GD)
            {
#pragma unroll
                for (int d = 0; d < DIM; ++d)
                    gs += ga[d] * Rq[R::rec + 4 + d];
            }
#pragma unroll
            for (int m = 0; m < MAXIT; ++m)
            {
                const int item = lane + 32 * m;
                if (item >= NITEM)
                    continue;
                const int ib = item / NJ, j = item % NJ;
                const bool urow = j < DIM;
                const int jj = urow ? j : 0;
                const T* gb = Rq + R::g + ib * DIM;
                T gab = T(0);
#pragma unroll
                for (int d = 0; d < DIM; ++d)
                    gab += ga[d] * gb[d];
                const T gaj = ga[jj], gbj = gb[jj];
                T c1 = lamw * gaj, c2 = muw * gbj, c3 = T(0);
                T Qb[DIM];
                if (LD || GD)
                {
                    // row jj of B_a^T s and all of B_b^T t (Voigt: 2D xx yy xy; 3D xx yy zz yz zx xy)
                    const T* sv = Rq + R::st;
                    T paj = T(0);
#pragma unroll
                    for (int d = 0; d < DIM; ++d)
                        paj += ga[d] * sv[d == jj ? jj : (DIM == 2 ? 2 : 6 - jj - d)];
                    BtS<T, DIM>(gb, Rq + R::st + VD, Qb);
                    if (LD)
                        c3 = paj;
                    if (GD)
                    {
                        const T Nb = sN[q * ND + ib];
                        c1 = urow ? c1 : T(0);
                        c2 = urow ? c2 : T(0);
                        c3 = urow ? T(0) : -Na;
                        const T d1 = urow ? paj : Rq[R::rec + 2] * Na + gs;
                        const T d2 = urow ? T(0) : Rq[R::rec + 3];
                        acc[m][DIM] += d1 * Nb + d2 * gab;
                    }
                }
#pragma unroll
                for (int l = 0; l < DIM; ++l)
                {
                    acc[m][l] += c1 * gb[l] + c2 * ga[l];
                    if (LD || GD)
                        acc[m][l] += c3 * Qb[l];
                }
                accd[m] += urow ? muw * gab : T(0);
            }
        }
#pragma unroll
        for (int m = 0; m < MAXIT; ++m)
        {
            const int j = (lane + 32 * m) % NJ;
#pragma unroll
            for (int l = 0; l < DIM; ++l)
                acc[m][l] += l == j ? accd[m] : T(0);
        }
        // add the items into the row buffer at the ranks of b (distinct positions: no conflicts)
#pragma unroll
        for (int m = 0; m < MAXIT; ++m)
        {
            const int item = lane + 32 * m;
            if (item >= NITEM)
                continue;
            const int j = item % NJ;
            if (j < DIM)
            {
                T* rw = row + j * kRowCap;
                const int pos = bUU + DIM * rk0[m];
#pragma unroll
                for (int l = 0; l < DIM; ++l)
                    rw[NG_IDX(pos + l, kRowCap, 42)] += acc[m][l];
                if (GD)
                    rw[NG_IDX(bUE + rk1[m], kRowCap, 42)] += acc[m][DIM];
            }
            else
            {
                T* rw = row + DIM * kRowCap;
                const int pos = bEU + DIM * rk0[m];
#pragma unroll
                for (int l = 0; l < DIM; ++l)
                    rw[NG_IDX(pos + l, kRowCap, 42)] += acc[m][l];
                rw[NG_IDX(bEE + rk1[m], kRowCap, 42)] += acc[m][DIM];
            }
        }
        __syncwarp();
    }
#pragma unroll
    for (int k = 0; k < NROWS; ++k)
        for (int q = lane; q < len[k]; q += 32)
            vals[NG_IDX(rs[k] + q, r.nnz, 43)] = row[k * kRowCap + q];
}

// Row gather applies when every displacement node has one eeq node with the same local index in all its cells
// (same interpolation for both fields, as in every gradient-damage set-up here) and the rows fit the buffer.
static bool RowsSupported(Ctx& c)
{
    if (c.rowsMode >= 0)
        return c.rowsMode == 1;
    c.rowsMode = 0;
    const int dS = c.prm.disp_slot;
    const Slot& D = c.slots[dS];
    if (c.prm.kind == NUTO_GPU_GRADIENT_DAMAGE)
    {
        const Slot& E = c.slots[c.prm.eeq_slot];
        if (E.nen != D.nen || E.nNodes != D.nNodes)
            return false;
        std::vector<int32_t> eOf(D.nNodes, -1);
        std::vector<char> seen(E.nNodes, 0);
        for (size_t i = 0; i < D.conn.size(); ++i)
        {
            int32_t& m = eOf[D.conn[i]];
            if (m < 0)
            {
                m = E.conn[i];
                if (seen[m])
                    return false;
                seen[m] = 1;
            }
            else if (m != E.conn[i])
                return false;
        }
        c.dEOf.alloc(eOf.size());
        NG_CUDA(cudaMemcpy(c.dEOf.p, eOf.data(), eOf.size() * sizeof(int32_t), cudaMemcpyHostToDevice));
        c.hEOf = eOf;
    }
    c.rowsMode = 1;
    return true;
}

static RowArgs MakeRowArgs(Ctx& c)
{
    const int ns = static_cast<int>(c.slots.size());
    const int dS = c.prm.disp_slot;
    const bool gd = c.prm.kind == NUTO_GPU_GRADIENT_DAMAGE;
    const int eS = gd ? c.prm.eeq_slot : dS;
    const Slot& D = c.slots[dS];
    RowArgs r{};
    r.nNodes = D.nNodes;
    r.nCells = c.nCells;
    r.nnz = c.nnz;
    r.nRows = c.nDofs;
    r.gdofD = D.dGdof.p;
    r.gdofE = c.slots[eS].dGdof.p;
    r.eOf = gd ? c.dEOf.p : nullptr;
    r.cellPtr = D.dCellPtr.p;
    r.cellIdx = D.dCellIdx.p;
    r.cellLoc = D.dCellLoc.p;
    r.rowPtr = c.dRowPtr.p;
    const int pr[4] = {dS * ns + dS, dS * ns + eS, eS * ns + dS, eS * ns + eS};
    for (int k = 0; k < 4; ++k)
    {
        r.rank[k] = c.pairs[pr[k]].rank;
        r.blk[k] = c.pairs[pr[k]].dBlk.p;
    }
    r.tabN = c.dTables.p + c.tabN[D.interp];
    return r;
}

template <typename T>
static void LaunchTangentRows(Ctx& c, const double* u, T* vals)
{
    CellArgs a = MakeCellArgs(c);
    ScatterArgs s = MakeScatterArgs(c);
    RowArgs r = MakeRowArgs(c);
    DispatchCfg(c, [&](auto cfg) {
        using C = decltype(cfg);
        using R = IpRecord<C::dim, C::nd, C::kind>;
        using Sh = RowShape<T, C::dim, C::nd, C::nip, C::kind>;
        const size_t recBytes = static_cast<size_t>(c.nCells) * C::nip * R::size * sizeof(T);
        if (c.dRecords.n < recBytes)
            c.dRecords.alloc(recBytes);
        T* recs = reinterpret_cast<T*>(c.dRecords.p);
        constexpr int CPB = TangentShape<C::nd, C::nip>::cpb;
        const int blocks = static_cast<int>((c.nCells + CPB - 1) / CPB);
        // the law is evaluated in FP64 and rounded into FP32 records: the loading/unloading and damage-threshold
        // branches then agree with the FP64 residual's (an FP32 eeq or strain near kappa_h or kappa0 can take the
        // other branch and change the coupling blocks of the tangent by far more than a rounding error)
        k_tangent<double, C::dim, C::nd, C::nip, C::kind, true, T><<<blocks, TangentShape<C::nd, C::nip>::threads, 0,
                                                                     c.stream>>>(a, c.law, s, 0, 0, 0, 0, u, recs);
        AfterLaunch(c, "k_tangent (records)");
        auto kern = k_tangent_rows<T, C::dim, C::nd, C::nip, C::kind>;
        if (Sh::smem > 48 * 1024)
            NG_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         static_cast<int>(Sh::smem)));
        const int64_t rowBlocks = (r.nNodes + Sh::warps - 1) / Sh::warps;
        kern<<<static_cast<unsigned>(rowBlocks), Sh::warps * 32, Sh::smem, c.stream>>>(r, recs, vals);
        AfterLaunch(c, "k_tangent_rows");
    });
    c.stats.kernel_launches += 2;
}

// the allocating set-up of nuto_gpu_build_matrix_noalloc (defined with its static array below)
static void PrepareNoAlloc(Ctx& c);

template <typename T>
static void LaunchTangentT(Ctx& c, const double* u, T* vals)
{
    // FP32: row gather (no atomics). FP64: the element kernel; on GB300's FP64 pipe the per-lane recomputation of
    // the rank-1 factors in the row kernel costs more than the FP64 atomics it saves.
    if (sizeof(T) == 4 && RowsSupported(c) && !c.forceAtomicTangent)
    {
        // linear cells: node rows from per-point records; Hex20: element matrices on the tensor cores + row
        // gather; otherwise FP64-law records + row gather
        if (!c.forceRecordTangent && FusedTangentSupported(c))
            LaunchTangentFused(c, u, reinterpret_cast<float*>(vals));
        else if (!c.forceRecordTangent && Tc20TangentSupported(c))
            LaunchTangentTc20(c, u, reinterpret_cast<float*>(vals));
        else
            LaunchTangentRows<T>(c, u, vals);
        PrepareNoAlloc(c);
        return;
    }
    NG_CUDA(cudaMemsetAsync(vals, 0, c.nnz * sizeof(T), c.stream));
    CellArgs a = MakeCellArgs(c);
    ScatterArgs s = MakeScatterArgs(c);
    const int ns = static_cast<int>(c.slots.size());
    const int dS = c.prm.disp_slot;
    const int eS = c.prm.kind == NUTO_GPU_GRADIENT_DAMAGE ? c.prm.eeq_slot : dS;
    DispatchCfg(c, [&](auto cfg) {
        using C = decltype(cfg);
        constexpr int CPB = TangentShape<C::nd, C::nip>::cpb;
        const int blocks = static_cast<int>((c.nCells + CPB - 1) / CPB);
        k_tangent<T, C::dim, C::nd, C::nip, C::kind, false><<<blocks, TangentShape<C::nd, C::nip>::threads, 0, c.stream>>>(
                a, c.law, s, dS * ns + dS, dS * ns + eS, eS * ns + dS, eS * ns + eS, u, vals);
    });
    AfterLaunch(c, "k_tangent");
    c.stats.kernel_launches += 1;
}

// FP64-accurate tangent for the exact final phase of the FP32 path: the element kernel with FP64 law evaluation and
// double-float node-pair products (Hex8 and Quad4; the larger Hex20 blocks do not fit the shared memory of the
// split inputs and use the FP64 products)
void LaunchTangentExact(Ctx& c, const double* u, double* vals)
{
    c.valsVersion++;
    NG_CUDA(cudaMemsetAsync(vals, 0, c.nnz * sizeof(double), c.stream));
    CellArgs a = MakeCellArgs(c);
    ScatterArgs s = MakeScatterArgs(c);
    const int ns = static_cast<int>(c.slots.size());
    const int dS = c.prm.disp_slot;
    const int eS = c.prm.kind == NUTO_GPU_GRADIENT_DAMAGE ? c.prm.eeq_slot : dS;
    DispatchCfg(c, [&](auto cfg) {
        using C = decltype(cfg);
        constexpr int CPB = TangentShape<C::nd, C::nip>::cpb;
        const int blocks = static_cast<int>((c.nCells + CPB - 1) / CPB);
        constexpr bool df = C::nd <= 8;
        k_tangent<double, C::dim, C::nd, C::nip, C::kind, false, double, df>
                <<<blocks, TangentShape<C::nd, C::nip>::threads, 0, c.stream>>>(
                        a, c.law, s, dS * ns + dS, dS * ns + eS, eS * ns + dS, eS * ns + eS, u, vals);
    });
    AfterLaunch(c, "k_tangent exact");
    c.stats.kernel_launches += 1;
}

void LaunchTangent(Ctx& c, const double* u, int precision, void* values)
{
    c.valsVersion++;
    if (precision == NUTO_GPU_FP32)
        LaunchTangentT<float>(c, u, static_cast<float*>(values));
    else
        LaunchTangentT<double>(c, u, static_cast<double*>(values));
}

// ---- history update: GradientDamage::Update (GradientDamage.h:122-125), EvolutionImplicit::Update
// (LocalIsotropicDamage.h:130-133) -------------------------------------------------------------------------------
template <int DIM, int ND, int NIP, int KIND>
__global__ void __launch_bounds__(128) k_history(CellArgs a, LawParams L, const double* __restrict__ u)
{
    constexpr int VD = DIM == 2 ? 3 : 6;
    const int64_t n = a.nCells;
    const int64_t it = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
    if (it >= n * NIP)
        return;
    const int64_t e = it % n;
    const int q = static_cast<int>(it / n);
    double& kh = a.kappa[NG_IDX(e * NIP + q, n * NIP, 7)];
    if (KIND == NUTO_GPU_GRADIENT_DAMAGE)
    {
        double eeq = 0;
        for (int nd = 0; nd < ND; ++nd)
            eeq += a.tabN_D[q * ND + nd] *
                   u[NG_IDX(a.gdofE[NG_IDX(a.connE[static_cast<int64_t>(nd) * n + e], a.nNodesE, 4)], a.nDofs, 5)];
        kh = fmax(kh, eeq);
        return;
    }
    const double* G = a.geo64 + NG_IDX(static_cast<int64_t>(q) * a.geoStride * n + e, a.geoSize, 6);
    double H[DIM][DIM];
#pragma unroll
    for (int i = 0; i < DIM; ++i)
#pragma unroll
        for (int j = 0; j < DIM; ++j)
            H[i][j] = 0;
    for (int nd = 0; nd < ND; ++nd)
    {
        const int64_t g = a.gdofD[NG_IDX(a.connD[static_cast<int64_t>(nd) * n + e], a.nNodesD, 2)];
#pragma unroll
        for (int c = 0; c < DIM; ++c)
        {
            const double uc = u[NG_IDX(g + c, a.nDofs, 3)];
#pragma unroll
            for (int d = 0; d < DIM; ++d)
                H[c][d] += uc * G[(1 + nd * DIM + d) * n];
        }
    }
    double eps[VD];
    StrainFromH<double, DIM>(H, eps);
    kh = fmax(MisesValue<double, DIM>(L, eps), kh);
}

void LaunchHistory(Ctx& c, const double* u)
{
    if (c.prm.kind == NUTO_GPU_MB_LINEAR_ELASTIC)
        return;
    CellArgs a = MakeCellArgs(c);
    const int64_t items = c.nCells * c.ip.nIp;
    const int blocks = static_cast<int>((items + 127) / 128);
    DispatchCfg(c, [&](auto cfg) {
        using C = decltype(cfg);
        if constexpr (C::kind != NUTO_GPU_MB_LINEAR_ELASTIC)
            k_history<C::dim, C::nd, C::nip, C::kind><<<blocks, 128, 0, c.stream>>>(a, c.law, u);
    });
    AfterLaunch(c, "k_history");
    c.stats.kernel_launches += 1;
}

// ---- lumped mass: SimpleAssembler::BuildDiagonallyLumpedMatrix (SimpleAssembler.cpp:67-98) of
// DynamicMomentumBalance::Hessian2 (DynamicMomentumBalance.h:22-30) ---------------------------------------------
// One thread per cell. The cell block is rho N^T N det J w with N the component-interleaved shape matrix, so its
// diagonal entry of (node a, component c) is rho sum_q w det J N_a^2, its diagonal sum ncomp times the sum of those
// and its full sum ncomp rho sum_q w det J (sum_a N_a)^2; the lumped entry is diagonal * (full / diagonal sum) /
// ncomp, the reference's scaling (DofType::GetNum divides it by the component count).
template <int DIM, int ND, int NIP>
__global__ void __launch_bounds__(128) k_lumped_mass(CellArgs a, int ncomp, double rho, double* __restrict__ m)
{
    const int64_t n = a.nCells;
    const int64_t e = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
    if (e >= n)
        return;
    double diag[ND];
#pragma unroll
    for (int i = 0; i < ND; ++i)
        diag[i] = 0;
    double full = 0;
    for (int q = 0; q < NIP; ++q)
    {
        const double wdj = a.geo64[NG_IDX(static_cast<int64_t>(q) * a.geoStride * n + e, a.geoSize, 6)];
        double sumN = 0;
#pragma unroll
        for (int i = 0; i < ND; ++i)
        {
            const double Ni = a.tabN_D[q * ND + i];
            diag[i] += rho * Ni * Ni * wdj;
            sumN += Ni;
        }
        full += rho * sumN * sumN * wdj;
    }
    double diagSum = 0;
#pragma unroll
    for (int i = 0; i < ND; ++i)
        diagSum += diag[i];
    const double scale = ((ncomp * full) / (ncomp * diagSum)) / ncomp;
#pragma unroll
    for (int i = 0; i < ND; ++i)
    {
        const int64_t g = a.gdofD[NG_IDX(a.connD[static_cast<int64_t>(i) * n + e], a.nNodesD, 2)];
        for (int c = 0; c < ncomp; ++c)
            atomicAdd(m + NG_IDX(g + c, a.nDofs, 8), diag[i] * scale);
    }
}

void LaunchLumpedMass(Ctx& c, double rho, double* m)
{
    NG_CUDA(cudaMemsetAsync(m, 0, c.nDofs * sizeof(double), c.stream));
    CellArgs a = MakeCellArgs(c);
    const int ncomp = c.slots[c.prm.disp_slot].ncomp;
    const int blocks = static_cast<int>((c.nCells + 127) / 128);
    DispatchCfg(c, [&](auto cfg) {
        using C = decltype(cfg);
        k_lumped_mass<C::dim, C::nd, C::nip><<<blocks, 128, 0, c.stream>>>(a, ncomp, rho, m);
    });
    AfterLaunch(c, "k_lumped_mass");
    c.stats.kernel_launches += 1;
}

// ---- boundary loads: NeumannBc<D>::ExternalLoad (NeumannBc.h:28-36) summed by SimpleAssembler::BuildVector -------
// One thread per face: f(node, c) += N_node p_c det J w with the codimension-1 Jacobian (Jacobian.h:51-88):
// det J = |dx/dxi| for Line2 faces in 2D, |dx/dxi x dx/deta| for Quad4 faces in 3D.
struct FaceArgs
{
    int64_t nFaces, nCoord, nNodes, nDofs;
    const int32_t* coordConn; // planar [i][face]
    const int32_t* dofConn;
    const double* coords;
    const int64_t* gdof;
    int nq;
    double gp[3], gw[3];
    double p[3];
};

template <int DIM, int NFE>
__global__ void __launch_bounds__(128) k_external_load(FaceArgs A, double* __restrict__ f)
{
    const int64_t e = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
    if (e >= A.nFaces)
        return;
    double X[NFE][DIM];
#pragma unroll
    for (int i = 0; i < NFE; ++i)
    {
        const int32_t cn = A.coordConn[NG_IDX(static_cast<int64_t>(i) * A.nFaces + e, NFE * A.nFaces, 11)];
#pragma unroll
        for (int d = 0; d < DIM; ++d)
            X[i][d] = A.coords[NG_IDX(static_cast<int64_t>(cn) * DIM + d, A.nCoord * DIM, 12)];
    }
    double fe[NFE][DIM];
#pragma unroll
    for (int i = 0; i < NFE; ++i)
#pragma unroll
        for (int d = 0; d < DIM; ++d)
            fe[i][d] = 0;
    const int nq2 = DIM == 2 ? 1 : A.nq;
    for (int qb = 0; qb < nq2; ++qb)
        for (int qa = 0; qa < A.nq; ++qa)
        {
            // tensor Gauss point, first coordinate fastest (IntegrationTypeTensorProduct.cpp:28-38)
            const double r = A.gp[qa], t = DIM == 2 ? 0. : A.gp[qb];
            const double w = DIM == 2 ? A.gw[qa] : A.gw[qa] * A.gw[qb];
            double N[NFE], dN[NFE][2];
            if (NFE == 2)
            {
                N[0] = 0.5 * (1. - r);
                N[1] = 0.5 * (1. + r);
                dN[0][0] = -0.5;
                dN[1][0] = 0.5;
                dN[0][1] = dN[1][1] = 0;
            }
            else
            {
                const double sr[4] = {-1, 1, 1, -1}, ss[4] = {-1, -1, 1, 1};
#pragma unroll
                for (int i = 0; i < NFE; ++i)
                {
                    N[i] = 0.25 * (1. + sr[i] * r) * (1. + ss[i] * t);
                    dN[i][0] = 0.25 * sr[i] * (1. + ss[i] * t);
                    dN[i][1] = 0.25 * ss[i] * (1. + sr[i] * r);
                }
            }
            double J[DIM][2];
#pragma unroll
            for (int d = 0; d < DIM; ++d)
            {
                J[d][0] = J[d][1] = 0;
#pragma unroll
                for (int i = 0; i < NFE; ++i)
                {
                    J[d][0] += X[i][d] * dN[i][0];
                    J[d][1] += X[i][d] * dN[i][1];
                }
            }
            double detJ;
            if (DIM == 2)
                detJ = sqrt(J[0][0] * J[0][0] + J[1][0] * J[1][0]);
            else
            {
                const double c0 = J[1][0] * J[2 % DIM][1] - J[2 % DIM][0] * J[1][1];
                const double c1 = J[2 % DIM][0] * J[0][1] - J[0][0] * J[2 % DIM][1];
                const double c2 = J[0][0] * J[1][1] - J[1][0] * J[0][1];
                detJ = sqrt(c0 * c0 + c1 * c1 + c2 * c2);
            }
            const double fac = detJ * w;
#pragma unroll
            for (int i = 0; i < NFE; ++i)
#pragma unroll
                for (int d = 0; d < DIM; ++d)
                    fe[i][d] += N[i] * A.p[d] * fac;
        }
#pragma unroll
    for (int i = 0; i < NFE; ++i)
    {
        const int32_t dn = A.dofConn[NG_IDX(static_cast<int64_t>(i) * A.nFaces + e, NFE * A.nFaces, 13)];
        const int64_t g = A.gdof[NG_IDX(dn, A.nNodes, 14)];
#pragma unroll
        for (int d = 0; d < DIM; ++d)
            atomicAdd(f + NG_IDX(g + d, A.nDofs, 15), fe[i][d]);
    }
}

void LaunchExternalLoad(Ctx& c, const BoundaryGroup& B, const double* p, double* f)
{
    NG_CUDA(cudaMemsetAsync(f, 0, c.nDofs * sizeof(double), c.stream));
    const Slot& S = c.slots[B.slot];
    FaceArgs A{};
    A.nFaces = B.nFaces;
    A.nCoord = c.nCoord;
    A.nNodes = S.nNodes;
    A.nDofs = c.nDofs;
    A.coordConn = B.coordConnT.p;
    A.dofConn = B.dofConnT.p;
    A.coords = c.dCoords.p;
    A.gdof = S.dGdof.p;
    A.nq = B.nq;
    for (int i = 0; i < 3; ++i)
    {
        A.gp[i] = B.gp[i];
        A.gw[i] = B.gw[i];
        A.p[i] = i < c.dim ? p[i] : 0.;
    }
    const unsigned blocks = static_cast<unsigned>((B.nFaces + 127) / 128);
    if (c.dim == 2)
        k_external_load<2, 2><<<blocks, 128, 0, c.stream>>>(A, f);
    else
        k_external_load<3, 4><<<blocks, 128, 0, c.stream>>>(A, f);
    AfterLaunch(c, "k_external_load");
    c.stats.kernel_launches += 1;
}

// ---- integration-point values for post-processing: Cell::Eval (Cell.h:80-93) -----------------------------------
// One thread per (cell, point): strain from the cached FP64 geometry, kappa = max(kappa_h, eeq or eps_eq)
// (GradientDamage::Kappa, GradientDamage.h:127-130; EvolutionImplicit), omega(kappa), the law's stress.
// out[(cell * NIP + q) * width + r].
template <int DIM, int ND, int NIP, int KIND>
__global__ void __launch_bounds__(128) k_eval_ip(CellArgs a, LawParams L, const double* __restrict__ u, int quantity,
                                                 double* __restrict__ out)
{
    constexpr int VD = DIM == 2 ? 3 : 6;
    const int64_t n = a.nCells;
    const int64_t it = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
    if (it >= n * NIP)
        return;
    const int64_t e = it / NIP;
    const int q = static_cast<int>(it % NIP);
    const double* G = a.geo64 + NG_IDX(static_cast<int64_t>(q) * a.geoStride * n + e, a.geoSize, 6);
    double H[DIM][DIM];
#pragma unroll
    for (int i = 0; i < DIM; ++i)
#pragma unroll
        for (int j = 0; j < DIM; ++j)
            H[i][j] = 0;
    for (int nd = 0; nd < ND; ++nd)
    {
        const int64_t g = a.gdofD[NG_IDX(a.connD[static_cast<int64_t>(nd) * n + e], a.nNodesD, 2)];
#pragma unroll
        for (int c = 0; c < DIM; ++c)
        {
            const double uc = u[NG_IDX(g + c, a.nDofs, 3)];
#pragma unroll
            for (int d = 0; d < DIM; ++d)
                H[c][d] += uc * G[(1 + nd * DIM + d) * n];
        }
    }
    double eps[VD];
    StrainFromH<double, DIM>(H, eps);
    double eqs = 0;
    if (KIND == NUTO_GPU_GRADIENT_DAMAGE)
    {
        for (int nd = 0; nd < ND; ++nd)
            eqs += a.tabN_D[q * ND + nd] *
                   u[NG_IDX(a.gdofE[NG_IDX(a.connE[static_cast<int64_t>(nd) * n + e], a.nNodesE, 4)], a.nDofs, 5)];
    }
    else if (KIND == NUTO_GPU_MB_LOCAL_DAMAGE)
        eqs = MisesValue<double, DIM>(L, eps);
    const double kh = a.kappa[NG_IDX(e * NIP + q, n * NIP, 7)];
    const double kap = KIND == NUTO_GPU_MB_LINEAR_ELASTIC ? 0. : fmax(kh, eqs);
    const double omega = KIND == NUTO_GPU_MB_LINEAR_ELASTIC ? 0. : DamageOmega<double>(L, kap);
    const int w = (quantity == NUTO_GPU_IP_STRAIN || quantity == NUTO_GPU_IP_STRESS) ? VD : 1;
    double* o = out + it * w;
    if (quantity == NUTO_GPU_IP_KAPPA)
        o[0] = kap;
    else if (quantity == NUTO_GPU_IP_DAMAGE)
        o[0] = omega;
    else if (quantity == NUTO_GPU_IP_EEQ)
        o[0] = KIND == NUTO_GPU_MB_LINEAR_ELASTIC ? MisesValue<double, DIM>(L, eps) : eqs;
    else if (quantity == NUTO_GPU_IP_STRAIN)
    {
#pragma unroll
        for (int r = 0; r < VD; ++r)
            o[r] = eps[r];
    }
    else
    {
        double sig[VD];
        if (KIND == NUTO_GPU_MB_LINEAR_ELASTIC)
            ElasticStress<double, DIM>(L, eps, sig);
        else
            LedStress<double, DIM>(L, eps, omega, sig);
        const double se = a.escale ? a.escale[e] : 1.;
#pragma unroll
        for (int r = 0; r < VD; ++r)
            o[r] = sig[r] * se;
    }
}

int IpWidth(const Ctx& c, int quantity)
{
    return (quantity == NUTO_GPU_IP_STRAIN || quantity == NUTO_GPU_IP_STRESS) ? (c.dim == 2 ? 3 : 6) : 1;
}

void LaunchEvalIp(Ctx& c, const double* u, int quantity, double* out)
{
    CellArgs a = MakeCellArgs(c);
    const int64_t items = c.nCells * c.ip.nIp;
    const int blocks = static_cast<int>((items + 127) / 128);
    DispatchCfg(c, [&](auto cfg) {
        using C = decltype(cfg);
        k_eval_ip<C::dim, C::nd, C::nip, C::kind><<<blocks, 128, 0, c.stream>>>(a, c.law, u, quantity, out);
    });
    AfterLaunch(c, "k_eval_ip");
    c.stats.kernel_launches += 1;
}

// ---- scatter of caller-given cell results (SimpleAssembler scatter, SimpleAssembler.cpp:53-59, 118-137) -----
struct SlotView
{
    int ncomp, nen;
    int64_t localOffset;
    const int32_t* connT;
    const int64_t* gdof;
};

struct SlotViews
{
    int ns;
    int nLocal;
    int64_t nDofs;
    SlotView s[kMaxSlots];
};

static SlotViews MakeSlotViews(const Ctx& c)
{
    SlotViews v{};
    v.ns = static_cast<int>(c.slots.size());
    v.nDofs = c.nDofs;
    int off = 0;
    for (int i = 0; i < v.ns; ++i)
    {
        v.s[i].ncomp = c.slots[i].ncomp;
        v.s[i].nen = c.slots[i].nen;
        v.s[i].localOffset = off;
        v.s[i].connT = c.slots[i].dConnT.p;
        v.s[i].gdof = c.slots[i].dGdof.p;
        off += c.slots[i].ncomp * c.slots[i].nen;
    }
    v.nLocal = off;
    return v;
}

__device__ __forceinline__ void LocalToSlot(const SlotViews& v, int i, int& slot, int& node, int& comp)
{
    slot = 0;
    while (slot + 1 < v.ns && i >= v.s[slot + 1].localOffset)
        ++slot;
    const int r = i - static_cast<int>(v.s[slot].localOffset);
    node = r / v.s[slot].ncomp;
    comp = r % v.s[slot].ncomp;
}

__global__ void k_cell_vectors(int64_t nCells, SlotViews v, const double* __restrict__ fe, double* __restrict__ f)
{
    const int64_t it = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
    if (it >= nCells * v.nLocal)
        return;
    const int64_t e = it / v.nLocal;
    const int i = static_cast<int>(it % v.nLocal);
    int s, node, comp;
    LocalToSlot(v, i, s, node, comp);
    const int64_t g = v.s[s].gdof[v.s[s].connT[static_cast<int64_t>(node) * nCells + e]] + comp;
    atomicAdd(f + NG_IDX(g, v.nDofs, 14), fe[it]);
}

template <typename T>
__global__ void k_cell_matrices(int64_t nCells, SlotViews v, ScatterArgs S, const double* __restrict__ ke,
                                T* __restrict__ vals)
{
    const int64_t nl = v.nLocal;
    const int64_t it = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
    if (it >= nCells * nl * nl)
        return;
    const int64_t e = it / (nl * nl);
    const int i = static_cast<int>((it / nl) % nl), j = static_cast<int>(it % nl);
    int sI, nI, cI, sJ, nJ, cJ;
    LocalToSlot(v, i, sI, nI, cI);
    LocalToSlot(v, j, sJ, nJ, cJ);
    const int32_t aI = v.s[sI].connT[static_cast<int64_t>(nI) * nCells + e];
    const int64_t row = v.s[sI].gdof[aI] + cI;
    const int p = sI * v.ns + sJ;
    const int rank = S.rank[p][static_cast<int64_t>(nI * v.s[sJ].nen + nJ) * nCells + e];
    const int64_t pos = S.rowPtr[NG_IDX(row, S.nRows, 9)] + S.blk[p][aI] + v.s[sJ].ncomp * rank + cJ;
    atomicAdd(vals + NG_IDX(pos, S.nnz, 15), static_cast<T>(ke[it]));
}

void LaunchCellVectors(Ctx& c, const double* fe, double* f)
{
    NG_CUDA(cudaMemsetAsync(f, 0, c.nDofs * sizeof(double), c.stream));
    SlotViews v = MakeSlotViews(c);
    const int64_t items = c.nCells * v.nLocal;
    k_cell_vectors<<<static_cast<unsigned>((items + 255) / 256), 256, 0, c.stream>>>(c.nCells, v, fe, f);
    AfterLaunch(c, "k_cell_vectors");
}

void LaunchCellMatrices(Ctx& c, const double* ke, int precision, void* values)
{
    c.valsVersion++;
    SlotViews v = MakeSlotViews(c);
    ScatterArgs s = MakeScatterArgs(c);
    const int64_t items = c.nCells * v.nLocal * v.nLocal;
    const unsigned blocks = static_cast<unsigned>((items + 255) / 256);
    if (precision == NUTO_GPU_FP32)
    {
        NG_CUDA(cudaMemsetAsync(values, 0, c.nnz * sizeof(float), c.stream));
        k_cell_matrices<float><<<blocks, 256, 0, c.stream>>>(c.nCells, v, s, ke, static_cast<float*>(values));
    }
    else
    {
        NG_CUDA(cudaMemsetAsync(values, 0, c.nnz * sizeof(double), c.stream));
        k_cell_matrices<double><<<blocks, 256, 0, c.stream>>>(c.nCells, v, s, ke, static_cast<double*>(values));
    }
    AfterLaunch(c, "k_cell_matrices");
}

// ---- FP32 tangent without allocation (nuto_gpu_build_matrix_noalloc) --------------------------------------------
// The row-gather tangent with its integration-point records in a fixed device array of this file instead of the
// context's record buffer, so that the call allocates nothing. The array is shared by every context on a device:
// calls that may overlap (other streams, other host threads) must be serialised by the caller. Nothing in it has
// to start at zero: every record is written before it is read, and every CSR value is written once.
constexpr size_t kStaticRecordFloats = size_t(1) << 22; // 16 MiB
constexpr int kMaxDevices = 64;
static __device__ __align__(256) float g_staticRecords[kStaticRecordFloats];
static std::mutex g_staticRecordsMutex;
static float* g_staticRecordsPtr[kMaxDevices] = {};

// Address of the record array on the current device; looked up once per device (cudaGetSymbolAddress).
static float* StaticRecords(int device)
{
    std::lock_guard<std::mutex> lock(g_staticRecordsMutex);
    NG_CHECK(device >= 0 && device < kMaxDevices, NUTO_GPU_EINVAL, "device index out of range");
    if (!g_staticRecordsPtr[device])
    {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_staticRecords);
        if (e != cudaSuccess)
            throw Error{NUTO_GPU_ECUDA, std::string("cudaGetSymbolAddress(static records): ") + cudaGetErrorString(e)};
        g_staticRecordsPtr[device] = static_cast<float*>(p);
    }
    return g_staticRecordsPtr[device];
}

// Everything of the no-alloc path that may take device memory, done by the first FP32 nuto_gpu_build_matrix of a
// context (which may allocate): the static array's address on this device, and the two kernels of the path loaded.
// With lazy module loading (the CUDA default) a kernel's code is loaded, into device memory, at its first launch or
// attribute query; without this, the first no-alloc call would be that first launch.
static void PrepareNoAlloc(Ctx& c)
{
    if (c.noAllocReady || !c.haveGeo || c.rowsMode != 1)
        return;
    StaticRecords(c.device);
    DispatchCfg(c, [&](auto cfg) {
        using C = decltype(cfg);
        cudaFuncAttributes at{};
        NG_CUDA(cudaFuncGetAttributes(&at, k_tangent<double, C::dim, C::nd, C::nip, C::kind, true, float>));
        NG_CUDA(cudaFuncGetAttributes(&at, k_tangent_rows<float, C::dim, C::nd, C::nip, C::kind>));
    });
    c.noAllocReady = true;
}

void LaunchTangentNoAlloc(Ctx& c, const double* u, float* vals)
{
    NG_CHECK(c.haveGeo && c.rowsMode >= 0, NUTO_GPU_ESTATE,
             "nuto_gpu_build_matrix_noalloc: call nuto_gpu_build_matrix (FP32) once first; that call completes the "
             "set-up that allocates (integration-point geometry, record layout)");
    NG_CHECK(c.rowsMode == 1, NUTO_GPU_EINVAL,
             "nuto_gpu_build_matrix_noalloc: the row-gather tangent does not apply to this set-up (the displacement "
             "and eeq fields need the same interpolation)");
    c.valsVersion++;
    CellArgs a = MakeCellArgs(c);
    ScatterArgs s = MakeScatterArgs(c);
    RowArgs r = MakeRowArgs(c);
    DispatchCfg(c, [&](auto cfg) {
        using C = decltype(cfg);
        using R = IpRecord<C::dim, C::nd, C::kind>;
        using Sh = RowShape<float, C::dim, C::nd, C::nip, C::kind>;
        const size_t need = static_cast<size_t>(c.nCells) * C::nip * R::size;
        if (need > kStaticRecordFloats)
            throw Error{NUTO_GPU_EINVAL,
                        "nuto_gpu_build_matrix_noalloc: the records need " + std::to_string(need) +
                                " floats, the static array holds " + std::to_string(kStaticRecordFloats) + " (at most " +
                                std::to_string(kStaticRecordFloats / (C::nip * R::size)) +
                                " cells of this kind); use nuto_gpu_build_matrix"};
        float* recs = StaticRecords(c.device);
        constexpr int CPB = TangentShape<C::nd, C::nip>::cpb;
        const int blocks = static_cast<int>((c.nCells + CPB - 1) / CPB);
        k_tangent<double, C::dim, C::nd, C::nip, C::kind, true, float><<<blocks, TangentShape<C::nd, C::nip>::threads,
                                                                          0, c.stream>>>(a, c.law, s, 0, 0, 0, 0, u,
                                                                                         recs);
        AfterLaunch(c, "k_tangent (records, static)");
        auto kern = k_tangent_rows<float, C::dim, C::nd, C::nip, C::kind>;
        if (Sh::smem > 48 * 1024)
            NG_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         static_cast<int>(Sh::smem)));
        const int64_t rowBlocks = (r.nNodes + Sh::warps - 1) / Sh::warps;
        kern<<<static_cast<unsigned>(rowBlocks), Sh::warps * 32, Sh::smem, c.stream>>>(r, recs, vals);
        AfterLaunch(c, "k_tangent_rows (static records)");
    });
    c.stats.kernel_launches += 2;
}

} // namespace nuto_gpu
