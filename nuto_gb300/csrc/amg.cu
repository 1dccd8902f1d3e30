// Aggregation multigrid preconditioner for the Krylov solvers. The reference has no iterative solver on this
// path (it factorises the matrix, EigenSparseSolve.cpp:22-73); this is the GB300-side replacement of that
// factorisation inside the Newton loop.
//
// Structure: one hierarchy per DOF slot (displacements, nonlocal equivalent strains), applied as one block
// Gauss-Seidel sweep in slot order: z_0 = V_0(v_0), z_1 = V_1(v_1 - K_10 z_0). For gradient damage K_10 (the
// dependence of the eeq equation on the local strain) is the strong coupling and K_01 vanishes outside the
// damaging zone, so the sweep is exact there up to the V-cycles.
//
// Hierarchy (host, once per pattern): the DOF nodes of a slot are grouped into aggregates by spatial binning.
// The bins start at one cell extent per axis and grow per level by doubling the axes that are shorter than the
// longest by more than half (all axes when none is), so stretched cells (the 1 x 1 x 4 beam) first coarsen across
// their short sides. Levels stop at kCoarsest nodes. Transfer is piecewise constant per component; constrained
// DOFs take part in neither restriction nor prolongation. Coarse operators keep the node-block CSR layout, so the
// node SpMV serves every level; level 0 is a diagonal-block view of the tangent itself.
//
// Per tangent (device, in the arithmetic of the tangent: FP32 or FP64): Galerkin coarse values A_c = P^T A P by
// one pass over the finer values with atomics; Jacobi diagonals and Gershgorin bounds of D^-1 A per level. Cycle: V(1,2) with Chebyshev-Jacobi
// smoothing on [lmax / 10, lmax] and a degree-6 Chebyshev solve on the coarsest level. The sweep is a fixed
// linear operator; GMRES uses it in flexible form (stored preconditioned basis) so rounding inside the cycle does
// not limit the attainable residual.
#include "spmv.cuh"

#include <algorithm>
#include <cstdlib>
#include <numeric>
#include <unordered_map>

namespace nuto_gpu
{

constexpr int kCoarsest = 64; // nodes on the coarsest level
constexpr int kMaxLevels = 12;
constexpr int kPreDegree = 1;
constexpr int kPostDegree = 2;
// Chebyshev degree on the coarsest level, per arithmetic of the cycle: measured on the damaged 64^3 tangent
// (time to a 1e-4 / 1e-7 relative residual), degree 10 made the FP32 cycle 10 % faster than degree 6 and the FP64
// cycle 3 % faster / 7 % slower
template <typename TA>
constexpr int CoarseDegree()
{
    return sizeof(TA) == 4 ? 10 : 6;
}
constexpr float kSmoothRatio = 10.f; // smoothing interval [lmax / ratio, lmax]
constexpr float kCoarseRatio = 30.f;

// vectors and coarse values of one level in the preconditioner's arithmetic TA (FP32 for FP32 tangents, FP64 for
// the plain FP64 path); on level 0 the vectors span the combined system and vals is unused (the tangent is used)
template <typename TA>
struct Num
{
    DBuf<TA> vals, dinv, e, b, t, d;
    DBuf<TA> nb; // coarse levels: the values in the padded layout of the level's SpMV
};

struct AmgLevel
{
    int ncomp = 1;
    int64_t nNodes = 0;
    int64_t nDofs = 0, nnz = 0;
    // level-0 views address the combined vectors: rows [off, off + nDofs) of the slot
    int64_t off = 0;
    std::vector<int64_t> hNbrPtr;
    std::vector<int32_t> hNbrIdx;
    std::vector<double> hCoords; // 3 per node
    // device structure of coarse levels (level 0 uses the context's pattern)
    DBuf<int64_t> gdof, rowPtr, nbrPtr;
    DBuf<int32_t> nbrIdx, nbrCol, blk;
    DBuf<int32_t> diagOff;  // per node: offset of the diagonal block in the node's row segment
    DBuf<int64_t> nbBase;   // coarse levels: per node, first value of the node's block in the padded layout
    int64_t nbTotal = 0;
    int nbSeg4 = 0;
    DBuf<uint8_t> zeroMask; // coarse levels have no constrained rows
    // transfer from the finer level
    DBuf<int32_t> aggOf;   // finer node -> node of this level
    DBuf<uint16_t> cRank;  // finer neighbour entry -> rank in this level's neighbour list
    // numerics, per arithmetic of the preconditioner (allocated on first use of that arithmetic)
    Num<float> n32;
    Num<double> n64;
    float lmax = 1.f;
    NodeSpmv spmv{};
};

template <typename TA>
static Num<TA>& N(AmgLevel& L);
template <>
Num<float>& N<float>(AmgLevel& L)
{
    return L.n32;
}
template <>
Num<double>& N<double>(AmgLevel& L)
{
    return L.n64;
}

// One sweep (all launches of both V-cycles) captured as a CUDA graph on fixed input/output vectors. The graph is
// recaptured after every set-up (the Chebyshev coefficients are kernel arguments) and the executable graph updated
// in place (same topology), so a sweep costs one launch on the host instead of about 150.
struct SweepGraph
{
    cudaGraphExec_t exec = nullptr;
    uint64_t setup = 0;      // set-up counter the graph was captured for
    const int* st = nullptr; // Krylov state pointer baked into the graph
    int64_t launches = 0;    // kernels per replay
};

struct Amg
{
    int ns = 0;
    std::vector<AmgLevel> h[kMaxSlots];
    DBuf<float> lmaxDev; // all levels of all hierarchies
    std::vector<float> lmaxHost;
    DBuf<float> in32, out32, res32; // combined-length work vectors of the sweep (FP32 cycle)
    DBuf<double> in64, out64, res64; // the same for the FP64 cycle
    int prec = 32;                   // arithmetic of the last set-up: that of the tangent values
    const void* fine = nullptr;      // the tangent of the last set-up (level-0 operator)
    const void* setupVals = nullptr;
    uint64_t setupVersion = 0;
    uint64_t setups = 0; // set-ups so far
    bool built = false;
    bool graphs = true;           // NUTO_GPU_GRAPHS=0 launches the sweep kernel by kernel
    SweepGraph graph[2][2];       // [FP64][symmetric]
    ~Amg()
    {
        for (auto& row : graph)
            for (SweepGraph& g : row)
                if (g.exec)
                    cudaGraphExecDestroy(g.exec);
        if (capStream)
            cudaStreamDestroy(capStream);
    }
    bool graphLaunched = false;    // a sweep graph was launched since the hierarchy was built
    std::string graphError; // why graphs were switched off (diagnostics)
    cudaStream_t capStream = nullptr; // private stream for graph capture (the context's may be the legacy stream)
};

void FreeAmg(Ctx& c)
{
    delete c.amg;
    c.amg = nullptr;
}

// ---- host: hierarchy -------------------------------------------------------------------------------------------
// natural coordinates of the local nodes (InterpolationQuadLinear / BrickLinear / BrickQuadratic order)
static void LocalNodeCoords(int interp, int n, double* xi)
{
    static const double h20[20][3] = {{-1, -1, -1}, {1, -1, -1}, {1, 1, -1}, {-1, 1, -1}, {-1, -1, 1}, {1, -1, 1},
                                      {1, 1, 1},    {-1, 1, 1},  {0, -1, -1}, {1, 0, -1},  {0, 1, -1},  {-1, 0, -1},
                                      {-1, -1, 0},  {1, -1, 0},  {1, 1, 0},   {-1, 1, 0},  {0, -1, 1},  {1, 0, 1},
                                      {0, 1, 1},    {-1, 0, 1}};
    static const double q4[4][2] = {{-1, -1}, {1, -1}, {1, 1}, {-1, 1}};
    if (interp == NUTO_GPU_QUAD4)
    {
        xi[0] = q4[n][0];
        xi[1] = q4[n][1];
        xi[2] = 0;
        return;
    }
    for (int d = 0; d < 3; ++d)
        xi[d] = h20[n][d];
}

// shape functions of the coordinate element (Quad4 / Hex8) at a natural point
static void GeoShape(int geo, const double* xi, double* N)
{
    if (geo == NUTO_GPU_QUAD4)
    {
        const double r = xi[0], s = xi[1];
        N[0] = 0.25 * (1 - r) * (1 - s);
        N[1] = 0.25 * (1 + r) * (1 - s);
        N[2] = 0.25 * (1 + r) * (1 + s);
        N[3] = 0.25 * (1 - r) * (1 + s);
        return;
    }
    const int sg[8][3] = {{-1, -1, -1}, {1, -1, -1}, {1, 1, -1}, {-1, 1, -1},
                          {-1, -1, 1},  {1, -1, 1},  {1, 1, 1},  {-1, 1, 1}};
    for (int i = 0; i < 8; ++i)
        N[i] = 0.125 * (1 + sg[i][0] * xi[0]) * (1 + sg[i][1] * xi[1]) * (1 + sg[i][2] * xi[2]);
}

// per node: offset of the node's own block inside its neighbour segment
static std::vector<int32_t> DiagOffsets(const std::vector<int64_t>& ptr, const std::vector<int32_t>& idx, int ncomp)
{
    const int64_t n = static_cast<int64_t>(ptr.size()) - 1;
    std::vector<int32_t> off(n, 0);
    for (int64_t a = 0; a < n; ++a)
    {
        const int32_t* first = idx.data() + ptr[a];
        const int32_t* last = idx.data() + ptr[a + 1];
        const int32_t* it = std::find(first, last, static_cast<int32_t>(a));
        NG_CHECK(it != last, NUTO_GPU_EINVAL, "a node is missing from its own neighbour list");
        off[a] = static_cast<int32_t>(ncomp * (it - first));
    }
    return off;
}

template <typename T>
static void UploadV(DBuf<T>& buf, const std::vector<T>& h)
{
    buf.alloc(h.size());
    if (!h.empty())
        NG_CUDA(cudaMemcpy(buf.p, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice));
}

// single-slot NodeSpmv of a coarse level
static void FillSpmv(AmgLevel& L)
{
    NodeSpmv& A = L.spmv;
    A = NodeSpmv{};
    A.ns = 1;
    A.ncomp[0] = L.ncomp;
    A.nNodes[0] = L.nNodes;
    A.firstWarp[0] = 0;
    A.totalWarps = L.nNodes;
    A.gdof[0] = L.gdof.p;
    A.nbrPtr[0] = L.nbrPtr.p;
    A.nbrIdx[0] = L.nbrIdx.p;
    A.nbrCol[0] = L.nbrCol.p;
    A.blk[0] = L.blk.p;
    A.nbrTotal[0] = static_cast<int64_t>(L.nbrIdx.n);
    A.rowPtr = L.rowPtr.p;
    A.nnz = L.nnz;
    A.nRows = L.nDofs;
}

// diagonal-block view of slot I of the context's tangent
static NodeSpmv SlotView(const Ctx& c, int I)
{
    const int ns = static_cast<int>(c.slots.size());
    const PairMap& M = c.pairs[I * ns + I];
    NodeSpmv A{};
    A.ns = 1;
    A.ncomp[0] = c.slots[I].ncomp;
    A.nNodes[0] = c.slots[I].nNodes;
    A.firstWarp[0] = 0;
    A.totalWarps = c.slots[I].nNodes;
    A.gdof[0] = c.slots[I].dGdof.p;
    A.nbrPtr[0] = M.dNbrPtr.p;
    A.nbrIdx[0] = M.dNbrIdx.p;
    A.nbrCol[0] = M.dNbrCol.p;
    A.blk[0] = M.dBlk.p;
    A.nbrTotal[0] = static_cast<int64_t>(M.dNbrIdx.n);
    A.rowPtr = c.dRowPtr.p;
    A.nnz = c.nnz;
    A.nRows = c.nDofs;
    if (c.nb.total > 0)
    {
        A.nbBase[0] = c.nb.pair[I * ns + I].base.p;
        A.nbOff[0] = c.nb.pair[I * ns + I].off;
        A.nbSeg4 = c.nb.pair[I * ns + I].maxSeg4;
        A.ncMaxRows = c.slots[I].ncomp;
        A.nb32 = c.nb.v32.p;
        A.nb64 = c.nb.v64.p;
        A.nbSrc32 = c.nb.src32;
        A.nbSrc64 = c.nb.src64;
    }
    return A;
}

// whole-row operator restricted to the rows of slot I (K_I0 z_0 + K_II z_I, used with z_I = 0)
static NodeSpmv RowsView(const Ctx& c, int I)
{
    NodeSpmv A = MakeNodeSpmv(c);
    if (I == 1)
    {
        A.firstWarp[1] = 0;
        A.totalWarps = A.nNodes[1];
    }
    else
        A.totalWarps = A.nNodes[0];
    return A;
}

static void GrowBins(double* bin, int dim)
{
    double mx = 0;
    for (int d = 0; d < dim; ++d)
        mx = std::max(mx, bin[d]);
    bool any = false;
    for (int d = 0; d < dim; ++d)
        any = any || bin[d] * 1.5 < mx;
    for (int d = 0; d < dim; ++d)
        if (!any || bin[d] * 1.5 < mx)
            bin[d] *= 2.0;
}

static void BuildSlotHierarchy(Ctx& c, int I, const double* ext, std::vector<AmgLevel>& H)
{
    const int ns = static_cast<int>(c.slots.size());
    const Slot& S = c.slots[I];
    H.clear();
    H.emplace_back();
    {
        AmgLevel& F = H[0];
        F.ncomp = S.ncomp;
        F.nNodes = S.nNodes;
        F.nDofs = S.nDofs;
        F.off = S.offset;
        F.hNbrPtr = c.pairs[I * ns + I].hNbrPtr;
        F.hNbrIdx = c.pairs[I * ns + I].hNbrIdx;
        // DOF-node coordinates: the coordinate element interpolated at the node's natural coordinates
        F.hCoords.assign(S.nNodes * 3, 0.);
        std::vector<char> done(S.nNodes, 0);
        for (int64_t e = 0; e < c.nCells; ++e)
            for (int n = 0; n < S.nen; ++n)
            {
                const int32_t node = S.conn[e * S.nen + n];
                if (done[node])
                    continue;
                done[node] = 1;
                double xi[3], N[8];
                LocalNodeCoords(S.interp, n, xi);
                GeoShape(c.geoInterp, xi, N);
                for (int d = 0; d < c.dim; ++d)
                {
                    double v = 0;
                    for (int g = 0; g < c.nge; ++g)
                        v += N[g] * c.hCoords[static_cast<size_t>(c.hGeoConn[e * c.nge + g]) * c.dim + d];
                    F.hCoords[node * 3 + d] = v;
                }
            }
        UploadV(F.diagOff, DiagOffsets(F.hNbrPtr, F.hNbrIdx, F.ncomp));
        F.spmv = SlotView(c, I);
    }
    double lo[3] = {1e300, 1e300, 1e300};
    for (int64_t a = 0; a < H[0].nNodes; ++a)
        for (int d = 0; d < 3; ++d)
            lo[d] = std::min(lo[d], H[0].hCoords[a * 3 + d]);
    double bin[3] = {ext[0], ext[1], ext[2]};
    GrowBins(bin, c.dim);

    for (int level = 1; level < kMaxLevels; ++level)
    {
        AmgLevel& Fi = H[level - 1];
        if (Fi.nNodes <= kCoarsest)
            break;
        AmgLevel C;
        C.ncomp = Fi.ncomp;
        std::unordered_map<int64_t, int32_t> keyToAgg;
        keyToAgg.reserve(Fi.nNodes / 4 + 16);
        std::vector<int32_t> agg(Fi.nNodes, -1);
        std::vector<double> sum;
        std::vector<int64_t> cnt;
        for (int64_t a = 0; a < Fi.nNodes; ++a)
        {
            int64_t key = 0;
            for (int d = 0; d < 3; ++d)
            {
                const double x = (Fi.hCoords[a * 3 + d] - lo[d]) / (d < c.dim ? bin[d] : 1.0);
                key = key * 2097152 + static_cast<int64_t>(std::floor(x + 1e-9));
            }
            auto it = keyToAgg.find(key);
            int32_t A;
            if (it == keyToAgg.end())
            {
                A = static_cast<int32_t>(keyToAgg.size());
                keyToAgg.emplace(key, A);
                sum.insert(sum.end(), {0., 0., 0.});
                cnt.push_back(0);
            }
            else
                A = it->second;
            agg[a] = A;
            for (int d = 0; d < 3; ++d)
                sum[A * 3 + d] += Fi.hCoords[a * 3 + d];
            cnt[A]++;
        }
        C.nNodes = static_cast<int64_t>(cnt.size());
        if (C.nNodes * 5 >= Fi.nNodes * 4)
            break; // the bins no longer merge nodes
        C.hCoords.resize(cnt.size() * 3);
        for (size_t A = 0; A < cnt.size(); ++A)
            for (int d = 0; d < 3; ++d)
                C.hCoords[A * 3 + d] = sum[A * 3 + d] / cnt[A];
        // members of every aggregate
        std::vector<int64_t> mptr(C.nNodes + 1, 0);
        for (int64_t a = 0; a < Fi.nNodes; ++a)
            mptr[agg[a] + 1]++;
        for (int64_t A = 0; A < C.nNodes; ++A)
            mptr[A + 1] += mptr[A];
        std::vector<int64_t> fill(mptr.begin(), mptr.end() - 1);
        std::vector<int32_t> mem(Fi.nNodes);
        for (int64_t a = 0; a < Fi.nNodes; ++a)
            mem[fill[agg[a]]++] = static_cast<int32_t>(a);
        // coarse neighbour lists (sorted by node index = DOF order on coarse levels)
        std::vector<std::vector<int32_t>> lists(C.nNodes);
#pragma omp parallel for schedule(dynamic, 256)
        for (int64_t A = 0; A < C.nNodes; ++A)
        {
            auto& v = lists[A];
            for (int64_t m = mptr[A]; m < mptr[A + 1]; ++m)
            {
                const int32_t a = mem[m];
                for (int64_t q = Fi.hNbrPtr[a]; q < Fi.hNbrPtr[a + 1]; ++q)
                    v.push_back(agg[Fi.hNbrIdx[q]]);
            }
            std::sort(v.begin(), v.end());
            v.erase(std::unique(v.begin(), v.end()), v.end());
        }
        C.hNbrPtr.assign(C.nNodes + 1, 0);
        int64_t maxLen = 0;
        for (int64_t A = 0; A < C.nNodes; ++A)
        {
            C.hNbrPtr[A + 1] = C.hNbrPtr[A] + static_cast<int64_t>(lists[A].size());
            maxLen = std::max(maxLen, static_cast<int64_t>(lists[A].size()) * C.ncomp);
        }
        if (maxLen > kMaxRowLen)
            break; // a denser coarse stencil than the SpMV supports: keep the finer level as the coarsest
        C.hNbrIdx.resize(C.hNbrPtr.back());
        for (int64_t A = 0; A < C.nNodes; ++A)
            std::copy(lists[A].begin(), lists[A].end(), C.hNbrIdx.begin() + C.hNbrPtr[A]);
        // rank of every finer neighbour entry in the coarse list of its aggregate
        std::vector<uint16_t> cr(Fi.hNbrIdx.size());
#pragma omp parallel for schedule(static)
        for (int64_t a = 0; a < Fi.nNodes; ++a)
        {
            const int32_t A = agg[a];
            const int32_t* first = C.hNbrIdx.data() + C.hNbrPtr[A];
            const int32_t* last = C.hNbrIdx.data() + C.hNbrPtr[A + 1];
            for (int64_t q = Fi.hNbrPtr[a]; q < Fi.hNbrPtr[a + 1]; ++q)
                cr[q] = static_cast<uint16_t>(std::lower_bound(first, last, agg[Fi.hNbrIdx[q]]) - first);
        }
        // node-block CSR of the coarse level
        C.nDofs = C.nNodes * C.ncomp;
        std::vector<int64_t> rowPtr(C.nDofs + 1, 0), gdof(C.nNodes);
        std::vector<int32_t> blk(C.nNodes, 0);
        for (int64_t A = 0; A < C.nNodes; ++A)
        {
            gdof[A] = A * C.ncomp;
            const int64_t len = C.ncomp * (C.hNbrPtr[A + 1] - C.hNbrPtr[A]);
            for (int k = 0; k < C.ncomp; ++k)
                rowPtr[A * C.ncomp + k + 1] = len;
        }
        for (int64_t r = 0; r < C.nDofs; ++r)
            rowPtr[r + 1] += rowPtr[r];
        C.nnz = rowPtr.back();
        UploadV(C.rowPtr, rowPtr);
        UploadV(C.gdof, gdof);
        UploadV(C.blk, blk);
        UploadV(C.nbrPtr, C.hNbrPtr);
        UploadV(C.nbrIdx, C.hNbrIdx);
        {
            std::vector<int32_t> col(C.hNbrIdx.size());
            for (size_t q = 0; q < col.size(); ++q)
                col[q] = C.hNbrIdx[q] * C.ncomp;
            UploadV(C.nbrCol, col);
        }
        UploadV(C.diagOff, DiagOffsets(C.hNbrPtr, C.hNbrIdx, C.ncomp));
        {
            // padded layout of the level: per node ncomp rows of ncomp * nn values, padded to multiples of 4
            std::vector<int64_t> base(C.nNodes);
            int64_t pos = 0;
            int mx = 0;
            for (int64_t A = 0; A < C.nNodes; ++A)
            {
                const int seg4 = static_cast<int>((C.ncomp * (C.hNbrPtr[A + 1] - C.hNbrPtr[A]) + 3) / 4 * 4);
                base[A] = pos;
                pos += static_cast<int64_t>(C.ncomp) * seg4;
                mx = std::max(mx, seg4);
            }
            UploadV(C.nbBase, base);
            C.nbTotal = pos;
            C.nbSeg4 = mx;
        }
        UploadV(C.aggOf, agg);
        UploadV(C.cRank, cr);
        C.zeroMask.alloc(C.nDofs);
        NG_CUDA(cudaMemset(C.zeroMask.p, 0, C.nDofs));
        FillSpmv(C);
        H.push_back(std::move(C));
        GrowBins(bin, c.dim);
    }
    H[0].nnz = c.nnz;
}

static void BuildHierarchy(Ctx& c)
{
    Amg& M = *c.amg;
    M.ns = static_cast<int>(c.slots.size());
    // median cell extent per axis (every 7th cell)
    double ext[3] = {1, 1, 1};
    for (int d = 0; d < c.dim; ++d)
    {
        std::vector<double> v;
        for (int64_t e = 0; e < c.nCells; e += 7)
        {
            double lo = 1e300, hi = -1e300;
            for (int g = 0; g < c.nge; ++g)
            {
                const double x = c.hCoords[static_cast<size_t>(c.hGeoConn[e * c.nge + g]) * c.dim + d];
                lo = std::min(lo, x);
                hi = std::max(hi, x);
            }
            v.push_back(hi - lo);
        }
        std::nth_element(v.begin(), v.begin() + v.size() / 2, v.end());
        ext[d] = v[v.size() / 2];
        NG_CHECK(ext[d] > 0, NUTO_GPU_EINVAL, "degenerate cells");
    }
    size_t total = 0;
    for (int I = 0; I < M.ns; ++I)
    {
        BuildSlotHierarchy(c, I, ext, M.h[I]);
        total += M.h[I].size();
    }
    M.lmaxDev.alloc(total);
    M.lmaxHost.assign(total, 0.f);
    M.setupVals = nullptr;
    M.built = true;
}

// ---- device: per-tangent set-up -----------------------------------------------------------------------------------
// Galerkin coarse values: one warp per finer node adds its (unconstrained) rows into the aggregate's rows
template <typename TA>
__global__ void __launch_bounds__(kBS) k_amg_coarsen(NodeSpmv F, const uint8_t* __restrict__ fmask,
                                                      const TA* __restrict__ fv, NodeSpmv C,
                                                      const int32_t* __restrict__ agg, const uint16_t* __restrict__ cr,
                                                      TA* cv)
{
    const int64_t a = (blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (a >= F.totalWarps)
        return;
    const int32_t A = agg[a];
    const int nc = F.ncomp[0];
    const int64_t g0 = F.gdof[0][a];
    const int64_t G0 = C.gdof[0][NG_IDX(A, C.nNodes[0], 31)];
    const int64_t q0 = F.nbrPtr[0][a];
    const int nn = static_cast<int>(F.nbrPtr[0][a + 1] - q0);
    for (int c = 0; c < nc; ++c)
    {
        if (fmask[g0 + c])
            continue;
        const int64_t off = F.rowPtr[g0 + c] + F.blk[0][a];
        const int64_t OFF = C.rowPtr[G0 + c];
        for (int k = lane; k < nn; k += 32)
        {
            const int64_t gb = F.gdof[0][F.nbrIdx[0][q0 + k]];
            const int64_t base = OFF + static_cast<int64_t>(nc) * cr[q0 + k];
            for (int d = 0; d < nc; ++d)
                if (!fmask[gb + d])
                    atomicAdd(cv + NG_IDX(base + d, C.nnz, 30), fv[off + nc * k + d]);
        }
    }
}

// Jacobi diagonal (0 where the DOF is constrained or the diagonal is not positive) and the Gershgorin bound
// max_r sum_j |a_rj| / a_rr of the spectral radius of D^-1 A (positive floats order like their bit patterns)
template <typename TA>
__global__ void __launch_bounds__(kBS) k_amg_diag(NodeSpmv A, const uint8_t* __restrict__ mask,
                                                   const TA* __restrict__ v, const int32_t* __restrict__ diagOff,
                                                   TA* dinv, float* lmax)
{
    const int64_t a = (blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (a >= A.totalWarps)
        return;
    const int nc = A.ncomp[0];
    const int64_t g0 = A.gdof[0][a];
    const int len = nc * static_cast<int>(A.nbrPtr[0][a + 1] - A.nbrPtr[0][a]);
    for (int c = 0; c < nc; ++c)
    {
        const int64_t r = g0 + c;
        const int64_t rs = A.rowPtr[r] + A.blk[0][a];
        float s = 0.f;
        for (int q = lane; q < len; q += 32)
            s += fabsf(static_cast<float>(v[NG_IDX(rs + q, A.nnz, 32)]));
#pragma unroll
        for (int o = 16; o > 0; o >>= 1)
            s += __shfl_down_sync(0xffffffffu, s, o);
        if (lane == 0)
        {
            const TA dg = v[NG_IDX(rs + diagOff[a] + c, A.nnz, 35)];
            const bool use = !mask[r] && dg > TA(0);
            dinv[r] = use ? TA(1) / dg : TA(0);
            if (use)
                atomicMax(reinterpret_cast<int*>(lmax), __float_as_int(s / static_cast<float>(dg)));
        }
    }
}

// ---- device: cycle kernels (each returns at once when the Krylov state is no longer RUN) ------------------------
__device__ __forceinline__ bool Idle(const int* st)
{
    return st && st[ST_STATE] != RUN;
}

// first Chebyshev step from zero: d = dinv b / theta; e = d
template <typename TA>
__global__ void k_cheb0(int64_t n, const TA* __restrict__ dinv, const TA* __restrict__ b, TA* d, TA* e, TA invTheta,
                        const int* st)
{
    PdlWait();
    PdlTrigger();
    const int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
    if (i >= n || Idle(st))
        return;
    const TA v = dinv[i] * b[i] * invTheta;
    d[i] = v;
    e[i] = v;
}

// first Chebyshev step from a nonzero e (t = A e): d = dinv (b - t) / theta; e += d
template <typename TA>
__global__ void k_cheb1(int64_t n, const TA* __restrict__ dinv, const TA* __restrict__ b, const TA* __restrict__ t,
                        TA* d, TA* e, TA invTheta, const int* st)
{
    PdlWait();
    PdlTrigger();
    const int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
    if (i >= n || Idle(st))
        return;
    const TA v = dinv[i] * (b[i] - t[i]) * invTheta;
    d[i] = v;
    e[i] += v;
}

// later Chebyshev steps (t = A e): d = c1 d + c2 dinv (b - t); e += d
template <typename TA>
__global__ void k_chebk(int64_t n, const TA* __restrict__ dinv, const TA* __restrict__ b, const TA* __restrict__ t,
                        TA* d, TA* e, TA c1, TA c2, const int* st)
{
    PdlWait();
    PdlTrigger();
    const int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
    if (i >= n || Idle(st))
        return;
    const TA v = c1 * d[i] + c2 * dinv[i] * (b[i] - t[i]);
    d[i] = v;
    e[i] += v;
}

// coarse b = P^T (b - t) with t = A e (cb zeroed before); constrained finer DOFs are skipped
template <typename TA>
__global__ void k_restrict(NodeSpmv F, const uint8_t* __restrict__ fmask, const TA* __restrict__ b,
                           const TA* __restrict__ t, const int32_t* __restrict__ agg, NodeSpmv C, TA* cb,
                           const int* st)
{
    PdlWait();
    PdlTrigger();
    const int64_t a = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
    if (a >= F.totalWarps || Idle(st))
        return;
    const int64_t g0 = F.gdof[0][a];
    const int64_t G0 = C.gdof[0][agg[a]];
    for (int c = 0; c < F.ncomp[0]; ++c)
        if (!fmask[g0 + c])
            atomicAdd(cb + NG_IDX(G0 + c, C.nRows, 33), b[g0 + c] - t[g0 + c]);
}

// e += P ce
template <typename TA>
__global__ void k_prolong(NodeSpmv F, const uint8_t* __restrict__ fmask, const int32_t* __restrict__ agg, NodeSpmv C,
                          const TA* __restrict__ ce, TA* e, const int* st)
{
    PdlWait();
    PdlTrigger();
    const int64_t a = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
    if (a >= F.totalWarps || Idle(st))
        return;
    const int64_t g0 = F.gdof[0][a];
    const int64_t G0 = C.gdof[0][agg[a]];
    for (int c = 0; c < F.ncomp[0]; ++c)
        if (!fmask[g0 + c])
            e[g0 + c] += ce[NG_IDX(G0 + c, C.nRows, 34)];
}

// y = a - b (elementwise); a == nullptr gives y = 0
template <typename TA>
__global__ void k_sub(int64_t n, const TA* a, const TA* b, TA* y, const int* st)
{
    PdlWait();
    PdlTrigger();
    const int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
    if (i >= n || Idle(st))
        return;
    y[i] = a ? a[i] - b[i] : TA(0);
}

template <typename TA, typename TB>
__global__ void k_convert(int64_t n, const TA* __restrict__ a, TB* __restrict__ b, const int* st)
{
    PdlWait();
    PdlTrigger();
    const int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
    if (i < n && !Idle(st))
        b[i] = static_cast<TB>(a[i]);
}

// ---- device: the coarsest levels in one block ----------------------------------------------------------------
// Levels with at most kTailNodes nodes (and every coarser one) do microseconds of work per launch; run as separate
// launches they cost about 29 launches per slot and cycle. One block of kTailThreads threads runs their whole
// V-cycle instead: the same Chebyshev recurrences (coefficients from the same double-precision formulas), the same
// restriction and prolongation, and a warp-per-node product on the coarse node-block CSR, with block barriers
// between the steps. The level vectors stay in global memory (L2-resident at these sizes).
constexpr int kTailNodes = 128;
constexpr int kTailMax = 8;
constexpr int kTailThreads = 1024;

template <typename TA>
struct TailLevel
{
    const int64_t* rowPtr;
    const int64_t* nbrPtr;
    const int32_t* nbrCol;
    const int32_t* agg; // this level's nodes -> nodes of the next coarser level (unused on the coarsest)
    const TA* vals;
    const TA* dinv;
    TA *b, *e, *t, *d;
    int64_t nNodes, nnz, nDofs, nbrTotal;
    int ncomp;
    double lmax;
};

template <typename TA>
struct TailArgs
{
    int nl;
    int pre, post, coarse;
    double smoothRatio, coarseRatio;
    TailLevel<TA> L[kTailMax];
};

template <typename TA>
__device__ void TailSpmv(const TailLevel<TA>& L, const TA* __restrict__ x, TA* __restrict__ y)
{
    const int lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    const int nc = L.ncomp;
    for (int64_t a = threadIdx.x >> 5; a < L.nNodes; a += nw)
    {
        const int64_t q0 = L.nbrPtr[a];
        const int len = static_cast<int>(L.nbrPtr[a + 1] - q0) * nc;
        TA s[kMaxComp];
#pragma unroll
        for (int c = 0; c < kMaxComp; ++c)
            s[c] = TA(0);
        for (int q = lane; q < len; q += 32)
        {
            const int k = q / nc, d = q - k * nc;
            const TA xv = x[NG_IDX(L.nbrCol[NG_IDX(q0 + k, L.nbrTotal, 70)] + d, L.nDofs, 71)];
#pragma unroll
            for (int c = 0; c < kMaxComp; ++c)
                if (c < nc)
                    s[c] += L.vals[NG_IDX(L.rowPtr[a * nc + c] + q, L.nnz, 72)] * xv;
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1)
#pragma unroll
            for (int c = 0; c < kMaxComp; ++c)
                s[c] += __shfl_down_sync(0xffffffffu, s[c], o);
        if (lane == 0)
            for (int c = 0; c < nc; ++c)
                y[a * nc + c] = s[c];
    }
}

// Chebyshev smoothing of A e = b on [lmax / ratio, lmax]; ends with a block barrier
template <typename TA>
__device__ void TailCheb(const TailLevel<TA>& L, int degree, bool fromZero, double ratio)
{
    const double lmax = L.lmax, lmin = L.lmax / ratio;
    const double theta = 0.5 * (lmax + lmin), delta = 0.5 * (lmax - lmin);
    const double sigma = theta / delta;
    double rho = 1. / sigma;
    const TA invTheta = TA(1. / theta);
    if (fromZero)
    {
        for (int64_t i = threadIdx.x; i < L.nDofs; i += blockDim.x)
        {
            const TA v = L.dinv[i] * L.b[i] * invTheta;
            L.d[i] = v;
            L.e[i] = v;
        }
    }
    else
    {
        TailSpmv(L, L.e, L.t);
        __syncthreads();
        for (int64_t i = threadIdx.x; i < L.nDofs; i += blockDim.x)
        {
            const TA v = L.dinv[i] * (L.b[i] - L.t[i]) * invTheta;
            L.d[i] = v;
            L.e[i] += v;
        }
    }
    __syncthreads();
    for (int k = 1; k < degree; ++k)
    {
        const double rhoNew = 1. / (2. * sigma - rho);
        const TA c1 = TA(rhoNew * rho), c2 = TA(2. * rhoNew / delta);
        TailSpmv(L, L.e, L.t);
        __syncthreads();
        for (int64_t i = threadIdx.x; i < L.nDofs; i += blockDim.x)
        {
            const TA v = c1 * L.d[i] + c2 * L.dinv[i] * (L.b[i] - L.t[i]);
            L.d[i] = v;
            L.e[i] += v;
        }
        __syncthreads();
        rho = rhoNew;
    }
}

// e = V-cycle(b) on the tail levels: the first level's b is the restriction from the finer level, its e is read by
// the finer level's prolongation
template <typename TA>
__global__ void __launch_bounds__(kTailThreads) k_amg_tail(TailArgs<TA> T, const int* st)
{
    PdlWait();
    PdlTrigger();
    if (Idle(st))
        return;
    for (int l = 0; l + 1 < T.nl; ++l)
    {
        const TailLevel<TA>& F = T.L[l];
        const TailLevel<TA>& C = T.L[l + 1];
        TailCheb(F, T.pre, true, T.smoothRatio);
        TailSpmv(F, F.e, F.t);
        for (int64_t i = threadIdx.x; i < C.nDofs; i += blockDim.x)
            C.b[i] = TA(0);
        __syncthreads();
        for (int64_t a = threadIdx.x; a < F.nNodes; a += blockDim.x)
        {
            const int64_t A = F.agg[a];
            for (int c = 0; c < F.ncomp; ++c)
                atomicAdd(C.b + NG_IDX(A * C.ncomp + c, C.nDofs, 73), F.b[a * F.ncomp + c] - F.t[a * F.ncomp + c]);
        }
        __syncthreads();
    }
    TailCheb(T.L[T.nl - 1], T.coarse, true, T.coarseRatio);
    for (int l = T.nl - 2; l >= 0; --l)
    {
        const TailLevel<TA>& F = T.L[l];
        const TailLevel<TA>& C = T.L[l + 1];
        for (int64_t a = threadIdx.x; a < F.nNodes; a += blockDim.x)
        {
            const int64_t A = F.agg[a];
            for (int c = 0; c < F.ncomp; ++c)
                F.e[a * F.ncomp + c] += C.e[NG_IDX(A * C.ncomp + c, C.nDofs, 74)];
        }
        __syncthreads();
        TailCheb(F, T.post, false, T.smoothRatio);
    }
}

// ---- host: set-up and application ------------------------------------------------------------------------------
static unsigned Blocks(int64_t n, int bs = 256)
{
    return static_cast<unsigned>((n + bs - 1) / bs);
}

// device vectors of every level in arithmetic TA (on first use of TA)
template <typename TA>
static void EnsureNum(Ctx& c, Amg& M)
{
    for (int I = 0; I < M.ns; ++I)
        for (size_t l = 0; l < M.h[I].size(); ++l)
        {
            AmgLevel& L = M.h[I][l];
            Num<TA>& U = N<TA>(L);
            const int64_t n = l == 0 ? c.nDofs : L.nDofs;
            if (U.dinv.n == static_cast<size_t>(n))
                continue;
            if (l > 0)
            {
                U.vals.alloc(L.nnz);
                U.nb.alloc(std::max<int64_t>(L.nbTotal, 4));
            }
            for (DBuf<TA>* b : {&U.dinv, &U.e, &U.b, &U.t, &U.d})
                b->alloc(n);
        }
}

// Builds the hierarchy on first use and the coarse operators for the tangent `vals` unless they were built for
// the same values already (same pointer and tangent version). The preconditioner works in the arithmetic of the
// tangent values: FP32 for FP32 tangents, FP64 for FP64 tangents.
template <typename TV>
void AmgSetup(Ctx& c, const TV* vals)
{
    HostClock hc(&c.hostMs[HP_AMG_SETUP]);
    if (!c.amg)
    {
        c.amg = new Amg();
        const char* gr = std::getenv("NUTO_GPU_GRAPHS");
        c.amg->graphs = !(gr && gr[0] == '0');
    }
    Amg& M = *c.amg;
    if (!M.built)
        BuildHierarchy(c);
    if (M.setupVals == static_cast<const void*>(vals) && M.setupVersion == c.valsVersion)
        return;
    EnsureNum<TV>(c, M);
    M.prec = sizeof(TV) == 4 ? 32 : 64;
    M.fine = vals;
    NG_CUDA(cudaMemsetAsync(M.lmaxDev.p, 0, M.lmaxHost.size() * sizeof(float), c.stream));
    size_t slot = 0;
    for (int I = 0; I < M.ns; ++I)
    {
        std::vector<AmgLevel>& H = M.h[I];
        H[0].spmv = SlotView(c, I);
        k_amg_diag<TV><<<Blocks(H[0].nNodes * 32), kBS, 0, c.stream>>>(H[0].spmv, c.dMask.p, vals, H[0].diagOff.p,
                                                                        N<TV>(H[0]).dinv.p, M.lmaxDev.p + slot);
        c.stats.kernel_launches += 1;
        for (size_t l = 1; l < H.size(); ++l)
        {
            AmgLevel& Fi = H[l - 1];
            AmgLevel& C = H[l];
            Num<TV>& CU = N<TV>(C);
            NG_CUDA(cudaMemsetAsync(CU.vals.p, 0, C.nnz * sizeof(TV), c.stream));
            k_amg_coarsen<TV><<<Blocks(Fi.nNodes * 32), kBS, 0, c.stream>>>(
                    Fi.spmv, l == 1 ? c.dMask.p : Fi.zeroMask.p, l == 1 ? vals : N<TV>(Fi).vals.p, C.spmv, C.aggOf.p,
                    C.cRank.p, CU.vals.p);
            k_amg_diag<TV><<<Blocks(C.nNodes * 32), kBS, 0, c.stream>>>(C.spmv, C.zeroMask.p, CU.vals.p, C.diagOff.p,
                                                                         CU.dinv.p, M.lmaxDev.p + slot + l);
            c.stats.kernel_launches += 2;
            if (C.nbTotal > 0)
            {
                // the level's products stream the padded layout (filled from the new Galerkin values)
                NodeSpmv& V = C.spmv;
                V.nbBase[0] = C.nbBase.p;
                V.nbOff[0] = 0;
                V.nbSeg4 = C.nbSeg4;
                V.ncMaxRows = C.ncomp;
                if constexpr (sizeof(TV) == 4)
                {
                    V.nb32 = CU.nb.p;
                    V.nbSrc32 = CU.vals.p;
                }
                else
                {
                    V.nb64 = CU.nb.p;
                    V.nbSrc64 = CU.vals.p;
                }
                k_nb_pack<TV><<<Blocks(C.nNodes * 32), kBS, 0, c.stream>>>(V, CU.vals.p, CU.nb.p);
                c.stats.kernel_launches += 1;
            }
        }
        slot += H.size();
    }
    AfterLaunch(c, "multigrid set-up");
    NG_CUDA(cudaMemcpyAsync(M.lmaxHost.data(), M.lmaxDev.p, M.lmaxHost.size() * sizeof(float),
                            cudaMemcpyDeviceToHost, c.stream));
    NG_CUDA(cudaStreamSynchronize(c.stream));
    slot = 0;
    for (int I = 0; I < M.ns; ++I)
        for (AmgLevel& L : M.h[I])
        {
            const float v = M.lmaxHost[slot++];
            L.lmax = v > 0.f ? v : 1.f;
        }
    M.setupVals = vals;
    M.setupVersion = c.valsVersion;
    M.setups++;
}
template void AmgSetup<float>(Ctx&, const float*);
template void AmgSetup<double>(Ctx&, const double*);

// Chebyshev smoothing of A e = b on [lmax / ratio, lmax]. Vectors are base pointers of the level (combined
// length on level 0); elementwise work runs over rows [off, off + n). fromZero starts at e = 0 (no product).
template <typename TA>
static void Chebyshev(Ctx& c, AmgLevel& L, const TA* vals, const uint8_t* mask, const TA* b, TA* e, int degree,
                      bool fromZero, float ratio, const int* st)
{
    Num<TA>& U = N<TA>(L);
    const int64_t n = L.nDofs, o = L.off;
    const double lmax = L.lmax, lmin = L.lmax / ratio;
    const double theta = 0.5 * (lmax + lmin), delta = 0.5 * (lmax - lmin);
    const double sigma = theta / delta;
    int* stw = const_cast<int*>(st); // the SpMV only reads the state when it computes no dot products
    double rho = 1. / sigma;
    if (fromZero)
        NG_CUDA(LaunchPdl(k_cheb0<TA>, Blocks(n), 256, 0, c.stream, n, U.dinv.p + o, b + o, U.d.p + o, e + o,
                          TA(1. / theta), st));
    else
    {
        SpmvNode<TA, TA, 0>(c.stream, L.spmv, vals, e, U.t.p, nullptr, nullptr, stw, 0, mask);
        NG_CUDA(LaunchPdl(k_cheb1<TA>, Blocks(n), 256, 0, c.stream, n, U.dinv.p + o, b + o, U.t.p + o, U.d.p + o,
                          e + o, TA(1. / theta), st));
        c.stats.kernel_launches += 1;
    }
    c.stats.kernel_launches += 1;
    for (int k = 1; k < degree; ++k)
    {
        const double rhoNew = 1. / (2. * sigma - rho);
        SpmvNode<TA, TA, 0>(c.stream, L.spmv, vals, e, U.t.p, nullptr, nullptr, stw, 0, mask);
        NG_CUDA(LaunchPdl(k_chebk<TA>, Blocks(n), 256, 0, c.stream, n, U.dinv.p + o, b + o, U.t.p + o, U.d.p + o,
                          e + o, TA(rhoNew * rho), TA(2. * rhoNew / delta), st));
        c.stats.kernel_launches += 2;
        rho = rhoNew;
    }
}

// first level (>= 1) from which every level has at most kTailNodes nodes, if they fit one tail launch; 0: none
static size_t TailStart(const std::vector<AmgLevel>& H)
{
    for (size_t l = 1; l < H.size(); ++l)
        if (H[l].nNodes <= kTailNodes)
            return H.size() - l <= static_cast<size_t>(kTailMax) ? l : 0;
    return 0;
}

// e = V-cycle(b) on level l of hierarchy H
template <typename TA>
static void VCycle(Ctx& c, std::vector<AmgLevel>& H, size_t l, const TA* b, TA* e, const int* st, bool sym)
{
    Amg& M = *c.amg;
    AmgLevel& L = H[l];
    Num<TA>& U = N<TA>(L);
    const TA* vals = l == 0 ? static_cast<const TA*>(M.fine) : U.vals.p;
    const uint8_t* mask = l == 0 ? c.dMask.p : L.zeroMask.p;
    if (l > 0 && l == TailStart(H))
    {
        // this level and every coarser one in one block (b = U.b, e = U.e of this level)
        TailArgs<TA> T{};
        T.nl = static_cast<int>(H.size() - l);
        T.pre = sym ? kPostDegree : kPreDegree;
        T.post = kPostDegree;
        T.coarse = CoarseDegree<TA>();
        T.smoothRatio = kSmoothRatio;
        T.coarseRatio = kCoarseRatio;
        for (int k = 0; k < T.nl; ++k)
        {
            AmgLevel& Lk = H[l + k];
            Num<TA>& Uk = N<TA>(Lk);
            TailLevel<TA>& D = T.L[k];
            D.rowPtr = Lk.rowPtr.p;
            D.nbrPtr = Lk.nbrPtr.p;
            D.nbrCol = Lk.nbrCol.p;
            D.agg = l + k + 1 < H.size() ? H[l + k + 1].aggOf.p : nullptr;
            D.vals = Uk.vals.p;
            D.dinv = Uk.dinv.p;
            D.b = Uk.b.p;
            D.e = Uk.e.p;
            D.t = Uk.t.p;
            D.d = Uk.d.p;
            D.nNodes = Lk.nNodes;
            D.nnz = Lk.nnz;
            D.nDofs = Lk.nDofs;
            D.nbrTotal = static_cast<int64_t>(Lk.nbrIdx.n);
            D.ncomp = Lk.ncomp;
            D.lmax = Lk.lmax;
        }
        // the level's b and e are the ones the caller passed (its own U.b, U.e)
        NG_CUDA(LaunchPdl(k_amg_tail<TA>, 1, kTailThreads, 0, c.stream, T, st));
        c.stats.kernel_launches += 1;
        return;
    }
    if (l + 1 == H.size())
    {
        Chebyshev<TA>(c, L, vals, mask, b, e, CoarseDegree<TA>(), true, kCoarseRatio, st);
        return;
    }
    AmgLevel& C = H[l + 1];
    Num<TA>& CU = N<TA>(C);
    int* stw = const_cast<int*>(st);
    Chebyshev<TA>(c, L, vals, mask, b, e, sym ? kPostDegree : kPreDegree, true, kSmoothRatio, st);
    SpmvNode<TA, TA, 0>(c.stream, L.spmv, vals, e, U.t.p, nullptr, nullptr, stw, 0, mask);
    NG_CUDA(LaunchPdl(k_sub<TA>, Blocks(C.nDofs), 256, 0, c.stream, C.nDofs, nullptr, nullptr, CU.b.p, st));
    NG_CUDA(LaunchPdl(k_restrict<TA>, Blocks(L.nNodes), 256, 0, c.stream, L.spmv, mask, b, U.t.p, C.aggOf.p, C.spmv,
                      CU.b.p, st));
    c.stats.kernel_launches += 3;
    VCycle<TA>(c, H, l + 1, CU.b.p, CU.e.p, st, sym);
    NG_CUDA(LaunchPdl(k_prolong<TA>, Blocks(L.nNodes), 256, 0, c.stream, L.spmv, mask, C.aggOf.p, C.spmv, CU.e.p, e,
                      st));
    c.stats.kernel_launches += 1;
    Chebyshev<TA>(c, L, vals, mask, b, e, kPostDegree, false, kSmoothRatio, st);
}

// block Gauss-Seidel sweep in slot order on combined vectors: z_0 = V_0(v_0), z_1 = V_1(v_1 - K_10 z_0)
template <typename TA>
static void Sweep(Ctx& c, const TA* v, TA* z, TA* res, const int* st, bool sym)
{
    Amg& M = *c.amg;
    VCycle<TA>(c, M.h[0], 0, v, z, st, sym);
    for (int I = 1; I < M.ns; ++I)
    {
        AmgLevel& L = M.h[I][0];
        const int64_t o = L.off, n = L.nDofs;
        // z_I = 0, res = K z on the rows of slot I, res = v_I - res
        NG_CUDA(LaunchPdl(k_sub<TA>, Blocks(n), 256, 0, c.stream, n, nullptr, nullptr, z + o, st));
        SpmvNode<TA, TA, 0>(c.stream, RowsView(c, I), static_cast<const TA*>(M.fine), z, res, nullptr, nullptr,
                            const_cast<int*>(st), 0, c.dMask.p);
        NG_CUDA(LaunchPdl(k_sub<TA>, Blocks(n), 256, 0, c.stream, n, v + o, res + o, res + o, st));
        c.stats.kernel_launches += 3;
        VCycle<TA>(c, M.h[I], 0, res, z, st, sym);
    }
}

// Runs Sweep<TA>(in, out) through the graph of (TA, sym), capturing or updating it when the set-up changed. Returns
// false when graphs are off or the capture failed (the caller then launches the sweep kernel by kernel).
template <typename TA>
static bool SweepGraphRun(Ctx& c, TA* in, TA* out, TA* res, const int* st, bool sym)
{
    Amg& M = *c.amg;
    if (!M.graphs)
        return false;
    SweepGraph& G = M.graph[sizeof(TA) == 8 ? 1 : 0][sym ? 1 : 0];
    if (!G.exec || G.setup != M.setups || G.st != st)
    {
        HostClock hc(&c.hostMs[HP_GRAPH]);
        const int64_t before = c.stats.kernel_launches;
        cudaGraph_t graph = nullptr;
        // Capture on a private stream: capture is not permitted on the legacy default stream, which a caller may
        // hand to nuto_gpu_create. Capturing records the launches without running them, so swapping the
        // context's stream for the duration does not reorder any work; the graph is launched on the context's
        // stream.
        if (!M.capStream)
            NG_CUDA(cudaStreamCreateWithFlags(&M.capStream, cudaStreamNonBlocking));
        const cudaError_t eb = cudaStreamBeginCapture(M.capStream, cudaStreamCaptureModeThreadLocal);
        if (eb != cudaSuccess)
        {
            cudaGetLastError();
            M.graphs = false;
            M.graphError = std::string("begin capture: ") + cudaGetErrorString(eb);
            return false;
        }
        const cudaStream_t own = c.stream;
        c.stream = M.capStream;
        try
        {
            Sweep<TA>(c, in, out, res, st, sym);
        }
        catch (...)
        {
            c.stream = own;
            cudaGraph_t g = nullptr;
            cudaStreamEndCapture(M.capStream, &g);
            if (g)
                cudaGraphDestroy(g);
            cudaGetLastError();
            throw;
        }
        c.stream = own;
        const cudaError_t ec = cudaStreamEndCapture(M.capStream, &graph);
        G.launches = c.stats.kernel_launches - before;
        c.stats.kernel_launches = before;
        bool ok = ec == cudaSuccess && graph != nullptr;
        if (!ok)
            M.graphError = std::string("end capture: ") + cudaGetErrorString(ec);
        if (ok && G.exec)
        {
            cudaGraphExecUpdateResultInfo info;
            if (cudaGraphExecUpdate(G.exec, graph, &info) != cudaSuccess)
            {
                cudaGetLastError();
                cudaGraphExecDestroy(G.exec);
                G.exec = nullptr;
            }
        }
        if (ok && !G.exec)
        {
            const cudaError_t ei = cudaGraphInstantiate(&G.exec, graph, 0);
            ok = ei == cudaSuccess;
            if (!ok)
                M.graphError = std::string("instantiate: ") + cudaGetErrorString(ei);
        }
        if (graph)
            cudaGraphDestroy(graph);
        if (!ok)
        {
            cudaGetLastError();
            if (G.exec)
                cudaGraphExecDestroy(G.exec);
            G.exec = nullptr;
            M.graphs = false;
            return false;
        }
        G.setup = M.setups;
        G.st = st;
    }
    NG_CUDA(cudaGraphLaunch(G.exec, c.stream));
    M.graphLaunched = true;
    c.stats.kernel_launches += G.launches;
    return true;
}

// z = M^-1 v for the tangent of the last AmgSetup, in that tangent's arithmetic (FP64 Krylov vectors with an
// FP32 tangent are converted). With st given, every kernel returns at once when the Krylov state is not RUN.
// sym = true runs equal pre- and post-smoothing (a symmetric cycle for PCG on a single slot); otherwise the
// cheaper V(1,2) for GMRES. The sweep runs as a CUDA graph on fixed vectors (input and output copied).
template <typename T>
void AmgApply(Ctx& c, const T* v, T* z, const int* st, bool sym)
{
    Amg& M = *c.amg;
    const int64_t n = c.nDofs;
    const size_t bytesN = static_cast<size_t>(n);
    if (M.prec == 64)
    {
        if constexpr (sizeof(T) == 8)
        {
            if (M.res64.n != bytesN)
            {
                M.res64.alloc(n);
                M.in64.alloc(n);
                M.out64.alloc(n);
            }
            if (M.graphs)
            {
                NG_CUDA(cudaMemcpyAsync(M.in64.p, v, n * sizeof(double), cudaMemcpyDeviceToDevice, c.stream));
                if (SweepGraphRun<double>(c, M.in64.p, M.out64.p, M.res64.p, st, sym))
                {
                    NG_CUDA(cudaMemcpyAsync(z, M.out64.p, n * sizeof(double), cudaMemcpyDeviceToDevice, c.stream));
                    return;
                }
            }
            Sweep<double>(c, v, z, M.res64.p, st, sym);
        }
        else
            throw Error{NUTO_GPU_EINVAL, "FP32 Krylov vectors with an FP64 multigrid set-up"};
        return;
    }
    if (M.res32.n != bytesN)
    {
        M.res32.alloc(n);
        M.in32.alloc(n);
        M.out32.alloc(n);
    }
    if constexpr (sizeof(T) == 4)
    {
        if (M.graphs)
        {
            NG_CUDA(cudaMemcpyAsync(M.in32.p, v, n * sizeof(float), cudaMemcpyDeviceToDevice, c.stream));
            if (SweepGraphRun<float>(c, M.in32.p, M.out32.p, M.res32.p, st, sym))
            {
                NG_CUDA(cudaMemcpyAsync(z, M.out32.p, n * sizeof(float), cudaMemcpyDeviceToDevice, c.stream));
                return;
            }
        }
        Sweep<float>(c, v, z, M.res32.p, st, sym);
    }
    else
    {
        NG_CUDA(LaunchPdl(k_convert<double, float>, Blocks(n), 256, 0, c.stream, n, v, M.in32.p, st));
        if (!SweepGraphRun<float>(c, M.in32.p, M.out32.p, M.res32.p, st, sym))
            Sweep<float>(c, M.in32.p, M.out32.p, M.res32.p, st, sym);
        NG_CUDA(LaunchPdl(k_convert<float, double>, Blocks(n), 256, 0, c.stream, n, M.out32.p, z, st));
        c.stats.kernel_launches += 2;
    }
}
template void AmgApply<float>(Ctx&, const float*, float*, const int*, bool);
template void AmgApply<double>(Ctx&, const double*, double*, const int*, bool);

bool AmgGraphActive(const Ctx& c)
{
    return c.amg && c.amg->graphs && c.amg->graphLaunched;
}

const char* AmgGraphStatus(const Ctx& c)
{
    if (!c.amg)
        return "no multigrid";
    if (c.amg->graphs)
        return "sweep graph on";
    return c.amg->graphError.empty() ? "sweep graph off" : c.amg->graphError.c_str();
}

int AmgLevels(const Ctx& c)
{
    return c.amg ? static_cast<int>(c.amg->h[0].size()) : 0;
}

} // namespace nuto_gpu
