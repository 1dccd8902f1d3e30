// C ABI entry points, context set-up and the CSR pattern builder of the GB300 element-assembly library.
#include "internal.cuh"

#include <algorithm>
#include <array>
#include <cstdlib>
#include <cstring>
#include <numeric>
#include <omp.h>

using namespace nuto_gpu;

struct nuto_gpu_ctx : public nuto_gpu::Ctx
{
};

namespace nuto_gpu
{

Ctx::~Ctx()
{
    FreeSolverWork(*this);
    FreeAmg(*this);
}

bool SyncCheck(const Ctx& c)
{
    return c.syncCheck;
}

cudaStream_t StreamOf(const Ctx& c)
{
    return c.stream;
}

// Gauss points: Legendre roots by Newton iteration from cos guesses and weights 2 / ((1 - x^2) P_n'(x)^2)
// (nuto/math/Legendre.cpp:8-66, nuto/math/Quadrature.cpp:26-39); tensor product with the first coordinate
// running fastest (nuto/mechanics/integrationtypes/IntegrationTypeTensorProduct.cpp:15-39).
static double LegendreP(int n, double x, int k)
{
    auto factorial = [](int i) -> int { return static_cast<int>(std::tgamma(i + 1)); };
    std::vector<double> v(n + 1, 0.);
    if (n >= k)
        v[k] = factorial(2 * k) / (std::pow(2, k) * factorial(k));
    for (int i = k + 1; i <= n; i++)
        v[i] = ((2. * i - 1.) * x * v[i - 1] - (i - 1. + k) * (i >= 2 ? v[i - 2] : 0.)) / (i - k);
    return v.back();
}

static void Gauss1D(int n, std::vector<double>& pts, std::vector<double>& w)
{
    pts.resize(n);
    for (int i = 1; i <= n; ++i)
    {
        double x = std::cos(M_PI * (4. * i - 1) / (4. * n + 2));
        for (int it = 0; it < 100; ++it)
        {
            const double xn = x - LegendreP(n, x, 0) / LegendreP(n, x, 1);
            const bool done = std::abs(x - xn) < 1e-15;
            x = xn;
            if (done)
                break;
        }
        pts[i - 1] = x;
    }
    std::sort(pts.begin(), pts.end());
    w.resize(n);
    for (int i = 0; i < n; ++i)
    {
        const double dl = LegendreP(n, pts[i], 1);
        w[i] = 2. / (1. - pts[i] * pts[i]) / (dl * dl);
    }
}

// Shape functions and natural derivatives of the three interpolations (InterpolationQuadLinear.cpp:37-80,
// InterpolationBrickLinear.cpp:37-132, InterpolationBrickQuadratic.cpp:37-262), evaluated once per Gauss point.
static void ShapeHost(int interp, const double* x, double* N, double* dN)
{
    if (interp == NUTO_GPU_QUAD4)
    {
        const double r = x[0], s = x[1];
        const double n[4] = {0.25 * (1 - r) * (1 - s), 0.25 * (1 + r) * (1 - s), 0.25 * (1 + r) * (1 + s),
                             0.25 * (1 - r) * (1 + s)};
        const double d[4][2] = {{-0.25 * (1 - s), -0.25 * (1 - r)},
                                {0.25 * (1 - s), -0.25 * (1 + r)},
                                {0.25 * (1 + s), 0.25 * (1 + r)},
                                {-0.25 * (1 + s), 0.25 * (1 - r)}};
        for (int i = 0; i < 4; ++i)
        {
            N[i] = n[i];
            dN[i * 3 + 0] = d[i][0];
            dN[i * 3 + 1] = d[i][1];
            dN[i * 3 + 2] = 0;
        }
        return;
    }
    const double r = x[0], s = x[1], t = x[2];
    const double pr = 1 + r, ps = 1 + s, pt = 1 + t, mr = 1 - r, ms = 1 - s, mt = 1 - t;
    if (interp == NUTO_GPU_HEX8)
    {
        // corner signs of the reference cube in local node order
        const int sg[8][3] = {{-1, -1, -1}, {1, -1, -1}, {1, 1, -1}, {-1, 1, -1},
                              {-1, -1, 1},  {1, -1, 1},  {1, 1, 1},  {-1, 1, 1}};
        for (int i = 0; i < 8; ++i)
        {
            const double a = 1 + sg[i][0] * r, b = 1 + sg[i][1] * s, c = 1 + sg[i][2] * t;
            N[i] = 0.125 * a * b * c;
            dN[i * 3 + 0] = 0.125 * sg[i][0] * b * c;
            dN[i * 3 + 1] = 0.125 * sg[i][1] * a * c;
            dN[i * 3 + 2] = 0.125 * sg[i][2] * a * b;
        }
        return;
    }
    // 20-node serendipity brick: corners 0-7, edge mid-nodes 8-19 (local coordinates of
    // InterpolationBrickQuadratic::LocalCoords)
    const int lc[20][3] = {{-1, -1, -1}, {1, -1, -1}, {1, 1, -1}, {-1, 1, -1}, {-1, -1, 1}, {1, -1, 1}, {1, 1, 1},
                           {-1, 1, 1},   {0, -1, -1}, {1, 0, -1}, {0, 1, -1},  {-1, 0, -1}, {-1, -1, 0}, {1, -1, 0},
                           {1, 1, 0},    {-1, 1, 0},  {0, -1, 1}, {1, 0, 1},   {0, 1, 1},   {-1, 0, 1}};
    (void)pr;
    (void)ps;
    (void)pt;
    (void)mr;
    (void)ms;
    (void)mt;
    for (int i = 0; i < 20; ++i)
    {
        const double xi = lc[i][0], eta = lc[i][1], ze = lc[i][2];
        if (i < 8)
        {
            const double a = 1 + xi * r, b = 1 + eta * s, c = 1 + ze * t;
            const double q = xi * r + eta * s + ze * t - 2;
            N[i] = 0.125 * a * b * c * q;
            dN[i * 3 + 0] = 0.125 * xi * b * c * (q + a);
            dN[i * 3 + 1] = 0.125 * eta * a * c * (q + b);
            dN[i * 3 + 2] = 0.125 * ze * a * b * (q + c);
        }
        else if (xi == 0)
        {
            const double b = 1 + eta * s, c = 1 + ze * t;
            N[i] = 0.25 * (1 - r * r) * b * c;
            dN[i * 3 + 0] = -0.5 * r * b * c;
            dN[i * 3 + 1] = 0.25 * (1 - r * r) * eta * c;
            dN[i * 3 + 2] = 0.25 * (1 - r * r) * b * ze;
        }
        else if (eta == 0)
        {
            const double a = 1 + xi * r, c = 1 + ze * t;
            N[i] = 0.25 * a * (1 - s * s) * c;
            dN[i * 3 + 0] = 0.25 * xi * (1 - s * s) * c;
            dN[i * 3 + 1] = -0.5 * s * a * c;
            dN[i * 3 + 2] = 0.25 * a * (1 - s * s) * ze;
        }
        else
        {
            const double a = 1 + xi * r, b = 1 + eta * s;
            N[i] = 0.25 * a * b * (1 - t * t);
            dN[i * 3 + 0] = 0.25 * xi * b * (1 - t * t);
            dN[i * 3 + 1] = 0.25 * a * eta * (1 - t * t);
            dN[i * 3 + 2] = -0.5 * t * a * b;
        }
    }
}

void BuildTables(Ctx& c)
{
    std::vector<double> p1, w1;
    Gauss1D(c.gauss, p1, w1);
    const int nIp = static_cast<int>(std::pow(c.gauss, c.dim));
    NG_CHECK(nIp <= kMaxIp, NUTO_GPU_EINVAL, "too many integration points");
    c.ip.nIp = nIp;
    c.ip.w.assign(nIp, 1.);
    std::vector<std::array<double, 3>> pts(nIp, {0., 0., 0.});
    for (int i = 0; i < nIp; ++i)
    {
        int power = 1;
        for (int d = 0; d < c.dim; ++d)
        {
            const int idx = (i / power) % c.gauss;
            c.ip.w[i] *= w1[idx];
            pts[i][d] = p1[idx];
            power *= c.gauss;
        }
    }
    std::vector<double> packed(c.ip.w);
    c.tabW = 0;
    for (int t = 0; t < 3; ++t)
    {
        if (InterpDim(t) != c.dim)
            continue;
        const int nen = NumNodes(t);
        c.ip.N[t].assign(static_cast<size_t>(nIp) * nen, 0.);
        c.ip.dN[t].assign(static_cast<size_t>(nIp) * nen * 3, 0.);
        for (int q = 0; q < nIp; ++q)
            ShapeHost(t, pts[q].data(), &c.ip.N[t][static_cast<size_t>(q) * nen], &c.ip.dN[t][static_cast<size_t>(q) * nen * 3]);
        c.tabN[t] = static_cast<int>(packed.size());
        packed.insert(packed.end(), c.ip.N[t].begin(), c.ip.N[t].end());
        c.tabDN[t] = static_cast<int>(packed.size());
        packed.insert(packed.end(), c.ip.dN[t].begin(), c.ip.dN[t].end());
    }
    c.dTables.alloc(packed.size());
    NG_CUDA(cudaMemcpy(c.dTables.p, packed.data(), packed.size() * sizeof(double), cudaMemcpyHostToDevice));
}

template <typename T>
static void Upload(DBuf<T>& buf, const std::vector<T>& h)
{
    buf.alloc(h.size());
    if (!h.empty())
        NG_CUDA(cudaMemcpy(buf.p, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice));
}

template <typename T>
static std::vector<T> Planar(const std::vector<T>& rowMajor, int64_t rows, int cols)
{
    std::vector<T> out(rowMajor.size());
    for (int64_t r = 0; r < rows; ++r)
        for (int k = 0; k < cols; ++k)
            out[static_cast<size_t>(k) * rows + r] = rowMajor[static_cast<size_t>(r) * cols + k];
    return out;
}

// CSR pattern of the combined matrix, in the order SimpleAssembler::BuildMatrix + setFromTriplets + ToEigen
// produce it (SimpleAssembler.cpp:100-156, DofMatrixSparseConvertEigen.h:40-67): every DOF pair of every cell,
// explicit zeros kept, rows and columns ordered by combined index = slot offset + DOF number. The pattern is
// structurally symmetric, so its CSR arrays equal the column pointers / row indices of NuTo's column-major
// matrix. Also builds, for the scatter, the rank of every cell's J-node among the sorted J-neighbours of its
// I-node and the start of each J block inside the rows of an I-node.
static void BuildPattern(Ctx& c)
{
    const int ns = static_cast<int>(c.slots.size());
    const int64_t nCells = c.nCells;

    struct NodeLists
    {
        std::vector<int64_t> ptr;
        std::vector<int32_t> idx;
    };
    // node -> cells adjacency per slot
    std::vector<NodeLists> cellsOf(ns);
    for (int I = 0; I < ns; ++I)
    {
        const Slot& S = c.slots[I];
        NodeLists& L = cellsOf[I];
        L.ptr.assign(S.nNodes + 1, 0);
        for (int64_t e = 0; e < nCells; ++e)
            for (int i = 0; i < S.nen; ++i)
                L.ptr[S.conn[e * S.nen + i] + 1]++;
        for (int64_t a = 0; a < S.nNodes; ++a)
            L.ptr[a + 1] += L.ptr[a];
        L.idx.resize(L.ptr.back());
        std::vector<int64_t> fill(L.ptr.begin(), L.ptr.end() - 1);
        // a cell lists every node once (checked in add_dof_type), so every (node, cell) pair appears once
        for (int64_t e = 0; e < nCells; ++e)
            for (int i = 0; i < S.nen; ++i)
                L.idx[fill[S.conn[e * S.nen + i]]++] = static_cast<int32_t>(e);
        std::vector<uint8_t> loc(L.idx.size());
        for (int64_t a = 0; a < S.nNodes; ++a)
            for (int64_t k = L.ptr[a]; k < L.ptr[a + 1]; ++k)
            {
                const int64_t e = L.idx[k];
                int i = 0;
                while (S.conn[e * S.nen + i] != a)
                    ++i;
                loc[k] = static_cast<uint8_t>(i);
            }
        Upload(c.slots[I].dCellPtr, L.ptr);
        Upload(c.slots[I].dCellIdx, L.idx);
        Upload(c.slots[I].dCellLoc, loc);
    }
    c.rowsMode = -1;
    c.fusedMode = -1;

    // neighbour lists per (I, J): J-nodes of all cells around an I-node, sorted by DOF number
    std::vector<NodeLists> nbr(ns * ns);
    for (int I = 0; I < ns; ++I)
        for (int J = 0; J < ns; ++J)
        {
            const Slot& SI = c.slots[I];
            const Slot& SJ = c.slots[J];
            NodeLists& N = nbr[I * ns + J];
            N.ptr.assign(SI.nNodes + 1, 0);
            std::vector<std::vector<int32_t>> tmp(SI.nNodes);
#pragma omp parallel for schedule(dynamic, 1024)
            for (int64_t a = 0; a < SI.nNodes; ++a)
            {
                std::vector<int32_t>& v = tmp[a];
                for (int64_t k = cellsOf[I].ptr[a]; k < cellsOf[I].ptr[a + 1]; ++k)
                {
                    const int64_t e = cellsOf[I].idx[k];
                    for (int j = 0; j < SJ.nen; ++j)
                        v.push_back(SJ.conn[e * SJ.nen + j]);
                }
                std::sort(v.begin(), v.end(), [&](int32_t x, int32_t y) { return SJ.dof0[x] < SJ.dof0[y]; });
                v.erase(std::unique(v.begin(), v.end()), v.end());
            }
            for (int64_t a = 0; a < SI.nNodes; ++a)
                N.ptr[a + 1] = N.ptr[a] + static_cast<int64_t>(tmp[a].size());
            N.idx.resize(N.ptr.back());
#pragma omp parallel for schedule(static)
            for (int64_t a = 0; a < SI.nNodes; ++a)
                std::copy(tmp[a].begin(), tmp[a].end(), N.idx.begin() + N.ptr[a]);
        }

    // row lengths and row pointers in combined order
    std::vector<int64_t> rowLen(c.nDofs, 0);
    for (int I = 0; I < ns; ++I)
    {
        const Slot& SI = c.slots[I];
#pragma omp parallel for schedule(static)
        for (int64_t a = 0; a < SI.nNodes; ++a)
        {
            int64_t len = 0;
            for (int J = 0; J < ns; ++J)
                len += static_cast<int64_t>(c.slots[J].ncomp) * (nbr[I * ns + J].ptr[a + 1] - nbr[I * ns + J].ptr[a]);
            for (int comp = 0; comp < SI.ncomp; ++comp)
                rowLen[SI.offset + SI.dof0[a] + comp] = len;
        }
    }
    c.hRowPtr.assign(c.nDofs + 1, 0);
    for (int64_t r = 0; r < c.nDofs; ++r)
        c.hRowPtr[r + 1] = c.hRowPtr[r] + rowLen[r];
    c.nnz = c.hRowPtr.back();
    NG_CHECK(c.nnz < (int64_t(1) << 40), NUTO_GPU_EINVAL, "pattern too large");
    NG_CHECK(*std::max_element(rowLen.begin(), rowLen.end()) <= 256, NUTO_GPU_EINVAL,
             "a row has more than 256 entries (unsupported element family)");
    c.avgRowLen = c.nDofs ? double(c.nnz) / double(c.nDofs) : 0;

    std::vector<int32_t> colIdx(c.nnz);
    std::vector<std::vector<int32_t>> blk(ns * ns);
    for (int I = 0; I < ns; ++I)
    {
        const Slot& SI = c.slots[I];
        for (int J = 0; J < ns; ++J)
            blk[I * ns + J].assign(SI.nNodes, 0);
#pragma omp parallel for schedule(static)
        for (int64_t a = 0; a < SI.nNodes; ++a)
        {
            int64_t pos0 = 0;
            for (int J = 0; J < ns; ++J)
            {
                blk[I * ns + J][a] = static_cast<int32_t>(pos0);
                const Slot& SJ = c.slots[J];
                const NodeLists& N = nbr[I * ns + J];
                for (int comp = 0; comp < SI.ncomp; ++comp)
                {
                    int64_t pos = c.hRowPtr[SI.offset + SI.dof0[a] + comp] + pos0;
                    for (int64_t k = N.ptr[a]; k < N.ptr[a + 1]; ++k)
                        for (int d = 0; d < SJ.ncomp; ++d)
                            colIdx[pos++] = static_cast<int32_t>(SJ.offset + SJ.dof0[N.idx[k]] + d);
                }
                pos0 += static_cast<int64_t>(SJ.ncomp) * (N.ptr[a + 1] - N.ptr[a]);
            }
        }
    }

    // per-cell rank tables (planar [i * nenJ + j][cell])
    std::vector<std::vector<uint8_t>> rank(ns * ns);
    for (int I = 0; I < ns; ++I)
        for (int J = 0; J < ns; ++J)
        {
            const Slot& SI = c.slots[I];
            const Slot& SJ = c.slots[J];
            const NodeLists& N = nbr[I * ns + J];
            std::vector<uint8_t>& R = rank[I * ns + J];
            R.resize(static_cast<size_t>(nCells) * SI.nen * SJ.nen);
            int bad = 0;
#pragma omp parallel for schedule(static) reduction(+ : bad)
            for (int64_t e = 0; e < nCells; ++e)
                for (int i = 0; i < SI.nen; ++i)
                {
                    const int32_t a = SI.conn[e * SI.nen + i];
                    const int32_t* first = N.idx.data() + N.ptr[a];
                    const int32_t* last = N.idx.data() + N.ptr[a + 1];
                    if (last - first > 255)
                        bad++;
                    for (int j = 0; j < SJ.nen; ++j)
                    {
                        const int32_t b = SJ.conn[e * SJ.nen + j];
                        const int32_t* it = std::lower_bound(first, last, b, [&](int32_t x, int32_t y) {
                            return SJ.dof0[x] < SJ.dof0[y];
                        });
                        R[static_cast<size_t>(i * SJ.nen + j) * nCells + e] = static_cast<uint8_t>(it - first);
                    }
                }
            NG_CHECK(bad == 0, NUTO_GPU_EINVAL, "more than 255 neighbour nodes around a node");
        }

    Upload(c.dRowPtr, c.hRowPtr);
    Upload(c.dColIdx, colIdx);
    for (int p = 0; p < ns * ns; ++p)
    {
        PairMap& M = c.pairs[p];
        M.rank = nullptr;
        for (int q = 0; q < p; ++q)
            if (rank[q] == rank[p])
            {
                M.rank = c.pairs[q].rank;
                break;
            }
        if (!M.rank)
        {
            Upload(M.dRank, rank[p]);
            M.rank = M.dRank.p;
        }
        Upload(M.dBlk, blk[p]);
        Upload(M.dNbrPtr, nbr[p].ptr);
        Upload(M.dNbrIdx, nbr[p].idx);
        {
            const Slot& SJ = c.slots[p % ns];
            std::vector<int32_t> col(nbr[p].idx.size());
            for (size_t q = 0; q < col.size(); ++q)
                col[q] = static_cast<int32_t>(SJ.offset + SJ.dof0[nbr[p].idx[q]]);
            Upload(M.dNbrCol, col);
        }
    }
    {
        // padded pair layout: per pair, the I-nodes' blocks of ncomp_I segments of ncomp_J * nn values, each
        // padded to a multiple of 4
        NbLayout& L = c.nb;
        L.src32 = L.src64 = nullptr;
        L.v32.free();
        L.v64.free();
        L.total = 0;
        L.maxSeg4 = 0;
        for (int p = 0; p < ns * ns; ++p)
        {
            const Slot& SI = c.slots[p / ns];
            const Slot& SJ = c.slots[p % ns];
            const std::vector<int64_t>& ptr = nbr[p].ptr;
            std::vector<int64_t> base(SI.nNodes);
            int64_t pos = 0;
            int mx = 0;
            for (int64_t a = 0; a < SI.nNodes; ++a)
            {
                const int seg4 = static_cast<int>((SJ.ncomp * (ptr[a + 1] - ptr[a]) + 3) / 4 * 4);
                base[a] = pos;
                pos += static_cast<int64_t>(SI.ncomp) * seg4;
                mx = std::max(mx, seg4);
            }
            L.pair[p].off = L.total;
            L.pair[p].maxSeg4 = mx;
            Upload(L.pair[p].base, base);
            L.total += (pos + 3) / 4 * 4;
            L.maxSeg4 = std::max(L.maxSeg4, mx);
        }
    }
    for (int p = 0; p < ns * ns; ++p)
    {
        PairMap& M = c.pairs[p];
        M.hNbrPtr = std::move(nbr[p].ptr);
        M.hNbrIdx = std::move(nbr[p].idx);
    }
    FreeAmg(c);
    c.havePattern = true;
}

static void SetupLaw(Ctx& c)
{
    const nuto_gpu_integrand& p = c.prm;
    LawParams& L = c.law;
    L.kind = p.kind;
    L.dim = p.dim;
    L.planeState = p.plane_state;
    L.damageApp = p.damage_application;
    L.interaction = p.interaction;
    L.E = p.E;
    L.nu = p.nu;
    // LinearElastic::CalculateC (LinearElastic.h:47-121)
    if (p.dim == 2 && p.plane_state == NUTO_GPU_PLANE_STRESS)
    {
        const double f = p.E / (1.0 - p.nu * p.nu);
        L.C11 = f;
        L.C12 = f * p.nu;
        L.C33 = f * 0.5 * (1.0 - p.nu);
    }
    else
    {
        const double f = p.E / ((1.0 + p.nu) * (1.0 - 2.0 * p.nu));
        L.C11 = f * (1.0 - p.nu);
        L.C12 = f * p.nu;
        L.C33 = p.E / (2. * (1.0 + p.nu));
    }
    // LinearElasticDamage (LinearElasticDamage.h:32-56)
    L.m3K = 3 * p.E / (3 - 6 * p.nu);
    L.m2G = 2 * p.E / (2 + 2 * p.nu);
    L.d2 = (p.dim == 2 && p.plane_state == NUTO_GPU_PLANE_STRESS) ? (1 + p.nu / (p.nu - 1)) : 1.0;
    L.kappa0 = p.kappa0;
    L.beta = p.beta;
    L.alpha = p.alpha;
    // ModifiedMisesStrainNorm (ModifiedMisesStrainNorm.h:70-78)
    L.k = p.k;
    L.K1 = (p.k - 1.) / (2. * p.k * (1 - 2 * p.nu));
    L.K2 = 3. / (p.k * (1. + p.nu) * (1. + p.nu));
    L.c = p.c;
    L.R = p.R;
    L.eta = p.eta;
}

// Combined mask and equation arrays of all slots' Dirichlet constraints (dependent DOF -> combined index).
static void RebuildConstraints(Ctx& c)
{
    std::vector<uint8_t> mask(c.nDofs, 0);
    std::vector<int64_t> idx;
    std::vector<double> A, B;
    for (size_t s = 0; s < c.slots.size(); ++s)
        for (size_t i = 0; i < c.depDofs[s].size(); ++i)
        {
            const int64_t g = c.slots[s].offset + c.depDofs[s][i];
            mask[g] = 1;
            idx.push_back(g);
            A.push_back(c.depA[s][i]);
            B.push_back(c.depB[s][i]);
        }
    Upload(c.dMask, mask);
    Upload(c.dDepIdx, idx);
    Upload(c.dDepA, A);
    Upload(c.dDepB, B);
    c.nDep = static_cast<int64_t>(idx.size());
}

} // namespace nuto_gpu

// ------------------------------------------------------------------------------------------------------------
// C ABI
// ------------------------------------------------------------------------------------------------------------
// message of the last failure that had no context to hold it (nuto_gpu_create)
static thread_local std::string tlsError;

template <typename F>
static int Guard(nuto_gpu_ctx* ctx, F&& f)
{
    if (!ctx)
        return NUTO_GPU_EINVAL;
    try
    {
        int dev = -1;
        NG_CUDA(cudaGetDevice(&dev));
        if (dev != ctx->device)
            NG_CUDA(cudaSetDevice(ctx->device));
        // a pending (non-sticky) error of an earlier call must not be reported as ours
        cudaGetLastError();
        return f();
    }
    catch (const Error& e)
    {
        ctx->err = e.msg;
        return e.code;
    }
    catch (const std::bad_alloc&)
    {
        ctx->err = "host allocation failed";
        return NUTO_GPU_ENOMEM;
    }
    catch (const std::exception& e)
    {
        ctx->err = e.what();
        return NUTO_GPU_EINVAL;
    }
}

// The second stream of nuto_gpu_build_system / _host and its fork and join events, created on first use. The
// highest priority: whenever an SM frees resources, the residual's few blocks are placed before the tangent's many,
// so they reach their slots early and keep them.
static void EnsureSideStream(Ctx& c)
{
    if (c.sideStream)
        return;
    int lo = 0, hi = 0; // numerically: lo >= hi
    NG_CUDA(cudaDeviceGetStreamPriorityRange(&lo, &hi));
    NG_CUDA(cudaStreamCreateWithPriority(&c.sideStream, cudaStreamNonBlocking, hi));
    NG_CUDA(cudaEventCreateWithFlags(&c.evFork, cudaEventDisableTiming));
    NG_CUDA(cudaEventCreateWithFlags(&c.evJoin, cudaEventDisableTiming));
}

// The copy stream of nuto_gpu_build_system_host's chunked values and its events, created on first use.
static void EnsureCopyStream(Ctx& c, int chunks)
{
    if (!c.copyStream)
    {
        NG_CUDA(cudaStreamCreateWithFlags(&c.copyStream, cudaStreamNonBlocking));
        NG_CUDA(cudaEventCreateWithFlags(&c.evCopy, cudaEventDisableTiming));
    }
    while (static_cast<int>(c.evChunks.size()) < chunks)
    {
        cudaEvent_t ev = nullptr;
        NG_CUDA(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
        c.evChunks.push_back(ev);
    }
}

// The rows of displacement node a are row(a) .. row(a) + ncomp - 1 and, for gradient damage, its eeq node's row.
// When both follow the node order without gaps (first-touch numbering of linear cells does that), the values of a
// node range are two contiguous ranges of the CSR values.
static bool RowsContiguous(Ctx& c)
{
    if (c.rowsContig >= 0)
        return c.rowsContig == 1;
    c.rowsContig = 0;
    const Slot& D = c.slots[c.prm.disp_slot];
    const bool gd = c.prm.kind == NUTO_GPU_GRADIENT_DAMAGE;
    if (gd && c.hEOf.size() != static_cast<size_t>(D.nNodes))
        return false;
    for (int64_t a = 1; a < D.nNodes; ++a)
    {
        if (D.dof0[a] != D.dof0[a - 1] + D.ncomp)
            return false;
        if (gd)
        {
            const Slot& E = c.slots[c.prm.eeq_slot];
            if (E.dof0[c.hEOf[a]] != E.dof0[c.hEOf[a - 1]] + 1)
                return false;
        }
    }
    c.rowsContig = 1;
    return true;
}

extern "C" {

int nuto_gpu_version(void)
{
    return 1;
}

int nuto_gpu_create(nuto_gpu_ctx** out, int device, void* stream)
{
    if (!out)
        return NUTO_GPU_EINVAL;
    *out = nullptr;
    int n = 0;
    const cudaError_t ce = cudaGetDeviceCount(&n);
    if (ce != cudaSuccess || device < 0 || device >= n)
    {
        tlsError = ce != cudaSuccess ? std::string("cudaGetDeviceCount: ") + cudaGetErrorString(ce)
                                     : "device " + std::to_string(device) + " out of range";
        cudaGetLastError();
        return NUTO_GPU_ECUDA;
    }
    auto* c = new nuto_gpu_ctx();
    c->device = device;
#ifdef NUTO_GPU_CHECKED
    c->syncCheck = true;
#else
    const char* sc = std::getenv("NUTO_GPU_SYNC_CHECK");
    c->syncCheck = sc && sc[0] == '1';
#endif
    const char* tk = std::getenv("NUTO_GPU_TANGENT");
    c->forceAtomicTangent = tk && std::string(tk) == "atomic";
    c->forceRecordTangent = tk && std::string(tk) == "records";
    c->tangentStaged = !(tk && std::string(tk) == "fused");
    if (tk && std::string(tk) == "pipelined")
    {
        c->tuning.tangentWarps = 4; // the double-buffered node-row kernel, not tuned
        c->tuning.tangentForm = 1;
    }
    const char* cr = std::getenv("NUTO_GPU_CELLS_RECORDS");
    c->cellsLawFused = !(cr && cr[0] == '1');
    if (tk && std::string(tk) == "cells")
    {
        c->tuning.tangentWarps = 4; // element matrices + row gather, not tuned
        c->tuning.tangentForm = 2;
    }
    // Hex20 FP32 tangent: tensor cores with split TF32 (default), one TF32 product (tf32) or records + row
    // gather (off)
    const char* t20 = std::getenv("NUTO_GPU_TC20");
    c->forceTc20Off = t20 && std::string(t20) == "off";
    c->tc20Split = t20 && std::string(t20) == "tf32" ? 1 : 3;
    c->tc20LawFp64 = t20 && std::string(t20) == "fp64law" ? 1 : 0;
    const char* at = std::getenv("NUTO_GPU_AUTOTUNE");
    c->tuning.enabled = !(at && at[0] == '0');
    const char* gr = std::getenv("NUTO_GPU_GMRES_RESTART");
    c->gmresRestart = gr ? std::atoi(gr) : 0;
    // nuto_gpu_build_system: residual blocks per SM beside the tangent (0: residual and tangent in sequence)
    const char* sr = std::getenv("NUTO_GPU_SYSTEM_RES_BLOCKS");
    if (sr)
        c->sysResBlocks = std::max(0, std::atoi(sr));
    const int rc = Guard(c, [&] {
        NG_CUDA(cudaSetDevice(device));
        NG_CUDA(cudaDeviceGetAttribute(&c->smCount, cudaDevAttrMultiProcessorCount, device));
        if (stream)
            c->stream = static_cast<cudaStream_t>(stream);
        else
        {
            NG_CUDA(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
            c->ownStream = true;
        }
        return NUTO_GPU_OK;
    });
    if (rc != NUTO_GPU_OK)
    {
        tlsError = c->err;
        delete c;
        return rc;
    }
    *out = c;
    return NUTO_GPU_OK;
}

int nuto_gpu_destroy(nuto_gpu_ctx* ctx)
{
    if (!ctx)
        return NUTO_GPU_OK;
    int rc = NUTO_GPU_OK;
    if (cudaSetDevice(ctx->device) != cudaSuccess || cudaStreamSynchronize(ctx->stream) != cudaSuccess)
        rc = NUTO_GPU_ECUDA;
    if (ctx->sideStream && cudaStreamSynchronize(ctx->sideStream) != cudaSuccess)
        rc = NUTO_GPU_ECUDA;
    if (ctx->evFork)
        cudaEventDestroy(ctx->evFork);
    if (ctx->evJoin)
        cudaEventDestroy(ctx->evJoin);
    if (ctx->sideStream)
        cudaStreamDestroy(ctx->sideStream);
    if (ctx->copyStream && cudaStreamSynchronize(ctx->copyStream) != cudaSuccess)
        rc = NUTO_GPU_ECUDA;
    if (ctx->copyStream)
        cudaStreamDestroy(ctx->copyStream);
    if (ctx->evCopy)
        cudaEventDestroy(ctx->evCopy);
    for (cudaEvent_t ev : ctx->evChunks)
        cudaEventDestroy(ev);
    const bool own = ctx->ownStream;
    cudaStream_t s = ctx->stream;
    delete ctx;
    if (own && cudaStreamDestroy(s) != cudaSuccess)
        rc = NUTO_GPU_ECUDA;
    if (rc != NUTO_GPU_OK)
        tlsError = std::string("nuto_gpu_destroy: ") + cudaGetErrorString(cudaGetLastError());
    cudaGetLastError();
    return rc;
}

const char* nuto_gpu_last_error(const nuto_gpu_ctx* ctx)
{
    return ctx ? ctx->err.c_str() : tlsError.c_str();
}

int nuto_gpu_synchronize(nuto_gpu_ctx* ctx)
{
    return Guard(ctx, [&] {
        NG_CUDA(cudaStreamSynchronize(ctx->stream));
        // a bounded device wait that gave up since the last synchronisation
        NG_CHECK(ReadDeviceStatus(*ctx) == 0, NUTO_GPU_ETIMEOUT, "a bounded device wait gave up");
        return NUTO_GPU_OK;
    });
}

int nuto_gpu_set_cells(nuto_gpu_ctx* ctx, int dim, int geoInterp, int64_t nCoord, const double* coords,
                       int64_t nCells, const int32_t* conn, int gauss)
{
    return Guard(ctx, [&] {
        NG_CHECK(dim == 2 || dim == 3, NUTO_GPU_EINVAL, "dim must be 2 or 3");
        NG_CHECK(geoInterp == NUTO_GPU_QUAD4 || geoInterp == NUTO_GPU_HEX8, NUTO_GPU_EINVAL,
                 "coordinate interpolation must be QUAD4 or HEX8");
        NG_CHECK(InterpDim(geoInterp) == dim, NUTO_GPU_EINVAL, "interpolation and dimension don't match");
        NG_CHECK(gauss >= 1 && gauss <= 3, NUTO_GPU_EINVAL, "1..3 Gauss points per direction supported");
        NG_CHECK(nCells > 0 && nCoord > 0 && coords && conn, NUTO_GPU_EINVAL, "empty cell group");
        NG_CHECK(nCells < (int64_t(1) << 31), NUTO_GPU_EINVAL, "too many cells");
        NG_CHECK(ctx->slots.empty(), NUTO_GPU_ESTATE, "set_cells must precede add_dof_type");
        ctx->dim = dim;
        ctx->geoInterp = geoInterp;
        ctx->nge = NumNodes(geoInterp);
        ctx->nCells = nCells;
        ctx->nCoord = nCoord;
        ctx->gauss = gauss;
        ctx->hCoords.assign(coords, coords + nCoord * dim);
        ctx->hGeoConn.assign(conn, conn + nCells * ctx->nge);
        for (int32_t v : ctx->hGeoConn)
            NG_CHECK(v >= 0 && v < nCoord, NUTO_GPU_EINVAL, "coordinate connectivity out of range");
        BuildTables(*ctx);
        Upload(ctx->dCoords, ctx->hCoords);
        Upload(ctx->dGeoConnT, Planar(ctx->hGeoConn, nCells, ctx->nge));
        ctx->haveCells = true;
        ctx->haveGeo = false;
        return NUTO_GPU_OK;
    });
}

int nuto_gpu_add_dof_type(nuto_gpu_ctx* ctx, int ncomp, int interp, int64_t nNodes, const int32_t* dofConn,
                          const int32_t* dofNumbers, int64_t nIndep, int64_t nDep, int* slotOut)
{
    return Guard(ctx, [&] {
        NG_CHECK(ctx->haveCells, NUTO_GPU_ESTATE, "set_cells first");
        NG_CHECK(static_cast<int>(ctx->slots.size()) < kMaxSlots, NUTO_GPU_EINVAL, "at most 2 DOF types");
        NG_CHECK(ncomp >= 1 && ncomp <= 3, NUTO_GPU_EINVAL, "1..3 components per DOF type");
        NG_CHECK(NumNodes(interp) > 0 && InterpDim(interp) == ctx->dim, NUTO_GPU_EINVAL,
                 "interpolation does not match the cell dimension");
        NG_CHECK(nIndep + nDep == nNodes * ncomp, NUTO_GPU_EINVAL,
                 "n_independent + n_dependent must equal n_dof_nodes * ncomp");
        Slot S;
        S.ncomp = ncomp;
        S.interp = interp;
        S.nen = NumNodes(interp);
        S.nNodes = nNodes;
        S.nDofs = nIndep + nDep;
        S.nIndep = nIndep;
        S.conn.assign(dofConn, dofConn + ctx->nCells * S.nen);
        for (int32_t v : S.conn)
            NG_CHECK(v >= 0 && v < nNodes, NUTO_GPU_EINVAL, "DOF connectivity out of range");
        for (int64_t e = 0; e < ctx->nCells; ++e)
            for (int i = 0; i < S.nen; ++i)
                for (int j = 0; j < i; ++j)
                    NG_CHECK(S.conn[e * S.nen + i] != S.conn[e * S.nen + j], NUTO_GPU_EINVAL,
                             "a cell lists a DOF node twice");
        S.dof0.resize(nNodes);
        std::vector<char> used(S.nDofs, 0);
        for (int64_t a = 0; a < nNodes; ++a)
        {
            const int32_t d0 = dofNumbers[a * ncomp];
            for (int comp = 0; comp < ncomp; ++comp)
            {
                const int32_t d = dofNumbers[a * ncomp + comp];
                NG_CHECK(d == d0 + comp, NUTO_GPU_EINVAL,
                         "components of a DOF node must have consecutive DOF numbers");
                NG_CHECK(d >= 0 && d < S.nDofs, NUTO_GPU_EINVAL, "DOF number out of range");
                NG_CHECK(!used[d], NUTO_GPU_EINVAL, "DOF number used twice");
                used[d] = 1;
            }
            S.dof0[a] = d0;
        }
        S.offset = ctx->nDofs;
        ctx->nDofs += S.nDofs;
        Upload(S.dConnT, Planar(S.conn, ctx->nCells, S.nen));
        std::vector<int64_t> g(nNodes);
        for (int64_t a = 0; a < nNodes; ++a)
            g[a] = S.offset + S.dof0[a];
        Upload(S.dGdof, g);
        ctx->slots.push_back(std::move(S));
        ctx->depDofs.emplace_back();
        ctx->depA.emplace_back();
        ctx->depB.emplace_back();
        ctx->havePattern = false;
        ctx->haveGeo = false;
        if (slotOut)
            *slotOut = static_cast<int>(ctx->slots.size()) - 1;
        return NUTO_GPU_OK;
    });
}

int nuto_gpu_set_dirichlet(nuto_gpu_ctx* ctx, int slot, int64_t nEq, const int32_t* dofs, const double* a,
                           const double* b)
{
    return Guard(ctx, [&] {
        NG_CHECK(slot >= 0 && slot < static_cast<int>(ctx->slots.size()), NUTO_GPU_EINVAL, "bad slot");
        const Slot& S = ctx->slots[slot];
        std::vector<char> seen(S.nDofs, 0);
        ctx->depDofs[slot].assign(dofs, dofs + nEq);
        ctx->depA[slot].assign(nEq, 0.);
        ctx->depB[slot].assign(nEq, 0.);
        for (int64_t i = 0; i < nEq; ++i)
        {
            NG_CHECK(dofs[i] >= 0 && dofs[i] < S.nDofs, NUTO_GPU_EINVAL, "dependent DOF out of range");
            NG_CHECK(!seen[dofs[i]], NUTO_GPU_EINVAL,
                     "The dependent dof of the new equation is already constrained as a dependent dof in another "
                     "equation.");
            seen[dofs[i]] = 1;
            if (a)
                ctx->depA[slot][i] = a[i];
            if (b)
                ctx->depB[slot][i] = b[i];
        }
        if (ctx->havePattern)
            RebuildConstraints(*ctx);
        return NUTO_GPU_OK;
    });
}

int nuto_gpu_build_pattern(nuto_gpu_ctx* ctx, int64_t* nDofs, int64_t* nnz)
{
    return Guard(ctx, [&] {
        NG_CHECK(!ctx->slots.empty(), NUTO_GPU_ESTATE, "add DOF types first");
        BuildPattern(*ctx);
        RebuildConstraints(*ctx);
        if (nDofs)
            *nDofs = ctx->nDofs;
        if (nnz)
            *nnz = ctx->nnz;
        return NUTO_GPU_OK;
    });
}

int nuto_gpu_copy_pattern(nuto_gpu_ctx* ctx, int64_t* rowPtr, int32_t* colIdx)
{
    return Guard(ctx, [&] {
        NG_CHECK(ctx->havePattern, NUTO_GPU_ESTATE, "build_pattern first");
        if (rowPtr)
            std::memcpy(rowPtr, ctx->hRowPtr.data(), ctx->hRowPtr.size() * sizeof(int64_t));
        if (colIdx)
            NG_CUDA(cudaMemcpy(colIdx, ctx->dColIdx.p, ctx->nnz * sizeof(int32_t), cudaMemcpyDeviceToHost));
        return NUTO_GPU_OK;
    });
}

int nuto_gpu_pattern_device(nuto_gpu_ctx* ctx, const int64_t** rp, const int32_t** ci)
{
    return Guard(ctx, [&] {
        NG_CHECK(ctx->havePattern, NUTO_GPU_ESTATE, "build_pattern first");
        if (rp)
            *rp = ctx->dRowPtr.p;
        if (ci)
            *ci = ctx->dColIdx.p;
        return NUTO_GPU_OK;
    });
}

int nuto_gpu_set_integrand(nuto_gpu_ctx* ctx, const nuto_gpu_integrand* p)
{
    return Guard(ctx, [&] {
        NG_CHECK(p, NUTO_GPU_EINVAL, "null parameters");
        NG_CHECK(p->dim == ctx->dim, NUTO_GPU_EINVAL, "integrand dimension differs from the cells");
        const int ns = static_cast<int>(ctx->slots.size());
        NG_CHECK(p->disp_slot >= 0 && p->disp_slot < ns, NUTO_GPU_EINVAL, "bad displacement slot");
        NG_CHECK(ctx->slots[p->disp_slot].ncomp == ctx->dim, NUTO_GPU_EINVAL,
                 "displacements need dim components");
        const int di = ctx->slots[p->disp_slot].interp;
        if (p->kind == NUTO_GPU_GRADIENT_DAMAGE)
        {
            NG_CHECK(p->eeq_slot >= 0 && p->eeq_slot < ns && p->eeq_slot != p->disp_slot, NUTO_GPU_EINVAL,
                     "bad eeq slot");
            NG_CHECK(ctx->slots[p->eeq_slot].ncomp == 1, NUTO_GPU_EINVAL, "eeq is a scalar DOF type");
            NG_CHECK(ctx->slots[p->eeq_slot].interp == di && di == ctx->geoInterp, NUTO_GPU_EINVAL,
                     "GradientDamage: displacement, eeq and coordinate interpolations must be equal");
        }
        else
        {
            NG_CHECK(p->kind == NUTO_GPU_MB_LINEAR_ELASTIC || p->kind == NUTO_GPU_MB_LOCAL_DAMAGE, NUTO_GPU_EINVAL,
                     "unknown integrand kind");
            NG_CHECK(di == ctx->geoInterp || (di == NUTO_GPU_HEX20 && ctx->geoInterp == NUTO_GPU_HEX8),
                     NUTO_GPU_EINVAL, "unsupported displacement interpolation");
        }
        ctx->prm = *p;
        SetupLaw(*ctx);
        ctx->dKappa.alloc(static_cast<size_t>(ctx->nCells) * ctx->ip.nIp);
        NG_CUDA(cudaMemsetAsync(ctx->dKappa.p, 0, ctx->dKappa.n * sizeof(double), ctx->stream));
        ctx->haveIntegrand = true;
        ctx->rowsMode = -1;
        ctx->fusedMode = -1;
        ctx->haveGeo = false;
        return NUTO_GPU_OK;
    });
}

int nuto_gpu_num_integration_points(const nuto_gpu_ctx* ctx)
{
    return ctx ? ctx->ip.nIp : 0;
}

int nuto_gpu_spmv(nuto_gpu_ctx* ctx, int precision, const void* d_values, const double* d_x, double* d_y,
                  int compensated)
{
    return Guard(ctx, [&] {
        NG_CHECK(ctx->havePattern, NUTO_GPU_ESTATE, "build_pattern first");
        NG_CHECK(precision == NUTO_GPU_FP32 || precision == NUTO_GPU_FP64, NUTO_GPU_EINVAL,
                 "precision NUTO_GPU_FP32 or NUTO_GPU_FP64");
        NG_CHECK(!compensated || precision == NUTO_GPU_FP32, NUTO_GPU_EINVAL,
                 "the compensated product takes FP32 values");
        NG_CHECK(d_values && d_x && d_y, NUTO_GPU_EINVAL, "null pointer");
        ctx->valsVersion++; // caller-supplied values may have changed behind the same pointer
        if (compensated)
            SpmvFull64Comp(*ctx, static_cast<const float*>(d_values), d_x, d_y);
        else
            SpmvFull64(*ctx, precision, d_values, d_x, d_y);
        NG_CUDA(cudaStreamSynchronize(ctx->stream));
        return NUTO_GPU_OK;
    });
}

int nuto_gpu_autotune_info(const nuto_gpu_ctx* ctx, int* choices, float* times_ms)
{
    if (!ctx)
        return NUTO_GPU_EINVAL;
    const Tuning& T = ctx->tuning;
    if (choices)
    {
        choices[0] = T.tangentWarps;
        choices[1] = T.tangentForm;
        for (int k = 0; k < 4; ++k)
            choices[2 + k] = T.spmvGroup[k];
    }
    if (times_ms)
    {
        for (int k = 0; k < 5; ++k)
            times_ms[k] = T.tangentMs[k];
        for (int p = 0; p < 4; ++p)
            for (int k = 0; k < 3; ++k)
                times_ms[5 + 3 * p + k] = T.spmvMs[p][k];
        times_ms[17] = T.tangentMs[5];
        times_ms[18] = T.tangentMs[6];
    }
    return NUTO_GPU_OK;
}

int nuto_gpu_multigrid_info(const nuto_gpu_ctx* ctx, int* levels, int* graph_active)
{
    if (!ctx || !levels || !graph_active)
        return NUTO_GPU_EINVAL;
    *levels = AmgLevels(*ctx);
    *graph_active = AmgGraphActive(*ctx) ? 1 : 0;
    return NUTO_GPU_OK;
}

int nuto_gpu_solver_layout(const nuto_gpu_ctx* ctx, int64_t* padded_values, int64_t* neighbour_entries)
{
    if (!ctx || !padded_values || !neighbour_entries)
        return NUTO_GPU_EINVAL;
    if (!ctx->havePattern)
        return NUTO_GPU_ESTATE;
    int64_t e = 0;
    for (const PairMap& M : ctx->pairs)
        e += static_cast<int64_t>(M.hNbrIdx.size());
    *padded_values = ctx->nb.total;
    *neighbour_entries = e;
    return NUTO_GPU_OK;
}

int nuto_gpu_set_history(nuto_gpu_ctx* ctx, const double* kappa)
{
    return Guard(ctx, [&] {
        NG_CHECK(ctx->haveIntegrand, NUTO_GPU_ESTATE, "set_integrand first");
        NG_CUDA(cudaMemcpyAsync(ctx->dKappa.p, kappa, ctx->dKappa.n * sizeof(double), cudaMemcpyHostToDevice,
                                ctx->stream));
        NG_CUDA(cudaStreamSynchronize(ctx->stream));
        return NUTO_GPU_OK;
    });
}

int nuto_gpu_set_spin_limit(nuto_gpu_ctx* ctx, long long iterations)
{
    return Guard(ctx, [&] {
        NG_CHECK(iterations >= 0, NUTO_GPU_EINVAL, "iterations >= 0");
        ctx->spinLimit = iterations;
        return NUTO_GPU_OK;
    });
}

int nuto_gpu_set_cell_scale(nuto_gpu_ctx* ctx, const double* scale)
{
    return Guard(ctx, [&] {
        NG_CHECK(ctx->haveCells, NUTO_GPU_ESTATE, "set_cells first");
        if (!scale)
        {
            ctx->dEScale.free();
            return NUTO_GPU_OK;
        }
        for (int64_t e = 0; e < ctx->nCells; ++e)
            NG_CHECK(std::isfinite(scale[e]) && scale[e] > 0., NUTO_GPU_EINVAL, "cell scale factors must be > 0");
        if (ctx->dEScale.n != static_cast<size_t>(ctx->nCells))
            ctx->dEScale.alloc(ctx->nCells);
        NG_CUDA(cudaMemcpyAsync(ctx->dEScale.p, scale, ctx->nCells * sizeof(double), cudaMemcpyHostToDevice,
                                ctx->stream));
        NG_CUDA(cudaStreamSynchronize(ctx->stream));
        return NUTO_GPU_OK;
    });
}

int nuto_gpu_get_history(nuto_gpu_ctx* ctx, double* kappa)
{
    return Guard(ctx, [&] {
        NG_CHECK(ctx->haveIntegrand, NUTO_GPU_ESTATE, "set_integrand first");
        NG_CUDA(cudaMemcpyAsync(kappa, ctx->dKappa.p, ctx->dKappa.n * sizeof(double), cudaMemcpyDeviceToHost,
                                ctx->stream));
        NG_CUDA(cudaStreamSynchronize(ctx->stream));
        return NUTO_GPU_OK;
    });
}

static void RequireReady(Ctx& c)
{
    NG_CHECK(c.havePattern, NUTO_GPU_ESTATE, "build_pattern first");
    NG_CHECK(c.haveIntegrand, NUTO_GPU_ESTATE, "set_integrand first");
    if (!c.haveGeo)
        BuildGeometryCache(c);
}

int nuto_gpu_history_device(nuto_gpu_ctx* ctx, double** d_kappa)
{
    return Guard(ctx, [&] {
        NG_CHECK(ctx->haveIntegrand, NUTO_GPU_ESTATE, "set_integrand first");
        NG_CHECK(d_kappa, NUTO_GPU_EINVAL, "d_kappa");
        *d_kappa = ctx->dKappa.p;
        return NUTO_GPU_OK;
    });
}

int nuto_gpu_transpose_values(nuto_gpu_ctx* ctx, int precision, const void* values, void* transposed)
{
    return Guard(ctx, [&] {
        NG_CHECK(ctx->havePattern, NUTO_GPU_ESTATE, "build_pattern first");
        NG_CHECK(precision == NUTO_GPU_FP32 || precision == NUTO_GPU_FP64, NUTO_GPU_EINVAL, "precision 32 or 64");
        NG_CHECK(values != transposed, NUTO_GPU_EINVAL, "the transposed values need their own buffer");
        LaunchTransposeValues(*ctx, precision, values, transposed);
        return NUTO_GPU_OK;
    });
}

int nuto_gpu_adjoint_history_load(nuto_gpu_ctx* ctx, const double* u, const double* kbar, double* ubar)
{
    return Guard(ctx, [&] {
        RequireReady(*ctx);
        LaunchAdjointHistoryLoad(*ctx, u, kbar, ubar);
        return NUTO_GPU_OK;
    });
}

int nuto_gpu_adjoint_step(nuto_gpu_ctx* ctx, const double* u, const double* lambda, const double* kbarIn,
                          double* kbarOut, double* gradE, double* gradParams)
{
    return Guard(ctx, [&] {
        RequireReady(*ctx);
        NG_CHECK(kbarIn != kbarOut, NUTO_GPU_EINVAL, "kbar_in and kbar_out must differ");
        LaunchAdjointStep(*ctx, u, lambda, kbarIn, kbarOut, gradE, gradParams);
        return NUTO_GPU_OK;
    });
}


int nuto_gpu_build_vector(nuto_gpu_ctx* ctx, const double* u, double* f)
{
    return Guard(ctx, [&] {
        RequireReady(*ctx);
        LaunchResidual(*ctx, u, f);
        return NUTO_GPU_OK;
    });
}

int nuto_gpu_build_matrix(nuto_gpu_ctx* ctx, const double* u, int precision, void* values)
{
    return Guard(ctx, [&] {
        RequireReady(*ctx);
        NG_CHECK(precision == NUTO_GPU_FP32 || precision == NUTO_GPU_FP64 || precision == NUTO_GPU_FP64X,
                 NUTO_GPU_EINVAL, "precision 32, 64 or 65");
        if (precision == NUTO_GPU_FP64X)
            LaunchTangentExact(*ctx, u, static_cast<double*>(values));
        else
            LaunchTangent(*ctx, u, precision, values);
        return NUTO_GPU_OK;
    });
}

int nuto_gpu_build_system(nuto_gpu_ctx* ctx, const double* u, int precision, void* values, double* f)
{
    return Guard(ctx, [&] {
        RequireReady(*ctx);
        NG_CHECK(precision == NUTO_GPU_FP32 || precision == NUTO_GPU_FP64, NUTO_GPU_EINVAL, "precision 32 or 64");
        NG_CHECK(values && f, NUTO_GPU_EINVAL, "values and f");
        Ctx& c = *ctx;
        // the first call (lazy set-up of geometry, records and tuning), and contexts that ask for it, run the two
        // launches in sequence on the context's stream
        if (c.systemCalls++ == 0 || c.sysResBlocks <= 0)
        {
            LaunchTangent(c, u, precision, values);
            LaunchResidual(c, u, f);
            return NUTO_GPU_OK;
        }
        EnsureSideStream(c);
        // fork: the residual (persistent grid, launched first so that its blocks hold their SM slots) on the side
        // stream; the tangent on the context's stream; join before anything else runs on the context's stream
        NG_CUDA(cudaEventRecord(c.evFork, c.stream));
        NG_CUDA(cudaStreamWaitEvent(c.sideStream, c.evFork, 0));
        const cudaStream_t main = c.stream;
        c.stream = c.sideStream;
        try
        {
            LaunchResidual(c, u, f, c.sysResBlocks);
        }
        catch (...)
        {
            c.stream = main;
            throw;
        }
        c.stream = main;
        LaunchTangent(c, u, precision, values);
        NG_CUDA(cudaEventRecord(c.evJoin, c.sideStream));
        NG_CUDA(cudaStreamWaitEvent(c.stream, c.evJoin, 0));
        return NUTO_GPU_OK;
    });
}

int nuto_gpu_build_system_host(nuto_gpu_ctx* ctx, const double* hU, int precision, void* hValues, double* hF)
{
    return Guard(ctx, [&] {
        RequireReady(*ctx);
        NG_CHECK(precision == NUTO_GPU_FP32 || precision == NUTO_GPU_FP64, NUTO_GPU_EINVAL, "precision 32 or 64");
        NG_CHECK(hU && hValues && hF, NUTO_GPU_EINVAL, "host state, values and f");
        Ctx& c = *ctx;
        const size_t valBytes = static_cast<size_t>(c.nnz) * (precision == NUTO_GPU_FP32 ? 4 : 8);
        if (c.dHostIoU.n != static_cast<size_t>(c.nDofs))
            c.dHostIoU.alloc(static_cast<size_t>(c.nDofs));
        if (c.dHostIoF.n != static_cast<size_t>(c.nDofs))
            c.dHostIoF.alloc(static_cast<size_t>(c.nDofs));
        if (c.dHostIoVals.n < valBytes)
            c.dHostIoVals.alloc(valBytes);
        const size_t vecBytes = static_cast<size_t>(c.nDofs) * sizeof(double);
        NG_CUDA(cudaMemcpyAsync(c.dHostIoU.p, hU, vecBytes, cudaMemcpyHostToDevice, c.stream));
        if (c.systemCalls++ == 0 || c.sysResBlocks <= 0)
        {
            LaunchTangent(c, c.dHostIoU.p, precision, c.dHostIoVals.p);
            NG_CUDA(cudaMemcpyAsync(hValues, c.dHostIoVals.p, valBytes, cudaMemcpyDeviceToHost, c.stream));
            LaunchResidual(c, c.dHostIoU.p, c.dHostIoF.p);
            NG_CUDA(cudaMemcpyAsync(hF, c.dHostIoF.p, vecBytes, cudaMemcpyDeviceToHost, c.stream));
            NG_CUDA(cudaStreamSynchronize(c.stream));
            return NUTO_GPU_OK;
        }
        EnsureSideStream(c);
        // the residual and its copy back on the side stream; the tangent and its copy back on the context's stream,
        // where the copy of the values starts as soon as the tangent is done, while the residual still runs
        NG_CUDA(cudaEventRecord(c.evFork, c.stream));
        NG_CUDA(cudaStreamWaitEvent(c.sideStream, c.evFork, 0));
        const cudaStream_t main = c.stream;
        c.stream = c.sideStream;
        try
        {
            LaunchResidual(c, c.dHostIoU.p, c.dHostIoF.p, c.sysResBlocks);
            NG_CUDA(cudaMemcpyAsync(hF, c.dHostIoF.p, vecBytes, cudaMemcpyDeviceToHost, c.stream));
        }
        catch (...)
        {
            c.stream = main;
            throw;
        }
        c.stream = main;
        // FP32 element-matrix form over rows that follow the node order: the row gather runs in node chunks, and each
        // chunk's values go to the host on a copy stream while the next chunks are gathered. (The row kernels writing
        // straight into mapped page-locked host memory were measured slower: 5.4 ms per 64^3 pass against 4.4 ms
        // with one copy after the tangent.)
        constexpr int kChunks = 4;
        const bool chunked = precision == NUTO_GPU_FP32 && c.tuning.tangentWarps != 0 && RowsContiguous(c);
        int chunkIdx = 0;
        if (chunked)
        {
            EnsureCopyStream(c, kChunks);
            const Slot& D = c.slots[c.prm.disp_slot];
            const bool gd = c.prm.kind == NUTO_GPU_GRADIENT_DAMAGE;
            float* hv = static_cast<float*>(hValues);
            const float* dv = reinterpret_cast<const float*>(c.dHostIoVals.p);
            c.rowChunks = kChunks;
            c.rowChunksDone = 0;
            c.onRowChunk = [&](int64_t a0, int64_t a1) {
                cudaEvent_t ev = c.evChunks[chunkIdx++];
                NG_CUDA(cudaEventRecord(ev, c.stream));
                NG_CUDA(cudaStreamWaitEvent(c.copyStream, ev, 0));
                auto copyRows = [&](int64_t r0, int64_t r1) {
                    const int64_t v0 = c.hRowPtr[r0], v1 = c.hRowPtr[r1];
                    if (v1 > v0)
                        NG_CUDA(cudaMemcpyAsync(hv + v0, dv + v0, (v1 - v0) * sizeof(float), cudaMemcpyDeviceToHost,
                                                c.copyStream));
                };
                copyRows(D.offset + D.dof0[a0], D.offset + D.dof0[a1 - 1] + D.ncomp);
                if (gd)
                {
                    const Slot& E = c.slots[c.prm.eeq_slot];
                    copyRows(E.offset + E.dof0[c.hEOf[a0]], E.offset + E.dof0[c.hEOf[a1 - 1]] + 1);
                }
            };
        }
        try
        {
            LaunchTangent(c, c.dHostIoU.p, precision, c.dHostIoVals.p);
        }
        catch (...)
        {
            c.onRowChunk = nullptr;
            c.rowChunks = 0;
            throw;
        }
        const bool copiedInChunks = chunked && c.rowChunksDone == kChunks;
        c.onRowChunk = nullptr;
        c.rowChunks = 0;
        if (copiedInChunks)
        {
            NG_CUDA(cudaEventRecord(c.evCopy, c.copyStream));
            NG_CUDA(cudaStreamWaitEvent(c.stream, c.evCopy, 0));
        }
        else
        {
            if (chunked && c.rowChunksDone > 0)
            {
                // a form without the chunk hook ran part of the way: wait for what was queued, then copy it all
                NG_CUDA(cudaEventRecord(c.evCopy, c.copyStream));
                NG_CUDA(cudaStreamWaitEvent(c.stream, c.evCopy, 0));
            }
            NG_CUDA(cudaMemcpyAsync(hValues, c.dHostIoVals.p, valBytes, cudaMemcpyDeviceToHost, c.stream));
        }
        NG_CUDA(cudaEventRecord(c.evJoin, c.sideStream));
        NG_CUDA(cudaStreamWaitEvent(c.stream, c.evJoin, 0));
        NG_CUDA(cudaStreamSynchronize(c.stream));
        return NUTO_GPU_OK;
    });
}

int nuto_gpu_build_matrix_noalloc(nuto_gpu_ctx* ctx, const double* u, float* values)
{
    return Guard(ctx, [&] {
        NG_CHECK(ctx->havePattern, NUTO_GPU_ESTATE, "build_pattern first");
        NG_CHECK(ctx->haveIntegrand, NUTO_GPU_ESTATE, "set_integrand first");
        LaunchTangentNoAlloc(*ctx, u, values);
        return NUTO_GPU_OK;
    });
}

int nuto_gpu_build_lumped_mass(nuto_gpu_ctx* ctx, double rho, double* m)
{
    return Guard(ctx, [&] {
        RequireReady(*ctx);
        LaunchLumpedMass(*ctx, rho, m);
        return NUTO_GPU_OK;
    });
}

int nuto_gpu_add_boundary_cells(nuto_gpu_ctx* ctx, int slot, int64_t nFaces, int nodesPerFace,
                                const int32_t* coordConn, const int32_t* dofConn, int gauss, int* group)
{
    return Guard(ctx, [&] {
        NG_CHECK(ctx->haveCells, NUTO_GPU_ESTATE, "set_cells first");
        NG_CHECK(slot >= 0 && slot < static_cast<int>(ctx->slots.size()), NUTO_GPU_EINVAL, "unknown slot");
        const Slot& S = ctx->slots[slot];
        NG_CHECK(S.ncomp == ctx->dim, NUTO_GPU_EINVAL, "boundary loads act on a displacement slot (ncomp == dim)");
        NG_CHECK((ctx->dim == 2 && nodesPerFace == 2) || (ctx->dim == 3 && nodesPerFace == 4), NUTO_GPU_EINVAL,
                 "boundary cells are Line2 in 2D and Quad4 in 3D");
        NG_CHECK(gauss >= 1 && gauss <= 3, NUTO_GPU_EINVAL, "1..3 Gauss points per direction supported");
        NG_CHECK(nFaces > 0 && coordConn && dofConn, NUTO_GPU_EINVAL, "empty boundary cell group");
        for (int64_t i = 0; i < nFaces * nodesPerFace; ++i)
        {
            NG_CHECK(coordConn[i] >= 0 && coordConn[i] < ctx->nCoord, NUTO_GPU_EINVAL,
                     "boundary coordinate connectivity out of range");
            NG_CHECK(dofConn[i] >= 0 && dofConn[i] < S.nNodes, NUTO_GPU_EINVAL, "boundary DOF connectivity out of range");
        }
        BoundaryGroup B;
        B.slot = slot;
        B.nfe = nodesPerFace;
        B.nFaces = nFaces;
        Upload(B.coordConnT, Planar(std::vector<int32_t>(coordConn, coordConn + nFaces * nodesPerFace), nFaces,
                                    nodesPerFace));
        Upload(B.dofConnT,
               Planar(std::vector<int32_t>(dofConn, dofConn + nFaces * nodesPerFace), nFaces, nodesPerFace));
        std::vector<double> pts, w;
        Gauss1D(gauss, pts, w);
        B.nq = gauss;
        for (int i = 0; i < gauss; ++i)
        {
            B.gp[i] = pts[i];
            B.gw[i] = w[i];
        }
        ctx->boundary.push_back(std::move(B));
        if (group)
            *group = static_cast<int>(ctx->boundary.size()) - 1;
        return NUTO_GPU_OK;
    });
}

int nuto_gpu_build_external_load(nuto_gpu_ctx* ctx, int group, const double* traction, double* f)
{
    return Guard(ctx, [&] {
        NG_CHECK(group >= 0 && group < static_cast<int>(ctx->boundary.size()), NUTO_GPU_EINVAL,
                 "unknown boundary cell group");
        NG_CHECK(traction, NUTO_GPU_EINVAL, "traction vector missing");
        LaunchExternalLoad(*ctx, ctx->boundary[group], traction, f);
        return NUTO_GPU_OK;
    });
}

int nuto_gpu_set_constant_gradient(nuto_gpu_ctx* ctx, const double* g)
{
    return Guard(ctx, [&] {
        if (!g)
        {
            ctx->dConstGrad.free();
            return NUTO_GPU_OK;
        }
        NG_CHECK(ctx->nDofs > 0, NUTO_GPU_ESTATE, "add the DOF types first");
        if (ctx->dConstGrad.n != static_cast<size_t>(ctx->nDofs))
            ctx->dConstGrad.alloc(ctx->nDofs);
        NG_CUDA(cudaMemcpyAsync(ctx->dConstGrad.p, g, ctx->nDofs * sizeof(double), cudaMemcpyDeviceToDevice,
                                ctx->stream));
        return NUTO_GPU_OK;
    });
}

int nuto_gpu_eval_ip(nuto_gpu_ctx* ctx, const double* u, int quantity, double* out)
{
    return Guard(ctx, [&] {
        RequireReady(*ctx);
        NG_CHECK(quantity >= NUTO_GPU_IP_KAPPA && quantity <= NUTO_GPU_IP_EEQ, NUTO_GPU_EINVAL,
                 "unknown integration-point quantity");
        LaunchEvalIp(*ctx, u, quantity, out);
        return NUTO_GPU_OK;
    });
}

int nuto_gpu_update_history(nuto_gpu_ctx* ctx, const double* u)
{
    return Guard(ctx, [&] {
        RequireReady(*ctx);
        LaunchHistory(*ctx, u);
        return NUTO_GPU_OK;
    });
}

int nuto_gpu_assemble_cell_vectors(nuto_gpu_ctx* ctx, const double* fe, double* f)
{
    return Guard(ctx, [&] {
        NG_CHECK(ctx->havePattern, NUTO_GPU_ESTATE, "build_pattern first");
        LaunchCellVectors(*ctx, fe, f);
        return NUTO_GPU_OK;
    });
}

int nuto_gpu_assemble_cell_matrices(nuto_gpu_ctx* ctx, const double* ke, int precision, void* values)
{
    return Guard(ctx, [&] {
        NG_CHECK(ctx->havePattern, NUTO_GPU_ESTATE, "build_pattern first");
        NG_CHECK(precision == NUTO_GPU_FP32 || precision == NUTO_GPU_FP64, NUTO_GPU_EINVAL, "precision 32 or 64");
        LaunchCellMatrices(*ctx, ke, precision, values);
        return NUTO_GPU_OK;
    });
}

int nuto_gpu_solve(nuto_gpu_ctx* ctx, int precision, int method, const void* values, const double* b, double* x,
                   double rtol, int maxit, int* iters, double* relres)
{
    return Guard(ctx, [&] {
        NG_CHECK(ctx->havePattern, NUTO_GPU_ESTATE, "build_pattern first");
        NG_CHECK(precision == NUTO_GPU_FP32 || precision == NUTO_GPU_FP64, NUTO_GPU_EINVAL, "precision 32 or 64");
        ctx->valsVersion++; // caller-supplied values may have changed behind the same pointer
        return SolveLinear(*ctx, precision, method, values, b, x, rtol, maxit, iters, relres);
    });
}

int nuto_gpu_set_preconditioner(nuto_gpu_ctx* ctx, int preconditioner)
{
    return Guard(ctx, [&] {
        NG_CHECK(preconditioner == NUTO_GPU_PRECOND_JACOBI || preconditioner == NUTO_GPU_PRECOND_AMG, NUTO_GPU_EINVAL,
                 "unknown preconditioner");
        ctx->precond = preconditioner;
        return NUTO_GPU_OK;
    });
}

int nuto_gpu_default_step_options(nuto_gpu_step_options* o)
{
    if (!o)
        return NUTO_GPU_EINVAL;
    o->precision = NUTO_GPU_FP32;
    o->method = NUTO_GPU_SOLVER_AUTO;
    o->newton_rtol = 1e-8;
    o->newton_atol = 0.0;
    o->max_newton = 20;
    o->line_search = 1;
    o->krylov_rtol = 1e-3;
    o->max_krylov = 20000;
    o->forcing = 1;
    o->exact_tangent_below = 1.0e4;
    o->forcing_floor = 0.5;
    return NUTO_GPU_OK;
}

int nuto_gpu_set_state(nuto_gpu_ctx* ctx, const double* x, double t, int resetHistory)
{
    return Guard(ctx, [&] {
        NG_CHECK(ctx->havePattern && ctx->haveIntegrand, NUTO_GPU_ESTATE, "pattern and integrand first");
        ctx->dX.alloc(ctx->nDofs);
        if (x)
            NG_CUDA(cudaMemcpyAsync(ctx->dX.p, x, ctx->nDofs * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
        else
            NG_CUDA(cudaMemsetAsync(ctx->dX.p, 0, ctx->nDofs * sizeof(double), ctx->stream));
        if (resetHistory)
            NG_CUDA(cudaMemsetAsync(ctx->dKappa.p, 0, ctx->dKappa.n * sizeof(double), ctx->stream));
        NG_CUDA(cudaStreamSynchronize(ctx->stream));
        ctx->time = t;
        ctx->haveState = true;
        return NUTO_GPU_OK;
    });
}

int nuto_gpu_get_state(nuto_gpu_ctx* ctx, double* x, double* t)
{
    return Guard(ctx, [&] {
        NG_CHECK(ctx->haveState, NUTO_GPU_ESTATE, "set_state first");
        if (x)
            NG_CUDA(cudaMemcpyAsync(x, ctx->dX.p, ctx->nDofs * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
        NG_CUDA(cudaStreamSynchronize(ctx->stream));
        if (t)
            *t = ctx->time;
        return NUTO_GPU_OK;
    });
}

int nuto_gpu_state_device(nuto_gpu_ctx* ctx, double** dx)
{
    return Guard(ctx, [&] {
        NG_CHECK(ctx->haveState, NUTO_GPU_ESTATE, "set_state first");
        *dx = ctx->dX.p;
        return NUTO_GPU_OK;
    });
}

int nuto_gpu_do_step(nuto_gpu_ctx* ctx, double tNew, const nuto_gpu_step_options* opts, int* iters)
{
    return Guard(ctx, [&] {
        NG_CHECK(ctx->haveState, NUTO_GPU_ESTATE, "set_state first");
        RequireReady(*ctx);
        nuto_gpu_step_options o;
        nuto_gpu_default_step_options(&o);
        if (opts)
            o = *opts;
        return DoStep(*ctx, tNew, o, iters);
    });
}

int nuto_gpu_do_step_host(nuto_gpu_ctx* ctx, double tNew, const nuto_gpu_step_options* opts, const double* xIn,
                          const double* kIn, double* xOut, double* kOut, int* iters)
{
    return Guard(ctx, [&] {
        NG_CHECK(ctx->haveState, NUTO_GPU_ESTATE, "set_state first");
        RequireReady(*ctx);
        if (xIn)
            NG_CUDA(cudaMemcpyAsync(ctx->dX.p, xIn, ctx->nDofs * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
        if (kIn)
            NG_CUDA(cudaMemcpyAsync(ctx->dKappa.p, kIn, ctx->dKappa.n * sizeof(double), cudaMemcpyHostToDevice,
                                    ctx->stream));
        nuto_gpu_step_options o;
        nuto_gpu_default_step_options(&o);
        if (opts)
            o = *opts;
        const int rc = DoStep(*ctx, tNew, o, iters);
        if (xOut)
            NG_CUDA(cudaMemcpyAsync(xOut, ctx->dX.p, ctx->nDofs * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
        if (kOut)
            NG_CUDA(cudaMemcpyAsync(kOut, ctx->dKappa.p, ctx->dKappa.n * sizeof(double), cudaMemcpyDeviceToHost,
                                    ctx->stream));
        NG_CUDA(cudaStreamSynchronize(ctx->stream));
        return rc;
    });
}

int nuto_gpu_get_stats(const nuto_gpu_ctx* ctx, nuto_gpu_stats* s)
{
    if (!ctx || !s)
        return NUTO_GPU_EINVAL;
    *s = ctx->stats;
    return NUTO_GPU_OK;
}

} // extern "C"
