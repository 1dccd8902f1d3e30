// Discrete adjoint of the quasistatic gradient-damage load path: the parts that run per load step of the reverse
// sweep. The reference has no adjoint; the forward it differentiates is QuasistaticSolver::DoStep
// (nuto/mechanics/tools/QuasistaticSolver.cpp:116-147) with GradientDamage::Gradient/Hessian0/Update
// (nuto/mechanics/integrands/GradientDamage.h:70-125) and DamageLawExponential (DamageLawExponential.h:40-52).
//
// Load step n solves R_n(u_n; kappa_{n-1}, p) = 0 on the independent DOFs and sets kappa_n = max(kappa_{n-1},
// eeq(u_n)) per integration point. With L a function of u_N and the parameters p = (E_e per cell, kappa0, beta),
// the reverse sweep n = N .. 1 at (u_n, kappa_{n-1}) is
//     ubar_n += sum over loading points (eeq >= kappa_{n-1}) of kbar_n N         (nuto_gpu_adjoint_history_load)
//     K_n^T lambda = ubar_n on the independent DOFs                              (nuto_gpu_transpose_values + solve)
//     s_ip = lambda . df_cell/domega_ip
//     dL/dkappa0 -= s_ip domega/dkappa0,  dL/dbeta -= s_ip domega/dbeta,  dL/dE_e -= lambda_u . f_u,e / E_e
//     kbar_{n-1} = kbar_n - s_ip domega/dkappa at unloading points, 0 at loading points   (nuto_gpu_adjoint_step)
// All sums run in a fixed order (per-cell vectors gathered per DOF, per-point partials reduced by one block), so
// the gradient is bitwise reproducible for given inputs.
#include "internal.cuh"

#include <algorithm>

namespace nuto_gpu
{

namespace
{

template <int DIM, int ND, int NIP>
struct AdjCfg
{
    static constexpr int dim = DIM, nd = ND, nip = NIP;
};

template <typename F>
void DispatchAdjoint(const Ctx& c, F&& f)
{
    const int nd = c.slots[c.prm.disp_slot].nen;
    NG_CHECK(c.prm.kind == NUTO_GPU_GRADIENT_DAMAGE, NUTO_GPU_EINVAL, "the adjoint needs the gradient-damage integrand");
    NG_CHECK(c.slots[c.prm.eeq_slot].nen == nd, NUTO_GPU_EINVAL,
             "the adjoint needs the same interpolation for displacements and eeq");
    if (c.dim == 2 && nd == 4 && c.ip.nIp == 4)
        return f(AdjCfg<2, 4, 4>{});
    if (c.dim == 2 && nd == 4 && c.ip.nIp == 9)
        return f(AdjCfg<2, 4, 9>{});
    if (c.dim == 3 && nd == 8 && c.ip.nIp == 8)
        return f(AdjCfg<3, 8, 8>{});
    if (c.dim == 3 && nd == 8 && c.ip.nIp == 27)
        return f(AdjCfg<3, 8, 27>{});
    throw Error{NUTO_GPU_EINVAL, "the adjoint supports Quad4 and Hex8 cells"};
}

// strain, eeq and its gradient of the state at one integration point (the FP64 residual's order of summation)
template <int DIM, int ND>
__device__ __forceinline__ void PointState(const CellArgs& a, const double* __restrict__ u, int64_t e, int q,
                                           double (&eps)[DIM == 2 ? 3 : 6], double& eeq, double (&ge)[DIM],
                                           double (&g)[ND][DIM], double& wdj)
{
    const int64_t n = a.nCells;
    const double* G = a.geo64 + NG_IDX(static_cast<int64_t>(q) * a.geoStride * n + e, a.geoSize, 60);
    wdj = G[0];
    double H[DIM][DIM];
#pragma unroll
    for (int i = 0; i < DIM; ++i)
    {
        ge[i] = 0.;
#pragma unroll
        for (int j = 0; j < DIM; ++j)
            H[i][j] = 0.;
    }
    eeq = 0.;
#pragma unroll
    for (int nd = 0; nd < ND; ++nd)
    {
#pragma unroll
        for (int d = 0; d < DIM; ++d)
            g[nd][d] = G[(1 + nd * DIM + d) * n];
        const int64_t gd = a.gdofD[NG_IDX(a.connD[static_cast<int64_t>(nd) * n + e], a.nNodesD, 61)];
#pragma unroll
        for (int c = 0; c < DIM; ++c)
        {
            const double uc = u[NG_IDX(gd + c, a.nDofs, 62)];
#pragma unroll
            for (int d = 0; d < DIM; ++d)
                H[c][d] += uc * g[nd][d];
        }
        const double ev = u[NG_IDX(a.gdofE[NG_IDX(a.connE[static_cast<int64_t>(nd) * n + e], a.nNodesE, 63)], a.nDofs, 64)];
        eeq += a.tabN_D[q * ND + nd] * ev;
#pragma unroll
        for (int d = 0; d < DIM; ++d)
            ge[d] += ev * g[nd][d];
    }
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
}

// cell vector entry (ND * DIM + nd) of cell e: sum over the cell's loading points of kbar N_nd (only the eeq
// entries are written and gathered); planar [entry][cell] like the residual's cell vectors
template <int DIM, int ND, int NIP>
__global__ void k_adjoint_history_load(CellArgs a, const double* __restrict__ u, const double* __restrict__ kbar,
                                       double* __restrict__ cellVec)
{
    const int64_t it = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
    const int64_t n = a.nCells;
    if (it >= n * ND)
        return;
    const int64_t e = it % n;
    const int nd = static_cast<int>(it / n);
    double ev[ND];
#pragma unroll
    for (int k = 0; k < ND; ++k)
        ev[k] = u[NG_IDX(a.gdofE[NG_IDX(a.connE[static_cast<int64_t>(k) * n + e], a.nNodesE, 65)], a.nDofs, 66)];
    double s = 0.;
    for (int q = 0; q < NIP; ++q)
    {
        double eeq = 0.;
#pragma unroll
        for (int k = 0; k < ND; ++k)
            eeq += a.tabN_D[q * ND + k] * ev[k];
        const double kh = a.kappa[NG_IDX(e * NIP + q, n * NIP, 67)];
        if (eeq >= kh)
            s += kbar[e * NIP + q] * a.tabN_D[q * ND + nd];
    }
    const int64_t nLocal = static_cast<int64_t>(ND) * (DIM + 1); // buffer extent for checked builds
    (void)nLocal;
    cellVec[NG_IDX((static_cast<int64_t>(ND) * DIM + nd) * n + e, nLocal * n, 68)] = s;
}

// one thread per (cell, point): s_ip, the history adjoint of the previous step and the per-point parts of the
// parameter derivatives (dL/dE_e summed per cell afterwards, kappa0 and beta over all points)
template <int DIM, int ND, int NIP>
__global__ void k_adjoint_point(CellArgs a, LawParams L, const double* __restrict__ u,
                                const double* __restrict__ lam, const double* __restrict__ kbarIn,
                                double* __restrict__ kbarOut, double* __restrict__ part)
{
    constexpr int VD = DIM == 2 ? 3 : 6;
    const int64_t n = a.nCells;
    const int64_t it = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
    if (it >= n * NIP)
        return;
    const int64_t e = it / NIP;
    const int q = static_cast<int>(it % NIP);
    double eps[VD], eeq, ge[DIM], g[ND][DIM], wdj;
    PointState<DIM, ND>(a, u, e, q, eps, eeq, ge, g, wdj);
    double epsL[VD], gl[DIM];
    {
        double eq2, ge2[DIM], g2[ND][DIM], w2;
        PointState<DIM, ND>(a, lam, e, q, epsL, eq2, ge2, g2, w2); // B lambda_u and grad lambda_eeq
#pragma unroll
        for (int d = 0; d < DIM; ++d)
            gl[d] = ge2[d];
    }
    const double kh = a.kappa[NG_IDX(e * NIP + q, n * NIP, 69)];
    const bool loading = eeq >= kh;
    const double kap = loading ? eeq : kh;
    const double omega = DamageOmega<double>(L, kap);
    const double se = a.escale ? a.escale[e] : 1.;
    double dsdw[VD], sig[VD];
    LedDstressDomega<double, DIM>(L, eps, dsdw);
    LedStress<double, DIM>(L, eps, omega, sig);
    double eL_dsdw = 0., eL_sig = 0., gl_ge = 0.;
#pragma unroll
    for (int v = 0; v < VD; ++v)
    {
        eL_dsdw += epsL[v] * dsdw[v];
        eL_sig += epsL[v] * sig[v];
    }
#pragma unroll
    for (int d = 0; d < DIM; ++d)
        gl_ge += gl[d] * ge[d];
    // s_ip = lambda . df/domega_ip: the displacement rows B^T dsigma/domega E_e/E w detJ, the eeq rows
    // c dg/domega (B_e^T grad eeq) w detJ
    const double s = se * wdj * eL_dsdw + L.c * InteractionDerivative<double>(L, omega) * wdj * gl_ge;
    double dk0 = 0., dbeta = 0., dkap = 0.;
    if (kap >= L.kappa0)
    {
        const double x = exp(L.beta * (L.kappa0 - kap));
        dk0 = -(1. - L.alpha + L.alpha * x) / kap - L.kappa0 / kap * L.alpha * L.beta * x;
        dbeta = -L.kappa0 / kap * L.alpha * (L.kappa0 - kap) * x;
        dkap = DamageDerivative<double>(L, kap);
    }
    kbarOut[it] = loading ? 0. : kbarIn[it] - s * dkap;
    // d f_u / d E_e = f_u / E_e: lambda_u . B^T sigma(E) w detJ / E (sigma of the base modulus)
    part[it] = -eL_sig * wdj / L.E;
    part[n * NIP + it] = -s * dk0;
    part[2 * n * NIP + it] = -s * dbeta;
}

// dL/dE_e += sum over the cell's points (one thread per cell)
__global__ void k_adjoint_cell_sum(int64_t nCells, int nip, const double* __restrict__ part, double* __restrict__ gE)
{
    const int64_t e = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
    if (e >= nCells)
        return;
    double s = 0.;
    for (int q = 0; q < nip; ++q)
        s += part[e * nip + q];
    gE[e] += s;
}

// out[k] += sum of in[k * m .. k * m + m) for k = 0, 1: one block, fixed order (strided partial sums per thread,
// then a tree in shared memory)
__global__ void __launch_bounds__(1024) k_adjoint_total(int64_t m, const double* __restrict__ in, double* __restrict__ out)
{
    __shared__ double sh[1024];
    for (int k = 0; k < 2; ++k)
    {
        double s = 0.;
        for (int64_t i = threadIdx.x; i < m; i += blockDim.x)
            s += in[k * m + i];
        sh[threadIdx.x] = s;
        __syncthreads();
        for (int w = blockDim.x / 2; w > 0; w >>= 1)
        {
            if (static_cast<int>(threadIdx.x) < w)
                sh[threadIdx.x] += sh[threadIdx.x + w];
            __syncthreads();
        }
        if (threadIdx.x == 0)
            out[k] += sh[0];
        __syncthreads();
    }
}

template <typename T>
__global__ void k_permute(int64_t nnz, const int64_t* __restrict__ perm, const T* __restrict__ in, T* __restrict__ out)
{
    const int64_t p = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
    if (p < nnz)
        out[p] = in[NG_IDX(perm[p], nnz, 70)];
}

// position of the transposed entry of every CSR entry (the pattern is structurally symmetric; columns sorted)
void BuildTransposePermutation(Ctx& c)
{
    std::vector<int32_t> col(c.nnz);
    NG_CUDA(cudaMemcpy(col.data(), c.dColIdx.p, c.nnz * sizeof(int32_t), cudaMemcpyDeviceToHost));
    std::vector<int64_t> perm(c.nnz);
    const std::vector<int64_t>& rp = c.hRowPtr;
    for (int64_t i = 0; i < c.nDofs; ++i)
        for (int64_t p = rp[i]; p < rp[i + 1]; ++p)
        {
            const int32_t j = col[p];
            const int32_t* b = col.data() + rp[j];
            const int32_t* f = col.data() + rp[j + 1];
            const int32_t* hit = std::lower_bound(b, f, static_cast<int32_t>(i));
            NG_CHECK(hit != f && *hit == i, NUTO_GPU_EINVAL, "the pattern is not structurally symmetric");
            perm[p] = rp[j] + (hit - b);
        }
    c.dTransPerm.alloc(perm.size());
    NG_CUDA(cudaMemcpy(c.dTransPerm.p, perm.data(), perm.size() * sizeof(int64_t), cudaMemcpyHostToDevice));
}

} // namespace

void LaunchTransposeValues(Ctx& c, int precision, const void* in, void* out)
{
    if (c.dTransPerm.n != static_cast<size_t>(c.nnz))
        BuildTransposePermutation(c);
    const unsigned blocks = static_cast<unsigned>((c.nnz + 255) / 256);
    if (precision == NUTO_GPU_FP32)
        k_permute<float><<<blocks, 256, 0, c.stream>>>(c.nnz, c.dTransPerm.p, static_cast<const float*>(in),
                                                       static_cast<float*>(out));
    else
        k_permute<double><<<blocks, 256, 0, c.stream>>>(c.nnz, c.dTransPerm.p, static_cast<const double*>(in),
                                                        static_cast<double*>(out));
    AfterLaunch(c, "k_permute");
    c.stats.kernel_launches += 1;
}

void LaunchAdjointHistoryLoad(Ctx& c, const double* u, const double* kbar, double* ubar)
{
    CellArgs a = CellArgsOf(c);
    const Slot& D = c.slots[c.prm.disp_slot];
    const Slot& E = c.slots[c.prm.eeq_slot];
    const int64_t nLocal = static_cast<int64_t>(D.nen) * (c.dim + 1);
    if (c.dCellVec.n != static_cast<size_t>(nLocal * c.nCells))
        c.dCellVec.alloc(static_cast<size_t>(nLocal * c.nCells));
    DispatchAdjoint(c, [&](auto cfg) {
        using C = decltype(cfg);
        const int64_t items = c.nCells * C::nd;
        k_adjoint_history_load<C::dim, C::nd, C::nip><<<static_cast<unsigned>((items + 127) / 128), 128, 0, c.stream>>>(
                a, u, kbar, c.dCellVec.p);
    });
    AfterLaunch(c, "k_adjoint_history_load");
    GatherCellVectors(c, E, 1, D.nen * c.dim, nLocal, ubar, true);
    c.stats.kernel_launches += 2;
}

void LaunchAdjointStep(Ctx& c, const double* u, const double* lam, const double* kbarIn, double* kbarOut,
                       double* gradE, double* gradParams)
{
    CellArgs a = CellArgsOf(c);
    const int64_t pts = c.nCells * c.ip.nIp;
    if (c.dAdjPart.n < static_cast<size_t>(3 * pts))
        c.dAdjPart.alloc(static_cast<size_t>(3 * pts));
    DispatchAdjoint(c, [&](auto cfg) {
        using C = decltype(cfg);
        k_adjoint_point<C::dim, C::nd, C::nip><<<static_cast<unsigned>((pts + 127) / 128), 128, 0, c.stream>>>(
                a, c.law, u, lam, kbarIn, kbarOut, c.dAdjPart.p);
    });
    AfterLaunch(c, "k_adjoint_point");
    k_adjoint_cell_sum<<<static_cast<unsigned>((c.nCells + 255) / 256), 256, 0, c.stream>>>(c.nCells, c.ip.nIp,
                                                                                           c.dAdjPart.p, gradE);
    AfterLaunch(c, "k_adjoint_cell_sum");
    k_adjoint_total<<<1, 1024, 0, c.stream>>>(pts, c.dAdjPart.p + pts, gradParams);
    AfterLaunch(c, "k_adjoint_total");
    c.stats.kernel_launches += 3;
}

} // namespace nuto_gpu
