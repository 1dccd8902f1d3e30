// TEST INFRASTRUCTURE ONLY — the oracle.
//
// CPU restatement of NuTo's element-assembly path (cell integration, integrands, constitutive laws,
// structured meshes, first-touch DOF numbering, SimpleAssembler::BuildVector/BuildMatrix with the
// reference's triplet + setFromTriplets assembly). It is the oracle for the CUDA path and the CPU
// baseline of the benchmark; it is never linked into the product library.
//
// Every function cites the reference file:line it restates (paths relative to the NuTo project root).
// The reference itself cannot be compiled in this environment (Eigen3/Boost/MUMPS are absent), so the
// restatement is pinned against the reference's own golden vectors and known-answer tests instead
// (applications/integrationtests/mechanics/results/Brick8N*.txt, test/mechanics/**).
#pragma once

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdint>
#include <list>
#include <stdexcept>
#include <string>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace nuto_oracle
{

// ------------------------------------------------------------------------------------------------
// Quadrature: nuto/math/Legendre.cpp:8-66, nuto/math/Quadrature.cpp:26-39,
//             nuto/mechanics/integrationtypes/IntegrationTypeTensorProduct.cpp:15-39
// ------------------------------------------------------------------------------------------------
inline double Legendre(int n, double x, int k = 0)
{
    auto factorial = [](int i) -> int { return static_cast<int>(std::tgamma(i + 1)); };
    std::vector<double> vals(n + 1, 0.);
    if (n >= k)
        vals[k] = factorial(2 * k) / (std::pow(2, k) * factorial(k));
    for (int i = k + 1; i <= n; i++)
    {
        double vm2 = i >= 2 ? vals[i - 2] : 0;
        vals[i] = ((2. * i - 1.) * x * vals[i - 1] - (i - 1. + k) * vm2) / (i - k);
    }
    return vals.back();
}

inline std::vector<double> LegendreRoots(int n)
{
    std::vector<double> xs(n);
    for (int i = 1; i <= n; i++)
        xs[i - 1] = std::cos(M_PI * (4. * i - 1) / (4. * n + 2));
    for (double& x : xs)
    {
        double xi = x;
        while (true)
        {
            double xnew = xi - Legendre(n, xi, 0) / Legendre(n, xi, 1);
            if (std::abs(xi - xnew) < 1e-15)
            {
                xi = xnew;
                break;
            }
            xi = xnew;
        }
        x = xi;
    }
    std::sort(xs.begin(), xs.end());
    return xs;
}

struct Quadrature
{
    int dim = 0;
    int n = 0;
    std::vector<std::array<double, 3>> points;
    std::vector<double> weights;
};

inline Quadrature TensorGauss(int dim, int nIps)
{
    std::vector<double> p1 = LegendreRoots(nIps);
    std::vector<double> w1;
    for (int i = 0; i < nIps; i++)
    {
        double dl = Legendre(nIps, p1[i], 1);
        w1.push_back(2. / (1. - p1[i] * p1[i]) / (dl * dl));
    }
    Quadrature q;
    q.dim = dim;
    int num = static_cast<int>(std::pow(nIps, dim));
    q.n = num;
    q.weights.assign(num, 1.);
    q.points.assign(num, {0., 0., 0.});
    for (int i = 0; i < num; i++)
    {
        int power = 1;
        for (int d = 0; d < dim; d++)
        {
            int index = (i / power) % nIps; // first coordinate fastest
            q.weights[i] *= w1[index];
            q.points[i][d] = p1[index];
            power *= nIps;
        }
    }
    return q;
}

// ------------------------------------------------------------------------------------------------
// Interpolations: nuto/mechanics/interpolation/InterpolationQuadLinear.cpp:37-80,
//                 InterpolationBrickLinear.cpp:37-132, InterpolationBrickQuadratic.cpp:37-262
// ------------------------------------------------------------------------------------------------
enum InterpType
{
    QUAD4 = 0,
    HEX8 = 1,
    HEX20 = 2
};

inline int NumNodes(int t)
{
    return t == QUAD4 ? 4 : (t == HEX8 ? 8 : 20);
}
inline int InterpDim(int t)
{
    return t == QUAD4 ? 2 : 3;
}

inline void LocalCoords(int t, int node, double* xi)
{
    static const double q4[4][2] = {{-1, -1}, {1, -1}, {1, 1}, {-1, 1}};
    static const double h20[20][3] = {{-1, -1, -1}, {1, -1, -1}, {1, 1, -1}, {-1, 1, -1}, {-1, -1, 1}, {1, -1, 1},
                                      {1, 1, 1},    {-1, 1, 1},  {0, -1, -1}, {1, 0, -1},  {0, 1, -1},  {-1, 0, -1},
                                      {-1, -1, 0},  {1, -1, 0},  {1, 1, 0},   {-1, 1, 0},  {0, -1, 1},  {1, 0, 1},
                                      {0, 1, 1},    {-1, 0, 1}};
    if (t == QUAD4)
    {
        xi[0] = q4[node][0];
        xi[1] = q4[node][1];
        xi[2] = 0;
    }
    else
    {
        xi[0] = h20[node][0];
        xi[1] = h20[node][1];
        xi[2] = h20[node][2];
    }
}

//! N[n], dN[n*3 + j] (derivative w.r.t. natural coordinate j)
inline void Shape(int t, const double* x, double* N, double* dN)
{
    if (t == QUAD4)
    {
        double r = x[0], s = x[1];
        N[0] = 0.25 * (1. - r) * (1. - s);
        N[1] = 0.25 * (1. + r) * (1. - s);
        N[2] = 0.25 * (1. + r) * (1. + s);
        N[3] = 0.25 * (1. - r) * (1. + s);
        dN[0 * 3 + 0] = -0.25 * (1. - s);
        dN[0 * 3 + 1] = -0.25 * (1. - r);
        dN[1 * 3 + 0] = +0.25 * (1. - s);
        dN[1 * 3 + 1] = -0.25 * (1. + r);
        dN[2 * 3 + 0] = +0.25 * (1. + s);
        dN[2 * 3 + 1] = +0.25 * (1. + r);
        dN[3 * 3 + 0] = -0.25 * (1. + s);
        dN[3 * 3 + 1] = +0.25 * (1. - r);
        for (int i = 0; i < 4; ++i)
            dN[i * 3 + 2] = 0;
        return;
    }
    const double r = x[0], s = x[1], u = x[2];
    const double pr = 1.0 + r, ps = 1.0 + s, pt = 1.0 + u;
    const double mr = 1.0 - r, ms = 1.0 - s, mt = 1.0 - u;
    if (t == HEX8)
    {
        N[0] = 0.125 * mr * ms * mt;
        N[1] = 0.125 * pr * ms * mt;
        N[2] = 0.125 * pr * ps * mt;
        N[3] = 0.125 * mr * ps * mt;
        N[4] = 0.125 * mr * ms * pt;
        N[5] = 0.125 * pr * ms * pt;
        N[6] = 0.125 * pr * ps * pt;
        N[7] = 0.125 * mr * ps * pt;
        const double d[8][3] = {{-0.125 * ms * mt, -0.125 * mr * mt, -0.125 * mr * ms},
                                {0.125 * ms * mt, -0.125 * pr * mt, -0.125 * pr * ms},
                                {0.125 * ps * mt, 0.125 * pr * mt, -0.125 * pr * ps},
                                {-0.125 * ps * mt, 0.125 * mr * mt, -0.125 * mr * ps},
                                {-0.125 * ms * pt, -0.125 * mr * pt, 0.125 * mr * ms},
                                {0.125 * ms * pt, -0.125 * pr * pt, 0.125 * pr * ms},
                                {0.125 * ps * pt, 0.125 * pr * pt, 0.125 * pr * ps},
                                {-0.125 * ps * pt, 0.125 * mr * pt, 0.125 * mr * ps}};
        for (int i = 0; i < 8; ++i)
            for (int j = 0; j < 3; ++j)
                dN[i * 3 + j] = d[i][j];
        return;
    }
    // HEX20 serendipity
    const double qr = 1.0 - r * r, qs = 1.0 - s * s, qt = 1.0 - u * u;
    N[0] = 0.125 * mr * ms * mt * (-r - s - u - 2);
    N[1] = 0.125 * pr * ms * mt * (r - s - u - 2);
    N[2] = 0.125 * pr * ps * mt * (r + s - u - 2);
    N[3] = 0.125 * mr * ps * mt * (-r + s - u - 2);
    N[4] = 0.125 * mr * ms * pt * (-r - s + u - 2);
    N[5] = 0.125 * pr * ms * pt * (r - s + u - 2);
    N[6] = 0.125 * pr * ps * pt * (r + s + u - 2);
    N[7] = 0.125 * mr * ps * pt * (-r + s + u - 2);
    N[8] = 0.25 * qr * ms * mt;
    N[9] = 0.25 * pr * qs * mt;
    N[10] = 0.25 * qr * ps * mt;
    N[11] = 0.25 * mr * qs * mt;
    N[12] = 0.25 * mr * ms * qt;
    N[13] = 0.25 * pr * ms * qt;
    N[14] = 0.25 * pr * ps * qt;
    N[15] = 0.25 * mr * ps * qt;
    N[16] = 0.25 * qr * ms * pt;
    N[17] = 0.25 * pr * qs * pt;
    N[18] = 0.25 * qr * ps * pt;
    N[19] = 0.25 * mr * qs * pt;
    const double d[20][3] = {
            {0.125 * ms * mt * (2 * r + s + u + 1), 0.125 * mr * mt * (r + 2 * s + u + 1),
             0.125 * mr * ms * (r + s + 2 * u + 1)},
            {0.125 * ms * mt * (2 * r - s - u - 1), -0.125 * pr * mt * (r - 2 * s - u - 1),
             -0.125 * pr * ms * (r - s - 2 * u - 1)},
            {0.125 * ps * mt * (2 * r + s - u - 1), 0.125 * pr * mt * (r + 2 * s - u - 1),
             -0.125 * pr * ps * (r + s - 2 * u - 1)},
            {0.125 * ps * mt * (2 * r - s + u + 1), -0.125 * mr * mt * (r - 2 * s + u + 1),
             0.125 * mr * ps * (r - s + 2 * u + 1)},
            {0.125 * ms * pt * (2 * r + s - u + 1), 0.125 * mr * pt * (r + 2 * s - u + 1),
             -0.125 * mr * ms * (r + s - 2 * u + 1)},
            {0.125 * ms * pt * (2 * r - s + u - 1), -0.125 * pr * pt * (r - 2 * s + u - 1),
             0.125 * pr * ms * (r - s + 2 * u - 1)},
            {0.125 * ps * pt * (2 * r + s + u - 1), 0.125 * pr * pt * (r + 2 * s + u - 1),
             0.125 * pr * ps * (r + s + 2 * u - 1)},
            {0.125 * ps * pt * (2 * r - s - u + 1), -0.125 * mr * pt * (r - 2 * s - u + 1),
             -0.125 * mr * ps * (r - s - 2 * u + 1)},
            {-0.5 * r * ms * mt, -0.25 * qr * mt, -0.25 * qr * ms},
            {0.25 * qs * mt, -0.5 * s * pr * mt, -0.25 * pr * qs},
            {-0.5 * r * ps * mt, 0.25 * qr * mt, -0.25 * qr * ps},
            {-0.25 * qs * mt, -0.5 * s * mr * mt, -0.25 * mr * qs},
            {-0.25 * ms * qt, -0.25 * mr * qt, -0.5 * u * mr * ms},
            {0.25 * ms * qt, -0.25 * pr * qt, -0.5 * u * pr * ms},
            {0.25 * ps * qt, 0.25 * pr * qt, -0.5 * u * pr * ps},
            {-0.25 * ps * qt, 0.25 * mr * qt, -0.5 * u * mr * ps},
            {-0.5 * r * ms * pt, -0.25 * qr * pt, 0.25 * qr * ms},
            {0.25 * qs * pt, -0.5 * s * pr * pt, 0.25 * pr * qs},
            {-0.5 * r * ps * pt, 0.25 * qr * pt, 0.25 * qr * ps},
            {-0.25 * qs * pt, -0.5 * s * mr * pt, 0.25 * mr * qs}};
    for (int i = 0; i < 20; ++i)
        for (int j = 0; j < 3; ++j)
            dN[i * 3 + j] = d[i][j];
}

// ------------------------------------------------------------------------------------------------
// Jacobian: nuto/mechanics/cell/Jacobian.h:16-48 (interpolation dim == global dim), :97-100
// ------------------------------------------------------------------------------------------------
struct Jacobian
{
    int dim = 0;
    double J[3][3] = {};
    double inv[3][3] = {};
    double det = 0;
};

//! X[n*dim + i] node coordinates, dN[n*3 + j] natural derivatives
inline Jacobian ComputeJacobian(int dim, int nNodes, const double* X, const double* dN)
{
    Jacobian jac;
    jac.dim = dim;
    for (int i = 0; i < dim; ++i)
        for (int j = 0; j < dim; ++j)
        {
            double s = 0;
            for (int n = 0; n < nNodes; ++n)
                s += X[n * dim + i] * dN[n * 3 + j];
            jac.J[i][j] = s;
        }
    if (dim == 2)
    {
        const double a = jac.J[0][0], b = jac.J[0][1], c = jac.J[1][0], d = jac.J[1][1];
        jac.det = a * d - b * c;
        jac.inv[0][0] = d / jac.det;
        jac.inv[0][1] = -b / jac.det;
        jac.inv[1][0] = -c / jac.det;
        jac.inv[1][1] = a / jac.det;
    }
    else
    {
        const double(&m)[3][3] = jac.J;
        const double c00 = m[1][1] * m[2][2] - m[1][2] * m[2][1];
        const double c10 = m[1][2] * m[2][0] - m[1][0] * m[2][2];
        const double c20 = m[1][0] * m[2][1] - m[1][1] * m[2][0];
        jac.det = m[0][0] * c00 + m[0][1] * c10 + m[0][2] * c20;
        const double id = 1. / jac.det;
        jac.inv[0][0] = c00 * id;
        jac.inv[1][0] = c10 * id;
        jac.inv[2][0] = c20 * id;
        jac.inv[0][1] = (m[0][2] * m[2][1] - m[0][1] * m[2][2]) * id;
        jac.inv[1][1] = (m[0][0] * m[2][2] - m[0][2] * m[2][0]) * id;
        jac.inv[2][1] = (m[0][1] * m[2][0] - m[0][0] * m[2][1]) * id;
        jac.inv[0][2] = (m[0][1] * m[1][2] - m[0][2] * m[1][1]) * id;
        jac.inv[1][2] = (m[0][2] * m[1][0] - m[0][0] * m[1][2]) * id;
        jac.inv[2][2] = (m[0][0] * m[1][1] - m[0][1] * m[1][0]) * id;
    }
    return jac;
}

//! dNdX[n*3 + k] = sum_j dN[n*3 + j] * inv[j][k]  (Jacobian::TransformDerivativeShapeFunctions)
inline void GlobalDerivatives(const Jacobian& jac, int nNodes, const double* dN, double* dNdX)
{
    for (int n = 0; n < nNodes; ++n)
        for (int k = 0; k < 3; ++k)
        {
            double s = 0;
            if (k < jac.dim)
                for (int j = 0; j < jac.dim; ++j)
                    s += dN[n * 3 + j] * jac.inv[j][k];
            dNdX[n * 3 + k] = s;
        }
}

// ------------------------------------------------------------------------------------------------
// Small dense matrix (row-major, dynamic) used by the integrands
// ------------------------------------------------------------------------------------------------
struct Mat
{
    int r = 0, c = 0;
    std::vector<double> v;
    Mat() = default;
    Mat(int rows, int cols)
        : r(rows)
        , c(cols)
        , v(static_cast<size_t>(rows) * cols, 0.)
    {
    }
    double& operator()(int i, int j)
    {
        return v[static_cast<size_t>(i) * c + j];
    }
    double operator()(int i, int j) const
    {
        return v[static_cast<size_t>(i) * c + j];
    }
};

inline Mat Mul(const Mat& a, const Mat& b)
{
    Mat out(a.r, b.c);
    for (int i = 0; i < a.r; ++i)
        for (int k = 0; k < a.c; ++k)
        {
            const double aik = a(i, k);
            if (aik == 0)
                continue;
            for (int j = 0; j < b.c; ++j)
                out(i, j) += aik * b(k, j);
        }
    return out;
}
inline Mat T(const Mat& a)
{
    Mat out(a.c, a.r);
    for (int i = 0; i < a.r; ++i)
        for (int j = 0; j < a.c; ++j)
            out(j, i) = a(i, j);
    return out;
}

// B operators: nuto/mechanics/cell/DifferentialOperators.h:16-90 (Voigt 3D: xx, yy, zz, yz, zx, xy)
inline Mat BStrain(int dim, int nNodes, const double* dNdX)
{
    if (dim == 2)
    {
        Mat B(3, nNodes * 2);
        for (int n = 0; n < nNodes; ++n)
        {
            const double gx = dNdX[n * 3 + 0], gy = dNdX[n * 3 + 1];
            B(0, 2 * n) = gx;
            B(1, 2 * n + 1) = gy;
            B(2, 2 * n) = gy;
            B(2, 2 * n + 1) = gx;
        }
        return B;
    }
    Mat B(6, nNodes * 3);
    for (int n = 0; n < nNodes; ++n)
    {
        const double gx = dNdX[n * 3 + 0], gy = dNdX[n * 3 + 1], gz = dNdX[n * 3 + 2];
        const int c = 3 * n;
        B(0, c) = gx;
        B(1, c + 1) = gy;
        B(2, c + 2) = gz;
        B(3, c + 1) = gz;
        B(3, c + 2) = gy;
        B(4, c) = gz;
        B(4, c + 2) = gx;
        B(5, c) = gy;
        B(5, c + 1) = gx;
    }
    return B;
}
inline Mat BGradient(int dim, int nNodes, const double* dNdX)
{
    Mat B(dim, nNodes);
    for (int n = 0; n < nNodes; ++n)
        for (int k = 0; k < dim; ++k)
            B(k, n) = dNdX[n * 3 + k];
    return B;
}
// Matrix::N: nuto/mechanics/cell/Matrix.h:8-14
inline Mat NMatrix(const double* N, int nNodes, int ncomp)
{
    Mat m(ncomp, ncomp * nNodes);
    for (int i = 0; i < nNodes; ++i)
        for (int c = 0; c < ncomp; ++c)
            m(c, i * ncomp + c) = N[i];
    return m;
}

// ------------------------------------------------------------------------------------------------
// Constitutive laws
// ------------------------------------------------------------------------------------------------
enum PlaneState
{
    PLANE_STRESS = 0,
    PLANE_STRAIN = 1
};
enum DamageApplication
{
    FULL = 0,
    UNILATERAL = 1
};

inline int VoigtDim(int dim)
{
    return dim == 1 ? 1 : (dim == 2 ? 3 : 6);
}

// LinearElastic::CalculateC: nuto/mechanics/constitutive/LinearElastic.h:47-121
inline Mat LinearElasticC(int dim, double E, double nu, int planeState)
{
    if (dim == 1)
    {
        Mat C(1, 1);
        C(0, 0) = E;
        return C;
    }
    double c11, c12, c33;
    auto coeff3D = [&]() {
        double f = E / ((1.0 + nu) * (1.0 - 2.0 * nu));
        c11 = f * (1.0 - nu);
        c12 = f * nu;
        c33 = E / (2. * (1.0 + nu));
    };
    if (dim == 2)
    {
        if (planeState == PLANE_STRESS)
        {
            double f = E / (1.0 - (nu * nu));
            c11 = f;
            c12 = f * nu;
            c33 = f * 0.5 * (1.0 - nu);
        }
        else
            coeff3D();
        Mat C(3, 3);
        C(0, 0) = c11;
        C(1, 0) = c12;
        C(0, 1) = c12;
        C(1, 1) = c11;
        C(2, 2) = c33;
        return C;
    }
    coeff3D();
    Mat C(6, 6);
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j)
            C(i, j) = (i == j) ? c11 : c12;
    for (int i = 3; i < 6; ++i)
        C(i, i) = c33;
    return C;
}

// LinearElasticDamage: nuto/mechanics/constitutive/LinearElasticDamage.h:32-122
struct LinearElasticDamage
{
    int dim = 3;
    int vd = 6;
    double m3K = 0, m2G = 0;
    int app = FULL;
    double D[6] = {}, D2[6] = {}, Pinv[6] = {};
    double Iv[6][6] = {}, PinvId[6][6] = {};

    LinearElasticDamage() = default;
    LinearElasticDamage(int d, double E, double nu, int damageApplication, int planeState)
        : dim(d)
        , vd(VoigtDim(d))
        , m3K(3 * E / (3 - 6 * nu))
        , m2G(2 * E / (2 + 2 * nu))
        , app(damageApplication)
    {
        if (dim == 1)
        {
            m3K = E;
            m2G = E;
        }
        for (int i = 0; i < vd; ++i)
        {
            D[i] = i < dim ? 1. : 0.;
            D2[i] = D[i];
            Pinv[i] = i < dim ? 1. : 0.5;
        }
        if (dim == 2 && planeState == PLANE_STRESS)
            for (int i = 0; i < vd; ++i)
                D2[i] *= (1 + nu / (nu - 1));
        for (int i = 0; i < vd; ++i)
            for (int j = 0; j < vd; ++j)
                Iv[i][j] = 1. / 3. * D[i] * D2[j];
        for (int i = 0; i < vd; ++i)
            for (int j = 0; j < vd; ++j)
                PinvId[i][j] = Pinv[i] * ((i == j ? 1. : 0.) - Iv[i][j]);
    }

    double H(double eV) const
    {
        if (app == UNILATERAL)
            return eV < 0 ? 0 : 1;
        return 1;
    }
    double VolStrain(const double* e) const
    {
        double s = 0;
        for (int i = 0; i < vd; ++i)
            s += D2[i] * e[i];
        return 1. / 3. * s;
    }
    void Stress(const double* strain, double omega, double* out) const
    {
        const double eV = VolStrain(strain);
        const double sV = (1. - omega * H(eV)) * m3K * eV;
        for (int i = 0; i < vd; ++i)
        {
            const double e = strain[i] - D[i] * eV;
            out[i] = D[i] * sV + (1. - omega) * m2G * Pinv[i] * e;
        }
    }
    void DstressDstrain(const double* strain, double omega, double* out /* vd x vd */) const
    {
        const double eV = VolStrain(strain);
        const double a = m3K * (1. - omega * H(eV));
        const double b = (1. - omega) * m2G;
        for (int i = 0; i < vd; ++i)
            for (int j = 0; j < vd; ++j)
                out[i * vd + j] = a * Iv[i][j] + b * PinvId[i][j];
    }
    void DstressDomega(const double* strain, double, double* out) const
    {
        const double eV = VolStrain(strain);
        const double dsV = -m3K * eV * H(eV);
        for (int i = 0; i < vd; ++i)
        {
            const double e = strain[i] - D[i] * eV;
            out[i] = D[i] * dsV - m2G * Pinv[i] * e;
        }
    }
};

// ModifiedMisesStrainNorm: nuto/mechanics/constitutive/ModifiedMisesStrainNorm.h:70-268,
// strain invariants: nuto/mechanics/constitutive/EngineeringStrainInvariants.h:32-71
struct ModifiedMises
{
    int dim = 3;
    double nu = 0, k = 10;
    int ps = PLANE_STRAIN;
    double K1 = 0, K2 = 0;

    ModifiedMises() = default;
    ModifiedMises(int d, double nu_, double k_, int planeState)
        : dim(d)
        , nu(nu_)
        , k(k_)
        , ps(planeState)
        , K1((k_ - 1.) / (2. * k_ * (1 - 2 * nu_)))
        , K2(3. / (k_ * (1. + nu_) * (1. + nu_)))
    {
    }

    void Strain3D(const double* s, double* v) const
    {
        for (int i = 0; i < 6; ++i)
            v[i] = 0;
        if (dim == 1)
        {
            v[0] = s[0];
            v[1] = -nu * s[0];
            v[2] = -nu * s[0];
        }
        else if (dim == 2)
        {
            v[0] = s[0];
            v[1] = s[1];
            v[2] = (ps == PLANE_STRESS) ? nu / (nu - 1.) * (s[0] + s[1]) : 0.;
            v[5] = s[2];
        }
        else
            for (int i = 0; i < 6; ++i)
                v[i] = s[i];
    }
    static double I1(const double* v)
    {
        return v[0] + v[1] + v[2];
    }
    static double J2(const double* v)
    {
        const double xx = v[0], yy = v[1], zz = v[2];
        const double yz = .5 * v[3], zx = .5 * v[4], xy = .5 * v[5];
        return 1. / 6. * ((xx - yy) * (xx - yy) + (yy - zz) * (yy - zz) + (zz - xx) * (zz - xx)) + xy * xy +
               yz * yz + zx * zx;
    }
    double Value(const double* strain) const
    {
        double v[6];
        Strain3D(strain, v);
        const double i1 = I1(v), j2 = J2(v);
        const double A = std::sqrt(K1 * K1 * i1 * i1 + K2 * j2);
        return K1 * i1 + A;
    }
    void Derivative(const double* s, double* d) const
    {
        double v[6];
        Strain3D(s, v);
        const double i1 = I1(v), j2 = J2(v);
        const double A = std::sqrt(K1 * K1 * i1 * i1 + K2 * j2);
        if (dim == 1)
        {
            const double dJ2 = 2. / 3. * s[0] * (1 + nu) * (1 + nu);
            const double dI1 = (1 - 2 * nu);
            d[0] = (A == 0) ? K1 * dI1 : K1 * dI1 + 1. / (2 * A) * (2 * K1 * K1 * i1 * dI1 + K2 * dJ2);
            return;
        }
        if (dim == 2)
        {
            if (ps == PLANE_STRAIN)
            {
                if (A == 0)
                {
                    d[0] = K1;
                    d[1] = K1;
                    d[2] = 0;
                }
                else
                {
                    const double dxx = 1. / 3. * (2 * s[0] - s[1]);
                    const double dyy = 1. / 3. * (2 * s[1] - s[0]);
                    const double dxy = 0.5 * s[2];
                    d[0] = K1 + 1. / (2 * A) * (2 * K1 * K1 * i1 + K2 * dxx);
                    d[1] = K1 + 1. / (2 * A) * (2 * K1 * K1 * i1 + K2 * dyy);
                    d[2] = 1. / (2 * A) * (K2 * dxy);
                }
            }
            else
            {
                const double dI1 = (1 + nu / (nu - 1));
                if (A == 0)
                {
                    d[0] = dI1 * K1;
                    d[1] = dI1 * K1;
                    d[2] = 0;
                }
                else
                {
                    const double sz = nu / (nu - 1.) * (s[0] + s[1]);
                    const double dxx = 1. / 3. * (2. * s[0] - s[1] - 2. * sz + 2 * nu / (nu - 1) * sz);
                    const double dyy = 1. / 3. * (2. * s[1] - s[0] - 2. * sz + 2 * nu / (nu - 1) * sz);
                    const double dxy = .5 * s[2];
                    d[0] = dI1 * K1 + 1. / (2. * A) * (2. * dI1 * K1 * K1 * i1 + K2 * dxx);
                    d[1] = dI1 * K1 + 1. / (2. * A) * (2. * dI1 * K1 * K1 * i1 + K2 * dyy);
                    d[2] = 1. / (2. * A) * (K2 * dxy);
                }
            }
            return;
        }
        if (A == 0)
        {
            d[0] = d[1] = d[2] = K1;
            d[3] = d[4] = d[5] = 0;
            return;
        }
        const double dxx = 1. / 3. * (2 * s[0] - s[1] - s[2]);
        const double dyy = 1. / 3. * (2 * s[1] - s[0] - s[2]);
        const double dzz = 1. / 3. * (2 * s[2] - s[0] - s[1]);
        d[0] = K1 + 1. / (2 * A) * (2 * K1 * K1 * i1 + K2 * dxx);
        d[1] = K1 + 1. / (2 * A) * (2 * K1 * K1 * i1 + K2 * dyy);
        d[2] = K1 + 1. / (2 * A) * (2 * K1 * K1 * i1 + K2 * dzz);
        d[3] = 1. / (2 * A) * K2 * 0.5 * s[3];
        d[4] = 1. / (2 * A) * K2 * 0.5 * s[4];
        d[5] = 1. / (2 * A) * K2 * 0.5 * s[5];
    }
};

// DamageLawExponential: nuto/mechanics/constitutive/damageLaws/DamageLawExponential.h:26-52
struct DamageExponential
{
    double kappa0 = 1e-4, beta = 100, alpha = 0.99;
    double Damage(double kappa) const
    {
        if (kappa < kappa0)
            return 0.;
        return 1 - kappa0 / kappa * (1 - alpha + alpha * std::exp(beta * (kappa0 - kappa)));
    }
    double Derivative(double kappa) const
    {
        if (kappa < kappa0)
            return 0.;
        return kappa0 / kappa * ((1 / kappa + beta) * alpha * std::exp(beta * (kappa0 - kappa)) + (1 - alpha) / kappa);
    }
    // partial derivatives of Damage in the law's parameters (kappa held), from the closed form above; zero below
    // kappa0 where the damage is identically zero (adjoint of the damage parameters only)
    double DKappa0(double kappa) const
    {
        if (kappa < kappa0)
            return 0.;
        const double x = std::exp(beta * (kappa0 - kappa));
        return -(1 - alpha + alpha * x) / kappa - kappa0 / kappa * alpha * beta * x;
    }
    double DBeta(double kappa) const
    {
        if (kappa < kappa0)
            return 0.;
        return -kappa0 / kappa * alpha * (kappa0 - kappa) * std::exp(beta * (kappa0 - kappa));
    }
};

// NonlocalInteraction::Constant / Decreasing: nuto/mechanics/integrands/GradientDamage.h:153-184
struct Interaction
{
    int kind = 0; // 0 constant, 1 decreasing
    double R = 0.005, eta = 5;
    double Factor(double omega) const
    {
        if (kind == 0)
            return 1;
        return ((1. - R) * std::exp(-eta * omega) + R - std::exp(-eta)) / (1. - std::exp(-eta));
    }
    double Derivative(double omega) const
    {
        if (kind == 0)
            return 0;
        return ((1. - R) * std::exp(-eta * omega)) / (1. - std::exp(-eta)) * -eta;
    }
};

// ------------------------------------------------------------------------------------------------
// Integrand parameters (plain C struct, shared with the C API)
// ------------------------------------------------------------------------------------------------
enum IntegrandKind
{
    MB_LINEAR_ELASTIC = 0, // MomentumBalance<D> + LinearElastic<D>
    MB_LOCAL_DAMAGE = 1, // MomentumBalance<D> + LocalIsotropicDamage<D> (EvolutionImplicit)
    GRADIENT_DAMAGE = 2 // GradientDamage<D, Constant|Decreasing, DamageLawExponential>
};

// integration-point quantities of EvalIp (Cell::Eval post-processing)
enum IpQuantity
{
    IP_KAPPA = 0,
    IP_DAMAGE = 1,
    IP_STRAIN = 2,
    IP_STRESS = 3,
    IP_EEQ = 4
};

struct IntegrandParams
{
    int kind;
    int dim;
    double E, nu;
    int plane_state;
    int damage_application;
    double kappa0, beta, alpha;
    double k;
    double c;
    int interaction;
    double R, eta;
};

// ------------------------------------------------------------------------------------------------
// Mesh + DOF layers: UnitMeshFem.cpp:36-125, MeshFemDofConvert.cpp:10-218, MeshFem.cpp:95-123,
// DofNumbering.cpp:7-58, ElementFem.h:33-75
// ------------------------------------------------------------------------------------------------
struct DofLayer
{
    int ncomp = 1;
    int interp = HEX8;
    int nEn = 8;
    int nNodes = 0;
    std::vector<int> conn; // nEl x nEn, DOF-node ids in creation order
    std::vector<double> nodeXYZ; // nNodes x 3 global coordinates of the DOF nodes
    std::vector<int> dofNumber; // nNodes x ncomp (DofNumbering::Build over NodesTotal(dof))
};

struct Mesh
{
    int dim = 3;
    int geoInterp = HEX8;
    int nGeoEn = 8;
    int nEl = 0;
    std::vector<double> coords; // coordinate nodes (dim each)
    std::vector<int> conn; // nEl x nGeoEn
    std::vector<DofLayer> layers;

    void ElementCoords(int e, double* X) const
    {
        for (int n = 0; n < nGeoEn; ++n)
            for (int d = 0; d < dim; ++d)
                X[n * dim + d] = coords[static_cast<size_t>(conn[static_cast<size_t>(e) * nGeoEn + n]) * dim + d];
    }
};

inline Mesh CreateQuads(int nx, int ny)
{
    Mesh m;
    m.dim = 2;
    m.geoInterp = QUAD4;
    m.nGeoEn = 4;
    for (int iy = 0; iy < ny + 1; ++iy)
        for (int ix = 0; ix < nx + 1; ++ix)
        {
            m.coords.push_back(static_cast<double>(ix) / nx);
            m.coords.push_back(static_cast<double>(iy) / ny);
        }
    for (int iy = 0; iy < ny; ++iy)
        for (int ix = 0; ix < nx; ++ix)
        {
            m.conn.push_back(ix + iy * (nx + 1));
            m.conn.push_back(ix + 1 + iy * (nx + 1));
            m.conn.push_back(ix + 1 + (iy + 1) * (nx + 1));
            m.conn.push_back(ix + (iy + 1) * (nx + 1));
        }
    m.nEl = nx * ny;
    return m;
}

inline Mesh CreateBricks(int nx, int ny, int nz)
{
    Mesh m;
    m.dim = 3;
    m.geoInterp = HEX8;
    m.nGeoEn = 8;
    const int X = nx + 1, Y = ny + 1, Z = nz + 1;
    for (int iz = 0; iz < Z; ++iz)
        for (int iy = 0; iy < Y; ++iy)
            for (int ix = 0; ix < X; ++ix)
            {
                m.coords.push_back(static_cast<double>(ix) / nx);
                m.coords.push_back(static_cast<double>(iy) / ny);
                m.coords.push_back(static_cast<double>(iz) / nz);
            }
    for (int iz = 0; iz < nz; ++iz)
        for (int iy = 0; iy < ny; ++iy)
            for (int ix = 0; ix < nx; ++ix)
            {
                const int b = ix + iy * X + iz * X * Y;
                const int u = b + X * Y;
                const int c[8] = {b, b + 1, b + 1 + X, b + X, u, u + 1, u + 1 + X, u + X};
                for (int i = 0; i < 8; ++i)
                    m.conn.push_back(c[i]);
            }
    m.nEl = nx * ny * nz;
    return m;
}

//! Interpolate(coordinateElement, xi) = N(xi) * X   (ElementInterface.h:31-34)
inline void InterpolateGeometry(const Mesh& m, int e, const double* xi, double* out3)
{
    double N[20], dN[60], X[60];
    Shape(m.geoInterp, xi, N, dN);
    m.ElementCoords(e, X);
    out3[0] = out3[1] = out3[2] = 0;
    for (int d = 0; d < m.dim; ++d)
    {
        double s = 0;
        for (int n = 0; n < m.nGeoEn; ++n)
            s += N[n] * X[n * m.dim + d];
        out3[d] = s;
    }
}

//! SubBoxes coordinate hash (MeshFemDofConvert.cpp:10-113) + AddDofInterpolation (:164-210).
//! DOF nodes are created in first-touch element order; an existing node within eps=1e-10 is reused.
inline int AddDofInterpolation(Mesh& m, int ncomp, int interp)
{
    if (interp < 0)
        interp = m.geoInterp;
    if (InterpDim(interp) != InterpDim(m.geoInterp))
        throw std::runtime_error("shape of interpolation and coordinate element don't match");
    const double eps = 1.e-10;
    const int boxes = 300;
    double start[3], end[3];
    {
        double xi[3] = {0, 0, 0};
        LocalCoords(m.geoInterp, 0, xi);
        // start = end = coordinates of node 0 of element 0
        for (int d = 0; d < 3; ++d)
            start[d] = end[d] = 0;
        for (int d = 0; d < m.dim; ++d)
            start[d] = end[d] = m.coords[static_cast<size_t>(m.conn[0]) * m.dim + d];
        for (int e = 0; e < m.nEl; ++e)
            for (int n = 0; n < m.nGeoEn; ++n)
                for (int d = 0; d < m.dim; ++d)
                {
                    const double x = m.coords[static_cast<size_t>(m.conn[static_cast<size_t>(e) * m.nGeoEn + n]) * m.dim + d];
                    start[d] = std::min(start[d], x);
                    end[d] = std::max(end[d], x);
                }
    }
    int subs[3] = {1, 1, 1};
    double delta[3];
    for (int d = 0; d < 3; ++d)
    {
        start[d] -= eps;
        end[d] += eps;
        if (d < m.dim)
            subs[d] = boxes;
        delta[d] = (end[d] - start[d]) / subs[d];
    }
    std::vector<std::vector<std::pair<std::array<double, 3>, int>>> data(static_cast<size_t>(subs[0]) * subs[1] * subs[2]);
    auto boxIndex = [&](int i, int j, int k) { return i + j * subs[0] + k * subs[1] * subs[0]; };

    DofLayer L;
    L.ncomp = ncomp;
    L.interp = interp;
    L.nEn = NumNodes(interp);
    L.conn.resize(static_cast<size_t>(m.nEl) * L.nEn);
    for (int e = 0; e < m.nEl; ++e)
        for (int n = 0; n < L.nEn; ++n)
        {
            double xi[3], x[3];
            LocalCoords(interp, n, xi);
            InterpolateGeometry(m, e, xi, x);
            const int i = static_cast<int>((x[0] - start[0]) / delta[0]);
            const int j = static_cast<int>((x[1] - start[1]) / delta[1]);
            const int k = static_cast<int>((x[2] - start[2]) / delta[2]);
            int found = -1;
            for (int kk : {k, k - 1, k + 1})
                for (int jj : {j, j - 1, j + 1})
                    for (int ii : {i, i - 1, i + 1})
                    {
                        if (found >= 0)
                            break;
                        if (ii < 0 || ii >= subs[0] || jj < 0 || jj >= subs[1] || kk < 0 || kk >= subs[2])
                            continue;
                        for (auto& entry : data[boxIndex(ii, jj, kk)])
                        {
                            const double dx = entry.first[0] - x[0], dy = entry.first[1] - x[1],
                                         dz = entry.first[2] - x[2];
                            if (dx * dx + dy * dy + dz * dz < eps * eps)
                            {
                                found = entry.second;
                                break;
                            }
                        }
                    }
            if (found < 0)
            {
                found = L.nNodes++;
                data[boxIndex(i, j, k)].push_back({{x[0], x[1], x[2]}, found});
                L.nodeXYZ.insert(L.nodeXYZ.end(), {x[0], x[1], x[2]});
            }
            L.conn[static_cast<size_t>(e) * L.nEn + n] = found;
        }
    // DofNumbering::Build over MeshFem::NodesTotal(dof): Group insertion order over elements/local nodes,
    // then consecutive numbers per node and component (DofNumbering.cpp:7-14, MeshFem.cpp:104-115).
    L.dofNumber.assign(static_cast<size_t>(L.nNodes) * ncomp, -1);
    std::vector<char> seen(L.nNodes, 0);
    int next = 0;
    for (int e = 0; e < m.nEl; ++e)
        for (int n = 0; n < L.nEn; ++n)
        {
            const int node = L.conn[static_cast<size_t>(e) * L.nEn + n];
            if (seen[node])
                continue;
            seen[node] = 1;
            for (int c = 0; c < ncomp; ++c)
                L.dofNumber[static_cast<size_t>(node) * ncomp + c] = next++;
        }
    m.layers.push_back(std::move(L));
    return static_cast<int>(m.layers.size()) - 1;
}

//! MeshFem::NodesAtAxis(direction, dof, offset, tol) (MeshFem.cpp:72-93): Group insertion order.
inline std::vector<int> NodesAtAxis(const Mesh& m, int layer, int dir, double offset, double tol = 1.e-10)
{
    const DofLayer& L = m.layers[layer];
    std::vector<int> out;
    std::vector<char> seen(L.nNodes, 0);
    for (int e = 0; e < m.nEl; ++e)
        for (int n = 0; n < L.nEn; ++n)
        {
            const int node = L.conn[static_cast<size_t>(e) * L.nEn + n];
            if (std::abs(L.nodeXYZ[static_cast<size_t>(node) * 3 + dir] - offset) < tol && !seen[node])
            {
                seen[node] = 1;
                out.push_back(node);
            }
        }
    return out;
}

// ------------------------------------------------------------------------------------------------
// Problem: cells (CellStorage::AddCells, consecutive ids), integrand, history, assembly
// ------------------------------------------------------------------------------------------------
struct CellResult
{
    // combined local layout: slot-major, then node, then component (ElementFem::GetDofNumbering)
    std::vector<double> f; // nLocal
    std::vector<double> K; // nLocal x nLocal
};

struct Problem
{
    const Mesh* mesh = nullptr;
    Quadrature q;
    std::vector<int> slots; // layers in the order of the `dofs` vector, e.g. {disp, eeq}
    IntegrandParams p{};
    std::vector<double> kappa; // nEl x nIp, the public mKappas member of the integrand / evolution
    // per-cell Young's modulus as a multiple of p.E (empty: 1 everywhere). The laws are linear in E, so the stress
    // and its derivatives scale with it; the equivalent strain and the eeq equation do not depend on E.
    std::vector<double> eScale;
    double EScale(int e) const
    {
        return eScale.empty() ? 1. : eScale[static_cast<size_t>(e)];
    }
    std::vector<int64_t> slotOffset; // combined global offset per slot (DofVectorConvertEigen.h:21-53)
    int64_t nDofs = 0;
    std::vector<int> localOffset; // local offset per slot inside a cell vector
    int nLocal = 0;

    LinearElasticDamage led;
    ModifiedMises norm;
    DamageExponential dmg;
    Interaction inter;
    Mat Cel;

    void Init()
    {
        const Mesh& m = *mesh;
        slotOffset.clear();
        localOffset.clear();
        nDofs = 0;
        nLocal = 0;
        for (int s : slots)
        {
            const DofLayer& L = m.layers[s];
            slotOffset.push_back(nDofs);
            nDofs += static_cast<int64_t>(L.nNodes) * L.ncomp;
            localOffset.push_back(nLocal);
            nLocal += L.nEn * L.ncomp;
        }
        kappa.assign(static_cast<size_t>(m.nEl) * q.n, 0.);
        led = LinearElasticDamage(p.dim, p.E, p.nu, p.damage_application, p.plane_state);
        norm = ModifiedMises(p.dim, p.nu, p.k, p.plane_state);
        dmg.kappa0 = p.kappa0;
        dmg.beta = p.beta;
        dmg.alpha = p.alpha;
        inter.kind = p.interaction;
        inter.R = p.R;
        inter.eta = p.eta;
        Cel = LinearElasticC(p.dim, p.E, p.nu, p.plane_state);
    }

    //! global combined DOF indices of a cell, slot-major (CellInterface::DofNumbering per dof type)
    void CellDofs(int e, std::vector<int64_t>& out) const
    {
        out.resize(nLocal);
        for (size_t s = 0; s < slots.size(); ++s)
        {
            const DofLayer& L = mesh->layers[slots[s]];
            for (int n = 0; n < L.nEn; ++n)
                for (int c = 0; c < L.ncomp; ++c)
                    out[localOffset[s] + n * L.ncomp + c] =
                            slotOffset[s] +
                            L.dofNumber[static_cast<size_t>(L.conn[static_cast<size_t>(e) * L.nEn + n]) * L.ncomp + c];
        }
    }

    //! Cell::IntegrateGeneric (Cell.h:105-119) of the integrand's Gradient (and Hessian0 if wantK).
    //! u is the combined global DOF vector (NodalValueMerger::Merge + CellData::GetNodeValues).
    void IntegrateCell(int e, const double* u, bool wantF, bool wantK, CellResult& res) const
    {
        const Mesh& m = *mesh;
        const int dim = m.dim;
        const int vd = VoigtDim(dim);
        res.f.assign(nLocal, 0.);
        if (wantK)
            res.K.assign(static_cast<size_t>(nLocal) * nLocal, 0.);
        double X[60];
        m.ElementCoords(e, X);
        std::vector<int64_t> dofs;
        CellDofs(e, dofs);
        std::vector<double> ue(nLocal);
        for (int i = 0; i < nLocal; ++i)
            ue[i] = u[dofs[i]];

        const DofLayer& Ld = m.layers[slots[0]];
        const int nd = Ld.nEn;
        const bool gd = p.kind == GRADIENT_DAMAGE;
        const DofLayer* Le = gd ? &m.layers[slots[1]] : nullptr;
        const int ne = gd ? Le->nEn : 0;
        const int od = localOffset[0], oe = gd ? localOffset[1] : 0;
        const int ndd = nd * dim;

        for (int ip = 0; ip < q.n; ++ip)
        {
            const double* xi = q.points[ip].data();
            const double w = q.weights[ip];
            double Ng[20], dNg[60];
            Shape(m.geoInterp, xi, Ng, dNg);
            const Jacobian jac = ComputeJacobian(dim, m.nGeoEn, X, dNg);
            const double fac = jac.det * w;

            double Nd[20], dNd[60], gd_[60];
            Shape(Ld.interp, xi, Nd, dNd);
            GlobalDerivatives(jac, nd, dNd, gd_);
            const Mat Bd = BStrain(dim, nd, gd_);
            double strain[6] = {0, 0, 0, 0, 0, 0};
            for (int r = 0; r < vd; ++r)
                for (int j = 0; j < ndd; ++j)
                    strain[r] += Bd(r, j) * ue[od + j];

            const double kh = kappa[static_cast<size_t>(e) * q.n + ip];

            if (!gd)
            {
                double sigma[6];
                Mat Ct(vd, vd);
                if (p.kind == MB_LINEAR_ELASTIC)
                {
                    for (int r = 0; r < vd; ++r)
                    {
                        sigma[r] = 0;
                        for (int c = 0; c < vd; ++c)
                            sigma[r] += Cel(r, c) * strain[c];
                    }
                    Ct = Cel;
                }
                else
                {
                    // LocalIsotropicDamage::Stress/Tangent (LocalIsotropicDamage.h:52-68) with EvolutionImplicit (:110-133)
                    const double eqs = norm.Value(strain);
                    const double kap = std::max(eqs, kh);
                    const double omega = dmg.Damage(kap);
                    led.Stress(strain, omega, sigma);
                    if (wantK)
                    {
                        const double dOdK = dmg.Derivative(kap);
                        double dK[6] = {0, 0, 0, 0, 0, 0};
                        if (eqs >= kh)
                            norm.Derivative(strain, dK);
                        double dsde[36], dsdw[6];
                        led.DstressDstrain(strain, omega, dsde);
                        led.DstressDomega(strain, omega, dsdw);
                        for (int r = 0; r < vd; ++r)
                            for (int c = 0; c < vd; ++c)
                                Ct(r, c) = dsde[r * vd + c] + dsdw[r] * dOdK * dK[c];
                    }
                }
                const double se = EScale(e);
                for (int r = 0; r < vd; ++r)
                    sigma[r] *= se;
                if (wantF)
                    for (int j = 0; j < ndd; ++j)
                    {
                        double s = 0;
                        for (int r = 0; r < vd; ++r)
                            s += Bd(r, j) * sigma[r];
                        res.f[od + j] += s * fac;
                    }
                if (wantK)
                {
                    for (double& v : Ct.v)
                        v *= se;
                    const Mat K = Mul(T(Bd), Mul(Ct, Bd));
                    for (int i = 0; i < ndd; ++i)
                        for (int j = 0; j < ndd; ++j)
                            res.K[static_cast<size_t>(od + i) * nLocal + od + j] += K(i, j) * fac;
                }
                continue;
            }

            // GradientDamage<D> (GradientDamage.h:70-135)
            double Ne[20], dNe[60], ge[60];
            Shape(Le->interp, xi, Ne, dNe);
            GlobalDerivatives(jac, ne, dNe, ge);
            const Mat Be = BGradient(dim, ne, ge);
            double eeq = 0;
            for (int n = 0; n < ne; ++n)
                eeq += Ne[n] * ue[oe + n];
            double geq[3] = {0, 0, 0};
            for (int k = 0; k < dim; ++k)
                for (int n = 0; n < ne; ++n)
                    geq[k] += Be(k, n) * ue[oe + n];
            const double kap = std::max(kh, eeq);
            const double omega = dmg.Damage(kap);
            const double g = inter.Factor(omega);
            const double se = EScale(e);
            if (wantF)
            {
                double sigma[6];
                led.Stress(strain, omega, sigma);
                for (int r = 0; r < vd; ++r)
                    sigma[r] *= se;
                for (int j = 0; j < ndd; ++j)
                {
                    double s = 0;
                    for (int r = 0; r < vd; ++r)
                        s += Bd(r, j) * sigma[r];
                    res.f[od + j] += s * fac;
                }
                const double diff = eeq - norm.Value(strain);
                for (int n = 0; n < ne; ++n)
                {
                    double s = Ne[n] * diff;
                    for (int k = 0; k < dim; ++k)
                        s += Be(k, n) * (p.c * g * geq[k]);
                    res.f[oe + n] += s * fac;
                }
            }
            if (wantK)
            {
                const double dKdE = eeq >= kh ? 1 : 0;
                const double dOdK = dmg.Derivative(kap);
                const double dgdw = inter.Derivative(omega);
                double dsde[36], dsdw[6], dnorm[6];
                led.DstressDstrain(strain, omega, dsde);
                led.DstressDomega(strain, omega, dsdw);
                for (int r = 0; r < vd; ++r)
                {
                    dsdw[r] *= se;
                    for (int c = 0; c < vd; ++c)
                        dsde[r * vd + c] *= se;
                }
                norm.Derivative(strain, dnorm);
                Mat Cw(vd, vd);
                for (int r = 0; r < vd; ++r)
                    for (int c = 0; c < vd; ++c)
                        Cw(r, c) = dsde[r * vd + c];
                const Mat Kdd = Mul(T(Bd), Mul(Cw, Bd));
                for (int i = 0; i < ndd; ++i)
                    for (int j = 0; j < ndd; ++j)
                        res.K[static_cast<size_t>(od + i) * nLocal + od + j] += Kdd(i, j) * fac;
                // (eeq, disp) = -Ne^T * dnorm^T * Bd
                for (int n = 0; n < ne; ++n)
                    for (int j = 0; j < ndd; ++j)
                    {
                        double s = 0;
                        for (int r = 0; r < vd; ++r)
                            s += dnorm[r] * Bd(r, j);
                        res.K[static_cast<size_t>(oe + n) * nLocal + od + j] += -Ne[n] * s * fac;
                    }
                // (eeq, eeq) = Ne^T Ne + c g Be^T Be + Be^T c geq dgdw dOdK dKdE Ne
                const double sc = p.c * dgdw * dOdK * dKdE;
                for (int a = 0; a < ne; ++a)
                    for (int b = 0; b < ne; ++b)
                    {
                        double bb = 0, bg = 0;
                        for (int k = 0; k < dim; ++k)
                        {
                            bb += Be(k, a) * Be(k, b);
                            bg += Be(k, a) * geq[k];
                        }
                        res.K[static_cast<size_t>(oe + a) * nLocal + oe + b] +=
                                (Ne[a] * Ne[b] + p.c * g * bb + bg * sc * Ne[b]) * fac;
                    }
                // (disp, eeq) = Bd^T (dsdw dOdK dKdE) Ne
                for (int i = 0; i < ndd; ++i)
                {
                    double s = 0;
                    for (int r = 0; r < vd; ++r)
                        s += Bd(r, i) * dsdw[r];
                    s *= dOdK * dKdE;
                    for (int n = 0; n < ne; ++n)
                        res.K[static_cast<size_t>(od + i) * nLocal + oe + n] += s * Ne[n] * fac;
                }
            }
        }
    }

    //! history update after convergence: GradientDamage::Update (GradientDamage.h:122-125) /
    //! EvolutionImplicit::Update (LocalIsotropicDamage.h:130-133), serial Cell::Apply (Cell.h:47-58)
    void UpdateHistory(const double* u)
    {
        const Mesh& m = *mesh;
        if (p.kind == MB_LINEAR_ELASTIC)
            return;
        const int dim = m.dim;
        const int vd = VoigtDim(dim);
        std::vector<int64_t> dofs;
        for (int e = 0; e < m.nEl; ++e)
        {
            double X[60];
            m.ElementCoords(e, X);
            CellDofs(e, dofs);
            const DofLayer& Ld = m.layers[slots[0]];
            for (int ip = 0; ip < q.n; ++ip)
            {
                const double* xi = q.points[ip].data();
                double Ng[20], dNg[60];
                Shape(m.geoInterp, xi, Ng, dNg);
                double& kh = kappa[static_cast<size_t>(e) * q.n + ip];
                if (p.kind == GRADIENT_DAMAGE)
                {
                    const DofLayer& Le = m.layers[slots[1]];
                    double Ne[20], dNe[60];
                    Shape(Le.interp, xi, Ne, dNe);
                    double eeq = 0;
                    for (int n = 0; n < Le.nEn; ++n)
                        eeq += Ne[n] * u[dofs[localOffset[1] + n]];
                    kh = std::max(kh, eeq);
                }
                else
                {
                    const Jacobian jac = ComputeJacobian(dim, m.nGeoEn, X, dNg);
                    double Nd[20], dNd[60], g[60];
                    Shape(Ld.interp, xi, Nd, dNd);
                    GlobalDerivatives(jac, Ld.nEn, dNd, g);
                    const Mat Bd = BStrain(dim, Ld.nEn, g);
                    double strain[6] = {0, 0, 0, 0, 0, 0};
                    for (int r = 0; r < vd; ++r)
                        for (int j = 0; j < Ld.nEn * dim; ++j)
                            strain[r] += Bd(r, j) * u[dofs[localOffset[0] + j]];
                    kh = std::max(norm.Value(strain), kh);
                }
            }
        }
    }

    //! Adjoint ingredients of cell e at the state u (gradient damage only), with the history kappa_h of the step:
    //! D (nLocal x nIp, row-major): column ip is d f_e / d omega_ip, the derivative of the cell vector with respect
    //!   to the damage at integration point ip with everything else held (displacement rows B^T dsigma/domega w detJ,
    //!   eeq rows Be^T c g'(omega) grad eeq w detJ);
    //! ipd (nIp x 5): kappa_trial = max(kappa_h, eeq), loading flag [eeq >= kappa_h], d omega/d kappa,
    //!   d omega/d kappa0, d omega/d beta at kappa_trial;
    //! N (nIp x ne): the eeq shape values (d eeq_ip / d eeq nodal values).
    void AdjointCell(int e, const double* u, double* D, double* ipd, double* Nout) const
    {
        const Mesh& m = *mesh;
        const int dim = m.dim;
        const int vd = VoigtDim(dim);
        double X[60];
        m.ElementCoords(e, X);
        std::vector<int64_t> dofs;
        CellDofs(e, dofs);
        const DofLayer& Ld = m.layers[slots[0]];
        const DofLayer& Le = m.layers[slots[1]];
        const int nd = Ld.nEn, ne = Le.nEn, ndd = nd * dim;
        const int od = localOffset[0], oe = localOffset[1];
        const double se = EScale(e);
        for (int i = 0; i < nLocal * q.n; ++i)
            D[i] = 0;
        for (int ip = 0; ip < q.n; ++ip)
        {
            const double* xi = q.points[ip].data();
            double Ng[20], dNg[60];
            Shape(m.geoInterp, xi, Ng, dNg);
            const Jacobian jac = ComputeJacobian(dim, m.nGeoEn, X, dNg);
            const double fac = jac.det * q.weights[ip];
            double Nd[20], dNd[60], gd_[60];
            Shape(Ld.interp, xi, Nd, dNd);
            GlobalDerivatives(jac, nd, dNd, gd_);
            const Mat Bd = BStrain(dim, nd, gd_);
            double strain[6] = {0, 0, 0, 0, 0, 0};
            for (int r = 0; r < vd; ++r)
                for (int j = 0; j < ndd; ++j)
                    strain[r] += Bd(r, j) * u[dofs[od + j]];
            double Ne[20], dNe[60], ge[60];
            Shape(Le.interp, xi, Ne, dNe);
            GlobalDerivatives(jac, ne, dNe, ge);
            const Mat Be = BGradient(dim, ne, ge);
            double eeq = 0, geq[3] = {0, 0, 0};
            for (int n = 0; n < ne; ++n)
            {
                eeq += Ne[n] * u[dofs[oe + n]];
                for (int k = 0; k < dim; ++k)
                    geq[k] += Be(k, n) * u[dofs[oe + n]];
            }
            const double kh = kappa[static_cast<size_t>(e) * q.n + ip];
            const double kap = std::max(kh, eeq);
            const double omega = dmg.Damage(kap);
            double dsdw[6];
            led.DstressDomega(strain, omega, dsdw);
            for (int j = 0; j < ndd; ++j)
            {
                double v = 0;
                for (int r = 0; r < vd; ++r)
                    v += Bd(r, j) * dsdw[r];
                D[static_cast<size_t>(od + j) * q.n + ip] = v * se * fac;
            }
            const double dg = inter.Derivative(omega);
            for (int n = 0; n < ne; ++n)
            {
                double v = 0;
                for (int k = 0; k < dim; ++k)
                    v += Be(k, n) * geq[k];
                D[static_cast<size_t>(oe + n) * q.n + ip] = p.c * dg * v * fac;
                Nout[ip * ne + n] = Ne[n];
            }
            double* o = ipd + ip * 5;
            o[0] = kap;
            o[1] = eeq >= kh ? 1. : 0.;
            o[2] = dmg.Derivative(kap);
            o[3] = dmg.DKappa0(kap);
            o[4] = dmg.DBeta(kap);
        }
    }

    //! DynamicMomentumBalance::Hessian2 (DynamicMomentumBalance.h:22-30) integrated over cell e: the (disp, disp)
    //! block rho N^T N det J w summed over the integration points (Cell.h:105-119), n_en*ncomp square, row-major.
    void MassCell(int e, double rho, std::vector<double>& M) const
    {
        const Mesh& m = *mesh;
        const DofLayer& Ld = m.layers[slots[0]];
        const int nl = Ld.nEn * Ld.ncomp;
        M.assign(static_cast<size_t>(nl) * nl, 0.);
        double X[60];
        m.ElementCoords(e, X);
        for (int ip = 0; ip < q.n; ++ip)
        {
            const double* xi = q.points[ip].data();
            double Ng[20], dNg[60];
            Shape(m.geoInterp, xi, Ng, dNg);
            const Jacobian jac = ComputeJacobian(m.dim, m.nGeoEn, X, dNg);
            double Nd[20], dNd[60];
            Shape(Ld.interp, xi, Nd, dNd);
            const Mat N = NMatrix(Nd, Ld.nEn, Ld.ncomp);
            const Mat NtN = Mul(T(N), N);
            const double fac = jac.det * q.weights[ip];
            for (int i = 0; i < nl * nl; ++i)
                M[i] += NtN.v[i] * rho * fac;
        }
    }

    //! Values at every integration point of cell e (Cell::Eval, Cell.h:80-93), for post-processing:
    //! IP_KAPPA GradientDamage::Kappa / EvolutionImplicit kappa, IP_DAMAGE omega(kappa), IP_STRAIN Nabla::Strain,
    //! IP_STRESS the law's stress, IP_EEQ the nonlocal eeq (gradient damage) or the local equivalent strain.
    //! out: q.n x IpWidth(quantity)
    int IpWidth(int quantity) const
    {
        return (quantity == IP_STRAIN || quantity == IP_STRESS) ? VoigtDim(mesh->dim) : 1;
    }
    void EvalCell(int e, const double* u, int quantity, double* out) const
    {
        const Mesh& m = *mesh;
        const int dim = m.dim;
        const int vd = VoigtDim(dim);
        const int w = IpWidth(quantity);
        double X[60];
        m.ElementCoords(e, X);
        std::vector<int64_t> dofs;
        CellDofs(e, dofs);
        const DofLayer& Ld = m.layers[slots[0]];
        const bool gd = p.kind == GRADIENT_DAMAGE;
        for (int ip = 0; ip < q.n; ++ip)
        {
            const double* xi = q.points[ip].data();
            double Ng[20], dNg[60];
            Shape(m.geoInterp, xi, Ng, dNg);
            const Jacobian jac = ComputeJacobian(dim, m.nGeoEn, X, dNg);
            double Nd[20], dNd[60], g[60];
            Shape(Ld.interp, xi, Nd, dNd);
            GlobalDerivatives(jac, Ld.nEn, dNd, g);
            const Mat Bd = BStrain(dim, Ld.nEn, g);
            double strain[6] = {0, 0, 0, 0, 0, 0};
            for (int r = 0; r < vd; ++r)
                for (int j = 0; j < Ld.nEn * dim; ++j)
                    strain[r] += Bd(r, j) * u[dofs[localOffset[0] + j]];
            const double kh = kappa[static_cast<size_t>(e) * q.n + ip];
            double eqs = 0;
            if (gd)
            {
                const DofLayer& Le = m.layers[slots[1]];
                double Ne[20], dNe[60];
                Shape(Le.interp, xi, Ne, dNe);
                for (int nn = 0; nn < Le.nEn; ++nn)
                    eqs += Ne[nn] * u[dofs[localOffset[1] + nn]];
            }
            else if (p.kind == MB_LOCAL_DAMAGE)
                eqs = norm.Value(strain);
            const double kap = p.kind == MB_LINEAR_ELASTIC ? 0. : std::max(kh, eqs);
            const double omega = p.kind == MB_LINEAR_ELASTIC ? 0. : dmg.Damage(kap);
            double* o = out + static_cast<size_t>(ip) * w;
            switch (quantity)
            {
            case IP_KAPPA:
                o[0] = kap;
                break;
            case IP_DAMAGE:
                o[0] = omega;
                break;
            case IP_EEQ:
                o[0] = p.kind == MB_LINEAR_ELASTIC ? norm.Value(strain) : eqs;
                break;
            case IP_STRAIN:
                for (int r = 0; r < vd; ++r)
                    o[r] = strain[r];
                break;
            case IP_STRESS:
                if (p.kind == MB_LINEAR_ELASTIC)
                    for (int r = 0; r < vd; ++r)
                    {
                        o[r] = 0;
                        for (int c = 0; c < vd; ++c)
                            o[r] += Cel(r, c) * strain[c];
                    }
                else
                    led.Stress(strain, omega, o);
                for (int r = 0; r < vd; ++r)
                    o[r] *= EScale(e);
                break;
            }
        }
    }
};

//! SimpleAssembler::BuildDiagonallyLumpedMatrix (SimpleAssembler.cpp:67-98) for one local block of one DOF type:
//! the diagonal scaled by (sum of all entries / sum of the diagonal) / number of components (DofType::GetNum).
inline void LumpHRZ(const double* M, int nl, int ncomp, double* out)
{
    double diagSum = 0, fullSum = 0;
    for (int i = 0; i < nl; ++i)
        diagSum += M[static_cast<size_t>(i) * nl + i];
    for (int i = 0; i < nl * nl; ++i)
        fullSum += M[i];
    for (int i = 0; i < nl; ++i)
        out[i] = M[static_cast<size_t>(i) * nl + i] * ((fullSum / diagSum) / ncomp);
}

//! BuildDiagonallyLumpedMatrix of DynamicMomentumBalance::Hessian2 over all cells into the combined vector
//! (displacement rows; the other slots stay zero), per-thread partial vectors summed at the end.
inline void BuildLumpedMass(const Problem& P, double rho, double* mvec)
{
    const int64_t n = P.nDofs;
    for (int64_t i = 0; i < n; ++i)
        mvec[i] = 0;
    const DofLayer& Ld = P.mesh->layers[P.slots[0]];
    const int nl = Ld.nEn * Ld.ncomp;
#pragma omp parallel
    {
        std::vector<double> local(n, 0.), M, lump(nl);
        std::vector<int64_t> dofs;
#pragma omp for nowait
        for (int e = 0; e < P.mesh->nEl; ++e)
        {
            P.MassCell(e, rho, M);
            LumpHRZ(M.data(), nl, Ld.ncomp, lump.data());
            P.CellDofs(e, dofs);
            for (int i = 0; i < nl; ++i)
                local[dofs[P.localOffset[0] + i]] += lump[i];
        }
#pragma omp critical
        for (int64_t i = 0; i < n; ++i)
            mvec[i] += local[i];
    }
}

// ------------------------------------------------------------------------------------------------
// Boundary cells: NeumannBc<D>::ExternalLoad (NeumannBc.h:28-36) on line cells in 2D and Quad4 cells in 3D, with
// the codimension-1 Jacobian (Jacobian.h:51-88): det J = |dx/dxi| for lines, |dx/dxi x dx/deta| for surfaces.
// ------------------------------------------------------------------------------------------------
//! shape functions of the boundary cell (Line2 natural coordinate in [-1, 1]; Quad4 as the volume Quad4)
inline void FaceShape(int nfe, const double* xi, double* N, double* dN /* nfe x 2 */)
{
    if (nfe == 2)
    {
        N[0] = 0.5 * (1. - xi[0]);
        N[1] = 0.5 * (1. + xi[0]);
        dN[0] = -0.5;
        dN[2] = 0.5;
        dN[1] = dN[3] = 0;
        return;
    }
    double N4[4], dN4[12];
    Shape(QUAD4, xi, N4, dN4);
    for (int i = 0; i < 4; ++i)
    {
        N[i] = N4[i];
        dN[i * 2 + 0] = dN4[i * 3 + 0];
        dN[i * 2 + 1] = dN4[i * 3 + 1];
    }
}

//! det J of a codimension-1 cell: X is nfe x dim, dN nfe x 2 (natural derivatives)
inline double FaceDetJ(int dim, int nfe, const double* X, const double* dN)
{
    double J[3][2] = {{0, 0}, {0, 0}, {0, 0}};
    const int nd = dim - 1;
    for (int d = 0; d < dim; ++d)
        for (int k = 0; k < nd; ++k)
            for (int i = 0; i < nfe; ++i)
                J[d][k] += X[i * dim + d] * dN[i * 2 + k];
    if (dim == 2)
    {
        // extended [J | n] with n = (J1, -J0) / |J|; det J = -det(extended) = |J|
        const double len = std::sqrt(J[0][0] * J[0][0] + J[1][0] * J[1][0]);
        const double n0 = J[1][0] / len, n1 = -J[0][0] / len;
        return -(J[0][0] * n1 - J[1][0] * n0);
    }
    // n = normalized(J_0 x J_1); det [J_0 J_1 n] = (J_0 x J_1) . n
    const double c0 = J[1][0] * J[2][1] - J[2][0] * J[1][1];
    const double c1 = J[2][0] * J[0][1] - J[0][0] * J[2][1];
    const double c2 = J[0][0] * J[1][1] - J[1][0] * J[0][1];
    const double len = std::sqrt(c0 * c0 + c1 * c1 + c2 * c2);
    return (c0 * c0 + c1 * c1 + c2 * c2) / len;
}

//! NeumannBc::ExternalLoad at one integration point: N^T p (nfe x dim, node-major)
inline void NeumannIp(int nfe, int dim, const double* N, const double* p, double* out)
{
    for (int i = 0; i < nfe; ++i)
        for (int c = 0; c < dim; ++c)
            out[i * dim + c] = N[i] * p[c];
}

//! SimpleAssembler::BuildVector of ExternalLoad over boundary cells into f (combined layout, added):
//! faceCoordConn nFaces x nfe coordinate nodes, faceDofs nFaces x nfe x dim combined DOF indices
inline void BuildExternalLoad(const Mesh& m, int nfe, int nFaces, const int* faceCoordConn, const int64_t* faceDofs,
                              const double* p, int gauss, double* f)
{
    const int dim = m.dim;
    const Quadrature q = TensorGauss(dim - 1, gauss);
    std::vector<double> fe(static_cast<size_t>(nfe) * dim), ipv(static_cast<size_t>(nfe) * dim);
    for (int e = 0; e < nFaces; ++e)
    {
        double X[12];
        for (int i = 0; i < nfe; ++i)
            for (int d = 0; d < dim; ++d)
                X[i * dim + d] = m.coords[static_cast<size_t>(faceCoordConn[e * nfe + i]) * dim + d];
        std::fill(fe.begin(), fe.end(), 0.);
        for (int ip = 0; ip < q.n; ++ip)
        {
            double N[4], dN[8];
            FaceShape(nfe, q.points[ip].data(), N, dN);
            const double fac = FaceDetJ(dim, nfe, X, dN) * q.weights[ip];
            NeumannIp(nfe, dim, N, p, ipv.data());
            for (size_t i = 0; i < fe.size(); ++i)
                fe[i] += ipv[i] * fac;
        }
        for (int i = 0; i < nfe * dim; ++i)
            f[faceDofs[static_cast<size_t>(e) * nfe * dim + i]] += fe[i];
    }
}

//! Cell::Eval of one quantity at every integration point of every cell: out is nEl x nIp x width
inline void EvalIp(const Problem& P, const double* u, int quantity, double* out)
{
    const int w = P.IpWidth(quantity);
#pragma omp parallel for
    for (int e = 0; e < P.mesh->nEl; ++e)
        P.EvalCell(e, u, quantity, out + static_cast<size_t>(e) * P.q.n * w);
}

// ------------------------------------------------------------------------------------------------
// Assembly: SimpleAssembler::BuildVector (SimpleAssembler.cpp:38-65) and ::BuildMatrix (:100-156) with
// Eigen::SparseMatrix::setFromTriplets semantics, combined by ToEigen (DofMatrixSparseConvertEigen.h:40-67)
// ------------------------------------------------------------------------------------------------
inline void BuildVector(const Problem& P, const double* u, double* f)
{
    const int64_t n = P.nDofs;
    for (int64_t i = 0; i < n; ++i)
        f[i] = 0;
#pragma omp parallel
    {
        std::vector<double> local(n, 0.);
        CellResult res;
        std::vector<int64_t> dofs;
#pragma omp for nowait
        for (int e = 0; e < P.mesh->nEl; ++e)
        {
            P.IntegrateCell(e, u, true, false, res);
            P.CellDofs(e, dofs);
            for (int i = 0; i < P.nLocal; ++i)
                local[dofs[i]] += res.f[i];
        }
#pragma omp critical
        for (int64_t i = 0; i < n; ++i)
            f[i] += local[i];
    }
}

struct Triplet
{
    int row, col;
    double value;
};

struct CscMatrix
{
    int64_t rows = 0, cols = 0;
    std::vector<int64_t> colPtr;
    std::vector<int32_t> rowIdx;
    std::vector<double> values;
};

//! Eigen::SparseMatrix<double, ColMajor>::setFromTriplets: duplicates summed in triplet order, explicit
//! zeros kept, row indices sorted inside every column.
template <typename TIt>
inline CscMatrix SetFromTriplets(int64_t rows, int64_t cols, TIt begin, TIt end)
{
    // pass 1: row-major (transposed) storage, entries within a row in triplet order
    std::vector<int64_t> rowCount(rows + 1, 0);
    int64_t nt = 0;
    for (TIt it = begin; it != end; ++it, ++nt)
        rowCount[it->row + 1]++;
    for (int64_t r = 0; r < rows; ++r)
        rowCount[r + 1] += rowCount[r];
    std::vector<int64_t> fill(rowCount.begin(), rowCount.end() - 1);
    std::vector<int32_t> tcol(nt);
    std::vector<double> tval(nt);
    for (TIt it = begin; it != end; ++it)
    {
        const int64_t pos = fill[it->row]++;
        tcol[pos] = it->col;
        tval[pos] = it->value;
    }
    // collapseDuplicates: first occurrence keeps its slot, later ones are added to it
    std::vector<int64_t> wi(cols, -1);
    std::vector<int64_t> crow(rows + 1, 0);
    std::vector<int32_t> ccol;
    std::vector<double> cval;
    ccol.reserve(nt);
    cval.reserve(nt);
    for (int64_t r = 0; r < rows; ++r)
    {
        const int64_t rowStart = static_cast<int64_t>(ccol.size());
        for (int64_t k = rowCount[r]; k < rowCount[r + 1]; ++k)
        {
            const int32_t c = tcol[k];
            if (wi[c] >= rowStart)
                cval[wi[c]] += tval[k];
            else
            {
                wi[c] = static_cast<int64_t>(ccol.size());
                ccol.push_back(c);
                cval.push_back(tval[k]);
            }
        }
        crow[r + 1] = static_cast<int64_t>(ccol.size());
    }
    // transpose into column-major storage (row indices come out sorted)
    CscMatrix m;
    m.rows = rows;
    m.cols = cols;
    m.colPtr.assign(cols + 1, 0);
    for (int32_t c : ccol)
        m.colPtr[c + 1]++;
    for (int64_t c = 0; c < cols; ++c)
        m.colPtr[c + 1] += m.colPtr[c];
    std::vector<int64_t> pos(m.colPtr.begin(), m.colPtr.end() - 1);
    m.rowIdx.resize(ccol.size());
    m.values.resize(ccol.size());
    for (int64_t r = 0; r < rows; ++r)
        for (int64_t k = crow[r]; k < crow[r + 1]; ++k)
        {
            const int64_t p = pos[ccol[k]]++;
            m.rowIdx[p] = static_cast<int32_t>(r);
            m.values[p] = cval[k];
        }
    return m;
}

//! BuildMatrix with std::list triplets per (dofI, dofJ) block and thread (SimpleAssembler.cpp:105-147), one
//! setFromTriplets per block (:149-154), then ToEigen's combine of the blocks in `dofs` order.
inline CscMatrix BuildMatrix(const Problem& P, const double* u)
{
    const int ns = static_cast<int>(P.slots.size());
    using TripletList = std::list<Triplet>;
    std::vector<TripletList> triplets(ns * ns);
    std::vector<int64_t> blockSize(ns);
    for (int s = 0; s < ns; ++s)
    {
        const DofLayer& L = P.mesh->layers[P.slots[s]];
        blockSize[s] = static_cast<int64_t>(L.nNodes) * L.ncomp;
    }
#pragma omp parallel
    {
        std::vector<TripletList> local(ns * ns);
        CellResult res;
#pragma omp for nowait
        for (int e = 0; e < P.mesh->nEl; ++e)
        {
            P.IntegrateCell(e, u, false, true, res);
            for (int sI = 0; sI < ns; ++sI)
            {
                const DofLayer& LI = P.mesh->layers[P.slots[sI]];
                for (int sJ = 0; sJ < ns; ++sJ)
                {
                    const DofLayer& LJ = P.mesh->layers[P.slots[sJ]];
                    const int nI = LI.nEn * LI.ncomp, nJ = LJ.nEn * LJ.ncomp;
                    for (int i = 0; i < nI; ++i)
                    {
                        const int gi = LI.dofNumber[static_cast<size_t>(LI.conn[static_cast<size_t>(e) * LI.nEn + i / LI.ncomp]) * LI.ncomp + i % LI.ncomp];
                        for (int j = 0; j < nJ; ++j)
                        {
                            const int gj = LJ.dofNumber[static_cast<size_t>(LJ.conn[static_cast<size_t>(e) * LJ.nEn + j / LJ.ncomp]) * LJ.ncomp + j % LJ.ncomp];
                            const double v = res.K[static_cast<size_t>(P.localOffset[sI] + i) * P.nLocal + P.localOffset[sJ] + j];
                            local[sI * ns + sJ].push_back({gi, gj, v});
                        }
                    }
                }
            }
        }
#pragma omp critical
        for (int b = 0; b < ns * ns; ++b)
            triplets[b].splice(triplets[b].end(), local[b]);
    }
    std::vector<CscMatrix> blocks(ns * ns);
    for (int sI = 0; sI < ns; ++sI)
        for (int sJ = 0; sJ < ns; ++sJ)
            blocks[sI * ns + sJ] = SetFromTriplets(blockSize[sI], blockSize[sJ], triplets[sI * ns + sJ].begin(),
                                                   triplets[sI * ns + sJ].end());
    if (ns == 1)
        return blocks[0];
    std::vector<Triplet> all;
    int64_t startRow = 0;
    for (int sI = 0; sI < ns; ++sI)
    {
        int64_t startCol = 0;
        for (int sJ = 0; sJ < ns; ++sJ)
        {
            const CscMatrix& B = blocks[sI * ns + sJ];
            for (int64_t c = 0; c < B.cols; ++c)
                for (int64_t k = B.colPtr[c]; k < B.colPtr[c + 1]; ++k)
                    all.push_back({static_cast<int>(B.rowIdx[k] + startRow), static_cast<int>(c + startCol), B.values[k]});
            startCol += blockSize[sJ];
        }
        startRow += blockSize[sI];
    }
    return SetFromTriplets(P.nDofs, P.nDofs, all.begin(), all.end());
}

} // namespace nuto_oracle
