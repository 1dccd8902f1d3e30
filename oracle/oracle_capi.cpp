// TEST INFRASTRUCTURE ONLY — C entry points of the oracle (the CPU restatement in nuto_oracle.hpp).
// Loaded by the tests and by the benchmark's CPU-baseline leg through ctypes; never by the product.
#include "nuto_oracle.hpp"

#include <cstring>
#include <memory>

using namespace nuto_oracle;

namespace
{
struct ProblemBox
{
    Problem P;
    CscMatrix K;
};
} // namespace

extern "C" {

void* oracle_mesh_quads(int nx, int ny)
{
    return new Mesh(CreateQuads(nx, ny));
}

void* oracle_mesh_bricks(int nx, int ny, int nz)
{
    return new Mesh(CreateBricks(nx, ny, nz));
}

void* oracle_mesh_from_arrays(int dim, int geoInterp, int nNodes, const double* coords, int nEl, const int* conn)
{
    auto* m = new Mesh();
    m->dim = dim;
    m->geoInterp = geoInterp;
    m->nGeoEn = NumNodes(geoInterp);
    m->coords.assign(coords, coords + static_cast<size_t>(nNodes) * dim);
    m->conn.assign(conn, conn + static_cast<size_t>(nEl) * m->nGeoEn);
    m->nEl = nEl;
    return m;
}

//! UnitMeshFem::Transform (UnitMeshFem.cpp:117-125) with the affine map x -> diag(s) x
void oracle_mesh_scale(void* mesh, double sx, double sy, double sz)
{
    auto* m = static_cast<Mesh*>(mesh);
    const double s[3] = {sx, sy, sz};
    for (size_t i = 0; i < m->coords.size(); ++i)
        m->coords[i] *= s[i % m->dim];
}

void oracle_mesh_free(void* mesh)
{
    delete static_cast<Mesh*>(mesh);
}

int oracle_mesh_num_elements(void* mesh)
{
    return static_cast<Mesh*>(mesh)->nEl;
}

int oracle_mesh_num_coord_nodes(void* mesh)
{
    auto* m = static_cast<Mesh*>(mesh);
    return static_cast<int>(m->coords.size() / m->dim);
}

void oracle_mesh_coords(void* mesh, double* out)
{
    auto* m = static_cast<Mesh*>(mesh);
    std::memcpy(out, m->coords.data(), m->coords.size() * sizeof(double));
}

void oracle_mesh_conn(void* mesh, int* out)
{
    auto* m = static_cast<Mesh*>(mesh);
    std::memcpy(out, m->conn.data(), m->conn.size() * sizeof(int));
}

int oracle_mesh_add_dof(void* mesh, int ncomp, int interp)
{
    try
    {
        return AddDofInterpolation(*static_cast<Mesh*>(mesh), ncomp, interp);
    }
    catch (...)
    {
        return -1;
    }
}

int oracle_layer_num_nodes(void* mesh, int layer)
{
    return static_cast<Mesh*>(mesh)->layers[layer].nNodes;
}

int oracle_layer_nen(void* mesh, int layer)
{
    return static_cast<Mesh*>(mesh)->layers[layer].nEn;
}

void oracle_layer_conn(void* mesh, int layer, int* out)
{
    const auto& L = static_cast<Mesh*>(mesh)->layers[layer];
    std::memcpy(out, L.conn.data(), L.conn.size() * sizeof(int));
}

void oracle_layer_node_coords(void* mesh, int layer, double* out)
{
    const auto& L = static_cast<Mesh*>(mesh)->layers[layer];
    std::memcpy(out, L.nodeXYZ.data(), L.nodeXYZ.size() * sizeof(double));
}

void oracle_layer_dof_numbers(void* mesh, int layer, int* out)
{
    const auto& L = static_cast<Mesh*>(mesh)->layers[layer];
    std::memcpy(out, L.dofNumber.data(), L.dofNumber.size() * sizeof(int));
}

int oracle_nodes_at_axis(void* mesh, int layer, int dir, double offset, int* out)
{
    auto nodes = NodesAtAxis(*static_cast<Mesh*>(mesh), layer, dir, offset);
    if (out)
        std::memcpy(out, nodes.data(), nodes.size() * sizeof(int));
    return static_cast<int>(nodes.size());
}

void* oracle_problem_create(void* mesh, int ipsPerDir, int nSlots, const int* slots, const IntegrandParams* p)
{
    auto* box = new ProblemBox();
    box->P.mesh = static_cast<Mesh*>(mesh);
    box->P.q = TensorGauss(box->P.mesh->dim, ipsPerDir);
    box->P.slots.assign(slots, slots + nSlots);
    box->P.p = *p;
    box->P.Init();
    return box;
}

void oracle_problem_free(void* prob)
{
    delete static_cast<ProblemBox*>(prob);
}

long long oracle_problem_num_dofs(void* prob)
{
    return static_cast<ProblemBox*>(prob)->P.nDofs;
}

int oracle_problem_num_ips(void* prob)
{
    return static_cast<ProblemBox*>(prob)->P.q.n;
}

void oracle_problem_set_kappa(void* prob, const double* kappa)
{
    auto& P = static_cast<ProblemBox*>(prob)->P;
    std::memcpy(P.kappa.data(), kappa, P.kappa.size() * sizeof(double));
}

void oracle_problem_get_kappa(void* prob, double* kappa)
{
    auto& P = static_cast<ProblemBox*>(prob)->P;
    std::memcpy(kappa, P.kappa.data(), P.kappa.size() * sizeof(double));
}

void oracle_build_vector(void* prob, const double* u, double* f)
{
    BuildVector(static_cast<ProblemBox*>(prob)->P, u, f);
}

long long oracle_build_matrix(void* prob, const double* u)
{
    auto* box = static_cast<ProblemBox*>(prob);
    box->K = BuildMatrix(box->P, u);
    return static_cast<long long>(box->K.values.size());
}

void oracle_matrix_copy(void* prob, long long* colPtr, int* rowIdx, double* values)
{
    auto* box = static_cast<ProblemBox*>(prob);
    for (size_t i = 0; i < box->K.colPtr.size(); ++i)
        colPtr[i] = box->K.colPtr[i];
    std::memcpy(rowIdx, box->K.rowIdx.data(), box->K.rowIdx.size() * sizeof(int));
    std::memcpy(values, box->K.values.data(), box->K.values.size() * sizeof(double));
}

void oracle_matrix_release(void* prob)
{
    static_cast<ProblemBox*>(prob)->K = CscMatrix();
}

void oracle_update_history(void* prob, const double* u)
{
    static_cast<ProblemBox*>(prob)->P.UpdateHistory(u);
}

void oracle_lumped_mass(void* prob, double rho, double* m)
{
    BuildLumpedMass(static_cast<ProblemBox*>(prob)->P, rho, m);
}

void oracle_lump_hrz(const double* M, int nl, int ncomp, double* out)
{
    LumpHRZ(M, nl, ncomp, out);
}

int oracle_ip_width(void* prob, int quantity)
{
    return static_cast<ProblemBox*>(prob)->P.IpWidth(quantity);
}

void oracle_eval_ip(void* prob, const double* u, int quantity, double* out)
{
    EvalIp(static_cast<ProblemBox*>(prob)->P, u, quantity, out);
}

void oracle_external_load(void* mesh, int nfe, int nFaces, const int* faceCoordConn, const long long* faceDofs,
                          const double* p, int gauss, double* f)
{
    std::vector<int64_t> dofs(faceDofs, faceDofs + static_cast<size_t>(nFaces) * nfe * static_cast<Mesh*>(mesh)->dim);
    BuildExternalLoad(*static_cast<Mesh*>(mesh), nfe, nFaces, faceCoordConn, dofs.data(), p, gauss, f);
}

void oracle_neumann_ip(int nfe, int dim, const double* xi, const double* p, double* out)
{
    double N[4], dN[8];
    FaceShape(nfe, xi, N, dN);
    NeumannIp(nfe, dim, N, p, out);
}

int oracle_cell_nlocal(void* prob)
{
    return static_cast<ProblemBox*>(prob)->P.nLocal;
}

void oracle_cell_dofs(void* prob, int cell, long long* out)
{
    std::vector<int64_t> dofs;
    static_cast<ProblemBox*>(prob)->P.CellDofs(cell, dofs);
    for (size_t i = 0; i < dofs.size(); ++i)
        out[i] = dofs[i];
}

void oracle_cell_integrate(void* prob, int cell, const double* u, double* fe, double* Ke)
{
    CellResult res;
    static_cast<ProblemBox*>(prob)->P.IntegrateCell(cell, u, fe != nullptr, Ke != nullptr, res);
    if (fe)
        std::memcpy(fe, res.f.data(), res.f.size() * sizeof(double));
    if (Ke)
        std::memcpy(Ke, res.K.data(), res.K.size() * sizeof(double));
}

//! per-cell Young's modulus as multiples of the integrand's E (null: 1 everywhere)
void oracle_problem_set_e_scale(void* prob, const double* scale)
{
    auto& P = static_cast<ProblemBox*>(prob)->P;
    if (scale)
        P.eScale.assign(scale, scale + P.mesh->nEl);
    else
        P.eScale.clear();
}

//! adjoint ingredients of one gradient-damage cell (Problem::AdjointCell); returns -1 for other integrands
int oracle_cell_adjoint(void* prob, int cell, const double* u, double* D, double* ipd, double* N)
{
    const auto& P = static_cast<ProblemBox*>(prob)->P;
    if (P.p.kind != GRADIENT_DAMAGE)
        return -1;
    P.AdjointCell(cell, u, D, ipd, N);
    return 0;
}

//! Cell::Integrate(ScalarFunction) with f == 1: the cell volume (test/mechanics/cell/Cell.cpp:100)
double oracle_cell_volume(void* prob, int cell)
{
    const auto& P = static_cast<ProblemBox*>(prob)->P;
    double X[60];
    P.mesh->ElementCoords(cell, X);
    double v = 0;
    for (int ip = 0; ip < P.q.n; ++ip)
    {
        double N[20], dN[60];
        Shape(P.mesh->geoInterp, P.q.points[ip].data(), N, dN);
        v += ComputeJacobian(P.mesh->dim, P.mesh->nGeoEn, X, dN).det * P.q.weights[ip];
    }
    return v;
}

void oracle_quadrature(int dim, int n, double* pts, double* w)
{
    Quadrature q = TensorGauss(dim, n);
    for (int i = 0; i < q.n; ++i)
    {
        for (int d = 0; d < dim; ++d)
            pts[i * dim + d] = q.points[i][d];
        w[i] = q.weights[i];
    }
}

void oracle_shape(int interp, const double* xi, double* N, double* dN)
{
    Shape(interp, xi, N, dN);
}

void oracle_set_threads(int n)
{
#ifdef _OPENMP
    omp_set_num_threads(n);
#else
    (void)n;
#endif
}

int oracle_max_threads()
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

// ---- constitutive-law entry points for the known-answer / finite-difference tests -----------------------
void oracle_linear_elastic_C(int dim, double E, double nu, int planeState, double* out)
{
    Mat C = LinearElasticC(dim, E, nu, planeState);
    std::memcpy(out, C.v.data(), C.v.size() * sizeof(double));
}

void oracle_led(int dim, double E, double nu, int app, int planeState, const double* strain, double omega,
                double* stress, double* dsde, double* dsdw)
{
    LinearElasticDamage led(dim, E, nu, app, planeState);
    if (stress)
        led.Stress(strain, omega, stress);
    if (dsde)
        led.DstressDstrain(strain, omega, dsde);
    if (dsdw)
        led.DstressDomega(strain, omega, dsdw);
}

double oracle_mises(int dim, double nu, double k, int planeState, const double* strain, double* deriv)
{
    ModifiedMises m(dim, nu, k, planeState);
    if (deriv)
        m.Derivative(strain, deriv);
    return m.Value(strain);
}

void oracle_damage_exp(double kappa0, double beta, double alpha, double kappa, double* omega, double* domega)
{
    DamageExponential d{kappa0, beta, alpha};
    *omega = d.Damage(kappa);
    *domega = d.Derivative(kappa);
}

//! LocalIsotropicDamage<dim>::Stress/Tangent with one history value (LocalIsotropicDamage.h:52-68)
void oracle_local_damage(int dim, double E, double nu, int app, int planeState, double kappa0, double beta,
                         double alpha, double k, double kappaHist, const double* strain, double* stress,
                         double* tangent)
{
    LinearElasticDamage led(dim, E, nu, app, planeState);
    ModifiedMises norm(dim, nu, k, planeState);
    DamageExponential dmg{kappa0, beta, alpha};
    const int vd = VoigtDim(dim);
    const double eqs = norm.Value(strain);
    const double kap = std::max(eqs, kappaHist);
    const double omega = dmg.Damage(kap);
    led.Stress(strain, omega, stress);
    double dsde[36], dsdw[6], dK[6] = {0, 0, 0, 0, 0, 0};
    led.DstressDstrain(strain, omega, dsde);
    led.DstressDomega(strain, omega, dsdw);
    if (eqs >= kappaHist)
        norm.Derivative(strain, dK);
    const double dOdK = dmg.Derivative(kap);
    for (int r = 0; r < vd; ++r)
        for (int c = 0; c < vd; ++c)
            tangent[r * vd + c] = dsde[r * vd + c] + dsdw[r] * dOdK * dK[c];
}

} // extern "C"
