// Internal declarations of the GB300 element-assembly library (not part of the C ABI).
#pragma once

#include <cuda_runtime.h>

#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <functional>
#include <string>
#include <vector>

#include "../../include/nuto_gpu.h"

namespace nuto_gpu
{

constexpr int kMaxSlots = 2;
constexpr int kMaxIp = 27;
constexpr int kMaxEn = 20;

// Status with message, thrown only inside the library and turned into a return code at the C boundary.
struct Error
{
    int code;
    std::string msg;
};

#define NG_CUDA(call)                                                                                            \
    do                                                                                                           \
    {                                                                                                            \
        cudaError_t e_ = (call);                                                                                 \
        if (e_ != cudaSuccess)                                                                                   \
            throw ::nuto_gpu::Error{e_ == cudaErrorMemoryAllocation ? NUTO_GPU_ENOMEM : NUTO_GPU_ECUDA,          \
                                    std::string(#call) + ": " + cudaGetErrorString(e_)};                          \
    } while (0)

#define NG_CHECK(cond, code, msg)                                                                                \
    do                                                                                                           \
    {                                                                                                            \
        if (!(cond))                                                                                             \
            throw ::nuto_gpu::Error{code, msg};                                                                  \
    } while (0)

// ---- checked builds ------------------------------------------------------------------------------------------
// Compiled with -DNUTO_GPU_CHECKED, every kernel index into a caller or library buffer goes through NG_IDX: an
// index outside [0, n) is recorded in a device flag (first violation wins) and replaced by 0, so the access
// stays inside the buffer. The host reads the flag after every launch (AfterLaunch) and reports the site.
struct CheckFlag
{
    int site;
    long long index;
    long long limit;
};
#ifdef NUTO_GPU_CHECKED
static __device__ CheckFlag g_check; // one per translation unit (no relocatable device code)
__device__ __forceinline__ long long CheckedIndex(long long i, long long n, int site)
{
    if (i >= 0 && i < n)
        return i;
    if (atomicCAS(&g_check.site, 0, site) == 0)
    {
        g_check.index = i;
        g_check.limit = n;
    }
    return 0;
}
#define NG_IDX(i, n, site) ::nuto_gpu::CheckedIndex(static_cast<long long>(i), static_cast<long long>(n), site)
#else
#define NG_IDX(i, n, site) (i)
#endif

// ---- programmatic dependent launch -----------------------------------------------------------------------------
// The kernels of the Krylov iteration and the multigrid cycle are launched with programmatic stream serialisation:
// a kernel's blocks may be scheduled while its predecessor in the stream drains, which hides most of the gap
// between the many short launches of a cycle. Every such kernel calls PdlWait() before its first global memory
// access (it returns once the predecessor grid has completed and its writes are visible; without the launch
// attribute it returns at once) and PdlTrigger() right after, so that its own successor may be scheduled once all
// of its blocks are running. NUTO_GPU_PDL=0 launches them normally.
__device__ __forceinline__ void PdlWait()
{
    asm volatile("griddepcontrol.wait;\n" ::: "memory");
}
__device__ __forceinline__ void PdlTrigger()
{
    asm volatile("griddepcontrol.launch_dependents;\n" ::: "memory");
}
bool PdlEnabled();
template <typename... KArgs, typename... Args>
inline cudaError_t LaunchPdl(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t stream,
                             Args... args)
{
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = PdlEnabled() ? 1 : 0;
    return cudaLaunchKernelEx(&cfg, kernel, static_cast<KArgs>(args)...);
}

struct Ctx;
bool SyncCheck(const Ctx& c);
cudaStream_t StreamOf(const Ctx& c);

// Checks the launch; with NUTO_GPU_SYNC_CHECK=1 in the environment (or a checked build) also synchronises the
// stream and reports faults and index violations with the kernel name.
static inline void AfterLaunch(Ctx& c, const char* kernel)
{
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess)
        throw Error{NUTO_GPU_ECUDA, std::string("launch of ") + kernel + ": " + cudaGetErrorString(e)};
    if (!SyncCheck(c))
        return;
    const cudaError_t s = cudaStreamSynchronize(StreamOf(c));
    if (s != cudaSuccess)
        throw Error{NUTO_GPU_ECUDA, std::string("after ") + kernel + ": " + cudaGetErrorString(s)};
#ifdef NUTO_GPU_CHECKED
    CheckFlag f{};
    NG_CUDA(cudaMemcpyFromSymbol(&f, g_check, sizeof(f)));
    if (f.site != 0)
    {
        const CheckFlag zero{};
        NG_CUDA(cudaMemcpyToSymbol(g_check, &zero, sizeof(zero)));
        throw Error{NUTO_GPU_ECUDA, std::string("index check failed in ") + kernel + " at site " +
                                        std::to_string(f.site) + ": index " + std::to_string(f.index) +
                                        " outside [0, " + std::to_string(f.limit) + ")"};
    }
#endif
}

inline int NumNodes(int interp)
{
    return interp == NUTO_GPU_QUAD4 ? 4 : (interp == NUTO_GPU_HEX8 ? 8 : (interp == NUTO_GPU_HEX20 ? 20 : -1));
}
inline int InterpDim(int interp)
{
    return interp == NUTO_GPU_QUAD4 ? 2 : 3;
}

// Device buffer owned by the context. Move-only: a copy would share the pointer and free it twice.
template <typename T>
struct DBuf
{
    T* p = nullptr;
    size_t n = 0;
    DBuf() = default;
    DBuf(const DBuf&) = delete;
    DBuf& operator=(const DBuf&) = delete;
    DBuf(DBuf&& o) noexcept
        : p(o.p)
        , n(o.n)
    {
        o.p = nullptr;
        o.n = 0;
    }
    DBuf& operator=(DBuf&& o) noexcept
    {
        if (this != &o)
        {
            free();
            p = o.p;
            n = o.n;
            o.p = nullptr;
            o.n = 0;
        }
        return *this;
    }
    void alloc(size_t count)
    {
        free();
        if (count == 0)
            return;
        NG_CUDA(cudaMalloc(&p, count * sizeof(T)));
        n = count;
    }
    void free()
    {
        if (p)
            cudaFree(p);
        p = nullptr;
        n = 0;
    }
    ~DBuf()
    {
        free();
    }
};

struct Slot
{
    int ncomp = 1;
    int interp = NUTO_GPU_HEX8;
    int nen = 8;
    int64_t nNodes = 0;
    int64_t nDofs = 0; // n_independent + n_dependent
    int64_t nIndep = 0;
    int64_t offset = 0; // first row of this slot in the combined system
    std::vector<int32_t> conn; // nCells x nen (host copy)
    std::vector<int32_t> dof0; // per node: dof number of component 0
    DBuf<int32_t> dConnT; // planar [n][cell]
    DBuf<int64_t> dGdof; // per node: combined index of component 0
    // node -> cells adjacency (cells in ascending order) with the node's local index in each cell
    DBuf<int64_t> dCellPtr;
    DBuf<int32_t> dCellIdx;
    DBuf<uint8_t> dCellLoc;
};

// Per (slot I, slot J) scatter map: rank of the J-node among the sorted J-neighbours of the I-node, per cell and
// local node pair, plus the start of the J block inside the rows of an I-node.
struct PairMap
{
    DBuf<uint8_t> dRank; // planar [i * nenJ + j][cell]
    uint8_t* rank = nullptr; // dRank.p or a shared table of an identical pair
    DBuf<int32_t> dBlk; // per I-node
    // J-neighbours of every I-node in CSR column order (the node-block SpMV reconstructs column indices from them)
    DBuf<int64_t> dNbrPtr; // nNodes_I + 1
    DBuf<int32_t> dNbrIdx;
    DBuf<int32_t> dNbrCol; // combined row of component 0 of each neighbour entry
    std::vector<int64_t> hNbrPtr; // host copies (multigrid hierarchy set-up)
    std::vector<int32_t> hNbrIdx;
};

// Device-side constants of one integrand (plain data passed by value to kernels).
struct LawParams
{
    int kind, dim;
    int planeState, damageApp, interaction;
    double E, nu;
    // LinearElastic C (Voigt)
    double C11, C12, C33;
    // LinearElasticDamage
    double m3K, m2G, d2; // d2: mD2 factor of the normal components (1 or 1 + nu/(nu-1))
    // damage law, strain norm, nonlocal interaction
    double kappa0, beta, alpha;
    double K1, K2, k;
    double c, R, eta;
};

// Integration-point tables (double): weights, shape values and natural derivatives per interpolation.
struct IpTables
{
    int nIp = 0;
    std::vector<double> w; // nIp
    std::vector<double> N[3]; // per interpolation: nIp x nen
    std::vector<double> dN[3]; // per interpolation: nIp x nen x 3
};

struct SolverWork;
struct Amg;

// Boundary cells of one DOF slot (NeumannBc loads): Line2 faces of a 2D mesh or Quad4 faces of a 3D mesh, on the
// context's coordinate nodes and the slot's DOF nodes.
struct BoundaryGroup
{
    int slot = 0;
    int nfe = 0; // nodes per face
    int64_t nFaces = 0;
    DBuf<int32_t> coordConnT; // planar [i][face]
    DBuf<int32_t> dofConnT;   // planar [i][face]
    int nq = 0;               // Gauss points per direction
    double gp[3] = {0, 0, 0}, gw[3] = {0, 0, 0};
};

// Solver copy of the tangent in the padded pair layout: for every slot pair (I, J) and I-node a, the node's ncomp_I
// row segments of the J-columns (ncomp_J values per J-neighbour, CSR column order) follow each other, each padded
// with zeros to a multiple of 4 values; every node block starts at a multiple of 4 values. The SpMV streams these
// blocks with 16-byte loads. Filled from the CSR values once per tangent (same pointer and version: reused).
struct NbLayout
{
    struct Pair
    {
        DBuf<int64_t> base; // per I-node: first value of the node's block, relative to off
        int64_t off = 0;    // first value of the pair
        int maxSeg4 = 0;    // longest padded segment
    };
    Pair pair[kMaxSlots * kMaxSlots];
    int64_t total = 0;
    int maxSeg4 = 0;
    DBuf<float> v32;
    DBuf<double> v64;
    const void* src32 = nullptr;
    const void* src64 = nullptr;
    uint64_t ver32 = 0, ver64 = 0;
};

// host wall time of the phases of a step (diagnostics, printed with NUTO_GPU_VERBOSE)
enum HostPhase
{
    HP_TANGENT,
    HP_RESIDUAL,
    HP_SOLVE,
    HP_AMG_SETUP,
    HP_GRAPH,
    HP_SYNC,
    HP_COUNT
};
struct HostClock
{
    double* acc;
    std::chrono::steady_clock::time_point t0;
    explicit HostClock(double* a)
        : acc(a), t0(std::chrono::steady_clock::now())
    {
    }
    ~HostClock()
    {
        *acc += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    }
};

// Launch shapes chosen by the autotuner (first use per context, timed with CUDA events; 0 = not tuned yet)
struct Tuning
{
    bool enabled = true;             // NUTO_GPU_AUTOTUNE=0 keeps the defaults
    int tangentWarps = 0;            // warps per block of the FP32 tangent's node-row kernel (2, 4, 8)
    int tangentForm = 0;             // 0 node rows, 1 double-buffered node rows on resident blocks, 2 element
                                     // matrices + row gather
    float tangentMs[7] = {0, 0, 0, 0, 0, 0, 0}; // one assembly with 2, 4, 8 warps per block; double-buffered with 2,
                                                // 4; element matrices with 2, 4
    int spmvGroup[4] = {0, 0, 0, 0}; // lanes per node of the fine-level product, per (value, vector) type pair
    float spmvMs[4][3] = {};         // one product with 4, 8, 16 lanes per node
};

struct Ctx
{
    int device = 0;
    cudaStream_t stream = nullptr;
    bool ownStream = false;
    std::string err;
    int smCount = 0;

    // cells
    bool haveCells = false;
    int dim = 3, geoInterp = NUTO_GPU_HEX8, nge = 8;
    int64_t nCells = 0, nCoord = 0;
    int gauss = 2;
    IpTables ip;
    DBuf<double> dCoords;
    DBuf<int32_t> dGeoConnT; // planar [n][cell]
    std::vector<double> hCoords;
    std::vector<int32_t> hGeoConn;
    DBuf<double> dTables; // w | N(interp) | dN(interp) packed, see TableOffsets
    int tabW = 0, tabN[3] = {0, 0, 0}, tabDN[3] = {0, 0, 0};

    // DOF types
    std::vector<Slot> slots;
    int64_t nDofs = 0;

    // Dirichlet constraints (combined indices)
    std::vector<std::vector<int32_t>> depDofs; // per slot
    std::vector<std::vector<double>> depA, depB; // per slot
    DBuf<uint8_t> dMask; // combined n_dofs: 1 = dependent
    DBuf<int64_t> dDepIdx;
    DBuf<double> dDepA, dDepB;
    int64_t nDep = 0;

    // pattern
    bool havePattern = false;
    int64_t nnz = 0;
    DBuf<int64_t> dRowPtr;
    DBuf<int32_t> dColIdx;
    std::vector<int64_t> hRowPtr;
    PairMap pairs[kMaxSlots * kMaxSlots];
    double avgRowLen = 0;

    // geometry caches per integration point: planar [(q * S + k)][cell], S = 1 + nen_d * dim
    bool haveGeo = false;
    DBuf<double> dGeo64;
    DBuf<float> dGeo32;
    int geoStride = 0;

    // row-gather tangent: integration-point records and the displacement-node -> eeq-node map
    int rowsMode = -1; // -1 not decided, 0 element-wise atomics, 1 row gather
    bool forceAtomicTangent = false; // NUTO_GPU_TANGENT=atomic selects the element-wise kernel
    bool forceRecordTangent = false; // NUTO_GPU_TANGENT=records selects records + row gather for linear cells
    int gmresRestart = 0;            // NUTO_GPU_GMRES_RESTART; 0 = the default length
    DBuf<int32_t> dEOf;
    DBuf<unsigned char> dRecords;
    // fused FP32 tangent: -1 not decided, 0 not applicable, 1 used; FP32 node coordinates relative to each cell's
    // first node (planar [(n * dim + d)][cell])
    Tuning tuning;
    int fusedMode = -1;
    bool tangentStaged = true; // per-point records computed once (NUTO_GPU_TANGENT=fused: recomputed per node warp)
    DBuf<float> dRelX;
    // Hex20 FP32 tangent on the tensor cores: -1 not decided, 0 not applicable, 1 used; split 3 = three TF32
    // products per contraction (hi.hi + hi.lo + lo.hi, FP32-level accuracy), 1 = one (NUTO_GPU_TC20=tf32);
    // per-point records and per-cell element matrices ([cell][a][i][b][j], FP32)
    int tc20Mode = -1;
    int tc20Split = 3;
    bool forceTc20Off = false; // NUTO_GPU_TC20=off
    int tc20LawFp64 = 0;       // NUTO_GPU_TC20=fp64law: the law of every point in FP64
    DBuf<float> dElemMats;
    bool cellsLawFused = true; // element-matrix form: the law in the cell kernel (NUTO_GPU_CELLS_RECORDS=1: records)
    DBuf<uint32_t> dPackedRanks; // element-matrix form: ranks of (cell entry of a node, b), packed, cell-list order
    // device status word of kernels with bounded waits (0 = fine, else NUTO_GPU_ETIMEOUT), read after a stream
    // synchronisation; spinLimit bounds every wait loop (iterations)
    DBuf<int> dStatus;
    long long spinLimit = 1LL << 22;
    // residual: the cell vectors of the last residual (planar [local entry][cell]) gathered per DOF
    DBuf<double> dCellVec;
    // nuto_gpu_build_system: the residual on a second stream beside the tangent, as a persistent grid of
    // sysResBlocks blocks per SM (the FP64 pipe needs few warps), the rest of every SM left to the tangent's
    // blocks; the first call of a context runs both in sequence (lazy set-up, autotuning)
    cudaStream_t sideStream = nullptr;
    cudaEvent_t evFork = nullptr, evJoin = nullptr;
    int sysResBlocks = 6;
    // nuto_gpu_build_system_host: device copies of the caller's host state, values and vector
    DBuf<double> dHostIoU, dHostIoF;
    DBuf<unsigned char> dHostIoVals;
    // the element-matrix form's row gather in node chunks, with a hook after each chunk (nuto_gpu_build_system_host
    // copies each chunk's values to the host while the next chunks run); 0 or 1: one launch
    int rowChunks = 0;
    std::function<void(int64_t, int64_t)> onRowChunk;
    int rowChunksDone = 0;
    cudaStream_t copyStream = nullptr;
    cudaEvent_t evCopy = nullptr;
    std::vector<cudaEvent_t> evChunks;
    std::vector<int32_t> hEOf; // displacement node -> eeq node (gradient damage, row-gather set-ups)
    int rowsContig = -1;       // -1 not checked; 1: consecutive nodes have consecutive rows (and eeq rows)
    bool noAllocReady = false; // nuto_gpu_build_matrix_noalloc: address looked up and kernels loaded
    int64_t systemCalls = 0;
    // adjoint: positions of the transposed entries, per-point partial derivatives
    DBuf<int64_t> dTransPerm;
    DBuf<double> dAdjPart;

    // integrand
    bool haveIntegrand = false;
    nuto_gpu_integrand prm{};
    LawParams law{};
    DBuf<double> dKappa; // nCells x nIp
    DBuf<double> dEScale; // per-cell factor of the integrand's Young's modulus (empty: 1 everywhere)

    // quasistatic state
    bool haveState = false;
    double time = 0;
    DBuf<double> dX;
    nuto_gpu_stats stats{};

    SolverWork* work = nullptr;
    Amg* amg = nullptr;
    std::vector<BoundaryGroup> boundary;
    NbLayout nb;
    DBuf<double> dConstGrad; // added to the residual of nuto_gpu_do_step (empty: none)
    int precond = NUTO_GPU_PRECOND_AMG;
    uint64_t valsVersion = 1; // bumped by every tangent assembly and every caller-supplied solve
    bool syncCheck = false; // NUTO_GPU_SYNC_CHECK=1 or a checked build
    double hostMs[HP_COUNT] = {};

    ~Ctx();
};

// ---- host helpers implemented in the .cu files ----
void BuildTables(Ctx& c);
void BuildGeometryCache(Ctx& c);
void LaunchResidual(Ctx& c, const double* u, double* f, int blocksPerSm = 0); // 0: one block per CPB cells
void LaunchTangent(Ctx& c, const double* u, int precision, void* values);
void LaunchTangentExact(Ctx& c, const double* u, double* vals);
void LaunchTangentNoAlloc(Ctx& c, const double* u, float* values);
bool FusedTangentSupported(Ctx& c);
void LaunchTangentFused(Ctx& c, const double* u, float* vals);
bool Tc20TangentSupported(Ctx& c);
void LaunchTangentTc20(Ctx& c, const double* u, float* vals);
int ReadDeviceStatus(Ctx& c); // after a stream synchronisation: the status word (and reset to 0)
void LaunchHistory(Ctx& c, const double* u);
void LaunchLumpedMass(Ctx& c, double rho, double* m);
void LaunchExternalLoad(Ctx& c, const BoundaryGroup& B, const double* p, double* f);
void LaunchEvalIp(Ctx& c, const double* u, int quantity, double* out);
int IpWidth(const Ctx& c, int quantity);
void LaunchCellVectors(Ctx& c, const double* fe, double* f);
void LaunchCellMatrices(Ctx& c, const double* ke, int precision, void* values);
int SolveLinear(Ctx& c, int precision, int method, const void* values, const double* b, double* x, double rtol,
                int maxit, int* iters, double* relres);
int DoStep(Ctx& c, double tNew, const nuto_gpu_step_options& o, int* iters);
void FreeSolverWork(Ctx& c);
void FreeAmg(Ctx& c);
template <typename TV>
void AmgSetup(Ctx& c, const TV* vals);
template <typename T>
void AmgApply(Ctx& c, const T* v, T* z, const int* st, bool sym);
int AmgLevels(const Ctx& c);
// y = K x for FP32 or FP64 CSR values and FP64 vectors (FP64 accumulation), and the compensated FP32 form
void SpmvFull64(Ctx& c, int precision, const void* vals, const double* x, double* y);
void SpmvFull64Comp(Ctx& c, const float* vals, const double* x, double* y);
const char* AmgGraphStatus(const Ctx& c);
// true when the last sweep ran as a CUDA graph
bool AmgGraphActive(const Ctx& c);
// fills the padded pair layout of TV from the CSR values `vals` unless it holds them already (same pointer and
// tangent version)
template <typename TV>
void EnsureNb(Ctx& c, const TV* vals);

// ---- kernel argument blocks (by value) ----
struct CellArgs
{
    int64_t nCells;
    int64_t nNodesD, nNodesE, nDofs, geoSize; // buffer extents for checked builds
    const int32_t* connD; // planar [n][cell]
    const int32_t* connE;
    const int64_t* gdofD; // per node: combined index of component 0
    const int64_t* gdofE;
    const double* tabN_D; // nIp x nenD
    const double* tabN_E;
    const double* geo64;
    const float* geo32;
    int geoStride;
    double* kappa;
    const double* escale; // per-cell Young's modulus factor (nullptr: 1)
};

struct ScatterArgs
{
    int64_t nnz, nRows; // buffer extents for checked builds
    const int64_t* rowPtr;
    const uint8_t* rank[kMaxSlots * kMaxSlots];
    const int32_t* blk[kMaxSlots * kMaxSlots];
};

CellArgs CellArgsOf(Ctx& c); // the geometry cache is built on first use
void GatherCellVectors(Ctx& c, const Slot& S, int ncomp, int off, int64_t nLocal, double* f, bool add);
void LaunchTransposeValues(Ctx& c, int precision, const void* in, void* out);
void LaunchAdjointHistoryLoad(Ctx& c, const double* u, const double* kbar, double* ubar);
void LaunchAdjointStep(Ctx& c, const double* u, const double* lam, const double* kbarIn, double* kbarOut,
                       double* gradE, double* gradParams);

// Engineering strain from the displacement gradient H[c][d] = sum_n u_nc dN_n/dx_d, Voigt order of
// Nabla::Strain (DifferentialOperators.h:24-90): 2D xx, yy, xy; 3D xx, yy, zz, yz, zx, xy.
template <typename T, int DIM>
__device__ __forceinline__ void StrainFromH(const T (&H)[DIM][DIM], T* e)
{
    if (DIM == 2)
    {
        e[0] = H[0][0];
        e[1] = H[1][1];
        e[2] = H[0][1] + H[1][0];
    }
    else
    {
        e[0] = H[0][0];
        e[1] = H[1][1];
        e[2] = H[2][2];
        e[3] = H[1][2] + H[2][1];
        e[4] = H[0][2] + H[2][0];
        e[5] = H[0][1] + H[1][0];
    }
}

// B_n^T s for the node with global gradient g (columns of the Voigt strain operator)
template <typename T, int DIM>
__device__ __forceinline__ void BtS(const T* g, const T* s, T* out)
{
    if (DIM == 2)
    {
        out[0] = g[0] * s[0] + g[1] * s[2];
        out[1] = g[1] * s[1] + g[0] * s[2];
    }
    else
    {
        out[0] = g[0] * s[0] + g[2] * s[4] + g[1] * s[5];
        out[1] = g[1] * s[1] + g[2] * s[3] + g[0] * s[5];
        out[2] = g[2] * s[2] + g[1] * s[3] + g[0] * s[4];
    }
}

// ------------------------------------------------------------------------------------------------------------
// Constitutive laws, device side, templated on the arithmetic type. Each cites the reference it restates.
// ------------------------------------------------------------------------------------------------------------
template <typename T>
__host__ __device__ inline T H_unilateral(const LawParams& p, T eV)
{
    return (p.damageApp == NUTO_GPU_DAMAGE_UNILATERAL && eV < T(0)) ? T(0) : T(1);
}

// Volumetric strain of LinearElasticDamage: 1/3 * mD2^T eps (LinearElasticDamage.h:58-66)
template <typename T, int DIM>
__host__ __device__ inline T VolStrain(const LawParams& p, const T* e)
{
    if (DIM == 2)
        return T(1. / 3.) * (T(p.d2) * e[0] + T(p.d2) * e[1]);
    return T(1. / 3.) * (e[0] + e[1] + e[2]);
}

// LinearElasticDamage::Stress (LinearElasticDamage.h:58-66)
template <typename T, int DIM>
__host__ __device__ inline void LedStress(const LawParams& p, const T* e, T omega, T* s)
{
    constexpr int VD = DIM == 2 ? 3 : 6;
    const T eV = VolStrain<T, DIM>(p, e);
    const T sV = (T(1) - omega * H_unilateral(p, eV)) * T(p.m3K) * eV;
    const T g = (T(1) - omega) * T(p.m2G);
#pragma unroll
    for (int i = 0; i < VD; ++i)
    {
        const bool normal = i < DIM;
        const T dev = normal ? e[i] - eV : e[i];
        s[i] = (normal ? sV : T(0)) + g * (normal ? dev : T(0.5) * dev);
    }
}

// LinearElasticDamage::DstressDomega (LinearElasticDamage.h:79-87)
template <typename T, int DIM>
__host__ __device__ inline void LedDstressDomega(const LawParams& p, const T* e, T* s)
{
    constexpr int VD = DIM == 2 ? 3 : 6;
    const T eV = VolStrain<T, DIM>(p, e);
    const T dsV = -T(p.m3K) * eV * H_unilateral(p, eV);
#pragma unroll
    for (int i = 0; i < VD; ++i)
    {
        const bool normal = i < DIM;
        const T dev = normal ? e[i] - eV : e[i];
        s[i] = (normal ? dsV : T(0)) - T(p.m2G) * (normal ? dev : T(0.5) * dev);
    }
}

// Isotropic split of LinearElasticDamage::DstressDstrain (LinearElasticDamage.h:68-77):
// a * Iv + b * PinvId = lambda * m m^T + mu * diag(2,..,2,1,..,1) with m the normal-component indicator.
// Iv = 1/3 mD mD2^T and Pinv m = m give lambda = d2 (a - b) / 3, mu = b / 2.
template <typename T, int DIM>
__host__ __device__ inline void LedTangentLameParams(const LawParams& p, const T* e, T omega, T& lam, T& mu)
{
    const T eV = VolStrain<T, DIM>(p, e);
    const T a = T(p.m3K) * (T(1) - omega * H_unilateral(p, eV));
    const T b = (T(1) - omega) * T(p.m2G);
    lam = T(DIM == 2 ? p.d2 : 1.0) * (a - b) / T(3);
    mu = b / T(2);
}

// ModifiedMisesStrainNorm::Value / Derivative (ModifiedMisesStrainNorm.h:139-268), plane strain/stress for 2D
template <typename T, int DIM>
__host__ __device__ inline T MisesValue(const LawParams& p, const T* e)
{
    T v0 = e[0], v1 = e[1], v2, v3, v4, v5;
    if (DIM == 2)
    {
        v2 = p.planeState == NUTO_GPU_PLANE_STRESS ? T(p.nu / (p.nu - 1.)) * (e[0] + e[1]) : T(0);
        v3 = T(0);
        v4 = T(0);
        v5 = e[2];
    }
    else
    {
        v2 = e[2];
        v3 = e[3];
        v4 = e[4];
        v5 = e[5];
    }
    const T I1 = v0 + v1 + v2;
    const T yz = T(.5) * v3, zx = T(.5) * v4, xy = T(.5) * v5;
    const T J2 = T(1. / 6.) * ((v0 - v1) * (v0 - v1) + (v1 - v2) * (v1 - v2) + (v2 - v0) * (v2 - v0)) + xy * xy +
                 yz * yz + zx * zx;
    const T K1 = T(p.K1), K2 = T(p.K2);
    const T A = sqrt(K1 * K1 * I1 * I1 + K2 * J2);
    return K1 * I1 + A;
}

template <typename T, int DIM>
__host__ __device__ inline void MisesDerivative(const LawParams& p, const T* s, T* d)
{
    const T K1 = T(p.K1), K2 = T(p.K2);
    if (DIM == 3)
    {
        const T I1 = s[0] + s[1] + s[2];
        const T yz = T(.5) * s[3], zx = T(.5) * s[4], xy = T(.5) * s[5];
        const T J2 = T(1. / 6.) * ((s[0] - s[1]) * (s[0] - s[1]) + (s[1] - s[2]) * (s[1] - s[2]) +
                                   (s[2] - s[0]) * (s[2] - s[0])) +
                     xy * xy + yz * yz + zx * zx;
        const T A = sqrt(K1 * K1 * I1 * I1 + K2 * J2);
        if (A == T(0))
        {
            d[0] = d[1] = d[2] = K1;
            d[3] = d[4] = d[5] = T(0);
            return;
        }
        const T inv2A = T(1) / (T(2) * A);
        const T dxx = T(1. / 3.) * (T(2) * s[0] - s[1] - s[2]);
        const T dyy = T(1. / 3.) * (T(2) * s[1] - s[0] - s[2]);
        const T dzz = T(1. / 3.) * (T(2) * s[2] - s[0] - s[1]);
        d[0] = K1 + inv2A * (T(2) * K1 * K1 * I1 + K2 * dxx);
        d[1] = K1 + inv2A * (T(2) * K1 * K1 * I1 + K2 * dyy);
        d[2] = K1 + inv2A * (T(2) * K1 * K1 * I1 + K2 * dzz);
        d[3] = inv2A * K2 * T(0.5) * s[3];
        d[4] = inv2A * K2 * T(0.5) * s[4];
        d[5] = inv2A * K2 * T(0.5) * s[5];
        return;
    }
    const T nu = T(p.nu);
    if (p.planeState == NUTO_GPU_PLANE_STRAIN)
    {
        const T I1 = s[0] + s[1];
        const T xy = T(.5) * s[2];
        const T J2 = T(1. / 6.) * ((s[0] - s[1]) * (s[0] - s[1]) + s[1] * s[1] + s[0] * s[0]) + xy * xy;
        const T A = sqrt(K1 * K1 * I1 * I1 + K2 * J2);
        if (A == T(0))
        {
            d[0] = K1;
            d[1] = K1;
            d[2] = T(0);
            return;
        }
        const T inv2A = T(1) / (T(2) * A);
        d[0] = K1 + inv2A * (T(2) * K1 * K1 * I1 + K2 * T(1. / 3.) * (T(2) * s[0] - s[1]));
        d[1] = K1 + inv2A * (T(2) * K1 * K1 * I1 + K2 * T(1. / 3.) * (T(2) * s[1] - s[0]));
        d[2] = inv2A * (K2 * T(0.5) * s[2]);
        return;
    }
    const T f = nu / (nu - T(1));
    const T sz = f * (s[0] + s[1]);
    const T I1 = s[0] + s[1] + sz;
    const T xy = T(.5) * s[2];
    const T J2 = T(1. / 6.) * ((s[0] - s[1]) * (s[0] - s[1]) + (s[1] - sz) * (s[1] - sz) + (sz - s[0]) * (sz - s[0])) +
                 xy * xy;
    const T A = sqrt(K1 * K1 * I1 * I1 + K2 * J2);
    const T dI1 = T(1) + f;
    if (A == T(0))
    {
        d[0] = dI1 * K1;
        d[1] = dI1 * K1;
        d[2] = T(0);
        return;
    }
    const T inv2A = T(1) / (T(2) * A);
    const T dxx = T(1. / 3.) * (T(2) * s[0] - s[1] - T(2) * sz + T(2) * f * sz);
    const T dyy = T(1. / 3.) * (T(2) * s[1] - s[0] - T(2) * sz + T(2) * f * sz);
    d[0] = dI1 * K1 + inv2A * (T(2) * dI1 * K1 * K1 * I1 + K2 * dxx);
    d[1] = dI1 * K1 + inv2A * (T(2) * dI1 * K1 * K1 * I1 + K2 * dyy);
    d[2] = inv2A * (K2 * T(0.5) * s[2]);
}

// DamageLawExponential (DamageLawExponential.h:40-52)
template <typename T>
__host__ __device__ inline T DamageOmega(const LawParams& p, T kappa)
{
    const T k0 = T(p.kappa0);
    if (kappa < k0)
        return T(0);
    return T(1) - k0 / kappa * (T(1) - T(p.alpha) + T(p.alpha) * exp(T(p.beta) * (k0 - kappa)));
}
template <typename T>
__host__ __device__ inline T DamageDerivative(const LawParams& p, T kappa)
{
    const T k0 = T(p.kappa0);
    if (kappa < k0)
        return T(0);
    return k0 / kappa *
           ((T(1) / kappa + T(p.beta)) * T(p.alpha) * exp(T(p.beta) * (k0 - kappa)) + (T(1) - T(p.alpha)) / kappa);
}

// NonlocalInteraction::Constant / Decreasing (GradientDamage.h:153-184)
template <typename T>
__host__ __device__ inline T InteractionFactor(const LawParams& p, T omega)
{
    if (p.interaction == NUTO_GPU_INTERACTION_CONSTANT)
        return T(1);
    const T eta = T(p.eta), R = T(p.R);
    return ((T(1) - R) * exp(-eta * omega) + R - exp(-eta)) / (T(1) - exp(-eta));
}
template <typename T>
__host__ __device__ inline T InteractionDerivative(const LawParams& p, T omega)
{
    if (p.interaction == NUTO_GPU_INTERACTION_CONSTANT)
        return T(0);
    const T eta = T(p.eta), R = T(p.R);
    return ((T(1) - R) * exp(-eta * omega)) / (T(1) - exp(-eta)) * -eta;
}

} // namespace nuto_gpu
