// rift_engine.cu -- host engine and C ABI (include/rift_gb300.h) of the GB300
// RIFT step.  The handle owns every device buffer and one CUDA stream; the
// per-step launch sequence is captured once into a CUDA graph and replayed.
//
// Device layout (FP32, pitched, ghost ring included, cell (j,i) at column i
// of row j):
//   A, B   [3][rows][pitch]  depth h, hu, hv  (U^n / U*; double-buffered so
//                            no CTA reads a cell another CTA is writing)
//   E      [4][rows][pitch]  eW, eE, eS, eN: face elevation minus the cell's
//                            reference elevation, differenced in FP64
//   nman, K, FA, FB, hmax, qmax, twet, tpeak, tdry, maps  [rows][pitch]
// Host keeps the FP64 reference elevation of every cell to rebuild
// w = Bref + h at output.
#include <cuda.h>
#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "../../include/rift_gb300.h"
#include "rift_grow.cuh"
#include "rift_kernels.cuh"
#include "rift_march.cuh"
#include "rift_update1.cuh"
#include "rift_persist.cuh"
#include "rift_ensemble.cuh"

using namespace rift;

namespace {

typedef CUresult (*PFN_encodeTiled)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*,
                                    const cuuint64_t*, const cuuint64_t*, const cuuint32_t*,
                                    const cuuint32_t*, CUtensorMapInterleave, CUtensorMapSwizzle,
                                    CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

PFN_encodeTiled getEncodeTiled() {
    static PFN_encodeTiled fn = nullptr;
    if (!fn) {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000,
                                             cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = (PFN_encodeTiled)p;
    }
    return fn;
}

}  // namespace

struct rift_handle {
    rift_grid_desc g{};
    int nx = 0, ny = 0, nBX = 0, nBY = 0, gridSize = 0, pitch = 0, rows = 0;
    int numSMs = 0, gridStage = 0, gridSpeed = 0, gridTrack = 0, gridDt = 0, gridMarch = 0;
    int gridUpdate = 0;  // k_update1: resident CTAs over half-strip items
    int gridMarch1 = 0;  // k_march<1>: its own occupancy (fewer registers than k_march<2>)
    int nSX = 0, nSY = 0;
    int marchMin = 0;  // active strips from which the march kernels run
    int gridGrow = 0;      // CTAs of the grow kernel of the graph path
    int gridPersist = 0;   // CTAs of the cooperative step kernel (0: unavailable)
    int persistMax = 0;    // it runs while the active tiles are at most this many
    GridBar* gbar = nullptr;
    int* owner = nullptr;  // [gridSize] tile table of the persistent loop
    int* tileFlag = nullptr;  // [gridSize] stage-1 completion of the persistent loop
    long long persistSteps = 0, graphSteps = 0;  // steps run by each path (diagnostics)
    long long launches = 0;  // kernels launched by the run paths (graph replays count their kernels)
    int graphKernels = 0;    // kernel nodes of the per-step graph
    int* strips = nullptr;
    uint8_t* stripFlag = nullptr;
    int marchRows = STRIP_TY;  // tile rows per march work item (1, 2 or 4)
    CUtensorMap tmAm{}, tmBm{}, tmEm{};  // 120 x 4-row boxes of the march kernels
    U1Maps tmU1{};                           // 116 x 7-row boxes of k_update1
    float* tmU1Rain[2] = {nullptr, nullptr};  // rain maps the boxes were encoded for
    cudaStream_t stream = nullptr;
    float *A = nullptr, *B = nullptr, *E = nullptr, *nman = nullptr, *K = nullptr;
    float* D = nullptr;  // [3] planes: the march's stage-1 divergence
    float *FA = nullptr, *FB = nullptr, *hmax = nullptr, *qmax = nullptr, *twet = nullptr;
    float *tpeak = nullptr, *tdry = nullptr;
    float* maps[3][2] = {{nullptr, nullptr}, {nullptr, nullptr}, {nullptr, nullptr}};
    int mapMode[3] = {0, 0, 0};
    uint8_t *wet = nullptr, *prevAct = nullptr;
    int *act = nullptr, *deact = nullptr, *inact = nullptr;
    float *mx = nullptr, *my = nullptr;
    int* srcIdx = nullptr;
    float* srcRate = nullptr;
    int *srcTileStart = nullptr, *srcTileList = nullptr;
    int nsrc = 0;
    float *serT = nullptr, *serR = nullptr;
    int serN[3] = {0, 0, 0};
    DevState* st = nullptr;
    DevState* hst = nullptr;  // pinned mirror
    // start of the volume ledger (rift_init, rift_set_state): interior sums
    // of h and F, and the source total at that moment
    double ledVol0 = 0.0, ledSoil0 = 0.0, ledAdded0 = 0.0;
    float* stage = nullptr;   // pinned host planes for field uploads / readbacks
    size_t stageFloats = 0;
    double* volPartial = nullptr;
    CUtensorMap tmA{}, tmB{}, tmE{};
    std::vector<double> Bref, BC, h0_;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t graphExec = nullptr;
    // one persistent step with its state copies, for rift_step: one graph
    // per grid size seen (the grid follows the active count)
    static constexpr int STEP_CACHE = 4;
    cudaGraphExec_t stepExec[STEP_CACHE] = {};
    int stepGrid[STEP_CACHE] = {};
    int stepNext = 0;
    bool stepGraphBroken = false;
    bool haveStatic = false, inited = false;
    // the device reads and writes pageable host memory through the host's
    // page tables (Grace: NVLink-C2C, address translation services): state
    // import and field export can run as kernels on the caller's arrays
    // (off by default: slower than the staged copies, measured)
    bool hostAccessOk = false;  // the device supports it
    bool hostAccess = false;    // and this handle uses it (rift_set_host_access)
    double* BrefD = nullptr;  // [ny][nx] FP64 reference elevations (host-access path)
    std::string err;

    bool has(uint32_t f) const { return (g.flags & f) != 0; }
    size_t plane() const { return (size_t)rows * pitch; }
};

// ---------------------------------------------------------------- host access
// State import straight from the caller's FP64 host arrays, read in place
// through the host's page tables: the same conversions as the host path
// (h = float(w - Bref) in FP64, then FP32), without a staging copy.
__global__ void k_import(const double* __restrict__ w, const double* __restrict__ hu,
                         const double* __restrict__ hv, const double* __restrict__ F,
                         const double* __restrict__ Bref, float* __restrict__ A, float* __restrict__ FA,
                         float* __restrict__ FB, size_t pl, int pitch, int nx, int ny) {
    const size_t n = (size_t)nx * ny;
    for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < n;
         c += (size_t)gridDim.x * blockDim.x) {
        const int j = (int)(c / (size_t)nx), i = (int)(c % (size_t)nx);
        const size_t d = (size_t)j * pitch + i;
        A[d] = __double2float_rn(__dsub_rn(w[c], Bref[c]));
        A[pl + d] = __double2float_rn(hu[c]);
        A[2 * pl + d] = __double2float_rn(hv[c]);
        if (F) {
            const float f = __double2float_rn(F[c]);
            FA[d] = f;
            FB[d] = f;
        }
    }
}

// Ghost cells from host-computed border triples (h, hu, hv): rows 2..ny-3
// (west pair, east pair), then columns 2..nx-3 (south pair, north pair).
__global__ void k_ghostsFromBorder(const float* __restrict__ gb, float* __restrict__ A, size_t pl,
                                   int pitch, int nx, int ny) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    const int nr = ny - 4, nc = nx - 4;
    auto put = [&](int j, int i, const float* v) {
        const size_t d = (size_t)j * pitch + i;
        A[d] = v[0];
        A[pl + d] = v[1];
        A[2 * pl + d] = v[2];
    };
    if (k < nr) {
        const int j = k + 2;
        const float* v = gb + 6 * (size_t)k;
        put(j, 0, v);
        put(j, 1, v);
        put(j, nx - 2, v + 3);
        put(j, nx - 1, v + 3);
    } else if (k < nr + nc) {
        const int i = k - nr + 2;
        const float* v = gb + 6 * (size_t)nr + 6 * (size_t)(k - nr);
        put(0, i, v);
        put(1, i, v);
        put(ny - 2, i, v + 3);
        put(ny - 1, i, v + 3);
    }
}

// Field export straight into the caller's FP64 host array (row stride ld):
// mode 0 the value, 1 w = Bref + h, 2 the clamped interior depth map.
__global__ void k_export(const float* __restrict__ src, const double* __restrict__ Bref,
                         double* __restrict__ out, size_t ld, int pitch, int nx, int ny, int mode) {
    const size_t n = (size_t)nx * ny;
    for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < n;
         c += (size_t)gridDim.x * blockDim.x) {
        const int j = (int)(c / (size_t)nx), i = (int)(c % (size_t)nx);
        const float v = src[(size_t)j * pitch + i];
        double r;
        if (mode == 1) {
            r = __dadd_rn(Bref[c], (double)v);
        } else if (mode == 2) {
            const bool in = i >= 2 && j >= 2 && i <= nx - 3 && j <= ny - 3;
            r = in ? (double)((v > kEps) ? v : 0.f) : 0.0;
        } else {
            r = (double)v;
        }
        out[(size_t)j * ld + i] = r;
    }
}

namespace {

int fail(rift_handle* h, int code, const std::string& msg) {
    if (h) h->err = msg;
    return code;
}

#define CUDA_TRY(h, call)                                                                   \
    do {                                                                                    \
        cudaError_t e_ = (call);                                                            \
        if (e_ != cudaSuccess)                                                              \
            return fail(h, e_ == cudaErrorMemoryAllocation ? RIFT_ERR_NOMEM : RIFT_ERR_CUDA, \
                        std::string(#call) + ": " + cudaGetErrorString(e_));                \
    } while (0)

Params makeParams(rift_handle* h) {
    Params P{};
    P.nx = h->nx;
    P.ny = h->ny;
    P.nBX = h->nBX;
    P.nBY = h->nBY;
    P.gridSize = h->gridSize;
    P.pitch = h->pitch;
    P.rows = h->rows;
    P.dx = (float)h->g.dx;
    P.dy = (float)h->g.dy;
    P.inv_dx = (float)(1.0 / h->g.dx);
    P.inv_dy = (float)(1.0 / h->g.dy);
    P.kappa = (float)h->g.kappa;
    P.psiDtheta = (float)(h->g.psi * h->g.dtheta);
    P.nodata = (float)h->g.nodata;
    P.dxd = h->g.dx;
    P.dyd = h->g.dy;
    P.kappad = h->g.kappa;
    P.kappaf = (float)h->g.kappa;
    P.squareCells = h->g.dx == h->g.dy;
    P.courant = h->g.courant;
    {
        int e = 0;
        const double m = std::frexp(h->g.courant, &e);
        P.courantScale = (m == 0.5 && h->g.courant > 0.0) ? (float)(1.0 / h->g.courant) : 0.f;
    }
    P.flags = h->g.flags;
    P.A = h->A;
    P.B = h->B;
    P.D = h->D;
    P.planeSize = (int)h->plane();
    P.E = h->E;
    P.nman = h->nman;
    P.K = h->K;
    P.FA = h->FA;
    P.FB = h->FB;
    P.hmax = h->hmax;
    P.qmax = h->qmax;
    P.twet = h->twet;
    P.tpeak = h->tpeak;
    P.tdry = h->tdry;
    for (int k = 0; k < 3; k++) {
        P.map0[k] = h->maps[k][0];
        P.map1[k] = h->maps[k][1];
        P.mapMode[k] = h->mapMode[k];
    }
    P.wet = h->wet;
    P.prevAct = h->prevAct;
    P.act = h->act;
    P.deact = h->deact;
    P.inact = h->inact;
    P.strips = h->strips;
    P.stripFlag = h->stripFlag;
    P.nSX = h->nSX;
    P.nSY = h->nSY;
    P.marchMin = h->marchMin;
    P.persistMax = h->persistMax;
    P.gbar = h->gbar;
    P.owner = h->owner;
    P.tileFlag = h->tileFlag;
    P.mx = h->mx;
    P.my = h->my;
    P.srcIdx = h->srcIdx;
    P.srcRate = h->srcRate;
    P.srcTileStart = h->srcTileStart;
    P.srcTileList = h->srcTileList;
    P.nsrc = h->nsrc;
    P.serT = h->serT;
    P.serR = h->serR;
    for (int k = 0; k < 3; k++) P.serN[k] = h->serN[k];
    P.st = h->st;
    return P;
}

int encodeMap(rift_handle* h, CUtensorMap* tm, float* base, int nfields, int boxW = SW,
              int boxH = SH) {
    PFN_encodeTiled enc = getEncodeTiled();
    if (!enc) return fail(h, RIFT_ERR_CUDA, "cuTensorMapEncodeTiled unavailable");
    cuuint64_t dims[3] = {(cuuint64_t)h->pitch, (cuuint64_t)h->rows, (cuuint64_t)nfields};
    cuuint64_t strides[2] = {(cuuint64_t)h->pitch * 4, (cuuint64_t)h->plane() * 4};
    cuuint32_t box[3] = {(cuuint32_t)boxW, (cuuint32_t)boxH, (cuuint32_t)nfields};
    cuuint32_t estr[3] = {1, 1, 1};
    CUresult r = enc(tm, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, base, dims, strides, box, estr,
                     CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                     CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return fail(h, RIFT_ERR_CUDA, "cuTensorMapEncodeTiled failed");
    return RIFT_OK;
}

void destroyGraph(rift_handle* h) {
    if (h->graphExec) cudaGraphExecDestroy(h->graphExec);
    if (h->graph) cudaGraphDestroy(h->graph);
    for (int k = 0; k < rift_handle::STEP_CACHE; k++) {
        if (h->stepExec[k]) cudaGraphExecDestroy(h->stepExec[k]);
        h->stepExec[k] = nullptr;
        h->stepGrid[k] = 0;
    }
    h->graphExec = nullptr;
    h->graph = nullptr;
}

// The launch sequence of one step (captured into the graph).
// The fixed flag set of the march instantiation for this run (0: the
// generic one reading the run's flags).
uint32_t marchFix(const rift_handle* h) {
    const uint32_t f = h->g.flags & CELL_FLAGS;
    if (((f & F_POINT) != 0) != (h->nsrc > 0)) return 0u;
    if (f == FIX_RAIN || f == FIX_INFIL_SRC || f == FIX_RAINMAP_DRAIN) return f;
    return 0u;
}

template <int STAGE, int STY>
void launchMarchRows(const rift_handle* h, const CUtensorMap& tmIn, const Params& P, cudaStream_t s,
                     int grid) {
    switch (marchFix(h)) {
        case FIX_RAIN: k_march<STAGE, FIX_RAIN, STY><<<grid, MT, 0, s>>>(tmIn, h->tmEm, P); break;
        case FIX_INFIL_SRC:
            k_march<STAGE, FIX_INFIL_SRC, STY><<<grid, MT, 0, s>>>(tmIn, h->tmEm, P);
            break;
        case FIX_RAINMAP_DRAIN:
            k_march<STAGE, FIX_RAINMAP_DRAIN, STY><<<grid, MT, 0, s>>>(tmIn, h->tmEm, P);
            break;
        default: k_march<STAGE, 0, STY><<<grid, MT, 0, s>>>(tmIn, h->tmEm, P);
    }
}

// The march pass of STAGE with the handle's work-item height.
template <int STAGE>
void launchMarch(const rift_handle* h, const CUtensorMap& tmIn, const Params& P, cudaStream_t s,
                 int grid) {
    switch (h->marchRows) {
        case 1: launchMarchRows<STAGE, 1>(h, tmIn, P, s, grid); break;
        case 4: launchMarchRows<STAGE, 4>(h, tmIn, P, s, grid); break;
        default: launchMarchRows<STAGE, 2>(h, tmIn, P, s, grid);
    }
}

// The persistent loop's instantiation for this run (two fixed flag sets).
const void* persistKernel(const rift_handle* h) {
    switch (marchFix(h)) {
        case FIX_RAIN: return (const void*)k_persist<FIX_RAIN>;
        case FIX_INFIL_SRC: return (const void*)k_persist<FIX_INFIL_SRC>;
        default: return (const void*)k_persist<>;
    }
}

template <uint32_t FIX>
constexpr uint32_t u1Smem() {
    return u1SmemBytes<(FIX & F_RAIN_G) != 0>();
}
template <uint32_t FIX>
void launchUpdate1Fix(const rift_handle* h, const Params& P, cudaStream_t s) {
    k_update1<FIX><<<h->gridUpdate, MT, u1Smem<FIX>(), s>>>(h->tmU1, P);
}

void launchUpdate1(const rift_handle* h, const Params& P, cudaStream_t s) {
    switch (marchFix(h)) {
        case FIX_RAIN: launchUpdate1Fix<FIX_RAIN>(h, P, s); break;
        case FIX_INFIL_SRC: launchUpdate1Fix<FIX_INFIL_SRC>(h, P, s); break;
        case FIX_RAINMAP_DRAIN: launchUpdate1Fix<FIX_RAINMAP_DRAIN>(h, P, s); break;
        default: launchUpdate1Fix<0>(h, P, s);
    }
}

// Boxes of the rain maps for k_update1 (the maps appear with rift_set_map).
void refreshUpdateMaps(rift_handle* h) {
    for (int k = 0; k < 2; k++)
        if (h->maps[0][k] && h->maps[0][k] != h->tmU1Rain[k]) {
            encodeMap(h, k ? &h->tmU1.r1 : &h->tmU1.r0, h->maps[0][k], 1, UBOXW, URC);
            h->tmU1Rain[k] = h->maps[0][k];
        }
}

void enqueueStep(rift_handle* h) {
    refreshUpdateMaps(h);
    Params P = makeParams(h);
    cudaStream_t s = h->stream;
    if (h->has(RIFT_F_RAIN_GRID) || h->has(RIFT_F_SURGE_GRID))
        k_track<<<h->gridTrack, NT, 0, s>>>(P);
    k_grow<<<h->gridGrow, NT, 0, s>>>(P);
    // per-tile and march variants of each pass; the device keeps one of them
    // (useMarch) and the other returns at once
    k_speed_dt<<<h->gridSpeed, NT, 0, s>>>(h->tmA, h->tmE, P);
    launchMarch<1>(h, h->tmAm, P, s, h->gridMarch1);  // fluxes, speeds, dt
    k_stage<1><<<h->gridStage, NT, 0, s>>>(h->tmA, h->tmE, P);
    launchUpdate1(h, P, s);
    if (!h->has(RIFT_F_EULER)) {
        k_stage<2><<<h->gridStage, NT, 0, s>>>(h->tmB, h->tmE, P);
        launchMarch<2>(h, h->tmBm, P, s, h->gridMarch);
    } else {
        k_commit<<<h->gridStage, NT, 0, s>>>(P);
    }
}

int buildGraph(rift_handle* h) {
    if (h->graphExec) return RIFT_OK;
    CUDA_TRY(h, cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
    enqueueStep(h);
    cudaError_t e = cudaStreamEndCapture(h->stream, &h->graph);
    if (e != cudaSuccess) return fail(h, RIFT_ERR_CUDA, std::string("capture: ") + cudaGetErrorString(e));
    CUDA_TRY(h, cudaGraphInstantiate(&h->graphExec, h->graph, 0));
    size_t nodes = 0;  // every node of the step graph is a kernel launch
    CUDA_TRY(h, cudaGraphGetNodes(h->graph, nullptr, &nodes));
    h->graphKernels = (int)nodes;
    return RIFT_OK;
}

const char* deviceErrorText(int err) {
    if (err & ERR_TILE_TABLE) return "persistent loop: tile table and active set disagree";
    if (err & ERR_BARRIER_TIMEOUT) return "device wait timed out (grid barrier)";
    return "device wait timed out (TMA barrier)";
}

int volumeSum(rift_handle* h, int what, double* out);
int ledgerStart(rift_handle* h);

int pullState(rift_handle* h) {
    CUDA_TRY(h, cudaMemcpyAsync(h->hst, h->st, sizeof(DevState), cudaMemcpyDeviceToHost, h->stream));
    CUDA_TRY(h, cudaStreamSynchronize(h->stream));
    if (h->hst->error) return fail(h, RIFT_ERR_CUDA, deviceErrorText(h->hst->error));
    return RIFT_OK;
}

int pushState(rift_handle* h) {
    CUDA_TRY(h, cudaMemcpyAsync(h->st, h->hst, sizeof(DevState), cudaMemcpyHostToDevice, h->stream));
    CUDA_TRY(h, cudaStreamSynchronize(h->stream));
    return RIFT_OK;
}

// Stream-ordered push for the step path: the host leaves the pinned mirror
// alone until the pull that ends the call, so no wait is needed here.
int pushStateAsync(rift_handle* h) {
    CUDA_TRY(h, cudaMemcpyAsync(h->st, h->hst, sizeof(DevState), cudaMemcpyHostToDevice, h->stream));
    return RIFT_OK;
}

inline size_t hidx(const rift_handle* h, int j, int i) { return (size_t)j * h->nx + i; }

// Reference elevation per cell: the cell's own BC in the interior, the BC of
// the interior cell a ghost copies from (ApplyBoundaries writes
// w_ghost = BC_interior + H), and for the four corner blocks the value the
// reference leaves there (InitGrid_k sets w = BC for i,j >= 2, else 0).
void buildReference(rift_handle* h, const double* BX, const double* BY) {
    const int nx = h->nx, ny = h->ny;
    h->BC.assign((size_t)nx * ny, 0.0);
    h->Bref.assign((size_t)nx * ny, 0.0);
    auto bx = [&](int j, int i) { return BX[(size_t)j * (nx + 1) + i]; };
    auto by = [&](int j, int i) { return BY[(size_t)j * nx + i]; };
    for (int j = 2; j < ny; j++)
        for (int i = 2; i < nx; i++)  // InitGrid_k:532
            h->BC[hidx(h, j, i)] = 0.25 * (bx(j, i + 1) + bx(j, i) + by(j + 1, i) + by(j, i));
    for (int j = 0; j < ny; j++)
        for (int i = 0; i < nx; i++) {
            bool xin = i >= 2 && i <= nx - 3, yin = j >= 2 && j <= ny - 3;
            double r;
            if (xin && yin)
                r = h->BC[hidx(h, j, i)];
            else if (yin)
                r = h->BC[hidx(h, j, i < 2 ? 2 : nx - 3)];
            else if (xin)
                r = h->BC[hidx(h, j < 2 ? 2 : ny - 3, i)];
            else
                r = h->BC[hidx(h, j, i)];
            h->Bref[hidx(h, j, i)] = r;
        }
}

float depthFromW(const rift_handle* h, double w, int j, int i) {
    return (float)(w - h->Bref[hidx(h, j, i)]);
}

// Critical-depth ghosts on the host (init / state upload), same rule as the
// device writeGhosts.
void hostGhosts(rift_handle* h, float* H, float* U, float* V) {
    const int nx = h->nx, ny = h->ny;
    auto crit = [](float q, float d) { return std::fmin(std::cbrt(q * q / kG), d); };
    for (int j = 2; j <= ny - 3; j++) {
        for (int side = 0; side < 2; side++) {
            int ii = side ? nx - 3 : 2;
            size_t c = hidx(h, j, ii);
            float HL = crit(U[c], H[c]);
            HL = (HL > kEps) ? HL : 0.f;
            int g0 = side ? nx - 2 : 0, g1 = side ? nx - 1 : 1;
            for (int gi : {g0, g1}) {
                size_t q = hidx(h, j, gi);
                H[q] = HL;
                U[q] = U[c];
                V[q] = V[c];
            }
        }
    }
    for (int i = 2; i <= nx - 3; i++) {
        for (int side = 0; side < 2; side++) {
            int jj = side ? ny - 3 : 2;
            size_t c = hidx(h, jj, i);
            float HB = crit(V[c], H[c]);
            int g0 = side ? ny - 2 : 0, g1 = side ? ny - 1 : 1;
            for (int gj : {g0, g1}) {
                size_t q = hidx(h, gj, i);
                H[q] = HB;
                U[q] = U[c];
                V[q] = V[c];
            }
        }
    }
}

int upField(rift_handle* h, float* dev, const float* host) {
    CUDA_TRY(h, cudaMemcpy2DAsync(dev, (size_t)h->pitch * 4, host, (size_t)h->nx * 4,
                                  (size_t)h->nx * 4, h->ny, cudaMemcpyHostToDevice, h->stream));
    return RIFT_OK;
}

int upField(rift_handle* h, float* dev, const std::vector<float>& host) {
    return upField(h, dev, host.data());
}

// Device plane -> host (nx x ny), synchronous.
int downField(rift_handle* h, const float* dev, float* host) {
    CUDA_TRY(h, cudaMemcpy2DAsync(host, (size_t)h->nx * 4, dev, (size_t)h->pitch * 4,
                                  (size_t)h->nx * 4, h->ny, cudaMemcpyDeviceToHost, h->stream));
    CUDA_TRY(h, cudaStreamSynchronize(h->stream));
    return RIFT_OK;
}

// `planes` host planes of nx x ny floats in pinned memory (kept by the
// handle; the caller finishes its copies before the next use).
float* stagePlanes(rift_handle* h, int planes) {
    const size_t need = (size_t)planes * h->nx * h->ny;
    if (h->stageFloats < need) {
        if (h->stage) cudaFreeHost(h->stage);
        h->stage = nullptr;
        h->stageFloats = 0;
        if (cudaMallocHost(&h->stage, need * 4) != cudaSuccess) {
            cudaGetLastError();
            h->stage = nullptr;
            return nullptr;
        }
        h->stageFloats = need;
    }
    return h->stage;
}

// fn(j0, j1) over row bands of [0, ny) on up to 16 host threads (inline for
// small grids).
template <class F>
void parallelRows(int ny, size_t cells, F fn) {
    unsigned nt = std::thread::hardware_concurrency();
    nt = std::max(1u, std::min(16u, nt));
    if (cells < (size_t)1 << 18 || nt == 1) {
        fn(0, ny);
        return;
    }
    std::vector<std::thread> th;
    const int per = (ny + (int)nt - 1) / (int)nt;
    for (unsigned t = 0; t < nt; t++) {
        const int j0 = (int)t * per, j1 = std::min(ny, j0 + per);
        if (j0 < j1) th.emplace_back(fn, j0, j1);
    }
    for (auto& x : th) x.join();
}

bool tileInGrid(const rift_handle* h, int b) {
    int i0 = (b % h->nBX) * TW + 2, j0 = (b / h->nBX) * TH + 2;
    return i0 < h->nx && j0 < h->ny;
}

// FP64 reference elevations on the device, for the host-access path.
int uploadBref(rift_handle* h) {
    const size_t n = (size_t)h->nx * h->ny;
    if (!h->BrefD) CUDA_TRY(h, cudaMalloc(&h->BrefD, n * 8));
    CUDA_TRY(h, cudaMemcpyAsync(h->BrefD, h->Bref.data(), n * 8, cudaMemcpyHostToDevice, h->stream));
    CUDA_TRY(h, cudaStreamSynchronize(h->stream));
    return RIFT_OK;
}

// Upload U (A and B), tile flags and lists.
int uploadState(rift_handle* h, const float* H, const float* U, const float* V,
                const std::vector<uint8_t>& wet,
                const std::vector<uint8_t>& activeFlags, const std::vector<int>& inactList) {
    const size_t pl = h->plane();
    int r;
    if (H && ((r = upField(h, h->A, H)) || (r = upField(h, h->A + pl, U)) ||
              (r = upField(h, h->A + 2 * pl, V))))
        return r;  // (H null: U^n is already on the device)
    CUDA_TRY(h, cudaMemcpyAsync(h->B, h->A, 3 * pl * 4, cudaMemcpyDeviceToDevice, h->stream));
    CUDA_TRY(h, cudaMemcpyAsync(h->wet, wet.data(), h->gridSize, cudaMemcpyHostToDevice, h->stream));
    CUDA_TRY(h, cudaMemcpyAsync(h->prevAct, activeFlags.data(), h->gridSize,
                                cudaMemcpyHostToDevice, h->stream));
    if (!inactList.empty())
        CUDA_TRY(h, cudaMemcpyAsync(h->inact, inactList.data(), inactList.size() * 4,
                                    cudaMemcpyHostToDevice, h->stream));
    h->hst->nInact = (int)inactList.size();
    // the scheduled count of the uploaded active set: the persistent
    // launch sizes its grid by it until the next grow publishes its own
    int nAct = 0;
    for (int b = 0; b < h->gridSize; b++)
        if (activeFlags[b] && (b % h->nBX) * TW + 2 <= h->nx - 3 && (b / h->nBX) * TH + 2 <= h->ny - 3)
            nAct++;
    h->hst->nActive = nAct;
    return RIFT_OK;
}

}  // namespace

extern "C" {

int rift_create(const rift_grid_desc* g, rift_handle** out) {
    if (!g || !out) return RIFT_ERR_ARG;
    *out = nullptr;
    if (g->h_nx < 5 || g->h_ny < 5 || !(g->dx > 0) || !(g->dy > 0) || !(g->kappa > 0) ||
        !(g->courant > 0))
        return RIFT_ERR_ARG;
    rift_handle* h = new rift_handle();
    h->g = *g;
    h->nx = g->h_nx;
    h->ny = g->h_ny;
    h->nBX = (h->nx + TW - 1) / TW;
    h->nBY = (h->ny + TH - 1) / TH;
    h->gridSize = h->nBX * h->nBY;
    // every staged block (columns 16bX .. 16bX+19, rows 14bY .. 14bY+17) lies
    // inside the allocation
    h->pitch = ((h->nBX * TW + 8) + 31) / 32 * 32;
    h->rows = h->nBY * TH + 4;
    *out = h;
    // cell offsets are 32-bit on the device: the largest field (4 planes)
    // must stay below 2^32 elements
    if (4.0 * (double)h->rows * (double)h->pitch >= 4294967296.0)
        return fail(h, RIFT_ERR_TOO_LARGE, "grid above 2^32 cells per 4-plane field");
    cudaError_t e = cudaSetDevice(g->device);
    if (e != cudaSuccess) return fail(h, RIFT_ERR_CUDA, cudaGetErrorString(e));
    int dev = g->device;
    cudaDeviceGetAttribute(&h->numSMs, cudaDevAttrMultiProcessorCount, dev);
    {
        int pageable = 0, hostTables = 0;
        cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccess, dev);
        cudaDeviceGetAttribute(&hostTables, cudaDevAttrPageableMemoryAccessUsesHostPageTables, dev);
        h->hostAccessOk = pageable == 1 && hostTables == 1;
    }
    CUDA_TRY(h, cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking));
    const size_t pl = h->plane() * 4;
    CUDA_TRY(h, cudaMalloc(&h->A, 3 * pl));
    CUDA_TRY(h, cudaMalloc(&h->B, 3 * pl));
    CUDA_TRY(h, cudaMalloc(&h->D, 3 * pl));
    CUDA_TRY(h, cudaMalloc(&h->E, 4 * pl));
    CUDA_TRY(h, cudaMalloc(&h->nman, pl));
    CUDA_TRY(h, cudaMemset(h->A, 0, 3 * pl));
    CUDA_TRY(h, cudaMemset(h->B, 0, 3 * pl));
    CUDA_TRY(h, cudaMemset(h->E, 0, 4 * pl));
    CUDA_TRY(h, cudaMemset(h->nman, 0, pl));
    auto opt = [&](float*& p, bool on) -> int {
        if (!on) return RIFT_OK;
        CUDA_TRY(h, cudaMalloc(&p, pl));
        CUDA_TRY(h, cudaMemset(p, 0, pl));
        return RIFT_OK;
    };
    int r;
    if ((r = opt(h->K, h->has(RIFT_F_INFILTRATION))) || (r = opt(h->FA, h->has(RIFT_F_INFILTRATION))) ||
        (r = opt(h->FB, h->has(RIFT_F_INFILTRATION))) || (r = opt(h->hmax, h->has(RIFT_F_SAVE_MAX))) ||
        (r = opt(h->qmax, h->has(RIFT_F_SAVE_MAX))) ||
        (r = opt(h->tpeak, h->has(RIFT_F_SAVE_MAX))) || (r = opt(h->tdry, h->has(RIFT_F_SAVE_MAX))) ||
        (r = opt(h->twet, h->has(RIFT_F_SAVE_ARRIVAL))))
        return r;
    const int G = h->gridSize;
    CUDA_TRY(h, cudaMalloc(&h->wet, G));
    CUDA_TRY(h, cudaMalloc(&h->prevAct, G));
    CUDA_TRY(h, cudaMalloc(&h->act, (size_t)G * 4));
    CUDA_TRY(h, cudaMalloc(&h->deact, (size_t)G * 4));
    CUDA_TRY(h, cudaMalloc(&h->inact, (size_t)G * 4));
    CUDA_TRY(h, cudaMalloc(&h->mx, (size_t)G * 4));
    CUDA_TRY(h, cudaMalloc(&h->my, (size_t)G * 4));
    CUDA_TRY(h, cudaMemset(h->wet, 0, G));
    CUDA_TRY(h, cudaMemset(h->prevAct, 0, G));
    CUDA_TRY(h, cudaMemset(h->mx, 0, (size_t)G * 4));
    CUDA_TRY(h, cudaMemset(h->my, 0, (size_t)G * 4));
    CUDA_TRY(h, cudaMalloc(&h->srcTileStart, ((size_t)G + 1) * 4));
    CUDA_TRY(h, cudaMemset(h->srcTileStart, 0, ((size_t)G + 1) * 4));
    CUDA_TRY(h, cudaMalloc(&h->serT, 3 * MAX_SERIES * 4));
    CUDA_TRY(h, cudaMalloc(&h->serR, 3 * MAX_SERIES * 4));
    CUDA_TRY(h, cudaMalloc(&h->st, sizeof(DevState)));
    CUDA_TRY(h, cudaMallocHost(&h->hst, sizeof(DevState)));
    std::memset(h->hst, 0, sizeof(DevState));
    CUDA_TRY(h, cudaMalloc(&h->volPartial, 2 * 1024 * sizeof(double)));
    if ((r = encodeMap(h, &h->tmA, h->A, 3)) || (r = encodeMap(h, &h->tmB, h->B, 3)) ||
        (r = encodeMap(h, &h->tmE, h->E, 4)) ||
        (r = encodeMap(h, &h->tmAm, h->A, 3, MBOXW, MRC)) ||
        (r = encodeMap(h, &h->tmBm, h->B, 3, MBOXW, MRC)) ||
        (r = encodeMap(h, &h->tmEm, h->E, 4, MBOXW, MRC)))
        return r;
    if ((r = encodeMap(h, &h->tmU1.a, h->A, 3, UBOXW, URC)) ||
        (r = encodeMap(h, &h->tmU1.d, h->D, 3, UBOXW, URC)) ||
        (r = encodeMap(h, &h->tmU1.n, h->nman, 1, UBOXW, URC)))
        return r;
    CUDA_TRY(h, cudaFuncSetAttribute(k_update1<0>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     u1Smem<0>()));
    CUDA_TRY(h, cudaFuncSetAttribute(k_update1<FIX_RAIN>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     u1Smem<FIX_RAIN>()));
    CUDA_TRY(h, cudaFuncSetAttribute(k_update1<FIX_INFIL_SRC>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, u1Smem<FIX_INFIL_SRC>()));
    CUDA_TRY(h, cudaFuncSetAttribute(k_update1<FIX_RAINMAP_DRAIN>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     u1Smem<FIX_RAINMAP_DRAIN>()));
    h->nSX = (h->nBX + STRIP_TX - 1) / STRIP_TX;
    h->nSY = (h->nBY + STRIP_TY - 1) / STRIP_TY;
    const int NS = h->nSX * h->nSY;
    CUDA_TRY(h, cudaMalloc(&h->strips, (size_t)NS * 4));
    CUDA_TRY(h, cudaMalloc(&h->stripFlag, NS));
    CUDA_TRY(h, cudaMemset(h->stripFlag, 0, NS));
    int occ = 1;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_stage<1>, NT, 0);
    if (occ < 1) occ = 1;
    h->gridStage = std::max(1, std::min(G, h->numSMs * occ));
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_march<2>, MT, 0);
    if (occ < 1) occ = 1;
    h->gridMarch = std::max(1, std::min(NS, h->numSMs * occ));
    int occ1 = 1;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ1, k_march<1>, MT, 0);
    h->gridMarch1 = std::max(1, std::min(NS, h->numSMs * std::max(occ1, 1)));
    int occU = 1;
    // the gridded-rain instantiation stages two more planes (3 CTAs per SM, 4 without)
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occU, k_update1<FIX_RAINMAP_DRAIN>, MT,
                                                  u1Smem<FIX_RAINMAP_DRAIN>());
    h->gridUpdate = std::max(1, std::min(2 * NS, h->numSMs * std::max(occU, 1)));
    // the march pays off once every resident march CTA has a strip of its own
    h->marchMin = h->numSMs * occ;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_speed_dt, NT, 0);
    if (occ < 1) occ = 1;
    h->gridSpeed = std::max(1, std::min(G, h->numSMs * occ));
    h->gridTrack = std::max(1, std::min(G, h->numSMs * 4));
    h->gridDt = std::max(1, std::min((G + 255) / 256, h->numSMs * 2));
    // the cooperative step kernel: every CTA resident at once
    int coop = 0;
    cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev);
    occ = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_persist<>, NT, 0);
    for (const void* fn : {(const void*)k_persist<FIX_RAIN>, (const void*)k_persist<FIX_INFIL_SRC>}) {
        int o = 0;  // every instantiation must fit the same cooperative grid
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o, fn, NT, 0);
        occ = std::min(occ, o);
    }
    if (coop && occ > 0) {
        h->gridPersist = std::min(h->numSMs * occ, PERSIST_MAX_CTAS);
        CUDA_TRY(h, cudaMalloc(&h->gbar, sizeof(GridBar)));
        CUDA_TRY(h, cudaMalloc(&h->owner, (size_t)G * 4));
        CUDA_TRY(h, cudaMalloc(&h->tileFlag, (size_t)G * 4));
    }
    h->gridGrow = std::max(1, std::min(NS, h->numSMs * 4));
    h->persistMax = h->gridPersist > 0 ? h->marchMin * STRIP_TX * STRIP_TY : 0;
    CUDA_TRY(h, cudaStreamSynchronize(h->stream));
    return RIFT_OK;
}

int rift_upload_static(rift_handle* h, const double* BX, const double* BY, const double* n,
                       const double* K_mps, const double* h0) {
    if (!h || !BX || !BY || !n) return RIFT_ERR_ARG;
    if (h->has(RIFT_F_INFILTRATION) && !K_mps) return fail(h, RIFT_ERR_ARG, "K required");
    const int nx = h->nx, ny = h->ny;
    buildReference(h, BX, BY);
    auto bx = [&](int j, int i) { return BX[(size_t)j * (nx + 1) + i]; };
    auto by = [&](int j, int i) { return BY[(size_t)j * nx + i]; };
    std::vector<float> e[4];
    for (auto& v : e) v.assign((size_t)nx * ny, 0.f);
    for (int j = 0; j < ny; j++)
        for (int i = 0; i < nx; i++) {
            size_t c = hidx(h, j, i);
            double r = h->Bref[c];
            e[0][c] = (float)(bx(j, i) - r);
            e[1][c] = (float)(bx(j, i + 1) - r);
            e[2][c] = (float)(by(j, i) - r);
            e[3][c] = (float)(by(j + 1, i) - r);
        }
    int rc;
    for (int f = 0; f < 4; f++)
        if ((rc = upField(h, h->E + f * h->plane(), e[f]))) return rc;
    std::vector<float> tmp((size_t)nx * ny);
    for (size_t c = 0; c < tmp.size(); c++) tmp[c] = (float)n[c];
    if ((rc = upField(h, h->nman, tmp))) return rc;
    if (h->K) {
        for (size_t c = 0; c < tmp.size(); c++) tmp[c] = (float)K_mps[c];
        if ((rc = upField(h, h->K, tmp))) return rc;
    }
    h->h0_.assign(h0 ? h0 : nullptr, h0 ? h0 + (size_t)nx * ny : nullptr);
    CUDA_TRY(h, cudaStreamSynchronize(h->stream));
    h->haveStatic = true;
    if (h->hostAccess && (rc = uploadBref(h))) return rc;
    return RIFT_OK;
}


// InitGrid (grid.cu:506-553) then ApplyBoundaries (simulator.cu:731):
// h = h0 (or 0), hu = hv = 0, every in-grid tile wet and active.
int rift_init(rift_handle* h, double t0) {
    if (!h) return RIFT_ERR_ARG;
    if (!h->haveStatic) return fail(h, RIFT_ERR_STATE, "upload_static first");
    const int nx = h->nx, ny = h->ny;
    const size_t N = (size_t)nx * ny;
    std::vector<float> H(N, 0.f), U(N, 0.f), V(N, 0.f);
    if (h->has(RIFT_F_H_INIT) && !h->h0_.empty())
        for (int j = 2; j < ny; j++)
            for (int i = 2; i < nx; i++) H[hidx(h, j, i)] = (float)h->h0_[hidx(h, j, i)];
    hostGhosts(h, H.data(), U.data(), V.data());
    std::vector<uint8_t> wet(h->gridSize), actf(h->gridSize);
    bool anyOut = false;
    for (int b = 0; b < h->gridSize; b++) {
        bool in = tileInGrid(h, b);
        wet[b] = actf[b] = in ? 1 : 0;
        if (!in) anyOut = true;
    }
    // before the first Grow the only negative active_blocks entries are the
    // -1 fills of tiles InitGrid_k never reached; TrackRainfall_k maps them
    // all to tile abs(-1) = 1
    std::vector<int> inact;
    if (anyOut && h->gridSize > 1) inact.push_back(1);
    // rates and map factors set before init survive it
    float keepF[3] = {h->hst->factor[0], h->hst->factor[1], h->hst->factor[2]};
    float keepRain = h->hst->rain_rate, keepDrain = h->hst->drain_rate;
    DevState keep = *h->hst;
    std::memset(h->hst, 0, sizeof(DevState));
    for (int k = 0; k < 3; k++) {
        h->hst->factor[k] = keepF[k];
        h->hst->map_timed[k] = keep.map_timed[k];
        h->hst->map_t0[k] = keep.map_t0[k];
        h->hst->map_t1[k] = keep.map_t1[k];
    }
    h->hst->rain_rate = keepRain;
    h->hst->drain_rate = keepDrain;
    h->hst->rain_sum[0] = keep.rain_sum[0];
    h->hst->rain_sum[1] = keep.rain_sum[1];
    int rc = uploadState(h, H.data(), U.data(), V.data(), wet, actf, inact);
    if (rc) return rc;
    const size_t pl = h->plane() * 4;
    if (h->FA) {
        CUDA_TRY(h, cudaMemsetAsync(h->FA, 0, pl, h->stream));
        CUDA_TRY(h, cudaMemsetAsync(h->FB, 0, pl, h->stream));
    }
    if (h->hmax) {
        CUDA_TRY(h, cudaMemsetAsync(h->hmax, 0, pl, h->stream));
        CUDA_TRY(h, cudaMemsetAsync(h->qmax, 0, pl, h->stream));
        CUDA_TRY(h, cudaMemsetAsync(h->tpeak, 0, pl, h->stream));
        CUDA_TRY(h, cudaMemsetAsync(h->tdry, 0, pl, h->stream));
    }
    if (h->twet) {
        std::vector<float> tw(N, 0.f);
        for (int j = 2; j < ny; j++)
            for (int i = 2; i < nx; i++) tw[hidx(h, j, i)] = -9999.f;
        if ((rc = upField(h, h->twet, tw))) return rc;
    }
    CUDA_TRY(h, cudaMemsetAsync(h->mx, 0, (size_t)h->gridSize * 4, h->stream));
    CUDA_TRY(h, cudaMemsetAsync(h->my, 0, (size_t)h->gridSize * 4, h->stream));
    DevState& s = *h->hst;
    s.t = t0;
    s.dt = (double)0.0000001f;  // simulator.cu:35
    s.dt_old = s.dt;
    s.t_stop = INFINITY;
    s.nInact = (int)inact.size();
    h->inited = true;
    return ledgerStart(h);
}

int rift_set_uniform_rates(rift_handle* h, double rain_mps, double drain_mps) {
    if (!h) return RIFT_ERR_ARG;
    if (!h->inited) {
        h->hst->rain_rate = (float)rain_mps;
        h->hst->drain_rate = (float)drain_mps;
        return RIFT_OK;
    }
    int rc = pullState(h);
    if (rc) return rc;
    h->hst->rain_rate = (float)rain_mps;
    h->hst->drain_rate = (float)drain_mps;
    return pushState(h);
}

// Simulator::updateSources (simulator.cu:903-907): the per-source rates of
// the cells rift_set_point_sources placed, copied to the device before the
// next step; the cells, their tile lists and the captured step graph stay.
int rift_set_point_rates(rift_handle* h, const double* rate, int32_t n) {
    if (!h || n < 0 || (n > 0 && !rate)) return RIFT_ERR_ARG;
    if (n != h->nsrc) return fail(h, RIFT_ERR_ARG, "rate count differs from the source count");
    if (n == 0) return RIFT_OK;
    std::vector<float> fr(n);
    for (int k = 0; k < n; k++) fr[k] = (float)rate[k];
    CUDA_TRY(h, cudaMemcpyAsync(h->srcRate, fr.data(), (size_t)n * 4, cudaMemcpyHostToDevice, h->stream));
    CUDA_TRY(h, cudaStreamSynchronize(h->stream));
    return RIFT_OK;
}

int rift_set_point_sources(rift_handle* h, const int32_t* idx, const double* rate, int32_t n) {
    if (!h || n < 0 || (n > 0 && (!idx || !rate))) return RIFT_ERR_ARG;
    cudaFree(h->srcIdx);
    cudaFree(h->srcRate);
    cudaFree(h->srcTileList);
    h->srcIdx = nullptr;
    h->srcRate = nullptr;
    h->srcTileList = nullptr;
    h->nsrc = n;
    std::vector<int> start(h->gridSize + 1, 0), list;
    if (n > 0) {
        std::vector<int> tileOf(n, -1);
        for (int k = 0; k < n; k++) {
            int i = idx[k] % h->nx, j = idx[k] / h->nx;
            if (idx[k] >= 0 && i >= 2 && j >= 2 && j < h->ny)
                tileOf[k] = ((j - 2) / TH) * h->nBX + (i - 2) / TW;
            if (tileOf[k] >= h->gridSize) tileOf[k] = -1;
            if (tileOf[k] >= 0) start[tileOf[k] + 1]++;
        }
        for (int b = 0; b < h->gridSize; b++) start[b + 1] += start[b];
        list.assign(std::max(1, start[h->gridSize]), 0);
        std::vector<int> fill(start.begin(), start.end() - 1);
        for (int k = 0; k < n; k++)
            if (tileOf[k] >= 0) list[fill[tileOf[k]]++] = k;
        std::vector<float> fr(n);
        for (int k = 0; k < n; k++) fr[k] = (float)rate[k];
        CUDA_TRY(h, cudaMalloc(&h->srcIdx, (size_t)n * 4));
        CUDA_TRY(h, cudaMalloc(&h->srcRate, (size_t)n * 4));
        CUDA_TRY(h, cudaMalloc(&h->srcTileList, list.size() * 4));
        CUDA_TRY(h, cudaMemcpyAsync(h->srcIdx, idx, (size_t)n * 4, cudaMemcpyHostToDevice, h->stream));
        CUDA_TRY(h, cudaMemcpyAsync(h->srcRate, fr.data(), (size_t)n * 4, cudaMemcpyHostToDevice, h->stream));
        CUDA_TRY(h, cudaMemcpyAsync(h->srcTileList, list.data(), list.size() * 4,
                                    cudaMemcpyHostToDevice, h->stream));
    }
    CUDA_TRY(h, cudaMemcpyAsync(h->srcTileStart, start.data(), start.size() * 4,
                                cudaMemcpyHostToDevice, h->stream));
    CUDA_TRY(h, cudaStreamSynchronize(h->stream));
    destroyGraph(h);
    return RIFT_OK;
}

int rift_set_map(rift_handle* h, int32_t which, const double* t0map, const double* t1map,
                 double factor) {
    if (!h || which < 0 || which > 2 || !t0map) return RIFT_ERR_ARG;
    const size_t N = (size_t)h->nx * h->ny, pl = h->plane() * 4;
    int newMode = t1map ? 2 : 1;
    for (int k = 0; k < newMode; k++)
        if (!h->maps[which][k]) {
            CUDA_TRY(h, cudaMalloc(&h->maps[which][k], pl));
            CUDA_TRY(h, cudaMemset(h->maps[which][k], 0, pl));
        }
    std::vector<float> tmp(N);
    int rc;
    // interior sums of the maps as the device holds them (rain volume ledger)
    auto interiorSum = [&]() {
        double sum = 0.0;
        for (int j = 2; j < h->ny - 2; j++)
            for (int i = 2; i < h->nx - 2; i++) sum += (double)tmp[hidx(h, j, i)];
        return sum;
    };
    double sums[2] = {0.0, 0.0};
    for (size_t c = 0; c < N; c++) tmp[c] = (float)t0map[c];
    sums[0] = interiorSum();
    if ((rc = upField(h, h->maps[which][0], tmp))) return rc;
    if (t1map) {
        for (size_t c = 0; c < N; c++) tmp[c] = (float)t1map[c];
        sums[1] = interiorSum();
        if ((rc = upField(h, h->maps[which][1], tmp))) return rc;
    }
    if (h->mapMode[which] != newMode) destroyGraph(h);
    h->mapMode[which] = newMode;
    if (h->inited && (rc = pullState(h))) return rc;
    h->hst->factor[which] = (float)factor;
    if (which == RIFT_MAP_RAIN) {
        h->hst->rain_sum[0] = sums[0];
        h->hst->rain_sum[1] = sums[1];
    }
    if (h->inited) return pushState(h);
    CUDA_TRY(h, cudaStreamSynchronize(h->stream));
    return RIFT_OK;
}

int rift_set_map_factor(rift_handle* h, int32_t which, double factor) {
    if (!h || which < 0 || which > 2 || !h->mapMode[which]) return RIFT_ERR_ARG;
    int rc = pullState(h);
    if (rc) return rc;
    h->hst->factor[which] = (float)factor;
    return pushState(h);
}

int rift_set_schedule(rift_handle* h, int32_t march_min_strips) {
    if (!h) return RIFT_ERR_ARG;
    int occ = 1;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_march<2>, MT, 0);
    h->marchMin = march_min_strips >= 0 ? march_min_strips : h->numSMs * std::max(occ, 1);
    destroyGraph(h);
    return RIFT_OK;
}

int rift_set_persistent(rift_handle* h, int32_t max_active_tiles) {
    if (!h) return RIFT_ERR_ARG;
    if (h->gridPersist == 0) {
        h->persistMax = 0;
        return max_active_tiles > 0 ? fail(h, RIFT_ERR_UNSUPPORTED, "no cooperative launch")
                                    : RIFT_OK;
    }
    h->persistMax = max_active_tiles >= 0 ? max_active_tiles
                                          : h->marchMin * STRIP_TX * STRIP_TY;
    destroyGraph(h);  // the step graph holds the bound
    return RIFT_OK;
}

int rift_set_map_times(rift_handle* h, int32_t which, double t0, double t1) {
    if (!h || which < 0 || which > 2 || !h->mapMode[which]) return RIFT_ERR_ARG;
    if (h->inited) {
        int rc = pullState(h);
        if (rc) return rc;
    }
    h->hst->map_timed[which] = (t1 > t0) ? 1 : 0;
    h->hst->map_t0[which] = t0;
    h->hst->map_t1[which] = t1;
    return h->inited ? pushState(h) : RIFT_OK;
}

int rift_set_series(rift_handle* h, int32_t which, const float* times, const float* rates,
                    int32_t n) {
    if (!h || which < 0 || which > 2 || n < 0 || n > MAX_SERIES || (n > 0 && (!times || !rates)))
        return RIFT_ERR_ARG;
    if (n > 0) {
        CUDA_TRY(h, cudaMemcpyAsync(h->serT + which * MAX_SERIES, times, (size_t)n * 4,
                                    cudaMemcpyHostToDevice, h->stream));
        CUDA_TRY(h, cudaMemcpyAsync(h->serR + which * MAX_SERIES, rates, (size_t)n * 4,
                                    cudaMemcpyHostToDevice, h->stream));
    }
    CUDA_TRY(h, cudaStreamSynchronize(h->stream));
    if (h->serN[which] != n) destroyGraph(h);
    h->serN[which] = n;
    return RIFT_OK;
}

namespace {

// One cooperative launch of the step loop for at most `nsteps` steps.  The
// grid is a whole number of CTAs per SM, enough for one active tile per CTA
// at the last known count (up to full occupancy): a smaller grid makes each
// grid barrier cheaper.
int persistGrid(const rift_handle* h) {
    // before the first step the count is unknown: full occupancy
    const int perSM = h->hst->nActive > 0 ? (h->hst->nActive + h->numSMs - 1) / h->numSMs
                                          : h->gridPersist / h->numSMs;
    return std::max(1, std::min(h->gridPersist, h->numSMs * perSM));
}

int launchPersist(rift_handle* h, int nsteps) {
    CUDA_TRY(h, cudaMemsetAsync(h->gbar, 0, GRIDBAR_CLEAR, h->stream));
    Params P = makeParams(h);
    const int grid = persistGrid(h);
    void* args[] = {(void*)&h->tmA, (void*)&h->tmB, (void*)&h->tmE, (void*)&P, (void*)&nsteps};
    CUDA_TRY(h, cudaLaunchCooperativeKernel(persistKernel(h), dim3(grid), dim3(NT), args, 0,
                                            h->stream));
    h->launches += 1;
    return RIFT_OK;
}

// Runs up to `nsteps` steps (state pushed, t_stop set; the host mirror of
// the device state current).  While the active set is small the cooperative
// step kernel runs the steps in one launch; once the active tiles outnumber
// persistMax it leaves at a step boundary and the per-step graph (tile or
// march kernels, chosen on the device) continues, in chunks of
// kGraphChunk steps after which the host checks for t_stop and looks at the
// active count again.
constexpr int kGraphChunk = 64;

int runSteps(rift_handle* h, int nsteps, bool* mirrorCurrent) {
    int rc;
    int left = nsteps;
    *mirrorCurrent = false;
    while (left > 0) {
        if (h->persistMax > 0 && h->hst->nActive <= h->persistMax) {
            const int before = h->hst->steps_done;
            if ((rc = launchPersist(h, left)) || (rc = pullState(h))) return rc;
            *mirrorCurrent = true;
            const int ran = h->hst->steps_done - before;
            h->persistSteps += ran;
            left -= ran;
            if (!h->hst->persistExit) break;  // all steps done, or t_stop reached
        }
        if (left <= 0) break;
        const int chunk = std::min(left, kGraphChunk);
        if ((rc = buildGraph(h))) return rc;
        for (int k = 0; k < chunk; k++) CUDA_TRY(h, cudaGraphLaunch(h->graphExec, h->stream));
        h->graphSteps += chunk;
        h->launches += (long long)chunk * h->graphKernels;
        left -= chunk;
        *mirrorCurrent = false;
        if (left > 0) {
            if ((rc = pullState(h))) return rc;
            *mirrorCurrent = true;
            if (h->hst->stop) break;
        }
    }
    CUDA_TRY(h, cudaGetLastError());
    return RIFT_OK;
}

}  // namespace

namespace {
// rift_step on the persistent loop as one graph: state push, barrier reset,
// the one-step cooperative launch, state pull -- one launch and one wait
// per step.  Rebuilt when the grid changes; false if the graph cannot be
// made (the caller launches directly).
bool stepGraph(rift_handle* h, int& rc) {
    rc = RIFT_OK;
    if (h->stepGraphBroken) return false;
    const int grid = persistGrid(h);
    int slot = -1;
    for (int k = 0; k < rift_handle::STEP_CACHE; k++)
        if (h->stepExec[k] && h->stepGrid[k] == grid) slot = k;
    if (slot < 0) {
        slot = h->stepNext;
        h->stepNext = (h->stepNext + 1) % rift_handle::STEP_CACHE;
        if (h->stepExec[slot]) cudaGraphExecDestroy(h->stepExec[slot]);
        h->stepExec[slot] = nullptr;
        Params P = makeParams(h);
        int one = 1;
        void* args[] = {(void*)&h->tmA, (void*)&h->tmB, (void*)&h->tmE, (void*)&P, (void*)&one};
        cudaGraph_t g = nullptr;
        if (cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
            h->stepGraphBroken = true;
            cudaGetLastError();
            return false;
        }
        cudaMemcpyAsync(h->st, h->hst, sizeof(DevState), cudaMemcpyHostToDevice, h->stream);
        cudaMemsetAsync(h->gbar, 0, GRIDBAR_CLEAR, h->stream);
        cudaLaunchCooperativeKernel(persistKernel(h), dim3(grid), dim3(NT), args, 0, h->stream);
        cudaMemcpyAsync(h->hst, h->st, sizeof(DevState), cudaMemcpyDeviceToHost, h->stream);
        cudaError_t e = cudaStreamEndCapture(h->stream, &g);
        if (e != cudaSuccess || !g ||
            cudaGraphInstantiate(&h->stepExec[slot], g, 0) != cudaSuccess) {
            if (g) cudaGraphDestroy(g);
            h->stepExec[slot] = nullptr;
            h->stepGraphBroken = true;
            cudaGetLastError();
            return false;
        }
        cudaGraphDestroy(g);
        h->stepGrid[slot] = grid;
    }
    const int before = h->hst->steps_done;
    cudaError_t e = cudaGraphLaunch(h->stepExec[slot], h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) {
        rc = fail(h, RIFT_ERR_CUDA, std::string("step graph: ") + cudaGetErrorString(e));
        return true;
    }
    if (h->hst->error) {
        rc = fail(h, RIFT_ERR_CUDA, deviceErrorText(h->hst->error));
        return true;
    }
    h->persistSteps += h->hst->steps_done - before;
    h->launches += 1;
    return true;
}
}  // namespace

int rift_run(rift_handle* h, int32_t nsteps, double t_stop, double* t, double* dt,
             int32_t* steps_done) {
    if (!h || nsteps < 0) return RIFT_ERR_ARG;
    if (!h->inited) return fail(h, RIFT_ERR_STATE, "init first");
    // every entry point leaves the pinned mirror equal to the device state
    h->hst->t_stop = t_stop;
    h->hst->steps_done = 0;
    int rc;
    bool current = false;
    if (nsteps == 1 && h->persistMax > 0 && h->hst->nActive <= h->persistMax &&
        stepGraph(h, rc)) {
        if (rc) return rc;
        if (t) *t = h->hst->t;
        if (dt) *dt = h->hst->dt;
        if (steps_done) *steps_done = h->hst->steps_done;
        return RIFT_OK;
    }
    if ((rc = pushStateAsync(h)) || (rc = runSteps(h, nsteps, &current))) return rc;
    if (!current && (rc = pullState(h))) return rc;
    if (t) *t = h->hst->t;
    if (dt) *dt = h->hst->dt;
    if (steps_done) *steps_done = h->hst->steps_done;
    return RIFT_OK;
}

int rift_step(rift_handle* h, double* t, double* dt) {
    int32_t done = 0;
    int rc = rift_run(h, 1, INFINITY, t, dt, &done);
    return rc;
}

int rift_get_time(rift_handle* h, double* t, double* dt) {
    if (!h) return RIFT_ERR_ARG;
    int rc = pullState(h);
    if (rc) return rc;
    if (t) *t = h->hst->t;
    if (dt) *dt = h->hst->dt;
    return RIFT_OK;
}

int rift_get_tile_grid(rift_handle* h, int32_t* nBX, int32_t* nBY) {
    if (!h) return RIFT_ERR_ARG;
    if (nBX) *nBX = h->nBX;
    if (nBY) *nBY = h->nBY;
    return RIFT_OK;
}

int rift_set_host_access(rift_handle* h, int32_t on) {
    if (!h) return RIFT_ERR_ARG;
    if (on && !h->hostAccessOk) return fail(h, RIFT_ERR_UNSUPPORTED, "device cannot access pageable host memory");
    h->hostAccess = on != 0;
    if (h->hostAccess && h->haveStatic) return uploadBref(h);
    return RIFT_OK;
}

int rift_get_host_access(rift_handle* h, int32_t* on) {
    if (!h || !on) return RIFT_ERR_ARG;
    *on = h->hostAccess ? 1 : 0;
    return RIFT_OK;
}

int rift_get_device_view(rift_handle* h, rift_device_view* v) {
    if (!h || !v) return RIFT_ERR_ARG;
    if (!h->haveStatic) return fail(h, RIFT_ERR_STATE, "upload the static fields first");
    const size_t pl = h->plane();
    v->h = h->A;
    v->hu = h->A + pl;
    v->hv = h->A + 2 * pl;
    v->e = h->E;
    v->n = h->nman;
    v->t = &h->st->t;
    v->dt = &h->st->dt;
    v->stream = (void*)h->stream;
    v->h_nx = h->nx;
    v->h_ny = h->ny;
    v->pitch = h->pitch;
    v->rows = h->rows;
    v->dx = h->g.dx;
    v->dy = h->g.dy;
    v->kappa = h->g.kappa;
    return RIFT_OK;
}

int rift_get_field(rift_handle* h, int32_t which, double* host, size_t ld) {
    if (!h || !host || ld < (size_t)h->nx) return RIFT_ERR_ARG;
    const int nx = h->nx, ny = h->ny;
    const size_t pl = h->plane();
    const size_t N = (size_t)nx * ny;
    if (h->hostAccess) {
        // written by the device straight into the caller's array
        const float* src = nullptr;
        int mode = 0;
        switch (which) {
            case RIFT_FIELD_W: src = h->BrefD ? h->A : nullptr; mode = 1; break;
            case RIFT_FIELD_HU: src = h->A + pl; break;
            case RIFT_FIELD_HV: src = h->A + 2 * pl; break;
            case RIFT_FIELD_H: src = h->A; mode = 2; break;
            case RIFT_FIELD_F: src = h->FA; break;
            case RIFT_FIELD_HMAX: src = h->hmax; break;
            case RIFT_FIELD_QMAX: src = h->qmax; break;
            case RIFT_FIELD_TPEAK: src = h->tpeak; break;
            case RIFT_FIELD_TDRY: src = h->tdry; break;
            case RIFT_FIELD_TWET: src = h->twet; break;
            default: break;
        }
        if (src) {
            k_export<<<h->numSMs * 8, 256, 0, h->stream>>>(src, h->BrefD, host, ld, h->pitch, nx, ny, mode);
            CUDA_TRY(h, cudaGetLastError());
            CUDA_TRY(h, cudaStreamSynchronize(h->stream));
            return RIFT_OK;
        }
    }
    float* const a = stagePlanes(h, 4);
    if (!a) return fail(h, RIFT_ERR_NOMEM, "pinned staging planes");
    float* const b = a + N;
    float* const c = a + 2 * N;
    int rc = 0;
    auto put = [&](auto fn) {
        parallelRows(ny, N, [&](int j0, int j1) {
            for (int j = j0; j < j1; j++)
                for (int i = 0; i < nx; i++) host[(size_t)j * ld + i] = fn(j, i);
        });
    };
    auto zero = [&](int, int) { return 0.0; };
    switch (which) {
        case RIFT_FIELD_W:
            if ((rc = downField(h, h->A, a))) return rc;
            put([&](int j, int i) { return h->Bref[hidx(h, j, i)] + (double)a[hidx(h, j, i)]; });
            break;
        case RIFT_FIELD_HU:
        case RIFT_FIELD_HV:
            if ((rc = downField(h, h->A + (which == RIFT_FIELD_HU ? 1 : 2) * pl, a))) return rc;
            put([&](int j, int i) { return (double)a[hidx(h, j, i)]; });
            break;
        case RIFT_FIELD_H:
            if ((rc = downField(h, h->A, a))) return rc;
            put([&](int j, int i) {
                bool in = i >= 2 && j >= 2 && i <= nx - 3 && j <= ny - 3;
                float v = a[hidx(h, j, i)];
                return in ? (double)((v > kEps) ? v : 0.f) : 0.0;
            });
            break;
        case RIFT_FIELD_Q:
            if ((rc = downField(h, h->A, a)) || (rc = downField(h, h->A + pl, b)) ||
                (rc = downField(h, h->A + 2 * pl, c)))
                return rc;
            put([&](int j, int i) {
                bool in = i >= 2 && j >= 2 && i <= nx - 3 && j <= ny - 3;
                if (!in) return 0.0;
                size_t q = hidx(h, j, i);
                float hc = (a[q] > kEps) ? a[q] : 0.f;
                float h2 = hc * hc;
                float fac = 2.f * hc / (h2 + std::fmax(h2, (float)h->g.kappa));
                float u = b[q] * fac, v = c[q] * fac;
                return (double)(hc * std::sqrt(v * v + u * u));
            });
            break;
        case RIFT_FIELD_BC:
            put([&](int j, int i) { return h->BC[hidx(h, j, i)]; });
            break;
        case RIFT_FIELD_F:
        case RIFT_FIELD_HMAX:
        case RIFT_FIELD_QMAX:
        case RIFT_FIELD_TPEAK:
        case RIFT_FIELD_TDRY:
        case RIFT_FIELD_TWET: {
            const float* src = which == RIFT_FIELD_F      ? h->FA
                               : which == RIFT_FIELD_HMAX ? h->hmax
                               : which == RIFT_FIELD_QMAX ? h->qmax
                               : which == RIFT_FIELD_TPEAK ? h->tpeak
                               : which == RIFT_FIELD_TDRY ? h->tdry
                                                          : h->twet;
            if (!src) {
                put(zero);
                break;
            }
            if ((rc = downField(h, src, a))) return rc;
            put([&](int j, int i) { return (double)a[hidx(h, j, i)]; });
            break;
        }
        default:
            return RIFT_ERR_ARG;
    }
    return RIFT_OK;
}

int rift_get_tiles(rift_handle* h, uint8_t* wet, int32_t* active, int32_t* n_active) {
    if (!h) return RIFT_ERR_ARG;
    int rc = pullState(h);
    if (rc) return rc;
    std::vector<uint8_t> flags(h->gridSize);
    // the active set of the last step is prevAct (the grow keeps it per tile)
    CUDA_TRY(h, cudaMemcpyAsync(flags.data(), h->prevAct, h->gridSize, cudaMemcpyDeviceToHost, h->stream));
    if (wet) CUDA_TRY(h, cudaMemcpyAsync(wet, h->wet, h->gridSize, cudaMemcpyDeviceToHost, h->stream));
    CUDA_TRY(h, cudaStreamSynchronize(h->stream));
    int k = 0;
    for (int b = 0; b < h->gridSize; b++)
        if (flags[b]) {
            if (active) active[k] = b;
            k++;
        }
    if (n_active) *n_active = k;
    return RIFT_OK;
}

int rift_get_tile_speeds(rift_handle* h, double* mx, double* my) {
    if (!h) return RIFT_ERR_ARG;
    std::vector<float> a(h->gridSize), b(h->gridSize);
    CUDA_TRY(h, cudaMemcpyAsync(a.data(), h->mx, (size_t)h->gridSize * 4, cudaMemcpyDeviceToHost, h->stream));
    CUDA_TRY(h, cudaMemcpyAsync(b.data(), h->my, (size_t)h->gridSize * 4, cudaMemcpyDeviceToHost, h->stream));
    CUDA_TRY(h, cudaStreamSynchronize(h->stream));
    for (int k = 0; k < h->gridSize; k++) {
        if (mx) mx[k] = a[k];
        if (my) my[k] = b[k];
    }
    return RIFT_OK;
}

// Simulator::ReadHotstart (simulator.cu:975-1090) followed by ApplyBoundaries
// (simulator.cu:731): state in the reference representation.
int rift_set_state(rift_handle* h, double t, double dt_prev, const double* w, const double* hu,
                   const double* hv, const double* F, const uint8_t* wet,
                   const int32_t* active_ids, int32_t n_active, const double* mx, const double* my) {
    if (!h || !w || !hu || !hv) return RIFT_ERR_ARG;
    if (!h->inited) return fail(h, RIFT_ERR_STATE, "init first");
    const int nx = h->nx, ny = h->ny;
    const size_t N = (size_t)nx * ny;
    int rc = pullState(h);  // also: no earlier copy still reads the staging planes
    if (rc) return rc;
    float* const H = stagePlanes(h, 4);
    if (!H) return fail(h, RIFT_ERR_NOMEM, "pinned staging planes");
    float* const U = H + N;
    float* const V = H + 2 * N;
    const bool direct = h->hostAccess && h->BrefD;
    // Once the import kernel reads the caller's arrays, every exit (the error
    // returns included) waits for the stream, so the caller may free them.
    struct SyncOnExit {
        cudaStream_t s;
        bool armed;
        ~SyncOnExit() {
            if (armed) cudaStreamSynchronize(s);
        }
    } guard{h->stream, false};
    if (direct) {
        // U^n (and F) converted on the device from the caller's arrays; the
        // ghost cells from the border, computed here as hostGhosts does
        guard.armed = true;
        const size_t pl = h->plane();
        const bool withF = F && h->FA;
        k_import<<<h->numSMs * 8, 256, 0, h->stream>>>(w, hu, hv, withF ? F : nullptr, h->BrefD, h->A,
                                                       h->FA, h->FB, pl, h->pitch, nx, ny);
        CUDA_TRY(h, cudaGetLastError());
        auto crit = [](float q, float d) { return std::fmin(std::cbrt(q * q / kG), d); };
        auto cell = [&](int j, int i, float* v) {
            const size_t c = hidx(h, j, i);
            v[0] = depthFromW(h, w[c], j, i);
            v[1] = (float)hu[c];
            v[2] = (float)hv[c];
        };
        float* gb = H;  // 6 (ny-4) + 6 (nx-4) floats of the pinned staging
        for (int j = 2; j <= ny - 3; j++)
            for (int side = 0; side < 2; side++) {
                float v[3];
                cell(j, side ? nx - 3 : 2, v);
                float HL = crit(v[1], v[0]);
                float* o = gb + 6 * (size_t)(j - 2) + 3 * side;
                o[0] = (HL > kEps) ? HL : 0.f;
                o[1] = v[1];
                o[2] = v[2];
            }
        for (int i = 2; i <= nx - 3; i++)
            for (int side = 0; side < 2; side++) {
                float v[3];
                cell(side ? ny - 3 : 2, i, v);
                float* o = gb + 6 * (size_t)(ny - 4) + 6 * (size_t)(i - 2) + 3 * side;
                o[0] = crit(v[2], v[0]);
                o[1] = v[1];
                o[2] = v[2];
            }
        const int nb = (ny - 4) + (nx - 4);
        k_ghostsFromBorder<<<(nb + 255) / 256, 256, 0, h->stream>>>(gb, h->A, pl, h->pitch, nx, ny);
        CUDA_TRY(h, cudaGetLastError());
    } else {
        parallelRows(ny, N, [&](int j0, int j1) {
            for (int j = j0; j < j1; j++)
                for (int i = 0; i < nx; i++) {
                    size_t c = hidx(h, j, i);
                    H[c] = depthFromW(h, w[c], j, i);
                    U[c] = (float)hu[c];
                    V[c] = (float)hv[c];
                }
        });
        hostGhosts(h, H, U, V);
    }
    std::vector<uint8_t> wetv(h->gridSize), actf(h->gridSize);
    CUDA_TRY(h, cudaMemcpyAsync(wetv.data(), h->wet, h->gridSize, cudaMemcpyDeviceToHost, h->stream));
    CUDA_TRY(h, cudaMemcpyAsync(actf.data(), h->prevAct, h->gridSize, cudaMemcpyDeviceToHost, h->stream));
    CUDA_TRY(h, cudaStreamSynchronize(h->stream));
    if (wet) std::copy(wet, wet + h->gridSize, wetv.begin());
    if (active_ids && n_active >= 0) {
        std::fill(actf.begin(), actf.end(), 0);
        for (int k = 0; k < n_active; k++)
            if (active_ids[k] >= 0 && active_ids[k] < h->gridSize) actf[active_ids[k]] = 1;
    }
    std::vector<int> inact;
    for (int b = 1; b < h->gridSize; b++)
        if (!actf[b]) inact.push_back(b);
    if ((rc = uploadState(h, direct ? nullptr : H, U, V, wetv, actf, inact))) return rc;
    if (direct) {
        // the caller's arrays stay in use until the import kernel is done
        CUDA_TRY(h, cudaStreamSynchronize(h->stream));
    } else if (F && h->FA) {
        float* const f = H + 3 * N;
        parallelRows(ny, N, [&](int j0, int j1) {
            for (size_t c = (size_t)j0 * nx; c < (size_t)j1 * nx; c++) f[c] = (float)F[c];
        });
        if ((rc = upField(h, h->FA, f)) || (rc = upField(h, h->FB, f))) return rc;
    }
    if (mx || my) {
        std::vector<float> a(h->gridSize), b(h->gridSize);
        for (int k = 0; k < h->gridSize; k++) {
            a[k] = mx ? (float)mx[k] : 0.f;
            b[k] = my ? (float)my[k] : 0.f;
        }
        CUDA_TRY(h, cudaMemcpyAsync(h->mx, a.data(), a.size() * 4, cudaMemcpyHostToDevice, h->stream));
        CUDA_TRY(h, cudaMemcpyAsync(h->my, b.data(), b.size() * 4, cudaMemcpyHostToDevice, h->stream));
    }
    h->hst->t = t;
    h->hst->dt = dt_prev;
    h->hst->dt_old = dt_prev;
    return ledgerStart(h);
}

int rift_mass_ledger(rift_handle* h, double* volume, double* added) {
    if (!h || !volume || !added) return RIFT_ERR_ARG;
    int rc = rift_volume(h, volume);
    if (rc || (rc = pullState(h))) return rc;
    *added = h->hst->v_added;
    return RIFT_OK;
}

int rift_mass_ledger_terms(rift_handle* h, rift_ledger* out) {
    if (!h || !out) return RIFT_ERR_ARG;
    if (!h->inited) return fail(h, RIFT_ERR_STATE, "init first");
    rift_ledger L{};
    int rc;
    if ((rc = volumeSum(h, 1, &L.volume)) || (rc = volumeSum(h, 2, &L.soil)) || (rc = pullState(h)))
        return rc;
    const DevState& s = *h->hst;
    L.volume0 = h->ledVol0;
    L.soil0 = h->ledSoil0;
    L.added = s.v_added - h->ledAdded0;
    L.drained = s.led[LED_DRAIN];
    L.infiltrated = s.led[LED_INFIL];
    L.clamped = s.led[LED_CLAMP];
    L.surge = s.led[LED_SURGE];
    L.boundary = s.led[LED_BOUND];
    *out = L;
    return RIFT_OK;
}

int rift_volume(rift_handle* h, double* volume) {
    if (!h || !volume) return RIFT_ERR_ARG;
    return volumeSum(h, 0, volume);
}

}  // extern "C"

namespace {
// Compensated volume sum (k_volume's `what`) into *out.
int volumeSum(rift_handle* h, int what, double* out) {
    Params P = makeParams(h);
    const int blocks = 1024;
    k_volume<<<blocks, 256, 0, h->stream>>>(P, h->volPartial, what);
    std::vector<double> part(2 * blocks);
    CUDA_TRY(h, cudaMemcpyAsync(part.data(), h->volPartial, part.size() * 8, cudaMemcpyDeviceToHost,
                                h->stream));
    CUDA_TRY(h, cudaStreamSynchronize(h->stream));
    double S = 0.0, C = 0.0;
    for (int b = 0; b < blocks; b++) {
        double v = part[2 * b];
        double t = S + v;
        C += (std::fabs(S) >= std::fabs(v)) ? (S - t) + v : (v - t) + S;
        S = t;
        C += part[2 * b + 1];
    }
    *out = S + C;
    return RIFT_OK;
}

// Start of the check_volume ledger: its terms zeroed, the volumes and the
// source total of this moment kept (the device state is synchronised).
int ledgerStart(rift_handle* h) {
    int rc;
    for (int k = 0; k < LED_N; k++) h->hst->led[k] = 0.0;
    h->hst->ledPend = 0.0;
    if ((rc = pushState(h))) return rc;
    h->ledAdded0 = h->hst->v_added;
    h->ledVol0 = h->ledSoil0 = NAN;  // kept only for check_volume runs
    if (!h->has(RIFT_F_CHECK_VOLUME)) return RIFT_OK;
    if ((rc = volumeSum(h, 1, &h->ledVol0)) || (rc = volumeSum(h, 2, &h->ledSoil0))) return rc;
    return RIFT_OK;
}
}  // namespace

extern "C" {

// Timed run for measurement: nsteps graph replays bracketed by CUDA events on
// the handle's stream (ms_total), then up to 20 more steps launched one by
// one with events around the two fused stage kernels (stage_ms: their mean
// duration per step, active_cells: mean active interior cells per step of
// that pass).  Active cells of the graph pass go to *active_total.
int rift_bench_run(rift_handle* h, int32_t nsteps, double* ms_total, double* active_total,
                   double* steps_done, double* stage_ms, double* active_cells) {
    if (!h || nsteps < 1) return RIFT_ERR_ARG;
    if (!h->inited) return fail(h, RIFT_ERR_STATE, "init first");
    int rc = pullState(h);
    if (rc) return rc;
    h->hst->t_stop = INFINITY;
    h->hst->steps_done = 0;
    h->hst->activeCells = 0;
    if ((rc = pushState(h)) || (rc = buildGraph(h))) return rc;
    cudaEvent_t e0, e1;
    CUDA_TRY(h, cudaEventCreate(&e0));
    CUDA_TRY(h, cudaEventCreate(&e1));
    CUDA_TRY(h, cudaStreamSynchronize(h->stream));
    // the timed region carries an NVTX range so that a profiler can select
    // exactly these launches (no cost without a profiler attached)
    nvtxRangePushA("rift_bench_timed");
    CUDA_TRY(h, cudaEventRecord(e0, h->stream));
    bool current = false;
    if ((rc = runSteps(h, nsteps, &current))) return rc;
    CUDA_TRY(h, cudaEventRecord(e1, h->stream));
    nvtxRangePop();
    CUDA_TRY(h, cudaEventSynchronize(e1));
    float ms = 0.f;
    CUDA_TRY(h, cudaEventElapsedTime(&ms, e0, e1));
    if ((rc = pullState(h))) return rc;
    if (ms_total) *ms_total = ms;
    if (steps_done) *steps_done = h->hst->steps_done;
    double graphCells = (double)h->hst->activeCells;
    // per-kernel pass
    const int M = std::min(nsteps, 20);
    h->hst->activeCells = 0;
    if ((rc = pushState(h))) return rc;
    refreshUpdateMaps(h);
    Params P = makeParams(h);
    cudaStream_t s = h->stream;
    double stageSum = 0.0;
    for (int k = 0; k < M; k++) {
        if (h->has(RIFT_F_RAIN_GRID) || h->has(RIFT_F_SURGE_GRID))
            k_track<<<h->gridTrack, NT, 0, s>>>(P);
        k_grow<<<h->gridGrow, NT, 0, s>>>(P);
        k_speed_dt<<<h->gridSpeed, NT, 0, s>>>(h->tmA, h->tmE, P);
        CUDA_TRY(h, cudaEventRecord(e0, s));
        launchMarch<1>(h, h->tmAm, P, s, h->gridMarch1);
        k_stage<1><<<h->gridStage, NT, 0, s>>>(h->tmA, h->tmE, P);
        launchUpdate1(h, P, s);
        if (!h->has(RIFT_F_EULER)) {
            k_stage<2><<<h->gridStage, NT, 0, s>>>(h->tmB, h->tmE, P);
            launchMarch<2>(h, h->tmBm, P, s, h->gridMarch);
            } else {
            k_commit<<<h->gridStage, NT, 0, s>>>(P);
        }
        CUDA_TRY(h, cudaEventRecord(e1, s));
        CUDA_TRY(h, cudaEventSynchronize(e1));
        float sm = 0.f;
        CUDA_TRY(h, cudaEventElapsedTime(&sm, e0, e1));
        stageSum += sm;
    }
    CUDA_TRY(h, cudaGetLastError());
    if ((rc = pullState(h))) return rc;
    if (stage_ms) *stage_ms = stageSum / M;
    if (active_cells) *active_cells = (double)h->hst->activeCells / M;
    if (active_total) *active_total = graphCells;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return RIFT_OK;
}

int rift_set_march_rows(rift_handle* h, int32_t tile_rows) {
    if (!h) return RIFT_ERR_ARG;
    if (tile_rows != 1 && tile_rows != 2 && tile_rows != 4)
        return fail(h, RIFT_ERR_ARG, "march work items are 1, 2 or 4 tile rows high");
    h->marchRows = tile_rows;
    destroyGraph(h);
    return RIFT_OK;
}

int rift_get_march_rows(rift_handle* h, int32_t* tile_rows) {
    if (!h || !tile_rows) return RIFT_ERR_ARG;
    *tile_rows = h->marchRows;
    return RIFT_OK;
}

int rift_get_path_stats(rift_handle* h, int64_t* persist_steps, int64_t* graph_steps) {
    if (!h) return RIFT_ERR_ARG;
    if (persist_steps) *persist_steps = h->persistSteps;
    if (graph_steps) *graph_steps = h->graphSteps;
    return RIFT_OK;
}

int rift_get_launch_count(rift_handle* h, int64_t* kernels) {
    if (!h || !kernels) return RIFT_ERR_ARG;
    *kernels = h->launches;
    return RIFT_OK;
}

int rift_get_table_steps(rift_handle* h, int64_t* table_steps) {
    if (!h || !table_steps) return RIFT_ERR_ARG;
    *table_steps = h->hst ? h->hst->tableSteps : 0;
    return RIFT_OK;
}

// ---------------------------------------------------------------- autotuner
namespace {
// Device regions that a step writes (state, outputs, tile arrays).
std::vector<std::pair<void*, size_t>> stepRegions(rift_handle* h) {
    const size_t pl = h->plane() * 4, G = (size_t)h->gridSize;
    const size_t NS = (size_t)h->nSX * h->nSY;
    std::vector<std::pair<void*, size_t>> r = {
        {h->A, 3 * pl}, {h->B, 3 * pl}, {h->wet, G}, {h->prevAct, G}, {h->act, 4 * G},
        {h->deact, 4 * G}, {h->inact, 4 * G}, {h->mx, 4 * G}, {h->my, 4 * G},
        {h->strips, 4 * NS}, {h->stripFlag, NS}, {h->srcRate, 4 * (size_t)h->nsrc}};
    for (float* p : {h->FA, h->FB, h->hmax, h->qmax, h->twet, h->tpeak, h->tdry})
        if (p) r.push_back({p, pl});
    return r;
}
}  // namespace

int rift_autotune(rift_handle* h, int32_t probe_steps, int32_t* choice, double* ms_per_step) {
    if (!h || probe_steps < 1) return RIFT_ERR_ARG;
    if (!h->inited) return fail(h, RIFT_ERR_STATE, "init first");
    int rc;
    auto regions = stepRegions(h);
    size_t total = 0;
    for (auto& r : regions) total += (r.first ? r.second : 0);
    char* scratch = nullptr;
    CUDA_TRY(h, cudaMalloc(&scratch, total));
    const DevState saved = *h->hst;  // the mirror equals the device state
    auto copyAll = [&](bool save) -> int {
        size_t off = 0;
        for (auto& r : regions) {
            if (!r.first || r.second == 0) continue;
            void* dst = save ? (void*)(scratch + off) : r.first;
            const void* src = save ? r.first : (const void*)(scratch + off);
            CUDA_TRY(h, cudaMemcpyAsync(dst, src, r.second, cudaMemcpyDeviceToDevice, h->stream));
            off += r.second;
        }
        return RIFT_OK;
    };
    const int keepPersist = h->persistMax, keepMarch = h->marchMin, keepRows = h->marchRows;
    // candidates: persistent loop; per-step graph with the tile kernels; with
    // the march kernels on work items of 2, 1 and 4 tile rows
    constexpr int NC = RIFT_AUTOTUNE_CANDIDATES;
    const int persistOf[NC] = {h->gridPersist > 0 ? INT32_MAX : -1, 0, 0, 0, 0};
    const int marchOf[NC] = {INT32_MAX, INT32_MAX, 0, 0, 0};
    const int rowsOf[NC] = {keepRows, keepRows, 2, 1, 4};
    double best = INFINITY;
    int pick = 1;
    double ms3[NC] = {NAN, NAN, NAN, NAN, NAN};
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    rc = copyAll(true);
    if (!rc && (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess))
        rc = fail(h, RIFT_ERR_CUDA, "cudaEventCreate");
    for (int c = 0; c < NC && !rc; c++) {
        if (persistOf[c] < 0) continue;
        h->persistMax = persistOf[c];
        h->marchMin = marchOf[c];
        h->marchRows = rowsOf[c];
        destroyGraph(h);
        *h->hst = saved;
        h->hst->t_stop = INFINITY;
        h->hst->steps_done = 0;
        bool current = false;
        if ((rc = copyAll(false)) || (rc = pushState(h))) break;
        if (cudaEventRecord(e0, h->stream) != cudaSuccess) {
            rc = fail(h, RIFT_ERR_CUDA, "cudaEventRecord");
            break;
        }
        if ((rc = runSteps(h, probe_steps, &current))) break;
        cudaEventRecord(e1, h->stream);
        if ((rc = pullState(h))) break;
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        ms3[c] = ms / probe_steps;
        if (ms3[c] < best) {
            best = ms3[c];
            pick = c;
        }
    }
    // restore the state; keep the chosen schedule
    if (!rc) {
        *h->hst = saved;
        if ((rc = copyAll(false)) == RIFT_OK) rc = pushState(h);
    }
    h->persistMax = rc ? keepPersist : (pick == 0 ? INT32_MAX : 0);
    h->marchMin = rc ? keepMarch : marchOf[pick];
    h->marchRows = rc ? keepRows : rowsOf[pick];
    destroyGraph(h);
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    cudaFree(scratch);
    if (rc) return rc;
    if (choice) *choice = pick;
    if (ms_per_step)
        for (int c = 0; c < NC; c++) ms_per_step[c] = ms3[c];
    return RIFT_OK;
}

// ---------------------------------------------------------------- ensembles
struct rift_ensemble {
    std::vector<rift_handle*> m;
    std::vector<double> memberSec;  // last run: device time from its start to each member's end
    int64_t soloCells = 0;          // members with at least this many interior cells run on their own
    long long launches = 0;         // ensemble kernels launched (members run on their own count theirs)
    cudaStream_t stream = nullptr;
    Params* dP = nullptr;
    CUtensorMap* dMaps = nullptr;
    EnsDev* dE = nullptr;
    int grid = 0;
    long long steps = 0;
    std::string err;
};

namespace {
int efail(rift_ensemble* e, int code, const std::string& msg) {
    if (e) e->err = msg;
    return code;
}

// A member large enough to run on its own per-step graph (rift_ensemble_set_solo_cells).
bool isSolo(const rift_ensemble* e, const rift_handle* h) {
    return e->soloCells > 0 && (int64_t)(h->nx - 4) * (h->ny - 4) >= e->soloCells;
}
#define ENS_TRY(e, call)                                                                        \
    do {                                                                                        \
        cudaError_t e_ = (call);                                                                \
        if (e_ != cudaSuccess)                                                                  \
            return efail(e, e_ == cudaErrorMemoryAllocation ? RIFT_ERR_NOMEM : RIFT_ERR_CUDA,   \
                         std::string(#call) + ": " + cudaGetErrorString(e_));                   \
    } while (0)
}  // namespace

int rift_ensemble_create(rift_handle* const* members, int32_t n, rift_ensemble** out) {
    if (!members || !out || n < 1 || n > ENS_MAX) return RIFT_ERR_ARG;
    *out = nullptr;
    for (int k = 0; k < n; k++) {
        if (!members[k]) return RIFT_ERR_ARG;
        if (!members[k]->inited) return RIFT_ERR_STATE;
        if (members[k]->g.device != members[0]->g.device) return RIFT_ERR_ARG;
        // the ensemble kernel keeps the source ledger only
        if (members[k]->has(RIFT_F_CHECK_VOLUME)) return RIFT_ERR_UNSUPPORTED;
        for (int q = 0; q < k; q++)
            if (members[q] == members[k]) return RIFT_ERR_ARG;
    }
    rift_ensemble* e = new rift_ensemble();
    e->m.assign(members, members + n);
    *out = e;
    ENS_TRY(e, cudaSetDevice(members[0]->g.device));
    int coop = 0, sms = 0, occ = 0;
    cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, members[0]->g.device);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, members[0]->g.device);
    ENS_TRY(e, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_ensemble, NT, 0));
    if (!coop || occ < 1) return efail(e, RIFT_ERR_UNSUPPORTED, "no cooperative launch");
    e->grid = sms * occ;
    ENS_TRY(e, cudaStreamCreateWithFlags(&e->stream, cudaStreamNonBlocking));
    ENS_TRY(e, cudaMalloc(&e->dP, sizeof(Params) * n));
    ENS_TRY(e, cudaMalloc(&e->dMaps, sizeof(CUtensorMap) * 3 * n));
    ENS_TRY(e, cudaMalloc(&e->dE, sizeof(EnsDev)));
    return RIFT_OK;
}

int rift_ensemble_run(rift_ensemble* e, double t_stop, int32_t max_steps, double* t_out,
                      int32_t* steps_out) {
    if (!e || max_steps < 0) return RIFT_ERR_ARG;
    const int n = (int)e->m.size();
    std::vector<Params> P(n);
    std::vector<CUtensorMap> maps(3 * (size_t)n);
    std::vector<int> live(n, 0);
    int nAlive = 0;
    for (int k = 0; k < n; k++) {
        rift_handle* h = e->m[k];
        ENS_TRY(e, cudaStreamSynchronize(h->stream));
        // every entry point leaves the pinned mirror equal to the device state
        h->hst->t_stop = t_stop;
        h->hst->steps_done = 0;
        ENS_TRY(e, cudaMemcpyAsync(h->st, h->hst, sizeof(DevState), cudaMemcpyHostToDevice, e->stream));
        P[k] = makeParams(h);
        maps[3 * k] = h->tmA;
        maps[3 * k + 1] = h->tmB;
        maps[3 * k + 2] = h->tmE;
        live[k] = (h->hst->t < t_stop && max_steps > 0 && !isSolo(e, h)) ? 1 : 0;
        nAlive += live[k];
    }
    ENS_TRY(e, cudaMemcpyAsync(e->dP, P.data(), sizeof(Params) * n, cudaMemcpyHostToDevice, e->stream));
    ENS_TRY(e, cudaMemcpyAsync(e->dMaps, maps.data(), sizeof(CUtensorMap) * 3 * n,
                               cudaMemcpyHostToDevice, e->stream));
    ENS_TRY(e, cudaMemsetAsync(e->dE, 0, sizeof(EnsDev), e->stream));
    ENS_TRY(e, cudaMemcpyAsync(e->dE->live[0], live.data(), sizeof(int) * n, cudaMemcpyHostToDevice,
                               e->stream));
    ENS_TRY(e, cudaMemcpyAsync(&e->dE->nAlive[0], &nAlive, sizeof(int), cudaMemcpyHostToDevice,
                               e->stream));
    EnsArgs A{e->dP, e->dMaps, e->dE, n, max_steps};
    void* args[] = {(void*)&A};
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    ENS_TRY(e, cudaEventCreate(&ev0));
    ENS_TRY(e, cudaEventCreate(&ev1));
    ENS_TRY(e, cudaEventRecord(ev0, e->stream));
    if (nAlive > 0) {
        ENS_TRY(e, cudaLaunchCooperativeKernel((const void*)k_ensemble, dim3(e->grid), dim3(NT), args, 0,
                                               e->stream));
        e->launches += 1;
    }
    ENS_TRY(e, cudaEventRecord(ev1, e->stream));
    ENS_TRY(e, cudaStreamSynchronize(e->stream));
    {  // each member's completion on the device clock
        std::vector<unsigned long long> done(n, 0ull);
        unsigned long long t0 = 0ull;
        ENS_TRY(e, cudaMemcpy(done.data(), e->dE->tDone, sizeof(unsigned long long) * n,
                              cudaMemcpyDeviceToHost));
        ENS_TRY(e, cudaMemcpy(&t0, &e->dE->t0, sizeof(t0), cudaMemcpyDeviceToHost));
        e->memberSec.assign(n, 0.0);
        for (int k = 0; k < n; k++)
            if (live[k] && done[k] >= t0) e->memberSec[k] = 1e-9 * (double)(done[k] - t0);
    }
    // The large members, one after another on their own per-step graphs (the
    // column march on dense grids), smallest first; each one's completion is
    // the CUDA-event time since the ensemble kernel's start.
    {
        float kernelMs = 0.f;
        ENS_TRY(e, cudaEventElapsedTime(&kernelMs, ev0, ev1));
        double offset = 1e-3 * kernelMs;
        std::vector<int> solo;
        for (int k = 0; k < n; k++)
            if (isSolo(e, e->m[k]) && e->m[k]->hst->t < t_stop && max_steps > 0) solo.push_back(k);
        std::sort(solo.begin(), solo.end(), [&](int a, int b) {
            return (int64_t)e->m[a]->nx * e->m[a]->ny < (int64_t)e->m[b]->nx * e->m[b]->ny;
        });
        for (int k : solo) {
            rift_handle* h = e->m[k];
            double tk = 0.0, dtk = 0.0;
            int32_t dk = 0;
            ENS_TRY(e, cudaEventRecord(ev0, h->stream));
            int r = rift_run(h, max_steps, t_stop, &tk, &dtk, &dk);
            if (r) {
                cudaEventDestroy(ev0);
                cudaEventDestroy(ev1);
                return efail(e, r, "member " + std::to_string(k) + ": " + h->err);
            }
            ENS_TRY(e, cudaEventRecord(ev1, h->stream));
            ENS_TRY(e, cudaEventSynchronize(ev1));
            float ms = 0.f;
            ENS_TRY(e, cudaEventElapsedTime(&ms, ev0, ev1));
            offset += 1e-3 * ms;
            e->memberSec[k] = dk > 0 ? offset : 0.0;
        }
    }
    cudaEventDestroy(ev0);
    cudaEventDestroy(ev1);
    int rc = RIFT_OK;
    for (int k = 0; k < n; k++) {
        rift_handle* h = e->m[k];
        int r = pullState(h);
        if (r && !rc) {
            rc = r;
            e->err = "member " + std::to_string(k) + ": " + h->err;
        }
        if (t_out) t_out[k] = h->hst->t;
        if (steps_out) steps_out[k] = h->hst->steps_done;
        e->steps += h->hst->steps_done;
    }
    return rc;
}

int rift_ensemble_launch_count(rift_ensemble* e, int64_t* kernels) {
    if (!e || !kernels) return RIFT_ERR_ARG;
    long long n = e->launches;
    for (rift_handle* h : e->m) n += h->launches;
    *kernels = n;
    return RIFT_OK;
}

int rift_ensemble_set_solo_cells(rift_ensemble* e, int64_t min_cells) {
    if (!e || min_cells < 0) return RIFT_ERR_ARG;
    e->soloCells = min_cells;
    return RIFT_OK;
}

int rift_ensemble_member_times(rift_ensemble* e, double* seconds) {
    if (!e || !seconds) return RIFT_ERR_ARG;
    for (size_t k = 0; k < e->m.size(); k++)
        seconds[k] = k < e->memberSec.size() ? e->memberSec[k] : 0.0;
    return RIFT_OK;
}

const char* rift_ensemble_last_error(rift_ensemble* e) { return e ? e->err.c_str() : "null ensemble"; }

void rift_ensemble_destroy(rift_ensemble* e) {
    if (!e) return;
    if (e->stream) cudaStreamSynchronize(e->stream);
    if (e->dP) cudaFree(e->dP);
    if (e->dMaps) cudaFree(e->dMaps);
    if (e->dE) cudaFree(e->dE);
    if (e->stream) cudaStreamDestroy(e->stream);
    delete e;
}

const char* rift_last_error(rift_handle* h) { return h ? h->err.c_str() : "null handle"; }

void rift_destroy(rift_handle* h) {
    if (!h) return;
    destroyGraph(h);
    if (h->stream) cudaStreamSynchronize(h->stream);
    for (float* p : {h->A, h->B, h->D, h->E, h->nman, h->K, h->FA, h->FB, h->hmax, h->qmax, h->twet,
                     h->tpeak, h->tdry, h->mx, h->my, h->srcRate, h->serT, h->serR})
        if (p) cudaFree(p);
    for (int k = 0; k < 3; k++)
        for (int q = 0; q < 2; q++)
            if (h->maps[k][q]) cudaFree(h->maps[k][q]);
    for (void* p : {(void*)h->gbar, (void*)h->owner, (void*)h->tileFlag,
                    (void*)h->strips, (void*)h->stripFlag, (void*)h->wet, (void*)h->prevAct,
                    (void*)h->act, (void*)h->deact,
                    (void*)h->inact, (void*)h->srcIdx, (void*)h->srcTileStart,
                    (void*)h->srcTileList, (void*)h->st, (void*)h->volPartial, (void*)h->BrefD})
        if (p) cudaFree(p);
    if (h->hst) cudaFreeHost(h->hst);
    if (h->stage) cudaFreeHost(h->stage);
    if (h->stream) cudaStreamDestroy(h->stream);
    delete h;
}

}  // extern "C"

// ------------------------------------------------------------------------
// rift_volume_noalloc: the volume sum for callers that must not allocate.
//
// Some callers cannot call cudaMalloc: a coupled model (the 1D sewer/channel
// side of a 1D-2D coupling, which the reference's main.cc stubs out) that
// checks the 2D mass balance from inside its own time loop, with its device
// memory handed out by its own pool or arena, or while it records work into
// a stream it does not want synchronised.  cudaMalloc and cudaFree
// synchronise the whole device and draw on memory such a caller has already
// budgeted, so this entry point takes only the caller's buffers and keeps its
// scratch -- one compensated partial sum per grid row -- in a fixed array
// that lives in this library's device image on every GPU that loads it.
//
// Limits and sharing rules:
//  - at most RIFT_NOALLOC_MAX_ROWS grid rows (ghost rows included); larger
//    grids are rejected with RIFT_ERR_TOO_LARGE before anything is launched;
//  - the array is shared by every call in the process on that device and
//    keeps the last call's partial sums.  Each call writes every row partial
//    it later reads, so nothing needs clearing, but two calls that overlap on
//    the GPU (different streams, or different host threads) overwrite each
//    other's partials: the caller serialises them;
//  - the first call on a device looks up the array's device address
//    (cudaGetSymbolAddress) with that device current; make that first call
//    before recording any stream capture on the device.  The address is kept
//    per device together with the id of the context it was looked up in; a
//    call from another context (after cudaDeviceReset the device's primary
//    context is a new one, and the module may load at a new address) looks
//    it up again before launching.
namespace {

constexpr int kNoAllocMaxRows = RIFT_NOALLOC_MAX_ROWS;
static __device__ __align__(256) double g_noallocRowSums[2 * kNoAllocMaxRows];

constexpr int kMaxDevices = 64;
std::mutex g_noallocMutex;
double* g_noallocPtr[kMaxDevices] = {nullptr};
unsigned long long g_noallocCtx[kMaxDevices] = {0};

// Id of the calling thread's current context (cuCtxGetCurrent + cuCtxGetId,
// reached through the runtime's driver entry points); 0 when unavailable.
unsigned long long currentContextId() {
    using GetCur = CUresult (*)(CUcontext*);
    using GetId = CUresult (*)(CUcontext, unsigned long long*);
    static GetCur getCur = nullptr;
    static GetId getId = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess && q == cudaDriverEntryPointSuccess)
            getCur = reinterpret_cast<GetCur>(p);
        p = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess && q == cudaDriverEntryPointSuccess)
            getId = reinterpret_cast<GetId>(p);
    });
    CUcontext ctx = nullptr;
    unsigned long long id = 0;
    if (!getCur || !getId || getCur(&ctx) != CUDA_SUCCESS || !ctx || getId(ctx, &id) != CUDA_SUCCESS)
        return 0;
    return id;
}

// One warp per interior row: Neumaier sum of (h [+ F]) over the row's
// interior cells, lanes combined in lane order.
__global__ void k_volume_rows_noalloc(const float* __restrict__ h, const float* __restrict__ F,
                                      int nx, int ny, long long ld, double* rows) {
    const int lane = threadIdx.x & 31;
    const int j = 2 + (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    if (j > ny - 3) return;
    double s = 0.0, c = 0.0;
    for (int i = 2 + lane; i <= nx - 3; i += 32) {
        double v = (double)h[(size_t)j * ld + i];
        if (F) v += (double)F[(size_t)j * ld + i];
        double t = s + v;
        c += (fabs(s) >= fabs(v)) ? (s - t) + v : (v - t) + s;
        s = t;
    }
    double S = 0.0, C = 0.0;
    for (int l = 0; l < 32; l++) {
        double vs = __shfl_sync(0xffffffffu, s, l);
        double vc = __shfl_sync(0xffffffffu, c, l);
        double t = S + vs;
        C += (fabs(S) >= fabs(vs)) ? (S - t) + vs : (vs - t) + S;
        S = t;
        C += vc;
    }
    if (lane == 0) {
        rows[2 * j] = S;
        rows[2 * j + 1] = C;
    }
}

// Rows combined into the caller's output by one warp: lane l sums the
// contiguous block of rows [2 + l*chunk, 2 + (l+1)*chunk) in row order, then
// the 32 lane sums are combined in lane order, so the result does not depend
// on timing.
__global__ void k_volume_final_noalloc(const double* rows, int ny, double* out) {
    if (blockIdx.x != 0) return;
    const int lane = threadIdx.x & 31;
    const int nrows = ny - 4;
    const int chunk = (nrows + 31) / 32;
    const int j0 = 2 + lane * chunk;
    const int j1 = min(j0 + chunk, ny - 2);
    double s = 0.0, c = 0.0;
    for (int j = j0; j < j1; j++) {
        const double v = rows[2 * j];
        const double t = s + v;
        c += (fabs(s) >= fabs(v)) ? (s - t) + v : (v - t) + s;
        s = t;
        c += rows[2 * j + 1];
    }
    double S = 0.0, C = 0.0;
    for (int l = 0; l < 32; l++) {
        const double vs = __shfl_sync(0xffffffffu, s, l);
        const double vc = __shfl_sync(0xffffffffu, c, l);
        const double t = S + vs;
        C += (fabs(S) >= fabs(vs)) ? (S - t) + vs : (vs - t) + S;
        S = t;
        C += vc;
    }
    if (lane == 0) out[0] = S + C;
}

}  // namespace

extern "C" int rift_volume_noalloc(const float* depth, const float* infil, int32_t h_nx,
                                   int32_t h_ny, int64_t ld, double* volume_dev, void* stream) {
    if (!depth || !volume_dev || h_nx < 5 || h_ny < 5 || ld < h_nx) return RIFT_ERR_ARG;
    if (h_ny > kNoAllocMaxRows) return RIFT_ERR_TOO_LARGE;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return RIFT_ERR_CUDA;
    double* rows = nullptr;
    {
        const unsigned long long ctx = currentContextId();
        std::lock_guard<std::mutex> lock(g_noallocMutex);
        if (!g_noallocPtr[dev] || ctx == 0 || g_noallocCtx[dev] != ctx) {
            void* p = nullptr;
            if (cudaGetSymbolAddress(&p, g_noallocRowSums) != cudaSuccess || !p)
                return RIFT_ERR_CUDA;
            g_noallocPtr[dev] = static_cast<double*>(p);
            g_noallocCtx[dev] = ctx;
        }
        rows = g_noallocPtr[dev];
    }
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const int rowsInterior = h_ny - 4;
    const int threads = 256;
    const int blocks = (rowsInterior * 32 + threads - 1) / threads;
    k_volume_rows_noalloc<<<blocks, threads, 0, s>>>(depth, infil, h_nx, h_ny, (long long)ld, rows);
    k_volume_final_noalloc<<<1, 32, 0, s>>>(rows, h_ny, volume_dev);
    return cudaGetLastError() == cudaSuccess ? RIFT_OK : RIFT_ERR_CUDA;
}
