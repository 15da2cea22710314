// rift_kernels.cuh -- device kernels of the GB300 step.
//
// One step (the body of Simulator::RunSimulation, simulator.cu:773-853):
//   k_track   : re-wet inactive tiles under gridded rain / surge
//               (TrackRainfall_k / TrackSurge_k, grid.cu:1224-1276); only
//               when a gridded rain or surge series is on
//   k_grow    : start of step (stop test, uniform-source interpolation of
//               simulator.cu:500-538), then the 4-neighbour dilation of the
//               wet tiles and the on-device compaction of the active /
//               inactive / deactivated tile lists and of the march strips
//               (Grow, grid.cu:1188-1322), chunked over the CTAs
//               (rift_grow.cuh)
//   k_speed_dt: per-tile local-speed maxima on U^n (the speed output of the
//               first ComputeFluxes, grid.cu:813-838), the max over every
//               tile (stale speeds of inactive tiles included) and, in
//               the last CTA, dt and t (Simulator::ComputeTimestep,
//               simulator.cu:540-566); also re-syncs the stage buffer of
//               tiles that just went inactive
//   k_stage<1>: fused flux + sources + friction + RK stage 1 + ghost cells
//               (ComputeFluxes_k + Integrate_1_k + ApplyBoundaries)
//   k_stage<2>: fused flux + sources + RK stage 2 + ghost cells + outputs +
//               tile wet flags + tile speeds
//               (ComputeFluxes_k + Integrate_2_k + ApplyBoundaries)
//   k_commit  : Euler mode only, copies the single stage's result back
// The tile kernels are persistent over the compacted list of active tiles.
// Each CTA stages a tile's halo'd block of (h, hu, hv) and of the four
// face-elevation offsets in shared memory with TMA (cp.async.bulk.tensor on
// 3-D maps over the stacked fields), double-buffered: the next tile's block
// is in flight while the current one is computed.
#pragma once
#include <cuda.h>
#include <cstdint>

#include "rift_device.cuh"

namespace rift {

constexpr int TW = 16;          // tile width  (BLOCK_COLS, grid.cu:19)
constexpr int TH = 14;          // tile height (BLOCK_ROWS, grid.cu:18)
constexpr int SW = TW + 4;      // staged block width  (2-cell halo)
constexpr int SH = TH + 4;      // staged block height
constexpr int NT = 256;         // threads per tile CTA
constexpr int STRIP_TX = 7;     // march work item: 7 x 2 tiles = 112 x 28 cells
constexpr int STRIP_TY = 2;
constexpr int MAX_SERIES = 4096;

// flag bits, identical to include/rift_gb300.h
constexpr uint32_t F_RAIN_U = 1u << 0, F_RAIN_G = 1u << 1, F_DRAIN_U = 1u << 2,
                   F_DRAIN_G = 1u << 3, F_INFIL = 1u << 4, F_SURGE = 1u << 5,
                   F_EULER = 1u << 6, F_SAVE_MAX = 1u << 7, F_SAVE_ARR = 1u << 8,
                   F_TILE_ACC = 1u << 9, F_POINT = 1u << 10, F_H_INIT = 1u << 11,
                   F_CHECKVOL = 1u << 12;

// Flags that change the per-cell update; a kernel instantiated with a fixed
// set FIX (!= 0) reads its flags from FIX instead of the run's flags: the
// engine picks such an instantiation only when the run's flags, masked with
// CELL_FLAGS, equal FIX (and point sources are present iff FIX has F_POINT).
constexpr uint32_t CELL_FLAGS = F_RAIN_U | F_RAIN_G | F_DRAIN_U | F_DRAIN_G | F_INFIL | F_SURGE |
                                F_EULER | F_SAVE_MAX | F_SAVE_ARR | F_TILE_ACC | F_POINT |
                                F_CHECKVOL;
// the fixed sets with march instantiations: uniform rain; infiltration with
// a point hydrograph; gridded rain with a uniform drain (all with tile
// acceleration)
constexpr uint32_t FIX_RAIN = F_RAIN_U | F_TILE_ACC;
constexpr uint32_t FIX_INFIL_SRC = F_INFIL | F_POINT | F_TILE_ACC;
constexpr uint32_t FIX_RAINMAP_DRAIN = F_RAIN_G | F_DRAIN_U | F_TILE_ACC;

template <uint32_t FIX>
__device__ __forceinline__ uint32_t cellFlags(uint32_t runFlags) {
    return FIX ? FIX : runFlags;
}

constexpr int ERR_TMA_TIMEOUT = 1;
constexpr int ERR_BARRIER_TIMEOUT = 2;
constexpr int ERR_TILE_TABLE = 4;  // persistent loop: tile table and scan disagree

// Device-resident scalars of the run (one per handle).
struct DevState {
    double t;          // simulated time, FP64 accumulator
    double dt;         // dt of the current step (after k_speed_dt)
    double dt_old;     // dt of the previous step (stage-1 source clamps)
    double t_stop;     // kernels idle once t >= t_stop at step start
    double map_t0[3];  // map interval [t0, t1) when the factor follows t
    double map_t1[3];
    int map_timed[3];
    float rain_rate;   // uniform rates, m/s, as the reference's float rates
    float drain_rate;
    float ser_interp[3];  // Source::interpolated_rate state, divided in place each step
    float factor[3];      // map interpolation factors
    unsigned max_bits[2];
    unsigned ticket;
    int nActive, nDeact, nInact;
    int nStrips;       // strips of the march kernels holding an active tile
    int stop;
    int persistExit;   // the persistent kernel left because the active set grew
    int tableSteps;    // steps the persistent loop ran from its tile table (no grow)
    int steps_done;
    unsigned long long activeCells;  // interior cells of active tiles, summed over steps
    int appendCnt[4];                // grow: list counters (zero between steps)
    unsigned long long appendCells;
    unsigned growTicket;
    unsigned staleBits[2];           // ensemble: stale speed maxima of inactive tiles
    double v_added;    // volume (depth x cells) the sources added since init
    double rain_sum[2];  // interior sums of the two rain maps (volume ledger)
    // check_volume ledger since init (depth x cells), LED_* order; ledPend:
    // stage-1 edge inflow rates summed before the step's dt is known
    double led[5];
    double ledPend;
    int error;
    int err_info;
};

struct Params {
    int nx, ny, nBX, nBY, gridSize;
    int pitch, rows;   // floats per row, rows per field plane
    float dx, dy, inv_dx, inv_dy, kappa, psiDtheta, nodata;
    double dxd, dyd, kappad, courant;
    float courantScale;  // 1/courant when courant is a power of two, else 0
    float kappaf;        // (float)kappa
    bool squareCells;    // dx == dy
    uint32_t flags;
    float* A;          // [3][rows][pitch]  U^n / U^{n+1}: h, hu, hv
    float* B;          // [3][rows][pitch]  U*
    float* D;          // [3][rows][pitch]  stage-1 flux divergence + bed source (march)
    int planeSize;     // rows * pitch
    const float* E;    // [4][rows][pitch]  eW, eE, eS, eN
    const float* nman; // [rows][pitch]
    const float* K;
    float* FA;         // F^n / F^{n+1}
    float* FB;         // F*
    float* hmax;
    float* qmax;
    float* twet;
    float* tpeak;
    float* tdry;
    const float* map0[3];
    const float* map1[3];
    int mapMode[3];    // 0 none, 1 hold, 2 interpolate
    uint8_t* wet;
    uint8_t* prevAct;  // active set of the current step (after the grow)
    int* act;          // active tiles that hold interior cells
    int* deact;
    int* inact;
    int* strips;       // march work items (strip ids) holding an active tile
    uint8_t* stripFlag;
    int nSX, nSY;      // strip grid (strips of 7 x 2 tiles)
    int marchMin;      // active strips from which the march kernels run
    int persistMax;    // the persistent step kernel runs while active tiles <= this
    struct GridBar* gbar;            // grid barrier of the persistent kernel
    int* owner;        // [gridSize] tile -> CTA of the persistent loop's tile table, or -1
    int* tileFlag;     // [gridSize] persistent loop: last step whose stage 1 the tile finished
    float* mx;
    float* my;
    const int* srcIdx;      // flat h-grid indices j*nx+i
    float* srcRate;         // per source, m/s
    const int* srcTileStart;  // CSR by tile: [gridSize+1]
    const int* srcTileList;   // source ordinals sorted by tile
    int nsrc;
    const float* serT;      // [3][MAX_SERIES]
    const float* serR;
    int serN[3];
    DevState* st;
};

// Offset of cell (j, i) of plane f: 32-bit arithmetic (the host keeps every
// field below 2^32 elements), zero-extended.
__device__ __forceinline__ size_t cidx(const Params& P, int f, int j, int i) {
    return (size_t)(((unsigned)f * (unsigned)P.rows + (unsigned)j) * (unsigned)P.pitch +
                    (unsigned)i);
}

// ---------------------------------------------------------------- PTX glue
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count)
                 : "memory");
}
__device__ __forceinline__ void fence_mbar_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void fence_proxy_async() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
                 "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        " selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* tm, uint64_t* bar, int x,
                                            int y, int z) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
        " [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(smem_u32(dst)),
        "l"((uint64_t)tm), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
        : "memory");
}
__device__ __forceinline__ void prefetch_tmap(const CUtensorMap* tm) {
    asm volatile("prefetch.tensormap [%0];" ::"l"((uint64_t)tm) : "memory");
}

// Bounded wait on an mbarrier phase; false after the spin limit (the caller
// records the error and leaves the tile loop).
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity) {
    for (int it = 0; it < (1 << 20); ++it)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}

// ------------------------------------------------------------- shared block
struct __align__(128) TileBuf {
    float in[3][SH][SW];    // h, hu, hv     (TMA destination, 4320 B)
    float pad0[8];          // keeps `e` 128-byte aligned
    float e[4][SH][SW];     // eW, eE, eS, eN (TMA destination, 5760 B)
};
static_assert(offsetof(TileBuf, e) % 128 == 0, "TMA destination alignment");
static_assert(sizeof(TileBuf) % 128 == 0, "TMA destination alignment");

struct __align__(128) StageSmem {
    TileBuf buf[2];
    struct {  // x and y reconstructions side by side: built in one phase
        struct {
            float P[3][TH][TW + 2];
            float M[3][TH][TW + 2];
        } x;
        struct {
            float P[3][TH + 2][TW];
            float M[3][TH + 2][TW];
        } y;
    } rec;
    float FX[3][TH][TW + 1];
    float FY[3][TH + 1][TW];
    float red[2][NT / 32];
    uint64_t bar[2];
};
constexpr uint32_t BYTES_IN = 3 * SH * SW * 4;
constexpr uint32_t BYTES_E = 4 * SH * SW * 4;

__device__ __forceinline__ void tileOrigin(const Params& P, int tile, int& bX, int& bY, int& i0,
                                           int& j0) {
    bX = tile % P.nBX;
    bY = tile / P.nBX;
    i0 = bX * TW + 2;
    j0 = bY * TH + 2;
}

// Gridded map value at a cell (hold or InterpGrid_k semantics, grid.cu:292-311).
// Map value from the cell's entries x0, x1 of the two maps (InterpGrid_k,
// grid.cu:292-311): hold mode reads x0; interpolation skips nodata entries.
__device__ __forceinline__ float mapFrom(const Params& P, int which, float x0, float x1,
                                         float factor) {
    // a series that was never set reads as its GridSeries fill value:
    // nodata for surge (allow_no_data), 0 otherwise
    if (P.mapMode[which] == 0) return which == 2 ? P.nodata : 0.f;
    if (P.mapMode[which] != 2) return x0;
    float nd = P.nodata;
    if (x1 == nd && x0 == nd) return nd;
    if (x1 == nd) return x0;
    if (x0 == nd) return x1;
    return factor * (x1 - x0) + x0;
}

__device__ __forceinline__ float mapValue(const Params& P, int which, size_t c, float factor) {
    if (P.mapMode[which] == 0) return which == 2 ? P.nodata : 0.f;
    const float x0 = P.map0[which][c];
    const float x1 = P.mapMode[which] == 2 ? P.map1[which][c] : 0.f;
    return mapFrom(P, which, x0, x1, factor);
}

// The cell's two rain-map entries, for a caller that loads them ahead of the
// update (cellSources with RAINPRE reads them from pre[6], pre[7]).
__device__ __forceinline__ void loadRainMaps(const Params& P, size_t c, float* q) {
    q[0] = P.mapMode[0] != 0 ? P.map0[0][c] : 0.f;
    q[1] = P.mapMode[0] == 2 ? P.map1[0][c] : 0.f;
}

// L1 prefetch of the gridded maps a cell update will read (rain, drain,
// surge), issued a row or a group of rows ahead.
__device__ __forceinline__ void prefetch_l1(const void* p) {
    asm volatile("prefetch.global.L1 [%0];" ::"l"(p));
}
__device__ __forceinline__ void prefetchMaps(const Params& P, uint32_t fl, size_t c) {
    const uint32_t use[3] = {F_RAIN_G, F_DRAIN_G, F_SURGE};
#pragma unroll
    for (int w = 0; w < 3; w++) {
        if (!(fl & use[w]) || P.mapMode[w] == 0) continue;
        prefetch_l1(P.map0[w] + c);
        if (P.mapMode[w] == 2) prefetch_l1(P.map1[w] + c);
    }
}

// Block-wide max (non-negative values); result valid in thread 0.
// Both speed maxima (valid in thread 0) and the OR of a vote (every thread)
// with one CTA barrier: the barrier of __syncthreads_or also orders the
// per-warp maxima written to red.
__device__ __forceinline__ bool blockMax2Or(float vx, float vy, bool vote, float (*red)[NT / 32],
                                            float& mx, float& my) {
    for (int o = 16; o > 0; o >>= 1) {
        vx = fmaxf(vx, __shfl_xor_sync(0xffffffffu, vx, o));
        vy = fmaxf(vy, __shfl_xor_sync(0xffffffffu, vy, o));
    }
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    if (l == 0) {
        red[0][w] = vx;
        red[1][w] = vy;
    }
    const bool any = __syncthreads_or(vote) != 0;
    mx = my = 0.f;
    if (threadIdx.x == 0)
        for (int k = 0; k < (int)(blockDim.x >> 5); k++) {
            mx = fmaxf(mx, red[0][k]);
            my = fmaxf(my, red[1][k]);
        }
    return any;
}

__device__ __forceinline__ float blockMax(float v, float* red) {
    for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
    int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    if (l == 0) red[w] = v;
    __syncthreads();
    float r = 0.f;
    if (threadIdx.x == 0)
        for (int k = 0; k < (int)(blockDim.x >> 5); k++) r = fmaxf(r, red[k]);
    return r;
}


// ---------------------------------------------------------------- ledger
// Volume ledger terms of a check_volume run (the reference's check_volume
// switch, grid.cu:23), each already weighted by its share of the step: an
// RK2 step moves the cell by half of each stage's rates times dt (Euler: all
// of the single stage), plus the clamps applied to the state.  With V the
// interior sum of h:
//   V(t) - V(0) = added - drained - infiltrated - clamped + surge + boundary
enum { LED_DRAIN = 0, LED_INFIL = 1, LED_CLAMP = 2, LED_SURGE = 3, LED_BOUND = 4, LED_N = 5 };

struct Led {
    float v[LED_N];
};

__device__ __forceinline__ void ledZero(Led& L) {
#pragma unroll
    for (int k = 0; k < LED_N; k++) L.v[k] = 0.f;
}

// Warp sums of the threads' terms into dst[0..LED_N) (FP64, one atomic per
// non-zero term and warp); every lane of the warp calls it.  Zeroes L.
__device__ __forceinline__ void flushLed(Led& L, double* dst) {
#pragma unroll
    for (int k = 0; k < LED_N; k++) {
        float v = L.v[k];
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if ((threadIdx.x & 31) == 0 && v != 0.f) atomicAdd(&dst[k], (double)v);
        L.v[k] = 0.f;
    }
}

// Inflow rate through the domain edge of interior cell (j, i) (m/s of
// depth): the mass flux of its west / south face at the first interior
// column / row, minus that of its east / north face at the last.
__device__ __forceinline__ float edgeInflow(const Params& P, int j, int i, float fW, float fE,
                                            float fS, float fN) {
    float r = 0.f;
    if (i == 2) r += fW * P.inv_dx;
    if (i == P.nx - 3) r -= fE * P.inv_dx;
    if (j == 2) r += fS * P.inv_dy;
    if (j == P.ny - 3) r -= fN * P.inv_dy;
    return r;
}

// ComputeTimestep's arithmetic (simulator.cu:540-566) from the maxima of
// the tile speeds: dt with the reference's rounding points (fmaxf on the
// scaled maxima, FP64 division), t += dt, and the step's entry in the
// volume ledger.
// maxx, maxy: float speed maxima.  When the Courant number is a power of
// two, float(max / courant) is the exact float product with 1/courant, and
// with square cells min(dx / fx, dx / fy) = dx / max(fx, fy) (rounded
// division is monotone in the divisor): one FP64 division instead of four,
// with the same result.
// dt of a step (Simulator::ComputeTimestep's arithmetic, simulator.cu:540-566)
// from the float speed maxima; t == 0 gives the reference's first-step dt.
__device__ __forceinline__ double stepDtAt(const Params& P, double t, float maxx, float maxy) {
    double dt;
    if (P.courantScale > 0.f) {
        const float fx = fmaxf(maxx * P.courantScale, P.kappaf);
        const float fy = fmaxf(maxy * P.courantScale, P.kappaf);
        if (P.squareCells) {
            const float f = fmaxf(fx, fy);
            dt = P.dxd / (double)f;
        } else {
            const double cx = P.dxd / (double)fx, cy = P.dyd / (double)fy;
            dt = cx < cy ? cx : cy;
        }
    } else {
        double cx = P.dxd / (double)fmaxf((float)((double)maxx / P.courant), P.kappaf);
        double cy = P.dyd / (double)fmaxf((float)((double)maxy / P.courant), P.kappaf);
        dt = cx < cy ? cx : cy;
    }
    if ((__double_as_longlong(t) << 1) == 0) dt = (double)0.000001f;  // t == 0.0
    return dt;
}
__device__ __forceinline__ double stepDtAt(const Params& P, double t, double maxx, double maxy) {
    return stepDtAt(P, t, (float)maxx, (float)maxy);
}

__device__ __forceinline__ double stepDt(const Params& P, const DevState* st, double maxx,
                                         double maxy) {
    return stepDtAt(P, st->t, maxx, maxy);
}

// The step's dt into the device state: dt_old, dt, t += dt, and the step's
// entry in the volume ledger (both RK stages, or the Euler stage, apply each
// source rate of this step for dt -- uniform rain on every interior cell,
// the point sources, the gridded rain map at this step's factor).
__device__ __forceinline__ void publishDt(const Params& P, DevState* st, double dt) {
    st->dt_old = st->dt;
    st->dt = dt;
    st->t = st->t + dt;
    double add = 0.0;
    if (P.flags & F_RAIN_U) add += (double)st->rain_rate * (double)(P.nx - 4) * (P.ny - 4);
    if (P.serN[2] > 0) {
        // every source holds the same float rate: the sequential FP64 sum of
        // nsrc copies is exact (under 2^29 terms), so it equals the product
        add += (double)P.nsrc * (double)P.srcRate[0];
    } else {
        for (int k = 0; k < P.nsrc; k++) add += (double)P.srcRate[k];
    }
    if ((P.flags & F_RAIN_G) && P.mapMode[0] != 0) {
        add += st->rain_sum[0];
        if (P.mapMode[0] == 2) add += (double)st->factor[0] * (st->rain_sum[1] - st->rain_sum[0]);
    }
    st->v_added += add * dt;
    // stage-1 edge inflow of a flux pass that ran before dt (the column
    // march).  Atomic: in the persistent loop other CTAs add their terms to
    // the same total while this runs.
    if ((P.flags & F_CHECKVOL) && st->ledPend != 0.0) {
        atomicAdd(&st->led[LED_BOUND], ((P.flags & F_EULER) ? 1.0 : 0.5) * dt * st->ledPend);
        st->ledPend = 0.0;
    }
}

__device__ __forceinline__ void computeDt(const Params& P, DevState* st, double maxx, double maxy) {
    publishDt(P, st, stepDt(P, st, maxx, maxy));
}

// Simulator::ComputeTimestep (simulator.cu:540-566) on device: thread 0 of
// each CTA adds the CTA's maxima of the new tile speeds (tmx, tmy) with one
// atomic; the last CTA to finish turns them, with the stale maxima the grow
// folded in, into dt with the reference's rounding points and advances t.
__device__ __forceinline__ void finishDt(const Params& P, float tmx, float tmy, bool* last) {
    DevState* st = P.st;
    const int tid = threadIdx.x;
    if (tid == 0) {
        atomicMax(&st->max_bits[0], __float_as_uint(tmx));
        atomicMax(&st->max_bits[1], __float_as_uint(tmy));
        __threadfence();
        *last = (atomicAdd(&st->ticket, 1u) == gridDim.x - 1);
    }
    __syncthreads();
    if (*last && tid == 0) {
        __threadfence();
        // speeds are non-negative: their bit patterns order like the values
        const unsigned bx = max(atomicOr(&st->max_bits[0], 0u), atomicExch(&st->staleBits[0], 0u));
        const unsigned by = max(atomicOr(&st->max_bits[1], 0u), atomicExch(&st->staleBits[1], 0u));
        computeDt(P, st, (double)__uint_as_float(bx), (double)__uint_as_float(by));
    }
}

// Re-sync U* with U^n on the tiles that went inactive this step (interior
// cells and the ghost cells they own): the stage kernels read U* in the halo
// of active tiles, and for an inactive tile U* = U^n.
__device__ __forceinline__ void resyncTile(const Params& P, int tile) {
    const int tid = threadIdx.x;
    const int bX = tile % P.nBX, bY = tile / P.nBX;
    for (int q = tid; q < TW * TH; q += blockDim.x) {
        const int i = bX * TW + q % TW + 2, j = bY * TH + q / TW + 2;
        auto cp = [&](int jj, int ii) {
            for (int f = 0; f < 3; f++) P.B[cidx(P, f, jj, ii)] = P.A[cidx(P, f, jj, ii)];
        };
        if (i < P.nx && j < P.ny) cp(j, i);
        if (i >= 2 && j >= 2 && i <= P.nx - 3 && j <= P.ny - 3) {
            if (i == 2) {
                cp(j, 0);
                cp(j, 1);
            }
            if (i == P.nx - 3) {
                cp(j, P.nx - 2);
                cp(j, P.nx - 1);
            }
            if (j == 2) {
                cp(0, i);
                cp(1, i);
            }
            if (j == P.ny - 3) {
                cp(P.ny - 2, i);
                cp(P.ny - 1, i);
            }
        }
    }
}

__device__ __forceinline__ void resyncDeactivated(const Params& P, int nDe) {
    for (int k = blockIdx.x; k < nDe; k += gridDim.x) resyncTile(P, P.deact[k]);
}

__device__ __forceinline__ void resyncDeactivated(const Params& P) {
    resyncDeactivated(P, P.st->nDeact);
}

// Schedule: the march kernels (strips of 7 x 2 tiles) run when at least
// P.marchMin strips hold active tiles; below that the per-tile kernels, whose
// finer work items keep a sparse or small grid spread over the GPU.  Both
// are launched every step; the one not chosen returns at once.
__device__ __forceinline__ bool useMarch(const Params& P) { return P.st->nStrips >= P.marchMin; }

// Thread 0 issues the TMA loads of one tile's staged block into `b`.
__device__ __forceinline__ void issueTile(TileBuf& b, uint64_t* bar, const CUtensorMap* tmIn,
                                          const CUtensorMap* tmE, const Params& P, int tile) {
    int bX = tile % P.nBX, bY = tile / P.nBX;
    fence_proxy_async();
    mbar_expect_tx(bar, BYTES_IN + BYTES_E);
    tma_load_3d(&b.in[0][0][0], tmIn, bar, bX * TW, bY * TH, 0);
    tma_load_3d(&b.e[0][0][0], tmE, bar, bX * TW, bY * TH, 0);
}

// Barriers of the tile buffers and the tensor-map prefetch (once per kernel).
__device__ __forceinline__ void tileInit(StageSmem& S, const CUtensorMap* tmIn,
                                         const CUtensorMap* tmE) {
    if (threadIdx.x == 0) {
        prefetch_tmap(tmIn);
        prefetch_tmap(tmE);
        mbar_init(&S.bar[0], 1);
        mbar_init(&S.bar[1], 1);
        fence_mbar_init();
    }
}

// Start of a tile loop: the CTA's first tile into buffer 0.
__device__ __forceinline__ void tileFirst(StageSmem& S, const CUtensorMap* tmIn,
                                          const CUtensorMap* tmE, const Params& P, int nAct) {
    if (threadIdx.x == 0 && (int)blockIdx.x < nAct)
        issueTile(S.buf[0], &S.bar[0], tmIn, tmE, P, P.act[blockIdx.x]);
    __syncthreads();
}

// Wait for the current tile (buffer b), then prefetch the CTA's next tile
// into the other buffer, whose readers all passed the barrier.
__device__ __forceinline__ bool tileAcquire(StageSmem& S, const CUtensorMap* tmIn,
                                            const CUtensorMap* tmE, const Params& P, int b,
                                            uint32_t* ph, int kNext, int nAct) {
    bool ok = mbar_wait_bounded(&S.bar[b], ph[b]);
    if (!__syncthreads_and(ok)) {
        // error path: one more bounded wait for the copy still in flight, so
        // that no TMA write lands after the CTA has left
        mbar_wait_bounded(&S.bar[b], ph[b]);
        return false;
    }
    ph[b] ^= 1u;
    if (threadIdx.x == 0 && kNext < nAct)
        issueTile(S.buf[b ^ 1], &S.bar[b ^ 1], tmIn, tmE, P, P.act[kNext]);
    return ok;
}

// ---------------------------------------------------------------- sources
// Uniform sources of Simulator::UpdateSource (simulator.cu:500-538): each CSV
// series is interpolated at float(t) (source.cc:65-73) and its float state
// divided in place every step.  IEEE float ops (_rn intrinsics) keep the host's
// arithmetic (no contraction, exact division).
// Called by one whole warp: the lanes test the intervals [T[i], T[i+1]) in
// parallel; the last interval holding t wins, as in the sequential loop.  A
// lane loads both ends of its interval and both rates at once, so a series of
// up to 33 points costs one round trip to memory.
__device__ __forceinline__ float seriesInterp(const float* T, const float* R, int n, float t,
                                              float cur) {
    const int lane = threadIdx.x & 31;
    bool found = false;
    float T0f = 0.f, T1f = 0.f, R0f = 0.f, R1f = 0.f;
    for (int base = 0; base + 1 < n; base += 32) {
        const int i = base + lane;
        float T0 = 0.f, T1 = 0.f, R0 = 0.f, R1 = 0.f;
        if (i + 1 < n) {
            T0 = T[i];
            T1 = T[i + 1];
            R0 = R[i];
            R1 = R[i + 1];
        }
        const bool m = (i + 1 < n) && t >= T0 && t < T1;
        const unsigned bal = __ballot_sync(0xffffffffu, m);
        if (bal) {  // warp-uniform
            const int src = 31 - __clz(bal);
            found = true;
            T0f = __shfl_sync(0xffffffffu, T0, src);
            T1f = __shfl_sync(0xffffffffu, T1, src);
            R0f = __shfl_sync(0xffffffffu, R0, src);
            R1f = __shfl_sync(0xffffffffu, R1, src);
        }
    }
    if (found) {
        float num = __fsub_rn(R1f, R0f);
        float den = __fsub_rn(T1f, T0f);
        cur = __fadd_rn(R0f, __fmul_rn(__fdiv_rn(num, den), __fsub_rn(t, T0f)));
    }
    return cur;
}

// Start of a step, part 1, by one thread: reset of the step's reductions and
// the map factors that follow t.  Runs before the step's grow.
__device__ __forceinline__ void beginStepResets(DevState* s) {
    s->stop = 0;
    s->steps_done += 1;
    s->max_bits[0] = 0u;
    s->max_bits[1] = 0u;
    s->ticket = 0u;
    // map factor following t (GridSeries::update computes it at the end
    // of the previous step from the same t, GridSeries.cu:398)
    for (int w = 0; w < 3; w++)
        if (s->map_timed[w])
            s->factor[w] = (float)((s->t - s->map_t0[w]) / (s->map_t1[w] - s->map_t0[w]));
}

// The step's uniform source rates at float(t) from the series state (one
// whole warp; writes nothing).  interp[w] gets the new series state.  The
// FP64 conversion of the hydrograph runs in one lane.
struct StepRates {
    float rainU, drainU, srcR;
    float interp[3];
};

// From the previous step's rates and series state `prev` (the rates of a
// series that is not set stay as they are).
__device__ StepRates stepRatesFrom(const Params& P, const StepRates& prev, double t) {
    const int lane = threadIdx.x & 31;
    const float tf = (float)t;
    StepRates q = prev;
    q.srcR = 0.f;
    if (P.serN[2] > 0) {  // hydrograph, cfs -> m^3/s -> m/s per source cell
        float v = seriesInterp(P.serT + 2 * MAX_SERIES, P.serR + 2 * MAX_SERIES, P.serN[2], tf,
                               q.interp[2]);
        v = __fdiv_rn(v, 35.3147f);
        float r = 0.f;
        if (lane == 0) r = (float)((double)v / P.dxd / P.dyd / (double)P.nsrc);
        q.srcR = __shfl_sync(0xffffffffu, r, 0);
        q.interp[2] = v;
    }
    if (P.serN[0] > 0) {  // hyetograph, mm/hr -> m/s
        float v = seriesInterp(P.serT, P.serR, P.serN[0], tf, q.interp[0]);
        v = __fdiv_rn(v, 3600.f * 1000.f);
        q.interp[0] = v;
        q.rainU = v;
    }
    if (P.serN[1] > 0) {  // drain, mm/hr -> m/s
        float v = seriesInterp(P.serT + MAX_SERIES, P.serR + MAX_SERIES, P.serN[1], tf,
                               q.interp[1]);
        v = __fdiv_rn(v, 3600.f * 1000.f);
        q.interp[1] = v;
        q.drainU = v;
    }
    return q;
}

// From the device state.
__device__ StepRates stepRates(const Params& P, const DevState* s, double t) {
    StepRates prev;
    prev.rainU = s->rain_rate;
    prev.drainU = s->drain_rate;
    prev.srcR = 0.f;
    for (int w = 0; w < 3; w++) prev.interp[w] = s->ser_interp[w];
    return stepRatesFrom(P, prev, t);
}

// The rates and the series state into the device state (one whole warp).
__device__ void writeRates(const Params& P, DevState* s, const StepRates& q) {
    const int lane = threadIdx.x & 31;
    if (P.serN[2] > 0)
        for (int k = lane; k < P.nsrc; k += 32) P.srcRate[k] = q.srcR;
    if (lane == 0) {
        for (int w = 0; w < 3; w++)
            if (P.serN[w] > 0) s->ser_interp[w] = q.interp[w];
        if (P.serN[0] > 0) s->rain_rate = q.rainU;
        if (P.serN[1] > 0) s->drain_rate = q.drainU;
    }
    __syncwarp();
}

// Start of a step, part 2, by one whole warp: the uniform source rates into
// the device state.  Only the cell updates and the volume ledger read them,
// so it may run any time between the previous step's stage 2 and this
// step's stage 1.
__device__ void beginStepRates(const Params& P, DevState* s) {
    writeRates(P, s, stepRates(P, s, s->t));
}

// Start of a step, by one whole warp: both parts.
__device__ void beginStep(const Params& P, DevState* s) {
    beginStepRates(P, s);
    if ((threadIdx.x & 31) == 0) beginStepResets(s);
}

// ---------------------------------------------------------------- k_track
// TrackRainfall_k / TrackSurge_k over the tiles that were inactive after the
// previous Grow.  The rows come from blockY * BLOCK_COLS (16), not 14, as in
// the reference.
// Factors of the gridded rain and surge maps at the start of the step (the
// tracking runs before the step's own factor update).
__device__ __forceinline__ void trackFactors(const Params& P, float& fac0, float& fac2) {
    const DevState* s = P.st;
    fac0 = s->factor[0];
    fac2 = s->factor[2];
    if (s->map_timed[0]) fac0 = (float)((s->t - s->map_t0[0]) / (s->map_t1[0] - s->map_t0[0]));
    if (s->map_timed[2]) fac2 = (float)((s->t - s->map_t0[2]) / (s->map_t1[2] - s->map_t0[2]));
}

// One inactive tile: re-wet it when a cell of the rows the reference checks
// has gridded rain above epsilon or a positive surge depth.
__device__ __forceinline__ void trackTile(const Params& P, int tile, float fac0, float fac2) {
    if (P.wet[tile]) return;  // uniform across the block
    const int bX = tile % P.nBX, bY = tile / P.nBX;
    bool hit = false;
    if (threadIdx.x < TW * TH) {
        int tx = threadIdx.x % TW, ty = threadIdx.x / TW;
        int i = bX * TW + tx + 2, j = bY * TW + ty + 2;
        if (i >= 2 && j >= 2 && i <= P.nx - 3 && j <= P.ny - 3) {
            size_t c = cidx(P, 0, j, i);
            if (P.flags & F_RAIN_G) {
                float v = mapValue(P, 0, c, fac0);
                if (v > kEps) hit = true;
            }
            if (P.flags & F_SURGE) {
                float v = mapValue(P, 2, c, fac2);
                if (v != P.nodata && v > 0.f) hit = true;
            }
        }
    }
    if (__syncthreads_or(hit) && threadIdx.x == 0) P.wet[tile] = 1;
}

__device__ __forceinline__ void trackTiles(const Params& P) {
    const int n = P.st->nInact;
    float fac0, fac2;
    trackFactors(P, fac0, fac2);
    if (n < 0) {  // no list (a step of the persistent loop's tile table): scan
        for (int b = blockIdx.x + 1; b < P.gridSize; b += gridDim.x)
            if (!P.prevAct[b]) trackTile(P, b, fac0, fac2);
        return;
    }
    for (int k = blockIdx.x; k < n; k += gridDim.x) trackTile(P, P.inact[k], fac0, fac2);
}

__global__ void __launch_bounds__(NT) k_track(Params P) {
    if (P.st->t >= P.st->t_stop) return;
    trackTiles(P);
}

// ------------------------------------------------------------- k_speed_dt
// Per-tile speed maxima of U^n over the scheduled active tiles (what the
// first ComputeFluxes of a step writes to mx/my, grid.cu:813-838); the max
// over all tiles, stale entries of inactive tiles included; in the last
// CTA, dt with the reference's rounding points (fmaxf of the scaled maxima,
// FP64 division) and t += dt.  Also re-syncs U* with U^n on tiles that went
// inactive this step (interior cells and the ghost cells they own).
// Local-speed maxima of one staged tile (the speed output of the first
// ComputeFluxes, grid.cu:813-838): depth and normal-momentum reconstruction,
// the east and north face of every interior cell.  Valid in thread 0.
__device__ __forceinline__ void tileSpeeds(StageSmem& S, const TileBuf& T, const Params& P, int i0,
                                           int j0, float& mxv, float& myv) {
    const int tid = threadIdx.x;
    const float kappa = P.kappa;
    float spx = 0.f, spy = 0.f;
    // x: depth + hu reconstruction of cells i0-1..i0+16 on the tile rows
    if (tid < TH * (TW + 2)) {
        int r = tid / (TW + 2), c = tid % (TW + 2);
        int sr = r + 2, sc = c + 1;
        RecN R = constructN(T.in[0][sr][sc], T.in[1][sr][sc], T.in[0][sr][sc + 1],
                            T.in[1][sr][sc + 1], T.in[0][sr][sc - 1], T.in[1][sr][sc - 1],
                            T.e[0][sr][sc], T.e[1][sr][sc], T.e[1][sr][sc] - T.e[0][sr][sc + 1],
                            T.e[1][sr][sc - 1] - T.e[0][sr][sc]);
        S.rec.x.P[0][r][c] = R.hP;
        S.rec.x.P[1][r][c] = R.qP;
        S.rec.x.M[0][r][c] = R.hM;
        S.rec.x.M[1][r][c] = R.qM;
    }
    __syncthreads();
    if (tid < TH * TW) {  // east face of tile cell (ty, tx)
        int ty = tid / TW, tx = tid % TW;
        if (i0 + tx <= P.nx - 3 && j0 + ty <= P.ny - 3)
            spx = faceSpeed(S.rec.x.P[0][ty][tx + 1], S.rec.x.P[1][ty][tx + 1],
                            S.rec.x.M[0][ty][tx + 2], S.rec.x.M[1][ty][tx + 2], kappa);
    }
    __syncthreads();
    // y: depth + hv reconstruction of rows j0..j0+14
    if (tid < (TH + 2) * TW) {
        int r = tid / TW, c = tid % TW;
        int sr = r + 1, sc = c + 2;
        RecN R = constructN(T.in[0][sr][sc], T.in[2][sr][sc], T.in[0][sr + 1][sc],
                            T.in[2][sr + 1][sc], T.in[0][sr - 1][sc], T.in[2][sr - 1][sc],
                            T.e[2][sr][sc], T.e[3][sr][sc], T.e[3][sr][sc] - T.e[2][sr + 1][sc],
                            T.e[3][sr - 1][sc] - T.e[2][sr][sc]);
        S.rec.y.P[0][r][c] = R.hP;
        S.rec.y.P[1][r][c] = R.qP;
        S.rec.y.M[0][r][c] = R.hM;
        S.rec.y.M[1][r][c] = R.qM;
    }
    __syncthreads();
    if (tid < TH * TW) {  // north face of tile cell (ty, tx)
        int ty = tid / TW, tx = tid % TW;
        if (i0 + tx <= P.nx - 3 && j0 + ty <= P.ny - 3)
            spy = faceSpeed(S.rec.y.P[0][ty + 1][tx], S.rec.y.P[1][ty + 1][tx],
                            S.rec.y.M[0][ty + 2][tx], S.rec.y.M[1][ty + 2][tx], kappa);
    }
    mxv = blockMax(spx, S.red[0]);
    myv = blockMax(spy, S.red[1]);
}

// Tile loop of the speed pass over the scheduled active tiles; thread 0
// keeps the CTA's maximum of the new tile speeds.  False after a TMA
// timeout (error recorded).
__device__ bool speedTiles(StageSmem& S, const CUtensorMap* tmA, const CUtensorMap* tmE,
                           const Params& P, int nAct, uint32_t* ph, float& tmx, float& tmy) {
    DevState* st = P.st;
    const int tid = threadIdx.x;
    tileFirst(S, tmA, tmE, P, nAct);
    int bsel = 0;
    for (int k = blockIdx.x; k < nAct; k += gridDim.x, bsel ^= 1) {
        const int tile = P.act[k];
        int bX, bY, i0, j0;
        tileOrigin(P, tile, bX, bY, i0, j0);
        if (!tileAcquire(S, tmA, tmE, P, bsel, ph, k + gridDim.x, nAct)) {
            if (tid == 0) atomicOr(&st->error, ERR_TMA_TIMEOUT);
            return false;
        }
        const TileBuf& T = S.buf[bsel];
        float mxv, myv;
        tileSpeeds(S, T, P, i0, j0, mxv, myv);
        if (tid == 0) {
            P.mx[tile] = mxv;
            P.my[tile] = myv;
            tmx = fmaxf(tmx, mxv);
            tmy = fmaxf(tmy, myv);
        }
        __syncthreads();
    }
    return true;
}

__global__ void __launch_bounds__(NT) k_speed_dt(const __grid_constant__ CUtensorMap tmA,
                                                 const __grid_constant__ CUtensorMap tmE, Params P) {
    __shared__ StageSmem S;
    __shared__ bool last;
    if (P.st->stop || useMarch(P)) return;
    tileInit(S, &tmA, &tmE);
    uint32_t ph[2] = {0u, 0u};
    float tmx = 0.f, tmy = 0.f;
    if (!speedTiles(S, &tmA, &tmE, P, P.st->nActive, ph, tmx, tmy)) return;
    __syncthreads();
    finishDt(P, tmx, tmy, &last);
    resyncDeactivated(P);
}

// ---------------------------------------------------------------- k_stage
// Ghost cells owned by interior cell (j, i): critical-depth outflow
// (ApplyBoundariesX_k: clamped at epsilon; ApplyBoundariesY_k: not).
// The ghost's reference elevation is that of the interior cell it copies,
// so its depth is the critical depth itself.
__device__ __forceinline__ void writeGhosts(const Params& P, float* U, int j, int i, float h,
                                            float hu, float hv) {
    auto put = [&](int jj, int ii, float gh) {
        U[cidx(P, 0, jj, ii)] = gh;
        U[cidx(P, 1, jj, ii)] = hu;
        U[cidx(P, 2, jj, ii)] = hv;
    };
    if (i == 2 || i == P.nx - 3) {
        float HL = criticalDepth(hu, h);
        HL = (HL > kEps) ? HL : 0.f;
        if (i == 2) {
            put(j, 0, HL);
            put(j, 1, HL);
        }
        if (i == P.nx - 3) {
            put(j, P.nx - 2, HL);
            put(j, P.nx - 1, HL);
        }
    }
    if (j == 2 || j == P.ny - 3) {
        float HB = criticalDepth(hv, h);
        if (j == 2) {
            put(0, i, HB);
            put(1, i, HB);
        }
        if (j == P.ny - 3) {
            put(P.ny - 2, i, HB);
            put(P.ny - 1, i, HB);
        }
    }
}

// Step-wide constants of a stage kernel.
struct StageConsts {
    float kappa, dtNew, dtSrc, invDtSrc, rainU, drainU, fac0, fac1, fac2;
    float wRate;   // ledger weight of this stage's rates: dt/2 (RK2) or dt (Euler)
    float wHalf;   // 1/2 (RK2) or 1 (Euler)
    float srcR;  // the hydrograph's rate per source cell (every source holds it)
    double tNew;
    uint32_t fl;
    bool euler;
    float* Uout;
    const float* Fin;
    float* Fout;
};

template <int STAGE>
__device__ __forceinline__ StageConsts stageConsts(const Params& P) {
    const DevState* st = P.st;
    StageConsts C;
    C.kappa = P.kappa;
    C.fl = P.flags;
    C.euler = (P.flags & F_EULER) != 0;
    C.dtNew = (float)st->dt;
    // source clamps use the dt passed to ComputeFluxes: the previous dt in
    // stage 1 (simulator.cu:786-792), the new one in stage 2
    C.dtSrc = (STAGE == 1) ? (float)st->dt_old : C.dtNew;
    C.invDtSrc = 1.f / C.dtSrc;
    C.tNew = st->t;
    C.rainU = st->rain_rate;
    C.drainU = st->drain_rate;
    C.fac0 = st->factor[0];
    C.fac1 = st->factor[1];
    C.fac2 = st->factor[2];
    C.srcR = (P.serN[2] > 0 && P.nsrc > 0) ? P.srcRate[0] : 0.f;
    C.Uout = (STAGE == 1) ? P.B : P.A;
    C.Fin = (STAGE == 1) ? P.FA : P.FB;
    C.Fout = (STAGE == 1) ? P.FB : P.FA;
    C.wHalf = C.euler ? 1.f : 0.5f;
    C.wRate = C.wHalf * C.dtNew;
    return C;
}

// stageConsts by thread 0, shared with the CTA (the FP64 loads and
// conversions once per CTA, not per thread).  Every thread of the CTA calls it.
template <int STAGE>
__device__ __forceinline__ StageConsts blockConsts(const Params& P) {
    __shared__ StageConsts sc;
    if (threadIdx.x == 0) sc = stageConsts<STAGE>(P);
    __syncthreads();
    return sc;
}

// stageConsts with the step's dt, previous dt and t given by the caller
// (a caller that computed dt itself before the device state holds it).
template <int STAGE>
__device__ __forceinline__ StageConsts stageConstsAt(const Params& P, double dtNew, double dtOld,
                                                     double tNew) {
    StageConsts C = stageConsts<STAGE>(P);
    C.dtNew = (float)dtNew;
    C.dtSrc = (STAGE == 1) ? (float)dtOld : C.dtNew;
    C.invDtSrc = 1.f / C.dtSrc;
    C.tNew = tNew;
    C.wRate = C.wHalf * C.dtNew;
    return C;
}

// Sources, friction, the RK stage, outputs and ghost cells of interior cell
// (j, i) of `tile`, given its flux divergence (dh, dhu, dhv) and its staged
// state and face offsets.  Returns the cell's vote for the tile wet flag.
// pre: the cell's own inputs loaded ahead of use -- stage 1: Manning n;
// stage 2: U^n (h, hu, hv); with PREF also pre[3] = F entering the stage,
// pre[4] = K, pre[5] = F^n (stage 2), else those are read here.
// Bed-slope source of the momentum equations (grid.cu:701,751-752).
__device__ __forceinline__ float bedSourceX(const Params& P, float hC, float eW, float eE) {
    return -kG * hC * ((eE - eW) * P.inv_dx);
}
__device__ __forceinline__ float bedSourceY(const Params& P, float hC, float eS, float eN) {
    return -kG * hC * ((eN - eS) * P.inv_dy);
}

// The per-cell update is split at dt: cellSources is everything that does
// not need the step's dt (for stage 1: the bed slope, the mass sources with
// their clamps at the previous dt, infiltration, Manning's G), cellFinish the
// rest.  cellUpdate runs both; the persistent loop runs cellSources before
// its dt barrier.
struct CellSrc {
    float dh, dhu, dhv;  // divergence + sources
    float hc;            // depth clamped at epsilon (grid.cu:748-749)
    float Fc, dF;        // infiltration: F entering the stage, rate
    float rainG;         // gridded rain at the cell
    float G;             // stage 1: semi-implicit Manning coefficient
    float drained;       // drain rate withdrawn (uniform + gridded, after the cap)
    bool srcCell;        // the cell holds a point source
};

// BED: add the bed-slope source here (false: the caller's dhu, dhv hold it).
// RAINPRE: the cell's rain-map entries were loaded ahead into pre[6], pre[7].
template <int STAGE, bool PREF = false, bool BED = true, uint32_t FIX = 0, bool RAINPRE = false>
__device__ __forceinline__ CellSrc cellSources(const Params& P, const StageConsts& C, int tile,
                                               int j, int i, float dh, float dhu, float dhv,
                                               float hC, float hu0, float hv0, float eW, float eE,
                                               float eS, float eN, const float* pre) {
    const uint32_t fl = cellFlags<FIX>(C.fl);
    const size_t c = cidx(P, 0, j, i);
    const float S1 = BED ? bedSourceX(P, hC, eW, eE) : 0.f;
    const float S2 = BED ? bedSourceY(P, hC, eS, eN) : 0.f;
    // mass sources, grid.cu:763-807
    float S0 = 0.f;
    if (fl & F_RAIN_U) S0 += C.rainU;
    float rainG = 0.f;
    if (fl & F_RAIN_G) {
        rainG = RAINPRE ? mapFrom(P, 0, pre[6], pre[7], C.fac0) : mapValue(P, 0, c, C.fac0);
        S0 += rainG;
    }
    const float cap = hC * C.invDtSrc;
    float drained = 0.f;
    if (fl & F_DRAIN_U) {
        const float d = (C.drainU > cap) ? cap : C.drainU;
        S0 -= d;
        drained += d;
    }
    if (fl & F_DRAIN_G) {
        float d = mapValue(P, 1, c, C.fac1);
        d = (d > cap) ? cap : d;
        S0 -= d;
        drained += d;
    }
    bool srcCell = false;
    if ((FIX == 0 || (FIX & F_POINT)) && P.nsrc > 0) {
        const int flat = j * P.nx + i;
        for (int q = P.srcTileStart[tile]; q < P.srcTileStart[tile + 1]; q++) {
            int sidx = P.srcTileList[q];
            if (P.srcIdx[sidx] == flat) {
                S0 += P.serN[2] > 0 ? C.srcR : P.srcRate[sidx];
                srcCell = true;
            }
        }
    }
    float dF = 0.f, Fc = 0.f;
    if (fl & F_INFIL) {
        Fc = PREF ? pre[3] : C.Fin[c];
        dF = greenAmpt(PREF ? pre[4] : P.K[c], Fc, P.psiDtheta, C.dtSrc, hC);
        S0 -= dF;
    }
    dh += S0;
    if (BED) {
        dhu += S1;
        dhv += S2;
    }
    CellSrc r;
    r.dh = dh;
    r.dhu = dhu;
    r.dhv = dhv;
    r.hc = (hC > kEps) ? hC : 0.f;  // grid.cu:748-749
    r.Fc = Fc;
    r.dF = dF;
    r.rainG = rainG;
    r.drained = drained;
    r.srcCell = srcCell;
    r.G = STAGE == 1 ? manningG(pre[0], hu0, hv0, hC, C.kappa) : 0.f;
    return r;
}

// The RK stage-1 combination of Integrate_1_k (grid.cu:856-922) from a
// cell's sources: the surge condition, the explicit depth update, the
// semi-implicit Manning division of the momenta and the epsilon clamp.
// Shared by the stage-1 pass and by the stage-2 march that rebuilds U* from
// U^n and the stored divergence, so both give the same bits.
template <uint32_t FIX = 0>
__device__ __forceinline__ void rk1Core(const Params& P, const StageConsts& C, size_t c,
                                        const CellSrc& src, float hC, float hu0, float hv0, Led* L,
                                        float& hN, float& huN, float& hvN) {
    const uint32_t fl = cellFlags<FIX>(C.fl);
    const float dtNew = C.dtNew, hc = src.hc;
    float dh = src.dh;
    if (fl & F_SURGE) {
        float sg = mapValue(P, 2, c, C.fac2);
        if (sg != P.nodata && sg > 0.f) {
            const float d0 = dh;
            dh = (sg - (hc + dh * dtNew)) / dtNew;
            if (L) L->v[LED_SURGE] += C.wRate * (dh - d0);
        }
    }
    hN = hc + dh * dtNew;
    const float den = 1.f / (1.f - dtNew * src.G);
    huN = (hu0 + src.dhu * dtNew) * den;
    hvN = (hv0 + src.dhv * dtNew) * den;
    if (L) L->v[LED_CLAMP] += C.wHalf * ((hC - hc) + ((hN > kEps) ? 0.f : hN));
    hN = (hN > kEps) ? hN : 0.f;
}

// edge: the work item holds a cell next to the ghost band (i or j at 2 or
// at n - 3); false skips the ghost tests for the items inside.
// L (check_volume runs, else null): the cell's ledger terms are added to it.
template <int STAGE, bool PREF = false, uint32_t FIX = 0>
__device__ __forceinline__ bool cellFinish(const Params& P, const StageConsts& C, int j, int i,
                                           const CellSrc& src, float hC, float hu0, float hv0,
                                           const float* pre, bool edge, Led* L = nullptr) {
    const uint32_t fl = cellFlags<FIX>(C.fl);
    const bool euler = FIX ? (FIX & F_EULER) != 0 : C.euler;
    const size_t c = cidx(P, 0, j, i);
    float dh = src.dh;
    const float dhu = src.dhu, dhv = src.dhv, hc = src.hc, Fc = src.Fc, dF = src.dF;
    const float rainG = src.rainG;
    const bool srcCell = src.srcCell;
    const float dtNew = C.dtNew;
    float hN, huN, hvN;
    bool wetCell = false;
    if (STAGE == 1) {
        // Integrate_1_k (grid.cu:856-922)
        rk1Core<FIX>(P, C, c, src, hC, hu0, hv0, L, hN, huN, hvN);
        if (fl & F_INFIL) C.Fout[c] = Fc + dF * dtNew;
        if (euler) {
            // Euler-mode outputs and wet flags (grid.cu:926-1023)
            const float uC = huN * velFactor(hN, C.kappa), vC = hvN * velFactor(hN, C.kappa);
            if (fl & F_SAVE_MAX) {
                float hm = P.hmax[c];
                if (hN > hm) P.tpeak[c] = (float)C.tNew;
                if (hN > 0.0762f) P.tdry[c] = (float)C.tNew;
                P.hmax[c] = fmaxf(hm, hN);
                P.qmax[c] = fmaxf(P.qmax[c], hN * sqrtf(vC * vC + uC * uC));
            }
            if (fl & F_SAVE_ARR) {
                if (P.twet[c] < 0.f && hN > kEps) P.twet[c] = (float)C.tNew;
            }
            wetCell = (hN > kEps) || srcCell || ((fl & F_RAIN_U) && C.rainU > 0.f) ||
                      ((fl & F_RAIN_G) && rainG > 0.f);
            if (fl & F_SURGE) {
                float sg = mapValue(P, 2, c, C.fac2);
                if (sg != P.nodata && sg > 0.f) wetCell = true;
            }
        }
    } else {
        // Integrate_2_k (grid.cu:1043-1171)
        const float hOld = pre[0];
        const float hOc = (hOld > kEps) ? hOld : 0.f;
        hN = 0.5f * (hOc + hc + dh * dtNew);
        huN = 0.5f * (pre[1] + hu0 + dhu * dtNew);
        hvN = 0.5f * (pre[2] + hv0 + dhv * dtNew);
        if (L) L->v[LED_CLAMP] += 0.5f * ((hOld - hOc) + (hC - hc)) + ((hN > kEps) ? 0.f : hN);
        hN = (hN > kEps) ? hN : 0.f;
        if (fl & F_INFIL) C.Fout[c] = 0.5f * ((PREF ? pre[5] : P.FA[c]) + Fc + dF * dtNew);
        if (fl & F_SAVE_MAX) {
            const float uC = huN * velFactor(hN, C.kappa);
            const float vC = hvN * velFactor(hN, C.kappa);
            P.hmax[c] = fmaxf(P.hmax[c], hN);
            P.qmax[c] = fmaxf(P.qmax[c], hN * sqrtf(vC * vC + uC * uC));
        }
        if (fl & F_SAVE_ARR) {
            if (P.twet[c] < 0.f && hN > kEps) P.twet[c] = (float)C.tNew;
        }
        wetCell = (hN > kEps) || srcCell || ((fl & F_RAIN_U) && C.rainU > 0.f) ||
                  ((fl & F_RAIN_G) && rainG > 0.f);
    }
    if (L) {
        L->v[LED_DRAIN] += C.wRate * src.drained;
        L->v[LED_INFIL] += C.wRate * dF;
    }
    C.Uout[cidx(P, 0, j, i)] = hN;
    C.Uout[cidx(P, 1, j, i)] = huN;
    C.Uout[cidx(P, 2, j, i)] = hvN;
    if (edge) writeGhosts(P, C.Uout, j, i, hN, huN, hvN);
    return wetCell;
}

template <int STAGE, bool PREF = false, bool BED = true, uint32_t FIX = 0, bool RAINPRE = false>
__device__ __forceinline__ bool cellUpdate(const Params& P, const StageConsts& C, int tile, int j,
                                           int i, float dh, float dhu, float dhv, float hC,
                                           float hu0, float hv0, float eW, float eE, float eS,
                                           float eN, const float* pre, bool edge = true,
                                           Led* L = nullptr) {
    const CellSrc src = cellSources<STAGE, PREF, BED, FIX, RAINPRE>(P, C, tile, j, i, dh, dhu, dhv,
                                                                    hC, hu0, hv0, eW, eE, eS, eN,
                                                                    pre);
    return cellFinish<STAGE, PREF, FIX>(P, C, j, i, src, hC, hu0, hv0, pre, edge, L);
}


// Flux divergence of every interior cell of a staged tile (the ComputeFluxes_k
// sweeps, grid.cu:659-746): x reconstruction of cells i0-1 .. i0+16 on the
// 14 tile rows and the 17 x faces, then the y reconstruction of rows
// j0-1 .. j0+14 and the 15 y faces.  Thread tid < 224 gets the divergence of
// cell (tid / 16, tid % 16); with SPEEDS, spx / spy get the local speed of
// the east / north face of that cell (0 outside the interior).
// bin (check_volume runs, else null): the cell's inflow rate through the
// domain edge (edgeInflow), 0 away from it.
template <bool SPEEDS>
__device__ __forceinline__ void tileFluxDiv(StageSmem& S, const TileBuf& T, const Params& P, int i0,
                                            int j0, float& dh, float& dhu, float& dhv, float& spx,
                                            float& spy, float* bin = nullptr) {
    // Two phases of the whole CTA: every thread builds one x and one y
    // reconstruction, then one x and one y face flux (the two directions are
    // independent until the divergence, so each thread has two chains in
    // flight and the tile needs two barriers, not four).
    const int tid = threadIdx.x;
    const float kappa = P.kappa;
    if (tid < TH * (TW + 2)) {
        int r = tid / (TW + 2), c = tid % (TW + 2);
        int sr = r + 2, sc = c + 1;
        Rec R = construct(T.in[0][sr][sc], T.in[1][sr][sc], T.in[2][sr][sc], T.in[0][sr][sc + 1],
                          T.in[1][sr][sc + 1], T.in[2][sr][sc + 1], T.in[0][sr][sc - 1],
                          T.in[1][sr][sc - 1], T.in[2][sr][sc - 1], T.e[0][sr][sc], T.e[1][sr][sc],
                          T.e[1][sr][sc] - T.e[0][sr][sc + 1], T.e[1][sr][sc - 1] - T.e[0][sr][sc]);
        S.rec.x.P[0][r][c] = R.hP;
        S.rec.x.P[1][r][c] = R.uP;
        S.rec.x.P[2][r][c] = R.vP;
        S.rec.x.M[0][r][c] = R.hM;
        S.rec.x.M[1][r][c] = R.uM;
        S.rec.x.M[2][r][c] = R.vM;
    }
    if (tid < (TH + 2) * TW) {
        int r = tid / TW, c = tid % TW;
        int sr = r + 1, sc = c + 2;
        Rec R = construct(T.in[0][sr][sc], T.in[1][sr][sc], T.in[2][sr][sc], T.in[0][sr + 1][sc],
                          T.in[1][sr + 1][sc], T.in[2][sr + 1][sc], T.in[0][sr - 1][sc],
                          T.in[1][sr - 1][sc], T.in[2][sr - 1][sc], T.e[2][sr][sc], T.e[3][sr][sc],
                          T.e[3][sr][sc] - T.e[2][sr + 1][sc], T.e[3][sr - 1][sc] - T.e[2][sr][sc]);
        S.rec.y.P[0][r][c] = R.hP;
        S.rec.y.P[1][r][c] = R.uP;
        S.rec.y.P[2][r][c] = R.vP;
        S.rec.y.M[0][r][c] = R.hM;
        S.rec.y.M[1][r][c] = R.uM;
        S.rec.y.M[2][r][c] = R.vM;
    }
    __syncthreads();
    spx = 0.f;
    spy = 0.f;
    // x face f lies between reconstructed cells f and f+1: the east face of
    // tile column f-1
    if (tid < TH * (TW + 1)) {
        int r = tid / (TW + 1), f = tid % (TW + 1);
        float fx[3];
        float sp = faceFlux<0>(S.rec.x.P[0][r][f], S.rec.x.P[1][r][f], S.rec.x.P[2][r][f],
                               S.rec.x.M[0][r][f + 1], S.rec.x.M[1][r][f + 1],
                               S.rec.x.M[2][r][f + 1], kappa, fx);
        S.FX[0][r][f] = fx[0];
        S.FX[1][r][f] = fx[1];
        S.FX[2][r][f] = fx[2];
        if (SPEEDS && f >= 1 && i0 + f - 1 <= P.nx - 3 && j0 + r <= P.ny - 3) spx = sp;
    }
    // y face r is the north face of tile row r-1
    if (tid < (TH + 1) * TW) {
        int r = tid / TW, c = tid % TW;
        float fy[3];
        float sp = faceFlux<1>(S.rec.y.P[0][r][c], S.rec.y.P[1][r][c], S.rec.y.P[2][r][c],
                               S.rec.y.M[0][r + 1][c], S.rec.y.M[1][r + 1][c],
                               S.rec.y.M[2][r + 1][c], kappa, fy);
        S.FY[0][r][c] = fy[0];
        S.FY[1][r][c] = fy[1];
        S.FY[2][r][c] = fy[2];
        if (SPEEDS && r >= 1 && i0 + c <= P.nx - 3 && j0 + r - 1 <= P.ny - 3) spy = sp;
    }
    __syncthreads();
    const int tx = tid % TW, ty = tid / TW;
    dh = dhu = dhv = 0.f;
    if (tid < TH * TW) {
        dh = -(S.FX[0][ty][tx + 1] - S.FX[0][ty][tx]) * P.inv_dx;
        dhu = -(S.FX[1][ty][tx + 1] - S.FX[1][ty][tx]) * P.inv_dx;
        dhv = -(S.FX[2][ty][tx + 1] - S.FX[2][ty][tx]) * P.inv_dx;
        dh += -(S.FY[0][ty + 1][tx] - S.FY[0][ty][tx]) * P.inv_dy;
        dhu += -(S.FY[1][ty + 1][tx] - S.FY[1][ty][tx]) * P.inv_dy;
        dhv += -(S.FY[2][ty + 1][tx] - S.FY[2][ty][tx]) * P.inv_dy;
    }
    if (bin) {
        *bin = 0.f;
        const int i = i0 + tx, j = j0 + ty;
        if (tid < TH * TW && i <= P.nx - 3 && j <= P.ny - 3)
            *bin = edgeInflow(P, j, i, S.FX[0][ty][tx], S.FX[0][ty][tx + 1], S.FY[0][ty][tx],
                              S.FY[0][ty + 1][tx]);
    }
}

// The cell's own global inputs for cellUpdate<STAGE, true> (pre[0..5]),
// loaded while the staged block is in flight.
template <int STAGE>
__device__ __forceinline__ void tilePrefetch(const Params& P, const StageConsts& C, int i0, int j0,
                                             float (&pre)[6]) {
    const int tid = threadIdx.x;
    for (int q = 0; q < 6; q++) pre[q] = 0.f;
    const int ip = i0 + tid % TW, jp = j0 + tid / TW;
    if (tid < TH * TW && ip <= P.nx - 3 && jp <= P.ny - 3) {
        const size_t c = cidx(P, 0, jp, ip);
        if (STAGE == 1) {
            pre[0] = P.nman[c];
        } else {
            pre[0] = P.A[c];
            pre[1] = P.A[cidx(P, 1, jp, ip)];
            pre[2] = P.A[cidx(P, 2, jp, ip)];
        }
        if (C.fl & F_INFIL) {
            pre[3] = C.Fin[c];
            pre[4] = P.K[c];
            if (STAGE == 2) pre[5] = P.FA[c];
        }
    }
}

// Update of the interior cell of thread tid < 224 of a staged tile from its
// divergence; returns its wet vote.
template <int STAGE, uint32_t FIX = 0>
__device__ __forceinline__ bool tileCellUpdate(const Params& P, const StageConsts& C,
                                               const TileBuf& T, int tile, int i0, int j0, float dh,
                                               float dhu, float dhv, const float (&pre)[6],
                                               Led* L = nullptr) {
    const int tid = threadIdx.x;
    const int tx = tid % TW, ty = tid / TW;
    const int i = i0 + tx, j = j0 + ty;
    if (tid >= TH * TW || i > P.nx - 3 || j > P.ny - 3) return false;
    const int r = ty + 2, c = tx + 2;
    // tile-uniform: does the tile reach the first or last interior row/column?
    const bool edge = i0 == 2 || j0 == 2 || i0 + TW - 1 >= P.nx - 3 || j0 + TH - 1 >= P.ny - 3;
    return cellUpdate<STAGE, true, true, FIX>(P, C, tile, j, i, dh, dhu, dhv, T.in[0][r][c], T.in[1][r][c],
                                   T.in[2][r][c], T.e[0][r][c], T.e[1][r][c], T.e[2][r][c],
                                   T.e[3][r][c], pre, edge, L);
}

// tileCellUpdate in its two halves (see cellSources / cellFinish).
template <int STAGE, uint32_t FIX = 0>
__device__ __forceinline__ CellSrc tileCellSources(const Params& P, const StageConsts& C,
                                                   const TileBuf& T, int tile, int i0, int j0,
                                                   float dh, float dhu, float dhv,
                                                   const float (&pre)[6]) {
    const int tid = threadIdx.x;
    const int tx = tid % TW, ty = tid / TW;
    const int i = i0 + tx, j = j0 + ty;
    CellSrc r{};
    if (tid >= TH * TW || i > P.nx - 3 || j > P.ny - 3) return r;
    const int rr = ty + 2, cc = tx + 2;
    return cellSources<STAGE, true, true, FIX>(P, C, tile, j, i, dh, dhu, dhv, T.in[0][rr][cc],
                                    T.in[1][rr][cc], T.in[2][rr][cc], T.e[0][rr][cc],
                                    T.e[1][rr][cc], T.e[2][rr][cc], T.e[3][rr][cc], pre);
}

template <int STAGE, uint32_t FIX = 0>
__device__ __forceinline__ bool tileCellFinish(const Params& P, const StageConsts& C,
                                               const TileBuf& T, int i0, int j0,
                                               const CellSrc& src, const float (&pre)[6],
                                               Led* L = nullptr) {
    const int tid = threadIdx.x;
    const int tx = tid % TW, ty = tid / TW;
    const int i = i0 + tx, j = j0 + ty;
    if (tid >= TH * TW || i > P.nx - 3 || j > P.ny - 3) return false;
    const int rr = ty + 2, cc = tx + 2;
    const bool edge = i0 == 2 || j0 == 2 || i0 + TW - 1 >= P.nx - 3 || j0 + TH - 1 >= P.ny - 3;
    return cellFinish<STAGE, true, FIX>(P, C, j, i, src, T.in[0][rr][cc], T.in[1][rr][cc],
                                   T.in[2][rr][cc], pre, edge, L);
}

// Tile flags (stage 2, or stage 1 in Euler mode) and stage-2 tile speeds.
template <int STAGE>
__device__ __forceinline__ bool tileFlags(const Params& P, const StageConsts& C, StageSmem& S,
                                          int tile, bool wetCell, float spx, float spy) {
    bool wetTile = false;
    if (STAGE == 2) {  // wet vote and both speed maxima with one barrier
        float mxv, myv;
        const bool any = blockMax2Or(spx, spy, wetCell, S.red, mxv, myv);
        wetTile = (!(C.fl & F_TILE_ACC)) || any;
        if (threadIdx.x == 0) {
            P.wet[tile] = (uint8_t)wetTile;
            P.mx[tile] = mxv;
            P.my[tile] = myv;
        }
    } else if (C.euler) {
        bool any = __syncthreads_or(wetCell);
        wetTile = (!(C.fl & F_TILE_ACC)) || any;
        if (threadIdx.x == 0) P.wet[tile] = (uint8_t)wetTile;
    }
    return wetTile;  // the tile's new wet flag (stage 2 or Euler), else false
}

// STAGE 1: reads U^n (A) -> writes U* (B), F* (FB).
// STAGE 2: reads U* (B) with halo and U^n (A) at the cell -> writes U^{n+1}
//          (A), F^{n+1} (FA), outputs, tile wet flags and tile speeds.
// Tile loop of RK stage STAGE over the scheduled active tiles.  False after
// a TMA timeout (error recorded).
template <int STAGE, uint32_t FIX = 0>
__device__ bool stageTiles(StageSmem& S, const CUtensorMap* tmIn, const CUtensorMap* tmE,
                           const Params& P, int nAct, uint32_t* ph,
                           const StageConsts* given = nullptr) {
    const int tid = threadIdx.x;
    tileFirst(S, tmIn, tmE, P, nAct);
    const StageConsts C = given ? *given : blockConsts<STAGE>(P);
    const bool led = (cellFlags<FIX>(C.fl) & F_CHECKVOL) != 0;
    Led L;
    ledZero(L);
    int bsel = 0;
    for (int k = blockIdx.x; k < nAct; k += gridDim.x, bsel ^= 1) {
        const int tile = P.act[k];
        int bX, bY, i0, j0;
        tileOrigin(P, tile, bX, bY, i0, j0);
        float pre[6];
        tilePrefetch<STAGE>(P, C, i0, j0, pre);
        if (!tileAcquire(S, tmIn, tmE, P, bsel, ph, k + gridDim.x, nAct)) {
            if (tid == 0) atomicOr(&P.st->error, ERR_TMA_TIMEOUT);
            return false;
        }
        const TileBuf& T = S.buf[bsel];
        float dh, dhu, dhv, spx, spy, bin = 0.f;
        tileFluxDiv<STAGE == 2>(S, T, P, i0, j0, dh, dhu, dhv, spx, spy, led ? &bin : nullptr);
        L.v[LED_BOUND] += C.wRate * bin;
        const bool wetCell =
            tileCellUpdate<STAGE, FIX>(P, C, T, tile, i0, j0, dh, dhu, dhv, pre, led ? &L : nullptr);
        tileFlags<STAGE>(P, C, S, tile, wetCell, spx, spy);
        __syncthreads();
    }
    if (led) flushLed(L, P.st->led);
    return true;
}

template <int STAGE>
__global__ void __launch_bounds__(NT) k_stage(const __grid_constant__ CUtensorMap tmIn,
                                              const __grid_constant__ CUtensorMap tmE, Params P) {
    __shared__ StageSmem S;
    if (P.st->stop || useMarch(P)) return;
    tileInit(S, &tmIn, &tmE);
    uint32_t ph[2] = {0u, 0u};
    stageTiles<STAGE>(S, &tmIn, &tmE, P, P.st->nActive, ph);
}

// ---------------------------------------------------------------- k_commit
// Euler mode (euler_integration, simulator.cu:801) has a single stage: its
// result, written to the stage buffer so that no CTA reads a halo cell
// another CTA is updating, is copied back over U^n for the active tiles
// (interior cells and the ghost cells they own), together with F.
__device__ __forceinline__ void commitTile(const Params& P, int tile) {
    const int tid = threadIdx.x;
    const int bX = tile % P.nBX, bY = tile / P.nBX;
    if (tid >= TW * TH) return;
    const int i = bX * TW + tid % TW + 2, j = bY * TH + tid / TW + 2;
    if (!(i <= P.nx - 3 && j <= P.ny - 3)) return;
    auto cp = [&](int jj, int ii) {
        for (int f = 0; f < 3; f++) P.A[cidx(P, f, jj, ii)] = P.B[cidx(P, f, jj, ii)];
    };
    cp(j, i);
    if (P.flags & F_INFIL) P.FA[cidx(P, 0, j, i)] = P.FB[cidx(P, 0, j, i)];
    if (i == 2) {
        cp(j, 0);
        cp(j, 1);
    }
    if (i == P.nx - 3) {
        cp(j, P.nx - 2);
        cp(j, P.nx - 1);
    }
    if (j == 2) {
        cp(0, i);
        cp(1, i);
    }
    if (j == P.ny - 3) {
        cp(P.ny - 2, i);
        cp(P.ny - 1, i);
    }
}

__device__ __forceinline__ void commitTiles(const Params& P, int nAct) {
    for (int k = blockIdx.x; k < nAct; k += gridDim.x) commitTile(P, P.act[k]);
}

__global__ void __launch_bounds__(NT) k_commit(Params P) {
    if (P.st->stop) return;
    commitTiles(P, P.st->nActive);
}

// ---------------------------------------------------------------- volume
// FP64 compensated (Neumaier) sum over interior cells of h + F (what = 0;
// F only with infiltration), h (what = 1) or F (what = 2); one partial per
// block, combined on the host with the same summation.
__global__ void k_volume(Params P, double* partial, int what) {
    double s = 0.0, c = 0.0;
    const int nInt = (P.nx - 4) * (P.ny - 4);
    const bool withH = what != 2, withF = what != 1 && (P.flags & F_INFIL) && P.FA;
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < nInt; q += gridDim.x * blockDim.x) {
        int i = q % (P.nx - 4) + 2, j = q / (P.nx - 4) + 2;
        double v = withH ? (double)P.A[cidx(P, 0, j, i)] : 0.0;
        if (withF) v += (double)P.FA[cidx(P, 0, j, i)];
        double t = s + v;
        c += (fabs(s) >= fabs(v)) ? (s - t) + v : (v - t) + s;
        s = t;
    }
    __shared__ double ss[256], cc[256];
    ss[threadIdx.x] = s;
    cc[threadIdx.x] = c;
    __syncthreads();
    if (threadIdx.x == 0) {
        double S = 0.0, C = 0.0;
        for (int k = 0; k < (int)blockDim.x; k++) {
            double v = ss[k];
            double t = S + v;
            C += (fabs(S) >= fabs(v)) ? (S - t) + v : (v - t) + S;
            S = t;
            C += cc[k];
        }
        partial[2 * blockIdx.x] = S;
        partial[2 * blockIdx.x + 1] = C;
    }
}

}  // namespace rift
