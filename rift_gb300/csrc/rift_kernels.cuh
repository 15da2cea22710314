// rift_kernels.cuh -- device kernels of the GB300 step.
//
// One step (the body of Simulator::RunSimulation, simulator.cu:773-853):
//   k_begin   : stop test, uniform-source interpolation (simulator.cu:500-538)
//   k_track   : re-wet inactive tiles under gridded rain / surge
//               (TrackRainfall_k / TrackSurge_k, grid.cu:1224-1276)
//   k_grow    : 4-neighbour dilation of the wet tiles and on-device
//               compaction of the active / inactive / deactivated tile lists
//               (Grow, grid.cu:1188-1322) with warp ballots and a block scan
//   k_speed   : per-tile local-speed maxima on U^n (the speed output of the
//               first ComputeFluxes, grid.cu:813-838); re-syncs the stage
//               buffer of tiles that just went inactive
//   k_dt      : max over every tile's speed (stale entries included, as
//               simulator.cu:544-545 does) -> dt, t (FP64)
//   k_stage<1>: fused flux + sources + friction + RK stage 1 + ghost cells
//               (ComputeFluxes_k + Integrate_1_k + ApplyBoundaries)
//   k_stage<2>: fused flux + sources + RK stage 2 + ghost cells + outputs +
//               tile wet flags + tile speeds
//               (ComputeFluxes_k + Integrate_2_k + ApplyBoundaries)
// Every stage kernel is persistent over the compacted active-tile list and
// stages each tile's halo'd block of (h, hu, hv) and the four face-elevation
// offsets in shared memory with TMA (cp.async.bulk.tensor, 3-D maps over the
// stacked fields) completing on an mbarrier.
#pragma once
#include <cuda.h>
#include <cstdint>

#include "rift_device.cuh"

namespace rift {

constexpr int TW = 16;          // tile width  (BLOCK_COLS, grid.cu:19)
constexpr int TH = 14;          // tile height (BLOCK_ROWS, grid.cu:18)
constexpr int SW = TW + 4;      // staged block width  (2-cell halo)
constexpr int SH = TH + 4;      // staged block height
constexpr int NT = 256;         // threads per stage CTA
constexpr int GROW_T = 1024;    // threads of the single-CTA grow kernel
constexpr int MAX_SERIES = 4096;

// flag bits, identical to include/rift_gb300.h
constexpr uint32_t F_RAIN_U = 1u << 0, F_RAIN_G = 1u << 1, F_DRAIN_U = 1u << 2,
                   F_DRAIN_G = 1u << 3, F_INFIL = 1u << 4, F_SURGE = 1u << 5,
                   F_EULER = 1u << 6, F_SAVE_MAX = 1u << 7, F_SAVE_ARR = 1u << 8,
                   F_TILE_ACC = 1u << 9, F_POINT = 1u << 10, F_H_INIT = 1u << 11;

constexpr int ERR_TMA_TIMEOUT = 1;

// Device-resident scalars of the run (one per handle).
struct DevState {
    double t;          // simulated time, FP64 accumulator
    double dt;         // dt of the current step (after k_dt)
    double dt_old;     // dt of the previous step (stage-1 source clamps)
    double t_stop;     // kernels idle once t >= t_stop at step start
    float rain_rate;   // uniform rates, m/s, as the reference's float rates
    float drain_rate;
    float ser_interp[3];  // Source::interpolated_rate state (A11)
    float factor[3];      // map interpolation factors
    unsigned max_bits[2];
    unsigned ticket;
    int nActive, nDeact, nInact;
    int stop;
    int steps_done;
    int error;
    int err_info;
};

struct Params {
    int nx, ny, nBX, nBY, gridSize;
    int pitch, rows;   // floats per row, rows per field plane
    float dx, dy, inv_dx, inv_dy, kappa, psiDtheta, nodata;
    double dxd, dyd, kappad, courant;
    uint32_t flags;
    float* A;          // [3][rows][pitch]  U^n / U^{n+1}: h, hu, hv
    float* B;          // [3][rows][pitch]  U*
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
    uint8_t* prevAct;
    int* act;
    int* deact;
    int* inact;
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

__device__ __forceinline__ size_t cidx(const Params& P, int f, int j, int i) {
    return ((size_t)f * P.rows + j) * P.pitch + i;
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

// Bounded wait on an mbarrier phase; returns false after the spin limit (the
// caller records the error and leaves the tile loop).
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity) {
    for (int it = 0; it < (1 << 20); ++it)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}

// ------------------------------------------------------------- shared block
struct __align__(128) StageSmem {
    float in[3][SH][SW];    // h, hu, hv     (TMA destination, 4320 B)
    float pad0[8];          // keeps `e` 128-byte aligned
    float e[4][SH][SW];     // eW, eE, eS, eN (TMA destination, 5760 B)
    union {
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
    uint64_t bar;
};
static_assert(offsetof(StageSmem, e) % 128 == 0, "TMA destination alignment");
constexpr uint32_t BYTES_IN = 3 * SH * SW * 4;
constexpr uint32_t BYTES_E = 4 * SH * SW * 4;

__device__ __forceinline__ bool tileHasInterior(const Params& P, int tile, int& i0, int& j0) {
    int bX = tile % P.nBX, bY = tile / P.nBX;
    i0 = bX * TW + 2;
    j0 = bY * TH + 2;
    return i0 <= P.nx - 3 && j0 <= P.ny - 3;
}

// Gridded map value at a cell (hold or InterpGrid_k semantics, grid.cu:292-311).
__device__ __forceinline__ float mapValue(const Params& P, int which, size_t c, float factor) {
    // a series that was never set reads as its GridSeries fill value:
    // nodata for surge (allow_no_data), 0 otherwise
    if (P.mapMode[which] == 0) return which == 2 ? P.nodata : 0.f;
    float x0 = P.map0[which][c];
    if (P.mapMode[which] != 2) return x0;
    float x1 = P.map1[which][c];
    float nd = P.nodata;
    if (x1 == nd && x0 == nd) return nd;
    if (x1 == nd) return x0;
    if (x0 == nd) return x1;
    return factor * (x1 - x0) + x0;
}

__device__ __forceinline__ float blockMax(float v, float* red, int slot) {
    for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
    int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    if (l == 0) red[w] = v;
    __syncthreads();
    float r = 0.f;
    if (threadIdx.x == 0) {
        for (int k = 0; k < NT / 32; k++) r = fmaxf(r, red[k]);
    }
    (void)slot;
    return r;  // valid in thread 0
}

// Issue the TMA loads of one tile's staged block and wait for them.
__device__ __forceinline__ bool stageTile(StageSmem& S, const CUtensorMap* tmIn,
                                          const CUtensorMap* tmE, int bX, int bY,
                                          uint32_t& phase) {
    if (threadIdx.x == 0) {
        fence_proxy_async();
        mbar_expect_tx(&S.bar, BYTES_IN + BYTES_E);
        tma_load_3d(&S.in[0][0][0], tmIn, &S.bar, bX * TW, bY * TH, 0);
        tma_load_3d(&S.e[0][0][0], tmE, &S.bar, bX * TW, bY * TH, 0);
    }
    bool ok = mbar_wait_bounded(&S.bar, phase);
    phase ^= 1u;
    return ok;
}

// ---------------------------------------------------------------- k_begin
// Start of a step: stop test and the uniform sources of
// Simulator::UpdateSource (simulator.cu:500-538): each CSV series is
// interpolated at float(t) (source.cc:65-73) and its float state divided in
// place (A11).  IEEE float ops (_rn intrinsics) keep the host arithmetic.
__device__ __forceinline__ float seriesInterp(const float* T, const float* R, int n, float t,
                                              float cur) {
    for (int i = 0; i + 1 < n; i++) {
        if (t >= T[i] && t < T[i + 1]) {
            float num = __fsub_rn(R[i + 1], R[i]);
            float den = __fsub_rn(T[i + 1], T[i]);
            cur = __fadd_rn(R[i], __fmul_rn(__fdiv_rn(num, den), __fsub_rn(t, T[i])));
        }
    }
    return cur;
}

__global__ void k_begin(Params P) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    DevState* s = P.st;
    if (s->t >= s->t_stop) {
        s->stop = 1;
        return;
    }
    s->stop = 0;
    s->steps_done += 1;
    s->max_bits[0] = 0u;
    s->max_bits[1] = 0u;
    s->ticket = 0u;
    const float tf = (float)s->t;
    if (P.serN[2] > 0) {  // hydrograph, cfs -> m^3/s -> m/s per source cell
        float v = seriesInterp(P.serT + 2 * MAX_SERIES, P.serR + 2 * MAX_SERIES, P.serN[2], tf,
                               s->ser_interp[2]);
        v = __fdiv_rn(v, 35.3147f);
        s->ser_interp[2] = v;
        double r = (double)v / P.dxd / P.dyd / (double)P.nsrc;
        for (int k = 0; k < P.nsrc; k++) P.srcRate[k] = (float)r;
    }
    if (P.serN[0] > 0) {  // hyetograph, mm/hr -> m/s
        float v = seriesInterp(P.serT, P.serR, P.serN[0], tf, s->ser_interp[0]);
        v = __fdiv_rn(v, 3600.f * 1000.f);
        s->ser_interp[0] = v;
        s->rain_rate = v;
    }
    if (P.serN[1] > 0) {  // drain, mm/hr -> m/s
        float v = seriesInterp(P.serT + MAX_SERIES, P.serR + MAX_SERIES, P.serN[1], tf,
                               s->ser_interp[1]);
        v = __fdiv_rn(v, 3600.f * 1000.f);
        s->ser_interp[1] = v;
        s->drain_rate = v;
    }
}

// ---------------------------------------------------------------- k_track
// TrackRainfall_k / TrackSurge_k over the tiles that were inactive after the
// previous Grow.  A9: the rows come from blockY * BLOCK_COLS (16), not 14.
__global__ void __launch_bounds__(NT) k_track(Params P) {
    const DevState* s = P.st;
    if (s->stop) return;
    const int n = s->nInact;
    for (int k = blockIdx.x; k < n; k += gridDim.x) {
        const int tile = P.inact[k];
        if (P.wet[tile]) continue;  // uniform across the block
        const int bX = tile % P.nBX, bY = tile / P.nBX;
        bool hit = false;
        if (threadIdx.x < TW * TH) {
            int tx = threadIdx.x % TW, ty = threadIdx.x / TW;
            int i = bX * TW + tx + 2, j = bY * TW + ty + 2;
            if (i >= 2 && j >= 2 && i <= P.nx - 3 && j <= P.ny - 3) {
                size_t c = cidx(P, 0, j, i);
                if (P.flags & F_RAIN_G) {
                    float v = mapValue(P, 0, c, s->factor[0]);
                    if (v > kEps) hit = true;
                }
                if (P.flags & F_SURGE) {
                    float v = mapValue(P, 2, c, s->factor[2]);
                    if (v != P.nodata && v > 0.f) hit = true;
                }
            }
        }
        if (__syncthreads_or(hit) && threadIdx.x == 0) P.wet[tile] = 1;
    }
}

// ---------------------------------------------------------------- k_grow
// Single CTA: active(t) = wet(t) | wet(4-neighbours), false outside the tile
// grid; tile 0 is always kept (A8: it encodes as 0, never negative).
// Compacts (ascending) the active ids, the inactive ids other than tile 0
// (tracked next step) and the tiles that went from active to inactive.
__device__ __forceinline__ int blockScanExclusive(int flag, int* warpSums, int& total) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    unsigned b = __ballot_sync(0xffffffffu, flag);
    int inWarp = __popc(b & ((1u << lane) - 1u));
    if (lane == 0) warpSums[w] = __popc(b);
    __syncthreads();
    if (w == 0) {
        int v = (lane < GROW_T / 32) ? warpSums[lane] : 0;
        int x = v;
        for (int o = 1; o < 32; o <<= 1) {
            int y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        if (lane < GROW_T / 32) warpSums[lane] = x - v;  // exclusive
        if (lane == 31) warpSums[32] = x;
    }
    __syncthreads();
    int r = warpSums[w] + inWarp;
    total = warpSums[32];
    __syncthreads();
    return r;
}

__global__ void __launch_bounds__(GROW_T) k_grow(Params P) {
    DevState* s = P.st;
    if (s->stop) return;
    __shared__ int sumsA[33], sumsD[33], sumsI[33];
    int baseA = 0, baseD = 0, baseI = 0;
    const int nBX = P.nBX, nBY = P.nBY;
    for (int b0 = 0; b0 < P.gridSize; b0 += GROW_T) {
        int b = b0 + threadIdx.x;
        int a = 0, d = 0, in = 0;
        if (b < P.gridSize) {
            int bX = b % nBX, bY = b / nBX;
            bool v = P.wet[b] || (bX > 0 && P.wet[b - 1]) || (bX < nBX - 1 && P.wet[b + 1]) ||
                     (bY > 0 && P.wet[b - nBX]) || (bY < nBY - 1 && P.wet[b + nBX]) || b == 0;
            a = v ? 1 : 0;
            d = (P.prevAct[b] && !v) ? 1 : 0;
            in = (!v && b != 0) ? 1 : 0;
        }
        int tA, tD, tI;
        int pa = blockScanExclusive(a, sumsA, tA);
        int pd = blockScanExclusive(d, sumsD, tD);
        int pi = blockScanExclusive(in, sumsI, tI);
        if (b < P.gridSize) {
            if (a) P.act[baseA + pa] = b;
            if (d) P.deact[baseD + pd] = b;
            if (in) P.inact[baseI + pi] = b;
            P.prevAct[b] = (uint8_t)a;
        }
        baseA += tA;
        baseD += tD;
        baseI += tI;
    }
    if (threadIdx.x == 0) {
        s->nActive = baseA;
        s->nDeact = baseD;
        s->nInact = baseI;
    }
}

// ---------------------------------------------------------------- k_speed
// Per-tile speed maxima of U^n over the active tiles (what the first
// ComputeFluxes of a step writes to mx/my, grid.cu:813-838), and the stage
// buffer re-sync of tiles that just went inactive (U* = U^n there).
__global__ void __launch_bounds__(NT) k_speed(const __grid_constant__ CUtensorMap tmA,
                                              const __grid_constant__ CUtensorMap tmE, Params P) {
    __shared__ StageSmem S;
    const DevState* st = P.st;
    if (st->stop) return;
    const int tid = threadIdx.x;
    if (tid == 0) {
        prefetch_tmap(&tmA);
        prefetch_tmap(&tmE);
        mbar_init(&S.bar, 1);
        fence_mbar_init();
    }
    __syncthreads();
    uint32_t phase = 0;
    const float kappa = P.kappa;
    const int nAct = st->nActive;
    for (int k = blockIdx.x; k < nAct; k += gridDim.x) {
        const int tile = P.act[k];
        int i0, j0;
        if (!tileHasInterior(P, tile, i0, j0)) {
            if (tid == 0) {
                P.mx[tile] = 0.f;
                P.my[tile] = 0.f;
            }
            continue;
        }
        const int bX = tile % P.nBX, bY = tile / P.nBX;
        __syncthreads();
        bool ok = stageTile(S, &tmA, &tmE, bX, bY, phase);
        if (!__syncthreads_and(ok)) {
            if (tid == 0) atomicOr(&P.st->error, ERR_TMA_TIMEOUT);
            return;
        }
        float spx = 0.f, spy = 0.f;
        // x: depth + hu reconstruction of cells i0-1..i0+16 on the tile rows
        if (tid < TH * (TW + 2)) {
            int r = tid / (TW + 2), c = tid % (TW + 2);
            int sr = r + 2, sc = c + 1;
            RecN R = constructN(S.in[0][sr][sc], S.in[1][sr][sc], S.in[0][sr][sc + 1],
                                S.in[1][sr][sc + 1], S.in[0][sr][sc - 1], S.in[1][sr][sc - 1],
                                S.e[0][sr][sc], S.e[1][sr][sc], S.e[1][sr][sc] - S.e[0][sr][sc + 1],
                                S.e[1][sr][sc - 1] - S.e[0][sr][sc]);
            S.rec.x.P[0][r][c] = R.hP;
            S.rec.x.P[1][r][c] = R.qP;
            S.rec.x.M[0][r][c] = R.hM;
            S.rec.x.M[1][r][c] = R.qM;
        }
        __syncthreads();
        if (tid < TH * TW) {  // east face of tile cell (ty, tx)
            int ty = tid / TW, tx = tid % TW;
            int i = i0 + tx, j = j0 + ty;
            if (i <= P.nx - 3 && j <= P.ny - 3)
                spx = faceSpeed(S.rec.x.P[0][ty][tx + 1], S.rec.x.P[1][ty][tx + 1],
                                S.rec.x.M[0][ty][tx + 2], S.rec.x.M[1][ty][tx + 2], kappa);
        }
        __syncthreads();
        // y: depth + hv reconstruction of rows j0-1..j0+14 (only j0..j0+14 needed)
        if (tid < (TH + 2) * TW) {
            int r = tid / TW, c = tid % TW;
            int sr = r + 1, sc = c + 2;
            RecN R = constructN(S.in[0][sr][sc], S.in[2][sr][sc], S.in[0][sr + 1][sc],
                                S.in[2][sr + 1][sc], S.in[0][sr - 1][sc], S.in[2][sr - 1][sc],
                                S.e[2][sr][sc], S.e[3][sr][sc], S.e[3][sr][sc] - S.e[2][sr + 1][sc],
                                S.e[3][sr - 1][sc] - S.e[2][sr][sc]);
            S.rec.y.P[0][r][c] = R.hP;
            S.rec.y.P[1][r][c] = R.qP;
            S.rec.y.M[0][r][c] = R.hM;
            S.rec.y.M[1][r][c] = R.qM;
        }
        __syncthreads();
        if (tid < TH * TW) {  // north face of tile cell (ty, tx)
            int ty = tid / TW, tx = tid % TW;
            int i = i0 + tx, j = j0 + ty;
            if (i <= P.nx - 3 && j <= P.ny - 3)
                spy = faceSpeed(S.rec.y.P[0][ty + 1][tx], S.rec.y.P[1][ty + 1][tx],
                                S.rec.y.M[0][ty + 2][tx], S.rec.y.M[1][ty + 2][tx], kappa);
        }
        float mxv = blockMax(spx, S.red[0], 0);
        __syncthreads();
        float myv = blockMax(spy, S.red[1], 1);
        if (tid == 0) {
            P.mx[tile] = mxv;
            P.my[tile] = myv;
        }
    }
    // re-sync U* with U^n on tiles that went inactive, including the ghost
    // cells their edge cells own
    const int nDe = st->nDeact;
    for (int k = blockIdx.x; k < nDe; k += gridDim.x) {
        const int tile = P.deact[k];
        const int bX = tile % P.nBX, bY = tile / P.nBX;
        if (tid < TW * TH) {
            int tx = tid % TW, ty = tid / TW;
            int i = bX * TW + tx + 2, j = bY * TH + ty + 2;
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
}

// ---------------------------------------------------------------- k_dt
// Simulator::ComputeTimestep (simulator.cu:540-566) on device.  The max runs
// over every tile (stale speeds of inactive tiles included, A5).  The last
// CTA to finish turns the maxima into dt with the reference's rounding
// points (fmaxf on the scaled maxima, FP64 division), then t += dt.
__global__ void __launch_bounds__(256) k_dt(Params P) {
    DevState* s = P.st;
    if (s->stop) return;
    float mx = 0.f, my = 0.f;
    for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < P.gridSize; b += gridDim.x * blockDim.x) {
        mx = fmaxf(mx, P.mx[b]);
        my = fmaxf(my, P.my[b]);
    }
    for (int o = 16; o > 0; o >>= 1) {
        mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
        my = fmaxf(my, __shfl_xor_sync(0xffffffffu, my, o));
    }
    __shared__ float rx[8], ry[8];
    __shared__ bool last;
    int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    if (l == 0) {
        rx[w] = mx;
        ry[w] = my;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int k = 1; k < (int)(blockDim.x >> 5); k++) {
            mx = fmaxf(mx, rx[k]);
            my = fmaxf(my, ry[k]);
        }
        // speeds are non-negative: their bit patterns order like the values
        atomicMax(&s->max_bits[0], __float_as_uint(mx));
        atomicMax(&s->max_bits[1], __float_as_uint(my));
        __threadfence();
        unsigned tk = atomicAdd(&s->ticket, 1u);
        last = (tk == gridDim.x - 1);
    }
    __syncthreads();
    if (last && threadIdx.x == 0) {
        __threadfence();
        double maxx = (double)__uint_as_float(atomicOr(&s->max_bits[0], 0u));
        double maxy = (double)__uint_as_float(atomicOr(&s->max_bits[1], 0u));
        double cx = P.dxd / (double)fmaxf((float)(maxx / P.courant), (float)P.kappad);
        double cy = P.dyd / (double)fmaxf((float)(maxy / P.courant), (float)P.kappad);
        double dt = cx < cy ? cx : cy;
        if (s->t == 0.0) dt = (double)0.000001f;
        s->dt_old = s->dt;
        s->dt = dt;
        s->t = s->t + dt;
    }
}

// ---------------------------------------------------------------- k_stage
// Ghost cells owned by interior cell (j, i): critical-depth outflow
// (ApplyBoundariesX_k: clamped at epsilon; ApplyBoundariesY_k: not, A4).
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

// STAGE 1: reads U^n (A) -> writes U* (B), F* (FB).
// STAGE 2: reads U* (B) with halo and U^n (A) at the cell -> writes U^{n+1}
//          (A), F^{n+1} (FA), outputs, tile wet flags and tile speeds.
template <int STAGE>
__global__ void __launch_bounds__(NT) k_stage(const __grid_constant__ CUtensorMap tmIn,
                                              const __grid_constant__ CUtensorMap tmE, Params P) {
    __shared__ StageSmem S;
    const DevState* st = P.st;
    if (st->stop) return;
    const int tid = threadIdx.x;
    if (tid == 0) {
        prefetch_tmap(&tmIn);
        prefetch_tmap(&tmE);
        mbar_init(&S.bar, 1);
        fence_mbar_init();
    }
    __syncthreads();
    uint32_t phase = 0;
    const float kappa = P.kappa;
    const uint32_t fl = P.flags;
    const bool euler = (fl & F_EULER) != 0;
    const float dtNew = (float)st->dt;
    // source clamps use the dt passed to ComputeFluxes: the previous dt in
    // stage 1 (simulator.cu:786-792), the new one in stage 2
    const float dtSrc = (STAGE == 1) ? (float)st->dt_old : dtNew;
    const float invDtSrc = 1.f / dtSrc;
    const double tNew = st->t;
    const float rainU = st->rain_rate, drainU = st->drain_rate;
    const float fac0 = st->factor[0], fac1 = st->factor[1], fac2 = st->factor[2];
    float* Uout = (STAGE == 1) ? P.B : P.A;
    const float* Fin = (STAGE == 1) ? P.FA : P.FB;
    float* Fout = (STAGE == 1) ? P.FB : P.FA;
    const int nAct = st->nActive;

    for (int k = blockIdx.x; k < nAct; k += gridDim.x) {
        const int tile = P.act[k];
        int i0, j0;
        if (!tileHasInterior(P, tile, i0, j0)) {
            if (STAGE == 2 && tid == 0) {
                P.mx[tile] = 0.f;
                P.my[tile] = 0.f;
            }
            continue;
        }
        const int bX = tile % P.nBX, bY = tile / P.nBX;
        __syncthreads();
        bool ok = stageTile(S, &tmIn, &tmE, bX, bY, phase);
        if (!__syncthreads_and(ok)) {
            if (tid == 0) atomicOr(&P.st->error, ERR_TMA_TIMEOUT);
            return;
        }
        // ---- x reconstruction: cells i0-1 .. i0+16 on the 14 tile rows
        if (tid < TH * (TW + 2)) {
            int r = tid / (TW + 2), c = tid % (TW + 2);
            int sr = r + 2, sc = c + 1;
            Rec R = construct(S.in[0][sr][sc], S.in[1][sr][sc], S.in[2][sr][sc],
                              S.in[0][sr][sc + 1], S.in[1][sr][sc + 1], S.in[2][sr][sc + 1],
                              S.in[0][sr][sc - 1], S.in[1][sr][sc - 1], S.in[2][sr][sc - 1],
                              S.e[0][sr][sc], S.e[1][sr][sc],
                              S.e[1][sr][sc] - S.e[0][sr][sc + 1],
                              S.e[1][sr][sc - 1] - S.e[0][sr][sc]);
            S.rec.x.P[0][r][c] = R.hP;
            S.rec.x.P[1][r][c] = R.uP;
            S.rec.x.P[2][r][c] = R.vP;
            S.rec.x.M[0][r][c] = R.hM;
            S.rec.x.M[1][r][c] = R.uM;
            S.rec.x.M[2][r][c] = R.vM;
        }
        __syncthreads();
        // ---- x faces: face f between reconstructed cells f and f+1
        float spx = 0.f, spy = 0.f;
        if (tid < TH * (TW + 1)) {
            int r = tid / (TW + 1), f = tid % (TW + 1);
            float fx[3];
            float sp = faceFlux<0>(S.rec.x.P[0][r][f], S.rec.x.P[1][r][f], S.rec.x.P[2][r][f],
                                   S.rec.x.M[0][r][f + 1], S.rec.x.M[1][r][f + 1],
                                   S.rec.x.M[2][r][f + 1], kappa, fx);
            S.FX[0][r][f] = fx[0];
            S.FX[1][r][f] = fx[1];
            S.FX[2][r][f] = fx[2];
            // face f is the east face of tile column f-1
            if (STAGE == 2 && f >= 1 && i0 + f - 1 <= P.nx - 3 && j0 + r <= P.ny - 3) spx = sp;
        }
        __syncthreads();
        const bool cellThread = tid < TH * TW;
        const int tx = tid % TW, ty = tid / TW;
        float dh = 0.f, dhu = 0.f, dhv = 0.f;
        if (cellThread) {
            dh = -(S.FX[0][ty][tx + 1] - S.FX[0][ty][tx]) * P.inv_dx;
            dhu = -(S.FX[1][ty][tx + 1] - S.FX[1][ty][tx]) * P.inv_dx;
            dhv = -(S.FX[2][ty][tx + 1] - S.FX[2][ty][tx]) * P.inv_dx;
        }
        // ---- y reconstruction: rows j0-1 .. j0+14 of the 16 tile columns
        if (tid < (TH + 2) * TW) {
            int r = tid / TW, c = tid % TW;
            int sr = r + 1, sc = c + 2;
            Rec R = construct(S.in[0][sr][sc], S.in[1][sr][sc], S.in[2][sr][sc],
                              S.in[0][sr + 1][sc], S.in[1][sr + 1][sc], S.in[2][sr + 1][sc],
                              S.in[0][sr - 1][sc], S.in[1][sr - 1][sc], S.in[2][sr - 1][sc],
                              S.e[2][sr][sc], S.e[3][sr][sc],
                              S.e[3][sr][sc] - S.e[2][sr + 1][sc],
                              S.e[3][sr - 1][sc] - S.e[2][sr][sc]);
            S.rec.y.P[0][r][c] = R.hP;
            S.rec.y.P[1][r][c] = R.uP;
            S.rec.y.P[2][r][c] = R.vP;
            S.rec.y.M[0][r][c] = R.hM;
            S.rec.y.M[1][r][c] = R.uM;
            S.rec.y.M[2][r][c] = R.vM;
        }
        __syncthreads();
        if (tid < (TH + 1) * TW) {
            int r = tid / TW, c = tid % TW;
            float fy[3];
            float sp = faceFlux<1>(S.rec.y.P[0][r][c], S.rec.y.P[1][r][c], S.rec.y.P[2][r][c],
                                   S.rec.y.M[0][r + 1][c], S.rec.y.M[1][r + 1][c],
                                   S.rec.y.M[2][r + 1][c], kappa, fy);
            S.FY[0][r][c] = fy[0];
            S.FY[1][r][c] = fy[1];
            S.FY[2][r][c] = fy[2];
            if (STAGE == 2 && r >= 1 && i0 + c <= P.nx - 3 && j0 + r - 1 <= P.ny - 3) spy = sp;
        }
        __syncthreads();
        bool wetCell = false;
        if (cellThread) {
            dh += -(S.FY[0][ty + 1][tx] - S.FY[0][ty][tx]) * P.inv_dy;
            dhu += -(S.FY[1][ty + 1][tx] - S.FY[1][ty][tx]) * P.inv_dy;
            dhv += -(S.FY[2][ty + 1][tx] - S.FY[2][ty][tx]) * P.inv_dy;
            const int i = i0 + tx, j = j0 + ty;
            if (i <= P.nx - 3 && j <= P.ny - 3) {
                const size_t c = cidx(P, 0, j, i);
                const float hC = S.in[0][ty + 2][tx + 2];
                const float hu0 = S.in[1][ty + 2][tx + 2];
                const float hv0 = S.in[2][ty + 2][tx + 2];
                const float eW = S.e[0][ty + 2][tx + 2], eE = S.e[1][ty + 2][tx + 2];
                const float eS = S.e[2][ty + 2][tx + 2], eN = S.e[3][ty + 2][tx + 2];
                // bed-slope source, grid.cu:701,751-752
                const float S1 = -kG * hC * ((eE - eW) * P.inv_dx);
                const float S2 = -kG * hC * ((eN - eS) * P.inv_dy);
                // mass sources, grid.cu:763-807
                float S0 = 0.f;
                if (fl & F_RAIN_U) S0 += rainU;
                float rainG = 0.f;
                if (fl & F_RAIN_G) {
                    rainG = mapValue(P, 0, c, fac0);
                    S0 += rainG;
                }
                const float cap = hC * invDtSrc;
                if (fl & F_DRAIN_U) S0 -= (drainU > cap) ? cap : drainU;
                if (fl & F_DRAIN_G) {
                    float d = mapValue(P, 1, c, fac1);
                    S0 -= (d > cap) ? cap : d;
                }
                bool srcCell = false;
                if (P.nsrc > 0) {
                    const int flat = j * P.nx + i;
                    for (int q = P.srcTileStart[tile]; q < P.srcTileStart[tile + 1]; q++) {
                        int sidx = P.srcTileList[q];
                        if (P.srcIdx[sidx] == flat) {
                            S0 += P.srcRate[sidx];
                            srcCell = true;
                        }
                    }
                }
                float dF = 0.f, Fc = 0.f;
                if (fl & F_INFIL) {
                    Fc = Fin[c];
                    dF = greenAmpt(P.K[c], Fc, P.psiDtheta, dtSrc, hC);
                    S0 -= dF;
                }
                dh += S0;
                dhu += S1;
                dhv += S2;
                const float hc = (hC > kEps) ? hC : 0.f;  // grid.cu:748-749
                float hN, huN, hvN;
                if (STAGE == 1) {
                    // Integrate_1_k (grid.cu:856-922)
                    const float G = manningG(P.nman[c], hu0, hv0, hC, kappa);
                    if (fl & F_SURGE) {
                        float sg = mapValue(P, 2, c, fac2);
                        if (sg != P.nodata && sg > 0.f) dh = (sg - (hc + dh * dtNew)) / dtNew;
                    }
                    hN = hc + dh * dtNew;
                    const float den = 1.f / (1.f - dtNew * G);
                    huN = (hu0 + dhu * dtNew) * den;
                    hvN = (hv0 + dhv * dtNew) * den;
                    hN = (hN > kEps) ? hN : 0.f;
                    if (fl & F_INFIL) Fout[c] = Fc + dF * dtNew;
                    if (euler) {
                        // Euler-mode outputs and wet flags (grid.cu:926-1023)
                        const float uC = huN * velFactor(hN, kappa), vC = hvN * velFactor(hN, kappa);
                        if (fl & F_SAVE_MAX) {
                            float hm = P.hmax[c];
                            if (hN > hm) P.tpeak[c] = (float)tNew;
                            if (hN > 0.0762f) P.tdry[c] = (float)tNew;
                            P.hmax[c] = fmaxf(hm, hN);
                            P.qmax[c] = fmaxf(P.qmax[c], hN * sqrtf(vC * vC + uC * uC));
                        }
                        if (fl & F_SAVE_ARR) {
                            if (P.twet[c] < 0.f && hN > kEps) P.twet[c] = (float)tNew;
                        }
                        wetCell = (hN > kEps) || srcCell || ((fl & F_RAIN_U) && rainU > 0.f) ||
                                  ((fl & F_RAIN_G) && rainG > 0.f);
                        if (fl & F_SURGE) {
                            float sg = mapValue(P, 2, c, fac2);
                            if (sg != P.nodata && sg > 0.f) wetCell = true;
                        }
                    }
                } else {
                    // Integrate_2_k (grid.cu:1043-1171)
                    const float hOld = P.A[cidx(P, 0, j, i)];
                    const float hOc = (hOld > kEps) ? hOld : 0.f;
                    hN = 0.5f * (hOc + hc + dh * dtNew);
                    huN = 0.5f * (P.A[cidx(P, 1, j, i)] + hu0 + dhu * dtNew);
                    hvN = 0.5f * (P.A[cidx(P, 2, j, i)] + hv0 + dhv * dtNew);
                    hN = (hN > kEps) ? hN : 0.f;
                    if (fl & F_INFIL) Fout[c] = 0.5f * (P.FA[c] + Fc + dF * dtNew);
                    if (fl & F_SAVE_MAX) {
                        const float uC = huN * velFactor(hN, kappa);
                        const float vC = hvN * velFactor(hN, kappa);
                        P.hmax[c] = fmaxf(P.hmax[c], hN);
                        P.qmax[c] = fmaxf(P.qmax[c], hN * sqrtf(vC * vC + uC * uC));
                    }
                    if (fl & F_SAVE_ARR) {
                        if (P.twet[c] < 0.f && hN > kEps) P.twet[c] = (float)tNew;
                    }
                    wetCell = (hN > kEps) || srcCell || ((fl & F_RAIN_U) && rainU > 0.f) ||
                              ((fl & F_RAIN_G) && rainG > 0.f);
                }
                Uout[cidx(P, 0, j, i)] = hN;
                Uout[cidx(P, 1, j, i)] = huN;
                Uout[cidx(P, 2, j, i)] = hvN;
                writeGhosts(P, Uout, j, i, hN, huN, hvN);
            }
        }
        // ---- tile flags and speeds
        if (STAGE == 2 || euler) {
            bool any = __syncthreads_or(wetCell);
            if (tid == 0) P.wet[tile] = (uint8_t)((!(fl & F_TILE_ACC)) || any);
        }
        if (STAGE == 2) {
            float mxv = blockMax(spx, S.red[0], 0);
            __syncthreads();
            float myv = blockMax(spy, S.red[1], 1);
            if (tid == 0) {
                P.mx[tile] = mxv;
                P.my[tile] = myv;
            }
        }
    }
}

// ---------------------------------------------------------------- volume
// FP64 compensated (Neumaier) sum of (h [+ F]) over interior cells; one
// partial per block, combined on the host with the same summation.
__global__ void k_volume(Params P, double* partial) {
    double s = 0.0, c = 0.0;
    const int nInt = (P.nx - 4) * (P.ny - 4);
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < nInt; q += gridDim.x * blockDim.x) {
        int i = q % (P.nx - 4) + 2, j = q / (P.nx - 4) + 2;
        double v = (double)P.A[cidx(P, 0, j, i)];
        if (P.flags & F_INFIL) v += (double)P.FA[cidx(P, 0, j, i)];
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
