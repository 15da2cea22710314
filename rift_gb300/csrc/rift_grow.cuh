// rift_grow.cuh -- the active-tile set of a step on device (Grow, grid.cu:1279-1322,
// Grow_k grid.cu:1188-1222), chunked over many CTAs.
//
// active(t) = wet(t) | wet(4-neighbours), false outside the tile grid; tile 0
// always (the reference encodes it as 0, never negative).  Four lists are
// compacted: the active tiles that hold interior cells (scheduled), the
// tiles that went from active to inactive (U* re-sync), the inactive tiles
// other than tile 0 (tracked next step under gridded rain / surge) and the
// strips of 7 x 2 tiles holding a scheduled tile (work items of the march
// kernels).  Active tiles without interior cells (the reference computes them
// and writes mx = my = 0) get their zero speeds here and are not scheduled.
//
// Each CTA owns a contiguous chunk of strips, 16 threads per strip (lanes
// 0..13 hold its tiles); entries are appended with one atomic per warp and
// list, and the last CTA publishes the counts.  The lists are not in
// ascending tile order: consumers need only the sets, and no result depends
// on the order (speed maxima are order-free, no float sum crosses tiles).
#pragma once
#include "rift_kernels.cuh"

namespace rift {

constexpr int GROW_LISTS = 4;            // scheduled active, deactivated, inactive, strips
constexpr int STRIPS_PER_ROUND = NT / 16;

// active(t) of tile b: wet itself or a wet 4-neighbour; tile 0 always.
// The five flags are loaded together (no short-circuit: a dry tile would
// otherwise wait for five loads in a row).
__device__ __forceinline__ bool tileGrows(const Params& P, int b) {
    const int bX = b % P.nBX, bY = b / P.nBX;
    const unsigned w = P.wet[b];
    const unsigned wW = bX > 0 ? P.wet[b - 1] : 0u;
    const unsigned wE = bX < P.nBX - 1 ? P.wet[b + 1] : 0u;
    const unsigned wS = bY > 0 ? P.wet[b - P.nBX] : 0u;
    const unsigned wN = bY < P.nBY - 1 ? P.wet[b + P.nBX] : 0u;
    return ((w | wW | wE | wS | wN) != 0u) || b == 0;
}

// Interior cells of tile b (0 for a tile wholly in the ghost band).
__device__ __forceinline__ int tileCells(const Params& P, int b) {
    const int bX = b % P.nBX, bY = b / P.nBX;
    const int i0 = bX * TW + 2, j0 = bY * TH + 2;
    if (i0 > P.nx - 3 || j0 > P.ny - 3) return 0;
    return (min(P.nx - 3, i0 + TW - 1) - i0 + 1) * (min(P.ny - 3, j0 + TH - 1) - j0 + 1);
}

// This CTA's strips [s0, s1).
__device__ __forceinline__ void stripChunk(const Params& P, int& s0, int& s1) {
    const int nS = P.nSX * P.nSY;
    const int L = (nS + gridDim.x - 1) / gridDim.x;
    s0 = min(nS, (int)blockIdx.x * L);
    s1 = min(nS, s0 + L);
}

// The tile of thread `tid` in the round starting at strip `base`, its list
// flags, and (lane 0 of each 16-lane group) the strip's flag.  All lanes of
// the warp must call it (ballot).
struct GrowItem {
    int b, strip, cells;
    bool v;
    int f[GROW_LISTS];
    float mxb, myb;  // the tile's speeds entering the step
};

__device__ __forceinline__ GrowItem growItem(const Params& P, int base, int s1) {
    GrowItem t;
    t.b = -1;
    t.v = false;
    t.cells = 0;
    t.mxb = t.myb = 0.f;
    for (int q = 0; q < GROW_LISTS; q++) t.f[q] = 0;
    const int lane = threadIdx.x & 31, r = threadIdx.x & 15;
    t.strip = base + (int)threadIdx.x / 16;
    const bool stripIn = t.strip < s1;
    if (stripIn && r < STRIP_TX * STRIP_TY) {
        const int sx = t.strip % P.nSX, sy = t.strip / P.nSX;
        const int bx = STRIP_TX * sx + r % STRIP_TX, by = STRIP_TY * sy + r / STRIP_TX;
        if (bx < P.nBX && by < P.nBY) {
            const int b = by * P.nBX + bx;
            t.b = b;
            const bool was = P.prevAct[b] != 0;
            t.mxb = P.mx[b];
            t.myb = P.my[b];
            t.v = tileGrows(P, b);
            t.cells = tileCells(P, b);
            t.f[0] = (t.v && t.cells > 0) ? 1 : 0;
            t.f[1] = (was && !t.v) ? 1 : 0;
            t.f[2] = (!t.v && b != 0) ? 1 : 0;
        }
    }
    const unsigned bal = __ballot_sync(0xffffffffu, t.f[0]);
    const unsigned grp = (bal >> (lane & 16)) & 0xffffu;
    t.f[3] = (stripIn && r == 0 && grp != 0u) ? 1 : 0;
    return t;
}

// One pass: each CTA's chunk of strips appends its entries to the four lists
// with one atomic per warp and list (the lists are sets: their order changes
// no result), writes the new active flags, folds the stale speeds of the
// tiles not active this step into DevState.staleBits (the stale entries
// ComputeTimestep's max includes, A5).  With PUBLISH the last CTA to finish
// publishes the list sizes and clears the counters for the next step;
// without, the caller reads the counters after a grid barrier and publishes
// them later (publishGrow).
template <bool PUBLISH = true>
__device__ void growAppend(const Params& P, unsigned* staleDst = nullptr) {
    DevState* s = P.st;
    const int tid = threadIdx.x, lane = tid & 31;
    int s0, s1;
    stripChunk(P, s0, s1);
    int* const lists[GROW_LISTS] = {P.act, P.deact, P.inact, P.strips};
    unsigned long long cells = 0ull;
    float smx = 0.f, smy = 0.f;
    for (int rb = s0; rb < s1; rb += STRIPS_PER_ROUND) {
        const GrowItem t = growItem(P, rb, s1);
        unsigned bal[GROW_LISTS];
        for (int q = 0; q < GROW_LISTS; q++) bal[q] = __ballot_sync(0xffffffffu, t.f[q]);
        // lane q reserves the warp's entries of list q: the four atomics are
        // in flight together
        const unsigned mineBal = lane == 0 ? bal[0] : lane == 1 ? bal[1] : lane == 2 ? bal[2] : bal[3];
        int base = 0;
        if (lane < GROW_LISTS && mineBal) base = atomicAdd(&s->appendCnt[lane], __popc(mineBal));
        const unsigned below = (1u << lane) - 1u;
        for (int q = 0; q < GROW_LISTS; q++) {
            const int bq = __shfl_sync(0xffffffffu, base, q);
            if (t.f[q]) lists[q][bq + __popc(bal[q] & below)] = q == 3 ? t.strip : t.b;
        }
        if (t.f[0]) cells += (unsigned long long)t.cells;
        if (t.b >= 0) {
            if (t.v && t.cells == 0) {
                P.mx[t.b] = 0.f;
                P.my[t.b] = 0.f;
            }
            if (!t.v) {  // a tile not active this step: its stale speeds count for dt (A5)
                smx = fmaxf(smx, t.mxb);
                smy = fmaxf(smy, t.myb);
            }
            P.prevAct[t.b] = (uint8_t)(t.v ? 1 : 0);
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        cells += __shfl_xor_sync(0xffffffffu, cells, o);
        smx = fmaxf(smx, __shfl_xor_sync(0xffffffffu, smx, o));
        smy = fmaxf(smy, __shfl_xor_sync(0xffffffffu, smy, o));
    }
    if (lane == 0 && cells) atomicAdd(&s->appendCells, cells);
    unsigned* const stale = staleDst ? staleDst : s->staleBits;
    if (lane == 0 && smx > 0.f) atomicMax(&stale[0], __float_as_uint(smx));
    if (lane == 0 && smy > 0.f) atomicMax(&stale[1], __float_as_uint(smy));
    if (!PUBLISH) return;
    __syncthreads();
    if (tid == 0) {
        __threadfence();
        if (atomicAdd(&s->growTicket, 1u) == gridDim.x - 1) {
            __threadfence();
            s->nActive = atomicExch(&s->appendCnt[0], 0);
            s->nDeact = atomicExch(&s->appendCnt[1], 0);
            s->nInact = atomicExch(&s->appendCnt[2], 0);
            s->nStrips = atomicExch(&s->appendCnt[3], 0);
            s->activeCells += atomicExch(&s->appendCells, 0ull);
            atomicExch(&s->growTicket, 0u);
        }
    }
}

// The grow's counters into the published list sizes, cleared for the next
// step (one thread; no CTA may append or read the counters meanwhile).
__device__ __forceinline__ void publishGrow(DevState* s) {
    s->nActive = s->appendCnt[0];
    s->nDeact = s->appendCnt[1];
    s->nInact = s->appendCnt[2];
    s->nStrips = s->appendCnt[3];
    s->activeCells += s->appendCells;
    for (int q = 0; q < GROW_LISTS; q++) s->appendCnt[q] = 0;
    s->appendCells = 0ull;
}

// Graph path: the stop test, the start of the step and the grow in one
// launch.
__global__ void __launch_bounds__(NT) k_grow(Params P) {
    DevState* s = P.st;
    if (s->t >= s->t_stop) {  // every CTA reads the same t
        if (blockIdx.x == 0 && threadIdx.x == 0) s->stop = 1;
        return;
    }
    if (blockIdx.x == 0 && threadIdx.x < 32) beginStep(P, s);
    growAppend(P);
}

}  // namespace rift
