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
// 0..13 hold its tiles).  Pass A counts the chunk's entries per list; pass B
// takes its offsets from the counts of the CTAs before it and writes its
// entries with warp ballots and one block scan per 16 strips.  The lists
// are not in ascending tile order (consumers only need the sets).
#pragma once
#include "rift_kernels.cuh"

namespace rift {

constexpr int GROW_LISTS = 4;            // scheduled active, deactivated, inactive, strips
constexpr int STRIPS_PER_ROUND = NT / 16;

struct GrowSmem {
    int wsum[GROW_LISTS][NT / 32 + 1];
    int red[GROW_LISTS][NT / 32];
    unsigned long long cred[NT / 32];
    int base[GROW_LISTS], total[GROW_LISTS];
    unsigned long long cells;
};

// active(t) of tile b: wet itself or a wet 4-neighbour; tile 0 always.
__device__ __forceinline__ bool tileGrows(const Params& P, int b) {
    const int bX = b % P.nBX, bY = b / P.nBX;
    return P.wet[b] || (bX > 0 && P.wet[b - 1]) || (bX < P.nBX - 1 && P.wet[b + 1]) ||
           (bY > 0 && P.wet[b - P.nBX]) || (bY < P.nBY - 1 && P.wet[b + P.nBX]) || b == 0;
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
};

__device__ __forceinline__ GrowItem growItem(const Params& P, int base, int s1) {
    GrowItem t;
    t.b = -1;
    t.v = false;
    t.cells = 0;
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
            t.v = tileGrows(P, b);
            t.cells = tileCells(P, b);
            t.f[0] = (t.v && t.cells > 0) ? 1 : 0;
            t.f[1] = (P.prevAct[b] && !t.v) ? 1 : 0;
            t.f[2] = (!t.v && b != 0) ? 1 : 0;
        }
    }
    const unsigned bal = __ballot_sync(0xffffffffu, t.f[0]);
    const unsigned grp = (bal >> (lane & 16)) & 0xffffu;
    t.f[3] = (stripIn && r == 0 && grp != 0u) ? 1 : 0;
    return t;
}

// Block reduction of per-thread list counts (and cells) into thread 0.
__device__ __forceinline__ void growReduce(GrowSmem& G, int (&c)[GROW_LISTS],
                                           unsigned long long& cells) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int o = 16; o > 0; o >>= 1) {
        for (int q = 0; q < GROW_LISTS; q++) c[q] += __shfl_xor_sync(0xffffffffu, c[q], o);
        cells += __shfl_xor_sync(0xffffffffu, cells, o);
    }
    if (lane == 0) {
        for (int q = 0; q < GROW_LISTS; q++) G.red[q][w] = c[q];
        G.cred[w] = cells;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int q = 0; q < GROW_LISTS; q++) {
            int x = 0;
            for (int k = 0; k < NT / 32; k++) x += G.red[q][k];
            c[q] = x;
        }
        unsigned long long cs = 0ull;
        for (int k = 0; k < NT / 32; k++) cs += G.cred[k];
        cells = cs;
    }
}

// Pass A: the chunk's list counts and cells, published per CTA.
__device__ void growCount(const Params& P, GrowSmem& G) {
    int s0, s1;
    stripChunk(P, s0, s1);
    int c[GROW_LISTS] = {0, 0, 0, 0};
    unsigned long long cells = 0ull;
    for (int base = s0; base < s1; base += STRIPS_PER_ROUND) {
        const GrowItem t = growItem(P, base, s1);
        for (int q = 0; q < GROW_LISTS; q++) c[q] += t.f[q];
        if (t.f[0]) cells += (unsigned long long)t.cells;
    }
    growReduce(G, c, cells);
    if (threadIdx.x == 0) {
        for (int q = 0; q < GROW_LISTS; q++) P.growCnt[blockIdx.x * GROW_LISTS + q] = c[q];
        P.growCells[blockIdx.x] = cells;
    }
}

// Pass B: offsets from the counts of the CTAs before this one, then the
// chunk's entries and the new active flags.  Returns the number of
// scheduled active tiles (all threads); CTA 0 publishes the list sizes.
__device__ int growWrite(const Params& P, GrowSmem& G) {
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    int pre[GROW_LISTS] = {0, 0, 0, 0}, tot[GROW_LISTS] = {0, 0, 0, 0};
    unsigned long long cells = 0ull, none = 0ull;
    for (int k = tid; k < (int)gridDim.x; k += NT) {
        for (int q = 0; q < GROW_LISTS; q++) {
            const int v = P.growCnt[k * GROW_LISTS + q];
            tot[q] += v;
            if (k < (int)blockIdx.x) pre[q] += v;
        }
        cells += P.growCells[k];
    }
    growReduce(G, pre, none);
    __syncthreads();
    growReduce(G, tot, cells);
    if (tid == 0) {
        for (int q = 0; q < GROW_LISTS; q++) {
            G.base[q] = pre[q];
            G.total[q] = tot[q];
        }
        G.cells = cells;
        if (blockIdx.x == 0) {
            DevState* s = P.st;
            s->nActive = tot[0];
            s->nDeact = tot[1];
            s->nInact = tot[2];
            s->nStrips = tot[3];
            s->activeCells += cells;
        }
    }
    __syncthreads();
    int base[GROW_LISTS] = {G.base[0], G.base[1], G.base[2], G.base[3]};
    const int nAct = G.total[0];
    int s0, s1;
    stripChunk(P, s0, s1);
    for (int rb = s0; rb < s1; rb += STRIPS_PER_ROUND) {
        const GrowItem t = growItem(P, rb, s1);
        int inWarp[GROW_LISTS];
        for (int q = 0; q < GROW_LISTS; q++) {
            const unsigned bal = __ballot_sync(0xffffffffu, t.f[q]);
            inWarp[q] = __popc(bal & ((1u << lane) - 1u));
            if (lane == 0) G.wsum[q][w] = __popc(bal);
        }
        __syncthreads();
        if (tid < GROW_LISTS) {  // thread q: exclusive scan of list q's warp totals
            int x = 0;
            for (int k = 0; k < NT / 32; k++) {
                const int y = G.wsum[tid][k];
                G.wsum[tid][k] = x;
                x += y;
            }
            G.wsum[tid][NT / 32] = x;
        }
        __syncthreads();
        if (t.f[0]) P.act[base[0] + G.wsum[0][w] + inWarp[0]] = t.b;
        if (t.f[1]) P.deact[base[1] + G.wsum[1][w] + inWarp[1]] = t.b;
        if (t.f[2]) P.inact[base[2] + G.wsum[2][w] + inWarp[2]] = t.b;
        if (t.f[3]) P.strips[base[3] + G.wsum[3][w] + inWarp[3]] = t.strip;
        if (t.b >= 0) {
            if (t.v && t.cells == 0) {
                P.mx[t.b] = 0.f;
                P.my[t.b] = 0.f;
            }
            P.prevAct[t.b] = (uint8_t)(t.v ? 1 : 0);
        }
        for (int q = 0; q < GROW_LISTS; q++) base[q] += G.wsum[q][NT / 32];
        __syncthreads();
    }
    return nAct;
}

// Graph path: pass A (with the stop test and the start of the step) and
// pass B as two launches over the same grid.
__global__ void __launch_bounds__(NT) k_grow_a(Params P) {
    __shared__ GrowSmem G;
    DevState* s = P.st;
    if (s->t >= s->t_stop) {  // every CTA reads the same t
        if (blockIdx.x == 0 && threadIdx.x == 0) s->stop = 1;
        return;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) beginStep(P, s);
    growCount(P, G);
}

__global__ void __launch_bounds__(NT) k_grow_b(Params P) {
    __shared__ GrowSmem G;
    if (P.st->stop) return;
    growWrite(P, G);
}

}  // namespace rift
