// rift_ensemble.cuh -- many independent simulations (members: scenarios on
// domains of uneven size) stepped by one persistent cooperative kernel.
//
// Each member is an engine handle with its own buffers, DevState and dt.
// Every iteration of k_ensemble advances every live member by one of its own
// steps, in five phases separated by grid barriers (six with tracking); in
// each phase the CTAs walk one device queue over all members' work items:
//   T  (members with gridded rain or surge) re-wet tracking of inactive tiles
//   G  grow: the strips of all live members (chunked over the CTAs) append
//      each member's lists; the start of each member's step (one warp per
//      member); the stale speed maxima of the tiles that are not active
//   S  speeds: (member, active tile) items -> tile speeds, member maxima;
//      (member, deactivated tile) items -> U* re-sync
//   D  dt: one thread per member -> dt, t, ledger, list sizes, liveness of
//      the member's next step
//   1  stage 1: (member, active tile) items
//   2  stage 2, or the Euler commit: (member, active tile) items
// The per-tile arithmetic is the single-member code (tileSpeeds,
// tileFluxDiv, cellUpdate, ...), so each member's results are those of a run
// of its own.  A member is live while t < t_stop and its step count is below
// the requested maximum; the kernel ends when no member is live.  Every
// wait is bounded (TMA mbarriers, grid barriers), as in k_persist.
#pragma once
#include "rift_grow.cuh"
#include "rift_kernels.cuh"
#include "rift_persist.cuh"

namespace rift {

constexpr int ENS_MAX = 1024;  // members per ensemble

// Device side of an ensemble.
struct EnsDev {
    GridBar bar;
    int live[2][ENS_MAX];  // liveness per step parity
    int nAlive[2];
    StageConsts consts[ENS_MAX][2];  // each member's stage constants of the step (phase D)
    unsigned long long t0;                // globaltimer at the kernel's start (ns)
    unsigned long long tDone[ENS_MAX];    // globaltimer when each member finished its last step
};

__device__ __forceinline__ unsigned long long globalTimerNs() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

struct EnsArgs {
    const Params* Ps;        // [n] member parameters
    const CUtensorMap* maps;  // [n][3]: A, B, E tile maps of each member
    EnsDev* dev;
    int n;
    int maxSteps;
};

struct EnsSmem {
    int offs[ENS_MAX + 1];   // prefix of the current queue's per-member counts
    int offs2[ENS_MAX + 1];  // a second queue of the same phase
};

// Exclusive prefix of per-member counts get(m) (0 for members not live)
// into offs[0..n]; all threads; offs[n] is the total.
template <class Get>
__device__ __forceinline__ void ensPrefix(int n, Get get, int* offs) {
    const int tid = threadIdx.x;
    constexpr int PER = (ENS_MAX + NT - 1) / NT;  // members per thread
    int v[PER], sum = 0;
    for (int q = 0; q < PER; q++) {
        const int m = tid * PER + q;
        v[q] = m < n ? get(m) : 0;
        sum += v[q];
    }
    // block scan of the per-thread sums (warp shuffles, then warp totals)
    __shared__ int wtot[NT / 32];
    const int lane = tid & 31, w = tid >> 5;
    int x = sum;
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) wtot[w] = x;
    __syncthreads();
    int before = 0;
    for (int k = 0; k < w; k++) before += wtot[k];
    int run = before + x - sum;  // exclusive prefix of this thread
    for (int q = 0; q < PER; q++) {
        const int m = tid * PER + q;
        if (m <= n) offs[m] = run;
        run += v[q];
    }
    if (tid == NT - 1) offs[n] = run;
    __syncthreads();
}

// Member of queue item g: offs[m] <= g < offs[m + 1] (binary search).
__device__ __forceinline__ int ensMember(const int* offs, int n, int g) {
    int lo = 0, hi = n - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (offs[mid] <= g)
            lo = mid;
        else
            hi = mid - 1;
    }
    return lo;
}


// Queue walk with the staged blocks of two consecutive items in flight:
// items g = blockIdx.x, += gridDim.x of a queue with prefix offs over the
// members; item g is tile act[g - offs[m]] of member m, staged from its map
// `which` (0: A, 1: B) and its face offsets.  pre(m, tile) runs before the
// wait, body(m, tile, T) on the staged block.  False after a TMA timeout
// (error recorded in the member's DevState).
template <class Pre, class Body>
__device__ bool ensTileLoop(StageSmem& S, const EnsArgs& E, const int* offs, int which,
                            uint32_t* ph, Pre pre, Body body) {
    const int tid = threadIdx.x, n = E.n;
    const int total = offs[n];
    auto issue = [&](int g, int b) {
        const int m = ensMember(offs, n, g);
        const Params& P = E.Ps[m];
        issueTile(S.buf[b], &S.bar[b], &E.maps[3 * m + which], &E.maps[3 * m + 2], P,
                  P.act[g - offs[m]]);
    };
    if (tid == 0 && (int)blockIdx.x < total) issue(blockIdx.x, 0);
    __syncthreads();
    int b = 0;
    for (int g = blockIdx.x; g < total; g += gridDim.x, b ^= 1) {
        const int m = ensMember(offs, n, g);
        const Params& P = E.Ps[m];
        const int tile = P.act[g - offs[m]];
        pre(m, tile);
        bool ok = mbar_wait_bounded(&S.bar[b], ph[b]);
        if (!__syncthreads_and(ok)) {
            mbar_wait_bounded(&S.bar[b], ph[b]);
            if (tid == 0) atomicOr(&P.st->error, ERR_TMA_TIMEOUT);
            return false;
        }
        ph[b] ^= 1u;
        if (tid == 0 && g + (int)gridDim.x < total) issue(g + gridDim.x, b ^ 1);
        body(m, tile, S.buf[b]);
        __syncthreads();
    }
    return true;
}

// The grow item of thread tid for global strip gs of the concatenated strip
// space (prefix offs over the live members): growItem's flags on the
// member's own tile grid.
__device__ __forceinline__ GrowItem ensGrowItem(const EnsArgs& E, const int* offs, int gs,
                                                 bool valid, int& m) {
    GrowItem t;
    t.b = -1;
    t.v = false;
    t.cells = 0;
    t.strip = -1;
    for (int q = 0; q < GROW_LISTS; q++) t.f[q] = 0;
    m = valid ? ensMember(offs, E.n, gs) : 0;
    const int lane = threadIdx.x & 31, r = threadIdx.x & 15;
    const Params& P = E.Ps[m];
    if (valid) {
        t.strip = gs - offs[m];
        if (r < STRIP_TX * STRIP_TY) {
            const int sx = t.strip % P.nSX, sy = t.strip / P.nSX;
            const int bx = STRIP_TX * sx + r % STRIP_TX, by = STRIP_TY * sy + r / STRIP_TX;
            if (bx < P.nBX && by < P.nBY) {
                const int bb = by * P.nBX + bx;
                t.b = bb;
                t.v = tileGrows(P, bb);
                t.cells = tileCells(P, bb);
                t.f[0] = (t.v && t.cells > 0) ? 1 : 0;
                t.f[1] = (P.prevAct[bb] && !t.v) ? 1 : 0;
                t.f[2] = (!t.v && bb != 0) ? 1 : 0;
            }
        }
    }
    const unsigned bal = __ballot_sync(0xffffffffu, t.f[0]);
    const unsigned grp = (bal >> (lane & 16)) & 0xffffu;
    t.f[3] = (valid && r == 0 && grp != 0u) ? 1 : 0;
    return t;
}

// Phase G for all live members: each CTA's chunk of the concatenated strips
// appends to the members' lists (one atomic per half-warp, member and list:
// the two halves of a warp may hold strips of two members) and folds the
// stale speeds of the tiles that are not active this step into the
// member's stale maxima.
__device__ void ensGrow(const EnsArgs& E, const int* offs) {
    const int tid = threadIdx.x, lane = tid & 31;
    const int total = offs[E.n];
    const int L = (total + gridDim.x - 1) / gridDim.x;
    const int s0 = min(total, (int)blockIdx.x * L), s1 = min(total, s0 + L);
    const unsigned half = (lane < 16) ? 0x0000ffffu : 0xffff0000u;
    const int leader = lane & 16;
    for (int rb = s0; rb < s1; rb += STRIPS_PER_ROUND) {
        const int gs = rb + tid / 16;
        int m;
        const GrowItem t = ensGrowItem(E, offs, gs, gs < s1, m);
        const Params& P = E.Ps[m];
        DevState* st = P.st;
        int* const lists[GROW_LISTS] = {P.act, P.deact, P.inact, P.strips};
        for (int q = 0; q < GROW_LISTS; q++) {
            const unsigned bal = __ballot_sync(0xffffffffu, t.f[q]) & half;
            int base = 0;
            if (lane == leader && bal) base = atomicAdd(&st->appendCnt[q], __popc(bal));
            base = __shfl_sync(0xffffffffu, base, leader);
            if (t.f[q]) lists[q][base + __popc(bal & ((1u << lane) - 1u))] = q == 3 ? t.strip : t.b;
        }
        // cells of the scheduled tiles and stale speeds, per half-warp
        unsigned long long cells = t.f[0] ? (unsigned long long)t.cells : 0ull;
        float smx = 0.f, smy = 0.f;
        if (t.b >= 0) {
            if (t.v && t.cells == 0) {
                P.mx[t.b] = 0.f;
                P.my[t.b] = 0.f;
            }
            if (!t.v) {
                smx = P.mx[t.b];
                smy = P.my[t.b];
            }
            P.prevAct[t.b] = (uint8_t)(t.v ? 1 : 0);
        }
        for (int o = 8; o > 0; o >>= 1) {
            cells += __shfl_xor_sync(0xffffffffu, cells, o);
            smx = fmaxf(smx, __shfl_xor_sync(0xffffffffu, smx, o));
            smy = fmaxf(smy, __shfl_xor_sync(0xffffffffu, smy, o));
        }
        if (lane == leader && gs < s1) {
            if (cells) atomicAdd(&st->appendCells, cells);
            if (smx > 0.f) atomicMax(&st->staleBits[0], __float_as_uint(smx));
            if (smy > 0.f) atomicMax(&st->staleBits[1], __float_as_uint(smy));
        }
    }
}

// The ensemble's step loop (one cooperative launch).
__global__ void __launch_bounds__(NT, 4) k_ensemble(EnsArgs E) {
    __shared__ StageSmem S;
    __shared__ EnsSmem Q;
    const int tid = threadIdx.x, n = E.n;
    EnsDev* D = E.dev;
    if (tid == 0) {
        mbar_init(&S.bar[0], 1);
        mbar_init(&S.bar[1], 1);
        fence_mbar_init();
    }
    __syncthreads();
    uint32_t ph[2] = {0u, 0u};
    unsigned barTarget = 0u;
    DevState* st0 = E.Ps[0].st;  // barrier timeouts are recorded in member 0
    if (blockIdx.x == 0 && tid == 0) D->t0 = globalTimerNs();  // before any member can finish
#define ENS_SYNC()                               \
    if (!gridSync(&D->bar, barTarget, st0)) return; \
    (void)0
    for (int step = 0;; step++) {
        const int cur = step & 1;
        if (D->nAlive[cur] == 0) return;  // every CTA reads the same count
        const int* live = D->live[cur];
        // ---- T: re-wet tracking of the members with gridded rain or surge
        // (a member without an inactive list -- last stepped by the
        // persistent loop's tile table -- scans its tiles instead)
        ensPrefix(n, [&](int m) {
            if (!live[m] || !(E.Ps[m].flags & (F_RAIN_G | F_SURGE))) return 0;
            const int k = E.Ps[m].st->nInact;
            return k >= 0 ? k : E.Ps[m].gridSize - 1;
        }, Q.offs);
        if (Q.offs[n] > 0) {  // the same total in every CTA
            for (int g = blockIdx.x; g < Q.offs[n]; g += gridDim.x) {
                const int m = ensMember(Q.offs, n, g);
                const Params& P = E.Ps[m];
                float fac0, fac2;
                trackFactors(P, fac0, fac2);
                const bool listed = P.st->nInact >= 0;
                const int b = listed ? P.inact[g - Q.offs[m]] : g - Q.offs[m] + 1;
                if (listed || !P.prevAct[b]) trackTile(P, b, fac0, fac2);
            }
            ENS_SYNC();
        }
        // ---- G: start of step (one warp per member), grow, stale maxima
        // the other parity's count was last read at the previous step's top
        if (tid == 0 && blockIdx.x == 0) D->nAlive[cur ^ 1] = 0;
        const int gw = blockIdx.x * (NT / 32) + (tid >> 5);
        for (int m = gw; m < n; m += gridDim.x * (NT / 32))
            if (live[m]) beginStep(E.Ps[m], E.Ps[m].st);
        ensPrefix(n, [&](int m) { return live[m] ? E.Ps[m].nSX * E.Ps[m].nSY : 0; }, Q.offs);
        ensGrow(E, Q.offs);
        ENS_SYNC();
        // ---- S: the stage-1 fluxes of the scheduled tiles give the tile
        // speeds, and each cell's divergence (bed-slope source folded in)
        // waits in the member's divergence planes for the update after dt;
        // U* re-sync of the deactivated tiles (the counts are final after the
        // barrier)
        ensPrefix(n, [&](int m) { return live[m] ? E.Ps[m].st->appendCnt[0] : 0; }, Q.offs);
        ensPrefix(n, [&](int m) { return live[m] ? E.Ps[m].st->appendCnt[1] : 0; }, Q.offs2);
        if (!ensTileLoop(S, E, Q.offs, 0, ph, [](int, int) {},
                         [&](int m, int tile, const TileBuf& T) {
                             const Params& P = E.Ps[m];
                             int bX, bY, i0, j0;
                             tileOrigin(P, tile, bX, bY, i0, j0);
                             float dh, dhu, dhv, spx, spy;
                             tileFluxDiv<true>(S, T, P, i0, j0, dh, dhu, dhv, spx, spy);
                             const int tx = tid % TW, ty = tid / TW;
                             if (tid < TH * TW && i0 + tx <= P.nx - 3 && j0 + ty <= P.ny - 3) {
                                 const int rr = ty + 2, cc = tx + 2;
                                 const float hC = T.in[0][rr][cc];
                                 const size_t c = cidx(P, 0, j0 + ty, i0 + tx);
                                 const size_t pl = (size_t)P.planeSize;
                                 P.D[c] = dh;
                                 P.D[c + pl] =
                                     dhu + bedSourceX(P, hC, T.e[0][rr][cc], T.e[1][rr][cc]);
                                 P.D[c + 2 * pl] =
                                     dhv + bedSourceY(P, hC, T.e[2][rr][cc], T.e[3][rr][cc]);
                             }
                             const float mxv = blockMax(spx, S.red[0]);
                             const float myv = blockMax(spy, S.red[1]);
                             if (tid == 0) {
                                 P.mx[tile] = mxv;
                                 P.my[tile] = myv;
                                 atomicMax(&P.st->max_bits[0], __float_as_uint(mxv));
                                 atomicMax(&P.st->max_bits[1], __float_as_uint(myv));
                             }
                         }))
            return;
        for (int g = blockIdx.x; g < Q.offs2[n]; g += gridDim.x) {
            const int m = ensMember(Q.offs2, n, g);
            resyncTile(E.Ps[m], E.Ps[m].deact[g - Q.offs2[m]]);
        }
        ENS_SYNC();
        // ---- D: dt of each member, list sizes, liveness of its next step
        for (int m = blockIdx.x * NT + tid; m < n; m += gridDim.x * NT) {
            int next = 0;
            if (live[m]) {
                const Params& P = E.Ps[m];
                DevState* st = P.st;
                const float mx = fmaxf(__uint_as_float(st->max_bits[0]),
                                       __uint_as_float(st->staleBits[0]));
                const float my = fmaxf(__uint_as_float(st->max_bits[1]),
                                       __uint_as_float(st->staleBits[1]));
                computeDt(P, st, (double)mx, (double)my);
                // the step's stage constants, once per member (the FP64
                // conversions stay out of the tile loops)
                D->consts[m][0] = stageConsts<1>(P);
                D->consts[m][1] = stageConsts<2>(P);
                st->staleBits[0] = st->staleBits[1] = 0u;
                st->nActive = st->appendCnt[0];
                st->nDeact = st->appendCnt[1];
                st->nInact = st->appendCnt[2];
                st->nStrips = st->appendCnt[3];
                st->appendCnt[0] = st->appendCnt[1] = st->appendCnt[2] = st->appendCnt[3] = 0;
                st->activeCells += st->appendCells;
                st->appendCells = 0ull;
                next = (st->t < st->t_stop && st->steps_done < E.maxSteps) ? 1 : 0;
                if (!next) st->stop = 1;
            }
            D->live[cur ^ 1][m] = next;
            if (next) atomicAdd(&D->nAlive[cur ^ 1], 1);
        }
        ENS_SYNC();
        // ---- 1: the rest of RK stage 1 of every scheduled tile, one thread
        // per cell, from U^n and the stored divergence (no staged block)
        ensPrefix(n, [&](int m) { return live[m] ? E.Ps[m].st->nActive : 0; }, Q.offs);
        for (int g = blockIdx.x; g < Q.offs[n]; g += gridDim.x) {
            const int m = ensMember(Q.offs, n, g);
            const Params& P = E.Ps[m];
            const StageConsts& C = D->consts[m][0];
            const int tile = P.act[g - Q.offs[m]];
            int bX, bY, i0, j0;
            tileOrigin(P, tile, bX, bY, i0, j0);
            const int tx = tid % TW, ty = tid / TW, i = i0 + tx, j = j0 + ty;
            const bool edge = i0 == 2 || j0 == 2 || i0 + TW - 1 >= P.nx - 3 || j0 + TH - 1 >= P.ny - 3;
            bool wet = false;
            if (tid < TH * TW && i <= P.nx - 3 && j <= P.ny - 3) {
                const size_t c = cidx(P, 0, j, i);
                const size_t pl = (size_t)P.planeSize;
                const float d0 = P.D[c], d1 = P.D[c + pl], d2 = P.D[c + 2 * pl];
                const float h = P.A[c], hu = P.A[c + pl], hv = P.A[c + 2 * pl];
                const float pre1[1] = {P.nman[c]};
                prefetchMaps(P, C.fl, c);
                wet = cellUpdate<1, false, false>(P, C, tile, j, i, d0, d1, d2, h, hu, hv, 0.f,
                                                  0.f, 0.f, 0.f, pre1, edge);
            }
            if (C.euler) {  // Euler mode: the tile wet flags come from this stage
                const bool any = __syncthreads_or(wet);
                if (tid == 0) P.wet[tile] = (uint8_t)((!(C.fl & F_TILE_ACC)) || any);
            }
        }
        ENS_SYNC();
        float pre[6];
        // ---- 2: RK stage 2 of the RK members, the commit of the Euler ones
        ensPrefix(n, [&](int m) { return live[m] && !(E.Ps[m].flags & F_EULER) ? E.Ps[m].st->nActive : 0; },
                  Q.offs);
        ensPrefix(n, [&](int m) { return live[m] && (E.Ps[m].flags & F_EULER) ? E.Ps[m].st->nActive : 0; },
                  Q.offs2);
        if (!ensTileLoop(S, E, Q.offs, 1, ph,
                         [&](int m, int tile) {
                             const Params& P = E.Ps[m];
                             int bX, bY, i0, j0;
                             tileOrigin(P, tile, bX, bY, i0, j0);
                             tilePrefetch<2>(P, D->consts[m][1], i0, j0, pre);
                         },
                         [&](int m, int tile, const TileBuf& T) {
                             const Params& P = E.Ps[m];
                             const StageConsts& C = D->consts[m][1];
                             int bX, bY, i0, j0;
                             tileOrigin(P, tile, bX, bY, i0, j0);
                             float dh, dhu, dhv, spx, spy;
                             tileFluxDiv<true>(S, T, P, i0, j0, dh, dhu, dhv, spx, spy);
                             const bool wet =
                                 tileCellUpdate<2>(P, C, T, tile, i0, j0, dh, dhu, dhv, pre);
                             tileFlags<2>(P, C, S, tile, wet, spx, spy);
                         }))
            return;
        for (int g = blockIdx.x; g < Q.offs2[n]; g += gridDim.x) {
            const int m = ensMember(Q.offs2, n, g);
            commitTile(E.Ps[m], E.Ps[m].act[g - Q.offs2[m]]);
        }
        ENS_SYNC();
        // members whose last step this iteration was: its end on the device clock
        for (int m = blockIdx.x * NT + tid; m < n; m += gridDim.x * NT)
            if (live[m] && !D->live[cur ^ 1][m]) D->tDone[m] = globalTimerNs();
    }
#undef ENS_SYNC
}

}  // namespace rift
