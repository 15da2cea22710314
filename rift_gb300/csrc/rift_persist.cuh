// rift_persist.cuh -- the whole step loop in one cooperative launch.
//
// For a small or mostly dry grid the step is a chain of short phases, and
// separate kernel launches spend more time starting and draining than
// working.  k_persist runs many steps in one cooperative launch (all CTAs
// resident), the phases separated by a grid barrier:
//   [track]  re-wet inactive tiles under gridded rain / surge
//   grow     each CTA appends the list entries of its chunk of strips; the
//            last one publishes the counts (rift_grow.cuh)
//   speed    tile speeds of U^n, dt and t (last CTA), U* re-sync
//   stage 1  RK stage 1 (per-tile code of k_stage<1>)
// With at most one active tile per CTA, the speed and stage-1 phases become
// one flux phase (its fluxes give the speeds) and an update after the dt
// barrier, so a step has one tile-flux phase fewer.
//   stage 2  RK stage 2, or the Euler commit
// The phases run the same device functions as the per-tile kernels, so the
// results are identical.  The kernel leaves at a step boundary when
// t >= t_stop, after the requested number of steps, or when the active set
// has outgrown P.persistMax (the host then continues with the per-step
// launches, whose march kernels suit a dense grid).
//
// Every wait is bounded: a grid barrier gives up after 2^22 polls, records
// ERR_BARRIER_TIMEOUT and the kernel returns; no TMA copy is in flight at a
// barrier (each tile loop consumes every load it issues).
#pragma once
#include "rift_grow.cuh"
#include "rift_kernels.cuh"

namespace rift {

constexpr int PERSIST_MAX_CTAS = 4096;

// Grid barrier state: one arrival counter on its own 128-byte line; then
// the tile table of the persistent loop (cleared with the counter before
// every launch).
struct GridBar {
    unsigned count[32];
    int freeTop;    // entries of freeStack
    int overflow;   // a claim found no free CTA: the table is void
    int ownedCnt;   // owned tiles found active this step
    int schedCnt;   // scheduled tiles found by the scan this step
    int slotTile[PERSIST_MAX_CTAS];   // CTA -> its tile, or -1
    int freeStack[PERSIST_MAX_CTAS];  // CTAs without a tile
};

__device__ __forceinline__ unsigned ld_relaxed_gpu(const unsigned* p) {
    unsigned v;
    asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p));
    return v;
}

__device__ __forceinline__ unsigned ld_acquire_gpu(const unsigned* p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void red_add_release_gpu(unsigned* p, unsigned v) {
    asm volatile("red.release.gpu.global.add.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ void fence_proxy_async_global() {
    asm volatile("fence.proxy.async.global;" ::: "memory");
}

// Grid-wide barrier.  Every CTA adds 1 to a monotonic counter with release
// semantics and polls it with acquire loads until it reaches gridDim.x times
// the number of barriers passed (`target`), so no reset is needed and a CTA
// may arrive at the next barrier before the slowest one has left this one.
// After the barrier, TMA loads (async proxy) see the generic-proxy writes made
// before it.  Measured on GB300: 1.2 us for 152 CTAs, 2.1 us for 608.  False
// after the poll limit (error recorded).
__device__ bool gridSync(GridBar* gb, unsigned& target, DevState* st) {
    __syncthreads();
    int ok = 1;
    if (threadIdx.x == 0) {
        target += gridDim.x;
        red_add_release_gpu(&gb->count[0], 1u);
        ok = 0;
        for (int it = 0; it < (1 << 22); ++it) {
            if ((int)(ld_acquire_gpu(&gb->count[0]) - target) >= 0) {
                ok = 1;
                break;
            }
            __nanosleep(20);
        }
        fence_proxy_async_global();
        if (!ok) atomicOr(&st->error, ERR_BARRIER_TIMEOUT);
    }
    return __syncthreads_and(ok) != 0;
}

// ------------------------------------------------------------ tile table
// With one scheduled tile per CTA and no tracking (no gridded rain or surge)
// and RK2, the loop keeps the tile -> CTA assignment from step to step
// instead of compacting the active set behind a grid barrier:
//   - at the start of a step each CTA tests its own tile (active iff it or a
//     4-neighbour is wet, tile 0 always) and gives the tile up if inactive;
//   - in the same phase a scan over all tiles writes the active flags, folds
//     the stale speeds of inactive tiles, re-syncs U* on deactivated tiles
//     and counts the scheduled tiles;
//   - a tile that turns wet in stage 2 gives a CTA to each neighbour with
//     interior cells that holds none.  A tile becomes active only next to a
//     tile that just turned wet (the others were active already), so the
//     table holds the next step's scheduled set.
// The owned active tiles are counted against the scan every step (a
// mismatch is an error, never a silent result).  A claim that finds no free
// CTA voids the table: the loop returns to the grow, and rebuilds the table
// from the grow's list once the active set fits the grid again.

// Rebuild, grow phase: no tile holds a CTA.
__device__ __forceinline__ void tableClear(const Params& P) {
    for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < P.gridSize; b += gridDim.x * blockDim.x)
        P.owner[b] = -1;
}

// Rebuild, after the grow's barrier (thread 0): CTA c takes act[c] or joins
// the free stack.
__device__ __forceinline__ void tableBuild(const Params& P, int nAct, int tile) {
    GridBar* T = P.gbar;
    const int c = blockIdx.x;
    T->slotTile[c] = tile;
    if (tile >= 0)
        P.owner[tile] = c;
    else
        T->freeStack[c - nAct] = c;
    if (c == 0) {
        T->freeTop = (int)gridDim.x - nAct;
        T->overflow = 0;
        T->ownedCnt = 0;
        T->schedCnt = 0;
    }
}

// Table step, flux phase: active flags, stale speeds, zero speeds of active
// tiles without interior cells, U* re-sync of deactivated tiles and the
// scheduled count over this CTA's chunk of tiles (what the grow does, less
// the lists).  deList/deCount: shared scratch (NT entries, count 0).
__device__ void scanTiles(const Params& P, int* deList, int* deCount) {
    DevState* s = P.st;
    const int tid = threadIdx.x, lane = tid & 31;
    const int per = (P.gridSize + (int)gridDim.x - 1) / (int)gridDim.x;
    const int b0 = min(P.gridSize, (int)blockIdx.x * per), b1 = min(P.gridSize, b0 + per);
    int sched = 0;
    unsigned long long cells = 0ull;
    float smx = 0.f, smy = 0.f;
    for (int base = b0; base < b1; base += blockDim.x) {
        const int b = base + tid;
        bool de = false;
        if (b < b1) {
            const bool v = tileGrows(P, b);
            const int nc = tileCells(P, b);
            de = P.prevAct[b] && !v;
            if (v && nc > 0) {
                sched++;
                cells += (unsigned long long)nc;
            }
            if (v && nc == 0) {
                P.mx[b] = 0.f;
                P.my[b] = 0.f;
            }
            if (!v) {  // stale speeds count for dt (A5)
                smx = fmaxf(smx, P.mx[b]);
                smy = fmaxf(smy, P.my[b]);
            }
            P.prevAct[b] = (uint8_t)(v ? 1 : 0);
        }
        const int nde = __syncthreads_count(de);
        if (nde) {  // rare: re-sync U* on this round's deactivated tiles
            if (de) deList[atomicAdd(deCount, 1)] = b;
            __syncthreads();
            for (int k = 0; k < nde; k++) resyncTile(P, deList[k]);
            __syncthreads();
            if (tid == 0) *deCount = 0;
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        sched += __shfl_xor_sync(0xffffffffu, sched, o);
        cells += __shfl_xor_sync(0xffffffffu, cells, o);
        smx = fmaxf(smx, __shfl_xor_sync(0xffffffffu, smx, o));
        smy = fmaxf(smy, __shfl_xor_sync(0xffffffffu, smy, o));
    }
    if (lane == 0) {
        if (sched) atomicAdd(&P.gbar->schedCnt, sched);
        if (cells) atomicAdd(&s->appendCells, cells);
        if (smx > 0.f) atomicMax(&s->staleBits[0], __float_as_uint(smx));
        if (smy > 0.f) atomicMax(&s->staleBits[1], __float_as_uint(smy));
    }
}

// Table step, flux phase (thread 0): this CTA gives up its inactive tile.
__device__ __forceinline__ void tableRelease(const Params& P, int tile) {
    GridBar* T = P.gbar;
    P.owner[tile] = -1;
    T->slotTile[blockIdx.x] = -1;
    T->freeStack[atomicAdd(&T->freeTop, 1)] = blockIdx.x;
}

// Stage 2 (threads 0..3, one neighbour each): `tile` turned wet; each
// neighbour with interior cells and no CTA gets one from the free stack.
__device__ __forceinline__ void tableClaim(const Params& P, int tile) {
    const int q = threadIdx.x;
    const int bX = tile % P.nBX, bY = tile / P.nBX;
    int nb = -1;
    if (q == 0 && bX > 0) nb = tile - 1;
    if (q == 1 && bX < P.nBX - 1) nb = tile + 1;
    if (q == 2 && bY > 0) nb = tile - P.nBX;
    if (q == 3 && bY < P.nBY - 1) nb = tile + P.nBX;
    if (nb < 0 || tileCells(P, nb) == 0) return;
    if (atomicCAS(&P.owner[nb], -1, -2) != -1) return;  // held, or claimed by another tile
    GridBar* T = P.gbar;
    const int k = atomicSub(&T->freeTop, 1) - 1;
    if (k < 0) {
        atomicExch(&T->overflow, 1);
        return;
    }
    const int c = T->freeStack[k];
    P.owner[nb] = c;
    T->slotTile[c] = nb;
}

// The step loop.  maxSteps: steps to attempt in this launch.
//
// Work off the critical path goes to the spare CTA (the last one; it holds
// no tile when the grid is larger than the active set): the step's source
// rates during the flux phase, the dt bookkeeping and the grow's counts
// during stage 2.  Every CTA reads the grow's counters itself after the
// grow's barrier, so the grow needs no last-CTA hand-off.
__global__ void __launch_bounds__(NT, 4) k_persist(const __grid_constant__ CUtensorMap tmA,
                                                const __grid_constant__ CUtensorMap tmB,
                                                const __grid_constant__ CUtensorMap tmE, Params P,
                                                int maxSteps) {
    __shared__ StageSmem S;
    __shared__ bool last;
    __shared__ StageConsts sC[2];
    __shared__ double sDt;
    DevState* st = P.st;
    const int tid = threadIdx.x;
    const uint32_t fl = P.flags;
    const bool track = (fl & (F_RAIN_G | F_SURGE)) != 0;
    const bool spare = blockIdx.x == gridDim.x - 1;
    tileInit(S, &tmA, &tmE);
    if (tid == 0) prefetch_tmap(&tmB);
    uint32_t ph[2] = {0u, 0u};
    unsigned barTarget = 0u;
    int nActPrev = 0;
    if (blockIdx.x == 0 && tid == 0) st->persistExit = 0;
#define RIFT_SYNC()                          \
    if (!gridSync(P.gbar, barTarget, st)) return; \
    (void)0
    for (int step = 0; step < maxSteps; step++) {
        // every CTA reads the same t (written before the last barrier)
        if (st->t >= st->t_stop) {
            if (blockIdx.x == 0 && tid == 0) st->stop = 1;
            return;
        }
        if (step > 0 && nActPrev > P.persistMax) {
            if (blockIdx.x == 0 && tid == 0) st->persistExit = 1;
            return;
        }
        if (track) {
            trackTiles(P);
            RIFT_SYNC();
        }
        if (blockIdx.x == 0 && tid == 0) beginStepResets(st);
        growAppend<false>(P);
        RIFT_SYNC();
        const int nAct = (int)ld_relaxed_gpu((const unsigned*)&st->appendCnt[0]);
        const int nDe = (int)ld_relaxed_gpu((const unsigned*)&st->appendCnt[1]);
        nActPrev = nAct;
        if (nAct <= (int)gridDim.x) {
            // At most one tile per CTA: stage 1's fluxes of U^n are the first
            // ComputeFluxes of the step, so they give this step's tile speeds,
            // and the tile's divergence waits in registers (its staged block
            // in shared memory) across the barrier.  After the barrier every
            // CTA computes the step's dt from the maxima itself; the spare CTA
            // publishes it during stage 2, when no CTA reads the old value.
            const bool mine = (int)blockIdx.x < nAct;
            int tile = 0, bX, bY, i0 = 0, j0 = 0;
            float pre[6], dh = 0.f, dhu = 0.f, dhv = 0.f, spx = 0.f, spy = 0.f;
            // t and dt of the previous step: published before the last barrier
            double tCur = 0.0, dtOld = 0.0;
            if (tid == 0) {
                tCur = st->t;
                dtOld = st->dt;
            }
            tileFirst(S, &tmA, &tmE, P, nAct);
            if (mine) {
                tile = P.act[blockIdx.x];
                tileOrigin(P, tile, bX, bY, i0, j0);
                tilePrefetch<1>(P, stageConsts<1>(P), i0, j0, pre);
                if (!tileAcquire(S, &tmA, &tmE, P, 0, ph, nAct, nAct)) {
                    if (tid == 0) atomicOr(&st->error, ERR_TMA_TIMEOUT);
                    return;
                }
                tileFluxDiv<true>(S, S.buf[0], P, i0, j0, dh, dhu, dhv, spx, spy);
                const float mxv = blockMax(spx, S.red[0]);
                const float myv = blockMax(spy, S.red[1]);
                if (tid == 0) {
                    P.mx[tile] = mxv;
                    P.my[tile] = myv;
                    atomicMax(&st->max_bits[0], __float_as_uint(mxv));
                    atomicMax(&st->max_bits[1], __float_as_uint(myv));
                }
                __syncthreads();
            }
            if (spare && tid < 32) beginStepRates(P, st);
            resyncDeactivated(P, nDe);
            RIFT_SYNC();
            // dt of this step (Simulator::ComputeTimestep), by thread 0 of
            // every CTA; the FP64 arithmetic stays in one thread
            if (tid == 0) {
                const unsigned mx0 = ld_relaxed_gpu(&st->max_bits[0]);
                const unsigned my0 = ld_relaxed_gpu(&st->max_bits[1]);
                const unsigned mx1 = ld_relaxed_gpu(&st->staleBits[0]);
                const unsigned my1 = ld_relaxed_gpu(&st->staleBits[1]);
                const double dtNew = stepDtAt(P, tCur, (double)__uint_as_float(max(mx0, mx1)),
                                              (double)__uint_as_float(max(my0, my1)));
                const double tNew = tCur + dtNew;
                sC[0] = stageConstsAt<1>(P, dtNew, dtOld, tNew);
                sC[1] = stageConstsAt<2>(P, dtNew, dtOld, tNew);
                sDt = dtNew;
            }
            __syncthreads();
            if (mine) {  // stage-1 update with this step's dt (Integrate_1_k)
                const StageConsts C1 = sC[0];
                const bool wetCell =
                    tileCellUpdate<1>(P, C1, S.buf[0], tile, i0, j0, dh, dhu, dhv, pre);
                tileFlags<1>(P, C1, S, tile, wetCell, 0.f, 0.f);
                __syncthreads();
            }
            RIFT_SYNC();
            if (!(fl & F_EULER)) {
                // stage 2 of the same tile: its U* block into the second buffer
                if (mine) {
                    if (tid == 0) issueTile(S.buf[1], &S.bar[1], &tmB, &tmE, P, tile);
                    const StageConsts C2 = sC[1];
                    tilePrefetch<2>(P, C2, i0, j0, pre);
                    const bool ok = mbar_wait_bounded(&S.bar[1], ph[1]);
                    if (!__syncthreads_and(ok)) {
                        mbar_wait_bounded(&S.bar[1], ph[1]);
                        if (tid == 0) atomicOr(&st->error, ERR_TMA_TIMEOUT);
                        return;
                    }
                    ph[1] ^= 1u;
                    float sx2, sy2;
                    tileFluxDiv<true>(S, S.buf[1], P, i0, j0, dh, dhu, dhv, sx2, sy2);
                    const bool wetCell =
                        tileCellUpdate<2>(P, C2, S.buf[1], tile, i0, j0, dh, dhu, dhv, pre);
                    tileFlags<2>(P, C2, S, tile, wetCell, sx2, sy2);
                    __syncthreads();
                }
            } else {
                commitTiles(P, nAct);
            }
            if (spare && tid == 0) {
                publishDt(P, st, sDt);
                st->staleBits[0] = st->staleBits[1] = 0u;
                publishGrow(st);
            }
            RIFT_SYNC();
            continue;
        }
        // speeds of U^n, dt, t, U* re-sync (k_speed_dt), then stage 1
        if (blockIdx.x == 0 && tid < 32) beginStepRates(P, st);
        float tmx = 0.f, tmy = 0.f;
        if (!speedTiles(S, &tmA, &tmE, P, nAct, ph, tmx, tmy)) return;
        __syncthreads();
        finishDt(P, tmx, tmy, &last);
        resyncDeactivated(P, nDe);
        RIFT_SYNC();
        if (tid == 0) {  // the stage constants, FP64 conversions in one thread
            sC[0] = stageConsts<1>(P);
            sC[1] = stageConsts<2>(P);
        }
        __syncthreads();
        if (!stageTiles<1>(S, &tmA, &tmE, P, nAct, ph, &sC[0])) return;
        RIFT_SYNC();
        if (!(fl & F_EULER)) {
            if (!stageTiles<2>(S, &tmB, &tmE, P, nAct, ph, &sC[1])) return;
        } else {
            commitTiles(P, nAct);
        }
        if (spare && tid == 0) publishGrow(st);
        RIFT_SYNC();
    }
#undef RIFT_SYNC
}

}  // namespace rift
