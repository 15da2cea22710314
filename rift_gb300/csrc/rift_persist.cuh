// rift_persist.cuh -- the whole step loop in one cooperative launch.
//
// For a small or mostly dry grid the step is a chain of short phases, and
// separate kernel launches spend more time starting and draining than
// working.  k_persist runs many steps in one cooperative launch (all CTAs
// resident), the phases separated by grid barriers:
//   [track]  re-wet inactive tiles under gridded rain / surge
//   grow     each CTA appends the list entries of its chunk of strips; every
//            CTA reads the counts after the barrier (rift_grow.cuh)
//   speed    tile speeds of U^n, dt and t (last CTA), U* re-sync
//   stage 1  RK stage 1 (per-tile code of k_stage<1>)
//   stage 2  RK stage 2, or the Euler commit
// With at most one scheduled tile per CTA (the usual case for a sparse
// grid) a step is shorter:
//   flux     the stage-1 fluxes of the CTA's tile give its speeds; the
//            divergence waits in registers, the stage-1 sources are computed
//            between the CTA's arrival at the dt barrier and its wait
//   update   dt in every CTA, the rest of the stage-1 update
//   stage 2  after a wait on the 4 edge neighbours' stage-1 flags, not a
//            grid barrier
// and, without tracking in RK2 mode, the tile table keeps each tile on its
// CTA from step to step so the grow phase and its barrier go away (see
// below).  The phases run the same device functions as the per-tile
// kernels, so the results are identical.  The kernel leaves at a step
// boundary when t >= t_stop, after the requested number of steps, or when
// the active set has outgrown P.persistMax (the host then continues with
// the per-step launches, whose march kernels suit a dense grid).
//
// Every wait is bounded: a grid barrier or a neighbour wait gives up after
// 2^22 polls, records ERR_BARRIER_TIMEOUT and the kernel returns; no TMA
// copy is in flight at a barrier (each tile loop consumes every load it
// issues).
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
    // step reductions of the fused steps, by step parity: a step's values
    // are cleared during the next step, when no CTA can still read them
    unsigned maxb[2][2];   // speed maxima of the scheduled tiles (bits)
    unsigned staleb[2][2]; // stale speed maxima of the inactive tiles (bits)
    int ownedCnt[2];       // owned tiles found active
    int schedCnt[2];       // scheduled tiles found by the scan
    int freeTop;           // entries of freeStack
    float nextRates[6];    // the next step's source rates and series state (spare CTA)
    // (the tables below are written before they are read in every launch:
    // only the part above is cleared, GRIDBAR_CLEAR bytes)
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
//
// A CTA may raise an event at a barrier (`raise`): its arrival adds
// BAR_EVENT + 1.  Every CTA leaves with the number of events raised there
// (*events): no barrier passes before every arrival is counted, and the
// arrivals at the next barrier that a slow poller may also see add less
// than BAR_EVENT in all (they raise nothing: the caller raises events at
// one barrier only, never at the one after it).  The event count then moves
// into `target`, so later barriers see none.
constexpr size_t GRIDBAR_CLEAR = offsetof(GridBar, slotTile);  // bytes cleared before a launch
constexpr unsigned BAR_EVENT = 1u << 16;  // > any grid (PERSIST_MAX_CTAS)
static_assert(BAR_EVENT > (unsigned)PERSIST_MAX_CTAS, "event unit above the arrivals");

__device__ bool gridSync(GridBar* gb, unsigned& target, DevState* st, bool raise = false,
                         int* events = nullptr) {
    __shared__ int sEvents;
    __syncthreads();
    int ok = 1;
    if (threadIdx.x == 0) {
        target += gridDim.x;
        red_add_release_gpu(&gb->count[0], raise ? BAR_EVENT + 1u : 1u);
        ok = 0;
        unsigned v = 0u;
        for (int it = 0; it < (1 << 22); ++it) {
            v = ld_acquire_gpu(&gb->count[0]);
            if ((int)(v - target) >= 0) {
                ok = 1;
                break;
            }
            __nanosleep(20);
        }
        fence_proxy_async_global();
        if (!ok) atomicOr(&st->error, ERR_BARRIER_TIMEOUT);
        const unsigned k = ok ? (v - target) / BAR_EVENT : 0u;
        target += k * BAR_EVENT;
        sEvents = (int)k;
    }
    ok = __syncthreads_and(ok);
    if (events) *events = sEvents;
    return ok != 0;
}

// The same barrier in two halves, so a CTA can work on its own data between
// its arrival and the wait: gridArrive after the CTA's writes that others
// read, gridWait before it reads theirs.  Between the halves the CTA writes
// nothing that another CTA reads.
__device__ __forceinline__ void gridArrive(GridBar* gb, unsigned& target) {
    __syncthreads();
    if (threadIdx.x == 0) {
        target += gridDim.x;
        red_add_release_gpu(&gb->count[0], 1u);
    }
}

__device__ bool gridWait(GridBar* gb, unsigned& target, DevState* st) {
    int ok = 1;
    if (threadIdx.x == 0) {
        ok = 0;
        unsigned v = 0u;
        for (int it = 0; it < (1 << 22); ++it) {
            v = ld_acquire_gpu(&gb->count[0]);
            if ((int)(v - target) >= 0) {
                ok = 1;
                break;
            }
            __nanosleep(20);
        }
        fence_proxy_async_global();
        if (!ok) atomicOr(&st->error, ERR_BARRIER_TIMEOUT);
        const unsigned k = ok ? (v - target) / BAR_EVENT : 0u;  // no events here; keep the count
        target += k * BAR_EVENT;
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
// CTA voids the table (an event at the barrier after stage 2): the loop
// returns to the grow, and rebuilds the table from the grow's list once the
// active set fits the grid again.

// Rebuild, after the grow's barrier (thread 0): CTA c takes act[c] or joins
// the free stack.
__device__ __forceinline__ void tableBuild(const Params& P, int nAct, int tile) {
    GridBar* T = P.gbar;
    const int c = blockIdx.x;
    T->slotTile[c] = tile;
    if (tile >= 0)
        P.owner[tile] = c;
    else
        T->freeStack[gridDim.x - 1 - c] = c;  // claims pop the lowest free CTA first
    if (c == 0) T->freeTop = (int)gridDim.x - nAct;
}

// Table step, flux phase: active flags, stale speeds, zero speeds of active
// tiles without interior cells, U* re-sync of deactivated tiles and the
// scheduled count over this CTA's chunk of tiles (what the grow does, less
// the lists), into staleDst[2] and *schedDst.  deList/deCount: shared
// scratch (NT entries, count 0).
// The scan runs on CTAs rank 0 .. nRank-1 of the scanners.
__device__ void scanTiles(const Params& P, unsigned* staleDst, int* schedDst, int* deList,
                          int* deCount, int rank, int nRank) {
    DevState* s = P.st;
    const int tid = threadIdx.x, lane = tid & 31;
    const int per = (P.gridSize + nRank - 1) / nRank;
    const int b0 = min(P.gridSize, rank * per), b1 = min(P.gridSize, b0 + per);
    int sched = 0;
    unsigned long long cells = 0ull;
    float smx = 0.f, smy = 0.f;
    for (int base = b0; base < b1; base += blockDim.x) {
        const int b = base + tid;
        bool de = false;
        if (b < b1) {
            // every load of the tile issued before any is used
            const bool was = P.prevAct[b] != 0;
            const float mxb = P.mx[b], myb = P.my[b];
            const bool v = tileGrows(P, b);
            const int nc = tileCells(P, b);
            de = was && !v;
            if (v && nc > 0) {
                sched++;
                cells += (unsigned long long)nc;
            }
            if (v && nc == 0) {
                P.mx[b] = 0.f;
                P.my[b] = 0.f;
            }
            if (!v) {  // stale speeds count for dt (A5)
                smx = fmaxf(smx, mxb);
                smy = fmaxf(smy, myb);
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
        if (sched) atomicAdd(schedDst, sched);
        if (cells) atomicAdd(&s->appendCells, cells);
        if (smx > 0.f) atomicMax(&staleDst[0], __float_as_uint(smx));
        if (smy > 0.f) atomicMax(&staleDst[1], __float_as_uint(smy));
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
__device__ __forceinline__ void tableClaim(const Params& P, int tile, int* overflow) {
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
        *overflow = 1;  // raised as an event at the barrier after stage 2
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
// Stage 1 -> stage 2 of the fused steps (RK2): a tile's stage 2 reads U*
// of its 4 edge neighbours only (2 cells deep; the ghost cells in that band
// are written by the tile itself or by those neighbours), so instead of a
// grid barrier each CTA publishes its tile's stage-1 completion and waits
// for the neighbours scheduled this step.  Thread q < 4 waits for
// neighbour q; bounded like every wait.
__device__ __forceinline__ void st_release_gpu(int* p, int v) {
    asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

__device__ __forceinline__ bool waitNeighbour(const Params& P, int tile, int q, int epoch) {
    const int bX = tile % P.nBX, bY = tile / P.nBX;
    int nb = -1;
    if (q == 0 && bX > 0) nb = tile - 1;
    if (q == 1 && bX < P.nBX - 1) nb = tile + 1;
    if (q == 2 && bY > 0) nb = tile - P.nBX;
    if (q == 3 && bY < P.nBY - 1) nb = tile + P.nBX;
    if (nb < 0 || !P.prevAct[nb] || tileCells(P, nb) == 0) return true;  // not scheduled
    for (int it = 0; it < (1 << 22); ++it) {
        if ((int)ld_acquire_gpu((const unsigned*)&P.tileFlag[nb]) >= epoch) return true;
        __nanosleep(20);
    }
    return false;
}

template <uint32_t FIX = 0>
__global__ void __launch_bounds__(NT, 4) k_persist(const __grid_constant__ CUtensorMap tmA,
                                                const __grid_constant__ CUtensorMap tmB,
                                                const __grid_constant__ CUtensorMap tmE, Params P,
                                                int maxSteps) {
    __shared__ StageSmem S;
    __shared__ bool last;
    __shared__ StageConsts sC[2];
    __shared__ double sDt;
    __shared__ int deList[NT];
    __shared__ int deCount;
    __shared__ int sFail;
    __shared__ int sSched;
    __shared__ int sOverflow;  // a claim of this CTA found no free CTA
    __shared__ StepRates sRates;  // this step's source rates (every CTA computes them)
    __shared__ StageConsts sPre;  // stage-1 constants without the step's dt
    __shared__ CellSrc sSrc[NT];  // stage-1 sources of each thread's cell
    DevState* st = P.st;
    GridBar* const T = P.gbar;
    const int tid = threadIdx.x;
    const uint32_t fl = P.flags;
    const bool track = (fl & (F_RAIN_G | F_SURGE)) != 0;
    const bool euler = (fl & F_EULER) != 0;
    const bool tableOk = !track && !euler && P.owner != nullptr;
    const bool spare = blockIdx.x == gridDim.x - 1;
    const bool led = (cellFlags<FIX>(fl) & F_CHECKVOL) != 0;  // check_volume ledger
    Led L;
    ledZero(L);
    tileInit(S, &tmA, &tmE);
    if (tid == 0) {
        prefetch_tmap(&tmB);
        deCount = 0;
        sOverflow = 0;
    }
    uint32_t ph[2] = {0u, 0u};
    unsigned barTarget = 0u;
    int nActPrev = 0;
    bool table = false;  // the tile table is valid (same in every CTA)
    int myTile = -1;     // table steps: the tile this CTA held through the last step
    int nScan = 1;       // table steps: CTAs of the scan (the last nScan)
    // t as every CTA computes it (st->t gets the same FP64 sum); t_stop is
    // fixed for the launch
    double tNow = st->t;
    double dtPrev = st->dt;  // the previous step's dt (stage-1 source clamps)
    bool haveNext = false;   // nextRates holds this step's rates (after a fused step)
    const double tStop = st->t_stop;
    int stepsDone = st->steps_done, tableSteps = st->tableSteps;  // used by CTA 0
    if (blockIdx.x == 0 && tid == 0) st->persistExit = 0;
#define RIFT_SYNC()                          \
    if (!gridSync(P.gbar, barTarget, st)) return; \
    (void)0
    for (int step = 0; step < maxSteps; step++) {
        if (tNow >= tStop) {
            if (blockIdx.x == 0 && tid == 0) st->stop = 1;
            return;
        }
        if (step > 0 && nActPrev > P.persistMax) {
            if (blockIdx.x == 0 && tid == 0) st->persistExit = 1;
            return;
        }
        const int par = step & 1;  // parity of this step's reductions
        if (track) {
            trackTiles(P);
            RIFT_SYNC();
        }
        int nAct, nDe = 0, tile = -1;
        bool built = false;
        if (table) {
            if (blockIdx.x == 0 && tid == 0) {  // counters kept in registers: no load
                st->stop = 0;
                st->steps_done = ++stepsDone;
                st->ticket = 0u;
                st->tableSteps = ++tableSteps;
            }
            // a CTA that kept its tile still holds it (claims take free CTAs
            // only); a free CTA looks whether a claim gave it one
            tile = myTile >= 0 ? myTile : T->slotTile[blockIdx.x];
            nAct = 0;  // not needed: every scheduled tile holds a CTA
        } else {
            if (blockIdx.x == 0 && tid == 0) {
                beginStepResets(st);
                stepsDone++;
            }
            growAppend<false>(P, T->staleb[par]);
            for (int b = blockIdx.x * NT + tid; b < P.gridSize; b += gridDim.x * NT) {
                P.tileFlag[b] = 0;
                if (tableOk) P.owner[b] = -1;
            }
            RIFT_SYNC();
            nAct = (int)ld_relaxed_gpu((const unsigned*)&st->appendCnt[0]);
            nDe = (int)ld_relaxed_gpu((const unsigned*)&st->appendCnt[1]);
            if (nAct <= (int)gridDim.x) {
                tile = (int)blockIdx.x < nAct ? P.act[blockIdx.x] : -1;
                if (tableOk) {
                    if (tid == 0) tableBuild(P, nAct, tile);
                    built = true;
                    const int freeCtas = (int)gridDim.x - nAct;
                    nScan = freeCtas >= 32 ? freeCtas : (int)gridDim.x;
                }
                myTile = tile;
            }
        }
        if (table || nAct <= (int)gridDim.x) {
            // At most one tile per CTA: stage 1's fluxes of U^n are the first
            // ComputeFluxes of the step, so they give this step's tile speeds,
            // and the tile's divergence waits in registers (its staged block
            // in shared memory) across the barrier.  After the barrier every
            // CTA computes the step's dt from the maxima itself; the spare CTA
            // publishes it during stage 2, when no CTA reads the old value.
            bool mine = tile >= 0;
            int bX, bY, i0 = 0, j0 = 0;
            float pre[6], dh = 0.f, dhu = 0.f, dhv = 0.f, spx = 0.f, spy = 0.f, bin1 = 0.f;
            if (tid == 0 && mine) issueTile(S.buf[0], &S.bar[0], &tmA, &tmE, P, tile);
            bool wetOld = false, live = true;
            if (mine) {
                tileOrigin(P, tile, bX, bY, i0, j0);
                tilePrefetch<1>(P, stageConsts<1>(P), i0, j0, pre);
                wetOld = P.wet[tile] != 0;
                if (table) live = tileGrows(P, tile);
            }
            // the scan runs on the CTAs that were free at the rebuild (the
            // highest ones; claims take the lowest free CTA first), so the
            // tile CTAs' flux phase does not wait for it
            if (table && (int)blockIdx.x >= (int)gridDim.x - nScan)
                scanTiles(P, T->staleb[par], &T->schedCnt[par], deList, &deCount,
                          (int)blockIdx.x - ((int)gridDim.x - nScan), nScan);
            if (mine) {
                const bool ok = mbar_wait_bounded(&S.bar[0], ph[0]);
                if (!__syncthreads_and(ok)) {
                    mbar_wait_bounded(&S.bar[0], ph[0]);
                    if (tid == 0) atomicOr(&st->error, ERR_TMA_TIMEOUT);
                    return;
                }
                ph[0] ^= 1u;
                if (live) {
                    tileFluxDiv<true>(S, S.buf[0], P, i0, j0, dh, dhu, dhv, spx, spy,
                                      led ? &bin1 : nullptr);
                    const float mxv = blockMax(spx, S.red[0]);
                    const float myv = blockMax(spy, S.red[1]);
                    if (tid == 0) {
                        P.mx[tile] = mxv;
                        P.my[tile] = myv;
                        atomicMax(&T->maxb[par][0], __float_as_uint(mxv));
                        atomicMax(&T->maxb[par][1], __float_as_uint(myv));
                        if (table) atomicAdd(&T->ownedCnt[par], 1);
                    }
                    __syncthreads();
                } else {
                    if (tid == 0) tableRelease(P, tile);
                    mine = false;
                }
                myTile = mine ? tile : -1;
            }
            // this step's source rates: computed by the spare CTA during the
            // last step's stage 2, or here in every CTA on the first fused
            // step of the launch (warp 1); the spare writes them to the device
            // state during stage 2, when no CTA reads the series state any more
            if (haveNext) {
                if (tid == 32) {
                    const float* r = T->nextRates;
                    StepRates q;
                    q.rainU = r[0];
                    q.drainU = r[1];
                    q.srcR = r[2];
                    q.interp[0] = r[3];
                    q.interp[1] = r[4];
                    q.interp[2] = r[5];
                    sRates = q;
                }
            } else if (tid >= 32 && tid < 64) {
                const StepRates q = stepRates(P, st, tNow);
                if (tid == 32) sRates = q;
            }
            if (!table) resyncDeactivated(P, nDe);
            // split barrier: the stage-1 sources (no dt needed) are computed
            // between this CTA's arrival and its wait
            gridArrive(P.gbar, barTarget);
            if (tid == 0) {
                StageConsts c = stageConstsAt<1>(P, dtPrev, dtPrev, tNow);
                c.rainU = sRates.rainU;
                c.drainU = sRates.drainU;
                c.srcR = sRates.srcR;
                sPre = c;
            }
            __syncthreads();
            // (kept in shared memory across the wait: registers stay free)
            if (mine) sSrc[tid] = tileCellSources<1, FIX>(P, sPre, S.buf[0], tile, i0, j0, dh, dhu, dhv, pre);
            if (!gridWait(P.gbar, barTarget, st)) return;
            // dt of this step (Simulator::ComputeTimestep), by thread 0 of
            // every CTA; the FP64 arithmetic stays in one thread
            if (tid == 0) {
                const unsigned mx0 = ld_relaxed_gpu(&T->maxb[par][0]);
                const unsigned my0 = ld_relaxed_gpu(&T->maxb[par][1]);
                const unsigned mx1 = ld_relaxed_gpu(&T->staleb[par][0]);
                const unsigned my1 = ld_relaxed_gpu(&T->staleb[par][1]);
                int fail = 0, sched = nAct;
                if (table) {
                    const int owned = (int)ld_relaxed_gpu((const unsigned*)&T->ownedCnt[par]);
                    sched = (int)ld_relaxed_gpu((const unsigned*)&T->schedCnt[par]);
                    fail = owned != sched;
                }
                const double dtNew = stepDtAt(P, tNow, __uint_as_float(max(mx0, mx1)),
                                              __uint_as_float(max(my0, my1)));
                const double tNew = tNow + dtNew;
                StageConsts c1 = stageConstsAt<1>(P, dtNew, dtPrev, tNew);
                StageConsts c2 = stageConstsAt<2>(P, dtNew, dtPrev, tNew);
                c1.rainU = c2.rainU = sRates.rainU;
                c1.drainU = c2.drainU = sRates.drainU;
                c1.srcR = c2.srcR = sRates.srcR;
                sC[0] = c1;
                sC[1] = c2;
                sDt = dtNew;
                sFail = fail;
                sSched = sched;
                if (fail && blockIdx.x == 0) atomicOr(&st->error, ERR_TILE_TABLE);
            }
            __syncthreads();
            if (sFail) return;  // every CTA read the same counts
            tNow = sC[1].tNew;
            dtPrev = sDt;
            nActPrev = sSched;
            if (mine) {  // the rest of the stage-1 update with this step's dt (Integrate_1_k)
                const StageConsts C1 = sC[0];
                L.v[LED_BOUND] += C1.wRate * bin1;
                const bool wetCell = tileCellFinish<1, FIX>(P, C1, S.buf[0], i0, j0, sSrc[tid], pre,
                                                            led ? &L : nullptr);
                tileFlags<1>(P, C1, S, tile, wetCell, 0.f, 0.f);
                __syncthreads();
            }
            if (!euler) {
                if (mine) {
                    // publish this tile's U*, wait for the scheduled neighbours'
                    if (tid == 0) st_release_gpu(&P.tileFlag[tile], step + 1);
                    const bool okN = tid < 4 ? waitNeighbour(P, tile, tid, step + 1) : true;
                    if (!__syncthreads_and(okN)) {
                        if (tid == 0) atomicOr(&st->error, ERR_BARRIER_TIMEOUT);
                        return;
                    }
                    // stage 2 of the same tile: its U* block into the second buffer
                    if (tid == 0) {
                        fence_proxy_async_global();
                        issueTile(S.buf[1], &S.bar[1], &tmB, &tmE, P, tile);
                    }
                    const StageConsts C2 = sC[1];
                    tilePrefetch<2>(P, C2, i0, j0, pre);
                    const bool ok = mbar_wait_bounded(&S.bar[1], ph[1]);
                    if (!__syncthreads_and(ok)) {
                        mbar_wait_bounded(&S.bar[1], ph[1]);
                        if (tid == 0) atomicOr(&st->error, ERR_TMA_TIMEOUT);
                        return;
                    }
                    ph[1] ^= 1u;
                    float sx2, sy2, bin2 = 0.f;
                    tileFluxDiv<true>(S, S.buf[1], P, i0, j0, dh, dhu, dhv, sx2, sy2,
                                      led ? &bin2 : nullptr);
                    L.v[LED_BOUND] += C2.wRate * bin2;
                    const bool wetCell = tileCellUpdate<2, FIX>(P, C2, S.buf[1], tile, i0, j0, dh, dhu,
                                                                dhv, pre, led ? &L : nullptr);
                    const bool wetNew = tileFlags<2>(P, C2, S, tile, wetCell, sx2, sy2);
                    if ((table || built) && wetNew && !wetOld && tid < 4)
                        tableClaim(P, tile, &sOverflow);
                    __syncthreads();
                }
            } else {
                RIFT_SYNC();
                commitTiles(P, nAct);
            }
            if (spare && tid < 32) {
                writeRates(P, st, sRates);
                // the next step's rates from this step's state, at its t
                const StepRates q = stepRatesFrom(P, sRates, tNow);
                if (tid == 0) {
                    float* r = T->nextRates;
                    r[0] = q.rainU;
                    r[1] = q.drainU;
                    r[2] = q.srcR;
                    r[3] = q.interp[0];
                    r[4] = q.interp[1];
                    r[5] = q.interp[2];
                }
            }
            if (spare && tid == 0) {
                publishDt(P, st, sDt);
                // the other parity: last read in the previous step
                T->maxb[par ^ 1][0] = T->maxb[par ^ 1][1] = 0u;
                T->staleb[par ^ 1][0] = T->staleb[par ^ 1][1] = 0u;
                T->ownedCnt[par ^ 1] = T->schedCnt[par ^ 1] = 0;
                if (table) {  // the scan's counts; the lists were not built
                    st->nActive = sSched;
                    st->nDeact = 0;
                    st->nInact = -1;
                    st->activeCells += st->appendCells;
                    st->appendCells = 0ull;
                } else {
                    publishGrow(st);
                }
            }
            if (led) flushLed(L, st->led);
            int voided = 0;
            if (!gridSync(P.gbar, barTarget, st, sOverflow != 0, &voided)) return;
            if (tid == 0) sOverflow = 0;
            table = (table || built) && voided == 0;
            haveNext = true;
            continue;
        }
        nActPrev = nAct;
        haveNext = false;
        // speeds of U^n, dt, t, U* re-sync (k_speed_dt), then stage 1; the
        // stale maxima of this step went to staleb[par]
        if (blockIdx.x == 0 && tid < 32) beginStepRates(P, st);
        float tmx = 0.f, tmy = 0.f;
        if (!speedTiles(S, &tmA, &tmE, P, nAct, ph, tmx, tmy)) return;
        if (tid == 0) {
            tmx = fmaxf(tmx, __uint_as_float(ld_relaxed_gpu(&T->staleb[par][0])));
            tmy = fmaxf(tmy, __uint_as_float(ld_relaxed_gpu(&T->staleb[par][1])));
        }
        __syncthreads();
        finishDt(P, tmx, tmy, &last);
        resyncDeactivated(P, nDe);
        RIFT_SYNC();
        if (tid == 0) {  // the stage constants, FP64 conversions in one thread
            sC[0] = stageConsts<1>(P);
            sC[1] = stageConsts<2>(P);
            sDt = st->dt;
        }
        __syncthreads();
        tNow = sC[1].tNew;  // published by finishDt before the barrier
        dtPrev = sDt;
        if (!stageTiles<1, FIX>(S, &tmA, &tmE, P, nAct, ph, &sC[0])) return;
        RIFT_SYNC();
        if (!euler) {
            if (!stageTiles<2, FIX>(S, &tmB, &tmE, P, nAct, ph, &sC[1])) return;
        } else {
            commitTiles(P, nAct);
        }
        if (spare && tid == 0) {
            T->maxb[par ^ 1][0] = T->maxb[par ^ 1][1] = 0u;
            T->staleb[par ^ 1][0] = T->staleb[par ^ 1][1] = 0u;
            T->ownedCnt[par ^ 1] = T->schedCnt[par ^ 1] = 0;
            publishGrow(st);
        }
        RIFT_SYNC();
    }
#undef RIFT_SYNC
}

}  // namespace rift
