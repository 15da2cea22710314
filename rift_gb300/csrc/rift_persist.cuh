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

// Grid barrier state: one arrival counter on its own 128-byte line.
struct GridBar {
    unsigned count[32];
};

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

// The step loop.  maxSteps: steps to attempt in this launch.
__global__ void __launch_bounds__(NT, 4) k_persist(const __grid_constant__ CUtensorMap tmA,
                                                const __grid_constant__ CUtensorMap tmB,
                                                const __grid_constant__ CUtensorMap tmE, Params P,
                                                int maxSteps) {
    __shared__ StageSmem S;
    __shared__ bool last;
    DevState* st = P.st;
    const int tid = threadIdx.x;
    const uint32_t fl = P.flags;
    const bool track = (fl & (F_RAIN_G | F_SURGE)) != 0;
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
        if (blockIdx.x == 0 && tid < 32) beginStep(P, st);
        growAppend(P);
        RIFT_SYNC();
        const int nAct = st->nActive;  // published by the grow's last CTA
        nActPrev = nAct;
        float tmx = 0.f, tmy = 0.f;
        if (nAct <= (int)gridDim.x) {
            // At most one tile per CTA: stage 1's fluxes of U^n are the first
            // ComputeFluxes of the step, so they give this step's tile speeds,
            // and the tile's divergence waits in registers (its staged block
            // in shared memory) across the barrier.  After the barrier every
            // CTA computes the step's dt from the maxima itself; CTA 0
            // publishes it during stage 2, when no CTA reads the old value.
            const bool mine = (int)blockIdx.x < nAct;
            int tile = 0, bX, bY, i0 = 0, j0 = 0;
            float pre[6], dh = 0.f, dhu = 0.f, dhv = 0.f, spx = 0.f, spy = 0.f;
            if (mine) {
                tile = P.act[blockIdx.x];
                tileOrigin(P, tile, bX, bY, i0, j0);
                tilePrefetch<1>(P, stageConsts<1>(P), i0, j0, pre);
            }
            tileFirst(S, &tmA, &tmE, P, nAct);
            if (mine) {
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
            resyncDeactivated(P);
            RIFT_SYNC();
            // dt of this step (Simulator::ComputeTimestep) in every CTA
            const unsigned bx = max(ld_acquire_gpu(&st->max_bits[0]), ld_acquire_gpu(&st->staleBits[0]));
            const unsigned by = max(ld_acquire_gpu(&st->max_bits[1]), ld_acquire_gpu(&st->staleBits[1]));
            const double dtOld = st->dt;
            const double dtNew = stepDt(P, st, (double)__uint_as_float(bx), (double)__uint_as_float(by));
            const double tNew = st->t + dtNew;
            if (mine) {  // stage-1 update with this step's dt (Integrate_1_k)
                const StageConsts C1 = stageConstsAt<1>(P, dtNew, dtOld, tNew);
                const bool wetCell =
                    tileCellUpdate<1>(P, C1, S.buf[0], tile, i0, j0, dh, dhu, dhv, pre);
                tileFlags<1>(P, C1, S, tile, wetCell, 0.f, 0.f);
                __syncthreads();
            }
            RIFT_SYNC();
            if (blockIdx.x == 0 && tid == 0) {
                publishDt(P, st, dtNew);
                st->staleBits[0] = st->staleBits[1] = 0u;
            }
            const StageConsts C2 = stageConstsAt<2>(P, dtNew, dtOld, tNew);
            if (!(fl & F_EULER)) {
                if (!stageTiles<2>(S, &tmB, &tmE, P, nAct, ph, &C2)) return;
            } else {
                commitTiles(P, nAct);
            }
            RIFT_SYNC();
            continue;
        } else {
            // speeds of U^n, dt, t, U* re-sync (k_speed_dt), then stage 1
            if (!speedTiles(S, &tmA, &tmE, P, nAct, ph, tmx, tmy)) return;
            __syncthreads();
            finishDt(P, tmx, tmy, &last);
            resyncDeactivated(P);
            RIFT_SYNC();
            if (!stageTiles<1>(S, &tmA, &tmE, P, nAct, ph)) return;
            RIFT_SYNC();
        }
        if (!(fl & F_EULER)) {
            if (!stageTiles<2>(S, &tmB, &tmE, P, nAct, ph)) return;
        } else {
            commitTiles(P, nAct);
        }
        RIFT_SYNC();
    }
#undef RIFT_SYNC
}

}  // namespace rift
