// rift_march.cuh -- the two fused RK stages as a column march over strips.
//
// Work item: a strip of 7 x 2 reference tiles (112 x 28 cells).  A CTA of
// four warps walks the strip row by row.  Lane l of warp w holds column
// 28w + l - 2 of the strip; lanes 2..29 own their column, lanes 0, 1, 30, 31
// supply the x halo (the warps overlap by four columns).  Per output row:
//   - the y reconstruction of the row above and the flux through the row's
//     north face come from registers rolled down the column (no recompute,
//     no shared memory);
//   - the x reconstruction takes its neighbours by warp shuffle, the flux
//     through the east face takes the east neighbour's west-face values by
//     shuffle, and the west-face flux is the west neighbour's east-face flux;
//   - the cell update (sources, friction, RK stage, outputs, ghost cells) is
//     the same arithmetic as grid.cu's Integrate kernels.
// Rows arrive in shared memory through TMA: 4-row chunks of the 120-column
// block of (h, hu, hv) and of the four face-elevation offsets, a 2-slot ring
// refilled as the march moves up (one barrier per chunk).
// A cell is updated only when its reference tile is active, so results and
// tile flags are those of the per-tile schedule of the reference.
//
// Stage 1 needs dt, and dt needs the speeds of stage 1's own fluxes (the
// first ComputeFluxes of the step).  So the stage-1 march computes the
// fluxes, the tile speeds and dt (last CTA), and stores each cell's flux
// divergence with the bed-slope source folded in (3 words); k_update1
// (rift_update1.cuh) then
// applies the rest of Integrate_1_k.  The step does one flux pass per stage
// and no separate speed pass.
#pragma once
#include "rift_kernels.cuh"

namespace rift {

constexpr int MW = 4;                              // warps per CTA
constexpr int MT = MW * 32;                        // threads per CTA
constexpr int MOWN = 28;                           // owned columns per warp
constexpr int MCOLS = STRIP_TX * TW;               // 112 columns per strip
constexpr int MBOXW = 120;                         // staged columns [112 sx - 4, 112 sx + 116)
constexpr int MRC = 4;                             // rows per staged chunk
constexpr int MNSLOT = 2;                          // chunk ring depth
constexpr int MHR = STRIP_TY * TH;                 // 28 output rows per strip
constexpr int MNROWS = MHR + 4;                    // 32 staged rows (2-row halo each side)
constexpr int MNCHUNK = (MNROWS + MRC - 1) / MRC;  // 8 chunks
static_assert(MW * MOWN == MCOLS, "strip width");
static_assert(MNROWS % MRC == 0, "whole chunks");
constexpr unsigned FULL = 0xffffffffu;

struct __align__(128) MarchSlot {
    float s[3][MRC][MBOXW];  // h, hu, hv     (5760 B)
    float e[4][MRC][MBOXW];  // eW, eE, eS, eN (7680 B)
};
static_assert(sizeof(MarchSlot) % 128 == 0, "TMA destination alignment");
static_assert(offsetof(MarchSlot, e) % 128 == 0, "TMA destination alignment");
constexpr uint32_t MBYTES_S = 3 * MRC * MBOXW * 4;
constexpr uint32_t MBYTES_E = 4 * MRC * MBOXW * 4;

// Work items of the march are 112 columns wide and STY reference tile rows
// high (STY = 1, 2 or 4: 14, 28 or 56 cells), chosen per handle
// (rift_set_march_rows, the autotuner).  The grow lists strips of 7 x 2
// tiles; an item of one tile row is half such a strip, one of four rows a
// pair of vertically adjacent strips.
constexpr int STY_MAX = 4;

struct __align__(128) MarchSmem {
    MarchSlot slot[MNSLOT];
    uint64_t bar[MNSLOT];
    unsigned tmx[STRIP_TX * STY_MAX];
    unsigned tmy[STRIP_TX * STY_MAX];
    int twet[STRIP_TX * STY_MAX];
    int tact[STRIP_TX * STY_MAX];
};

// Does strip (sx, sy) of the grow's 7 x 2 strips hold an active tile?
__device__ __forceinline__ bool stripHasActive(const Params& P, int sx, int sy) {
    for (int q = 0; q < STRIP_TX * STRIP_TY; q++) {
        const int bx = STRIP_TX * sx + q % STRIP_TX, by = STRIP_TY * sy + q / STRIP_TX;
        if (bx < P.nBX && by < P.nBY && P.prevAct[by * P.nBX + bx] && bx * TW + 2 <= P.nx - 3 &&
            by * TH + 2 <= P.ny - 3)
            return true;
    }
    return false;
}

// Work item `item` of an STY-row march: its strip column and first tile row;
// false when the item is covered by another one (STY = 4: the upper strip of
// a pair whose lower strip is listed).  Items: 2 x the listed strips for
// STY = 1, the listed strips otherwise.
template <int STY>
__device__ __forceinline__ bool marchItem(const Params& P, int item, int& sx, int& by0) {
    if (STY == 1) {
        const int st = P.strips[item >> 1];
        sx = st % P.nSX;
        by0 = STRIP_TY * (st / P.nSX) + (item & 1);
        return true;
    }
    const int st = P.strips[item];
    sx = st % P.nSX;
    const int sy = st / P.nSX;
    if (STY == 2) {
        by0 = STRIP_TY * sy;
        return true;
    }
    if (sy & 1) {  // pairs (2p, 2p + 1): the upper one alone only without its partner
        if (stripHasActive(P, sx, sy - 1)) return false;
        by0 = STRIP_TY * (sy - 1);
    } else {
        by0 = STRIP_TY * sy;
    }
    return true;
}

template <int STY>
__host__ __device__ constexpr int marchItems(int nStrips) {
    return STY == 1 ? 2 * nStrips : nStrips;
}

struct Row {  // one staged row at this lane's column
    float h, u, v, eW, eE, eS, eN;
};

__device__ __forceinline__ Row loadRow(const MarchSlot& S, int r, int col) {
    Row x;
    x.h = S.s[0][r][col];
    x.u = S.s[1][r][col];
    x.v = S.s[2][r][col];
    x.eW = S.e[0][r][col];
    x.eE = S.e[1][r][col];
    x.eS = S.e[2][r][col];
    x.eN = S.e[3][r][col];
    return x;
}

// y reconstruction of row c between rows m (below) and p (above)
__device__ __forceinline__ Rec constructY(const Row& m, const Row& c, const Row& p) {
    return construct(c.h, c.u, c.v, p.h, p.u, p.v, m.h, m.u, m.v, c.eS, c.eN, c.eN - p.eS,
                     m.eN - c.eS);
}

__device__ __forceinline__ void issueChunk(MarchSmem& S, int slot, const CUtensorMap* tmIn,
                                           const CUtensorMap* tmE, int xs, int ys) {
    fence_proxy_async();
    mbar_expect_tx(&S.bar[slot], MBYTES_S + MBYTES_E);
    tma_load_3d(&S.slot[slot].s[0][0][0], tmIn, &S.bar[slot], xs, ys, 0);
    tma_load_3d(&S.slot[slot].e[0][0][0], tmE, &S.bar[slot], xs, ys, 0);
}

// Error path of a timed-out ring wait on chunk c: wait, bounded, for the
// chunks still in flight (c .. c+MNSLOT-1), so that no TMA write lands after
// the CTA has left.  `par` holds the slots' parities before chunk c's wait.
__device__ __forceinline__ void marchDrain(MarchSmem& S, uint32_t par, int c, int nchunk = MNCHUNK) {
    for (int k = c; k < c + MNSLOT && k < nchunk; k++)
        mbar_wait_bounded(&S.bar[k % MNSLOT], (par >> (k % MNSLOT)) & 1u);
}

// STAGE 1: reads U^n (A) -> flux divergence + bed source (D), tile speed
//          maxima, dt and t (ComputeFluxes' speed output and
//          ComputeTimestep), re-sync of U* on tiles that went inactive.
// STAGE 2: reads U* (B) and U^n (A) at the cell -> writes U^{n+1} (A),
//          F^{n+1} (FA), outputs, tile wet flags and tile speeds.
// Resident CTAs per SM the march kernels are compiled for: the stage-1 flux
// pass fits 8 (64 registers, 27 KB shared memory; measured 1% faster on the
// 8192^2 step than 6), stage 2 needs its 80 registers at 6.
#ifndef RIFT_MARCH1_MINB
#define RIFT_MARCH1_MINB 8
#endif
#ifndef RIFT_MARCH2_MINB
#define RIFT_MARCH2_MINB 6
#endif

template <int STAGE, uint32_t FIX = 0, int STY = STRIP_TY>
__global__ void __launch_bounds__(MT, STAGE == 1 ? RIFT_MARCH1_MINB : RIFT_MARCH2_MINB)
    k_march(const __grid_constant__ CUtensorMap tmIn,
                                              const __grid_constant__ CUtensorMap tmE, Params P) {
    __shared__ MarchSmem S;
    __shared__ bool last;
    if (P.st->stop || !useMarch(P)) return;
    // rain maps read ahead with U^n when the instantiation has gridded rain
    constexpr bool RAINPRE = STAGE == 2 && (FIX & F_RAIN_G) != 0;
    constexpr int HR = STY * TH;                      // output rows per item
    constexpr int NCHUNK = (HR + 4 + MRC - 1) / MRC;  // staged chunks (2-row halo each side)
    constexpr int NT_ = STRIP_TX * STY;                // tiles per item
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int nItems = marchItems<STY>(P.st->nStrips);
    const StageConsts C = blockConsts<STAGE>(P);
    float tmxAll = 0.f, tmyAll = 0.f;
    if (tid == 0) {
        prefetch_tmap(&tmIn);
        prefetch_tmap(&tmE);
        for (int k = 0; k < MNSLOT; k++) mbar_init(&S.bar[k], 1);
        fence_mbar_init();
    }
    __syncthreads();
    uint32_t par = 0u;                          // wait parity, one bit per ring slot
    const int lc = MOWN * warp + lane - 2;      // column relative to the strip's first interior column
    const int col = lc + 6;                     // staged column
    const bool owned = lane >= 2 && lane <= 29;
    const int tcol = owned ? lc / TW : 0;       // tile column inside the strip
    const float kappa = C.kappa;
    // check_volume ledger: stage 1 sums the edge inflow rates (dt is not
    // known yet), stage 2 the weighted terms of its cells
    const bool led = (cellFlags<FIX>(C.fl) & F_CHECKVOL) != 0;
    Led L;
    ledZero(L);

    for (int item = blockIdx.x; item < nItems; item += gridDim.x) {
        int sx, by0;
        if (!marchItem<STY>(P, item, sx, by0)) continue;  // item-uniform
        const int X0 = MCOLS * sx + 2, Y0 = TH * by0 + 2;
        // item-uniform: does the item reach the first or last interior row/column?
        const bool edgeStrip =
            X0 == 2 || Y0 == 2 || X0 + MCOLS - 1 >= P.nx - 3 || Y0 + HR - 1 >= P.ny - 3;
        const int xs = MCOLS * sx - 4, ys = Y0 - 2;
        const int i = X0 + lc;
        __syncthreads();  // the previous item no longer reads the ring or the tile tables
        if (tid < NT_) {
            const int bx = STRIP_TX * sx + tid % STRIP_TX, by = by0 + tid / STRIP_TX;
            int a = 0;
            if (bx < P.nBX && by < P.nBY)
                a = P.prevAct[by * P.nBX + bx] && (bx * TW + 2 <= P.nx - 3) &&
                    (by * TH + 2 <= P.ny - 3);
            S.tact[tid] = a;
            S.tmx[tid] = 0u;
            S.tmy[tid] = 0u;
            S.twet[tid] = 0;
        }
        if (tid == 0)
            for (int c = 0; c < MNSLOT; c++) issueChunk(S, c, &tmIn, &tmE, xs, ys + c * MRC);
        bool ok = mbar_wait_bounded(&S.bar[0], par & 1u);
        if (!__syncthreads_and(ok)) {
            marchDrain(S, par, 0, NCHUNK);
            if (tid == 0) atomicOr(&P.st->error, ERR_TMA_TIMEOUT);
            return;
        }
        par ^= 1u;
        // prologue: staged rows 0..3; y reconstruction of rows 1 and 2 and the
        // flux through the south face of row 2 (the first output row)
        const Row r0 = loadRow(S.slot[0], 0, col);
        const Row r1 = loadRow(S.slot[0], 1, col);
        Row cur = loadRow(S.slot[0], 2, col);
        Row nxt = loadRow(S.slot[0], 3, col);
        float fS0, fS1, fS2, yPh, yPu, yPv;
        {
            const Rec y1 = constructY(r0, r1, cur);
            const Rec y2 = constructY(r1, cur, nxt);
            float f[3];
            faceFlux<1>(y1.hP, y1.uP, y1.vP, y2.hM, y2.uM, y2.vM, kappa, f);
            fS0 = f[0];
            fS1 = f[1];
            fS2 = f[2];
            yPh = y2.hP;
            yPu = y2.uP;
            yPv = y2.vP;
        }
        // centre values of the first output row (stage 2: U^n, and the rain
        // maps when the instantiation reads them ahead), loaded ahead of use
        const bool colIn = owned && i <= P.nx - 3;
        // row jj's centre values into d (U^n; the rain maps, or an L1 hint)
        auto loadCentre = [&](float (&d)[8], int jj) {
            const size_t cn = cidx(P, 0, jj, i);
            d[0] = P.A[cn];
            d[1] = P.A[cn + P.planeSize];
            d[2] = P.A[cn + 2 * (size_t)P.planeSize];
            if (RAINPRE)
                loadRainMaps(P, cn, d + 6);
            else
                prefetchMaps(P, cellFlags<FIX>(C.fl), cn);
        };
        float pre[8], nextPre[8];
#pragma unroll
        for (int q = 0; q < 8; q++) pre[q] = nextPre[q] = 0.f;
        if (STAGE == 2 && colIn && Y0 <= P.ny - 3) loadCentre(pre, Y0);
        float accMx = 0.f, accMy = 0.f;
        bool accWet = false;
        // two rows per iteration: the compiler interleaves their independent
        // work (7% faster than one row at the same 80 registers)
#pragma unroll 2
        for (int R = 2; R <= HR + 1; R++) {
            const int lead = R + 2;
            if (lead % MRC == 0) {  // entering chunk c: refill the slot chunk c-1 used
                const int c = lead / MRC;
                __syncthreads();
                if (tid == 0 && c - 1 + MNSLOT < NCHUNK)
                    issueChunk(S, (c - 1) % MNSLOT, &tmIn, &tmE, xs, ys + (c - 1 + MNSLOT) * MRC);
                const int sl = c % MNSLOT;
                bool ok2 = mbar_wait_bounded(&S.bar[sl], (par >> sl) & 1u);
                if (!__syncthreads_and(ok2)) {
                    marchDrain(S, par, c, NCHUNK);
                    if (tid == 0) atomicOr(&P.st->error, ERR_TMA_TIMEOUT);
                    return;
                }
                par ^= (1u << sl);
            }
            const Row ld = loadRow(S.slot[(lead / MRC) % MNSLOT], lead % MRC, col);
            const int j = Y0 + R - 2;
            // centre values of the next output row, in flight during this one
            if (STAGE == 2 && colIn && j + 1 <= P.ny - 3) loadCentre(nextPre, j + 1);
            const int tslot = ((R - 2) / TH) * STRIP_TX + tcol;
            const bool cellOn = colIn && S.tact[tslot] && j <= P.ny - 3;
            float spx, spy;
            {
                // y: reconstruction of row R+1, flux through the north face of row R
                const Rec yn = constructY(cur, nxt, ld);
                float fN[3];
                spy = faceFlux<1>(yPh, yPu, yPv, yn.hM, yn.uM, yn.vM, kappa, fN);
                // x: reconstruction of row R, neighbours by shuffle
                const float hm = __shfl_up_sync(FULL, cur.h, 1), hp = __shfl_down_sync(FULL, cur.h, 1);
                const float um = __shfl_up_sync(FULL, cur.u, 1), up = __shfl_down_sync(FULL, cur.u, 1);
                const float vm = __shfl_up_sync(FULL, cur.v, 1), vp = __shfl_down_sync(FULL, cur.v, 1);
                const float eEm = __shfl_up_sync(FULL, cur.eE, 1);
                const float eWp = __shfl_down_sync(FULL, cur.eW, 1);
                const Rec xr = construct(cur.h, cur.u, cur.v, hp, up, vp, hm, um, vm, cur.eW,
                                         cur.eE, cur.eE - eWp, eEm - cur.eW);
                const float rh = __shfl_down_sync(FULL, xr.hM, 1);
                const float ru = __shfl_down_sync(FULL, xr.uM, 1);
                const float rv = __shfl_down_sync(FULL, xr.vM, 1);
                float fE[3];
                spx = faceFlux<0>(xr.hP, xr.uP, xr.vP, rh, ru, rv, kappa, fE);
                const float fW0 = __shfl_up_sync(FULL, fE[0], 1);
                const float fW1 = __shfl_up_sync(FULL, fE[1], 1);
                const float fW2 = __shfl_up_sync(FULL, fE[2], 1);
                if (cellOn) {
                    if (led && edgeStrip) {
                        const float r = edgeInflow(P, j, i, fW0, fE[0], fS0, fN[0]);
                        L.v[LED_BOUND] += STAGE == 1 ? r : C.wRate * r;
                    }
                    const float dh = -(fE[0] - fW0) * P.inv_dx - (fN[0] - fS0) * P.inv_dy;
                    const float dhu = -(fE[1] - fW1) * P.inv_dx - (fN[1] - fS1) * P.inv_dy;
                    const float dhv = -(fE[2] - fW2) * P.inv_dx - (fN[2] - fS2) * P.inv_dy;
                    if (STAGE == 1) {
                        // divergence + bed-slope source (dt-free) for k_update1
                        const size_t c = cidx(P, 0, j, i);
                        P.D[c] = dh;
                        P.D[c + P.planeSize] = dhu + bedSourceX(P, cur.h, cur.eW, cur.eE);
                        P.D[c + 2 * (size_t)P.planeSize] = dhv + bedSourceY(P, cur.h, cur.eS, cur.eN);
                    } else {
                        const int tile = (by0 + (R - 2) / TH) * P.nBX + STRIP_TX * sx + tcol;
                        accWet |= cellUpdate<STAGE, false, true, FIX, RAINPRE>(P, C, tile, j, i, dh, dhu, dhv, cur.h, cur.u,
                                                    cur.v, cur.eW, cur.eE, cur.eS, cur.eN, pre,
                                                    edgeStrip, led ? &L : nullptr);
                    }
                }
                fS0 = fN[0];
                fS1 = fN[1];
                fS2 = fN[2];
                yPh = yn.hP;
                yPu = yn.uP;
                yPv = yn.vP;
            }
            if (cellOn) {
                accMx = fmaxf(accMx, spx);
                accMy = fmaxf(accMy, spy);
            }
            if ((R - 2) % TH == TH - 1) {  // last row of a tile row: fold into the tile
                if (owned) {
                    atomicMax(&S.tmx[tslot], __float_as_uint(accMx));
                    atomicMax(&S.tmy[tslot], __float_as_uint(accMy));
                    if (STAGE == 2 && accWet) atomicOr(&S.twet[tslot], 1);
                }
                accMx = 0.f;
                accMy = 0.f;
                accWet = false;
            }
            pre[0] = nextPre[0];
            pre[1] = nextPre[1];
            pre[2] = nextPre[2];
            pre[6] = nextPre[6];
            pre[7] = nextPre[7];

            cur = nxt;
            nxt = ld;
        }
        __syncthreads();
        if (tid < NT_ && S.tact[tid]) {
            const int bx = STRIP_TX * sx + tid % STRIP_TX, by = by0 + tid / STRIP_TX;
            const int b = by * P.nBX + bx;
            if (STAGE == 2) P.wet[b] = (uint8_t)((!(C.fl & F_TILE_ACC)) || S.twet[tid]);
            P.mx[b] = __uint_as_float(S.tmx[tid]);
            P.my[b] = __uint_as_float(S.tmy[tid]);
        }
        if (STAGE == 1) {  // thread 0 keeps this CTA's maximum of new tile speeds
            __syncthreads();
            if (tid == 0)
                for (int k = 0; k < NT_; k++)
                    if (S.tact[k]) {
                        tmxAll = fmaxf(tmxAll, __uint_as_float(S.tmx[k]));
                        tmyAll = fmaxf(tmyAll, __uint_as_float(S.tmy[k]));
                    }
        }
    }
    if (led) {
        if (STAGE == 1) {
            float r = L.v[LED_BOUND];
            for (int o = 16; o > 0; o >>= 1) r += __shfl_xor_sync(FULL, r, o);
            if (lane == 0 && r != 0.f) atomicAdd(&P.st->ledPend, (double)r);
            __threadfence();  // before the dt ticket: the last CTA folds ledPend
        } else {
            flushLed(L, P.st->led);
        }
    }
    if (STAGE == 1) {
        __syncthreads();
        finishDt(P, tmxAll, tmyAll, &last);
        resyncDeactivated(P);
    }
}

}  // namespace rift
