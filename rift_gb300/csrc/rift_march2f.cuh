// rift_march2f.cuh -- RK stage 2 of the column march with the rest of stage 1
// folded in: U* is rebuilt on the fly from U^n and the stored divergence.
//
// The march splits RK stage 1 at dt: k_march<1> computes the stage-1 fluxes
// of U^n (they give dt) and stores each cell's divergence D; the stage-1
// update U* = f(U^n, D, sources, friction) is pointwise.  So stage 2 does not
// need U* in memory: for every staged cell this kernel stages U^n and D by
// TMA and applies the stage-1 update itself (rk1Core, the same arithmetic as
// k_update1), then marches stage 2 exactly as k_march<2> does.  The staged
// cells of a strip overlap its neighbours' by two cells, so halo cells are
// updated by more than one CTA, each with the same bits; only the strip's own
// cells write results.
//
// A strip qualifies when its staged block holds no ghost cell (the critical
// depth ghosts of U* depend on the neighbouring interior U*); the others run
// k_update1 + k_march<2>, and k_update1 also keeps U* of the strips next to
// them (stripBandM), whose cells they stage.  Euler runs have no stage 2 and
// keep the split.
#pragma once
#include "rift_march.cuh"

namespace rift {

struct __align__(128) FusedSlot {
    float a[3][MRC][MBOXW];  // U^n: h, hu, hv      (5760 B)
    float d[3][MRC][MBOXW];  // stage-1 divergence  (5760 B)
    float e[4][MRC][MBOXW];  // eW, eE, eS, eN       (7680 B)
};
static_assert(sizeof(FusedSlot) % 128 == 0, "TMA destination alignment");
static_assert(offsetof(FusedSlot, d) % 128 == 0, "TMA destination alignment");
static_assert(offsetof(FusedSlot, e) % 128 == 0, "TMA destination alignment");
constexpr uint32_t FBYTES = 10 * MRC * MBOXW * 4;
constexpr int FACT_W = STRIP_TX + 2, FACT_H = STRIP_TY + 2;  // tiles around a strip

struct __align__(128) FusedSmem {
    FusedSlot slot[MNSLOT];
    uint64_t bar[MNSLOT];
    unsigned tmx[STRIP_TX * STRIP_TY];
    unsigned tmy[STRIP_TX * STRIP_TY];
    int twet[STRIP_TX * STRIP_TY];
    int act[FACT_H][FACT_W];  // tiles 7sx-1 .. 7sx+7, 2sy-1 .. 2sy+2
};

__device__ __forceinline__ void issueFused(FusedSmem& S, int slot, const CUtensorMap* tmA,
                                           const CUtensorMap* tmD, const CUtensorMap* tmE, int xs,
                                           int ys) {
    fence_proxy_async();
    mbar_expect_tx(&S.bar[slot], FBYTES);
    tma_load_3d(&S.slot[slot].a[0][0][0], tmA, &S.bar[slot], xs, ys, 0);
    tma_load_3d(&S.slot[slot].d[0][0][0], tmD, &S.bar[slot], xs, ys, 0);
    tma_load_3d(&S.slot[slot].e[0][0][0], tmE, &S.bar[slot], xs, ys, 0);
}

__device__ __forceinline__ void fusedDrain(FusedSmem& S, uint32_t par, int c) {
    for (int k = c; k < c + MNSLOT && k < MNCHUNK; k++)
        mbar_wait_bounded(&S.bar[k % MNSLOT], (par >> (k % MNSLOT)) & 1u);
}

// U* of staged cell (row r of slot, column col; global cell (j, i)) and its
// face offsets.  A cell of an inactive tile keeps U^n (its U* buffer is a
// copy of U^n).  L (check_volume runs): the stage-1 ledger terms of the
// cells this CTA owns.
template <uint32_t FIX>
__device__ __forceinline__ Row fusedRow(const FusedSmem& S, const FusedSlot& Z, const Params& P,
                                        const StageConsts& C1, int r, int col, int j, int i,
                                        int bx0, int by0, Led* L) {
    Row x;
    const float hn = Z.a[0][r][col], un = Z.a[1][r][col], vn = Z.a[2][r][col];
    x.eW = Z.e[0][r][col];
    x.eE = Z.e[1][r][col];
    x.eS = Z.e[2][r][col];
    x.eN = Z.e[3][r][col];
    const int bx = (i - 2) / TW, by = (j - 2) / TH;
    if (S.act[by - by0][bx - bx0]) {
        const float pre[1] = {P.nman[cidx(P, 0, j, i)]};
        const CellSrc src = cellSources<1, false, false, FIX>(
            P, C1, by * P.nBX + bx, j, i, Z.d[0][r][col], Z.d[1][r][col], Z.d[2][r][col], hn, un,
            vn, 0.f, 0.f, 0.f, 0.f, pre);
        rk1Core<FIX>(P, C1, cidx(P, 0, j, i), src, hn, un, vn, L, x.h, x.u, x.v);
        if (L) {
            L->v[LED_DRAIN] += C1.wRate * src.drained;
            L->v[LED_INFIL] += C1.wRate * src.dF;
        }
    } else {
        x.h = hn;
        x.u = un;
        x.v = vn;
    }
    return x;
}

// RK stage 2 of the qualifying strips: reads U^n (A) and D with a halo,
// writes U^{n+1} (A), F^{n+1} (FA), outputs, tile wet flags and tile speeds,
// as k_march<2> with U* from fusedRow.
template <uint32_t FIX = 0>
__global__ void __launch_bounds__(MT, 4) k_march2f(const __grid_constant__ CUtensorMap tmA,
                                                const __grid_constant__ CUtensorMap tmD,
                                                const __grid_constant__ CUtensorMap tmE, Params P) {
    __shared__ FusedSmem S;
    if (P.st->stop || !useMarch(P) || !P.fuse) return;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int nItems = P.st->nStrips;
    const StageConsts C1 = blockConsts<1>(P);
    const StageConsts C = blockConsts<2>(P);
    if (tid == 0) {
        prefetch_tmap(&tmA);
        prefetch_tmap(&tmD);
        prefetch_tmap(&tmE);
        for (int k = 0; k < MNSLOT; k++) mbar_init(&S.bar[k], 1);
        fence_mbar_init();
    }
    __syncthreads();
    uint32_t par = 0u;
    const int lc = MOWN * warp + lane - 2;
    const int col = lc + 6;
    const bool owned = lane >= 2 && lane <= 29;
    const int tcol = owned ? lc / TW : 0;
    const float kappa = C.kappa;
    const uint32_t fl = cellFlags<FIX>(C.fl);
    const bool led = (fl & F_CHECKVOL) != 0;
    const bool infil = (fl & F_INFIL) != 0;
    Led L;
    ledZero(L);

    for (int item = blockIdx.x; item < nItems; item += gridDim.x) {
        const int strip = P.strips[item];
        const int sx = strip % P.nSX, sy = strip / P.nSX;
        if (!stripFusableM(P, sx, sy)) continue;  // strip-uniform
        const int X0 = MCOLS * sx + 2, Y0 = MHR * sy + 2;
        const int xs = MCOLS * sx - 4, ys = Y0 - 2;
        const int i = X0 + lc;
        const int bx0 = STRIP_TX * sx - 1, by0 = STRIP_TY * sy - 1;
        __syncthreads();  // the previous item no longer reads the ring or the tile tables
        if (tid < STRIP_TX * STRIP_TY) {
            S.tmx[tid] = 0u;
            S.tmy[tid] = 0u;
            S.twet[tid] = 0;
        }
        for (int q = tid; q < FACT_W * FACT_H; q += MT) {
            const int bx = bx0 + q % FACT_W, by = by0 + q / FACT_W;
            // a qualifying strip's neighbourhood lies inside the tile grid
            S.act[q / FACT_W][q % FACT_W] = P.prevAct[by * P.nBX + bx];
        }
        if (tid == 0)
            for (int c = 0; c < MNSLOT; c++)
                issueFused(S, c, &tmA, &tmD, &tmE, xs, ys + c * MRC);
        bool ok = mbar_wait_bounded(&S.bar[0], par & 1u);
        if (!__syncthreads_and(ok)) {
            fusedDrain(S, par, 0);
            if (tid == 0) atomicOr(&P.st->error, ERR_TMA_TIMEOUT);
            return;
        }
        par ^= 1u;
        // ledger of the stage-1 update: the strip's own cells, once
        auto rowLed = [&](int j) -> Led* {
            return (led && owned && j >= Y0 && j < Y0 + MHR) ? &L : nullptr;
        };
        const Row r0 = fusedRow<FIX>(S, S.slot[0], P, C1, 0, col, ys, i, bx0, by0, rowLed(ys));
        const Row r1 = fusedRow<FIX>(S, S.slot[0], P, C1, 1, col, ys + 1, i, bx0, by0, rowLed(ys + 1));
        Row cur = fusedRow<FIX>(S, S.slot[0], P, C1, 2, col, ys + 2, i, bx0, by0, rowLed(ys + 2));
        Row nxt = fusedRow<FIX>(S, S.slot[0], P, C1, 3, col, ys + 3, i, bx0, by0, rowLed(ys + 3));
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
        // the own cell's U^n (and F, K) of the first output row, loaded ahead of use
        float pre[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f}, nextPre[6];
        auto loadPre = [&](int j, float* q) {
            const size_t c = cidx(P, 0, j, i);
            q[0] = P.A[c];
            q[1] = P.A[c + P.planeSize];
            q[2] = P.A[c + 2 * (size_t)P.planeSize];
            if (infil) {
                q[5] = P.FA[c];
                q[4] = P.K[c];
            }
        };
        if (owned) loadPre(Y0, pre);
        float accMx = 0.f, accMy = 0.f;
        bool accWet = false;
#pragma unroll 2
        for (int R = 2; R <= MHR + 1; R++) {
            const int lead = R + 2;
            if (lead % MRC == 0) {  // entering chunk c: refill the slot chunk c-1 used
                const int c = lead / MRC;
                __syncthreads();
                if (tid == 0 && c - 1 + MNSLOT < MNCHUNK)
                    issueFused(S, (c - 1) % MNSLOT, &tmA, &tmD, &tmE, xs, ys + (c - 1 + MNSLOT) * MRC);
                const int sl = c % MNSLOT;
                bool ok2 = mbar_wait_bounded(&S.bar[sl], (par >> sl) & 1u);
                if (!__syncthreads_and(ok2)) {
                    fusedDrain(S, par, c);
                    if (tid == 0) atomicOr(&P.st->error, ERR_TMA_TIMEOUT);
                    return;
                }
                par ^= (1u << sl);
            }
            const Row ld = fusedRow<FIX>(S, S.slot[(lead / MRC) % MNSLOT], P, C1, lead % MRC, col,
                                         ys + lead, i, bx0, by0, rowLed(ys + lead));
            const int j = Y0 + R - 2;
            if (owned && R <= MHR) loadPre(j + 1, nextPre);
            const int tslot = ((R - 2) / TH) * STRIP_TX + tcol;
            const bool cellOn = owned && S.act[1 + (R - 2) / TH][1 + tcol];
            float spx, spy;
            {
                const Rec yn = constructY(cur, nxt, ld);
                float fN[3];
                spy = faceFlux<1>(yPh, yPu, yPv, yn.hM, yn.uM, yn.vM, kappa, fN);
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
                    const float dh = -(fE[0] - fW0) * P.inv_dx - (fN[0] - fS0) * P.inv_dy;
                    const float dhu = -(fE[1] - fW1) * P.inv_dx - (fN[1] - fS1) * P.inv_dy;
                    const float dhv = -(fE[2] - fW2) * P.inv_dx - (fN[2] - fS2) * P.inv_dy;
                    if (infil) {
                        // F* of the cell (the stage-1 update of F, k_update1's arithmetic)
                        const float dF1 = greenAmpt(pre[4], pre[5], P.psiDtheta, C1.dtSrc, pre[0]);
                        pre[3] = pre[5] + dF1 * C1.dtNew;
                    }
                    const int tile = (STRIP_TY * sy + (R - 2) / TH) * P.nBX + STRIP_TX * sx + tcol;
                    accWet |= cellUpdate<2, true, true, FIX>(P, C, tile, j, i, dh, dhu, dhv, cur.h,
                                                             cur.u, cur.v, cur.eW, cur.eE, cur.eS,
                                                             cur.eN, pre, false, led ? &L : nullptr);
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
            if ((R - 2) % TH == TH - 1) {
                if (owned) {
                    atomicMax(&S.tmx[tslot], __float_as_uint(accMx));
                    atomicMax(&S.tmy[tslot], __float_as_uint(accMy));
                    if (accWet) atomicOr(&S.twet[tslot], 1);
                }
                accMx = 0.f;
                accMy = 0.f;
                accWet = false;
            }
#pragma unroll
            for (int q = 0; q < 6; q++) pre[q] = nextPre[q];
            cur = nxt;
            nxt = ld;
        }
        __syncthreads();
        if (tid < STRIP_TX * STRIP_TY) {
            const int bx = STRIP_TX * sx + tid % STRIP_TX, by = STRIP_TY * sy + tid / STRIP_TX;
            if (S.act[1 + tid / STRIP_TX][1 + tid % STRIP_TX]) {
                const int b = by * P.nBX + bx;
                P.wet[b] = (uint8_t)((!(C.fl & F_TILE_ACC)) || S.twet[tid]);
                P.mx[b] = __uint_as_float(S.tmx[tid]);
                P.my[b] = __uint_as_float(S.tmy[tid]);
            }
        }
    }
    if (led) flushLed(L, P.st->led);
}

}  // namespace rift
