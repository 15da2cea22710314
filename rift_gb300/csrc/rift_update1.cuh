// rift_update1.cuh -- the rest of Integrate_1_k (grid.cu:856-1023) on the
// march's items once dt is known: sources, friction, the RK stage, outputs
// and ghost cells, from U^n and the divergence k_march<1> stored; in Euler
// mode also the tile wet flags.
//
// No halo, so the work item is half a strip (one tile row of 7 tiles,
// 112 x 14 cells): finer items balance the grid.  One thread per column.
// An item's rows arrive in two 7-row chunks -- U^n (3 planes), the
// divergence (3), n, and with gridded rain the rain maps -- through a
// 2-slot ring of TMA copies that runs one chunk ahead, across items, so the
// copies of the next chunk overlap the update of this one.  (Loading the
// same values into registers two rows at a time, the copies' latency was
// exposed: 71% of the copy bandwidth; measured 1.9% slower per config-3
// step than this kernel.)
#pragma once
#include "rift_march.cuh"

namespace rift {

constexpr int URC = 7;                          // rows per chunk (two chunks per item)
constexpr int UBOXW = 116;                      // staged columns [112 sx, 112 sx + 116)
constexpr int UNSLOT = 2;                       // chunk ring depth
constexpr uint32_t U1PLANE = URC * UBOXW * 4;   // 3248 B
constexpr uint32_t U1_OFF_A = 0;                // U^n, 3 planes (one copy)
constexpr uint32_t U1_OFF_D = 9856;             // divergence, 3 planes (one copy)
constexpr uint32_t U1_OFF_N = 19712;            // Manning n
constexpr uint32_t U1_OFF_R0 = 23040;           // rain map at t0
constexpr uint32_t U1_OFF_R1 = 26368;           // rain map at t1
static_assert(U1_OFF_D >= 3 * U1PLANE && U1_OFF_N >= U1_OFF_D + 3 * U1PLANE, "slot layout");
static_assert(U1_OFF_R0 >= U1_OFF_N + U1PLANE && U1_OFF_R1 >= U1_OFF_R0 + U1PLANE, "slot layout");
static_assert(U1_OFF_D % 128 == 0 && U1_OFF_N % 128 == 0 && U1_OFF_R0 % 128 == 0 &&
                  U1_OFF_R1 % 128 == 0,
              "TMA destination alignment");
template <bool RAIN>
__host__ __device__ constexpr uint32_t u1SlotBytes() {
    return RAIN ? 29696u : 23040u;  // 128-byte multiples
}
template <bool RAIN>
__host__ __device__ constexpr uint32_t u1SmemBytes() {
    return UNSLOT * u1SlotBytes<RAIN>() + 128;  // + barriers and tile tables
}
static_assert(u1SlotBytes<true>() >= U1_OFF_R1 + U1PLANE && u1SlotBytes<false>() >= U1_OFF_N + U1PLANE &&
                  u1SlotBytes<true>() % 128 == 0 && u1SlotBytes<false>() % 128 == 0,
              "slot sizes");
static_assert(UNSLOT * 8 + 2 * STRIP_TX * 4 + 16 <= 128, "barriers and tile tables after the ring");

// Tensor maps of the staged planes (116 x 7-row boxes).
struct U1Maps {
    CUtensorMap a, d, n, r0, r1;
};

// Item k of this CTA's sequence: its strip column and tile row.
__device__ __forceinline__ void u1Item(const Params& P, int item, int& sx, int& by) {
    const int strip = P.strips[item >> 1];
    sx = strip % P.nSX;
    by = STRIP_TY * (strip / P.nSX) + (item & 1);
}

template <uint32_t FIX = 0>
__global__ void __launch_bounds__(MT, 3) k_update1(const __grid_constant__ U1Maps M, Params P) {
    constexpr bool RAIN = (FIX & F_RAIN_G) != 0;
    constexpr uint32_t SLOT = u1SlotBytes<RAIN>();
    extern __shared__ __align__(128) unsigned char u1raw[];
    uint64_t* bar = reinterpret_cast<uint64_t*>(u1raw + UNSLOT * SLOT);
    int* tact = reinterpret_cast<int*>(u1raw + UNSLOT * SLOT + 16);
    int* twet = tact + STRIP_TX;
    if (P.st->stop || !useMarch(P)) return;
    const int tid = threadIdx.x;
    const int nItems = 2 * P.st->nStrips;
    const StageConsts C = blockConsts<1>(P);
    const bool led = (cellFlags<FIX>(C.fl) & F_CHECKVOL) != 0;
    const int nRain = RAIN ? P.mapMode[0] : 0;  // rain planes staged: 0, 1 or 2
    Led L;
    ledZero(L);
    const int myItems =
        ((int)blockIdx.x < nItems) ? (nItems - 1 - (int)blockIdx.x) / (int)gridDim.x + 1 : 0;
    const int nChunks = 2 * myItems;
    if (tid == 0) {
        prefetch_tmap(&M.a);
        prefetch_tmap(&M.d);
        prefetch_tmap(&M.n);
        for (int k = 0; k < UNSLOT; k++) mbar_init(&bar[k], 1);
        fence_mbar_init();
    }
    __syncthreads();
    // chunk q of this CTA's sequence into slot q % UNSLOT (thread 0)
    auto issue = [&](int q) {
        int sx, by;
        u1Item(P, (int)blockIdx.x + (q >> 1) * (int)gridDim.x, sx, by);
        const int xs = MCOLS * sx, ys = by * TH + 2 + URC * (q & 1);
        unsigned char* z = u1raw + (q % UNSLOT) * SLOT;
        uint64_t* b = &bar[q % UNSLOT];
        fence_proxy_async();
        mbar_expect_tx(b, (7u + (uint32_t)nRain) * U1PLANE);
        tma_load_3d(z + U1_OFF_A, &M.a, b, xs, ys, 0);
        tma_load_3d(z + U1_OFF_D, &M.d, b, xs, ys, 0);
        tma_load_3d(z + U1_OFF_N, &M.n, b, xs, ys, 0);
        if (RAIN && nRain >= 1) tma_load_3d(z + U1_OFF_R0, &M.r0, b, xs, ys, 0);
        if (RAIN && nRain >= 2) tma_load_3d(z + U1_OFF_R1, &M.r1, b, xs, ys, 0);
    };
    if (tid == 0)
        for (int q = 0; q < UNSLOT && q < nChunks; q++) issue(q);
    uint32_t par = 0u;
    bool wetAny = false;
    for (int q = 0; q < nChunks; q++) {
        const int c = q & 1, sl = q % UNSLOT;
        int sx, by;
        u1Item(P, (int)blockIdx.x + (q >> 1) * (int)gridDim.x, sx, by);
        const int X0 = MCOLS * sx + 2, Y0 = by * TH + 2;
        const bool edgeStrip =
            X0 == 2 || Y0 == 2 || X0 + MCOLS - 1 >= P.nx - 3 || Y0 + TH - 1 >= P.ny - 3;
        if (c == 0) {
            __syncthreads();  // the previous item no longer reads the tile tables
            if (tid < STRIP_TX) {
                const int bx = STRIP_TX * sx + tid;
                int a = 0;
                if (bx < P.nBX && by < P.nBY)
                    a = P.prevAct[by * P.nBX + bx] && (bx * TW + 2 <= P.nx - 3) && (Y0 <= P.ny - 3);
                tact[tid] = a;
                twet[tid] = 0;
            }
            wetAny = false;
        }
        const bool ok = mbar_wait_bounded(&bar[sl], (par >> sl) & 1u);
        if (!__syncthreads_and(ok)) {
            // let the copies in flight land before the CTA's memory goes
            for (int k = q; k < q + UNSLOT && k < nChunks; k++)
                mbar_wait_bounded(&bar[k % UNSLOT], (par >> (k % UNSLOT)) & 1u);
            if (tid == 0) atomicOr(&P.st->error, ERR_TMA_TIMEOUT);
            return;
        }
        par ^= (1u << sl);
        const float* z = reinterpret_cast<const float*>(u1raw + sl * SLOT);
        const int i = X0 + tid, slot = tid / TW;
        if (tid < MCOLS && i <= P.nx - 3 && tact[slot]) {
            const int tile = by * P.nBX + STRIP_TX * sx + slot;
            constexpr int PL = URC * UBOXW;
#pragma unroll 1
            for (int r = 0; r < URC; r++) {
                const int j = Y0 + URC * c + r;
                if (j > P.ny - 3) break;
                const int o = r * UBOXW + tid + 2;
                const float* a = z + U1_OFF_A / 4 + o;
                const float* d = z + U1_OFF_D / 4 + o;
                const float pre[8] = {z[U1_OFF_N / 4 + o], 0.f, 0.f, 0.f, 0.f, 0.f,
                                      (RAIN && nRain >= 1) ? z[U1_OFF_R0 / 4 + o] : 0.f,
                                      (RAIN && nRain >= 2) ? z[U1_OFF_R1 / 4 + o] : 0.f};
                wetAny |= cellUpdate<1, false, false, FIX, RAIN>(
                    P, C, tile, j, i, d[0], d[PL], d[2 * PL], a[0], a[PL], a[2 * PL], 0.f, 0.f, 0.f,
                    0.f, pre, edgeStrip, led ? &L : nullptr);
            }
        }
        __syncthreads();  // slot sl is free again
        if (tid == 0 && q + UNSLOT < nChunks) issue(q + UNSLOT);
        if (c == 1 && C.euler) {
            if (wetAny && tid < MCOLS) atomicOr(&twet[slot], 1);
            __syncthreads();
            if (tid < STRIP_TX && tact[tid])
                P.wet[by * P.nBX + STRIP_TX * sx + tid] =
                    (uint8_t)((!(C.fl & F_TILE_ACC)) || twet[tid]);
        }
    }
    if (led) flushLed(L, P.st->led);
}

}  // namespace rift
