// rift_closure.cu -- learned sub-grid flux closure on a 2x-coarsened grid.
//
// The net (6 -> 32 channels 5x5, 32 -> 32 3x3, 32 -> 4 1x1, ReLU between)
// runs tile by tile: a CTA stages a 22 x 22 block of the six input channels,
// computes layer 1 on the 18 x 18 cells that layer 2 needs, and layers 2 and
// 3 on the 16 x 16 output cells.  Every contraction is an implicit GEMM on
// the BF16 tensor cores (mma.sync m16n8k16, FP32 accumulation): the rows of
// an MMA tile are 16 cells, the columns output channels, and the reduction
// runs over (tap, input channel).  Layer 1 activations stay in shared memory
// as BF16 in channels-last rows of 40 (32 channels + 8 of padding, so the
// fragment loads of eight consecutive cells fall in distinct banks); layer 2
// outputs stay in registers, and their accumulator fragments are the A
// fragments of layer 3 without leaving the thread.
//
// The training kernel recomputes the forward pass of its tile and runs the
// backward pass in the same CTA: layer-3 gradients on the CUDA cores (4 x 32
// weights), the layer-2 and layer-1 weight gradients and the layer-1
// activation gradient as tensor-core GEMMs.  Weight gradients stay in
// registers across every tile a CTA visits and are added to the global
// gradient once per CTA.
//
// The flux kernel evaluates the step's central-upwind face flux
// (rift_device.cuh) on a handle's state, for the time-integrated fluxes
// through coarse faces that make the training targets.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <string>

#include "../../include/rift_closure.h"
#include "rift_device.cuh"

namespace rc {

constexpr int CIN = 6, C1 = 32, COUT = 4;
constexpr int K1 = 150, K1P = 160, K2 = 288;
constexpr int OT = 16;           // output tile side
constexpr int R1 = OT + 2;       // layer-1 region side (18)
constexpr int RI = OT + 6;       // input region side (22)
constexpr int NR1 = R1 * R1;     // 324
constexpr int NRI = RI * RI;     // 484
constexpr int M1T = (NR1 + 15) / 16;  // 21 MMA row tiles of layer 1
constexpr int SA = 40;           // BF16 row stride of the activation tiles
constexpr int CB = 8;            // BF16 input channels per cell: h, hu, hv, b_hi, b_lo, n, rain, 0
constexpr int NTAP1 = 26;        // layer-1 taps, the 26th a zero-weight pad
constexpr int K1B = NTAP1 * CB;  // 208: layer-1 reduction over the BF16 inputs
constexpr int SW1 = K1B + 8, SW2 = 296, SW3 = 40;  // BF16 row strides of the weights
constexpr int NT = 256;
constexpr int BEDBIT = 1 << 20, OFFMASK = BEDBIT - 1;

constexpr int OFF_W1 = RIFT_CLOSURE_OFF_W1, OFF_B1 = RIFT_CLOSURE_OFF_B1;
constexpr int OFF_W2 = RIFT_CLOSURE_OFF_W2, OFF_B2 = RIFT_CLOSURE_OFF_B2;
constexpr int OFF_W3 = RIFT_CLOSURE_OFF_W3, OFF_B3 = RIFT_CLOSURE_OFF_B3;
static_assert(OFF_B1 == OFF_W1 + C1 * K1P && OFF_W2 == OFF_B1 + C1 && OFF_B2 == OFF_W2 + C1 * K2 &&
                  OFF_W3 == OFF_B2 + C1 && OFF_B3 == OFF_W3 + 8 * C1 &&
                  RIFT_CLOSURE_NPARAM == OFF_B3 + 8,
              "parameter layout");

struct NetSmem {
    float xs[NRI * CIN];       // scaled inputs (FP32), channels last
    uint16_t xb[NRI * CB];     // the same as BF16 rows of 8; the bed relative to bref, in two halves
    uint16_t a1[NR1 * SA];     // layer-1 activations (BF16); dZ1 in the backward pass
    uint16_t w1[C1 * SW1];     // W1 over the BF16 inputs: [o][tap*8 + c8]
    uint16_t w2[C1 * SW2];     // W2[o][k]
    uint16_t w3[8 * SW3];      // W3[o][c], rows 4..7 zero
    float b1[C1], b2[C1], b3[8];
    float sbed[C1];            // sum over taps of layer 1's (BF16) bed weights
    int toff[NTAP1];           // cell offset of each layer-1 tap in the input block
    int koffE[K1P];            // xs offset of each layer-1 reduction index (weight gradient)
    float bref;                // the block's reference bed (scaled)
    int red[4];
};

struct TrainSmem {
    NetSmem n;
    uint16_t a2[OT * OT * SA];  // layer-2 activations, then dZ2
    uint16_t w2t[K2 * SA];      // W2 transposed: [k][o]
    float dout[OT * OT * 4];
    float w3f[4 * C1];
    double red[NT / 32];
};

__device__ __forceinline__ uint16_t bf(float x) { return __bfloat16_as_ushort(__float2bfloat16_rn(x)); }
__device__ __forceinline__ float fb(uint16_t x) { return __bfloat162float(__ushort_as_bfloat16(x)); }
__device__ __forceinline__ uint32_t pack2(float lo, float hi) {
    return (uint32_t)bf(lo) | ((uint32_t)bf(hi) << 16);
}
__device__ __forceinline__ uint32_t pack16(uint16_t lo, uint16_t hi) {
    return (uint32_t)lo | ((uint32_t)hi << 16);
}
__device__ __forceinline__ uint32_t ld32(const uint16_t* p) {
    return *reinterpret_cast<const uint32_t*>(p);
}
__device__ __forceinline__ void st32(uint16_t* p, uint32_t v) { *reinterpret_cast<uint32_t*>(p) = v; }
__device__ __forceinline__ float relu(float x) { return fmaxf(x, 0.f); }

// D += A(16x16, row) * B(16x8, col), BF16 inputs, FP32 accumulators.
// Fragments (g = lane/4, t = lane%4): a[0] rows g, cols 2t..2t+1; a[1] rows
// g+8; a[2] rows g, cols 2t+8..; a[3] rows g+8, cols 2t+8..; b0 rows (k)
// 2t..2t+1 of col g, b1 rows 2t+8..; d[0..1] row g cols 2t..2t+1, d[2..3]
// row g+8.
__device__ __forceinline__ void mma16816(float d[4], const uint32_t a[4], uint32_t b0, uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, "
        "{%8,%9}, {%0,%1,%2,%3};"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// Four 8x8 BF16 matrices from shared memory; lane l gives the address of
// row l%8 of matrix l/8, and r[i] receives matrix i in the MMA fragment
// layout (thread T: row T/4, columns 2(T%4), 2(T%4)+1).  Row addresses are
// 16-byte aligned.
__device__ __forceinline__ void ldsm4(uint32_t r[4], const void* p) {
    const uint32_t a = (uint32_t)__cvta_generic_to_shared(p);
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
                 : "r"(a));
}

// Weights (BF16), biases and the layer-1 offset tables, once per CTA.
// Layer 1 reads the BF16 input rows (h, hu, hv, b_hi, b_lo, n, rain, 0):
// both bed halves take the bed weight.
__device__ void stageNet(NetSmem& S, const float* __restrict__ P) {
    const int tid = threadIdx.x;
    constexpr int MAP[CB] = {0, 1, 2, 3, 3, 4, 5, -1};
    for (int i = tid; i < C1 * SW1; i += NT) {
        const int o = i / SW1, k = i % SW1, tap = k / CB, c = MAP[k % CB];
        S.w1[i] = bf(k < K1B && tap < 25 && c >= 0 ? P[OFF_W1 + o * K1P + tap * CIN + c] : 0.f);
    }
    for (int i = tid; i < C1 * SW2; i += NT) {
        int o = i / SW2, k = i % SW2;
        S.w2[i] = bf(k < K2 ? P[OFF_W2 + o * K2 + k] : 0.f);
    }
    for (int i = tid; i < 8 * SW3; i += NT) {
        int o = i / SW3, k = i % SW3;
        S.w3[i] = bf(o < COUT && k < C1 ? P[OFF_W3 + o * C1 + k] : 0.f);
    }
    if (tid < C1) {
        S.b1[tid] = P[OFF_B1 + tid];
        S.b2[tid] = P[OFF_B2 + tid];
        float sb = 0.f;
        for (int tap = 0; tap < 25; tap++) sb += fb(bf(P[OFF_W1 + tid * K1P + tap * CIN + 3]));
        S.sbed[tid] = sb;
    }
    if (tid < 8) S.b3[tid] = tid < COUT ? P[OFF_B3 + tid] : 0.f;
    if (tid < NTAP1) S.toff[tid] = tid < 25 ? (tid / 5) * RI + tid % 5 : 0;
    for (int k = tid; k < K1P; k += NT) {
        int e = -1;
        if (k < K1) {
            int tap = k / CIN, c = k % CIN;
            e = ((tap / 5) * RI + tap % 5) * CIN + c;
            if (c == 3) e |= BEDBIT;
        }
        S.koffE[k] = e;
    }
}

// The 22 x 22 input block whose corner is image cell (Y0, X0) of sample s:
// FP32 (xs) and BF16 rows (xb).  The BF16 bed is b - bref, bref the bed of
// the block's centre cell, split into a BF16 value and its BF16 remainder
// (16 significant bits together).
__device__ void stageInput(NetSmem& S, const rift_closure_src& src, int s, int Y0, int X0) {
    const size_t sbase = (size_t)s * (size_t)src.sample_stride;
    auto at = [&](int ry, int rx) {
        int y = min(max(Y0 + ry, 0), src.H - 1), x = min(max(X0 + rx, 0), src.W - 1);
        return sbase + (size_t)y * (size_t)src.pitch + (size_t)x;
    };
    const float bref = (src.plane[3] ? __ldg(src.plane[3] + at(RI / 2, RI / 2)) : src.value[3]) * src.scale[3];
    if (threadIdx.x == 0) S.bref = bref;
    for (int i = threadIdx.x; i < NRI; i += NT) {
        const size_t off = at(i / RI, i % RI);
        float v[CIN];
#pragma unroll
        for (int c = 0; c < CIN; c++) {
            v[c] = (src.plane[c] ? __ldg(src.plane[c] + off) : src.value[c]) * src.scale[c];
            S.xs[i * CIN + c] = v[c];
        }
        const float br = v[3] - bref;
        const uint16_t bh = bf(br);
        const uint16_t bl = bf(br - fb(bh));
        uint4 w;
        w.x = pack2(v[0], v[1]);
        w.y = pack16(bf(v[2]), bh);
        w.z = pack16(bl, bf(v[4]));
        w.w = pack16(bf(v[5]), 0);
        *reinterpret_cast<uint4*>(&S.xb[i * CB]) = w;
    }
}

// Layer-1 input k (tap, channel) of the cell whose 5x5 window starts at xs
// offset `base`, FP32: the bed relative to the window's centre bc.
__device__ __forceinline__ float featElem(const NetSmem& S, int base, float bc, int e) {
    if (e < 0) return 0.f;
    float v = S.xs[base + (e & OFFMASK)];
    return (e & BEDBIT) ? v - bc : v;
}
__device__ __forceinline__ int winBase(int q) { return ((q / R1) * RI + q % R1) * CIN; }
__device__ __forceinline__ float winBed(const NetSmem& S, int base) {
    return S.xs[base + (2 * RI + 2) * CIN + 3];
}

// Layer 1 on the 18 x 18 region: a1 = relu(W1 x + b1), BF16.  A warp owns
// row tiles warp, warp+8 and (warps 0..4) warp+16.  One k step covers two
// taps of the 8-channel BF16 input rows, so each 8 x 8 block of an A
// fragment is 8 cells' rows of one tap and comes with one ldmatrix; the
// bed enters relative to bref and the epilogue subtracts (centre bed -
// bref) x (sum of the bed weights), which makes it relative to the
// window's centre.
__device__ void conv1(NetSmem& S, int warp, int lane) {
    const int g = lane >> 2, t = lane & 3;
    constexpr int MPW = (M1T + 7) / 8;  // 3
    const bool third = warp + 16 < M1T;
    // this lane's ldmatrix rows: row (lane & 15) of each of its row tiles,
    // the tap of the k step's second half for lanes 16..31
    const int lrow = lane & 15, lhalf = lane >> 4;
    int rowCell[MPW];
#pragma unroll
    for (int j = 0; j < MPW; j++) {
        const int q = min(min(warp + 8 * j, M1T - 1) * 16 + lrow, NR1 - 1);
        rowCell[j] = (q / R1) * RI + q % R1;
    }
    // weights: lanes address rows n (two column tiles per ldmatrix)
    const int wrow = (lane & 7) + ((lane >> 4) << 3), wk = ((lane >> 3) & 1) * 8;
    float acc[MPW][4][4] = {};
#pragma unroll 1
    for (int ks = 0; ks < K1B / 16; ks++) {
        uint32_t bw[4][2];
#pragma unroll
        for (int np = 0; np < 2; np++) {
            uint32_t r[4];
            ldsm4(r, &S.w1[(np * 16 + wrow) * SW1 + ks * 16 + wk]);
            bw[2 * np][0] = r[0];
            bw[2 * np][1] = r[1];
            bw[2 * np + 1][0] = r[2];
            bw[2 * np + 1][1] = r[3];
        }
        const int toff = S.toff[2 * ks + lhalf];
#pragma unroll
        for (int j = 0; j < MPW; j++) {
            if (j == MPW - 1 && !third) break;
            uint32_t a[4];
            ldsm4(a, &S.xb[(rowCell[j] + toff) * CB]);
            // ldmatrix order: rows 0-7 tap A, rows 8-15 tap A, rows 0-7 tap B, rows 8-15 tap B
#pragma unroll
            for (int nt = 0; nt < 4; nt++) mma16816(acc[j][nt], a, bw[nt][0], bw[nt][1]);
        }
    }
    const float bref = S.bref;
#pragma unroll
    for (int j = 0; j < MPW; j++) {
        const int mt = warp + 8 * j;
        if (mt >= M1T) break;
        const int r0 = mt * 16 + g, r1 = r0 + 8;
        const float c0 = winBed(S, winBase(min(r0, NR1 - 1))) - bref;
        const float c1 = winBed(S, winBase(min(r1, NR1 - 1))) - bref;
#pragma unroll
        for (int nt = 0; nt < 4; nt++) {
            const int o = nt * 8 + 2 * t;
            const float s0 = S.sbed[o], s1 = S.sbed[o + 1];
            if (r0 < NR1)
                st32(&S.a1[r0 * SA + o], pack2(relu(acc[j][nt][0] + S.b1[o] - c0 * s0),
                                               relu(acc[j][nt][1] + S.b1[o + 1] - c0 * s1)));
            if (r1 < NR1)
                st32(&S.a1[r1 * SA + o], pack2(relu(acc[j][nt][2] + S.b1[o] - c1 * s0),
                                               relu(acc[j][nt][3] + S.b1[o + 1] - c1 * s1)));
        }
    }
}

// Layers 2 and 3 on output rows warp and warp+8 (one weight fragment load
// for both; A and B fragments by ldmatrix).  z2: layer-2 pre-activations
// (accumulator fragments); out[m]: layer-3 outputs of rows g and g+8 of
// output row warp+8m, channels 2t and 2t+1 (t < 2 valid).
__device__ void conv23(const NetSmem& S, int warp, int lane, float z2[2][4][4], float out[2][4]) {
    const int g = lane >> 2, t = lane & 3;
    const int lrow = lane & 15, lk = (lane >> 4) * 8;  // A: row, k offset of this lane's address
    const int wrow = (lane & 7) + ((lane >> 4) << 3), wk = ((lane >> 3) & 1) * 8;
    float acc[2][4][4] = {};
#pragma unroll 1
    for (int tap = 0; tap < 9; tap++) {
        const int dy = tap / 3, dx = tap % 3;
        const uint16_t* p0 = &S.a1[((warp + dy) * R1 + lrow + dx) * SA + lk];
        const uint16_t* p1 = p0 + 8 * R1 * SA;
#pragma unroll
        for (int kb = 0; kb < 2; kb++) {
            const int kk = tap * 32 + kb * 16;
            uint32_t bw[4][2];
#pragma unroll
            for (int np = 0; np < 2; np++) {
                uint32_t r[4];
                ldsm4(r, &S.w2[(np * 16 + wrow) * SW2 + kk + wk]);
                bw[2 * np][0] = r[0];
                bw[2 * np][1] = r[1];
                bw[2 * np + 1][0] = r[2];
                bw[2 * np + 1][1] = r[3];
            }
#pragma unroll
            for (int m = 0; m < 2; m++) {
                uint32_t a[4];
                ldsm4(a, (m ? p1 : p0) + kb * 16);
#pragma unroll
                for (int nt = 0; nt < 4; nt++) mma16816(acc[m][nt], a, bw[nt][0], bw[nt][1]);
            }
        }
    }
#pragma unroll
    for (int m = 0; m < 2; m++) {
#pragma unroll
        for (int nt = 0; nt < 4; nt++) {
            const int o = nt * 8 + 2 * t;
            z2[m][nt][0] = acc[m][nt][0] + S.b2[o];
            z2[m][nt][1] = acc[m][nt][1] + S.b2[o + 1];
            z2[m][nt][2] = acc[m][nt][2] + S.b2[o];
            z2[m][nt][3] = acc[m][nt][3] + S.b2[o + 1];
        }
        float acc3[4] = {};
#pragma unroll
        for (int kb = 0; kb < 2; kb++) {
            uint32_t a[4];
            a[0] = pack2(relu(z2[m][2 * kb][0]), relu(z2[m][2 * kb][1]));
            a[1] = pack2(relu(z2[m][2 * kb][2]), relu(z2[m][2 * kb][3]));
            a[2] = pack2(relu(z2[m][2 * kb + 1][0]), relu(z2[m][2 * kb + 1][1]));
            a[3] = pack2(relu(z2[m][2 * kb + 1][2]), relu(z2[m][2 * kb + 1][3]));
            const uint16_t* w = &S.w3[g * SW3 + kb * 16 + 2 * t];
            mma16816(acc3, a, ld32(w), ld32(w + 8));
        }
        const int c = 2 * t;  // b3 holds 8 entries, zero past the fourth
        out[m][0] = acc3[0] + S.b3[c];
        out[m][1] = acc3[1] + S.b3[c + 1];
        out[m][2] = acc3[2] + S.b3[c];
        out[m][3] = acc3[3] + S.b3[c + 1];
    }
}

struct TileGeom {
    int s, Y, X;  // sample and image coordinates of the tile's first output cell
};
__device__ __forceinline__ TileGeom tileGeom(const rift_closure_src& src, int tile) {
    const int tx = (src.OW + OT - 1) / OT, ty = (src.OH + OT - 1) / OT;
    TileGeom G;
    G.s = tile / (tx * ty);
    int r = tile % (tx * ty);
    G.Y = src.oy0 + (r / tx) * OT;
    G.X = src.ox0 + (r % tx) * OT;
    return G;
}
__host__ __device__ __forceinline__ int tileCount(const rift_closure_src& src) {
    return src.samples * ((src.OW + OT - 1) / OT) * ((src.OH + OT - 1) / OT);
}

// ------------------------------------------------- tcgen05 forward (inference)
// The forward pass of k_forward and k_closure on the 5th-generation tensor
// cores: layers 1 and 2 are tcgen05.mma (kind::f16, BF16 operands from
// shared memory, FP32 accumulators in tensor memory), issued by one thread;
// layer 3 (32 -> 4) runs in FP32 on the CUDA cores in the layer-2 epilogue.
//
// Implicit GEMM without an im2col copy.  The input block and the layer-1
// activations are stored as cells of 8 BF16 channels (16 bytes, one row of
// an 8 x 16-byte core matrix), cell (y, x) of the 22-wide block at linear
// index y*22 + x.  An MMA row is a linear cell index m, so the eight rows of
// a core matrix are eight consecutive cells (16-byte stride) and the row
// groups are 128 bytes apart; the operand of tap (dy, dx) is the same
// layout started dy*22 + dx cells later.  Rows whose column m % 22 is past
// the valid width compute values that no valid output reads.
//  layer 1: M = 512 rows (4 tiles of 128; the 18 x 18 region is rows
//           m < 396 with m % 22 < 18), N = 32, K = 15 steps of 16: taps
//           (dy, dx) and (dy+1, dx) for dy = 0, 2, 4 (dy = 5 carries zero
//           weights), the two 8-channel K chunks 22 cells apart;
//  layer 2: M = 384 rows (3 tiles; the 16 x 16 outputs are rows m < 352
//           with m % 22 < 16), N = 32, K = 9 taps x 2 steps of 16 over the
//           four 8-channel planes of the layer-1 activations.
// Tensor memory: 128 columns, one 32-column accumulator per M tile (layer 2
// reuses the columns of layer 1 once its epilogue has read them).  A CTA
// holds 74 KB of shared memory and 80 registers per thread, so three run on
// an SM (384 of the 512 tensor-memory columns); the epilogues read the
// accumulators 8 columns at a time to stay within the registers.
constexpr int XBC = 640;             // BF16 input cells staged (reads reach m + 5*22 + 4 < 640)
constexpr int A1C = 432;             // layer-1 cells kept per plane (layer 2 reads < 384 + 46)
constexpr int M1TC = 4, M2TC = 3;    // M tiles of 128 rows
constexpr int KS1 = 15, KS2 = 18;    // K steps of 16
constexpr int NTAPT = 26;            // layer-1 weight blocks: the 25 taps, then one of zeros
constexpr uint32_t TMEM_COLS = 128;
constexpr uint32_t A1PLANE = A1C * 16;  // bytes per 8-channel plane
// instruction descriptor, kind::f16: FP32 accumulator (bits 4-5 = 1), A and B
// BF16 (bits 7-9, 10-12 = 1), both K-major, N >> 3 at bits 17-22, M >> 4 at
// bits 24-28
constexpr uint32_t IDESC = (1u << 4) | (1u << 7) | (1u << 10) | ((32u >> 3) << 17) | ((128u >> 4) << 24);

struct __align__(128) TcSmem {
    uint16_t xb[XBC * 8];        // input cells (BF16 x 8), zero past the 22 x 22 block
    uint16_t a1[4][A1C * 8];     // layer-1 activations, channels 8p..8p+7 in plane p
    uint16_t w1t[NTAPT * 32 * 8];  // [dy*5 + dx][o][c8]; block 25 all zero
    uint16_t w2t[36 * 32 * 8];   // [tap*4 + c/8][o][c%8]
    float xh[NRI];               // scaled FP32 depth of the input cells
    float xbed[NRI];             // scaled FP32 bed of the input cells
    float w3[COUT][C1];
    float b1[C1], b2[C1], b3[COUT], sbed[C1];
    float bref;
    int red[2];
    uint64_t bar;
    uint32_t tmem;
};
static_assert(offsetof(TcSmem, a1) % 16 == 0 && offsetof(TcSmem, w1t) % 16 == 0 &&
                  offsetof(TcSmem, w2t) % 16 == 0 && offsetof(TcSmem, bar) % 8 == 0,
              "operand alignment");

__device__ int g_tc_error;  // 1: a tensor-core completion wait gave up

__device__ __forceinline__ uint32_t saddr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// Shared-memory matrix descriptor (tcgen05): start address, leading (K)
// and stride (M/N) byte offsets, each >> 4; version 1 at bit 46; no swizzle.
__device__ __forceinline__ uint64_t sdesc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((addr & 0x3FFFFu) >> 4) | ((uint64_t)(lbo >> 4) << 16) |
           ((uint64_t)(sbo >> 4) << 32) | (1ull << 46);
}
__device__ __forceinline__ void tc_mma(uint32_t d, uint64_t a, uint64_t b, bool acc) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d),
        "l"(a), "l"(b), "r"(IDESC), "r"((uint32_t)acc)
        : "memory");
}
__device__ __forceinline__ void tc_commit(uint64_t* bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                     saddr(bar))
                 : "memory");
}
__device__ __forceinline__ void tc_before_sync() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_after_sync() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void proxy_fence() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void bar_init(uint64_t* bar) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(saddr(bar)) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
// Bounded wait on an mbarrier phase: false after the spin limit.
__device__ __forceinline__ bool bar_wait(uint64_t* bar, uint32_t parity) {
    for (int it = 0; it < (1 << 22); ++it) {
        uint32_t ok;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
            " selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(ok)
            : "r"(saddr(bar)), "r"(parity)
            : "memory");
        if (ok) return true;
    }
    return false;
}
// 32 consecutive FP32 columns of this thread's tensor-memory lane.
__device__ __forceinline__ void tc_ld32(uint32_t taddr, float v[32]) {
    uint32_t r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,"
        "%15,%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
          "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
          "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]),
          "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]),
          "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr)
        : "memory");
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int k = 0; k < 32; k++) v[k] = __uint_as_float(r[k]);
}

// 8 consecutive FP32 columns of this thread's tensor-memory lane.
__device__ __forceinline__ void tc_ld8(uint32_t taddr, float v[8]) {
    uint32_t r[8];
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
                   "=r"(r[7])
                 : "r"(taddr)
                 : "memory");
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int k = 0; k < 8; k++) v[k] = __uint_as_float(r[k]);
}

// Weights in the operand layouts, biases, the bed-weight sums; the zero pad
// of the input cells.  Tensor memory (warp 0) and the completion barrier.
__device__ void tcSetup(TcSmem& S, const float* __restrict__ P) {
    const int tid = threadIdx.x;
    constexpr int MAP[CB] = {0, 1, 2, 3, 3, 4, 5, -1};
    for (int i = tid; i < NTAPT * 32 * 8; i += NT) {
        const int T = i / 256, o = (i / 8) % 32, c8 = i % 8, c = MAP[c8];
        S.w1t[i] = bf(T < 25 && c >= 0 ? P[OFF_W1 + o * K1P + T * CIN + c] : 0.f);
    }
    for (int i = tid; i < 36 * 32 * 8; i += NT) {
        const int blk = i / 256, o = (i / 8) % 32, c8 = i % 8;
        S.w2t[i] = bf(P[OFF_W2 + o * K2 + (blk >> 2) * 32 + (blk & 3) * 8 + c8]);
    }
    for (int i = tid; i < COUT * C1; i += NT) S.w3[i / C1][i % C1] = P[OFF_W3 + i];
    for (int i = tid; i < (XBC - NRI) * 8; i += NT) S.xb[NRI * 8 + i] = 0;
    if (tid < C1) {
        S.b1[tid] = P[OFF_B1 + tid];
        S.b2[tid] = P[OFF_B2 + tid];
        float sb = 0.f;
        for (int tap = 0; tap < 25; tap++) sb += fb(bf(P[OFF_W1 + tid * K1P + tap * CIN + 3]));
        S.sbed[tid] = sb;
    }
    if (tid < COUT) S.b3[tid] = P[OFF_B3 + tid];
    if (tid == 0) bar_init(&S.bar);
    if (tid < 32) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                         saddr(&S.tmem)),
                     "r"(TMEM_COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_before_sync();
    __syncthreads();
    tc_after_sync();
}

__device__ void tcTeardown(TcSmem& S) {
    tc_before_sync();
    __syncthreads();
    tc_after_sync();
    if (threadIdx.x < 32)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(S.tmem),
                     "r"(TMEM_COLS)
                     : "memory");
}

// A block's raw inputs in registers: this thread's cells i = tid and
// tid + NT of the 22 x 22 block (484 < 2 NT), and the block's reference bed.
// Loaded one block ahead, while the tensor cores work on the current one.
struct TcInput {
    float v[2][CIN];
    float bref;
};
__device__ void tcLoadInput(TcInput& R, const rift_closure_src& src, int s, int Y0, int X0) {
    const size_t sbase = (size_t)s * (size_t)src.sample_stride;
    auto at = [&](int ry, int rx) {
        int y = min(max(Y0 + ry, 0), src.H - 1), x = min(max(X0 + rx, 0), src.W - 1);
        return sbase + (size_t)y * (size_t)src.pitch + (size_t)x;
    };
    R.bref = src.plane[3] ? __ldg(src.plane[3] + at(RI / 2, RI / 2)) : src.value[3];
#pragma unroll
    for (int k = 0; k < 2; k++) {
        const int i = threadIdx.x + k * NT;
        if (i >= NRI) break;
        const size_t off = at(i / RI, i % RI);
#pragma unroll
        for (int c = 0; c < CIN; c++) R.v[k][c] = src.plane[c] ? __ldg(src.plane[c] + off) : src.value[c];
    }
}

// The loaded block into shared memory: scaled FP32 values (xs) and the
// BF16 cells of the layer-1 operand (the bed relative to bref in two
// halves); each writer fences its shared stores for the async proxy.
__device__ void tcStoreInput(TcSmem& S, const TcInput& R, const rift_closure_src& src) {
    const float bref = R.bref * src.scale[3];
    if (threadIdx.x == 0) S.bref = bref;
#pragma unroll
    for (int k = 0; k < 2; k++) {
        const int i = threadIdx.x + k * NT;
        if (i >= NRI) break;
        float v[CIN];
#pragma unroll
        for (int c = 0; c < CIN; c++) v[c] = R.v[k][c] * src.scale[c];
        S.xh[i] = v[0];
        S.xbed[i] = v[3];
        const float br = v[3] - bref;
        const uint16_t bh = bf(br);
        const uint16_t bl = bf(br - fb(bh));
        uint4 w;
        w.x = pack2(v[0], v[1]);
        w.y = pack16(bf(v[2]), bh);
        w.z = pack16(bl, bf(v[4]));
        w.w = pack16(bf(v[5]), 0);
        *reinterpret_cast<uint4*>(&S.xb[i * CB]) = w;
    }
    proxy_fence();
}

// Thread 0: the MMAs of one layer, then their completion on the barrier.
// The loops unroll completely: every operand offset is a compile-time
// constant added to a base descriptor (its address field counts 16-byte
// units, and no shared address reaches 256 KB, so the sum never carries out
// of the field), so the issuing thread spends a few instructions per MMA.
__device__ void tcIssue1(const TcSmem& S, uint32_t tmem) {
    tc_after_sync();
    // B: the K chunks of step s are taps (dy, dx) and (dy + 1, dx), dy = 2(s/5), five weight
    // blocks apart; for dy = 4 the second chunk is the zero block
    const uint64_t a0 = sdesc(saddr(S.xb), RI * 16, 128), b0 = sdesc(saddr(S.w1t), 0, 128);
#pragma unroll
    for (int mt = 0; mt < M1TC; mt++)
#pragma unroll
        for (int s = 0; s < KS1; s++) {
            const uint32_t cell = mt * 128 + (s / 5) * 2 * RI + s % 5;  // 16-byte cells
            const uint32_t T0 = (s / 5) * 10 + s % 5, T1 = s < 10 ? T0 + 5 : 25;
            const uint64_t lbo = (uint64_t)((T1 - T0) * 512 / 16) << 16;
            tc_mma(tmem + mt * 32, a0 + cell, b0 + T0 * (512 / 16) + lbo, s > 0);
        }
    tc_commit(const_cast<uint64_t*>(&S.bar));
}
__device__ void tcIssue2(const TcSmem& S, uint32_t tmem) {
    tc_after_sync();
    const uint64_t a0 = sdesc(saddr(S.a1), A1PLANE, 128), b0 = sdesc(saddr(S.w2t), 512, 128);
#pragma unroll
    for (int mt = 0; mt < M2TC; mt++)
#pragma unroll
        for (int s = 0; s < KS2; s++) {
            const int tap = s >> 1, kb = s & 1;
            const uint32_t cell = kb * 2 * A1C + mt * 128 + (tap / 3) * RI + tap % 3;
            tc_mma(tmem + mt * 32, a0 + cell, b0 + (tap * 4 + 2 * kb) * (512 / 16), s > 0);
        }
    tc_commit(const_cast<uint64_t*>(&S.bar));
}

// Wait for the layer's MMAs (every thread); false (and the device error
// flag set) when the wait gave up, after a second bounded wait for them.
__device__ bool tcWait(TcSmem& S, uint32_t& phase) {
    const bool ok = __syncthreads_and(bar_wait(&S.bar, phase));
    if (!ok) {
        bar_wait(&S.bar, phase);
        if (threadIdx.x == 0) atomicOr(&g_tc_error, 1);
    }
    phase ^= 1u;
    tc_after_sync();
    return ok;
}

// Layer-1 epilogue: rows of M tiles warp/4 and warp/4 + 2 at this warp's
// tensor-memory lanes -> relu(acc + b1 - (centre bed - bref) sbed) as BF16
// into the activation planes.
__device__ void tcEpilogue1(TcSmem& S, uint32_t tmem) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, lg = warp & 3;
    const float bref = S.bref;
#pragma unroll 1
    for (int mt = warp >> 2; mt < M1TC; mt += 2) {
        const int m = mt * 128 + 32 * lg + lane;
        const float cb = S.xbed[min(m, A1C - 1) + 2 * RI + 2] - bref;
#pragma unroll
        for (int p = 0; p < 4; p++) {  // 8 channels (one plane) at a time
            float v[8];
            tc_ld8(tmem + ((uint32_t)(32 * lg) << 16) + mt * 32 + 8 * p, v);
            if (m >= A1C) continue;
            uint4 w;
            uint32_t q[4];
#pragma unroll
            for (int e = 0; e < 4; e++) {
                const int o = 8 * p + 2 * e;
                q[e] = pack2(relu(v[2 * e] + S.b1[o] - cb * S.sbed[o]),
                             relu(v[2 * e + 1] + S.b1[o + 1] - cb * S.sbed[o + 1]));
            }
            w.x = q[0];
            w.y = q[1];
            w.z = q[2];
            w.w = q[3];
            *reinterpret_cast<uint4*>(&S.a1[p][m * 8]) = w;
        }
    }
    proxy_fence();
    tc_before_sync();
}

// Layer-2 epilogue and layer 3 for the row of M tile mt at this thread's
// lane: out = W3 relu(acc + b2) + b3.  Returns the output cell's index in
// the 16 x 16 tile (oy*16 + ox), or -1 for a row that is not an output.
__device__ int tcOutputs(const TcSmem& S, uint32_t tmem, int mt, float out[COUT]) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, lg = warp & 3;
    const int m = mt * 128 + 32 * lg + lane, oy = m / RI, ox = m % RI;
#pragma unroll
    for (int c = 0; c < COUT; c++) out[c] = S.b3[c];
#pragma unroll
    for (int q = 0; q < 4; q++) {  // 8 channels at a time
        float v[8];
        tc_ld8(tmem + ((uint32_t)(32 * lg) << 16) + mt * 32 + 8 * q, v);
#pragma unroll
        for (int k = 0; k < 8; k++) {
            const float a = relu(v[k] + S.b2[8 * q + k]);
#pragma unroll
            for (int c = 0; c < COUT; c++) out[c] = fmaf(S.w3[c][8 * q + k], a, out[c]);
        }
    }
    return (oy >= OT || ox >= OT) ? -1 : oy * OT + ox;
}

// One tcgen05.mma (M 128, N 32, K 16) on fixed BF16 values, with the
// operand layout of the forward pass (K-major, no swizzle, 8-row groups
// 128 bytes apart, the two K chunks LBO bytes apart: 2048 for A, 512 for B),
// and the accumulator read back through tcgen05.ld: out[row * 32 + col] = D.
// A[r][k] = (r % 7) - 3 + (k % 5) / 4, B[n][k] = (n % 5) - 2 + (k % 3) / 2,
// so every product and sum is exact in FP32.  The buffers are larger than
// the operands so that any reading of the two offsets stays inside them.
__global__ void __launch_bounds__(128) k_tc_selftest(float* __restrict__ out) {
    __shared__ __align__(128) uint16_t a[16384];
    __shared__ __align__(128) uint16_t b[1024];
    __shared__ uint64_t bar;
    __shared__ uint32_t tm;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    for (int i = tid; i < 16384; i += 128) a[i] = 0;
    for (int i = tid; i < 1024; i += 128) b[i] = 0;
    __syncthreads();
    for (int i = tid; i < 128 * 16; i += 128) {
        const int r = i / 16, k = i % 16;
        a[((r / 8) * 128 + (k / 8) * 2048 + (r % 8) * 16) / 2 + k % 8] = bf((r % 7) - 3 + 0.25f * (k % 5));
    }
    for (int i = tid; i < 32 * 16; i += 128) {
        const int n = i / 16, k = i % 16;
        b[((n / 8) * 128 + (k / 8) * 512 + (n % 8) * 16) / 2 + k % 8] = bf((n % 5) - 2 + 0.5f * (k % 3));
    }
    proxy_fence();
    if (tid == 0) bar_init(&bar);
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(saddr(&tm)),
                     "r"(TMEM_COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_before_sync();
    __syncthreads();
    tc_after_sync();
    const uint32_t tmem = tm;
    if (tid == 0) {
        tc_mma(tmem, sdesc(saddr(a), 2048, 128), sdesc(saddr(b), 512, 128), false);
        tc_commit(&bar);
    }
    const bool ok = __syncthreads_and(bar_wait(&bar, 0));
    if (!ok) {
        bar_wait(&bar, 0);
        if (tid == 0) atomicOr(&g_tc_error, 1);
    }
    tc_after_sync();
    if (ok) {
        float v[32];
        tc_ld32(tmem + ((uint32_t)(32 * warp) << 16), v);
#pragma unroll
        for (int c = 0; c < 32; c++) out[(32 * warp + lane) * 32 + c] = v[c];
    }
    tc_before_sync();
    __syncthreads();
    tc_after_sync();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS)
                     : "memory");
}

// ------------------------------------------------------------------ forward
// Raw net outputs of every output cell of src.
__global__ void __launch_bounds__(NT, 3) k_forward(rift_closure_src src, const float* __restrict__ P,
                                                   float* __restrict__ out) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    TcSmem& S = *reinterpret_cast<TcSmem*>(smem_raw);
    const int warp = threadIdx.x >> 5;
    tcSetup(S, P);
    const uint32_t tmem = S.tmem;
    uint32_t phase = 0;
    const int ntile = tileCount(src);
    TcInput R;
    if ((int)blockIdx.x < ntile) {
        const TileGeom G0 = tileGeom(src, blockIdx.x);
        tcLoadInput(R, src, G0.s, G0.Y - 3, G0.X - 3);
    }
    for (int tile = blockIdx.x; tile < ntile; tile += gridDim.x) {
        const TileGeom G = tileGeom(src, tile);
        __syncthreads();
        tcStoreInput(S, R, src);
        __syncthreads();
        if (threadIdx.x == 0) tcIssue1(S, tmem);
        if (tile + (int)gridDim.x < ntile) {  // the next block's inputs, during the MMAs
            const TileGeom Gn = tileGeom(src, tile + gridDim.x);
            tcLoadInput(R, src, Gn.s, Gn.Y - 3, Gn.X - 3);
        }
        if (!tcWait(S, phase)) break;
        tcEpilogue1(S, tmem);
        __syncthreads();
        if (threadIdx.x == 0) tcIssue2(S, tmem);
        if (!tcWait(S, phase)) break;
#pragma unroll
        for (int k = 0; k < 2; k++) {
            const int mt = (warp >> 2) + 2 * k;
            if (mt >= M2TC) break;
            float o[COUT];
            const int q = tcOutputs(S, tmem, mt, o);
            if (q < 0) continue;
            const int y = G.Y + q / OT - src.oy0, x = G.X + q % OT - src.ox0;
            if (y >= src.OH || x >= src.OW) continue;
#pragma unroll
            for (int c = 0; c < COUT; c++)
                out[(((size_t)G.s * COUT + c) * src.OH + y) * src.OW + x] = o[c];
        }
        tc_before_sync();
    }
    tcTeardown(S);
}

// ----------------------------------------------------------------- training
struct TrainArgs {
    rift_closure_src src;
    const float* P;
    const float* target;
    const float* weight;
    float lossScale;
    float* grad;
    double* loss;
};

__global__ void __launch_bounds__(NT, 1) k_train(TrainArgs A) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    TrainSmem& T = *reinterpret_cast<TrainSmem*>(smem_raw);
    NetSmem& S = T.n;
    const rift_closure_src& src = A.src;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31, g = lane >> 2, t = lane & 3;
    stageNet(S, A.P);
    for (int i = tid; i < K2 * SA; i += NT) {
        int k = i / SA, o = i % SA;
        T.w2t[i] = bf(o < C1 ? A.P[OFF_W2 + o * K2 + k] : 0.f);
    }
    for (int i = tid; i < 4 * C1; i += NT) T.w3f[i] = A.P[OFF_W3 + i];

    // gradient accumulators held across tiles
    float gW2[9][4] = {};   // layer-2 weight tiles (rows k, cols o), see w2Tile
    float gW1[5][4] = {};   // layer-1 weight tiles, see w1Tile
    float gW3 = 0.f, gB3 = 0.f, gB2 = 0.f, gB1 = 0.f;
    double lossAcc = 0.0;

    const int ntile = tileCount(src);
    for (int tile = blockIdx.x; tile < ntile; tile += gridDim.x) {
        const TileGeom G = tileGeom(src, tile);
        __syncthreads();
        stageInput(S, src, G.s, G.Y - 3, G.X - 3);
        __syncthreads();
        conv1(S, warp, lane);
        __syncthreads();
        float z2[2][4][4], o[2][4];
        conv23(S, warp, lane, z2, o);

        // loss and d loss / d out; layer-2 activations to shared memory
#pragma unroll
        for (int m = 0; m < 2; m++) {
            const int oy = warp + 8 * m;
#pragma unroll
            for (int r = 0; r < 2; r++) {
                const int ox = g + 8 * r, p = oy * OT + ox;
                if (t < 2) {
                    const int y = G.Y + oy - src.oy0, x = G.X + ox - src.ox0;
                    const bool in = y < src.OH && x < src.OW;
#pragma unroll
                    for (int e = 0; e < 2; e++) {
                        const int ch = 2 * t + e;
                        float d = 0.f;
                        if (in) {
                            size_t at = (((size_t)G.s * COUT + ch) * src.OH + y) * src.OW + x;
                            float w = __ldg(A.weight + at);
                            float diff = o[m][2 * r + e] - __ldg(A.target + at);
                            lossAcc += (double)(w * diff * diff);
                            d = 2.f * w * diff * A.lossScale;
                        }
                        T.dout[p * 4 + ch] = d;
                    }
                }
#pragma unroll
                for (int nt = 0; nt < 4; nt++)
                    st32(&T.a2[p * SA + nt * 8 + 2 * t],
                         pack2(relu(z2[m][nt][2 * r]), relu(z2[m][nt][2 * r + 1])));
            }
        }
        __syncthreads();
        // layer 3: dW3, db3 (CUDA cores)
        {
            const int pr = tid & 127, half = tid >> 7, oc = pr >> 5, c = pr & 31;
            float acc = 0.f;
            for (int p = half * 128; p < half * 128 + 128; p++) acc += T.dout[p * 4 + oc] * fb(T.a2[p * SA + c]);
            gW3 += acc;
            if (tid < COUT) {
                float b = 0.f;
                for (int p = 0; p < OT * OT; p++) b += T.dout[p * 4 + tid];
                gB3 += b;
            }
        }
        __syncthreads();
        // dZ2 = (W3^T dout) * relu'(z2), in place of a2
        {
            const int p = tid;
            const float d0 = T.dout[p * 4], d1 = T.dout[p * 4 + 1], d2 = T.dout[p * 4 + 2],
                        d3 = T.dout[p * 4 + 3];
#pragma unroll 8
            for (int c = 0; c < C1; c++) {
                float a = fb(T.a2[p * SA + c]);
                float v = d0 * T.w3f[c] + d1 * T.w3f[C1 + c] + d2 * T.w3f[2 * C1 + c] + d3 * T.w3f[3 * C1 + c];
                T.a2[p * SA + c] = bf(a > 0.f ? v : 0.f);
            }
        }
        __syncthreads();
        {
            const int c = tid & 31, part = tid >> 5;
            float b = 0.f;
            for (int p = part; p < OT * OT; p += 8) b += fb(T.a2[p * SA + c]);
            gB2 += b;
        }
        // dW2[k][o] += sum_p a1[p + tap(k)][ch(k)] dZ2[p][o]: 18 x 4 MMA tiles,
        // nine per warp (rows w and w+8 with every column tile, then one of
        // the rows 16..17)
#pragma unroll 1
        for (int oyp = 0; oyp < OT; oyp++) {
            uint32_t bfr[4][2];
#pragma unroll
            for (int nt = 0; nt < 4; nt++) {
                const uint16_t* d = &T.a2[(oyp * OT + 2 * t) * SA + nt * 8 + g];
                bfr[nt][0] = pack16(d[0], d[SA]);
                bfr[nt][1] = pack16(d[8 * SA], d[9 * SA]);
            }
#pragma unroll
            for (int j = 0; j < 3; j++) {
                const int mt = j < 2 ? warp + 8 * j : 16 + (warp >> 2);
                const int tap = mt >> 1, ch = (mt & 1) * 16 + g, dy = tap / 3, dx = tap % 3;
                const uint16_t* r = &S.a1[((oyp + dy) * R1 + 2 * t + dx) * SA + ch];
                uint32_t a[4];
                a[0] = pack16(r[0], r[SA]);
                a[1] = pack16(r[8], r[SA + 8]);
                a[2] = pack16(r[8 * SA], r[9 * SA]);
                a[3] = pack16(r[8 * SA + 8], r[9 * SA + 8]);
                if (j < 2) {
#pragma unroll
                    for (int nt = 0; nt < 4; nt++) mma16816(gW2[4 * j + nt], a, bfr[nt][0], bfr[nt][1]);
                } else {
                    const int nt = warp & 3;
                    mma16816(gW2[8], a, bfr[nt][0], bfr[nt][1]);
                }
            }
        }
        __syncthreads();
        // dA1[q][c] = sum_{tap,o} dZ2[q - tap][o] W2[o][tap*32 + c]; dZ1 = dA1 * relu'(z1),
        // written over a1 (each element read and written by the same thread)
        for (int mt = warp; mt < M1T; mt += NT / 32) {
            const int q0 = mt * 16 + g, q1 = q0 + 8;
            const int qy0 = q0 / R1, qx0 = q0 % R1, qy1 = q1 / R1, qx1 = q1 % R1;
            float acc[4][4] = {};
#pragma unroll 1
            for (int tap = 0; tap < 9; tap++) {
                const int dy = tap / 3, dx = tap % 3;
                const int py0 = qy0 - dy, px0 = qx0 - dx, py1 = qy1 - dy, px1 = qx1 - dx;
                const bool v0 = q0 < NR1 && py0 >= 0 && py0 < OT && px0 >= 0 && px0 < OT;
                const bool v1 = q1 < NR1 && py1 >= 0 && py1 < OT && px1 >= 0 && px1 < OT;
                const uint16_t* d0 = &T.a2[(v0 ? py0 * OT + px0 : 0) * SA + 2 * t];
                const uint16_t* d1 = &T.a2[(v1 ? py1 * OT + px1 : 0) * SA + 2 * t];
#pragma unroll
                for (int ob = 0; ob < 2; ob++) {
                    uint32_t a[4];
                    a[0] = v0 ? ld32(d0 + ob * 16) : 0u;
                    a[1] = v1 ? ld32(d1 + ob * 16) : 0u;
                    a[2] = v0 ? ld32(d0 + ob * 16 + 8) : 0u;
                    a[3] = v1 ? ld32(d1 + ob * 16 + 8) : 0u;
#pragma unroll
                    for (int nt = 0; nt < 4; nt++) {
                        const uint16_t* w = &T.w2t[(tap * 32 + nt * 8 + g) * SA + ob * 16 + 2 * t];
                        mma16816(acc[nt], a, ld32(w), ld32(w + 8));
                    }
                }
            }
#pragma unroll
            for (int nt = 0; nt < 4; nt++) {
                const int c = nt * 8 + 2 * t;
                if (q0 < NR1) {
                    uint16_t* z = &S.a1[q0 * SA + c];
                    st32(z, pack2(fb(z[0]) > 0.f ? acc[nt][0] : 0.f, fb(z[1]) > 0.f ? acc[nt][1] : 0.f));
                }
                if (q1 < NR1) {
                    uint16_t* z = &S.a1[q1 * SA + c];
                    st32(z, pack2(fb(z[0]) > 0.f ? acc[nt][2] : 0.f, fb(z[1]) > 0.f ? acc[nt][3] : 0.f));
                }
            }
        }
        __syncthreads();
        {
            const int c = tid & 31, part = tid >> 5;
            float b = 0.f;
            for (int q = part; q < NR1; q += 8) b += fb(S.a1[q * SA + c]);
            gB1 += b;
        }
        // dW1[k][o] += sum_q x(q, k) dZ1[q][o]: 10 x 4 MMA tiles, five per warp
        {
            const int mtA = warp, mtB = 8 + (warp >> 2), ntB = warp & 3;
            const int eA0 = S.koffE[mtA * 16 + g], eA1 = S.koffE[mtA * 16 + g + 8];
            const int eB0 = S.koffE[mtB * 16 + g], eB1 = S.koffE[mtB * 16 + g + 8];
#pragma unroll 1
            for (int ks = 0; ks < M1T; ks++) {
                int bs[4];
                float bc[4];
                uint16_t dz[4][4];
#pragma unroll
                for (int u = 0; u < 4; u++) {
                    const int q = ks * 16 + 2 * t + (u & 1) + 8 * (u >> 1);
                    bs[u] = winBase(min(q, NR1 - 1));
                    bc[u] = winBed(S, bs[u]);
#pragma unroll
                    for (int nt = 0; nt < 4; nt++) dz[u][nt] = q < NR1 ? S.a1[q * SA + nt * 8 + g] : (uint16_t)0;
                }
                uint32_t a[4];
                a[0] = pack2(featElem(S, bs[0], bc[0], eA0), featElem(S, bs[1], bc[1], eA0));
                a[1] = pack2(featElem(S, bs[0], bc[0], eA1), featElem(S, bs[1], bc[1], eA1));
                a[2] = pack2(featElem(S, bs[2], bc[2], eA0), featElem(S, bs[3], bc[3], eA0));
                a[3] = pack2(featElem(S, bs[2], bc[2], eA1), featElem(S, bs[3], bc[3], eA1));
#pragma unroll
                for (int nt = 0; nt < 4; nt++)
                    mma16816(gW1[nt], a, pack16(dz[0][nt], dz[1][nt]), pack16(dz[2][nt], dz[3][nt]));
                a[0] = pack2(featElem(S, bs[0], bc[0], eB0), featElem(S, bs[1], bc[1], eB0));
                a[1] = pack2(featElem(S, bs[0], bc[0], eB1), featElem(S, bs[1], bc[1], eB1));
                a[2] = pack2(featElem(S, bs[2], bc[2], eB0), featElem(S, bs[3], bc[3], eB0));
                a[3] = pack2(featElem(S, bs[2], bc[2], eB1), featElem(S, bs[3], bc[3], eB1));
                mma16816(gW1[4], a, pack16(dz[0][ntB], dz[1][ntB]), pack16(dz[2][ntB], dz[3][ntB]));
            }
        }
    }

    // one addition per CTA of every gradient it holds
#pragma unroll
    for (int j = 0; j < 9; j++) {
        const int mt = j < 8 ? warp + 8 * (j >> 2) : 16 + (warp >> 2);
        const int nt = j < 8 ? (j & 3) : (warp & 3);
        const int k0 = mt * 16 + g, o0 = nt * 8 + 2 * t;
        atomicAdd(&A.grad[OFF_W2 + o0 * K2 + k0], gW2[j][0]);
        atomicAdd(&A.grad[OFF_W2 + (o0 + 1) * K2 + k0], gW2[j][1]);
        atomicAdd(&A.grad[OFF_W2 + o0 * K2 + k0 + 8], gW2[j][2]);
        atomicAdd(&A.grad[OFF_W2 + (o0 + 1) * K2 + k0 + 8], gW2[j][3]);
    }
#pragma unroll
    for (int j = 0; j < 5; j++) {
        const int mt = j < 4 ? warp : 8 + (warp >> 2);
        const int nt = j < 4 ? j : (warp & 3);
        const int k0 = mt * 16 + g, o0 = nt * 8 + 2 * t;
        if (k0 < K1) {
            atomicAdd(&A.grad[OFF_W1 + o0 * K1P + k0], gW1[j][0]);
            atomicAdd(&A.grad[OFF_W1 + (o0 + 1) * K1P + k0], gW1[j][1]);
        }
        if (k0 + 8 < K1) {
            atomicAdd(&A.grad[OFF_W1 + o0 * K1P + k0 + 8], gW1[j][2]);
            atomicAdd(&A.grad[OFF_W1 + (o0 + 1) * K1P + k0 + 8], gW1[j][3]);
        }
    }
    atomicAdd(&A.grad[OFF_W3 + (tid & 127)], gW3);
    if (tid < COUT) atomicAdd(&A.grad[OFF_B3 + tid], gB3);
    atomicAdd(&A.grad[OFF_B2 + (tid & 31)], gB2);
    atomicAdd(&A.grad[OFF_B1 + (tid & 31)], gB1);
    // loss: warp sums, then one atomic per CTA
    for (int s = 16; s > 0; s >>= 1) lossAcc += __shfl_xor_sync(0xffffffffu, lossAcc, s);
    if (lane == 0) T.red[warp] = lossAcc;
    __syncthreads();
    if (tid == 0) {
        double s = 0.0;
        for (int w = 0; w < NT / 32; w++) s += T.red[w];
        atomicAdd(A.loss, s * (double)A.lossScale);
    }
}

// --------------------------------------------------------------------- Adam
__global__ void k_adam(float* __restrict__ p, float* __restrict__ gr, float* __restrict__ m,
                       float* __restrict__ v, int n, float lr, float b1, float b2, float eps,
                       float bias1, float bias2) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        float gi = gr[i];
        float mi = b1 * m[i] + (1.f - b1) * gi;
        float vi = b2 * v[i] + (1.f - b2) * gi * gi;
        m[i] = mi;
        v[i] = vi;
        p[i] -= lr * (mi / bias1) / (sqrtf(vi / bias2) + eps);
        gr[i] = 0.f;
    }
}

// ------------------------------------------------------------ face fluxes
// Central-upwind flux through the east (DIR 0) or north (DIR 1) face of
// cell (j, i) of a handle's U^n, built as the step builds it: the
// reconstruction of both cells (construct) and the face flux (faceFlux).
template <int DIR>
__device__ __forceinline__ void faceFluxAt(const rift_device_view& V, int j, int i, float f[3]) {
    const size_t pitch = (size_t)V.pitch, pl = (size_t)V.rows * pitch;
    const int sj = DIR ? 1 : 0, si = DIR ? 0 : 1;
    auto at = [&](const float* P, int jj, int ii) { return __ldg(P + (size_t)jj * pitch + ii); };
    const float* eM = V.e + (DIR ? 2 : 0) * pl;  // eW / eS
    const float* eP = V.e + (DIR ? 3 : 1) * pl;  // eE / eN
    float hh[4], uu[4], vv[4], em[4], ep[4];
#pragma unroll
    for (int k = 0; k < 4; k++) {  // cells -1 .. +2 along DIR
        const int jj = j + (k - 1) * sj, ii = i + (k - 1) * si;
        hh[k] = at(V.h, jj, ii);
        uu[k] = at(V.hu, jj, ii);
        vv[k] = at(V.hv, jj, ii);
        em[k] = at(eM, jj, ii);
        ep[k] = at(eP, jj, ii);
    }
    const float kappa = (float)V.kappa;
    rift::Rec L = rift::construct(hh[1], uu[1], vv[1], hh[2], uu[2], vv[2], hh[0], uu[0], vv[0], em[1],
                                  ep[1], ep[1] - em[2], ep[0] - em[1]);
    rift::Rec R = rift::construct(hh[2], uu[2], vv[2], hh[3], uu[3], vv[3], hh[1], uu[1], vv[1], em[2],
                                  ep[2], ep[2] - em[3], ep[1] - em[2]);
    rift::faceFlux<DIR>(L.hP, L.uP, L.vP, R.hM, R.uM, R.vM, kappa, f);
}

__global__ void k_faceflux(rift_device_view V, int ratio, float w, float* __restrict__ acc,
                           int apitch, int arows, int anx, int any) {
    const int I = 2 + blockIdx.x * blockDim.x + threadIdx.x;
    const int J = 2 + blockIdx.y * blockDim.y + threadIdx.y;
    if (I > anx - 3 || J > any - 3) return;
    const size_t pl = (size_t)arows * apitch, c = (size_t)J * apitch + I;
    float fe[3], fn[3];
    float e0, e1, n0, n2;
    if (ratio == 1) {
        faceFluxAt<0>(V, J, I, fe);
        faceFluxAt<1>(V, J, I, fn);
        e0 = fe[0], e1 = fe[1], n0 = fn[0], n2 = fn[2];
    } else {
        const int jf = 2 * (J - 2) + 2, jf2 = jf + 1, i0 = 2 * (I - 2) + 2;
        float fa[3], fb2[3];
        faceFluxAt<0>(V, jf, i0 + 1, fa);
        faceFluxAt<0>(V, jf2, i0 + 1, fb2);
        e0 = 0.5f * (fa[0] + fb2[0]);
        e1 = 0.5f * (fa[1] + fb2[1]);
        faceFluxAt<1>(V, jf2, i0, fa);
        faceFluxAt<1>(V, jf2, i0 + 1, fb2);
        n0 = 0.5f * (fa[0] + fb2[0]);
        n2 = 0.5f * (fa[2] + fb2[2]);
    }
    acc[c] += w * e0;
    acc[pl + c] += w * e1;
    acc[2 * pl + c] += w * n0;
    acc[3 * pl + c] += w * n2;
}

// ----------------------------------------------------------- closure step
struct ApplyArgs {
    rift_closure_src src;
    const float* P;
    float osc[4];
    float* corr;
    size_t plane;
    int pitch, nx, ny;
    float dtw, inv_dx, inv_dy, hmin, lim, tau;
    uint8_t* fell;  // per 16 x 16 block: 1 when it fell back to the plain solve
    int* counters;
};

// Net outputs -> gated, limited face corrections of every 16 x 16 block of
// interior cells (zeros for dry blocks and blocks that fall back).
__global__ void __launch_bounds__(NT, 3) k_closure(ApplyArgs A) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    TcSmem& S = *reinterpret_cast<TcSmem*>(smem_raw);
    const rift_closure_src& src = A.src;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    tcSetup(S, A.P);
    const uint32_t tmem = S.tmem;
    uint32_t phase = 0;
    const float hminS = A.hmin * src.scale[0], invS0 = 1.f / src.scale[0];
    const int ntile = tileCount(src);
    TcInput R;
    if ((int)blockIdx.x < ntile) {
        const TileGeom G0 = tileGeom(src, blockIdx.x);
        tcLoadInput(R, src, 0, G0.Y - 3, G0.X - 3);
    }
    for (int tile = blockIdx.x; tile < ntile; tile += gridDim.x) {
        const TileGeom G = tileGeom(src, tile);
        __syncthreads();
        if (tid == 0) S.red[0] = 0;
        tcStoreInput(S, R, src);
        if (tile + (int)gridDim.x < ntile) {  // the next block's inputs, in flight meanwhile
            const TileGeom Gn = tileGeom(src, tile + gridDim.x);
            tcLoadInput(R, src, 0, Gn.Y - 3, Gn.X - 3);
        }
        __syncthreads();
        int wet = 0;
        for (int i = tid; i < (OT + 1) * (OT + 1); i += NT) {
            int ry = 3 + i / (OT + 1), rx = 3 + i % (OT + 1);
            wet |= S.xh[ry * RI + rx] > hminS;
        }
        if (!__syncthreads_or(wet)) {
            if (tid == 0) A.fell[tile] = 0;
            for (int i = tid; i < OT * OT; i += NT) {
                int y = G.Y + i / OT, x = G.X + i % OT;
                if (y - src.oy0 >= src.OH || x - src.ox0 >= src.OW) continue;
                size_t c = (size_t)y * A.pitch + x;
#pragma unroll
                for (int ch = 0; ch < 4; ch++) A.corr[ch * A.plane + c] = 0.f;
            }
            continue;
        }
        if (tid == 0) tcIssue1(S, tmem);
        if (!tcWait(S, phase)) break;
        tcEpilogue1(S, tmem);
        __syncthreads();
        if (tid == 0) tcIssue2(S, tmem);
        if (!tcWait(S, phase)) break;
        // this thread's output cells (up to two) and their four corrections:
        // east-face mass and momentum, north-face mass and momentum
        int cell[2] = {-1, -1};
        float cv[2][4] = {};
        float ind = 0.f;
#pragma unroll
        for (int k = 0; k < 2; k++) {
            const int mt = (warp >> 2) + 2 * k;
            if (mt >= M2TC) break;
            float o[COUT];
            const int q = tcOutputs(S, tmem, mt, o);
            if (q < 0) continue;
            const int oy = q / OT, ox = q % OT, y = G.Y + oy, x = G.X + ox;
            if (y - src.oy0 >= src.OH || x - src.ox0 >= src.OW) continue;
            cell[k] = q;
            const float hc = S.xh[(oy + 3) * RI + ox + 3] * invS0;
#pragma unroll
            for (int f = 0; f < 2; f++) {
                const bool east = f == 0;
                const float inv = east ? A.inv_dx : A.inv_dy;
                const int yn = east ? y : y + 1, xn = east ? x + 1 : x;
                const float hn = S.xh[(oy + 3 + (east ? 0 : 1)) * RI + ox + 3 + (east ? 1 : 0)] * invS0;
                const bool ok = x >= 3 && y >= 3 && xn <= A.nx - 4 && yn <= A.ny - 4 && hc > A.hmin &&
                                hn > A.hmin;
                float vm = ok ? o[2 * f] * A.osc[2 * f] : 0.f;
                const float vq = ok ? o[2 * f + 1] * A.osc[2 * f + 1] : 0.f;
                const float hd = vm > 0.f ? hc : hn;
                if (ok) {
                    ind = fmaxf(ind, fabsf(vm) * A.dtw * inv / hd);
                    const float cap = A.lim * hd / (A.dtw * inv);
                    vm = fminf(fmaxf(vm, -cap), cap);
                }
                cv[k][2 * f] = vm;
                cv[k][2 * f + 1] = vq;
            }
        }
        tc_before_sync();
        for (int s = 16; s > 0; s >>= 1) ind = fmaxf(ind, __shfl_xor_sync(0xffffffffu, ind, s));
        if (lane == 0) atomicMax(&S.red[0], __float_as_int(ind));
        __syncthreads();
        const bool fallback = __int_as_float(S.red[0]) > A.tau;
#pragma unroll
        for (int k = 0; k < 2; k++) {
            if (cell[k] < 0) continue;
            const size_t c = (size_t)(G.Y + cell[k] / OT) * A.pitch + G.X + cell[k] % OT;
#pragma unroll
            for (int ch = 0; ch < 4; ch++) A.corr[ch * A.plane + c] = fallback ? 0.f : cv[k][ch];
        }
        if (tid == 0) {
            A.fell[tile] = fallback ? 1 : 0;
            atomicAdd(&A.counters[0], 1);
            if (fallback) atomicAdd(&A.counters[1], 1);
        }
    }
    tcTeardown(S);
}

// U^n -= dtw x divergence of the face corrections (cells one inside the
// ghost ring and beyond).  A face is corrected only when neither of the
// 16 x 16 blocks of its two cells fell back: both cells then see the same
// correction (mass stays conserved) and every cell of a fallen-back block
// keeps the plain solve exactly.
__global__ void k_apply(float* __restrict__ h, float* __restrict__ hu, float* __restrict__ hv,
                        const float* __restrict__ corr, const uint8_t* __restrict__ fell, size_t plane,
                        int pitch, int nx, int ny, float sx, float sy) {
    const int i = 3 + blockIdx.x * blockDim.x + threadIdx.x;
    const int j = 3 + blockIdx.y * blockDim.y + threadIdx.y;
    if (i > nx - 4 || j > ny - 4) return;
    // a tensor-core wait of k_closure gave up: some blocks' corrections were
    // not written, so the whole step keeps the plain solve
    if (*(volatile int*)&g_tc_error) return;
    const int tx = (nx - 4 + OT - 1) / OT;
    const int bx = (i - 2) / OT, by = (j - 2) / OT;
    const bool own = fell[by * tx + bx] != 0;
    if (own) return;  // every face of this cell touches its own block
    const bool westOff = ((i - 2) % OT == 0) && fell[by * tx + bx - 1];
    const bool eastOff = ((i - 1) % OT == 0) && (i + 1 <= nx - 3) && fell[by * tx + bx + 1];
    const bool southOff = ((j - 2) % OT == 0) && fell[(by - 1) * tx + bx];
    const bool northOff = ((j - 1) % OT == 0) && (j + 1 <= ny - 3) && fell[(by + 1) * tx + bx];
    const size_t c = (size_t)j * pitch + i;
    const float mE = eastOff ? 0.f : corr[c], mW = westOff ? 0.f : corr[c - 1];
    const float mN = northOff ? 0.f : corr[2 * plane + c], mS = southOff ? 0.f : corr[2 * plane + c - pitch];
    const float uE = eastOff ? 0.f : corr[plane + c], uW = westOff ? 0.f : corr[plane + c - 1];
    const float vN = northOff ? 0.f : corr[3 * plane + c], vS = southOff ? 0.f : corr[3 * plane + c - pitch];
    if (mE == 0.f && mW == 0.f && mN == 0.f && mS == 0.f && uE == 0.f && uW == 0.f && vN == 0.f &&
        vS == 0.f)
        return;
    h[c] -= sx * (mE - mW) + sy * (mN - mS);
    hu[c] -= sx * (uE - uW);
    hv[c] -= sy * (vN - vS);
}

}  // namespace rc

// ------------------------------------------------------------------- C ABI
namespace {
thread_local std::string g_err;

int fail(int code, const std::string& msg) {
    g_err = msg;
    return code;
}

int launched(const char* what) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail(RIFT_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
    return RIFT_OK;
}

bool srcOk(const rift_closure_src* s) {
    return s && s->samples >= 1 && s->H >= 1 && s->W >= 1 && s->pitch >= s->W && s->OH >= 1 &&
           s->OW >= 1 && s->oy0 >= 0 && s->ox0 >= 0 && s->sample_stride >= 0 &&
           (s->samples == 1 || s->sample_stride >= (int64_t)s->pitch * s->H);
}

// Resident CTAs of kernel k with `smem` bytes, over every SM, capped by the
// tile count.
int residentGrid(const void* k, size_t smem, int tiles, int* out) {
    int dev = 0, sms = 0, occ = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return fail(RIFT_ERR_CUDA, "no device");
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    // the whole shared-memory carveout, so that the occupancy below (and the
    // launch) can place three 74 KB tensor-core CTAs on an SM
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k, cudaFuncAttributePreferredSharedMemoryCarveout,
                                 (int)cudaSharedmemCarveoutMaxShared);
    if (e != cudaSuccess) return fail(RIFT_ERR_CUDA, cudaGetErrorString(e));
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k, rc::NT, smem);
    if (e != cudaSuccess || occ < 1) return fail(RIFT_ERR_CUDA, "closure kernel does not fit an SM");
    // The same count from the SM's own limits (the occupancy call above gave
    // one CTA per SM for an 85 KB tensor-core kernel on GB300, where two fit
    // in shared memory and registers): CTAs per SM by shared memory (with
    // the per-block reservation) and by registers (allocated per warp in
    // units of 256), at most 4 (4 x 128 tensor-memory columns).  The kernels
    // loop over tiles with no CTA waiting on another, so a CTA that does not
    // fit simply starts when one ends.
    cudaFuncAttributes fa{};
    int smemSM = 0, resv = 0;
    if (cudaFuncGetAttributes(&fa, k) == cudaSuccess &&
        cudaDeviceGetAttribute(&smemSM, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev) == cudaSuccess &&
        cudaDeviceGetAttribute(&resv, cudaDevAttrReservedSharedMemoryPerBlock, dev) == cudaSuccess) {
        const size_t perBlock = smem + fa.sharedSizeBytes + (size_t)resv;
        const int bySmem = (int)((size_t)smemSM / perBlock);
        const int regsWarp = ((fa.numRegs * 32 + 255) / 256) * 256;
        const int byRegs = regsWarp > 0 ? 65536 / (regsWarp * (rc::NT / 32)) : 1;
        int mine = bySmem < byRegs ? bySmem : byRegs;
        mine = mine < 4 ? mine : 4;
        occ = occ > mine ? occ : mine;
    }
    *out = tiles < sms * occ ? tiles : sms * occ;
    return RIFT_OK;
}
}  // namespace

extern "C" {

int rift_closure_forward(const rift_closure_src* src, const float* params, float* out, void* stream) {
    if (!srcOk(src) || !params || !out) return fail(RIFT_ERR_ARG, "rift_closure_forward: bad argument");
    const size_t smem = sizeof(rc::TcSmem);
    const int tiles = rc::tileCount(*src);
    int grid = 0, rc_;
    if ((rc_ = residentGrid((const void*)rc::k_forward, smem, tiles, &grid))) return rc_;
    rc::k_forward<<<grid, rc::NT, smem, (cudaStream_t)stream>>>(*src, params, out);
    return launched("k_forward");
}

int rift_closure_train(const rift_closure_src* src, const float* params, const float* target,
                       const float* weight, float loss_scale, float* grad, double* loss, void* stream) {
    if (!srcOk(src) || !params || !target || !weight || !grad || !loss)
        return fail(RIFT_ERR_ARG, "rift_closure_train: bad argument");
    const size_t smem = sizeof(rc::TrainSmem);
    const int tiles = rc::tileCount(*src);
    int grid = 0, rc_;
    if ((rc_ = residentGrid((const void*)rc::k_train, smem, tiles, &grid))) return rc_;
    rc::TrainArgs A{*src, params, target, weight, loss_scale, grad, loss};
    rc::k_train<<<grid, rc::NT, smem, (cudaStream_t)stream>>>(A);
    return launched("k_train");
}

int rift_closure_adam(float* params, float* grad, float* m, float* v, int32_t n, float lr, float beta1,
                      float beta2, float eps, float bias1, float bias2, void* stream) {
    if (!params || !grad || !m || !v || n < 1 || !(bias1 > 0.f) || !(bias2 > 0.f))
        return fail(RIFT_ERR_ARG, "rift_closure_adam: bad argument");
    const int blocks = (n + 255) / 256;
    rc::k_adam<<<blocks, 256, 0, (cudaStream_t)stream>>>(params, grad, m, v, n, lr, beta1, beta2, eps,
                                                         bias1, bias2);
    return launched("k_adam");
}

int rift_closure_face_flux(const rift_device_view* view, int32_t ratio, float weight, float* acc,
                           int32_t acc_pitch, int32_t acc_rows, int32_t acc_nx, int32_t acc_ny) {
    if (!view || !acc || (ratio != 1 && ratio != 2) || acc_nx < 5 || acc_ny < 5 || acc_pitch < acc_nx ||
        acc_rows < acc_ny)
        return fail(RIFT_ERR_ARG, "rift_closure_face_flux: bad argument");
    if (view->h_nx - 4 != ratio * (acc_nx - 4) || view->h_ny - 4 != ratio * (acc_ny - 4))
        return fail(RIFT_ERR_ARG, "rift_closure_face_flux: grids do not match the ratio");
    dim3 blk(32, 8), grd((acc_nx - 4 + 31) / 32, (acc_ny - 4 + 7) / 8);
    rc::k_faceflux<<<grd, blk, 0, (cudaStream_t)view->stream>>>(*view, ratio, weight, acc, acc_pitch,
                                                                 acc_rows, acc_nx, acc_ny);
    return launched("k_faceflux");
}

int rift_closure_apply(const rift_device_view* view, const rift_closure_src* src, const float* params,
                       const float* oscale_host, float dtw, float hmin, float lim, float tau, float* corr,
                       uint8_t* block_fell, int32_t* counters) {
    if (!view || !srcOk(src) || !params || !oscale_host || !corr || !block_fell || !counters ||
        !(hmin > 0.f) || !(lim > 0.f) || !(src->scale[0] > 0.f) || src->samples != 1)
        return fail(RIFT_ERR_ARG, "rift_closure_apply: bad argument");
    // Each of a cell's four faces may carry up to lim x its depth out of it:
    // a cell deeper than hmin keeps at least hmin (1 - 4 lim), which must stay
    // above the wet threshold so that no wet cell is dried.
    if (!(lim < 0.25f) || !(hmin * (1.f - 4.f * lim) > 1.19209e-07f))
        return fail(RIFT_ERR_ARG, "rift_closure_apply: lim must be < 0.25 and hmin (1 - 4 lim) > 1.19e-7 m");
    if (src->H != view->h_ny || src->W != view->h_nx || src->pitch != view->pitch || src->oy0 != 2 ||
        src->ox0 != 2 || src->OH != view->h_ny - 4 || src->OW != view->h_nx - 4)
        return fail(RIFT_ERR_ARG, "rift_closure_apply: src is not the view's interior");
    if (!(dtw > 0.f)) return RIFT_OK;
    cudaStream_t st = (cudaStream_t)view->stream;
    rc::ApplyArgs A{};
    A.src = *src;
    A.P = params;
    for (int c = 0; c < 4; c++) A.osc[c] = oscale_host[c];
    A.corr = corr;
    A.plane = (size_t)view->rows * view->pitch;
    A.pitch = view->pitch;
    A.nx = view->h_nx;
    A.ny = view->h_ny;
    A.dtw = dtw;
    A.inv_dx = (float)(1.0 / view->dx);
    A.inv_dy = (float)(1.0 / view->dy);
    A.hmin = hmin;
    A.lim = lim;
    A.tau = tau;
    A.fell = block_fell;
    A.counters = counters;
    const size_t smem = sizeof(rc::TcSmem);
    const int tiles = rc::tileCount(*src);
    int grid = 0, rc_;
    if ((rc_ = residentGrid((const void*)rc::k_closure, smem, tiles, &grid))) return rc_;
    rc::k_closure<<<grid, rc::NT, smem, st>>>(A);
    if ((rc_ = launched("k_closure"))) return rc_;
    dim3 blk(32, 8), grd((view->h_nx - 6 + 31) / 32, (view->h_ny - 6 + 7) / 8);
    rc::k_apply<<<grd, blk, 0, st>>>(view->h, view->hu, view->hv, corr, block_fell, A.plane, view->pitch,
                                     view->h_nx, view->h_ny, (float)(dtw / view->dx), (float)(dtw / view->dy));
    return launched("k_apply");
}

int rift_closure_selftest(float* out, void* stream) {
    if (!out) return fail(RIFT_ERR_ARG, "rift_closure_selftest: bad argument");
    rc::k_tc_selftest<<<1, 128, 0, (cudaStream_t)stream>>>(out);
    return launched("k_tc_selftest");
}

int rift_closure_check(void* stream) {
    cudaError_t e = cudaStreamSynchronize((cudaStream_t)stream);
    if (e != cudaSuccess) return fail(RIFT_ERR_CUDA, std::string("rift_closure_check: ") + cudaGetErrorString(e));
    int flag = 0;
    const int zero = 0;
    if (cudaMemcpyFromSymbol(&flag, rc::g_tc_error, sizeof(int)) != cudaSuccess ||
        cudaMemcpyToSymbol(rc::g_tc_error, &zero, sizeof(int)) != cudaSuccess)
        return fail(RIFT_ERR_CUDA, "rift_closure_check: status read failed");
    if (flag) return fail(RIFT_ERR_CUDA, "rift_closure_check: a tensor-core completion wait gave up");
    return RIFT_OK;
}

const char* rift_closure_last_error(void) { return g_err.c_str(); }

}  // extern "C"
