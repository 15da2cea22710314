// rift_divdf.h -- dx / f correctly rounded in FP64 from integer arithmetic.
//
// On GB300 a dependent FP64 division takes about 640 cycles of latency; the
// step's dt (a double divided by a float) sits on the critical path of every
// step.  divDF computes the same correctly rounded quotient (round to
// nearest even) with two 64-bit integer divisions: long division of the
// mantissas, Q = floor(mx * 2^26 / mf), which has 55 or 56 bits; its top 53
// bits are the quotient's mantissa, rounded with the bits below them and the
// remainder as the sticky bit.  Host and device share this code, so the
// tests check it against the FP64 division on the CPU.
#pragma once
#include <cstdint>
#include <cstring>

#ifdef __CUDACC__
#define RIFT_HD __host__ __device__ __forceinline__
#else
#define RIFT_HD inline
#endif

namespace rift {

// dx = mx * 2^ex with mx a 53-bit integer (top bit 52): a normal double.
RIFT_HD void splitDouble(double dx, uint64_t* mx, int* ex) {
    uint64_t b;
    memcpy(&b, &dx, 8);
    *mx = (b & ((1ull << 52) - 1)) | (1ull << 52);
    *ex = (int)((b >> 52) & 0x7ff) - 1023 - 52;
}

// RN(dx / f) for a positive normal double dx = mx * 2^ex and a positive
// normal float f.  Returns false (leaving *out) when f is not a positive
// normal float or the quotient leaves the normal range.
RIFT_HD bool divDF(uint64_t mx, int ex, float f, double* out) {
    uint32_t fb;
    memcpy(&fb, &f, 4);
    const int ef = (int)((fb >> 23) & 0xffu);
    if (ef == 0 || ef == 0xff || (fb >> 31)) return false;
    const uint64_t mf = (uint64_t)((fb & 0x7fffffu) | 0x800000u);  // f = mf * 2^(ef-150)
    const uint64_t n1 = mx >> 6, n0 = (mx & 63u) << 26;
    const uint64_t q1 = n1 / mf, r1 = n1 - q1 * mf;
    const uint64_t m = (r1 << 32) | n0;
    const uint64_t q0 = m / mf, r0 = m - q0 * mf;
    const uint64_t Q = (q1 << 32) + q0;  // 2^54 < Q < 2^56
    const int nb = (Q >> 55) ? 3 : 2;
    uint64_t mant = Q >> nb;
    const uint64_t rem = Q & ((1ull << nb) - 1), half = 1ull << (nb - 1);
    if (rem > half || (rem == half && (r0 != 0 || (mant & 1)))) mant++;
    int E = nb + ex - ef + 124;  // quotient = mant * 2^E
    if (mant >> 53) {
        mant >>= 1;
        E++;
    }
    const int be = E + 52 + 1023;
    if (be <= 0 || be >= 0x7ff) return false;
    const uint64_t bits = ((uint64_t)be << 52) | (mant & ((1ull << 52) - 1));
    memcpy(out, &bits, 8);
    return true;
}

}  // namespace rift
