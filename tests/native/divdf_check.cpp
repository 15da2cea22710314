// divDF (rift_gb300/csrc/rift_divdf.h) against the FP64 division: random
// operands, exact quotients and their float neighbours (near ties), and the
// bench grids' cell sizes.  Prints the number of cases and mismatches.
#include <cmath>
#include <cstdio>
#include <random>

#include "../../rift_gb300/csrc/rift_divdf.h"

int main() {
    std::mt19937_64 rng(12345);
    std::uniform_real_distribution<double> U(0.0, 1.0);
    long n = 0, bad = 0;
    auto check = [&](double dx, float f) {
        uint64_t mx;
        int ex;
        rift::splitDouble(dx, &mx, &ex);
        double got;
        if (!rift::divDF(mx, ex, f, &got)) return;
        n++;
        if (got != dx / (double)f) {
            if (bad < 5) std::printf("mismatch dx=%.17g f=%.9g\n", dx, f);
            bad++;
        }
    };
    for (int i = 0; i < 3000000; i++) {
        check(std::ldexp(1.0 + U(rng), (int)(rng() % 16) - 4),
              (float)std::ldexp(1.0 + U(rng), (int)(rng() % 40) - 20));
        double dx = std::ldexp((double)(1 + rng() % 100000), -(int)(rng() % 10));
        float f = (float)(dx / (double)(1 + rng() % 1000));
        check(dx, f);
        check(dx, std::nextafter(f, 0.f));
        check(dx, std::nextafter(f, 1e30f));
        for (double cell : {2.0, 4.0, 5.0, 10.0}) check(cell, (float)std::ldexp(1.0 + U(rng), (int)(rng() % 12) - 6));
    }
    std::printf("%ld %ld\n", n, bad);
    return bad != 0;
}
