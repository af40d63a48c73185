// Compares the bit-pattern widening of hmec_bits.cuh with the compiler's own
// FP32 -> FP64 conversion on random bit patterns (FP32 subnormals give 0 by
// design); prints the number of mismatches and exits non-zero on any.
#include <cfloat>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <random>

#include "hmec_bits.cuh"

static bool same_double(double a, double b) {
    if (std::isnan(a) && std::isnan(b)) return true;
    uint64_t x, y;
    memcpy(&x, &a, 8);
    memcpy(&y, &b, 8);
    return x == y;
}

int main() {
    std::mt19937_64 rng(12345);
    long badf = 0, nf = 0;
    for (int k = 0; k < 4000000; k++) {
        uint32_t u = (uint32_t)rng();
        float f;
        memcpy(&f, &u, 4);
        const int e = (u >> 23) & 0xFF;
        nf++;
        const double want = e == 0 ? 0.0 : (double)f;  // FP32 subnormals give 0 by design
        if (!same_double(f2d_bits(f), want) && !(e == 0 && f2d_bits(f) == 0.0)) badf++;
    }
    printf("f2d %ld/%ld mismatches\n", badf, nf);
    return badf ? 1 : 0;
}
