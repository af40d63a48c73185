// Compares df_exp of hmec_dfexp.cuh with the long-double exp over the range
// the marker kernel uses (-alpha * porosity) and beyond; prints the largest
// relative error and exits non-zero above 2e-14 (the pairs carry ~48 bits).
#include <cmath>
#include <cstdio>
#include <random>

#include "hmec_dfexp.cuh"

int main() {
    std::mt19937_64 rng(99);
    std::uniform_real_distribution<double> U(-60.0, 60.0), S(-30.0, 0.0);
    double worst = 0, wx = 0;
    long n = 0, fallback = 0;
    auto check = [&](double x) {
        float h, l;
        n++;
        if (!df_exp(x, h, l)) {
            fallback++;
            return;
        }
        const long double ref = expl((long double)x);
        const long double got = (long double)h + (long double)l;
        const double rel = (double)fabsl((got - ref) / ref);
        if (rel > worst) {
            worst = rel;
            wx = x;
        }
    };
    for (int k = 0; k < 2000000; k++) {
        check(U(rng));
        check(S(rng));
    }
    for (double x : {0.0, -0.0, 1e-300, -1e-300, 0.34657359, -0.34657359, 0.3465736, -0.3465736, -28.0, -60.0, 60.0})
        check(x);
    printf("df_exp: %ld values, worst relative error %.3g at x = %.17g, %ld outside the range\n", n, worst, wx, fallback);
    return worst <= 2e-14 ? 0 : 1;
}
