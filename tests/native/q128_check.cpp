// Host check of the software binary128 (q128.cuh) against GCC f128:
// random add/sub/mul/div/floor results must match bit for bit, and the
// resampling recurrence built from them must match the f128 one.
#if defined(__aarch64__)
typedef long double f128;
#define floorq floorl
#else
#include <quadmath.h>
typedef __float128 f128;
#endif
#include <cstdio>
#include <cstring>
#include <cstdint>
#include <random>
#include "../../smc_inversion_fort_gb300/csrc/q128.cuh"
using namespace smc;
static void bits_of(f128 x, uint64_t &hi, uint64_t &lo) {
    unsigned char b[16]; memcpy(b, &x, 16); memcpy(&lo, b, 8); memcpy(&hi, b + 8, 8);
}
static f128 to_f(q128 a) {
    uint64_t hi, lo; q128_bits(a, hi, lo); unsigned char b[16];
    memcpy(b, &lo, 8); memcpy(b + 8, &hi, 8); f128 x; memcpy(&x, b, 16); return x;
}
int main(int argc, char **argv) {
    long n = argc > 1 ? atol(argv[1]) : 200000;
    std::mt19937_64 rng(12345);
    std::uniform_real_distribution<double> U(-1.0, 1.0);
    long bad = 0;
    for (long t = 0; t < n; ++t) {
        double x = U(rng) * std::ldexp(1.0, (int)(rng() % 40) - 20);
        double y = U(rng) * std::ldexp(1.0, (int)(rng() % 40) - 20);
        double z = U(rng);
        q128 a = q128_add(q128_from_double(x), q128_from_double(z * 1e-17));
        q128 b = q128_from_double(y);
        f128 fa = (f128)x + (f128)(z * 1e-17), fb = y;
        f128 ref[4] = {fa + fb, fa - fb, fa * fb, fa / fb};
        q128 got[4] = {q128_add(a, b), q128_sub(a, b), q128_mul(a, b), q128_div(a, b)};
        for (int k = 0; k < 4; ++k) {
            uint64_t h1, l1, h2, l2; bits_of(ref[k], h1, l1); q128_bits(got[k], h2, l2);
            if (ref[k] == 0) { h1 &= ~(1ull << 63); h2 &= ~(1ull << 63); }
            if (h1 != h2 || l1 != l2) { if (bad < 10) printf("op %d mismatch x=%a y=%a\n", k, x, y); ++bad; }
        }
        f128 fl = floorq(ref[2] * 1000);
        if ((long long)fl != q128_floor(q128_mul(got[2], q128_from_int(1000)))) { if (bad < 10) printf("floor mismatch\n"); ++bad; }
    }
    // resampling recurrence
    for (int rep = 0; rep < 200; ++rep) {
        int N = 1 + rng() % 700;
        std::vector<double> w(N); double s = 0;
        for (auto &v : w) { v = std::exp(8 * U(rng)); s += v; }
        for (auto &v : w) v /= s;
        double uh = (double)(rng() >> 11) * 0x1.0p-53, ul = (double)(rng() >> 11) * 0x1.0p-106;
        f128 u = ((f128)uh + ul) / N; q128 qu = q128_div(q128_add(q128_from_double(uh), q128_from_double(ul)), q128_from_int(N));
        for (int i = 0; i < N; ++i) {
            int a1 = (int)floorq(((f128)w[i] - u) * N) + 1;
            u = u + (f128)a1 / N - w[i];
            q128 wi = q128_from_double(w[i]);
            long long a2 = q128_floor(q128_mul(q128_sub(wi, qu), q128_from_int(N))) + 1;
            qu = q128_sub(q128_add(qu, q128_div(q128_from_int(a2), q128_from_int(N))), wi);
            if (a1 != a2 || to_f(qu) != u) { if (bad < 10) printf("recurrence mismatch rep %d i %d\n", rep, i); ++bad; break; }
        }
    }
    printf("mismatches %ld\n", bad);
    return bad != 0;
}
