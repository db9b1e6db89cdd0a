// fmt_check.cpp — checks the device text formatter (nii2mesh_gb300/csrc/fmt.cuh,
// compiled here for the host) against the C library's printf("%g") and
// printf("%d"), which the reference's text writers call (src/meshify.c:683-723).
//
// usage: fmt_check N SEED  -> prints "<cases> <mismatches>", exit 1 on a mismatch
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <random>

#include "../../nii2mesh_gb300/csrc/fmt.cuh"

static long long g_cases = 0, g_bad = 0;

static void check_g(double v) {
    char want[64], got[64];
    snprintf(want, sizeof want, "%g", v);
    const int n = n2mfmt::fmt_g6(v, got);
    got[n] = 0;
    g_cases++;
    if (strcmp(want, got)) {
        if (g_bad < 20) printf("%%g mismatch %.17g: want '%s' got '%s'\n", v, want, got);
        g_bad++;
    }
    if (!isfinite(v) || v == 0) return;
    // the wide path on the same value
    uint64_t bits;
    memcpy(&bits, &v, 8);
    const int ex = (int)((bits >> 52) & 0x7FF);
    const uint64_t fr = bits & ((1ull << 52) - 1);
    const int m2 = n2mfmt::fmt_g6_wide(ex ? (fr | (1ull << 52)) : fr, (ex ? ex : 1) - 1075, bits >> 63, got);
    got[m2] = 0;
    g_cases++;
    if (strcmp(want, got)) {
        if (g_bad < 20) printf("%%g (wide) mismatch %.17g: want '%s' got '%s'\n", v, want, got);
        g_bad++;
    }
}

static void check_d(int v) {
    char want[32], got[32];
    snprintf(want, sizeof want, "%d", v);
    const int n = n2mfmt::fmt_d(v, got);
    got[n] = 0;
    g_cases++;
    if (strcmp(want, got)) {
        if (g_bad < 20) printf("%%d mismatch %d: want '%s' got '%s'\n", v, want, got);
        g_bad++;
    }
}

int main(int argc, char **argv) {
    const long long N = argc > 1 ? atoll(argv[1]) : 1000000;
    std::mt19937_64 rng(argc > 2 ? strtoull(argv[2], nullptr, 10) : 1);
    std::uniform_real_distribution<double> uni(-1000.0, 1000.0);
    // special values, powers of ten and their neighbours, rounding ties
    const double specials[] = {0.0, -0.0, INFINITY, -INFINITY, NAN, -NAN, 1.0, -1.0, 0.5, 1e-4, 1e-5, 9.99995e-5,
                               9.999949e-5, 99999.95, 999999.5, 999999.4999, 999999.5000001, 100000.0, 1e6, 1e15, 1e16,
                               1e17, 1e22, 1e23, 1e37, 1e38, 1e-17, 1e-18, 1e-300, 5e-324, 2.2250738585072014e-308,
                               1.7976931348623157e308, 123456.5, 123457.5, 1234565.0, 1234575.0, 0.1, 0.2, 0.3, 12.5,
                               2.5e-5, 0.0001234565, 1.5, 2.5, 3.5};
    for (double v : specials) {
        check_g(v);
        check_g(nextafter(v, INFINITY));
        check_g(nextafter(v, -INFINITY));
    }
    for (int e = -330; e <= 310; e++) {
        const double p = pow(10.0, e);
        check_g(p);
        check_g(nextafter(p, 0.0));
        check_g(nextafter(p, INFINITY));
        check_g(-p * 9.999995);
    }
    for (long long k = 100000; k < 1000000; k += 997) {   // exact ties at the seventh digit
        check_g((double)k + 0.5);
        check_g((double)(10 * k + 5));
        check_g(((double)k + 0.5) / 1024.0);
    }
    const int ints[] = {0, 1, -1, 9, 10, 99, 100, 2147483647, -2147483647 - 1, 123456789, -42};
    for (int v : ints) check_d(v);
    for (long long i = 0; i < N; i++) {
        uint64_t r = rng();
        double v;
        switch (i % 6) {
        case 0:   // any bit pattern
            memcpy(&v, &r, 8);
            break;
        case 1:   // mesh coordinates
            v = uni(rng);
            break;
        case 2: {   // float coordinates widened to double (vertices of a float grid)
            const float f = (float)uni(rng);
            v = f;
            break;
        }
        case 3:   // grid positions with small fractions
            v = (double)(int)(r % 2048) - 1024 + (double)((r >> 20) % 4096) / 4096.0;
            break;
        case 4:   // wide magnitude range
            v = ldexp((double)(r >> 11) / 9007199254740992.0 + 0.5, (int)((r >> 3) % 400) - 200);
            break;
        default:   // six-digit decimals (shortest representation near ties)
            v = (double)(int64_t)(r % 2000000000ull - 1000000000ull) / 1000.0;
            break;
        }
        check_g(v);
        check_d((int)(uint32_t)(r >> 17));
    }
    printf("%lld %lld\n", g_cases, g_bad);
    return g_bad ? 1 : 0;
}
