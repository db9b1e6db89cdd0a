// Host-side check of the double-float smoothing tap (nii2mesh_gb300/csrc/exact.cuh):
// tap5_exact must equal the reference's double sequence bit-for-bit.
// Usage: exact_check <samples> <seed>; prints "<mismatches> <fast-path fraction>".
#include "../../nii2mesh_gb300/csrc/exact.cuh"
#include <cstdio>
#include <cstdlib>
#include <random>

int main(int argc, char **argv) {
    long n = argc > 1 ? atol(argv[1]) : 1000000;
    std::mt19937_64 rng(argc > 2 ? atol(argv[2]) : 1);
    std::normal_distribution<float> nd(0.f, 1.f);
    std::uniform_real_distribution<float> ud(0.f, 1.f);
    long bad = 0, fast = 0;
    for (long i = 0; i < n; i++) {
        float v[5];
        int mode = (int)(i % 8);
        for (int k = 0; k < 5; k++) {
            switch (mode) {
            case 0: v[k] = nd(rng) * 1000.f; break;                                   // mixed sign
            case 1: v[k] = (float)(int)(ud(rng) * 256.f); break;                       // u8 data
            case 2: v[k] = (float)(ud(rng) < 0.5f); break;                             // binary mask
            case 3: v[k] = -1000.f + nd(rng) * 20.f + (ud(rng) < 0.3f ? 1400.f : 0.f); break;  // CT-like
            case 4: v[k] = ldexpf(1.f + ud(rng), (int)(ud(rng) * 60) - 30); break;     // wide exponents
            case 5: v[k] = 100.f + nd(rng) * 1e-3f; break;                             // near-constant
            case 6: v[k] = (ud(rng) < 0.5f ? 1.f : -1.f) * ldexpf(1.f, (int)(ud(rng) * 8)); break;  // powers of 2
            default: v[k] = (ud(rng) < 0.02f) ? 0.f : nd(rng); break;
            }
        }
        float r;
        if (tap5_fast(v[0], v[1], v[2], v[3], v[4], &r)) {
            fast++;
            if (f2u(r) != f2u(tap5_double(v[0], v[1], v[2], v[3], v[4]))) {
                if (bad < 10) printf("mismatch %a %a %a %a %a\n", v[0], v[1], v[2], v[3], v[4]);
                bad++;
            }
        }
    }
    printf("%ld %.6f\n", bad, (double)fast / n);
    return bad != 0;
}
