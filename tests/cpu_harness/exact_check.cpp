// Host-side check of the smoothing tap sums (nii2mesh_gb300/csrc/exact.cuh):
// whenever tap5_fast or tap5_split (with the window as its group) accepts a
// tap, its result must equal the reference's double sequence bit for bit.
// Usage: exact_check <samples> <seed>; prints
//   "<mismatches> <tap5_fast fraction on ordinary data> <tap5_split fraction on CT-like data>".
#include "../../nii2mesh_gb300/csrc/exact.cuh"
#include <cstdio>
#include <cstdlib>
#include <random>

int main(int argc, char **argv) {
    long n = argc > 1 ? atol(argv[1]) : 1000000;
    std::mt19937_64 rng(argc > 2 ? atol(argv[2]) : 1);
    std::normal_distribution<float> nd(0.f, 1.f);
    std::uniform_real_distribution<float> ud(0.f, 1.f);
    const int NF = 16;
    long bad = 0, fm[NF] = {0}, sm[NF] = {0}, nm[NF] = {0};
    for (long i = 0; i < n; i++) {
        float v[5];
        const int mode = (int)(i % NF);
        const float scale = ldexpf(1.f, (int)(ud(rng) * 200) - 100);   // one binade scale per sample
        for (int k = 0; k < 5; k++) {
            switch (mode) {
            case 0: v[k] = nd(rng) * 1000.f; break;                                   // mixed sign
            case 1: v[k] = (float)(int)(ud(rng) * 256.f); break;                       // u8 data
            case 2: v[k] = (float)(ud(rng) < 0.5f); break;                             // binary mask
            case 3: v[k] = -1000.f + nd(rng) * 20.f + (ud(rng) < 0.3f ? 1400.f : 0.f); break;  // CT-like
            case 4: v[k] = ldexpf(1.f + ud(rng), (int)(ud(rng) * 60) - 30); break;     // wide exponents
            case 5: v[k] = 100.f + nd(rng) * 1e-3f; break;                             // near-constant
            case 6: v[k] = (ud(rng) < 0.5f ? 1.f : -1.f) * ldexpf(1.f, (int)(ud(rng) * 8)); break;  // powers of 2
            case 7: v[k] = (ud(rng) < 0.02f) ? 0.f : nd(rng); break;
            case 8: { uint32_t b = (uint32_t)rng(); v[k] = u2f(b); if (!isfinite(v[k])) v[k] = 0.f; break; }   // any finite bits
            case 9: v[k] = (ud(rng) < 0.5f ? 0.f : -0.f) + ((ud(rng) < 0.2f) ? ldexpf(nd(rng), -140) : 0.f); break;  // zeros, subnormals
            case 10: v[k] = ldexpf(nd(rng), (int)(ud(rng) * 40) + 85); break;          // near the upper cut
            case 11: v[k] = -1000.f + nd(rng) * 20.f; break;                           // one binade: many exact midpoints
            case 12: v[k] = -1000.f + nd(rng) * 20.f + (ud(rng) < 0.05f ? 3000.f : 0.f); break;   // CT air + salt
            case 13: v[k] = (k < 3 ? -1.f : 1.f) * (300.f + nd(rng) * 200.f); break;  // cancellation
            case 14: v[k] = scale * (1.f + ud(rng) * 63.f) * (ud(rng) < 0.5f ? 1.f : -1.f); break;  // spread <= 6, any scale
            default: v[k] = ldexpf(1.f + ud(rng), (int)(ud(rng) * 7)) * (ud(rng) < 0.5f ? 1.f : -1.f); break;
            }
        }
        const float want = tap5_double(v[0], v[1], v[2], v[3], v[4]);
        float r;
        nm[mode]++;
        if (tap5_fast(v[0], v[1], v[2], v[3], v[4], &r)) {
            fm[mode]++;
            if (f2u(r) != f2u(want)) {
                if (bad < 10) printf("tap5_fast mismatch %a %a %a %a %a\n", v[0], v[1], v[2], v[3], v[4]);
                bad++;
            }
        }
        if (tap5_split_window(v[0], v[1], v[2], v[3], v[4], &r)) {
            sm[mode]++;
            if (f2u(r) != f2u(want)) {
                if (bad < 10) printf("tap5_split mismatch %a %a %a %a %a\n", v[0], v[1], v[2], v[3], v[4]);
                bad++;
            }
        }
    }
    if (getenv("EXACT_CHECK_MODES"))
        for (int k = 0; k < NF; k++)
            printf("family %d: fast %.5f split %.5f\n", k, nm[k] ? (double)fm[k] / nm[k] : 0.0,
                   nm[k] ? (double)sm[k] / nm[k] : 0.0);
    long fo = 0, no = 0, so = 0, nc = 0;   // ordinary data: every family but random bits, zeros/subnormals, huge values
    for (int k = 0; k < NF; k++)
        if (k < 8 || k == 11) { fo += fm[k]; no += nm[k]; }
    for (int k : {3, 11, 12}) { so += sm[k]; nc += nm[k]; }   // CT-like families
    printf("%ld %.6f %.6f\n", bad, no ? (double)fo / no : 0.0, nc ? (double)so / nc : 0.0);
    return bad != 0;
}
