// mc33.cuh — the Lewiner MC33 cube decisions (src/MarchingCubes.c:276-795)
// and lookup tables on the device, shared by the single-volume and the
// batched atlas marching-cubes kernels.
#pragma once
#include "mc_tables.h"
#include "n2m_internal.cuh"

namespace mc33 {
static __device__ const signed char d_lut[N2M_LUT_BLOB_SIZE] = N2M_LUT_BLOB_INIT;

#define L1(T, a) ((int)d_lut[N2M_##T##_OFF + (a)])
#define L2(T, a, b) ((int)d_lut[N2M_##T##_OFF + (a)*N2M_##T##_S0 + (b)])
#define L3(T, a, b, c) ((int)d_lut[N2M_##T##_OFF + (a)*N2M_##T##_S0 + (b)*N2M_##T##_S1 + (c)])
#define O2(T, a) (N2M_##T##_OFF + (a)*N2M_##T##_S0)
#define O3(T, a, b) (N2M_##T##_OFF + (a)*N2M_##T##_S0 + (b)*N2M_##T##_S1)

// ---- MC33 decisions (src/MarchingCubes.c:276-795) ---------------------------
__device__ __forceinline__ bool test_face(const float *c, int face) {
    float A = 0.f, B = 0.f, C = 0.f, D = 0.f;
    switch (face < 0 ? -face : face) {
    case 1: A = c[0]; B = c[4]; C = c[5]; D = c[1]; break;
    case 2: A = c[1]; B = c[5]; C = c[6]; D = c[2]; break;
    case 3: A = c[2]; B = c[6]; C = c[7]; D = c[3]; break;
    case 4: A = c[3]; B = c[7]; C = c[4]; D = c[0]; break;
    case 5: A = c[0]; B = c[3]; C = c[2]; D = c[1]; break;
    case 6: A = c[4]; B = c[7]; C = c[6]; D = c[5]; break;
    default: break;
    }
    const float det = __fsub_rn(__fmul_rn(A, C), __fmul_rn(B, D));
    if (fabsf(det) < N2M_FLT_EPS) return face >= 0;
    return __fmul_rn(__fmul_rn((float)face, A), det) >= 0.f;
}

__device__ __forceinline__ float lerp_t(const float *c, int a, int b, float t) {
    return __fadd_rn(c[a], __fmul_rn(__fsub_rn(c[b], c[a]), t));
}

// reference edge of the interior test: t = c[p]/(c[p]-c[q]); Bt, Ct, Dt
// interpolate three corner pairs (src/MarchingCubes.c:337-431)
static __constant__ signed char k_ie[12][8] = {
    {0, 1, 3, 2, 7, 6, 4, 5}, {1, 2, 0, 3, 4, 7, 5, 6}, {2, 3, 1, 0, 5, 4, 6, 7}, {3, 0, 2, 1, 6, 5, 7, 4},
    {4, 5, 7, 6, 3, 2, 0, 1}, {5, 6, 4, 7, 0, 3, 1, 2}, {6, 7, 5, 4, 1, 0, 2, 3}, {7, 4, 6, 5, 2, 1, 3, 0},
    {0, 4, 3, 7, 2, 6, 1, 5}, {1, 5, 0, 4, 3, 7, 2, 6}, {2, 6, 1, 5, 0, 4, 3, 7}, {3, 7, 2, 6, 1, 5, 0, 4}};

static __device__ bool test_interior(const float *c, int kase, int config, int subconfig, int s) {
    float At = 0.f, Bt = 0.f, Ct = 0.f, Dt = 0.f;
    if (kase == 4 || kase == 10) {
        const float d40 = __fsub_rn(c[4], c[0]), d62 = __fsub_rn(c[6], c[2]);
        const float d73 = __fsub_rn(c[7], c[3]), d51 = __fsub_rn(c[5], c[1]);
        const float a = __fsub_rn(__fmul_rn(d40, d62), __fmul_rn(d73, d51));
        const float b = __fsub_rn(__fsub_rn(__fadd_rn(__fmul_rn(c[2], d40), __fmul_rn(c[0], d62)), __fmul_rn(c[1], d73)),
                                  __fmul_rn(c[3], d51));
        const float t = __fdiv_rn(-b, __fmul_rn(2.f, a));
        if (t < 0.f || t > 1.f) return s > 0;
        At = __fadd_rn(c[0], __fmul_rn(d40, t));
        Bt = __fadd_rn(c[3], __fmul_rn(d73, t));
        Ct = __fadd_rn(c[2], __fmul_rn(d62, t));
        Dt = __fadd_rn(c[1], __fmul_rn(d51, t));
    } else {
        int edge = -1;
        switch (kase) {
        case 6: edge = L2(TEST6, config, 2); break;
        case 7: edge = L2(TEST7, config, 4); break;
        case 12: edge = L2(TEST12, config, 3); break;
        case 13: edge = L3(TILING13_5_1, config, subconfig, 0); break;
        default: break;
        }
        if (edge >= 0 && edge < 12) {
            const signed char *e = k_ie[edge];
            const float t = __fdiv_rn(c[e[0]], __fsub_rn(c[e[0]], c[e[1]]));
            Bt = lerp_t(c, e[2], e[3], t);
            Ct = lerp_t(c, e[4], e[5], t);
            Dt = lerp_t(c, e[6], e[7], t);
        }
    }
    const int test = (At >= 0.f) + 2 * (Bt >= 0.f) + 4 * (Ct >= 0.f) + 8 * (Dt >= 0.f);
    const float det = __fsub_rn(__fmul_rn(At, Ct), __fmul_rn(Bt, Dt));
    switch (test) {
    case 5: if (det < N2M_FLT_EPS) return s > 0; break;
    case 10: if (det >= N2M_FLT_EPS) return s > 0; break;
    case 7: case 11: case 13: case 14: case 15: return s < 0;
    default: return s > 0;
    }
    return s < 0;
}

struct Tiling {
    int off;    // blob offset of 3*n edge codes
    int n;      // triangles
    bool cv;    // needs the c-vertex (code 12)
};

// process_cube's decision tree (src/MarchingCubes.c:458-795)
static __device__ Tiling select_tiling(const float *c, int lut, bool classic) {
    Tiling T = {0, 0, false};
    if (classic) {
        T.off = O2(CASESCLASSIC, lut);
        int n = 0;
        while (n < 5 && d_lut[T.off + 3 * n] != -1) n++;
        T.n = n;
        return T;
    }
    const int kase = L2(CASES, lut, 0), cf = L2(CASES, lut, 1);
    int sub = 0;
    switch (kase) {
    case 1: T = {O2(TILING1, cf), 1, false}; break;
    case 2: T = {O2(TILING2, cf), 2, false}; break;
    case 3:
        T = test_face(c, L1(TEST3, cf)) ? Tiling{O2(TILING3_2, cf), 4, false} : Tiling{O2(TILING3_1, cf), 2, false};
        break;
    case 4:
        T = test_interior(c, 4, cf, 0, L1(TEST4, cf)) ? Tiling{O2(TILING4_1, cf), 2, false}
                                                       : Tiling{O2(TILING4_2, cf), 6, false};
        break;
    case 5: T = {O2(TILING5, cf), 3, false}; break;
    case 6:
        if (test_face(c, L2(TEST6, cf, 0))) T = {O2(TILING6_2, cf), 5, false};
        else if (test_interior(c, 6, cf, 0, L2(TEST6, cf, 1))) T = {O2(TILING6_1_1, cf), 3, false};
        else T = {O2(TILING6_1_2, cf), 9, true};
        break;
    case 7:
        if (test_face(c, L2(TEST7, cf, 0))) sub += 1;
        if (test_face(c, L2(TEST7, cf, 1))) sub += 2;
        if (test_face(c, L2(TEST7, cf, 2))) sub += 4;
        switch (sub) {
        case 0: T = {O2(TILING7_1, cf), 3, false}; break;
        case 1: T = {O3(TILING7_2, cf, 0), 5, false}; break;
        case 2: T = {O3(TILING7_2, cf, 1), 5, false}; break;
        case 3: T = {O3(TILING7_3, cf, 0), 9, true}; break;
        case 4: T = {O3(TILING7_2, cf, 2), 5, false}; break;
        case 5: T = {O3(TILING7_3, cf, 1), 9, true}; break;
        case 6: T = {O3(TILING7_3, cf, 2), 9, true}; break;
        default:
            T = test_interior(c, 7, cf, 0, L2(TEST7, cf, 3)) ? Tiling{O2(TILING7_4_2, cf), 9, false}
                                                              : Tiling{O2(TILING7_4_1, cf), 5, false};
        }
        break;
    case 8: T = {O2(TILING8, cf), 2, false}; break;
    case 9: T = {O2(TILING9, cf), 4, false}; break;
    case 10:
        if (test_face(c, L2(TEST10, cf, 0))) {
            T = test_face(c, L2(TEST10, cf, 1)) ? Tiling{O2(TILING10_1_1_B, cf), 4, false}
                                                : Tiling{O2(TILING10_2, cf), 8, true};
        } else if (test_face(c, L2(TEST10, cf, 1))) {
            T = {O2(TILING10_2_B, cf), 8, true};
        } else {
            T = test_interior(c, 10, cf, 0, L2(TEST10, cf, 2)) ? Tiling{O2(TILING10_1_1, cf), 4, false}
                                                               : Tiling{O2(TILING10_1_2, cf), 8, false};
        }
        break;
    case 11: T = {O2(TILING11, cf), 4, false}; break;
    case 12:
        if (test_face(c, L2(TEST12, cf, 0))) {
            T = test_face(c, L2(TEST12, cf, 1)) ? Tiling{O2(TILING12_1_1_B, cf), 4, false}
                                                : Tiling{O2(TILING12_2, cf), 8, true};
        } else if (test_face(c, L2(TEST12, cf, 1))) {
            T = {O2(TILING12_2_B, cf), 8, true};
        } else {
            T = test_interior(c, 12, cf, 0, L2(TEST12, cf, 2)) ? Tiling{O2(TILING12_1_1, cf), 4, false}
                                                               : Tiling{O2(TILING12_1_2, cf), 8, false};
        }
        break;
    case 13: {
        for (int f = 0; f < 6; f++)
            if (test_face(c, L2(TEST13, cf, f))) sub += 1 << f;
        const int sc = L1(SUBCONFIG13, sub);
        if (sc == 0) T = {O2(TILING13_1, cf), 4, false};
        else if (sc >= 1 && sc <= 6) T = {O3(TILING13_2, cf, sc - 1), 6, false};
        else if (sc >= 7 && sc <= 18) T = {O3(TILING13_3, cf, sc - 7), 10, true};
        else if (sc >= 19 && sc <= 22) T = {O3(TILING13_4, cf, sc - 19), 12, true};
        else if (sc >= 23 && sc <= 26)
            T = test_interior(c, 13, cf, sc - 23, L2(TEST13, cf, 6)) ? Tiling{O3(TILING13_5_1, cf, sc - 23), 6, false}
                                                                    : Tiling{O3(TILING13_5_2, cf, sc - 23), 10, false};
        else if (sc >= 27 && sc <= 38) T = {O3(TILING13_3_B, cf, sc - 27), 10, true};
        else if (sc >= 39 && sc <= 44) T = {O3(TILING13_2_B, cf, sc - 39), 6, false};
        else if (sc == 45) T = {O2(TILING13_1_B, cf), 4, false};
        break;
    }
    case 14: T = {O2(TILING14, cf), 4, false}; break;
    default: break;
    }
    return T;
}

// The tiling of configurations that need no face or interior test (every
// classic configuration; Lewiner cases 1, 2, 5, 8, 9, 11, 14), without the
// corner values.  Returns false for the ambiguous cases.
__device__ __forceinline__ bool quick_tiling(int lut, bool classic, Tiling &T) {
    if (classic) {
        T.off = O2(CASESCLASSIC, lut);
        int n = 0;
        while (n < 5 && d_lut[T.off + 3 * n] != -1) n++;
        T.n = n;
        T.cv = false;
        return true;
    }
    const int cf = L2(CASES, lut, 1);
    switch (L2(CASES, lut, 0)) {
    case 1: T = {O2(TILING1, cf), 1, false}; return true;
    case 2: T = {O2(TILING2, cf), 2, false}; return true;
    case 5: T = {O2(TILING5, cf), 3, false}; return true;
    case 8: T = {O2(TILING8, cf), 2, false}; return true;
    case 9: T = {O2(TILING9, cf), 4, false}; return true;
    case 11: T = {O2(TILING11, cf), 4, false}; return true;
    case 14: T = {O2(TILING14, cf), 4, false}; return true;
    default: return false;
    }
}

__device__ __forceinline__ int cube_lut(const float *c) {
    int lut = 0;
    for (int p = 0; p < 8; p++) lut |= (c[p] > 0.f) << p;
    return lut;
}

// distance of a grid coordinate 0 <= f < 2^22 to the nearest integer; adding
// 1.5 * 2^23 rounds to an integer in the FP32 adder (rintf would issue on
// the conversion pipe, which this part shares with FP64)
__device__ __forceinline__ float frac_dist(float f) {
    const float r = __fsub_rn(__fadd_rn(f, 12582912.f), 12582912.f);
    return fabsf(__fsub_rn(f, r));
}

// cube edge e of the tiling tables: owner corner, axis, the two corners it
// interpolates (owner first)
static __constant__ signed char k_edge[12][4] = {{0, 0, 0, 1}, {1, 1, 1, 2}, {3, 0, 3, 2}, {0, 1, 0, 3},
                                         {4, 0, 4, 5}, {5, 1, 5, 6}, {7, 0, 7, 6}, {4, 1, 4, 7},
                                         {0, 2, 0, 4}, {1, 2, 1, 5}, {2, 2, 2, 6}, {3, 2, 3, 7}};

__device__ __forceinline__ float edge_u(float c0, float c1) {
    const float den = __fsub_rn(c0, c1);
    return den != 0.f ? __fdiv_rn(c0, den) : 0.5f;
}

}  // namespace mc33
