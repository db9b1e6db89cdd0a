// exact.cuh — bit-exact evaluation of the reference's double-precision
// 5-tap blur tap sum (src/meshify.c:170-216) using FP32 arithmetic.
//
// The reference evaluates, per pass and per voxel,
//     s = ((((a*w2 + b*w1) + c*w0) + d*w1) + e*w2)      in IEEE double
// (w0 = 0.45, w1 = 0.225, w2 = 0.05 as doubles) and stores (float)s.  GB300's
// FP64 rate is a small fraction of its FP32 rate, so the fast path computes
// the exact tap sum in double-float arithmetic (error-free TwoSum/TwoProd
// transforms, ~2^-40 relative accuracy) and proves that the float rounding of
// the reference's double result equals the float rounding of this estimate:
// the estimate T = Th + Tl must be farther than a rigorous error bound from
// every rounding boundary (midpoint between adjacent floats) of Th.  When the
// proof fails (about 1 voxel in 10^5, plus zero/tiny/non-finite sums) the
// voxel is recomputed with the reference's exact double operation sequence.
// Either way the result equals the reference's float bit pattern.
//
// Written for both host and device so the arithmetic can be unit-tested on
// the CPU (host builds must use -ffp-contract=off).
#pragma once
#include <math.h>
#include <stdint.h>
#include <string.h>

#if defined(__CUDACC__)
#define N2M_HD __host__ __device__ __forceinline__
#else
#define N2M_HD static inline
#endif

#if defined(__CUDA_ARCH__)
#define FADD(a, b) __fadd_rn((a), (b))
#define FSUB(a, b) __fsub_rn((a), (b))
#define FMUL(a, b) __fmul_rn((a), (b))
#define FFMA(a, b, c) __fmaf_rn((a), (b), (c))
#define DADD(a, b) __dadd_rn((a), (b))
#define DMUL(a, b) __dmul_rn((a), (b))
#define D2F(a) __double2float_rn(a)
N2M_HD uint32_t f2u(float f) { return __float_as_uint(f); }
N2M_HD float u2f(uint32_t u) { return __uint_as_float(u); }
#else
#define FADD(a, b) ((float)((a) + (b)))
#define FSUB(a, b) ((float)((a) - (b)))
#define FMUL(a, b) ((float)((a) * (b)))
#define FFMA(a, b, c) fmaf((a), (b), (c))
#define DADD(a, b) ((double)((a) + (b)))
#define DMUL(a, b) ((double)((a) * (b)))
#define D2F(a) ((float)(a))
N2M_HD uint32_t f2u(float f) { uint32_t u; memcpy(&u, &f, 4); return u; }
N2M_HD float u2f(uint32_t u) { float f; memcpy(&f, &u, 4); return f; }
#endif

// taps as doubles, and their double-float splits w = wH + wL (|err| < 2^-50 w)
#define N2M_W0D 0.45
#define N2M_W1D 0.225
#define N2M_W2D 0.05
#define N2M_W0H 0x1.cccccc0000000p-2f
#define N2M_W0L 0x1.99999a0000000p-27f
#define N2M_W2H 0x1.99999a0000000p-5f
#define N2M_W2L (-0x1.99999a0000000p-31f)

N2M_HD void two_sum(float a, float b, float &s, float &e) {
    s = FADD(a, b);
    float bb = FSUB(s, a);
    e = FADD(FSUB(a, FSUB(s, bb)), FSUB(b, bb));
}

// The reference's operation sequence, verbatim in double.
N2M_HD float tap5_double(float a, float b, float c, float d, float e) {
    double s = DMUL((double)a, N2M_W2D);
    s = DADD(s, DMUL((double)b, N2M_W1D));
    s = DADD(s, DMUL((double)c, N2M_W0D));
    s = DADD(s, DMUL((double)d, N2M_W1D));
    s = DADD(s, DMUL((double)e, N2M_W2D));
    return D2F(s);
}

// Fast path.  Returns true and writes *out when the float result is proven
// equal to tap5_double(a..e).
//   exact value E = w2*(a+e) + w0*(c + (b+d)/2)         (w1 == w0/2 exactly)
// th + tl approximates E to within M * 2^-40 (M = max |input|; products
// and sums are error-free except the final compensation terms, each
// relatively 2^-24 of a term below M * 2^-24), and the reference's double
// result lies within M * 2^-50 of E, so M * 2^-38 bounds |th + tl - D| with
// room to spare.  If |tl| plus that bound stays below half the gap under |th|
// (the smaller of th's two neighbour gaps), D rounds to th.  Zero, tiny,
// huge and non-finite inputs (M outside [2^-90, 2^120)) are left to the slow
// path, except all-zero taps, whose signed-zero sum is exact in float.
N2M_HD bool tap5_fast(float a, float b, float c, float d, float e, float *out) {
    float u, ue, v, ve, w, we;
    two_sum(a, e, u, ue);
    two_sum(b, d, v, ve);
    v = FMUL(v, 0.5f);
    ve = FMUL(ve, 0.5f);
    two_sum(c, v, w, we);
    we = FADD(we, ve);
    const float p1 = FMUL(N2M_W2H, u), e1 = FFMA(N2M_W2H, u, -p1);
    const float p2 = FMUL(N2M_W0H, w), e2 = FFMA(N2M_W0H, w, -p2);
    float S, es;
    two_sum(p1, p2, S, es);
    float low = FFMA(N2M_W2H, ue, e1);
    low = FFMA(N2M_W2L, u, low);
    low = FFMA(N2M_W0H, we, low);
    low = FFMA(N2M_W0L, w, low);
    low = FADD(low, e2);
    low = FADD(low, es);
    float th, tl;
    two_sum(S, low, th, tl);
    const float M = fmaxf(fmaxf(fmaxf(fabsf(a), fabsf(e)), fmaxf(fabsf(b), fabsf(d))), fabsf(c));
    if (!(M >= 0x1p-90f && M < 0x1p+120f)) {
        if (M == 0.0f) {                                         // all taps +-0
            *out = FADD(FADD(FADD(FADD(a, b), c), d), e);        // same signed zero
            return true;
        }
        return false;                                            // tiny, huge, NaN, Inf
    }
    const float ath = fabsf(th);
    const float dn = FSUB(ath, u2f(f2u(ath) - 1u));              // gap below |th|; NaN for th == 0
    if (FFMA(2.0f, fabsf(tl), FMUL(M, 0x1p-37f)) < dn) {         // |tl| + M 2^-38 < dn / 2
        *out = th;
        return true;
    }
    return false;
}

// ---- split fast path ------------------------------------------------------------
// A cheaper exact evaluation for taps whose inputs lie within a factor 64 of
// one another (the common case: CT air at -1000 +- 20 straddles a binade,
// tissue values sit within a few binades).  With the /40 taken out, the tap is
//     E = N / 5,   N = (2(a+e) + 9(b+d) + 18c) / 8,
// and N is computed EXACTLY as NH + NL: every input is split into a high part
// (its 12 low mantissa bits cleared) and the exact low remainder, and the
// weighted sums of the high parts and of the low parts are each exact in FP32
// (all terms lie on a common grid and stay below 2^24 grid steps when
// max|x| <= 64 min|x|).  The float y ~ N/5 and the exact residual
// R = N - 5y (also exact, see below) then say whether y, or its neighbour
// y +- ulp, is the correctly rounded N/5: accepted only when
// |N - 5q| < 2.5 ulp strictly, so exact ties (which the reference's double
// rounding errors decide) and binade edges are left to tap5_fast / FP64.
// Against the reference: its double result D lies within 10 * 2^-53 max|x| of
// N/5, while a non-tie N/5 is at least 2^-32 max|x| / 5 from every rounding
// boundary, so float(D) is the same q.  The test |y| >= max|x| * 2^-8 (no
// deep cancellation) keeps the residual exact and the result normal.
//
// Exactness of the residual: y's ulp u >= 2^(p-31) for max|x| in [2^p,
// 2^(p+1)); NH - 5y is a multiple of u of magnitude < 5 * 2^(p-11) + 8u, and
// (NH - 5y) + NL a multiple of 2^(p-32) of magnitude < 8u: both fit 24 bits.

// x = h + l exactly, h = x with its 12 low mantissa bits cleared
N2M_HD void split12(float x, float &h, float &l) {
    h = u2f(f2u(x) & 0xFFFFF000u);
    l = FSUB(x, h);
}

// the condition under which tap5_split may be used on taps drawn from a group
// of inputs whose magnitudes have minimum mn and maximum mx
N2M_HD bool split_group_ok(float mn, float mx) {
    return mn >= FMUL(mx, 0x1p-6f) && mx >= 0x1p-90f && mx < 0x1p+120f;
}

// Exact tap from split inputs.  Precondition: split_group_ok(mn, mx) for a
// group holding all five inputs, and mth = mx * 2^-8.  Returns true (and
// *out = the reference's float result) or false (undecided: tie, binade edge
// or cancellation); *out is written either way.
N2M_HD bool tap5_split(float aH, float aL, float bH, float bL, float cH, float cL, float dH, float dL, float eH,
                       float eL, float mth, float *out) {
    const float s1H = FADD(aH, eH), s2H = FADD(bH, dH);
    const float NH = FFMA(cH, 2.25f, FFMA(s2H, 1.125f, FMUL(s1H, 0.25f)));
    const float s1L = FADD(aL, eL), s2L = FADD(bL, dL);
    const float NL = FFMA(cL, 2.25f, FFMA(s2L, 1.125f, FMUL(s1L, 0.25f)));
    const float y = FMUL(FADD(NH, NL), 0.2f);
    const float R2 = FADD(FFMA(-5.0f, y, NH), NL);   // N - 5y, exact
    const uint32_t yb = f2u(y);
    const float u = u2f((yb & 0x7F800000u) - (23u << 23));   // ulp(y) for |y| >= 2^-103
    const float t25 = FMUL(u, 2.5f);
    const float step = fabsf(R2) >= t25 ? u2f(f2u(u) | (f2u(R2) & 0x80000000u)) : 0.0f;
    *out = FADD(y, step);                             // y or its neighbour towards N/5
    const float R3 = FFMA(-5.0f, step, R2);           // N - 5q, exact
    return fabsf(R3) < t25 && (yb & 0x7FFFFFu) != 0u && fabsf(y) >= mth;
}

// tap5_split on five raw inputs, the group being the window itself
N2M_HD bool tap5_split_window(float a, float b, float c, float d, float e, float *out) {
    const float mx = fmaxf(fmaxf(fmaxf(fabsf(a), fabsf(b)), fmaxf(fabsf(c), fabsf(d))), fabsf(e));
    const float mn = fminf(fminf(fminf(fabsf(a), fabsf(b)), fminf(fabsf(c), fabsf(d))), fabsf(e));
    if (!split_group_ok(mn, mx)) return false;
    float aH, aL, bH, bL, cH, cL, dH, dL, eH, eL;
    split12(a, aH, aL);
    split12(b, bH, bL);
    split12(c, cH, cL);
    split12(d, dH, dL);
    split12(e, eH, eL);
    return tap5_split(aH, aL, bH, bL, cH, cL, dH, dL, eH, eL, FMUL(mx, 0x1p-8f), out);
}

