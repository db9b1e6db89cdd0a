// fmt.cuh — printf("%g") and printf("%d") of the reference's text writers
// (save_obj, save_off, save_json: src/meshify.c:683-723) on the device.
//
// %g (precision 6, C99 7.19.6.1): the value rounded to 6 significant digits
// (round half to even on exact ties, as glibc's exact conversion does); X =
// the decimal exponent of that rounded value; style f with 5 - X decimals when
// -4 <= X < 6, else style e with 5 decimals and an exponent of at least two
// digits; trailing zeros and a trailing point removed.
//
// The digits are exact.  fmt_g6 scales |v| = m * 2^e by 10^(5-X) in 128-bit
// integers when that fits (about 1e-17 <= |v| < 2^120, every coordinate of a
// mesh in practice) and otherwise expands m * 2^e exactly in base 10^9 limbs
// (fmt_g6_wide).  tests/cpu_harness/fmt_check.cpp compares both with the C
// library's snprintf.
#pragma once
#include <stdint.h>

#ifdef __CUDACC__
#define N2M_HD __host__ __device__
#define N2M_NOINLINE __noinline__
#else
#define N2M_HD
#define N2M_NOINLINE __attribute__((noinline))
#endif

namespace n2mfmt {

typedef unsigned __int128 u128;

N2M_HD inline int clz64(unsigned long long x) {
#ifdef __CUDA_ARCH__
    return __clzll((long long)x);
#else
    return __builtin_clzll(x);
#endif
}

N2M_HD inline u128 pow10_128(int k) {   // 0 <= k <= 38
    u128 r = 1;
    for (int i = 0; i < k; i++) r *= 10u;
    return r;
}

N2M_HD inline int bitlen128(u128 x) {
    const unsigned long long hi = (unsigned long long)(x >> 64), lo = (unsigned long long)x;
    if (hi) return 128 - clz64(hi);
    return lo ? 64 - clz64(lo) : 0;
}

// character sinks: a char buffer, or 32-bit words of a 4-byte-aligned buffer
// (no per-thread array, so the device formatter stays in registers)
struct CharSink {
    char *p;
    int n = 0;
    N2M_HD void put(char c) { p[n++] = c; }
};
struct WordSink {
    unsigned *dst;
    unsigned cur = 0;
    int n = 0;
    N2M_HD void put(char c) {
        cur |= (unsigned)(unsigned char)c << (8 * (n & 3));
        if ((n & 3) == 3) {
            dst[n >> 2] = cur;
            cur = 0;
        }
        ++n;
    }
    N2M_HD void done() {
        if (n & 3) dst[n >> 2] = cur;
    }
};

// the 6 significant digits D (10^5 <= D < 10^6) with decimal exponent X in %g style
template <class S>
N2M_HD inline void emit_g6(unsigned D, int X, bool neg, S &out) {
    unsigned dg = 0;   // digit i (0 = most significant) in bits 4(5-i)..
    for (int i = 0; i < 6; i++) {
        dg |= (D % 10u) << (4 * i);
        D /= 10u;
    }
    auto digit = [&](int i) { return (char)('0' + ((dg >> (4 * (5 - i))) & 15u)); };
    int nd = 6;   // significant digits after removing trailing zeros
    while (nd > 1 && ((dg >> (4 * (6 - nd))) & 15u) == 0) nd--;
    if (neg) out.put('-');
    if (X >= -4 && X < 6) {
        if (X >= 0) {
            for (int i = 0; i <= X; i++) out.put(digit(i));
            if (nd > X + 1) {
                out.put('.');
                for (int i = X + 1; i < nd; i++) out.put(digit(i));
            }
        } else {
            out.put('0');
            out.put('.');
            for (int i = 0; i < -X - 1; i++) out.put('0');
            for (int i = 0; i < nd; i++) out.put(digit(i));
        }
    } else {
        out.put(digit(0));
        if (nd > 1) {
            out.put('.');
            for (int i = 1; i < nd; i++) out.put(digit(i));
        }
        out.put('e');
        int ax = X;
        if (ax < 0) {
            out.put('-');
            ax = -ax;
        } else {
            out.put('+');
        }
        if (ax >= 100) {
            out.put((char)('0' + ax / 100));
            ax %= 100;
        }
        out.put((char)('0' + ax / 10));
        out.put((char)('0' + ax % 10));
    }
}

// 6 significant digits of m * 2^e (m > 0) by exact expansion in base 10^9 (any double)
N2M_HD N2M_NOINLINE inline int fmt_g6_wide(unsigned long long m, int e, bool neg, char *out) {
    // value = big * 10^-dexp, big in base 1e9 limbs (least significant first)
    unsigned limb[96];
    int nl = 0, dexp = 0;
    while (m) {
        limb[nl++] = (unsigned)(m % 1000000000ull);
        m /= 1000000000ull;
    }
    // e >= 0: multiply by 2^e (by 2^28 at a time); e < 0: m / 2^s = m * 5^s / 10^s
    int rem = e >= 0 ? e : -e;
    const unsigned step_mul = e >= 0 ? (1u << 28) : 244140625u;   // 2^28 or 5^12
    const int step = e >= 0 ? 28 : 12;
    while (rem > 0) {
        unsigned mul;
        if (rem >= step) {
            mul = step_mul;
            rem -= step;
        } else {
            mul = 1;
            for (int i = 0; i < rem; i++) mul *= e >= 0 ? 2u : 5u;
            rem = 0;
        }
        unsigned long long carry = 0;
        for (int i = 0; i < nl; i++) {
            const unsigned long long t = (unsigned long long)limb[i] * mul + carry;
            limb[i] = (unsigned)(t % 1000000000ull);
            carry = t / 1000000000ull;
        }
        while (carry) {
            limb[nl++] = (unsigned)(carry % 1000000000ull);
            carry /= 1000000000ull;
        }
    }
    if (e < 0) dexp = -e;
    // digits of the top limbs: number of decimal digits of the big integer
    unsigned top = limb[nl - 1];
    int topd = 1;
    for (unsigned t = top; t >= 10u; t /= 10u) topd++;
    const int ndig = topd + 9 * (nl - 1);
    // digit k (0 = most significant)
    auto digit = [&](int k) -> unsigned {
        const int pos = ndig - 1 - k;   // position from the least significant digit
        unsigned v = limb[pos / 9];
        for (int i = 0; i < pos % 9; i++) v /= 10u;
        return v % 10u;
    };
    unsigned D = 0;
    for (int k = 0; k < 6; k++) D = D * 10u + (k < ndig ? digit(k) : 0u);
    int X = ndig - 1 - dexp;
    if (ndig > 6) {
        const unsigned r = digit(6);
        bool sticky = false;
        for (int k = 7; k < ndig && !sticky; k++) sticky = digit(k) != 0;
        if (r > 5 || (r == 5 && (sticky || (D & 1u)))) D++;
        if (D == 1000000u) {
            D = 100000u;
            X++;
        }
    }
    CharSink cs{out};
    emit_g6(D, X, neg, cs);
    return cs.n;
}

// the wide path through a sink (kept out of line: its limb array is only touched for rare values)
template <class S>
N2M_HD N2M_NOINLINE void fmt_g6_wide_to(unsigned long long m, int e, bool neg, S &out) {
    char b[16];
    const int n = fmt_g6_wide(m, e, neg, b);
    for (int i = 0; i < n; i++) out.put(b[i]);
}

// printf("%g", v) into a sink (at most 13 characters)
template <class S>
N2M_HD inline void fmt_g6(double v, S &out) {
    unsigned long long bits;
#ifdef __CUDA_ARCH__
    bits = (unsigned long long)__double_as_longlong(v);
#else
    __builtin_memcpy(&bits, &v, 8);
#endif
    const bool neg = bits >> 63;
    const int ex = (int)((bits >> 52) & 0x7FF);
    const unsigned long long fr = bits & ((1ull << 52) - 1);
    if (ex == 0x7FF) {
        if (neg) out.put('-');
        out.put(fr ? 'n' : 'i');
        out.put(fr ? 'a' : 'n');
        out.put(fr ? 'n' : 'f');
        return;
    }
    if (ex == 0 && fr == 0) {
        if (neg) out.put('-');
        out.put('0');
        return;
    }
    const unsigned long long m = ex ? (fr | (1ull << 52)) : fr;
    const int e = (ex ? ex : 1) - 1075;
    const int E2 = e + (64 - clz64(m)) - 1;        // 2^E2 <= |v| < 2^(E2+1)
    if (E2 < -56 || E2 > 119) {
        fmt_g6_wide_to(m, e, neg, out);
        return;
    }
    int X = (E2 * 78913) >> 18;                     // floor(E2 * log10(2)): X or X-1 of the true exponent
    for (int iter = 0; iter < 3; iter++) {
        const int k = 5 - X;                        // scale by 10^k
        u128 T, R, half;                            // T = floor(|v| 10^k); fraction R / (2 half)
        bool exact_half_known = true;
        if (k >= 0) {
            if (k > 22) {
                fmt_g6_wide_to(m, e, neg, out);
                return;
            }
            const u128 N = (u128)m * pow10_128(k);
            if (e >= 0) {
                if (bitlen128(N) + e > 127) {
                    fmt_g6_wide_to(m, e, neg, out);
                    return;
                }
                T = N << e;
                R = 0;
                half = 1;
            } else {
                const int s = -e;
                if (s > 126) {
                    fmt_g6_wide_to(m, e, neg, out);
                    return;
                }
                T = N >> s;
                R = N & ((((u128)1) << s) - 1);
                half = ((u128)1) << (s - 1);
            }
        } else {
            const int j = -k;
            if (j > 37) {
                fmt_g6_wide_to(m, e, neg, out);
                return;
            }
            u128 M = m, Dv = pow10_128(j);
            if (e >= 0) {
                if (64 - clz64(m) + e > 127) {
                    fmt_g6_wide_to(m, e, neg, out);
                    return;
                }
                M = M << e;
            } else {
                if (bitlen128(Dv) + (-e) > 126) {
                    fmt_g6_wide_to(m, e, neg, out);
                    return;
                }
                Dv = Dv << (-e);
            }
            T = M / Dv;
            R = M % Dv;
            // compare 2R with Dv: R / Dv > 1/2 <=> 2R > Dv
            exact_half_known = false;
            half = Dv;   // compare 2R against Dv below
        }
        if (T < 100000u) {
            X--;
            continue;
        }
        if (T >= 1000000u) {
            X++;
            continue;
        }
        unsigned D = (unsigned)T;
        int cmp;   // sign of (fraction - 1/2)
        if (exact_half_known) cmp = R > half ? 1 : (R == half ? 0 : -1);
        else cmp = 2 * R > half ? 1 : (2 * R == half ? 0 : -1);
        if (cmp > 0 || (cmp == 0 && (D & 1u))) D++;
        if (D == 1000000u) {
            D = 100000u;
            X++;
        }
        emit_g6(D, X, neg, out);
        return;
    }
    fmt_g6_wide_to(m, e, neg, out);
}

// printf("%d", v) into a sink
template <class S>
N2M_HD inline void fmt_d(int v, S &out) {
    unsigned u = v < 0 ? 0u - (unsigned)v : (unsigned)v;
    if (v < 0) out.put('-');
    unsigned long long dg = 0;   // decimal digits, 4 bits each, least significant first
    int k = 0;
    do {
        dg |= (unsigned long long)(u % 10u) << (4 * k++);
        u /= 10u;
    } while (u);
    while (k) out.put((char)('0' + ((dg >> (4 * --k)) & 15u)));
}

// char-buffer forms (return the length)
N2M_HD inline int fmt_g6(double v, char *out) {
    CharSink cs{out};
    fmt_g6(v, cs);
    return cs.n;
}
N2M_HD inline int fmt_d(int v, char *out) {
    CharSink cs{out};
    fmt_d(v, cs);
    return cs.n;
}

}  // namespace n2mfmt
