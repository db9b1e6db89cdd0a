// isolevel.cu — Otsu isolevel (setThreshold, src/isolevel.c:245-277) with the
// robust range of nifti_robust_range (src/isolevel.c:35-139) and the Otsu
// search of nii_otsu (src/isolevel.c:141-243), for nii2mesh's default
// isolevel (src/nii2mesh.c:586).
//
// Device passes over the volume: (1) min/max of the non-NaN voxels and the
// NaN count, (2) the 1001-bin histogram the 2nd/98th percentiles are read
// from, (3) the 256-bin histogram on the robust range.  Bin indices are the
// reference's float arithmetic, (int)round((v - mn) * scl), rounded half away
// from zero.  The percentile walk and the Otsu tables are a few hundred
// operations on the host, in the reference's order and double arithmetic; the
// three-level search (modes 1 and 3: about 2.7 M triples of bins) runs on the
// device with the same double sums and the reference's tie rule.
#include <float.h>
#include <math.h>

#include <algorithm>
#include <vector>

#include "n2m_internal.cuh"

namespace {
constexpr int NB_RANGE = 1001, NB_OTSU = 256;

struct ThRange {
    int vmin, vmax;                  // ordered-int min/max of the non-NaN voxels
    unsigned long long nnan;
    unsigned long long pad;
};

// (int)round(x) for the bin of a finite product; NaN (0 * inf on a constant
// volume) goes to bin 0, like the reference's clamp does on every platform
__device__ __forceinline__ long long bin_of(float x) {
    if (!(x == x)) return 0;
    const float r = roundf(x);
    if (r >= 9.0e18f) return 9000000000000000000ll;
    if (r <= -9.0e18f) return -9000000000000000000ll;
    return (long long)r;
}

__global__ void __launch_bounds__(256) k_th_range(const float *__restrict__ v, long long n, ThRange *out) {
    float mn = INFINITY, mx = -INFINITY;
    unsigned long long nn = 0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const float x = __ldg(v + i);
        if (x != x) { nn++; continue; }
        mn = fminf(mn, x);
        mx = fmaxf(mx, x);
    }
    for (int o = 16; o; o >>= 1) {
        mn = fminf(mn, __shfl_xor_sync(0xffffffffu, mn, o));
        mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
        nn += __shfl_xor_sync(0xffffffffu, nn, o);
    }
    if ((threadIdx.x & 31) == 0) {
        if (mn <= mx) {
            atomicMin(&out->vmin, f2ord(mn));
            atomicMax(&out->vmax, f2ord(mx));
        }
        if (nn) atomicAdd(&out->nnan, nn);
    }
}

// histogram of bin_of((v - mn) * scl) over the non-NaN voxels, bins clamped
// to [0, nb-1] (the 256-bin pass clamps like the reference; the 1001-bin
// indices are in range for every finite volume)
template <int NBINS>
__global__ void __launch_bounds__(256) k_th_hist(const float *__restrict__ v, long long n, float mn, float scl,
                                                 unsigned *hist) {
    __shared__ unsigned h[NBINS];
    for (int i = threadIdx.x; i < NBINS; i += blockDim.x) h[i] = 0;
    __syncthreads();
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const float x = __ldg(v + i);
        if (x != x) continue;
        long long b = bin_of(__fmul_rn(__fsub_rn(x, mn), scl));
        b = b < NBINS - 1 ? b : NBINS - 1;
        b = b > 0 ? b : 0;
        atomicAdd(&h[b], 1u);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < NBINS; i += blockDim.x)
        if (h[i]) atomicAdd(&hist[i], h[i]);
}

// Three-level Otsu search: thread (l, m) scans h = m+1 .. nb-2 for the first
// maximum of P[l] + P[l+1][m] + P[m+1][h] + P[h+1][nb-1] (left-to-right double
// sums); the block keeps the first maximum in (l, m, h) order.
struct Best {
    double v;
    unsigned idx;   // l << 16 | m << 8 | h
};

__global__ void __launch_bounds__(256) k_otsu3(const double *__restrict__ P, int nb, Best *out) {
    const int l = blockIdx.x, m = l + 1 + threadIdx.x;
    Best b = {-INFINITY, 0xffffffffu};
    if (l < nb - 3 && m < nb - 2) {
        const double base = __dadd_rn(P[l], P[(l + 1) * nb + m]);
        for (int h = m + 1; h < nb - 1; h++) {
            const double v = __dadd_rn(__dadd_rn(base, P[(m + 1) * nb + h]), P[(h + 1) * nb + nb - 1]);
            if (v > b.v) {
                b.v = v;
                b.idx = (unsigned)l << 16 | (unsigned)m << 8 | (unsigned)h;
            }
        }
    }
    __shared__ Best part[256];
    part[threadIdx.x] = b;
    __syncthreads();
    for (int s = 128; s; s >>= 1) {
        if (threadIdx.x < s) {
            const Best o = part[threadIdx.x + s];
            Best &me = part[threadIdx.x];
            if (o.v > me.v || (o.v == me.v && o.idx < me.idx)) me = o;
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) out[l] = part[0];
}

// the reference's table transform (src/isolevel.c:156-180), host, double
void otsu_table(const unsigned *H, int nb, std::vector<double> &P) {
    double Sum = 0.0;
    for (int v = 0; v < nb; v++) Sum = Sum + H[v];
    P.assign((size_t)nb * nb, 0.0);
    std::vector<double> S((size_t)nb * nb, 0.0);
    P[0] = H[0];
    S[0] = H[0];
    for (int v = 1; v < nb; v++) {
        const double prob = H[v] / Sum;
        P[v] = P[v - 1] + prob;
        S[v] = S[v - 1] + (v + 1) * prob;
    }
    for (int u = 1; u < nb; u++)
        for (int v = u; v < nb; v++) {
            P[(size_t)u * nb + v] = P[v] - P[u - 1];
            S[(size_t)u * nb + v] = S[v] - S[u - 1];
        }
    for (int u = 0; u < nb; u++)
        for (int v = u; v < nb; v++) {
            const size_t k = (size_t)u * nb + v;
            if (P[k] != 0) P[k] = (S[k] * S[k]) / P[k];
        }
}

unsigned grid_for(long long n) {
    long long b = (n + 255) / 256;
    if (b > 152 * 8) b = 152 * 8;
    return b > 0 ? (unsigned)b : 1u;
}
}  // namespace

n2m_status isolevel_otsu(const float *d_img, long long nvox, int mode123, ThresholdWork &w, cudaStream_t s,
                         float *result) {
    *result = 1.0f;   // the reference's value when there are no voxels
    if (nvox < 1) return N2M_OK;
    if (nvox > 2147483647ll) {
        n2m_set_error("setThreshold: %lld voxels exceed the reference's int count", nvox);
        return N2M_ERR_TOO_LARGE;
    }
    // one buffer: range | 1001 + 256 bins | Best[256] at a 16-byte boundary (it holds doubles)
    const size_t best_off = (sizeof(ThRange) + (NB_RANGE + NB_OTSU) * sizeof(unsigned) + 15) / 16 * 16;
    CKS(w.buf.ensure(best_off + 256 * sizeof(Best)));
    ThRange *d_r = w.buf.as<ThRange>();
    unsigned *d_h1 = (unsigned *)(d_r + 1), *d_h2 = d_h1 + NB_RANGE;
    Best *d_best = (Best *)((char *)w.buf.p + best_off);
    ThRange hr;
    ThRange *h_r = &hr;
    std::vector<unsigned> hist_v(NB_RANGE);
    unsigned *h_hist = hist_v.data();
    std::vector<Best> best_v(256);
    Best *h_best = best_v.data();

    // (1) range of the non-NaN voxels (src/isolevel.c:47-61)
    *h_r = ThRange{f2ord_host(INFINITY), f2ord_host(-INFINITY), 0, 0};
    CK(cudaMemcpyAsync(d_r, h_r, sizeof(ThRange), cudaMemcpyHostToDevice, s));
    { k_th_range<<<grid_for(nvox), 256, 0, s>>>(d_img, nvox, d_r); N2M_COUNT(); }
    CKL();
    CK(cudaMemcpyAsync(h_r, d_r, sizeof(ThRange), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    float pct2 = 0.0f, pct98 = 1.0f;
    const float mn = ord2f(h_r->vmin), mx = ord2f(h_r->vmax);
    const long long nvalid = nvox - (long long)h_r->nnan;
    if (nvalid > 0) {   // otherwise all NaN: the initial 0..1 (src/isolevel.c:63-64)
        if (mn == mx) {
            pct2 = mn;
            pct98 = mx;
        } else {
            const size_t n2pct = (size_t)round(nvalid * 0.02);
            if (n2pct < 1 || nvalid < 100) {
                pct2 = mn;
                pct98 = mx;
            } else {
                // (2) percentile histogram (src/isolevel.c:83-101), walk (:102-133)
                const float scl = (NB_RANGE - 1) / (mx - mn);
                CK(cudaMemsetAsync(d_h1, 0, NB_RANGE * sizeof(unsigned), s));
                { k_th_hist<NB_RANGE><<<grid_for(nvox), 256, 0, s>>>(d_img, nvox, mn, scl, d_h1); N2M_COUNT(); }
                CKL();
                CK(cudaMemcpyAsync(h_hist, d_h1, NB_RANGE * sizeof(unsigned), cudaMemcpyDeviceToHost, s));
                CK(cudaStreamSynchronize(s));
                size_t n = 0, lo = 0;
                while (n < n2pct && lo < (size_t)NB_RANGE) n += h_hist[lo++];
                lo--;
                n = 0;
                int hi = NB_RANGE;
                while (n < n2pct && hi > 0) n += h_hist[--hi];
                if ((int)lo == hi) {
                    int ok = -1;
                    while (ok != 0) {
                        if (lo > 0) {
                            lo--;
                            if (h_hist[lo] > 0) ok = 0;
                        }
                        if (ok != 0 && hi < NB_RANGE - 1) {
                            hi++;
                            if (h_hist[hi] > 0) ok = 0;
                        }
                        if (lo == 0 && hi == NB_RANGE - 1) ok = 0;
                    }
                }
                pct2 = (float)lo / scl + mn;
                pct98 = (float)hi / scl + mn;
            }
        }
    }
    // (3) Otsu histogram on the robust range (src/isolevel.c:250-262)
    const float scl = (NB_OTSU - 1) / (pct98 - pct2);
    CK(cudaMemsetAsync(d_h2, 0, NB_OTSU * sizeof(unsigned), s));
    { k_th_hist<NB_OTSU><<<grid_for(nvox), 256, 0, s>>>(d_img, nvox, pct2, scl, d_h2); N2M_COUNT(); }
    CKL();
    CK(cudaMemcpyAsync(h_hist, d_h2, NB_OTSU * sizeof(unsigned), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    double Sum = 0.0;
    for (int v = 0; v < NB_OTSU; v++) Sum = Sum + h_hist[v];
    int dark = 0, mid = 0, bright = 0;
    if (Sum > 0) {
        otsu_table(h_hist, NB_OTSU, w.P);
        const std::vector<double> &P = w.P;
        const int nb = NB_OTSU;
        if (mode123 == 1 || mode123 == 3) {
            // three boundaries (src/isolevel.c:182-205): start from the quartiles, keep the first strict maximum
            int lo = (int)(0.25 * nb), mi = (int)(0.50 * nb), hi = (int)(0.75 * nb);
            const double start = P[lo] + P[(size_t)(lo + 1) * nb + mi] + P[(size_t)(mi + 1) * nb + hi] +
                                 P[(size_t)(hi + 1) * nb + 255];
            CKS(w.table.ensure((size_t)nb * nb * sizeof(double)));
            CK(cudaMemcpyAsync(w.table.p, P.data(), (size_t)nb * nb * sizeof(double), cudaMemcpyHostToDevice, s));
            { k_otsu3<<<nb - 3, 256, 0, s>>>(w.table.as<double>(), nb, d_best); N2M_COUNT(); }
            CKL();
            CK(cudaMemcpyAsync(h_best, d_best, (nb - 3) * sizeof(Best), cudaMemcpyDeviceToHost, s));
            CK(cudaStreamSynchronize(s));
            Best g = {-INFINITY, 0xffffffffu};
            for (int l = 0; l < nb - 3; l++)
                if (h_best[l].v > g.v || (h_best[l].v == g.v && h_best[l].idx < g.idx)) g = h_best[l];
            if (g.v > start) {
                lo = (int)(g.idx >> 16);
                mi = (int)((g.idx >> 8) & 255u);
                hi = (int)(g.idx & 255u);
            }
            dark = lo;
            mid = mi;
            bright = hi;
        } else {
            // one boundary (src/isolevel.c:222-236)
            int thresh = (int)(0.25 * nb);
            double best = P[thresh] + P[(size_t)(thresh + 1) * nb + nb - 1];
            for (int i = 0; i < nb - 1; i++) {
                const double v = P[i] + P[(size_t)(i + 1) * nb + nb - 1];
                if (v > best) {
                    thresh = i;
                    best = v;
                }
            }
            dark = mid = bright = thresh;
        }
    }
    if (mode123 == 1) *result = (dark / scl) + pct2;
    else if (mode123 == 3) *result = (bright / scl) + pct2;
    else *result = (mid / scl) + pct2;
    return N2M_OK;
}
