// smooth_core.cuh — the fused three-pass pre-smooth of one output column
// (32 x 16 voxels, a run of z slices), shared by the single-volume kernel and
// the batched atlas kernel.  See smooth.cu for the design; this header only
// holds the tile loop, parameterised by where input voxels come from and
// where results go.
#pragma once
#include <float.h>
#include <limits.h>

#include "exact.cuh"
#include "n2m_internal.cuh"

namespace smooth {
constexpr int STX = 32, STY = 16, SZC = 32;

// running range / bbox / non-finite count of the values a thread produced
struct Acc {
    float mn, mx;
    int lo0, lo1, lo2, hi0, hi1, hi2;
    unsigned nf;
    __device__ void init() {
        mn = FLT_MAX; mx = -FLT_MAX;
        lo0 = lo1 = lo2 = INT_MAX;
        hi0 = hi1 = hi2 = INT_MIN;
        nf = 0;
    }
    __device__ __forceinline__ void add(float v, int x, int y, int z, float iso) {
        if (!isfinite(v)) { nf++; return; }
        mn = fminf(mn, v);
        mx = fmaxf(mx, v);
        if (v >= iso) {
            lo0 = min(lo0, x); lo1 = min(lo1, y); lo2 = min(lo2, z);
            hi0 = max(hi0, x); hi1 = max(hi1, y); hi2 = max(hi2, z);
        }
    }
    // the K values of one lane's run along z (x, y fixed; z = z0 + k), those
    // whose bit is set in `take`: min/max per value, the bbox once per run
    template <int K>
    __device__ __forceinline__ void add_run(const float (&r)[K], unsigned take, int x, int y, int z0, float iso) {
        unsigned ge = 0;
#pragma unroll
        for (int k = 0; k < K; k++) {
            if (!(take >> k & 1u)) continue;
            const float v = r[k];
            if (!isfinite(v)) { nf++; continue; }
            mn = fminf(mn, v);
            mx = fmaxf(mx, v);
            ge |= (unsigned)(v >= iso) << k;
        }
        if (ge) {
            lo0 = min(lo0, x); lo1 = min(lo1, y); lo2 = min(lo2, z0 + __ffs(ge) - 1);
            hi0 = max(hi0, x); hi1 = max(hi1, y); hi2 = max(hi2, z0 + 31 - __clz(ge));
        }
    }
    // block-wide reduction, one set of atomics per CTA
    __device__ void flush(VolStats *st, bool minmax) {
        const unsigned full = 0xffffffffu;
        for (int o = 16; o; o >>= 1) {
            mn = fminf(mn, __shfl_xor_sync(full, mn, o));
            mx = fmaxf(mx, __shfl_xor_sync(full, mx, o));
            lo0 = min(lo0, __shfl_xor_sync(full, lo0, o)); lo1 = min(lo1, __shfl_xor_sync(full, lo1, o));
            lo2 = min(lo2, __shfl_xor_sync(full, lo2, o)); hi0 = max(hi0, __shfl_xor_sync(full, hi0, o));
            hi1 = max(hi1, __shfl_xor_sync(full, hi1, o)); hi2 = max(hi2, __shfl_xor_sync(full, hi2, o));
            nf += __shfl_xor_sync(full, nf, o);
        }
        __shared__ Acc part[32];
        const int nthr = blockDim.x * blockDim.y;
        const int tid = threadIdx.y * blockDim.x + threadIdx.x;
        if ((tid & 31) == 0) part[tid >> 5] = *this;
        __syncthreads();
        if (tid == 0) {
            Acc a = part[0];
            for (int w = 1; w < (nthr + 31) / 32; w++) {
                const Acc &b = part[w];
                a.mn = fminf(a.mn, b.mn); a.mx = fmaxf(a.mx, b.mx);
                a.lo0 = min(a.lo0, b.lo0); a.lo1 = min(a.lo1, b.lo1); a.lo2 = min(a.lo2, b.lo2);
                a.hi0 = max(a.hi0, b.hi0); a.hi1 = max(a.hi1, b.hi1); a.hi2 = max(a.hi2, b.hi2);
                a.nf += b.nf;
            }
            if (minmax && a.mn <= a.mx) {
                atomicMin(&st->vmin, f2ord(a.mn));
                atomicMax(&st->vmax, f2ord(a.mx));
            }
            if (a.lo0 != INT_MAX) {
                atomicMin(&st->lo[0], a.lo0); atomicMin(&st->lo[1], a.lo1); atomicMin(&st->lo[2], a.lo2);
                atomicMax(&st->hi[0], a.hi0); atomicMax(&st->hi[1], a.hi1); atomicMax(&st->hi[2], a.hi2);
            }
            if (a.nf) atomicAdd(&st->nonfinite, a.nf);
        }
    }
};

// Evaluations whose fast path cannot prove the rounding (about 2.5 % on data
// whose voxels share an exponent: their exact tap sum often lands exactly on
// a float rounding midpoint) are queued in shared memory and evaluated with
// the reference's double sequence by the whole CTA at once, so each FP64
// instruction serves up to 32 queued voxels instead of stalling a warp for one.
struct QItem {
    float v[5];
    int dst;
};
constexpr int NT = STX * STY;
constexpr int QCAP = (STY + 4) * STX;

__device__ __forceinline__ void enqueue(QItem *q, int *qn, float a, float b, float c, float d, float e, int dst) {
    const int k = atomicAdd(qn, 1);
    q[k].v[0] = a; q[k].v[1] = b; q[k].v[2] = c; q[k].v[3] = d; q[k].v[4] = e;
    q[k].dst = dst;
}

__device__ __forceinline__ void drain(const QItem *q, int n, float *dst, int tid) {
    for (int i = tid; i < n; i += NT) dst[q[i].dst] = tap5_double(q[i].v[0], q[i].v[1], q[i].v[2], q[i].v[3], q[i].v[4]);
}

// Computes outputs (x, y, z) for x in [x0, min(x0+32, ox1)), y in
// [y0, min(y0+16, oy1)), z in [z0, zend).  src.load(x, y, z) returns input
// voxels (called only inside the volume); sink.put(x, y, z, v) stores a
// result; acc collects the range/bbox of this thread's results.  Blur rows
// within 2 voxels of a face of the nx x ny x nz volume keep their input.
template <class Src, class Sink>
__device__ __forceinline__ void column(const Src &src, Sink &sink, Acc &acc, float iso, int x0, int y0, int z0, int zend,
                                       int ox1, int oy1, int nx, int ny, int nz) {
    __shared__ float raw[STY + 4][STX + 4];
    __shared__ float xs[STY + 4][STX];
    __shared__ float fix[NT];
    __shared__ QItem q[QCAP];
    __shared__ int qn[3];
    const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * STX + tx;
    const int gx = x0 + tx, gy = y0 + ty;
    const int zlo = max(z0 - 2, 0), zhi = min(zend + 2, nz);
    const bool own = gx < ox1 && gy < oy1;
    const bool xin = gx >= 2 && gx <= nx - 3, yin = gy >= 2 && gy <= ny - 3;
    float r0 = 0.f, r1 = 0.f, r2 = 0.f, r3 = 0.f, r4 = 0.f;
    for (int zi = zlo; zi < zhi; zi++) {
        for (int i = tid; i < (STY + 4) * (STX + 4); i += NT) {
            const int r = i / (STX + 4), c = i - r * (STX + 4);
            const int yy = y0 - 2 + r, xx = x0 - 2 + c;
            raw[r][c] = (yy >= 0 && yy < ny && xx >= 0 && xx < nx) ? src.load(xx, yy, zi) : 0.f;
        }
        if (tid < 3) qn[tid] = 0;
        __syncthreads();
        // x pass (rows y0-2 .. y0+STY+1)
        for (int r = ty; r < STY + 4; r += STY) {
            const int yy = y0 - 2 + r;
            float v = 0.f;
            if (gx < nx && yy >= 0 && yy < ny) {
                if (xin) {
                    if (!tap5_fast(raw[r][tx], raw[r][tx + 1], raw[r][tx + 2], raw[r][tx + 3], raw[r][tx + 4], &v))
                        enqueue(q, &qn[0], raw[r][tx], raw[r][tx + 1], raw[r][tx + 2], raw[r][tx + 3], raw[r][tx + 4],
                                r * STX + tx);
                } else {
                    v = raw[r][tx + 2];
                }
            }
            xs[r][tx] = v;
        }
        __syncthreads();
        if (int n = qn[0]) {
            drain(q, n, &xs[0][0], tid);
            __syncthreads();
        }
        // y pass
        float Y = 0.f;
        bool yq = false;
        if (own) {
            if (yin) {
                yq = !tap5_fast(xs[ty][tx], xs[ty + 1][tx], xs[ty + 2][tx], xs[ty + 3][tx], xs[ty + 4][tx], &Y);
                if (yq) enqueue(q, &qn[1], xs[ty][tx], xs[ty + 1][tx], xs[ty + 2][tx], xs[ty + 3][tx], xs[ty + 4][tx], tid);
            } else {
                Y = xs[ty + 2][tx];
            }
        }
        __syncthreads();
        if (int n = qn[1]) {
            drain(q, n, fix, tid);
            __syncthreads();
            if (yq) Y = fix[tid];
        }
        r0 = r1; r1 = r2; r2 = r3; r3 = r4; r4 = Y;
        // z pass
        const int zo = zi - 2;
        const bool zint = own && zo >= z0 && zo < zend && zo >= 2 && zo <= nz - 3;
        float o = 0.f;
        bool zq = false;
        if (zint) {
            zq = !tap5_fast(r0, r1, r2, r3, r4, &o);
            if (zq) enqueue(q, &qn[2], r0, r1, r2, r3, r4, tid);
        }
        __syncthreads();
        if (int n = qn[2]) {   // owners read the y results before the barrier above
            drain(q, n, fix, tid);
            __syncthreads();
            if (zq) o = fix[tid];
        }
        if (zint) {
            sink.put(gx, gy, zo, o);
            acc.add(o, gx, gy, zo, iso);
        }
        if (own && zi >= z0 && zi < zend && (zi < 2 || zi > nz - 3)) {   // rows left unfiltered along z
            sink.put(gx, gy, zi, Y);
            acc.add(Y, gx, gy, zi, iso);
        }
        __syncthreads();
    }
}
}  // namespace smooth
