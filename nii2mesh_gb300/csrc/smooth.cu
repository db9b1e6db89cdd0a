// smooth.cu — pre-smooth (src/meshify.c:170-216) and the volume reductions of
// meshify (range, bbox; src/meshify.c:305-371).
//
// k_smooth: one fused pass for all three separable blur passes.  A CTA owns a
// 32x16 column of output voxels and streams along z over a chunk of slices:
// per input slice it stages the raw slice (+2 halo in x and y) in shared
// memory, runs the x pass for the 16+4 rows it needs, the y pass for its own
// 16 rows, and keeps the last five y-pass results of each column in registers,
// so the z pass needs no further memory traffic.  Every tap sum is rounded
// exactly as the reference's double arithmetic rounds it (exact.cuh), so the
// output is bit-identical to quick_smooth().  The range (min/max), the count
// of non-finite voxels and the bbox of voxels >= iso are reduced in the same
// pass.  Algorithmic traffic: 4 B read + 4 B written per voxel.
#include <float.h>

#include <algorithm>

#include "exact.cuh"
#include "n2m_internal.cuh"

namespace {
constexpr int STX = 32, STY = 16, SZC = 32;

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

__global__ void __launch_bounds__(NT, 2) k_smooth(const float *__restrict__ in, float *__restrict__ out, int nx,
                                                  int ny, int nz, float iso, VolStats *st) {
    __shared__ float raw[STY + 4][STX + 4];
    __shared__ float xs[STY + 4][STX];
    __shared__ float fix[NT];
    __shared__ QItem q[QCAP];
    __shared__ int qn[3];
    const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * STX + tx;
    const int x0 = blockIdx.x * STX, y0 = blockIdx.y * STY, z0 = blockIdx.z * SZC;
    const int gx = x0 + tx, gy = y0 + ty;
    const int zend = min(z0 + SZC, nz);
    const int zlo = max(z0 - 2, 0), zhi = min(zend + 2, nz);
    const size_t nxy = (size_t)nx * ny;
    const bool own = gx < nx && gy < ny;
    const bool xin = gx >= 2 && gx <= nx - 3, yin = gy >= 2 && gy <= ny - 3;
    float r0 = 0.f, r1 = 0.f, r2 = 0.f, r3 = 0.f, r4 = 0.f;
    Acc acc;
    acc.init();
    for (int zi = zlo; zi < zhi; zi++) {
        const float *slice = in + (size_t)zi * nxy;
        for (int i = tid; i < (STY + 4) * (STX + 4); i += NT) {
            const int r = i / (STX + 4), c = i - r * (STX + 4);
            const int yy = y0 - 2 + r, xx = x0 - 2 + c;
            float v = 0.f;
            if (yy >= 0 && yy < ny && xx >= 0 && xx < nx) v = __ldg(slice + (size_t)yy * nx + xx);
            raw[r][c] = v;
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
                if (yq) enqueue(q, &qn[1], xs[ty][tx], xs[ty + 1][tx], xs[ty + 2][tx],
                                xs[ty + 3][tx], xs[ty + 4][tx], tid);
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
            out[(size_t)zo * nxy + (size_t)gy * nx + gx] = o;
            acc.add(o, gx, gy, zo, iso);
        }
        if (own && zi >= z0 && zi < zend && (zi < 2 || zi > nz - 3)) {   // rows left unfiltered along z
            out[(size_t)zi * nxy + (size_t)gy * nx + gx] = Y;
            acc.add(Y, gx, gy, zi, iso);
        }
        __syncthreads();
    }
    acc.flush(st, true);
}

// range / bbox / non-finite count of an existing volume
__global__ void __launch_bounds__(256) k_stats(const float *__restrict__ vol, int nx, int ny, int nz, float iso,
                                               VolStats *st, bool minmax) {
    Acc acc;
    acc.init();
    const int y = blockIdx.y, z = blockIdx.z;
    const float *row = vol + ((size_t)z * ny + y) * nx;
    for (int x = blockIdx.x * blockDim.x + threadIdx.x; x < nx; x += gridDim.x * blockDim.x)
        acc.add(__ldg(row + x), x, y, z, iso);
    acc.flush(st, minmax);
}
}  // namespace

void stats_init_host(VolStats *h) {
    h->vmin = INT_MAX;
    h->vmax = INT_MIN;
    for (int i = 0; i < 3; i++) { h->lo[i] = INT_MAX; h->hi[i] = INT_MIN; }
    h->nonfinite = 0;
    h->pad = 0;
}

n2m_status launch_smooth(const float *in, float *out, int nx, int ny, int nz, float iso, VolStats *st,
                         cudaStream_t s) {
    dim3 grid((nx + STX - 1) / STX, (ny + STY - 1) / STY, (nz + SZC - 1) / SZC);
    { k_smooth<<<grid, dim3(STX, STY), 0, s>>>(in, out, nx, ny, nz, iso, st); N2M_COUNT(); }
    CKL();
    return N2M_OK;
}

namespace {
// transposed 5-tap pass along one axis: out_j = sum over interior rows i with
// |i-j| <= 2 of w_|i-j| g_i, plus g_j where j itself is a row left unfiltered
__global__ void k_smooth_T(const float *__restrict__ g, float *__restrict__ out, int nx, int ny, int nz, int axis) {
    const long long n = (long long)nx * ny * nz;
    const long long stride = axis == 0 ? 1 : (axis == 1 ? nx : (long long)nx * ny);
    const int len = axis == 0 ? nx : (axis == 1 ? ny : nz);
    const float w[3] = {0.45f, 0.225f, 0.05f};
    for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < n; v += (long long)gridDim.x * blockDim.x) {
        const long long q = v / stride;
        const int j = (int)(axis == 0 ? q % nx : (axis == 1 ? q % ny : q));
        float acc = (j < 2 || j > len - 3) ? g[v] : 0.f;
        for (int d = -2; d <= 2; d++) {
            const int i = j + d;
            if (i >= 2 && i <= len - 3) acc += w[d < 0 ? -d : d] * g[v + d * stride];
        }
        out[v] = acc;
    }
}
}  // namespace

n2m_status launch_smooth_adjoint(const float *g, float *tmp, float *out, int nx, int ny, int nz, cudaStream_t s) {
    const long long n = (long long)nx * ny * nz;
    const unsigned blocks = (unsigned)std::min<long long>((n + 255) / 256, 152 * 64);
    { k_smooth_T<<<blocks, 256, 0, s>>>(g, out, nx, ny, nz, 2); N2M_COUNT(); }
    { k_smooth_T<<<blocks, 256, 0, s>>>(out, tmp, nx, ny, nz, 1); N2M_COUNT(); }
    { k_smooth_T<<<blocks, 256, 0, s>>>(tmp, out, nx, ny, nz, 0); N2M_COUNT(); }
    CKL();
    return N2M_OK;
}

n2m_status launch_stats(const float *vol, int nx, int ny, int nz, float iso, bool minmax, VolStats *st,
                        cudaStream_t s) {
    dim3 grid((nx + 255) / 256 > 4 ? 4 : (nx + 255) / 256, ny, nz);
    { k_stats<<<grid, 256, 0, s>>>(vol, nx, ny, nz, iso, st, minmax); N2M_COUNT(); }
    CKL();
    return N2M_OK;
}
