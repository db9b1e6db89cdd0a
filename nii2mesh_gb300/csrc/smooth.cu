// smooth.cu — pre-smooth (src/meshify.c:170-216) and the volume reductions of
// meshify (range, bbox; src/meshify.c:305-371).
//
// The blur is three separable 5-tap passes (x, then y, then z) whose every
// tap sum is rounded exactly as the reference's double arithmetic rounds it
// (exact.cuh), so the output is bit-identical to quick_smooth().  One
// streaming kernel per pass (k_pass_x, k_pass_axis): a fast FP32 proof
// decides ~97 % of the taps, the rest are batched per warp and recomputed in
// FP64 by full warps; the z pass also reduces the range (min/max), the count
// of non-finite voxels and the bbox of voxels >= iso.  Traffic: 8 B per voxel
// per pass, three passes.  (The batched atlas smooths its sub-boxes with the
// fused column routine of smooth_core.cuh instead.)
#include <float.h>
#include <math.h>
#include <stddef.h>
#include <stdlib.h>

#include <cuda.h>            // CUtensorMap and its enums (the encoder comes from the driver at run time)
#include <cudaTypedefs.h>

#include <algorithm>
#include <map>
#include <mutex>

#include "smooth_core.cuh"

namespace {
using namespace smooth;

// range / bbox / non-finite count of an existing volume: a bounded grid whose
// warps stride over the rows, so the block flushes (one set of atomics each)
// stay few; every reduction is a min, max or count, so the order is free
__global__ void __launch_bounds__(256) k_stats(const float *__restrict__ vol, int nx, int ny, int nz, float iso,
                                               VolStats *st, bool minmax) {
    Acc acc;
    acc.init();
    const long long nrows = (long long)ny * nz;
    const int wpb = blockDim.x >> 5, lane = threadIdx.x & 31;
    for (long long r = (long long)blockIdx.x * wpb + (threadIdx.x >> 5); r < nrows; r += (long long)gridDim.x * wpb) {
        const int z = (int)(r / ny), y = (int)(r - (long long)z * ny);
        const float *row = vol + r * nx;
#pragma unroll 4
        for (int x = lane; x < nx; x += 32) acc.add(__ldg(row + x), x, y, z, iso);
    }
    acc.flush(st, minmax);
}
}  // namespace

void stats_init_host(VolStats *h) {
    h->vmin = INT_MAX;
    h->vmax = INT_MIN;
    for (int i = 0; i < 3; i++) { h->lo[i] = INT_MAX; h->hi[i] = INT_MIN; }
    h->nonfinite = 0;
    h->masked = 0;
}

// ---- three separable passes with batched exact fix-ups -------------------------
// x pass in -> out, y pass out -> tmp, z pass tmp -> out (with the range and
// bbox reductions).  Each pass evaluates every tap with the fast path; the
// voxels whose rounding the fast path cannot prove (about 2.5 % on data whose
// voxels share an exponent) are staged per warp in shared memory and, 32 at a
// time, recomputed with the reference's double sequence by the full warp, so
// each FP64 instruction serves 32 voxels.  A pass never reads its own
// outputs, so fix-ups can run whenever a batch is full.  Passes run at full
// occupancy with no redundant taps and no block-wide waits.
namespace {
constexpr unsigned FULL = 0xffffffffu;

// The pass being run: input, output, tap stride (1, nx or nx*ny) and, for
// the z pass, the reductions.
struct Pass {
    const float *in;
    float *out;
    unsigned stride;
    int nx, ny;
    unsigned nxy;
    float iso;
    VolStats *st;
};

// Per-warp stack of failed voxels in shared memory (sized by the kernel for
// 31 leftover entries plus what its steps push between drains).  All 32 lanes
// call push, drain and finish together; push adds at most 32 entries, drain
// recomputes full batches of 32.
template <bool STATS>
struct FixStage {
    unsigned *buf;
    int n;   // warp-uniform fill
    __device__ __forceinline__ void run(const Pass &P, Acc &acc, int lo, int cnt, int lane) {
        __syncwarp();
        if (lane < cnt) {
            const unsigned v = buf[lo + lane];
            const float *p = P.in + v;
            const long long s = P.stride;
            const float r = tap5_double(p[-2 * s], p[-s], p[0], p[s], p[2 * s]);
            P.out[v] = r;
            if (STATS) acc.add(r, (int)(v % (unsigned)P.nx), (int)((v / (unsigned)P.nx) % (unsigned)P.ny), (int)(v / P.nxy), P.iso);
        }
        __syncwarp();
    }
    __device__ __forceinline__ void push(bool fail, unsigned vox, int lane) {
        const unsigned m = __ballot_sync(FULL, fail);
        if (fail) buf[n + __popc(m & ((1u << lane) - 1u))] = vox;
        n += __popc(m);
    }
    // every lane queues the voxels base + k * step for the set bits k of fm
    // (one warp scan of the lanes' counts instead of one ballot per output)
    __device__ __forceinline__ void push_mask(unsigned fm, unsigned base, unsigned step, int lane) {
        if (!__any_sync(FULL, fm != 0u)) return;
        const int c = __popc(fm);
        int incl = c;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int t = __shfl_up_sync(FULL, incl, o);
            if (lane >= o) incl += t;
        }
        int at = n + incl - c;
        while (fm) {
            const int k = __ffs(fm) - 1;
            fm &= fm - 1u;
            buf[at++] = base + (unsigned)k * step;
        }
        n += __shfl_sync(FULL, incl, 31);
    }
    __device__ __forceinline__ void drain(const Pass &P, Acc &acc, int lane) {
        while (n >= 32) {
            n -= 32;
            run(P, acc, n, 32, lane);
        }
    }
    __device__ __forceinline__ void finish(const Pass &P, Acc &acc, int lane) {
        drain(P, acc, lane);
        if (n) run(P, acc, 0, n, lane);
        n = 0;
    }
};

// K outputs from the K + 4 inputs w[0 .. K+3] of one lane (output k is the tap
// sum of w[k .. k+4]).  When the K + 4 magnitudes lie within a factor 64 of one
// another the split path decides each tap (exact.cuh: tap5_split), otherwise
// tap5_fast; bit k of the returned mask marks an output neither could decide
// (r[k] is then a placeholder that the FP64 fix-up overwrites).
template <int K>
__device__ __forceinline__ unsigned taps_run(const float (&w)[K + 4], float (&r)[K]) {
    float mx = fabsf(w[0]), mn = fabsf(w[0]);
#pragma unroll
    for (int k = 1; k < K + 4; k++) {
        mx = fmaxf(mx, fabsf(w[k]));
        mn = fminf(mn, fabsf(w[k]));
    }
    unsigned fm = 0;
    if (split_group_ok(mn, mx)) {
        float h[K + 4], l[K + 4];
#pragma unroll
        for (int k = 0; k < K + 4; k++) split12(w[k], h[k], l[k]);
        const float mth = FMUL(mx, 0x1p-8f);
#pragma unroll
        for (int k = 0; k < K; k++) {
            float t;
            if (!tap5_split(h[k], l[k], h[k + 1], l[k + 1], h[k + 2], l[k + 2], h[k + 3], l[k + 3], h[k + 4], l[k + 4],
                            mth, &t))
                fm |= 1u << k;
            r[k] = t;
        }
    } else {
#pragma unroll
        for (int k = 0; k < K; k++) {
            float t = w[k + 2];
            if (!tap5_fast(w[k], w[k + 1], w[k + 2], w[k + 3], w[k + 4], &t)) fm |= 1u << k;
            r[k] = t;
        }
    }
    return fm;
}

// x pass: each warp takes whole rows (rows row0 .. row1-1 of the volume).
__global__ void __launch_bounds__(256) k_pass_x(Pass P, unsigned row0, unsigned row1) {
    __shared__ unsigned stage_buf[8][64];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    FixStage<false> F{stage_buf[w], 0};   // < 32 entries between steps, + 32
    Acc acc;   // unused by the x pass
    const int nx = P.nx;
    const unsigned nwarps = gridDim.x * (blockDim.x / 32);
    for (unsigned row = row0 + blockIdx.x * (blockDim.x / 32) + w; row < row1; row += nwarps) {
        const unsigned r0 = row * (unsigned)nx;
        for (int x0 = 0; x0 < nx; x0 += 32) {
            const int x = x0 + lane;
            const unsigned v = r0 + (unsigned)x;
            bool fail = false;
            if (x < nx) {
                float o;
                if (x >= 2 && x <= nx - 3) {
                    const float *p = P.in + v;
                    fail = !tap5_fast(__ldg(p - 2), __ldg(p - 1), __ldg(p), __ldg(p + 1), __ldg(p + 2), &o);
                } else {
                    o = __ldg(P.in + v);
                }
                if (!fail) P.out[v] = o;
            }
            F.push(fail, v, lane);
            F.drain(P, acc, lane);
        }
    }
    F.finish(P, acc, lane);
}

// x pass for rows whose length is a multiple of 4 (16-byte aligned rows):
// each thread takes 4 consecutive voxels with three float4 loads (its own and
// the neighbours' halves, mostly L1 hits) and one float4 store; voxels whose
// fast path fails are stored as placeholders and fixed by the same warp.
__global__ void __launch_bounds__(256) k_pass_x4(Pass P, unsigned row0, unsigned row1) {
    __shared__ unsigned stage_buf[8][32 * 5];   // < 32 between drains, + 4 per lane per step
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    FixStage<false> F{stage_buf[w], 0};
    Acc acc;   // unused by the x pass
    const int nx = P.nx, nq = nx / 4;
    const unsigned nwarps = gridDim.x * (blockDim.x / 32);
    for (unsigned row = row0 + blockIdx.x * (blockDim.x / 32) + w; row < row1; row += nwarps) {
        const float4 *r4 = reinterpret_cast<const float4 *>(P.in + (size_t)row * nx);
        float4 *o4 = reinterpret_cast<float4 *>(P.out + (size_t)row * nx);
        for (int q0 = 0; q0 < nq; q0 += 32) {
            const int q = q0 + lane, x0 = 4 * q;
            const bool act = q < nq;
            const float4 zero = make_float4(0.f, 0.f, 0.f, 0.f);
            const float4 A = act && q > 0 ? __ldg(r4 + q - 1) : zero;
            const float4 B = act ? __ldg(r4 + q) : zero;
            const float4 C = act && q + 1 < nq ? __ldg(r4 + q + 1) : zero;
            // x0-2 .. x0+5; past the row ends (only face voxels read them) stand-ins from
            // this quad, so that the group test of the split path sees row values only
            const float w[8] = {q > 0 ? A.z : B.x, q > 0 ? A.w : B.x, B.x, B.y, B.z, B.w,
                                q + 1 < nq ? C.x : B.w, q + 1 < nq ? C.y : B.w};
            float o[4];
            unsigned fm = 0;
            if (act) {
                fm = taps_run<4>(w, o);
#pragma unroll
                for (int j = 0; j < 4; j++)
                    if (x0 + j < 2 || x0 + j > nx - 3) {   // face voxels keep their input
                        o[j] = w[2 + j];
                        fm &= ~(1u << j);
                    }
                o4[q] = make_float4(o[0], o[1], o[2], o[3]);
            }
            F.push_mask(fm, row * (unsigned)nx + (unsigned)x0, 1u, lane);
            F.drain(P, acc, lane);
        }
    }
    F.finish(P, acc, lane);
}

// y and z passes: the volume is viewed as (outer, len, inner) with the pass
// axis of length len and stride inner.  A task is SEGS consecutive groups of
// 32 inner positions and a run of K positions along the axis; each lane
// slides a register window along the axis.  STATS: the z pass, which also
// reduces range and bbox.
// Outputs positions [p_lo, p_hi) along the axis of outer slices
// [outer0, outer0 + nouter) (the staged upload runs the passes slab by slab).
template <int K, int SEGS, bool STATS>
__global__ void __launch_bounds__(256, 4) k_pass_axis(Pass P, int len, unsigned outer0, unsigned nouter, int p_lo,
                                                      int p_hi) {
    __shared__ unsigned stage_buf[8][32 * (K + 1)];   // < 32 entries between segments, + up to 32 K per segment
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    FixStage<STATS> F{stage_buf[wid], 0};
    const unsigned inner = P.stride;
    const unsigned nseg = (inner + 31) / 32, nchunk = (nseg + SEGS - 1) / SEGS;
    const unsigned nrun = (unsigned)(p_hi - p_lo + K - 1) / K;
    const unsigned ntask = nchunk * nrun * nouter;
    const unsigned nwarps = gridDim.x * (blockDim.x / 32);
    Acc acc;
    acc.init();
    for (unsigned t = blockIdx.x * (blockDim.x / 32) + wid; t < ntask; t += nwarps) {
        const unsigned chunk = t % nchunk, rest = t / nchunk;
        const int p0 = p_lo + (int)(rest % nrun) * K;
        const unsigned o = outer0 + rest / nrun;
        const unsigned sbeg = chunk * SEGS, send = min(sbeg + SEGS, nseg);
        const bool interior = p0 >= 2 && p0 + K <= len - 2 && p0 + K <= p_hi;   // no face rows, whole run inside
        for (unsigned seg = sbeg; seg < send; seg++) {
            const unsigned i = seg * 32 + lane;
            const bool act = i < inner;
            const unsigned base = o * (unsigned)len * inner + i;
            float w[K + 4];
            int gx = 0, gy = 0;
            if (STATS) { gx = (int)(i % (unsigned)P.nx); gy = (int)(i / (unsigned)P.nx); }
            if (interior) {
                const float *q = P.in + base + (unsigned)(p0 - 2) * inner;
#pragma unroll
                for (int k = 0; k < K + 4; k++) w[k] = act ? __ldg(q + (unsigned)k * inner) : 0.f;
                float r[K];
                unsigned fm = 0;
                if (act) {
                    fm = taps_run<K>(w, r);
#pragma unroll
                    for (int k = 0; k < K; k++) P.out[base + (unsigned)(p0 + k) * inner] = r[k];   // placeholder where fm has bit k
                    if (STATS) acc.add_run<K>(r, ~fm, gx, gy, p0, P.iso);
                }
                F.push_mask(fm, base + (unsigned)p0 * inner, inner, lane);
            } else {
#pragma unroll
                for (int k = 0; k < K + 4; k++) {
                    const int pos = p0 - 2 + k;
                    w[k] = (act && pos >= 0 && pos < len) ? __ldg(P.in + base + (unsigned)pos * inner) : 0.f;
                }
#pragma unroll
                for (int k = 0; k < K; k++) {
                    const int pos = p0 + k;
                    bool fail = false;
                    const unsigned v = base + (unsigned)pos * inner;
                    if (act && pos < p_hi) {
                        float r = w[k + 2];
                        if (pos >= 2 && pos <= len - 3) fail = !tap5_fast(w[k], w[k + 1], w[k + 2], w[k + 3], w[k + 4], &r);
                        if (!fail) {
                            P.out[v] = r;
                            if (STATS) acc.add(r, gx, gy, pos, P.iso);
                        }
                    }
                    F.push(fail, v, lane);
                }
            }
            F.drain(P, acc, lane);
        }
    }
    F.finish(P, acc, lane);
    if (STATS) acc.flush(P.st, true);
}

// resident CTAs of a kernel on the current device, or 0 when the query fails
int resident_blocks(const void *fn, int threads) {
    int dev = 0, sms = 0, per_sm = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, threads, 0) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return sms * std::max(per_sm, 1);
}

constexpr int KRUN = 8, KSEG = 8;

// resident CTAs of each pass kernel, per device ordinal: queried on the first
// call on that device and kept once every query succeeded (a failed query
// gives 4 CTAs per SM of this call's device and is asked again next time)
struct PassGrids {
    int x, x4, a, z;
};
PassGrids pass_grids() {
    static std::mutex mu;
    static std::map<int, PassGrids> known;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) cudaGetLastError();
    {
        std::lock_guard<std::mutex> lk(mu);
        auto it = known.find(dev);
        if (it != known.end()) return it->second;
    }
    PassGrids g{resident_blocks((const void *)k_pass_x, 256), resident_blocks((const void *)k_pass_x4, 256),
                resident_blocks((const void *)k_pass_axis<KRUN, KSEG, false>, 256),
                resident_blocks((const void *)k_pass_axis<KRUN, KSEG, true>, 256)};
    if (g.x && g.x4 && g.a && g.z) {
        std::lock_guard<std::mutex> lk(mu);
        known[dev] = g;
        return g;
    }
    int sms = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms <= 0) {
        cudaGetLastError();
        sms = 152;
    }
    if (!g.x) g.x = 4 * sms;
    if (!g.x4) g.x4 = 4 * sms;
    if (!g.a) g.a = 4 * sms;
    if (!g.z) g.z = 4 * sms;
    return g;
}
}  // namespace

bool smooth_can_stage(int nx, int ny, int nz) { return (size_t)nx * ny * nz < ((size_t)1 << 32); }

// three passes; row and slice indices are 32-bit, so volumes stay below 2^32
// voxels (meshify accepts at most 2^31-1)
n2m_status launch_smooth(const float *in, float *out, float *tmp, int nx, int ny, int nz, float iso, VolStats *st,
                         cudaStream_t s, const StagedInput *stage) {
    const size_t n = (size_t)nx * ny * nz;
    if (n >= ((size_t)1 << 32)) {
        n2m_set_error("smoothing supports fewer than 2^32 voxels");
        return N2M_ERR_TOO_LARGE;
    }
    const PassGrids G = pass_grids();
    const int gx = G.x, gx4 = G.x4, ga = G.a, gz = G.z;
    const unsigned nxy = (unsigned)nx * ny;
    const Pass px{in, out, 1u, nx, ny, nxy, iso, st}, py{out, tmp, (unsigned)nx, nx, ny, nxy, iso, st},
        pz{tmp, out, nxy, nx, ny, nxy, iso, st};
    // 16-byte rows: the float4 x pass
    const bool x4 = nx % 4 == 0 && ((uintptr_t)in & 15) == 0 && ((uintptr_t)out & 15) == 0;
    auto pass_x = [&](unsigned r0, unsigned r1, unsigned g) -> n2m_status {
        if (x4) { k_pass_x4<<<std::min<unsigned>(g, (unsigned)gx4), 256, 0, s>>>(px, r0, r1); N2M_COUNT(); }
        else { k_pass_x<<<std::min<unsigned>(g, (unsigned)gx), 256, 0, s>>>(px, r0, r1); N2M_COUNT(); }
        CKL();
        return N2M_OK;
    };
    if (stage && stage->host) {
        // the copy stream may only overwrite `in` once earlier work on s is done with it
        CK(cudaEventRecord(stage->ev[N2M_STAGE_SLABS], s));
        CK(cudaStreamWaitEvent(stage->copy, stage->ev[N2M_STAGE_SLABS], 0));
        // per slab: x and y passes as soon as it has arrived, then the z pass of
        // every slice whose five y-pass inputs are done
        int zdone = 0;
        for (int k = 0; k < N2M_STAGE_SLABS; k++) {
            const int z0 = (int)((long long)nz * k / N2M_STAGE_SLABS), z1 = (int)((long long)nz * (k + 1) / N2M_STAGE_SLABS);
            if (z1 <= z0) continue;
            const size_t off = (size_t)z0 * nxy, bytes = (size_t)(z1 - z0) * nxy * sizeof(float);
            CK(cudaMemcpyAsync((float *)in + off, stage->host + off, bytes, cudaMemcpyHostToDevice, stage->copy));
            CK(cudaEventRecord(stage->ev[k], stage->copy));
            CK(cudaStreamWaitEvent(s, stage->ev[k], 0));
            const unsigned r0 = (unsigned)z0 * ny, r1 = (unsigned)z1 * ny;
            CKS(pass_x(r0, r1, std::max<unsigned>(1u, (r1 - r0 + 7) / 8)));
            { k_pass_axis<KRUN, KSEG, false><<<ga, 256, 0, s>>>(py, ny, (unsigned)z0, (unsigned)(z1 - z0), 0, ny); N2M_COUNT(); }
            const int zready = z1 == nz ? nz : z1 - 2;
            if (zready > zdone) {
                { k_pass_axis<KRUN, KSEG, true><<<gz, 256, 0, s>>>(pz, nz, 0u, 1u, zdone, zready); N2M_COUNT(); }
                zdone = zready;
            }
        }
    } else {
        CKS(pass_x(0u, (unsigned)ny * nz, 0xffffffffu));
        { k_pass_axis<KRUN, KSEG, false><<<ga, 256, 0, s>>>(py, ny, 0u, (unsigned)nz, 0, ny); N2M_COUNT(); }
        { k_pass_axis<KRUN, KSEG, true><<<gz, 256, 0, s>>>(pz, nz, 0u, 1u, 0, nz); N2M_COUNT(); }
    }
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
    const long long rows = (long long)ny * nz;
    const unsigned grid = (unsigned)std::max<long long>(1, std::min<long long>((rows + 7) / 8, 152 * 8));   // 8 rows per block
    { k_stats<<<grid, 256, 0, s>>>(vol, nx, ny, nz, iso, st, minmax); N2M_COUNT(); }
    CKL();
    return N2M_OK;
}

// ==== pre-smooth with exact rounding on demand ===================================
// Marching cubes reads the smoothed volume in two ways only: the sign of every
// grid point (value >= iso, and value - iso against the FLT_EPSILON clamp) and
// the values at the corners of the cubes the surface crosses.  So the volume
// is first smoothed approximately in one fused FP32 pass (pass A: one read and
// one write per voxel), with a rigorous error bound; the few voxels whose sign
// the bound leaves open, and the candidates for the volume's minimum and
// maximum, are recomputed with the reference's double sequence (pass B).
// After the sign words, the corners of every cube with mixed signs are marked
// (mc.cu: k_need) and the exact three-pass smoothing runs on those voxels
// only, the x and y passes on the voxels those depend on (marks dilated by +-2
// slices, then +-2 rows), each pass one thread per marked voxel.  Every value
// marching cubes reads is then the reference's float, bit for bit.
//
// Error bound of pass A: each pass evaluates the tap sum as an FP32 FMA chain
// with the weights rounded to float: at most 7 * 2^-24 * M from the reference's
// float of the same inputs (M = the largest input magnitude in the window; the
// weights sum to 1, so every partial sum is below M), and the errors of earlier
// passes carry through with total weight 1: after three passes at most
// 21 * 2^-24 * M < 2^-19 * M, M being any bound on the input magnitudes the
// voxel depends on.  A warp uses the largest magnitude it has read so far.
namespace {
constexpr int OW_Y = 8, OW_Z = 32;   // pass A warp task: 32 x 8 x 32 output voxels
constexpr float OW0 = 0.45f, OW1 = 0.225f, OW2 = 0.05f;

__device__ __forceinline__ float fma5(float a, float b, float c, float d, float e) {
    return __fmaf_rn(e, OW2, __fmaf_rn(d, OW1, __fmaf_rn(c, OW0, __fmaf_rn(b, OW1, __fmul_rn(a, OW2)))));
}

__device__ __forceinline__ void od_flag(OdStats *st, unsigned f) { atomicOr(&st->flags, f); }

// ---- TMA and mbarrier primitives (inline PTX) ----
__device__ __forceinline__ unsigned smem_u32(const void *p) { return (unsigned)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(unsigned long long *bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_fence_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
__device__ __forceinline__ void mbar_expect_tx(unsigned long long *bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(unsigned long long *bar, unsigned parity) {
    unsigned ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
__device__ __forceinline__ void tma_load_3d(void *dst, const CUtensorMap *map, unsigned long long *bar, int x, int y,
                                            int z) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];"
        ::"r"(smem_u32(dst)), "l"(map), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
        : "memory");
}
// order this thread's earlier generic-proxy accesses to shared memory before later TMA writes
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// Pass A: the input volume through a TMA tensor map (nx a multiple of 4, so
// that the rows are 16-byte aligned); boxes of 40 x 12 x 1 floats, x0 - 4 ..
// x0 + 35 and y0 - 2 .. y0 + 9 of one slice (outside the volume the copy fills
// zeros).  A warp takes 32 x 8 columns of 32 slices (lane = x): its lane 0
// keeps OA_S slices in flight in the warp's own ring of shared-memory stages,
// each completing on its mbarrier; the x pass reads the stage, the y pass runs
// over the 12 rows in registers, the z pass over a five-slice ring of the
// eight rows' y values.  Each output is classified on the spot:
// |v - iso| <= B + 4 eps -> listed as undecided, else v >= iso -> bbox.  At the
// end of its task the warp lists the outputs within 2.5 B of its minimum
// (maximum) with their value and B (range candidates) and offers min + B
// (max - B) as a bound on the volume's exact extreme.  Waits give up after a
// fixed number of polls (flag OD_TIMEOUT), after waiting, also bounded, for the
// warp's copies still in flight.
constexpr int OA_S = 4, OA_BW = 40, OA_BH = 12, OA_WARPS = 4;
constexpr unsigned OA_BYTES = OA_BW * OA_BH * 4;
constexpr int OA_POLLS = 1 << 22;
struct __align__(128) OaStage {
    float v[OA_BH][OA_BW];
};

__global__ void __launch_bounds__(OA_WARPS * 32) k_od_approx(const __grid_constant__ CUtensorMap tmap, float *out,
                                                             int nx, int ny, int nz, int z_lo, int z_hi, float iso,
                                                             OdStats *st, OdLists L) {
    const unsigned FULL = 0xffffffffu;
    __shared__ OaStage stage[OA_WARPS][OA_S];
    __shared__ unsigned long long bars[OA_WARPS][OA_S];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    OaStage *sg = stage[wid];
    unsigned long long *bw = bars[wid];
    if (lane == 0) {
        for (int k = 0; k < OA_S; k++) mbar_init(&bw[k], 1);
        mbar_fence_init();
    }
    __syncwarp();
    unsigned issued = 0, used = 0;   // loads issued / consumed by this warp (stage = n % OA_S, parity = n / OA_S)
    const unsigned nxs = (unsigned)(nx + 31) / 32, nys = (unsigned)(ny + OW_Y - 1) / OW_Y;
    const unsigned nzs = (unsigned)(z_hi - z_lo + OW_Z - 1) / OW_Z;
    const unsigned ntask = nxs * nys * nzs;
    const size_t nxy = (size_t)nx * ny;
    bool timed_out = false;
    for (unsigned task = blockIdx.x * OA_WARPS + wid; task < ntask && !timed_out; task += gridDim.x * OA_WARPS) {
        const unsigned xs = task % nxs, t2 = task / nxs;
        const int y0 = (int)(t2 % nys) * OW_Y, zs = z_lo + (int)(t2 / nys) * OW_Z, ze = min(zs + OW_Z, z_hi);
        const int x0 = (int)xs * 32, x = x0 + lane;
        const bool ownx = x < nx, xint = x >= 2 && x <= nx - 3;
        // every slice zs-2 .. ze+1 is loaded (outside the volume: zeros, read only by outputs that ignore them)
        int znext = zs - 2;
        const int zlast = ze + 1;
        auto issue = [&]() {
            if (lane == 0) {
                const unsigned k = issued % OA_S;
                fence_proxy_async();
                mbar_expect_tx(&bw[k], OA_BYTES);
                tma_load_3d(&sg[k], &tmap, &bw[k], x0 - 4, y0 - 2, znext);
            }
            issued++;
            znext++;
        };
        while (znext <= zlast && issued - used < (unsigned)OA_S) issue();
        float zr[5][OW_Y];   // y values of slices z-2 .. z+2 (slot 4 newest)
#pragma unroll
        for (int a = 0; a < 5; a++)
#pragma unroll
            for (int k = 0; k < OW_Y; k++) zr[a][k] = 0.f;
        float mrun = 0.f, lmin = INFINITY, lmax = -INFINITY, B = 0.f;
        float lmin2 = INFINITY, lmax2 = -INFINITY;   // second smallest / largest
        unsigned jmin = 0, jmax = 0;                 // where lmin / lmax are
        int bzl = INT_MAX, bzh = INT_MIN;
        unsigned ymask = 0;                          // rows with a decided voxel >= iso
        unsigned sgn = 0;                            // this slice's sign bits, bit kk = row y0 + kk
        float nanacc = 0.f;                          // becomes NaN if an output is NaN or infinite
        for (int zi = zs - 2; zi <= zlast; zi++) {
            const unsigned k = used % OA_S, par = (used / OA_S) & 1u;
            bool ok = false;
            for (int it = 0; it < OA_POLLS && !ok; it++) ok = mbar_try_wait(&bw[k], par);
            if (!__all_sync(FULL, ok)) {
                timed_out = true;
                break;
            }
#pragma unroll
            for (int a = 0; a < 4; a++)
#pragma unroll
                for (int kk = 0; kk < OW_Y; kk++) zr[a][kk] = zr[a + 1][kk];
            const OaStage &S = sg[k];
            float xv[OA_BH];
#pragma unroll
            for (int r = 0; r < OA_BH; r++) {
                const float *q = &S.v[r][lane + 2];   // x - 2 .. x + 2
                const float a = q[0], b = q[1], c = q[2], d = q[3], e = q[4];
                mrun = fmaxf(mrun, fmaxf(fabsf(a), fabsf(e)));   // lanes together cover x0-2 .. x0+33
                xv[r] = xint ? fma5(a, b, c, d, e) : c;
            }
#pragma unroll
            for (int kk = 0; kk < OW_Y; kk++) {
                const int yy = y0 + kk;
                zr[4][kk] = (yy >= 2 && yy <= ny - 3) ? fma5(xv[kk], xv[kk + 1], xv[kk + 2], xv[kk + 3], xv[kk + 4])
                                                      : xv[kk + 2];
            }
            __syncwarp();   // every lane is done with the stage
            used++;
            if (znext <= zlast) issue();
            float m = mrun;
            for (int o = 16; o; o >>= 1) m = fmaxf(m, __shfl_xor_sync(FULL, m, o));
            B = m * 0x1p-19f;   // bounds every output whose inputs have been read
            const int z = zi - 2;
            sgn = 0;
            if (z >= zs && z < ze && ownx) {
                const bool zint = z >= 2 && z <= nz - 3;
                const float band = B + 4.0f * N2M_FLT_EPS;
                const unsigned j0 = (unsigned)((size_t)z * nxy + (size_t)y0 * nx + x);
                unsigned ge = 0;
#pragma unroll
                for (int kk = 0; kk < OW_Y; kk++) {
                    if (y0 + kk >= ny) continue;
                    const float zv = zint ? fma5(zr[0][kk], zr[1][kk], zr[2][kk], zr[3][kk], zr[4][kk]) : zr[2][kk];
                    const unsigned j = j0 + (unsigned)kk * (unsigned)nx;
                    out[j] = zv;
                    nanacc = __fmaf_rn(zv, 0.f, nanacc);
                    const bool lo = zv < lmin, hi = zv > lmax;
                    lmin2 = lo ? lmin : fminf(lmin2, zv);
                    jmin = lo ? j : jmin;
                    lmin = fminf(lmin, zv);
                    lmax2 = hi ? lmax : fmaxf(lmax2, zv);
                    jmax = hi ? j : jmax;
                    lmax = fmaxf(lmax, zv);
                    const float dv = __fsub_rn(zv, iso);
                    sgn |= (unsigned)(dv > -N2M_FLT_EPS) << kk;   // provisional for undecided voxels
                    const bool und = fabsf(dv) <= band;
                    if (und) {
                        const unsigned q = atomicAdd(&L.cnt[0], 1u);
                        if (q < L.cap) L.unc[q] = j;
                    }
                    ge |= (unsigned)(!und && zv >= iso) << kk;
                }
                if (ge) {
                    ymask |= ge;
                    bzl = min(bzl, z);
                    bzh = z;
                }
            }
            if (z >= zs && z < ze) {   // warp-uniform: the tile's 8 row words, lanes 0-7, one sector
                unsigned mine = 0;
#pragma unroll
                for (int kk = 0; kk < OW_Y; kk++) {
                    const unsigned b = __ballot_sync(FULL, (sgn >> kk) & 1u);
                    mine = lane == kk ? b : mine;
                }
                if (lane < OW_Y) L.vsign[od_vsign_word((unsigned)x0, (unsigned)(y0 + lane), (unsigned)z, L.wv, L.nys)] = mine;
            }
        }
        if (timed_out) break;
        // huge, infinite or NaN input (an unbounded B), or a non-finite output
        const bool bad = !(B < 0x1p+120f * 0x1p-19f) || nanacc != 0.f;
        if (__any_sync(FULL, bad)) {   // the exact three-pass path handles the volume
            if (lane == 0) od_flag(st, OD_FALLBACK);
            continue;
        }
        // bbox of the decided voxels >= iso
        {
            const bool any = ymask != 0u;
            int byl = any ? y0 + __ffs(ymask) - 1 : INT_MAX, byh = any ? y0 + 31 - __clz(ymask) : INT_MIN;
            int xl = any ? x : INT_MAX, xh = any ? x : INT_MIN;
            for (int o = 16; o; o >>= 1) {
                xl = min(xl, __shfl_xor_sync(FULL, xl, o)); xh = max(xh, __shfl_xor_sync(FULL, xh, o));
                byl = min(byl, __shfl_xor_sync(FULL, byl, o)); byh = max(byh, __shfl_xor_sync(FULL, byh, o));
                bzl = min(bzl, __shfl_xor_sync(FULL, bzl, o)); bzh = max(bzh, __shfl_xor_sync(FULL, bzh, o));
            }
            if (lane == 0 && xl != INT_MAX) {
                atomicMin(&st->vs.lo[0], xl); atomicMax(&st->vs.hi[0], xh);
                atomicMin(&st->vs.lo[1], byl); atomicMax(&st->vs.hi[1], byh);
                atomicMin(&st->vs.lo[2], bzl); atomicMax(&st->vs.hi[2], bzh);
            }
        }
        // range candidates of this task
        float wmin = lmin, wmax = lmax;
        for (int o = 16; o; o >>= 1) {
            wmin = fminf(wmin, __shfl_xor_sync(FULL, wmin, o));
            wmax = fmaxf(wmax, __shfl_xor_sync(FULL, wmax, o));
        }
        if (lane == 0) {
            atomicMin(&st->umin, f2ord(__fadd_ru(wmin, B)));
            atomicMax(&st->lmax, f2ord(__fsub_rd(wmax, B)));
        }
        const float cmin = __fadd_ru(wmin, 2.5f * B), cmax = __fsub_rd(wmax, 2.5f * B);
        // a lane with one candidate lists it directly; with more (its second extreme is
        // close too: plateaus) it re-reads its outputs
        if (ownx && lmin <= cmin && lmin2 > cmin) {
            const unsigned q = atomicAdd(&L.cnt[1], 1u);
            if (q < L.cap) L.cmin[q] = OdCand{jmin, lmin, B};
        }
        if (ownx && lmax >= cmax && lmax2 < cmax) {
            const unsigned q = atomicAdd(&L.cnt[2], 1u);
            if (q < L.cap) L.cmax[q] = OdCand{jmax, lmax, B};
        }
        if (ownx && (lmin2 <= cmin || lmax2 >= cmax)) {
            const bool wmn = lmin2 <= cmin, wmx = lmax2 >= cmax;
            for (int z = zs; z < ze; z++) {
                float v[OW_Y];
#pragma unroll
                for (int kk = 0; kk < OW_Y; kk++)
                    v[kk] = y0 + kk < ny ? out[(size_t)z * nxy + (size_t)(y0 + kk) * nx + x] : 0.f;
#pragma unroll
                for (int kk = 0; kk < OW_Y; kk++) {
                    if (y0 + kk >= ny) continue;
                    const unsigned j = (unsigned)((size_t)z * nxy + (size_t)(y0 + kk) * nx + x);
                    if (wmn && v[kk] <= cmin) {
                        const unsigned q = atomicAdd(&L.cnt[1], 1u);
                        if (q < L.cap) L.cmin[q] = OdCand{j, v[kk], B};
                    }
                    if (wmx && v[kk] >= cmax) {
                        const unsigned q = atomicAdd(&L.cnt[2], 1u);
                        if (q < L.cap) L.cmax[q] = OdCand{j, v[kk], B};
                    }
                }
            }
        }
    }
    if (timed_out) {
        // no further copies are issued; wait (bounded) for the ones in flight before leaving
        if (lane == 0) od_flag(st, OD_FALLBACK | OD_TIMEOUT);
        while (used < issued) {
            const unsigned k = used % OA_S, par = (used / OA_S) & 1u;
            for (int it = 0; it < OA_POLLS; it++)
                if (mbar_try_wait(&bw[k], par)) break;
            used++;
        }
    }
}

// the reference's smoothed value of voxel (x, y, z), every tap in its double sequence
__device__ float od_exact_at(const float *__restrict__ in, int x, int y, int z, int nx, int ny, int nz) {
    const size_t nxy = (size_t)nx * ny;
    auto X = [&](int yy, int zz) -> float {
        const float *p = in + (size_t)zz * nxy + (size_t)yy * nx + x;
        return (x < 2 || x > nx - 3) ? p[0] : tap5_double(p[-2], p[-1], p[0], p[1], p[2]);
    };
    auto Y = [&](int zz) -> float {
        return (y < 2 || y > ny - 3) ? X(y, zz) : tap5_double(X(y - 2, zz), X(y - 1, zz), X(y, zz), X(y + 1, zz), X(y + 2, zz));
    };
    return (z < 2 || z > nz - 3) ? Y(z) : tap5_double(Y(z - 2), Y(z - 1), Y(z), Y(z + 1), Y(z + 2));
}

// Pass B: undecided voxels get their exact value (and join the bbox if >= iso);
// the range is the exact extreme over the candidates that can still reach it
// (value - B <= the smallest min + B of any task; the same for the maximum)
__global__ void k_od_resolve(const float *__restrict__ in, float *out, int nx, int ny, int nz, float iso, OdStats *st,
                             OdLists L, unsigned nu, unsigned nmin, unsigned nmax, bool at_or_above) {
    const unsigned n = nu + nmin + nmax;
    const float umin = ord2f(st->umin), lmax = ord2f(st->lmax);
    for (unsigned i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        unsigned j;
        int which;
        if (i < nu) {
            which = 0;
            j = L.unc[i];
        } else if (i < nu + nmin) {
            const OdCand c = L.cmin[i - nu];
            if (__fsub_rd(c.v, c.b) > umin) continue;
            which = 1;
            j = c.j;
        } else {
            const OdCand c = L.cmax[i - nu - nmin];
            if (__fadd_ru(c.v, c.b) < lmax) continue;
            which = 2;
            j = c.j;
        }
        const unsigned x = j % (unsigned)nx, r = j / (unsigned)nx, y = r % (unsigned)ny, z = r / (unsigned)ny;
        const float v = od_exact_at(in, (int)x, (int)y, (int)z, nx, ny, nz);
        if (which == 0) {
            out[j] = v;
            unsigned *sw = L.vsign + od_vsign_word(x, y, z, L.wv, L.nys);
            if (at_or_above ? v >= iso : __fsub_rn(v, iso) > -N2M_FLT_EPS) atomicOr(sw, 1u << (x & 31));
            else atomicAnd(sw, ~(1u << (x & 31)));
            if (v >= iso) {
                atomicMin(&st->vs.lo[0], (int)x); atomicMax(&st->vs.hi[0], (int)x);
                atomicMin(&st->vs.lo[1], (int)y); atomicMax(&st->vs.hi[1], (int)y);
                atomicMin(&st->vs.lo[2], (int)z); atomicMax(&st->vs.hi[2], (int)z);
            }
        } else if (which == 1) {
            atomicMin(&st->vs.vmin, f2ord(v));
        } else {
            atomicMax(&st->vs.vmax, f2ord(v));
        }
    }
}

// ---- marks -> the exact passes on marked voxels ----------------------------------
// Bitmaps are linear in the voxel index (bit j & 31 of word j >> 5).

// 32 bits of `bm` starting at bit `s` (a signed voxel offset), zero outside [0, nvox)
__device__ __forceinline__ unsigned bits_at(const unsigned *__restrict__ bm, long long s, long long nvox) {
    if (s <= -32 || s >= nvox) return 0u;
    const long long w = s >= 0 ? s >> 5 : -((31 - s) >> 5);
    const int sh = (int)(s - (w << 5));
    const long long nw = (nvox + 31) >> 5;
    const unsigned lo = (w >= 0 && w < nw) ? __ldg(bm + w) : 0u;
    const unsigned hi = (w + 1 >= 0 && w + 1 < nw) ? __ldg(bm + w + 1) : 0u;
    unsigned v = __funnelshift_r(lo, hi, sh);
    const long long end = nvox - s;   // bits at or past nvox are zero
    if (end < 32) v &= (1u << end) - 1u;
    if (s < 0) v &= ~0u << (unsigned)(-s);
    return v;
}

// dst = OR over d in [-2, 2] of src shifted by d * stride voxels; per word the
// number of set bits of dst into cnt[w].{y|z} (and of src into cnt[w].x)
template <int FIELD>
__global__ void k_od_dilate(const unsigned *__restrict__ src, unsigned *dst, long long nvox, long long stride,
                            uint4 *cnt) {
    const long long nw = (nvox + 31) >> 5;
    const bool aligned = (stride & 31) == 0 && (nvox & 31) == 0;   // whole-word shifts (e.g. rows of 512)
    const long long sw = stride >> 5;
    for (long long w = (long long)blockIdx.x * blockDim.x + threadIdx.x; w < nw; w += (long long)gridDim.x * blockDim.x) {
        unsigned acc = 0;
        if (aligned) {
#pragma unroll
            for (int d = -2; d <= 2; d++) {
                const long long ws = w + d * sw;
                if (ws >= 0 && ws < nw) acc |= __ldg(src + ws);
            }
        } else {
#pragma unroll
            for (int d = -2; d <= 2; d++) acc |= bits_at(src, (w << 5) + d * stride, nvox);
        }
        dst[w] = acc;
        if (FIELD == 1) {
            cnt[w] = make_uint4((unsigned)__popc(src[w]), (unsigned)__popc(acc), 0u, 0u);
        } else {
            cnt[w].z = (unsigned)__popc(acc);
        }
    }
}

// the set bits of the three bitmaps as voxel indices, in order, at the scanned
// word offsets (x: z marks, y: y marks, z: x marks); a warp takes 32 words and
// writes each word's indices with one coalesced store per lane
__device__ __forceinline__ void scatter_word(unsigned m, unsigned o, unsigned base, unsigned *list, int lane) {
    if (m >> lane & 1u) list[o + __popc(m & ((1u << lane) - 1u))] = base + (unsigned)lane;
}
__global__ void k_od_scatter(const unsigned *__restrict__ bz, const unsigned *__restrict__ by,
                             const unsigned *__restrict__ bx, const uint4 *__restrict__ off, long long nw,
                             unsigned *lz, unsigned *ly, unsigned *lx) {
    const int lane = threadIdx.x & 31;
    const long long nwarps = (long long)gridDim.x * (blockDim.x >> 5);
    for (long long w0 = ((long long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5)) * 32; w0 < nw; w0 += nwarps * 32) {
        const long long wl = w0 + lane;
        const unsigned mz = wl < nw ? bz[wl] : 0u, my = wl < nw ? by[wl] : 0u, mx = wl < nw ? bx[wl] : 0u;
        const uint4 o = wl < nw ? off[wl] : make_uint4(0u, 0u, 0u, 0u);
        unsigned busy = __ballot_sync(0xffffffffu, (mz | my | mx) != 0u);
        while (busy) {
            const int k = __ffs(busy) - 1;
            busy &= busy - 1u;
            const unsigned base = (unsigned)((w0 + k) << 5);
            scatter_word(__shfl_sync(0xffffffffu, mz, k), __shfl_sync(0xffffffffu, o.x, k), base, lz, lane);
            scatter_word(__shfl_sync(0xffffffffu, my, k), __shfl_sync(0xffffffffu, o.y, k), base, ly, lane);
            scatter_word(__shfl_sync(0xffffffffu, mx, k), __shfl_sync(0xffffffffu, o.z, k), base, lx, lane);
        }
    }
}

// one exact pass on the listed voxels: dst[v] = tap sum of src along the axis
// (stride 1, nx or nx*ny; coordinate along the axis = (v / div) % len), or
// src[v] on the two face layers; one thread per voxel, OE_U list entries per
// thread in flight at once (a warp takes OE_U runs of 32 consecutive entries),
// undecided taps queued per warp for the FP64 fix-up
constexpr int OE_U = 4;
__global__ void __launch_bounds__(256) k_od_exact(const unsigned *__restrict__ list, const unsigned *__restrict__ cnt,
                                                  const float *__restrict__ src, float *dst, unsigned stride,
                                                  unsigned div, unsigned len, unsigned long long mdiv,
                                                  unsigned long long mlen) {
    __shared__ unsigned stage_buf[8][32 * (OE_U + 1)];   // < 32 between drains, + 32 per entry
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    FixStage<false> F{stage_buf[wid], 0};
    Acc acc;   // unused
    const Pass P{src, dst, stride, 0, 0, 0u, 0.f, nullptr};
    const unsigned n = *cnt;
    const unsigned nwarps = gridDim.x * (blockDim.x >> 5), gw = blockIdx.x * (blockDim.x >> 5) + (unsigned)wid;
    for (unsigned i0 = gw * 32u * OE_U; i0 < n; i0 += nwarps * 32u * OE_U) {   // warp-uniform
        unsigned v[OE_U];
        bool act[OE_U], inner[OE_U];
        float a[OE_U][5];
#pragma unroll
        for (int u = 0; u < OE_U; u++) {
            const unsigned i = i0 + (unsigned)u * 32u + (unsigned)lane;
            act[u] = i < n;
            v[u] = act[u] ? __ldg(list + i) : 0u;
        }
#pragma unroll
        for (int u = 0; u < OE_U; u++) {
            const unsigned q = div == 1u ? v[u] : (unsigned)__umul64hi(v[u], mdiv);   // v / div
            const unsigned c = q - (unsigned)__umul64hi(q, mlen) * len;               // q % len
            inner[u] = act[u] && c >= 2u && c + 2u < len;
            const float *p = src + v[u];
            if (inner[u]) {
                a[u][0] = __ldg(p - 2 * (size_t)stride);
                a[u][1] = __ldg(p - (size_t)stride);
                a[u][3] = __ldg(p + stride);
                a[u][4] = __ldg(p + 2 * (size_t)stride);
            }
            a[u][2] = act[u] ? __ldg(p) : 0.f;
        }
#pragma unroll
        for (int u = 0; u < OE_U; u++) {
            bool fail = false;
            if (act[u]) {
                float r = a[u][2];
                if (inner[u] && !tap5_split_window(a[u][0], a[u][1], a[u][2], a[u][3], a[u][4], &r))
                    fail = !tap5_fast(a[u][0], a[u][1], a[u][2], a[u][3], a[u][4], &r);
                if (!fail) dst[v[u]] = r;
            }
            F.push(fail, v[u], lane);
        }
        F.drain(P, acc, lane);
    }
    F.finish(P, acc, lane);
}

// The labelling's effect on the exact values the z pass just wrote at the
// listed voxels (src/meshify.c:330-342): kept voxels raised to iso (fill);
// with largest, voxels neither kept nor in the kept set's dilation (the
// 26-neighbourhood without (-1,-1,-1), interior voxels; src/meshify.c:218-264)
// are the minimum.
__global__ void k_od_post(const unsigned *__restrict__ list, const unsigned *__restrict__ cnt, float *out, LabelPost L,
                          int nx, int ny, int nz) {
    const unsigned n = *cnt;
    auto bit = [&](int x, int y, int z) -> unsigned {
        return (__ldg(L.K + ((size_t)z * ny + y) * L.W + ((unsigned)x >> 5)) >> (x & 31)) & 1u;
    };
    for (unsigned i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const unsigned j = list[i], x = j % (unsigned)nx, r = j / (unsigned)nx, y = r % (unsigned)ny, z = r / (unsigned)ny;
        if (bit(x, y, z)) {
            if (L.fill) out[j] = fmaxf(out[j], L.iso);
            continue;
        }
        if (!L.largest) continue;
        bool on = false;
        if (x > 0 && y > 0 && z > 0 && x + 1 < (unsigned)nx && y + 1 < (unsigned)ny && z + 1 < (unsigned)nz) {
            for (int dz = -1; dz <= 1 && !on; dz++)
                for (int dy = -1; dy <= 1 && !on; dy++)
                    for (int dx = -1; dx <= 1 && !on; dx++)
                        if (!(dx == -1 && dy == -1 && dz == -1)) on = bit((int)x + dx, (int)y + dy, (int)z + dz);
        }
        if (!on) out[j] = L.mn;
    }
}

// floor(2^64 / d) + 1: __umul64hi(n, m) = n / d for every 32-bit n (d >= 2)
unsigned long long od_magic(unsigned d) { return d <= 1u ? 0ull : ~0ull / d + 1ull; }

int od_grid(const void *fn, int threads) {
    int dev = 0, sms = 0, per_sm = 0, g = 0;
    if (cudaGetDevice(&dev) == cudaSuccess && cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) == cudaSuccess &&
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, threads, 0) == cudaSuccess)
        g = sms * std::max(per_sm, 1);
    cudaGetLastError();
    return g > 0 ? g : 152 * 4;
}

PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
    static std::once_flag once;
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    std::call_once(once, [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = (PFN_cuTensorMapEncodeTiled_v12000)p;
        cudaGetLastError();
    });
    return fn;
}
}  // namespace

bool od_eligible(const float *in, int nx, int ny, int nz) {
    return nx % 4 == 0 && ((uintptr_t)in & 15u) == 0 && (size_t)nx * ny * nz < ((size_t)1 << 32) && nx >= 5 &&
           ny >= 5 && nz >= 5;
}

n2m_status od_approx(const float *in, float *out, int nx, int ny, int nz, float iso, OdWork &w, cudaStream_t s,
                     const StagedInput *stage) {
    const size_t n = (size_t)nx * ny * nz;
    auto encode = tensor_map_encoder();
    if (!encode) {
        n2m_set_error("cuTensorMapEncodeTiled is not available from the driver");
        return N2M_ERR_CUDA;
    }
    CUtensorMap tmap;
    {
        const cuuint64_t gdim[3] = {(cuuint64_t)nx, (cuuint64_t)ny, (cuuint64_t)nz};
        const cuuint64_t gstride[2] = {(cuuint64_t)nx * 4u, (cuuint64_t)nx * ny * 4u};
        const cuuint32_t box[3] = {OA_BW, OA_BH, 1}, estr[3] = {1, 1, 1};
        const CUresult r = encode(&tmap, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, (void *)in, gdim, gstride, box, estr,
                                  CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                                  CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
        if (r != CUDA_SUCCESS) {
            n2m_set_error("cuTensorMapEncodeTiled failed (%d)", (int)r);
            return N2M_ERR_CUDA;
        }
    }
    w.cap = (unsigned)std::min<size_t>(n / 64 + 4096, 1u << 22);
    CKS(w.st.ensure(sizeof(OdStats)));
    CKS(w.unc.ensure((size_t)w.cap * sizeof(unsigned)));
    CKS(w.cmin.ensure((size_t)w.cap * sizeof(OdCand)));
    CKS(w.cmax.ensure((size_t)w.cap * sizeof(OdCand)));
    OdStats h{};
    stats_init_host(&h.vs);
    h.vs.vmin = INT_MAX;   // filled by pass B from the candidates
    h.vs.vmax = INT_MIN;
    h.umin = INT_MAX;
    h.lmax = INT_MIN;
    CK(cudaMemcpyAsync(w.st.p, &h, sizeof(OdStats), cudaMemcpyHostToDevice, s));
    const unsigned wv = (unsigned)(nx + 31) / 32, nys = (unsigned)(ny + 7) / 8;
    CKS(w.vsign.ensure((size_t)nz * nys * wv * 8 * sizeof(unsigned)));
    OdStats *st = w.st.as<OdStats>();
    OdLists L{w.unc.as<unsigned>(), w.cmin.as<OdCand>(), w.cmax.as<OdCand>(),
              (unsigned *)((char *)w.st.p + offsetof(OdStats, cnt)), w.cap, w.vsign.as<unsigned>(), wv, nys};
    const int grid = od_grid((const void *)k_od_approx, OA_WARPS * 32);
    auto launch = [&](int z_lo, int z_hi) -> n2m_status {
        if (z_hi <= z_lo) return N2M_OK;
        k_od_approx<<<grid, OA_WARPS * 32, 0, s>>>(tmap, out, nx, ny, nz, z_lo, z_hi, iso, st, L);
        N2M_COUNT();
        CKL();
        return N2M_OK;
    };
    if (stage && stage->host) {
        // the copy stream may only overwrite `in` once earlier work on s is done with it
        CK(cudaEventRecord(stage->ev[N2M_STAGE_SLABS], s));
        CK(cudaStreamWaitEvent(stage->copy, stage->ev[N2M_STAGE_SLABS], 0));
        const size_t nxy = (size_t)nx * ny;
        int zdone = 0;
        for (int k = 0; k < N2M_STAGE_SLABS; k++) {
            const int z0 = (int)((long long)nz * k / N2M_STAGE_SLABS), z1 = (int)((long long)nz * (k + 1) / N2M_STAGE_SLABS);
            if (z1 <= z0) continue;
            CK(cudaMemcpyAsync((float *)in + (size_t)z0 * nxy, stage->host + (size_t)z0 * nxy,
                               (size_t)(z1 - z0) * nxy * sizeof(float), cudaMemcpyHostToDevice, stage->copy));
            CK(cudaEventRecord(stage->ev[k], stage->copy));
            CK(cudaStreamWaitEvent(s, stage->ev[k], 0));
            const int zready = z1 == nz ? nz : z1 - 2;   // outputs whose input slices (+-2) have arrived
            if (zready - zdone >= 32 || zready == nz) {
                CKS(launch(zdone, zready));
                zdone = zready;
            }
        }
    } else {
        CKS(launch(0, nz));
    }
    return N2M_OK;
}

n2m_status od_resolve(const float *in, float *out, int nx, int ny, int nz, float iso, OdWork &w, VolStats *dst,
                      cudaStream_t s, bool *fallback, bool at_or_above) {
    OdStats h;
    CK(cudaMemcpyAsync(&h, w.st.p, sizeof(OdStats), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    if (h.flags & OD_TIMEOUT) {
        n2m_set_error("pre-smooth: a tile copy did not complete");
        return N2M_ERR_TIMEOUT;
    }
    *fallback = (h.flags & OD_FALLBACK) != 0 || h.cnt[0] > w.cap || h.cnt[1] > w.cap || h.cnt[2] > w.cap ||
                h.cnt[1] == 0 || h.cnt[2] == 0;
    if (*fallback) return N2M_OK;
    OdLists L{w.unc.as<unsigned>(), w.cmin.as<OdCand>(), w.cmax.as<OdCand>(),
              (unsigned *)((char *)w.st.p + offsetof(OdStats, cnt)), w.cap, w.vsign.as<unsigned>(),
              (unsigned)(nx + 31) / 32, (unsigned)(ny + 7) / 8};
    const unsigned tot = h.cnt[0] + h.cnt[1] + h.cnt[2];
    const unsigned blocks = std::max(1u, std::min((tot + 127) / 128, 152u * 8u));
    k_od_resolve<<<blocks, 128, 0, s>>>(in, out, nx, ny, nz, iso, w.st.as<OdStats>(), L, h.cnt[0], h.cnt[1], h.cnt[2],
                                        at_or_above);
    N2M_COUNT();
    CKL();
    CK(cudaMemcpyAsync(dst, w.st.p, sizeof(VolStats), cudaMemcpyDeviceToDevice, s));   // vs is the first member
    return N2M_OK;
}

n2m_status od_repair(const OdRepair &r, cudaStream_t s) {
    OdWork &w = *r.w;
    const int nx = r.dim[0], ny = r.dim[1], nz = r.dim[2];
    const long long nvox = (long long)nx * ny * nz, nw = (nvox + 31) >> 5;
    CKS(w.need_y.ensure((size_t)nw * sizeof(unsigned)));
    CKS(w.need_x.ensure((size_t)nw * sizeof(unsigned)));
    CKS(w.off.ensure((size_t)nw * sizeof(uint4)));
    CKS(w.list.ensure((size_t)3 * nvox * sizeof(unsigned)));   // every list fits any marking
    CKS(w.lcnt.ensure(sizeof(uint4)));
    uint4 *off = w.off.as<uint4>();
    unsigned *cnt = w.lcnt.as<unsigned>();   // z, y, x counts
    unsigned *lz = w.list.as<unsigned>(), *ly = lz + nvox, *lx = ly + nvox;
    const unsigned dblocks = (unsigned)std::min<long long>((nw + 255) / 256, 152 * 16);
    // y values needed by marked z outputs (+-2 slices), x values by those (+-2 rows)
    { k_od_dilate<1><<<dblocks, 256, 0, s>>>(w.need_z.as<unsigned>(), w.need_y.as<unsigned>(), nvox, (long long)nx * ny,
                                             off); N2M_COUNT(); }
    { k_od_dilate<2><<<dblocks, 256, 0, s>>>(w.need_y.as<unsigned>(), w.need_x.as<unsigned>(), nvox, (long long)nx,
                                             off); N2M_COUNT(); }
    CKL();
    CKS(scan_uint4(off, (size_t)nw, (uint4 *)cnt, *r.scan, s));
    { const unsigned sblocks = (unsigned)std::min<long long>((nw + 255) / 256, 152 * 16);
      k_od_scatter<<<sblocks, 256, 0, s>>>(w.need_z.as<unsigned>(), w.need_y.as<unsigned>(), w.need_x.as<unsigned>(), off,
                                           nw, lz, ly, lx); N2M_COUNT(); }
    CKL();
    const int xb = od_grid((const void *)k_od_exact, 256);
    const unsigned uxy = (unsigned)nx * (unsigned)ny;
    { k_od_exact<<<xb, 256, 0, s>>>(lx, cnt + 2, r.in, r.tmp1, 1u, 1u, (unsigned)nx, 0ull, od_magic((unsigned)nx)); N2M_COUNT(); }
    { k_od_exact<<<xb, 256, 0, s>>>(ly, cnt + 1, r.tmp1, r.tmp2, (unsigned)nx, (unsigned)nx, (unsigned)ny,
                                    od_magic((unsigned)nx), od_magic((unsigned)ny)); N2M_COUNT(); }
    { k_od_exact<<<xb, 256, 0, s>>>(lz, cnt + 0, r.tmp2, r.out, uxy, uxy, (unsigned)nz, od_magic(uxy),
                                    od_magic((unsigned)nz)); N2M_COUNT(); }
    if (r.post) { k_od_post<<<xb, 256, 0, s>>>(lz, cnt + 0, r.out, *r.post, nx, ny, nz); N2M_COUNT(); }
    CKL();
    return N2M_OK;
}
