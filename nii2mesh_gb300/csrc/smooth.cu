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

#include <stdlib.h>

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
    h->pad = 0;
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
