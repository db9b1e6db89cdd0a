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

#include "smooth_core.cuh"

namespace {
using namespace smooth;

struct VolSrc {
    const float *in;
    int nx;
    size_t nxy;
    __device__ __forceinline__ float load(int x, int y, int z) const {
        return __ldg(in + (size_t)z * nxy + (size_t)y * nx + x);
    }
};
struct VolSink {
    float *out;
    int nx;
    size_t nxy;
    __device__ __forceinline__ void put(int x, int y, int z, float v) { out[(size_t)z * nxy + (size_t)y * nx + x] = v; }
};

__global__ void __launch_bounds__(NT, 2) k_smooth(const float *__restrict__ in, float *__restrict__ out, int nx,
                                                  int ny, int nz, float iso, VolStats *st) {
    const size_t nxy = (size_t)nx * ny;
    VolSrc src{in, nx, nxy};
    VolSink sink{out, nx, nxy};
    Acc acc;
    acc.init();
    const int z0 = blockIdx.z * SZC;
    column(src, sink, acc, iso, blockIdx.x * STX, blockIdx.y * STY, z0, min(z0 + SZC, nz), nx, ny, nx, ny, nz);
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
