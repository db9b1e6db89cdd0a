// scan.cu — device-wide exclusive prefix sum of uint4 vectors (component-wise),
// in place.  Reduce-then-scan: per-tile sums, a single-CTA scan of the tile
// sums (looping for any count), then a per-tile scan that adds its offset.
// Used to number marching-cubes vertices/triangles and to compact meshes.
#include "n2m_internal.cuh"

namespace {
constexpr int SB = 256;          // threads per CTA
constexpr int SI = 8;            // items per thread
constexpr int TILE = SB * SI;    // items per tile

__device__ __forceinline__ uint4 add4(uint4 a, uint4 b) { return make_uint4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w); }

// block-wide exclusive scan of one uint4 per thread; returns the block total
__device__ uint4 block_exscan(uint4 &v) {
    __shared__ uint4 wsum[SB / 32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    uint4 incl = v;
    for (int o = 1; o < 32; o <<= 1) {
        uint4 t;
        t.x = __shfl_up_sync(0xffffffffu, incl.x, o); t.y = __shfl_up_sync(0xffffffffu, incl.y, o);
        t.z = __shfl_up_sync(0xffffffffu, incl.z, o); t.w = __shfl_up_sync(0xffffffffu, incl.w, o);
        if (lane >= o) incl = add4(incl, t);
    }
    if (lane == 31) wsum[wid] = incl;
    __syncthreads();
    if (wid == 0) {
        uint4 s = lane < SB / 32 ? wsum[lane] : make_uint4(0, 0, 0, 0);
        uint4 si = s;
        for (int o = 1; o < 32; o <<= 1) {
            uint4 t;
            t.x = __shfl_up_sync(0xffffffffu, si.x, o); t.y = __shfl_up_sync(0xffffffffu, si.y, o);
            t.z = __shfl_up_sync(0xffffffffu, si.z, o); t.w = __shfl_up_sync(0xffffffffu, si.w, o);
            if (lane >= o) si = add4(si, t);
        }
        if (lane < SB / 32) wsum[lane] = make_uint4(si.x - s.x, si.y - s.y, si.z - s.z, si.w - s.w);
    }
    __syncthreads();
    const uint4 woff = wsum[wid];
    uint4 total;
    // total = exclusive offset of the last warp + its inclusive sum
    __shared__ uint4 tot;
    if (threadIdx.x == SB - 1) tot = add4(woff, incl);
    const uint4 ex = make_uint4(incl.x - v.x, incl.y - v.y, incl.z - v.z, incl.w - v.w);
    v = add4(woff, ex);
    __syncthreads();
    total = tot;
    __syncthreads();
    return total;
}

__global__ void __launch_bounds__(SB) k_tile_sums(const uint4 *__restrict__ d, size_t n, uint4 *part) {
    const size_t base = (size_t)blockIdx.x * TILE;
    uint4 s = make_uint4(0, 0, 0, 0);
    for (int i = 0; i < SI; i++) {
        const size_t k = base + (size_t)i * SB + threadIdx.x;
        if (k < n) s = add4(s, d[k]);
    }
    uint4 t = block_exscan(s);
    if (threadIdx.x == 0) part[blockIdx.x] = t;
}

__global__ void __launch_bounds__(SB) k_scan_parts(uint4 *part, size_t np, uint4 *total) {
    uint4 carry = make_uint4(0, 0, 0, 0);
    for (size_t base = 0; base < np; base += SB) {
        const size_t k = base + threadIdx.x;
        uint4 v = k < np ? part[k] : make_uint4(0, 0, 0, 0);
        uint4 t = block_exscan(v);
        if (k < np) part[k] = add4(v, carry);
        carry = add4(carry, t);
    }
    if (threadIdx.x == 0) *total = carry;
}

__global__ void __launch_bounds__(SB) k_tile_scan(uint4 *d, size_t n, const uint4 *part) {
    // each thread owns SI consecutive items of the tile
    const size_t base = (size_t)blockIdx.x * TILE + (size_t)threadIdx.x * SI;
    uint4 it[SI];
    uint4 s = make_uint4(0, 0, 0, 0);
    for (int i = 0; i < SI; i++) {
        it[i] = base + i < n ? d[base + i] : make_uint4(0, 0, 0, 0);
        s = add4(s, it[i]);
    }
    block_exscan(s);
    uint4 run = add4(s, part[blockIdx.x]);
    for (int i = 0; i < SI; i++) {
        if (base + i < n) d[base + i] = run;
        run = add4(run, it[i]);
    }
}
}  // namespace

n2m_status scan_uint4(uint4 *d, size_t n, uint4 *d_total, ScanWork &w, cudaStream_t s) {
    if (n == 0) {
        CK(cudaMemsetAsync(d_total, 0, sizeof(uint4), s));
        return N2M_OK;
    }
    const size_t tiles = (n + TILE - 1) / TILE;
    CKS(w.part.ensure(tiles * sizeof(uint4)));
    { k_tile_sums<<<(unsigned)tiles, SB, 0, s>>>(d, n, w.part.as<uint4>()); N2M_COUNT(); }
    { k_scan_parts<<<1, SB, 0, s>>>(w.part.as<uint4>(), tiles, d_total); N2M_COUNT(); }
    { k_tile_scan<<<(unsigned)tiles, SB, 0, s>>>(d, n, w.part.as<uint4>()); N2M_COUNT(); }
    CKL();
    return N2M_OK;
}

// ---- uint32 variant (same three-kernel scheme) ------------------------------
namespace {
__device__ unsigned block_exscan_u32(unsigned &v) {
    __shared__ unsigned wsum[SB / 32];
    __shared__ unsigned tot;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    unsigned incl = v;
    for (int o = 1; o < 32; o <<= 1) {
        const unsigned t = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += t;
    }
    if (lane == 31) wsum[wid] = incl;
    __syncthreads();
    if (wid == 0) {
        const unsigned s = lane < SB / 32 ? wsum[lane] : 0u;
        unsigned si = s;
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned t = __shfl_up_sync(0xffffffffu, si, o);
            if (lane >= o) si += t;
        }
        if (lane < SB / 32) wsum[lane] = si - s;
    }
    __syncthreads();
    const unsigned woff = wsum[wid];
    if (threadIdx.x == SB - 1) tot = woff + incl;
    v = woff + incl - v;
    __syncthreads();
    const unsigned total = tot;
    __syncthreads();
    return total;
}

__global__ void __launch_bounds__(SB) k_tile_sums_u32(const unsigned *__restrict__ d, size_t n, unsigned *part) {
    const size_t base = (size_t)blockIdx.x * TILE;
    unsigned s = 0;
    for (int i = 0; i < SI; i++) {
        const size_t k = base + (size_t)i * SB + threadIdx.x;
        if (k < n) s += d[k];
    }
    const unsigned t = block_exscan_u32(s);
    if (threadIdx.x == 0) part[blockIdx.x] = t;
}

__global__ void __launch_bounds__(SB) k_scan_parts_u32(unsigned *part, size_t np, unsigned *total) {
    unsigned carry = 0;
    for (size_t base = 0; base < np; base += SB) {
        const size_t k = base + threadIdx.x;
        unsigned v = k < np ? part[k] : 0u;
        const unsigned t = block_exscan_u32(v);
        if (k < np) part[k] = v + carry;
        carry += t;
    }
    if (threadIdx.x == 0) *total = carry;
}

__global__ void __launch_bounds__(SB) k_tile_scan_u32(unsigned *d, size_t n, const unsigned *part) {
    const size_t base = (size_t)blockIdx.x * TILE + (size_t)threadIdx.x * SI;
    unsigned it[SI], s = 0;
    for (int i = 0; i < SI; i++) {
        it[i] = base + i < n ? d[base + i] : 0u;
        s += it[i];
    }
    block_exscan_u32(s);
    unsigned run = s + part[blockIdx.x];
    for (int i = 0; i < SI; i++) {
        if (base + i < n) d[base + i] = run;
        run += it[i];
    }
}
}  // namespace

n2m_status scan_u32(unsigned *d, size_t n, unsigned *d_total, ScanWork &w, cudaStream_t s) {
    if (n == 0) {
        CK(cudaMemsetAsync(d_total, 0, sizeof(unsigned), s));
        return N2M_OK;
    }
    const size_t tiles = (n + TILE - 1) / TILE;
    CKS(w.part.ensure(tiles * sizeof(unsigned)));
    { k_tile_sums_u32<<<(unsigned)tiles, SB, 0, s>>>(d, n, w.part.as<unsigned>()); N2M_COUNT(); }
    { k_scan_parts_u32<<<1, SB, 0, s>>>(w.part.as<unsigned>(), tiles, d_total); N2M_COUNT(); }
    { k_tile_scan_u32<<<(unsigned)tiles, SB, 0, s>>>(d, n, w.part.as<unsigned>()); N2M_COUNT(); }
    CKL();
    return N2M_OK;
}
