// mc.cu — Lewiner MC33 marching cubes (src/MarchingCubes.c:116-1143) as two
// passes over the padded bounding-box grid, plus the classic case table of
// the same framework (-o 1).
//
// Numbering is the reference's: the edge vertices of grid point p (its +x,
// +y, +z edges, in that order) come after those of every point before p in
// raster order; c-vertices follow all edge vertices in cube raster order;
// triangles are in cube raster order, tiling order within a cube.  So the
// mesh is the reference's mesh before its weld, vertex for vertex.
//
// count pass: the sign bit of every grid point, packed in 32-point "words"
//   (ballots); then one thread per word derives its three edge-crossing masks
//   and the triangle and c-vertex counts of its 32 cubes with bit operations
//   and the MC33 decision of the few cubes that cross the surface.
// scan: exclusive scan over words -> vertex/triangle/c-vertex offsets.
// emit pass: a warp takes 32 active words (words that own output) at a time
//   and works through their edge vertices and triangles densely; an edge
//   vertex id anywhere in the grid is offset(word) + popcounts of the word's
//   masks below the point, so every edge is emitted exactly once (this
//   replaces the reference's vertex weld for shared edges).
// Vertices whose final coordinates sit within 1.5e-5 of a grid point (edge
// vertices) or of a grid plane (c-vertices) are recorded as weld candidates:
// only such vertices can lie within the weld tolerance (1e-5) of another.
#include <float.h>

#include <algorithm>
#include <atomic>

#include "mc33.cuh"

namespace {
using namespace mc33;
struct GV {  // device view of the padded grid
    const float *vol;
    int dx, dy, dz;
    long long nvox, dxy;
    int lo0, lo1, lo2, NX, NY, NZ;
    unsigned NXY, NG;
    float iso, edge_max, pad;
};

// value of grid point (x,y,z) minus isolevel, as marchingCubes() builds it
// (src/MarchingCubes.c:1097-1115, incl. the row wrap past x = dim0-1), with
// meshify's edge darkening (src/meshify.c:348-369) applied on the fly and
// run()'s FLT_EPSILON clamp (src/MarchingCubes.c:131-132).
__device__ __forceinline__ float gval(const GV &g, int x, int y, int z) {
    const long long j = (long long)(g.lo0 + x) + (long long)(y + g.lo1) * g.dx + (long long)(z + g.lo2) * g.dxy;
    float v;
    if (j < g.nvox) {
        v = __ldg(g.vol + j);
        // the voxel j really is: the grid ends at dim, so a coordinate is past the volume by at most
        // one (the padding column / row), which wraps into the next row / slice
        int vx = g.lo0 + x, vy = y + g.lo1, vz = z + g.lo2;
        if (vx >= g.dx) {
            vx -= g.dx;
            vy++;
        }
        if (vy >= g.dy) {
            vy -= g.dy;
            vz++;
        }
        if (vx == 0 || vy == 0 || vz == 0 || vx == g.dx - 1 || vy == g.dy - 1 || vz == g.dz - 1)
            v = fminf(g.edge_max, v);
        v = __fsub_rn(v, g.iso);
    } else {
        v = g.pad;
    }
    if (fabsf(v) < N2M_FLT_EPS) v = N2M_FLT_EPS;
    return v;
}

// ---- count pass ---------------------------------------------------------------
// Words are row-aligned: word (z*NY + y)*WX + xw holds grid points
// x = 32*xw + lane of row (y, z); WX = ceil(NX/32).  Word order is raster
// order, so numbering by an exclusive scan over words is the reference's.

// Triangle count of each cube configuration whose MC33 tiling needs no face
// or interior test (Lewiner cases 0, 1, 2, 5, 8, 9, 11, 14; every
// configuration of the classic table); 0x80 marks the ambiguous ones.
__device__ __forceinline__ unsigned char quick_count(int lut, bool classic) {
    if (classic) {
        const int off = O2(CASESCLASSIC, lut);
        int n = 0;
        while (n < 5 && d_lut[off + 3 * n] != -1) n++;
        return (unsigned char)n;
    }
    switch (L2(CASES, lut, 0)) {
    case 0: return 0;
    case 1: return 1;
    case 2: case 8: return 2;
    case 5: return 3;
    case 9: case 11: case 14: return 4;
    default: return 0x80;
    }
}

// triangles | c-vertices << 16 of a cube whose tiling needs face/interior tests
__device__ __noinline__ unsigned ambiguous_count(const GV &g, int x, int y, int z, int lut, bool classic) {
    const float c[8] = {gval(g, x, y, z),         gval(g, x + 1, y, z),         gval(g, x + 1, y + 1, z),
                        gval(g, x, y + 1, z),     gval(g, x, y, z + 1),         gval(g, x + 1, y, z + 1),
                        gval(g, x + 1, y + 1, z + 1), gval(g, x, y + 1, z + 1)};
    const Tiling T = select_tiling(c, lut, classic);
    return (unsigned)T.n | (T.cv ? 1u << 16 : 0u);
}

// Count pass, part 1: the sign (grid value > 0) of every grid point as one
// bit, word-aligned like the counts (bit x&31 of signs[(z*NY + y)*WX + x/32]).
// A warp takes whole rows, SW words at a time with all their loads in
// flight.  Runs of SW words strictly inside the volume and the grid read the
// volume directly.  Border words (the first and last of a row, every word of a
// row on a face) apply gval's cases lane by lane on the linear voxel index
// j = row start + x: the padding column (x one past the volume) is the next
// row's first voxel, which is on a face; a row on a face of the volume (or the
// padding row, which wraps to y = 0 of the next slice) has every point
// darkened; j past the volume is the padding value.
constexpr int SW = 16;

__device__ __forceinline__ unsigned border_word(const GV &g, long long rb, bool rface, int xw, int lane) {
    const int x = xw * 32 + lane, vx = g.lo0 + x;
    float d = g.pad;
    if (x < g.NX && rb + x < g.nvox) {
        const float v = __ldg(g.vol + rb + x);
        d = __fsub_rn((rface || vx == 0 || vx >= g.dx - 1) ? fminf(g.edge_max, v) : v, g.iso);
    }
    // the FLT_EPSILON clamp maps (-eps, eps) to +eps: positive <=> d > -eps
    return __ballot_sync(0xffffffffu, x < g.NX && d > -N2M_FLT_EPS);
}

// vsign (may be null): the volume's sign bitmap (OdWork::vsign, wv words per row,
// nys groups of 8 rows); a direct word is then two bitmap words shifted into place
__global__ void __launch_bounds__(256) k_signs(GV g, unsigned WX, unsigned nrows, unsigned *signs,
                                               const unsigned *__restrict__ vsign, unsigned wv, unsigned nys) {
    const int lane = threadIdx.x & 31;
    // words xw whose 32 points lie strictly inside the volume in x and inside the grid
    const int xs0 = max(0, (1 - g.lo0 + 31) / 32);
    const int xs1 = min((g.dx - 2 - g.lo0 - 31) >= 0 ? (g.dx - 2 - g.lo0 - 31) / 32 : -1, g.NX / 32 - 1);
    for (unsigned row = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; row < nrows; row += (gridDim.x * blockDim.x) >> 5) {
        const int y = (int)(row % (unsigned)g.NY), z = (int)(row / (unsigned)g.NY);
        const int vy = g.lo1 + y, vz = g.lo2 + z;
        const bool rface = !(vy >= 1 && vy <= g.dy - 2 && vz >= 1 && vz <= g.dz - 2);
        const long long rb = (long long)g.lo0 + (long long)vy * g.dx + (long long)vz * g.dxy;   // j of grid x = 0
        const float *rp = g.vol + rb + lane;
        unsigned *out = signs + (size_t)row * WX;
        const int f0 = rface ? (int)WX : xs0, f1 = rface ? (int)WX : xs1 + 1;   // direct words [f0, f1)
        for (int xw = 0; xw < min(f0, (int)WX); xw++) {
            const unsigned m = border_word(g, rb, rface, xw, lane);
            if (lane == 0) out[xw] = m;
        }
        if (vsign && f0 < f1) {   // direct words from the bitmap: lane k takes word f0 + k, f0 + 32 + k, ...
            for (int xw = f0 + lane; xw < f1; xw += 32) {
                const int vx0 = g.lo0 + xw * 32;   // 1 <= vx0 and vx0 + 31 <= dx - 2: both words lie in the row
                const int sh = vx0 & 31;
                const size_t wlo = od_vsign_word((unsigned)vx0, (unsigned)vy, (unsigned)vz, wv, nys);
                const unsigned lo = __ldg(vsign + wlo), hi = sh ? __ldg(vsign + wlo + 8) : 0u;   // next x word: +8
                out[xw] = __funnelshift_r(lo, hi, sh);
            }
        }
        for (int xw0 = f0; xw0 < (vsign ? f0 : f1); xw0 += SW) {
            float raw[SW];
#pragma unroll
            for (int k = 0; k < SW; k++) raw[k] = xw0 + k < f1 ? __ldg(rp + (xw0 + k) * 32) : 0.f;
            unsigned mine = 0;
#pragma unroll
            for (int k = 0; k < SW; k++) {
                const unsigned m = __ballot_sync(0xffffffffu, __fsub_rn(raw[k], g.iso) > -N2M_FLT_EPS);
                if (lane == k) mine = m;
            }
            if (lane < SW && xw0 + lane < f1) out[xw0 + lane] = mine;
        }
        for (int xw = max(f1, f0); xw < (int)WX; xw++) {
            const unsigned m = border_word(g, rb, rface, xw, lane);
            if (lane == 0) out[xw] = m;
        }
    }
}

// Count pass, part 2: one thread per word, 32 cubes at a time as bit masks.
// Corner k of the word's 32 cubes is a mask of the sign bits: the +x corners
// are the row shifted down by one with bit 0 of the next word on top.  Edge
// crossings are XORs; a cube needs a table lookup only if its corners are
// not all equal (about 3 % of them), and a value fetch only if its MC33 tiling
// needs a face or interior test.
__global__ void __launch_bounds__(256) k_words(GV g, bool classic, unsigned WX, unsigned nwords,
                                               const unsigned *__restrict__ signs, uint4 *words, uint4 *counts) {
    __shared__ unsigned char quick[256];
    quick[threadIdx.x] = quick_count(threadIdx.x, classic);
    __syncthreads();
    const unsigned rowstride = WX, slicestride = WX * (unsigned)g.NY;
    for (unsigned w = blockIdx.x * blockDim.x + threadIdx.x; w < nwords; w += gridDim.x * blockDim.x) {
        const unsigned xw = w % WX, row = w / WX;
        const int y = (int)(row % (unsigned)g.NY), z = (int)(row / (unsigned)g.NY);
        const int x0 = (int)xw * 32;
        const bool hy = y < g.NY - 1, hz = z < g.NZ - 1, nx = xw + 1 < WX;
        const unsigned inm = x0 + 32 <= g.NX ? 0xffffffffu : (1u << (g.NX - x0)) - 1u;   // x < NX
        const unsigned hxm = x0 + 33 <= g.NX ? 0xffffffffu : (g.NX - 1 - x0 > 0 ? (1u << (g.NX - 1 - x0)) - 1u : 0u);
        // corners: a = (y, z), b = (y+1, z), c = (y, z+1), d = (y+1, z+1); "1" = the +x neighbours
        const unsigned a0 = __ldg(signs + w);
        const unsigned a1 = __funnelshift_r(a0, nx ? __ldg(signs + w + 1) : 0u, 1);
        unsigned b0 = 0, b1 = 0, c0 = 0, c1 = 0, d0 = 0, d1 = 0;
        if (hy) {
            b0 = __ldg(signs + w + rowstride);
            b1 = __funnelshift_r(b0, nx ? __ldg(signs + w + rowstride + 1) : 0u, 1);
        }
        if (hz) {
            c0 = __ldg(signs + w + slicestride);
            c1 = __funnelshift_r(c0, nx ? __ldg(signs + w + slicestride + 1) : 0u, 1);
        }
        if (hy && hz) {
            d0 = __ldg(signs + w + slicestride + rowstride);
            d1 = __funnelshift_r(d0, nx ? __ldg(signs + w + slicestride + rowstride + 1) : 0u, 1);
        }
        const unsigned xm = (a0 ^ a1) & hxm;
        const unsigned ym = hy ? (a0 ^ b0) & inm : 0u;
        const unsigned zm = hz ? (a0 ^ c0) & inm : 0u;
        unsigned cnt = 0;
        if (hy && hz) {
            const unsigned any = a0 | a1 | b0 | b1 | c0 | c1 | d0 | d1, all = a0 & a1 & b0 & b1 & c0 & c1 & d0 & d1;
            unsigned mix = any & ~all & hxm;
            while (mix) {
                const int i = __ffs(mix) - 1;
                mix &= mix - 1;
                // corners 0..7 of the tables: (x,y,z) (x+1,y,z) (x+1,y+1,z) (x,y+1,z) and the same at z+1
                const int lut = (int)((a0 >> i) & 1u) | (int)((a1 >> i) & 1u) << 1 | (int)((b1 >> i) & 1u) << 2 |
                                (int)((b0 >> i) & 1u) << 3 | (int)((c0 >> i) & 1u) << 4 | (int)((c1 >> i) & 1u) << 5 |
                                (int)((d1 >> i) & 1u) << 6 | (int)((d0 >> i) & 1u) << 7;
                const unsigned q = quick[lut];
                cnt += (q & 0x80u) ? ambiguous_count(g, x0 + i, y, z, lut, classic) : q;
            }
        }
        const unsigned nv = __popc(xm) + __popc(ym) + __popc(zm);
        words[w] = make_uint4(xm, ym, zm, 0u);
        counts[w] = make_uint4(nv, cnt & 0xffffu, cnt >> 16, (nv | cnt) ? 1u : 0u);
    }
}

// Marks for the exact pre-smooth on demand: the voxel behind every corner of
// every cube whose corner signs differ (the only cubes whose values marching
// cubes reads), as bits of a linear bitmap over the volume.  A grid point's
// voxel is gval's linear index j (row wrap included); j past the volume is the
// padding value, which needs no voxel.
__global__ void __launch_bounds__(256) k_need(GV g, unsigned WX, unsigned nwords, const unsigned *__restrict__ signs,
                                              unsigned *need) {
    const unsigned rowstride = WX, slicestride = WX * (unsigned)g.NY;
    for (unsigned w = blockIdx.x * blockDim.x + threadIdx.x; w < nwords; w += gridDim.x * blockDim.x) {
        const unsigned xw = w % WX, row = w / WX;
        const int y = (int)(row % (unsigned)g.NY), z = (int)(row / (unsigned)g.NY);
        if (y >= g.NY - 1 || z >= g.NZ - 1) continue;   // no cubes start on the last row / slice
        const int x0 = (int)xw * 32;
        const bool nx = xw + 1 < WX;
        const unsigned hxm = x0 + 33 <= g.NX ? 0xffffffffu : (g.NX - 1 - x0 > 0 ? (1u << (g.NX - 1 - x0)) - 1u : 0u);
        const unsigned a0 = __ldg(signs + w), b0 = __ldg(signs + w + rowstride), c0 = __ldg(signs + w + slicestride),
                       d0 = __ldg(signs + w + slicestride + rowstride);
        const unsigned a1 = __funnelshift_r(a0, nx ? __ldg(signs + w + 1) : 0u, 1);
        const unsigned b1 = __funnelshift_r(b0, nx ? __ldg(signs + w + rowstride + 1) : 0u, 1);
        const unsigned c1 = __funnelshift_r(c0, nx ? __ldg(signs + w + slicestride + 1) : 0u, 1);
        const unsigned d1 = __funnelshift_r(d0, nx ? __ldg(signs + w + slicestride + rowstride + 1) : 0u, 1);
        const unsigned any = a0 | a1 | b0 | b1 | c0 | c1 | d0 | d1, all = a0 & a1 & b0 & b1 & c0 & c1 & d0 & d1;
        const unsigned mix = any & ~all & hxm;
        if (!mix) continue;
        const unsigned cm = mix | (mix << 1), carry = mix >> 31;   // corners x and x + 1 of each mixed cube
#pragma unroll
        for (int r = 0; r < 4; r++) {
            const long long j = (long long)(g.lo0 + x0) + (long long)(y + (r & 1) + g.lo1) * g.dx +
                                (long long)(z + (r >> 1) + g.lo2) * g.dxy;
            od_need_mark(need, j, cm, g.nvox);
            if (carry) od_need_mark(need, j + 32, 1u, g.nvox);
        }
    }
}

// active word list from the scanned counts (counts.w: exclusive count of
// active words before w), in word order
__global__ void k_active(const uint4 *__restrict__ offs, const uint4 *__restrict__ total, unsigned nwords,
                         unsigned *active) {
    const unsigned tot = total->w;
    for (unsigned w = blockIdx.x * blockDim.x + threadIdx.x; w < nwords; w += gridDim.x * blockDim.x) {
        const unsigned a = offs[w].w, b = w + 1 < nwords ? offs[w + 1].w : tot;
        if (b != a) active[a] = w;
    }
}

// ---- emit pass -------------------------------------------------------------------
// grid value at p (strictly inside the volume: no darkening, wrap or padding)
__device__ __forceinline__ float ival(const GV &g, const float *p) {
    const float v = __fsub_rn(__ldg(p), g.iso);
    return fabsf(v) < N2M_FLT_EPS ? N2M_FLT_EPS : v;
}

// exact float -> double by assembling the bits in integer registers (a
// conversion instruction would issue on the pipe this part shares with FP64;
// a predicated one still issues)
__device__ __forceinline__ double f2d(float f) {
    const unsigned u = __float_as_uint(f), e = (u >> 23) & 0xffu, m = u & 0x7fffffu;
    const unsigned long long sign = (unsigned long long)(u & 0x80000000u) << 32;
    unsigned long long de, dm;
    if (e == 0xffu) {               // Inf, NaN
        de = 0x7ffull;
        dm = (unsigned long long)m << 29;
    } else if (e != 0u) {           // normal
        de = e + 896u;
        dm = (unsigned long long)m << 29;
    } else if (m != 0u) {           // subnormal: m * 2^-149, leading bit p
        const int p = 31 - __clz((int)m);
        de = (unsigned long long)(p - 149 + 1023);
        dm = ((unsigned long long)m << (52 - p)) & 0xfffffffffffffull;
    } else {                        // signed zero
        de = 0;
        dm = 0;
    }
    return __longlong_as_double((long long)(sign | (de << 52) | dm));
}

// exact float of 0 <= v < 2^23 by bit assembly (no I2F conversion)
__device__ __forceinline__ float i2f_small(int v) { return __int_as_float(0x4B000000 | v) - 8388608.f; }

// tiling edge code 0..11 -> owner offset (bit 0: +x, 1: +y, 2: +z) and axis (bits 3-4)
__device__ __forceinline__ unsigned edge_code(int code) {
    constexpr unsigned long long k = (0x00ull << 0) | (0x09ull << 5) | (0x02ull << 10) | (0x08ull << 15) | (0x04ull << 20) |
                                     (0x0dull << 25) | (0x06ull << 30) | (0x0cull << 35) | (0x10ull << 40) |
                                     (0x11ull << 45) | (0x13ull << 50) | (0x12ull << 55);
    return (unsigned)(k >> (5 * code)) & 31u;
}

// id of the vertex on the `axis` edge of grid point (x,y,z) (the edge must cross)
__device__ __forceinline__ int vid(const uint4 *__restrict__ words, const uint4 *__restrict__ offs, unsigned NY,
                                   unsigned WX, int x, int y, int z, int axis) {
    const unsigned w = ((unsigned)z * NY + (unsigned)y) * WX + ((unsigned)x >> 5), l = (unsigned)x & 31u;
    const uint4 m = words[w];
    const unsigned lt = (1u << l) - 1u;
    unsigned id = offs[w].x + __popc(m.x & lt) + __popc(m.y & lt) + __popc(m.z & lt);
    if (axis >= 1) id += (m.x >> l) & 1u;
    if (axis == 2) id += (m.y >> l) & 1u;
    return (int)id;
}

__device__ __forceinline__ void add_cand(int *cand, unsigned *n, int cap, int id) {
    const unsigned k = atomicAdd(n, 1u);
    if (k < (unsigned)cap) cand[k] = id;
}

// c-vertex of a cube: mean of its crossing edge vertices (src/MarchingCubes.c:1029-1082)
__device__ __noinline__ void emit_cvertex(const float *c, int x, int y, int z, float flo0, float flo1, float flo2,
                                          int v12, vec3d *pts, int *ccand, unsigned *nccand, int cap) {
    float n = 0.f, sx = 0.f, sy = 0.f, sz = 0.f;
    for (int e = 0; e < 12; e++) {
        const int own = k_edge[e][0], ax = k_edge[e][1], ca = k_edge[e][2], cbn = k_edge[e][3];
        if ((c[ca] > 0.f) == (c[cbn] > 0.f)) continue;
        const float u = edge_u(c[ca], c[cbn]);
        float px = (float)(x + ((own ^ (own >> 1)) & 1)), py = (float)(y + ((own >> 1) & 1)), pz = (float)(z + ((own >> 2) & 1));
        if (ax == 0) px = __fadd_rn(px, u);
        else if (ax == 1) py = __fadd_rn(py, u);
        else pz = __fadd_rn(pz, u);
        n = __fadd_rn(n, 1.f);
        sx = __fadd_rn(sx, px); sy = __fadd_rn(sy, py); sz = __fadd_rn(sz, pz);
    }
    if (n > 0.f) { sx = __fdiv_rn(sx, n); sy = __fdiv_rn(sy, n); sz = __fdiv_rn(sz, n); }
    const float X = __fadd_rn(sx, flo0), Y = __fadd_rn(sy, flo1), Z = __fadd_rn(sz, flo2);
    pts[v12] = {f2d(X), f2d(Y), f2d(Z)};
    if (fminf(frac_dist(X), fminf(frac_dist(Y), frac_dist(Z))) < 1.5e-5f) add_cand(ccand, nccand, cap, v12);
}

// corner values of cube (x, y, z), by gval's rules (simple: strictly inside
// the volume)
__device__ __noinline__ void cube_values(const GV &g, bool simple, int x, int y, int z, float *c) {
    if (simple) {
        const float *p = g.vol + ((long long)(g.lo0 + x) + (long long)(y + g.lo1) * g.dx + (long long)(z + g.lo2) * g.dxy);
        const long long sy = g.dx, sz = g.dxy;
        c[0] = ival(g, p); c[1] = ival(g, p + 1); c[2] = ival(g, p + 1 + sy); c[3] = ival(g, p + sy);
        c[4] = ival(g, p + sz); c[5] = ival(g, p + 1 + sz); c[6] = ival(g, p + 1 + sy + sz); c[7] = ival(g, p + sy + sz);
    } else {
        c[0] = gval(g, x, y, z); c[1] = gval(g, x + 1, y, z); c[2] = gval(g, x + 1, y + 1, z); c[3] = gval(g, x, y + 1, z);
        c[4] = gval(g, x, y, z + 1); c[5] = gval(g, x + 1, y, z + 1); c[6] = gval(g, x + 1, y + 1, z + 1);
        c[7] = gval(g, x, y + 1, z + 1);
    }
}

// Group emit: a warp takes 32 consecutive active words, one per lane.  Each
// lane lists its word's edge vertices and the triangles of its unambiguous
// cubes into warp-private shared-memory lists (positions from the scanned
// offsets, so the lists come out in output order); then all 32 lanes work
// through the lists densely.  Ambiguous cubes (face/interior tests, maybe a
// c-vertex) and list overflow are handled by the owning lane directly.
constexpr int EG_WARPS = 4, EG_VCAP = 1024, EG_TCAP = 1024;
constexpr unsigned EG_HOLE = 0xffffffffu;

__device__ __forceinline__ void emit_vertex(const GV &g, bool simple, int x0, int y, int z, int p, int ax, int id,
                                            float flo0, float flo1, float flo2, vec3d *pts, int *cand, unsigned *ncand,
                                            int cap) {
    const int px = x0 + p;
    float c0, c1;
    if (simple) {
        const float *q = g.vol + ((long long)(g.lo0 + px) + (long long)(y + g.lo1) * g.dx + (long long)(z + g.lo2) * g.dxy);
        c0 = ival(g, q);
        c1 = ival(g, q + (ax == 0 ? 1ll : (ax == 1 ? (long long)g.dx : g.dxy)));
    } else {
        c0 = gval(g, px, y, z);
        c1 = gval(g, px + (ax == 0), y + (ax == 1), z + (ax == 2));
    }
    const float u = edge_u(c0, c1);
    const float fx = i2f_small(px), fy = i2f_small(y), fz = i2f_small(z);
    float X = __fadd_rn(fx, flo0), Y = __fadd_rn(fy, flo1), Z = __fadd_rn(fz, flo2), axv;
    if (ax == 0) axv = X = __fadd_rn(__fadd_rn(fx, u), flo0);
    else if (ax == 1) axv = Y = __fadd_rn(__fadd_rn(fy, u), flo1);
    else axv = Z = __fadd_rn(__fadd_rn(fz, u), flo2);
    pts[id] = {f2d(X), f2d(Y), f2d(Z)};
    if (frac_dist(axv) < 1.5e-5f) add_cand(cand, ncand, cap, id);
}

__device__ __forceinline__ void emit_triangle(const uint4 *__restrict__ words, const uint4 *__restrict__ offs,
                                              unsigned NY, unsigned WX, int x, int y, int z, int off, int v12,
                                              vec3i *dst) {
    int tv[3];
#pragma unroll
    for (int t = 0; t < 3; t++) {
        const int code = d_lut[off + t];
        int v = -1;
        if (code >= 0 && code < 12) {
            const unsigned ec = edge_code(code);
            v = vid(words, offs, NY, WX, x + (int)(ec & 1u), y + (int)((ec >> 1) & 1u), z + (int)((ec >> 2) & 1u),
                    (int)(ec >> 3));
        } else if (code == 12) {
            v = v12;
        }
        tv[t] = v;
    }
    *dst = {tv[2], tv[1], tv[0]};
}

__global__ void __launch_bounds__(EG_WARPS * 32) k_emit(GV g, bool classic, unsigned WX, const uint4 *__restrict__ words,
                                                          const uint4 *__restrict__ offs, const unsigned *__restrict__ signs,
                                                          const unsigned *__restrict__ active, unsigned nactive,
                                                          uint4 totals, vec3d *pts, vec3i *tris, int *cand,
                                                          unsigned *ncand, int *ccand, unsigned *nccand, int cap,
                                                          unsigned *next_group) {
    __shared__ unsigned short vitem[EG_WARPS][EG_VCAP];   // lane << 7 | point << 2 | axis
    __shared__ unsigned titem[EG_WARPS][EG_TCAP];          // lane << 27 | point << 22 | tiling offset, or a hole
    __shared__ unsigned qtile[256];                        // unambiguous tilings: offset << 8 | triangles; 0xff: tests
    for (int i = threadIdx.x; i < 256; i += EG_WARPS * 32) {
        Tiling T = {0, 0, false};
        qtile[i] = quick_tiling(i, classic, T) ? (unsigned)T.off << 8 | (unsigned)T.n : 0xffu;
    }
    __syncthreads();
    const unsigned lane = threadIdx.x & 31u, wid = threadIdx.x >> 5;
    const float flo0 = (float)g.lo0, flo1 = (float)g.lo1, flo2 = (float)g.lo2;
    const unsigned slice = WX * (unsigned)g.NY, NY = (unsigned)g.NY;
    const unsigned ngroups = (nactive + 31) / 32;
    for (;;) {   // groups are handed out one at a time: their work varies a lot
        unsigned grp = 0;
        if (lane == 0) grp = atomicAdd(next_group, 1u);
        grp = __shfl_sync(0xffffffffu, grp, 0);
        if (grp >= ngroups) break;
        const unsigned aw = grp * 32 + lane;
        const bool live = aw < nactive;
        const unsigned w = live ? active[aw] : active[nactive - 1];
        const unsigned row = w / WX, xw = w - row * WX;
        const int z = (int)(row / NY), y = (int)(row - (unsigned)z * NY);
        const int x0 = (int)(xw * 32u);
        const uint4 o = offs[w];
        const uint4 m = live ? words[w] : make_uint4(0u, 0u, 0u, 0u);
        const bool simple = g.lo0 + x0 >= 1 && g.lo0 + x0 + 32 <= g.dx - 2 && g.lo1 + y >= 1 && g.lo1 + y + 1 <= g.dy - 2 &&
                            g.lo2 + z >= 1 && g.lo2 + z + 1 <= g.dz - 2;
        const unsigned vbase = __shfl_sync(0xffffffffu, o.x, 0), tbase = __shfl_sync(0xffffffffu, o.y, 0);
        // ---- list the word's edge vertices (ids consecutive from o.x)
        {
            unsigned k = o.x - vbase;
            unsigned pm = m.x | m.y | m.z;
            while (pm) {
                const int p = __ffs(pm) - 1;
                pm &= pm - 1;
#pragma unroll
                for (int ax = 0; ax < 3; ax++) {
                    const unsigned mk = ax == 0 ? m.x : (ax == 1 ? m.y : m.z);
                    if (!((mk >> p) & 1u)) continue;
                    if (k < (unsigned)EG_VCAP) vitem[wid][k] = (unsigned short)(lane << 7 | (unsigned)p << 2 | (unsigned)ax);
                    else emit_vertex(g, simple, x0, y, z, p, ax, (int)(vbase + k), flo0, flo1, flo2, pts, cand, ncand, cap);
                    k++;
                }
            }
        }
        // ---- list the triangles of the word's cubes (positions from o.y)
        const bool hy = y < g.NY - 1, hz = z < g.NZ - 1, nxw = xw + 1 < WX;
        if (live && hy && hz) {
            const unsigned a0 = __ldg(signs + w), b0 = __ldg(signs + w + WX), c0 = __ldg(signs + w + slice),
                           d0 = __ldg(signs + w + slice + WX);
            unsigned an = 0, bn = 0, cn = 0, dn = 0;
            if (nxw) {
                an = __ldg(signs + w + 1); bn = __ldg(signs + w + WX + 1);
                cn = __ldg(signs + w + slice + 1); dn = __ldg(signs + w + slice + WX + 1);
            }
            const unsigned a1 = __funnelshift_r(a0, an, 1), b1 = __funnelshift_r(b0, bn, 1), c1 = __funnelshift_r(c0, cn, 1),
                           d1 = __funnelshift_r(d0, dn, 1);
            const unsigned hxm = x0 + 33 <= g.NX ? 0xffffffffu : (g.NX - 1 - x0 > 0 ? (1u << (g.NX - 1 - x0)) - 1u : 0u);
            unsigned mix = (a0 | a1 | b0 | b1 | c0 | c1 | d0 | d1) & ~(a0 & a1 & b0 & b1 & c0 & c1 & d0 & d1) & hxm;
            unsigned k = o.y - tbase;
            int cv = (int)(totals.x + o.z);
            while (mix) {
                const int p = __ffs(mix) - 1;
                mix &= mix - 1;
                const int lut = (int)((a0 >> p) & 1u) | (int)((a1 >> p) & 1u) << 1 | (int)((b1 >> p) & 1u) << 2 |
                                (int)((b0 >> p) & 1u) << 3 | (int)((c0 >> p) & 1u) << 4 | (int)((c1 >> p) & 1u) << 5 |
                                (int)((d1 >> p) & 1u) << 6 | (int)((d0 >> p) & 1u) << 7;
                const unsigned q = qtile[lut];
                if (q != 0xffu) {
                    const int off = (int)(q >> 8), n = (int)(q & 0xffu);
                    for (int j = 0; j < n; j++, k++) {
                        if (k < (unsigned)EG_TCAP) titem[wid][k] = lane << 27 | (unsigned)p << 22 | (unsigned)(off + 3 * j);
                        else emit_triangle(words, offs, NY, WX, x0 + p, y, z, off + 3 * j, -1, tris + tbase + k);
                    }
                } else {   // face/interior tests and the c-vertex: this lane
                    float cl[8];
                    cube_values(g, simple, x0 + p, y, z, cl);
                    const Tiling T = select_tiling(cl, lut, classic);
                    int v12 = -1;
                    if (T.cv) {
                        v12 = cv++;
                        emit_cvertex(cl, x0 + p, y, z, flo0, flo1, flo2, v12, pts, ccand, nccand, cap);
                    }
                    for (int j = 0; j < T.n; j++, k++) {
                        emit_triangle(words, offs, NY, WX, x0 + p, y, z, T.off + 3 * j, v12, tris + tbase + k);
                        if (k < (unsigned)EG_TCAP) titem[wid][k] = EG_HOLE;
                    }
                }
            }
        }
        // ---- group totals: the last live lane's end positions
        const unsigned nl = min(32u, nactive - grp * 32);
        const uint4 ol = offs[__shfl_sync(0xffffffffu, w, nl - 1)];   // every lane reads the same word
        const unsigned lastw = __shfl_sync(0xffffffffu, w, nl - 1);
        const uint4 ml = words[lastw];
        unsigned ntl = 0;   // triangles of the last word: next word's offset minus its own
        {
            const unsigned nw = (unsigned)WX * (unsigned)g.NY * (unsigned)g.NZ;
            const unsigned next_y = lastw + 1 < nw ? offs[lastw + 1].y : totals.y;
            ntl = next_y - ol.y;
        }
        const unsigned nvg = min((unsigned)EG_VCAP, ol.x + __popc(ml.x) + __popc(ml.y) + __popc(ml.z) - vbase);
        const unsigned ntg = min((unsigned)EG_TCAP, ol.y + ntl - tbase);
        __syncwarp();
        // ---- dense vertices
        for (unsigned b = 0; b < nvg; b += 32) {
            const unsigned k = b + lane;
            const unsigned e = k < nvg ? vitem[wid][k] : 0u;
            const int l = (int)(e >> 7);
            const int sx0 = __shfl_sync(0xffffffffu, x0, l), sy = __shfl_sync(0xffffffffu, y, l),
                      sz = __shfl_sync(0xffffffffu, z, l);
            const bool ssimple = __shfl_sync(0xffffffffu, simple, l);
            if (k < nvg)
                emit_vertex(g, ssimple, sx0, sy, sz, (int)((e >> 2) & 31u), (int)(e & 3u), (int)(vbase + k), flo0, flo1, flo2,
                            pts, cand, ncand, cap);
        }
        // ---- dense triangles
        for (unsigned b = 0; b < ntg; b += 32) {
            const unsigned k = b + lane;
            const unsigned e = k < ntg ? titem[wid][k] : EG_HOLE;
            const int l = (int)((e >> 27) & 31u);
            const int sx0 = __shfl_sync(0xffffffffu, x0, l), sy = __shfl_sync(0xffffffffu, y, l),
                      sz = __shfl_sync(0xffffffffu, z, l);
            if (e != EG_HOLE)
                emit_triangle(words, offs, NY, WX, sx0 + (int)((e >> 22) & 31u), sy, sz, (int)(e & 0x3fffffu), -1,
                              tris + tbase + k);
        }
        __syncwarp();   // the lists are reused by the next group
    }
}

// ---- adjoint of the vertex positions w.r.t. the processed volume -----------------
// Same value fetch as gval, also returning the voxel the value depends on (-1
// for padding, a darkened boundary voxel clamped to edge_max, or a value
// clamped to FLT_EPSILON: those are constant in the forward pass).
__device__ __forceinline__ float gval_src(const GV &g, int x, int y, int z, long long &src) {
    const long long j = (long long)(g.lo0 + x) + (long long)(y + g.lo1) * g.dx + (long long)(z + g.lo2) * g.dxy;
    float v;
    src = -1;
    if (j < g.nvox) {
        v = __ldg(g.vol + j);
        src = j;
        int vx = g.lo0 + x, vy = y + g.lo1, vz = z + g.lo2;   // wrapped as in gval
        if (vx >= g.dx) {
            vx -= g.dx;
            vy++;
        }
        if (vy >= g.dy) {
            vy -= g.dy;
            vz++;
        }
        if ((vx == 0 || vy == 0 || vz == 0 || vx == g.dx - 1 || vy == g.dy - 1 || vz == g.dz - 1) && !(v <= g.edge_max)) {
            v = g.edge_max;
            src = -1;
        }
        v = __fsub_rn(v, g.iso);
    } else {
        v = g.pad;
    }
    if (fabsf(v) < N2M_FLT_EPS) {
        v = N2M_FLT_EPS;
        src = -1;
    }
    return v;
}

// u = c0/(c0-c1): du/dc0 = -c1/(c0-c1)^2, du/dc1 = c0/(c0-c1)^2
__device__ __forceinline__ void edge_adjoint(float gax, float c0, float c1, long long s0, long long s1, float *gs) {
    const float den = c0 - c1;
    if (den == 0.f || gax == 0.f) return;
    const float inv2 = 1.f / (den * den);
    if (s0 >= 0) atomicAdd(gs + s0, -gax * c1 * inv2);
    if (s1 >= 0) atomicAdd(gs + s1, gax * c0 * inv2);
}

__device__ __forceinline__ float comp(const float3 &v, int a) { return a == 0 ? v.x : (a == 1 ? v.y : v.z); }

// one warp per active word, mirroring k_emit; gv = dL/d(raw vertex position)
__global__ void __launch_bounds__(256) k_mc_backward(GV g, bool classic, unsigned WX, const uint4 *__restrict__ words,
                                                     const uint4 *__restrict__ offs, const unsigned *__restrict__ active,
                                                     unsigned nactive, uint4 totals, const float3 *__restrict__ gv,
                                                     float *gs) {
    const unsigned lane = threadIdx.x & 31u;
    for (unsigned aw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; aw < nactive; aw += (gridDim.x * blockDim.x) >> 5) {
        const unsigned w = active[aw];
        const unsigned row = w / WX, xw = w - row * WX;
        const int z = (int)(row / (unsigned)g.NY), y = (int)(row - (unsigned)z * (unsigned)g.NY);
        const int x = (int)(xw * 32u + lane);
        const uint4 o = offs[w];
        const uint4 m = words[w];
        const bool in = x < g.NX;
        const bool hx = in && x < g.NX - 1, hy = in && y < g.NY - 1, hz = in && z < g.NZ - 1;
        const bool cube = hx && hy && hz;
        const bool ex = (m.x >> lane) & 1u, ey = (m.y >> lane) & 1u, ez = (m.z >> lane) & 1u;
        float c[8];
        long long sr[8];
        if (in) {
            c[0] = gval_src(g, x, y, z, sr[0]);
            c[1] = hx ? gval_src(g, x + 1, y, z, sr[1]) : c[0];
            c[3] = hy ? gval_src(g, x, y + 1, z, sr[3]) : c[0];
            c[4] = hz ? gval_src(g, x, y, z + 1, sr[4]) : c[0];
            if (cube) {
                c[2] = gval_src(g, x + 1, y + 1, z, sr[2]);
                c[5] = gval_src(g, x + 1, y, z + 1, sr[5]);
                c[6] = gval_src(g, x + 1, y + 1, z + 1, sr[6]);
                c[7] = gval_src(g, x, y + 1, z + 1, sr[7]);
            }
        }
        if (ex | ey | ez) {
            const unsigned lt = (1u << lane) - 1u;
            int id = (int)(o.x + __popc(m.x & lt) + __popc(m.y & lt) + __popc(m.z & lt));
            if (ex) { edge_adjoint(gv[id].x, c[0], c[1], sr[0], sr[1], gs); id++; }
            if (ey) { edge_adjoint(gv[id].y, c[0], c[3], sr[0], sr[3], gs); id++; }
            if (ez) edge_adjoint(gv[id].z, c[0], c[4], sr[0], sr[4], gs);
        }
        Tiling T = {0, 0, false};
        if (cube) {
            const int lut = cube_lut(c);
            if (lut != 0 && lut != 255) T = select_tiling(c, lut, classic);
        }
        int cb = T.cv;
        for (int d = 1; d < 32; d <<= 1) {
            const int b = __shfl_up_sync(0xffffffffu, cb, d);
            if ((int)lane >= d) cb += b;
        }
        cb -= T.cv;
        if (!T.cv) continue;
        // c-vertex = mean of the cube's crossing edge vertices
        const float3 gc = gv[totals.x + o.z + cb];
        int n = 0;
        for (int e = 0; e < 12; e++) n += (c[k_edge[e][2]] > 0.f) != (c[k_edge[e][3]] > 0.f);
        if (!n) continue;
        const float inv = 1.f / (float)n;
        for (int e = 0; e < 12; e++) {
            const int ax = k_edge[e][1], ca = k_edge[e][2], cbn = k_edge[e][3];
            if ((c[ca] > 0.f) == (c[cbn] > 0.f)) continue;
            edge_adjoint(comp(gc, ax) * inv, c[ca], c[cbn], sr[ca], sr[cbn], gs);
        }
    }
}

// vertices within 1.5e-5 of a c-vertex candidate become weld candidates too
__global__ void k_ccand(const vec3d *__restrict__ pts, int np, const int *__restrict__ cc, int ncc, int *cand,
                        unsigned *ncand, int cap) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < np; i += gridDim.x * blockDim.x) {
        const vec3d a = pts[i];
        for (int k = 0; k < ncc; k++) {
            const int j = cc[k];
            if (j == i) continue;
            const vec3d b = pts[j];
            const double dx = a.x - b.x, dy = a.y - b.y, dz = a.z - b.z;
            if (fabs(dx) < 1.5e-5 && fabs(dy) < 1.5e-5 && fabs(dz) < 1.5e-5) {
                unsigned q = atomicAdd(ncand, 1u);
                if (q < (unsigned)cap) cand[q] = i;
                break;
            }
        }
    }
}

GV make_gv(const McGrid &g) {
    GV v;
    v.vol = g.vol;
    v.dx = g.dim[0]; v.dy = g.dim[1]; v.dz = g.dim[2];
    v.dxy = (long long)g.dim[0] * g.dim[1];
    v.nvox = v.dxy * g.dim[2];
    v.lo0 = g.lo[0]; v.lo1 = g.lo[1]; v.lo2 = g.lo[2];
    v.NX = g.n[0]; v.NY = g.n[1]; v.NZ = g.n[2];
    v.NXY = (unsigned)g.n[0] * (unsigned)g.n[1];
    v.NG = v.NXY * (unsigned)g.n[2];
    v.iso = g.iso; v.edge_max = g.edge_max; v.pad = g.pad_val;
    return v;
}
}  // namespace

// counts: per word {vertices, triangles, c-vertices, active}; after the scan,
// exclusive offsets; totals.w = number of active words (listed in w.cand)
n2m_status mc_count(const McGrid &g, int variant, McWork &w, ScanWork &sw, uint4 *d_total, cudaStream_t s,
                    const OdRepair *repair) {
    const GV v = make_gv(g);
    const unsigned WX = (unsigned)((g.n[0] + 31) / 32);
    const size_t nwords = (size_t)WX * g.n[1] * g.n[2];
    if (nwords >= 0xffffffffULL) {
        n2m_set_error("grid too large");
        return N2M_ERR_TOO_LARGE;
    }
    CKS(w.words.ensure(nwords * sizeof(uint4)));
    CKS(w.counts.ensure(nwords * sizeof(uint4)));
    CKS(w.cand.ensure((nwords + 1) * sizeof(unsigned)));
    CKS(w.signs.ensure(nwords * sizeof(unsigned)));
    {
        const unsigned nrows = (unsigned)g.n[1] * (unsigned)g.n[2];
        const unsigned blocks = std::min<unsigned>((nrows + 7) / 8, 152u * 16u);
        k_signs<<<blocks, 256, 0, s>>>(v, WX, nrows, w.signs.as<unsigned>(),
                                       repair && !repair->post ? repair->w->vsign.as<unsigned>() : nullptr,
                                       (unsigned)(g.dim[0] + 31) / 32, (unsigned)(g.dim[1] + 7) / 8);
        N2M_COUNT();
    }
    if (repair) {   // exact smoothed values where the cubes below read them
        const size_t nvw = (size_t)((v.nvox + 31) >> 5);
        CKS(repair->w->need_z.ensure(nvw * sizeof(unsigned)));
        CK(cudaMemsetAsync(repair->w->need_z.p, 0, nvw * sizeof(unsigned), s));
        const unsigned blocks = (unsigned)std::min<size_t>((nwords + 255) / 256, 152u * 16u);
        k_need<<<blocks, 256, 0, s>>>(v, WX, (unsigned)nwords, w.signs.as<unsigned>(), repair->w->need_z.as<unsigned>());
        N2M_COUNT();
        CKL();
        CKS(od_repair(*repair, s));
    }
    {
        const unsigned blocks = (unsigned)std::min<size_t>((nwords + 255) / 256, 152u * 16u);
        k_words<<<blocks, 256, 0, s>>>(v, variant == N2M_CUBES_CLASSIC_TABLE, WX, (unsigned)nwords, w.signs.as<unsigned>(),
                                       w.words.as<uint4>(), w.counts.as<uint4>());
        N2M_COUNT();
    }
    CKL();
    CKS(scan_uint4(w.counts.as<uint4>(), nwords, d_total, sw, s));
    const unsigned blocks = (unsigned)std::min<size_t>((nwords + 255) / 256, 152u * 16u);
    { k_active<<<blocks, 256, 0, s>>>(w.counts.as<uint4>(), d_total, (unsigned)nwords, w.cand.as<unsigned>()); N2M_COUNT(); }
    CKL();
    return N2M_OK;
}

n2m_status mc_emit(const McGrid &g, int variant, McWork &w, const McCounts &c, vec3d *d_pts, vec3i *d_tris,
                   int *d_cand, unsigned *d_ncand, int cand_cap, cudaStream_t s) {
    const GV v = make_gv(g);
    const unsigned WX = (unsigned)((g.n[0] + 31) / 32);
    const unsigned nact = c.nactive;
    if (nact == 0) return N2M_OK;
    // CTAs of k_emit that fit the GPU at once, per device ordinal (the emit takes
    // its work from an atomic counter, so any grid is correct; this one is fastest)
    static std::atomic<int> resident_of[64];
    int dev = 0;
    CK(cudaGetDevice(&dev));
    int resident = dev < 64 ? resident_of[dev].load(std::memory_order_relaxed) : 0;
    if (!resident) {
        int sms = 0, per_sm = 0;
        CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_emit, EG_WARPS * 32, 0));
        resident = sms * std::max(per_sm, 1);
        if (dev < 64) resident_of[dev].store(resident, std::memory_order_relaxed);
    }
    const unsigned gblocks = std::min<unsigned>(((nact + 31) / 32 + EG_WARPS - 1) / EG_WARPS, (unsigned)resident);
    CKS(w.ctr.ensure(sizeof(unsigned)));
    CK(cudaMemsetAsync(w.ctr.p, 0, sizeof(unsigned), s));
    { k_emit<<<gblocks, EG_WARPS * 32, 0, s>>>(v, variant == N2M_CUBES_CLASSIC_TABLE, WX, w.words.as<uint4>(), w.counts.as<uint4>(), w.signs.as<unsigned>(), w.cand.as<unsigned>(), nact, make_uint4(c.nv_edge, c.nt, c.nc, 0), d_pts, d_tris, d_cand, d_ncand, d_cand + cand_cap, d_ncand + 1, cand_cap, w.ctr.as<unsigned>()); N2M_COUNT(); }
    CKL();
    return N2M_OK;
}

n2m_status mc_backward(const McGrid &g, int variant, McWork &w, const McCounts &c, const float3 *d_gv, float *d_gs,
                       cudaStream_t s) {
    const GV v = make_gv(g);
    const unsigned WX = (unsigned)((g.n[0] + 31) / 32);
    if (c.nactive == 0) return N2M_OK;
    const unsigned blocks = std::min<unsigned>((c.nactive + 7) / 8, 152u * 16u);
    { k_mc_backward<<<blocks, 256, 0, s>>>(v, variant == N2M_CUBES_CLASSIC_TABLE, WX, w.words.as<uint4>(), w.counts.as<uint4>(), w.cand.as<unsigned>(), c.nactive, make_uint4(c.nv_edge, c.nt, c.nc, 0), d_gv, d_gs); N2M_COUNT(); }
    CKL();
    return N2M_OK;
}

n2m_status mc_ccand_scan(const vec3d *d_pts, int np, const int *d_ccand, int nccand, int *d_cand,
                         unsigned *d_ncand, int cand_cap, cudaStream_t s) {
    if (nccand <= 0) return N2M_OK;
    const int blocks = (np + 255) / 256 < 4096 ? (np + 255) / 256 : 4096;
    { k_ccand<<<blocks > 0 ? blocks : 1, 256, 0, s>>>(d_pts, np, d_ccand, nccand, d_cand, d_ncand, cand_cap); N2M_COUNT(); }
    CKL();
    return N2M_OK;
}
