// oldcubes.cu — Bourke's classic marching cubes as the reference's
// USE_CLASSIC_CUBES build runs it (src/oldcubes.c:22-40, :401-463, :465-522),
// with edge-owned vertices instead of three private vertices per triangle.
//
// Cubes span [lo, hi-2] (absolute voxel coordinates, no padding).  A corner
// bit is set when value < isolevel.  The reference interpolates every copy
// of an edge vertex in double, oriented as the copying cube lists the edge,
// and its weld keeps the position of the LAST copy (src/meshify.c:99-100).
// Each edge here is computed once, in double, in the orientation of the last
// cube (raster order) that uses it, so positions are the reference's
// post-weld positions bit for bit.  The weld candidates (the few vertices near
// a grid point) can merge with vertices of other edges; the reference merges
// copies, so oc_copies / oc_copy_positions list every triangle corner that
// names a candidate (3*triangle + corner, its order in the reference's
// triangle soup) with the position the emitting cube gives that copy, and the
// host weld groups the copies as the reference does.
#include <algorithm>
#include <atomic>

#include "mc_tables.h"
#include "n2m_internal.cuh"

namespace {
__device__ const unsigned short d_edge[256] = N2M_CLASSIC_EDGE_INIT;
__device__ const signed char d_tri[256 * 16] = N2M_CLASSIC_TRI_INIT;

struct OV {
    const float *vol;
    int dx, dy, dz;
    long long dxy;
    int lo0, lo1, lo2, hi0, hi1, hi2;   // cube range [lo, hi-2]
    int NX, NY, NZ;                     // grid points: hi - lo
    unsigned NXY, NG, WX;   // WX: sign words per row
    float iso, edge_max;
};

// darkened voxel value (src/meshify.c:368-369)
__device__ __forceinline__ float oval(const OV &g, int X, int Y, int Z) {
    float v = __ldg(g.vol + (long long)Z * g.dxy + (long long)Y * g.dx + X);
    if (X == 0 || Y == 0 || Z == 0 || X == g.dx - 1 || Y == g.dy - 1 || Z == g.dz - 1) v = fminf(g.edge_max, v);
    return v;
}

__device__ __forceinline__ int ocube_ntri(int ci) {
    if (!d_edge[ci]) return 0;
    int n = 0;
    while (n < 5 && d_tri[ci * 16 + 3 * n] != -1) n++;
    return n;
}

// configuration of cube i of a word from its corner masks, in Bourke's corner
// order (x,y,z) (x+1,y,z) (x+1,y+1,z) (x,y+1,z) and the same at z+1
__device__ __forceinline__ int ocube_index(unsigned a0, unsigned a1, unsigned b0, unsigned b1, unsigned c0, unsigned c1,
                                           unsigned d0, unsigned d1, int i) {
    return (int)((a0 >> i) & 1u) | (int)((a1 >> i) & 1u) << 1 | (int)((b1 >> i) & 1u) << 2 | (int)((b0 >> i) & 1u) << 3 |
           (int)((c0 >> i) & 1u) << 4 | (int)((c1 >> i) & 1u) << 5 | (int)((d1 >> i) & 1u) << 6 | (int)((d0 >> i) & 1u) << 7;
}

// ---- count pass ---------------------------------------------------------------
// Sign words are row-aligned: bit x & 31 of signs[(z*NY + y)*WX + x/32] is set
// when grid point (x, y, z) is below the isolevel, darkened value included
// (points x >= NX read as 0).  Word order is raster order, so numbering by an
// exclusive scan over words gives the raster order of the reference's cubes.
constexpr int OS_W = 16;   // words of a row loaded at once per lane

// Sign words from the values of row rp (grid x = 0 at rp[0]), words [xa, xb):
// a warp takes OS_W words at a time with all their loads in flight.
__device__ __forceinline__ void oc_value_words(const OV &g, const float *rp, bool rface, unsigned xa, unsigned xb,
                                               unsigned *out, int lane) {
    if (xb - xa <= 2u) {   // the border words around the bitmap's: one at a time
        for (unsigned xw = xa; xw < xb; xw++) {
            const int x = (int)xw * 32 + lane, vx = g.lo0 + x;
            float v = x < g.NX ? __ldg(rp + x) : 0.f;
            if (rface || vx == 0 || vx == g.dx - 1) v = fminf(g.edge_max, v);
            const unsigned m = __ballot_sync(0xffffffffu, x < g.NX && v < g.iso);
            if (lane == 0) out[xw] = m;
        }
        return;
    }
    for (unsigned xw0 = xa; xw0 < xb; xw0 += OS_W) {
        float raw[OS_W];
#pragma unroll
        for (int k = 0; k < OS_W; k++) {
            const int x = (int)(xw0 + k) * 32 + lane;
            raw[k] = xw0 + k < xb && x < g.NX ? __ldg(rp + x) : 0.f;
        }
        unsigned mine = 0;
#pragma unroll
        for (int k = 0; k < OS_W; k++) {
            const int x = (int)(xw0 + k) * 32 + lane, vx = g.lo0 + x;
            const float v = rface || vx == 0 || vx == g.dx - 1 ? fminf(g.edge_max, raw[k]) : raw[k];
            const unsigned m = __ballot_sync(0xffffffffu, x < g.NX && v < g.iso);
            if (lane == k) mine = m;
        }
        if (lane < OS_W && xw0 + lane < xb) out[xw0 + lane] = mine;
    }
}

// A warp takes whole rows.  vsign (may be null): the volume's sign bitmap with
// bit = value >= iso (OdWork::vsign, wv words per row, nys groups of 8 rows);
// words whose points all lie strictly inside the volume are then the
// complement of two bitmap words shifted into place, the rest read values.
__global__ void __launch_bounds__(256) k_oc_signs(OV g, unsigned nrows, unsigned *signs, const unsigned *__restrict__ vsign,
                                                  unsigned wv, unsigned nys) {
    const int lane = threadIdx.x & 31;
    const unsigned WX = g.WX;
    // words xw whose 32 voxels lie in columns 1 .. dx-2
    const unsigned xs0 = (unsigned)max(0, (32 - g.lo0) / 32);
    const int xs1 = g.dx - 33 - g.lo0 >= 0 ? (g.dx - 33 - g.lo0) / 32 : -1;
    for (unsigned row = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; row < nrows; row += (gridDim.x * blockDim.x) >> 5) {
        const int y = (int)(row % (unsigned)g.NY), z = (int)(row / (unsigned)g.NY);
        const int vy = g.lo1 + y, vz = g.lo2 + z;
        const bool rface = vy == 0 || vz == 0 || vy == g.dy - 1 || vz == g.dz - 1;
        const float *rp = g.vol + (long long)vz * g.dxy + (long long)vy * g.dx + g.lo0;
        unsigned *out = signs + (size_t)row * WX;
        unsigned f0 = WX, f1 = WX;   // direct words [f0, f1)
        if (vsign && !rface) {
            f0 = min(xs0, WX);
            f1 = max(f0, (unsigned)min(xs1 + 1, (int)WX));
        }
        oc_value_words(g, rp, rface, 0, f0, out, lane);
        for (unsigned xw = f0 + lane; xw < f1; xw += 32) {
            const int x0 = (int)xw * 32, vx0 = g.lo0 + x0, sh = vx0 & 31;
            const size_t wlo = od_vsign_word((unsigned)vx0, (unsigned)vy, (unsigned)vz, wv, nys);
            const unsigned lo = __ldg(vsign + wlo), hi = sh ? __ldg(vsign + wlo + 8) : 0u;   // next x word: +8
            const unsigned inm = x0 + 32 <= g.NX ? 0xffffffffu : (1u << (g.NX - x0)) - 1u;
            out[xw] = ~__funnelshift_r(lo, hi, sh) & inm;
        }
        oc_value_words(g, rp, rface, f1, WX, out, lane);
    }
}

// Marks for the exact pre-smooth on demand: the voxel of every corner of
// every cube whose corner signs differ (the only cubes whose values the emit
// reads), as bits of a linear bitmap over the volume.
__global__ void __launch_bounds__(256) k_oc_need(OV g, unsigned nwords, const unsigned *__restrict__ signs,
                                                 unsigned *need) {
    const unsigned WX = g.WX, slice = WX * (unsigned)g.NY;
    const long long nvox = g.dxy * g.dz;
    for (unsigned w = blockIdx.x * blockDim.x + threadIdx.x; w < nwords; w += gridDim.x * blockDim.x) {
        const unsigned row = w / WX, xw = w - row * WX;
        const int z = (int)(row / (unsigned)g.NY), y = (int)(row - (unsigned)z * (unsigned)g.NY);
        if (y >= g.NY - 1 || z >= g.NZ - 1) continue;   // no cubes start on the last row / slice
        const int x0 = (int)xw * 32;
        const bool nx = xw + 1 < WX;
        const unsigned hxm = x0 + 33 <= g.NX ? 0xffffffffu : (g.NX - 1 - x0 > 0 ? (1u << (g.NX - 1 - x0)) - 1u : 0u);
        const unsigned a0 = __ldg(signs + w), b0 = __ldg(signs + w + WX), c0 = __ldg(signs + w + slice),
                       d0 = __ldg(signs + w + slice + WX);
        const unsigned a1 = __funnelshift_r(a0, nx ? __ldg(signs + w + 1) : 0u, 1);
        const unsigned b1 = __funnelshift_r(b0, nx ? __ldg(signs + w + WX + 1) : 0u, 1);
        const unsigned c1 = __funnelshift_r(c0, nx ? __ldg(signs + w + slice + 1) : 0u, 1);
        const unsigned d1 = __funnelshift_r(d0, nx ? __ldg(signs + w + slice + WX + 1) : 0u, 1);
        const unsigned mix = (a0 | a1 | b0 | b1 | c0 | c1 | d0 | d1) & ~(a0 & a1 & b0 & b1 & c0 & c1 & d0 & d1) & hxm;
        if (!mix) continue;
        const unsigned cm = mix | (mix << 1), carry = mix >> 31;   // corners x and x + 1 of each mixed cube
#pragma unroll
        for (int r = 0; r < 4; r++) {
            const long long j = (long long)(g.lo0 + x0) + (long long)(g.lo1 + y + (r & 1)) * g.dx +
                                (long long)(g.lo2 + z + (r >> 1)) * g.dxy;
            od_need_mark(need, j, cm, nvox);
            if (carry) od_need_mark(need, j + 32, 1u, nvox);
        }
    }
}

// One thread per word, 32 grid points at a time as bit masks: corner k of the
// word's 32 cubes is a mask of sign bits (the +x corners are the row shifted
// down by one with bit 0 of the next word on top), edge crossings are XORs, and
// only cubes whose corners are not all equal take a table lookup.
// counts: {edge vertices, triangles, 0, active}.
__global__ void __launch_bounds__(256) k_oc_words(OV g, unsigned nwords, const unsigned *__restrict__ signs,
                                                  uint4 *words, uint4 *counts) {
    __shared__ unsigned char ntri[256];
    ntri[threadIdx.x] = (unsigned char)ocube_ntri(threadIdx.x);
    __syncthreads();
    const unsigned WX = g.WX, slice = WX * (unsigned)g.NY;
    for (unsigned w = blockIdx.x * blockDim.x + threadIdx.x; w < nwords; w += gridDim.x * blockDim.x) {
        const unsigned row = w / WX, xw = w - row * WX;
        const int z = (int)(row / (unsigned)g.NY), y = (int)(row - (unsigned)z * (unsigned)g.NY);
        const int x0 = (int)xw * 32;
        const bool hy = y < g.NY - 1, hz = z < g.NZ - 1, nx = xw + 1 < WX;
        const unsigned inm = x0 + 32 <= g.NX ? 0xffffffffu : (1u << (g.NX - x0)) - 1u;   // x < NX
        const unsigned hxm = x0 + 33 <= g.NX ? 0xffffffffu : (g.NX - 1 - x0 > 0 ? (1u << (g.NX - 1 - x0)) - 1u : 0u);
        // a = (y, z), b = (y+1, z), c = (y, z+1), d = (y+1, z+1); "1" = the +x neighbours
        const unsigned a0 = __ldg(signs + w), a1 = __funnelshift_r(a0, nx ? __ldg(signs + w + 1) : 0u, 1);
        unsigned b0 = 0, b1 = 0, c0 = 0, c1 = 0, d0 = 0, d1 = 0;
        if (hy) {
            b0 = __ldg(signs + w + WX);
            b1 = __funnelshift_r(b0, nx ? __ldg(signs + w + WX + 1) : 0u, 1);
        }
        if (hz) {
            c0 = __ldg(signs + w + slice);
            c1 = __funnelshift_r(c0, nx ? __ldg(signs + w + slice + 1) : 0u, 1);
        }
        if (hy && hz) {
            d0 = __ldg(signs + w + slice + WX);
            d1 = __funnelshift_r(d0, nx ? __ldg(signs + w + slice + WX + 1) : 0u, 1);
        }
        const unsigned xm = (a0 ^ a1) & hxm, ym = hy ? (a0 ^ b0) & inm : 0u, zm = hz ? (a0 ^ c0) & inm : 0u;
        unsigned nt = 0;
        if (hy && hz) {
            unsigned mix = (a0 | a1 | b0 | b1 | c0 | c1 | d0 | d1) & ~(a0 & a1 & b0 & b1 & c0 & c1 & d0 & d1) & hxm;
            while (mix) {
                const int i = __ffs(mix) - 1;
                mix &= mix - 1;
                nt += ntri[ocube_index(a0, a1, b0, b1, c0, c1, d0, d1, i)];
            }
        }
        const unsigned nv = __popc(xm) + __popc(ym) + __popc(zm);
        words[w] = make_uint4(xm, ym, zm, 0u);
        counts[w] = make_uint4(nv, nt, 0u, (nv | nt) ? 1u : 0u);
    }
}

// active word list from the scanned counts (counts.w: exclusive count of active
// words before w), in word order
__global__ void k_oc_active(const uint4 *__restrict__ offs, const uint4 *__restrict__ total, unsigned nwords,
                            unsigned *active) {
    const unsigned tot = total->w;
    for (unsigned w = blockIdx.x * blockDim.x + threadIdx.x; w < nwords; w += gridDim.x * blockDim.x) {
        const unsigned a = offs[w].w, b = w + 1 < nwords ? offs[w + 1].w : tot;
        if (b != a) active[a] = w;
    }
}

// ---- emit pass -------------------------------------------------------------------
// id of the edge vertex owned by grid point (x, y, z) along axis ax: the word's
// offset plus the crossings of the points before it, x then y then z at a point
__device__ __forceinline__ int oc_vid(const uint4 *__restrict__ words, const uint4 *__restrict__ offs, unsigned WX,
                                      unsigned NY, int x, int y, int z, int ax) {
    const unsigned w = ((unsigned)z * NY + (unsigned)y) * WX + ((unsigned)x >> 5), l = (unsigned)x & 31u;
    const uint4 m = words[w];
    const unsigned lt = (1u << l) - 1u;
    unsigned id = offs[w].x + __popc(m.x & lt) + __popc(m.y & lt) + __popc(m.z & lt);
    if (ax >= 1) id += (m.x >> l) & 1u;
    if (ax == 2) id += (m.y >> l) & 1u;
    return (int)id;
}

// VertexInterp (src/oldcubes.c:22-40) along one axis: p = p1 + mu*(p2-p1)
// with mu = (iso - v1)/(v2 - v1); only the coordinate along the edge moves.
__device__ __forceinline__ double interp(double iso, double p1, double p2, double v1, double v2) {
    const double mu = __ddiv_rn(__dsub_rn(iso, v1), __dsub_rn(v2, v1));
    return __dadd_rn(p1, __dmul_rn(mu, __dsub_rn(p2, p1)));
}

// The edge vertex of grid point (x, y, z) along axis ax, interpolated as the
// last cube (raster order) that lists the edge orients it; a position within
// 1.5e-5 of a grid coordinate makes the vertex a weld candidate.
__device__ __forceinline__ void oc_vertex(const OV &g, int x, int y, int z, int ax, int id, vec3d *pts, int *cand,
                                          unsigned *ncand, int cap) {
    const int X = g.lo0 + x, Y = g.lo1 + y, Z = g.lo2 + z;
    const double iso = (double)g.iso, dX = X, dY = Y, dZ = Z;
    const double v0 = oval(g, X, Y, Z);
    const int c0 = g.lo0, c1 = g.lo1, c2 = g.lo2, e0 = g.hi0 - 2, e1 = g.hi1 - 2, e2 = g.hi2 - 2;
    double r;
    vec3d P;
    if (ax == 0) {   // last user: (X,Y,Z) fwd > (X,Y-1,Z) rev > (X,Y,Z-1) fwd > (X,Y-1,Z-1) rev
        const double v1 = oval(g, X + 1, Y, Z);
        bool fwd;
        if (Y <= e1 && Z <= e2) fwd = true;
        else if (Y - 1 >= c1 && Z <= e2) fwd = false;
        else if (Y <= e1 && Z - 1 >= c2) fwd = true;
        else fwd = false;
        r = fwd ? interp(iso, dX, dX + 1.0, v0, v1) : interp(iso, dX + 1.0, dX, v1, v0);
        P = {r, dY, dZ};
    } else if (ax == 1) {   // (X,Y,Z) rev > (X-1,Y,Z) fwd > (X,Y,Z-1) rev > (X-1,Y,Z-1) fwd
        const double v3 = oval(g, X, Y + 1, Z);
        bool fwd;
        if (X <= e0 && Z <= e2) fwd = false;
        else if (X - 1 >= c0 && Z <= e2) fwd = true;
        else if (X <= e0 && Z - 1 >= c2) fwd = false;
        else fwd = true;
        r = fwd ? interp(iso, dY, dY + 1.0, v0, v3) : interp(iso, dY + 1.0, dY, v3, v0);
        P = {dX, r, dZ};
    } else {   // every user lists the z edge bottom to top
        r = interp(iso, dZ, dZ + 1.0, v0, (double)oval(g, X, Y, Z + 1));
        P = {dX, dY, r};
    }
    pts[id] = P;
    if (fabs(r - rint(r)) < 1.5e-5) {
        const unsigned k = atomicAdd(ncand, 1u);
        if (k < (unsigned)cap) cand[k] = id;
    }
}

// Bourke edge 0..11 -> owning grid point offset (bit 0: +x, 1: +y, 2: +z) and axis (bits 3-4)
__device__ __forceinline__ unsigned oc_edge(int e) {
    constexpr unsigned long long k = (0x00ull << 0) | (0x09ull << 5) | (0x02ull << 10) | (0x08ull << 15) | (0x04ull << 20) |
                                     (0x0dull << 25) | (0x06ull << 30) | (0x0cull << 35) | (0x10ull << 40) |
                                     (0x11ull << 45) | (0x13ull << 50) | (0x12ull << 55);
    return (unsigned)(k >> (5 * e)) & 31u;
}

// triangle j of configuration ci of the cube at grid point (x, y, z)
__device__ __forceinline__ void oc_triangle(const uint4 *__restrict__ words, const uint4 *__restrict__ offs, unsigned WX,
                                            unsigned NY, int x, int y, int z, int ci, int j, vec3i *dst) {
    int tv[3];
#pragma unroll
    for (int t = 0; t < 3; t++) {
        const unsigned ec = oc_edge(d_tri[ci * 16 + 3 * j + t]);
        tv[t] = oc_vid(words, offs, WX, NY, x + (int)(ec & 1u), y + (int)((ec >> 1) & 1u), z + (int)((ec >> 2) & 1u),
                       (int)(ec >> 3));
    }
    *dst = {tv[0], tv[1], tv[2]};
}

// A warp takes 32 active words at a time (one per lane), lists their edge
// vertices and triangles in shared memory (ids and positions are consecutive
// within the group) and then emits the lists with all lanes busy.  Items past
// a list's capacity are emitted by the lane that found them.
constexpr int OE_WARPS = 4, OE_VCAP = 1024, OE_TCAP = 1024;

__global__ void __launch_bounds__(OE_WARPS * 32) k_oc_emit(OV g, const unsigned *__restrict__ signs,
                                                          const uint4 *__restrict__ words, const uint4 *__restrict__ offs,
                                                          const unsigned *__restrict__ active, unsigned nactive,
                                                          vec3d *pts, vec3i *tris, int *cand, unsigned *ncand, int cap,
                                                          unsigned *next_group) {
    __shared__ unsigned short vitem[OE_WARPS][OE_VCAP];   // lane << 7 | point << 2 | axis
    __shared__ unsigned titem[OE_WARPS][OE_TCAP];          // lane << 27 | point << 22 | configuration << 3 | triangle
    __shared__ unsigned char ntri[256];
    for (int i = threadIdx.x; i < 256; i += OE_WARPS * 32) ntri[i] = (unsigned char)ocube_ntri(i);
    __syncthreads();
    const unsigned lane = threadIdx.x & 31u, wid = threadIdx.x >> 5;
    const unsigned WX = g.WX, NY = (unsigned)g.NY, slice = WX * NY;
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
        const int z = (int)(row / NY), y = (int)(row - (unsigned)z * NY), x0 = (int)(xw * 32u);
        const uint4 o = offs[w];
        const uint4 m = live ? words[w] : make_uint4(0u, 0u, 0u, 0u);
        const unsigned vbase = __shfl_sync(0xffffffffu, o.x, 0), tbase = __shfl_sync(0xffffffffu, o.y, 0);
        unsigned kv = o.x - vbase;   // the word's edge vertices
        for (unsigned pm = m.x | m.y | m.z; pm; pm &= pm - 1) {
            const int p = __ffs(pm) - 1;
#pragma unroll
            for (int ax = 0; ax < 3; ax++) {
                const unsigned mk = ax == 0 ? m.x : (ax == 1 ? m.y : m.z);
                if (!((mk >> p) & 1u)) continue;
                if (kv < (unsigned)OE_VCAP) vitem[wid][kv] = (unsigned short)(lane << 7 | (unsigned)p << 2 | (unsigned)ax);
                else oc_vertex(g, x0 + p, y, z, ax, (int)(vbase + kv), pts, cand, ncand, cap);
                kv++;
            }
        }
        unsigned kt = o.y - tbase;   // the word's triangles
        if (live && y < g.NY - 1 && z < g.NZ - 1) {
            const bool nx = xw + 1 < WX;
            const unsigned a0 = __ldg(signs + w), b0 = __ldg(signs + w + WX), c0 = __ldg(signs + w + slice),
                           d0 = __ldg(signs + w + slice + WX);
            unsigned an = 0, bn = 0, cn = 0, dn = 0;
            if (nx) {
                an = __ldg(signs + w + 1); bn = __ldg(signs + w + WX + 1);
                cn = __ldg(signs + w + slice + 1); dn = __ldg(signs + w + slice + WX + 1);
            }
            const unsigned a1 = __funnelshift_r(a0, an, 1), b1 = __funnelshift_r(b0, bn, 1),
                           c1 = __funnelshift_r(c0, cn, 1), d1 = __funnelshift_r(d0, dn, 1);
            const unsigned hxm = x0 + 33 <= g.NX ? 0xffffffffu : (g.NX - 1 - x0 > 0 ? (1u << (g.NX - 1 - x0)) - 1u : 0u);
            for (unsigned mix = (a0 | a1 | b0 | b1 | c0 | c1 | d0 | d1) & ~(a0 & a1 & b0 & b1 & c0 & c1 & d0 & d1) & hxm; mix;
                 mix &= mix - 1) {
                const int p = __ffs(mix) - 1;
                const int ci = ocube_index(a0, a1, b0, b1, c0, c1, d0, d1, p), n = ntri[ci];
                for (int j = 0; j < n; j++, kt++) {
                    if (kt < (unsigned)OE_TCAP) titem[wid][kt] = lane << 27 | (unsigned)p << 22 | (unsigned)ci << 3 | (unsigned)j;
                    else oc_triangle(words, offs, WX, NY, x0 + p, y, z, ci, j, tris + tbase + kt);
                }
            }
        }
        // lanes past the last live one repeat its word with no items: the
        // largest end is the group's end
        const unsigned nvg = min((unsigned)OE_VCAP, __reduce_max_sync(0xffffffffu, kv));
        const unsigned ntg = min((unsigned)OE_TCAP, __reduce_max_sync(0xffffffffu, kt));
        __syncwarp();
        for (unsigned b = 0; b < nvg; b += 32) {
            const unsigned k = b + lane;
            const unsigned e = k < nvg ? vitem[wid][k] : 0u;
            const int l = (int)(e >> 7);
            const int sx0 = __shfl_sync(0xffffffffu, x0, l), sy = __shfl_sync(0xffffffffu, y, l),
                      sz = __shfl_sync(0xffffffffu, z, l);
            if (k < nvg)
                oc_vertex(g, sx0 + (int)((e >> 2) & 31u), sy, sz, (int)(e & 3u), (int)(vbase + k), pts, cand, ncand, cap);
        }
        for (unsigned b = 0; b < ntg; b += 32) {
            const unsigned k = b + lane;
            const unsigned e = k < ntg ? titem[wid][k] : 0u;
            const int l = (int)(e >> 27);
            const int sx0 = __shfl_sync(0xffffffffu, x0, l), sy = __shfl_sync(0xffffffffu, y, l),
                      sz = __shfl_sync(0xffffffffu, z, l);
            if (k < ntg)
                oc_triangle(words, offs, WX, NY, sx0 + (int)((e >> 22) & 31u), sy, sz, (int)((e >> 3) & 0xffu),
                            (int)(e & 7u), tris + tbase + k);
        }
        __syncwarp();   // the lists are reused by the next group
    }
}

// weld candidates as a bitmap over the vertices
__global__ void k_oc_candbits(const int *__restrict__ cand, unsigned ncand, unsigned *bits) {
    for (unsigned i = blockIdx.x * blockDim.x + threadIdx.x; i < ncand; i += gridDim.x * blockDim.x) {
        const unsigned v = (unsigned)cand[i];
        atomicOr(bits + (v >> 5), 1u << (v & 31u));
    }
}

// every triangle corner (3*t + c) that names a weld candidate (bit set)
__global__ void k_oc_copies(const vec3i *__restrict__ tris, unsigned nt, const unsigned *__restrict__ bits,
                            unsigned *out, unsigned *count, unsigned cap) {
    for (unsigned t = blockIdx.x * blockDim.x + threadIdx.x; t < nt; t += gridDim.x * blockDim.x) {
        const vec3i T = tris[t];
        const int v[3] = {T.x, T.y, T.z};
#pragma unroll
        for (int c = 0; c < 3; c++)
            if ((__ldg(bits + ((unsigned)v[c] >> 5)) >> ((unsigned)v[c] & 31u)) & 1u) {
                const unsigned k = atomicAdd(count, 1u);
                if (k < cap) out[k] = 3u * t + (unsigned)c;
            }
    }
}

// Bourke's corners (bit 0: +x, 1: +y, 2: +z) and each edge's two corners, in
// the order VertexInterp takes them (src/oldcubes.c:418-441)
__constant__ unsigned char c_corner[8] = {0, 1, 3, 2, 4, 5, 7, 6};
__constant__ unsigned char c_edge_ab[12][2] = {{0, 1}, {1, 2}, {2, 3}, {3, 0}, {4, 5}, {5, 6},
                                               {6, 7}, {7, 4}, {0, 4}, {1, 5}, {2, 6}, {3, 7}};

// The copy of a vertex that corner q = 3t + c holds in the reference's
// triangle soup: the cube that emitted triangle t (the word whose triangle
// range holds t, then the cube within it) and the position that cube's
// VertexInterp gives, in the edge's orientation within that cube.
__global__ void k_oc_copy_pos(OV g, const unsigned *__restrict__ signs, const uint4 *__restrict__ offs, unsigned nwords,
                              const vec3i *__restrict__ tris, const unsigned *__restrict__ qs, unsigned n, int *vid,
                              vec3d *pos) {
    const unsigned WX = g.WX, slice = WX * (unsigned)g.NY;
    const double iso = (double)g.iso;
    for (unsigned i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const unsigned q = qs[i], t = q / 3u, c = q - 3u * t;
        unsigned lo = 0, hi = nwords - 1;   // the last word whose first triangle is <= t
        while (lo < hi) {
            const unsigned mid = lo + (hi - lo + 1) / 2;
            if (offs[mid].y <= t) lo = mid;
            else hi = mid - 1;
        }
        const unsigned w = lo, row = w / WX, xw = w - row * WX;
        const int z = (int)(row / (unsigned)g.NY), y = (int)(row - (unsigned)z * (unsigned)g.NY), x0 = (int)xw * 32;
        const bool nx = xw + 1 < WX;
        const unsigned hxm = x0 + 33 <= g.NX ? 0xffffffffu : (g.NX - 1 - x0 > 0 ? (1u << (g.NX - 1 - x0)) - 1u : 0u);
        const unsigned a0 = signs[w], b0 = signs[w + WX], c0 = signs[w + slice], d0 = signs[w + slice + WX];
        const unsigned a1 = __funnelshift_r(a0, nx ? signs[w + 1] : 0u, 1), b1 = __funnelshift_r(b0, nx ? signs[w + WX + 1] : 0u, 1),
                       c1 = __funnelshift_r(c0, nx ? signs[w + slice + 1] : 0u, 1),
                       d1 = __funnelshift_r(d0, nx ? signs[w + slice + WX + 1] : 0u, 1);
        unsigned k = t - offs[w].y;
        int p = 0, ci = 0;
        for (unsigned mix = (a0 | a1 | b0 | b1 | c0 | c1 | d0 | d1) & ~(a0 & a1 & b0 & b1 & c0 & c1 & d0 & d1) & hxm; mix;
             mix &= mix - 1) {
            p = __ffs(mix) - 1;
            ci = ocube_index(a0, a1, b0, b1, c0, c1, d0, d1, p);
            const unsigned nc = (unsigned)ocube_ntri(ci);
            if (k < nc) break;
            k -= nc;
        }
        const int e = d_tri[ci * 16 + 3 * (int)k + (int)c];
        const unsigned ca = c_corner[c_edge_ab[e][0]], cb = c_corner[c_edge_ab[e][1]];
        const int X = g.lo0 + x0 + p, Y = g.lo1 + y, Z = g.lo2 + z;
        const int ax = X + (int)(ca & 1u), ay = Y + (int)((ca >> 1) & 1u), az = Z + (int)(ca >> 2);
        const int bx = X + (int)(cb & 1u), by = Y + (int)((cb >> 1) & 1u), bz = Z + (int)(cb >> 2);
        const double va = oval(g, ax, ay, az), vb = oval(g, bx, by, bz);
        const double mu = __ddiv_rn(__dsub_rn(iso, va), __dsub_rn(vb, va));
        vec3d P = {(double)ax, (double)ay, (double)az};
        if (ax != bx) P.x = __dadd_rn(P.x, __dmul_rn(mu, (double)(bx - ax)));
        if (ay != by) P.y = __dadd_rn(P.y, __dmul_rn(mu, (double)(by - ay)));
        if (az != bz) P.z = __dadd_rn(P.z, __dmul_rn(mu, (double)(bz - az)));
        const vec3i T = tris[t];
        vid[i] = c == 0 ? T.x : (c == 1 ? T.y : T.z);
        pos[i] = P;
    }
}

OV make_ov(const float *vol, const int dim[3], const int lo[3], const int hi[3], float iso, float edge_max) {
    OV g;
    g.vol = vol;
    g.dx = dim[0]; g.dy = dim[1]; g.dz = dim[2];
    g.dxy = (long long)dim[0] * dim[1];
    g.lo0 = lo[0]; g.lo1 = lo[1]; g.lo2 = lo[2];
    g.hi0 = hi[0]; g.hi1 = hi[1]; g.hi2 = hi[2];
    g.NX = hi[0] - lo[0]; g.NY = hi[1] - lo[1]; g.NZ = hi[2] - lo[2];
    g.NXY = (unsigned)g.NX * (unsigned)g.NY;
    g.NG = g.NXY * (unsigned)g.NZ;
    g.WX = (unsigned)(g.NX + 31) / 32;
    g.iso = iso;
    g.edge_max = edge_max;
    return g;
}
}  // namespace

n2m_status oc_count(const float *vol, const int dim[3], const int lo[3], const int hi[3], float iso,
                     float edge_max, McWork &w, ScanWork &sw, uint4 *d_total, cudaStream_t s, const OdRepair *repair) {
    const OV g = make_ov(vol, dim, lo, hi, iso, edge_max);
    if (g.NX < 2 || g.NY < 2 || g.NZ < 2) {
        CK(cudaMemsetAsync(d_total, 0, sizeof(uint4), s));
        return N2M_OK;
    }
    const size_t nwords = (size_t)g.WX * g.NY * g.NZ;
    if (nwords >= 0xffffffffULL) {
        n2m_set_error("grid too large");
        return N2M_ERR_TOO_LARGE;
    }
    CKS(w.words.ensure(nwords * sizeof(uint4)));
    CKS(w.counts.ensure(nwords * sizeof(uint4)));
    CKS(w.signs.ensure(nwords * sizeof(unsigned)));
    CKS(w.cand.ensure((nwords + 1) * sizeof(unsigned)));
    const unsigned nrows = (unsigned)g.NY * (unsigned)g.NZ;
    const unsigned wblocks = (unsigned)std::min<size_t>((nwords + 255) / 256, 152u * 16u);
    { k_oc_signs<<<std::min<unsigned>((nrows + 7) / 8, 152u * 16u), 256, 0, s>>>(g, nrows, w.signs.as<unsigned>(), repair && !repair->post ? repair->w->vsign.as<unsigned>() : nullptr, (unsigned)(dim[0] + 31) / 32, (unsigned)(dim[1] + 7) / 8); N2M_COUNT(); }
    if (repair) {   // exact smoothed values where the emit reads them
        const size_t nvw = ((size_t)dim[0] * dim[1] * dim[2] + 31) / 32;
        CKS(repair->w->need_z.ensure(nvw * sizeof(unsigned)));
        CK(cudaMemsetAsync(repair->w->need_z.p, 0, nvw * sizeof(unsigned), s));
        { k_oc_need<<<wblocks, 256, 0, s>>>(g, (unsigned)nwords, w.signs.as<unsigned>(), repair->w->need_z.as<unsigned>()); N2M_COUNT(); }
        CKL();
        CKS(od_repair(*repair, s));
    }
    { k_oc_words<<<wblocks, 256, 0, s>>>(g, (unsigned)nwords, w.signs.as<unsigned>(), w.words.as<uint4>(), w.counts.as<uint4>()); N2M_COUNT(); }
    CKL();
    CKS(scan_uint4(w.counts.as<uint4>(), nwords, d_total, sw, s));
    { k_oc_active<<<wblocks, 256, 0, s>>>(w.counts.as<uint4>(), d_total, (unsigned)nwords, w.cand.as<unsigned>()); N2M_COUNT(); }
    CKL();
    return N2M_OK;
}

n2m_status oc_emit(const float *vol, const int dim[3], const int lo[3], const int hi[3], float iso, float edge_max,
                    McWork &w, const McCounts &c, vec3d *d_pts, vec3i *d_tris, int *d_cand, unsigned *d_ncand,
                    int cand_cap, cudaStream_t s) {
    const OV g = make_ov(vol, dim, lo, hi, iso, edge_max);
    const unsigned nact = c.nactive;
    if (nact == 0) return N2M_OK;
    // CTAs of k_oc_emit that fit the GPU at once, per device ordinal (groups come
    // from an atomic counter, so any grid is correct)
    static std::atomic<int> resident_of[64];
    int dev = 0;
    CK(cudaGetDevice(&dev));
    int resident = dev < 64 ? resident_of[dev].load(std::memory_order_relaxed) : 0;
    if (!resident) {
        int sms = 0, per_sm = 0;
        CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_oc_emit, OE_WARPS * 32, 0));
        resident = sms * std::max(per_sm, 1);
        if (dev < 64) resident_of[dev].store(resident, std::memory_order_relaxed);
    }
    const unsigned gblocks = std::min<unsigned>(((nact + 31) / 32 + OE_WARPS - 1) / OE_WARPS, (unsigned)resident);
    CKS(w.ctr.ensure(sizeof(unsigned)));
    CK(cudaMemsetAsync(w.ctr.p, 0, sizeof(unsigned), s));
    { k_oc_emit<<<gblocks, OE_WARPS * 32, 0, s>>>(g, w.signs.as<unsigned>(), w.words.as<uint4>(), w.counts.as<uint4>(), w.cand.as<unsigned>(), nact, d_pts, d_tris, d_cand, d_ncand, cand_cap, w.ctr.as<unsigned>()); N2M_COUNT(); }
    CKL();
    return N2M_OK;
}

n2m_status oc_copies(const vec3i *d_tris, int nt, int nv, const int *d_cand, int ncand, unsigned *d_bits,
                     unsigned *d_out, unsigned *d_count, unsigned cap, cudaStream_t s) {
    CK(cudaMemsetAsync(d_bits, 0, (size_t)(nv + 31) / 32 * sizeof(unsigned), s));
    CK(cudaMemsetAsync(d_count, 0, sizeof(unsigned), s));
    { k_oc_candbits<<<(unsigned)std::max(1, std::min((ncand + 255) / 256, 1024)), 256, 0, s>>>(d_cand, (unsigned)ncand, d_bits); N2M_COUNT(); }
    { k_oc_copies<<<(unsigned)std::max(1, std::min((nt + 255) / 256, 152 * 16)), 256, 0, s>>>(d_tris, (unsigned)nt, d_bits, d_out, d_count, cap); N2M_COUNT(); }
    CKL();
    return N2M_OK;
}

n2m_status oc_copy_positions(const float *vol, const int dim[3], const int lo[3], const int hi[3], float iso,
                             float edge_max, const McWork &w, const vec3i *d_tris, const unsigned *d_q, int n, int *d_vid,
                             vec3d *d_pos, cudaStream_t s) {
    const OV g = make_ov(vol, dim, lo, hi, iso, edge_max);
    const size_t nwords = (size_t)g.WX * g.NY * g.NZ;
    if (n <= 0 || nwords == 0) return N2M_OK;
    { k_oc_copy_pos<<<(unsigned)std::min((n + 127) / 128, 1024), 128, 0, s>>>(g, w.signs.as<unsigned>(), w.counts.as<uint4>(), (unsigned)nwords, d_tris, d_q, (unsigned)n, d_vid, d_pos); N2M_COUNT(); }
    CKL();
    return N2M_OK;
}
