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
// post-weld positions bit for bit.  For the weld candidates (the few vertices
// near a grid point), oc_lastuse records the index of the vertex's last copy in
// the reference's pre-weld vertex list (3*triangle + corner) so that
// near-corner clusters keep the same survivor.
#include <algorithm>

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
    unsigned NXY, NG;
    float iso, edge_max;
};

// darkened voxel value (src/meshify.c:368-369)
__device__ __forceinline__ float oval(const OV &g, int X, int Y, int Z) {
    float v = __ldg(g.vol + (long long)Z * g.dxy + (long long)Y * g.dx + X);
    if (X == 0 || Y == 0 || Z == 0 || X == g.dx - 1 || Y == g.dy - 1 || Z == g.dz - 1) v = fminf(g.edge_max, v);
    return v;
}

struct OP {
    bool ex, ey, ez;
    int X, Y, Z;         // absolute point
    float v[5];          // p0, p1 (+x), -, p3 (+y), p4 (+z) in Bourke's corner numbering
};

__device__ __forceinline__ int ocube_ntri(int ci) {
    if (!d_edge[ci]) return 0;
    int n = 0;
    while (n < 5 && d_tri[ci * 16 + 3 * n] != -1) n++;
    return n;
}

// Signs of the grid: bit p & 31 of word p >> 5 is set when grid point p
// (linear in the grid) is below the isolevel, darkened value included.  The
// count and the emit read a cube's eight corners as bits of this bitmap.
__global__ void __launch_bounds__(256) k_oc_signs(OV g, unsigned *bits) {
    const unsigned nw = (g.NG + 31u) >> 5;
    const int lane = threadIdx.x & 31;
    for (unsigned w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; w < nw; w += (gridDim.x * blockDim.x) >> 5) {
        const unsigned p = w * 32u + (unsigned)lane;
        bool b = false;
        if (p < g.NG) {
            const int z = (int)(p / g.NXY);
            const unsigned r = p - (unsigned)z * g.NXY;
            const int y = (int)(r / (unsigned)g.NX), x = (int)(r - (unsigned)y * (unsigned)g.NX);
            b = oval(g, g.lo0 + x, g.lo1 + y, g.lo2 + z) < g.iso;
        }
        const unsigned m = __ballot_sync(0xffffffffu, b);
        if (lane == 0) bits[w] = m;
    }
}

// 32 sign bits starting at grid point q (bits past the grid read as 0)
__device__ __forceinline__ unsigned obits(const unsigned *__restrict__ bits, unsigned q, unsigned nw) {
    const unsigned w = q >> 5, sh = q & 31u;
    const unsigned lo = w < nw ? __ldg(bits + w) : 0u, hi = sh && w + 1 < nw ? __ldg(bits + w + 1) : 0u;
    return __funnelshift_r(lo, hi, sh);
}

// a grid point's edges and cube from the sign bits; the warp's 32 consecutive
// points p0 .. p0+31 share the eight shifted words
struct OB {
    bool in, ex, ey, ez, cube;
    int x, y, z, ci;
};
__device__ __forceinline__ OB oc_point(const OV &g, const unsigned *__restrict__ bits, unsigned p0, int lane) {
    const unsigned nw = (g.NG + 31u) >> 5, NX = (unsigned)g.NX, NXY = g.NXY;
    const unsigned B0 = obits(bits, p0, nw), B1 = obits(bits, p0 + 1, nw), B3 = obits(bits, p0 + NX, nw),
                   B2 = obits(bits, p0 + NX + 1, nw), B4 = obits(bits, p0 + NXY, nw), B5 = obits(bits, p0 + NXY + 1, nw),
                   B7 = obits(bits, p0 + NXY + NX, nw), B6 = obits(bits, p0 + NXY + NX + 1, nw);
    OB q;
    const unsigned p = p0 + (unsigned)lane;
    q.in = p < g.NG;
    q.ex = q.ey = q.ez = q.cube = false;
    q.ci = 0;
    q.x = q.y = q.z = 0;
    if (!q.in) return q;
    q.z = (int)(p / NXY);
    const unsigned r = p - (unsigned)q.z * NXY;
    q.y = (int)(r / NX);
    q.x = (int)(r - (unsigned)q.y * NX);
    const bool hx = q.x < g.NX - 1, hy = q.y < g.NY - 1, hz = q.z < g.NZ - 1;
    const unsigned b0 = (B0 >> lane) & 1u;
    q.ex = hx && ((B1 >> lane) & 1u) != b0;
    q.ey = hy && ((B3 >> lane) & 1u) != b0;
    q.ez = hz && ((B4 >> lane) & 1u) != b0;
    if (hx && hy && hz) {   // Bourke's corner order p0 .. p7
        q.cube = true;
        q.ci = (int)(b0 | ((B1 >> lane) & 1u) << 1 | ((B2 >> lane) & 1u) << 2 | ((B3 >> lane) & 1u) << 3 |
                     ((B4 >> lane) & 1u) << 4 | ((B5 >> lane) & 1u) << 5 | ((B6 >> lane) & 1u) << 6 |
                     ((B7 >> lane) & 1u) << 7);
    }
    return q;
}

__global__ void __launch_bounds__(256) k_oc_count(OV g, const unsigned *__restrict__ bits, uint4 *words, uint4 *counts) {
    const unsigned nw = (g.NG + 31u) >> 5;
    const int lane = threadIdx.x & 31;
    for (unsigned w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; w < nw; w += (gridDim.x * blockDim.x) >> 5) {
        const OB q = oc_point(g, bits, w * 32u, lane);
        int nt = q.cube ? ocube_ntri(q.ci) : 0;
        const unsigned xm = __ballot_sync(0xffffffffu, q.ex), ym = __ballot_sync(0xffffffffu, q.ey),
                       zm = __ballot_sync(0xffffffffu, q.ez);
        for (int o = 16; o; o >>= 1) nt += __shfl_xor_sync(0xffffffffu, nt, o);
        if (lane == 0) {
            words[w] = make_uint4(xm, ym, zm, 0u);
            counts[w] = make_uint4(__popc(xm) + __popc(ym) + __popc(zm), (unsigned)nt, 0u, 0u);
        }
    }
}

__device__ __forceinline__ int ovid(const uint4 *__restrict__ words, const uint4 *__restrict__ offs, unsigned q,
                                    int axis) {
    const unsigned w = q >> 5, l = q & 31u;
    const uint4 m = words[w];
    const unsigned lt = (1u << l) - 1u;
    unsigned id = offs[w].x + __popc(m.x & lt) + __popc(m.y & lt) + __popc(m.z & lt);
    if (axis >= 1) id += (m.x >> l) & 1u;
    if (axis == 2) id += (m.y >> l) & 1u;
    return (int)id;
}

// VertexInterp (src/oldcubes.c:22-40) along one axis: p = p1 + mu*(p2-p1)
// with mu = (iso - v1)/(v2 - v1); only the coordinate along the edge moves.
__device__ __forceinline__ double interp(double iso, double p1, double p2, double v1, double v2) {
    const double mu = __ddiv_rn(__dsub_rn(iso, v1), __dsub_rn(v2, v1));
    return __dadd_rn(p1, __dmul_rn(mu, __dsub_rn(p2, p1)));
}

__global__ void __launch_bounds__(256) k_oc_emit(OV g, const unsigned *__restrict__ bits, const uint4 *__restrict__ words,
                                                 const uint4 *__restrict__ offs, uint4 totals, vec3d *pts, vec3i *tris,
                                                 int *cand, unsigned *ncand, int cap) {
    const unsigned p = blockIdx.x * 256u + threadIdx.x;
    const unsigned w = p >> 5, lane = threadIdx.x & 31u;
    const unsigned nwords = (g.NG + 31u) >> 5;
    if (w >= nwords) return;
    const uint4 o = offs[w];
    const uint4 on = (w + 1 < nwords) ? offs[w + 1] : totals;
    const uint4 m = words[w];
    if ((m.x | m.y | m.z) == 0u && on.y == o.y) return;   // warp-uniform
    const OB b = oc_point(g, bits, w * 32u, (int)lane);
    const double iso = (double)g.iso;
    if (b.ex | b.ey | b.ez) {
        const unsigned lt = (1u << lane) - 1u;
        int id = (int)(o.x + __popc(m.x & lt) + __popc(m.y & lt) + __popc(m.z & lt));
        OP q;   // the values this point's edges interpolate
        q.X = g.lo0 + b.x; q.Y = g.lo1 + b.y; q.Z = g.lo2 + b.z;
        q.ex = b.ex; q.ey = b.ey; q.ez = b.ez;
        q.v[0] = oval(g, q.X, q.Y, q.Z);
        if (q.ex) q.v[1] = oval(g, q.X + 1, q.Y, q.Z);
        if (q.ey) q.v[3] = oval(g, q.X, q.Y + 1, q.Z);
        if (q.ez) q.v[4] = oval(g, q.X, q.Y, q.Z + 1);
        const double X = q.X, Y = q.Y, Z = q.Z;
        const double v0 = q.v[0];
        const int c0 = g.lo0, c1 = g.lo1, c2 = g.lo2, e0 = g.hi0 - 2, e1 = g.hi1 - 2, e2 = g.hi2 - 2;
        if (q.ex) {  // last user: (X,Y,Z) fwd > (X,Y-1,Z) rev > (X,Y,Z-1) fwd > (X,Y-1,Z-1) rev
            const double v1 = q.v[1];
            bool fwd;
            if (q.Y <= e1 && q.Z <= e2) fwd = true;
            else if (q.Y - 1 >= c1 && q.Z <= e2) fwd = false;
            else if (q.Y <= e1 && q.Z - 1 >= c2) fwd = true;
            else fwd = false;
            const double x = fwd ? interp(iso, X, X + 1.0, v0, v1) : interp(iso, X + 1.0, X, v1, v0);
            pts[id] = {x, Y, Z};
            if (fabs(x - rint(x)) < 1.5e-5) { unsigned k = atomicAdd(ncand, 1u); if (k < (unsigned)cap) cand[k] = id; }
            id++;
        }
        if (q.ey) {  // (X,Y,Z) rev > (X-1,Y,Z) fwd > (X,Y,Z-1) rev > (X-1,Y,Z-1) fwd
            const double v3 = q.v[3];
            bool fwd;
            if (q.X <= e0 && q.Z <= e2) fwd = false;
            else if (q.X - 1 >= c0 && q.Z <= e2) fwd = true;
            else if (q.X <= e0 && q.Z - 1 >= c2) fwd = false;
            else fwd = true;
            const double y = fwd ? interp(iso, Y, Y + 1.0, v0, v3) : interp(iso, Y + 1.0, Y, v3, v0);
            pts[id] = {X, y, Z};
            if (fabs(y - rint(y)) < 1.5e-5) { unsigned k = atomicAdd(ncand, 1u); if (k < (unsigned)cap) cand[k] = id; }
            id++;
        }
        if (q.ez) {  // every user lists the z edge bottom to top
            const double z = interp(iso, Z, Z + 1.0, v0, (double)q.v[4]);
            pts[id] = {X, Y, z};
            if (fabs(z - rint(z)) < 1.5e-5) { unsigned k = atomicAdd(ncand, 1u); if (k < (unsigned)cap) cand[k] = id; }
        }
    }
    const int ci = b.ci;
    const int nt = b.cube ? ocube_ntri(ci) : 0;
    int tb = nt;
    for (int d = 1; d < 32; d <<= 1) {
        const int a = __shfl_up_sync(0xffffffffu, tb, d);
        if ((int)lane >= d) tb += a;
    }
    tb -= nt;
    if (nt == 0) return;
    const unsigned NX = (unsigned)g.NX, NXY = g.NXY;
    const long long tri0 = (long long)o.y + tb;
    int tv[3];
    for (int t = 0; t < 3 * nt; t++) {
        int v;
        switch (d_tri[ci * 16 + t]) {   // Bourke edge -> owning grid point and axis
        case 0: v = ovid(words, offs, p, 0); break;
        case 1: v = ovid(words, offs, p + 1, 1); break;
        case 2: v = ovid(words, offs, p + NX, 0); break;
        case 3: v = ovid(words, offs, p, 1); break;
        case 4: v = ovid(words, offs, p + NXY, 0); break;
        case 5: v = ovid(words, offs, p + NXY + 1, 1); break;
        case 6: v = ovid(words, offs, p + NXY + NX, 0); break;
        case 7: v = ovid(words, offs, p + NXY, 1); break;
        case 8: v = ovid(words, offs, p, 2); break;
        case 9: v = ovid(words, offs, p + 1, 2); break;
        case 10: v = ovid(words, offs, p + NX + 1, 2); break;
        default: v = ovid(words, offs, p + NX, 2); break;
        }
        tv[t % 3] = v;
        if (t % 3 == 2) tris[tri0 + t / 3] = {tv[0], tv[1], tv[2]};
    }
}

// weld candidates as a bitmap over the vertices
__global__ void k_oc_candbits(const int *__restrict__ cand, unsigned ncand, unsigned *bits) {
    for (unsigned i = blockIdx.x * blockDim.x + threadIdx.x; i < ncand; i += gridDim.x * blockDim.x) {
        const unsigned v = (unsigned)cand[i];
        atomicOr(bits + (v >> 5), 1u << (v & 31u));
    }
}

// last copy of every candidate vertex: the largest 3*triangle + corner that names it
__global__ void k_oc_lastuse(const vec3i *__restrict__ tris, unsigned nt, const unsigned *__restrict__ bits,
                             long long *lastuse) {
    for (unsigned t = blockIdx.x * blockDim.x + threadIdx.x; t < nt; t += gridDim.x * blockDim.x) {
        const vec3i T = tris[t];
        const int v[3] = {T.x, T.y, T.z};
#pragma unroll
        for (int c = 0; c < 3; c++)
            if ((__ldg(bits + ((unsigned)v[c] >> 5)) >> ((unsigned)v[c] & 31u)) & 1u)
                atomicMax(&lastuse[v[c]], 3ll * t + c);
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
    g.iso = iso;
    g.edge_max = edge_max;
    return g;
}
}  // namespace

n2m_status oc_count(const float *vol, const int dim[3], const int lo[3], const int hi[3], float iso,
                     float edge_max, McWork &w, ScanWork &sw, uint4 *d_total, cudaStream_t s) {
    const OV g = make_ov(vol, dim, lo, hi, iso, edge_max);
    if (g.NX < 2 || g.NY < 2 || g.NZ < 2) {
        CK(cudaMemsetAsync(d_total, 0, sizeof(uint4), s));
        return N2M_OK;
    }
    const size_t nwords = ((size_t)g.NG + 31) / 32;
    CKS(w.words.ensure(nwords * sizeof(uint4)));
    CKS(w.counts.ensure(nwords * sizeof(uint4)));
    CKS(w.signs.ensure(nwords * sizeof(unsigned)));
    const unsigned blocks = (unsigned)std::min<size_t>((nwords + 7) / 8, 152u * 16u);   // a warp per word
    { k_oc_signs<<<blocks, 256, 0, s>>>(g, w.signs.as<unsigned>()); N2M_COUNT(); }
    { k_oc_count<<<blocks, 256, 0, s>>>(g, w.signs.as<unsigned>(), w.words.as<uint4>(), w.counts.as<uint4>()); N2M_COUNT(); }
    CKL();
    return scan_uint4(w.counts.as<uint4>(), nwords, d_total, sw, s);
}

n2m_status oc_emit(const float *vol, const int dim[3], const int lo[3], const int hi[3], float iso, float edge_max,
                    McWork &w, const McCounts &c, vec3d *d_pts, vec3i *d_tris, int *d_cand, unsigned *d_ncand,
                    int cand_cap, cudaStream_t s) {
    const OV g = make_ov(vol, dim, lo, hi, iso, edge_max);
    { k_oc_emit<<<(unsigned)(((size_t)g.NG + 255) / 256), 256, 0, s>>>(g, w.signs.as<unsigned>(), w.words.as<uint4>(), w.counts.as<uint4>(),
                                                                     make_uint4(c.nv_edge, c.nt, 0, 0), d_pts, d_tris,
                                                                     d_cand, d_ncand, cand_cap); N2M_COUNT(); }
    CKL();
    return N2M_OK;
}

n2m_status oc_lastuse(const vec3i *d_tris, int nt, int nv, const int *d_cand, int ncand, unsigned *d_bits,
                      long long *d_lastuse, cudaStream_t s) {
    CK(cudaMemsetAsync(d_bits, 0, (size_t)(nv + 31) / 32 * sizeof(unsigned), s));
    { k_oc_candbits<<<(unsigned)std::max(1, std::min((ncand + 255) / 256, 1024)), 256, 0, s>>>(d_cand, (unsigned)ncand, d_bits); N2M_COUNT(); }
    { k_oc_lastuse<<<(unsigned)std::max(1, std::min((nt + 255) / 256, 152 * 16)), 256, 0, s>>>(d_tris, (unsigned)nt, d_bits, d_lastuse); N2M_COUNT(); }
    CKL();
    return N2M_OK;
}
