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
// post-weld positions bit for bit.  d_lastuse records, per vertex, the index
// of its last copy in the reference's pre-weld vertex list (3*triangle +
// corner) so that near-corner clusters keep the same survivor.
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
    bool in, ex, ey, ez, cube;
    int X, Y, Z;         // absolute point
    float v[8];          // corners in Bourke order: p0..p7
};

__device__ __forceinline__ void oclassify(const OV &g, unsigned p, OP &q) {
    q.in = p < g.NG;
    q.ex = q.ey = q.ez = q.cube = false;
    if (!q.in) return;
    const int z = (int)(p / g.NXY);
    const unsigned r = p - (unsigned)z * g.NXY;
    const int y = (int)(r / (unsigned)g.NX), x = (int)(r - (unsigned)y * (unsigned)g.NX);
    q.X = g.lo0 + x; q.Y = g.lo1 + y; q.Z = g.lo2 + z;
    const bool hx = x < g.NX - 1, hy = y < g.NY - 1, hz = z < g.NZ - 1;
    q.v[0] = oval(g, q.X, q.Y, q.Z);
    q.v[1] = hx ? oval(g, q.X + 1, q.Y, q.Z) : q.v[0];
    q.v[3] = hy ? oval(g, q.X, q.Y + 1, q.Z) : q.v[0];
    q.v[4] = hz ? oval(g, q.X, q.Y, q.Z + 1) : q.v[0];
    const bool b0 = q.v[0] < g.iso;
    q.ex = hx && ((q.v[1] < g.iso) != b0);
    q.ey = hy && ((q.v[3] < g.iso) != b0);
    q.ez = hz && ((q.v[4] < g.iso) != b0);
    if (hx && hy && hz) {
        q.cube = true;
        q.v[2] = oval(g, q.X + 1, q.Y + 1, q.Z);
        q.v[5] = oval(g, q.X + 1, q.Y, q.Z + 1);
        q.v[6] = oval(g, q.X + 1, q.Y + 1, q.Z + 1);
        q.v[7] = oval(g, q.X, q.Y + 1, q.Z + 1);
    }
}

__device__ __forceinline__ int ocube_index(const OP &q, float iso) {
    int ci = 0;
    for (int c = 0; c < 8; c++) ci |= (q.v[c] < iso) << c;
    return ci;
}

__device__ __forceinline__ int ocube_ntri(int ci) {
    if (!d_edge[ci]) return 0;
    int n = 0;
    while (n < 5 && d_tri[ci * 16 + 3 * n] != -1) n++;
    return n;
}

__global__ void __launch_bounds__(256) k_oc_count(OV g, uint4 *words, uint4 *counts) {
    const unsigned p = blockIdx.x * 256u + threadIdx.x;
    OP q;
    oclassify(g, p, q);
    int nt = q.cube ? ocube_ntri(ocube_index(q, g.iso)) : 0;
    const unsigned xm = __ballot_sync(0xffffffffu, q.ex), ym = __ballot_sync(0xffffffffu, q.ey),
                   zm = __ballot_sync(0xffffffffu, q.ez);
    for (int o = 16; o; o >>= 1) nt += __shfl_xor_sync(0xffffffffu, nt, o);
    const unsigned w = p >> 5;
    if ((threadIdx.x & 31) == 0 && w * 32u < g.NG) {
        words[w] = make_uint4(xm, ym, zm, 0u);
        counts[w] = make_uint4(__popc(xm) + __popc(ym) + __popc(zm), (unsigned)nt, 0u, 0u);
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

__global__ void __launch_bounds__(256) k_oc_emit(OV g, const uint4 *__restrict__ words, const uint4 *__restrict__ offs,
                                                 uint4 totals, vec3d *pts, vec3i *tris, int *cand, unsigned *ncand,
                                                 int cap, long long *lastuse) {
    const unsigned p = blockIdx.x * 256u + threadIdx.x;
    const unsigned w = p >> 5, lane = threadIdx.x & 31u;
    const unsigned nwords = (g.NG + 31u) >> 5;
    if (w >= nwords) return;
    const uint4 o = offs[w];
    const uint4 on = (w + 1 < nwords) ? offs[w + 1] : totals;
    const uint4 m = words[w];
    if ((m.x | m.y | m.z) == 0u && on.y == o.y) return;
    OP q;
    oclassify(g, p, q);
    const double iso = (double)g.iso;
    if (q.ex | q.ey | q.ez) {
        const unsigned lt = (1u << lane) - 1u;
        int id = (int)(o.x + __popc(m.x & lt) + __popc(m.y & lt) + __popc(m.z & lt));
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
    int nt = 0, ci = 0;
    if (q.cube) {
        ci = ocube_index(q, g.iso);
        nt = ocube_ntri(ci);
    }
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
        atomicMax(&lastuse[v], 3 * tri0 + t);
        if (t % 3 == 2) tris[tri0 + t / 3] = {tv[0], tv[1], tv[2]};
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
    { k_oc_count<<<(unsigned)(((size_t)g.NG + 255) / 256), 256, 0, s>>>(g, w.words.as<uint4>(), w.counts.as<uint4>()); N2M_COUNT(); }
    CKL();
    return scan_uint4(w.counts.as<uint4>(), nwords, d_total, sw, s);
}

n2m_status oc_emit(const float *vol, const int dim[3], const int lo[3], const int hi[3], float iso, float edge_max,
                    McWork &w, const McCounts &c, vec3d *d_pts, vec3i *d_tris, int *d_cand, unsigned *d_ncand,
                    int cand_cap, long long *d_lastuse, cudaStream_t s) {
    const OV g = make_ov(vol, dim, lo, hi, iso, edge_max);
    { k_oc_emit<<<(unsigned)(((size_t)g.NG + 255) / 256), 256, 0, s>>>(g, w.words.as<uint4>(), w.counts.as<uint4>(),
                                                                     make_uint4(c.nv_edge, c.nt, 0, 0), d_pts, d_tris,
                                                                     d_cand, d_ncand, cand_cap, d_lastuse); N2M_COUNT(); }
    CKL();
    return N2M_OK;
}
