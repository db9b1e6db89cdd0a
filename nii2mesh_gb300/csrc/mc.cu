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
// count pass: one thread per grid point; a warp covers 32 consecutive points
//   (a "word").  Edge crossings are ballots (three 32-bit masks per word);
//   triangle and c-vertex counts come from the cube's MC33 decision.
// scan: exclusive scan over words -> vertex/triangle/c-vertex offsets.
// emit pass: only words that own output recompute their cubes; an edge
//   vertex id anywhere in the grid is offset(word) + popcounts of the word's
//   masks below the lane, so every edge is emitted exactly once (this replaces
//   the reference's vertex weld for shared edges).
// Vertices whose final coordinates sit within 1.5e-5 of a grid point (edge
// vertices) or of a grid plane (c-vertices) are recorded as weld candidates:
// only such vertices can lie within the weld tolerance (1e-5) of another.
#include <float.h>

#include <algorithm>

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
        int vx = g.lo0 + x, vy = y + g.lo1, vz = z + g.lo2;
        if (vx >= g.dx || vy >= g.dy) {
            vz = (int)(j / g.dxy);
            const long long r = j - (long long)vz * g.dxy;
            vy = (int)(r / g.dx);
            vx = (int)(r - (long long)vy * g.dx);
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
constexpr int TY = 8, TZ = 8;          // a CTA covers one word column x 8 rows x 8 slices

__global__ void __launch_bounds__(256) k_count(GV g, bool classic, unsigned WX, uint4 *words, uint4 *counts,
                                               unsigned *active, unsigned *nactive) {
    __shared__ float sv[TZ + 1][TY + 1][33];
    const int x0 = blockIdx.x * 32, y0 = blockIdx.y * TY, z0 = blockIdx.z * TZ;
    // tile and halo strictly inside the volume: no darkening, wrap or padding
    const bool simple = g.lo0 + x0 >= 1 && g.lo0 + x0 + 32 <= g.dx - 2 && g.lo1 + y0 >= 1 &&
                        g.lo1 + y0 + TY <= g.dy - 2 && g.lo2 + z0 >= 1 && g.lo2 + z0 + TZ <= g.dz - 2;
    for (int i = threadIdx.x; i < (TZ + 1) * (TY + 1) * 33; i += 256) {
        const int xx = i % 33, r = i / 33, yy = r % (TY + 1), zz = r / (TY + 1);
        float v;
        if (simple) {
            const unsigned j = (unsigned)(g.lo0 + x0 + xx) + (unsigned)(y0 + yy + g.lo1) * (unsigned)g.dx +
                               (unsigned)(z0 + zz + g.lo2) * (unsigned)g.dxy;
            v = __fsub_rn(__ldg(g.vol + j), g.iso);
            if (fabsf(v) < N2M_FLT_EPS) v = N2M_FLT_EPS;
        } else {
            v = gval(g, x0 + xx, y0 + yy, z0 + zz);
        }
        sv[zz][yy][xx] = v;
    }
    __syncthreads();
    const int wy = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int y = y0 + wy, x = x0 + lane;
    if (y >= g.NY) return;                           // whole warp
    for (int zz = 0; zz < TZ; zz++) {
        const int z = z0 + zz;
        if (z >= g.NZ) break;                        // whole warp
        const bool in = x < g.NX;
        const bool hx = in && x < g.NX - 1, hy = in && y < g.NY - 1, hz = in && z < g.NZ - 1;
        const float c0 = sv[zz][wy][lane];
        const bool s0 = c0 > 0.f;
        const bool ex = hx && ((sv[zz][wy][lane + 1] > 0.f) != s0);
        const bool ey = hy && ((sv[zz][wy + 1][lane] > 0.f) != s0);
        const bool ez = hz && ((sv[zz + 1][wy][lane] > 0.f) != s0);
        int nt = 0, nc = 0;
        if (hx && hy && hz) {
            float c[8] = {c0, sv[zz][wy][lane + 1], sv[zz][wy + 1][lane + 1], sv[zz][wy + 1][lane],
                          sv[zz + 1][wy][lane], sv[zz + 1][wy][lane + 1], sv[zz + 1][wy + 1][lane + 1],
                          sv[zz + 1][wy + 1][lane]};
            const int lut = cube_lut(c);
            if (lut != 0 && lut != 255) {
                const Tiling T = select_tiling(c, lut, classic);
                nt = T.n;
                nc = T.cv;
            }
        }
        const unsigned xm = __ballot_sync(0xffffffffu, ex), ym = __ballot_sync(0xffffffffu, ey),
                       zm = __ballot_sync(0xffffffffu, ez);
        for (int o = 16; o; o >>= 1) {
            nt += __shfl_xor_sync(0xffffffffu, nt, o);
            nc += __shfl_xor_sync(0xffffffffu, nc, o);
        }
        if (lane == 0) {
            const unsigned w = ((unsigned)z * (unsigned)g.NY + (unsigned)y) * WX + blockIdx.x;
            const unsigned nv = __popc(xm) + __popc(ym) + __popc(zm);
            const bool act = nv | nt | nc;
            words[w] = make_uint4(xm, ym, zm, 0u);
            counts[w] = make_uint4(nv, (unsigned)nt, (unsigned)nc, act);
            if (act) active[atomicAdd(nactive, 1u)] = w;
        }
    }
}

// ---- emit pass -------------------------------------------------------------------
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

// one warp per active word
__global__ void __launch_bounds__(256) k_emit(GV g, bool classic, unsigned WX, const uint4 *__restrict__ words,
                                              const uint4 *__restrict__ offs, const unsigned *__restrict__ active,
                                              unsigned nactive, unsigned nwords, uint4 totals, vec3d *pts,
                                              vec3i *tris, int *cand, unsigned *ncand, int *ccand, unsigned *nccand,
                                              int cap) {
    const unsigned lane = threadIdx.x & 31u;
    const float flo0 = (float)g.lo0, flo1 = (float)g.lo1, flo2 = (float)g.lo2;
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
        if (in) {
            c[0] = gval(g, x, y, z);
            c[1] = hx ? gval(g, x + 1, y, z) : c[0];
            c[3] = hy ? gval(g, x, y + 1, z) : c[0];
            c[4] = hz ? gval(g, x, y, z + 1) : c[0];
            if (cube) {
                c[2] = gval(g, x + 1, y + 1, z);
                c[5] = gval(g, x + 1, y, z + 1);
                c[6] = gval(g, x + 1, y + 1, z + 1);
                c[7] = gval(g, x, y + 1, z + 1);
            }
        }
        // edge vertices owned by this point (src/MarchingCubes.c:935-1026)
        if (ex | ey | ez) {
            const unsigned lt = (1u << lane) - 1u;
            int id = (int)(o.x + __popc(m.x & lt) + __popc(m.y & lt) + __popc(m.z & lt));
            const float fx = (float)x, fy = (float)y, fz = (float)z;
            if (ex) {
                const float X = __fadd_rn(__fadd_rn(fx, edge_u(c[0], c[1])), flo0);
                pts[id] = {(double)X, (double)__fadd_rn(fy, flo1), (double)__fadd_rn(fz, flo2)};
                if (frac_dist(X) < 1.5e-5f) add_cand(cand, ncand, cap, id);
                id++;
            }
            if (ey) {
                const float Y = __fadd_rn(__fadd_rn(fy, edge_u(c[0], c[3])), flo1);
                pts[id] = {(double)__fadd_rn(fx, flo0), (double)Y, (double)__fadd_rn(fz, flo2)};
                if (frac_dist(Y) < 1.5e-5f) add_cand(cand, ncand, cap, id);
                id++;
            }
            if (ez) {
                const float Z = __fadd_rn(__fadd_rn(fz, edge_u(c[0], c[4])), flo2);
                pts[id] = {(double)__fadd_rn(fx, flo0), (double)__fadd_rn(fy, flo1), (double)Z};
                if (frac_dist(Z) < 1.5e-5f) add_cand(cand, ncand, cap, id);
            }
        }
        Tiling T = {0, 0, false};
        if (cube) {
            const int lut = cube_lut(c);
            if (lut != 0 && lut != 255) T = select_tiling(c, lut, classic);
        }
        int tb = T.n, cb = T.cv;   // warp exclusive scans
        for (int d = 1; d < 32; d <<= 1) {
            const int a = __shfl_up_sync(0xffffffffu, tb, d), b = __shfl_up_sync(0xffffffffu, cb, d);
            if ((int)lane >= d) { tb += a; cb += b; }
        }
        tb -= T.n;
        cb -= T.cv;
        if (T.n == 0) continue;
        int v12 = -1;
        if (T.cv) {   // c-vertex: mean of the cube's edge vertices (src/MarchingCubes.c:1029-1082)
            v12 = (int)(totals.x + o.z + cb);
            float n = 0.f, sx = 0.f, sy = 0.f, sz = 0.f;
            for (int e = 0; e < 12; e++) {
                const int own = k_edge[e][0], ax = k_edge[e][1], ca = k_edge[e][2], cbn = k_edge[e][3];
                if ((c[ca] > 0.f) == (c[cbn] > 0.f)) continue;
                const float u = edge_u(c[ca], c[cbn]);
                float px = (float)(x + ((own ^ (own >> 1)) & 1)), py = (float)(y + ((own >> 1) & 1)),
                      pz = (float)(z + ((own >> 2) & 1));
                if (ax == 0) px = __fadd_rn(px, u);
                else if (ax == 1) py = __fadd_rn(py, u);
                else pz = __fadd_rn(pz, u);
                n = __fadd_rn(n, 1.f);
                sx = __fadd_rn(sx, px); sy = __fadd_rn(sy, py); sz = __fadd_rn(sz, pz);
            }
            if (n > 0.f) { sx = __fdiv_rn(sx, n); sy = __fdiv_rn(sy, n); sz = __fdiv_rn(sz, n); }
            const float X = __fadd_rn(sx, flo0), Y = __fadd_rn(sy, flo1), Z = __fadd_rn(sz, flo2);
            pts[v12] = {(double)X, (double)Y, (double)Z};
            if (fminf(frac_dist(X), fminf(frac_dist(Y), frac_dist(Z))) < 1.5e-5f) add_cand(ccand, nccand, cap, v12);
        }
        // triangles, stored reversed (v3,v2,v1) as marchingCubes() returns them
        const unsigned NY = (unsigned)g.NY;
        int tv[3];
        for (int t = 0; t < 3 * T.n; t++) {
            const int code = d_lut[T.off + t];
            int v;
            switch (code) {
            case 0: v = vid(words, offs, NY, WX, x, y, z, 0); break;
            case 1: v = vid(words, offs, NY, WX, x + 1, y, z, 1); break;
            case 2: v = vid(words, offs, NY, WX, x, y + 1, z, 0); break;
            case 3: v = vid(words, offs, NY, WX, x, y, z, 1); break;
            case 4: v = vid(words, offs, NY, WX, x, y, z + 1, 0); break;
            case 5: v = vid(words, offs, NY, WX, x + 1, y, z + 1, 1); break;
            case 6: v = vid(words, offs, NY, WX, x, y + 1, z + 1, 0); break;
            case 7: v = vid(words, offs, NY, WX, x, y, z + 1, 1); break;
            case 8: v = vid(words, offs, NY, WX, x, y, z, 2); break;
            case 9: v = vid(words, offs, NY, WX, x + 1, y, z, 2); break;
            case 10: v = vid(words, offs, NY, WX, x + 1, y + 1, z, 2); break;
            case 11: v = vid(words, offs, NY, WX, x, y + 1, z, 2); break;
            case 12: v = v12; break;
            default: v = -1; break;
            }
            tv[t % 3] = v;
            if (t % 3 == 2) tris[o.y + tb + t / 3] = {tv[2], tv[1], tv[0]};
        }
    }
    (void)nwords;
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
        int vx = g.lo0 + x, vy = y + g.lo1, vz = z + g.lo2;
        if (vx >= g.dx || vy >= g.dy) {
            vz = (int)(j / g.dxy);
            const long long r = j - (long long)vz * g.dxy;
            vy = (int)(r / g.dx);
            vx = (int)(r - (long long)vy * g.dx);
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
n2m_status mc_count(const McGrid &g, int variant, McWork &w, ScanWork &sw, uint4 *d_total, cudaStream_t s) {
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
    unsigned *active = w.cand.as<unsigned>();
    CK(cudaMemsetAsync(active + nwords, 0, sizeof(unsigned), s));
    dim3 grid(WX, (g.n[1] + TY - 1) / TY, (g.n[2] + TZ - 1) / TZ);
    { k_count<<<grid, 256, 0, s>>>(v, variant == N2M_CUBES_CLASSIC_TABLE, WX, w.words.as<uint4>(), w.counts.as<uint4>(), active, active + nwords); N2M_COUNT(); }
    CKL();
    return scan_uint4(w.counts.as<uint4>(), nwords, d_total, sw, s);
}

n2m_status mc_emit(const McGrid &g, int variant, McWork &w, const McCounts &c, vec3d *d_pts, vec3i *d_tris,
                   int *d_cand, unsigned *d_ncand, int cand_cap, cudaStream_t s) {
    const GV v = make_gv(g);
    const unsigned WX = (unsigned)((g.n[0] + 31) / 32);
    const size_t nwords = (size_t)WX * g.n[1] * g.n[2];
    const unsigned nact = c.nactive;
    if (nact == 0) return N2M_OK;
    const unsigned blocks = std::min<unsigned>((nact + 7) / 8, 152u * 16u);
    { k_emit<<<blocks, 256, 0, s>>>(v, variant == N2M_CUBES_CLASSIC_TABLE, WX, w.words.as<uint4>(), w.counts.as<uint4>(), w.cand.as<unsigned>(), nact, (unsigned)nwords, make_uint4(c.nv_edge, c.nt, c.nc, 0), d_pts, d_tris, d_cand, d_ncand, d_cand + cand_cap, d_ncand + 1, cand_cap); N2M_COUNT(); }
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
