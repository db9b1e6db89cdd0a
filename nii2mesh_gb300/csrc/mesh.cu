// mesh.cu — per-mesh stages after marching cubes:
//   * weld fix-up (src/meshify.c:45-106): applies the merges the host decided
//     for the few near-grid-point candidates (vertex compaction + remap);
//   * remove_degenerate_triangles (src/meshify.c:113-168): FP32 area filter
//     with a rigorous error margin, the reference's FP64 predicate for the
//     rest, stable compaction;
//   * the weld's adjoint (a welded vertex's gradient back to its raw vertex);
//   * apply_sform (src/meshify.c:1021-1045).
// laplacian_smoothHC is in hc.cu.
#include <float.h>

#include "n2m_internal.cuh"

namespace {
// ---- weld -------------------------------------------------------------------
__device__ __forceinline__ int lower_bound(const int *a, int n, int v) {
    int lo = 0, hi = n;
    while (lo < hi) {
        const int m = (lo + hi) >> 1;
        if (a[m] < v) lo = m + 1;
        else hi = m;
    }
    return lo;
}

// removed[k] (sorted) merges into keep[k]; override ids (sorted) take pos.
__global__ void k_weld_verts(const vec3d *__restrict__ in, int np, const int *__restrict__ removed, int nrem,
                             const int *__restrict__ ov_id, const vec3d *__restrict__ ov_pos, int nov,
                             vec3d *__restrict__ out) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < np; i += gridDim.x * blockDim.x) {
        const int r = lower_bound(removed, nrem, i);
        if (r < nrem && removed[r] == i) continue;
        const int o = lower_bound(ov_id, nov, i);
        out[i - r] = (o < nov && ov_id[o] == i) ? ov_pos[o] : in[i];
    }
}

__global__ void k_weld_tris(vec3i *t, int nt, const int *__restrict__ removed, const int *__restrict__ keep,
                            int nrem) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nt; i += gridDim.x * blockDim.x) {
        int v[3] = {t[i].x, t[i].y, t[i].z};
        for (int k = 0; k < 3; k++) {
            int r = lower_bound(removed, nrem, v[k]);
            if (r < nrem && removed[r] == v[k]) {
                v[k] = keep[r];
                r = lower_bound(removed, nrem, v[k]);
            }
            v[k] -= r;
        }
        t[i] = {v[0], v[1], v[2]};
    }
}

// ---- degenerate triangles --------------------------------------------------------
__device__ __forceinline__ double dist_d(vec3d a, vec3d b) {
    const double dx = __dsub_rn(a.x, b.x), dy = __dsub_rn(a.y, b.y), dz = __dsub_rn(a.z, b.z);
    return __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz)));
}

// the reference predicate, operation for operation (src/meshify.c:119-144)
__device__ bool degenerate_ref(vec3d A, vec3d B, vec3d C) {
    const double l = dist_d(A, B), m = dist_d(A, C), n = dist_d(B, C);
    const double c = fmin(fmin(l, m), n), a = fmax(fmax(l, m), n);
    const double b = __dsub_rn(__dsub_rn(__dadd_rn(__dadd_rn(l, m), n), a), c);
    const double cab = __dsub_rn(c, __dsub_rn(a, b));
    if (cab <= 0.0) return true;
    const double q = __dmul_rn(__dmul_rn(__dmul_rn(__dadd_rn(a, __dadd_rn(b, c)), cab), __dadd_rn(c, __dsub_rn(a, b))),
                               __dadd_rn(a, __dsub_rn(b, c)));
    return __dmul_rn(0.25, __dsqrt_rn(q)) < (double)FLT_EPSILON;
}

// True iff the triangle is degenerate under the reference predicate.  Fast
// path: the area from an FP32 cross product of (double) edge vectors, minus a
// bound on its rounding error, exceeding 4e-7 (> 3x FLT_EPSILON) proves the
// triangle is kept.
// float value of d if d is exactly a float (zero or normal), by bit assembly:
// the F2F conversion issues on the FP64 pipe, a small fraction of the integer
// rate on this part
__device__ __forceinline__ bool d2f_exact(double d, float &f) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(d);
    const unsigned e = (unsigned)(b >> 52) & 0x7ffu;
    const unsigned long long m = b & 0xfffffffffffffull;
    const unsigned sign = (unsigned)(b >> 32) & 0x80000000u;
    if (e == 0 && m == 0) { f = __uint_as_float(sign); return true; }
    if ((m & 0x1fffffffull) || e < 897u || e > 1150u) return false;   // low bits set or outside the normal float range
    f = __uint_as_float(sign | ((e - 896u) << 23) | (unsigned)(m >> 29));
    return true;
}

__device__ __forceinline__ bool degenerate(vec3d A, vec3d B, vec3d C) {
    float ax, ay, az, bx, by, bz, qx, qy, qz;
    float ux, uy, uz, vx, vy, vz;
    if (d2f_exact(A.x, ax) & d2f_exact(A.y, ay) & d2f_exact(A.z, az) & d2f_exact(B.x, bx) & d2f_exact(B.y, by) &
        d2f_exact(B.z, bz) & d2f_exact(C.x, qx) & d2f_exact(C.y, qy) & d2f_exact(C.z, qz)) {
        // float coordinates: the FP32 difference is the double difference rounded to float
        ux = bx - ax; uy = by - ay; uz = bz - az;
        vx = qx - ax; vy = qy - ay; vz = qz - az;
    } else {
        ux = (float)(B.x - A.x); uy = (float)(B.y - A.y); uz = (float)(B.z - A.z);
        vx = (float)(C.x - A.x); vy = (float)(C.y - A.y); vz = (float)(C.z - A.z);
    }
    const float cx = uy * vz - uz * vy, cy = uz * vx - ux * vz, cz = ux * vy - uy * vx;
    const float cr = sqrtf(cx * cx + cy * cy + cz * cz);
    const float nu = sqrtf(ux * ux + uy * uy + uz * uz), nv = sqrtf(vx * vx + vy * vy + vz * vz);
    if (0.5f * (cr - 1e-6f * nu * nv) > 4e-7f && isfinite(cr)) return false;
    return degenerate_ref(A, B, C);
}

constexpr int CB = 256;   // compaction tile = one CTA

__global__ void __launch_bounds__(CB) k_deg_count(const vec3d *__restrict__ p, const vec3i *__restrict__ t, int nt,
                                                  unsigned *keep, unsigned *tile_cnt) {
    const int i = blockIdx.x * CB + threadIdx.x;
    unsigned k = 0;
    if (i < nt) {
        const vec3i T = t[i];
        k = !degenerate(p[T.x], p[T.y], p[T.z]);
        keep[i] = k;
    }
    k = __syncthreads_count(k);
    if (threadIdx.x == 0) tile_cnt[blockIdx.x] = k;
}

__global__ void __launch_bounds__(CB) k_deg_compact(const vec3i *__restrict__ t, int nt, const unsigned *keep,
                                                    const unsigned *tile_off, vec3i *out) {
    __shared__ unsigned wcnt[CB / 32];
    const int i = blockIdx.x * CB + threadIdx.x;
    const unsigned k = i < nt ? keep[i] : 0u;
    const unsigned b = __ballot_sync(0xffffffffu, k);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) wcnt[wid] = __popc(b);
    __syncthreads();
    unsigned off = tile_off[blockIdx.x];
    for (int w = 0; w < wid; w++) off += wcnt[w];
    if (k) out[off + __popc(b & ((1u << lane) - 1u))] = t[i];
}

// raw vertex gradient: every kept raw vertex receives its welded vertex's
// gradient, except that a merged group's gradient goes to the member whose
// position it kept
__global__ void k_weld_back(const float3 *__restrict__ go, int nv_raw, const int *__restrict__ removed, int nrem,
                            const int *__restrict__ ov_id, const int *__restrict__ ov_src, int nov, float3 *graw) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nv_raw; i += gridDim.x * blockDim.x) {
        const int r = lower_bound(removed, nrem, i);
        if (r < nrem && removed[r] == i) continue;
        const int o = lower_bound(ov_id, nov, i);
        const int src = (o < nov && ov_id[o] == i) ? ov_src[o] : i;
        const float3 g = go[i - r];
        atomicAdd(&graw[src].x, g.x);
        atomicAdd(&graw[src].y, g.y);
        atomicAdd(&graw[src].z, g.z);
    }
}

__global__ void k_sform(vec3d *p, int np, double a0, double a1, double a2, double a3, double b0, double b1, double b2,
                        double b3, double c0, double c1, double c2, double c3) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < np; i += gridDim.x * blockDim.x) {
        const vec3d v = p[i];
        p[i].x = __dadd_rn(__dadd_rn(__dadd_rn(__dmul_rn(v.x, a0), __dmul_rn(v.y, a1)), __dmul_rn(v.z, a2)), a3);
        p[i].y = __dadd_rn(__dadd_rn(__dadd_rn(__dmul_rn(v.x, b0), __dmul_rn(v.y, b1)), __dmul_rn(v.z, b2)), b3);
        p[i].z = __dadd_rn(__dadd_rn(__dadd_rn(__dmul_rn(v.x, c0), __dmul_rn(v.y, c1)), __dmul_rn(v.z, c2)), c3);
    }
}

__global__ void k_flip(vec3i *t, int nt) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nt; i += gridDim.x * blockDim.x) {
        const int x = t[i].x;
        t[i].x = t[i].y;
        t[i].y = x;
    }
}

inline unsigned gs(size_t n) {
    size_t b = (n + 255) / 256;
    if (b > 152 * 32) b = 152 * 32;
    return b ? (unsigned)b : 1u;
}
}  // namespace

n2m_status mesh_apply_weld(vec3d *d_pts, vec3i *d_tris, int np, int nt, const int *d_removed, const int *d_keep,
                           int nrem, const int *d_ov_id, const vec3d *d_ov_pos, int nov, vec3d *d_out,
                           cudaStream_t s) {
    { k_weld_verts<<<gs(np), 256, 0, s>>>(d_pts, np, d_removed, nrem, d_ov_id, d_ov_pos, nov, d_out); N2M_COUNT(); }
    { k_weld_tris<<<gs(nt), 256, 0, s>>>(d_tris, nt, d_removed, d_keep, nrem); N2M_COUNT(); }
    CKL();
    return N2M_OK;
}

n2m_status mesh_remove_degenerate(const vec3d *d_pts, const vec3i *d_tris_in, int nt, vec3i *d_tris_out,
                                  unsigned *d_nt_out, DegWork &w, ScanWork &sw, cudaStream_t s) {
    const int tiles = (nt + CB - 1) / CB;
    if (nt == 0) {
        CK(cudaMemsetAsync(d_nt_out, 0, sizeof(unsigned), s));
        return N2M_OK;
    }
    CKS(w.flags.ensure((size_t)nt * sizeof(unsigned)));
    CKS(w.tmp.ensure((size_t)tiles * sizeof(unsigned)));
    { k_deg_count<<<tiles, CB, 0, s>>>(d_pts, d_tris_in, nt, w.flags.as<unsigned>(), w.tmp.as<unsigned>()); N2M_COUNT(); }
    CKL();
    CKS(scan_u32(w.tmp.as<unsigned>(), tiles, d_nt_out, sw, s));
    { k_deg_compact<<<tiles, CB, 0, s>>>(d_tris_in, nt, w.flags.as<unsigned>(), w.tmp.as<unsigned>(), d_tris_out); N2M_COUNT(); }
    CKL();
    return N2M_OK;
}

n2m_status mesh_weld_backward(const float3 *d_go, int np_final, int nv_raw, const int *d_removed, int nrem,
                              const int *d_ov_id, const int *d_ov_src, int nov, float3 *d_graw, cudaStream_t s) {
    CK(cudaMemsetAsync(d_graw, 0, (size_t)nv_raw * sizeof(float3), s));
    { k_weld_back<<<gs(nv_raw), 256, 0, s>>>(d_go, nv_raw, d_removed, nrem, d_ov_id, d_ov_src, nov, d_graw); N2M_COUNT(); }
    CKL();
    (void)np_final;
    return N2M_OK;
}

n2m_status mesh_apply_sform(vec3d *d_pts, vec3i *d_tris, int np, int nt, const float sx[4], const float sy[4],
                            const float sz[4], cudaStream_t s) {
    { k_sform<<<gs(np), 256, 0, s>>>(d_pts, np, sx[0], sx[1], sx[2], sx[3], sy[0], sy[1], sy[2], sy[3], sz[0], sz[1],
                                   sz[2], sz[3]); N2M_COUNT(); }
    const double px = (double)(sx[0] + sx[1] + sx[2]), py = (double)(sy[0] + sy[1] + sy[2]),
                 pz = (double)(sz[0] + sz[1] + sz[2]);
    const float det = (float)(px * py * pz);
    if (det < 0.0) { k_flip<<<gs(nt), 256, 0, s>>>(d_tris, nt); N2M_COUNT(); }
    CKL();
    return N2M_OK;
}

