// hc.cu — laplacian_smoothHC (src/quadric.c:316-394) and its adjoint: CSR
// gather kernels in FP32 on displacements from the original positions (HC is
// affine-equivariant); border vertices (update_mesh(0), src/quadric.c:184-212)
// keep their input.  The results are compared within a tolerance with the
// reference's FP64 smoothing, so this unit is compiled with FMA contraction
// (the units with bit-exact duties are not).  Also the allocation-free entry
// point n2m_smooth_hc_noalloc.
#include <float.h>

#include "n2m_internal.cuh"

namespace {
inline unsigned gs(size_t n) {
    size_t b = (n + 255) / 256;
    if (b > 152 * 32) b = 152 * 32;
    return b ? (unsigned)b : 1u;
}

// ---- HC smoothing ----------------------------------------------------------------
// A triangle with an index outside [0, np) is skipped here and in k_fill_refs
// (so it never enters the CSR and nothing downstream reads past the vertex
// arrays) and raises *bad; k_hc_out then leaves every vertex untouched and the
// entry points report N2M_ERR_BAD_ARGS.
__device__ __forceinline__ bool tri_in_range(const vec3i &T, int np) {
    return (unsigned)T.x < (unsigned)np && (unsigned)T.y < (unsigned)np && (unsigned)T.z < (unsigned)np;
}

__global__ void k_degree(const vec3i *__restrict__ t, int nt, int np, unsigned *deg, unsigned *bad) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nt; i += gridDim.x * blockDim.x) {
        const vec3i T = t[i];
        if (!tri_in_range(T, np)) {
            *bad = 1u;
            continue;
        }
        atomicAdd(&deg[T.x], 1u);
        atomicAdd(&deg[T.y], 1u);
        atomicAdd(&deg[T.z], 1u);
    }
}

__global__ void k_fill_refs(const vec3i *__restrict__ t, int nt, int np, const unsigned *__restrict__ start,
                            unsigned *fill, int *refs) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nt; i += gridDim.x * blockDim.x) {
        const vec3i T = t[i];
        if (!tri_in_range(T, np)) continue;
        const int v[3] = {T.x, T.y, T.z};
        for (int s = 0; s < 3; s++) refs[start[v[s]] + atomicAdd(&fill[v[s]], 1u)] = 3 * i + s;
    }
}

// order each vertex's (triangle, slot) references as the reference visits them
__global__ void k_sort_refs(const unsigned *__restrict__ start, int np, int *refs) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < np; i += gridDim.x * blockDim.x) {
        const int a = (int)start[i], b = (int)start[i + 1];
        for (int k = a + 1; k < b; k++) {
            const int v = refs[k];
            int j = k - 1;
            while (j >= a && refs[j] > v) { refs[j + 1] = refs[j]; j--; }
            refs[j + 1] = v;
        }
    }
}

__device__ __forceinline__ void others(const vec3i *t, int ref, int &a, int &b) {
    const vec3i T = t[ref / 3];
    const int s = ref % 3;
    a = s == 0 ? T.y : T.x;
    b = s == 2 ? T.y : T.z;
}

// Lo = L(o) - o in double (once), original positions o kept in double
__global__ void k_hc_init(const vec3d *__restrict__ o, const vec3i *__restrict__ t, const unsigned *__restrict__ start,
                          const int *__restrict__ refs, int np, float3 *Lo, float3 *P, unsigned char *hasnb) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < np; i += gridDim.x * blockDim.x) {
        const int a0 = (int)start[i], a1 = (int)start[i + 1];
        P[i] = make_float3(0.f, 0.f, 0.f);
        hasnb[i] = a1 > a0;
        if (a1 == a0) { Lo[i] = make_float3(0.f, 0.f, 0.f); continue; }
        double sx = 0, sy = 0, sz = 0;
        for (int k = a0; k < a1; k++) {
            int a, b;
            others(t, refs[k], a, b);
            sx += o[a].x + o[b].x; sy += o[a].y + o[b].y; sz += o[a].z + o[b].z;
        }
        const double n = 2.0 * (a1 - a0);
        Lo[i] = make_float3((float)(sx / n - o[i].x), (float)(sy / n - o[i].y), (float)(sz / n - o[i].z));
    }
}

__device__ __forceinline__ float3 lap(const float3 *__restrict__ X, const vec3i *__restrict__ t,
                                      const int *__restrict__ refs, int a0, int a1) {
    float sx = 0.f, sy = 0.f, sz = 0.f;
    for (int k = a0; k < a1; k++) {
        int a, b;
        others(t, refs[k], a, b);
        const float3 A = X[a], B = X[b];
        sx += A.x + B.x; sy += A.y + B.y; sz += A.z + B.z;
    }
    const float inv = 1.f / (2.f * (float)(a1 - a0));
    return make_float3(sx * inv, sy * inv, sz * inv);
}

// first half of an HC iteration: Pn = L(p) - o, B = Pn - (1-alpha) Q
__global__ void k_hc_a(const float3 *__restrict__ P, const float3 *__restrict__ Lo, const vec3i *__restrict__ t,
                       const unsigned *__restrict__ start, const int *__restrict__ refs,
                       const unsigned char *__restrict__ hasnb, int np, float alpha1, float3 *Pn, float3 *B) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < np; i += gridDim.x * blockDim.x) {
        const float3 q = P[i];
        float3 pn = q;
        if (hasnb[i]) {
            const float3 l = lap(P, t, refs, (int)start[i], (int)start[i + 1]);
            const float3 lo = Lo[i];
            pn = make_float3(lo.x + l.x, lo.y + l.y, lo.z + l.z);
        }
        Pn[i] = pn;
        B[i] = make_float3(pn.x - alpha1 * q.x, pn.y - alpha1 * q.y, pn.z - alpha1 * q.z);
    }
}

// second half: P = Pn - (beta B + (1-beta) L(B))
__global__ void k_hc_b(const float3 *__restrict__ Pn, const float3 *__restrict__ B, const vec3i *__restrict__ t,
                       const unsigned *__restrict__ start, const int *__restrict__ refs,
                       const unsigned char *__restrict__ hasnb, int np, float beta, float beta1, float3 *P) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < np; i += gridDim.x * blockDim.x) {
        const float3 b = B[i];
        float3 lb = b;
        if (hasnb[i]) lb = lap(B, t, refs, (int)start[i], (int)start[i + 1]);
        const float3 pn = Pn[i];
        P[i] = make_float3(pn.x - (beta * b.x + beta1 * lb.x), pn.y - (beta * b.y + beta1 * lb.y),
                           pn.z - (beta * b.z + beta1 * lb.z));
    }
}

// border flags: an id seen exactly once among a vertex's incident triangles
__global__ void k_border(const vec3i *__restrict__ t, const unsigned *__restrict__ start, const int *__restrict__ refs,
                         int np, unsigned char *border) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < np; i += gridDim.x * blockDim.x) {
        const int a0 = (int)start[i], a1 = (int)start[i + 1];
        for (int k = a0; k < a1; k++) {
            const vec3i T = t[refs[k] / 3];
            const int cand[3] = {T.x, T.y, T.z};
            for (int c = 0; c < 3; c++) {
                const int id = cand[c];
                int cnt = 0;
                for (int k2 = a0; k2 < a1 && cnt < 2; k2++) {
                    const vec3i U = t[refs[k2] / 3];
                    cnt += (U.x == id) + (U.y == id) + (U.z == id);
                }
                if (cnt == 1) border[id] = 1;
            }
        }
    }
}

__global__ void k_hc_out(vec3d *o, const float3 *__restrict__ P, const unsigned char *__restrict__ border, int np,
                         bool lock, const unsigned *__restrict__ bad) {
    if (*bad) return;   // a triangle index was out of range: leave the mesh as it was
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < np; i += gridDim.x * blockDim.x) {
        if (lock && border[i]) continue;
        const float3 d = P[i];
        o[i].x += (double)d.x; o[i].y += (double)d.y; o[i].z += (double)d.z;
    }
}

// ---- HC adjoint ------------------------------------------------------------------------
// One iteration is p' = A p + B o with L the (row-normalised) neighbour mean:
//   A = beta(1-alpha) I + (1-beta)(2-alpha) L - (1-beta) L^2,  B = alpha beta I + alpha(1-beta) L.
// Backward: lambda = dL/dp_K; per iteration g_o += B^T lambda, lambda = A^T lambda; finally
// g_o += lambda (p_0 = o).  L^T y at j sums y_i / num_i over the same (triangle, slot)
// references (the neighbour relation is symmetric); isolated vertices are identity rows.
__global__ void k_scale_inv(const float3 *__restrict__ Y, const unsigned *__restrict__ start, int np, float3 *Ys) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < np; i += gridDim.x * blockDim.x) {
        const int d = (int)(start[i + 1] - start[i]);
        const float s = d ? 1.f / (2.f * (float)d) : 0.f;
        const float3 y = Y[i];
        Ys[i] = make_float3(y.x * s, y.y * s, y.z * s);
    }
}

__global__ void k_lapT(const float3 *__restrict__ Ys, const float3 *__restrict__ Y, const vec3i *__restrict__ t,
                       const unsigned *__restrict__ start, const int *__restrict__ refs, int np, float3 *out) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < np; i += gridDim.x * blockDim.x) {
        const int a0 = (int)start[i], a1 = (int)start[i + 1];
        if (a0 == a1) { out[i] = Y[i]; continue; }
        float sx = 0.f, sy = 0.f, sz = 0.f;
        for (int k = a0; k < a1; k++) {
            int a, b;
            others(t, refs[k], a, b);
            const float3 A = Ys[a], B = Ys[b];
            sx += A.x + B.x; sy += A.y + B.y; sz += A.z + B.z;
        }
        out[i] = make_float3(sx, sy, sz);
    }
}

__global__ void k_hcT_init(const float3 *__restrict__ g, const unsigned char *__restrict__ border, int np, bool lock,
                           float3 *lam, float3 *go) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < np; i += gridDim.x * blockDim.x) {
        const bool b = lock && border[i];
        lam[i] = b ? make_float3(0.f, 0.f, 0.f) : g[i];
        go[i] = b ? g[i] : make_float3(0.f, 0.f, 0.f);
    }
}

// go += ab*lam + a1b*t1 ; lam = c0*lam + c1*t1 - c2*t2
__global__ void k_hcT_step(float3 *lam, const float3 *__restrict__ t1, const float3 *__restrict__ t2, float3 *go, int np,
                           float ab, float a1b, float c0, float c1, float c2) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < np; i += gridDim.x * blockDim.x) {
        const float3 l = lam[i], u = t1[i], v = t2[i];
        float3 o = go[i];
        o.x += ab * l.x + a1b * u.x; o.y += ab * l.y + a1b * u.y; o.z += ab * l.z + a1b * u.z;
        go[i] = o;
        lam[i] = make_float3(c0 * l.x + c1 * u.x - c2 * v.x, c0 * l.y + c1 * u.y - c2 * v.y, c0 * l.z + c1 * u.z - c2 * v.z);
    }
}

__global__ void k_add3(float3 *go, const float3 *__restrict__ lam, int np) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < np; i += gridDim.x * blockDim.x) {
        const float3 l = lam[i];
        go[i].x += l.x; go[i].y += l.y; go[i].z += l.z;
    }
}
}  // namespace

n2m_status mesh_smooth_hc(vec3d *d_pts, const vec3i *d_tris, int np, int nt, double alpha, double beta, int iter,
                          bool lock_edges, HcWork &w, ScanWork &sw, cudaStream_t s) {
    if (np <= 0 || iter <= 0) return N2M_OK;
    CKS(w.start.ensure(((size_t)np + 1) * sizeof(unsigned)));
    CKS(w.fill.ensure((size_t)np * sizeof(unsigned)));
    CKS(w.refs.ensure((size_t)3 * (nt > 0 ? nt : 1) * sizeof(int)));
    CKS(w.P.ensure((size_t)np * sizeof(float3)));
    CKS(w.Q.ensure((size_t)np * sizeof(float3)));
    CKS(w.B.ensure((size_t)np * sizeof(float3)));
    CKS(w.Lo.ensure((size_t)np * sizeof(float3)));
    CKS(w.hasnb.ensure((size_t)np));
    CKS(w.border.ensure((size_t)np));
    CKS(w.bad.ensure(sizeof(unsigned)));
    unsigned *start = w.start.as<unsigned>();
    CK(cudaMemsetAsync(start, 0, ((size_t)np + 1) * sizeof(unsigned), s));
    CK(cudaMemsetAsync(w.fill.p, 0, (size_t)np * sizeof(unsigned), s));
    CK(cudaMemsetAsync(w.bad.p, 0, sizeof(unsigned), s));
    { k_degree<<<gs(nt), 256, 0, s>>>(d_tris, nt, np, start, w.bad.as<unsigned>()); N2M_COUNT(); }
    CKL();
    CKS(scan_u32(start, (size_t)np + 1, start + np + 0, sw, s));  // start[np] receives the total as well
    { k_fill_refs<<<gs(nt), 256, 0, s>>>(d_tris, nt, np, start, w.fill.as<unsigned>(), w.refs.as<int>()); N2M_COUNT(); }
    { k_sort_refs<<<gs(np), 256, 0, s>>>(start, np, w.refs.as<int>()); N2M_COUNT(); }
    { k_hc_init<<<gs(np), 256, 0, s>>>(d_pts, d_tris, start, w.refs.as<int>(), np, w.Lo.as<float3>(), w.P.as<float3>(),
                                     w.hasnb.as<unsigned char>()); N2M_COUNT(); }
    CKL();
    const float a1 = (float)(1.0 - alpha), b = (float)beta, b1 = (float)(1.0 - beta);
    for (int it = 0; it < iter; it++) {
        { k_hc_a<<<gs(np), 256, 0, s>>>(w.P.as<float3>(), w.Lo.as<float3>(), d_tris, start, w.refs.as<int>(),
                                      w.hasnb.as<unsigned char>(), np, a1, w.Q.as<float3>(), w.B.as<float3>()); N2M_COUNT(); }
        { k_hc_b<<<gs(np), 256, 0, s>>>(w.Q.as<float3>(), w.B.as<float3>(), d_tris, start, w.refs.as<int>(),
                                      w.hasnb.as<unsigned char>(), np, b, b1, w.P.as<float3>()); N2M_COUNT(); }
    }
    CKL();
    if (lock_edges) {
        CK(cudaMemsetAsync(w.border.p, 0, (size_t)np, s));
        { k_border<<<gs(np), 256, 0, s>>>(d_tris, start, w.refs.as<int>(), np, w.border.as<unsigned char>()); N2M_COUNT(); }
    }
    { k_hc_out<<<gs(np), 256, 0, s>>>(d_pts, w.P.as<float3>(), w.border.as<unsigned char>(), np, lock_edges,
                                    w.bad.as<unsigned>()); N2M_COUNT(); }
    CKL();
    return N2M_OK;
}

n2m_status mesh_smooth_hc_check(HcWork &w, int np, int iter, cudaStream_t s) {
    if (np <= 0 || iter <= 0) return N2M_OK;
    unsigned bad = 0;
    CK(cudaMemcpyAsync(&bad, w.bad.p, sizeof(unsigned), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    if (bad) {
        n2m_set_error("HC smoothing: a triangle index is outside [0, nvert); the vertices were left unchanged");
        return N2M_ERR_BAD_ARGS;
    }
    return N2M_OK;
}

n2m_status mesh_smooth_hc_backward(const vec3i *d_tris, int np, double alpha, double beta, int iter, bool lock_edges,
                                   HcWork &w, const float3 *d_g, float3 *d_go, cudaStream_t s) {
    // buffers of the forward: start, refs, border; scratch: P (lambda), Q (t1), B (t2), Lo (scaled)
    const unsigned *start = w.start.as<unsigned>();
    const int *refs = w.refs.as<int>();
    float3 *lam = w.P.as<float3>(), *t1 = w.Q.as<float3>(), *t2 = w.B.as<float3>(), *ys = w.Lo.as<float3>();
    { k_hcT_init<<<gs(np), 256, 0, s>>>(d_g, w.border.as<unsigned char>(), np, lock_edges, lam, d_go); N2M_COUNT(); }
    const float al = (float)alpha, be = (float)beta;
    const float ab = al * be, a1b = al * (1.f - be);
    const float c0 = be * (1.f - al), c1 = (1.f - be) * (2.f - al), c2 = 1.f - be;
    for (int it = 0; it < iter; it++) {
        { k_scale_inv<<<gs(np), 256, 0, s>>>(lam, start, np, ys); N2M_COUNT(); }
        { k_lapT<<<gs(np), 256, 0, s>>>(ys, lam, d_tris, start, refs, np, t1); N2M_COUNT(); }
        { k_scale_inv<<<gs(np), 256, 0, s>>>(t1, start, np, ys); N2M_COUNT(); }
        { k_lapT<<<gs(np), 256, 0, s>>>(ys, t1, d_tris, start, refs, np, t2); N2M_COUNT(); }
        { k_hcT_step<<<gs(np), 256, 0, s>>>(lam, t1, t2, d_go, np, ab, a1b, c0, c1, c2); N2M_COUNT(); }
    }
    { k_add3<<<gs(np), 256, 0, s>>>(d_go, lam, np); N2M_COUNT(); }
    CKL();
    return N2M_OK;
}

// ---- allocation-free HC smoothing ---------------------------------------------------
// For callers that cannot call cudaMalloc: code running inside another
// framework's captured or allocation-controlled region, or a host program that
// owns all device memory through its own pool.  The scratch of the HC
// smoothing (CSR incidence, displacement buffers, flags) lives in one
// file-scope device array of fixed size, so the entry point allocates nothing.
// Limits: N2M_NOALLOC_MAX_VERTS vertices and N2M_NOALLOC_MAX_TRIS triangles
// (about 11 MB, held by every GPU that loads the library until exit).
namespace {
constexpr size_t NA_V = N2M_NOALLOC_MAX_VERTS, NA_T = N2M_NOALLOC_MAX_TRIS;
constexpr size_t na_align(size_t b) { return (b + 255) & ~(size_t)255; }
constexpr size_t NA_START = 0;
constexpr size_t NA_FILL = NA_START + na_align((NA_V + 1) * 4);
constexpr size_t NA_REFS = NA_FILL + na_align(NA_V * 4);
constexpr size_t NA_P = NA_REFS + na_align(NA_T * 3 * 4);
constexpr size_t NA_Q = NA_P + na_align(NA_V * 12);
constexpr size_t NA_B = NA_Q + na_align(NA_V * 12);
constexpr size_t NA_LO = NA_B + na_align(NA_V * 12);
constexpr size_t NA_HASNB = NA_LO + na_align(NA_V * 12);
constexpr size_t NA_BORDER = NA_HASNB + na_align(NA_V);
constexpr size_t NA_BAD = NA_BORDER + na_align(NA_V);
constexpr size_t NA_TOTAL = NA_BAD + na_align(4);

static __device__ __align__(256) unsigned char g_noalloc_scratch[NA_TOTAL];

// exclusive scan of n <= NA_V + 1 counts in one CTA (n is small by construction)
__global__ void __launch_bounds__(1024) k_scan_small(unsigned *d, int n) {
    __shared__ unsigned part[1024];
    __shared__ unsigned carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int base = 0; base < n; base += 1024) {
        const int i = base + threadIdx.x;
        const unsigned v = i < n ? d[i] : 0u;
        part[threadIdx.x] = v;
        __syncthreads();
        for (int o = 1; o < 1024; o <<= 1) {
            const unsigned t = threadIdx.x >= o ? part[threadIdx.x - o] : 0u;
            __syncthreads();
            part[threadIdx.x] += t;
            __syncthreads();
        }
        if (i < n) d[i] = carry + part[threadIdx.x] - v;
        __syncthreads();
        if (threadIdx.x == 1023) carry += part[1023];
        __syncthreads();
    }
}
}  // namespace

// Every call looks up the device address of the scratch array on the current
// device (cudaGetSymbolAddress allocates nothing), so the address is never
// stale, e.g. after the caller reset the device.  The first call on a device
// may load the library's device code; make it before any stream capture.
extern "C" n2m_status n2m_smooth_hc_noalloc(vec3d *d_verts, const vec3i *d_tris, int nvert, int ntri, double alpha,
                                            double beta, int iter, bool lock_edges, void *stream) {
    if (nvert < 0 || ntri < 0 || (nvert > 0 && !d_verts) || (ntri > 0 && !d_tris)) {
        n2m_set_error("n2m_smooth_hc_noalloc: bad arguments");
        return N2M_ERR_BAD_ARGS;
    }
    if ((size_t)nvert > NA_V || (size_t)ntri > NA_T) {
        n2m_set_error("n2m_smooth_hc_noalloc: mesh of %d vertices / %d triangles exceeds the fixed scratch "
                      "(max %d vertices, %d triangles)", nvert, ntri, N2M_NOALLOC_MAX_VERTS, N2M_NOALLOC_MAX_TRIS);
        return N2M_ERR_TOO_LARGE;
    }
    if (nvert == 0 || iter <= 0) return N2M_OK;
    unsigned char *base = nullptr;
    CK(cudaGetSymbolAddress((void **)&base, g_noalloc_scratch));
    cudaStream_t s = (cudaStream_t)stream;
    unsigned *start = (unsigned *)(base + NA_START), *fill = (unsigned *)(base + NA_FILL);
    int *refs = (int *)(base + NA_REFS);
    float3 *P = (float3 *)(base + NA_P), *Q = (float3 *)(base + NA_Q), *B = (float3 *)(base + NA_B),
           *Lo = (float3 *)(base + NA_LO);
    unsigned char *hasnb = base + NA_HASNB, *border = base + NA_BORDER;
    unsigned *bad = (unsigned *)(base + NA_BAD);
    // the array keeps the previous call's contents: clear what must start at zero
    CK(cudaMemsetAsync(start, 0, ((size_t)nvert + 1) * sizeof(unsigned), s));
    CK(cudaMemsetAsync(fill, 0, (size_t)nvert * sizeof(unsigned), s));
    CK(cudaMemsetAsync(bad, 0, sizeof(unsigned), s));
    { k_degree<<<gs(ntri), 256, 0, s>>>(d_tris, ntri, nvert, start, bad); N2M_COUNT(); }
    { k_scan_small<<<1, 1024, 0, s>>>(start, nvert + 1); N2M_COUNT(); }
    { k_fill_refs<<<gs(ntri), 256, 0, s>>>(d_tris, ntri, nvert, start, fill, refs); N2M_COUNT(); }
    { k_sort_refs<<<gs(nvert), 256, 0, s>>>(start, nvert, refs); N2M_COUNT(); }
    { k_hc_init<<<gs(nvert), 256, 0, s>>>(d_verts, d_tris, start, refs, nvert, Lo, P, hasnb); N2M_COUNT(); }
    const float a1 = (float)(1.0 - alpha), b = (float)beta, b1 = (float)(1.0 - beta);
    for (int it = 0; it < iter; it++) {
        { k_hc_a<<<gs(nvert), 256, 0, s>>>(P, Lo, d_tris, start, refs, hasnb, nvert, a1, Q, B); N2M_COUNT(); }
        { k_hc_b<<<gs(nvert), 256, 0, s>>>(Q, B, d_tris, start, refs, hasnb, nvert, b, b1, P); N2M_COUNT(); }
    }
    if (lock_edges) {
        CK(cudaMemsetAsync(border, 0, (size_t)nvert, s));
        { k_border<<<gs(nvert), 256, 0, s>>>(d_tris, start, refs, nvert, border); N2M_COUNT(); }
    }
    { k_hc_out<<<gs(nvert), 256, 0, s>>>(d_verts, P, border, nvert, lock_edges, bad); N2M_COUNT(); }
    CKL();
    // the validity flag comes back through pageable host memory: a plain copy, no allocation
    unsigned h_bad = 0;
    CK(cudaMemcpyAsync(&h_bad, bad, sizeof(unsigned), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    if (h_bad) {
        n2m_set_error("n2m_smooth_hc_noalloc: a triangle index is outside [0, nvert); the vertices were left unchanged");
        return N2M_ERR_BAD_ARGS;
    }
    return N2M_OK;
}
