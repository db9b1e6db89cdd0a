// label.cu — connected-component labelling for meshify's largest-cluster and
// bubble-fill options (src/bwlabel.c:429-543, src/meshify.c:323-342).
//
// GPU union-find: every foreground voxel starts as its own root; each voxel
// unites with its already-visited half-neighbourhood (3 offsets for
// 6-connectivity, 9 for 18, 13 for 26) by CAS-hooking the larger root under
// the smaller one, then a flatten pass points every voxel at its root.  The
// root of a component is therefore its first voxel in raster order, which is
// exactly how the reference numbers labels (first appearance) and breaks
// size ties (lowest label wins).
#include "n2m_internal.cuh"
#include "uf.cuh"

namespace {
using namespace uf;
struct Dims {
    int nx, ny, nz;
    long long nxy, n;
};

__global__ void k_mask(const float *__restrict__ vol, long long n, float iso, unsigned char *m) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        m[i] = vol[i] >= iso;
}

__global__ void k_nonzero(const float *__restrict__ vol, long long n, unsigned char *m) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        m[i] = vol[i] != 0.0f;
}

// L[i] = i where m[i] == want, else -1
// Union-find start: every voxel of the wanted class points at the start of its
// run along x (ballot within the warp; a run entering the warp from the left
// points at the voxel before the warp), so x links need no union; others -1.
__global__ void k_uf_init(const unsigned char *__restrict__ m, Dims d, unsigned char want, int *L) {
    const long long n = d.n;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const int lane = threadIdx.x & 31;
        // the lanes of this step: consecutive voxels, a prefix of the warp
        const long long left = n - (i - lane);
        const unsigned act = left >= 32 ? 0xffffffffu : (1u << left) - 1u;
        const bool fg = m[i] == want;
        const bool left_fg = __shfl_up_sync(act, fg, 1);
        const bool xpos = (i % d.nx) != 0;
        const bool cont = fg && xpos && (lane > 0 ? left_fg : m[i - 1] == want);
        const unsigned starts = __ballot_sync(act, fg && !cont);
        int parent = -1;
        if (fg) {
            const unsigned le = starts & (lane == 31 ? 0xffffffffu : (2u << lane) - 1u);
            parent = le ? (int)(i - (lane - (31 - __clz(le)))) : (int)(i - lane - 1);
        }
        L[i] = parent;
    }
}

__constant__ signed char k_half[13][3] = {{-1, 0, 0},  {0, -1, 0}, {0, 0, -1},  {-1, -1, 0}, {1, -1, 0},
                                          {-1, 0, -1}, {1, 0, -1}, {0, -1, -1}, {0, 1, -1},  {-1, -1, -1},
                                          {1, -1, -1}, {-1, 1, -1}, {1, 1, -1}};

__global__ void k_uf_merge(int *L, Dims d, int nnb) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < d.n; i += (long long)gridDim.x * blockDim.x) {
        if (L[i] < 0) continue;
        const int z = (int)(i / d.nxy);
        const long long r = i - z * d.nxy;
        const int y = (int)(r / d.nx), x = (int)(r - (long long)y * d.nx);
        // the -x neighbour (k = 0) is linked by the run start; a contact whose two
        // left voxels also touch is implied by theirs (both pairs lie in the same runs)
        const bool left = x > 0 && L[i - 1] >= 0;
        for (int k = 1; k < nnb; k++) {
            const int xx = x + k_half[k][0], yy = y + k_half[k][1], zz = z + k_half[k][2];
            if (xx < 0 || yy < 0 || zz < 0 || xx >= d.nx || yy >= d.ny) continue;
            const long long j = zz * d.nxy + (long long)yy * d.nx + xx;
            const int lj = L[j];
            if (lj < 0 || (left && xx > 0 && L[j - 1] >= 0)) continue;
            if (lj != L[i]) unite(L, (int)i, (int)j);
        }
    }
}

__global__ void k_uf_flatten(int *L, long long n, unsigned *nroots) {
    unsigned c = 0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const int p = L[i];
        if (p < 0) continue;
        if (p == (int)i) c++;
        else L[i] = find_root(L, p);
    }
    if (nroots && c) atomicAdd(nroots, c);
}

// background components touching a face of the volume
__global__ void k_edge_roots(const int *__restrict__ L, Dims d, unsigned char *edge) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < d.n; i += (long long)gridDim.x * blockDim.x) {
        const int r = L[i];
        if (r < 0) continue;
        const int z = (int)(i / d.nxy);
        const long long rr = i - z * d.nxy;
        const int y = (int)(rr / d.nx), x = (int)(rr - (long long)y * d.nx);
        if (x == 0 || y == 0 || z == 0 || x == d.nx - 1 || y == d.ny - 1 || z == d.nz - 1) edge[r] = 1;
    }
}

// bubbles (background components away from every face) become foreground,
// only when the background has at least two components (src/bwlabel.c:488-491)
__global__ void k_fill_bubbles(const int *__restrict__ L, long long n, const unsigned char *__restrict__ edge,
                               const unsigned *__restrict__ ncomp, unsigned char *m) {
    if (*ncomp <= 1) return;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const int r = L[i];
        if (r >= 0 && !edge[r]) m[i] = 1;
    }
}

__global__ void k_sizes(const int *__restrict__ L, long long n, unsigned *cnt) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const int r = L[i];
        const unsigned grp = __match_any_sync(__activemask(), r);   // lanes sharing a root add together
        if (r >= 0 && (threadIdx.x & 31) == __ffs(grp) - 1) atomicAdd(&cnt[r], __popc(grp));
    }
}

// largest component; ties go to the smallest root (first in raster order)
__global__ void k_best(const int *__restrict__ L, const unsigned *__restrict__ cnt, long long n,
                       unsigned long long *best) {
    unsigned long long b = 0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        if (L[i] == (int)i) {
            const unsigned long long k = ((unsigned long long)cnt[i] << 32) | (0xffffffffu - (unsigned)i);
            b = k > b ? k : b;
        }
    for (int o = 16; o; o >>= 1) {
        const unsigned long long t = __shfl_xor_sync(0xffffffffu, b, o);
        b = t > b ? t : b;
    }
    if ((threadIdx.x & 31) == 0 && b) atomicMax(best, b);
}

__global__ void k_keep_best(const int *__restrict__ L, long long n, const unsigned long long *__restrict__ best,
                            unsigned char *keep) {
    const unsigned long long b = *best;
    const int root = b ? (int)(0xffffffffu - (unsigned)(b & 0xffffffffu)) : -2;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        keep[i] = L[i] == root;
}

__global__ void k_fill_iso(float *vol, long long n, const unsigned char *__restrict__ keep, float iso) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        if (keep[i]) vol[i] = fmaxf(vol[i], iso);
}

// dilate (26-neighbourhood without the (-1,-1,-1) neighbour, interior voxels
// only; src/meshify.c:218-264) fused with the mask-out img = mn
__global__ void k_dilate_maskout(const unsigned char *__restrict__ keep, Dims d, float *vol, float mn) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < d.n; i += (long long)gridDim.x * blockDim.x) {
        bool on = keep[i];
        if (!on) {
            const int z = (int)(i / d.nxy);
            const long long rr = i - z * d.nxy;
            const int y = (int)(rr / d.nx), x = (int)(rr - (long long)y * d.nx);
            if (x > 0 && y > 0 && z > 0 && x < d.nx - 1 && y < d.ny - 1 && z < d.nz - 1) {
                for (int dz = -1; dz <= 1 && !on; dz++)
                    for (int dy = -1; dy <= 1 && !on; dy++)
                        for (int dx = -1; dx <= 1; dx++) {
                            if ((dx | dy | dz) == 0 || (dx == -1 && dy == -1 && dz == -1)) continue;
                            if (keep[i + dz * d.nxy + (long long)dy * d.nx + dx]) { on = true; break; }
                        }
            }
        }
        if (!on) vol[i] = mn;
    }
}

// bwlabel() output: label = 1 + rank of the component's root among roots
__global__ void k_root_flags(const int *__restrict__ L, long long n, unsigned *flag) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        flag[i] = L[i] == (int)i;
}

__global__ void k_write_labels(const int *__restrict__ L, long long n, const unsigned *__restrict__ rank, float *vol) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const int r = L[i];
        vol[i] = r < 0 ? 0.0f : (float)(rank[r] + 1u);
    }
}

__global__ void k_write_keep(const unsigned char *__restrict__ keep, long long n, float *vol) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        vol[i] = keep[i] ? 1.0f : 0.0f;
}

__global__ void k_nl_from(const unsigned *nroots, const unsigned long long *best, bool only_largest, int *nl) {
    *nl = only_largest ? (*nroots > 0 ? 1 : 0) : (int)*nroots;
}

inline unsigned gsz(long long n) {
    long long b = (n + 255) / 256;
    if (b > 152 * 64) b = 152 * 64;
    return b ? (unsigned)b : 1u;
}

n2m_status components(LabelWork &w, Dims d, unsigned char want, int conn, unsigned *d_nroots, cudaStream_t s) {
    int *L = w.lab.as<int>();
    { k_uf_init<<<gsz(d.n), 256, 0, s>>>(w.mask.as<unsigned char>(), d, want, L); N2M_COUNT(); }
    { k_uf_merge<<<gsz(d.n), 256, 0, s>>>(L, d, conn == 6 ? 3 : conn == 18 ? 9 : 13); N2M_COUNT(); }
    if (d_nroots) CK(cudaMemsetAsync(d_nroots, 0, sizeof(unsigned), s));
    { k_uf_flatten<<<gsz(d.n), 256, 0, s>>>(L, d.n, d_nroots); N2M_COUNT(); }
    CKL();
    return N2M_OK;
}

// misc layout: [0] nroots bg, [1] nroots fg, [2..3] best (u64), [4] nl
struct Misc {
    unsigned nbg, nfg;
    unsigned long long best;
    int nl, pad;
};

n2m_status label_core(LabelWork &w, Dims d, int conn, bool only_largest, bool fill_bubbles, cudaStream_t s) {
    CKS(w.lab.ensure((size_t)d.n * sizeof(int)));
    CKS(w.keep.ensure((size_t)d.n));
    CKS(w.misc.ensure(sizeof(Misc)));
    Misc *misc = w.misc.as<Misc>();
    CK(cudaMemsetAsync(misc, 0, sizeof(Misc), s));
    if (fill_bubbles) {
        CKS(w.edge.ensure((size_t)d.n));
        CKS(components(w, d, 0, 6, &misc->nbg, s));
        CK(cudaMemsetAsync(w.edge.p, 0, (size_t)d.n, s));
        { k_edge_roots<<<gsz(d.n), 256, 0, s>>>(w.lab.as<int>(), d, w.edge.as<unsigned char>()); N2M_COUNT(); }
        { k_fill_bubbles<<<gsz(d.n), 256, 0, s>>>(w.lab.as<int>(), d.n, w.edge.as<unsigned char>(), &misc->nbg,
                                                w.mask.as<unsigned char>()); N2M_COUNT(); }
        CKL();
    }
    CKS(components(w, d, 1, conn, &misc->nfg, s));
    if (only_largest) {
        CKS(w.cnt.ensure((size_t)d.n * sizeof(unsigned)));
        CK(cudaMemsetAsync(w.cnt.p, 0, (size_t)d.n * sizeof(unsigned), s));
        { k_sizes<<<gsz(d.n), 256, 0, s>>>(w.lab.as<int>(), d.n, w.cnt.as<unsigned>()); N2M_COUNT(); }
        { k_best<<<gsz(d.n), 256, 0, s>>>(w.lab.as<int>(), w.cnt.as<unsigned>(), d.n, &misc->best); N2M_COUNT(); }
        { k_keep_best<<<gsz(d.n), 256, 0, s>>>(w.lab.as<int>(), d.n, &misc->best, w.keep.as<unsigned char>()); N2M_COUNT(); }
    } else {
        CK(cudaMemcpyAsync(w.keep.p, w.mask.p, (size_t)d.n, cudaMemcpyDeviceToDevice, s));
    }
    { k_nl_from<<<1, 1, 0, s>>>(&misc->nfg, &misc->best, only_largest, &misc->nl); N2M_COUNT(); }
    CKL();
    return N2M_OK;
}
}  // namespace

n2m_status run_labelling(float *vol, int nx, int ny, int nz, float iso, float mn, bool only_largest,
                         bool fill_bubbles, LabelWork &w, cudaStream_t s) {
    Dims d{nx, ny, nz, (long long)nx * ny, (long long)nx * ny * nz};
    if (d.n > 0x7fffffffLL) {
        n2m_set_error("labelling supports at most 2^31-1 voxels");
        return N2M_ERR_TOO_LARGE;
    }
    CKS(w.mask.ensure((size_t)d.n));
    { k_mask<<<gsz(d.n), 256, 0, s>>>(vol, d.n, iso, w.mask.as<unsigned char>()); N2M_COUNT(); }
    CKL();
    CKS(label_core(w, d, 18, only_largest, fill_bubbles, s));
    if (fill_bubbles) { k_fill_iso<<<gsz(d.n), 256, 0, s>>>(vol, d.n, w.keep.as<unsigned char>(), iso); N2M_COUNT(); }
    if (only_largest) { k_dilate_maskout<<<gsz(d.n), 256, 0, s>>>(w.keep.as<unsigned char>(), d, vol, mn); N2M_COUNT(); }
    CKL();
    return N2M_OK;
}

n2m_status run_bwlabel(float *vol, int nx, int ny, int nz, int conn, bool only_largest, bool fill_bubbles,
                       LabelWork &w, ScanWork &sw, int *d_nl, cudaStream_t s) {
    Dims d{nx, ny, nz, (long long)nx * ny, (long long)nx * ny * nz};
    if (d.n > 0x7fffffffLL) {
        n2m_set_error("labelling supports at most 2^31-1 voxels");
        return N2M_ERR_TOO_LARGE;
    }
    CKS(w.mask.ensure((size_t)d.n));
    { k_nonzero<<<gsz(d.n), 256, 0, s>>>(vol, d.n, w.mask.as<unsigned char>()); N2M_COUNT(); }
    CKL();
    CKS(label_core(w, d, conn, only_largest, fill_bubbles, s));
    if (only_largest) {
        { k_write_keep<<<gsz(d.n), 256, 0, s>>>(w.keep.as<unsigned char>(), d.n, vol); N2M_COUNT(); }
    } else {
        CKS(w.cnt.ensure(((size_t)d.n + 1) * sizeof(unsigned)));
        unsigned *rank = w.cnt.as<unsigned>();
        CK(cudaMemsetAsync(rank + d.n, 0, sizeof(unsigned), s));
        { k_root_flags<<<gsz(d.n), 256, 0, s>>>(w.lab.as<int>(), d.n, rank); N2M_COUNT(); }
        CKL();
        CKS(scan_u32(rank, (size_t)d.n + 1, rank + d.n, sw, s));
        { k_write_labels<<<gsz(d.n), 256, 0, s>>>(w.lab.as<int>(), d.n, rank, vol); N2M_COUNT(); }
    }
    CK(cudaMemcpyAsync(d_nl, &w.misc.as<Misc>()->nl, sizeof(int), cudaMemcpyDeviceToDevice, s));
    CKL();
    return N2M_OK;
}
