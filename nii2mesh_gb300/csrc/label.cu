// label.cu — connected-component labelling for meshify's largest-cluster and
// bubble-fill options (src/bwlabel.c:429-543, src/meshify.c:323-342).
//
// GPU union-find: every voxel of the class starts linked to the first voxel of
// its run along x; each voxel unites with its already-visited
// half-neighbourhood (3 offsets for 6-connectivity, 9 for 18, 13 for 26) by
// CAS-hooking the larger root under the smaller one, then a flatten pass
// points every voxel at its root.  The root of a component is therefore its
// first voxel in raster order, which is exactly how the reference numbers
// labels (first appearance) and breaks size ties (lowest label wins).
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
        const bool xpos = (unsigned)i % (unsigned)d.nx != 0u;   // n < 2^31
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

// Union of each voxel of the class (m == want) with its half-neighbours of
// k_half[1 .. NNB-1] (the -x neighbour is linked by the run start).  A contact
// whose two left voxels also touch is implied by theirs (both pairs lie in the
// same runs) and is skipped.  One warp per row (y, z), 32 voxels a word: the
// class bits of the row and of the rows (y-1, z), (y, z-1), (y-1, z-1),
// (y+1, z-1) give every contact of a word by shifts; only the lanes holding
// one touch L.
template <int NNB>
__global__ void __launch_bounds__(256) k_uf_merge(const unsigned char *__restrict__ m, unsigned char want, int *L, Dims d) {
    static_assert(NNB == 3 || NNB == 9 || NNB == 13, "6-, 18- or 26-connectivity");
    const int lane = threadIdx.x & 31;
    const long long nrows = (long long)d.ny * d.nz;
    const int nw = (d.nx + 31) / 32;
    constexpr int NR = NNB == 3 ? 3 : 5;
    // rows: 0 = (y, z), 1 = (y-1, z), 2 = (y, z-1), 3 = (y-1, z-1), 4 = (y+1, z-1)
    const int RY[5] = {0, -1, 0, -1, 1}, RZ[5] = {0, 0, -1, -1, -1};
    for (long long r = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5; r < nrows;
         r += ((long long)gridDim.x * blockDim.x) >> 5) {
        const int z = (int)(r / d.ny), y = (int)(r - (long long)z * d.ny);
        auto word = [&](int dy, int dz, int xw) -> unsigned {
            const int yy = y + dy, zz = z + dz, x = xw * 32 + lane;
            const bool in = yy >= 0 && zz >= 0 && yy < d.ny && zz < d.nz && x < d.nx;
            return __ballot_sync(0xffffffffu, in && m[zz * d.nxy + (long long)yy * d.nx + x] == want);
        };
        unsigned pw[NR], cw[NR];
#pragma unroll
        for (int k = 0; k < NR; k++) {
            pw[k] = 0u;
            cw[k] = word(RY[k], RZ[k], 0);
        }
        for (int xw = 0; xw < nw; xw++) {
            unsigned nx[NR];
#pragma unroll
            for (int k = 0; k < NR; k++) nx[k] = word(RY[k], RZ[k], xw + 1);
            // S(k, dx): bit x = class of voxel x + dx of row k (dx in -2 .. 1)
            auto S = [&](int k, int dx) -> unsigned {
                return dx == 0 ? cw[k] : dx > 0 ? (cw[k] >> dx) | (nx[k] << (32 - dx)) : (cw[k] << -dx) | (pw[k] >> (32 + dx));
            };
            const unsigned F = cw[0], left = S(0, -1);
            auto contact = [&](int k, int dx) -> unsigned { return ((F & S(k, dx) & ~(left & S(k, dx - 1))) >> lane) & 1u; };
            // bit k-1 of this lane's set: a contact with k_half[k]
            unsigned set = contact(1, 0) | contact(2, 0) << 1;   // (0,-1,0) (0,0,-1)
            if constexpr (NNB >= 9)
                set |= contact(1, -1) << 2 | contact(1, 1) << 3     // (-1,-1,0) (1,-1,0)
                     | contact(2, -1) << 4 | contact(2, 1) << 5     // (-1,0,-1) (1,0,-1)
                     | contact(3, 0) << 6 | contact(4, 0) << 7;     // (0,-1,-1) (0,1,-1)
            if constexpr (NNB == 13)
                set |= contact(3, -1) << 8 | contact(3, 1) << 9     // (-1,-1,-1) (1,-1,-1)
                     | contact(4, -1) << 10 | contact(4, 1) << 11;  // (-1,1,-1) (1,1,-1)
            const int x = xw * 32 + lane;
            if (set && x < d.nx) {
                const int i = (int)(r * d.nx + x);
                do {
                    const int k = __ffs(set);
                    set &= set - 1u;
                    const int j = i + k_half[k][0] + k_half[k][1] * d.nx + k_half[k][2] * (int)d.nxy;
                    if (L[j] != L[i]) unite(L, i, j);
                } while (set);
            }
#pragma unroll
            for (int k = 0; k < NR; k++) {
                pw[k] = cw[k];
                cw[k] = nx[k];
            }
        }
    }
}

// every voxel of the class points at its root; lanes sharing a parent (the
// voxels of one run) walk its chain once
__global__ void k_uf_flatten(int *L, long long n, unsigned *nroots) {
    unsigned c = 0;
    const int lane = threadIdx.x & 31;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const int p = L[i];
        const unsigned grp = __match_any_sync(__activemask(), p);
        const int lead = __ffs(grp) - 1;
        int root = 0;
        if (lane == lead && p >= 0) root = find_root(L, p);
        root = __shfl_sync(grp, root, lead);
        if (p < 0) continue;
        if (p == (int)i) c++;
        else L[i] = root;
    }
    if (nroots && c) atomicAdd(nroots, c);
}

// background components touching a face of the volume: one thread per face
// voxel (slices z = 0 and z = nz-1 whole; rows y = 0 and y = ny-1 and
// columns x = 0 and x = nx-1 of the slices between; a voxel on two faces is
// visited twice, which writes the same flag)
__global__ void k_edge_roots(const int *__restrict__ L, Dims d, unsigned char *edge) {
    const long long inner = d.nz > 2 ? d.nz - 2 : 0;
    const long long nface_z = d.nz > 1 ? 2 * d.nxy : d.nxy, nrow = inner * d.nx, ncol = inner * d.ny;
    const long long total = nface_z + 2 * nrow + 2 * ncol;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total; t += (long long)gridDim.x * blockDim.x) {
        long long i;
        if (t < nface_z) {
            i = t < d.nxy ? t : (long long)(d.nz - 1) * d.nxy + (t - d.nxy);
        } else if (t < nface_z + 2 * nrow) {
            const long long u = t - nface_z, side = u / nrow, v = u - side * nrow;
            const long long z = 1 + v / d.nx, x = v - (z - 1) * d.nx;
            i = z * d.nxy + (side ? (long long)(d.ny - 1) * d.nx : 0) + x;
        } else {
            const long long u = t - nface_z - 2 * nrow, side = u / ncol, v = u - side * ncol;
            const long long z = 1 + v / d.ny, y = v - (z - 1) * d.ny;
            i = z * d.nxy + y * d.nx + (side ? d.nx - 1 : 0);
        }
        const int r = L[i];
        if (r >= 0) edge[r] = 1;
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
// only; src/meshify.c:218-264) fused with the mask-out img = mn.  One warp per
// row, 32 voxels a word: with R3 = K(x-1)|K(x)|K(x+1) and R2 = K(x)|K(x+1) of a
// row, the neighbourhood is R3 of rows y-1..y+1 in slices z and z+1, R3 of rows
// y and y+1 in slice z-1, and R2 of row y-1 in slice z-1.
__global__ void __launch_bounds__(256) k_dilate_maskout(const unsigned char *__restrict__ keep, Dims d, float *vol, float mn) {
    const int lane = threadIdx.x & 31;
    const long long nrows = (long long)d.ny * d.nz;
    const int nw = (d.nx + 31) / 32;
    // rows used: 0..2 = y-1..y+1 in slice z, 3..5 in slice z+1, 6 = (y, z-1), 7 = (y+1, z-1), 8 = (y-1, z-1)
    const int DY[9] = {-1, 0, 1, -1, 0, 1, 0, 1, -1}, DZ[9] = {0, 0, 0, 1, 1, 1, -1, -1, -1};
    for (long long r = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5; r < nrows;
         r += ((long long)gridDim.x * blockDim.x) >> 5) {
        const int z = (int)(r / d.ny), y = (int)(r - (long long)z * d.ny);
        const bool ryz = y > 0 && z > 0 && y < d.ny - 1 && z < d.nz - 1;
        auto word = [&](int dy, int dz, int xw) -> unsigned {
            const int yy = y + dy, zz = z + dz, x = xw * 32 + lane;
            const bool in = yy >= 0 && zz >= 0 && yy < d.ny && zz < d.nz && x < d.nx;
            return __ballot_sync(0xffffffffu, in && keep[zz * d.nxy + (long long)yy * d.nx + x] != 0);
        };
        unsigned prev[9], cur[9];
#pragma unroll
        for (int k = 0; k < 9; k++) {
            prev[k] = 0u;
            cur[k] = word(DY[k], DZ[k], 0);
        }
        for (int xw = 0; xw < nw; xw++) {
            unsigned on = 0u;
#pragma unroll
            for (int k = 0; k < 9; k++) {
                const unsigned nxt = word(DY[k], DZ[k], xw + 1);
                const unsigned right = (cur[k] >> 1) | (nxt << 31);   // K(x+1)
                on |= cur[k] | right | (k < 8 ? (cur[k] << 1) | (prev[k] >> 31) : 0u);   // row 8: no K(x-1)
                prev[k] = cur[k];
                cur[k] = nxt;
            }
            const int x = xw * 32 + lane;
            if (x < d.nx) {
                const bool kept = (prev[1] >> lane) & 1u;   // row (y, z): prev holds word xw now
                const bool interior = ryz && x > 0 && x < d.nx - 1;
                if (!(kept || (interior && ((on >> lane) & 1u)))) vol[r * d.nx + x] = mn;
            }
        }
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
    const unsigned gr = gsz((long long)d.ny * d.nz * 32);   // one warp per row
    const unsigned char *m = w.mask.as<unsigned char>();
    if (conn == 6) { k_uf_merge<3><<<gr, 256, 0, s>>>(m, want, L, d); N2M_COUNT(); }
    else if (conn == 18) { k_uf_merge<9><<<gr, 256, 0, s>>>(m, want, L, d); N2M_COUNT(); }
    else { k_uf_merge<13><<<gr, 256, 0, s>>>(m, want, L, d); N2M_COUNT(); }
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
        { k_edge_roots<<<gsz(2 * d.nxy + 2 * (long long)d.nz * (d.nx + d.ny)), 256, 0, s>>>(w.lab.as<int>(), d, w.edge.as<unsigned char>()); N2M_COUNT(); }
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
    if (only_largest) { k_dilate_maskout<<<gsz((long long)d.ny * d.nz * 32), 256, 0, s>>>(w.keep.as<unsigned char>(), d, vol, mn); N2M_COUNT(); }
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
