// atlas.cu — batched atlas meshing (the per-label loop of src/nii2mesh.c:492-583).
//
// The reference binarises the whole volume for every label (`lo < v < hi`,
// src/nii2mesh.c:555-563) and runs the full meshify on it.  Outside the
// label's bounding box + 2 voxels the smoothed mask is exactly 0, so every
// stage can run on a sub-box (bbox + 3, clipped to the volume) instead:
// smoothing keeps the volume's own face rule (global coordinates), the
// background outside the sub-box joins the sub-box's boundary shell (so
// bubble detection and the largest-cluster tie-break are unchanged), and the
// marching-cubes fetch returns 0 for voxels outside the sub-box.
//
// All labels' sub-boxes live in one float arena.  Each stage is ONE launch
// of persistent CTAs that pull work items (a smoothing column, a chunk of
// voxels, a marching-cubes tile, an active word) of any label from a global
// atomic queue, so hundreds of labels of very different sizes share the GPU
// in each launch.  Vertex/triangle numbering comes from one scan over the
// words of every label's grid: each label's mesh is a contiguous range in
// the concatenated output, numbered exactly as the single-volume path.
#include <string.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "mc33.cuh"
#include "runs.cuh"
#include "smooth_core.cuh"
#include "uf.cuh"

namespace {
using namespace mc33;
using namespace runs;

struct ABox {
    int label;
    int o[3], n[3];            // sub-box origin and size (global voxel coordinates)
    long long arena;           // arena offset of the sub-box
    unsigned tile0;            // first smoothing column / voxel chunk item of this box
    unsigned chunk0;
    int full;                  // sub-box covers the whole volume
    int fail;                  // N2M status of this label (0 = ok)
    int vmin, vmax;            // ordered-int range of the smoothed sub-box
    int amin;                  // ordered-int min after clustering
    float iso, edge_max, pad;
    int blo[3], bhi[3];        // bbox of voxels >= iso (global)
    unsigned nbg, nfg;         // component counts
    unsigned long long best;   // largest component (size << 32 | ~root)
    // marching-cubes grid (global origin lo, size gn), filled by the host
    int glo[3], gn[3];
    unsigned WX, word0, ctile0;
    // clustering on x-runs: bit words per row, first row and first bit word across the boxes
    unsigned W, row0, bw0;
};

struct AtlasVol {
    const short *lab;
    int nx, ny, nz;
    long long nxy, nvox;
};

__device__ __forceinline__ int find_item(const ABox *b, int nb, unsigned item, unsigned ABox::*field) {
    int lo = 0, hi = nb - 1;
    while (lo < hi) {
        const int m = (lo + hi + 1) >> 1;
        if (b[m].*field <= item) lo = m;
        else hi = m - 1;
    }
    return lo;
}

// ---- S0: per-label voxel count, bounding box and the largest label ---------------
// A thread scans 32 consecutive voxels of a row and issues its atomics once per
// run of equal labels (labels are spatially coherent, so runs are long).
__device__ __forceinline__ void hist_flush(int l, int maxlab, unsigned c, int x0, int x1, int y, int z, unsigned *cnt,
                                           int *bb) {
    if (l < 1 || l > maxlab || !c) return;
    atomicAdd(&cnt[l], c);
    int *b = bb + 6 * l;
    atomicMin(b + 0, x0); atomicMin(b + 1, y); atomicMin(b + 2, z);
    atomicMax(b + 3, x1); atomicMax(b + 4, y); atomicMax(b + 5, z);
}

__global__ void k_a_hist(AtlasVol v, int maxlab, unsigned *cnt, int *bb, int *vmax) {
    int mx = 0;
    const unsigned spr = (unsigned)(v.nx + 31) / 32;
    const long long nseg = (long long)spr * v.ny * v.nz;
    for (long long sg = blockIdx.x * (long long)blockDim.x + threadIdx.x; sg < nseg; sg += (long long)gridDim.x * blockDim.x) {
        const long long row = sg / spr;
        const int xs = (int)(sg - row * spr) * 32;
        const int z = (int)(row / v.ny), y = (int)(row - (long long)z * v.ny);
        const short *p = v.lab + row * v.nx;
        int cur = -1, x0 = 0, x1 = 0;
        unsigned c = 0;
        const int xe = min(xs + 32, v.nx);
        for (int x = xs; x < xe; x++) {
            const int l = p[x];
            mx = max(mx, l);
            if (l != cur) {
                hist_flush(cur, maxlab, c, x0, x1, y, z, cnt, bb);
                cur = l;
                c = 0;
                x0 = x;
            }
            c++;
            x1 = x;
        }
        hist_flush(cur, maxlab, c, x0, x1, y, z, cnt, bb);
    }
    for (int o = 16; o; o >>= 1) mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    if ((threadIdx.x & 31) == 0) atomicMax(vmax, mx);
}

// ---- S1: binarise + pre-smooth every sub-box (one persistent launch) -------------
struct MaskSrc {
    const short *lab;
    int nx;
    long long nxy;
    int label;
    __device__ __forceinline__ float load(int x, int y, int z) const {
        return lab[(long long)z * nxy + (long long)y * nx + x] == label ? 1.f : 0.f;
    }
};
struct ArenaSink {
    float *a;
    int o0, o1, o2, n0, n1;
    __device__ __forceinline__ void put(int x, int y, int z, float v) {
        a[((long long)(z - o2) * n1 + (y - o1)) * n0 + (x - o0)] = v;
    }
};

__global__ void __launch_bounds__(smooth::NT, 2) k_a_smooth(AtlasVol v, ABox *boxes, int nb, unsigned nitems,
                                                          unsigned *queue, float *arena, bool smooth_on) {
    __shared__ unsigned item;
    __shared__ int bi;
    for (;;) {
        if (threadIdx.x == 0 && threadIdx.y == 0) {
            item = atomicAdd(queue, 1u);
            bi = item < nitems ? find_item(boxes, nb, item, &ABox::tile0) : 0;
        }
        __syncthreads();
        const unsigned it = item;
        const int b = bi;
        __syncthreads();
        if (it >= nitems) return;
        ABox &B = boxes[b];
        const unsigned local = it - B.tile0;
        const int tx = (B.n[0] + smooth::STX - 1) / smooth::STX, ty = (B.n[1] + smooth::STY - 1) / smooth::STY;
        const int cx = local % tx, cy = (local / tx) % ty, cz = local / (tx * ty);
        const int x0 = B.o[0] + cx * smooth::STX, y0 = B.o[1] + cy * smooth::STY, z0 = B.o[2] + cz * smooth::SZC;
        const int zend = min(z0 + smooth::SZC, B.o[2] + B.n[2]);
        MaskSrc src{v.lab, v.nx, v.nxy, B.label};
        ArenaSink sink{arena + B.arena, B.o[0], B.o[1], B.o[2], B.n[0], B.n[1]};
        smooth::Acc acc;
        acc.init();
        if (smooth_on) {
            smooth::column(src, sink, acc, 0.5f, x0, y0, z0, zend, B.o[0] + B.n[0], B.o[1] + B.n[1], v.nx, v.ny, v.nz);
        } else {
            const int gx = x0 + threadIdx.x, gy = y0 + threadIdx.y;
            if (gx < B.o[0] + B.n[0] && gy < B.o[1] + B.n[1])
                for (int z = z0; z < zend; z++) {
                    const float o = src.load(gx, gy, z);
                    sink.put(gx, gy, z, o);
                    acc.add(o, gx, gy, z, 0.5f);
                }
        }
        // range of this column into the box
        float mn = acc.mn, mx = acc.mx;
        for (int o = 16; o; o >>= 1) {
            mn = fminf(mn, __shfl_xor_sync(0xffffffffu, mn, o));
            mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
        }
        if (((threadIdx.y * blockDim.x + threadIdx.x) & 31) == 0 && mn <= mx) {
            atomicMin(&B.vmin, f2ord(mn));
            atomicMax(&B.vmax, f2ord(mx));
        }
        __syncthreads();
    }
}

// ---- S2: per-label isolevel (src/meshify.c:305-321 with iso 0.5) ------------------
__global__ void k_a_iso(ABox *boxes, int nb) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= nb) return;
    ABox &B = boxes[b];
    float mn = ord2f(B.vmin), mx = ord2f(B.vmax);
    if (!B.full) mn = fminf(mn, 0.f);   // voxels outside the sub-box are exactly 0
    float iso = 0.5f;
    if (mn == mx) B.fail = N2M_ERR_NO_VARIABILITY;
    if (iso <= mn || iso > mx) iso = (float)(0.5 * (double)__fadd_rn(mn, mx));
    B.iso = iso;
    B.vmin = f2ord(mn);
    B.edge_max = (float)(0.75 * (double)__fadd_rn(mn, iso));
    B.amin = INT_MAX;
}

// ---- S3: clustering on the arena ----------------------------------------------------
// voxels are processed in chunks of 1024 of one box
constexpr int CH = 1024;

struct VoxCtx {
    int b;
    long long i;         // arena index
    int x, y, z;         // local coordinates
};

template <class F>
__device__ __forceinline__ void for_chunks(const ABox *boxes, int nb, unsigned nchunks, unsigned *queue, unsigned ch, F f) {
    __shared__ unsigned item;
    __shared__ int bi;
    for (;;) {
        if (threadIdx.x == 0) {
            item = atomicAdd(queue, 1u);
            bi = item < nchunks ? find_item(boxes, nb, item, &ABox::chunk0) : 0;
        }
        __syncthreads();
        const unsigned it = item;
        const int b = bi;
        __syncthreads();
        if (it >= nchunks) return;
        const ABox &B = boxes[b];
        const unsigned n0 = (unsigned)B.n[0], n01 = (unsigned)B.n[0] * (unsigned)B.n[1];
        const unsigned nvb = n01 * (unsigned)B.n[2];
        for (unsigned k = threadIdx.x; k < ch; k += blockDim.x) {
            const unsigned loc = (it - B.chunk0) * ch + k;
            if (loc >= nvb) break;
            const unsigned z = loc / n01, r = loc - z * n01;
            const unsigned y = r / n0, x = r - y * n0;
            f(VoxCtx{b, B.arena + loc, (int)x, (int)y, (int)z}, B);
        }
    }
}

// The clustering of label.cu on every sub-box: class masks as bit words per
// box (bit x & 31 of word B.bw0 + (z*n1 + y)*B.W + x/32, local coordinates),
// union-find parents in L (arena-indexed) at the first voxel of each x-run
// only, boxes independent of one another.  A row kernel takes one row of one
// box per warp (lanes over its words, 32 at a time); rows and words are
// numbered across the boxes (B.row0, B.bw0).  The background's face contacts
// are the box's faces (src/meshify.c:332-336 on the binarised sub-box).
__device__ __forceinline__ bool skip_box(const ABox &B) { return B.fail != 0; }

__device__ __forceinline__ unsigned ab_valid(const ABox &B, unsigned w) {
    const int x0 = (int)w * 32;
    return x0 + 32 <= B.n[0] ? FULL : (1u << (B.n[0] - x0)) - 1u;
}
// foreground (want 1) or background (want 0) bits of word w of local row lr
__device__ __forceinline__ unsigned ab_class(const unsigned *Bits, const ABox &B, unsigned lr, unsigned w, unsigned want) {
    const unsigned b = Bits[B.bw0 + lr * B.W + w];
    return want ? b : ~b & ab_valid(B, w);
}

// class bits: smoothed value >= the box's isolevel
__global__ void __launch_bounds__(256) k_ab_bits(const ABox *boxes, int nb, unsigned nrows, const float *arena,
                                                 unsigned *Bits) {
    const int lane = threadIdx.x & 31;
    for (unsigned gr = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; gr < nrows; gr += (gridDim.x * blockDim.x) >> 5) {
        const ABox &B = boxes[find_item(boxes, nb, gr, &ABox::row0)];
        const unsigned lr = gr - B.row0;
        const float *rp = arena + B.arena + (long long)lr * B.n[0];
        for (unsigned w = 0; w < B.W; w++) {
            const int x = (int)w * 32 + lane;
            const unsigned m = __ballot_sync(FULL, x < B.n[0] && rp[x] >= B.iso);
            if (lane == 0) Bits[B.bw0 + lr * B.W + w] = m;
        }
    }
}

// every run start of the class links to itself; z8 / z32 (may be null) zeroed there
__global__ void k_ab_init(const ABox *boxes, int nb, unsigned nbw, const unsigned *__restrict__ Bits, unsigned want,
                          int *L, unsigned char *z8, unsigned *z32) {
    for (unsigned gw = blockIdx.x * blockDim.x + threadIdx.x; gw < nbw; gw += gridDim.x * blockDim.x) {
        const ABox &B = boxes[find_item(boxes, nb, gw, &ABox::bw0)];
        const unsigned lw = gw - B.bw0, lr = lw / B.W, w = lw - lr * B.W;
        const unsigned c = ab_class(Bits, B, lr, w, want), pc = w ? ab_class(Bits, B, lr, w - 1, want) : 0u;
        const long long base = B.arena + (long long)lr * B.n[0] + (long long)w * 32;
        for (unsigned st = c & ~((c << 1) | (pc >> 31)); st; st &= st - 1) {
            const int s = (int)(base + __ffs(st) - 1);
            L[s] = s;
            if (z8) z8[s] = 0;
            if (z32) z32[s] = 0;
        }
    }
}

// union of touching runs with the rows before them in the box (rows (y-1, z),
// (y, z-1), and for 18-connectivity x offsets -1..1 and rows (y-1, z-1),
// (y+1, z-1)); a contact counts where the voxels before it do not also touch
// A row kernel's rows: AB_SEG lanes per row (one word per lane, wider rows in
// chunks), 32 / AB_SEG rows per warp, each with its own box
constexpr int AB_SEG = 4;

template <int NNB>
__global__ void __launch_bounds__(256) k_ab_merge(const ABox *boxes, int nb, unsigned nrows,
                                                  const unsigned *__restrict__ Bits, unsigned want, int *L) {
    static_assert(NNB == 3 || NNB == 9, "6- or 18-connectivity");
    constexpr int NR = NNB == 3 ? 3 : 5;
    const int RY[5] = {0, -1, 0, -1, 1}, RZ[5] = {0, 0, -1, -1, -1};
    const int lane = threadIdx.x & 31, li = lane & (AB_SEG - 1);
    const unsigned rpw = 32u / AB_SEG, rsub = (unsigned)lane / AB_SEG, nwarps = (gridDim.x * blockDim.x) >> 5;
    for (unsigned rb = ((blockIdx.x * blockDim.x + threadIdx.x) >> 5) * rpw; rb < nrows; rb += nwarps * rpw) {
        const unsigned gr = rb + rsub;
        const ABox &B = boxes[gr < nrows ? find_item(boxes, nb, gr, &ABox::row0) : 0];
        const bool rowok = gr < nrows && !skip_box(B);
        const int n0 = B.n[0], n1 = B.n[1], n2 = B.n[2];
        const unsigned lr = rowok ? gr - B.row0 : 0u, W = rowok ? B.W : 0u;
        const int z = (int)(lr / (unsigned)n1), y = (int)(lr - (unsigned)z * (unsigned)n1);
        bool kok[NR];
        unsigned rk[NR];
#pragma unroll
        for (int k = 0; k < NR; k++) {
            const int yy = y + RY[k], zz = z + RZ[k];
            kok[k] = rowok && yy >= 0 && zz >= 0 && yy < n1 && zz < n2;
            rk[k] = kok[k] ? (unsigned)zz * (unsigned)n1 + (unsigned)yy : 0u;
        }
        int cst[NR];
        unsigned cwd[NR];
#pragma unroll
        for (int k = 0; k < NR; k++) { cst[k] = -1; cwd[k] = 0u; }
        const unsigned wmax = __reduce_max_sync(FULL, W);
        for (unsigned c0 = 0; c0 < wmax; c0 += AB_SEG) {
            const unsigned w = c0 + (unsigned)li;
            const bool ok = w < W;
            const int x0 = (int)w * 32;
            WordRuns R[NR];
            unsigned nk[NR];
#pragma unroll
            for (int k = 0; k < NR; k++) {
                const unsigned c = ok && kok[k] ? ab_class(Bits, B, rk[k], w, want) : 0u;
                R[k] = word_runs(c, x0, li, AB_SEG, cst[k], cwd[k]);
                const unsigned dn = __shfl_down_sync(FULL, c, 1, AB_SEG);
                nk[k] = li < AB_SEG - 1 ? (w + 1 < W ? dn : 0u)
                                        : (kok[k] && w + 1 < W ? ab_class(Bits, B, rk[k], w + 1, want) : 0u);
            }
            const unsigned F = R[0].c;
            if (!F) continue;
            const unsigned left = (F << 1) | (R[0].pc >> 31);
            auto S = [&](int k, int dx) -> unsigned {
                const WordRuns &q = R[k];
                return dx == 0 ? q.c : dx == 1 ? (q.c >> 1) | (nk[k] << 31)
                                     : dx == -1 ? (q.c << 1) | (q.pc >> 31) : (q.c << 2) | (q.pc >> 30);
            };
            const long long base0 = B.arena + (long long)lr * n0;
            auto link = [&](int k, int dx) {
                unsigned m = F & S(k, dx) & ~(left & S(k, dx - 1));
                if (!m) return;
                const WordRuns &q = R[k];
                const long long basek = B.arena + (long long)rk[k] * n0;
                for (; m; m &= m - 1) {
                    const int b = __ffs(m) - 1, xx = b + dx;
                    const int sk = xx < 0 ? q.cs : xx > 31 ? ((q.c >> 31) & 1u ? q.start_of(31) : x0 + 32) : q.start_of(xx);
                    const int i = (int)(base0 + R[0].start_of(b)), j = (int)(basek + sk);
                    if (L[i] != L[j]) uf::unite(L, i, j);
                }
            };
            link(1, 0);
            link(2, 0);
            if constexpr (NNB == 9) {
                link(1, -1); link(1, 1); link(2, -1); link(2, 1); link(3, 0); link(4, 0);
            }
        }
    }
}

// every run start points at its root (read-only root search: the one store is
// the final root); roots are counted per box
__global__ void k_ab_flatten(ABox *boxes, int nb, unsigned nbw, const unsigned *__restrict__ Bits, unsigned want, int *L,
                             bool fg) {
    for (unsigned gw = blockIdx.x * blockDim.x + threadIdx.x; gw < nbw; gw += gridDim.x * blockDim.x) {
        const int b = find_item(boxes, nb, gw, &ABox::bw0);
        const ABox &B = boxes[b];
        const unsigned lw = gw - B.bw0, lr = lw / B.W, w = lw - lr * B.W;
        const unsigned c = ab_class(Bits, B, lr, w, want), pc = w ? ab_class(Bits, B, lr, w - 1, want) : 0u;
        const long long base = B.arena + (long long)lr * B.n[0] + (long long)w * 32;
        unsigned nroots = 0;
        for (unsigned st = c & ~((c << 1) | (pc >> 31)); st; st &= st - 1) {
            const int s = (int)(base + __ffs(st) - 1);
            const int root = uf::find_root(L, s);
            if (root == s) nroots++;
            else L[s] = root;
        }
        if (nroots) atomicAdd(fg ? &boxes[b].nfg : &boxes[b].nbg, nroots);
    }
}

// background components touching a face of the box flag their root: every run
// of a row on a y or z face, the runs holding x = 0 and x = n0-1 of the others
__global__ void k_ab_edges(const ABox *boxes, int nb, unsigned nbw, const unsigned *__restrict__ Bits, const int *L,
                           unsigned char *edge) {
    for (unsigned gw = blockIdx.x * blockDim.x + threadIdx.x; gw < nbw; gw += gridDim.x * blockDim.x) {
        const ABox &B = boxes[find_item(boxes, nb, gw, &ABox::bw0)];
        const int n0 = B.n[0], n1 = B.n[1], n2 = B.n[2];
        const unsigned lw = gw - B.bw0, lr = lw / B.W, w = lw - lr * B.W;
        const int z = (int)(lr / (unsigned)n1), y = (int)(lr - (unsigned)z * (unsigned)n1);
        const unsigned c = ab_class(Bits, B, lr, w, 0u);
        if (!c) continue;
        const long long base = B.arena + (long long)lr * n0;
        auto mark = [&](long long j) {
            const int r = L[j];
            if (!edge[r]) edge[r] = 1;
        };
        if (y == 0 || z == 0 || y == n1 - 1 || z == n2 - 1) {
            const unsigned pc = w ? ab_class(Bits, B, lr, w - 1, 0u) : 0u;
            for (unsigned st = c & ~((c << 1) | (pc >> 31)); st; st &= st - 1) mark(base + w * 32 + __ffs(st) - 1);
            continue;
        }
        if (w == 0 && (c & 1u)) mark(base);
        if (w == B.W - 1) {
            int b = (n0 - 1) & 31;
            if (!((c >> b) & 1u)) continue;
            unsigned ww = w, cc = c;
            for (;;) {   // back to the run's start (x = 0 of a background run is one)
                const unsigned pc = ww ? ab_class(Bits, B, lr, ww - 1, 0u) : 0u;
                const int ls = last_start(cc & ~((cc << 1) | (pc >> 31)), (int)ww * 32, b);
                if (ls >= 0) {
                    mark(base + ls);
                    break;
                }
                ww--;
                b = 31;
                cc = pc;
            }
        }
    }
}

// bubbles (background components away from the box faces) become foreground,
// when the box's background has at least two components (src/bwlabel.c:488-491)
__global__ void __launch_bounds__(256) k_ab_fill(const ABox *boxes, int nb, unsigned nrows, unsigned *Bits, const int *L,
                                                 const unsigned char *__restrict__ edge) {
    const int lane = threadIdx.x & 31, li = lane & (AB_SEG - 1);
    const unsigned rpw = 32u / AB_SEG, rsub = (unsigned)lane / AB_SEG, nwarps = (gridDim.x * blockDim.x) >> 5;
    for (unsigned rb = ((blockIdx.x * blockDim.x + threadIdx.x) >> 5) * rpw; rb < nrows; rb += nwarps * rpw) {
        const unsigned gr = rb + rsub;
        const ABox &B = boxes[gr < nrows ? find_item(boxes, nb, gr, &ABox::row0) : 0];
        const bool rowok = gr < nrows && B.nbg > 1;
        const unsigned lr = rowok ? gr - B.row0 : 0u, W = rowok ? B.W : 0u;
        const long long base = B.arena + (long long)lr * B.n[0];
        int cst = -1;
        unsigned cwd = 0;
        const unsigned wmax = __reduce_max_sync(FULL, W);
        for (unsigned c0 = 0; c0 < wmax; c0 += AB_SEG) {
            const unsigned w = c0 + (unsigned)li;
            const unsigned c = w < W ? ab_class(Bits, B, lr, w, 0u) : 0u;
            const WordRuns R = word_runs(c, (int)w * 32, li, AB_SEG, cst, cwd);
            unsigned fill = 0;
            for (unsigned rem = c; rem;) {
                const int b = __ffs(rem) - 1;
                const unsigned pm = piece_at(rem, b);
                rem &= ~pm;
                if (!edge[L[base + R.start_of(b)]]) fill |= pm;
            }
            // every lane has read its neighbours' words (word_runs) before any write
            if (fill) Bits[B.bw0 + lr * B.W + w] |= fill;
        }
    }
}

// component sizes at the roots (each run adds its length at its end)
__global__ void __launch_bounds__(256) k_ab_sizes(const ABox *boxes, int nb, unsigned nrows,
                                                  const unsigned *__restrict__ Bits, const int *L, unsigned *cnt) {
    const int lane = threadIdx.x & 31, li = lane & (AB_SEG - 1);
    const unsigned rpw = 32u / AB_SEG, rsub = (unsigned)lane / AB_SEG, nwarps = (gridDim.x * blockDim.x) >> 5;
    for (unsigned rb = ((blockIdx.x * blockDim.x + threadIdx.x) >> 5) * rpw; rb < nrows; rb += nwarps * rpw) {
        const unsigned gr = rb + rsub;
        const ABox &B = boxes[gr < nrows ? find_item(boxes, nb, gr, &ABox::row0) : 0];
        const bool rowok = gr < nrows;
        const unsigned lr = rowok ? gr - B.row0 : 0u, W = rowok ? B.W : 0u;
        const long long base = B.arena + (long long)lr * B.n[0];
        int cst = -1;
        unsigned cwd = 0;
        const unsigned wmax = __reduce_max_sync(FULL, W);
        for (unsigned c0 = 0; c0 < wmax; c0 += AB_SEG) {
            const unsigned w = c0 + (unsigned)li;
            const unsigned c = w < W ? ab_class(Bits, B, lr, w, 1u) : 0u;
            const WordRuns R = word_runs(c, (int)w * 32, li, AB_SEG, cst, cwd);
            const unsigned dn = __shfl_down_sync(FULL, c, 1, AB_SEG);
            const unsigned nxt = li < AB_SEG - 1 ? (w + 1 < W ? dn : 0u) : (w + 1 < W ? ab_class(Bits, B, lr, w + 1, 1u) : 0u);
            for (unsigned ends = c & ~((c >> 1) | (nxt << 31)); ends; ends &= ends - 1) {
                const int e = __ffs(ends) - 1, st = R.start_of(e);
                atomicAdd(&cnt[L[base + st]], (unsigned)(R.x0 + e - st + 1));
            }
        }
    }
}

// largest component per box; ties go to the smallest root (first in raster order)
__global__ void k_ab_best(ABox *boxes, int nb, unsigned nbw, const unsigned *__restrict__ Bits, const int *L,
                          const unsigned *__restrict__ cnt) {
    for (unsigned gw = blockIdx.x * blockDim.x + threadIdx.x; gw < nbw; gw += gridDim.x * blockDim.x) {
        const int b = find_item(boxes, nb, gw, &ABox::bw0);
        const ABox &B = boxes[b];
        const unsigned lw = gw - B.bw0, lr = lw / B.W, w = lw - lr * B.W;
        const unsigned c = ab_class(Bits, B, lr, w, 1u), pc = w ? ab_class(Bits, B, lr, w - 1, 1u) : 0u;
        const long long base = B.arena + (long long)lr * B.n[0] + (long long)w * 32;
        for (unsigned st = c & ~((c << 1) | (pc >> 31)); st; st &= st - 1) {
            const int s = (int)(base + __ffs(st) - 1);
            if (L[s] != s) continue;
            const unsigned loc = (unsigned)(s - B.arena);
            atomicMax(&boxes[b].best, ((unsigned long long)cnt[s] << 32) | (0xffffffffu - loc));
        }
    }
}

// bits of the voxels of each box's largest component
__global__ void __launch_bounds__(256) k_ab_keep(const ABox *boxes, int nb, unsigned nrows, const unsigned *__restrict__ Bits,
                                                 const int *L, unsigned *K) {
    const int lane = threadIdx.x & 31, li = lane & (AB_SEG - 1);
    const unsigned rpw = 32u / AB_SEG, rsub = (unsigned)lane / AB_SEG, nwarps = (gridDim.x * blockDim.x) >> 5;
    for (unsigned rb = ((blockIdx.x * blockDim.x + threadIdx.x) >> 5) * rpw; rb < nrows; rb += nwarps * rpw) {
        const unsigned gr = rb + rsub;
        const ABox &B = boxes[gr < nrows ? find_item(boxes, nb, gr, &ABox::row0) : 0];
        const bool rowok = gr < nrows;
        const long long root = B.best ? B.arena + (long long)(0xffffffffu - (unsigned)(B.best & 0xffffffffu)) : -2;
        const unsigned lr = rowok ? gr - B.row0 : 0u, W = rowok ? B.W : 0u;
        const long long base = B.arena + (long long)lr * B.n[0];
        int cst = -1;
        unsigned cwd = 0;
        const unsigned wmax = __reduce_max_sync(FULL, W);
        for (unsigned c0 = 0; c0 < wmax; c0 += AB_SEG) {
            const unsigned w = c0 + (unsigned)li;
            const unsigned c = w < W ? ab_class(Bits, B, lr, w, 1u) : 0u;
            const WordRuns R = word_runs(c, (int)w * 32, li, AB_SEG, cst, cwd);
            unsigned keep = 0;
            for (unsigned rem = c; rem;) {
                const int b = __ffs(rem) - 1;
                const unsigned pm = piece_at(rem, b);
                rem &= ~pm;
                if ((long long)L[base + R.start_of(b)] == root) keep |= pm;
            }
            if (w < W) K[B.bw0 + lr * B.W + w] = keep;
        }
    }
}

// The clustered sub-box (src/meshify.c:332-342): kept voxels (K) raised to the
// box's isolevel when FILL; with LARGEST, a voxel neither kept nor, away from
// the volume faces, next to a kept voxel (all 26 neighbours except
// (-1,-1,-1), src/meshify.c:252) becomes the box minimum.  A warp per row; the
// dilation bits of 32 words at a time lane-parallel (lane l: word c0 + l).
template <bool LARGEST, bool FILL>
__global__ void __launch_bounds__(256) k_ab_final(const ABox *boxes, int nb, unsigned nrows, const unsigned *__restrict__ K,
                                                  float *arena, int nx, int ny, int nz) {
    const int lane = threadIdx.x & 31;
    const int DY[9] = {-1, 0, 1, -1, 0, 1, 0, 1, -1}, DZ[9] = {0, 0, 0, 1, 1, 1, -1, -1, -1};
    for (unsigned gr = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; gr < nrows; gr += (gridDim.x * blockDim.x) >> 5) {
        const ABox &B = boxes[find_item(boxes, nb, gr, &ABox::row0)];
        const int n0 = B.n[0], n1 = B.n[1], n2 = B.n[2];
        const unsigned lr = gr - B.row0, W = B.W;
        const int z = (int)(lr / (unsigned)n1), y = (int)(lr - (unsigned)z * (unsigned)n1);
        float *row = arena + B.arena + (long long)lr * n0;
        const unsigned *K0 = K + B.bw0;
        if (!LARGEST) {
            for (unsigned w = 0; w < W; w++) {
                const unsigned kw = K0[lr * W + w];
                const int x = (int)w * 32 + lane;
                if (x < n0 && ((kw >> lane) & 1u)) row[x] = fmaxf(row[x], B.iso);
            }
            continue;
        }
        const float vmin = ord2f(B.vmin);
        const int gy = B.o[1] + y, gz = B.o[2] + z;
        const bool ryz = gy > 0 && gz > 0 && gy < ny - 1 && gz < nz - 1;
        unsigned carry[9];
#pragma unroll
        for (int k = 0; k < 9; k++) carry[k] = 0u;
        for (unsigned c0 = 0; c0 < W; c0 += 32) {
            unsigned on = 0u, kept = 0u;
#pragma unroll
            for (int k = 0; k < 9; k++) {
                const int yy = y + DY[k], zz = z + DZ[k];
                const bool in = yy >= 0 && zz >= 0 && yy < n1 && zz < n2;
                const unsigned rb = in ? ((unsigned)zz * (unsigned)n1 + (unsigned)yy) * W : 0u;
                const unsigned cur = in && c0 + lane < W ? K0[rb + c0 + lane] : 0u;
                unsigned prv = __shfl_up_sync(FULL, cur, 1), nxt = __shfl_down_sync(FULL, cur, 1);
                if (lane == 0) prv = carry[k];
                if (lane == 31) nxt = in && c0 + 32 < W ? K0[rb + c0 + 32] : 0u;
                carry[k] = __shfl_sync(FULL, cur, 31);
                on |= cur | (cur >> 1) | (nxt << 31) | (k < 8 ? (cur << 1) | (prv >> 31) : 0u);   // row 8: no K(x-1)
                if (k == 1) kept = cur;
            }
            const unsigned wend = min(W, c0 + 32);
            if (!__any_sync(FULL, on != 0u)) {   // nothing kept within reach
                for (int x = (int)c0 * 32 + lane; x < min(n0, (int)wend * 32); x += 32) row[x] = vmin;
                continue;
            }
            for (unsigned w = c0; w < wend; w++) {
                const unsigned onw = __shfl_sync(FULL, on, (int)(w - c0)), kw = __shfl_sync(FULL, kept, (int)(w - c0));
                const int x = (int)w * 32 + lane;
                if (x >= n0) continue;
                const bool kp = (kw >> lane) & 1u;
                const int gx = B.o[0] + x;
                const bool interior = ryz && gx > 0 && gx < nx - 1;
                if (!(kp || (interior && ((onw >> lane) & 1u)))) row[x] = vmin;
                else if (FILL && kp) row[x] = fmaxf(row[x], B.iso);
            }
        }
    }
}

// ---- S4: bbox of voxels >= iso and the range after clustering -------------------------
// reduced per chunk (all its voxels belong to one box): one set of atomics per chunk
__global__ void __launch_bounds__(256) k_a_stats(ABox *boxes, int nb, unsigned nch, unsigned *queue, unsigned ch,
                                                 const float *arena) {
    __shared__ unsigned item;
    __shared__ int bi;
    __shared__ int red[8][7];
    for (;;) {
        if (threadIdx.x == 0) {
            item = atomicAdd(queue, 1u);
            bi = item < nch ? find_item(boxes, nb, item, &ABox::chunk0) : 0;
        }
        __syncthreads();
        const unsigned it = item;
        const int b = bi;
        __syncthreads();
        if (it >= nch) return;
        const ABox &B = boxes[b];
        const unsigned n0 = (unsigned)B.n[0], n01 = (unsigned)B.n[0] * (unsigned)B.n[1], nvb = n01 * (unsigned)B.n[2];
        int v[7] = {INT_MAX, INT_MAX, INT_MAX, INT_MAX, INT_MIN, INT_MIN, INT_MIN};   // amin, lo xyz, hi xyz
        for (unsigned k = threadIdx.x; k < ch; k += blockDim.x) {
            const unsigned loc = (it - B.chunk0) * ch + k;
            if (loc >= nvb) break;
            const float f = arena[B.arena + loc];
            v[0] = min(v[0], f2ord(f));
            if (f >= B.iso) {
                const unsigned z = loc / n01, r = loc - z * n01, y = r / n0, x = r - y * n0;
                v[1] = min(v[1], (int)x); v[2] = min(v[2], (int)y); v[3] = min(v[3], (int)z);
                v[4] = max(v[4], (int)x); v[5] = max(v[5], (int)y); v[6] = max(v[6], (int)z);
            }
        }
        for (int o = 16; o; o >>= 1)
            for (int j = 0; j < 7; j++) {
                const int t = __shfl_xor_sync(0xffffffffu, v[j], o);
                v[j] = j < 4 ? min(v[j], t) : max(v[j], t);
            }
        if ((threadIdx.x & 31) == 0)
            for (int j = 0; j < 7; j++) red[threadIdx.x >> 5][j] = v[j];
        __syncthreads();
        if (threadIdx.x == 0) {
            for (int w = 1; w < (int)(blockDim.x >> 5); w++)
                for (int j = 0; j < 7; j++) v[j] = j < 4 ? min(v[j], red[w][j]) : max(v[j], red[w][j]);
            ABox &W = boxes[b];
            atomicMin(&W.amin, v[0]);
            if (v[1] != INT_MAX) {
                atomicMin(&W.blo[0], B.o[0] + v[1]); atomicMin(&W.blo[1], B.o[1] + v[2]); atomicMin(&W.blo[2], B.o[2] + v[3]);
                atomicMax(&W.bhi[0], B.o[0] + v[4]); atomicMax(&W.bhi[1], B.o[1] + v[5]); atomicMax(&W.bhi[2], B.o[2] + v[6]);
            }
        }
        __syncthreads();
    }
}

__global__ void k_a_pad(ABox *boxes, int nb) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= nb) return;
    ABox &B = boxes[b];
    float amin = ord2f(B.amin);
    if (!B.full) amin = fminf(amin, 0.f);
    B.pad = __fsub_rn(fminf(amin, B.edge_max), B.iso);
}

// ---- S5-S7: marching cubes over every label's padded grid ------------------------------
// grid value (x,y,z) of box B minus isolevel, as the single-volume gval
__device__ __forceinline__ float agval(const AtlasVol &v, const ABox &B, const float *arena, int x, int y, int z) {
    const long long j = (long long)(B.glo[0] + x) + (long long)(y + B.glo[1]) * v.nx + (long long)(z + B.glo[2]) * v.nxy;
    float val;
    if (j < v.nvox) {
        // the box grid ends at the volume's dims: a coordinate past them by one wraps into the next row / slice
        int vx = B.glo[0] + x, vy = y + B.glo[1], vz = z + B.glo[2];
        if (vx >= v.nx) {
            vx -= v.nx;
            vy++;
        }
        if (vy >= v.ny) {
            vy -= v.ny;
            vz++;
        }
        const int lx = vx - B.o[0], ly = vy - B.o[1], lz = vz - B.o[2];
        val = (lx >= 0 && ly >= 0 && lz >= 0 && lx < B.n[0] && ly < B.n[1] && lz < B.n[2])
                  ? arena[B.arena + ((long long)lz * B.n[1] + ly) * B.n[0] + lx]
                  : 0.f;
        if (vx == 0 || vy == 0 || vz == 0 || vx == v.nx - 1 || vy == v.ny - 1 || vz == v.nz - 1)
            val = fminf(B.edge_max, val);
        val = __fsub_rn(val, B.iso);
    } else {
        val = B.pad;
    }
    if (fabsf(val) < N2M_FLT_EPS) val = N2M_FLT_EPS;
    return val;
}

constexpr int TY = 8, TZ = 8;

__global__ void __launch_bounds__(256) k_a_count(AtlasVol v, const ABox *boxes, int nb, unsigned nitems, unsigned *queue,
                                                 const float *arena, bool classic, uint4 *words, uint4 *counts,
                                                 unsigned *active, unsigned *nactive) {
    __shared__ float sv[TZ + 1][TY + 1][33];
    __shared__ unsigned item;
    __shared__ int bi;
    for (;;) {
        if (threadIdx.x == 0) {
            item = atomicAdd(queue, 1u);
            bi = item < nitems ? find_item(boxes, nb, item, &ABox::ctile0) : 0;
        }
        __syncthreads();
        const unsigned it = item;
        const int b = bi;
        if (it >= nitems) return;
        const ABox &B = boxes[b];
        const unsigned local = it - B.ctile0;
        const int ty = (B.gn[1] + TY - 1) / TY;
        const int cx = local % B.WX, cy = (local / B.WX) % ty, cz = local / (B.WX * ty);
        const int x0 = cx * 32, y0 = cy * TY, z0 = cz * TZ;
        for (int i = threadIdx.x; i < (TZ + 1) * (TY + 1) * 33; i += 256) {
            const int xx = i % 33, r = i / 33, yy = r % (TY + 1), zz = r / (TY + 1);
            sv[zz][yy][xx] = agval(v, B, arena, x0 + xx, y0 + yy, z0 + zz);
        }
        __syncthreads();
        const int wy = threadIdx.x >> 5, lane = threadIdx.x & 31;
        const int y = y0 + wy, x = x0 + lane;
        if (y < B.gn[1]) {
            for (int zz = 0; zz < TZ; zz++) {
                const int z = z0 + zz;
                if (z >= B.gn[2]) break;
                const bool in = x < B.gn[0];
                const bool hx = in && x < B.gn[0] - 1, hy = in && y < B.gn[1] - 1, hz = in && z < B.gn[2] - 1;
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
                    const unsigned w = B.word0 + ((unsigned)z * (unsigned)B.gn[1] + (unsigned)y) * B.WX + (unsigned)cx;
                    const unsigned nv = __popc(xm) + __popc(ym) + __popc(zm);
                    const bool act = nv | nt | nc;
                    words[w] = make_uint4(xm, ym, zm, 0u);
                    counts[w] = make_uint4(nv, (unsigned)nt, (unsigned)nc, act);
                    if (act) active[atomicAdd(nactive, 1u)] = w;
                }
            }
        }
        __syncthreads();
    }
}

__device__ __forceinline__ int avid(const uint4 *__restrict__ words, const uint4 *__restrict__ offs, const ABox &B,
                                    unsigned cshift, int x, int y, int z, int axis) {
    const unsigned w = B.word0 + ((unsigned)z * (unsigned)B.gn[1] + (unsigned)y) * B.WX + ((unsigned)x >> 5);
    const unsigned l = (unsigned)x & 31u;
    const uint4 m = words[w];
    const unsigned lt = (1u << l) - 1u;
    unsigned id = offs[w].x + cshift + __popc(m.x & lt) + __popc(m.y & lt) + __popc(m.z & lt);
    if (axis >= 1) id += (m.x >> l) & 1u;
    if (axis == 2) id += (m.y >> l) & 1u;
    return (int)id;
}

// per box: the scan values at its first word (edge vertices, triangles and
// c-vertices of all earlier boxes), from which its contiguous ranges follow
struct BoxOff {
    unsigned e, t, c;
};

__global__ void k_a_emit(AtlasVol v, const ABox *boxes, const BoxOff *boff, int nb, const uint4 *__restrict__ words,
                         const uint4 *__restrict__ offs, const unsigned *__restrict__ active, unsigned nactive,
                         const float *arena, bool classic, vec3d *pts, vec3i *tris, int *cand, unsigned *ncand,
                         int *ccand, unsigned *nccand, int cap) {
    const unsigned lane = threadIdx.x & 31u;
    for (unsigned aw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; aw < nactive; aw += (gridDim.x * blockDim.x) >> 5) {
        const unsigned w = active[aw];
        const int b = find_item(boxes, nb, w, &ABox::word0);
        const ABox &B = boxes[b];
        const unsigned cshift = boff[b].c;                        // c-vertices of earlier boxes
        const unsigned cbase = boff[b + 1].e + 0u;                // this box's c-vertices follow its edge vertices
        const unsigned lw = w - B.word0;
        const unsigned row = lw / B.WX, xw = lw - row * B.WX;
        const int z = (int)(row / (unsigned)B.gn[1]), y = (int)(row - (unsigned)z * (unsigned)B.gn[1]);
        const int x = (int)(xw * 32u + lane);
        const uint4 o = offs[w];
        const uint4 m = words[w];
        const bool in = x < B.gn[0];
        const bool hx = in && x < B.gn[0] - 1, hy = in && y < B.gn[1] - 1, hz = in && z < B.gn[2] - 1;
        const bool cube = hx && hy && hz;
        const bool ex = (m.x >> lane) & 1u, ey = (m.y >> lane) & 1u, ez = (m.z >> lane) & 1u;
        float c[8];
        if (in) {
            c[0] = agval(v, B, arena, x, y, z);
            c[1] = hx ? agval(v, B, arena, x + 1, y, z) : c[0];
            c[3] = hy ? agval(v, B, arena, x, y + 1, z) : c[0];
            c[4] = hz ? agval(v, B, arena, x, y, z + 1) : c[0];
            if (cube) {
                c[2] = agval(v, B, arena, x + 1, y + 1, z);
                c[5] = agval(v, B, arena, x + 1, y, z + 1);
                c[6] = agval(v, B, arena, x + 1, y + 1, z + 1);
                c[7] = agval(v, B, arena, x, y + 1, z + 1);
            }
        }
        const float flo0 = (float)B.glo[0], flo1 = (float)B.glo[1], flo2 = (float)B.glo[2];
        if (ex | ey | ez) {
            const unsigned lt = (1u << lane) - 1u;
            int id = (int)(o.x + cshift + __popc(m.x & lt) + __popc(m.y & lt) + __popc(m.z & lt));
            const float fx = (float)x, fy = (float)y, fz = (float)z;
            if (ex) {
                const float X = __fadd_rn(__fadd_rn(fx, edge_u(c[0], c[1])), flo0);
                pts[id] = {(double)X, (double)__fadd_rn(fy, flo1), (double)__fadd_rn(fz, flo2)};
                if (frac_dist(X) < 1.5e-5f) { unsigned k = atomicAdd(ncand, 1u); if (k < (unsigned)cap) cand[k] = id; }
                id++;
            }
            if (ey) {
                const float Y = __fadd_rn(__fadd_rn(fy, edge_u(c[0], c[3])), flo1);
                pts[id] = {(double)__fadd_rn(fx, flo0), (double)Y, (double)__fadd_rn(fz, flo2)};
                if (frac_dist(Y) < 1.5e-5f) { unsigned k = atomicAdd(ncand, 1u); if (k < (unsigned)cap) cand[k] = id; }
                id++;
            }
            if (ez) {
                const float Z = __fadd_rn(__fadd_rn(fz, edge_u(c[0], c[4])), flo2);
                pts[id] = {(double)__fadd_rn(fx, flo0), (double)__fadd_rn(fy, flo1), (double)Z};
                if (frac_dist(Z) < 1.5e-5f) { unsigned k = atomicAdd(ncand, 1u); if (k < (unsigned)cap) cand[k] = id; }
            }
        }
        Tiling T = {0, 0, false};
        if (cube) {
            const int lut = cube_lut(c);
            if (lut != 0 && lut != 255) T = select_tiling(c, lut, classic);
        }
        int tb = T.n, cb = T.cv;
        for (int d = 1; d < 32; d <<= 1) {
            const int a = __shfl_up_sync(0xffffffffu, tb, d), bb = __shfl_up_sync(0xffffffffu, cb, d);
            if ((int)lane >= d) { tb += a; cb += bb; }
        }
        tb -= T.n;
        cb -= T.cv;
        if (T.n == 0) continue;
        int v12 = -1;
        if (T.cv) {
            v12 = (int)(cbase + o.z + cb);
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
            if (fminf(frac_dist(X), fminf(frac_dist(Y), frac_dist(Z))) < 1.5e-5f) {
                unsigned k = atomicAdd(nccand, 1u);
                if (k < (unsigned)cap) ccand[k] = v12;
            }
        }
        int tv[3];
        for (int t = 0; t < 3 * T.n; t++) {
            const int code = d_lut[T.off + t];
            int vv;
            switch (code) {
            case 0: vv = avid(words, offs, B, cshift, x, y, z, 0); break;
            case 1: vv = avid(words, offs, B, cshift, x + 1, y, z, 1); break;
            case 2: vv = avid(words, offs, B, cshift, x, y + 1, z, 0); break;
            case 3: vv = avid(words, offs, B, cshift, x, y, z, 1); break;
            case 4: vv = avid(words, offs, B, cshift, x, y, z + 1, 0); break;
            case 5: vv = avid(words, offs, B, cshift, x + 1, y, z + 1, 1); break;
            case 6: vv = avid(words, offs, B, cshift, x, y + 1, z + 1, 0); break;
            case 7: vv = avid(words, offs, B, cshift, x, y, z + 1, 1); break;
            case 8: vv = avid(words, offs, B, cshift, x, y, z, 2); break;
            case 9: vv = avid(words, offs, B, cshift, x + 1, y, z, 2); break;
            case 10: vv = avid(words, offs, B, cshift, x + 1, y + 1, z, 2); break;
            case 11: vv = avid(words, offs, B, cshift, x, y + 1, z, 2); break;
            case 12: vv = v12; break;
            default: vv = -1; break;
            }
            tv[t % 3] = vv;
            if (t % 3 == 2) tris[o.y + tb + t / 3] = {tv[2], tv[1], tv[0]};
        }
    }
}

// scan values at the first word of every box (and the totals after the last)
__global__ void k_a_boxoff(const ABox *boxes, int nb, const uint4 *offs, uint4 total, BoxOff *boff) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b > nb) return;
    if (b == nb) {
        boff[b] = {total.x, total.y, total.z};
        return;
    }
    const uint4 o = offs[boxes[b].word0];
    boff[b] = {o.x, o.y, o.z};
}

// binarise the whole volume for one label (the per-label loop)
__global__ void k_binarize(const short *lab, long long n, int label, float *out) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        out[i] = lab[i] == label ? 1.f : 0.f;
}

__global__ void k_offset_tris(vec3i *t, int n, int off) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        t[i].x -= off; t[i].y -= off; t[i].z -= off;
    }
}
}  // namespace


// ---- host side ------------------------------------------------------------------------
namespace {
inline unsigned pgrid(unsigned items, unsigned per_sm) {
    const unsigned cap = 152u * per_sm;
    return std::max(1u, std::min(items, cap));
}

double d3(const vec3d &a, const vec3d &b) {
    const double dx = a.x - b.x, dy = a.y - b.y, dz = a.z - b.z;
    return sqrt(dx * dx + dy * dy + dz * dz);
}
uint32_t kbits(float f) {
    uint32_t u;
    memcpy(&u, &f, 4);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}

__global__ void k_a_fill_bb(int *bb, int n) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) bb[i] = (i % 6) < 3 ? INT_MAX : INT_MIN;
}

__global__ void k_a_gather(const vec3d *p, const int *ids, int n, vec3d *out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = p[ids[i]];
}

// kept triangles before each box's first triangle, from the degenerate filter's flags
__global__ void k_a_kept(const unsigned *tri_start, int nb, const unsigned *flags, const unsigned *tile_off, int tile,
                         unsigned total_kept, unsigned *kept_before) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b > nb) return;
    const unsigned t = tri_start[b];
    unsigned k;
    if (b == nb) k = total_kept;
    else {
        const unsigned tb = t / tile;
        k = tile_off[tb];
        for (unsigned i = tb * tile; i < t; i++) k += flags[i];
    }
    kept_before[b] = k;
}

// triangle indices relative to their own mesh
__global__ void k_a_localize(vec3i *t, unsigned nt, const unsigned *tri_start, const unsigned *vert_start, int nb) {
    for (unsigned i = blockIdx.x * blockDim.x + threadIdx.x; i < nt; i += gridDim.x * blockDim.x) {
        int lo = 0, hi = nb - 1;
        while (lo < hi) {
            const int m = (lo + hi + 1) >> 1;
            if (tri_start[m] <= i) lo = m;
            else hi = m - 1;
        }
        const int o = (int)vert_start[lo];
        t[i].x -= o; t[i].y -= o; t[i].z -= o;
    }
}
}  // namespace

namespace {
unsigned set_chunks(std::vector<ABox> &boxes, unsigned ch) {
    unsigned chunks = 0;
    for (auto &B : boxes) {
        B.chunk0 = chunks;
        chunks += (unsigned)(((long long)B.n[0] * B.n[1] * B.n[2] + ch - 1) / ch);
    }
    return chunks;
}

// smoothing, isolevel, clustering and range/bbox: device-only work (no host
// synchronisation), enqueued for timing by the autotuner or captured as a graph
struct Segment {
    AtlasVol v;
    ABox *db;
    int nb;
    unsigned tiles;
    float *ar;
    bool smooth_on, only_largest, fill_bubbles;
    int nx, ny, nz;
    unsigned *q;
    long long arena;
    unsigned nrows, nbw;   // rows and bit words of all the boxes

    n2m_status ensure(AtlasWork &w) {
        if (only_largest || fill_bubbles) {
            CKS(w.mask.ensure((size_t)nbw * sizeof(unsigned)));
            if (only_largest) CKS(w.keep.ensure((size_t)nbw * sizeof(unsigned)));
            CKS(w.lab.ensure((size_t)arena * sizeof(int)));
            if (fill_bubbles) CKS(w.edge.ensure((size_t)arena));
            if (only_largest) CKS(w.ucnt.ensure((size_t)arena * sizeof(unsigned)));
        }
        return N2M_OK;
    }

    n2m_status enqueue(AtlasWork &w, unsigned ch, unsigned per_sm, unsigned chunks, cudaStream_t s) {
        int qi = 0;
        CK(cudaMemsetAsync(q, 0, 32 * sizeof(unsigned), s));
        { k_a_smooth<<<pgrid(tiles, 2), dim3(smooth::STX, smooth::STY), 0, s>>>(v, db, nb, tiles, q + qi++, ar, smooth_on); N2M_COUNT(); }
        { k_a_iso<<<(nb + 127) / 128, 128, 0, s>>>(db, nb); N2M_COUNT(); }
        const unsigned g = pgrid(chunks, per_sm);
        if (only_largest || fill_bubbles) {
            unsigned *Bm = w.mask.as<unsigned>();
            int *L = w.lab.as<int>();
            const unsigned rg = std::max(1u, std::min((nrows + 7) / 8, 152u * 16u));     // a warp per row
            const unsigned sg = std::max(1u, std::min((nrows * AB_SEG / 32 + 8) / 8, 152u * 16u));   // AB_SEG lanes per row
            const unsigned wg = std::max(1u, std::min((nbw + 255) / 256, 152u * 16u));   // a thread per word
            { k_ab_bits<<<rg, 256, 0, s>>>(db, nb, nrows, ar, Bm); N2M_COUNT(); }
            if (fill_bubbles) {
                unsigned char *edge = w.edge.as<unsigned char>();
                { k_ab_init<<<wg, 256, 0, s>>>(db, nb, nbw, Bm, 0u, L, edge, nullptr); N2M_COUNT(); }
                { k_ab_merge<3><<<sg, 256, 0, s>>>(db, nb, nrows, Bm, 0u, L); N2M_COUNT(); }
                { k_ab_flatten<<<wg, 256, 0, s>>>(db, nb, nbw, Bm, 0u, L, false); N2M_COUNT(); }
                { k_ab_edges<<<wg, 256, 0, s>>>(db, nb, nbw, Bm, L, edge); N2M_COUNT(); }
                { k_ab_fill<<<sg, 256, 0, s>>>(db, nb, nrows, Bm, L, edge); N2M_COUNT(); }
            }
            unsigned *cnt = only_largest ? w.ucnt.as<unsigned>() : nullptr;
            { k_ab_init<<<wg, 256, 0, s>>>(db, nb, nbw, Bm, 1u, L, nullptr, cnt); N2M_COUNT(); }
            { k_ab_merge<9><<<sg, 256, 0, s>>>(db, nb, nrows, Bm, 1u, L); N2M_COUNT(); }
            { k_ab_flatten<<<wg, 256, 0, s>>>(db, nb, nbw, Bm, 1u, L, true); N2M_COUNT(); }
            const unsigned *K = Bm;
            if (only_largest) {
                unsigned *Kb = w.keep.as<unsigned>();
                { k_ab_sizes<<<sg, 256, 0, s>>>(db, nb, nrows, Bm, L, cnt); N2M_COUNT(); }
                { k_ab_best<<<wg, 256, 0, s>>>(db, nb, nbw, Bm, L, cnt); N2M_COUNT(); }
                { k_ab_keep<<<sg, 256, 0, s>>>(db, nb, nrows, Bm, L, Kb); N2M_COUNT(); }
                K = Kb;
            }
            if (only_largest && fill_bubbles) { k_ab_final<true, true><<<rg, 256, 0, s>>>(db, nb, nrows, K, ar, nx, ny, nz); N2M_COUNT(); }
            else if (only_largest) { k_ab_final<true, false><<<rg, 256, 0, s>>>(db, nb, nrows, K, ar, nx, ny, nz); N2M_COUNT(); }
            else { k_ab_final<false, true><<<rg, 256, 0, s>>>(db, nb, nrows, K, ar, nx, ny, nz); N2M_COUNT(); }
        }
        { k_a_stats<<<g, 256, 0, s>>>(db, nb, chunks, q + qi++, ch, ar); N2M_COUNT(); }
        { k_a_pad<<<(nb + 127) / 128, 128, 0, s>>>(db, nb); N2M_COUNT(); }
        CKL();
        return N2M_OK;
    }
};
}  // namespace

n2m_status atlas_hist(const short *d_lab, const int dim[3], AtlasWork &w, cudaStream_t s, int *maxlab,
                      std::vector<unsigned> &cnt, std::vector<int> &bb) {
    const int ML = 32767;
    CKS(w.cnt.ensure((ML + 1) * sizeof(unsigned)));
    CKS(w.bb.ensure((size_t)(ML + 1) * 6 * sizeof(int) + 16));
    CK(cudaMemsetAsync(w.cnt.p, 0, (ML + 1) * sizeof(unsigned), s));
    int *dvmax = (int *)(w.bb.as<int>() + (ML + 1) * 6);
    CK(cudaMemsetAsync(dvmax, 0, sizeof(int), s));
    { k_a_fill_bb<<<256, 256, 0, s>>>(w.bb.as<int>(), (ML + 1) * 6); N2M_COUNT(); }
    AtlasVol v{d_lab, dim[0], dim[1], dim[2], (long long)dim[0] * dim[1], (long long)dim[0] * dim[1] * dim[2]};
    { k_a_hist<<<pgrid((unsigned)std::min<long long>((v.nvox + 255) / 256, 1u << 30), 32), 256, 0, s>>>(v, ML, w.cnt.as<unsigned>(), w.bb.as<int>(), dvmax); N2M_COUNT(); }
    CKL();
    int mx = 0;
    CK(cudaMemcpyAsync(&mx, dvmax, sizeof(int), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    *maxlab = mx;
    cnt.assign(mx + 1, 0u);
    bb.assign((size_t)(mx + 1) * 6, 0);
    if (mx >= 1) {
        CK(cudaMemcpyAsync(cnt.data(), w.cnt.p, (mx + 1) * sizeof(unsigned), cudaMemcpyDeviceToHost, s));
        CK(cudaMemcpyAsync(bb.data(), w.bb.p, (size_t)(mx + 1) * 6 * sizeof(int), cudaMemcpyDeviceToHost, s));
        CK(cudaStreamSynchronize(s));
    }
    return N2M_OK;
}

n2m_status atlas_binarize(const short *d_lab, long long n, int label, float *out, cudaStream_t s) {
    { k_binarize<<<pgrid((unsigned)std::min<long long>((n + 255) / 256, 1u << 30), 32), 256, 0, s>>>(d_lab, n, label, out); N2M_COUNT(); }
    CKL();
    return N2M_OK;
}

n2m_status atlas_offset_tris(vec3i *t, int n, int off, cudaStream_t s) {
    if (n > 0 && off) { k_offset_tris<<<pgrid((n + 255) / 256, 16), 256, 0, s>>>(t, n, off); N2M_COUNT(); }
    CKL();
    return N2M_OK;
}

n2m_status atlas_batched(const short *d_lab, const int dim[3], const n2m_options &o, AtlasWork &w, ScanWork &sw,
                         DegWork &dw, HcWork &hw, cudaStream_t s, std::vector<n2m_atlas_mesh> &out, vec3d **d_pts,
                         vec3i **d_tris, int64_t *npts, int64_t *ntris, float *ms_stage) {
    cudaEvent_t ev[6];
    for (auto &e : ev) CK(cudaEventCreate(&e));
    struct EvGuard {
        cudaEvent_t *e;
        ~EvGuard() { for (int i = 0; i < 6; i++) cudaEventDestroy(e[i]); }
    } guard{ev};
    CK(cudaEventRecord(ev[0], s));
    int maxlab = 0;
    std::vector<unsigned> cnt;
    std::vector<int> bb;
    CKS(atlas_hist(d_lab, dim, w, s, &maxlab, cnt, bb));
    if (maxlab < 1) {
        n2m_set_error("intensity range not consistent with an indexed atlas");
        return N2M_ERR_BAD_ARGS;
    }
    AtlasVol v{d_lab, dim[0], dim[1], dim[2], (long long)dim[0] * dim[1], (long long)dim[0] * dim[1] * dim[2]};
    // ---- sub-boxes
    std::vector<ABox> boxes;
    long long arena = 0;
    unsigned tiles = 0;
    unsigned long long rows = 0, bwords = 0;
    for (int l = 1; l <= maxlab; l++) {
        if (!cnt[l]) continue;
        ABox B;
        memset(&B, 0, sizeof(B));
        B.label = l;
        bool full = true;
        for (int a = 0; a < 3; a++) {
            const int lo = std::max(bb[6 * l + a] - 3, 0), hi = std::min(bb[6 * l + 3 + a] + 3, dim[a] - 1);
            B.o[a] = lo;
            B.n[a] = hi - lo + 1;
            full = full && lo == 0 && B.n[a] == dim[a];
        }
        B.full = full;
        B.arena = arena;
        arena += (long long)B.n[0] * B.n[1] * B.n[2];
        B.tile0 = tiles;
        tiles += (unsigned)(((B.n[0] + smooth::STX - 1) / smooth::STX) * ((B.n[1] + smooth::STY - 1) / smooth::STY) *
                            ((B.n[2] + smooth::SZC - 1) / smooth::SZC));
        B.chunk0 = 0;   // set per chunk size below
        B.W = (unsigned)(B.n[0] + 31) / 32;
        B.row0 = rows;
        B.bw0 = bwords;
        rows += (unsigned long long)B.n[1] * B.n[2];
        bwords += (unsigned long long)B.W * B.n[1] * B.n[2];
        B.vmin = INT_MAX;
        B.vmax = INT_MIN;
        for (int a = 0; a < 3; a++) { B.blo[a] = INT_MAX; B.bhi[a] = INT_MIN; }
        boxes.push_back(B);
    }
    const int nb = (int)boxes.size();
    if (arena >= 0x7fffffffLL) {
        n2m_set_error("atlas arena exceeds 2^31 voxels");
        return N2M_ERR_TOO_LARGE;
    }
    CKS(w.boxes.ensure((size_t)nb * sizeof(ABox)));
    CKS(w.queue.ensure(96 * sizeof(unsigned)));
    CKS(w.arena.ensure((size_t)arena * sizeof(float)));
    ABox *db = w.boxes.as<ABox>();
    unsigned *q = w.queue.as<unsigned>();
    CK(cudaMemcpyAsync(db, boxes.data(), nb * sizeof(ABox), cudaMemcpyHostToDevice, s));
    CK(cudaMemsetAsync(q, 0, 96 * sizeof(unsigned), s));
    float *ar = w.arena.as<float>();
    const bool smooth_on = o.pre_smooth && dim[0] >= 5 && dim[1] >= 5 && dim[2] >= 5;
    Segment seg{v, db, nb, tiles, ar, smooth_on, o.only_largest, o.fill_bubbles, dim[0], dim[1], dim[2], q, arena,
                (unsigned)rows, (unsigned)bwords};
    CKS(seg.ensure(w));
    // pick chunk size and persistent-grid width once per context (autotuner)
    if (!w.tuned) {
        float best = 1e30f;
        const unsigned cands[][2] = {{512, 4}, {1024, 8}, {1024, 16}, {2048, 8}, {4096, 8}, {4096, 16}};
        for (const auto &cd : cands) {
            std::vector<ABox> bx(boxes);
            const unsigned nch = set_chunks(bx, cd[0]);
            CK(cudaMemcpyAsync(db, bx.data(), nb * sizeof(ABox), cudaMemcpyHostToDevice, s));
            CK(cudaEventRecord(ev[1], s));
            CKS(seg.enqueue(w, cd[0], cd[1], nch, s));
            CK(cudaEventRecord(ev[2], s));
            CK(cudaEventSynchronize(ev[2]));
            float ms = 0.f;
            cudaEventElapsedTime(&ms, ev[1], ev[2]);
            if (ms < best) { best = ms; w.chunk = cd[0]; w.per_sm = cd[1]; }
        }
        w.tuned = true;
        w.tuned_ms = best;
    }
    const unsigned chunks = set_chunks(boxes, w.chunk);
    CK(cudaMemcpyAsync(db, boxes.data(), nb * sizeof(ABox), cudaMemcpyHostToDevice, s));
    CK(cudaEventRecord(ev[1], s));
    // the smoothing + clustering + range/bbox segment runs as one CUDA graph
    cudaGraph_t graph = nullptr;
    CK(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    const n2m_status cst = seg.enqueue(w, w.chunk, w.per_sm, chunks, s);
    const cudaError_t ce = cudaStreamEndCapture(s, &graph);
    if (cst != N2M_OK || ce != cudaSuccess) {
        if (graph) cudaGraphDestroy(graph);
        CKS(cst);
        CK(ce);
    }
    cudaGraphExec_t exec = (cudaGraphExec_t)w.exec;
    bool updated = false;
    if (exec) {
        cudaGraphExecUpdateResultInfo info;
        updated = cudaGraphExecUpdate(exec, graph, &info) == cudaSuccess;
        if (!updated) {
            cudaGetLastError();
            cudaGraphExecDestroy(exec);
            exec = nullptr;
        }
    }
    if (!exec) {
        const cudaError_t ie = cudaGraphInstantiate(&exec, graph, 0);
        if (ie != cudaSuccess) {
            cudaGraphDestroy(graph);
            CK(ie);
        }
    }
    w.exec = exec;
    cudaGraphDestroy(graph);
    CK(cudaGraphLaunch(exec, s));
    CK(cudaEventRecord(ev[2], s));
    int qi = 32;
    CK(cudaMemcpyAsync(boxes.data(), db, nb * sizeof(ABox), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    CK(cudaEventRecord(ev[3], s));
    // ---- marching-cubes grids
    unsigned words = 0, ctiles = 0;
    for (auto &B : boxes) {
        if (!B.fail && B.blo[0] > B.bhi[0]) B.fail = N2M_ERR_EMPTY;
        B.word0 = words;
        B.ctile0 = ctiles;
        if (B.fail) {
            B.WX = 0;
            for (int a = 0; a < 3; a++) B.gn[a] = 0;
            continue;
        }
        for (int a = 0; a < 3; a++) {
            const int lo = std::max(B.blo[a] - 1, 0), hi = std::min(B.bhi[a] + 2, dim[a]);
            B.glo[a] = lo;
            B.gn[a] = hi - lo + 1;
        }
        B.WX = (unsigned)((B.gn[0] + 31) / 32);
        words += B.WX * (unsigned)B.gn[1] * (unsigned)B.gn[2];
        ctiles += B.WX * (unsigned)((B.gn[1] + TY - 1) / TY) * (unsigned)((B.gn[2] + TZ - 1) / TZ);
    }
    CK(cudaMemcpyAsync(db, boxes.data(), nb * sizeof(ABox), cudaMemcpyHostToDevice, s));
    CKS(w.words.ensure(((size_t)words + 1) * sizeof(uint4)));
    CKS(w.counts.ensure(((size_t)words + 1) * sizeof(uint4)));
    CKS(w.active.ensure(((size_t)words + 2) * sizeof(unsigned)));
    CKS(w.tot.ensure(sizeof(uint4) + (size_t)(nb + 1) * sizeof(BoxOff)));
    unsigned *act = w.active.as<unsigned>();
    CK(cudaMemsetAsync(act + words, 0, sizeof(unsigned), s));
    const bool classic = o.cubes == N2M_CUBES_CLASSIC_TABLE;
    if (ctiles) { k_a_count<<<pgrid(ctiles, 4), 256, 0, s>>>(v, db, nb, ctiles, q + qi++, ar, classic, w.words.as<uint4>(), w.counts.as<uint4>(), act, act + words); N2M_COUNT(); }
    CKL();
    uint4 *dtot = w.tot.as<uint4>();
    BoxOff *dboff = (BoxOff *)(dtot + 1);
    CKS(scan_uint4(w.counts.as<uint4>(), words, dtot, sw, s));
    uint4 tot;
    CK(cudaMemcpyAsync(&tot, dtot, sizeof(uint4), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    { k_a_boxoff<<<(nb + 128) / 128, 128, 0, s>>>(db, nb, w.counts.as<uint4>(), tot, dboff); N2M_COUNT(); }
    std::vector<BoxOff> boff(nb + 1);
    CK(cudaMemcpyAsync(boff.data(), dboff, (nb + 1) * sizeof(BoxOff), cudaMemcpyDeviceToHost, s));
    const unsigned nv = tot.x + tot.z, nt = tot.y, nact = *(&tot.w);
    CKS(w.pts.ensure((size_t)std::max(nv, 1u) * sizeof(vec3d)));
    CKS(w.tris.ensure((size_t)std::max(nt, 1u) * sizeof(vec3i)));
    const int cap = (int)std::min<unsigned>(nv / 16 + 65536, 1u << 26);
    CKS(w.cand.ensure((size_t)2 * cap * sizeof(int) + 2 * sizeof(unsigned)));
    int *cand = w.cand.as<int>();
    unsigned *ncand = (unsigned *)(cand + 2 * cap);
    CK(cudaMemsetAsync(ncand, 0, 2 * sizeof(unsigned), s));
    if (nact) { k_a_emit<<<pgrid((nact + 7) / 8, 16), 256, 0, s>>>(v, db, dboff, nb, w.words.as<uint4>(), w.counts.as<uint4>(), act, nact, ar, classic, w.pts.as<vec3d>(), w.tris.as<vec3i>(), cand, ncand, cand + cap, ncand + 1, cap); N2M_COUNT(); }
    CKL();
    unsigned nc[2];
    CK(cudaMemcpyAsync(nc, ncand, 2 * sizeof(unsigned), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    CK(cudaEventRecord(ev[4], s));
    if (nc[0] > (unsigned)cap || nc[1] > (unsigned)cap) {
        n2m_set_error("weld candidate overflow");
        return N2M_ERR_INTERNAL;
    }
    if (nc[1]) {
        CK(cudaMemcpyAsync(cand + nc[0], cand + cap, nc[1] * sizeof(int), cudaMemcpyDeviceToDevice, s));
        unsigned t2 = nc[0] + nc[1];
        CK(cudaMemcpyAsync(ncand, &t2, sizeof(unsigned), cudaMemcpyHostToDevice, s));
        CKS(mc_ccand_scan(w.pts.as<vec3d>(), (int)nv, cand + cap, (int)nc[1], cand, ncand, cap, s));
        CK(cudaMemcpyAsync(nc, ncand, sizeof(unsigned), cudaMemcpyDeviceToHost, s));
        CK(cudaStreamSynchronize(s));
    }
    // per box vertex ranges [vs, ve)
    std::vector<unsigned> vs(nb + 1), ts(nb + 1);
    for (int b = 0; b <= nb; b++) { vs[b] = boff[b].e + boff[b].c; ts[b] = boff[b].t; }
    // ---- weld (per box: the reference welds each label's mesh on its own)
    std::vector<int> removed, keepv, ov_id;
    std::vector<vec3d> ov_pos;
    if (nc[0]) {
        std::vector<int> ids(nc[0]);
        CK(cudaMemcpyAsync(ids.data(), cand, nc[0] * sizeof(int), cudaMemcpyDeviceToHost, s));
        CK(cudaStreamSynchronize(s));
        std::sort(ids.begin(), ids.end());
        ids.erase(std::unique(ids.begin(), ids.end()), ids.end());
        const int n = (int)ids.size();
        std::vector<int> firsts;
        for (int b = 0; b < nb; b++) if (vs[b + 1] > vs[b]) firsts.push_back((int)vs[b]);
        std::vector<int> all(ids);
        all.insert(all.end(), firsts.begin(), firsts.end());
        CKS(w.gath.ensure(all.size() * (sizeof(int) + sizeof(vec3d)) + 16));
        vec3d *dpos = w.gath.as<vec3d>();
        int *dids = (int *)(dpos + all.size());
        CK(cudaMemcpyAsync(dids, all.data(), all.size() * sizeof(int), cudaMemcpyHostToDevice, s));
        { k_a_gather<<<((int)all.size() + 255) / 256, 256, 0, s>>>(w.pts.as<vec3d>(), dids, (int)all.size(), dpos); N2M_COUNT(); }
        std::vector<vec3d> pos(all.size());
        CK(cudaMemcpyAsync(pos.data(), dpos, all.size() * sizeof(vec3d), cudaMemcpyDeviceToHost, s));
        CK(cudaStreamSynchronize(s));
        int i0 = 0;
        for (int b = 0; b < nb && i0 < n; b++) {
            int i1 = i0;
            while (i1 < n && (unsigned)ids[i1] < vs[b + 1]) i1++;
            if (i1 == i0) continue;
            const int fi = (int)(std::lower_bound(firsts.begin(), firsts.end(), (int)vs[b]) - firsts.begin());
            const vec3d v0 = pos[n + fi];
            const int m = i1 - i0;
            std::vector<float> key(m);
            std::vector<int> srt(m), grp(m, -1);
            for (int k = 0; k < m; k++) { key[k] = (float)d3(v0, pos[i0 + k]); srt[k] = k; }
            std::sort(srt.begin(), srt.end(), [&](int a, int c) {
                return kbits(key[a]) != kbits(key[c]) ? kbits(key[a]) < kbits(key[c]) : ids[i0 + a] < ids[i0 + c];
            });
            int ng = 0;
            for (int k = 0; k < m; k++) {
                const int a = srt[k];
                if (grp[a] >= 0) continue;
                for (int j = k; j < m && (key[srt[j]] - key[a]) < 0.00001f; j++)
                    if (d3(pos[i0 + a], pos[i0 + srt[j]]) < 0.00001f) grp[srt[j]] = ng;
                ng++;
            }
            std::vector<int> gk(ng, INT32_MAX), gl(ng, -1), gs(ng, 0);
            for (int k = 0; k < m; k++) {
                const int g = grp[k];
                gs[g]++;
                gk[g] = std::min(gk[g], ids[i0 + k]);
                if (gl[g] < 0 || ids[i0 + k] > ids[i0 + gl[g]]) gl[g] = k;
            }
            for (int k = 0; k < m; k++) {
                const int g = grp[k];
                if (gs[g] < 2) continue;
                if (ids[i0 + k] != gk[g]) { removed.push_back(ids[i0 + k]); keepv.push_back(gk[g]); }
                else if (gl[g] != k) { ov_id.push_back(ids[i0 + k]); ov_pos.push_back(pos[i0 + gl[g]]); }
            }
            i0 = i1;
        }
    }
    vec3d *pts = w.pts.as<vec3d>();
    unsigned np = nv;
    std::vector<unsigned> vs_new(vs);
    if (!removed.empty()) {
        // ids are grouped by box and ascending within each box, so `removed`
        // is sorted; `ov_id` likewise
        const int nr = (int)removed.size(), no = (int)ov_id.size();
        CKS(w.weld.ensure((size_t)(2 * nr + no + 1) * sizeof(int) + (size_t)(no + 1) * sizeof(vec3d)));
        vec3d *dov = w.weld.as<vec3d>();
        int *drem = (int *)(dov + no + 1), *dkeep = drem + nr, *dovid = dkeep + nr;
        std::vector<int> ri(nr);
        for (int i = 0; i < nr; i++) ri[i] = i;
        std::sort(ri.begin(), ri.end(), [&](int a, int b2) { return removed[a] < removed[b2]; });
        std::vector<int> r2, k2;
        for (int i : ri) { r2.push_back(removed[i]); k2.push_back(keepv[i]); }
        if (no) CK(cudaMemcpyAsync(dov, ov_pos.data(), no * sizeof(vec3d), cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(drem, r2.data(), nr * sizeof(int), cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(dkeep, k2.data(), nr * sizeof(int), cudaMemcpyHostToDevice, s));
        if (no) CK(cudaMemcpyAsync(dovid, ov_id.data(), no * sizeof(int), cudaMemcpyHostToDevice, s));
        np = nv - nr;
        CKS(w.pts2.ensure((size_t)np * sizeof(vec3d)));
        CKS(mesh_apply_weld(pts, w.tris.as<vec3i>(), (int)nv, (int)nt, drem, dkeep, nr, dovid, dov, no,
                            w.pts2.as<vec3d>(), s));
        pts = w.pts2.as<vec3d>();
        for (int b = 0; b <= nb; b++)
            vs_new[b] = vs[b] - (unsigned)(std::lower_bound(r2.begin(), r2.end(), (int)vs[b]) - r2.begin());
        CK(cudaStreamSynchronize(s));
    }
    // ---- degenerate triangles, per-box triangle ranges after compaction
    CKS(w.tris2.ensure((size_t)std::max(nt, 1u) * sizeof(vec3i)));
    CKS(w.ranges.ensure((size_t)(4 * (nb + 1) + 2) * sizeof(unsigned)));
    unsigned *dts = w.ranges.as<unsigned>(), *dkept = dts + (nb + 1), *dvs = dkept + (nb + 1), *dntf = dvs + (nb + 1);
    CKS(mesh_remove_degenerate(pts, w.tris.as<vec3i>(), (int)nt, w.tris2.as<vec3i>(), dntf, dw, sw, s));
    unsigned ntf = 0;
    CK(cudaMemcpyAsync(&ntf, dntf, sizeof(unsigned), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    CK(cudaMemcpyAsync(dts, ts.data(), (nb + 1) * sizeof(unsigned), cudaMemcpyHostToDevice, s));
    if (nt) { k_a_kept<<<(nb + 128) / 128, 128, 0, s>>>(dts, nb, dw.flags.as<unsigned>(), dw.tmp.as<unsigned>(), 256, ntf, dkept); N2M_COUNT(); }
    else CK(cudaMemsetAsync(dkept, 0, (nb + 1) * sizeof(unsigned), s));
    std::vector<unsigned> kept(nb + 1);
    CK(cudaMemcpyAsync(kept.data(), dkept, (nb + 1) * sizeof(unsigned), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    vec3i *tris = w.tris2.as<vec3i>();
    // ---- HC post-smoothing of all meshes at once (they share no vertex)
    CK(cudaEventRecord(ev[5], s));
    if (o.post_smooth > 0 && np > 0)
        CKS(mesh_smooth_hc(pts, tris, (int)np, (int)ntf, 0.1, 0.5, o.post_smooth, true, hw, sw, s));
    // ---- triangle indices local to their mesh
    CK(cudaMemcpyAsync(dkept, kept.data(), (nb + 1) * sizeof(unsigned), cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(dvs, vs_new.data(), (nb + 1) * sizeof(unsigned), cudaMemcpyHostToDevice, s));
    if (ntf) { k_a_localize<<<pgrid((ntf + 255) / 256, 16), 256, 0, s>>>(tris, ntf, dkept, dvs, nb); N2M_COUNT(); }
    CKL();
    CK(cudaStreamSynchronize(s));
    out.clear();
    for (int b = 0; b < nb; b++) {
        n2m_atlas_mesh d;
        d.label = boxes[b].label;
        d.status = boxes[b].fail;
        d.nvert = (int)(vs_new[b + 1] - vs_new[b]);
        d.ntri = (int)(kept[b + 1] - kept[b]);
        d.vert_offset = vs_new[b];
        d.tri_offset = kept[b];
        if (!d.status && (d.nvert < 3 || d.ntri < 1)) d.status = N2M_ERR_EMPTY;
        out.push_back(d);
    }
    *d_pts = pts;
    *d_tris = tris;
    *npts = np;
    *ntris = ntf;
    if (ms_stage) {
        for (int i = 0; i < 5; i++) cudaEventElapsedTime(&ms_stage[i], ev[i], ev[i + 1]);
    }
    return N2M_OK;
}
