// label.cu — connected-component labelling for meshify's largest-cluster and
// bubble-fill options (src/bwlabel.c:429-543, src/meshify.c:323-342) and the
// drop-in bwlabel().
//
// Runs, not voxels.  The class masks are bit words (bit x & 31 of word
// row*W + x/32, W = ceil(nx/32) words per row), and union-find links exist
// only at the first voxel of every run along x: a run is one set of voxels
// for any connectivity, so a component is a set of runs.  Two runs in
// neighbouring rows are united once per overlap (the contact whose left
// neighbours do not also touch), hooking the larger root under the smaller,
// so the root of a component is its first voxel in raster order: that is how
// the reference numbers labels (first appearance) and breaks size ties (lowest
// label wins).  Flattening, face contacts, bubble filling, component sizes and
// the kept component all work per run; only the final pass over the volume
// (fill to iso, dilation, mask-out and the range/bbox of the result) touches
// every voxel.
//
// Row kernels give each row `seg` lanes (a power of two, one word per lane,
// rows of more than 32 words in chunks of 32): the start of the run holding a
// word's first voxel comes from a max-scan of the last run start of the words
// before it.
#include <algorithm>

#include "n2m_internal.cuh"
#include "runs.cuh"
#include "smooth_core.cuh"
#include "uf.cuh"

namespace {
using namespace uf;
using namespace runs;

struct LD {
    int nx, ny, nz;
    long long nxy, n;
    unsigned W;       // words per row
    unsigned nrows;   // ny * nz
    unsigned nwords;  // W * nrows
    int seg;          // lanes per row in the row kernels
};

__device__ __forceinline__ unsigned valid_bits(const LD &d, unsigned w) {
    const int x0 = (int)w * 32;
    return x0 + 32 <= d.nx ? FULL : (1u << (d.nx - x0)) - 1u;
}

// foreground bits (want 1) or background bits (want 0) of word w of row r
__device__ __forceinline__ unsigned class_word(const unsigned *B, const LD &d, unsigned r, unsigned w, unsigned want) {
    const unsigned b = B[(size_t)r * d.W + w];
    return want ? b : ~b & valid_bits(d, w);
}

// the class word after this lane's word (0 past the row); all lanes call it
__device__ __forceinline__ unsigned next_word(const unsigned *B, const LD &d, unsigned c, bool rowok, unsigned r,
                                              unsigned w, int li, int seg, unsigned want) {
    const unsigned dn = __shfl_down_sync(FULL, c, 1, seg);
    if (li < seg - 1) return w + 1 < d.W ? dn : 0u;
    return rowok && w + 1 < d.W ? class_word(B, d, r, w + 1, want) : 0u;
}

// Class bits of the volume: value >= iso (meshify's mask), or value != 0
// (bwlabel's).  A warp takes whole rows, 16 words at a time in flight.
__global__ void __launch_bounds__(256) k_lab_bits(const float *__restrict__ vol, LD d, float iso, bool nonzero,
                                                  unsigned *B) {
    constexpr int K = 16;
    const int lane = threadIdx.x & 31;
    for (unsigned r = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; r < d.nrows; r += (gridDim.x * blockDim.x) >> 5) {
        const float *rp = vol + (long long)r * d.nx;
        unsigned *out = B + (size_t)r * d.W;
        for (unsigned w0 = 0; w0 < d.W; w0 += K) {
            float v[K];
#pragma unroll
            for (int k = 0; k < K; k++) {
                const int x = (int)(w0 + k) * 32 + lane;
                v[k] = w0 + k < d.W && x < d.nx ? __ldg(rp + x) : 0.f;
            }
            unsigned mine = 0;
#pragma unroll
            for (int k = 0; k < K; k++) {
                const int x = (int)(w0 + k) * 32 + lane;
                const unsigned m = __ballot_sync(FULL, x < d.nx && (nonzero ? v[k] != 0.0f : v[k] >= iso));
                if (lane == k) mine = m;
            }
            if (lane < K && w0 + lane < d.W) out[w0 + lane] = mine;
        }
    }
}

// Class bits from a sign bitmap (bit = value >= iso; OdWork::vsign layout:
// wv = W words per row, the 8 row words of a 32 x 8 tile of a slice adjacent)
__global__ void k_lab_bits_vsign(const unsigned *__restrict__ vsign, LD d, unsigned nys, unsigned *B) {
    for (unsigned i = blockIdx.x * blockDim.x + threadIdx.x; i < d.nwords; i += gridDim.x * blockDim.x) {
        const unsigned r = i / d.W, w = i - r * d.W, z = r / (unsigned)d.ny, y = r - z * (unsigned)d.ny;
        B[i] = __ldg(vsign + od_vsign_word(w * 32u, y, z, d.W, nys)) & valid_bits(d, w);
    }
}

// every run start of the class links to itself; z8 / z32 (may be null) are
// zeroed at the run starts (the edge flags and sizes the roots will carry)
__global__ void k_run_init(const unsigned *__restrict__ B, LD d, unsigned want, int *L, unsigned char *z8,
                           unsigned *z32) {
    for (unsigned i = blockIdx.x * blockDim.x + threadIdx.x; i < d.nwords; i += gridDim.x * blockDim.x) {
        const unsigned r = i / d.W, w = i - r * d.W;
        const unsigned c = class_word(B, d, r, w, want), pc = w ? class_word(B, d, r, w - 1, want) : 0u;
        const long long base = (long long)r * d.nx + (long long)w * 32;
        for (unsigned st = c & ~((c << 1) | (pc >> 31)); st; st &= st - 1) {
            const int s = (int)(base + __ffs(st) - 1);
            L[s] = s;
            if (z8) z8[s] = 0;
            if (z32) z32[s] = 0;
        }
    }
}

// Union of the runs of the class with those of the rows before them: rows
// (y-1, z) and (y, z-1) for 6-connectivity, with x offsets -1..1 for 18 and
// rows (y-1, z-1), (y+1, z-1) for 18 (x offset 0) and 26 (-1..1).  A contact
// of voxel x with voxel x+dx of row k counts only if voxels x-1 and x+dx-1
// do not also touch: one union per overlap of two runs.
template <int NNB>
__global__ void __launch_bounds__(256, 6) k_run_merge(const unsigned *__restrict__ B, LD d, unsigned want, int *L) {
    static_assert(NNB == 3 || NNB == 9 || NNB == 13, "6-, 18- or 26-connectivity");
    constexpr int NR = NNB == 3 ? 3 : 5;
    const int RY[5] = {0, -1, 0, -1, 1}, RZ[5] = {0, 0, -1, -1, -1};
    const int lane = threadIdx.x & 31, seg = d.seg, li = lane & (seg - 1);
    const unsigned rpw = 32u / (unsigned)seg, rsub = (unsigned)lane / (unsigned)seg;
    const unsigned nw = (gridDim.x * blockDim.x) >> 5;
    for (unsigned rb = ((blockIdx.x * blockDim.x + threadIdx.x) >> 5) * rpw; rb < d.nrows; rb += nw * rpw) {
        const unsigned r = rb + rsub;
        const bool rowok = r < d.nrows;
        const int z = rowok ? (int)(r / (unsigned)d.ny) : 0, y = rowok ? (int)(r - (unsigned)z * (unsigned)d.ny) : 0;
        bool kok[NR];
        unsigned rk[NR];
#pragma unroll
        for (int k = 0; k < NR; k++) {
            const int yy = y + RY[k], zz = z + RZ[k];
            kok[k] = rowok && yy >= 0 && zz >= 0 && yy < d.ny && zz < d.nz;
            rk[k] = kok[k] ? (unsigned)zz * (unsigned)d.ny + (unsigned)yy : 0u;
        }
        int cst[NR];
        unsigned cwd[NR];
#pragma unroll
        for (int k = 0; k < NR; k++) { cst[k] = -1; cwd[k] = 0u; }
        for (unsigned c0 = 0; c0 < d.W; c0 += (unsigned)seg) {
            const unsigned w = c0 + (unsigned)li;
            const bool ok = w < d.W;
            const int x0 = (int)w * 32;
            WordRuns R[NR];
            unsigned nk[NR];
#pragma unroll
            for (int k = 0; k < NR; k++) {
                const unsigned c = ok && kok[k] ? class_word(B, d, rk[k], w, want) : 0u;
                R[k] = word_runs(c, x0, li, seg, cst[k], cwd[k]);
                nk[k] = next_word(B, d, c, kok[k], rk[k], w, li, seg, want);
            }
            const unsigned F = R[0].c;
            if (!F) continue;
            const unsigned left = (F << 1) | (R[0].pc >> 31);
            auto S = [&](int k, int dx) -> unsigned {
                const WordRuns &q = R[k];
                return dx == 0 ? q.c : dx == 1 ? (q.c >> 1) | (nk[k] << 31)
                                     : dx == -1 ? (q.c << 1) | (q.pc >> 31) : (q.c << 2) | (q.pc >> 30);
            };
            const long long base0 = (long long)r * d.nx;
            auto link = [&](int k, int dx) {
                unsigned m = F & S(k, dx) & ~(left & S(k, dx - 1));
                if (!m) return;
                const WordRuns &q = R[k];
                const long long basek = (long long)rk[k] * d.nx;
                for (; m; m &= m - 1) {
                    const int b = __ffs(m) - 1, xx = b + dx;
                    const int sk = xx < 0 ? q.cs : xx > 31 ? ((q.c >> 31) & 1u ? q.start_of(31) : x0 + 32) : q.start_of(xx);
                    const int i = (int)(base0 + R[0].start_of(b)), j = (int)(basek + sk);
                    if (L[i] != L[j]) unite(L, i, j);
                }
            };
            link(1, 0);
            link(2, 0);
            if constexpr (NNB >= 9) {
                link(1, -1); link(1, 1); link(2, -1); link(2, 1); link(3, 0); link(4, 0);
            }
            if constexpr (NNB == 13) {
                link(3, -1); link(3, 1); link(4, -1); link(4, 1);
            }
        }
    }
}

// every run start of the class points at its root; roots are counted.  The
// root search only reads: the one store of this kernel is a start's final
// root (a path-halving store could overwrite a root another thread has just
// stored with a lower ancestor).
__global__ void k_run_flatten(const unsigned *__restrict__ B, LD d, unsigned want, int *L, unsigned *nroots) {
    unsigned cnt = 0;
    for (unsigned i = blockIdx.x * blockDim.x + threadIdx.x; i < d.nwords; i += gridDim.x * blockDim.x) {
        const unsigned r = i / d.W, w = i - r * d.W;
        const unsigned c = class_word(B, d, r, w, want), pc = w ? class_word(B, d, r, w - 1, want) : 0u;
        const long long base = (long long)r * d.nx + (long long)w * 32;
        for (unsigned st = c & ~((c << 1) | (pc >> 31)); st; st &= st - 1) {
            const int s = (int)(base + __ffs(st) - 1);
            const int root = find_root(L, s);
            if (root == s) cnt++;
            else L[s] = root;
        }
    }
    for (int o = 16; o; o >>= 1) cnt += __shfl_xor_sync(FULL, cnt, o);
    if ((threadIdx.x & 31) == 0 && cnt) atomicAdd(nroots, cnt);
}

// Background components touching a face of the volume flag their root:
// items [0, nrows) take the runs holding x = 0 and x = nx-1 of a row, the items
// after them one word each of the rows on a y or z face (every run in it).  A
// flag is stored only if it is not set yet (most items name the same root).
__global__ void k_run_edges(const unsigned *__restrict__ B, LD d, const int *__restrict__ L, unsigned char *edge) {
    const unsigned nzf = d.nz > 1 ? 2u : 1u, nyf = d.ny > 1 ? 2u : 1u;
    const unsigned zrows = nzf * (unsigned)d.ny, yrows = d.nz > 2 ? nyf * (unsigned)(d.nz - 2) : 0u;
    const unsigned total = d.nrows + (zrows + yrows) * d.W;
    auto mark = [&](long long j) {
        const int root = L[j];
        if (!edge[root]) edge[root] = 1;
    };
    for (unsigned t = blockIdx.x * blockDim.x + threadIdx.x; t < total; t += gridDim.x * blockDim.x) {
        if (t < d.nrows) {
            const unsigned r = t;
            const long long base = (long long)r * d.nx;
            if (class_word(B, d, r, 0, 0u) & 1u) mark(base);
            unsigned w = d.W - 1;
            int b = (d.nx - 1) & 31;
            unsigned c = class_word(B, d, r, w, 0u);
            if (!((c >> b) & 1u)) continue;
            for (;;) {   // back to the run's start (x = 0 of a background run is one)
                const unsigned pc = w ? class_word(B, d, r, w - 1, 0u) : 0u;
                const int ls = last_start(c & ~((c << 1) | (pc >> 31)), (int)w * 32, b);
                if (ls >= 0) {
                    mark(base + ls);
                    break;
                }
                w--;
                b = 31;
                c = pc;
            }
            continue;
        }
        const unsigned u = t - d.nrows, fr = u / d.W, w = u - fr * d.W;
        unsigned r;
        if (fr < zrows) {   // slices z = 0 and z = nz-1
            const unsigned side = fr / (unsigned)d.ny, y = fr - side * (unsigned)d.ny;
            r = (side ? (unsigned)(d.nz - 1) * (unsigned)d.ny : 0u) + y;
        } else {            // rows y = 0 and y = ny-1 of the slices between
            const unsigned v = fr - zrows, side = v / (unsigned)(d.nz - 2), z = 1 + v - side * (unsigned)(d.nz - 2);
            r = z * (unsigned)d.ny + (side ? (unsigned)(d.ny - 1) : 0u);
        }
        const unsigned c = class_word(B, d, r, w, 0u), pc = w ? class_word(B, d, r, w - 1, 0u) : 0u;
        const long long base = (long long)r * d.nx + (long long)w * 32;
        for (unsigned st = c & ~((c << 1) | (pc >> 31)); st; st &= st - 1) mark(base + __ffs(st) - 1);
    }
}

// bubbles (background components away from every face) become foreground,
// only when the background has at least two components (src/bwlabel.c:488-491)
__global__ void __launch_bounds__(256) k_run_fill(unsigned *B, LD d, const int *__restrict__ L,
                                                  const unsigned char *__restrict__ edge, const unsigned *__restrict__ nbg) {
    if (*nbg <= 1) return;
    const int lane = threadIdx.x & 31, seg = d.seg, li = lane & (seg - 1);
    const unsigned rpw = 32u / (unsigned)seg, rsub = (unsigned)lane / (unsigned)seg;
    const unsigned nw = (gridDim.x * blockDim.x) >> 5;
    for (unsigned rb = ((blockIdx.x * blockDim.x + threadIdx.x) >> 5) * rpw; rb < d.nrows; rb += nw * rpw) {
        const unsigned r = rb + rsub;
        const bool rowok = r < d.nrows;
        const long long base = (long long)r * d.nx;
        int cst = -1;
        unsigned cwd = 0;
        for (unsigned c0 = 0; c0 < d.W; c0 += (unsigned)seg) {
            const unsigned w = c0 + (unsigned)li;
            const unsigned c = rowok && w < d.W ? class_word(B, d, r, w, 0u) : 0u;
            const WordRuns R = word_runs(c, (int)w * 32, li, seg, cst, cwd);
            unsigned fill = 0;
            for (unsigned rem = c; rem;) {   // the word's pieces of runs
                const int b = __ffs(rem) - 1;
                const unsigned pm = piece_at(rem, b);
                rem &= ~pm;
                if (!edge[L[base + R.start_of(b)]]) fill |= pm;
            }
            // every lane has read its neighbours' words (word_runs) before any write
            if (fill) B[(size_t)r * d.W + w] |= fill;
        }
    }
}

// component sizes: every run adds its length to its root (at the run's end)
__global__ void __launch_bounds__(256) k_run_sizes(const unsigned *__restrict__ B, LD d, const int *__restrict__ L,
                                                   unsigned *cnt) {
    const int lane = threadIdx.x & 31, seg = d.seg, li = lane & (seg - 1);
    const unsigned rpw = 32u / (unsigned)seg, rsub = (unsigned)lane / (unsigned)seg;
    const unsigned nw = (gridDim.x * blockDim.x) >> 5;
    for (unsigned rb = ((blockIdx.x * blockDim.x + threadIdx.x) >> 5) * rpw; rb < d.nrows; rb += nw * rpw) {
        const unsigned r = rb + rsub;
        const bool rowok = r < d.nrows;
        const long long base = (long long)r * d.nx;
        int cst = -1;
        unsigned cwd = 0;
        for (unsigned c0 = 0; c0 < d.W; c0 += (unsigned)seg) {
            const unsigned w = c0 + (unsigned)li;
            const unsigned c = rowok && w < d.W ? class_word(B, d, r, w, 1u) : 0u;
            const WordRuns R = word_runs(c, (int)w * 32, li, seg, cst, cwd);
            const unsigned nxt = next_word(B, d, c, rowok, r, w, li, seg, 1u);
            for (unsigned ends = c & ~((c >> 1) | (nxt << 31)); ends; ends &= ends - 1) {
                const int e = __ffs(ends) - 1, s = R.start_of(e);
                atomicAdd(&cnt[L[base + s]], (unsigned)(R.x0 + e - s + 1));
            }
        }
    }
}

// largest component; ties go to the smallest root (first in raster order)
__global__ void k_run_best(const unsigned *__restrict__ B, LD d, const int *__restrict__ L,
                           const unsigned *__restrict__ cnt, unsigned long long *best) {
    unsigned long long b = 0;
    for (unsigned i = blockIdx.x * blockDim.x + threadIdx.x; i < d.nwords; i += gridDim.x * blockDim.x) {
        const unsigned r = i / d.W, w = i - r * d.W;
        const unsigned c = class_word(B, d, r, w, 1u), pc = w ? class_word(B, d, r, w - 1, 1u) : 0u;
        const long long base = (long long)r * d.nx + (long long)w * 32;
        for (unsigned st = c & ~((c << 1) | (pc >> 31)); st; st &= st - 1) {
            const int s = (int)(base + __ffs(st) - 1);
            if (L[s] != s) continue;
            const unsigned long long k = ((unsigned long long)cnt[s] << 32) | (0xffffffffu - (unsigned)s);
            b = k > b ? k : b;
        }
    }
    for (int o = 16; o; o >>= 1) {
        const unsigned long long t = __shfl_xor_sync(FULL, b, o);
        b = t > b ? t : b;
    }
    if ((threadIdx.x & 31) == 0 && b) atomicMax(best, b);
}

// bits of the voxels of the largest component
__global__ void __launch_bounds__(256) k_run_keep(const unsigned *__restrict__ B, LD d, const int *__restrict__ L,
                                                  const unsigned long long *__restrict__ best, unsigned *K) {
    const unsigned long long bk = *best;
    const int root = bk ? (int)(0xffffffffu - (unsigned)(bk & 0xffffffffu)) : -2;
    const int lane = threadIdx.x & 31, seg = d.seg, li = lane & (seg - 1);
    const unsigned rpw = 32u / (unsigned)seg, rsub = (unsigned)lane / (unsigned)seg;
    const unsigned nw = (gridDim.x * blockDim.x) >> 5;
    for (unsigned rb = ((blockIdx.x * blockDim.x + threadIdx.x) >> 5) * rpw; rb < d.nrows; rb += nw * rpw) {
        const unsigned r = rb + rsub;
        const bool rowok = r < d.nrows;
        const long long base = (long long)r * d.nx;
        int cst = -1;
        unsigned cwd = 0;
        for (unsigned c0 = 0; c0 < d.W; c0 += (unsigned)seg) {
            const unsigned w = c0 + (unsigned)li;
            const unsigned c = rowok && w < d.W ? class_word(B, d, r, w, 1u) : 0u;
            const WordRuns R = word_runs(c, (int)w * 32, li, seg, cst, cwd);
            unsigned keep = 0;
            for (unsigned rem = c; rem;) {
                const int b = __ffs(rem) - 1;
                const unsigned pm = piece_at(rem, b);
                rem &= ~pm;
                if (L[base + R.start_of(b)] == root) keep |= pm;
            }
            if (rowok && w < d.W) K[(size_t)r * d.W + w] = keep;
        }
    }
}

__global__ void k_nl_from(const unsigned *nroots, bool only_largest, int *nl) {
    *nl = only_largest ? (*nroots > 0 ? 1 : 0) : (int)*nroots;
}

// The labelled volume, one warp per row, 32 voxels a word, with the range and
// bbox of the result.  Kept voxels (K) are raised to iso when FILL; with
// LARGEST, voxels neither kept nor in the dilation of the kept set (the
// 26-neighbourhood without (-1,-1,-1), interior voxels only;
// src/meshify.c:218-264) become mn and are not read.  With R3 = K(x-1) | K(x) |
// K(x+1) and R2 = K(x) | K(x+1) of a row, the dilation is R3 of rows y-1..y+1
// in slices z and z+1, R3 of rows y and y+1 in slice z-1, and R2 of row y-1 in
// slice z-1.  The keep words of a row are loaded 32 at a time (lane l holds
// word c0 + l) and broadcast; 32 words with no kept voxel within reach are
// written without being read.
template <bool LARGEST, bool FILL, bool ONE>   // ONE: rows of at most 32 words
__global__ void __launch_bounds__(256) k_lab_final(const unsigned *__restrict__ K, LD d, float *vol, float iso, float mn,
                                                   VolStats *st, bool vec4) {
    smooth::Acc acc;
    acc.init();
    unsigned masked = 0;
    const int lane = threadIdx.x & 31;
    // rows used: 0..2 = y-1..y+1 in slice z, 3..5 in slice z+1, 6 = (y, z-1), 7 = (y+1, z-1), 8 = (y-1, z-1)
    const int DY[9] = {-1, 0, 1, -1, 0, 1, 0, 1, -1}, DZ[9] = {0, 0, 0, 1, 1, 1, -1, -1, -1};
    for (unsigned r = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; r < d.nrows; r += (gridDim.x * blockDim.x) >> 5) {
        const int z = (int)(r / (unsigned)d.ny), y = (int)(r - (unsigned)z * (unsigned)d.ny);
        float *row = vol + (long long)r * d.nx;
        if (!LARGEST) {
            const unsigned *K0 = K + (size_t)r * d.W;
            for (unsigned c0 = 0; c0 < d.W; c0 += 32) {
                const unsigned kk = c0 + lane < d.W ? K0[c0 + lane] : 0u;
                const unsigned wend = min(d.W, c0 + 32);
#pragma unroll 4
                for (unsigned w = c0; w < wend; w++) {
                    const unsigned kw = __shfl_sync(FULL, kk, (int)(w - c0));
                    const int x = (int)w * 32 + lane;
                    if (x >= d.nx) continue;
                    float v = row[x];
                    if (FILL && ((kw >> lane) & 1u)) {
                        v = fmaxf(v, iso);
                        row[x] = v;
                    }
                    acc.add(v, x, y, z, iso);
                }
            }
            continue;
        }
        const bool ryz = y > 0 && z > 0 && y < d.ny - 1 && z < d.nz - 1;
        unsigned carry[9];   // word c0 - 1 of each row
#pragma unroll
        for (int k = 0; k < 9; k++) carry[k] = 0u;
        for (unsigned c0 = 0; c0 < d.W; c0 += 32) {
            // lane l: word c0 + l of the kept set and of its dilation (the row's own word for
            // `kept`); the words next to it come from the neighbouring lanes
            unsigned on = 0u, kept = 0u;
#pragma unroll
            for (int k = 0; k < 9; k++) {
                const int yy = y + DY[k], zz = z + DZ[k];
                const bool in = yy >= 0 && zz >= 0 && yy < d.ny && zz < d.nz;
                const unsigned *Kk = K + ((size_t)(in ? zz : 0) * d.ny + (in ? yy : 0)) * d.W;
                const unsigned cur = in && c0 + lane < d.W ? Kk[c0 + lane] : 0u;
                unsigned prv = __shfl_up_sync(FULL, cur, 1), nxt = __shfl_down_sync(FULL, cur, 1);
                if (lane == 0) prv = carry[k];
                if (lane == 31) nxt = !ONE && in && c0 + 32 < d.W ? Kk[c0 + 32] : 0u;
                if (!ONE) carry[k] = __shfl_sync(FULL, cur, 31);
                on |= cur | (cur >> 1) | (nxt << 31) | (k < 8 ? (cur << 1) | (prv >> 31) : 0u);   // row 8: no K(x-1)
                if (k == 1) kept = cur;
            }
            const unsigned wend = min(d.W, c0 + 32);
            if (!__any_sync(FULL, on != 0u)) {   // nothing kept within reach: all mn
                const int xb = (int)c0 * 32, xe = min(d.nx, (int)wend * 32);
                if (vec4) {   // rows of a multiple of 4 voxels on 16-byte boundaries
                    float4 *r4 = (float4 *)(row + xb);
                    for (int q = lane; q < (xe - xb) >> 2; q += 32) {
                        r4[q] = make_float4(mn, mn, mn, mn);
                        masked += 4;
                    }
                } else {
                    for (int x = xb + lane; x < xe; x += 32) {
                        row[x] = mn;
                        masked++;
                    }
                }
                acc.mn = fminf(acc.mn, mn);
                acc.mx = fmaxf(acc.mx, mn);
                continue;
            }
            for (unsigned w = c0; w < wend; w++) {
                const unsigned onw = __shfl_sync(FULL, on, (int)(w - c0)), kw = __shfl_sync(FULL, kept, (int)(w - c0));
                const int x = (int)w * 32 + lane;
                if (x >= d.nx) continue;
                const bool kp = (kw >> lane) & 1u;
                const bool interior = ryz && x > 0 && x < d.nx - 1;
                float v;
                if (!(kp || (interior && ((onw >> lane) & 1u)))) {
                    v = mn;
                    row[x] = v;
                    masked++;
                } else {
                    v = row[x];
                    if (FILL && kp) {
                        v = fmaxf(v, iso);
                        row[x] = v;
                    }
                }
                acc.add(v, x, y, z, iso);
            }
        }
    }
    for (int o = 16; o; o >>= 1) masked += __shfl_xor_sync(FULL, masked, o);
    if (lane == 0 && masked) atomicAdd(&st->masked, masked);
    acc.flush(st, true);
}

// bwlabel() output: 0/1 of the kept set
__global__ void __launch_bounds__(256) k_write_keep(const unsigned *__restrict__ K, LD d, float *vol) {
    const int lane = threadIdx.x & 31;
    for (unsigned r = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; r < d.nrows; r += (gridDim.x * blockDim.x) >> 5) {
        float *row = vol + (long long)r * d.nx;
        for (unsigned w = 0; w < d.W; w++) {
            const unsigned kw = K[(size_t)r * d.W + w];
            const int x = (int)w * 32 + lane;
            if (x < d.nx) row[x] = (kw >> lane) & 1u ? 1.0f : 0.0f;
        }
    }
}

// bwlabel() labels: 1 + rank of the component's root among the roots in
// raster order.  Roots per word, then (after a scan) each root's rank.
__global__ void k_root_count(const unsigned *__restrict__ B, LD d, const int *__restrict__ L, unsigned *rc) {
    for (unsigned i = blockIdx.x * blockDim.x + threadIdx.x; i < d.nwords; i += gridDim.x * blockDim.x) {
        const unsigned r = i / d.W, w = i - r * d.W;
        const unsigned c = class_word(B, d, r, w, 1u), pc = w ? class_word(B, d, r, w - 1, 1u) : 0u;
        const long long base = (long long)r * d.nx + (long long)w * 32;
        unsigned n = 0;
        for (unsigned st = c & ~((c << 1) | (pc >> 31)); st; st &= st - 1) {
            const int s = (int)(base + __ffs(st) - 1);
            n += L[s] == s;
        }
        rc[i] = n;
    }
}

__global__ void k_root_rank(const unsigned *__restrict__ B, LD d, const int *__restrict__ L,
                            const unsigned *__restrict__ rc, unsigned *rank) {
    for (unsigned i = blockIdx.x * blockDim.x + threadIdx.x; i < d.nwords; i += gridDim.x * blockDim.x) {
        const unsigned r = i / d.W, w = i - r * d.W;
        const unsigned c = class_word(B, d, r, w, 1u), pc = w ? class_word(B, d, r, w - 1, 1u) : 0u;
        const long long base = (long long)r * d.nx + (long long)w * 32;
        unsigned k = rc[i];
        for (unsigned st = c & ~((c << 1) | (pc >> 31)); st; st &= st - 1) {
            const int s = (int)(base + __ffs(st) - 1);
            if (L[s] == s) rank[s] = k++;
        }
    }
}

__global__ void __launch_bounds__(256) k_write_labels(const unsigned *__restrict__ B, LD d, const int *__restrict__ L,
                                                      const unsigned *__restrict__ rank, float *vol) {
    const int lane = threadIdx.x & 31;
    for (unsigned r = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; r < d.nrows; r += (gridDim.x * blockDim.x) >> 5) {
        float *row = vol + (long long)r * d.nx;
        const long long base = (long long)r * d.nx;
        int carry = -1;   // last run start of the words before
        unsigned pc = 0;
        for (unsigned w = 0; w < d.W; w++) {
            const unsigned c = B[(size_t)r * d.W + w];
            const unsigned starts = c & ~((c << 1) | (pc >> 31));
            const int x0 = (int)w * 32, x = x0 + lane;
            if (x < d.nx) {
                float v = 0.0f;
                if ((c >> lane) & 1u) {
                    const int s0 = last_start(starts, x0, lane);
                    v = (float)(rank[L[base + (s0 >= 0 ? s0 : carry)]] + 1u);
                }
                row[x] = v;
            }
            if (starts) carry = x0 + 31 - __clz(starts);
            pc = c;
        }
    }
}

inline unsigned gsz(long long n) {
    long long b = (n + 255) / 256;
    if (b > 152 * 64) b = 152 * 64;
    return b ? (unsigned)b : 1u;
}
// row kernels: one warp per 32/seg rows
inline unsigned rgrid(const LD &d) {
    const long long warps = ((long long)d.nrows * d.seg + 31) / 32;
    return (unsigned)std::max<long long>(1, std::min<long long>((warps + 7) / 8, 152 * 16));
}
// one warp per row
inline unsigned wgrid(const LD &d) {
    return (unsigned)std::max<long long>(1, std::min<long long>(((long long)d.nrows + 7) / 8, 152 * 16));
}

LD make_ld(int nx, int ny, int nz) {
    LD d;
    d.nx = nx; d.ny = ny; d.nz = nz;
    d.nxy = (long long)nx * ny;
    d.n = d.nxy * nz;
    d.W = (unsigned)(nx + 31) / 32;
    d.nrows = (unsigned)ny * (unsigned)nz;
    d.nwords = d.W * d.nrows;
    d.seg = 1;
    while (d.seg < 32 && (unsigned)d.seg < d.W) d.seg <<= 1;
    return d;
}

n2m_status components(LabelWork &w, const LD &d, unsigned want, int conn, unsigned *d_nroots, unsigned char *z8,
                      unsigned *z32, cudaStream_t s) {
    int *L = w.lab.as<int>();
    const unsigned *B = w.mask.as<unsigned>();
    { k_run_init<<<gsz(d.nwords), 256, 0, s>>>(B, d, want, L, z8, z32); N2M_COUNT(); }
    if (conn == 6) { k_run_merge<3><<<rgrid(d), 256, 0, s>>>(B, d, want, L); N2M_COUNT(); }
    else if (conn == 18) { k_run_merge<9><<<rgrid(d), 256, 0, s>>>(B, d, want, L); N2M_COUNT(); }
    else { k_run_merge<13><<<rgrid(d), 256, 0, s>>>(B, d, want, L); N2M_COUNT(); }
    { k_run_flatten<<<gsz(d.nwords), 256, 0, s>>>(B, d, want, L, d_nroots); N2M_COUNT(); }
    CKL();
    return N2M_OK;
}

struct Misc {
    unsigned nbg, nfg;
    unsigned long long best;
    int nl, pad;
};

// the class bits in w.mask on entry; *keep: the kept voxels' bits on return
// (the foreground after filling, or its largest component)
n2m_status label_core(LabelWork &w, const LD &d, int conn, bool only_largest, bool fill_bubbles, cudaStream_t s,
                      const unsigned **keep) {
    CKS(w.lab.ensure((size_t)d.n * sizeof(int)));
    CKS(w.misc.ensure(sizeof(Misc)));
    Misc *misc = w.misc.as<Misc>();
    CK(cudaMemsetAsync(misc, 0, sizeof(Misc), s));
    unsigned *B = w.mask.as<unsigned>();
    if (fill_bubbles) {
        CKS(w.edge.ensure((size_t)d.n));
        CKS(components(w, d, 0u, 6, &misc->nbg, w.edge.as<unsigned char>(), nullptr, s));
        { k_run_edges<<<gsz((long long)d.nrows + 4ll * (d.nx + d.ny + d.nz) * d.W), 256, 0, s>>>(B, d, w.lab.as<int>(), w.edge.as<unsigned char>()); N2M_COUNT(); }
        { k_run_fill<<<rgrid(d), 256, 0, s>>>(B, d, w.lab.as<int>(), w.edge.as<unsigned char>(), &misc->nbg); N2M_COUNT(); }
        CKL();
    }
    if (only_largest) CKS(w.cnt.ensure((size_t)d.n * sizeof(unsigned)));
    CKS(components(w, d, 1u, conn, &misc->nfg, nullptr, only_largest ? w.cnt.as<unsigned>() : nullptr, s));
    *keep = B;
    if (only_largest) {
        CKS(w.keep.ensure((size_t)d.nwords * sizeof(unsigned)));
        { k_run_sizes<<<rgrid(d), 256, 0, s>>>(B, d, w.lab.as<int>(), w.cnt.as<unsigned>()); N2M_COUNT(); }
        { k_run_best<<<gsz(d.nwords), 256, 0, s>>>(B, d, w.lab.as<int>(), w.cnt.as<unsigned>(), &misc->best); N2M_COUNT(); }
        { k_run_keep<<<rgrid(d), 256, 0, s>>>(B, d, w.lab.as<int>(), &misc->best, w.keep.as<unsigned>()); N2M_COUNT(); }
        *keep = w.keep.as<unsigned>();
    }
    { k_nl_from<<<1, 1, 0, s>>>(&misc->nfg, only_largest, &misc->nl); N2M_COUNT(); }
    CKL();
    return N2M_OK;
}

n2m_status class_bits(LabelWork &w, const LD &d, const float *vol, float iso, bool nonzero, cudaStream_t s) {
    if (d.n > 0x7fffffffLL) {
        n2m_set_error("labelling supports at most 2^31-1 voxels");
        return N2M_ERR_TOO_LARGE;
    }
    CKS(w.mask.ensure((size_t)d.nwords * sizeof(unsigned)));
    { k_lab_bits<<<wgrid(d), 256, 0, s>>>(vol, d, iso, nonzero, w.mask.as<unsigned>()); N2M_COUNT(); }
    CKL();
    return N2M_OK;
}
}  // namespace

n2m_status run_labelling(float *vol, int nx, int ny, int nz, float iso, float mn, bool only_largest,
                         bool fill_bubbles, LabelWork &w, VolStats *st, cudaStream_t s, const unsigned *vsign,
                         LabelPost *post) {
    const LD d = make_ld(nx, ny, nz);
    if (vsign) {
        if (d.n > 0x7fffffffLL) {
            n2m_set_error("labelling supports at most 2^31-1 voxels");
            return N2M_ERR_TOO_LARGE;
        }
        CKS(w.mask.ensure((size_t)d.nwords * sizeof(unsigned)));
        { k_lab_bits_vsign<<<gsz(d.nwords), 256, 0, s>>>(vsign, d, (unsigned)(ny + 7) / 8, w.mask.as<unsigned>()); N2M_COUNT(); }
        CKL();
    } else {
        CKS(class_bits(w, d, vol, iso, false, s));
    }
    const unsigned *K;
    CKS(label_core(w, d, 18, only_largest, fill_bubbles, s, &K));
    if (post) *post = LabelPost{K, d.W, mn, iso, fill_bubbles, only_largest};
    const unsigned g = wgrid(d);
    const bool v4 = nx % 4 == 0 && ((uintptr_t)vol & 15) == 0, one = d.W <= 32;
    if (only_largest && fill_bubbles && one) { k_lab_final<true, true, true><<<g, 256, 0, s>>>(K, d, vol, iso, mn, st, v4); N2M_COUNT(); }
    else if (only_largest && fill_bubbles) { k_lab_final<true, true, false><<<g, 256, 0, s>>>(K, d, vol, iso, mn, st, v4); N2M_COUNT(); }
    else if (only_largest && one) { k_lab_final<true, false, true><<<g, 256, 0, s>>>(K, d, vol, iso, mn, st, v4); N2M_COUNT(); }
    else if (only_largest) { k_lab_final<true, false, false><<<g, 256, 0, s>>>(K, d, vol, iso, mn, st, v4); N2M_COUNT(); }
    else if (fill_bubbles) { k_lab_final<false, true, false><<<g, 256, 0, s>>>(K, d, vol, iso, mn, st, v4); N2M_COUNT(); }
    else { k_lab_final<false, false, false><<<g, 256, 0, s>>>(K, d, vol, iso, mn, st, v4); N2M_COUNT(); }
    CKL();
    return N2M_OK;
}

n2m_status run_bwlabel(float *vol, int nx, int ny, int nz, int conn, bool only_largest, bool fill_bubbles,
                       LabelWork &w, ScanWork &sw, int *d_nl, cudaStream_t s) {
    const LD d = make_ld(nx, ny, nz);
    CKS(class_bits(w, d, vol, 0.0f, true, s));
    const unsigned *K;
    CKS(label_core(w, d, conn, only_largest, fill_bubbles, s, &K));
    if (only_largest) {
        { k_write_keep<<<wgrid(d), 256, 0, s>>>(K, d, vol); N2M_COUNT(); }
    } else {
        CKS(w.rc.ensure(((size_t)d.nwords + 1) * sizeof(unsigned)));
        CKS(w.cnt.ensure((size_t)d.n * sizeof(unsigned)));
        unsigned *rc = w.rc.as<unsigned>();
        CK(cudaMemsetAsync(rc + d.nwords, 0, sizeof(unsigned), s));
        { k_root_count<<<gsz(d.nwords), 256, 0, s>>>(K, d, w.lab.as<int>(), rc); N2M_COUNT(); }
        CKL();
        CKS(scan_u32(rc, (size_t)d.nwords + 1, rc + d.nwords, sw, s));
        { k_root_rank<<<gsz(d.nwords), 256, 0, s>>>(K, d, w.lab.as<int>(), rc, w.cnt.as<unsigned>()); N2M_COUNT(); }
        { k_write_labels<<<wgrid(d), 256, 0, s>>>(K, d, w.lab.as<int>(), w.cnt.as<unsigned>(), vol); N2M_COUNT(); }
    }
    CK(cudaMemcpyAsync(d_nl, &w.misc.as<Misc>()->nl, sizeof(int), cudaMemcpyDeviceToDevice, s));
    CKL();
    return N2M_OK;
}
