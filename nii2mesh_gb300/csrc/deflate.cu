// deflate.cu — gzip (RFC 1952), zlib (RFC 1950) and raw deflate (RFC 1951)
// streams of a device buffer, for the mesh writers: save_mz3 writes its file
// through gzopen/gzwrite (src/meshify.c:602-679) and save_gii zlib-compresses
// each data array before base64 (src/meshify.c:863-873, 904-914).  zlib at its
// default level does ~15 MB/s on one core; here the input is cut into 16-32 KB
// chunks (sized so that k_lz runs in one wave), each coded by one warp as one
// dynamic-Huffman block:
//
//   k_lz        match finding and parsing.  A 4-byte hash table per warp in
//               shared memory holds the two most recent positions of each hash
//               from earlier 32-byte tiles; inside a tile the most recent earlier
//               lanes with the same hash come from __match_any_sync (two
//               candidates per position; on mesh bytes this lands within ~5 %
//               of zlib's level-6 size).  The parse is greedy with one-step lazy
//               evaluation, walked over the tile's match-start ballot (one step
//               per match, not per byte).  Emits 32-bit tokens and the block's
//               symbol histogram.
//   k_huff      canonical Huffman codes (lengths <= 15; code-length code <= 7)
//               and the block header for a group of neighbouring chunks (as few
//               as let the groups run in one wave) from their summed histogram;
//               each chunk's coded size from its own histogram, and a stored
//               block instead when that is smaller.
//   scan        chunk byte offsets (every chunk ends on a byte boundary: a
//               non-final dynamic block is followed by an empty stored block, the
//               "sync flush" of RFC 1951 3.2.4).
//   k_bits      one warp per chunk writes its bits through a shared-memory ring
//               of 32-bit words (shared atomics; no global atomics), flushed as
//               bytes in order.
//   k_cksum     CRC-32 (gzip) or Adler-32 (zlib): every 1 KB segment's share of
//               the checksum is independent (CRC-32 is linear over XOR), so
//               threads reduce them with warp shuffles and one atomic per block.
//
// The compressed bytes differ from zlib's (different match search); the
// decompressed bytes are identical, which is the parity the tests check.
#include "n2m_internal.cuh"

namespace {
constexpr int DF_CHUNK_MIN = 16384, DF_CHUNK_MAX = 32768;   // input bytes per block (chosen per call)
constexpr int DF_HBITS = 10, DF_HSIZE = 1 << DF_HBITS;   // hash buckets per chunk, two positions each
constexpr int LZ_WARPS = 16;                     // chunks per CTA of k_lz (4.6 KB of shared memory each: 48 warps / SM)
constexpr int DF_WARPS = 4;                      // chunks per CTA of k_huff
constexpr int BITS_WARPS = 8;                    // chunks per CTA of k_bits
constexpr int DF_MAXLEN = 258;
constexpr int DF_NLIT = 286, DF_NDIST = 30, DF_NSYM = 320;   // histogram stride: 286 + 30, padded
constexpr int DF_HDR_WORDS = 160;                // block header bits per code (<= 4498 used)
constexpr int DF_SEG = 1024;                     // checksum segment
constexpr unsigned CRC_POLY = 0xEDB88320u;       // CRC-32, reflected
constexpr unsigned ADLER_MOD = 65521u;

struct DfInfo {
    unsigned hdr_bits;   // block header bits (BFINAL, BTYPE, code description)
    unsigned stored;     // 1: the chunk is written as a stored block
    unsigned ntok;
    unsigned len;        // input bytes of the chunk
};

__device__ __forceinline__ unsigned load4(const unsigned *__restrict__ w, long long p) {
    const long long i = p >> 2;
    const unsigned sh = (unsigned)(p & 3) * 8u;
    const unsigned lo = __ldg(w + i);
    if (!sh) return lo;
    return __funnelshift_r(lo, __ldg(w + i + 1), sh);
}

// length of the match of p against c (first 4 bytes known equal), at most maxl
__device__ __forceinline__ int match_len(const unsigned *__restrict__ src, long long p, long long c, int maxl) {
    int l = 4;
    while (l < maxl) {
        const unsigned x = load4(src, p + l) ^ load4(src, c + l);
        if (x) return min(l + ((__ffs(x) - 1) >> 3), maxl);
        l += 4;
    }
    return maxl;
}

// RFC 1951 3.2.5: length 3..258 -> symbol 257..285 + extra bits
__host__ __device__ __forceinline__ void len_code(unsigned L, unsigned &sym, unsigned &nx, unsigned &xv) {
    if (L == 258) {
        sym = 285;
        nx = xv = 0;
        return;
    }
    const unsigned v = L - 3;
    if (v < 8) {
        sym = 257 + v;
        nx = xv = 0;
        return;
    }
#ifdef __CUDA_ARCH__
    const unsigned nb = 31 - __clz(v);
#else
    const unsigned nb = 31 - __builtin_clz(v);
#endif
    sym = 257 + 4 * (nb - 1) + ((v >> (nb - 2)) & 3u);
    nx = nb - 2;
    xv = v & ((1u << nx) - 1);
}
// distance 1..32768 -> symbol 0..29 + extra bits
__host__ __device__ __forceinline__ void dist_code(unsigned d, unsigned &sym, unsigned &nx, unsigned &xv) {
    const unsigned v = d - 1;
    if (v < 4) {
        sym = v;
        nx = xv = 0;
        return;
    }
#ifdef __CUDA_ARCH__
    const unsigned nb = 31 - __clz(v);
#else
    const unsigned nb = 31 - __builtin_clz(v);
#endif
    sym = 2 * nb + ((v >> (nb - 1)) & 1u);
    nx = nb - 1;
    xv = v & ((1u << nx) - 1);
}
__device__ __forceinline__ unsigned len_extra_bits(unsigned sym) { return (sym < 265 || sym == 285) ? 0u : (sym - 261) / 4; }
__device__ __forceinline__ unsigned dist_extra_bits(unsigned d) { return d < 4 ? 0u : d / 2 - 1; }

// ---- match finding and parsing --------------------------------------------------------------
// src must have n + 8 readable bytes (4-byte aligned); chunks of ch bytes; tokens: ch per chunk.
// Hash bucket: the chunk offsets of the two most recent positions with that hash
// (newest in the low half, 0xFFFF = none).  Histogram: 16-bit counts in pairs.
__global__ void __launch_bounds__(32 * LZ_WARPS, 3) k_lz(const unsigned *__restrict__ src, long long n, int nchunks,
                                                         int ch, unsigned *__restrict__ tokens,
                                                         DfInfo *__restrict__ info, unsigned *__restrict__ ghist) {
    extern __shared__ unsigned sm_ht[];   // LZ_WARPS tables of DF_HSIZE buckets
    __shared__ unsigned hist_s[LZ_WARPS][DF_NSYM / 2];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int chunk = blockIdx.x * LZ_WARPS + warp;
    if (chunk >= nchunks) return;   // whole warp; no block barrier below
    unsigned *ht = sm_ht + warp * DF_HSIZE;
    unsigned *hist = hist_s[warp];
    for (int i = lane; i < DF_HSIZE; i += 32) ht[i] = 0xFFFFFFFFu;
    for (int i = lane; i < DF_NSYM / 2; i += 32) hist[i] = 0;
    __syncwarp();
    const long long c0 = (long long)chunk * ch;
    const int len_c = (int)min((long long)ch, n - c0);
    unsigned *tok = tokens + (size_t)chunk * ch;
    const unsigned lt = (1u << lane) - 1;
    int next = 0, ntk = 0;
    for (int t0 = 0; t0 < len_c; t0 += 32) {
        const int o = t0 + lane;
        const bool in = o < len_c, valid = o + 4 <= len_c;
        const unsigned w4 = in ? load4(src, c0 + o) : 0u;
        const unsigned h = valid ? (w4 * 2654435761u) >> (32 - DF_HBITS) : (0x10000u | (unsigned)lane);   // lanes
        // without 4 bytes get keys no hash can take
        const unsigned same = __match_any_sync(0xffffffffu, h);
        // candidates, most recent first: earlier lanes of this tile with the same hash, then the bucket
        const unsigned lower = same & lt;
        int c1 = -1, c2 = -1;
        unsigned bk = 0xFFFFFFFFu;
        if (valid) {
            bk = ht[h];
            const int b0 = (bk & 0xFFFFu) != 0xFFFFu ? (int)(bk & 0xFFFFu) : -1;
            const int b1 = (bk >> 16) != 0xFFFFu ? (int)(bk >> 16) : -1;
            if (lower) {
                const int q1 = 31 - __clz(lower);
                c1 = t0 + q1;
                const unsigned l2 = lower & ~(1u << q1);
                c2 = l2 ? t0 + 31 - __clz(l2) : b0;
            } else {
                c1 = b0;
                c2 = b1;
            }
        }
        __syncwarp();
        if (valid && (same >> lane) == 1u)   // the last lane of each hash keeps itself and the one before
            ht[h] = ((lower ? (unsigned)(t0 + 31 - __clz(lower)) : (bk & 0xFFFFu)) << 16) | (unsigned)o;
        int mlen = 0, mdist = 0;
        if (valid) {
            const int maxl = min(DF_MAXLEN, len_c - o);
            if (c1 >= 0 && load4(src, c0 + c1) == w4) {
                mlen = match_len(src, c0 + o, c0 + c1, maxl);
                mdist = o - c1;
            }
            if (c2 >= 0 && mlen < maxl && load4(src, c0 + c2) == w4) {
                const int l = match_len(src, c0 + o, c0 + c2, maxl);
                if (l > mlen) {
                    mlen = l;
                    mdist = o - c2;
                }
            }
        }
        // greedy parse with one-step lazy evaluation over the match starts of this tile
        const unsigned mm = __ballot_sync(0xffffffffu, mlen >= 4);
        const unsigned tmask = (len_c - t0 >= 32) ? 0xffffffffu : ((1u << (len_c - t0)) - 1);
        unsigned lit = 0, mat = 0;
        int pos = next - t0;
        while (pos < 32) {
            const unsigned rest = mm & (0xffffffffu << pos);
            if (!rest) {
                lit |= 0xffffffffu << pos;
                pos = 32;
                break;
            }
            const int q = __ffs(rest) - 1;
            lit |= ((1u << q) - 1) & (0xffffffffu << pos);
            const int lq = __shfl_sync(0xffffffffu, mlen, q);
            const int lq1 = __shfl_sync(0xffffffffu, mlen, (q + 1) & 31);
            if (q < 31 && lq1 > lq) {
                lit |= 1u << q;
                pos = q + 1;
                continue;
            }
            mat |= 1u << q;
            pos = q + lq;
        }
        next = t0 + pos;
        lit &= tmask;
        const unsigned all = lit | mat;
        if ((all >> lane) & 1u) {
            unsigned t;
            if ((mat >> lane) & 1u) {
                t = 0x80000000u | ((unsigned)(mlen - 3) << 15) | (unsigned)(mdist - 1);
                unsigned sym, nx, xv;
                len_code((unsigned)mlen, sym, nx, xv);
                atomicAdd(&hist[sym >> 1], 1u << (16 * (sym & 1u)));
                dist_code((unsigned)mdist, sym, nx, xv);
                sym += DF_NLIT;
                atomicAdd(&hist[sym >> 1], 1u << (16 * (sym & 1u)));
            } else {
                t = w4 & 0xFFu;
                atomicAdd(&hist[t >> 1], 1u << (16 * (t & 1u)));
            }
            tok[ntk + __popc(all & lt)] = t;
        }
        ntk += __popc(all);
    }
    __syncwarp();
    if (lane == 0) {
        info[chunk].ntok = (unsigned)ntk;
        info[chunk].len = (unsigned)max(len_c, 0);
    }
    for (int i = lane; i < DF_NSYM; i += 32)   // unpacked; symbol 256 (end of block) once
        ghist[(size_t)chunk * DF_NSYM + i] = ((hist[i >> 1] >> (16 * (i & 1))) & 0xFFFFu) + (i == 256 ? 1u : 0u);
}

// ---- per-chunk Huffman codes ----------------------------------------------------------------
struct HuffScratch {
    unsigned keys[512];                 // sort keys: frequency << 9 | symbol
    unsigned w[2 * DF_NLIT];            // internal node weights (nodes m .. 2m-2)
    unsigned short par[2 * DF_NLIT];    // parent of every node
    unsigned char dep[2 * DF_NLIT];
    unsigned freq[DF_NSYM];             // histogram (phantom symbols added for the code construction)
    unsigned char len[DF_NSYM];         // code lengths: literal/length 0..285, distance 286..315
    unsigned code[DF_NSYM];             // bit-reversed code | length << 16
    unsigned short rle[DF_NSYM];        // code-length symbols: symbol | extra value << 5
    unsigned clf[19], clc[19];
    unsigned char cll[19];
    unsigned cnt[16];                   // codes per length, then the next code of each length
    unsigned hdr[DF_HDR_WORDS];
};

// warp-wide bitonic sort of keys[0, n), n a power of two
__device__ void warp_sort(unsigned *keys, int n, int lane) {
    for (int k = 2; k <= n; k <<= 1)
        for (int j = k >> 1; j > 0; j >>= 1) {
            for (int i = lane; i < n; i += 32) {
                const int l = i ^ j;
                if (l > i) {
                    const unsigned a = keys[i], b = keys[l];
                    if ((a > b) == ((i & k) == 0)) {
                        keys[i] = b;
                        keys[l] = a;
                    }
                }
            }
            __syncwarp();
        }
}

// Huffman code lengths (<= limit) of f[0, nsym) into L[0, nsym); at least two
// symbols of f must be nonzero.  Frequencies are halved until the tree fits.
__device__ void build_lengths(HuffScratch &S, const unsigned *f, int nsym, int limit, unsigned char *L, int lane) {
    const int padn = nsym <= 32 ? 32 : 512;
    for (int shift = 0;; shift++) {
        for (int i = lane; i < padn; i += 32) {
            unsigned k = 0xFFFFFFFFu;
            if (i < nsym && f[i]) k = ((shift ? ((f[i] >> shift) | 1u) : f[i]) << 9) | (unsigned)i;
            S.keys[i] = k;
        }
        __syncwarp();
        warp_sort(S.keys, padn, lane);
        int ok = 1, m = 0;
        if (lane == 0) {
            while (m < padn && S.keys[m] != 0xFFFFFFFFu) m++;
            // two queues: sorted leaves 0..m-1 and internal nodes m.. in creation order
            int li = 0, ii = m, ni = m;
            for (int k = 0; k < m - 1; k++) {
                int ab[2];
                unsigned wab[2];
                for (int t = 0; t < 2; t++) {
                    if (li < m && (ii >= ni || (S.keys[li] >> 9) <= S.w[ii])) {
                        ab[t] = li;
                        wab[t] = S.keys[li] >> 9;
                        li++;
                    } else {
                        ab[t] = ii;
                        wab[t] = S.w[ii];
                        ii++;
                    }
                }
                S.w[ni] = wab[0] + wab[1];
                S.par[ab[0]] = (unsigned short)ni;
                S.par[ab[1]] = (unsigned short)ni;
                ni++;
            }
            const int root = 2 * m - 2;
            S.dep[root] = 0;
            int maxd = 0;
            for (int j = root - 1; j >= 0; j--) {
                S.dep[j] = S.dep[S.par[j]] + 1;
                if (j < m && S.dep[j] > maxd) maxd = S.dep[j];
            }
            ok = maxd <= limit;
        }
        ok = __shfl_sync(0xffffffffu, ok, 0);
        m = __shfl_sync(0xffffffffu, m, 0);
        __syncwarp();
        if (ok) {
            for (int i = lane; i < nsym; i += 32) L[i] = 0;
            __syncwarp();
            for (int i = lane; i < m; i += 32) L[S.keys[i] & 511u] = S.dep[i];
            __syncwarp();
            return;
        }
    }
}

// canonical codes (RFC 1951 3.2.2), stored bit-reversed for LSB-first output; warp-wide:
// a symbol's code is the first code of its length plus the number of smaller
// symbols of that length (ranked 32 symbols at a time with __match_any_sync)
__device__ void assign_codes(const unsigned char *L, unsigned *code, int nsym, unsigned *cnt, int lane) {
    if (lane < 16) cnt[lane] = 0;
    __syncwarp();
    for (int s = lane; s < nsym; s += 32)
        if (L[s]) atomicAdd(&cnt[L[s]], 1u);
    __syncwarp();
    if (lane == 0) {
        unsigned c = 0, prev = 0;
        for (int b = 1; b < 16; b++) {
            c = (c + prev) << 1;
            prev = cnt[b];
            cnt[b] = c;
        }
    }
    __syncwarp();
    for (int base = 0; base < nsym; base += 32) {
        const int sym = base + lane;
        const unsigned l = sym < nsym ? L[sym] : 0u;
        const unsigned peers = __match_any_sync(0xffffffffu, l);
        const unsigned c = cnt[l] + __popc(peers & ((1u << lane) - 1));
        if (sym < nsym) code[sym] = l ? ((__brev(c) >> (32 - l)) | (l << 16)) : 0u;
        __syncwarp();
        if (l && (peers >> lane) == 1u) cnt[l] += __popc(peers);   // the last lane of each length
        __syncwarp();
    }
}

struct BitSink {
    unsigned *buf;
    unsigned pos;
    __device__ void put(unsigned v, unsigned nb) {   // nb <= 25
        if (!nb) return;
        const unsigned wi = pos >> 5, sh = pos & 31;
        buf[wi] |= v << sh;
        if (sh + nb > 32) buf[wi + 1] |= v >> (32 - sh);
        pos += nb;
    }
};

__constant__ unsigned char c_clorder[19] = {16, 17, 18, 0, 8, 7, 9, 6, 10, 5, 11, 4, 12, 3, 13, 2, 14, 1, 15};

// One code for a group of G neighbouring chunks (G set per call so that the
// groups fit one wave: each warp's tree build is a serial chain), from their
// summed histogram; each chunk keeps its own block (header, size, stored or
// not).  The header is written with BFINAL = 0; k_bits sets it on the last chunk.
__global__ void __launch_bounds__(32 * DF_WARPS) k_huff(const unsigned *__restrict__ ghist, int nchunks, int G,
                                                        DfInfo *__restrict__ info, unsigned *__restrict__ gcodes,
                                                        unsigned *__restrict__ ghdr, unsigned *__restrict__ sizes) {
    __shared__ HuffScratch sc[DF_WARPS];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int group = blockIdx.x * DF_WARPS + warp;
    const int c0 = group * G, c1 = min(c0 + G, nchunks);
    if (c0 >= nchunks) return;
    HuffScratch &S = sc[warp];
    for (int i = lane; i < DF_NSYM; i += 32) {
        unsigned f = 0;
        if (i < DF_NLIT + DF_NDIST)
            for (int c = c0; c < c1; c++) f += ghist[(size_t)c * DF_NSYM + i];
        S.freq[i] = f;
    }
    for (int i = lane; i < DF_HDR_WORDS; i += 32) S.hdr[i] = 0;
    __syncwarp();
    if (lane == 0) {
        // every code needs two symbols: phantoms 0/1 where the block uses fewer
        int used = 0;
        for (int i = 0; i < DF_NLIT; i++) used += S.freq[i] != 0;
        for (int i = 0; used < 2; i++)
            if (!S.freq[i]) S.freq[i] = 1, used++;
        used = 0;
        for (int i = 0; i < DF_NDIST; i++) used += S.freq[DF_NLIT + i] != 0;
        for (int i = 0; used < 2; i++)
            if (!S.freq[DF_NLIT + i]) S.freq[DF_NLIT + i] = 1, used++;
    }
    __syncwarp();
    build_lengths(S, S.freq, DF_NLIT, 15, S.len, lane);
    build_lengths(S, S.freq + DF_NLIT, DF_NDIST, 15, S.len + DF_NLIT, lane);
    int ncl = 0;
    assign_codes(S.len, S.code, DF_NLIT, S.cnt, lane);
    assign_codes(S.len + DF_NLIT, S.code + DF_NLIT, DF_NDIST, S.cnt, lane);
    if (lane == 0) {
        int hlit = DF_NLIT, hdist = DF_NDIST;
        while (hlit > 257 && !S.len[hlit - 1]) hlit--;
        while (hdist > 1 && !S.len[DF_NLIT + hdist - 1]) hdist--;
        // run-length code of the code lengths (runs may cross from literal/length to distance)
        const int total = hlit + hdist;
        int nr = 0;
        for (int i = 0; i < total;) {
            const unsigned v = i < hlit ? S.len[i] : S.len[DF_NLIT + i - hlit];
            int run = 1;
            while (i + run < total && (i + run < hlit ? S.len[i + run] : S.len[DF_NLIT + i + run - hlit]) == v) run++;
            int r = run;
            if (v == 0) {
                while (r >= 11) {
                    const int c = min(r, 138);
                    S.rle[nr++] = (unsigned short)(18 | (c - 11) << 5);
                    r -= c;
                }
                if (r >= 3) {
                    S.rle[nr++] = (unsigned short)(17 | (r - 3) << 5);
                    r = 0;
                }
                while (r-- > 0) S.rle[nr++] = 0;
            } else {
                S.rle[nr++] = (unsigned short)v;
                r--;
                while (r >= 3) {
                    const int c = min(r, 6);
                    S.rle[nr++] = (unsigned short)(16 | (c - 3) << 5);
                    r -= c;
                }
                while (r-- > 0) S.rle[nr++] = (unsigned short)v;
            }
            i += run;
        }
        for (int i = 0; i < 19; i++) S.clf[i] = 0;
        for (int i = 0; i < nr; i++) S.clf[S.rle[i] & 31]++;
        int used = 0;
        for (int i = 0; i < 19; i++) used += S.clf[i] != 0;
        for (int i = 0; used < 2; i++)
            if (!S.clf[i]) S.clf[i] = 1, used++;
        S.keys[0] = (unsigned)hlit;   // handed to the other lanes' code below through shared memory
        S.keys[1] = (unsigned)hdist;
        S.keys[2] = (unsigned)nr;
        ncl = 0;
    }
    __syncwarp();
    const int hlit = (int)S.keys[0], hdist = (int)S.keys[1], nr = (int)S.keys[2];
    __syncwarp();
    build_lengths(S, S.clf, 19, 7, S.cll, lane);
    assign_codes(S.cll, S.clc, 19, S.cnt, lane);
    if (lane == 0) {
        ncl = 19;
        while (ncl > 4 && !S.cll[c_clorder[ncl - 1]]) ncl--;
        BitSink b{S.hdr, 0};
        b.put(0u, 1);   // BFINAL (set by k_bits on the last chunk)
        b.put(2u, 2);   // BTYPE 10: dynamic Huffman codes
        b.put((unsigned)(hlit - 257), 5);
        b.put((unsigned)(hdist - 1), 5);
        b.put((unsigned)(ncl - 4), 4);
        for (int k = 0; k < ncl; k++) b.put(S.cll[c_clorder[k]], 3);
        for (int i = 0; i < nr; i++) {
            const unsigned sym = S.rle[i] & 31u, x = S.rle[i] >> 5;
            b.put(S.clc[sym] & 0xFFFFu, S.clc[sym] >> 16);
            if (sym == 16) b.put(x, 2);
            else if (sym == 17) b.put(x, 3);
            else if (sym == 18) b.put(x, 7);
        }
        S.keys[3] = b.pos;
    }
    __syncwarp();
    for (int chunk = c0; chunk < c1; chunk++) {   // each chunk's coded size with its own frequencies
        const bool last = chunk == nchunks - 1;
        const unsigned *f = ghist + (size_t)chunk * DF_NSYM;
        unsigned long long bits = 0;
        for (int i = lane; i < DF_NLIT + DF_NDIST; i += 32) {
            const unsigned fi = f[i];
            if (fi)
                bits += (unsigned long long)fi * (S.len[i] + (i < DF_NLIT ? (i > 256 ? len_extra_bits((unsigned)i) : 0u)
                                                                          : dist_extra_bits((unsigned)(i - DF_NLIT))));
        }
        for (int d = 16; d > 0; d >>= 1) bits += __shfl_xor_sync(0xffffffffu, bits, d);
        if (lane == 0) {
            const unsigned hb = S.keys[3];
            bits += hb;
            const unsigned long long dyn = last ? (bits + 7) / 8 : (bits + 3 + 7) / 8 + 4;
            const unsigned len = info[chunk].len;
            const unsigned long long st = 5ull + len;
            const bool stored = st <= dyn;
            info[chunk].hdr_bits = hb;
            info[chunk].stored = stored;
            sizes[chunk] = (unsigned)(stored ? st : dyn);
        }
    }
    __syncwarp();
    for (int i = lane; i < DF_NLIT + DF_NDIST; i += 32) gcodes[(size_t)group * DF_NSYM + i] = S.code[i];
    for (int i = lane; i < DF_HDR_WORDS; i += 32) ghdr[(size_t)group * DF_HDR_WORDS + i] = S.hdr[i];
}

// ---- bit output -------------------------------------------------------------------------------
constexpr int RING = 128;   // words; one put advances at most 32 * 57 bits

// warp-wide: lane i appends v (nb <= 57 bits) after lanes < i; complete words go to dst as bytes
// (never past lim, the planned size of the chunk)
__device__ __forceinline__ void ring_put(unsigned *ring, unsigned &bp, unsigned &fw, unsigned long long v, unsigned nb,
                                         unsigned char *__restrict__ dst, unsigned lim, int lane) {
    unsigned x = nb;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const unsigned y = __shfl_up_sync(0xffffffffu, x, d);
        if (lane >= d) x += y;
    }
    const unsigned total = __shfl_sync(0xffffffffu, x, 31);
    if (nb) {
        const unsigned p = bp + x - nb, wi = p >> 5, sh = p & 31;
        const unsigned long long vs = v << sh;
        atomicOr(&ring[wi & (RING - 1)], (unsigned)vs);
        if (sh + nb > 32) atomicOr(&ring[(wi + 1) & (RING - 1)], (unsigned)(vs >> 32));
        if (sh + nb > 64) atomicOr(&ring[(wi + 2) & (RING - 1)], (unsigned)(v >> (64 - sh)));
    }
    bp += total;
    __syncwarp();
    const unsigned full = bp >> 5;
    for (unsigned w = fw + lane; w < full; w += 32) {
        const unsigned val = ring[w & (RING - 1)];
        ring[w & (RING - 1)] = 0;
        for (unsigned b = 0; b < 4; b++)
            if (4 * w + b < lim) dst[4 * w + b] = (unsigned char)(val >> (8 * b));
    }
    fw = full;
    __syncwarp();
}

__global__ void __launch_bounds__(32 * BITS_WARPS) k_bits(const unsigned char *__restrict__ src, const unsigned *__restrict__ tokens,
                                                        const DfInfo *__restrict__ info, const unsigned *__restrict__ gcodes,
                                                        const unsigned *__restrict__ ghdr, const unsigned *__restrict__ offs,
                                                        int nchunks, int ch, int G, unsigned char *__restrict__ out,
                                                        unsigned *__restrict__ err) {
    __shared__ unsigned ring_s[BITS_WARPS][RING];
    __shared__ unsigned code_s[BITS_WARPS][DF_NLIT + DF_NDIST];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int chunk = blockIdx.x * BITS_WARPS + warp;
    if (chunk >= nchunks) return;
    const DfInfo I = info[chunk];
    const bool last = chunk == nchunks - 1;
    unsigned char *dst = out + offs[chunk];
    const unsigned lim = offs[chunk + 1] - offs[chunk];   // planned size: no byte is written beyond it
    const size_t c0 = (size_t)chunk * ch;
    if (I.stored) {
        if (lim != 5 + I.len) {
            if (lane == 0) atomicOr(err, 1u);
            return;
        }
        if (lane == 0) {
            dst[0] = last ? 1 : 0;   // BFINAL, BTYPE 00, then padding to the byte
            dst[1] = (unsigned char)I.len;
            dst[2] = (unsigned char)(I.len >> 8);
            dst[3] = (unsigned char)~I.len;
            dst[4] = (unsigned char)(~I.len >> 8);
        }
        for (unsigned i = lane; i < I.len; i += 32) dst[5 + i] = src[c0 + i];
        return;
    }
    unsigned *ring = ring_s[warp];
    unsigned *code = code_s[warp];
    for (int i = lane; i < RING; i += 32) ring[i] = 0;
    const int group = chunk / G;
    for (int i = lane; i < DF_NLIT + DF_NDIST; i += 32) code[i] = gcodes[(size_t)group * DF_NSYM + i];
    __syncwarp();
    unsigned bp = 0, fw = 0;
    const unsigned *hdr = ghdr + (size_t)group * DF_HDR_WORDS;
    for (unsigned w0 = 0; w0 * 32 < I.hdr_bits; w0 += 32) {
        const unsigned wi = w0 + lane;
        unsigned nb = 0;
        unsigned long long v = 0;
        if (wi * 32 < I.hdr_bits) {
            nb = min(32u, I.hdr_bits - wi * 32);
            v = hdr[wi] & (nb == 32 ? 0xffffffffu : ((1u << nb) - 1));
            if (wi == 0 && last) v |= 1u;   // BFINAL
        }
        ring_put(ring, bp, fw, v, nb, dst, lim, lane);
    }
    const unsigned *tok = tokens + c0;
    unsigned tnext = lane < I.ntok ? tok[lane] : 0u;   // the next group's tokens are loaded one group ahead
    for (unsigned t0 = 0; t0 < I.ntok; t0 += 32) {
        unsigned nb = 0;
        unsigned long long v = 0;
        const unsigned t = tnext;
        if (t0 + 32 + lane < I.ntok) tnext = tok[t0 + 32 + lane];
        if (t0 + lane < I.ntok) {
            if (t & 0x80000000u) {
                unsigned ls, lx, lv, ds, dx, dv;
                len_code(((t >> 15) & 0xFFu) + 3, ls, lx, lv);
                dist_code((t & 0x7FFFu) + 1, ds, dx, dv);
                const unsigned lc = code[ls], dc = code[DF_NLIT + ds];
                const unsigned ll = lc >> 16, dl = dc >> 16;
                v = (unsigned long long)(lc & 0xFFFFu) | ((unsigned long long)lv << ll) |
                    ((unsigned long long)(dc & 0xFFFFu) << (ll + lx)) | ((unsigned long long)dv << (ll + lx + dl));
                nb = ll + lx + dl + dx;
            } else {
                const unsigned c = code[t];
                v = c & 0xFFFFu;
                nb = c >> 16;
            }
        }
        ring_put(ring, bp, fw, v, nb, dst, lim, lane);
    }
    {   // end of block; then the empty stored block that byte-aligns a non-final chunk
        const unsigned c = code[256];
        ring_put(ring, bp, fw, lane == 0 ? (c & 0xFFFFu) : 0ull, lane == 0 ? (c >> 16) : 0u, dst, lim, lane);
        if (!last) {
            ring_put(ring, bp, fw, 0ull, lane == 0 ? 3u : 0u, dst, lim, lane);
            bp = (bp + 7) & ~7u;
            ring_put(ring, bp, fw, lane == 0 ? 0xFFFF0000ull : 0ull, lane == 0 ? 32u : 0u, dst, lim, lane);
        }
    }
    const unsigned nbytes = (bp + 7) >> 3;
    for (unsigned w = fw + lane; w * 4 < nbytes; w += 32) {
        const unsigned val = ring[w & (RING - 1)];
        for (unsigned b = 0; b < 4 && 4 * w + b < nbytes && 4 * w + b < lim; b++)
            dst[4 * w + b] = (unsigned char)(val >> (8 * b));
    }
    if (lane == 0 && nbytes != lim) atomicOr(err, 1u);
}

// ---- checksums ----------------------------------------------------------------------------------
__device__ __forceinline__ unsigned gf2_mul(unsigned a, unsigned b) {   // a*b mod the CRC-32 polynomial (reflected)
    unsigned p = 0;
#pragma unroll 4
    for (int i = 0; i < 32; i++) {   // bit 31-i of a is the coefficient of x^i
        if (a & (0x80000000u >> i)) p ^= b;
        b = (b & 1u) ? (b >> 1) ^ CRC_POLY : b >> 1;
    }
    return p;
}

// Checksum of the whole input from independent 1 KB segments, one per thread:
// CRC-32 is linear over XOR, crc(A1 .. Ak) = XOR_i crc(A_i) * x^(8 * bytes after A_i)
// mod P; Adler-32's sums add up with the same weights (B gains, for every byte,
// the number of bytes from it to the end).  Warp and block reductions, one
// atomic per block into acc (CRC: acc[0] XOR; Adler: acc[0] += sum of bytes,
// acc[1] += weighted sum).
struct XPow {
    unsigned p[40];   // x^(8 * 2^k) mod P
};
__global__ void __launch_bounds__(256) k_cksum(const unsigned *__restrict__ src, long long n, int adler, XPow xp,
                                             unsigned long long *__restrict__ acc) {
    // slicing-by-4 tables: tab[0] the byte table, tab[k][i] = tab[k-1][i] advanced by one zero byte
    __shared__ unsigned tab[4][256];
    __shared__ unsigned long long red[2][8];
    for (int i = threadIdx.x; i < 256; i += blockDim.x) {
        unsigned c = (unsigned)i;
        for (int k = 0; k < 8; k++) c = (c & 1u) ? (c >> 1) ^ CRC_POLY : c >> 1;
        tab[0][i] = c;
    }
    __syncthreads();
    for (int i = threadIdx.x; i < 256; i += blockDim.x) {
        unsigned c = tab[0][i];
        for (int k = 1; k < 4; k++) {
            c = (c >> 8) ^ tab[0][c & 0xFFu];
            tab[k][i] = c;
        }
    }
    __syncthreads();
    const long long nseg = (n + DF_SEG - 1) / DF_SEG;
    const long long seg = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    unsigned long long a = 0, b = 0;
    if (seg < nseg) {
        const long long s0 = seg * DF_SEG;
        const unsigned L = (unsigned)min((long long)DF_SEG, n - s0);
        const unsigned long long after = (unsigned long long)(n - s0 - L);
        const unsigned *p = src + s0 / 4;
        if (!adler) {
            unsigned crc = 0xFFFFFFFFu;
            unsigned i = 0;
            for (; i + 4 <= L; i += 4) {   // four bytes per step
                const unsigned c = crc ^ __ldg(p + i / 4);
                crc = tab[3][c & 0xFFu] ^ tab[2][(c >> 8) & 0xFFu] ^ tab[1][(c >> 16) & 0xFFu] ^ tab[0][c >> 24];
            }
            if (i < L) {   // the last 1-3 bytes of the input
                const unsigned w = __ldg(p + i / 4);
                for (unsigned k = 0; i + k < L; k++) crc = tab[0][(crc ^ (w >> (8 * k))) & 0xFFu] ^ (crc >> 8);
            }
            unsigned x = 0x80000000u;   // x^(8 after)
            unsigned long long e = after;
            for (int k = 0; e; k++, e >>= 1)
                if (e & 1) x = gf2_mul(x, xp.p[k]);
            a = gf2_mul(~crc, x);
        } else {
            unsigned sm = 0, ws = 0;
            for (unsigned i = 0; i < L; i += 4) {
                const unsigned w = __ldg(p + i / 4);
                for (unsigned k = 0; k < 4 && i + k < L; k++) {
                    const unsigned v = (w >> (8 * k)) & 0xFFu;
                    sm += v;
                    ws += (L - i - k) * v;
                }
            }
            a = sm;
            b = ws + (after % ADLER_MOD) * (unsigned long long)sm;
        }
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int d = 16; d > 0; d >>= 1) {
        const unsigned long long oa = __shfl_xor_sync(0xffffffffu, a, d), ob = __shfl_xor_sync(0xffffffffu, b, d);
        if (adler) {
            a += oa;
            b += ob;
        } else {
            a ^= oa;
        }
    }
    if (lane == 0) {
        red[0][warp] = a;
        red[1][warp] = b;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < (int)(blockDim.x >> 5); w++) {
            if (adler) {
                a += red[0][w];
                b += red[1][w];
            } else {
                a ^= red[0][w];
            }
        }
        if (adler) {
            atomicAdd(acc, a);
            atomicAdd(acc + 1, b);
        } else {
            atomicXor(acc, a);
        }
    }
}

XPow xpow_table() {   // host: x^(8 * 2^k) mod P by repeated squaring
    auto mul = [](unsigned a, unsigned b) {
        unsigned p = 0;
        for (int i = 0; i < 32; i++) {
            if (a & (0x80000000u >> i)) p ^= b;
            b = (b & 1u) ? (b >> 1) ^ CRC_POLY : b >> 1;
        }
        return p;
    };
    XPow t;
    t.p[0] = 0x00800000u;   // x^8
    for (int k = 1; k < 40; k++) t.p[k] = mul(t.p[k - 1], t.p[k - 1]);
    return t;
}

// container header and trailer around the stream of `body` bytes
__global__ void k_wrap(unsigned char *out, int container, unsigned long long body, long long n,
                       const unsigned long long *__restrict__ acc) {
    if (threadIdx.x || blockIdx.x) return;
    if (container == N2M_DEFLATE_GZIP) {
        const unsigned char h[10] = {0x1f, 0x8b, 8, 0, 0, 0, 0, 0, 0, 3};   // no name, mtime 0, OS Unix (as gzopen writes)
        for (int i = 0; i < 10; i++) out[i] = h[i];
        unsigned char *t = out + 10 + body;
        const unsigned c = (unsigned)acc[0], sz = (unsigned)n;
        for (int i = 0; i < 4; i++) t[i] = (unsigned char)(c >> (8 * i));
        for (int i = 0; i < 4; i++) t[4 + i] = (unsigned char)(sz >> (8 * i));
    } else if (container == N2M_DEFLATE_ZLIB) {
        out[0] = 0x78;   // deflate, 32 KB window
        out[1] = 0x9c;   // default level; (0x78 * 256 + 0x9c) % 31 == 0
        unsigned char *t = out + 2 + body;
        const unsigned A = (unsigned)((1ull + acc[0]) % ADLER_MOD);
        const unsigned B = (unsigned)(((unsigned long long)n % ADLER_MOD + acc[1] % ADLER_MOD) % ADLER_MOD);
        const unsigned c = (B << 16) | A;
        for (int i = 0; i < 4; i++) t[i] = (unsigned char)(c >> (24 - 8 * i));   // big-endian
    }
}
}  // namespace

size_t deflate_bound(size_t n) {
    const size_t nchunks = n ? (n + DF_CHUNK_MIN - 1) / DF_CHUNK_MIN : 1;
    return n + 5 * nchunks + 18;
}

void deflate_release(DeflateWork &w) {
    DevBuf *bufs[] = {&w.tok, &w.info, &w.hist, &w.codes, &w.hdr, &w.sizes, &w.misc, &w.out};
    for (DevBuf *b : bufs) b->release();
    if (w.side) cudaStreamDestroy((cudaStream_t)w.side);
    if (w.ev_in) cudaEventDestroy((cudaEvent_t)w.ev_in);
    if (w.ev_ck) cudaEventDestroy((cudaEvent_t)w.ev_ck);
    w.side = w.ev_in = w.ev_ck = nullptr;
}

n2m_status deflate_device(const void *d_src, size_t n, int container, DeflateWork &w, ScanWork &sw, cudaStream_t s,
                          size_t *out_len) {
    if (((uintptr_t)d_src & 3) || container < N2M_DEFLATE_RAW || container > N2M_DEFLATE_GZIP || n > 0x7fffffffull) {
        n2m_set_error("deflate: bad arguments (source not 4-byte aligned, unknown container or more than 2^31-1 bytes)");
        return N2M_ERR_BAD_ARGS;
    }
    const int smem = LZ_WARPS * DF_HSIZE * (int)sizeof(unsigned);
    if (!w.lz_slots) {   // chunks k_lz keeps in flight on the whole GPU
        int dev = 0, sms = 0, per_sm = 0;
        CK(cudaGetDevice(&dev));
        CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        CK(cudaFuncSetAttribute(k_lz, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
        CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_lz, 32 * LZ_WARPS, smem));
        w.lz_slots = std::max(1, sms * per_sm * LZ_WARPS);
        CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_huff, 32 * DF_WARPS, 0));
        w.huff_slots = std::max(1, sms * per_sm * DF_WARPS);
        CK(cudaStreamCreateWithFlags((cudaStream_t *)&w.side, cudaStreamNonBlocking));
        CK(cudaEventCreateWithFlags((cudaEvent_t *)&w.ev_in, cudaEventDisableTiming));
        CK(cudaEventCreateWithFlags((cudaEvent_t *)&w.ev_ck, cudaEventDisableTiming));
    }
    // chunk size: the input in one wave of k_lz when 16-32 KB chunks allow it (every warp's
    // time is set by its chunk's serial tile loop, so a second, partial wave costs nearly a full one)
    size_t ch = (n + w.lz_slots - 1) / w.lz_slots;
    ch = std::min<size_t>(DF_CHUNK_MAX, std::max<size_t>(DF_CHUNK_MIN, (ch + 4095) / 4096 * 4096));
    const int nchunks = n ? (int)((n + ch - 1) / ch) : 1;
    const long long nseg = (long long)((n + DF_SEG - 1) / DF_SEG);
    CKS(w.tok.ensure((size_t)nchunks * ch * sizeof(unsigned)));
    CKS(w.info.ensure((size_t)nchunks * sizeof(DfInfo)));
    CKS(w.hist.ensure((size_t)nchunks * DF_NSYM * sizeof(unsigned)));
    CKS(w.codes.ensure((size_t)nchunks * DF_NSYM * sizeof(unsigned)));
    CKS(w.hdr.ensure((size_t)nchunks * DF_HDR_WORDS * sizeof(unsigned)));
    CKS(w.sizes.ensure((size_t)(nchunks + 1) * sizeof(unsigned)));
    CKS(w.misc.ensure(4 * sizeof(unsigned long long)));
    unsigned long long *acc = w.misc.as<unsigned long long>();   // [0], [1] checksum sums, [2] error flag
    CK(cudaMemsetAsync(acc, 0, 4 * sizeof(unsigned long long), s));
    // the checksum runs on the side stream next to k_lz (latency-bound, leaves bandwidth over)
    const int adler = container == N2M_DEFLATE_ZLIB;
    const bool cksum = container != N2M_DEFLATE_RAW && nseg > 0;
    if (cksum) {
        static const XPow xp = xpow_table();
        CK(cudaEventRecord((cudaEvent_t)w.ev_in, s));
        CK(cudaStreamWaitEvent((cudaStream_t)w.side, (cudaEvent_t)w.ev_in, 0));
        k_cksum<<<(unsigned)((nseg + 255) / 256), 256, 0, (cudaStream_t)w.side>>>((const unsigned *)d_src, (long long)n,
                                                                                adler, xp, acc);
        N2M_COUNT();
        CKL();
        CK(cudaEventRecord((cudaEvent_t)w.ev_ck, (cudaStream_t)w.side));
    }
    // chunks per Huffman code: the fewest that let the code builders run in one wave
    const int G = std::max(1, (nchunks + w.huff_slots - 1) / w.huff_slots);
    const int ngroups = (nchunks + G - 1) / G;
    const unsigned blocks = (unsigned)((ngroups + DF_WARPS - 1) / DF_WARPS);
    CK(cudaFuncSetAttribute(k_lz, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
    k_lz<<<(unsigned)((nchunks + LZ_WARPS - 1) / LZ_WARPS), 32 * LZ_WARPS, smem, s>>>(
        (const unsigned *)d_src, (long long)n, nchunks, (int)ch, w.tok.as<unsigned>(), w.info.as<DfInfo>(),
        w.hist.as<unsigned>());
    N2M_COUNT();
    CKL();
    k_huff<<<blocks, 32 * DF_WARPS, 0, s>>>(w.hist.as<unsigned>(), nchunks, G, w.info.as<DfInfo>(),
                                           w.codes.as<unsigned>(), w.hdr.as<unsigned>(), w.sizes.as<unsigned>());
    N2M_COUNT();
    CKL();
    CKS(scan_u32(w.sizes.as<unsigned>(), (size_t)nchunks, w.sizes.as<unsigned>() + nchunks, sw, s));
    unsigned body = 0;
    CK(cudaMemcpyAsync(&body, w.sizes.as<unsigned>() + nchunks, sizeof(unsigned), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    const size_t head = container == N2M_DEFLATE_GZIP ? 10 : container == N2M_DEFLATE_ZLIB ? 2 : 0;
    const size_t tail = container == N2M_DEFLATE_GZIP ? 8 : container == N2M_DEFLATE_ZLIB ? 4 : 0;
    const size_t total = head + body + tail;
    CKS(w.out.ensure(total + 16));
    unsigned char *out = w.out.as<unsigned char>();
    k_bits<<<(unsigned)((nchunks + BITS_WARPS - 1) / BITS_WARPS), 32 * BITS_WARPS, 0, s>>>(
        (const unsigned char *)d_src, w.tok.as<unsigned>(), w.info.as<DfInfo>(), w.codes.as<unsigned>(),
        w.hdr.as<unsigned>(), w.sizes.as<unsigned>(), nchunks, (int)ch, G, out + head, (unsigned *)(acc + 2));
    N2M_COUNT();
    CKL();
    if (cksum) CK(cudaStreamWaitEvent(s, (cudaEvent_t)w.ev_ck, 0));
    if (container != N2M_DEFLATE_RAW) {
        k_wrap<<<1, 1, 0, s>>>(out, container, body, (long long)n, acc);
        N2M_COUNT();
        CKL();
    }
    *out_len = total;
    return N2M_OK;
}

n2m_status deflate_check(DeflateWork &w, cudaStream_t s) {
    unsigned err = 0;
    CK(cudaMemcpyAsync(&err, w.misc.as<unsigned long long>() + 2, sizeof(unsigned), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    if (err) {
        n2m_set_error("deflate: coded size differs from the planned size");
        return N2M_ERR_INTERNAL;
    }
    return N2M_OK;
}
