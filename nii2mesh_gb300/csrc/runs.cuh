// runs.cuh — x-runs of a class in row-aligned bit words (bit x & 31 of a row's
// word x / 32): run starts, the start of the run holding a bit, and the row
// kernels' per-lane view of one word.  Shared by the single-volume labelling
// and the batched atlas clustering.
#pragma once

namespace runs {
constexpr unsigned FULL = 0xffffffffu;

// x of the highest run start at or below bit b, or -1
__device__ __forceinline__ int last_start(unsigned starts, int x0, int b) {
    const unsigned hs = starts & (b == 31 ? FULL : (2u << b) - 1u);
    return hs ? x0 + 31 - __clz(hs) : -1;
}

// one lane's word of a row in a row kernel: class bits, the class word before
// it, run starts, and cs = start (x) of the run holding the voxel before the word
struct WordRuns {
    unsigned c, pc, starts;
    int x0, cs;
    __device__ __forceinline__ int start_of(int b) const {   // run of bit b (set in c)
        const int s = last_start(starts, x0, b);
        return s >= 0 ? s : cs;
    }
};

// carry_start / carry_word: the row's last run start and last class word of
// the chunks before this one (-1 / 0 before the first); all lanes call it
__device__ __forceinline__ WordRuns word_runs(unsigned c, int x0, int li, int seg, int &carry_start,
                                              unsigned &carry_word) {
    WordRuns r;
    r.c = c;
    r.x0 = x0;
    const unsigned up = __shfl_up_sync(FULL, c, 1, seg);
    r.pc = li == 0 ? carry_word : up;
    r.starts = c & ~((c << 1) | (r.pc >> 31));
    int incl = r.starts ? x0 + 31 - __clz(r.starts) : -1;
    for (int d = 1; d < seg; d <<= 1) {
        const int t = __shfl_up_sync(FULL, incl, d, seg);
        if (li >= d) incl = max(incl, t);
    }
    const int excl = __shfl_up_sync(FULL, incl, 1, seg);
    r.cs = max(carry_start, li == 0 ? -1 : excl);
    carry_start = max(carry_start, __shfl_sync(FULL, incl, seg - 1, seg));
    carry_word = __shfl_sync(FULL, c, seg - 1, seg);
    return r;
}

// bits (x mask) of the piece of a run that starts at bit b of class word rem
__device__ __forceinline__ unsigned piece_at(unsigned rem, int b) {
    const unsigned ones = ~(rem >> b);
    const int len = ones ? __ffs(ones) - 1 : 32 - b;
    return (len == 32 ? FULL : (1u << len) - 1u) << b;
}

}  // namespace runs
