// uf.cuh — lock-free union-find on an int32 parent array (roots point to
// themselves; hooking always links the larger root under the smaller one, so
// a component's root is its smallest index).  Shared by the single-volume and
// the batched atlas labelling kernels.
#pragma once

namespace uf {
__device__ __forceinline__ int find_root(const int *L, int i) {
    int p = ((volatile const int *)L)[i];
    while (p != i) {
        i = p;
        p = ((volatile const int *)L)[i];
    }
    return i;
}

// root search with path halving: a non-root's parent is replaced by its
// grandparent.  Only non-roots are written and every value written is an
// ancestor (a smaller index), so the racy writes never undo a hook.
__device__ __forceinline__ int find_halve(int *L, int i) {
    volatile int *V = L;
    int p = V[i];
    while (p != i) {
        const int g = V[p];
        if (g != p) V[i] = g;
        i = p;
        p = g == p ? p : V[i];
    }
    return i;
}

__device__ __forceinline__ void unite(int *L, int a, int b) {
    for (;;) {
        a = find_halve(L, a);
        b = find_halve(L, b);
        if (a == b) return;
        if (a < b) { const int t = a; a = b; b = t; }
        const int old = atomicCAS(&L[a], a, b);
        if (old == a) return;
        a = old;
    }
}

}  // namespace uf
