// n2m_internal.cuh — shared declarations of the CUDA implementation.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>

#include <atomic>
#include <string>
#include <vector>

#include "../../include/n2m_gpu.h"

#define N2M_FLT_EPS 1.19209290e-07f

// ---- error plumbing ---------------------------------------------------------
void n2m_set_error(const char *fmt, ...);
#define CK(call)                                                                          \
    do {                                                                                  \
        cudaError_t e_ = (call);                                                          \
        if (e_ != cudaSuccess) {                                                          \
            n2m_set_error("%s:%d %s: %s", __FILE__, __LINE__, #call, cudaGetErrorString(e_)); \
            return e_ == cudaErrorMemoryAllocation ? N2M_ERR_OOM : N2M_ERR_CUDA;          \
        }                                                                                 \
    } while (0)
#define CKS(st)                                   \
    do {                                          \
        n2m_status s_ = (st);                     \
        if (s_ != N2M_OK) return s_;              \
    } while (0)
#define CKL()  CK(cudaGetLastError())

// process-wide count of kernel launches (reported by n2m_kernel_launches)
extern std::atomic<long long> g_n2m_launches;
#define N2M_COUNT() g_n2m_launches.fetch_add(1, std::memory_order_relaxed)

// ---- grow-only device buffers -----------------------------------------------
struct DevBuf {
    void *p = nullptr;
    size_t cap = 0;
    n2m_status ensure(size_t bytes);
    void release();
    template <class T> T *as() const { return reinterpret_cast<T *>(p); }
};

// ---- ordered-int encoding of floats for atomicMin/atomicMax ------------------
__device__ __forceinline__ int f2ord(float f) {
    int i = __float_as_int(f);
    return i >= 0 ? i : i ^ 0x7fffffff;
}
inline int f2ord_host(float f) {
    int i;
    memcpy(&i, &f, 4);
    return i >= 0 ? i : i ^ 0x7fffffff;
}
__host__ __device__ __forceinline__ float ord2f(int i) {
    int j = i >= 0 ? i : i ^ 0x7fffffff;
#ifdef __CUDA_ARCH__
    return __int_as_float(j);
#else
    float f;
    memcpy(&f, &j, 4);
    return f;
#endif
}

// Reductions produced by the volume passes (device-resident, read back once).
struct VolStats {
    int vmin, vmax;          // ordered-int min/max of the volume
    int lo[3], hi[3];        // bbox of voxels >= iso (unpadded, inclusive)
    unsigned nonfinite;      // NaN/Inf voxels
    unsigned masked;         // voxels the labelling set to the minimum (run_labelling)
};

// ---- kernels' host launchers (stream-ordered, no syncs) ----------------------
// smooth.cu
// A host volume copied to `in` slab by slab on the `copy` stream while the
// x pass of the slabs already copied runs (the three-pass path only).
constexpr int N2M_STAGE_SLABS = 16;
struct StagedInput {
    const float *host = nullptr;
    cudaStream_t copy = nullptr;
    cudaEvent_t ev[N2M_STAGE_SLABS + 1] = {};
};
// tmp: one volume of scratch; stage: see StagedInput (may be null)
n2m_status launch_smooth(const float *in, float *out, float *tmp, int nx, int ny, int nz, float iso, VolStats *st,
                         cudaStream_t s, const StagedInput *stage = nullptr);
// whether launch_smooth can take a StagedInput for this volume
bool smooth_can_stage(int nx, int ny, int nz);

// Pre-smooth with exact rounding on demand (smooth.cu): od_approx smooths the
// whole volume approximately (one fused FP32 pass, rigorous error bound) and
// lists the voxels whose sign against iso it cannot decide and the candidates
// for the volume's range; od_resolve gives those their exact values and fills
// `dst` (exact range, bbox, no non-finite count) unless *fallback (a
// non-finite or huge input, a list overflow): then the caller runs
// launch_smooth instead.  Marching cubes marks the corners of the cubes the
// surface crosses in need_z (mc.cu: mc_count with an OdRepair), and od_repair
// writes the reference's exact value at every marked voxel of `out`.
enum : unsigned { OD_FALLBACK = 1u, OD_TIMEOUT = 2u };
struct OdStats {
    VolStats vs;             // bbox of decided voxels >= iso; exact range after od_resolve
    unsigned flags;
    unsigned cnt[3];         // undecided, min candidates, max candidates
    int umin, lmax;          // ordered: smallest task min + B, largest task max - B
};
struct OdCand {              // a range candidate: voxel, approximate value, its bound
    unsigned j;
    float v, b;
};
struct OdLists {
    unsigned *unc;
    OdCand *cmin, *cmax;
    unsigned *cnt;
    unsigned cap;
    unsigned *vsign;         // sign bitmap of the smoothed volume (see OdWork)
    unsigned wv, nys;        // its words per row, groups of 8 rows per slice
};
struct OdWork {
    DevBuf st, unc, cmin, cmax, need_z, need_y, need_x, off, list, lcnt;
    // bit x & 31 of word od_vsign_word(x, y, z): the smoothed value of voxel (x, y, z)
    // minus iso is above -FLT_EPSILON (Lewiner's sign before edge darkening), or with
    // od_resolve's at_or_above, the value is >= iso (the complement of oldcubes'
    // sign); exact for every voxel once od_resolve has run
    DevBuf vsign;
    unsigned cap = 0;
};
struct ScanWork;
// What meshify's labelling did to each voxel (src/meshify.c:330-342), for the
// exact values the repair writes afterwards: voxels of K (bit x & 31 of word
// (z*ny + y)*W + x/32) are raised to iso when fill; with largest, voxels
// neither in K nor in its dilation are the minimum mn.
struct LabelPost {
    const unsigned *K;
    unsigned W;
    float mn, iso;
    bool fill, largest;
};
struct OdRepair {
    const float *in;         // the raw volume
    float *tmp1, *tmp2;      // exact x and y pass values (written at marked voxels only)
    float *out;              // the approximately smoothed volume, exact where marked
    int dim[3];
    OdWork *w;
    ScanWork *scan;
    const LabelPost *post = nullptr;   // the volume was labelled: the repaired values get the same treatment
};
// the sign bitmap's word of voxel (x, y, z): the 8 row words of one 32 x 8 tile of a
// slice are adjacent (one 32-byte sector, written at once by pass A)
__host__ __device__ __forceinline__ size_t od_vsign_word(unsigned x, unsigned y, unsigned z, unsigned wv, unsigned nys) {
    return (((size_t)z * nys + (y >> 3)) * wv + (x >> 5)) * 8u + (y & 7u);
}
// marks the voxels j .. j+31 whose bits are set in a linear bitmap over nvox voxels
__device__ __forceinline__ void od_need_mark(unsigned *need, long long j, unsigned bits, long long nvox) {
    if (j >= nvox || !bits) return;
    if (nvox - j < 32) bits &= (1u << (unsigned)(nvox - j)) - 1u;
    const long long w = j >> 5;
    const int sh = (int)(j & 31);
    const unsigned p0 = bits << sh, p1 = sh ? bits >> (32 - sh) : 0u;
    if (p0) atomicOr(need + w, p0);
    if (p1) atomicOr(need + w + 1, p1);
}
// whether the on-demand path applies: rows a multiple of 16 bytes (TMA tiles), fewer than 2^32 voxels
bool od_eligible(const float *in, int nx, int ny, int nz);
n2m_status od_approx(const float *in, float *out, int nx, int ny, int nz, float iso, OdWork &w, cudaStream_t s,
                     const StagedInput *stage = nullptr);
n2m_status od_resolve(const float *in, float *out, int nx, int ny, int nz, float iso, OdWork &w, VolStats *dst,
                      cudaStream_t s, bool *fallback, bool at_or_above = false);
n2m_status od_repair(const OdRepair &r, cudaStream_t s);
// transposed pre-smooth: g_img = Sx^T Sy^T Sz^T g (tmp: one volume of scratch)
n2m_status launch_smooth_adjoint(const float *g, float *tmp, float *out, int nx, int ny, int nz, cudaStream_t s);
n2m_status launch_stats(const float *vol, int nx, int ny, int nz, float iso, bool minmax, VolStats *st,
                        cudaStream_t s);
void stats_init_host(VolStats *h);

// scan.cu: exclusive scan of uint4 (component-wise) in place; total -> *d_total
struct ScanWork {
    DevBuf part;
};
n2m_status scan_uint4(uint4 *d, size_t n, uint4 *d_total, ScanWork &w, cudaStream_t s);
n2m_status scan_u32(unsigned *d, size_t n, unsigned *d_total, ScanWork &w, cudaStream_t s);

// label.cu
struct LabelWork {
    DevBuf lab, mask, keep, cnt, edge, rc, misc;
};
// meshify's labelling of vol in place; st: the range and bbox of the result
// (accumulated into, like launch_stats) and the count of masked voxels.
// vsign (may be null): a sign bitmap (OdWork::vsign with od_resolve's
// at_or_above) to take the mask from instead of vol; post (may be null): what
// the labelling did, for values computed later
n2m_status run_labelling(float *vol, int nx, int ny, int nz, float iso, float mn, bool only_largest,
                         bool fill_bubbles, LabelWork &w, VolStats *st, cudaStream_t s, const unsigned *vsign = nullptr,
                         LabelPost *post = nullptr);
// bwlabel() semantics on a float volume (nonzero = foreground); *d_nl gets the label count
n2m_status run_bwlabel(float *vol, int nx, int ny, int nz, int conn, bool only_largest, bool fill_bubbles,
                       LabelWork &w, ScanWork &sw, int *d_nl, cudaStream_t s);

// decode.cu: NIfTI voxel cast (bytes per voxel 0 = unsupported datatype)
int nifti_bytes_per_voxel(int datatype);
n2m_status launch_cast(const void *d_raw, int datatype, float slope, float inter, long long n, float *d_out,
                       cudaStream_t s);

// deflate.cu: gzip / zlib / raw deflate of n bytes at d_src (4-byte aligned, n + 8
// readable bytes); the stream goes to w.out, its length to *out_len (synchronizes
// once to size the output).  deflate_check reads back the emitter's self-check.
struct DeflateWork {
    DevBuf tok, info, hist, codes, hdr, sizes, misc, out;
    int lz_slots = 0;                                       // chunks the match finder keeps in flight
    int huff_slots = 0;                                     // warps the code builder keeps in flight
    void *side = nullptr, *ev_in = nullptr, *ev_ck = nullptr;   // checksum stream and its events
};
size_t deflate_bound(size_t n);
void deflate_release(DeflateWork &w);
n2m_status deflate_device(const void *d_src, size_t n, int container, DeflateWork &w, ScanWork &sw, cudaStream_t s,
                          size_t *out_len);
n2m_status deflate_check(DeflateWork &w, cudaStream_t s);

// writers.cu: the bytes save_mesh() writes, assembled in device memory
struct WriterWork {
    DevBuf mt, mp, pack, pack2, lens, flag, out;
    DeflateWork df;
    void *host = nullptr;   // pinned staging for file writes
    size_t host_cap = 0;
};
int mesh_format_of(const char *fnm);   // N2M_FMT_*, or -1 (save_mesh appends ".mz3")
const char *file_ext(const char *fnm);  // where strip_ext cuts the name
n2m_status encode_mesh_device(int format, const vec3i *d_t, const vec3d *d_p, int nt, int np, bool gz, WriterWork &w,
                              ScanWork &sw, cudaStream_t s, const unsigned char **d_out, size_t *len);

// isolevel.cu: setThreshold (Otsu on the robust range) of a device volume
struct ThresholdWork {
    DevBuf buf, table;
    std::vector<double> P;
};
n2m_status isolevel_otsu(const float *d_img, long long nvox, int mode123, ThresholdWork &w, cudaStream_t s,
                         float *result);

// mc.cu
struct McGrid {
    const float *vol;        // processed volume (before edge darkening)
    int dim[3];              // volume dims
    int lo[3];               // grid origin in the volume
    int n[3];                // grid size (NX, NY, NZ)
    float iso, edge_max, pad_val;   // pad_val = float(min' - iso)
};
struct McWork {
    DevBuf words, counts, cand, verts_tmp, tris_tmp, signs, ctr;
};
struct McCounts {
    unsigned nv_edge, nt, nc, nactive;
};
// repair: marks the corners of the cubes with mixed signs in repair->w->need_z
// after the sign pass and runs od_repair before any value is read (null: none)
// (with a repair and no labelling, the sign words of grid points strictly inside
// the volume come from repair->w->vsign instead of the values)
n2m_status mc_count(const McGrid &g, int variant, McWork &w, ScanWork &sw, uint4 *d_total, cudaStream_t s,
                    const OdRepair *repair = nullptr);
n2m_status mc_emit(const McGrid &g, int variant, McWork &w, const McCounts &c, vec3d *d_pts, vec3i *d_tris,
                   int *d_cand, unsigned *d_ncand, int cand_cap, cudaStream_t s);
n2m_status mc_backward(const McGrid &g, int variant, McWork &w, const McCounts &c, const float3 *d_gv, float *d_gs,
                       cudaStream_t s);
n2m_status mc_ccand_scan(const vec3d *d_pts, int np, const int *d_ccand, int nccand, int *d_cand,
                         unsigned *d_ncand, int cand_cap, cudaStream_t s);

// oldcubes.cu
// repair: as for mc_count (vsign must then hold od_resolve's at_or_above sign)
n2m_status oc_count(const float *vol, const int dim[3], const int lo[3], const int hi[3], float iso, float edge_max,
                    McWork &w, ScanWork &sw, uint4 *d_total, cudaStream_t s, const OdRepair *repair = nullptr);
n2m_status oc_emit(const float *vol, const int dim[3], const int lo[3], const int hi[3], float iso, float edge_max,
                    McWork &w, const McCounts &c, vec3d *d_pts, vec3i *d_tris, int *d_cand, unsigned *d_ncand,
                    int cand_cap, cudaStream_t s);
// the copies of the ncand weld candidates in the reference's triangle soup: every
// corner 3*t + c naming one, into d_out (at most cap; *d_count = how many there
// are); d_bits: nv bits of scratch
n2m_status oc_copies(const vec3i *d_tris, int nt, int nv, const int *d_cand, int ncand, unsigned *d_bits,
                     unsigned *d_out, unsigned *d_count, unsigned cap, cudaStream_t s);
// the vertex id each listed corner names and the position the cube that emitted
// its triangle interpolates for it (needs oc_count's words of the same grid)
n2m_status oc_copy_positions(const float *vol, const int dim[3], const int lo[3], const int hi[3], float iso,
                             float edge_max, const McWork &w, const vec3i *d_tris, const unsigned *d_q, int n, int *d_vid,
                             vec3d *d_pos, cudaStream_t s);

// mesh.cu
n2m_status mesh_apply_weld(vec3d *d_pts, vec3i *d_tris, int np, int nt, const int *d_removed, const int *d_keep,
                           int nrem, const int *d_ov_id, const vec3d *d_ov_pos, int nov, vec3d *d_out,
                           cudaStream_t s);
struct DegWork {
    DevBuf flags, tmp;
};
n2m_status mesh_remove_degenerate(const vec3d *d_pts, const vec3i *d_tris_in, int nt, vec3i *d_tris_out,
                                  unsigned *d_nt_out, DegWork &w, ScanWork &sw, cudaStream_t s);
struct HcWork {
    DevBuf start, refs, fill, P, Q, B, Lo, border, hasnb, bad;
};
// Triangles with an index outside [0, np) are skipped and flagged; the flag
// makes the last kernel leave d_pts unchanged.  mesh_smooth_hc_check waits for
// the stream and returns N2M_ERR_BAD_ARGS when the flag was raised (entry
// points that take the caller's triangles call it; meshify's own meshes are
// valid by construction).
n2m_status mesh_smooth_hc(vec3d *d_pts, const vec3i *d_tris, int np, int nt, double alpha, double beta, int iter,
                          bool lock_edges, HcWork &w, ScanWork &sw, cudaStream_t s);
n2m_status mesh_smooth_hc_check(HcWork &w, int np, int iter, cudaStream_t s);
// adjoint of mesh_smooth_hc (uses the CSR and border flags the forward left in w)
n2m_status mesh_smooth_hc_backward(const vec3i *d_tris, int np, double alpha, double beta, int iter, bool lock_edges,
                                   HcWork &w, const float3 *d_g, float3 *d_go, cudaStream_t s);
// grad of raw (pre-weld) vertices from grad of welded vertices
n2m_status mesh_weld_backward(const float3 *d_go, int np_final, int nv_raw, const int *d_removed, int nrem,
                              const int *d_ov_id, const int *d_ov_src, int nov, float3 *d_graw, cudaStream_t s);
n2m_status mesh_apply_sform(vec3d *d_pts, vec3i *d_tris, int np, int nt, const float sx[4], const float sy[4],
                            const float sz[4], cudaStream_t s);

// atlas.cu
#include <vector>
struct AtlasWork {
    DevBuf cnt, bb, boxes, queue, arena, mask, keep, lab, edge, ucnt, words, counts, active, tot, pts, pts2, tris, tris2,
        cand, gath, weld, ranges;
    void *exec = nullptr;            // cudaGraphExec_t of the smoothing + clustering segment
    bool tuned = false;              // autotuned work-item size and grid width
    unsigned chunk = 1024, per_sm = 8;
    float tuned_ms = 0.f;
};
n2m_status atlas_hist(const short *d_lab, const int dim[3], AtlasWork &w, cudaStream_t s, int *maxlab,
                      std::vector<unsigned> &cnt, std::vector<int> &bb);
n2m_status atlas_binarize(const short *d_lab, long long n, int label, float *out, cudaStream_t s);
n2m_status atlas_offset_tris(vec3i *t, int n, int off, cudaStream_t s);
n2m_status atlas_batched(const short *d_lab, const int dim[3], const n2m_options &o, AtlasWork &w, ScanWork &sw,
                         DegWork &dw, HcWork &hw, cudaStream_t s, std::vector<n2m_atlas_mesh> &out, vec3d **d_pts,
                         vec3i **d_tris, int64_t *npts, int64_t *ntris, float *ms_stage);
