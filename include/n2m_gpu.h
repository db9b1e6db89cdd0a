/* n2m_gpu.h — C ABI of the GB300 volume->mesh path (libn2m_gpu.so).
 *
 * Two layers:
 *  1. Drop-in entry points with the reference's exact signatures and semantics
 *     (same names, argument meaning, 0/1 return codes, malloc'd outputs the
 *     caller frees with free()).  Link libn2m_gpu.so instead of meshify.o /
 *     quadric.o / MarchingCubes.o / bwlabel.o / isolevel.o.
 *  2. n2m_* entry points: explicit status codes, a context (CUDA stream +
 *     workspace), device-resident variants, the adjoint and the batched atlas.
 *
 * All compute runs on the GPU; there is no CPU fallback.  If no CUDA device is
 * usable every entry point fails with N2M_ERR_NO_DEVICE (drop-in calls return
 * EXIT_FAILURE and print the reason).
 */
#ifndef N2M_GPU_H
#define N2M_GPU_H

#include <stdbool.h>
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#ifndef MESHIFY_TYPES_H
#define MESHIFY_TYPES_H
/* Same layout as the reference's mesh types (src/meshtypes.h:4-10). */
typedef struct { double x, y, z; } vec3d;
typedef struct { int x, y, z; } vec3i;
#endif

typedef enum {
    N2M_OK = 0,
    N2M_ERR_NO_DEVICE = 1,      /* no usable CUDA device / extension not loaded */
    N2M_ERR_CUDA = 2,           /* a CUDA runtime call failed (see n2m_last_error) */
    N2M_ERR_OOM = 3,            /* device or host allocation failed */
    N2M_ERR_BAD_ARGS = 4,       /* null pointer, bad dims, unsupported option */
    N2M_ERR_NO_VARIABILITY = 5, /* min == max after pre-smooth (src/meshify.c:312) */
    N2M_ERR_EMPTY = 6,          /* marching cubes found < 3 vertices or no triangle */
    N2M_ERR_NONFINITE = 7,      /* NaN/Inf in the volume entering the mesher */
    N2M_ERR_TOO_LARGE = 8,      /* counts exceed the 32-bit index range of vec3i */
    N2M_ERR_TIMEOUT = 9,        /* a bounded device-side wait gave up */
    N2M_ERR_INTERNAL = 10
} n2m_status;

/* cube variants: the reference selects these with -o and the
 * USE_CLASSIC_CUBES build flag (src/meshify.c:25-29). */
typedef enum { N2M_CUBES_MC33 = 0, N2M_CUBES_CLASSIC_TABLE = 1, N2M_CUBES_OLDCUBES = 2 } n2m_cubes;

typedef struct n2m_context n2m_context;

typedef struct {
    int cubes;          /* n2m_cubes */
    float isolevel;
    bool pre_smooth;    /* -p */
    bool only_largest;  /* -l */
    bool fill_bubbles;  /* -b */
    int post_smooth;    /* -s: HC iterations (alpha 0.1, beta 0.5, edges locked) */
    bool verbose;       /* per-stage CUDA-event timings on stdout */
} n2m_options;

/* Per-call report (optional out-parameter). */
typedef struct {
    float isolevel_used;     /* after the out-of-range fallback */
    float vmin, vmax;        /* range of the (smoothed) volume */
    int lo[3], hi[3];        /* padded bounding box handed to marching cubes */
    int64_t nvert_raw, ntri_raw;  /* before weld / degenerate removal */
    int64_t nvert, ntri;     /* final */
    int welded;              /* vertices merged by the weld */
    int degenerate;          /* triangles removed */
    float ms_total;          /* device time of the call (CUDA events) */
    /* device time per stage (CUDA events on the context stream):
     * [0] pre-smooth kernel (or the range pass), [1] clustering + range/bbox,
     * [2] marching-cubes count pass + scan, [3] emit pass, [4] weld,
     * [5] degenerate removal, [6] HC post-smoothing, [7] host-memory calls
     * only: the mesh's way into the caller's memory after the device work
     * (waiting for the output pages, device-to-host copy; host clock) */
    float ms_stage[8];
    int64_t kernel_launches; /* kernels this call launched */
    float ms_smooth_pass_a;  /* device time of the fused approximate pre-smooth kernel of the
                              * exact-on-demand path (inside ms_stage[0]); 0 when the exact
                              * three passes ran */
} n2m_report;

/* ---- context ------------------------------------------------------------ */
/* A context owns a CUDA stream and a grow-only device workspace.  Contexts are
 * independent; one context must not be used by two threads at once.  The
 * drop-in entry points use a per-thread default context. */
n2m_status n2m_context_create(n2m_context **ctx, int device);
void n2m_context_destroy(n2m_context *ctx);
void *n2m_context_stream(n2m_context *ctx);          /* cudaStream_t */
const char *n2m_last_error(void);                    /* per-thread message */
const char *n2m_status_string(int status);
int n2m_device_count(void);
long long n2m_kernel_launches(void);                 /* process-wide kernel launch counter */

/* ---- drop-in entry points ------------------------------------------------ */
/* replaces meshify() (src/meshify.h:9).  originalMC: 0 = Lewiner MC33,
 * 1 = classic case table in the Lewiner framework.  `img` is read only (the
 * reference smooths it in place; no caller reads it afterwards,
 * src/nii2mesh.c:573,589).  *t and *p are malloc'd; free() them. */
int meshify(float *img, short dim[3], int originalMC, float isolevel, vec3i **t, vec3d **p, int *nt, int *np,
            bool preSmooth, bool onlyLargest, bool fillBubbles, bool verbose);
/* replaces laplacian_smoothHC() (src/quadric.h:7); verts updated in place. */
void laplacian_smoothHC(vec3d *verts, vec3i *tris, int nvert, int ntri, double alpha, double beta, int iter,
                        bool lockEdges);
/* replaces marchingCubes() (src/MarchingCubes.h:19 / src/oldcubes.h:9). */
int marchingCubes(float *img, short dim[3], int lo[3], int hi[3], int originalMC, float isolevel, vec3d **vs,
                  vec3i **ts, int *nv, int *nt);
/* replaces bwlabel() (src/bwlabel.h:10) for conn 6/18/26; img overwritten. */
int bwlabel(float *img, int conn, size_t dim[3], bool onlyLargest, bool fillBubbles);
/* replaces apply_sform() (src/meshify.h:10). */
void apply_sform(vec3i *t, vec3d *p, int nt, int np, float srow_x[4], float srow_y[4], float srow_z[4]);
/* replaces setThreshold() (src/isolevel.h:7, body src/isolevel.c:245-277):
 * Otsu isolevel on the robust (2nd-98th percentile) range; mode 1 dark,
 * 2 medium, 3 bright.  img is a host array of nvox floats. */
float setThreshold(float *img, int nvox, int darkMediumBright123);
/* replaces save_mesh() (src/meshify.h:8, body src/meshify.c:984-1019): the
 * format follows the file name's extension as in the reference (.mz3, .gii,
 * .inflated/.pial FreeSurfer, .json, .off, .obj, .ply, .stl, .vtk; any other
 * name gets ".mz3" appended); isGz writes mz3 as gzip and GIfTI arrays
 * zlib-compressed.  The file is encoded on the GPU.  Returns EXIT_SUCCESS or
 * EXIT_FAILURE (file not writable, no device). */
int save_mesh(const char *fnm, vec3i *tris, vec3d *pts, int ntri, int npt, bool isGz);
/* The rest of meshify.h (src/meshify.h:7-11), so that the reference's program
 * links without meshify.o: strip_ext() cuts a file name at its extension in
 * place (src/meshify.c:973-982), clockMsec() is a monotonic clock in
 * milliseconds and timediff() the rounded difference of two of its readings
 * (src/meshify.c:266-284). */
void strip_ext(char *fname);
double clockMsec(void);
long timediff(double startTimeMsec, double endTimeMsec);
/* Mirrors the USE_CLASSIC_CUBES build flag for the drop-in marchingCubes()
 * and meshify(): nonzero selects Bourke's oldcubes. Returns the old value. */
int n2m_set_oldcubes(int enable);

/* ---- explicit-status API -------------------------------------------------- */
/* Host buffers in/out; meshes malloc'd like meshify(). */
n2m_status n2m_meshify(n2m_context *ctx, const float *img, const int dim[3], const n2m_options *opt, vec3i **t,
                       vec3d **p, int *nt, int *np, n2m_report *rep);

/* n2m_meshify into caller-owned host buffers (t: t_cap triangles, p: p_cap
 * vertices; pinned memory copies fastest): no allocation and no page faulting
 * per call, for callers that mesh many volumes.  *nt and *np get the mesh's
 * counts; when it does not fit the call fails with N2M_ERR_TOO_LARGE and *nt,
 * *np say how much room it needs. */
n2m_status n2m_meshify_into(n2m_context *ctx, const float *img, const int dim[3], const n2m_options *opt, vec3i *t,
                            int64_t t_cap, vec3d *p, int64_t p_cap, int *nt, int *np, n2m_report *rep);

/* Device-resident variant: d_img is a device pointer (float32, x fastest).
 * The mesh stays in context-owned device memory (valid until the next call on
 * ctx): *d_t (vec3i[*nt]) and *d_p (vec3d[*np]). */
n2m_status n2m_meshify_device(n2m_context *ctx, const float *d_img, const int dim[3], const n2m_options *opt,
                              vec3i **d_t, vec3d **d_p, int *nt, int *np, n2m_report *rep);

/* Adjoint (no counterpart in the reference; the spec differentiation
 * path).  After an n2m_meshify_device / n2m_meshify call on ctx with Lewiner
 * cubes and no clustering (only_largest = fill_bubbles = false), maps
 * dL/d(vertex) (device float32, np x 3, the mesh of that call) to dL/d(voxel)
 * (device float32, one per input voxel) for the fixed topology of that call:
 * through the HC post-smoothing iterations (recomputed adjoint recursion),
 * the weld, the edge interpolation u = c0/(c0-c1) and c-vertex means, and the
 * transposed pre-smooth stencil.  Values clamped to FLT_EPSILON, padding and
 * darkened edge voxels are constants of the forward pass (zero gradient).  If
 * pre_smooth was false the forward's input buffer must still be valid. */
n2m_status n2m_meshify_backward(n2m_context *ctx, const float *d_grad_pts, float *d_grad_img);

/* ---- atlas (src/nii2mesh.c:492-583) ---------------------------------------------
 * Meshes every label 1..max of a label volume as its own binary mask (the
 * reference's `lo < v < hi` window around each integer label) at isolevel
 * 0.5, with opt's pre-smooth / largest-cluster / bubble-fill / post-smooth
 * options (opt->isolevel is ignored).  N2M_ATLAS_BATCHED runs all labels
 * together on per-label sub-boxes (one launch per stage over a shared work
 * queue); N2M_ATLAS_LOOP runs the full single-volume pipeline once per label.
 * Both give the same meshes.  Labels without voxels are skipped, as in the
 * reference.  Results are concatenated; triangle indices are local to their
 * mesh. */
typedef enum { N2M_ATLAS_BATCHED = 0, N2M_ATLAS_LOOP = 1 } n2m_atlas_mode;
typedef struct {
    int label;
    int status;                      /* N2M_OK, or why this label has no mesh */
    int nvert, ntri;
    int64_t vert_offset, tri_offset; /* into the concatenated vertex / triangle arrays */
} n2m_atlas_mesh;
/* d_labels: device int16 volume (x fastest).  Meshes stay in context-owned
 * device memory until the next call on ctx; *meshes points into the context. */
n2m_status n2m_atlas_device(n2m_context *ctx, const int16_t *d_labels, const int dim[3], const n2m_options *opt,
                            int mode, int *nmesh, const n2m_atlas_mesh **meshes, vec3d **d_pts, vec3i **d_tris,
                            int64_t *npts, int64_t *ntris, n2m_report *rep);
/* Host volume in; everything malloc'd (free() each array). */
n2m_status n2m_atlas(n2m_context *ctx, const int16_t *labels, const int dim[3], const n2m_options *opt, int mode,
                     int *nmesh, n2m_atlas_mesh **meshes, vec3d **pts, vec3i **tris, int64_t *npts, int64_t *ntris);

/* NIfTI voxel types that load_nii() casts to float (src/nii2mesh.c:114-175). */
enum { N2M_DT_UINT8 = 2, N2M_DT_INT16 = 4, N2M_DT_FLOAT32 = 16, N2M_DT_UINT16 = 512 };
/* Device cast of raw NIfTI voxels, out[i] = raw[i] * scl_slope + scl_inter
 * (scl_slope 0 means 1), as load_nii() does on the host (src/nii2mesh.c:160-175). */
n2m_status n2m_cast_voxels_device(n2m_context *ctx, const void *d_raw, int datatype, float scl_slope, float scl_inter,
                                  int64_t nvox, float *d_out);
/* n2m_meshify on raw NIfTI voxels in host memory: the voxels are sent as
 * they are (1, 2 or 4 bytes each) and cast on the device. */
n2m_status n2m_meshify_typed(n2m_context *ctx, const void *img, int datatype, float scl_slope, float scl_inter,
                             const int dim[3], const n2m_options *opt, vec3i **t, vec3d **p, int *nt, int *np,
                             n2m_report *rep);

/* Otsu isolevel of setThreshold() (src/isolevel.c:245-277) with an explicit
 * status: img is a host array (n2m_set_threshold) or a device array
 * (n2m_set_threshold_device) of nvox floats; the value goes to *iso. */
n2m_status n2m_set_threshold(n2m_context *ctx, const float *img, int64_t nvox, int mode, float *iso);
n2m_status n2m_set_threshold_device(n2m_context *ctx, const float *d_img, int64_t nvox, int mode, float *iso);

/* ---- mesh writers (save_mesh, src/meshify.c:602-1019) -------------------------- */
typedef enum {
    N2M_FMT_MZ3 = 0,        /* .mz3 (gzip when is_gz) */
    N2M_FMT_GII = 1,        /* .gii: base64 arrays (zlib + base64 when is_gz) */
    N2M_FMT_FREESURFER = 2, /* .inflated / .pial */
    N2M_FMT_JSON = 3,
    N2M_FMT_OFF = 4,
    N2M_FMT_OBJ = 5,
    N2M_FMT_PLY = 6,
    N2M_FMT_STL = 7,
    N2M_FMT_VTK = 8
} n2m_mesh_format;
/* The format save_mesh() picks for a file name; -1 when it appends ".mz3". */
int n2m_mesh_format_of(const char *fnm);
/* The bytes save_mesh() writes for `format`, in malloc'd memory (*out, *out_len;
 * release with free()).  Host mesh (n2m_encode_mesh) or device mesh
 * (n2m_encode_mesh_device, e.g. the result of n2m_meshify_device).  The
 * FreeSurfer format embeds the current local time like the reference. */
n2m_status n2m_encode_mesh(n2m_context *ctx, int format, const vec3i *tris, const vec3d *pts, int ntri, int npt,
                           int is_gz, unsigned char **out, size_t *out_len);
n2m_status n2m_encode_mesh_device(n2m_context *ctx, int format, const vec3i *d_tris, const vec3d *d_pts, int ntri,
                                  int npt, int is_gz, unsigned char **out, size_t *out_len);
/* The same bytes left in context-owned device memory (*d_out, valid until the
 * next call on ctx), for callers that send them on from the GPU. */
n2m_status n2m_encode_mesh_to_device(n2m_context *ctx, int format, const vec3i *d_tris, const vec3d *d_pts, int ntri,
                                     int npt, int is_gz, const unsigned char **d_out, size_t *out_len);
/* save_mesh() with a status: host mesh, or a mesh already in device memory. */
n2m_status n2m_save_mesh(n2m_context *ctx, const char *fnm, const vec3i *tris, const vec3d *pts, int ntri, int npt,
                         int is_gz);
n2m_status n2m_save_mesh_device(n2m_context *ctx, const char *fnm, const vec3i *d_tris, const vec3d *d_pts, int ntri,
                                int npt, int is_gz);
/* Deflate nbytes of device memory (< 2^31) as a raw deflate stream, a zlib
 * stream or a gzip file body into malloc'd memory (*out, *out_len). */
#define N2M_DEFLATE_RAW 0
#define N2M_DEFLATE_ZLIB 1
#define N2M_DEFLATE_GZIP 2
n2m_status n2m_deflate_device(n2m_context *ctx, const void *d_src, size_t nbytes, int container, unsigned char **out,
                              size_t *out_len);

/* HC smoothing of device-resident meshes (d_verts updated in place).  A
 * triangle index outside [0, nvert) makes the call fail with N2M_ERR_BAD_ARGS
 * and leaves d_verts unchanged (the kernels skip such triangles, so nothing is
 * read or written out of bounds). */
n2m_status n2m_smooth_hc_device(n2m_context *ctx, vec3d *d_verts, const vec3i *d_tris, int nvert, int ntri,
                                double alpha, double beta, int iter, bool lock_edges);

/* ---- allocation-free entry point -----------------------------------------------
 * No counterpart in the reference.  HC smoothing (same semantics as
 * n2m_smooth_hc_device) for callers that cannot call cudaMalloc: code inside
 * another framework's captured or allocation-controlled region, or programs
 * whose device memory all comes from their own pool.  All scratch lives in one
 * fixed device array inside the library (about 11 MB, held by every GPU that
 * loads the library until the process exits), so meshes are limited to
 * N2M_NOALLOC_MAX_VERTS vertices and N2M_NOALLOC_MAX_TRIS triangles; larger
 * meshes fail with N2M_ERR_TOO_LARGE before any work is queued.  d_verts and
 * d_tris are device pointers; the work runs on `stream` (a cudaStream_t,
 * NULL = legacy default stream) and the call returns once it has finished: it
 * reads back a 4-byte flag into host stack memory, and a triangle index
 * outside [0, nvert) fails with N2M_ERR_BAD_ARGS with d_verts unchanged.
 * Each call looks up the array's device address on the current device (this
 * allocates nothing); the first call on a device may load the library's
 * device code, so make it before any stream capture.  Every call shares the
 * one array: calls whose work overlaps on the GPU race and corrupt each
 * other's results. */
#define N2M_NOALLOC_MAX_VERTS 131072
#define N2M_NOALLOC_MAX_TRIS 262144
n2m_status n2m_smooth_hc_noalloc(vec3d *d_verts, const vec3i *d_tris, int nvert, int ntri, double alpha,
                                 double beta, int iter, bool lock_edges, void *stream);

/* ---- test hook -------------------------------------------------------------------
 * Host-side fault injection: the after-th device buffer allocation from now on
 * (0 = the next one) fails with N2M_ERR_OOM, once; a negative value disarms.
 * Returns the previous setting.  Every entry point must then fail cleanly and
 * the context stay usable. */
int n2m_debug_fail_allocations(int after);

#ifdef __cplusplus
}
#endif
#endif /* N2M_GPU_H */
