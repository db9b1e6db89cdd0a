/* n2m_oracle.h — CPU restatement of nii2mesh's volume->mesh path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker the parity tests,
 * smoke() and bench.py's CPU-baseline leg compare the CUDA path against.  No
 * product code links or calls it.  Every function restates one reference
 * function (cited file:line, paths relative to the nii2mesh project) in plain
 * single-threaded C, with the same floating-point operation order.  It must be
 * compiled with -ffp-contract=off -fsigned-char so that aarch64 hosts produce
 * the same bits as x86-64 (gcc contracts a*b+c into FMAs on aarch64, and
 * `char` is unsigned there).
 *
 * Parity pin: the oracle is checked against the reference itself compiled
 * from its own sources (oracle/_ref, built by oracle/build_ref.sh) and against
 * golden fixtures the reference produced (tests/golden/).
 */
#ifndef N2M_ORACLE_H
#define N2M_ORACLE_H
#include <stdbool.h>
#include <stddef.h>

typedef struct { double x, y, z; } or_vec3d;   /* src/meshtypes.h:4-6  */
typedef struct { int x, y, z; } or_vec3i;      /* src/meshtypes.h:8-10 */

/* cube variants: 0 = Lewiner MC33, 1 = Lewiner framework with the classic
 * case table (-o 1), 2 = Bourke oldcubes (the USE_CLASSIC_CUBES build). */
enum { OR_MC33 = 0, OR_MC_CLASSIC_TABLE = 1, OR_OLDCUBES = 2 };

int or_quick_smooth(float *img, int nx, int ny, int nz);
int or_bwlabel(float *img, int conn, const size_t dim[3], bool onlyLargest, bool fillBubbles);
void or_dilate26(float *img, const size_t dim[3]);

/* Stages of meshify() before marching cubes (src/meshify.c:286-371): smooth,
 * range/iso fallback, clustering, edge darken, bbox.  img is modified in
 * place exactly as the reference modifies it.  Returns 0 on success. */
int or_prepare_volume(float *img, const short dim[3], float *isolevel, bool preSmooth,
                      bool onlyLargest, bool fillBubbles, int lo[3], int hi[3], float *mn_out);

int or_marching_cubes(float *img, const short dim[3], const int lo[3], const int hi[3], int variant,
                      float isolevel, or_vec3d **vs, or_vec3i **ts, int *nv, int *nt);
int or_marching_cubes_sources(float *img, const short dim[3], const int lo[3], const int hi[3], int originalMC,
                              float isolevel, or_vec3d **vs, or_vec3i **ts, int *nv, int *nt, int **src);
/* Raw Lewiner run() on an already iso-subtracted grid (the MC self-test,
 * src/MarchingCubes.c:1374-1405): vertices in grid coordinates (float). */
int or_mc_raw(const float *data, int nx, int ny, int nz, int originalMC, float **verts, int **tris,
              int *nv, int *nt);
int or_unify_vertices(or_vec3d **pts, or_vec3i *tris, int npt, int ntri);
int or_remove_degenerate_triangles(or_vec3d *pts, or_vec3i **tris, int ntri);
int or_meshify(float *img, const short dim[3], int variant, float isolevel, or_vec3i **t, or_vec3d **p,
               int *nt, int *np, bool preSmooth, bool onlyLargest, bool fillBubbles);
void or_laplacian_smoothHC(or_vec3d *verts, const or_vec3i *tris, int nvert, int ntri, double alpha,
                           double beta, int iter, bool lockEdges);
void or_laplacian_smooth(or_vec3d *verts, const or_vec3i *tris, int nvert, int ntri);
void or_border_vertices(const or_vec3i *tris, int nvert, int ntri, unsigned char *border);
void or_apply_sform(or_vec3i *t, or_vec3d *p, int nt, int np, const float srow_x[4],
                    const float srow_y[4], const float srow_z[4]);
float or_set_threshold(const float *img, int nvox, int darkMediumBright123);
/* One atlas label (src/nii2mesh.c:550-571): binarize label `label` of `img`
 * into `out` (0/1 floats), returns the voxel count. */
int or_binarize_label(const float *img, int nvox, int label, float *out);
/* The analytic self-test fields (src/MarchingCubes.c:1282-1361) on 60^3. */
int or_selftest_field(int obj, float *out);
void or_free(void *p);

#endif
