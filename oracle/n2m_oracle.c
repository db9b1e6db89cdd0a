/* n2m_oracle.c — CPU restatement of nii2mesh's volume->mesh path.
 *
 * TEST INFRASTRUCTURE ONLY (see n2m_oracle.h): the checker that the CUDA path
 * is compared against; never linked into the product.  Each function cites the
 * reference function it restates (paths relative to the nii2mesh project).
 * The arithmetic keeps the reference's operation order and precision so that
 * results are bit-identical; compile with -ffp-contract=off -fsigned-char.
 */
#include "n2m_oracle.h"

#include <float.h>
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "../nii2mesh_gb300/csrc/mc_tables.h"

#define LUT1(T, a) ((int)n2m_lut_blob[N2M_##T##_OFF + (a)])
#define LUT2(T, a, b) ((int)n2m_lut_blob[N2M_##T##_OFF + (a)*N2M_##T##_S0 + (b)])
#define LUT3(T, a, b, c) ((int)n2m_lut_blob[N2M_##T##_OFF + (a)*N2M_##T##_S0 + (b)*N2M_##T##_S1 + (c)])
#define PTR2(T, a) (&n2m_lut_blob[N2M_##T##_OFF + (a)*N2M_##T##_S0])
#define PTR3(T, a, b) (&n2m_lut_blob[N2M_##T##_OFF + (a)*N2M_##T##_S0 + (b)*N2M_##T##_S1])

void or_free(void *p) { free(p); }

/* ------------------------------------------------------------------------ */
/* quick_smooth: src/meshify.c:170-216.  Separable 5-tap blur; the taps are
 * double constants so every product and sum is double, rounded to float once
 * per pass.  Voxels within 2 of a face along the pass axis keep their value. */
int or_quick_smooth(float *img, int nx, int ny, int nz) {
    if (nx < 5 || ny < 5 || nz < 5) return 1;
    const double w0 = 0.45, w1 = 0.225, w2 = 0.05;
    size_t nxy = (size_t)nx * ny, n = nxy * nz;
    float *tmp = (float *)malloc(n * sizeof(float));
    memcpy(tmp, img, n * sizeof(float));
    for (int z = 0; z < nz; z++)
        for (int y = 0; y < ny; y++) {
            const float *s = img + (size_t)z * nxy + (size_t)y * nx;
            float *d = tmp + (size_t)z * nxy + (size_t)y * nx;
            for (int x = 2; x < nx - 2; x++)
                d[x] = (float)((s[x - 2] * w2) + (s[x - 1] * w1) + (s[x] * w0) + (s[x + 1] * w1) + (s[x + 2] * w2));
        }
    memcpy(img, tmp, n * sizeof(float));
    for (int z = 0; z < nz; z++)
        for (int y = 2; y < ny - 2; y++)
            for (int x = 0; x < nx; x++) {
                size_t v = (size_t)z * nxy + (size_t)y * nx + x;
                tmp[v] = (float)((img[v - 2 * nx] * w2) + (img[v - nx] * w1) + (img[v] * w0) + (img[v + nx] * w1) +
                                 (img[v + 2 * nx] * w2));
            }
    memcpy(img, tmp, n * sizeof(float));
    for (int z = 2; z < nz - 2; z++)
        for (int y = 0; y < ny; y++)
            for (int x = 0; x < nx; x++) {
                size_t v = (size_t)z * nxy + (size_t)y * nx + x;
                img[v] = (float)((tmp[v - 2 * nxy] * w2) + (tmp[v - nxy] * w1) + (tmp[v] * w0) + (tmp[v + nxy] * w1) +
                                 (tmp[v + 2 * nxy] * w2));
            }
    free(tmp);
    return 0;
}

/* ------------------------------------------------------------------------ */
/* bwlabelCore: src/bwlabel.c:429-477 with do_initial_labelling :154-245,
 * check_previous_slice :94-131, fill_tratab :54-90 and translate_labels
 * :249-277.  Raster-order provisional labels, an equivalence table whose
 * roots always point at the smaller label (root search capped at 100 hops
 * as in the reference), then final labels numbered by first appearance. */
typedef struct { uint32_t *t; size_t n, cap; } eqtab;

static void eq_merge(eqtab *tt, const uint32_t *nb, int nset) {
    uint32_t roots[16], lowest = UINT32_MAX;
    for (int i = 0; i < nset; i++) {
        uint32_t j = nb[i];
        int hops = 0;
        while (tt->t[j - 1] != j) {
            j = tt->t[j - 1];
            if (++hops > 100) { fprintf(stderr, "\nOoh no!!"); break; }
        }
        roots[i] = j;
        if (j < lowest) lowest = j;
    }
    for (int i = 0; i < nset; i++) tt->t[roots[i] - 1] = lowest;
}

static int label_core(float *img, int conn, const size_t dim[3], bool onlyLargest) {
    if (conn != 6 && conn != 18 && conn != 26) return 0;
    if (dim[0] < 2 || dim[1] < 2 || dim[2] < 1) return 0;
    const size_t X = dim[0], Y = dim[1], Z = dim[2], XY = X * Y, n = XY * Z;
    uint32_t *il = (uint32_t *)calloc(n, sizeof(uint32_t));
    eqtab tt = {(uint32_t *)calloc(10000, sizeof(uint32_t)), 0, 10000};
    uint32_t next = 1;
#define IL(x, y, z) il[(size_t)(z)*XY + (size_t)(y)*X + (x)]
    for (size_t z = 0; z < Z; z++)
        for (size_t y = 0; y < Y; y++)
            for (size_t x = 0; x < X; x++) {
                if (img[z * XY + y * X + x] == 0.0f) continue;
                uint32_t nb[16], prev[9], l;
                int nset = 0, np = 0;
                if (z) { /* neighbours in the previous slice */
                    if ((l = IL(x, y, z - 1))) prev[np++] = l;
                    if (conn >= 18) {
                        if (x && (l = IL(x - 1, y, z - 1))) prev[np++] = l;
                        if (y && (l = IL(x, y - 1, z - 1))) prev[np++] = l;
                        if (x < X - 1 && (l = IL(x + 1, y, z - 1))) prev[np++] = l;
                        if (y < Y - 1 && (l = IL(x, y + 1, z - 1))) prev[np++] = l;
                    }
                    if (conn == 26) {
                        if (x && y && (l = IL(x - 1, y - 1, z - 1))) prev[np++] = l;
                        if (x < X - 1 && y && (l = IL(x + 1, y - 1, z - 1))) prev[np++] = l;
                        if (x && y < Y - 1 && (l = IL(x - 1, y + 1, z - 1))) prev[np++] = l;
                        if (x < X - 1 && y < Y - 1 && (l = IL(x + 1, y + 1, z - 1))) prev[np++] = l;
                    }
                    if (np) { eq_merge(&tt, prev, np); nb[nset++] = prev[0]; }
                }
                if (x && (l = IL(x - 1, y, z))) nb[nset++] = l;
                if (y && (l = IL(x, y - 1, z))) nb[nset++] = l;
                if (conn >= 18) {
                    if (y && x && (l = IL(x - 1, y - 1, z))) nb[nset++] = l;
                    if (y && x < X - 1 && (l = IL(x + 1, y - 1, z))) nb[nset++] = l;
                }
                if (nset) {
                    IL(x, y, z) = nb[0];
                    eq_merge(&tt, nb, nset);
                } else {
                    IL(x, y, z) = next;
                    if (next >= tt.cap) {
                        tt.t = (uint32_t *)realloc(tt.t, (tt.cap + 10000) * sizeof(uint32_t));
                        memset(tt.t + tt.cap, 0, 10000 * sizeof(uint32_t));
                        tt.cap += 10000;
                    }
                    tt.t[next - 1] = next;
                    next++;
                }
            }
#undef IL
    uint32_t nprov = next - 1;
    for (uint32_t i = 0; i < nprov; i++) { /* resolve every label to its root */
        uint32_t j = i;
        while (tt.t[j] != j + 1) j = tt.t[j] - 1;
        tt.t[i] = j + 1;
    }
    uint32_t *first = (uint32_t *)calloc(nprov + 1, sizeof(uint32_t));
    uint32_t ncomp = 0;
    uint32_t *lab = il; /* relabel in place: final label by first appearance */
    for (size_t i = 0; i < n; i++) {
        if (!il[i]) continue;
        uint32_t r = tt.t[il[i] - 1];
        if (!first[r]) first[r] = ++ncomp;
        lab[i] = first[r];
    }
    free(first);
    free(tt.t);
    int nl = (int)ncomp;
    if (nl > 0 && onlyLargest) {
        uint32_t *count = (uint32_t *)calloc(ncomp + 1, sizeof(uint32_t));
        for (size_t i = 0; i < n; i++) count[lab[i]]++;
        uint32_t best = 0, bestN = 0;
        for (uint32_t j = 1; j <= ncomp; j++)
            if (count[j] > bestN) { bestN = count[j]; best = j; }
        free(count);
        for (size_t i = 0; i < n; i++) lab[i] = (lab[i] == best);
        nl = 1;
    }
    for (size_t i = 0; i < n; i++) img[i] = (float)lab[i];
    free(il);
    return nl;
}

/* bwlabel: src/bwlabel.c:478-543.  Optional bubble fill (background
 * components under 6-connectivity that touch no face of the volume are set to
 * 1, but only when the background has at least two components), then the
 * labelling of the foreground. */
int or_bwlabel(float *img, int conn, const size_t dim[3], bool onlyLargest, bool fillBubbles) {
    if (!fillBubbles) return label_core(img, conn, dim, onlyLargest);
    const size_t X = dim[0], Y = dim[1], Z = dim[2], XY = X * Y, n = XY * Z;
    float *inv = (float *)malloc(n * sizeof(float));
    for (size_t i = 0; i < n; i++) inv[i] = (img[i] == 0.0f) ? 1.0f : 0.0f;
    int nInv = label_core(inv, 6, dim, false);
    if (nInv <= 1) {
        free(inv);
        return label_core(img, conn, dim, onlyLargest);
    }
    unsigned char *edge = (unsigned char *)calloc((size_t)nInv + 1, 1);
#define MARK(i) edge[(uint32_t)lroundf(inv[(i)])] = 1
    for (size_t z = 0; z < Z; z++)
        for (size_t y = 0; y < Y; y++)
            for (size_t x = 0; x < X; x++)
                if (x == 0 || y == 0 || z == 0 || x == X - 1 || y == Y - 1 || z == Z - 1) MARK(z * XY + y * X + x);
#undef MARK
    for (size_t i = 0; i < n; i++)
        if (!edge[(uint32_t)lroundf(inv[i])]) img[i] = 1.0f;
    free(edge);
    free(inv);
    return label_core(img, conn, dim, onlyLargest);
}

/* dilate(..., is26=true): src/meshify.c:218-264.  Interior voxels become 1 if
 * any of 25 neighbours is > 0: the reference's offset list starts at index 1,
 * so the (-1,-1,-1) neighbour is never examined. */
void or_dilate26(float *img, const size_t dim[3]) {
    const long X = (long)dim[0], Y = (long)dim[1], Z = (long)dim[2], XY = X * Y, n = XY * Z;
    unsigned char *grow = (unsigned char *)calloc((size_t)n, 1);
    long off[26];
    int k = 0;
    for (int dz = -1; dz <= 1; dz++)
        for (int dy = -1; dy <= 1; dy++)
            for (int dx = -1; dx <= 1; dx++)
                if (dx || dy || dz) off[k++] = dx + dy * X + dz * XY;
    for (long z = 1; z < Z - 1; z++)
        for (long y = 1; y < Y - 1; y++)
            for (long x = 1; x < X - 1; x++) {
                long v = z * XY + y * X + x;
                for (int q = 1; q < 26; q++)
                    if (img[v + off[q]] > 0) grow[v] = 1;
            }
    for (long v = 1; v < n; v++)
        if (grow[v]) img[v] = 1.0f;
    free(grow);
}

/* ------------------------------------------------------------------------ */
/* meshify stages before marching cubes: src/meshify.c:294-371. */
int or_prepare_volume(float *img, const short dim[3], float *isolevel, bool preSmooth, bool onlyLargest,
                      bool fillBubbles, int lo[3], int hi[3], float *mn_out) {
    const int NX = dim[0], NY = dim[1], NZ = dim[2];
    const int nvox = NX * NY * NZ;
    float iso = *isolevel;
    if (preSmooth) or_quick_smooth(img, NX, NY, NZ);
    float mx = img[0], mn = img[0];
    for (int i = 0; i < nvox; i++) {
        mx = fmaxf(mx, img[i]);
        mn = fminf(mn, img[i]);
    }
    if (mn == mx) return 1; /* "No variability in image intensity" */
    if (iso <= mn || iso > mx) iso = (float)(0.5 * (mn + mx));
    if (onlyLargest || fillBubbles) {
        float *mask = (float *)calloc((size_t)nvox, sizeof(float));
        size_t d3[3] = {(size_t)NX, (size_t)NY, (size_t)NZ};
        for (int i = 0; i < nvox; i++)
            if (img[i] >= iso) mask[i] = 1;
        or_bwlabel(mask, 18, d3, onlyLargest, fillBubbles);
        if (fillBubbles)
            for (int i = 0; i < nvox; i++)
                if (mask[i] != 0) img[i] = (float)fmax(img[i], iso);
        if (onlyLargest) {
            or_dilate26(mask, d3);
            for (int i = 0; i < nvox; i++)
                if (mask[i] == 0) img[i] = mn;
        }
        free(mask);
    }
    const float edgeMax = (float)(0.75 * (mn + iso));
    lo[0] = NX; lo[1] = NY; lo[2] = NZ;
    hi[0] = hi[1] = hi[2] = 0;
    int v = 0;
    for (int z = 0; z < NZ; z++)
        for (int y = 0; y < NY; y++)
            for (int x = 0; x < NX; x++, v++) {
                if (img[v] >= iso) {
                    if (x < lo[0]) lo[0] = x;
                    if (y < lo[1]) lo[1] = y;
                    if (z < lo[2]) lo[2] = z;
                    if (x > hi[0]) hi[0] = x;
                    if (y > hi[1]) hi[1] = y;
                    if (z > hi[2]) hi[2] = z;
                }
                if (x == 0 || y == 0 || z == 0 || x == NX - 1 || y == NY - 1 || z == NZ - 1)
                    img[v] = fminf(edgeMax, img[v]);
            }
    for (int i = 0; i < 3; i++) {
        lo[i] = lo[i] - 1 > 0 ? lo[i] - 1 : 0;
        hi[i] = hi[i] + 2 < dim[i] ? hi[i] + 2 : dim[i];
    }
    *isolevel = iso;
    if (mn_out) *mn_out = mn;
    return 0;
}

/* ------------------------------------------------------------------------ */
/* Lewiner MC33: src/MarchingCubes.c.  The grid holds value-minus-isolevel. */
typedef struct {
    int nx, ny, nz, original;
    const float *d;
    int *xv, *yv, *zv;           /* vertex id owned by each grid point's +x/+y/+z edge */
    float *vp;                   /* vertex positions (x,y,z), grid coordinates */
    int nv, capv;
    int *tr;                     /* triangles (v1,v2,v3) in emission order */
    int nt, capt;
    int *src;                    /* optional: per vertex (kind, grid index, axis); kind 1 = c-vertex */
    int cur_kind, cur_index, cur_axis;
    int i, j, k, kase, config, subconfig;
    float cube[8];
} mcx;

static inline size_t gi(const mcx *m, int i, int j, int k) {
    return (size_t)i + (size_t)j * m->nx + (size_t)k * m->nx * m->ny;
}

static int push_vertex(mcx *m, float x, float y, float z) {
    if (m->nv >= m->capv) {
        m->capv = m->capv ? 2 * m->capv : 65536;
        m->vp = (float *)realloc(m->vp, (size_t)m->capv * 3 * sizeof(float));
        m->src = (int *)realloc(m->src, (size_t)m->capv * 3 * sizeof(int));
    }
    m->src[3 * m->nv] = m->cur_kind; m->src[3 * m->nv + 1] = m->cur_index; m->src[3 * m->nv + 2] = m->cur_axis;
    m->vp[3 * m->nv] = x; m->vp[3 * m->nv + 1] = y; m->vp[3 * m->nv + 2] = z;
    return m->nv++;
}

/* compute_intersection_points: src/MarchingCubes.c:235-270 with
 * add_{x,y,z}_vertex :935-1026 (normals omitted: never read downstream). */
static void mc_edge_vertices(mcx *m) {
    for (int k = 0; k < m->nz; k++)
        for (int j = 0; j < m->ny; j++)
            for (int i = 0; i < m->nx; i++) {
                float c0 = m->d[gi(m, i, j, k)];
                float c1 = i < m->nx - 1 ? m->d[gi(m, i + 1, j, k)] : c0;
                float c3 = j < m->ny - 1 ? m->d[gi(m, i, j + 1, k)] : c0;
                float c4 = k < m->nz - 1 ? m->d[gi(m, i, j, k + 1)] : c0;
                if (fabsf(c0) < FLT_EPSILON) c0 = FLT_EPSILON;
                if (fabsf(c1) < FLT_EPSILON) c1 = FLT_EPSILON;
                if (fabsf(c3) < FLT_EPSILON) c3 = FLT_EPSILON;
                if (fabsf(c4) < FLT_EPSILON) c4 = FLT_EPSILON;
                int ex, ey, ez;
                if (c0 < 0) { ex = c1 > 0; ey = c3 > 0; ez = c4 > 0; }
                else { ex = c1 < 0; ey = c3 < 0; ez = c4 < 0; }
                size_t g = gi(m, i, j, k);
                m->cur_kind = 0; m->cur_index = (int)g;
                m->cur_axis = 0;
                if (ex) {
                    float den = c0 - c1, u = den != 0.0f ? c0 / den : 0.5f;
                    m->xv[g] = push_vertex(m, (float)i + u, (float)j, (float)k);
                }
                m->cur_axis = 1;
                if (ey) {
                    float den = c0 - c3, u = den != 0.0f ? c0 / den : 0.5f;
                    m->yv[g] = push_vertex(m, (float)i, (float)j + u, (float)k);
                }
                m->cur_axis = 2;
                if (ez) {
                    float den = c0 - c4, u = den != 0.0f ? c0 / den : 0.5f;
                    m->zv[g] = push_vertex(m, (float)i, (float)j, (float)k + u);
                }
            }
}

/* test_face: src/MarchingCubes.c:276-295 */
static int mc_test_face(const mcx *m, int face) {
    static const int fc[6][4] = {{0, 4, 5, 1}, {1, 5, 6, 2}, {2, 6, 7, 3}, {3, 7, 4, 0}, {0, 3, 2, 1}, {4, 7, 6, 5}};
    float A = 0, B = 0, C = 0, D = 0;
    int f = face < 0 ? -face : face;
    if (f >= 1 && f <= 6) {
        A = m->cube[fc[f - 1][0]]; B = m->cube[fc[f - 1][1]];
        C = m->cube[fc[f - 1][2]]; D = m->cube[fc[f - 1][3]];
    }
    float det = A * C - B * D;
    if (fabsf(det) < FLT_EPSILON) return face >= 0;
    return (float)face * A * det >= 0;
}

/* test_interior: src/MarchingCubes.c:301-453.  For cases 6/7/12/13 the
 * reference edge `e` runs from corner ea to eb; the three opposite parallel
 * edges give Bt, Ct, Dt. */
static int mc_test_interior(const mcx *m, int s) {
    const float *c = m->cube;
    float t, At = 0, Bt = 0, Ct = 0, Dt = 0;
    int edge = -1;
    /* per reference edge: t = c[p]/(c[p]-c[q]), then Bt/Ct/Dt interpolate
     * corner pairs (b0->b1), (c0->c1), (d0->d1) — src/MarchingCubes.c:337-431 */
    static const int E[12][8] = {
        {0, 1, 3, 2, 7, 6, 4, 5}, {1, 2, 0, 3, 4, 7, 5, 6}, {2, 3, 1, 0, 5, 4, 6, 7}, {3, 0, 2, 1, 6, 5, 7, 4},
        {4, 5, 7, 6, 3, 2, 0, 1}, {5, 6, 4, 7, 0, 3, 1, 2}, {6, 7, 5, 4, 1, 0, 2, 3}, {7, 4, 6, 5, 2, 1, 3, 0},
        {0, 4, 3, 7, 2, 6, 1, 5}, {1, 5, 0, 4, 3, 7, 2, 6}, {2, 6, 1, 5, 0, 4, 3, 7}, {3, 7, 2, 6, 1, 5, 0, 4}};
    switch (m->kase) {
    case 4:
    case 10: {
        float a = (c[4] - c[0]) * (c[6] - c[2]) - (c[7] - c[3]) * (c[5] - c[1]);
        float b = c[2] * (c[4] - c[0]) + c[0] * (c[6] - c[2]) - c[1] * (c[7] - c[3]) - c[3] * (c[5] - c[1]);
        t = -b / (2 * a);
        if (t < 0 || t > 1) return s > 0;
        At = c[0] + (c[4] - c[0]) * t;
        Bt = c[3] + (c[7] - c[3]) * t;
        Ct = c[2] + (c[6] - c[2]) * t;
        Dt = c[1] + (c[5] - c[1]) * t;
        break;
    }
    case 6: case 7: case 12: case 13:
        switch (m->kase) {
        case 6: edge = LUT2(TEST6, m->config, 2); break;
        case 7: edge = LUT2(TEST7, m->config, 4); break;
        case 12: edge = LUT2(TEST12, m->config, 3); break;
        case 13: edge = LUT3(TILING13_5_1, m->config, m->subconfig, 0); break;
        }
        if (edge >= 0 && edge < 12) {
            const int *e = E[edge];
            t = c[e[0]] / (c[e[0]] - c[e[1]]);
            At = 0;
            Bt = c[e[2]] + (c[e[3]] - c[e[2]]) * t;
            Ct = c[e[4]] + (c[e[5]] - c[e[4]]) * t;
            Dt = c[e[6]] + (c[e[7]] - c[e[6]]) * t;
        }
        break;
    default: break;
    }
    int test = 0;
    if (At >= 0) test += 1;
    if (Bt >= 0) test += 2;
    if (Ct >= 0) test += 4;
    if (Dt >= 0) test += 8;
    switch (test) {
    case 5: if (At * Ct - Bt * Dt < FLT_EPSILON) return s > 0; break;
    case 10: if (At * Ct - Bt * Dt >= FLT_EPSILON) return s > 0; break;
    case 7: case 11: case 13: case 14: case 15: return s < 0;
    default: return s > 0;
    }
    return s < 0;
}

/* add_c_vertex: src/MarchingCubes.c:1029-1082 — float mean of the cube's
 * existing edge vertices, visited in edge order 0..11. */
static int mc_c_vertex(mcx *m) {
    const int i = m->i, j = m->j, k = m->k;
    m->cur_kind = 1; m->cur_index = (int)gi(m, i, j, k); m->cur_axis = -1;
    const int *ids[12] = {&m->xv[gi(m, i, j, k)],         &m->yv[gi(m, i + 1, j, k)],
                          &m->xv[gi(m, i, j + 1, k)],     &m->yv[gi(m, i, j, k)],
                          &m->xv[gi(m, i, j, k + 1)],     &m->yv[gi(m, i + 1, j, k + 1)],
                          &m->xv[gi(m, i, j + 1, k + 1)], &m->yv[gi(m, i, j, k + 1)],
                          &m->zv[gi(m, i, j, k)],         &m->zv[gi(m, i + 1, j, k)],
                          &m->zv[gi(m, i + 1, j + 1, k)], &m->zv[gi(m, i, j + 1, k)]};
    float n = 0, x = 0, y = 0, z = 0;
    for (int e = 0; e < 12; e++) {
        int v = *ids[e];
        if (v == -1) continue;
        ++n;
        x += m->vp[3 * v]; y += m->vp[3 * v + 1]; z += m->vp[3 * v + 2];
    }
    if (n > 0) { x /= n; y /= n; z /= n; }
    return push_vertex(m, x, y, z);
}

/* add_triangle: src/MarchingCubes.c:803-859 */
static void mc_add_triangles(mcx *m, const signed char *trig, int n, int v12) {
    const int i = m->i, j = m->j, k = m->k;
    int tv[3] = {-1, -1, -1};
    for (int t = 0; t < 3 * n; t++) {
        switch (trig[t]) {
        case 0: tv[t % 3] = m->xv[gi(m, i, j, k)]; break;
        case 1: tv[t % 3] = m->yv[gi(m, i + 1, j, k)]; break;
        case 2: tv[t % 3] = m->xv[gi(m, i, j + 1, k)]; break;
        case 3: tv[t % 3] = m->yv[gi(m, i, j, k)]; break;
        case 4: tv[t % 3] = m->xv[gi(m, i, j, k + 1)]; break;
        case 5: tv[t % 3] = m->yv[gi(m, i + 1, j, k + 1)]; break;
        case 6: tv[t % 3] = m->xv[gi(m, i, j + 1, k + 1)]; break;
        case 7: tv[t % 3] = m->yv[gi(m, i, j, k + 1)]; break;
        case 8: tv[t % 3] = m->zv[gi(m, i, j, k)]; break;
        case 9: tv[t % 3] = m->zv[gi(m, i + 1, j, k)]; break;
        case 10: tv[t % 3] = m->zv[gi(m, i + 1, j + 1, k)]; break;
        case 11: tv[t % 3] = m->zv[gi(m, i, j + 1, k)]; break;
        case 12: tv[t % 3] = v12; break;
        default: break;
        }
        if (t % 3 == 2) {
            if (m->nt >= m->capt) {
                m->capt = m->capt ? 2 * m->capt : 65536;
                m->tr = (int *)realloc(m->tr, (size_t)m->capt * 3 * sizeof(int));
            }
            m->tr[3 * m->nt] = tv[0]; m->tr[3 * m->nt + 1] = tv[1]; m->tr[3 * m->nt + 2] = tv[2];
            m->nt++;
        }
    }
}

/* process_cube: src/MarchingCubes.c:458-795 */
static void mc_process_cube(mcx *m, int lut) {
    if (m->original) {
        const signed char *tt = &n2m_lut_blob[N2M_CASESCLASSIC_OFF + lut * N2M_CASESCLASSIC_S0];
        int nt = 0;
        while (tt[3 * nt] != -1) nt++;
        mc_add_triangles(m, tt, nt, -1);
        return;
    }
    const int cf = LUT2(CASES, lut, 1);
    m->kase = LUT2(CASES, lut, 0);
    m->config = cf;
    m->subconfig = 0;
    int v12 = -1;
    switch (m->kase) {
    case 0: break;
    case 1: mc_add_triangles(m, PTR2(TILING1, cf), 1, -1); break;
    case 2: mc_add_triangles(m, PTR2(TILING2, cf), 2, -1); break;
    case 3:
        if (mc_test_face(m, LUT1(TEST3, cf))) mc_add_triangles(m, PTR2(TILING3_2, cf), 4, -1);
        else mc_add_triangles(m, PTR2(TILING3_1, cf), 2, -1);
        break;
    case 4:
        if (mc_test_interior(m, LUT1(TEST4, cf))) mc_add_triangles(m, PTR2(TILING4_1, cf), 2, -1);
        else mc_add_triangles(m, PTR2(TILING4_2, cf), 6, -1);
        break;
    case 5: mc_add_triangles(m, PTR2(TILING5, cf), 3, -1); break;
    case 6:
        if (mc_test_face(m, LUT2(TEST6, cf, 0))) mc_add_triangles(m, PTR2(TILING6_2, cf), 5, -1);
        else if (mc_test_interior(m, LUT2(TEST6, cf, 1))) mc_add_triangles(m, PTR2(TILING6_1_1, cf), 3, -1);
        else { v12 = mc_c_vertex(m); mc_add_triangles(m, PTR2(TILING6_1_2, cf), 9, v12); }
        break;
    case 7:
        if (mc_test_face(m, LUT2(TEST7, cf, 0))) m->subconfig += 1;
        if (mc_test_face(m, LUT2(TEST7, cf, 1))) m->subconfig += 2;
        if (mc_test_face(m, LUT2(TEST7, cf, 2))) m->subconfig += 4;
        switch (m->subconfig) {
        case 0: mc_add_triangles(m, PTR2(TILING7_1, cf), 3, -1); break;
        case 1: mc_add_triangles(m, PTR3(TILING7_2, cf, 0), 5, -1); break;
        case 2: mc_add_triangles(m, PTR3(TILING7_2, cf, 1), 5, -1); break;
        case 3: v12 = mc_c_vertex(m); mc_add_triangles(m, PTR3(TILING7_3, cf, 0), 9, v12); break;
        case 4: mc_add_triangles(m, PTR3(TILING7_2, cf, 2), 5, -1); break;
        case 5: v12 = mc_c_vertex(m); mc_add_triangles(m, PTR3(TILING7_3, cf, 1), 9, v12); break;
        case 6: v12 = mc_c_vertex(m); mc_add_triangles(m, PTR3(TILING7_3, cf, 2), 9, v12); break;
        case 7:
            if (mc_test_interior(m, LUT2(TEST7, cf, 3))) mc_add_triangles(m, PTR2(TILING7_4_2, cf), 9, -1);
            else mc_add_triangles(m, PTR2(TILING7_4_1, cf), 5, -1);
            break;
        }
        break;
    case 8: mc_add_triangles(m, PTR2(TILING8, cf), 2, -1); break;
    case 9: mc_add_triangles(m, PTR2(TILING9, cf), 4, -1); break;
    case 10:
        if (mc_test_face(m, LUT2(TEST10, cf, 0))) {
            if (mc_test_face(m, LUT2(TEST10, cf, 1))) mc_add_triangles(m, PTR2(TILING10_1_1_B, cf), 4, -1);
            else { v12 = mc_c_vertex(m); mc_add_triangles(m, PTR2(TILING10_2, cf), 8, v12); }
        } else {
            if (mc_test_face(m, LUT2(TEST10, cf, 1))) { v12 = mc_c_vertex(m); mc_add_triangles(m, PTR2(TILING10_2_B, cf), 8, v12); }
            else if (mc_test_interior(m, LUT2(TEST10, cf, 2))) mc_add_triangles(m, PTR2(TILING10_1_1, cf), 4, -1);
            else mc_add_triangles(m, PTR2(TILING10_1_2, cf), 8, -1);
        }
        break;
    case 11: mc_add_triangles(m, PTR2(TILING11, cf), 4, -1); break;
    case 12:
        if (mc_test_face(m, LUT2(TEST12, cf, 0))) {
            if (mc_test_face(m, LUT2(TEST12, cf, 1))) mc_add_triangles(m, PTR2(TILING12_1_1_B, cf), 4, -1);
            else { v12 = mc_c_vertex(m); mc_add_triangles(m, PTR2(TILING12_2, cf), 8, v12); }
        } else {
            if (mc_test_face(m, LUT2(TEST12, cf, 1))) { v12 = mc_c_vertex(m); mc_add_triangles(m, PTR2(TILING12_2_B, cf), 8, v12); }
            else if (mc_test_interior(m, LUT2(TEST12, cf, 2))) mc_add_triangles(m, PTR2(TILING12_1_1, cf), 4, -1);
            else mc_add_triangles(m, PTR2(TILING12_1_2, cf), 8, -1);
        }
        break;
    case 13: {
        for (int f = 0; f < 6; f++)
            if (mc_test_face(m, LUT2(TEST13, cf, f))) m->subconfig += 1 << f;
        int sc = LUT1(SUBCONFIG13, m->subconfig);
        if (sc == 0) mc_add_triangles(m, PTR2(TILING13_1, cf), 4, -1);
        else if (sc >= 1 && sc <= 6) mc_add_triangles(m, PTR3(TILING13_2, cf, sc - 1), 6, -1);
        else if (sc >= 7 && sc <= 18) { v12 = mc_c_vertex(m); mc_add_triangles(m, PTR3(TILING13_3, cf, sc - 7), 10, v12); }
        else if (sc >= 19 && sc <= 22) { v12 = mc_c_vertex(m); mc_add_triangles(m, PTR3(TILING13_4, cf, sc - 19), 12, v12); }
        else if (sc >= 23 && sc <= 26) {
            m->subconfig = sc - 23;
            if (mc_test_interior(m, LUT2(TEST13, cf, 6))) mc_add_triangles(m, PTR3(TILING13_5_1, cf, sc - 23), 6, -1);
            else mc_add_triangles(m, PTR3(TILING13_5_2, cf, sc - 23), 10, -1);
        } else if (sc >= 27 && sc <= 38) { v12 = mc_c_vertex(m); mc_add_triangles(m, PTR3(TILING13_3_B, cf, sc - 27), 10, v12); }
        else if (sc >= 39 && sc <= 44) mc_add_triangles(m, PTR3(TILING13_2_B, cf, sc - 39), 6, -1);
        else if (sc == 45) mc_add_triangles(m, PTR2(TILING13_1_B, cf), 4, -1);
        break;
    }
    case 14: mc_add_triangles(m, PTR2(TILING14, cf), 4, -1); break;
    }
}

/* run: src/MarchingCubes.c:116-155 */
static void mc_run(mcx *m) {
    size_t g = (size_t)m->nx * m->ny * m->nz;
    m->xv = (int *)malloc(g * sizeof(int));
    m->yv = (int *)malloc(g * sizeof(int));
    m->zv = (int *)malloc(g * sizeof(int));
    memset(m->xv, -1, g * sizeof(int));
    memset(m->yv, -1, g * sizeof(int));
    memset(m->zv, -1, g * sizeof(int));
    mc_edge_vertices(m);
    for (m->k = 0; m->k < m->nz - 1; m->k++)
        for (m->j = 0; m->j < m->ny - 1; m->j++)
            for (m->i = 0; m->i < m->nx - 1; m->i++) {
                int lut = 0;
                for (int p = 0; p < 8; p++) {
                    float v = m->d[gi(m, m->i + ((p ^ (p >> 1)) & 1), m->j + ((p >> 1) & 1), m->k + ((p >> 2) & 1))];
                    if (fabsf(v) < FLT_EPSILON) v = FLT_EPSILON;
                    m->cube[p] = v;
                    if (v > 0) lut += 1 << p;
                }
                mc_process_cube(m, lut);
            }
    free(m->xv); free(m->yv); free(m->zv);
}

int or_mc_raw(const float *data, int nx, int ny, int nz, int originalMC, float **verts, int **tris, int *nv, int *nt) {
    mcx m;
    memset(&m, 0, sizeof(m));
    m.nx = nx; m.ny = ny; m.nz = nz; m.original = originalMC; m.d = data;
    mc_run(&m);
    *verts = m.vp; *tris = m.tr; *nv = m.nv; *nt = m.nt;
    free(m.src);
    return 0;
}

/* marchingCubes wrapper (Lewiner): src/MarchingCubes.c:1086-1143.  The grid
 * spans the padded bbox; a grid point maps to linear voxel index
 * lo0+x + (y+lo1)*dim0 + (z+lo2)*dim0*dim1 (so x past the row end reads the
 * next row), and indices past the volume hold min-minus-isolevel. */
/* when set, mc_lewiner hands out the per-vertex sources (test use only) */
static int **mc_sources_out = NULL;

static int mc_lewiner(float *img, const short dim[3], const int lo[3], const int hi[3], int originalMC, float iso,
                      or_vec3d **vs, or_vec3i **ts, int *nv, int *nt) {
    const int NX = hi[0] - lo[0] + 1, NY = hi[1] - lo[1] + 1, NZ = hi[2] - lo[2] + 1;
    const long inXYZ = (long)dim[0] * dim[1] * dim[2], inX = dim[0], inXY = (long)dim[0] * dim[1];
    float mn = img[0];
    for (long i = 0; i < inXYZ; i++) mn = (float)fmin(mn, img[i]);
    mn = mn - iso;
    float *g = (float *)malloc((size_t)NX * NY * NZ * sizeof(float));
    size_t o = 0;
    for (int z = 0; z < NZ; z++)
        for (int y = 0; y < NY; y++) {
            long zy = (long)(y + lo[1]) * inX + (long)(z + lo[2]) * inXY;
            for (int x = 0; x < NX; x++, o++) {
                long j = lo[0] + x + zy;
                g[o] = j < inXYZ ? img[j] - iso : mn;
            }
        }
    mcx m;
    memset(&m, 0, sizeof(m));
    m.nx = NX; m.ny = NY; m.nz = NZ; m.original = originalMC; m.d = g;
    mc_run(&m);
    free(g);
    if (m.nv < 3 || m.nt < 1) { free(m.vp); free(m.tr); free(m.src); return 1; }
    *vs = (or_vec3d *)malloc((size_t)m.nv * sizeof(or_vec3d));
    for (int i = 0; i < m.nv; i++) {
        (*vs)[i].x = m.vp[3 * i] + lo[0];
        (*vs)[i].y = m.vp[3 * i + 1] + lo[1];
        (*vs)[i].z = m.vp[3 * i + 2] + lo[2];
    }
    *ts = (or_vec3i *)malloc((size_t)m.nt * sizeof(or_vec3i));
    for (int i = 0; i < m.nt; i++) {
        (*ts)[i].x = m.tr[3 * i + 2];
        (*ts)[i].y = m.tr[3 * i + 1];
        (*ts)[i].z = m.tr[3 * i];
    }
    *nv = m.nv; *nt = m.nt;
    if (mc_sources_out) { *mc_sources_out = m.src; m.src = NULL; }
    free(m.vp); free(m.tr); free(m.src);
    return 0;
}

/* oldcubes marchingCubes/PolygoniseCube/VertexInterp: src/oldcubes.c:22-40,
 * :401-463, :465-522.  Bit set when value < isolevel; double interpolation;
 * three private vertices per triangle. */
static or_vec3d old_interp(double iso, or_vec3d p1, or_vec3d p2, double v1, double v2) {
    double mu = (iso - v1) / (v2 - v1);
    or_vec3d p = {p1.x + mu * (p2.x - p1.x), p1.y + mu * (p2.y - p1.y), p1.z + mu * (p2.z - p1.z)};
    return p;
}

static int mc_oldcubes(const float *img, const short dim[3], const int lo[3], const int hi[3], float isolevel,
                       or_vec3d **vs, or_vec3i **ts, int *nv, int *nt) {
    static const int ea[12] = {0, 1, 2, 3, 4, 5, 6, 7, 0, 1, 2, 3}, eb[12] = {1, 2, 3, 0, 5, 6, 7, 4, 4, 5, 6, 7};
    static const int cx[8] = {0, 1, 1, 0, 0, 1, 1, 0}, cy[8] = {0, 0, 1, 1, 0, 0, 1, 1}, cz[8] = {0, 0, 0, 0, 1, 1, 1, 1};
    const long NX = dim[0], NXY = (long)dim[0] * dim[1];
    const double iso = isolevel;
    size_t cap = 65536 * 16, n = 0;
    or_vec3d *pts = (or_vec3d *)malloc(cap * sizeof(or_vec3d));
    for (int z = lo[2]; z < hi[2] - 1; z++)
        for (int y = lo[1]; y < hi[1] - 1; y++)
            for (int x = lo[0]; x < hi[0] - 1; x++) {
                double val[8];
                or_vec3d p[8];
                int ci = 0;
                for (int c = 0; c < 8; c++) {
                    val[c] = img[(long)(z + cz[c]) * NXY + (long)(y + cy[c]) * NX + x + cx[c]];
                    if (val[c] < iso) ci |= 1 << c;
                    p[c].x = x + cx[c]; p[c].y = y + cy[c]; p[c].z = z + cz[c];
                }
                int em = n2m_classic_edge[ci];
                if (!em) continue;
                or_vec3d vl[12];
                for (int e = 0; e < 12; e++)
                    if (em & (1 << e)) vl[e] = old_interp(iso, p[ea[e]], p[eb[e]], val[ea[e]], val[eb[e]]);
                if (n + 30 > cap) { cap = cap * 3 / 2; pts = (or_vec3d *)realloc(pts, cap * sizeof(or_vec3d)); }
                const signed char *tri = &n2m_classic_tri[ci * 16];
                for (int t = 0; tri[t] != -1; t += 3) {
                    pts[n++] = vl[tri[t]];
                    pts[n++] = vl[tri[t + 1]];
                    pts[n++] = vl[tri[t + 2]];
                }
            }
    if (n < 3) { free(pts); return 1; }
    *vs = pts;
    int ntri = (int)(n / 3);
    *ts = (or_vec3i *)malloc((size_t)ntri * sizeof(or_vec3i));
    for (int i = 0; i < ntri; i++) { (*ts)[i].x = 3 * i; (*ts)[i].y = 3 * i + 1; (*ts)[i].z = 3 * i + 2; }
    *nv = (int)n; *nt = ntri;
    return 0;
}

/* Lewiner marching cubes that also reports, per vertex, where it comes from:
 * (0, grid point, axis) for edge vertices, (1, cube, -1) for c-vertices,
 * grid indices over the padded box (hi-lo+1 points per axis). */
int or_marching_cubes_sources(float *img, const short dim[3], const int lo[3], const int hi[3], int originalMC,
                              float isolevel, or_vec3d **vs, or_vec3i **ts, int *nv, int *nt, int **src) {
    mc_sources_out = src;
    int r = mc_lewiner(img, dim, lo, hi, originalMC, isolevel, vs, ts, nv, nt);
    mc_sources_out = NULL;
    return r;
}

int or_marching_cubes(float *img, const short dim[3], const int lo[3], const int hi[3], int variant, float isolevel,
                      or_vec3d **vs, or_vec3i **ts, int *nv, int *nt) {
    if (variant == OR_OLDCUBES) return mc_oldcubes(img, dim, lo, hi, isolevel, vs, ts, nv, nt);
    return mc_lewiner(img, dim, lo, hi, variant == OR_MC_CLASSIC_TABLE, isolevel, vs, ts, nv, nt);
}

/* ------------------------------------------------------------------------ */
/* unify_vertices: src/meshify.c:45-106 (key sort: src/radixsort.c:277-362,
 * a stable ascending sort of float keys).  Key = float distance to vertex 0;
 * greedy grouping within 1e-5 in key order; ids renumbered in sort order
 * when anything merged, positions last-writer-wins. */
typedef struct { uint32_t key; uint32_t idx; } keyidx;
static int cmp_keyidx(const void *a, const void *b) {
    const keyidx *p = (const keyidx *)a, *q = (const keyidx *)b;
    if (p->key != q->key) return p->key < q->key ? -1 : 1;
    return p->idx < q->idx ? -1 : (p->idx > q->idx);
}
static double dist3(or_vec3d a, or_vec3d b) {
    double dx = a.x - b.x, dy = a.y - b.y, dz = a.z - b.z;
    return sqrt(dx * dx + dy * dy + dz * dz);
}
static uint32_t float_order_bits(float f) {
    uint32_t u;
    memcpy(&u, &f, 4);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}

int or_unify_vertices(or_vec3d **inpt, or_vec3i *tris, int npt, int ntri) {
    or_vec3d *pts = *inpt;
    keyidx *ki = (keyidx *)malloc((size_t)npt * sizeof(keyidx));
    float *key = (float *)malloc((size_t)npt * sizeof(float));
    int *old2new = (int *)malloc((size_t)npt * sizeof(int));
    for (int i = 0; i < npt; i++) {
        key[i] = (float)dist3(pts[0], pts[i]);
        ki[i].key = float_order_bits(key[i]);
        ki[i].idx = (uint32_t)i;
        old2new[i] = -1;
    }
    qsort(ki, (size_t)npt, sizeof(keyidx), cmp_keyidx);
    const float tol = 0.00001f;
    int nnew = 0;
    for (int i = 0; i < npt; i++) {
        if (old2new[ki[i].idx] >= 0) continue;
        float k0 = key[ki[i].idx];
        or_vec3d p0 = pts[ki[i].idx];
        for (int j = i; j < npt && (key[ki[j].idx] - k0) < tol; j++)
            if (dist3(p0, pts[ki[j].idx]) < tol) old2new[ki[j].idx] = nnew;
        nnew++;
    }
    free(ki);
    free(key);
    if (nnew == npt) { free(old2new); return npt; }
    for (int i = 0; i < ntri; i++) {
        tris[i].x = old2new[tris[i].x];
        tris[i].y = old2new[tris[i].y];
        tris[i].z = old2new[tris[i].z];
    }
    or_vec3d *np = (or_vec3d *)malloc((size_t)nnew * sizeof(or_vec3d));
    for (int i = 0; i < npt; i++) np[old2new[i]] = pts[i];
    free(pts);
    *inpt = np;
    free(old2new);
    return nnew;
}

/* remove_degenerate_triangles: src/meshify.c:113-168 */
int or_remove_degenerate_triangles(or_vec3d *pts, or_vec3i **intris, int ntri) {
    or_vec3i *tris = *intris;
    int keep = 0;
    unsigned char *bad = (unsigned char *)calloc((size_t)ntri, 1);
    for (int i = 0; i < ntri; i++) {
        double l = dist3(pts[tris[i].x], pts[tris[i].y]);
        double m = dist3(pts[tris[i].x], pts[tris[i].z]);
        double n = dist3(pts[tris[i].y], pts[tris[i].z]);
        double c = fmin(fmin(l, m), n);
        double a = fmax(fmax(l, m), n);
        double b = l + m + n - a - c;
        if ((c - (a - b)) <= 0.0) { bad[i] = 1; continue; }
        double area4 = 0.25 * sqrt((a + (b + c)) * (c - (a - b)) * (c + (a - b)) * (a + (b - c)));
        if (area4 < FLT_EPSILON) bad[i] = 1;
    }
    for (int i = 0; i < ntri; i++)
        if (!bad[i]) tris[keep++] = tris[i];
    free(bad);
    return keep;
}

int or_meshify(float *img, const short dim[3], int variant, float isolevel, or_vec3i **t, or_vec3d **p, int *nt,
               int *np, bool preSmooth, bool onlyLargest, bool fillBubbles) {
    int lo[3], hi[3];
    if (or_prepare_volume(img, dim, &isolevel, preSmooth, onlyLargest, fillBubbles, lo, hi, NULL)) return 1;
    or_vec3d *pts = NULL;
    or_vec3i *tris = NULL;
    int npt, ntri;
    if (or_marching_cubes(img, dim, lo, hi, variant, isolevel, &pts, &tris, &npt, &ntri)) return 1;
    npt = or_unify_vertices(&pts, tris, npt, ntri);
    if (npt < 3) { free(pts); free(tris); return 1; }
    ntri = or_remove_degenerate_triangles(pts, &tris, ntri);
    *t = tris; *p = pts; *nt = ntri; *np = npt;
    return 0;
}

/* ------------------------------------------------------------------------ */
/* laplacian_smooth: src/quadric.c:316-341 — Jacobi mean over the two other
 * vertices of every incident triangle (accumulated in triangle order). */
void or_laplacian_smooth(or_vec3d *v, const or_vec3i *t, int nv, int nt) {
    or_vec3d *sum = (or_vec3d *)calloc((size_t)nv, sizeof(or_vec3d));
    int *num = (int *)calloc((size_t)nv, sizeof(int));
    for (int i = 0; i < nt; i++) {
        int a = t[i].x, b = t[i].y, c = t[i].z;
        num[a] += 2;
        sum[a].x = sum[a].x + (v[b].x + v[c].x); sum[a].y = sum[a].y + (v[b].y + v[c].y); sum[a].z = sum[a].z + (v[b].z + v[c].z);
        num[b] += 2;
        sum[b].x = sum[b].x + (v[a].x + v[c].x); sum[b].y = sum[b].y + (v[a].y + v[c].y); sum[b].z = sum[b].z + (v[a].z + v[c].z);
        num[c] += 2;
        sum[c].x = sum[c].x + (v[a].x + v[b].x); sum[c].y = sum[c].y + (v[a].y + v[b].y); sum[c].z = sum[c].z + (v[a].z + v[b].z);
    }
    for (int i = 0; i < nv; i++) {
        if (num[i] <= 0) continue;
        v[i].x = sum[i].x / num[i]; v[i].y = sum[i].y / num[i]; v[i].z = sum[i].z / num[i];
    }
    free(sum); free(num);
}

/* border flags of update_mesh(0): src/quadric.c:144-215.  For each vertex,
 * count how often every vertex id occurs among its incident triangles; an id
 * seen exactly once lies on an edge used by a single triangle. */
void or_border_vertices(const or_vec3i *t, int nv, int nt, unsigned char *border) {
    int *start = (int *)calloc((size_t)nv + 1, sizeof(int));
    for (int i = 0; i < nt; i++) { start[t[i].x + 1]++; start[t[i].y + 1]++; start[t[i].z + 1]++; }
    for (int i = 0; i < nv; i++) start[i + 1] += start[i];
    int *fill = (int *)calloc((size_t)nv, sizeof(int));
    int *ref = (int *)malloc((size_t)3 * nt * sizeof(int) + 1);
    for (int i = 0; i < nt; i++) {
        const int vv[3] = {t[i].x, t[i].y, t[i].z};
        for (int j = 0; j < 3; j++) ref[start[vv[j]] + fill[vv[j]]++] = i;
    }
    if (nv > 0) memset(border, 0, (size_t)nv);
    int cap = 64, *ids = (int *)malloc(cap * sizeof(int)), *cnt = (int *)malloc(cap * sizeof(int));
    for (int v = 0; v < nv; v++) {
        int nid = 0;
        for (int r = start[v]; r < start[v + 1]; r++) {
            const int vv[3] = {t[ref[r]].x, t[ref[r]].y, t[ref[r]].z};
            for (int k = 0; k < 3; k++) {
                int o = 0;
                while (o < nid && ids[o] != vv[k]) o++;
                if (o == nid) {
                    if (nid == cap) { cap *= 2; ids = (int *)realloc(ids, cap * sizeof(int)); cnt = (int *)realloc(cnt, cap * sizeof(int)); }
                    ids[nid] = vv[k]; cnt[nid] = 1; nid++;
                } else cnt[o]++;
            }
        }
        for (int o = 0; o < nid; o++)
            if (cnt[o] == 1) border[ids[o]] = 1;
    }
    free(ids); free(cnt); free(ref); free(fill); free(start);
}

/* laplacian_smoothHC: src/quadric.c:343-394 (HC filter of Vollmer et al.). */
void or_laplacian_smoothHC(or_vec3d *verts, const or_vec3i *tris, int nv, int nt, double alpha, double beta, int iter,
                           bool lockEdges) {
    const double a1 = 1.0 - alpha, b1 = 1.0 - beta;
    or_vec3d *p = (or_vec3d *)malloc((size_t)nv * sizeof(or_vec3d));
    or_vec3d *q = (or_vec3d *)malloc((size_t)nv * sizeof(or_vec3d));
    or_vec3d *b = (or_vec3d *)malloc((size_t)nv * sizeof(or_vec3d));
    memcpy(p, verts, (size_t)nv * sizeof(or_vec3d));
    for (int it = 0; it < iter; it++) {
        memcpy(q, p, (size_t)nv * sizeof(or_vec3d));
        or_laplacian_smooth(p, tris, nv, nt);
        for (int i = 0; i < nv; i++) {
            b[i].x = p[i].x - (verts[i].x * alpha + q[i].x * a1);
            b[i].y = p[i].y - (verts[i].y * alpha + q[i].y * a1);
            b[i].z = p[i].z - (verts[i].z * alpha + q[i].z * a1);
        }
        memcpy(q, b, (size_t)nv * sizeof(or_vec3d));
        or_laplacian_smooth(q, tris, nv, nt);
        for (int i = 0; i < nv; i++) {
            p[i].x = p[i].x - (b[i].x * beta + q[i].x * b1);
            p[i].y = p[i].y - (b[i].y * beta + q[i].y * b1);
            p[i].z = p[i].z - (b[i].z * beta + q[i].z * b1);
        }
    }
    free(q); free(b);
    if (!lockEdges) {
        memcpy(verts, p, (size_t)nv * sizeof(or_vec3d));
        free(p);
        return;
    }
    unsigned char *border = (unsigned char *)malloc((size_t)nv + 1);
    or_border_vertices(tris, nv, nt, border);
    for (int i = 0; i < nv; i++)
        if (!border[i]) verts[i] = p[i];
    free(border); free(p);
}

/* apply_sform: src/meshify.c:1021-1045 */
void or_apply_sform(or_vec3i *t, or_vec3d *p, int nt, int np, const float sx[4], const float sy[4], const float sz[4]) {
    for (int i = 0; i < np; i++) {
        or_vec3d v = p[i];
        p[i].x = (v.x * sx[0]) + (v.y * sx[1]) + (v.z * sx[2]) + sx[3];
        p[i].y = (v.x * sy[0]) + (v.y * sy[1]) + (v.z * sy[2]) + sy[3];
        p[i].z = (v.x * sz[0]) + (v.y * sz[1]) + (v.z * sz[2]) + sz[3];
    }
    double px = sx[0] + sx[1] + sx[2], py = sy[0] + sy[1] + sy[2], pz = sz[0] + sz[1] + sz[2];
    float det = (float)(px * py * pz);
    if (det >= 0.0) return;
    for (int i = 0; i < nt; i++) { int x = t[i].x; t[i].x = t[i].y; t[i].y = x; }
}

/* ------------------------------------------------------------------------ */
/* setThreshold: src/isolevel.c:245-277 with nifti_robust_range :35-139 and
 * nii_otsu :141-243 (modes 3 and 5). */
static void robust_range(const float *img, int nvox, float *pct2, float *pct98) {
    *pct2 = 0.0f; *pct98 = 1.0f;
    if (nvox < 1) return;
    float mn = INFINITY, mx = -INFINITY;
    size_t nZero = 0, nNan = 0;
    for (int i = 0; i < nvox; i++) {
        if (isnan(img[i])) { nNan++; continue; }
        if (img[i] == 0.0f) nZero++;
        mn = (float)fmin(img[i], mn);
        mx = (float)fmax(img[i], mx);
    }
    if (nZero > 0 && mn > 0.0f) mn = 0.0f;
    if (mn > mx) return;
    if (mn == mx) { *pct2 = mn; *pct98 = mx; return; }
    nZero = nNan;
    size_t n2pct = (size_t)round((nvox - nZero) * 0.02);
    if (n2pct < 1 || (nvox - nZero) < 100) { *pct2 = mn; *pct98 = mx; return; }
    enum { NB = 1001 };
    float scl = (NB - 1) / (mx - mn);
    static int hist[NB];
    memset(hist, 0, sizeof(hist));
    for (int i = 0; i < nvox; i++) {
        if (isnan(img[i])) continue;
        hist[(int)round((img[i] - mn) * scl)]++;
    }
    size_t n = 0, lo = 0;
    while (n < n2pct) n += hist[lo++];
    lo--;
    n = 0;
    int hi = NB;
    while (n < n2pct) n += hist[--hi];
    if ((int)lo == hi) {
        int ok = -1;
        while (ok != 0) {
            if (lo > 0) { lo--; if (hist[lo] > 0) ok = 0; }
            if (ok != 0 && hi < NB - 1) { hi++; if (hist[hi] > 0) ok = 0; }
            if (lo == 0 && hi == NB - 1) ok = 0;
        }
    }
    *pct2 = (lo) / scl + mn;
    *pct98 = (hi) / scl + mn;
}

static int otsu(const int *H, int nBin, int mode, int *dark, int *mid, int *bright) {
    *dark = *mid = *bright = 0;
    double Sum = 0.0;
    for (int v = 0; v < nBin; v++) Sum = Sum + H[v];
    if (Sum <= 0) return 0;
    double *P = (double *)malloc((size_t)nBin * nBin * sizeof(double));
    double *S = (double *)malloc((size_t)nBin * nBin * sizeof(double));
    P[0] = H[0]; S[0] = H[0];
    for (int v = 1; v < nBin; v++) {
        double prob = H[v] / Sum;
        P[v] = P[v - 1] + prob;
        S[v] = S[v - 1] + (v + 1) * prob;
    }
    for (int u = 1; u < nBin; u++)
        for (int v = u; v < nBin; v++) {
            P[u * nBin + v] = P[v] - P[u - 1];
            S[u * nBin + v] = S[v] - S[u - 1];
        }
    for (int u = 0; u < nBin; u++)
        for (int v = u; v < nBin; v++)
            if (P[u * nBin + v] != 0) P[u * nBin + v] = (S[u * nBin + v] * S[u * nBin + v]) / P[u * nBin + v];
    int thresh = 0;
    if (mode == 1 || mode == 5) {
        int lo = (int)(0.25 * nBin), mi = (int)(0.50 * nBin), hi = (int)(0.75 * nBin);
        double best = P[lo] + P[(lo + 1) * nBin + mi] + P[(mi + 1) * nBin + hi] + P[(hi + 1) * nBin + 255];
        for (int l = 0; l < nBin - 3; l++)
            for (int m = l + 1; m < nBin - 2; m++)
                for (int h = m + 1; h < nBin - 1; h++) {
                    double v = P[l] + P[(l + 1) * nBin + m] + P[(m + 1) * nBin + h] + P[(h + 1) * nBin + 255];
                    if (v > best) { lo = l; mi = m; hi = h; best = v; }
                }
        thresh = mode == 1 ? hi : lo;
        *dark = lo; *mid = mi; *bright = hi;
    } else {
        thresh = (int)(0.25 * nBin);
        double best = P[thresh] + P[(thresh + 1) * nBin + nBin - 1];
        for (int i = 0; i < nBin - 1; i++) {
            double v = P[i] + P[(i + 1) * nBin + nBin - 1];
            if (v > best) { thresh = i; best = v; }
        }
        *dark = *mid = *bright = thresh;
    }
    free(P); free(S);
    return thresh;
}

float or_set_threshold(const float *img, int nvox, int mode123) {
    float mn, mx;
    robust_range(img, nvox, &mn, &mx);
    float scl = (256 - 1) / (mx - mn);
    int hist[256];
    memset(hist, 0, sizeof(hist));
    for (int i = 0; i < nvox; i++) {
        if (isnan(img[i])) continue;
        int idx = (int)round((img[i] - mn) * scl);
        idx = idx < 255 ? idx : 255;
        idx = idx > 0 ? idx : 0;
        hist[idx]++;
    }
    int dark, mid, bright;
    if (mode123 == 1 || mode123 == 3) {
        otsu(hist, 256, 5, &dark, &mid, &bright);
        return mode123 == 1 ? (dark / scl) + mn : (bright / scl) + mn;
    }
    otsu(hist, 256, 3, &dark, &mid, &bright);
    return (mid / scl) + mn;
}

/* atlas binarisation: src/nii2mesh.c:553-563 */
int or_binarize_label(const float *img, int nvox, int label, float *out) {
    int n1 = 0;
    float lo = label - 0.5, hi = label + 0.5;
    for (int j = 0; j < nvox; j++) {
        int n = (img[j] > lo) && (img[j] < hi);
        out[j] = (float)n;
        n1 += n;
    }
    return n1;
}

/* ------------------------------------------------------------------------ */
/* The ten analytic self-test fields, src/MarchingCubes.c:1282-1361 (60^3). */
int or_selftest_field(int obj, float *out) {
    const int N = 60;
    if (obj < 0 || obj > 9) return 1;
    float sx = (float)N / 16, sy = (float)N / 16, sz = (float)N / 16;
    float tx = (float)N / (2 * sx), ty = (float)N / (2 * sy) + 1.5f, tz = (float)N / (2 * sz);
    float r = 1.85f, R = 4;
    int vox = 0;
    for (int k = 0; k < N; k++) {
        float z = ((float)k) / sz - tz;
        for (int j = 0; j < N; j++) {
            float y = ((float)j) / sy - ty;
            for (int i = 0; i < N; i++) {
                float x = ((float)i) / sx - tx, val = 0;
                float a, b, c, d;
                switch (obj) {
                case 0:
                    val = z * z * x * x - z * z * z * z - 2 * z * x * x + 2 * z * z * z + x * x - z * z - (x * x - z) * (x * x - z) -
                          y * y * y * y - 2 * x * x * y * y - y * y * z * z + 2 * y * y * z + y * y;
                    break;
                case 1:
                    val = ((x - 2) * (x - 2) + (y - 2) * (y - 2) + (z - 2) * (z - 2) - 1) *
                          ((x + 2) * (x + 2) + (y - 2) * (y - 2) + (z - 2) * (z - 2) - 1) *
                          ((x - 2) * (x - 2) + (y + 2) * (y + 2) + (z - 2) * (z - 2) - 1);
                    break;
                case 2: val = x + y + z - 3; break;
                case 3:
                    val = (x * x + y * y + z * z + 0.45f * 0.45f) * (x * x + y * y + z * z + 0.45f * 0.45f) -
                          16 * 0.45f * 0.45f * (x * x + z * z) - 0.5f * 0.5f;
                    break;
                case 4: val = x * x * x * x - 5 * x * x + y * y * y * y - 5 * y * y + z * z * z * z - 5 * z * z + 11.8; break;
                case 5:
                    val = (x * x + y * y + z * z - 0.95f * 25) * (x * x + y * y + z * z - 0.95f * 25) -
                          0.8f * ((z - 5) * (z - 5) - 2 * x * x) * ((z + 5) * (z + 5) - 2 * y * y);
                    break;
                case 6:
                    b = 2; d = 6; a = 2; c = 3;
                    val = (x * x + y * y + z * z + b * b - d * d) * (x * x + y * y + z * z + b * b - d * d) -
                          4 * ((a * x - c * d) * (a * x - c * d) + b * b * y * y);
                    break;
                case 7:
                    val = ((x * x + y * y + z * z + R * R - r * r) * (x * x + y * y + z * z + R * R - r * r) - 4 * R * R * (x * x + y * y)) *
                          ((x * x + (y + R) * (y + R) + z * z + R * R - r * r) * (x * x + (y + R) * (y + R) + z * z + R * R - r * r) -
                           4 * R * R * ((y + R) * (y + R) + z * z));
                    break;
                case 8:
                    val = -26.5298 * (1 - x) * (1 - y) * (1 - z) + 81.9199 * x * (1 - y) * (1 - z) - 100.68 * x * y * (1 - z) +
                          3.5498 * (1 - x) * y * (1 - z) + 24.1201 * (1 - x) * (1 - y) * z - 74.4702 * x * (1 - y) * z +
                          91.5298 * x * y * z - 3.22998 * (1 - x) * y * z;
                    break;
                case 9: val = x * x + y * y - 0.5 * (0.995 * z * z + 0.005 - z * z * z) + 0.0025; break;
                }
                out[vox++] = val;
            }
        }
    }
    return 0;
}
