/* table_check.c — checks the packed marching-cubes tables (mc_tables.h) against
 * the reference's own tables, independently of the script that generated them.
 *
 *   table_check ours        writes every table as reconstructed from
 *                           mc_tables.h, element by element as little-endian
 *                           int32, in a fixed table order
 *   table_check ref         (built with -DWITH_REFERENCE -I <reference src>)
 *                           compares every element of the reference's
 *                           LookUpTable.h tables and oldcubes.c's edgeTable /
 *                           triTable (their declarations copied out of the
 *                           function that holds them into classic_tables.inc
 *                           by the test), as the C compiler reads them, with the
 *                           packed copy; prints each mismatch, exits 1 on any;
 *                           then writes the reference's tables in the same
 *                           stream format
 * The test hashes both streams: equal streams mean equal tables, and the hash
 * of the reference's stream is committed for machines without the reference.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "mc_tables.h"

#ifdef WITH_REFERENCE
#include "LookUpTable.h"
/* oldcubes.c declares its two tables inside PolygoniseCube; the test copies
   their declarations, initialisers verbatim, into classic_tables.inc */
#include "classic_tables.inc"
#endif

/* name in the reference, key of its N2M_<key>_OFF macro, element count */
#define LEWINER_TABLES(X)                                                                                 \
    X(cases, CASES, 256 * 2) X(tiling1, TILING1, 16 * 3) X(tiling2, TILING2, 24 * 6) X(test3, TEST3, 24)  \
    X(tiling3_1, TILING3_1, 24 * 6) X(tiling3_2, TILING3_2, 24 * 12) X(test4, TEST4, 8)                   \
    X(tiling4_1, TILING4_1, 8 * 6) X(tiling4_2, TILING4_2, 8 * 18) X(tiling5, TILING5, 48 * 9)            \
    X(test6, TEST6, 48 * 3) X(tiling6_1_1, TILING6_1_1, 48 * 9) X(tiling6_1_2, TILING6_1_2, 48 * 27)       \
    X(tiling6_2, TILING6_2, 48 * 15) X(test7, TEST7, 16 * 5) X(tiling7_1, TILING7_1, 16 * 9)               \
    X(tiling7_2, TILING7_2, 16 * 3 * 15) X(tiling7_3, TILING7_3, 16 * 3 * 27)                              \
    X(tiling7_4_1, TILING7_4_1, 16 * 15) X(tiling7_4_2, TILING7_4_2, 16 * 27) X(tiling8, TILING8, 6 * 6)  \
    X(tiling9, TILING9, 8 * 12) X(test10, TEST10, 6 * 3) X(tiling10_1_1, TILING10_1_1, 6 * 12)             \
    X(tiling10_1_1_, TILING10_1_1_B, 6 * 12) X(tiling10_1_2, TILING10_1_2, 6 * 24)                         \
    X(tiling10_2, TILING10_2, 6 * 24) X(tiling10_2_, TILING10_2_B, 6 * 24) X(tiling11, TILING11, 12 * 12)  \
    X(test12, TEST12, 24 * 4) X(tiling12_1_1, TILING12_1_1, 24 * 12) X(tiling12_1_1_, TILING12_1_1_B, 24 * 12) \
    X(tiling12_1_2, TILING12_1_2, 24 * 24) X(tiling12_2, TILING12_2, 24 * 24)                               \
    X(tiling12_2_, TILING12_2_B, 24 * 24) X(test13, TEST13, 2 * 7) X(subconfig13, SUBCONFIG13, 64)         \
    X(tiling13_1, TILING13_1, 2 * 12) X(tiling13_1_, TILING13_1_B, 2 * 12)                                 \
    X(tiling13_2, TILING13_2, 2 * 6 * 18) X(tiling13_2_, TILING13_2_B, 2 * 6 * 18)                         \
    X(tiling13_3, TILING13_3, 2 * 12 * 30) X(tiling13_3_, TILING13_3_B, 2 * 12 * 30)                       \
    X(tiling13_4, TILING13_4, 2 * 4 * 36) X(tiling13_5_1, TILING13_5_1, 2 * 4 * 18)                        \
    X(tiling13_5_2, TILING13_5_2, 2 * 4 * 30) X(tiling14, TILING14, 12 * 12)                               \
    X(casesClassic, CASESCLASSIC, 256 * 16)

static void put(int v) {
    unsigned char b[4] = {(unsigned char)v, (unsigned char)(v >> 8), (unsigned char)(v >> 16), (unsigned char)(v >> 24)};
    fwrite(b, 1, 4, stdout);
}

static void dump_ours(void) {
#define OURS(name, key, n) \
    for (int i = 0; i < (n); i++) put(n2m_lut_blob[N2M_##key##_OFF + i]);
    LEWINER_TABLES(OURS)
    for (int i = 0; i < 256; i++) put(n2m_classic_edge[i]);
    for (int i = 0; i < 4096; i++) put(n2m_classic_tri[i]);
}

#ifdef WITH_REFERENCE
static int compare_and_dump_ref(void) {
    int bad = 0;
#define CMP(name, key, n)                                                                           \
    if (sizeof(name) != (size_t)(n)) {                                                              \
        fprintf(stderr, "%s: %zu elements in the reference, %d expected\n", #name, sizeof(name), n); \
        bad++;                                                                                      \
    }                                                                                               \
    for (int i = 0; i < (n); i++) {                                                                 \
        const int r = ((const signed char *)name)[i], o = n2m_lut_blob[N2M_##key##_OFF + i];        \
        if (r != o) {                                                                               \
            fprintf(stderr, "%s[%d]: reference %d, packed %d\n", #name, i, r, o);                   \
            bad++;                                                                                  \
        }                                                                                           \
    }
    LEWINER_TABLES(CMP)
    for (int i = 0; i < 256; i++)
        if (edgeTable[i] != n2m_classic_edge[i]) {
            fprintf(stderr, "edgeTable[%d]: reference %d, packed %d\n", i, edgeTable[i], n2m_classic_edge[i]);
            bad++;
        }
    for (int i = 0; i < 4096; i++)
        if (triTable[i / 16][i % 16] != n2m_classic_tri[i]) {
            fprintf(stderr, "triTable[%d][%d]: reference %d, packed %d\n", i / 16, i % 16, triTable[i / 16][i % 16],
                    n2m_classic_tri[i]);
            bad++;
        }
#define REF(name, key, n) \
    for (int i = 0; i < (n); i++) put(((const signed char *)name)[i]);
    LEWINER_TABLES(REF)
    for (int i = 0; i < 256; i++) put(edgeTable[i]);
    for (int i = 0; i < 4096; i++) put(triTable[i / 16][i % 16]);
    return bad;
}
#endif

int main(int argc, char **argv) {
    if (argc == 2 && !strcmp(argv[1], "ours")) {
        dump_ours();
        return 0;
    }
#ifdef WITH_REFERENCE
    if (argc == 2 && !strcmp(argv[1], "ref")) return compare_and_dump_ref() ? 1 : 0;
#endif
    fprintf(stderr, "usage: table_check ours|ref\n");
    return 2;
}
