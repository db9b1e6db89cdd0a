#!/usr/bin/env python3
"""Generate ``mc_tables.h`` — the marching-cubes lookup data in this project's
packed layout.

The Lewiner MC33 case/tiling/test tables (``src/LookUpTable.h``) and Bourke's
classic ``edgeTable``/``triTable`` (``src/oldcubes.c:87-400``) are *data* that
must be identical bit-for-bit to the reference's, otherwise cube topology
differs.  This script reads the reference's tables once, checks their shapes,
and re-encodes every table into a single flat ``int8`` blob plus per-table
offset/shape macros, which is the layout the CPU oracle and the CUDA kernels
both index.  The generated header is committed; the script only needs the
reference tree when the tables are regenerated.

Usage: python gen_mc_tables.py <reference-src-dir> <out-header>
"""
import re
import sys
from pathlib import Path

# (name in the reference, expected shape) — every table process_cube /
# test_interior index (src/MarchingCubes.c:458-795, :301-453).
LEWINER = [
    ("cases", (256, 2)), ("tiling1", (16, 3)), ("tiling2", (24, 6)),
    ("test3", (24,)), ("tiling3_1", (24, 6)), ("tiling3_2", (24, 12)),
    ("test4", (8,)), ("tiling4_1", (8, 6)), ("tiling4_2", (8, 18)),
    ("tiling5", (48, 9)), ("test6", (48, 3)), ("tiling6_1_1", (48, 9)),
    ("tiling6_1_2", (48, 27)), ("tiling6_2", (48, 15)), ("test7", (16, 5)),
    ("tiling7_1", (16, 9)), ("tiling7_2", (16, 3, 15)), ("tiling7_3", (16, 3, 27)),
    ("tiling7_4_1", (16, 15)), ("tiling7_4_2", (16, 27)), ("tiling8", (6, 6)),
    ("tiling9", (8, 12)), ("test10", (6, 3)), ("tiling10_1_1", (6, 12)),
    ("tiling10_1_1_", (6, 12)), ("tiling10_1_2", (6, 24)), ("tiling10_2", (6, 24)),
    ("tiling10_2_", (6, 24)), ("tiling11", (12, 12)), ("test12", (24, 4)),
    ("tiling12_1_1", (24, 12)), ("tiling12_1_1_", (24, 12)), ("tiling12_1_2", (24, 24)),
    ("tiling12_2", (24, 24)), ("tiling12_2_", (24, 24)), ("test13", (2, 7)),
    ("subconfig13", (64,)), ("tiling13_1", (2, 12)), ("tiling13_1_", (2, 12)),
    ("tiling13_2", (2, 6, 18)), ("tiling13_2_", (2, 6, 18)), ("tiling13_3", (2, 12, 30)),
    ("tiling13_3_", (2, 12, 30)), ("tiling13_4", (2, 4, 36)), ("tiling13_5_1", (2, 4, 18)),
    ("tiling13_5_2", (2, 4, 30)), ("tiling14", (12, 12)), ("casesClassic", (256, 16)),
]


def strip_comments(src):
    src = re.sub(r"/\*.*?\*/", " ", src, flags=re.S)
    return re.sub(r"//[^\n]*", " ", src)


def table_values(src, name):
    m = re.search(r"\b" + re.escape(name) + r"\s*((?:\[\s*\d+\s*\])+)\s*=\s*\{", src)
    if not m:
        raise SystemExit(f"table {name} not found")
    dims = tuple(int(d) for d in re.findall(r"\d+", m.group(1)))
    depth, i = 1, m.end()
    while depth:
        c = src[i]
        depth += (c == "{") - (c == "}")
        i += 1
    body = src[m.end():i - 1]
    vals = [int(v, 0) for v in re.findall(r"-?(?:0x[0-9a-fA-F]+|\d+)", body)]
    n = 1
    for d in dims:
        n *= d
    if len(vals) != n:
        raise SystemExit(f"table {name}: {len(vals)} values for shape {dims}")
    return dims, vals


def main():
    ref, out = Path(sys.argv[1]), Path(sys.argv[2])
    lut = strip_comments((ref / "LookUpTable.h").read_text())
    old = strip_comments((ref / "oldcubes.c").read_text())
    blob, lines = [], []
    for name, shape in LEWINER:
        dims, vals = table_values(lut, name)
        if dims != shape:
            raise SystemExit(f"table {name}: shape {dims} != {shape}")
        key = name.upper().rstrip("_") + ("_B" if name.endswith("_") else "")
        lines.append(f"#define N2M_{key}_OFF {len(blob)}")
        # row strides so that element [a][b][c] = blob[OFF + a*S0 + b*S1 + c]
        strides = []
        for k in range(len(dims)):
            s = 1
            for d in dims[k + 1:]:
                s *= d
            strides.append(s)
        for k, s in enumerate(strides[:-1]):
            lines.append(f"#define N2M_{key}_S{k} {s}")
        blob.extend(vals)
    assert all(-128 <= v <= 127 for v in blob)
    _, edge = table_values(old, "edgeTable")
    _, tri = table_values(old, "triTable")
    assert len(edge) == 256 and len(tri) == 4096
    with out.open("w") as f:
        f.write("/* GENERATED by gen_mc_tables.py — do not edit.\n"
                " * Marching-cubes lookup data in this project's packed layout:\n"
                " *  - Lewiner et al. MC33 case, test and tiling tables (one int8 blob,\n"
                " *    element [a][b][c] of table T at N2M_T_OFF + a*N2M_T_S0 + b*N2M_T_S1 + c);\n"
                " *  - Bourke's classic edge mask and triangle table.\n"
                " * The values are the published tables, identical to the ones the reference\n"
                " * indexes (src/LookUpTable.h, src/oldcubes.c:87-400); only the layout is ours. */\n")
        f.write("#ifndef N2M_MC_TABLES_H\n#define N2M_MC_TABLES_H\n\n")
        f.write("\n".join(lines) + "\n")
        f.write(f"#define N2M_LUT_BLOB_SIZE {len(blob)}\n\n")

        def emit(ctype, name, vals, per=24):
            # initializer as a macro so host code and __device__ arrays share it
            f.write(f"#define {name.upper()}_INIT {{ \\\n")
            for i in range(0, len(vals), per):
                f.write("  " + ",".join(str(v) for v in vals[i:i + per]) + ", \\\n")
            f.write("}\n")
            f.write(f"static const {ctype} {name}[{len(vals)}] = {name.upper()}_INIT;\n\n")
        emit("signed char", "n2m_lut_blob", blob)
        emit("unsigned short", "n2m_classic_edge", edge, 16)
        emit("signed char", "n2m_classic_tri", tri, 16)
        f.write("#endif /* N2M_MC_TABLES_H */\n")
    print(f"wrote {out}: blob {len(blob)} bytes")


if __name__ == "__main__":
    main()
