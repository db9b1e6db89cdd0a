#!/bin/sh
# Build the reference nii2mesh C path from its own, unmodified sources into
# oracle/_ref/ (git-ignored).  Used only to pin the oracle restatement and to
# generate the golden fixtures; never shipped, never called by the product.
#   libn2m_ref_lewiner.so : meshify + Lewiner MarchingCubes.c   (`make lewiner`)
#   libn2m_ref_classic.so : meshify + oldcubes.c                (`make` default)
#   mctest                : MarchingCubes.c -DMC_SELF_TEST       (self-test)
#   libn2m_ref_cli.so     : the nii2mesh program with its main() renamed, for
#                           load_nii (NIfTI voxel cast fixtures)
#   nii2mesh, nii2mesh_classic : the nii2mesh program itself (`make lewiner`
#                           and the default `make` build), for whole-program
#                           known answers
# -ffp-contract=off and -fsigned-char make an aarch64 build produce the same
# bits as the x86-64 one.  Usage: oracle/build_ref.sh <reference-src-dir>
set -e
[ $# -ge 1 ] || { echo "usage: $0 <reference-src-dir>" >&2; exit 2; }
SRC=$1
HERE=$(cd "$(dirname "$0")" && pwd)
OUT="$HERE/_ref"
[ -f "$SRC/meshify.c" ] || { echo "reference sources not found at $SRC" >&2; exit 1; }
mkdir -p "$OUT"
CF="-O2 -fPIC -ffp-contract=off -fsigned-char -DNII2MESH -w"
COMMON="$SRC/isolevel.c $SRC/meshify.c $SRC/quadric.c $SRC/bwlabel.c $SRC/radixsort.c"
ZL=""
if printf '#include <zlib.h>\nint main(void){return 0;}\n' | cc -x c - -lz -o /dev/null 2>/dev/null; then
  ZL="-DHAVE_ZLIB -lz"
fi
cc $CF -shared -o "$OUT/libn2m_ref_lewiner.so" $COMMON "$SRC/MarchingCubes.c" $ZL -lm
cc $CF -shared -DUSE_CLASSIC_CUBES -o "$OUT/libn2m_ref_classic.so" $COMMON "$SRC/oldcubes.c" $ZL -lm
cc -O2 -ffp-contract=off -fsigned-char -w -DMC_SELF_TEST -o "$OUT/mctest" "$SRC/MarchingCubes.c" -lm
cc $CF -shared -DHAVE_FORMATS -Dmain=n2m_ref_cli_main -o "$OUT/libn2m_ref_cli.so" $COMMON "$SRC/MarchingCubes.c" \
   "$SRC/nii2mesh.c" "$SRC/base64.c" $ZL -lm
PF="-O2 -ffp-contract=off -fsigned-char -DNII2MESH -DHAVE_FORMATS -w"
cc $PF -o "$OUT/nii2mesh" $COMMON "$SRC/MarchingCubes.c" "$SRC/nii2mesh.c" "$SRC/base64.c" $ZL -lm
cc $PF -DUSE_CLASSIC_CUBES -o "$OUT/nii2mesh_classic" $COMMON "$SRC/oldcubes.c" "$SRC/nii2mesh.c" "$SRC/base64.c" $ZL -lm
echo "built $OUT"
