#!/bin/sh
# Compiles the LDA_X + LDA_C_PW subset of the reference tree's vendored
# libxc 6.2.2 (ExLib/libxc/libxc-6.2.2/src) into oracle/_ref/libxc_lda.so.
# The reference sources are compiled where they lie; only the small headers,
# the trimmed functional table and stubs in oracle/libxc_subset are ours.
# lda.c includes "funcs_lda.c" relative to its own directory, so it is staged
# through a symlink next to the trimmed table.  Output goes to oracle/_ref only.
#
# The DEReK tree is taken from the first argument or DEREK_REFERENCE; a tree
# named that way must be a DEReK checkout (Source/electronic.f90 and the
# vendored libxc present), else this fails.  With neither given, the build
# container's mount point below is tried, and the checker is skipped (exit 0)
# when no DEReK tree is there; a directory there that is not one also fails.
set -e
HERE=$(cd "$(dirname "$0")" && pwd)
REF=${1:-$DEREK_REFERENCE}
EXPLICIT=1
if [ -z "$REF" ]; then
  REF=/root/reference
  EXPLICIT=0
  if [ ! -e "$REF" ]; then
    echo "no DEReK tree (set DEREK_REFERENCE); skipping the libxc checker" >&2
    exit 0
  fi
fi
SRC=$REF/ExLib/libxc/libxc-6.2.2/src
OUT=$HERE/_ref
if [ ! -f "$REF/Source/electronic.f90" ] || [ ! -f "$SRC/lda_c_pw.c" ]; then
  echo "$REF is not a DEReK tree with libxc 6.2.2 vendored (explicit=$EXPLICIT)" >&2
  exit 1
fi
mkdir -p "$OUT/stage"
cp "$HERE"/libxc_subset/funcs_lda.c "$HERE"/libxc_subset/funcs_hyb_lda.c "$OUT/stage/"
ln -sf "$SRC/lda.c" "$OUT/stage/lda.c"
${CC:-gcc} -O2 -fPIC -shared -w \
  -I"$HERE/libxc_subset" -I"$SRC" \
  -o "$OUT/libxc_lda.so" \
  "$HERE/libxc_subset/ref_lda.c" "$HERE/libxc_subset/stubs.c" \
  "$OUT/stage/lda.c" \
  "$SRC/functionals.c" "$SRC/func_info.c" "$SRC/lda_x.c" "$SRC/lda_c_pw.c" \
  "$SRC/references.c" "$SRC/util.c" "$SRC/mix_func.c" "$SRC/version.c" \
  "$SRC/func_reference.c" -lm
echo "built $OUT/libxc_lda.so"
