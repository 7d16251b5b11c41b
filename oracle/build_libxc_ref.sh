#!/bin/sh
# Compiles the LDA_X + LDA_C_PW subset of the reference tree's vendored
# libxc 6.2.2 (ExLib/libxc/libxc-6.2.2/src) into oracle/_ref/libxc_lda.so.
# The reference sources are compiled where they lie; only the small headers,
# the trimmed functional table and stubs in oracle/libxc_subset are ours.
# lda.c includes "funcs_lda.c" relative to its own directory, so it is staged
# through a symlink next to the trimmed table.  Output goes to oracle/_ref only.
set -e
HERE=$(cd "$(dirname "$0")" && pwd)
REF=${DEREK_REFERENCE:-/root/reference}
SRC=$REF/ExLib/libxc/libxc-6.2.2/src
OUT=$HERE/_ref
if [ ! -d "$SRC" ]; then
  echo "libxc sources not found at $SRC; skipping the libxc checker" >&2
  exit 0
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
