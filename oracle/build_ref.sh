#!/bin/sh
# Compiles the reference's own dense-path graph store, refresh and push from
# the reference sources where they lie into oracle/_ref/libtsvd_ref.so (test
# infrastructure: it pins the CPU oracle; nothing in the product uses it).
#
# The six functions are taken from Code/ppr_computation_store_dynamic.h by line
# range; the rest of that header needs MKL, Eigen, Boost and emhash, none of
# which exist here, so frpca.c, the log/SVD code and the drivers stay
# unbuildable. Outputs go only to oracle/_ref/.
set -e
HERE=$(cd "$(dirname "$0")" && pwd)
REF=${TSVD_REFERENCE_DIR:-/root/reference/Code}
OUT="$HERE/_ref"
if [ ! -f "$REF/ppr_computation_store_dynamic.h" ]; then
  echo "reference sources not found at $REF; skipping oracle/_ref" >&2
  exit 0
fi
mkdir -p "$OUT"
H="$REF/ppr_computation_store_dynamic.h"
INC="$OUT/ref_functions.inc"
: > "$INC"
for spec in \
  1394:1498:nodegree_DenseDynamicForwardPush \
  2035:2121:nodegree_DenseUndirected_Refresh_PPR_initialization \
  2945:3030:nodegree_DenseDirectedDynamicForwardPush \
  3356:3437:nodegree_DenseDirectedDynamicForwardPushTranspose \
  3811:3898:nodegree_DenseDirected_Refresh_PPR_initialization \
  4133:4228:nodegree_DenseDirected_Refresh_PPR_initialization_Transpose; do
  a=${spec%%:*}; rest=${spec#*:}; b=${rest%%:*}; name=${rest#*:}
  first=$(sed -n "${a}p" "$H")
  case "$first" in
    "void $name("*) ;;
    *) echo "unexpected line $a in $H (wanted $name)" >&2; exit 1 ;;
  esac
  [ "$(sed -n "${b}p" "$H")" = "}" ] || { echo "line $b of $H is not the end of $name" >&2; exit 1; }
  sed -n "${a},${b}p" "$H" >> "$INC"
done
${CXX:-g++} -O2 -ffp-contract=off -fPIC -shared -std=c++14 -w \
  -I"$REF" -I"$OUT" "$HERE/ref_shim.cpp" -o "$OUT/libtsvd_ref.so"
echo "built $OUT/libtsvd_ref.so"
