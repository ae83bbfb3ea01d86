#!/bin/sh
# Compiles the reference's own dense-path graph store, refresh and push from
# the reference sources where they lie into oracle/_ref/libtsvd_ref.so (test
# infrastructure: it pins the CPU oracle; nothing in the product uses it).
#
# The six refresh/push functions and the four log-transform functions are taken
# from Code/ppr_computation_store_dynamic.h by line range; the rest of that
# header needs MKL, Eigen, Boost and emhash, none of which exist here, so the
# drivers stay unbuildable.
#
# Second library, oracle/_ref/libtsvd_ref_frpca.so: the reference's frpca.c and
# matrix_vector_functions_intel_mkl{,_ext}.c compiled unchanged against the MKL
# stand-in in oracle/mkl_shim/ (dense BLAS/LAPACKE from the OpenBLAS bundled
# with scipy; sparse products and random streams in mkl_shim.c), wrapped by
# oracle/ref_frpca_shim.c. Outputs go only to oracle/_ref/.
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
  4133:4228:nodegree_DenseDirected_Refresh_PPR_initialization_Transpose \
  2527:2561:Log_sparse_matrix_entries \
  2598:2638:Log_sparse_matrix_entries_LP \
  2649:2732:Log_sparse_matrix_entries_with_norm_computation \
  2742:2826:Log_sparse_matrix_entries_with_norm_computation_LP; do
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

OB=$(${PYTHON:-python3} -c "import scipy, os, glob; print((glob.glob(os.path.join(os.path.dirname(scipy.__file__), '..', 'scipy.libs', 'libscipy_openblas-*.so')) + [''])[0])")
if [ -z "$OB" ] || [ ! -f "$REF/frpca.c" ]; then
  echo "scipy OpenBLAS or frpca.c not found; skipping oracle/_ref/libtsvd_ref_frpca.so" >&2
  exit 0
fi
${CC:-gcc} -O2 -ffp-contract=off -fPIC -shared -std=gnu99 -w \
  -I"$HERE/mkl_shim" -I"$REF" \
  "$REF/frpca.c" "$REF/matrix_vector_functions_intel_mkl.c" \
  "$REF/matrix_vector_functions_intel_mkl_ext.c" \
  "$HERE/mkl_shim/mkl_shim.c" "$HERE/ref_frpca_shim.c" \
  "$OB" -Wl,-rpath,"$(dirname "$OB")" -lm -o "$OUT/libtsvd_ref_frpca.so"
echo "built $OUT/libtsvd_ref_frpca.so"
