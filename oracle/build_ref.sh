#!/bin/sh
# Compiles the reference's own dense-path graph store, refresh and push into
# oracle/_ref/libtsvd_ref.so, and its frPCA into oracle/_ref/libtsvd_ref_frpca.so
# (test infrastructure and the CPU reference arm of bench.py: they pin the CPU
# oracle and time the reference on the host cores; nothing in the product
# uses them).
#
# Step 1 (where the reference sources are present, TSVD_REFERENCE_DIR or the
# default below): stage the pieces that compile without MKL, Eigen, Boost or
# emhash into oracle/_ref/src/ (git-ignored, never committed):
#   * from Code/ppr_computation_store_dynamic.h, by line range, the six
#     refresh/push functions and the four log-transform functions (the rest
#     of that header needs the missing libraries, so the drivers stay
#     unbuildable);
#   * Code/Graph_dynamic.h and Code/my_queue.h, included by those functions;
#   * Code/frpca.c and Code/matrix_vector_functions_intel_mkl{,_ext}.{c,h}.
# Step 2 (wherever oracle/_ref/src/ exists, e.g. on a machine without the
# reference sources that received this directory): compile
#   * ref_shim.cpp (+ the staged functions) -> libtsvd_ref.so;
#   * the staged frpca.c and MKL helper files against the MKL stand-in in
#     oracle/mkl_shim/ (dense BLAS/LAPACKE from the OpenBLAS bundled with
#     scipy; sparse products and random streams in mkl_shim.c), wrapped by
#     oracle/ref_frpca_shim.c -> libtsvd_ref_frpca.so.
# Outputs go only to oracle/_ref/.
set -e
HERE=$(cd "$(dirname "$0")" && pwd)
REF=${TSVD_REFERENCE_DIR:-/root/reference/Code}
OUT="$HERE/_ref"
SRC="$OUT/src"

if [ -f "$REF/ppr_computation_store_dynamic.h" ]; then
  mkdir -p "$SRC"
  H="$REF/ppr_computation_store_dynamic.h"
  INC="$SRC/ref_functions.inc"
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
  for f in Graph_dynamic.h my_queue.h frpca.c matrix_vector_functions_intel_mkl.c \
           matrix_vector_functions_intel_mkl.h matrix_vector_functions_intel_mkl_ext.c \
           matrix_vector_functions_intel_mkl_ext.h; do
    [ -f "$REF/$f" ] && cp "$REF/$f" "$SRC/$f"
  done
fi

if [ ! -f "$SRC/ref_functions.inc" ]; then
  echo "reference sources not found at $REF and nothing staged in $SRC; skipping oracle/_ref" >&2
  exit 0
fi
${CXX:-g++} -O2 -ffp-contract=off -fPIC -shared -std=c++14 -pthread -w \
  -I"$SRC" "$HERE/ref_shim.cpp" -o "$OUT/libtsvd_ref.so"
echo "built $OUT/libtsvd_ref.so"

OB=$(${PYTHON:-python3} -c "import scipy, os, glob; print((glob.glob(os.path.join(os.path.dirname(scipy.__file__), '..', 'scipy.libs', 'libscipy_openblas-*.so')) + [''])[0])")
if [ -z "$OB" ] || [ ! -f "$SRC/frpca.c" ]; then
  echo "scipy OpenBLAS or frpca.c not found; skipping oracle/_ref/libtsvd_ref_frpca.so" >&2
  exit 0
fi
${CC:-gcc} -O2 -ffp-contract=off -fPIC -shared -std=gnu99 -pthread -w \
  -I"$HERE/mkl_shim" -I"$SRC" \
  "$SRC/frpca.c" "$SRC/matrix_vector_functions_intel_mkl.c" \
  "$SRC/matrix_vector_functions_intel_mkl_ext.c" \
  "$HERE/mkl_shim/mkl_shim.c" "$HERE/ref_frpca_shim.c" \
  "$OB" -Wl,-rpath,"$(dirname "$OB")" -lm -o "$OUT/libtsvd_ref_frpca.so"
echo "built $OUT/libtsvd_ref_frpca.so"
