#!/usr/bin/env bash
# build_ref_gpu.sh -- the reference's own GPU code, built with nvcc for
# sm_103a (test and measurement infrastructure).
#
#   build_ref_gpu.sh --stage   copy the reference's translation units and
#                              headers from REF into oracle/_ref/gpu_src/
#                              (git-ignored; it travels to the GPU machine,
#                              where the reference tree does not exist) and
#                              generate kernel_functions_L4.cu there: the
#                              reference file with exactly the five commented
#                              lines of the L4 father walk of its GPU label
#                              kernel (kernel_functions.cu:739-743) re-enabled.
#   build_ref_gpu.sh --build   compile from oracle/_ref/gpu_src/ (nvcc, -O3,
#                              -arch sm_103a, as the reference's Zcompile.sh
#                              does for its own arch) into oracle/_ref/:
#                                G2H_ref               every unit unmodified,
#                                                      its own main (the G2H CLI)
#                                ref_gpu_harness_L4    the units with the L4 GPU
#                                                      kernel and ref_harness.cpp
#                                                      (REF_GPU_BUILD) as main
#
# REF names the reference tree; this recipe is the one place that knows its
# default location in the build container (/root/reference).  --stage exits
# 3 when the tree is absent; --build exits 3 when nothing was staged.
set -euo pipefail
HERE=$(cd "$(dirname "$0")" && pwd)
OUT="$HERE/_ref"
SRC="$OUT/gpu_src"
OBJ="$OUT/gpu_obj"
mode=${1:---build}

if [ "$mode" = "--stage" ]; then
  REF=${REF:-/root/reference}
  if [ ! -f "$REF/Graph_D.cuh" ] || [ ! -f "$REF/kernel_functions.cu" ]; then
    echo "build_ref_gpu.sh: reference tree not found at $REF (nothing to stage)" >&2
    exit 3
  fi
  mkdir -p "$SRC"
  for f in "$REF"/*.cu "$REF"/*.cuh; do
    cmp -s "$f" "$SRC/$(basename "$f")" 2>/dev/null || cp "$f" "$SRC/"
  done
  python3 - "$SRC/kernel_functions.cu" "$SRC/kernel_functions_L4.cu.tmp" <<'EOF'
import re, sys
src, dst = sys.argv[1], sys.argv[2]
lines = open(src, 'rb').read().split(b'\n')
assert b'L4 label' in lines[737], lines[737]           # line 738: the block's comment stays
for i in range(738, 743):                                # lines 739..743
    lines[i] = re.sub(rb'^(\s*)//', rb'\1', lines[i])
assert b'int fatherID = nodeID;' in lines[738] and b'atomicMin' in lines[741], lines[738:743]
open(dst, 'wb').write(b'\n'.join(lines))
EOF
  if cmp -s "$SRC/kernel_functions_L4.cu.tmp" "$SRC/kernel_functions_L4.cu"; then
    rm -f "$SRC/kernel_functions_L4.cu.tmp"
  else
    mv "$SRC/kernel_functions_L4.cu.tmp" "$SRC/kernel_functions_L4.cu"
  fi
  exit 0
fi

if [ "$mode" != "--build" ]; then
  echo "usage: build_ref_gpu.sh --stage | --build" >&2
  exit 2
fi
if [ ! -f "$SRC/Graph_D.cuh" ] || [ ! -f "$SRC/kernel_functions_L4.cu" ]; then
  echo "build_ref_gpu.sh: no staged reference sources in $SRC" >&2
  exit 3
fi
CUDA=${CUDA_HOME:-/usr/local/cuda}
NVCC="$CUDA/bin/nvcc"
FLAGS="-O3 -diag-suppress 20012 -w -gencode arch=compute_103a,code=sm_103a -I$SRC"
mkdir -p "$OBJ"
UNITS="Graph_Fundamental GraphPartition TreeStructure Traditional_H2H H2HConsturction Query tanslate Display kernel"
pids=()
compile() {  # src obj [extra flags]
  local src=$1 obj=$2
  shift 2
  if [ ! -f "$obj" ] || [ "$src" -nt "$obj" ]; then
    $NVCC $FLAGS "$@" -c "$src" -o "$obj.tmp$$" && mv "$obj.tmp$$" "$obj"
  fi
}
for u in $UNITS main kernel_functions kernel_functions_L4; do
  compile "$SRC/$u.cu" "$OBJ/$u.o" & pids+=($!)
done
compile "$HERE/ref_harness.cpp" "$OBJ/ref_gpu_harness.o" -x cu -DREF_GPU_BUILD & pids+=($!)
rc=0
for p in "${pids[@]}"; do wait "$p" || rc=1; done
[ $rc -eq 0 ] || { echo "build_ref_gpu.sh: compile failed" >&2; exit 1; }
COMMON=""
for u in $UNITS; do COMMON="$COMMON $OBJ/$u.o"; done
$NVCC -gencode arch=compute_103a,code=sm_103a -o "$OUT/G2H_ref" $COMMON "$OBJ/kernel_functions.o" "$OBJ/main.o"
$NVCC -gencode arch=compute_103a,code=sm_103a -o "$OUT/ref_gpu_harness_L4" $COMMON "$OBJ/kernel_functions_L4.o" \
  "$OBJ/ref_gpu_harness.o"
echo "built $OUT/G2H_ref $OUT/ref_gpu_harness_L4"
