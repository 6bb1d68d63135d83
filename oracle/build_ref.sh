#!/usr/bin/env bash
# build_ref.sh -- CPU-only build of the reference's own translation units
# (test infrastructure).  Compiles the reference sources where they lie (REF;
# this recipe is the one place that knows the default location of the
# reference tree, /root/reference, in the build container) with g++ and Thrust's CPP device system, plus the
# harness and stubs in this directory, into oracle/_ref/ (git-ignored):
#
#   oracle/_ref/ref_harness_L3   the reference as shipped (L3 labels)
#   oracle/_ref/ref_harness_L4   the same with the commented L4 father-walk
#                                block of makeH2HLabel_noHub_multiThred
#                                (H2HConsturction.cu:851-857) re-enabled; the
#                                patched translation unit is generated into
#                                oracle/_ref/src/ and never committed.
#
# The reference's own build script (Zcompile.sh) is not used.
set -euo pipefail
REF=${REF:-/root/reference}
HERE=$(cd "$(dirname "$0")" && pwd)
OUT="$HERE/_ref"
CUDA=${CUDA_HOME:-/usr/local/cuda}
if [ ! -f "$REF/Graph_D.cuh" ]; then
  echo "build_ref.sh: reference tree not found at $REF (nothing to build)" >&2
  exit 3
fi
mkdir -p "$OUT/src" "$OUT/obj"
CXX=${CXX:-g++}
FLAGS="-x c++ -std=c++17 -O2 -w -I$CUDA/include -I$CUDA/include/cccl -I$REF -I$HERE -DTHRUST_DEVICE_SYSTEM=THRUST_DEVICE_SYSTEM_CPP"

# L4 variant: uncomment exactly the seven lines of the L4 block.
python3 - "$REF/H2HConsturction.cu" "$OUT/src/H2HConsturction_L4.cu" <<'EOF'
import sys, re
src, dst = sys.argv[1], sys.argv[2]
lines = open(src, 'rb').read().split(b'\n')
blk = range(850, 857)  # 0-based indices of lines 851..857
assert b'L4 label' in lines[849], lines[849]
for i in blk:
    lines[i] = re.sub(rb'^(\s*)//', rb'\1', lines[i])
assert b'fatherID = (int64_t)father[fatherID]' in lines[852]
open(dst, 'wb').write(b'\n'.join(lines))
EOF

UNITS="Graph_Fundamental GraphPartition TreeStructure Traditional_H2H Query tanslate Display"
pids=()
for u in $UNITS; do
  $CXX $FLAGS -c "$REF/$u.cu" -o "$OUT/obj/$u.o" & pids+=($!)
done
$CXX $FLAGS -c "$REF/H2HConsturction.cu" -o "$OUT/obj/H2HConsturction_L3.o" & pids+=($!)
$CXX $FLAGS -c "$OUT/src/H2HConsturction_L4.cu" -o "$OUT/obj/H2HConsturction_L4.o" & pids+=($!)
$CXX -std=c++17 -O2 -w -I$CUDA/include -I$CUDA/include/cccl -I$REF -I$HERE \
  -DTHRUST_DEVICE_SYSTEM=THRUST_DEVICE_SYSTEM_CPP -c "$HERE/ref_stubs.cpp" -o "$OUT/obj/ref_stubs.o" & pids+=($!)
$CXX -std=c++17 -O2 -w -I$CUDA/include -I$CUDA/include/cccl -I$REF -I$HERE \
  -DTHRUST_DEVICE_SYSTEM=THRUST_DEVICE_SYSTEM_CPP -c "$HERE/ref_harness.cpp" -o "$OUT/obj/ref_harness.o" & pids+=($!)
gcc -std=c11 -O2 -c "$HERE/h2h_oracle.c" -o "$OUT/obj/h2h_oracle.o" & pids+=($!)
for p in "${pids[@]}"; do wait "$p"; done
OBJS=""
for u in $UNITS; do OBJS="$OBJS $OUT/obj/$u.o"; done
COMMON="$OBJS $OUT/obj/ref_stubs.o $OUT/obj/ref_harness.o $OUT/obj/h2h_oracle.o -lpthread"
$CXX -o "$OUT/ref_harness_L3" $COMMON "$OUT/obj/H2HConsturction_L3.o"
$CXX -o "$OUT/ref_harness_L4" $COMMON "$OUT/obj/H2HConsturction_L4.o"
echo "built $OUT/ref_harness_L3 $OUT/ref_harness_L4"
