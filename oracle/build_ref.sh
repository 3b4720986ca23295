#!/bin/sh
# Compile the reference's CUDA kernel, unmodified, from its own source file into a
# cubin for sm_103a.  Test infrastructure: the cubin is the parity pin that
# oracle/ref_runner.cu loads on the GPU.  Output goes to oracle/_ref/ only.
#
#   REF   the reference checkout (also NBODY_REFERENCE_DIR; default: a checkout
#         named "reference" beside this repository)
#
# Flags: -use_fast_math is the reference's release flag (src/CMakeLists.txt:51);
# DISABLE_GL is the no_render build's define (src/CMakeLists.txt:41).  The
# reference sets no architecture; sm_103a is the GPU it runs on here.
set -e
HERE=$(cd "$(dirname "$0")" && pwd)
REF=${REF:-${NBODY_REFERENCE_DIR:-$HERE/../../reference}}
OUT="$HERE/_ref"
if [ ! -f "$REF/src/simulator.cu" ]; then
  echo "build_ref.sh: $REF/src/simulator.cu not found; reference kernel not built" >&2
  exit 0
fi
mkdir -p "$OUT"
nvcc -cubin -gencode arch=compute_103a,code=sm_103a -use_fast_math -DDISABLE_GL \
  -I"$REF/src" "$REF/src/simulator.cu" -o "$OUT/simulator_sm103a.cubin" -Xptxas -v \
  > "$OUT/ptxas.log" 2>&1
echo "build_ref.sh: wrote $OUT/simulator_sm103a.cubin"
