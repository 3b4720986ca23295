#!/bin/sh
# Parity pins built from the reference's own, unmodified sources.  Test
# infrastructure; output goes to oracle/_ref/ only.
#
#   _ref/simulator_sm103a.cubin   the reference kernel (src/simulator.cu) for
#                                 sm_103a, loaded on the GPU by oracle/ref_runner.cu
#   _ref/ref_ic_dump              the reference's DiskGalaxySimulator constructor
#                                 (src/simulator.cu + src/sim_param.cpp) linked with
#                                 oracle/ref_ic_host.cpp in place of the CUDA runtime,
#                                 so that it writes the reference's own initial state
#                                 on a host without a GPU (oracle/ref_ic_dump.cpp)
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

# The initial-state dump: the reference's host code as its CMake build compiles it
# (nvcc for simulator.cu, the C++ compiler for sim_param.cpp), no CUDA runtime.
OBJ="$OUT/ic_obj"
mkdir -p "$OBJ"
nvcc -c -gencode arch=compute_103a,code=sm_103a -use_fast_math -DDISABLE_GL -I"$REF/src" \
  "$REF/src/simulator.cu" -o "$OBJ/simulator.o"
g++ -c -O2 -DDISABLE_GL -I"$REF/src" -I"${CUDA_HOME:-/usr/local/cuda}/include" \
  "$REF/src/sim_param.cpp" -o "$OBJ/sim_param.o"
g++ -c -O2 -I"$REF/src" -I"${CUDA_HOME:-/usr/local/cuda}/include" "$HERE/ref_ic_dump.cpp" \
  -o "$OBJ/ref_ic_dump.o"
g++ -c -O2 -I"${CUDA_HOME:-/usr/local/cuda}/include" "$HERE/ref_ic_host.cpp" \
  -o "$OBJ/ref_ic_host.o"
g++ -o "$OUT/ref_ic_dump" "$OBJ/ref_ic_dump.o" "$OBJ/simulator.o" "$OBJ/sim_param.o" \
  "$OBJ/ref_ic_host.o" -lm
echo "build_ref.sh: wrote $OUT/ref_ic_dump"
