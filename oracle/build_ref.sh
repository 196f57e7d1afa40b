#!/usr/bin/env bash
# Build the reference's own CUDA tissue solver (the LiverCudaSim plugin) as a Linux shared library,
# oracle/_ref/libLiverCudaSim.so, for sm_103a.  Test infrastructure: the GPU parity tests drive it
# through the same LCS_* harness as libgbtissue.so to pin the CPU oracle against the reference.
#
#   stage:  when REFERENCE_ROOT names the reference checkout, copy the plugin's native sources
#           (unmodified) into the git-ignored oracle/_ref/src, so they travel to a GPU machine with
#           the working tree (REFERENCE_ROOT=<reference checkout> bash oracle/build_ref.sh stage);
#   build:  compile oracle/_ref/src with nvcc (-rdc) and g++ directly, no CMake.  The only shims are
#           a force-included overload for the CUDA 13 cudaGraphAddNode signature (oracle/ref_shim.h)
#           and __declspec(x) defined away for plugin_api.cpp.
set -euo pipefail
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
REF_TREE="${REFERENCE_ROOT:+$REFERENCE_ROOT/endoscopic_tissue/native/vendor}"
OUT="$HERE/_ref"
SRC="$OUT/src"
mode="${1:-all}"

if [[ "$mode" == "all" || "$mode" == "stage" ]]; then
  if [[ -n "$REF_TREE" && -d "$REF_TREE" ]]; then
    rm -rf "$SRC"
    mkdir -p "$SRC"
    cp -r "$REF_TREE/cuda" "$REF_TREE/src" "$SRC/"
  fi
fi
[[ "$mode" == "stage" ]] && exit 0
if [[ ! -d "$SRC/cuda" ]]; then
  echo "reference sources not staged (oracle/_ref/src missing)" >&2
  exit 3
fi
NVCC="${NVCC:-nvcc}"
FLAGS=(-gencode arch=compute_103a,code=sm_103a -O3 -std=c++17 -rdc=true -Xcompiler -fPIC -include "$HERE/ref_shim.h" -I"$SRC/cuda" -w)
mkdir -p "$OUT/obj"
pids=()
for f in physics cut dc_recon haptics xpbd/xpbd_solver; do
  "$NVCC" "${FLAGS[@]}" -c "$SRC/cuda/$f.cu" -o "$OUT/obj/$(basename $f).o" &
  pids+=($!)
done
g++ -std=c++17 -O2 -fPIC -w "-D__declspec(x)=" -I"$SRC/cuda" -I/usr/local/cuda/include -c "$SRC/src/plugin_api.cpp" -o "$OUT/obj/plugin_api.o"
for p in "${pids[@]}"; do wait "$p"; done
"$NVCC" -gencode arch=compute_103a,code=sm_103a -shared -o "$OUT/libLiverCudaSim.so" "$OUT"/obj/*.o
echo "built $OUT/libLiverCudaSim.so"
