#!/bin/bash
# Builds the reference's own GPU code (mfranzreb/ECL_wavelet, unmodified
# headers and sources) together with baseline/ref_driver.cu into
# baseline/_ref/ref_driver (asserts live, as the reference's default
# RelWithDebInfo build) and baseline/_ref/ref_driver_ndebug (-DNDEBUG).
#
# Where the reference checkout exists (EWT_REFERENCE_DIR, default
# /root/reference) its include/ and src/ trees are first copied to
# baseline/_ref/src/ (git-ignored, never committed), so that a machine
# without the checkout can build from that copy.  Flags follow the
# reference's CMakeLists.txt: C++20, -O3 -g, --default-stream per-thread,
# OpenMP, separable compilation; the GPU is sm_103a, and
# cuda13_compat.h supplies the four-argument cudaGraphAddDependencies
# that CUDA 13 dropped.  Exit 3: no sources to build from.
set -euo pipefail
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
OUT="$HERE/_ref"
SRC="$OUT/src"
REF="${EWT_REFERENCE_DIR:-/root/reference}"
if [ -d "$REF/include/ecl_wavelet" ] && [ -d "$REF/src/bitarray" ]; then
  mkdir -p "$SRC"
  chmod -R u+w "$SRC"
  rm -rf "$SRC/include" "$SRC/src"
  cp -rp "$REF/include" "$REF/src" "$SRC/"
  chmod -R u+w "$SRC"
  cp "$REF/LICENSE" "$SRC/" 2>/dev/null || true
fi
if [ ! -f "$SRC/include/ecl_wavelet/tree/wavelet_tree.cuh" ]; then
  echo "reference sources not found (neither $REF nor $SRC)" >&2
  exit 3
fi
NVCC="${CUDA_HOME:-/usr/local/cuda}/bin/nvcc"
[ -x "$NVCC" ] || NVCC=nvcc
FLAGS=(-std=c++20 -O3 -g -gencode arch=compute_103a,code=sm_103a
       --default-stream per-thread -rdc=true -Xcompiler -fopenmp
       --expt-relaxed-constexpr -include "$HERE/cuda13_compat.h"
       -I "$SRC/include")
UNITS=("$SRC/src/bitarray/bit_array.cu" "$SRC/src/bitarray/rank_select.cu"
       "$SRC/src/utils/utils.cu" "$HERE/ref_driver.cu")
build_variant() {  # $1 = output name, $2.. = extra flags
  local name="$1"; shift
  local obj="$OUT/obj_$name"
  mkdir -p "$obj"
  : > "$obj/build.log"
  local pids=() objs=()
  for u in "${UNITS[@]}"; do
    local o="$obj/$(basename "$u").o"
    objs+=("$o")
    "$NVCC" "${FLAGS[@]}" "$@" -c "$u" -o "$o" >> "$obj/build.log" 2>&1 &
    pids+=($!)
  done
  local failed=0
  for p in "${pids[@]}"; do wait "$p" || failed=1; done
  if [ "$failed" = 1 ]; then
    grep -i "error" "$obj/build.log" | head -20 >&2
    return 1
  fi
  "$NVCC" -gencode arch=compute_103a,code=sm_103a -rdc=true "${objs[@]}" \
    -o "$OUT/$name" -lgomp
}
# up to date: both binaries newer than every source, the driver and the shim
newest=$(find "$SRC/include" "$SRC/src" "$HERE/ref_driver.cu" "$HERE/cuda13_compat.h" \
         "$HERE/build_ref.sh" -type f -printf '%T@\n' | sort -n | tail -1)
fresh=1
for b in "$OUT/ref_driver" "$OUT/ref_driver_ndebug"; do
  if [ ! -x "$b" ] || [ "$(stat -c %Y "$b")" -lt "${newest%.*}" ]; then fresh=0; fi
done
if [ "$fresh" = 1 ]; then
  echo "up to date: $OUT/ref_driver and $OUT/ref_driver_ndebug"
  exit 0
fi
build_variant ref_driver &
P1=$!
build_variant ref_driver_ndebug -DNDEBUG &
P2=$!
wait $P1
wait $P2
echo "built $OUT/ref_driver and $OUT/ref_driver_ndebug"
