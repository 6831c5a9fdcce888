#!/usr/bin/env bash
# build_ref.sh -- compile the reference's own mixture code for the host
# (TEST INFRASTRUCTURE ONLY; runs only where the reference checkout exists).
#
# Output: oracle/_ref/libnmgref.so (git-ignored). Everything this script
# writes goes under oracle/_ref/. The reference sources are compiled where
# they lie; the build directory holds a symlink overlay of the reference's
# src/ in which five headers are replaced by copies with host/CUDA-13 fixes
# that do not touch the guiding arithmetic:
#   util/check.h        MSVC-only "..."##LOG token paste -> plain concatenation
#   core/device/memory.h  cudaMemPrefetchAsync changed signature in CUDA 13
#                         (call replaced by cudaSuccess; prefetch is unused here)
#   core/vulkan/cuvk.h  enum cast for the Vulkan handle type; computeMode was
#                       removed from cudaDeviceProp in CUDA 13
#   core/mesh.h, core/scenegraph.h  Eigen Affine3f copy-init rejected by g++ 13
#                                   (default-initialised instead; unused here)
# plus soac-generated SOA headers and a config.h written from config.in.h.
# tiny-cuda-nn's kernel headers get host-callable copies of their own
# (tcnn_host_headers.py) for oracle/ref_tcnn_kernels.cu.
# krr::Primes (a device table of util/tables.cpp that the host pass cannot
# define) gets a host stub; the Halton sampler that reads it is not used.
set -euo pipefail
REF=${NMG_REFERENCE:-/root/reference}
HERE=$(cd "$(dirname "$0")" && pwd)
OUT=$HERE/_ref
B=$OUT/build
SRC=$REF/src
if [ ! -d "$SRC/render/guided" ]; then
  echo "reference checkout not found at $REF (set NMG_REFERENCE)" >&2
  exit 3
fi
if [ "${1:-}" = "--check" ]; then exit 0; fi
mkdir -p "$B/gen/render/wavefront" "$B/gen/render/guided"

# 1. soac (SOA code generator) and the two generated headers
g++ -std=c++17 -O1 -include cstring "$SRC/backend/src/util/soac.cpp" -o "$B/soac"
"$B/soac" "$SRC/backend/src/render/wavefront/workitem.soa" > "$B/gen/render/wavefront/workitem_soa.h"
"$B/soac" "$SRC/render/guided/guideditem.soa" > "$B/gen/render/guided/guideditem_soa.h"

# 2. config.h from config.in.h
sed -e 's/#cmakedefine01[[:space:]]*KRR_PLATFORM_WINDOWS/#define KRR_PLATFORM_WINDOWS 0/' \
    -e 's/#cmakedefine01[[:space:]]*KRR_PLATFORM_LINUX/#define KRR_PLATFORM_LINUX 1/' \
    -e 's/#cmakedefine01[[:space:]]*KRR_PLATFORM_UNKNOWN/#define KRR_PLATFORM_UNKNOWN 0/' \
    -e 's/#cmakedefine01[[:space:]]*KRR_BUILD_STARLIGHT/#define KRR_BUILD_STARLIGHT 0/' \
    -e 's/\${[A-Z_]*}//g' "$SRC/backend/src/core/config.in.h" > "$B/gen/config.h"

# 3. symlink overlay + patched copies
rm -rf "$B/overlay"
cp -rs "$SRC" "$B/overlay"
patch_copy() {  # patch_copy <path under src/> <sed args...>
  local rel=$1; shift
  rm -f "$B/overlay/$rel"
  sed "$@" "$SRC/$rel" > "$B/overlay/$rel"
}
patch_copy backend/src/util/check.h -e 's/"Error (%s: line %d): "##LOG/"Error (%s: line %d): " LOG/'
patch_copy backend/src/core/device/memory.h \
  -e 's#cudaMemPrefetchAsync(iter.first, iter.second, 0, 0 /\* stream \*/)#cudaSuccess#'
patch_copy backend/src/core/vulkan/cuvk.h \
  -e 's#semaphoreGetFdInfoKHR.handleType\([[:space:]]*\)= handleType;#semaphoreGetFdInfoKHR.handleType\1= (VkExternalSemaphoreHandleTypeFlagBits) handleType;#' \
  -e 's#(deviceProp.computeMode != cudaComputeModeProhibited)#(true)#'
patch_copy backend/src/core/mesh.h -e 's#Affine3f transform\([[:space:]]*\)= Affine3f::Identity();#Affine3f transform;#'
patch_copy backend/src/core/scenegraph.h -e 's#Affine3f \(m[A-Za-z]*Transform\) = Affine3f::Identity();#Affine3f \1;#'

# 4. compile the shim against the overlay (host code only is used; the
#    device pass needs an arch tcnn accepts)
R=$B/overlay; T=$R/ext/tcnn; BS=$R/backend/src; E=$BS/ext
INC="-I$R -I$BS -I$BS/core -I$BS/core/math/include -I$BS/core/math/3rdparty/eigen -I$E -I$E/json \
 -I$E/nvrhi/include -I$E/nvrhi/thirdparty/Vulkan-Headers/include -I$E/glfw/include -I$E/imgui -I$E/image \
 -I$R/ext/optix/include -I$T/include -I$T/dependencies -I$T/dependencies/fmt/include -I$B/gen"
printf 'namespace krr { extern const int Primes[1000]; const int Primes[1000] = {2, 3, 5, 7, 11}; }\n' > "$B/primes_stub.cpp"
nvcc -std=c++17 -arch=sm_90 -DTCNN_MIN_GPU_ARCH=90 --extended-lambda --expt-relaxed-constexpr \
  -Xcompiler -fPIC,-ffp-contract=off -D'__assume(x)=' $INC -c "$HERE/ref_shim.cu" -o "$B/ref_shim.o"
g++ -fPIC -c "$B/primes_stub.cpp" -o "$B/primes_stub.o"

# 5. tcnn's encoding and optimiser kernels as host functions: host-callable
#    copies of their headers (cut before the classes, qualifiers widened; see
#    tcnn_host_headers.py) ahead of the originals on the include path
rm -rf "$B/tcnn_host"
python3 "$HERE/tcnn_host_headers.py" "$T/include" "$B/tcnn_host"
TINC="-I$B/tcnn_host -I$T/include -I$T/dependencies -I$T/dependencies/fmt/include"
nvcc -std=c++17 -arch=sm_90 -DTCNN_MIN_GPU_ARCH=90 --extended-lambda --expt-relaxed-constexpr \
  -Xcompiler -fPIC,-ffp-contract=off $TINC -c "$HERE/ref_tcnn_kernels.cu" -o "$B/ref_tcnn_kernels.o"
# 6. tcnn's own grid-encoding constructor (level offsets, parameter count) from
#    the unmodified headers, with the vendored fmt's format.cc
TCI="-I$T/include -I$T/dependencies -I$T/dependencies/fmt/include"
nvcc -std=c++17 -arch=sm_90 -DTCNN_MIN_GPU_ARCH=90 --extended-lambda --expt-relaxed-constexpr \
  -Xcompiler -fPIC $TCI -c "$HERE/ref_tcnn_layout.cu" -o "$B/ref_tcnn_layout.o"
g++ -std=c++17 -O1 -fPIC -I"$T/dependencies/fmt/include" -c "$T/dependencies/fmt/src/format.cc" -o "$B/fmt_format.o"
nvcc -shared -arch=sm_90 "$B/ref_shim.o" "$B/primes_stub.o" "$B/ref_tcnn_kernels.o" "$B/ref_tcnn_layout.o" \
  "$B/fmt_format.o" -o "$OUT/libnmgref.so"
echo "built $OUT/libnmgref.so"
