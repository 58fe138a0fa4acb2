#!/usr/bin/env bash
# TEST INFRASTRUCTURE.  Compiles the reference's own host code (SurfaceGrowth.cpp and the
# host functions of SurfaceGrowth.cu) from the read-only reference tree into
# oracle/_ref/libsgref_host.so, together with oracle/ref/ref_host_harness.cpp, which exposes a
# small C entry surface for tests/golden/make_golden.py.  Nothing is copied out of the
# reference tree; the output directory is git-ignored.
#
# The reference needs a few Windows/old-CUDA headers that do not exist here; tiny stand-ins
# are written into oracle/_ref/shim: <tchar.h>, <conio.h> and empty
# sm_11/sm_12_atomic_functions.h.  cudaThreadExit (removed from CUDA 13) maps to
# cudaDeviceReset.  SurfaceGrowth.cpp's calls into the CUDA wrappers are renamed to
# sgref_* stubs (the harness) so that parameter derivation, RNG and the result-file header
# run without a GPU.  It also builds the reference kernels as cubins (end of file).
# Usage: oracle/ref/build_ref.sh REFERENCE_ROOT   (or SG_REFERENCE_ROOT in the environment)
set -euo pipefail
REF=${1:-${SG_REFERENCE_ROOT:-}}
if [ -z "$REF" ]; then
  echo "usage: build_ref.sh REFERENCE_ROOT (or set SG_REFERENCE_ROOT)" >&2
  exit 3
fi
SRC="$REF/SurfaceGrowthConsole"
HERE=$(cd "$(dirname "$0")" && pwd)
OUT="$HERE/../_ref"
CUDA=${CUDA_HOME:-/usr/local/cuda}
if [ ! -f "$SRC/SurfaceGrowth.cpp" ]; then
  echo "reference sources not found under $SRC" >&2
  exit 3
fi
mkdir -p "$OUT/shim"
printf '#pragma once\n#define TCHAR char\n#define _TCHAR char\n#define _tfopen fopen\n' > "$OUT/shim/tchar.h"
printf '#pragma once\nstatic inline int _getch(void) { return 0; }\n' > "$OUT/shim/conio.h"
printf '#pragma once\n' > "$OUT/shim/sm_11_atomic_functions.h"
printf '#pragma once\n' > "$OUT/shim/sm_12_atomic_functions.h"
INC="-I$OUT/shim -I$SRC -I$CUDA/include"
RENAME="-D_tmain=sgref_unused_main -DCudaInitW=sgref_CudaInitW -DSetParametersW=sgref_SetParametersW -DInitCoordsW=sgref_InitCoordsW -DDoComputationsW=sgref_DoComputationsW"
# host parameter code: plain g++, no FMA contraction (the reference is an x86 build)
g++ -O1 -ffp-contract=off -fPIC -w $INC $RENAME -c "$SRC/SurfaceGrowth.cpp" -o "$OUT/ref_cpp.o"
# host functions of the CUDA translation unit (device code is compiled but never run here)
"$CUDA/bin/nvcc" -O1 -Xcompiler -fPIC,-ffp-contract=off -w $INC -DcudaThreadExit=cudaDeviceReset \
  -gencode arch=compute_103a,code=sm_103a -c "$SRC/SurfaceGrowth.cu" -o "$OUT/ref_cu.o"
g++ -O1 -ffp-contract=off -fPIC -w $INC -c "$HERE/ref_host_harness.cpp" -o "$OUT/ref_harness.o"
g++ -shared -o "$OUT/libsgref_host.so" "$OUT/ref_cpp.o" "$OUT/ref_cu.o" "$OUT/ref_harness.o" \
  -L"$CUDA/lib64" -lcudart -Wl,-rpath,"$CUDA/lib64"
echo "built $OUT/libsgref_host.so"
# The reference's device code alone, unmodified, as sm_103a cubins for oracle/ref/refkern.cpp:
# one without FMA contraction (the operation order the oracle and the PLAIN kernels follow,
# for parity) and one with nvcc's default flags (the reference as shipped, for timing).
NVFLAGS="-cubin -gencode arch=compute_103a,code=sm_103a -w $INC -DcudaThreadExit=cudaDeviceReset"
"$CUDA/bin/nvcc" $NVFLAGS -fmad=false "$SRC/SurfaceGrowth.cu" -o "$OUT/sgref_kernels_nofma.cubin"
"$CUDA/bin/nvcc" $NVFLAGS "$SRC/SurfaceGrowth.cu" -o "$OUT/sgref_kernels.cubin"
echo "built $OUT/sgref_kernels_nofma.cubin $OUT/sgref_kernels.cubin"
# The reference's host program itself (SurfaceGrowth.cpp, unchanged) linked against libsgmd.so
# instead of its own SurfaceGrowth.cu: the drop-in check of the C ABI (tests/test_abi.py).
SGLIB="$HERE/../../surfacegrowthconsole_gb300/lib"
if [ -f "$SGLIB/libsgmd.so" ]; then
  g++ -O1 -ffp-contract=off -w $INC -D_tmain=main -c "$SRC/SurfaceGrowth.cpp" -o "$OUT/sugr_main.o"
  g++ "$OUT/sugr_main.o" -o "$OUT/sugr_on_sgmd" -L"$SGLIB" -lsgmd -Wl,-rpath,"$SGLIB" \
    -L"$CUDA/lib64" -lcudart -Wl,-rpath,"$CUDA/lib64"
  echo "built $OUT/sugr_on_sgmd"
fi
