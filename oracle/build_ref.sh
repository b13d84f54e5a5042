#!/usr/bin/env bash
# Compile the parts of the reference that build on their own into oracle/_ref/libmpcref.so,
# used only to pin the oracle (tests/golden/make_golden.py).  The reference's own Makefile is
# not used (it is syntactically invalid); its sources are compiled where they lie:
#   plasma.c       with g++ (C++ semantics, as nvcc would compile it), plus standard headers;
#   propagation.c  with nvcc as CUDA C++, plus standard headers, an MPI type stub and the
#                  declarations of the two kernels it launches under another name;
#   kernels.cu     with nvcc (its kernels are linked but never launched by the wrapper).
# The forced-include shims below only add declarations; no reference code is copied.
# Reads the reference sources (read-only) from the directory named by MPC_REFERENCE, writes only
# oracle/_ref/.  Without MPC_REFERENCE, or where it names no reference tree, nothing is built.
set -euo pipefail
REF=${MPC_REFERENCE:-}
HERE=$(cd "$(dirname "$0")" && pwd)
OUT="$HERE/_ref"
CUDA=${CUDA_HOME:-/usr/local/cuda}
NVCC=${NVCC:-$CUDA/bin/nvcc}
if [ -z "$REF" ] || [ ! -f "$REF/plasma.c" ]; then
  echo "reference sources not found (MPC_REFERENCE='$REF'); oracle/_ref not built" >&2
  exit 0
fi
mkdir -p "$OUT"
if [ -f "$OUT/libmpcref.so" ] && [ "$OUT/libmpcref.so" -nt "$HERE/ref_wrap.cpp" ] && [ "$OUT/libmpcref.so" -nt "$0" ]; then
  exit 0
fi
# plasma.c's ioniz reads Iion[2] of a two-element block (plasma.c:153,163).  The shim gives every
# allocation of plasma.c a zeroed tail and puts the value ref_ioniz states (mpcref_iion2) in
# slot 2 of each two-double block, so that the read is defined and the same on every host.
cat > "$OUT/shim_host.h" <<'EOF'
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <cmath>
extern "C" double mpcref_iion2;
static inline void* mpcref_malloc(size_t n) {
    double* p = (double*)calloc(1, n + 4 * sizeof(double));
    if (p && n == 2 * sizeof(double)) p[2] = mpcref_iion2;
    return p;
}
#define malloc(n) mpcref_malloc(n)
EOF
cat > "$OUT/shim_cu.h" <<'EOF'
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <cmath>
#include <cufft.h>
#include <cuda_runtime.h>
typedef int MPI_Datatype;
#define MPI_COMM_WORLD 0
#define MPI_STATUS_IGNORE 0
static inline int MPI_Send(const void*, int, MPI_Datatype, int, int, int) { return 0; }
static inline int MPI_Recv(void*, int, MPI_Datatype, int, int, int, int) { return 0; }
__global__ void propagTCUDA(cuDoubleComplex *A, const cuDoubleComplex *exponent, int *dims);
__global__ void propagRCUDA(cuDoubleComplex *A, const cuDoubleComplex *exponent, int *dims, int dir);
#include "plasma.h"
#include "kernels.h"
EOF
g++ -x c++ -include "$OUT/shim_host.h" -O2 -fPIC -ffp-contract=off -c -I"$REF" -I"$CUDA/include" "$REF/plasma.c" -o "$OUT/plasma.o"
"$NVCC" -x cu -include "$OUT/shim_cu.h" -rdc=true -O2 -Xcompiler -fPIC -c -I"$REF" "$REF/propagation.c" -o "$OUT/propagation.o" 2>"$OUT/propagation.warnings"
"$NVCC" -x cu -rdc=true -O2 -Xcompiler -fPIC -c -I"$REF" "$REF/kernels.cu" -o "$OUT/kernels.o"
"$NVCC" -x cu -include "$OUT/shim_cu.h" -rdc=true -O2 -Xcompiler -fPIC -c -I"$REF" "$HERE/ref_wrap.cpp" -o "$OUT/ref_wrap.o"
"$NVCC" -shared -Xcompiler -fPIC -o "$OUT/libmpcref.so" "$OUT/plasma.o" "$OUT/propagation.o" "$OUT/kernels.o" \
  "$OUT/ref_wrap.o" -lcufft -lcudart
echo "built $OUT/libmpcref.so"
