#!/bin/sh
# Builds the reference program for the host CPU, from its unmodified sources where they
# lie, into oracle/_ref/calcIR_ref.  TEST INFRASTRUCTURE ONLY: its outputs pin the FP64
# oracle (tests/golden/make_golden.py); nothing in the product uses it.
#
# The reference is one CUDA C file written against MAGMA, libxdrfile and cuFFT, none of
# which exist here.  The recipe
#   - reads calcIR.cu in place and strips the kernel launch configurations <<<...>>> on
#     the fly (sed into g++'s standard input), so every kernel call becomes an ordinary
#     function call;
#   - defines __global__/__host__/__device__ away and gives the kernels one "thread"
#     (blockIdx = threadIdx = 0, blockDim = gridDim = 1), so each grid-stride loop runs
#     over all indices;
#   - resolves magma_v2.h, xdrfile*.h, xtc_seek.h and cufft.h to the shims in
#     oracle/refshim (host BLAS, Jacobi eigensolver, direct C2R, CIRTRJ01 reader);
#   - turns glibc's _FORTIFY_SOURCE off: the reference allocates its output file name
#     with strlen(outf)+9 bytes (calcIR.cu:194) and strcat's 11-character suffixes into it
#     (calcIR.cu:844-895), 3 bytes too many, which fortified strcat aborts on.  With an
#     output prefix of at most 12 characters the write stays inside glibc's 24-byte
#     minimum allocation, so the golden runs use short prefixes.
# Usage: oracle/build_ref.sh [reference_dir]
# The reference directory is the argument, else $CALCIR_REFERENCE_DIR, else the place the
# reference sources are mounted read-only in the build container.
set -e
REF=${1:-${CALCIR_REFERENCE_DIR:-/root/reference}}
HERE=$(cd "$(dirname "$0")" && pwd)
OUT="$HERE/_ref"
if [ ! -f "$REF/calcIR.cu" ]; then
    echo "reference sources not found at $REF" >&2
    exit 2
fi
mkdir -p "$OUT"
sed -e 's/<<<[^>]*>>>//g' "$REF/calcIR.cu" | \
    g++ -x c++ -std=c++14 -O2 -ffp-contract=off -w -U_FORTIFY_SOURCE -D_FORTIFY_SOURCE=0 \
        -D__global__= -D__host__= -D__device__= \
        -I"$HERE/refshim" -iquote "$REF" -include "$HERE/refshim/cuda_host_shim.h" \
        -c - -o "$OUT/calcIR_host.o"
g++ -std=c++14 -O2 -ffp-contract=off -I"$HERE/refshim" -c "$HERE/refshim/refshim.cpp" -o "$OUT/refshim.o"
g++ -o "$OUT/calcIR_ref" "$OUT/calcIR_host.o" "$OUT/refshim.o" -lm
echo "$OUT/calcIR_ref"
