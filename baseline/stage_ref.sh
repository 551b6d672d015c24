#!/bin/sh
# Stages the reference's own two programs for timing on the GPU machine, in the
# git-ignored baseline/_ref/src/ (the GPU machine has no reference tree, and this
# folder travels there with the repository's working copy; it is never
# committed).  The copies are the reference's files with only what stops
# them from building or running at the benchmark's sizes changed:
#
#   seismic_CPML_2D_poroelastic_withCUDA.cu (the reference's CUDA program)
#     the grid, spacing, time step, receiver counts, snapshot interval and
#     C-PML width, hard-coded at cu:486-510, become macros set at compile
#     time (POE_NX POE_NZ POE_DX POE_DT POE_PANJ POE_PANJ2 POE_SAMP
#     POE_NPML); book.h (HANDLE_ERROR from "CUDA by Example", not in the
#     reference tree) and conio.h (Windows console) get small stand-ins.
#   seismic_CPML_2d_poroelastic.cpp (its serial C++ twin)
#     the same constants (cpp:59-78); a win.h stand-in, included first,
#     maps _tmain, _TCHAR and sprintf_s to their standard forms and brings in
#     the C headers the Windows build got through its other headers.
#
# The reference tree is $POE2D_REFERENCE, or else a folder named "reference"
# beside the repository's own folder.  Exits 0 without staging when it is
# absent.
set -e
HERE=$(cd "$(dirname "$0")" && pwd)
REF=${POE2D_REFERENCE:-$(cd "$HERE/../.." && pwd)/reference}
CU="$REF/seismic_CPML_2D_poroelastic_withCUDA.cu"
CPP="$REF/seismic_CPML_2d_poroelastic.cpp"
OUT="$HERE/_ref/src"
if [ ! -r "$CU" ] || [ ! -r "$CPP" ]; then
    echo "stage_ref: reference sources not found under $REF; skipping"
    exit 0
fi
mkdir -p "$OUT"
printf '#pragma once\n' > "$OUT/conio.h"
cat > "$OUT/book.h" <<'EOH'
#pragma once
#include <cstdio>
#include <cstdlib>
#include <cuda_runtime.h>
static void poe_handle_error(cudaError_t e, const char *file, int line)
{
    if (e != cudaSuccess) {
        std::printf("%s in %s at line %d\n", cudaGetErrorString(e), file, line);
        std::exit(EXIT_FAILURE);
    }
}
#define HANDLE_ERROR(e) (poe_handle_error((e), __FILE__, __LINE__))
EOH
cat > "$OUT/win.h" <<'EOH'
#pragma once
#include <cmath>
#include <cstdio>
#include <cstdlib>
#define _tmain main
typedef char _TCHAR;
#define sprintf_s sprintf
EOH
sed -e 's/^  int NX = 13599;/  int NX = POE_NX;/' \
    -e 's/^  int NZ = 2439;/  int NZ = POE_NZ;/' \
    -e 's/^  float DELTAX = 1.25;/  float DELTAX = POE_DX;/' \
    -e 's/^  int panj=122;/  int panj=POE_PANJ;/' \
    -e 's/^  int panj2=680;/  int panj2=POE_PANJ2;/' \
    -e 's/^  int samp =  5000;/  int samp = POE_SAMP;/' \
    -e 's/^  float DELTAT =95e-06;/  float DELTAT = POE_DT;/' \
    -e 's/^  int NPOINTS_PML = 10;/  int NPOINTS_PML = POE_NPML;/' \
    "$CU" > "$OUT/ref_cuda.cu"
sed -e 's/^\tint NX = 13599;/\tint NX = POE_NX;/' \
    -e 's/^\tint NZ = 2439;/\tint NZ = POE_NZ;/' \
    -e 's/^\tfloat DELTAX = 1.25;/\tfloat DELTAX = POE_DX;/' \
    -e 's/^\tint panj = 122;/\tint panj = POE_PANJ;/' \
    -e 's/^\tint panj2 = 680;/\tint panj2 = POE_PANJ2;/' \
    -e 's/^\tint samp = 5000;/\tint samp = POE_SAMP;/' \
    -e 's/^\tfloat DELTAT = 95e-06;/\tfloat DELTAT = POE_DT;/' \
    -e 's/^\tint NPOINTS_PML = 10;/\tint NPOINTS_PML = POE_NPML;/' \
    "$CPP" > "$OUT/ref_cpu.cpp"
n=$(grep -c 'POE_' "$OUT/ref_cuda.cu"); m=$(grep -c 'POE_' "$OUT/ref_cpu.cpp")
if [ "$n" -ne 8 ] || [ "$m" -ne 8 ]; then
    echo "stage_ref: expected 8 substituted constants in each program, found $n and $m" >&2
    exit 1
fi
echo "stage_ref: $OUT"
