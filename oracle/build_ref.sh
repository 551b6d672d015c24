#!/bin/sh
# Builds oracle/_ref/libpoe2d_ref.so: the reference's OWN kernel and set-up
# lines, compiled for the host CPU, used only to pin the oracle restatement
# (test infrastructure).  The reference lines are streamed from the read-only
# reference tree straight into the compiler; no copy of them is written.
#
#   cu:41-45     #defines (PI, faktor, ...)
#   cu:49-422    the seven __global__ kernels
#   cu:553-575   medium tables        cu:646-661  medium-ID lookup
#   cu:682-713   coefficient derivation
#   cu:840-845   PML constants        cu:908-909  PML scalars
#   cu:985-1159  PML profile builder
#
# The reference tree is $POE2D_REFERENCE, or else a folder named
# "reference" beside the repository's own folder.  Exits 0 without building
# when the reference tree is absent (GPU hosts).
set -e
HERE=$(cd "$(dirname "$0")" && pwd)
REF=${POE2D_REFERENCE:-$(cd "$HERE/../.." && pwd)/reference}
CU="$REF/seismic_CPML_2D_poroelastic_withCUDA.cu"
OUT="$HERE/_ref"
if [ ! -r "$CU" ]; then
    echo "build_ref: reference source not found ($CU); skipping"
    exit 0
fi
mkdir -p "$OUT"
H="$HERE/ref_harness"
{
    cat "$H/pre_common.inc"
    sed -n '41,45p' "$CU"
    sed -n '49,422p' "$CU"
    cat "$H/post_kernels.inc"
    cat "$H/pre_coeffs.inc"
    sed -n '553,575p;646,661p;682,713p' "$CU"
    cat "$H/post_coeffs.inc"
    cat "$H/pre_pml.inc"
    sed -n '840,845p;908,909p;985,1159p' "$CU"
    cat "$H/post_pml.inc"
} | ${CXX:-g++} -x c++ -std=c++17 -O2 -ffp-contract=off -fPIC -shared -w -o "$OUT/libpoe2d_ref.so" -
echo "build_ref: $OUT/libpoe2d_ref.so"
