#!/bin/bash
# Builds the reference's serial step (PARALLEL 0) as a CPU oracle into
# oracle/_ref/, from the reference's own sources where they lie.
#   usage: oracle/build_ref.sh [REFERENCE_ROOT]
#   (default: $GA_REFERENCE_ROOT, else /root/reference)
# Only include/stdafx.h is copied into the build folder, with PARALLEL set to
# 0 as the serial Makefile path expects; every other reference file is
# compiled in place, unmodified.  main.cpp and files.cpp are replaced by
# oracle/ref/ref_harness.cpp (in-memory initial state, bundle dump) and FFTW3
# by oracle/ref/fftw_shim.cpp.  g++ -O3 as in the reference Makefile; no FMA
# contraction, so x86 and Arm hosts compute the same values.
# TEST INFRASTRUCTURE: the output is never shipped or called by the library.
set -euo pipefail
REF=${1:-${GA_REFERENCE_ROOT:-/root/reference}}
HERE=$(cd "$(dirname "$0")" && pwd)
OUT="$HERE/_ref"
if [ ! -f "$REF/source/pressure.cpp" ]; then
    echo "reference sources not found under $REF" >&2
    exit 3
fi
mkdir -p "$OUT/include" "$OUT/include_par" "$OUT/obj"
sed 's/^#define PARALLEL 1/#define PARALLEL 0/' "$REF/include/stdafx.h" > "$OUT/include/stdafx.h"
grep -q '^#define PARALLEL 0' "$OUT/include/stdafx.h"
# the monsoon initialisers (data_initializer.cpp) fill the parallel build's
# full-domain arrays; a second copy with ENERGY 1 selects that macro mapping
# while keeping the serial index arithmetic (oracle/ref/itcz_harness.cpp)
sed 's/^#define ENERGY 0/#define ENERGY 1/' "$OUT/include/stdafx.h" > "$OUT/include_par/stdafx.h"
grep -q '^#define ENERGY 1' "$OUT/include_par/stdafx.h"
# the linearised model (linear_integrate_rk3) is a compile-time switch of the
# same sources: a third copy with ISLINEAR 1 (the first definition in the file,
# the one the build's branch selects), built into ref_harness_lin
mkdir -p "$OUT/include_lin" "$OUT/obj_lin"
awk 'done == 0 && /^#define ISLINEAR 0/ {print "#define ISLINEAR 1"; done = 1; next} {print}' \
    "$OUT/include/stdafx.h" > "$OUT/include_lin/stdafx.h"
grep -q '^#define ISLINEAR 1' "$OUT/include_lin/stdafx.h"
# the hydrostatic equation set likewise (HYDROSTATIC 1), built into ref_harness_hyd
mkdir -p "$OUT/include_hyd" "$OUT/obj_hyd"
awk 'done == 0 && /^#define HYDROSTATIC 0/ {print "#define HYDROSTATIC 1"; done = 1; next} {print}' \
    "$OUT/include/stdafx.h" > "$OUT/include_hyd/stdafx.h"
grep -q '^#define HYDROSTATIC 1' "$OUT/include_hyd/stdafx.h"
CXXFLAGS="-O3 -ffp-contract=off -w -I$OUT/include -I$HERE/ref/shim -I$REF/include"
SRCS="solver initializer data_initializer interpolate fluxes pressure advection turbulence damping
      boundaries util Heating kessler rutledge microphysics energy trajectory laplacian
      process_input driver_serial"
pids=()
for s in $SRCS; do
    g++ $CXXFLAGS -c "$REF/source/$s.cpp" -o "$OUT/obj/$s.o" & pids+=($!)
done
g++ $CXXFLAGS -c "$HERE/ref/ref_harness.cpp" -o "$OUT/obj/ref_harness.o" & pids+=($!)
PARFLAGS="-O3 -ffp-contract=off -w -I$OUT/include_par -I$HERE/ref/shim -I$REF/include"
mkdir -p "$OUT/obj_par"
g++ $PARFLAGS -c "$REF/source/data_initializer.cpp" -o "$OUT/obj_par/data_initializer.o" & pids+=($!)
g++ $CXXFLAGS -c "$HERE/ref/itcz_harness.cpp" -o "$OUT/obj_par/itcz_harness.o" & pids+=($!)
g++ $CXXFLAGS -c "$HERE/ref/fftw_shim.cpp" -o "$OUT/obj/fftw_shim.o" & pids+=($!)
g++ $CXXFLAGS -c "$HERE/ref/files_stub.cpp" -o "$OUT/obj/files_stub.o" & pids+=($!)
gcc -O3 -ffp-contract=off -c "$HERE/ora_fft.c" -o "$OUT/obj/ora_fft.o" & pids+=($!)
LINFLAGS="-O3 -ffp-contract=off -w -I$OUT/include_lin -I$HERE/ref/shim -I$REF/include"
for s in $SRCS; do
    g++ $LINFLAGS -c "$REF/source/$s.cpp" -o "$OUT/obj_lin/$s.o" & pids+=($!)
done
g++ $LINFLAGS -c "$HERE/ref/ref_harness.cpp" -o "$OUT/obj_lin/ref_harness.o" & pids+=($!)
HYDFLAGS="-O3 -ffp-contract=off -w -I$OUT/include_hyd -I$HERE/ref/shim -I$REF/include"
for s in $SRCS; do
    g++ $HYDFLAGS -c "$REF/source/$s.cpp" -o "$OUT/obj_hyd/$s.o" & pids+=($!)
done
g++ $HYDFLAGS -c "$HERE/ref/ref_harness.cpp" -o "$OUT/obj_hyd/ref_harness.o" & pids+=($!)
for p in "${pids[@]}"; do wait "$p"; done
g++ -o "$OUT/ref_harness" "$OUT"/obj/*.o -lm
g++ -o "$OUT/ref_harness_lin" "$OUT"/obj_lin/*.o "$OUT/obj/fftw_shim.o" "$OUT/obj/files_stub.o" \
    "$OUT/obj/ora_fft.o" -lm
g++ -o "$OUT/ref_harness_hyd" "$OUT"/obj_hyd/*.o "$OUT/obj/fftw_shim.o" "$OUT/obj/files_stub.o" \
    "$OUT/obj/ora_fft.o" -lm
COMMON_OBJS=$(ls "$OUT"/obj/*.o | grep -v -e '/data_initializer.o$' -e '/ref_harness.o$')
g++ -o "$OUT/itcz_harness" $COMMON_OBJS "$OUT"/obj_par/*.o -lm
echo "built $OUT/ref_harness $OUT/ref_harness_lin $OUT/ref_harness_hyd $OUT/itcz_harness"
