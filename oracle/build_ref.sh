#!/usr/bin/env bash
# Builds the Landau-Poisson reference's own C++ sources, read in place from
# the reference checkout (default /root/reference; override with LP_REF_DIR),
# into oracle/_ref/libref.so for use as a test oracle and CPU timing baseline.
#
# The reference needs MPI, FFTW3 and MKL-LAPACK, which this machine lacks; the
# headers in oracle/shim/ and oracle/shim/shim_impl.cpp stand in for them.
# No reference file is copied or edited: main() is renamed with -Dmain=... so
# that oracle/ref_harness.cpp can drive the routines.  The uninitialised
# private H[2] of RK3 (source/advection_1.cpp:431) is made deterministic with
# -ftrivial-auto-var-init=zero, which gives it the value 0; that flag does not
# reach OpenMP private copies, so advection_1.cpp is compiled without OpenMP
# (its loops then run on one thread).
#
# Output goes only to oracle/_ref/ (git-ignored).  Exits 0 without building
# when the reference checkout is absent.
set -euo pipefail
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
REF="${LP_REF_DIR:-/root/reference}"
SRC="$REF/source"
OUT="$HERE/_ref"
if [ ! -d "$SRC" ]; then
  echo "build_ref: no reference sources at $SRC; skipping"
  exit 0
fi
mkdir -p "$OUT/obj"
CXX="${CXX:-g++}"
FLAGS=(-O2 -fPIC -ffp-contract=off -ftrivial-auto-var-init=zero -w
       -I"$HERE/shim" -I"$SRC")
UNITS=(LP_ompi_1 collisionRoutines_1 conservationRoutines SetInit_1 advection_1
       PoissonFunctions PoissonVariables MomentCalculations EntropyCalculations
       MarginalCreation NegativityChecks PoissonPrint)
# two libraries: the default build (libref.so) and the two-species variant
# compiled with the reference's own FullandLinear switch (libref_lin.so)
build() {
  local obj="$1" lib="$2"; shift 2
  mkdir -p "$obj"
  local pids=()
  for u in "${UNITS[@]}"; do
    local extra=(-fopenmp)
    [ "$u" = LP_ompi_1 ] && extra+=(-Dmain=lp_reference_main_unused)
    [ "$u" = advection_1 ] && extra=()
    "$CXX" "${FLAGS[@]}" "$@" "${extra[@]}" -c "$SRC/$u.cpp" -o "$obj/$u.o" &
    pids+=($!)
  done
  "$CXX" "${FLAGS[@]}" "$@" -fopenmp -c "$HERE/shim/shim_impl.cpp" -o "$obj/shim_impl.o" & pids+=($!)
  "$CXX" "${FLAGS[@]}" "$@" -fopenmp -c "$HERE/ref_harness.cpp" -o "$obj/ref_harness.o" & pids+=($!)
  for p in "${pids[@]}"; do wait "$p"; done
  "$CXX" -shared -fopenmp -o "$lib" "$obj"/*.o
  echo "build_ref: built $lib"
}
build "$OUT/obj" "$OUT/libref.so"
build "$OUT/obj_lin" "$OUT/libref_lin.so" -DFullandLinear
