#!/bin/bash
# ORACLE / TEST INFRASTRUCTURE ONLY.
# Compiles the reference's own hot-path C++ (unmodified, read in place from
# the reference tree) plus the project's FFTW stand-in and C harness into
# oracle/_ref/libpyorbit_ref.so.  Flags follow the reference's
# conf/Linux/make_root_config (-O3) with MPI off (-DUSE_MPI=0: no MPI here).
# Runs only where the reference tree exists; outputs only into oracle/_ref/.
# Usage: build_ref.sh [REFERENCE_ROOT]; the root defaults to $PYORBIT_REF,
# else to a directory named "reference" beside the repository.
set -euo pipefail
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
REF=${1:-${PYORBIT_REF:-$(dirname "$(dirname "$HERE")")/reference}}
OUT="$HERE/_ref"
if [ ! -d "$REF/src/spacecharge" ]; then
  echo "reference tree not found at $REF; skipping" >&2
  exit 0
fi
mkdir -p "$OUT/obj"
PYINC=$(python3 -c 'import sysconfig;print(sysconfig.get_paths()["include"])')
INC="-I$HERE/fftw_shim -I$PYINC"
for d in src/orbit src/orbit/ParticlesAttributes src/orbit/BunchDiagnostics src/spacecharge src/teapot src/utils src/utils/bunch src/mpi; do
  INC="$INC -I$REF/$d"
done
SRCS="src/spacecharge/Grid1D.cc src/spacecharge/Grid2D.cc src/spacecharge/PoissonSolver2D.cc
src/spacecharge/PoissonSolverFFT2D.cc src/spacecharge/SpaceChargeCalc2p5D.cc src/spacecharge/BaseBoundary2D.cc
src/spacecharge/SpaceChargeCalc2p5Drb.cc src/spacecharge/ShapedBoundary2D.cc
src/orbit/BunchDiagnostics/BunchTwissAnalysis.cc src/orbit/BunchDiagnostics/BunchTuneAnalysis.cc
src/teapot/teapotbase.cc src/orbit/Bunch.cc src/orbit/SyncPart.cc src/orbit/OrbitConst.cc
src/utils/BufferStore.cc src/utils/CppPyWrapper.cc src/utils/AttributesBucket.cc src/utils/StringUtils.cc
src/utils/bunch/BunchExtremaCalculator.cc src/mpi/orbit_mpi.cc"
for f in "$REF"/src/orbit/ParticlesAttributes/*.cc; do SRCS="$SRCS ${f#$REF/}"; done
CXXFLAGS="-O3 -fPIC -DUSE_MPI=0 -std=c++11 -w"
pids=()
objs=()
for s in $SRCS; do
  o="$OUT/obj/$(echo "$s" | tr '/' '_' ).o"
  objs+=("$o")
  g++ $CXXFLAGS $INC -c "$REF/$s" -o "$o" &
  pids+=($!)
done
g++ $CXXFLAGS $INC -c "$HERE/ref_harness.cc" -o "$OUT/obj/ref_harness.o" & pids+=($!)
gcc -O3 -fPIC -c "$HERE/fftw_shim/fftw_shim.c" -o "$OUT/obj/fftw_shim.o" & pids+=($!)
gcc -O3 -fPIC -c "$HERE/fft.c" -o "$OUT/obj/fft.o" & pids+=($!)
for p in "${pids[@]}"; do wait "$p"; done
PYLIB=$(python3 -c 'import sysconfig;print(sysconfig.get_config_var("LIBDIR"))')
PYVER=$(python3 -c 'import sysconfig;print(sysconfig.get_config_var("LDVERSION"))')
g++ -shared -o "$OUT/libpyorbit_ref.so" "${objs[@]}" "$OUT/obj/ref_harness.o" "$OUT/obj/fftw_shim.o" "$OUT/obj/fft.o" \
  -L"$PYLIB" -lpython"$PYVER" -lpthread -lm
echo "built $OUT/libpyorbit_ref.so"
