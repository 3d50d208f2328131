#!/bin/sh
# Builds the reference's hot-path sources (src/gpu/cdi.cu, cudaConfig.cu,
# cub_wrap.cu, src/post_gpu/cdi.cc, misc.cc, propagator.cc, src/independant/readConfig.cc,
# memManager.cc) as HOST code from where they lie in the reference checkout,
# through the emulation headers in oracle/refshim, into oracle/_ref/ref_harness.
# The kernels' explicit "<<<grid, block>>>" launches are rewritten on the way
# into the compiler (a sed filter on a pipe); nothing is copied into the repo.
# Test infrastructure (the oracle pin); needs g++ only, no GPU.
set -e
REF=${1:-/root/reference}
HERE=$(cd "$(dirname "$0")" && pwd)
OUT="$HERE/_ref"
SHIM="$HERE/refshim"
mkdir -p "$OUT/obj"
CXX="g++ -std=c++17 -O2 -w -fPIC -include $SHIM/cdxref_defs.h -I$SHIM -I$REF/include -I$REF/src/gpu"
LAUNCH='s/\([A-Za-z_][A-Za-z0-9_]*\(<[A-Za-z0-9_ ,:]*>\)\{0,1\}\)[ ]*<<<\([^>]*\)>>>/for (cdxref::Launch cdxref_l_(\3); cdxref_l_.next();) \1/g'
for f in src/gpu/cdi.cu src/gpu/cudaConfig.cu src/gpu/cub_wrap.cu; do
  o="$OUT/obj/$(basename "$f").o"
  sed "$LAUNCH" "$REF/$f" | $CXX -x c++ - -I"$REF/$(dirname "$f")" -c -o "$o"
done
for f in src/post_gpu/cdi.cc src/post_gpu/misc.cc src/post_gpu/propagator.cc src/independant/readConfig.cc src/independant/memManager.cc; do
  $CXX -c "$REF/$f" -o "$OUT/obj/$(basename "$f").o"
done
$CXX -DCDXREF_WITH_MISC -DCDXREF_WITH_PROPAGATOR -c "$SHIM/cdxref_stubs.cc" -o "$OUT/obj/cdxref_stubs.o"
$CXX -c "$SHIM/ref_harness.cc" -o "$OUT/obj/ref_harness.o"
g++ -o "$OUT/ref_harness" "$OUT"/obj/*.o
echo "built $OUT/ref_harness"

# Ptychography pin: the reference's ptycho driver (util/ptycho.cpp, compiled
# into pty_harness.cc), its kernels (src/gpu/ptycho.cu), the propagator, the
# FISTA object step, the Zernike pupil fit (src/gpu/beamDecomposition.cu) and
# the misc helpers (findMiddle, createCircleMask, shiftWave) it calls.
PO="$OUT/obj_pty"
mkdir -p "$PO"
sed "$LAUNCH" "$REF/src/gpu/ptycho.cu" | $CXX -x c++ - -I"$REF/src/gpu" -c -o "$PO/ptycho.cu.o"
# the Zernike pupil fit synchronises its blocks: its launches go through
# cdxref::coop (a generic lambda calls the kernel by name, default arguments kept)
COOP='s/\([A-Za-z_][A-Za-z0-9_]*\(<[A-Za-z0-9_ ,:]*>\)\{0,1\}\)[ ]*<<<\(.*\)>>>/cdxref::coop(\3, [](auto... cdxref_a_) { \1(cdxref_a_...); })/g'
sed "$COOP" "$REF/src/gpu/beamDecomposition.cu" | $CXX -x c++ - -I"$REF/src/gpu" -c -o "$PO/beamDecomposition.cu.o"
$CXX -c "$REF/src/post_gpu/propagator.cc" -o "$PO/propagator.cc.o"
$CXX -c "$REF/src/post_gpu/FISTA.cc" -o "$PO/FISTA.cc.o"
$CXX -DCDXREF_WITH_PROPAGATOR -DCDXREF_WITH_MISC -DCDXREF_WITH_PTYCHO_KERNELS -DCDXREF_WITH_FISTA -c "$SHIM/cdxref_stubs.cc" -o "$PO/cdxref_stubs.o"
$CXX -c "$SHIM/pty_stubs.cc" -o "$PO/pty_stubs.o"
$CXX -include "$SHIM/cdxref_ptycho.h" -DCDXREF_PTYCHO_CPP="\"$REF/util/ptycho.cpp\"" -c "$SHIM/pty_harness.cc" \
  -o "$PO/pty_harness.o"
g++ -pthread -o "$OUT/pty_harness" "$PO"/*.o "$OUT/obj/cudaConfig.cu.o" "$OUT/obj/cdi.cu.o" "$OUT/obj/cub_wrap.cu.o" \
  "$OUT/obj/misc.cc.o" "$OUT/obj/memManager.cc.o" "$OUT/obj/readConfig.cc.o"
echo "built $OUT/pty_harness"
