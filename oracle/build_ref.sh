#!/bin/sh
# build_ref.sh -- compile the reference engine from its own sources, in place,
# into oracle/_ref/ (git-ignored).  TEST INFRASTRUCTURE ONLY.
#
# Usage: sh oracle/build_ref.sh [REFERENCE_ROOT]
#   REFERENCE_ROOT: the argument, else $RESYNTH_REFERENCE_ROOT, else /root/reference
#
# Outputs:
#   oracle/_ref/libref_st.so   single-threaded engine (the bit-exact oracle pin)
#   oracle/_ref/libref_mt.so   threaded engine, 8 pthreads (the reference default)
#   oracle/_ref/testSynth_ref  the reference's own smoke test, linked to libref_st
#
# The reference is built standalone (-DSYNTH_LIB_ALONE).  Its lib/buildSwitches.h
# forces GLib threads, which this image lacks, so a small switch header written
# here (never a copy of the reference's) is found first through the old GCC
# include-path split "-I<shim> -I- -I<lib>", which stops quoted includes from
# searching the including file's own directory first.  Nothing under the
# reference tree is modified or copied.
set -e
REF=${1:-${RESYNTH_REFERENCE_ROOT:-/root/reference}}
LIB="$REF/lib"
HERE=$(cd "$(dirname "$0")" && pwd)
OUT="$HERE/_ref"
[ -f "$LIB/engine.c" ] || { echo "reference sources not found under $LIB" >&2; exit 1; }
mkdir -p "$OUT/shim_st" "$OUT/shim_mt" "$OUT/shim_test" "$OUT/obj_st" "$OUT/obj_mt"

write_switches() {  # $1 = dir, $2 = threaded (1/0)
  {
    echo "/* generated by oracle/build_ref.sh: standalone build switches */"
    echo "#ifdef SYNTH_LIB_ALONE"
    echo "#define USE_GLIB_PROXY TRUE"
    echo "#else"
    echo "#define SYNTH_USE_GLIB TRUE"
    echo "#endif"
    echo "#define DEEP_PROGRESS"
    if [ "$2" = 1 ]; then
      echo "#define SYNTH_THREADED TRUE"
      echo "#define THREAD_LIMIT 8"
    else
      echo "#define THREAD_LIMIT 1"
    fi
  } > "$1/buildSwitches.h"
}
write_switches "$OUT/shim_st" 0
write_switches "$OUT/shim_mt" 1
# testSynth.c includes engineParams.h twice and the header has no guard.
cat > "$OUT/shim_test/engineParams.h" <<EOT
/* generated by oracle/build_ref.sh: include guard around the reference header */
#ifndef REF_ENGINE_PARAMS_GUARD
#define REF_ENGINE_PARAMS_GUARD
#include "$LIB/engineParams.h"
#endif
EOT

CC=${CC:-gcc}
CFLAGS="-O3 -std=gnu99 -fPIC -DSYNTH_LIB_ALONE -fgnu89-inline -w"
SRCS="imageSynth.c glibProxy.c engineParams.c imageFormat.c progress.c"
for v in st mt; do
  objs=""
  for s in $SRCS; do
    o="$OUT/obj_$v/${s%.c}.o"
    $CC $CFLAGS -I"$OUT/shim_$v" -I- -I"$LIB" -c "$LIB/$s" -o "$o" 2>/dev/null
    objs="$objs $o"
  done
  $CC $CFLAGS -I"$OUT/shim_$v" -I- -I"$LIB" -c "$HERE/ref_harness.c" -o "$OUT/obj_$v/ref_harness.o" 2>/dev/null
  $CC -shared -Wl,-Bsymbolic -o "$OUT/libref_$v.so" $objs "$OUT/obj_$v/ref_harness.o" -lm -lpthread
done
$CC $CFLAGS -I"$OUT/shim_test" -I"$OUT/shim_st" -I- -I"$LIB" -c "$REF/src/testSynth.c" -o "$OUT/obj_st/testSynth.o" 2>/dev/null
$CC -o "$OUT/testSynth_ref" "$OUT/obj_st/testSynth.o" -L"$OUT" -lref_st -Wl,-rpath,"$OUT" -lm -lpthread
echo "built: $OUT/libref_st.so $OUT/libref_mt.so $OUT/testSynth_ref"
