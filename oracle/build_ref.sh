#!/bin/bash
# ORACLE / TEST INFRASTRUCTURE ONLY.
#
# Compiles the reference MoTeX CLI from its own sources (motex.cc,
# functions.cc, binomial.cc under the reference tree) with g++ directly --
# not the reference's Makefiles -- into oracle/_ref/:
#   motexCPU, motexOMP            linked with the libflasm.so shipped in
#                                 libFLASM.zip (x86-64 hosts only)
#   motexCPU_port, motexOMP_port  linked with the restated flasm_port.cc
#   flasm_difftest                restated flasm vs shipped .so (x86-64 only)
# libdatrie is replaced by datrie_set.cc (same API subset, exact-string set);
# MPFR/GMP are not used (-D_USE_MPFR off), so only the long-double p-value
# code of the out-of-scope statistics writers is compiled.
#
# usage: oracle/build_ref.sh [reference-dir]
# The reference tree is the argument, else $MOTEX_REFERENCE_DIR, else the
# place this build host keeps it (/root/reference); this recipe is the one
# file that names that place.  Exit status 2: no reference sources there.
#
# Every product is written under a temporary name and renamed into place,
# and only when it is older than its sources.  A reference run that is
# using oracle/_ref/ (full-size runs take hours) therefore never sees its
# executable or its mapped libflasm.so truncated by a concurrent rebuild --
# extracting the library over itself in place did exactly that and killed
# such a run with SIGBUS.
set -euo pipefail
HERE="$(cd "$(dirname "$0")" && pwd)"
REF="${1:-${MOTEX_REFERENCE_DIR:-/root/reference}}"
OUT="$HERE/_ref"
if [ ! -f "$REF/motex.cc" ]; then
  echo "build_ref: no reference sources at $REF" >&2
  exit 2
fi
mkdir -p "$OUT"
CXX="${CXX:-g++}"
FLAGS="-O3 -w -fpermissive -I$HERE/include -I$HERE"
SRCS="$REF/motex.cc $REF/functions.cc $REF/binomial.cc $HERE/datrie_set.cc"
DEPS="$SRCS $REF/motexdefs.h $HERE/include/libflasm.h $HERE/include/datrie/trie.h $0"

# stale TARGET DEP...: true when TARGET is missing or older than a DEP
stale() {
  local t="$1"; shift
  [ -e "$t" ] || return 0
  for d in "$@"; do [ "$d" -nt "$t" ] && return 0; done
  return 1
}

# build TARGET CMD...: run CMD with -o TARGET.tmp.$$, then rename over TARGET
build() {
  local t="$1"; shift
  "$@" -o "$t.tmp.$$" && mv -f "$t.tmp.$$" "$t"
}

if stale "$OUT/motexCPU_port" $DEPS "$HERE/flasm_port.cc" "$HERE/motex_core.h"; then
  build "$OUT/motexCPU_port" "$CXX" $FLAGS -D_USE_CPU $SRCS "$HERE/flasm_port.cc" &
fi
if stale "$OUT/motexOMP_port" $DEPS "$HERE/flasm_port.cc" "$HERE/motex_core.h"; then
  build "$OUT/motexOMP_port" "$CXX" $FLAGS -D_USE_OMP -fopenmp $SRCS "$HERE/flasm_port.cc" &
fi

if [ "$(uname -m)" = "x86_64" ] && [ -f "$REF/libFLASM.zip" ]; then
  LIBDIR="$OUT/libFLASM/lib"
  if stale "$LIBDIR/libflasm.so" "$REF/libFLASM.zip"; then
    python3 - "$REF/libFLASM.zip" "$LIBDIR" <<'PY'
import os, sys, zipfile
src, libdir = sys.argv[1], sys.argv[2]
os.makedirs(libdir, exist_ok=True)
data = zipfile.ZipFile(src).read('libFLASM/lib/libflasm.so')
dst = os.path.join(libdir, 'libflasm.so')
tmp = dst + '.tmp.%d' % os.getpid()
with open(tmp, 'wb') as f:
    f.write(data)
os.chmod(tmp, 0o755)
os.replace(tmp, dst)
PY
  fi
  LINK="-L$LIBDIR -lflasm -Wl,-rpath,$LIBDIR"
  if stale "$OUT/motexCPU" $DEPS "$LIBDIR/libflasm.so"; then
    build "$OUT/motexCPU" "$CXX" $FLAGS -D_USE_CPU $SRCS $LINK &
  fi
  if stale "$OUT/motexOMP" $DEPS "$LIBDIR/libflasm.so"; then
    build "$OUT/motexOMP" "$CXX" $FLAGS -D_USE_OMP -fopenmp $SRCS $LINK &
  fi
  if stale "$OUT/flasm_difftest" "$HERE/flasm_difftest.cc" "$HERE/flasm_port.cc" "$HERE/motex_core.h" \
       "$LIBDIR/libflasm.so" "$0"; then
    "$CXX" -O2 -I"$HERE/include" -I"$HERE" -Dlibflasm=libflasm_port -c "$HERE/flasm_port.cc" \
      -o "$OUT/flasm_port_ns.o.tmp.$$" && mv -f "$OUT/flasm_port_ns.o.tmp.$$" "$OUT/flasm_port_ns.o"
    build "$OUT/flasm_difftest" "$CXX" -O2 -I"$HERE/include" "$HERE/flasm_difftest.cc" "$OUT/flasm_port_ns.o" $LINK &
  fi
fi
wait
echo "build_ref: built into $OUT"
