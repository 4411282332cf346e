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
# usage: oracle/build_ref.sh [reference-dir]   (default /root/reference)
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

"$CXX" $FLAGS -D_USE_CPU -o "$OUT/motexCPU_port" $SRCS "$HERE/flasm_port.cc" &
"$CXX" $FLAGS -D_USE_OMP -fopenmp -o "$OUT/motexOMP_port" $SRCS "$HERE/flasm_port.cc" &

if [ "$(uname -m)" = "x86_64" ] && [ -f "$REF/libFLASM.zip" ]; then
  python3 - "$REF/libFLASM.zip" "$OUT" <<'PY'
import sys, zipfile
z = zipfile.ZipFile(sys.argv[1])
z.extract('libFLASM/lib/libflasm.so', sys.argv[2])
PY
  LIBDIR="$OUT/libFLASM/lib"
  LINK="-L$LIBDIR -lflasm -Wl,-rpath,$LIBDIR"
  "$CXX" $FLAGS -D_USE_CPU -o "$OUT/motexCPU" $SRCS $LINK &
  "$CXX" $FLAGS -D_USE_OMP -fopenmp -o "$OUT/motexOMP" $SRCS $LINK &
  "$CXX" -O2 -I"$HERE/include" -I"$HERE" -Dlibflasm=libflasm_port -c "$HERE/flasm_port.cc" -o "$OUT/flasm_port_ns.o"
  "$CXX" -O2 -I"$HERE/include" -o "$OUT/flasm_difftest" "$HERE/flasm_difftest.cc" "$OUT/flasm_port_ns.o" $LINK &
fi
wait
echo "build_ref: built into $OUT"
