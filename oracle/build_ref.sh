#!/usr/bin/env bash
# Builds the reference FAZ command-line tool and its bundled zstd 1.4.5 from the
# read-only reference checkout into oracle/_ref/ (git-ignored). Used only to pin
# the oracle and to generate golden fixtures; the product never links it.
# Usage: oracle/build_ref.sh REFERENCE_ROOT   (the reference FAZ checkout)
set -euo pipefail
if [ $# -lt 1 ] || [ -z "$1" ]; then
  echo "usage: $0 REFERENCE_ROOT" >&2
  exit 2
fi
REF=$1
HERE="$(cd "$(dirname "$0")" && pwd)"
OUT="$HERE/_ref"
if [ ! -d "$REF/include/QoZ" ]; then
  echo "reference checkout not found at $REF; nothing built" >&2
  exit 0
fi
mkdir -p "$OUT/obj"
ZSRC=$(ls "$REF"/zstd/common/*.c "$REF"/zstd/compress/*.c "$REF"/zstd/decompress/*.c)
objs=()
for f in $ZSRC; do
  o="$OUT/obj/$(basename "${f%.c}").o"
  if [ ! -f "$o" ] || [ "$f" -nt "$o" ]; then
    gcc -O3 -fPIC -DZSTD_MULTITHREAD=0 -I"$REF/zstd" -I"$REF/zstd/common" -c "$f" -o "$o" &
  fi
  objs+=("$o")
done
wait
ar rcs "$OUT/libzstd145.a" "${objs[@]}"
gcc -shared -o "$OUT/libzstd145.so" "${objs[@]}"
PYINC=$(python3 -c 'import sysconfig;print(sysconfig.get_paths()["include"])')
PBINC=$(python3 -c 'import pybind11;print(pybind11.get_include())')
PYLIBDIR=$(python3 -c 'import sysconfig;print(sysconfig.get_config_var("LIBDIR"))')
PYVER=$(python3 -c 'import sys;print(f"{sys.version_info[0]}.{sys.version_info[1]}")')
if [ ! -x "$OUT/faz" ] || [ "$REF/test/faz.cpp" -nt "$OUT/faz" ]; then
  g++ -O3 -std=c++17 -fopenmp -DFAZ_DEBUG_TIMINGS=0 \
      -I"$HERE/refstub" -I"$REF/include" -I"$REF/zstd" -I"$PBINC" -I"$PYINC" \
      "$REF/test/faz.cpp" -o "$OUT/faz" \
      "$OUT/libzstd145.a" -L"$PYLIBDIR" -lpython$PYVER -lpthread -ldl
fi
echo "built $OUT/faz and $OUT/libzstd145.{a,so}"
