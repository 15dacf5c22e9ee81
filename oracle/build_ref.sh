#!/usr/bin/env bash
# Compiles the reference library's own, unmodified C++ sources (utils, containers,
# physics and the pybind11 module; HDF5 I/O and plugins left out, as the
# reference's CI does with RAGNAR_USE_HDF5=OFF) against the Kokkos-API shim in
# oracle/kokkos_shim, into oracle/_ref/ragnar<ext>.  Nothing is copied: the
# sources are read where they lie.  Runs only where the reference tree exists.
set -euo pipefail
REF=${RAGNAR_REFERENCE_DIR:-/root/reference}
HERE=$(cd "$(dirname "$0")" && pwd)
OUT="$HERE/_ref"
if [ ! -d "$REF/src" ]; then
  echo "reference tree not found at $REF; skipping reference build" >&2
  exit 0
fi
PY=${PYTHON:-python3}
PYINC=$($PY -c 'import sysconfig; print(sysconfig.get_paths()["include"])')
EXT=$($PY -c 'import sysconfig; print(sysconfig.get_config_var("EXT_SUFFIX"))')
PBINC=$($PY -c 'import pybind11; print(pybind11.get_include())' 2>/dev/null || \
        $PY -c 'import os, torch; print(os.path.join(os.path.dirname(torch.__file__), "include"))')
mkdir -p "$OUT/obj"
SRCS="$REF/src/pyinterface.cpp"
for d in utils containers physics; do
  SRCS="$SRCS $(ls "$REF"/src/$d/*.cpp)"
done
CXXFLAGS="-std=c++20 -O3 -fPIC -fopenmp -fvisibility=hidden -I$REF/src -I$HERE/kokkos_shim -I$PBINC -I$PYINC"
pids=()
objs=()
for s in $SRCS; do
  o="$OUT/obj/$(echo "${s#$REF/src/}" | tr '/' '_').o"
  objs+=("$o")
  g++ $CXXFLAGS -c "$s" -o "$o" &
  pids+=($!)
done
for p in "${pids[@]}"; do wait "$p"; done
g++ -shared -fopenmp "${objs[@]}" -o "$OUT/ragnar$EXT"
echo "built $OUT/ragnar$EXT"
