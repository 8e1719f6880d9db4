#!/usr/bin/env bash
# Builds the reference SeeMPS (Cython backend) OUTSIDE this repository so that
# tests/golden/make_golden.py can import it and record golden vectors.
# Recipe: out-of-tree copy, setup.py build_ext, copy the built core into src/,
# stub h5py (only the HDF5 I/O imports it) and shim importlib.metadata.version.
# Usage: oracle/build_reference.sh REFERENCE_DIR OUT_DIR
#   REFERENCE_DIR  a checkout of the reference SeeMPS (read only)
#   OUT_DIR        a scratch directory outside this repository for the build
set -euo pipefail
if [ $# -ne 2 ]; then
  echo "usage: $0 REFERENCE_DIR OUT_DIR" >&2
  exit 2
fi
REF=$1
OUT=$2
mkdir -p "$OUT"
cp -r "$REF/src" "$REF/setup.py" "$OUT/"
chmod -R u+w "$OUT"
cd "$OUT"
python3 setup.py build_ext --inplace > build.log 2>&1 || true   # the in-place copy fails with the src/ layout
cp build/lib.*/seemps/cython/core.*.so src/seemps/cython/
mkdir -p shim/h5py
: > shim/h5py/__init__.py
cat > shim/sitecustomize.py <<'PY'
import importlib.metadata as m
_v = m.version
m.version = lambda n: "3.2-ref" if n == "seemps" else _v(n)
PY
echo "PYTHONPATH=$OUT/shim:$OUT/src"
