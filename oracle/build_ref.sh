#!/usr/bin/env bash
# Compiles the reference's Monte Carlo extension from its own sources, where they
# lie ($MCD_REFERENCE_ROOT, by default the read-only checkout of this machine),
# into oracle/_ref/, and records that place in oracle/_ref/REFERENCE_ROOT for
# oracle/ref_loader.py.  Nothing of the
# reference is copied: only the compiled module is written, and oracle/ref_loader.py
# loads it next to the reference's own pure-Python `mc_dagprop.types` module.
#
# Flags follow the reference's setup.py (Linux: -O3 -std=c++20 -flto).
# pybind11 headers come from the pybind11 package when it is installed, else from
# the copy that ships inside PyTorch.
set -euo pipefail
REF="${MCD_REFERENCE_ROOT:-/root/reference}"
HERE="$(cd "$(dirname "$0")" && pwd)"
OUT="$HERE/_ref"
SRC="$REF/src/mc_dagprop/monte_carlo/_core.cpp"
if [ ! -f "$SRC" ]; then
  echo "reference sources not found at $REF; oracle/_ref not built" >&2
  exit 3
fi
mkdir -p "$OUT"
PYINC="$(python3 -c 'import sysconfig; print(sysconfig.get_paths()["include"])')"
PB11="$(python3 - << 'PY'
try:
    import pybind11
    print(pybind11.get_include())
except Exception:
    import os, torch
    print(os.path.join(os.path.dirname(torch.__file__), "include"))
PY
)"
SUFFIX="$(python3 -c 'import sysconfig; print(sysconfig.get_config_var("EXT_SUFFIX"))')"
g++ -O3 -std=c++20 -flto -shared -fPIC -I"$PYINC" -I"$PB11" -I"$REF/src/mc_dagprop/monte_carlo" \
    "$SRC" -o "$OUT/_core$SUFFIX"
printf "%s\n" "$REF" > "$OUT/REFERENCE_ROOT"
echo "built $OUT/_core$SUFFIX"
