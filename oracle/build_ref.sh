#!/usr/bin/env bash
# Builds the reference's own permanent module (piquasso._math.permanent) straight
# from its C++ sources, without the reference's CMake, into oracle/_ref/.
#
# Test infrastructure only: the result is used to pin the oracle and to generate
# the golden fixtures under tests/golden/.  It is never shipped or measured as the
# product.  The reference sources are compiled where they lie; nothing is copied.
#
# Sources (reference paths): piquasso/_math/permanent.cpp (pybind11 module),
# src/permanent.cpp, src/permanent_laplace.cpp and the headers in src/.
# Flags follow the reference's Release build: -O3 -std=c++17 -fopenmp.
set -euo pipefail

HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
# the reference checkout: PQ_REFERENCE_DIR, else a directory named "reference"
# beside this repository
REF="${PQ_REFERENCE_DIR:-$(dirname "$(dirname "$HERE")")/reference}"
OUT="$HERE/_ref"

if [ ! -f "$REF/src/permanent.cpp" ]; then
    echo "build_ref: reference sources not found at $REF; skipping" >&2
    exit 0
fi

mkdir -p "$OUT"
PY=${PYTHON:-python3}
EXT_SUFFIX=$($PY -c "import sysconfig; print(sysconfig.get_config_var('EXT_SUFFIX'))")
PY_INC=$($PY -c "import sysconfig; print(sysconfig.get_paths()['include'])")
# pybind11 headers: the pip package if present, else the copy bundled with torch.
PYBIND_INC=$($PY -c "
try:
    import pybind11; print(pybind11.get_include())
except ImportError:
    import os, torch; print(os.path.join(os.path.dirname(torch.__file__), 'include'))
")

mkdir -p "$OUT/piquasso/_math"
touch "$OUT/piquasso/__init__.py" "$OUT/piquasso/_math/__init__.py"

g++ -O3 -std=c++17 -fopenmp -fPIC -shared -DNDEBUG \
    -I"$REF/src" -I"$PYBIND_INC" -I"$PY_INC" \
    "$REF/piquasso/_math/permanent.cpp" "$REF/src/permanent.cpp" "$REF/src/permanent_laplace.cpp" \
    -o "$OUT/piquasso/_math/permanent$EXT_SUFFIX"

echo "build_ref: built $OUT/piquasso/_math/permanent$EXT_SUFFIX"
