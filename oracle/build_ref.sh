#!/bin/sh
# Builds the reference's own Gofrt path (and MSD and neighbour lists) into
# oracle/_ref/ (TEST INFRASTRUCTURE).
#
# Compiles the unmodified reference sources lib/src/gofrt.cpp, lib/src/msd.cpp,
# lib/src/neighbour.cpp, lib/src/basetrajectory.cpp and
# lib/src/trajectory_numpy.cpp where they lie in the reference tree, plus
# oracle/ref_shim.cpp, into one Python extension pyanalisi_ref.  The
# reference's CMake build is not used (its pybind11 submodule is empty); this
# recipe replaces it for these five files only.
#
# -ffp-contract=off pins the arithmetic to separate IEEE mul/add, which is what
# an x86-64 build of the reference does by default; without it GCC on aarch64
# would fuse d2+=x*x (lib/include/basetrajectory.h:215-217) into FMAs.
#
# Usage: oracle/build_ref.sh REFERENCE_ROOT   (or with $ANALISI_REF set)
set -e
HERE=$(cd "$(dirname "$0")" && pwd)
REF=${1:-${ANALISI_REF:?"usage: build_ref.sh REFERENCE_ROOT (or set ANALISI_REF)"}}
OUT="$HERE/_ref"
if [ ! -f "$REF/lib/src/gofrt.cpp" ]; then
    echo "reference sources not found at $REF; oracle/_ref not built" >&2
    exit 3
fi
PY=${PYTHON:-python3}
PYBIND_INC=$($PY - <<'EOF'
import os
try:
    import pybind11
    print(pybind11.get_include())
except ImportError:
    import torch
    print(os.path.join(os.path.dirname(torch.__file__), "include"))
EOF
)
PYINC=$($PY -c "import sysconfig; print(sysconfig.get_paths()['include'])")
SUFFIX=$($PY -c "import sysconfig; print(sysconfig.get_config_var('EXT_SUFFIX'))")
mkdir -p "$OUT/cfg"
cat > "$OUT/cfg/config.h" <<'EOF'
#ifndef CONFIG_H
#define CONFIG_H
#define PYTHON_SUPPORT "oracle"
static const char *_info_msg = "analisi reference Gofrt path built as a test oracle";
#endif
EOF
${CXX:-g++} -std=c++17 -O3 -ffp-contract=off -fPIC -shared -w \
    -I"$OUT/cfg" -I"$REF/lib/include" -I"$REF/eigen3" -I"$PYBIND_INC" -I"$PYINC" \
    "$REF/lib/src/gofrt.cpp" "$REF/lib/src/msd.cpp" "$REF/lib/src/neighbour.cpp" \
    "$REF/lib/src/basetrajectory.cpp" \
    "$REF/lib/src/trajectory_numpy.cpp" "$HERE/ref_shim.cpp" \
    -o "$OUT/pyanalisi_ref$SUFFIX" -lpthread
echo "built $OUT/pyanalisi_ref$SUFFIX"
