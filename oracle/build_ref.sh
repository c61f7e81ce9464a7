#!/usr/bin/env bash
# Build the reference's own CEUpdater (CEMC, cpp/src) as a test oracle.
#
# Reads the reference sources where they lie (default /root/reference, or $1)
# and writes ONLY into oracle/_ref/.  It does not run the reference's setup.py:
# it compiles the eleven CEUpdater sources with the reference's own flags
# (-std=c++11 -fopenmp -O3, setup.py:34) and wraps them with the reference's
# own Cython binding (cemc/cpp_ext/pyce_updater.pyx) through a one-line .pyx.
# numpy >= 2 rejects ce_updater.cpp's PyObject* -> PyArrayObject* conversions;
# ref_numpy2_shim.cpp supplies cast overloads and includes the unmodified file.
# Needs cython, g++, Python and numpy headers; exits 0 with a message when the
# reference tree is absent (as on machines that only run the product).
set -euo pipefail
REF=${1:-${CEMC_REFERENCE:-/root/reference}}
HERE=$(cd "$(dirname "$0")" && pwd)
OUT="$HERE/_ref"
if [ ! -d "$REF/cpp/src" ]; then
  echo "build_ref: reference sources not found at $REF; skipping"
  exit 0
fi
command -v cython >/dev/null || { echo "build_ref: cython not available; skipping"; exit 0; }
mkdir -p "$OUT"
PY=${PYTHON:-python3}
PYINC=$($PY -c "import sysconfig;print(sysconfig.get_paths()['include'])")
NPINC=$($PY -c "import numpy;print(numpy.get_include())")
SUFFIX=$($PY -c "import sysconfig;print(sysconfig.get_config_var('EXT_SUFFIX'))")
CXXFLAGS="-std=c++11 -fopenmp -O3 -fPIC -w -DNDEBUG -DNPY_OUT_ARRAY=NPY_ARRAY_OUT_ARRAY -I$REF/cpp/include -I$REF/cpp/src -I$PYINC -I$NPINC"
printf '# distutils: language = c++\ninclude "cemc/cpp_ext/pyce_updater.pyx"\n' > "$OUT/cemc_ref_updater.pyx"
cython -3 --cplus -I "$REF" "$OUT/cemc_ref_updater.pyx" -o "$OUT/cemc_ref_updater.cpp"
SRCS="cf_history_tracker additional_tools cluster named_array row_sparse_struct_matrix symbols_with_numbers basis_function linear_vib_correction mc_observers init_numpy_api"
pids=()
for s in $SRCS; do
  g++ $CXXFLAGS -c "$REF/cpp/src/$s.cpp" -o "$OUT/$s.o" & pids+=($!)
done
g++ $CXXFLAGS -c "$HERE/ref_numpy2_shim.cpp" -o "$OUT/ce_updater.o" & pids+=($!)
g++ $CXXFLAGS -c "$OUT/cemc_ref_updater.cpp" -o "$OUT/wrap.o" & pids+=($!)
for p in "${pids[@]}"; do wait "$p"; done
g++ -shared -fopenmp "$OUT"/*.o -o "$OUT/cemc_ref_updater$SUFFIX"
echo "build_ref: built $OUT/cemc_ref_updater$SUFFIX"
