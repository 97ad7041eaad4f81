#!/usr/bin/env bash
# Builds the reference ANUGA Python package (Cython + C extensions) by hand
# into baseline/_ref/ so that tests/golden/make_golden.py can import it and
# write golden fixtures.  The reference's own build uses meson-python, which
# is not installed in this image, so each .pyx is cythonized and compiled
# with gcc directly.  Output never leaves baseline/_ref/ (git-ignored).
#
# Usage: bash tests/golden/build_reference_pkg.sh [/path/to/reference]
set -euo pipefail
REF=${1:-/root/reference}
HERE=$(cd "$(dirname "$0")/../.." && pwd)
OUT=$HERE/baseline/_ref
mkdir -p "$OUT"
rm -rf "$OUT/anuga"
cp -r "$REF/anuga" "$OUT/anuga"
chmod -R u+w "$OUT/anuga"
PYINC=$(python3 -c 'import sysconfig; print(sysconfig.get_paths()["include"])')
NPINC=$(python3 -c 'import numpy; print(numpy.get_include())')
SUFFIX=$(python3 -c 'import sysconfig; print(sysconfig.get_config_var("EXT_SUFFIX"))')
cd "$OUT"
build_one() {
  pyx=$1
  dir=$(dirname "$pyx"); base=$(basename "$pyx" .pyx)
  cplus=""; ext=c; cc=gcc
  if [ "$base" = neighbour_table_ext ]; then cplus="--cplus"; ext=cpp; cc=g++; fi
  extra=""
  case "$base" in
    *openmp*) extra="-fopenmp";;
  esac
  srcs="$dir/$base.$ext"
  if [ "$base" = fitsmooth_ext ]; then
    srcs="$srcs anuga/utilities/quad_tree.c anuga/utilities/sparse_dok.c anuga/utilities/sparse_csr.c"
  fi
  if ! cython -3 $cplus -I anuga/utilities "$pyx" -o "$dir/$base.$ext" > "$dir/$base.cython.log" 2>&1; then
    echo "cython failed: $pyx"; return 0
  fi
  if ! $cc -O2 -ffp-contract=off $extra -shared -fPIC -DNPY_NO_DEPRECATED_API=NPY_1_7_API_VERSION \
      -I"$NPINC" -I"$PYINC" -Ianuga/utilities -I"$dir" $srcs -o "$dir/$base$SUFFIX" -lm > "$dir/$base.cc.log" 2>&1; then
    echo "compile failed: $pyx"; return 0
  fi
}
export -f build_one
export NPINC PYINC SUFFIX
find anuga -name '*.pyx' | xargs -P 8 -I{} bash -c 'build_one {}'
# Import shims for Python packages the reference imports but this image lacks.
mkdir -p _shims/meshpy _shims/matplotlib
cat > _shims/dill.py << 'PY'
from pickle import *  # noqa: F401,F403  (stand-in: the reference only pickles)
PY
cat > _shims/pymetis.py << 'PY'
def part_graph(*a, **k):
    raise ImportError("pymetis is not available")
PY
cat > _shims/meshpy/__init__.py << 'PY'
PY
cat > _shims/meshpy/triangle.py << 'PY'
def build(*a, **k):
    raise ImportError("meshpy.triangle is not available")
class MeshInfo:
    pass
PY
cat > _shims/matplotlib/__init__.py << 'PY'
def use(*a, **k):
    pass
PY
for sub in pyplot cm colors tri animation patches collections lines; do
cat > _shims/matplotlib/$sub.py << 'PY'
def __getattr__(name):
    def _f(*a, **k):
        return None
    return _f
PY
done
cat > _shims/netCDF4.py << 'PY'
import numpy
import scipy.io
from scipy.io import _netcdf
# netCDF4 variables have a length (the record count of the first dimension)
_netcdf.netcdf_variable.__len__ = lambda self: self.shape[0]
class Dataset(scipy.io.netcdf_file):
    def __init__(self, filename, mode='r', format=None, **kw):
        mode = {'wl': 'w', 'w4': 'w'}.get(mode, mode)
        super().__init__(filename, mode, version=2, mmap=False)
    def createVariable(self, name, datatype, dimensions=(), **kw):
        # the classic format has no 64-bit integers
        dt = numpy.dtype(datatype)
        if dt.kind in 'iu' and dt.itemsize == 8:
            datatype = 'i'
        return super().createVariable(name, datatype, dimensions)
PY
echo "reference package built into $OUT"
