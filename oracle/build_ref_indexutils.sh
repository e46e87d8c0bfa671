#!/bin/sh
# Compiles the reference's own LUT post-processing module
# (mauve/indexutils.pyx) from the read-only reference checkout into
# oracle/_ref/ for pinning the LUT oracle.  Test infrastructure only.
#   sh oracle/build_ref_indexutils.sh <reference checkout>   (or MAUVE_REFERENCE=<dir>)
# One mechanical substitution is applied to a generated copy: the numpy
# Cython type np.int_t, which NumPy 2's .pxd no longer declares, becomes
# np.int64_t (NumPy 2's default integer on 64-bit Linux).  Nothing else of
# the source changes.
set -e
REF=${1:-$MAUVE_REFERENCE}
if [ -z "$REF" ] || [ ! -d "$REF/mauve" ]; then
  echo "build_ref_indexutils.sh: give the reference checkout as the first argument or in MAUVE_REFERENCE" >&2
  exit 2
fi
OUT=oracle/_ref
mkdir -p "$OUT"
sed 's/np\.int_t\b/np.int64_t/g' "$REF/mauve/indexutils.pyx" > "$OUT/indexutils.pyx"
python3 -m cython -3 "$OUT/indexutils.pyx" -o "$OUT/indexutils.c"
EXT=$(python3 -c "import sysconfig; print(sysconfig.get_config_var('EXT_SUFFIX'))")
INC=$(python3 -c "import sysconfig; print(sysconfig.get_paths()['include'])")
NPINC=$(python3 -c "import numpy; print(numpy.get_include())")
gcc -shared -fPIC -O2 -w -I"$INC" -I"$NPINC" "$OUT/indexutils.c" -o "$OUT/indexutils$EXT"
