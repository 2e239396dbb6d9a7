#!/usr/bin/env bash
# Test infrastructure: compiles the reference library's own C sources (where
# they lie, read-only) into oracle/_ref/libbf_ref.so, plus the golden-data
# driver oracle/_ref/ref_dump built from oracle/ref_dump.c.
#
# The reference's Meson build cannot run in this image (no meson, GSL, system
# LAPACK, ARPACK, SuiteSparse), so this recipe compiles src/*.c directly with
# gcc and a shim include directory (oracle/ref_shim) that maps CBLAS/LAPACKE
# onto the scipy-bundled OpenBLAS.  Files that need SuiteSparse or Python.h,
# and util_math.c (absent from the reference's own source list), are skipped.
#
# Usage: oracle/build_ref.sh [REFERENCE_ROOT]
# Exits 0 without building when the reference sources are absent.
set -euo pipefail

REF=${1:-${BF_REFERENCE_ROOT:-/root/reference}}
HERE=$(cd "$(dirname "$0")" && pwd)
OUT="$HERE/_ref"

if [ ! -f "$REF/src/fac_helm2.c" ]; then
  echo "build_ref: reference sources not found under $REF; nothing built"
  exit 0
fi

OPENBLAS=$(python3 - <<'PY'
import glob, os, scipy
libs = os.path.join(os.path.dirname(scipy.__file__), os.pardir, "scipy.libs")
cands = sorted(glob.glob(os.path.join(libs, "libscipy_openblas*.so")))
print(os.path.realpath(cands[0]) if cands else "")
PY
)
if [ -z "$OPENBLAS" ]; then
  echo "build_ref: scipy-bundled OpenBLAS not found; nothing built"
  exit 0
fi
# The shim headers map names onto scipy_-prefixed exports; check they exist.
EXPORTS=$(nm -D --defined-only "$OPENBLAS")
if ! grep -q " scipy_cblas_zgemm$" <<<"$EXPORTS"; then
  echo "build_ref: $OPENBLAS does not export scipy_cblas_zgemm; nothing built"
  exit 0
fi

mkdir -p "$OUT/obj"
CFLAGS="-std=gnu11 -O2 -fPIC -DBF_DOUBLE -DBF_LINUX -I$REF/include -I$HERE/ref_shim -w"
SKIP=" chol_csr_real.c cholmod.c lu_csr_real.c mat_python.c util_math.c "

pids=()
for f in "$REF"/src/*.c; do
  b=$(basename "$f")
  case "$SKIP" in *" $b "*) continue ;; esac
  gcc $CFLAGS -c "$f" -o "$OUT/obj/${b%.c}.o" &
  pids+=($!)
done
gcc $CFLAGS -c "$HERE/ref_shim/ref_stubs.c" -o "$OUT/obj/_oracle_stubs.o" &
pids+=($!)
for p in "${pids[@]}"; do wait "$p"; done

gcc -shared -o "$OUT/libbf_ref.so" "$OUT"/obj/*.o "$OPENBLAS" -lm \
    -Wl,--no-undefined -Wl,-rpath,"$(dirname "$OPENBLAS")"

gcc -std=gnu11 -O2 -DBF_DOUBLE -DBF_LINUX -I"$REF/include" -I"$HERE/ref_shim" \
    "$HERE/ref_dump.c" -o "$OUT/ref_dump" -L"$OUT" -lbf_ref "$OPENBLAS" -lm \
    -Wl,-rpath,"$OUT" -Wl,-rpath,"$(dirname "$OPENBLAS")"

# where the reference lies (its headers compile tests/integration's adapter)
echo "$REF" > "$OUT/reference_root.txt"
echo "$OPENBLAS" > "$OUT/openblas_path.txt"
echo "build_ref: built $OUT/libbf_ref.so and $OUT/ref_dump"
