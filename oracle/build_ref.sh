#!/usr/bin/env bash
# Builds the unmodified reference sources (read in place, never copied) with
# the project's shim headers into oracle/_ref/ldg_ref.  Test infrastructure:
# the binary generates the golden vectors under tests/golden/ and validates
# the C restatement in oracle/ldg_oracle.c.
#
#   REF_DIR   the reference checkout (required; unset = nothing to build)
#   OPENBLAS  scipy's bundled OpenBLAS (found through python if unset)
set -euo pipefail
HERE="$(cd "$(dirname "$0")" && pwd)"
REF_DIR="${REF_DIR:-}"
OUT="$HERE/_ref"
if [ -z "$REF_DIR" ]; then
  echo "build_ref: REF_DIR (the reference checkout) is not set; skipping" >&2
  exit 0
fi
if [ ! -f "$REF_DIR/solver.cpp" ]; then
  echo "build_ref: no reference sources at $REF_DIR; skipping" >&2
  exit 0
fi
if [ -z "${OPENBLAS:-}" ]; then
  OPENBLAS="$(python3 - <<'EOF'
import glob, os, scipy
libs = sorted(glob.glob(os.path.join(os.path.dirname(scipy.__file__) + ".libs", "libscipy_openblas-*.so")))
print(libs[0] if libs else "")
EOF
)"
fi
if [ -z "$OPENBLAS" ] || [ ! -f "$OPENBLAS" ]; then
  echo "build_ref: scipy's OpenBLAS not found; skipping" >&2
  exit 0
fi
mkdir -p "$OUT"
SRCS=""
for f in solver.cpp mesh.cpp dgMath.cpp io.cpp MPIUtil.cpp; do SRCS="$SRCS $REF_DIR/$f"; done
g++ -O3 -std=c++11 -w -I"$HERE/ref_shim" -I"$REF_DIR" \
    "$HERE/ref_driver.cpp" $SRCS \
    "$OPENBLAS" -Wl,-rpath,"$(dirname "$OPENBLAS")" -lm \
    -o "$OUT/ldg_ref"
echo "build_ref: built $OUT/ldg_ref"
