#!/bin/sh
# Builds oracle/_ref/libfvens_ref.so from the reference's own pointwise
# physics sources, compiled where they lie.  Test-only: used to pin the
# oracle's restatement and to generate the committed golden fixtures.
# Usage: build_ref.sh [REFERENCE_ROOT]
#   REFERENCE_ROOT defaults to $FVENS_REFERENCE, else /root/reference.
# Where the sources are found, their root is recorded in
# oracle/_ref/reference_root.txt for the tests that read the reference's own
# inputs (meshes, control files); absent sources skip those steps.
set -e
REF=${1:-${FVENS_REFERENCE:-/root/reference}}
HERE=$(cd "$(dirname "$0")" && pwd)
OUT="$HERE/../_ref"
if [ ! -d "$REF/src" ]; then
  echo "reference sources not found at $REF; skipping oracle/_ref" >&2
  exit 0
fi
mkdir -p "$OUT"
g++ -std=c++14 -O2 -ffp-contract=off -fPIC -shared -w \
    -I"$HERE/eigen_stub" -I"$REF/src" \
    "$HERE/ref_wrap.cpp" -o "$OUT/libfvens_ref.so"
(cd "$REF" && pwd) > "$OUT/reference_root.txt"
echo "built $OUT/libfvens_ref.so"
