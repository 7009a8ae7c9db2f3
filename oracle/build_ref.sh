#!/usr/bin/env bash
# TEST INFRASTRUCTURE: compile the reference's own stage sources, unmodified and in place, together with
# oracle/ref_glue.cpp into oracle/_ref/libsister_ref.so. The reference needs SSE4.1/4.2 intrinsics, so
# this only builds on x86-64 hosts that have the reference tree, named by the first argument or SISTER_REFERENCE.
#     bash oracle/build_ref.sh REFERENCE_TREE
set -euo pipefail
REF="${1:-${SISTER_REFERENCE:-}}"
if [ -z "$REF" ]; then echo "usage: build_ref.sh REFERENCE_TREE (or set SISTER_REFERENCE)" >&2; exit 2; fi
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
OUT="$HERE/_ref"
if [ ! -d "$REF/cpp/src/sister" ]; then echo "reference tree not found at $REF" >&2; exit 3; fi
case "$(uname -m)" in x86_64|amd64) ;; *) echo "reference needs x86 SSE4.1 intrinsics; $(uname -m) host" >&2; exit 4;; esac
mkdir -p "$OUT"
SRC="$REF/cpp/src/sister"
g++ -std=c++17 -O3 -msse4.1 -msse4.2 -fopenmp -fPIC -shared -w \
    -I "$REF/cpp/include/sister" \
    "$SRC/census.cpp" "$SRC/postprocess.cpp" "$SRC/sgm.cpp" "$HERE/ref_glue.cpp" \
    -o "$OUT/libsister_ref.so.tmp"
mv "$OUT/libsister_ref.so.tmp" "$OUT/libsister_ref.so"
echo "built $OUT/libsister_ref.so"
