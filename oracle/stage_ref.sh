#!/bin/sh
# Stages the reference library's sources for oracle/ref.mk on hosts without a reference checkout.
#
#   sh oracle/stage_ref.sh [REFERENCE_CHECKOUT]      (default: /root/reference)
#
# Copies the checkout's blend2d/ directory (library sources and headers, without its *_test.cpp
# unit tests) to baseline/_ref/blend2d-src/, which .gitignore keeps out of history: it is the
# reference installation of the benchmark's reference arm, not part of this repository's
# sources. oracle/ref.mk builds from there by default.
set -e
REF="${1:-/root/reference}"
HERE="$(cd "$(dirname "$0")" && pwd)"
DEST="$HERE/../baseline/_ref/blend2d-src"
[ -f "$REF/blend2d/blend2d.h" ] || { echo "no reference checkout at $REF" >&2; exit 1; }
rm -rf "$DEST"
mkdir -p "$DEST"
(cd "$REF" && find blend2d -type f ! -name '*_test.cpp' | tar -cf - -T -) | (cd "$DEST" && tar -xf -)
echo "staged $(find "$DEST" -type f | wc -l) files from $REF into $DEST"
