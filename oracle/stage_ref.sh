#!/bin/sh
# Stages the reference library's sources for oracle/ref.mk on hosts without a reference checkout.
#
#   sh oracle/stage_ref.sh [REFERENCE_CHECKOUT]      (default: /root/reference)
#
# Copies the checkout's blend2d/ directory (library sources and headers, without its *_test.cpp
# unit tests) to baseline/_ref/blend2d-src/, which .gitignore keeps out of history: it is the
# reference installation of the benchmark's reference arm, not part of this repository's
# sources. oracle/ref.mk builds from there by default. The reference's test font goes to
# baseline/_ref/fonts/ (text scenes of tests/native/blcontext_check.cpp).
set -e
REF="${1:-/root/reference}"
HERE="$(cd "$(dirname "$0")" && pwd)"
DEST="$HERE/../baseline/_ref/blend2d-src"
[ -f "$REF/blend2d/blend2d.h" ] || { echo "no reference checkout at $REF" >&2; exit 1; }
rm -rf "$DEST"
mkdir -p "$DEST"
(cd "$REF" && find blend2d -type f ! -name '*_test.cpp' | tar -cf - -T -) | (cd "$DEST" && tar -xf -)
# the reference's test font, for the text scenes of the BLContext binding check
FONTS="$HERE/../baseline/_ref/fonts"
mkdir -p "$FONTS"
[ -f "$REF/blend2d-testing/resources/ABeeZee-Regular.ttf" ] && cp "$REF/blend2d-testing/resources/ABeeZee-Regular.ttf" "$FONTS/"
echo "staged $(find "$DEST" -type f | wc -l) files from $REF into $DEST"
