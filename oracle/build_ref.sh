#!/usr/bin/env bash
# Builds oracle/_ref/libpbref.so from the reference's own sources where they
# lie (cuda/periodicBrinkman.h), against the stand-in matrix.h under
# oracle/ref_shim/.  Only runs where the reference tree is present; the
# output is git-ignored.  The reference's #include "../../include/matrix.h"
# resolves through -I oracle/ref_shim/a/b to oracle/ref_shim/include/.
set -euo pipefail
here="$(cd "$(dirname "$0")" && pwd)"
ref="${PB_REFERENCE_DIR:-/root/reference}/cuda"
if [ ! -f "$ref/periodicBrinkman.h" ]; then
  echo "reference sources not found at $ref; skipping" >&2
  exit 0
fi
mkdir -p "$here/_ref"
nvcc -O2 -std=c++17 -Xcompiler -fPIC -shared -w \
  -ftz=false -prec-div=true -prec-sqrt=true \
  -I "$here/ref_shim/a/b" -I "$ref" \
  -o "$here/_ref/libpbref.so" "$here/ref_wrap.cu"
echo "built $here/_ref/libpbref.so"
