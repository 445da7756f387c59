#!/usr/bin/env bash
# Builds oracle/_ref/libpbref.so from the reference's own sources where they
# lie (cuda/periodicBrinkman.h), against the stand-in matrix.h under
# oracle/ref_shim/.  Only runs where the reference tree is present
# (PB_REFERENCE_DIR, default /root/reference); the output is git-ignored.
# The reference's #include "../../include/matrix.h" resolves through
# -I oracle/_ref/inc/a/b to a link to oracle/ref_shim/include/.
set -euo pipefail
here="$(cd "$(dirname "$0")" && pwd)"
ref="${PB_REFERENCE_DIR:-/root/reference}/cuda"
if [ ! -f "$ref/periodicBrinkman.h" ]; then
  echo "reference sources not found at $ref; skipping" >&2
  exit 0
fi
mkdir -p "$here/_ref/inc/a/b"
# "../../include/matrix.h" seen from _ref/inc/a/b is _ref/inc/include/matrix.h
ln -sfn "$here/ref_shim/include" "$here/_ref/inc/include"
nvcc -O2 -std=c++17 -Xcompiler -fPIC -shared -w \
  -ftz=false -prec-div=true -prec-sqrt=true \
  -I "$here/_ref/inc/a/b" -I "$ref" \
  -o "$here/_ref/libpbref.so" "$here/ref_wrap.cu"
echo "built $here/_ref/libpbref.so"
# The reference's CUDA kernels (kernelReal, kernelFourier) as a device-only
# image for the GPU machine, where its sources are absent: a cubin for sm_103a
# (device code carries no host architecture) and PTX for the driver to
# compile where a cubin is not accepted.  The reference's flags (no flush to
# zero, IEEE division and square root); NDEBUG drops its device-side assert,
# whose launch condition oracle/ref_launch.cpp meets by construction.
for kind in cubin ptx; do
  if [ "$kind" = cubin ]; then arch=(-gencode arch=compute_103a,code=sm_103a); else arch=(-arch=compute_103a); fi
  nvcc "-$kind" "${arch[@]}" -O3 -std=c++17 -w -DNDEBUG \
    -ftz=false -prec-div=true -prec-sqrt=true \
    -I "$here/_ref/inc/a/b" -I "$ref" \
    -o "$here/_ref/ref_kernels.$kind" "$here/ref_kernels.cu"
done
echo "built $here/_ref/ref_kernels.cubin and .ptx"
