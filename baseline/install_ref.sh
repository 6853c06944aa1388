#!/bin/sh
# Stage the reference's CUDA kernel headers (tossenxD/big-int cuda/*.cu.h)
# into baseline/_ref/cuda/ so the reference kernels can be compiled on the
# GPU machine, where the reference checkout does not exist.  baseline/_ref/ is
# git-ignored: nothing of the reference enters the repository's history.
# Usage: REF=<reference checkout> sh install_ref.sh
set -e
HERE=$(cd "$(dirname "$0")" && pwd)
if [ -z "${REF:-}" ] || [ ! -f "$REF/cuda/ker-mul.cu.h" ]; then
    echo "REF does not name a reference checkout with cuda/ker-mul.cu.h; nothing staged"
    exit 0
fi
mkdir -p "$HERE/_ref/cuda"
cp "$REF/cuda/ker-helpers.cu.h" "$REF/cuda/ker-add.cu.h" "$REF/cuda/ker-mul.cu.h" "$HERE/_ref/cuda/"
echo "staged reference kernels in $HERE/_ref/cuda"
