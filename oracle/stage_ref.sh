#!/bin/sh
# Copies the inputs of oracle/Makefile's `ref` target -- the reference's headers and its DFT sources --
# into baseline/_ref/kfr.  That folder is git-ignored, so the copy is never committed; it travels with the
# working tree to machines that have no copy of the reference (the GPU host), where `make -C oracle ref`
# then compiles KFR itself for the timed CPU baseline.
#
# Usage: oracle/stage_ref.sh <path of the kfr source tree>
set -eu
src=${1:?usage: stage_ref.sh <path of the kfr source tree>}
here=$(cd "$(dirname "$0")" && pwd)
dst="$here/../baseline/_ref/kfr"
rm -rf "$dst"
mkdir -p "$dst/src"
cp -r "$src/include" "$dst/include"
cp -r "$src/src/dft" "$dst/src/dft"
cp "$src/LICENSE.txt" "$dst/LICENSE.txt"
echo "staged $src -> $dst"
