#!/bin/sh
# Builds a symlink farm of the reference's FVMR/src tree under $2 (inside
# oracle/_ref) so its Windows-style include paths resolve on a case-sensitive
# file system: every directory is recreated, every file is a symlink to the
# original, and the spellings the sources use but the tree does not have are
# added as extra symlinks.  Nothing under the reference is modified.
# Oracle build only.
set -e
SRC="$1"
FARM="$2"
rm -rf "$FARM"
mkdir -p "$FARM"
( cd "$SRC" && find . -type d ) | while read -r d; do mkdir -p "$FARM/$d"; done
( cd "$SRC" && find . -type f ) | while read -r f; do ln -s "$SRC/$f" "$FARM/$f"; done
# case variants named by #include lines in the reference
mkdir -p "$FARM/gpu/dataType"
for f in "$SRC"/gpu/datatype/*; do ln -sf "$f" "$FARM/gpu/dataType/$(basename "$f")"; done
ln -sf "$SRC/gpu/datatype/Datatype.h" "$FARM/gpu/datatype/DataType.h"
ln -sf "$SRC/gpu/datatype/Datatype.h" "$FARM/gpu/dataType/DataType.h"
ln -sf "$SRC/global/GlobalPara.h" "$FARM/global/globalPara.h"
# the oracle build is headless: the GUI class header is replaced by a stub
ln -sf "$(cd "$(dirname "$0")" && pwd)/shim/WinGui_headless.h" "$FARM/gui/WinGui.h"
