#!/bin/sh
# ORACLE / CPU BASELINE — test infrastructure only.
#
# Stages the reference's source tree (its src/ directory, read-only at the
# path given, default /root/reference) into baseline/_ref/src, which git
# ignores.  The copy travels with the repository to machines that have no
# reference tree, where oracle/ref/Makefile compiles the reference's own
# block code and drivers from it (REF defaults to that copy).
set -e
SRC=${1:-/root/reference}
ROOT=$(cd "$(dirname "$0")/../.." && pwd)
DST="$ROOT/baseline/_ref"
[ -d "$SRC/src/blocks" ] || { echo "no reference tree at $SRC" >&2; exit 1; }
mkdir -p "$DST"
rm -rf "$DST/src"
cp -R "$SRC/src" "$DST/src"
chmod -R u+w "$DST/src"
echo "$SRC" > "$DST/STAGED_FROM"
