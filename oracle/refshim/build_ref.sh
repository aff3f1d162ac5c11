#!/usr/bin/env bash
# Builds oracle/_ref/libglref.so: the reference's own cell kernels
# (femgl/src/cell_mat_vec/*.cc) and material parameters (matep/src/matep.cc),
# compiled unmodified from the reference tree against the minimal deal.II
# stand-ins in oracle/refshim/.  TEST INFRASTRUCTURE: the product never links it.
#
# Usage: oracle/refshim/build_ref.sh [REFERENCE_ROOT]
# REFERENCE_ROOT is the argument, else $GL_REFERENCE.  Exits 0 and prints "skipped"
# when neither names a reference tree.
set -euo pipefail
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
ORACLE="$(dirname "$HERE")"
REF="${1:-${GL_REFERENCE:-}}"
OUT="$ORACLE/_ref"
if [ -z "$REF" ] || [ ! -d "$REF/femgl/src/cell_mat_vec" ]; then
  echo "build_ref: no reference tree given (argument or GL_REFERENCE): skipped"
  exit 0
fi
mkdir -p "$OUT/inc"
SRCS=("$REF"/femgl/src/cell_mat_vec/*.cc "$REF/matep/src/matep.cc")
# Empty headers for every deal.II include and for the project headers the kernel
# sources include but do not use (their bodies need only FullMatrix/Vector); the PDW
# initial-state header is compiled from its place in the tree.
for f in "${SRCS[@]}" "$REF/femgl/inc/pdw_config.h"; do
  grep -h -o '#include *<deal.II/[^>]*>' "$f" | sed 's/#include *<\(.*\)>/\1/' || true
done | sort -u | while read -r h; do
  mkdir -p "$OUT/inc/$(dirname "$h")"
  : > "$OUT/inc/$h"
done
for h in confreader.h dirichlet.h BinA.h; do : > "$OUT/inc/$h"; done
# the PDW header is taken from the reference tree (its includes are the empty stubs)
g++ -O2 -std=c++17 -fPIC -w -c -I "$HERE" -I "$OUT/inc" -I "$REF/femgl/inc" "$HERE/ref_pdw.cc" -o "$OUT/ref_pdw.o"
g++ -O2 -std=c++17 -fPIC -shared -w \
  -I "$HERE" -I "$OUT/inc" -I "$REF/matep/inc" \
  "${SRCS[@]}" "$HERE/ref_capi.cc" "$OUT/ref_pdw.o" -o "$OUT/libglref.so.tmp"
mv "$OUT/libglref.so.tmp" "$OUT/libglref.so"
echo "build_ref: built $OUT/libglref.so"
