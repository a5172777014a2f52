#!/bin/sh
# Compiles the reference's standalone-buildable sources for this path
# (Gauss rules, Legendre tables, CG/GMRES/BiCGstab templates) with the driver
# oracle/ref_driver.cpp into oracle/_ref/, runs it, and writes the golden
# vectors tests/golden/ref_tables.json and tests/golden/ref_krylov.json.
# Needs the dune-fem source tree (located by ref_src.sh); without it this
# recipe does nothing (the committed golden vectors stay as they are).  The
# reference's own build system is not used.
set -e
HERE=$(cd "$(dirname "$0")" && pwd)
if ! REF=$(sh "$HERE/ref_src.sh"); then
  echo "dune-fem sources not present: golden vectors left as committed"
  exit 0
fi
OUT="$HERE/_ref"
GOLD="$HERE/../tests/golden"
mkdir -p "$OUT" "$GOLD"
CXX=${CXX:-g++}
$CXX -O2 -std=c++17 -I"$HERE/shim" -I"$REF" \
  "$HERE/ref_driver.cpp" "$REF/dune/fem/space/shapefunctionset/legendrepolynomials.cc" \
  -o "$OUT/ref_driver"
"$OUT/ref_driver" tables > "$GOLD/ref_tables.json"
"$OUT/ref_driver" krylov > "$GOLD/ref_krylov.json"
echo "wrote $GOLD/ref_tables.json $GOLD/ref_krylov.json"
