#!/bin/sh
# Compiles the reference's standalone-buildable sources for this path
# (Gauss rules, Legendre tables, CG/GMRES/BiCGstab templates) with the driver
# oracle/ref_driver.cpp (with the oracle's operator, oracle.cpp) into
# oracle/_ref/, the reference's DG elliptic operator and its assembled
# Jacobian (dgelliptic.hh over legendre.hh) with oracle/ref_dgelliptic.cpp,
# its explicit time loop
# (timeprovider.hh, rungekutta/explicit.hh, butchertable.cc) over that
# operator with oracle/ref_timeloop.cpp, its Newton solver
# (newtoninverseoperator.hh) with oracle/ref_newton.cpp, and its
# stationary-iteration preconditioners (fempreconditioning.hh over
# spmatrix.hh) with oracle/ref_precond.cpp, all against the grid shim in
# oracle/shim_dg; runs them, and writes the golden vectors
# tests/golden/ref_tables.json, ref_krylov.json, ref_krylov_sipg.json,
# ref_dgelliptic.json, ref_dgelliptic_jacobian.json, ref_legendre_order.json
# (the hierarchical shape-function order), ref_timeloop.json,
# ref_newton.json and ref_precond.json.
# Needs the dune-fem source tree (located by ref_src.sh); without it this
# recipe does nothing (the committed golden vectors stay as they are).  With
# --compile-only it builds the drivers and writes nothing.  The reference's
# own build system is not used.
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
LEG="$REF/dune/fem/space/shapefunctionset/legendrepolynomials.cc"
# the drivers compile in parallel; each failure is reported
$CXX -O2 -std=c++17 -pthread -I"$HERE/shim" -I"$REF" \
  "$HERE/ref_driver.cpp" "$HERE/oracle.cpp" "$LEG" -o "$OUT/ref_driver" &
P1=$!
$CXX -O2 -std=c++17 -I"$HERE/shim_dg" -I"$HERE/shim" -I"$REF" \
  "$HERE/ref_dgelliptic.cpp" "$LEG" -o "$OUT/ref_dgelliptic" &
P2=$!
$CXX -O2 -std=c++17 -I"$HERE/shim_dg" -I"$HERE/shim" -I"$REF" \
  "$HERE/ref_timeloop.cpp" "$LEG" "$REF/dune/fem/solver/rungekutta/butchertable.cc" -o "$OUT/ref_timeloop" &
P3=$!
$CXX -O2 -std=c++17 -I"$HERE/shim_dg" -I"$HERE/shim" -I"$REF" \
  "$HERE/ref_newton.cpp" "$LEG" -o "$OUT/ref_newton" &
P4=$!
$CXX -O2 -std=c++17 -I"$HERE/shim_dg" -I"$HERE/shim" -I"$REF" \
  "$HERE/ref_precond.cpp" "$LEG" -o "$OUT/ref_precond" &
P5=$!
FAIL=0
for P in $P1 $P2 $P3 $P4 $P5; do
  wait "$P" || FAIL=1
done
if [ "$FAIL" != 0 ]; then
  echo "make_ref_golden.sh: a reference driver did not compile" >&2
  exit 1
fi
if [ "$1" = "--compile-only" ]; then
  echo "built $OUT/ref_driver $OUT/ref_dgelliptic $OUT/ref_timeloop $OUT/ref_newton $OUT/ref_precond"
  exit 0
fi
"$OUT/ref_driver" tables > "$GOLD/ref_tables.json"
"$OUT/ref_driver" krylov > "$GOLD/ref_krylov.json"
"$OUT/ref_driver" sipg > "$GOLD/ref_krylov_sipg.json"
"$OUT/ref_dgelliptic" > "$GOLD/ref_dgelliptic.json"
"$OUT/ref_dgelliptic" jacobian > "$GOLD/ref_dgelliptic_jacobian.json"
"$OUT/ref_dgelliptic" hierarchical > "$GOLD/ref_legendre_order.json"
"$OUT/ref_timeloop" > "$GOLD/ref_timeloop.json"
"$OUT/ref_newton" > "$GOLD/ref_newton.json"
"$OUT/ref_precond" > "$GOLD/ref_precond.json"
echo "wrote $GOLD/ref_tables.json $GOLD/ref_krylov.json $GOLD/ref_krylov_sipg.json $GOLD/ref_dgelliptic.json" \
  "$GOLD/ref_dgelliptic_jacobian.json $GOLD/ref_legendre_order.json $GOLD/ref_timeloop.json" \
  "$GOLD/ref_newton.json $GOLD/ref_precond.json"
