#!/bin/sh
# Prints the directory of the dune-fem source tree that the recipes under
# oracle/ compile parts of (GBFEM_REFERENCE_SRC, else the tree's location in
# the build container); exits 1 when no such tree is present (for example on
# a machine that only runs the tests).
REF=${GBFEM_REFERENCE_SRC:-/root/reference}
if [ -d "$REF/dune/fem/solver/linear" ]; then
  echo "$REF"
else
  exit 1
fi
