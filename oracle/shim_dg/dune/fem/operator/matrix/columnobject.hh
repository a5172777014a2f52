// Stands in for the dune header of the same path when compiling dune-fem's
// DGEllipticOperator against the shim grid layer: every name that header
// would provide to dgelliptic.hh / legendre.hh comes from minidune.hh.
#include "minidune.hh"
