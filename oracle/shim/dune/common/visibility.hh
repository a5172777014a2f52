// Minimal stand-in for dune-common's visibility macros (symbol export only).
#ifndef GBFEM_SHIM_DUNE_COMMON_VISIBILITY_HH
#define GBFEM_SHIM_DUNE_COMMON_VISIBILITY_HH
#define DUNE_EXPORT
#define DUNE_PRIVATE
#endif
