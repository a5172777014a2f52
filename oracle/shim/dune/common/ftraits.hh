// Minimal stand-in for dune-common's FieldTraits for real scalar types.
#ifndef GBFEM_SHIM_DUNE_COMMON_FTRAITS_HH
#define GBFEM_SHIM_DUNE_COMMON_FTRAITS_HH
namespace Dune {
template <class T>
struct FieldTraits {
  typedef T field_type;
  typedef T real_type;
};
}  // namespace Dune
#endif
