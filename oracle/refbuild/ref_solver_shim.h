// Stand-in declaration for the one direct-solver entry point that the
// reference's gmm headers name unconditionally (gmm_solver_Schwarz_additive.h)
// when neither MUMPS nor SuperLU is configured.  It is never called on the
// assembly path; calling it throws.
#ifndef REF_SOLVER_SHIM_H
#define REF_SOLVER_SHIM_H
#ifdef __cplusplus
#include <stdexcept>
namespace gmm {
template <typename MAT, typename VECTX, typename VECTB>
bool MUMPS_solve(const MAT &, const VECTX &, const VECTB &,
                 bool = false, bool = false) {
  throw std::runtime_error("no direct solver in this reference build");
}
}
#endif
#endif
