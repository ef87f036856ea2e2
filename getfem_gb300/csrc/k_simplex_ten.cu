// Affine-simplex element pass for forms with a constant anisotropic gradient
// coupling (GFGPU_TERM_GRADGRAD_TENSOR): the TEN instances of the element
// pass templates (k_simplex_tile.cuh), at the default 4 threads per element.
// T[(a,v),(b,w)] gains |J| c sum_{k,l} D[(a,k),(b,l)] g_vk g_wl, which is
// the reference's per-point contraction of (D : Grad_u) : Grad_Test_u
// (getfem_generic_assembly_compile_and_exec.cc:2276-3771, summed over the
// Gauss points with the element's own rule) factored through the constant
// gradients of an affine simplex.
#include "k_simplex_tile.cuh"

namespace gfgpu {

bool form_has_tensor(const gfgpu_form &f) {
  for (int t = 0; t < f.n_terms; ++t)
    if (f.terms[t].kind == GFGPU_TERM_GRADGRAD_TENSOR) return true;
  return false;
}

cudaError_t launch_simplex_element_pass_tensor(Plan &P, bool with_u, int64_t tile0,
                                               int64_t tile1, bool ku) {
  if (P.n_elements == 0) return cudaSuccess;
  const int64_t ntiles = (P.n_elements + 31) / 32;  // 32 elements per block
  if (tile1 < 0 || tile1 > ntiles) tile1 = ntiles;
  if (tile1 <= tile0) return cudaSuccess;
  const unsigned blocks = unsigned(tile1 - tile0);
  SlotPtrs sp;
  for (int i = 0; i < GFGPU_MAX_SLOTS; ++i) sp.p[i] = P.slot_ptr[i];
  const double *fsrc = nullptr;
  double fscale = 0.0;
  bool mass = false;
  simplex_source_of(P, fsrc, fscale, mass);
#define GFGPU_EPT(D, Q, N, MS, KUV)                                                            \
  simplex_element_pass<D, Q, N, MS, true, KUV, kEpWarps, true>                                 \
      <<<blocks, kEpThreads, 0, P.stream>>>(P.n_elements, P.d_points, P.d_cv, P.d_enode,       \
                                            P.d_stab, P.lay, P.form, sp, fsrc, fscale,          \
                                            with_u ? P.slot_ptr[GFGPU_SLOT_U] : nullptr,        \
                                            P.d_elem, P.d_err, tile0)
#define GFGPU_EPT4(D, Q, N)                        \
  do {                                             \
    if (mass && ku) GFGPU_EPT(D, Q, N, true, true); \
    else if (mass) GFGPU_EPT(D, Q, N, true, false); \
    else if (ku) GFGPU_EPT(D, Q, N, false, true);   \
    else GFGPU_EPT(D, Q, N, false, false);          \
  } while (0)
  const int d = P.dim, k = P.degree, q = P.qdim;
  if (d == 2 && k == 1 && q == 1) GFGPU_EPT4(2, 1, 3);
  else if (d == 2 && k == 2 && q == 1) GFGPU_EPT4(2, 1, 6);
  else if (d == 2 && k == 1 && q == 2) GFGPU_EPT4(2, 2, 3);
  else if (d == 2 && k == 2 && q == 2) GFGPU_EPT4(2, 2, 6);
  else if (d == 3 && k == 1 && q == 1) GFGPU_EPT4(3, 1, 4);
  else if (d == 3 && k == 2 && q == 1) GFGPU_EPT4(3, 1, 10);
  else if (d == 3 && k == 1 && q == 3) GFGPU_EPT4(3, 3, 4);
  else if (d == 3 && k == 2 && q == 3) GFGPU_EPT4(3, 3, 10);
  else return cudaErrorInvalidValue;
#undef GFGPU_EPT4
#undef GFGPU_EPT
  P.launches++;
  return cudaGetLastError();
}

}  // namespace gfgpu
