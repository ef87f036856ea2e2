// GetFEM-side drop-in of the GPU assembly (compiled against GetFEM's own
// headers; see Makefile in this directory).
//
// ga_workspace::add_expression (src/getfem_generic_assembly_workspace.cc:545)
// parses, types and derives a GWFL expression into analysed trees, one per
// assembly order (tree_description, getfem/getfem_generic_assembly.h:306).
// This library takes over at the point where the reference's compiler starts
// (ga_compile, src/getfem_generic_assembly_compile_and_exec.cc:7910, called
// from ga_workspace::assembly, workspace.cc:791):
//
//   lower_workspace   walks the analysed trees of one order and lowers each
//                     to the descriptor of include/gfgpu.h (gfgpu_form), or
//                     rejects it (GMM_ASSERT1, the reference's error
//                     convention): no CPU fallback;
//   assembly          (gfgpu_workspace.cc) is a definition of
//                     getfem::ga_workspace::assembly(size_type, bool) that
//                     runs the lowered forms on the GPU through the C ABI and
//                     adds the results into the workspace's matrix, vector or
//                     potential with the reference's ownership rules.  Linked
//                     into a program (or preloaded) before a shared GetFEM
//                     library, it replaces the reference's definition, so
//                     add_expression, asm_* and model::assembly callers stay
//                     unchanged.
#pragma once

#include <string>
#include <vector>

#include "getfem/getfem_generic_assembly.h"
#include "gfgpu.h"

namespace gfgpu_getfem {

// The lowered form of one (variable, mesh_im, region) group of trees.
struct Lowered {
  std::string var;                       // the fem variable (test functions)
  const getfem::mesh_im *mim = nullptr;
  const getfem::mesh_region *rg = nullptr;
  gfgpu_form form{};
  // data slot k (k >= 1) holds the workspace datum slot_names[k]; slot 0 is
  // the variable; slot_kind[k]: GFGPU_COEF_ELEMENT (one value per element),
  // GFGPU_COEF_NODAL (a scalar field on the variable's scalar mesh_fem) or
  // 0 for a field on the variable's mesh_fem (a load)
  std::vector<std::string> slot_names{""};
  std::vector<int> slot_kind{0};
};

// Lowers every assembly tree of `order` (0 potential, 1 residual, 2
// tangent) of the workspace; trees over the same variable, mesh_im and
// region are merged into one form.  Unsupported trees raise gmm::gmm_error
// with the reason.
std::vector<Lowered> lower_workspace(const getfem::ga_workspace &ws, size_t order);

// Runs the lowered forms of `order` on the GPU and adds the results: order 2
// into *K, order 1 into *V, order 0 into *potential (each at the variable's
// interval).  Plans are cached per discretisation and form.
void assemble(getfem::ga_workspace &ws, size_t order, getfem::model_real_sparse_matrix *K,
              getfem::base_vector *V, double *potential);

// Destroys the cached GPU plans.
void release_plans();

// One line of JSON describing a lowered form (terms with their coefficient
// kinds, values and data names), for tests.
std::string to_json(const Lowered &L);

}  // namespace gfgpu_getfem
