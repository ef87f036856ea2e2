// getfem::ga_workspace::assembly on the GPU.
//
// This file defines the member function that src/getfem_generic_assembly_
// workspace.cc:791 defines in the reference.  Linked into a program before
// a shared GetFEM library (or preloaded), it takes the place of the
// reference's definition for every caller: ga_workspace users, the asm_*
// functions (getfem/getfem_assembling.h) and model::assembly
// (src/getfem_models.cc:2646-2730, one workspace per OpenMP thread over that
// thread's partition of the region).  The steps are the reference's, with
// the compile and exec replaced:
//
//   1. the sizes of the model are brought up to date (workspace.cc:793-795);
//   2. the analysed trees of the order are lowered (gfgpu_lower.cc), or the
//      call fails with gmm::gmm_error (the reference's error convention) —
//      there is no CPU fallback;
//   3. the targets are prepared with the reference's ownership rule
//      (workspace.cc:803-845): a matrix or vector the workspace owns is
//      cleared and sized, one set by the caller (set_assembled_matrix /
//      set_assembled_vector) is added into;
//   4. each lowered (variable, mesh_im, region) group runs as a GPU plan of
//      the C ABI (include/gfgpu.h) over the elements of its region (the
//      mr_visitor walk of ga_exec, compile_and_exec.cc:8789, which visits
//      only the current thread's partition inside model::assembly's parallel
//      section), and its CSR / vector / potential is added into the targets
//      at the variable's interval.
//
// Plans are cached per (mesh, mesh_fem, mesh_im, element list, form), so a
// Newton loop pays the plan and pattern build once; the data (the variable
// and the coefficients) are copied to the plan at every call.  GPU calls are
// serialised by a mutex (OpenMP threads of model::assembly each hold their
// own plan).
#include <array>
#include <cmath>
#include <cstring>
#include <iostream>
#include <map>
#include <memory>
#include <mutex>
#include <sstream>

#include "getfem/getfem_generic_assembly.h"
#include "getfem/getfem_integration.h"
#include "getfem/getfem_models.h"
#include "gfgpu_getfem.h"

namespace gfgpu_getfem {
namespace {

struct PlanEntry {
  gfgpu_plan *plan = nullptr;
  std::vector<bgeot::size_type> cvs;  // the plan's elements, in order
  // the CSR pattern on the host, copied when the plan's pattern is built or
  // grows (its nnz changes: a repaired pattern only gains entries), not on
  // every assembly
  std::vector<int64_t> rowptr;
  std::vector<int32_t> colidx;
  std::vector<double> vals;
  ~PlanEntry() {
    if (plan) gfgpu_plan_destroy(plan);
  }
};

std::mutex g_mutex;
std::map<std::string, std::unique_ptr<PlanEntry>> g_plans;

void check(int rc, const char *what) {
  if (rc != GFGPU_OK)
    throw gmm::gmm_error(std::string("gfgpu: ") + what + ": " + gfgpu_last_error());
}

// Element types are identified by structure, not by name: GetFEM's names of
// finite elements and integration methods live in per-thread naming
// systems, and inside model::assembly's OpenMP section a worker thread sees
// FEM_QK(3,2) as FEM_PRODUCT(FEM_PRODUCT(FEM_PK(1,2),...)).

// The Lagrange nodes of FEM_PK(dim,K) / FEM_QK(dim,K) in GetFEM's order
// (lattice points, first coordinate fastest; for PK those of sum <= K).
std::vector<std::array<double, 3>> lattice_nodes(int dim, int kind, int K) {
  std::vector<std::array<double, 3>> out;
  const int n2 = dim == 3 ? K : 0;
  for (int k = 0; k <= n2; ++k)
    for (int j = 0; j <= K; ++j)
      for (int i = 0; i <= K; ++i) {
        if (kind == GFGPU_SIMPLEX && i + j + k > K) continue;
        out.push_back({double(i) / K, double(j) / K, dim == 3 ? double(k) / K : 0.0});
      }
  return out;
}

// kind and degree of a Lagrange FEM_PK / FEM_QK element, by its node count
// and node positions
void fem_kind(getfem::pfem pf, bgeot::size_type cv, int dim, int &kind, int &degree) {
  GMM_ASSERT1(int(pf->dim()) == dim && pf->target_dim() == 1 && pf->is_lagrange() &&
                  pf->is_equivalent() && pf->is_polynomial(),
              "gfgpu: finite element not lowered (a scalar Lagrange FEM_PK / FEM_QK is needed)");
  const size_t nb = pf->nb_dof(cv), nv = pf->basic_structure(cv)->nb_points();
  kind = nv == size_t(dim + 1) ? GFGPU_SIMPLEX : nv == (size_t(1) << dim) ? GFGPU_HEX : -1;
  GMM_ASSERT1(kind >= 0, "gfgpu: element shape not lowered");
  degree = -1;
  for (int K = 1; K <= 6 && degree < 0; ++K) {
    const auto nodes = lattice_nodes(dim, kind, K);
    if (nodes.size() != nb) continue;
    bool same = true;
    for (size_t i = 0; i < nb && same; ++i) {
      const bgeot::base_node &x = pf->node_of_dof(cv, i);
      for (int d = 0; d < dim; ++d) same &= std::fabs(x[d] - nodes[i][d]) < 1e-12;
    }
    GMM_ASSERT1(same, "gfgpu: finite element with another node order");
    degree = K;
  }
  GMM_ASSERT1(degree > 0, "gfgpu: finite element degree not lowered");
}

// the name of the integration method for the C ABI: the candidate whose
// points and weights (gfgpu_quadrature) are those of the method
std::string im_name(getfem::pintegration_method pim, int dim, int kind) {
  GMM_ASSERT1(pim->type() == getfem::IM_APPROX, "gfgpu: exact integration is not lowered");
  const getfem::papprox_integration pai = pim->approx_method();
  const size_t nq = pai->nb_points_on_convex();
  std::vector<std::string> cands;
  char buf[64];
  if (kind == GFGPU_HEX) {
    for (int k = 1; k <= 31; k += 2) {
      std::snprintf(buf, sizeof buf, "IM_GAUSS_PARALLELEPIPED(%d,%d)", dim, k);
      cands.push_back(buf);
    }
  } else {
    for (int k = 1; k <= 20; ++k) {
      std::snprintf(buf, sizeof buf, dim == 2 ? "IM_TRIANGLE(%d)" : "IM_TETRAHEDRON(%d)", k);
      cands.push_back(buf);
    }
  }
  for (const std::string &c : cands) {
    int32_t d = 0, n = 0;
    if (gfgpu_quadrature(c.c_str(), &d, &n, nullptr, nullptr) != GFGPU_OK) continue;
    if (d != dim || size_t(n) != nq) continue;
    std::vector<double> pts(static_cast<size_t>(n) * dim), w(static_cast<size_t>(n));
    if (gfgpu_quadrature(c.c_str(), &d, &n, pts.data(), w.data()) != GFGPU_OK) continue;
    bool same = true;
    for (size_t q = 0; q < nq && same; ++q) {
      same &= std::fabs(w[q] - pai->coeff(q)) < 1e-14;
      for (int k = 0; k < dim; ++k) same &= std::fabs(pts[q * dim + k] - pai->point(q)[k]) < 1e-14;
    }
    if (same) return c;
  }
  throw gmm::gmm_error("gfgpu: integration method not lowered");
}

uint64_t fnv(const void *p, size_t n, uint64_t h = 1469598103934665603ull) {
  const unsigned char *c = static_cast<const unsigned char *>(p);
  for (size_t i = 0; i < n; ++i) h = (h ^ c[i]) * 1099511628211ull;
  return h;
}

PlanEntry &plan_for(const getfem::ga_workspace &ws, const Lowered &L) {
  const getfem::mesh_fem &mf = *ws.associated_mf(L.var);
  const getfem::mesh &m = mf.linked_mesh();
  GMM_ASSERT1(!mf.is_reduced(), "gfgpu: reduced mesh_fem (extension matrices) not lowered");
  GMM_ASSERT1(&L.mim->linked_mesh() == &m, "gfgpu: mesh_im and mesh_fem on different meshes");
  std::vector<bgeot::size_type> cvs;
  for (getfem::mr_visitor v(*L.rg, m, true); !v.finished(); ++v) {
    GMM_ASSERT1(v.is_face() == false, "gfgpu: boundary (face) terms are not lowered");
    cvs.push_back(v.cv());
  }
  // the discretisation of the plan: all mesh points, the region's elements
  const int dim = int(m.dim());
  GMM_ASSERT1(m.points().index().card() == m.points().size() &&
                  m.points().index().last_true() + 1 == m.points().size(),
              "gfgpu: mesh point indices must be contiguous");
  std::vector<double> pts(m.points().size() * dim);
  for (bgeot::size_type ip = 0; ip < m.points().size(); ++ip)
    for (int d = 0; d < dim; ++d) pts[ip * dim + d] = m.points()[ip][d];
  // a plan per (mesh and its coordinates, mesh_fem, mesh_im, elements, form)
  std::ostringstream key;
  key << &m << ':' << fnv(pts.data(), pts.size() * sizeof(double)) << ':' << &mf << ':'
      << mf.nb_dof() << ':' << L.mim << ':' << cvs.size() << ':'
      << fnv(cvs.data(), cvs.size() * sizeof(cvs[0])) << ':' << fnv(&L.form, sizeof(L.form));
  auto it = g_plans.find(key.str());
  if (it != g_plans.end()) return *it->second;
  int kind = -1, degree = -1;
  std::string im;
  std::vector<int64_t> cvpts, dofs;
  size_t nbg = 0, nb = 0;
  getfem::pfem pf0 = nullptr;
  getfem::pintegration_method pim0 = nullptr;
  bgeot::pgeometric_trans pgt0 = nullptr;
  for (bgeot::size_type cv : cvs) {
    // one finite element, integration method and geometric transformation
    // per region (identified once, compared by pointer afterwards)
    getfem::pfem pf = mf.fem_of_element(cv);
    getfem::pintegration_method pim = L.mim->int_method_of_element(cv);
    bgeot::pgeometric_trans pgt = m.trans_of_convex(cv);
    if (!pf0) {
      pf0 = pf;
      pim0 = pim;
      pgt0 = pgt;
      fem_kind(pf, cv, dim, kind, degree);
      im = im_name(pim, dim, kind);
      // the geometric transformation of a degree-1 simplex or hexahedron
      GMM_ASSERT1(pgt->nb_points() == (kind == GFGPU_SIMPLEX ? size_t(dim + 1) : size_t(1) << dim) &&
                      pgt->dim() == bgeot::dim_type(dim),
                  "gfgpu: geometric transformation not lowered (GT_PK(dim,1) / GT_QK(dim,1))");
    }
    GMM_ASSERT1(pf == pf0 && pim == pim0 && pgt == pgt0,
                "gfgpu: one element type, finite element and integration method per region");
    const auto &P = m.ind_points_of_convex(cv);
    const auto &D = mf.ind_scalar_basic_dof_of_element(cv);
    if (!nbg) nbg = P.size(), nb = D.size();
    for (auto p : P) cvpts.push_back(int64_t(p));
    for (auto d : D) dofs.push_back(int64_t(d));
  }
  std::string imc;
  for (char c : im)
    if (c != ' ') imc += c;
  gfgpu_space S{};
  S.dim = dim;
  S.kind = kind < 0 ? GFGPU_SIMPLEX : kind;
  S.degree = degree < 0 ? 1 : degree;
  S.qdim = int(mf.get_qdim());
  S.im = imc.c_str();
  S.n_points = int64_t(m.points().size());
  S.n_elements = int64_t(cvs.size());
  S.n_dof = int64_t(mf.nb_dof());
  S.points = pts.data();
  S.cvpts = cvpts.data();
  S.dofs = dofs.data();
  auto e = std::make_unique<PlanEntry>();
  e->cvs = cvs;
  check(gfgpu_plan_create(&S, &L.form, nullptr, &e->plan), "plan creation");
  PlanEntry &ref = *e;
  g_plans[key.str()] = std::move(e);
  return ref;
}

// The plan's data slots from the workspace's current values.
void bind_data(const getfem::ga_workspace &ws, const Lowered &L, PlanEntry &E) {
  const auto &U = ws.value(L.var);
  check(gfgpu_set_data(E.plan, GFGPU_SLOT_U, &U[0], int64_t(gmm::vect_size(U)), 0), "variable");
  for (size_t k = 1; k < L.slot_names.size(); ++k) {
    const std::string &nm = L.slot_names[k];
    const auto &V = ws.value(nm);
    if (L.slot_kind[k] == GFGPU_COEF_ELEMENT) {
      // per element of the plan, through the P0 mesh_fem's numbering
      const getfem::mesh_fem &m0 = *ws.associated_mf(nm);
      std::vector<double> ev(E.cvs.size());
      for (size_t i = 0; i < E.cvs.size(); ++i) ev[i] = V[m0.ind_basic_dof_of_element(E.cvs[i])[0]];
      check(gfgpu_set_data(E.plan, int32_t(k), ev.data(), int64_t(ev.size()), 0), nm.c_str());
    } else {
      check(gfgpu_set_data(E.plan, int32_t(k), &V[0], int64_t(gmm::vect_size(V)), 0), nm.c_str());
    }
  }
}

// K(off + i, off + j) += CSR values (rows i, columns j), column by column.
void add_csr(getfem::model_real_sparse_matrix &K, size_t off, const std::vector<int64_t> &rowptr,
             const std::vector<int32_t> &colidx, const std::vector<double> &vals) {
  const size_t n = rowptr.size() - 1;
  GMM_ASSERT1(gmm::mat_nrows(K) >= off + n && gmm::mat_ncols(K) >= off + n,
              "gfgpu: assembled matrix too small");
  // CSR -> per-column lists, rows ascending (counting sort by column)
  std::vector<int64_t> cptr(n + 1, 0);
  for (int32_t c : colidx) cptr[size_t(c) + 1]++;
  for (size_t j = 0; j < n; ++j) cptr[j + 1] += cptr[j];
  std::vector<int64_t> fill(cptr.begin(), cptr.end() - 1);
  std::vector<std::pair<int32_t, double>> cv(colidx.size());
  for (size_t i = 0; i < n; ++i)
    for (int64_t p = rowptr[i]; p < rowptr[i + 1]; ++p)
      cv[size_t(fill[size_t(colidx[size_t(p)])]++)] = {int32_t(i), vals[size_t(p)]};
  for (size_t j = 0; j < n; ++j) {
    auto &col = K.col(off + j);
    const int64_t a = cptr[j], b = cptr[j + 1];
    if (a == b) continue;
    if (col.nb_stored() == 0) {
      col.base_resize(size_t(b - a));
      auto it = col.begin();
      for (int64_t p = a; p < b; ++p, ++it) {
        it->c = off + size_t(cv[size_t(p)].first);
        it->e = cv[size_t(p)].second;
      }
    } else {
      for (int64_t p = a; p < b; ++p) {
        const size_t r = off + size_t(cv[size_t(p)].first);
        col.w(r, col.r(r) + cv[size_t(p)].second);
      }
    }
  }
}

}  // namespace

void assemble(getfem::ga_workspace &ws, size_t order, getfem::model_real_sparse_matrix *K,
              getfem::base_vector *V, double *potential) {
  std::vector<Lowered> forms = lower_workspace(ws, order);
  std::lock_guard<std::mutex> lock(g_mutex);
  for (const Lowered &L : forms) {
    if (L.form.n_terms == 0) continue;
    PlanEntry &E = plan_for(ws, L);
    bind_data(ws, L, E);
    const size_t off = ws.interval_of_variable(L.var).first();
    if (order == 0) {
      double e = 0.0;
      check(gfgpu_assemble(E.plan, 0, 0, &e), "potential");
      *potential += e;
    } else if (order == 1) {
      check(gfgpu_assemble(E.plan, 1, 0, nullptr), "vector assembly");
      check(gfgpu_sync(E.plan), "vector assembly");
      const size_t n = ws.associated_mf(L.var)->nb_dof();
      std::vector<double> r(n);
      check(gfgpu_copy_result(E.plan, GFGPU_RESULT_VECTOR, r.data()), "vector copy");
      GMM_ASSERT1(gmm::vect_size(*V) >= off + n, "gfgpu: assembled vector too small");
      for (size_t i = 0; i < n; ++i) (*V)[off + i] += r[i];
    } else {
      check(gfgpu_assemble(E.plan, 2, 0, nullptr), "matrix assembly");
      check(gfgpu_sync(E.plan), "matrix assembly");
      int64_t nr = 0, nnz = 0;
      check(gfgpu_pattern_size(E.plan, &nr, &nnz), "pattern");
      if (E.rowptr.size() != static_cast<size_t>(nr) + 1 ||
          E.colidx.size() != static_cast<size_t>(nnz)) {
        E.rowptr.assign(static_cast<size_t>(nr) + 1, 0);
        E.colidx.assign(static_cast<size_t>(nnz), 0);
        check(gfgpu_pattern_copy(E.plan, E.rowptr.data(), E.colidx.data()), "pattern copy");
      }
      E.vals.resize(static_cast<size_t>(nnz));
      check(gfgpu_copy_result(E.plan, GFGPU_RESULT_VALUES, E.vals.data()), "values copy");
      add_csr(*K, off, E.rowptr, E.colidx, E.vals);
    }
  }
}

void release_plans() {
  std::lock_guard<std::mutex> lock(g_mutex);
  g_plans.clear();
}

}  // namespace gfgpu_getfem

namespace getfem {

void ga_workspace::assembly(size_type order, bool condensation) {
  const ga_workspace *w = this;
  while (w->parent_workspace) w = w->parent_workspace;
  if (w->md) w->md->nb_dof();  // sizes of the model up to date
  GMM_ASSERT1(!condensation,
              "gfgpu: static condensation through ga_workspace is not lowered for the GPU");
  GMM_ASSERT1(order <= 2, "gfgpu: assembly order " << order);
  if (order == 2) {
    if (K.use_count()) {
      gmm::clear(*K);
      gmm::resize(*K, nb_prim_dof, nb_prim_dof);
    }
  } else if (order == 1) {
    if (V.use_count()) {
      gmm::clear(*V);
      gmm::resize(*V, nb_prim_dof);
    } else {
      GMM_ASSERT1(V->size() == nb_prim_dof, "Wrong size of assembled vector in workspace");
    }
  }
  if (order == 0) assemb_t.adjust_sizes(bgeot::multi_index());
  gmm::clear(assemb_t.as_vector());
  double pot = 0.0;
  try {
    gfgpu_getfem::assemble(*this, order, order == 2 ? K.get() : nullptr,
                           order == 1 ? V.get() : nullptr, &pot);
  } catch (const std::exception &e) {
    // inside model::assembly's OpenMP section GetFEM rethrows a thread's
    // exception from a destructor, which ends the program without the
    // message: say it here first
    std::cerr << "ga_workspace::assembly(" << order << "): " << e.what() << std::endl;
    throw;
  }
  if (order == 0) assemb_t[0] += pot;
}

}  // namespace getfem
