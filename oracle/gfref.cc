// ORACLE — test infrastructure only.  A CPU restatement of GetFEM's generic
// assembly hot path for the forms of include/gfgpu.h, used by tests/, by
// __graft_entry__.smoke() and by bench.py's CPU-baseline leg as the checker.
// Nothing in the getfem_gb300 package links, loads or calls this file.
//
// What it restates (paths relative to the GetFEM source tree):
//  * ga_exec element / Gauss-point loop
//      src/getfem_generic_assembly_compile_and_exec.cc:8750-8869
//  * geometric transformation K = G grad(phi_geo), J = |det K|, B = K^{-T}
//      src/bgeot_geometric_trans.cc:270-286 (compute_K_matrix), :321-413
//  * real base gradients  grad = grad_ref . B^T
//      src/getfem_fem.cc:160-200 (pfp_grad_base_value / spec_mat_tmult_)
//  * Lagrange bases as polynomial products
//      src/getfem_fem.cc:727-781 (PK_fem_::calc_base_func), :792-826 (product)
//  * matrix accumulation elem += coeff * t over Gauss points, then
//    add_elem_matrix into a column-major matrix of sorted sparse columns,
//    dropping entries with |e| <= 1e-14 * max|elem| and skipping all-zero
//    element matrices
//      compile_and_exec.cc:5419-5470 (standard_vector), :4853-4936
//  * vector accumulation V[dof+q] += elem  (no threshold)
//      compile_and_exec.cc:4669-4735
//  * Compressible neo-Hookean PK2 law and its derivative
//      src/getfem_nonlinear_elasticity.cc:45-262 (invariants), :503-600
//      (Mooney_Rivlin_hyperelastic_law with compressible and neohookean),
//      :1770-1838 (AHL_wrapper_sigma value / derivative)
//  * OpenMP element partition with per-thread private outputs and a final
//    reduction (src/getfem_models.cc:2686-2730,
//    getfem/getfem_accumulated_distro.h:150-223)
//  * an internal im_data variable p (one value per element Gauss point) and
//    its static condensation at order 2, instruction by instruction at each
//    Gauss point: the KIQ / KQJ / KQQ tensors copied from the term
//    (compile_and_exec.cc:8219-8310), extraction of the cached residual
//    (:4804-4830), ga_instruction_condensation_sub (:5562-5671: KQQ^-1,
//    KQJpr = KQQ^-1 KQJ, RQpr = KQQ^-1 R_Q / coeff), the KQJpr rows
//    (imd_mf assembly, :5192-5230, no coeff) and RQpr written into the
//    internal rows (:4737-4765, initialize), condensation_super_K / _R
//    (:5718-5790) assembled with coeff into K and the primary rows of V
#include "gfref.h"
#include "../getfem_gb300/csrc/host/refpoly.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <stdexcept>
#include <string>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

// ------------------------------------------------------------ elements
// Base functions built and evaluated with the reference's polynomial
// arithmetic (getfem_gb300/csrc/host/refpoly.h restates bgeot::polynomial
// and PK_fem_::calc_base_func, src/getfem_fem.cc:727-749, :792-826).
using gfgpu::refpoly::Poly;

struct Element {
  int dim, kind, degree, nb;
  std::vector<Poly> base;                // nb
  std::vector<std::vector<Poly>> dbase;  // nb x dim
  Element(int dim_, int kind_, int degree_) : dim(dim_), kind(kind_), degree(degree_) {
    int K = degree;
    int ext[3] = {1, 1, 1};
    for (int d = 0; d < dim; ++d) ext[d] = K + 1;
    int c[3];
    for (c[2] = 0; c[2] < ext[2]; ++c[2])
      for (c[1] = 0; c[1] < ext[1]; ++c[1])
        for (c[0] = 0; c[0] < ext[0]; ++c[0]) {
          int s = 0;
          for (int d = 0; d < dim; ++d) s += c[d];
          if (kind == GFGPU_SIMPLEX && s > K) continue;
          base.push_back(kind == GFGPU_SIMPLEX ? gfgpu::refpoly::pk_base(dim, K, c)
                                               : gfgpu::refpoly::qk_base(dim, K, c));
        }
    nb = int(base.size());
    dbase.resize(nb);
    for (int i = 0; i < nb; ++i)
      for (int d = 0; d < dim; ++d) dbase[i].push_back(base[i].derivative(d));
  }
};

// -------------------------------------------------------------- quadrature
// Point sets of the integration methods (cubature/TRIANGLE_2.IM,
// TRIANGLE_4.IM, TETRA_2.IM, TETRA_5.IM orbits expanded; Gauss-Legendre
// IM_GAUSS1D and its tensor product IM_GAUSS_PARALLELEPIPED), in the
// reference's order of points.
struct Rule {
  int dim = 0;
  std::vector<std::vector<double>> pts;
  std::vector<double> w;
};

// approx_integration::add_point_full_symmetric for simplices
// (src/getfem_integration.cc:278-303): with pt3 = (x, 1 - sum x), every
// index vector ind (ind[0] fastest, digits 0..dim) with distinct digits gives
// the point (pt3[ind[0]], ..., pt3[ind[dim-1]]), added unless already present
// (add_point_norepeat, :271-276).  The points are listed in that order, which
// is the order im_data numbers them.
void add_full_symmetric(Rule &r, int dim, std::vector<double> x, double w) {
  std::vector<double> pt3(x);
  double last = 1.0;
  for (int k = 0; k < dim; ++k) last -= x[k];
  pt3.push_back(last);
  std::vector<int> ind(dim, 0);
  const size_t first = r.pts.size();
  for (;;) {
    std::vector<bool> used(dim + 1, false);
    bool good = true;
    for (int k = 0; k < dim; ++k) {
      if (used[ind[k]]) {
        good = false;
        break;
      }
      used[ind[k]] = true;
    }
    if (good) {
      std::vector<double> pt2(dim);
      for (int k = 0; k < dim; ++k) pt2[k] = pt3[ind[k]];
      if (std::find(r.pts.begin() + first, r.pts.end(), pt2) == r.pts.end())
        r.pts.push_back(pt2), r.w.push_back(w);
    }
    int k = 0;
    ind[0]++;
    while (ind[k] == dim + 1) {
      ind[k++] = 0;
      if (k == dim) {
        r.dim = dim;
        return;
      }
      ind[k]++;
    }
  }
}

void gauss01(int n, std::vector<double> &x, std::vector<double> &w) {
  // Golub-Welsch would do; Newton on P_n in long double is enough here.
  x.assign(n, 0);
  w.assign(n, 0);
  const long double pi = 3.141592653589793238462643383279502884L;
  for (int k = 0; k < n; ++k) {
    long double z = cosl(pi * (k + 0.75L) / (n + 0.5L)), p1 = 0, p0 = 0, dp = 1;
    for (int it = 0; it < 200; ++it) {
      p0 = 1;
      p1 = z;
      for (int j = 2; j <= n; ++j) {
        long double p2 = ((2 * j - 1) * z * p1 - (j - 1) * p0) / j;
        p0 = p1;
        p1 = p2;
      }
      if (n == 1) p0 = 1, p1 = z;
      dp = n == 1 ? 1 : n * (z * p1 - p0) / (z * z - 1);
      long double dz = p1 / dp;
      z -= dz;
      if (fabsl(dz) < 1e-20L) break;
    }
    x[k] = double((1 - z) / 2);
    w[k] = double(1 / ((1 - z * z) * dp * dp));
  }
  // IM_GAUSS1D lists its points as the symmetric pairs (x, 1 - x), x
  // ascending, then the midpoint (the order of the reference's im_points)
  std::vector<double> xs, ws;
  for (int k = 0; k < n / 2; ++k) {
    xs.push_back(x[k]), ws.push_back(w[k]);
    xs.push_back(x[n - 1 - k]), ws.push_back(w[n - 1 - k]);
  }
  if (n % 2) xs.push_back(x[n / 2]), ws.push_back(w[n / 2]);
  x = xs;
  w = ws;
}

bool make_rule(const std::string &nm, Rule &r) {
  std::string s;
  for (char c : nm)
    if (c != ' ') s += c;
  r = Rule();
  // the generating points and weights of cubature/TRIANGLE_2.IM,
  // TRIANGLE_4.IM, TETRA_2.IM and TETRA_5.IM (node type 1: full symmetric;
  // type 0: the point alone)
  if (s == "IM_TRIANGLE(2)") {
    add_full_symmetric(r, 2, {1. / 6, 1. / 6}, 1. / 6);
  } else if (s == "IM_TRIANGLE(4)") {
    add_full_symmetric(r, 2, {0.445948490915965, 0.445948490915965}, 0.111690794839005);
    add_full_symmetric(r, 2, {0.091576213509771, 0.091576213509771}, 0.054975871827661);
  } else if (s == "IM_TETRAHEDRON(2)") {
    add_full_symmetric(r, 3, {0.13819660112501052, 0.13819660112501052, 0.13819660112501052},
                       1. / 24);
  } else if (s == "IM_TETRAHEDRON(5)") {
    r.pts.push_back({0.25, 0.25, 0.25}), r.w.push_back(0.019753086419753086), r.dim = 3;
    add_full_symmetric(r, 3, {0.31979362782962991, 0.31979362782962991, 0.31979362782962991},
                       0.011511367871045398);
    add_full_symmetric(r, 3, {0.091971078052723033, 0.091971078052723033, 0.091971078052723033},
                       0.01198951396316977);
    add_full_symmetric(r, 3, {0.056350832689629156, 0.056350832689629156, 0.44364916731037084},
                       0.008818342151675485);
  } else if (s.rfind("IM_GAUSS_PARALLELEPIPED(", 0) == 0) {
    int N = 0, K = 0;
    if (sscanf(s.c_str(), "IM_GAUSS_PARALLELEPIPED(%d,%d)", &N, &K) != 2) return false;
    std::vector<double> x, w;
    gauss01(K / 2 + 1, x, w);
    int m = int(x.size());
    int nq = 1;
    for (int d = 0; d < N; ++d) nq *= m;
    r.dim = N;
    for (int t = 0; t < nq; ++t) {
      int u = t;
      std::vector<double> p(N);
      double wt = 1;
      for (int d = 0; d < N; ++d) p[d] = x[u % m], wt *= w[u % m], u /= m;
      r.pts.push_back(p);
      r.w.push_back(wt);
    }
  } else {
    return false;
  }
  return true;
}

// ------------------------------------------------- sparse matrix (rsvector)
struct Entry {
  int64_t c;
  double e;
};
using Column = std::vector<Entry>;

// add_elem_matrix (compile_and_exec.cc:4853-4936): insertion sort of the
// row DOFs, then per column either a fresh fill or a binary-search merge.
void add_elem_matrix(std::vector<Column> &K, const std::vector<int64_t> &dofs1,
                     const std::vector<int64_t> &dofs2, std::vector<size_t> &sorted,
                     const std::vector<double> &elem, double threshold) {
  size_t s1 = dofs1.size();
  sorted.resize(s1);
  for (size_t i = 0; i < s1; ++i) {
    size_t j = i;
    while (j > 0 && dofs1[i] < dofs1[sorted[j - 1]]) {
      sorted[j] = sorted[j - 1];
      --j;
    }
    sorted[j] = i;
  }
  const double *it = elem.data();
  for (size_t jc = 0; jc < dofs2.size(); ++jc, it += s1) {
    Column &col = K[dofs2[jc]];
    size_t nb = col.size();
    if (nb == 0) {
      for (size_t k : sorted)
        if (std::fabs(it[k]) > threshold) col.push_back({dofs1[k], it[k]});
      continue;
    }
    size_t ind = 0;
    for (size_t k : sorted) {
      double v = it[k];
      if (!(std::fabs(v) > threshold)) continue;
      int64_t c = dofs1[k];
      size_t count = nb - ind;
      while (count > 0) {
        size_t step = count / 2, l = ind + step;
        if (col[l].c < c) {
          ind = l + 1;
          count -= step + 1;
        } else {
          count = step;
        }
      }
      if (ind != nb && col[ind].c == c) {
        col[ind].e += v;
      } else {
        col.insert(col.begin() + ind, Entry{c, v});
        ++nb;
      }
      ++ind;
    }
  }
}

// sum of two sorted sparse columns (the reduction of per-thread copies)
void add_column(Column &dst, const Column &src) {
  Column out;
  out.reserve(dst.size() + src.size());
  size_t i = 0, j = 0;
  while (i < dst.size() || j < src.size()) {
    if (j == src.size() || (i < dst.size() && dst[i].c < src[j].c)) out.push_back(dst[i++]);
    else if (i == dst.size() || src[j].c < dst[i].c) out.push_back(src[j++]);
    else {
      out.push_back({dst[i].c, dst[i].e + src[j].e});
      ++i, ++j;
    }
  }
  dst.swap(out);
}

// ------------------------------------------------------ hyperelastic law
// compressible neo-Hookean (Mooney-Rivlin with compressible = neohookean =
// true), parameters [C1; D1]: S = 2 C1 dj1 + 2 (D1 - D1/sqrt(i3)) di3 with
// the invariants of C = I + 2E.
void inv3(const double *A, double *Ai, double &det) {
  double a0 = A[4] * A[8] - A[5] * A[7];
  double a1 = A[5] * A[6] - A[3] * A[8];
  double a2 = A[3] * A[7] - A[4] * A[6];
  det = A[0] * a0 + A[1] * a1 + A[2] * a2;
  // column-major A(i,j) = A[i + 3j]; inverse via cofactors
  double c[9];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      int i1 = (i + 1) % 3, i2 = (i + 2) % 3, j1 = (j + 1) % 3, j2 = (j + 2) % 3;
      c[i + 3 * j] = A[i1 + 3 * j1] * A[i2 + 3 * j2] - A[i1 + 3 * j2] * A[i2 + 3 * j1];
    }
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) Ai[i + 3 * j] = c[j + 3 * i] / det;
}

// S(E) (3x3, column-major) and, if gs != nullptr, dS/dE (3x3x3x3,
// gs[i + 3j + 9k + 27l] = (i,j,k,l)).  det_trans = det(I + Grad_u).
void neohookean_law(const double *E, double C1, double D1, double det_trans, double *S,
                    double *gs) {
  double C[9];
  for (int k = 0; k < 9; ++k) C[k] = 2 * E[k];
  for (int i = 0; i < 3; ++i) C[i * 4] += 1.0;
  double Ci[9], i3;
  inv3(C, Ci, i3);
  double i1 = C[0] + C[4] + C[8];
  double p13 = std::pow(std::fabs(i3), -1.0 / 3.0);
  double di3[9], dj1[9];
  for (int k = 0; k < 9; ++k) di3[k] = Ci[k] * i3;
  for (int k = 0; k < 9; ++k) dj1[k] = ((k % 4 == 0 ? 1.0 : 0.0) - i1 / (3 * i3) * di3[k]) * p13;
  double dd = D1 - D1 / std::sqrt(std::fabs(i3));
  for (int k = 0; k < 9; ++k) S[k] = 2 * C1 * dj1[k] + 2 * dd * di3[k];
  if (det_trans <= 0)
    for (int k = 0; k < 9; ++k) S[k] += 1e200 * C[k];
  if (!gs) return;
  auto Cinv = [&](int i, int j) { return Ci[i + 3 * j]; };
  auto I3 = [&](int i, int j) { return i == j ? 1.0 : 0.0; };
  double coeff1 = 1.0 / (3 * i3), coeff2 = 4 * coeff1 * coeff1 * i1;
  double A22 = D1 / (2 * std::pow(std::fabs(i3), 1.5));
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j)
      for (int k = 0; k < 3; ++k)
        for (int l = 0; l < 3; ++l) {
          double ddi3 = i3 / 2 *
                        (Cinv(j, i) * Cinv(l, k) - Cinv(j, k) * Cinv(l, i) + Cinv(i, j) * Cinv(l, k) -
                         Cinv(i, k) * Cinv(l, j));
          double ddj1 = (-i1 * coeff1 * ddi3 + di3[i + 3 * j] * di3[k + 3 * l] * coeff2 -
                         (I3(i, j) * di3[k + 3 * l] + I3(k, l) * di3[i + 3 * j]) * coeff1) *
                        p13;
          gs[i + 3 * j + 9 * k + 27 * l] =
              4 * C1 * ddj1 + 4 * dd * ddi3 + 4 * A22 * di3[i + 3 * j] * di3[k + 3 * l];
        }
}

// Strain energy of the compressible neo-Hookean law
// (getfem_nonlinear_elasticity.cc:503-527 with compressible = neohookean =
// true): W = C1 (j1 - 3) + D1 (sqrt|i3| - 1)^2 with C = I + 2E, i1 = tr C,
// i3 = det C, j1 = i1 |i3|^(-1/3); 1e200 when det(I + Grad_u) <= 0.
double neohookean_energy(const double *E, double C1, double D1, double det_trans) {
  if (det_trans <= 0) return 1e200;
  double C[9];
  for (int k = 0; k < 9; ++k) C[k] = 2 * E[k];
  for (int i = 0; i < 3; ++i) C[i * 4] += 1.0;
  double Ci[9], i3;
  inv3(C, Ci, i3);
  const double i1 = C[0] + C[4] + C[8];
  const double j1 = i1 * std::pow(std::fabs(i3), -1.0 / 3.0);
  const double r = std::sqrt(std::fabs(i3)) - 1.0;
  return C1 * (j1 - 3.0) + D1 * (r * r);
}

// ------------------------------------------------------------ assembly core
struct Problem {
  gfref_problem p;
  Element fe, gt;
  Rule rule;
  int nbg;  // geometric nodes
  // tables per Gauss point
  std::vector<double> val, grad, ggrad;  // nq x nb, nq x nb x dim, nq x nbg x dim
  Problem(const gfref_problem &pp)
      : p(pp), fe(pp.dim, pp.kind, pp.degree), gt(pp.dim, pp.kind, 1) {
    nbg = gt.nb;
  }
};

double coef_at(const gfref_problem &p, const gfgpu_coef &c, int64_t e, const int64_t *edofs,
               const double *phi, int nb) {
  switch (c.kind) {
    case GFGPU_COEF_CONST: return c.value;
    case GFGPU_COEF_ELEMENT: return c.value * p.slots[c.slot][e];
    case GFGPU_COEF_NODAL: {
      // scalar field on the scalar mesh_fem: its DOF of a node is the
      // variable's first-component DOF divided by qdim
      double s = 0;
      for (int i = 0; i < nb; ++i) s += phi[i] * p.slots[c.slot][edofs[i] / p.qdim];
      return c.value * s;
    }
    default: return 0.0;
  }
}

struct Outputs {
  std::vector<Column> K;
  std::vector<double> V;
  double E = 0;
  // internal variable: order 1 its residual; order 2 (condensation) the
  // internal solution RQpr and the coupling rows KQJpr (shared arrays,
  // indexed by element Gauss point, so threads write disjoint parts)
  bool condense = false;
  double *Vint = nullptr, *coupling = nullptr;
};

// ga_exec restated for elements [e0, e1).
void exec_range(Problem &P, int order, int64_t e0, int64_t e1, Outputs &out) {
  const gfref_problem &p = P.p;
  const int dim = p.dim, nb = P.fe.nb, nbg = P.nbg, qd = p.qdim, nq = int(P.rule.w.size());
  const int s = nb * qd;
  std::vector<double> elem(order == 2 ? size_t(s) * s : size_t(s));
  std::vector<double> G(nbg * dim), g(nb * dim), t(order == 2 ? size_t(s) * s : size_t(s));
  // condensation: the condensed part of the element matrix (assembled by its
  // own instruction, with its own threshold) and the condensed vector
  std::vector<double> elemC(out.condense ? size_t(s) * s : 0), elemR(out.condense ? s : 0);
  std::vector<double> kiq(s), kqj(s);
  std::vector<int64_t> dofs(s);
  std::vector<size_t> sorted;
  for (int64_t e = e0; e < e1; ++e) {
    for (int v = 0; v < nbg; ++v)
      for (int d = 0; d < dim; ++d) G[v * dim + d] = p.points[p.cvpts[e * nbg + v] * dim + d];
    const int64_t *edofs = p.dofs + e * nb;
    std::fill(elem.begin(), elem.end(), 0.0);
    std::fill(elemC.begin(), elemC.end(), 0.0);
    std::fill(elemR.begin(), elemR.end(), 0.0);
    for (int q = 0; q < nq; ++q) {
      // K(d,m) = sum_v G(d,v) dphi_v/dxi_m ; J = |det K| ; B = K^{-T}
      double Km[9] = {0}, B[9];
      const double *gg = &P.ggrad[size_t(q) * nbg * dim];
      for (int d = 0; d < dim; ++d)
        for (int m = 0; m < dim; ++m) {
          double a = 0;
          for (int v = 0; v < nbg; ++v) a += G[v * dim + d] * gg[v * dim + m];
          Km[d + dim * m] = a;
        }
      double det;
      if (dim == 2) {
        det = Km[0] * Km[3] - Km[1] * Km[2];
        B[0] = Km[3] / det, B[1] = -Km[2] / det, B[2] = -Km[1] / det, B[3] = Km[0] / det;
      } else {
        double Ki[9];
        inv3(Km, Ki, det);
        // B = K^{-T}: B(d,m) = Ki(m,d)
        for (int d = 0; d < 3; ++d)
          for (int m = 0; m < 3; ++m) B[d + 3 * m] = Ki[m + 3 * d];
      }
      if (det == 0) throw std::runtime_error("Non invertible matrix");
      double coeff = std::fabs(det) * P.rule.w[q];
      const double *phi = &P.val[size_t(q) * nb];
      const double *gr = &P.grad[size_t(q) * nb * dim];
      for (int i = 0; i < nb; ++i)
        for (int d = 0; d < dim; ++d) {
          double a = 0;
          for (int m = 0; m < dim; ++m) a += gr[i * dim + m] * B[d + dim * m];
          g[i * dim + d] = a;
        }
      std::fill(t.begin(), t.end(), 0.0);
      for (int ti = 0; ti < p.form.n_terms; ++ti) {
        const gfgpu_term &T = p.form.terms[ti];
        const double sc = T.scale;
        if (T.kind == GFGPU_TERM_GRADGRAD) {
          double c0 = coef_at(p, T.c[0], e, edofs, phi, nb) * sc;
          double c1 = coef_at(p, T.c[1], e, edofs, phi, nb) * sc;
          double c2 = coef_at(p, T.c[2], e, edofs, phi, nb) * sc;
          if (order == 2) {
            // t[(i,a),(j,b)] = c0 g_ia g_jb + c1 d_ab g_i.g_j + c2 g_ib g_ja
            for (int j = 0; j < nb; ++j) {
              const double *gj = &g[j * dim];
              for (int i = 0; i < nb; ++i) {
                const double *gi = &g[i * dim];
                double gg = 0;
                for (int k = 0; k < dim; ++k) gg += gi[k] * gj[k];
                gg *= c1;
                if (qd == 1) {
                  t[size_t(j) * s + i] += gg;
                  continue;
                }
                for (int b = 0; b < qd; ++b) {
                  double *tc = &t[size_t(j * qd + b) * s + i * qd];
                  for (int a = 0; a < qd; ++a)
                    tc[a] += c0 * gi[a] * gj[b] + c2 * gi[b] * gj[a] + (a == b ? gg : 0.0);
                }
              }
            }
          } else {
            // Grad_u (qd x dim)
            double Gu[9] = {0};
            for (int j = 0; j < nb; ++j)
              for (int b = 0; b < qd; ++b) {
                double uj = p.slots[GFGPU_SLOT_U][edofs[j] + b];
                for (int l = 0; l < dim; ++l) Gu[b * dim + l] += uj * g[j * dim + l];
              }
            double div = 0;
            if (qd > 1)
              for (int a = 0; a < qd; ++a) div += Gu[a * dim + a];
            for (int i = 0; i < nb; ++i)
              for (int a = 0; a < qd; ++a) {
                double v = 0;
                for (int k = 0; k < dim; ++k) {
                  double Dk = c1 * Gu[a * dim + k];
                  if (qd > 1) Dk += (k == a ? c0 * div : 0.0) + c2 * Gu[k * dim + a];
                  v += Dk * g[i * dim + k];
                }
                if (order == 1) t[i * qd + a] += v;
              }
            if (order == 0) {
              // the bilinear form at (u, u): D:Grad_u:Grad_u
              double v = 0;
              for (int a = 0; a < qd; ++a)
                for (int k = 0; k < dim; ++k) {
                  double Dk = c1 * Gu[a * dim + k];
                  if (qd > 1) Dk += (k == a ? c0 * div : 0.0) + c2 * Gu[k * dim + a];
                  v += Dk * Gu[a * dim + k];
                }
              t[0] += v;
            }
          }
        } else if (T.kind == GFGPU_TERM_GRADGRAD_TENSOR) {
          // (D : Grad_u) : Grad_Test_u, D[(a,k),(b,l)] = tensor[(a*dim+k)*nd + b*dim+l]
          const double c =
              (T.c[0].kind == GFGPU_COEF_NONE ? 1.0 : coef_at(p, T.c[0], e, edofs, phi, nb)) * sc;
          const double *D = p.form.tensor;
          const int nd = qd * dim;
          if (order == 2) {
            for (int j = 0; j < nb; ++j)
              for (int b = 0; b < qd; ++b)
                for (int i = 0; i < nb; ++i)
                  for (int a = 0; a < qd; ++a) {
                    double v = 0;
                    for (int k = 0; k < dim; ++k) {
                      double w = 0;
                      for (int l = 0; l < dim; ++l)
                        w += D[(a * dim + k) * nd + b * dim + l] * g[j * dim + l];
                      v += w * g[i * dim + k];
                    }
                    t[size_t(j * qd + b) * s + i * qd + a] += c * v;
                  }
          } else {
            double Gu[9] = {0};
            for (int j = 0; j < nb; ++j)
              for (int b = 0; b < qd; ++b) {
                double uj = p.slots[GFGPU_SLOT_U][edofs[j] + b];
                for (int l = 0; l < dim; ++l) Gu[b * dim + l] += uj * g[j * dim + l];
              }
            // (D : Grad_u)[a,k]
            double DG[9] = {0};
            for (int r = 0; r < nd; ++r)
              for (int q2 = 0; q2 < nd; ++q2) DG[r] += D[r * nd + q2] * Gu[q2];
            if (order == 1) {
              for (int i = 0; i < nb; ++i)
                for (int a = 0; a < qd; ++a) {
                  double v = 0;
                  for (int k = 0; k < dim; ++k) v += DG[a * dim + k] * g[i * dim + k];
                  t[i * qd + a] += c * v;
                }
            } else {
              double v = 0;
              for (int r = 0; r < nd; ++r) v += DG[r] * Gu[r];
              t[0] += c * v;
            }
          }
        } else if (T.kind == GFGPU_TERM_MASS) {
          double c0 = coef_at(p, T.c[0], e, edofs, phi, nb) * sc;
          if (order == 2) {
            for (int j = 0; j < nb; ++j)
              for (int b = 0; b < qd; ++b)
                for (int i = 0; i < nb; ++i) t[size_t(j * qd + b) * s + i * qd + b] += c0 * phi[i] * phi[j];
          } else {
            double uq[3] = {0, 0, 0};
            for (int j = 0; j < nb; ++j)
              for (int b = 0; b < qd; ++b) uq[b] += phi[j] * p.slots[GFGPU_SLOT_U][edofs[j] + b];
            if (order == 1) {
              for (int i = 0; i < nb; ++i)
                for (int a = 0; a < qd; ++a) t[i * qd + a] += c0 * uq[a] * phi[i];
            } else {
              for (int a = 0; a < qd; ++a) t[0] += c0 * uq[a] * uq[a];
            }
          }
        } else if (T.kind == GFGPU_TERM_SOURCE) {
          double c0 = (T.c[0].kind == GFGPU_COEF_NONE ? 1.0 : coef_at(p, T.c[0], e, edofs, phi, nb)) * sc;
          double f[3] = {0, 0, 0};
          for (int j = 0; j < nb; ++j)
            for (int b = 0; b < qd; ++b) f[b] += phi[j] * p.slots[T.field_slot][edofs[j] + b];
          if (order == 1) {
            for (int i = 0; i < nb; ++i)
              for (int a = 0; a < qd; ++a) t[i * qd + a] += c0 * f[a] * phi[i];
          } else if (order == 0) {
            for (int j = 0; j < nb; ++j)
              for (int a = 0; a < qd; ++a) t[0] += c0 * f[a] * phi[j] * p.slots[GFGPU_SLOT_U][edofs[j] + a];
          }
        } else if (T.kind == GFGPU_TERM_INTERNAL_P) {
          // u equation (c0 p Id):Grad_Test_u, p equation
          // scale (p + c2 p^3 + c1 Div_u) Test_p; p at element Gauss point q
          const double sp = coef_at(p, T.c[0], e, edofs, phi, nb);
          const double kb = coef_at(p, T.c[1], e, edofs, phi, nb);
          const double c3 = coef_at(p, T.c[2], e, edofs, phi, nb);
          const int64_t iq = e * nq + q;
          const double pv = p.slots[T.field_slot][iq];
          if (order == 1) {
            double div = 0;
            for (int j = 0; j < nb; ++j)
              for (int b = 0; b < qd; ++b) div += p.slots[GFGPU_SLOT_U][edofs[j] + b] * g[j * dim + b];
            for (int i = 0; i < nb; ++i)
              for (int a = 0; a < qd; ++a) t[i * qd + a] += (sp * pv) * g[i * dim + a];
            // ga_instruction_vector_assembly_imd: V[I + index] += coeff * t
            out.Vint[iq] += coeff * (sc * ((pv + c3 * (pv * pv * pv)) + kb * div));
          } else if (order == 2 && out.condense) {
            for (int i = 0; i < nb; ++i)
              for (int a = 0; a < qd; ++a) {
                kiq[i * qd + a] = sp * g[i * dim + a];        // K_IQ: d/dp of the u equation
                kqj[i * qd + a] = sc * (kb * g[i * dim + a]); // K_QJ: d/du of the p equation
              }
            const double kqq = sc * (1.0 + c3 * (3.0 * (pv * pv)));  // K_QQ
            const double inv = 1.0 / kqq;                              // lu_inverse, 1 x 1
            const double rq = p.slots[T.aux_slot][iq];                 // cached residual
            const double rqpr = (0.0 + inv * rq) / coeff;
            double *crow = out.coupling + size_t(iq) * s;
            for (int c = 0; c < s; ++c) crow[c] = 0.0 + inv * kqj[c];   // KQJpr
            out.Vint[iq] = rqpr;
            for (int j = 0; j < s; ++j)
              for (int i = 0; i < s; ++i) elemC[size_t(j) * s + i] += coeff * (0.0 - kiq[i] * crow[j]);
            for (int i = 0; i < s; ++i) elemR[i] += coeff * (0.0 - kiq[i] * rqpr);
          }
        } else if (T.kind == GFGPU_TERM_NEOHOOKEAN) {
          double C1 = coef_at(p, T.c[0], e, edofs, phi, nb);
          double D1 = coef_at(p, T.c[1], e, edofs, phi, nb);
          // Gu(i,j) = d u_i / d x_j, column-major Gu[i + 3j]
          double Gu[9] = {0};
          for (int j = 0; j < nb; ++j)
            for (int b = 0; b < 3; ++b) {
              double uj = p.slots[GFGPU_SLOT_U][edofs[j] + b];
              for (int l = 0; l < 3; ++l) Gu[b + 3 * l] += uj * g[j * 3 + l];
            }
          double E[9], F[9];
          for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) {
              double a = 0;
              for (int m = 0; m < 3; ++m) a += Gu[m + 3 * i] * Gu[m + 3 * j];
              E[i + 3 * j] = 0.5 * (a + Gu[i + 3 * j] + Gu[j + 3 * i]);
              F[i + 3 * j] = Gu[i + 3 * j] + (i == j ? 1.0 : 0.0);
            }
          double detF = F[0] * (F[4] * F[8] - F[5] * F[7]) - F[3] * (F[1] * F[8] - F[2] * F[7]) +
                        F[6] * (F[1] * F[5] - F[2] * F[4]);
          double S[9], gs[81];
          if (order == 0) {
            t[0] += sc * neohookean_energy(E, C1, D1, detF);
            continue;
          }
          neohookean_law(E, C1, D1, detF, S, order == 2 ? gs : nullptr);
          if (order == 1) {
            // (F S)(a,k) Grad_Test_u(a,k)
            for (int i = 0; i < nb; ++i)
              for (int a = 0; a < 3; ++a) {
                double v = 0;
                for (int k = 0; k < 3; ++k) {
                  double FS = 0;
                  for (int m = 0; m < 3; ++m) FS += F[a + 3 * m] * S[m + 3 * k];
                  v += FS * g[i * 3 + k];
                }
                t[i * 3 + a] += sc * v;
              }
          } else if (order == 2) {
            // A[a,k,b,l] = d_ab S(l,k) + sum_{m,n} F(a,m) F(b,n) gs(m,k,n,l)
            double A[81];
            for (int a = 0; a < 3; ++a)
              for (int k = 0; k < 3; ++k)
                for (int b = 0; b < 3; ++b)
                  for (int l = 0; l < 3; ++l) {
                    double v = (a == b) ? S[l + 3 * k] : 0.0;
                    for (int m = 0; m < 3; ++m)
                      for (int n = 0; n < 3; ++n)
                        v += F[a + 3 * m] * F[b + 3 * n] * gs[m + 3 * k + 9 * n + 27 * l];
                    A[a + 3 * k + 9 * b + 27 * l] = v;
                  }
            for (int j = 0; j < nb; ++j)
              for (int b = 0; b < 3; ++b)
                for (int i = 0; i < nb; ++i)
                  for (int a = 0; a < 3; ++a) {
                    double v = 0;
                    for (int k = 0; k < 3; ++k)
                      for (int l = 0; l < 3; ++l) v += A[a + 3 * k + 9 * b + 27 * l] * g[i * 3 + k] * g[j * 3 + l];
                    t[size_t(j * 3 + b) * s + i * 3 + a] += sc * v;
                  }
          }
        }
      }
      if (order == 0) {
        out.E += t[0] * coeff;
      } else {
        for (size_t k = 0; k < t.size(); ++k) elem[k] += coeff * t[k];
      }
    }
    if (order == 2) {
      for (int i = 0; i < nb; ++i)
        for (int a = 0; a < qd; ++a) dofs[i * qd + a] = edofs[i] + a;
      double ninf = 0;
      for (double v : elem) ninf = std::max(ninf, std::fabs(v));
      if (ninf != 0) add_elem_matrix(out.K, dofs, dofs, sorted, elem, ninf * 1e-14);
      if (out.condense) {
        double ninfc = 0;
        for (double v : elemC) ninfc = std::max(ninfc, std::fabs(v));
        if (ninfc != 0) add_elem_matrix(out.K, dofs, dofs, sorted, elemC, ninfc * 1e-14);
        for (int k = 0; k < s; ++k) out.V[dofs[k]] += elemR[k];
      }
    } else if (order == 1) {
      for (int i = 0; i < nb; ++i)
        for (int a = 0; a < qd; ++a) out.V[edofs[i] + a] += elem[i * qd + a];
    }
  }
}

Problem *prepare(const gfref_problem *pp) {
  Problem *P = new Problem(*pp);
  if (!make_rule(pp->im, P->rule)) {
    delete P;
    return nullptr;
  }
  const int dim = pp->dim, nb = P->fe.nb, nbg = P->nbg, nq = int(P->rule.w.size());
  P->val.resize(size_t(nq) * nb);
  P->grad.resize(size_t(nq) * nb * dim);
  P->ggrad.resize(size_t(nq) * nbg * dim);
  for (int q = 0; q < nq; ++q) {
    const double *x = P->rule.pts[q].data();
    for (int i = 0; i < nb; ++i) {
      P->val[q * nb + i] = P->fe.base[i].eval(x);
      for (int d = 0; d < dim; ++d) P->grad[(q * nb + i) * dim + d] = P->fe.dbase[i][d].eval(x);
    }
    for (int v = 0; v < nbg; ++v)
      for (int d = 0; d < dim; ++d) P->ggrad[(q * nbg + v) * dim + d] = P->gt.dbase[v][d].eval(x);
  }
  return P;
}

struct MatrixResult {
  int64_t n = 0;
  std::vector<int64_t> rowptr;
  std::vector<int64_t> colidx;
  std::vector<double> vals;
};

int nthreads_of(int requested) {
#ifdef _OPENMP
  return requested > 0 ? requested : omp_get_max_threads();
#else
  (void)requested;
  return 1;
#endif
}

}  // namespace

extern "C" {

int gfref_tables(int dim, int kind, int degree, const char *im, int *nq, double *pts, double *w,
                 double *val, double *grad) {
  Rule r;
  if (!make_rule(im, r)) return 2;
  *nq = int(r.w.size());
  if (!pts) return 0;
  Element fe(dim, kind, degree);
  for (int q = 0; q < *nq; ++q) {
    for (int d = 0; d < dim; ++d) pts[q * dim + d] = r.pts[q][d];
    w[q] = r.w[q];
    for (int i = 0; i < fe.nb; ++i) {
      val[q * fe.nb + i] = fe.base[i].eval(r.pts[q].data());
      for (int d = 0; d < dim; ++d) grad[(q * fe.nb + i) * dim + d] = fe.dbase[i][d].eval(r.pts[q].data());
    }
  }
  return 0;
}

void *gfref_assemble_condensed(const gfref_problem *pp, int nthreads, int64_t *nnz, double *V,
                               double *Vint, double *coupling);

void *gfref_assemble_matrix(const gfref_problem *pp, int nthreads, int64_t *nnz) {
  return gfref_assemble_condensed(pp, nthreads, nnz, nullptr, nullptr, nullptr);
}

// Order 2; with V != nullptr the static condensation of the internal
// variable: K condensed, V (n_dof) += the condensed primary rows, Vint
// (n_elements * nq) = RQpr, coupling (n_elements * nq * nb * qdim, element
// DOFs in local order) = KQJpr.
void *gfref_assemble_condensed(const gfref_problem *pp, int nthreads, int64_t *nnz, double *V,
                               double *Vint, double *coupling) {
  Problem *P = prepare(pp);
  if (!P) return nullptr;
  int T = nthreads_of(nthreads);
  std::vector<Outputs> outs(T);
  int64_t E = pp->n_elements;
  bool failed = false;
#pragma omp parallel num_threads(T)
  {
    int tid = 0;
#ifdef _OPENMP
    tid = omp_get_thread_num();
#endif
    outs[tid].K.assign(pp->n_dof, Column());
    if (V) {
      outs[tid].condense = true;
      outs[tid].V.assign(pp->n_dof, 0.0);
      outs[tid].Vint = Vint;
      outs[tid].coupling = coupling;
    }
    int64_t e0 = E * tid / T, e1 = E * (tid + 1) / T;
    try {
      exec_range(*P, 2, e0, e1, outs[tid]);
    } catch (...) {
#pragma omp critical
      failed = true;
    }
  }
  // reduction of the per-thread copies, column by column
  for (int t = 1; t < T; ++t)
    for (int64_t c = 0; c < pp->n_dof; ++c)
      if (!outs[t].K[c].empty()) add_column(outs[0].K[c], outs[t].K[c]);
  if (V)
    for (int t = 0; t < T; ++t)
      for (int64_t i = 0; i < pp->n_dof; ++i) V[i] += outs[t].V[i];
  delete P;
  if (failed) return nullptr;
  MatrixResult *M = new MatrixResult;
  int64_t n = pp->n_dof;
  M->n = n;
  M->rowptr.assign(n + 1, 0);
  for (int64_t c = 0; c < n; ++c)
    for (auto &en : outs[0].K[c]) M->rowptr[en.c + 1]++;
  for (int64_t i = 0; i < n; ++i) M->rowptr[i + 1] += M->rowptr[i];
  M->colidx.resize(M->rowptr[n]);
  M->vals.resize(M->rowptr[n]);
  std::vector<int64_t> fill(M->rowptr.begin(), M->rowptr.end() - 1);
  for (int64_t c = 0; c < n; ++c)
    for (auto &en : outs[0].K[c]) {
      int64_t k = fill[en.c]++;
      M->colidx[k] = c;
      M->vals[k] = en.e;
    }
  *nnz = M->rowptr[n];
  return M;
}

void gfref_matrix_copy(void *h, int64_t *rowptr, int64_t *colidx, double *vals) {
  MatrixResult *M = static_cast<MatrixResult *>(h);
  std::memcpy(rowptr, M->rowptr.data(), sizeof(int64_t) * M->rowptr.size());
  std::memcpy(colidx, M->colidx.data(), sizeof(int64_t) * M->colidx.size());
  std::memcpy(vals, M->vals.data(), sizeof(double) * M->vals.size());
}

void gfref_matrix_free(void *h) { delete static_cast<MatrixResult *>(h); }

int gfref_assemble_vector_internal(const gfref_problem *pp, int nthreads, double *V,
                                   double *Vint);

int gfref_assemble_vector(const gfref_problem *pp, int nthreads, double *V) {
  return gfref_assemble_vector_internal(pp, nthreads, V, nullptr);
}

// Order 1; Vint (n_elements * nq) += the residual of an internal variable.
int gfref_assemble_vector_internal(const gfref_problem *pp, int nthreads, double *V,
                                   double *Vint) {
  for (int t = 0; t < pp->form.n_terms; ++t)
    if (pp->form.terms[t].kind == GFGPU_TERM_INTERNAL_P && !Vint) return 3;
  Problem *P = prepare(pp);
  if (!P) return 2;
  int T = nthreads_of(nthreads);
  std::vector<Outputs> outs(T);
  int64_t E = pp->n_elements;
  bool failed = false;
#pragma omp parallel num_threads(T)
  {
    int tid = 0;
#ifdef _OPENMP
    tid = omp_get_thread_num();
#endif
    outs[tid].V.assign(pp->n_dof, 0.0);
    outs[tid].Vint = Vint;
    int64_t e0 = E * tid / T, e1 = E * (tid + 1) / T;
    try {
      exec_range(*P, 1, e0, e1, outs[tid]);
    } catch (...) {
#pragma omp critical
      failed = true;
    }
  }
  delete P;
  if (failed) return 4;
  for (int t = 0; t < T; ++t)
    for (int64_t i = 0; i < pp->n_dof; ++i) V[i] += outs[t].V[i];
  return 0;
}

int gfref_assemble_potential(const gfref_problem *pp, int nthreads, double *E) {
  Problem *P = prepare(pp);
  if (!P) return 2;
  int T = nthreads_of(nthreads);
  std::vector<Outputs> outs(T);
  int64_t NE = pp->n_elements;
  bool failed = false;
#pragma omp parallel num_threads(T)
  {
    int tid = 0;
#ifdef _OPENMP
    tid = omp_get_thread_num();
#endif
    int64_t e0 = NE * tid / T, e1 = NE * (tid + 1) / T;
    try {
      exec_range(*P, 0, e0, e1, outs[tid]);
    } catch (...) {
#pragma omp critical
      failed = true;
    }
  }
  delete P;
  if (failed) return 4;
  double s = 0;
  for (int t = 0; t < T; ++t) s += outs[t].E;
  *E = s;
  return 0;
}

}  // extern "C"
