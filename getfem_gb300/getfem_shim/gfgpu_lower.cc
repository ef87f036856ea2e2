// Lowering of GetFEM's analysed GWFL trees to gfgpu_form.
//
// A tree after semantic analysis and derivation (ga_semantic_analysis,
// src/getfem_generic_assembly_semantic.cc; the derivative loop of
// ga_workspace::add_tree, src/getfem_generic_assembly_workspace.cc:439-543)
// is evaluated symbolically at one integration point: every tensor entry is
// a polynomial in
//   test-function symbols   Test_u[a], Grad_Test_u[a,k] (test 1), the same
//                           for Test2 (test 2),
//   variable symbols        u[a], Grad_u[a,k],
//   data symbols            the value of a fem datum at the point (one per
//                           component),
// with the tensor operations of GWFL (the shapes the reference's compiler
// gives them, compile_and_exec.cc:5826-7700): + - unary -, * (scalar
// scaling, matrix-vector, matrix-matrix, order-4 by order-2), . (last index
// with first), : (last two with first two), @ (tensor product), .* ./
// (componentwise), / (by a constant), ', Sym, Skew, Trace, Deviator, Div.
// Fixed-size constants and folded constants enter as numbers.  The
// polynomial of the root is then matched against the descriptor families:
//
//   order 2   sum of Test x Test2 monomials: D[(a,k),(b,l)] of
//             Grad_Test_u[a,k] Grad_Test2_u[b,l] must be the isotropic
//             c0 d_ak d_bl + c1 d_ab d_kl + c2 d_al d_kb and the
//             Test_u[a] Test2_u[b] part cm d_ab, each coefficient a constant
//             plus data symbols with one factor each (GRADGRAD / MASS terms);
//   order 1   the same with u / Grad_u in place of Test2 (K u), plus
//             alpha f[a] Test_u[a] with f a field on the variable's mesh_fem
//             (SOURCE);
//   order 0   a potential quadratic in (u, Grad_u), read by polarisation
//             (the bilinear part B, 2 B for its derivative), plus alpha f.u.
//
// The compressible neo-Hookean brick form
//   ((Id(meshdim)+Grad_u)*(Compressible_Neo_Hookean_PK2(Grad_u,[C1;D1]))):Grad_Test_u
// (src/getfem_nonlinear_elasticity.cc:2319-2320) and the potential
// Compressible_Neo_Hookean_potential(Grad_u,[C1;D1]) are matched by the
// structure of their analysed trees; their derivative trees (order 2 of the
// brick form, orders 1 and 2 of the potential) are accepted as the
// NEOHOOKEAN term when the tree they were derived from (same expression) was
// matched.  Everything else is rejected.
#include <algorithm>
#include <cmath>
#include <map>
#include <set>
#include <sstream>

#include "getfem/getfem_generic_assembly_tree.h"
#include "gfgpu_getfem.h"

namespace gfgpu_getfem {

namespace {

using bgeot::size_type;
using getfem::ga_tree_node;
using getfem::pga_tree_node;

[[noreturn]] void reject(const std::string &why) {
  throw gmm::gmm_error("gfgpu: expression not lowered for the GPU (no CPU fallback): " + why);
}

// ------------------------------------------------------------ symbols

enum SymKind { T1V = 0, T1G, T2V, T2G, UV, UG, DATA };

struct Sym {
  int kind, a, k, data;  // component, derivative, data index (DATA)
  bool operator<(const Sym &o) const {
    return std::tie(kind, a, k, data) < std::tie(o.kind, o.a, o.k, o.data);
  }
};

using Mono = std::vector<int>;  // sorted symbol ids
using Poly = std::map<Mono, double>;

struct Tensor {
  std::vector<size_t> sz;  // sizes, first index fastest
  std::vector<Poly> v;
  size_t order() const { return sz.size(); }
  size_t size() const { return v.size(); }
};

Tensor make(const std::vector<size_t> &sz) {
  Tensor t;
  t.sz = sz;
  size_t n = 1;
  for (size_t s : sz) n *= s;
  t.v.assign(n, Poly{});
  return t;
}

Poly pconst(double c) {
  Poly p;
  if (c != 0.0) p[Mono{}] = c;
  return p;
}

void padd(Poly &a, const Poly &b, double s = 1.0) {
  for (const auto &kv : b) {
    double &x = a[kv.first];
    x += s * kv.second;
    if (x == 0.0) a.erase(kv.first);
  }
}

Poly pmul(const Poly &a, const Poly &b) {
  Poly r;
  for (const auto &x : a)
    for (const auto &y : b) {
      Mono m = x.first;
      m.insert(m.end(), y.first.begin(), y.first.end());
      std::sort(m.begin(), m.end());
      double &z = r[m];
      z += x.second * y.second;
      if (z == 0.0) r.erase(m);
    }
  return r;
}

bool pconstant(const Poly &p, double &c) {
  c = 0.0;
  for (const auto &kv : p) {
    if (!kv.first.empty()) return false;
    c = kv.second;
  }
  return true;
}

// ----------------------------------------------------------- context

struct DataInfo {
  std::string name;
  int kind;  // GFGPU_COEF_ELEMENT, GFGPU_COEF_NODAL or 0 (field on the variable's mesh_fem)
  size_t q;  // components
};

struct Ctx {
  const getfem::ga_workspace &ws;
  std::string var;
  size_t Q = 1, N = 3;  // variable components, mesh dimension
  const getfem::mesh_fem *mf = nullptr;
  std::vector<Sym> syms;
  std::map<Sym, int> ids;
  std::vector<DataInfo> data;
  std::map<std::string, int> data_of;

  int sym(int kind, int a, int k = 0, int d = -1) {
    Sym s{kind, a, k, d};
    auto it = ids.find(s);
    if (it != ids.end()) return it->second;
    const int id = int(syms.size());
    syms.push_back(s);
    ids[s] = id;
    return id;
  }
  Poly psym(int kind, int a, int k = 0, int d = -1) {
    Poly p;
    p[Mono{sym(kind, a, k, d)}] = 1.0;
    return p;
  }
};

// The fem DOFs of mf2 are those of the variable's mesh_fem, component by
// component (same fem on every element, DOFs numbered alike).
bool same_nodes(const getfem::mesh_fem &a, const getfem::mesh_fem &b) {
  if (&a.linked_mesh() != &b.linked_mesh()) return false;
  const size_t qa = a.get_qdim(), qb = b.get_qdim();
  if (a.nb_basic_dof() / qa != b.nb_basic_dof() / qb) return false;
  for (dal::bv_visitor cv(a.convex_index()); !cv.finished(); ++cv) {
    if (!b.convex_index().is_in(cv) || a.fem_of_element(cv) != b.fem_of_element(cv)) return false;
    const auto &da = a.ind_scalar_basic_dof_of_element(cv);
    const auto &db = b.ind_scalar_basic_dof_of_element(cv);
    if (da.size() != db.size()) return false;
    for (size_t i = 0; i < da.size(); ++i)
      if (da[i] / qa != db[i] / qb) return false;
  }
  return true;
}

bool is_p0(const getfem::mesh_fem &m) {
  if (m.get_qdim() != 1) return false;
  for (dal::bv_visitor cv(m.convex_index()); !cv.finished(); ++cv)
    if (m.nb_basic_dof_of_element(cv) != 1) return false;
  return m.nb_basic_dof() == m.convex_index().card();
}

// A named datum used by value: a number tensor (fixed-size constant) or
// data symbols (fem data).
Tensor datum(Ctx &C, const std::string &name) {
  const auto &ws = C.ws;
  if (name == C.var) {
    Tensor t = make(C.Q == 1 ? std::vector<size_t>{} : std::vector<size_t>{C.Q});
    for (size_t a = 0; a < C.Q; ++a) t.v[a] = C.psym(UV, int(a));
    return t;
  }
  if (!ws.variable_exists(name)) reject("unknown name " + name);
  if (ws.associated_im_data(name)) reject(name + " is im_data (internal variables are not lowered here)");
  const getfem::mesh_fem *mf = ws.associated_mf(name);
  if (!mf) {
    // fixed-size constant: its value, as a number tensor
    if (!ws.is_constant(name)) reject(name + " is a variable without a mesh_fem");
    const auto &val = ws.value(name);
    const bgeot::multi_index qd = ws.qdims(name);
    std::vector<size_t> sz;
    for (size_t i = 0; i < qd.size(); ++i)
      if (!(qd.size() == 1 && qd[0] == 1)) sz.push_back(qd[i]);
    Tensor t = make(sz);
    if (t.size() != gmm::vect_size(val)) reject("size of constant " + name);
    for (size_t i = 0; i < t.size(); ++i) t.v[i] = pconst(val[i]);
    return t;
  }
  if (!ws.is_constant(name)) reject("variable " + name + " besides " + C.var);
  int kind;
  size_t q = mf->get_qdim();
  if (q == 1 && is_p0(*mf)) kind = GFGPU_COEF_ELEMENT;
  else if (q == 1 && same_nodes(*mf, *C.mf)) kind = GFGPU_COEF_NODAL;
  else if (q == C.Q && same_nodes(*mf, *C.mf)) kind = 0;
  else reject("datum " + name + " is neither per element, nor on the variable's nodes");
  if (ws.qdims(name).size() > 1) reject("tensor-valued datum " + name);
  auto it = C.data_of.find(name);
  int d;
  if (it == C.data_of.end()) {
    d = int(C.data.size());
    C.data.push_back({name, kind, q});
    C.data_of[name] = d;
  } else {
    d = it->second;
  }
  Tensor t = make(q == 1 ? std::vector<size_t>{} : std::vector<size_t>{q});
  for (size_t a = 0; a < q; ++a) t.v[a] = C.psym(DATA, int(a), 0, d);
  return t;
}

Tensor add(const Tensor &A, const Tensor &B, double s) {
  if (A.sz != B.sz) reject("sizes of a sum");
  Tensor r = A;
  for (size_t i = 0; i < r.size(); ++i) padd(r.v[i], B.v[i], s);
  return r;
}

Tensor scale(const Tensor &A, const Poly &s) {
  Tensor r = A;
  for (auto &p : r.v) p = pmul(p, s);
  return r;
}

// sum over the last n indices of A and the first n of B
Tensor contract(const Tensor &A, const Tensor &B, size_t n) {
  if (A.order() < n || B.order() < n) reject("contraction of a low-order tensor");
  size_t m = 1;
  for (size_t i = 0; i < n; ++i) {
    if (A.sz[A.order() - n + i] != B.sz[i]) reject("sizes of a contraction");
    m *= B.sz[i];
  }
  std::vector<size_t> sz(A.sz.begin(), A.sz.end() - n);
  sz.insert(sz.end(), B.sz.begin() + n, B.sz.end());
  Tensor r = make(sz);
  const size_t na = A.size() / m, nb = B.size() / m;
  // first index fastest: A = (free_a, contracted), B = (contracted, free_b)
  for (size_t ib = 0; ib < nb; ++ib)
    for (size_t ia = 0; ia < na; ++ia) {
      Poly &acc = r.v[ia + na * ib];
      for (size_t c = 0; c < m; ++c) padd(acc, pmul(A.v[ia + na * c], B.v[c + m * ib]));
    }
  return r;
}

Tensor transpose(const Tensor &A) {
  if (A.order() == 0) return A;
  if (A.order() != 2) reject("transpose of a tensor of order " + std::to_string(A.order()));
  Tensor r = make({A.sz[1], A.sz[0]});
  for (size_t i = 0; i < A.sz[0]; ++i)
    for (size_t j = 0; j < A.sz[1]; ++j) r.v[j + A.sz[1] * i] = A.v[i + A.sz[0] * j];
  return r;
}

Poly trace(const Tensor &A) {
  if (A.order() != 2 || A.sz[0] != A.sz[1]) reject("trace of a non-square tensor");
  Poly p;
  for (size_t i = 0; i < A.sz[0]; ++i) padd(p, A.v[i + A.sz[0] * i]);
  return p;
}

Tensor scalar_tensor(const Poly &p) {
  Tensor t = make({});
  t.v[0] = p;
  return t;
}

bool is_scalar(const Tensor &t) { return t.size() == 1 && t.order() <= 1; }

struct NHOp {};  // a neo-Hookean operator node (matched by structure only)

Tensor eval(Ctx &C, const pga_tree_node n);

Tensor eval_test(Ctx &C, const pga_tree_node n, bool grad, bool div) {
  if (n->name != C.var) reject("test function of " + n->name + " (the group's variable is " + C.var + ")");
  const int t = int(n->test_function_type);
  if (t != 1 && t != 2) reject("test function type");
  const int kv = t == 1 ? T1V : T2V, kg = t == 1 ? T1G : T2G;
  if (div) {
    if (C.Q != C.N) reject("Div of a field with qdim != dim");
    Poly p;
    for (size_t a = 0; a < C.Q; ++a) padd(p, C.psym(kg, int(a), int(a)));
    return scalar_tensor(p);
  }
  if (!grad) {
    Tensor r = make(C.Q == 1 ? std::vector<size_t>{} : std::vector<size_t>{C.Q});
    for (size_t a = 0; a < C.Q; ++a) r.v[a] = C.psym(kv, int(a));
    return r;
  }
  Tensor r = make(C.Q == 1 ? std::vector<size_t>{C.N} : std::vector<size_t>{C.Q, C.N});
  for (size_t a = 0; a < C.Q; ++a)
    for (size_t k = 0; k < C.N; ++k) r.v[a + C.Q * k] = C.psym(kg, int(a), int(k));
  return r;
}

Tensor eval_op(Ctx &C, const pga_tree_node n) {
  using namespace getfem;
  const auto &ch = n->children;
  switch (n->op_type) {
    case GA_PLUS: return add(eval(C, ch[0]), eval(C, ch[1]), 1.0);
    case GA_MINUS: return add(eval(C, ch[0]), eval(C, ch[1]), -1.0);
    case GA_UNARY_MINUS: return scale(eval(C, ch[0]), pconst(-1.0));
    case GA_MULT: {
      Tensor A = eval(C, ch[0]), B = eval(C, ch[1]);
      if (A.order() == 0) return scale(B, A.v[0]);
      if (B.order() == 0) return scale(A, B.v[0]);
      if (A.order() == 2 && (B.order() == 1 || B.order() == 2)) return contract(A, B, 1);
      if (A.order() == 4 && B.order() == 2) return contract(A, B, 2);
      reject("product of tensors of orders " + std::to_string(A.order()) + " and " +
             std::to_string(B.order()));
    }
    case GA_DIV: {
      Tensor A = eval(C, ch[0]), B = eval(C, ch[1]);
      double b;
      if (B.order() != 0 || !pconstant(B.v[0], b) || b == 0.0)
        reject("division by a non-constant");
      return scale(A, pconst(1.0 / b));
    }
    case GA_DOT: {
      Tensor A = eval(C, ch[0]), B = eval(C, ch[1]);
      if (A.order() == 0 || B.order() == 0) reject("'.' with a scalar");
      return contract(A, B, 1);
    }
    case GA_COLON: {
      Tensor A = eval(C, ch[0]), B = eval(C, ch[1]);
      if (A.order() < 2 || B.order() < 2) reject("':' of tensors of order < 2");
      return contract(A, B, 2);
    }
    case GA_TMULT: {
      Tensor A = eval(C, ch[0]), B = eval(C, ch[1]);
      std::vector<size_t> sz = A.sz;
      sz.insert(sz.end(), B.sz.begin(), B.sz.end());
      Tensor r = make(sz);
      for (size_t j = 0; j < B.size(); ++j)
        for (size_t i = 0; i < A.size(); ++i) r.v[i + A.size() * j] = pmul(A.v[i], B.v[j]);
      return r;
    }
    case GA_DOTMULT: {
      Tensor A = eval(C, ch[0]), B = eval(C, ch[1]);
      if (A.sz != B.sz) reject("sizes of '.*'");
      for (size_t i = 0; i < A.size(); ++i) A.v[i] = pmul(A.v[i], B.v[i]);
      return A;
    }
    case GA_DOTDIV: {
      Tensor A = eval(C, ch[0]), B = eval(C, ch[1]);
      if (A.sz != B.sz) reject("sizes of './'");
      for (size_t i = 0; i < A.size(); ++i) {
        double b;
        if (!pconstant(B.v[i], b) || b == 0.0) reject("'./' by a non-constant");
        A.v[i] = pmul(A.v[i], pconst(1.0 / b));
      }
      return A;
    }
    case GA_QUOTE: return transpose(eval(C, ch[0]));
    case GA_SYM: {
      Tensor A = eval(C, ch[0]);
      return scale(add(A, transpose(A), 1.0), pconst(0.5));
    }
    case GA_SKEW: {
      Tensor A = eval(C, ch[0]);
      return scale(add(A, transpose(A), -1.0), pconst(0.5));
    }
    case GA_TRACE: return scalar_tensor(trace(eval(C, ch[0])));
    case GA_DEVIATOR: {
      Tensor A = eval(C, ch[0]);
      Poly tr = trace(A);
      const double inv = 1.0 / double(A.sz[0]);
      for (size_t i = 0; i < A.sz[0]; ++i) padd(A.v[i + A.sz[0] * i], tr, -inv);
      return A;
    }
    default: reject("GWFL operation of token type " + std::to_string(int(n->op_type)));
  }
}

Tensor eval(Ctx &C, const pga_tree_node n) {
  using namespace getfem;
  switch (n->node_type) {
    case GA_NODE_OP: return eval_op(C, n);
    case GA_NODE_CONSTANT: case GA_NODE_ZERO: {
      if (n->test_function_type != 0 && n->test_function_type != size_type(-1)) {
        if (n->node_type == GA_NODE_ZERO) {
          std::vector<size_t> sz;
          for (size_t i = 0; i < n->tensor_order(); ++i) sz.push_back(n->tensor_proper_size(i));
          return make(sz);
        }
        reject("constant with test functions");
      }
      const auto &t = n->tensor();
      std::vector<size_t> sz;
      for (size_t i = 0; i < t.sizes().size(); ++i) sz.push_back(t.sizes()[i]);
      if (sz.size() == 1 && sz[0] == 1) sz.clear();
      Tensor r = make(sz);
      if (r.size() != t.size()) reject("constant sizes");
      if (n->node_type == GA_NODE_CONSTANT)
        for (size_t i = 0; i < r.size(); ++i) r.v[i] = pconst(t[i]);
      return r;
    }
    case GA_NODE_VAL: return datum(C, n->name);
    case GA_NODE_GRAD: case GA_NODE_DIVERG: {
      if (n->name != C.var) reject("gradient of datum " + n->name);
      if (n->node_type == GA_NODE_DIVERG) {
        if (C.Q != C.N) reject("Div of a field with qdim != dim");
        Poly p;
        for (size_t a = 0; a < C.Q; ++a) padd(p, C.psym(UG, int(a), int(a)));
        return scalar_tensor(p);
      }
      Tensor r = make(C.Q == 1 ? std::vector<size_t>{C.N} : std::vector<size_t>{C.Q, C.N});
      for (size_t a = 0; a < C.Q; ++a)
        for (size_t k = 0; k < C.N; ++k) r.v[a + C.Q * k] = C.psym(UG, int(a), int(k));
      return r;
    }
    case GA_NODE_VAL_TEST: return eval_test(C, n, false, false);
    case GA_NODE_GRAD_TEST: return eval_test(C, n, true, false);
    case GA_NODE_DIVERG_TEST: return eval_test(C, n, false, true);
    case GA_NODE_PARAMS:
      if (!n->children.empty() && n->children[0]->node_type == GA_NODE_OPERATOR) throw NHOp{};
      if (n->children.size() >= 3 && n->children[0]->node_type == GA_NODE_RESHAPE) {
        // Reshape(t, sizes...): the components keep their (Fortran) order;
        // the sizes are the node's own, fixed by the semantic analysis
        if (n->test_function_type != 0 && n->test_function_type != size_type(-1))
          reject("Reshape of an expression with test functions");
        Tensor A = eval(C, n->children[1]);
        std::vector<size_t> sz;
        for (size_t i = 0; i < n->tensor().sizes().size(); ++i) sz.push_back(n->tensor().sizes()[i]);
        size_t total = 1;
        for (size_t x : sz) total *= x;
        if (total != A.size()) reject("Reshape sizes");
        if (sz.size() == 1 && sz[0] == 1) sz.clear();
        A.sz = sz;
        return A;
      }
      reject("function call " + (n->children.empty() ? std::string("?") : n->children[0]->name) +
             " on non-constant arguments");
    default:
      reject("node type " + std::to_string(int(n->node_type)) +
             (n->name.empty() ? std::string() : " (" + n->name + ")"));
  }
}

// ------------------------------------------------------------ matching

// A coefficient polynomial (no variable or test symbols) as descriptor
// coefficients: the constant, then one entry per datum.
struct CoefParts {
  double c = 0.0;
  std::map<int, double> per_data;  // data index -> factor
};

CoefParts coef_parts(Ctx &C, const Poly &p, const char *what) {
  CoefParts r;
  for (const auto &kv : p) {
    if (kv.first.empty()) {
      r.c += kv.second;
      continue;
    }
    if (kv.first.size() != 1) reject(std::string(what) + " is not linear in the data");
    const Sym &s = C.syms[kv.first[0]];
    if (s.kind != DATA || C.data[s.data].kind == 0)
      reject(std::string(what) + " depends on a field that is not a scalar coefficient");
    r.per_data[s.data] += kv.second;
  }
  return r;
}

bool near(double a, double b, double scale) { return std::fabs(a - b) <= 1e-13 * scale; }

// Splits a polynomial into the bilinear blocks of (left, right) symbol
// pairs: left symbols of kinds lv/lg, right ones of kinds rv/rg.  Returns
// false if a monomial does not have exactly one of each.
struct Blocks {
  // [(a,k)] x [(b,l)] -> coefficient polynomial in the data; value rows use k = -1
  std::map<std::tuple<int, int, int, int>, Poly> m;
};

void split_bilinear(Ctx &C, const Poly &P, int lv, int lg, int rv, int rg, Blocks &B,
                    Poly *rest) {
  for (const auto &kv : P) {
    int li = -1, ri = -1;
    Mono other;
    bool symmetric_square = false;
    for (size_t i = 0; i < kv.first.size(); ++i) {
      const int id = kv.first[i];
      const Sym &s = C.syms[id];
      const bool is_l = s.kind == lv || s.kind == lg, is_r = s.kind == rv || s.kind == rg;
      if (is_l && li < 0) li = id;
      else if (is_r && ri < 0) ri = id;
      else if (is_l && lv == rv && ri < 0) { ri = id; symmetric_square = true; }
      else other.push_back(id);
    }
    if (li < 0 || ri < 0) {
      if (!rest) reject("a term without both test functions");
      (*rest)[kv.first] = kv.second;
      continue;
    }
    for (int id : other) {
      const int k = C.syms[id].kind;
      if (k != DATA) reject("a term of degree > 2 in the test functions or the variable");
    }
    const Sym &L = C.syms[li], &R = C.syms[ri];
    auto key = std::make_tuple(L.a, L.kind == lg ? L.k : -1, R.a, R.kind == rg ? R.k : -1);
    Poly &dst = B.m[key];
    if (lv == rv && li != ri) {
      // a quadratic form: the monomial x_i x_j (i != j) is B_ij + B_ji
      auto key2 = std::make_tuple(R.a, R.kind == rg ? R.k : -1, L.a, L.kind == lg ? L.k : -1);
      Poly half;
      half[other] = 0.5 * kv.second;
      padd(dst, half);
      padd(B.m[key2], half);
    } else {
      Poly one;
      one[other] = kv.second;
      padd(dst, one);
    }
    (void)symmetric_square;
  }
}

Poly block_at(const Blocks &B, int a, int k, int b, int l) {
  auto it = B.m.find(std::make_tuple(a, k, b, l));
  return it == B.m.end() ? Poly{} : it->second;
}

gfgpu_coef mkcoef(int kind, int slot, double v) {
  gfgpu_coef c{};
  c.kind = kind;
  c.slot = slot;
  c.value = v;
  return c;
}

struct TermSink {
  Lowered *L;
  Ctx *C;
  int slot_of(int d) {
    const std::string &nm = C->data[d].name;
    for (size_t k = 1; k < L->slot_names.size(); ++k)
      if (L->slot_names[k] == nm) return int(k);
    L->slot_names.push_back(nm);
    L->slot_kind.push_back(C->data[d].kind);
    return int(L->slot_names.size()) - 1;
  }
  void push(const gfgpu_term &t) {
    if (L->form.n_terms >= GFGPU_MAX_TERMS) reject("more than GFGPU_MAX_TERMS terms");
    L->form.terms[L->form.n_terms++] = t;
  }
  // a GRADGRAD_TENSOR term with its tensor (one per form)
  void push_tensor(const gfgpu_term &t, const std::vector<double> &D) {
    for (int k = 0; k < L->form.n_terms; ++k)
      if (L->form.terms[k].kind == GFGPU_TERM_GRADGRAD_TENSOR)
        reject("more than one anisotropic gradient coupling in one form");
    if (D.size() > size_t(GFGPU_MAX_TENSOR)) reject("coupling tensor too large");
    push(t);
    for (size_t i = 0; i < D.size(); ++i) L->form.tensor[i] = D[i];
  }
};

// GRADGRAD / MASS terms of bilinear blocks (lv/lg x rv/rg), scaled by `sc`.
// With allow_tensor, the gradient coupling of one coefficient source (the
// constant part, or one per-element datum) may be a constant symmetric
// anisotropic D[(a,k),(b,l)]: a GRADGRAD_TENSOR term.
void emit_bilinear(Ctx &C, TermSink &S, const Blocks &B, double sc, bool allow_tensor) {
  const int Q = int(C.Q), N = int(C.N);
  // value-gradient couplings are not lowered
  for (const auto &kv : B.m) {
    const int k = std::get<1>(kv.first), l = std::get<3>(kv.first);
    if ((k < 0) != (l < 0) && !kv.second.empty()) reject("value-gradient couplings");
  }
  // per coefficient source (constant = -1, else a data index): c0 c1 c2 cm
  std::map<int, std::array<double, 4>> coefs;
  std::set<int> aniso;  // sources whose gradient coupling is not isotropic
  auto parts = [&](const Poly &p, int which, const char *what) {
    CoefParts cp = coef_parts(C, p, what);
    coefs[-1][which] += 0.0;
    if (cp.c != 0.0) coefs[-1][which] = cp.c;
    for (const auto &d : cp.per_data) coefs[d.first][which] = d.second;
  };
  // read c0, c1, c2 off single-coefficient entries, then check every entry
  if (Q == 1) {
    parts(block_at(B, 0, 0, 0, 0), 1, "the gradient coefficient");
  } else {
    parts(block_at(B, 0, 0, 1, 1), 0, "the div-div coefficient");
    parts(block_at(B, 0, 1, 0, 1), 1, "the grad-grad coefficient");
    parts(block_at(B, 0, 1, 1, 0), 2, "the transposed-gradient coefficient");
  }
  parts(block_at(B, 0, -1, 0, -1), 3, "the mass coefficient");
  for (auto &kv : coefs)
    for (int w = 0; w < 4; ++w) (void)kv.second[w];
  // every entry must be what the coefficients predict
  for (int a = 0; a < Q; ++a)
    for (int k = -1; k < N; ++k)
      for (int b = 0; b < Q; ++b)
        for (int l = -1; l < N; ++l) {
          if ((k < 0) != (l < 0)) continue;
          Poly pred;
          auto addc = [&](int w, bool on) {
            if (!on) return;
            for (const auto &kv : coefs) {
              const double x = kv.second[w];
              if (x == 0.0) continue;
              Mono m;
              if (kv.first >= 0) m.push_back(C.sym(DATA, 0, 0, kv.first));
              Poly t;
              t[m] = x;
              padd(pred, t);
            }
          };
          if (k < 0) {
            addc(3, a == b);
          } else {
            addc(0, Q > 1 && a == k && b == l);
            addc(1, a == b && k == l);
            addc(2, Q > 1 && a == l && k == b);
          }
          const Poly got = block_at(B, a, k, b, l);
          double scale = 1.0;
          for (const auto &kv : got) scale = std::max(scale, std::fabs(kv.second));
          std::set<Mono> keys;
          for (const auto &kv : got) keys.insert(kv.first);
          for (const auto &kv : pred) keys.insert(kv.first);
          for (const Mono &m : keys) {
            const auto ig = got.find(m);
            const auto ip = pred.find(m);
            const double g = ig == got.end() ? 0.0 : ig->second;
            const double p = ip == pred.end() ? 0.0 : ip->second;
            if (!near(g, p, scale)) {
              if (k < 0) reject("anisotropic mass term");
              // the source whose coupling is not isotropic: the constant, or
              // one scalar coefficient datum
              if (m.size() > 1 ||
                  (m.size() == 1 && (C.syms[m[0]].kind != DATA || C.data[C.syms[m[0]].data].kind == 0)))
                reject("gradient coupling is not isotropic");
              aniso.insert(m.empty() ? -1 : C.syms[m[0]].data);
            }
          }
        }
  // an anisotropic source: its whole gradient coupling as the tensor
  int ten_src = -2;
  std::vector<double> Dten;
  if (!aniso.empty()) {
    if (!allow_tensor || (Q != 1 && Q != N)) reject("gradient coupling is not isotropic");
    if (aniso.size() > 1) reject("anisotropic couplings from more than one coefficient");
    ten_src = *aniso.begin();
    const int ND = Q * N;
    Dten.assign(size_t(ND) * ND, 0.0);
    Mono key;
    if (ten_src >= 0) key.push_back(C.sym(DATA, 0, 0, ten_src));
    for (int a = 0; a < Q; ++a)
      for (int k = 0; k < N; ++k)
        for (int b = 0; b < Q; ++b)
          for (int l = 0; l < N; ++l) {
            const Poly got = block_at(B, a, k, b, l);
            const auto it = got.find(key);
            Dten[size_t(a * N + k) * ND + b * N + l] = it == got.end() ? 0.0 : it->second;
          }
    for (int r = 0; r < ND; ++r)
      for (int c = 0; c < ND; ++c)
        if (Dten[size_t(r) * ND + c] != Dten[size_t(c) * ND + r])
          reject("anisotropic gradient coupling is not symmetric");
    if (ten_src >= 0 && C.data[ten_src].kind != GFGPU_COEF_ELEMENT)
      reject("anisotropic coupling scaled by a nodal field");
    coefs[ten_src];  // the source gets its term below
  }
  // terms: the constant part first, then per datum (GRADGRAD, then MASS)
  std::vector<int> order{-1};
  for (const auto &kv : coefs)
    if (kv.first >= 0) order.push_back(kv.first);
  for (int src : order) {
    auto it = coefs.find(src);
    if (it == coefs.end()) continue;
    const auto &c = it->second;
    const int kind = src < 0 ? GFGPU_COEF_CONST : C.data[src].kind;
    const int slot = src < 0 ? 0 : S.slot_of(src);
    if (src == ten_src) {
      gfgpu_term t{};
      t.kind = GFGPU_TERM_GRADGRAD_TENSOR;
      t.scale = sc;
      t.c[0] = src < 0 ? mkcoef(GFGPU_COEF_NONE, 0, 0.0) : mkcoef(kind, slot, 1.0);
      S.push_tensor(t, Dten);
    } else if (c[0] != 0.0 || c[1] != 0.0 || c[2] != 0.0) {
      gfgpu_term t{};
      t.kind = GFGPU_TERM_GRADGRAD;
      t.scale = sc;
      for (int w = 0; w < 3; ++w)
        t.c[w] = c[w] != 0.0 ? mkcoef(kind, slot, c[w]) : mkcoef(GFGPU_COEF_NONE, 0, 0.0);
      S.push(t);
    }
    if (c[3] != 0.0) {
      gfgpu_term t{};
      t.kind = GFGPU_TERM_MASS;
      t.scale = sc;
      t.c[0] = mkcoef(kind, slot, c[3]);
      S.push(t);
    }
  }
}

// SOURCE terms: alpha f[a] Test_u[a] (monomials Test1 value x one
// component of a field datum on the variable's mesh_fem).
void emit_source(Ctx &C, TermSink &S, const Poly &P, double sc) {
  std::map<int, Blocks> per_field;
  for (const auto &kv : P) {
    int ti = -1, fi = -1;
    for (int id : kv.first) {
      const Sym &s = C.syms[id];
      if ((s.kind == T1V || s.kind == T1G) && ti < 0) ti = id;
      else if (s.kind == DATA && fi < 0 &&
               (C.data[s.data].kind == 0 ||
                (C.data[s.data].kind == GFGPU_COEF_NODAL && C.Q == 1)))
        fi = id;  // a field on the variable's mesh_fem (for a scalar variable,
                  // the scalar field on its nodes)
      else if (s.kind == DATA) reject("sources scaled by element data are not lowered");
      else reject("source term of degree > 1");
    }
    if (ti < 0) reject("a term without the test function");
    if (fi < 0) reject("constant source terms are not lowered");
    if (C.syms[ti].kind == T1G) reject("gradient source terms");
    const Sym &T = C.syms[ti], &F = C.syms[fi];
    Poly one;
    one[Mono{}] = kv.second;
    padd(per_field[F.data].m[std::make_tuple(T.a, -1, F.a, -1)], one);
  }
  for (const auto &pf : per_field) {
    const Blocks &B = pf.second;
    double alpha = 0.0;
    pconstant(block_at(B, 0, -1, 0, -1), alpha);
    double scale = std::max(1.0, std::fabs(alpha));
    for (int a = 0; a < int(C.Q); ++a)
      for (int b = 0; b < int(C.Q); ++b) {
        double x = 0.0;
        pconstant(block_at(B, a, -1, b, -1), x);
        if (!near(x, a == b ? alpha : 0.0, scale)) reject("anisotropic source");
      }
    gfgpu_term t{};
    t.kind = GFGPU_TERM_SOURCE;
    t.scale = sc * alpha;
    t.field_slot = S.slot_of(pf.first);
    S.push(t);
  }
}

// ----------------------------------------------- neo-Hookean structure

bool is_identity_constant(const pga_tree_node n, size_t N) {
  if (n->node_type != getfem::GA_NODE_CONSTANT) return false;
  const auto &t = n->tensor();
  if (t.sizes().size() != 2 || t.sizes()[0] != N || t.sizes()[1] != N) return false;
  for (size_t i = 0; i < N; ++i)
    for (size_t j = 0; j < N; ++j)
      if (t[i + N * j] != (i == j ? 1.0 : 0.0)) return false;
  return true;
}

bool is_grad_var(const pga_tree_node n, const std::string &var) {
  return n->node_type == getfem::GA_NODE_GRAD && n->name == var;
}

// PARAMS(OPERATOR name, Grad_u, C_MATRIX[p1; p2]) with derivative flags
// der1 = d1, der2 = d2: returns the two parameter subtrees
bool match_nh_call(const pga_tree_node n, const std::string &var, const char *opname, size_t d1,
                   size_t d2, pga_tree_node &p1, pga_tree_node &p2) {
  using namespace getfem;
  if (n->node_type != GA_NODE_PARAMS || n->children.size() != 3) return false;
  const pga_tree_node op = n->children[0];
  if (op->node_type != GA_NODE_OPERATOR || op->name != opname || op->der1 != d1 || op->der2 != d2)
    return false;
  if (!is_grad_var(n->children[1], var)) return false;
  const pga_tree_node m = n->children[2];
  if (m->node_type == GA_NODE_C_MATRIX && m->children.size() == 2) {
    p1 = m->children[0];
    p2 = m->children[1];
    return true;
  }
  if (m->node_type == GA_NODE_CONSTANT && m->tensor().size() == 2) {
    p1 = p2 = m;  // folded constant vector: both read from it
    return true;
  }
  return false;
}

// ((Id+Grad_u)*NH_PK2(Grad_u,[p1;p2])):Grad_Test_u
bool match_nh_brick(const pga_tree_node r, const std::string &var, pga_tree_node &p1,
                    pga_tree_node &p2) {
  using namespace getfem;
  if (r->node_type != GA_NODE_OP || r->op_type != GA_COLON) return false;
  const pga_tree_node lhs = r->children[0], rhs = r->children[1];
  if (rhs->node_type != GA_NODE_GRAD_TEST || rhs->name != var || rhs->test_function_type != 1)
    return false;
  if (lhs->node_type != GA_NODE_OP || lhs->op_type != GA_MULT) return false;
  const pga_tree_node F = lhs->children[0], S = lhs->children[1];
  if (F->node_type != GA_NODE_OP || F->op_type != GA_PLUS) return false;
  const bool f_ok = (is_identity_constant(F->children[0], 3) && is_grad_var(F->children[1], var)) ||
                    (is_identity_constant(F->children[1], 3) && is_grad_var(F->children[0], var));
  return f_ok && match_nh_call(S, var, "Compressible_Neo_Hookean_PK2", 0, 0, p1, p2);
}

// every operator call in the tree is of the named operator, on Grad_u, with
// parameters equal (as lowered coefficients) to the given ones
void collect_nh_calls(const pga_tree_node n, std::vector<pga_tree_node> &out) {
  if (n->node_type == getfem::GA_NODE_PARAMS && !n->children.empty() &&
      n->children[0]->node_type == getfem::GA_NODE_OPERATOR) {
    const std::string &op = n->children[0]->name;
    if (op != "Compressible_Neo_Hookean_PK2" && op != "Compressible_Neo_Hookean_potential")
      reject("nonlinear operator " + op);
    out.push_back(n);
  }
  for (const auto &c : n->children) collect_nh_calls(c, out);
}

gfgpu_coef law_param(Ctx &C, TermSink &S, const pga_tree_node p, int which, const pga_tree_node m) {
  Poly v;
  if (p == m) {  // folded constant vector [p1; p2]
    v = pconst(m->tensor()[which]);
  } else {
    Tensor t = eval(C, p);
    if (!is_scalar(t)) reject("a law parameter is not a scalar");
    v = t.v[0];
  }
  CoefParts cp = coef_parts(C, v, "a hyperelastic parameter");
  if (cp.per_data.size() > 1 || (cp.per_data.size() == 1 && cp.c != 0.0))
    reject("a law parameter must be one field times a constant");
  if (cp.per_data.empty()) return mkcoef(GFGPU_COEF_CONST, 0, cp.c);
  const auto &d = *cp.per_data.begin();
  return mkcoef(C.data[d.first].kind, S.slot_of(d.first), d.second);
}

std::string expr_key(const getfem::ga_workspace::tree_description &td) {
  const pga_tree_node r = td.ptree ? td.ptree->root : nullptr;
  return r && r->expr ? *r->expr : std::string();
}

}  // namespace

std::vector<Lowered> lower_workspace(const getfem::ga_workspace &ws, size_t order) {
  std::vector<Lowered> out;
  // expressions whose neo-Hookean tree of the lower order matched (their
  // derivative trees are the NEOHOOKEAN term too)
  std::set<std::string> nh_brick, nh_potential;
  for (size_t i = 0; i < ws.nb_trees(); ++i) {
    const auto &td = ws.tree_info(i);
    if (!td.ptree || !td.ptree->root) continue;
    const std::string &var = td.name_test1;
    pga_tree_node p1, p2;
    if (td.order == 1 && match_nh_brick(td.ptree->root, var, p1, p2)) nh_brick.insert(expr_key(td));
    if (td.order == 0) {
      // the potential's variable: the one Grad_u of its call
      const pga_tree_node r = td.ptree->root;
      if (r->node_type == getfem::GA_NODE_PARAMS && r->children.size() == 3 &&
          r->children[1]->node_type == getfem::GA_NODE_GRAD &&
          match_nh_call(r, r->children[1]->name, "Compressible_Neo_Hookean_potential", 0, 0, p1, p2))
        nh_potential.insert(expr_key(td));
    }
  }
  for (size_t i = 0; i < ws.nb_trees(); ++i) {
    const auto &td = ws.tree_info(i);
    if (td.order != order) continue;
    if (!td.ptree || !td.ptree->root) continue;
    if (td.operation != getfem::ga_workspace::ASSEMBLY) reject("assignment / interpolation trees");
    if (!td.interpolate_name_test1.empty() || !td.interpolate_name_test2.empty() ||
        !td.secondary_domain.empty())
      reject("interpolate transformations and secondary domains");
    const pga_tree_node root = td.ptree->root;
    // the variable: the test function's, or for a potential the variable
    // whose value or gradient appears
    std::string var = order >= 1 ? td.name_test1 : std::string();
    if (order == 2 && td.name_test2 != td.name_test1) reject("coupling of two variables");
    if (order == 0) {
      std::vector<pga_tree_node> st{root};
      while (!st.empty() && var.empty()) {
        pga_tree_node n = st.back();
        st.pop_back();
        if ((n->node_type == getfem::GA_NODE_GRAD || n->node_type == getfem::GA_NODE_VAL ||
             n->node_type == getfem::GA_NODE_DIVERG) &&
            ws.variable_exists(n->name) && !ws.is_constant(n->name))
          var = n->name;
        for (const auto &c : n->children) st.push_back(c);
      }
      if (var.empty()) reject("a potential without a variable");
    }
    if (!ws.variable_exists(var) || ws.is_constant(var)) reject("test function of a constant");
    if (ws.is_internal_variable(var) || ws.associated_im_data(var))
      reject("internal im_data variables (condensation) are not lowered here");
    const getfem::mesh_fem *mf = ws.associated_mf(var);
    if (!mf) reject(var + " has no mesh_fem");
    // the group of (var, mim, region)
    Lowered *L = nullptr;
    for (auto &x : out)
      if (x.var == var && x.mim == td.mim && x.rg == td.rg) L = &x;
    if (!L) {
      out.emplace_back();
      L = &out.back();
      L->var = var;
      L->mim = td.mim;
      L->rg = td.rg;
    }
    Ctx C{ws, var};
    C.mf = mf;
    C.Q = mf->get_qdim();
    C.N = mf->linked_mesh().dim();
    TermSink S{L, &C};
    pga_tree_node p1, p2;
    const std::string key = expr_key(td);
    // neo-Hookean forms, by structure
    const bool nh_here = [&] {
      std::vector<pga_tree_node> calls;
      collect_nh_calls(root, calls);
      return !calls.empty();
    }();
    if (nh_here) {
      if (C.N != 3 || C.Q != 3) reject("neo-Hookean law is 3-D only");
      std::vector<pga_tree_node> calls;
      collect_nh_calls(root, calls);
      const bool brick = nh_brick.count(key) != 0, pot = nh_potential.count(key) != 0;
      const char *opname = brick ? "Compressible_Neo_Hookean_PK2" : "Compressible_Neo_Hookean_potential";
      if (!brick && !pot) reject("nonlinear operator outside the neo-Hookean brick form and potential");
      bool ok = order == (brick ? 1u : 0u) || (order == 2) || (pot && order == 1);
      if (order == 1 && brick) ok = match_nh_brick(root, var, p1, p2);
      if (!ok) reject("neo-Hookean tree of an unexpected shape");
      // every call: the same operator on Grad_u, parameters as the first
      gfgpu_coef c1{}, c2{};
      for (size_t k = 0; k < calls.size(); ++k) {
        const pga_tree_node n = calls[k];
        const pga_tree_node op = n->children[0];
        if (op->name != opname) reject("mixed nonlinear operators");
        pga_tree_node q1, q2;
        if (!match_nh_call(n, var, opname, op->der1, op->der2, q1, q2))
          reject("neo-Hookean operator call of an unexpected shape");
        const gfgpu_coef a1 = law_param(C, S, q1, 0, n->children[2]);
        const gfgpu_coef a2 = law_param(C, S, q2, 1, n->children[2]);
        if (k == 0) {
          c1 = a1;
          c2 = a2;
        } else if (a1.kind != c1.kind || a1.slot != c1.slot || a1.value != c1.value ||
                   a2.kind != c2.kind || a2.slot != c2.slot || a2.value != c2.value) {
          reject("neo-Hookean calls with different parameters");
        }
      }
      gfgpu_term t{};
      t.kind = GFGPU_TERM_NEOHOOKEAN;
      t.scale = 1.0;
      t.c[0] = c1;
      t.c[1] = c2;
      S.push(t);
      continue;
    }
    Tensor R;
    try {
      R = eval(C, root);
    } catch (const NHOp &) {
      reject("nonlinear operator outside the neo-Hookean forms");
    }
    if (!is_scalar(R)) reject("the integrand is not a scalar");
    const Poly &P = R.v[0];
    if (order == 2) {
      Blocks B;
      split_bilinear(C, P, T1V, T1G, T2V, T2G, B, nullptr);
      emit_bilinear(C, S, B, 1.0, true);
    } else if (order == 1) {
      Blocks B;
      Poly rest;
      split_bilinear(C, P, T1V, T1G, UV, UG, B, &rest);
      emit_bilinear(C, S, B, 1.0, true);
      emit_source(C, S, rest, 1.0);
    } else {
      // potential: the quadratic part B(u, u) by polarisation, and the
      // linear part alpha f.u
      Blocks B;
      Poly rest;
      split_bilinear(C, P, UV, UG, UV, UG, B, &rest);
      // (anisotropic couplings are not lowered for potentials)
      if (!B.m.empty()) emit_bilinear(C, S, B, 1.0, false);
      // rest: monomials linear in u with a field datum (u takes the test
      // function's place for the source matcher)
      Poly lin;
      for (const auto &kv : rest) {
        Mono m;
        for (int id : kv.first) {
          const Sym &s = C.syms[id];
          m.push_back(s.kind == UV ? C.sym(T1V, s.a) : s.kind == UG ? C.sym(T1G, s.a, s.k) : id);
        }
        std::sort(m.begin(), m.end());
        lin[m] = kv.second;
      }
      if (!lin.empty()) {
        bool has_u = false;
        for (const auto &kv : lin)
          for (int id : kv.first) has_u |= C.syms[id].kind == T1V || C.syms[id].kind == T1G;
        if (!has_u) reject("potential terms independent of the variable");
        emit_source(C, S, lin, 1.0);
      }
    }
  }
  return out;
}

std::string to_json(const Lowered &L) {
  std::ostringstream s;
  s.precision(17);
  s << "{\"var\": \"" << L.var << "\", \"terms\": [";
  for (int t = 0; t < L.form.n_terms; ++t) {
    const gfgpu_term &T = L.form.terms[t];
    s << (t ? ", " : "") << "{\"kind\": " << T.kind << ", \"scale\": " << T.scale
      << ", \"field\": \"" << (T.kind == GFGPU_TERM_SOURCE ? L.slot_names[T.field_slot] : "")
      << "\", \"c\": [";
    for (int k = 0; k < 3; ++k) {
      const gfgpu_coef &c = T.c[k];
      s << (k ? ", " : "") << "{\"kind\": " << c.kind << ", \"value\": " << c.value
        << ", \"data\": \""
        << ((c.kind == GFGPU_COEF_ELEMENT || c.kind == GFGPU_COEF_NODAL) ? L.slot_names[c.slot] : "")
        << "\"}";
    }
    s << "]";
    if (T.kind == GFGPU_TERM_GRADGRAD_TENSOR) {
      s << ", \"tensor\": [";
      for (int i = 0; i < GFGPU_MAX_TENSOR; ++i) s << (i ? ", " : "") << L.form.tensor[i];
      s << "]";
    }
    s << "}";
  }
  s << "]}";
  return s.str();
}

}  // namespace gfgpu_getfem
