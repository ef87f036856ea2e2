// Polynomials of GetFEM's base functions, tabulated as the reference
// tabulates them.
//
// GetFEM stores a Lagrange base function as a bgeot::polynomial: the
// coefficients of its monomials in graded order (src/getfem/bgeot_poly.h:
// 100-160, index of x0^i0..x_{n-1}^i_{n-1} from alpha(n,d) = C(n+d,d),
// src/bgeot_poly.cc:46-103), built by products of linear factors
// (PK_fem_::calc_base_func, src/getfem_fem.cc:727-749) and by direct
// products for FEM_QK (src/getfem_fem.cc:792-826), and evaluates it with a
// nested scheme (bgeot_poly.h:452-533).  For high degrees (FEM_QK(3,4): total
// degree 12) evaluating the monomial form loses ~1e-10 absolutely; to
// agree with the reference to 1e-12 the tables must carry the same
// rounding.  This header restates that arithmetic operation for operation:
// the order in which products are accumulated into coefficients, the
// coefficient-wise scalings, the derivative, and the evaluation order.
// Compile it with -ffp-contract=off so no multiply-add is fused.
#pragma once
#include <cstddef>
#include <vector>

namespace gfgpu {
namespace refpoly {

// number of monomials of degree <= d in n variables; alpha(n,-1) = 0
inline size_t alpha(int n, int d) {
  if (d < 0) return 0;
  size_t r = 1;
  for (int k = 1; k <= n; ++k) r = r * size_t(d + k) / size_t(k);
  return r;
}

inline size_t index_of(const std::vector<int> &e) {
  int n = int(e.size()), d = 0;
  for (int x : e) d += x;
  size_t idx = 0;
  for (int i = 0; i < n && d > 0; ++i) {
    idx += alpha(n - i, d - 1);
    d -= e[i];
  }
  return idx;
}

// exponent vectors in index order (power_index::operator++, bgeot_poly.cc:53-68)
inline std::vector<std::vector<int>> powers(int n, int deg) {
  std::vector<std::vector<int>> out;
  std::vector<int> e(n, 0);
  size_t total = alpha(n, deg);
  for (size_t k = 0; k < total; ++k) {
    out.push_back(e);
    if (n == 0) break;
    int l = n - 2;
    while (l >= 0 && e[l] == 0) --l;
    int a = e[n - 1];
    e[n - 1] = 0;
    e[l + 1] = a + 1;
    if (l >= 0) e[l]--;
  }
  return out;
}

struct Poly {
  int n = 0, d = 0;
  std::vector<double> c;
  Poly() {}
  Poly(int n_, int d_) : n(n_), d(d_), c(alpha(n_, d_), 0.0) {}
  static Poly one(int n) {
    Poly p(n, 0);
    p.c[0] = 1.0;
    return p;
  }
  static Poly var(int n, int k) {  // polynomial(n, 1, k): x_k, degree 1
    Poly p(n, 1);
    p.c[1 + k] = 1.0;
    return p;
  }
  void change_degree(int dd) {
    c.resize(alpha(n, dd), 0.0);
    d = dd;
  }
  void add_monomial(double coeff, const std::vector<int> &e) {
    size_t i = index_of(e);
    if (i >= c.size()) {
      int dd = 0;
      for (int x : e) dd += x;
      change_degree(dd);
    }
    c[i] += coeff;
  }
  Poly scaled(double s) const {
    Poly r = *this;
    for (double &v : r.c) v *= s;
    return r;
  }
  Poly minus(const Poly &Q) const {
    Poly r = *this;
    if (Q.d > r.d) r.change_degree(Q.d);
    for (size_t k = 0; k < Q.c.size(); ++k) r.c[k] -= Q.c[k];
    return r;
  }
  // P *= Q (bgeot_poly.h:346-377)
  void mul(const Poly &Q) {
    Poly aux = *this;
    change_degree(0);
    c[0] = 0.0;
    std::vector<std::vector<int>> pq = powers(Q.n, Q.d), pa = powers(aux.n, aux.d);
    std::vector<int> tot(n);
    for (size_t iq = Q.c.size(); iq-- > 0;) {
      if (Q.c[iq] == 0.0) continue;
      for (size_t ia = aux.c.size(); ia-- > 0;) {
        if (aux.c[ia] == 0.0) continue;
        for (int k = 0; k < n; ++k) tot[k] = pa[ia][k] + pq[iq][k];
        add_monomial(Q.c[iq] * aux.c[ia], tot);
      }
    }
  }
  // P.direct_product(Q): variables of Q follow those of P (bgeot_poly.h:380-400)
  void direct_product(const Poly &Q) {
    Poly aux = *this;
    n = n + Q.n;
    d = 0;
    c.assign(1, 0.0);
    std::vector<std::vector<int>> pq = powers(Q.n, Q.d), pa = powers(aux.n, aux.d);
    std::vector<int> tot(n);
    for (size_t iq = Q.c.size(); iq-- > 0;) {
      if (Q.c[iq] == 0.0) continue;
      for (size_t ia = aux.c.size(); ia-- > 0;) {
        if (aux.c[ia] == 0.0) continue;
        for (int k = 0; k < aux.n; ++k) tot[k] = pa[ia][k];
        for (int k = 0; k < Q.n; ++k) tot[aux.n + k] = pq[iq][k];
        add_monomial(Q.c[iq] * aux.c[ia], tot);
      }
    }
  }
  // d/dx_k (bgeot_poly.h:420-432)
  Poly derivative(int k) const {
    Poly r = *this;
    std::vector<std::vector<int>> pw = powers(n, d);
    for (size_t i = 0; i < r.c.size(); ++i) {
      double v = r.c[i];
      if (v != 0.0 && pw[i][k] > 0) {
        std::vector<int> e = pw[i];
        e[k]--;
        r.c[index_of(e)] = v * double(e[k] + 1);
      }
      r.c[i] = 0.0;
    }
    if (r.d > 0) r.change_degree(r.d - 1);
    return r;
  }

  // the nested form of the explicit low-degree cases of polynomial::eval:
  // E(m, v) = P[m] + x_0 E(m+e_0, 0) + ... + x_v E(m+e_v, v), summed left
  // to right, truncated at the degree
  double nested(std::vector<int> &m, int v, int deg, const double *x) const {
    double s = c[index_of(m)];
    if (deg == d) return s;
    for (int w = 0; w <= v; ++w) {
      m[w]++;
      double inner = nested(m, w, deg + 1, x);
      m[w]--;
      s = s + x[w] * inner;
    }
    return s;
  }
  // Horner scheme of polynomial::horner (bgeot_poly.h:434-449)
  double horner(std::vector<int> &mi, int k, int de, const double *x) const {
    if (k == 0) return c[index_of(mi)];
    double v = x[k - 1], res = 0.0;
    for (int e = d - de; e >= 0; --e) {
      mi[k - 1] = e;
      double h = horner(mi, k - 1, de + e, x);
      res = h + v * res;
    }
    mi[k - 1] = 0;
    return res;
  }
  double eval(const double *x) const {
    if (d == 0) return c[0];
    if (d == 1) {
      double s = c[0];
      for (int i = 0; i < n; ++i) s += x[i] * c[i + 1];
      return s;
    }
    if (n >= 1 && n <= 3 && d <= 6) {
      std::vector<int> m(n, 0);
      return nested(m, n - 1, 0, x);
    }
    std::vector<int> mi(n, 0);
    return horner(mi, n, 0, x);
  }
};

// PK_fem_::calc_base_func for the node of lattice coordinates lat (sum <= K)
inline Poly pk_base(int N, int K, const int *lat) {
  Poly l0 = Poly::one(N), l1 = Poly::one(N);
  Poly p = l0;
  if (K == 0) return p;
  for (int nn = 0; nn < N; ++nn) l0 = l0.minus(Poly::var(N, nn));
  std::vector<int> w(N + 1);
  w[0] = K;
  for (int nn = 1; nn <= N; ++nn) w[nn] = lat[nn - 1], w[0] -= w[nn];
  for (int nn = 0; nn <= N; ++nn)
    for (int j = 0; j < w[nn]; ++j) {
      const Poly base = nn == 0 ? l0 : Poly::var(N, nn - 1);
      Poly f = base.scaled(double(K) / double(j + 1)).minus(l1.scaled(double(j) / double(j + 1)));
      p.mul(f);
    }
  return p;
}

// FEM_QK(N,K) base function of lattice (i0,..,i_{N-1}):
// FEM_PRODUCT(FEM_QK(N-1,K), FEM_PK(1,K)) recursively, FEM_QK(1,K) = FEM_PK(1,K)
inline Poly qk_base(int N, int K, const int *lat) {
  Poly p = pk_base(1, K, &lat[0]);
  for (int d = 1; d < N; ++d) p.direct_product(pk_base(1, K, &lat[d]));
  return p;
}

}  // namespace refpoly
}  // namespace gfgpu
