// Host-side reference elements, quadrature, structured meshes and DOF
// numbering.  See refelem.h for the GetFEM behaviour each part mirrors.
#include "refelem.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <stdexcept>
#include <unordered_map>

namespace gfgpu {

// ---------------------------------------------------------------- elements

RefElement::RefElement(int dim_, int kind_, int degree_)
    : dim(dim_), kind(kind_), degree(degree_) {
  if (dim < 1 || dim > 3 || degree < 0 || degree > 8)
    throw std::invalid_argument("unsupported reference element");
  const int K = degree;
  // Node ordering (getfem_fem.cc:753-766 and bgeot simplex_of_reference):
  // lattice points with the first coordinate varying fastest; for the
  // simplex only points with coordinate sum <= K.
  int c[3] = {0, 0, 0};
  int ext[3] = {1, 1, 1};
  for (int d = 0; d < dim; ++d) ext[d] = K + 1;
  for (c[2] = 0; c[2] < ext[2]; ++c[2])
    for (c[1] = 0; c[1] < ext[1]; ++c[1])
      for (c[0] = 0; c[0] < ext[0]; ++c[0]) {
        int s = 0;
        for (int d = 0; d < dim; ++d) s += c[d];
        if (kind == SIMPLEX && s > K) continue;
        for (int d = 0; d < dim; ++d) lattice.push_back(c[d]);
      }
  nb = int(lattice.size()) / dim;
  if (K == 0) nb = 1, lattice.assign(dim, 0);
  // the base functions as the reference builds them (see refpoly.h)
  for (int i = 0; i < nb; ++i) {
    const int *c = &lattice[i * dim];
    base.push_back(kind == SIMPLEX || K == 0 ? refpoly::pk_base(dim, K, c)
                                             : refpoly::qk_base(dim, K, c));
    std::vector<refpoly::Poly> g;
    for (int d = 0; d < dim; ++d) g.push_back(base.back().derivative(d));
    dbase.push_back(g);
  }
}

void RefElement::node(int i, double *x) const {
  for (int d = 0; d < dim; ++d)
    x[d] = degree == 0 ? (kind == SIMPLEX ? 1.0 / (dim + 1) : 0.5)
                       : double(lattice[i * dim + d]) / degree;
}

void RefElement::eval(const double *x, double *val, double *grad) const {
  for (int i = 0; i < nb; ++i) {
    val[i] = base[i].eval(x);
    for (int d = 0; d < dim; ++d) grad[i * dim + d] = dbase[i][d].eval(x);
  }
}

// --------------------------------------------------------------- quadrature

// Expanded point sets of the simplex rules used here.  The orbit parameters
// and weights are those of cubature/TRIANGLE_{2,4}.IM and
// cubature/TETRA_{2,5}.IM; points are listed in the order in which
// approx_integration::add_point_full_symmetric generates them.
static const double kTri2[] = {
    1. / 6, 1. / 6, 1. / 6,
    2. / 3, 1. / 6, 1. / 6,
    1. / 6, 2. / 3, 1. / 6};
static const double kTri4[] = {
    0.445948490915965, 0.445948490915965, 0.111690794839005,
    0.10810301816807, 0.445948490915965, 0.111690794839005,
    0.445948490915965, 0.10810301816807, 0.111690794839005,
    0.091576213509771, 0.091576213509771, 0.054975871827661,
    0.8168475729804581, 0.091576213509771, 0.054975871827661,
    0.091576213509771, 0.8168475729804581, 0.054975871827661};
static const double kTet2[] = {
    0.13819660112501053, 0.13819660112501053, 0.13819660112501053, 1. / 24,
    0.5854101966249684, 0.13819660112501053, 0.13819660112501053, 1. / 24,
    0.13819660112501053, 0.5854101966249684, 0.13819660112501053, 1. / 24,
    0.13819660112501053, 0.13819660112501053, 0.5854101966249684, 1. / 24};
static const double kTet5[] = {
    0.25, 0.25, 0.25, 0.019753086419753086,
    0.3197936278296299, 0.3197936278296299, 0.3197936278296299, 0.011511367871045398,
    0.04061911651111039, 0.3197936278296299, 0.3197936278296299, 0.011511367871045398,
    0.3197936278296299, 0.04061911651111039, 0.3197936278296299, 0.011511367871045398,
    0.3197936278296299, 0.3197936278296299, 0.04061911651111039, 0.011511367871045398,
    0.09197107805272303, 0.09197107805272303, 0.09197107805272303, 0.01198951396316977,
    0.7240867658418311, 0.09197107805272303, 0.09197107805272303, 0.01198951396316977,
    0.09197107805272303, 0.7240867658418311, 0.09197107805272303, 0.01198951396316977,
    0.09197107805272303, 0.09197107805272303, 0.7240867658418311, 0.01198951396316977,
    0.44364916731037085, 0.056350832689629156, 0.056350832689629156, 0.008818342151675485,
    0.056350832689629156, 0.44364916731037085, 0.056350832689629156, 0.008818342151675485,
    0.44364916731037085, 0.44364916731037085, 0.056350832689629156, 0.008818342151675485,
    0.056350832689629156, 0.056350832689629156, 0.44364916731037085, 0.008818342151675485,
    0.44364916731037085, 0.056350832689629156, 0.44364916731037085, 0.008818342151675485,
    0.056350832689629156, 0.44364916731037085, 0.44364916731037085, 0.008818342151675485};

// Gauss-Legendre rule with n points on [0,1] by Newton iteration on the
// Legendre polynomial (long double), listed as GetFEM lists IM_GAUSS1D:
// symmetric pairs (x, 1-x) with x ascending, then the midpoint.
static void gauss_legendre01(int n, std::vector<double> &x, std::vector<double> &w) {
  std::vector<long double> xs(n), ws(n);
  const long double pi = 3.14159265358979323846264338327950288L;
  for (int k = 0; k < n; ++k) {
    long double z = cosl(pi * (k + 0.75L) / (n + 0.5L));
    for (int it = 0; it < 100; ++it) {
      long double p0 = 1, p1 = z;
      for (int j = 2; j <= n; ++j) {
        long double p2 = ((2 * j - 1) * z * p1 - (j - 1) * p0) / j;
        p0 = p1;
        p1 = p2;
      }
      if (n == 1) p0 = 1;  // P_0
      long double dp = n * (z * p1 - p0) / (z * z - 1);
      if (n == 1) dp = 1;
      long double dz = p1 / dp;
      z -= dz;
      if (fabsl(dz) < 1e-19L) break;
    }
    long double p0 = 1, p1 = z;
    for (int j = 2; j <= n; ++j) {
      long double p2 = ((2 * j - 1) * z * p1 - (j - 1) * p0) / j;
      p0 = p1;
      p1 = p2;
    }
    long double dp = (n == 1) ? 1 : n * (z * p1 - p0) / (z * z - 1);
    xs[k] = z;  // descending in k on [-1,1]
    ws[k] = 2 / ((1 - z * z) * dp * dp);
  }
  // map to [0,1]; xs[k] for k < n/2 are the points near +1
  x.clear();
  w.clear();
  for (int k = 0; k < n / 2; ++k) {
    long double lo = (1 - xs[k]) / 2, wk = ws[k] / 2;
    x.push_back(double(lo));
    w.push_back(double(wk));
    x.push_back(double(1 - lo));
    w.push_back(double(wk));
  }
  if (n % 2) {
    x.push_back(0.5);
    w.push_back(double(ws[n / 2] / 2));
  }
}

static bool parse_args(const std::string &name, const std::string &prefix, std::vector<int> &a) {
  if (name.compare(0, prefix.size(), prefix) != 0) return false;
  std::string rest = name.substr(prefix.size());
  if (rest.empty() || rest.back() != ')') return false;
  rest.pop_back();
  a.clear();
  size_t p = 0;
  while (p < rest.size()) {
    size_t q = rest.find(',', p);
    if (q == std::string::npos) q = rest.size();
    a.push_back(std::stoi(rest.substr(p, q - p)));
    p = q + 1;
  }
  return true;
}

bool quadrature_by_name(const std::string &name_in, Quadrature &q) {
  std::string name;
  for (char c : name_in)
    if (c != ' ') name += c;
  q = Quadrature();
  q.name = name;
  std::vector<int> a;
  const double *tab = nullptr;
  int n = 0, dim = 0;
  if (parse_args(name, "IM_TRIANGLE(", a) && a.size() == 1) {
    dim = 2;
    if (a[0] == 2) tab = kTri2, n = 3;
    else if (a[0] == 4) tab = kTri4, n = 6;
  } else if (parse_args(name, "IM_TETRAHEDRON(", a) && a.size() == 1) {
    dim = 3;
    if (a[0] == 2) tab = kTet2, n = 4;
    else if (a[0] == 5) tab = kTet5, n = 15;
  } else if ((parse_args(name, "IM_GAUSS1D(", a) && a.size() == 1) ||
             (parse_args(name, "IM_GAUSS_PARALLELEPIPED(", a) && a.size() == 2)) {
    dim = a.size() == 1 ? 1 : a[0];
    int K = a.back();
    if (dim < 1 || dim > 3 || K < 0 || K > 99) return false;
    std::vector<double> x, w;
    gauss_legendre01(K / 2 + 1, x, w);
    int m = int(x.size());
    q.dim = dim;
    q.nq = 1;
    for (int d = 0; d < dim; ++d) q.nq *= m;
    // tensor product, first coordinate fastest (IM_GAUSS_PARALLELEPIPED
    // = product of IM_GAUSS1D, getfem_integration.cc:842-845)
    for (int t = 0; t < q.nq; ++t) {
      int r = t;
      double wt = 1.0;
      for (int d = 0; d < dim; ++d) {
        int i = r % m;
        r /= m;
        q.pts.push_back(x[i]);
        wt *= w[i];
      }
      q.w.push_back(wt);
    }
    return true;
  }
  if (!tab) return false;
  q.dim = dim;
  q.nq = n;
  for (int i = 0; i < n; ++i) {
    for (int d = 0; d < dim; ++d) q.pts.push_back(tab[i * (dim + 1) + d]);
    q.w.push_back(tab[i * (dim + 1) + dim]);
  }
  return true;
}

// --------------------------------------------------------------------- mesh

// Simplex splits of the unit square / cube (vertex indices into the
// parallelepiped's points, first coordinate fastest), as in
// bgeot_convex_ref_simplexified.cc:28-39.
static const int kSplit2[2][3] = {{3, 0, 2}, {3, 0, 1}};
static const int kSplit3[6][4] = {{3, 7, 0, 1}, {7, 0, 5, 4}, {7, 0, 1, 5},
                                  {3, 7, 0, 2}, {6, 7, 0, 4}, {6, 7, 0, 2}};

void regular_unit_mesh(int dim, int kind, int nx, const double *jitter, Mesh &m) {
  if (dim < 2 || dim > 3 || nx < 1) throw std::invalid_argument("regular_unit_mesh: bad size");
  m = Mesh();
  m.dim = dim;
  m.kind = kind;
  const int ncorner = 1 << dim;
  m.nbpt = kind == SIMPLEX ? dim + 1 : ncorner;
  const int64_t L = nx + 1;
  int64_t nlat = 1;
  for (int d = 0; d < dim; ++d) nlat *= L;
  std::vector<int64_t> id_of_lattice(nlat, -1);
  const double h = 1. / double(nx) * 1.;
  int64_t ncubes = 1;
  for (int d = 0; d < dim; ++d) ncubes *= nx;
  std::vector<int> verts;
  int tab[3] = {0, 0, 0};
  for (int64_t c = 0; c < ncubes; ++c) {
    int64_t r = c;
    int total = 0;
    for (int d = 0; d < dim; ++d) tab[d] = int(r % nx), r /= nx, total += tab[d];
    verts.clear();
    if (kind == SIMPLEX) {
      // for dim != 3 every other cube uses the split rotated by half the
      // corners (getfem_regular_meshes.cc:62-66)
      int shift = ((total & 1) && dim != 3) ? ncorner / 2 : 0;
      int ns = dim == 2 ? 2 : 6;
      for (int s = 0; s < ns; ++s)
        for (int l = 0; l <= dim; ++l) {
          int p = dim == 2 ? kSplit2[s][l] : kSplit3[s][l];
          verts.push_back((p + shift) % ncorner);
        }
    } else {
      for (int p = 0; p < ncorner; ++p) verts.push_back(p);
    }
    int nv = m.nbpt;
    for (size_t k = 0; k < verts.size(); k += nv) {
      for (int l = 0; l < nv; ++l) {
        int p = verts[k + l];
        int64_t flat = 0, stride = 1;
        int lat[3];
        for (int d = 0; d < dim; ++d) {
          lat[d] = tab[d] + ((p >> d) & 1);
          flat += lat[d] * stride;
          stride *= L;
        }
        int64_t &id = id_of_lattice[flat];
        if (id < 0) {
          id = m.n_points++;
          for (int d = 0; d < dim; ++d) {
            // coordinates as the first cube (in cube order) containing the
            // point computes them: its origin plus one cell width
            int cb = std::max(lat[d] - 1, 0);
            double x = double(cb) * h + double(lat[d] - cb) * h;
            m.points.push_back(x);
            m.lattice.push_back(lat[d]);
          }
        }
        m.cvpts.push_back(id);
      }
      m.n_elements++;
    }
  }
  if (jitter) {
    for (int64_t i = 0; i < m.n_points; ++i) {
      bool interior = true;
      int64_t flat = 0, stride = 1;
      for (int d = 0; d < dim; ++d) {
        int l = m.lattice[i * dim + d];
        if (l <= 0 || l >= nx) interior = false;
        flat += l * stride;
        stride *= L;
      }
      if (interior)
        for (int d = 0; d < dim; ++d) m.points[i * dim + d] += jitter[flat * dim + d];
    }
  }
}

// ---------------------------------------------------------------- DOF maps

namespace {
// A DOF node is identified by the vertices that carry a nonzero weight in
// its barycentric (simplex) or multilinear (cube) expression, with those
// integer weights.  Shared nodes of neighbouring elements get equal keys.
struct NodeKey {
  int n = 0;
  int64_t v[8];
  int32_t w[8];
  bool operator==(const NodeKey &o) const {
    if (n != o.n) return false;
    for (int i = 0; i < n; ++i)
      if (v[i] != o.v[i] || w[i] != o.w[i]) return false;
    return true;
  }
};
struct NodeKeyHash {
  size_t operator()(const NodeKey &k) const {
    uint64_t h = 0x9e3779b97f4a7c15ULL ^ uint64_t(k.n);
    for (int i = 0; i < k.n; ++i) {
      h ^= uint64_t(k.v[i]) * 0xbf58476d1ce4e5b9ULL + uint64_t(uint32_t(k.w[i]));
      h = (h ^ (h >> 31)) * 0x94d049bb133111ebULL;
    }
    return size_t(h ^ (h >> 29));
  }
};
}  // namespace

int64_t enumerate_dofs(int dim, int kind, int degree, int qdim, int64_t n_elements,
                       const int64_t *cvpts, std::vector<int64_t> &dofs) {
  RefElement fe(dim, kind, degree);
  const int nb = fe.nb;
  dofs.assign(size_t(n_elements) * nb, 0);
  if (degree == 0) {
    for (int64_t e = 0; e < n_elements; ++e) dofs[e] = e * qdim;
    return n_elements * qdim;
  }
  const int nv = kind == SIMPLEX ? dim + 1 : (1 << dim);
  const int K = degree;
  // per local node: list of (local vertex, weight)
  std::vector<std::vector<std::pair<int, int>>> support(nb);
  for (int i = 0; i < nb; ++i) {
    const int *c = &fe.lattice[i * dim];
    if (kind == SIMPLEX) {
      int w0 = K;
      for (int d = 0; d < dim; ++d) w0 -= c[d];
      if (w0) support[i].push_back({0, w0});
      for (int d = 0; d < dim; ++d)
        if (c[d]) support[i].push_back({d + 1, c[d]});
    } else {
      for (int p = 0; p < nv; ++p) {
        int w = 1;
        for (int d = 0; d < dim; ++d) w *= ((p >> d) & 1) ? c[d] : (K - c[d]);
        if (w) support[i].push_back({p, w});
      }
    }
  }
  std::unordered_map<NodeKey, int64_t, NodeKeyHash> ids;
  ids.reserve(size_t(n_elements) * 2 + 16);
  int64_t next = 0;
  std::vector<std::pair<int64_t, int32_t>> tmp;
  for (int64_t e = 0; e < n_elements; ++e) {
    const int64_t *vp = cvpts + e * nv;
    for (int i = 0; i < nb; ++i) {
      tmp.clear();
      for (auto &s : support[i]) tmp.push_back({vp[s.first], s.second});
      std::sort(tmp.begin(), tmp.end());
      NodeKey k;
      k.n = int(tmp.size());
      for (int j = 0; j < k.n; ++j) k.v[j] = tmp[j].first, k.w[j] = tmp[j].second;
      auto it = ids.find(k);
      int64_t id;
      if (it == ids.end()) {
        id = next++;
        ids.emplace(k, id);
      } else {
        id = it->second;
      }
      dofs[size_t(e) * nb + i] = id * qdim;
    }
  }
  return next * qdim;
}

void dof_node_coordinates(const Mesh &m, int degree, int64_t n_dof, int qdim,
                          const std::vector<int64_t> &dofs, std::vector<double> &xyz) {
  RefElement fe(m.dim, m.kind, degree);
  RefElement gt(m.dim, m.kind, 1);
  int64_t nn = n_dof / qdim;
  xyz.assign(size_t(nn) * m.dim, 0.0);
  std::vector<double> val(gt.nb), grad(gt.nb * m.dim);
  double x[3];
  for (int64_t e = 0; e < m.n_elements; ++e) {
    for (int i = 0; i < fe.nb; ++i) {
      fe.node(i, x);
      gt.eval(x, val.data(), grad.data());
      int64_t node = dofs[size_t(e) * fe.nb + i] / qdim;
      for (int d = 0; d < m.dim; ++d) {
        double s = 0;
        for (int v = 0; v < gt.nb; ++v) s += val[v] * m.points[m.cvpts[e * gt.nb + v] * m.dim + d];
        xyz[node * m.dim + d] = s;
      }
    }
  }
}

}  // namespace gfgpu
