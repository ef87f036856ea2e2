// C ABI of the host-side input builders (no device code): structured
// meshes, DOF numbering and reference-element tables.
#include <cstring>
#include <exception>
#include <string>

#include "../../include/gfgpu.h"
#include "host/refelem.h"

namespace gfgpu {
thread_local std::string g_last_error;
void set_last_error(const std::string &s) { g_last_error = s; }
}  // namespace gfgpu

using namespace gfgpu;

extern "C" {

const char *gfgpu_version(void) { return "gfgpu 0.1 (sm_103a)"; }

const char *gfgpu_last_error(void) { return g_last_error.c_str(); }

int gfgpu_regular_unit_mesh(int32_t dim, int32_t kind, int32_t nx, const double *jitter,
                            int64_t *n_points, int64_t *n_elements, double *points,
                            int64_t *cvpts) {
  try {
    if (dim < 2 || dim > 3 || (kind != GFGPU_SIMPLEX && kind != GFGPU_HEX) || nx < 1) {
      set_last_error("regular_unit_mesh: bad arguments");
      return GFGPU_E_INVALID;
    }
    if (!points) {
      int64_t np = 1, ne = 1;
      for (int d = 0; d < dim; ++d) np *= (nx + 1), ne *= nx;
      if (kind == GFGPU_SIMPLEX) ne *= (dim == 2 ? 2 : 6);
      *n_points = np;
      *n_elements = ne;
      return GFGPU_OK;
    }
    Mesh m;
    regular_unit_mesh(dim, kind, nx, jitter, m);
    *n_points = m.n_points;
    *n_elements = m.n_elements;
    std::memcpy(points, m.points.data(), m.points.size() * sizeof(double));
    std::memcpy(cvpts, m.cvpts.data(), m.cvpts.size() * sizeof(int64_t));
    return GFGPU_OK;
  } catch (const std::exception &e) {
    set_last_error(e.what());
    return GFGPU_E_INVALID;
  }
}

int gfgpu_enumerate_dofs(int32_t dim, int32_t kind, int32_t degree, int32_t qdim,
                         int64_t n_elements, const int64_t *cvpts, int64_t *dofs,
                         int64_t *n_dof) {
  try {
    if (qdim < 1 || qdim > 3) {
      set_last_error("enumerate_dofs: bad qdim");
      return GFGPU_E_INVALID;
    }
    std::vector<int64_t> d;
    *n_dof = enumerate_dofs(dim, kind, degree, qdim, n_elements, cvpts, d);
    std::memcpy(dofs, d.data(), d.size() * sizeof(int64_t));
    return GFGPU_OK;
  } catch (const std::exception &e) {
    set_last_error(e.what());
    return GFGPU_E_INVALID;
  }
}

int gfgpu_nb_basis(int32_t dim, int32_t kind, int32_t degree, int32_t *nb) {
  try {
    RefElement fe(dim, kind, degree);
    *nb = fe.nb;
    return GFGPU_OK;
  } catch (const std::exception &e) {
    set_last_error(e.what());
    return GFGPU_E_INVALID;
  }
}

int gfgpu_quadrature(const char *im, int32_t *dim, int32_t *nq, double *pts, double *w) {
  Quadrature q;
  if (!im || !quadrature_by_name(im, q)) {
    set_last_error(std::string("unsupported integration method ") + (im ? im : "(null)"));
    return GFGPU_E_UNSUPPORTED;
  }
  *dim = q.dim;
  *nq = q.nq;
  if (pts) std::memcpy(pts, q.pts.data(), q.pts.size() * sizeof(double));
  if (w) std::memcpy(w, q.w.data(), q.w.size() * sizeof(double));
  return GFGPU_OK;
}

int gfgpu_basis_tables(int32_t dim, int32_t kind, int32_t degree, const char *im, double *val,
                       double *grad) {
  try {
    Quadrature q;
    if (!im || !quadrature_by_name(im, q) || q.dim != dim) {
      set_last_error("unsupported integration method");
      return GFGPU_E_UNSUPPORTED;
    }
    RefElement fe(dim, kind, degree);
    for (int k = 0; k < q.nq; ++k)
      fe.eval(&q.pts[size_t(k) * dim], val + size_t(k) * fe.nb, grad + size_t(k) * fe.nb * dim);
    return GFGPU_OK;
  } catch (const std::exception &e) {
    set_last_error(e.what());
    return GFGPU_E_INVALID;
  }
}

}  // extern "C"
