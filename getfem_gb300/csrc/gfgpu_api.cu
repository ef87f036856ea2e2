// C ABI of the device plans: creation (upload of the discretisation,
// node adjacency, tables), data slots, assembly and result access.
#include <cub/cub.cuh>
#include <cstdio>
#include <mutex>
#include <map>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <exception>
#include <new>
#include <string>
#include <vector>

#include "host/refelem.h"
#include "plan.h"

namespace gfgpu {
void set_last_error(const std::string &s);
}

using namespace gfgpu;

struct gfgpu_plan_s : public Plan {};

namespace gfgpu {
cudaError_t batch_gather_attr(size_t smem);
}

// A batch of affine-simplex plans launched together.
struct gfgpu_batch_s {
  std::vector<gfgpu_plan *> plans;
  // element pass: items grouped by element type, tile offsets per group
  BatchItem *d_eitems[kBatchElementTypes] = {};
  int64_t *d_tile0[kBatchElementTypes] = {};
  int en[kBatchElementTypes] = {};
  int64_t entiles[kBatchElementTypes] = {};
  int64_t elements = 0;
  // gather: items grouped by component count
  BatchItem *d_gitems[4] = {};
  int64_t *d_node0[4] = {};
  int gn[4] = {};
  int64_t gnodes[4] = {};
  size_t gwarp[4] = {};
  int grid_ep = 0, grid_ga = 0;
  int *d_err = nullptr;
  // the gather by valence class (per component count): nodes of every mesh
  // whose valence bucket has at most 2^c adjacent elements, as item << 32 |
  // node, with the class's slot and adjacency maxima
  struct GatherClass {
    int64_t *d_list = nullptr;
    int64_t n = 0;
    int ms = 1, mad = 1;
    size_t wb = 0;
  };
  std::vector<GatherClass> gclass[4];
};

namespace {

#define GF_CUDA(call)                                                          \
  do {                                                                         \
    cudaError_t ce_ = (call);                                                  \
    if (ce_ != cudaSuccess) {                                                  \
      set_last_error(std::string(#call) + ": " + cudaGetErrorString(ce_));     \
      return ce_ == cudaErrorMemoryAllocation ? GFGPU_E_NOMEM : GFGPU_E_CUDA;  \
    }                                                                          \
  } while (0)

template <class T>
int dalloc(T **p, size_t n) {
  *p = nullptr;
  if (n == 0) n = 1;
  const cudaError_t ce = cudaMalloc(reinterpret_cast<void **>(p), n * sizeof(T));
  if (ce != cudaSuccess) {
    set_last_error("cudaMalloc of " + std::to_string(n * sizeof(T)) + " bytes: " +
                   cudaGetErrorString(ce));
    return ce == cudaErrorMemoryAllocation ? GFGPU_E_NOMEM : GFGPU_E_CUDA;
  }
  return GFGPU_OK;
}

template <class T>
void dfree(T *&p) {
  if (p) cudaFree(const_cast<void *>(reinterpret_cast<const void *>(p)));
  p = nullptr;
}

}  // namespace

namespace gfgpu {
// The forms the affine-simplex element pass lowers: GRADGRAD / MASS with
// constant or per-element coefficients, one GRADGRAD_TENSOR (a constant
// symmetric D, constant or per-element factor), SOURCE with a field on the
// variable's mesh_fem and a constant factor.
bool simplex_form_supported(const gfgpu_form &f, int qdim, int dim, std::string &why) {
  if (f.n_terms < 1 || f.n_terms > GFGPU_MAX_TERMS) {
    why = "empty form";
    return false;
  }
  int nsrc = 0, nten = 0;
  for (int t = 0; t < f.n_terms; ++t) {
    const gfgpu_term &T = f.terms[t];
    if (T.kind == GFGPU_TERM_GRADGRAD_TENSOR) {
      if (++nten > 1) {
        why = "at most one anisotropic (tensor) gradient coupling";
        return false;
      }
      if (qdim != 1 && qdim != dim) {
        why = "qdim must be 1 or the mesh dimension";
        return false;
      }
      if (T.c[0].kind != GFGPU_COEF_NONE && T.c[0].kind != GFGPU_COEF_CONST &&
          T.c[0].kind != GFGPU_COEF_ELEMENT) {
        why = "the tensor coupling's factor must be constant or per element";
        return false;
      }
      if (T.c[0].kind == GFGPU_COEF_ELEMENT && (T.c[0].slot < 0 || T.c[0].slot >= GFGPU_MAX_SLOTS)) {
        why = "bad coefficient slot";
        return false;
      }
      const int nd = qdim * dim;
      for (int r = 0; r < nd; ++r)
        for (int c = 0; c < nd; ++c) {
          const double x = f.tensor[r * nd + c];
          if (!std::isfinite(x) || x != f.tensor[c * nd + r]) {
            why = "the coupling tensor must be finite and symmetric, D[(a,k),(b,l)] == D[(b,l),(a,k)]";
            return false;
          }
        }
      continue;
    }
    if (T.kind == GFGPU_TERM_GRADGRAD || T.kind == GFGPU_TERM_MASS) {
      int nc = T.kind == GFGPU_TERM_GRADGRAD ? 3 : 1;
      for (int k = 0; k < nc; ++k)
        if (T.c[k].kind == GFGPU_COEF_NODAL) {
          why = "nodal coefficient fields need the Gauss-point path (not built for simplices)";
          return false;
        }
      if (T.kind == GFGPU_TERM_GRADGRAD && qdim == 1 &&
          (T.c[0].kind != GFGPU_COEF_NONE || T.c[2].kind != GFGPU_COEF_NONE)) {
        why = "div/transpose couplings need a vector field with qdim == dim";
        return false;
      }
      if (T.kind == GFGPU_TERM_GRADGRAD && qdim > 1 && qdim != dim) {
        why = "qdim must equal the mesh dimension";
        return false;
      }
    } else if (T.kind == GFGPU_TERM_SOURCE) {
      if (++nsrc > 1) {
        why = "at most one source term";
        return false;
      }
      if (T.c[0].kind != GFGPU_COEF_NONE && T.c[0].kind != GFGPU_COEF_CONST) {
        why = "source factor must be constant";
        return false;
      }
      if (T.field_slot <= 0 || T.field_slot >= GFGPU_MAX_SLOTS) {
        why = "bad source field slot";
        return false;
      }
    } else {
      why = "term kind not lowered on simplices";
      return false;
    }
  }
  return true;
}
}  // namespace gfgpu

namespace {
// The forms of the Gauss-point kernels: GRADGRAD / MASS / SOURCE terms
// with constant, per-element or nodal coefficients and at most one internal
// pressure term (LAW_ISO), or one compressible neo-Hookean term on a 3-D
// vector field (LAW_NH).
bool gauss_form_supported(const gfgpu_form &f, int qdim, int dim, int &law, std::string &why) {
  if (f.n_terms < 1 || f.n_terms > GFGPU_MAX_TERMS) {
    why = "empty form";
    return false;
  }
  law = LAW_ISO;
  int n_int = 0;
  for (int t = 0; t < f.n_terms; ++t) {
    const gfgpu_term &T = f.terms[t];
    if (T.kind == GFGPU_TERM_NEOHOOKEAN) {
      if (f.n_terms != 1) {
        why = "a neo-Hookean term is lowered alone";
        return false;
      }
      if (qdim != 3 || dim != 3) {
        why = "neo-Hookean law is 3-D only";
        return false;
      }
      law = LAW_NH;
    } else if (T.kind == GFGPU_TERM_GRADGRAD) {
      if (qdim == 1 && (T.c[0].kind != GFGPU_COEF_NONE || T.c[2].kind != GFGPU_COEF_NONE)) {
        why = "div/transpose couplings need a vector field with qdim == dim";
        return false;
      }
      if (qdim > 1 && qdim != dim) {
        why = "qdim must equal the mesh dimension";
        return false;
      }
    } else if (T.kind == GFGPU_TERM_SOURCE) {
      if (T.field_slot <= 0 || T.field_slot >= GFGPU_MAX_SLOTS) {
        why = "bad source field slot";
        return false;
      }
    } else if (T.kind == GFGPU_TERM_INTERNAL_P) {
      if (++n_int > 1) {
        why = "at most one internal-variable term";
        return false;
      }
      if (qdim != 3 || dim != 3) {
        why = "internal pressure terms are lowered for 3-D vector fields";
        return false;
      }
      if (T.field_slot <= 0 || T.field_slot >= GFGPU_MAX_SLOTS || T.aux_slot <= 0 ||
          T.aux_slot >= GFGPU_MAX_SLOTS || T.aux_slot == T.field_slot) {
        why = "bad internal variable slots";
        return false;
      }
    } else if (T.kind != GFGPU_TERM_MASS) {
      why = "unknown term kind";
      return false;
    }
  }
  if (n_int && law == LAW_NH) {
    why = "internal variables with the neo-Hookean law are not lowered";
    return false;
  }
  return true;
}

int status_from_err(int e) {
  if (e & ERR_JACOBIAN) {
    set_last_error("Non invertible matrix (det of the geometric transformation is 0)");
    return GFGPU_E_JACOBIAN;
  }
  if (e & ERR_NAN) {
    set_last_error("non-finite value in assembly");
    return GFGPU_E_NAN;
  }
  if (e & ERR_CAPACITY) {
    set_last_error("a DOF node couples to more nodes than the kernel holds");
    return GFGPU_E_UNSUPPORTED;
  }
  if (e & ERR_TIMEOUT) {
    set_last_error("device wait timed out");
    return GFGPU_E_TIMEOUT;
  }
  if (e & ERR_PATTERN) {
    set_last_error("element entries outside the cached CSR pattern (entries that were zero "
                   "when the pattern was built are nonzero now)");
    return GFGPU_E_STATE;
  }
  return GFGPU_OK;
}

int build_pattern(Plan &P) {
  P.pattern_builds++;
  // counts per row and per node (int64: the scans accumulate in the input
  // type, and the node-level total passes 2^31 on large meshes)
  GF_CUDA(cudaMemsetAsync(P.d_count, 0, (P.n_dof + 1) * sizeof(int64_t), P.stream));
  GF_CUDA(cudaMemsetAsync(P.d_ncount, 0, (P.n_nodes + 1) * sizeof(int64_t), P.stream));
  GF_CUDA(launch_pattern_count(P));
  size_t need = 0, need2 = 0, need3 = 0;
  cub::DeviceScan::ExclusiveSum(nullptr, need, P.d_count, P.d_rowptr, P.n_dof + 1);
  cub::DeviceScan::ExclusiveSum(nullptr, need2, P.d_ncount, P.d_nptr, P.n_nodes + 1);
  int64_t *d_max = nullptr;
  cub::DeviceReduce::Max(nullptr, need3, P.d_ncount, d_max, P.n_nodes + 1);
  need = std::max(need, std::max(need2, need3 + 16));
  if (need > P.cub_bytes) {
    dfree(P.d_cub);
    GF_CUDA(cudaMalloc(&P.d_cub, need));
    P.cub_bytes = need;
  }
  GF_CUDA(cub::DeviceScan::ExclusiveSum(P.d_cub, P.cub_bytes, P.d_count, P.d_rowptr, P.n_dof + 1,
                                        P.stream));
  GF_CUDA(cub::DeviceScan::ExclusiveSum(P.d_cub, P.cub_bytes, P.d_ncount, P.d_nptr,
                                        P.n_nodes + 1, P.stream));
  P.launches += 2;
  int64_t nnz = 0, nn = 0;
  GF_CUDA(cudaMemcpyAsync(&nnz, P.d_rowptr + P.n_dof, sizeof(int64_t), cudaMemcpyDeviceToHost,
                          P.stream));
  GF_CUDA(cudaMemcpyAsync(&nn, P.d_nptr + P.n_nodes, sizeof(int64_t), cudaMemcpyDeviceToHost,
                          P.stream));
  // max slots per node
  int64_t *d_mx = P.d_count;  // reuse: counts are consumed
  GF_CUDA(cub::DeviceReduce::Max(P.d_cub, P.cub_bytes, P.d_ncount, d_mx, P.n_nodes + 1, P.stream));
  P.launches++;
  int64_t mx64 = 0;
  GF_CUDA(cudaMemcpyAsync(&mx64, d_mx, sizeof(int64_t), cudaMemcpyDeviceToHost, P.stream));
  GF_CUDA(cudaStreamSynchronize(P.stream));
  int herr = 0;
  GF_CUDA(cudaMemcpy(&herr, P.d_err, sizeof(int), cudaMemcpyDeviceToHost));
  if (herr) return status_from_err(herr);
  dfree(P.d_colidx);
  dfree(P.d_vals);
  dfree(P.d_ncol);
  dfree(P.d_nbits);
  dfree(P.d_slotmap);
  int rc;
  if ((rc = dalloc(&P.d_colidx, size_t(nnz)))) return rc;
  if ((rc = dalloc(&P.d_vals, size_t(nnz)))) return rc;
  if ((rc = dalloc(&P.d_ncol, size_t(nn)))) return rc;
  if ((rc = dalloc(&P.d_nbits, size_t(nn)))) return rc;
  if ((rc = dalloc(&P.d_slotmap, size_t(P.n_elements) * P.nb * P.nb))) return rc;
  P.nnz = nnz;
  P.max_slots = int32_t(mx64);
  GF_CUDA(launch_pattern_fill(P));
  // the node-level column lists feed the fill, and (affine simplices) the
  // row gather's K u of the fused K + R assembly
  GF_CUDA(cudaStreamSynchronize(P.stream));
  if (!P.affine_simplex) dfree(P.d_ncol);
  // row pointers on the host (chunked copies of gfgpu_assemble_host)
  P.h_rowptr.resize(size_t(P.n_dof + 1));
  GF_CUDA(cudaMemcpy(P.h_rowptr.data(), P.d_rowptr, size_t(P.n_dof + 1) * sizeof(int64_t),
                     cudaMemcpyDeviceToHost));
  // pattern slots per valence bucket of the row gather
  if (!P.h_order.empty()) {
    std::vector<int64_t> nptr(size_t(P.n_nodes + 1));
    GF_CUDA(cudaMemcpy(nptr.data(), P.d_nptr, nptr.size() * sizeof(int64_t),
                       cudaMemcpyDeviceToHost));
    P.bucket_ms.assign(P.h_bucket.size() - 1, 0);
    for (size_t b = 0; b + 1 < P.h_bucket.size(); ++b)
      for (int64_t i = P.h_bucket[b]; i < P.h_bucket[b + 1]; ++i) {
        const int32_t n = P.h_order[size_t(i)];
        P.bucket_ms[b] = std::max<int32_t>(P.bucket_ms[b], int32_t(nptr[n + 1] - nptr[n]));
      }
  }
  return GFGPU_OK;
}

// Waits for the plan's stream and maps its error word to a status.  With
// repair, an ERR_PATTERN alone (the last gather met element entries the
// cached pattern lacks) is resolved as the reference would store them: the
// pattern is rebuilt from the current element matrices (the reference
// rebuilds K's sparse columns at every assembly) and the gather runs again.
int check_err(Plan &P, bool repair = false) {
  int herr = 0;
  GF_CUDA(cudaStreamSynchronize(P.stream));
  GF_CUDA(cudaMemcpy(&herr, P.d_err, sizeof(int), cudaMemcpyDeviceToHost));
  if (repair && herr == ERR_PATTERN) {
    GF_CUDA(cudaMemsetAsync(P.d_err, 0, sizeof(int), P.stream));
    int rc = build_pattern(P);
    if (rc) return rc;
    GF_CUDA(launch_gather(P, true, P.last_want_R));
    GF_CUDA(cudaStreamSynchronize(P.stream));
    GF_CUDA(cudaMemcpy(&herr, P.d_err, sizeof(int), cudaMemcpyDeviceToHost));
  }
  return status_from_err(herr);
}

// The parallelepiped kernels of a plan need parallelepipeds: after
// gfgpu_set_points moved the vertices off them, orders 1 and 2 fail loudly.
// ------------------------------------------------- launch configurations

std::mutex g_tune_mutex;
std::map<std::string, LaunchConfig> g_tuned;  // family|GPU -> configuration

std::string gpu_name() {
  int dev = 0;
  cudaDeviceProp prop;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaGetDeviceProperties(&prop, dev) != cudaSuccess)
    return "unknown";
  std::string n(prop.name);
  for (char &c : n)
    if (c == ' ' || c == '|') c = '_';
  return n;
}

// the kernels a plan's K pass runs: element kind and degree, components,
// Gauss points, which element kernel
std::string family_key(const Plan &P) {
  std::string k = P.affine_simplex ? "simplex" : P.affine_hex ? "parallelepiped" : "gauss";
  k += "-d" + std::to_string(P.dim) + "-k" + std::to_string(P.kind) + "-p" +
       std::to_string(P.degree) + "-q" + std::to_string(P.qdim) + "-nq" + std::to_string(P.nq) +
       "-law" + std::to_string(P.law);
  // forms with an anisotropic coupling run their own element-pass instances
  if (P.affine_simplex && form_has_tensor(P.form)) k += "-tensor";
  return k + "|" + gpu_name();
}

std::vector<int> ep_candidates(const Plan &P) {
  // (the anisotropic-coupling instances exist at 4 threads per element)
  if (P.affine_simplex && form_has_tensor(P.form)) return {4};
  if (P.affine_simplex) return {2, 4, 8};
  return {128, 256, 512};
}

void recorded_launch(Plan &P) {
  std::lock_guard<std::mutex> lock(g_tune_mutex);
  auto it = g_tuned.find(family_key(P));
  if (it != g_tuned.end()) P.tune = it->second;
}

int check_geometry(const Plan &P) {
  if (P.affine_hex && !P.parallelepiped) {
    set_last_error("the mesh points set by gfgpu_set_points no longer form parallelepipeds, "
                   "which this plan's element kernel requires: create a new plan");
    return GFGPU_E_UNSUPPORTED;
  }
  return GFGPU_OK;
}

// The upper triangle of the current pattern (entries with column >= row):
// per-row skips, row pointers (device and host) and the value buffer.
int build_upper(Plan &P) {
  if (P.upper_build == P.pattern_builds && P.d_urowptr) return GFGPU_OK;
  dfree(P.d_urowptr);
  dfree(P.d_uskip);
  dfree(P.d_uvals);
  P.upper_build = -1;
  int rc;
  if ((rc = dalloc(&P.d_urowptr, size_t(P.n_dof + 1)))) return rc;
  if ((rc = dalloc(&P.d_uskip, size_t(P.n_dof)))) return rc;
  // row lengths into d_count (scratch of n_dof + 1, free after a pattern build)
  GF_CUDA(cudaMemsetAsync(P.d_count, 0, size_t(P.n_dof + 1) * sizeof(int64_t), P.stream));
  GF_CUDA(launch_upper_count(P, P.d_count));
  size_t need = 0;
  cub::DeviceScan::ExclusiveSum(nullptr, need, P.d_count, P.d_urowptr, P.n_dof + 1);
  if (need > P.cub_bytes) {
    dfree(P.d_cub);
    GF_CUDA(cudaMalloc(&P.d_cub, need));
    P.cub_bytes = need;
  }
  GF_CUDA(cub::DeviceScan::ExclusiveSum(P.d_cub, P.cub_bytes, P.d_count, P.d_urowptr,
                                        P.n_dof + 1, P.stream));
  P.launches++;
  P.h_urowptr.resize(size_t(P.n_dof + 1));
  GF_CUDA(cudaMemcpyAsync(P.h_urowptr.data(), P.d_urowptr, size_t(P.n_dof + 1) * sizeof(int64_t),
                          cudaMemcpyDeviceToHost, P.stream));
  GF_CUDA(cudaStreamSynchronize(P.stream));
  P.nnz_upper = P.h_urowptr.back();
  if ((rc = dalloc(&P.d_uvals, size_t(P.nnz_upper)))) return rc;
  P.upper_build = P.pattern_builds;
  return GFGPU_OK;
}

}  // namespace

extern "C" {

int gfgpu_plan_create(const gfgpu_space *space, const gfgpu_form *form, void *cuda_stream,
                      gfgpu_plan **out) {
  if (!space || !form || !out) {
    set_last_error("null argument");
    return GFGPU_E_INVALID;
  }
  *out = nullptr;
  const gfgpu_space &S = *space;
  if (S.dim < 2 || S.dim > 3 || (S.kind != GFGPU_SIMPLEX && S.kind != GFGPU_HEX) ||
      S.degree < 1 || S.qdim < 1 || S.qdim > 3 || S.n_elements < 0 || S.n_points < 0 ||
      S.n_dof < 0 || S.n_dof % S.qdim || !S.im) {
    set_last_error("gfgpu_plan_create: bad space");
    return GFGPU_E_INVALID;
  }
  if (S.n_elements > 0 && (!S.points || !S.cvpts || !S.dofs)) {
    set_last_error("gfgpu_plan_create: missing arrays");
    return GFGPU_E_INVALID;
  }
  int dev_count = 0;
  if (cudaGetDeviceCount(&dev_count) != cudaSuccess || dev_count == 0) {
    set_last_error("no CUDA device");
    return GFGPU_E_CUDA;
  }
  gfgpu_plan *P = new (std::nothrow) gfgpu_plan();
  if (!P) return GFGPU_E_NOMEM;
  int rc = GFGPU_OK;
  try {
    P->dim = S.dim;
    P->kind = S.kind;
    P->degree = S.degree;
    P->qdim = S.qdim;
    P->im = S.im;
    P->form = *form;
    P->stream = static_cast<cudaStream_t>(cuda_stream);
    P->n_points = S.n_points;
    P->n_elements = S.n_elements;
    P->n_dof = S.n_dof;
    P->n_nodes = S.n_dof / S.qdim;
    RefElement fe(S.dim, S.kind, S.degree);
    P->nb = fe.nb;
    P->nbg = S.kind == GFGPU_SIMPLEX ? S.dim + 1 : (1 << S.dim);
    std::string why, err;
    if ((S.kind == GFGPU_SIMPLEX && S.degree > 2) || (S.kind == GFGPU_HEX && S.dim != 3)) {
      set_last_error("element not lowered: FEM_PK(dim,1|2) on simplices, FEM_QK(3,K) on hexahedra");
      delete P;
      return GFGPU_E_UNSUPPORTED;
    }
    // orders 1 and 2: the affine-simplex pass for the linear forms on
    // simplices, else the Gauss-point element kernel; order 0: the
    // Gauss-point potential kernel
    if (S.kind == GFGPU_SIMPLEX && simplex_form_supported(P->form, S.qdim, S.dim, why)) {
      P->affine_simplex = true;
      if ((rc = build_simplex_tables(*P, err)) != GFGPU_OK) {
        set_last_error(err);
        delete P;
        return rc;
      }
    } else if (std::string gwhy; !gauss_form_supported(P->form, S.qdim, S.dim, P->law, gwhy)) {
      // an anisotropic coupling is lowered by the simplex pass only: its
      // reason is the one to report on simplices
      set_last_error("form not supported: " +
                     (S.kind == GFGPU_SIMPLEX && form_has_tensor(P->form) ? why : gwhy));
      delete P;
      return GFGPU_E_UNSUPPORTED;
    }
    if ((rc = build_gauss_tables(*P, err)) != GFGPU_OK) {
      set_last_error(err);
      delete P;
      return rc;
    }
    if (S.kind == GFGPU_HEX) {
      P->parallelepiped = mesh_is_parallelepiped(S.points, S.cvpts, S.n_elements);
      P->axis_aligned =
          P->parallelepiped && mesh_is_axis_aligned(S.points, S.cvpts, S.n_elements);
      P->h_cvpts.assign(S.cvpts, S.cvpts + S.n_elements * 8);
    }
    if (!P->affine_simplex) {
      // parallelepiped hexahedra with a scalar isotropic form take the
      // reference-tensor kernel; the rest the Gauss-point kernel
      if (S.kind == GFGPU_HEX && P->law == LAW_ISO && affine_hex_form_ok(P->form, S.qdim) &&
          affine_hex_available(S.degree) && P->parallelepiped) {
        P->affine_hex = true;
        P->kmat = true;
        build_affine_hex_tables(*P);
        build_affine_hex_sumfac(*P);
      } else {
        P->kmat = S.dim == 3 && gauss_element_available(S.kind, P->law, S.degree, S.qdim, P->nq);
        gauss_element_layout(*P);
      }
    }
    for (int t = 0; t < P->form.n_terms; ++t)
      if (P->form.terms[t].kind == GFGPU_TERM_INTERNAL_P) P->ip_term = t;
    // every other lowered term has a symmetric element matrix, which every
    // element kernel computes once per pair and mirrors: K is symmetric bit
    // for bit
    P->symmetric = P->ip_term < 0;
    // potentials of forms with an internal variable are not lowered
    P->kpot = P->ip_term < 0 && gauss_potential_available(S.dim, S.kind, S.degree, S.qdim, P->law);
    if (!P->kmat && !P->kpot) {
      set_last_error("no kernel for this element, integration method and form");
      delete P;
      return GFGPU_E_UNSUPPORTED;
    }
    // launch configuration: the family's default, or the one recorded by
    // gfgpu_tune / gfgpu_tune_load for this family on this GPU model
    P->tune.ep_threads = P->affine_simplex ? 4 : 256;
    P->tune.gather_warps = 4;
    recorded_launch(*P);
    const int64_t E = S.n_elements, nb = P->nb, nbg = P->nbg;
    // validate and convert indices
    std::vector<int32_t> cv(size_t(E * nbg)), en(size_t(E * nb));
    for (int64_t k = 0; k < E * nbg; ++k) {
      if (S.cvpts[k] < 0 || S.cvpts[k] >= S.n_points) throw std::runtime_error("bad convex point index");
      cv[k] = int32_t(S.cvpts[k]);
    }
    for (int64_t k = 0; k < E * nb; ++k) {
      if (S.dofs[k] < 0 || S.dofs[k] >= S.n_dof || S.dofs[k] % S.qdim)
        throw std::runtime_error("bad DOF index");
      en[k] = int32_t(S.dofs[k] / S.qdim);
    }
    // node -> (element, local node) adjacency, element order within a node
    std::vector<int32_t> aptr(size_t(P->n_nodes + 1), 0), adj(size_t(E * nb));
    for (int64_t k = 0; k < E * nb; ++k) aptr[en[k] + 1]++;
    for (int64_t i = 0; i < P->n_nodes; ++i) {
      P->max_adj = std::max(P->max_adj, aptr[i + 1]);
      aptr[i + 1] += aptr[i];
    }
    {
      std::vector<int32_t> fill(aptr.begin(), aptr.end() - 1);
      for (int64_t e = 0; e < E; ++e)
        for (int li = 0; li < nb; ++li) adj[fill[en[e * nb + li]]++] = int32_t(e * nb + li);
    }
    // point -> (element, vertex) adjacency for the shape gradient
    std::vector<int32_t> pptr(size_t(S.n_points + 1), 0), padj(size_t(E * nbg));
    for (int64_t k = 0; k < E * nbg; ++k) pptr[cv[k] + 1]++;
    for (int64_t i = 0; i < S.n_points; ++i) pptr[i + 1] += pptr[i];
    {
      std::vector<int32_t> fill(pptr.begin(), pptr.end() - 1);
      for (int64_t k = 0; k < E * nbg; ++k) padj[fill[cv[k]]++] = int32_t(k);
    }
    if (P->ip_term >= 0) P->h_en = en;
    // valence buckets of the row gather (ceil(log2(adjacent elements)))
    {
      auto bucket_of = [](int32_t v) {
        int b = 0;
        while ((int64_t(1) << b) < v) ++b;
        return b;
      };
      std::vector<int64_t> cnt(34, 0);
      std::vector<int32_t> mad(33, 0);
      for (int64_t i = 0; i < P->n_nodes; ++i) {
        const int32_t v = aptr[i + 1] - aptr[i];
        const int b = bucket_of(v);
        cnt[b + 1]++;
        mad[b] = std::max(mad[b], v);
      }
      for (int b = 0; b < 33; ++b) cnt[b + 1] += cnt[b];
      P->h_order.assign(size_t(P->n_nodes), 0);
      std::vector<int64_t> fill(cnt.begin(), cnt.end() - 1);
      for (int64_t i = 0; i < P->n_nodes; ++i)
        P->h_order[size_t(fill[bucket_of(aptr[i + 1] - aptr[i])]++)] = int32_t(i);
      // buckets of fewer nodes than one wave of blocks join the next one (a
      // launch of a few blocks is mostly tail)
      const int64_t small = 152 * 8 * 4;
      P->h_bucket.assign(1, 0);
      P->bucket_mad.clear();
      int32_t carry = 0;
      std::vector<int> merged_of(33, 0), pending;
      for (int b = 0; b < 33; ++b) {
        if (cnt[b + 1] == cnt[b]) continue;
        carry = std::max(carry, mad[b]);
        pending.push_back(b);
        const bool last = cnt[b + 1] == cnt[33];
        if (cnt[b + 1] - P->h_bucket.back() < small && !last) continue;
        P->h_bucket.push_back(cnt[b + 1]);
        P->bucket_mad.push_back(carry);
        for (int q : pending) merged_of[q] = int(P->h_bucket.size()) - 2;
        pending.clear();
        carry = 0;
      }
      // the same buckets within each chunk of gfgpu_assemble_host: chunk c
      // keeps its nodes [n0, n1) in positions [n0, n1) of h_corder, ordered
      // by bucket; h_cbucket[c * (nmb + 1) + m] starts bucket m
      const int nmb = int(P->h_bucket.size()) - 1;
      P->h_corder.assign(size_t(P->n_nodes), 0);
      P->h_cbucket.assign(size_t(kHostChunks) * (nmb + 1), 0);
      for (int c = 0; c < kHostChunks && nmb > 0; ++c) {
        const int64_t n0 = P->n_nodes * c / kHostChunks, n1 = P->n_nodes * (c + 1) / kHostChunks;
        int64_t *cb = P->h_cbucket.data() + size_t(c) * (nmb + 1);
        std::vector<int64_t> ccnt(size_t(nmb + 1), 0);
        for (int64_t i = n0; i < n1; ++i) ccnt[merged_of[bucket_of(aptr[i + 1] - aptr[i])] + 1]++;
        cb[0] = n0;
        for (int m = 0; m < nmb; ++m) cb[m + 1] = cb[m] + ccnt[m + 1];
        std::vector<int64_t> cfill(cb, cb + nmb);
        for (int64_t i = n0; i < n1; ++i)
          P->h_corder[size_t(cfill[merged_of[bucket_of(aptr[i + 1] - aptr[i])]]++)] = int32_t(i);
      }
    }
    // host-buffer assembly: for each gather chunk of DOF nodes, one past the
    // largest element adjacent to it (adjacency codes are sorted by element)
    P->h_chunk_eend.assign(kHostChunks, 0);
    for (int c = 0; c < kHostChunks; ++c) {
      const int64_t n0 = P->n_nodes * c / kHostChunks, n1 = P->n_nodes * (c + 1) / kHostChunks;
      int64_t eend = c ? P->h_chunk_eend[c - 1] : 0;
      for (int64_t i = n0; i < n1; ++i)
        if (aptr[i + 1] > aptr[i]) eend = std::max<int64_t>(eend, adj[aptr[i + 1] - 1] / nb + 1);
      P->h_chunk_eend[c] = eend;
    }
    P->max_cand = int32_t(P->max_adj * nb);
    if (P->max_cand > 4096) throw std::runtime_error("node valence too large for the pattern kernel");
    if (P->nb > 128) throw std::runtime_error("more than 128 local nodes per element");
    if (P->max_cand > 32767) throw std::runtime_error("row slot index exceeds int16");
#define CHK(x)                   \
  if ((rc = (x)) != GFGPU_OK) { \
    gfgpu_plan_destroy(P);       \
    return rc;                   \
  }
    CHK(dalloc(&P->d_points, size_t(S.n_points * S.dim)));
    CHK(dalloc(&P->d_cv, cv.size()));
    CHK(dalloc(&P->d_enode, en.size()));
    CHK(dalloc(&P->d_adj_ptr, aptr.size()));
    CHK(dalloc(&P->d_adj, adj.size()));
    CHK(dalloc(&P->d_stab, 1));

    CHK(dalloc(&P->d_vec, size_t(S.n_dof)));
    CHK(dalloc(&P->d_pot, 1));
    CHK(dalloc(&P->d_err, 1));
    CHK(dalloc(&P->d_count, size_t(S.n_dof + 1)));
    CHK(dalloc(&P->d_ncount, size_t(P->n_nodes + 1)));
    CHK(dalloc(&P->d_rowptr, size_t(S.n_dof + 1)));
    CHK(dalloc(&P->d_nptr, size_t(P->n_nodes + 1)));
    auto up = [&](void *dst, const void *src, size_t bytes) -> int {
      GF_CUDA(cudaMemcpy(dst, src, bytes, cudaMemcpyHostToDevice));
      return GFGPU_OK;
    };
    CHK(up(P->d_points, S.points, size_t(S.n_points * S.dim) * sizeof(double)));
    CHK(up(P->d_cv, cv.data(), cv.size() * sizeof(int32_t)));
    CHK(up(P->d_enode, en.data(), en.size() * sizeof(int32_t)));
    CHK(up(P->d_adj_ptr, aptr.data(), aptr.size() * sizeof(int32_t)));
    CHK(up(P->d_adj, adj.data(), adj.size() * sizeof(int32_t)));
    CHK(up(P->d_stab, &P->stab, sizeof(SimplexTables)));
    if (!P->h_aff.empty()) {
      CHK(dalloc(&P->d_aff, P->h_aff.size()));
      CHK(up(P->d_aff, P->h_aff.data(), P->h_aff.size() * sizeof(double)));
    }
    if (!P->h_sf.empty()) {
      CHK(dalloc(&P->d_sf, P->h_sf.size()));
      CHK(up(P->d_sf, P->h_sf.data(), P->h_sf.size() * sizeof(double)));
    }
    if (!P->h_tri.empty()) {
      CHK(dalloc(&P->d_tri, P->h_tri.size()));
      CHK(up(P->d_tri, P->h_tri.data(), P->h_tri.size() * sizeof(int32_t)));
    }
    if (!P->h_corder.empty()) {
      CHK(dalloc(&P->d_corder, P->h_corder.size()));
      CHK(up(P->d_corder, P->h_corder.data(), P->h_corder.size() * sizeof(int32_t)));
    }
    if (!P->h_order.empty()) {
      CHK(dalloc(&P->d_order, P->h_order.size()));
      CHK(up(P->d_order, P->h_order.data(), P->h_order.size() * sizeof(int32_t)));
    }
    CHK(dalloc(&P->d_padj_ptr, pptr.size()));
    CHK(dalloc(&P->d_padj, padj.size()));
    CHK(up(P->d_padj_ptr, pptr.data(), pptr.size() * sizeof(int32_t)));
    CHK(up(P->d_padj, padj.data(), padj.size() * sizeof(int32_t)));
    {
      CHK(dalloc(&P->d_hval, P->h_val.size()));
      CHK(dalloc(&P->d_hgrad, P->h_grad.size()));
      CHK(dalloc(&P->d_ggrad, P->h_ggrad.size()));
      CHK(dalloc(&P->d_hw, P->h_w.size()));
      CHK(up(P->d_hval, P->h_val.data(), P->h_val.size() * sizeof(double)));
      CHK(up(P->d_hgrad, P->h_grad.data(), P->h_grad.size() * sizeof(double)));
      CHK(up(P->d_ggrad, P->h_ggrad.data(), P->h_ggrad.size() * sizeof(double)));
      CHK(up(P->d_hw, P->h_w.data(), P->h_w.size() * sizeof(double)));
      // transposed copies for the lane-per-Gauss-point kernels
      const int nq = P->nq, nbb = P->nb, D = P->dim;
      std::vector<double> vt(size_t(nbb) * nq), gt(size_t(nbb) * D * nq);
      for (int q = 0; q < nq; ++q)
        for (int j = 0; j < nbb; ++j) {
          vt[size_t(j) * nq + q] = P->h_val[size_t(q) * nbb + j];
          for (int m = 0; m < D; ++m)
            gt[(size_t(j) * D + m) * nq + q] = P->h_grad[(size_t(q) * nbb + j) * D + m];
        }
      CHK(dalloc(&P->d_hvalT, vt.size()));
      CHK(dalloc(&P->d_hgradT, gt.size()));
      CHK(up(P->d_hvalT, vt.data(), vt.size() * sizeof(double)));
      CHK(up(P->d_hgradT, gt.data(), gt.size() * sizeof(double)));
    }
    GF_CUDA(cudaMemset(P->d_err, 0, sizeof(int)));
    GF_CUDA(cudaMemset(P->d_vec, 0, size_t(S.n_dof) * sizeof(double)));
#undef CHK
  } catch (const std::exception &e) {
    set_last_error(e.what());
    gfgpu_plan_destroy(P);
    return GFGPU_E_INVALID;
  }
  *out = P;
  return GFGPU_OK;
}

void gfgpu_plan_destroy(gfgpu_plan *P) {
  if (!P) return;
  dfree(P->d_points);
  dfree(P->d_cv);
  dfree(P->d_enode);
  dfree(P->d_adj_ptr);
  dfree(P->d_adj);
  dfree(P->d_stab);
  dfree(P->d_hval);
  dfree(P->d_hgrad);
  dfree(P->d_ggrad);
  dfree(P->d_hw);
  dfree(P->d_hvalT);
  dfree(P->d_hgradT);
  dfree(P->d_tri);
  dfree(P->d_aff);
  dfree(P->d_sf);
  dfree(P->d_padj_ptr);
  dfree(P->d_padj);
  dfree(P->d_epart);
  dfree(P->d_npart);
  dfree(P->d_xpart);
  dfree(P->d_int);
  dfree(P->d_kqj);
  dfree(P->d_order);
  dfree(P->d_corder);
  dfree(P->d_elem);
  dfree(P->d_rowptr);
  dfree(P->d_colidx);
  dfree(P->d_vals);
  dfree(P->d_urowptr);
  dfree(P->d_uskip);
  dfree(P->d_uvals);
  dfree(P->d_nptr);
  dfree(P->d_ncol);
  dfree(P->d_nbits);
  dfree(P->d_slotmap);
  dfree(P->d_vec);
  dfree(P->d_pot);
  dfree(P->d_err);
  dfree(P->d_count);
  dfree(P->d_ncount);
  dfree(P->d_cub);
  for (int i = 0; i < GFGPU_MAX_SLOTS; ++i) dfree(P->slot_own[i]);
  for (int i = 0; i < 4; ++i)
    if (P->ev[i]) cudaEventDestroy(P->ev[i]);
  for (int c = 0; c < kHostChunks; ++c) {
    if (P->chunk_ev[c]) cudaEventDestroy(P->chunk_ev[c]);
    if (P->range_ev[c]) cudaEventDestroy(P->range_ev[c]);
  }
  for (cudaStream_t cs : P->copy_stream)
    if (cs) cudaStreamDestroy(cs);
  for (cudaStream_t gs : P->gather_stream)
    if (gs) cudaStreamDestroy(gs);
  delete P;
}

int gfgpu_set_data(gfgpu_plan *P, int32_t slot, const double *values, int64_t n,
                   int32_t on_device) {
  if (!P || slot < 0 || slot >= GFGPU_MAX_SLOTS || n < 0 || (n > 0 && !values)) {
    set_last_error("gfgpu_set_data: bad arguments");
    return GFGPU_E_INVALID;
  }
  if (on_device) {
    dfree(P->slot_own[slot]);
    P->slot_ptr[slot] = values;
    P->slot_n[slot] = n;
    return GFGPU_OK;
  }
  if (!P->slot_own[slot] || P->slot_n[slot] != n) {
    dfree(P->slot_own[slot]);
    int rc = dalloc(&P->slot_own[slot], size_t(n));
    if (rc) return rc;
  }
  P->slot_n[slot] = n;
  P->slot_ptr[slot] = P->slot_own[slot];
  if (n) GF_CUDA(cudaMemcpyAsync(P->slot_own[slot], values, size_t(n) * sizeof(double),
                                 cudaMemcpyHostToDevice, P->stream));
  return GFGPU_OK;
}

static int check_slots(Plan &P, bool need_u) {
  if (need_u && (!P.slot_ptr[GFGPU_SLOT_U] || P.slot_n[GFGPU_SLOT_U] != P.n_dof)) {
    set_last_error("variable u (slot 0) not set or of wrong size");
    return GFGPU_E_STATE;
  }
  if (P.ip_term >= 0) {
    const gfgpu_term &T = P.form.terms[P.ip_term];
    const int64_t n_int = P.n_elements * P.nq;
    if (!P.slot_ptr[T.field_slot] || P.slot_n[T.field_slot] != n_int) {
      set_last_error("internal variable slot not set or of wrong size (n_elements * nq)");
      return GFGPU_E_STATE;
    }
    if (P.cmode == 2 && (!P.slot_ptr[T.aux_slot] || P.slot_n[T.aux_slot] != n_int)) {
      set_last_error("condensation needs the internal residual (aux slot, n_elements * nq)");
      return GFGPU_E_STATE;
    }
  }
  for (int t = 0; t < P.form.n_terms; ++t) {
    const gfgpu_term &T = P.form.terms[t];
    for (int k = 0; k < 3; ++k)
    {
      if ((T.c[k].kind == GFGPU_COEF_ELEMENT || T.c[k].kind == GFGPU_COEF_NODAL) &&
          (T.c[k].slot < 0 || T.c[k].slot >= GFGPU_MAX_SLOTS)) {
        set_last_error("coefficient slot out of range");
        return GFGPU_E_INVALID;
      }
      if (T.c[k].kind == GFGPU_COEF_ELEMENT &&
          (!P.slot_ptr[T.c[k].slot] || P.slot_n[T.c[k].slot] != P.n_elements)) {
        set_last_error("per-element coefficient slot not set or of wrong size");
        return GFGPU_E_STATE;
      }
      if (T.c[k].kind == GFGPU_COEF_NODAL &&
          (!P.slot_ptr[T.c[k].slot] || P.slot_n[T.c[k].slot] != P.n_nodes)) {
        set_last_error("nodal coefficient slot not set or of wrong size");
        return GFGPU_E_STATE;
      }
    }
    if (T.kind == GFGPU_TERM_SOURCE &&
        (!P.slot_ptr[T.field_slot] || P.slot_n[T.field_slot] != P.n_dof)) {
      set_last_error("source field slot not set or of wrong size");
      return GFGPU_E_STATE;
    }
  }
  return GFGPU_OK;
}

int gfgpu_assemble(gfgpu_plan *P, int32_t order, int32_t flags, double *potential) {
  if (!P || order < 0 || order > 2) {
    set_last_error("gfgpu_assemble: bad arguments");
    return GFGPU_E_INVALID;
  }
  if (order == 0) {
    if (!P->kpot) {
      set_last_error("order 0 is not lowered for this element and form");
      return GFGPU_E_UNSUPPORTED;
    }
    int rc = check_slots(*P, true);
    if (rc) return rc;
    if (!P->d_epart && (rc = dalloc(&P->d_epart, size_t(P->n_elements)))) return rc;
    GF_CUDA(cudaMemsetAsync(P->d_err, 0, sizeof(int), P->stream));
    GF_CUDA(launch_potential(*P, P->d_pot));
    if (potential) {
      GF_CUDA(cudaMemcpyAsync(potential, P->d_pot, sizeof(double), cudaMemcpyDeviceToHost,
                              P->stream));
      return check_err(*P);
    }
    return GFGPU_OK;
  }
  if (!P->kmat) {
    set_last_error("orders 1 and 2 are not lowered for this element, integration method and form");
    return GFGPU_E_UNSUPPORTED;
  }
  if (int grc = check_geometry(*P)) return grc;
  const bool condense = (flags & GFGPU_CONDENSATION) != 0;
  if (condense && (P->ip_term < 0 || order != 2)) {
    set_last_error("GFGPU_CONDENSATION: order 2 of a form with an internal variable only");
    return GFGPU_E_INVALID;
  }
  if (P->ip_term >= 0 && order == 2 && !condense) {
    set_last_error("order 2 of a form with an internal variable is lowered with condensation only");
    return GFGPU_E_UNSUPPORTED;
  }
  P->cmode = P->ip_term < 0 ? 0 : (condense ? 2 : 1);
  P->sf_requested = (flags & GFGPU_SUM_FACTORISATION) != 0;
  const bool want_K = order == 2;
  // with condensation the vector is the condensed right-hand side
  const bool want_R = order == 1 || (flags & 2) || condense;
  int rc = check_slots(*P, want_R || P->law == LAW_NH);
  if (rc) return rc;
  if (P->ip_term >= 0) {
    const size_t n_int = size_t(P->n_elements) * P->nq;
    if (!P->d_int && (rc = dalloc(&P->d_int, n_int))) return rc;
    if (condense && !P->d_kqj && (rc = dalloc(&P->d_kqj, n_int * P->nb * P->qdim))) return rc;
  }
  // a pattern built without the condensed coupling may miss its entries
  const bool repattern = condense && P->nnz >= 0 && P->pattern_cmode != 2;
  // element scratch, allocated at the first order-1 or order-2 assembly
  if (!P->d_elem && (rc = dalloc(&P->d_elem, size_t(P->n_elements) * P->lay.stride))) return rc;
  const bool prof = (flags & GFGPU_PROFILE) != 0;
  if (prof && !P->ev[0])
    for (int i = 0; i < 4; ++i) GF_CUDA(cudaEventCreate(&P->ev[i]));
  GF_CUDA(cudaMemsetAsync(P->d_err, 0, sizeof(int), P->stream));
  if (prof) GF_CUDA(cudaEventRecord(P->ev[0], P->stream));
  // affine simplices with K stored: V_e holds the loads, and the row gather
  // adds K u from the node's assembled rows (nnz FMAs instead of K_e u_e in
  // the FP64-bound element pass)
  P->r_from_rows = P->affine_simplex && want_K;
  if (P->affine_simplex)
    GF_CUDA(launch_simplex_element_pass(*P, want_R, 0, -1, !P->r_from_rows));
  // the Gauss kernel skips the tangent and K_e when only the vector is
  // wanted and the pattern (which reads the K_e thresholds) exists
  else if (P->affine_hex) GF_CUDA(launch_affine_hex_pass(*P, want_K || P->nnz < 0));
  else GF_CUDA(launch_hex_element_pass(*P, want_K || P->nnz < 0));
  if (prof) GF_CUDA(cudaEventRecord(P->ev[1], P->stream));
  if ((want_K && (P->nnz < 0 || (flags & GFGPU_REBUILD_PATTERN) || repattern)) || P->nnz < 0) {
    // the pattern is built at the first order-2 assembly; an order-1
    // assembly needs the node-level part of it for its row walk
    if ((rc = build_pattern(*P))) return rc;
    P->pattern_cmode = P->cmode;
  }
  if (prof) GF_CUDA(cudaEventRecord(P->ev[2], P->stream));
  P->last_want_R = want_R;
  GF_CUDA(launch_gather(*P, want_K, want_R));
  if (prof) GF_CUDA(cudaEventRecord(P->ev[3], P->stream));
  P->profiled = prof;
  return GFGPU_OK;
}

int gfgpu_potential_gradient(gfgpu_plan *P, int32_t slot, double *grad, int64_t n,
                             int32_t on_device) {
  if (!P || !grad || (slot != GFGPU_SLOT_POINTS && (slot < 1 || slot >= GFGPU_MAX_SLOTS))) {
    set_last_error("gfgpu_potential_gradient: bad arguments");
    return GFGPU_E_INVALID;
  }
  if (!P->kpot) {
    set_last_error("order 0 is not lowered for this element and form");
    return GFGPU_E_UNSUPPORTED;
  }
  int rc = check_slots(*P, true);
  if (rc) return rc;
  // what the slot holds, from the form's coefficients
  int64_t need = 0;
  bool nodal = false;
  if (slot == GFGPU_SLOT_POINTS) {
    need = P->n_points * P->dim;
  } else {
    bool el = false, nd = false;
    for (int t = 0; t < P->form.n_terms; ++t)
      for (int k = 0; k < 3; ++k)
        if (P->form.terms[t].c[k].slot == slot) {
          el |= P->form.terms[t].c[k].kind == GFGPU_COEF_ELEMENT;
          nd |= P->form.terms[t].c[k].kind == GFGPU_COEF_NODAL;
        }
    if (el == nd) {
      set_last_error(el ? "slot used both as element and nodal coefficient"
                        : "slot is not a coefficient of the form");
      return GFGPU_E_INVALID;
    }
    nodal = nd;
    need = nodal ? P->n_nodes : P->n_elements;
  }
  if (n != need) {
    set_last_error("gfgpu_potential_gradient: gradient has " + std::to_string(need) + " entries");
    return GFGPU_E_INVALID;
  }
  if (!P->d_epart && (rc = dalloc(&P->d_epart, size_t(P->n_elements)))) return rc;
  double *dst = grad, *tmp = nullptr;
  if (!on_device) {
    if ((rc = dalloc(&tmp, size_t(need)))) return rc;
    dst = tmp;
  }
  GF_CUDA(cudaMemsetAsync(P->d_err, 0, sizeof(int), P->stream));
  cudaError_t ce;
  if (slot == GFGPU_SLOT_POINTS) {
    if (!P->d_xpart && (rc = dalloc(&P->d_xpart, size_t(P->n_elements) * P->nbg * P->dim))) {
      dfree(tmp);
      return rc;
    }
    ce = launch_shape_gradient(*P, dst);
  } else {
    if (nodal && !P->d_npart && (rc = dalloc(&P->d_npart, size_t(P->n_elements) * P->nb))) {
      dfree(tmp);
      return rc;
    }
    ce = launch_coef_gradient(*P, slot, nodal, dst);
  }
  if (ce == cudaSuccess && tmp)
    ce = cudaMemcpyAsync(grad, tmp, size_t(need) * sizeof(double), cudaMemcpyDeviceToHost,
                         P->stream);
  if (ce == cudaSuccess) ce = cudaStreamSynchronize(P->stream);
  dfree(tmp);
  if (ce != cudaSuccess) {
    set_last_error(std::string("gfgpu_potential_gradient: ") + cudaGetErrorString(ce));
    return GFGPU_E_CUDA;
  }
  return check_err(*P);
}

int gfgpu_set_points(gfgpu_plan *P, const double *points, int64_t n, int32_t on_device) {
  if (!P || !points || n != P->n_points * P->dim) {
    set_last_error("gfgpu_set_points: bad arguments");
    return GFGPU_E_INVALID;
  }
  GF_CUDA(cudaMemcpyAsync(P->d_points, points, size_t(n) * sizeof(double),
                          on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice,
                          P->stream));
  GF_CUDA(cudaStreamSynchronize(P->stream));
  if (P->kind == GFGPU_HEX) {
    // hexahedra: are the elements still parallelepipeds (constant Jacobian)?
    const double *hp = points;
    std::vector<double> tmp;
    if (on_device) {
      tmp.resize(size_t(n));
      GF_CUDA(cudaMemcpy(tmp.data(), points, size_t(n) * sizeof(double), cudaMemcpyDeviceToHost));
      hp = tmp.data();
    }
    P->parallelepiped = mesh_is_parallelepiped(hp, P->h_cvpts.data(), P->n_elements);
    P->axis_aligned =
        P->parallelepiped && mesh_is_axis_aligned(hp, P->h_cvpts.data(), P->n_elements);
  }
  return GFGPU_OK;
}

int gfgpu_batch_create(gfgpu_plan *const *plans, int32_t n, gfgpu_batch **out) {
  if (!plans || n < 1 || !out) {
    set_last_error("gfgpu_batch_create: bad arguments");
    return GFGPU_E_INVALID;
  }
  *out = nullptr;
  for (int i = 0; i < n; ++i)
    if (!plans[i]) {
      set_last_error("gfgpu_batch_create: null plan");
      return GFGPU_E_INVALID;
    }
  gfgpu_batch *B = new (std::nothrow) gfgpu_batch();
  if (!B) return GFGPU_E_NOMEM;
  auto fail = [&](int rc, const std::string &msg) {
    if (!msg.empty()) set_last_error(msg);
    gfgpu_batch_destroy(B);
    return rc;
  };
  std::vector<BatchItem> eitems[kBatchElementTypes];
  std::vector<int64_t> tile0[kBatchElementTypes];
  for (int t = 0; t < kBatchElementTypes; ++t) tile0[t].push_back(0);
  std::vector<BatchItem> gitems[4];
  std::vector<int64_t> node0[4];
  for (int q = 0; q < 4; ++q) node0[q].push_back(0);
  int rc;
  if ((rc = dalloc(&B->d_err, 1))) return fail(rc, "");
  if (cudaMemset(B->d_err, 0, sizeof(int)) != cudaSuccess)
    return fail(GFGPU_E_CUDA, "gfgpu_batch_create: cudaMemset failed");
  for (int i = 0; i < n; ++i) {
    Plan &P = *plans[i];
    if (!P.affine_simplex)
      return fail(GFGPU_E_UNSUPPORTED, "gfgpu_batch_create: batches take affine-simplex plans");
    if (form_has_tensor(P.form))
      return fail(GFGPU_E_UNSUPPORTED,
                  "gfgpu_batch_create: forms with an anisotropic coupling are not batched");
    if (P.nnz < 0)
      return fail(GFGPU_E_STATE, "gfgpu_batch_create: assemble each plan (order 2) first");
    if (!P.slot_ptr[GFGPU_SLOT_U] || P.slot_n[GFGPU_SLOT_U] != P.n_dof)
      return fail(GFGPU_E_STATE, "gfgpu_batch_create: variable u (slot 0) not set");
    if ((rc = check_slots(P, true))) return fail(rc, "");
    BatchItem it;
    bool mass;
    simplex_source_of(P, it.fsrc, it.fscale, mass);
    it.etype = simplex_batch_type(P.dim, P.degree, P.qdim, mass);
    it.qd = P.qdim;
    it.E = P.n_elements;
    it.n_nodes = P.n_nodes;
    it.pts = P.d_points;
    it.cv = P.d_cv;
    it.enode = P.d_enode;
    it.tab = P.d_stab;
    it.L = P.lay;
    it.form = P.form;
    for (int k = 0; k < GFGPU_MAX_SLOTS; ++k) it.slots.p[k] = P.slot_ptr[k];
    it.u = P.slot_ptr[GFGPU_SLOT_U];
    it.elem = P.d_elem;
    it.err = B->d_err;
    it.adj_ptr = P.d_adj_ptr;
    it.adj = P.d_adj;
    it.nptr = P.d_nptr;
    it.nbits = P.d_nbits;
    it.slotmap = P.d_slotmap;
    it.rowptr = P.d_rowptr;
    it.vals = P.d_vals;
    it.vec = P.d_vec;
    it.ncol = P.d_ncol;
    if (!it.ncol)
      return fail(GFGPU_E_STATE, "gfgpu_batch_create: the plan's node column lists are missing");
    if (it.etype < 0 || P.lay.s > 32)
      return fail(GFGPU_E_UNSUPPORTED, "gfgpu_batch_create: element not batched");
    eitems[it.etype].push_back(it);
    tile0[it.etype].push_back(tile0[it.etype].back() + (P.n_elements + 31) / 32);
    B->elements += P.n_elements;
    gitems[it.qd].push_back(it);
    node0[it.qd].push_back(node0[it.qd].back() + P.n_nodes);
    B->plans.push_back(plans[i]);
  }
  auto upload = [&](void *dst, const void *src, size_t bytes) -> int {
    GF_CUDA(cudaMemcpy(dst, src, bytes, cudaMemcpyHostToDevice));
    return GFGPU_OK;
  };
  for (int t = 0; t < kBatchElementTypes; ++t) {
    B->en[t] = int(eitems[t].size());
    B->entiles[t] = tile0[t].back();
    if (!B->en[t]) continue;
    if ((rc = dalloc(&B->d_eitems[t], eitems[t].size()))) return fail(rc, "");
    if ((rc = dalloc(&B->d_tile0[t], tile0[t].size()))) return fail(rc, "");
    if ((rc = upload(B->d_eitems[t], eitems[t].data(), eitems[t].size() * sizeof(BatchItem))))
      return fail(rc, "");
    if ((rc = upload(B->d_tile0[t], tile0[t].data(), tile0[t].size() * sizeof(int64_t))))
      return fail(rc, "");
  }
  for (int q = 1; q <= 3; ++q) {
    B->gn[q] = int(gitems[q].size());
    B->gnodes[q] = node0[q].back();
    if (!B->gn[q]) continue;
    if ((rc = dalloc(&B->d_gitems[q], gitems[q].size()))) return fail(rc, "");
    if ((rc = dalloc(&B->d_node0[q], node0[q].size()))) return fail(rc, "");
    if ((rc = upload(B->d_gitems[q], gitems[q].data(), gitems[q].size() * sizeof(BatchItem))))
      return fail(rc, "");
    if ((rc = upload(B->d_node0[q], node0[q].data(), node0[q].size() * sizeof(int64_t))))
      return fail(rc, "");
  }
  // the class lists: every node of every mesh by its own valence (class c:
  // at most 2^c adjacent elements), in mesh order, with the class maxima of
  // slots and adjacent elements
  for (int q = 1; q <= 3; ++q) {
    auto &cls = B->gclass[q];
    std::vector<std::vector<int64_t>> lists;
    for (size_t item = 0; item < gitems[q].size(); ++item) {
      const BatchItem &it = gitems[q][item];
      std::vector<int32_t> aptr(size_t(it.n_nodes + 1));
      std::vector<int64_t> nptr(size_t(it.n_nodes + 1));
      if ((rc = [&]() -> int {
            GF_CUDA(cudaMemcpy(aptr.data(), it.adj_ptr, aptr.size() * sizeof(int32_t),
                               cudaMemcpyDeviceToHost));
            GF_CUDA(cudaMemcpy(nptr.data(), it.nptr, nptr.size() * sizeof(int64_t),
                               cudaMemcpyDeviceToHost));
            return GFGPU_OK;
          }()))
        return fail(rc, "");
      for (int64_t node = 0; node < it.n_nodes; ++node) {
        const int mad = std::max(1, aptr[size_t(node + 1)] - aptr[size_t(node)]);
        const int ms = std::max<int64_t>(1, nptr[size_t(node + 1)] - nptr[size_t(node)]);
        int c = 0;
        while ((1 << c) < mad) ++c;
        if (cls.size() <= size_t(c)) {
          cls.resize(size_t(c) + 1);
          lists.resize(size_t(c) + 1);
        }
        cls[size_t(c)].ms = std::max(cls[size_t(c)].ms, ms);
        cls[size_t(c)].mad = std::max(cls[size_t(c)].mad, mad);
        lists[size_t(c)].push_back((int64_t(item) << 32) | node);
      }
    }
    for (size_t c = 0; c < cls.size(); ++c) {
      auto &k = cls[c];
      k.n = int64_t(lists[c].size());
      if (!k.n) continue;
      for (const BatchItem &it : gitems[q])
        k.wb = std::max(k.wb, batch_gather_class_bytes(it, k.ms, k.mad));
      B->gwarp[q] = std::max(B->gwarp[q], k.wb);
      if ((rc = dalloc(&k.d_list, lists[c].size()))) return fail(rc, "");
      if ((rc = upload(k.d_list, lists[c].data(), lists[c].size() * sizeof(int64_t))))
        return fail(rc, "");
    }
  }
  size_t gmax = 0;
  for (int q = 1; q <= 3; ++q) gmax = std::max(gmax, B->gwarp[q]);
  cudaError_t ce = batch_gather_attr(4 * gmax);
  if (ce != cudaSuccess)
    return fail(GFGPU_E_CUDA, std::string("gfgpu_batch_create: ") + cudaGetErrorString(ce));
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  B->grid_ep = 8 * std::max(sms, 1);
  for (int q = 1; q <= 3; ++q)
    for (const auto &k : B->gclass[q]) B->grid_ga += k.n > 0;
  *out = B;
  return GFGPU_OK;
}

static int batch_element_passes(gfgpu_batch *B, cudaStream_t st, int grid_ep) {
  for (int t = 0; t < kBatchElementTypes; ++t)
    if (B->en[t])
      GF_CUDA(launch_batch_element_pass(B->d_eitems[t], B->d_tile0[t], B->en[t], B->entiles[t],
                                        int(std::min<int64_t>(grid_ep, B->entiles[t])), t, st));
  return GFGPU_OK;
}

// the row gathers of a batch: one launch per component count and valence
// class
static int batch_gathers(gfgpu_batch *B, cudaStream_t st) {
  for (int q = 1; q <= 3; ++q)
    for (const auto &k : B->gclass[q])
      if (k.n)
        GF_CUDA(launch_batch_gather_list(B->d_gitems[q], k.d_list, k.n, q, k.ms, k.mad, k.wb, st));
  return GFGPU_OK;
}

static int batch_launch(gfgpu_batch *B, cudaStream_t st, int grid_ep) {
  // a fresh error word for this assembly (a memset node in a captured graph)
  GF_CUDA(cudaMemsetAsync(B->d_err, 0, sizeof(int), st));
  int rc = batch_element_passes(B, st, grid_ep);
  if (rc) return rc;
  return batch_gathers(B, st);
}

int gfgpu_batch_assemble(gfgpu_batch *B, void *stream) {
  if (!B) return GFGPU_E_INVALID;
  return batch_launch(B, static_cast<cudaStream_t>(stream), B->grid_ep);
}

int gfgpu_batch_tune(gfgpu_batch *B, void *stream, int32_t *grid_ep, int32_t *gather_launches) {
  if (!B) return GFGPU_E_INVALID;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  // the timing events, destroyed on every return
  struct Events {
    cudaEvent_t e[2] = {};
    ~Events() {
      for (cudaEvent_t x : e)
        if (x) cudaEventDestroy(x);
    }
  } ev;
  GF_CUDA(cudaEventCreate(&ev.e[0]));
  GF_CUDA(cudaEventCreate(&ev.e[1]));
  cudaEvent_t e0 = ev.e[0], e1 = ev.e[1];
  const int mult[] = {1, 2, 4, 8, 16, 32};
  float best_ep = 1e30f;
  for (int m : mult) {
    const int g = m * std::max(sms, 1);
    float t_ep = 0;
    for (int rep = 0; rep < 3; ++rep) {
      GF_CUDA(cudaEventRecord(e0, st));
      int rc = batch_element_passes(B, st, g);
      if (rc) return rc;
      GF_CUDA(cudaEventRecord(e1, st));
      GF_CUDA(cudaEventSynchronize(e1));
      float t;
      GF_CUDA(cudaEventElapsedTime(&t, e0, e1));
      t_ep = rep == 0 ? t : std::min(t_ep, t);
    }
    if (t_ep < best_ep) best_ep = t_ep, B->grid_ep = g;
  }
  // the gathers are one launch per component count and valence class
  int nga = 0;
  for (int q = 1; q <= 3; ++q)
    for (const auto &k : B->gclass[q]) nga += k.n > 0;
  B->grid_ga = nga;
  if (grid_ep) *grid_ep = B->grid_ep;
  if (gather_launches) *gather_launches = B->grid_ga;
  return GFGPU_OK;
}

int gfgpu_batch_sync(gfgpu_batch *B, void *stream) {
  if (!B) return GFGPU_E_INVALID;
  int herr = 0;
  GF_CUDA(cudaStreamSynchronize(static_cast<cudaStream_t>(stream)));
  GF_CUDA(cudaMemcpy(&herr, B->d_err, sizeof(int), cudaMemcpyDeviceToHost));
  return status_from_err(herr);
}

int64_t gfgpu_batch_elements(gfgpu_batch *B) { return B ? B->elements : -1; }

void gfgpu_batch_destroy(gfgpu_batch *B) {
  if (!B) return;
  for (int t = 0; t < kBatchElementTypes; ++t) {
    dfree(B->d_eitems[t]);
    dfree(B->d_tile0[t]);
  }
  for (int q = 0; q < 4; ++q) {
    dfree(B->d_gitems[q]);
    dfree(B->d_node0[q]);
    for (auto &k : B->gclass[q]) dfree(k.d_list);
  }
  dfree(B->d_err);
  delete B;
}

int gfgpu_sync(gfgpu_plan *P) {
  if (!P) return GFGPU_E_INVALID;
  return check_err(*P, true);
}

}  // extern "C"

namespace {

// the smallest element range of the chunked host-buffer assembly: one wave
// of the simplex pass's blocks (SMs x 6 resident blocks of 32 elements)
int64_t min_range_tiles() {
  static int64_t tiles = 0;
  if (!tiles) {
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
      sms = 132;
    tiles = int64_t(6) * sms;
  }
  return tiles;
}

// Launches made while it lives go to stream s instead of the plan's stream.
struct StreamScope {
  Plan &P;
  cudaStream_t saved;
  StreamScope(Plan &p, cudaStream_t s) : P(p), saved(p.stream) { P.stream = s; }
  ~StreamScope() { P.stream = saved; }
};

// The host-buffer assembly of gfgpu_assemble_host (upper = false: the full
// CSR values) and gfgpu_assemble_host_upper (upper = true: the values of
// the entries with column >= row, in the order of gfgpu_pattern_upper).

int assemble_host(gfgpu_plan *P, const double *u, double *vals, double *vec, bool upper) {
  int rc;
  if (u && (rc = gfgpu_set_data(P, GFGPU_SLOT_U, u, P->n_dof, 0))) return rc;
  if (P->nnz < 0 || !vals || !P->kmat || P->h_rowptr.empty()) {
    // first assembly (the pattern is built) or no matrix wanted
    if ((rc = gfgpu_assemble(P, 2, vec ? GFGPU_WITH_VECTOR : 0, nullptr))) return rc;
    if (vals && !upper)
      GF_CUDA(cudaMemcpyAsync(vals, P->d_vals, size_t(P->nnz) * sizeof(double),
                              cudaMemcpyDeviceToHost, P->stream));
    if (vec) GF_CUDA(cudaMemcpyAsync(vec, P->d_vec, size_t(P->n_dof) * sizeof(double),
                                     cudaMemcpyDeviceToHost, P->stream));
    if ((rc = check_err(*P))) return rc;
    if (!vals || !upper) return GFGPU_OK;
    // the upper values of the first call: the gather once more in upper mode
    if ((rc = build_upper(*P))) return rc;
    P->upper_out = true;
    cudaError_t ce = launch_gather(*P, true, false);
    P->upper_out = false;
    GF_CUDA(ce);
    GF_CUDA(cudaMemcpyAsync(vals, P->d_uvals, size_t(P->nnz_upper) * sizeof(double),
                            cudaMemcpyDeviceToHost, P->stream));
    return check_err(*P);
  }
  if ((rc = check_slots(*P, true))) return rc;
  if ((rc = check_geometry(*P))) return rc;
  if (upper && (rc = build_upper(*P))) return rc;
  const std::vector<int64_t> &hptr = upper ? P->h_urowptr : P->h_rowptr;
  double *dvals = upper ? P->d_uvals : P->d_vals;
  // The element pass, then the row gather in chunks of DOF nodes; the rows
  // of each chunk (contiguous in the CSR) are copied to the host while the
  // next chunks are gathered.  (Writing the values from the gather straight
  // into page-locked host memory was 2.5x slower: its stores are 8-byte
  // scattered.)
  if (!P->copy_stream[0]) {
    // two copy streams (two copy engines), chunks alternating between them;
    // gather streams at the device's highest priority
    int prio_lo = 0, prio_hi = 0;
    GF_CUDA(cudaDeviceGetStreamPriorityRange(&prio_lo, &prio_hi));
    GF_CUDA(cudaStreamCreateWithFlags(&P->copy_stream[0], cudaStreamNonBlocking));
    GF_CUDA(cudaStreamCreateWithFlags(&P->copy_stream[1], cudaStreamNonBlocking));
    for (cudaStream_t &gs : P->gather_stream)
      GF_CUDA(cudaStreamCreateWithPriority(&gs, cudaStreamNonBlocking, prio_hi));
    for (int c = 0; c < kHostChunks; ++c) {
      GF_CUDA(cudaEventCreateWithFlags(&P->chunk_ev[c], cudaEventDisableTiming));
      GF_CUDA(cudaEventCreateWithFlags(&P->range_ev[c], cudaEventDisableTiming));
    }
  }
  GF_CUDA(cudaMemsetAsync(P->d_err, 0, sizeof(int), P->stream));
  // Affine simplices: the element pass runs on the plan's stream in element
  // ranges, each far enough for the next gather chunk (h_chunk_eend).  Chunk
  // c's gather waits for its range and runs on gather stream c % 3: the
  // gathers' blocks take SMs ahead of the element pass's (priority), so the
  // copies of the first chunks start early, and the three streams fill each
  // other's launch tails.  Every chunk writes its own rows: the results do
  // not depend on the order the streams run in.
  int64_t tiles_done = 0;
  P->r_from_rows = P->affine_simplex;
  if (P->affine_hex) GF_CUDA(launch_affine_hex_pass(*P, true));
  else if (!P->affine_simplex) GF_CUDA(launch_hex_element_pass(*P, true));
  const int qd = P->qdim;
  P->upper_out = upper;
  for (int c = 0; c < kHostChunks; ++c) {
    const int64_t n0 = P->n_nodes * c / kHostChunks, n1 = P->n_nodes * (c + 1) / kHostChunks;
    if (P->affine_simplex) {
      const int64_t ntiles = (P->n_elements + 31) / 32;
      const int64_t need = c == kHostChunks - 1 ? ntiles : (P->h_chunk_eend[c] + 31) / 32;
      // each range launch covers at least min_range_tiles() tiles (a range
      // of less than a wave leaves SMs idle), so it may run ahead of the
      // next chunks' needs
      if (need > tiles_done) {
        const int64_t upto = std::min(ntiles, std::max(need, tiles_done + min_range_tiles()));
        cudaError_t ce = launch_simplex_element_pass(*P, true, tiles_done, upto, false);
        if (ce != cudaSuccess) P->upper_out = false;
        GF_CUDA(ce);
        tiles_done = upto;
      }
    }
    cudaStream_t gs = P->gather_stream[c % kGatherStreams];
    GF_CUDA(cudaEventRecord(P->range_ev[c], P->stream));
    GF_CUDA(cudaStreamWaitEvent(gs, P->range_ev[c], 0));
    cudaError_t ce;
    {
      StreamScope on_gs(*P, gs);
      ce = launch_gather_chunk(*P, vec != nullptr, c);
    }
    if (ce != cudaSuccess) P->upper_out = false;
    GF_CUDA(ce);
    cudaStream_t cs = P->copy_stream[c & 1];
    GF_CUDA(cudaEventRecord(P->chunk_ev[c], gs));
    GF_CUDA(cudaStreamWaitEvent(cs, P->chunk_ev[c], 0));
    const int64_t r0 = hptr[size_t(n0 * qd)], r1 = hptr[size_t(n1 * qd)];
    if (r1 > r0)
      GF_CUDA(cudaMemcpyAsync(vals + r0, dvals + r0, size_t(r1 - r0) * sizeof(double),
                              cudaMemcpyDeviceToHost, cs));
    if (vec && n1 > n0)
      GF_CUDA(cudaMemcpyAsync(vec + n0 * qd, P->d_vec + n0 * qd,
                              size_t((n1 - n0) * qd) * sizeof(double), cudaMemcpyDeviceToHost,
                              cs));
  }
  P->upper_out = false;
  // later work on the plan's stream follows every gather
  for (int c = kHostChunks - kGatherStreams; c < kHostChunks; ++c)
    GF_CUDA(cudaStreamWaitEvent(P->stream, P->chunk_ev[c], 0));
  GF_CUDA(cudaStreamSynchronize(P->copy_stream[0]));
  GF_CUDA(cudaStreamSynchronize(P->copy_stream[1]));
  P->last_want_R = vec != nullptr;
  const int64_t nnz0 = P->nnz, builds0 = P->pattern_builds;
  int rc2 = check_err(*P, true);
  if (rc2 != GFGPU_OK || P->pattern_builds == builds0) return rc2;
  if (P->nnz != nnz0) {
    // the pattern grew: the caller's buffer is sized for the old one
    set_last_error("the CSR pattern grew (entries that were zero at the pattern build are "
                   "nonzero now): read gfgpu_pattern_size / the new pattern and call again");
    return GFGPU_E_STATE;
  }
  if (vals && !upper) {
    // rebuilt with the same size: copy the repaired values again
    GF_CUDA(cudaMemcpy(vals, P->d_vals, size_t(P->nnz) * sizeof(double),
                       cudaMemcpyDeviceToHost));
  } else if (vals) {
    // the repair gathered the full CSR: the upper values once more
    if ((rc = build_upper(*P))) return rc;
    P->upper_out = true;
    cudaError_t ce = launch_gather(*P, true, false);
    P->upper_out = false;
    GF_CUDA(ce);
    GF_CUDA(cudaMemcpyAsync(vals, P->d_uvals, size_t(P->nnz_upper) * sizeof(double),
                            cudaMemcpyDeviceToHost, P->stream));
    if ((rc = check_err(*P))) return rc;
  }
  if (vec) GF_CUDA(cudaMemcpy(vec, P->d_vec, size_t(P->n_dof) * sizeof(double),
                              cudaMemcpyDeviceToHost));
  return rc2;
}

}  // namespace

extern "C" {

int gfgpu_assemble_host(gfgpu_plan *P, const double *u, double *vals, double *vec) {
  if (!P) return GFGPU_E_INVALID;
  return assemble_host(P, u, vals, vec, false);
}

int gfgpu_assemble_host_upper(gfgpu_plan *P, const double *u, double *upper_vals, double *vec) {
  if (!P) return GFGPU_E_INVALID;
  if (!P->symmetric) {
    set_last_error("gfgpu_assemble_host_upper: the form's matrix is not symmetric");
    return GFGPU_E_UNSUPPORTED;
  }
  return assemble_host(P, u, upper_vals, vec, true);
}

int gfgpu_pattern_upper(gfgpu_plan *P, int64_t *nnz_upper, int64_t *rowptr, int32_t *colidx) {
  if (!P || !nnz_upper) return GFGPU_E_INVALID;
  if (P->nnz < 0) {
    set_last_error("no pattern yet: assemble order 2 first");
    return GFGPU_E_STATE;
  }
  int rc;
  if ((rc = build_upper(*P))) return rc;
  *nnz_upper = P->nnz_upper;
  if (rowptr) std::copy(P->h_urowptr.begin(), P->h_urowptr.end(), rowptr);
  if (colidx && P->nnz_upper > 0) {
    int32_t *d_ucol = nullptr;
    if ((rc = dalloc(&d_ucol, size_t(P->nnz_upper)))) return rc;
    cudaError_t ce = launch_upper_fill(*P, d_ucol);
    if (ce == cudaSuccess)
      ce = cudaMemcpyAsync(colidx, d_ucol, size_t(P->nnz_upper) * sizeof(int32_t),
                           cudaMemcpyDeviceToHost, P->stream);
    if (ce == cudaSuccess) ce = cudaStreamSynchronize(P->stream);
    dfree(d_ucol);
    GF_CUDA(ce);
  }
  return GFGPU_OK;
}

int gfgpu_pattern_size(gfgpu_plan *P, int64_t *n_rows, int64_t *nnz) {
  if (!P) return GFGPU_E_INVALID;
  if (P->nnz < 0) {
    set_last_error("no pattern yet: assemble order 2 first");
    return GFGPU_E_STATE;
  }
  *n_rows = P->n_dof;
  *nnz = P->nnz;
  return GFGPU_OK;
}

int gfgpu_pattern_copy(gfgpu_plan *P, int64_t *rowptr, int32_t *colidx) {
  if (!P) return GFGPU_E_INVALID;
  if (P->nnz < 0) {
    set_last_error("no pattern yet: assemble order 2 first");
    return GFGPU_E_STATE;
  }
  GF_CUDA(cudaStreamSynchronize(P->stream));
  if (rowptr) GF_CUDA(cudaMemcpy(rowptr, P->d_rowptr, size_t(P->n_dof + 1) * sizeof(int64_t),
                                 cudaMemcpyDeviceToHost));
  if (colidx) GF_CUDA(cudaMemcpy(colidx, P->d_colidx, size_t(P->nnz) * sizeof(int32_t),
                                 cudaMemcpyDeviceToHost));
  return GFGPU_OK;
}

int gfgpu_device_csr(gfgpu_plan *P, const int64_t **rowptr, const int32_t **colidx,
                     double **vals) {
  if (!P) return GFGPU_E_INVALID;
  if (P->nnz < 0) {
    set_last_error("no pattern yet: assemble order 2 first");
    return GFGPU_E_STATE;
  }
  if (rowptr) *rowptr = P->d_rowptr;
  if (colidx) *colidx = P->d_colidx;
  if (vals) *vals = P->d_vals;
  return GFGPU_OK;
}

int gfgpu_device_vector(gfgpu_plan *P, double **vec) {
  if (!P || !vec) return GFGPU_E_INVALID;
  *vec = P->d_vec;
  return GFGPU_OK;
}

int64_t gfgpu_launch_count(gfgpu_plan *P) { return P ? P->launches : -1; }

int gfgpu_get_launch(gfgpu_plan *P, gfgpu_launch *l) {
  if (!P || !l) return GFGPU_E_INVALID;
  l->ep_threads = P->tune.ep_threads;
  l->gather_warps = P->tune.gather_warps;
  return GFGPU_OK;
}

int gfgpu_set_launch(gfgpu_plan *P, const gfgpu_launch *l) {
  if (!P || !l) return GFGPU_E_INVALID;
  const auto eps = ep_candidates(*P);
  const bool ep_ok = std::find(eps.begin(), eps.end(), l->ep_threads) != eps.end();
  const bool gw_ok = l->gather_warps == 2 || l->gather_warps == 4 || l->gather_warps == 8;
  if (!ep_ok || !gw_ok) {
    set_last_error("gfgpu_set_launch: ep_threads " + std::to_string(l->ep_threads) +
                   " / gather_warps " + std::to_string(l->gather_warps) +
                   " is not a candidate of this plan's kernels");
    return GFGPU_E_INVALID;
  }
  P->tune.ep_threads = l->ep_threads;
  P->tune.gather_warps = l->gather_warps;
  return GFGPU_OK;
}

int gfgpu_tune(gfgpu_plan *P, int32_t reps, gfgpu_launch *best) {
  if (!P || reps < 1) return GFGPU_E_INVALID;
  if (!P->kmat) {
    set_last_error("gfgpu_tune: the plan has no element-matrix kernel");
    return GFGPU_E_UNSUPPORTED;
  }
  int rc;
  const int flags = GFGPU_WITH_VECTOR | (P->ip_term >= 0 ? GFGPU_CONDENSATION : 0);
  if (P->nnz < 0 && (rc = gfgpu_assemble(P, 2, flags, nullptr))) return rc;
  if ((rc = check_err(*P, true))) return rc;
  // median over reps of the element-pass (w = 0) or gather (w = 1) time
  auto time_of = [&](int w, float &med) -> int {
    std::vector<float> t;
    for (int r = 0; r <= reps; ++r) {  // the first run warms up
      int rc2 = gfgpu_assemble(P, 2, flags | GFGPU_PROFILE, nullptr);
      if (rc2) return rc2;
      float k[2];
      if ((rc2 = gfgpu_kernel_times(P, k, 2))) return rc2;
      if (r) t.push_back(k[w]);
    }
    if ((rc = check_err(*P, true))) return rc;
    std::sort(t.begin(), t.end());
    med = t[t.size() / 2];
    return GFGPU_OK;
  };
  float bt = 0.0f;
  int be = P->tune.ep_threads;
  for (int ep : ep_candidates(*P)) {
    P->tune.ep_threads = ep;
    float m;
    if ((rc = time_of(0, m))) return rc;
    if (ep == ep_candidates(*P)[0] || m < bt) bt = m, be = ep;
  }
  P->tune.ep_threads = be;
  int bg = P->tune.gather_warps;
  for (int gw : {2, 4, 8}) {
    P->tune.gather_warps = gw;
    float m;
    if ((rc = time_of(1, m))) return rc;
    if (gw == 2 || m < bt) bt = m, bg = gw;
  }
  P->tune.gather_warps = bg;
  {
    std::lock_guard<std::mutex> lock(g_tune_mutex);
    g_tuned[family_key(*P)] = P->tune;
  }
  if (best) {
    best->ep_threads = P->tune.ep_threads;
    best->gather_warps = P->tune.gather_warps;
  }
  return GFGPU_OK;
}

int gfgpu_tune_save(const char *path) {
  if (!path) return GFGPU_E_INVALID;
  std::lock_guard<std::mutex> lock(g_tune_mutex);
  FILE *f = std::fopen(path, "w");
  if (!f) {
    set_last_error(std::string("gfgpu_tune_save: cannot write ") + path);
    return GFGPU_E_INVALID;
  }
  for (const auto &kv : g_tuned)
    std::fprintf(f, "%s %d %d\n", kv.first.c_str(), kv.second.ep_threads, kv.second.gather_warps);
  std::fclose(f);
  return GFGPU_OK;
}

int gfgpu_tune_load(const char *path) {
  if (!path) return GFGPU_E_INVALID;
  FILE *f = std::fopen(path, "r");
  if (!f) {
    set_last_error(std::string("gfgpu_tune_load: cannot read ") + path);
    return GFGPU_E_INVALID;
  }
  std::map<std::string, LaunchConfig> got;
  char key[512];
  int ep = 0, gw = 0, n = 0;
  while ((n = std::fscanf(f, "%511s %d %d", key, &ep, &gw)) == 3) {
    const bool ok = (ep == 2 || ep == 4 || ep == 8 || ep == 128 || ep == 256 || ep == 512) &&
                    (gw == 2 || gw == 4 || gw == 8);
    if (!ok) {
      std::fclose(f);
      set_last_error(std::string("gfgpu_tune_load: bad configuration for ") + key);
      return GFGPU_E_INVALID;
    }
    LaunchConfig c;
    c.ep_threads = ep;
    c.gather_warps = gw;
    got[key] = c;
  }
  const bool bad = n != EOF;
  std::fclose(f);
  if (bad) {
    set_last_error(std::string("gfgpu_tune_load: malformed line in ") + path);
    return GFGPU_E_INVALID;
  }
  std::lock_guard<std::mutex> lock(g_tune_mutex);
  for (const auto &kv : got) g_tuned[kv.first] = kv.second;
  return GFGPU_OK;
}

int gfgpu_kernel_times(gfgpu_plan *P, float *times, int32_t n) {
  if (!P || !times || n < 2) return GFGPU_E_INVALID;
  if (!P->profiled) {
    set_last_error("last assembly was not profiled (GFGPU_PROFILE)");
    return GFGPU_E_STATE;
  }
  GF_CUDA(cudaEventSynchronize(P->ev[3]));
  GF_CUDA(cudaEventElapsedTime(&times[0], P->ev[0], P->ev[1]));
  GF_CUDA(cudaEventElapsedTime(&times[1], P->ev[2], P->ev[3]));
  return GFGPU_OK;
}

int gfgpu_internal_size(gfgpu_plan *P, int64_t *n_int, int64_t *row_len) {
  if (!P || !n_int || !row_len) {
    set_last_error("gfgpu_internal_size: bad arguments");
    return GFGPU_E_INVALID;
  }
  const bool has = P->ip_term >= 0;
  *n_int = has ? P->n_elements * P->nq : 0;
  *row_len = has ? int64_t(P->nb) * P->qdim : 0;
  return GFGPU_OK;
}

int gfgpu_copy_result(gfgpu_plan *P, int32_t which, void *dst) {
  if (!P || !dst || which < 0 || which > GFGPU_RESULT_COUPLING_COLIDX) {
    set_last_error("gfgpu_copy_result: bad arguments");
    return GFGPU_E_INVALID;
  }
  if (which >= GFGPU_RESULT_INTERNAL) {
    const size_t n_int = size_t(P->n_elements) * P->nq, row = size_t(P->nb) * P->qdim;
    if (P->ip_term < 0 || !P->d_int || (which != GFGPU_RESULT_INTERNAL && !P->d_kqj)) {
      set_last_error("no internal-variable result: assemble a form with an internal variable "
                     "(order 1, or order 2 with GFGPU_CONDENSATION for the coupling)");
      return GFGPU_E_STATE;
    }
    if (which == GFGPU_RESULT_COUPLING_COLIDX) {
      // the element's DOFs in local order, once per Gauss point
      std::vector<int32_t> cols(n_int * row);
      const int nb = P->nb, qd = P->qdim, nq = P->nq;
      for (int64_t e = 0; e < P->n_elements; ++e)
        for (int q = 0; q < nq; ++q) {
          int32_t *c = cols.data() + (size_t(e) * nq + q) * row;
          for (int j = 0; j < nb; ++j)
            for (int b = 0; b < qd; ++b) c[j * qd + b] = P->h_en[size_t(e) * nb + j] * qd + b;
        }
      GF_CUDA(cudaMemcpy(dst, cols.data(), cols.size() * sizeof(int32_t), cudaMemcpyDefault));
      return GFGPU_OK;
    }
    const double *src = which == GFGPU_RESULT_INTERNAL ? P->d_int : P->d_kqj;
    const size_t bytes = (which == GFGPU_RESULT_INTERNAL ? n_int : n_int * row) * sizeof(double);
    GF_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDefault, P->stream));
    return check_err(*P);
  }
  if (which != GFGPU_RESULT_VECTOR && P->nnz < 0) {
    set_last_error("no pattern yet: assemble order 2 first");
    return GFGPU_E_STATE;
  }
  // the last assembly must be complete (and its pattern repaired) first
  int rc = check_err(*P, true);
  if (rc) return rc;
  const void *src = nullptr;
  size_t bytes = 0;
  switch (which) {
    case GFGPU_RESULT_ROWPTR: src = P->d_rowptr, bytes = size_t(P->n_dof + 1) * 8; break;
    case GFGPU_RESULT_COLIDX: src = P->d_colidx, bytes = size_t(P->nnz) * 4; break;
    case GFGPU_RESULT_VALUES: src = P->d_vals, bytes = size_t(P->nnz) * 8; break;
    default: src = P->d_vec, bytes = size_t(P->n_dof) * 8; break;
  }
  if (bytes) GF_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDefault, P->stream));
  return check_err(*P);
}

}  // extern "C"
