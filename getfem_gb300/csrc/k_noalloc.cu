// Vector assembly without any device allocation (gfgpu_assemble_vector_noalloc).
//
// Some callers cannot allocate device memory: code that runs inside a
// memory budget owned by another allocator (a framework's caching allocator,
// a fixed arena sized at start-up, an embedded solver handed a fixed pool)
// must not call cudaMalloc behind that allocator's back.  This entry point
// assembles the vector of an affine-simplex form from the caller's device
// arrays into the caller's device output, with its scratch (the element
// vectors) and its reference tables in file-scope static device arrays of
// fixed size.  It does wait for its stream once per call, to read the
// device error word (a non-invertible Jacobian, a non-finite value or an
// adjacency entry out of range) and return it as the status.
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "k_common.cuh"
#include "plan.h"

namespace gfgpu {
void set_last_error(const std::string &s);
}

using namespace gfgpu;

namespace {

constexpr size_t kScratchDoubles = GFGPU_NOALLOC_SCRATCH_BYTES / sizeof(double);

// Scratch shared by every call on a device: element vectors, `vstride`
// doubles per element.  Each call overwrites the slots of all its elements
// before reading them, so nothing has to start at zero.
static __device__ __align__(256) double g_scratch[kScratchDoubles];
static __device__ SimplexTables g_tables;
static __device__ int g_err;

constexpr int kMaxDevices = 64;
struct DeviceSymbols {
  bool ready = false;
  double *scratch = nullptr;
  SimplexTables *tables = nullptr;
  int *err = nullptr;
};
DeviceSymbols g_dev[kMaxDevices];
std::mutex g_mutex;

// Device addresses of the static arrays, looked up once per device with that
// device current (the host-side names are stand-ins, not device addresses).
int device_symbols(DeviceSymbols *&out) {
  int dev = 0;
  cudaError_t ce = cudaGetDevice(&dev);
  if (ce != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
    set_last_error("gfgpu_assemble_vector_noalloc: no current CUDA device");
    return GFGPU_E_CUDA;
  }
  std::lock_guard<std::mutex> lock(g_mutex);
  DeviceSymbols &d = g_dev[dev];
  if (!d.ready) {
    if ((ce = cudaGetSymbolAddress(reinterpret_cast<void **>(&d.scratch), g_scratch)) != cudaSuccess ||
        (ce = cudaGetSymbolAddress(reinterpret_cast<void **>(&d.tables), g_tables)) != cudaSuccess ||
        (ce = cudaGetSymbolAddress(reinterpret_cast<void **>(&d.err), g_err)) != cudaSuccess) {
      set_last_error(std::string("gfgpu_assemble_vector_noalloc: cudaGetSymbolAddress: ") +
                     cudaGetErrorString(ce));
      return GFGPU_E_CUDA;
    }
    d.ready = true;
  }
  out = &d;
  return GFGPU_OK;
}

// R[(i,a)] = sum over the elements e of node i (ascending e, local node li)
// of V_e[li*qd + a]: deterministic, no atomics.
// An adjacency entry outside [0, n_elements*nb) is skipped and flagged
// (ERR_CAPACITY): the adjacency is the caller's data.
__global__ void node_sum(int64_t n_nodes, int qd, int nb, int64_t n_codes,
                         const int32_t *__restrict__ adj_ptr, const int32_t *__restrict__ adj,
                         const double *__restrict__ v, int vstride, double *__restrict__ out,
                         int *__restrict__ err) {
  const int64_t t = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  if (t >= n_nodes * qd) return;
  const int64_t node = t / qd;
  const int a = int(t % qd);
  double r = 0.0;
  for (int k = adj_ptr[node]; k < adj_ptr[node + 1]; ++k) {
    const int code = adj[k];
    if (code < 0 || code >= n_codes) {
      set_err(err, ERR_CAPACITY);
      continue;
    }
    r += v[int64_t(code / nb) * vstride + (code % nb) * qd + a];
  }
  if (!isfinite(r)) set_err(err, ERR_NAN);
  out[t] = r;
}

}  // namespace

extern "C" int gfgpu_assemble_vector_noalloc(const gfgpu_noalloc_args *A, const gfgpu_form *form,
                                             void *cuda_stream) {
  // Every pointer the kernels dereference is checked here, so that a
  // caller's mistake is a status, not a fault on the device.
  if (!A || !form || A->dim < 2 || A->dim > 3 || A->degree < 1 || A->degree > 2 ||
      (A->qdim != 1 && A->qdim != A->dim) || A->n_elements < 0 || A->n_nodes < 0 || !A->im ||
      (A->n_elements > 0 && (!A->points || !A->cvpts || !A->enode)) ||
      (A->n_nodes > 0 && (!A->adj_ptr || !A->adj || !A->vec))) {
    set_last_error("gfgpu_assemble_vector_noalloc: bad arguments");
    return GFGPU_E_INVALID;
  }
  if (form->n_terms < 1 || form->n_terms > GFGPU_MAX_TERMS) {
    set_last_error("gfgpu_assemble_vector_noalloc: form has " + std::to_string(form->n_terms) +
                   " terms (1 to GFGPU_MAX_TERMS allowed)");
    return GFGPU_E_INVALID;
  }
  SimplexTables tab;
  KeLayout lay;
  int nq = 0;
  std::string why;
  int rc = fill_simplex_tables(A->dim, A->degree, A->qdim, A->im, tab, lay, nq, why);
  if (rc) {
    set_last_error("gfgpu_assemble_vector_noalloc: " + why);
    return rc;
  }
  const int vstride = lay.rowstride;  // V_e rounded up to 4 doubles
  if (double(A->n_elements) * vstride > double(kScratchDoubles)) {
    set_last_error("gfgpu_assemble_vector_noalloc: " + std::to_string(A->n_elements) +
                   " elements need " + std::to_string(A->n_elements * vstride * 8) +
                   " bytes of scratch; the maximum is GFGPU_NOALLOC_SCRATCH_BYTES = " +
                   std::to_string(GFGPU_NOALLOC_SCRATCH_BYTES));
    return GFGPU_E_INVALID;
  }
  if (!simplex_form_supported(*form, A->qdim, A->dim, why)) {
    set_last_error("gfgpu_assemble_vector_noalloc: form not lowered on simplices: " + why);
    return GFGPU_E_UNSUPPORTED;
  }
  if (form_has_tensor(*form)) {
    set_last_error("gfgpu_assemble_vector_noalloc: anisotropic couplings need a plan");
    return GFGPU_E_UNSUPPORTED;
  }
  // data slots the element pass reads: u, every per-element coefficient,
  // the load field of a source term
  const bool has_elements = A->n_elements > 0;
  if (has_elements && !A->slots[GFGPU_SLOT_U]) {
    set_last_error("gfgpu_assemble_vector_noalloc: variable u (slot 0) missing");
    return GFGPU_E_INVALID;
  }
  for (int t = 0; t < form->n_terms && has_elements; ++t) {
    const gfgpu_term &T = form->terms[t];
    for (int k = 0; k < 3; ++k)
      if (T.c[k].kind == GFGPU_COEF_ELEMENT &&
          (T.c[k].slot < 0 || T.c[k].slot >= GFGPU_MAX_SLOTS || !A->slots[T.c[k].slot])) {
        set_last_error("gfgpu_assemble_vector_noalloc: per-element coefficient slot " +
                       std::to_string(T.c[k].slot) + " out of range or missing");
        return GFGPU_E_INVALID;
      }
    if (T.kind == GFGPU_TERM_SOURCE && !A->slots[T.field_slot]) {
      set_last_error("gfgpu_assemble_vector_noalloc: source field slot " +
                     std::to_string(T.field_slot) + " missing");
      return GFGPU_E_INVALID;
    }
  }
  DeviceSymbols *d = nullptr;
  if ((rc = device_symbols(d))) return rc;
  cudaStream_t st = static_cast<cudaStream_t>(cuda_stream);
  cudaError_t ce;
  // tables and error word: copies into the static arrays, no allocation
  if ((ce = cudaMemcpyToSymbolAsync(g_tables, &tab, sizeof(tab), 0, cudaMemcpyHostToDevice, st)) !=
          cudaSuccess ||
      (ce = cudaMemsetAsync(d->err, 0, sizeof(int), st)) != cudaSuccess) {
    set_last_error(std::string("gfgpu_assemble_vector_noalloc: ") + cudaGetErrorString(ce));
    return GFGPU_E_CUDA;
  }
  if (has_elements) {
    ce = launch_simplex_vector_pass(A->dim, A->degree, A->qdim, A->n_elements, A->points,
                                    A->cvpts, A->enode, d->tables, *form, A->slots, d->scratch,
                                    vstride, d->err, st);
    if (ce == cudaSuccess && A->n_nodes > 0) {
      const int64_t n = A->n_nodes * A->qdim;
      node_sum<<<unsigned((n + 255) / 256), 256, 0, st>>>(A->n_nodes, A->qdim, lay.nb,
                                                          A->n_elements * lay.nb, A->adj_ptr,
                                                          A->adj, d->scratch, vstride, A->vec,
                                                          d->err);
      ce = cudaGetLastError();
    }
  } else if (A->n_nodes > 0) {
    // no element contributes: the vector is zero (the adjacency is not read)
    ce = cudaMemsetAsync(A->vec, 0, size_t(A->n_nodes) * A->qdim * sizeof(double), st);
  }
  int herr = 0;
  if (ce == cudaSuccess) ce = cudaMemcpyAsync(&herr, d->err, sizeof(int), cudaMemcpyDeviceToHost, st);
  if (ce == cudaSuccess) ce = cudaStreamSynchronize(st);
  if (ce != cudaSuccess) {
    set_last_error(std::string("gfgpu_assemble_vector_noalloc: ") + cudaGetErrorString(ce));
    return GFGPU_E_CUDA;
  }
  if (herr & ERR_JACOBIAN) {
    set_last_error("Non invertible matrix (det of the geometric transformation is 0)");
    return GFGPU_E_JACOBIAN;
  }
  if (herr & ERR_NAN) {
    set_last_error("non-finite value in assembly");
    return GFGPU_E_NAN;
  }
  if (herr & ERR_CAPACITY) {
    set_last_error("gfgpu_assemble_vector_noalloc: adjacency entry outside [0, n_elements*nb)");
    return GFGPU_E_INVALID;
  }
  return GFGPU_OK;
}
