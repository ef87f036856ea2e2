// DOF enumeration on the device: mesh_fem::enumerate_dof
// (getfem_mesh_fem.cc:320-460) for Lagrange FEM_PK / FEM_QK, numbering the
// nodes in the order of their first encounter (elements in order, local
// nodes in order) with qdim consecutive DOFs per node.
//
// A node is identified by its support: the vertices of the element with a
// nonzero barycentric (PK) or tensor-product (QK) integer weight, with the
// weights.  Nodes with at most 4 support vertices (all PK nodes in 2-D and
// 3-D, QK nodes on vertices, edges and faces) get a 128-bit key of 4 sorted
// (vertex id: 25 bits, weight: 7 bits) words; a QK node interior to its cell
// belongs to that cell alone and gets a key made of its (element, local
// node) index.  Sorting the keys (stable radix sorts), marking the first key
// of each run of equal keys and ranking the runs by their smallest (element,
// local node) index gives the reference's numbering.
#include <cub/cub.cuh>

#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include "host/refelem.h"
#include "k_common.cuh"
#include "plan.h"

namespace gfgpu {
void set_last_error(const std::string &s);
}

using namespace gfgpu;

namespace {

constexpr int kMaxNbDofs = 125;
constexpr uint64_t kInterior = ~0ull;

struct NodeSupport {
  int8_t n[kMaxNbDofs];           // support size (> 4: interior)
  int8_t v[kMaxNbDofs][4];        // local vertices
  int8_t w[kMaxNbDofs][4];        // weights
};

__global__ void make_keys(int64_t E, int nb, int nv, const int64_t *__restrict__ cv,
                          const NodeSupport *__restrict__ sup, uint64_t *__restrict__ hi,
                          uint64_t *__restrict__ lo, uint32_t *__restrict__ idx) {
  const int64_t t = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  if (t >= E * nb) return;
  const int64_t e = t / nb;
  const int i = int(t % nb);
  idx[t] = uint32_t(t);
  const int n = sup->n[i];
  if (n > 4) {
    hi[t] = kInterior;
    lo[t] = uint64_t(t);
    return;
  }
  uint32_t vid[4], wt[4];
  for (int k = 0; k < n; ++k) {
    vid[k] = uint32_t(cv[e * nv + sup->v[i][k]]);
    wt[k] = uint32_t(sup->w[i][k]);
  }
  for (int a = 1; a < n; ++a) {  // insertion sort by vertex id
    const uint32_t x = vid[a], y = wt[a];
    int b = a - 1;
    while (b >= 0 && vid[b] > x) {
      vid[b + 1] = vid[b];
      wt[b + 1] = wt[b];
      --b;
    }
    vid[b + 1] = x;
    wt[b + 1] = y;
  }
  uint32_t word[4];
  for (int k = 0; k < 4; ++k) word[k] = k < n ? ((vid[k] << 7) | wt[k]) : 0xffffffffu;
  hi[t] = (uint64_t(word[0]) << 32) | word[1];
  lo[t] = (uint64_t(word[2]) << 32) | word[3];
}

__global__ void gather_u64(int64_t n, const uint64_t *__restrict__ src,
                           const uint32_t *__restrict__ perm, uint64_t *__restrict__ dst) {
  const int64_t t = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  if (t < n) dst[t] = src[perm[t]];
}

__global__ void run_heads(int64_t n, const uint64_t *__restrict__ hi,
                          const uint64_t *__restrict__ lo, uint32_t *__restrict__ head) {
  const int64_t t = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  if (t >= n) return;
  head[t] = (t == 0 || hi[t] != hi[t - 1] || lo[t] != lo[t - 1]) ? 1u : 0u;
}

// runs are numbered by the inclusive scan of the heads (1-based); the first
// index of run r is the (element, local node) index at its head
__global__ void run_first(int64_t n, const uint32_t *__restrict__ head,
                          const uint32_t *__restrict__ runid, const uint32_t *__restrict__ idx,
                          uint32_t *__restrict__ first, uint32_t *__restrict__ rid) {
  const int64_t t = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  if (t >= n || !head[t]) return;
  const uint32_t r = runid[t] - 1;
  first[r] = idx[t];
  rid[r] = r;
}

__global__ void rank_of_run(int64_t nr, const uint32_t *__restrict__ rid_sorted,
                            uint32_t *__restrict__ rank) {
  const int64_t t = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  if (t < nr) rank[rid_sorted[t]] = uint32_t(t);
}

__global__ void assign_dofs(int64_t n, int qdim, const uint32_t *__restrict__ runid,
                            const uint32_t *__restrict__ idx, const uint32_t *__restrict__ rank,
                            int64_t *__restrict__ dofs) {
  const int64_t t = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  if (t < n) dofs[idx[t]] = int64_t(rank[runid[t] - 1]) * qdim;
}

template <class T>
struct DevArr {
  T *p = nullptr;
  ~DevArr() {
    if (p) cudaFree(p);
  }
  cudaError_t alloc(size_t n) { return cudaMalloc(&p, (n ? n : 1) * sizeof(T)); }
};

}  // namespace

extern "C" int gfgpu_device_available(void) {
  int n = 0;
  return cudaGetDeviceCount(&n) == cudaSuccess && n > 0 ? 1 : 0;
}

extern "C" int gfgpu_enumerate_dofs_device(int32_t dim, int32_t kind, int32_t degree, int32_t qdim,
                                           int64_t n_elements, const int64_t *cvpts,
                                           int64_t *dofs, int64_t *n_dof) {
  if (dim < 2 || dim > 3 || (kind != GFGPU_SIMPLEX && kind != GFGPU_HEX) || degree < 1 ||
      qdim < 1 || n_elements < 0 || (n_elements > 0 && (!cvpts || !dofs)) || !n_dof) {
    set_last_error("gfgpu_enumerate_dofs_device: bad arguments");
    return GFGPU_E_INVALID;
  }
  RefElement fe(dim, kind, degree);
  const int nb = fe.nb, nv = kind == GFGPU_SIMPLEX ? dim + 1 : (1 << dim);
  const int64_t n = n_elements * nb;
  if (nb > kMaxNbDofs || n >= (int64_t(1) << 32) || degree > 4) {
    set_last_error("gfgpu_enumerate_dofs_device: element or mesh too large for the device keys");
    return GFGPU_E_UNSUPPORTED;
  }
  // support of each local node
  NodeSupport sup;
  std::memset(&sup, 0, sizeof(sup));
  for (int i = 0; i < nb; ++i) {
    const int *c = &fe.lattice[i * dim];
    int cnt = 0;
    auto add = [&](int v, int w) {
      if (cnt < 4) sup.v[i][cnt] = int8_t(v), sup.w[i][cnt] = int8_t(w);
      ++cnt;
    };
    if (kind == GFGPU_SIMPLEX) {
      int w0 = degree;
      for (int d = 0; d < dim; ++d) w0 -= c[d];
      if (w0) add(0, w0);
      for (int d = 0; d < dim; ++d)
        if (c[d]) add(d + 1, c[d]);
    } else {
      for (int p = 0; p < nv; ++p) {
        int w = 1;
        for (int d = 0; d < dim; ++d) w *= ((p >> d) & 1) ? c[d] : (degree - c[d]);
        if (w) add(p, w);
      }
    }
    sup.n[i] = int8_t(cnt > 4 ? 8 : cnt);
  }
  int64_t maxv = 0;
  for (int64_t k = 0; k < n_elements * nv; ++k) maxv = cvpts[k] > maxv ? cvpts[k] : maxv;
  if (maxv >= (int64_t(1) << 25)) {
    set_last_error("gfgpu_enumerate_dofs_device: more than 2^25 mesh vertices");
    return GFGPU_E_UNSUPPORTED;
  }
  if (n == 0) {
    *n_dof = 0;
    return GFGPU_OK;
  }
  cudaStream_t st = nullptr;
  DevArr<int64_t> d_cv, d_dofs;
  DevArr<NodeSupport> d_sup;
  DevArr<uint64_t> hi, lo, k1, k2;
  DevArr<uint32_t> idx, idx1, idx2, head, runid, first, rid, first_s, rid_s, rank;
  DevArr<unsigned char> tmp;
  cudaError_t ce = cudaSuccess;
#define DC(x) \
  if (ce == cudaSuccess) ce = (x)
  DC(d_cv.alloc(size_t(n_elements) * nv));
  DC(d_dofs.alloc(size_t(n)));
  DC(d_sup.alloc(1));
  for (auto *a : {&hi, &lo, &k1, &k2}) DC(a->alloc(size_t(n)));
  for (auto *a : {&idx, &idx1, &idx2, &head, &runid, &first, &rid, &first_s, &rid_s, &rank})
    DC(a->alloc(size_t(n)));
  size_t tb = 0, tb2 = 0;
  DC(cub::DeviceRadixSort::SortPairs(nullptr, tb, lo.p, k1.p, idx.p, idx1.p, n));
  DC(cub::DeviceScan::InclusiveSum(nullptr, tb2, head.p, runid.p, n));
  tb = std::max(tb, tb2);
  DC(tmp.alloc(tb));
  DC(cudaMemcpyAsync(d_cv.p, cvpts, size_t(n_elements) * nv * sizeof(int64_t),
                     cudaMemcpyHostToDevice, st));
  DC(cudaMemcpyAsync(d_sup.p, &sup, sizeof(sup), cudaMemcpyHostToDevice, st));
  const unsigned g = unsigned((n + 255) / 256);
  if (ce == cudaSuccess) {
    make_keys<<<g, 256, 0, st>>>(n_elements, nb, nv, d_cv.p, d_sup.p, hi.p, lo.p, idx.p);
    ce = cudaGetLastError();
  }
  // stable LSD: by lo, then by hi
  DC(cub::DeviceRadixSort::SortPairs(tmp.p, tb, lo.p, k1.p, idx.p, idx1.p, n, 0, 64, st));
  if (ce == cudaSuccess) gather_u64<<<g, 256, 0, st>>>(n, hi.p, idx1.p, k2.p);
  DC(cub::DeviceRadixSort::SortPairs(tmp.p, tb, k2.p, k1.p, idx1.p, idx2.p, n, 0, 64, st));
  // k1: sorted hi; k2: lo in the same order
  if (ce == cudaSuccess) gather_u64<<<g, 256, 0, st>>>(n, lo.p, idx2.p, k2.p);
  if (ce == cudaSuccess) run_heads<<<g, 256, 0, st>>>(n, k1.p, k2.p, head.p);
  DC(cub::DeviceScan::InclusiveSum(tmp.p, tb, head.p, runid.p, n, st));
  uint32_t nruns = 0;
  DC(cudaMemcpyAsync(&nruns, runid.p + (n - 1), sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
  DC(cudaStreamSynchronize(st));
  if (ce == cudaSuccess) run_first<<<g, 256, 0, st>>>(n, head.p, runid.p, idx2.p, first.p, rid.p);
  // runs ordered by their first (element, local node) index
  DC(cub::DeviceRadixSort::SortPairs(tmp.p, tb, first.p, first_s.p, rid.p, rid_s.p,
                                     int64_t(nruns), 0, 32, st));
  const unsigned gr = unsigned((nruns + 255) / 256);
  if (ce == cudaSuccess && nruns) rank_of_run<<<gr, 256, 0, st>>>(nruns, rid_s.p, rank.p);
  if (ce == cudaSuccess)
    assign_dofs<<<g, 256, 0, st>>>(n, qdim, runid.p, idx2.p, rank.p, d_dofs.p);
  DC(cudaGetLastError());
  DC(cudaMemcpyAsync(dofs, d_dofs.p, size_t(n) * sizeof(int64_t), cudaMemcpyDeviceToHost, st));
  DC(cudaStreamSynchronize(st));
#undef DC
  if (ce != cudaSuccess) {
    set_last_error(std::string("gfgpu_enumerate_dofs_device: ") + cudaGetErrorString(ce));
    return ce == cudaErrorMemoryAllocation ? GFGPU_E_NOMEM : GFGPU_E_CUDA;
  }
  *n_dof = int64_t(nruns) * qdim;
  return GFGPU_OK;
}
