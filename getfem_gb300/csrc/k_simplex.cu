// Affine-simplex element pass (sm_103a, FP64).
//
// GetFEM's exec loop (getfem_generic_assembly_compile_and_exec.cc:8750-8869)
// recomputes, at every Gauss point q of every element, the geometric
// transformation (J, B), the real base gradients grad_ref . B^T and the
// contraction, and accumulates elem += J w_q t_q.  On an affine simplex B
// and J are constant, so the Gauss-point sum factors through a small
// per-element tensor and a fixed reference tensor (the idea of
// getfem_mat_elem.cc:433 for linear geotrans):
//
//   elem[(i,a),(j,b)] = sum_{v,w} G[i,j,v,w] T[(a,v),(b,w)] + cm M[i,j] d_ab
//   T[(a,v),(b,w)] = |J| (c0 g_va g_wb + c1 d_ab g_v.g_w + c2 g_vb g_wa
//                         + ct sum_{k,l} D[(a,k),(b,l)] g_vk g_wl)
//
// (the last part for a constant anisotropic coupling D, GRADGRAD_TENSOR)
// with g_v the real gradients of the barycentric coordinates and
// G[i,j,v,w] = sum_q w_q c_iv(x_q) c_jw(x_q) (grad phi_i = sum_v c_iv
// grad lambda_v) computed with the element's own quadrature rule, so the
// result is the reference's Gauss-point sum in exact arithmetic.  G is
// sparse: c_iv = 0 unless vertex v carries weight in node i.
//
// A block of 4 warps handles 32 elements (lane = element in every warp).
// FP64 is the bound on this part, and an FP64 warp instruction occupies the
// SM's FP64 pipe for many cycles whatever the number of active lanes, so
// control flow is uniform within each warp: warp 0 computes the geometry,
// all warps fill T (symmetric: upper triangle, in shared memory), and warp w
// builds rows w, w+4, ... of the element matrices.  Rows of the element matrix are
// built in registers and stored with 32-byte vector stores, so every DRAM
// sector is written whole.  The pass also writes the element's whole
// contribution to the assembled vector, V = K_e u_e + scale |J| M f (no
// threshold, as the reference's vector assembly), and the drop threshold
// 1e-14 max|elem| over all entries (compile_and_exec.cc:5453) into the
// element scratch read by the row gather.
#include "k_simplex_tile.cuh"

namespace gfgpu {

// ---------------------------------------------------------------- host

// Sparse barycentric reference tensor of FEM_PK(dim, degree) for the
// quadrature rule `im`, the reference mass matrix, and the element scratch
// layout.
int fill_simplex_tables(int dim, int K, int qdim, const std::string &im, SimplexTables &t,
                        KeLayout &lay, int &nq, std::string &errmsg) {
  RefElement fe(dim, SIMPLEX, K);
  Quadrature q;
  if (!quadrature_by_name(im, q) || q.dim != dim) {
    errmsg = "unsupported integration method " + im;
    return GFGPU_E_UNSUPPORTED;
  }
  if (fe.nb > kMaxNb || K > 2) {
    errmsg = "simplex element pass supports degree <= 2";
    return GFGPU_E_UNSUPPORTED;
  }
  const int nb = fe.nb, nv = dim + 1;
  std::memset(&t, 0, sizeof(t));
  t.nb = nb;
  t.nv = nv;
  t.dim = dim;
  // c_iv(x) = d phi_i / d lambda_v for phi_i = prod_v P_{w_v}(lambda_v)
  auto factor = [&](int w, double lam, double &f, double &df) {
    f = 1.0;
    df = 0.0;
    for (int j = 0; j < w; ++j) {
      double a = (K * lam - j) / (j + 1), da = double(K) / (j + 1);
      df = df * a + f * da;
      f *= a;
    }
  };
  std::vector<double> cvals(size_t(q.nq) * nb * nv), phi(size_t(q.nq) * nb);
  std::vector<int> w(size_t(nb) * nv);
  for (int i = 0; i < nb; ++i) {
    int s = 0;
    for (int d = 0; d < dim; ++d) w[i * nv + d + 1] = fe.lattice[i * dim + d], s += fe.lattice[i * dim + d];
    w[i * nv] = K - s;
  }
  std::vector<double> val(nb), grad(size_t(nb) * dim);
  for (int qq = 0; qq < q.nq; ++qq) {
    double lam[4];
    lam[0] = 1.0;
    for (int d = 0; d < dim; ++d) lam[d + 1] = q.pts[qq * dim + d], lam[0] -= lam[d + 1];
    fe.eval(&q.pts[qq * dim], val.data(), grad.data());
    for (int i = 0; i < nb; ++i) {
      double f[4], df[4];
      for (int v = 0; v < nv; ++v) factor(w[i * nv + v], lam[v], f[v], df[v]);
      phi[qq * nb + i] = val[i];  // the reference's tabulated base values
      for (int v = 0; v < nv; ++v) {
        double c = df[v];
        for (int u = 0; u < nv; ++u)
          if (u != v) c *= f[u];
        cvals[(size_t(qq) * nb + i) * nv + v] = c;
      }
    }
  }
  for (int i = 0; i < nb; ++i)
    for (int j = 0; j < nb; ++j) {
      int pij = i * nb + j, n = 0;
      for (int v = 0; v < nv; ++v) {
        if (w[i * nv + v] == 0) continue;
        for (int u = 0; u < nv; ++u) {
          if (w[j * nv + u] == 0) continue;
          double s = 0;
          for (int qq = 0; qq < q.nq; ++qq)
            s += q.w[qq] * cvals[(size_t(qq) * nb + i) * nv + v] * cvals[(size_t(qq) * nb + j) * nv + u];
          if (n >= kMaxPairTerms) {
            errmsg = "internal: too many reference tensor terms";
            return GFGPU_E_UNSUPPORTED;
          }
          t.vw[pij * kMaxPairTerms + n] = int8_t(v * nv + u);
          t.gval[pij * kMaxPairTerms + n] = s;
          ++n;
        }
      }
      t.nterm[pij] = int8_t(n);
      // the kernels unroll the terms from the compile-time node supports
      const int ni = pk_sup_n(dim, nb, i), nj = pk_sup_n(dim, nb, j);
      bool same = n == ni * nj;
      for (int ti = 0; same && ti < ni; ++ti)
        for (int tj = 0; tj < nj; ++tj)
          same = same && t.vw[pij * kMaxPairTerms + ti * nj + tj] ==
                             int8_t(pk_sup_v(dim, nb, i, ti) * nv + pk_sup_v(dim, nb, j, tj));
      if (!same) {
        errmsg = "internal: node supports differ from the element's lattice";
        return GFGPU_E_UNSUPPORTED;
      }
      double m = 0;
      for (int qq = 0; qq < q.nq; ++qq) m += q.w[qq] * phi[qq * nb + i] * phi[qq * nb + j];
      t.mass[pij] = m;
    }
  nq = q.nq;
  const int qd = qdim, s = nb * qd;
  lay.nb = nb;
  lay.qd = qd;
  lay.s = s;
  // rows padded to a multiple of 4 doubles (scalar fields), or node blocks
  // of 4 / 12 doubles (vector fields): whole 32-byte sectors either way
  lay.rowstride = (s + 3) & ~3;
  lay.blk = qd == 1 ? 0 : (qd == 2 ? 4 : 12);
  lay.rowblk = qd == 1 ? lay.rowstride : nb * lay.blk;
  lay.off_vec = qd == 1 ? s * lay.rowstride : (nb * (nb + 1) / 2) * lay.blk;
  lay.off_thr = lay.off_vec + lay.rowstride;
  lay.stride = lay.off_thr + 4;
  lay.linear = true;
  return GFGPU_OK;
}

// ---------------------------------------------------------------- batched

namespace {

// the element-pass instances of the batched launch, (dim, degree, qdim, mass)
constexpr int kBatchTypes = 16;

template <int T>
struct BatchType;
#define GFGPU_BT(T, D, Q, N, MS)                        \
  template <>                                           \
  struct BatchType<T> {                                 \
    static constexpr int DIM = D, QD = Q, NB = N;       \
    static constexpr bool MASS = MS;                    \
  };
GFGPU_BT(0, 2, 1, 3, false) GFGPU_BT(1, 2, 1, 6, false) GFGPU_BT(2, 2, 2, 3, false)
GFGPU_BT(3, 2, 2, 6, false) GFGPU_BT(4, 3, 1, 4, false) GFGPU_BT(5, 3, 1, 10, false)
GFGPU_BT(6, 3, 3, 4, false) GFGPU_BT(7, 3, 3, 10, false) GFGPU_BT(8, 2, 1, 3, true)
GFGPU_BT(9, 2, 1, 6, true) GFGPU_BT(10, 2, 2, 3, true) GFGPU_BT(11, 2, 2, 6, true)
GFGPU_BT(12, 3, 1, 4, true) GFGPU_BT(13, 3, 1, 10, true) GFGPU_BT(14, 3, 3, 4, true)
GFGPU_BT(15, 3, 3, 10, true)
#undef GFGPU_BT

// Persistent element pass over the tiles of the meshes of one element type
// in a batch: block b takes tiles b, b + grid, ...; the mesh of a tile is
// found by binary search in the tile offsets.  One launch per element type
// keeps each type's own register and shared-memory footprint.
template <int T>
__global__ void __launch_bounds__(kEpThreads) batch_element_pass(
    const BatchItem *__restrict__ items, const int64_t *__restrict__ tile0, int nitems,
    int64_t ntiles) {
  using B = BatchType<T>;
  __shared__ EpShared<B::DIM, B::QD, B::NB, false> sh;
  for (int64_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
    int lo = 0, hi = nitems - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (tile0[mid] <= t) lo = mid;
      else hi = mid - 1;
    }
    const BatchItem &it = items[lo];
    __syncthreads();  // the previous tile is done with the shared memory
    // K u is formed by the batched gather from the assembled rows
    simplex_element_tile<B::DIM, B::QD, B::NB, B::MASS, true, false>(
        sh, t - tile0[lo], it.E, it.pts, it.cv, it.enode, it.tab, it.L, it.form, it.slots,
        it.fsrc, it.fscale, it.u, it.elem, it.err);
  }
}

}  // namespace

int simplex_batch_type(int dim, int degree, int qdim, bool mass) {
  int base;
  if (dim == 2) base = (qdim == 1 ? 0 : 2) + (degree == 1 ? 0 : 1);
  else base = 4 + (qdim == 1 ? 0 : 2) + (degree == 1 ? 0 : 1);
  if (degree < 1 || degree > 2 || (qdim != 1 && qdim != dim)) return -1;
  return base + (mass ? 8 : 0);
}

void simplex_source_of(const Plan &P, const double *&fsrc, double &fscale, bool &mass) {
  fsrc = nullptr;
  fscale = 0.0;
  mass = false;
  for (int t = 0; t < P.form.n_terms; ++t) {
    const gfgpu_term &T = P.form.terms[t];
    if (T.kind == GFGPU_TERM_SOURCE) {
      fsrc = P.slot_ptr[T.field_slot];
      fscale = T.scale * (T.c[0].kind == GFGPU_COEF_CONST ? T.c[0].value : 1.0);
    }
    if (T.kind == GFGPU_TERM_MASS) mass = true;
  }
}

cudaError_t launch_batch_element_pass(const BatchItem *items, const int64_t *tile0, int nitems,
                                     int64_t ntiles, int grid, int etype, cudaStream_t st) {
  if (ntiles == 0) return cudaSuccess;
  switch (etype) {
#define GFGPU_BL(T)                                                                  \
  case T:                                                                            \
    batch_element_pass<T><<<grid, kEpThreads, 0, st>>>(items, tile0, nitems, ntiles); \
    break;
    GFGPU_BL(0) GFGPU_BL(1) GFGPU_BL(2) GFGPU_BL(3) GFGPU_BL(4) GFGPU_BL(5) GFGPU_BL(6)
    GFGPU_BL(7) GFGPU_BL(8) GFGPU_BL(9) GFGPU_BL(10) GFGPU_BL(11) GFGPU_BL(12) GFGPU_BL(13)
    GFGPU_BL(14) GFGPU_BL(15)
#undef GFGPU_BL
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

int build_simplex_tables(Plan &P, std::string &errmsg) {
  return fill_simplex_tables(P.dim, P.degree, P.qdim, P.im, P.stab, P.lay, P.nq, errmsg);
}

cudaError_t launch_simplex_element_pass(Plan &P, bool with_u, int64_t tile0, int64_t tile1,
                                        bool ku) {
  if (form_has_tensor(P.form)) return launch_simplex_element_pass_tensor(P, with_u, tile0, tile1, ku);
  if (P.n_elements == 0) return cudaSuccess;
  const int64_t ntiles = (P.n_elements + 31) / 32;  // 32 elements per block
  if (tile1 < 0 || tile1 > ntiles) tile1 = ntiles;
  if (tile1 <= tile0) return cudaSuccess;
  const unsigned blocks = unsigned(tile1 - tile0);
  SlotPtrs sp;
  for (int i = 0; i < GFGPU_MAX_SLOTS; ++i) sp.p[i] = P.slot_ptr[i];
  const double *fsrc = nullptr;
  double fscale = 0.0;
  bool mass = false;
  for (int t = 0; t < P.form.n_terms; ++t) {
    const gfgpu_term &T = P.form.terms[t];
    if (T.kind == GFGPU_TERM_SOURCE) {
      fsrc = P.slot_ptr[T.field_slot];
      fscale = T.scale * (T.c[0].kind == GFGPU_COEF_CONST ? T.c[0].value : 1.0);
    }
    if (T.kind == GFGPU_TERM_MASS) mass = true;
  }
#define GFGPU_EP1(D, Q, N, MS, KUV, WV)                                                        \
  simplex_element_pass<D, Q, N, MS, true, KUV, WV><<<blocks, 32 * WV, 0, P.stream>>>(          \
      P.n_elements, P.d_points, P.d_cv, P.d_enode, P.d_stab, P.lay, P.form, sp, fsrc, fscale,   \
      with_u ? P.slot_ptr[GFGPU_SLOT_U] : nullptr, P.d_elem, P.d_err, tile0)
  // the K pass runs with the plan's threads per element (autotuned); a KU
  // pass with the default
  const int w = ku ? kEpWarps : P.tune.ep_threads;
#define GFGPU_EPW(D, Q, N, MS)                                                                 \
  do {                                                                                         \
    if (w == 2) GFGPU_EP1(D, Q, N, MS, false, 2);                                              \
    else if (w == 8) GFGPU_EP1(D, Q, N, MS, false, 8);                                         \
    else GFGPU_EP1(D, Q, N, MS, false, 4);                                                     \
  } while (0)
#define GFGPU_EP(D, Q, N)                                                                      \
  do {                                                                                         \
    if (mass && ku) GFGPU_EP1(D, Q, N, true, true, 4);                                         \
    else if (mass) GFGPU_EPW(D, Q, N, true);                                                   \
    else if (ku) GFGPU_EP1(D, Q, N, false, true, 4);                                           \
    else GFGPU_EPW(D, Q, N, false);                                                            \
  } while (0)
  const int d = P.dim, k = P.degree, q = P.qdim;
  if (d == 2 && k == 1 && q == 1) GFGPU_EP(2, 1, 3);
  else if (d == 2 && k == 2 && q == 1) GFGPU_EP(2, 1, 6);
  else if (d == 2 && k == 1 && q == 2) GFGPU_EP(2, 2, 3);
  else if (d == 2 && k == 2 && q == 2) GFGPU_EP(2, 2, 6);
  else if (d == 3 && k == 1 && q == 1) GFGPU_EP(3, 1, 4);
  else if (d == 3 && k == 2 && q == 1) GFGPU_EP(3, 1, 10);
  else if (d == 3 && k == 1 && q == 3) GFGPU_EP(3, 3, 4);
  else if (d == 3 && k == 2 && q == 3) GFGPU_EP(3, 3, 10);
  else return cudaErrorInvalidValue;
#undef GFGPU_EP
#undef GFGPU_EPW
#undef GFGPU_EP1
  P.launches++;
  return cudaGetLastError();
}

// The element pass storing only the element vectors V_e = K_e u_e + load
// (layout: V_e at offset 0, `vstride` doubles per element), for callers that
// assemble the vector alone.
cudaError_t launch_simplex_vector_pass(int dim, int degree, int qdim, int64_t E,
                                       const double *pts, const int32_t *cv, const int32_t *enode,
                                       const SimplexTables *tab, const gfgpu_form &form,
                                       const double *const *slot, double *vout, int vstride,
                                       int *err, cudaStream_t stream) {
  if (E == 0) return cudaSuccess;
  KeLayout L;
  L.qd = qdim;
  L.off_vec = 0;
  L.off_thr = 0;
  L.stride = vstride;
  SlotPtrs sp;
  for (int i = 0; i < GFGPU_MAX_SLOTS; ++i) sp.p[i] = slot[i];
  const double *fsrc = nullptr;
  double fscale = 0.0;
  bool mass = false;
  for (int t = 0; t < form.n_terms; ++t) {
    const gfgpu_term &T = form.terms[t];
    if (T.kind == GFGPU_TERM_SOURCE) {
      fsrc = slot[T.field_slot];
      fscale = T.scale * (T.c[0].kind == GFGPU_COEF_CONST ? T.c[0].value : 1.0);
    }
    if (T.kind == GFGPU_TERM_MASS) mass = true;
  }
  const unsigned blocks = unsigned((E + 31) / 32);
#define GFGPU_VP(D, Q, N)                                                                       \
  do {                                                                                          \
    if (mass)                                                                                   \
      simplex_element_pass<D, Q, N, true, false, true><<<blocks, kEpThreads, 0, stream>>>(      \
          E, pts, cv, enode, tab, L, form, sp, fsrc, fscale, slot[GFGPU_SLOT_U], vout, err, 0); \
    else                                                                                        \
      simplex_element_pass<D, Q, N, false, false, true><<<blocks, kEpThreads, 0, stream>>>(     \
          E, pts, cv, enode, tab, L, form, sp, fsrc, fscale, slot[GFGPU_SLOT_U], vout, err, 0); \
  } while (0)
  const int d = dim, k = degree, q = qdim;
  if (d == 2 && k == 1 && q == 1) GFGPU_VP(2, 1, 3);
  else if (d == 2 && k == 2 && q == 1) GFGPU_VP(2, 1, 6);
  else if (d == 2 && k == 1 && q == 2) GFGPU_VP(2, 2, 3);
  else if (d == 2 && k == 2 && q == 2) GFGPU_VP(2, 2, 6);
  else if (d == 3 && k == 1 && q == 1) GFGPU_VP(3, 1, 4);
  else if (d == 3 && k == 2 && q == 1) GFGPU_VP(3, 1, 10);
  else if (d == 3 && k == 1 && q == 3) GFGPU_VP(3, 3, 4);
  else if (d == 3 && k == 2 && q == 3) GFGPU_VP(3, 3, 10);
  else return cudaErrorInvalidValue;
#undef GFGPU_VP
  return cudaGetLastError();
}

}  // namespace gfgpu
