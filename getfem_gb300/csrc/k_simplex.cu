// Affine-simplex assembly kernels (sm_103a, FP64).
//
// GetFEM's exec loop (getfem_generic_assembly_compile_and_exec.cc:8750-8869)
// recomputes, at every Gauss point q of every element, the geometric
// transformation (J, B), the real base gradients grad_ref . B^T and the
// contraction, accumulates elem += J w_q t_q and inserts elem into the sparse
// matrix.  On an affine simplex B and J are constant, so the Gauss-point sum
// factors through a small per-element tensor and a fixed reference tensor
// (the idea of getfem_mat_elem.cc:433 for linear geotrans):
//
//   elem[(i,a),(j,b)] = sum_{v,w} G[i,j,v,w] T_e[a,b,v,w] + cm_e M[i,j] d_ab
//   T_e[a,b,v,w] = |J| (c0 g_va g_wb + c1 d_ab g_v.g_w + c2 g_vb g_wa)
//
// with g_v the real gradients of the barycentric coordinates and
// G[i,j,v,w] = sum_q w_q c_iv(x_q) c_jw(x_q) (grad phi_i = sum_v c_iv
// grad lambda_v), computed with the element's own quadrature rule, so the
// result is the reference's Gauss-point sum in exact arithmetic.
//
// Pass 1 (element pass): one thread per element writes T_e, cm_e, |J| and
// the drop threshold 1e-14 max|elem| (compile_and_exec.cc:5453).
// Pass 2 (row gather): one warp per DOF node walks the node's elements in
// element order, expands the contributions of its rows, drops those with
// |e| <= threshold (compile_and_exec.cc:4889) and writes the CSR row values
// and the residual.  No atomics: every K entry is summed in element order,
// as the reference's column merge sums it.
// The sparsity pattern is built by the same warp-per-node walk.
#include <cub/cub.cuh>

#include <cmath>
#include <cstdio>

#include "host/refelem.h"
#include "plan.h"

namespace gfgpu {

namespace {

constexpr int kWarp = 32;
constexpr int kMaxLocal = 128;  // local nodes per element held in shared memory

__device__ __forceinline__ void set_err(int *err, int bit) { atomicOr(err, bit); }

// --------------------------------------------------------- element pass

template <int DIM, int QD>
__global__ void __launch_bounds__(128) simplex_element_pass(
    int64_t E, const double *__restrict__ pts, const int32_t *__restrict__ cv,
    const SimplexTables *__restrict__ tab, SimplexLayout lay, gfgpu_form form,
    SlotPtrs slots, bool psd_hint, double *__restrict__ out,
    int *__restrict__ err) {
  constexpr int NV = DIM + 1;
  int64_t e = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  if (e >= E) return;
  double x[NV][DIM];
#pragma unroll
  for (int v = 0; v < NV; ++v) {
    int p = __ldg(cv + e * NV + v);
#pragma unroll
    for (int d = 0; d < DIM; ++d) x[v][d] = __ldg(pts + int64_t(p) * DIM + d);
  }
  // K(d,m) = x_{m+1,d} - x_{0,d}; B = K^{-T}; g_v = B grad_ref(lambda_v)
  double K[DIM][DIM], g[NV][DIM], det;
#pragma unroll
  for (int d = 0; d < DIM; ++d)
#pragma unroll
    for (int m = 0; m < DIM; ++m) K[d][m] = x[m + 1][d] - x[0][d];
  if (DIM == 2) {
    det = K[0][0] * K[1][1] - K[0][1] * K[1][0];
    double id = 1.0 / det;
    // B = K^{-T}: B(d,m) = inv(K)(m,d)
    double Ki[2][2] = {{K[1][1] * id, -K[0][1] * id}, {-K[1][0] * id, K[0][0] * id}};
#pragma unroll
    for (int v = 1; v < NV; ++v)
#pragma unroll
      for (int d = 0; d < DIM; ++d) g[v][d] = Ki[v - 1][d];
  } else {
    double c00 = K[1][1] * K[2][2] - K[1][2] * K[2][1];
    double c01 = K[1][2] * K[2][0] - K[1][0] * K[2][2];
    double c02 = K[1][0] * K[2][1] - K[1][1] * K[2][0];
    det = K[0][0] * c00 + K[0][1] * c01 + K[0][2] * c02;
    double id = 1.0 / det;
    // inverse(K)(m,d) = cofactor(d,m)/det
    double Ki[3][3];
    Ki[0][0] = c00 * id;
    Ki[1][0] = c01 * id;
    Ki[2][0] = c02 * id;
    Ki[0][1] = (K[0][2] * K[2][1] - K[0][1] * K[2][2]) * id;
    Ki[1][1] = (K[0][0] * K[2][2] - K[0][2] * K[2][0]) * id;
    Ki[2][1] = (K[0][1] * K[2][0] - K[0][0] * K[2][1]) * id;
    Ki[0][2] = (K[0][1] * K[1][2] - K[0][2] * K[1][1]) * id;
    Ki[1][2] = (K[0][2] * K[1][0] - K[0][0] * K[1][2]) * id;
    Ki[2][2] = (K[0][0] * K[1][1] - K[0][1] * K[1][0]) * id;
#pragma unroll
    for (int v = 1; v < NV; ++v)
#pragma unroll
      for (int d = 0; d < DIM; ++d) g[v][d] = Ki[v - 1][d];
  }
#pragma unroll
  for (int d = 0; d < DIM; ++d) {
    double s = 0;
#pragma unroll
    for (int v = 1; v < NV; ++v) s += g[v][d];
    g[0][d] = -s;
  }
  double *o = out + e * lay.stride;
  if (det == 0.0) {
    set_err(err, ERR_JACOBIAN);
    for (int k = 0; k < lay.stride; ++k) o[k] = 0.0;
    return;
  }
  const double J = fabs(det);
  // coefficients (element constants) summed over the terms of each kind
  double c0 = 0, c1 = 0, c2 = 0, cmass = 0;
  for (int t = 0; t < form.n_terms; ++t) {
    const gfgpu_term &T = form.terms[t];
    auto cval = [&](const gfgpu_coef &c) -> double {
      if (c.kind == GFGPU_COEF_CONST) return c.value;
      if (c.kind == GFGPU_COEF_ELEMENT) return c.value * slots.p[c.slot][e];
      return 0.0;
    };
    if (T.kind == GFGPU_TERM_GRADGRAD) {
      c0 += T.scale * cval(T.c[0]);
      c1 += T.scale * cval(T.c[1]);
      c2 += T.scale * cval(T.c[2]);
    } else if (T.kind == GFGPU_TERM_MASS) {
      cmass += T.scale * cval(T.c[0]);
    }
  }
  double Tl[QD * QD * NV * NV];
#pragma unroll
  for (int a = 0; a < QD; ++a)
#pragma unroll
    for (int b = 0; b < QD; ++b)
#pragma unroll
      for (int v = 0; v < NV; ++v)
#pragma unroll
        for (int w = 0; w < NV; ++w) {
          double s = 0;
          if (a == b) {
            double gg = 0;
#pragma unroll
            for (int k = 0; k < DIM; ++k) gg += g[v][k] * g[w][k];
            s = c1 * gg;
          }
          if (QD > 1) s += c0 * g[v][a] * g[w][b] + c2 * g[v][b] * g[w][a];
          double val = J * s;
          Tl[((a * QD + b) * NV + v) * NV + w] = val;
          o[((a * QD + b) * NV + v) * NV + w] = val;
        }
  const double cm = J * cmass;
  o[lay.off_cm] = cm;
  o[lay.off_jw] = J;
  // threshold: max |elem|.  For a positive semi-definite element matrix the
  // largest entry is on the diagonal (|e_ij| <= sqrt(e_ii e_jj)).
  bool psd = psd_hint && cmass >= 0;
  if (QD > 1) psd = psd && (c1 + c2 >= 0) && (c1 - c2 >= 0) && (c1 + c2 + DIM * c0 >= 0);
  else psd = psd && c1 >= 0;
  const int nb = tab->nb;
  double mx = 0;
  for (int i = 0; i < nb; ++i) {
    int jlo = psd ? i : 0, jhi = psd ? i + 1 : nb;
    for (int j = jlo; j < jhi; ++j) {
      int pij = i * nb + j;
      int nt = tab->nterm[pij];
#pragma unroll
      for (int a = 0; a < QD; ++a)
#pragma unroll
        for (int b = 0; b < QD; ++b) {
          if (psd && a != b) continue;
          double s = 0;
          for (int t = 0; t < nt; ++t) {
            int vw = tab->vw[pij * kMaxPairTerms + t];
            s += tab->gval[pij * kMaxPairTerms + t] * Tl[(a * QD + b) * NV * NV + vw];
          }
          if (a == b) s += cm * tab->mass[pij];
          mx = fmax(mx, fabs(s));
        }
    }
  }
  if (!isfinite(mx)) set_err(err, ERR_NAN);
  o[lay.off_thr] = mx * 1e-14;
}

// Contribution of element e's local entry ((li,a),(lj,b)).
struct SimplexSource {
  const double *elem;
  const SimplexTables *tab;
  SimplexLayout lay;
  int qd, nv, nb;
  __device__ __forceinline__ double thr(int e) const { return elem[int64_t(e) * lay.stride + lay.off_thr]; }
  __device__ __forceinline__ double value(int e, int li, int lj, int a, int b) const {
    const double *T = elem + int64_t(e) * lay.stride;
    const int pij = li * nb + lj;
    const int nt = tab->nterm[pij];
    const double *Tab = T + (a * qd + b) * nv * nv;
    double c = 0;
    for (int t = 0; t < nt; ++t)
      c += tab->gval[pij * kMaxPairTerms + t] * Tab[tab->vw[pij * kMaxPairTerms + t]];
    if (a == b) c += T[lay.off_cm] * tab->mass[pij];
    return c;
  }
  __device__ __forceinline__ double jw(int e) const { return elem[int64_t(e) * lay.stride + lay.off_jw]; }
  __device__ __forceinline__ double mass(int li, int lj) const { return tab->mass[li * nb + lj]; }
};

// ------------------------------------------------------ warp utilities

// Bitonic sort of n (power of two) ints in shared memory by one warp.
__device__ void warp_sort(int *a, int n) {
  const int lane = threadIdx.x & 31;
  for (int k = 2; k <= n; k <<= 1) {
    for (int j = k >> 1; j > 0; j >>= 1) {
      for (int i = lane; i < n; i += kWarp) {
        int ixj = i ^ j;
        if (ixj > i) {
          int x = a[i], y = a[ixj];
          bool up = (i & k) == 0;
          if ((x > y) == up) a[i] = y, a[ixj] = x;
        }
      }
      __syncwarp();
    }
  }
}

// In-place unique of a sorted array; returns the new length.
__device__ int warp_unique(int *a, int n) {
  const int lane = threadIdx.x & 31;
  int out = 0;
  for (int base = 0; base < n; base += kWarp) {
    int i = base + lane;
    int x = i < n ? a[i] : 0;
    bool first = i < n && (i == 0 || a[i - 1] != x);
    unsigned m = __ballot_sync(0xffffffffu, first);
    __syncwarp();
    if (first) a[out + __popc(m & ((1u << lane) - 1))] = x;
    out += __popc(m);
    __syncwarp();
  }
  return out;
}

__device__ __forceinline__ int bsearch_slot(const int *s, int n, int key) {
  int lo = 0, hi = n;
  while (lo < hi) {
    int mid = (lo + hi) >> 1;
    if (s[mid] < key) lo = mid + 1;
    else hi = mid;
  }
  return (lo < n && s[lo] == key) ? lo : -1;
}

// --------------------------------------------------------- pattern build

// Per warp: candidate list (max_cand ints, rounded to a power of two) and a
// keep mask per candidate slot, then counts (MODE 0) or column indices
// (MODE 1).
template <class Src, int MODE>
__global__ void __launch_bounds__(128) pattern_kernel(
    int64_t n_nodes, int qd, int nb, const int32_t *__restrict__ adj_ptr,
    const int32_t *__restrict__ adj, const int32_t *__restrict__ enode, Src src, int cap,
    int64_t *__restrict__ rowcount, int32_t *__restrict__ ncount,
    const int64_t *__restrict__ rowptr, int32_t *__restrict__ colidx,
    const int64_t *__restrict__ nptr, int32_t *__restrict__ ncol, int *__restrict__ err) {
  extern __shared__ int smem[];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  int *cand = smem + wib * (2 * cap + kMaxLocal);
  unsigned *bits = reinterpret_cast<unsigned *>(cand + cap);
  int *ljs = reinterpret_cast<int *>(bits + cap);
  int64_t node = blockIdx.x * int64_t(blockDim.x >> 5) + wib;
  if (node >= n_nodes) return;
  const int a0 = adj_ptr[node], a1 = adj_ptr[node + 1];
  int n = 0;
  for (int k = a0; k < a1; ++k) {
    int el = adj[k] / nb;
    if (n + nb > cap) {
      if (lane == 0) set_err(err, ERR_CAPACITY);
      return;
    }
    for (int j = lane; j < nb; j += kWarp) cand[n + j] = enode[int64_t(el) * nb + j];
    n += nb;
  }
  int np = 1;
  while (np < n) np <<= 1;
  for (int j = n + lane; j < np; j += kWarp) cand[j] = 0x7fffffff;
  __syncwarp();
  warp_sort(cand, np);
  int ns = warp_unique(cand, n);
  for (int j = lane; j < ns; j += kWarp) bits[j] = 0u;
  __syncwarp();
  const int qq = qd * qd;
  for (int k = a0; k < a1; ++k) {
    const int el = adj[k] / nb, li = adj[k] % nb;
    const double thr = src.thr(el);
    for (int j = lane; j < nb; j += kWarp) ljs[j] = bsearch_slot(cand, ns, enode[int64_t(el) * nb + j]);
    __syncwarp();
    for (int c = lane; c < nb * qq; c += kWarp) {
      int lj = c / qq, ab = c % qq;
      double v = src.value(el, li, lj, ab / qd, ab % qd);
      if (fabs(v) > thr) atomicOr(&bits[ljs[lj]], 1u << ab);
    }
    __syncwarp();
  }
  if (MODE == 0) {
    for (int a = 0; a < qd; ++a) {
      unsigned am = ((1u << qd) - 1u) << (a * qd);
      int cnt = 0;
      for (int j = lane; j < ns; j += kWarp) cnt += __popc(bits[j] & am);
      for (int o = 16; o > 0; o >>= 1) cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
      if (lane == 0) rowcount[node * qd + a] = cnt;
    }
    int kept = 0;
    for (int j = lane; j < ns; j += kWarp) kept += bits[j] != 0u;
    for (int o = 16; o > 0; o >>= 1) kept += __shfl_xor_sync(0xffffffffu, kept, o);
    if (lane == 0) ncount[node] = kept;
  } else {
    for (int a = 0; a < qd; ++a) {
      unsigned am = ((1u << qd) - 1u) << (a * qd);
      int64_t base = rowptr[node * qd + a];
      const int64_t rowend = rowptr[node * qd + a + 1];
      for (int j0 = 0; j0 < ns; j0 += kWarp) {
        int j = j0 + lane;
        unsigned m = j < ns ? (bits[j] & am) : 0u;
        int c = __popc(m);
        int incl = c;
        for (int o = 1; o < 32; o <<= 1) {
          int y = __shfl_up_sync(0xffffffffu, incl, o);
          if (lane >= o) incl += y;
        }
        int total = __shfl_sync(0xffffffffu, incl, 31);
        int pos = incl - c;
        if (j < ns)
          for (int b = 0; b < qd; ++b)
            if (m & (1u << (a * qd + b))) {
              // the count pass sized the row; never write past it
              if (base + pos < rowend) colidx[base + pos] = cand[j] * qd + b;
              else set_err(err, ERR_CAPACITY);
              ++pos;
            }
        base += total;
      }
    }
    int64_t nb0 = nptr[node];
    const int64_t nend = nptr[node + 1];
    for (int j0 = 0; j0 < ns; j0 += kWarp) {
      int j = j0 + lane;
      bool keep = j < ns && bits[j] != 0u;
      unsigned m = __ballot_sync(0xffffffffu, keep);
      int64_t at = nb0 + __popc(m & ((1u << lane) - 1u));
      if (keep) {
        if (at < nend) ncol[at] = cand[j];
        else set_err(err, ERR_CAPACITY);
      }
      nb0 += __popc(m);
    }
  }
}

// ------------------------------------------------------------ row gather

template <class Src>
__global__ void __launch_bounds__(128) gather_kernel(
    int64_t n_nodes, int qd, int nb, const int32_t *__restrict__ adj_ptr,
    const int32_t *__restrict__ adj, const int32_t *__restrict__ enode, Src src, int ms,
    const int64_t *__restrict__ nptr, const int32_t *__restrict__ ncol,
    const int64_t *__restrict__ rowptr, const int32_t *__restrict__ colidx,
    double *__restrict__ vals, bool want_K, bool want_R, const double *__restrict__ u,
    const double *__restrict__ fsrc, double fscale, double *__restrict__ vec,
    int *__restrict__ err) {
  extern __shared__ double dsm[];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const int qq = qd * qd;
  // per warp: acc[ms*qq] doubles, then pos[ms*qq] ints, slots[ms] ints, ljs[nb]
  const size_t per_warp = size_t(ms) * qq * 8 + size_t(ms) * qq * 4 + size_t(ms) * 4 + 4 * kMaxLocal;
  char *base = reinterpret_cast<char *>(dsm) + wib * ((per_warp + 15) / 16 * 16);
  double *acc = reinterpret_cast<double *>(base);
  int *pos = reinterpret_cast<int *>(acc + size_t(ms) * qq);
  int *slots = pos + size_t(ms) * qq;
  int *ljs = slots + ms;
  int64_t node = blockIdx.x * int64_t(blockDim.x >> 5) + wib;
  if (node >= n_nodes) return;
  const int64_t s0 = nptr[node];
  const int ns = int(nptr[node + 1] - s0);
  if (ns > ms) {
    if (lane == 0) set_err(err, ERR_CAPACITY);
    return;
  }
  if (want_K) {
    for (int j = lane; j < ns; j += kWarp) slots[j] = ncol[s0 + j];
    for (int j = lane; j < ns * qq; j += kWarp) pos[j] = -1, acc[j] = 0.0;
    __syncwarp();
    for (int a = 0; a < qd; ++a) {
      const int64_t r0 = rowptr[node * qd + a], r1 = rowptr[node * qd + a + 1];
      for (int64_t p = r0 + lane; p < r1; p += kWarp) {
        int col = colidx[p];
        int s = bsearch_slot(slots, ns, col / qd);
        if (s >= 0) pos[(s * qd + a) * qd + col % qd] = int(p - r0);
      }
    }
    __syncwarp();
  }
  double racc[3] = {0.0, 0.0, 0.0};
  const int a0 = adj_ptr[node], a1 = adj_ptr[node + 1];
  for (int k = a0; k < a1; ++k) {
    const int el = adj[k] / nb, li = adj[k] % nb;
    const int32_t *en = enode + int64_t(el) * nb;
    if (want_K) {
      for (int j = lane; j < nb; j += kWarp) ljs[j] = bsearch_slot(slots, ns, en[j]);
      __syncwarp();
    }
    const double thr = src.thr(el);
    for (int c = lane; c < nb * qq; c += kWarp) {
      const int lj = c / qq, ab = c % qq, a = ab / qd, b = ab % qd;
      const double v = src.value(el, li, lj, a, b);
      if (want_R) {
        double uv = u[int64_t(en[lj]) * qd + b];
        if (a == 0) racc[0] += v * uv;
        else if (a == 1) racc[1] += v * uv;
        else racc[2] += v * uv;
      }
      if (want_K && fabs(v) > thr) {
        int s = ljs[lj];
        if (s >= 0) {
          int q = (s * qd + a) * qd + b;
          if (pos[q] >= 0) acc[q] += v;
        }
      }
    }
    if (want_R && fsrc) {
      const double jw = src.jw(el) * fscale;
      for (int c = lane; c < nb * qd; c += kWarp) {
        const int lj = c / qd, a = c % qd;
        double v = jw * src.mass(li, lj) * fsrc[int64_t(en[lj]) * qd + a];
        if (a == 0) racc[0] += v;
        else if (a == 1) racc[1] += v;
        else racc[2] += v;
      }
    }
    if (want_K) __syncwarp();
  }
  if (want_K) {
    __syncwarp();
    for (int a = 0; a < qd; ++a) {
      const int64_t r0 = rowptr[node * qd + a];
      for (int j = lane; j < ns * qd; j += kWarp) {
        int s = j / qd, b = j % qd;
        int q = (s * qd + a) * qd + b;
        int p = pos[q];
        if (p >= 0) vals[r0 + p] = acc[q];
      }
    }
  }
  if (want_R) {
    for (int a = 0; a < qd; ++a) {
      double r = racc[a];
      for (int o = 16; o > 0; o >>= 1) r += __shfl_xor_sync(0xffffffffu, r, o);
      if (lane == 0) {
        if (!isfinite(r)) set_err(err, ERR_NAN);
        vec[node * qd + a] = r;
      }
    }
  }
}

SimplexSource make_simplex_source(Plan &P) {
  SimplexSource s;
  s.elem = P.d_elem;
  s.tab = P.d_stab;
  s.lay = P.lay;
  s.qd = P.qdim;
  s.nv = P.dim + 1;
  s.nb = P.nb;
  return s;
}

constexpr int kWarpsPerBlock = 4;

size_t pattern_smem(int cap) { return size_t(kWarpsPerBlock) * (2 * cap + kMaxLocal) * sizeof(int); }
size_t gather_smem(int ms, int qd) {
  size_t per = size_t(ms) * qd * qd * 12 + size_t(ms) * 4 + 4 * kMaxLocal;
  return size_t(kWarpsPerBlock) * ((per + 15) / 16 * 16);
}

}  // namespace

// ---------------------------------------------------------------- host

// Sparse barycentric reference tensor of FEM_PK(dim, degree) for the plan's
// quadrature rule, and the reference mass matrix.
int build_simplex_tables(Plan &P, std::string &errmsg) {
  const int dim = P.dim, K = P.degree;
  RefElement fe(dim, SIMPLEX, K);
  Quadrature q;
  if (!quadrature_by_name(P.im, q) || q.dim != dim) {
    errmsg = "unsupported integration method " + P.im;
    return GFGPU_E_UNSUPPORTED;
  }
  if (fe.nb > kMaxNb || K > 2) {
    errmsg = "simplex element pass supports degree <= 2";
    return GFGPU_E_UNSUPPORTED;
  }
  const int nb = fe.nb, nv = dim + 1;
  SimplexTables &t = P.stab;
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
  for (int qq = 0; qq < q.nq; ++qq) {
    double lam[4];
    lam[0] = 1.0;
    for (int d = 0; d < dim; ++d) lam[d + 1] = q.pts[qq * dim + d], lam[0] -= lam[d + 1];
    for (int i = 0; i < nb; ++i) {
      double f[4], df[4];
      for (int v = 0; v < nv; ++v) factor(w[i * nv + v], lam[v], f[v], df[v]);
      double val = 1.0;
      for (int v = 0; v < nv; ++v) val *= f[v];
      phi[qq * nb + i] = val;
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
      double m = 0;
      for (int qq = 0; qq < q.nq; ++qq) m += q.w[qq] * phi[qq * nb + i] * phi[qq * nb + j];
      t.mass[pij] = m;
    }
  P.nq = q.nq;
  const int qd = P.qdim;
  P.lay.nT = qd * qd * nv * nv;
  P.lay.off_cm = P.lay.nT;
  P.lay.off_jw = P.lay.nT + 1;
  P.lay.off_thr = P.lay.nT + 2;
  P.lay.stride = P.lay.nT + 3;
  return GFGPU_OK;
}

SlotPtrs slot_ptrs(const Plan &P) {
  SlotPtrs sp;
  for (int i = 0; i < GFGPU_MAX_SLOTS; ++i) sp.p[i] = P.slot_ptr[i];
  return sp;
}

cudaError_t launch_simplex_element_pass(Plan &P) {
  const int threads = 128;
  const unsigned blocks = unsigned((P.n_elements + threads - 1) / threads);
  if (P.n_elements == 0) return cudaSuccess;
  SlotPtrs sp = slot_ptrs(P);
#define GFGPU_EP(D, Q)                                                                 \
  simplex_element_pass<D, Q><<<blocks, threads, 0, P.stream>>>(                        \
      P.n_elements, P.d_points, P.d_cv, P.d_stab, P.lay, P.form, sp, P.psd, P.d_elem, P.d_err)
  if (P.dim == 2 && P.qdim == 1) GFGPU_EP(2, 1);
  else if (P.dim == 2 && P.qdim == 2) GFGPU_EP(2, 2);
  else if (P.dim == 3 && P.qdim == 1) GFGPU_EP(3, 1);
  else if (P.dim == 3 && P.qdim == 3) GFGPU_EP(3, 3);
  else return cudaErrorInvalidValue;
#undef GFGPU_EP
  P.launches++;
  return cudaGetLastError();
}

cudaError_t launch_pattern_count(Plan &P) {
  const int cap = P.max_cand < 32 ? 32 : P.max_cand;
  int np = 1;
  while (np < cap) np <<= 1;
  size_t smem = pattern_smem(np);
  cudaError_t ce = cudaFuncSetAttribute(pattern_kernel<SimplexSource, 0>,
                                        cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
  if (ce != cudaSuccess) return ce;
  const unsigned blocks = unsigned((P.n_nodes + kWarpsPerBlock - 1) / kWarpsPerBlock);
  pattern_kernel<SimplexSource, 0><<<blocks, kWarpsPerBlock * 32, smem, P.stream>>>(
      P.n_nodes, P.qdim, P.nb, P.d_adj_ptr, P.d_adj, P.d_enode, make_simplex_source(P), np,
      P.d_count, P.d_ncount, nullptr, nullptr, nullptr, nullptr, P.d_err);
  P.launches++;
  return cudaGetLastError();
}

cudaError_t launch_pattern_fill(Plan &P) {
  const int cap = P.max_cand < 32 ? 32 : P.max_cand;
  int np = 1;
  while (np < cap) np <<= 1;
  size_t smem = pattern_smem(np);
  cudaError_t ce = cudaFuncSetAttribute(pattern_kernel<SimplexSource, 1>,
                                        cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
  if (ce != cudaSuccess) return ce;
  const unsigned blocks = unsigned((P.n_nodes + kWarpsPerBlock - 1) / kWarpsPerBlock);
  pattern_kernel<SimplexSource, 1><<<blocks, kWarpsPerBlock * 32, smem, P.stream>>>(
      P.n_nodes, P.qdim, P.nb, P.d_adj_ptr, P.d_adj, P.d_enode, make_simplex_source(P), np,
      nullptr, nullptr, P.d_rowptr, P.d_colidx, P.d_nptr, P.d_ncol, P.d_err);
  P.launches++;
  return cudaGetLastError();
}

cudaError_t launch_gather(Plan &P, bool want_K, bool want_R) {
  const int ms = P.max_slots < 1 ? 1 : P.max_slots;
  size_t smem = gather_smem(ms, P.qdim);
  cudaError_t ce = cudaFuncSetAttribute(gather_kernel<SimplexSource>,
                                        cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
  if (ce != cudaSuccess) return ce;
  const double *fsrc = nullptr;
  double fscale = 0.0;
  for (int t = 0; t < P.form.n_terms; ++t) {
    const gfgpu_term &T = P.form.terms[t];
    if (T.kind == GFGPU_TERM_SOURCE) {
      fsrc = P.slot_ptr[T.field_slot];
      fscale = T.scale * (T.c[0].kind == GFGPU_COEF_CONST ? T.c[0].value : 1.0);
    }
  }
  const unsigned blocks = unsigned((P.n_nodes + kWarpsPerBlock - 1) / kWarpsPerBlock);
  gather_kernel<SimplexSource><<<blocks, kWarpsPerBlock * 32, smem, P.stream>>>(
      P.n_nodes, P.qdim, P.nb, P.d_adj_ptr, P.d_adj, P.d_enode, make_simplex_source(P), ms,
      P.d_nptr, P.d_ncol, P.d_rowptr, P.d_colidx, P.d_vals, want_K, want_R,
      P.slot_ptr[GFGPU_SLOT_U], fsrc, fscale, P.d_vec, P.d_err);
  P.launches++;
  return cudaGetLastError();
}

}  // namespace gfgpu
