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
//   T[(a,v),(b,w)] = |J| (c0 g_va g_wb + c1 d_ab g_v.g_w + c2 g_vb g_wa)
//
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
#include <cmath>
#include <cstring>

#include "host/refelem.h"
#include "k_common.cuh"
#include "plan.h"

namespace gfgpu {

namespace {

constexpr int kEpWarps = 4;            // warps per block (share 32 elements)
constexpr int kEpThreads = 32 * kEpWarps;

}  // namespace

// Supports of the nodes of FEM_PK(DIM,K), K <= 2, in GetFEM's node order
// (lattice points, first coordinate fastest): the barycentric vertices with a
// nonzero weight, ascending.  The reference-tensor terms of a node pair (i,j)
// are supp(i) x supp(j) in this order (checked against the host tables).
__host__ __device__ constexpr int pk_sup_n(int dim, int nb, int i) {
  if (nb == dim + 1) return 1;  // P1: node i is vertex i
  // P2: vertices are the nodes with a single weight
  if (dim == 2) return (i == 0 || i == 2 || i == 5) ? 1 : 2;
  return (i == 0 || i == 2 || i == 5 || i == 9) ? 1 : 2;
}
__host__ __device__ constexpr int pk_sup_v(int dim, int nb, int i, int t) {
  if (nb == dim + 1) return i;
  // P2 triangle: (0),(0,1),(1),(0,2),(1,2),(2); tetrahedron adds (0,3),(1,3),(2,3),(3)
  switch (i) {
    case 0: return 0;
    case 1: return t == 0 ? 0 : 1;
    case 2: return 1;
    case 3: return t == 0 ? 0 : 2;
    case 4: return t == 0 ? 1 : 2;
    case 5: return 2;
    case 6: return t == 0 ? 0 : 3;
    case 7: return t == 0 ? 1 : 3;
    case 8: return t == 0 ? 2 : 3;
    default: return 3;
  }
}

// Shared memory of one 32-element tile of the simplex element pass (KU:
// with the staging of u and of the warps' parts of K_e u_e, which a pass
// leaving K u to the row gather does not reserve).
template <int DIM, int QD, int NB, bool KU = true, int W = kEpWarps>
struct EpShared {
  static constexpr int NV = DIM + 1, M = QD * NV, NTP = M * (M + 1) / 2;
  static constexpr int S = NB * QD;
  // rows: g (NV x DIM), J c1 g_v.g_w (v <= w), then J c0, J c1, J c2, J cmass, J
  static constexpr int KC = NV * DIM, KX = KC + NV * (NV + 1) / 2;
  static constexpr int NG = KX + 8;
  double s_gval[NB * NB * kMaxPairTerms];
  double s_mass[NB * NB];
  double Gs[NG][32];     // geometry of the tile's 32 elements
  union {
    struct {
      double Tp[NTP][32];         // upper triangle of T per element
      double Us[KU ? S : 1][32];  // u at the element's DOFs
    } a;                          // while the blocks of K_e are built
    double Rs[KU ? W : 1][KU ? S : 1][32];  // then: each warp's part of R_e
  } x;
  unsigned long long mxs[W][32];
};

// One tile (32 elements, 4 warps) of the element pass; every thread of the
// block calls it (it synchronises the block).
// KU: V_e holds K_e u_e + the load (else the load only: the fused K + R
// assembly forms K u from the assembled rows in the row gather)
template <int DIM, int QD, int NB, bool MASS, bool STORE_K, bool KU = true, int W = kEpWarps>
__device__ __forceinline__ void simplex_element_tile(
    EpShared<DIM, QD, NB, KU, W> &sh, int64_t tile, int64_t E, const double *__restrict__ pts,
    const int32_t *__restrict__ cv, const int32_t *__restrict__ enode,
    const SimplexTables *__restrict__ tab, const KeLayout &L, const gfgpu_form &form,
    const SlotPtrs &slots, const double *__restrict__ fsrc, double fscale,
    const double *__restrict__ u, double *__restrict__ out, int *__restrict__ err) {
  using SH = EpShared<DIM, QD, NB, KU, W>;
  constexpr int NV = SH::NV, M = SH::M;
  constexpr int S = SH::S, RS = (S + 3) & ~3;
  auto &s_gval = sh.s_gval;
  auto &s_mass = sh.s_mass;
  auto &Gs = sh.Gs;
  auto &Tp = sh.x.a.Tp;
  auto &mxs = sh.mxs;
  auto &Us = sh.x.a.Us;
  auto &Rs = sh.x.Rs;
  // the term values (their (v,w) structure is compile time, pk_sup_*)
  for (int k = threadIdx.x; k < NB * NB; k += blockDim.x) s_mass[k] = tab->mass[k];
  for (int k = threadIdx.x; k < NB * NB * kMaxPairTerms; k += blockDim.x)
    s_gval[k] = tab->gval[k];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int64_t e = tile * int64_t(32) + lane;
  const bool active = e < E;
  // ---- warp 0: geometry and coefficients (lane = element)
  if (wid == 0) {
    double g[NV][DIM], det = 0.0;
    double c0 = 0, c1 = 0, c2 = 0, cmass = 0;
    if (active) {
      double x[NV][DIM];
#pragma unroll
      for (int v = 0; v < NV; ++v) {
        const int p = __ldg(cv + e * NV + v);
#pragma unroll
        for (int d = 0; d < DIM; ++d) x[v][d] = __ldg(pts + int64_t(p) * DIM + d);
      }
      // K(d,m) = x_{m+1,d} - x_{0,d}; J = |det K|; g_v = K^{-T} grad_ref(lambda_v)
      double K[DIM][DIM];
#pragma unroll
      for (int d = 0; d < DIM; ++d)
#pragma unroll
        for (int m = 0; m < DIM; ++m) K[d][m] = x[m + 1][d] - x[0][d];
      if (DIM == 2) {
        det = K[0][0] * K[1][1] - K[0][1] * K[1][0];
        const double id = 1.0 / det;
        g[1][0] = K[1][1] * id, g[1][1] = -K[0][1] * id;
        g[2][0] = -K[1][0] * id, g[2][1] = K[0][0] * id;
      } else {
        const double c00 = K[1][1] * K[2][2] - K[1][2] * K[2][1];
        const double c01 = K[1][2] * K[2][0] - K[1][0] * K[2][2];
        const double c02 = K[1][0] * K[2][1] - K[1][1] * K[2][0];
        det = K[0][0] * c00 + K[0][1] * c01 + K[0][2] * c02;
        const double id = 1.0 / det;
        g[1][0] = c00 * id, g[2][0] = c01 * id, g[3][0] = c02 * id;
        g[1][1] = (K[0][2] * K[2][1] - K[0][1] * K[2][2]) * id;
        g[2][1] = (K[0][0] * K[2][2] - K[0][2] * K[2][0]) * id;
        g[3][1] = (K[0][1] * K[2][0] - K[0][0] * K[2][1]) * id;
        g[1][2] = (K[0][1] * K[1][2] - K[0][2] * K[1][1]) * id;
        g[2][2] = (K[0][2] * K[1][0] - K[0][0] * K[1][2]) * id;
        g[3][2] = (K[0][0] * K[1][1] - K[0][1] * K[1][0]) * id;
      }
#pragma unroll
      for (int d = 0; d < DIM; ++d) {
        double s = 0;
#pragma unroll
        for (int v = 1; v < NV; ++v) s += g[v][d];
        g[0][d] = -s;
      }
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
    } else {
#pragma unroll
      for (int v = 0; v < NV; ++v)
#pragma unroll
        for (int d = 0; d < DIM; ++d) g[v][d] = 0.0;
    }
    const bool bad = active && det == 0.0;
    if (bad) set_err(err, ERR_JACOBIAN);
    const double J = bad ? 0.0 : fabs(det);
#pragma unroll
    for (int v = 0; v < NV; ++v)
#pragma unroll
      for (int d = 0; d < DIM; ++d) Gs[v * DIM + d][lane] = bad ? 0.0 : g[v][d];
    // J c1 g_v.g_w, shared by the QD diagonal blocks of T
    int kvw = SH::KC;
#pragma unroll
    for (int v = 0; v < NV; ++v)
#pragma unroll
      for (int w = v; w < NV; ++w, ++kvw) {
        double gg = 0;
#pragma unroll
        for (int d = 0; d < DIM; ++d) gg += g[v][d] * g[w][d];
        Gs[kvw][lane] = bad ? 0.0 : (J * c1) * gg;
      }
    Gs[SH::KX + 0][lane] = J * c0;
    Gs[SH::KX + 1][lane] = J * c1;
    Gs[SH::KX + 2][lane] = J * c2;
    Gs[SH::KX + 3][lane] = J * cmass;
    Gs[SH::KX + 4][lane] = J;
  }
  __syncthreads();
  // ---- all warps: T[(a,v),(b,w)] = J (c0 g_va g_wb + c1 d_ab g_v.g_w + c2 g_vb g_wa),
  // row p = (a,v) by one warp (rows dealt in snake order, which balances the
  // rows' lengths M - p): J c0 g_va and J c2 g_vb are formed once per row,
  // so an entry costs one multiply and one FMA (plus the c1 term on the
  // diagonal blocks)
  {
    const double Jc0 = Gs[SH::KX + 0][lane], Jc2 = Gs[SH::KX + 2][lane];
#pragma unroll
    for (int p = 0; p < M; ++p) {
      const int pos = p % W;
      if (((p / W) & 1 ? W - 1 - pos : pos) != wid) continue;  // warp-uniform
      const int a = p / NV, v = p % NV;
      double s0 = 0.0, ub[QD];
      if constexpr (QD > 1) {
        s0 = Jc0 * Gs[v * DIM + a][lane];
#pragma unroll
        for (int b = 0; b < QD; ++b) ub[b] = Jc2 * Gs[v * DIM + b][lane];
      }
      int k = p * M - (p * (p - 1)) / 2;
#pragma unroll
      for (int q = p; q < M; ++q, ++k) {
        const int b = q / NV, w = q % NV;
        double val = 0.0;
        if constexpr (QD > 1) val = fma(ub[b], Gs[w * DIM + a][lane], s0 * Gs[w * DIM + b][lane]);
        if (a == b) val += Gs[SH::KC + v * NV - (v * (v - 1)) / 2 + (w - v)][lane];
        Tp[k][lane] = val;
      }
    }
  }
  __syncthreads();
  // ---- u at the element's DOFs
  if constexpr (KU) {
    for (int j = wid; j < NB; j += W) {
      const int nd = active ? __ldg(enode + e * NB + j) : 0;
#pragma unroll
      for (int b = 0; b < QD; ++b)
        Us[j * QD + b][lane] = (active && u) ? __ldg(u + int64_t(nd) * QD + b) : 0.0;
    }
  }
  __syncthreads();
  const double cm = Gs[SH::KX + 3][lane], jf = Gs[SH::KX + 4][lane] * fscale;
  double *o = out + e * L.stride;
  unsigned long long mx = 0ull;  // abs_key of the largest |entry|
  // load term of row r = (i,a): scale |J| sum_j M[i,j] f[(j,a)]
  auto load_of = [&](int i, int a) -> double {
    if (!(fsrc && active)) return 0.0;
    double s = 0.0;
#pragma unroll
    for (int j = 0; j < NB; ++j) {
      const int nd = __ldg(enode + e * NB + j);
      s += s_mass[i * NB + j] * __ldg(fsrc + int64_t(nd) * QD + a);
    }
    return jf * s;
  };
  // T[(a,v),(b,w)] from its upper triangle
  auto tp = [&](int a, int v, int b, int w) -> double {
    int p = a * NV + v, q = b * NV + w;
    if (p > q) {
      const int t = p;
      p = q;
      q = t;
    }
    return Tp[p * M - (p * (p - 1)) / 2 + (q - p)][lane];
  };
  if constexpr (QD == 1) {
    // ---- scalar fields: warp w builds rows r = w, w + 4, ... in registers,
    // adds each into R_e = K_e u_e (no threshold, as the reference's vector
    // assembly) and writes it with 32-byte stores
    for (int r = wid; r < S; r += W) {
      const int i = r;
      double row[RS];
#pragma unroll
      for (int j = 0; j < NB; ++j) {
        // entry (i, j) is computed as entry (min, max): the same terms in the
        // same order as its mirror (j, i), so K_e is symmetric bit for bit
        const int p = i < j ? i : j, q = i < j ? j : i;
        const int ppq = p * NB + q;
        double x = MASS ? cm * s_mass[ppq] : 0.0;
        const int np_ = pk_sup_n(DIM, NB, p), nq_ = pk_sup_n(DIM, NB, q);
#pragma unroll
        for (int tp_ = 0; tp_ < 2; ++tp_)
#pragma unroll
          for (int tq = 0; tq < 2; ++tq)
            if (tp_ < np_ && tq < nq_)
              x += s_gval[ppq * kMaxPairTerms + tp_ * nq_ + tq] *
                 tp(0, pk_sup_v(DIM, NB, p, tp_), 0, pk_sup_v(DIM, NB, q, tq));
        row[j] = x;
      }
#pragma unroll
      for (int c = S; c < RS; ++c) row[c] = 0.0;
      double rv = load_of(i, 0);
#pragma unroll
      for (int c = 0; c < S; ++c) {
        if constexpr (KU) rv += row[c] * Us[c][lane];
        const unsigned long long kv = abs_key(row[c]);
        mx = kv > mx ? kv : mx;
      }
      if (active) {
        if (STORE_K) {
          double4_32a *dst = reinterpret_cast<double4_32a *>(o + r * RS);
#pragma unroll
          for (int c = 0; c < RS; c += 4)
            dst[c / 4] = make_double4_32a(row[c], row[c + 1], row[c + 2], row[c + 3]);
        }
        o[L.off_vec + r] = rv;
      }
    }
    mxs[wid][lane] = mx;
    __syncthreads();
  } else {
    // ---- vector fields: node pairs (i <= j) dealt round-robin to the 4
    // warps.  K_e is symmetric (G[i,j,v,w] = G[j,i,w,v], T symmetric), so
    // the block K_e[(i,.),(j,.)] = sum_t g_t T[(.,v_t),(.,w_t)] (+ mass) is
    // computed and stored once, as whole 32-byte sectors (upper node-block
    // layout); each warp accumulates its blocks' part of
    // R_e = K_e u_e in registers, and the parts are summed in warp order.
    constexpr int BLK = QD == 2 ? 4 : 12;
    double Rp[S];
#pragma unroll
    for (int c = 0; c < S; ++c) Rp[c] = 0.0;
    int pidx = 0;
#pragma unroll
    for (int i = 0; i < NB; ++i) {
#pragma unroll
      for (int j = i; j < NB; ++j, ++pidx) {
        if (pidx % W != wid) continue;  // warp-uniform
        const int pij = i * NB + j;
        const double mij = MASS ? cm * s_mass[pij] : 0.0;
        double B[QD][QD];
#pragma unroll
        for (int a = 0; a < QD; ++a)
#pragma unroll
          for (int b = 0; b < QD; ++b) B[a][b] = (MASS && a == b) ? mij : 0.0;
        const int ni = pk_sup_n(DIM, NB, i), nj = pk_sup_n(DIM, NB, j);
#pragma unroll
        for (int ti = 0; ti < 2; ++ti) {
          if (ti >= ni) continue;
#pragma unroll
          for (int tj = 0; tj < 2; ++tj) {
            if (tj >= nj) continue;
            const int v = pk_sup_v(DIM, NB, i, ti), w = pk_sup_v(DIM, NB, j, tj);
            const double gv = s_gval[pij * kMaxPairTerms + ti * nj + tj];
#pragma unroll
            for (int a = 0; a < QD; ++a)
#pragma unroll
              for (int b = 0; b < QD; ++b) B[a][b] += gv * tp(a, v, b, w);
          }
        }
#pragma unroll
        for (int a = 0; a < QD; ++a)
#pragma unroll
          for (int b = 0; b < QD; ++b) {
            if constexpr (KU) {
              Rp[i * QD + a] += B[a][b] * Us[j * QD + b][lane];
              if (i != j) Rp[j * QD + b] += B[a][b] * Us[i * QD + a][lane];
            }
            const unsigned long long kv = abs_key(B[a][b]);
            mx = kv > mx ? kv : mx;
          }
        if (STORE_K && active) {
          // upper node-block layout: block (i,j), i <= j, only (the row
          // gather reads (j,i) as its transpose)
          double4_32a *dij = reinterpret_cast<double4_32a *>(o + ke_block(NB, i, j) * BLK);
          if constexpr (QD == 2) {
            dij[0] = make_double4_32a(B[0][0], B[0][1], B[1][0], B[1][1]);
          } else {
            dij[0] = make_double4_32a(B[0][0], B[0][1], B[0][2], B[1][0]);
            dij[1] = make_double4_32a(B[1][1], B[1][2], B[2][0], B[2][1]);
            dij[2] = make_double4_32a(B[2][2], 0.0, 0.0, 0.0);
          }
        }
      }
    }
    mxs[wid][lane] = mx;
    __syncthreads();  // every warp is done with T and u
    if constexpr (KU) {
#pragma unroll
      for (int c = 0; c < S; ++c) Rs[wid][c][lane] = Rp[c];
      __syncthreads();
    }
    for (int r = wid; r < S; r += W) {
      double rv = load_of(r / QD, r % QD);
      if constexpr (KU) {
#pragma unroll
        for (int k = 0; k < W; ++k) rv += Rs[k][r][lane];
      }
      if (active) o[L.off_vec + r] = rv;
    }
  }
  if (wid == 0 && active) {
    unsigned long long m = mxs[0][lane];
#pragma unroll
    for (int k = 1; k < W; ++k) m = mxs[k][lane] > m ? mxs[k][lane] : m;
    const double mxd = abs_of_key(m);
    if (!isfinite(mxd)) set_err(err, ERR_NAN);
    if (STORE_K) o[L.off_thr] = mxd * 1e-14;
#pragma unroll
    for (int c = S; c < RS; ++c) o[L.off_vec + c] = 0.0;
  }
}

namespace {

// W warps share the tile's 32 elements (W threads per element): the rows of
// T and the node-pair blocks of K_e are dealt to the warps, each computed by
// one warp whatever W is, so K_e and the loads are the same bits for every W
// (the per-warp parts of K_e u_e of a KU pass are summed in warp order and
// depend on W: KU passes keep the default)
template <int DIM, int QD, int NB, bool MASS, bool STORE_K, bool KU, int W = kEpWarps>
__global__ void __launch_bounds__(32 * W) simplex_element_pass(
    int64_t E, const double *__restrict__ pts, const int32_t *__restrict__ cv,
    const int32_t *__restrict__ enode, const SimplexTables *__restrict__ tab, KeLayout L,
    gfgpu_form form, SlotPtrs slots, const double *__restrict__ fsrc, double fscale,
    const double *__restrict__ u, double *__restrict__ out, int *__restrict__ err,
    int64_t tile0) {
  __shared__ EpShared<DIM, QD, NB, KU, W> sh;
  simplex_element_tile<DIM, QD, NB, MASS, STORE_K, KU, W>(sh, tile0 + blockIdx.x, E, pts, cv,
                                                      enode, tab, L, form, slots, fsrc, fscale, u,
                                                      out, err);
}

}  // namespace

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
