// The affine-simplex element pass as device templates: shared-memory
// layout, the tile function and the kernel.  Included by k_simplex.cu (the
// isotropic forms and the host side) and k_simplex_ten.cu (the instances
// with a constant anisotropic coupling), so that the two sets of instances
// compile in parallel and the isotropic kernels are the same code whether
// or not the anisotropic ones exist.
#pragma once

#include <cmath>
#include <cstring>
#include <type_traits>

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
// TEN: the form has a GRADGRAD_TENSOR term (constant anisotropic coupling)
template <int DIM, int QD, int NB, bool MASS, bool STORE_K, bool KU = true, int W = kEpWarps,
          bool TEN = false>
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
    double c0 = 0, c1 = 0, c2 = 0, cmass = 0, cten = 0;
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
        } else if (TEN && T.kind == GFGPU_TERM_GRADGRAD_TENSOR) {
          cten += T.scale * (T.c[0].kind == GFGPU_COEF_NONE ? 1.0 : cval(T.c[0]));
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
    if constexpr (TEN) Gs[SH::KX + 5][lane] = J * cten;
  }
  __syncthreads();
  // ---- all warps: T[(a,v),(b,w)] = J (c0 g_va g_wb + c1 d_ab g_v.g_w + c2 g_vb g_wa),
  // row p = (a,v) by one warp (rows dealt in snake order, which balances the
  // rows' lengths M - p): J c0 g_va and J c2 g_vb are formed once per row,
  // so an entry costs one multiply and one FMA (plus the c1 term on the
  // diagonal blocks).  A GRADGRAD_TENSOR term (TEN) adds J c sum_{k,l}
  // D[(a,k),(b,l)] g_vk g_wl: per row h[b][l] = sum_k D[(a,k),(b,l)] g_vk,
  // then dim FMAs per entry; D is symmetric, so the upper triangle is T
  {
    const double Jc0 = Gs[SH::KX + 0][lane], Jc2 = Gs[SH::KX + 2][lane];
    const double Jct = TEN ? Gs[SH::KX + 5][lane] : 0.0;
    constexpr int ND = QD * DIM;
    constexpr bool kTen = TEN;
    {
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
        double h[kTen ? QD : 1][DIM];
        if constexpr (kTen) {
#pragma unroll
          for (int b = 0; b < QD; ++b)
#pragma unroll
            for (int l = 0; l < DIM; ++l) {
              double x = 0.0;
#pragma unroll
              for (int kk = 0; kk < DIM; ++kk)
                x = fma(form.tensor[(a * DIM + kk) * ND + b * DIM + l], Gs[v * DIM + kk][lane], x);
              h[b][l] = x;
            }
        }
        int k = p * M - (p * (p - 1)) / 2;
#pragma unroll
        for (int q = p; q < M; ++q, ++k) {
          const int b = q / NV, w = q % NV;
          double val = 0.0;
          if constexpr (QD > 1) val = fma(ub[b], Gs[w * DIM + a][lane], s0 * Gs[w * DIM + b][lane]);
          if (a == b) val += Gs[SH::KC + v * NV - (v * (v - 1)) / 2 + (w - v)][lane];
          if constexpr (kTen) {
            double tv = 0.0;
#pragma unroll
            for (int l = 0; l < DIM; ++l) tv = fma(h[b][l], Gs[w * DIM + l][lane], tv);
            val = fma(Jct, tv, val);
          }
          Tp[k][lane] = val;
        }
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
template <int DIM, int QD, int NB, bool MASS, bool STORE_K, bool KU, int W = kEpWarps,
          bool TEN = false>
__global__ void __launch_bounds__(32 * W) simplex_element_pass(
    int64_t E, const double *__restrict__ pts, const int32_t *__restrict__ cv,
    const int32_t *__restrict__ enode, const SimplexTables *__restrict__ tab, KeLayout L,
    gfgpu_form form, SlotPtrs slots, const double *__restrict__ fsrc, double fscale,
    const double *__restrict__ u, double *__restrict__ out, int *__restrict__ err,
    int64_t tile0) {
  __shared__ EpShared<DIM, QD, NB, KU, W> sh;
  simplex_element_tile<DIM, QD, NB, MASS, STORE_K, KU, W, TEN>(sh, tile0 + blockIdx.x, E, pts, cv,
                                                           enode, tab, L, form, slots, fsrc,
                                                           fscale, u, out, err);
}

}  // namespace

}  // namespace gfgpu
