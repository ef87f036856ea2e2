// Element kernel for scalar FEM_QK(3,K) on parallelepiped hexahedra (GT_QK(3,1)
// with constant Jacobian), FP64: the high-order case (FEM_QK(3,4),
// IM_GAUSS_PARALLELEPIPED(3,9): 125 basis functions, 125 Gauss points).
//
// When K = sum_v x_v grad(phi_geo_v) is the same at every Gauss point, the
// reference's per-point contraction (getfem_generic_assembly_compile_and_exec.cc:
// 8750-8869; t(i,j) += c J w_q grad phi_i . grad phi_j with the real gradients
// B grad_ref phi, getfem_fem.cc:160-200) factors into reference tensors:
//   K_e[i,j] = c |J| sum_{m<=n} M'_mn G_mn[i,j],   M = B^T B,
//   G_mm[i,j] = sum_q w_q dm phi_i dm phi_j,
//   G_mn[i,j] = sum_q w_q (dm phi_i dn phi_j + dn phi_i dm phi_j)  (m < n),
// plus c_m |J| Mhat[i,j] (Mhat = sum_q w_q phi_i phi_j) for a mass term and
// c_f |J| Mhat f_e for a load.  The tables are summed on the host in long
// double from the reference-tabulated gradients at the Gauss points (the same
// values the reference's fem_precomp holds), so every element costs 6 FMAs per
// entry instead of 3 x 125.
//
// One CTA per element.  K_e is symmetric: each thread owns upper-triangle
// entries (tables read coalesced from L2) and writes both (r,c) and (c,r).
// V_e = K_e u_e + load is then formed by one thread per row from the
// (symmetric) columns just written.
//
// The vector-only pass (matrix-free R = K u + load) is sum-factorised: the
// FEM_QK(3,K) basis is the tensor product of the FEM_PK(1,K) basis
// (tproduct_femi, getfem_fem.cc:792-826) and IM_GAUSS_PARALLELEPIPED the
// tensor product of IM_GAUSS1D, so the reference's per-point sums
//   V_e[i] = sum_q w_q |J| (grad phi_i . c1 B^T B grad u(q) + phi_i h(q)),
//   h = c_m u + c_f f,
// are done as 1D contractions, direction by direction: about 11 k FMAs per
// Q4 element instead of the 110 k of forming each K_e entry from 7 tables.
#include <cmath>
#include <cstdio>
#include <cstring>

#include "host/refelem.h"
#include "k_common.cuh"
#include "plan.h"

namespace gfgpu {

namespace {

constexpr int kAffThreads = 256;
constexpr int kAffTables = 7;  // G_00, G_11, G_22, G_01, G_02, G_12, Mhat

// Geometry of parallelepiped element e, lane-parallel in one warp (an FP64
// warp instruction occupies the pipe as long with one active lane as with
// 32): K(d,m) = sum_v x_v[d] dphi_v/dxi_m on lanes 0-8, det and B = K^{-T}
// (cofactor / det) on lanes 0-8, M = B^T B upper triangle (00, 11, 22, 01,
// 02, 12) on lanes 0-5.  Writes g[0..8] = K, g[9..17] = B, g[18..23] = M,
// g[24] = |det| (0 for a degenerate element, which sets ERR_JACOBIAN).
// edges: K from the edge vectors x_{e_m} - x_0 (exact differences: an
// axis-aligned element gets exact zeros off the diagonal of K, B and M)
__device__ __forceinline__ void parallelepiped_geometry(int lane, int64_t e,
                                                        const double *__restrict__ pts,
                                                        const int32_t *__restrict__ cv,
                                                        const double *__restrict__ ggrad0,
                                                        double *g, int *err, bool edges = false) {
  if (lane < 9) {
    const int d = lane % 3, m = lane / 3;
    if (edges) {
      g[lane] = pts[int64_t(cv[e * 8 + (1 << m)]) * 3 + d] - pts[int64_t(cv[e * 8]) * 3 + d];
    } else {
      double s = 0.0;
      for (int v = 0; v < 8; ++v) s += pts[int64_t(cv[e * 8 + v]) * 3 + d] * ggrad0[v * 3 + m];
      g[lane] = s;
    }
  }
  __syncwarp();
  if (lane < 9) {
    const double *K = g;
    const double a0 = K[4] * K[8] - K[5] * K[7];
    const double a1 = K[5] * K[6] - K[3] * K[8];
    const double a2 = K[3] * K[7] - K[4] * K[6];
    const double det = K[0] * a0 + K[1] * a1 + K[2] * a2;
    const int i = lane % 3, j = lane / 3;
    const int i1 = (i + 1) % 3, i2 = (i + 2) % 3, j1 = (j + 1) % 3, j2 = (j + 2) % 3;
    g[9 + lane] = (K[i1 + 3 * j1] * K[i2 + 3 * j2] - K[i1 + 3 * j2] * K[i2 + 3 * j1]) / det;
    if (lane == 0) {
      if (det == 0.0) set_err(err, ERR_JACOBIAN);
      g[24] = det == 0.0 ? 0.0 : fabs(det);
    }
  }
  __syncwarp();
  if (lane < 6) {
    const int m = lane < 3 ? lane : (lane == 5 ? 1 : 0);
    const int n = lane < 3 ? lane : (lane == 3 ? 1 : 2);
    const double *B = g + 9;
    double s = 0.0;
    for (int d = 0; d < 3; ++d) s += B[d + 3 * m] * B[d + 3 * n];
    g[18 + lane] = s;
  }
  __syncwarp();
}

// T threads per element (the CTA of the element); every entry and row is
// computed by one thread in the same order whatever T is (same bits).
// AX: an axis-aligned mesh (the host checks every element exactly): K from
// the edge vectors, the off-diagonal metric terms exact zeros, and K_e from
// G_00, G_11, G_22 (and the mass table when the form has a mass term) only.
template <int NB, bool WANT_K, int T = kAffThreads, bool AX = false>
__global__ void __launch_bounds__(T) affine_hex_kernel(
    int64_t E, const double *__restrict__ pts, const int32_t *__restrict__ cv,
    const int32_t *__restrict__ enode, const double *__restrict__ tabs,
    const int32_t *__restrict__ tri, const double *__restrict__ ggrad0, KeLayout L,
    gfgpu_form form, SlotPtrs slots, double *__restrict__ out, int *__restrict__ err) {
  constexpr int NT = NB * (NB + 1) / 2;
  constexpr int NN = NB * NB;
  __shared__ double cp[kAffTables];  // coefficients of the tables
  __shared__ double cf;              // load factor c_f |J|
  __shared__ double us[NB], fs[NB];
  __shared__ unsigned long long smax;
  __shared__ double geo[25];         // K, B, B^T B, |J|
  const int64_t e = blockIdx.x;
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  const double *u = slots.p[GFGPU_SLOT_U];
  int src_slot = -1;
  for (int t = 0; t < form.n_terms; ++t)
    if (form.terms[t].kind == GFGPU_TERM_SOURCE) src_slot = form.terms[t].field_slot;
  for (int j = tid; j < NB; j += T) {
    const int32_t n = enode[e * NB + j];
    us[j] = u ? u[n] : 0.0;
    fs[j] = src_slot >= 0 ? slots.p[src_slot][n] : 0.0;
  }
  if (wid == 0) {
    parallelepiped_geometry(lane, e, pts, cv, ggrad0, geo, err, AX);
    if (lane == 0) {
      smax = 0ull;
      const double J = geo[24];
      double c1 = 0.0, cm = 0.0, csrc = 0.0;
      for (int t = 0; t < form.n_terms; ++t) {
        const gfgpu_term &Tm = form.terms[t];
        auto val = [&](const gfgpu_coef &c) {
          if (c.kind == GFGPU_COEF_CONST) return c.value;
          if (c.kind == GFGPU_COEF_ELEMENT) return c.value * slots.p[c.slot][e];
          return 0.0;
        };
        if (Tm.kind == GFGPU_TERM_GRADGRAD) c1 += Tm.scale * val(Tm.c[1]);
        else if (Tm.kind == GFGPU_TERM_MASS) cm += Tm.scale * val(Tm.c[0]);
        else if (Tm.kind == GFGPU_TERM_SOURCE)
          csrc += Tm.scale * (Tm.c[0].kind == GFGPU_COEF_NONE ? 1.0 : val(Tm.c[0]));
      }
      const double cJ = c1 * J;
      for (int k = 0; k < 6; ++k) cp[k] = cJ * geo[18 + k];
      cp[6] = cm * J;
      cf = csrc * J;
    }
  }
  __syncthreads();
  double c[kAffTables];
#pragma unroll
  for (int p = 0; p < kAffTables; ++p) c[p] = cp[p];
  // a mass term (block-uniform, from the form)
  bool hasm = false;
  for (int t = 0; t < form.n_terms; ++t) hasm |= form.terms[t].kind == GFGPU_TERM_MASS;
  double *o = out + e * L.stride;
  if constexpr (WANT_K) {
    unsigned long long mx = 0ull;
    for (int ent = tid; ent < NT; ent += T) {
      const int rc = tri[ent];
      const int r = rc >> 16, col = rc & 0xffff;
      const int idx = r * NB + col;
      double v = c[0] * tabs[idx];
      if constexpr (AX) {
        v = fma(c[1], tabs[NN + idx], v);
        v = fma(c[2], tabs[2 * NN + idx], v);
        if (hasm) v = fma(c[6], tabs[6 * NN + idx], v);
      } else {
#pragma unroll
        for (int p = 1; p < kAffTables; ++p) v = fma(c[p], tabs[p * NN + idx], v);
      }
      o[r * L.rowstride + col] = v;
      if (r != col) o[col * L.rowstride + r] = v;
      const unsigned long long bits = abs_key(v);
      mx = bits > mx ? bits : mx;
    }
    atomicMax(&smax, mx);
    __syncthreads();  // the rows of K_e are visible to the block
  }
  // V_e[r] = sum_c K_e[r,c] u_c + c_f sum_c Mhat[r,c] f_c, one thread per row.
  // K_e and the tables are symmetric bit for bit (both halves of K_e are one
  // value; the tables' (i,j) and (j,i) sums add the same products), so thread
  // r walks column r instead: the loads coalesce across threads and no warp
  // reduction is needed (one FMA per entry; the butterfly of a warp per row
  // cost more FP64 instructions than the row's FMAs).
  for (int r = tid; r < NB; r += T) {
    double s = 0.0, sf = 0.0;
    for (int col = 0; col < NB; ++col) {
      const int idx = col * NB + r;
      double k;
      if constexpr (WANT_K) {
        k = o[col * L.rowstride + r];
      } else {
        k = c[0] * tabs[idx];
        if constexpr (AX) {
          k = fma(c[1], tabs[NN + idx], k);
          k = fma(c[2], tabs[2 * NN + idx], k);
          if (hasm) k = fma(c[6], tabs[6 * NN + idx], k);
        } else {
#pragma unroll
          for (int p = 1; p < kAffTables; ++p) k = fma(c[p], tabs[p * NN + idx], k);
        }
      }
      s = fma(k, us[col], s);
      if (src_slot >= 0) sf = fma(tabs[6 * NN + idx], fs[col], sf);
    }
    const double v = fma(cf, sf, s);
    if (!isfinite(v)) set_err(err, ERR_NAN);
    o[L.off_vec + r] = v;
  }
  if constexpr (WANT_K) {
    if (tid == 0) {
      const double m = abs_of_key(smax);
      if (!isfinite(m)) set_err(err, ERR_NAN);
      o[L.off_thr] = m * 1e-14;
    }
  }
}

// Vector-only pass (matrix-free R = K u) of a GRADGRAD-only form through the
// reference tensors: R_e[r] = sum_p c_p (G_p u_e)[r], c_p = c1 |J| M_p, with
// K from the element's edge vectors (exact differences).  On an axis-aligned
// mesh (NP = 3) only G_00, G_11, G_22 enter: 3 FMAs per element and entry
// instead of forming each entry of K_e from 7 tables (8 operations) and
// multiplying.  Thread r walks column r of each table (tables symmetric:
// coalesced loads) for EQ elements of the block at once, so each table load
// feeds EQ FMAs.
template <int NB, int NP, int EQ>
__global__ void __launch_bounds__(128) affine_scalar_apply_kernel(
    int64_t E, const double *__restrict__ pts, const int32_t *__restrict__ cv,
    const int32_t *__restrict__ enode, const double *__restrict__ tabs, KeLayout L,
    gfgpu_form form, SlotPtrs slots, double *__restrict__ out, int *__restrict__ err) {
  constexpr int NN = NB * NB;
  static_assert(NB <= 128, "one thread per row");
  __shared__ double us[EQ][NB];
  __shared__ double cfs[EQ][NP];
  const int tid = threadIdx.x;
  const int64_t e0 = int64_t(blockIdx.x) * EQ;
  const int ne = E - e0 < EQ ? int(E - e0) : EQ;
  const double *u = slots.p[GFGPU_SLOT_U];
  for (int z = tid; z < NB * EQ; z += 128) {
    const int k = z / NB, j = z - k * NB;
    us[k][j] = (k < ne && u) ? u[enode[(e0 + k) * NB + j]] : 0.0;
  }
  if (tid < EQ) {
    const int k = tid;
    double m[NP];
#pragma unroll
    for (int p = 0; p < NP; ++p) m[p] = 0.0;
    if (k < ne) {
      const int64_t e = e0 + k;
      const int32_t *c = cv + e * 8;
      double K[9], B[9];
#pragma unroll
      for (int mm = 0; mm < 3; ++mm)
#pragma unroll
        for (int d = 0; d < 3; ++d)
          K[d + 3 * mm] = pts[int64_t(c[1 << mm]) * 3 + d] - pts[int64_t(c[0]) * 3 + d];
      const double a0 = K[4] * K[8] - K[5] * K[7];
      const double a1 = K[5] * K[6] - K[3] * K[8];
      const double a2 = K[3] * K[7] - K[4] * K[6];
      const double det = K[0] * a0 + K[1] * a1 + K[2] * a2;
#pragma unroll
      for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) {
          const int i1 = (i + 1) % 3, i2 = (i + 2) % 3, j1 = (j + 1) % 3, j2 = (j + 2) % 3;
          B[i + 3 * j] = (K[i1 + 3 * j1] * K[i2 + 3 * j2] - K[i1 + 3 * j2] * K[i2 + 3 * j1]) / det;
        }
      if (det == 0.0) set_err(err, ERR_JACOBIAN);
      const double J = det == 0.0 ? 0.0 : fabs(det);
      double c1 = 0.0;
      for (int t = 0; t < form.n_terms; ++t) {
        const gfgpu_term &Tm = form.terms[t];
        const gfgpu_coef &cc = Tm.c[1];
        const double v = cc.kind == GFGPU_COEF_CONST     ? cc.value
                         : cc.kind == GFGPU_COEF_ELEMENT ? cc.value * slots.p[cc.slot][e]
                                                         : 0.0;
        c1 += Tm.scale * v;
      }
      const double cJ = c1 * J;
      // M_mn = sum_d B(d,m) B(d,n), table order 00 11 22 01 02 12
#pragma unroll
      for (int p = 0; p < NP; ++p) {
        const int pm = p < 3 ? p : (p == 5 ? 1 : 0), pn = p < 3 ? p : (p == 3 ? 1 : 2);
        double sum = 0.0;
        for (int d = 0; d < 3; ++d) sum += B[d + 3 * pm] * B[d + 3 * pn];
        m[p] = cJ * sum;
      }
    }
#pragma unroll
    for (int p = 0; p < NP; ++p) cfs[k][p] = m[p];
  }
  __syncthreads();
  if (tid >= NB) return;
  const int r = tid;
  double acc[EQ][NP];
#pragma unroll
  for (int k = 0; k < EQ; ++k)
#pragma unroll
    for (int p = 0; p < NP; ++p) acc[k][p] = 0.0;
  for (int c = 0; c < NB; ++c) {
    double g[NP];
#pragma unroll
    for (int p = 0; p < NP; ++p) g[p] = tabs[p * NN + c * NB + r];
#pragma unroll
    for (int k = 0; k < EQ; ++k) {
      const double uc = us[k][c];
#pragma unroll
      for (int p = 0; p < NP; ++p) acc[k][p] = fma(g[p], uc, acc[k][p]);
    }
  }
#pragma unroll
  for (int k = 0; k < EQ; ++k) {
    if (k >= ne) break;
    double v = cfs[k][0] * acc[k][0];
#pragma unroll
    for (int p = 1; p < NP; ++p) v = fma(cfs[k][p], acc[k][p], v);
    if (!isfinite(v)) set_err(err, ERR_NAN);
    out[(e0 + k) * L.stride + L.off_vec + r] = v;
  }
}

// 1D tables of the sum factorisation: values and derivatives of the 1D
// basis at the 1D Gauss points (N[q][a], D[q][a]), the 1D weights, and the
// tensor index a + P1 (b + P1 c) of each local DOF
template <int P1, int Q1>
struct SumFac {
  double N[Q1][P1], D[Q1][P1], w[Q1];
  int perm[P1 * P1 * P1];
};

constexpr int kSfThreads = 128;

template <int P1, int Q1, bool HASV>
__global__ void __launch_bounds__(kSfThreads) affine_hex_apply_kernel(
    int64_t E, const double *__restrict__ pts, const int32_t *__restrict__ cv,
    const int32_t *__restrict__ enode, const SumFac<P1, Q1> *__restrict__ sf,
    const double *__restrict__ ggrad0, KeLayout L, gfgpu_form form, SlotPtrs slots,
    double *__restrict__ out, int *__restrict__ err) {
  constexpr int NB = P1 * P1 * P1;
  constexpr int M3 = (P1 > Q1 ? P1 : Q1) * (P1 > Q1 ? P1 : Q1) * (P1 > Q1 ? P1 : Q1);
  __shared__ double sN[Q1][P1], sD[Q1][P1], sw[Q1];
  __shared__ double cM[6], cJ;            // c1 |J| B^T B (upper), |J|
  __shared__ double geo[25];              // K, B, B^T B, |J|
  __shared__ double U[M3], Hd[M3];        // u and h = c_m u + c_f f (tensor order)
  __shared__ double A0[M3], A1[M3], A2[M3], A3[M3];
  __shared__ double B0[M3], B1[M3], B2[M3], B3[M3];
  const int64_t e = blockIdx.x;
  const int tid = threadIdx.x;
  if (e >= E) return;
  for (int t = tid; t < Q1 * P1; t += kSfThreads) {
    sN[t / P1][t % P1] = sf->N[t / P1][t % P1];
    sD[t / P1][t % P1] = sf->D[t / P1][t % P1];
  }
  if (tid < Q1) sw[tid] = sf->w[tid];
  const double *u = slots.p[GFGPU_SLOT_U];
  int src_slot = -1;
  double cm = 0.0, csrc = 0.0, c1 = 0.0;
  for (int t = 0; t < form.n_terms; ++t) {
    const gfgpu_term &T = form.terms[t];
    auto val = [&](const gfgpu_coef &c) {
      if (c.kind == GFGPU_COEF_CONST) return c.value;
      if (c.kind == GFGPU_COEF_ELEMENT) return c.value * slots.p[c.slot][e];
      return 0.0;
    };
    if (T.kind == GFGPU_TERM_GRADGRAD) c1 += T.scale * val(T.c[1]);
    else if (T.kind == GFGPU_TERM_MASS) cm += T.scale * val(T.c[0]);
    else if (T.kind == GFGPU_TERM_SOURCE) {
      src_slot = T.field_slot;
      csrc += T.scale * (T.c[0].kind == GFGPU_COEF_NONE ? 1.0 : val(T.c[0]));
    }
  }
  for (int i = tid; i < NB; i += kSfThreads) {
    const int32_t n = enode[e * NB + i];
    const int p = sf->perm[i];
    const double ui = u ? u[n] : 0.0;
    U[p] = ui;
    if (HASV) Hd[p] = cm * ui + (src_slot >= 0 ? csrc * slots.p[src_slot][n] : 0.0);
  }
  if (tid < 32) {
    parallelepiped_geometry(tid, e, pts, cv, ggrad0, geo, err);
    if (tid < 6) cM[tid] = c1 * geo[24] * geo[18 + tid];
    if (tid == 0) cJ = geo[24];
  }
  __syncthreads();
  // ---- x: A0 = N_x u, A1 = D_x u, A2 = N_x h          [c][b][qx]
  for (int t = tid; t < P1 * P1 * Q1; t += kSfThreads) {
    const int qx = t % Q1, cb = t / Q1;
    double s0 = 0.0, s1 = 0.0, s2 = 0.0;
#pragma unroll
    for (int a = 0; a < P1; ++a) {
      const double x = U[cb * P1 + a];
      s0 = fma(sN[qx][a], x, s0);
      s1 = fma(sD[qx][a], x, s1);
      if (HASV) s2 = fma(sN[qx][a], Hd[cb * P1 + a], s2);
    }
    A0[t] = s0, A1[t] = s1;
    if (HASV) A2[t] = s2;
  }
  __syncthreads();
  // ---- y: B0 = N_y A1 (d/dx), B1 = D_y A0 (d/dy), B2 = N_y A0 (d/dz), B3 = N_y A2
  for (int t = tid; t < P1 * Q1 * Q1; t += kSfThreads) {
    const int qx = t % Q1, qy = (t / Q1) % Q1, c = t / (Q1 * Q1);
    double s0 = 0.0, s1 = 0.0, s2 = 0.0, s3 = 0.0;
#pragma unroll
    for (int b = 0; b < P1; ++b) {
      const int k = (c * P1 + b) * Q1 + qx;
      s0 = fma(sN[qy][b], A1[k], s0);
      s1 = fma(sD[qy][b], A0[k], s1);
      s2 = fma(sN[qy][b], A0[k], s2);
      if (HASV) s3 = fma(sN[qy][b], A2[k], s3);
    }
    B0[t] = s0, B1[t] = s1, B2[t] = s2;
    if (HASV) B3[t] = s3;
  }
  __syncthreads();
  // ---- z: gradient and value at the Gauss points, then the fluxes
  // (A0..A3 reused as fx, fy, fz, fh on [qz][qy][qx])
  for (int t = tid; t < Q1 * Q1 * Q1; t += kSfThreads) {
    const int qx = t % Q1, qy = (t / Q1) % Q1, qz = t / (Q1 * Q1);
    double gx = 0.0, gy = 0.0, gz = 0.0, hv = 0.0;
#pragma unroll
    for (int c = 0; c < P1; ++c) {
      const int k = (c * Q1 + qy) * Q1 + qx;
      gx = fma(sN[qz][c], B0[k], gx);
      gy = fma(sN[qz][c], B1[k], gy);
      gz = fma(sD[qz][c], B2[k], gz);
      if (HASV) hv = fma(sN[qz][c], B3[k], hv);
    }
    const double w = sw[qx] * sw[qy] * sw[qz];
    A0[t] = w * (cM[0] * gx + cM[3] * gy + cM[4] * gz);
    A1[t] = w * (cM[3] * gx + cM[1] * gy + cM[5] * gz);
    A2[t] = w * (cM[4] * gx + cM[5] * gy + cM[2] * gz);
    if (HASV) A3[t] = w * cJ * hv;
  }
  __syncthreads();
  // ---- z^T: B0 = N_z^T fx, B1 = N_z^T fy, B2 = D_z^T fz + N_z^T fh   [c][qy][qx]
  for (int t = tid; t < P1 * Q1 * Q1; t += kSfThreads) {
    const int qx = t % Q1, qy = (t / Q1) % Q1, c = t / (Q1 * Q1);
    double s0 = 0.0, s1 = 0.0, s2 = 0.0;
#pragma unroll
    for (int qz = 0; qz < Q1; ++qz) {
      const int k = (qz * Q1 + qy) * Q1 + qx;
      s0 = fma(sN[qz][c], A0[k], s0);
      s1 = fma(sN[qz][c], A1[k], s1);
      s2 = fma(sD[qz][c], A2[k], s2);
      if (HASV) s2 = fma(sN[qz][c], A3[k], s2);
    }
    B0[t] = s0, B1[t] = s1, B2[t] = s2;
  }
  __syncthreads();
  // ---- y^T: A0 = N_y^T B0 (-> D_x^T), A1 = D_y^T B1 + N_y^T B2 (-> N_x^T)   [c][b][qx]
  for (int t = tid; t < P1 * P1 * Q1; t += kSfThreads) {
    const int qx = t % Q1, b = (t / Q1) % P1, c = t / (Q1 * P1);
    double s0 = 0.0, s1 = 0.0;
#pragma unroll
    for (int qy = 0; qy < Q1; ++qy) {
      const int k = (c * Q1 + qy) * Q1 + qx;
      s0 = fma(sN[qy][b], B0[k], s0);
      s1 = fma(sD[qy][b], B1[k], s1);
      s1 = fma(sN[qy][b], B2[k], s1);
    }
    A0[t] = s0, A1[t] = s1;
  }
  __syncthreads();
  // ---- x^T: V_e = D_x^T A0 + N_x^T A1, written in local DOF order
  double *o = out + e * L.stride;
  for (int i = tid; i < NB; i += kSfThreads) {
    const int p = sf->perm[i];
    const int a = p % P1, cb = p / P1;
    double s = 0.0;
#pragma unroll
    for (int qx = 0; qx < Q1; ++qx) {
      s = fma(sD[qx][a], A0[cb * Q1 + qx], s);
      s = fma(sN[qx][a], A1[cb * Q1 + qx], s);
    }
    if (!isfinite(s)) set_err(err, ERR_NAN);
    o[L.off_vec + i] = s;
  }
}

}  // namespace

// The forms of this kernel: scalar GRADGRAD (c1), MASS and SOURCE terms with
// constant or per-element coefficients.
bool affine_hex_form_ok(const gfgpu_form &f, int qdim) {
  if (qdim != 1) return false;
  for (int t = 0; t < f.n_terms; ++t) {
    const gfgpu_term &T = f.terms[t];
    if (T.kind != GFGPU_TERM_GRADGRAD && T.kind != GFGPU_TERM_MASS && T.kind != GFGPU_TERM_SOURCE)
      return false;
    for (int k = 0; k < 3; ++k)
      if (T.c[k].kind == GFGPU_COEF_NODAL) return false;
  }
  return true;
}

// True when every element of the mesh is a parallelepiped: x_v = x_0 +
// sum_d l_d(v) (x_{e_d} - x_0) for the GT_QK(3,1) vertex lattice l(v).
bool mesh_is_parallelepiped(const double *pts, const int64_t *cv, int64_t E) {
  for (int64_t e = 0; e < E; ++e) {
    const int64_t *c = cv + e * 8;
    const double *x0 = pts + c[0] * 3;
    double ed[3][3], scale = 0.0;
    for (int d = 0; d < 3; ++d)
      for (int k = 0; k < 3; ++k) {
        ed[d][k] = pts[c[1 << d] * 3 + k] - x0[k];
        scale = std::max(scale, std::fabs(ed[d][k]));
      }
    for (int v = 0; v < 8; ++v)
      for (int k = 0; k < 3; ++k) {
        double x = x0[k];
        for (int d = 0; d < 3; ++d)
          if (v & (1 << d)) x += ed[d][k];
        if (std::fabs(x - pts[c[v] * 3 + k]) > 1e-13 * scale) return false;
      }
  }
  return true;
}

// True when every element is a box whose edges from vertex 0 (to vertices 1,
// 2 and 4) each have exactly one nonzero coordinate difference, on distinct
// axes: the Jacobian from those edges is a permuted diagonal matrix.
bool mesh_is_axis_aligned(const double *pts, const int64_t *cv, int64_t E) {
  for (int64_t e = 0; e < E; ++e) {
    const int64_t *c = cv + e * 8;
    int axes = 0;
    for (int d = 0; d < 3; ++d) {
      int nz = 0, ax = 0;
      for (int k = 0; k < 3; ++k)
        if (pts[c[1 << d] * 3 + k] - pts[c[0] * 3 + k] != 0.0) ++nz, ax = k;
      if (nz != 1 || (axes & (1 << ax))) return false;
      axes |= 1 << ax;
    }
  }
  return true;
}

// Reference tensors (long double sums over the Gauss points of the
// reference-tabulated values) and the upper-triangle entry list.
void build_affine_hex_tables(Plan &P) {
  const int nb = P.nb, nq = P.nq;
  const int pm[6][2] = {{0, 0}, {1, 1}, {2, 2}, {0, 1}, {0, 2}, {1, 2}};
  P.h_aff.assign(size_t(kAffTables) * nb * nb, 0.0);
  std::vector<long double> acc(size_t(nb) * nb);
  for (int p = 0; p < kAffTables; ++p) {
    std::fill(acc.begin(), acc.end(), 0.0L);
    for (int q = 0; q < nq; ++q) {
      const long double w = P.h_w[q];
      const double *g = &P.h_grad[size_t(q) * nb * 3];
      const double *v = &P.h_val[size_t(q) * nb];
      for (int i = 0; i < nb; ++i)
        for (int j = 0; j < nb; ++j) {
          long double t;
          if (p == 6) {
            t = (long double)v[i] * v[j];
          } else {
            const int m = pm[p][0], n = pm[p][1];
            t = (long double)g[i * 3 + m] * g[j * 3 + n];
            if (m != n) t += (long double)g[i * 3 + n] * g[j * 3 + m];
          }
          acc[size_t(i) * nb + j] += w * t;
        }
    }
    for (size_t k = 0; k < acc.size(); ++k) P.h_aff[size_t(p) * nb * nb + k] = double(acc[k]);
  }
  P.h_tri.clear();
  for (int r = 0; r < nb; ++r)
    for (int c = r; c < nb; ++c) P.h_tri.push_back((r << 16) | c);
  const int s = nb;
  P.lay.nb = nb;
  P.lay.qd = 1;
  P.lay.s = s;
  P.lay.rowstride = (s + 3) & ~3;
  P.lay.off_vec = s * P.lay.rowstride;
  P.lay.off_thr = P.lay.off_vec + P.lay.rowstride;
  P.lay.stride = P.lay.off_thr + 4;
  P.lay.blk = 0;
  P.lay.rowblk = P.lay.rowstride;
  P.lay.linear = true;
}

bool affine_hex_available(int degree) { return degree == 1 || degree == 2 || degree == 3 || degree == 4; }

namespace {

// The 1D tables of the sum factorisation, checked against the 3-D tables
// (values and gradients at every Gauss point): false (no sum factorisation)
// if the basis or the rule does not factor to 1e-9.  *exact: they agree to
// 1e-14 (values) / 1e-13 (gradients).  The reference evaluates the QK basis
// from its expanded monomial coefficients; for K >= 3 that evaluation is off
// the exact tensor product by 1e-12 (K = 3) to 1.5e-10 (K = 4), so only
// K <= 2 reproduces the reference's sums to its own rounding.
template <int P1, int Q1>
bool make_sumfac(const Plan &P, int K1d, std::vector<double> &blob, bool *exact) {
  SumFac<P1, Q1> t{};
  RefElement e1(1, SIMPLEX, P1 - 1), e3(3, HEX, P1 - 1);
  Quadrature q1;
  if (!quadrature_by_name("IM_GAUSS1D(" + std::to_string(K1d) + ")", q1) || q1.nq != Q1 ||
      e1.nb != P1 || e3.nb != P1 * P1 * P1 || P.nq != Q1 * Q1 * Q1)
    return false;
  for (int q = 0; q < Q1; ++q) {
    double v[P1], g[P1];
    e1.eval(&q1.pts[q], v, g);
    for (int j = 0; j < P1; ++j) {
      const int a = e1.lattice[j];
      t.N[q][a] = v[j];
      t.D[q][a] = g[j];
    }
    t.w[q] = q1.w[q];
  }
  for (int i = 0; i < e3.nb; ++i)
    t.perm[i] = e3.lattice[i * 3] + P1 * (e3.lattice[i * 3 + 1] + P1 * e3.lattice[i * 3 + 2]);
  // the 3-D rule is the tensor product, first coordinate fastest
  double ev = 0.0, eg = 0.0;
  for (int q = 0; q < P.nq; ++q) {
    const int qx = q % Q1, qy = (q / Q1) % Q1, qz = q / (Q1 * Q1);
    if (std::fabs(P.h_w[q] - t.w[qx] * t.w[qy] * t.w[qz]) > 1e-15) return false;
    for (int i = 0; i < e3.nb; ++i) {
      const int a = e3.lattice[i * 3], b = e3.lattice[i * 3 + 1], c = e3.lattice[i * 3 + 2];
      const double v = t.N[qx][a] * t.N[qy][b] * t.N[qz][c];
      const double g[3] = {t.D[qx][a] * t.N[qy][b] * t.N[qz][c],
                           t.N[qx][a] * t.D[qy][b] * t.N[qz][c],
                           t.N[qx][a] * t.N[qy][b] * t.D[qz][c]};
      ev = std::max(ev, std::fabs(v - P.h_val[size_t(q) * P.nb + i]));
      for (int d = 0; d < 3; ++d)
        eg = std::max(eg, std::fabs(g[d] - P.h_grad[(size_t(q) * P.nb + i) * 3 + d]));
    }
  }
  if (ev > 1e-9 || eg > 1e-8) return false;
  *exact = ev <= 1e-14 && eg <= 1e-13;
  blob.assign((sizeof(t) + 7) / 8, 0.0);
  std::memcpy(blob.data(), &t, sizeof(t));
  return true;
}

}  // namespace

// Sum-factorisation tables of a parallelepiped plan (P.h_sf; empty if the
// element / rule pair is not one of the instantiated ones or does not factor).
void build_affine_hex_sumfac(Plan &P) {
  P.h_sf.clear();
  int N = 0, K = 0;
  if (sscanf(P.im.c_str(), "IM_GAUSS_PARALLELEPIPED(%d,%d)", &N, &K) != 2 || N != 3) return;
  const int P1 = P.degree + 1, Q1 = K / 2 + 1;
  bool ok = false, exact = false;
  if (P1 == 2 && Q1 == 2) ok = make_sumfac<2, 2>(P, K, P.h_sf, &exact);
  else if (P1 == 2 && Q1 == 3) ok = make_sumfac<2, 3>(P, K, P.h_sf, &exact);
  else if (P1 == 3 && Q1 == 3) ok = make_sumfac<3, 3>(P, K, P.h_sf, &exact);
  else if (P1 == 4 && Q1 == 4) ok = make_sumfac<4, 4>(P, K, P.h_sf, &exact);
  else if (P1 == 5 && Q1 == 5) ok = make_sumfac<5, 5>(P, K, P.h_sf, &exact);
  if (!ok) P.h_sf.clear();
  P.sf_exact = ok && exact;
}

cudaError_t launch_affine_hex_pass(Plan &P, bool want_K) {
  if (P.n_elements == 0) return cudaSuccess;
  SlotPtrs sp;
  for (int i = 0; i < GFGPU_MAX_SLOTS; ++i) sp.p[i] = P.slot_ptr[i];
  if (P.slot_n[GFGPU_SLOT_U] != P.n_dof) sp.p[GFGPU_SLOT_U] = nullptr;
  const unsigned grid = unsigned(P.n_elements);
  if (!want_K && P.d_sf && (P.sf_exact || P.sf_requested)) {
    // vector only: sum factorisation
    bool hasv = false;
    for (int t = 0; t < P.form.n_terms; ++t)
      hasv |= P.form.terms[t].kind == GFGPU_TERM_MASS || P.form.terms[t].kind == GFGPU_TERM_SOURCE;
    const int P1 = P.degree + 1, Q1 = int(std::lround(std::cbrt(double(P.nq))));
#define SFK(A, B)                                                                               \
  do {                                                                                         \
    const auto *tab = reinterpret_cast<const SumFac<A, B> *>(P.d_sf);                          \
    if (hasv)                                                                                  \
      affine_hex_apply_kernel<A, B, true><<<grid, kSfThreads, 0, P.stream>>>(                   \
          P.n_elements, P.d_points, P.d_cv, P.d_enode, tab, P.d_ggrad, P.lay, P.form, sp,     \
          P.d_elem, P.d_err);                                                                  \
    else                                                                                       \
      affine_hex_apply_kernel<A, B, false><<<grid, kSfThreads, 0, P.stream>>>(                  \
          P.n_elements, P.d_points, P.d_cv, P.d_enode, tab, P.d_ggrad, P.lay, P.form, sp,     \
          P.d_elem, P.d_err);                                                                  \
  } while (0)
    if (P1 == 2 && Q1 == 2) SFK(2, 2);
    else if (P1 == 2 && Q1 == 3) SFK(2, 3);
    else if (P1 == 3 && Q1 == 3) SFK(3, 3);
    else if (P1 == 4 && Q1 == 4) SFK(4, 4);
    else if (P1 == 5 && Q1 == 5) SFK(5, 5);
    else return cudaErrorInvalidValue;
#undef SFK
    P.launches++;
    return cudaGetLastError();
  }
  if (!want_K) {
    // a GRADGRAD-only form: the vector through the reference tensors, several
    // elements per block
    bool gg = P.form.n_terms > 0;
    for (int t = 0; t < P.form.n_terms; ++t) gg &= P.form.terms[t].kind == GFGPU_TERM_GRADGRAD;
    if (gg) {
#define APK(NBV, NPV, EQV)                                                                    \
  affine_scalar_apply_kernel<NBV, NPV, EQV>                                                  \
      <<<unsigned((P.n_elements + EQV - 1) / EQV), 128, 0, P.stream>>>(                     \
          P.n_elements, P.d_points, P.d_cv, P.d_enode, P.d_aff, P.lay, P.form, sp, P.d_elem, \
          P.d_err)
#define APN(NBV)          \
  do {                    \
    if (P.axis_aligned)   \
      APK(NBV, 3, 8);     \
    else                  \
      APK(NBV, 6, 4);     \
  } while (0)
      switch (P.nb) {
        case 8: APN(8); break;
        case 27: APN(27); break;
        case 64: APN(64); break;
        case 125: APN(125); break;
        default: return cudaErrorInvalidValue;
      }
#undef APN
#undef APK
      P.launches++;
      return cudaGetLastError();
    }
  }
  // the K pass with the plan's threads per element (autotuned)
  const int tk = P.tune.ep_threads;
#define AFFKX(NB, TT, AXV)                                                                     \
  affine_hex_kernel<NB, true, TT, AXV><<<grid, TT, 0, P.stream>>>(                             \
      P.n_elements, P.d_points, P.d_cv, P.d_enode, P.d_aff, P.d_tri, P.d_ggrad, P.lay, P.form, \
      sp, P.d_elem, P.d_err)
#define AFFK(NB, TT)              \
  do {                            \
    if (P.axis_aligned)           \
      AFFKX(NB, TT, true);        \
    else                          \
      AFFKX(NB, TT, false);       \
  } while (0)
#define AFF(NB)                                                                                \
  do {                                                                                         \
    if (want_K && tk == 128) AFFK(NB, 128);                                                    \
    else if (want_K && tk == 512) AFFK(NB, 512);                                               \
    else if (want_K) AFFK(NB, 256);                                                            \
    else                                                                                       \
      affine_hex_kernel<NB, false><<<grid, kAffThreads, 0, P.stream>>>(                         \
          P.n_elements, P.d_points, P.d_cv, P.d_enode, P.d_aff, P.d_tri, P.d_ggrad, P.lay,     \
          P.form, sp, P.d_elem, P.d_err);                                                      \
  } while (0)
  switch (P.nb) {
    case 8: AFF(8); break;
    case 27: AFF(27); break;
    case 64: AFF(64); break;
    case 125: AFF(125); break;
    default: return cudaErrorInvalidValue;
  }
#undef AFF
#undef AFFK
#undef AFFKX
  P.launches++;
  return cudaGetLastError();
}

}  // namespace gfgpu
