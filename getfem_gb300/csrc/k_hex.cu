// Gauss-point element kernel for 3-D elements (GT_QK(3,1) + FEM_QK(3,K)
// hexahedra, GT_PK(3,1) + FEM_PK(3,K) tetrahedra), FP64.
//
// The reference's exec loop (getfem_generic_assembly_compile_and_exec.cc:
// 8750-8869) for one element per CTA, with the Gauss points processed in
// parallel where the reference processes them in sequence:
//
//  A1  one thread per Gauss point q: K = sum_v x_v grad(phi_geo_v)(q),
//      J = |det K|, B = K^{-T} (bgeot_geometric_trans.cc:270-413), real
//      gradients g_qj = B grad_ref(phi_j)(q) (getfem_fem.cc:160-200) and
//      Grad_u.  Isotropic forms: the pointwise tangent
//        A[a,k,b,l] = c0 d_ak d_bl + c1 d_ab d_kl + c2 d_al d_kb
//      with the coefficients at q (constant, per element or nodal), the
//      stress P = A:Grad_u, the mass and load factors.  Neo-Hookean:
//      F = I + Grad_u, C = F^T F and the law's state at q.
//  A2  (neo-Hookean) all threads: dS/dE (81 entries per q) from that state,
//      the law of getfem_nonlinear_elasticity.cc:503-600 with the
//      compressible neo-Hookean switches of :1770-1838.
//  A3  (neo-Hookean) all threads: A[a,k,b,l] = d_ab S_lk +
//      sum_mn F_am F_bn dS_mk/dE_nl, the derivative of F S(E) in Grad_u.
//  B   per q, all threads: Z[(a,k),(j,b)] = sum_l A[a,k,b,l] g_jl in shared
//      memory, then each thread adds sum_k g_ik Z[(a,k),(j,b)] to the
//      element-matrix entries it owns (registers).
//  C   R_e[(i,a)] = sum_q P_q[a,k] g_qik (+ mass, load).
//
// An internal im_data pressure (GFGPU_TERM_INTERNAL_P) lives at the Gauss
// points, so its block K_pp of the element matrix is diagonal, one scalar per
// point, and the reference's element-level static condensation
// (compile_and_exec.cc:5562-5790: invert KQQ, KQJpr = KQQ^-1 KQJ, RQpr =
// KQQ^-1 R_Q / coeff, K_IJ -= K_IQ KQJpr, R_I -= K_IQ RQpr) reduces to a
// per-point Schur complement done in A1: with K_up = c0 Div(Test_u),
// K_pu = scale k Div_u and K_pp = scale (1 + 3 c2 p^2), the condensed
// tangent adds -c0 k / (1 + 3 c2 p^2) to the isotropic c0 d_ak d_bl part,
// the condensed residual is -c0 RQpr Div(Test_u) per point, and the
// coupling rows KQJpr = k / (1 + 3 c2 p^2) Div(phi_j) are written per point.
//
// All per-q quantities are scaled by w_q J.  Output: the element scratch
// layout read by the pattern build and the row gather (K_e rows, V_e = R_e,
// threshold 1e-14 max|K_e|).
#include <cmath>

#include "host/refelem.h"
#include "k_common.cuh"
#include "plan.h"

namespace gfgpu {

namespace {

constexpr int kHexThreads = 256;
constexpr int kLaw = 40;  // per-q neo-Hookean state for the tangent (doubles)
constexpr int kRes = 36;  // per-q residual state (doubles)

// neo-Hookean state offsets
enum { LF = 0, LS = 9, LCI = 18, LI1 = 27, LI3, LP13, LDD, LC1, LD1, LWJ, LK1, LK2, LA22 };
// residual state offsets: neo-Hookean F S (9) and the term scale; isotropic
// Grad_u (row-major, 9), div, then 3 values per term
enum { RFS = 0, RSC = 9, RGU = 0, RDIV = 9, RTERM = 10 };

// This file is compiled with -fmad=false: the geometry, the law and the
// residual round like the reference's sequence of products and sums (the
// neo-Hookean stress near F = I is a difference of nearly equal terms, so
// contracted roundings would show up in the residual).  The element-matrix
// contraction uses explicit fma().

// 3x3 inverse by cofactors, divided by the determinant (column-major).
__device__ __forceinline__ void inv3d(const double *A, double *Ai, double &det) {
  const double a0 = A[4] * A[8] - A[5] * A[7];
  const double a1 = A[5] * A[6] - A[3] * A[8];
  const double a2 = A[3] * A[7] - A[4] * A[6];
  det = A[0] * a0 + A[1] * a1 + A[2] * a2;
  double c[9];
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      const int i1 = (i + 1) % 3, i2 = (i + 2) % 3, j1 = (j + 1) % 3, j2 = (j + 2) % 3;
      c[i + 3 * j] = A[i1 + 3 * j1] * A[i2 + 3 * j2] - A[i1 + 3 * j2] * A[i2 + 3 * j1];
    }
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) Ai[i + 3 * j] = c[j + 3 * i] / det;
}

__device__ __forceinline__ double coef_at(const gfgpu_coef &c, const SlotPtrs &slots, int64_t e,
                                          const int32_t *en, const double *phi, int nb) {
  if (c.kind == GFGPU_COEF_CONST) return c.value;
  if (c.kind == GFGPU_COEF_ELEMENT) return c.value * slots.p[c.slot][e];
  if (c.kind == GFGPU_COEF_NODAL) {
    double s = 0.0;
    for (int j = 0; j < nb; ++j) s += phi[j] * slots.p[c.slot][en[j]];
    return c.value * s;
  }
  return 0.0;
}

// dS_ij/dE_kl of the compressible neo-Hookean law from the state at q
// (coeff1 = 1/(3 i3), coeff2 = 4 coeff1^2 i1 and A22 = D1 / (2 |i3|^1.5) are
// computed once per point).
__device__ __forceinline__ double nh_dsde(const double *st, int i, int j, int k, int l) {
  const double *Ci = st + LCI;
  const double i1 = st[LI1], i3 = st[LI3], p13 = st[LP13], dd = st[LDD], C1 = st[LC1];
  const double coeff1 = st[LK1], coeff2 = st[LK2], A22 = st[LA22];
  const double dij = Ci[i + 3 * j] * i3, dkl = Ci[k + 3 * l] * i3;
  const double ddi3 = i3 / 2.0 *
                      (Ci[j + 3 * i] * Ci[l + 3 * k] - Ci[j + 3 * k] * Ci[l + 3 * i] +
                       Ci[i + 3 * j] * Ci[l + 3 * k] - Ci[i + 3 * k] * Ci[l + 3 * j]);
  const double ddj1 = (-i1 * coeff1 * ddi3 + dij * dkl * coeff2 -
                       ((i == j ? 1.0 : 0.0) * dkl + (k == l ? 1.0 : 0.0) * dij) * coeff1) *
                      p13;
  return 4.0 * C1 * ddj1 + 4.0 * dd * ddi3 + 4.0 * A22 * dij * dkl;
}

template <int QD, int NB, int NBG, int NQ, int LAW>
struct HexSmem {
  static constexpr int S = NB * QD, NA = 3 * QD;
  static constexpr int n_g = NQ * NB * 3, n_A = NQ * NA * NA, n_c = NQ, n_m = NQ,
                       n_r = NQ * kRes, n_u = S, n_x = NBG * 3;
  static constexpr int n_law = LAW == LAW_NH ? NQ * kLaw : 0;
  // phase B builds Z for kQG Gauss points at a time (fewer block barriers)
  static constexpr int kQG = 3;
  static constexpr int n_Z = kQG * NA * S, n_GS = LAW == LAW_NH ? NQ * 81 : 0;
  static constexpr int n_W = n_Z > n_GS ? n_Z : n_GS;
  static constexpr int o_g = 0, o_A = o_g + n_g, o_c = o_A + n_A, o_m = o_c + n_c,
                       o_r = o_m + n_m, o_u = o_r + n_r, o_x = o_u + n_u, o_law = o_x + n_x,
                       o_W = o_law + n_law, total = o_W + n_W;
  static constexpr size_t bytes = size_t(total) * 8;
  // phase B: the upper triangle of K_e (r <= c), entries dealt round-robin
  static constexpr int NT = S * (S + 1) / 2;
};

// T threads per element (the CTA of the element): every entry of K_e, every
// Z product and every row of the residual is computed by one thread in the
// same order whatever T is, so the results are the same bits for every T.
template <int QD, int NB, int NBG, int NQ, int LAW, bool WANT_K, int T = kHexThreads>
__global__ void __launch_bounds__(T, 512 / T) hex_element_kernel(
    int64_t E, const double *__restrict__ pts, const int32_t *__restrict__ cv,
    const int32_t *__restrict__ enode, const double *__restrict__ hval,
    const double *__restrict__ hgrad, const double *__restrict__ ggrad,
    const double *__restrict__ hw, const int32_t *__restrict__ tri, KeLayout L,
    gfgpu_form form, SlotPtrs slots, double *__restrict__ out, int *__restrict__ err,
    int ipt, int cmode, double *__restrict__ out_int, double *__restrict__ out_kqj) {
  using M = HexSmem<QD, NB, NBG, NQ, LAW>;
  constexpr int S = M::S, NA = M::NA;
  extern __shared__ __align__(16) double sm[];
  double *gq = sm + M::o_g;   // [q][j][d] real gradients
  double *Aq = sm + M::o_A;   // [q][ak][bl] w J A
  double *cq = sm + M::o_c;   // [q] w J
  double *mq = sm + M::o_m;   // [q] w J (mass coefficient)
  double *rq = sm + M::o_r;   // [q][kRes] residual state
  double *us = sm + M::o_u;   // [j*QD + a]
  double *xs = sm + M::o_x;   // [v][d]
  double *law = sm + M::o_law;
  double *W = sm + M::o_W;    // dS/dE [q][81] in A2-A3, then Z [ak][c] in B
  __shared__ int32_t ens[NB];
  __shared__ unsigned long long smax;
  const int64_t e = blockIdx.x;
  const int tid = threadIdx.x;
  if (tid < NBG * 3) xs[tid] = pts[int64_t(cv[e * NBG + tid / 3]) * 3 + tid % 3];
  if (tid < NB) ens[tid] = enode[e * NB + tid];
  if (tid == 0) smax = 0ull;
  __syncthreads();
  const double *u = slots.p[GFGPU_SLOT_U];
  for (int c = tid; c < S; c += T)
    us[c] = u ? u[int64_t(ens[c / QD]) * QD + c % QD] : 0.0;
  __syncthreads();
  // ---------------------------------------------------------------- A1
  for (int q = tid; q < NQ; q += T) {
    double K[9];
#pragma unroll
    for (int d = 0; d < 3; ++d)
#pragma unroll
      for (int m = 0; m < 3; ++m) {
        double s = 0.0;
#pragma unroll
        for (int v = 0; v < NBG; ++v) s += xs[v * 3 + d] * ggrad[(q * NBG + v) * 3 + m];
        K[d + 3 * m] = s;
      }
    double Ki[9], det;
    inv3d(K, Ki, det);
    const bool bad = det == 0.0;
    if (bad) set_err(err, ERR_JACOBIAN);
    const double wJ = bad ? 0.0 : fabs(det) * hw[q];
    cq[q] = wJ;
    double Gu[QD][3];
#pragma unroll
    for (int a = 0; a < QD; ++a) Gu[a][0] = Gu[a][1] = Gu[a][2] = 0.0;
    for (int j = 0; j < NB; ++j) {
      const double *hg = hgrad + (q * NB + j) * 3;
      const double r0 = hg[0], r1 = hg[1], r2 = hg[2];
      double gj[3];
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        // B(d,m) = Ki(m,d)
        gj[d] = bad ? 0.0 : Ki[3 * d] * r0 + Ki[1 + 3 * d] * r1 + Ki[2 + 3 * d] * r2;
        gq[(q * NB + j) * 3 + d] = gj[d];
      }
#pragma unroll
      for (int a = 0; a < QD; ++a)
#pragma unroll
        for (int d = 0; d < 3; ++d) Gu[a][d] += us[j * QD + a] * gj[d];
    }
    const double *phi = hval + q * NB;
    double *rs = rq + q * kRes;
    if constexpr (LAW == LAW_NH) {
      double C1 = 0.0, D1 = 0.0, sc = 0.0;
      for (int t = 0; t < form.n_terms; ++t)
        if (form.terms[t].kind == GFGPU_TERM_NEOHOOKEAN) {
          C1 = coef_at(form.terms[t].c[0], slots, e, ens, phi, NB);
          D1 = coef_at(form.terms[t].c[1], slots, e, ens, phi, NB);
          sc = form.terms[t].scale;
        }
      double *st = law + q * kLaw;
      double F[9], C[9];
#pragma unroll
      for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) {
          double s = 0.0;
#pragma unroll
          for (int m = 0; m < 3; ++m) s += Gu[m][i] * Gu[m][j];
          // C = I + 2E with E = (Gu^T Gu + Gu + Gu^T) / 2
          C[i + 3 * j] = 2.0 * (0.5 * (s + Gu[i][j] + Gu[j][i])) + (i == j ? 1.0 : 0.0);
          F[i + 3 * j] = Gu[i][j] + (i == j ? 1.0 : 0.0);
        }
      const double detF = F[0] * (F[4] * F[8] - F[5] * F[7]) - F[3] * (F[1] * F[8] - F[2] * F[7]) +
                          F[6] * (F[1] * F[5] - F[2] * F[4]);
      double Ci[9], i3;
      inv3d(C, Ci, i3);
      const double i1 = C[0] + C[4] + C[8];
      const double p13 = pow(fabs(i3), -1.0 / 3.0);
      const double dd = D1 - D1 / sqrt(fabs(i3));
      double Sm[9];
#pragma unroll
      for (int k = 0; k < 9; ++k) {
        const double di3 = Ci[k] * i3;
        const double dj1 = ((k % 4 == 0 ? 1.0 : 0.0) - i1 / (3.0 * i3) * di3) * p13;
        Sm[k] = 2.0 * C1 * dj1 + 2.0 * dd * di3;
        if (detF <= 0.0) Sm[k] += 1e200 * C[k];
      }
#pragma unroll
      for (int k = 0; k < 9; ++k) {
        st[LF + k] = F[k];
        st[LS + k] = Sm[k];
        st[LCI + k] = Ci[k];
      }
      st[LI1] = i1, st[LI3] = i3, st[LP13] = p13, st[LDD] = dd, st[LC1] = C1, st[LD1] = D1;
      {
        const double coeff1 = 1.0 / (3.0 * i3);
        st[LK1] = coeff1;
        st[LK2] = 4.0 * coeff1 * coeff1 * i1;
        st[LA22] = D1 / (2.0 * pow(fabs(i3), 1.5));
      }
      st[LWJ] = wJ * sc;
#pragma unroll
      for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int k = 0; k < 3; ++k) {
          double s = 0.0;
#pragma unroll
          for (int m = 0; m < 3; ++m) s += F[a + 3 * m] * Sm[m + 3 * k];
          rs[RFS + a * 3 + k] = s;
        }
      rs[RSC] = sc;
      mq[q] = 0.0;
    } else {
      // tangent: coefficients summed over the terms; residual: one record
      // per term, evaluated in term order in phase C
      double c0 = 0, c1 = 0, c2 = 0, cm = 0;
#pragma unroll
      for (int a = 0; a < QD; ++a)
#pragma unroll
        for (int d = 0; d < 3; ++d) rs[RGU + a * 3 + d] = Gu[a][d];
      double div = 0.0;
#pragma unroll
      for (int a = 0; a < QD; ++a) div += Gu[a][a < 3 ? a : 0];
      rs[RDIV] = div;
      for (int t = 0; t < form.n_terms; ++t) {
        const gfgpu_term &Tm = form.terms[t];
        double *tv = rs + RTERM + 3 * t;
        const double sc = Tm.scale;
        if (Tm.kind == GFGPU_TERM_GRADGRAD) {
          const double a0 = coef_at(Tm.c[0], slots, e, ens, phi, NB) * sc;
          const double a1 = coef_at(Tm.c[1], slots, e, ens, phi, NB) * sc;
          const double a2 = coef_at(Tm.c[2], slots, e, ens, phi, NB) * sc;
          tv[0] = a0, tv[1] = a1, tv[2] = a2;
          c0 += a0, c1 += a1, c2 += a2;
        } else if (Tm.kind == GFGPU_TERM_MASS) {
          const double a0 = coef_at(Tm.c[0], slots, e, ens, phi, NB) * sc;
          cm += a0;
          double uq[QD];
#pragma unroll
          for (int b = 0; b < QD; ++b) uq[b] = 0.0;
          for (int j = 0; j < NB; ++j)
#pragma unroll
            for (int b = 0; b < QD; ++b) uq[b] += phi[j] * us[j * QD + b];
#pragma unroll
          for (int b = 0; b < QD; ++b) tv[b] = a0 * uq[b];
        } else if (Tm.kind == GFGPU_TERM_INTERNAL_P) {
          // the internal pressure at this Gauss point (im_data index e*NQ+q)
          const double sp = coef_at(Tm.c[0], slots, e, ens, phi, NB);
          const double kb = coef_at(Tm.c[1], slots, e, ens, phi, NB);
          const double c3 = coef_at(Tm.c[2], slots, e, ens, phi, NB);
          const int64_t iq = e * NQ + q;
          const double p = slots.p[Tm.field_slot][iq];
          if (cmode == 2) {
            // K_pp^-1, then KQJpr and RQpr as the reference forms them
            const double inv = 1.0 / (sc * (1.0 + c3 * (3.0 * (p * p))));
            if (!isfinite(inv)) set_err(err, ERR_NAN);
            const double kq = inv * (sc * kb);
            const double rqpr = bad ? 0.0 : (inv * slots.p[Tm.aux_slot][iq]) / wJ;
            c0 += -(sp * kq);
            tv[0] = -(sp * rqpr);
            tv[1] = kq;
            out_int[iq] = rqpr;
          } else {
            tv[0] = sp * p;
            tv[1] = 0.0;
            out_int[iq] = wJ * (sc * ((p + c3 * (p * p * p)) + kb * div));
          }
        } else if (Tm.kind == GFGPU_TERM_SOURCE) {
          const double a0 =
              (Tm.c[0].kind == GFGPU_COEF_NONE ? 1.0 : coef_at(Tm.c[0], slots, e, ens, phi, NB)) * sc;
          const double *f = slots.p[Tm.field_slot];
          double fv[QD];
#pragma unroll
          for (int b = 0; b < QD; ++b) fv[b] = 0.0;
          for (int j = 0; j < NB; ++j)
#pragma unroll
            for (int b = 0; b < QD; ++b) fv[b] += phi[j] * f[int64_t(ens[j]) * QD + b];
#pragma unroll
          for (int b = 0; b < QD; ++b) tv[b] = a0 * fv[b];
        }
      }
#pragma unroll
      for (int a = 0; a < QD; ++a)
#pragma unroll
        for (int k = 0; k < 3; ++k)
#pragma unroll
          for (int b = 0; b < QD; ++b)
#pragma unroll
            for (int l = 0; l < 3; ++l) {
              double v = (a == b && k == l) ? c1 : 0.0;
              if constexpr (QD == 3)
                v += (a == k && b == l ? c0 : 0.0) + (a == l && k == b ? c2 : 0.0);
              Aq[(q * NA + a * 3 + k) * NA + b * 3 + l] = wJ * v;
            }
      mq[q] = wJ * cm;
    }
  }
  __syncthreads();
  if constexpr (LAW == LAW_ISO && QD == 3) {
    // coupling rows KQJpr(e*NQ + q, (j, b)) = kq_q g_qjb: with QD == 3 the
    // row entry (j, b) of point q is gq[q*S + j*3 + b]
    if (cmode == 2 && ipt >= 0) {
      double *ok = out_kqj + e * (NQ * S);
      for (int z = tid; z < NQ * S; z += T)
        ok[z] = rq[(z / S) * kRes + RTERM + 3 * ipt + 1] * gq[z];
    }
  }
  if constexpr (LAW == LAW_NH && WANT_K) {
    // ---------------------------------------------------------------- A2
    for (int z = tid; z < NQ * 81; z += T) {
      const int q = z / 81, r = z % 81;
      W[z] = nh_dsde(law + q * kLaw, r % 3, (r / 3) % 3, (r / 9) % 3, r / 27);
    }
    __syncthreads();
    // ---------------------------------------------------------------- A3
    for (int z = tid; z < NQ * 81; z += T) {
      const int q = z / 81, r = z % 81, ak = r / 9, bl = r % 9;
      const int a = ak / 3, k = ak % 3, b = bl / 3, l = bl % 3;
      const double *st = law + q * kLaw;
      const double *gs = W + q * 81;
      double v = (a == b) ? st[LS + l + 3 * k] : 0.0;
#pragma unroll
      for (int m = 0; m < 3; ++m) {
        double h = 0.0;
#pragma unroll
        for (int n = 0; n < 3; ++n) h = fma(st[LF + b + 3 * n], gs[m + 3 * k + 9 * n + 27 * l], h);
        v = fma(st[LF + a + 3 * m], h, v);
      }
      Aq[z] = st[LWJ] * v;
    }
    __syncthreads();
  }
  double *o = out + e * L.stride;
  if constexpr (WANT_K) {
    // -------------------------------------------------------------- B
    // K_e is symmetric (isotropic tangent; hyperelastic tangent): each thread
    // owns upper-triangle entries (r, c), r = i*QD + a <= c = j*QD + b, and
    // accumulates sum_k g_ik Z[(a,k), c] with Z = A g_j per Gauss point.
    constexpr int NE = (M::NT + T - 1) / T;
    int goff[NE], zoff[NE];
    bool own[NE], dg[NE];
#pragma unroll
    for (int k = 0; k < NE; ++k) {
      const int ent = tid + T * k;
      own[k] = ent < M::NT;
      const int rc = own[k] ? tri[ent] : 0;
      const int r = rc >> 16, c = rc & 0xffff;
      goff[k] = (r / QD) * 3;
      zoff[k] = (r % QD) * 3 * S + c;
      dg[k] = (c % QD) == (r % QD);  // mass couples equal components
    }
    double acc[NE];
#pragma unroll
    for (int k = 0; k < NE; ++k) acc[k] = 0.0;
    constexpr int QG = M::kQG, NZ = NA * S;
    for (int q0 = 0; q0 < NQ; q0 += QG) {
      const int nqg = NQ - q0 < QG ? NQ - q0 : QG;
      for (int z = tid; z < nqg * NZ; z += T) {
        const int t = z / NZ, zz = z - t * NZ, q = q0 + t;
        const int ak = zz / S, cz = zz % S, j = cz / QD, b = cz % QD;
        const double *A = Aq + (q * NA + ak) * NA + b * 3;
        const double *gz = gq + (q * NB + j) * 3;
        W[z] = fma(A[0], gz[0], fma(A[1], gz[1], A[2] * gz[2]));
      }
      __syncthreads();
      for (int t = 0; t < nqg; ++t) {
        const int q = q0 + t;
        const double *gi = gq + q * NB * 3;
        const double *Wt = W + t * NZ;
#pragma unroll
        for (int k = 0; k < NE; ++k) {
          if (own[k]) {
            const double *g = gi + goff[k];
            const double *Z = Wt + zoff[k];
            double v = fma(g[0], Z[0], acc[k]);
            v = fma(g[1], Z[S], v);
            acc[k] = fma(g[2], Z[2 * S], v);
          }
        }
        const double mqq = mq[q];
        if (mqq != 0.0) {
          const double *phi = hval + q * NB;
#pragma unroll
          for (int k = 0; k < NE; ++k) {
            if (own[k] && dg[k]) {
              const int ent = tid + T * k;
              const int rc = tri[ent];
              acc[k] = fma(mqq * phi[(rc >> 16) / QD], phi[(rc & 0xffff) / QD], acc[k]);
            }
          }
        }
      }
      __syncthreads();
    }
    // ------------------------------------------------------------ outputs
    unsigned long long mx = 0ull;
#pragma unroll
    for (int k = 0; k < NE; ++k) {
      if (own[k]) {
        const int rc = tri[tid + T * k];
        const int r = rc >> 16, c = rc & 0xffff;
        o[r * L.rowstride + c] = acc[k];
        if (r != c) o[c * L.rowstride + r] = acc[k];
        const unsigned long long bits = abs_key(acc[k]);
        mx = bits > mx ? bits : mx;
      }
    }
    atomicMax(&smax, mx);
  }
  // ---------------------------------------------------------------- C
  // R_e(i,a) = sum_q wJ_q t_q(i,a), t_q as the reference's exec loop forms
  // it (term by term, products and sums in its order)
  for (int r = tid; r < S; r += T) {
    const int i = r / QD, ra = r % QD;
    double s = 0.0;
    for (int q = 0; q < NQ; ++q) {
      const double *g = gq + (q * NB + i) * 3;
      const double *rs = rq + q * kRes;
      double t = 0.0;
      if constexpr (LAW == LAW_NH) {
        double v = 0.0;
#pragma unroll
        for (int k = 0; k < 3; ++k) v += rs[RFS + ra * 3 + k] * g[k];
        t = rs[RSC] * v;
      } else {
        const double phi_i = hval[q * NB + i];
        for (int tt = 0; tt < form.n_terms; ++tt) {
          const int kind = form.terms[tt].kind;
          const double *tv = rs + RTERM + 3 * tt;
          if (kind == GFGPU_TERM_INTERNAL_P) {
            // order 1: p Div(Test_u); condensation: -c0 RQpr Div(Test_u)
            t += tv[0] * g[ra];
          } else if (cmode == 2) {
            // the condensed vector holds the condensation terms only
          } else if (kind == GFGPU_TERM_GRADGRAD) {
            double v = 0.0;
#pragma unroll
            for (int k = 0; k < 3; ++k) {
              double Dk = tv[1] * rs[RGU + ra * 3 + k];
              if constexpr (QD > 1)
                Dk += (k == ra ? tv[0] * rs[RDIV] : 0.0) + tv[2] * rs[RGU + k * 3 + ra];
              v += Dk * g[k];
            }
            t += v;
          } else {
            t += tv[ra] * phi_i;
          }
        }
      }
      s += cq[q] * t;
    }
    if (!isfinite(s)) set_err(err, ERR_NAN);
    o[L.off_vec + r] = s;
  }
  if constexpr (WANT_K) {
    __syncthreads();
    if (tid == 0) {
      const double m = abs_of_key(smax);
      if (!isfinite(m)) set_err(err, ERR_NAN);
      o[L.off_thr] = m * 1e-14;
    }
  }
}

template <int QD, int NB, int NBG, int NQ, int LAW>
cudaError_t launch_hex_t(Plan &P, const SlotPtrs &sp, bool want_K) {
  using M = HexSmem<QD, NB, NBG, NQ, LAW>;
  // threads per element: the plan's (autotuned) for the K pass, the
  // default for a vector-only pass
  const int T = want_K ? P.tune.ep_threads : kHexThreads;
  auto kern = !want_K ? hex_element_kernel<QD, NB, NBG, NQ, LAW, false>
              : T == 128 ? hex_element_kernel<QD, NB, NBG, NQ, LAW, true, 128>
              : T == 512 ? hex_element_kernel<QD, NB, NBG, NQ, LAW, true, 512>
                         : hex_element_kernel<QD, NB, NBG, NQ, LAW, true, 256>;
  const int threads = !want_K ? kHexThreads : (T == 128 || T == 512) ? T : 256;
  cudaError_t ce = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        int(M::bytes));
  if (ce != cudaSuccess) return ce;
  kern<<<unsigned(P.n_elements), threads, M::bytes, P.stream>>>(
      P.n_elements, P.d_points, P.d_cv, P.d_enode, P.d_hval, P.d_hgrad, P.d_ggrad, P.d_hw,
      P.d_tri, P.lay, P.form, sp, P.d_elem, P.d_err, P.ip_term, P.cmode, P.d_int, P.d_kqj);
  return cudaGetLastError();
}

}  // namespace

bool gauss_element_available(int kind, int law, int degree, int qdim, int nq) {
  if (kind == HEX) {
    const bool nq_ok = (degree == 1 && (nq == 8 || nq == 27)) || (degree == 2 && nq == 27);
    if (law == LAW_NH) return qdim == 3 && nq_ok;
    return (qdim == 1 || qdim == 3) && nq_ok;
  }
  // tetrahedra: the neo-Hookean law, and the isotropic forms of 3-D vector
  // fields that the simplex pass does not take (internal variables)
  return qdim == 3 && ((degree == 2 && nq == 15) || (degree == 1 && (nq == 4 || nq == 15)));
}

// Element scratch layout of the Gauss-point kernel.
void gauss_element_layout(Plan &P) {
  const int s = P.nb * P.qdim;
  P.lay.nb = P.nb;
  P.lay.qd = P.qdim;
  P.lay.s = s;
  P.lay.rowstride = (s + 3) & ~3;
  P.lay.off_vec = s * P.lay.rowstride;
  P.lay.off_thr = P.lay.off_vec + P.lay.rowstride;
  P.lay.stride = P.lay.off_thr + 4;
  P.lay.blk = 0;
  P.lay.rowblk = P.qdim * P.lay.rowstride;
  P.lay.linear = P.law != LAW_NH;
  // upper-triangle entries (r << 16 | c), row-major
  P.h_tri.clear();
  for (int r = 0; r < s; ++r)
    for (int c = r; c < s; ++c) P.h_tri.push_back((r << 16) | c);
}

cudaError_t launch_hex_element_pass(Plan &P, bool want_K) {
  if (P.n_elements == 0) return cudaSuccess;
  SlotPtrs sp;
  for (int i = 0; i < GFGPU_MAX_SLOTS; ++i) sp.p[i] = P.slot_ptr[i];
  // u is read for the residual whenever it is set; a u of another size is
  // treated as absent (the order-2 assembly of a linear form needs none)
  if (P.slot_n[GFGPU_SLOT_U] != P.n_dof) sp.p[GFGPU_SLOT_U] = nullptr;
  const int k = P.degree, q = P.qdim, nq = P.nq;
  cudaError_t ce = cudaErrorInvalidValue;
  if (P.kind != HEX) {
    if (P.law == LAW_NH && k == 2 && nq == 15) ce = launch_hex_t<3, 10, 4, 15, LAW_NH>(P, sp, want_K);
    else if (P.law == LAW_NH && k == 1 && nq == 4) ce = launch_hex_t<3, 4, 4, 4, LAW_NH>(P, sp, want_K);
    else if (P.law == LAW_NH && k == 1 && nq == 15) ce = launch_hex_t<3, 4, 4, 15, LAW_NH>(P, sp, want_K);
    else if (q == 3 && k == 2 && nq == 15) ce = launch_hex_t<3, 10, 4, 15, LAW_ISO>(P, sp, want_K);
    else if (q == 3 && k == 1 && nq == 4) ce = launch_hex_t<3, 4, 4, 4, LAW_ISO>(P, sp, want_K);
    else if (q == 3 && k == 1 && nq == 15) ce = launch_hex_t<3, 4, 4, 15, LAW_ISO>(P, sp, want_K);
  } else if (P.law == LAW_NH) {
    if (k == 2 && nq == 27) ce = launch_hex_t<3, 27, 8, 27, LAW_NH>(P, sp, want_K);
    else if (k == 1 && nq == 8) ce = launch_hex_t<3, 8, 8, 8, LAW_NH>(P, sp, want_K);
    else if (k == 1 && nq == 27) ce = launch_hex_t<3, 8, 8, 27, LAW_NH>(P, sp, want_K);
  } else if (q == 1) {
    if (k == 1 && nq == 8) ce = launch_hex_t<1, 8, 8, 8, LAW_ISO>(P, sp, want_K);
    else if (k == 1 && nq == 27) ce = launch_hex_t<1, 8, 8, 27, LAW_ISO>(P, sp, want_K);
    else if (k == 2 && nq == 27) ce = launch_hex_t<1, 27, 8, 27, LAW_ISO>(P, sp, want_K);
  } else if (q == 3) {
    if (k == 1 && nq == 8) ce = launch_hex_t<3, 8, 8, 8, LAW_ISO>(P, sp, want_K);
    else if (k == 1 && nq == 27) ce = launch_hex_t<3, 8, 8, 27, LAW_ISO>(P, sp, want_K);
    else if (k == 2 && nq == 27) ce = launch_hex_t<3, 27, 8, 27, LAW_ISO>(P, sp, want_K);
  }
  if (ce == cudaSuccess) P.launches++;
  return ce;
}

}  // namespace gfgpu
