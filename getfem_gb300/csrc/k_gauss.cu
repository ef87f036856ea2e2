// Potentials (order-0 assembly) and their adjoint gradients, FP64, for every
// element the plans take (GT_PK(N,1) + FEM_PK(N,1|2) simplices, GT_QK(3,1) +
// FEM_QK(3,1|2|4) hexahedra).
//
// Order 0 of the reference's exec loop (getfem_generic_assembly_compile_and_exec.cc:
// 8750-8869 with ga_instruction_scalar_assembly :4656-4667): E += t(q) J w_q
// over elements and Gauss points, t the scalar integrand.  Integrands:
//   GRADGRAD  D:Grad_u with D_ak = c1 Grad_u(a,k) + c0 div_u d_ak + c2 Grad_u(k,a)
//   MASS      c u.u        SOURCE  c f.u
//   NEOHOOKEAN W = C1 (j1 - 3) + D1 (sqrt|i3| - 1)^2, the strain energy of
//             getfem_nonlinear_elasticity.cc:503-527 (1e200 if det F <= 0).
//
// One warp per element, one lane per Gauss point (q = lane, lane + 32, ...).
// Three modes share the pointwise code:
//   MODE_ENERGY  per-element energy  E_e = sum_q w_q J psi(q)
//   MODE_COEF    derivative of E in one data slot: per element (element
//                coefficient) and per (element, local node) (nodal
//                coefficient); the node partials are gathered afterwards
//   MODE_SHAPE   derivative of E in the mesh vertex coordinates x_v, with the
//                DOF values held fixed: dE/dx_v[d] = sum_q w_q J (psi G_v[d] -
//                sum_{a,k} P[a,k] Grad_u(a,d) G_v[k]), G_v = B grad(phi_geo_v),
//                P = dpsi/dGrad_u; per (element, vertex), gathered per point.
// Per-element results are combined by deterministic reductions (fixed order).
#include <cmath>

#include "host/refelem.h"
#include "k_common.cuh"
#include "plan.h"

namespace gfgpu {

namespace {

constexpr int kGpWarps = 4;

template <int DIM>
__device__ __forceinline__ void geo_inverse(const double *K, double *B, double &det) {
  // B(d,m) = B[d + DIM m] = K^{-T}, as the reference's closed forms
  if constexpr (DIM == 2) {
    det = K[0] * K[3] - K[1] * K[2];
    B[0] = K[3] / det, B[1] = -K[2] / det, B[2] = -K[1] / det, B[3] = K[0] / det;
  } else {
    const double a0 = K[4] * K[8] - K[5] * K[7];
    const double a1 = K[5] * K[6] - K[3] * K[8];
    const double a2 = K[3] * K[7] - K[4] * K[6];
    det = K[0] * a0 + K[1] * a1 + K[2] * a2;
    double c[9];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) {
        const int i1 = (i + 1) % 3, i2 = (i + 2) % 3, j1 = (j + 1) % 3, j2 = (j + 2) % 3;
        c[i + 3 * j] = K[i1 + 3 * j1] * K[i2 + 3 * j2] - K[i1 + 3 * j2] * K[i2 + 3 * j1];
      }
    // Ki(i,j) = c(j,i) / det ; B(d,m) = Ki(m,d) = c(d,m) / det
#pragma unroll
    for (int k = 0; k < 9; ++k) B[k] = c[k] / det;
  }
}

// phi: the base values at the Gauss point, phi_j = phi[j * ps]
__device__ __forceinline__ double coef_val(const gfgpu_coef &c, const SlotPtrs &slots, int64_t e,
                                           const int32_t *en, const double *phi, int nb,
                                           int ps) {
  if (c.kind == GFGPU_COEF_CONST) return c.value;
  if (c.kind == GFGPU_COEF_ELEMENT) return c.value * slots.p[c.slot][e];
  if (c.kind == GFGPU_COEF_NODAL) {
    double s = 0.0;
    for (int j = 0; j < nb; ++j) s += phi[j * ps] * slots.p[c.slot][en[j]];
    return c.value * s;
  }
  return 0.0;
}

// derivative factor of a coefficient in the data of slot ws: d c / d theta_e
// (element) or d c / d theta_j = factor * phi_j (nodal)
__device__ __forceinline__ void coef_dfac(const gfgpu_coef &c, int ws, double &fe, double &fn) {
  fe = fn = 0.0;
  if (c.slot != ws) return;
  if (c.kind == GFGPU_COEF_ELEMENT) fe = c.value;
  if (c.kind == GFGPU_COEF_NODAL) fn = c.value;
}

// c + a b: one rounding (fma) or two (the reference's operation order; this
// file is compiled with -fmad=false so that the unfused form stays unfused)
template <bool FUSE>
__device__ __forceinline__ double madd(double a, double b, double c) {
  if constexpr (FUSE) return fma(a, b, c);
  else return c + a * b;
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// SHAPE: mode 2 (shape derivative), compiled apart so that modes 0 and 1 do
// not carry its per-vertex partials in registers.  const_jac: the Jacobian
// is the same at every Gauss point (affine simplices, parallelepipeds), so K,
// det and B are formed once per element, from the first point's table.
template <int DIM, int QD, int NB, int NBG, int LAW, bool SHAPE>
__global__ void __launch_bounds__(kGpWarps * 32) gauss_potential_kernel(
    int64_t E, int nq, int mode, int wslot, int const_jac, const double *__restrict__ pts,
    const int32_t *__restrict__ cv, const int32_t *__restrict__ enode,
    const double *__restrict__ hval, const double *__restrict__ hvalT,
    const double *__restrict__ hgradT, const double *__restrict__ ggrad,
    const double *__restrict__ hw, gfgpu_form form,
    SlotPtrs slots, double *__restrict__ out_e, double *__restrict__ out_n,
    double *__restrict__ out_x, int *__restrict__ err) {
  constexpr int S = NB * QD;
  // the neo-Hookean energy keeps the reference's unfused operation order
  // (j1 - 3 cancels); the quadratic integrands use fused multiply-adds
  constexpr bool kFuse = LAW != LAW_NH;
  __shared__ double us_all[kGpWarps][S];
  __shared__ double xs_all[kGpWarps][NBG * DIM];
  __shared__ int32_t en_all[kGpWarps][NB];
  __shared__ double dn_all[kGpWarps][32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int64_t e = int64_t(blockIdx.x) * kGpWarps + w;
  if (e >= E) return;
  double *us = us_all[w];
  double *xs = xs_all[w];
  int32_t *en = en_all[w];
  double *dn = dn_all[w];
  for (int j = lane; j < NB; j += 32) en[j] = enode[e * NB + j];
  for (int k = lane; k < NBG * DIM; k += 32)
    xs[k] = pts[int64_t(cv[e * NBG + k / DIM]) * DIM + k % DIM];
  __syncwarp();
  const double *u = slots.p[GFGPU_SLOT_U];
  for (int c = lane; c < S; c += 32) us[c] = u[int64_t(en[c / QD]) * QD + c % QD];
  __syncwarp();
  // u(x_q) is needed by the mass and source integrands only
  bool need_val = false;
  for (int t = 0; t < form.n_terms; ++t)
    need_val |= form.terms[t].kind == GFGPU_TERM_MASS || form.terms[t].kind == GFGPU_TERM_SOURCE;
  double acc = 0.0;                  // energy or element-coefficient derivative
  constexpr int NX = SHAPE ? NBG * DIM : 1;
  double accx[NX];                   // shape derivative partials of this lane
#pragma unroll
  for (int k = 0; k < NX; ++k) accx[k] = 0.0;
  double accn[(NB + 31) / 32];       // nodal partials, node j = lane + 32 r
#pragma unroll
  for (int r = 0; r < (NB + 31) / 32; ++r) accn[r] = 0.0;
  double B[DIM * DIM], det = 0.0;
  for (int q0 = 0; q0 < nq; q0 += 32) {
    const int q = q0 + lane;
    const bool act = q < nq;
    const int qq = act ? q : 0;
    if (!const_jac || q0 == 0) {
      const int qg = const_jac ? 0 : qq;
      double K[DIM * DIM];
#pragma unroll
      for (int d = 0; d < DIM; ++d)
#pragma unroll
        for (int m = 0; m < DIM; ++m) {
          double s = 0.0;
#pragma unroll
          for (int v = 0; v < NBG; ++v)
            s = madd<kFuse>(xs[v * DIM + d], ggrad[(qg * NBG + v) * DIM + m], s);
          K[d + DIM * m] = s;
        }
      geo_inverse<DIM>(K, B, det);
    }
    if (act && det == 0.0) set_err(err, ERR_JACOBIAN);
    const double wJ = (act && det != 0.0) ? fabs(det) * hw[qq] : 0.0;
    // Grad_u in reference coordinates, Gr(a,m) = sum_j u_ja dphi_j/dxi_m, then
    // Grad_u(a,d) = sum_m B(d,m) Gr(a,m); u(x_q).  The tables are read
    // transposed (Gauss point fastest), so the lanes' loads coalesce.
    double Gu[QD][DIM], Gr[QD][DIM], uq[QD];
#pragma unroll
    for (int a = 0; a < QD; ++a) {
      uq[a] = 0.0;
#pragma unroll
      for (int m = 0; m < DIM; ++m) Gr[a][m] = 0.0;
    }
    const double *phi = hvalT + qq;  // phi_j = phi[j * nq]
    for (int j = 0; j < NB; ++j) {
      double r[DIM];
#pragma unroll
      for (int m = 0; m < DIM; ++m) r[m] = hgradT[int64_t(j * DIM + m) * nq + qq];
#pragma unroll
      for (int a = 0; a < QD; ++a) {
        const double ua = us[j * QD + a];
#pragma unroll
        for (int m = 0; m < DIM; ++m) Gr[a][m] = madd<kFuse>(ua, r[m], Gr[a][m]);
      }
    }
    if (need_val) {
      for (int j = 0; j < NB; ++j) {
        const double ph = phi[int64_t(j) * nq];
#pragma unroll
        for (int a = 0; a < QD; ++a) uq[a] = madd<kFuse>(ph, us[j * QD + a], uq[a]);
      }
    }
#pragma unroll
    for (int a = 0; a < QD; ++a)
#pragma unroll
      for (int d = 0; d < DIM; ++d) {
        double s = 0.0;
#pragma unroll
        for (int m = 0; m < DIM; ++m) s = madd<kFuse>(B[d + DIM * m], Gr[a][m], s);
        Gu[a][d] = s;
      }
    // integrand psi, P = dpsi/dGrad_u, and the coefficient derivatives
    double psi = 0.0, de = 0.0, dnq = 0.0;
    double P[QD][DIM];
#pragma unroll
    for (int a = 0; a < QD; ++a)
#pragma unroll
      for (int d = 0; d < DIM; ++d) P[a][d] = 0.0;
    if constexpr (LAW == LAW_NH) {
      const gfgpu_term &T = form.terms[0];
      const double sc = T.scale;
      const double C1 = coef_val(T.c[0], slots, e, en, phi, NB, nq);
      const double D1 = coef_val(T.c[1], slots, e, en, phi, NB, nq);
      double F[9], C[9];
#pragma unroll
      for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) {
          double s = 0.0;
#pragma unroll
          for (int m = 0; m < 3; ++m) s += Gu[m][i] * Gu[m][j];
          C[i + 3 * j] = 2.0 * (0.5 * (s + Gu[i][j] + Gu[j][i])) + (i == j ? 1.0 : 0.0);
          F[i + 3 * j] = Gu[i][j] + (i == j ? 1.0 : 0.0);
        }
      const double detF = F[0] * (F[4] * F[8] - F[5] * F[7]) - F[3] * (F[1] * F[8] - F[2] * F[7]) +
                          F[6] * (F[1] * F[5] - F[2] * F[4]);
      double Cb[9], i3;
      geo_inverse<3>(C, Cb, i3);  // Cb(d,m) = C^{-T}(d,m) = C^{-1}(d,m) (C symmetric)
      const double i1 = C[0] + C[4] + C[8];
      const double p13 = pow(fabs(i3), -1.0 / 3.0);
      const double j1 = i1 * p13;
      const double r = sqrt(fabs(i3)) - 1.0;
      if (detF > 0.0) {
        psi = sc * (C1 * (j1 - 3.0) + D1 * (r * r));
        double f1e, f1n, f2e, f2n;
        coef_dfac(T.c[0], wslot, f1e, f1n);
        coef_dfac(T.c[1], wslot, f2e, f2n);
        const double dW1 = sc * (j1 - 3.0), dW2 = sc * (r * r);
        de = dW1 * f1e + dW2 * f2e;
        dnq = dW1 * f1n + dW2 * f2n;
        if constexpr (SHAPE) {
          // P = sc F S(E), S the law's second Piola-Kirchhoff stress
          const double dd = D1 - D1 / sqrt(fabs(i3));
          double Sm[9];
#pragma unroll
          for (int k = 0; k < 9; ++k) {
            const double di3 = Cb[k] * i3;
            const double dj1 = ((k % 4 == 0 ? 1.0 : 0.0) - i1 / (3.0 * i3) * di3) * p13;
            Sm[k] = 2.0 * C1 * dj1 + 2.0 * dd * di3;
          }
#pragma unroll
          for (int a = 0; a < 3; ++a)
#pragma unroll
            for (int k = 0; k < 3; ++k) {
              double s = 0.0;
#pragma unroll
              for (int m = 0; m < 3; ++m) s += F[a + 3 * m] * Sm[m + 3 * k];
              P[a][k] = sc * s;
            }
        }
      } else {
        psi = sc * 1e200;
      }
    } else {
      double div = 0.0;
      if constexpr (QD > 1) {
#pragma unroll
        for (int a = 0; a < QD; ++a) div += Gu[a][a < DIM ? a : 0];
      }
      for (int t = 0; t < form.n_terms; ++t) {
        const gfgpu_term &T = form.terms[t];
        const double sc = T.scale;
        if (T.kind == GFGPU_TERM_GRADGRAD) {
          const double c0 = coef_val(T.c[0], slots, e, en, phi, NB, nq) * sc;
          const double c1 = coef_val(T.c[1], slots, e, en, phi, NB, nq) * sc;
          const double c2 = coef_val(T.c[2], slots, e, en, phi, NB, nq) * sc;
          double v = 0.0, gg = 0.0, gt = 0.0;
#pragma unroll
          for (int a = 0; a < QD; ++a)
#pragma unroll
            for (int k = 0; k < DIM; ++k) {
              double Dk = c1 * Gu[a][k];
              if constexpr (QD > 1) Dk += (k == a ? c0 * div : 0.0) + c2 * Gu[k < QD ? k : 0][a];
              v += Dk * Gu[a][k];
              gg += Gu[a][k] * Gu[a][k];
              if constexpr (QD > 1) gt += Gu[k < QD ? k : 0][a] * Gu[a][k];
              if constexpr (SHAPE) P[a][k] += 2.0 * Dk;
            }
          psi += v;
          double fe, fn;
          coef_dfac(T.c[0], wslot, fe, fn);
          de += sc * div * div * fe, dnq += sc * div * div * fn;
          coef_dfac(T.c[1], wslot, fe, fn);
          de += sc * gg * fe, dnq += sc * gg * fn;
          coef_dfac(T.c[2], wslot, fe, fn);
          de += sc * gt * fe, dnq += sc * gt * fn;
        } else if (T.kind == GFGPU_TERM_MASS) {
          const double c0 = coef_val(T.c[0], slots, e, en, phi, NB, nq) * sc;
          double uu = 0.0;
#pragma unroll
          for (int a = 0; a < QD; ++a) {
            psi += c0 * uq[a] * uq[a];
            uu += uq[a] * uq[a];
          }
          double fe, fn;
          coef_dfac(T.c[0], wslot, fe, fn);
          de += sc * uu * fe, dnq += sc * uu * fn;
        } else if (T.kind == GFGPU_TERM_SOURCE) {
          const bool none = T.c[0].kind == GFGPU_COEF_NONE;
          const double c0 = (none ? 1.0 : coef_val(T.c[0], slots, e, en, phi, NB, nq)) * sc;
          const double *f = slots.p[T.field_slot];
          double fq[QD];
#pragma unroll
          for (int a = 0; a < QD; ++a) fq[a] = 0.0;
          for (int j = 0; j < NB; ++j)
#pragma unroll
            for (int a = 0; a < QD; ++a) fq[a] += phi[int64_t(j) * nq] * f[int64_t(en[j]) * QD + a];
          double fu = 0.0;
          for (int j = 0; j < NB; ++j)
#pragma unroll
            for (int a = 0; a < QD; ++a) {
              psi += c0 * fq[a] * phi[int64_t(j) * nq] * us[j * QD + a];
              fu += fq[a] * phi[int64_t(j) * nq] * us[j * QD + a];
            }
          if (!none) {
            double fe, fn;
            coef_dfac(T.c[0], wslot, fe, fn);
            de += sc * fu * fe, dnq += sc * fu * fn;
          }
        }
      }
    }
    if (!act) psi = de = dnq = 0.0;
    if constexpr (!SHAPE) {
      if (mode == 0) {
        acc += psi * wJ;
      } else if (mode == 1) {
        acc += de * wJ;
        dn[lane] = dnq * wJ;
        __syncwarp();
        const int nlast = nq - q0 < 32 ? nq - q0 : 32;
#pragma unroll
        for (int r = 0; r < (NB + 31) / 32; ++r) {
          const int j = lane + 32 * r;
          if (j < NB) {
            double s = 0.0;
            for (int l = 0; l < nlast; ++l) s += dn[l] * hval[(q0 + l) * NB + j];
            accn[r] += s;
          }
        }
        __syncwarp();
      }
    } else {
      // H(d,k) = psi d_dk - sum_a P(a,k) Grad_u(a,d); dE/dx_v[d] += wJ H(d,:).G_v
      double H[DIM][DIM];
#pragma unroll
      for (int d = 0; d < DIM; ++d)
#pragma unroll
        for (int k = 0; k < DIM; ++k) {
          double s = d == k ? psi : 0.0;
#pragma unroll
          for (int a = 0; a < QD; ++a) s -= P[a][k] * Gu[a][d];
          H[d][k] = act ? wJ * s : 0.0;
        }
#pragma unroll
      for (int v = 0; v < NBG; ++v) {
        const double *gg = ggrad + (qq * NBG + v) * DIM;
        double Gv[DIM];
#pragma unroll
        for (int k = 0; k < DIM; ++k) {
          double s = 0.0;
#pragma unroll
          for (int m = 0; m < DIM; ++m) s += gg[m] * B[k + DIM * m];
          Gv[k] = s;
        }
#pragma unroll
        for (int d = 0; d < DIM; ++d) {
          double s = 0.0;
#pragma unroll
          for (int k = 0; k < DIM; ++k) s += H[d][k] * Gv[k];
          accx[v * DIM + d] += s;
        }
      }
    }
  }
  if constexpr (!SHAPE) {
    const double tot = warp_sum(acc);
    if (lane == 0) {
      if (!isfinite(tot) && mode == 1) set_err(err, ERR_NAN);
      out_e[e] = tot;
    }
    if (mode == 1 && out_n) {
#pragma unroll
      for (int r = 0; r < (NB + 31) / 32; ++r) {
        const int j = lane + 32 * r;
        if (j < NB) out_n[e * NB + j] = accn[r];
      }
    }
  } else {
#pragma unroll
    for (int k = 0; k < NBG * DIM; ++k) {
      const double tot = warp_sum(accx[k]);
      if (lane == 0) out_x[e * NBG * DIM + k] = tot;
    }
  }
}

// Potentials and element-coefficient derivatives (modes 0 and 1) of scalar
// isotropic forms on parallelepiped hexahedra, kEw elements per warp: the
// per-point reference gradients Gr(m) = sum_j u_j dphi_j/dxi_m of the warp's
// elements share every table load (one load feeds kEw FMAs; with one element
// per warp the kernel waited on those loads), and each element's sums are
// formed with the same operations in the same order as
// gauss_potential_kernel's (the same bits).  Forms with GRADGRAD terms only,
// coefficients constant or per element.
constexpr int kEw = 4;

template <int NB>
__global__ void __launch_bounds__(kGpWarps * 32) affine_scalar_potential_kernel(
    int64_t E, int nq, int mode, int wslot, const double *__restrict__ pts,
    const int32_t *__restrict__ cv, const int32_t *__restrict__ enode,
    const double *__restrict__ hgradT, const double *__restrict__ ggrad,
    const double *__restrict__ hw, gfgpu_form form, SlotPtrs slots, double *__restrict__ out_e,
    int *__restrict__ err) {
  constexpr int DIM = 3, NBG = 8;
  __shared__ double us_all[kGpWarps][NB][kEw];
  __shared__ double B_all[kGpWarps][kEw][9];
  __shared__ double det_all[kGpWarps][kEw];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int64_t e0 = (int64_t(blockIdx.x) * kGpWarps + w) * kEw;
  if (e0 >= E) return;
  const int ne = E - e0 < kEw ? int(E - e0) : kEw;
  double(*us)[kEw] = us_all[w];
  const double *u = slots.p[GFGPU_SLOT_U];
  for (int z = lane; z < NB * kEw; z += 32) {
    const int j = z / kEw, k = z - j * kEw;
    us[j][k] = k < ne ? u[enode[(e0 + k) * NB + j]] : 0.0;
  }
  // geometry of element e0 + k on lane k (K from the first point's geometric
  // gradients: the Jacobian is constant)
  if (lane < kEw) {
    double B[9], det = 0.0;
    if (lane < ne) {
      double K[9];
#pragma unroll
      for (int d = 0; d < DIM; ++d)
#pragma unroll
        for (int m = 0; m < DIM; ++m) {
          double s = 0.0;
#pragma unroll
          for (int v = 0; v < NBG; ++v)
            s = fma(pts[int64_t(cv[(e0 + lane) * NBG + v]) * DIM + d], ggrad[v * DIM + m], s);
          K[d + DIM * m] = s;
        }
      geo_inverse<DIM>(K, B, det);
      if (det == 0.0) set_err(err, ERR_JACOBIAN);
    } else {
#pragma unroll
      for (int k = 0; k < 9; ++k) B[k] = 0.0;
    }
#pragma unroll
    for (int k = 0; k < 9; ++k) B_all[w][lane][k] = B[k];
    det_all[w][lane] = det;
  }
  __syncwarp();
  double acc[kEw];
#pragma unroll
  for (int k = 0; k < kEw; ++k) acc[k] = 0.0;
  for (int q0 = 0; q0 < nq; q0 += 32) {
    const int q = q0 + lane;
    const bool act = q < nq;
    const int qq = act ? q : 0;
    double Gr[kEw][DIM];
#pragma unroll
    for (int k = 0; k < kEw; ++k)
#pragma unroll
      for (int m = 0; m < DIM; ++m) Gr[k][m] = 0.0;
    for (int j = 0; j < NB; ++j) {
      double r[DIM];
#pragma unroll
      for (int m = 0; m < DIM; ++m) r[m] = hgradT[int64_t(j * DIM + m) * nq + qq];
#pragma unroll
      for (int k = 0; k < kEw; ++k) {
        const double uj = us[j][k];
#pragma unroll
        for (int m = 0; m < DIM; ++m) Gr[k][m] = fma(uj, r[m], Gr[k][m]);
      }
    }
#pragma unroll
    for (int k = 0; k < kEw; ++k) {
      const double *B = B_all[w][k];
      const double det = det_all[w][k];
      const double wJ = (act && det != 0.0) ? fabs(det) * hw[qq] : 0.0;
      double Gu[DIM];
#pragma unroll
      for (int d = 0; d < DIM; ++d) {
        double s = 0.0;
#pragma unroll
        for (int m = 0; m < DIM; ++m) s = fma(B[d + DIM * m], Gr[k][m], s);
        Gu[d] = s;
      }
      const int64_t e = e0 + k;
      const int64_t ec = k < ne ? e : e0;
      double psi = 0.0, de = 0.0;
      for (int t = 0; t < form.n_terms; ++t) {
        const gfgpu_term &T = form.terms[t];
        const double sc = T.scale;
        const double c1 = coef_val(T.c[1], slots, ec, nullptr, nullptr, NB, nq) * sc;
        double v = 0.0, gg = 0.0;
#pragma unroll
        for (int d = 0; d < DIM; ++d) {
          const double Dk = c1 * Gu[d];
          v += Dk * Gu[d];
          gg += Gu[d] * Gu[d];
        }
        psi += v;
        double fe, fn;
        coef_dfac(T.c[1], wslot, fe, fn);
        de += sc * gg * fe;
      }
      if (!act) psi = de = 0.0;
      acc[k] += (mode == 0 ? psi : de) * wJ;
    }
  }
#pragma unroll
  for (int k = 0; k < kEw; ++k) {
    const double tot = warp_sum(acc[k]);
    if (lane == 0 && k < ne) {
      if (!isfinite(tot) && mode == 1) set_err(err, ERR_NAN);
      out_e[e0 + k] = tot;
    }
  }
}

// The same potentials through the reference tensors of the parallelepiped
// plan (G_00, G_11, G_22, G_01, G_02, G_12: sum_q w_q of the products of
// reference derivatives, summed on the host from the reference's tabulated
// gradients): sum_q w_q |J| |grad u|^2 = |J| sum_p M_p u^T G_p u with
// M = B^T B and the Jacobian K from the element's edge vectors (x_{e_m} -
// x_0, exact differences).  On axis-aligned elements K, B and M are diagonal
// (exact zeros) and only G_00, G_11, G_22 enter (NP = 3): 4 FP64 operations
// per element and upper-triangle entry (a multiply and three FMAs), 31.5 k per
// Q4 element against 49 k through the Gauss points; otherwise NP = 6.  EQ
// elements per block share every table load; per-thread partial sums, then
// warp and block sums in a fixed order.
constexpr int kQfThreads = 256;

template <int NB, int NP, int EQ>
__global__ void __launch_bounds__(kQfThreads) affine_scalar_quadform_kernel(
    int64_t E, int mode, int wslot, const double *__restrict__ pts,
    const int32_t *__restrict__ cv, const int32_t *__restrict__ enode,
    const double *__restrict__ tabs, const int32_t *__restrict__ tri, gfgpu_form form,
    SlotPtrs slots, double *__restrict__ out_e, int *__restrict__ err) {
  constexpr int DIM = 3, NT = NB * (NB + 1) / 2, NN = NB * NB;
  constexpr int NW = kQfThreads / 32;
  __shared__ double us[EQ][NB];
  __shared__ double mc[EQ][NP];
  __shared__ double cfs[EQ];
  __shared__ double part[NW][EQ][NP];
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  const int64_t e0 = int64_t(blockIdx.x) * EQ;
  const int ne = E - e0 < EQ ? int(E - e0) : EQ;
  const double *u = slots.p[GFGPU_SLOT_U];
  for (int z = tid; z < NB * EQ; z += kQfThreads) {
    const int k = z / NB, j = z - k * NB;
    us[k][j] = k < ne ? u[enode[(e0 + k) * NB + j]] : 0.0;
  }
  if (tid < EQ) {
    const int k = tid;
    double m[NP], cf = 0.0;
#pragma unroll
    for (int p = 0; p < NP; ++p) m[p] = 0.0;
    if (k < ne) {
      const int64_t e = e0 + k;
      const int32_t *c = cv + e * 8;
      double K[9], B[9], det = 0.0;
#pragma unroll
      for (int mm = 0; mm < DIM; ++mm)
#pragma unroll
        for (int d = 0; d < DIM; ++d)
          K[d + DIM * mm] = pts[int64_t(c[1 << mm]) * DIM + d] - pts[int64_t(c[0]) * DIM + d];
      geo_inverse<DIM>(K, B, det);
      if (det == 0.0) set_err(err, ERR_JACOBIAN);
      const double J = det == 0.0 ? 0.0 : fabs(det);
      // M_mn = sum_d B(d,m) B(d,n), in the table order 00 11 22 01 02 12
#pragma unroll
      for (int p = 0; p < NP; ++p) {
        const int pm = p < 3 ? p : (p == 5 ? 1 : 0), pn = p < 3 ? p : (p == 3 ? 1 : 2);
        double sum = 0.0;
#pragma unroll
        for (int d = 0; d < DIM; ++d) sum = fma(B[d + DIM * pm], B[d + DIM * pn], sum);
        m[p] = J * sum;
      }
      for (int t = 0; t < form.n_terms; ++t) {
        const gfgpu_term &T = form.terms[t];
        if (mode == 0) {
          cf += coef_val(T.c[1], slots, e, nullptr, nullptr, NB, 1) * T.scale;
        } else {
          double fe, fn;
          coef_dfac(T.c[1], wslot, fe, fn);
          cf += T.scale * fe;
        }
      }
    }
#pragma unroll
    for (int p = 0; p < NP; ++p) mc[k][p] = m[p];
    cfs[k] = cf;
  }
  __syncthreads();
  double Q[EQ][NP];
#pragma unroll
  for (int k = 0; k < EQ; ++k)
#pragma unroll
    for (int p = 0; p < NP; ++p) Q[k][p] = 0.0;
  for (int ent = tid; ent < NT; ent += kQfThreads) {
    const int rc = tri[ent];
    const int r = rc >> 16, c = rc & 0xffff, idx = r * NB + c;
    const double two = r == c ? 1.0 : 2.0;
    double g[NP];
#pragma unroll
    for (int p = 0; p < NP; ++p) g[p] = two * tabs[p * NN + idx];
#pragma unroll
    for (int k = 0; k < EQ; ++k) {
      const double pr = us[k][r] * us[k][c];
#pragma unroll
      for (int p = 0; p < NP; ++p) Q[k][p] = fma(g[p], pr, Q[k][p]);
    }
  }
#pragma unroll
  for (int k = 0; k < EQ; ++k)
#pragma unroll
    for (int p = 0; p < NP; ++p) {
      const double v = warp_sum(Q[k][p]);
      if (lane == 0) part[wid][k][p] = v;
    }
  __syncthreads();
  if (tid < EQ && tid < ne) {
    const int k = tid;
    double s2 = 0.0;
#pragma unroll
    for (int p = 0; p < NP; ++p) {
      double q = 0.0;
      for (int w = 0; w < NW; ++w) q += part[w][k][p];
      s2 = fma(mc[k][p], q, s2);
    }
    const double tot = cfs[k] * s2;
    if (!isfinite(tot) && mode == 1) set_err(err, ERR_NAN);
    out_e[e0 + k] = tot;
  }
}

// Sum of n values in a fixed order (one block): deterministic.
__global__ void __launch_bounds__(1024) ordered_sum(const double *__restrict__ v, int64_t n,
                                                    double *__restrict__ out) {
  __shared__ double s[1024];
  const int t = threadIdx.x;
  const int64_t per = (n + 1023) / 1024;
  double a = 0.0;
  for (int64_t i = t * per; i < (t + 1) * per && i < n; ++i) a += v[i];
  s[t] = a;
  __syncthreads();
  for (int o = 512; o > 0; o >>= 1) {
    if (t < o) s[t] += s[t + o];
    __syncthreads();
  }
  if (t == 0) *out = s[0];
}

// out[n] = sum over the adjacency codes of node n of part[code]
__global__ void adjacency_gather(int64_t n, int width, const int32_t *__restrict__ ptr,
                                 const int32_t *__restrict__ adj, int nper,
                                 const double *__restrict__ part, double *__restrict__ out) {
  const int64_t t = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  if (t >= n * width) return;
  const int64_t node = t / width;
  const int d = int(t % width);
  double s = 0.0;
  for (int k = ptr[node]; k < ptr[node + 1]; ++k) s += part[int64_t(adj[k]) * width + d];
  (void)nper;
  out[t] = s;
}

template <int DIM, int QD, int NB, int NBG, int LAW>
cudaError_t launch_gp(Plan &P, int mode, int wslot, const SlotPtrs &sp, double *oe, double *on,
                      double *ox) {
  const unsigned blocks = unsigned((P.n_elements + kGpWarps - 1) / kGpWarps);
  const int cj = P.kind == SIMPLEX || P.parallelepiped;
  auto kern = mode == 2 ? gauss_potential_kernel<DIM, QD, NB, NBG, LAW, true>
                        : gauss_potential_kernel<DIM, QD, NB, NBG, LAW, false>;
  kern<<<blocks, kGpWarps * 32, 0, P.stream>>>(
      P.n_elements, P.nq, mode, wslot, cj, P.d_points, P.d_cv, P.d_enode, P.d_hval, P.d_hvalT,
      P.d_hgradT, P.d_ggrad, P.d_hw, P.form, sp, oe, on, ox, P.d_err);
  return cudaGetLastError();
}

// The forms affine_scalar_potential_kernel takes: GRADGRAD terms only, with
// constant or per-element coefficients and no c0 / c2 part.
bool affine_scalar_potential_ok(const Plan &P, int mode) {
  if (P.kind != HEX || !P.parallelepiped || P.law != LAW_ISO || P.qdim != 1 || P.dim != 3 ||
      mode > 1 || P.form.n_terms < 1)
    return false;
  if (P.degree != 1 && P.degree != 2 && P.degree != 4) return false;
  for (int t = 0; t < P.form.n_terms; ++t) {
    const gfgpu_term &T = P.form.terms[t];
    if (T.kind != GFGPU_TERM_GRADGRAD) return false;
    if (T.c[0].kind != GFGPU_COEF_NONE || T.c[2].kind != GFGPU_COEF_NONE) return false;
    if (T.c[1].kind != GFGPU_COEF_CONST && T.c[1].kind != GFGPU_COEF_ELEMENT) return false;
  }
  return true;
}

template <int NB>
cudaError_t launch_asp(Plan &P, int mode, int wslot, const SlotPtrs &sp, double *oe) {
  const int64_t per_block = int64_t(kGpWarps) * kEw;
  const unsigned blocks = unsigned((P.n_elements + per_block - 1) / per_block);
  affine_scalar_potential_kernel<NB><<<blocks, kGpWarps * 32, 0, P.stream>>>(
      P.n_elements, P.nq, mode, wslot, P.d_points, P.d_cv, P.d_enode, P.d_hgradT, P.d_ggrad,
      P.d_hw, P.form, sp, oe, P.d_err);
  return cudaGetLastError();
}

cudaError_t dispatch_gp(Plan &P, int mode, int wslot, double *oe, double *on, double *ox) {
  SlotPtrs sp;
  for (int i = 0; i < GFGPU_MAX_SLOTS; ++i) sp.p[i] = P.slot_ptr[i];
  const int k = P.degree, q = P.qdim;
  if (!on && affine_scalar_potential_ok(P, mode) && P.affine_hex && P.d_aff && P.d_tri) {
    // reference tensors of the parallelepiped plan: 3 of them on an
    // axis-aligned mesh (8 elements per block), else 6 (4 per block)
#define QFK(NBV, NPV, EQV)                                                                    \
  affine_scalar_quadform_kernel<NBV, NPV, EQV>                                               \
      <<<unsigned((P.n_elements + EQV - 1) / EQV), kQfThreads, 0, P.stream>>>(               \
          P.n_elements, mode, wslot, P.d_points, P.d_cv, P.d_enode, P.d_aff, P.d_tri, P.form, \
          sp, oe, P.d_err)
#define QFN(NBV)              \
  do {                        \
    if (P.axis_aligned)       \
      QFK(NBV, 3, 8);         \
    else                      \
      QFK(NBV, 6, 4);         \
  } while (0)
    if (k == 4) QFN(125);
    else if (k == 2) QFN(27);
    else QFN(8);
#undef QFN
#undef QFK
    return cudaGetLastError();
  }
  if (!on && affine_scalar_potential_ok(P, mode)) {
    if (k == 4) return launch_asp<125>(P, mode, wslot, sp, oe);
    if (k == 2) return launch_asp<27>(P, mode, wslot, sp, oe);
    return launch_asp<8>(P, mode, wslot, sp, oe);
  }
  if (P.law == LAW_NH) {
    if (P.kind == HEX && k == 2) return launch_gp<3, 3, 27, 8, LAW_NH>(P, mode, wslot, sp, oe, on, ox);
    if (P.kind == HEX && k == 1) return launch_gp<3, 3, 8, 8, LAW_NH>(P, mode, wslot, sp, oe, on, ox);
    if (P.kind == SIMPLEX && k == 2) return launch_gp<3, 3, 10, 4, LAW_NH>(P, mode, wslot, sp, oe, on, ox);
    if (P.kind == SIMPLEX && k == 1) return launch_gp<3, 3, 4, 4, LAW_NH>(P, mode, wslot, sp, oe, on, ox);
    return cudaErrorInvalidValue;
  }
#define GP(D, Q, NB, NBG) return launch_gp<D, Q, NB, NBG, LAW_ISO>(P, mode, wslot, sp, oe, on, ox)
  if (P.kind == SIMPLEX && P.dim == 2) {
    if (k == 1 && q == 1) GP(2, 1, 3, 3);
    if (k == 2 && q == 1) GP(2, 1, 6, 3);
    if (k == 1 && q == 2) GP(2, 2, 3, 3);
    if (k == 2 && q == 2) GP(2, 2, 6, 3);
  } else if (P.kind == SIMPLEX && P.dim == 3) {
    if (k == 1 && q == 1) GP(3, 1, 4, 4);
    if (k == 2 && q == 1) GP(3, 1, 10, 4);
    if (k == 1 && q == 3) GP(3, 3, 4, 4);
    if (k == 2 && q == 3) GP(3, 3, 10, 4);
  } else if (P.kind == HEX) {
    if (k == 1 && q == 1) GP(3, 1, 8, 8);
    if (k == 2 && q == 1) GP(3, 1, 27, 8);
    if (k == 4 && q == 1) GP(3, 1, 125, 8);
    if (k == 1 && q == 3) GP(3, 3, 8, 8);
    if (k == 2 && q == 3) GP(3, 3, 27, 8);
  }
#undef GP
  return cudaErrorInvalidValue;
}

}  // namespace

bool gauss_potential_available(int dim, int kind, int degree, int qdim, int law) {
  if (law == LAW_NH) return dim == 3 && qdim == 3 && degree <= 2;
  if (kind == SIMPLEX) return degree <= 2 && (qdim == 1 || qdim == dim);
  return dim == 3 && ((degree <= 2 && (qdim == 1 || qdim == 3)) || (degree == 4 && qdim == 1));
}

// Gauss tables of any element (values, reference gradients, geometric
// gradients, weights) into the plan's host vectors.
int build_gauss_tables(Plan &P, std::string &errmsg) {
  RefElement fe(P.dim, P.kind, P.degree), gt(P.dim, P.kind, 1);
  Quadrature q;
  if (!quadrature_by_name(P.im, q) || q.dim != P.dim) {
    errmsg = "unsupported integration method " + P.im;
    return GFGPU_E_UNSUPPORTED;
  }
  P.nq = q.nq;
  const int D = P.dim;
  P.h_val.assign(size_t(q.nq) * fe.nb, 0.0);
  P.h_grad.assign(size_t(q.nq) * fe.nb * D, 0.0);
  P.h_ggrad.assign(size_t(q.nq) * gt.nb * D, 0.0);
  std::vector<double> gv(gt.nb);
  for (int k = 0; k < q.nq; ++k) {
    fe.eval(&q.pts[size_t(k) * D], &P.h_val[size_t(k) * fe.nb], &P.h_grad[size_t(k) * fe.nb * D]);
    gt.eval(&q.pts[size_t(k) * D], gv.data(), &P.h_ggrad[size_t(k) * gt.nb * D]);
  }
  P.h_w = q.w;
  return GFGPU_OK;
}

cudaError_t launch_potential(Plan &P, double *d_out) {
  if (P.n_elements == 0) return cudaMemsetAsync(d_out, 0, sizeof(double), P.stream);
  cudaError_t ce = dispatch_gp(P, 0, -1, P.d_epart, nullptr, nullptr);
  if (ce != cudaSuccess) return ce;
  ordered_sum<<<1, 1024, 0, P.stream>>>(P.d_epart, P.n_elements, d_out);
  P.launches += 2;
  return cudaGetLastError();
}

cudaError_t launch_coef_gradient(Plan &P, int slot, bool nodal, double *d_out) {
  if (P.n_elements == 0) return cudaSuccess;
  cudaError_t ce = dispatch_gp(P, 1, slot, nodal ? P.d_epart : d_out, nodal ? P.d_npart : nullptr,
                               nullptr);
  if (ce != cudaSuccess) return ce;
  P.launches++;
  if (nodal) {
    const int64_t n = P.n_nodes;
    adjacency_gather<<<unsigned((n + 255) / 256), 256, 0, P.stream>>>(
        n, 1, P.d_adj_ptr, P.d_adj, P.nb, P.d_npart, d_out);
    P.launches++;
  }
  return cudaGetLastError();
}

cudaError_t launch_shape_gradient(Plan &P, double *d_out) {
  if (P.n_elements == 0) return cudaMemsetAsync(d_out, 0, sizeof(double) * P.n_points * P.dim,
                                                P.stream);
  cudaError_t ce = dispatch_gp(P, 2, -1, nullptr, nullptr, P.d_xpart);
  if (ce != cudaSuccess) return ce;
  const int64_t n = P.n_points;
  adjacency_gather<<<unsigned((n * P.dim + 255) / 256), 256, 0, P.stream>>>(
      n, P.dim, P.d_padj_ptr, P.d_padj, P.nbg, P.d_xpart, d_out);
  P.launches += 2;
  return cudaGetLastError();
}

}  // namespace gfgpu
