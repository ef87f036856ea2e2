// Linear solves on a plan's assembled CSR: Dirichlet conditions by
// elimination and conjugate gradients, FP64, on the device.
//
//  - gfgpu_dirichlet_eliminate: the reference model's dof constraints on a
//    linear symmetric problem (getfem_models.cc:2806-2870): rhs -= K(:,D) g,
//    rhs(D) = g, rows and columns D of K cleared, K(d,d) = 1.  The CSR
//    pattern is kept (cleared entries hold 0).
//  - gfgpu_cg: gmm::cg (gmm_solver_cg.h:84-157) with the identity or the
//    diagonal (Jacobi) preconditioner and gmm::iteration's stop rule
//    (gmm_iter.h:113-150): stop when ||r||_2 <= ||b||_2 resmax or after
//    maxiter iterations; x = 0 when b = 0.
//
// SpMV is HBM-bound: one group of G lanes per row (G from the mean row
// length), coalesced reads of the row's column indices and values.  Dot
// products are summed per block in a fixed tree order, then over blocks in a
// fixed order, so a solve is reproducible bit for bit.  The scalars of the
// recurrence (rho, q.p, alpha) stay on the device; the host reads ||r||^2
// once per iteration for the stop test.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <string>
#include <vector>

#include "k_common.cuh"
#include "plan.h"

namespace gfgpu {
void set_last_error(const std::string &s);
}

using namespace gfgpu;

namespace {

constexpr int kSolveThreads = 256;

// block-level fixed-order sum of one value per thread; result in thread 0
__device__ __forceinline__ double block_sum(double v, double *sh) {
  const int t = threadIdx.x;
  sh[t] = v;
  __syncthreads();
  for (int o = kSolveThreads / 2; o > 0; o >>= 1) {
    if (t < o) sh[t] += sh[t + o];
    __syncthreads();
  }
  return sh[0];
}

// y = A x (G lanes per row); if w: partial[block] = sum_rows w_i y_i
template <int G>
__global__ void __launch_bounds__(kSolveThreads) spmv_kernel(
    int64_t n, const int64_t *__restrict__ rowptr, const int32_t *__restrict__ colidx,
    const double *__restrict__ vals, const double *__restrict__ x, double *__restrict__ y,
    const double *__restrict__ w, double *__restrict__ partial) {
  __shared__ double sh[kSolveThreads];
  constexpr int RPB = kSolveThreads / G;
  const int g = threadIdx.x / G, l = threadIdx.x % G;
  const int64_t row = int64_t(blockIdx.x) * RPB + g;
  double s = 0.0;
  if (row < n) {
    const int64_t b = rowptr[row], e = rowptr[row + 1];
    for (int64_t k = b + l; k < e; k += G) s = fma(vals[k], x[colidx[k]], s);
  }
#pragma unroll
  for (int o = G / 2; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o, G);
  double d = 0.0;
  if (row < n && l == 0) {
    y[row] = s;
    if (w) d = w[row] * s;
  }
  if (partial) {
    const double t = block_sum(d, sh);
    if (threadIdx.x == 0) partial[blockIdx.x] = t;
  }
}

// sum of nb partials in a fixed order into *out
__global__ void __launch_bounds__(kSolveThreads) finish_sum(const double *__restrict__ partial,
                                                            int64_t nb, double *__restrict__ out) {
  __shared__ double sh[kSolveThreads];
  double a = 0.0;
  for (int64_t i = threadIdx.x; i < nb; i += kSolveThreads) a += partial[i];
  const double t = block_sum(a, sh);
  if (threadIdx.x == 0) *out = t;
}

// partial[block] = sum a_i b_i
__global__ void __launch_bounds__(kSolveThreads) dot_kernel(int64_t n, const double *__restrict__ a,
                                                            const double *__restrict__ b,
                                                            double *__restrict__ partial) {
  __shared__ double sh[kSolveThreads];
  double s = 0.0;
  for (int64_t i = blockIdx.x * int64_t(kSolveThreads) + threadIdx.x; i < n;
       i += int64_t(gridDim.x) * kSolveThreads)
    s = fma(a[i], b[i], s);
  const double t = block_sum(s, sh);
  if (threadIdx.x == 0) partial[blockIdx.x] = t;
}

// r = b - q (q = A x)
__global__ void residual_init(int64_t n, const double *__restrict__ b, const double *__restrict__ q,
                              double *__restrict__ r) {
  const int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  if (i < n) r[i] = b[i] - q[i];
}

// alpha = rho / qp; x += alpha p; r -= alpha q; z = dinv r (if dinv);
// partials: r.r and z.r
__global__ void __launch_bounds__(kSolveThreads) cg_step(
    int64_t n, const double *__restrict__ sc, double *__restrict__ x, double *__restrict__ r,
    const double *__restrict__ p, const double *__restrict__ q, const double *__restrict__ dinv,
    double *__restrict__ z, double *__restrict__ prr, double *__restrict__ pzr) {
  __shared__ double sh[kSolveThreads];
  const double alpha = sc[0] / sc[1];  // rho / (q.p)
  double rr = 0.0, zr = 0.0;
  for (int64_t i = blockIdx.x * int64_t(kSolveThreads) + threadIdx.x; i < n;
       i += int64_t(gridDim.x) * kSolveThreads) {
    x[i] = fma(alpha, p[i], x[i]);
    const double ri = fma(-alpha, q[i], r[i]);
    r[i] = ri;
    rr = fma(ri, ri, rr);
    if (dinv) {
      const double zi = dinv[i] * ri;
      z[i] = zi;
      zr = fma(zi, ri, zr);
    }
  }
  double t = block_sum(rr, sh);
  if (threadIdx.x == 0) prr[blockIdx.x] = t;
  __syncthreads();
  if (dinv) {
    t = block_sum(zr, sh);
    if (threadIdx.x == 0) pzr[blockIdx.x] = t;
  }
}

// p = z + (rho_new / rho_old) p
__global__ void cg_direction(int64_t n, const double *__restrict__ sc_new,
                             const double *__restrict__ sc_old, const double *__restrict__ z,
                             double *__restrict__ p) {
  const int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  if (i < n) p[i] = fma(*sc_new / *sc_old, p[i], z[i]);
}

__global__ void copy_scale(int64_t n, const double *__restrict__ a, const double *__restrict__ d,
                           double *__restrict__ out) {
  const int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  if (i < n) out[i] = d ? d[i] * a[i] : a[i];
}

// diagonal inverse (Jacobi); a missing or zero diagonal sets ERR_NAN
__global__ void diag_inverse(int64_t n, const int64_t *__restrict__ rowptr,
                             const int32_t *__restrict__ colidx, const double *__restrict__ vals,
                             double *__restrict__ dinv, int *__restrict__ err) {
  const int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  if (i >= n) return;
  double d = 0.0;
  for (int64_t k = rowptr[i]; k < rowptr[i + 1]; ++k)
    if (colidx[k] == i) d = vals[k];
  if (d == 0.0) set_err(err, ERR_NAN);
  dinv[i] = d == 0.0 ? 0.0 : 1.0 / d;
}

// Dirichlet elimination, one thread per row (rows of FEM matrices are short)
__global__ void dirichlet_rows(int64_t n, const int64_t *__restrict__ rowptr,
                               const int32_t *__restrict__ colidx, double *__restrict__ vals,
                               const uint8_t *__restrict__ mask, const double *__restrict__ g,
                               double *__restrict__ rhs, int *__restrict__ err) {
  const int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  if (i >= n) return;
  const int64_t b = rowptr[i], e = rowptr[i + 1];
  if (mask[i]) {
    bool diag = false;
    for (int64_t k = b; k < e; ++k) {
      const bool dk = colidx[k] == i;
      vals[k] = dk ? 1.0 : 0.0;
      diag |= dk;
    }
    if (!diag) set_err(err, ERR_CAPACITY);
    if (rhs) rhs[i] = g[i];
  } else {
    double s = rhs ? rhs[i] : 0.0;
    for (int64_t k = b; k < e; ++k) {
      const int32_t j = colidx[k];
      if (mask[j]) {
        s = fma(-vals[k], g[j], s);
        vals[k] = 0.0;
      }
    }
    if (rhs) rhs[i] = s;
  }
}

template <int G>
void launch_spmv(const Plan &P, const double *x, double *y, const double *w, double *partial,
                 cudaStream_t st) {
  constexpr int RPB = kSolveThreads / G;
  const unsigned blocks = unsigned((P.n_dof + RPB - 1) / RPB);
  spmv_kernel<G><<<blocks, kSolveThreads, 0, st>>>(P.n_dof, P.d_rowptr, P.d_colidx, P.d_vals, x,
                                                   y, w, partial);
}

int spmv_group(const Plan &P) {
  const double mean = P.n_dof ? double(P.nnz) / double(P.n_dof) : 1.0;
  int G = 1;
  while (G < 32 && G < mean) G <<= 1;
  return G;
}

unsigned spmv_blocks(const Plan &P) {
  const int G = spmv_group(P);
  const int RPB = kSolveThreads / G;
  return unsigned((P.n_dof + RPB - 1) / RPB);
}

void spmv(const Plan &P, const double *x, double *y, const double *w, double *partial,
          cudaStream_t st) {
  switch (spmv_group(P)) {
    case 1: launch_spmv<1>(P, x, y, w, partial, st); break;
    case 2: launch_spmv<2>(P, x, y, w, partial, st); break;
    case 4: launch_spmv<4>(P, x, y, w, partial, st); break;
    case 8: launch_spmv<8>(P, x, y, w, partial, st); break;
    case 16: launch_spmv<16>(P, x, y, w, partial, st); break;
    default: launch_spmv<32>(P, x, y, w, partial, st); break;
  }
}

// CG of a small system in one block (n <= kCgSmallMax): the same recurrence
// and stop rule, every step on the device (no host round trip per
// iteration; the multi-kernel loop spent ~45 us per iteration on launches
// and the stop-test read at 4225 unknowns).  Dot products: per-thread
// partials over rows tid, tid + 1024, ..., then a warp tree and a tree over
// the 32 warps, in a fixed order.  A launch runs at most `seg` iterations
// and leaves the recurrence state in st[] (st[0] iterations, st[1] the
// relative residual, st[2] ||r||, st[3] rho, st[4] r.r, st[5] z.r,
// st[6] 1 when done, st[7] ||b||); the host launches again until done, so a
// large maxiter never makes one long-running kernel.
constexpr int kCgSmallThreads = 1024;
constexpr int64_t kCgSmallMax = 32768;
constexpr int64_t kCgSegment = 2000;  // ~20 ms of iterations at 4225 unknowns

__device__ __forceinline__ double block_sum_1024(double v, double *sh) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  __syncthreads();  // sh free (a previous sum's readers are done)
  if (lane == 0) sh[w] = v;
  __syncthreads();
  double t = sh[lane];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
  return t;  // every thread holds the total
}

__global__ void __launch_bounds__(kCgSmallThreads, 1) cg_small_kernel(
    int64_t n, const int64_t *__restrict__ rowptr, const int32_t *__restrict__ colidx,
    const double *__restrict__ vals, const double *__restrict__ b, double *__restrict__ x,
    double *__restrict__ r, double *__restrict__ p, double *__restrict__ q, double *z,
    const double *__restrict__ dinv, double resmax, int64_t maxiter, int resume, int64_t seg,
    double *__restrict__ st) {
  __shared__ double sh[32];
  const int tid = threadIdx.x;
  constexpr int T = kCgSmallThreads;
  auto spmv = [&](const double *v, double *y) {
    for (int64_t i = tid; i < n; i += T) {
      double s = 0.0;
      for (int64_t k = rowptr[i]; k < rowptr[i + 1]; ++k) s = fma(vals[k], v[colidx[k]], s);
      y[i] = s;
    }
  };
  const double *zz = dinv ? z : r;
  double rhsn, rho, rr, zr = 0.0, res = 0.0;
  int64_t nit;
  if (!resume) {
    double bb = 0.0;
    for (int64_t i = tid; i < n; i += T) bb = fma(b[i], b[i], bb);
    rhsn = sqrt(fabs(block_sum_1024(bb, sh)));
    nit = 0;
    if (rhsn == 0.0) {
      for (int64_t i = tid; i < n; i += T) x[i] = 0.0;
      if (tid == 0) {
        st[0] = 0.0, st[1] = 0.0, st[2] = 0.0, st[6] = 1.0, st[7] = 0.0;
      }
      return;
    }
    // r = b - A x; z = P r; rho = z.r; p = z
    spmv(x, q);
    __syncthreads();
    double r2 = 0.0, z2 = 0.0;
    for (int64_t i = tid; i < n; i += T) {
      const double ri = b[i] - q[i];
      r[i] = ri;
      const double zi = dinv ? dinv[i] * ri : ri;
      if (dinv) z[i] = zi;
      p[i] = zi;
      r2 = fma(ri, ri, r2);
      z2 = fma(zi, ri, z2);
    }
    rr = block_sum_1024(r2, sh);
    rho = dinv ? block_sum_1024(z2, sh) : rr;
  } else {
    nit = int64_t(st[0]);
    rho = st[3], rr = st[4], zr = st[5], rhsn = st[7];
  }
  bool done = false;
  for (int64_t k = 0;; ++k) {
    res = sqrt(rr);
    if (isnan(res) || res <= rhsn * resmax || nit >= maxiter) {
      done = true;
      break;
    }
    if (k >= seg) break;
    if (nit > 0) {
      const double rho_old = rho;
      rho = dinv ? zr : rr;
      const double beta = rho / rho_old;
      for (int64_t i = tid; i < n; i += T) p[i] = fma(beta, p[i], zz[i]);
      __syncthreads();
    }
    // q = A p; alpha = rho / q.p; x += alpha p; r -= alpha q; z = P r
    spmv(p, q);
    double qp = 0.0;
    for (int64_t i = tid; i < n; i += T) qp = fma(q[i], p[i], qp);
    qp = block_sum_1024(qp, sh);
    const double alpha = rho / qp;
    double r2 = 0.0, z2 = 0.0;
    for (int64_t i = tid; i < n; i += T) {
      x[i] = fma(alpha, p[i], x[i]);
      const double ri = fma(-alpha, q[i], r[i]);
      r[i] = ri;
      r2 = fma(ri, ri, r2);
      if (dinv) {
        const double zi = dinv[i] * ri;
        z[i] = zi;
        z2 = fma(zi, ri, z2);
      }
    }
    rr = block_sum_1024(r2, sh);
    if (dinv) zr = block_sum_1024(z2, sh);
    ++nit;
  }
  if (tid == 0) {
    st[0] = double(nit);
    st[1] = res / rhsn;
    st[2] = res;
    st[3] = rho, st[4] = rr, st[5] = zr;
    st[6] = done ? 1.0 : 0.0;
    st[7] = rhsn;
  }
}

struct CgScratch {
  double *r = nullptr, *p = nullptr, *q = nullptr, *z = nullptr, *dinv = nullptr;
  double *part = nullptr, *part2 = nullptr, *sc = nullptr;
  ~CgScratch() {
    for (double *a : {r, p, q, z, dinv, part, part2, sc})
      if (a) cudaFree(a);
  }
};

#define SOLVE_CUDA(call)                                                            \
  do {                                                                              \
    cudaError_t ce_ = (call);                                                       \
    if (ce_ != cudaSuccess) {                                                       \
      set_last_error(std::string(#call) + ": " + cudaGetErrorString(ce_));          \
      return ce_ == cudaErrorMemoryAllocation ? GFGPU_E_NOMEM : GFGPU_E_CUDA;       \
    }                                                                               \
  } while (0)

int read_err(Plan &P) {
  int herr = 0;
  SOLVE_CUDA(cudaMemcpyAsync(&herr, P.d_err, sizeof(int), cudaMemcpyDeviceToHost, P.stream));
  SOLVE_CUDA(cudaStreamSynchronize(P.stream));
  if (herr & ERR_CAPACITY) {
    set_last_error("a constrained row has no diagonal entry in the pattern");
    return GFGPU_E_STATE;
  }
  if (herr & ERR_NAN) {
    set_last_error("zero or missing diagonal entry (Jacobi preconditioner)");
    return GFGPU_E_NAN;
  }
  return GFGPU_OK;
}

}  // namespace

extern "C" int gfgpu_dirichlet_eliminate(gfgpu_plan *plan, const int64_t *dofs, int64_t n,
                                         const double *values, double *rhs) {
  Plan *P = reinterpret_cast<Plan *>(plan);
  if (!P || n < 0 || (n > 0 && !dofs)) {
    set_last_error("gfgpu_dirichlet_eliminate: bad arguments");
    return GFGPU_E_INVALID;
  }
  if (P->nnz < 0) {
    set_last_error("no assembled matrix: assemble order 2 first");
    return GFGPU_E_STATE;
  }
  std::vector<uint8_t> mask(size_t(P->n_dof), 0);
  std::vector<double> g(size_t(P->n_dof), 0.0);
  for (int64_t k = 0; k < n; ++k) {
    if (dofs[k] < 0 || dofs[k] >= P->n_dof) {
      set_last_error("gfgpu_dirichlet_eliminate: DOF index out of range");
      return GFGPU_E_INVALID;
    }
    mask[size_t(dofs[k])] = 1;
    g[size_t(dofs[k])] = values ? values[k] : 0.0;
  }
  uint8_t *dm = nullptr;
  double *dg = nullptr;
  SOLVE_CUDA(cudaMalloc(&dm, mask.size()));
  if (cudaMalloc(&dg, g.size() * sizeof(double)) != cudaSuccess) {
    cudaFree(dm);
    set_last_error("gfgpu_dirichlet_eliminate: out of device memory");
    return GFGPU_E_NOMEM;
  }
  cudaError_t ce = cudaMemcpyAsync(dm, mask.data(), mask.size(), cudaMemcpyHostToDevice, P->stream);
  if (ce == cudaSuccess)
    ce = cudaMemcpyAsync(dg, g.data(), g.size() * sizeof(double), cudaMemcpyHostToDevice, P->stream);
  if (ce == cudaSuccess) ce = cudaMemsetAsync(P->d_err, 0, sizeof(int), P->stream);
  if (ce == cudaSuccess && P->n_dof > 0) {
    dirichlet_rows<<<unsigned((P->n_dof + 255) / 256), 256, 0, P->stream>>>(
        P->n_dof, P->d_rowptr, P->d_colidx, P->d_vals, dm, dg, rhs, P->d_err);
    ce = cudaGetLastError();
  }
  if (ce == cudaSuccess) ce = cudaStreamSynchronize(P->stream);
  cudaFree(dm);
  cudaFree(dg);
  if (ce != cudaSuccess) {
    set_last_error(std::string("gfgpu_dirichlet_eliminate: ") + cudaGetErrorString(ce));
    return GFGPU_E_CUDA;
  }
  P->launches++;
  return read_err(*P);
}

extern "C" int gfgpu_cg(gfgpu_plan *plan, const double *b, double *x, double resmax,
                        int64_t maxiter, int32_t precond, int64_t *iterations, double *residual) {
  Plan *P = reinterpret_cast<Plan *>(plan);
  if (!P || !b || !x || resmax < 0 || maxiter < 0 || precond < 0 || precond > 1) {
    set_last_error("gfgpu_cg: bad arguments");
    return GFGPU_E_INVALID;
  }
  if (P->nnz < 0) {
    set_last_error("no assembled matrix: assemble order 2 first");
    return GFGPU_E_STATE;
  }
  const int64_t n = P->n_dof;
  cudaStream_t st = P->stream;
  const unsigned vb = unsigned(std::min<int64_t>((n + kSolveThreads - 1) / kSolveThreads, 1184));
  const unsigned sb = spmv_blocks(*P);
  const unsigned nbp = std::max(vb, sb);
  CgScratch W;
  SOLVE_CUDA(cudaMalloc(&W.r, n * sizeof(double) + 8));
  SOLVE_CUDA(cudaMalloc(&W.p, n * sizeof(double) + 8));
  SOLVE_CUDA(cudaMalloc(&W.q, n * sizeof(double) + 8));
  SOLVE_CUDA(cudaMalloc(&W.part, nbp * sizeof(double)));
  SOLVE_CUDA(cudaMalloc(&W.part2, nbp * sizeof(double)));
  SOLVE_CUDA(cudaMalloc(&W.sc, 8 * sizeof(double)));
  // scalars: sc[0] rho, sc[1] q.p, sc[2] r.r, sc[3] rho_old, sc[4] b.b
  if (precond == 1) {
    SOLVE_CUDA(cudaMalloc(&W.z, n * sizeof(double) + 8));
    SOLVE_CUDA(cudaMalloc(&W.dinv, n * sizeof(double) + 8));
  }
  SOLVE_CUDA(cudaMemsetAsync(P->d_err, 0, sizeof(int), st));
  const unsigned eb = unsigned((n + 255) / 256);
  double h[8];
  if (n <= kCgSmallMax) {
    // one block runs the solve, kCgSegment iterations per launch
    if (precond == 1) {
      diag_inverse<<<eb, 256, 0, st>>>(n, P->d_rowptr, P->d_colidx, P->d_vals, W.dinv, P->d_err);
      P->launches++;
    }
    for (int resume = 0;; resume = 1) {
      cg_small_kernel<<<1, kCgSmallThreads, 0, st>>>(n, P->d_rowptr, P->d_colidx, P->d_vals, b,
                                                     x, W.r, W.p, W.q, W.z,
                                                     precond == 1 ? W.dinv : nullptr, resmax,
                                                     maxiter, resume, kCgSegment, W.sc);
      P->launches++;
      SOLVE_CUDA(cudaGetLastError());
      SOLVE_CUDA(cudaMemcpyAsync(h, W.sc, 8 * sizeof(double), cudaMemcpyDeviceToHost, st));
      SOLVE_CUDA(cudaStreamSynchronize(st));
      if (h[6] != 0.0) break;
    }
    if (iterations) *iterations = int64_t(h[0]);
    if (residual) *residual = h[1];
    int rc = read_err(*P);
    if (rc) return rc;
    if (std::isnan(h[2])) {
      set_last_error("gfgpu_cg: residual is NaN");
      return GFGPU_E_NAN;
    }
    return GFGPU_OK;
  }
  // ||b||
  dot_kernel<<<vb, kSolveThreads, 0, st>>>(n, b, b, W.part);
  finish_sum<<<1, kSolveThreads, 0, st>>>(W.part, vb, W.sc + 4);
  SOLVE_CUDA(cudaMemcpyAsync(h, W.sc + 4, sizeof(double), cudaMemcpyDeviceToHost, st));
  SOLVE_CUDA(cudaStreamSynchronize(st));
  const double rhsn = std::sqrt(std::fabs(h[0]));
  int64_t nit = 0;
  double res = 0.0;
  if (rhsn == 0.0) {
    SOLVE_CUDA(cudaMemsetAsync(x, 0, n * sizeof(double), st));
  } else {
    if (precond == 1)
      diag_inverse<<<eb, 256, 0, st>>>(n, P->d_rowptr, P->d_colidx, P->d_vals, W.dinv, P->d_err);
    // r = b - A x; z = P r; rho = z.r; p = z
    spmv(*P, x, W.q, nullptr, nullptr, st);
    residual_init<<<eb, 256, 0, st>>>(n, b, W.q, W.r);
    const double *z = W.r;
    if (precond == 1) {
      copy_scale<<<eb, 256, 0, st>>>(n, W.r, W.dinv, W.z);
      z = W.z;
    }
    dot_kernel<<<vb, kSolveThreads, 0, st>>>(n, W.r, W.r, W.part);
    finish_sum<<<1, kSolveThreads, 0, st>>>(W.part, vb, W.sc + 2);
    dot_kernel<<<vb, kSolveThreads, 0, st>>>(n, z, W.r, W.part);
    finish_sum<<<1, kSolveThreads, 0, st>>>(W.part, vb, W.sc + 0);
    copy_scale<<<eb, 256, 0, st>>>(n, z, nullptr, W.p);
    SOLVE_CUDA(cudaGetLastError());
    for (;;) {
      SOLVE_CUDA(cudaMemcpyAsync(h, W.sc + 2, sizeof(double), cudaMemcpyDeviceToHost, st));
      SOLVE_CUDA(cudaStreamSynchronize(st));
      res = std::sqrt(h[0]);
      if (std::isnan(res)) break;
      if (res <= rhsn * resmax || nit >= maxiter) break;
      if (nit > 0) {
        // rho_old = rho; rho = z.r (r.r for the identity); p = z + rho/rho_old p
        SOLVE_CUDA(cudaMemcpyAsync(W.sc + 3, W.sc + 0, sizeof(double), cudaMemcpyDeviceToDevice,
                                   st));
        if (precond == 1) {
          finish_sum<<<1, kSolveThreads, 0, st>>>(W.part2, vb, W.sc + 0);
        } else {
          SOLVE_CUDA(cudaMemcpyAsync(W.sc + 0, W.sc + 2, sizeof(double), cudaMemcpyDeviceToDevice,
                                     st));
        }
        cg_direction<<<eb, 256, 0, st>>>(n, W.sc + 0, W.sc + 3, z, W.p);
      }
      // q = A p; q.p; alpha; x += alpha p; r -= alpha q
      spmv(*P, W.p, W.q, W.p, W.part, st);
      finish_sum<<<1, kSolveThreads, 0, st>>>(W.part, sb, W.sc + 1);
      cg_step<<<vb, kSolveThreads, 0, st>>>(n, W.sc, x, W.r, W.p, W.q, W.dinv, W.z, W.part,
                                            W.part2);
      finish_sum<<<1, kSolveThreads, 0, st>>>(W.part, vb, W.sc + 2);
      SOLVE_CUDA(cudaGetLastError());
      ++nit;
      P->launches += 5;
    }
  }
  if (iterations) *iterations = nit;
  if (residual) *residual = rhsn == 0.0 ? 0.0 : res / rhsn;
  int rc = read_err(*P);
  if (rc) return rc;
  if (std::isnan(res)) {
    set_last_error("gfgpu_cg: residual is NaN");
    return GFGPU_E_NAN;
  }
  return GFGPU_OK;
}
