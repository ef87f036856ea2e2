// Sparsity pattern build and row gather over element matrices (sm_103a, FP64).
//
// Every element kernel of the backend writes, per element e, its element
// matrix K_e (s x s, s = nb*qd, rows = test DOFs (li,a), row-major with an
// even row stride), an element vector V_e (s) and the drop threshold
// 1e-14 max|K_e| (compile_and_exec.cc:5453) into a scratch array.  The two
// kernels here turn those into the global CSR matrix and vector:
//
//  * pattern (once per mesh): one warp per DOF node gathers the nodes of
//    the node's elements, sorts and uniques them in shared memory, and marks
//    the (row component, column component) pairs that at least one element
//    inserts, i.e. |e| > threshold (add_elem_matrix, compile_and_exec.cc:
//    4853-4936: an entry exists if any element inserted it; sums that cancel
//    stay stored).  Row lengths, column indices, a node-level slot list with
//    keep bits, and the slot of every local node of every adjacent element
//    (slotmap) are written.
//
//  * gather (every assembly): one warp per DOF node walks the node's
//    elements in ascending order.  The node's rows of K_e are double-buffered
//    in shared memory with cp.async; lane (lj,b) adds K_e[(li,a),(lj,b)] to
//    the row accumulator of slot(lj) when it is above the element's
//    threshold and in the pattern.  Each CSR entry is therefore summed in
//    element order, like the reference's column merge, without atomics:
//    results are bit-reproducible.  The vector is R = sum V_e, where each
//    element kernel has put its whole contribution (K_e u_e + load for a
//    linear form, with no threshold as in the reference's vector assembly,
//    or the element residual of a nonlinear form) into V_e; in the fused
//    K + R assembly of affine simplices V_e holds the load only and the warp
//    adds K u over the node's assembled rows.  The nodes are launched in
//    buckets of similar valence (number of adjacent elements), each launch
//    with its own shared-memory footprint.
#include <atomic>
#include <cub/cub.cuh>
#include <type_traits>

#include "k_common.cuh"
#include "plan.h"

namespace gfgpu {

namespace {

constexpr int kMaxLocal = 128;  // local nodes per element held in shared memory
constexpr int kWarpsPerBlock = 4;

// ------------------------------------------------------------- pattern

template <int MODE>
__global__ void __launch_bounds__(128) pattern_kernel(
    int64_t n_nodes, KeLayout L, const int32_t *__restrict__ adj_ptr,
    const int32_t *__restrict__ adj, const int32_t *__restrict__ enode,
    const double *__restrict__ elem, int cap, int64_t *__restrict__ rowcount,
    int64_t *__restrict__ ncount, const int64_t *__restrict__ rowptr,
    int32_t *__restrict__ colidx, const int64_t *__restrict__ nptr, int32_t *__restrict__ ncol,
    uint16_t *__restrict__ nbits, int16_t *__restrict__ slotmap, int *__restrict__ err) {
  extern __shared__ int smem[];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  int *cand = smem + wib * (3 * cap + kMaxLocal);
  unsigned *bits = reinterpret_cast<unsigned *>(cand + cap);
  int *keptidx = reinterpret_cast<int *>(bits + cap);
  int *ljs = keptidx + cap;
  const int64_t node = blockIdx.x * int64_t(blockDim.x >> 5) + wib;
  if (node >= n_nodes) return;
  const int nb = L.nb, qd = L.qd;
  const int a0 = adj_ptr[node], a1 = adj_ptr[node + 1];
  int n = 0;
  for (int k = a0; k < a1; ++k) {
    const int el = adj[k] / nb;
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
  const int ns = warp_unique(cand, n);
  for (int j = lane; j < ns; j += kWarp) bits[j] = 0u;
  __syncwarp();
  for (int k = a0; k < a1; ++k) {
    const int el = adj[k] / nb, li = adj[k] % nb;
    const double *Ke = elem + int64_t(el) * L.stride;
    const unsigned long long thr = abs_key(Ke[L.off_thr]);
    for (int j = lane; j < nb; j += kWarp) ljs[j] = bsearch_slot(cand, ns, enode[int64_t(el) * nb + j]);
    __syncwarp();
    for (int c = lane; c < nb * qd; c += kWarp) {
      const int lj = c / qd, b = c % qd;
      unsigned m = 0u;
      for (int a = 0; a < qd; ++a)
        if (abs_greater(Ke[ke_sym_entry(L, li, a, c)], thr))
          m |= 1u << (a * qd + b);
      if (m) atomicOr(&bits[ljs[lj]], m);
    }
    __syncwarp();
  }
  if (MODE == 0) {
    for (int a = 0; a < qd; ++a) {
      const unsigned am = ((1u << qd) - 1u) << (a * qd);
      int cnt = 0;
      for (int j = lane; j < ns; j += kWarp) cnt += __popc(bits[j] & am);
      for (int o = 16; o > 0; o >>= 1) cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
      if (lane == 0) rowcount[node * qd + a] = cnt;
    }
    int kept = 0;
    for (int j = lane; j < ns; j += kWarp) kept += bits[j] != 0u;
    for (int o = 16; o > 0; o >>= 1) kept += __shfl_xor_sync(0xffffffffu, kept, o);
    if (lane == 0) ncount[node] = kept;
    return;
  }
  for (int a = 0; a < qd; ++a) {
    const unsigned am = ((1u << qd) - 1u) << (a * qd);
    int64_t base = rowptr[node * qd + a];
    const int64_t rowend = rowptr[node * qd + a + 1];
    for (int j0 = 0; j0 < ns; j0 += kWarp) {
      const int j = j0 + lane;
      const unsigned m = j < ns ? (bits[j] & am) : 0u;
      const int c = __popc(m);
      int incl = c;
      for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += y;
      }
      const int total = __shfl_sync(0xffffffffu, incl, 31);
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
    const int j = j0 + lane;
    const bool keep = j < ns && bits[j] != 0u;
    const unsigned m = __ballot_sync(0xffffffffu, keep);
    const int rank = int(nb0 - nptr[node]) + __popc(m & ((1u << lane) - 1u));
    const int64_t at = nb0 + __popc(m & ((1u << lane) - 1u));
    if (j < ns) keptidx[j] = keep ? rank : -1;
    if (keep) {
      if (at < nend) {
        ncol[at] = cand[j];
        nbits[at] = uint16_t(bits[j]);
      } else {
        set_err(err, ERR_CAPACITY);
      }
    }
    nb0 += __popc(m);
  }
  __syncwarp();
  for (int k = a0; k < a1; ++k) {
    const int el = adj[k] / nb;
    for (int j = lane; j < nb; j += kWarp) {
      const int full = bsearch_slot(cand, ns, enode[int64_t(el) * nb + j]);
      slotmap[int64_t(k) * nb + j] = int16_t(full >= 0 ? keptidx[full] : -1);
    }
  }
}

// -------------------------------------------------------------- gather

// Sums v[0..Q) over the 32 lanes; lane a < Q returns the total of v[a].
// Recursive halving: the first levels exchange half of the components, so
// Q = 3 (padded to 4) takes 6 FP64 adds per lane instead of 15 (a butterfly
// per component).  Fixed order: deterministic.
template <int Q>
__device__ __forceinline__ double warp_sum_components(const double (&v)[Q], int lane) {
  if constexpr (Q == 1) {
    double x = v[0];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
    return x;
  } else {
    // 4 slots: after level 16 a lane keeps the pair {2h, 2h + 1}, after
    // level 8 the component c = 2h + h2, summed over its 8-lane group
    const double w0 = v[0], w1 = Q > 1 ? v[1] : 0.0, w2 = Q > 2 ? v[2] : 0.0,
                 w3 = Q > 3 ? v[3] : 0.0;
    const bool h = (lane >> 4) & 1, h2 = (lane >> 3) & 1;
    double k0 = h ? w2 : w0, k1 = h ? w3 : w1;
    const double s0 = h ? w0 : w2, s1 = h ? w1 : w3;
    k0 += __shfl_xor_sync(0xffffffffu, s0, 16);
    k1 += __shfl_xor_sync(0xffffffffu, s1, 16);
    double x = h2 ? k1 : k0;
    x += __shfl_xor_sync(0xffffffffu, h2 ? k0 : k1, 8);
#pragma unroll
    for (int o = 4; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
    // component a sits in lanes 8a .. 8a + 7
    return __shfl_sync(0xffffffffu, x, (lane & 3) * 8);
  }
}

constexpr int kGatherBufs = 2;  // row blocks per warp: the current one and the next

__host__ __device__ __forceinline__ size_t gather_warp_bytes(int ms, int qd, int rowblk,
                                                             int mad) {
  // row blocks, slot accumulators, element-vector staging (mad * qd),
  // adjacency split, keep bits
  const size_t b = size_t(kGatherBufs * rowblk) * 8 + size_t(ms) * qd * qd * 8 +
                   size_t(mad) * qd * 8 + size_t(mad) * 8 + size_t(ms) * 2;
  return (b + 15) / 16 * 16;
}

// The row gather of one DOF node by one warp (QD components, R =
// ceil(nb*qd/32) lane rounds over the columns of a row); `base` is the
// warp's shared-memory area of gather_warp_bytes(ms, QD, rowblk, mad).
template <int QD, int R, bool UP = false>
__device__ __forceinline__ void gather_node(
    char *base, int64_t node, const KeLayout &L, const int32_t *__restrict__ adj_ptr,
    const int32_t *__restrict__ adj, const double *__restrict__ elem, int ms, int mad,
    const int64_t *__restrict__ nptr, const uint16_t *__restrict__ nbits,
    const int16_t *__restrict__ slotmap, const int64_t *__restrict__ rowptr,
    double *__restrict__ vals, bool want_K, bool want_R, double *__restrict__ vec,
    int *__restrict__ err, const int32_t *__restrict__ ncol = nullptr,
    const double *__restrict__ u = nullptr, UpperOut up = UpperOut{}) {
  constexpr int QQ = QD * QD;
  const int lane = threadIdx.x & 31;
  const int nb = L.nb, S = L.s, blk = L.rowblk;
  double *Kbuf = reinterpret_cast<double *>(base);                // kGatherBufs x blk
  double *acc = Kbuf + kGatherBufs * blk;                          // ms * QQ
  double *vbuf = acc + size_t(ms) * QQ;                            // mad * QD
  int *adjs = reinterpret_cast<int *>(vbuf + size_t(mad) * QD);   // mad
  int *adjl = adjs + mad;                                          // mad
  uint16_t *bits = reinterpret_cast<uint16_t *>(adjl + mad);      // ms
  const int64_t s0 = nptr[node];
  const int ns = int(nptr[node + 1] - s0);
  const int a0 = adj_ptr[node], nadj = adj_ptr[node + 1] - a0;
  if (ns > ms || nadj > mad) {
    if (lane == 0) set_err(err, ERR_CAPACITY);
    return;
  }
  // adjacency codes e*nb + li, split once (lane-parallel): adjs[j] = e,
  // adjl[j] = li
  for (int j = lane; j < nadj; j += kWarp) {
    const int code = adj[a0 + j];
    adjs[j] = code / nb;
    adjl[j] = code - (code / nb) * nb;
  }
  if (want_K) {
    for (int j = lane; j < ns * QQ; j += kWarp) acc[j] = 0.0;
    for (int j = lane; j < ns; j += kWarp) bits[j] = nbits[s0 + j];
  }
  __syncwarp();
  const int nchunk = blk / 2;  // 16-byte chunks of the row block
  // node blocks of kBlk doubles (the simplex pass's vector layouts, at most
  // 64 chunks: nb <= 10 for 3 components): lane-invariant node block j and
  // part of the lane's chunks lane and lane + 32
  constexpr int kBlk = QD == 2 ? 4 : 12, kCpb = kBlk / 2;
  static_assert(kMaxNb * 12 / 2 <= 2 * kWarp, "node-block row chunks exceed two per lane");
  int cj[2], cpart[2];
#pragma unroll
  for (int r = 0; r < 2; ++r) {
    const int c = lane + kWarp * r;
    cj[r] = c < nchunk ? c / kCpb : -1;
    cpart[r] = c - (c / kCpb) * kCpb;
  }
  // the rows of local node li of element k into stage k % kGatherBufs: the
  // contiguous row block (row layout), or its nb node blocks (li, j), those
  // with j < li taken from the stored (j, li)
  auto issue = [&](int k) {
    const double *Ke = elem + int64_t(adjs[k]) * L.stride;
    double *dst = Kbuf + (k % kGatherBufs) * blk;
    const int li = adjl[k];
    if (L.blk) {
#pragma unroll
      for (int r = 0; r < 2; ++r) {
        const int j = cj[r];
        if (j < 0) continue;
        const int lo = j < li ? j : li, hi = j < li ? li : j;
        cp_async16(dst + 2 * (lane + kWarp * r), Ke + ke_block(nb, lo, hi) * kBlk + 2 * cpart[r]);
      }
    } else {
      const double *src = Ke + int64_t(li) * blk;
      for (int c = lane; c < nchunk; c += kWarp) cp_async16(dst + 2 * c, src + 2 * c);
    }
  };
  // per-lane data of an element: slots of the columns the lane handles,
  // threshold, and the element vector entry of component `lane`
  auto fetch = [&](int k, int (&s_)[R], double &t_, double &v_) {
    const int el = adjs[k], li = adjl[k];
    const double *Ke = elem + int64_t(el) * L.stride;
#pragma unroll
    for (int r = 0; r < R; ++r) {
      const int c = lane + 32 * r;
      s_[r] = (c < S && want_K) ? slotmap[int64_t(a0 + k) * nb + c / QD] : -1;
    }
    t_ = Ke[L.off_thr];
    v_ = (want_R && lane < QD) ? Ke[L.off_vec + li * QD + lane] : 0.0;
  };
  // two stages: element k is processed while k+1 is in flight
  int sl0[R];
  double thr0 = 0.0, ve0 = 0.0;
#pragma unroll
  for (int r = 0; r < R; ++r) sl0[r] = -1;
  if (nadj > 0) {
    if (want_K) issue(0);
    fetch(0, sl0, thr0, ve0);
  }
  cp_async_commit();
  double rvec = 0.0;
  // an entry above its element's threshold without a slot: the cached
  // pattern (built from earlier element matrices) misses it
  bool miss = false;
  for (int k = 0; k < nadj; ++k) {
    int sl1[R];
    double thr1 = 0.0, ve1 = 0.0;
#pragma unroll
    for (int r = 0; r < R; ++r) sl1[r] = -1;
    if (k + 1 < nadj) {
      if (want_K) issue(k + 1);
      fetch(k + 1, sl1, thr1, ve1);
    }
    cp_async_commit();
    cp_async_wait1();  // the group of element k is complete
    __syncwarp();
    // fused K + R: the element vectors are staged and summed with K u below
    if (ncol && want_K) {
      if (lane < QD) vbuf[k * QD + lane] = ve0;
    } else {
      rvec += ve0;
    }
    if (want_K) {
      const double *Kb = Kbuf + (k % kGatherBufs) * blk;
      const unsigned long long tb = abs_key(thr0);
      // the node's first element stores into the zeroed accumulators (an
      // element touches each accumulator once): no FP64 add for it.  Node
      // blocks are read as ke_sym_entry reads them: a block (li, lj) with
      // lj < li (staged from (lj, li)) transposed, a diagonal block from its
      // upper half; K is symmetric bit for bit
      const int li0 = adjl[k];
      auto add_block = [&](auto first) {
#pragma unroll
        for (int r = 0; r < R; ++r) {
          const int c = lane + 32 * r;
          if (c < S) {
            const int b = c % QD;
            const unsigned sb = sl0[r] >= 0 ? bits[sl0[r]] : 0u;
            const int lj = c / QD;
            const int c0 = L.blk ? lj * L.blk + b : c;
            const int cstep = L.blk ? QD : L.rowstride;
            const bool lower = L.blk && lj < li0, dblk = L.blk && lj == li0;
#pragma unroll
            for (int a = 0; a < QD; ++a) {
              // (a, b) of the block at c0 - b + a*QD + b; its transpose
              // (b, a) at c0 - b + b*QD + a
              const int off = (lower || (dblk && a > b)) ? c0 - b + b * QD + a : c0 + a * cstep;
              const double x = Kb[off];
              if (abs_greater(x, tb)) {
                if ((sb >> (a * QD + b)) & 1u) {
                  double &dst = acc[(sl0[r] * QD + a) * QD + b];
                  if constexpr (decltype(first)::value) dst = x;
                  else dst += x;
                } else {
                  miss = true;
                }
              }
            }
          }
        }
      };
      if (k == 0) add_block(std::true_type{});
      else add_block(std::false_type{});
    }
    __syncwarp();
#pragma unroll
    for (int r = 0; r < R; ++r) sl0[r] = sl1[r];
    thr0 = thr1, ve0 = ve1;
  }
  if (__any_sync(0xffffffffu, miss) && lane == 0) set_err(err, ERR_PATTERN);
  // ncol given (fused K + R of a linear form): the element vectors held the
  // loads only; add K u over the node's assembled rows (slot s: column node
  // ncol[s0 + s]; entries never added are zero), summed in a fixed order
  double rk = 0.0;
  if (ncol && want_K && want_R) {
    double part[QD];
#pragma unroll
    for (int a = 0; a < QD; ++a) part[a] = 0.0;
    {
      // staged element vectors: lanes < (32/QD)*QD step over them keeping
      // the component lane % QD (one add per 32 entries)
      constexpr int kStep = (kWarp / QD) * QD;
      const int ca = lane % QD;
      double pl = 0.0;
      if (lane < kStep)
        for (int t = lane; t < nadj * QD; t += kStep) pl += vbuf[t];
#pragma unroll
      for (int a = 0; a < QD; ++a)
        if (a == ca) part[a] = pl;
    }
    for (int j = lane; j < ns; j += kWarp) {
      const int64_t cn = ncol[s0 + j];
      double uc[QD];
#pragma unroll
      for (int b = 0; b < QD; ++b) uc[b] = u[cn * QD + b];
#pragma unroll
      for (int a = 0; a < QD; ++a)
#pragma unroll
        for (int b = 0; b < QD; ++b) part[a] = fma(acc[(j * QD + a) * QD + b], uc[b], part[a]);
    }
    rk = warp_sum_components<QD>(part, lane);
  }
  if (want_K) {
#pragma unroll
    for (int a = 0; a < QD; ++a) {
      const unsigned am = ((1u << QD) - 1u) << (a * QD);
      const int64_t row = node * QD + a;
      const int64_t p0 = rowptr[row];
      int64_t p = p0;
      const int64_t pend = rowptr[row + 1];
      // upper-triangle output: entry k of the row (k >= skip[row], the
      // first column >= row) goes to up.vals[up.rowptr[row] + k - skip]
      int64_t ub = 0, ustart = 0, uend = 0;
      if constexpr (UP) {
        ustart = up.rowptr[row];
        ub = ustart - up.skip[row];
        uend = up.rowptr[row + 1];
      }
      for (int j0 = 0; j0 < ns; j0 += kWarp) {
        const int j = j0 + lane;
        const unsigned m = j < ns ? (unsigned(bits[j]) & am) : 0u;
        const int c = __popc(m);
        int incl = c;
        for (int o = 1; o < 32; o <<= 1) {
          const int y = __shfl_up_sync(0xffffffffu, incl, o);
          if (lane >= o) incl += y;
        }
        int64_t q = p + incl - c;
        if (m) {
#pragma unroll
          for (int b = 0; b < QD; ++b)
            if (m & (1u << (a * QD + b))) {
              const double x = acc[(j * QD + a) * QD + b];
              if constexpr (!UP) {
                if (q < pend) vals[q] = x;
                else set_err(err, ERR_CAPACITY);
              } else {
                const int64_t t = ub + (q - p0);
                if (t >= ustart) {
                  if (t < uend) up.vals[t] = x;
                  else set_err(err, ERR_CAPACITY);
                }
              }
              ++q;
            }
        }
        p += __shfl_sync(0xffffffffu, incl, 31);
      }
    }
  }
  if (want_R && lane < QD) {
    rvec += rk;
    if (!isfinite(rvec)) set_err(err, ERR_NAN);
    vec[node * QD + lane] = rvec;
  }
}

// Warps take the nodes i0, i0 + 1, ... < i1 of `order` (or the nodes i
// themselves when order is null).
// BW: the largest block (warps) the instance is compiled for; the register
// budget follows it: 40 resident warps per SM (10 blocks of 4 warps, the
// shared-memory limit of the common buckets), 47 registers per thread, no
// spills
template <int QD, int R, bool UP = false, int BW = 4>
__global__ void __launch_bounds__(32 * BW, 40 / BW) gather_kernel(
    int64_t i0, int64_t i1, const int32_t *__restrict__ order, KeLayout L,
    const int32_t *__restrict__ adj_ptr, const int32_t *__restrict__ adj,
    const double *__restrict__ elem, int ms, int mad, const int64_t *__restrict__ nptr,
    const uint16_t *__restrict__ nbits, const int16_t *__restrict__ slotmap,
    const int64_t *__restrict__ rowptr, double *__restrict__ vals, bool want_K, bool want_R,
    double *__restrict__ vec, int *__restrict__ err, const int32_t *__restrict__ ncol,
    const double *__restrict__ u, UpperOut up) {
  extern __shared__ __align__(16) double dsm[];
  const int wib = threadIdx.x >> 5;
  char *base = reinterpret_cast<char *>(dsm) + wib * gather_warp_bytes(ms, QD, L.rowblk, mad);
  const int64_t i = i0 + blockIdx.x * int64_t(blockDim.x >> 5) + wib;
  if (i >= i1) return;
  const int64_t node = order ? int64_t(order[i]) : i;
  gather_node<QD, R, UP>(base, node, L, adj_ptr, adj, elem, ms, mad, nptr, nbits, slotmap, rowptr,
                         vals, want_K, want_R, vec, err, ncol, u, up);
}

// Upper-triangle pattern of a CSR with sorted columns: skip[r] = number of
// entries of row r with a column < r; ulen[r] = the others.
__global__ void upper_count_kernel(int64_t n, const int64_t *__restrict__ rowptr,
                                   const int32_t *__restrict__ colidx, int32_t *__restrict__ skip,
                                   int64_t *__restrict__ ulen) {
  const int64_t r = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  if (r >= n) return;
  int64_t lo = rowptr[r], hi = rowptr[r + 1];
  const int64_t start = lo, end = hi;
  while (lo < hi) {  // first column >= r
    const int64_t mid = (lo + hi) >> 1;
    if (int64_t(colidx[mid]) < r) lo = mid + 1;
    else hi = mid;
  }
  skip[r] = int32_t(lo - start);
  ulen[r] = end - lo;
}

// Upper-triangle column indices (entries k >= skip[r] of every row).
__global__ void upper_fill_kernel(int64_t n, const int64_t *__restrict__ rowptr,
                                  const int32_t *__restrict__ colidx,
                                  const int32_t *__restrict__ skip,
                                  const int64_t *__restrict__ urowptr,
                                  int32_t *__restrict__ ucol) {
  const int64_t r = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  if (r >= n) return;
  const int64_t s = rowptr[r] + skip[r], len = urowptr[r + 1] - urowptr[r];
  for (int64_t k = 0; k < len; ++k) ucol[urowptr[r] + k] = colidx[s + k];
}

// Vector-only gather (no matrix): one thread per DOF node adds the QD
// components of its adjacent elements' vectors in adjacency order, the
// order gather_node sums them in, so R is the same bit for bit; no shared
// memory, so the launch runs at full occupancy.
template <int QD>
__global__ void __launch_bounds__(256) vector_gather_kernel(
    int64_t n0, int64_t n1, KeLayout L, const int32_t *__restrict__ adj_ptr,
    const int32_t *__restrict__ adj, const double *__restrict__ elem,
    double *__restrict__ vec, int *__restrict__ err) {
  const int64_t node = n0 + blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  if (node >= n1) return;
  const int a0 = adj_ptr[node], a1 = adj_ptr[node + 1];
  const int nb = L.nb;
  double r[QD];
#pragma unroll
  for (int a = 0; a < QD; ++a) r[a] = 0.0;
  for (int k = a0; k < a1; ++k) {
    const int code = adj[k];
    const int e = code / nb;
    const double *v = elem + int64_t(e) * L.stride + L.off_vec + (code - e * nb) * QD;
#pragma unroll
    for (int a = 0; a < QD; ++a) r[a] += v[a];
  }
  bool bad = false;
#pragma unroll
  for (int a = 0; a < QD; ++a) {
    bad |= !isfinite(r[a]);
    vec[node * QD + a] = r[a];
  }
  if (bad) set_err(err, ERR_NAN);
}

// Row gather of a batch by valence class: warp w takes entry w of `list`
// (item << 32 | DOF node of the item's mesh); every node of a class has at
// most ms slots and mad adjacent elements, so a launch reserves only its own
// class's shared memory (as the single-mesh gather's valence buckets do).
template <int QD>
__global__ void __launch_bounds__(128) batch_gather_list_kernel(
    const BatchItem *__restrict__ items, const int64_t *__restrict__ list, int64_t n, int ms,
    int mad, size_t warp_bytes) {
  extern __shared__ __align__(16) double dsm[];
  const int wib = threadIdx.x >> 5;
  const int64_t g = blockIdx.x * int64_t(blockDim.x >> 5) + wib;
  if (g >= n) return;
  char *base = reinterpret_cast<char *>(dsm) + wib * warp_bytes;
  const int64_t code = list[g];
  const BatchItem &it = items[code >> 32];
  gather_node<QD, 1>(base, code & 0xffffffffll, it.L, it.adj_ptr, it.adj, it.elem, ms, mad,
                     it.nptr, it.nbits, it.slotmap, it.rowptr, it.vals, true, true, it.vec, it.err,
                     it.ncol, it.u);
}

size_t pattern_smem(int cap) { return size_t(kWarpsPerBlock) * (3 * cap + kMaxLocal) * sizeof(int); }

int pattern_cap(const Plan &P) {
  int cap = P.max_cand < 32 ? 32 : P.max_cand;
  int np = 1;
  while (np < cap) np <<= 1;
  return np;
}

template <int QD, int R, bool UP>
cudaError_t launch_gather_tu(Plan &P, bool want_K, bool want_R, int64_t i0, int64_t i1,
                             const int32_t *order, int ms, int mad) {
  ms = ms < 1 ? 1 : ms;
  mad = mad < 1 ? 1 : mad;
  // warps per block: the plan's (autotuned), fewer when the block would
  // exceed the shared memory of an SM
  static int smem_max = 0;
  if (!smem_max) {
    int dev = 0;
    cudaGetDevice(&dev);
    if (cudaDeviceGetAttribute(&smem_max, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) !=
        cudaSuccess)
      smem_max = 48 * 1024;
  }
  const size_t wb = gather_warp_bytes(ms, QD, P.lay.rowblk, mad);
  int warps = P.tune.gather_warps;
  while (warps > 1 && size_t(warps) * wb > size_t(smem_max)) warps /= 2;
  const size_t smem = size_t(warps) * wb;
  // the dynamic shared-memory limit of this instantiation, raised only when
  // a launch needs more (per device; a host call between launches otherwise)
  static std::atomic<int> limit[16];
  int dev = 0;
  cudaError_t ce = cudaGetDevice(&dev);
  if (ce != cudaSuccess) return ce;
  if (dev < 0 || dev >= 16 || int(smem) > limit[dev].load()) {
    ce = cudaFuncSetAttribute(gather_kernel<QD, R, UP, 4>,
                              cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
    if (ce != cudaSuccess) return ce;
    ce = cudaFuncSetAttribute(gather_kernel<QD, R, UP, 8>,
                              cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
    if (ce != cudaSuccess) return ce;
    if (dev >= 0 && dev < 16) {
      int cur = limit[dev].load();
      while (int(smem) > cur && !limit[dev].compare_exchange_weak(cur, int(smem))) {
      }
    }
  }
  if (i1 <= i0) return cudaSuccess;
  const unsigned blocks = unsigned((i1 - i0 + warps - 1) / warps);
  auto kern = warps > 4 ? gather_kernel<QD, R, UP, 8> : gather_kernel<QD, R, UP, 4>;
  kern<<<blocks, warps * 32, smem, P.stream>>>(
      i0, i1, order, P.lay, P.d_adj_ptr, P.d_adj, P.d_elem, ms, mad, P.d_nptr, P.d_nbits,
      P.d_slotmap, P.d_rowptr, P.d_vals, want_K, want_R, P.d_vec, P.d_err,
      P.r_from_rows ? P.d_ncol : nullptr, P.slot_ptr[GFGPU_SLOT_U],
      UP ? UpperOut{P.d_uvals, P.d_urowptr, P.d_uskip} : UpperOut{});
  P.launches++;
  return cudaGetLastError();
}

template <int QD, int R>
cudaError_t launch_gather_t(Plan &P, bool want_K, bool want_R, int64_t i0, int64_t i1,
                            const int32_t *order, int ms, int mad) {
  // the upper-triangle output is a separate instance: the plain gather
  // carries none of its work
  if (P.upper_out) return launch_gather_tu<QD, R, true>(P, want_K, want_R, i0, i1, order, ms, mad);
  return launch_gather_tu<QD, R, false>(P, want_K, want_R, i0, i1, order, ms, mad);
}

template <int QD>
cudaError_t launch_gather_q(Plan &P, bool want_K, bool want_R, int64_t i0, int64_t i1,
                            const int32_t *order, int ms, int mad) {
  const int rounds = (P.lay.s + 31) / 32;
  switch (rounds) {
    case 1: return launch_gather_t<QD, 1>(P, want_K, want_R, i0, i1, order, ms, mad);
    case 2: return launch_gather_t<QD, 2>(P, want_K, want_R, i0, i1, order, ms, mad);
    case 3: return launch_gather_t<QD, 3>(P, want_K, want_R, i0, i1, order, ms, mad);
    case 4: return launch_gather_t<QD, 4>(P, want_K, want_R, i0, i1, order, ms, mad);
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t launch_vector_gather(Plan &P, int64_t n0, int64_t n1) {
  if (n1 <= n0) return cudaSuccess;
  constexpr int kThreads = 256;
  const unsigned blocks = unsigned((n1 - n0 + kThreads - 1) / kThreads);
  switch (P.qdim) {
    case 1:
      vector_gather_kernel<1><<<blocks, kThreads, 0, P.stream>>>(
          n0, n1, P.lay, P.d_adj_ptr, P.d_adj, P.d_elem, P.d_vec, P.d_err);
      break;
    case 2:
      vector_gather_kernel<2><<<blocks, kThreads, 0, P.stream>>>(
          n0, n1, P.lay, P.d_adj_ptr, P.d_adj, P.d_elem, P.d_vec, P.d_err);
      break;
    case 3:
      vector_gather_kernel<3><<<blocks, kThreads, 0, P.stream>>>(
          n0, n1, P.lay, P.d_adj_ptr, P.d_adj, P.d_elem, P.d_vec, P.d_err);
      break;
    default: return cudaErrorInvalidValue;
  }
  P.launches++;
  return cudaGetLastError();
}

cudaError_t launch_gather_list(Plan &P, bool want_K, bool want_R, int64_t i0, int64_t i1,
                               const int32_t *order, int ms, int mad) {
  switch (P.qdim) {
    case 1: return launch_gather_q<1>(P, want_K, want_R, i0, i1, order, ms, mad);
    case 2: return launch_gather_q<2>(P, want_K, want_R, i0, i1, order, ms, mad);
    case 3: return launch_gather_q<3>(P, want_K, want_R, i0, i1, order, ms, mad);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace

cudaError_t launch_pattern_count(Plan &P) {
  const int cap = pattern_cap(P);
  const size_t smem = pattern_smem(cap);
  cudaError_t ce = cudaFuncSetAttribute(pattern_kernel<0>,
                                        cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
  if (ce != cudaSuccess) return ce;
  const unsigned blocks = unsigned((P.n_nodes + kWarpsPerBlock - 1) / kWarpsPerBlock);
  pattern_kernel<0><<<blocks, kWarpsPerBlock * 32, smem, P.stream>>>(
      P.n_nodes, P.lay, P.d_adj_ptr, P.d_adj, P.d_enode, P.d_elem, cap, P.d_count, P.d_ncount,
      nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, P.d_err);
  P.launches++;
  return cudaGetLastError();
}

cudaError_t launch_pattern_fill(Plan &P) {
  const int cap = pattern_cap(P);
  const size_t smem = pattern_smem(cap);
  cudaError_t ce = cudaFuncSetAttribute(pattern_kernel<1>,
                                        cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
  if (ce != cudaSuccess) return ce;
  const unsigned blocks = unsigned((P.n_nodes + kWarpsPerBlock - 1) / kWarpsPerBlock);
  pattern_kernel<1><<<blocks, kWarpsPerBlock * 32, smem, P.stream>>>(
      P.n_nodes, P.lay, P.d_adj_ptr, P.d_adj, P.d_enode, P.d_elem, cap, nullptr, nullptr,
      P.d_rowptr, P.d_colidx, P.d_nptr, P.d_ncol, P.d_nbits, P.d_slotmap, P.d_err);
  P.launches++;
  return cudaGetLastError();
}

cudaError_t launch_upper_count(Plan &P, int64_t *d_ulen) {
  if (P.n_dof == 0) return cudaSuccess;
  const unsigned blocks = unsigned((P.n_dof + 255) / 256);
  upper_count_kernel<<<blocks, 256, 0, P.stream>>>(P.n_dof, P.d_rowptr, P.d_colidx, P.d_uskip,
                                                   d_ulen);
  P.launches++;
  return cudaGetLastError();
}

cudaError_t launch_upper_fill(Plan &P, int32_t *d_ucol) {
  if (P.n_dof == 0) return cudaSuccess;
  const unsigned blocks = unsigned((P.n_dof + 255) / 256);
  upper_fill_kernel<<<blocks, 256, 0, P.stream>>>(P.n_dof, P.d_rowptr, P.d_colidx, P.d_uskip,
                                                  P.d_urowptr, d_ucol);
  P.launches++;
  return cudaGetLastError();
}

size_t batch_gather_class_bytes(const BatchItem &it, int ms, int mad) {
  return gather_warp_bytes(ms, it.qd, it.L.rowblk, mad);
}

cudaError_t launch_batch_gather_list(const BatchItem *items, const int64_t *list, int64_t n,
                                     int qd, int ms, int mad, size_t warp_bytes,
                                     cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  const size_t smem = size_t(kWarpsPerBlock) * warp_bytes;
  const unsigned blocks = unsigned((n + kWarpsPerBlock - 1) / kWarpsPerBlock);
  switch (qd) {
    case 1:
      batch_gather_list_kernel<1><<<blocks, kWarpsPerBlock * 32, smem, st>>>(items, list, n, ms,
                                                                              mad, warp_bytes);
      break;
    case 2:
      batch_gather_list_kernel<2><<<blocks, kWarpsPerBlock * 32, smem, st>>>(items, list, n, ms,
                                                                              mad, warp_bytes);
      break;
    case 3:
      batch_gather_list_kernel<3><<<blocks, kWarpsPerBlock * 32, smem, st>>>(items, list, n, ms,
                                                                              mad, warp_bytes);
      break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

cudaError_t batch_gather_attr(size_t smem) {
  cudaError_t ce;
  if ((ce = cudaFuncSetAttribute(batch_gather_list_kernel<1>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem))) !=
      cudaSuccess)
    return ce;
  if ((ce = cudaFuncSetAttribute(batch_gather_list_kernel<2>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem))) !=
      cudaSuccess)
    return ce;
  return cudaFuncSetAttribute(batch_gather_list_kernel<3>,
                              cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
}

cudaError_t launch_gather_range(Plan &P, bool want_K, bool want_R, int64_t n0, int64_t n1) {
  if (!want_K) return want_R ? launch_vector_gather(P, n0, n1) : cudaSuccess;
  return launch_gather_list(P, want_K, want_R, n0, n1, nullptr, P.max_slots, P.max_adj);
}

cudaError_t launch_gather_chunk(Plan &P, bool want_R, int c) {
  const int nmb = int(P.h_bucket.size()) - 1;
  if (P.d_corder && nmb > 0 && P.bucket_ms.size() == size_t(nmb) &&
      P.h_cbucket.size() == size_t(kHostChunks) * (nmb + 1)) {
    const int64_t *cb = P.h_cbucket.data() + size_t(c) * (nmb + 1);
    for (int m = 0; m < nmb; ++m) {
      if (cb[m + 1] <= cb[m]) continue;
      cudaError_t ce = launch_gather_list(P, true, want_R, cb[m], cb[m + 1], P.d_corder,
                                          P.bucket_ms[m], P.bucket_mad[m]);
      if (ce != cudaSuccess) return ce;
    }
    return cudaSuccess;
  }
  const int64_t n0 = P.n_nodes * c / kHostChunks, n1 = P.n_nodes * (c + 1) / kHostChunks;
  return launch_gather_range(P, true, want_R, n0, n1);
}

// The whole gather: one launch per valence bucket (nodes with similar
// element counts, so the 4 warps of a block finish together and each launch
// reserves only its own bucket's shared memory), else one launch over all
// nodes; a vector-only gather is one thread per node.
cudaError_t launch_gather(Plan &P, bool want_K, bool want_R) {
  if (!want_K) return launch_gather_range(P, want_K, want_R, 0, P.n_nodes);
  if (P.d_order && P.bucket_ms.size() + 1 == P.h_bucket.size()) {
    for (size_t b = 0; b + 1 < P.h_bucket.size(); ++b) {
      cudaError_t ce = launch_gather_list(P, want_K, want_R, P.h_bucket[b], P.h_bucket[b + 1],
                                          P.d_order, P.bucket_ms[b], P.bucket_mad[b]);
      if (ce != cudaSuccess) return ce;
    }
    return cudaSuccess;
  }
  return launch_gather_range(P, want_K, want_R, 0, P.n_nodes);
}

}  // namespace gfgpu
