// Internal plan structure shared by the C-ABI layer and the kernels.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <vector>

#include "../../include/gfgpu.h"

namespace gfgpu {

// device error word bits
enum : int {
  ERR_JACOBIAN = 1,   // det K == 0
  ERR_NAN = 2,        // non-finite value
  ERR_CAPACITY = 4,   // a node touches more DOF nodes than the kernel holds
  ERR_TIMEOUT = 8,
  ERR_PATTERN = 16    // an element entry above its drop threshold has no slot in
                      // the cached CSR pattern (the pattern must grow)
};

// Terms of the sparse barycentric reference tensor of a P_K simplex:
// grad phi_i = sum_v c_iv grad lambda_v with c_iv = 0 unless vertex v
// carries weight in node i, so
//   int grad_a phi_i grad_b phi_j = |J| sum_{v,w} G[i,j,v,w] g_v[a] g_w[b].
// For each local pair (i,j) the nonzero (v,w) are listed.
constexpr int kMaxNb = 10;      // P2 tetrahedron
constexpr int kMaxPairTerms = 4;  // |supp(i)| * |supp(j)| for degree <= 2

struct SimplexTables {
  int nb, nv, dim;
  // per (i,j): count, packed (v*nv+w), values
  int8_t nterm[kMaxNb * kMaxNb];
  int8_t vw[kMaxNb * kMaxNb * kMaxPairTerms];
  double gval[kMaxNb * kMaxNb * kMaxPairTerms];
  double mass[kMaxNb * kMaxNb];  // reference mass matrix sum_q w_q phi_i phi_j
};

// Upper-triangle output of the row gather (gfgpu_assemble_host_upper):
// entries with column >= row, row r at vals[rowptr[r] ..), skip[r] = the
// entries of row r left of its diagonal.  vals == nullptr: the full CSR.
struct UpperOut {
  double *vals = nullptr;
  const int64_t *rowptr = nullptr;
  const int32_t *skip = nullptr;
};

// Per-element scratch written by every element kernel and read by the
// pattern build and the row gather (doubles):
//   K_e   s x s, row (li,a) = li*qd + a at offset row*rowstride (rowstride even)
//   V_e   s entries at off_vec: the element's contribution to the assembled
//         vector (K_e u_e + load for linear forms, the element residual of a
//         nonlinear form)
//   thr   1e-14 max|K_e| at off_thr
// stride is even, so every element block and every row is 16-byte aligned.
// Two layouts of K_e:
//   rows (blk == 0): row (li,a) at (li*qd + a) * rowstride;
//   upper node blocks (blk > 0, vector fields of the simplex pass): K_e is
//         symmetric and only its node blocks (i,j) with i <= j are stored,
//         block (i,j) at ke_block(nb, i, j) * blk (row by row: (0,0) (0,1)
//         .. (0,nb-1) (1,1) ..), entry (a,b) at a*qd + b; blk = 4 (qd 2) or
//         12 (qd 3, 9 entries and 3 zeros), so every block is whole 32-byte
//         sectors.  Block (i,j), i > j, is block (j,i) transposed.
// rowblk: the doubles of one local node's rows (row layout) or of its nb
// node blocks (node-block layout), the row gather's staging unit.
struct KeLayout {
  int nb = 0, qd = 0, s = 0;
  int rowstride = 0, off_vec = 0, off_thr = 0, stride = 0;
  int blk = 0, rowblk = 0;
  bool linear = true;  // R = K_full u + sum V_e (else R = sum V_e)
};

// index of the stored node block (i,j), i <= j, of the upper node-block layout
__host__ __device__ __forceinline__ int ke_block(int nb, int i, int j) {
  return i * nb - (i * (i - 1)) / 2 + (j - i);
}

// Offset from the element's base of the entry K_e[(li,a), c] (c = lj*qd + b)
// that the pattern build and the row gather use.  Node blocks: a block below
// the diagonal is read transposed from its mirror, and a diagonal block
// (lj == li) from its upper half (a > b reads (b, a)): the simplex pass
// computes the two halves of a diagonal block as the same terms summed in
// another order, and this makes every assembled K symmetric bit for bit.
__host__ __device__ __forceinline__ int ke_sym_entry(const KeLayout &L, int li, int a, int c) {
  if (L.blk) {
    const int lj = c / L.qd, b = c % L.qd;
    const bool tr = lj < li || (lj == li && a > b);
    const int blk = lj < li ? ke_block(L.nb, lj, li) : ke_block(L.nb, li, lj);
    return blk * L.blk + (tr ? b * L.qd + a : a * L.qd + b);
  }
  return li * L.rowblk + a * L.rowstride + c;
}

struct SlotPtrs {
  const double *p[GFGPU_MAX_SLOTS];
};

struct DeviceBuf {
  void *p = nullptr;
  size_t bytes = 0;
};

// pointwise law of a Gauss-point element kernel
enum : int {
  LAW_ISO = 0,  // GRADGRAD / MASS / SOURCE terms: isotropic linear tangent
  LAW_NH = 1    // compressible neo-Hookean PK2 term
};

constexpr int kHostChunks = 16;    // gather chunks of gfgpu_assemble_host
constexpr int kGatherStreams = 3;  // streams the chunks' gathers rotate over

// Launch configuration of a plan's kernels (gfgpu_set_launch, gfgpu_tune).
// ep_threads: threads per element of the element pass that stores K_e:
// affine simplices 2, 4 or 8 (warps sharing a tile of 32 elements, one lane
// per element in each), Gauss-point and parallelepiped hexahedra 128, 256
// or 512 (the CTA of one element).  gather_warps: warps per block of the row
// gather (one warp per DOF node), 2, 4 or 8.  Every choice computes each
// entry with the same operations in the same order: the results are the
// same bits.
struct LaunchConfig {
  int ep_threads = 0;
  int gather_warps = 4;
};

struct Plan {
  LaunchConfig tune;
  // discretisation
  int dim = 0, kind = 0, degree = 0, qdim = 0, nb = 0, nbg = 0, nq = 0;
  int64_t n_points = 0, n_elements = 0, n_dof = 0, n_nodes = 0;
  std::string im;
  gfgpu_form form{};
  cudaStream_t stream = nullptr;
  bool affine_simplex = false;  // simplex element pass applies
  int law = LAW_ISO;
  bool psd = true;

  // device arrays
  double *d_points = nullptr;   // n_points x dim
  int32_t *d_cv = nullptr;      // E x nbg
  int32_t *d_enode = nullptr;   // E x nb  (DOF node ids)
  int32_t *d_adj_ptr = nullptr; // n_nodes + 1
  int32_t *d_adj = nullptr;     // (e*nb + li), sorted by e within a node
  int32_t max_adj = 0;          // largest adjacency
  int32_t max_cand = 0;         // largest sum of nb over a node's elements

  // data slots
  const double *slot_ptr[GFGPU_MAX_SLOTS] = {};
  double *slot_own[GFGPU_MAX_SLOTS] = {};
  int64_t slot_n[GFGPU_MAX_SLOTS] = {};

  // tables
  SimplexTables stab{};
  SimplexTables *d_stab = nullptr;
  KeLayout lay{};
  // Gauss-point tables (hexahedra): values nq x nb, reference gradients
  // nq x nb x dim, geometric gradients nq x nbg x dim, weights nq
  std::vector<double> h_val, h_grad, h_ggrad, h_w;
  double *d_hval = nullptr, *d_hgrad = nullptr, *d_ggrad = nullptr, *d_hw = nullptr;
  // the same tables transposed (Gauss point fastest): values nb x nq,
  // reference gradients (nb*dim) x nq, for kernels with a lane per point
  double *d_hvalT = nullptr, *d_hgradT = nullptr;
  std::vector<int32_t> h_tri;  // upper-triangle entries of K_e (Gauss kernel)
  int32_t *d_tri = nullptr;
  // every element a parallelepiped (hexahedra; checked again by
  // gfgpu_set_points): the Jacobian is constant, and the affine_hex kernels
  // apply
  bool parallelepiped = false;
  // every element an axis-aligned box (edge vectors with one nonzero
  // component each): the off-diagonal metric terms are exactly zero
  bool axis_aligned = false;
  std::vector<int64_t> h_cvpts;  // E x 8 vertex ids of the hexahedra, for that check
  // parallelepiped hexahedra: reference tensors (7 x nb x nb)
  bool affine_hex = false;
  std::vector<double> h_aff;
  double *d_aff = nullptr;
  // sum factorisation of the vector-only pass (tensor-product basis on a
  // parallelepiped): 1D tables, empty when the basis does not factor
  std::vector<double> h_sf;
  double *d_sf = nullptr;
  bool sf_exact = false;      // the 1D tables reproduce the reference's 3-D ones
  bool sf_requested = false;  // GFGPU_SUM_FACTORISATION on the current call
  bool kmat = true;        // an element-matrix kernel exists (orders 1 and 2)
  bool kpot = false;       // the Gauss-point potential kernel exists (order 0)
  // point -> (element, vertex) adjacency, codes e * nbg + v sorted by e
  int32_t *d_padj_ptr = nullptr, *d_padj = nullptr;
  // per-element partials of potentials and gradients (allocated on use)
  double *d_epart = nullptr, *d_npart = nullptr, *d_xpart = nullptr;
  // internal im_data variable (GFGPU_TERM_INTERNAL_P): term index, the
  // mode of the current pass (0 none, 1 order-1 residuals, 2 condensation),
  // the mode the CSR pattern was built in, the per-Gauss-point results
  // (n_elements*nq) and the coupling rows (n_elements*nq x nb*qdim)
  int ip_term = -1;
  int cmode = 0;
  bool last_want_R = false;     // the last gather's vector flag (pattern repair)
  // the fused K + R assembly of an affine-simplex plan: V_e holds the load
  // only and the row gather adds K u from the assembled rows (d_ncol kept)
  bool r_from_rows = false;
  int64_t pattern_builds = 0;
  int pattern_cmode = -1;
  double *d_int = nullptr, *d_kqj = nullptr;
  std::vector<int32_t> h_en;    // E x nb DOF node ids (coupling columns)

  // element pass scratch
  double *d_elem = nullptr;     // E x lay.stride
  // outputs
  int64_t *d_rowptr = nullptr;  // n_dof + 1
  int32_t *d_colidx = nullptr;  // nnz
  double *d_vals = nullptr;     // nnz
  int64_t nnz = -1;
  int64_t *d_nptr = nullptr;    // node-level pattern: n_nodes + 1
  int32_t *d_ncol = nullptr;
  uint16_t *d_nbits = nullptr;  // keep bits (a*qd+b) of each node-level slot
  int16_t *d_slotmap = nullptr; // per adjacency entry and local node: slot or -1
  int32_t max_slots = 0;
  double *d_vec = nullptr;      // n_dof
  double *d_pot = nullptr;      // 1
  int *d_err = nullptr;
  int64_t *d_count = nullptr;   // scratch row counts (n_dof + 1)
  int64_t *d_ncount = nullptr;  // (n_nodes + 1)
  void *d_cub = nullptr;
  size_t cub_bytes = 0;
  int64_t launches = 0;
  cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
  bool profiled = false;
  // host-buffer assembly: row pointers on the host, a copy stream and one
  // event per gather chunk (device-to-host copies overlap the gather)
  std::vector<int64_t> h_rowptr;
  // per gather chunk of DOF nodes: one past the largest element adjacent to
  // a node of the chunk (the element pass runs ahead of the gather that far)
  std::vector<int64_t> h_chunk_eend;
  // valence buckets of the row gather: DOF nodes ordered by bucket
  // (ceil(log2(number of adjacent elements))), node order kept within a
  // bucket; bucket b is d_order[h_bucket[b] .. h_bucket[b+1]) with at most
  // bucket_ms[b] pattern slots (set at the pattern build) and bucket_mad[b]
  // adjacent elements per node
  int32_t *d_order = nullptr;
  std::vector<int64_t> h_bucket;
  std::vector<int32_t> h_order, bucket_ms, bucket_mad;
  // the same buckets within each gather chunk of gfgpu_assemble_host
  // (chunk c: nodes [n0, n1) of the chunk, ordered by bucket, in positions
  // [n0, n1) of d_corder; bucket m of chunk c starts at
  // h_cbucket[c * (buckets + 1) + m])
  int32_t *d_corder = nullptr;
  std::vector<int32_t> h_corder;
  std::vector<int64_t> h_cbucket;
  // gfgpu_assemble_host: the chunks' row gathers on kGatherStreams streams
  // of the device's highest priority (their blocks go ahead of the element
  // pass's ranges on the plan's stream), the copies on two copy streams
  cudaStream_t copy_stream[2] = {nullptr, nullptr};
  cudaStream_t gather_stream[kGatherStreams] = {};
  cudaEvent_t chunk_ev[kHostChunks] = {};
  cudaEvent_t range_ev[kHostChunks] = {};
  // upper triangle of a symmetric K (gfgpu_assemble_host_upper): row
  // pointers (device and host), the entries of each row left of its
  // diagonal, the values; built for the pattern of build number upper_build
  bool symmetric = false;       // the form's K is symmetric bit for bit
  bool upper_out = false;       // the current gather writes d_uvals only
  int64_t *d_urowptr = nullptr;
  int32_t *d_uskip = nullptr;
  double *d_uvals = nullptr;
  int64_t nnz_upper = -1, upper_build = -1;
  std::vector<int64_t> h_urowptr;
};

// One mesh of a batched launch: everything the element pass and the row
// gather of an affine-simplex plan read (device pointers).
struct BatchItem {
  int32_t etype = 0;   // element-pass instance (simplex_batch_type)
  int32_t qd = 1;      // gather: components
  int64_t E = 0, n_nodes = 0;
  const double *pts = nullptr;
  const int32_t *cv = nullptr, *enode = nullptr;
  const SimplexTables *tab = nullptr;
  KeLayout L{};
  gfgpu_form form{};
  SlotPtrs slots{};
  const double *fsrc = nullptr;
  double fscale = 0.0;
  const double *u = nullptr;
  double *elem = nullptr;
  int *err = nullptr;
  const int32_t *adj_ptr = nullptr, *adj = nullptr;
  const int64_t *nptr = nullptr;
  const uint16_t *nbits = nullptr;
  const int16_t *slotmap = nullptr;
  const int64_t *rowptr = nullptr;
  double *vals = nullptr, *vec = nullptr;
  // node-level column lists: the gather forms K u from the assembled rows
  // (the element pass leaves it out)
  const int32_t *ncol = nullptr;
};

// batched launches (k_simplex.cu, k_assemble.cu)
int simplex_batch_type(int dim, int degree, int qdim, bool mass);
void simplex_source_of(const Plan &P, const double *&fsrc, double &fscale, bool &mass);
constexpr int kBatchElementTypes = 16;
cudaError_t launch_batch_element_pass(const BatchItem *items, const int64_t *tile0, int nitems,
                                     int64_t ntiles, int grid, int etype, cudaStream_t st);
size_t batch_gather_class_bytes(const BatchItem &it, int ms, int mad);
cudaError_t launch_batch_gather_list(const BatchItem *items, const int64_t *list, int64_t n,
                                     int qd, int ms, int mad, size_t warp_bytes, cudaStream_t st);
// kernels (k_simplex.cu)
// tiles [tile0, tile1) of 32 elements (tile1 < 0: to the last element);
// ku: V_e includes K_e u_e (false: the load only, K u formed by the gather)
cudaError_t launch_simplex_element_pass(Plan &P, bool with_u, int64_t tile0 = 0,
                                        int64_t tile1 = -1, bool ku = true);
// (k_simplex_ten.cu) the same for forms with a GRADGRAD_TENSOR term, which
// launch_simplex_element_pass hands over to it
bool form_has_tensor(const gfgpu_form &f);
cudaError_t launch_simplex_element_pass_tensor(Plan &P, bool with_u, int64_t tile0, int64_t tile1,
                                               bool ku);
cudaError_t launch_pattern_count(Plan &P);
cudaError_t launch_pattern_fill(Plan &P);
cudaError_t launch_gather(Plan &P, bool want_K, bool want_R);
// the gather of DOF nodes [n0, n1) (their rows of the CSR and of R)
cudaError_t launch_gather_range(Plan &P, bool want_K, bool want_R, int64_t n0, int64_t n1);
// the K (+ R) gather of host chunk c (of kHostChunks), per valence bucket
cudaError_t launch_gather_chunk(Plan &P, bool want_R, int c);
// upper-triangle pattern: per-row counts into d_ulen (and P.d_uskip), then
// the column indices into d_ucol (after P.d_urowptr is scanned)
cudaError_t launch_upper_count(Plan &P, int64_t *d_ulen);
cudaError_t launch_upper_fill(Plan &P, int32_t *d_ucol);
int build_simplex_tables(Plan &P, std::string &err);
int fill_simplex_tables(int dim, int degree, int qdim, const std::string &im, SimplexTables &t,
                        KeLayout &lay, int &nq, std::string &err);
// whether the affine-simplex element pass lowers the form (why: the reason if not)
bool simplex_form_supported(const gfgpu_form &f, int qdim, int dim, std::string &why);
// potentials and adjoint gradients (k_gauss.cu)
bool gauss_potential_available(int dim, int kind, int degree, int qdim, int law);
int build_gauss_tables(Plan &P, std::string &err);
cudaError_t launch_potential(Plan &P, double *d_out);
cudaError_t launch_coef_gradient(Plan &P, int slot, bool nodal, double *d_out);
cudaError_t launch_shape_gradient(Plan &P, double *d_out);
// parallelepiped hexahedra (k_affine_hex.cu)
bool affine_hex_form_ok(const gfgpu_form &f, int qdim);
bool mesh_is_parallelepiped(const double *pts, const int64_t *cv, int64_t E);
bool mesh_is_axis_aligned(const double *pts, const int64_t *cv, int64_t E);
bool affine_hex_available(int degree);
void build_affine_hex_tables(Plan &P);
void build_affine_hex_sumfac(Plan &P);
cudaError_t launch_affine_hex_pass(Plan &P, bool want_K);
// Gauss-point element kernels (k_hex.cu)
bool gauss_element_available(int kind, int law, int degree, int qdim, int nq);
void gauss_element_layout(Plan &P);
cudaError_t launch_hex_element_pass(Plan &P, bool want_K);
cudaError_t launch_simplex_vector_pass(int dim, int degree, int qdim, int64_t E,
                                       const double *pts, const int32_t *cv, const int32_t *enode,
                                       const SimplexTables *tab, const gfgpu_form &form,
                                       const double *const *slot, double *vout, int vstride,
                                       int *err, cudaStream_t stream);

}  // namespace gfgpu
