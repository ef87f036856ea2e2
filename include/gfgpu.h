/*
 * gfgpu — GB300 (sm_103a) backend for GetFEM's generic assembly hot path.
 *
 * C ABI only: plain pointers and sizes, no C++ or torch types, no
 * exceptions.  Every entry point returns a gfgpu_status (0 = success); the
 * text of the last error of the calling thread is available from
 * gfgpu_last_error().
 *
 * The hot path this library replaces is the execution of compiled GWFL
 * instructions over every element and Gauss point:
 *   ga_workspace::assembly           src/getfem_generic_assembly_workspace.cc:791
 *   ga_exec                          src/getfem_generic_assembly_compile_and_exec.cc:8750-9047
 * A host-side shim in ga_workspace::assembly lowers the analysed GWFL tree to
 * a gfgpu_form (the point where ga_compile starts,
 * compile_and_exec.cc:8030-8047), creates one plan per (mesh_im, region,
 * expression set) and calls gfgpu_assemble*; unsupported trees are rejected
 * with GFGPU_E_UNSUPPORTED at plan creation.  There is no CPU fallback.
 */
#ifndef GFGPU_H
#define GFGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
  GFGPU_OK = 0,
  GFGPU_E_INVALID = 1,     /* bad argument (the GMM_ASSERT1 size checks) */
  GFGPU_E_UNSUPPORTED = 2, /* element / integration / expression not lowered */
  GFGPU_E_CUDA = 3,        /* CUDA runtime error or no device */
  GFGPU_E_JACOBIAN = 4,    /* det of the geometric transformation is 0
                              ("Non invertible matrix",
                              bgeot_geometric_trans.cc:380) */
  GFGPU_E_NAN = 5,         /* non-finite value produced on the device */
  GFGPU_E_TIMEOUT = 6,     /* a bounded device-side wait gave up */
  GFGPU_E_NOMEM = 7,       /* device allocation failed */
  GFGPU_E_STATE = 8        /* call out of sequence (e.g. no pattern yet) */
} gfgpu_status;

/* Element families: GT_PK(dim,1) + FEM_PK(dim,degree) and
   GT_QK(dim,1) + FEM_QK(dim,degree). */
typedef enum { GFGPU_SIMPLEX = 0, GFGPU_HEX = 1 } gfgpu_elem_kind;

/* ------------------------------------------------------------------ */
/* Form descriptor: the lowered GWFL expression                        */
/* ------------------------------------------------------------------ */

/* Where a scalar coefficient comes from. */
typedef enum {
  GFGPU_COEF_NONE = 0,
  GFGPU_COEF_CONST = 1,   /* a fixed-size constant (add_fixed_size_constant) */
  GFGPU_COEF_ELEMENT = 2, /* one value per element: a FEM_PK/QK(dim,0)
                             constant (add_fem_constant on a P0 mesh_fem) */
  GFGPU_COEF_NODAL = 3    /* a scalar field on the variable's scalar mesh_fem,
                             interpolated at each Gauss point */
} gfgpu_coef_kind;

typedef struct {
  int32_t kind;  /* gfgpu_coef_kind */
  int32_t slot;  /* data slot for ELEMENT / NODAL (gfgpu_set_data) */
  double value;  /* CONST value; multiplies ELEMENT / NODAL values */
} gfgpu_coef;

typedef enum {
  /* int D(x) : Grad_u (x) Grad_Test_u with the isotropic tensor
     D[a,k,b,l] = c0 d_ak d_bl + c1 d_ab d_kl + c2 d_al d_kb
     (test component a, derivative k; trial component b, derivative l).
     Scalar Laplacian: c1.  Linear elasticity (lambda*Div_u*Id+2*mu*Sym(Grad_u)):
     c0 = lambda, c1 = c2 = mu. */
  GFGPU_TERM_GRADGRAD = 1,
  /* int c u.Test_u */
  GFGPU_TERM_MASS = 2,
  /* int f.Test_u with f a field on the variable's mesh_fem (qdim
     components, slot `field_slot`), scaled by c[0] (CONST 1 if NONE) */
  GFGPU_TERM_SOURCE = 3,
  /* int ((Id+Grad_u)*Compressible_Neo_Hookean_PK2(Grad_u,[C1;D1])):Grad_Test_u
     (getfem_nonlinear_elasticity.cc:2319-2320, law :503-600), C1 = c[0],
     D1 = c[1]; dim 3 only */
  GFGPU_TERM_NEOHOOKEAN = 4,
  /* A displacement / pressure pair whose pressure p is an internal im_data
     variable (ga_workspace::add_internal_im_variable, getfem/
     getfem_generic_assembly.h:459; one scalar per element Gauss point,
     index e*nq + q as im_data::index_of_point numbers them for a mesh_im
     over all convexes, src/getfem_im_data.cc:110-118, :187-197):
       u equation   (c[0] p Id(dim)) : Grad_Test_u
       p equation   scale (p + c[2] p^3 + c[1] Div_u) Test_p
     field_slot: p (n_elements*nq values); aux_slot: the residual of the p
     rows that static condensation reads (the internal part of the assembled
     vector, workspace.cc:826-833).  3-D vector fields (qdim == dim == 3),
     Gauss-point kernel, at most one such term per form.  Order 1 assembles
     the u residual and the p residual (gfgpu_copy_result
     GFGPU_RESULT_INTERNAL); order 2 needs GFGPU_CONDENSATION. */
  GFGPU_TERM_INTERNAL_P = 5,
  /* int (D : Grad_u) : Grad_Test_u with a constant, possibly anisotropic
     tensor D[(a,k),(b,l)] (test component a, derivative k; trial component
     b, derivative l): gfgpu_form.tensor holds its (qdim*dim)^2 entries,
     row (a,k) = a*dim + k, column (b,l) = b*dim + l, and must be symmetric
     (D[(a,k),(b,l)] == D[(b,l),(a,k)], so that K is).  The term is scaled
     by scale * c[0] (c[0] NONE: 1; CONST or ELEMENT).  Examples:
     (A*Grad_u).Grad_Test_u for a scalar field and a symmetric matrix A
     (D[(0,k),(0,l)] = A[k,l]); (Reshape(C,3,3,3,3):Grad_u):Grad_Test_u
     for a 3-D vector field and a stiffness C with major symmetry
     (D[(a,k),(b,l)] = C[a,k,b,l]).  Plans on affine simplices only (the
     Gauss-point and hexahedral kernels, batches and the allocation-free
     entry reject it), at most one per form, orders 1 and 2 (not
     potentials). */
  GFGPU_TERM_GRADGRAD_TENSOR = 6
} gfgpu_term_kind;

typedef struct {
  int32_t kind;       /* gfgpu_term_kind */
  int32_t field_slot; /* SOURCE: the load field; INTERNAL_P: p */
  double scale;       /* overall factor of the term (e.g. -1) */
  gfgpu_coef c[3];
  int32_t aux_slot;   /* INTERNAL_P: residual of the p rows (order 2) */
  int32_t reserved;
} gfgpu_term;

#define GFGPU_MAX_TERMS 8
/* entries of the constant tensor of a GFGPU_TERM_GRADGRAD_TENSOR term:
   (qdim*dim)^2 <= 81 */
#define GFGPU_MAX_TENSOR 81
typedef struct {
  int32_t n_terms;
  gfgpu_term terms[GFGPU_MAX_TERMS];
  double tensor[GFGPU_MAX_TENSOR]; /* D of the GRADGRAD_TENSOR term, if any */
} gfgpu_form;

/* Data slots.  Slot 0 is the variable u (n_dof values). */
#define GFGPU_SLOT_U 0
#define GFGPU_MAX_SLOTS 8
/* Pseudo-slot naming the mesh vertex coordinates (gfgpu_potential_gradient). */
#define GFGPU_SLOT_POINTS (-1)

/* The discretisation: mesh, mesh_fem DOF map and mesh_im.  All arrays are
   host memory and are copied at plan creation. */
typedef struct {
  int32_t dim;        /* 2 or 3 */
  int32_t kind;       /* gfgpu_elem_kind */
  int32_t degree;     /* K of FEM_PK/FEM_QK */
  int32_t qdim;       /* 1 or dim */
  const char *im;     /* "IM_TRIANGLE(2)", "IM_TETRAHEDRON(5)",
                         "IM_GAUSS_PARALLELEPIPED(3,5)", ... */
  int64_t n_points;
  int64_t n_elements;
  int64_t n_dof;
  const double *points;  /* n_points x dim */
  const int64_t *cvpts;  /* n_elements x (dim+1 | 2^dim) */
  const int64_t *dofs;   /* n_elements x nb: first-component DOF of each
                            local node (mesh_fem::ind_scalar_basic_dof_of_element,
                            getfem/getfem_mesh_fem.h:461) */
} gfgpu_space;

typedef struct gfgpu_plan_s gfgpu_plan;

/* ------------------------------------------------------------------ */
/* Library                                                              */
/* ------------------------------------------------------------------ */
const char *gfgpu_version(void);
const char *gfgpu_last_error(void);

/* ------------------------------------------------------------------ */
/* Input builders (host only).  These mirror the reference routines a
   caller without GetFEM needs to produce a gfgpu_space.               */
/* ------------------------------------------------------------------ */

/* getfem::regular_unit_mesh (src/getfem_regular_meshes.cc:237) with
   GT_PK(dim,1) (kind SIMPLEX) or GT_QK(dim,1) (kind HEX).  Call with
   points == NULL to get the sizes.  jitter (optional) holds
   (nx+1)^dim x dim offsets in lattice order, applied to interior vertices. */
int gfgpu_regular_unit_mesh(int32_t dim, int32_t kind, int32_t nx, const double *jitter,
                            int64_t *n_points, int64_t *n_elements,
                            double *points, int64_t *cvpts);

/* mesh_fem::enumerate_dof (src/getfem_mesh_fem.cc:320) for FEM_PK/QK(dim,degree)
   with qdim components.  dofs: n_elements x nb (see gfgpu_space.dofs). */
int gfgpu_enumerate_dofs(int32_t dim, int32_t kind, int32_t degree, int32_t qdim,
                         int64_t n_elements, const int64_t *cvpts,
                         int64_t *dofs, int64_t *n_dof);
/* The same numbering computed on the device (sort of packed node keys;
   meshes of fewer than 2^25 vertices and 2^32 element nodes, degree <= 4):
   host arrays in and out, same results as gfgpu_enumerate_dofs. */
int gfgpu_enumerate_dofs_device(int32_t dim, int32_t kind, int32_t degree, int32_t qdim,
                                int64_t n_elements, const int64_t *cvpts,
                                int64_t *dofs, int64_t *n_dof);
/* 1 when a CUDA device is visible, else 0. */
int gfgpu_device_available(void);

/* Number of local scalar basis functions of FEM_PK/QK(dim,degree). */
int gfgpu_nb_basis(int32_t dim, int32_t kind, int32_t degree, int32_t *nb);

/* Integration method tables (approx_integration points and weights,
   src/getfem_integration.cc): call with pts == NULL to get nq. */
int gfgpu_quadrature(const char *im, int32_t *dim, int32_t *nq, double *pts, double *w);

/* Base values (nq x nb) and reference gradients (nq x nb x dim) of
   FEM_PK/QK(dim,degree) at the points of `im` (fem_precomp_,
   getfem/getfem_fem.h:653-700). */
int gfgpu_basis_tables(int32_t dim, int32_t kind, int32_t degree, const char *im,
                       double *val, double *grad);

/* ------------------------------------------------------------------ */
/* Plans: one per (discretisation, form).  One GPU, one stream per plan;
   a plan is not shared between host threads.                          */
/* ------------------------------------------------------------------ */

/* Uploads the mesh, DOF map and tables; lowers the form.  Returns
   GFGPU_E_UNSUPPORTED for element/integration/form combinations the
   kernels do not implement.  cuda_stream is a cudaStream_t (NULL = the
   default stream). */
int gfgpu_plan_create(const gfgpu_space *space, const gfgpu_form *form, void *cuda_stream,
                      gfgpu_plan **plan);
void gfgpu_plan_destroy(gfgpu_plan *plan);

/* Sets data slot `slot` (n values).  on_device != 0: `values` is a device
   pointer that the plan reads in place at each assembly (no copy); else
   the host values are copied to a plan-owned device buffer now. */
int gfgpu_set_data(gfgpu_plan *plan, int32_t slot, const double *values, int64_t n,
                   int32_t on_device);

/* Sparsity pattern (CSR, rows = test DOFs, columns ascending).  Built on
   the device at the first order-2 assembly with the reference's rule: an
   element entry e is inserted only if |e| > 1e-14 * max|elem|
   (compile_and_exec.cc:4889, :5453), the union over elements is kept, and
   entries that sum to zero stay stored.  Later assemblies reuse it; when an
   element entry above its threshold has no slot in it (an entry that was
   exactly zero at the build, e.g. a tangent at u = 0), the gather flags it
   and gfgpu_sync rebuilds the pattern from the current element matrices and
   gathers again (pointers from gfgpu_device_csr and earlier sizes are then
   stale).  gfgpu_assemble_host returns GFGPU_E_STATE if its pattern grew. */
int gfgpu_pattern_size(gfgpu_plan *plan, int64_t *n_rows, int64_t *nnz);
int gfgpu_pattern_copy(gfgpu_plan *plan, int64_t *rowptr, int32_t *colidx);
/* Device pointers of the plan's CSR (valid until the plan is destroyed or
   the pattern is rebuilt). */
int gfgpu_device_csr(gfgpu_plan *plan, const int64_t **rowptr, const int32_t **colidx,
                     double **vals);
/* Device pointer of the plan's assembled vector (n_dof). */
int gfgpu_device_vector(gfgpu_plan *plan, double **vec);

#define GFGPU_REBUILD_PATTERN 1 /* rebuild the CSR pattern at this call */
#define GFGPU_WITH_VECTOR 2     /* order 2: also produce the order-1 vector
                                   in the same pass */
#define GFGPU_PROFILE 4         /* record CUDA events around each kernel of
                                   this call (gfgpu_kernel_times) */
#define GFGPU_SUM_FACTORISATION 16 /* order 1 on parallelepiped hexahedra with a
                                   scalar form and the pattern built: the
                                   matrix-free R = K u + load by 1D
                                   contractions with the exact tensor-product
                                   basis, also for FEM_QK(3,3|4), where the
                                   reference's monomial evaluation of the basis
                                   is off the tensor product by 1e-12..1.5e-10
                                   (so R differs from the reference's at that
                                   level); FEM_QK(3,1|2) use it by default */
#define GFGPU_CONDENSATION 8    /* order 2 of a form with an INTERNAL_P term:
                                   static condensation of p
                                   (ga_workspace::assembly(2, true),
                                   compile_and_exec.cc:5562-5790, :8429-8640).
                                   K <- K_uu - K_up K_pp^-1 K_pu (condensed,
                                   into the CSR); vector <- -K_up K_pp^-1 R_p
                                   (the prim rows of the reference's V, which
                                   it zeroes first); GFGPU_RESULT_INTERNAL <-
                                   K_pp^-1 R_p / (w J) per Gauss point;
                                   GFGPU_RESULT_COUPLING <- K_pp^-1 K_pu, one
                                   row of nb*qdim entries per Gauss point
                                   (the internal coupling matrix KQJpr,
                                   getfem_generic_assembly.h:409-419) */

/* Assembles on the device.  order 2: K values into the plan's CSR (the
   pattern is built at the first call, or when GFGPU_REBUILD_PATTERN);
   order 1: the residual vector; order 0: the potential (*potential, host).
   Results overwrite the plan's buffers; a caller that accumulates (as
   GetFEM does into an external K, workspace.cc:803-845) adds them. */
int gfgpu_assemble(gfgpu_plan *plan, int32_t order, int32_t flags, double *potential);

/* Assembly from and to host memory, for callers holding host buffers:
   copies u (slot 0, n_dof doubles) to the device, assembles order 2 and
   order 1, and copies the K values (nnz) and the residual (n_dof) back.
   Any of u / vals / vec may be NULL to skip that copy. */
int gfgpu_assemble_host(gfgpu_plan *plan, const double *u, double *vals, double *vec);

/* The same for a symmetric K, delivering only its upper triangle: the values
   of the entries with column >= row, row by row in the order of
   gfgpu_pattern_upper (about half of nnz), so that half the bytes cross the
   host link.  K is symmetric bit for bit for every form without an
   INTERNAL_P term (each element kernel computes a symmetric element matrix
   once per entry pair and mirrors it; GetFEM's own K is symmetric for these
   forms too), so mirroring the upper values gives the full K exactly.  A
   GetFEM-side caller adds each value at (i, j) and, off the diagonal, at
   (j, i) when it copies the result into its col_matrix (the add of
   workspace.cc:803-845).  GFGPU_E_UNSUPPORTED for a form with an INTERNAL_P
   term.  The plan's device CSR values (gfgpu_device_csr) are not updated by
   this call. */
int gfgpu_assemble_host_upper(gfgpu_plan *plan, const double *u, double *upper_vals,
                              double *vec);

/* Upper triangle of the plan's pattern (entries with column >= row):
   *nnz_upper, and when non-NULL the row pointers (n_dof + 1 int64) and the
   column indices (nnz_upper int32), host memory. */
int gfgpu_pattern_upper(gfgpu_plan *plan, int64_t *nnz_upper, int64_t *rowptr,
                        int32_t *colidx);

/* Copies a result of the plan into caller memory (host or device; the
   copy direction is inferred from the pointer):
   which = 0: row pointers (n_dof+1 int64), 1: column indices (nnz int32),
   2: K values (nnz double), 3: assembled vector (n_dof double).
   Waits for the copy to finish. */
#define GFGPU_RESULT_ROWPTR 0
#define GFGPU_RESULT_COLIDX 1
#define GFGPU_RESULT_VALUES 2
#define GFGPU_RESULT_VECTOR 3
/* Forms with an INTERNAL_P term (n_int = n_elements * nq rows, index
   e*nq + q; each coupling row has nb*qdim entries, the element's DOFs in
   local order (node-major, component fastest), stored unsorted and without
   the 1e-14 drop of add_elem_matrix):
   4: internal vector (n_int double): order 1 the p residual, order 2 with
      condensation the internal solution K_pp^-1 R_p / (w J);
   5: coupling values (n_int * nb*qdim double), 6: their column DOFs
      (n_int * nb*qdim int32). */
#define GFGPU_RESULT_INTERNAL 4
#define GFGPU_RESULT_COUPLING 5
#define GFGPU_RESULT_COUPLING_COLIDX 6
int gfgpu_copy_result(gfgpu_plan *plan, int32_t which, void *dst);
/* Sizes of the internal-variable results: n_int rows, row_len entries per
   coupling row (0, 0 for forms without an INTERNAL_P term). */
int gfgpu_internal_size(gfgpu_plan *plan, int64_t *n_int, int64_t *row_len);

/* Adjoint of the potential (order-0 assembly of the plan's form, with u and
   the data fixed) with respect to
     slot >= 1            a coefficient slot of the form: per-element data
                          (n = n_elements) or nodal data (n = n_dof / qdim);
     GFGPU_SLOT_POINTS    the mesh vertex coordinates (n = n_points * dim),
                          the DOF values held fixed (shape derivative).
   grad is device memory if on_device, else host memory; waits for the
   result.  In the reference the coefficient gradient is the order-1
   assembly of the potential with that datum declared as a variable
   (ga_workspace::add_fem_variable + assembly(1), GWFL Diff,
   getfem_generic_assembly_workspace.cc:791); the shape derivative has no
   counterpart there. */
int gfgpu_potential_gradient(gfgpu_plan *plan, int32_t slot, double *grad, int64_t n,
                             int32_t on_device);

/* Replaces the mesh vertex coordinates (n = n_points * dim doubles, device
   memory if on_device); the DOF map and the CSR pattern are kept.  Waits for
   the copy.  Hexahedra are checked again for parallelepipeds: a plan whose
   order-1/2 kernel needs them (scalar isotropic forms on parallelepipeds)
   then returns GFGPU_E_UNSUPPORTED from those assemblies until the points
   form parallelepipeds again; potentials (order 0) stay available. */
int gfgpu_set_points(gfgpu_plan *plan, const double *points, int64_t n, int32_t on_device);

/* Dirichlet conditions by elimination on the plan's assembled K (after an
   order-2 assembly), as the reference model's dof constraints on a linear
   symmetric problem (getfem_models.cc:2806-2870): for the n constrained
   DOFs dofs[k] with values g_k (values may be NULL for zeros),
   rhs -= K(:, D) g on the other rows, rhs(D) = g, rows and columns D of K
   cleared and K(d,d) = 1.  rhs is a device vector of n_dof entries (or NULL
   to change K only).  The CSR pattern is kept.  Waits for the result. */
int gfgpu_dirichlet_eliminate(gfgpu_plan *plan, const int64_t *dofs, int64_t n,
                              const double *values, double *rhs);

/* Conjugate gradients on the plan's K: gmm::cg (gmm/gmm_solver_cg.h:84-157)
   with precond 0 = identity, 1 = diagonal (Jacobi), and gmm::iteration's
   stop rule (gmm/gmm_iter.h:113-150): stops when ||r||_2 <= ||b||_2 resmax
   or after maxiter iterations; x = 0 when b = 0.  b and x are device
   vectors of n_dof entries; x holds the initial guess and receives the
   solution.  *iterations and *residual (= ||r|| / ||b||) are optional. */
int gfgpu_cg(gfgpu_plan *plan, const double *b, double *x, double resmax, int64_t maxiter,
             int32_t precond, int64_t *iterations, double *residual);

/* ------------------------------------------------------------------ */
/* Batched assembly of many meshes (independent plans), few launches. */
/* The reference assembles one mesh per ga_workspace::assembly call;   */
/* a batch replaces a loop of such calls over independent workspaces.  */
typedef struct gfgpu_batch_s gfgpu_batch;

/* Groups n affine-simplex plans (each assembled once at order 2, so that
   its CSR pattern exists, and with u and its data set) into one batch.
   The plans' device buffers are referenced, not copied: data changed in
   place (coefficients, u) is seen by the next batched assembly; a plan
   whose data pointers change must be re-batched. */
int gfgpu_batch_create(gfgpu_plan *const *plans, int32_t n, gfgpu_batch **out);
/* K values and order-1 vectors of every plan of the batch: one persistent
   element-pass launch per element type over the elements of all its meshes,
   and one row-gather launch per component count and valence class (the DOF
   nodes of all meshes with at most 2^c adjacent elements), on `stream`.
   Only kernel launches and a memset of the error word are issued, so the
   call can be captured in a CUDA graph and replayed. */
int gfgpu_batch_assemble(gfgpu_batch *batch, void *cuda_stream);
/* Times the element-pass launches over grid sizes of 1, 2, 4, ..., 32
   blocks per SM and keeps the fastest (optional outputs: that grid, and the
   number of row-gather launches, whose grids follow their node counts). */
int gfgpu_batch_tune(gfgpu_batch *batch, void *cuda_stream, int32_t *grid_elem,
                     int32_t *gather_launches);
/* Waits for `stream` and reports the batch's device error word. */
int gfgpu_batch_sync(gfgpu_batch *batch, void *cuda_stream);
int64_t gfgpu_batch_elements(gfgpu_batch *batch);
void gfgpu_batch_destroy(gfgpu_batch *batch);

/* Waits for the plan's stream and reports the device error word
   (GFGPU_E_JACOBIAN / GFGPU_E_NAN) of the last assembly. */
int gfgpu_sync(gfgpu_plan *plan);

/* Durations (ms, CUDA events on the plan's stream) of the kernels of the
   last gfgpu_assemble call made with GFGPU_PROFILE: times[0] = element
   pass, times[1] = row gather.  Waits for the stream. */
int gfgpu_kernel_times(gfgpu_plan *plan, float *times, int32_t n);

/* Throughput microbenchmark of this GPU's FP64 FMA pipe (kind 0), FP64
   tensor pipe (kind 1, mma.sync m8n8k4 f64), or both at once (kind 2: half
   the warps on each; near the sum of the two when they do not share issue
   resources, near either alone when they do), in TFLOP/s; used as the
   compute roofline of the FP64 kernels. */
int gfgpu_fp64_peak(int32_t kind, double *tflops);

/* ------------------------------------------------------------------ */
/* Vector assembly that allocates no device memory.                    */
/* This entry point has no counterpart in the reference.               */
/* ------------------------------------------------------------------ */

/* Some callers cannot allocate device memory: code that works inside a
   memory budget owned by another allocator (a framework's caching
   allocator, an arena sized at start-up, a solver embedded in a host
   program that hands it a fixed pool) must not call cudaMalloc behind that
   allocator's back.  For them, gfgpu_assemble_vector_noalloc assembles the
   vector (order 1) of an affine-simplex form -- the same result as a plan's
   gfgpu_assemble(plan, 1) -- from the caller's device arrays into the
   caller's device output, and calls no cudaMalloc, cudaFree or other
   allocating routine.

   Its scratch (one vector of rowstride doubles per element, rowstride = the
   element's DOF count rounded up to 4) lives in a static device array of
   GFGPU_NOALLOC_SCRATCH_BYTES that every GPU which loads the library holds
   until the process exits.  The largest mesh is
   GFGPU_NOALLOC_SCRATCH_BYTES / (8 * rowstride) elements: 524 288 P2
   tetrahedra with 3 components (rowstride 32), 1 398 101 with one
   (rowstride 12); larger meshes are rejected with GFGPU_E_INVALID.

   - The first call on a device looks up the device addresses of the static
     arrays (cudaGetSymbolAddress, with that device current) and keeps them
     for the life of the process; make that first call before any stream
     capture, and do not use the entry point across a cudaDeviceReset (the
     kept addresses belong to the context that was reset).
   - Every call shares the arrays, which keep the last call's contents: each
     call writes every element's slot before reading it and overwrites the
     output, so nothing has to be cleared, but calls that overlap on the GPU
     race: issue them on one stream, one after another.
   - Each call waits for its stream (cudaStreamSynchronize) to read the
     device error word before returning the status, so it is not an
     asynchronous call.
   - Every pointer the kernels read is checked on the host first: null
     arrays, per-element coefficient or load slots that are missing or out
     of range, and forms of more than GFGPU_MAX_TERMS terms return
     GFGPU_E_INVALID without a launch; an adjacency entry outside
     [0, n_elements * nb) is skipped on the device and reported as
     GFGPU_E_INVALID.

   Inputs (device memory): points (n_points x dim), cvpts (n_elements x
   (dim+1) vertex ids), enode (n_elements x nb: DOF node of each local node,
   i.e. first-component DOF / qdim), the node-to-element adjacency adj_ptr
   (n_nodes + 1) and adj (entries element*nb + local node, ascending element
   order within each node), data slots as for a plan (slot 0 = u).  Output:
   vec (n_nodes*qdim), overwritten. */
#define GFGPU_NOALLOC_SCRATCH_BYTES ((size_t)128 << 20)
typedef struct {
  int32_t dim, degree, qdim;
  const char *im;
  int64_t n_elements, n_nodes;
  const double *points;
  const int32_t *cvpts;
  const int32_t *enode;
  const int32_t *adj_ptr;
  const int32_t *adj;
  const double *slots[GFGPU_MAX_SLOTS];
  double *vec;
} gfgpu_noalloc_args;
int gfgpu_assemble_vector_noalloc(const gfgpu_noalloc_args *args, const gfgpu_form *form,
                                  void *cuda_stream);

/* ------------------------------------------------------------------ */
/* Launch configuration and autotuning.                                 */
/* ------------------------------------------------------------------ */

/* Threads per element of the element pass that stores K_e, and warps per
   block of the row gather (one warp per DOF node).  Candidates:
     ep_threads    affine simplices 2, 4, 8 (warps sharing a 32-element
                   tile: that many threads per element; 4 only for a form
                   with a GRADGRAD_TENSOR term); Gauss-point and
                   parallelepiped hexahedra 128, 256, 512 (the CTA of one
                   element);
     gather_warps  2, 4, 8.
   Every candidate computes each entry with the same operations in the same
   order: K and R are the same bits whatever the configuration.  (The
   reference has no launch configuration; ga_exec runs one element at a
   time, compile_and_exec.cc:8750-8869.) */
typedef struct {
  int32_t ep_threads;
  int32_t gather_warps;
} gfgpu_launch;
int gfgpu_get_launch(gfgpu_plan *plan, gfgpu_launch *launch);
/* GFGPU_E_INVALID for a value that is not a candidate of the plan's kernels. */
int gfgpu_set_launch(gfgpu_plan *plan, const gfgpu_launch *launch);
/* Times every candidate on the plan's own order-2 assembly (K and R; the
   pattern is built first if needed): the element-pass candidates, then the
   gather candidates with the best element pass, `reps` profiled assemblies
   each (median of the CUDA-event times).  Keeps the fastest in the plan,
   records it for plans of the same family on this GPU model (element kind,
   dimension, degree, qdim, kernel), and returns it in *best (may be NULL). */
int gfgpu_tune(gfgpu_plan *plan, int32_t reps, gfgpu_launch *best);
/* The recorded configurations: written to / read from a text file (one
   line per family: "<family>|<GPU name> <ep_threads> <gather_warps>").
   Plans created after gfgpu_tune_load (or a gfgpu_tune of the same family)
   start with the recorded configuration. */
int gfgpu_tune_save(const char *path);
int gfgpu_tune_load(const char *path);

/* Number of kernel launches issued by the plan since creation. */
int64_t gfgpu_launch_count(gfgpu_plan *plan);

#ifdef __cplusplus
}
#endif
#endif /* GFGPU_H */
