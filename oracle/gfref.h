/* ORACLE — test infrastructure only (see gfref.cc).  C ABI of the CPU
 * restatement of GetFEM's generic-assembly hot path. */
#ifndef GFREF_H
#define GFREF_H
#include <stdint.h>
#include "../include/gfgpu.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
  int32_t dim, kind, degree, qdim;
  const char *im;
  int64_t n_points, n_elements, n_dof;
  const double *points;
  const int64_t *cvpts;
  const int64_t *dofs;
  gfgpu_form form;
  const double *slots[GFGPU_MAX_SLOTS]; /* slot 0 = u */
} gfref_problem;

/* nthreads <= 0: all OpenMP threads. */
void *gfref_assemble_matrix(const gfref_problem *p, int nthreads, int64_t *nnz);
void gfref_matrix_copy(void *h, int64_t *rowptr, int64_t *colidx, double *vals);
void gfref_matrix_free(void *h);
int gfref_assemble_vector(const gfref_problem *p, int nthreads, double *V);
/* Forms with an internal variable (GFGPU_TERM_INTERNAL_P): order 1 with its
   residual (n_elements * nq), and order 2 with static condensation. */
int gfref_assemble_vector_internal(const gfref_problem *p, int nthreads, double *V,
                                   double *Vint);
void *gfref_assemble_condensed(const gfref_problem *p, int nthreads, int64_t *nnz, double *V,
                               double *Vint, double *coupling);
int gfref_assemble_potential(const gfref_problem *p, int nthreads, double *E);
int gfref_tables(int dim, int kind, int degree, const char *im, int *nq, double *pts,
                 double *w, double *val, double *grad);

#ifdef __cplusplus
}
#endif
#endif
