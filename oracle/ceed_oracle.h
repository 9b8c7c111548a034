/*
 * CPU oracle for the tensor-H1 hexahedral operator-apply path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of the algorithm
 * of libCEED's serial reference backend (`/cpu/self/ref/serial`) for the one
 * path that the GB300 backend accelerates.  Only the test suite, the smoke
 * check and the CPU-baseline leg of the benchmark may load it, and only as the
 * checker or the timed CPU baseline.  The product library never links it.
 *
 * Parity pin: tests/golden/ holds vectors produced by the real reference
 * (oracle/Makefile builds libCEED's interface + ref backend + gallery from
 * the reference sources; oracle/ref_harness.c drives it through the public
 * libCEED API).  tests/test_oracle_golden.py checks this restatement against
 * those vectors.
 *
 * Layout conventions (all follow the reference CPU backend):
 *   L-vector   : node-major, component k of node n at off + k*comp_stride
 *   E-vector   : [elem][comp][node]  (backends/ref/ceed-ref-restriction.c:767-779)
 *   Q-vector   : per element [eval-dim][comp][qpt]  (backends/ref/ceed-ref-basis.c:88-91)
 *   qdata      : [elem][comp][qpt]  (CEED_STRIDES_BACKEND on the ref backend)
 *   1D matrices: row-major Q x P  (include/ceed-impl.h CeedBasis_private)
 */
#ifndef CEED_ORACLE_H
#define CEED_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum { ORC_GAUSS = 0, ORC_GAUSS_LOBATTO = 1 };
enum { ORC_NOTRANSPOSE = 0, ORC_TRANSPOSE = 1 };
enum { ORC_EVAL_NONE = 0, ORC_EVAL_INTERP = 1, ORC_EVAL_GRAD = 2, ORC_EVAL_WEIGHT = 16 };

/* QFunction kinds of the gallery (include/ceed/jit-source/gallery/ *.h) plus the
 * kappa-weighted diffusion used by the differentiable operator. */
enum {
  ORC_QF_MASS_APPLY          = 0, /* ceed-massapply.h            */
  ORC_QF_POISSON3D_APPLY     = 1, /* ceed-poisson3dapply.h       */
  ORC_QF_VECMASS_APPLY       = 2, /* ceed-vectormassapply.h      */
  ORC_QF_VECPOISSON3D_APPLY  = 3, /* ceed-vectorpoisson3dapply.h */
  ORC_QF_POISSON3D_KAPPA     = 4, /* Poisson3DApply with qdata scaled by kappa per point */
};

/* Counter-based splitmix64 stream: value i of stream `seed`, uniform on [lo, hi). */
double orc_uniform(uint64_t seed, uint64_t i, double lo, double hi);
void   orc_fill_uniform(uint64_t seed, int64_t n, double lo, double hi, double *x);

/* Quadrature rules and the 1D Lagrange basis on Gauss-Lobatto nodes. */
int orc_gauss_quadrature(int Q, double *q_ref, double *q_weight);
int orc_lobatto_quadrature(int Q, double *q_ref, double *q_weight);
int orc_h1_lagrange_1d(int P, int Q, int quad_mode, double *interp_1d, double *grad_1d, double *q_ref_1d, double *q_weight_1d);
int orc_collocated_grad(int P, int Q, const double *interp_1d, const double *grad_1d, double *collo_grad_1d);

/* Structured box mesh on [0,1]^3 with nx*ny*nz hexahedra. */
void orc_box_vertices(int nx, int ny, int nz, double noise, uint64_t seed, double *coords);
void orc_box_offsets(int nx, int ny, int nz, int P, int ncomp_interlaced, int32_t *offsets);

/* Element restriction. */
void orc_rstr_gather(int64_t num_elem, int elem_size, int num_comp, int64_t comp_stride, const int32_t *offsets, const double *l_vec,
                     double *e_vec);
void orc_rstr_scatter_add(int64_t num_elem, int elem_size, int num_comp, int64_t comp_stride, const int32_t *offsets, const double *e_vec,
                          double *l_vec);

/* Tensor basis on `num_elem` elements, E/Q layouts as described above. */
int orc_basis_apply(int dim, int P, int Q, int num_comp, const double *interp_1d, const double *grad_1d, const double *q_weight_1d,
                    int64_t num_elem, int t_mode, int eval_mode, const double *u, double *v);

/* Geometric factors: coordinates on the vertex grid through a trilinear (P=2) basis. */
int orc_qdata_build(int nx, int ny, int nz, int Q, int quad_mode, int kind_poisson, const double *coords, double *qdata);

/* Operator apply: v = A u (Apply semantics: v is overwritten).  kappa may be NULL. */
typedef struct {
  int            qf;         /* ORC_QF_* */
  int            P, Q;       /* 1D nodes / quadrature points */
  int            num_comp;   /* field components (1 or 3) */
  int64_t        num_elem;
  int64_t        comp_stride;
  int64_t        l_size;     /* length of u and v */
  const int32_t *offsets;    /* [num_elem][P^3] */
  const double  *interp_1d;  /* Q x P */
  const double  *grad_1d;    /* Q x P */
  const double  *qdata;      /* [elem][qcomp][Q^3] */
  const double  *kappa;      /* [elem][Q^3] or NULL */
} orc_operator;

int orc_operator_apply(const orc_operator *op, const double *u, double *v, int add);

/* The same apply in the blocked form of /cpu/self/opt/blocked (ceed_oracle_blocked.c): blocks of 8 elements with the
 * element index innermost.  Requires Q >= P.  Equal to orc_operator_apply up to the order of the scatter's additions
 * within a block. */
int orc_operator_apply_blocked(const orc_operator *op, const double *u, double *v, int add);

/* Adjoint of the kappa-weighted diffusion with respect to kappa:
 * g[e][q] = sum_ij (grad w)_i D_ij (grad u)_j at point q (w = output cotangent). */
int orc_kappa_grad(const orc_operator *op, const double *u, const double *w, double *g);

#ifdef __cplusplus
}
#endif
#endif
