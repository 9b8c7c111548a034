/*
 * CPU oracle for the tensor-H1 hexahedral operator-apply path.
 *
 * TEST INFRASTRUCTURE ONLY: a restatement of libCEED's serial reference
 * backend used as the checker (and as the timed CPU baseline when the
 * reference library itself cannot run).  Every function names the reference
 * file:line whose algorithm it follows.  Built with -ffp-contract=off so that
 * x86 and Arm hosts round identically, like the reference's -std=c11 build.
 */
#include "ceed_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#define ORC_EPSILON 1e-16 /* include/ceed/ceed-f64.h CEED_EPSILON */

/* ---------------------------------------------------------------------------------------------------------------------
 * Random inputs: counter-based splitmix64, so element i of a stream is independent of how the stream is chunked.
 * -------------------------------------------------------------------------------------------------------------------*/
static inline uint64_t orc_mix(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

double orc_uniform(uint64_t seed, uint64_t i, double lo, double hi) {
  uint64_t z = orc_mix(seed * 0xD1B54A32D192ED03ull + (i + 1) * 0x9E3779B97F4A7C15ull);
  double   u = (double)(z >> 11) * (1.0 / 9007199254740992.0);
  return lo + (hi - lo) * u;
}

void orc_fill_uniform(uint64_t seed, int64_t n, double lo, double hi, double *x) {
  for (int64_t i = 0; i < n; i++) x[i] = orc_uniform(seed, (uint64_t)i, lo, hi);
}

/* ---------------------------------------------------------------------------------------------------------------------
 * Quadrature: Newton iteration on Legendre polynomials.
 * Follows interface/ceed-basis.c:2529-2570 (Gauss) and :2581-2634 (Gauss-Lobatto).
 * -------------------------------------------------------------------------------------------------------------------*/
int orc_gauss_quadrature(int Q, double *q_ref, double *q_weight) {
  const double PI = 4.0 * atan(1.0);

  for (int i = 0; i <= Q / 2; i++) {
    double x = cos(PI * (double)(2 * i + 1) / ((double)(2 * Q)));
    double p0 = 1.0, p1 = x, p2 = 0.0, dp2;

    for (int j = 2; j <= Q; j++) {
      p2 = (((double)(2 * j - 1)) * x * p1 - ((double)(j - 1)) * p0) / ((double)(j));
      p0 = p1;
      p1 = p2;
    }
    dp2 = (x * p2 - p0) * (double)Q / (x * x - 1.0);
    x   = x - p2 / dp2;
    for (int k = 0; k < 100 && fabs(p2) > 10 * ORC_EPSILON; k++) {
      p0 = 1.0;
      p1 = x;
      for (int j = 2; j <= Q; j++) {
        p2 = (((double)(2 * j - 1)) * x * p1 - ((double)(j - 1)) * p0) / ((double)(j));
        p0 = p1;
        p1 = p2;
      }
      dp2 = (x * p2 - p0) * (double)Q / (x * x - 1.0);
      x   = x - p2 / dp2;
    }
    double w = 2.0 / ((1.0 - x * x) * dp2 * dp2);

    q_weight[i]         = w;
    q_weight[Q - 1 - i] = w;
    q_ref[i]            = -x;
    q_ref[Q - 1 - i]    = x;
  }
  return 0;
}

int orc_lobatto_quadrature(int Q, double *q_ref, double *q_weight) {
  const double PI = 4.0 * atan(1.0);

  if (Q < 2) return 1;
  double w = 2.0 / ((double)(Q * (Q - 1)));
  if (q_weight) {
    q_weight[0]     = w;
    q_weight[Q - 1] = w;
  }
  q_ref[0]     = -1.0;
  q_ref[Q - 1] = 1.0;
  for (int i = 1; i <= (Q - 1) / 2; i++) {
    double x = cos(PI * (double)(i) / (double)(Q - 1));
    double p0 = 1.0, p1 = x, p2 = 0.0, dp2, d2p2;

    for (int j = 2; j < Q; j++) {
      p2 = (((double)(2 * j - 1)) * x * p1 - ((double)(j - 1)) * p0) / ((double)(j));
      p0 = p1;
      p1 = p2;
    }
    dp2  = (x * p2 - p0) * (double)Q / (x * x - 1.0);
    d2p2 = (2 * x * dp2 - (double)(Q * (Q - 1)) * p2) / (1.0 - x * x);
    x    = x - dp2 / d2p2;
    for (int k = 0; k < 100 && fabs(dp2) > 10 * ORC_EPSILON; k++) {
      p0 = 1.0;
      p1 = x;
      for (int j = 2; j < Q; j++) {
        p2 = (((double)(2 * j - 1)) * x * p1 - ((double)(j - 1)) * p0) / ((double)(j));
        p0 = p1;
        p1 = p2;
      }
      dp2  = (x * p2 - p0) * (double)Q / (x * x - 1.0);
      d2p2 = (2 * x * dp2 - (double)(Q * (Q - 1)) * p2) / (1.0 - x * x);
      x    = x - dp2 / d2p2;
    }
    w = 2.0 / (((double)(Q * (Q - 1))) * p2 * p2);
    if (q_weight) {
      q_weight[i]         = w;
      q_weight[Q - 1 - i] = w;
    }
    q_ref[i]         = -x;
    q_ref[Q - 1 - i] = x;
  }
  return 0;
}

/* Lagrange basis on P Gauss-Lobatto nodes evaluated at Q points: Fornberg's recurrence for the
 * interpolation weights and first derivatives.  Follows interface/ceed-basis.c:1617-1680. */
int orc_h1_lagrange_1d(int P, int Q, int quad_mode, double *interp_1d, double *grad_1d, double *q_ref_1d, double *q_weight_1d) {
  double *nodes = (double *)calloc((size_t)P, sizeof(double));

  if (!nodes || P < 2 || Q < 1) {
    free(nodes);
    return 1;
  }
  orc_lobatto_quadrature(P, nodes, NULL);
  if (quad_mode == ORC_GAUSS) orc_gauss_quadrature(Q, q_ref_1d, q_weight_1d);
  else if (orc_lobatto_quadrature(Q, q_ref_1d, q_weight_1d)) {
    free(nodes);
    return 1;
  }
  memset(interp_1d, 0, sizeof(double) * (size_t)(P * Q));
  memset(grad_1d, 0, sizeof(double) * (size_t)(P * Q));
  for (int i = 0; i < Q; i++) {
    double c1 = 1.0, c3 = nodes[0] - q_ref_1d[i];

    interp_1d[i * P + 0] = 1.0;
    for (int j = 1; j < P; j++) {
      double c2 = 1.0, c4 = c3;

      c3 = nodes[j] - q_ref_1d[i];
      for (int k = 0; k < j; k++) {
        double dx = nodes[j] - nodes[k];

        c2 *= dx;
        if (k == j - 1) {
          grad_1d[i * P + j]   = c1 * (interp_1d[i * P + k] - c4 * grad_1d[i * P + k]) / c2;
          interp_1d[i * P + j] = -c1 * c4 * interp_1d[i * P + k] / c2;
        }
        grad_1d[i * P + k]   = (c3 * grad_1d[i * P + k] - interp_1d[i * P + k]) / dx;
        interp_1d[i * P + k] = c3 * interp_1d[i * P + k] / dx;
      }
      c1 = c2;
    }
  }
  free(nodes);
  return 0;
}

/* Householder reflection A <- (I - b v v^T) A of the m x n block A (row stride `row`, column stride `col`), v[0] = 1
 * implied; interface/ceed-basis.c:104-112. */
static void orc_householder_reflect(double *A, const double *v, double b, int m, int n, int row, int col) {
  for (int j = 0; j < n; j++) {
    double w = A[j * col];

    for (int i = 1; i < m; i++) w += v[i] * A[i * row + j * col];
    A[j * col] -= b * w;
    for (int i = 1; i < m; i++) A[i * row + j * col] -= b * w * v[i];
  }
}

/* Pseudoinverse of the full-column-rank m x n (m >= n) row-major matrix `mat` into the n x m `pinv`: Householder QR,
 * Q^T applied to the identity, back substitution with R (CeedQRFactorization, CeedHouseholderApplyQ and
 * CeedMatrixPseudoinverse, interface/ceed-basis.c:1188-1300).  The same steps in the same order, so the tables round
 * as the reference's do. */
static int orc_pseudoinverse(const double *mat, int m, int n, double *pinv) {
  double *a = (double *)malloc(sizeof(double) * (size_t)(m * n)), *tau = (double *)calloc((size_t)m, sizeof(double));
  double *id = (double *)calloc((size_t)(m * m), sizeof(double)), *v = (double *)calloc((size_t)m, sizeof(double));

  if (!a || !tau || !id || !v || n > m) {
    free(a), free(tau), free(id), free(v);
    return 1;
  }
  memcpy(a, mat, sizeof(double) * (size_t)(m * n));
  for (int i = 0; i < n && i < m - 1; i++) {
    double sigma = 0.0;

    v[i] = a[i + n * i];
    for (int j = i + 1; j < m; j++) {
      v[j] = a[i + n * j];
      sigma += v[j] * v[j];
    }
    const double norm = sqrt(v[i] * v[i] + sigma), r_ii = -copysign(norm, v[i]);

    v[i] -= r_ii;
    tau[i] = 2 * v[i] * v[i] / (v[i] * v[i] + sigma);
    for (int j = i + 1; j < m; j++) v[j] /= v[i];
    orc_householder_reflect(&a[i * n + i + 1], &v[i], tau[i], m - i, n - i - 1, n, 1);
    a[i + n * i] = r_ii;
    for (int j = i + 1; j < m; j++) a[i + n * j] = v[j];
  }
  for (int i = 0; i < m; i++) id[i * m + i] = 1.0;
  for (int i = 0; i < n; i++) { /* Q^T id: reflectors in order */
    for (int j = i + 1; j < m; j++) v[j] = a[j * n + i];
    orc_householder_reflect(&id[i * m], &v[i], tau[i], m - i, m, m, 1);
  }
  for (int j = 0; j < m; j++) { /* pinv = R^{-1} Q^T, column by column */
    pinv[j + m * (n - 1)] = id[j + m * (n - 1)] / a[n * n - 1];
    for (int i = n - 2; i >= 0; i--) {
      pinv[j + m * i] = id[j + m * i];
      for (int k = i + 1; k < n; k++) pinv[j + m * i] -= a[k + n * i] * pinv[j + m * k];
      pinv[j + m * i] /= a[i + n * i];
    }
  }
  free(a), free(tau), free(id), free(v);
  return 0;
}

/* Collocated derivative on the quadrature points, G * B^+ (Q x Q), as in interface/ceed-basis.c:750-772: B^+ by the
 * Householder pseudoinverse above, then the product with the sums over k in ascending order
 * (CeedMatrixMatrixMultiply, interface/ceed-basis.c:1163-1174). */
int orc_collocated_grad(int P, int Q, const double *interp_1d, const double *grad_1d, double *collo_grad_1d) {
  double *pinv = (double *)calloc((size_t)(P * Q), sizeof(double)); /* P x Q */

  if (!pinv || Q < P || orc_pseudoinverse(interp_1d, Q, P, pinv)) {
    free(pinv);
    return 1;
  }
  for (int i = 0; i < Q; i++)
    for (int j = 0; j < Q; j++) {
      double s = 0.0;

      for (int k = 0; k < P; k++) s += grad_1d[k + i * P] * pinv[j + k * Q];
      collo_grad_1d[j + i * Q] = s;
    }
  free(pinv);
  return 0;
}

/* ---------------------------------------------------------------------------------------------------------------------
 * Structured box mesh.  Vertex (i,j,k) sits at (i/nx, j/ny, k/nz); vertices interior to the box move by
 * noise*h*U[-1,1) per coordinate (stream `seed`, counter 3*vertex+coordinate), so the box faces stay planar.
 * Coordinates are component-major: coords[c*num_vertices + v] (comp_stride = num_vertices).
 * -------------------------------------------------------------------------------------------------------------------*/
void orc_box_vertices(int nx, int ny, int nz, double noise, uint64_t seed, double *coords) {
  const int64_t nvx = nx + 1, nvy = ny + 1, nvz = nz + 1, nv = nvx * nvy * nvz;
  const int     n[3] = {nx, ny, nz};

  for (int64_t k = 0; k < nvz; k++)
    for (int64_t j = 0; j < nvy; j++)
      for (int64_t i = 0; i < nvx; i++) {
        const int64_t v        = i + nvx * (j + nvy * k);
        const int64_t ijk[3]   = {i, j, k};
        const int     interior = i > 0 && i < nx && j > 0 && j < ny && k > 0 && k < nz;

        for (int c = 0; c < 3; c++) {
          double x = (double)ijk[c] / (double)n[c];

          if (interior) x += noise * (1.0 / (double)n[c]) * orc_uniform(seed, (uint64_t)(3 * v + c), -1.0, 1.0);
          coords[c * nv + v] = x;
        }
      }
}

/* Offsets of a degree-(P-1) H1 field on the box: element e = ex + nx*(ey + ny*ez), local node
 * lx + P*(ly + P*lz), global node gx + ndx*(gy + ndy*gz) with ndx = nx*(P-1)+1.  With ncomp_interlaced > 1 the
 * offsets are scaled by it (interlaced components, comp_stride = 1).  Pattern of examples/ceed/ex1-volume.c
 * BuildCartesianRestriction. */
void orc_box_offsets(int nx, int ny, int nz, int P, int ncomp_interlaced, int32_t *offsets) {
  const int64_t p = P - 1, ndx = nx * p + 1, ndy = ny * p + 1;
  const int     scale = ncomp_interlaced > 1 ? ncomp_interlaced : 1;

  for (int64_t ez = 0; ez < nz; ez++)
    for (int64_t ey = 0; ey < ny; ey++)
      for (int64_t ex = 0; ex < nx; ex++) {
        const int64_t e = ex + nx * (ey + ny * ez);

        for (int64_t lz = 0; lz < P; lz++)
          for (int64_t ly = 0; ly < P; ly++)
            for (int64_t lx = 0; lx < P; lx++) {
              const int64_t g = (ex * p + lx) + ndx * ((ey * p + ly) + ndy * (ez * p + lz));

              offsets[e * P * P * P + lx + P * (ly + P * lz)] = (int32_t)(g * scale);
            }
      }
}

/* ---------------------------------------------------------------------------------------------------------------------
 * Element restriction, offset form.  Gather follows backends/ref/ceed-ref-restriction.c:59-75; the transpose adds in
 * element order as in :220-242.  E-vector layout [elem][comp][node].
 * -------------------------------------------------------------------------------------------------------------------*/
void orc_rstr_gather(int64_t num_elem, int elem_size, int num_comp, int64_t comp_stride, const int32_t *offsets, const double *l_vec,
                     double *e_vec) {
  for (int64_t e = 0; e < num_elem; e++)
    for (int k = 0; k < num_comp; k++)
      for (int i = 0; i < elem_size; i++)
        e_vec[(e * num_comp + k) * elem_size + i] = l_vec[offsets[e * elem_size + i] + k * comp_stride];
}

void orc_rstr_scatter_add(int64_t num_elem, int elem_size, int num_comp, int64_t comp_stride, const int32_t *offsets, const double *e_vec,
                          double *l_vec) {
  for (int64_t e = 0; e < num_elem; e++)
    for (int k = 0; k < num_comp; k++)
      for (int i = 0; i < elem_size; i++)
        l_vec[offsets[e * elem_size + i] + k * comp_stride] += e_vec[(e * num_comp + k) * elem_size + i];
}

/* ---------------------------------------------------------------------------------------------------------------------
 * Tensor contraction v[a][j][c] (+)= sum_b t[j,b] u[a][b][c]; t is J x B (NOTRANSPOSE) or B x J read transposed.
 * Loop order and accumulation order of backends/ref/ceed-ref-tensor.c:16-38.
 * -------------------------------------------------------------------------------------------------------------------*/
static void orc_contract(int A, int B, int C, int J, const double *t, int t_mode, int add, const double *u, double *v) {
  const int s0 = t_mode == ORC_TRANSPOSE ? 1 : B, s1 = t_mode == ORC_TRANSPOSE ? J : 1;

  if (!add)
    for (int q = 0; q < A * J * C; q++) v[q] = 0.0;
  for (int a = 0; a < A; a++)
    for (int b = 0; b < B; b++)
      for (int j = 0; j < J; j++) {
        const double tq = t[j * s0 + b * s1];

        for (int c = 0; c < C; c++) v[(a * J + j) * C + c] += tq * u[(a * B + b) * C + c];
      }
}

static int ipow(int b, int e) {
  int r = 1;

  while (e-- > 0) r *= b;
  return r;
}

/* One element of backends/ref/ceed-ref-basis.c:19-194 (num_elem = 1, the way the ref operator calls it).
 * `colo` is the collocated gradient (Q x Q) when Q >= P and the basis is not collocated, else NULL. */
static void orc_basis_apply_elem(int dim, int P_1d, int Q_1d, int num_comp, const double *interp_1d, const double *grad_1d,
                                 const double *colo, int is_collocated, const double *q_weight_1d, int t_mode, int eval_mode,
                                 const double *u, double *v, double *tmp0, double *tmp1, double *interp_buf) {
  const int add       = t_mode == ORC_TRANSPOSE;
  const int num_qpts  = ipow(Q_1d, dim);
  double   *tmp[2]    = {tmp0, tmp1};

  if (eval_mode == ORC_EVAL_INTERP) {
    if (is_collocated) {
      memcpy(v, u, sizeof(double) * (size_t)(num_comp * num_qpts));
      return;
    }
    int P = P_1d, Q = Q_1d;

    if (t_mode == ORC_TRANSPOSE) {
      P = Q_1d;
      Q = P_1d;
    }
    int pre = num_comp * ipow(P, dim - 1), post = 1;

    for (int d = 0; d < dim; d++) {
      orc_contract(pre, P, post, Q, interp_1d, t_mode, add && (d == dim - 1), d == 0 ? u : tmp[d % 2], d == dim - 1 ? v : tmp[(d + 1) % 2]);
      pre /= P;
      post *= Q;
    }
  } else if (eval_mode == ORC_EVAL_GRAD) {
    int P = P_1d, Q = Q_1d;

    if (t_mode == ORC_TRANSPOSE) {
      P = Q_1d;
      Q = Q_1d;
    }
    int pre = num_comp * ipow(P, dim - 1), post = 1;

    if (colo) {
      for (int d = 0; d < dim; d++) {
        orc_contract(pre, P, post, Q, t_mode == ORC_NOTRANSPOSE ? interp_1d : colo, t_mode, (t_mode == ORC_TRANSPOSE) && (d > 0),
                     t_mode == ORC_NOTRANSPOSE ? (d == 0 ? u : tmp[d % 2]) : &u[d * num_qpts * num_comp],
                     t_mode == ORC_NOTRANSPOSE ? (d == dim - 1 ? interp_buf : tmp[(d + 1) % 2]) : interp_buf);
        pre /= P;
        post *= Q;
      }
      P = Q_1d;
      Q = Q_1d;
      if (t_mode == ORC_TRANSPOSE) {
        P = Q_1d;
        Q = P_1d;
      }
      pre  = num_comp * ipow(P, dim - 1);
      post = 1;
      for (int d = 0; d < dim; d++) {
        orc_contract(pre, P, post, Q, t_mode == ORC_NOTRANSPOSE ? colo : interp_1d, t_mode, (t_mode == ORC_TRANSPOSE && (d == dim - 1)),
                     t_mode == ORC_NOTRANSPOSE ? interp_buf : (d == 0 ? interp_buf : tmp[d % 2]),
                     t_mode == ORC_NOTRANSPOSE ? &v[d * num_qpts * num_comp] : (d == dim - 1 ? v : tmp[(d + 1) % 2]));
        pre /= P;
        post *= Q;
      }
    } else if (is_collocated) {
      for (int d = 0; d < dim; d++) {
        orc_contract(pre, P, post, Q, grad_1d, t_mode, add && (d > 0), t_mode == ORC_NOTRANSPOSE ? u : &u[d * num_comp * num_qpts],
                     t_mode == ORC_TRANSPOSE ? v : &v[d * num_comp * num_qpts]);
        pre /= P;
        post *= Q;
      }
    } else {
      if (t_mode == ORC_TRANSPOSE) {
        P = Q_1d;
        Q = P_1d;
      }
      for (int p = 0; p < dim; p++) {
        pre  = num_comp * ipow(P, dim - 1);
        post = 1;
        for (int d = 0; d < dim; d++) {
          orc_contract(pre, P, post, Q, (p == d) ? grad_1d : interp_1d, t_mode, add && (d == dim - 1),
                       d == 0 ? (t_mode == ORC_NOTRANSPOSE ? u : &u[p * num_comp * num_qpts]) : tmp[d % 2],
                       d == dim - 1 ? (t_mode == ORC_TRANSPOSE ? v : &v[p * num_comp * num_qpts]) : tmp[(d + 1) % 2]);
          pre /= P;
          post *= Q;
        }
      }
    }
  } else if (eval_mode == ORC_EVAL_WEIGHT) {
    const int Q = Q_1d;

    for (int d = 0; d < dim; d++) {
      const int pre = ipow(Q, dim - d - 1), post = ipow(Q, d);

      for (int i = 0; i < pre; i++)
        for (int j = 0; j < Q; j++)
          for (int k = 0; k < post; k++) {
            const int idx = (i * Q + j) * post + k;

            v[idx] = q_weight_1d[j] * (d == 0 ? 1 : v[idx]);
          }
    }
  }
}

static int orc_is_collocated(int P, int Q, const double *interp_1d) {
  if (P != Q) return 0;
  for (int i = 0; i < Q; i++)
    for (int j = 0; j < P; j++)
      if (fabs(interp_1d[i * P + j] - (i == j ? 1.0 : 0.0)) > 1e-14) return 0;
  return 1;
}

/* Basis workspace: collocated gradient and scratch buffers, built once per basis. */
typedef struct {
  int     dim, P, Q, num_comp, is_colloc;
  double *colo, *t0, *t1, *ib;
} orc_basis_ws;

static int orc_basis_ws_init(orc_basis_ws *ws, int dim, int P, int Q, int num_comp, const double *interp_1d, const double *grad_1d) {
  const int    mx   = P > Q ? P : Q;
  const size_t work = (size_t)num_comp * (size_t)ipow(mx, dim);

  ws->dim = dim, ws->P = P, ws->Q = Q, ws->num_comp = num_comp;
  ws->is_colloc = orc_is_collocated(P, Q, interp_1d);
  ws->colo      = NULL;
  ws->t0        = (double *)calloc(work, sizeof(double));
  ws->t1        = (double *)calloc(work, sizeof(double));
  ws->ib        = (double *)calloc(work, sizeof(double));
  if (!ws->t0 || !ws->t1 || !ws->ib) return 1;
  if (Q >= P && !ws->is_colloc) {
    ws->colo = (double *)calloc((size_t)(Q * Q), sizeof(double));
    if (!ws->colo) return 1;
    orc_collocated_grad(P, Q, interp_1d, grad_1d, ws->colo);
  }
  return 0;
}

static void orc_basis_ws_free(orc_basis_ws *ws) {
  free(ws->colo);
  free(ws->t0);
  free(ws->t1);
  free(ws->ib);
}

static void orc_basis_ws_apply(const orc_basis_ws *ws, const double *interp_1d, const double *grad_1d, const double *q_weight_1d, int64_t num_elem,
                               int t_mode, int eval_mode, const double *u, double *v) {
  const int num_nodes = ipow(ws->P, ws->dim), num_qpts = ipow(ws->Q, ws->dim);
  const int qcomp = eval_mode == ORC_EVAL_GRAD ? ws->dim : 1;
  const int n_in  = eval_mode == ORC_EVAL_WEIGHT ? 0 : (t_mode == ORC_NOTRANSPOSE ? num_nodes * ws->num_comp : num_qpts * ws->num_comp * qcomp);
  const int n_out = eval_mode == ORC_EVAL_WEIGHT ? num_qpts : (t_mode == ORC_NOTRANSPOSE ? num_qpts * ws->num_comp * qcomp : num_nodes * ws->num_comp);

  for (int64_t e = 0; e < num_elem; e++) {
    double *ve = v + e * n_out;

    if (t_mode == ORC_TRANSPOSE)
      for (int i = 0; i < n_out; i++) ve[i] = 0.0;
    orc_basis_apply_elem(ws->dim, ws->P, ws->Q, ws->num_comp, interp_1d, grad_1d, ws->colo, ws->is_colloc, q_weight_1d, t_mode, eval_mode,
                         u ? u + e * n_in : NULL, ve, ws->t0, ws->t1, ws->ib);
  }
}

int orc_basis_apply(int dim, int P, int Q, int num_comp, const double *interp_1d, const double *grad_1d, const double *q_weight_1d,
                    int64_t num_elem, int t_mode, int eval_mode, const double *u, double *v) {
  orc_basis_ws ws;

  if (orc_basis_ws_init(&ws, dim, P, Q, num_comp, interp_1d, grad_1d)) {
    orc_basis_ws_free(&ws);
    return 1;
  }
  orc_basis_ws_apply(&ws, interp_1d, grad_1d, q_weight_1d, num_elem, t_mode, eval_mode, u, v);
  orc_basis_ws_free(&ws);
  return 0;
}

/* ---------------------------------------------------------------------------------------------------------------------
 * Gallery QFunctions, restated per point with the reference's evaluation order.
 * -------------------------------------------------------------------------------------------------------------------*/
/* include/ceed/jit-source/gallery/ceed-mass3dbuild.h */
static double orc_qf_mass3d_build(const double J[3][3], double w) {
  return (J[0][0] * (J[1][1] * J[2][2] - J[1][2] * J[2][1]) - J[0][1] * (J[1][0] * J[2][2] - J[1][2] * J[2][0]) +
          J[0][2] * (J[1][0] * J[2][1] - J[1][1] * J[2][0])) *
         w;
}

/* include/ceed/jit-source/gallery/ceed-poisson3dbuild.h */
static void orc_qf_poisson3d_build(const double J[3][3], double w, double qd[6]) {
  double A[3][3];

  for (int j = 0; j < 3; j++)
    for (int k = 0; k < 3; k++)
      A[k][j] = J[(k + 1) % 3][(j + 1) % 3] * J[(k + 2) % 3][(j + 2) % 3] - J[(k + 2) % 3][(j + 1) % 3] * J[(k + 1) % 3][(j + 2) % 3];
  const double qw = w / (J[0][0] * A[0][0] + J[0][1] * A[0][1] + J[0][2] * A[0][2]);

  qd[0] = qw * (A[0][0] * A[0][0] + A[0][1] * A[0][1] + A[0][2] * A[0][2]);
  qd[1] = qw * (A[1][0] * A[1][0] + A[1][1] * A[1][1] + A[1][2] * A[1][2]);
  qd[2] = qw * (A[2][0] * A[2][0] + A[2][1] * A[2][1] + A[2][2] * A[2][2]);
  qd[3] = qw * (A[1][0] * A[2][0] + A[1][1] * A[2][1] + A[1][2] * A[2][2]);
  qd[4] = qw * (A[0][0] * A[2][0] + A[0][1] * A[2][1] + A[0][2] * A[2][2]);
  qd[5] = qw * (A[0][0] * A[1][0] + A[0][1] * A[1][1] + A[0][2] * A[1][2]);
}

/* include/ceed/jit-source/gallery/ceed-poisson3dapply.h (one component; Voigt order 0 5 4 / 5 1 3 / 4 3 2) */
static void orc_qf_poisson3d_apply(const double ug[3], const double qd[6], double vg[3]) {
  const double D[3][3] = {
      {qd[0], qd[5], qd[4]},
      {qd[5], qd[1], qd[3]},
      {qd[4], qd[3], qd[2]}
  };

  for (int j = 0; j < 3; j++) vg[j] = (ug[0] * D[0][j] + ug[1] * D[1][j] + ug[2] * D[2][j]);
}

/* Setup operator of the geometric factors: coordinates (3 components, comp_stride = num_vertices) through the
 * trilinear basis, GRAD at Q^3 Gauss points, WEIGHT, then Mass3DBuild or Poisson3DBuild per point.  This is what
 * CeedOperatorApply does for the gallery build QFunctions on the ref backend (backends/ref/ceed-ref-operator.c:381-476). */
int orc_qdata_build(int nx, int ny, int nz, int Q, int quad_mode, int kind_poisson, const double *coords, double *qdata) {
  const int64_t num_elem = (int64_t)nx * ny * nz, nv = (int64_t)(nx + 1) * (ny + 1) * (nz + 1);
  const int     Q3 = Q * Q * Q;
  double        interp[2 * 16], grad[2 * 16], qref[16], qw[16];
  int32_t      *off = (int32_t *)malloc(sizeof(int32_t) * (size_t)(num_elem * 8));
  double       *xe = (double *)malloc(sizeof(double) * 24), *dx = (double *)malloc(sizeof(double) * (size_t)(9 * Q3));
  double       *w = (double *)malloc(sizeof(double) * (size_t)Q3);

  if (Q > 16 || !off || !xe || !dx || !w) return 1;
  orc_h1_lagrange_1d(2, Q, quad_mode, interp, grad, qref, qw);
  orc_box_offsets(nx, ny, nz, 2, 1, off);
  orc_basis_apply(3, 2, Q, 1, interp, grad, qw, 1, ORC_NOTRANSPOSE, ORC_EVAL_WEIGHT, NULL, w);
  for (int64_t e = 0; e < num_elem; e++) {
    orc_rstr_gather(1, 8, 3, nv, off + e * 8, coords, xe);
    orc_basis_apply(3, 2, Q, 3, interp, grad, qw, 1, ORC_NOTRANSPOSE, ORC_EVAL_GRAD, xe, dx);
    for (int q = 0; q < Q3; q++) {
      double J[3][3];

      for (int d = 0; d < 3; d++)
        for (int c = 0; c < 3; c++) J[d][c] = dx[(d * 3 + c) * Q3 + q];
      if (kind_poisson) {
        double qd[6];

        orc_qf_poisson3d_build(J, w[q], qd);
        for (int k = 0; k < 6; k++) qdata[(e * 6 + k) * Q3 + q] = qd[k];
      } else {
        qdata[e * Q3 + q] = orc_qf_mass3d_build(J, w[q]);
      }
    }
  }
  free(off);
  free(xe);
  free(dx);
  free(w);
  return 0;
}

/* ---------------------------------------------------------------------------------------------------------------------
 * Operator apply, following CeedOperatorApplyAdd_Ref (backends/ref/ceed-ref-operator.c:381-476): gather the whole
 * mesh, then per element basis -> QFunction -> basis^T into the output E-vector, then one scatter-add in element order.
 * CeedOperatorApply zeroes the output first (interface/ceed-operator.c:2283-2290).
 * -------------------------------------------------------------------------------------------------------------------*/
static void orc_qf_apply_elem(const orc_operator *op, int64_t e, const double *uq, double *vq) {
  const int     Q3 = op->Q * op->Q * op->Q, nc = op->num_comp;
  const double *qd = op->qdata;

  switch (op->qf) {
    case ORC_QF_MASS_APPLY: /* ceed-massapply.h */
      for (int q = 0; q < Q3; q++) vq[q] = uq[q] * qd[e * Q3 + q];
      break;
    case ORC_QF_VECMASS_APPLY: /* ceed-vectormassapply.h */
      for (int q = 0; q < Q3; q++)
        for (int c = 0; c < 3; c++) vq[c * Q3 + q] = uq[c * Q3 + q] * qd[e * Q3 + q];
      break;
    case ORC_QF_POISSON3D_APPLY:
    case ORC_QF_POISSON3D_KAPPA:
    case ORC_QF_VECPOISSON3D_APPLY: /* ceed-poisson3dapply.h, ceed-vectorpoisson3dapply.h */
      for (int q = 0; q < Q3; q++) {
        double d6[6];

        for (int k = 0; k < 6; k++) d6[k] = qd[(e * 6 + k) * Q3 + q];
        if (op->qf == ORC_QF_POISSON3D_KAPPA) {
          const double kap = op->kappa[e * Q3 + q];

          for (int k = 0; k < 6; k++) d6[k] *= kap;
        }
        for (int c = 0; c < nc; c++) {
          double ug[3], vg[3];

          for (int d = 0; d < 3; d++) ug[d] = uq[(d * nc + c) * Q3 + q];
          orc_qf_poisson3d_apply(ug, d6, vg);
          for (int d = 0; d < 3; d++) vq[(d * nc + c) * Q3 + q] = vg[d];
        }
      }
      break;
  }
}

static int orc_is_grad_qf(int qf) { return qf == ORC_QF_POISSON3D_APPLY || qf == ORC_QF_VECPOISSON3D_APPLY || qf == ORC_QF_POISSON3D_KAPPA; }

int orc_operator_apply(const orc_operator *op, const double *u, double *v, int add) {
  const int     P = op->P, Q = op->Q, P3 = P * P * P, Q3 = Q * Q * Q, nc = op->num_comp;
  const int     emode = orc_is_grad_qf(op->qf) ? ORC_EVAL_GRAD : ORC_EVAL_INTERP, qc = emode == ORC_EVAL_GRAD ? 3 : 1;
  const int64_t ne = op->num_elem;
  double       *e_in = (double *)malloc(sizeof(double) * (size_t)(ne * nc * P3));
  double       *e_out = (double *)malloc(sizeof(double) * (size_t)(ne * nc * P3));
  double       *uq = (double *)malloc(sizeof(double) * (size_t)(qc * nc * Q3));
  double       *vq = (double *)malloc(sizeof(double) * (size_t)(qc * nc * Q3));

  orc_basis_ws   ws;

  if (!e_in || !e_out || !uq || !vq || orc_basis_ws_init(&ws, 3, P, Q, nc, op->interp_1d, op->grad_1d)) return 1;
  if (!add)
    for (int64_t i = 0; i < op->l_size; i++) v[i] = 0.0;
  orc_rstr_gather(ne, P3, nc, op->comp_stride, op->offsets, u, e_in);
  for (int64_t e = 0; e < ne; e++) {
    orc_basis_ws_apply(&ws, op->interp_1d, op->grad_1d, NULL, 1, ORC_NOTRANSPOSE, emode, e_in + e * nc * P3, uq);
    orc_qf_apply_elem(op, e, uq, vq);
    orc_basis_ws_apply(&ws, op->interp_1d, op->grad_1d, NULL, 1, ORC_TRANSPOSE, emode, vq, e_out + e * nc * P3);
  }
  orc_rstr_scatter_add(ne, P3, nc, op->comp_stride, op->offsets, e_out, v);
  orc_basis_ws_free(&ws);
  free(e_in);
  free(e_out);
  free(uq);
  free(vq);
  return 0;
}

/* dL/dkappa for y = A(kappa) u with cotangent w = dL/dy: y = sum_e E^T G^T (kappa D) G E u, so
 * dL/dkappa[e][q] = (G E w)_q . D_q (G E u)_q.  Restated with the same basis and QFunction pieces as above. */
int orc_kappa_grad(const orc_operator *op, const double *u, const double *w, double *g) {
  const int     P = op->P, Q = op->Q, P3 = P * P * P, Q3 = Q * Q * Q;
  const int64_t ne = op->num_elem;
  double       *ue = (double *)malloc(sizeof(double) * (size_t)P3), *we = (double *)malloc(sizeof(double) * (size_t)P3);
  double       *gu = (double *)malloc(sizeof(double) * (size_t)(3 * Q3)), *gw = (double *)malloc(sizeof(double) * (size_t)(3 * Q3));

  orc_basis_ws   ws;

  if (!ue || !we || !gu || !gw || op->num_comp != 1 || orc_basis_ws_init(&ws, 3, P, Q, 1, op->interp_1d, op->grad_1d)) return 1;
  for (int64_t e = 0; e < ne; e++) {
    orc_rstr_gather(1, P3, 1, op->comp_stride, op->offsets + e * P3, u, ue);
    orc_rstr_gather(1, P3, 1, op->comp_stride, op->offsets + e * P3, w, we);
    orc_basis_ws_apply(&ws, op->interp_1d, op->grad_1d, NULL, 1, ORC_NOTRANSPOSE, ORC_EVAL_GRAD, ue, gu);
    orc_basis_ws_apply(&ws, op->interp_1d, op->grad_1d, NULL, 1, ORC_NOTRANSPOSE, ORC_EVAL_GRAD, we, gw);
    for (int q = 0; q < Q3; q++) {
      double d6[6], ug[3], vg[3];

      for (int k = 0; k < 6; k++) d6[k] = op->qdata[(e * 6 + k) * Q3 + q];
      for (int d = 0; d < 3; d++) ug[d] = gu[d * Q3 + q];
      orc_qf_poisson3d_apply(ug, d6, vg);
      g[e * Q3 + q] = gw[0 * Q3 + q] * vg[0] + gw[1 * Q3 + q] * vg[1] + gw[2 * Q3 + q] * vg[2];
    }
  }
  orc_basis_ws_free(&ws);
  free(ue);
  free(we);
  free(gu);
  free(gw);
  return 0;
}
