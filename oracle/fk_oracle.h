/* CPU oracle for the Feynman-Kac hot path of SpAc -- TEST INFRASTRUCTURE.
 *
 * A scalar FP64 restatement of the reference's path stepping, exit rule,
 * per-node reductions and stencils.  Only tests/, __graft_entry__.smoke() and
 * bench.py's CPU-baseline leg may load it, and only as the checker or the
 * timed CPU baseline; the product library never links or calls it.
 *
 * Parity pinning: with rng_mode = ORC_RNG_SEQUENTIAL the oracle consumes the
 * same random numbers, in the same order, as the reference compiled from its
 * own sources against oracle/shim (one OpenMP thread), and reproduces its
 * outputs bit for bit (tests/test_oracle_pin.py, tests/golden/).  With
 * rng_mode = ORC_RNG_PHILOX it draws the counter-based Philox4x32-10 stream
 * that the GPU kernels draw, so GPU and oracle follow the same paths.
 */
#ifndef SPAC_FK_ORACLE_H
#define SPAC_FK_ORACLE_H
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

enum { ORC_RNG_PHILOX = 0, ORC_RNG_SEQUENTIAL = 1 };
enum { ORC_SHAPE_RECT = 0, ORC_SHAPE_CIRCLE = 1 };
/* ORC_PROBLEM_ROBIN: ANISO with reflecting rectangle sides, prob = (side
 * mask 1: x = x0, 2: y = y0, 4: x = x1, 8: y = y1; varphi; rho; -).
 * ORC_PROBLEM_MONEGROS: BVPs/Monegros_Revamped.hpp (c = -1);
 * ORC_PROBLEM_MONEGROS_POISSON: BVPs/Monegros_Poisson.hpp (c = 0). */
enum { ORC_PROBLEM_FRANKE = 0, ORC_PROBLEM_MONEGROS = 1, ORC_PROBLEM_ANISO = 2, ORC_PROBLEM_DISK = 3,
       ORC_PROBLEM_ROBIN = 4, ORC_PROBLEM_MONEGROS_POISSON = 5 };
enum { ORC_OUT_INSIDE = 0, ORC_OUT_DOMAIN = 1, ORC_OUT_SUBDOMAIN = 2 };

typedef struct {
  int problem;      /* ORC_PROBLEM_* */
  int cv;           /* 0: F = 0; 1: exact-gradient control variate F = -sigma^T grad u; 2: MLP;
                       3: tabulated grad u_hat (orc_cv_table) */
  int dom_shape;    /* ORC_SHAPE_* */
  double dom[4];    /* rect: x0,y0,x1,y1; circle: r,cx,cy */
  double prob[4];   /* disk problem: cx, cy, R */
  const void* mlp;  /* cv == 2: orc_mlp*; cv == 3: orc_cv_table* */
} orc_bvp;

/* cv == 3: F = -sigma^T grad u_hat with grad u_hat interpolated bilinearly in
 * FP64 from FP32 values on a grid x grid lattice of rect (x0, y0, x1, y1):
 * the pair (d/dx, d/dy) of lattice point (i, j), at x0 + (x1 - x0) i /
 * (grid - 1), y0 + (y1 - y0) j / (grid - 1), at tab[2 (j grid + i)] (the
 * layout of fk_mlp_get_table, one region); the point is clamped into the
 * rectangle, as the GPU's FK_CV_MLP step does. */
typedef struct {
  int grid;
  double rect[4];
  const float* tab;
} orc_cv_table;

typedef struct {
  int shape;        /* ORC_SHAPE_* */
  double p[4];
} orc_shape;

/* reference arc stencil (Interfaz): nodes on a circle arc, theta-IMQ RBF */
typedef struct {
  double cx, cy, radius, c2;
  int interior;       /* arc code of Interfaz::Inicia_Cuadrado (-11,-22,-33,-44,-1,-2,-3,-4) */
  int n;
  const double* theta;  /* n node angles */
  const double* iPsi;   /* n x n column-major inverse of Psi */
} orc_arc;

/* Gaussian k-nearest-node stencil on a patch-boundary node set */
typedef struct {
  int m;              /* patch-boundary nodes */
  const double* xy;   /* 2*m coordinates */
  int k;              /* stencil size (20) */
  double eps;         /* Gaussian shape: phi(r) = exp(-(eps r)^2) */
} orc_knn;

/* per-path exit record */
typedef struct {
  double x, y, Y, Z, xi, t;
  int outcome, steps;
} orc_exit;

/* Philox4x32-10 block: out = Philox(ctr, key) */
void orc_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);

void* orc_session_new(int rng_mode, uint64_t seed);
void orc_session_free(void* s);
/* stream id folded into every Philox counter of the following calls */
void orc_session_set_stream(void* s, uint32_t stream);

int orc_circulo(const double p[3], double x, double y, double out[5]);
int orc_rectangulo(const double p[4], double x, double y, double out[5]);
/* u, g, c, f, b0, b1, s00, s01, s10, s11, F0, F1 */
int orc_coefficients(const orc_bvp* b, double x, double y, double out[12]);

/* One path (Simulacion_OMP loop body).  item/path select the Philox counter. */
int orc_path(void* s, const orc_bvp* b, const orc_shape* sub, double x0, double y0, double h,
             uint32_t item, uint32_t path, int max_steps, orc_exit* out);

/* Solve_OMP_Analytic(X0, N, h, rho, bvp): out = phi, phiphi, phi_VR, phiphi_VR,
 * xi, xixi, xiphi, APL, RNGC.  sub == NULL: subdomain = domain. */
int orc_point_solve(void* s, const orc_bvp* b, const orc_shape* sub, double x, double y,
                    unsigned N, double h, uint32_t item, double out[9]);

/* Solve_OMP_Analytic(nudo, N, h, rho, bvp, interfaz) with the arc stencil:
 * G[n] (averaged), B, stats[9].  frontera != 0: B = g(x), G untouched. */
int orc_node_solve_arc(void* s, const orc_bvp* b, double x, double y, int frontera,
                       const orc_arc* arc, unsigned N, double h, uint32_t item,
                       double* G, double* B, double stats[9]);

/* Same with a rectangular patch and the Gaussian k-nearest stencil.  G has m
 * entries.  extra[0..3]: sum of (Z + Y*u(X_tau) + xi) and its square, the
 * count of domain exits, the sum of steps. */
int orc_node_solve_knn(void* s, const orc_bvp* b, double x, double y, const orc_shape* patch,
                       const orc_knn* st, unsigned N, double h, uint32_t item, double* G,
                       double* B, double stats[9], double extra[4]);

/* Gauss-Jordan inverse with full pivoting, FP64 (Eigen FullPivLU::inverse
 * stand-in used by Interfaz::Calcula_Psi).  a: n x n column-major. */
int orc_full_pivot_inverse(int n, const double* a, double* inv);

/* Interfaz::Calcula_Psi: Psi_ij = 1/sqrt((t_i-t_j)^2 + c2), returns ||iPsi||_F ||Psi||_F */
double orc_calcula_psi(int n, const double* theta, double c2, double* iPsi);

/* Gaussian k-nearest stencil weights at a point: writes the window (k local
 * indices, ascending) and the weights w = A_W^{-1} phi_W(x). */
int orc_knn_weights(const orc_knn* st, double x, double y, int* idx, double* w);

/* SistemaLineal::Actualiza_GB(nudo) on CSR arrays: B[row] += b; G added to
 * consecutive entries starting at the column cols[0]. */
int orc_actualiza_gb(int row, int nG, const int* cols, const double* G, double b, const int* rowptr,
                     const int* colidx, double* val, double* B);

/* PseudoespectralCirculoSolver::Inicializa(centro, radio, n_circle, n_radial,
 * theta0, bvp) + Resuelve(bvp, nudos_interior, nudos_periferia): n_periph
 * periphery nodes at angles periph_theta, n_inner interior nodes at inner_xy.
 * G (n_inner x n_periph, row-major) = nudos_interior[p].G[periphery i],
 * B[p] = nudos_interior[p].B.  n_circle even, n_radial odd. */
int orc_ps_disk(const orc_bvp* b, double cx, double cy, double radius, int n_circle, int n_radial, double theta0,
                int n_periph, const double* periph_theta, int n_inner, const double* inner_xy, double* G,
                double* B);

/* --- learned control variate: MLP 2 -> W -> W -> W -> 1 with SiLU ---------- */
typedef struct {
  int width;
  double in_lo[2], in_scale[2];   /* input normalisation: z = (x - lo) * scale */
  const double* W1; const double* b1;   /* W x 2, W */
  const double* W2; const double* b2;   /* W x W, W */
  const double* W3; const double* b3;   /* W x W, W */
  const double* W4; const double* b4;   /* 1 x W, 1 */
} orc_mlp;
/* value and gradient w.r.t. (x, y) */
int orc_mlp_eval(const orc_mlp* m, double x, double y, double out[3]);
/* mean squared error loss over a batch and its gradient w.r.t. all parameters
 * (same packing as the weights: W1,b1,W2,b2,W3,b3,W4,b4) */
double orc_mlp_loss_grad(const orc_mlp* m, int n, const double* xy, const double* target, double* grad);

#ifdef __cplusplus
}
#endif
#endif
