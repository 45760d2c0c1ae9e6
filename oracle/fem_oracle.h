/*
 * fem_oracle.h -- TEST INFRASTRUCTURE ONLY.
 *
 * CPU restatement of the reference's element-by-element (EbE) linear
 * elasticity path (moarseniy/CudaFEMproject), used by tests/ as the parity reference,
 * by __graft_entry__.smoke() and by bench.py's cpu_baseline leg. The product
 * (cudafemproject_gb300) never links, loads or calls this code.
 *
 * Parity is pinned: the FP32 element-local port (orc_ebe_*_f32) is checked
 * against the reference's own CPU build (oracle/ref.mk + oracle/ref_driver.cpp)
 * and against the reference's golden fixtures testing/{test_rect_pcg,9task_3}_test/results.vtk.
 *
 * Two families live here:
 *   orc_ebe_*   a step-by-step restatement of the reference algorithm with
 *               element-local vectors and sort-based assembly, templated on
 *               float / double (femfunc.cpp:3-381, cpu_fem_utils.cpp:182-750,
 *               cpu_matrix.cpp:74-305, datakeeper.cpp:96-213, fem_utils.cpp:53-82);
 *   orc_*       an FP64 global-vector form of the same mathematics (stored
 *               element matrices, CSR gather assembly, OpenMP), fast enough for
 *               the ~1e5-element parity cases. Its "compat" mode reproduces the
 *               reference's numerical quirks, "consistent" mode is textbook.
 */
#ifndef FEM_ORACLE_H
#define FEM_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_problem {
  int32_t dim;                 /* 2 (CST, plane stress) or 3 (linear tetrahedra) */
  int64_t n_nodes, n_elems;
  const double *nodes;         /* [n_nodes][dim] */
  const int32_t *elems;        /* [n_elems][dim+1], 0-based node ids */
  int64_t n_constraints;
  const int32_t *cons;         /* [n_constraints][2]: node, Constraint::Type code */
  int64_t n_loads;
  const int32_t *load_node;    /* [n_loads] */
  const double *load_vec;      /* [n_loads][dim] */
  int64_t n_faces;
  const int32_t *face_nodes;   /* [n_faces][dim+1]: dim face nodes, then the opposite node */
  const int32_t *face_elem;    /* [n_faces] adjacent element */
  const double *face_normal;   /* [n_faces][dim] as written in stress.txt (normalised on use) */
  const double *face_pressure; /* [n_faces] */
  const double *elem_E;        /* [n_elems] per-element Young's modulus, or NULL */
  double E, nu, rho;
  int32_t consistent;          /* 0: reproduce the reference (compat), 1: textbook */
} orc_problem;

enum { ORC_WAVELET_NONE = 0, ORC_WAVELET_RICKER = 1, ORC_WAVELET_BERLAGE = 2 };

typedef struct orc_wavelet {
  int32_t type;
  double freq, timeshift, ampl;
} orc_wavelet;

typedef struct orc_dyn {
  double beta1, beta2, dt, endtime;
} orc_dyn;

/* ---- wavelets, in the reference's float arithmetic (fem_utils.cpp:53-82) ---- */
float orc_wavelet_value_f32(const orc_wavelet *w, float t);

/* ---- element-local port (float / double) -------------------------------- */
/* Static solve (gpuCalculateFEM_EbE_vec, femfunc.cpp:3-23). u_out: [n_nodes][dim]. */
int orc_ebe_static_f32(const orc_problem *p, const orc_wavelet *w, double eps, float *u_out, int32_t *iters);
int orc_ebe_static_f64(const orc_problem *p, const orc_wavelet *w, double eps, double *u_out, int32_t *iters);
/* Dynamics (gpuCalculateFEM_DYN, femfunc.cpp:130-381). */
int orc_ebe_dyn_f32(const orc_problem *p, const orc_wavelet *w, const orc_dyn *d, float *u_out,
                    int32_t *steps, int64_t *pcg_iters);
int orc_ebe_dyn_f64(const orc_problem *p, const orc_wavelet *w, const orc_dyn *d, double *u_out,
                    int32_t *steps, int64_t *pcg_iters);
/* Setup arrays as the reference builds them (genMask, calculateKlocals, getDiagonal, initFlocals).
 * Any output pointer may be NULL. Klocals keep the reference's column-major 12x12 / 6x6 layout. */
int orc_ebe_setup_f32(const orc_problem *p, const orc_wavelet *w, float *mask, float *adj,
                      float *klocals, float *diagk, float *flocals, float *areas);
/* Wall-clock of setup and of k PCG iterations (FP32, single thread): the CPU baseline leg. */
int orc_ebe_time_f32(const orc_problem *p, int32_t k, double *setup_s, double *iter_s);

/* The same port set up once, then timed in samples of k PCG iterations. */
typedef struct orc_ebe_timer orc_ebe_timer;
int orc_ebe_timer_create(const orc_problem *p, orc_ebe_timer **out);
double orc_ebe_timer_iters(orc_ebe_timer *t, int32_t k);
void orc_ebe_timer_info(const orc_ebe_timer *t, double *setup_s, double *init_s);
void orc_ebe_timer_free(orc_ebe_timer *t);
/* OpenMP threads the FP64 form uses (1 without OpenMP). */
int orc_num_threads(void);

/* ---- FP64 global-vector form ------------------------------------------------ */
typedef struct orc_ctx orc_ctx;
int orc_setup(const orc_problem *p, orc_ctx **out);
void orc_free(orc_ctx *c);
int64_t orc_ndof(const orc_ctx *c);
/* DOF map mask[e*w + dim*a + d] = dim*elem[e][a] + d (cpu_fem_utils.cpp:182-213). */
void orc_get_mask(const orc_ctx *c, int32_t *mask);
/* Number of elements touching each DOF (genAdjElements). */
void orc_get_adjacency(const orc_ctx *c, int32_t *adj);
/* Per-DOF constrained flag, decoded exactly as datakeeper.cpp:139-171. */
void orc_get_bc(const orc_ctx *c, uint8_t *constrained);
/* Element stiffness matrices with constraints applied, row-major [e][w][w]. */
void orc_get_element_matrices(const orc_ctx *c, double *ke);
/* Global assembled diagonal of the constrained operator. */
void orc_get_diag(const orc_ctx *c, double *d);
/* Global right-hand side at time t (initFlocals / calcFlocals then assembly). */
void orc_get_rhs(orc_ctx *c, const orc_wavelet *w, double t, double *f);
/* Assembles K' once into dim x dim node blocks (the same element matrices,
 * summed per node pair in element order); orc_matvec then multiplies with the
 * assembled copy, which reads about a quarter of the bytes of the element
 * matrices on tet meshes. Call it before any solve it should speed up. */
int orc_assemble(orc_ctx *c);
/* y = K' x, K' the constrained stiffness. */
void orc_matvec(const orc_ctx *c, const double *x, double *y);
/* Jacobi PCG from x = 0. rule 0: stop when gamma < tol*gamma0 (reference rule,
 * gamma = r.M^-1.r); rule 1: stop when ||r||_2 <= tol*||f||_2 (recursive r). */
int orc_pcg(const orc_ctx *c, const double *f, double *x, double tol, int32_t rule, int32_t maxit,
            int32_t *iters);
/* The same, starting from the x passed in (rule 1 compares ||f - K'x|| with tol*||f||). */
int orc_pcg_warm(const orc_ctx *c, const double *f, double *x, double tol, int32_t rule, int32_t maxit,
                 int32_t *iters);
/* Dynamics (GN22), compat or consistent per the problem flag. pcg_tol/pcg_rule
 * are used by the implicit scheme (compat uses rule 0, tol 1e-4 like the reference). */
int orc_dyn_run(orc_ctx *c, const orc_wavelet *w, const orc_dyn *d, double pcg_tol, int32_t pcg_rule,
                double *u_out, int32_t *steps, int64_t *pcg_iters);
/* Explicit GN22 (beta2 = 0) receiver-misfit loss and its gradient in the
 * per-element Young's moduli by the discrete adjoint (all states stored):
 * L = 1/2 sum_{n=1..N} sum_r |d_n[node_r] - obs[n-1][r]|^2 (obs [N][n_rec][dim]).
 * Consistent semantics only. Returns L; g [n_elems]. */
double orc_dyn_adjoint(orc_ctx *c, const orc_wavelet *w, const orc_dyn *d, int32_t n_rec, const int32_t *rec_nodes,
                       const double *obs, double *g);
/* Per-element strain = B u_e, stress = D strain (D scaled by E_e / E) and
 * von Mises stress (deprecated/femfunc/femfunc.cpp:42-106); outputs
 * [n_elems][3(dim-1)] and [n_elems], any may be NULL. */
void orc_element_stress(const orc_ctx *c, const double *u, double *strain, double *stress, double *mises);
/* Adjoint sensitivity for a solved static state: dL/dE_e = -lambda_e^T (K_e / E_e) u_e. */
void orc_grad_E(const orc_ctx *c, const double *lambda, const double *u, double *g);

#ifdef __cplusplus
}
#endif
#endif
