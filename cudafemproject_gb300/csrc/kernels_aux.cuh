// Setup, conversion, dynamics and reference-compatibility kernels.
#pragma once

#include "kernels.cuh"

namespace cfem {

// ------------------------------------------------------------------ geometry
// Per element: shape gradients from the inverse Jacobian (FP64), volume
// V = |det J| / dim!, scaled gradients G = sqrt(V * s_e) grad N_a (FP64 and
// FP32 copies), the element's diagonal of K_e accumulated into the assembled
// diagonal, lumped and consistent mass terms.
// (reference: genCoordinates, calculateArea, genGradientMatrix(3D),
//  calculateKlocal, getDiagonal, calculateMlocals: cpu_fem_utils.cpp:221-520, 598-734)
struct GeomParams {
  int64_t ne, gstride;
  const double *coords;   // [nn][dim] new node order
  const int32_t *conn;    // [ne][dim+1] new node ids, new element order, original vertex order
  const double *escale;   // [ne] E_e / E or nullptr
  double lam, mu;
  double rho, lump_c, cons_c;  // lumped mass per DOF = lump_c * rho * V ; consistent coeff = cons_c * rho * V
  double *G64; float *G32; double *vol;
  double *diagK;          // node vectors (atomic)
  double *mlump;          // node vectors (atomic) lumped mass
  double *mc64; float *mc32;  // per element consistent-mass coefficient
  double *diag_local;     // [ne][w] element diagonal of K in original element/slot order (or nullptr)
  const int32_t *elem_new2old;
  int *err;
  const double *lam_e, *mu_e;  // per-element material (new order) or nullptr
};

template <int DIM>
__global__ void k_geometry(GeomParams P) {
  constexpr int NV = DIM + 1, VW = DIM == 3 ? 4 : 2, W = 6 * (DIM - 1);
  int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (e >= P.ne) return;
  int v[NV];
  double X[NV][DIM];
#pragma unroll
  for (int a = 0; a < NV; ++a) {
    v[a] = P.conn[e * NV + a];
#pragma unroll
    for (int d = 0; d < DIM; ++d) X[a][d] = P.coords[(int64_t)v[a] * DIM + d];
  }
  double J[DIM][DIM];  // J[d][a-1] = x_a,d - x_0,d
#pragma unroll
  for (int d = 0; d < DIM; ++d)
#pragma unroll
    for (int a = 1; a < NV; ++a) J[d][a - 1] = X[a][d] - X[0][d];
  double det, inv[DIM][DIM];  // inv[a][d] = d xi_a / d x_d
  if (DIM == 3) {
    double c00 = J[1][1] * J[2][2] - J[1][2] * J[2][1];
    double c01 = J[1][2] * J[2][0] - J[1][0] * J[2][2];
    double c02 = J[1][0] * J[2][1] - J[1][1] * J[2][0];
    det = J[0][0] * c00 + J[0][1] * c01 + J[0][2] * c02;
    double id = 1.0 / det;
    inv[0][0] = c00 * id;
    inv[1][0] = c01 * id;
    inv[2][0] = c02 * id;
    inv[0][1] = (J[0][2] * J[2][1] - J[0][1] * J[2][2]) * id;
    inv[1][1] = (J[0][0] * J[2][2] - J[0][2] * J[2][0]) * id;
    inv[2][1] = (J[0][1] * J[2][0] - J[0][0] * J[2][1]) * id;
    inv[0][2] = (J[0][1] * J[1][2] - J[0][2] * J[1][1]) * id;
    inv[1][2] = (J[0][2] * J[1][0] - J[0][0] * J[1][2]) * id;
    inv[2][2] = (J[0][0] * J[1][1] - J[0][1] * J[1][0]) * id;
  } else {
    det = J[0][0] * J[1][1] - J[0][1] * J[1][0];
    double id = 1.0 / det;
    inv[0][0] = J[1][1] * id;
    inv[0][1] = -J[0][1] * id;
    inv[1][0] = -J[1][0] * id;
    inv[1][1] = J[0][0] * id;
  }
  const double V = fabs(det) / (DIM == 3 ? 6.0 : 2.0);
  if (!(V > 0) || !isfinite(V)) {
    atomicOr(P.err, 1);
    return;
  }
  const double s = P.escale ? P.escale[e] : 1.0;
  const double sc = sqrt(V * s);
  double g[NV][DIM];
#pragma unroll
  for (int d = 0; d < DIM; ++d) {
    double s0 = 0;
#pragma unroll
    for (int a = 1; a < NV; ++a) {
      g[a][d] = inv[a - 1][d] * sc;
      s0 += g[a][d];
    }
    g[0][d] = -s0;
  }
#pragma unroll
  for (int a = 1; a < NV; ++a)
#pragma unroll
    for (int d = 0; d < DIM; ++d) {
      P.G64[(size_t)((a - 1) * DIM + d) * P.gstride + e] = g[a][d];
      P.G32[(size_t)((a - 1) * DIM + d) * P.gstride + e] = (float)g[a][d];
    }
  P.vol[e] = V;
  const double mass = P.rho * V;
  if (P.mc64) { P.mc64[e] = P.cons_c * mass; P.mc32[e] = (float)(P.cons_c * mass); }
  const int64_t eo = P.elem_new2old ? P.elem_new2old[e] : e;
#pragma unroll
  for (int a = 0; a < NV; ++a) {
    double sq[DIM], tot = 0;
#pragma unroll
    for (int d = 0; d < DIM; ++d) { sq[d] = g[a][d] * g[a][d]; tot += sq[d]; }
#pragma unroll
    for (int d = 0; d < DIM; ++d) {
      // D = lam 1(x)1 + 2 mu I (Voigt, engineering shear): diag of B^T D B
      const double lam = P.lam_e ? P.lam_e[e] : P.lam, mu = P.mu_e ? P.mu_e[e] : P.mu;
      double kd = (lam + 2 * mu) * sq[d] + mu * (tot - sq[d]);
      atomicAdd(P.diagK + (int64_t)v[a] * VW + d, kd);
      if (P.mlump) atomicAdd(P.mlump + (int64_t)v[a] * VW + d, P.lump_c * mass);
      if (P.diag_local) P.diag_local[eo * W + DIM * a + d] = kd;
    }
  }
}

// ------------------------------------------------------------------ layout conversion
// caller order [nn][dim] (FP64) -> node vectors [nn][VW] (T) in locality order
template <typename T, int DIM>
__global__ void k_to_internal(int64_t nn, const double *src, const int32_t *new2old, T *dst, double scale) {
  constexpr int VW = DIM == 3 ? 4 : 2;
  int64_t n = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (n >= nn) return;
  int64_t o = new2old[n];
  NodeV<T, VW> v;
#pragma unroll
  for (int d = 0; d < VW; ++d) v.v[d] = d < DIM ? (T)(src[o * DIM + d] * scale) : T(0);
  stv<T, VW>(dst, n, v);
}

template <typename T, int DIM>
__global__ void k_to_caller(int64_t nn, const T *src, const int32_t *new2old, double *dst) {
  constexpr int VW = DIM == 3 ? 4 : 2;
  int64_t n = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (n >= nn) return;
  int64_t o = new2old[n];
  NodeV<T, VW> v = ldv<T, VW>(src, n);
#pragma unroll
  for (int d = 0; d < DIM; ++d) dst[o * DIM + d] = (double)v.v[d];
}

// dinv = 1 / diag (0 where diag == 0), in T
template <typename T>
__global__ void k_invert(int64_t n, const double *diag, T *dinv) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  double d = diag[i];
  dinv[i] = d != 0 ? (T)(1.0 / d) : T(0);
}

template <typename TA, typename TB>
__global__ void k_convert(int64_t n, const TA *a, TB *b) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) b[i] = (TB)a[i];
}

// y = a*x + b*y over raw arrays
static __global__ void k_axpby64(int64_t n, double a, const double *x, double b, double *y) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) y[i] = a * x[i] + b * y[i];
}

// Refinement: r64 = f - u64 (u64 = K x64), u64 = 0, r32 = (float) r64, ||r||^2 and ||f||^2.
struct ResParams {
  int64_t nvec;
  const double *f;
  double *u, *r;
  float *r32;
  double *out;       // [2]: ||r||^2, ||f||^2
  double *partials;
  unsigned int *count;
};
static __global__ void __launch_bounds__(kThreads) k_residual(ResParams P) {
  double acc[2] = {0, 0};
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < P.nvec; i += (int64_t)gridDim.x * blockDim.x) {
    double r = P.f[i] - P.u[i];
    P.u[i] = 0;
    P.r[i] = r;
    if (P.r32) P.r32[i] = (float)r;
    acc[0] += r * r;
    acc[1] += P.f[i] * P.f[i];
  }
  if (grid_sum_last<2>(acc, P.partials, P.count)) { P.out[0] = acc[0]; P.out[1] = acc[1]; }
}

// Continued PCG run: z += (gamma / gamma_prev) p_last on the DOF lanes (the
// fourth lane carries M^-1, see k_pcg_init), gamma from the init kernel's
// scalars (nothing to do once they say done).
template <typename T, int DIM>
__global__ void k_fold_direction(int64_t nn, const Scalars *sc, double gamma_prev, const T *p_last, T *z) {
  constexpr int VW = DIM == 3 ? 4 : 2;
  if (sc->done) return;
  const T beta = (T)(sc->gamma / gamma_prev);
  int64_t n = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (n >= nn) return;
  NodeV<T, VW> zv = ldv<T, VW>(z, n);
  const NodeV<T, VW> pv = ldv<T, VW>(p_last, n);
#pragma unroll
  for (int d = 0; d < DIM; ++d) zv.v[d] += beta * pv.v[d];
  stv<T, VW>(z, n, zv);
}

// x64 += (double) x32 on the DOF lanes (vw 4: the fourth lane of x32 carries
// M^-1, see k_pcg_init)
static __global__ void k_accumulate(int64_t n, const float *x32, double *x64, int vw) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n && !(vw == 4 && (i & 3) == 3)) x64[i] += (double)x32[i];
}

// ------------------------------------------------------------------ dynamics (GN22)
// femfunc.cpp:258-310. The predictor d_new = d + dt v + 0.5(1-beta2)dt^2 a is
// fused into the matvec stage (MV_DYN); these kernels finish the step.
template <typename T>
struct DynParams {
  int64_t n_nodes;
  T *v, *a, *y, *rhs;      // rhs: implicit PCG right-hand side (out)
  T *d;                    // current displacement buffer (implicit corrector)
  const T *FA, *FB;        // load parts
  const double *coef;      // [steps+1][2] time factors of FA, FB
  const T *minv;           // explicit: inverse assembled lumped mass
  const T *anew;           // implicit: solved acceleration
  T c_old, c_new, c_d;     // v += c_old a_old + c_new a_new ; d += c_d a_new
  DynState *st;
  const int32_t *recv;     // receiver nodes (new ids) or nullptr
  int n_recv;
  double *trace;           // [steps][n_recv][dim]
  int dim;
  const T *dto;            // explicit, end of step fused: the step's new displacements
  int parity;              // explicit, end of step fused: the step's parity in the graph
};

// explicit: a_new = (F(t) - K d) / M ; v += (1-beta1) dt a_old + beta1 dt a_new.
// END_STEP: the step also ends here (receivers of P.dto recorded by CTA 0, the
// step counter advanced through the parity pair of DynState) instead of in
// k_dyn_end_step.
template <typename T, int DIM, bool END_STEP = false>
__global__ void k_dyn_explicit(DynParams<T> P) {
  constexpr int VW = DIM == 3 ? 4 : 2;
  griddep_wait();               // y (and the new displacements) from the step's matvec
  griddep_launch_dependents();  // (the end-of-step kernel or the next matvec)
  // thread 0 reads the step and its load factors once per CTA (every thread
  // reading the same line would queue at one L2 slice)
  __shared__ T s_coef[2];
  __shared__ int s_step;
  if (threadIdx.x == 0) {
    const int step = END_STEP ? P.st->pstep[P.parity] : P.st->step;
    s_step = step;
    s_coef[0] = (T)P.coef[2 * step];
    s_coef[1] = (T)P.coef[2 * step + 1];
  }
  __syncthreads();
  const T ca = s_coef[0], cb = s_coef[1];
  if (END_STEP && blockIdx.x == 0)
    for (int i = threadIdx.x; i < P.n_recv * P.dim; i += blockDim.x) {
      const int r = i / P.dim, k = i % P.dim;
      P.trace[((int64_t)(s_step - 1) * P.n_recv + r) * P.dim + k] = (double)P.dto[(int64_t)P.recv[r] * VW + k];
    }
  for (int64_t n = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; n < P.n_nodes; n += (int64_t)gridDim.x * blockDim.x) {
    NodeV<T, VW> y = ldv<T, VW>(P.y, n), fa = ldv<T, VW>(P.FA, n), fb = ldv<T, VW>(P.FB, n);
    NodeV<T, VW> mi = ldv<T, VW>(P.minv, n), a = ldv<T, VW>(P.a, n), v = ldv<T, VW>(P.v, n), zero;
#pragma unroll
    for (int d = 0; d < VW; ++d) zero.v[d] = 0;
#pragma unroll
    for (int d = 0; d < DIM; ++d) {
      T an = (ca * fa.v[d] + cb * fb.v[d] - y.v[d]) * mi.v[d];
      v.v[d] += P.c_old * a.v[d] + P.c_new * an;
      a.v[d] = an;
    }
    stv<T, VW>(P.a, n, a);
    stv<T, VW>(P.v, n, v);
    stv<T, VW>(P.y, n, zero);
  }
  if (END_STEP && blockIdx.x == 0 && threadIdx.x == 0) P.st->pstep[P.parity ^ 1] = s_step + 1;
}

// implicit: rhs = F(t) - K d ; y = 0
template <typename T, int DIM>
__global__ void k_dyn_rhs(DynParams<T> P) {
  constexpr int VW = DIM == 3 ? 4 : 2;
  __shared__ T s_coef[2];  // (read once per CTA, see k_dyn_explicit)
  if (threadIdx.x == 0) {
    const int step = P.st->step;
    s_coef[0] = (T)P.coef[2 * step];
    s_coef[1] = (T)P.coef[2 * step + 1];
  }
  __syncthreads();
  const T ca = s_coef[0], cb = s_coef[1];
  for (int64_t n = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; n < P.n_nodes; n += (int64_t)gridDim.x * blockDim.x) {
    NodeV<T, VW> y = ldv<T, VW>(P.y, n), fa = ldv<T, VW>(P.FA, n), fb = ldv<T, VW>(P.FB, n), r, zero;
#pragma unroll
    for (int d = 0; d < VW; ++d) { zero.v[d] = 0; r.v[d] = 0; }
#pragma unroll
    for (int d = 0; d < DIM; ++d) r.v[d] = ca * fa.v[d] + cb * fb.v[d] - y.v[d];
    stv<T, VW>(P.rhs, n, r);
    stv<T, VW>(P.y, n, zero);
  }
}

// implicit corrector: v += c_old a_old + c_new a_new ; d += c_d a_new ; a_old = a_new
template <typename T, int DIM>
__global__ void k_dyn_correct(DynParams<T> P) {
  constexpr int VW = DIM == 3 ? 4 : 2;
  for (int64_t n = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; n < P.n_nodes; n += (int64_t)gridDim.x * blockDim.x) {
    NodeV<T, VW> a = ldv<T, VW>(P.a, n), an = ldv<T, VW>(P.anew, n), v = ldv<T, VW>(P.v, n), d = ldv<T, VW>(P.d, n);
#pragma unroll
    for (int k = 0; k < DIM; ++k) {
      v.v[k] += P.c_old * a.v[k] + P.c_new * an.v[k];
      d.v[k] += P.c_d * an.v[k];
      a.v[k] = an.v[k];
    }
    stv<T, VW>(P.a, n, a);
    stv<T, VW>(P.v, n, v);
    stv<T, VW>(P.d, n, d);
  }
}

// Ends a step: records receiver displacements and advances the step counter.
template <typename T>
__global__ void k_dyn_end_step(DynParams<T> P, const T *d, int VW) {
  griddep_wait();
  griddep_launch_dependents();  // the next step's matvec starts streaming its blocks
  const int step = P.st->step;
  for (int i = threadIdx.x; i < P.n_recv * P.dim; i += blockDim.x) {
    int r = i / P.dim, k = i % P.dim;
    P.trace[((int64_t)(step - 1) * P.n_recv + r) * P.dim + k] = (double)d[(int64_t)P.recv[r] * VW + k];
  }
  __syncthreads();
  if (threadIdx.x == 0) P.st->step = step + 1;
}

static __global__ void k_dyn_advance(DynState *st) {
  if (threadIdx.x == 0 && blockIdx.x == 0) st->step += 1;
}

// ------------------------------------------------------------------ reference re-sorting quirk
// The reference assembles an element-local vector by sorting it by DOF key in
// place (cpu_fem_utils.cpp:437-445): after each assembly the source holds its
// values in key order. For sources that are assembled repeatedly (lumped mass
// in explicit dynamics, preconditioner diagonal in implicit dynamics) the next
// assembly then mixes values of different elements. These kernels reproduce
// it: out[dof] = sum of the DOF's slots in element order, then src = src[perm].
static __global__ void k_assemble_slots(int64_t ndof, int dim, int vw, const int64_t *seg, const int32_t *perm,
                                 const double *src, const int32_t *old2new, double *out_node_vec, int invert,
                                 float *out32) {
  int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (k >= ndof) return;
  double acc = 0;
  for (int64_t j = seg[k]; j < seg[k + 1]; ++j) acc += src[perm[j]];
  int64_t node = k / dim, d = k % dim;
  int64_t idx = (int64_t)old2new[node] * vw + d;
  double v = invert ? (acc != 0 ? 1.0 / acc : 0.0) : acc;
  out_node_vec[idx] = v;
  if (out32) out32[idx] = (float)v;
}

static __global__ void k_permute(int64_t n, const int32_t *perm, const double *src, double *dst) {
  int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (j < n) dst[j] = src[perm[j]];
}

// ------------------------------------------------------------------ element matrices (checks)
// K'_e rebuilt in FP64 from G: K_e = G^T D G, then applyConstraints.
template <int DIM>
__global__ void k_element_matrices(int64_t first, int64_t count, const int32_t *elem_old2new, const double *G64,
                                   int64_t gstride, const int32_t *conn, const uint8_t *bits, double lam, double mu,
                                   double *ke) {
  constexpr int NV = DIM + 1, W = 6 * (DIM - 1);
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= count) return;
  int64_t e = elem_old2new[first + i];
  double g[NV][DIM];
#pragma unroll
  for (int d = 0; d < DIM; ++d) {
    double s0 = 0;
#pragma unroll
    for (int a = 1; a < NV; ++a) {
      g[a][d] = G64[(size_t)((a - 1) * DIM + d) * gstride + e];
      s0 += g[a][d];
    }
    g[0][d] = -s0;
  }
  double *K = ke + i * W * W;
  for (int a = 0; a < NV; ++a)
    for (int b = 0; b < NV; ++b)
      for (int p = 0; p < DIM; ++p)
        for (int q = 0; q < DIM; ++q) {
          // (B^T D B)_{ap,bq} = lam g_ap g_bq + mu (g_a.g_b delta_pq + g_aq g_bp)
          double dot = 0;
          for (int k = 0; k < DIM; ++k) dot += g[a][k] * g[b][k];
          double v = lam * g[a][p] * g[b][q] + mu * ((p == q ? dot : 0.0) + g[a][q] * g[b][p]);
          int r = DIM * a + p, c = DIM * b + q;
          int na = conn[e * NV + a], nb = conn[e * NV + b];
          bool cr = bits[na] >> p & 1u, cc = bits[nb] >> q & 1u;
          if (r != c && (cr || cc)) v = 0;
          K[r * W + c] = v;
        }
}

// dL/dE_e = -(1/E_e) lambda_e^T K'_e u_e (gradient form; constrained slots keep K_e's diagonal)
template <int DIM>
__global__ void k_grad_young(int64_t ne, const double *G64, int64_t gstride, const int32_t *conn, const uint8_t *bits,
                             double lam, double mu, const double *lamv, const double *uv, const double *young,
                             const int32_t *elem_new2old, double *g_out, int accumulate = 0) {
  constexpr int NV = DIM + 1, VW = DIM == 3 ? 4 : 2;
  int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (e >= ne) return;
  double G[DIM * DIM], u[NV][DIM], l[NV][DIM], f[NV][DIM];
  for (int k = 0; k < DIM * DIM; ++k) G[k] = G64[(size_t)k * gstride + e];
  double diag_terms = 0;
  for (int a = 0; a < NV; ++a) {
    int n = conn[e * NV + a];
    unsigned b = bits[n];
    for (int d = 0; d < DIM; ++d) {
      bool c = b >> d & 1u;
      u[a][d] = c ? 0.0 : uv[(int64_t)n * VW + d];
      l[a][d] = c ? 0.0 : lamv[(int64_t)n * VW + d];
    }
  }
  element_force<double, DIM>(u, G, lam, mu, 1.0, 0.0, f);
  double acc = 0;
  for (int a = 0; a < NV; ++a)
    for (int d = 0; d < DIM; ++d) acc += l[a][d] * f[a][d];
  // constrained slots: K_e diagonal term
  double g0[DIM];
  for (int d = 0; d < DIM; ++d) {
    g0[d] = 0;
    for (int a = 1; a < NV; ++a) g0[d] -= G[(a - 1) * DIM + d];
  }
  for (int a = 0; a < NV; ++a) {
    int n = conn[e * NV + a];
    unsigned b = bits[n];
    if (!b) continue;
    double sq[DIM], tot = 0;
    for (int d = 0; d < DIM; ++d) {
      double gd = a == 0 ? g0[d] : G[(a - 1) * DIM + d];
      sq[d] = gd * gd;
      tot += sq[d];
    }
    for (int d = 0; d < DIM; ++d)
      if (b >> d & 1u) {
        double kd = (lam + 2 * mu) * sq[d] + mu * (tot - sq[d]);
        diag_terms += lamv[(int64_t)n * VW + d] * kd * uv[(int64_t)n * VW + d];
      }
  }
  int64_t eo = elem_new2old[e];
  const double v = -(acc + diag_terms) / young[eo];
  g_out[eo] = accumulate ? g_out[eo] + v : v;
}

// ---- explicit GN22 adjoint (reverse of one step; see cfem_dyn_adjoint) ----
// receiver misfit: db[node_r] += d_n[node_r] - obs_n[r]
static __global__ void k_adj_receivers(int n_rec, int dim, int vw, const int32_t *recv, const double *d,
                                       const double *obs_n, double *db) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n_rec * dim) return;
  int r = i / dim, q = i % dim;
  int64_t k = (int64_t)recv[r] * vw + q;
  db[k] += d[k] - obs_n[i];
}

// w = (a_bar + h_new v_bar) / M ; a_bar = h_old v_bar
static __global__ void k_adj_pre(int64_t n, double h_old, double h_new, const double *minv, const double *vb,
                                 double *ab, double *wb) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  double an = ab[i] + h_new * vb[i];
  wb[i] = an * minv[i];
  ab[i] = h_old * vb[i];
}

// d_tot = d_bar - K w ; d_bar = d_tot ; v_bar += dt d_tot ; a_bar += c2 d_tot ; y = 0
static __global__ void k_adj_post(int64_t n, double dt, double c2, double *y, double *db, double *vb, double *ab) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  double t = db[i] - y[i];
  y[i] = 0;
  db[i] = t;
  vb[i] += dt * t;
  ab[i] += c2 * t;
}

// Element strain / stress recovery (deprecated/femfunc/femfunc.cpp:42-106:
// deformation = B u_e, stress = D deformation), Voigt order (xx, yy, xy) in 2D
// and (xx, yy, zz, xy, yz, xz) in 3D with engineering shear strains, plus the
// von Mises stress (plane stress in 2D).
template <int DIM>
__global__ void k_element_stress(int64_t ne, const double *G64, int64_t gstride, const double *vol, const double *escale,
                                 const int32_t *conn, const double *u, double lam, double mu,
                                 const int32_t *elem_new2old, double *strain, double *stress, double *mises) {
  constexpr int NV = DIM + 1, VW = DIM == 3 ? 4 : 2, S = 3 * (DIM - 1);
  int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (e >= ne) return;
  const double s_e = escale ? escale[e] : 1.0;
  const double inv = 1.0 / sqrt(vol[e] * s_e);
  double g[NV][DIM];
  for (int d = 0; d < DIM; ++d) {
    double s0 = 0;
    for (int a = 1; a < NV; ++a) {
      g[a][d] = G64[(size_t)((a - 1) * DIM + d) * gstride + e] * inv;
      s0 += g[a][d];
    }
    g[0][d] = -s0;
  }
  double H[DIM][DIM] = {};
  for (int a = 0; a < NV; ++a) {
    const int64_t n = conn[e * NV + a];
    for (int i = 0; i < DIM; ++i)
      for (int j = 0; j < DIM; ++j) H[i][j] += u[n * VW + i] * g[a][j];
  }
  double eps[S], sig[S];
  const double L = lam * s_e, M = mu * s_e;
  if (DIM == 2) {
    eps[0] = H[0][0]; eps[1] = H[1][1]; eps[2] = H[0][1] + H[1][0];
    const double tr = eps[0] + eps[1];
    sig[0] = L * tr + 2 * M * eps[0]; sig[1] = L * tr + 2 * M * eps[1]; sig[2] = M * eps[2];
  } else {
    eps[0] = H[0][0]; eps[1] = H[1][1]; eps[2] = H[2][2];
    eps[3] = H[0][1] + H[1][0]; eps[4] = H[1][2] + H[2][1]; eps[5] = H[0][2] + H[2][0];
    const double tr = eps[0] + eps[1] + eps[2];
    for (int i = 0; i < 3; ++i) sig[i] = L * tr + 2 * M * eps[i];
    for (int i = 3; i < 6; ++i) sig[i] = M * eps[i];
  }
  const int64_t eo = elem_new2old[e];
  for (int i = 0; i < S; ++i) {
    if (strain) strain[eo * S + i] = eps[i];
    if (stress) stress[eo * S + i] = sig[i];
  }
  if (mises) {
    double m2;
    if (DIM == 2) m2 = sig[0] * sig[0] - sig[0] * sig[1] + sig[1] * sig[1] + 3 * sig[2] * sig[2];
    else
      m2 = 0.5 * ((sig[0] - sig[1]) * (sig[0] - sig[1]) + (sig[1] - sig[2]) * (sig[1] - sig[2]) +
                  (sig[2] - sig[0]) * (sig[2] - sig[0])) + 3 * (sig[3] * sig[3] + sig[4] * sig[4] + sig[5] * sig[5]);
    mises[eo] = sqrt(m2);
  }
}

}  // namespace cfem
