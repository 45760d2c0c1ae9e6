/*
 * fem_oracle.c -- TEST INFRASTRUCTURE ONLY (see fem_oracle.h).
 *
 * CPU restatement of the reference's EbE elasticity path. Used by tests/ as
 * the parity reference and by bench.py's cpu_baseline leg; never by the product.
 */
#include "fem_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

/* Ricker / Berlage in the reference's float arithmetic (fem_utils.cpp:53-82).
 * The phase uses double M_PI exactly as the reference expression does. */
static float ricker_f32(float t, float ampl, float freq) {
  float tmp = (float)(M_PI * freq * t - M_PI);
  return ampl * (1.f - 2.f * tmp * tmp) * expf(-1.f * tmp * tmp);
}

static float berlage_f32(float t, float ampl, float freq) {
  float w0 = (float)(2 * M_PI * freq);
  float w1 = w0 / sqrtf(3.f);
  return ampl * w1 * w1 / 4.f * expf(-1.f * w1 * t) *
         (sinf(w0 * t) * (1.f / (w1 * w1 * w1) + t / (w1 * w1) - t * t / w1) -
          cosf(w0 * t) * sqrtf(3.f) * (t * t / w1 + t / (w1 * w1)));
}

float orc_wavelet_value_f32(const orc_wavelet *w, float t) {
  if (!w) return 0.f;
  float ts = (float)w->timeshift;
  if (t < ts) return 0.f;
  if (w->type == ORC_WAVELET_RICKER) return ricker_f32(t - ts, (float)w->ampl, (float)w->freq);
  if (w->type == ORC_WAVELET_BERLAGE) return berlage_f32(t - ts, (float)w->ampl, (float)w->freq);
  return 0.f;
}

#define REAL float
#define SFX _f32
#include "ebe_port.inc"
#undef REAL
#undef SFX
#define REAL double
#define SFX _f64
#include "ebe_port.inc"
#undef REAL
#undef SFX

int orc_ebe_static_f32(const orc_problem *p, const orc_wavelet *w, double eps, float *u_out, int32_t *iters) {
  return ebe_static_impl_f32(p, w, eps, u_out, iters);
}
int orc_ebe_static_f64(const orc_problem *p, const orc_wavelet *w, double eps, double *u_out, int32_t *iters) {
  return ebe_static_impl_f64(p, w, eps, u_out, iters);
}
int orc_ebe_dyn_f32(const orc_problem *p, const orc_wavelet *w, const orc_dyn *d, float *u_out, int32_t *steps,
                    int64_t *pcg_iters) {
  return ebe_dyn_impl_f32(p, w, d, u_out, steps, pcg_iters);
}
int orc_ebe_dyn_f64(const orc_problem *p, const orc_wavelet *w, const orc_dyn *d, double *u_out, int32_t *steps,
                    int64_t *pcg_iters) {
  return ebe_dyn_impl_f64(p, w, d, u_out, steps, pcg_iters);
}

int orc_ebe_setup_f32(const orc_problem *p, const orc_wavelet *w, float *mask, float *adj, float *klocals,
                      float *diagk, float *flocals, float *areas) {
  ebe_f32 m;
  int rc = ebe_init_f32(&m, p);
  if (rc) { ebe_free_f32(&m); return rc; }
  int64_t n = m.ne * m.w;
  ebe_klocals_f32(&m);
  ebe_face_lengths_f32(&m);
  ebe_flocals_f32(&m, w, 0.f);
  if (mask) for (int64_t i = 0; i < n; ++i) mask[i] = (float)m.mask[i];
  if (adj) for (int64_t k = 0; k < m.nd; ++k) adj[k] = m.adj[k];
  if (klocals) memcpy(klocals, m.K, sizeof(float) * n * m.w);
  if (diagk)
    for (int64_t e = 0; e < m.ne; ++e)
      for (int j = 0; j < m.w; ++j) diagk[e * m.w + j] = m.K[e * m.w * m.w + m.w * j + j];
  if (flocals) memcpy(flocals, m.Fl, sizeof(float) * n);
  if (areas) memcpy(areas, m.area, sizeof(float) * m.ne);
  ebe_free_f32(&m);
  return 0;
}

static double wall_s(void) {
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return ts.tv_sec + 1e-9 * ts.tv_nsec;
}

int orc_ebe_time_f32(const orc_problem *p, int32_t k, double *setup_s, double *iter_s) {
  double t0 = wall_s();
  ebe_f32 m;
  int rc = ebe_init_f32(&m, p);
  if (rc) { ebe_free_f32(&m); return rc; }
  int64_t n = m.ne * m.w;
  ebe_klocals_f32(&m);
  float *diag = (float *)malloc(sizeof(float) * n);
  for (int64_t e = 0; e < m.ne; ++e)
    for (int j = 0; j < m.w; ++j) diag[e * m.w + j] = m.K[e * m.w * m.w + m.w * j + j];
  ebe_face_lengths_f32(&m);
  ebe_flocals_f32(&m, NULL, 0.f);
  cgm_f32 v;
  cgm_alloc_f32(&v, n);
  memcpy(v.r, m.Fl, sizeof(float) * n);
  double t1 = wall_s();
  /* k iterations of the same loop body as ebe_pcg_f32 (no stopping test). */
  ebe_asm_gather_f32(&m, diag, v.mm);
  for (int64_t i = 0; i < n; ++i) v.z[i] = v.r[i] / v.mm[i];
  ebe_asm_gather_f32(&m, v.z, v.s);
  float gamma = ebe_dot_f32(v.r, v.s, n);
  memcpy(v.p, v.s, sizeof(float) * n);
  double t2 = wall_s();
  for (int it = 0; it < k; ++it) {
    ebe_bmm_f32(&m, v.p, v.u);
    float sum = ebe_dot_f32(v.p, v.u, n), alpha = gamma / sum;
    ebe_axpby_f32(v.x, 1.f, v.p, alpha, n);
    ebe_axpby_f32(v.r, 1.f, v.u, -1.f * alpha, n);
    for (int64_t i = 0; i < n; ++i) v.z[i] = v.r[i] / v.mm[i];
    ebe_asm_gather_f32(&m, v.z, v.s);
    float gnew = ebe_dot_f32(v.r, v.s, n);
    ebe_axpby_f32(v.p, gnew / gamma, v.s, 1.f, n);
    gamma = gnew;
  }
  double t3 = wall_s();
  if (setup_s) *setup_s = t1 - t0;
  if (iter_s) *iter_s = k > 0 ? (t3 - t2) / k : 0;
  free(diag);
  cgm_free_f32(&v);
  ebe_free_f32(&m);
  return 0;
}

/* ======================= FP64 global-vector form ======================== */

struct orc_ctx {
  ebe_f64 m;        /* mask, stable permutation, K_e (constrained, FP64), |det| */
  int dim, w, nv, consistent;
  int64_t ne, nn, nd;
  double *Ee;       /* per-element Young's modulus */
  double *vol;      /* element volume (area in 2D) */
  double *diag;     /* assembled diagonal of K' */
  double *yloc;     /* ne*w scratch */
  double *Floc;     /* ne*w scratch for RHS slot semantics */
  double *press;    /* current face pressures (reference semantics, Q8) */
  double *press0;   /* file pressures */
  double *fscale;   /* consistent traction factor per face: L/2 (2D) or A/3 (3D) */
  double rho, E;
  int32_t *ctype;   /* per-node constraint code or 0 */
  /* optional assembled copy of K' in dim x dim node blocks (orc_assemble) */
  int64_t *bptr;    /* nn+1 row starts (node rows) */
  int32_t *bcol;    /* block column nodes, ascending per row */
  double *bval;     /* [block][dim][dim] */
};

int64_t orc_ndof(const orc_ctx *c) { return c->nd; }

static double dsum_blocks(const double *a, const double *b, int64_t n) {
  /* deterministic: fixed-size blocks summed in order */
  const int64_t BS = 4096;
  int64_t nb = (n + BS - 1) / BS;
  double *part = (double *)malloc(sizeof(double) * (nb > 0 ? nb : 1));
#pragma omp parallel for schedule(static)
  for (int64_t bi = 0; bi < nb; ++bi) {
    double acc = 0;
    int64_t e = (bi + 1) * BS < n ? (bi + 1) * BS : n;
    for (int64_t i = bi * BS; i < e; ++i) acc += a[i] * (b ? b[i] : a[i]);
    part[bi] = acc;
  }
  double s = 0;
  for (int64_t bi = 0; bi < nb; ++bi) s += part[bi];
  free(part);
  return s;
}

/* assembled[dof] = sum over the DOF's element slots, in element order */
static void gsum(const orc_ctx *c, const double *loc, double *glob) {
  const ebe_f64 *m = &c->m;
#pragma omp parallel for schedule(static)
  for (int64_t k = 0; k < c->nd; ++k) {
    double acc = 0;
    for (int64_t j = m->seg[k]; j < m->seg[k + 1]; ++j) acc += loc[m->perm[j]];
    glob[k] = acc;
  }
}

int orc_setup(const orc_problem *p, orc_ctx **out) {
  orc_ctx *c = (orc_ctx *)calloc(1, sizeof(orc_ctx));
  int rc = ebe_init_f64(&c->m, p);
  if (rc) { ebe_free_f64(&c->m); free(c); return rc; }
  ebe_klocals_f64(&c->m);
  ebe_face_lengths_f64(&c->m);
  c->dim = p->dim; c->w = c->m.w; c->nv = p->dim + 1; c->consistent = p->consistent;
  c->ne = p->n_elems; c->nn = p->n_nodes; c->nd = c->m.nd; c->rho = p->rho; c->E = p->E;
  c->Ee = (double *)malloc(sizeof(double) * c->ne);
  c->vol = (double *)malloc(sizeof(double) * c->ne);
  const int w = c->w;
  for (int64_t e = 0; e < c->ne; ++e) {
    c->Ee[e] = p->elem_E ? p->elem_E[e] : p->E;
    c->vol[e] = c->m.area[e] / (c->dim == 2 ? 2.0 : 6.0);
    if (p->elem_E) {
      double sc = p->elem_E[e] / p->E;
      for (int i = 0; i < w * w; ++i) c->m.K[e * w * w + i] *= sc;
    }
  }
  c->yloc = (double *)malloc(sizeof(double) * c->ne * w);
  c->Floc = (double *)calloc((size_t)(c->ne * w), sizeof(double));
  double *dloc = (double *)malloc(sizeof(double) * c->ne * w);
  for (int64_t e = 0; e < c->ne; ++e)
    for (int j = 0; j < w; ++j) dloc[e * w + j] = c->m.K[e * w * w + w * j + j];
  c->diag = (double *)malloc(sizeof(double) * c->nd);
  gsum(c, dloc, c->diag);
  free(dloc);
  c->ctype = (int32_t *)calloc((size_t)c->nn, sizeof(int32_t));
  for (int64_t i = 0; i < p->n_constraints; ++i) c->ctype[p->cons[2 * i]] = p->cons[2 * i + 1];
  int64_t nf = c->m.nf;
  c->press = (double *)malloc(sizeof(double) * (nf > 0 ? nf : 1));
  c->press0 = (double *)malloc(sizeof(double) * (nf > 0 ? nf : 1));
  c->fscale = (double *)malloc(sizeof(double) * (nf > 0 ? nf : 1));
  for (int64_t f = 0; f < nf; ++f) {
    c->press[f] = c->press0[f] = p->face_pressure[f];
    if (c->dim == 2) {
      c->fscale[f] = 0.5 * c->m.flen[f];
    } else {
      /* flen holds 0.5*|a x b|^2 (reference quirk); the area is 0.5*|a x b| */
      double cr2 = 2.0 * c->m.flen[f];
      c->fscale[f] = 0.5 * sqrt(cr2) / 3.0;
    }
  }
  *out = c;
  return 0;
}

void orc_free(orc_ctx *c) {
  if (!c) return;
  ebe_free_f64(&c->m);
  free(c->Ee); free(c->vol); free(c->diag); free(c->yloc); free(c->Floc); free(c->press); free(c->press0);
  free(c->fscale); free(c->ctype);
  free(c->bptr); free(c->bcol); free(c->bval);
  free(c);
}

void orc_get_mask(const orc_ctx *c, int32_t *mask) { memcpy(mask, c->m.mask, sizeof(int32_t) * c->ne * c->w); }

void orc_get_adjacency(const orc_ctx *c, int32_t *adj) {
  for (int64_t k = 0; k < c->nd; ++k) adj[k] = (int32_t)(c->m.seg[k + 1] - c->m.seg[k]);
}

void orc_get_bc(const orc_ctx *c, uint8_t *cons) { memcpy(cons, c->m.cdof, (size_t)c->nd); }

void orc_get_element_matrices(const orc_ctx *c, double *ke) {
  const int w = c->w;
  for (int64_t e = 0; e < c->ne; ++e)
    for (int r = 0; r < w; ++r)
      for (int q = 0; q < w; ++q) ke[e * w * w + r * w + q] = c->m.K[e * w * w + r + q * w];
}

void orc_get_diag(const orc_ctx *c, double *d) { memcpy(d, c->diag, sizeof(double) * c->nd); }

static int cmp_i32(const void *a, const void *b) {
  const int32_t x = *(const int32_t *)a, y = *(const int32_t *)b;
  return (x > y) - (x < y);
}

/* Node neighbours of node i (itself included), sorted and unique; returns the count. */
static int64_t node_row(const orc_ctx *c, const int64_t *eptr, const int32_t *elist, int64_t i, int32_t *buf) {
  const int nv = c->nv;
  int64_t n = 0;
  for (int64_t k = eptr[i]; k < eptr[i + 1]; ++k)
    for (int b = 0; b < nv; ++b) buf[n++] = c->m.el[(int64_t)elist[k] * nv + b];
  qsort(buf, (size_t)n, sizeof(int32_t), cmp_i32);
  int64_t u = 0;
  for (int64_t k = 0; k < n; ++k)
    if (u == 0 || buf[k] != buf[u - 1]) buf[u++] = buf[k];
  return u;
}

int orc_assemble(orc_ctx *c) {
  const int dim = c->dim, nv = c->nv, w = c->w, bs = dim * dim;
  const int64_t nn = c->nn, ne = c->ne;
  if (c->bptr) return 0;
  /* node -> incident elements, in element order */
  int64_t *eptr = (int64_t *)calloc((size_t)nn + 1, sizeof(int64_t));
  int32_t *elist = (int32_t *)malloc(sizeof(int32_t) * (size_t)(ne * nv));
  for (int64_t e = 0; e < ne; ++e)
    for (int a = 0; a < nv; ++a) eptr[c->m.el[e * nv + a] + 1]++;
  int maxdeg = 0;
  for (int64_t i = 0; i < nn; ++i) {
    if (eptr[i + 1] > maxdeg) maxdeg = (int)eptr[i + 1];
    eptr[i + 1] += eptr[i];
  }
  int64_t *fill = (int64_t *)malloc(sizeof(int64_t) * (size_t)nn);
  memcpy(fill, eptr, sizeof(int64_t) * (size_t)nn);
  for (int64_t e = 0; e < ne; ++e)
    for (int a = 0; a < nv; ++a) elist[fill[c->m.el[e * nv + a]]++] = (int32_t)e;
  free(fill);
  c->bptr = (int64_t *)calloc((size_t)nn + 1, sizeof(int64_t));
  const size_t bufn = (size_t)maxdeg * nv + 1;
#pragma omp parallel
  {
    int32_t *buf = (int32_t *)malloc(sizeof(int32_t) * bufn);
#pragma omp for schedule(static)
    for (int64_t i = 0; i < nn; ++i) c->bptr[i + 1] = node_row(c, eptr, elist, i, buf);
    free(buf);
  }
  for (int64_t i = 0; i < nn; ++i) c->bptr[i + 1] += c->bptr[i];
  c->bcol = (int32_t *)malloc(sizeof(int32_t) * (size_t)(c->bptr[nn] > 0 ? c->bptr[nn] : 1));
  c->bval = (double *)calloc((size_t)c->bptr[nn] * bs + 1, sizeof(double));
  /* each row sums its blocks over its incident elements in element order */
#pragma omp parallel
  {
    int32_t *buf = (int32_t *)malloc(sizeof(int32_t) * bufn);
#pragma omp for schedule(static)
    for (int64_t i = 0; i < nn; ++i) {
      const int64_t r0 = c->bptr[i], n = node_row(c, eptr, elist, i, buf);
      memcpy(c->bcol + r0, buf, sizeof(int32_t) * (size_t)n);
      for (int64_t k = eptr[i]; k < eptr[i + 1]; ++k) {
        const int64_t e = elist[k];
        const double *K = c->m.K + e * w * w; /* column-major: K[row + col * w] */
        int a = 0;
        while (c->m.el[e * nv + a] != i) ++a;
        for (int b = 0; b < nv; ++b) {
          const int32_t j = c->m.el[e * nv + b];
          const int32_t *hit = (const int32_t *)bsearch(&j, c->bcol + r0, (size_t)n, sizeof(int32_t), cmp_i32);
          double *blk = c->bval + (r0 + (hit - (c->bcol + r0))) * bs;
          for (int di = 0; di < dim; ++di)
            for (int dj = 0; dj < dim; ++dj) blk[di * dim + dj] += K[(dim * a + di) + (dim * b + dj) * w];
        }
      }
    }
    free(buf);
  }
  free(eptr);
  free(elist);
  return 0;
}

void orc_matvec(const orc_ctx *c, const double *x, double *y) {
  const int w = c->w;
  const ebe_f64 *m = &c->m;
  if (c->bptr) {
    const int dim = c->dim, bs = dim * dim;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < c->nn; ++i) {
      double acc[3] = {0, 0, 0};
      for (int64_t k = c->bptr[i]; k < c->bptr[i + 1]; ++k) {
        const double *blk = c->bval + k * bs, *xj = x + (int64_t)dim * c->bcol[k];
        for (int di = 0; di < dim; ++di)
          for (int dj = 0; dj < dim; ++dj) acc[di] += blk[di * dim + dj] * xj[dj];
      }
      for (int di = 0; di < dim; ++di) y[(int64_t)dim * i + di] = acc[di];
    }
    return;
  }
#pragma omp parallel for schedule(static)
  for (int64_t e = 0; e < c->ne; ++e) {
    double xe[12];
    for (int k = 0; k < w; ++k) xe[k] = x[m->mask[e * w + k]];
    const double *K = m->K + e * w * w;
    for (int n = 0; n < w; ++n) {
      double acc = 0;
      for (int k = 0; k < w; ++k) acc += xe[k] * K[k + n * w];
      c->yloc[e * w + n] = acc;
    }
  }
  gsum(c, c->yloc, y);
}

/* Stress recovery per element (deprecated/femfunc/femfunc.cpp:42-106):
 * strain = B u_e with the element's B (rows xx, yy, [zz,] xy, [yz, xz];
 * engineering shear), stress = D strain with D scaled by E_e / E. The
 * reference's von Mises line for 2D is commented out there; the textbook
 * formula is used (2D: its commented expression; 3D: the usual invariant).
 * The element B of the current reference divides the cofactors by |det|
 * (cpu_fem_utils.cpp:396, 434), which is -grad N on an element of negative
 * orientation: K_e = B'DB does not see the sign, a strain does. B is taken
 * times sign(det) here, so that strain = sym(grad u) on every element. */
void orc_element_stress(const orc_ctx *c, const double *u, double *strain, double *stress, double *mises) {
  const int w = c->w, s = c->m.s;
  const ebe_f64 *m = &c->m;
#pragma omp parallel for schedule(static)
  for (int64_t e = 0; e < c->ne; ++e) {
    double eps[6] = {0, 0, 0, 0, 0, 0}, sig[6] = {0, 0, 0, 0, 0, 0};
    const double *B = m->B + e * s * w;
    const int nv = c->nv, dim = c->dim;
    const double *x0 = m->nodes + (int64_t)m->el[e * nv] * dim;
    double a[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
    for (int k = 1; k < nv; ++k)
      for (int d = 0; d < dim; ++d) a[k - 1][d] = m->nodes[(int64_t)m->el[e * nv + k] * dim + d] - x0[d];
    const double det = dim == 2 ? a[0][0] * a[1][1] - a[0][1] * a[1][0]
                                : a[0][0] * (a[1][1] * a[2][2] - a[1][2] * a[2][1]) -
                                      a[0][1] * (a[1][0] * a[2][2] - a[1][2] * a[2][0]) +
                                      a[0][2] * (a[1][0] * a[2][1] - a[1][1] * a[2][0]);
    const double sgn = det < 0 ? -1.0 : 1.0;
    for (int i = 0; i < s; ++i) {
      for (int j = 0; j < w; ++j) eps[i] += B[i * w + j] * u[m->mask[e * w + j]];
      eps[i] *= sgn;
    }
    const double sc = c->Ee[e] / c->E;
    for (int i = 0; i < s; ++i) {
      for (int k = 0; k < s; ++k) sig[i] += m->D[i + k * s] * eps[k];
      sig[i] *= sc;
    }
    for (int i = 0; i < s; ++i) {
      if (strain) strain[e * s + i] = eps[i];
      if (stress) stress[e * s + i] = sig[i];
    }
    if (mises) {
      double m2;
      if (c->dim == 2)
        m2 = sig[0] * sig[0] - sig[0] * sig[1] + sig[1] * sig[1] + 3 * sig[2] * sig[2];
      else
        m2 = 0.5 * ((sig[0] - sig[1]) * (sig[0] - sig[1]) + (sig[1] - sig[2]) * (sig[1] - sig[2]) +
                    (sig[2] - sig[0]) * (sig[2] - sig[0])) +
             3 * (sig[3] * sig[3] + sig[4] * sig[4] + sig[5] * sig[5]);
      mises[e] = sqrt(m2);
    }
  }
}

/* Time factor applied to file loads in consistent mode. */
static double consistent_scale(const orc_wavelet *wv, float t) {
  if (!wv || wv->type == ORC_WAVELET_NONE) return 1.0;
  if (wv->ampl == 0) return 0.0;
  return (double)orc_wavelet_value_f32(wv, t) / wv->ampl;
}

void orc_get_rhs(orc_ctx *c, const orc_wavelet *wv, double t_in, double *f) {
  const int dim = c->dim, w = c->w, nv = c->nv;
  const ebe_f64 *m = &c->m;
  float t = (float)t_in;
  if (!c->consistent) {
    /* compat: slot semantics of calcPressures, then calcLoads overwriting all slots */
    if (m->nl > 0) {
      double *loads = (double *)calloc((size_t)c->nd, sizeof(double));
      for (int64_t l = 0; l < m->nl; ++l)
        for (int d = 0; d < dim; ++d) loads[(int64_t)dim * m->lnode[l] + d] = m->lvec[l * dim + d];
      for (int64_t k = 0; k < c->nd; ++k) f[k] = loads[k] * (double)(m->seg[k + 1] - m->seg[k]);
      free(loads);
      if (m->nf > 0) {
        double v = (double)orc_wavelet_value_f32(wv, t);
        if (v != 0) for (int64_t q = 0; q < m->nf; ++q) c->press[q] = v;
      }
      return;
    }
    memset(c->Floc, 0, sizeof(double) * c->ne * w);
    if (m->nf > 0) {
      double v = (double)orc_wavelet_value_f32(wv, t);
      if (v != 0) for (int64_t q = 0; q < m->nf; ++q) c->press[q] = v;
      double coeff = dim == 2 ? -0.5 : -1.0 / 12.0;
      for (int64_t q = 0; q < m->nf; ++q) {
        int64_t e = m->felem[q];
        for (int i = 0; i < dim; ++i) {
          int node = m->fnodes[q * nv + i], loc = -1;
          for (int a = 0; a < nv; ++a)
            if (m->el[e * nv + a] == node) { loc = a; break; }
          if (loc < 0) continue;
          for (int j = 0; j < dim; ++j) {
            int masked = c->ctype[node] & j;
            c->Floc[e * w + dim * loc + j] = masked ? 0.0 : coeff * c->press[q] * m->flen[q] * m->fnorm[q * dim + j];
          }
        }
      }
    }
    gsum(c, c->Floc, f);
    return;
  }
  /* consistent: accumulate tractions p*L/2 (2D) or p*A/3 (3D) per face node and
   * point loads once, both scaled by the wavelet; constrained DOFs get zero. */
  memset(f, 0, sizeof(double) * c->nd);
  double s = consistent_scale(wv, t);
  for (int64_t q = 0; q < m->nf; ++q)
    for (int i = 0; i < dim; ++i) {
      int node = m->fnodes[q * nv + i];
      for (int j = 0; j < dim; ++j)
        f[(int64_t)dim * node + j] += -c->press0[q] * s * c->fscale[q] * m->fnorm[q * dim + j];
    }
  for (int64_t l = 0; l < m->nl; ++l)
    for (int d = 0; d < dim; ++d) f[(int64_t)dim * m->lnode[l] + d] += m->lvec[l * dim + d] * s;
  for (int64_t k = 0; k < c->nd; ++k)
    if (m->cdof[k]) f[k] = 0;
}

/* Generic Jacobi PCG on an operator given by a callback. */
typedef void (*orc_op)(const orc_ctx *c, const double *x, double *y, void *user);

static void op_k(const orc_ctx *c, const double *x, double *y, void *user) {
  (void)user;
  orc_matvec(c, x, y);
}

static int pcg_generic(const orc_ctx *c, orc_op op, void *user, const double *dinv_src, const double *f,
                       double *x, int warm, double tol, int rule, int maxit, int32_t *iters) {
  int64_t n = c->nd;
  double *r = (double *)malloc(sizeof(double) * n), *z = (double *)malloc(sizeof(double) * n);
  double *pp = (double *)malloc(sizeof(double) * n), *u = (double *)malloc(sizeof(double) * n);
  if (warm) {
    op(c, x, u, user);
    for (int64_t i = 0; i < n; ++i) r[i] = f[i] - u[i];
  } else {
    memset(x, 0, sizeof(double) * n);
    memcpy(r, f, sizeof(double) * n);
  }
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n; ++i) z[i] = r[i] / dinv_src[i];
  memcpy(pp, z, sizeof(double) * n);
  double g0 = dsum_blocks(r, z, n), g = g0;
  double fn = sqrt(dsum_blocks(f, NULL, n));
  int it = 0, rc = 0;
  if (rule == 1 && sqrt(dsum_blocks(r, NULL, n)) <= tol * fn) goto done;
  if (g0 == 0) goto done;
  for (;;) {
    ++it;
    op(c, pp, u, user);
    double sg = dsum_blocks(pp, u, n), alpha = g / sg;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) { x[i] += alpha * pp[i]; r[i] -= alpha * u[i]; z[i] = r[i] / dinv_src[i]; }
    double gn = dsum_blocks(r, z, n);
    if (rule == 0 && gn < tol * g0) break;
    if (rule == 1 && sqrt(dsum_blocks(r, NULL, n)) <= tol * fn) break;
    if (!isfinite(gn)) { rc = -3; break; }
    if (it >= maxit) { rc = -4; break; }
    double beta = gn / g;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) pp[i] = z[i] + beta * pp[i];
    g = gn;
  }
done:
  if (iters) *iters = it;
  free(r); free(z); free(pp); free(u);
  return rc;
}

int orc_pcg(const orc_ctx *c, const double *f, double *x, double tol, int32_t rule, int32_t maxit,
            int32_t *iters) {
  return pcg_generic(c, op_k, NULL, c->diag, f, x, 0, tol, rule, maxit, iters);
}

int orc_pcg_warm(const orc_ctx *c, const double *f, double *x, double tol, int32_t rule, int32_t maxit,
                 int32_t *iters) {
  return pcg_generic(c, op_k, NULL, c->diag, f, x, 1, tol, rule, maxit, iters);
}

/* Element mass blocks: lumped (per DOF) or consistent (w x w, same-component coupling). */
/* The same FP32 port, set up once and then timed in samples of k iterations
 * (the reference arm of the benchmark times one sample per step). */
struct orc_ebe_timer {
  ebe_f32 m;
  cgm_f32 v;
  float gamma;
  int64_t n;
  double setup_s, init_s;
};

int orc_ebe_timer_create(const orc_problem *p, orc_ebe_timer **out) {
  orc_ebe_timer *t = (orc_ebe_timer *)calloc(1, sizeof(orc_ebe_timer));
  double t0 = wall_s();
  int rc = ebe_init_f32(&t->m, p);
  if (rc) { ebe_free_f32(&t->m); free(t); return rc; }
  ebe_f32 *m = &t->m;
  const int64_t n = m->ne * m->w;
  t->n = n;
  ebe_klocals_f32(m);
  float *diag = (float *)malloc(sizeof(float) * n);
  for (int64_t e = 0; e < m->ne; ++e)
    for (int j = 0; j < m->w; ++j) diag[e * m->w + j] = m->K[e * m->w * m->w + m->w * j + j];
  ebe_face_lengths_f32(m);
  ebe_flocals_f32(m, NULL, 0.f);
  cgm_alloc_f32(&t->v, n);
  memcpy(t->v.r, m->Fl, sizeof(float) * n);
  double t1 = wall_s();
  ebe_asm_gather_f32(m, diag, t->v.mm);
  for (int64_t i = 0; i < n; ++i) t->v.z[i] = t->v.r[i] / t->v.mm[i];
  ebe_asm_gather_f32(m, t->v.z, t->v.s);
  t->gamma = ebe_dot_f32(t->v.r, t->v.s, n);
  memcpy(t->v.p, t->v.s, sizeof(float) * n);
  free(diag);
  t->setup_s = t1 - t0;
  t->init_s = wall_s() - t1;
  *out = t;
  return 0;
}

/* k more iterations of the loop body of ebe_pcg_f32 (no stopping test);
 * returns their wall time in seconds. */
double orc_ebe_timer_iters(orc_ebe_timer *t, int32_t k) {
  ebe_f32 *m = &t->m;
  cgm_f32 *v = &t->v;
  const int64_t n = t->n;
  double t0 = wall_s();
  for (int it = 0; it < k; ++it) {
    ebe_bmm_f32(m, v->p, v->u);
    float sum = ebe_dot_f32(v->p, v->u, n), alpha = t->gamma / sum;
    ebe_axpby_f32(v->x, 1.f, v->p, alpha, n);
    ebe_axpby_f32(v->r, 1.f, v->u, -1.f * alpha, n);
    for (int64_t i = 0; i < n; ++i) v->z[i] = v->r[i] / v->mm[i];
    ebe_asm_gather_f32(m, v->z, v->s);
    float gnew = ebe_dot_f32(v->r, v->s, n);
    ebe_axpby_f32(v->p, gnew / t->gamma, v->s, 1.f, n);
    t->gamma = gnew;
  }
  return wall_s() - t0;
}

void orc_ebe_timer_info(const orc_ebe_timer *t, double *setup_s, double *init_s) {
  if (setup_s) *setup_s = t->setup_s;
  if (init_s) *init_s = t->init_s;
}

void orc_ebe_timer_free(orc_ebe_timer *t) {
  if (!t) return;
  cgm_free_f32(&t->v);
  ebe_free_f32(&t->m);
  free(t);
}

int orc_num_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

static void mass_coeffs(const orc_ctx *c, int64_t e, int lumped, double *md, double *mo) {
  /* md: diagonal (or lumped) entry, mo: same-component off-diagonal entry */
  double mass = c->rho * c->vol[e];
  if (!c->consistent) {
    if (c->dim == 2) { *md = lumped ? mass / 3 : mass / 6; *mo = lumped ? 0 : mass / 12; }
    else { *md = lumped ? mass / 12 : mass / 24; *mo = lumped ? 0 : mass / 48; }
  } else {
    if (c->dim == 2) { *md = lumped ? mass / 3 : mass / 6; *mo = lumped ? 0 : mass / 12; }
    else { *md = lumped ? mass / 4 : mass / 10; *mo = lumped ? 0 : mass / 20; }
  }
}

typedef struct { double cK; } dyn_op_user;

/* consistent implicit operator: P (M + cK K) P + (I - P) diag(M + cK K) */
static void op_mk(const orc_ctx *c, const double *x, double *y, void *user) {
  const dyn_op_user *du = (const dyn_op_user *)user;
  const int w = c->w, dim = c->dim, nv = c->nv;
  const ebe_f64 *m = &c->m;
  orc_matvec(c, x, y);
  for (int64_t k = 0; k < c->nd; ++k) y[k] *= du->cK;
#pragma omp parallel for schedule(static)
  for (int64_t e = 0; e < c->ne; ++e) {
    double md, mo;
    mass_coeffs(c, e, 0, &md, &mo);
    for (int a = 0; a < nv; ++a)
      for (int d = 0; d < dim; ++d) {
        int64_t da = m->mask[e * w + dim * a + d];
        double acc = md * x[da];
        if (!m->cdof[da])
          for (int b = 0; b < nv; ++b) {
            if (b == a) continue;
            int64_t db = m->mask[e * w + dim * b + d];
            if (!m->cdof[db]) acc += mo * x[db];
          }
        c->yloc[e * w + dim * a + d] = acc;
      }
  }
  double *tmp = (double *)malloc(sizeof(double) * c->nd);
  gsum(c, c->yloc, tmp);
  for (int64_t k = 0; k < c->nd; ++k) y[k] += tmp[k];
  free(tmp);
}

int orc_dyn_run(orc_ctx *c, const orc_wavelet *wv, const orc_dyn *dp, double pcg_tol, int32_t pcg_rule,
                double *u_out, int32_t *steps_out, int64_t *pcg_out) {
  const int w = c->w;
  const int64_t nd = c->nd, nloc = c->ne * w;
  const ebe_f64 *m = &c->m;
  double beta1 = dp->beta1, beta2 = dp->beta2, dt = dp->dt;
  int is_explicit = beta2 == 0;
  float dtf = (float)dp->dt, endf = (float)dp->endtime;
  int relax = endf < 0, endnt = relax ? 1 : (int)(endf / dtf);
  double *d = (double *)calloc((size_t)nd, sizeof(double)), *v = (double *)calloc((size_t)nd, sizeof(double));
  double *a = (double *)calloc((size_t)nd, sizeof(double)), *r = (double *)malloc(sizeof(double) * nd);
  double *f = (double *)malloc(sizeof(double) * nd), *masm = (double *)malloc(sizeof(double) * nd);
  double *eloc = (double *)malloc(sizeof(double) * nloc), *etmp = (double *)malloc(sizeof(double) * nloc);
  double cK = 0.5 * beta2 * dt * dt;
  /* element-local source of the diagonal used by the explicit solve / preconditioner */
  for (int64_t e = 0; e < c->ne; ++e) {
    double md, mo;
    mass_coeffs(c, e, is_explicit, &md, &mo);
    for (int j = 0; j < w; ++j)
      eloc[e * w + j] = is_explicit ? md : cK * m->K[e * w * w + w * j + j] + md;
  }
  for (int64_t k = 0; k < c->m.nf; ++k) c->press[k] = c->press0[k];
  dyn_op_user du = {cK};
  int rc = 0, nt = 1;
  int64_t total = 0;
  for (;;) {
    float t = (float)nt * dtf;
    for (int64_t k = 0; k < nd; ++k) {
      d[k] += dt * v[k] + 0.5 * (1 - beta2) * dt * dt * a[k];
      v[k] += (1 - beta1) * dt * a[k];
    }
    orc_matvec(c, d, r);
    orc_get_rhs(c, wv, (double)t, f);
    for (int64_t k = 0; k < nd; ++k) r[k] = f[k] - r[k];
    /* assembled diagonal; compat re-sorts the element-local source in place
     * each time it is assembled (cpu_fem_utils.cpp:437-445) */
    gsum(c, eloc, masm);
    if (!c->consistent) {
      for (int64_t j = 0; j < nloc; ++j) etmp[j] = eloc[m->perm[j]];
      memcpy(eloc, etmp, sizeof(double) * nloc);
    }
    if (is_explicit) {
      for (int64_t k = 0; k < nd; ++k) a[k] = r[k] / masm[k];
    } else {
      int32_t it = 0;
      if (!c->consistent)
        rc = pcg_generic(c, op_k, NULL, masm, r, a, 0, 1e-4, 0, 1000000, &it);
      else
        rc = pcg_generic(c, op_mk, &du, masm, r, a, 1, pcg_tol, pcg_rule, 1000000, &it);
      total += it;
      if (rc) break;
    }
    for (int64_t k = 0; k < nd; ++k) {
      v[k] += beta1 * dt * a[k];
      if (!is_explicit) d[k] += 0.5 * beta2 * dt * dt * a[k];
    }
    ++nt;
    if (nt > endnt) break;
  }
  memcpy(u_out, d, sizeof(double) * nd);
  if (steps_out) *steps_out = nt - 1;
  if (pcg_out) *pcg_out = total;
  free(d); free(v); free(a); free(r); free(f); free(masm); free(eloc); free(etmp);
  return rc;
}

void orc_grad_E(const orc_ctx *c, const double *lambda, const double *u, double *g) {
  const int w = c->w;
  const ebe_f64 *m = &c->m;
#pragma omp parallel for schedule(static)
  for (int64_t e = 0; e < c->ne; ++e) {
    double le[12], ue[12];
    for (int k = 0; k < w; ++k) { le[k] = lambda[m->mask[e * w + k]]; ue[k] = u[m->mask[e * w + k]]; }
    const double *K = m->K + e * w * w;
    double acc = 0;
    for (int n = 0; n < w; ++n) {
      double t = 0;
      for (int k = 0; k < w; ++k) t += le[k] * K[k + n * w];
      acc += t * ue[n];
    }
    g[e] = -acc / c->Ee[e];
  }
}

/* Per-element accumulation g_e += -(1/E_e) w_e^T K'_e d_e. */
static void grad_acc(const orc_ctx *c, const double *wv, const double *dv, double *g) {
  const int w = c->w;
  const ebe_f64 *m = &c->m;
#pragma omp parallel for schedule(static)
  for (int64_t e = 0; e < c->ne; ++e) {
    double we[12], de[12];
    for (int k = 0; k < w; ++k) { we[k] = wv[m->mask[e * w + k]]; de[k] = dv[m->mask[e * w + k]]; }
    const double *K = m->K + e * w * w;
    double acc = 0;
    for (int n = 0; n < w; ++n) {
      double t = 0;
      for (int k = 0; k < w; ++k) t += we[k] * K[k + n * w];
      acc += t * de[n];
    }
    g[e] -= acc / c->Ee[e];
  }
}

double orc_dyn_adjoint(orc_ctx *c, const orc_wavelet *wv, const orc_dyn *dp, int32_t n_rec, const int32_t *rec,
                       const double *obs, double *g) {
  const int dim = c->dim, w = c->w;
  const int64_t nd = c->nd;
  const double beta1 = dp->beta1, dt = dp->dt;
  const float dtf = (float)dp->dt, endf = (float)dp->endtime;
  int N = endf < 0 ? 1 : (int)(endf / dtf);
  if (N < 1) N = 1;
  const double h_old = (1 - beta1) * dt, h_new = beta1 * dt, cpred = 0.5 * dt * dt;
  /* lumped mass (consistent: rho V / (dim+1) per DOF) */
  double *mloc = (double *)malloc(sizeof(double) * c->ne * w), *M = (double *)malloc(sizeof(double) * nd);
  for (int64_t e = 0; e < c->ne; ++e) {
    double md, mo;
    mass_coeffs(c, e, 1, &md, &mo);
    for (int j = 0; j < w; ++j) mloc[e * w + j] = md;
  }
  gsum(c, mloc, M);
  free(mloc);
  double *D = (double *)calloc((size_t)(N + 1) * nd, sizeof(double));  /* all displacements */
  double *v = (double *)calloc((size_t)nd, sizeof(double)), *a = (double *)calloc((size_t)nd, sizeof(double));
  double *f = (double *)malloc(sizeof(double) * nd), *y = (double *)malloc(sizeof(double) * nd);
  for (int64_t k = 0; k < c->m.nf; ++k) c->press[k] = c->press0[k];
  double L = 0;
  for (int n = 1; n <= N; ++n) {
    float t = (float)n * dtf;
    double *dn = D + (size_t)n * nd, *dm = D + (size_t)(n - 1) * nd;
    for (int64_t k = 0; k < nd; ++k) dn[k] = dm[k] + dt * v[k] + cpred * a[k];
    orc_matvec(c, dn, y);
    orc_get_rhs(c, wv, (double)t, f);
    for (int64_t k = 0; k < nd; ++k) {
      double an = (f[k] - y[k]) / M[k];
      v[k] += h_old * a[k] + h_new * an;
      a[k] = an;
    }
    for (int r = 0; r < n_rec; ++r)
      for (int q = 0; q < dim; ++q) {
        double diff = dn[(int64_t)rec[r] * dim + q] - obs[((size_t)(n - 1) * n_rec + r) * dim + q];
        L += 0.5 * diff * diff;
      }
  }
  /* reverse sweep */
  double *db = (double *)calloc((size_t)nd, sizeof(double)), *vb = (double *)calloc((size_t)nd, sizeof(double));
  double *ab = (double *)calloc((size_t)nd, sizeof(double)), *wb = (double *)malloc(sizeof(double) * nd);
  memset(g, 0, sizeof(double) * c->ne);
  for (int n = N; n >= 1; --n) {
    double *dn = D + (size_t)n * nd;
    for (int r = 0; r < n_rec; ++r)
      for (int q = 0; q < dim; ++q) {
        int64_t k = (int64_t)rec[r] * dim + q;
        db[k] += dn[k] - obs[((size_t)(n - 1) * n_rec + r) * dim + q];
      }
    /* v_n = v + h_old a + h_new a_n ; a_n = M^-1 (F - K d_n) ; d_n = d + dt v + c a */
    for (int64_t k = 0; k < nd; ++k) {
      double an_b = ab[k] + h_new * vb[k];
      wb[k] = an_b / M[k];
      ab[k] = h_old * vb[k];
    }
    grad_acc(c, wb, dn, g);
    orc_matvec(c, wb, y);
    for (int64_t k = 0; k < nd; ++k) {
      double dtot = db[k] - y[k];
      db[k] = dtot;
      vb[k] += dt * dtot;
      ab[k] += cpred * dtot;
    }
  }
  free(D); free(v); free(a); free(f); free(y); free(db); free(vb); free(ab); free(wb); free(M);
  return L;
}
