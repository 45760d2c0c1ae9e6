// Batched independent meshes: PCG vector kernels with per-instance scalars.
//
// All instances share one node numbering in which every patch owns a
// contiguous node range [own_first[p], own_first[p+1]) and the patches of an
// instance are contiguous. The vector kernels therefore work patch by patch:
// a CTA updates the nodes a patch owns with that patch's instance scalars and
// writes the patch's partial sums; the last CTA adds them per instance
// (instance_sums: fixed order) and runs each instance's stopping test. Nodes of
// converged instances are not touched (their u stays zero: the matvec skips
// their patches).
#pragma once

#include "kernels.cuh"

namespace cfem {

template <typename T>
struct BatchVecParams {
  int n_patches, n_inst;
  const int32_t *patch_inst, *own_first, *inst_patch_off;
  Scalars *isc;
  BatchCtl *ctl;
  double *pp;        // [n_patches][3] per-patch partials
  double *scratch;   // [n_inst][3]
  int k_active;      // instances 0..k_active-1 take part (the others are done from the start)
};

// init != 0: r = f, x = 0, z = M^-1 r, gamma0 (all instances).
// init == 0: x += alpha p, r -= alpha u, z = M^-1 r, u = 0, gamma' and ||r||^2.
template <typename T>
__global__ void __launch_bounds__(kThreads) k_batch_vec(BatchVecParams<T> P, T *x, T *r, T *z, const T *p, T *u,
                                                       const T *f, const T *dinv, int init) {
  constexpr int VW = 4, DIM = 3;
  if (!init && P.ctl->all_done) return;
  for (int patch = blockIdx.x; patch < P.n_patches; patch += gridDim.x) {
    const int inst = P.patch_inst[patch];
    const Scalars &s = P.isc[inst];
    DotAcc<T> acc[3];
    const bool frozen = !init && s.done;
    if (frozen) continue;  // (uniform per CTA) its instance's sums are no longer read
    {
      const T alpha = init ? T(0) : (T)s.alpha;
      for (int n = P.own_first[patch] + threadIdx.x; n < P.own_first[patch + 1]; n += blockDim.x) {
        NodeV<T, VW> zero;
#pragma unroll
        for (int d = 0; d < VW; ++d) zero.v[d] = 0;
        const NodeV<T, VW> di = ldv<T, VW>(dinv, n);
        NodeV<T, VW> rv, xx, zz = zero;
        if (init) {
          rv = ldv<T, VW>(f, n);
          xx = zero;
        } else {
          rv = ldv<T, VW>(r, n);
          xx = ldv<T, VW>(x, n);
          const NodeV<T, VW> pv = ldv<T, VW>(p, n), uv = ldv<T, VW>(u, n);
#pragma unroll
          for (int d = 0; d < DIM; ++d) {
            xx.v[d] += alpha * pv.v[d];
            rv.v[d] -= alpha * uv.v[d];
          }
        }
        T rz = 0, rr = 0;
#pragma unroll
        for (int d = 0; d < DIM; ++d) {
          zz.v[d] = rv.v[d] * di.v[d];
          rz += rv.v[d] * zz.v[d];
          rr += rv.v[d] * rv.v[d];
        }
        acc[0].add(rz);
        acc[1].add(rr);
        if (init) acc[2].add(rr);
        stv<T, VW>(x, n, xx);
        stv<T, VW>(r, n, rv);
        stv<T, VW>(z, n, zz);
        stv<T, VW>(u, n, zero);
      }
    }
    // block_total synchronises: uniform for the whole CTA
    const double t0 = block_total<T>(acc[0]), t1 = block_total<T>(acc[1]), t2 = block_total<T>(acc[2]);
    if (threadIdx.x == 0) {
      P.pp[(size_t)patch * 3 + 0] = t0;
      P.pp[(size_t)patch * 3 + 1] = t1;
      P.pp[(size_t)patch * 3 + 2] = t2;
    }
  }
  __shared__ bool last;
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) last = atomicAdd(&P.ctl->count_up, 1u) == gridDim.x - 1;
  __syncthreads();
  if (!last) return;
  __threadfence();
  instance_sums<3>(P.pp, 3, P.inst_patch_off, P.n_inst, P.scratch, init ? nullptr : P.isc);
  __syncthreads();
  __shared__ int s_active;
  if (threadIdx.x == 0) s_active = 0;
  __syncthreads();
  for (int i = threadIdx.x; i < P.n_inst; i += blockDim.x) {
    Scalars &m = P.isc[i];
    const double a = P.scratch[i * 3], b = P.scratch[i * 3 + 1], e = P.scratch[i * 3 + 2];
    if (init) {
      m.gamma0 = m.gamma = m.gamma_prev = a;
      m.rr = b;
      m.ff = e;
      m.iter = 0;
      m.sigma = m.alpha = m.beta = 0;
      m.done = 0;
      if (i >= P.k_active || a == 0.0) m.done = 1;
      else if (m.rule == 1 && sqrt(b) <= m.tol * sqrt(e)) m.done = 1;
      else if (!isfinite(a)) m.done = 2;
    } else if (!m.done) {
      m.gamma_prev = m.gamma;
      m.gamma = a;
      m.beta = a / m.gamma_prev;
      m.rr = b;
      m.iter += 1;
      if (!isfinite(a) || !isfinite(m.alpha)) m.done = 2;
      else if (m.rule == 0 && a < m.tol * m.gamma0) m.done = 1;
      else if (m.rule == 1 && sqrt(b) <= m.tol * sqrt(m.ff)) m.done = 1;
      else if (m.iter >= m.maxit) m.done = 3;
    }
    if (!m.done) atomicAdd(&s_active, 1);
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    if (!init) P.ctl->iter += 1;
    P.ctl->all_done = s_active == 0;
    P.ctl->count_up = 0;
  }
}

// FP64 true residual per instance: r = f - Kx (Kx given in u), ||r||^2 and
// ||f||^2 per instance into out[n_inst][2]; r32 = r for instances with
// active[i] != 0, else 0 (the next inner solve's right-hand side).
static __global__ void __launch_bounds__(kThreads) k_batch_residual(BatchVecParams<double> P, const double *f,
                                                                    const double *u, double *r, float *r32,
                                                                    const int *active, double *out) {
  constexpr int VW = 4, DIM = 3;
  for (int patch = blockIdx.x; patch < P.n_patches; patch += gridDim.x) {
    const int inst = P.patch_inst[patch];
    DotAcc<double> acc[2];
    for (int n = P.own_first[patch] + threadIdx.x; n < P.own_first[patch + 1]; n += blockDim.x) {
      const NodeV<double, VW> fv = ldv<double, VW>(f, n), uv = ldv<double, VW>(u, n);
      NodeV<double, VW> rv;
      NodeV<float, VW> r3;
#pragma unroll
      for (int d = 0; d < VW; ++d) {
        rv.v[d] = d < DIM ? fv.v[d] - uv.v[d] : 0.0;
        r3.v[d] = active[inst] ? (float)rv.v[d] : 0.f;
      }
      double rr = 0, ff = 0;
#pragma unroll
      for (int d = 0; d < DIM; ++d) {
        rr += rv.v[d] * rv.v[d];
        ff += fv.v[d] * fv.v[d];
      }
      acc[0].add(rr);
      acc[1].add(ff);
      stv<double, VW>(r, n, rv);
      stv<float, VW>(r32, n, r3);
    }
    const double t0 = block_total<double>(acc[0]), t1 = block_total<double>(acc[1]);
    if (threadIdx.x == 0) {
      P.pp[(size_t)patch * 3 + 0] = t0;
      P.pp[(size_t)patch * 3 + 1] = t1;
      P.pp[(size_t)patch * 3 + 2] = 0;
    }
  }
  __shared__ bool last;
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) last = atomicAdd(&P.ctl->count_up, 1u) == gridDim.x - 1;
  __syncthreads();
  if (!last) return;
  __threadfence();
  instance_sums<3>(P.pp, 3, P.inst_patch_off, P.n_inst, P.scratch);
  __syncthreads();
  for (int i = threadIdx.x; i < P.n_inst; i += blockDim.x) {
    out[i * 2] = P.scratch[i * 3];
    out[i * 2 + 1] = P.scratch[i * 3 + 1];
  }
  if (threadIdx.x == 0) P.ctl->count_up = 0;
}

}  // namespace cfem
