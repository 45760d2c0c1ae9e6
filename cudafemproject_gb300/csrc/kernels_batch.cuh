// Batched independent meshes: PCG vector kernels with per-instance scalars.
//
// All instances share one node numbering in which every patch owns a
// contiguous node range [own_first[p], own_first[p+1]) and the patches of an
// instance are contiguous, so every instance owns one contiguous node range.
// The vector step works flat over those ranges (k_batch_vec_flat); the FP64
// residual works patch by patch with per-patch partials that the last CTA adds
// per instance (instance_sums: fixed order). Nodes of converged instances are
// not touched (their u stays zero: the matvec skips their patches).
#pragma once

#include "kernels.cuh"

namespace cfem {

constexpr int kMaxBatchInstances = 8192;  // k_batch_vec_flat: 4 n + 2 ints of shared memory

template <typename T>
struct BatchVecParams {
  int n_patches, n_inst;
  const int32_t *patch_inst, *own_first, *inst_patch_off;
  Scalars *isc;
  BatchCtl *ctl;
  double *pp;        // [n_patches][3] per-patch partials
  double *scratch;   // [n_inst][3]
  int k_active;      // instances 0..k_active-1 take part (the others are done from the start)
  double *seg;       // [grid][n_inst][3] per (CTA, instance segment) partials of k_batch_vec_flat
};

// init != 0: r = f, x = 0, z = M^-1 r, gamma0 (all instances).
// init == 0: x += alpha p, r -= alpha u, z = M^-1 r, u = 0, gamma' and ||r||^2.
// Flat over the owned nodes of the instances that take part
// (those not yet converged; at init all of them: x = 0, r = f everywhere, the
// first k_active start iterating). The instances' node
// ranges are contiguous (own_first over their patch ranges); every CTA builds
// the same list of active ranges, takes one contiguous chunk of their
// concatenation, works through it with four nodes in flight per thread, and
// writes one partial per (CTA, instance segment). The last CTA adds each
// instance's partials in CTA order (one warp per instance: a fixed order) and
// runs the stopping tests. Dynamic shared memory: 4 n_inst + 2 ints.
template <typename T>
__global__ void __launch_bounds__(kThreads) k_batch_vec_flat(BatchVecParams<T> P, T *x, T *r, T *z, const T *p, T *u,
                                                            const T *f, const T *dinv, int init) {
  constexpr int VW = 4, DIM = 3, U = 4;
  if (!init && P.ctl->all_done) return;
  extern __shared__ int s_dyn[];
  const int n = P.n_inst;
  int *s_off = s_dyn;                 // [n + 1] prefix of the active ranges' node counts
  int *s_ids = s_off + n + 1;         // [n] instance of the a-th active range
  int *s_cnt = s_ids + n;             // [n] node count, 0 if not active
  int *s_lo = s_cnt + n;              // [n + 1] first owned node of each instance (internal order)
  __shared__ int s_nact;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const int lo = P.own_first[P.inst_patch_off[i]], hi = P.own_first[P.inst_patch_off[i + 1]];
    const bool act = init || P.isc[i].done == 0;
    s_lo[i] = lo;
    s_cnt[i] = act ? hi - lo : 0;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    int a = 0, off = 0;
    s_off[0] = 0;
    for (int i = 0; i < n; ++i)
      if (s_cnt[i] > 0) {
        s_ids[a] = i;
        off += s_cnt[i];
        s_off[++a] = off;
      }
    s_nact = a;
  }
  __syncthreads();
  const int nact = s_nact, total = s_off[nact];
  const int chunk = (total + (int)gridDim.x - 1) / (int)gridDim.x;
  // index of the active range holding position j (0 <= j < total)
  auto range_of = [&](int j) {
    int lo = 0, hi = nact - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (s_off[mid] <= j) lo = mid; else hi = mid - 1;
    }
    return lo;
  };
  int beg = (int)blockIdx.x * chunk;
  const int end = min(beg + chunk, total);
  int a = beg < end ? range_of(beg) : 0;
  for (int sg = 0; beg < end; ++sg, ++a) {
    const int inst = s_ids[a];
    const int seg_end = min(end, s_off[a + 1]);
    const int base = s_lo[inst] - s_off[a];  // node = base + position
    const T alpha = init ? T(0) : (T)P.isc[inst].alpha;
    DotAcc<T> acc[3];
    for (int j0 = beg + threadIdx.x; j0 < seg_end; j0 += blockDim.x * U) {
      NodeV<T, VW> di[U], rv[U], xx[U], pv[U], uv[U];
#pragma unroll
      for (int k = 0; k < U; ++k) {
        const int j = j0 + k * blockDim.x;
        if (j >= seg_end) continue;
        const int64_t nd = base + j;
        di[k] = ldv<T, VW>(dinv, nd);
        if (init) {
          rv[k] = ldv<T, VW>(f, nd);
        } else {
          rv[k] = ldv<T, VW>(r, nd);
          xx[k] = ldv<T, VW>(x, nd);
          pv[k] = ldv<T, VW>(p, nd);
          uv[k] = ldv<T, VW>(u, nd);
        }
      }
#pragma unroll
      for (int k = 0; k < U; ++k) {
        const int j = j0 + k * blockDim.x;
        if (j >= seg_end) continue;
        const int64_t nd = base + j;
        NodeV<T, VW> zero, zz;
#pragma unroll
        for (int d = 0; d < VW; ++d) zero.v[d] = zz.v[d] = 0;
        if (init) {
          xx[k] = zero;
        } else {
#pragma unroll
          for (int d = 0; d < DIM; ++d) {
            xx[k].v[d] += alpha * pv[k].v[d];
            rv[k].v[d] -= alpha * uv[k].v[d];
          }
        }
        T rz = 0, rr = 0;
#pragma unroll
        for (int d = 0; d < DIM; ++d) {
          zz.v[d] = rv[k].v[d] * di[k].v[d];
          rz += rv[k].v[d] * zz.v[d];
          rr += rv[k].v[d] * rv[k].v[d];
        }
        acc[0].add(rz);
        acc[1].add(rr);
        if (init) acc[2].add(rr);
        stv<T, VW>(x, nd, xx[k]);
        stv<T, VW>(r, nd, rv[k]);
        stv<T, VW>(z, nd, zz);
        stv<T, VW>(u, nd, zero);
      }
    }
    const double t0 = block_total<T>(acc[0]), t1 = block_total<T>(acc[1]), t2 = block_total<T>(acc[2]);
    if (threadIdx.x == 0) {
      double *o = P.seg + ((size_t)blockIdx.x * n + sg) * 3;
      o[0] = t0;
      o[1] = t1;
      o[2] = t2;
    }
    beg = seg_end;
  }
  __shared__ bool last;
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) last = atomicAdd(&P.ctl->count_up, 1u) == gridDim.x - 1;
  __syncthreads();
  if (!last) return;
  __threadfence();
  // per active range a: the CTAs c_lo .. c_hi cover it; its segment is number
  // a - range_of(c_lo * chunk) in CTA c_lo and number 0 in the others
  {
    const int lane = threadIdx.x & 31, nwarp = blockDim.x >> 5;
    for (int aa = threadIdx.x >> 5; aa < nact; aa += nwarp) {
      const int c_lo = s_off[aa] / chunk, c_hi = (s_off[aa + 1] - 1) / chunk;
      const int sg_lo = aa - range_of(c_lo * chunk);
      double t[3] = {0, 0, 0};
      for (int c = c_lo + lane; c <= c_hi; c += 32) {
        const double *o = P.seg + ((size_t)c * n + (c == c_lo ? sg_lo : 0)) * 3;
#pragma unroll
        for (int q = 0; q < 3; ++q) t[q] += __ldcg(o + q);
      }
#pragma unroll
      for (int q = 0; q < 3; ++q)
        for (int o = 16; o > 0; o >>= 1) t[q] += __shfl_down_sync(0xffffffffu, t[q], o);
      if (lane == 0) {
        double *sc = P.scratch + (size_t)s_ids[aa] * 3;
        sc[0] = t[0];
        sc[1] = t[1];
        sc[2] = t[2];
      }
    }
  }
  __syncthreads();
  __shared__ int s_active;
  if (threadIdx.x == 0) s_active = 0;
  __syncthreads();
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    Scalars &m = P.isc[i];
    const bool took_part = s_cnt[i] > 0;
    const double a0 = took_part ? P.scratch[i * 3] : 0.0, b = took_part ? P.scratch[i * 3 + 1] : 0.0,
                 e = took_part ? P.scratch[i * 3 + 2] : 0.0;
    if (init) {
      m.gamma0 = m.gamma = m.gamma_prev = a0;
      m.rr = b;
      m.ff = e;
      m.iter = 0;
      m.sigma = m.alpha = m.beta = 0;
      m.done = 0;
      if (i >= P.k_active || a0 == 0.0) m.done = 1;
      else if (m.rule == 1 && sqrt(b) <= m.tol * sqrt(e)) m.done = 1;
      else if (!isfinite(a0)) m.done = 2;
    } else if (!m.done) {
      m.gamma_prev = m.gamma;
      m.gamma = a0;
      m.beta = a0 / m.gamma_prev;
      m.rr = b;
      m.iter += 1;
      if (!isfinite(a0) || !isfinite(m.alpha)) m.done = 2;
      else if (m.rule == 0 && a0 < m.tol * m.gamma0) m.done = 1;
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
