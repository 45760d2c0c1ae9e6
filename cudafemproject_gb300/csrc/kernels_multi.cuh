// Multi-right-hand-side EbE PCG: k load cases on one mesh (3D, edge-fan form).
//
// Node vectors hold all K cases of a node contiguously: [node][K][4] (K >= k,
// a power of two <= kMaxCases; unused cases stay zero). The matvec loads each
// patch block (kernels_fan_tma.cuh) once and applies it to the K cases in
// passes of R: every half-fan thread evaluates its tets for R cases at once,
// so each gradient read from shared memory serves R cases. Every case has its
// own PCG scalars and stopping test; a converged case is frozen (its passes
// are skipped once all R cases of a pass are done).
#pragma once

#include "kernels.cuh"
#include "kernels_fan_tma.cuh"

namespace cfem {

constexpr int kMaxCases = 256;

struct MultiScalars {  // per case
  double gamma, gamma_prev, gamma0, sigma, alpha, beta, rr, ff;
  int done, iters;  // done: 0 running, 1 converged, 2 diverged, 3 iteration cap
};

struct MultiCtl {  // shared by the cases of one solve
  double tol;
  int rule, maxit, iter, all_done;
  int k_active;     // cases 0..k_active-1 are real, the rest are padding
  unsigned int count_mv, count_up;
};

template <typename T>
struct MultiParams {
  int n_patches;
  const int32_t *node_off, *own;
  const T *diagA;       // [node][4] diagonal of the operator (constrained DOFs)
  T lam, mu;
  int K;                // cases per node (power of two)
  int64_t n_nodes;
  MultiScalars *sc;     // [K]
  MultiCtl *ctl;
  double *partials;     // [grid][K] (matvec) / [grid][K][3] (vector kernels)
  FanTmaParams F;       // patch blocks (layout and fan offsets)
};

// Shared memory of k_matvec_multi: one patch block, R force lists, R staged node blocks.
inline size_t multi_smem_bytes(const FanBlockLayout &L, int R) {
  const int fs_bytes = kFanForces * kFanThreads * 4 * (int)sizeof(float);
  return (size_t)L.bytes + (size_t)R * fs_bytes + (size_t)R * L.npn * 4 * sizeof(float) + 16 +
         (size_t)kMaxCases * sizeof(double) + 64;
}

// Last-block helper: per case c < K the sums over the grid's blocks b of
// partials[(b * K + c) * NQ + k], in a fixed order, into out[c * NQ + k].
// Many cases: one thread per case with eight interleaved partial sums, so that
// its loads overlap. Few cases: one warp per case, four interleaved partial
// sums per lane and a shuffle tree. Called by all threads of the last block.
template <int NQ>
__device__ __forceinline__ void case_sums(const double *partials, int nblocks, int K, double *out) {
  if (K >= 128) {
    for (int c = threadIdx.x; c < K; c += blockDim.x) {
#pragma unroll
      for (int k = 0; k < NQ; ++k) {
        double s8[8] = {0, 0, 0, 0, 0, 0, 0, 0};
        int b = 0;
        for (; b + 8 <= nblocks; b += 8)
#pragma unroll
          for (int q = 0; q < 8; ++q) s8[q] += __ldcg(partials + ((size_t)(b + q) * K + c) * NQ + k);
#pragma unroll
        for (int q = 0; q < 7; ++q)
          if (b + q < nblocks) s8[q] += __ldcg(partials + ((size_t)(b + q) * K + c) * NQ + k);
        out[c * NQ + k] = ((s8[0] + s8[1]) + (s8[2] + s8[3])) + ((s8[4] + s8[5]) + (s8[6] + s8[7]));
      }
    }
    return;
  }
  const int lane = threadIdx.x & 31, nwarp = blockDim.x >> 5;
  for (int c = threadIdx.x >> 5; c < K; c += nwarp) {
#pragma unroll
    for (int k = 0; k < NQ; ++k) {
      double s4[4] = {0, 0, 0, 0};
      int b = lane;
      for (; b + 96 < nblocks; b += 128)
#pragma unroll
        for (int q = 0; q < 4; ++q) s4[q] += __ldcg(partials + ((size_t)(b + 32 * q) * K + c) * NQ + k);
#pragma unroll
      for (int q = 0; q < 3; ++q)
        if (b + 32 * q < nblocks) s4[q] += __ldcg(partials + ((size_t)(b + 32 * q) * K + c) * NQ + k);
      double t = (s4[0] + s4[1]) + (s4[2] + s4[3]);
      for (int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
      if (lane == 0) out[c * NQ + k] = t;
    }
  }
}

// y_c += K' p_c for the K cases. PCG (MODE MV_PCG): p_c = z_c + beta_c p_old_c
// staged on the fly (written back by the owning patch), sigma_c = p_c.K'p_c.
// PLAIN: y_c += K' x_c. FP32 only (the patch blocks hold FP32 gradients).
template <int MODE, int R>
__global__ void __launch_bounds__(kHfanThreads) k_matvec_multi(MultiParams<float> P, const float *x, const float *pold,
                                                               float *pnew, float *y) {
  using T = float;
  constexpr int DIM = 3, VW = 4;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  const FanBlockLayout &L = P.F.L;
  const int K = P.K;
  unsigned char *B = smem_raw;
  // case-fastest layouts: the R cases of one node (or force slot) are adjacent
  T *fs = reinterpret_cast<T *>(smem_raw + L.bytes);                            // [kFanForces * kFanThreads][R][4]
  constexpr int FS = kFanForces * kFanThreads * VW;
  T *sp = fs + (size_t)R * FS;                                                  // [npn][R][4]
  uint64_t *bar = reinterpret_cast<uint64_t *>(sp + (size_t)R * L.npn * VW);
  double *s_en = reinterpret_cast<double *>(bar + 2);                           // [K] energies of this block
  if (MODE == MV_PCG && P.ctl->all_done) return;
  for (int c = threadIdx.x; c < K; c += blockDim.x) s_en[c] = 0;
  if (threadIdx.x == 0) {
    mbar_init(&bar[0], 1);
    fence_mbar_init();
  }
  __syncthreads();
  const uint16_t *fstart = reinterpret_cast<const uint16_t *>(B + L.fstart_off);
  const int32_t *nodes = reinterpret_cast<const int32_t *>(B + L.nodes_off);
  const uint8_t *bits = B + L.bits_off;
  int it = 0;
  for (int patch = blockIdx.x; patch < P.n_patches; patch += gridDim.x, ++it) {
    fence_proxy_async();  // earlier reads of the block precede the copy that overwrites it
    __syncthreads();
    if (threadIdx.x == 0) {
      mbar_expect_tx(&bar[0], (unsigned)L.bytes);
      bulk_load(B, P.F.blocks + (size_t)patch * L.bytes, (unsigned)L.bytes, &bar[0]);
    }
    const bool ok = mbar_wait_bounded(&bar[0], (unsigned)(it & 1));
    if (__syncthreads_or(!ok)) {
      if (threadIdx.x == 0) atomicOr(P.F.err, kErrTmaTimeout);
      return;
    }
    const int32_t *hdr = reinterpret_cast<const int32_t *>(B + L.hdr_off);
    const int nn = hdr[0], own = hdr[1];
    const int h = threadIdx.x & 1;
    int slot[6];
    const int nk = load_half_slots(B + L.slot_off, threadIdx.x, slot);
    for (int c0 = 0; c0 < K; c0 += R) {
      if (MODE == MV_PCG) {
        // every thread evaluates the pass's cases itself; the barrier's AND
        // makes the decision uniform without a shared flag
        int all = 1;
#pragma unroll
        for (int r = 0; r < R; ++r) all &= P.sc[c0 + r].done != 0;
        if (__syncthreads_and(all)) continue;
      }
      // 1. stage: items (node i, case r), case fastest
      for (int q = threadIdx.x; q < nn * R; q += kHfanThreads) {
        const int i = q / R, r = q - i * R, c = c0 + r;
        const int g = nodes[i];
        const int64_t idx = (int64_t)g * K + c;
        NodeV<T, VW> v = ldv<T, VW>(x, idx);
        if (MODE == MV_PCG) {
          const MultiScalars &s = P.sc[c];
          if (!s.done && s.beta != 0.0) {
            const T beta = (T)s.beta;
            const NodeV<T, VW> po = ldv<T, VW>(pold, idx);
#pragma unroll
            for (int d = 0; d < DIM; ++d) v.v[d] += beta * po.v[d];
          }
          if (i >= own) stv<T, VW>(pnew, idx, v);
        }
        const unsigned bb = bits[i];
        NodeV<T, VW> m;
#pragma unroll
        for (int d = 0; d < VW; ++d) m.v[d] = (d < DIM && !(bb >> d & 1u)) ? v.v[d] : T(0);
        stv<T, VW>(sp, (int64_t)i * R + r, m);
      }
      __syncthreads();
      // 2. half-fans, R cases per thread
      T fv[R][6][DIM];
      T e_fan[R];
      {
        T uv[R][6][DIM];
#pragma unroll
        for (int k = 0; k < 6; ++k) {
          const int li = k < nk ? slot[k] : 0;
#pragma unroll
          for (int r = 0; r < R; ++r) {
            NodeV<T, VW> s;
#pragma unroll
            for (int d = 0; d < VW; ++d) s.v[d] = 0;
            if (k < nk) s = ldv<T, VW>(sp, (int64_t)li * R + r);
#pragma unroll
            for (int d = 0; d < DIM; ++d) {
              uv[r][k][d] = s.v[d];
              fv[r][k][d] = 0;
            }
          }
        }
#pragma unroll
        for (int r = 0; r < R; ++r) e_fan[r] = 0;
#pragma unroll
        for (int jj = 0; jj < 3; ++jj) {
          if (jj + 3 < nk) {
            T G[9];
            load_tet_G(B + L.g_off, threadIdx.x, jj, G);
#pragma unroll
            for (int r = 0; r < R; ++r) {
              T u[4][DIM], fe[4][DIM];
#pragma unroll
              for (int d = 0; d < DIM; ++d) {
                u[0][d] = uv[r][0][d];
                u[1][d] = uv[r][1][d];
                u[2][d] = uv[r][2 + jj][d];
                u[3][d] = uv[r][3 + jj][d];
              }
              element_force<T, DIM>(u, G, P.lam, P.mu, T(1), T(0), fe);
#pragma unroll
              for (int d = 0; d < DIM; ++d) {
                if (MODE == MV_PCG)
                  e_fan[r] += u[0][d] * fe[0][d] + u[1][d] * fe[1][d] + u[2][d] * fe[2][d] + u[3][d] * fe[3][d];
                fv[r][0][d] += fe[0][d];
                fv[r][1][d] += fe[1][d];
                fv[r][2 + jj][d] += fe[2][d];
                fv[r][3 + jj][d] += fe[3][d];
              }
            }
          }
        }
      }
#pragma unroll
      for (int r = 0; r < R; ++r) combine_half_forces<T, DIM>(fv[r], h);
#pragma unroll
      for (int r = 0; r < R; ++r)
#pragma unroll
        for (int k = 0; k < 6; ++k)
          if (k < nk && half_writes(h, k)) {
            NodeV<T, VW> o;
#pragma unroll
            for (int d = 0; d < VW; ++d) o.v[d] = d < DIM ? fv[r][k][d] : T(0);
            stv<T, VW>(fs, (int64_t)half_fpos(B + L.fpos_off, threadIdx.x, k) * R + r, o);
          }
      __syncthreads();
      // 3. node sums: items (node i, case r)
      DotAcc<T> e_diag[R];
      for (int q = threadIdx.x; q < nn * R; q += kHfanThreads) {
        const int i = q / R, r = q - i * R, c = c0 + r;
        const int g = nodes[i];
        const unsigned bb = bits[i];
        T acc[DIM] = {0, 0, 0};
        const int k1 = fstart[i + 1];
        for (int k = fstart[i]; k < k1; ++k) {
          const NodeV<T, VW> fo = ldv<T, VW>(fs, (int64_t)k * R + r);
#pragma unroll
          for (int d = 0; d < DIM; ++d) acc[d] += fo.v[d];
        }
        NodeV<T, VW> out;
        bool any = false;
#pragma unroll
        for (int d = 0; d < VW; ++d) {
          T val = (d < DIM && !(bb >> d & 1u)) ? acc[d < DIM ? d : 0] : T(0);
          out.v[d] = val;
          any |= val != T(0);
        }
        const int64_t idx = (int64_t)g * K + c;
        if (bb && i >= own) {
          NodeV<T, VW> v = ldv<T, VW>(MODE == MV_PCG ? pnew : x, idx);  // this block wrote pnew[idx] while staging
          NodeV<T, VW> dg = ldv<T, VW>(P.diagA, g);
#pragma unroll
          for (int d = 0; d < DIM; ++d)
            if (bb >> d & 1u) {
              T t = dg.v[d] * v.v[d];
              out.v[d] = t;
              any |= t != T(0);
              if (MODE == MV_PCG) {
#pragma unroll
                for (int rr = 0; rr < R; ++rr)
                  if (rr == r) e_diag[rr].add(t * v.v[d]);
              }
            }
        }
        if (any) atomic_addv<T, VW>(y, idx, out, DIM);
      }
      // per-case energies of this pass, summed over the block in a fixed order
      if (MODE == MV_PCG) {
        __shared__ double s_red[R][kHfanThreads / 32];
        const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
        for (int r = 0; r < R; ++r) {
          Comp32 cm;
          cm.add(e_fan[r]);
          cm.merge(e_diag[r].c.hi, e_diag[r].c.lo);
          for (int o = 16; o > 0; o >>= 1) {
            const float h2 = __shfl_down_sync(0xffffffffu, cm.hi, o), l2 = __shfl_down_sync(0xffffffffu, cm.lo, o);
            cm.merge(h2, l2);
          }
          if (lane == 0) s_red[r][wid] = (double)cm.hi + (double)cm.lo;
        }
        __syncthreads();
        if (threadIdx.x < R) {
          double t = 0;
          for (int w = 0; w < kHfanThreads / 32; ++w) t += s_red[threadIdx.x][w];
          s_en[c0 + threadIdx.x] += t;
        }
      }
      __syncthreads();  // sp / fs of this pass are free again
    }
  }
  if (MODE != MV_PCG) return;
  // per-case grid sums: the last block adds the block partials in block order
  for (int c = threadIdx.x; c < K; c += blockDim.x) P.partials[(size_t)blockIdx.x * K + c] = s_en[c];
  __shared__ bool last;
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) last = atomicAdd(&P.ctl->count_mv, 1u) == gridDim.x - 1;
  __syncthreads();
  if (!last) return;
  __threadfence();
  __shared__ double s_tot[kMaxCases];
  case_sums<1>(P.partials, gridDim.x, K, s_tot);
  __syncthreads();
  for (int c = threadIdx.x; c < K; c += blockDim.x) {
    const double t = s_tot[c];
    MultiScalars &s = P.sc[c];
    s.sigma = t;
    s.alpha = s.done ? 0.0 : s.gamma / t;
  }
  if (threadIdx.x == 0) P.ctl->count_mv = 0;
}

// Per case: init (r = f, x = 0) or update (x += alpha p, r -= alpha u),
// z = M^-1 r, u = 0, gamma = r.z, ||r||^2, per-case stopping tests. Items are
// (node, case) with the case fastest; the grid stride is a multiple of K, so
// a thread always works on the same case.
template <typename T>
__global__ void __launch_bounds__(kThreads) k_pcg_multi_vec(MultiParams<T> P, T *xv, T *r, T *z, const T *p, T *u,
                                                           const T *f, const T *dinv, int init) {
  constexpr int DIM = 3, VW = 4;
  if (!init && P.ctl->all_done) return;
  const int K = P.K;
  const int c = threadIdx.x & (K - 1);
  const MultiScalars &s = P.sc[c];
  const bool frozen = !init && s.done;
  const T alpha = init || frozen ? T(0) : (T)s.alpha;
  DotAcc<T> acc[3];  // r.z, r.r, f.f
  const int64_t n_items = P.n_nodes * K;
  // U items per thread per round, all loads issued before any is used; the
  // stride is a multiple of K, so every item of a thread is case c
  constexpr int U = 4;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t q0 = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q0 < n_items; q0 += stride * U) {
    NodeV<T, VW> zero;
#pragma unroll
    for (int d = 0; d < VW; ++d) zero.v[d] = 0;
    if (frozen) {
#pragma unroll
      for (int k = 0; k < U; ++k)
        if (q0 + k * stride < n_items) stv<T, VW>(u, q0 + k * stride, zero);
      continue;
    }
    NodeV<T, VW> di[U], rv[U], xx[U], pp[U], uu[U];
#pragma unroll
    for (int k = 0; k < U; ++k) {
      const int64_t q = q0 + k * stride;
      if (q >= n_items) continue;
      di[k] = ldv<T, VW>(dinv, q / K);
      if (init) {
        rv[k] = ldv<T, VW>(f, q);
      } else {
        rv[k] = ldv<T, VW>(r, q);
        xx[k] = ldv<T, VW>(xv, q);
        pp[k] = ldv<T, VW>(p, q);
        uu[k] = ldv<T, VW>(u, q);
      }
    }
#pragma unroll
    for (int k = 0; k < U; ++k) {
      const int64_t q = q0 + k * stride;
      if (q >= n_items) continue;
      NodeV<T, VW> zz = zero;
      if (init) {
        xx[k] = zero;
      } else {
#pragma unroll
        for (int d = 0; d < DIM; ++d) {
          xx[k].v[d] += alpha * pp[k].v[d];
          rv[k].v[d] -= alpha * uu[k].v[d];
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
      stv<T, VW>(xv, q, xx[k]);
      stv<T, VW>(r, q, rv[k]);
      stv<T, VW>(z, q, zz);
      stv<T, VW>(u, q, zero);
    }
  }
  // block partials per case: threads c, c + K, ... in order
  __shared__ double red[3][kThreads];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    if constexpr (sizeof(T) == 4) red[k][threadIdx.x] = (double)acc[k].c.hi + (double)acc[k].c.lo;
    else red[k][threadIdx.x] = acc[k].s;
  }
  __syncthreads();
  for (int cc = threadIdx.x; cc < K; cc += blockDim.x) {
    double a = 0, b = 0, e = 0;
    for (int t = cc; t < (int)blockDim.x; t += K) { a += red[0][t]; b += red[1][t]; e += red[2][t]; }
    double *pt = P.partials + ((size_t)blockIdx.x * K + cc) * 3;
    pt[0] = a; pt[1] = b; pt[2] = e;
  }
  __shared__ bool last;
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) last = atomicAdd(&P.ctl->count_up, 1u) == gridDim.x - 1;
  __syncthreads();
  if (!last) return;
  __threadfence();
  __shared__ int s_active;
  if (threadIdx.x == 0) s_active = 0;
  __syncthreads();
  double *s_tot = &red[0][0];  // [K][3] (K <= kThreads)
  case_sums<3>(P.partials, gridDim.x, K, s_tot);
  __syncthreads();
  for (int cc = threadIdx.x; cc < K; cc += blockDim.x) {
    const double a = s_tot[cc * 3], b = s_tot[cc * 3 + 1], e = s_tot[cc * 3 + 2];
    MultiScalars &m = P.sc[cc];
    if (init) {
      m.gamma0 = m.gamma = m.gamma_prev = a;
      m.rr = b;
      m.ff = e;
      m.iters = 0;
      m.sigma = m.alpha = m.beta = 0;
      m.done = 0;
      if (cc >= P.ctl->k_active || a == 0.0) m.done = 1;
      else if (P.ctl->rule == 1 && sqrt(b) <= P.ctl->tol * sqrt(e)) m.done = 1;
      else if (!isfinite(a)) m.done = 2;
    } else if (!m.done) {
      m.gamma_prev = m.gamma;
      m.gamma = a;
      m.beta = a / m.gamma_prev;
      m.rr = b;
      m.iters += 1;
      if (!isfinite(a) || !isfinite(m.alpha)) m.done = 2;
      else if (P.ctl->rule == 0 && a < P.ctl->tol * m.gamma0) m.done = 1;
      else if (P.ctl->rule == 1 && sqrt(b) <= P.ctl->tol * sqrt(m.ff)) m.done = 1;
      else if (m.iters >= P.ctl->maxit) m.done = 3;
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

// caller order F[c][n_dof] (FP64) -> dst[node][K][4] (T), scaled; cases >= k zero
template <typename T>
__global__ void k_multi_to_internal(int64_t nn, int K, int k, int64_t nd, const double *F, const int32_t *new2old,
                                    T *dst) {
  int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (q >= nn * K) return;
  const int64_t n = q / K;
  const int c = (int)(q - n * K);
  const int64_t o = new2old[n];
  NodeV<T, 4> v;
#pragma unroll
  for (int d = 0; d < 4; ++d) v.v[d] = (c < k && d < 3) ? (T)F[(size_t)c * nd + o * 3 + d] : T(0);
  stv<T, 4>(dst, q, v);
}

template <typename T>
__global__ void k_multi_to_caller(int64_t nn, int K, int k, int64_t nd, const T *src, const int32_t *new2old,
                                  double *U) {
  int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (q >= nn * K) return;
  const int64_t n = q / K;
  const int c = (int)(q - n * K);
  if (c >= k) return;
  const int64_t o = new2old[n];
  const NodeV<T, 4> v = ldv<T, 4>(src, q);
#pragma unroll
  for (int d = 0; d < 3; ++d) U[(size_t)c * nd + o * 3 + d] = (double)v.v[d];
}

// one case of a [node][K][4] array <-> a [node][4] array
template <typename TA, typename TB>
__global__ void k_case_copy(int64_t nn, int K, int c, const TA *src, TB *dst, int to_single) {
  int64_t n = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (n >= nn) return;
  const int64_t a = to_single ? n * K + c : n, b = to_single ? n : n * K + c;
  const NodeV<TA, 4> v = ldv<TA, 4>(src, a);
  NodeV<TB, 4> w;
#pragma unroll
  for (int d = 0; d < 4; ++d) w.v[d] = (TB)v.v[d];
  stv<TB, 4>(dst, b, w);
}

// x64 += d32 over whole multi arrays
static __global__ void k_multi_accumulate(int64_t n, const float *d, double *x) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) x[i] += (double)d[i];
}

}  // namespace cfem
