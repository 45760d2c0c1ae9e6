// Multi-right-hand-side EbE PCG: k load cases on one mesh (3D, edge-fan form).
//
// Node vectors hold all K cases of a node contiguously: [node][K][4] (K >= k,
// a power of two <= kMaxCases; unused cases stay zero). The matvec works on
// items (patch, chunk of C cases): the lanes of a warp hold C cases of 32 / C
// half-fans, so a node's values for the chunk are one contiguous C x 16-byte
// load, every gradient read from the patch block (kernels_fan_tma.cuh) is a
// broadcast serving C cases, and the forces go to the block's node-sorted
// force list ([entry][3][C]), whose runs the node sums add up without atomics. Every case has
// its own PCG scalars and stopping test; a converged case is frozen (its items
// are skipped once all C cases of a chunk are done).
#pragma once

#include "kernels.cuh"
#include "kernels_fan_tma.cuh"

namespace cfem {

constexpr int kMaxCases = 256;
constexpr int kSumGroup = 16;  // blocks per group of the first level of the per-case grid sums

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
  double *gpart;        // [grid / kSumGroup][K][3] group sums of the partials
  unsigned *gcnt_mv, *gcnt_up;  // [grid / kSumGroup] group tickets of the matvec / vector kernel
  FanTmaParams F;       // patch blocks (layout and fan offsets)
};

// Shared memory of k_matvec_multi<MODE, C> for K cases: the patch block, the
// staged node values [npn][C][4], per-case energies [K] and warp partials
// [8][C] (double), the mbarrier, the force list [kFanForces x kFanThreads][3][C],
// per-case beta and done flags [K].
struct MultiSmem {
  int sp, en, red, bar, fs, beta, done, bytes;
};
__host__ __device__ inline MultiSmem multi_smem(const FanBlockLayout &L, int C, int K) {
  MultiSmem m{};
  int off = L.bytes;
  m.sp = off; off += L.npn * C * 16;
  m.en = off; off += K * 8;
  m.red = off; off += (kHfanThreads / 32) * C * 8;
  m.bar = off; off += 16;
  m.fs = off; off += kFanForces * kFanThreads * 3 * C * 4;
  m.beta = off; off += K * 4;
  m.done = off; off += K * 4;
  m.bytes = off;
  return m;
}

// Per-case grid sums in two fixed-order levels. Every block calls it (all
// threads) once its partials part[(b * K + c) * NQ + k] are written. The last
// block of each group of kSumGroup blocks adds the group's partials in block
// order into gpart[(g * K + c) * NQ + k]; the last of those group finishers
// adds the groups in group order into out[c * NQ + k] (shared memory) and
// returns true there, false everywhere else (uniform per block). Each level
// is one round of independent loads per sum instead of a chain over all blocks.
// The tickets return to zero for the next launch.
template <int NQ>
__device__ __forceinline__ bool tree_case_sums(const double *part, double *gpart, unsigned *gcnt, unsigned *top, int K,
                                               double *out) {
  __shared__ bool s_last;
  const int n = K * NQ;
  const int g = blockIdx.x / kSumGroup, ng = (gridDim.x + kSumGroup - 1) / kSumGroup;
  const int b0 = g * kSumGroup, nb = min(kSumGroup, (int)gridDim.x - b0);
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) s_last = atomicAdd(&gcnt[g], 1u) == (unsigned)(nb - 1);
  __syncthreads();
  if (!s_last) return false;
  __threadfence();
  for (int j = threadIdx.x; j < n; j += blockDim.x) {
    double v[kSumGroup];
#pragma unroll
    for (int q = 0; q < kSumGroup; ++q) v[q] = q < nb ? __ldcg(part + (size_t)(b0 + q) * n + j) : 0.0;
    double t = 0;
#pragma unroll
    for (int q = 0; q < kSumGroup; ++q) t += v[q];
    gpart[(size_t)g * n + j] = t;
  }
  if (threadIdx.x == 0) gcnt[g] = 0;
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) s_last = atomicAdd(top, 1u) == (unsigned)(ng - 1);
  __syncthreads();
  if (!s_last) return false;
  __threadfence();
  for (int j = threadIdx.x; j < n; j += blockDim.x) {
    double t = 0;
    for (int g0 = 0; g0 < ng; g0 += kSumGroup) {
      double v[kSumGroup];
#pragma unroll
      for (int q = 0; q < kSumGroup; ++q) v[q] = g0 + q < ng ? __ldcg(gpart + (size_t)(g0 + q) * n + j) : 0.0;
#pragma unroll
      for (int q = 0; q < kSumGroup; ++q) t += v[q];
    }
    out[j] = t;
  }
  if (threadIdx.x == 0) *top = 0;
  __syncthreads();
  return true;
}

// y_c += K' p_c for the K cases. PCG (MODE MV_PCG): p_c = z_c + beta_c p_old_c
// staged on the fly (written back by the owning patch), sigma_c = p_c.K'p_c.
// PLAIN: y_c += K' x_c. FP32 only (the patch blocks hold FP32 gradients).
//
// Items q = patch * (K / C) + chunk; CTA b takes the contiguous items
// [n b / G, n (b + 1) / G), so the chunks of a patch reuse its block. Lane l of
// warp w holds case l % C of half-fan (round * 8 + w) * (32 / C) + l / C: the
// two halves of a fan are lanes l and l ^ C. A thread's case (l % C) is the
// same in every phase, so its energy partial needs no exchange until the end
// of the item.
template <int MODE, int C>
__global__ void __launch_bounds__(kHfanThreads, C <= 2 ? 3 : 2) k_matvec_multi(MultiParams<float> P, const float *x,
                                                                  const float *pold, float *pnew, float *y) {
  using T = float;
  constexpr int DIM = 3, VW = 4, NW = kHfanThreads / 32;
  constexpr int HPW = 32 / C;                    // half-fans per warp and round
  constexpr int ROUNDS = kHfanThreads / (NW * HPW);
  constexpr int SU = C <= 2 ? 2 : 4;             // staging items in flight per thread
  static_assert(C == 2 || C == 4 || C == 8, "C: 2, 4 or 8 cases per item");
  extern __shared__ __align__(128) unsigned char smem_raw[];
  const FanBlockLayout &L = P.F.L;
  const int K = P.K, NC = K / C;
  const MultiSmem S = multi_smem(L, C, K);
  unsigned char *B = smem_raw;
  T *sp = reinterpret_cast<T *>(smem_raw + S.sp);
  double *s_en = reinterpret_cast<double *>(smem_raw + S.en);
  double *s_red = reinterpret_cast<double *>(smem_raw + S.red);
  uint64_t *bar = reinterpret_cast<uint64_t *>(smem_raw + S.bar);
  T *fs = reinterpret_cast<T *>(smem_raw + S.fs);
  T *s_beta = reinterpret_cast<T *>(smem_raw + S.beta);
  int *s_done = reinterpret_cast<int *>(smem_raw + S.done);
  if (MODE == MV_PCG) {  // (thread 0 reads the shared flag, see k_pcg_multi_vec)
    if (threadIdx.x == 0) s_done[0] = P.ctl->all_done;
    __syncthreads();
    const bool all = s_done[0] != 0;
    __syncthreads();
    if (all) return;
  }
  for (int c = threadIdx.x; c < K; c += blockDim.x) {
    s_en[c] = 0;
    s_done[c] = 0;
    s_beta[c] = 0;
    if (MODE == MV_PCG) {
      const MultiScalars &sc = P.sc[c];
      s_done[c] = sc.done;
      s_beta[c] = sc.done ? T(0) : (T)sc.beta;
    }
  }
  if (threadIdx.x == 0) {
    mbar_init(&bar[0], 1);
    fence_mbar_init();
  }
  __syncthreads();
  const uint16_t *fstart = reinterpret_cast<const uint16_t *>(B + L.fstart_off);
  const int32_t *nodes = reinterpret_cast<const int32_t *>(B + L.nodes_off);
  const uint8_t *bits = B + L.bits_off;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int cl = lane & (C - 1), hs = lane / C, h = hs & 1;
  const T lam = P.lam, mu = P.mu;
  const int64_t n_items = (int64_t)P.n_patches * NC;
  const int64_t q0 = n_items * blockIdx.x / gridDim.x, q1 = n_items * (blockIdx.x + 1) / gridDim.x;
  int cur = -1;
  unsigned nload = 0;
  for (int64_t q = q0; q < q1; ++q) {
    const int patch = (int)(q / NC), c0 = (int)(q - (int64_t)patch * NC) * C;
    if (MODE == MV_PCG) {
      bool all = true;  // (uniform: read from shared memory)
#pragma unroll
      for (int r = 0; r < C; ++r) all &= s_done[c0 + r] != 0;
      if (all) continue;
    }
    if (patch != cur) {
      fence_proxy_async();  // earlier reads of the block precede the copy that overwrites it
      __syncthreads();
      if (threadIdx.x == 0) {
        mbar_expect_tx(&bar[0], (unsigned)L.bytes);
        bulk_load(B, P.F.blocks + (size_t)patch * L.bytes, (unsigned)L.bytes, &bar[0]);
      }
      const bool ok = mbar_wait_bounded(&bar[0], nload & 1u);
      ++nload;
      if (__syncthreads_or(!ok)) {
        if (threadIdx.x == 0) atomicOr(P.F.err, kErrTmaTimeout);
        return;
      }
      cur = patch;
    }
    const int32_t *hdr = reinterpret_cast<const int32_t *>(B + L.hdr_off);
    const int nn = hdr[0], own = hdr[1];
    const int n_it = nn * C;  // staging / output items (node i, case cl): it = i * C + cl
    const T beta = MODE == MV_PCG ? s_beta[c0 + cl] : T(0);
    const bool case_done = MODE == MV_PCG && s_done[c0 + cl] != 0;
    // 1. stage the chunk's node values: C cases of a node are one contiguous load
    for (int i0 = threadIdx.x; i0 < n_it; i0 += SU * kHfanThreads) {
      NodeV<T, VW> v[SU], w[SU];
      int gi[SU];
#pragma unroll
      for (int u = 0; u < SU; ++u) {
        const int it = i0 + u * kHfanThreads;
        gi[u] = it < n_it ? nodes[it / C] : -1;
        if (gi[u] >= 0) {
          const int64_t idx = (int64_t)gi[u] * K + c0 + cl;
          v[u] = ldv<T, VW>(x, idx);
          if (MODE == MV_PCG && beta != T(0)) w[u] = ldv<T, VW>(pold, idx);
        }
      }
#pragma unroll
      for (int u = 0; u < SU; ++u) {
        if (gi[u] < 0) continue;
        const int it = i0 + u * kHfanThreads, i = it / C;
        if (MODE == MV_PCG) {
          if (beta != T(0)) {
#pragma unroll
            for (int d = 0; d < DIM; ++d) v[u].v[d] += beta * w[u].v[d];
          }
          // a stopped case keeps its last direction (a continued refinement
          // step starts from it); its lanes still compute, unused
          if (i >= own && !case_done) stv<T, VW>(pnew, (int64_t)gi[u] * K + c0 + cl, v[u]);
        }
        const unsigned bb = bits[i];
        NodeV<T, VW> m;
#pragma unroll
        for (int d = 0; d < VW; ++d) m.v[d] = (d < DIM && !(bb >> d & 1u)) ? v[u].v[d] : T(0);
        stv<T, VW>(sp, it, m);
      }
    }
    __syncthreads();
    // 2. half-fans: forces relative to P (missing tets have zero gradients),
    //    halves combined by shuffle, written to the force list
    Comp32 energy;
#pragma unroll 1
    for (int rd = 0; rd < ROUNDS; ++rd) {
      const int hf = (rd * NW + wid) * HPW + hs;
      int slot[6];
      const int nk = load_half_slots(B + L.slot_off, hf, slot);
      T du[6][DIM], fv[6][DIM];
#pragma unroll
      for (int k = 0; k < 6; ++k) {
        NodeV<T, VW> s;
#pragma unroll
        for (int d = 0; d < VW; ++d) s.v[d] = 0;
        if (k < nk) s = ldv<T, VW>(sp, slot[k] * C + cl);
#pragma unroll
        for (int d = 0; d < DIM; ++d) {
          du[k][d] = s.v[d];
          fv[k][d] = 0;
        }
      }
#pragma unroll
      for (int k = 1; k < 6; ++k)
#pragma unroll
        for (int d = 0; d < DIM; ++d) du[k][d] -= du[0][d];
#pragma unroll
      for (int jj = 0; jj < 3; ++jj) {
        T G[9];
        load_tet_G(B + L.g_off, hf, jj, G);
        tet_forces_acc<T>(du[1], du[2 + jj], du[3 + jj], G, lam, mu, fv[1], fv[2 + jj], fv[3 + jj]);
      }
#pragma unroll
      for (int d = 0; d < DIM; ++d) fv[0][d] = -(fv[1][d] + fv[2][d] + fv[3][d] + fv[4][d] + fv[5][d]);
      if (MODE == MV_PCG) {  // the forces sum to zero: sum_k u_k.f_k = sum_k>0 du_k.f_k
        T e = 0;
#pragma unroll
        for (int k = 1; k < 6; ++k)
#pragma unroll
          for (int d = 0; d < DIM; ++d) e += du[k][d] * fv[k][d];
        energy.add(e);
      }
      combine_half_forces<T, DIM, C>(fv, h);
#pragma unroll
      for (int k = 0; k < 6; ++k)
        if (k < nk && half_writes(h, k)) {
          T *o = fs + half_fpos(B + L.fpos_off, hf, k) * (3 * C) + cl;
#pragma unroll
          for (int d = 0; d < DIM; ++d) o[d * C] = fv[k][d];
        }
    }
    __syncthreads();
    // 3. node sums over contiguous force runs, constrained DOFs: (I - P) diag(A) p on owned nodes
    for (int it = threadIdx.x; it < n_it; it += kHfanThreads) {
      const int i = it / C;
      const unsigned bb = bits[i];
      T acc[DIM] = {0, 0, 0};
      const int k1 = fstart[i + 1];
      for (int k = fstart[i]; k < k1; ++k) {
        const T *f = fs + k * (3 * C) + cl;
#pragma unroll
        for (int d = 0; d < DIM; ++d) acc[d] += f[d * C];
      }
      NodeV<T, VW> out;
      bool any = false;
#pragma unroll
      for (int d = 0; d < DIM; ++d) {
        out.v[d] = (bb >> d & 1u) ? T(0) : acc[d];
        any |= out.v[d] != T(0);
      }
      out.v[3] = 0;
      const int g = nodes[i];
      const int64_t idx = (int64_t)g * K + c0 + cl;
      if (bb && i >= own) {
        const NodeV<T, VW> v = ldv<T, VW>(MODE == MV_PCG ? pnew : x, idx);  // this block wrote pnew[idx] while staging
        const NodeV<T, VW> dg = ldv<T, VW>(P.diagA, g);
#pragma unroll
        for (int d = 0; d < DIM; ++d)
          if (bb >> d & 1u) {
            const T t = dg.v[d] * v.v[d];
            out.v[d] = t;
            any |= t != T(0);
            if (MODE == MV_PCG) energy.add(t * v.v[d]);
          }
      }
      if (any) atomic_addv<T, VW>(y, idx, out, DIM);
    }
    if (MODE == MV_PCG) {  // per-case energy of the item: lanes of one case, then warps in order
#pragma unroll
      for (int o = C; o < 32; o <<= 1) {
        const float h2 = __shfl_xor_sync(0xffffffffu, energy.hi, o), l2 = __shfl_xor_sync(0xffffffffu, energy.lo, o);
        energy.merge(h2, l2);
      }
      if (lane < C) s_red[wid * C + lane] = (double)energy.hi + (double)energy.lo;
    }
    __syncthreads();  // sp, fs and s_red of this item are complete
    if (MODE == MV_PCG && threadIdx.x < C) {
      double t = 0;
#pragma unroll
      for (int w = 0; w < NW; ++w) t += s_red[w * C + threadIdx.x];
      s_en[c0 + threadIdx.x] += t;
    }
  }
  if (MODE != MV_PCG) return;
  // per-case grid sums (fixed-order tree), alpha_c = gamma_c / sigma_c in the last block
  __syncthreads();
  for (int c = threadIdx.x; c < K; c += blockDim.x) P.partials[(size_t)blockIdx.x * K + c] = s_en[c];
  __syncthreads();
  double *s_tot = s_en;  // (the block's own energies are in the partials now)
  if (!tree_case_sums<1>(P.partials, P.gpart, P.gcnt_mv, &P.ctl->count_mv, K, s_tot)) return;
  for (int c = threadIdx.x; c < K; c += blockDim.x) {
    const double t = s_tot[c];
    MultiScalars &s = P.sc[c];
    s.sigma = t;
    s.alpha = s.done ? 0.0 : s.gamma / t;
  }
}

// z_c += beta_c p_c for every (node, case) item, p_c read from pB when
// parity_c is 0, from pA when 1 (cases with beta_c = 0 are left alone): the
// first direction of a continued multi-RHS run.
static __global__ void k_multi_fold(int64_t n_items, int K, const float *beta, const int *parity, const float *pA,
                                    const float *pB, float *z) {
  const int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (q >= n_items) return;
  const int c = (int)(q % K);
  const float b = beta[c];
  if (b == 0.f) return;
  const NodeV<float, 4> p = ldv<float, 4>(parity[c] ? pA : pB, q);
  NodeV<float, 4> v = ldv<float, 4>(z, q);
#pragma unroll
  for (int d = 0; d < 3; ++d) v.v[d] += b * p.v[d];
  stv<float, 4>(z, q, v);
}

// Per case: init (r = f, x = 0) or update (x += alpha p, r -= alpha u),
// z = M^-1 r, u = 0, gamma = r.z, ||r||^2, per-case stopping tests. Items are
// (node, case) with the case fastest; the grid stride is a multiple of K, so
// a thread always works on the same case.
template <typename T>
__global__ void __launch_bounds__(kThreads) k_pcg_multi_vec(MultiParams<T> P, T *xv, T *r, T *z, const T *p, T *u,
                                                           const T *f, const T *dinv, int init) {
  constexpr int DIM = 3, VW = 4;
  const int K = P.K;
  // the case scalars once per CTA (one thread per case), the shared flag by
  // thread 0: every thread reading the same lines would queue at one L2 slice
  __shared__ T s_alpha[kMaxCases];
  __shared__ int s_frozen[kMaxCases], s_all;
  if (threadIdx.x == 0) s_all = init ? 0 : P.ctl->all_done;
  for (int cc = threadIdx.x; cc < K; cc += blockDim.x) {
    const MultiScalars &sc = P.sc[cc];
    const int fz = !init && sc.done;
    s_frozen[cc] = fz;
    s_alpha[cc] = init || fz ? T(0) : (T)sc.alpha;
  }
  __syncthreads();
  if (s_all) return;
  const int c = threadIdx.x & (K - 1);
  const bool frozen = s_frozen[c] != 0;
  const T alpha = s_alpha[c];
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
  __syncthreads();  // (red is reused for the totals)
  double *s_tot = &red[0][0];  // [K][3] (K <= kThreads)
  if (!tree_case_sums<3>(P.partials, P.gpart, P.gcnt_up, &P.ctl->count_up, K, s_tot)) return;
  __shared__ int s_active;
  if (threadIdx.x == 0) s_active = 0;
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
