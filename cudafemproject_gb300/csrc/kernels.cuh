// sm_103a kernels of the element-by-element (EbE) elasticity path.
//
// Data layout in HBM (all in the locality order built by prep.cpp):
//  * node vectors: VW values per node (VW = 4 in 3D, 2 in 2D) so that a node is
//    one 16-byte (FP32) or 32-byte (FP64) load; the 3D pad lane is zero, except
//    in the PCG's x, r, z and p, where it carries the Jacobi inverse of one DOF
//    (k_pcg_init); kernels read the DOF lanes only;
//  * element operator, gradient form: G = sqrt(V * E_e/E) * grad N_a for the
//    local nodes a = 1..dim (N_0 follows from the partition of unity), stored
//    structure-of-arrays [ncomp][gstride] so a warp reads 128 coalesced bytes
//    per component: 36 B per tetrahedron in FP32 (16 B per triangle);
//  * patches: consecutive runs of elements handled by one CTA, with their node
//    list (halo nodes first, then the contiguous range the patch owns) and a
//    16-bit local connectivity (8 B per element).
//
// The matvec of a patch (reference: Matrix::bmm u_e = p_e^T K_e then the
// sort/reduce assembly, femfunc.cpp:66-67 + cpu_fem_utils.cpp:437-459):
//   stage  : gather the patch's node vectors into shared memory (coalesced,
//            mostly L2 hits), applying the PCG direction update p = z + beta p
//            on the fly and masking constrained DOFs;
//   compute: per element H = sum_a u_a (x) G_a, sigma = lam tr(H) I + mu (H+H^T),
//            f_a = sigma G_a (+ consistent mass), accumulated with shared atomics;
//   flush  : one float4 atomicAdd per patch node into the global result.
// The reference's applyConstraints (cpu_fem_utils.cpp:461-476) keeps K_e's
// diagonal and zeroes the off-diagonal rows/columns of constrained DOFs, i.e.
// K' = P K P + (I-P) diag(K); the masked stage/flush realise P K P and the
// owner of a node adds the (I-P) diag(K) term.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "tma.cuh"

namespace cfem {

constexpr int kThreads = 256;

struct Scalars {
  double gamma, gamma_prev, gamma0, sigma;
  double rr, ff, tol;
  int rule, maxit, iter, done;  // done: 0 running, 1 converged, 2 diverged, 3 iteration cap
  unsigned int count_spare, count_up;  // count_up: grid-sum ticket of the init kernel
  int u_iter;  // iterations completed when the last update ran (-1: none since the init kernel)
  int loops;   // device-side loop: graph bodies started in this run (k_pcg_update)
  // alpha = gamma / sigma (set by CTA 0 of the update from the matvec's block
  // partials), beta = gamma / gamma_prev (set by CTA 0 of the matvec from the
  // update's block partials, 0 before the first direction): every CTA derives
  // them identically, so no thread divides differently
  double alpha, beta;
  int loop_ok, pad2;  // device-side loop: the body count is within the cap (k_pcg_update)
};

struct DynState {
  int step;
  unsigned int count;
  // explicit steps in a two-step graph: the step of parity q reads pstep[q]
  // and its CTA 0 writes pstep[q ^ 1] (no CTA reads what its own kernel writes)
  int pstep[2];
};

// ------------------------------------------------------------------ helpers
template <typename T, int VW>
struct NodeV {
  T v[VW];
};

template <typename T, int VW>
__device__ __forceinline__ NodeV<T, VW> ldv(const T *p, int64_t node) {
  NodeV<T, VW> r;
  if constexpr (sizeof(T) == 4 && VW == 4) {
    float4 a = reinterpret_cast<const float4 *>(p)[node];
    r.v[0] = a.x; r.v[1] = a.y; r.v[2] = a.z; r.v[3] = a.w;
  } else if constexpr (sizeof(T) == 4 && VW == 2) {
    float2 a = reinterpret_cast<const float2 *>(p)[node];
    r.v[0] = a.x; r.v[1] = a.y;
  } else if constexpr (VW == 4) {
    double2 a = reinterpret_cast<const double2 *>(p)[2 * node];
    double2 b = reinterpret_cast<const double2 *>(p)[2 * node + 1];
    r.v[0] = a.x; r.v[1] = a.y; r.v[2] = b.x; r.v[3] = b.y;
  } else {
    double2 a = reinterpret_cast<const double2 *>(p)[node];
    r.v[0] = a.x; r.v[1] = a.y;
  }
  return r;
}

template <typename T, int VW>
__device__ __forceinline__ void stv(T *p, int64_t node, const NodeV<T, VW> &r) {
  if constexpr (sizeof(T) == 4 && VW == 4) {
    reinterpret_cast<float4 *>(p)[node] = make_float4(r.v[0], r.v[1], r.v[2], r.v[3]);
  } else if constexpr (sizeof(T) == 4 && VW == 2) {
    reinterpret_cast<float2 *>(p)[node] = make_float2(r.v[0], r.v[1]);
  } else if constexpr (VW == 4) {
    reinterpret_cast<double2 *>(p)[2 * node] = make_double2(r.v[0], r.v[1]);
    reinterpret_cast<double2 *>(p)[2 * node + 1] = make_double2(r.v[2], r.v[3]);
  } else {
    reinterpret_cast<double2 *>(p)[node] = make_double2(r.v[0], r.v[1]);
  }
}

template <typename T, int VW>
__device__ __forceinline__ void stv_zero(T *p, int64_t node) {
  NodeV<T, VW> z;
#pragma unroll
  for (int d = 0; d < VW; ++d) z.v[d] = T(0);
  stv<T, VW>(p, node, z);
}

template <typename T, int VW>
__device__ __forceinline__ void atomic_addv(T *p, int64_t node, const NodeV<T, VW> &r, int dim) {
  if constexpr (sizeof(T) == 4 && VW == 4) {
    atomicAdd(reinterpret_cast<float4 *>(p) + node, make_float4(r.v[0], r.v[1], r.v[2], 0.f));
  } else if constexpr (sizeof(T) == 4 && VW == 2) {
    atomicAdd(reinterpret_cast<float2 *>(p) + node, make_float2(r.v[0], r.v[1]));
  } else {
    for (int d = 0; d < dim; ++d) atomicAdd(p + node * VW + d, r.v[d]);
  }
}

// Sum N doubles over the block; result valid in thread 0.
template <int N>
__device__ __forceinline__ void block_sum(double (&v)[N]) {
  __shared__ double red[N][kThreads / 32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < N; ++k) {
    double x = v[k];
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
    if (lane == 0) red[k][wid] = x;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < N; ++k) {
      double s = 0;
      for (int i = 0; i < (int)(blockDim.x >> 5); ++i) s += red[k][i];
      v[k] = s;
    }
  }
  __syncthreads();
}

// Sum of the per-block partials in the last block: strided per-thread sums,
// a shuffle tree per warp and the warp totals in warp order, so the result is
// a fixed function of the partials. Result valid in thread 0.
template <int N>
__device__ __forceinline__ void last_block_total(double (&v)[N], const double *partials) {
  __shared__ double red2[N][kThreads / 32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < N; ++k) {
    double s = 0;
    for (int b = threadIdx.x; b < (int)gridDim.x; b += blockDim.x) s += __ldcg(partials + (size_t)b * N + k);
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if (lane == 0) red2[k][wid] = s;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < N; ++k) {
      double t = 0;
      for (int i = 0; i < (int)(blockDim.x >> 5); ++i) t += red2[k][i];
      v[k] = t;
    }
  }
}

// Publishes this block's partial sums (thread 0 holds them after block_sum);
// returns true in thread 0 of the last block to finish, which then holds the
// grid totals. The ticket counter is reset for the next launch.
template <int N>
__device__ __forceinline__ bool publish_and_total(double (&v)[N], double *partials, unsigned int *count) {
  __shared__ bool last;
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < N; ++k) partials[(size_t)blockIdx.x * N + k] = v[k];
    __threadfence();
    unsigned int t = atomicAdd(count, 1u);
    last = (t == gridDim.x - 1);
  }
  __syncthreads();
  if (!last) return false;
  __threadfence();
  last_block_total<N>(v, partials);
  if (threadIdx.x == 0) *count = 0;
  return threadIdx.x == 0;
}

// Grid sum of N doubles per thread (block order, scheduling-independent).
template <int N>
__device__ __forceinline__ bool grid_sum_last(double (&v)[N], double *partials, unsigned int *count) {
  block_sum<N>(v);
  return publish_and_total<N>(v, partials, count);
}

// ---- compensated FP32 accumulation ------------------------------------------
// GB300's FP64 pipe is narrow, so the FP32 kernels accumulate their dot
// products as unevaluated float pairs (hi + lo, Knuth's TwoSum) per thread and
// per warp, and switch to FP64 only for the warp totals, the block and the
// grid sums. The pair carries about 48 significant bits.
struct Comp32 {
  float hi = 0.f, lo = 0.f;
  __device__ __forceinline__ void add(float v) {
    const float s = hi + v, bp = s - hi;
    lo += (hi - (s - bp)) + (v - bp);
    hi = s;
  }
  __device__ __forceinline__ void merge(float h2, float l2) {
    const float s = hi + h2, bp = s - hi;
    lo = lo + l2 + ((hi - (s - bp)) + (h2 - bp));
    hi = s;
  }
};

// Per-thread accumulator in the working precision's reduction type.
template <typename T>
struct DotAcc {
  double s = 0;
  __device__ __forceinline__ void add(double v) { s += v; }
};
template <>
struct DotAcc<float> {
  Comp32 c;
  __device__ __forceinline__ void add(float v) { c.add(v); }
};

// Block total of one accumulator per thread (all threads call; valid in thread 0).
template <typename T>
__device__ __forceinline__ double block_total(const DotAcc<T> &a) {
  __shared__ double red_bt[kThreads / 32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  double w;
  if constexpr (sizeof(T) == 8) {
    w = a.s;
    for (int o = 16; o > 0; o >>= 1) w += __shfl_down_sync(0xffffffffu, w, o);
  } else {
    Comp32 c = a.c;
    for (int o = 16; o > 0; o >>= 1) {
      const float h2 = __shfl_down_sync(0xffffffffu, c.hi, o), l2 = __shfl_down_sync(0xffffffffu, c.lo, o);
      c.merge(h2, l2);
    }
    w = (double)c.hi + (double)c.lo;
  }
  if (lane == 0) red_bt[wid] = w;
  __syncthreads();
  double t = 0;
  if (threadIdx.x == 0)
    for (int i = 0; i < (int)(blockDim.x >> 5); ++i) t += red_bt[i];
  __syncthreads();
  return t;
}

// Grid sum of N accumulators per thread; true in thread 0 of the last block,
// whose v then holds the totals.
template <int N, typename T>
__device__ __forceinline__ bool grid_sum_acc(DotAcc<T> (&a)[N], double (&v)[N], double *partials, unsigned int *count) {
  if constexpr (sizeof(T) == 8) {
#pragma unroll
    for (int k = 0; k < N; ++k) v[k] = a[k].s;
    return grid_sum_last<N>(v, partials, count);
  } else {
    __shared__ double red[N][kThreads / 32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < N; ++k) {
      Comp32 c = a[k].c;
      for (int o = 16; o > 0; o >>= 1) {
        const float h2 = __shfl_down_sync(0xffffffffu, c.hi, o), l2 = __shfl_down_sync(0xffffffffu, c.lo, o);
        c.merge(h2, l2);
      }
      if (lane == 0) red[k][wid] = (double)c.hi + (double)c.lo;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
#pragma unroll
      for (int k = 0; k < N; ++k) {
        double s = 0;
        for (int i = 0; i < (int)(blockDim.x >> 5); ++i) s += red[k][i];
        v[k] = s;
      }
    }
    __syncthreads();
    return publish_and_total<N>(v, partials, count);
  }
}


// ---- single-mesh PCG scalars without a last-block phase ---------------------
// The PCG-form matvec and the update kernel of a single-mesh PCG pass their
// grid sums as per-block partials only: each block stores its partial sums
// (no fence, no ticket, no block waiting for the others), and every CTA of the
// kernel that follows adds them after its dependency wait, in block order: the
// same order in every CTA, so all CTAs derive bit-identical scalars. CTA 0
// then publishes them for the kernel after it and for the host. A kernel
// reads only Scalars fields that the kernel before it wrote:
//   matvec reads  u_iter, gamma_prev, alpha (update) and the constants,
//          writes gamma, rr, iter, beta, done;
//   update reads  gamma, iter, done (matvec),
//          writes alpha, sigma, gamma_prev, u_iter.
// u_iter < 0 (init kernel): no update yet; the matvec takes the init kernel's
// scalars and beta = 0.

// Thread 0 stores the block totals of N accumulators at part[blockIdx.x * N + k]
// (all threads call; red: N x 8 doubles of shared scratch).
template <int N, typename T>
__device__ __forceinline__ void store_block_partials(const DotAcc<T> (&a)[N], double *part, double *red) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < N; ++k) {
    double w;
    if constexpr (sizeof(T) == 8) {
      w = a[k].s;
      for (int o = 16; o > 0; o >>= 1) w += __shfl_down_sync(0xffffffffu, w, o);
    } else {
      Comp32 c = a[k].c;
      for (int o = 16; o > 0; o >>= 1) {
        const float h2 = __shfl_down_sync(0xffffffffu, c.hi, o), l2 = __shfl_down_sync(0xffffffffu, c.lo, o);
        c.merge(h2, l2);
      }
      w = (double)c.hi + (double)c.lo;
    }
    if (lane == 0) red[k * 8 + wid] = w;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < N; ++k) {
      double t = 0;
      for (int i = 0; i < (int)(blockDim.x >> 5); ++i) t += red[k * 8 + i];
      part[(size_t)blockIdx.x * N + k] = t;
    }
  }
}

// First half of a fixed-order sum of per-block partials: thread t adds
// part[b * N + k] for b = t, t + blockDim, ... in turn (two loads in flight),
// a shuffle tree per warp, lane 0 stores the warp sum at red[k * 8 + warp].
// After a barrier, partials_total() adds the warp sums in warp order. Blocks
// of at most 256 threads.
template <int N>
__device__ __forceinline__ void partials_warp_sums(const double *part, int nblocks, double *red) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int B = blockDim.x;
  double sum[N];
#pragma unroll
  for (int k = 0; k < N; ++k) sum[k] = 0;
  for (int b0 = threadIdx.x; b0 < nblocks; b0 += 2 * B) {
    double v[2][N];
#pragma unroll
    for (int q = 0; q < 2; ++q)
#pragma unroll
      for (int k = 0; k < N; ++k) v[q][k] = b0 + q * B < nblocks ? __ldcg(part + (size_t)(b0 + q * B) * N + k) : 0.0;
#pragma unroll
    for (int q = 0; q < 2; ++q)
#pragma unroll
      for (int k = 0; k < N; ++k)
        if (b0 + q * B < nblocks) sum[k] += v[q][k];
  }
#pragma unroll
  for (int k = 0; k < N; ++k) {
    double x = sum[k];
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
    if (lane == 0) red[k * 8 + wid] = x;
  }
}
__device__ __forceinline__ double partials_total(const double *red, int k) {
  double t = 0;
  for (int i = 0; i < (int)(blockDim.x >> 5); ++i) t += red[k * 8 + i];
  return t;
}

// Start of a single-mesh PCG-form matvec (all threads, after the dependency
// wait): r.z and r.r of the update before it, beta and the stopping test
// (reference rule gamma < tol gamma0, residual rule ||r|| <= tol ||f||, the
// iteration cap). Returns true once the solve has stopped (uniform). Thread 0
// alone reads the scalars, in the same round trip as every thread's partial
// loads, and shares the result through red (24 doubles of shared scratch):
// the CTAs of a grid reading the same line thread by thread would queue at
// one L2 slice.
template <typename T>
__device__ __forceinline__ bool pcg_matvec_scalars(Scalars *s, const double *up_part, int n_up, T &beta,
                                                   double *red) {
  int ui = 0, done0 = 0, rule = 0, maxit = 0;
  double alpha = 0, tol = 0, g0 = 0, ff = 0, gp = 1;
  if (threadIdx.x == 0) {
    ui = s->u_iter;
    done0 = s->done;
    alpha = s->alpha;
    tol = s->tol;
    g0 = s->gamma0;
    ff = s->ff;
    gp = s->gamma_prev;
    rule = s->rule;
    maxit = s->maxit;
  }
  partials_warp_sums<2>(up_part, n_up, red);  // (ignored before the first update)
  __syncthreads();
  if (threadIdx.x == 0) {
    double b = 0;
    int done = done0;
    if (ui >= 0) {
      const double g = partials_total(red, 0), rr = partials_total(red, 1);
      const int it = ui + 1;
      done = 0;
      if (!isfinite(g) || !isfinite(alpha)) done = 2;
      else if (rule == 0 && g < tol * g0) done = 1;
      else if (rule == 1 && sqrt(rr) <= tol * sqrt(ff)) done = 1;
      else if (it >= maxit) done = 3;
      b = g / gp;
      if (blockIdx.x == 0) {
        s->gamma = g;
        s->rr = rr;
        s->iter = it;
        s->beta = b;
        s->done = done;
      }
    }
    red[18] = b;
    red[19] = (double)done;
  }
  __syncthreads();
  beta = T(red[18]);
  const bool stop = red[19] != 0.0;
  __syncthreads();  // (red may be reused)
  return stop;
}

// ------------------------------------------------------------------ element kernel
// Stiffness (and consistent mass) action of one element in gradient form.
// u[a][d]: masked nodal values; G: dim*dim gradient components of nodes 1..dim.
template <typename T, int DIM>
__device__ __forceinline__ void element_force(const T (&u)[DIM + 1][DIM], const T (&G)[DIM * DIM], T lam, T mu,
                                              T cK, T mcoef, T (&f)[DIM + 1][DIM]) {
  T H[DIM][DIM];
#pragma unroll
  for (int i = 0; i < DIM; ++i)
#pragma unroll
    for (int j = 0; j < DIM; ++j) {
      T h = 0;
#pragma unroll
      for (int a = 1; a <= DIM; ++a) h += (u[a][i] - u[0][i]) * G[(a - 1) * DIM + j];
      H[i][j] = h;
    }
  T tr = 0;
#pragma unroll
  for (int i = 0; i < DIM; ++i) tr += H[i][i];
  T S[DIM][DIM];
#pragma unroll
  for (int i = 0; i < DIM; ++i)
#pragma unroll
    for (int j = 0; j < DIM; ++j) S[i][j] = cK * (mu * (H[i][j] + H[j][i]) + (i == j ? lam * tr : T(0)));
#pragma unroll
  for (int d = 0; d < DIM; ++d) f[0][d] = 0;
#pragma unroll
  for (int a = 1; a <= DIM; ++a)
#pragma unroll
    for (int i = 0; i < DIM; ++i) {
      T s = 0;
#pragma unroll
      for (int j = 0; j < DIM; ++j) s += S[i][j] * G[(a - 1) * DIM + j];
      f[a][i] = s;
      f[0][i] -= s;
    }
  if (mcoef != T(0)) {
#pragma unroll
    for (int d = 0; d < DIM; ++d) {
      T sum = 0;
#pragma unroll
      for (int a = 0; a <= DIM; ++a) sum += u[a][d];
#pragma unroll
      for (int a = 0; a <= DIM; ++a) f[a][d] += mcoef * (u[a][d] + sum);
    }
  }
}

// Stiffness action of a tet from vertex differences du_a = u_a - u_0 (a = 1..3),
// added to the forces f1..f3 on vertices 1..3 (the force on vertex 0 is minus
// their sum): H = sum_a du_a (x) G_a, S = lam tr(H) I + mu (H + H^T),
// f_a += S G_a, each component one fused multiply-add chain into f_a.
// lam, mu already carry the operator's stiffness factor.
template <typename T>
__device__ __forceinline__ void tet_forces_acc(const T (&d1)[3], const T (&d2)[3], const T (&d3)[3], const T (&G)[9],
                                               T lam, T mu, T (&f1)[3], T (&f2)[3], T (&f3)[3]) {
  T H[3][3];
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) H[i][j] = d1[i] * G[j] + d2[i] * G[3 + j] + d3[i] * G[6 + j];
  const T tr = H[0][0] + H[1][1] + H[2][2];
  T S[3][3];
  const T two_mu = mu + mu;
#pragma unroll
  for (int i = 0; i < 3; ++i) S[i][i] = two_mu * H[i][i] + lam * tr;
  S[0][1] = S[1][0] = mu * (H[0][1] + H[1][0]);
  S[0][2] = S[2][0] = mu * (H[0][2] + H[2][0]);
  S[1][2] = S[2][1] = mu * (H[1][2] + H[2][1]);
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    f1[i] = fma(S[i][2], G[2], fma(S[i][1], G[1], fma(S[i][0], G[0], f1[i])));
    f2[i] = fma(S[i][2], G[5], fma(S[i][1], G[4], fma(S[i][0], G[3], f2[i])));
    f3[i] = fma(S[i][2], G[8], fma(S[i][1], G[7], fma(S[i][0], G[6], f3[i])));
  }
}

// ------------------------------------------------------------------ matvec
enum MvMode { MV_PLAIN = 0, MV_PCG = 1, MV_DYN = 2 };

// Control block of a batched solve (independent meshes).
struct BatchCtl {
  int iter, all_done;
  unsigned int count_mv, count_up;
};

template <typename T>
struct MvParams {
  int n_patches;
  const int32_t *elem_off, *node_off, *nodes, *own;
  const uint2 *lconn;
  const uint8_t *bits;
  const T *G;        // [ncomp][gstride]
  int64_t gstride;
  const T *mcoef;    // per element consistent-mass coefficient, or nullptr
  T lam, mu, cK, cM;
  const T *diagA;    // node vectors: diagonal of the operator (used on constrained DOFs)
  const T *x;        // PLAIN: x; PCG: z; DYN: d_old
  const T *x2;       // PCG: p_old; DYN: v
  const T *x3;       // DYN: a
  T *xout;           // PCG: p_new; DYN: d_new (owned nodes only)
  T *y;              // result accumulation (zero on entry)
  T *yzero;          // PCG: zeroed at the owned nodes (the next iteration's y), or nullptr
  Scalars *sc;       // PCG scalars (single mesh)
  double *partials;  // [gridDim] partial sums of p.Ap
  const double *up_part;  // PCG: r.z, r.r partials of the update before it, n_up blocks
  int n_up;
  T c1, c2;          // DYN: d_new = d + c1 v + c2 a
  const uint16_t *inc, *inc_start;  // per-patch incidence lists (prep.hpp)
  int pe, np_max;    // element slots per patch, node slots per patch (multiple of 4)
  // batch of independent meshes (all nullptr for a single mesh): every patch
  // belongs to one instance with its own material and PCG scalars
  const int32_t *patch_inst;      // [n_patches]
  const T *pmat;                  // [n_patches][2]: lambda, mu
  Scalars *isc;                   // [n_inst] per-instance PCG scalars
  BatchCtl *bctl;
  double *patch_energy;           // [n_patches] per-patch p.Ap
  const int32_t *inst_patch_off;  // [n_inst + 1]
  int n_inst;
};

// Last-block helper for batches: per instance i, the sum of vals[p*stride + k]
// over its contiguous patch range, one warp per instance (each lane keeps four
// interleaved partial sums so that its loads overlap, then a shuffle tree: a
// fixed order). Instances with skip[i] != 0 (when skip is given) are left
// out. Called by all threads of one block.
template <int N>
__device__ __forceinline__ void instance_sums(const double *vals, int stride, const int32_t *inst_patch_off, int n_inst,
                                              double *out /* [n_inst][N] */, const Scalars *skip = nullptr) {
  const int lane = threadIdx.x & 31, nwarp = blockDim.x >> 5;
  for (int i = threadIdx.x >> 5; i < n_inst; i += nwarp) {
    if (skip && skip[i].done) continue;
    const int p0 = inst_patch_off[i], p1 = inst_patch_off[i + 1];
#pragma unroll
    for (int k = 0; k < N; ++k) {
      double s4[4] = {0, 0, 0, 0};
      int p = p0 + lane;
      for (; p + 96 < p1; p += 128)
#pragma unroll
        for (int q = 0; q < 4; ++q) s4[q] += __ldcg(vals + (size_t)(p + 32 * q) * stride + k);
#pragma unroll
      for (int q = 0; q < 3; ++q)
        if (p + 32 * q < p1) s4[q] += __ldcg(vals + (size_t)(p + 32 * q) * stride + k);
      double s = (s4[0] + s4[1]) + (s4[2] + s4[3]);
      for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
      if (lane == 0) out[(size_t)i * N + k] = s;
    }
  }
}

// One CTA per patch (grid-stride over patches). Three phases per patch:
//  1. stage: the patch's node values (PCG: p = z + beta p_old, written back for
//     the nodes the patch owns; DYN: the predictor), constrained DOFs zeroed;
//     the patch's incidence lists are copied next to them;
//  2. elements: one thread per element computes its nodal forces from the
//     scaled gradients and stores them with plain stores into its own slots
//     fs[a][le] (no atomics, conflict-free: consecutive threads, consecutive slots);
//  3. nodes: one thread per patch node sums its incidences in a fixed order,
//     masks constrained DOFs / adds the (I - P) diag term on owned nodes, and
//     adds the result into y (global atomics: a node can be in several patches).
template <typename T, int DIM, int MODE>
__global__ void __launch_bounds__(kThreads) k_matvec(MvParams<T> P) {
  constexpr int VW = DIM == 3 ? 4 : 2;
  constexpr int NV = DIM + 1;
  constexpr int NC = DIM * DIM;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T *sp = reinterpret_cast<T *>(smem_raw);                                     // [np_max][VW]
  T *fs = sp + (size_t)P.np_max * VW;                                          // [NV][pe][VW]
  uint16_t *si = reinterpret_cast<uint16_t *>(fs + (size_t)NV * P.pe * VW);  // [4 pe] codes
  uint16_t *ss = si + 4 * P.pe;                                                // [np_max + 1] starts
  int32_t *sg = reinterpret_cast<int32_t *>(ss + ((P.np_max + 2) & ~1));       // [np_max] node ids
  uint8_t *sb = reinterpret_cast<uint8_t *>(sg + P.np_max);                    // [np_max] BC bits
  __shared__ double red_pcg[24];
  T beta = 0;
  if (MODE == MV_PCG && pcg_matvec_scalars<T>(P.sc, P.up_part, P.n_up, beta, red_pcg)) return;
  DotAcc<T> energy;
  for (int patch = blockIdx.x; patch < P.n_patches; patch += gridDim.x) {
    const int nb = P.node_off[patch], nn = P.node_off[patch + 1] - nb, own = P.own[patch];
    const int e0 = P.elem_off[patch], ne = P.elem_off[patch + 1] - e0;
    // 1. stage
    {
      const uint2 *src = reinterpret_cast<const uint2 *>(P.inc + (size_t)4 * e0);  // 4 codes per element
      for (int q = threadIdx.x; q < ne; q += blockDim.x) reinterpret_cast<uint2 *>(si)[q] = src[q];
      for (int i = threadIdx.x; i <= nn; i += blockDim.x) ss[i] = P.inc_start[nb + patch + i];
    }
    for (int i = threadIdx.x; i < nn; i += blockDim.x) {
      const int g = P.nodes[nb + i];
      NodeV<T, VW> v = ldv<T, VW>(P.x, g);
      if (MODE == MV_PCG) {
        if (beta != T(0)) {
          NodeV<T, VW> po = ldv<T, VW>(P.x2, g);
#pragma unroll
          for (int d = 0; d < DIM; ++d) v.v[d] += beta * po.v[d];
        }
        if (i >= own) {
          stv<T, VW>(P.xout, g, v);
          if (P.yzero) stv_zero<T, VW>(P.yzero, g);
        }
      } else if (MODE == MV_DYN) {
        NodeV<T, VW> vv = ldv<T, VW>(P.x2, g), aa = ldv<T, VW>(P.x3, g);
#pragma unroll
        for (int d = 0; d < DIM; ++d) v.v[d] += P.c1 * vv.v[d] + P.c2 * aa.v[d];
        if (i >= own) stv<T, VW>(P.xout, g, v);
      }
      const unsigned b = P.bits[g];
      NodeV<T, VW> m;
#pragma unroll
      for (int d = 0; d < VW; ++d) m.v[d] = (d < DIM && !(b >> d & 1u)) ? v.v[d] : T(0);
      stv<T, VW>(sp, i, m);
      sg[i] = g;
      sb[i] = (uint8_t)b;
    }
    __syncthreads();
    // 2. elements
    for (int le = threadIdx.x; le < ne; le += blockDim.x) {
      const int e = e0 + le;
      const uint2 c = P.lconn[e];
      int li[4] = {(int)(c.x & 0xffffu), (int)(c.x >> 16), (int)(c.y & 0xffffu), (int)(c.y >> 16)};
      T G[NC];
#pragma unroll
      for (int k = 0; k < NC; ++k) G[k] = P.G[(size_t)k * P.gstride + e];
      T u[NV][DIM], f[NV][DIM];
#pragma unroll
      for (int a = 0; a < NV; ++a) {
        const NodeV<T, VW> s = ldv<T, VW>(sp, li[a]);
#pragma unroll
        for (int d = 0; d < DIM; ++d) u[a][d] = s.v[d];
      }
      const T mc = P.mcoef ? P.cM * P.mcoef[e] : T(0);
      element_force<T, DIM>(u, G, P.lam, P.mu, P.cK, mc, f);
      // p_e.A_e p_e in the working precision; one FP64 add per element (the
      // FP64 pipe of this part is narrow, so no per-term double arithmetic)
      T e_elem = 0;
#pragma unroll
      for (int a = 0; a < NV; ++a) {
        NodeV<T, VW> o;
#pragma unroll
        for (int d = 0; d < VW; ++d) o.v[d] = d < DIM ? f[a][d] : T(0);
#pragma unroll
        for (int d = 0; d < DIM; ++d)
          if (MODE == MV_PCG) e_elem += u[a][d] * f[a][d];
        stv<T, VW>(fs, (size_t)a * P.pe + le, o);
      }
      if (MODE == MV_PCG) energy.add(e_elem);
    }
    __syncthreads();
    // 3. nodes
    for (int i = threadIdx.x; i < nn; i += blockDim.x) {
      const int g = sg[i];
      const unsigned b = sb[i];
      T acc[DIM];
#pragma unroll
      for (int d = 0; d < DIM; ++d) acc[d] = 0;
      const int k1 = ss[i + 1];
      for (int k = ss[i]; k < k1; ++k) {
        const unsigned code = si[k];
        const NodeV<T, VW> f = ldv<T, VW>(fs, (size_t)(code & 3u) * P.pe + (code >> 2));
#pragma unroll
        for (int d = 0; d < DIM; ++d) acc[d] += f.v[d];
      }
      NodeV<T, VW> r;
      bool any = false;
#pragma unroll
      for (int d = 0; d < VW; ++d) {
        T val = (d < DIM && !(b >> d & 1u)) ? acc[d < DIM ? d : 0] : T(0);
        r.v[d] = val;
        any |= val != T(0);
      }
      if (b && i >= own) {
        // (I - P) diag(A) x on the constrained DOFs of an owned node
        NodeV<T, VW> v = ldv<T, VW>(P.x, g);
        if (MODE == MV_PCG && beta != T(0)) {
          NodeV<T, VW> po = ldv<T, VW>(P.x2, g);
#pragma unroll
          for (int d = 0; d < DIM; ++d) v.v[d] += beta * po.v[d];
        } else if (MODE == MV_DYN) {
          NodeV<T, VW> vv = ldv<T, VW>(P.x2, g), aa = ldv<T, VW>(P.x3, g);
#pragma unroll
          for (int d = 0; d < DIM; ++d) v.v[d] += P.c1 * vv.v[d] + P.c2 * aa.v[d];
        }
        NodeV<T, VW> dg = ldv<T, VW>(P.diagA, g);
#pragma unroll
        for (int d = 0; d < DIM; ++d)
          if (b >> d & 1u) {
            T t = dg.v[d] * v.v[d];
            r.v[d] = t;
            any |= t != T(0);
            if (MODE == MV_PCG) energy.add(t * v.v[d]);
          }
      }
      if (any) atomic_addv<T, VW>(P.y, g, r, DIM);
    }
    __syncthreads();
  }
  if (MODE == MV_PCG) {  // p.Ap partials; the update kernel forms sigma and alpha
    const DotAcc<T> ea[1] = {energy};
    store_block_partials<1, T>(ea, P.partials, red_pcg);
  }
}

// Shared-memory bytes of k_matvec for a patch layout.
inline size_t matvec_smem_bytes(int dim, size_t tsize, int pe, int np_max) {
  const int vw = dim == 3 ? 4 : 2;
  return (size_t)np_max * vw * tsize + (size_t)(dim + 1) * pe * vw * tsize + (size_t)4 * pe * 2 +
         (size_t)((np_max + 2) & ~1) * 2 + (size_t)np_max * 5;
}

// ------------------------------------------------------------------ PCG vector kernels
template <typename T>
struct VecParams {
  int64_t n_nodes;
  T *x, *r, *z, *p, *u;
  const T *dinv;
  const T *f;        // init: right-hand side
  Scalars *sc;
  double *partials;  // init: grid-sum scratch
  const double *mv_part;  // update: p.Ap partials of the matvec before it, n_mv blocks
  int n_mv;
  double *up_part;        // update: its own r.z, r.r partials [grid][2]
  // PCG iterations inside a CUDA-graph WHILE node (0: loop on the host); see
  // k_pcg_update
  unsigned long long cond;
  int cond_role;   // bit 0: first update of the body, bit 1: last
  int cond_chunk;  // iterations per body
};

// r = f - u (warm) or f; x = 0 unless warm; z = M^-1 r; u = 0; gamma0 = r.z.
// In 3D the spare fourth lanes carry M^-1 for the update kernel: x.w = M^-1
// of the x DOF, r.w of the y DOF, z.w (and so p.w, which the matvec copies
// from z) of the z DOF. Every kernel that reads these vectors for their
// values uses only the first three lanes.
template <typename T, int DIM>
__global__ void __launch_bounds__(kThreads) k_pcg_init(VecParams<T> P, int warm) {
  constexpr int VW = DIM == 3 ? 4 : 2;
  DotAcc<T> acc[3];  // r.z, r.r, f.f
  for (int64_t n = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; n < P.n_nodes; n += (int64_t)gridDim.x * blockDim.x) {
    NodeV<T, VW> f = ldv<T, VW>(P.f, n), di = ldv<T, VW>(P.dinv, n), r, z, zero;
    NodeV<T, VW> u = ldv<T, VW>(P.u, n);
#pragma unroll
    for (int d = 0; d < VW; ++d) { zero.v[d] = 0; r.v[d] = 0; z.v[d] = 0; }
    if constexpr (DIM == 3) {
      r.v[3] = di.v[1];
      z.v[3] = di.v[2];
    }
    T rz = 0, rr = 0, ff = 0;
#pragma unroll
    for (int d = 0; d < DIM; ++d) {
      r.v[d] = warm ? f.v[d] - u.v[d] : f.v[d];
      z.v[d] = r.v[d] * di.v[d];
      rz += r.v[d] * z.v[d];
      rr += r.v[d] * r.v[d];
      ff += f.v[d] * f.v[d];
    }
    acc[0].add(rz);
    acc[1].add(rr);
    acc[2].add(ff);
    stv<T, VW>(P.r, n, r);
    stv<T, VW>(P.z, n, z);
    stv<T, VW>(P.u, n, zero);
    if constexpr (DIM == 3) {
      NodeV<T, VW> x = zero;
      if (warm) x = ldv<T, VW>(P.x, n);
      x.v[3] = di.v[0];
      stv<T, VW>(P.x, n, x);
    } else if (!warm) {
      stv<T, VW>(P.x, n, zero);
    }
  }
  double tot[3];
  if (grid_sum_acc<3, T>(acc, tot, P.partials, &P.sc->count_up)) {
    const double *acc = tot;
    Scalars *s = P.sc;
    s->gamma0 = s->gamma = s->gamma_prev = acc[0];
    s->rr = acc[1];
    s->ff = acc[2];
    s->iter = 0;
    s->u_iter = -1;
    s->sigma = 0;
    s->alpha = 0;
    s->beta = 0;
    int done = 0;
    if (acc[0] == 0.0) done = 1;
    if (s->rule == 1 && sqrt(acc[1]) <= s->tol * sqrt(acc[2])) done = 1;
    if (!isfinite(acc[0])) done = 2;
    s->done = done;
  }
}

// alpha = gamma / p.Ap; x += alpha p; r -= alpha u; z = M^-1 r; gamma' = r.z.
// u is left as it is: the matvec of the next iteration accumulates into the
// other u buffer, which the matvec before it zeroed (MvParams::yzero).
// Thread t handles nodes t, t + T, t + 2T, ... (T threads in the grid), U of
// them per round with all their loads in flight. In 3D, M^-1 comes from the
// fourth lanes of x, r and p (k_pcg_init), so a node costs four loads; in 2D
// from dinv. x and r (and dinv) are not written by the matvec this kernel
// waits for (its predecessor, the update before it, has completed once that
// matvec passed its own wait), so the first round's loads of them go out
// before the wait.
// LOOP: the instance for the graph WHILE node (the condition calls below);
// the host-loop instance leaves them out, which also keeps it profilable
// (ncu does not profile kernels that set a graph condition).
template <typename T, int DIM, bool LOOP = false>
__global__ void __launch_bounds__(kThreads, 2) k_pcg_update(VecParams<T> P) {
  constexpr int VW = DIM == 3 ? 4 : 2;
  constexpr int U = sizeof(T) == 4 ? 4 : 2;
  const int64_t nthr = (int64_t)gridDim.x * blockDim.x;
  int64_t base = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  NodeV<T, VW> x[U], r[U], p[U], u[U], di[U];
  auto load_own = [&]() {
#pragma unroll
    for (int q = 0; q < U; ++q) {
      const int64_t n = base + (int64_t)q * nthr;
      if (n < P.n_nodes) {
        x[q] = ldv<T, VW>(P.x, n);
        r[q] = ldv<T, VW>(P.r, n);
        if constexpr (DIM != 3) di[q] = ldv<T, VW>(P.dinv, n);
      }
    }
  };
  auto load_mv = [&]() {
#pragma unroll
    for (int q = 0; q < U; ++q) {
      const int64_t n = base + (int64_t)q * nthr;
      if (n < P.n_nodes) {
        p[q] = ldv<T, VW>(P.p, n);
        u[q] = ldv<T, VW>(P.u, n);
      }
    }
  };
  load_own();
  griddep_wait();               // A p and the p.Ap partials come from the matvec before it
  griddep_launch_dependents();  // the next matvec may start streaming its blocks
  // Device-side loop (one thread of CTA 0; the updates of a body run one
  // after another, so no two calls race): the first update of a body counts
  // the body and clears the condition, the last one sets it to "the matvec
  // before it found the run not done, and the body count is within
  // maxit / chunk + 16". A body ends the loop unless its last update sets it,
  // and the cap ends it whatever the scalars do.
  const bool cond_thread = LOOP && blockIdx.x == 0 && threadIdx.x == 0;
  if constexpr (LOOP) {
    if (cond_thread && (P.cond_role & 1)) {
      const int nl = ++P.sc->loops;
      P.sc->loop_ok = nl <= P.sc->maxit / P.cond_chunk + 16;
      cudaGraphSetConditional(P.cond, 0u);
    }
  }
  load_mv();
  // thread 0 reads the scalars while every thread loads the matvec's partials
  // (see pcg_matvec_scalars); alpha = gamma / sigma in thread 0, shared
  Scalars *s = P.sc;
  __shared__ double red_pcg[24];
  int done0 = 0, it0 = 0;
  double gamma = 0;
  if (threadIdx.x == 0) {
    done0 = s->done;
    gamma = s->gamma;
    it0 = s->iter;
    if constexpr (LOOP)
      if (cond_thread && (P.cond_role & 2)) cudaGraphSetConditional(P.cond, (done0 == 0 && s->loop_ok) ? 1u : 0u);
  }
  partials_warp_sums<1>(P.mv_part, P.n_mv, red_pcg);
  __syncthreads();
  if (threadIdx.x == 0) {
    const double sig = partials_total(red_pcg, 0), a = gamma / sig;
    red_pcg[18] = a;
    red_pcg[19] = (double)done0;
    if (blockIdx.x == 0 && !done0) {
      s->sigma = sig;
      s->alpha = a;
      s->gamma_prev = gamma;
      s->u_iter = it0;
    }
  }
  __syncthreads();
  if (red_pcg[19] != 0.0) return;
  const double alpha_d = red_pcg[18];
  const T alpha = (T)alpha_d;
  DotAcc<T> acc[2];
  for (bool first = true; base < P.n_nodes; base += U * nthr, first = false) {
    if (!first) {
      load_own();
      load_mv();
    }
#pragma unroll
    for (int q = 0; q < U; ++q) {
      const int64_t n = base + (int64_t)q * nthr;
      if (n >= P.n_nodes) continue;
      NodeV<T, VW> z;
#pragma unroll
      for (int d = 0; d < VW; ++d) z.v[d] = 0;
      T m[DIM];
      if constexpr (DIM == 3) {
        m[0] = x[q].v[3];
        m[1] = r[q].v[3];
        m[2] = p[q].v[3];
        z.v[3] = p[q].v[3];
      } else {
#pragma unroll
        for (int d = 0; d < DIM; ++d) m[d] = di[q].v[d];
      }
      T rz = 0, rr = 0;
#pragma unroll
      for (int d = 0; d < DIM; ++d) {
        x[q].v[d] += alpha * p[q].v[d];
        r[q].v[d] -= alpha * u[q].v[d];
        z.v[d] = r[q].v[d] * m[d];
        rz += r[q].v[d] * z.v[d];
        rr += r[q].v[d] * r[q].v[d];
      }
      acc[0].add(rz);
      acc[1].add(rr);
      stv<T, VW>(P.x, n, x[q]);
      stv<T, VW>(P.r, n, r[q]);
      stv<T, VW>(P.z, n, z);
    }
  }
  // r.z, r.r partials; the next matvec forms gamma, beta and the stopping test
  store_block_partials<2, T>(acc, P.up_part, red_pcg);
}

}  // namespace cfem
