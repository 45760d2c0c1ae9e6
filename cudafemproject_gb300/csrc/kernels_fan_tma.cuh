// Edge-fan EbE matvec with the per-patch data streamed by bulk asynchronous
// copies. Two threads share a fan: half h evaluates tets 3h .. 3h+2 and owns
// the six node slots P, Q, R_3h .. R_3h+3 (kHalfSlots = 12 slots per fan, of
// which 9 distinct nodes: half 0 writes the shared P, Q, R_3 forces of both).
// Everything a patch needs apart from the node vectors lives in one
// contiguous, 128-byte aligned block of the "patch block" array:
//   [header: 4 i32]                        patch nodes, first owned node, fans, 0
//   [slot: 3 x kHfanThreads u32]           patch-local nodes of the six slots of half-thread t = 2 fan + h,
//                                          two u16 per word (slot 2q low, 2q+1 high), kNoSlot if absent
//   [fpos: 3 x kHfanThreads u32]           position of each written slot force in the node-sorted list
//   [fstart: nps u16]                      node i sums forces fstart[i] .. fstart[i+1]-1
//   [nodes: npn i32] [bits: npn u8]        global node ids and constraint bits of the patch nodes
//   [G: 3 x (2 x kHfanThreads float4 + kHfanThreads float)]
//                                          scaled gradients of tet jj of half-thread t in fan vertex
//                                          order (row (b-1)*3 + d): rows 0-3, rows 4-7, row 8
// The per-half-thread tables are thread-interleaved, so the two halves of a
// fan (adjacent lanes) never read the same bank.
// One copy per patch, issued two patches ahead into a double buffer, so the
// operator stream overlaps the arithmetic of the current patch. The forces of
// a patch are written into the G region of its own buffer once every thread
// has read its gradients, and the node sums read them back contiguously.
//
// Geometry blocks (GEO) replace the 54 gradient rows by the patch nodes'
// coordinates relative to the patch's first node, FP32 float4 (16 bytes per
// patch node instead of 36 bytes per tet), and optionally a per-tet
// sqrt(E_e / E) row block [kFanMax x kFanThreads]. The gradients are formed
// from the coordinates in registers (G_b = sqrt(V_e E_e / E) grad N_b from the
// cofactors of the edge matrix), and the forces go to a separate shared region.
#pragma once

#include "kernels.cuh"
#include "prep.hpp"
#include "tma.cuh"

namespace cfem {

constexpr int kStageUnroll = 2;      // node gathers in flight per thread while staging a patch
constexpr int kHalfSlots = 12;       // node slots per fan: 2 halves x (P, Q, 4 ring vertices)
constexpr int kFanForces = 9;        // force-list entries per fan (the halves share P, Q and R_3)
constexpr int kHfanThreads = 2 * kFanThreads;
constexpr uint16_t kNoSlot = 0xFFFF;  // absent slot of a half-thread

// fan slot (0 = P, 1 = Q, 2 + k = R_k) of half h's slot hs
__host__ __device__ __forceinline__ int half_slot_to_fan(int h, int hs) { return hs < 2 ? hs : hs + 3 * h; }
// number of valid slots of half h of a fan of length len (0 if the half has no tet)
__host__ __device__ __forceinline__ int half_slot_count(int h, int len) {
  return len > 3 * h ? 3 + (len - 3 * h < 3 ? len - 3 * h : 3) : 0;
}
// whether half h writes slot hs to the force list: the halves share P, Q and
// R_3 (slot 5 of half 0 = slot 2 of half 1), whose forces half 0 writes after
// a lane shuffle with half 1 (combine_half_forces)
__host__ __device__ __forceinline__ bool half_writes(int h, int hs) { return h == 0 || hs >= 3; }

// Adds half 1's P, Q and R_3 forces to half 0's (lanes l and l ^ X: X = 1 for
// one case per lane pair, X = C when the lanes of a half-fan carry C cases);
// every lane of the warp takes part.
template <typename T, int DIM, int X = 1>
__device__ __forceinline__ void combine_half_forces(T (&fv)[6][DIM], int h) {
#pragma unroll
  for (int d = 0; d < DIM; ++d) {
    const T p = __shfl_xor_sync(0xffffffffu, fv[0][d], X);
    const T q = __shfl_xor_sync(0xffffffffu, fv[1][d], X);
    const T r = __shfl_xor_sync(0xffffffffu, h ? fv[2][d] : fv[5][d], X);
    if (h == 0) {
      fv[0][d] += p;
      fv[1][d] += q;
      fv[5][d] += r;
    }
  }
}

// Slots of half-thread t: patch-local node indices, and how many are valid
// (a prefix: 3 + the half's tets, or 0).
__device__ __forceinline__ int load_half_slots(const unsigned char *slot_tab, int t, int (&s)[6]) {
  const uint32_t *w = reinterpret_cast<const uint32_t *>(slot_tab);
  int nk = 0;
#pragma unroll
  for (int q = 0; q < 3; ++q) {
    const uint32_t v = w[q * kHfanThreads + t];
    s[2 * q] = (int)(v & 0xFFFFu);
    s[2 * q + 1] = (int)(v >> 16);
  }
#pragma unroll
  for (int k = 0; k < 6; ++k) nk += s[k] != kNoSlot;
  return nk;
}

// Force-list position of slot k of half-thread t.
__device__ __forceinline__ int half_fpos(const unsigned char *fpos_tab, int t, int k) {
  const uint32_t v = reinterpret_cast<const uint32_t *>(fpos_tab)[(k >> 1) * kHfanThreads + t];
  return (int)((k & 1) ? v >> 16 : v & 0xFFFFu);
}

// Scaled gradients of tet jj of half-thread t (2 float4 + 1 float).
__device__ __forceinline__ void load_tet_G(const unsigned char *g_tab, int t, int jj, float (&G)[9]) {
  const unsigned char *base = g_tab + (size_t)jj * (9 * kHfanThreads * 4);
  const float4 a = reinterpret_cast<const float4 *>(base)[t];
  const float4 b = reinterpret_cast<const float4 *>(base)[kHfanThreads + t];
  G[0] = a.x; G[1] = a.y; G[2] = a.z; G[3] = a.w;
  G[4] = b.x; G[5] = b.y; G[6] = b.z; G[7] = b.w;
  G[8] = reinterpret_cast<const float *>(base + 2 * kHfanThreads * 16)[t];
}
// byte offset of gradient row k of tet jj of half-thread t inside the G region
__host__ __device__ __forceinline__ int tet_G_offset(int t, int jj, int k) {
  const int base = jj * (9 * kHfanThreads * 4);
  return k < 8 ? base + ((k >> 2) * kHfanThreads + t) * 16 + (k & 3) * 4 : base + 2 * kHfanThreads * 16 + t * 4;
}

struct FanBlockLayout {
  int bytes;        // per patch, multiple of 128
  int hdr_off, slot_off, fpos_off, fstart_off, nodes_off, bits_off;
  int g_off;        // gradient blocks: G rows; geometry blocks: end of the shared prefix
  int x_off, c_off; // geometry blocks: coordinates, per-tet scale rows (-1: none); else -1
  int nps, npn;     // fstart entries, node entries per patch
};

inline FanBlockLayout fan_block_layout(int np_max, size_t tsize) {
  FanBlockLayout L{};
  auto up = [](int x, int a) { return (x + a - 1) / a * a; };
  L.nps = up(np_max + 1, 8);
  L.npn = up(np_max, 4);
  int off = 0;
  L.hdr_off = off; off += 16;
  L.slot_off = off; off += 3 * kHfanThreads * 4;
  L.fpos_off = off; off += 3 * kHfanThreads * 4;
  L.fstart_off = off; off += L.nps * 2;
  L.nodes_off = off; off += L.npn * 4;
  L.bits_off = off; off += up(L.npn, 16);
  L.g_off = up(off, 128);
  L.bytes = up(L.g_off + (int)(kFanMax * 9 * kFanThreads * tsize), 128);
  L.x_off = L.c_off = -1;
  return L;
}

// Geometry block: the same prefix (header .. bits), then coordinates and, with
// per-element moduli, the scale rows.
inline FanBlockLayout fan_geo_block_layout(int np_max, bool with_scale) {
  FanBlockLayout L = fan_block_layout(np_max, sizeof(float));
  int off = L.g_off;
  L.x_off = off; off += L.npn * 16;
  L.c_off = -1;
  if (with_scale) { L.c_off = off; off += kFanMax * kFanThreads * 4; }
  L.bytes = (off + 127) / 128 * 128;
  return L;
}

constexpr int kForceBytes = kFanForces * kFanThreads * 16;  // separate force list of geometry blocks

// Geometry blocks: two buffers, the force list, and two stages of the node
// vectors a PCG-form matvec reads (z and p_old), gathered one patch ahead.
// Gradient blocks: two buffers and the staged node values.
inline size_t fan_tma_smem_bytes(const FanBlockLayout &L, size_t tsize) {
  if (L.x_off >= 0) return (size_t)2 * L.bytes + kForceBytes + (size_t)4 * L.npn * 4 * tsize + 16;
  return (size_t)2 * L.bytes + (size_t)L.npn * 4 * tsize + 16;
}

// Scaled gradients of the fan tet (P, Q, R_j, R_j+1) from the edge vectors
// a = x_Q - x_P, b = x_Rj - x_P, c = x_Rj+1 - x_P: grad N_Q = (b x c) / det,
// grad N_Rj = (c x a) / det, grad N_Rj+1 = (a x b) / det with det = a . (b x c),
// scaled by sqrt(V sc^2), V = |det| / 6: G = cof * sign(det) * sc / sqrt(6 |det|).
// Tets that do not exist (valid false) get zero gradients.
__device__ __forceinline__ void geo_gradients(const float (&a)[3], const float (&b)[3], const float (&c)[3], float sc,
                                              bool valid, float (&G)[9]) {
  float c1[3], c2[3], c3[3];
  c1[0] = b[1] * c[2] - b[2] * c[1];
  c1[1] = b[2] * c[0] - b[0] * c[2];
  c1[2] = b[0] * c[1] - b[1] * c[0];
  c2[0] = c[1] * a[2] - c[2] * a[1];
  c2[1] = c[2] * a[0] - c[0] * a[2];
  c2[2] = c[0] * a[1] - c[1] * a[0];
  c3[0] = a[1] * b[2] - a[2] * b[1];
  c3[1] = a[2] * b[0] - a[0] * b[2];
  c3[2] = a[0] * b[1] - a[1] * b[0];
  const float det = a[0] * c1[0] + a[1] * c1[1] + a[2] * c1[2];
  const float s = valid ? copysignf(rsqrtf(6.0f * fabsf(det)), det) * sc : 0.0f;
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    G[d] = c1[d] * s;
    G[3 + d] = c2[d] * s;
    G[6 + d] = c3[d] * s;
  }
}

struct FanTmaParams {
  const unsigned char *blocks;  // [n_patches][L.bytes]
  FanBlockLayout L;
  const int32_t *fan_off;       // [n_patches + 1]
  const int32_t *fan_elem_off;  // [n_fans + 1] (consistent-mass coefficients)
  int *err;                     // kErrTmaTimeout on a copy that never completed
  int evict_first;              // blocks larger than about half the L2: stream them with an
                                // evict-first policy, so that the node vectors stay resident
  // Self-test of the copy-timeout path (cfem_selftest_copy_timeout), zero
  // otherwise: the first copy of patch skip_patch_plus1 - 1 is never issued,
  // and the waits give up after wait_limit cycles.
  int skip_patch_plus1;
  long long wait_limit;
};

// MASS: the instance for operators with a consistent mass term (P.mcoef set;
// implicit dynamics); BATCH: the instance for batched independent meshes
// (P.patch_inst set). Both are kept apart so that the single-mesh static
// instance carries none of their registers.
template <typename T, int MODE, bool GEO = false, bool MASS = false, bool BATCH = false>
// (3 CTAs per SM: the shared memory of a CTA allows 3, the register bound makes them fit)
__global__ void __launch_bounds__(kHfanThreads, 3) k_matvec_fan_tma(MvParams<T> P, FanTmaParams F) {
  static_assert(sizeof(T) == 4, "patch blocks are FP32");
  constexpr int DIM = 3, VW = 4;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  const FanBlockLayout &L = F.L;
  unsigned char *buf0 = smem_raw, *buf1 = smem_raw + L.bytes;
  unsigned char *tail = smem_raw + 2 * (size_t)L.bytes;
  T *fgeo = reinterpret_cast<T *>(tail);                          // GEO: [kFanForces x kFanThreads][4] forces
  if (GEO) tail += kForceBytes;
  T *sp = reinterpret_cast<T *>(tail);                            // [npn][4] staged node values
  // GEO: [2 stages][z, p_old][npn][4] (PCG form; the other modes use stage 0 as sp)
  uint64_t *bar = reinterpret_cast<uint64_t *>(sp + (size_t)(GEO ? 4 : 1) * L.npn * VW);
  // PCG-form geometry kernel: the node vectors of the next patch are gathered
  // by cp.async while the current one finishes, so their latency is hidden
  constexpr bool PREFETCH = GEO && MODE == MV_PCG;
  const int stage_stride = 2 * L.npn * VW;
  constexpr bool batch = BATCH;
  const long long lim = F.wait_limit > 0 ? F.wait_limit : kWaitCycles;
  T lam = P.lam, mu = P.mu;
  __shared__ unsigned warps_done[2];  // warps finished with buffer 0 / 1 (see the end of the patch loop)
  if (threadIdx.x == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    fence_mbar_init();
    warps_done[0] = warps_done[1] = 0;
  }
  __syncthreads();
  const int step = gridDim.x;
  // Batched PCG: patches of converged instances are skipped, and their blocks
  // are not copied at all (the convergence flags come from the previous
  // kernel; up to kDoneCache instances they are cached in shared memory).
  // Every other patch is live.
  constexpr int kDoneCache = 256;  // (static shared memory of the kernel must stay small: 3 CTAs per SM)
  __shared__ unsigned char inst_done[kDoneCache];
  auto patch_live = [&](int q) -> bool {
    if (!(batch && MODE == MV_PCG)) return true;
    const int i = P.patch_inst[q];
    return i < kDoneCache ? inst_done[i] == 0 : P.isc[i].done == 0;
  };
  auto issue_copy = [&](int q, int k) {  // block of patch q into buffer k
    mbar_expect_tx(&bar[k], (unsigned)L.bytes);
    if (F.evict_first)
      bulk_load_hint(k ? buf1 : buf0, F.blocks + (size_t)q * L.bytes, (unsigned)L.bytes, &bar[k],
                     l2_evict_first_policy());
    else
      bulk_load(k ? buf1 : buf0, F.blocks + (size_t)q * L.bytes, (unsigned)L.bytes, &bar[k]);
  };
  // Single mesh: the first two blocks (static operator data) are on their way
  // before the wait for the previous kernel; everything below reads what that
  // kernel wrote.
  if (threadIdx.x == 0 && !batch)
    for (int k = 0; k < 2; ++k)
      if (blockIdx.x + k * step < P.n_patches && blockIdx.x + k * step != F.skip_patch_plus1 - 1)
        issue_copy(blockIdx.x + k * step, k);
  griddep_wait();
  // single mesh: beta and the stopping test from the update's partials (every
  // CTA alike; the staging area, not in use yet, is the reduction scratch).
  // Stored-gradient blocks defer this to the first patch, after that patch's
  // first gathers are on their way (they do not depend on beta).
  T beta = 0;
  double *red_pcg = reinterpret_cast<double *>(sp);
  const bool defer = MODE == MV_PCG && !GEO && !batch;
  const bool stopped = MODE == MV_PCG && !defer &&
                       (batch ? P.bctl->all_done != 0 : pcg_matvec_scalars<T>(P.sc, P.up_part, P.n_up, beta, red_pcg));
  if (stopped) {
    if (threadIdx.x == 0 && !batch)  // let the copies issued above land before the CTA exits
      for (int k = 0; k < 2; ++k)
        if (blockIdx.x + k * step < P.n_patches) mbar_wait_bounded(&bar[k], 0u, lim);
    return;
  }
  if (batch && MODE == MV_PCG) {
    for (int i = threadIdx.x; i < P.n_inst && i < kDoneCache; i += blockDim.x) inst_done[i] = P.isc[i].done != 0;
    __syncthreads();
  }
  if (threadIdx.x == 0 && batch)
    for (int k = 0; k < 2; ++k)
      if (blockIdx.x + k * step < P.n_patches && patch_live(blockIdx.x + k * step))
        issue_copy(blockIdx.x + k * step, k);
  unsigned phase = 0;  // bit b: parity of the next completion of buffer b's barrier
  // gathers of the node vectors of the patch in buffer Bq into stage st
  auto issue_gathers = [&](const unsigned char *Bq, T *st) {
    const int32_t *nq = reinterpret_cast<const int32_t *>(Bq + L.nodes_off);
    const int nnq = reinterpret_cast<const int32_t *>(Bq + L.hdr_off)[0];
    for (int i = threadIdx.x; i < nnq; i += kHfanThreads) {
      const int64_t g = nq[i];
      cp_async16(st + (size_t)i * VW, P.x + g * VW);
      if (beta != T(0)) cp_async16(st + (size_t)(L.npn + i) * VW, P.x2 + g * VW);
    }
  };
  if constexpr (PREFETCH) {
    if (blockIdx.x < P.n_patches && mbar_wait_bounded(&bar[0], 0u, lim)) issue_gathers(buf0, sp);
    cp_async_commit();
  }
  DotAcc<T> energy;
  int it = 0;
  for (int patch = blockIdx.x; patch < P.n_patches; patch += step, ++it) {
    const int b = it & 1;
    unsigned char *B = b ? buf1 : buf0;
    // Every thread waits for the block itself; the staging barrier below
    // makes a failed copy a uniform exit (a thread whose wait failed reads
    // nothing of the block before it).
    // the kernel after this one (launched with programmatic dependent launch)
    // may start once every CTA is on its last patch: its CTAs take the SMs of
    // the CTAs that finish early and wait there for this grid to complete
    if (patch + step >= P.n_patches) griddep_launch_dependents();
    const bool live = patch_live(patch);
    bool ok = true;
    if (live) {
      ok = mbar_wait_bounded(&bar[b], (phase >> b) & 1u, lim);
      phase ^= 1u << b;
    }
    auto copy_failed = [&]() {
      if (PREFETCH) cp_async_wait<0>();
      if (threadIdx.x == 0) {
        atomicOr(F.err, kErrTmaTimeout);
        if (patch + step < P.n_patches && patch_live(patch + step))
          mbar_wait_bounded(&bar[b ^ 1], (phase >> (b ^ 1)) & 1u, lim);
      }
    };
    if (batch && __syncthreads_or(!ok)) {  // (uniform: batch is a template parameter)
      copy_failed();
      return;
    }
    const uint16_t *fstart = reinterpret_cast<const uint16_t *>(B + L.fstart_off);
    const int32_t *nodes = reinterpret_cast<const int32_t *>(B + L.nodes_off);
    const uint8_t *bits = B + L.bits_off;
    const int32_t *hdr = reinterpret_cast<const int32_t *>(B + L.hdr_off);
    const int nn = ok ? hdr[0] : 0, own = ok ? hdr[1] : 0;
    bool skip = false;
    if (batch) {  // the patch's instance: material, direction update, convergence mask
      lam = P.pmat[2 * patch];
      mu = P.pmat[2 * patch + 1];
      if (MODE == MV_PCG) {
        skip = !live;
        beta = T(P.isc[P.patch_inst[patch]].beta);
      }
    }
    if (!skip) {
    T *spp = sp;  // staged node values of this patch
    if constexpr (PREFETCH) {
      // 1. the gathered z and p_old of this patch: p = z + beta p_old, owned
      //    nodes written out, constrained DOFs masked, in place
      cp_async_wait<0>();
      if (__syncthreads_or(!ok)) {
        copy_failed();
        return;
      }
      spp = sp + (size_t)(it & 1) * stage_stride;
      for (int i = threadIdx.x; i < nn; i += kHfanThreads) {
        NodeV<T, VW> v = ldv<T, VW>(spp, i);
        if (beta != T(0)) {
          const NodeV<T, VW> w = ldv<T, VW>(spp + (size_t)L.npn * VW, i);
#pragma unroll
          for (int d = 0; d < DIM; ++d) v.v[d] += beta * w.v[d];
        }
        if (i >= own) {
          stv<T, VW>(P.xout, nodes[i], v);
          if (P.yzero) stv_zero<T, VW>(P.yzero, nodes[i]);
        }
        const unsigned bb = bits[i];
        NodeV<T, VW> m;
#pragma unroll
        for (int d = 0; d < VW; ++d) m.v[d] = (d < DIM && !(bb >> d & 1u)) ? v.v[d] : T(0);
        stv<T, VW>(spp, i, m);
      }
    } else {
    // 1. stage node values: each thread issues the gathers of all its nodes
    //    (up to kStageUnroll) before using any of them
    constexpr int SU = kStageUnroll;
    NodeV<T, VW> v[SU], w[SU], a3[SU];
    int gi[SU];
    auto stage_load = [&](int i0, bool with_w) {
#pragma unroll
      for (int q = 0; q < SU; ++q) {
        const int i = i0 + q * kHfanThreads;
        gi[q] = i < nn ? nodes[i] : -1;
        if (gi[q] >= 0) {
          v[q] = ldv<T, VW>(P.x, gi[q]);
          if (with_w || MODE == MV_DYN) w[q] = ldv<T, VW>(P.x2, gi[q]);
          if (MODE == MV_DYN) a3[q] = ldv<T, VW>(P.x3, gi[q]);
        }
      }
    };
    int i0 = threadIdx.x;
    bool loaded = false;
    if (defer && it == 0) {
      // first patch: this thread's first gathers, then the scalar exchange
      // (uniform); the loaded values are combined once beta is known
      stage_load(i0, true);
      if (pcg_matvec_scalars<T>(P.sc, P.up_part, P.n_up, beta, red_pcg)) {
        if (threadIdx.x == 0) {  // the copies issued above land before the CTA exits
          if (!ok) mbar_wait_bounded(&bar[b], 0u, lim);
          if (patch + step < P.n_patches) mbar_wait_bounded(&bar[b ^ 1], (phase >> (b ^ 1)) & 1u, lim);
        }
        return;
      }
      loaded = true;
    }
    for (; i0 < nn; i0 += SU * kHfanThreads, loaded = false) {
      if (!loaded) stage_load(i0, MODE == MV_PCG && beta != T(0));
#pragma unroll
      for (int q = 0; q < SU; ++q) {
        const int i = i0 + q * kHfanThreads;
        if (gi[q] < 0) continue;
        if (MODE == MV_PCG) {
          if (beta != T(0)) {
#pragma unroll
            for (int d = 0; d < DIM; ++d) v[q].v[d] += beta * w[q].v[d];
          }
          if (i >= own) {
            stv<T, VW>(P.xout, gi[q], v[q]);
            if (P.yzero) stv_zero<T, VW>(P.yzero, gi[q]);
          }
        } else if (MODE == MV_DYN) {
#pragma unroll
          for (int d = 0; d < DIM; ++d) v[q].v[d] += P.c1 * w[q].v[d] + P.c2 * a3[q].v[d];
          if (i >= own) stv<T, VW>(P.xout, gi[q], v[q]);
        }
        const unsigned bb = bits[i];
        NodeV<T, VW> m;
#pragma unroll
        for (int d = 0; d < VW; ++d) m.v[d] = (d < DIM && !(bb >> d & 1u)) ? v[q].v[d] : T(0);
        stv<T, VW>(sp, i, m);
      }
    }
    }  // PREFETCH
    if (__syncthreads_or(!ok)) {
      copy_failed();
      return;
    }
    // 2. half a fan per thread (tets 3h .. 3h+2), forces kept in registers.
    //    Missing tets have zero gradients, so the three tets are straight-line
    //    code; differences to P are formed once per node slot.
    const int fl = threadIdx.x >> 1, h = threadIdx.x & 1;
    int slot[6];
    const int nk = load_half_slots(B + L.slot_off, threadIdx.x, slot);
    T fv[6][DIM];
    {
      T du[6][DIM];  // node values of the slots (differences to P after step a)
      T dx[6][DIM];  // GEO: coordinates of the slots relative to P
      const float *Xs = reinterpret_cast<const float *>(B + (GEO ? L.x_off : 0));
#pragma unroll
      for (int k = 0; k < 6; ++k) {
        NodeV<T, VW> s, xk;
#pragma unroll
        for (int d = 0; d < VW; ++d) s.v[d] = xk.v[d] = 0;
        if (k < nk) {
          s = ldv<T, VW>(spp, slot[k]);
          if (GEO) xk = ldv<T, VW>(reinterpret_cast<const T *>(Xs), slot[k]);
        }
#pragma unroll
        for (int d = 0; d < DIM; ++d) {
          du[k][d] = s.v[d];
          dx[k][d] = xk.v[d];
          fv[k][d] = 0;
        }
      }
      if (GEO) {
#pragma unroll
        for (int k = 1; k < 6; ++k)
#pragma unroll
          for (int d = 0; d < DIM; ++d) dx[k][d] -= dx[0][d];
      }
      // gradients of tet jj of this half: from the block, or from the coordinates
      auto tet_G = [&](int jj, T (&G)[9]) {
        const int j = 3 * h + jj;
        if constexpr (GEO) {
          const float sc = L.c_off >= 0 ? reinterpret_cast<const float *>(B + L.c_off)[j * kFanThreads + fl] : 1.0f;
          geo_gradients(dx[1], dx[2 + jj], dx[3 + jj], sc, jj + 3 < nk, G);
        } else {
          load_tet_G(B + L.g_off, threadIdx.x, jj, G);
        }
      };
      if constexpr (!MASS) {
        const T lamk = lam * P.cK, muk = mu * P.cK;
#pragma unroll
        for (int k = 1; k < 6; ++k)
#pragma unroll
          for (int d = 0; d < DIM; ++d) du[k][d] -= du[0][d];
#pragma unroll
        for (int jj = 0; jj < 3; ++jj) {
          T G[9];
          tet_G(jj, G);
          tet_forces_acc<T>(du[1], du[2 + jj], du[3 + jj], G, lamk, muk, fv[1], fv[2 + jj], fv[3 + jj]);
        }
#pragma unroll
        for (int d = 0; d < DIM; ++d) fv[0][d] = -(fv[1][d] + fv[2][d] + fv[3][d] + fv[4][d] + fv[5][d]);
        if (MODE == MV_PCG) {  // p.Ap of this half-fan: the forces sum to zero, so sum_k u_k.f_k = sum_k>0 du_k.f_k
          T e_fan = 0;
#pragma unroll
          for (int k = 1; k < 6; ++k)
#pragma unroll
            for (int d = 0; d < DIM; ++d) e_fan += du[k][d] * fv[k][d];
          energy.add(e_fan);
        }
      } else {  // consistent mass term: forces do not sum to zero per tet
        const int64_t fe0 = nk ? F.fan_elem_off[F.fan_off[patch] + fl] : 0;
#pragma unroll
        for (int jj = 0; jj < 3; ++jj) {
          const int j = 3 * h + jj;
          if (jj + 3 < nk) {
            T G[9];
            tet_G(jj, G);
            T u[4][DIM], fe[4][DIM];
#pragma unroll
            for (int d = 0; d < DIM; ++d) {
              u[0][d] = du[0][d];
              u[1][d] = du[1][d];
              u[2][d] = du[2 + jj][d];
              u[3][d] = du[3 + jj][d];
            }
            element_force<T, DIM>(u, G, P.lam, P.mu, P.cK, P.cM * P.mcoef[fe0 + j], fe);
#pragma unroll
            for (int d = 0; d < DIM; ++d) {
              fv[0][d] += fe[0][d];
              fv[1][d] += fe[1][d];
              fv[2 + jj][d] += fe[2][d];
              fv[3 + jj][d] += fe[3][d];
            }
          }
        }
        if (MODE == MV_PCG) {
          T e_fan = 0;
#pragma unroll
          for (int k = 0; k < 6; ++k)
#pragma unroll
            for (int d = 0; d < DIM; ++d) e_fan += du[k][d] * fv[k][d];
          energy.add(e_fan);
        }
      }
    }
    // the force list: the consumed G region of the buffer once every thread has
    // read its gradients, or (GEO) the separate force region
    if (!GEO) __syncthreads();
    T *fs = GEO ? fgeo : reinterpret_cast<T *>(B + L.g_off);
    combine_half_forces<T, DIM>(fv, h);
#pragma unroll
    for (int k = 0; k < 6; ++k)
      if (k < nk && half_writes(h, k)) {
        NodeV<T, VW> o;
#pragma unroll
        for (int d = 0; d < VW; ++d) o.v[d] = d < DIM ? fv[k][d] : T(0);
        stv<T, VW>(fs, half_fpos(B + L.fpos_off, threadIdx.x, k), o);
      }
    if constexpr (PREFETCH) {  // the next patch's gathers overlap the node sums below
      if (patch + step < P.n_patches && mbar_wait_bounded(&bar[b ^ 1], (phase >> (b ^ 1)) & 1u, lim))
        issue_gathers(b ? buf0 : buf1, sp + (size_t)((it + 1) & 1) * stage_stride);
      cp_async_commit();
    }
    __syncthreads();
    // 3. node sums over contiguous force runs
    for (int i = threadIdx.x; i < nn; i += kHfanThreads) {
      const int g = nodes[i];
      const unsigned bb = bits[i];
      T acc3[DIM] = {0, 0, 0};
      const int k1 = fstart[i + 1];
#pragma unroll 4
      for (int k = fstart[i]; k < k1; ++k) {
        const NodeV<T, VW> fo = ldv<T, VW>(fs, k);
#pragma unroll
        for (int d = 0; d < DIM; ++d) acc3[d] += fo.v[d];
      }
      NodeV<T, VW> r;
      bool any = false;
#pragma unroll
      for (int d = 0; d < VW; ++d) {
        T val = (d < DIM && !(bb >> d & 1u)) ? acc3[d < DIM ? d : 0] : T(0);
        r.v[d] = val;
        any |= val != T(0);
      }
      if (bb && i >= own) {
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
          if (bb >> d & 1u) {
            T t = dg.v[d] * v.v[d];
            r.v[d] = t;
            any |= t != T(0);
            if (MODE == MV_PCG) energy.add(t * v.v[d]);
          }
      }
      if (any) atomic_addv<T, VW>(P.y, g, r, DIM);
    }
    }  // !skip
    if (MODE == MV_PCG && batch) {  // p.Ap per patch; summed per instance at the end
      const double t = block_total<T>(energy);
      if (threadIdx.x == 0) P.patch_energy[patch] = t;
      energy = DotAcc<T>();
    }
    // Buffer b is free again once every warp is done with it. Each thread
    // orders its own generic-proxy accesses of the buffer before the bulk copy
    // that refills it; the last warp to finish issues that copy, so the other
    // warps go on to the next patch without waiting here.
    fence_proxy_async();
    __syncwarp();
    if ((threadIdx.x & 31) == 0) {
      __threadfence_block();
      if (atomicAdd(&warps_done[b], 1u) == kHfanThreads / 32 - 1) {
        __threadfence_block();
        warps_done[b] = 0;
        if (patch + 2 * step < P.n_patches && patch_live(patch + 2 * step)) issue_copy(patch + 2 * step, b);
      }
    }
  }
  if (MODE == MV_PCG && !batch) {  // p.Ap partials; the update kernel forms sigma and alpha
    // (every warp is past the last patch's compute phase: the staging area is free)
    const DotAcc<T> ea[1] = {energy};
    store_block_partials<1, T>(ea, P.partials, red_pcg);
  } else if (MODE == MV_PCG) {  // per-instance sigma and alpha from the per-patch sums
    __shared__ bool last;
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) last = atomicAdd(&P.bctl->count_mv, 1u) == gridDim.x - 1;
    __syncthreads();
    if (!last) return;
    __threadfence();
    instance_sums<1>(P.patch_energy, 1, P.inst_patch_off, P.n_inst, P.partials, P.isc);
    __syncthreads();
    for (int i = threadIdx.x; i < P.n_inst; i += blockDim.x) {
      Scalars &si = P.isc[i];
      if (!si.done) {
        si.sigma = P.partials[i];
        si.alpha = si.gamma / si.sigma;
      }
    }
    if (threadIdx.x == 0) P.bctl->count_mv = 0;
  }
}

// Coordinates of the patch nodes relative to the patch's first node, FP32,
// into the geometry blocks (one CTA per patch; padding slots repeat node 0).
static __global__ void k_fan_block_coords(const int32_t *node_off, const int32_t *nodes, const double *coords,
                                          unsigned char *blkg, FanBlockLayout L) {
  const int p = blockIdx.x;
  const int base = node_off[p], n = node_off[p + 1] - base;
  const int g0 = nodes[base];
  float4 *X = reinterpret_cast<float4 *>(blkg + (size_t)p * L.bytes + L.x_off);
  for (int i = threadIdx.x; i < L.npn; i += blockDim.x) {
    const int g = i < n ? nodes[base + i] : g0;
    float4 v;
    v.x = (float)(coords[(size_t)g * 3 + 0] - coords[(size_t)g0 * 3 + 0]);
    v.y = (float)(coords[(size_t)g * 3 + 1] - coords[(size_t)g0 * 3 + 1]);
    v.z = (float)(coords[(size_t)g * 3 + 2] - coords[(size_t)g0 * 3 + 2]);
    v.w = 0.0f;
    X[i] = v;
  }
}

// sqrt(E_e / E) of every tet into the scale rows of the geometry blocks.
static __global__ void k_fan_block_scales(int64_t ne, const double *escale, const int32_t *fan_pos,
                                          const int32_t *fan_patch, const int32_t *fan_off, unsigned char *blkg,
                                          FanBlockLayout L) {
  int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (e >= ne) return;
  const int fp = fan_pos[e];
  const int f = fp >> 3, j = fp & 7;
  const int p = fan_patch[f];
  float *C = reinterpret_cast<float *>(blkg + (size_t)p * L.bytes + L.c_off);
  C[j * kFanThreads + (f - fan_off[p])] = (float)sqrt(escale[e]);
}

// Scaled gradients into the G part of the FP32 patch blocks from the
// element-order FP64 gradients, in fan vertex order.
static __global__ void k_fan_block_gradients(int64_t ne, const double *G64, int64_t gstride, const int32_t *fan_pos,
                                             const uint8_t *fan_perm, const int32_t *fan_patch, const int32_t *fan_off,
                                             unsigned char *blk32, FanBlockLayout L32) {
  int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (e >= ne) return;
  double g[4][3];
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    double s0 = 0;
#pragma unroll
    for (int a = 1; a < 4; ++a) {
      g[a][d] = G64[(size_t)((a - 1) * 3 + d) * gstride + e];
      s0 += g[a][d];
    }
    g[0][d] = -s0;
  }
  const int fp = fan_pos[e];
  const int f = fp >> 3, j = fp & 7;
  const int p = fan_patch[f];
  const int fl = f - fan_off[p];
  const int t = 2 * fl + j / 3, jj = j % 3;  // half-thread and its tet
  unsigned char *G32b = blk32 + (size_t)p * L32.bytes + L32.g_off;
  const unsigned perm = fan_perm[e];
#pragma unroll
  for (int b = 1; b < 4; ++b) {
    const int a = (perm >> (2 * b)) & 3u;
#pragma unroll
    for (int d = 0; d < 3; ++d)
      *reinterpret_cast<float *>(G32b + tet_G_offset(t, jj, (b - 1) * 3 + d)) = (float)g[a][d];
  }
}

}  // namespace cfem
