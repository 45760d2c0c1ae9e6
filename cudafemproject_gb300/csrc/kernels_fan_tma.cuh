// Edge-fan EbE matvec with the per-patch data streamed by bulk asynchronous
// copies. Two threads share a fan: half h evaluates tets 3h .. 3h+2 and owns
// the six node slots P, Q, R_3h .. R_3h+3 (kHalfSlots = 12 force slots per fan).
// Everything a patch needs apart from the node vectors lives in one
// contiguous, 128-byte aligned block of the "patch block" array:
//   [slot: kFanSlots x kFanThreads u16]   patch-local nodes P, Q, R_0.. of each fan, then its length
//   [fpos: kHalfSlots x kFanThreads u16]  position of each (fan, half slot) force in the node-sorted list
//   [fstart: nps u16]                      node i sums forces fstart[i] .. fstart[i+1]-1
//   [nodes: npn i32] [bits: npn u8]        global node ids and constraint bits of the patch nodes
//   [G: 9 kFanMax x kFanThreads T]         scaled gradients in fan vertex order, row (j*9 + (b-1)*3 + d)
// One copy per patch, issued two patches ahead into a double buffer, so the
// operator stream overlaps the arithmetic of the current patch. The forces of
// a patch are written into the G region of its own buffer once every thread
// has read its gradients, and the node sums read them back contiguously.
#pragma once

#include "kernels.cuh"
#include "prep.hpp"
#include "tma.cuh"

namespace cfem {

constexpr int kStageUnroll = 2;      // node gathers in flight per thread while staging a patch
constexpr int kHalfSlots = 12;       // force slots per fan: 2 halves x (P, Q, 4 ring vertices)
constexpr int kHfanThreads = 2 * kFanThreads;

// fan slot (0 = P, 1 = Q, 2 + k = R_k) of half h's slot hs
__host__ __device__ __forceinline__ int half_slot_to_fan(int h, int hs) { return hs < 2 ? hs : hs + 3 * h; }
// number of valid slots of half h of a fan of length len (0 if the half has no tet)
__host__ __device__ __forceinline__ int half_slot_count(int h, int len) {
  return len > 3 * h ? 3 + (len - 3 * h < 3 ? len - 3 * h : 3) : 0;
}

struct FanBlockLayout {
  int bytes;        // per patch, multiple of 128
  int slot_off, fpos_off, fstart_off, nodes_off, bits_off, g_off;
  int nps, npn;     // fstart entries, node entries per patch
};

inline FanBlockLayout fan_block_layout(int np_max, size_t tsize) {
  FanBlockLayout L{};
  auto up = [](int x, int a) { return (x + a - 1) / a * a; };
  L.nps = up(np_max + 1, 8);
  L.npn = up(np_max, 4);
  int off = 0;
  L.slot_off = off; off += kFanSlots * kFanThreads * 2;
  L.fpos_off = off; off += kHalfSlots * kFanThreads * 2;
  L.fstart_off = off; off += L.nps * 2;
  L.nodes_off = off; off += L.npn * 4;
  L.bits_off = off; off += up(L.npn, 16);
  L.g_off = up(off, 128);
  L.bytes = up(L.g_off + (int)(kFanMax * 9 * kFanThreads * tsize), 128);
  return L;
}

inline size_t fan_tma_smem_bytes(const FanBlockLayout &L, size_t tsize) {
  return (size_t)2 * L.bytes + (size_t)L.npn * 4 * tsize + 16;
}

struct FanTmaParams {
  const unsigned char *blocks;  // [n_patches][L.bytes]
  FanBlockLayout L;
  const int32_t *fan_off;       // [n_patches + 1]
  const int32_t *fan_elem_off;  // [n_fans + 1] (consistent-mass coefficients)
  int *err;                     // kErrTmaTimeout on a copy that never completed
};

template <typename T, int MODE>
// (3 CTAs per SM: the shared memory of a CTA allows 3, the register bound makes them fit)
__global__ void __launch_bounds__(kHfanThreads, 3) k_matvec_fan_tma(MvParams<T> P, FanTmaParams F) {
  constexpr int DIM = 3, VW = 4;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  const FanBlockLayout &L = F.L;
  unsigned char *buf0 = smem_raw, *buf1 = smem_raw + L.bytes;
  T *sp = reinterpret_cast<T *>(smem_raw + 2 * (size_t)L.bytes);  // [npn][4] staged node values
  uint64_t *bar = reinterpret_cast<uint64_t *>(sp + (size_t)L.npn * VW);
  const bool batch = P.patch_inst != nullptr;
  if (MODE == MV_PCG && (batch ? P.bctl->all_done : P.sc->done)) return;
  T beta = 0;
  if (MODE == MV_PCG && !batch) beta = T(P.sc->beta);
  T lam = P.lam, mu = P.mu;
  if (threadIdx.x == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    fence_mbar_init();
  }
  __syncthreads();
  const int step = gridDim.x;
  if (threadIdx.x == 0) {
    for (int k = 0; k < 2; ++k) {
      const int q = blockIdx.x + k * step;
      if (q < P.n_patches) {
        mbar_expect_tx(&bar[k], (unsigned)L.bytes);
        bulk_load(k ? buf1 : buf0, F.blocks + (size_t)q * L.bytes, (unsigned)L.bytes, &bar[k]);
      }
    }
  }
  DotAcc<T> energy;
  int it = 0;
  for (int patch = blockIdx.x; patch < P.n_patches; patch += step, ++it) {
    const int b = it & 1;
    unsigned char *B = b ? buf1 : buf0;
    const bool ok = mbar_wait_bounded(&bar[b], (unsigned)((it >> 1) & 1));
    if (__syncthreads_or(!ok)) {
      if (threadIdx.x == 0) {
        atomicOr(F.err, kErrTmaTimeout);
        if (patch + step < P.n_patches) mbar_wait_bounded(&bar[b ^ 1], (unsigned)(((it + 1) >> 1) & 1));
      }
      return;
    }
    const uint16_t *sl = reinterpret_cast<const uint16_t *>(B + L.slot_off);
    const uint16_t *fpos = reinterpret_cast<const uint16_t *>(B + L.fpos_off);
    const uint16_t *fstart = reinterpret_cast<const uint16_t *>(B + L.fstart_off);
    const int32_t *nodes = reinterpret_cast<const int32_t *>(B + L.nodes_off);
    const uint8_t *bits = B + L.bits_off;
    const T *Gs = reinterpret_cast<const T *>(B + L.g_off);
    const int nn = P.node_off[patch + 1] - P.node_off[patch], own = P.own[patch];
    const int nf = F.fan_off[patch + 1] - F.fan_off[patch];
    bool skip = false;
    if (batch) {  // the patch's instance: material, direction update, convergence mask
      lam = P.pmat[2 * patch];
      mu = P.pmat[2 * patch + 1];
      if (MODE == MV_PCG) {
        const Scalars &si = P.isc[P.patch_inst[patch]];
        skip = si.done != 0;
        beta = T(si.beta);
      }
    }
    if (!skip) {
    // 1. stage node values: each thread issues the gathers of all its nodes
    //    (up to kStageUnroll) before using any of them
    constexpr int SU = kStageUnroll;
    for (int i0 = threadIdx.x; i0 < nn; i0 += SU * kHfanThreads) {
      NodeV<T, VW> v[SU], w[SU], a3[SU];
      int gi[SU];
#pragma unroll
      for (int q = 0; q < SU; ++q) {
        const int i = i0 + q * kHfanThreads;
        gi[q] = i < nn ? nodes[i] : -1;
        if (gi[q] >= 0) {
          v[q] = ldv<T, VW>(P.x, gi[q]);
          if ((MODE == MV_PCG && beta != T(0)) || MODE == MV_DYN) w[q] = ldv<T, VW>(P.x2, gi[q]);
          if (MODE == MV_DYN) a3[q] = ldv<T, VW>(P.x3, gi[q]);
        }
      }
#pragma unroll
      for (int q = 0; q < SU; ++q) {
        const int i = i0 + q * kHfanThreads;
        if (gi[q] < 0) continue;
        if (MODE == MV_PCG) {
          if (beta != T(0)) {
#pragma unroll
            for (int d = 0; d < DIM; ++d) v[q].v[d] += beta * w[q].v[d];
          }
          if (i >= own) stv<T, VW>(P.xout, gi[q], v[q]);
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
    __syncthreads();
    // 2. half a fan per thread (tets 3h .. 3h+2), forces kept in registers.
    //    Missing tets have zero gradients in the block, so the three tets are
    //    straight-line code; differences to P are formed once per node slot.
    const int fl = threadIdx.x >> 1, h = threadIdx.x & 1;
    const int len = fl < nf ? sl[(kFanSlots - 1) * kFanThreads + fl] : 0;
    const int nk = half_slot_count(h, len);
    T fv[6][DIM];
    {
      T uv[6][DIM];
#pragma unroll
      for (int k = 0; k < 6; ++k) {
        NodeV<T, VW> s;
#pragma unroll
        for (int d = 0; d < VW; ++d) s.v[d] = 0;
        if (k < nk) s = ldv<T, VW>(sp, sl[half_slot_to_fan(h, k) * kFanThreads + fl]);
#pragma unroll
        for (int d = 0; d < DIM; ++d) {
          uv[k][d] = s.v[d];
          fv[k][d] = 0;
        }
      }
      if (P.mcoef == nullptr) {
        const T lamk = lam * P.cK, muk = mu * P.cK;
        T du[6][DIM];
#pragma unroll
        for (int k = 1; k < 6; ++k)
#pragma unroll
          for (int d = 0; d < DIM; ++d) du[k][d] = uv[k][d] - uv[0][d];
#pragma unroll
        for (int jj = 0; jj < 3; ++jj) {
          const int j = 3 * h + jj;
          T G[9];
#pragma unroll
          for (int k = 0; k < 9; ++k) G[k] = Gs[(j * 9 + k) * kFanThreads + fl];
          T f1[3], f2[3], f3[3];
          tet_forces_rel<T>(du[1], du[2 + jj], du[3 + jj], G, lamk, muk, f1, f2, f3);
#pragma unroll
          for (int d = 0; d < DIM; ++d) {
            fv[1][d] += f1[d];
            fv[2 + jj][d] += f2[d];
            fv[3 + jj][d] += f3[d];
          }
        }
#pragma unroll
        for (int d = 0; d < DIM; ++d) fv[0][d] = -(fv[1][d] + fv[2][d] + fv[3][d] + fv[4][d] + fv[5][d]);
      } else {  // consistent mass term: forces do not sum to zero per tet
        const int64_t fe0 = nk ? F.fan_elem_off[F.fan_off[patch] + fl] : 0;
#pragma unroll
        for (int jj = 0; jj < 3; ++jj) {
          const int j = 3 * h + jj;
          if (nk && j < len) {
            T G[9];
#pragma unroll
            for (int k = 0; k < 9; ++k) G[k] = Gs[(j * 9 + k) * kFanThreads + fl];
            T u[4][DIM], fe[4][DIM];
#pragma unroll
            for (int d = 0; d < DIM; ++d) {
              u[0][d] = uv[0][d];
              u[1][d] = uv[1][d];
              u[2][d] = uv[2 + jj][d];
              u[3][d] = uv[3 + jj][d];
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
      }
      if (MODE == MV_PCG) {  // p.Ap of this half-fan: sum over its node slots of u . f
        T e_fan = 0;
#pragma unroll
        for (int k = 0; k < 6; ++k)
#pragma unroll
          for (int d = 0; d < DIM; ++d) e_fan += uv[k][d] * fv[k][d];
        energy.add(e_fan);
      }
    }
    __syncthreads();  // every thread has read its gradients: the G region becomes the force list
    T *fs = reinterpret_cast<T *>(B + L.g_off);
#pragma unroll
    for (int k = 0; k < 6; ++k)
      if (k < nk) {
        NodeV<T, VW> o;
#pragma unroll
        for (int d = 0; d < VW; ++d) o.v[d] = d < DIM ? fv[k][d] : T(0);
        stv<T, VW>(fs, fpos[(h * 6 + k) * kFanThreads + fl], o);
      }
    __syncthreads();
    // 3. node sums over contiguous force runs
    for (int i = threadIdx.x; i < nn; i += kHfanThreads) {
      const int g = nodes[i];
      const unsigned bb = bits[i];
      T acc[DIM] = {0, 0, 0};
      const int k1 = fstart[i + 1];
      for (int k = fstart[i]; k < k1; ++k) {
        const NodeV<T, VW> fo = ldv<T, VW>(fs, k);
#pragma unroll
        for (int d = 0; d < DIM; ++d) acc[d] += fo.v[d];
      }
      NodeV<T, VW> r;
      bool any = false;
#pragma unroll
      for (int d = 0; d < VW; ++d) {
        T val = (d < DIM && !(bb >> d & 1u)) ? acc[d < DIM ? d : 0] : T(0);
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
    // Buffer b is free again. Every thread orders its own generic-proxy
    // accesses of it (the force stores and reads) before the bulk copy that
    // refills it, then the barrier makes that true for all of them.
    fence_proxy_async();
    __syncthreads();
    if (threadIdx.x == 0 && patch + 2 * step < P.n_patches) {
      mbar_expect_tx(&bar[b], (unsigned)L.bytes);
      bulk_load(B, F.blocks + (size_t)(patch + 2 * step) * L.bytes, (unsigned)L.bytes, &bar[b]);
    }
  }
  if (MODE == MV_PCG && !batch) {
    DotAcc<T> ea[1] = {energy};
    double v[1];
    if (grid_sum_acc<1, T>(ea, v, P.partials, &P.sc->count_mv)) {
      P.sc->sigma = v[0];
      P.sc->alpha = P.sc->gamma / v[0];
    }
  } else if (MODE == MV_PCG) {  // per-instance sigma and alpha from the per-patch sums
    __shared__ bool last;
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) last = atomicAdd(&P.bctl->count_mv, 1u) == gridDim.x - 1;
    __syncthreads();
    if (!last) return;
    __threadfence();
    instance_sums<1>(P.patch_energy, 1, P.inst_patch_off, P.n_inst, P.partials);
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
  float *G32b = reinterpret_cast<float *>(blk32 + (size_t)p * L32.bytes + L32.g_off);
  const unsigned perm = fan_perm[e];
#pragma unroll
  for (int b = 1; b < 4; ++b) {
    const int a = (perm >> (2 * b)) & 3u;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      const int row = j * 9 + (b - 1) * 3 + d;
      G32b[row * kFanThreads + fl] = (float)g[a][d];
    }
  }
}

}  // namespace cfem
