// EbE matvec over edge fans (3D): one thread evaluates a whole fan of up to
// kFanMax tets sharing the edge PQ, tet j being {P, Q, R_j, R_j+1}. The fan's
// node values are read from shared memory once per fan (len + 3 reads instead
// of 4 per tet) and its forces are summed in registers, so a fan of 6 tets
// writes 9 force slots instead of 24. The scaled gradients are stored per fan
// in fan vertex order: Gf[(j*9 + (b-1)*3 + d)][f] = grad N_b of tet j, b = 1..3
// (vertex 0 = P implicitly minus their sum).
#pragma once

#include "kernels.cuh"
#include "prep.hpp"

namespace cfem {

struct FanParams {
  const int32_t *fan_off;       // [n_patches + 1] first fan of each patch
  const int32_t *fan_elem_off;  // [n_fans + 1] first element of each fan (new element order)
  const uint16_t *slot;         // [kFanSlots][fstride]: patch-local nodes P, Q, R_0.., then the length
  const uint16_t *finc;         // per patch: incidence codes fl*16 + slot, sorted by node
  const uint16_t *finc_start;   // per patch: nn + 1 offsets into the patch's codes
  int64_t fstride;
};

// Shared-memory bytes of k_matvec_fan.
inline size_t fan_smem_bytes(size_t tsize, int np_max) {
  constexpr int NS = kFanMax + 3;
  return (size_t)np_max * 4 * tsize + (size_t)NS * kFanThreads * 4 * tsize + (size_t)kFanSlots * kFanThreads * 2 +
         (size_t)((np_max + 2) & ~1) * 2 + (size_t)np_max * 5;
}

// Same contract and phases as k_matvec (kernels.cuh), with the element phase
// done fan by fan.
template <typename T, int MODE>
__global__ void __launch_bounds__(kFanThreads) k_matvec_fan(MvParams<T> P, FanParams F, const T *__restrict__ Gf) {
  constexpr int DIM = 3, VW = 4, NS = kFanMax + 3;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T *sp = reinterpret_cast<T *>(smem_raw);                                             // [np_max][4]
  T *fs = sp + (size_t)P.np_max * VW;                                                  // [NS][kFanThreads][4]
  uint16_t *si = reinterpret_cast<uint16_t *>(fs + (size_t)NS * kFanThreads * VW);  // [kFanSlots * kFanThreads]
  uint16_t *ss = si + kFanSlots * kFanThreads;                                         // [np_max + 1]
  int32_t *sg = reinterpret_cast<int32_t *>(ss + ((P.np_max + 2) & ~1));              // [np_max]
  uint8_t *sb = reinterpret_cast<uint8_t *>(sg + P.np_max);                            // [np_max]
  __shared__ double red_pcg[24];
  T beta = 0;
  if (MODE == MV_PCG && pcg_matvec_scalars<T>(P.sc, P.up_part, P.n_up, beta, red_pcg)) return;
  DotAcc<T> energy;
  for (int patch = blockIdx.x; patch < P.n_patches; patch += gridDim.x) {
    const int nb = P.node_off[patch], nn = P.node_off[patch + 1] - nb, own = P.own[patch];
    const int f0 = F.fan_off[patch], nf = F.fan_off[patch + 1] - f0;
    const T lam = P.patch_inst ? P.pmat[2 * patch] : P.lam, mu = P.patch_inst ? P.pmat[2 * patch + 1] : P.mu;
    // 1. stage: incidence codes (kFanSlots per fan, 4-byte aligned), offsets, node values
    {
      const uint32_t *src = reinterpret_cast<const uint32_t *>(F.finc + (size_t)kFanSlots * f0);
      for (int q = threadIdx.x; q < nf * kFanSlots / 2; q += blockDim.x) reinterpret_cast<uint32_t *>(si)[q] = src[q];
      for (int i = threadIdx.x; i <= nn; i += blockDim.x) ss[i] = F.finc_start[nb + patch + i];
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
    // 2. fans: differences to P once per fan node, each tet's stiffness forces
    //    accumulated into the forces on Q, R_j, R_j+1 (tet_forces_acc); the
    //    force on P is minus the sum of the others (the stiffness forces of a
    //    tet sum to zero), plus the mass forces when there is a mass term
    for (int fl = threadIdx.x; fl < nf; fl += blockDim.x) {
      const int64_t f = f0 + fl;
      const int len = F.slot[(size_t)(kFanSlots - 1) * F.fstride + f];
      T u0[DIM], du[NS][DIM], fv[NS][DIM], corr[DIM];
      {
        const NodeV<T, VW> s0 = ldv<T, VW>(sp, F.slot[f]);
#pragma unroll
        for (int d = 0; d < DIM; ++d) {
          u0[d] = s0.v[d];
          corr[d] = 0;
        }
      }
#pragma unroll
      for (int k = 1; k < NS; ++k) {
        NodeV<T, VW> s;
#pragma unroll
        for (int d = 0; d < VW; ++d) s.v[d] = 0;
        if (k < len + 3) s = ldv<T, VW>(sp, F.slot[(size_t)k * F.fstride + f]);
#pragma unroll
        for (int d = 0; d < DIM; ++d) {
          du[k][d] = s.v[d] - u0[d];
          fv[k][d] = 0;
        }
      }
      const int64_t fe0 = P.mcoef ? F.fan_elem_off[f] : 0;
      const T lamk = P.cK * lam, muk = P.cK * mu;
#pragma unroll
      for (int j = 0; j < kFanMax; ++j) {
        if (j < len) {
          T G[9];
#pragma unroll
          for (int k = 0; k < 9; ++k) G[k] = Gf[(size_t)(j * 9 + k) * F.fstride + f];
          tet_forces_acc<T>(du[1], du[2 + j], du[3 + j], G, lamk, muk, fv[1], fv[2 + j], fv[3 + j]);
          if (P.mcoef) {  // f_a += m (u_a + sum_b u_b) on all four vertices
            const T mc = P.cM * P.mcoef[fe0 + j];
#pragma unroll
            for (int d = 0; d < DIM; ++d) {
              const T a0 = u0[d], a1 = du[1][d] + u0[d], a2 = du[2 + j][d] + u0[d], a3 = du[3 + j][d] + u0[d];
              const T sum = a0 + a1 + a2 + a3;
              const T m0 = mc * (a0 + sum), m1 = mc * (a1 + sum), m2 = mc * (a2 + sum), m3 = mc * (a3 + sum);
              fv[1][d] += m1;
              fv[2 + j][d] += m2;
              fv[3 + j][d] += m3;
              corr[d] += m0 + m1 + m2 + m3;
            }
          }
        }
      }
      // P: corr - sum of the others; p.Ap of the fan = u_P.corr + sum_k du_k.f_k
      T fP[DIM], e_fan = 0;
#pragma unroll
      for (int d = 0; d < DIM; ++d) {
        T t = 0;
#pragma unroll
        for (int k = 1; k < NS; ++k) t += fv[k][d];
        fP[d] = corr[d] - t;
        if (MODE == MV_PCG) {
          e_fan += u0[d] * corr[d];
#pragma unroll
          for (int k = 1; k < NS; ++k) e_fan += du[k][d] * fv[k][d];
        }
      }
      {
        NodeV<T, VW> o;
#pragma unroll
        for (int d = 0; d < VW; ++d) o.v[d] = d < DIM ? fP[d] : T(0);
        stv<T, VW>(fs, fl, o);
      }
#pragma unroll
      for (int k = 1; k < NS; ++k)
        if (k < len + 3) {
          NodeV<T, VW> o;
#pragma unroll
          for (int d = 0; d < VW; ++d) o.v[d] = d < DIM ? fv[k][d] : T(0);
          stv<T, VW>(fs, (size_t)k * kFanThreads + fl, o);
        }
      if (MODE == MV_PCG) energy.add(e_fan);
    }
    __syncthreads();
    // 3. nodes
    for (int i = threadIdx.x; i < nn; i += blockDim.x) {
      const int g = sg[i];
      const unsigned b = sb[i];
      T acc[DIM] = {0, 0, 0};
      const int k1 = ss[i + 1];
      for (int k = ss[i]; k < k1; ++k) {
        const unsigned code = si[k];
        const NodeV<T, VW> fo = ldv<T, VW>(fs, (size_t)(code & 15u) * kFanThreads + (code >> 4));
#pragma unroll
        for (int d = 0; d < DIM; ++d) acc[d] += fo.v[d];
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

// Scaled gradients in fan vertex order from the element-order FP64 gradients
// (G[(a-1)*3+d][e], vertex 0 = minus the sum): Gf[(j*9+(b-1)*3+d)][f] =
// grad N of the element vertex that is fan vertex b.
static __global__ void k_fan_gradients(int64_t ne, const double *G64, int64_t gstride, const int32_t *fan_pos,
                                const uint8_t *fan_perm, double *Gf64, float *Gf32, int64_t fstride) {
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
  const int64_t f = fp >> 3;
  const int j = fp & 7;
  const unsigned perm = fan_perm[e];
#pragma unroll
  for (int b = 1; b < 4; ++b) {
    const int a = (perm >> (2 * b)) & 3u;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      const size_t idx = (size_t)(j * 9 + (b - 1) * 3 + d) * fstride + f;
      Gf64[idx] = g[a][d];
      Gf32[idx] = (float)g[a][d];
    }
  }
}

}  // namespace cfem
