// Internals shared by the C-ABI translation units (context.cu, context_dyn.cu).
#pragma once

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <memory>
#include <string>
#include <vector>

#include "../../include/cfem.h"
#include "kernels.cuh"
#include "kernels_fan.cuh"
#include "kernels_fan_tma.cuh"
#include "kernels_multi.cuh"
#include "kernels_batch.cuh"
#include "prep.hpp"

namespace cfem {
namespace detail {

extern thread_local std::string g_last_error;

struct MultiState;                    // multi-RHS work arrays (context_multi.cu)
void destroy_multi(MultiState *m);

struct Fail {
  cfem_status st;
  std::string msg;
};

#define CK(call)                                                                                   \
  do {                                                                                             \
    cudaError_t e_ = (call);                                                                       \
    if (e_ != cudaSuccess)                                                                         \
      throw Fail{e_ == cudaErrorMemoryAllocation ? CFEM_ERR_OUT_OF_MEMORY : CFEM_ERR_CUDA,          \
                 std::string(#call) + ": " + cudaGetErrorString(e_)};                              \
  } while (0)

#define CKL() CK(cudaGetLastError())

template <typename T>
struct DBuf {
  T *p = nullptr;
  size_t n = 0;
  DBuf() = default;
  DBuf(const DBuf &) = delete;
  DBuf &operator=(const DBuf &) = delete;
  ~DBuf() { release(); }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
  }
  void alloc(size_t count) {
    release();
    if (count == 0) return;
    CK(cudaMalloc(&p, count * sizeof(T)));
    n = count;
  }
  void zero(cudaStream_t s) {
    if (p) CK(cudaMemsetAsync(p, 0, n * sizeof(T), s));
  }
  void upload(const T *h, size_t count, cudaStream_t s) {
    alloc(count);
    if (count) CK(cudaMemcpyAsync(p, h, count * sizeof(T), cudaMemcpyHostToDevice, s));
  }
};

template <typename T>
struct Vecs {
  DBuf<T> x, r, z, pA, pB, u, uB, f, dinv, diagA;  // u, uB: A p of even, odd PCG iterations
};

inline int pcg_chunk_from_env() {
  const char *e = std::getenv("CFEM_PCG_CHUNK");
  const int v = e ? std::atoi(e) : 16;
  return v < 2 ? 16 : (v + 1) & ~1;
}

struct GraphCache {
  cudaGraphExec_t exec = nullptr;
  bool device_loop = false;  // exec is a WHILE node around the iterations (one launch per solve)
  const void *key0 = nullptr;
  double key1 = 0, key2 = 0;
  ~GraphCache() { reset(); }
  void reset() {
    if (exec) cudaGraphExecDestroy(exec);
    exec = nullptr;
  }
};

inline unsigned nblk(int64_t n, int t = kThreads) { return (unsigned)((n + t - 1) / t); }

}  // namespace detail
}  // namespace cfem

using namespace cfem;
using namespace cfem::detail;

struct cfem_ctx {
  cudaStream_t stream = nullptr;       // the stream all work is issued on (capturable)
  cudaStream_t user_stream = nullptr;  // the caller's stream; work is ordered after it
  bool own_stream = false;
  cudaEvent_t ev_in = nullptr;
  int device = 0, n_sm = 0, l2_bytes = 0;
  int grid_upd = 0;  // PCG update kernel (3D)
  int dim = 0, nv = 0, w = 0, vw = 0, ncomp = 0;
  int64_t nn = 0, ne = 0, nd = 0, nvec = 0;
  int semantics = 0, form = CFEM_FORM_GRADIENT, verbose = 0;
  double E = 0, nu = 0, rho = 0, lam = 0, mu = 0;
  Prep prep;
  RhsParts rhs;
  std::vector<double> young;  // per-element Young's modulus (caller order), empty if uniform
  std::vector<int32_t> elems_caller;  // caller connectivity (reference slot order for the re-sorting quirk)
  double lump_c = 0, cons_c = 0;
  // mesh on device
  DBuf<int32_t> elem_off, node_off, nodes, own, node_new2old, elem_new2old, elem_old2new, conn;
  DBuf<uint2> lconn;
  DBuf<uint16_t> inc, inc_start;  // per-patch incidence lists
  // edge-fan form (3D): fan tables, gradients in fan vertex order
  bool fans = false;
  int64_t fstride = 0;
  DBuf<int32_t> fan_off, fan_elem_off, fan_pos;
  DBuf<uint16_t> fan_slot, finc, finc_start;
  DBuf<uint8_t> fan_perm;
  DBuf<double> Gf64;
  DBuf<float> Gf32;
  size_t smem_fan64 = 0, smem_fan32 = 0;
  int grid_fan = 0;
  // edge-fan form, FP32, with bulk-copied patch blocks (kernels_fan_tma.cuh)
  bool fan_tma = true;
  FanBlockLayout L32{};
  DBuf<unsigned char> blk32;
  DBuf<int32_t> fan_patch;
  DBuf<int> tma_err;
  int *h_tma_err = nullptr;
  int selftest_skip_plus1 = 0;       // FanTmaParams::skip_patch_plus1 (cfem_selftest_copy_timeout only)
  long long selftest_wait_limit = 0;  // FanTmaParams::wait_limit (likewise)
  size_t smem_ft32 = 0;
  int grid_ft32 = 0;
  // geometry blocks (FP32 single-RHS matvec of CFEM_FORM_GEOMETRY_FAN): the
  // prefix of blk32, then patch-relative coordinates and per-tet moduli scales
  bool geo = false;
  FanBlockLayout Lg{};
  DBuf<unsigned char> blkg;
  size_t smem_geo = 0;
  int grid_geo = 0;
  int np_slots = 0;               // node slots per patch in shared memory
  DBuf<uint8_t> bits;
  DBuf<double> coords, escale, young_d;
  // operator
  int64_t gstride = 0;
  DBuf<double> G64, vol, diagK, mlump, mcdiag, mc64;
  DBuf<float> G32, mc32, diagK32;
  DBuf<double> FA, FB;
  DBuf<float> FA32, FB32;
  // work
  Vecs<double> v64;
  Vecs<float> v32;
  DBuf<double> io, tmp64, tmp64b, rr;
  DBuf<Scalars> sc;  // [0] FP64 solve, [1] FP32 solve, [2] misc counters
  DBuf<double> partials;     // grid-sum scratch; the PCG-form matvec's p.Ap partials
  DBuf<double> partials_up;  // r.z, r.r partials of the PCG update kernel [grid][2]
  DBuf<unsigned int> counters;
  DBuf<int> err;
  Scalars *h_sc = nullptr;
  double *h_rr = nullptr;
  int grid_mv = 0, grid_vec = 0;
  size_t smem64 = 0, smem32 = 0;
  // PCG iterations per graph body (even: the A p buffers alternate);
  // CFEM_PCG_CHUNK overrides it (rounded up to even)
  int chunk = pcg_chunk_from_env();
  // run the PCG iterations from the host, `chunk` per graph launch, instead of
  // inside a graph WHILE node (CFEM_HOST_LOOP set in the environment)
  bool host_loop = std::getenv("CFEM_HOST_LOOP") != nullptr;
  MultiState *multi = nullptr;
  // batch of independent meshes (cfem_create_batch); n_inst == 0 for one mesh
  int n_inst = 0;
  std::vector<int32_t> elem_group;               // caller element -> instance
  std::vector<double> inst_lam, inst_mu;
  std::vector<int64_t> inst_node_off, inst_elem_off;  // caller order
  DBuf<int32_t> patch_inst, inst_patch_off, own_first;
  DBuf<float> pmat32;
  DBuf<double> pmat64, lam_e, mu_e;
  int64_t launches = 0;  // kernels issued since the counter was last reset
  GraphCache graph64, graph32;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  // reference re-sorting quirk (compat dynamics)
  DBuf<int64_t> seg;
  DBuf<int32_t> perm, node_old2new;
  DBuf<double> slot_src, slot_tmp;

  ~cfem_ctx() {
    graph64.reset();
    graph32.reset();
    if (h_sc) cudaFreeHost(h_sc);
    if (h_rr) cudaFreeHost(h_rr);
    if (h_tma_err) cudaFreeHost(h_tma_err);
    if (multi) destroy_multi(multi);
    if (ev0) cudaEventDestroy(ev0);
    if (ev1) cudaEventDestroy(ev1);
    if (ev_in) cudaEventDestroy(ev_in);
    if (own_stream && stream) cudaStreamDestroy(stream);
  }
};


namespace cfem {
namespace detail {

// FP32_REFINE inner tolerances from which the inner PCG carries its search
// direction across the refinement steps (the tolerance is then the factor by
// which its recursive residual drops between FP64 true-residual replacements).
constexpr double kContinueTol = 0.2;
// A refinement step whose FP64 residual norm^2 falls by less than this is at
// the FP64 floor: a step cuts the norm by about the inner tolerance tol (at
// least halves it for tol up to 0.25), so the test allows twice that.
inline double refine_stall_ratio(double tol) { return std::min(0.9, std::max(0.25, 4.0 * tol * tol)); }

struct PcgResult {
  int status = CFEM_OK;
  int iters = 0;
  double gamma0 = 0, gamma = 0, rr = 0, ff = 0;
  double gamma_prev = 0;  // the gamma of the last step length (alpha = gamma_prev / p.Ap)
};

MvParams<double> base_mv_d(cfem_ctx *c);
MvParams<float> base_mv_f(cfem_ctx *c);
void launch_mv_d(cfem_ctx *c, int mode, const MvParams<double> &P);
void launch_mv_f(cfem_ctx *c, int mode, const MvParams<float> &P);
PcgResult run_pcg_d(cfem_ctx *c, Vecs<double> &V, double cK, double cM, const double *mcoef, int warm, double tol,
                    int rule, int maxit);
PcgResult run_pcg_f(cfem_ctx *c, Vecs<float> &V, float cK, float cM, const float *mcoef, int warm, double tol,
                    int rule, int maxit);
void to_internal_d(cfem_ctx *c, const double *src, double *dst, double scale = 1.0);
void to_internal_f(cfem_ctx *c, const double *src, float *dst, double scale = 1.0);
void to_caller_d(cfem_ctx *c, const double *src, double *dst);
void to_caller_f(cfem_ctx *c, const float *src, double *dst);
void set_diag_vectors(cfem_ctx *c, const double *diagA64);
void true_residual(cfem_ctx *c, const double *f, const double *x, double *r, float *r32, double &rr, double &ff);
void true_residual_async(cfem_ctx *c, const double *f, const double *x, double *r, float *r32, double *out2);
void make_rhs(cfem_ctx *c, double a, double b, double *dst);
cfem_status run_guarded(const std::function<cfem_status()> &fn);
void check_ctx(const cfem_ctx *c);
// Throws if a bulk-copy wait of the edge-fan matvec timed out (synchronises the stream).
// Launch with programmatic stream serialization: the kernel may start while
// the previous kernel in the stream runs (it calls griddep_wait before reading
// that kernel's results). Used for the matvec / update pairs of the PCG loop
// and the kernels of an explicit dynamics step. Every kernel launched this
// way waits for its predecessor before it finishes, so completion stays
// ordered along the stream.
template <typename... KArgs, typename... Args>
inline void launch_pdl(void (*kern)(KArgs...), dim3 g, dim3 b, size_t smem, cudaStream_t s, Args... args) {
  cudaLaunchConfig_t cfg{};
  cfg.gridDim = g;
  cfg.blockDim = b;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  CK(cudaLaunchKernelEx(&cfg, kern, args...));
}

void check_copy_error(cfem_ctx *c);
// Orders the context's stream after the caller's stream (device inputs written there).
void enter(cfem_ctx *c);
cfem_solve_params default_params();
cfem_status solve_internal(cfem_ctx *c, const cfem_solve_params *prm, cfem_solve_info *info);
void rebuild_operator(cfem_ctx *c);
void setup_context(cfem_ctx *c, const cfem_mesh *m, const cfem_material *mat, const cfem_options *opt);
void attach_stream(cfem_ctx *c, cudaStream_t s);

template <typename T>
inline MvParams<T> base_mv(cfem_ctx *c) {
  if constexpr (sizeof(T) == 8) return base_mv_d(c); else return base_mv_f(c);
}
template <typename T>
inline void launch_mv(cfem_ctx *c, int mode, const MvParams<T> &P) {
  if constexpr (sizeof(T) == 8) launch_mv_d(c, mode, P); else launch_mv_f(c, mode, P);
}
template <typename T>
inline PcgResult run_pcg(cfem_ctx *c, Vecs<T> &V, T cK, T cM, const T *mcoef, int warm, double tol, int rule, int maxit) {
  if constexpr (sizeof(T) == 8) return run_pcg_d(c, V, cK, cM, mcoef, warm, tol, rule, maxit);
  else return run_pcg_f(c, V, cK, cM, mcoef, warm, tol, rule, maxit);
}
template <typename T>
inline void to_internal(cfem_ctx *c, const double *src, T *dst, double scale = 1.0) {
  if constexpr (sizeof(T) == 8) to_internal_d(c, src, dst, scale); else to_internal_f(c, src, dst, scale);
}
template <typename T>
inline void to_caller(cfem_ctx *c, const T *src, double *dst) {
  if constexpr (sizeof(T) == 8) to_caller_d(c, src, dst); else to_caller_f(c, src, dst);
}

}  // namespace detail
}  // namespace cfem
