// cfem_pcg_multi: k load cases on one mesh.
//
// With the FP32 edge-fan operator (3D), the cases run as one multi-RHS PCG:
// every matvec streams the patch blocks once for all cases of a batch (at most
// kMaxCases), each case keeps its own scalars and stopping test, and FP32_REFINE
// wraps it in an FP64 iterative refinement whose true residuals f_c - K x_c are
// formed case by case with the FP64 operator. Other forms and FP64 solve the
// cases one after the other.
#include <chrono>
#include <cstdlib>

#include "context_internal.cuh"
#include "kernels_aux.cuh"

namespace cfem {
namespace detail {

struct MultiState {
  int K = 0, C = 0;  // cases per solve (power of two), cases per matvec item
  DBuf<float> x, r, z, pA, pB, u, f;  // [node][K][4]
  DBuf<double> x64, f64, r64, io;     // [node][K][4]; io: caller-order staging
  DBuf<double> s_f, s_x, s_r;         // one case in the single-RHS layout
  DBuf<MultiScalars> sc;
  DBuf<MultiCtl> ctl;
  DBuf<double> partials, gpart;
  DBuf<unsigned> gcnt;  // group tickets: [0, n) matvec, [n, 2n) vector kernel
  DBuf<int> active;
  DBuf<double> res_norms;  // [K][2] ||r_c||^2, ||f_c||^2 of the FP64 true residuals
  DBuf<float> fold_beta;  // [K] continuation of the next run: z_c += beta_c p_last_c
  DBuf<int> fold_par;     // [K] p_last_c in pA (1) or pB (0)
  MultiCtl *h_ctl = nullptr;
  std::vector<MultiScalars> h_sc;
  int grid_mv = 0, grid_vec = 0;
  size_t smem = 0;
  cudaGraphExec_t graph = nullptr;
  ~MultiState() {
    if (graph) cudaGraphExecDestroy(graph);
    if (h_ctl) cudaFreeHost(h_ctl);
  }
};

void destroy_multi(MultiState *m) { delete m; }

namespace {

template <int C>
void launch_mvm(cfem_ctx *c, MultiState &M, int mode, const MultiParams<float> &P, const float *x, const float *pold,
                float *pnew, float *y) {
  dim3 g(M.grid_mv), b(kHfanThreads);
  if (mode == MV_PCG) k_matvec_multi<MV_PCG, C><<<g, b, M.smem, c->stream>>>(P, x, pold, pnew, y);
  else k_matvec_multi<MV_PLAIN, C><<<g, b, M.smem, c->stream>>>(P, x, pold, pnew, y);
  CKL();
  c->launches += 1;
}

void launch_mvm_c(cfem_ctx *c, MultiState &M, int mode, const MultiParams<float> &P, const float *x,
                  const float *pold, float *pnew, float *y) {
  if (M.C == 2) launch_mvm<2>(c, M, mode, P, x, pold, pnew, y);
  else if (M.C == 4) launch_mvm<4>(c, M, mode, P, x, pold, pnew, y);
  else launch_mvm<8>(c, M, mode, P, x, pold, pnew, y);
}

template <int C>
const void *mvm_kernel_c(int mode) {
  return mode == MV_PCG ? (const void *)k_matvec_multi<MV_PCG, C> : (const void *)k_matvec_multi<MV_PLAIN, C>;
}
const void *mvm_kernel(int C, int mode) {
  return C == 2 ? mvm_kernel_c<2>(mode) : C == 4 ? mvm_kernel_c<4>(mode) : mvm_kernel_c<8>(mode);
}

MultiParams<float> multi_params(cfem_ctx *c, MultiState &M) {
  MultiParams<float> P{};
  P.n_patches = c->prep.n_patches;
  P.node_off = c->node_off.p;
  P.own = c->own.p;
  P.diagA = c->v32.diagA.p;
  P.lam = (float)c->lam;
  P.mu = (float)c->mu;
  P.K = M.K;
  P.n_nodes = c->nn;
  P.sc = M.sc.p;
  P.ctl = M.ctl.p;
  P.partials = M.partials.p;
  P.gpart = M.gpart.p;
  P.gcnt_mv = M.gcnt.p;
  P.gcnt_up = M.gcnt.p + M.gcnt.n / 2;
  P.F.blocks = c->blk32.p;
  P.F.L = c->L32;
  P.F.fan_off = c->fan_off.p;
  P.F.fan_elem_off = c->fan_elem_off.p;
  P.F.err = c->tma_err.p;
  return P;
}

// Sets the launch shape for items of C cases; false if they do not fit in
// shared memory.
bool configure_c(cfem_ctx *c, MultiState &M, int C) {
  int optin = 0;
  CK(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, c->device));
  const size_t smem = (size_t)multi_smem(c->L32, C, M.K).bytes;
  if (smem + 1024 > (size_t)optin) return false;  // (+ the kernel's static shared memory)
  M.C = C;
  M.smem = smem;
  for (int mode : {MV_PLAIN, MV_PCG})
    CK(cudaFuncSetAttribute(mvm_kernel(C, mode), cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  int occ = 1;
  CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, mvm_kernel(C, MV_PCG), kHfanThreads, M.smem));
  const int64_t items = (int64_t)c->prep.n_patches * (M.K / C);
  M.grid_mv = (int)std::min<int64_t>(items, (int64_t)c->n_sm * std::max(occ, 1));
  if (M.graph) {
    cudaGraphExecDestroy(M.graph);
    M.graph = nullptr;
  }
  return true;
}

// Cases per item: the variant with the shortest matvec on this mesh and
// batch size, timed on the context's stream (PLAIN form, current vectors; the
// best of three runs of four launches each). CFEM_MULTI_CASES=2|4|8 fixes it
// (when that width fits in shared memory).
void autotune_c(cfem_ctx *c, MultiState &M) {
  float best = 1e30f;
  int best_c = 0, forced = 0;
  if (const char *e = std::getenv("CFEM_MULTI_CASES")) forced = std::atoi(e);
  if ((forced != 2 && forced != 4 && forced != 8) || forced > M.K || !configure_c(c, M, forced)) forced = 0;
  for (int C : {2, 4, 8}) {
    if (C > M.K) break;
    if (forced && C != forced) continue;
    if (!configure_c(c, M, C)) continue;
    MultiParams<float> P = multi_params(c, M);
    launch_mvm_c(c, M, MV_PLAIN, P, M.f.p, nullptr, nullptr, M.u.p);  // warm-up
    for (int rep = 0; rep < 3; ++rep) {
      CK(cudaEventRecord(c->ev0, c->stream));
      for (int i = 0; i < 4; ++i) launch_mvm_c(c, M, MV_PLAIN, P, M.f.p, nullptr, nullptr, M.u.p);
      CK(cudaEventRecord(c->ev1, c->stream));
      CK(cudaEventSynchronize(c->ev1));
      float ms = 0;
      CK(cudaEventElapsedTime(&ms, c->ev0, c->ev1));
      if (ms < best) { best = ms; best_c = C; }
    }
  }
  if (!best_c) throw Fail{CFEM_ERR_INVALID_ARGUMENT, "multi-RHS patch too large for shared memory"};
  configure_c(c, M, best_c);
  M.u.zero(c->stream);
  if (c->verbose) std::printf("multi-RHS: K=%d cases, C=%d cases per item, %d CTAs\n", M.K, M.C, M.grid_mv);
}

MultiState &multi_state(cfem_ctx *c, int K) {
  if (c->multi && c->multi->K == K) return *c->multi;
  if (c->multi) { destroy_multi(c->multi); c->multi = nullptr; }
  auto *M = new MultiState();
  c->multi = M;
  M->K = K;
  const size_t n = (size_t)c->nn * K * 4;
  for (auto *b : {&M->x, &M->r, &M->z, &M->pA, &M->pB, &M->u, &M->f}) {
    b->alloc(n);
    b->zero(c->stream);
  }
  for (auto *b : {&M->x64, &M->f64, &M->r64}) b->alloc(n);
  M->io.alloc((size_t)K * c->nd);
  for (auto *b : {&M->s_f, &M->s_x, &M->s_r}) b->alloc(c->nvec);
  M->sc.alloc(K);
  M->sc.zero(c->stream);
  M->ctl.alloc(1);
  M->ctl.zero(c->stream);
  M->active.alloc(K);
  M->res_norms.alloc((size_t)2 * K);
  M->fold_beta.alloc(K);
  M->fold_par.alloc(K);
  CK(cudaMallocHost(&M->h_ctl, sizeof(MultiCtl)));
  M->h_sc.resize(K);
  // four items per thread per round: two CTAs per SM keep enough loads in flight
  M->grid_vec = (int)std::min<int64_t>(std::max<int64_t>(1, (int64_t)(((size_t)c->nn * K + kThreads - 1) / kThreads)),
                                       (int64_t)c->n_sm * 2);
  const int max_mv_grid = c->n_sm * 8;
  const int max_grid = std::max(max_mv_grid, M->grid_vec);
  M->partials.alloc((size_t)max_grid * K * 3);
  const int max_groups = (max_grid + kSumGroup - 1) / kSumGroup;
  M->gpart.alloc((size_t)max_groups * K * 3);
  M->gcnt.alloc((size_t)2 * max_groups);
  M->gcnt.zero(c->stream);
  return *M;
}

void launch_vec(cfem_ctx *c, MultiState &M, const MultiParams<float> &P, const float *p, int init) {
  k_pcg_multi_vec<float><<<M.grid_vec, kThreads, 0, c->stream>>>(P, M.x.p, M.r.p, M.z.p, p, M.u.p, M.f.p,
                                                                  c->v32.dinv.p, init);
  CKL();
  c->launches += 1;
}

// Continuation of a multi-RHS run: per case the last run's iteration count (0:
// start afresh) and the gamma of its last step length.
struct MultiCont {
  std::vector<int> iters;
  std::vector<double> gamma_prev;
};

// Multi-RHS FP32 PCG on M.f (cases >= k_active are padding). Returns after
// every case has stopped; per-case results in M.h_sc. With `cont`, cases with
// a previous run start from the conjugate-gradient step off its last direction
// (z_c + gamma_c / gamma_prev_c p_last_c), as run_pcg_t does for one case.
void run_pcg_multi(cfem_ctx *c, MultiState &M, int k_active, double tol, int rule, int maxit,
                   const MultiCont *cont = nullptr) {
  MultiCtl h{};
  h.tol = tol;
  h.rule = rule;
  h.maxit = maxit > 0 ? maxit : 1000000;
  h.k_active = k_active;
  CK(cudaMemcpyAsync(M.ctl.p, &h, sizeof(MultiCtl), cudaMemcpyHostToDevice, c->stream));
  M.gcnt.zero(c->stream);  // (tickets of a launch that stopped early are not left behind)
  MultiParams<float> P = multi_params(c, M);
  launch_vec(c, M, P, nullptr, 1);
  if (cont) {
    CK(cudaMemcpyAsync(M.h_sc.data(), M.sc.p, sizeof(MultiScalars) * M.K, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    std::vector<float> beta(M.K, 0.f);
    std::vector<int> par(M.K, 0);
    bool any = false;
    for (int cs = 0; cs < M.K && cs < (int)cont->iters.size(); ++cs) {
      if (M.h_sc[cs].done || cont->iters[cs] <= 0 || !(cont->gamma_prev[cs] > 0)) continue;
      beta[cs] = (float)(M.h_sc[cs].gamma / cont->gamma_prev[cs]);
      par[cs] = (cont->iters[cs] - 1) & 1;
      any = true;
    }
    if (any) {
      CK(cudaMemcpyAsync(M.fold_beta.p, beta.data(), sizeof(float) * M.K, cudaMemcpyHostToDevice, c->stream));
      CK(cudaMemcpyAsync(M.fold_par.p, par.data(), sizeof(int) * M.K, cudaMemcpyHostToDevice, c->stream));
      const int64_t items = (int64_t)c->nn * M.K;
      k_multi_fold<<<nblk(items), kThreads, 0, c->stream>>>(items, M.K, M.fold_beta.p, M.fold_par.p, M.pA.p, M.pB.p,
                                                            M.z.p);
      CKL();
      CK(cudaStreamSynchronize(c->stream));  // (beta and par are pageable)
    }
  }
  if (!M.graph) {
    cudaGraph_t graph;
    const int64_t before = c->launches;
    CK(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
    try {
      for (int it = 0; it < c->chunk; ++it) {
        float *pold = (it & 1) ? M.pB.p : M.pA.p;
        float *pnew = (it & 1) ? M.pA.p : M.pB.p;
        launch_mvm_c(c, M, MV_PCG, P, M.z.p, pold, pnew, M.u.p);
        launch_vec(c, M, P, pnew, 0);
      }
    } catch (...) {
      cudaGraph_t broken = nullptr;
      cudaStreamEndCapture(c->stream, &broken);
      if (broken) cudaGraphDestroy(broken);
      (void)cudaGetLastError();
      throw;
    }
    CK(cudaStreamEndCapture(c->stream, &graph));
    c->launches = before;
    CK(cudaGraphInstantiate(&M.graph, graph, 0));
    cudaGraphDestroy(graph);
  }
  const int64_t max_launches = (int64_t)h.maxit / c->chunk + 16;
  int last_iter = -1, stalled = 0;
  for (int64_t launch = 0;; ++launch) {
    if (launch > max_launches || stalled > 4) {
      check_copy_error(c);
      throw Fail{CFEM_ERR_CUDA, "multi-RHS PCG recurrence stopped advancing on the device"};
    }
    CK(cudaGraphLaunch(M.graph, c->stream));
    c->launches += 2 * c->chunk;
    CK(cudaMemcpyAsync(M.h_ctl, M.ctl.p, sizeof(MultiCtl), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    if (M.h_ctl->all_done) break;
    stalled = M.h_ctl->iter == last_iter ? stalled + 1 : 0;
    last_iter = M.h_ctl->iter;
  }
  check_copy_error(c);
  CK(cudaMemcpy(M.h_sc.data(), M.sc.p, sizeof(MultiScalars) * M.K, cudaMemcpyDeviceToHost));
}

__global__ void k_multi_cast_active(int64_t nn, int K, const double *r64, const int *active, float *f32) {
  int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (q >= nn * K) return;
  const int c = (int)(q % K);
  const NodeV<double, 4> v = ldv<double, 4>(r64, q);
  NodeV<float, 4> w;
#pragma unroll
  for (int d = 0; d < 4; ++d) w.v[d] = active[c] ? (float)v.v[d] : 0.f;
  stv<float, 4>(f32, q, w);
}

int status_of(int done) { return done == 1 ? CFEM_OK : done == 2 ? CFEM_ERR_DIVERGED : CFEM_ERR_NOT_CONVERGED; }

// One batch of kb <= kMaxCases cases. F, U: [kb][n_dof] caller order.
cfem_status solve_batch(cfem_ctx *c, const cfem_solve_params &p, int kb, const double *F, double *U,
                        cfem_solve_info *info) {
  int K = 1;
  while (K < kb) K <<= 1;
  MultiState &M = multi_state(c, K);
  const int64_t nn = c->nn;
  const size_t nitems = (size_t)nn * K;
  c->launches = 0;
  set_diag_vectors(c, c->diagK.p);
  CK(cudaMemcpyAsync(M.io.p, F, sizeof(double) * (size_t)kb * c->nd, cudaMemcpyDefault, c->stream));
  k_multi_to_internal<double><<<nblk(nitems), kThreads, 0, c->stream>>>(nn, K, kb, c->nd, M.io.p,
                                                                         c->node_new2old.p, M.f64.p);
  CKL();
  if (!M.C) {
    k_convert<double, float><<<nblk(nitems * 4), kThreads, 0, c->stream>>>(nitems * 4, M.f64.p, M.f.p);
    CKL();
    autotune_c(c, M);
  }
  CK(cudaEventRecord(c->ev0, c->stream));
  std::vector<int> iters(kb, 0), outer(kb, 0), status(kb, CFEM_ERR_NOT_CONVERGED);
  std::vector<double> gamma0(kb, 0), gamma(kb, 0), rr(kb, 0), ff(kb, 0), rr_prev(kb, -1);
  std::vector<int> stalls(kb, 0);
  std::vector<double> norms(2 * (size_t)kb, 0.0);
  auto residuals = [&](bool all) {
    // r_c = f_c - K' x_c in FP64 with ||r_c||^2 and ||f_c||^2 for the cases
    // still running (all: every case), all queued on the stream and read back once
    auto wanted = [&](int cs) { return all || (status[cs] != CFEM_OK && status[cs] != CFEM_ERR_DIVERGED); };
    int queued = 0;
    for (int cs = 0; cs < kb; ++cs) {
      if (!wanted(cs)) continue;
      k_case_copy<double, double><<<nblk(nn), kThreads, 0, c->stream>>>(nn, K, cs, M.f64.p, M.s_f.p, 1);
      k_case_copy<double, double><<<nblk(nn), kThreads, 0, c->stream>>>(nn, K, cs, M.x64.p, M.s_x.p, 1);
      CKL();
      true_residual_async(c, M.s_f.p, M.s_x.p, M.s_r.p, nullptr, M.res_norms.p + 2 * cs);
      k_case_copy<double, double><<<nblk(nn), kThreads, 0, c->stream>>>(nn, K, cs, M.s_r.p, M.r64.p, 0);
      CKL();
      ++queued;
    }
    if (!queued) return;
    CK(cudaMemcpyAsync(norms.data(), M.res_norms.p, sizeof(double) * 2 * kb, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    check_copy_error(c);
    for (int cs = 0; cs < kb; ++cs) {
      if (!wanted(cs)) continue;
      rr[cs] = norms[2 * cs];
      ff[cs] = norms[2 * cs + 1];
    }
  };
  if (p.precision == CFEM_FP32) {
    k_convert<double, float><<<nblk(nitems * 4), kThreads, 0, c->stream>>>(nitems * 4, M.f64.p, M.f.p);
    CKL();
    run_pcg_multi(c, M, kb, p.tol, p.stop_rule, p.max_iter);
    for (int cs = 0; cs < kb; ++cs) {
      iters[cs] = M.h_sc[cs].iters;
      gamma0[cs] = M.h_sc[cs].gamma0;
      gamma[cs] = M.h_sc[cs].gamma;
      status[cs] = status_of(M.h_sc[cs].done);
    }
    k_convert<float, double><<<nblk(nitems * 4), kThreads, 0, c->stream>>>(nitems * 4, M.x.p, M.x64.p);
    CKL();
  } else {  // FP32 inner PCG in FP64 iterative refinement, per-case outer tests
    M.x64.zero(c->stream);
    CK(cudaMemcpyAsync(M.r64.p, M.f64.p, sizeof(double) * nitems * 4, cudaMemcpyDeviceToDevice, c->stream));
    residuals(false);
    const double outer_tol = p.outer_tol > 0 ? p.outer_tol : 1e-12;
    const int max_outer = p.max_outer > 0 ? p.max_outer : 50;
    const double stall = refine_stall_ratio(p.tol);
    // loose inner tolerances: every case continues its last direction (see solve_internal)
    MultiCont cont{std::vector<int>(K, 0), std::vector<double>(K, 0.0)};
    const bool continued = p.tol >= kContinueTol;
    std::vector<int> act(K, 0);
    for (int round = 0; round <= max_outer; ++round) {
      int n_act = 0;
      for (int cs = 0; cs < kb; ++cs) {
        act[cs] = 0;
        if (status[cs] == CFEM_OK || status[cs] == CFEM_ERR_DIVERGED) continue;
        const bool conv = std::sqrt(rr[cs]) <= outer_tol * std::sqrt(ff[cs]);
        // the FP64 true residual has a floor near eps64 * ||K|| ||x||: two
        // refinement steps in a row that no longer reduce it as a step should
        // end the case
        stalls[cs] = rr_prev[cs] >= 0 && rr[cs] > stall * rr_prev[cs] ? stalls[cs] + 1 : 0;
        const bool stalled = stalls[cs] >= 2;
        if (conv || stalled || ff[cs] == 0.0) { status[cs] = CFEM_OK; continue; }
        if (round == max_outer) continue;
        act[cs] = 1;
        ++n_act;
      }
      if (!n_act) break;
      CK(cudaMemcpyAsync(M.active.p, act.data(), sizeof(int) * K, cudaMemcpyHostToDevice, c->stream));
      k_multi_cast_active<<<nblk(nitems), kThreads, 0, c->stream>>>(nn, K, M.r64.p, M.active.p, M.f.p);
      CKL();
      run_pcg_multi(c, M, kb, p.tol, p.stop_rule, p.max_iter, continued ? &cont : nullptr);
      for (int cs = 0; cs < kb; ++cs) {
        if (!act[cs]) continue;
        const int d = M.h_sc[cs].done;
        cont.iters[cs] = d == 1 || d == 3 ? M.h_sc[cs].iters : 0;
        cont.gamma_prev[cs] = M.h_sc[cs].gamma_prev;
        iters[cs] += M.h_sc[cs].iters;
        if (outer[cs] == 0) gamma0[cs] = M.h_sc[cs].gamma0;
        gamma[cs] = M.h_sc[cs].gamma;
        outer[cs] += 1;
        if (M.h_sc[cs].done == 2) status[cs] = CFEM_ERR_DIVERGED;
        rr_prev[cs] = rr[cs];
      }
      k_multi_accumulate<<<nblk(nitems * 4), kThreads, 0, c->stream>>>(nitems * 4, M.x.p, M.x64.p);
      CKL();
      residuals(false);
    }
  }
  CK(cudaEventRecord(c->ev1, c->stream));
  CK(cudaEventSynchronize(c->ev1));
  float ms = 0;
  CK(cudaEventElapsedTime(&ms, c->ev0, c->ev1));
  if (p.precision == CFEM_FP32) residuals(true);  // relative residuals for the report
  k_multi_to_caller<double><<<nblk(nitems), kThreads, 0, c->stream>>>(nn, K, kb, c->nd, M.x64.p, c->node_new2old.p,
                                                                        M.io.p);
  CKL();
  CK(cudaMemcpyAsync(U, M.io.p, sizeof(double) * (size_t)kb * c->nd, cudaMemcpyDefault, c->stream));
  check_copy_error(c);
  cfem_status worst = CFEM_OK;
  for (int cs = 0; cs < kb; ++cs) {
    if (info) {
      cfem_solve_info &in = info[cs];
      in = cfem_solve_info{};
      in.status = status[cs];
      in.iterations = iters[cs];
      in.outer_iterations = outer[cs];
      in.rel_residual = ff[cs] > 0 ? std::sqrt(rr[cs] / ff[cs]) : std::sqrt(rr[cs]);
      in.gamma0 = gamma0[cs];
      in.gamma = gamma[cs];
      in.solve_ms = ms;
      in.kernel_launches = c->launches;
    }
    if (status[cs] != CFEM_OK && worst == CFEM_OK) worst = (cfem_status)status[cs];
  }
  return worst;
}

}  // namespace
}  // namespace detail
}  // namespace cfem

using namespace cfem;
using namespace cfem::detail;

extern "C" cfem_status cfem_pcg_multi(cfem_ctx *ctx, const cfem_solve_params *prm, int32_t k, const double *F, double *U,
                                      cfem_solve_info *info) {
  return run_guarded([&]() -> cfem_status {
    check_ctx(ctx);
    enter(ctx);
    if (k <= 0 || !F || !U) throw Fail{CFEM_ERR_INVALID_ARGUMENT, "bad multi-RHS arguments"};
    cfem_solve_params p = prm ? *prm : default_params();
    cfem_status worst = CFEM_OK;
    const bool batched = ctx->fans && ctx->fan_tma && k > 1 &&
                         (p.precision == CFEM_FP32 || p.precision == CFEM_FP32_REFINE);
    if (batched) {
      for (int b0 = 0; b0 < k; b0 += kMaxCases) {
        const int kb = std::min(kMaxCases, k - b0);
        cfem_status st = solve_batch(ctx, p, kb, F + (size_t)b0 * ctx->nd, U + (size_t)b0 * ctx->nd,
                                     info ? info + b0 : nullptr);
        if (st != CFEM_OK && worst == CFEM_OK) worst = st;
      }
      return worst;
    }
    for (int i = 0; i < k; ++i) {
      cfem_solve_info inf{};
      to_internal<double>(ctx, F + (size_t)i * ctx->nd, ctx->v64.f.p);
      cfem_status st = solve_internal(ctx, &p, &inf);
      to_caller<double>(ctx, ctx->v64.x.p, U + (size_t)i * ctx->nd);
      if (info) info[i] = inf;
      if (st != CFEM_OK && worst == CFEM_OK) worst = st;
    }
    CK(cudaStreamSynchronize(ctx->stream));
    return worst;
  });
}
