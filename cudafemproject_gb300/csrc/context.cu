// C-ABI implementation (include/cfem.h): context lifetime, static solvers.
//
// Host orchestration only; the arithmetic lives in kernels.cuh / kernels_aux.cuh.
// PCG iterations are issued as captured CUDA graphs of 2*chunk kernels
// (matvec with fused direction update, then the vector update), replayed until
// the device-side stopping flag is set; all scalar recurrences stay on the GPU.
#include <mutex>

#include "context_internal.cuh"
#include "kernels_aux.cuh"

namespace cfem {
namespace detail {

thread_local std::string g_last_error;

template <typename T>
MvParams<T> base_mv_t(cfem_ctx *c) {
  MvParams<T> P{};
  P.n_patches = c->prep.n_patches;
  P.elem_off = c->elem_off.p;
  P.node_off = c->node_off.p;
  P.nodes = c->nodes.p;
  P.own = c->own.p;
  P.lconn = c->lconn.p;
  P.bits = c->bits.p;
  if constexpr (sizeof(T) == 8) P.G = c->G64.p; else P.G = c->G32.p;
  P.gstride = c->gstride;
  P.mcoef = nullptr;
  P.lam = (T)c->lam;
  P.mu = (T)c->mu;
  P.cK = 1;
  P.cM = 0;
  P.partials = c->partials.p;
  P.up_part = c->partials_up.p;
  P.n_up = c->dim == 3 ? c->grid_upd : c->grid_vec;
  P.inc = c->inc.p;
  P.inc_start = c->inc_start.p;
  P.pe = c->prep.patch_elems;
  P.np_max = c->np_slots;
  return P;
}

template <typename T>
void launch_mv_t(cfem_ctx *c, int mode, const MvParams<T> &P) {
  if (c->n_inst && !P.patch_inst)
    throw Fail{CFEM_ERR_UNSUPPORTED, "a context of batched meshes supports cfem_batch_static_solve only"};
  // FP32: patch blocks streamed by bulk copies. FP64 keeps the plain fan
  // kernel below: it is bound by the FP64 pipe, and its twice-as-large blocks
  // would leave one CTA per SM.
  if constexpr (sizeof(T) == 4) {
    if (c->fans && c->fan_tma) {
      FanTmaParams F{};
      F.blocks = c->blk32.p;
      F.L = c->L32;
      F.fan_off = c->fan_off.p;
      F.fan_elem_off = c->fan_elem_off.p;
      F.err = c->tma_err.p;
      F.skip_patch_plus1 = c->selftest_skip_plus1;
      F.wait_limit = c->selftest_wait_limit;
      const double l2_half = 0.5 * c->l2_bytes;
      F.evict_first = (double)c->L32.bytes * c->prep.n_patches > l2_half;
      if (c->geo && !P.patch_inst) {
        F.blocks = c->blkg.p;
        F.L = c->Lg;
        F.evict_first = (double)c->Lg.bytes * c->prep.n_patches > l2_half;
        dim3 g(c->grid_geo), b(kHfanThreads);
        if (P.mcoef && mode == MV_PLAIN)
          k_matvec_fan_tma<float, MV_PLAIN, true, true><<<g, b, c->smem_geo, c->stream>>>(P, F);
        else if (P.mcoef && mode == MV_PCG)
          launch_pdl(k_matvec_fan_tma<float, MV_PCG, true, true>, g, b, c->smem_geo, c->stream, P, F);
        else if (mode == MV_PLAIN) k_matvec_fan_tma<float, MV_PLAIN, true><<<g, b, c->smem_geo, c->stream>>>(P, F);
        else if (mode == MV_PCG) launch_pdl(k_matvec_fan_tma<float, MV_PCG, true>, g, b, c->smem_geo, c->stream, P, F);
        else launch_pdl(k_matvec_fan_tma<float, MV_DYN, true>, g, b, c->smem_geo, c->stream, P, F);
        CKL();
        c->launches += 1;
        return;
      }
      dim3 g(c->grid_ft32), b(kHfanThreads);
      if (P.patch_inst) {
        if (mode != MV_PCG || P.mcoef) throw Fail{CFEM_ERR_UNSUPPORTED, "batched meshes: PCG-form static matvec only"};
        launch_pdl(k_matvec_fan_tma<float, MV_PCG, false, false, true>, g, b, c->smem_ft32, c->stream, P, F);
      } else if (P.mcoef && mode == MV_PLAIN)
        k_matvec_fan_tma<float, MV_PLAIN, false, true><<<g, b, c->smem_ft32, c->stream>>>(P, F);
      else if (P.mcoef && mode == MV_PCG)
        launch_pdl(k_matvec_fan_tma<float, MV_PCG, false, true>, g, b, c->smem_ft32, c->stream, P, F);
      else if (mode == MV_PLAIN) k_matvec_fan_tma<float, MV_PLAIN><<<g, b, c->smem_ft32, c->stream>>>(P, F);
      else if (mode == MV_PCG) launch_pdl(k_matvec_fan_tma<float, MV_PCG>, g, b, c->smem_ft32, c->stream, P, F);
      else launch_pdl(k_matvec_fan_tma<float, MV_DYN>, g, b, c->smem_ft32, c->stream, P, F);
      CKL();
      c->launches += 1;
      return;
    }
  }
  if (c->fans && c->dim == 3) {
    FanParams F{c->fan_off.p, c->fan_elem_off.p, c->fan_slot.p, c->finc.p, c->finc_start.p, c->fstride};
    const T *Gf;
    if constexpr (sizeof(T) == 8) Gf = c->Gf64.p; else Gf = c->Gf32.p;
    const size_t smem = sizeof(T) == 8 ? c->smem_fan64 : c->smem_fan32;
    dim3 g(c->grid_fan), b(kFanThreads);
    if (mode == MV_PLAIN) k_matvec_fan<T, MV_PLAIN><<<g, b, smem, c->stream>>>(P, F, Gf);
    else if (mode == MV_PCG) k_matvec_fan<T, MV_PCG><<<g, b, smem, c->stream>>>(P, F, Gf);
    else k_matvec_fan<T, MV_DYN><<<g, b, smem, c->stream>>>(P, F, Gf);
    CKL();
    c->launches += 1;
    return;
  }
  size_t smem = sizeof(T) == 8 ? c->smem64 : c->smem32;
  dim3 g(c->grid_mv), b(kThreads);
  if (c->dim == 3) {
    if (mode == MV_PLAIN) k_matvec<T, 3, MV_PLAIN><<<g, b, smem, c->stream>>>(P);
    else if (mode == MV_PCG) k_matvec<T, 3, MV_PCG><<<g, b, smem, c->stream>>>(P);
    else k_matvec<T, 3, MV_DYN><<<g, b, smem, c->stream>>>(P);
  } else {
    if (mode == MV_PLAIN) k_matvec<T, 2, MV_PLAIN><<<g, b, smem, c->stream>>>(P);
    else if (mode == MV_PCG) k_matvec<T, 2, MV_PCG><<<g, b, smem, c->stream>>>(P);
    else k_matvec<T, 2, MV_DYN><<<g, b, smem, c->stream>>>(P);
  }
  CKL();
  c->launches += 1;
}

// Grid of the PCG-form matvec that launch_mv_t runs for precision T (the
// number of p.Ap partials the update kernel adds up).
template <typename T>
int pcg_mv_grid(const cfem_ctx *c) {
  if constexpr (sizeof(T) == 4)
    if (c->fans && c->fan_tma) return c->geo ? c->grid_geo : c->grid_ft32;
  if (c->fans && c->dim == 3) return c->grid_fan;
  return c->grid_mv;
}

template <typename T>
VecParams<T> vec_params(cfem_ctx *c, Vecs<T> &V, T *p, Scalars *sc) {
  VecParams<T> P{};
  P.n_nodes = c->nn;
  P.x = V.x.p; P.r = V.r.p; P.z = V.z.p; P.p = p; P.u = V.u.p;
  P.dinv = V.dinv.p;
  P.f = V.f.p;
  P.sc = sc;
  P.partials = c->partials.p;
  P.mv_part = c->partials.p;
  P.n_mv = pcg_mv_grid<T>(c);
  P.up_part = c->partials_up.p;
  return P;
}

template <typename T>
void launch_init(cfem_ctx *c, const VecParams<T> &P, int warm) {
  if (c->dim == 3) k_pcg_init<T, 3><<<c->grid_vec, kThreads, 0, c->stream>>>(P, warm);
  else k_pcg_init<T, 2><<<c->grid_vec, kThreads, 0, c->stream>>>(P, warm);
  CKL();
  c->launches += 1;
}

template <typename T>
void launch_update(cfem_ctx *c, const VecParams<T> &P) {
  if (c->dim == 3 && P.cond) launch_pdl(k_pcg_update<T, 3, true>, dim3(c->grid_upd), dim3(kThreads), 0, c->stream, P);
  else if (c->dim == 3) launch_pdl(k_pcg_update<T, 3>, dim3(c->grid_upd), dim3(kThreads), 0, c->stream, P);
  else if (P.cond) k_pcg_update<T, 2, true><<<c->grid_vec, kThreads, 0, c->stream>>>(P);
  else k_pcg_update<T, 2><<<c->grid_vec, kThreads, 0, c->stream>>>(P);
  CKL();
  c->launches += 1;
}

// Jacobi PCG on A x = V.f with A = cM*M + cK*K' (mcoef selects the mass term).
// V.x holds the warm start when warm != 0. Returns after the device flag says done.
template <typename T>
PcgResult run_pcg_t(cfem_ctx *c, Vecs<T> &V, T cK, T cM, const T *mcoef, int warm, double tol, int rule, int maxit,
                    const T *cont_p = nullptr, double cont_gamma_prev = 0) {
  Scalars *sc = c->sc.p + (sizeof(T) == 8 ? 0 : 1);
  Scalars h{};
  h.tol = tol;
  h.rule = rule;
  h.maxit = maxit > 0 ? maxit : 1000000;
  CK(cudaMemcpyAsync(sc, &h, sizeof(Scalars), cudaMemcpyHostToDevice, c->stream));
  MvParams<T> mv = base_mv<T>(c);
  mv.cK = cK;
  mv.cM = cM;
  mv.mcoef = mcoef;
  mv.diagA = V.diagA.p;
  mv.sc = sc;
  if (warm) {
    mv.x = V.x.p;
    mv.y = V.u.p;
    V.u.zero(c->stream);
    launch_mv<T>(c, MV_PLAIN, mv);
  }
  launch_init<T>(c, vec_params<T>(c, V, V.pA.p, sc), warm);
  if (cont_p && cont_gamma_prev > 0) {
    // Continuation of an earlier run on a new residual: its last direction
    // p_last stays, and the first direction becomes the conjugate-gradient
    // step from it, z + (gamma / gamma_prev) p_last, folded into z here (the
    // first matvec takes p = z).
    if (c->dim == 3) k_fold_direction<T, 3><<<nblk(c->nn), kThreads, 0, c->stream>>>(c->nn, sc, cont_gamma_prev, cont_p, V.z.p);
    else k_fold_direction<T, 2><<<nblk(c->nn), kThreads, 0, c->stream>>>(c->nn, sc, cont_gamma_prev, cont_p, V.z.p);
    CKL();
    c->launches += 1;
  }
  GraphCache &gc = sizeof(T) == 8 ? c->graph64 : c->graph32;
  // directions alternate between pA and pB, A p between u and uB: the matvec
  // of iteration `it` accumulates into one u buffer and zeroes the other for
  // iteration it + 1 (the init kernel zeroes u for iteration 0; chunk is even)
  auto capture_iterations = [&](unsigned long long cond) {
    for (int it = 0; it < c->chunk; ++it) {
      T *pold = (it & 1) ? V.pB.p : V.pA.p;
      T *pnew = (it & 1) ? V.pA.p : V.pB.p;
      T *ucur = (it & 1) ? V.uB.p : V.u.p;
      MvParams<T> m = mv;
      m.x = V.z.p;
      m.x2 = pold;
      m.xout = pnew;
      m.y = ucur;
      m.yzero = (it & 1) ? V.u.p : V.uB.p;
      launch_mv<T>(c, MV_PCG, m);
      VecParams<T> up = vec_params<T>(c, V, pnew, sc);
      up.u = ucur;
      up.cond = cond;
      up.cond_role = (it == 0 ? 1 : 0) | (it == c->chunk - 1 ? 2 : 0);
      up.cond_chunk = c->chunk;
      launch_update<T>(c, up);
    }
  };
  if (!gc.exec || gc.key0 != (const void *)mcoef || gc.key1 != (double)cK || gc.key2 != (double)cM) {
    gc.reset();
    const int64_t launches_before_capture = c->launches;
    // Preferred: the iterations inside a CUDA-graph WHILE node, so a solve is
    // one graph launch and the loop runs without host round trips. Where the
    // runtime does not build it, a graph of `chunk` iterations that the host
    // relaunches until the device flag says done.
    if (!c->host_loop) {
      cudaGraph_t graph = nullptr;
      cudaGraphExec_t exec = nullptr;
      cudaGraphConditionalHandle h = 0;
      bool ok = cudaGraphCreate(&graph, 0) == cudaSuccess &&
                cudaGraphConditionalHandleCreate(&h, graph, 1, cudaGraphCondAssignDefault) == cudaSuccess;
      cudaGraph_t body = nullptr;
      if (ok) {
        cudaGraphNodeParams np{};
        np.type = cudaGraphNodeTypeConditional;
        np.conditional.handle = h;
        np.conditional.type = cudaGraphCondTypeWhile;
        np.conditional.size = 1;
        cudaGraphNode_t node;
        ok = cudaGraphAddNode(&node, graph, nullptr, nullptr, 0, &np) == cudaSuccess;
        if (ok) body = np.conditional.phGraph_out[0];
      }
      if (ok) ok = cudaStreamBeginCaptureToGraph(c->stream, body, nullptr, nullptr, 0,
                                                 cudaStreamCaptureModeThreadLocal) == cudaSuccess;
      if (ok) {
        try {
          capture_iterations(h);
        } catch (...) {
          ok = false;
        }
        cudaGraph_t captured = nullptr;
        if (cudaStreamEndCapture(c->stream, &captured) != cudaSuccess) ok = false;
      }
      if (ok) ok = cudaGraphInstantiate(&exec, graph, 0) == cudaSuccess;
      if (graph) cudaGraphDestroy(graph);
      (void)cudaGetLastError();
      if (ok) {
        gc.exec = exec;
        gc.device_loop = true;
      } else if (exec) {
        cudaGraphExecDestroy(exec);
      }
    }
    if (!gc.exec) {
      cudaGraph_t graph;
      CK(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
      try {
        capture_iterations(0);
      } catch (...) {
        cudaGraph_t broken = nullptr;
        cudaStreamEndCapture(c->stream, &broken);
        if (broken) cudaGraphDestroy(broken);
        (void)cudaGetLastError();
        throw;
      }
      CK(cudaStreamEndCapture(c->stream, &graph));
      CK(cudaGraphInstantiate(&gc.exec, graph, 0));
      cudaGraphDestroy(graph);
      gc.device_loop = false;
    }
    c->launches = launches_before_capture;
    gc.key0 = mcoef;
    gc.key1 = cK;
    gc.key2 = cM;
  }
  PcgResult res;
  if (gc.device_loop) {
    CK(cudaGraphLaunch(gc.exec, c->stream));
    CK(cudaMemcpyAsync(c->h_sc, sc, sizeof(Scalars), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    c->launches += (int64_t)2 * c->chunk * c->h_sc->loops;
    if (c->verbose)
      std::printf("iteration %d gamma %.6e gamma0 %.6e (%d loops)\n", c->h_sc->iter, c->h_sc->gamma, c->h_sc->gamma0,
                  c->h_sc->loops);
    if (!c->h_sc->done) {
      check_copy_error(c);
      throw Fail{CFEM_ERR_CUDA, "PCG recurrence stopped advancing on the device"};
    }
  } else {
    // Every replay advances the iteration count by `chunk` unless the device
    // flag is set; the cap below only guards against a stalled recurrence.
    const int64_t max_launches = (int64_t)h.maxit / c->chunk + 16;
    int last_iter = -1, stalled = 0;
    for (int64_t launch = 0;; ++launch) {
      if (launch > max_launches || stalled > 4) {
        check_copy_error(c);
        throw Fail{CFEM_ERR_CUDA, "PCG recurrence stopped advancing on the device"};
      }
      CK(cudaGraphLaunch(gc.exec, c->stream));
      c->launches += 2 * c->chunk;
      CK(cudaMemcpyAsync(c->h_sc, sc, sizeof(Scalars), cudaMemcpyDeviceToHost, c->stream));
      CK(cudaStreamSynchronize(c->stream));
      if (c->verbose)
        std::printf("iteration %d gamma %.6e gamma0 %.6e\n", c->h_sc->iter, c->h_sc->gamma, c->h_sc->gamma0);
      if (c->h_sc->done) break;
      stalled = c->h_sc->iter == last_iter ? stalled + 1 : 0;
      last_iter = c->h_sc->iter;
    }
  }
  check_copy_error(c);
  res.iters = c->h_sc->iter;
  res.gamma0 = c->h_sc->gamma0;
  res.gamma = c->h_sc->gamma;
  res.rr = c->h_sc->rr;
  res.ff = c->h_sc->ff;
  res.gamma_prev = c->h_sc->gamma_prev;
  int d = c->h_sc->done;
  res.status = d == 1 ? CFEM_OK : d == 2 ? CFEM_ERR_DIVERGED : CFEM_ERR_NOT_CONVERGED;
  return res;
}

// caller-order FP64 array (host or device) -> internal node vector of type T
template <typename T>
void to_internal_t(cfem_ctx *c, const double *src, T *dst, double scale) {
  CK(cudaMemcpyAsync(c->io.p, src, sizeof(double) * c->nd, cudaMemcpyDefault, c->stream));
  if (c->dim == 3) k_to_internal<T, 3><<<nblk(c->nn), kThreads, 0, c->stream>>>(c->nn, c->io.p, c->node_new2old.p, dst, scale);
  else k_to_internal<T, 2><<<nblk(c->nn), kThreads, 0, c->stream>>>(c->nn, c->io.p, c->node_new2old.p, dst, scale);
  CKL();
}

template <typename T>
void to_caller_t(cfem_ctx *c, const T *src, double *dst) {
  if (c->dim == 3) k_to_caller<T, 3><<<nblk(c->nn), kThreads, 0, c->stream>>>(c->nn, src, c->node_new2old.p, c->io.p);
  else k_to_caller<T, 2><<<nblk(c->nn), kThreads, 0, c->stream>>>(c->nn, src, c->node_new2old.p, c->io.p);
  CKL();
  CK(cudaMemcpyAsync(dst, c->io.p, sizeof(double) * c->nd, cudaMemcpyDefault, c->stream));
}

MvParams<double> base_mv_d(cfem_ctx *c) { return base_mv_t<double>(c); }
MvParams<float> base_mv_f(cfem_ctx *c) { return base_mv_t<float>(c); }
void launch_mv_d(cfem_ctx *c, int mode, const MvParams<double> &P) { launch_mv_t<double>(c, mode, P); }
void launch_mv_f(cfem_ctx *c, int mode, const MvParams<float> &P) { launch_mv_t<float>(c, mode, P); }
PcgResult run_pcg_d(cfem_ctx *c, Vecs<double> &V, double cK, double cM, const double *mcoef, int warm, double tol,
                    int rule, int maxit) {
  return run_pcg_t<double>(c, V, cK, cM, mcoef, warm, tol, rule, maxit);
}
PcgResult run_pcg_f(cfem_ctx *c, Vecs<float> &V, float cK, float cM, const float *mcoef, int warm, double tol,
                    int rule, int maxit) {
  return run_pcg_t<float>(c, V, cK, cM, mcoef, warm, tol, rule, maxit);
}
void to_internal_d(cfem_ctx *c, const double *src, double *dst, double scale) { to_internal_t<double>(c, src, dst, scale); }
void to_internal_f(cfem_ctx *c, const double *src, float *dst, double scale) { to_internal_t<float>(c, src, dst, scale); }
void to_caller_d(cfem_ctx *c, const double *src, double *dst) { to_caller_t<double>(c, src, dst); }
void to_caller_f(cfem_ctx *c, const float *src, double *dst) { to_caller_t<float>(c, src, dst); }

// FP64 true residual r = f - K' x (f, x internal FP64; x == nullptr stands
// for x = 0), ||r||^2 and ||f||^2 into the device doubles out2[0], out2[1];
// queued on the context's stream.
void true_residual_async(cfem_ctx *c, const double *f, const double *x, double *r, float *r32, double *out2) {
  c->tmp64.zero(c->stream);
  if (x) {  // (x == nullptr: x = 0, K' x = 0)
    MvParams<double> mv = base_mv<double>(c);
    mv.diagA = c->diagK.p;
    mv.x = x;
    mv.y = c->tmp64.p;
    launch_mv<double>(c, MV_PLAIN, mv);
  }
  ResParams P{};
  P.nvec = c->nvec;
  P.f = f;
  P.u = c->tmp64.p;
  P.r = r;
  P.r32 = r32;
  P.out = out2;
  P.partials = c->partials.p;
  P.count = c->counters.p;
  k_residual<<<c->grid_vec, kThreads, 0, c->stream>>>(P);
  CKL();
}

// The same, waited for: returns ||r||^2, ||f||^2.
void true_residual(cfem_ctx *c, const double *f, const double *x, double *r, float *r32, double &rr, double &ff) {
  true_residual_async(c, f, x, r, r32, c->rr.p);
  CK(cudaMemcpyAsync(c->h_rr, c->rr.p, 2 * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  rr = c->h_rr[0];
  ff = c->h_rr[1];
  check_copy_error(c);
}

void set_diag_vectors(cfem_ctx *c, const double *diagA64) {
  // dinv and diagA for both precisions from one FP64 diagonal (internal layout)
  k_invert<double><<<nblk(c->nvec), kThreads, 0, c->stream>>>(c->nvec, diagA64, c->v64.dinv.p);
  k_invert<float><<<nblk(c->nvec), kThreads, 0, c->stream>>>(c->nvec, diagA64, c->v32.dinv.p);
  CK(cudaMemcpyAsync(c->v64.diagA.p, diagA64, sizeof(double) * c->nvec, cudaMemcpyDeviceToDevice, c->stream));
  k_convert<double, float><<<nblk(c->nvec), kThreads, 0, c->stream>>>(c->nvec, diagA64, c->v32.diagA.p);
  CKL();
}

// Static-type solve of K' x = f (f internal FP64 in c->v64.f). Result in c->v64.x.
cfem_status solve_internal(cfem_ctx *c, const cfem_solve_params *prm, cfem_solve_info *info) {
  cfem_solve_info inf{};
  c->launches = 0;
  set_diag_vectors(c, c->diagK.p);
  CK(cudaEventRecord(c->ev0, c->stream));
  const int prec = prm->precision;
  int status = CFEM_OK;
  if (prec == CFEM_FP64) {
    PcgResult r = run_pcg<double>(c, c->v64, 1.0, 0.0, nullptr, 0, prm->tol, prm->stop_rule, prm->max_iter);
    status = r.status;
    inf.iterations = r.iters;
    inf.gamma0 = r.gamma0;
    inf.gamma = r.gamma;
  } else if (prec == CFEM_FP32) {
    k_convert<double, float><<<nblk(c->nvec), kThreads, 0, c->stream>>>(c->nvec, c->v64.f.p, c->v32.f.p);
    CKL();
    PcgResult r = run_pcg<float>(c, c->v32, 1.f, 0.f, nullptr, 0, prm->tol, prm->stop_rule, prm->max_iter);
    status = r.status;
    inf.iterations = r.iters;
    inf.gamma0 = r.gamma0;
    inf.gamma = r.gamma;
    k_convert<float, double><<<nblk(c->nvec), kThreads, 0, c->stream>>>(c->nvec, c->v32.x.p, c->v64.x.p);
    CKL();
  } else if (prec == CFEM_FP32_REFINE) {
    // x64 = 0; r64 = f; repeat: solve K d = r (FP32), x64 += d, r64 = f - K64 x64
    c->v64.x.zero(c->stream);
    double rr = 0, ff = 0;
    true_residual(c, c->v64.f.p, nullptr, c->v64.r.p, c->v32.f.p, rr, ff);  // x = 0: r = f
    const double outer_tol = prm->outer_tol > 0 ? prm->outer_tol : 1e-12;
    const int max_outer = prm->max_outer > 0 ? prm->max_outer : 50;
    int outer = 0, total = 0;
    status = CFEM_ERR_NOT_CONVERGED;
    double rr_prev = -1;
    int cont_iters = 0;  // iterations of the previous FP32 run (0: start the next one afresh)
    double cont_gprev = 0;
    const double stall = refine_stall_ratio(prm->tol);
    int stalls = 0;
    while (outer < max_outer) {
      if (std::sqrt(rr) <= outer_tol * std::sqrt(ff)) { status = CFEM_OK; break; }
      // The FP64 true residual has a floor near eps64 * ||K|| ||x||; once two
      // refinement steps in a row no longer reduce it as a step should (halve
      // it; a continued step reduces it by about the replacement factor tol)
      // the iterate is converged in FP64. (One such step alone can be an FP32
      // run that ended early, well above the floor.)
      stalls = rr_prev >= 0 && rr > stall * rr_prev ? stalls + 1 : 0;
      if (stalls >= 2) { status = CFEM_OK; break; }
      rr_prev = rr;
      // With a loose inner tolerance (a residual-replacement factor, at least
      // kContinueTol), from the second step on the FP32 PCG continues with its
      // last direction (the step it ended on was taken with gamma_prev;
      // iteration i writes its direction to pB when i is even, to pA when odd)
      // instead of restarting from z: the FP64 true residual replaces the
      // recursive one and the Krylov directions found so far keep serving.
      // Replaced seldom, the recursive residual drifts too far from the true
      // one for the old direction to stay conjugate, so tighter inner
      // tolerances restart.
      PcgResult r = cont_iters > 0 && prm->tol >= kContinueTol
                        ? run_pcg_t<float>(c, c->v32, 1.f, 0.f, nullptr, 0, prm->tol, prm->stop_rule, prm->max_iter,
                                           ((cont_iters - 1) & 1) ? c->v32.pA.p : c->v32.pB.p, cont_gprev)
                        : run_pcg<float>(c, c->v32, 1.f, 0.f, nullptr, 0, prm->tol, prm->stop_rule, prm->max_iter);
      cont_iters = r.status == CFEM_OK || r.status == CFEM_ERR_NOT_CONVERGED ? r.iters : 0;
      cont_gprev = r.gamma_prev;
      total += r.iters;
      if (outer == 0) inf.gamma0 = r.gamma0;
      inf.gamma = r.gamma;
      if (r.status == CFEM_ERR_DIVERGED) { status = CFEM_ERR_DIVERGED; break; }
      k_accumulate<<<nblk(c->nvec), kThreads, 0, c->stream>>>(c->nvec, c->v32.x.p, c->v64.x.p, c->vw);
      CKL();
      ++outer;
      true_residual(c, c->v64.f.p, c->v64.x.p, c->v64.r.p, c->v32.f.p, rr, ff);
    }
    if (status != CFEM_OK && std::sqrt(rr) <= outer_tol * std::sqrt(ff)) status = CFEM_OK;
    inf.iterations = total;
    inf.outer_iterations = outer;
  } else {
    throw Fail{CFEM_ERR_INVALID_ARGUMENT, "unknown precision"};
  }
  CK(cudaEventRecord(c->ev1, c->stream));
  CK(cudaEventSynchronize(c->ev1));
  float ms = 0;
  CK(cudaEventElapsedTime(&ms, c->ev0, c->ev1));
  inf.solve_ms = ms;
  inf.kernel_launches = c->launches;
  double rr = 0, ff = 0;
  true_residual(c, c->v64.f.p, c->v64.x.p, c->tmp64b.p, nullptr, rr, ff);
  inf.rel_residual = ff > 0 ? std::sqrt(rr / ff) : std::sqrt(rr);
  inf.status = status;
  if (info) *info = inf;
  return (cfem_status)status;
}

// F(t) = a FA + b FB into the internal FP64 vector dst
void make_rhs(cfem_ctx *c, double a, double b, double *dst) {
  CK(cudaMemsetAsync(dst, 0, sizeof(double) * c->nvec, c->stream));
  if (a != 0) k_axpby64<<<nblk(c->nvec), kThreads, 0, c->stream>>>(c->nvec, a, c->FA.p, 1.0, dst);
  if (b != 0) k_axpby64<<<nblk(c->nvec), kThreads, 0, c->stream>>>(c->nvec, b, c->FB.p, 1.0, dst);
  CKL();
}

// ======================================================================== C-ABI
cfem_status run_guarded(const std::function<cfem_status()> &fn) {
  (void)cudaGetLastError();  // a failure of an earlier call must not leak into this one
  try {
    return fn();
  } catch (const Fail &f) {
    g_last_error = f.msg;
    return f.st;
  } catch (const std::bad_alloc &) {
    g_last_error = "host out of memory";
    return CFEM_ERR_OUT_OF_MEMORY;
  } catch (const std::exception &e) {
    g_last_error = e.what();
    return CFEM_ERR_INVALID_ARGUMENT;
  }
}

void setup_context(cfem_ctx *c, const cfem_mesh *m, const cfem_material *mat, const cfem_options *opt) {
  c->dim = m->dim;
  c->nv = m->dim + 1;
  c->w = 6 * (m->dim - 1);
  c->vw = m->dim == 3 ? 4 : 2;
  c->ncomp = m->dim * m->dim;
  c->nn = m->n_nodes;
  c->ne = m->n_elems;
  c->nd = c->nn * c->dim;
  c->nvec = c->nn * c->vw;
  c->semantics = opt ? opt->semantics : CFEM_COMPAT;
  const int req_form = opt ? opt->matvec_form : CFEM_FORM_AUTO;
  if (req_form == CFEM_FORM_STORED_KE)
    throw Fail{CFEM_ERR_UNSUPPORTED, "stored K_e form is not built in this library version"};
  if (req_form < CFEM_FORM_AUTO || req_form > CFEM_FORM_GEOMETRY_FAN)
    throw Fail{CFEM_ERR_INVALID_ARGUMENT, "unknown matvec_form"};
  if ((req_form == CFEM_FORM_GRADIENT_FAN || req_form == CFEM_FORM_GEOMETRY_FAN) && m->dim != 3)
    throw Fail{CFEM_ERR_INVALID_ARGUMENT, "the edge-fan forms are for tetrahedra (dim 3)"};
  c->fans = m->dim == 3 && req_form != CFEM_FORM_GRADIENT;
  c->geo = c->fans && req_form == CFEM_FORM_GEOMETRY_FAN;
  c->form = c->geo ? CFEM_FORM_GEOMETRY_FAN : c->fans ? CFEM_FORM_GRADIENT_FAN : CFEM_FORM_GRADIENT;
  c->verbose = opt ? opt->verbose : 0;
  c->E = mat ? mat->young_modulus : 2e7;
  c->nu = mat ? mat->poisson_ratio : 0.3;
  c->rho = mat ? mat->rho : 2400.0;
  if (!(c->E > 0) || !(c->nu > -1.0) || !(c->nu < 0.5)) throw Fail{CFEM_ERR_INVALID_ARGUMENT, "invalid material"};
  if (c->dim == 3) {
    c->lam = c->E * c->nu / ((1 + c->nu) * (1 - 2 * c->nu));
    c->mu = c->E / (2 * (1 + c->nu));
  } else {  // plane stress (datakeeper.cpp:100-104)
    c->lam = c->E * c->nu / (1 - c->nu * c->nu);
    c->mu = c->E / (2 * (1 + c->nu));
  }
  CK(cudaGetDevice(&c->device));
  CK(cudaDeviceGetAttribute(&c->n_sm, cudaDevAttrMultiProcessorCount, c->device));
  CK(cudaDeviceGetAttribute(&c->l2_bytes, cudaDevAttrL2CacheSize, c->device));
  int pe = opt && opt->patch_elems > 0 ? opt->patch_elems : (c->fans ? kFanMax * kFanThreads : 512);
  // the per-incidence force slots of a patch must fit in shared memory
  pe = std::min(std::max((pe + 31) / 32 * 32, 32), m->dim == 2 ? 2048 : 1024);
  if (c->n_inst && !c->fans) throw Fail{CFEM_ERR_UNSUPPORTED, "batched meshes need the 3D edge-fan form"};
  std::string err = build_prep(*m, pe, c->fans, c->prep, c->elem_group.empty() ? nullptr : c->elem_group.data());
  if (!err.empty()) throw Fail{CFEM_ERR_MESH, err};
  err = build_rhs(*m, c->prep, c->semantics, c->rhs);
  if (!err.empty()) throw Fail{CFEM_ERR_MESH, err};
  c->elems_caller.assign(m->elems, m->elems + c->ne * c->nv);
  if (m->elem_young) {
    c->young.assign(m->elem_young, m->elem_young + c->ne);
    for (double y : c->young)
      if (!(y > 0)) throw Fail{CFEM_ERR_INVALID_ARGUMENT, "per-element Young's modulus must be positive"};
  }
  const Prep &P = c->prep;
  cudaStream_t s = c->stream;
  c->elem_off.upload(P.p_elem_off.data(), P.p_elem_off.size(), s);
  c->node_off.upload(P.p_node_off.data(), P.p_node_off.size(), s);
  c->nodes.upload(P.p_nodes.data(), P.p_nodes.size(), s);
  c->own.upload(P.p_own.data(), P.p_own.size(), s);
  c->node_new2old.upload(P.node_new2old.data(), P.node_new2old.size(), s);
  c->node_old2new.upload(P.node_old2new.data(), P.node_old2new.size(), s);
  c->elem_new2old.upload(P.elem_new2old.data(), P.elem_new2old.size(), s);
  c->elem_old2new.upload(P.elem_old2new.data(), P.elem_old2new.size(), s);
  c->lconn.upload(reinterpret_cast<const uint2 *>(P.lconn.data()), (size_t)c->ne, s);
  {
    c->inc.upload(P.inc.data(), P.inc.size(), s);
    c->inc_start.upload(P.inc_start.data(), P.inc_start.size(), s);
  }
  if (c->fans) {
    c->fstride = (P.n_fans + 31) / 32 * 32;
    std::vector<uint16_t> slot((size_t)kFanSlots * c->fstride, 0);
    for (int64_t f = 0; f < P.n_fans; ++f)
      for (int k = 0; k < kFanSlots; ++k) slot[(size_t)k * c->fstride + f] = P.fan_slot[f * kFanSlots + k];
    c->fan_slot.upload(slot.data(), slot.size(), s);
    c->fan_off.upload(P.p_fan_off.data(), P.p_fan_off.size(), s);
    c->fan_elem_off.upload(P.fan_elem_off.data(), P.fan_elem_off.size(), s);
    c->finc.upload(P.finc.data(), P.finc.size(), s);
    c->finc_start.upload(P.finc_start.data(), P.finc_start.size(), s);
    std::vector<int32_t> pos(c->ne);
    for (int64_t f = 0; f < P.n_fans; ++f)
      for (int32_t e = P.fan_elem_off[f]; e < P.fan_elem_off[f + 1]; ++e) pos[e] = (int32_t)(f * 8 + (e - P.fan_elem_off[f]));
    c->fan_pos.upload(pos.data(), pos.size(), s);
    c->fan_perm.upload(P.fan_perm.data(), P.fan_perm.size(), s);
    // patch blocks: the non-gradient prefix is built here, the gradients by
    // k_fan_block_gradients whenever the operator is (re)built
    std::vector<int32_t> fan_patch(P.n_fans);
    for (int p = 0; p < P.n_patches; ++p)
      for (int32_t f = P.p_fan_off[p]; f < P.p_fan_off[p + 1]; ++f) fan_patch[f] = p;
    c->fan_patch.upload(fan_patch.data(), fan_patch.size(), s);
    c->L32 = fan_block_layout(P.np_max, sizeof(float));
    const size_t pre = (size_t)c->L32.g_off;
    std::vector<unsigned char> hb(pre * P.n_patches, 0);
    for (int p = 0; p < P.n_patches; ++p) {
      unsigned char *B = hb.data() + pre * p;
      uint32_t *sl = reinterpret_cast<uint32_t *>(B + c->L32.slot_off);
      uint32_t *fp = reinterpret_cast<uint32_t *>(B + c->L32.fpos_off);
      uint16_t *fst = reinterpret_cast<uint16_t *>(B + c->L32.fstart_off);
      int32_t *nd = reinterpret_cast<int32_t *>(B + c->L32.nodes_off);
      uint8_t *bt = B + c->L32.bits_off;
      const int f0 = P.p_fan_off[p], nf = P.p_fan_off[p + 1] - f0;
      const int nb = P.p_node_off[p], n = P.p_node_off[p + 1] - nb;
      int32_t *hdr = reinterpret_cast<int32_t *>(B + c->L32.hdr_off);
      hdr[0] = n;
      hdr[1] = P.p_own[p];
      hdr[2] = nf;
      hdr[3] = 0;
      // slots of half-thread t = 2 fl + h (kNoSlot where absent), two per word
      for (int t = 0; t < kHfanThreads; ++t) {
        const int fl = t >> 1, h = t & 1;
        const int len = fl < nf ? P.fan_slot[(size_t)(f0 + fl) * kFanSlots + kFanSlots - 1] : 0;
        for (int k = 0; k < 6; ++k) {
          const uint32_t v = k < half_slot_count(h, len)
                                 ? P.fan_slot[(size_t)(f0 + fl) * kFanSlots + half_slot_to_fan(h, k)]
                                 : kNoSlot;
          sl[(k >> 1) * kHfanThreads + t] |= v << (16 * (k & 1));
        }
      }
      // half-fan incidences (fan fl, half h, slot hs), counting-sorted by node
      std::vector<int> cnt(n + 1, 0);
      for (int fl = 0; fl < nf; ++fl) {
        const int len = P.fan_slot[(size_t)(f0 + fl) * kFanSlots + kFanSlots - 1];
        for (int h = 0; h < 2; ++h)
          for (int hs = 0; hs < half_slot_count(h, len); ++hs)
            if (half_writes(h, hs)) ++cnt[P.fan_slot[(size_t)(f0 + fl) * kFanSlots + half_slot_to_fan(h, hs)] + 1];
      }
      for (int i = 0; i < n; ++i) cnt[i + 1] += cnt[i];
      const int total = cnt[n];
      for (int i = 0; i < c->L32.nps; ++i) fst[i] = (uint16_t)(i <= n ? cnt[i] : total);
      // Positions inside a node's run are free to choose (the node sum adds
      // the whole run). The kernel stores slot hs of all half-threads of a warp
      // with one 16-byte store instruction, served eight lanes (a quarter warp)
      // per shared-memory wavefront when their addresses fall in different
      // 16-byte bank groups (position mod 8; the force list starts 128-byte
      // aligned). Positions are handed out per quarter warp and slot, the
      // lanes with the fewest free positions first, each taking a free position
      // of its node's run in a bank group no other lane of the quarter warp
      // has taken where the run allows it.
      std::vector<uint8_t> taken(total, 0);
      for (int q0 = 0; q0 < 2 * nf; q0 += 8)
        for (int hs = 0; hs < 6; ++hs) {
          int lane_t[8], lane_node[8], m = 0;
          for (int t = q0; t < q0 + 8 && t < 2 * nf; ++t) {
            const int fl = t >> 1, h = t & 1;
            const int len = P.fan_slot[(size_t)(f0 + fl) * kFanSlots + kFanSlots - 1];
            if (hs < half_slot_count(h, len) && half_writes(h, hs)) {
              lane_t[m] = t;
              lane_node[m] = P.fan_slot[(size_t)(f0 + fl) * kFanSlots + half_slot_to_fan(h, hs)];
              ++m;
            }
          }
          auto free_in_run = [&](int node) {
            int k = 0;
            for (int p = cnt[node]; p < cnt[node + 1]; ++p) k += !taken[p];
            return k;
          };
          unsigned used = 0;
          bool done[8] = {false, false, false, false, false, false, false, false};
          for (int r = 0; r < m; ++r) {
            int best = -1, best_free = 1 << 30;
            for (int e = 0; e < m; ++e)
              if (!done[e]) {
                const int fr = free_in_run(lane_node[e]);
                if (fr < best_free) best = e, best_free = fr;
              }
            const int node = lane_node[best];
            int pos = -1;
            for (int p = cnt[node]; p < cnt[node + 1] && pos < 0; ++p)
              if (!taken[p] && !((used >> (p & 7)) & 1u)) pos = p;
            for (int p = cnt[node]; p < cnt[node + 1] && pos < 0; ++p)
              if (!taken[p]) pos = p;
            taken[pos] = 1;
            used |= 1u << (pos & 7);
            done[best] = true;
            fp[(hs >> 1) * kHfanThreads + lane_t[best]] |= (uint32_t)pos << (16 * (hs & 1));
          }
        }
      for (int i = 0; i < c->L32.npn; ++i) {
        nd[i] = i < n ? P.p_nodes[nb + i] : P.p_nodes[nb];
        bt[i] = i < n ? P.node_bits[P.p_nodes[nb + i]] : 0;
      }
    }
    c->blk32.alloc((size_t)c->L32.bytes * P.n_patches);
    c->blk32.zero(s);
    CK(cudaMemcpy2DAsync(c->blk32.p, c->L32.bytes, hb.data(), pre, pre, P.n_patches, cudaMemcpyHostToDevice, s));
    CK(cudaStreamSynchronize(s));  // hb is pageable and goes out of scope
    c->tma_err.alloc(1);
    c->tma_err.zero(s);
    CK(cudaMallocHost(&c->h_tma_err, sizeof(int)));
  }
  if (c->n_inst) {
    // instance tables: patch -> instance, instance patch ranges, owned node ranges, materials
    std::vector<int32_t> pinst(P.n_patches), ipo(c->n_inst + 1, 0), ofirst(P.n_patches + 1);
    std::vector<float> pm32(2 * (size_t)P.n_patches);
    std::vector<double> pm64(2 * (size_t)P.n_patches), le(c->ne), me(c->ne);
    int64_t running = 0;
    for (int p = 0; p < P.n_patches; ++p) {
      pinst[p] = c->elem_group[P.elem_new2old[P.p_elem_off[p]]];
      if (p && pinst[p] < pinst[p - 1]) throw Fail{CFEM_ERR_MESH, "internal error: batch patches out of order"};
      ++ipo[pinst[p] + 1];
      ofirst[p] = (int32_t)running;
      const int nb = P.p_node_off[p], n = P.p_node_off[p + 1] - nb, own = P.p_own[p];
      if (own < n && P.p_nodes[nb + own] != running) throw Fail{CFEM_ERR_MESH, "internal error: owned node ranges"};
      running += n - own;
      pm32[2 * p] = (float)c->inst_lam[pinst[p]];
      pm32[2 * p + 1] = (float)c->inst_mu[pinst[p]];
      pm64[2 * p] = c->inst_lam[pinst[p]];
      pm64[2 * p + 1] = c->inst_mu[pinst[p]];
    }
    ofirst[P.n_patches] = (int32_t)running;
    if (running != c->nn) throw Fail{CFEM_ERR_MESH, "internal error: owned node count"};
    for (int i = 0; i < c->n_inst; ++i) ipo[i + 1] += ipo[i];
    for (int64_t e = 0; e < c->ne; ++e) {
      const int g = c->elem_group[P.elem_new2old[e]];
      le[e] = c->inst_lam[g];
      me[e] = c->inst_mu[g];
    }
    c->patch_inst.upload(pinst.data(), pinst.size(), s);
    c->inst_patch_off.upload(ipo.data(), ipo.size(), s);
    c->own_first.upload(ofirst.data(), ofirst.size(), s);
    c->pmat32.upload(pm32.data(), pm32.size(), s);
    c->pmat64.upload(pm64.data(), pm64.size(), s);
    c->lam_e.upload(le.data(), le.size(), s);
    c->mu_e.upload(me.data(), me.size(), s);
    CK(cudaStreamSynchronize(s));
  }
  c->bits.upload(P.node_bits.data(), P.node_bits.size(), s);
  // coordinates and global connectivity in the new order (setup + checks)
  {
    std::vector<double> xyz((size_t)c->nn * c->dim);
    for (int64_t n = 0; n < c->nn; ++n)
      for (int d = 0; d < c->dim; ++d) xyz[n * c->dim + d] = m->nodes[(int64_t)P.node_new2old[n] * c->dim + d];
    c->coords.upload(xyz.data(), xyz.size(), s);
    std::vector<int32_t> cn((size_t)c->ne * c->nv);
    for (int64_t e = 0; e < c->ne; ++e)
      for (int a = 0; a < c->nv; ++a)
        cn[e * c->nv + a] = P.node_old2new[m->elems[(int64_t)P.elem_new2old[e] * c->nv + a]];
    c->conn.upload(cn.data(), cn.size(), s);
  }
  rebuild_operator(c);
  // right-hand side parts in the internal layout
  c->io.alloc(c->nd);
  c->FA.alloc(c->nvec);
  c->FB.alloc(c->nvec);
  c->FA32.alloc(c->nvec);
  c->FB32.alloc(c->nvec);
  c->v64.f.alloc(c->nvec);
  // work vectors
  for (auto *b : {&c->v64.x, &c->v64.r, &c->v64.z, &c->v64.pA, &c->v64.pB, &c->v64.u, &c->v64.uB, &c->v64.dinv,
                  &c->v64.diagA}) {
    b->alloc(c->nvec);
    b->zero(s);
  }
  c->v64.f.zero(s);
  for (auto *b : {&c->v32.x, &c->v32.r, &c->v32.z, &c->v32.pA, &c->v32.pB, &c->v32.u, &c->v32.uB, &c->v32.f,
                  &c->v32.dinv, &c->v32.diagA}) {
    b->alloc(c->nvec);
    b->zero(s);
  }
  c->tmp64.alloc(c->nvec);
  c->tmp64b.alloc(c->nvec);
  c->tmp64.zero(s);
  c->tmp64b.zero(s);
  to_internal<double>(c, c->rhs.FA.data(), c->FA.p);
  to_internal<double>(c, c->rhs.FB.data(), c->FB.p);
  k_convert<double, float><<<nblk(c->nvec), kThreads, 0, s>>>(c->nvec, c->FA.p, c->FA32.p);
  k_convert<double, float><<<nblk(c->nvec), kThreads, 0, s>>>(c->nvec, c->FB.p, c->FB32.p);
  CKL();
  // launch shapes
  c->np_slots = (P.np_max + 3) / 4 * 4;
  c->smem64 = matvec_smem_bytes(c->dim, sizeof(double), P.patch_elems, c->np_slots);
  c->smem32 = matvec_smem_bytes(c->dim, sizeof(float), P.patch_elems, c->np_slots);
  // The limit is an attribute of the kernel function (shared by every context
  // in the process), so it is raised once to the device maximum; each launch
  // still requests only its own patch size.
  int smem_optin = 0;
  CK(cudaDeviceGetAttribute(&smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, c->device));
  if (c->smem64 + 8192 > (size_t)smem_optin)
    throw Fail{CFEM_ERR_INVALID_ARGUMENT, "patch too large for shared memory: lower patch_elems"};
  auto set_smem = [&](const void *k, size_t) {
    CK(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_optin - 8192));
  };
  int occ = 1;
  if (c->dim == 3) {
    set_smem((const void *)k_matvec<double, 3, MV_PLAIN>, c->smem64);
    set_smem((const void *)k_matvec<double, 3, MV_PCG>, c->smem64);
    set_smem((const void *)k_matvec<double, 3, MV_DYN>, c->smem64);
    set_smem((const void *)k_matvec<float, 3, MV_PLAIN>, c->smem32);
    set_smem((const void *)k_matvec<float, 3, MV_PCG>, c->smem32);
    set_smem((const void *)k_matvec<float, 3, MV_DYN>, c->smem32);
    CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_matvec<float, 3, MV_PCG>, kThreads, c->smem32));
  } else {
    set_smem((const void *)k_matvec<double, 2, MV_PLAIN>, c->smem64);
    set_smem((const void *)k_matvec<double, 2, MV_PCG>, c->smem64);
    set_smem((const void *)k_matvec<double, 2, MV_DYN>, c->smem64);
    set_smem((const void *)k_matvec<float, 2, MV_PLAIN>, c->smem32);
    set_smem((const void *)k_matvec<float, 2, MV_PCG>, c->smem32);
    set_smem((const void *)k_matvec<float, 2, MV_DYN>, c->smem32);
    CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_matvec<float, 2, MV_PCG>, kThreads, c->smem32));
  }
  occ = std::max(occ, 1);
  c->grid_mv = (int)std::min<int64_t>(P.n_patches, (int64_t)c->n_sm * occ);
  if (c->fans) {
    c->smem_fan64 = fan_smem_bytes(sizeof(double), c->np_slots);
    c->smem_fan32 = fan_smem_bytes(sizeof(float), c->np_slots);
    if (c->smem_fan64 + 8192 > (size_t)smem_optin)
      throw Fail{CFEM_ERR_INVALID_ARGUMENT, "fan patch too large for shared memory: lower patch_elems"};
    for (const void *k : {(const void *)k_matvec_fan<double, MV_PLAIN>, (const void *)k_matvec_fan<double, MV_PCG>,
                          (const void *)k_matvec_fan<double, MV_DYN>, (const void *)k_matvec_fan<float, MV_PLAIN>,
                          (const void *)k_matvec_fan<float, MV_PCG>, (const void *)k_matvec_fan<float, MV_DYN>})
      CK(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_optin - 8192));
    int occf = 1;
    CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occf, k_matvec_fan<float, MV_PCG>, kFanThreads, c->smem_fan32));
    c->grid_fan = (int)std::min<int64_t>(P.n_patches, (int64_t)c->n_sm * std::max(occf, 1));
    c->smem_ft32 = fan_tma_smem_bytes(c->L32, sizeof(float));
    if (c->smem_ft32 + 8192 > (size_t)smem_optin) c->fan_tma = false;
    if (c->fan_tma) {
      for (const void *k : {(const void *)k_matvec_fan_tma<float, MV_PLAIN>, (const void *)k_matvec_fan_tma<float, MV_PCG>,
                            (const void *)k_matvec_fan_tma<float, MV_DYN>,
                            (const void *)k_matvec_fan_tma<float, MV_PLAIN, false, true>,
                            (const void *)k_matvec_fan_tma<float, MV_PCG, false, true>,
                            (const void *)k_matvec_fan_tma<float, MV_PCG, false, false, true>})
        CK(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_optin - 8192));
      int o32 = 1;
      CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o32, k_matvec_fan_tma<float, MV_PCG>, kHfanThreads, c->smem_ft32));
      c->grid_ft32 = (int)std::min<int64_t>(P.n_patches, (int64_t)c->n_sm * std::max(o32, 1));
    }
    if (c->geo && !c->fan_tma) throw Fail{CFEM_ERR_INVALID_ARGUMENT, "fan patch too large for shared memory: lower patch_elems"};
    if (c->geo) {
      // the largest layout (with scale rows) bounds the shared memory of every later rebuild
      const size_t smem_max = fan_tma_smem_bytes(fan_geo_block_layout(P.np_max, true), sizeof(float));
      for (const void *k : {(const void *)k_matvec_fan_tma<float, MV_PLAIN, true>,
                            (const void *)k_matvec_fan_tma<float, MV_PCG, true>,
                            (const void *)k_matvec_fan_tma<float, MV_DYN, true>,
                            (const void *)k_matvec_fan_tma<float, MV_PLAIN, true, true>,
                            (const void *)k_matvec_fan_tma<float, MV_PCG, true, true>})
        CK(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_max));
    }
  }
  c->grid_vec = (int)std::min<int64_t>(std::max<int64_t>(1, nblk(c->nn)), (int64_t)c->n_sm * 4);
  // PCG update: two CTAs per SM keep enough loads in flight for the bandwidth
  // and leave room for the next matvec's CTAs to start early (PDL)
  c->grid_upd = (int)std::min<int64_t>(std::max<int64_t>(1, nblk(c->nn)), (int64_t)c->n_sm * 2);
  if (c->geo) {  // the grid of the largest geometry layout fits every later one
    int og = 1;
    const size_t smem_max = fan_tma_smem_bytes(fan_geo_block_layout(P.np_max, true), sizeof(float));
    CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&og, k_matvec_fan_tma<float, MV_PCG, true>, kHfanThreads,
                                                     smem_max));
    c->grid_geo = (int)std::min<int64_t>(P.n_patches, (int64_t)c->n_sm * std::max(og, 1));
  }
  int maxgrid = std::max({c->grid_mv, c->grid_vec, c->grid_fan, c->grid_ft32, c->grid_geo});
  c->partials.alloc((size_t)maxgrid * 4);
  c->partials_up.alloc((size_t)std::max(c->grid_upd, c->grid_vec) * 2);
  c->partials_up.zero(s);
  c->counters.alloc(4);
  c->counters.zero(s);
  c->rr.alloc(4);
  c->sc.alloc(3);
  c->sc.zero(s);
  CK(cudaMallocHost(&c->h_sc, sizeof(Scalars)));
  CK(cudaMallocHost(&c->h_rr, 4 * sizeof(double)));
  CK(cudaEventCreate(&c->ev0));
  CK(cudaEventCreate(&c->ev1));
  CK(cudaStreamSynchronize(s));
}

// Geometry blocks from the gradient blocks' prefix (slot .. bits), the
// patch-relative coordinates and, with per-element moduli, the scale rows.
static void build_geo_blocks(cfem_ctx *c) {
  cudaStream_t s = c->stream;
  const Prep &P = c->prep;
  const bool with_scale = !c->young.empty();
  const FanBlockLayout L = fan_geo_block_layout(P.np_max, with_scale);
  if (!c->blkg.p || L.bytes != c->Lg.bytes || L.c_off != c->Lg.c_off) c->blkg.alloc((size_t)L.bytes * P.n_patches);
  c->Lg = L;
  c->blkg.zero(s);
  CK(cudaMemcpy2DAsync(c->blkg.p, L.bytes, c->blk32.p, c->L32.bytes, (size_t)c->L32.g_off, P.n_patches,
                       cudaMemcpyDeviceToDevice, s));
  k_fan_block_coords<<<P.n_patches, 128, 0, s>>>(c->node_off.p, c->nodes.p, c->coords.p, c->blkg.p, L);
  CKL();
  if (with_scale) {
    k_fan_block_scales<<<nblk(c->ne), kThreads, 0, s>>>(c->ne, c->escale.p, c->fan_pos.p, c->fan_patch.p, c->fan_off.p,
                                                        c->blkg.p, L);
    CKL();
  }
  c->smem_geo = fan_tma_smem_bytes(L, sizeof(float));
}

// (Re)builds the element operator: scaled gradients, volumes, assembled
// diagonal and masses (calculateKlocals / calculateMlocals equivalents).
void rebuild_operator(cfem_ctx *c) {
  cudaStream_t s = c->stream;
  const Prep &P = c->prep;
  (void)P;
  if (!c->young.empty()) {
    std::vector<double> sc(c->ne);
    for (int64_t e = 0; e < c->ne; ++e) sc[e] = c->young[c->prep.elem_new2old[e]] / c->E;
    c->escale.upload(sc.data(), sc.size(), s);
    c->young_d.upload(c->young.data(), c->young.size(), s);
  }
  c->gstride = (c->ne + 31) / 32 * 32;
  c->G64.alloc((size_t)c->ncomp * c->gstride);
  c->G32.alloc((size_t)c->ncomp * c->gstride);
  c->vol.alloc(c->ne);
  c->mc64.alloc(c->ne);
  c->mc32.alloc(c->ne);
  c->diagK.alloc(c->nvec);
  c->mlump.alloc(c->nvec);
  c->mcdiag.alloc(c->nvec);
  c->diagK.zero(s);
  c->mlump.zero(s);
  c->mcdiag.zero(s);
  if (!c->err.p) c->err.alloc(1);
  c->err.zero(s);
  c->G64.zero(s);
  c->G32.zero(s);
  // mass factors: lumped per DOF and consistent coefficient (M_ab = c (1 + delta_ab) rho V)
  double &lump_c = c->lump_c, &cons_c = c->cons_c;
  if (c->dim == 2) { lump_c = 1.0 / 3; cons_c = 1.0 / 12; }
  else if (c->semantics == CFEM_COMPAT) { lump_c = 1.0 / 12; cons_c = 1.0 / 48; }  // cpu_fem_utils.cpp:656-726
  else { lump_c = 1.0 / 4; cons_c = 1.0 / 20; }
  GeomParams gp{};
  gp.ne = c->ne;
  gp.gstride = c->gstride;
  gp.coords = c->coords.p;
  gp.conn = c->conn.p;
  gp.escale = c->escale.p;
  gp.lam = c->lam;
  gp.mu = c->mu;
  gp.rho = c->rho;
  gp.lump_c = lump_c;
  gp.cons_c = cons_c;
  gp.G64 = c->G64.p;
  gp.G32 = c->G32.p;
  gp.vol = c->vol.p;
  gp.diagK = c->diagK.p;
  gp.mlump = c->mlump.p;
  gp.mc64 = c->mc64.p;
  gp.mc32 = c->mc32.p;
  gp.diag_local = nullptr;
  gp.elem_new2old = c->elem_new2old.p;
  gp.err = c->err.p;
  gp.lam_e = c->lam_e.p;
  gp.mu_e = c->mu_e.p;
  if (c->dim == 3) k_geometry<3><<<nblk(c->ne), kThreads, 0, s>>>(gp);
  else k_geometry<2><<<nblk(c->ne), kThreads, 0, s>>>(gp);
  CKL();
  if (c->fans) {
    if (!c->Gf64.p) {
      c->Gf64.alloc((size_t)kFanMax * 9 * c->fstride);
      c->Gf32.alloc((size_t)kFanMax * 9 * c->fstride);
    }
    c->Gf64.zero(s);
    c->Gf32.zero(s);
    k_fan_gradients<<<nblk(c->ne), kThreads, 0, s>>>(c->ne, c->G64.p, c->gstride, c->fan_pos.p, c->fan_perm.p, c->Gf64.p,
                                                     c->Gf32.p, c->fstride);
    CKL();
    k_fan_block_gradients<<<nblk(c->ne), kThreads, 0, s>>>(c->ne, c->G64.p, c->gstride, c->fan_pos.p, c->fan_perm.p,
                                                           c->fan_patch.p, c->fan_off.p, c->blk32.p, c->L32);
    CKL();
    if (c->geo) build_geo_blocks(c);
  }
  // consistent-mass diagonal: 2 * cons_c * rho * V per DOF, assembled = mlump * 2 cons_c / lump_c
  k_axpby64<<<nblk(c->nvec), kThreads, 0, s>>>(c->nvec, 2 * cons_c / lump_c, c->mlump.p, 0.0, c->mcdiag.p);
  CKL();
  int herr = 0;
  c->diagK32.alloc(c->nvec);
  k_convert<double, float><<<nblk(c->nvec), kThreads, 0, s>>>(c->nvec, c->diagK.p, c->diagK32.p);
  CKL();
  CK(cudaMemcpyAsync(&herr, c->err.p, sizeof(int), cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  if (herr) throw Fail{CFEM_ERR_MESH, "an element has zero or non-finite volume"};
}

void enter(cfem_ctx *c) {
  if (c->own_stream) {
    CK(cudaEventRecord(c->ev_in, c->user_stream));
    CK(cudaStreamWaitEvent(c->stream, c->ev_in, 0));
  }
}

// The legacy default stream cannot be captured into a CUDA graph; a context
// given it (or NULL) issues its work on a stream of its own and orders that
// stream after the caller's at every entry point that reads caller memory.
void attach_stream(cfem_ctx *c, cudaStream_t s) {
  if (c->own_stream && c->stream) {
    CK(cudaStreamSynchronize(c->stream));
    cudaStreamDestroy(c->stream);
    c->stream = nullptr;
    c->own_stream = false;
  }
  c->user_stream = s;
  if (s == nullptr || s == cudaStreamLegacy || s == cudaStreamPerThread) {
    CK(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
    c->own_stream = true;
    if (!c->ev_in) CK(cudaEventCreateWithFlags(&c->ev_in, cudaEventDisableTiming));
  } else {
    c->stream = s;
  }
}

void check_copy_error(cfem_ctx *c) {
  if (!c->h_tma_err) return;
  CK(cudaMemcpyAsync(c->h_tma_err, c->tma_err.p, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  if (*c->h_tma_err) {
    c->tma_err.zero(c->stream);
    throw Fail{CFEM_ERR_CUDA, "a bulk copy of the edge-fan matvec did not complete in time"};
  }
}

void check_ctx(const cfem_ctx *c) {
  if (!c) throw Fail{CFEM_ERR_INVALID_ARGUMENT, "null context"};
}

cfem_solve_params default_params() {
  cfem_solve_params p{};
  p.precision = CFEM_FP64;
  p.stop_rule = CFEM_STOP_REFERENCE;
  p.tol = 1e-8;
  p.max_iter = 1000000;
  p.outer_tol = 1e-12;
  p.max_outer = 50;
  return p;
}

}  // namespace detail
}  // namespace cfem

extern "C" {

int32_t cfem_abi_version(void) { return CFEM_ABI_VERSION; }

const char *cfem_last_error_string(void) { return g_last_error.c_str(); }

// used by the C++ host layer (femfunc.cpp) to report its own failures
void cfem_set_error_string(const char *msg) { g_last_error = msg ? msg : ""; }

cfem_status cfem_create(cfem_ctx **out, const cfem_mesh *mesh, const cfem_material *mat, const cfem_options *opt,
                        void *stream) {
  return run_guarded([&]() -> cfem_status {
    if (!out || !mesh) throw Fail{CFEM_ERR_INVALID_ARGUMENT, "null argument"};
    *out = nullptr;
    if (!mesh->nodes || !mesh->elems) throw Fail{CFEM_ERR_INVALID_ARGUMENT, "mesh without nodes or elements"};
    if ((mesh->n_constraints > 0 && !mesh->constraints) || (mesh->n_loads > 0 && (!mesh->load_nodes || !mesh->load_vectors)) ||
        (mesh->n_faces > 0 && (!mesh->face_nodes || !mesh->face_elems || !mesh->face_normals || !mesh->face_pressures)))
      throw Fail{CFEM_ERR_INVALID_ARGUMENT, "mesh count given without its array"};
    std::unique_ptr<cfem_ctx> c(new cfem_ctx());
    attach_stream(c.get(), (cudaStream_t)stream);
    setup_context(c.get(), mesh, mat, opt);
    *out = c.release();
    return CFEM_OK;
  });
}

void cfem_destroy(cfem_ctx *ctx) {
  if (!ctx) return;
  cudaStreamSynchronize(ctx->stream);
  delete ctx;
}

cfem_status cfem_set_stream(cfem_ctx *ctx, void *stream) {
  return run_guarded([&]() -> cfem_status {
    check_ctx(ctx);
    CK(cudaStreamSynchronize(ctx->stream));
    attach_stream(ctx, (cudaStream_t)stream);
    ctx->graph64.reset();
    ctx->graph32.reset();
    return CFEM_OK;
  });
}

cfem_status cfem_synchronize(cfem_ctx *ctx) {
  return run_guarded([&]() -> cfem_status {
    check_ctx(ctx);
    CK(cudaStreamSynchronize(ctx->stream));
    return CFEM_OK;
  });
}

cfem_status cfem_get_counts(const cfem_ctx *ctx, int64_t *counts) {
  return run_guarded([&]() -> cfem_status {
    check_ctx(ctx);
    if (!counts) throw Fail{CFEM_ERR_INVALID_ARGUMENT, "null counts"};
    counts[0] = ctx->dim; counts[1] = ctx->nn; counts[2] = ctx->ne; counts[3] = ctx->nd;
    counts[4] = ctx->prep.n_patches; counts[5] = ctx->form;
    return CFEM_OK;
  });
}

cfem_status cfem_dof_map(const cfem_ctx *ctx, int32_t *mask) {
  return run_guarded([&]() -> cfem_status {
    check_ctx(ctx);
    if (!mask) throw Fail{CFEM_ERR_INVALID_ARGUMENT, "null mask"};
    // element-local slot (caller element e, vertex a, component d) -> dim*node + d
    const Prep &P = ctx->prep;
    for (int patch = 0; patch < P.n_patches; ++patch)
      for (int64_t ei = P.p_elem_off[patch]; ei < P.p_elem_off[patch + 1]; ++ei) {
        int64_t e = P.elem_new2old[ei];
        for (int a = 0; a < ctx->nv; ++a) {
          int g = P.p_nodes[P.p_node_off[patch] + P.lconn[ei * 4 + a]];
          int64_t node = P.node_new2old[g];
          for (int d = 0; d < ctx->dim; ++d) mask[e * ctx->w + ctx->dim * a + d] = (int32_t)(ctx->dim * node + d);
        }
      }
    return CFEM_OK;
  });
}

cfem_status cfem_adjacency(const cfem_ctx *ctx, int32_t *adj) {
  return run_guarded([&]() -> cfem_status {
    check_ctx(ctx);
    if (!adj) throw Fail{CFEM_ERR_INVALID_ARGUMENT, "null adj"};
    std::fill(adj, adj + ctx->nd, 0);
    const Prep &P = ctx->prep;
    for (int patch = 0; patch < P.n_patches; ++patch)
      for (int64_t ei = P.p_elem_off[patch]; ei < P.p_elem_off[patch + 1]; ++ei)
        for (int a = 0; a < ctx->nv; ++a) {
          int64_t node = P.node_new2old[P.p_nodes[P.p_node_off[patch] + P.lconn[ei * 4 + a]]];
          for (int d = 0; d < ctx->dim; ++d) adj[node * ctx->dim + d] += 1;
        }
    return CFEM_OK;
  });
}

cfem_status cfem_bc_mask(const cfem_ctx *ctx, uint8_t *constrained) {
  return run_guarded([&]() -> cfem_status {
    check_ctx(ctx);
    if (!constrained) throw Fail{CFEM_ERR_INVALID_ARGUMENT, "null output"};
    const Prep &P = ctx->prep;
    for (int64_t g = 0; g < ctx->nn; ++g) {
      int64_t o = P.node_new2old[g];
      for (int d = 0; d < ctx->dim; ++d) constrained[o * ctx->dim + d] = (P.node_bits[g] >> d) & 1u;
    }
    return CFEM_OK;
  });
}

cfem_status cfem_renumbering(const cfem_ctx *ctx, int32_t *node_new2old, int32_t *elem_new2old) {
  return run_guarded([&]() -> cfem_status {
    check_ctx(ctx);
    if (node_new2old) std::copy(ctx->prep.node_new2old.begin(), ctx->prep.node_new2old.end(), node_new2old);
    if (elem_new2old) std::copy(ctx->prep.elem_new2old.begin(), ctx->prep.elem_new2old.end(), elem_new2old);
    return CFEM_OK;
  });
}

cfem_status cfem_element_matrices(cfem_ctx *ctx, int64_t first, int64_t count, double *ke) {
  return run_guarded([&]() -> cfem_status {
    check_ctx(ctx);
    if (ctx->n_inst) throw Fail{CFEM_ERR_UNSUPPORTED, "not available for a context of batched meshes"};
    if (!ke || first < 0 || count < 0 || first + count > ctx->ne) throw Fail{CFEM_ERR_INVALID_ARGUMENT, "bad element range"};
    if (count == 0) return CFEM_OK;
    DBuf<double> out;
    out.alloc((size_t)count * ctx->w * ctx->w);
    if (ctx->dim == 3)
      k_element_matrices<3><<<nblk(count), kThreads, 0, ctx->stream>>>(first, count, ctx->elem_old2new.p, ctx->G64.p, ctx->gstride,
                                                                        ctx->conn.p, ctx->bits.p, ctx->lam, ctx->mu, out.p);
    else
      k_element_matrices<2><<<nblk(count), kThreads, 0, ctx->stream>>>(first, count, ctx->elem_old2new.p, ctx->G64.p, ctx->gstride,
                                                                        ctx->conn.p, ctx->bits.p, ctx->lam, ctx->mu, out.p);
    CKL();
    CK(cudaMemcpyAsync(ke, out.p, sizeof(double) * out.n, cudaMemcpyDefault, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    return CFEM_OK;
  });
}

cfem_status cfem_diagonal(cfem_ctx *ctx, double *diag) {
  return run_guarded([&]() -> cfem_status {
    check_ctx(ctx);
    if (!diag) throw Fail{CFEM_ERR_INVALID_ARGUMENT, "null output"};
    to_caller<double>(ctx, ctx->diagK.p, diag);
    CK(cudaStreamSynchronize(ctx->stream));
    return CFEM_OK;
  });
}

cfem_status cfem_rhs(cfem_ctx *ctx, const cfem_wavelet *w, double t, double *f) {
  return run_guarded([&]() -> cfem_status {
    check_ctx(ctx);
    if (!f) throw Fail{CFEM_ERR_INVALID_ARGUMENT, "null output"};
    RhsSchedule sch;
    sch.semantics = ctx->semantics;
    sch.has_loads = ctx->rhs.has_loads;
    sch.w = w;
    double a = 0, b = 0;
    if (t != 0.0) sch.eval(0.f, a, b);  // initFlocals(0) precedes calcFlocals(t)
    sch.eval((float)t, a, b);
    make_rhs(ctx, a, b, ctx->tmp64b.p);
    to_caller<double>(ctx, ctx->tmp64b.p, f);
    CK(cudaStreamSynchronize(ctx->stream));
    return CFEM_OK;
  });
}

cfem_status cfem_selftest_copy_timeout(cfem_ctx *ctx) {
  return run_guarded([&]() -> cfem_status {
    check_ctx(ctx);
    if (!(ctx->fans && ctx->fan_tma) || ctx->n_inst)
      throw Fail{CFEM_ERR_UNSUPPORTED, "the copy-timeout self-test needs a single-mesh 3D edge-fan context"};
    enter(ctx);
    // one FP32 matvec whose first block of patch 0 is never requested, with
    // the waits bounded at ~1 ms: CTA 0 must give up, flag the failure and
    // return, and the host must report it
    MvParams<float> mv = base_mv<float>(ctx);
    mv.diagA = ctx->v32.diagA.p;
    mv.x = ctx->v32.z.p;
    mv.y = ctx->v32.u.p;
    ctx->v32.z.zero(ctx->stream);
    ctx->v32.u.zero(ctx->stream);
    ctx->selftest_skip_plus1 = 1;
    ctx->selftest_wait_limit = 2000000;
    try {
      launch_mv<float>(ctx, MV_PLAIN, mv);
    } catch (...) {
      ctx->selftest_skip_plus1 = 0;
      ctx->selftest_wait_limit = 0;
      throw;
    }
    ctx->selftest_skip_plus1 = 0;
    ctx->selftest_wait_limit = 0;
    try {
      check_copy_error(ctx);
    } catch (const Fail &f) {
      if (f.st == CFEM_ERR_CUDA) return CFEM_OK;  // detected, reported and cleared
      throw;
    }
    throw Fail{CFEM_ERR_CUDA, "self-test: a withheld bulk copy was not reported"};
  });
}

cfem_status cfem_matvec(cfem_ctx *ctx, int32_t precision, const void *x, void *y) {
  return run_guarded([&]() -> cfem_status {
    check_ctx(ctx);
    enter(ctx);
    if (!x || !y) throw Fail{CFEM_ERR_INVALID_ARGUMENT, "null vector"};
    if (precision == CFEM_FP64) {
      to_internal<double>(ctx, (const double *)x, ctx->v64.z.p);
      MvParams<double> mv = base_mv<double>(ctx);
      mv.diagA = ctx->diagK.p;
      mv.x = ctx->v64.z.p;
      mv.y = ctx->tmp64.p;
      ctx->tmp64.zero(ctx->stream);
      launch_mv<double>(ctx, MV_PLAIN, mv);
      to_caller<double>(ctx, ctx->tmp64.p, (double *)y);
    } else if (precision == CFEM_FP32) {
      // float in/out: stage through FP64 conversion buffers
      DBuf<double> xin;
      xin.alloc(ctx->nd);
      DBuf<float> xf;
      xf.alloc(ctx->nd);
      CK(cudaMemcpyAsync(xf.p, x, sizeof(float) * ctx->nd, cudaMemcpyDefault, ctx->stream));
      k_convert<float, double><<<nblk(ctx->nd), kThreads, 0, ctx->stream>>>(ctx->nd, xf.p, xin.p);
      CKL();
      to_internal<float>(ctx, xin.p, ctx->v32.z.p);
      k_convert<double, float><<<nblk(ctx->nvec), kThreads, 0, ctx->stream>>>(ctx->nvec, ctx->diagK.p, ctx->v32.diagA.p);
      MvParams<float> mv = base_mv<float>(ctx);
      mv.diagA = ctx->v32.diagA.p;
      mv.x = ctx->v32.z.p;
      mv.y = ctx->v32.u.p;
      ctx->v32.u.zero(ctx->stream);
      launch_mv<float>(ctx, MV_PLAIN, mv);
      to_caller<float>(ctx, ctx->v32.u.p, xin.p);
      k_convert<double, float><<<nblk(ctx->nd), kThreads, 0, ctx->stream>>>(ctx->nd, xin.p, xf.p);
      CKL();
      CK(cudaMemcpyAsync(y, xf.p, sizeof(float) * ctx->nd, cudaMemcpyDefault, ctx->stream));
      ctx->v32.u.zero(ctx->stream);
    } else {
      throw Fail{CFEM_ERR_INVALID_ARGUMENT, "matvec precision must be CFEM_FP64 or CFEM_FP32"};
    }
    check_copy_error(ctx);
    return CFEM_OK;
  });
}

cfem_status cfem_pcg(cfem_ctx *ctx, const cfem_solve_params *prm, const double *f, double *u, cfem_solve_info *info) {
  return run_guarded([&]() -> cfem_status {
    check_ctx(ctx);
    enter(ctx);
    if (!f || !u) throw Fail{CFEM_ERR_INVALID_ARGUMENT, "null vector"};
    cfem_solve_params p = prm ? *prm : default_params();
    to_internal<double>(ctx, f, ctx->v64.f.p);
    cfem_status st = solve_internal(ctx, &p, info);
    to_caller<double>(ctx, ctx->v64.x.p, u);
    CK(cudaStreamSynchronize(ctx->stream));
    return st;
  });
}

cfem_status cfem_static_solve(cfem_ctx *ctx, const cfem_wavelet *w, const cfem_solve_params *prm, double *u,
                              cfem_solve_info *info) {
  return run_guarded([&]() -> cfem_status {
    check_ctx(ctx);
    if (!u) throw Fail{CFEM_ERR_INVALID_ARGUMENT, "null output"};
    cfem_solve_params p = prm ? *prm : default_params();
    RhsSchedule sch;
    sch.semantics = ctx->semantics;
    sch.has_loads = ctx->rhs.has_loads;
    sch.w = w;
    double a = 0, b = 0;
    sch.eval(0.f, a, b);  // initFlocals(0, wavelet)
    make_rhs(ctx, a, b, ctx->v64.f.p);
    cfem_status st = solve_internal(ctx, &p, info);
    to_caller<double>(ctx, ctx->v64.x.p, u);
    CK(cudaStreamSynchronize(ctx->stream));
    return st;
  });
}

cfem_status cfem_profile_matvec(cfem_ctx *ctx, int32_t precision, int32_t n_launches, double *ms_per_launch,
                                double *bytes_per_launch) {
  return run_guarded([&]() -> cfem_status {
    check_ctx(ctx);
    if (n_launches <= 0) throw Fail{CFEM_ERR_INVALID_ARGUMENT, "n_launches must be positive"};
    // scalars that make the kernel take its full path: an update has run
    // (u_iter 0) whose partials give r.z = 1 against gamma_prev = 1, so
    // beta = 1, and no stopping rule fires
    Scalars h{};
    h.iter = 1;
    h.u_iter = 0;
    h.gamma = h.gamma_prev = h.gamma0 = 1.0;
    h.alpha = h.beta = 1.0;
    h.maxit = 1 << 30;
    Scalars *sc = ctx->sc.p + 2;
    CK(cudaMemcpyAsync(sc, &h, sizeof(Scalars), cudaMemcpyHostToDevice, ctx->stream));
    ctx->partials_up.zero(ctx->stream);
    static const double one[2] = {1.0, 1.0};
    CK(cudaMemcpyAsync(ctx->partials_up.p, one, sizeof(one), cudaMemcpyHostToDevice, ctx->stream));
    const size_t ts = precision == CFEM_FP64 ? 8 : 4;
    auto run = [&](int n) {
      for (int i = 0; i < n; ++i) {
        if (precision == CFEM_FP64) {
          MvParams<double> mv = base_mv<double>(ctx);
          mv.diagA = ctx->v64.diagA.p;
          mv.sc = sc;
          mv.x = ctx->v64.z.p;
          mv.x2 = (i & 1) ? ctx->v64.pB.p : ctx->v64.pA.p;
          mv.xout = (i & 1) ? ctx->v64.pA.p : ctx->v64.pB.p;
          mv.y = (i & 1) ? ctx->v64.uB.p : ctx->v64.u.p;
          mv.yzero = (i & 1) ? ctx->v64.u.p : ctx->v64.uB.p;
          launch_mv<double>(ctx, MV_PCG, mv);
        } else {
          MvParams<float> mv = base_mv<float>(ctx);
          mv.diagA = ctx->v32.diagA.p;
          mv.sc = sc;
          mv.x = ctx->v32.z.p;
          mv.x2 = (i & 1) ? ctx->v32.pB.p : ctx->v32.pA.p;
          mv.xout = (i & 1) ? ctx->v32.pA.p : ctx->v32.pB.p;
          mv.y = (i & 1) ? ctx->v32.uB.p : ctx->v32.u.p;
          mv.yzero = (i & 1) ? ctx->v32.u.p : ctx->v32.uB.p;
          launch_mv<float>(ctx, MV_PCG, mv);
        }
      }
    };
    run(3);  // warm-up
    CK(cudaEventRecord(ctx->ev0, ctx->stream));
    run(n_launches);
    CK(cudaEventRecord(ctx->ev1, ctx->stream));
    CK(cudaEventSynchronize(ctx->ev1));
    float ms = 0;
    CK(cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1));
    if (ms_per_launch) *ms_per_launch = ms / n_launches;
    // algorithmic bytes: the operator (stored gradients + 8 bytes of connectivity
    // per element; geometry form: the streamed patch blocks, which hold the
    // connectivity, scatter tables and coordinates) and five node-vector
    // streams (z and p_old read, p and A p written, the next A p zeroed)
    if (bytes_per_launch)
      *bytes_per_launch = (ctx->geo && precision == CFEM_FP32
                               ? (double)ctx->prep.n_patches * ctx->Lg.bytes
                               : (double)ctx->ne * (ctx->ncomp * ts + 8)) +
                          (double)ctx->nn * ctx->vw * ts * 5;
    // leave the work vectors clean for the next solve
    if (precision == CFEM_FP64) {
      ctx->v64.u.zero(ctx->stream);
      ctx->v64.uB.zero(ctx->stream);
    } else {
      ctx->v32.u.zero(ctx->stream);
      ctx->v32.uB.zero(ctx->stream);
    }
    check_copy_error(ctx);
    return CFEM_OK;
  });
}

// Elements per CTA patch: every candidate builds the context (renumbering,
// fans, patch blocks) and times the FP32 PCG-form matvec on the device.
cfem_status cfem_autotune_patch_elems(const cfem_mesh *mesh, const cfem_material *mat, const cfem_options *opt,
                                      const int32_t *candidates, int32_t n_candidates, int32_t *best,
                                      double *ms_per_launch) {
  return run_guarded([&]() -> cfem_status {
    if (!mesh || !best) throw Fail{CFEM_ERR_INVALID_ARGUMENT, "null argument"};
    std::vector<int32_t> cand;
    if (candidates && n_candidates > 0) cand.assign(candidates, candidates + n_candidates);
    else if (mesh->dim == 3 && (!opt || opt->matvec_form != CFEM_FORM_GRADIENT)) cand = {192, 384, 576, 768};
    else cand = {256, 512, 1024};
    cfem_options o = opt ? *opt : cfem_options{CFEM_COMPAT, CFEM_FORM_AUTO, 0, 0};
    double best_ms = 1e300;
    *best = 0;
    for (size_t i = 0; i < cand.size(); ++i) {
      if (cand[i] <= 0) throw Fail{CFEM_ERR_INVALID_ARGUMENT, "candidate patch sizes must be positive"};
      o.patch_elems = cand[i];
      cfem_ctx *c = nullptr;
      cfem_status st = cfem_create(&c, mesh, mat, &o, nullptr);
      if (st != CFEM_OK) return st;
      double ms = 0, bytes = 0;
      st = cfem_profile_matvec(c, CFEM_FP32, 3, &ms, &bytes);            // warm-up
      if (st == CFEM_OK) st = cfem_profile_matvec(c, CFEM_FP32, 20, &ms, &bytes);
      cfem_destroy(c);
      if (st != CFEM_OK) return st;
      if (ms_per_launch) ms_per_launch[i] = ms;
      if (ms < best_ms) {
        best_ms = ms;
        *best = cand[i];
      }
    }
    return CFEM_OK;
  });
}

}  // extern "C"

// dynamics, multi-RHS and adjoint entry points live in context_dyn.cu

// ============================================================ no-allocation matvec
// cfem_matvec_energy_noalloc: y = K' x and e = x.K'x for callers that cannot
// allocate device memory (see include/cfem.h). Its only scratch is this fixed
// array: the per-block partial sums of e, the ticket counter of the last-block
// reduction and the result slot. It is allocated when the library is loaded
// and is held by every GPU that loads the library until the process exits.
namespace cfem {
namespace detail {

constexpr int kNoAllocMaxBlocks = 4096;  // CFEM_NOALLOC_MAX_BLOCKS in include/cfem.h
constexpr int kNoAllocCounter = kNoAllocMaxBlocks;      // slot holding the ticket counter
constexpr int kNoAllocResult = kNoAllocMaxBlocks + 1;   // slot holding x.K'x
constexpr int kNoAllocDoubles = kNoAllocMaxBlocks + 32;  // 32.9 KB in total

static __device__ __align__(256) double g_noalloc_scratch[kNoAllocDoubles];

// The PLAIN matvec reading x and accumulating y directly in the caller's node
// order (no staging copies), with x.K'x reduced through the scratch array.
template <int DIM>
__global__ void __launch_bounds__(kThreads) k_matvec_noalloc(MvParams<double> P, const double *xc, double *yc,
                                                             const int32_t *new2old, double *scratch) {
  constexpr int VW = DIM == 3 ? 4 : 2;
  constexpr int NC = DIM * DIM;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  double *sp = reinterpret_cast<double *>(smem_raw);
  double energy = 0;
  for (int patch = blockIdx.x; patch < P.n_patches; patch += gridDim.x) {
    const int nb = P.node_off[patch], nn = P.node_off[patch + 1] - nb, own = P.own[patch];
    const int e0 = P.elem_off[patch], ne = P.elem_off[patch + 1] - e0;
    double *sy = sp + (size_t)nn * VW;
    for (int i = threadIdx.x; i < nn; i += blockDim.x) {
      const int g = P.nodes[nb + i];
      const int64_t o = new2old[g];
      const unsigned b = P.bits[g];
      for (int d = 0; d < VW; ++d) sp[(size_t)i * VW + d] = (d < DIM && !(b >> d & 1u)) ? xc[o * DIM + d] : 0.0;
      for (int d = 0; d < DIM; ++d) sy[(size_t)d * nn + i] = 0;
    }
    __syncthreads();
    for (int le = threadIdx.x; le < ne; le += blockDim.x) {
      const int e = e0 + le;
      const uint2 c = P.lconn[e];
      const int li[4] = {(int)(c.x & 0xffffu), (int)(c.x >> 16), (int)(c.y & 0xffffu), (int)(c.y >> 16)};
      double G[NC];
      for (int k = 0; k < NC; ++k) G[k] = P.G[(size_t)k * P.gstride + e];
      double u[DIM + 1][DIM], f[DIM + 1][DIM];
      for (int a = 0; a <= DIM; ++a)
        for (int d = 0; d < DIM; ++d) u[a][d] = sp[(size_t)li[a] * VW + d];
      element_force<double, DIM>(u, G, P.lam, P.mu, 1.0, 0.0, f);
      for (int a = 0; a <= DIM; ++a)
        for (int d = 0; d < DIM; ++d) {
          energy += u[a][d] * f[a][d];
          atomicAdd(sy + (size_t)d * nn + li[a], f[a][d]);
        }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < nn; i += blockDim.x) {
      const int g = P.nodes[nb + i];
      const int64_t o = new2old[g];
      const unsigned b = P.bits[g];
      for (int d = 0; d < DIM; ++d) {
        double val = (b >> d & 1u) ? 0.0 : sy[(size_t)d * nn + i];
        if ((b >> d & 1u) && i >= own) {  // (I - P) diag(K) x on constrained DOFs
          const double xv = xc[o * DIM + d];
          val = P.diagA[(int64_t)g * VW + d] * xv;
          energy += val * xv;
        }
        if (val != 0.0) atomicAdd(yc + o * DIM + d, val);
      }
    }
    __syncthreads();
  }
  double v[1] = {energy};
  if (grid_sum_last<1>(v, scratch, reinterpret_cast<unsigned int *>(scratch + kNoAllocCounter)))
    scratch[kNoAllocResult] = v[0];
}

// Device address of the scratch array, resolved once per device.
double *noalloc_scratch(int device) {
  static std::mutex mu;
  static std::vector<double *> addr;
  std::lock_guard<std::mutex> lock(mu);
  if ((int)addr.size() <= device) addr.resize(device + 1, nullptr);
  if (!addr[device]) {
    void *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return nullptr;
    int optin = 0;
    if (cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, device) != cudaSuccess) return nullptr;
    if (cudaFuncSetAttribute((const void *)k_matvec_noalloc<3>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             optin - 8192) != cudaSuccess ||
        cudaFuncSetAttribute((const void *)k_matvec_noalloc<2>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             optin - 8192) != cudaSuccess)
      return nullptr;
    addr[device] = static_cast<double *>(p);
  }
  return addr[device];
}

}  // namespace detail
}  // namespace cfem

extern "C" cfem_status cfem_matvec_energy_noalloc(cfem_ctx *ctx, const double *x, double *y, double *energy) {
  using namespace cfem::detail;
  if (!ctx || !x || !y) {
    g_last_error = "cfem_matvec_energy_noalloc: null argument";
    return CFEM_ERR_INVALID_ARGUMENT;
  }
  (void)cudaGetLastError();
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev != ctx->device) {
    g_last_error = "cfem_matvec_energy_noalloc: the context's device must be current";
    return CFEM_ERR_INVALID_ARGUMENT;
  }
  if (ctx->n_inst) {
    g_last_error = "cfem_matvec_energy_noalloc: not available for a context of batched meshes";
    return CFEM_ERR_UNSUPPORTED;
  }
  if (ctx->grid_mv > kNoAllocMaxBlocks) {
    g_last_error = "cfem_matvec_energy_noalloc: the context needs " + std::to_string(ctx->grid_mv) +
                   " blocks, more than the " + std::to_string(kNoAllocMaxBlocks) + " the fixed scratch holds";
    return CFEM_ERR_INVALID_ARGUMENT;
  }
  double *scratch = noalloc_scratch(dev);
  if (!scratch) {
    g_last_error = "cfem_matvec_energy_noalloc: cudaGetSymbolAddress of the scratch array failed";
    return CFEM_ERR_CUDA;
  }
  cudaStream_t s = ctx->stream;
  if (ctx->own_stream) {
    if (cudaEventRecord(ctx->ev_in, ctx->user_stream) != cudaSuccess || cudaStreamWaitEvent(s, ctx->ev_in, 0) != cudaSuccess) {
      g_last_error = "cfem_matvec_energy_noalloc: cannot order after the caller's stream";
      return CFEM_ERR_CUDA;
    }
  }
  // y accumulates and the ticket counter must start at zero
  if (cudaMemsetAsync(y, 0, sizeof(double) * ctx->nd, s) != cudaSuccess ||
      cudaMemsetAsync(scratch + kNoAllocCounter, 0, sizeof(double), s) != cudaSuccess) {
    g_last_error = "cfem_matvec_energy_noalloc: cudaMemsetAsync failed";
    return CFEM_ERR_CUDA;
  }
  MvParams<double> P = base_mv_d(ctx);
  P.diagA = ctx->diagK.p;
  if (ctx->dim == 3)
    k_matvec_noalloc<3><<<ctx->grid_mv, kThreads, ctx->smem64, s>>>(P, x, y, ctx->node_new2old.p, scratch);
  else
    k_matvec_noalloc<2><<<ctx->grid_mv, kThreads, ctx->smem64, s>>>(P, x, y, ctx->node_new2old.p, scratch);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess && energy)
    e = cudaMemcpyAsync(energy, scratch + kNoAllocResult, sizeof(double), cudaMemcpyDefault, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) {
    g_last_error = std::string("cfem_matvec_energy_noalloc: ") + cudaGetErrorString(e);
    return CFEM_ERR_CUDA;
  }
  return CFEM_OK;
}
