// C-ABI implementation, part 2: GN22 dynamics (gpuCalculateFEM_DYN,
// femfunc.cpp:130-381), multi-RHS PCG, adjoint sensitivities, material update.
#include "context_internal.cuh"
#include "kernels_aux.cuh"

namespace cfem {
namespace detail {

// Element-local source of the implicit preconditioner in the reference's slot
// order: cK * diag(K_e) + diag(M_e) (femfunc.cpp:203-213).
template <int DIM>
__global__ void k_slot_diag(int64_t ne, const double *G64, int64_t gstride, double lam, double mu, const double *vol,
                            double rho, double cK, double mdiag_c, const int32_t *elem_new2old, double *out) {
  constexpr int NV = DIM + 1, W = 6 * (DIM - 1);
  int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (e >= ne) return;
  double g[NV][DIM];
  for (int d = 0; d < DIM; ++d) {
    double s0 = 0;
    for (int a = 1; a < NV; ++a) {
      g[a][d] = G64[(size_t)((a - 1) * DIM + d) * gstride + e];
      s0 += g[a][d];
    }
    g[0][d] = -s0;
  }
  const int64_t eo = elem_new2old[e];
  const double md = mdiag_c * rho * vol[e];
  for (int a = 0; a < NV; ++a) {
    double sq[DIM], tot = 0;
    for (int d = 0; d < DIM; ++d) { sq[d] = g[a][d] * g[a][d]; tot += sq[d]; }
    for (int d = 0; d < DIM; ++d) {
      double kd = (lam + 2 * mu) * sq[d] + mu * (tot - sq[d]);
      out[eo * W + DIM * a + d] = cK * kd + md;
    }
  }
}

__global__ void k_slot_mass(int64_t ne, int w, const double *vol, double c, const int32_t *elem_new2old, double *out) {
  int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (e >= ne) return;
  const int64_t eo = elem_new2old[e];
  const double m = c * vol[e];
  for (int j = 0; j < w; ++j) out[eo * w + j] = m;
}

// Stable sort of the DOF keys of all element slots (counting sort == the
// multimap order of cpu_matrix.cpp:189-223), in the caller's numbering.
void build_slot_perm(cfem_ctx *c, const int32_t *elems_caller) {
  if (c->perm.p) return;
  const int64_t nloc = c->ne * c->w, nd = c->nd;
  std::vector<int64_t> cnt(nd + 1, 0);
  std::vector<int32_t> mask(nloc);
  for (int64_t e = 0; e < c->ne; ++e)
    for (int a = 0; a < c->nv; ++a)
      for (int d = 0; d < c->dim; ++d) mask[e * c->w + c->dim * a + d] = elems_caller[e * c->nv + a] * c->dim + d;
  for (int64_t i = 0; i < nloc; ++i) cnt[mask[i] + 1]++;
  for (int64_t k = 0; k < nd; ++k) cnt[k + 1] += cnt[k];
  std::vector<int64_t> pos(cnt.begin(), cnt.end());
  std::vector<int32_t> perm(nloc);
  for (int64_t i = 0; i < nloc; ++i) perm[pos[mask[i]]++] = (int32_t)i;
  c->perm.upload(perm.data(), perm.size(), c->stream);
  c->seg.upload(cnt.data(), cnt.size(), c->stream);
  c->slot_src.alloc(nloc);
  c->slot_tmp.alloc(nloc);
}

// assembled node vector (FP64) of the slot source, then the in-place re-sort
void slot_assemble_and_resort(cfem_ctx *c, double *out64) {
  k_assemble_slots<<<nblk(c->nd), kThreads, 0, c->stream>>>(c->nd, c->dim, c->vw, c->seg.p, c->perm.p, c->slot_src.p,
                                                            c->node_old2new.p, out64, 0, nullptr);
  k_permute<<<nblk(c->ne * c->w), kThreads, 0, c->stream>>>(c->ne * c->w, c->perm.p, c->slot_src.p, c->slot_tmp.p);
  CKL();
  std::swap(c->slot_src.p, c->slot_tmp.p);
}

void set_pcg_vectors(cfem_ctx *c, const double *diag_op, const double *diag_pre) {
  k_invert<double><<<nblk(c->nvec), kThreads, 0, c->stream>>>(c->nvec, diag_pre, c->v64.dinv.p);
  k_invert<float><<<nblk(c->nvec), kThreads, 0, c->stream>>>(c->nvec, diag_pre, c->v32.dinv.p);
  CK(cudaMemcpyAsync(c->v64.diagA.p, diag_op, sizeof(double) * c->nvec, cudaMemcpyDeviceToDevice, c->stream));
  k_convert<double, float><<<nblk(c->nvec), kThreads, 0, c->stream>>>(c->nvec, diag_op, c->v32.diagA.p);
  CKL();
}

// The explicit update with the end of the step fused in (receivers, step
// counter through DynState::pstep, P.parity and P.dto set by the caller).
template <typename T>
void launch_dyn_explicit_step(cfem_ctx *c, const DynParams<T> &P) {
  if (c->dim == 3) launch_pdl(k_dyn_explicit<T, 3, true>, dim3(c->grid_vec), dim3(kThreads), 0, c->stream, P);
  else k_dyn_explicit<T, 2, true><<<c->grid_vec, kThreads, 0, c->stream>>>(P);
  CKL();
}
template <typename T>
void launch_dyn_rhs(cfem_ctx *c, const DynParams<T> &P) {
  if (c->dim == 3) k_dyn_rhs<T, 3><<<c->grid_vec, kThreads, 0, c->stream>>>(P);
  else k_dyn_rhs<T, 2><<<c->grid_vec, kThreads, 0, c->stream>>>(P);
  CKL();
}
template <typename T>
void launch_dyn_correct(cfem_ctx *c, const DynParams<T> &P) {
  if (c->dim == 3) k_dyn_correct<T, 3><<<c->grid_vec, kThreads, 0, c->stream>>>(P);
  else k_dyn_correct<T, 2><<<c->grid_vec, kThreads, 0, c->stream>>>(P);
  CKL();
}

template <typename T>
cfem_status run_dyn(cfem_ctx *c, const cfem_dyn_params *prm, const cfem_wavelet *w, double *u_out, cfem_dyn_info *info,
                    const int32_t *elems_caller) {
  const double beta1 = prm->beta1, beta2 = prm->beta2, dt = prm->dt;
  const bool expl = beta2 == 0.0;
  const float dtf = (float)prm->dt, endf = (float)prm->endtime;
  if (!(dtf > 0)) throw Fail{CFEM_ERR_INVALID_ARGUMENT, "dt must be positive"};
  int nsteps = endf < 0 ? 1 : (int)(endf / dtf);  // femfunc.cpp:218-225
  if (nsteps < 1) nsteps = 1;                     // the do-while runs at least one step
  const bool compat = c->semantics == CFEM_COMPAT;
  // time factors of the load parts for t = 0 (initFlocals) and every step
  RhsSchedule sch;
  sch.semantics = c->semantics;
  sch.has_loads = c->rhs.has_loads;
  sch.w = w;
  std::vector<double> coef(2 * (size_t)(nsteps + 1));
  sch.eval(0.f, coef[0], coef[1]);
  for (int s = 1; s <= nsteps; ++s) sch.eval((float)s * dtf, coef[2 * s], coef[2 * s + 1]);
  DBuf<double> dcoef;
  dcoef.upload(coef.data(), coef.size(), c->stream);
  Vecs<T> &V = [&]() -> Vecs<T> & {
    if constexpr (sizeof(T) == 8) return c->v64; else return c->v32;
  }();
  DBuf<T> d0, d1, vel, acc, y, minv;
  for (auto *b : {&d0, &d1, &vel, &acc, &y}) { b->alloc(c->nvec); b->zero(c->stream); }
  DBuf<DynState> st;
  st.alloc(1);
  DynState hs{};
  hs.step = 1;
  hs.pstep[0] = 1;  // explicit: the first step has parity 0
  CK(cudaMemcpyAsync(st.p, &hs, sizeof(hs), cudaMemcpyHostToDevice, c->stream));
  const int nrec = prm->n_receivers > 0 && prm->receiver_nodes && prm->receiver_trace ? prm->n_receivers : 0;
  DBuf<int32_t> recv;
  DBuf<double> trace;
  if (nrec) {
    std::vector<int32_t> rn(nrec);
    for (int i = 0; i < nrec; ++i) {
      int32_t o = prm->receiver_nodes[i];
      if (o < 0 || o >= c->nn) throw Fail{CFEM_ERR_INVALID_ARGUMENT, "receiver node out of range"};
      rn[i] = c->prep.node_old2new[o];
    }
    recv.upload(rn.data(), rn.size(), c->stream);
    trace.alloc((size_t)nsteps * nrec * c->dim);
  }
  const T *FA, *FB;
  if constexpr (sizeof(T) == 8) { FA = c->FA.p; FB = c->FB.p; } else { FA = c->FA32.p; FB = c->FB32.p; }
  DynParams<T> dp{};
  dp.n_nodes = c->nn;
  dp.v = vel.p;
  dp.a = acc.p;
  dp.y = y.p;
  dp.FA = FA;
  dp.FB = FB;
  dp.coef = dcoef.p;
  dp.st = st.p;
  dp.recv = recv.p;
  dp.n_recv = nrec;
  dp.trace = trace.p;
  dp.dim = c->dim;
  dp.c_old = (T)((1 - beta1) * dt);
  dp.c_new = (T)(beta1 * dt);
  dp.c_d = (T)(0.5 * beta2 * dt * dt);
  MvParams<T> mv = base_mv<T>(c);
  if constexpr (sizeof(T) == 8) mv.diagA = c->diagK.p; else mv.diagA = c->diagK32.p;  // r = F - K' d
  mv.c1 = (T)dt;
  mv.c2 = (T)(0.5 * (1 - beta2) * dt * dt);
  mv.x2 = vel.p;
  mv.x3 = acc.p;
  mv.y = y.p;
  DBuf<double> diag_pre, diag_op;
  diag_pre.alloc(c->nvec);
  diag_op.alloc(c->nvec);
  bool resort = false;
  const double cK = 0.5 * beta2 * dt * dt;
  // operator / mass factors per semantics (cpu_fem_utils.cpp:598-734)
  const double lump_c = c->dim == 2 ? 1.0 / 3 : (compat ? 1.0 / 12 : 1.0 / 4);
  const double mdiag_c = c->dim == 2 ? 1.0 / 6 : (compat ? 1.0 / 24 : 1.0 / 10);
  if (compat) {
    build_slot_perm(c, elems_caller);
    if (expl) {
      k_slot_mass<<<nblk(c->ne), kThreads, 0, c->stream>>>(c->ne, c->w, c->vol.p, lump_c * c->rho, c->elem_new2old.p,
                                                           c->slot_src.p);
    } else {
      if (c->dim == 3)
        k_slot_diag<3><<<nblk(c->ne), kThreads, 0, c->stream>>>(c->ne, c->G64.p, c->gstride, c->lam, c->mu, c->vol.p,
                                                                 c->rho, cK, mdiag_c, c->elem_new2old.p, c->slot_src.p);
      else
        k_slot_diag<2><<<nblk(c->ne), kThreads, 0, c->stream>>>(c->ne, c->G64.p, c->gstride, c->lam, c->mu, c->vol.p,
                                                                 c->rho, cK, mdiag_c, c->elem_new2old.p, c->slot_src.p);
    }
    CKL();
    resort = true;
  }
  if (expl) {
    minv.alloc(c->nvec);
    if (!compat) {
      k_invert<T><<<nblk(c->nvec), kThreads, 0, c->stream>>>(c->nvec, c->mlump.p, minv.p);
      CKL();
    }
    set_pcg_vectors(c, c->diagK.p, c->diagK.p);  // diagA: constrained term of K'
  } else {
    if (compat) {
      CK(cudaMemcpyAsync(diag_op.p, c->diagK.p, sizeof(double) * c->nvec, cudaMemcpyDeviceToDevice, c->stream));
    } else {
      // A = M + cK K': diagonal cK diag(K) + diag(M)
      CK(cudaMemcpyAsync(diag_op.p, c->mcdiag.p, sizeof(double) * c->nvec, cudaMemcpyDeviceToDevice, c->stream));
      k_axpby64<<<nblk(c->nvec), kThreads, 0, c->stream>>>(c->nvec, cK, c->diagK.p, 1.0, diag_op.p);
      CKL();
      set_pcg_vectors(c, diag_op.p, diag_op.p);
    }
  }
  dp.minv = minv.p;
  const T *mc = nullptr;
  if constexpr (sizeof(T) == 8) mc = c->mc64.p; else mc = c->mc32.p;
  const T opK = compat ? T(1) : (T)cK, opM = compat ? T(0) : T(1);
  const T *opmc = compat ? nullptr : mc;
  if (!expl) {
    mv.cK = 1;  // r = F - K' d uses the plain stiffness
    mv.cM = 0;
  }
  CK(cudaEventRecord(c->ev0, c->stream));
  int64_t pcg_total = 0;
  int status = CFEM_OK;
  T *dcur = d0.p, *dnext = d1.p;
  V.x.zero(c->stream);  // acceleration warm start / PCG solution
  auto one_step = [&](T *from, T *to, int parity) {
    mv.x = from;
    mv.xout = to;
    launch_mv<T>(c, MV_DYN, mv);
    if (expl) {
      if (resort) {
        slot_assemble_and_resort(c, diag_pre.p);
        k_invert<T><<<nblk(c->nvec), kThreads, 0, c->stream>>>(c->nvec, diag_pre.p, minv.p);
        CKL();
      }
      DynParams<T> de = dp;
      de.dto = to;
      de.parity = parity;
      launch_dyn_explicit_step<T>(c, de);
    }
  };
  if (expl) {
    // two steps per captured graph (the displacement buffers alternate)
    cudaGraphExec_t exec = nullptr;
    int pairs = nsteps / 2;
    if (pairs > 0) {
      cudaGraph_t g;
      CK(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
      try {
        one_step(d0.p, d1.p, 0);
        one_step(d1.p, d0.p, 1);
      } catch (...) {
        cudaGraph_t broken = nullptr;
        cudaStreamEndCapture(c->stream, &broken);
        if (broken) cudaGraphDestroy(broken);
        (void)cudaGetLastError();
        throw;
      }
      CK(cudaStreamEndCapture(c->stream, &g));
      CK(cudaGraphInstantiate(&exec, g, 0));
      cudaGraphDestroy(g);
      for (int i = 0; i < pairs; ++i) CK(cudaGraphLaunch(exec, c->stream));
      cudaGraphExecDestroy(exec);
      // the resort swaps are captured: after an even number of steps slot_src is back in place
    }
    dcur = d0.p;
    if (nsteps & 1) {  // (after the pairs the next step's counter is pstep[0])
      one_step(d0.p, d1.p, 0);
      dcur = d1.p;
    }
  } else {
    for (int s = 1; s <= nsteps; ++s) {
      mv.x = dcur;
      mv.xout = dnext;
      launch_mv<T>(c, MV_DYN, mv);
      dp.rhs = V.f.p;
      launch_dyn_rhs<T>(c, dp);
      if (compat) {
        slot_assemble_and_resort(c, diag_pre.p);
        set_pcg_vectors(c, diag_op.p, diag_pre.p);
      }
      const double tol = compat ? 1e-4 : (prm->pcg_tol > 0 ? prm->pcg_tol : 1e-10);
      const int rule = compat ? CFEM_STOP_REFERENCE : prm->stop_rule;
      const int warm = compat ? 0 : prm->warm_start;
      PcgResult r = run_pcg<T>(c, V, opK, opM, opmc, warm, tol, rule, prm->max_iter);
      pcg_total += r.iters;
      if (r.status != CFEM_OK) { status = r.status; break; }
      dp.anew = V.x.p;
      dp.d = dnext;
      launch_dyn_correct<T>(c, dp);
      k_dyn_end_step<T><<<1, kThreads, 0, c->stream>>>(dp, dnext, c->vw);
      CKL();
      std::swap(dcur, dnext);
    }
  }
  CK(cudaEventRecord(c->ev1, c->stream));
  CK(cudaEventSynchronize(c->ev1));
  float ms = 0;
  CK(cudaEventElapsedTime(&ms, c->ev0, c->ev1));
  to_caller<T>(c, dcur, u_out);
  if (nrec) CK(cudaMemcpyAsync(prm->receiver_trace, trace.p, sizeof(double) * trace.n, cudaMemcpyDefault, c->stream));
  check_copy_error(c);
  if (info) {
    info->status = status;
    info->steps = nsteps;
    info->pcg_iterations = pcg_total;
    info->solve_ms = ms;
  }
  return (cfem_status)status;
}

// Explicit GN22 receiver-misfit adjoint with sqrt(N) checkpointing (FP64).
cfem_status run_dyn_adjoint(cfem_ctx *c, const cfem_dyn_params *prm, const cfem_wavelet *w, int n_rec,
                            const int32_t *rec_nodes, const double *obs, double *loss, double *dLdE,
                            cfem_dyn_info *info) {
  if (prm->beta2 != 0.0) throw Fail{CFEM_ERR_UNSUPPORTED, "the dynamics adjoint covers the explicit scheme (beta2 = 0)"};
  if (c->semantics != CFEM_CONSISTENT)
    throw Fail{CFEM_ERR_UNSUPPORTED, "the dynamics adjoint needs consistent semantics (no per-step re-sorted masses)"};
  if (n_rec <= 0 || !rec_nodes || !obs) throw Fail{CFEM_ERR_INVALID_ARGUMENT, "receivers and observations required"};
  const double beta1 = prm->beta1, dt = prm->dt;
  const float dtf = (float)prm->dt, endf = (float)prm->endtime;
  if (!(dtf > 0)) throw Fail{CFEM_ERR_INVALID_ARGUMENT, "dt must be positive"};
  int N = endf < 0 ? 1 : (int)(endf / dtf);
  if (N < 1) N = 1;
  const int C = (int)std::ceil(std::sqrt((double)N));
  const int64_t nv = c->nvec;
  const double h_old = (1 - beta1) * dt, h_new = beta1 * dt, c2 = 0.5 * dt * dt;
  RhsSchedule sch;
  sch.semantics = c->semantics;
  sch.has_loads = c->rhs.has_loads;
  sch.w = w;
  std::vector<double> coef(2 * (size_t)(N + 1));
  sch.eval(0.f, coef[0], coef[1]);
  for (int s = 1; s <= N; ++s) sch.eval((float)s * dtf, coef[2 * s], coef[2 * s + 1]);
  DBuf<double> dcoef, minv, vel, acc, y, dA, dB, trace, obs_d, gE;
  DBuf<int32_t> recv;
  dcoef.upload(coef.data(), coef.size(), c->stream);
  for (auto *b : {&minv, &vel, &acc, &y, &dA, &dB}) { b->alloc(nv); b->zero(c->stream); }
  k_invert<double><<<nblk(nv), kThreads, 0, c->stream>>>(nv, c->mlump.p, minv.p);
  std::vector<int32_t> rn(n_rec);
  for (int i = 0; i < n_rec; ++i) {
    if (rec_nodes[i] < 0 || rec_nodes[i] >= c->nn) throw Fail{CFEM_ERR_INVALID_ARGUMENT, "receiver node out of range"};
    rn[i] = c->prep.node_old2new[rec_nodes[i]];
  }
  recv.upload(rn.data(), rn.size(), c->stream);
  trace.alloc((size_t)N * n_rec * c->dim);
  obs_d.alloc((size_t)N * n_rec * c->dim);
  CK(cudaMemcpyAsync(obs_d.p, obs, sizeof(double) * obs_d.n, cudaMemcpyDefault, c->stream));
  gE.alloc(c->ne);
  gE.zero(c->stream);
  DBuf<DynState> st;
  st.alloc(1);
  // checkpoints of (d, v, a) after steps 0, C, 2C, ... and one segment of displacements
  const int ncp = N / C + 1;
  DBuf<double> cps, seg;
  cps.alloc((size_t)ncp * 3 * nv);
  seg.alloc((size_t)(C + 1) * nv);
  const double *young = c->young_d.p;
  DBuf<double> yd;
  if (!young) {
    std::vector<double> yv(c->ne, c->E);
    yd.upload(yv.data(), yv.size(), c->stream);
    young = yd.p;
  }
  DynParams<double> dp{};
  dp.n_nodes = c->nn;
  dp.v = vel.p;
  dp.a = acc.p;
  dp.y = y.p;
  dp.FA = c->FA.p;
  dp.FB = c->FB.p;
  dp.coef = dcoef.p;
  dp.st = st.p;
  dp.dim = c->dim;
  dp.minv = minv.p;
  dp.c_old = h_old;
  dp.c_new = h_new;
  MvParams<double> mv = base_mv<double>(c);
  mv.diagA = c->diagK.p;
  mv.c1 = dt;
  mv.c2 = c2;
  mv.x2 = vel.p;
  mv.x3 = acc.p;
  mv.y = y.p;
  auto set_step = [&](int step) {
    DynState hs{};
    hs.step = step;
    CK(cudaMemcpyAsync(st.p, &hs, sizeof(hs), cudaMemcpyHostToDevice, c->stream));
  };
  auto step = [&](const double *from, double *to, bool record) {
    mv.x = from;
    mv.xout = to;
    launch_mv<double>(c, MV_DYN, mv);
    if (c->dim == 3) k_dyn_explicit<double, 3><<<c->grid_vec, kThreads, 0, c->stream>>>(dp);
    else k_dyn_explicit<double, 2><<<c->grid_vec, kThreads, 0, c->stream>>>(dp);
    DynParams<double> de = dp;
    if (record) { de.recv = recv.p; de.n_recv = n_rec; de.trace = trace.p; } else { de.n_recv = 0; }
    k_dyn_end_step<double><<<1, kThreads, 0, c->stream>>>(de, to, c->vw);
    CKL();
  };
  auto save_cp = [&](int k, const double *d) {
    double *base = cps.p + (size_t)k * 3 * nv;
    CK(cudaMemcpyAsync(base, d, sizeof(double) * nv, cudaMemcpyDeviceToDevice, c->stream));
    CK(cudaMemcpyAsync(base + nv, vel.p, sizeof(double) * nv, cudaMemcpyDeviceToDevice, c->stream));
    CK(cudaMemcpyAsync(base + 2 * nv, acc.p, sizeof(double) * nv, cudaMemcpyDeviceToDevice, c->stream));
  };
  CK(cudaEventRecord(c->ev0, c->stream));
  // forward with checkpoints
  set_step(1);
  double *cur = dA.p, *nxt = dB.p;
  save_cp(0, cur);
  for (int n = 1; n <= N; ++n) {
    step(cur, nxt, true);
    std::swap(cur, nxt);
    if (n % C == 0 && n / C < ncp) save_cp(n / C, cur);
  }
  std::vector<double> htrace(trace.n);
  CK(cudaMemcpyAsync(htrace.data(), trace.p, sizeof(double) * trace.n, cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  std::vector<double> hobs(obs_d.n);
  CK(cudaMemcpy(hobs.data(), obs_d.p, sizeof(double) * obs_d.n, cudaMemcpyDeviceToHost));
  double L = 0;
  for (size_t i = 0; i < htrace.size(); ++i) L += 0.5 * (htrace[i] - hobs[i]) * (htrace[i] - hobs[i]);
  // reverse sweep
  DBuf<double> db, vb, ab, wb;
  for (auto *b : {&db, &vb, &ab, &wb}) { b->alloc(nv); b->zero(c->stream); }
  for (int s = (N - 1) / C; s >= 0; --s) {
    const int k0 = s * C, k1 = std::min(N, k0 + C);
    // restore the checkpoint after step k0 and recompute steps k0+1..k1
    const double *base = cps.p + (size_t)s * 3 * nv;
    CK(cudaMemcpyAsync(seg.p, base, sizeof(double) * nv, cudaMemcpyDeviceToDevice, c->stream));
    CK(cudaMemcpyAsync(vel.p, base + nv, sizeof(double) * nv, cudaMemcpyDeviceToDevice, c->stream));
    CK(cudaMemcpyAsync(acc.p, base + 2 * nv, sizeof(double) * nv, cudaMemcpyDeviceToDevice, c->stream));
    set_step(k0 + 1);
    for (int n = k0 + 1; n <= k1; ++n) step(seg.p + (size_t)(n - 1 - k0) * nv, seg.p + (size_t)(n - k0) * nv, false);
    for (int n = k1; n > k0; --n) {
      const double *dn = seg.p + (size_t)(n - k0) * nv;
      k_adj_receivers<<<nblk(n_rec * c->dim), kThreads, 0, c->stream>>>(n_rec, c->dim, c->vw, recv.p, dn,
                                                                       obs_d.p + (size_t)(n - 1) * n_rec * c->dim, db.p);
      k_adj_pre<<<nblk(nv), kThreads, 0, c->stream>>>(nv, h_old, h_new, minv.p, vb.p, ab.p, wb.p);
      if (c->dim == 3)
        k_grad_young<3><<<nblk(c->ne), kThreads, 0, c->stream>>>(c->ne, c->G64.p, c->gstride, c->conn.p, c->bits.p,
                                                                 c->lam, c->mu, wb.p, dn, young, c->elem_new2old.p,
                                                                 gE.p, 1);
      else
        k_grad_young<2><<<nblk(c->ne), kThreads, 0, c->stream>>>(c->ne, c->G64.p, c->gstride, c->conn.p, c->bits.p,
                                                                 c->lam, c->mu, wb.p, dn, young, c->elem_new2old.p,
                                                                 gE.p, 1);
      MvParams<double> m2 = base_mv<double>(c);
      m2.diagA = c->diagK.p;
      m2.x = wb.p;
      m2.y = y.p;
      launch_mv<double>(c, MV_PLAIN, m2);
      k_adj_post<<<nblk(nv), kThreads, 0, c->stream>>>(nv, dt, c2, y.p, db.p, vb.p, ab.p);
      CKL();
    }
  }
  CK(cudaEventRecord(c->ev1, c->stream));
  CK(cudaEventSynchronize(c->ev1));
  float ms = 0;
  CK(cudaEventElapsedTime(&ms, c->ev0, c->ev1));
  if (dLdE) CK(cudaMemcpyAsync(dLdE, gE.p, sizeof(double) * c->ne, cudaMemcpyDefault, c->stream));
  check_copy_error(c);
  if (loss) *loss = L;
  if (info) {
    info->status = CFEM_OK;
    info->steps = N;
    info->pcg_iterations = 0;
    info->solve_ms = ms;
  }
  return CFEM_OK;
}

}  // namespace detail
}  // namespace cfem

extern "C" {

cfem_status cfem_dyn_adjoint(cfem_ctx *ctx, const cfem_dyn_params *prm, const cfem_wavelet *w, int32_t n_rec,
                             const int32_t *rec_nodes, const double *obs, double *loss, double *dLdE,
                             cfem_dyn_info *info) {
  return run_guarded([&]() -> cfem_status {
    check_ctx(ctx);
    if (!prm) throw Fail{CFEM_ERR_INVALID_ARGUMENT, "null parameters"};
    enter(ctx);
    return run_dyn_adjoint(ctx, prm, w, n_rec, rec_nodes, obs, loss, dLdE, info);
  });
}


cfem_status cfem_dyn(cfem_ctx *ctx, const cfem_dyn_params *prm, const cfem_wavelet *w, double *u, cfem_dyn_info *info) {
  return run_guarded([&]() -> cfem_status {
    check_ctx(ctx);
    enter(ctx);
    if (!prm || !u) throw Fail{CFEM_ERR_INVALID_ARGUMENT, "null argument"};
    if (prm->precision == CFEM_FP64) return run_dyn<double>(ctx, prm, w, u, info, ctx->elems_caller.data());
    if (prm->precision == CFEM_FP32) return run_dyn<float>(ctx, prm, w, u, info, ctx->elems_caller.data());
    throw Fail{CFEM_ERR_INVALID_ARGUMENT, "dynamics precision must be CFEM_FP64 or CFEM_FP32"};
  });
}

cfem_status cfem_adjoint(cfem_ctx *ctx, const cfem_solve_params *prm, const double *u, const double *dLdu, double *dLdE,
                         double *dLdf, cfem_solve_info *info) {
  return run_guarded([&]() -> cfem_status {
    check_ctx(ctx);
    enter(ctx);
    if (!u || !dLdu) throw Fail{CFEM_ERR_INVALID_ARGUMENT, "null input"};
    cfem_solve_params p = prm ? *prm : default_params();
    // lambda = K'^-1 dL/du (K' symmetric)
    to_internal<double>(ctx, dLdu, ctx->v64.f.p);
    cfem_status st = solve_internal(ctx, &p, info);
    if (dLdf) to_caller<double>(ctx, ctx->v64.x.p, dLdf);
    if (dLdE) {
      DBuf<double> uin, g, yd;
      uin.alloc(ctx->nvec);
      g.alloc(ctx->ne);
      to_internal<double>(ctx, u, uin.p);
      const double *young = ctx->young_d.p;
      if (!young) {
        std::vector<double> yv(ctx->ne, ctx->E);
        yd.upload(yv.data(), yv.size(), ctx->stream);
        young = yd.p;
      }
      if (ctx->dim == 3)
        k_grad_young<3><<<nblk(ctx->ne), kThreads, 0, ctx->stream>>>(ctx->ne, ctx->G64.p, ctx->gstride, ctx->conn.p, ctx->bits.p,
                                                                    ctx->lam, ctx->mu, ctx->v64.x.p, uin.p, young,
                                                                    ctx->elem_new2old.p, g.p);
      else
        k_grad_young<2><<<nblk(ctx->ne), kThreads, 0, ctx->stream>>>(ctx->ne, ctx->G64.p, ctx->gstride, ctx->conn.p, ctx->bits.p,
                                                                    ctx->lam, ctx->mu, ctx->v64.x.p, uin.p, young,
                                                                    ctx->elem_new2old.p, g.p);
      CKL();
      CK(cudaMemcpyAsync(dLdE, g.p, sizeof(double) * ctx->ne, cudaMemcpyDefault, ctx->stream));
    }
    CK(cudaStreamSynchronize(ctx->stream));
    return st;
  });
}

cfem_status cfem_element_stress(cfem_ctx *ctx, const double *u, double *strain, double *stress, double *mises) {
  return run_guarded([&]() -> cfem_status {
    check_ctx(ctx);
    if (ctx->n_inst) throw Fail{CFEM_ERR_UNSUPPORTED, "not available for a context of batched meshes"};
    if (!u) throw Fail{CFEM_ERR_INVALID_ARGUMENT, "null displacement"};
    enter(ctx);
    const int S = 3 * (ctx->dim - 1);
    DBuf<double> uin, de, ds, dm;
    uin.alloc(ctx->nvec);
    uin.zero(ctx->stream);
    to_internal<double>(ctx, u, uin.p);
    if (strain) de.alloc((size_t)ctx->ne * S);
    if (stress) ds.alloc((size_t)ctx->ne * S);
    if (mises) dm.alloc(ctx->ne);
    if (ctx->dim == 3)
      k_element_stress<3><<<nblk(ctx->ne), kThreads, 0, ctx->stream>>>(ctx->ne, ctx->G64.p, ctx->gstride, ctx->vol.p, ctx->escale.p,
                                                                        ctx->conn.p, uin.p, ctx->lam, ctx->mu, ctx->elem_new2old.p,
                                                                        de.p, ds.p, dm.p);
    else
      k_element_stress<2><<<nblk(ctx->ne), kThreads, 0, ctx->stream>>>(ctx->ne, ctx->G64.p, ctx->gstride, ctx->vol.p, ctx->escale.p,
                                                                        ctx->conn.p, uin.p, ctx->lam, ctx->mu, ctx->elem_new2old.p,
                                                                        de.p, ds.p, dm.p);
    CKL();
    if (strain) CK(cudaMemcpyAsync(strain, de.p, sizeof(double) * de.n, cudaMemcpyDefault, ctx->stream));
    if (stress) CK(cudaMemcpyAsync(stress, ds.p, sizeof(double) * ds.n, cudaMemcpyDefault, ctx->stream));
    if (mises) CK(cudaMemcpyAsync(mises, dm.p, sizeof(double) * dm.n, cudaMemcpyDefault, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    return CFEM_OK;
  });
}

cfem_status cfem_set_young(cfem_ctx *ctx, const double *elem_young) {
  return run_guarded([&]() -> cfem_status {
    check_ctx(ctx);
    if (ctx->n_inst) throw Fail{CFEM_ERR_UNSUPPORTED, "not available for a context of batched meshes"};
    enter(ctx);
    if (!elem_young) throw Fail{CFEM_ERR_INVALID_ARGUMENT, "null array"};
    std::vector<double> yv(ctx->ne);
    // on the context's stream, which enter() ordered after the caller's
    CK(cudaMemcpyAsync(yv.data(), elem_young, sizeof(double) * ctx->ne, cudaMemcpyDefault, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    for (double y : yv)
      if (!(y > 0)) throw Fail{CFEM_ERR_INVALID_ARGUMENT, "per-element Young's modulus must be positive"};
    ctx->young = yv;
    rebuild_operator(ctx);
    // captured PCG iterations hold operator buffers that the rebuild may have replaced
    ctx->graph64.reset();
    ctx->graph32.reset();
    return CFEM_OK;
  });
}

}  // extern "C"
