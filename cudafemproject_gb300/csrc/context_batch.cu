// Batched independent meshes (cfem_create_batch / cfem_batch_static_solve).
//
// n tet meshes, each with its own material, live in one context: their node
// and element arrays are concatenated (instance-major, caller order), the
// locality renumbering keeps every instance's elements, fans, patches and
// owned nodes contiguous, and each patch carries its instance's lambda and mu.
// One solve runs all instances together: every matvec launch covers the
// patches of all instances (persistent CTAs), every instance has its own PCG
// scalars and stopping test, and a converged instance is masked out (its
// patches and nodes are skipped). The iterations replay from a captured CUDA
// graph; FP32_REFINE adds a per-instance FP64 iterative refinement.
#include "context_internal.cuh"
#include "kernels_aux.cuh"

namespace cfem {
namespace detail {
namespace {

struct BatchBufs {
  DBuf<Scalars> isc;
  DBuf<BatchCtl> ctl;
  DBuf<double> pe, pp, scratch, rrff, seg;
  DBuf<int> active;
};

template <typename T>
BatchVecParams<T> vec_params_batch(cfem_ctx *c, BatchBufs &B, int k_active) {
  BatchVecParams<T> P{};
  P.n_patches = c->prep.n_patches;
  P.n_inst = c->n_inst;
  P.patch_inst = c->patch_inst.p;
  P.own_first = c->own_first.p;
  P.inst_patch_off = c->inst_patch_off.p;
  P.isc = B.isc.p;
  P.ctl = B.ctl.p;
  P.pp = B.pp.p;
  P.scratch = B.scratch.p;
  P.k_active = k_active;
  return P;
}

template <typename T>
void batch_mv(cfem_ctx *c, BatchBufs &B, MvParams<T> &mv) {
  mv.patch_inst = c->patch_inst.p;
  if constexpr (sizeof(T) == 8) mv.pmat = c->pmat64.p; else mv.pmat = c->pmat32.p;
  mv.isc = B.isc.p;
  mv.bctl = B.ctl.p;
  mv.patch_energy = B.pe.p;
  mv.inst_patch_off = c->inst_patch_off.p;
  mv.n_inst = c->n_inst;
}

int vec_grid(cfem_ctx *c) { return (int)std::min<int64_t>(c->prep.n_patches, (int64_t)c->n_sm * 8); }
// flat vector step (k_batch_vec_flat): two CTAs per SM, four nodes in flight per thread
int flat_grid(cfem_ctx *c) { return c->n_sm * 2; }
size_t flat_smem(cfem_ctx *c) { return (size_t)(4 * c->n_inst + 2) * sizeof(int); }

// FP32 PCG of every instance on c->v32.f; instances with a zero right-hand
// side are done at once. Per-instance results are returned in out.
void run_batch_pcg(cfem_ctx *c, BatchBufs &B, double tol, int rule, int maxit, std::vector<Scalars> &out) {
  std::vector<Scalars> h(c->n_inst);
  for (auto &s : h) {
    s = Scalars{};
    s.tol = tol;
    s.rule = rule;
    s.maxit = maxit > 0 ? maxit : 1000000;
  }
  CK(cudaMemcpyAsync(B.isc.p, h.data(), sizeof(Scalars) * h.size(), cudaMemcpyHostToDevice, c->stream));
  B.ctl.zero(c->stream);
  Vecs<float> &V = c->v32;
  BatchVecParams<float> vp = vec_params_batch<float>(c, B, c->n_inst);
  const int gv = flat_grid(c);
  const size_t sv = flat_smem(c);
  vp.seg = B.seg.p;
  k_batch_vec_flat<float><<<gv, kThreads, sv, c->stream>>>(vp, V.x.p, V.r.p, V.z.p, nullptr, V.u.p, V.f.p, V.dinv.p, 1);
  CKL();
  c->launches += 1;
  MvParams<float> mv = base_mv<float>(c);
  mv.diagA = V.diagA.p;
  batch_mv<float>(c, B, mv);
  cudaGraph_t graph;
  cudaGraphExec_t exec = nullptr;
  const int64_t before = c->launches;
  CK(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
  try {
    for (int it = 0; it < c->chunk; ++it) {
      float *pold = (it & 1) ? V.pB.p : V.pA.p;
      float *pnew = (it & 1) ? V.pA.p : V.pB.p;
      MvParams<float> m = mv;
      m.x = V.z.p;
      m.x2 = pold;
      m.xout = pnew;
      m.y = V.u.p;
      launch_mv<float>(c, MV_PCG, m);
      k_batch_vec_flat<float><<<gv, kThreads, sv, c->stream>>>(vp, V.x.p, V.r.p, V.z.p, pnew, V.u.p, V.f.p, V.dinv.p, 0);
      CKL();
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
  cudaError_t ie = cudaGraphInstantiate(&exec, graph, 0);
  cudaGraphDestroy(graph);
  if (ie != cudaSuccess) throw Fail{CFEM_ERR_CUDA, std::string("graph instantiation: ") + cudaGetErrorString(ie)};
  struct ExecGuard {
    cudaGraphExec_t e;
    ~ExecGuard() { cudaGraphExecDestroy(e); }
  } guard{exec};
  BatchCtl *hctl = reinterpret_cast<BatchCtl *>(c->h_rr);  // 16 of the 32 pinned scratch bytes
  const int64_t max_launches = (int64_t)(maxit > 0 ? maxit : 1000000) / c->chunk + 16;
  int last_iter = -1, stalled = 0;
  for (int64_t launch = 0;; ++launch) {
    if (launch > max_launches || stalled > 4) {
      check_copy_error(c);
      throw Fail{CFEM_ERR_CUDA, "batched PCG recurrence stopped advancing on the device"};
    }
    CK(cudaGraphLaunch(exec, c->stream));
    c->launches += 2 * c->chunk;
    CK(cudaMemcpyAsync(hctl, B.ctl.p, sizeof(BatchCtl), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    if (hctl->all_done) break;
    stalled = hctl->iter == last_iter ? stalled + 1 : 0;
    last_iter = hctl->iter;
  }
  check_copy_error(c);
  out.resize(c->n_inst);
  CK(cudaMemcpy(out.data(), B.isc.p, sizeof(Scalars) * c->n_inst, cudaMemcpyDeviceToHost));
}

// tmp64 = K64 x64 (all instances, FP64 operator with per-patch materials)
void batch_kx(cfem_ctx *c, BatchBufs &B) {
  MvParams<double> mv = base_mv<double>(c);
  mv.diagA = c->diagK.p;
  batch_mv<double>(c, B, mv);
  mv.x = c->v64.x.p;
  mv.y = c->tmp64.p;
  c->tmp64.zero(c->stream);
  launch_mv<double>(c, MV_PLAIN, mv);
}

// r64 = f64 - tmp64 per instance; f32 = r64 on active instances, 0 elsewhere;
// rr/ff per instance.
void batch_residual(cfem_ctx *c, BatchBufs &B, const std::vector<int> &active, std::vector<double> &rr,
                    std::vector<double> &ff) {
  CK(cudaMemcpyAsync(B.active.p, active.data(), sizeof(int) * c->n_inst, cudaMemcpyHostToDevice, c->stream));
  BatchVecParams<double> vp = vec_params_batch<double>(c, B, c->n_inst);
  B.ctl.zero(c->stream);
  k_batch_residual<<<vec_grid(c), kThreads, 0, c->stream>>>(vp, c->v64.f.p, c->tmp64.p, c->v64.r.p, c->v32.f.p,
                                                             B.active.p, B.rrff.p);
  CKL();
  std::vector<double> h(2 * (size_t)c->n_inst);
  CK(cudaMemcpyAsync(h.data(), B.rrff.p, sizeof(double) * h.size(), cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  check_copy_error(c);
  rr.resize(c->n_inst);
  ff.resize(c->n_inst);
  for (int i = 0; i < c->n_inst; ++i) {
    rr[i] = h[2 * i];
    ff[i] = h[2 * i + 1];
  }
}

int status_of_done(int done) { return done == 1 ? CFEM_OK : done == 2 ? CFEM_ERR_DIVERGED : CFEM_ERR_NOT_CONVERGED; }

}  // namespace
}  // namespace detail
}  // namespace cfem

using namespace cfem;
using namespace cfem::detail;

extern "C" cfem_status cfem_create_batch(cfem_ctx **out, int32_t n, const cfem_mesh *meshes,
                                         const cfem_material *mats, const cfem_options *opt, void *stream) {
  return run_guarded([&]() -> cfem_status {
    if (!out || !meshes || !mats || n <= 0) throw Fail{CFEM_ERR_INVALID_ARGUMENT, "bad batch arguments"};
    // the vector step keeps four ints per instance in shared memory
    if (n > kMaxBatchInstances)
      throw Fail{CFEM_ERR_INVALID_ARGUMENT, "at most " + std::to_string(kMaxBatchInstances) + " meshes per batch"};
    *out = nullptr;
    cfem_mesh all{};
    all.dim = 3;
    std::vector<double> nodes, lvec, fnorm, fpress;
    std::vector<int32_t> elems, cons, lnode, fnodes, felem, group;
    std::unique_ptr<cfem_ctx> c(new cfem_ctx());
    c->n_inst = n;
    c->inst_node_off.assign(1, 0);
    c->inst_elem_off.assign(1, 0);
    for (int i = 0; i < n; ++i) {
      const cfem_mesh &m = meshes[i];
      if (m.dim != 3) throw Fail{CFEM_ERR_INVALID_ARGUMENT, "batched meshes must be 3D"};
      if (!m.nodes || !m.elems || m.n_nodes <= 0 || m.n_elems <= 0)
        throw Fail{CFEM_ERR_INVALID_ARGUMENT, "batch mesh " + std::to_string(i) + " has no nodes or elements"};
      if (m.elem_young) throw Fail{CFEM_ERR_UNSUPPORTED, "per-element Young's modulus in a batch"};
      if ((m.n_constraints > 0 && !m.constraints) || (m.n_loads > 0 && (!m.load_nodes || !m.load_vectors)) ||
          (m.n_faces > 0 && (!m.face_nodes || !m.face_elems || !m.face_normals || !m.face_pressures)))
        throw Fail{CFEM_ERR_INVALID_ARGUMENT, "mesh count given without its array"};
      const double E = mats[i].young_modulus, nu = mats[i].poisson_ratio;
      if (!(E > 0) || !(nu > -1.0) || !(nu < 0.5)) throw Fail{CFEM_ERR_INVALID_ARGUMENT, "invalid material"};
      c->inst_lam.push_back(E * nu / ((1 + nu) * (1 - 2 * nu)));
      c->inst_mu.push_back(E / (2 * (1 + nu)));
      const int32_t noff = (int32_t)c->inst_node_off.back(), eoff = (int32_t)c->inst_elem_off.back();
      nodes.insert(nodes.end(), m.nodes, m.nodes + 3 * m.n_nodes);
      for (int64_t k = 0; k < 4 * m.n_elems; ++k) {
        if (m.elems[k] < 0 || m.elems[k] >= m.n_nodes)
          throw Fail{CFEM_ERR_MESH, "batch mesh " + std::to_string(i) + " references a node out of range"};
        elems.push_back(m.elems[k] + noff);
      }
      group.insert(group.end(), (size_t)m.n_elems, i);
      for (int64_t k = 0; k < m.n_constraints; ++k) {
        cons.push_back(m.constraints[2 * k] + noff);
        cons.push_back(m.constraints[2 * k + 1]);
      }
      for (int64_t k = 0; k < m.n_loads; ++k) {
        lnode.push_back(m.load_nodes[k] + noff);
        for (int d = 0; d < 3; ++d) lvec.push_back(m.load_vectors[3 * k + d]);
      }
      for (int64_t k = 0; k < m.n_faces; ++k) {
        for (int a = 0; a < 4; ++a) fnodes.push_back(m.face_nodes[4 * k + a] + noff);
        felem.push_back(m.face_elems[k] + eoff);
        for (int d = 0; d < 3; ++d) fnorm.push_back(m.face_normals[3 * k + d]);
        fpress.push_back(m.face_pressures[k]);
      }
      c->inst_node_off.push_back(noff + m.n_nodes);
      c->inst_elem_off.push_back(eoff + m.n_elems);
    }
    all.n_nodes = c->inst_node_off.back();
    all.nodes = nodes.data();
    all.n_elems = c->inst_elem_off.back();
    all.elems = elems.data();
    all.n_constraints = (int64_t)cons.size() / 2;
    all.constraints = cons.empty() ? nullptr : cons.data();
    all.n_loads = (int64_t)lnode.size();
    all.load_nodes = lnode.empty() ? nullptr : lnode.data();
    all.load_vectors = lvec.empty() ? nullptr : lvec.data();
    all.n_faces = (int64_t)felem.size();
    all.face_nodes = fnodes.empty() ? nullptr : fnodes.data();
    all.face_elems = felem.empty() ? nullptr : felem.data();
    all.face_normals = fnorm.empty() ? nullptr : fnorm.data();
    all.face_pressures = fpress.empty() ? nullptr : fpress.data();
    c->elem_group = std::move(group);
    attach_stream(c.get(), (cudaStream_t)stream);
    cfem_options o = opt ? *opt : cfem_options{CFEM_CONSISTENT, CFEM_FORM_AUTO, 0, 0};
    if (o.matvec_form == CFEM_FORM_AUTO) o.matvec_form = CFEM_FORM_GRADIENT_FAN;
    setup_context(c.get(), &all, &mats[0], &o);
    *out = c.release();
    return CFEM_OK;
  });
}

extern "C" cfem_status cfem_batch_info(const cfem_ctx *ctx, int32_t *n, int64_t *node_off, int64_t *elem_off) {
  return run_guarded([&]() -> cfem_status {
    check_ctx(ctx);
    if (!ctx->n_inst) throw Fail{CFEM_ERR_INVALID_ARGUMENT, "not a context of batched meshes"};
    if (n) *n = ctx->n_inst;
    if (node_off) std::copy(ctx->inst_node_off.begin(), ctx->inst_node_off.end(), node_off);
    if (elem_off) std::copy(ctx->inst_elem_off.begin(), ctx->inst_elem_off.end(), elem_off);
    return CFEM_OK;
  });
}

extern "C" cfem_status cfem_batch_static_solve(cfem_ctx *ctx, const cfem_solve_params *prm, double *u,
                                               cfem_solve_info *info) {
  return run_guarded([&]() -> cfem_status {
    check_ctx(ctx);
    if (!ctx->n_inst) throw Fail{CFEM_ERR_INVALID_ARGUMENT, "not a context of batched meshes"};
    if (!u) throw Fail{CFEM_ERR_INVALID_ARGUMENT, "null output"};
    if (!ctx->fan_tma) throw Fail{CFEM_ERR_UNSUPPORTED, "batched solve needs the FP32 edge-fan matvec"};
    enter(ctx);
    cfem_solve_params p = prm ? *prm : default_params();
    if (p.precision != CFEM_FP32 && p.precision != CFEM_FP32_REFINE)
      throw Fail{CFEM_ERR_UNSUPPORTED, "batched solves run in CFEM_FP32 or CFEM_FP32_REFINE"};
    cfem_ctx *c = ctx;
    const int n = c->n_inst;
    BatchBufs B;
    B.isc.alloc(n);
    B.ctl.alloc(1);
    B.pe.alloc(c->prep.n_patches);
    B.pp.alloc((size_t)c->prep.n_patches * 3);
    B.seg.alloc((size_t)flat_grid(c) * n * 3);
    if (flat_smem(c) > 48 * 1024)
      CK(cudaFuncSetAttribute((const void *)k_batch_vec_flat<float>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)flat_smem(c)));
    B.scratch.alloc((size_t)n * 3);
    B.rrff.alloc((size_t)n * 2);
    B.active.alloc(n);
    c->launches = 0;
    set_diag_vectors(c, c->diagK.p);
    RhsSchedule sch;
    sch.semantics = c->semantics;
    sch.has_loads = c->rhs.has_loads;
    double a = 0, b = 0;
    sch.eval(0.f, a, b);  // initFlocals(0) of every instance
    make_rhs(c, a, b, c->v64.f.p);
    CK(cudaEventRecord(c->ev0, c->stream));
    std::vector<int> iters(n, 0), outer(n, 0), status(n, CFEM_ERR_NOT_CONVERGED), act(n, 1), none(n, 0);
    std::vector<double> rr, ff, rr_prev(n, -1), g0(n, 0), g1(n, 0);
    std::vector<int> stalls(n, 0);
    std::vector<Scalars> res;
    if (p.precision == CFEM_FP32) {
      k_convert<double, float><<<nblk(c->nvec), kThreads, 0, c->stream>>>(c->nvec, c->v64.f.p, c->v32.f.p);
      CKL();
      run_batch_pcg(c, B, p.tol, p.stop_rule, p.max_iter, res);
      for (int i = 0; i < n; ++i) {
        iters[i] = res[i].iter;
        g0[i] = res[i].gamma0;
        g1[i] = res[i].gamma;
        status[i] = status_of_done(res[i].done);
      }
      k_convert<float, double><<<nblk(c->nvec), kThreads, 0, c->stream>>>(c->nvec, c->v32.x.p, c->v64.x.p);
      CKL();
    } else {
      c->v64.x.zero(c->stream);
      c->tmp64.zero(c->stream);           // K x for x = 0
      batch_residual(c, B, act, rr, ff);  // r = f, f32 = f on every instance
      const double outer_tol = p.outer_tol > 0 ? p.outer_tol : 1e-12;
      const int max_outer = p.max_outer > 0 ? p.max_outer : 50;
      for (int round = 0; round <= max_outer; ++round) {
        int n_act = 0;
        for (int i = 0; i < n; ++i) {
          act[i] = 0;
          if (status[i] == CFEM_OK || status[i] == CFEM_ERR_DIVERGED) continue;
          const bool conv = std::sqrt(rr[i]) <= outer_tol * std::sqrt(ff[i]);
          // the FP64 true residual has a floor near eps64 * ||K|| ||x||: two
          // refinement steps in a row that no longer reduce it as a step
          // should end the instance
          stalls[i] = rr_prev[i] >= 0 && rr[i] > refine_stall_ratio(p.tol) * rr_prev[i] ? stalls[i] + 1 : 0;
          const bool stalled = stalls[i] >= 2;
          if (conv || stalled || ff[i] == 0.0) { status[i] = CFEM_OK; continue; }
          if (round == max_outer) continue;
          act[i] = 1;
          ++n_act;
        }
        if (!n_act) break;
        if (round > 0) {  // f32 = r64 on the still active instances (tmp64 still holds K x)
          std::vector<double> rr2, ff2;
          batch_residual(c, B, act, rr2, ff2);
        }
        run_batch_pcg(c, B, p.tol, p.stop_rule, p.max_iter, res);
        for (int i = 0; i < n; ++i) {
          if (!act[i]) continue;
          iters[i] += res[i].iter;
          if (outer[i] == 0) g0[i] = res[i].gamma0;
          g1[i] = res[i].gamma;
          outer[i] += 1;
          if (res[i].done == 2) status[i] = CFEM_ERR_DIVERGED;
          rr_prev[i] = rr[i];
        }
        k_accumulate<<<nblk(c->nvec), kThreads, 0, c->stream>>>(c->nvec, c->v32.x.p, c->v64.x.p, c->vw);
        CKL();
        batch_kx(c, B);
        batch_residual(c, B, none, rr, ff);
      }
    }
    CK(cudaEventRecord(c->ev1, c->stream));
    CK(cudaEventSynchronize(c->ev1));
    float ms = 0;
    CK(cudaEventElapsedTime(&ms, c->ev0, c->ev1));
    if (p.precision == CFEM_FP32) {
      batch_kx(c, B);
      batch_residual(c, B, none, rr, ff);
    }
    to_caller<double>(c, c->v64.x.p, u);
    CK(cudaStreamSynchronize(c->stream));
    cfem_status worst = CFEM_OK;
    for (int i = 0; i < n; ++i) {
      if (info) {
        cfem_solve_info &in = info[i];
        in = cfem_solve_info{};
        in.status = status[i];
        in.iterations = iters[i];
        in.outer_iterations = outer[i];
        in.rel_residual = ff[i] > 0 ? std::sqrt(rr[i] / ff[i]) : std::sqrt(rr[i]);
        in.gamma0 = g0[i];
        in.gamma = g1[i];
        in.solve_ms = ms;
        in.kernel_launches = c->launches;
      }
      if (status[i] != CFEM_OK && worst == CFEM_OK) worst = (cfem_status)status[i];
    }
    return worst;
  });
}
