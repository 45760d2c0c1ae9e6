// femfunc_gb300.cpp -- see femfunc_gb300.h.
#include "femfunc_gb300.h"

#include <iostream>
#include <stdexcept>
#include <string>

namespace gb300 {

namespace {

std::vector<double> widen_f(const Matrix *m) {
  return std::vector<double>(m->get_data(), m->get_data() + m->get_numElements());
}

std::vector<int32_t> widen_i(const Matrix *m) {
  std::vector<int32_t> v(m->get_numElements());
  for (size_t i = 0; i < v.size(); ++i) v[i] = static_cast<int32_t>(m->get_data()[i]);
  return v;
}

void check(cfem_status st, const char *what) {
  if (st != CFEM_OK) throw std::runtime_error(std::string(what) + ": " + cfem_last_error_string());
}

// One context per call, destroyed on every path.
struct Context {
  cfem_ctx *ctx = nullptr;
  explicit Context(const TaskArrays &t) {
    cfem_options opt{};
    opt.semantics = CFEM_COMPAT;
    opt.matvec_form = CFEM_FORM_AUTO;
    check(cfem_create(&ctx, &t.mesh, &t.material, &opt, nullptr), "cfem_create");
  }
  ~Context() { cfem_destroy(ctx); }
};

void store(dataKeeper &dk, const std::vector<double> &u) {
  float *out = dk.get_displacements()->get_data();
  for (size_t i = 0; i < u.size(); ++i) out[i] = static_cast<float>(u[i]);
}

}  // namespace

TaskArrays widen(const dataKeeper &dk) {
  TaskArrays t;
  const size_t dim = dk.get_dim(), nn = dk.get_nodesCount();
  t.nodes = widen_f(dk.get_nodes());
  t.elems = widen_i(dk.get_elementsIds());
  // The decoded DOF list is the exact constraint set (rows of constraints.txt
  // for the same node accumulate there, while constraintsTypes keeps only the
  // last code). Per node, the DOF bits map back to a code that decodes to the
  // same DOFs: x,y -> UX, UY; in 3D every code with an x or y bit also sets z
  // (Constraint::UZ == 3, femstruct.h:39-52), so the sets are {x,z}, {y,z} and
  // {x,y,z}.
  std::vector<uint8_t> bits(nn, 0);
  const Matrix *ids = dk.get_constraintsIds();  // read unconditionally, as cpu_fem_utils.cpp:21 does
  for (size_t k = 0; k < ids->get_numElements(); ++k) {
    const size_t dof = static_cast<size_t>(ids->get_data()[k]);
    bits[dof / dim] |= static_cast<uint8_t>(1u << (dof % dim));
  }
  for (size_t n = 0; n < nn; ++n) {
    const unsigned b = bits[n] & 3u;
    if (!bits[n]) continue;
    const int32_t code = b == 3u ? (dim == 3 ? 7 : 3) : static_cast<int32_t>(b);
    t.constraints.push_back(static_cast<int32_t>(n));
    t.constraints.push_back(code);
  }
  if (dk.get_loadsCount() > 0) {
    t.load_nodes = widen_i(dk.get_loadsNodes());
    t.load_vectors = widen_f(dk.get_loadsVectors());
  }
  if (dk.get_boundaryEdgesCount() > 0) {
    t.face_nodes = widen_i(dk.get_boundaryNodes());
    t.face_elems = widen_i(dk.get_boundaryAdjElems());
    t.face_normals = widen_f(dk.get_boundaryNormals());
    t.face_pressures = widen_f(dk.get_boundaryPressures());
  }
  cfem_mesh &m = t.mesh;
  m.dim = static_cast<int32_t>(dim);
  m.n_nodes = static_cast<int64_t>(nn);
  m.nodes = t.nodes.data();
  m.n_elems = static_cast<int64_t>(dk.get_elementsCount());
  m.elems = t.elems.data();
  m.n_constraints = static_cast<int64_t>(t.constraints.size() / 2);
  m.constraints = t.constraints.empty() ? nullptr : t.constraints.data();
  m.n_loads = static_cast<int64_t>(t.load_nodes.size());
  m.load_nodes = t.load_nodes.empty() ? nullptr : t.load_nodes.data();
  m.load_vectors = t.load_vectors.empty() ? nullptr : t.load_vectors.data();
  m.n_faces = static_cast<int64_t>(t.face_elems.size());
  m.face_nodes = t.face_nodes.empty() ? nullptr : t.face_nodes.data();
  m.face_elems = t.face_elems.empty() ? nullptr : t.face_elems.data();
  m.face_normals = t.face_normals.empty() ? nullptr : t.face_normals.data();
  m.face_pressures = t.face_pressures.empty() ? nullptr : t.face_pressures.data();
  m.elem_young = nullptr;
  const MechanicalParams mp = dk.getMechParams();
  t.material.young_modulus = mp.youngModulus;
  t.material.poisson_ratio = mp.poissonRatio;
  t.material.rho = dk.getTaskType() == "dynamic" ? mp.rho : 2400.0;  // rho is read for dynamic tasks only
  return t;
}

cfem_wavelet wavelet(const WaveletParams &w) {
  cfem_wavelet c{};
  c.type = w.waveletType == "ricker" ? CFEM_WAVELET_RICKER
           : w.waveletType == "berlage" ? CFEM_WAVELET_BERLAGE : CFEM_WAVELET_NONE;
  c.freq = w.freq;
  c.timeshift = w.timeshift;
  c.ampl = w.ampl;
  return c;
}

void calculateFEM_EbE_vec(dataKeeper &dk, bool verbose) {
  const TaskArrays t = widen(dk);
  Context c(t);
  cfem_solve_params prm{};
  prm.precision = CFEM_FP32;
  prm.stop_rule = CFEM_STOP_REFERENCE;
  prm.tol = 1e-8;
  prm.max_iter = 1000000;
  prm.outer_tol = 1e-12;
  prm.max_outer = 50;
  const cfem_wavelet w = wavelet(dk.getWaveletParams());
  std::vector<double> u(dk.get_nodesCount() * dk.get_dim());
  cfem_solve_info info{};
  check(cfem_static_solve(c.ctx, &w, &prm, u.data(), &info), "gpuCalculateFEM_EbE_vec");
  if (verbose) std::cout << "PCG iterations = " << info.iterations << ", gamma0 = " << info.gamma0 << "\n";
  store(dk, u);
}

void calculateFEM_DYN(dataKeeper &dk, bool verbose) {
  const TaskArrays t = widen(dk);
  Context c(t);
  const MechanicalParams mp = dk.getMechParams();
  cfem_dyn_params prm{};
  prm.beta1 = mp.beta1;
  prm.beta2 = mp.beta2;
  prm.dt = mp.dt;
  prm.endtime = mp.endtime;
  prm.precision = CFEM_FP32;
  prm.pcg_tol = 1e-4;
  prm.stop_rule = CFEM_STOP_REFERENCE;
  prm.max_iter = 1000000;
  const cfem_wavelet w = wavelet(dk.getWaveletParams());
  std::vector<double> u(dk.get_nodesCount() * dk.get_dim());
  cfem_dyn_info info{};
  check(cfem_dyn(c.ctx, &prm, &w, u.data(), &info), "gpuCalculateFEM_DYN");
  if (verbose) std::cout << "time steps = " << info.steps << ", PCG iterations = " << info.pcg_iterations << "\n";
  store(dk, u);
}

}  // namespace gb300
