// C++ mirror of the reference's solver interface (include/cfem_femfunc.hpp)
// over the C-ABI: run_config JSON, prepared-mesh reader, solver entry points,
// VTK writer.
#include "../../include/cfem_femfunc.hpp"

#include <algorithm>
#include <cctype>
#include <cstring>
#include <cmath>
#include <cstdio>
#include <fstream>
#include <iostream>
#include <map>
#include <memory>
#include <sstream>

extern "C" void cfem_set_error_string(const char *msg);

namespace cfem_ref {

namespace {

// ---------------------------------------------------------------- minimal JSON
struct Json {
  enum Kind { Null, Bool, Number, String, Array, Object } kind = Null;
  bool b = false;
  double num = 0;
  std::string str;
  std::vector<Json> arr;
  std::map<std::string, Json> obj;
  bool has(const std::string &k) const { return kind == Object && obj.count(k); }
  const Json &at(const std::string &k) const {
    auto it = obj.find(k);
    if (kind != Object || it == obj.end()) throw Error(CFEM_ERR_IO, "run_config: missing key '" + k + "'");
    return it->second;
  }
  double number(const std::string &k, double def) const {
    if (!has(k)) return def;
    const Json &v = at(k);
    if (v.kind == Number) return v.num;
    if (v.kind == Bool) return v.b ? 1 : 0;
    throw Error(CFEM_ERR_IO, "run_config: key '" + k + "' is not a number");
  }
  std::string string(const std::string &k, const std::string &def) const {
    if (!has(k)) return def;
    const Json &v = at(k);
    if (v.kind != String) throw Error(CFEM_ERR_IO, "run_config: key '" + k + "' is not a string");
    return v.str;
  }
};

class JsonParser {
 public:
  explicit JsonParser(const std::string &s) : s_(s) {}
  Json parse() {
    Json v = value();
    ws();
    if (i_ != s_.size()) fail("trailing characters");
    return v;
  }

 private:
  const std::string &s_;
  size_t i_ = 0;
  [[noreturn]] void fail(const std::string &m) {
    throw Error(CFEM_ERR_IO, "run_config JSON: " + m + " at offset " + std::to_string(i_));
  }
  void ws() {
    while (i_ < s_.size() && std::isspace((unsigned char)s_[i_])) ++i_;
  }
  bool lit(const char *w) {
    size_t n = std::char_traits<char>::length(w);
    if (s_.compare(i_, n, w) == 0) { i_ += n; return true; }
    return false;
  }
  Json value() {
    ws();
    if (i_ >= s_.size()) fail("unexpected end");
    Json v;
    char c = s_[i_];
    if (c == '{') {
      v.kind = Json::Object;
      ++i_;
      ws();
      if (i_ < s_.size() && s_[i_] == '}') { ++i_; return v; }
      for (;;) {
        ws();
        if (i_ >= s_.size() || s_[i_] != '"') fail("expected key");
        std::string k = string();
        ws();
        if (i_ >= s_.size() || s_[i_] != ':') fail("expected ':'");
        ++i_;
        v.obj[k] = value();
        ws();
        if (i_ < s_.size() && s_[i_] == ',') { ++i_; continue; }
        if (i_ < s_.size() && s_[i_] == '}') { ++i_; return v; }
        fail("expected ',' or '}'");
      }
    }
    if (c == '[') {
      v.kind = Json::Array;
      ++i_;
      ws();
      if (i_ < s_.size() && s_[i_] == ']') { ++i_; return v; }
      for (;;) {
        v.arr.push_back(value());
        ws();
        if (i_ < s_.size() && s_[i_] == ',') { ++i_; continue; }
        if (i_ < s_.size() && s_[i_] == ']') { ++i_; return v; }
        fail("expected ',' or ']'");
      }
    }
    if (c == '"') { v.kind = Json::String; v.str = string(); return v; }
    if (lit("true")) { v.kind = Json::Bool; v.b = true; return v; }
    if (lit("false")) { v.kind = Json::Bool; v.b = false; return v; }
    if (lit("null")) return v;
    size_t start = i_;
    while (i_ < s_.size() && (std::isdigit((unsigned char)s_[i_]) || std::strchr("+-.eE", s_[i_]))) ++i_;
    if (start == i_) fail("unexpected character");
    v.kind = Json::Number;
    v.num = std::strtod(s_.substr(start, i_ - start).c_str(), nullptr);
    return v;
  }
  std::string string() {
    ++i_;  // opening quote
    std::string out;
    while (i_ < s_.size() && s_[i_] != '"') {
      char c = s_[i_++];
      if (c == '\\' && i_ < s_.size()) {
        char e = s_[i_++];
        switch (e) {
          case 'n': out += '\n'; break;
          case 't': out += '\t'; break;
          case 'r': out += '\r'; break;
          case 'b': out += '\b'; break;
          case 'f': out += '\f'; break;
          case 'u': {
            if (i_ + 4 > s_.size()) fail("bad escape");
            unsigned cp = std::stoul(s_.substr(i_, 4), nullptr, 16);
            i_ += 4;
            if (cp < 0x80) out += (char)cp;
            else if (cp < 0x800) { out += (char)(0xc0 | (cp >> 6)); out += (char)(0x80 | (cp & 0x3f)); }
            else { out += (char)(0xe0 | (cp >> 12)); out += (char)(0x80 | ((cp >> 6) & 0x3f)); out += (char)(0x80 | (cp & 0x3f)); }
            break;
          }
          default: out += e;
        }
      } else {
        out += c;
      }
    }
    if (i_ >= s_.size()) fail("unterminated string");
    ++i_;
    return out;
  }
};

// fs::joinString (Tools.cpp:73-92): join with '/', collapse doubled slashes.
std::string join(const std::string &a, const std::string &b) {
  std::string s = a + "/" + b;
  std::string out;
  for (size_t i = 0; i < s.size(); ++i)
    if (!(s[i] == '/' && !out.empty() && out.back() == '/')) out += s[i];
  return out;
}

std::vector<double> read_block(const std::string &path, size_t &count, size_t ncols, bool required) {
  std::ifstream f(path);
  if (!f) {
    if (required) throw Error(CFEM_ERR_IO, "cannot open " + path);
    count = 0;
    return {};
  }
  double n = 0;
  if (!(f >> n)) throw Error(CFEM_ERR_IO, path + ": missing count");
  count = (size_t)n;
  std::vector<double> v(count * ncols);
  for (size_t i = 0; i < v.size(); ++i) {
    double x;
    if (!(f >> x)) throw Error(CFEM_ERR_IO, path + ": expected " + std::to_string(v.size()) + " values");
    v[i] = (double)(float)x;  // the reference stores every value as float
  }
  return v;
}

void check(cfem_status st, const char *where) {
  if (st != CFEM_OK) throw Error(st, std::string(where) + ": " + cfem_last_error_string());
}

}  // namespace

// ---------------------------------------------------------------- dataKeeper
dataKeeper::dataKeeper(std::string configPath, std::string task) : taskName(std::move(task)) {
  parseJsonConfig(configPath);
  parseFiles();
}

dataKeeper::~dataKeeper() {
  if (ctx) cfem_destroy(ctx);
}

void dataKeeper::parseJsonConfig(const std::string &configPath) {
  std::ifstream f(configPath);
  if (!f) throw Error(CFEM_ERR_IO, "cannot open run_config " + configPath);
  std::stringstream ss;
  ss << f.rdbuf();
  Json cfg = JsonParser(ss.str()).parse();
  DIM = (size_t)cfg.at("DIM").num;
  if (DIM != 2 && DIM != 3) throw Error(CFEM_ERR_INVALID_ARGUMENT, "DIM must be 2 or 3");
  paths.proj_dir = cfg.string("CudaFEMproject_path", "undefined_path");
  paths.work_dir = cfg.string("working_path", "undefined_path");
  paths.res_dir = join(paths.work_dir, "/fem_results/" + std::to_string(DIM) + "D/" + taskName);
  paths.prep_mesh_dir = join(paths.work_dir, "/prepared_meshes/" + std::to_string(DIM) + "D/" + taskName);
  paths.output_vtk = join(paths.res_dir, "/results.vtk");
  mechParams.youngModulus = (float)cfg.number("youngModulus", 2e7);
  mechParams.poissonRatio = (float)cfg.number("poissonRatio", 0.3);
  save_segy = cfg.number("save_segy", 0) != 0;
  taskType = cfg.string("task_type", "static");
  // the C++ reference compares "dynamic", its Python driver "DYNAMICS" (run_fem.py:21-23)
  std::string lower;
  for (char c : taskType) lower += (char)std::tolower((unsigned char)c);
  if (lower == "dynamic" || lower == "dynamics") {
    taskType = "dynamic";
    mechParams.rho = (float)cfg.number("rho", 2400.0);
    mechParams.beta1 = (float)cfg.number("beta1", 0.5);
    mechParams.beta2 = (float)cfg.number("beta2", 0.0);
    mechParams.damping_alpha = (float)cfg.number("damping_alpha", 0.0);
    mechParams.damping_beta = (float)cfg.number("damping_beta", 0.0);
    mechParams.dt = (float)cfg.number("dt", 1e-3);
    mechParams.endtime = (float)cfg.number("endtime", 0.1);
  }
  if (cfg.has("wavelet")) {
    const Json &w = cfg.at("wavelet");
    waveParams.waveletType = w.string("WaveletType", "default");
    waveParams.freq = (float)w.number("freq", 15.0);
    waveParams.timeshift = (float)w.number("timeshift", 0.0);
    waveParams.ampl = (float)w.number("ampl", 1.0);
  }
  if (cfg.has("gb300")) {
    const Json &g = cfg.at("gb300");
    std::string sem = g.string("semantics", "compat"), prec = g.string("precision", "fp32"),
                rule = g.string("stop_rule", "reference");
    gb300.semantics = sem == "consistent" ? CFEM_CONSISTENT : CFEM_COMPAT;
    gb300.precision = prec == "fp64" ? CFEM_FP64 : prec == "fp32_refine" ? CFEM_FP32_REFINE : CFEM_FP32;
    gb300.stop_rule = rule == "residual" ? CFEM_STOP_RESIDUAL : CFEM_STOP_REFERENCE;
    gb300.tol = g.number("tol", -1);
    gb300.outer_tol = g.number("outer_tol", 1e-12);
    gb300.max_iter = (int)g.number("max_iter", 1000000);
    gb300.patch_elems = (int)g.number("patch_elems", 0);
  }
}

void dataKeeper::parseFiles() {
  const std::string &d = paths.prep_mesh_dir;
  const size_t nv = DIM + 1;
  nodes = read_block(join(d, "nodes.txt"), nodesCount, DIM, true);
  std::vector<double> el = read_block(join(d, "elements.txt"), elementsCount, nv, true);
  if (nodesCount == 0 || elementsCount == 0) throw Error(CFEM_ERR_MESH, "task without nodes or elements");
  elementsIds.assign(el.size(), 0);
  for (size_t i = 0; i < el.size(); ++i) elementsIds[i] = (int32_t)el[i];
  std::vector<double> cs = read_block(join(d, "constraints.txt"), constraintsCount, 2, false);
  constraints.assign(cs.size(), 0);
  for (size_t i = 0; i < cs.size(); ++i) constraints[i] = (int32_t)cs[i];
  std::vector<double> ld = read_block(join(d, "loads.txt"), loadsCount, DIM + 1, false);
  loadsNodes.resize(loadsCount);
  loadsVectors.resize(loadsCount * DIM);
  for (size_t i = 0; i < loadsCount; ++i) {
    loadsNodes[i] = (int32_t)ld[i * (DIM + 1)];
    for (size_t j = 0; j < DIM; ++j) loadsVectors[i * DIM + j] = ld[i * (DIM + 1) + 1 + j];
  }
  const size_t sc = (DIM + 1) + 1 + DIM + 1;
  std::vector<double> st = read_block(join(d, "stress.txt"), boundaryEdgesCount, sc, false);
  boundaryNodes.resize(boundaryEdgesCount * (DIM + 1));
  boundaryAdjElems.resize(boundaryEdgesCount);
  boundaryNormals.resize(boundaryEdgesCount * DIM);
  boundaryPressures.resize(boundaryEdgesCount);
  for (size_t i = 0; i < boundaryEdgesCount; ++i) {
    const double *r = st.data() + i * sc;
    for (size_t j = 0; j <= DIM; ++j) boundaryNodes[i * (DIM + 1) + j] = (int32_t)r[j];
    boundaryAdjElems[i] = (int32_t)r[DIM + 1];
    for (size_t j = 0; j < DIM; ++j) boundaryNormals[i * DIM + j] = r[DIM + 2 + j];
    boundaryPressures[i] = r[2 * DIM + 2];
  }
  displacements = HostMatrix(nodesCount, DIM);
  displacements64.assign(nodesCount * DIM, 0.0);
}

void dataKeeper::ShowInfo() const {
  std::cout << "==========INFO==========\nTask name = " << taskName << "\nNodes count = " << nodesCount
            << "\nElements count = " << elementsCount << "\nConstraints count = " << constraintsCount
            << "\nLoads count = " << loadsCount << "\nBoundary edges with b.c. count = " << boundaryEdgesCount
            << "\n========================\n\n";
}

cfem_mesh dataKeeper::mesh_view() const {
  cfem_mesh m{};
  m.dim = (int32_t)DIM;
  m.n_nodes = (int64_t)nodesCount;
  m.nodes = nodes.data();
  m.n_elems = (int64_t)elementsCount;
  m.elems = elementsIds.data();
  m.n_constraints = (int64_t)constraintsCount;
  m.constraints = constraints.empty() ? nullptr : constraints.data();
  m.n_loads = (int64_t)loadsCount;
  m.load_nodes = loadsNodes.empty() ? nullptr : loadsNodes.data();
  m.load_vectors = loadsVectors.empty() ? nullptr : loadsVectors.data();
  m.n_faces = (int64_t)boundaryEdgesCount;
  m.face_nodes = boundaryNodes.empty() ? nullptr : boundaryNodes.data();
  m.face_elems = boundaryAdjElems.empty() ? nullptr : boundaryAdjElems.data();
  m.face_normals = boundaryNormals.empty() ? nullptr : boundaryNormals.data();
  m.face_pressures = boundaryPressures.empty() ? nullptr : boundaryPressures.data();
  m.elem_young = nullptr;
  return m;
}

cfem_material dataKeeper::material() const {
  return cfem_material{mechParams.youngModulus, mechParams.poissonRatio, mechParams.rho};
}

cfem_wavelet dataKeeper::wavelet() const {
  cfem_wavelet w{};
  w.type = waveParams.waveletType == "ricker" ? CFEM_WAVELET_RICKER
           : waveParams.waveletType == "berlage" ? CFEM_WAVELET_BERLAGE : CFEM_WAVELET_NONE;
  w.freq = waveParams.freq;
  w.timeshift = waveParams.timeshift;
  w.ampl = waveParams.ampl;
  return w;
}

cfem_ctx *dataKeeper::context() {
  if (!ctx) {
    cfem_mesh m = mesh_view();
    cfem_material mat = material();
    cfem_options opt{};
    opt.semantics = gb300.semantics;
    opt.matvec_form = CFEM_FORM_GRADIENT;
    opt.patch_elems = gb300.patch_elems;
    check(cfem_create(&ctx, &m, &mat, &opt, nullptr), "cfem_create");
  }
  return ctx;
}

// ---------------------------------------------------------------- solvers
namespace {
cfem_solve_params static_params(const dataKeeper &dk, double default_eps) {
  const Gb300Options &g = dk.getGb300Options();
  cfem_solve_params p{};
  p.precision = g.precision;
  p.stop_rule = g.stop_rule;
  p.tol = g.tol > 0 ? g.tol : default_eps;
  p.max_iter = g.max_iter;
  p.outer_tol = g.outer_tol;
  p.max_outer = 50;
  return p;
}

void store(dataKeeper &dk, const std::vector<double> &u) {
  dk.displacements_fp64() = u;
  HostMatrix *m = dk.get_displacements();
  for (size_t i = 0; i < u.size(); ++i) m->get_data()[i] = (float)u[i];
}

void report_static(const cfem_solve_info &inf, bool verbose) {
  if (verbose)
    std::cout << "PCG iterations = " << inf.iterations << " (outer " << inf.outer_iterations << ")\ngamma0\t\t\t= "
              << inf.gamma0 << "\ngamma_new\t\t= " << inf.gamma << "\nrelative residual\t= " << inf.rel_residual
              << "\nsolve time [ms]\t\t= " << inf.solve_ms << "\n";
}
}  // namespace

void gpuCalculateFEM_EbE_vec(DEVICE_NAME, dataKeeper &dk, bool PRINT_DEBUG_INFO, SolveReport *report) {
  cfem_ctx *c = dk.context();
  cfem_solve_params p = static_params(dk, 1e-8);
  cfem_wavelet w = dk.wavelet();
  std::vector<double> u(dk.get_nodesCount() * dk.get_dim());
  cfem_solve_info inf{};
  cfem_status st = cfem_static_solve(c, &w, &p, u.data(), &inf);
  report_static(inf, PRINT_DEBUG_INFO);
  if (report) report->static_info = inf;
  check(st, "gpuCalculateFEM_EbE_vec");
  store(dk, u);
}

void gpuPCG_EbE_vec(std::vector<double> &displacements, DEVICE_NAME, dataKeeper &dk, const std::vector<double> &rhs,
                    float eps, bool PRINT_DEBUG_INFO, SolveReport *report) {
  cfem_ctx *c = dk.context();
  const size_t nd = dk.get_nodesCount() * dk.get_dim();
  if (rhs.size() != nd) throw Error(CFEM_ERR_INVALID_ARGUMENT, "rhs size differs from n_nodes * DIM");
  cfem_solve_params p = static_params(dk, eps);
  displacements.assign(nd, 0.0);
  cfem_solve_info inf{};
  cfem_status st = cfem_pcg(c, &p, rhs.data(), displacements.data(), &inf);
  report_static(inf, PRINT_DEBUG_INFO);
  if (report) report->static_info = inf;
  check(st, "gpuPCG_EbE_vec");
}

ElementsData *ElementsData::setElementsData(DEVICE_NAME device, dataKeeper &dk) {
  return new ElementsData(device, dk);
}

void ElementOperator::getDiagonal(size_t, HostMatrix &diag) const {
  dataKeeper &dk = ed_->keeper();
  std::vector<double> d(dk.get_nodesCount() * dk.get_dim());
  check(cfem_diagonal(dk.context(), d.data()), "getDiagonal");
  HostMatrix m(dk.get_nodesCount(), dk.get_dim());
  for (size_t i = 0; i < d.size(); ++i) m[i] = (float)d[i];
  m.copy(diag);
}

void ElementsData::initFlocals(float t, const WaveletParams &w) {
  cfem_wavelet cw = dk_.wavelet();
  cw.type = w.waveletType == "ricker" ? CFEM_WAVELET_RICKER
            : w.waveletType == "berlage" ? CFEM_WAVELET_BERLAGE : CFEM_WAVELET_NONE;
  cw.freq = w.freq;
  cw.timeshift = w.timeshift;
  cw.ampl = w.ampl;
  std::vector<double> f(dk_.get_nodesCount() * dk_.get_dim());
  check(cfem_rhs(dk_.context(), &cw, (double)t, f.data()), "initFlocals");
  HostMatrix m(dk_.get_nodesCount(), dk_.get_dim());
  for (size_t i = 0; i < f.size(); ++i) m[i] = (float)f[i];
  m.copy(Flocals_);
}

void gpuPCG_EbE_vec(HostMatrix &displacements, DEVICE_NAME deviceType, dataKeeper &FEMdata, ElementsData &elemsData,
                    bool doAssemblyRes, float eps, bool PRINT_DEBUG_INFO) {
  const size_t dim = FEMdata.get_dim(), nn = FEMdata.get_nodesCount(), nd = nn * dim;
  HostMatrix *r = elemsData.get_r();
  if (r->get_numElements() != nd)
    throw Error(CFEM_ERR_INVALID_ARGUMENT, "gpuPCG_EbE_vec: elemsData.get_r() holds " +
                                               std::to_string(r->get_numElements()) + " values, n_nodes * DIM is " +
                                               std::to_string(nd) + " (initFlocals, then get_Flocals()->copy(*get_r()))");
  std::vector<double> f(r->get_data(), r->get_data() + nd), u;
  gpuPCG_EbE_vec(u, deviceType, FEMdata, f, eps, PRINT_DEBUG_INFO, nullptr);
  if (doAssemblyRes) {
    HostMatrix out(nn, dim);
    for (size_t i = 0; i < nd; ++i) out[i] = (float)u[i];
    out.copy(displacements);
  } else {
    const std::vector<int32_t> &el = FEMdata.get_elementsIds();
    const size_t nv = dim + 1, ne = FEMdata.get_elementsCount(), w = nv * dim;
    HostMatrix out(ne, w);
    for (size_t e = 0; e < ne; ++e)
      for (size_t a = 0; a < nv; ++a)
        for (size_t d = 0; d < dim; ++d) out(e, a * dim + d) = (float)u[(size_t)el[e * nv + a] * dim + d];
    out.copy(displacements);
  }
}

void gpuCalculateFEM_DYN(DEVICE_NAME, dataKeeper &dk, bool PRINT_DEBUG_INFO, SolveReport *report) {
  cfem_ctx *c = dk.context();
  const MechanicalParams mp = dk.getMechParams();
  const Gb300Options &g = dk.getGb300Options();
  cfem_dyn_params p{};
  p.beta1 = mp.beta1;
  p.beta2 = mp.beta2;
  p.dt = mp.dt;
  p.endtime = mp.endtime;
  p.precision = g.precision == CFEM_FP64 ? CFEM_FP64 : CFEM_FP32;
  p.pcg_tol = g.tol > 0 ? g.tol : 1e-4;
  p.stop_rule = g.stop_rule;
  p.max_iter = g.max_iter;
  p.warm_start = g.semantics == CFEM_CONSISTENT;
  cfem_wavelet w = dk.wavelet();
  std::vector<double> u(dk.get_nodesCount() * dk.get_dim());
  cfem_dyn_info inf{};
  cfem_status st = cfem_dyn(c, &p, &w, u.data(), &inf);
  if (PRINT_DEBUG_INFO)
    std::cout << "time steps = " << inf.steps << ", PCG iterations = " << inf.pcg_iterations
              << ", time [ms] = " << inf.solve_ms << "\n";
  if (report) report->dyn_info = inf;
  check(st, "gpuCalculateFEM_DYN");
  store(dk, u);
}

// ---------------------------------------------------------------- VTK (VTKfile.cpp:281-386)
void MakeVTKfile2D(const std::string &output_vtk, const std::vector<double> &nodes, const std::vector<int32_t> &elements,
                   const HostMatrix &displacements) {
  std::ofstream out(output_vtk);
  if (!out) throw Error(CFEM_ERR_IO, "cannot write " + output_vtk);
  const size_t dim = 2, nn = nodes.size() / dim, ne = elements.size() / (dim + 1);
  out << "# vtk DataFile Version 1.0\nresults.vtk  2D Unstructured Grid of Triangles\nASCII\n\nDATASET "
         "UNSTRUCTURED_GRID\nPOINTS "
      << nn << " float\n";
  for (size_t i = 0; i < nn; ++i) {
    for (size_t j = 0; j < dim; ++j) out << (float)nodes[i * dim + j] << " ";
    out << "0.0\n";
  }
  out << "\nCELLS " << ne << " " << ne * 4 << "\n";
  for (size_t i = 0; i < ne; ++i) {
    out << dim + 1 << " ";
    for (size_t j = 0; j <= dim; ++j) out << (float)elements[i * (dim + 1) + j] << " ";
    out << "\n";
  }
  out << "\nCELL_TYPES " << ne << "\n";
  for (size_t i = 0; i < ne; ++i) out << 5 << "\n";
  out << "\nPOINT_DATA " << nn << "\n";
  out << "\nVECTORS displacements float\n";
  for (size_t i = 0; i < displacements.get_numRows(); ++i) {
    for (size_t j = 0; j < displacements.get_numCols(); ++j) out << displacements(i, j) << " ";
    out << "0.0\n";
  }
  out << "\nSCALARS summary float\nLOOKUP_TABLE default\n";
  for (size_t i = 0; i < displacements.get_numRows(); ++i) {
    float s = 0.f;
    for (size_t j = 0; j < displacements.get_numCols(); ++j) s += displacements(i, j) * displacements(i, j);
    out << std::sqrt(s) << "\n";
  }
}

void MakeVTKfile3D(const std::string &output_vtk, const std::vector<double> &nodes, const std::vector<int32_t> &elements,
                   const HostMatrix &displacements) {
  std::ofstream out(output_vtk);
  if (!out) throw Error(CFEM_ERR_IO, "cannot write " + output_vtk);
  const size_t dim = 3, nn = nodes.size() / dim, ne = elements.size() / (dim + 1);
  out << "# vtk DataFile Version 1.0\nresults.vtk  3D Unstructured Grid of Triangles\nASCII\n\nDATASET "
         "UNSTRUCTURED_GRID\nPOINTS "
      << nn << " float\n";
  for (size_t i = 0; i < nn; ++i) {
    for (size_t j = 0; j < dim; ++j) out << (float)nodes[i * dim + j] << " ";
    out << "\n";
  }
  out << "CELLS " << ne << " " << ne * 5 << "\n";
  for (size_t i = 0; i < ne; ++i) {
    out << dim + 1 << " ";
    for (size_t j = 0; j <= dim; ++j) out << (float)elements[i * (dim + 1) + j] << " ";
    out << "\n";
  }
  out << "CELL_TYPES " << ne << "\n";
  for (size_t i = 0; i < ne; ++i) out << 10 << "\n";
  out << "\nPOINT_DATA " << nn << "\n";
  out << "\nVECTORS displacements float\n";
  for (size_t i = 0; i < displacements.get_numRows(); ++i) {
    for (size_t j = 0; j < displacements.get_numCols(); ++j) out << displacements(i, j) << " ";
    out << "\n";
  }
  out << "\nSCALARS summary float\nLOOKUP_TABLE default\n";
  for (size_t i = 0; i < displacements.get_numRows(); ++i) {
    float s = 0.f;
    for (size_t j = 0; j < displacements.get_numCols(); ++j) s += displacements(i, j) * displacements(i, j);
    out << std::sqrt(s) << "\n";
  }
}

void WriteResults(dataKeeper &dk, ResultsDataKeeper &) { WriteResults(dk); }

void WriteResults(dataKeeper &dk) {
  const dataPaths p = dk.getDataPaths();
  if (dk.get_dim() == 2)
    MakeVTKfile2D(p.output_vtk, dk.get_nodes(), dk.get_elementsIds(), *dk.get_displacements());
  else
    MakeVTKfile3D(p.output_vtk, dk.get_nodes(), dk.get_elementsIds(), *dk.get_displacements());
}

}  // namespace cfem_ref

namespace cfem_ref {
std::vector<std::string> readTaskList(const std::string &configPath) {
  std::ifstream f(configPath);
  if (!f) throw Error(CFEM_ERR_IO, "cannot open run_config " + configPath);
  std::stringstream ss;
  ss << f.rdbuf();
  Json cfg = JsonParser(ss.str()).parse();
  std::vector<std::string> out;
  if (!cfg.has("task")) return out;
  const Json &t = cfg.at("task");
  if (t.kind == Json::String) out.push_back(t.str);
  for (const Json &v : t.arr)
    if (v.kind == Json::String) out.push_back(v.str);
  return out;
}
}  // namespace cfem_ref

extern "C" CFEM_API cfem_status cfem_write_vtk(const char *path, int32_t dim, const double *nodes, int64_t n_nodes,
                                               const int32_t *elems, int64_t n_elems, const float *u) {
  try {
    if (!path || (dim != 2 && dim != 3) || n_nodes < 0 || n_elems < 0 || (n_nodes && (!nodes || !u)) ||
        (n_elems && !elems))
      throw cfem_ref::Error(CFEM_ERR_INVALID_ARGUMENT, "bad cfem_write_vtk arguments");
    std::vector<double> nv(nodes, nodes + n_nodes * dim);
    std::vector<int32_t> ev(elems, elems + n_elems * (dim + 1));
    cfem_ref::HostMatrix d((size_t)n_nodes, (size_t)dim);
    std::copy(u, u + n_nodes * dim, d.get_data());
    if (dim == 2) cfem_ref::MakeVTKfile2D(path, nv, ev, d);
    else cfem_ref::MakeVTKfile3D(path, nv, ev, d);
    return CFEM_OK;
  } catch (const cfem_ref::Error &e) {
    cfem_set_error_string(e.what());
    return e.status;
  } catch (const std::exception &e) {
    cfem_set_error_string(e.what());
    return CFEM_ERR_IO;
  }
}

extern "C" CFEM_API cfem_status cfem_run_task(const char *config_path, const char *task, int32_t write_vtk,
                                              double *u_out, int64_t n_out, cfem_solve_info *static_info,
                                              cfem_dyn_info *dyn_info) {
  try {
    if (!config_path || !task) throw cfem_ref::Error(CFEM_ERR_INVALID_ARGUMENT, "null config path or task");
    cfem_ref::dataKeeper dk(config_path, task);
    cfem_ref::SolveReport rep;
    if (dk.getTaskType() == "dynamic")
      cfem_ref::gpuCalculateFEM_DYN(cfem_ref::GB300, dk, false, &rep);
    else
      cfem_ref::gpuCalculateFEM_EbE_vec(cfem_ref::GB300, dk, false, &rep);
    if (static_info) *static_info = rep.static_info;
    if (dyn_info) *dyn_info = rep.dyn_info;
    if (u_out) {
      const std::vector<double> &u = dk.get_displacements64();
      if ((int64_t)u.size() > n_out) throw cfem_ref::Error(CFEM_ERR_INVALID_ARGUMENT, "u_out too small");
      std::copy(u.begin(), u.end(), u_out);
    }
    if (write_vtk) cfem_ref::WriteResults(dk);
    return CFEM_OK;
  } catch (const cfem_ref::Error &e) {
    cfem_set_error_string(e.what());
    return e.status;
  } catch (const std::exception &e) {
    cfem_set_error_string(e.what());
    return CFEM_ERR_IO;
  }
}
