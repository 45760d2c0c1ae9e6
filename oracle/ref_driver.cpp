// Test infrastructure only (never shipped or measured as the product).
//
// A small driver, written for this project, that runs the reference's own CPU
// path through its public API (FEMproject/femfunc/src/femfunc.h:20-24,
// FEMproject/DataKeeper/src/datakeeper.h:56-139,
// FEMproject/fem_utils/include/fem_utils_cpu.h:24-148). It is linked against
// the unmodified reference sources by oracle/ref.mk.
//
//   ref_driver static <config.json> <task> <out.bin>   displacements, float32 n_nodes*DIM
//   ref_driver dyn    <config.json> <task> <out.bin>   same, after gpuCalculateFEM_DYN
//   ref_driver dump   <config.json> <task> <outdir>    setup arrays (mask, adjElements,
//                                                       Klocals, Flocals, constraints ...)
//   ref_driver iters  <config.json> <task> <k>         setup time + k timed PCG iterations
//   ref_driver segy   <out.sgy> <receivers.txt> <nodes.txt> <dim> <dof> <type> <n_elems>
//                     receiver text file -> SEG-Y by the reference's segyUtils convert()
//
// Every mode prints one JSON line on stdout with timings and counters.
#include <VTKfile.h>
#include <femfunc.h>
#include <segyUtils.h>

#include <chrono>
#include <cstdio>
#include <fstream>
#include <sstream>
#include <string>

namespace {

double now_s() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

void write_bin(const std::string &path, const Matrix &m) {
  std::ofstream f(path, std::ios::binary);
  f.write(reinterpret_cast<const char *>(m.get_data()), sizeof(float) * m.get_numElements());
}

// Counts "Iteration #" lines printed by the reference's verbose PCG
// (femfunc.cpp:61-63) while the solver's std::cout output is captured.
int count_iterations(const std::string &text) {
  int n = 0;
  size_t pos = 0;
  while ((pos = text.find("Iteration #", pos)) != std::string::npos) { ++n; pos += 11; }
  return n;
}

int run_solve(bool dyn, const std::string &cfg, const std::string &task, const std::string &out) {
  double t0 = now_s();
  dataKeeper dk(cfg, task);
  double t1 = now_s();
  std::stringstream captured;
  std::streambuf *old = std::cout.rdbuf(captured.rdbuf());
  if (dyn)
    gpuCalculateFEM_DYN(CPU, dk, true);
  else
    gpuCalculateFEM_EbE_vec(CPU, dk, true);
  std::cout.rdbuf(old);
  double t2 = now_s();
  write_bin(out, *dk.get_displacements());
  std::printf("{\"parse_s\": %.6f, \"solve_s\": %.6f, \"pcg_iterations\": %d, \"nodes\": %zu, \"elements\": %zu}\n",
              t1 - t0, t2 - t1, count_iterations(captured.str()), dk.get_nodesCount(), dk.get_elementsCount());
  return 0;
}

// Static CPU solve, then the reference's own results writer (VTKfile.cpp
// MakeVTKfile2D/3D) on the task's nodes, elements and displacements.
int run_vtk(const std::string &cfg, const std::string &task, const std::string &out_vtk) {
  dataKeeper dk(cfg, task);
  std::stringstream captured;
  std::streambuf *old = std::cout.rdbuf(captured.rdbuf());
  gpuCalculateFEM_EbE_vec(CPU, dk, false);
  if (dk.get_dim() == 2)
    MakeVTKfile2D(out_vtk, *dk.get_nodes(), *dk.get_elementsIds(), *dk.get_displacements());
  else
    MakeVTKfile3D(out_vtk, *dk.get_nodes(), *dk.get_elementsIds(), *dk.get_displacements());
  std::cout.rdbuf(old);
  std::printf("{\"mode\": \"vtk\", \"nodes\": %zu, \"elements\": %zu}\n", dk.get_nodesCount(), dk.get_elementsCount());
  return 0;
}

int run_dump(const std::string &cfg, const std::string &task, const std::string &dir) {
  dataKeeper dk(cfg, task);
  ElementsData *ed = ElementsData::setElementsData(CPU, dk);
  double t0 = now_s();
  ed->genMask();
  double t1 = now_s();
  ed->calculateKlocals();
  double t2 = now_s();
  ed->get_Klocals()->getDiagonal(6 * (dk.get_dim() - 1), *ed->get_diagK());
  ed->initFlocals(0.f, dk.getWaveletParams());
  write_bin(dir + "/mask.bin", *ed->get_mask());
  write_bin(dir + "/adjElements.bin", *ed->get_adjElements());
  write_bin(dir + "/Klocals.bin", *ed->get_Klocals());
  write_bin(dir + "/diagK.bin", *ed->get_diagK());
  write_bin(dir + "/Flocals.bin", *ed->get_Flocals());
  write_bin(dir + "/elementsAreas.bin", *ed->get_elementsAreas());
  write_bin(dir + "/Blocals.bin", *ed->get_Blocals());
  write_bin(dir + "/D.bin", *dk.get_D());
  if (dk.get_constraintsIds() && dk.get_constraintsIds()->get_numElements() > 0) {
    write_bin(dir + "/constraintsIds.bin", *dk.get_constraintsIds());
    write_bin(dir + "/constraintsTypes.bin", *dk.get_constraintsTypes());
  }
  // Mass matrices are only built by the dynamics driver; dump both variants.
  MechanicalParams mp = dk.getMechParams();
  if (mp.rho == 0.f) mp.rho = 1.f;
  ed->calculateMlocals(true, mp);
  write_bin(dir + "/Mlumped.bin", *ed->get_Mlocals());
  ed->calculateMlocals(false, mp);
  write_bin(dir + "/Mconsistent.bin", *ed->get_Mlocals());
  std::printf("{\"genMask_s\": %.6f, \"calculateKlocals_s\": %.6f, \"rho\": %g}\n", t1 - t0, t2 - t1, mp.rho);
  delete ed;
  return 0;
}

// Times the reference's setup and k iterations of its PCG loop body, issued
// through the same public calls, in the same order, as femfunc.cpp:41-111.
int run_iters(const std::string &cfg, const std::string &task, int k) {
  dataKeeper dk(cfg, task);
  const size_t DIM = dk.get_dim(), ne = dk.get_elementsCount();
  const size_t nd = dk.get_nodesCount() * DIM, w = 6 * (DIM - 1);
  double t0 = now_s();
  ElementsData *ed = ElementsData::setElementsData(CPU, dk);
  ed->genMask();
  ed->calculateKlocals();
  ed->get_Klocals()->getDiagonal(w, *ed->get_diagK());
  ed->initFlocals(0.f, dk.getWaveletParams());
  ed->get_Flocals()->copy(*ed->get_r());
  double t1 = now_s();
  Matrix *r = ed->get_r(), *m = ed->get_m(), *z = ed->get_z(), *s = ed->get_s(),
         *p = ed->get_p(), *u = ed->get_u(), *x = ed->get_x();
  ed->reductionWithMaskAndTransform(*ed->get_diagK(), *m, nd);
  r->divideElementwise(*m, *z);
  ed->reductionWithMaskAndTransform(*z, *s, nd);
  float gamma = r->dotProduct(*s);
  s->copy(*p);
  double t2 = now_s();
  double t_mv = 0, t_asm = 0;
  for (int it = 0; it < k; ++it) {
    double a = now_s();
    u->bmm(*p, 1, w, true, *ed->get_Klocals(), w, false, ne);
    double b = now_s();
    float sum = p->dotProduct(*u);
    float alpha = gamma / sum;
    x->addWeighted(*p, 1.f, alpha);
    r->addWeighted(*u, 1.f, -alpha);
    r->divideElementwise(*m, *z);
    double c = now_s();
    ed->reductionWithMaskAndTransform(*z, *s, nd);
    double d = now_s();
    float gamma_new = r->dotProduct(*s);
    p->addWeighted(*s, gamma_new / gamma, 1.f);
    gamma = gamma_new;
    t_mv += b - a;
    t_asm += d - c;
  }
  double t3 = now_s();
  std::printf("{\"setup_s\": %.6f, \"pcg_init_s\": %.6f, \"iters\": %d, \"iter_s\": %.6f, \"matvec_s\": %.6f, "
              "\"assemble_s\": %.6f, \"nodes\": %zu, \"elements\": %zu, \"gamma\": %g}\n",
              t1 - t0, t2 - t1, k, (t3 - t2) / k, t_mv / k, t_asm / k, dk.get_nodesCount(), ne, gamma);
  delete ed;
  return 0;
}

}  // namespace

int main(int argc, char **argv) {
  if (argc < 5) {
    std::fprintf(stderr, "usage: %s static|dyn|dump|vtk|iters <config.json> <task> <out|k>\n", argv[0]);
    return 2;
  }
  std::string mode = argv[1];
  if (mode == "segy" && argc >= 9) {
    // nodes.txt: the prepared-mesh node file (count, then DIM coordinates per line)
    std::ifstream nf(argv[4]);
    size_t n = 0;
    nf >> n;
    const int dim = std::atoi(argv[5]);
    CPU_Matrix nodes(n, dim);
    for (size_t i = 0; i < n; ++i)
      for (int d = 0; d < dim; ++d) nf >> nodes(i, d);
    convert(argv[2], argv[3], (ReceiversType::eType)std::atoi(argv[7]), nodes, std::atoi(argv[6]),
            std::atoi(argv[8]), n);
    std::printf("{\"mode\": \"segy\"}\n");
    return 0;
  }
  if (mode == "static") return run_solve(false, argv[2], argv[3], argv[4]);
  if (mode == "dyn") return run_solve(true, argv[2], argv[3], argv[4]);
  if (mode == "dump") return run_dump(argv[2], argv[3], argv[4]);
  if (mode == "vtk") return run_vtk(argv[2], argv[3], argv[4]);
  if (mode == "iters") return run_iters(argv[2], argv[3], std::atoi(argv[4]));
  std::fprintf(stderr, "unknown mode %s\n", mode.c_str());
  return 2;
}
