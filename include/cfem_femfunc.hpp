// cfem_femfunc.hpp -- C++ mirror of the reference's solver interface on top of
// the C-ABI (include/cfem.h).
//
// Same names and argument meaning as the reference's
//   FEMproject/femfunc/src/femfunc.h:20-24        gpuCalculateFEM_EbE_vec, gpuPCG_EbE_vec,
//                                                 gpuCalculateFEM_DYN, WriteResults
//   FEMproject/DataKeeper/src/datakeeper.h:56-139 dataKeeper (run_config + prepared mesh)
//   FEMproject/VTKfile/src/VTKfile.cpp:281-386    MakeVTKfile2D / MakeVTKfile3D
// so that a caller of the reference switches by changing the include and the
// DEVICE_NAME. Differences in error behaviour: the reference calls exit() on a
// failed assertion or a NaN; this layer throws cfem_ref::Error carrying the
// cfem_status code. Extra run_config keys under "gb300" (ignored by the
// reference) select precision, semantics and stopping rule.
#pragma once

#include <stdexcept>
#include <string>
#include <vector>

#include "cfem.h"

namespace cfem_ref __attribute__((visibility("default"))) {

// The reference's backend switch (matrix_pack_cpu.h:19-23) plus the GB300 path.
// CPU / CUDA / ONEAPI are accepted and run on the GB300 path as well: this
// library has exactly one compute path.
enum DEVICE_NAME { CPU, CUDA, ONEAPI, GB300 };

class Error : public std::runtime_error {
 public:
  Error(cfem_status st, const std::string &what) : std::runtime_error(what), status(st) {}
  cfem_status status;
};

struct MechanicalParams {  // datakeeper.h:21-30
  float poissonRatio = 0.3f, youngModulus = 2e7f, rho = 2400.f;
  float damping_alpha = 0.f, damping_beta = 0.f;
  float dt = 1e-3f, endtime = 0.1f;
  float beta1 = 0.5f, beta2 = 0.f;
};

struct WaveletParams {  // datakeeper.h:32-37
  std::string waveletType = "default";
  float timeshift = 0.f, freq = 15.f, ampl = 1.f;
};

struct dataPaths {  // datakeeper.h:39-53
  std::string proj_dir, prep_mesh_dir, work_dir, res_dir, output_vtk;
  std::string getResDir() { return res_dir; }
};

// Options of this implementation ("gb300" block of run_config).
struct Gb300Options {
  int semantics = CFEM_COMPAT;
  int precision = CFEM_FP32;       // the reference computes in FP32
  int stop_rule = CFEM_STOP_REFERENCE;
  double tol = -1;                 // < 0: the reference's eps (1e-8 static, 1e-4 dynamics)
  double outer_tol = 1e-12;
  int max_iter = 1000000;
  int patch_elems = 0;
};

// Minimal row-major float matrix standing in for the reference's CPU_Matrix
// where callers read results (get_numRows / get_numCols / get_data / (i, j)).
class HostMatrix {
 public:
  HostMatrix() = default;
  HostMatrix(size_t rows, size_t cols) : rows_(rows), cols_(cols), data_(rows * cols, 0.f) {}
  size_t get_numRows() const { return rows_; }
  size_t get_numCols() const { return cols_; }
  size_t get_numElements() const { return data_.size(); }
  float *get_data() { return data_.data(); }
  const float *get_data() const { return data_.data(); }
  float &operator()(size_t i, size_t j) { return data_[j + i * cols_]; }
  float operator()(size_t i, size_t j) const { return data_[j + i * cols_]; }
  float &operator[](size_t i) { return data_[i]; }
  void setTo(float v) { std::fill(data_.begin(), data_.end(), v); }
  // Matrix::copy(Matrix &tgt) (matrix_pack_cpu.h): tgt takes this matrix's shape and values.
  void copy(HostMatrix &tgt) const {
    tgt.rows_ = rows_;
    tgt.cols_ = cols_;
    tgt.data_ = data_;
  }

 private:
  size_t rows_ = 0, cols_ = 0;
  std::vector<float> data_;
};

// run_config JSON + prepared-mesh reader (datakeeper.cpp:6-252).
class dataKeeper {
 public:
  dataKeeper(std::string configPath, std::string taskName);
  ~dataKeeper();
  dataKeeper(const dataKeeper &) = delete;
  dataKeeper &operator=(const dataKeeper &) = delete;

  std::string getTaskName() const { return taskName; }
  std::string getTaskType() const { return taskType; }
  WaveletParams getWaveletParams() const { return waveParams; }
  dataPaths getDataPaths() const { return paths; }
  MechanicalParams getMechParams() const { return mechParams; }
  const Gb300Options &getGb300Options() const { return gb300; }
  Gb300Options &getGb300Options() { return gb300; }

  size_t get_dim() const { return DIM; }
  size_t get_elementsCount() const { return elementsCount; }
  size_t get_nodesCount() const { return nodesCount; }
  size_t get_boundaryEdgesCount() const { return boundaryEdgesCount; }
  size_t get_loadsCount() const { return loadsCount; }
  size_t get_constraintsCount() const { return constraintsCount; }

  const std::vector<double> &get_nodes() const { return nodes; }
  const std::vector<int32_t> &get_elementsIds() const { return elementsIds; }
  HostMatrix *get_displacements() { return &displacements; }
  const std::vector<double> &get_displacements64() const { return displacements64; }
  std::vector<double> &displacements_fp64() { return displacements64; }

  // Lazily created GPU context for this task.
  cfem_ctx *context();
  cfem_mesh mesh_view() const;
  cfem_material material() const;
  cfem_wavelet wavelet() const;
  void ShowInfo() const;

 private:
  void parseJsonConfig(const std::string &path);
  void parseFiles();

  std::string taskName, taskType = "static";
  bool save_segy = false;
  size_t DIM = 0, nodesCount = 0, elementsCount = 0, boundaryEdgesCount = 0, loadsCount = 0, constraintsCount = 0;
  std::vector<double> nodes, loadsVectors, boundaryNormals, boundaryPressures;
  std::vector<int32_t> elementsIds, constraints, loadsNodes, boundaryNodes, boundaryAdjElems;
  HostMatrix displacements;
  std::vector<double> displacements64;
  MechanicalParams mechParams;
  dataPaths paths;
  WaveletParams waveParams;
  Gb300Options gb300;
  cfem_ctx *ctx = nullptr;
};

struct SolveReport {
  cfem_solve_info static_info{};
  cfem_dyn_info dyn_info{};
};

// datakeeper.h:200-226: the options and containers the reference's
// WriteResults receives. The reference's WriteResults writes displacements
// only and ignores them (femfunc.cpp:384-390); so does this one.
class ResultsDataKeeper {
 public:
  ResultsDataKeeper(bool withStressAlongAxis, bool withSmooth, bool withMises, int nodesCount)
      : withStressAlongAxis(withStressAlongAxis), withSmooth(withSmooth), withMises(withMises) {
    (void)nodesCount;
  }
  bool withStressAlongAxis;
  bool withSmooth;
  bool withMises;
  std::vector<HostMatrix> Deformation;
  std::vector<HostMatrix> Stress;
  std::vector<float> sigma_mises;
  std::vector<float> epsilon_mises;
  std::vector<float> StressComponents;
  std::vector<float> MisesComponents;
  std::vector<float> StressComponentsSmooth;
  HostMatrix SmoothStress;
};

// The diagonal of the element operator as the reference reads it with
// Klocals->getDiagonal(6 * (DIM - 1), diagK) (femfunc.cpp:10): here the
// assembled diagonal of K' (n_nodes x DIM), which is what the reference's PCG
// forms from it by assembly (femfunc.cpp:40).
class ElementsData;
class ElementOperator {
 public:
  explicit ElementOperator(ElementsData *ed) : ed_(ed) {}
  void getDiagonal(size_t blockSize, HostMatrix &diag) const;

 private:
  ElementsData *ed_;
};

// fem_utils.h:24-148 (ElementsData), the calls a caller of gpuPCG_EbE_vec makes
// (femfunc.cpp:3-23): the factory, genMask, calculateKlocals, getDiagonal,
// initFlocals and the PCG vectors r and Flocals. The reference keeps those
// vectors element-local (n_elems x 6(DIM-1), their assembly is the global
// vector); this mirror keeps them assembled (n_nodes x DIM, caller node order),
// which is the same right-hand side for the same solve. Like the reference's,
// they are float. Mask, element matrices and geometry live in the GPU context
// of the dataKeeper, built when it is first needed.
class ElementsData {
 public:
  static ElementsData *setElementsData(DEVICE_NAME device, dataKeeper &dk);  // fem_utils.cpp:41-51
  DEVICE_NAME get_device() const { return device_; }
  void genMask() {}           // the DOF map is built with the context
  void calculateKlocals() {}  // likewise the element operator (never stored as 12 x 12 matrices)
  ElementOperator *get_Klocals() { return &klocals_; }
  HostMatrix *get_diagK() { return &diagK_; }
  // cpu_fem_utils.cpp:522-596 at time t with the run_config wavelet: the
  // assembled right-hand side (tractions and point loads) into Flocals.
  void initFlocals(float t, const WaveletParams &w);
  HostMatrix *get_Flocals() { return &Flocals_; }
  HostMatrix *get_r() { return &r_; }
  dataKeeper &keeper() { return dk_; }

 private:
  ElementsData(DEVICE_NAME device, dataKeeper &dk) : device_(device), dk_(dk), klocals_(this) {}
  DEVICE_NAME device_;
  dataKeeper &dk_;
  ElementOperator klocals_;
  HostMatrix diagK_, Flocals_, r_;
};

// femfunc.cpp:3-23: static solve; result in dk.get_displacements().
void gpuCalculateFEM_EbE_vec(DEVICE_NAME deviceType, dataKeeper &FEMdata, bool PRINT_DEBUG_INFO,
                             SolveReport *report = nullptr);
// femfunc.cpp:25-128 in the reference's argument order: Jacobi PCG for
// K' u = r with the right-hand side the caller left in elemsData.get_r()
// (femfunc.cpp:17: Flocals copied into r), stopping factor eps on
// gamma = r.M^-1.r. doAssemblyRes true: displacements becomes n_nodes x DIM
// (femfunc.cpp:100-105); false: the element-local copy x_e = u[mask_e],
// n_elems x 6(DIM-1) (femfunc.cpp:107), as the reference's unassembled x.
void gpuPCG_EbE_vec(HostMatrix &displacements, DEVICE_NAME deviceType, dataKeeper &FEMdata, ElementsData &elemsData,
                    bool doAssemblyRes, float eps, bool PRINT_DEBUG_INFO);
// The same solve for an FP64 right-hand side f (n_nodes * DIM) and an FP64
// result; precision and stopping rule from the run_config "gb300" block.
void gpuPCG_EbE_vec(std::vector<double> &displacements, DEVICE_NAME devType, dataKeeper &FEMdata,
                    const std::vector<double> &rhs, float eps, bool PRINT_DEBUG_INFO, SolveReport *report = nullptr);
// femfunc.cpp:130-381: GN22 dynamics; result in dk.get_displacements().
void gpuCalculateFEM_DYN(DEVICE_NAME devType, dataKeeper &dk, bool PRINT_DEBUG_INFO, SolveReport *report = nullptr);
// femfunc.cpp:384-390 / VTKfile.cpp:281-386: legacy ASCII VTK at dk.getDataPaths().output_vtk.
void WriteResults(dataKeeper &dk, ResultsDataKeeper &RESdata);
void WriteResults(dataKeeper &dk);
// The run_config "task" list (run_fem.py:16-18); a plain string is one task.
std::vector<std::string> readTaskList(const std::string &configPath);
void MakeVTKfile2D(const std::string &output_vtk, const std::vector<double> &nodes, const std::vector<int32_t> &elements,
                   const HostMatrix &displacements);
void MakeVTKfile3D(const std::string &output_vtk, const std::vector<double> &nodes, const std::vector<int32_t> &elements,
                   const HostMatrix &displacements);

}  // namespace cfem_ref
