// femfunc_gb300.h -- the GB300 branch a maintainer of moarseniy/CudaFEMproject
// adds to the reference's own femfunc library.
//
// It reads the task from the reference's dataKeeper
// (FEMproject/DataKeeper/src/datakeeper.h:56-139: float Matrix arrays for nodes,
// elements, constraint DOFs, point loads and boundary faces), widens it into
// the flat arrays of the C-ABI (include/cfem.h), solves on the GPU and writes
// the result back into dk.get_displacements(), exactly where the reference's
// solvers leave it (femfunc.cpp:20, femfunc.cpp:100-111). Wiring, two lines in
// the reference plus an enum value:
//
//   matrix_pack_cpu.h:19-23   enum DEVICE_NAME { CPU, CUDA, ONEAPI, GB300 };
//   femfunc.cpp:3, first line of gpuCalculateFEM_EbE_vec:
//       if (deviceType == GB300) { gb300::calculateFEM_EbE_vec(FEMdata, PRINT_DEBUG_INFO); return; }
//   femfunc.cpp:130, first line of gpuCalculateFEM_DYN:
//       if (devType == GB300) { gb300::calculateFEM_DYN(dk, PRINT_DEBUG_INFO); return; }
//
// and link the femfunc library with -lcfem_gb300. Compiled only against the
// reference's headers (never part of libcfem_gb300.so).
#pragma once

#include <datakeeper.h>

#include <cstdint>
#include <vector>

#include "cfem.h"

namespace gb300 {

// The task of a dataKeeper as C-ABI arrays; `mesh` points into the vectors.
struct TaskArrays {
  std::vector<double> nodes, load_vectors, face_normals, face_pressures;
  std::vector<int32_t> elems, constraints, load_nodes, face_nodes, face_elems;
  cfem_mesh mesh{};
  cfem_material material{};
};

// Widens every array of the task: node coordinates, connectivity, constraint
// codes (rebuilt per node from the decoded DOF list, datakeeper.cpp:139-171, so
// that the library's decode gives the same DOFs), point loads
// (datakeeper.cpp:173-185) and boundary faces with their normals and
// pressures (datakeeper.cpp:187-213).
TaskArrays widen(const dataKeeper &dk);

// run_config wavelet block (datakeeper.cpp:36-47) for cfem_rhs / cfem_dyn.
cfem_wavelet wavelet(const WaveletParams &w);

// gpuCalculateFEM_EbE_vec on the GPU: compat semantics, FP32 PCG with the
// reference's stopping rule gamma < 1e-8 gamma0 (femfunc.cpp:20). Throws
// std::runtime_error with cfem_last_error_string() on failure.
void calculateFEM_EbE_vec(dataKeeper &dk, bool verbose);

// gpuCalculateFEM_DYN on the GPU (GN22 with the run_config's beta1, beta2, dt,
// endtime; implicit PCG to gamma < 1e-4 gamma0 as femfunc.cpp:302).
void calculateFEM_DYN(dataKeeper &dk, bool verbose);

}  // namespace gb300
