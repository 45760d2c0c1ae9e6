// Host-side preparation of a mesh for the sm_103a kernels.
//
// * Locality renumbering: elements sorted by the Morton code of their centroid
//   (isotropic quantisation), cut into fixed-size patches (one CTA each), nodes
//   numbered by first touch in that order. A patch's node set is then "halo"
//   nodes (ids below the patch's first new id) followed by a contiguous range of
//   nodes it owns. The permutations are a deterministic function of the mesh.
// * DOF map, adjacency and constraint decode exactly as the reference:
//   mask = dim*node + d (cpu_fem_utils.cpp:182-213), constrained DOFs from the
//   Constraint::Type bit tests & UX, & UY, & UZ (datakeeper.cpp:139-171,
//   femstruct.h:39-52; note UZ == 3).
// * Right-hand sides in both semantics (cpu_fem_utils.cpp:522-596).
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "../../include/cfem.h"

namespace cfem {

// Edge fans: at most kFanMax tets sharing one edge, evaluated by one thread;
// a patch holds at most kFanThreads fans (one CTA of that many threads).
constexpr int kFanMax = 6;
constexpr int kFanSlots = kFanMax + 4;  // P, Q, R_0..R_kFanMax, length
constexpr int kFanThreads = 128;

struct Prep {
  int dim = 0, nv = 0, w = 0;
  int64_t nn = 0, ne = 0;
  int patch_elems = 0;
  int n_patches = 0;
  int np_max = 0;  // max nodes in one patch
  std::vector<int32_t> elem_new2old, elem_old2new, node_new2old, node_old2new;
  std::vector<int32_t> p_elem_off, p_node_off, p_nodes, p_own;
  std::vector<uint16_t> lconn;     // [ne][4] local node index inside the patch (new element order)
  // Per patch, the transpose of lconn: for every patch-local node the codes
  // le*4 + a of the (patch-local element, vertex) pairs touching it, in
  // increasing order. inc is [ne][4] like lconn (patch p's codes start at
  // 4*elem_off[p]); inc_start holds nn+1 offsets per patch, patch p's at
  // node_off[p] + p.
  std::vector<uint16_t> inc, inc_start;
  // Edge fans (3D, when requested). Elements are numbered fan by fan: fan f
  // holds elements fan_elem_off[f] .. fan_elem_off[f+1]-1, element j of it
  // being {P, Q, R_j, R_j+1}. fan_slot[f][0..kFanMax+2] are the patch-local
  // node indices of P, Q, R_0..R_kFanMax (unused tail repeats the last ring
  // vertex) and fan_slot[f][kFanSlots-1] the fan length. fan_perm[e] packs,
  // two bits per fan vertex b, which vertex of the element's own connectivity
  // it is. finc / finc_start: per patch the incidence lists of the fan slots
  // (codes fl*16 + slot, fl the patch-local fan), laid out like inc / inc_start
  // with patch p's codes starting at kFanSlots*p_fan_off[p].
  bool fans = false;
  int64_t n_fans = 0;
  std::vector<int32_t> fan_elem_off, p_fan_off, fan_ring;
  std::vector<uint8_t> fan_perm;
  std::vector<uint16_t> fan_slot, finc, finc_start;
  std::vector<uint8_t> node_bits;  // [nn] new order: bit d set if DOF d is constrained
  std::vector<uint8_t> dof_bc;     // [nn*dim] original order
  std::vector<int32_t> ctype;      // [nn] original order: last Constraint::Type code or 0
};

// Returns an empty string on success, else the error message.
// elem_group (optional, per element): elements of different groups never share
// a patch and are ordered group by group (independent meshes of a batch).
std::string build_prep(const cfem_mesh &m, int patch_elems, bool use_fans, Prep &out,
                       const int32_t *elem_group = nullptr);

// Wavelet value in the reference's float arithmetic (fem_utils.cpp:53-82).
float wavelet_value(const cfem_wavelet *w, float t);

// Right-hand side pieces in the caller's DOF order (n_nodes*dim, FP64):
// F(t) = a(t) * FA + b(t) * FB. For the reference semantics FA is the face
// load for unit pressure on every face and FB the face load for the file
// pressures (or, with point loads, the nodal loads times the number of
// adjacent elements: calcLoads overwrites every element slot, Q4); for the
// consistent semantics FA is the full load at unit time factor and FB = 0.
struct RhsParts {
  std::vector<double> FA, FB;
  bool has_loads = false;
};
std::string build_rhs(const cfem_mesh &m, const Prep &prep, int semantics, RhsParts &out);

// Time factors (a, b) of the reference's pressure state machine
// (cpu_fem_utils.cpp:564-569): the pressure of every face becomes wavelet(t)
// whenever that value is non-zero and otherwise keeps its previous value.
struct RhsSchedule {
  int semantics = 0;
  bool has_loads = false;
  bool state_is_wavelet = false;
  double state_value = 0;
  const cfem_wavelet *w = nullptr;
  double ampl = 1;
  void reset() { state_is_wavelet = false; state_value = 0; }
  void eval(float t, double &a, double &b);
};

}  // namespace cfem
