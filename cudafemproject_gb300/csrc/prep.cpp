// Host-side mesh preparation; see prep.hpp.
#include "prep.hpp"

#include <array>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>

namespace cfem {

namespace {

inline uint64_t spread3(uint64_t v) {  // 21 bits -> every third bit
  v &= 0x1fffff;
  v = (v | v << 32) & 0x1f00000000ffffULL;
  v = (v | v << 16) & 0x1f0000ff0000ffULL;
  v = (v | v << 8) & 0x100f00f00f00f00fULL;
  v = (v | v << 4) & 0x10c30c30c30c30c3ULL;
  v = (v | v << 2) & 0x1249249249249249ULL;
  return v;
}

inline uint64_t spread2(uint64_t v) {  // 32 bits -> every second bit
  v &= 0xffffffffULL;
  v = (v | v << 16) & 0x0000ffff0000ffffULL;
  v = (v | v << 8) & 0x00ff00ff00ff00ffULL;
  v = (v | v << 4) & 0x0f0f0f0f0f0f0f0fULL;
  v = (v | v << 2) & 0x3333333333333333ULL;
  v = (v | v << 1) & 0x5555555555555555ULL;
  return v;
}

}  // namespace

std::string build_prep(const cfem_mesh &m, int patch_elems, bool use_fans, Prep &P, const int32_t *elem_group) {
  const int dim = m.dim;
  if (dim != 2 && dim != 3) return "dim must be 2 or 3";
  if (m.n_nodes <= 0 || m.n_elems <= 0) return "mesh has no nodes or no elements";
  if (m.n_nodes > (int64_t)INT32_MAX / 4 || m.n_elems > (int64_t)INT32_MAX / 12) return "mesh too large for int32 DOF ids";
  const int nv = dim + 1;
  P.dim = dim; P.nv = nv; P.w = 6 * (dim - 1);
  P.nn = m.n_nodes; P.ne = m.n_elems;
  P.patch_elems = patch_elems;
  const int64_t nn = m.n_nodes, ne = m.n_elems;
  std::vector<int32_t> used(nn, 0);
  for (int64_t i = 0; i < ne * nv; ++i) {
    int32_t v = m.elems[i];
    if (v < 0 || v >= nn) return "element " + std::to_string(i / nv) + " references node " + std::to_string(v) + " out of range";
    used[v] = 1;
  }
  for (int64_t i = 0; i < nn; ++i)
    if (!used[i])
      return "node " + std::to_string(i) + " belongs to no element (the reference compacts DOF ids, so every node must be used)";
  for (int64_t e = 0; e < ne; ++e)
    for (int a = 0; a < nv; ++a)
      for (int b = a + 1; b < nv; ++b)
        if (m.elems[e * nv + a] == m.elems[e * nv + b]) return "element " + std::to_string(e) + " repeats a node";

  // ---- Morton order of element centroids (isotropic quantisation) ----
  double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
  for (int64_t i = 0; i < nn; ++i)
    for (int d = 0; d < dim; ++d) {
      double x = m.nodes[i * dim + d];
      if (!std::isfinite(x)) return "node " + std::to_string(i) + " has a non-finite coordinate";
      lo[d] = std::min(lo[d], x); hi[d] = std::max(hi[d], x);
    }
  double ext = 0;
  for (int d = 0; d < dim; ++d) ext = std::max(ext, hi[d] - lo[d]);
  if (ext <= 0) ext = 1;
  const double qmax = dim == 3 ? 2097151.0 : 4294967295.0;
  std::vector<std::pair<uint64_t, int32_t>> key(ne);
  for (int64_t e = 0; e < ne; ++e) {
    double c[3] = {0, 0, 0};
    for (int a = 0; a < nv; ++a)
      for (int d = 0; d < dim; ++d) c[d] += m.nodes[(int64_t)m.elems[e * nv + a] * dim + d];
    uint64_t q[3] = {0, 0, 0};
    for (int d = 0; d < dim; ++d) {
      double t = (c[d] / nv - lo[d]) / ext;
      t = std::min(std::max(t, 0.0), 1.0);
      q[d] = (uint64_t)(t * qmax);
    }
    uint64_t k = dim == 3 ? (spread3(q[0]) | spread3(q[1]) << 1 | spread3(q[2]) << 2) : (spread2(q[0]) | spread2(q[1]) << 1);
    key[e] = {k, (int32_t)e};
  }
  std::sort(key.begin(), key.end());
  // independent meshes of a batch stay apart: group first, locality order inside a group
  if (elem_group)
    std::stable_sort(key.begin(), key.end(), [&](const std::pair<uint64_t, int32_t> &a,
                                                 const std::pair<uint64_t, int32_t> &b) {
      return elem_group[a.second] < elem_group[b.second];
    });
  P.elem_new2old.resize(ne);
  P.elem_old2new.resize(ne);
  for (int64_t i = 0; i < ne; ++i) {
    P.elem_new2old[i] = key[i].second;
    P.elem_old2new[key[i].second] = (int32_t)i;
  }
  key.clear();
  key.shrink_to_fit();

  // ---- edge fans (3D): chains of up to kFanMax tets around one edge ----
  // Greedy in locality order: the seed tet takes the edge of its own with the
  // most unassigned tets around it, and the unassigned tets around that edge
  // are chained through their shared faces, starting from the seed. Tet j of a
  // fan is {P, Q, R_j, R_j+1}; a closed ring has R_len == R_0. Without fans
  // every element is its own fan of length 1.
  const int pe = patch_elems;
  P.fan_elem_off.clear();
  P.fan_ring.clear();
  P.fan_perm.assign(ne, 0);
  if (use_fans && dim == 3) {
    // node -> tets (counting sort)
    std::vector<int32_t> nt_off(nn + 1, 0), nt(ne * 4);
    for (int64_t i = 0; i < ne * 4; ++i) ++nt_off[m.elems[i] + 1];
    for (int64_t i = 0; i < nn; ++i) nt_off[i + 1] += nt_off[i];
    {
      std::vector<int32_t> pos(nt_off.begin(), nt_off.end() - 1);
      for (int64_t e = 0; e < ne; ++e)
        for (int a = 0; a < 4; ++a) nt[pos[m.elems[e * 4 + a]]++] = (int32_t)e;
    }
    std::vector<uint8_t> taken(ne, 0);
    std::vector<int32_t> order;
    order.reserve(ne);
    P.fan_elem_off.push_back(0);
    static const int kEdge[6][2] = {{0, 1}, {0, 2}, {0, 3}, {1, 2}, {1, 3}, {2, 3}};
    std::vector<int32_t> around, best, chain;
    for (int64_t i = 0; i < ne; ++i) {
      const int32_t t = P.elem_new2old[i];
      if (taken[t]) continue;
      const int32_t *vt = m.elems + (int64_t)t * 4;
      int best_k = 0;
      best.clear();
      for (int k = 0; k < 6; ++k) {
        const int32_t p = vt[kEdge[k][0]], q = vt[kEdge[k][1]];
        around.clear();
        for (int32_t j = nt_off[p]; j < nt_off[p + 1]; ++j) {
          const int32_t s = nt[j];
          if (taken[s]) continue;
          const int32_t *vs = m.elems + (int64_t)s * 4;
          if (vs[0] == q || vs[1] == q || vs[2] == q || vs[3] == q) around.push_back(s);
        }
        if (around.size() > best.size()) { best = around; best_k = k; }
      }
      const int32_t p = vt[kEdge[best_k][0]], q = vt[kEdge[best_k][1]];
      auto others = [&](int32_t s, int32_t &x, int32_t &y) {
        const int32_t *vs = m.elems + (int64_t)s * 4;
        x = -1; y = -1;
        for (int a = 0; a < 4; ++a)
          if (vs[a] != p && vs[a] != q) { if (x < 0) x = vs[a]; else y = vs[a]; }
      };
      auto in_chain = [&](int32_t s) { return std::find(chain.begin(), chain.end(), s) != chain.end(); };
      chain.assign(1, t);
      int32_t left, right;
      others(t, left, right);
      bool closed = false;
      // extend through R_right, then (if still open) backwards through R_left
      while ((int)chain.size() < kFanMax && !closed) {
        int32_t next = -1, nv2 = -1;
        for (int32_t s : best) {
          if (in_chain(s)) continue;
          int32_t x, y;
          others(s, x, y);
          if (x == right) { next = s; nv2 = y; break; }
          if (y == right) { next = s; nv2 = x; break; }
        }
        if (next < 0) break;
        chain.push_back(next);
        right = nv2;
        if (right == left) closed = true;
      }
      while ((int)chain.size() < kFanMax && !closed) {
        int32_t prev = -1, nv2 = -1;
        for (int32_t s : best) {
          if (in_chain(s)) continue;
          int32_t x, y;
          others(s, x, y);
          if (x == left) { prev = s; nv2 = y; break; }
          if (y == left) { prev = s; nv2 = x; break; }
        }
        if (prev < 0) break;
        chain.insert(chain.begin(), prev);
        left = nv2;
      }
      // ring vertices R_0..R_len: walk the chain from the left end
      const int len = (int)chain.size();
      std::array<int32_t, kFanMax + 3> ring{};
      ring[0] = p;
      ring[1] = q;
      int32_t cur = left;
      for (int j = 0; j < len; ++j) {
        int32_t x, y;
        others(chain[j], x, y);
        ring[2 + j] = cur;
        cur = x == cur ? y : x;
      }
      ring[2 + len] = cur;
      for (int j = 0; j < len; ++j) {
        const int32_t s = chain[j];
        taken[s] = 1;
        const int32_t *vs = m.elems + (int64_t)s * 4;
        const int32_t fv[4] = {p, q, ring[2 + j], ring[3 + j]};
        uint8_t perm = 0;
        for (int bb = 0; bb < 4; ++bb) {
          int a = 0;
          while (a < 4 && vs[a] != fv[bb]) ++a;
          if (a == 4) return "internal error: edge fan does not match its tets";
          perm |= (uint8_t)(a << (2 * bb));
        }
        P.fan_perm[s] = perm;  // indexed by old id here, permuted to the new order below
        order.push_back(s);
      }
      for (int k = 0; k < kFanMax + 3; ++k) P.fan_ring.push_back(k < len + 3 ? ring[k] : ring[2 + len]);
      P.fan_elem_off.push_back((int32_t)order.size());
    }
    std::vector<uint8_t> perm_new(ne);
    for (int64_t i = 0; i < ne; ++i) {
      P.elem_new2old[i] = order[i];
      P.elem_old2new[order[i]] = (int32_t)i;
      perm_new[i] = P.fan_perm[order[i]];
    }
    P.fan_perm.swap(perm_new);
  } else {
    P.fan_elem_off.resize(ne + 1);
    for (int64_t i = 0; i <= ne; ++i) P.fan_elem_off[i] = (int32_t)i;
  }
  P.n_fans = (int64_t)P.fan_elem_off.size() - 1;
  P.fans = use_fans && dim == 3;
  // ---- patches: consecutive fans, at most patch_elems elements and kFanThreads fans each ----
  P.p_elem_off.clear();
  P.p_fan_off.clear();
  {
    int64_t f = 0;
    while (f < P.n_fans) {
      P.p_fan_off.push_back((int32_t)f);
      P.p_elem_off.push_back(P.fan_elem_off[f]);
      int64_t f1 = f;
      auto group_of = [&](int64_t fan) { return elem_group ? elem_group[P.elem_new2old[P.fan_elem_off[fan]]] : 0; };
      while (f1 < P.n_fans && (f1 - f) < (P.fans ? kFanThreads : pe) &&
             P.fan_elem_off[f1 + 1] - P.fan_elem_off[f] <= pe && group_of(f1) == group_of(f))
        ++f1;
      f = f1;
    }
    P.n_patches = (int)P.p_fan_off.size();
    P.p_fan_off.push_back((int32_t)P.n_fans);
    P.p_elem_off.push_back((int32_t)ne);
  }
  P.node_old2new.assign(nn, -1);
  P.node_new2old.resize(nn);
  int32_t next = 0;
  std::vector<int32_t> first_new(P.n_patches + 1, 0);
  for (int p = 0; p < P.n_patches; ++p) {
    first_new[p] = next;
    for (int64_t ei = P.p_elem_off[p]; ei < P.p_elem_off[p + 1]; ++ei) {
      int64_t e = P.elem_new2old[ei];
      for (int a = 0; a < nv; ++a) {
        int32_t o = m.elems[e * nv + a];
        if (P.node_old2new[o] < 0) {
          P.node_old2new[o] = next;
          P.node_new2old[next] = o;
          ++next;
        }
      }
    }
  }
  first_new[P.n_patches] = next;
  P.p_node_off.resize(P.n_patches + 1);
  P.p_own.resize(P.n_patches);
  P.p_nodes.clear();
  P.p_nodes.reserve((size_t)(nn * 1.6) + 16);
  P.lconn.assign(ne * 4, 0);
  if (P.fans) {
    P.fan_slot.assign(P.n_fans * kFanSlots, 0);
    for (int64_t f = 0; f < P.n_fans; ++f)
      P.fan_slot[f * kFanSlots + kFanSlots - 1] = (uint16_t)(P.fan_elem_off[f + 1] - P.fan_elem_off[f]);
  }
  std::vector<int32_t> mark(nn, -1), loc(nn, 0);
  std::vector<int32_t> list;
  P.np_max = 0;
  for (int p = 0; p < P.n_patches; ++p) {
    const int64_t e0 = P.p_elem_off[p], e1 = P.p_elem_off[p + 1];
    list.clear();
    for (int64_t ei = e0; ei < e1; ++ei) {
      int64_t e = P.elem_new2old[ei];
      for (int a = 0; a < nv; ++a) {
        int32_t g = P.node_old2new[m.elems[e * nv + a]];
        if (mark[g] != p) { mark[g] = p; list.push_back(g); }
      }
    }
    std::sort(list.begin(), list.end());
    if (list.size() > 65535) return "patch has more than 65535 nodes";
    P.p_node_off[p] = (int32_t)P.p_nodes.size();
    int own = (int)(std::lower_bound(list.begin(), list.end(), first_new[p]) - list.begin());
    P.p_own[p] = own;
    for (size_t i = 0; i < list.size(); ++i) { loc[list[i]] = (int32_t)i; P.p_nodes.push_back(list[i]); }
    P.np_max = std::max<int>(P.np_max, (int)list.size());
    for (int64_t ei = e0; ei < e1; ++ei) {
      int64_t e = P.elem_new2old[ei];
      for (int a = 0; a < nv; ++a) P.lconn[ei * 4 + a] = (uint16_t)loc[P.node_old2new[m.elems[e * nv + a]]];
    }
    if (P.fans)
      for (int64_t f = P.p_fan_off[p]; f < P.p_fan_off[p + 1]; ++f)
        for (int k = 0; k < kFanMax + 3; ++k)
          P.fan_slot[f * kFanSlots + k] = (uint16_t)loc[P.node_old2new[P.fan_ring[f * (kFanMax + 3) + k]]];
  }
  P.p_node_off[P.n_patches] = (int32_t)P.p_nodes.size();
  // ---- incidence lists (counting sort of each patch's (element, vertex) pairs by node) ----
  P.inc.assign(ne * 4, 0);
  P.inc_start.assign(P.p_nodes.size() + P.n_patches, 0);
  {
    std::vector<int32_t> pos;
    for (int p = 0; p < P.n_patches; ++p) {
      const int64_t e0 = P.p_elem_off[p], e1 = P.p_elem_off[p + 1];
      const int n = P.p_node_off[p + 1] - P.p_node_off[p];
      pos.assign(n + 1, 0);
      for (int64_t ei = e0; ei < e1; ++ei)
        for (int a = 0; a < nv; ++a) ++pos[P.lconn[ei * 4 + a] + 1];
      for (int i = 0; i < n; ++i) pos[i + 1] += pos[i];
      uint16_t *st = P.inc_start.data() + P.p_node_off[p] + p;
      for (int i = 0; i <= n; ++i) st[i] = (uint16_t)pos[i];
      for (int64_t ei = e0; ei < e1; ++ei)
        for (int a = 0; a < nv; ++a) P.inc[e0 * 4 + pos[P.lconn[ei * 4 + a]]++] = (uint16_t)((ei - e0) * 4 + a);
    }
  }
  // ---- fan incidence lists: codes fl*16 + slot (slot 0 = P, 1 = Q, 2 + k = R_k) ----
  if (P.fans) {
    P.finc.assign(P.n_fans * kFanSlots, 0);
    P.finc_start.assign(P.p_nodes.size() + P.n_patches, 0);
    std::vector<int32_t> pos;
    for (int p = 0; p < P.n_patches; ++p) {
      const int64_t f0 = P.p_fan_off[p], f1 = P.p_fan_off[p + 1];
      const int n = P.p_node_off[p + 1] - P.p_node_off[p];
      pos.assign(n + 1, 0);
      for (int64_t f = f0; f < f1; ++f) {
        const int len = P.fan_slot[f * kFanSlots + kFanSlots - 1];
        for (int k = 0; k < len + 3; ++k) ++pos[P.fan_slot[f * kFanSlots + k] + 1];
      }
      for (int i = 0; i < n; ++i) pos[i + 1] += pos[i];
      uint16_t *st = P.finc_start.data() + P.p_node_off[p] + p;
      for (int i = 0; i <= n; ++i) st[i] = (uint16_t)pos[i];
      for (int64_t f = f0; f < f1; ++f) {
        const int len = P.fan_slot[f * kFanSlots + kFanSlots - 1];
        for (int k = 0; k < len + 3; ++k)
          P.finc[f0 * kFanSlots + pos[P.fan_slot[f * kFanSlots + k]]++] = (uint16_t)((f - f0) * 16 + k);
      }
    }
  }

  // ---- constraints (datakeeper.cpp:139-171) ----
  P.dof_bc.assign(nn * dim, 0);
  P.ctype.assign(nn, 0);
  for (int64_t i = 0; i < m.n_constraints; ++i) {
    int32_t node = m.constraints[2 * i], type = m.constraints[2 * i + 1];
    if (node < 0 || node >= nn) return "constraint " + std::to_string(i) + " names node " + std::to_string(node) + " out of range";
    P.ctype[node] = type;
    if (type & 1) P.dof_bc[(int64_t)dim * node + 0] = 1;
    if (type & 2) P.dof_bc[(int64_t)dim * node + 1] = 1;
    if (dim == 3 && (type & 3)) P.dof_bc[(int64_t)dim * node + 2] = 1;
  }
  P.node_bits.assign(nn, 0);
  for (int64_t o = 0; o < nn; ++o) {
    uint8_t b = 0;
    for (int d = 0; d < dim; ++d)
      if (P.dof_bc[o * dim + d]) b |= (uint8_t)(1u << d);
    P.node_bits[P.node_old2new[o]] = b;
  }
  return "";
}

float wavelet_value(const cfem_wavelet *w, float t) {
  if (!w) return 0.f;
  const float ts = (float)w->timeshift;
  if (t < ts) return 0.f;
  const float ampl = (float)w->ampl, freq = (float)w->freq;
  t = t - ts;
  if (w->type == CFEM_WAVELET_RICKER) {
    float tmp = (float)(M_PI * freq * t - M_PI);
    return ampl * (1.f - 2.f * tmp * tmp) * std::exp(-1.f * tmp * tmp);
  }
  if (w->type == CFEM_WAVELET_BERLAGE) {
    float w0 = (float)(2 * M_PI * freq);
    float w1 = w0 / std::sqrt(3.f);
    return ampl * w1 * w1 / 4.f * std::exp(-1.f * w1 * t) *
           (std::sin(w0 * t) * (1.f / (w1 * w1 * w1) + t / (w1 * w1) - t * t / w1) -
            std::cos(w0 * t) * std::sqrt(3.f) * (t * t / w1 + t / (w1 * w1)));
  }
  return 0.f;
}

void RhsSchedule::eval(float t, double &a, double &b) {
  if (semantics == CFEM_CONSISTENT) {
    if (!w || w->type == CFEM_WAVELET_NONE) { a = 1; b = 0; return; }
    a = w->ampl != 0 ? (double)wavelet_value(w, t) / w->ampl : 0.0;
    b = 0;
    return;
  }
  float v = wavelet_value(w, t);
  if (v != 0.f) { state_is_wavelet = true; state_value = v; }
  if (has_loads) { a = 0; b = 1; return; }  // calcLoads overwrites every slot
  if (state_is_wavelet) { a = state_value; b = 0; } else { a = 0; b = 1; }
}

std::string build_rhs(const cfem_mesh &m, const Prep &P, int semantics, RhsParts &out) {
  const int dim = m.dim, nv = dim + 1, w = 6 * (dim - 1);
  const int64_t nd = m.n_nodes * dim;
  out.FA.assign(nd, 0.0);
  out.FB.assign(nd, 0.0);
  out.has_loads = m.n_loads > 0;
  // normalised face normals and face measures (datakeeper.cpp:201-209, cpu_fem_utils.cpp:247-272)
  std::vector<double> nrm(m.n_faces * dim), flen(m.n_faces), fmeas(m.n_faces);
  for (int64_t f = 0; f < m.n_faces; ++f) {
    double l2 = 0;
    for (int j = 0; j < dim; ++j) l2 += m.face_normals[f * dim + j] * m.face_normals[f * dim + j];
    if (!(l2 > 0)) return "face " + std::to_string(f) + " has a zero normal";
    for (int j = 0; j < dim; ++j) nrm[f * dim + j] = m.face_normals[f * dim + j] / std::sqrt(l2);
    for (int i = 0; i < nv; ++i) {
      int32_t v = m.face_nodes[f * nv + i];
      if (v < 0 || v >= m.n_nodes) return "face " + std::to_string(f) + " names node out of range";
    }
    if (m.face_elems[f] < 0 || m.face_elems[f] >= m.n_elems) return "face " + std::to_string(f) + " names element out of range";
    const double *a = m.nodes + (int64_t)m.face_nodes[f * nv + 0] * dim;
    const double *b = m.nodes + (int64_t)m.face_nodes[f * nv + 1] * dim;
    if (dim == 2) {
      double L = std::sqrt((b[0] - a[0]) * (b[0] - a[0]) + (b[1] - a[1]) * (b[1] - a[1]));
      flen[f] = L;          // reference measure
      fmeas[f] = 0.5 * L;   // consistent: t*L/2 per node
    } else {
      const double *c = m.nodes + (int64_t)m.face_nodes[f * nv + 2] * dim;
      double ax = b[0] - a[0], ay = b[1] - a[1], az = b[2] - a[2];
      double bx = c[0] - a[0], by = c[1] - a[1], bz = c[2] - a[2];
      double c1 = ay * bz - az * by, c2 = az * bx - ax * bz, c3 = ax * by - ay * bx;
      double cr2 = c1 * c1 + c2 * c2 + c3 * c3;
      flen[f] = 0.5 * cr2;                   // reference: 0.5*|a x b|^2 (no square root)
      fmeas[f] = 0.5 * std::sqrt(cr2) / 3.0;  // consistent: t*A/3 per node
    }
  }
  if (semantics == CFEM_COMPAT) {
    if (out.has_loads) {
      // calcLoads: nodal load array (last entry wins) gathered into every element
      // slot, then assembled: each DOF gets load * (number of adjacent elements).
      std::vector<double> loads(nd, 0.0);
      std::vector<int32_t> adj(m.n_nodes, 0);
      for (int64_t i = 0; i < m.n_elems * nv; ++i) adj[m.elems[i]]++;
      for (int64_t l = 0; l < m.n_loads; ++l) {
        int32_t node = m.load_nodes[l];
        if (node < 0 || node >= m.n_nodes) return "load " + std::to_string(l) + " names node out of range";
        for (int d = 0; d < dim; ++d) loads[(int64_t)dim * node + d] = m.load_vectors[l * dim + d];
      }
      for (int64_t k = 0; k < nd; ++k) out.FB[k] = loads[k] * adj[k / dim];
      return "";
    }
    // calcPressures: each face writes (not adds) coeff*p*L*n_j into the element
    // slot of its nodes; the last face to write a slot wins. Q5: component j is
    // zeroed when (constraint code of the node) & j.
    const double coeff = dim == 2 ? -0.5 : -1.0 / 12.0;
    std::vector<double> slotA((size_t)m.n_elems * w, 0.0), slotB((size_t)m.n_elems * w, 0.0);
    std::vector<uint8_t> touched((size_t)m.n_elems * w, 0);
    for (int64_t f = 0; f < m.n_faces; ++f) {
      int64_t e = m.face_elems[f];
      for (int i = 0; i < dim; ++i) {
        int32_t node = m.face_nodes[f * nv + i];
        int loc = -1;
        for (int a = 0; a < nv; ++a)
          if (m.elems[e * nv + a] == node) { loc = a; break; }
        if (loc < 0) continue;  // reference prints "Wrong index" and writes out of range; skipped here
        for (int j = 0; j < dim; ++j) {
          bool masked = (P.ctype[node] & j) != 0;
          size_t s = (size_t)e * w + dim * loc + j;
          slotA[s] = masked ? 0.0 : coeff * 1.0 * flen[f] * nrm[f * dim + j];
          slotB[s] = masked ? 0.0 : coeff * m.face_pressures[f] * flen[f] * nrm[f * dim + j];
          touched[s] = 1;
        }
      }
    }
    for (int64_t e = 0; e < m.n_elems; ++e)
      for (int a = 0; a < nv; ++a)
        for (int j = 0; j < dim; ++j) {
          size_t s = (size_t)e * w + dim * a + j;
          if (!touched[s]) continue;
          int64_t dof = (int64_t)dim * m.elems[e * nv + a] + j;
          out.FA[dof] += slotA[s];
          out.FB[dof] += slotB[s];
        }
    return "";
  }
  // consistent: accumulate t*L/2 (2D) or t*A/3 (3D) per face node plus point
  // loads once; constrained DOFs get no load.
  for (int64_t f = 0; f < m.n_faces; ++f)
    for (int i = 0; i < dim; ++i) {
      int32_t node = m.face_nodes[f * nv + i];
      for (int j = 0; j < dim; ++j)
        out.FA[(int64_t)dim * node + j] += -m.face_pressures[f] * fmeas[f] * nrm[f * dim + j];
    }
  for (int64_t l = 0; l < m.n_loads; ++l) {
    int32_t node = m.load_nodes[l];
    if (node < 0 || node >= m.n_nodes) return "load " + std::to_string(l) + " names node out of range";
    for (int d = 0; d < dim; ++d) out.FA[(int64_t)dim * node + d] += m.load_vectors[l * dim + d];
  }
  for (int64_t k = 0; k < nd; ++k)
    if (P.dof_bc[k]) out.FA[k] = 0;
  return "";
}

}  // namespace cfem
