// LS-DYNA keyword (.k) meshes -> prepared-mesh arrays, host code.
//
// Reads a keyword file the way the reference's converter does
// (mesh_parser_lib/parser_src/parser_lib.py:36-378, driven by
// mesh_parser_lib/fem_parser.py), with the same rules as
// cudafemproject_gb300/kfile.py:
//   *NODE              the line after the keyword is skipped; "nid x y [z]" lines up to a "$" line
//   *ELEMENT_SOLID/SHELL "eid pid n1 n2 ..." lines; the first dim + 1 nodes after eid, pid
//   *SET_NODE_LIST     the next line (stripped) is the set key; node ids follow
//   *BOUNDARY_SPC_SET  "sid cid dofx dofy [dofz]": constraint code of the flags for every node of set sid
//   *DEFINE_CURVE      the next line is the key; the value is the second number of the last data line
//   *LOAD_NODE_SET     "sid dof lcid": the first card whose set exists loads every node of the set
//   *LOAD_SEGMENT      "lcid sf at n1 n2 [n3 n4]": face of the first element (file order) holding it,
//                      normal (y2-y1, -(x2-x1)) / (p2-p1) x (p3-p1) turned away from the remaining node
// Node ids are matched as text, as the reference's converter does. One pass
// over the file and hash maps keep it linear in the file size (the reference's
// face search scans all elements per face).
#include <algorithm>
#include <cctype>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <fstream>
#include <functional>
#include <map>
#include <stdexcept>
#include <string>
#include <unordered_map>
#include <vector>

#include "cfem.h"

namespace cfem {
namespace detail {
extern thread_local std::string g_last_error;
}
}  // namespace cfem

struct cfem_kfile {
  int dim = 3;
  std::vector<double> nodes;  // [n][dim]
  std::vector<int32_t> elems;  // [e][dim + 1]
  std::vector<int32_t> cons;   // [c][2] node, constraint code
  std::vector<int32_t> load_node;
  std::vector<double> load_vec;  // [l][dim]
  std::vector<int32_t> face_nodes;  // [f][dim + 1]: face nodes, then the element's remaining node
  std::vector<int32_t> face_elem;
  std::vector<double> face_normal;  // [f][dim]
  std::vector<double> face_pressure;
};

namespace {

struct KError : std::runtime_error {
  cfem_status st;
  KError(cfem_status s, const std::string &m) : std::runtime_error(m), st(s) {}
};

std::vector<std::string> split_ws(const std::string &s) {
  std::vector<std::string> out;
  size_t i = 0, n = s.size();
  while (i < n) {
    while (i < n && std::isspace((unsigned char)s[i])) ++i;
    size_t j = i;
    while (j < n && !std::isspace((unsigned char)s[j])) ++j;
    if (j > i) out.emplace_back(s, i, j - i);
    i = j;
  }
  return out;
}

std::string strip(const std::string &s) {
  size_t a = 0, b = s.size();
  while (a < b && std::isspace((unsigned char)s[a])) ++a;
  while (b > a && std::isspace((unsigned char)s[b - 1])) --b;
  return s.substr(a, b - a);
}

bool blank(const std::string &s) { return strip(s).empty(); }
bool comment(const std::string &s) {
  const std::string t = strip(s);
  return !t.empty() && t[0] == '$';
}

double to_double(const std::string &t) {
  size_t used = 0;
  const double v = std::stod(t, &used);
  if (used != t.size()) throw KError(CFEM_ERR_MESH, "not a number: '" + t + "'");
  return v;
}

int to_int(const std::string &t) {
  size_t used = 0;
  const long long v = std::stoll(t, &used);
  if (used != t.size()) throw KError(CFEM_ERR_MESH, "not an integer: '" + t + "'");
  return (int)v;
}

void read_k(const char *path, int dim, cfem_kfile &K) {
  if (dim != 2 && dim != 3) throw KError(CFEM_ERR_INVALID_ARGUMENT, "dim must be 2 or 3");
  std::ifstream in(path);
  if (!in) throw KError(CFEM_ERR_IO, std::string("cannot open ") + path);
  K.dim = dim;
  // blocks: keyword and its lines, in file order
  std::vector<std::pair<std::string, std::vector<std::string>>> blocks;
  std::string line;
  while (std::getline(in, line)) {
    if (!line.empty() && line.back() == '\r') line.pop_back();
    if (!line.empty() && line[0] == '*') blocks.emplace_back(strip(line), std::vector<std::string>{});
    else if (!blocks.empty()) blocks.back().second.push_back(line);
  }
  std::vector<std::string> node_ids;
  std::vector<double> coords;
  std::vector<std::vector<std::string>> elems_raw;
  std::vector<std::string> set_order;  // keys in first-definition order
  std::unordered_map<std::string, std::vector<std::string>> sets;
  std::vector<std::vector<std::string>> spcs, node_loads, segments;
  std::unordered_map<std::string, std::string> curves;
  for (auto &blk : blocks) {
    const std::string &kw = blk.first;
    std::vector<std::string> data;
    for (auto &l : blk.second)
      if (!blank(l) && !comment(l)) data.push_back(l);
    if (kw == "*NODE") {
      for (size_t i = 1; i < blk.second.size(); ++i) {
        const std::string &l = blk.second[i];
        if (strip(l) == "$") break;
        if (comment(l) || blank(l)) continue;
        const auto tok = split_ws(l);
        if ((int)tok.size() < dim + 1) throw KError(CFEM_ERR_MESH, "short *NODE line: '" + l + "'");
        node_ids.push_back(tok[0]);
        for (int d = 0; d < dim; ++d) coords.push_back(to_double(tok[1 + d]));
      }
    } else if (kw == "*ELEMENT_SOLID" || kw == "*ELEMENT_SHELL") {
      for (auto &l : data) {
        const auto tok = split_ws(l);
        std::vector<std::string> e;
        for (int a = 2; a < 2 + dim + 1 && a < (int)tok.size(); ++a) e.push_back(tok[a]);
        elems_raw.push_back(e);
      }
    } else if (kw == "*SET_NODE_LIST" && !data.empty()) {
      const std::string key = strip(data[0]);
      std::vector<std::string> members;
      for (size_t i = 1; i < data.size(); ++i)
        for (auto &t : split_ws(data[i])) members.push_back(t);
      if (!sets.count(key)) set_order.push_back(key);
      sets[key] = members;
    } else if (kw == "*BOUNDARY_SPC_SET" && !data.empty()) {
      spcs.push_back(split_ws(data[0]));
    } else if (kw == "*DEFINE_CURVE" && !data.empty()) {
      if (data.size() > 1) {
        const auto tok = split_ws(data.back());
        if (tok.size() < 2) throw KError(CFEM_ERR_MESH, "*DEFINE_CURVE data line without a value");
        curves[strip(data[0])] = tok[1];
      }
    } else if (kw == "*LOAD_NODE_SET" && !data.empty()) {
      node_loads.push_back(split_ws(data[0]));
    } else if (kw == "*LOAD_SEGMENT" && !data.empty()) {
      segments.push_back(split_ws(data[0]));
    }
  }
  std::unordered_map<std::string, int32_t> index;
  index.reserve(node_ids.size() * 2);
  for (size_t i = 0; i < node_ids.size(); ++i) index[node_ids[i]] = (int32_t)i;  // a repeated id: the last one
  auto node_of = [&](const std::string &t) {
    auto it = index.find(t);
    if (it == index.end()) throw KError(CFEM_ERR_MESH, "unknown node id '" + t + "'");
    return it->second;
  };
  K.nodes = coords;
  const int nv = dim + 1;
  K.elems.reserve(elems_raw.size() * nv);
  for (auto &e : elems_raw) {
    if ((int)e.size() != nv) throw KError(CFEM_ERR_MESH, "element with fewer than dim + 1 nodes");
    for (auto &t : e) K.elems.push_back(node_of(t));
  }
  // constraints: code of the flags (femstruct.h:39-52)
  auto code_of = [&](const std::vector<int> &f) -> int {
    if (dim == 2) {
      if (f[0] && !f[1]) return 1;
      if (!f[0] && f[1]) return 2;
      if (f[0] && f[1]) return 3;
      return 0;
    }
    const int m = (f[0] ? 1 : 0) | (f[1] ? 2 : 0) | (f[2] ? 4 : 0);
    static const int codes[8] = {0, 1, 2, 4, 3, 5, 6, 7};  // (x, y, xy, z, xz, yz, xyz) by flag bits
    return codes[m];
  };
  for (auto &spc : spcs) {
    if ((int)spc.size() < 2 + dim) throw KError(CFEM_ERR_MESH, "short *BOUNDARY_SPC_SET card");
    std::vector<int> flags(dim);
    for (int d = 0; d < dim; ++d) flags[d] = to_int(spc[2 + d]) != 0;
    for (auto &key : set_order) {
      if (spc[0] != key) continue;
      for (int d = 0; d < dim; ++d)
        if (to_int(spc[2 + d]) != 0 && to_int(spc[2 + d]) != 1)
          throw KError(CFEM_ERR_MESH, "*BOUNDARY_SPC_SET " + spc[0] + ": flags must be 0 or 1");
      const int code = code_of(flags);
      if (!code) throw KError(CFEM_ERR_MESH, "*BOUNDARY_SPC_SET " + spc[0] + ": no constrained DOF");
      for (auto &m : sets[key]) {
        K.cons.push_back(node_of(m));
        K.cons.push_back(code);
      }
    }
  }
  // nodal loads: the first card whose set exists
  for (auto &ld : node_loads) {
    if (ld.empty() || !sets.count(ld[0])) continue;
    if (ld.size() < 3) throw KError(CFEM_ERR_MESH, "short *LOAD_NODE_SET card");
    auto cv = curves.find(ld[2]);
    if (cv == curves.end()) throw KError(CFEM_ERR_MESH, "*LOAD_NODE_SET names curve " + ld[2] + ", which is not defined");
    const int axis = to_int(ld[1]) - 1;
    if (axis < 0 || axis >= dim) throw KError(CFEM_ERR_MESH, "*LOAD_NODE_SET: bad direction " + ld[1]);
    const double val = to_double(cv->second);
    for (auto &m : sets[ld[0]]) {
      K.load_node.push_back(node_of(m));
      for (int d = 0; d < dim; ++d) K.load_vec.push_back(d == axis ? val : 0.0);
    }
    break;
  }
  // pressure faces: each face of the first element (file order) that has it
  if (!segments.empty()) {
    std::map<std::vector<int32_t>, std::pair<int32_t, int32_t>> face_to_elem;
    const int64_t ne = (int64_t)elems_raw.size();
    for (int64_t e = 0; e < ne; ++e)
      for (int skip = 0; skip < nv; ++skip) {
        std::vector<int32_t> f;
        for (int a = 0; a < nv; ++a)
          if (a != skip) f.push_back(K.elems[e * nv + a]);
        std::sort(f.begin(), f.end());
        face_to_elem.emplace(f, std::make_pair((int32_t)e, K.elems[e * nv + skip]));
      }
    for (auto &sg : segments) {
      if ((int)sg.size() < 3 + dim) throw KError(CFEM_ERR_MESH, "short *LOAD_SEGMENT card");
      auto cv = curves.find(sg[0]);
      if (cv == curves.end()) throw KError(CFEM_ERR_MESH, "*LOAD_SEGMENT names curve " + sg[0] + ", which is not defined");
      std::vector<int32_t> fn;
      for (int a = 0; a < dim; ++a) fn.push_back(node_of(sg[3 + a]));
      std::vector<int32_t> key = fn;
      std::sort(key.begin(), key.end());
      auto hit = face_to_elem.find(key);
      if (hit == face_to_elem.end()) throw KError(CFEM_ERR_MESH, "*LOAD_SEGMENT face belongs to no element");
      const int32_t ei = hit->second.first, opp = hit->second.second;
      auto X = [&](int32_t n, int d) { return K.nodes[(size_t)n * dim + d]; };
      double nrm[3] = {0, 0, 0};
      if (dim == 2) {
        nrm[0] = X(fn[1], 1) - X(fn[0], 1);
        nrm[1] = -(X(fn[1], 0) - X(fn[0], 0));
      } else {
        double a[3], b[3];
        for (int d = 0; d < 3; ++d) {
          a[d] = X(fn[1], d) - X(fn[0], d);
          b[d] = X(fn[2], d) - X(fn[0], d);
        }
        nrm[0] = a[1] * b[2] - a[2] * b[1];
        nrm[1] = a[2] * b[0] - a[0] * b[2];
        nrm[2] = a[0] * b[1] - a[1] * b[0];
      }
      double dot = 0;
      for (int d = 0; d < dim; ++d) dot += nrm[d] * (X(opp, d) - X(fn[0], d));
      if (dot > 0)
        for (int d = 0; d < dim; ++d) nrm[d] = -nrm[d];
      for (int a = 0; a < dim; ++a) K.face_nodes.push_back(fn[a]);
      K.face_nodes.push_back(opp);
      K.face_elem.push_back(ei);
      for (int d = 0; d < dim; ++d) K.face_normal.push_back(nrm[d]);
      K.face_pressure.push_back(to_double(cv->second));
    }
  }
}

cfem_status guarded(const std::function<void()> &fn) {
  try {
    fn();
    return CFEM_OK;
  } catch (const KError &e) {
    cfem::detail::g_last_error = e.what();
    return e.st;
  } catch (const std::bad_alloc &) {
    cfem::detail::g_last_error = "host out of memory";
    return CFEM_ERR_OUT_OF_MEMORY;
  } catch (const std::exception &e) {
    cfem::detail::g_last_error = std::string("keyword file: ") + e.what();
    return CFEM_ERR_MESH;
  }
}

}  // namespace

extern "C" {

cfem_status cfem_kfile_read(const char *path, int32_t dim, cfem_kfile **out) {
  return guarded([&] {
    if (!path || !out) throw KError(CFEM_ERR_INVALID_ARGUMENT, "null argument");
    *out = nullptr;
    auto *k = new cfem_kfile;
    try {
      read_k(path, dim, *k);
    } catch (...) {
      delete k;
      throw;
    }
    *out = k;
  });
}

cfem_status cfem_kfile_sizes(const cfem_kfile *k, int64_t *n_nodes, int64_t *n_elems, int64_t *n_constraints,
                             int64_t *n_loads, int64_t *n_faces) {
  return guarded([&] {
    if (!k) throw KError(CFEM_ERR_INVALID_ARGUMENT, "null keyword file");
    if (n_nodes) *n_nodes = (int64_t)k->nodes.size() / k->dim;
    if (n_elems) *n_elems = (int64_t)k->elems.size() / (k->dim + 1);
    if (n_constraints) *n_constraints = (int64_t)k->cons.size() / 2;
    if (n_loads) *n_loads = (int64_t)k->load_node.size();
    if (n_faces) *n_faces = (int64_t)k->face_elem.size();
  });
}

cfem_status cfem_kfile_get(const cfem_kfile *k, double *nodes, int32_t *elems, int32_t *constraints, int32_t *load_nodes,
                           double *load_vectors, int32_t *face_nodes, int32_t *face_elems, double *face_normals,
                           double *face_pressures) {
  return guarded([&] {
    if (!k) throw KError(CFEM_ERR_INVALID_ARGUMENT, "null keyword file");
    auto put = [](auto *dst, const auto &v) {
      if (dst && !v.empty()) std::memcpy(dst, v.data(), v.size() * sizeof(v[0]));
    };
    put(nodes, k->nodes);
    put(elems, k->elems);
    put(constraints, k->cons);
    put(load_nodes, k->load_node);
    put(load_vectors, k->load_vec);
    put(face_nodes, k->face_nodes);
    put(face_elems, k->face_elem);
    put(face_normals, k->face_normal);
    put(face_pressures, k->face_pressure);
  });
}

void cfem_kfile_free(cfem_kfile *k) { delete k; }

}  // extern "C"
