// Mesh ingest, global edge numbering, PEC edge sets, mesh quality.
//
// Edge numbering follows src/mesh_gmsh.cpp:104-147 of the reference: edges
// are numbered in order of first appearance while scanning tetrahedra
// (local pairs (0,1),(0,2),(0,3),(1,2),(1,3),(2,3)) and then triangles
// ((0,1),(1,2),(2,0)); an edge stores its nodes with n0 < n1 and a local
// edge has orientation +1 iff its first node id is the smaller.  The lookup
// structure here is a per-node adjacency list (first node -> (second node,
// edge id)) instead of a hash map; the numbering it produces is the same.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <fstream>
#include <iostream>
#include <limits>
#include <sstream>
#include <stdexcept>

#include "edgefem.hpp"

namespace edgefem {

namespace {
std::atomic<std::uint64_t> g_mesh_uid{1};

constexpr int kTetPairs[6][2] = {{0, 1}, {0, 2}, {0, 3}, {1, 2}, {1, 3}, {2, 3}};
constexpr int kTriPairs[3][2] = {{0, 1}, {1, 2}, {2, 0}};

struct EdgeTable {
  // For node index a (dense), list of (node index b > a, edge id).
  std::vector<std::vector<std::pair<int, int>>> adj;
  explicit EdgeTable(std::size_t n_nodes) : adj(n_nodes) {}
  int find_or_add(int a, int b, int next_id, bool &added) {
    if (a > b) std::swap(a, b);
    auto &lst = adj[a];
    for (const auto &pr : lst)
      if (pr.first == b) {
        added = false;
        return pr.second;
      }
    lst.emplace_back(b, next_id);
    added = true;
    return next_id;
  }
};

void build_edges(Mesh &mesh) {
  EdgeTable table(mesh.nodes.size());
  mesh.edges.clear();
  auto visit = [&](Element &el, const int (*pairs)[2], int npairs) {
    for (int e = 0; e < npairs; ++e) {
      const std::int64_t a = el.conn[pairs[e][0]];
      const std::int64_t b = el.conn[pairs[e][1]];
      const int ia = mesh.nodeIndex.at(a);
      const int ib = mesh.nodeIndex.at(b);
      bool added = false;
      // The table is keyed by dense index; order by node id for n0 < n1.
      int id = table.find_or_add(ia, ib, static_cast<int>(mesh.edges.size()), added);
      if (added) mesh.edges.push_back(Edge{std::min(a, b), std::max(a, b)});
      el.edges[e] = id;
      el.edge_orient[e] = (a < b) ? 1 : -1;
    }
  };
  for (auto &t : mesh.tets) visit(t, kTetPairs, 6);
  for (auto &t : mesh.tris) visit(t, kTriPairs, 3);
  mesh.edgeIndex.clear();
  mesh.edgeIndex.reserve(mesh.edges.size() * 2);
  for (std::size_t i = 0; i < mesh.edges.size(); ++i)
    mesh.edgeIndex.emplace(make_edge_key(mesh.edges[i].n0, mesh.edges[i].n1), static_cast<int>(i));
}

double tet_signed_volume(const Mesh &mesh, const Element &t) {
  const Vec3 &a = mesh.nodes[mesh.nodeIndex.at(t.conn[0])].xyz;
  const Vec3 &b = mesh.nodes[mesh.nodeIndex.at(t.conn[1])].xyz;
  const Vec3 &c = mesh.nodes[mesh.nodeIndex.at(t.conn[2])].xyz;
  const Vec3 &d = mesh.nodes[mesh.nodeIndex.at(t.conn[3])].xyz;
  const double ux = b.x - a.x, uy = b.y - a.y, uz = b.z - a.z;
  const double vx = c.x - a.x, vy = c.y - a.y, vz = c.z - a.z;
  const double wx = d.x - a.x, wy = d.y - a.y, wz = d.z - a.z;
  return (ux * (vy * wz - vz * wy) - uy * (vx * wz - vz * wx) + uz * (vx * wy - vy * wx)) / 6.0;
}

void warn_quality(const Mesh &mesh, const std::string &label) {
  if (mesh.tets.empty()) return;
  auto r = validate_mesh(mesh);
  if (r.num_degenerate_tets > 0)
    std::cerr << "WARNING: Mesh '" << label << "' contains " << r.num_degenerate_tets
              << " degenerate (zero-volume) tetrahedra. Results may be inaccurate." << std::endl;
  if (r.num_inverted_tets > 0)
    std::cerr << "WARNING: Mesh '" << label << "' contains " << r.num_inverted_tets
              << " inverted tetrahedra. Results may be inaccurate." << std::endl;
  if (r.max_aspect_ratio > 100.0)
    std::cerr << "WARNING: Mesh '" << label << "' has extreme aspect ratio (" << r.max_aspect_ratio
              << "). Consider refining the mesh for better accuracy." << std::endl;
}
}  // namespace

Mesh load_gmsh_v2(const std::string &path) {
  std::ifstream in(path);
  if (!in) throw std::runtime_error("Failed to open mesh file: " + path);
  Mesh mesh;
  std::string line;
  while (std::getline(in, line)) {
    if (!line.empty() && line.back() == '\r') line.pop_back();
    if (line == "$Nodes") {
      long long n = 0;
      in >> n;
      mesh.nodes.reserve(static_cast<std::size_t>(n));
      for (long long i = 0; i < n; ++i) {
        std::int64_t id;
        double x, y, z;
        in >> id >> x >> y >> z;
        mesh.nodeIndex[id] = static_cast<int>(mesh.nodes.size());
        mesh.nodes.push_back(Node{id, Vec3{x, y, z}});
      }
    } else if (line == "$Elements") {
      long long m = 0;
      in >> m;
      for (long long i = 0; i < m; ++i) {
        std::int64_t id;
        int type, ntags;
        in >> id >> type >> ntags;
        Element e;
        e.id = id;
        for (int t = 0; t < ntags; ++t) {
          int tag;
          in >> tag;
          if (t == 0) e.phys = tag;
        }
        if (type == 2) {
          e.type = ElemType::Tri3;
          for (int k = 0; k < 3; ++k) in >> e.conn[k];
          mesh.tris.push_back(e);
        } else if (type == 1) {
          std::int64_t a, b;
          in >> a >> b;  // boundary lines are not used by the 3D path
        } else if (type == 4) {
          e.type = ElemType::Tet4;
          for (int k = 0; k < 4; ++k) in >> e.conn[k];
          mesh.tets.push_back(e);
        } else {
          std::string rest;
          std::getline(in, rest);
        }
      }
    }
  }
  build_edges(mesh);
  mesh.uid = g_mesh_uid++;
  warn_quality(mesh, path);
  return mesh;
}

Mesh mesh_from_arrays(const std::int64_t *node_ids, const double *xyz, std::int64_t n_nodes,
                      const std::int64_t *tets, const std::int32_t *tet_phys, std::int64_t n_tets,
                      const std::int64_t *tris, const std::int32_t *tri_phys, std::int64_t n_tris) {
  Mesh mesh;
  mesh.nodes.resize(static_cast<std::size_t>(n_nodes));
  mesh.nodeIndex.reserve(static_cast<std::size_t>(n_nodes) * 2);
  for (std::int64_t i = 0; i < n_nodes; ++i) {
    mesh.nodes[i] = Node{node_ids[i], Vec3{xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]}};
    if (!mesh.nodeIndex.emplace(node_ids[i], static_cast<int>(i)).second)
      throw std::runtime_error("mesh_from_arrays: duplicate node id " + std::to_string(node_ids[i]));
  }
  mesh.tets.resize(static_cast<std::size_t>(n_tets));
  for (std::int64_t t = 0; t < n_tets; ++t) {
    Element &e = mesh.tets[t];
    e.id = t + 1;
    e.type = ElemType::Tet4;
    for (int k = 0; k < 4; ++k) {
      e.conn[k] = tets[4 * t + k];
      if (!mesh.nodeIndex.count(e.conn[k]))
        throw std::runtime_error("mesh_from_arrays: tetrahedron references unknown node id");
    }
    e.phys = tet_phys ? tet_phys[t] : 0;
  }
  mesh.tris.resize(static_cast<std::size_t>(n_tris));
  for (std::int64_t s = 0; s < n_tris; ++s) {
    Element &e = mesh.tris[s];
    e.id = n_tets + s + 1;
    e.type = ElemType::Tri3;
    for (int k = 0; k < 3; ++k) {
      e.conn[k] = tris[3 * s + k];
      if (!mesh.nodeIndex.count(e.conn[k]))
        throw std::runtime_error("mesh_from_arrays: triangle references unknown node id");
    }
    e.phys = tri_phys ? tri_phys[s] : 0;
  }
  build_edges(mesh);
  mesh.uid = g_mesh_uid++;
  return mesh;
}

namespace {
// Spread the low 21 bits of v to every third bit (Morton / Z-order code).
std::uint64_t spread3(std::uint64_t v) {
  v &= 0x1fffffULL;
  v = (v | (v << 32)) & 0x1f00000000ffffULL;
  v = (v | (v << 16)) & 0x1f0000ff0000ffULL;
  v = (v | (v << 8)) & 0x100f00f00f00f00fULL;
  v = (v | (v << 4)) & 0x10c30c30c30c30c3ULL;
  v = (v | (v << 2)) & 0x1249249249249249ULL;
  return v;
}
}  // namespace

Mesh locality_renumbered(const Mesh &mesh, std::vector<int> *edge_map) {
  Vec3 lo{std::numeric_limits<double>::max(), std::numeric_limits<double>::max(),
          std::numeric_limits<double>::max()};
  Vec3 hi{-lo.x, -lo.y, -lo.z};
  for (const auto &nd : mesh.nodes) {
    lo.x = std::min(lo.x, nd.xyz.x), lo.y = std::min(lo.y, nd.xyz.y), lo.z = std::min(lo.z, nd.xyz.z);
    hi.x = std::max(hi.x, nd.xyz.x), hi.y = std::max(hi.y, nd.xyz.y), hi.z = std::max(hi.z, nd.xyz.z);
  }
  const double span = std::max({hi.x - lo.x, hi.y - lo.y, hi.z - lo.z, 1e-300});
  const double scale = static_cast<double>((1 << 21) - 1) / span;
  auto code = [&](double x, double y, double z) {
    const auto q = [&](double v, double l) {
      const double t = std::floor((v - l) * scale);
      return static_cast<std::uint64_t>(t < 0 ? 0.0 : (t > 2097151.0 ? 2097151.0 : t));
    };
    return spread3(q(x, lo.x)) | (spread3(q(y, lo.y)) << 1) | (spread3(q(z, lo.z)) << 2);
  };
  auto order_by = [](const std::vector<std::uint64_t> &keys) {
    std::vector<int> ord(keys.size());
    for (std::size_t i = 0; i < ord.size(); ++i) ord[i] = static_cast<int>(i);
    std::stable_sort(ord.begin(), ord.end(), [&](int a, int b) { return keys[a] < keys[b]; });
    return ord;
  };
  Mesh out;
  out.tets = mesh.tets;
  out.tris = mesh.tris;
  // nodes in Z-order of their coordinates
  std::vector<std::uint64_t> nkey(mesh.nodes.size());
  for (std::size_t i = 0; i < nkey.size(); ++i) nkey[i] = code(mesh.nodes[i].xyz.x, mesh.nodes[i].xyz.y, mesh.nodes[i].xyz.z);
  const std::vector<int> nord = order_by(nkey);
  out.nodes.resize(mesh.nodes.size());
  out.nodeIndex.reserve(mesh.nodes.size() * 2);
  for (std::size_t i = 0; i < nord.size(); ++i) {
    out.nodes[i] = mesh.nodes[nord[i]];
    out.nodeIndex.emplace(out.nodes[i].id, static_cast<int>(i));
  }
  // edges in Z-order of their midpoints
  std::vector<std::uint64_t> ekey(mesh.edges.size());
  for (std::size_t e = 0; e < ekey.size(); ++e) {
    const Vec3 &a = mesh.nodes[mesh.nodeIndex.at(mesh.edges[e].n0)].xyz;
    const Vec3 &b = mesh.nodes[mesh.nodeIndex.at(mesh.edges[e].n1)].xyz;
    ekey[e] = code(0.5 * (a.x + b.x), 0.5 * (a.y + b.y), 0.5 * (a.z + b.z));
  }
  const std::vector<int> eord = order_by(ekey);
  std::vector<int> emap(mesh.edges.size());
  out.edges.resize(mesh.edges.size());
  for (std::size_t k = 0; k < eord.size(); ++k) {
    emap[eord[k]] = static_cast<int>(k);
    out.edges[k] = mesh.edges[eord[k]];
  }
  for (auto &t : out.tets)
    for (int k = 0; k < 6; ++k) t.edges[k] = emap[t.edges[k]];
  for (auto &t : out.tris)
    for (int k = 0; k < 3; ++k) t.edges[k] = emap[t.edges[k]];
  out.uid = g_mesh_uid++;
  if (edge_map) *edge_map = std::move(emap);
  return out;
}

MeshQualityReport validate_mesh(const Mesh &mesh) {
  MeshQualityReport r;
  r.min_volume = std::numeric_limits<double>::max();
  for (std::size_t i = 0; i < mesh.tets.size(); ++i) {
    const auto &t = mesh.tets[i];
    const double vol = tet_signed_volume(mesh, t);
    double emin = std::numeric_limits<double>::max(), emax = 0;
    for (const auto &pr : kTetPairs) {
      const Vec3 &p = mesh.nodes[mesh.nodeIndex.at(t.conn[pr[0]])].xyz;
      const Vec3 &q = mesh.nodes[mesh.nodeIndex.at(t.conn[pr[1]])].xyz;
      const double d = std::sqrt((p.x - q.x) * (p.x - q.x) + (p.y - q.y) * (p.y - q.y) +
                                 (p.z - q.z) * (p.z - q.z));
      emin = std::min(emin, d);
      emax = std::max(emax, d);
    }
    const double ar = emin < std::numeric_limits<double>::epsilon()
                          ? std::numeric_limits<double>::infinity()
                          : emax / emin;
    r.min_volume = std::min(r.min_volume, vol);
    r.max_aspect_ratio = std::max(r.max_aspect_ratio, ar);
    if (std::abs(vol) < 1e-15) {
      r.num_degenerate_tets++;
      r.bad_tet_indices.push_back(static_cast<int>(i));
    } else if (vol < 0) {
      r.num_inverted_tets++;
      r.bad_tet_indices.push_back(static_cast<int>(i));
    }
  }
  return r;
}

BC build_edge_pec(const Mesh &mesh, int pec_tag) {
  BC bc;
  for (const auto &tri : mesh.tris)
    if (tri.phys == pec_tag)
      for (int k = 0; k < 3; ++k) bc.dirichlet_edges.insert(tri.edges[k]);
  if (bc.dirichlet_edges.empty()) {
    std::ostringstream oss;
    oss << "WARNING: build_edge_pec() found no edges for PEC tag " << pec_tag << ".\n";
    std::cerr << oss.str();
  }
  return bc;
}

}  // namespace edgefem
