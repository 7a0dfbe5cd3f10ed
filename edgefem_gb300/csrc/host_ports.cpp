// Port set-up on the host: analytic TE10 mode, the discrete 2D port mode,
// lumped-port weights, and the small element matrices they use.
//
// The 2D port mode restates src/ports/wave_port.cpp:410-514: K_s e = kc² M_s e
// on the free (non-PEC) port-face edges, picking the eigenvalue closest to
// the target (π/a)² among kc² >= 1e-6·max(target, 1).  The reference runs a
// dense generalized eigensolver; here the selected pair is found by
// shift-invert inverse iteration with shift = target on a banded LU of
// (K_s − σ M_s) after a reverse Cuthill–McKee ordering, which returns the
// same eigenpair whenever it is the one nearest the target (the gradient
// null space sits at kc² ≈ 0, far from it).  The eigenvalue is confirmed
// against the selection rule afterwards.
#include <algorithm>
#include <cmath>
#include <deque>
#include <limits>
#include <numeric>
#include <set>
#include <stdexcept>

#include "edgefem.hpp"

namespace edgefem {

namespace {
constexpr double kC0 = 299792458.0;
constexpr double kEta0 = 376.730313668;  // port_eigensolve.cpp:15
constexpr double kPi = 3.14159265358979323846;
constexpr int kTetPairs[6][2] = {{0, 1}, {0, 2}, {0, 3}, {1, 2}, {1, 3}, {2, 3}};
constexpr int kTriPairs[3][2] = {{0, 1}, {1, 2}, {2, 0}};

inline Vec3 sub(const Vec3 &a, const Vec3 &b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline Vec3 cross(const Vec3 &a, const Vec3 &b) {
  return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
inline double dot(const Vec3 &a, const Vec3 &b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline Vec3 scale(const Vec3 &a, double s) { return {a.x * s, a.y * s, a.z * s}; }
inline double norm(const Vec3 &a) { return std::sqrt(dot(a, a)); }

struct TriGeom {
  bool ok = false;
  double area = 0;
  Vec3 n_hat;
  Vec3 g[3];      // in-plane barycentric gradients
  double curl[3]; // 2 (g_a x g_b).n for local edges
};

TriGeom tri_geom(const std::array<Vec3, 3> &v) {
  TriGeom t;
  Vec3 nrm = cross(sub(v[1], v[0]), sub(v[2], v[0]));
  const double area2 = norm(nrm);
  if (area2 < 1e-30) return t;
  t.ok = true;
  t.n_hat = scale(nrm, 1.0 / area2);
  t.area = area2 / 2.0;
  t.g[0] = scale(cross(t.n_hat, sub(v[2], v[1])), 1.0 / area2);
  t.g[1] = scale(cross(t.n_hat, sub(v[0], v[2])), 1.0 / area2);
  t.g[2] = scale(cross(t.n_hat, sub(v[1], v[0])), 1.0 / area2);
  for (int le = 0; le < 3; ++le)
    t.curl[le] = 2.0 * dot(cross(t.g[kTriPairs[le][0]], t.g[kTriPairs[le][1]]), t.n_hat);
  return t;
}

std::array<Vec3, 3> tri_vertices(const Mesh &mesh, const Element &tri) {
  std::array<Vec3, 3> v;
  for (int k = 0; k < 3; ++k) v[k] = mesh.nodes[mesh.nodeIndex.at(tri.conn[k])].xyz;
  return v;
}

// Banded LU with partial pivoting (row interchanges), LAPACK gbtrf layout
// idea: kl sub-diagonals, ku super-diagonals, fill-in up to kl+ku.
struct BandLU {
  int n = 0, kl = 0, ku = 0, ld = 0;
  std::vector<double> ab;  // column-major band, ld = 2*kl+ku+1
  std::vector<int> piv;
  double &at(int i, int j) { return ab[static_cast<std::size_t>(j) * ld + (kl + ku + i - j)]; }
  bool factor() {
    piv.assign(n, 0);
    const int kv = ku + kl;
    for (int j = 0; j < n; ++j) {
      const int km = std::min(kl, n - 1 - j);
      int p = j;
      double best = std::abs(at(j, j));
      for (int i = j + 1; i <= j + km; ++i)
        if (std::abs(at(i, j)) > best) {
          best = std::abs(at(i, j));
          p = i;
        }
      piv[j] = p;
      if (best == 0.0) return false;
      const int jend = std::min(j + kv, n - 1);
      if (p != j)
        for (int c = j; c <= jend; ++c) std::swap(at(j, c), at(p, c));
      const double inv = 1.0 / at(j, j);
      for (int i = j + 1; i <= j + km; ++i) at(i, j) *= inv;
      for (int c = j + 1; c <= jend; ++c) {
        const double u = at(j, c);
        if (u == 0.0) continue;
        for (int i = j + 1; i <= j + km; ++i) at(i, c) -= at(i, j) * u;
      }
    }
    return true;
  }
  void solve(std::vector<double> &b) {
    const int kv = ku + kl;
    for (int j = 0; j < n; ++j) {
      if (piv[j] != j) std::swap(b[j], b[piv[j]]);
      const int km = std::min(kl, n - 1 - j);
      for (int i = j + 1; i <= j + km; ++i) b[i] -= at(i, j) * b[j];
    }
    for (int j = n - 1; j >= 0; --j) {
      b[j] /= at(j, j);
      const int i0 = std::max(0, j - kv);
      for (int i = i0; i < j; ++i) b[i] -= at(i, j) * b[j];
    }
  }
};

// Reverse Cuthill-McKee ordering of a symmetric adjacency structure.
std::vector<int> rcm_order(const std::vector<std::vector<int>> &adj) {
  const int n = static_cast<int>(adj.size());
  std::vector<int> order;
  order.reserve(n);
  std::vector<char> seen(n, 0);
  std::vector<int> deg(n);
  for (int i = 0; i < n; ++i) deg[i] = static_cast<int>(adj[i].size());
  while (static_cast<int>(order.size()) < n) {
    int start = -1;
    for (int i = 0; i < n; ++i)
      if (!seen[i] && (start < 0 || deg[i] < deg[start])) start = i;
    // pseudo-peripheral: BFS twice from the min-degree node, take the last.
    for (int pass = 0; pass < 2; ++pass) {
      std::vector<char> s2(n, 0);
      std::deque<int> q{start};
      s2[start] = 1;
      int last = start;
      while (!q.empty()) {
        int u = q.front();
        q.pop_front();
        last = u;
        for (int v : adj[u])
          if (!s2[v] && !seen[v]) {
            s2[v] = 1;
            q.push_back(v);
          }
      }
      start = last;
    }
    std::deque<int> q{start};
    seen[start] = 1;
    while (!q.empty()) {
      int u = q.front();
      q.pop_front();
      order.push_back(u);
      std::vector<int> nb;
      for (int v : adj[u])
        if (!seen[v]) nb.push_back(v);
      std::sort(nb.begin(), nb.end(), [&](int a, int b) { return deg[a] < deg[b]; });
      for (int v : nb) {
        seen[v] = 1;
        q.push_back(v);
      }
    }
  }
  std::reverse(order.begin(), order.end());
  return order;
}

// Sign convention for a port-mode vector: the integral over the port face of
// the mode field sum_e w_e N_e (integral of N_e over a flat triangle is
// (A/3)(g_b - g_a), src/ports/lumped_port.cpp:86-87) must be positive on the
// coordinate axis where it is largest.
double mode_sign(const Mesh &mesh, int surface_tag, const std::vector<double> &v_full) {
  Vec3 E{0, 0, 0};
  for (const auto &tri : mesh.tris) {
    if (tri.phys != surface_tag) continue;
    TriGeom g = tri_geom(tri_vertices(mesh, tri));
    if (!g.ok) continue;
    for (int le = 0; le < 3; ++le) {
      const double w = v_full[tri.edges[le]] * tri.edge_orient[le] * g.area / 3.0;
      Vec3 d = sub(g.g[kTriPairs[le][1]], g.g[kTriPairs[le][0]]);
      E.x += w * d.x;
      E.y += w * d.y;
      E.z += w * d.z;
    }
  }
  const double c[3] = {E.x, E.y, E.z};
  int ax = 0;
  for (int k = 1; k < 3; ++k)
    if (std::abs(c[k]) > std::abs(c[ax])) ax = k;
  return c[ax] < 0 ? -1.0 : 1.0;
}
}  // namespace

std::array<double, 9> triangle_whitney_mass_matrix(const std::array<Vec3, 3> &v) {
  std::array<double, 9> M{};
  TriGeom g = tri_geom(v);
  if (!g.ok) return M;
  auto lam = [&](int i, int j) { return i == j ? g.area / 6.0 : g.area / 12.0; };
  for (int i = 0; i < 3; ++i) {
    const int a = kTriPairs[i][0], b = kTriPairs[i][1];
    for (int j = 0; j < 3; ++j) {
      const int c = kTriPairs[j][0], d = kTriPairs[j][1];
      M[3 * i + j] = dot(g.g[b], g.g[d]) * lam(a, c) - dot(g.g[b], g.g[c]) * lam(a, d) -
                     dot(g.g[a], g.g[d]) * lam(b, c) + dot(g.g[a], g.g[c]) * lam(b, d);
    }
  }
  return M;
}

void whitney_element_matrices(const std::array<Vec3, 4> &v, double K[36], double M[36]) {
  // B = [v0-v3, v1-v3, v2-v3] (columns); g_i = rows of B^{-1} = columns of B^{-T}.
  const Vec3 c0 = sub(v[0], v[3]), c1 = sub(v[1], v[3]), c2 = sub(v[2], v[3]);
  const double det = dot(c0, cross(c1, c2));
  const double inv = 1.0 / det;
  Vec3 g[4];
  g[0] = scale(cross(c1, c2), inv);
  g[1] = scale(cross(c2, c0), inv);
  g[2] = scale(cross(c0, c1), inv);
  g[3] = scale(Vec3{g[0].x + g[1].x + g[2].x, g[0].y + g[1].y + g[2].y, g[0].z + g[1].z + g[2].z}, -1.0);
  const double V = std::abs(det) / 6.0;
  Vec3 cu[6];
  for (int i = 0; i < 6; ++i) cu[i] = scale(cross(g[kTetPairs[i][0]], g[kTetPairs[i][1]]), 2.0);
  auto li = [&](int p, int q) { return p == q ? V / 10.0 : V / 20.0; };
  for (int i = 0; i < 6; ++i) {
    const int a = kTetPairs[i][0], b = kTetPairs[i][1];
    for (int j = 0; j < 6; ++j) {
      const int c = kTetPairs[j][0], d = kTetPairs[j][1];
      K[6 * i + j] = V * dot(cu[i], cu[j]);
      M[6 * i + j] = dot(g[b], g[d]) * li(a, c) - dot(g[b], g[c]) * li(a, d) -
                     dot(g[a], g[d]) * li(b, c) + dot(g[a], g[c]) * li(b, d);
    }
  }
}

PortMode solve_te10_mode(const RectWaveguidePort &port, double freq) {
  PortMode mode;
  mode.pol = ModePolarization::TE;
  mode.fc = kC0 / (2.0 * port.a);
  const double k = 2.0 * kPi * freq / kC0;
  const double kc = kPi / port.a;
  mode.kc = kc;
  mode.omega = 2.0 * kPi * freq;
  const double mu0 = 4.0 * kPi * 1e-7;
  mode.mu = mu0;
  mode.eps = 1.0 / (mu0 * kC0 * kC0);
  const double beta = std::sqrt(std::max(0.0, k * k - kc * kc));
  mode.beta = beta;
  mode.Z0 = beta > 0 ? kEta0 * k / beta : 0.0;
  return mode;
}

std::vector<double> solve_port_mode_2d(const Mesh &mesh, int surface_tag,
                                       const std::unordered_set<int> &pec_edges,
                                       double target_kc_sq, double &kc_sq_out) {
  const std::size_t m = mesh.edges.size();
  kc_sq_out = 0.0;
  std::vector<double> v_full(m, 0.0);
  std::unordered_map<int, int> local;
  std::vector<int> port_edges;
  for (const auto &tri : mesh.tris) {
    if (tri.phys != surface_tag) continue;
    for (int le = 0; le < 3; ++le) {
      int ge = tri.edges[le];
      if (pec_edges.count(ge) || local.count(ge)) continue;
      local[ge] = static_cast<int>(port_edges.size());
      port_edges.push_back(ge);
    }
  }
  const int n = static_cast<int>(port_edges.size());
  if (n == 0) return v_full;

  // Element contributions as (i, j, k_val, m_val) in local numbering.
  struct Trip {
    int i, j;
    double k, m;
  };
  std::vector<Trip> trips;
  std::vector<std::vector<int>> adj(n);
  for (const auto &tri : mesh.tris) {
    if (tri.phys != surface_tag) continue;
    auto v = tri_vertices(mesh, tri);
    TriGeom g = tri_geom(v);
    if (!g.ok) continue;
    auto Ml = triangle_whitney_mass_matrix(v);
    for (int i = 0; i < 3; ++i) {
      auto it = local.find(tri.edges[i]);
      if (it == local.end()) continue;
      for (int j = 0; j < 3; ++j) {
        auto jt = local.find(tri.edges[j]);
        if (jt == local.end()) continue;
        const double s = tri.edge_orient[i] * tri.edge_orient[j];
        trips.push_back({it->second, jt->second, s * g.curl[i] * g.curl[j] * g.area, s * Ml[3 * i + j]});
        if (it->second != jt->second) adj[it->second].push_back(jt->second);
      }
    }
  }
  for (auto &a : adj) {
    std::sort(a.begin(), a.end());
    a.erase(std::unique(a.begin(), a.end()), a.end());
  }
  std::vector<int> perm = rcm_order(adj);  // perm[new] = old
  std::vector<int> iperm(n);
  for (int i = 0; i < n; ++i) iperm[perm[i]] = i;
  int bw = 0;
  for (const auto &t : trips) bw = std::max(bw, std::abs(iperm[t.i] - iperm[t.j]));

  // Sparse K_s and M_s in the new ordering (for Rayleigh quotients).
  std::vector<std::vector<std::pair<int, std::pair<double, double>>>> rowsKM(n);
  for (const auto &t : trips) rowsKM[iperm[t.i]].push_back({iperm[t.j], {t.k, t.m}});
  auto apply = [&](const std::vector<double> &x, std::vector<double> &kx, std::vector<double> &mx) {
    kx.assign(n, 0.0);
    mx.assign(n, 0.0);
    for (int i = 0; i < n; ++i)
      for (const auto &e : rowsKM[i]) {
        kx[i] += e.second.first * x[e.first];
        mx[i] += e.second.second * x[e.first];
      }
  };

  const double sigma = target_kc_sq;
  BandLU lu;
  lu.n = n;
  lu.kl = lu.ku = bw;
  lu.ld = 2 * bw + bw + 1;
  lu.ab.assign(static_cast<std::size_t>(lu.ld) * n, 0.0);
  for (const auto &t : trips) lu.at(iperm[t.i], iperm[t.j]) += t.k - sigma * t.m;
  if (!lu.factor()) {
    // Shift hit an eigenvalue exactly: perturb and refactor.
    lu.ab.assign(static_cast<std::size_t>(lu.ld) * n, 0.0);
    const double s2 = sigma * (1.0 + 1e-9);
    for (const auto &t : trips) lu.at(iperm[t.i], iperm[t.j]) += t.k - s2 * t.m;
    if (!lu.factor()) return v_full;
  }
  // Start vector: smooth positive field (deterministic).
  // The iterate converges linearly with ratio |λ1-σ|/|λ2-σ|; stop when it no
  // longer moves (up to the sign flip a negative 1/(λ1-σ) causes).
  // With the shift next to the TE10 value the solve is ill-conditioned and
  // the iterate's rounding noise can stay above 1e-14: stop as well once the
  // change has stopped shrinking at a level below 1e-10 (the noise floor).
  std::vector<double> x(n), kx, mx;
  for (int i = 0; i < n; ++i) x[i] = 1.0 + 0.001 * std::sin(0.7 * i);
  double lambda = 0, prev_change = std::numeric_limits<double>::infinity();
  for (int it = 0; it < 300; ++it) {
    apply(x, kx, mx);
    std::vector<double> y = mx;
    lu.solve(y);
    double nrm = 0;
    for (double v : y) nrm += v * v;
    nrm = std::sqrt(nrm);
    if (!(nrm > 0) || !std::isfinite(nrm)) return v_full;
    double dp = 0, dm = 0, xmax = 0;
    for (int i = 0; i < n; ++i) {
      const double xi = y[i] / nrm;
      dp = std::max(dp, std::abs(xi - x[i]));
      dm = std::max(dm, std::abs(xi + x[i]));
      xmax = std::max(xmax, std::abs(xi));
      x[i] = xi;
    }
    const double change = std::min(dp, dm);
    if (it > 2 && change < 1e-14 * xmax) break;
    if (it > 4 && change < 1e-10 * xmax && change > 0.5 * prev_change) break;
    prev_change = change;
  }
  apply(x, kx, mx);
  lambda = std::inner_product(x.begin(), x.end(), kx.begin(), 0.0) /
           std::inner_product(x.begin(), x.end(), mx.begin(), 0.0);
  const double kc_min = 1e-6 * std::max(target_kc_sq, 1.0);
  if (!(lambda >= kc_min)) return v_full;
  // M-normalise (the dense solver returns M-orthonormal eigenvectors).
  apply(x, kx, mx);
  const double xmx = std::inner_product(x.begin(), x.end(), mx.begin(), 0.0);
  const double s = 1.0 / std::sqrt(xmx);
  for (int i = 0; i < n; ++i) v_full[port_edges[perm[i]]] = x[i] * s;
  const double sg = mode_sign(mesh, surface_tag, v_full);
  if (sg < 0)
    for (auto &v : v_full) v = -v;
  kc_sq_out = lambda;
  return v_full;
}

WavePort build_wave_port_2d(const Mesh &mesh, int surface_tag, const PortMode &mode,
                            const std::unordered_set<int> &pec_edges, double target_kc_sq) {
  WavePort port;
  port.surface_tag = surface_tag;
  port.mode = mode;
  double kc_sq = 0.0;
  auto v = solve_port_mode_2d(mesh, surface_tag, pec_edges, target_kc_sq, kc_sq);
  if (kc_sq > 0.0) port.mode.kc = std::sqrt(kc_sq);
  std::set<int> es;
  for (const auto &tri : mesh.tris)
    if (tri.phys == surface_tag)
      for (int le = 0; le < 3; ++le) es.insert(tri.edges[le]);
  port.edges.assign(es.begin(), es.end());
  port.weights.resize(port.edges.size());
  for (std::size_t k = 0; k < port.edges.size(); ++k) port.weights[k] = v[port.edges[k]];
  return port;
}

WavePort build_lumped_port(const Mesh &mesh, const LumpedPortConfig &cfg) {
  std::set<int> es;
  for (const auto &tri : mesh.tris)
    if (tri.phys == cfg.surface_tag)
      for (int e = 0; e < 3; ++e) es.insert(tri.edges[e]);
  if (es.empty())
    throw std::runtime_error("build_lumped_port: no triangles found with surface_tag = " +
                             std::to_string(cfg.surface_tag));
  std::vector<int> edges(es.begin(), es.end());
  std::unordered_map<int, std::size_t> pos;
  for (std::size_t i = 0; i < edges.size(); ++i) pos[edges[i]] = i;
  const double en = norm(cfg.e_direction);
  const Vec3 e_dir = scale(cfg.e_direction, 1.0 / en);
  VecC w(edges.size(), 0.0);
  if (cfg.weight_mode == LumpedPortWeightMode::SurfaceIntegral) {
    for (const auto &tri : mesh.tris) {
      if (tri.phys != cfg.surface_tag) continue;
      TriGeom g = tri_geom(tri_vertices(mesh, tri));
      if (!g.ok) continue;
      for (int le = 0; le < 3; ++le) {
        const int a = kTriPairs[le][0], b = kTriPairs[le][1];
        const double integral = (g.area / 3.0) * dot(sub(g.g[b], g.g[a]), e_dir);
        w[pos[tri.edges[le]]] += cplx(tri.edge_orient[le] * integral, 0.0);
      }
    }
  } else {
    for (std::size_t i = 0; i < edges.size(); ++i) {
      const Edge &ed = mesh.edges[edges[i]];
      const Vec3 &p0 = mesh.nodes[mesh.nodeIndex.at(ed.n0)].xyz;
      const Vec3 &p1 = mesh.nodes[mesh.nodeIndex.at(ed.n1)].xyz;
      w[i] = cplx(dot(sub(p1, p0), e_dir), 0.0);
    }
  }
  double wn = 0;
  for (auto &c : w) wn += std::norm(c);
  wn = std::sqrt(wn);
  if (wn > 1e-15)
    for (auto &c : w) c *= std::sqrt(cfg.z0) / wn;
  WavePort port;
  port.surface_tag = cfg.surface_tag;
  port.edges = edges;
  port.weights = w;
  port.mode.Z0 = cfg.z0;
  return port;
}

}  // namespace edgefem
