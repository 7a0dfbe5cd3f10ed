// Device runtime for the plain FP64 path (host code).
#include "device.hpp"

#include <cuda_runtime_api.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <map>
#include <mutex>
#include <set>
#include <stdexcept>
#include <unordered_map>

#include "edgefem_gb300_kernels.h"
#include "sc_layout.h"

namespace edgefem {

namespace {
constexpr double kC0 = 299792458.0;
thread_local std::string g_last_error;
}  // namespace

const std::string &last_error() { return g_last_error; }
void set_last_error(const std::string &msg) { g_last_error = msg; }

void cuda_check(int code, const char *what) {
  if (code != 0) {
    std::string msg = std::string(what) + ": " + cudaGetErrorString(static_cast<cudaError_t>(code));
    throw std::runtime_error(msg);
  }
}

void DevBuf::alloc(std::size_t bytes) {
  release();
  if (bytes == 0) bytes = 16;
  cuda_check(cudaMalloc(&p_, bytes), "cudaMalloc");
  n_ = bytes;
}
void DevBuf::release() {
  if (p_) cudaFree(p_);
  p_ = nullptr;
  n_ = 0;
}
void DevBuf::zero(CUstream_st *s) { cuda_check(cudaMemsetAsync(p_, 0, n_, s), "cudaMemsetAsync"); }
namespace {
std::atomic<long long> g_h2d{0}, g_d2h{0};
}
void count_h2d(long long b) { g_h2d += b; }
void count_d2h(long long b) { g_d2h += b; }
void transfer_counters(long long *h2d, long long *d2h) {
  if (h2d) *h2d = g_h2d.load();
  if (d2h) *d2h = g_d2h.load();
}

void DevBuf::upload(const void *src, std::size_t bytes, CUstream_st *s) {
  if (bytes > n_) throw std::runtime_error("DevBuf::upload overflow");
  count_h2d(static_cast<long long>(bytes));
  cuda_check(cudaMemcpyAsync(p_, src, bytes, cudaMemcpyHostToDevice, s), "cudaMemcpyAsync H2D");
}
void DevBuf::download(void *dst, std::size_t bytes, CUstream_st *s) const {
  if (bytes > n_) throw std::runtime_error("DevBuf::download overflow");
  count_d2h(static_cast<long long>(bytes));
  cuda_check(cudaMemcpyAsync(dst, p_, bytes, cudaMemcpyDeviceToHost, s), "cudaMemcpyAsync D2H");
  cuda_check(cudaStreamSynchronize(s), "cudaStreamSynchronize");
}

CUstream_st *stream() {
  static cudaStream_t s = [] {
    cudaStream_t st = nullptr;
    cuda_check(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking), "cudaStreamCreate");
    return st;
  }();
  return s;
}

// ------------------------------------------------------------- mesh cache
namespace {
std::mutex g_cache_mu;
std::vector<std::shared_ptr<MeshDev>> g_cache;  // most recent last
constexpr std::size_t kCacheSize = 3;
}  // namespace

std::shared_ptr<MeshDev> mesh_device(const Mesh &mesh, const BC &bc,
                                     const std::vector<std::vector<int>> &blocks) {
  std::vector<int> pec(bc.dirichlet_edges.begin(), bc.dirichlet_edges.end());
  std::sort(pec.begin(), pec.end());
  std::lock_guard<std::mutex> lk(g_cache_mu);
  for (std::size_t i = 0; i < g_cache.size(); ++i) {
    auto &c = g_cache[i];
    if (c->uid == mesh.uid && c->pec_sorted == pec && c->blocks == blocks) {
      auto hit = c;
      g_cache.erase(g_cache.begin() + i);
      g_cache.push_back(hit);
      return hit;
    }
  }
  auto md = std::make_shared<MeshDev>();
  md->uid = mesh.uid;
  md->pec_sorted = pec;
  md->blocks = blocks;
  md->pat = build_pattern(mesh, blocks);
  md->n = md->pat.n;
  md->nnz = md->pat.nnz();
  md->T = static_cast<int>(mesh.tets.size());
  CUstream_st *s = stream();
  std::vector<double> xyz(3 * mesh.nodes.size());
  for (std::size_t i = 0; i < mesh.nodes.size(); ++i) {
    xyz[3 * i] = mesh.nodes[i].xyz.x;
    xyz[3 * i + 1] = mesh.nodes[i].xyz.y;
    xyz[3 * i + 2] = mesh.nodes[i].xyz.z;
  }
  std::vector<int> tn(4 * mesh.tets.size()), te(6 * mesh.tets.size());
  std::vector<std::uint8_t> ts(mesh.tets.size());
  for (std::size_t t = 0; t < mesh.tets.size(); ++t) {
    std::uint8_t bits = 0;
    for (int k = 0; k < 4; ++k) tn[4 * t + k] = mesh.nodeIndex.at(mesh.tets[t].conn[k]);
    for (int k = 0; k < 6; ++k) te[6 * t + k] = mesh.tets[t].edges[k];
    for (int e = 0; e < 6; ++e)
      if (mesh.tets[t].edge_orient[e] < 0) bits |= static_cast<std::uint8_t>(1u << e);
    ts[t] = bits;
  }
  std::vector<std::uint8_t> ip(md->n, 0);
  for (int e : pec)
    if (e >= 0 && e < md->n) ip[e] = 1;
  md->xyz = to_device(xyz, s);
  md->tet_nodes = to_device(tn, s);
  md->tet_signs = to_device(ts, s);
  md->tet_edges = to_device(te, s);
  md->slots = to_device(md->pat.slots, s);
  md->color_tets = to_device(md->pat.color_tets, s);
  md->rowptr = to_device(md->pat.rowptr, s);
  md->colidx = to_device(md->pat.colidx, s);
  md->diag = to_device(md->pat.diag, s);
  md->is_pec = to_device(ip, s);
  // Discrete gradient G (edge-node incidence) without PEC rows.
  md->nn = static_cast<int>(mesh.nodes.size());
  md->enodes_h.assign(2 * static_cast<std::size_t>(md->n), -1);
  std::vector<int> deg(md->nn + 1, 0);
  for (int e = 0; e < md->n; ++e) {
    if (ip[e]) continue;
    const int a = mesh.nodeIndex.at(mesh.edges[e].n0), b = mesh.nodeIndex.at(mesh.edges[e].n1);
    md->enodes_h[2 * e] = a;
    md->enodes_h[2 * e + 1] = b;
    deg[a + 1]++;
    deg[b + 1]++;
  }
  for (int i = 0; i < md->nn; ++i) deg[i + 1] += deg[i];
  md->nptr_h = deg;
  md->nedge_h.assign(deg[md->nn], 0);
  md->nsign_h.assign(deg[md->nn], 0);
  {
    std::vector<int> fill(deg.begin(), deg.end() - 1);
    for (int e = 0; e < md->n; ++e) {
      if (ip[e]) continue;
      const int a = md->enodes_h[2 * e], b = md->enodes_h[2 * e + 1];
      md->nedge_h[fill[a]] = e;
      md->nsign_h[fill[a]++] = -1;
      md->nedge_h[fill[b]] = e;
      md->nsign_h[fill[b]++] = 1;
    }
  }
  md->enodes = to_device(md->enodes_h, s);
  {
    std::vector<double> w(3 * static_cast<std::size_t>(md->n), 0.0);
    for (int e = 0; e < md->n; ++e) {
      const int a = md->enodes_h[2 * e], b = md->enodes_h[2 * e + 1];
      if (a < 0) continue;
      w[3 * e] = 0.5 * (mesh.nodes[b].xyz.x - mesh.nodes[a].xyz.x);
      w[3 * e + 1] = 0.5 * (mesh.nodes[b].xyz.y - mesh.nodes[a].xyz.y);
      w[3 * e + 2] = 0.5 * (mesh.nodes[b].xyz.z - mesh.nodes[a].xyz.z);
    }
    md->piw = to_device(w, s);
  }
  md->nptr = to_device(md->nptr_h, s);
  md->nedge = to_device(md->nedge_h, s);
  md->nsign = to_device(md->nsign_h, s);
  cuda_check(cudaStreamSynchronize(s), "mesh upload");
  g_cache.push_back(md);
  if (g_cache.size() > kCacheSize) g_cache.erase(g_cache.begin());
  return md;
}

void assemble_device(const MeshDev &md, const VecC &cK, const VecC &cM, cplx diag_value,
                     const TermList *terms, const VecC *coefs, DevBuf &values) {
  CUstream_st *s = stream();
  if (values.bytes() < static_cast<std::size_t>(md.nnz) * 16) values.alloc(static_cast<std::size_t>(md.nnz) * 16);
  values.zero(s);
  DevBuf dK = to_device(cK, s), dM = to_device(cM, s);
  const auto &off = md.pat.color_offsets;
  for (std::size_t c = 0; c + 1 < off.size(); ++c)
    cuda_check(efgk_assemble_color(md.xyz.as<double>(), md.tet_nodes.as<int32_t>(), md.tet_signs.as<uint8_t>(),
                                   md.slots.as<int32_t>(), md.color_tets.as<int32_t>(), off[c], off[c + 1],
                                   dK.as<double>(), dM.as<double>(), nullptr, nullptr, values.as<double>(), s),
               "assemble_color");
  cuda_check(efgk_dirichlet(md.n, md.rowptr.as<int32_t>(), md.colidx.as<int32_t>(), md.is_pec.as<uint8_t>(),
                            diag_value.real(), diag_value.imag(), values.as<double>(), s),
             "dirichlet");
  if (terms && !terms->slot.empty()) {
    DevBuf ds = to_device(terms->slot, s), dt = to_device(terms->term, s), dv = to_device(terms->val, s),
           dc = to_device(*coefs, s);
    cuda_check(efgk_add_terms(static_cast<int64_t>(terms->slot.size()), ds.as<int32_t>(), dt.as<int32_t>(),
                              dv.as<double>(), dc.as<double>(), values.as<double>(), s),
               "add_terms");
    cuda_check(cudaStreamSynchronize(s), "assemble");
  } else {
    cuda_check(cudaStreamSynchronize(s), "assemble");
  }
}

// --------------------------------------------------------------- Krylov
KrylovResult krylov64(const MeshDev *md, int n, const int *rowptr, const int *colidx, const int *diag_slot,
                      const double *vals, const double *b, double *x, const std::string &method, double tol,
                      int maxit, int aux_level) {
  CUstream_st *s = stream();
  const std::size_t vb = static_cast<std::size_t>(n) * 16;
  DevBuf dinv(vb), sc(SB_SIZE * 8 > SC_SIZE * 8 ? SB_SIZE * 8 : SC_SIZE * 8);
  cuda_check(efgk_diag_inverse64(n, diag_slot, vals, dinv.as<double>(), s), "diag_inverse");
  // Auxiliary-space preconditioner: Dn = diag(G^T A G) from the assembled values.
  DevBuf dn, dninv, tvec, scratch, dp, dpinv, tpvec, scratch2;
  EfgkAux aux{};
  const bool have_aux = (aux_level == 1 || aux_level == 2) && md && md->nn > 0 && md->n == n;
  if (have_aux) {
    dn.alloc(static_cast<std::size_t>(md->nn) * 16);
    dninv.alloc(static_cast<std::size_t>(md->nn) * 16);
    tvec.alloc(static_cast<std::size_t>(md->nn) * 16);
    scratch.alloc(16);
    dn.zero(s);
    tvec.zero(s);
    cuda_check(efgk_aux_diag64(n, rowptr, colidx, vals, md->enodes.as<int32_t>(), dn.as<double>(), s), "aux_diag");
    cuda_check(efgk_aux_recip64(md->nn, dn.as<double>(), 1e-12, scratch.as<double>(), dninv.as<double>(), s),
               "aux_recip");
    aux.enodes = md->enodes.as<int32_t>();
    aux.nptr = md->nptr.as<int32_t>();
    aux.nedge = md->nedge.as<int32_t>();
    aux.nsign = md->nsign.as<int8_t>();
    aux.dninv = dninv.as<double>();
    aux.t = tvec.as<double>();
    aux.nn = md->nn;
    if (aux_level >= 2) {
      // vector-nodal space: omega / diag(Pi^T A Pi) per (node, component)
      const std::size_t b3 = 3 * static_cast<std::size_t>(md->nn) * 16;
      dp.alloc(b3);
      dpinv.alloc(b3);
      tpvec.alloc(b3);
      scratch2.alloc(16);
      dp.zero(s);
      tpvec.zero(s);
      cuda_check(efgk_aux_pi_diag64(n, rowptr, colidx, vals, md->enodes.as<int32_t>(), md->piw.as<double>(),
                                    1.0 / kVectorAuxWeight, dp.as<double>(), s),
                 "aux_pi_diag");
      cuda_check(efgk_aux_recip64(3 * md->nn, dp.as<double>(), 1e-12, scratch2.as<double>(), dpinv.as<double>(), s),
                 "aux_pi_recip");
      aux.npi = 3;
      aux.piw = md->piw.as<double>();
      aux.dpinv = dpinv.as<double>();
      aux.tp = tpvec.as<double>();
    }
  }
  DevBuf bjinv, bjz, bjsing;
  if (aux_level == 3) {
    bjinv.alloc(static_cast<std::size_t>(EFGK_BJ_DOUBLES(n)) * 8);
    bjz.alloc(vb);
    bjsing.alloc(16);
    bjsing.zero(s);
    cuda_check(efgk_bjacobi_setup64(n, rowptr, colidx, vals, bjinv.as<double>(), bjsing.as<int32_t>(), s),
               "bjacobi_setup");
    aux = EfgkAux{};
    aux.bj_inv = bjinv.as<double>();
    aux.z = bjz.as<double>();
    aux.bj_bs = EFGK_BJ_BS;
  }
  const EfgkAux *auxp = (have_aux || aux_level == 3) ? &aux : nullptr;
  sc.zero(s);
  double *hs = nullptr;
  cuda_check(cudaMallocHost(reinterpret_cast<void **>(&hs), 32 * sizeof(double)), "cudaMallocHost");
  std::unique_ptr<double, void (*)(double *)> hold(hs, [](double *p) { cudaFreeHost(p); });
  const bool cocg = (method == "cocg");
  std::vector<DevBuf> v;
  const int nv = cocg ? 3 : 8;
  for (int i = 0; i < nv; ++i) v.emplace_back(vb);
  const int base_status = cocg ? SC_STATUS : SB_STATUS;
  const int base_iters = cocg ? SC_ITERS : SB_ITERS;
  const int base_rr = cocg ? SC_LASTRR : SB_LASTRR;
  const int base_bb = cocg ? SC_BB : SB_BB;
  double init[SB_SIZE] = {0};
  if (cocg) {
    init[SC_TOL2] = tol * tol;
    init[SC_MAXIT] = maxit;
  } else {
    init[SB_TOL2] = tol * tol;
    init[SB_MAXIT] = maxit;
    init[SB_RHO] = 1.0;
    init[SB_ALPHA] = 1.0;
    init[SB_OMEGA] = 1.0;
  }
  std::memcpy(hs, init, sizeof(double) * SB_SIZE);
  cuda_check(cudaMemcpyAsync(sc.as<double>(), hs, sizeof(double) * SB_SIZE, cudaMemcpyHostToDevice, s), "sc init");
  if (cocg) {
    cuda_check(efgk_cocg64_init(n, b, dinv.as<double>(), x, v[0].as<double>(), v[1].as<double>(), sc.as<double>(),
                                auxp, s),
               "cocg init");
  } else {
    cuda_check(efgk_bicgstab64_init(n, b, x, v[0].as<double>(), v[1].as<double>(), v[2].as<double>(),
                                    v[3].as<double>(), sc.as<double>(), s),
               "bicgstab init");
  }
  // Capture a chunk of iterations as one graph; replay until the device
  // status leaves "running".
  const int chunk = cocg ? 16 : 8;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  cuda_check(cudaStreamSynchronize(s), "krylov init");
  cuda_check(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal), "begin capture");
  int err = 0;
  for (int k = 0; k < chunk && err == 0; ++k) {
    if (cocg)
      err = efgk_cocg64_step(n, rowptr, colidx, vals, dinv.as<double>(), x, v[0].as<double>(), v[1].as<double>(),
                             v[2].as<double>(), sc.as<double>(), k & 1, auxp, s);
    else
      err = efgk_bicgstab64_step(n, rowptr, colidx, vals, dinv.as<double>(), x, v[0].as<double>(),
                                 v[1].as<double>(), v[2].as<double>(), v[3].as<double>(), v[4].as<double>(),
                                 v[5].as<double>(), v[6].as<double>(), v[7].as<double>(), sc.as<double>(), auxp,
                                 s);
  }
  cudaError_t ce = cudaStreamEndCapture(s, &graph);
  cuda_check(err, "krylov capture");
  cuda_check(ce, "end capture");
  cuda_check(cudaGraphInstantiate(&exec, graph, 0), "graph instantiate");
  KrylovResult res;
  const int max_chunks = maxit / chunk + 2;
  cudaEvent_t ev0, ev1;
  cuda_check(cudaEventCreate(&ev0), "cudaEventCreate");
  cuda_check(cudaEventCreate(&ev1), "cudaEventCreate");
  cuda_check(cudaEventRecord(ev0, s), "cudaEventRecord");
  for (int c = 0; c < max_chunks; ++c) {
    cuda_check(cudaGraphLaunch(exec, s), "graph launch");
    cuda_check(cudaMemcpyAsync(hs, sc.as<double>(), sizeof(double) * SB_SIZE, cudaMemcpyDeviceToHost, s), "sc");
    count_d2h(sizeof(double) * SB_SIZE);
    cuda_check(cudaStreamSynchronize(s), "krylov chunk");
    if (hs[base_status] != EFGK_RUNNING) break;
  }
  cuda_check(cudaEventRecord(ev1, s), "cudaEventRecord");
  cuda_check(cudaEventSynchronize(ev1), "cudaEventSynchronize");
  float dev_ms = 0;
  cudaEventElapsedTime(&dev_ms, ev0, ev1);
  cudaEventDestroy(ev0);
  cudaEventDestroy(ev1);
  cudaGraphExecDestroy(exec);
  cudaGraphDestroy(graph);
  const double st = hs[base_status];
  res.iters = static_cast<int>(hs[base_iters]);
  const double bb = hs[base_bb];
  res.residual = bb > 0 ? std::sqrt(hs[base_rr] / bb) : 0.0;
  res.converged = (st == EFGK_CONVERGED);
  res.status = st == EFGK_CONVERGED ? "converged"
               : st == EFGK_BREAKDOWN ? "breakdown"
               : st == EFGK_MAXIT     ? "Solver did not converge within max iterations"
                                      : "running";
  if (bb == 0.0) {  // b = 0: x = 0 is exact
    res.converged = true;
    res.residual = 0.0;
  }
  auto &tot = krylov_totals();
  tot.iters += res.iters;
  tot.max_residual = std::max(tot.max_residual, res.residual);
  tot.solves += 1;
  tot.device_ms += dev_ms;
  return res;
}

KrylovTotals &krylov_totals() {
  static thread_local KrylovTotals t;
  return t;
}

// ------------------------------------------------------------ materials
void tet_coefficients(const Mesh &mesh, const MaxwellParams &p, double omega, VecC &inv_mu, VecC &eps) {
  const std::size_t T = mesh.tets.size();
  inv_mu.resize(T);
  eps.resize(T);
  if (!p.eps_r_tet.empty() && p.eps_r_tet.size() != T)
    throw std::runtime_error("MaxwellParams.eps_r_tet must have one entry per tetrahedron");
  for (std::size_t t = 0; t < T; ++t) {
    inv_mu[t] = 1.0 / p.get_mu_r(mesh.tets[t].phys, omega);
    eps[t] = p.tet_eps(mesh, t, omega);
  }
}

// --------------------------------------------------------------- ports
PortSurface port_surface_mass(const Mesh &mesh, int surface_tag, const std::unordered_set<int> &pec) {
  std::map<std::pair<int, int>, double> acc;
  for (const auto &tri : mesh.tris) {
    if (tri.phys != surface_tag) continue;
    std::array<Vec3, 3> v;
    for (int k = 0; k < 3; ++k) v[k] = mesh.nodes[mesh.nodeIndex.at(tri.conn[k])].xyz;
    auto Ml = triangle_whitney_mass_matrix(v);
    for (int i = 0; i < 3; ++i) {
      const int gi = tri.edges[i];
      if (pec.count(gi)) continue;
      for (int j = 0; j < 3; ++j) {
        const int gj = tri.edges[j];
        if (pec.count(gj)) continue;
        acc[{gi, gj}] += tri.edge_orient[i] * tri.edge_orient[j] * Ml[3 * i + j];
      }
    }
  }
  PortSurface ps;
  for (const auto &kv : acc) {
    ps.rows.push_back(kv.first.first);
    ps.cols.push_back(kv.first.second);
    ps.vals.push_back(kv.second);
  }
  return ps;
}

int port_beta_tet(const Mesh &mesh, int surface_tag) {
  struct H {
    std::size_t operator()(const std::array<std::int64_t, 3> &a) const {
      return std::hash<std::int64_t>()(a[0] * 1000003 ^ a[1] * 7919 ^ a[2]);
    }
  };
  std::unordered_set<std::array<std::int64_t, 3>, H> faces;
  for (const auto &tri : mesh.tris) {
    if (tri.phys != surface_tag) continue;
    std::array<std::int64_t, 3> f{tri.conn[0], tri.conn[1], tri.conn[2]};
    std::sort(f.begin(), f.end());
    faces.insert(f);
  }
  if (faces.empty()) return -1;
  static const int tf[4][3] = {{0, 1, 2}, {0, 1, 3}, {0, 2, 3}, {1, 2, 3}};
  for (std::size_t t = 0; t < mesh.tets.size(); ++t) {
    const auto &c = mesh.tets[t].conn;
    for (const auto &f3 : tf) {
      std::array<std::int64_t, 3> f{c[f3[0]], c[f3[1]], c[f3[2]]};
      std::sort(f.begin(), f.end());
      if (faces.count(f)) return static_cast<int>(t);
    }
  }
  return -1;
}

}  // namespace edgefem
