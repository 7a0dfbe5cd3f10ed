// Reference-facing C-ABI (include/edgefem_gb300.h) over the C++ host API.
#include "edgefem_gb300.h"
#include "edgefem_gb300_kernels.h"

#include <cuda_runtime_api.h>

#include <cstring>
#include <exception>
#include <memory>
#include <stdexcept>

#include <algorithm>

#include "batched.hpp"
#include "device.hpp"
#include "edgefem.hpp"
#include "pattern.hpp"

using namespace edgefem;

struct efg_mesh_s {
  Mesh mesh;
};
struct efg_spmat_s {
  SpMatC A;
};

namespace {

template <class F>
int guarded(F &&f) {
  try {
    set_last_error("");
    return f();
  } catch (const std::exception &e) {
    set_last_error(e.what());
    return -1;
  } catch (...) {
    set_last_error("unknown error");
    return -1;
  }
}

void need(const void *p, const char *what) {
  if (!p) throw std::invalid_argument(std::string("null argument: ") + what);
}

MaxwellParams to_params(const efg_maxwell_params *cp, std::size_t n_tets) {
  MaxwellParams p;
  if (!cp) return p;
  p.omega = cp->omega;
  p.eps_r = cplx(cp->eps_r[0], cp->eps_r[1]);
  p.mu_r = cplx(cp->mu_r[0], cp->mu_r[1]);
  for (int i = 0; i < cp->n_eps_regions; ++i)
    p.eps_r_regions[cp->eps_region_tags[i]] = cplx(cp->eps_region_vals[2 * i], cp->eps_region_vals[2 * i + 1]);
  for (int i = 0; i < cp->n_mu_regions; ++i)
    p.mu_r_regions[cp->mu_region_tags[i]] = cplx(cp->mu_region_vals[2 * i], cp->mu_region_vals[2 * i + 1]);
  for (int i = 0; i < cp->n_debye; ++i) {
    DebyeMaterial d;
    d.eps_s = cp->debye_params[3 * i];
    d.eps_inf = cp->debye_params[3 * i + 1];
    d.tau = cp->debye_params[3 * i + 2];
    if (!(d.tau > 0)) throw std::invalid_argument("DebyeMaterial: tau must be positive");
    p.eps_models[cp->debye_tags[i]] = d;
  }
  if (cp->eps_tet) {
    p.eps_r_tet.resize(n_tets);
    for (std::size_t t = 0; t < n_tets; ++t) p.eps_r_tet[t] = cplx(cp->eps_tet[2 * t], cp->eps_tet[2 * t + 1]);
  }
  p.use_abc = cp->use_abc != 0;
  for (int i = 0; i < cp->n_abc_tags; ++i) p.abc_surface_tags.insert(cp->abc_tags[i]);
  p.port_abc_scale = cp->port_abc_scale;
  p.use_port_abc = cp->use_port_abc != 0;
  p.port_abc_type = cp->port_abc_type;
  if (p.port_abc_type < 0 || p.port_abc_type > 4) throw std::invalid_argument("port_abc_type must be 0..4");
  return p;
}

BC to_bc(const int32_t *pec, int64_t n) {
  BC bc;
  for (int64_t i = 0; i < n; ++i) bc.dirichlet_edges.insert(pec[i]);
  return bc;
}

PortMode to_mode(const efg_port_mode &m) {
  PortMode o;
  o.fc = m.fc;
  o.kc = m.kc;
  o.omega = m.omega;
  o.eps = cplx(m.eps[0], m.eps[1]);
  o.mu = cplx(m.mu[0], m.mu[1]);
  o.beta = cplx(m.beta[0], m.beta[1]);
  o.Z0 = cplx(m.Z0[0], m.Z0[1]);
  return o;
}
void from_mode(const PortMode &m, efg_port_mode *o) {
  o->fc = m.fc;
  o->kc = m.kc;
  o->omega = m.omega;
  o->eps[0] = m.eps.real(), o->eps[1] = m.eps.imag();
  o->mu[0] = m.mu.real(), o->mu[1] = m.mu.imag();
  o->beta[0] = m.beta.real(), o->beta[1] = m.beta.imag();
  o->Z0[0] = m.Z0.real(), o->Z0[1] = m.Z0.imag();
}

std::vector<WavePort> to_ports(const efg_wave_port *ports, int32_t n) {
  std::vector<WavePort> out(n);
  for (int i = 0; i < n; ++i) {
    out[i].surface_tag = ports[i].surface_tag;
    out[i].mode = to_mode(ports[i].mode);
    out[i].edges.assign(ports[i].edges, ports[i].edges + ports[i].n_edges);
    out[i].weights.resize(ports[i].n_edges);
    for (int64_t k = 0; k < ports[i].n_edges; ++k)
      out[i].weights[k] = cplx(ports[i].weights[2 * k], ports[i].weights[2 * k + 1]);
  }
  return out;
}

SolveOptions to_opts(const efg_solve_options *o, bool eigen_default) {
  SolveOptions s;
  if (eigen_default) {
    s.use_bicgstab = false;
    s.max_iterations = 200000;
  }
  if (!o) return s;
  s.use_bicgstab = o->use_bicgstab != 0;
  s.use_direct = o->use_direct != 0;
  s.tolerance = o->tolerance;
  s.max_iterations = o->max_iterations;
  s.verbose = o->verbose != 0;
  s.preconditioner = o->preconditioner;
  s.use_ilut = o->use_ilut != 0;
  return s;
}

int count_nan_columns(const MatC &S) {
  int bad = 0;
  for (std::size_t c = 0; c < (S.empty() ? 0 : S[0].size()); ++c)
    if (!(S[0][c] == S[0][c])) ++bad;
  return bad;
}

void write_matrix(const MatC &S, double *out) {
  const std::size_t P = S.size();
  for (std::size_t r = 0; r < P; ++r)
    for (std::size_t c = 0; c < P; ++c) {
      out[2 * (r * P + c)] = S[r][c].real();
      out[2 * (r * P + c) + 1] = S[r][c].imag();
    }
}

MatC read_matrix(int32_t n, const double *S) {
  if (n < 0) throw std::invalid_argument("matrix size must be >= 0");
  if (n > 0) need(S, "S");
  MatC M(static_cast<std::size_t>(n), VecC(static_cast<std::size_t>(n)));
  for (int32_t r = 0; r < n; ++r)
    for (int32_t c = 0; c < n; ++c) M[r][c] = cplx(S[2 * (r * n + c)], S[2 * (r * n + c) + 1]);
  return M;
}

void copy_str(char *dst, std::size_t cap, const std::string &s) {
  std::strncpy(dst, s.c_str(), cap - 1);
  dst[cap - 1] = '\0';
}

}  // namespace

extern "C" {

const char *efg_last_error(void) { return last_error().c_str(); }
int efg_abi_version(void) { return 5; }
int efg_device_count(void) {
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return n;
}

int efg_build_edges_gpu(int64_t n_nodes, const int64_t *node_ids, int64_t n_tets, const int32_t *tet_nodes,
                        int64_t n_tris, const int32_t *tri_nodes, int64_t *edge_nodes, int32_t *tet_edges,
                        int8_t *tet_orient, int32_t *tri_edges, int8_t *tri_orient, int64_t *n_edges,
                        double *device_ms) {
  return guarded([&] {
    need(n_edges, "n_edges");
    if (n_nodes < 0 || n_nodes > 0x7fffffffLL || n_tets < 0 || n_tris < 0)
      throw std::invalid_argument("build_edges_gpu: negative or too large size");
    const int64_t m = 6 * n_tets + 3 * n_tris;
    if (m >= 0x7fffffffLL) throw std::invalid_argument("build_edges_gpu: 6 n_tets + 3 n_tris must be < 2^31");
    if (n_tets > 0) need(tet_nodes, "tet_nodes"), need(tet_edges, "tet_edges"), need(tet_orient, "tet_orient");
    if (n_tris > 0) need(tri_nodes, "tri_nodes"), need(tri_edges, "tri_edges"), need(tri_orient, "tri_orient");
    if (m > 0) need(node_ids, "node_ids"), need(edge_nodes, "edge_nodes");
    CUstream_st *s = stream();
    const int nn = static_cast<int>(n_nodes);
    DevBuf ids(std::max<int64_t>(8 * n_nodes, 16)), tet(std::max<int64_t>(16 * n_tets, 16)),
        tri(std::max<int64_t>(12 * n_tris, 16));
    if (n_nodes > 0) ids.upload(node_ids, 8 * n_nodes, s);
    if (n_tets > 0) tet.upload(tet_nodes, 16 * n_tets, s);
    if (n_tris > 0) tri.upload(tri_nodes, 12 * n_tris, s);
    DevBuf oe(std::max<int64_t>(4 * m, 16)), oo(std::max<int64_t>(m, 16)), en(std::max<int64_t>(8 * m, 16)), ne(16);
    DevBuf scratch(static_cast<std::size_t>(efgk_build_edges_scratch_bytes(n_tets, n_tris, nn)));
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (device_ms) {
      cuda_check(cudaEventCreate(&e0), "cudaEventCreate");
      cuda_check(cudaEventCreate(&e1), "cudaEventCreate");
      cuda_check(cudaEventRecord(e0, s), "cudaEventRecord");
    }
    cuda_check(efgk_build_edges(n_tets, tet.as<int32_t>(), n_tris, tri.as<int32_t>(), nn, ids.as<int64_t>(),
                                oe.as<int32_t>(), oo.as<int8_t>(), en.as<int32_t>(), ne.as<int32_t>(),
                                scratch.as<void>(), s),
               "efgk_build_edges");
    if (device_ms) {
      cuda_check(cudaEventRecord(e1, s), "cudaEventRecord");
      cuda_check(cudaEventSynchronize(e1), "cudaEventSynchronize");
      float ms = 0.f;
      cudaEventElapsedTime(&ms, e0, e1);
      *device_ms = ms;
      cudaEventDestroy(e0);
      cudaEventDestroy(e1);
    }
    int32_t n = 0;
    ne.download(&n, 4, s);
    if (n < 0) throw std::invalid_argument("build_edges_gpu: node index out of range");
    if (n_tets > 0) {
      oe.download(tet_edges, 4 * 6 * n_tets, s);
      oo.download(tet_orient, 6 * n_tets, s);
    }
    if (n_tris > 0) {
      std::vector<int32_t> e(3 * n_tris);
      std::vector<int8_t> o(3 * n_tris);
      cuda_check(cudaMemcpyAsync(e.data(), oe.as<int32_t>() + 6 * n_tets, 12 * n_tris, cudaMemcpyDeviceToHost, s),
                 "cudaMemcpyAsync D2H");
      cuda_check(cudaMemcpyAsync(o.data(), oo.as<int8_t>() + 6 * n_tets, 3 * n_tris, cudaMemcpyDeviceToHost, s),
                 "cudaMemcpyAsync D2H");
      cuda_check(cudaStreamSynchronize(s), "cudaStreamSynchronize");
      count_d2h(15 * n_tris);
      std::copy(e.begin(), e.end(), tri_edges);
      std::copy(o.begin(), o.end(), tri_orient);
    }
    std::vector<int32_t> pairs(2 * static_cast<std::size_t>(n));
    if (n > 0) en.download(pairs.data(), 8 * static_cast<std::size_t>(n), s);
    for (int64_t i = 0; i < 2 * static_cast<int64_t>(n); ++i) edge_nodes[i] = node_ids[pairs[i]];
    *n_edges = n;
    return 0;
  });
}

int efg_mesh_create(const int64_t *node_ids, const double *xyz, int64_t n_nodes, const int64_t *tets,
                    const int32_t *tet_phys, int64_t n_tets, const int64_t *tris, const int32_t *tri_phys,
                    int64_t n_tris, efg_mesh_t *out) {
  return guarded([&] {
    need(out, "out");
    if (n_nodes > 0) need(node_ids, "node_ids"), need(xyz, "xyz");
    if (n_tets > 0) need(tets, "tets");
    if (n_tris > 0) need(tris, "tris");
    auto m = std::make_unique<efg_mesh_s>();
    m->mesh = mesh_from_arrays(node_ids, xyz, n_nodes, tets, tet_phys, n_tets, tris, tri_phys, n_tris);
    *out = m.release();
    return 0;
  });
}

int efg_mesh_load_gmsh_v2(const char *path, efg_mesh_t *out) {
  return guarded([&] {
    need(path, "path");
    need(out, "out");
    auto m = std::make_unique<efg_mesh_s>();
    m->mesh = load_gmsh_v2(path);
    *out = m.release();
    return 0;
  });
}

void efg_mesh_destroy(efg_mesh_t mesh) { delete mesh; }

int efg_mesh_sizes(efg_mesh_t m, int64_t *nn, int64_t *nt, int64_t *ns, int64_t *ne) {
  return guarded([&] {
    need(m, "mesh");
    if (nn) *nn = static_cast<int64_t>(m->mesh.nodes.size());
    if (nt) *nt = static_cast<int64_t>(m->mesh.tets.size());
    if (ns) *ns = static_cast<int64_t>(m->mesh.tris.size());
    if (ne) *ne = static_cast<int64_t>(m->mesh.edges.size());
    return 0;
  });
}

int efg_mesh_arrays(efg_mesh_t m, int64_t *node_ids, double *xyz, int64_t *tets, int32_t *tet_phys, int64_t *tris,
                    int32_t *tri_phys) {
  return guarded([&] {
    need(m, "mesh");
    const Mesh &M = m->mesh;
    for (std::size_t i = 0; i < M.nodes.size(); ++i) {
      if (node_ids) node_ids[i] = M.nodes[i].id;
      if (xyz) xyz[3 * i] = M.nodes[i].xyz.x, xyz[3 * i + 1] = M.nodes[i].xyz.y, xyz[3 * i + 2] = M.nodes[i].xyz.z;
    }
    for (std::size_t t = 0; t < M.tets.size(); ++t) {
      if (tets)
        for (int k = 0; k < 4; ++k) tets[4 * t + k] = M.tets[t].conn[k];
      if (tet_phys) tet_phys[t] = M.tets[t].phys;
    }
    for (std::size_t s = 0; s < M.tris.size(); ++s) {
      if (tris)
        for (int k = 0; k < 3; ++k) tris[3 * s + k] = M.tris[s].conn[k];
      if (tri_phys) tri_phys[s] = M.tris[s].phys;
    }
    return 0;
  });
}

int efg_mesh_topology(efg_mesh_t m, int64_t *edge_nodes, int32_t *tet_edges, int8_t *tet_orient, int32_t *tri_edges,
                      int8_t *tri_orient) {
  return guarded([&] {
    need(m, "mesh");
    const Mesh &M = m->mesh;
    if (edge_nodes)
      for (std::size_t e = 0; e < M.edges.size(); ++e) edge_nodes[2 * e] = M.edges[e].n0, edge_nodes[2 * e + 1] = M.edges[e].n1;
    for (std::size_t t = 0; t < M.tets.size(); ++t)
      for (int k = 0; k < 6; ++k) {
        if (tet_edges) tet_edges[6 * t + k] = M.tets[t].edges[k];
        if (tet_orient) tet_orient[6 * t + k] = static_cast<int8_t>(M.tets[t].edge_orient[k]);
      }
    for (std::size_t s = 0; s < M.tris.size(); ++s)
      for (int k = 0; k < 3; ++k) {
        if (tri_edges) tri_edges[3 * s + k] = M.tris[s].edges[k];
        if (tri_orient) tri_orient[3 * s + k] = static_cast<int8_t>(M.tris[s].edge_orient[k]);
      }
    return 0;
  });
}

int efg_validate_mesh(efg_mesh_t m, int32_t *nd, int32_t *ni, double *minv, double *maxar) {
  return guarded([&] {
    need(m, "mesh");
    auto r = validate_mesh(m->mesh);
    if (nd) *nd = r.num_degenerate_tets;
    if (ni) *ni = r.num_inverted_tets;
    if (minv) *minv = r.min_volume;
    if (maxar) *maxar = r.max_aspect_ratio;
    return 0;
  });
}

int efg_validate_mesh_gpu(efg_mesh_t m, int32_t *nd, int32_t *ni, double *minv, double *maxar, int8_t *tet_flag,
                          double *device_ms) {
  return guarded([&] {
    need(m, "mesh");
    const Mesh &mesh = m->mesh;
    const int64_t T = static_cast<int64_t>(mesh.tets.size()), NN = static_cast<int64_t>(mesh.nodes.size());
    std::vector<double> xyz(3 * NN);
    for (int64_t i = 0; i < NN; ++i)
      xyz[3 * i] = mesh.nodes[i].xyz.x, xyz[3 * i + 1] = mesh.nodes[i].xyz.y, xyz[3 * i + 2] = mesh.nodes[i].xyz.z;
    std::vector<int32_t> tn(4 * T);
    for (int64_t t = 0; t < T; ++t)
      for (int k = 0; k < 4; ++k) tn[4 * t + k] = mesh.nodeIndex.at(mesh.tets[t].conn[k]);
    CUstream_st *s = stream();
    DevBuf dx = to_device(xyz, s), dt = to_device(tn, s), flag(std::max<int64_t>(T, 16)), out(16), cnt(16);
    DevBuf scratch(static_cast<std::size_t>(efgk_validate_mesh_scratch_bytes(T)));
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (device_ms) {
      cuda_check(cudaEventCreate(&e0), "cudaEventCreate");
      cuda_check(cudaEventCreate(&e1), "cudaEventCreate");
      cuda_check(cudaEventRecord(e0, s), "cudaEventRecord");
    }
    cuda_check(efgk_validate_mesh(T, dx.as<double>(), dt.as<int32_t>(), flag.as<int8_t>(), out.as<double>(),
                                  cnt.as<int32_t>(), scratch.as<void>(), s),
               "efgk_validate_mesh");
    if (device_ms) {
      cuda_check(cudaEventRecord(e1, s), "cudaEventRecord");
      cuda_check(cudaEventSynchronize(e1), "cudaEventSynchronize");
      float ms = 0.f;
      cudaEventElapsedTime(&ms, e0, e1);
      *device_ms = ms;
      cudaEventDestroy(e0);
      cudaEventDestroy(e1);
    }
    double o[2];
    int32_t c[2];
    out.download(o, sizeof o, s);
    cnt.download(c, sizeof c, s);
    if (tet_flag && T > 0) flag.download(tet_flag, static_cast<std::size_t>(T), s);
    if (nd) *nd = c[0];
    if (ni) *ni = c[1];
    if (minv) *minv = o[0];
    if (maxar) *maxar = o[1];
    return 0;
  });
}

int efg_build_edge_pec(efg_mesh_t m, int pec_tag, int32_t *out, int64_t cap, int64_t *count) {
  return guarded([&] {
    need(m, "mesh");
    BC bc = build_edge_pec(m->mesh, pec_tag);
    std::vector<int> v(bc.dirichlet_edges.begin(), bc.dirichlet_edges.end());
    std::sort(v.begin(), v.end());
    if (count) *count = static_cast<int64_t>(v.size());
    if (out) {
      if (cap < static_cast<int64_t>(v.size())) throw std::invalid_argument("efg_build_edge_pec: capacity too small");
      std::copy(v.begin(), v.end(), out);
    }
    return 0;
  });
}

int efg_pattern(efg_mesh_t m, int32_t *rowptr, int32_t *colidx, int64_t *nnz, int32_t *n_colors) {
  return guarded([&] {
    need(m, "mesh");
    Pattern P = build_pattern(m->mesh, {});
    if (nnz) *nnz = P.nnz();
    if (n_colors) *n_colors = static_cast<int32_t>(P.color_offsets.size()) - 1;
    if (rowptr) std::copy(P.rowptr.begin(), P.rowptr.end(), rowptr);
    if (colidx) std::copy(P.colidx.begin(), P.colidx.end(), colidx);
    return 0;
  });
}

int efg_element_matrices(const double *x, double *K36, double *M36) {
  return guarded([&] {
    need(x, "xyz4");
    std::array<Vec3, 4> v;
    for (int k = 0; k < 4; ++k) v[k] = Vec3{x[3 * k], x[3 * k + 1], x[3 * k + 2]};
    double K[36], M[36];
    whitney_element_matrices(v, K, M);
    if (K36) std::memcpy(K36, K, sizeof(K));
    if (M36) std::memcpy(M36, M, sizeof(M));
    return 0;
  });
}

int efg_triangle_mass(const double *x, double *M9) {
  return guarded([&] {
    need(x, "xyz3");
    need(M9, "M9");
    std::array<Vec3, 3> v;
    for (int k = 0; k < 3; ++k) v[k] = Vec3{x[3 * k], x[3 * k + 1], x[3 * k + 2]};
    auto M = triangle_whitney_mass_matrix(v);
    std::copy(M.begin(), M.end(), M9);
    return 0;
  });
}

int efg_solve_te10_mode(double a, double b, double freq, efg_port_mode *out) {
  return guarded([&] {
    need(out, "out");
    RectWaveguidePort port;
    port.a = a;
    port.b = b;
    from_mode(solve_te10_mode(port, freq), out);
    return 0;
  });
}

int efg_build_wave_port_2d(efg_mesh_t m, int surface_tag, const efg_port_mode *mode, const int32_t *pec,
                           int64_t n_pec, double target_kc_sq, int32_t *edges_out, double *weights_out,
                           int64_t capacity, int64_t *count, double *kc_out) {
  return guarded([&] {
    need(m, "mesh");
    need(mode, "mode");
    BC bc = to_bc(pec, n_pec);
    WavePort wp = build_wave_port_2d(m->mesh, surface_tag, to_mode(*mode), bc.dirichlet_edges, target_kc_sq);
    if (count) *count = static_cast<int64_t>(wp.edges.size());
    if (kc_out) *kc_out = wp.mode.kc;
    if (edges_out) {
      if (capacity < static_cast<int64_t>(wp.edges.size())) throw std::invalid_argument("capacity too small");
      for (std::size_t k = 0; k < wp.edges.size(); ++k) {
        edges_out[k] = wp.edges[k];
        if (weights_out) weights_out[2 * k] = wp.weights[k].real(), weights_out[2 * k + 1] = wp.weights[k].imag();
      }
    }
    return 0;
  });
}

int efg_build_lumped_port(efg_mesh_t m, int surface_tag, double z0, const double *e_dir3, int weight_mode,
                          int32_t *edges_out, double *weights_out, int64_t capacity, int64_t *count) {
  return guarded([&] {
    need(m, "mesh");
    need(e_dir3, "e_dir");
    LumpedPortConfig cfg;
    cfg.surface_tag = surface_tag;
    cfg.z0 = z0;
    cfg.e_direction = Vec3{e_dir3[0], e_dir3[1], e_dir3[2]};
    cfg.weight_mode = weight_mode ? LumpedPortWeightMode::Projection : LumpedPortWeightMode::SurfaceIntegral;
    WavePort wp = build_lumped_port(m->mesh, cfg);
    if (count) *count = static_cast<int64_t>(wp.edges.size());
    if (edges_out) {
      if (capacity < static_cast<int64_t>(wp.edges.size())) throw std::invalid_argument("capacity too small");
      for (std::size_t k = 0; k < wp.edges.size(); ++k) {
        edges_out[k] = wp.edges[k];
        if (weights_out) weights_out[2 * k] = wp.weights[k].real(), weights_out[2 * k + 1] = wp.weights[k].imag();
      }
    }
    return 0;
  });
}

void efg_maxwell_params_default(efg_maxwell_params *p) {
  if (!p) return;
  std::memset(p, 0, sizeof(*p));
  p->eps_r[0] = 1.0;
  p->mu_r[0] = 1.0;
  p->port_abc_scale = 1.0;
  p->port_abc_type = 1;
}

void efg_solve_options_default(efg_solve_options *o) {
  if (!o) return;
  SolveOptions s;
  o->use_bicgstab = s.use_bicgstab;
  o->use_direct = s.use_direct;
  o->tolerance = s.tolerance;
  o->max_iterations = s.max_iterations;
  o->verbose = s.verbose;
  o->preconditioner = s.preconditioner;
  o->use_ilut = s.use_ilut ? 1 : 0;
}

int efg_spmat_create(int32_t n, int64_t nnz, const int32_t *rowptr, const int32_t *colidx, const double *values,
                     efg_spmat_t *out) {
  return guarded([&] {
    need(out, "out");
    need(rowptr, "rowptr");
    if (nnz > 0) need(colidx, "colidx"), need(values, "values");
    if (rowptr[n] != nnz) throw std::invalid_argument("efg_spmat_create: rowptr[n] != nnz");
    auto s = std::make_unique<efg_spmat_s>();
    s->A.rows = s->A.cols = n;
    s->A.outer.assign(rowptr, rowptr + n + 1);
    s->A.inner.assign(colidx, colidx + nnz);
    s->A.values.resize(nnz);
    for (int64_t k = 0; k < nnz; ++k) {
      if (colidx[k] < 0 || colidx[k] >= n) throw std::invalid_argument("efg_spmat_create: column out of range");
      s->A.values[k] = cplx(values[2 * k], values[2 * k + 1]);
    }
    for (int32_t r = 0; r < n; ++r)
      if (rowptr[r + 1] < rowptr[r]) throw std::invalid_argument("efg_spmat_create: rowptr not monotone");
    *out = s.release();
    return 0;
  });
}

int efg_spmat_info(efg_spmat_t A, int32_t *n, int64_t *nnz) {
  return guarded([&] {
    need(A, "A");
    if (n) *n = A->A.rows;
    if (nnz) *nnz = A->A.nonZeros();
    return 0;
  });
}

int efg_spmat_export(efg_spmat_t A, int32_t *rowptr, int32_t *colidx, double *values) {
  return guarded([&] {
    need(A, "A");
    if (rowptr) std::copy(A->A.outer.begin(), A->A.outer.end(), rowptr);
    if (colidx) std::copy(A->A.inner.begin(), A->A.inner.end(), colidx);
    if (values)
      for (std::size_t k = 0; k < A->A.values.size(); ++k)
        values[2 * k] = A->A.values[k].real(), values[2 * k + 1] = A->A.values[k].imag();
    return 0;
  });
}

void efg_spmat_destroy(efg_spmat_t A) { delete A; }

int efg_assemble_maxwell(efg_mesh_t m, const efg_maxwell_params *p, const int32_t *pec, int64_t n_pec,
                         const efg_wave_port *ports, int32_t n_ports, int32_t active, efg_spmat_t *A_out,
                         double *b_out) {
  return guarded([&] {
    need(m, "mesh");
    need(A_out, "A_out");
    auto asmbl = assemble_maxwell(m->mesh, to_params(p, m->mesh.tets.size()), to_bc(pec, n_pec),
                                  to_ports(ports, n_ports), active);
    auto s = std::make_unique<efg_spmat_s>();
    s->A = std::move(asmbl.A);
    if (b_out)
      for (std::size_t i = 0; i < asmbl.b.size(); ++i) b_out[2 * i] = asmbl.b[i].real(), b_out[2 * i + 1] = asmbl.b[i].imag();
    *A_out = s.release();
    return 0;
  });
}

int efg_solve_linear(efg_spmat_t A, const double *b, const efg_solve_options *opts, double *x_out,
                     efg_solve_result *result) {
  return guarded([&] {
    need(A, "A");
    need(b, "b");
    VecC bv(A->A.rows);
    for (int i = 0; i < A->A.rows; ++i) bv[i] = cplx(b[2 * i], b[2 * i + 1]);
    SolveResult r = solve_linear(A->A, bv, to_opts(opts, false));
    if (x_out)
      for (std::size_t i = 0; i < r.x.size(); ++i) x_out[2 * i] = r.x[i].real(), x_out[2 * i + 1] = r.x[i].imag();
    if (result) {
      result->iters = r.iters;
      result->residual = r.residual;
      result->converged = r.converged;
      copy_str(result->method, sizeof(result->method), r.method);
      copy_str(result->error_message, sizeof(result->error_message), r.error_message);
    }
    if (r.x.empty() && !r.error_message.empty()) throw std::runtime_error(r.error_message);
    return r.converged ? 0 : 1;
  });
}

int efg_calculate_sparams(efg_mesh_t m, const efg_maxwell_params *p, const int32_t *pec, int64_t n_pec,
                          const efg_wave_port *ports, int32_t n_ports, const efg_solve_options *opts, double *S_out) {
  return guarded([&] {
    need(m, "mesh");
    need(S_out, "S_out");
    MatC S = calculate_sparams(m->mesh, to_params(p, m->mesh.tets.size()), to_bc(pec, n_pec),
                               to_ports(ports, n_ports), to_opts(opts, false));
    write_matrix(S, S_out);
    return count_nan_columns(S);
  });
}

int efg_normalize_port_weights(efg_mesh_t m, const efg_maxwell_params *p, const int32_t *pec, int64_t n_pec,
                               efg_wave_port *ports, int32_t n_ports, const efg_solve_options *opts) {
  return guarded([&] {
    need(m, "mesh");
    auto pv = to_ports(ports, n_ports);
    normalize_port_weights(m->mesh, to_params(p, m->mesh.tets.size()), to_bc(pec, n_pec), pv,
                           to_opts(opts, false));
    for (int i = 0; i < n_ports; ++i)
      for (int64_t k = 0; k < ports[i].n_edges; ++k)
        ports[i].weights[2 * k] = pv[i].weights[k].real(), ports[i].weights[2 * k + 1] = pv[i].weights[k].imag();
    return 0;
  });
}

int efg_calculate_sparams_eigenmode(efg_mesh_t m, const efg_maxwell_params *p, const int32_t *pec, int64_t n_pec,
                                    const efg_wave_port *ports, int32_t n_ports, const efg_solve_options *opts,
                                    double *S_out, efg_solve_result *stats) {
  return guarded([&] {
    need(m, "mesh");
    need(S_out, "S_out");
    SolveOptions o = to_opts(opts, true);
    krylov_totals() = KrylovTotals();
    MatC S = calculate_sparams_eigenmode_opts(m->mesh, to_params(p, m->mesh.tets.size()), to_bc(pec, n_pec),
                                              to_ports(ports, n_ports), o, nullptr);
    write_matrix(S, S_out);
    if (stats) {
      std::memset(stats, 0, sizeof(*stats));
      const auto &tot = krylov_totals();
      stats->iters = static_cast<int32_t>(tot.iters);
      stats->residual = tot.max_residual;
      stats->converged = count_nan_columns(S) == 0;
      copy_str(stats->method, sizeof(stats->method), o.use_bicgstab ? "BiCGSTAB+Jacobi(GPU-FP64)" : "COCG+Jacobi(GPU-FP64)");
    }
    return count_nan_columns(S);
  });
}

int efg_assemble_maxwell_km(efg_mesh_t m, const efg_maxwell_params *p, const int32_t *pec, int64_t n_pec,
                            efg_spmat_t *K_out, efg_spmat_t *M_out) {
  return guarded([&] {
    need(m, "mesh");
    need(K_out, "K_out");
    need(M_out, "M_out");
    KMMatrices km = assemble_maxwell_km(m->mesh, to_params(p, m->mesh.tets.size()), to_bc(pec, n_pec));
    auto k = std::make_unique<efg_spmat_s>();
    auto mm = std::make_unique<efg_spmat_s>();
    k->A = std::move(km.K);
    mm->A = std::move(km.M);
    *K_out = k.release();
    *M_out = mm.release();
    return 0;
  });
}

int efg_frequency_sweep(efg_mesh_t m, const efg_maxwell_params *p, const int32_t *pec, int64_t n_pec,
                        const efg_wave_port *ports, int32_t n_ports, const double *freqs, int32_t n_freqs,
                        const efg_solve_options *opts, double *S_out) {
  return guarded([&] {
    need(m, "mesh");
    need(freqs, "freqs");
    need(S_out, "S_out");
    std::vector<double> f(freqs, freqs + n_freqs);
    SweepResult r = frequency_sweep(m->mesh, to_params(p, m->mesh.tets.size()), to_bc(pec, n_pec),
                                    to_ports(ports, n_ports), f, to_opts(opts, false));
    int bad = 0;
    const std::size_t P = n_ports;
    for (std::size_t i = 0; i < r.S_matrices.size(); ++i) {
      write_matrix(r.S_matrices[i], S_out + 2 * P * P * i);
      bad += count_nan_columns(r.S_matrices[i]);
    }
    return bad;
  });
}

void efg_batch_options_default(efg_batch_options *o) {
  if (!o) return;
  BatchOptions b;
  o->tolerance = b.tolerance;
  o->max_iterations = b.max_iterations;
  o->refine_interval = b.refine_interval;
  o->rows_per_block = b.rows_per_block;
  o->use_graph = b.use_graph;
  o->verbose = b.verbose;
  o->time_spmm = b.time_spmm;
  o->precision = b.precision;
  o->formulation = b.formulation;
  o->vector_aux = b.vector_aux;
  o->reorder = b.reorder;
  o->rb_samples = b.rb_samples;
}

}  // extern "C"

namespace {
struct BatchInputs {
  std::vector<BatchInstance> bi;
  std::vector<BC> bcs;
  BatchOptions bo;
};

BatchInputs to_batch(const efg_batch_instance *inst, int32_t n_inst, const efg_batch_options *opts) {
  need(inst, "inst");
  BatchInputs in;
  in.bi.resize(n_inst);
  in.bcs.resize(n_inst);
  for (int i = 0; i < n_inst; ++i) {
    need(inst[i].mesh, "instance mesh");
    in.bi[i].mesh = &inst[i].mesh->mesh;
    in.bi[i].params = to_params(&inst[i].params, inst[i].mesh->mesh.tets.size());
    in.bcs[i] = to_bc(inst[i].pec, inst[i].n_pec);
    in.bi[i].bc = &in.bcs[i];
    in.bi[i].ports = to_ports(inst[i].ports, inst[i].n_ports);
  }
  if (opts) {
    in.bo.tolerance = opts->tolerance;
    in.bo.max_iterations = opts->max_iterations;
    in.bo.refine_interval = opts->refine_interval;
    in.bo.rows_per_block = opts->rows_per_block;
    in.bo.use_graph = opts->use_graph != 0;
    in.bo.verbose = opts->verbose != 0;
    in.bo.time_spmm = opts->time_spmm != 0;
    in.bo.precision = opts->precision;
    in.bo.formulation = opts->formulation;
    in.bo.vector_aux = opts->vector_aux;
    in.bo.reorder = opts->reorder;
    in.bo.rb_samples = opts->rb_samples;
  }
  return in;
}

int write_batch(const std::vector<std::vector<MatC>> &S, const BatchStats &st, double *S_out,
                efg_batch_stats *stats) {
  int bad = 0;
  std::size_t off = 0;
  for (const auto &inst : S)
    for (const auto &m : inst) {
      const std::size_t P = m.size();
      write_matrix(m, S_out + off);
      off += 2 * P * P;
      bad += count_nan_columns(m);
    }
  if (stats) {
    std::memset(stats, 0, sizeof(*stats));
    stats->solve_ms = st.solve_ms;
    stats->setup_ms = st.setup_ms;
    int mx = 0, mn = 1 << 30, nc = 0;
    double mr = 0;
    for (std::size_t k = 0; k < st.iterations.size(); ++k) {
      mx = std::max(mx, st.iterations[k]);
      mn = std::min(mn, st.iterations[k]);
      nc += st.converged[k];
      mr = std::max(mr, st.residual[k]);
    }
    stats->max_iters = mx;
    stats->min_iters = st.iterations.empty() ? 0 : mn;
    stats->n_converged = nc;
    stats->n_total = static_cast<int32_t>(st.iterations.size());
    stats->max_residual = mr;
    stats->spmm_launches = st.spmm_launches;
    stats->spmm_ms = st.spmm_ms;
    stats->spmm_timed = st.spmm_timed;
    stats->kernel_launches = st.kernel_launches;
    stats->rb_samples = st.rb_samples;
    stats->rb_basis = st.rb_basis;
    stats->rb_done_at_guess = st.rb_done_at_guess;
    stats->rb_ms = st.rb_ms;
    stats->rb_sample_ms = st.rb_sample_ms;
  }
  return bad;
}
}  // namespace

struct efg_batch_s {
  std::unique_ptr<BatchSolver> solver;
};

extern "C" {

int efg_frequency_sweep_batched(efg_mesh_t m, const efg_maxwell_params *p, const int32_t *pec, int64_t n_pec,
                                const efg_wave_port *ports, int32_t n_ports, const double *freqs, int32_t n_freqs,
                                const efg_batch_options *opts, double *S_out, efg_batch_stats *stats) {
  return guarded([&] {
    need(m, "mesh");
    need(freqs, "freqs");
    need(S_out, "S_out");
    efg_batch_instance one{};
    one.mesh = m;
    one.params = *p;
    one.pec = pec;
    one.n_pec = n_pec;
    one.ports = ports;
    one.n_ports = n_ports;
    BatchInputs in = to_batch(&one, 1, opts);
    in.bo.formulation = 1;  // the driven-port (w w^H / Z0) form of frequency_sweep
    BatchStats st;
    std::vector<double> f(freqs, freqs + n_freqs);
    auto S = sparams_eigenmode_batched(in.bi, f, in.bo, &st);
    return write_batch(S, st, S_out, stats);
  });
}

int efg_sparams_eigenmode_batched(const efg_batch_instance *inst, int32_t n_inst, const double *freqs,
                                  int32_t n_freqs, const efg_batch_options *opts, double *S_out,
                                  efg_batch_stats *stats) {
  return guarded([&] {
    need(freqs, "freqs");
    need(S_out, "S_out");
    BatchInputs in = to_batch(inst, n_inst, opts);
    BatchStats st;
    std::vector<double> f(freqs, freqs + n_freqs);
    auto S = sparams_eigenmode_batched(in.bi, f, in.bo, &st);
    return write_batch(S, st, S_out, stats);
  });
}

int efg_batch_create(const efg_batch_instance *inst, int32_t n_inst, const double *freqs, int32_t n_freqs,
                     const efg_batch_options *opts, efg_batch_t *out) {
  return guarded([&] {
    need(freqs, "freqs");
    need(out, "out");
    BatchInputs in = to_batch(inst, n_inst, opts);
    std::vector<double> f(freqs, freqs + n_freqs);
    auto h = std::make_unique<efg_batch_s>();
    h->solver = std::make_unique<BatchSolver>(in.bi, f, in.bo);
    *out = h.release();
    return 0;
  });
}

int efg_batch_solve(efg_batch_t h, double *S_out, efg_batch_stats *stats) {
  return guarded([&] {
    need(h, "handle");
    need(S_out, "S_out");
    BatchStats st;
    auto S = h->solver->solve(&st);
    return write_batch(S, st, S_out, stats);
  });
}

int efg_batch_info(efg_batch_t h, int64_t *rows, int64_t *nnz, int32_t *rhs, int32_t *rpc) {
  return guarded([&] {
    need(h, "handle");
    if (rows) *rows = h->solver->rows();
    if (nnz) *nnz = h->solver->nnz();
    if (rhs) *rhs = h->solver->rhs();
    if (rpc) *rpc = h->solver->rows_per_chunk();
    return 0;
  });
}

void efg_batch_destroy(efg_batch_t h) { delete h; }

int efg_batch_rhs_stats(efg_batch_t h, int32_t *status, int32_t *iters, double *residual) {
  return guarded([&] {
    need(h, "handle");
    const auto &s = h->solver->last_status();
    const auto &it = h->solver->last_iters();
    const auto &r = h->solver->last_residual();
    for (std::size_t i = 0; i < s.size(); ++i) {
      if (status) status[i] = s[i];
      if (iters) iters[i] = it[i];
      if (residual) residual[i] = r[i];
    }
    return 0;
  });
}

void efg_krylov_totals(int32_t reset, int64_t *iters, int32_t *solves, double *max_residual, double *device_ms) {
  auto &t = krylov_totals();
  if (iters) *iters = t.iters;
  if (solves) *solves = t.solves;
  if (max_residual) *max_residual = t.max_residual;
  if (device_ms) *device_ms = t.device_ms;
  if (reset) t = KrylovTotals();
}

void efg_transfer_counters(int64_t *h2d, int64_t *d2h) {
  long long a = 0, b = 0;
  transfer_counters(&a, &b);
  if (h2d) *h2d = a;
  if (d2h) *d2h = b;
}

int efg_sparams_eigenmode_adjoint(efg_mesh_t m, const efg_maxwell_params *p, const int32_t *pec, int64_t n_pec,
                                  const efg_wave_port *ports, int32_t n_ports, int32_t out_j, int32_t in_i,
                                  const efg_solve_options *opts, double *grad_out, double *S_out) {
  return guarded([&] {
    need(m, "mesh");
    need(grad_out, "grad_out");
    MatC S;
    auto g = sparams_eigenmode_adjoint(m->mesh, to_params(p, m->mesh.tets.size()), to_bc(pec, n_pec),
                                       to_ports(ports, n_ports), out_j, in_i, &S, to_opts(opts, true));
    std::copy(g.begin(), g.end(), grad_out);
    if (S_out) write_matrix(S, S_out);
    return count_nan_columns(S);
  });
}

int efg_sparams_driven_adjoint(efg_mesh_t m, const efg_maxwell_params *p, const int32_t *pec, int64_t n_pec,
                               const efg_wave_port *ports, int32_t n_ports, int32_t out_j, int32_t in_i,
                               const efg_solve_options *opts, double *grad_out, double *S_out) {
  return guarded([&] {
    need(m, "mesh");
    need(grad_out, "grad_out");
    MatC S;
    auto g = sparams_driven_adjoint(m->mesh, to_params(p, m->mesh.tets.size()), to_bc(pec, n_pec),
                                    to_ports(ports, n_ports), out_j, in_i, &S, to_opts(opts, true));
    std::copy(g.begin(), g.end(), grad_out);
    if (S_out) write_matrix(S, S_out);
    return count_nan_columns(S);
  });
}

// ------------------------------------------ network parameters, Touchstone

int efg_compute_coupling(int32_t n, const double *S, double freq, double z0, double *Z, double *Y) {
  return guarded([&] {
    const CouplingMatrix cm = compute_coupling(read_matrix(n, S), freq, z0);
    if (Z) write_matrix(cm.Z, Z);
    if (Y) write_matrix(cm.Y, Y);
    return 0;
  });
}

int efg_mutual_coupling_db(int32_t n, const double *S, double *db) {
  return guarded([&] {
    need(db, "db");
    CouplingMatrix cm;
    cm.S = read_matrix(n, S);
    cm.num_ports = n;
    const auto out = mutual_coupling_db(cm);
    for (int32_t r = 0; r < n; ++r)
      for (int32_t c = 0; c < n; ++c) db[r * n + c] = out[r][c];
    return 0;
  });
}

int efg_active_reflection(int32_t n, const double *S, const double *excitation, double *gamma) {
  return guarded([&] {
    need(gamma, "gamma");
    if (n > 0) need(excitation, "excitation");
    VecC a(static_cast<std::size_t>(std::max(n, 0)));
    for (int32_t i = 0; i < n; ++i) a[i] = cplx(excitation[2 * i], excitation[2 * i + 1]);
    const VecC g = active_reflection(read_matrix(n, S), a);
    for (int32_t i = 0; i < n; ++i) gamma[2 * i] = g[i].real(), gamma[2 * i + 1] = g[i].imag();
    return 0;
  });
}

int efg_is_passive(int32_t n, const double *S, double tol) {
  return guarded([&] { return is_passive(read_matrix(n, S), tol) ? 1 : 0; });
}

int efg_check_passivity(int32_t n, const double *S, double tol) {
  return guarded([&] { return check_passivity(read_matrix(n, S), tol) ? 1 : 0; });
}

int efg_is_lossless(int32_t n, const double *S, double tol) {
  return guarded([&] { return is_lossless(read_matrix(n, S), tol) ? 1 : 0; });
}

int efg_is_reciprocal(int32_t n, const double *S, double tol) {
  return guarded([&] { return is_reciprocal(read_matrix(n, S), tol) ? 1 : 0; });
}

int efg_singular_values(int32_t n, const double *S, double *sv) {
  return guarded([&] {
    need(sv, "sv");
    const auto v = singular_values(read_matrix(n, S));
    std::copy(v.begin(), v.end(), sv);
    return 0;
  });
}

int efg_write_touchstone_nport(const char *path, int32_t n_freq, const double *freq, int32_t num_ports,
                               const double *S, int32_t format, double z0) {
  return guarded([&] {
    need(path, "path");
    if (format < 0 || format > 2) throw std::invalid_argument("format must be 0 (RI), 1 (MA) or 2 (DB)");
    if (n_freq < 0 || num_ports < 0) throw std::invalid_argument("sizes must be >= 0");
    if (n_freq > 0) need(freq, "freq");
    std::vector<double> f(freq, freq + n_freq);
    std::vector<MatC> Sm;
    const std::size_t stride = 2 * static_cast<std::size_t>(num_ports) * num_ports;
    for (int32_t k = 0; k < n_freq; ++k) Sm.push_back(read_matrix(num_ports, S ? S + k * stride : nullptr));
    TouchstoneOptions o;
    o.format = static_cast<TouchstoneFormat>(format);
    o.z0 = z0;
    write_touchstone_nport(path, f, Sm, o);
    return 0;
  });
}

int efg_write_touchstone(const char *path, int32_t n_freq, const double *freq, const double *s2) {
  return guarded([&] {
    need(path, "path");
    if (n_freq < 0) throw std::invalid_argument("n_freq must be >= 0");
    if (n_freq > 0) need(freq, "freq"), need(s2, "s2");
    std::vector<double> f(freq, freq + n_freq);
    std::vector<SParams2> d(static_cast<std::size_t>(n_freq));
    for (int32_t k = 0; k < n_freq; ++k) {
      const double *v = s2 + 8 * k;
      d[k] = SParams2{cplx(v[0], v[1]), cplx(v[2], v[3]), cplx(v[4], v[5]), cplx(v[6], v[7])};
    }
    write_touchstone(path, f, d);
    return 0;
  });
}

int efg_touchstone_extension(int32_t num_ports, char *buf, int32_t buf_len) {
  return guarded([&] {
    need(buf, "buf");
    const std::string e = touchstone_extension(num_ports);
    if (buf_len < static_cast<int32_t>(e.size()) + 1) throw std::invalid_argument("buffer too small");
    copy_str(buf, static_cast<std::size_t>(buf_len), e);
    return 0;
  });
}

// ------------------------------------------------------ field post-processing

namespace {
VecC read_cvec(const double *x, std::size_t n) {
  VecC v(n);
  for (std::size_t i = 0; i < n; ++i) v[i] = cplx(x[2 * i], x[2 * i + 1]);
  return v;
}
void write_fields(const std::vector<Vec3C> &E, double *out) {
  for (std::size_t i = 0; i < E.size(); ++i)
    for (int j = 0; j < 3; ++j) out[6 * i + 2 * j] = E[i][j].real(), out[6 * i + 2 * j + 1] = E[i][j].imag();
}
}  // namespace

int efg_compute_barycentric(const double *vertices, const double *point, double *lambda) {
  return guarded([&] {
    need(vertices, "vertices"), need(point, "point"), need(lambda, "lambda");
    std::array<Vec3, 4> v;
    for (int k = 0; k < 4; ++k) v[k] = Vec3{vertices[3 * k], vertices[3 * k + 1], vertices[3 * k + 2]};
    const auto l = compute_barycentric(v, Vec3{point[0], point[1], point[2]});
    std::copy(l.begin(), l.end(), lambda);
    return 0;
  });
}

int efg_evaluate_edge_field(const double *vertices, const int32_t *edge_orient, const double *edge_dofs,
                            const double *point, double *E) {
  return guarded([&] {
    need(vertices, "vertices"), need(edge_orient, "edge_orient"), need(edge_dofs, "edge_dofs");
    need(point, "point"), need(E, "E");
    std::array<Vec3, 4> v;
    for (int k = 0; k < 4; ++k) v[k] = Vec3{vertices[3 * k], vertices[3 * k + 1], vertices[3 * k + 2]};
    std::array<int, 6> o;
    std::array<cplx, 6> d;
    for (int k = 0; k < 6; ++k) o[k] = edge_orient[k], d[k] = cplx(edge_dofs[2 * k], edge_dofs[2 * k + 1]);
    write_fields({evaluate_edge_field(v, o, d, Vec3{point[0], point[1], point[2]})}, E);
    return 0;
  });
}

int efg_evaluate_field(efg_mesh_t m, const double *x, int64_t n_points, const int32_t *tet_of,
                       const double *points, double *E) {
  return guarded([&] {
    need(m, "mesh"), need(x, "x"), need(E, "E");
    const VecC sol = read_cvec(x, m->mesh.edges.size());
    if (!tet_of && !points) {
      write_fields(evaluate_field_at_centroids(m->mesh, sol), E);
      return 0;
    }
    need(tet_of, "tet_of"), need(points, "points");
    if (n_points < 0) throw std::invalid_argument("n_points must be >= 0");
    std::vector<int> to(tet_of, tet_of + n_points);
    std::vector<Vec3> pts(static_cast<std::size_t>(n_points));
    for (int64_t i = 0; i < n_points; ++i) pts[i] = Vec3{points[3 * i], points[3 * i + 1], points[3 * i + 2]};
    write_fields(evaluate_field_at_points(m->mesh, sol, to, pts), E);
    return 0;
  });
}

void efg_vtk_options_default(efg_vtk_options *o) {
  if (!o) return;
  const VTKExportOptions d;
  o->export_magnitude = d.export_magnitude, o->export_phase = d.export_phase;
  o->export_real = d.export_real, o->export_imag = d.export_imag, o->export_vector = d.export_vector;
}

int efg_export_fields_vtk(efg_mesh_t m, const double *x, const char *path, const efg_vtk_options *opts,
                          int32_t legacy) {
  return guarded([&] {
    need(m, "mesh"), need(x, "x"), need(path, "path");
    VTKExportOptions o;
    if (opts) {
      o.export_magnitude = opts->export_magnitude != 0, o.export_phase = opts->export_phase != 0;
      o.export_real = opts->export_real != 0, o.export_imag = opts->export_imag != 0;
      o.export_vector = opts->export_vector != 0;
    }
    const VecC sol = read_cvec(x, m->mesh.edges.size());
    if (legacy)
      export_fields_vtk_legacy(m->mesh, sol, path, o);
    else
      export_fields_vtk(m->mesh, sol, path, o);
    return 0;
  });
}

}  // extern "C"
