// Reference-named drivers: assemble_maxwell, solve_linear,
// calculate_sparams(_eigenmode), normalize_port_weights,
// assemble_maxwell_km, frequency_sweep, and the eigenmode adjoint.
//
// Semantics follow src/assemble_maxwell.cpp, src/solver.cpp and
// src/sweep.cpp of jman4162/EdgeFEM; assembly, solve and port-overlap
// extraction run on the GPU in FP64 (the plain form).
#include <cuda_runtime_api.h>

#include <algorithm>
#include <cmath>
#include <iostream>
#include <limits>
#include <map>
#include <set>
#include <stdexcept>

#include "device.hpp"
#include "edgefem.hpp"
#include "edgefem_gb300_kernels.h"

namespace edgefem {

namespace {
constexpr double kC0 = 299792458.0;
constexpr double kPi = 3.14159265358979323846;
const cplx kNaN(std::numeric_limits<double>::quiet_NaN(), std::numeric_limits<double>::quiet_NaN());

MatC nan_matrix(std::size_t P) { return MatC(P, VecC(P, kNaN)); }

void warn_nonconverged(const KrylovResult &r, const std::string &method, const std::string &ctx) {
  std::cerr << "WARNING: Solver did not converge in " << ctx << " (method=" << method << ", iters=" << r.iters
            << ", residual=" << r.residual << ", error: " << r.status << "). S-parameters may be unreliable."
            << std::endl;
}

// Sparse vector over a few rows.
struct SpVec {
  std::vector<int> idx;
  VecC val;
};

SpVec ms_times(const PortSurface &ms, const std::map<int, cplx> &e) {
  std::map<int, cplx> acc;
  for (std::size_t k = 0; k < ms.rows.size(); ++k) {
    auto it = e.find(ms.cols[k]);
    if (it != e.end()) acc[ms.rows[k]] += ms.vals[k] * it->second;
  }
  SpVec out;
  for (auto &kv : acc) {
    out.idx.push_back(kv.first);
    out.val.push_back(kv.second);
  }
  return out;
}

// Device port-overlap lists: out[l] = sum_k c[l][k] x[idx[l][k]].
struct OverlapLists {
  DevBuf off, idx, c, out;
  int nlists = 0;
  void build(const std::vector<SpVec> &lists) {
    nlists = static_cast<int>(lists.size());
    std::vector<int> o{0}, ix;
    VecC cv;
    for (const auto &l : lists) {
      ix.insert(ix.end(), l.idx.begin(), l.idx.end());
      cv.insert(cv.end(), l.val.begin(), l.val.end());
      o.push_back(static_cast<int>(ix.size()));
    }
    off = to_device(o, stream());
    idx = to_device(ix, stream());
    c = to_device(cv, stream());
    out.alloc(16 * std::max(1, nlists));
  }
  VecC eval(const double *x) {
    VecC r(nlists);
    cuda_check(efgk_port_overlaps64(nlists, off.as<int32_t>(), idx.as<int32_t>(), c.as<double>(), x, 0,
                                    out.as<double>(), stream()),
               "port_overlaps");
    out.download(r.data(), 16 * nlists, stream());
    return r;
  }
};

// Preconditioner level of the mesh-aware drivers: Jacobi without ILUT, the
// requested level otherwise.
int driver_prec(const SolveOptions &o) { return o.use_ilut ? o.preconditioner : 0; }

std::string method_name(bool cocg, int prec = 0) {
  static const char *const names[] = {"Jacobi", "AuxGrad", "AuxSpace", "BlockJacobi"};
  return std::string(cocg ? "COCG+" : "BiCGSTAB+") + names[prec >= 0 && prec <= 3 ? prec : 0] + "(GPU-FP64)";
}

// Eigenmode set-up shared by the plain driver and the adjoint.
struct EigenmodeSetup {
  std::vector<cplx> betas;
  std::vector<int> beta_tets;
  std::vector<PortSurface> ms;
  std::vector<std::map<int, cplx>> e;  // normalised port vectors (non-PEC)
  std::vector<SpVec> c;                // M_s e
  bool evanescent = false;
};

EigenmodeSetup eigenmode_setup(const Mesh &mesh, const MaxwellParams &p, const BC &bc,
                               const std::vector<WavePort> &ports) {
  EigenmodeSetup su;
  const std::size_t P = ports.size();
  const double k0 = p.omega / kC0;
  for (std::size_t i = 0; i < P; ++i) {
    const int t = port_beta_tet(mesh, ports[i].surface_tag);
    cplx em(1.0, 0.0);
    if (t >= 0) em = p.tet_eps(mesh, t, p.omega) * p.get_mu_r(mesh.tets[t].phys, p.omega);
    const double kc = ports[i].mode.kc;
    const cplx bsq = em * k0 * k0 - kc * kc;
    su.beta_tets.push_back(t);
    if (bsq.real() <= 0) {
      const double fc = kc * kC0 / (2.0 * kPi * std::sqrt(std::abs(em.real())));
      std::cerr << "WARNING: Frequency " << p.omega / (2 * kPi) / 1e9 << " GHz is below cutoff " << fc / 1e9
                << " GHz for port " << i << " — mode is evanescent, S-parameters are NaN." << std::endl;
      su.evanescent = true;
    }
    su.betas.push_back(std::sqrt(bsq));
  }
  for (std::size_t i = 0; i < P; ++i) {
    su.ms.push_back(port_surface_mass(mesh, ports[i].surface_tag, bc.dirichlet_edges));
    std::map<int, cplx> e;
    for (std::size_t k = 0; k < ports[i].edges.size(); ++k) {
      const int ed = ports[i].edges[k];
      if (!bc.dirichlet_edges.count(ed) && k < ports[i].weights.size()) e[ed] = ports[i].weights[k];
    }
    SpVec me = ms_times(su.ms[i], e);
    double nsq = 0;
    for (std::size_t k = 0; k < me.idx.size(); ++k) {
      auto it = e.find(me.idx[k]);
      if (it != e.end()) nsq += std::real(std::conj(it->second) * me.val[k]);
    }
    if (nsq > 1e-30) {
      const double s = 1.0 / std::sqrt(nsq);
      for (auto &kv : e) kv.second *= s;
      for (auto &v : me.val) v *= s;
    }
    su.e.push_back(e);
    su.c.push_back(me);
  }
  return su;
}

void add_port_terms(const MeshDev &md, const EigenmodeSetup &su, double alpha, TermList &terms, VecC &coefs) {
  for (std::size_t i = 0; i < su.ms.size(); ++i) {
    const auto &ms = su.ms[i];
    for (std::size_t k = 0; k < ms.rows.size(); ++k) {
      const int s = md.pat.slot_of(ms.rows[k], ms.cols[k]);
      if (s < 0) throw std::runtime_error("port surface entry outside the tetrahedral pattern");
      terms.add(s, static_cast<int>(i), ms.vals[k]);
    }
    coefs.push_back(cplx(0.0, alpha) * su.betas[i]);
  }
}

}  // namespace

WwhTerms wwh_terms(const Mesh &mesh, const MaxwellParams &p, const BC &bc, const std::vector<WavePort> &ports) {
  WwhTerms t;
  for (std::size_t i = 0; i < ports.size(); ++i) {
    const auto &pt = ports[i];
    if (pt.weights.size() != pt.edges.size()) continue;
    if (pt.mode.Z0 == cplx(0.0)) continue;
    std::vector<int> ed;
    std::vector<cplx> w;
    for (std::size_t a = 0; a < pt.edges.size(); ++a)
      if (!bc.dirichlet_edges.count(pt.edges[a])) {
        ed.push_back(pt.edges[a]);
        w.push_back(pt.weights[a]);
      }
    t.blocks.push_back(ed);
    t.w.push_back(w);
    t.port_of_block.push_back(static_cast<int>(i));
  }
  if (p.use_abc) {
    std::set<int> ab;
    for (const auto &tri : mesh.tris) {
      if (!p.abc_surface_tags.empty() && !p.abc_surface_tags.count(tri.phys)) continue;
      for (int e = 0; e < 3; ++e)
        if (!bc.dirichlet_edges.count(tri.edges[e])) ab.insert(tri.edges[e]);
    }
    t.abc_edges.assign(ab.begin(), ab.end());
  }
  return t;
}

namespace {

// Assemble the w w^H system on the device; returns the mesh-device handle.
std::shared_ptr<MeshDev> assemble_wwh(const Mesh &mesh, const MaxwellParams &p, const BC &bc,
                                      const std::vector<WavePort> &ports, bool with_ports, DevBuf &values) {
  WwhTerms wt = with_ports ? wwh_terms(mesh, p, bc, ports) : wwh_terms(mesh, p, bc, {});
  // Only blocks that are not already inside the tetrahedral pattern need to
  // extend it; pass all of them (the pattern builder merges duplicates).
  auto md = mesh_device(mesh, bc, wt.blocks);
  VecC inv_mu, eps;
  tet_coefficients(mesh, p, p.omega, inv_mu, eps);
  const double k0 = p.omega / kC0;
  VecC cM(eps.size());
  for (std::size_t t = 0; t < eps.size(); ++t) cM[t] = -(k0 * k0) * eps[t];
  TermList terms;
  VecC coefs;
  for (std::size_t b = 0; b < wt.blocks.size(); ++b) {
    const auto &ed = wt.blocks[b];
    for (std::size_t a = 0; a < ed.size(); ++a)
      for (std::size_t c = 0; c < ed.size(); ++c)
        terms.add(md->pat.slot_of(ed[a], ed[c]), static_cast<int>(b), wt.w[b][a] * std::conj(wt.w[b][c]));
    coefs.push_back(1.0 / ports[wt.port_of_block[b]].mode.Z0);
  }
  if (!wt.abc_edges.empty()) {
    const int term = static_cast<int>(coefs.size());
    for (int e : wt.abc_edges) terms.add(md->pat.diag[e], term, 1.0);
    coefs.push_back(cplx(0.0, k0));
  }
  if (with_ports && p.use_port_abc && p.port_abc_type != 0) {
    // Legacy port ABC (src/assemble_maxwell.cpp:274-313), with that file's
    // constants mu0 = 4 pi 1e-7, eps0 = 1/(mu0 c0^2), eta0 = mu0 c0.
    const double mu0 = 4.0 * kPi * 1e-7, eps0 = 1.0 / (mu0 * kC0 * kC0), eta0 = mu0 * kC0;
    for (const auto &port : ports) {
      if (port.mode.Z0 == cplx(0.0)) continue;
      const double bsq = k0 * k0 - port.mode.kc * port.mode.kc;
      if (!(bsq > 0)) continue;
      const double beta = std::sqrt(bsq), z = port.mode.Z0.real();
      cplx c;
      switch (p.port_abc_type) {
        case 1: c = cplx(0.0, beta); break;
        case 2: c = cplx(0.0, beta / k0); break;
        case 3: c = cplx(0.0, beta * std::sqrt(z / eta0)); break;
        case 4: c = cplx(0.0, p.omega * eps0 / z); break;
        default: throw std::invalid_argument("port_abc_type must be 0..4");
      }
      const int term = static_cast<int>(coefs.size());
      for (int e : port.edges)
        if (!bc.dirichlet_edges.count(e)) terms.add(md->pat.diag[e], term, 1.0);
      coefs.push_back(c);
    }
  }
  assemble_device(*md, inv_mu, cM, 1.0, &terms, &coefs, values);
  return md;
}

VecC wwh_rhs(const BC &bc, const std::vector<WavePort> &ports, int active, int n) {
  VecC b(n, 0.0);
  if (active < 0 || active >= static_cast<int>(ports.size())) return b;
  const auto &pt = ports[active];
  if (pt.weights.size() != pt.edges.size() || pt.mode.Z0 == cplx(0.0)) return b;
  const cplx scale = 2.0 / std::sqrt(pt.mode.Z0);
  for (std::size_t a = 0; a < pt.edges.size(); ++a)
    if (!bc.dirichlet_edges.count(pt.edges[a])) b[pt.edges[a]] += scale * pt.weights[a];
  return b;
}

SpMatC download_matrix(const std::shared_ptr<MeshDev> &md, const DevBuf &values) {
  SpMatC A;
  A.rows = A.cols = md->n;
  A.outer = md->pat.rowptr;
  A.inner = md->pat.colidx;
  A.values.resize(md->nnz);
  values.download(A.values.data(), static_cast<std::size_t>(md->nnz) * 16, stream());
  A.origin = md;
  return A;
}
}  // namespace

cplx SpMatC::coeff(int r, int c) const {
  auto b = inner.begin() + outer[r], e = inner.begin() + outer[r + 1];
  auto it = std::lower_bound(b, e, c);
  if (it == e || *it != c) return 0.0;
  return values[it - inner.begin()];
}

std::vector<VecC> SpMatC::to_dense() const {
  std::vector<VecC> D(rows, VecC(cols, 0.0));
  for (int r = 0; r < rows; ++r)
    for (int k = outer[r]; k < outer[r + 1]; ++k) D[r][inner[k]] += values[k];
  return D;
}

MaxwellAssembly assemble_maxwell(const Mesh &mesh, const MaxwellParams &p, const BC &bc,
                                 const std::vector<WavePort> &ports, int active_port_idx) {
  DevBuf values;
  auto md = assemble_wwh(mesh, p, bc, ports, true, values);
  MaxwellAssembly out;
  out.A = download_matrix(md, values);
  out.b = wwh_rhs(bc, ports, active_port_idx, md->n);
  return out;
}

SolveResult solve_linear(const SpMatC &A, const VecC &b, const SolveOptions &opt) {
  SolveResult res;
  const bool cocg = !opt.use_bicgstab;
  // Preconditioner: Jacobi without ILUT (the reference's diagonal-
  // preconditioned form); otherwise the requested auxiliary space when the
  // matrix carries its mesh data, block-Jacobi when it does not.
  int prec = opt.use_ilut ? opt.preconditioner : 0;
  if (prec < 0 || prec > 3) prec = 2;
  const MeshDev *md = A.origin && A.origin->n == A.rows ? A.origin.get() : nullptr;
  if ((prec == 1 || prec == 2) && !md) prec = 3;
  res.method = method_name(cocg, prec);
  try {
    if (A.rows != A.cols || static_cast<std::size_t>(A.rows) != b.size())
      throw std::runtime_error("solve_linear: dimension mismatch");
    const int n = A.rows;
    std::vector<int> diag(n);
    for (int r = 0; r < n; ++r) {
      auto bb = A.inner.begin() + A.outer[r], ee = A.inner.begin() + A.outer[r + 1];
      auto it = std::lower_bound(bb, ee, r);
      if (it == ee || *it != r) throw std::runtime_error("solve_linear: missing diagonal entry in row " + std::to_string(r));
      diag[r] = static_cast<int>(it - A.inner.begin());
    }
    CUstream_st *s = stream();
    DevBuf rp = to_device(A.outer, s), ci = to_device(A.inner, s), va = to_device(A.values, s),
           dg = to_device(diag, s), db = to_device(b, s), dx(static_cast<std::size_t>(n) * 16);
    auto kr = krylov64(md, n, rp.as<int>(), ci.as<int>(), dg.as<int>(), va.as<double>(), db.as<double>(),
                       dx.as<double>(), cocg ? "cocg" : "bicgstab", opt.tolerance, opt.max_iterations, prec);
    res.iters = kr.iters;
    res.residual = kr.residual;
    res.converged = kr.converged;
    if (!kr.converged) res.error_message = kr.status;
    res.x.resize(n);
    dx.download(res.x.data(), static_cast<std::size_t>(n) * 16, s);
  } catch (const std::exception &e) {
    res.converged = false;
    res.error_message = e.what();
    set_last_error(e.what());
  }
  if (opt.verbose)
    std::cerr << "Solver: " << res.method << " " << (res.converged ? "CONVERGED" : "FAILED") << " in " << res.iters
              << " iterations, residual=" << res.residual << "\n";
  if (opt.progress_callback) opt.progress_callback(res.iters, res.residual);
  return res;
}

MatC calculate_sparams(const Mesh &mesh, const MaxwellParams &p, const BC &bc, const std::vector<WavePort> &ports,
                       const SolveOptions &opts) {
  return calculate_sparams_opts(mesh, p, bc, ports, opts, nullptr);
}

MatC calculate_sparams_opts(const Mesh &mesh, const MaxwellParams &p, const BC &bc,
                            const std::vector<WavePort> &ports, const SolveOptions &opts,
                            std::vector<VecC> *solutions) {
  const std::size_t P = ports.size();
  if (solutions) solutions->assign(P, VecC());
  MatC S(P, VecC(P, 0.0));
  if (P == 0) return S;
  DevBuf values;
  auto md = assemble_wwh(mesh, p, bc, ports, true, values);
  const int n = md->n;
  std::vector<SpVec> lists(P);
  for (std::size_t j = 0; j < P; ++j)
    for (std::size_t k = 0; k < ports[j].edges.size(); ++k)
      if (!bc.dirichlet_edges.count(ports[j].edges[k]) && k < ports[j].weights.size()) {
        lists[j].idx.push_back(ports[j].edges[k]);
        lists[j].val.push_back(std::conj(ports[j].weights[k]));
      }
  OverlapLists ol;
  ol.build(lists);
  DevBuf db(static_cast<std::size_t>(n) * 16), dx(static_cast<std::size_t>(n) * 16);
  const bool cocg = !opts.use_bicgstab;
  for (std::size_t i = 0; i < P; ++i) {
    VecC b = wwh_rhs(bc, ports, static_cast<int>(i), n);
    db.upload(b.data(), b.size() * 16, stream());
    auto kr = krylov64(md.get(), n, md->rowptr.as<int>(), md->colidx.as<int>(), md->diag.as<int>(),
                       values.as<double>(), db.as<double>(), dx.as<double>(), cocg ? "cocg" : "bicgstab",
                       opts.tolerance, opts.max_iterations, driver_prec(opts));
    if (!kr.converged) {
      warn_nonconverged(kr, method_name(cocg, driver_prec(opts)), "calculate_sparams (active port " + std::to_string(i) + ")");
      for (std::size_t j = 0; j < P; ++j) S[j][i] = kNaN;
      continue;
    }
    VecC V = ol.eval(dx.as<double>());
    if (solutions) {
      (*solutions)[i].resize(static_cast<std::size_t>(n));
      dx.download((*solutions)[i].data(), static_cast<std::size_t>(n) * 16, stream());
    }
    const cplx vinc = std::sqrt(ports[i].mode.Z0);
    for (std::size_t j = 0; j < P; ++j) S[j][i] = (i == j) ? (V[j] - vinc) / vinc : V[j] / vinc;
  }
  return S;
}

void normalize_port_weights(const Mesh &mesh, const MaxwellParams &p, const BC &bc, std::vector<WavePort> &ports,
                            const SolveOptions &opts) {
  if (ports.empty()) return;
  DevBuf values;
  auto md = assemble_wwh(mesh, p, bc, {}, false, values);
  const int n = md->n;
  DevBuf db(static_cast<std::size_t>(n) * 16), dx(static_cast<std::size_t>(n) * 16);
  const bool cocg = !opts.use_bicgstab;
  for (auto &port : ports) {
    if (port.weights.size() != port.edges.size()) continue;
    if (port.mode.Z0 == cplx(0.0)) continue;
    VecC rhs(n, 0.0);
    SpVec cl;
    int free_count = 0;
    for (std::size_t k = 0; k < port.edges.size(); ++k)
      if (!bc.dirichlet_edges.count(port.edges[k])) {
        rhs[port.edges[k]] = port.weights[k];
        cl.idx.push_back(port.edges[k]);
        cl.val.push_back(std::conj(port.weights[k]));
        ++free_count;
      }
    db.upload(rhs.data(), rhs.size() * 16, stream());
    auto kr = krylov64(md.get(), n, md->rowptr.as<int>(), md->colidx.as<int>(), md->diag.as<int>(),
                       values.as<double>(), db.as<double>(), dx.as<double>(), cocg ? "cocg" : "bicgstab",
                       opts.tolerance, opts.max_iterations, driver_prec(opts));
    if (!kr.converged) {
      warn_nonconverged(kr, method_name(cocg, driver_prec(opts)), "normalize_port_weights");
      std::cerr << "  Skipping normalization for this port due to solver failure." << std::endl;
      continue;
    }
    double wn = 0;
    for (auto &w : port.weights) wn += std::norm(w);
    if (std::sqrt(wn) < 1e-15) {
      std::cerr << "WARNING: Port weight vector norm is near-zero." << std::endl;
      continue;
    }
    OverlapLists ol;
    ol.build({cl});
    const double mag = std::abs(ol.eval(dx.as<double>())[0]);
    const double target = std::real(port.mode.Z0);
    std::cerr << "  Port normalization: free_edges=" << free_count << ", wAinvw_exact=" << mag
              << ", target=Z0=" << target << ", ratio=" << mag / target << std::endl;
    if (mag > 1e-15 && target > 1e-15) {
      const double alpha = std::sqrt(target / mag);
      for (auto &w : port.weights) w *= alpha;
    }
  }
}

MatC calculate_sparams_eigenmode(const Mesh &mesh, const MaxwellParams &p, const BC &bc,
                                 const std::vector<WavePort> &ports) {
  SolveOptions o;
  o.use_bicgstab = false;
  o.tolerance = 1e-10;
  o.max_iterations = 200000;
  return calculate_sparams_eigenmode_opts(mesh, p, bc, ports, o, nullptr);
}

MatC calculate_sparams_eigenmode_opts(const Mesh &mesh, const MaxwellParams &p, const BC &bc,
                                      const std::vector<WavePort> &ports, const SolveOptions &opts,
                                      std::vector<VecC> *solutions) {
  const std::size_t P = ports.size();
  if (P == 0) return {};
  EigenmodeSetup su = eigenmode_setup(mesh, p, bc, ports);
  if (su.evanescent) return nan_matrix(P);
  auto md = mesh_device(mesh, bc, {});
  const int n = md->n;
  VecC inv_mu, eps;
  tet_coefficients(mesh, p, p.omega, inv_mu, eps);
  const double k0 = p.omega / kC0;
  VecC cM(eps.size());
  for (std::size_t t = 0; t < eps.size(); ++t) cM[t] = -(k0 * k0) * eps[t];
  TermList terms;
  VecC coefs;
  add_port_terms(*md, su, p.port_abc_scale, terms, coefs);
  DevBuf values;
  assemble_device(*md, inv_mu, cM, 1.0, &terms, &coefs, values);
  std::vector<SpVec> lists(P);
  for (std::size_t j = 0; j < P; ++j) {
    lists[j].idx = su.c[j].idx;
    for (auto v : su.c[j].val) lists[j].val.push_back(std::conj(v));  // e^H M_s x
  }
  OverlapLists ol;
  ol.build(lists);
  MatC S(P, VecC(P, 0.0));
  DevBuf db(static_cast<std::size_t>(n) * 16), dx(static_cast<std::size_t>(n) * 16);
  const bool cocg = !opts.use_bicgstab;
  if (solutions) solutions->assign(P, VecC());
  for (std::size_t a = 0; a < P; ++a) {
    VecC b(n, 0.0);
    const cplx s = 2.0 * cplx(0.0, p.port_abc_scale) * su.betas[a];
    for (std::size_t k = 0; k < su.c[a].idx.size(); ++k) b[su.c[a].idx[k]] = s * su.c[a].val[k];
    db.upload(b.data(), b.size() * 16, stream());
    auto kr = krylov64(md.get(), n, md->rowptr.as<int>(), md->colidx.as<int>(), md->diag.as<int>(),
                       values.as<double>(), db.as<double>(), dx.as<double>(), cocg ? "cocg" : "bicgstab",
                       opts.tolerance, opts.max_iterations, driver_prec(opts));
    if (!kr.converged) {
      warn_nonconverged(kr, method_name(cocg, driver_prec(opts)),
                        "calculate_sparams_eigenmode (active port " + std::to_string(a) + ")");
      for (std::size_t j = 0; j < P; ++j) S[j][a] = kNaN;
      continue;
    }
    VecC V = ol.eval(dx.as<double>());
    for (std::size_t j = 0; j < P; ++j) S[j][a] = V[j] - (j == a ? 1.0 : 0.0);
    if (solutions) {
      (*solutions)[a].resize(n);
      dx.download((*solutions)[a].data(), static_cast<std::size_t>(n) * 16, stream());
    }
  }
  return S;
}

SpMatC KMMatrices::combine(double omega) const {
  const double k0 = omega / kC0;
  SpMatC A = K;
  if (K.inner != M.inner || K.outer != M.outer) throw std::runtime_error("KMMatrices: K and M patterns differ");
  for (std::size_t k = 0; k < A.values.size(); ++k) A.values[k] = K.values[k] - (k0 * k0) * M.values[k];
  return A;
}

KMMatrices assemble_maxwell_km(const Mesh &mesh, const MaxwellParams &p, const BC &bc) {
  // src/sweep.cpp:90-172: static materials only (dispersive models ignored,
  // as there).
  auto md = mesh_device(mesh, bc, {});
  const std::size_t T = mesh.tets.size();
  VecC inv_mu(T), eps(T), zero(T, 0.0);
  for (std::size_t t = 0; t < T; ++t) {
    inv_mu[t] = 1.0 / p.get_mu_r(mesh.tets[t].phys, 0.0);
    if (!p.eps_r_tet.empty()) eps[t] = p.eps_r_tet[t];
    else {
      auto it = p.eps_r_regions.find(mesh.tets[t].phys);
      eps[t] = it != p.eps_r_regions.end() ? it->second : p.eps_r;
    }
  }
  KMMatrices km;
  DevBuf vk, vm;
  assemble_device(*md, inv_mu, zero, 1.0, nullptr, nullptr, vk);
  assemble_device(*md, zero, eps, 0.0, nullptr, nullptr, vm);
  km.K = download_matrix(md, vk);
  km.M = download_matrix(md, vm);
  return km;
}

SweepResult frequency_sweep(const Mesh &mesh, const MaxwellParams &p, const BC &bc,
                            const std::vector<WavePort> &ports, const std::vector<double> &frequencies,
                            const SolveOptions &opts) {
  SweepResult r;
  r.frequencies = frequencies;
  if (ports.empty() || frequencies.empty()) return r;
  for (double f : frequencies) {
    MaxwellParams pf = p;
    pf.omega = 2.0 * kPi * f;
    r.S_matrices.push_back(calculate_sparams(mesh, pf, bc, ports, opts));
  }
  return r;
}

// Adjoint of the eigenmode S-parameters with respect to the real part of each
// tetrahedron's permittivity (mu = 1 assumed for the port term).
//   S_ji = c_j^T x_i - delta_ji,  A x_i = b_i,  A = A^T (complex symmetric).
//   lambda_j = A^{-1} c_j = x_j / (2 j alpha beta_j)  (b_j = 2 j alpha beta_j c_j),
//   so the adjoint costs no extra solve.
//   Volume term: dA/deps_t = -k0^2 (signed M_loc(t))  =>  dS = k0^2 lambda^T M x.
//   Port term: beta_p depends on eps of the tetrahedron t_p the reference reads
//   it from (src/assemble_maxwell.cpp:660-684); it enters A (j alpha beta_p M_s,p)
//   and b_p.
std::vector<double> sparams_eigenmode_adjoint(const Mesh &mesh, const MaxwellParams &p, const BC &bc,
                                              const std::vector<WavePort> &ports, int out_j, int in_i,
                                              MatC *S_out, const SolveOptions &opts) {
  const int P = static_cast<int>(ports.size());
  if (out_j < 0 || out_j >= P || in_i < 0 || in_i >= P)
    throw std::invalid_argument("sparams_eigenmode_adjoint: port index out of range");
  std::vector<VecC> X;
  MatC S = calculate_sparams_eigenmode_opts(mesh, p, bc, ports, opts, &X);
  if (S_out) *S_out = S;
  const std::size_t T = mesh.tets.size();
  std::vector<double> grad(T, std::numeric_limits<double>::quiet_NaN());
  if (X.empty() || X[out_j].empty() || X[in_i].empty()) return grad;
  EigenmodeSetup su = eigenmode_setup(mesh, p, bc, ports);
  const double k0 = p.omega / kC0;
  const double alpha = p.port_abc_scale;
  const cplx lam_scale = 1.0 / (2.0 * cplx(0.0, alpha) * su.betas[out_j]);
  const int n = static_cast<int>(mesh.edges.size());
  VecC lam(n);
  for (int k = 0; k < n; ++k) lam[k] = X[out_j][k] * lam_scale;
  const VecC &xi = X[in_i];
  auto md = mesh_device(mesh, bc, {});
  CUstream_st *s = stream();
  DevBuf dl = to_device(lam, s), dx = to_device(xi, s), dout(T * 16);
  cuda_check(efgk_adjoint_contract(static_cast<int>(T), md->xyz.as<double>(), md->tet_nodes.as<int32_t>(),
                                   md->tet_signs.as<uint8_t>(), md->tet_edges.as<int32_t>(), dl.as<double>(),
                                   dx.as<double>(), k0 * k0, dout.as<double>(), s),
             "adjoint_contract");
  VecC dS(T);
  dout.download(dS.data(), T * 16, s);
  for (int pp = 0; pp < P; ++pp) {
    const int t = su.beta_tets[pp];
    if (t < 0) continue;
    const cplx mu = p.get_mu_r(mesh.tets[t].phys, p.omega);
    const cplx dbeta = (k0 * k0) * mu / (2.0 * su.betas[pp]);
    // lambda^T M_s,p x_i
    cplx lMx = 0.0;
    const auto &ms = su.ms[pp];
    for (std::size_t k = 0; k < ms.rows.size(); ++k) lMx += lam[ms.rows[k]] * ms.vals[k] * xi[ms.cols[k]];
    cplx term = -cplx(0.0, alpha) * dbeta * lMx;
    if (pp == in_i) {
      cplx lc = 0.0;
      for (std::size_t k = 0; k < su.c[pp].idx.size(); ++k) lc += lam[su.c[pp].idx[k]] * su.c[pp].val[k];
      term += 2.0 * cplx(0.0, alpha) * dbeta * lc;
    }
    dS[t] += term;
  }
  const cplx Sji = S[out_j][in_i];
  for (std::size_t t = 0; t < T; ++t) grad[t] = 2.0 * std::real(std::conj(Sji) * dS[t]);
  return grad;
}

// Adjoint of the driven-port S-parameters (calculate_sparams) with respect to
// a real change of each tetrahedron's relative permittivity.
//   S_ji = (c_j^T x_i - delta_ji sqrt(Z0_i)) / sqrt(Z0_i),  A x_i = b_i,
//   c_j = conj(w_j) on the non-PEC port edges, b_i = 2 w_i / sqrt(Z0_i).
// With real port weights A = A^T (the w w^T / Z0 blocks, the jk0 ABC
// diagonal and the Dirichlet rows keep it complex symmetric) and
// b_j = (2 / sqrt(Z0_j)) c_j, so the adjoint vector of c_j is
// lambda_j = A^{-1} c_j = (sqrt(Z0_j) / 2) x_j: no extra solve.
// The permittivity enters only the volume term -k0^2 eps_t M_loc(t) (port
// weights, Z0 and the ABC do not depend on it), so
//   dS_ji / deps_t = (k0^2 / sqrt(Z0_i)) lambda_j,loc^T M_loc(t) x_i,loc.
// A Debye tetrahedron is perturbed about its eps(omega) in the same way.
std::vector<double> sparams_driven_adjoint(const Mesh &mesh, const MaxwellParams &p, const BC &bc,
                                           const std::vector<WavePort> &ports, int out_j, int in_i,
                                           MatC *S_out, const SolveOptions &opts) {
  const int P = static_cast<int>(ports.size());
  if (out_j < 0 || out_j >= P || in_i < 0 || in_i >= P)
    throw std::invalid_argument("sparams_driven_adjoint: port index out of range");
  for (const auto &pt : ports)
    for (const cplx &w : pt.weights)
      if (w.imag() != 0.0)
        throw std::invalid_argument("sparams_driven_adjoint: port weights must be real (the adjoint uses A = A^T)");
  if (p.use_port_abc) throw std::invalid_argument("sparams_driven_adjoint: the legacy port ABC is not supported");
  std::vector<VecC> X;
  MatC S = calculate_sparams_opts(mesh, p, bc, ports, opts, &X);
  if (S_out) *S_out = S;
  const std::size_t T = mesh.tets.size();
  std::vector<double> grad(T, std::numeric_limits<double>::quiet_NaN());
  if (X[out_j].empty() || X[in_i].empty()) return grad;
  const double k0 = p.omega / kC0;
  const cplx lam_scale = std::sqrt(ports[out_j].mode.Z0) / (2.0 * std::sqrt(ports[in_i].mode.Z0));
  const int n = static_cast<int>(mesh.edges.size());
  VecC lam(n);
  for (int k = 0; k < n; ++k) lam[k] = X[out_j][k] * lam_scale;
  auto md = mesh_device(mesh, bc, {});
  CUstream_st *s = stream();
  DevBuf dl = to_device(lam, s), dx = to_device(X[in_i], s), dout(T * 16);
  cuda_check(efgk_adjoint_contract(static_cast<int>(T), md->xyz.as<double>(), md->tet_nodes.as<int32_t>(),
                                   md->tet_signs.as<uint8_t>(), md->tet_edges.as<int32_t>(), dl.as<double>(),
                                   dx.as<double>(), k0 * k0, dout.as<double>(), s),
             "adjoint_contract");
  VecC dS(T);
  dout.download(dS.data(), T * 16, s);
  const cplx Sji = S[out_j][in_i];
  for (std::size_t t = 0; t < T; ++t) grad[t] = 2.0 * std::real(std::conj(Sji) * dS[t]);
  return grad;
}

}  // namespace edgefem
