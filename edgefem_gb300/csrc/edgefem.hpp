// C++ host API of edgefem-gb300.
//
// Same entry-point names and semantics as jman4162/EdgeFEM's C++ library
// (include/edgefem/{mesh,bc,maxwell,solver,sweep}.hpp and
// include/edgefem/ports/*.hpp), with project-owned containers in place of
// Eigen types: VecC is std::vector<std::complex<double>>, SpMatC is a
// compressed-sparse-row matrix.  Every compute step runs on the GPU through
// the kernel-level C-ABI in include/edgefem_gb300_kernels.h; nothing here
// falls back to a CPU solve.
#pragma once

#include <array>
#include <complex>
#include <cstdint>
#include <functional>
#include <memory>
#include <string>
#include <unordered_map>
#include <unordered_set>
#include <vector>

namespace edgefem {

using cplx = std::complex<double>;
using VecC = std::vector<cplx>;

struct Vec3 {
  double x = 0, y = 0, z = 0;
};

// ------------------------------------------------------------------- mesh
// include/edgefem/mesh.hpp:13-52
struct Node {
  std::int64_t id;
  Vec3 xyz;
};
struct Edge {
  std::int64_t n0;
  std::int64_t n1;
};
enum class ElemType : int { Tri3 = 2, Tet4 = 4 };
struct Element {
  std::int64_t id = 0;
  ElemType type = ElemType::Tet4;
  std::array<std::int64_t, 4> conn{};
  int phys = 0;
  std::array<int, 6> edges{};
  std::array<int, 6> edge_orient{};
};
struct Mesh {
  std::vector<Node> nodes;
  std::vector<Element> tets;
  std::vector<Element> tris;
  std::vector<Edge> edges;
  std::unordered_map<std::uint64_t, int> edgeIndex;
  std::unordered_map<std::int64_t, int> nodeIndex;
  // Monotonic id used to key device-resident caches (not in the reference).
  std::uint64_t uid = 0;
};

// include/edgefem/mesh.hpp:56-60
inline std::uint64_t make_edge_key(std::int64_t a, std::int64_t b) {
  if (a > b) std::swap(a, b);
  return (static_cast<std::uint64_t>(a) << 32) ^ static_cast<std::uint64_t>(b);
}

// src/mesh_gmsh.cpp:15-101 (throws std::runtime_error if unreadable)
Mesh load_gmsh_v2(const std::string &path);
// Build a mesh from plain arrays (what load_gmsh_v2 produces), numbering
// edges exactly like src/mesh_gmsh.cpp:104-147.
Mesh mesh_from_arrays(const std::int64_t *node_ids, const double *xyz, std::int64_t n_nodes,
                      const std::int64_t *tets, const std::int32_t *tet_phys, std::int64_t n_tets,
                      const std::int64_t *tris, const std::int32_t *tri_phys, std::int64_t n_tris);

// A copy of `mesh` with its edges and nodes renumbered in Z-order (Morton
// code) of their positions (edge midpoints, node coordinates), tets and
// triangles kept in order; edge_map receives old edge -> new edge.  Used
// inside the batched engine for gather locality (not in the reference).
Mesh locality_renumbered(const Mesh &mesh, std::vector<int> *edge_map);

// src/mesh_quality.cpp:52-83
struct MeshQualityReport {
  int num_degenerate_tets = 0;
  int num_inverted_tets = 0;
  double min_volume = 0;
  double max_aspect_ratio = 0;
  std::vector<int> bad_tet_indices;
  bool is_valid() const { return num_degenerate_tets == 0 && num_inverted_tets == 0; }
};
MeshQualityReport validate_mesh(const Mesh &mesh);

// --------------------------------------------------------------------- bc
// include/edgefem/bc.hpp:10-13, src/bc.cpp:47-80
struct BC {
  std::unordered_set<int> dirichlet_nodes;
  std::unordered_set<int> dirichlet_edges;
};
BC build_edge_pec(const Mesh &mesh, int pec_tag);

// ------------------------------------------------------------------ ports
// include/edgefem/ports/port_eigensolve.hpp:12-31
struct RectWaveguidePort {
  double a = 0;
  double b = 0;
};
enum class ModePolarization { TE, TM };
struct PortMode {
  ModePolarization pol = ModePolarization::TE;
  double fc = 0.0;
  double kc = 0.0;
  double omega = 0.0;
  cplx eps = 0.0;
  cplx mu = 0.0;
  cplx beta = 0.0;
  cplx Z0 = 0.0;
};
// include/edgefem/ports/wave_port.hpp:19-24
struct WavePort {
  int surface_tag = 0;
  PortMode mode;
  std::vector<int> edges;
  VecC weights;
};
// src/ports/port_eigensolve.cpp:45-65
PortMode solve_te10_mode(const RectWaveguidePort &port, double freq);
// src/ports/wave_port.cpp:410-514.  Eigenvector sign: the port-face integral
// of the mode field is positive along its dominant coordinate axis.
std::vector<double> solve_port_mode_2d(const Mesh &mesh, int surface_tag,
                                       const std::unordered_set<int> &pec_edges,
                                       double target_kc_sq, double &kc_sq_out);
// src/ports/wave_port.cpp:516-546
WavePort build_wave_port_2d(const Mesh &mesh, int surface_tag, const PortMode &mode,
                            const std::unordered_set<int> &pec_edges, double target_kc_sq);
// src/edge_basis.cpp:89-130, local edges (0,1),(1,2),(2,0)
std::array<double, 9> triangle_whitney_mass_matrix(const std::array<Vec3, 3> &v);
// src/edge_basis.cpp:48-87 (row-major 6x6)
void whitney_element_matrices(const std::array<Vec3, 4> &v, double K[36], double M[36]);

// include/edgefem/ports/lumped_port.hpp:24-29, src/ports/lumped_port.cpp:97-160
enum class LumpedPortWeightMode { SurfaceIntegral, Projection };
struct LumpedPortConfig {
  int surface_tag = 0;
  double z0 = 50.0;
  Vec3 e_direction{0, 0, 1};
  LumpedPortWeightMode weight_mode = LumpedPortWeightMode::SurfaceIntegral;
};
WavePort build_lumped_port(const Mesh &mesh, const LumpedPortConfig &config);

// -------------------------------------------------------------- materials
// include/edgefem/materials/dispersive.hpp:48-71 (Debye); the other models
// of that header are outside the accelerated path.
struct DebyeMaterial {
  double eps_s = 1, eps_inf = 1, tau = 1;
  cplx eval_eps(double omega) const { return eps_inf + (eps_s - eps_inf) / cplx(1.0, omega * tau); }
};

// ------------------------------------------------------------ parameters
// include/edgefem/maxwell.hpp:46-143 (PML fields omitted: out of the path)
struct MaxwellParams {
  double omega = 0.0;
  cplx eps_r = 1.0;
  cplx mu_r = 1.0;
  std::unordered_map<int, cplx> eps_r_regions;
  std::unordered_map<int, cplx> mu_r_regions;
  std::unordered_map<int, DebyeMaterial> eps_models;
  bool use_abc = false;
  // Legacy port ABC (include/edgefem/maxwell.hpp:36-82): a diagonal term on
  // every non-PEC port edge of the w w^H formulation; type 0 None, 1 Beta
  // (j beta, default), 2 BetaNorm (j beta/k0), 3 ImpedanceMatch
  // (j beta sqrt(Z0/eta0)), 4 ModalAdmittance (j omega eps0/Z0).
  bool use_port_abc = false;
  int port_abc_type = 1;
  std::unordered_set<int> abc_surface_tags;
  double port_abc_scale = 1.0;
  // Extension: per-tetrahedron complex permittivity (mesh.tets order).  When
  // non-empty it replaces the region lookup for every tetrahedron.
  VecC eps_r_tet;

  cplx get_eps_r(int phys_tag, double w) const {
    auto m = eps_models.find(phys_tag);
    if (m != eps_models.end()) return m->second.eval_eps(w);
    auto it = eps_r_regions.find(phys_tag);
    return it != eps_r_regions.end() ? it->second : eps_r;
  }
  cplx get_mu_r(int phys_tag, double) const {
    auto it = mu_r_regions.find(phys_tag);
    return it != mu_r_regions.end() ? it->second : mu_r;
  }
  cplx tet_eps(const Mesh &mesh, std::size_t t, double w) const {
    return eps_r_tet.empty() ? get_eps_r(mesh.tets[t].phys, w) : eps_r_tet[t];
  }
};

// ---------------------------------------------------------------- sparse
// Compressed sparse rows.  Matrices assembled here are structurally
// symmetric, so these arrays also equal the compressed-column arrays of the
// reference's column-major Eigen matrices.
struct MeshDev;
struct SpMatC {
  int rows = 0, cols = 0;
  std::vector<int> outer;   // size rows+1
  std::vector<int> inner;   // column indices, sorted within a row
  VecC values;
  // Mesh data of the matrices assemble_maxwell returns (the edge-node
  // incidence of their mesh): solve_linear uses it for the auxiliary-space
  // preconditioner.  Empty for matrices built from raw CSR arrays.
  std::shared_ptr<const MeshDev> origin;
  int nonZeros() const { return static_cast<int>(inner.size()); }
  cplx coeff(int r, int c) const;
  std::vector<VecC> to_dense() const;
};

struct MaxwellAssembly {
  SpMatC A;
  VecC b;
};

// -------------------------------------------------------------- solver
// include/edgefem/solver.hpp:16-55.  The iterative method runs on the GPU:
// complex-symmetric COCG (use_bicgstab=false) or BiCGStab (default), FP64.
// ILUT and SparseLU are not provided and there is no CPU fallback; with
// use_ilut (default) the preconditioner is the strongest one available for
// the matrix (see `preconditioner`), with use_ilut = false it is Jacobi,
// as the reference's diagonal-preconditioned BiCGSTAB.
using SolverProgressCallback = std::function<void(int, double)>;
struct SolveOptions {
  bool use_bicgstab = true;
  bool use_direct = false;
  double tolerance = 1e-10;
  int max_iterations = 10000;
  bool use_ilut = true;
  double ilut_fill_factor = 10.0;
  double ilut_drop_tolerance = 1e-4;
  bool auto_fallback = true;
  bool verbose = false;
  SolverProgressCallback progress_callback = nullptr;
  int progress_interval = 100;
  // 0: Jacobi; 1: Jacobi plus the nodal auxiliary-space (discrete gradient)
  // correction; 2: 1 plus the vector-nodal space; 3: block-Jacobi on
  // 16-row diagonal blocks.  1 and 2 need mesh data: the drivers have it,
  // and solve_linear has it for matrices from assemble_maxwell (SpMatC::
  // origin); on any other matrix solve_linear uses 3 in their place.
  int preconditioner = 2;
};
struct SolveResult {
  std::string method;
  int iters = 0;
  double residual = 0.0;
  bool converged = false;
  std::string error_message;
  VecC x;
};
SolveResult solve_linear(const SpMatC &A, const VecC &b, const SolveOptions &opt = SolveOptions());

// ----------------------------------------------------- maxwell drivers
// src/assemble_maxwell.cpp
MaxwellAssembly assemble_maxwell(const Mesh &mesh, const MaxwellParams &p, const BC &bc,
                                 const std::vector<WavePort> &ports, int active_port_idx = -1);
using MatC = std::vector<VecC>;  // dense row-major small matrix, S[row][col]
MatC calculate_sparams(const Mesh &mesh, const MaxwellParams &p, const BC &bc,
                       const std::vector<WavePort> &ports, const SolveOptions &opts = SolveOptions());
// Same; `solutions`, when given, receives the solution vector of each active
// port (empty for a port whose solve did not converge).
MatC calculate_sparams_opts(const Mesh &mesh, const MaxwellParams &p, const BC &bc,
                            const std::vector<WavePort> &ports, const SolveOptions &opts,
                            std::vector<VecC> *solutions);
void normalize_port_weights(const Mesh &mesh, const MaxwellParams &p, const BC &bc,
                            std::vector<WavePort> &ports, const SolveOptions &opts = SolveOptions());
MatC calculate_sparams_eigenmode(const Mesh &mesh, const MaxwellParams &p, const BC &bc,
                                 const std::vector<WavePort> &ports);
// Same with explicit solver options (the reference always uses defaults);
// `solutions`, when given, receives the solution vector of each active port.
MatC calculate_sparams_eigenmode_opts(const Mesh &mesh, const MaxwellParams &p, const BC &bc,
                                      const std::vector<WavePort> &ports, const SolveOptions &opts,
                                      std::vector<VecC> *solutions);

// src/sweep.cpp:82-172
struct KMMatrices {
  SpMatC K;
  SpMatC M;
  SpMatC combine(double omega) const;
};
KMMatrices assemble_maxwell_km(const Mesh &mesh, const MaxwellParams &p, const BC &bc);
struct SweepResult {
  std::vector<double> frequencies;
  std::vector<MatC> S_matrices;
};
// src/sweep.cpp:174-349
SweepResult frequency_sweep(const Mesh &mesh, const MaxwellParams &p, const BC &bc,
                            const std::vector<WavePort> &ports, const std::vector<double> &frequencies,
                            const SolveOptions &opts = SolveOptions());

// ------------------------------------------------------ field post-processing
// include/edgefem/edge_basis.hpp:36-57 and include/edgefem/io/vtk_export.hpp
using Vec3C = std::array<cplx, 3>;
std::array<double, 4> compute_barycentric(const std::array<Vec3, 4> &vertices, const Vec3 &point);
Vec3C evaluate_edge_field(const std::array<Vec3, 4> &vertices, const std::array<int, 6> &edge_orient,
                          const std::array<cplx, 6> &edge_dofs, const Vec3 &point);
// E of an edge solution at points (point i in tet tet_of[i]) / at every tet
// centroid, evaluated on the GPU.
std::vector<Vec3C> evaluate_field_at_points(const Mesh &mesh, const VecC &solution, const std::vector<int> &tet_of,
                                            const std::vector<Vec3> &points);
std::vector<Vec3C> evaluate_field_at_centroids(const Mesh &mesh, const VecC &solution);
struct VTKExportOptions {
  bool export_magnitude = true;
  bool export_phase = true;
  bool export_real = false;
  bool export_imag = false;
  bool export_vector = true;
};
void export_fields_vtk(const Mesh &mesh, const VecC &solution, const std::string &filename,
                       const VTKExportOptions &options = VTKExportOptions());
void export_fields_vtk_legacy(const Mesh &mesh, const VecC &solution, const std::string &filename,
                              const VTKExportOptions &options = VTKExportOptions());

// ------------------------------------------ network parameters, Touchstone
// include/edgefem/coupling.hpp:9-59 (src/coupling.cpp)
struct CouplingMatrix {
  MatC Z, Y, S;
  double frequency = 0;
  double z0 = 50.0;
  int num_ports = 0;
};
CouplingMatrix compute_coupling(const MatC &S, double freq, double z0 = 50.0);
std::vector<std::vector<double>> mutual_coupling_db(const CouplingMatrix &cm);
VecC active_reflection(const MatC &S, const VecC &excitation);
bool is_passive(const MatC &S, double tol = 1e-6);
bool is_lossless(const MatC &S, double tol = 1e-6);
bool is_reciprocal(const MatC &S, double tol = 1e-6);
// Singular values of a square S, largest first (eigenvalues of S^H S).
std::vector<double> singular_values(const MatC &S);
// pyedgefem.cpp:701-730: is_passive with a warning on stderr when violated.
bool check_passivity(const MatC &S, double tol = 1e-6);

// include/edgefem/io/touchstone.hpp:12-45 (src/io/touchstone.cpp)
enum class TouchstoneFormat { RI = 0, MA = 1, DB = 2 };
struct TouchstoneOptions {
  TouchstoneFormat format = TouchstoneFormat::RI;
  double z0 = 50.0;
};
// include/edgefem/ports/port_eigensolve.hpp:36-42
struct SParams2 {
  cplx s11, s21, s12, s22;
};
void write_touchstone(const std::string &path, const std::vector<double> &freq, const std::vector<SParams2> &data);
void write_touchstone_nport(const std::string &path, const std::vector<double> &freq,
                            const std::vector<MatC> &S_matrices, const TouchstoneOptions &opts = TouchstoneOptions());
std::string touchstone_extension(int num_ports);

// ------------------------------------------------------- chosen forms
// S-parameters of several mesh instances at several frequencies, solved
// together: block COCG over all (instance, frequency, port) right-hand sides
// in one batched launch sequence (double-float vectors by default), with
// true-residual confirmation and FP64 port-overlap extraction.
struct BatchOptions {
  double tolerance = 1e-8;      // relative FP64 residual ||b - A x|| / ||b||
  int max_iterations = 40000;
  int refine_interval = 0;      // 0: chosen by the autotuner
  int rows_per_block = 0;       // 0: chosen by the autotuner
  bool use_graph = true;
  bool verbose = false;
  // Bracket every SpMM launch of the solve with CUDA events (measurement).
  bool time_spmm = false;
  // Krylov arithmetic: 2 = double-float vectors with K and M applied in
  // double-float (default); 1 = double-float with M in FP32; 0 = complex64
  // vectors (FP32 recurrences restarted at each FP64 residual replacement).
  int precision = 2;
  // 0: eigenmode wave ports (calculate_sparams_eigenmode); 1: driven ports
  // in the w w^H / Z0 form with the jk0 absorbing boundary and Debye media
  // (calculate_sparams / frequency_sweep).
  int formulation = 0;
  // Add the vector-nodal auxiliary space (Hiptmair-Xu Pi term) to the
  // double-float engine's preconditioner (fewer iterations, a heavier node
  // pass).
  int vector_aux = 1;
  // Renumber each instance's edges and nodes in Z-order of their positions
  // inside the engine, so that consecutive rows (and the p rows and node
  // values they gather) are close in space.  S does not depend on it.  Off
  // by default: on the 40x20x100 slab guide it saves about 2% of the solve
  // and adds about 2 s of set-up (the pattern of the renumbered copy).
  int reorder = 0;
  // Reduced-basis initial guesses (double-float engine): with rb_samples > 0
  // and at least twice as many frequencies, the sweep first solves
  // rb_samples evenly spaced sample frequencies (capped at 64 / ports) to a
  // tenth of the tolerance, makes their solutions an orthonormal basis Q of
  // each instance, and starts every column from the Galerkin solution
  // x0 = Q (Q^T A(f) Q)^-1 Q^T b of its own A(f) and b.  Columns whose true
  // residual b - A x0 already meets the tolerance are done; the others
  // iterate from x0.  S and the tolerance are those of the cold solve.
  int rb_samples = 16;
};
struct BatchInstance {
  const Mesh *mesh = nullptr;
  MaxwellParams params;         // omega ignored
  const BC *bc = nullptr;
  std::vector<WavePort> ports;
};
struct BatchStats {
  std::vector<int> iterations;  // per (instance, frequency, port)
  std::vector<double> residual;
  std::vector<int> converged;
  double solve_ms = 0, setup_ms = 0;
  // reduced-basis phase (rb_samples): sample frequencies solved, basis
  // vectors kept per instance (smallest), columns done at their Galerkin
  // guess, milliseconds of basis and guess construction (host clock)
  int rb_samples = 0, rb_basis = 0, rb_done_at_guess = 0;
  double rb_ms = 0, rb_sample_ms = 0;  // + device time of the sample solve
  long long spmm_launches = 0;
  // summed SpMM launch time (time_spmm only) of the launches at the full
  // column width: the sample engine's when the reduced-basis phase is on
  // (the main engine is compacted to its few remaining columns at once)
  double spmm_ms = 0;
  long long spmm_timed = 0;      // launches in spmm_ms
  long long kernel_launches = 0; // all kernels of the solve
};

// Bytes copied host->device and device->host by this library so far.
void transfer_counters(long long *h2d, long long *d2h);
// S[instance][frequency] -> P x P matrix.  Non-converged columns are NaN.
std::vector<std::vector<MatC>> sparams_eigenmode_batched(const std::vector<BatchInstance> &inst,
                                                         const std::vector<double> &freqs,
                                                         const BatchOptions &opt, BatchStats *stats);

// d|S_ji|^2 / d eps_r(tet) for every tetrahedron (real permittivity change),
// from the forward eigenmode solve and its complex-symmetric adjoint.
std::vector<double> sparams_eigenmode_adjoint(const Mesh &mesh, const MaxwellParams &p, const BC &bc,
                                              const std::vector<WavePort> &ports, int out_j, int in_i,
                                              MatC *S_out, const SolveOptions &opts = SolveOptions());
// The same for the driven ports of calculate_sparams (lumped or wave ports
// with real weights, w w^T / Z0 port blocks, jk0 ABC, Debye media): no extra
// solve, the adjoint vector is a scaled forward solution.
std::vector<double> sparams_driven_adjoint(const Mesh &mesh, const MaxwellParams &p, const BC &bc,
                                           const std::vector<WavePort> &ports, int out_j, int in_i,
                                           MatC *S_out, const SolveOptions &opts = SolveOptions());

// Last CUDA/host error message of the calling thread (empty if none).
const std::string &last_error();
void set_last_error(const std::string &msg);

}  // namespace edgefem
