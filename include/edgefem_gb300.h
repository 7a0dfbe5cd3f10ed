/* Reference-facing C-ABI of edgefem-gb300 (libedgefem_gb300.so).
 *
 * Flat, FFI-friendly forms of jman4162/EdgeFEM's hot-path entry points
 * (C++ names in edgefem_gb300/csrc/edgefem.hpp).  Plain pointers and sizes
 * only; complex numbers are interleaved (re, im) doubles; matrices are
 * row-major.  All pointers are HOST pointers.  Return value: 0 = success,
 * < 0 = error (message from efg_last_error()), > 0 = number of solves that
 * did not converge (their S columns are NaN, as in the reference).
 * No C++ exception crosses this boundary.
 */
#ifndef EDGEFEM_GB300_H
#define EDGEFEM_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct efg_mesh_s *efg_mesh_t;
typedef struct efg_spmat_s *efg_spmat_t;

/* Error message of the last failing call on this thread ("" if none). */
const char *efg_last_error(void);
/* Library ABI version (increments on incompatible change). */
int efg_abi_version(void);
/* Number of CUDA devices visible (0 without a GPU); never fails. */
int efg_device_count(void);

/* ------------------------------------------------------------------ mesh */
/* Replaces load_gmsh_v2 + build_edges (src/mesh_gmsh.cpp:15-147,
 * include/edgefem/mesh.hpp:43-60): a mesh from plain arrays.  Node ids are
 * arbitrary int64; tets/tris reference node ids. */
int efg_mesh_create(const int64_t *node_ids, const double *xyz, int64_t n_nodes, const int64_t *tets,
                    const int32_t *tet_phys, int64_t n_tets, const int64_t *tris, const int32_t *tri_phys,
                    int64_t n_tris, efg_mesh_t *out);
/* load_gmsh_v2 (src/mesh_gmsh.cpp:15-101). */
int efg_mesh_load_gmsh_v2(const char *path, efg_mesh_t *out);
void efg_mesh_destroy(efg_mesh_t mesh);
int efg_mesh_sizes(efg_mesh_t mesh, int64_t *n_nodes, int64_t *n_tets, int64_t *n_tris, int64_t *n_edges);
/* Mesh arrays (any output pointer may be NULL). */
int efg_mesh_arrays(efg_mesh_t mesh, int64_t *node_ids, double *xyz, int64_t *tets, int32_t *tet_phys,
                    int64_t *tris, int32_t *tri_phys);
/* Edge numbering and orientation (Mesh::edges, Element::edges/edge_orient). */
int efg_mesh_topology(efg_mesh_t mesh, int64_t *edge_nodes, int32_t *tet_edges, int8_t *tet_orient,
                      int32_t *tri_edges, int8_t *tri_orient);
/* build_edges (src/mesh_gmsh.cpp:104-147) on the GPU: the same numbering
 * and orientations as efg_mesh_topology, from host arrays.  tet_nodes [4T]
 * and tri_nodes [3S] are dense node indices into node_ids [n_nodes].
 * edge_nodes needs room for 2 (6T + 3S) ids (the edge count is at most
 * 6T + 3S); it receives node ids, smaller first.  device_ms (may be NULL):
 * device time of the numbering kernels, host copies excluded. */
int efg_build_edges_gpu(int64_t n_nodes, const int64_t *node_ids, int64_t n_tets, const int32_t *tet_nodes,
                        int64_t n_tris, const int32_t *tri_nodes, int64_t *edge_nodes, int32_t *tet_edges,
                        int8_t *tet_orient, int32_t *tri_edges, int8_t *tri_orient, int64_t *n_edges,
                        double *device_ms);
/* validate_mesh (src/mesh_quality.cpp:52-83). */
int efg_validate_mesh(efg_mesh_t mesh, int32_t *num_degenerate, int32_t *num_inverted, double *min_volume,
                      double *max_aspect_ratio);
/* validate_mesh on the GPU: the same report, bit-identical, plus per tet
 * (tet_flag, host, may be NULL) 1 degenerate, 2 inverted, 0 otherwise
 * (the reference's bad_tet_indices, src/mesh_quality.cpp:71-77).
 * device_ms (may be NULL): device time of the quality kernels. */
int efg_validate_mesh_gpu(efg_mesh_t mesh, int32_t *num_degenerate, int32_t *num_inverted, double *min_volume,
                          double *max_aspect_ratio, int8_t *tet_flag, double *device_ms);

/* build_edge_pec (src/bc.cpp:47-80): sorted PEC edge ids.  Pass out=NULL to
 * query the count. */
int efg_build_edge_pec(efg_mesh_t mesh, int pec_tag, int32_t *out, int64_t capacity, int64_t *count);

/* Host-side CSR pattern of the assembled matrix (no dense port blocks) and
 * the number of tetrahedron colours; rowptr/colidx may be NULL to query. */
int efg_pattern(efg_mesh_t mesh, int32_t *rowptr, int32_t *colidx, int64_t *nnz, int32_t *n_colors);

/* Element kernels: whitney_curl_curl_matrix / whitney_mass_matrix
 * (src/edge_basis.cpp:48-87) for 4 vertices (12 doubles), row-major 6x6;
 * triangle_whitney_mass_matrix (:89-130) for 3 vertices, row-major 3x3. */
int efg_element_matrices(const double *xyz4, double *K36, double *M36);
int efg_triangle_mass(const double *xyz3, double *M9);

/* ----------------------------------------------------------------- ports */
typedef struct {
  double fc, kc, omega;
  double eps[2], mu[2], beta[2], Z0[2];
} efg_port_mode; /* PortMode, include/edgefem/ports/port_eigensolve.hpp:19-31 */

/* solve_te10_mode (src/ports/port_eigensolve.cpp:45-65). */
int efg_solve_te10_mode(double a, double b, double freq, efg_port_mode *out);

typedef struct {
  int32_t surface_tag;
  int64_t n_edges;
  const int32_t *edges;   /* global edge ids */
  double *weights;        /* complex, n_edges; written by efg_normalize_port_weights */
  efg_port_mode mode;
} efg_wave_port; /* WavePort, include/edgefem/ports/wave_port.hpp:19-24 */

/* build_wave_port_2d (src/ports/wave_port.cpp:516-546).  Writes up to
 * `capacity` edges/weights, the count, and the discrete cutoff kc.  Pass
 * edges_out=NULL to query the count. */
int efg_build_wave_port_2d(efg_mesh_t mesh, int surface_tag, const efg_port_mode *mode, const int32_t *pec,
                           int64_t n_pec, double target_kc_sq, int32_t *edges_out, double *weights_out,
                           int64_t capacity, int64_t *count, double *kc_out);
/* build_lumped_port (src/ports/lumped_port.cpp:97-160); weight_mode 0 =
 * SurfaceIntegral, 1 = Projection. */
int efg_build_lumped_port(efg_mesh_t mesh, int surface_tag, double z0, const double *e_dir3, int weight_mode,
                          int32_t *edges_out, double *weights_out, int64_t capacity, int64_t *count);

/* ------------------------------------------------------------ parameters */
typedef struct {
  double omega;
  double eps_r[2];
  double mu_r[2];
  int32_t n_eps_regions;
  const int32_t *eps_region_tags;
  const double *eps_region_vals; /* complex */
  int32_t n_mu_regions;
  const int32_t *mu_region_tags;
  const double *mu_region_vals;  /* complex */
  int32_t n_debye;
  const int32_t *debye_tags;
  const double *debye_params;    /* (eps_s, eps_inf, tau) per model */
  const double *eps_tet;         /* NULL, or complex per tetrahedron */
  int32_t use_abc;
  int32_t n_abc_tags;
  const int32_t *abc_tags;
  double port_abc_scale;
  int32_t use_port_abc;          /* legacy port ABC (maxwell.hpp:80-82) */
  int32_t port_abc_type;         /* 0 None, 1 Beta (default), 2 BetaNorm, 3 ImpedanceMatch,
                                    4 ModalAdmittance */
} efg_maxwell_params; /* MaxwellParams, include/edgefem/maxwell.hpp:46-143 */

typedef struct {
  int32_t use_bicgstab;
  int32_t use_direct;     /* accepted, no direct solver: the GPU iterative method runs */
  double tolerance;
  int32_t max_iterations;
  int32_t verbose;
  int32_t preconditioner; /* 0 Jacobi, 1 Jacobi + nodal gradient space, 2 (default) 1 + vector-nodal
                             space, 3 block-Jacobi (16-row diagonal blocks).  1 and 2 need mesh data:
                             the drivers have it, efg_solve_linear has it for matrices from
                             efg_assemble_maxwell and uses 3 in their place on other matrices */
  int32_t use_ilut;       /* 1 (default): the preconditioner above, the stand-in for the reference's
                             ILUT; 0: Jacobi, as the reference's BiCGSTAB without ILUT */
} efg_solve_options; /* SolveOptions, include/edgefem/solver.hpp:16-46 */

typedef struct {
  int32_t iters;
  double residual;
  int32_t converged;
  char method[64];
  char error_message[160];
} efg_solve_result; /* SolveResult, include/edgefem/solver.hpp:48-55 */

/* Fills the reference defaults (omega 0, eps_r = mu_r = 1, scale 1, ...). */
void efg_maxwell_params_default(efg_maxwell_params *p);
void efg_solve_options_default(efg_solve_options *o);

/* ---------------------------------------------------------- sparse matrix */
int efg_spmat_create(int32_t n, int64_t nnz, const int32_t *rowptr, const int32_t *colidx, const double *values,
                     efg_spmat_t *out);
int efg_spmat_info(efg_spmat_t A, int32_t *n, int64_t *nnz);
int efg_spmat_export(efg_spmat_t A, int32_t *rowptr, int32_t *colidx, double *values);
void efg_spmat_destroy(efg_spmat_t A);

/* ---------------------------------------------------------- entry points */
/* assemble_maxwell (src/assemble_maxwell.cpp:46-350): A (new handle) and b
 * (2n doubles). */
int efg_assemble_maxwell(efg_mesh_t mesh, const efg_maxwell_params *p, const int32_t *pec, int64_t n_pec,
                         const efg_wave_port *ports, int32_t n_ports, int32_t active_port, efg_spmat_t *A_out,
                         double *b_out);
/* solve_linear (src/solver.cpp:35-193) on the GPU; x_out: 2n doubles. */
int efg_solve_linear(efg_spmat_t A, const double *b, const efg_solve_options *opts, double *x_out,
                     efg_solve_result *result);
/* Allocation-free variant of efg_solve_linear's FP64 COCG with the Jacobi
 * preconditioner (no counterpart in the reference).  It is the Jacobi form
 * only: it agrees with efg_solve_linear run with preconditioner 0 (or
 * use_ilut 0), not with that call's default auxiliary-space or
 * block-Jacobi preconditioners, whose iteration counts differ widely.
 * For callers that cannot allocate device memory (a host whose device
 * memory is all owned by its own pool, or code that runs where cudaMalloc
 * is not allowed): it makes no cudaMalloc, cudaFree or other allocating
 * call.  Its work vectors live in a fixed file-scope device array sized
 * for EFG_NOALLOC_MAX_ROWS rows (8 MiB); larger n is rejected with an
 * error (-1, efg_last_error).
 * EXCEPTION to the host-pointer rule above: rowptr/colidx (int32 CSR of an
 * n x n matrix, every row holding its diagonal: a row without one is
 * rejected with an error), vals (nnz complex), b and x (n complex) are
 * DEVICE pointers on the current device; stream is a cudaStream_t (NULL =
 * default stream).  x is overwritten (starts at 0).
 * The call returns when the solve has finished: 0 converged, 1 not
 * converged, < 0 error; iterations/residual/converged may be NULL.
 * Every call looks up the array's address on the current device (nothing
 * is cached across a context reset); the first lookup on a device may load
 * the module holding the array: make the first call before any stream
 * capture there.  Calls that overlap on one device share the array and
 * race: serialise them. */
#define EFG_NOALLOC_MAX_ROWS 131072
int efg_solve_linear_device_noalloc(int32_t n, const int32_t *rowptr, const int32_t *colidx, const double *vals,
                                    const double *b, double *x, double tolerance, int32_t max_iterations,
                                    void *stream, int32_t *iterations, double *residual, int32_t *converged);
/* calculate_sparams (src/assemble_maxwell.cpp:352-394); S_out: P*P complex. */
int efg_calculate_sparams(efg_mesh_t mesh, const efg_maxwell_params *p, const int32_t *pec, int64_t n_pec,
                          const efg_wave_port *ports, int32_t n_ports, const efg_solve_options *opts,
                          double *S_out);
/* normalize_port_weights (src/assemble_maxwell.cpp:396-494): rescales each
 * port's weights array in place. */
int efg_normalize_port_weights(efg_mesh_t mesh, const efg_maxwell_params *p, const int32_t *pec, int64_t n_pec,
                               efg_wave_port *ports, int32_t n_ports, const efg_solve_options *opts);
/* calculate_sparams_eigenmode (src/assemble_maxwell.cpp:637-787), the plain
 * unbatched FP64 GPU solve.  opts may be NULL (COCG, tol 1e-10). */
int efg_calculate_sparams_eigenmode(efg_mesh_t mesh, const efg_maxwell_params *p, const int32_t *pec,
                                    int64_t n_pec, const efg_wave_port *ports, int32_t n_ports,
                                    const efg_solve_options *opts, double *S_out, efg_solve_result *stats);
/* assemble_maxwell_km (src/sweep.cpp:90-172): two new handles. */
int efg_assemble_maxwell_km(efg_mesh_t mesh, const efg_maxwell_params *p, const int32_t *pec, int64_t n_pec,
                            efg_spmat_t *K_out, efg_spmat_t *M_out);
/* frequency_sweep (src/sweep.cpp:174-349); S_out: nf*P*P complex. */
int efg_frequency_sweep(efg_mesh_t mesh, const efg_maxwell_params *p, const int32_t *pec, int64_t n_pec,
                        const efg_wave_port *ports, int32_t n_ports, const double *freqs, int32_t n_freqs,
                        const efg_solve_options *opts, double *S_out);

/* ------------------------------------------------------------ chosen forms */
typedef struct {
  efg_mesh_t mesh;
  efg_maxwell_params params; /* omega ignored */
  const int32_t *pec;
  int64_t n_pec;
  const efg_wave_port *ports;
  int32_t n_ports;
} efg_batch_instance;

typedef struct {
  double tolerance;        /* relative FP64 residual, default 1e-8 */
  int32_t max_iterations;  /* default 40000 */
  int32_t refine_interval; /* FP64 residual-replacement period, 0 = auto */
  int32_t rows_per_block;  /* 0 = auto */
  int32_t use_graph;       /* 1 = CUDA graphs (default) */
  int32_t verbose;
  int32_t time_spmm;       /* 1 = CUDA-event timing of every SpMM launch */
  int32_t precision;       /* 2 = double-float K and M (default), 1 = double-float K, FP32 M,
                              0 = complex64 vectors */
  int32_t formulation;     /* 0 = eigenmode wave ports (calculate_sparams_eigenmode);
                              1 = driven ports in the w w^H/Z0 form with the jk0 ABC and
                              Debye media (calculate_sparams / frequency_sweep) */
  int32_t vector_aux;      /* 1 = add the vector-nodal (Pi) auxiliary space to the
                              double-float preconditioner (default), 0 = gradient space only */
  int32_t reorder;         /* 1 = renumber edges and nodes in Z-order of their positions inside
                              the engine, for gather locality; 0 = mesh order (default) */
  int32_t rb_samples;      /* reduced-basis initial guesses (double-float engine): sample
                              frequencies, default 16, 0 = off, capped at 64 / ports.  With at
                              least twice as many frequencies, that many evenly spaced sample
                              frequencies are solved first (to a tenth of the tolerance); every
                              column then starts from the Galerkin solution of its own A(f) x = b
                              on the orthonormalised sample solutions and iterates only if its
                              true residual there is above the tolerance.  No reference
                              counterpart (the reference solves each frequency from zero,
                              src/sweep.cpp:249-329). */
} efg_batch_options;

typedef struct {
  double solve_ms;         /* device time of the solve (CUDA events) */
  double setup_ms;
  int32_t max_iters;
  int32_t min_iters;
  int32_t n_converged;
  int32_t n_total;
  double max_residual;
  int64_t spmm_launches;
  double spmm_ms;          /* summed SpMM launch time when time_spmm = 1, launches at the full
                              column width only: the sample engine's (rb_samples x ports
                              columns, rounded up to a power of two) when rb_samples > 0 */
  int64_t spmm_timed;
  int64_t kernel_launches; /* kernels launched by the solve */
  int32_t rb_samples;      /* reduced-basis phase: sample frequencies solved (0 = off) */
  int32_t rb_basis;        /* basis vectors kept (smallest over instances) */
  int32_t rb_done_at_guess;/* columns whose Galerkin guess already met the tolerance */
  int32_t rb_reserved;
  double rb_ms;            /* host time of basis and guess construction */
  double rb_sample_ms;     /* device time of the sample-frequency solve */
} efg_batch_stats;

/* Plain-path Krylov totals of this thread since the last reset: iterations,
 * solves, largest final residual, device milliseconds (any output may be
 * NULL); reset != 0 zeroes them after reading.  No reference counterpart:
 * the reference's drivers report per-solve SolveResult only. */
void efg_krylov_totals(int32_t reset, int64_t *iters, int32_t *solves, double *max_residual, double *device_ms);
/* Bytes this library has copied host->device and device->host so far. */
void efg_transfer_counters(int64_t *h2d, int64_t *d2h);

void efg_batch_options_default(efg_batch_options *o);

/* Eigenmode S-parameters of n_inst meshes at n_freqs frequencies in one
 * batched complex64 COCG with FP64 residual replacement.  Every instance
 * must have the same number of ports P.  S_out: n_inst*n_freqs*P*P complex
 * ([inst][freq][row][col]).  No reference counterpart (the reference loops
 * calculate_sparams_eigenmode per frequency, waveguide.py:423-434). */
int efg_sparams_eigenmode_batched(const efg_batch_instance *inst, int32_t n_inst, const double *freqs,
                                  int32_t n_freqs, const efg_batch_options *opts, double *S_out,
                                  efg_batch_stats *stats);

/* frequency_sweep (src/sweep.cpp:174-349) as one batched solve: every
 * frequency x active port of the driven-port (w w^H / Z0) system, with the
 * jk0 ABC and a Debye material, in the double-float engine.  Same arguments
 * and S layout as efg_frequency_sweep (S_out: n_freqs*P*P complex);
 * formulation is forced to 1.  Non-converged columns are NaN. */
int efg_frequency_sweep_batched(efg_mesh_t mesh, const efg_maxwell_params *p, const int32_t *pec, int64_t n_pec,
                                const efg_wave_port *ports, int32_t n_ports, const double *freqs,
                                int32_t n_freqs, const efg_batch_options *opts, double *S_out,
                                efg_batch_stats *stats);

/* The same solve split in two: efg_batch_create does all set-up (pattern,
 * FP64 assembly packed to the solve's operator arrays, port tables, autotuned
 * chunking) and leaves it resident on the GPU; efg_batch_solve runs one full
 * solve from x = 0 (callable repeatedly).  The instances' meshes must outlive
 * the handle only during efg_batch_create. */
typedef struct efg_batch_s *efg_batch_t;
int efg_batch_create(const efg_batch_instance *inst, int32_t n_inst, const double *freqs, int32_t n_freqs,
                     const efg_batch_options *opts, efg_batch_t *out);
int efg_batch_solve(efg_batch_t h, double *S_out, efg_batch_stats *stats);
/* rows, nonzeros, right-hand sides per row, rows per chunk chosen by the autotuner */
int efg_batch_info(efg_batch_t h, int64_t *rows, int64_t *nnz, int32_t *rhs, int32_t *rows_per_chunk);
void efg_batch_destroy(efg_batch_t h);
/* Per (instance, rhs) outcome of the last efg_batch_solve, index b*R + rhs
 * with R from efg_batch_info: status (1 converged, 2 breakdown, 3 max
 * iterations, 4 padding), iterations, relative FP64 residual. */
int efg_batch_rhs_stats(efg_batch_t h, int32_t *status, int32_t *iters, double *residual);

/* d|S_ji|^2 / d eps_r for every tetrahedron (grad_out: n_tets doubles) and
 * the S matrix (P*P complex).  No reference counterpart. */
int efg_sparams_eigenmode_adjoint(efg_mesh_t mesh, const efg_maxwell_params *p, const int32_t *pec,
                                  int64_t n_pec, const efg_wave_port *ports, int32_t n_ports, int32_t out_j,
                                  int32_t in_i, const efg_solve_options *opts, double *grad_out, double *S_out);
/* The same for the driven ports of calculate_sparams (w w^T / Z0 port
 * blocks, jk0 ABC, Debye media; real port weights): d|S_ji|^2 / d eps_r
 * per tetrahedron from the forward solves alone (the adjoint vector of a
 * driven port is its scaled forward solution).  No reference counterpart;
 * it differentiates src/assemble_maxwell.cpp:352-394. */
int efg_sparams_driven_adjoint(efg_mesh_t mesh, const efg_maxwell_params *p, const int32_t *pec, int64_t n_pec,
                               const efg_wave_port *ports, int32_t n_ports, int32_t out_j, int32_t in_i,
                               const efg_solve_options *opts, double *grad_out, double *S_out);

/* ----------------------------------------------------- field post-processing
 * Fields are [n][3] complex (6 doubles per point); x is the edge solution
 * (one complex value per mesh edge). */
/* compute_barycentric (src/edge_basis.cpp:131-151): vertices 4 x 3, lambda 4
 * (host arithmetic on one tetrahedron). */
int efg_compute_barycentric(const double *vertices, const double *point, double *lambda);
/* evaluate_edge_field (src/edge_basis.cpp:162-193) at one point of one
 * tetrahedron: vertices 4 x 3, edge_orient 6 (+1/-1), edge_dofs 6 complex. */
int efg_evaluate_edge_field(const double *vertices, const int32_t *edge_orient, const double *edge_dofs,
                            const double *point, double *E);
/* The same on the GPU for many points: point i lies in tet tet_of[i];
 * with tet_of and points both NULL, E at every tet centroid (n_points
 * ignored, E holds num_tets points).  No single reference function: the
 * field loop of src/io/vtk_export.cpp:52-64. */
int efg_evaluate_field(efg_mesh_t mesh, const double *x, int64_t n_points, const int32_t *tet_of,
                       const double *points, double *E);
/* VTKExportOptions (include/edgefem/io/vtk_export.hpp:10-26). */
typedef struct {
  int32_t export_magnitude, export_phase, export_real, export_imag, export_vector;
} efg_vtk_options;
void efg_vtk_options_default(efg_vtk_options *opts);
/* export_fields_vtk (src/io/vtk_export.cpp:44-200, .vtu) or, with legacy != 0,
 * export_fields_vtk_legacy (:202-272, .vtk); opts may be NULL (defaults). */
int efg_export_fields_vtk(efg_mesh_t mesh, const double *x, const char *path, const efg_vtk_options *opts,
                          int32_t legacy);

/* ------------------------------------------ network parameters, Touchstone
 * Square S matrices of n ports, row-major complex (2 n^2 doubles). */
/* compute_coupling (src/coupling.cpp:9-50): Z = z0 (I+S)(I-S)^-1 and
 * Y = (I-S)(I+S)^-1 / z0, a singular factor regularised by 1e-12 I; Z or Y
 * may be NULL. */
int efg_compute_coupling(int32_t n, const double *S, double freq, double z0, double *Z, double *Y);
/* mutual_coupling_db (src/coupling.cpp:52-65): 20 log10 max(|S_ij|, 1e-20), n x n doubles. */
int efg_mutual_coupling_db(int32_t n, const double *S, double *db);
/* active_reflection (src/coupling.cpp:67-94): (S a)_i / a_i, 0 where |a_i| < 1e-20. */
int efg_active_reflection(int32_t n, const double *S, const double *excitation, double *gamma);
/* is_passive / is_lossless / is_reciprocal (src/coupling.cpp:96-136) and
 * check_passivity (python/pyedgefem.cpp:701-730, warns on stderr):
 * 1 true, 0 false, < 0 error. */
int efg_is_passive(int32_t n, const double *S, double tol);
int efg_check_passivity(int32_t n, const double *S, double tol);
int efg_is_lossless(int32_t n, const double *S, double tol);
int efg_is_reciprocal(int32_t n, const double *S, double tol);
/* Singular values of S, largest first (n doubles); no counterpart in the
 * reference (it calls Eigen's JacobiSVD inside is_passive). */
int efg_singular_values(int32_t n, const double *S, double *sv);
/* write_touchstone_nport (src/io/touchstone.cpp:64-139): S is
 * [n_freq][num_ports][num_ports] complex; format 0 RI, 1 MA, 2 DB. */
int efg_write_touchstone_nport(const char *path, int32_t n_freq, const double *freq, int32_t num_ports,
                               const double *S, int32_t format, double z0);
/* write_touchstone (src/io/touchstone.cpp:48-60), 2-port legacy form: s2 is
 * [n_freq][4] complex in the order s11, s21, s12, s22. */
int efg_write_touchstone(const char *path, int32_t n_freq, const double *freq, const double *s2);
/* touchstone_extension (src/io/touchstone.cpp:141-149): ".s<N>p" into buf. */
int efg_touchstone_extension(int32_t num_ports, char *buf, int32_t buf_len);

#ifdef __cplusplus
}
#endif
#endif
