/* Kernel-level C-ABI of edgefem-gb300: the thin layer between the C++ host
 * library and the sm_103a kernels.  Every pointer argument is a DEVICE
 * pointer unless its comment says "host"; complex numbers are interleaved
 * (re, im) pairs.  Every function enqueues work on `stream` and returns a
 * cudaError_t value cast to int (0 = success); none allocates memory.
 *
 * These entry points have no reference counterpart one by one: together they
 * replace the Eigen-based assembly and solve of jman4162/EdgeFEM
 * (src/assemble_maxwell.cpp:114-347, src/solver.cpp:35-193,
 * src/sweep.cpp:82-329).
 */
#ifndef EDGEFEM_GB300_KERNELS_H
#define EDGEFEM_GB300_KERNELS_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct CUstream_st *efgk_stream_t;

/* ---------------------------------------------------------------- assembly
 * One colour of the tetrahedron scatter (src/assemble_maxwell.cpp:114-204,
 * src/edge_basis.cpp:14-87).  For tets color_tets[begin..end): forms the 6x6
 * Whitney curl-curl K and mass M blocks from FP64 node coordinates and adds
 * s_i s_j (cK[t] K_ij + cM[t] M_ij) at out[slots[36 t + 6 i + j]].  cK/cM are
 * complex per tet; a NULL array means the uniform value cK0/cM0 (host). */
int efgk_assemble_color(const double *xyz, const int32_t *tet_nodes, const uint8_t *tet_signs,
                        const int32_t *slots, const int32_t *color_tets, int64_t begin, int64_t end,
                        const double *cK, const double *cM, const double *cK0_host,
                        const double *cM0_host, double *out, efgk_stream_t stream);

/* Adjoint sensitivity contraction (no reference counterpart): for every tet,
 * out[t] = scale * sum_ij (s_i lam[e_i]) M_ij (s_j x[e_j]) with the FP64 mass
 * block M recomputed from the node coordinates; lam, x, out complex. */
int efgk_adjoint_contract(int32_t T, const double *xyz, const int32_t *tet_nodes, const uint8_t *tet_signs,
                          const int32_t *tet_edges, const double *lam, const double *x, double scale,
                          double *out, efgk_stream_t stream);

/* Electric field from an edge solution x (complex, one value per edge) at
 * nq query points, evaluate_edge_field (src/edge_basis.cpp:162-193) per
 * point: point q lies in tet tet_of[q] (tet q when tet_of is NULL) at
 * pts[3q..3q+2] (the tet's centroid when pts is NULL); E is [nq][3] complex.
 * tet_nodes are 0-based node indices into xyz, tet_signs bit i set when
 * local edge i runs against its global orientation. */
int efgk_edge_field(int64_t nq, const double *xyz, const int32_t *tet_nodes, const uint8_t *tet_signs,
                    const int32_t *tet_edges, const int32_t *tet_of, const double *pts, const double *x,
                    double *E, efgk_stream_t stream);

/* Dirichlet rows/columns (src/assemble_maxwell.cpp:322-347): entries in a PEC
 * row or PEC column become 0, the diagonal of a PEC row becomes diag_value. */
int efgk_dirichlet(int32_t n, const int32_t *rowptr, const int32_t *colidx, const uint8_t *is_pec,
                   double diag_re, double diag_im, double *values, efgk_stream_t stream);

/* values[slot[k]] += coef[term[k]] * val[k] for k < count (port and ABC
 * terms, src/assemble_maxwell.cpp:212-265, 738-746).  coef is complex,
 * val is complex. */
int efgk_add_terms(int64_t count, const int32_t *slot, const int32_t *term, const double *val,
                   const double *coef, double *values, efgk_stream_t stream);

/* out = a*K + b*M (+ c*M2 if M2 != NULL) over nnz complex values; a, b, c host. */
int efgk_blend(int64_t nnz, const double *K, const double *M, const double *M2, const double *a_host,
               const double *b_host, const double *c_host, double *out, efgk_stream_t stream);

/* --------------------------------------------------------- FP64 Krylov (plain)
 * `sc` is the device scalar block of one solve (layout in
 * edgefem_gb300/csrc/sc_layout.h).
 *
 * Auxiliary-space (nodal gradient) preconditioner data, all device arrays:
 * enodes[2e], enodes[2e+1] = tail and head node index of edge e, or -1, -1
 * for a PEC edge; nptr/nedge/nsign = per node its incident non-PEC edges
 * and the incidence sign (+1 head, -1 tail); dninv = 1/diag(G^T A G) per
 * node (complex); t = complex work vector of nn entries.  With npi = 3
 * the vector-nodal space is added: piw = per edge (x_head - x_tail)/2 (3
 * doubles), dpinv = omega / diag(Pi^T A Pi) per (node, component) (complex,
 * 3 nn), tp = complex work vector of 3 nn entries.  A NULL EfgkAux selects
 * the Jacobi preconditioner alone.
 *
 * Block-Jacobi instead (bj_bs > 0, nn = 0, the preconditioner for a CSR
 * matrix without mesh data): bj_inv = the inverses of the diagonal blocks
 * of bj_bs consecutive rows (efgk_bjacobi_setup64), z = complex work vector
 * of n entries.  Zero-initialised fields select neither. */
struct EfgkAux {
  const int32_t *enodes;
  const int32_t *nptr;
  const int32_t *nedge;
  const int8_t *nsign;
  const double *dninv;
  double *t;
  int32_t nn;
  int32_t npi;
  const double *piw;
  const double *dpinv;
  double *tp;
  const double *bj_inv;
  double *z;
  int32_t bj_bs;
};
/* Block size of the block-Jacobi preconditioner and the size in doubles of
 * its inverse array for n rows: EFGK_BJ_BS x EFGK_BJ_BS complex per block of
 * EFGK_BJ_BS rows (the last block padded with identity rows). */
#define EFGK_BJ_BS 16
#define EFGK_BJ_DOUBLES(n) (2LL * EFGK_BJ_BS * EFGK_BJ_BS * (((long long)(n) + EFGK_BJ_BS - 1) / EFGK_BJ_BS))
/* Inverses of the EFGK_BJ_BS x EFGK_BJ_BS diagonal blocks of the complex
 * CSR matrix (sorted columns), by Gauss-Jordan elimination with partial
 * pivoting in FP64, stored column-major per block (binv[blk][col][row]).  A
 * block with a zero pivot falls back to the inverse of its diagonal (ones
 * where that is zero) and counts in *nsingular (device int, added to). */
int efgk_bjacobi_setup64(int32_t n, const int32_t *rowptr, const int32_t *colidx, const double *vals, double *binv,
                         int32_t *nsingular, efgk_stream_t stream);
int efgk_spmv64(int32_t n, const int32_t *rowptr, const int32_t *colidx, const double *vals,
                const double *x, double *y, efgk_stream_t stream);
/* y = A x with A, x, y complex64 (interleaved floats) and FP32 accumulation:
 * the operator product of an FP32 Krylov iteration on the same CSR pattern
 * (the complex FP32 form of the Eigen SpMV inside BiCGSTAB,
 * src/solver.cpp:54-99).  Runs on the FP32 pipes at HBM rate; the FP64
 * product above is bound by GB300's FP64 pipe. */
int efgk_spmv32(int32_t n, const int32_t *rowptr, const int32_t *colidx, const float *vals,
                const float *x, float *y, efgk_stream_t stream);
/* The same complex64 product with the matrix streamed through shared
 * memory by bulk asynchronous copies (cp.async.bulk into two stages per
 * CTA, mbarrier completion): nnz = rowptr[n]; colidx and vals must be
 * 16-byte aligned (cudaErrorMisalignedAddress otherwise).  status is a
 * device int the caller zeroes: set to 1 if a copy never completed (the
 * kernel's waits are bounded). */
int efgk_spmv32_bulk(int32_t n, int32_t nnz, const int32_t *rowptr, const int32_t *colidx, const float *vals,
                     const float *x, float *y, int32_t *status, efgk_stream_t stream);
/* The same complex64 product on a sliced-ELLPACK copy (slices of 32 rows,
 * rows sorted by decreasing length inside windows of 1024 rows, entries of
 * a slice column-major, padded with zeros): every warp load of the matrix
 * is one contiguous line.  Build the copy once: efgk_sell32_plan fills perm
 * (n int32, the row at each sorted position) and slice_ptr ((n + 31) / 32 +
 * 1 int64 entry offsets) and returns the padded entry count in *entries
 * (host; the call synchronises the stream); allocate that many int32
 * columns and complex64 values and call efgk_sell32_fill.  rowptr, colidx,
 * vals, perm, slice_ptr, sell_col, sell_val, x, y are device pointers. */
int efgk_sell32_plan(int32_t n, const int32_t *rowptr, int32_t *perm, int64_t *slice_ptr, int64_t *entries,
                     efgk_stream_t stream);
int efgk_sell32_fill(int32_t n, const int32_t *rowptr, const int32_t *colidx, const float *vals,
                     const int32_t *perm, const int64_t *slice_ptr, int32_t *sell_col, float *sell_val,
                     efgk_stream_t stream);
int efgk_spmv32_sell(int32_t n, const int32_t *perm, const int64_t *slice_ptr, const int32_t *sell_col,
                     const float *sell_val, const float *x, float *y, efgk_stream_t stream);
/* dn += diag(G^T A G) (complex, nn entries; zero it first). */
int efgk_aux_diag64(int32_t n, const int32_t *rowptr, const int32_t *colidx, const double *vals,
                    const int32_t *enodes, double *dn, efgk_stream_t stream);
/* dp += scale * diag(Pi^T A Pi) (complex, 3 nn entries [node][component];
 * zero it first); piw: 3 weights per edge. */
int efgk_aux_pi_diag64(int32_t n, const int32_t *rowptr, const int32_t *colidx, const double *vals,
                       const int32_t *enodes, const double *piw, double scale, double *dp, efgk_stream_t stream);
/* dninv = 1/dn where |dn| > rel_floor * max|dn|, else 0; scratch: 1 double. */
int efgk_aux_recip64(int32_t nn, const double *dn, double rel_floor, double *scratch, double *dninv,
                     efgk_stream_t stream);
int efgk_cocg64_init(int32_t n, const double *b, const double *dinv, double *x, double *r, double *p,
                     double *sc, const struct EfgkAux *aux, efgk_stream_t stream);
int efgk_cocg64_step(int32_t n, const int32_t *rowptr, const int32_t *colidx, const double *vals,
                     const double *dinv, double *x, double *r, double *p, double *q, double *sc,
                     int parity, const struct EfgkAux *aux, efgk_stream_t stream);
int efgk_bicgstab64_init(int32_t n, const double *b, double *x, double *r, double *rhat, double *p,
                         double *v, double *sc, efgk_stream_t stream);
int efgk_bicgstab64_step(int32_t n, const int32_t *rowptr, const int32_t *colidx, const double *vals,
                         const double *dinv, double *x, double *r, const double *rhat, double *p,
                         double *v, double *s, double *t, double *phat, double *shat, double *sc,
                         const struct EfgkAux *aux, efgk_stream_t stream);
int efgk_diag_inverse64(int32_t n, const int32_t *diag_slot, const double *vals, double *dinv,
                        efgk_stream_t stream);
/* dot[k] = sum_i c[k][i] * x[idx[k][i]] (unconjugated) over small port lists:
 * offsets[k]..offsets[k+1] index into idx/c.  out: complex per list. */
int efgk_port_overlaps64(int32_t nlists, const int32_t *offsets, const int32_t *idx, const double *c,
                         const double *x, int64_t x_stride, double *out, efgk_stream_t stream);

/* ------------------------------------------------------- batched FP32 engine
 * `bt` is a HOST pointer to a struct EfgkBatch (edgefem_gb300/csrc/
 * batch_layout.h) whose array members are device pointers; it is passed to
 * the kernels by value.  Parity = iteration & 1. */
struct EfgkBatch;
/* q = A(f) p for every right-hand side, with p^T q per (instance, rhs). */
int efgk_batch_spmm(const struct EfgkBatch *bt, int parity, efgk_stream_t stream);
/* The same SpMM with an explicit grid size and right-hand sides per lane
 * (1, 2 or 4; 0 = R/32), as chosen by the autotuner. */
int efgk_batch_spmm_grid(const struct EfgkBatch *bt, int parity, int grid_blocks, int rhs_per_lane,
                         efgk_stream_t stream);
/* x_c += alpha p, r -= alpha q, |r|^2, r^T D^-1 r; then the node pass
 * t = Dn^-1 G^T r adding s^T t (rho' complete). */
int efgk_batch_update(const struct EfgkBatch *bt, int parity, efgk_stream_t stream);
/* Residual-replacement checkpoint after `iters_done` more iterations: flag
 * right-hand sides whose |r| fell by delta (or below tol), and for them
 * x64 += x_c, r = b - A x64 in FP64, recompute rho' and |r|^2, decide
 * convergence on that true residual; stop at max_iters. */
int efgk_batch_checkpoint(const struct EfgkBatch *bt, int parity, int iters_done, efgk_stream_t stream);
/* p = D^-1 r + G t + beta p.  Bit 1 of `parity`: a checkpoint ran in this
 * iteration, and right-hand sides whose residual it replaced restart with
 * beta = 0. */
int efgk_batch_pupdate(const struct EfgkBatch *bt, int parity, efgk_stream_t stream);
/* r = b, |b|^2, t, p = D^-1 r + G t, status (x64 = x_c = t = 0 and the
 * accumulators zeroed beforehand). */
int efgk_batch_init(const struct EfgkBatch *bt, efgk_stream_t stream);
/* x64 += x_c and the port overlaps S_acc[b][j][rhs] = e_j^H Ms_j x. */
int efgk_batch_finish(const struct EfgkBatch *bt, efgk_stream_t stream);
/* One instance's FP64 assembled K, M (complex, nnz) -> packed nonzeros
 * {col + col_off, K, M} (FP32), global column indices, K64 real, M64 complex. */
int efgk_batch_pack(int64_t nnz, const int32_t *col_local, int32_t col_off, const double *K, const double *M,
                    void *nz, int32_t *colidx, double *K64, double *M64, efgk_stream_t stream);
/* Diagonals of K and M (via the diagonal slots) in FP32. */
int efgk_batch_diag(int32_t n, const int32_t *diag_slot, const double *K64, const double *M64, float *kd32,
                    float *md32, efgk_stream_t stream);

/* Double-float form of the batched engine (vectors xd, rd, pd, qd, td and
 * the operator's low words nzlo of struct EfgkBatch).  Same phases and
 * parity convention as the complex64 form above.  m_mode 1 applies M with
 * its low words in double-float, 0 in FP32 on the high words, 2 as 1 with
 * K - k0^2 M formed once per frequency for port pairs (becomes 3 when P or
 * rhs_per_lane is odd), 3 as 2 with the coefficient formed per right-hand
 * side; + 16: tile-major work order (the grid sweeps the rows once per
 * column tile); grid_blocks and rhs_per_lane 0 pick defaults.  pupdate: bit 1 of parity restarts the
 * directions of right-hand sides whose residual was just replaced. */
int efgk_batch_dd_spmm(const struct EfgkBatch *bt, int parity, int grid_blocks, int rhs_per_lane, int m_mode,
                       efgk_stream_t stream);
int efgk_batch_dd_update(const struct EfgkBatch *bt, int parity, efgk_stream_t stream);
int efgk_batch_dd_checkpoint(const struct EfgkBatch *bt, int parity, int iters_done, efgk_stream_t stream);
int efgk_batch_dd_pupdate(const struct EfgkBatch *bt, int parity, efgk_stream_t stream);
int efgk_batch_dd_init(const struct EfgkBatch *bt, efgk_stream_t stream);
int efgk_batch_dd_finish(const struct EfgkBatch *bt, efgk_stream_t stream);
/* out[row][c] = in[row][map[c]] (zero where map[c] < 0) for complex dd
 * ([rows][r_old] -> [rows][r_new] float4 arrays; in and out must not
 * overlap): repacks the running right-hand-side columns of a batch. */
int efgk_batch_gather_cols(int64_t rows, int32_t r_old, int32_t r_new, const int32_t *map, const void *in,
                           void *out, efgk_stream_t stream);
/* out[row][map[c]] = in[row][c] for c < r_in with map[c] >= 0 (complex dd,
 * [rows][r_in] -> [rows][r_out]); the other columns of out are kept. */
int efgk_batch_scatter_cols(int64_t rows, int32_t r_in, int32_t r_out, const int32_t *map, const void *in,
                            void *out, efgk_stream_t stream);

/* Reduced-basis initial guesses of a sweep (kernels_rb.cu), complex FP64
 * vectors (double2) of one instance's n edge rows; Q and W row-major
 * [n][ld], k <= 128 columns in use (k <= 64 for efgk_rb_gram).
 * load_col: v = x[row0 + i][col] (complex dd [rows][r] source), |v|^2 added
 *   to *nrm.
 * orth_step: h = Q[:, :k]^H v (h: k complex, zeroed here), v -= Q h.
 * norm2: |v|^2 added to *nrm.  set_col: Q[:, j] = scale v.
 * apply: W[:, :k] = A Q[:, :k] for A = K (kind 0, real nnz doubles),
 *   M (1, complex) or M_D (2, real) on the engine's CSR rows row0 .. row0+n.
 * gram: G = Q[:, :k]^T W[:, :k] (k x k complex, no conjugate; zeroed here).
 * combine: x[row0 + i][c] = sum_t Q[i][t] Y[t][c] for c < r, Y k x r complex
 *   row-major, written as complex dd into the [rows][r] x.
 * gather_rows: out[i][t] = Q[idx[i]][t] for i < m, t < k. */
int efgk_rb_load_col(int64_t n, const void *x, int32_t r, int64_t row0, int32_t col, double *v, double *nrm,
                     efgk_stream_t stream);
int efgk_rb_orth_step(int64_t n, const double *Q, int32_t ld, int32_t k, double *v, double *h,
                      efgk_stream_t stream);
int efgk_rb_norm2(int64_t n, const double *v, double *nrm, efgk_stream_t stream);
int efgk_rb_set_col(int64_t n, const double *v, double scale, double *Q, int32_t ld, int32_t j,
                    efgk_stream_t stream);
int efgk_rb_apply(int64_t n, int64_t row0, const int32_t *rowptr, const int32_t *colidx, const double *a64,
                  int32_t kind, const double *Q, int32_t ld, int32_t k, double *W, efgk_stream_t stream);
int efgk_rb_gram(int64_t n, const double *Q, const double *W, int32_t ld, int32_t k, double *G,
                 efgk_stream_t stream);
int efgk_rb_combine(int64_t n, const double *Q, int32_t ld, int32_t k, const double *Y, int32_t r, void *x,
                    int64_t row0, efgk_stream_t stream);
int efgk_rb_gather_rows(int32_t m, const int32_t *idx, const double *Q, int32_t ld, int32_t k, double *out,
                        efgk_stream_t stream);
/* Restart of the double-float batch from the x already in the batch: r = b -
 * A x (true residual, all columns) with |r|^2 and r^T z into parity slot 1,
 * then t and p = z. */
int efgk_batch_dd_restart(const struct EfgkBatch *bt, efgk_stream_t stream);
/* nzlo[k] = (K64 - k, M64.re - m_re, M64.im - m_im, 0) for the packed nz. */
/* Debye-region mass MD (real, nnz doubles): high word into nzlo[k].w, low
 * word into mdlo[k] (after efgk_batch_pack_lo). */
int efgk_batch_pack_md(int64_t nnz, const double *MD64, void *nzlo, float *mdlo, efgk_stream_t stream);
int efgk_batch_pack_lo(int64_t nnz, const void *nz, const double *K64, const double *M64, void *nzlo,
                       efgk_stream_t stream);

/* ------------------------------------------------------------ mesh ingest
 * Global edge numbering on the device, identical to build_edges
 * (src/mesh_gmsh.cpp:104-147, include/edgefem/mesh.hpp:56-60): edges are
 * numbered by first appearance scanning the tetrahedra's local pairs
 * (0,1),(0,2),(0,3),(1,2),(1,3),(2,3), then the triangles' (0,1),(1,2),(2,0).
 * Occurrence o = 6 t + e (tetrahedron t) or 6 T + 3 s + e (triangle s).
 * tet_nodes [4T] and tri_nodes [3S] hold dense node indices 0..nn-1;
 * node_ids [nn] the node ids that set the orientation.  Outputs:
 * occ_edge[o] (edge id), occ_orient[o] (+1 iff the pair's first node has
 * the smaller id, else -1), edge_nodes[2i], [2i+1] = dense indices of edge
 * i's nodes, smaller id first (room for 6T + 3S edges), *n_edges (one
 * device int32) = the edge count, or -1 if a node index was out of range
 * (outputs then undefined).  scratch: efgk_build_edges_scratch_bytes(T, S,
 * nn) bytes, 256-byte aligned, any content.  Requires 6T + 3S < 2^31. */
int64_t efgk_build_edges_scratch_bytes(int64_t T, int64_t S, int32_t nn);
int efgk_build_edges(int64_t T, const int32_t *tet_nodes, int64_t S, const int32_t *tri_nodes, int32_t nn,
                     const int64_t *node_ids, int32_t *occ_edge, int8_t *occ_orient, int32_t *edge_nodes,
                     int32_t *n_edges, void *scratch, efgk_stream_t stream);
/* validate_mesh (src/mesh_quality.cpp:10-83): per tet the signed volume
 * (p1-p0).((p2-p0) x (p3-p0))/6 and the longest/shortest edge ratio (+inf
 * when the shortest is below DBL_EPSILON), computed without fused
 * multiply-adds in the host's order of operations.  xyz [3 nn], tet_nodes
 * [4T] dense node indices.  tet_flag[t] (may be NULL) = 1 if |vol| < 1e-15,
 * 2 if vol < 0, else 0; out[0] = min volume (DBL_MAX for T = 0), out[1] =
 * max ratio (0 for T = 0); counts[0] degenerate, counts[1] inverted.
 * scratch: efgk_validate_mesh_scratch_bytes(T) bytes, 256-byte aligned. */
int64_t efgk_validate_mesh_scratch_bytes(int64_t T);
int efgk_validate_mesh(int64_t T, const double *xyz, const int32_t *tet_nodes, int8_t *tet_flag, double *out,
                       int32_t *counts, void *scratch, efgk_stream_t stream);

#ifdef __cplusplus
}
#endif
#endif
