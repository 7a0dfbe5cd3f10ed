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
 * Shared scalar block for one plain COCG/BiCGStab solve: see EfgkScalars64
 * in the host library.  `sc` points at it on the device. */
int efgk_spmv64(int32_t n, const int32_t *rowptr, const int32_t *colidx, const double *vals,
                const double *x, double *y, efgk_stream_t stream);
int efgk_cocg64_init(int32_t n, const double *b, const double *dinv, double *x, double *r, double *p,
                     double *sc, efgk_stream_t stream);
int efgk_cocg64_step(int32_t n, const int32_t *rowptr, const int32_t *colidx, const double *vals,
                     const double *dinv, double *x, double *r, double *p, double *q, double *sc,
                     int parity, efgk_stream_t stream);
int efgk_bicgstab64_init(int32_t n, const double *b, double *x, double *r, double *rhat, double *p,
                         double *v, double *sc, efgk_stream_t stream);
int efgk_bicgstab64_step(int32_t n, const int32_t *rowptr, const int32_t *colidx, const double *vals,
                         const double *dinv, double *x, double *r, const double *rhat, double *p,
                         double *v, double *s, double *t, double *phat, double *shat, double *sc,
                         efgk_stream_t stream);
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
/* x_c += alpha p, r -= alpha q, rho' = r^T D^-1 r, |r|^2. */
int efgk_batch_update(const struct EfgkBatch *bt, int parity, efgk_stream_t stream);
/* p = D^-1 r + beta p; bit 1 of `parity_check` requests the convergence test. */
int efgk_batch_pupdate(const struct EfgkBatch *bt, int parity_check, efgk_stream_t stream);
/* FP64 refinement: x64 += x_c, x_c = 0, r = b - A x64 (FP64), rho', |r|^2. */
int efgk_batch_flush_residual(const struct EfgkBatch *bt, int parity, efgk_stream_t stream);
/* r = b, |b|^2, p = D^-1 r, status (x64 = x_c = 0 beforehand). */
int efgk_batch_init(const struct EfgkBatch *bt, efgk_stream_t stream);
/* x64 += x_c and the port overlaps S_acc[b][j][rhs] = e_j^H Ms_j x. */
int efgk_batch_finish(const struct EfgkBatch *bt, efgk_stream_t stream);
/* FP64 assembled K, M (complex, nnz) -> K32 real, M32 complex, K64 real, M64 complex. */
int efgk_batch_pack(int64_t nnz, const double *K, const double *M, float *K32, float *M32, double *K64,
                    double *M64, efgk_stream_t stream);
/* Diagonals of K and M (via the diagonal slots) in FP32 and FP64. */
int efgk_batch_diag(int32_t n, const int32_t *diag_slot, const double *K64, const double *M64, float *kd32,
                    float *md32, double *kd64, double *md64, efgk_stream_t stream);

#ifdef __cplusplus
}
#endif
#endif
