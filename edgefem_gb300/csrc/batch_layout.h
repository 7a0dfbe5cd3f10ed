// Device-side description of one batched solve: B mesh instances
// stacked block-diagonally (N edge rows and NN nodes in total), R = F*P
// right-hand sides per row (frequency f, active port a at column f*P + a),
// vectors stored row-major [rows][R] so a row's right-hand sides are
// contiguous.
//
// The operator of instance b at frequency f is
//   A_bf = K_b - k0_f^2 (M_b + eps_D(f) MD_b) + sum_c coef[b,c,f] * S_{b,c}
// with K real (1/mu_r real), M complex (non-dispersive eps_r baked in), MD
// the real mass of the Debye region (unit permittivity; zero without one)
// and the side terms S_{b,c} stored as a small side CSR over port (and
// absorbing-boundary) rows, c < C:
//   eigenmode ports:  S_p = Ms_p (port surface mass), coef = j alpha beta_p(f);
//   driven ports:     S_p = w_p w_p^T, coef = 1/Z0_p; S_C-1 = ABC diagonal,
//                     coef = j k0_f.
// Right-hand side of column f*P + a: rcoef[b,a,f] * c_a with c_a the port
// vector (eigenmode: Ms_a e_a, driven: w_a), which is also the overlap
// vector of the S extraction.
//
// Preconditioner per right-hand side: z = D^-1 r + G Dn^-1 G^T r
// (+ omega Pi Dp^-1 Pi^T r with npi = 3) with the Jacobi diagonal D, the
// nodal diagonal Dn = diag(G^T A_bf G) and, for the vector-nodal space Pi
// (Pi[e, (n, d)] = (x_head - x_tail)_d / 2 for both end nodes n of edge e,
// the edge interpolant of a linear nodal vector field), Dp =
// diag(Pi^T A_bf Pi) per (node, component); all formed on the fly from
// per-row / per-node components (the Pi components are stored divided by
// omega).
#pragma once

#include <stdint.h>

#ifdef __CUDACC__
#include <cuda_runtime.h>
#else
#include <vector_types.h>
#endif

// One stored nonzero: column, K value, M value (16 bytes, one vector load).
struct EfgkNz {
  int32_t col;
  float k;
  float mre, mim;
};

struct EfgkBatch {
  int32_t N;          // total edge rows
  int32_t NN;         // total nodes
  int32_t R;          // right-hand sides per row (power of two, 4..128)
  int32_t F, P;       // frequencies, ports (F*P <= R)
  int32_t C;          // side-term coefficient rows per instance (>= P)
  int32_t B;          // instances
  // row chunks (never straddle instances), distributed over the blocks of
  // each launch
  int32_t n_chunks;
  const int32_t *chunk_inst, *chunk_begin, *chunk_end;
  int32_t n_nchunks;  // node chunks
  const int32_t *nchunk_inst, *nchunk_begin, *nchunk_end;
  // matrix (global row/column numbering)
  const int32_t *rowptr;
  const EfgkNz *nz;
  const int32_t *colidx;   // for the FP64 residual
  const double *K64;
  const double2 *M64;
  const float *kd32;       // K diagonal per row
  const float2 *md32;      // M diagonal per row
  // port-face side CSR: rows with sidx[row] >= 0 own entries sptr[s]..sptr[s+1]
  const int32_t *sidx;
  const int32_t *sptr;
  const int32_t *scol;
  const float *sval32;
  const double *sval64;
  const int32_t *scidx;    // coefficient row b*C + c of each entry
  const float *sdiag32;    // [n_srows][C] diagonal of each side term
  const double2 *cval;     // [n_srows][P] port vector c_p
  const int32_t *srow_inst;
  const int32_t *srow_row;
  int32_t n_srows;
  // gradient: per edge (tail, head) global node, (-1,-1) for PEC; per node
  // incident edges and signs; nodal diagonal components
  const int2 *enodes;
  const int32_t *nptr, *nedge;
  const signed char *nsign;
  const int4 *ninc;        // per incidence {edge, or ~edge at its tail; 3 vector-nodal weights}
  const float *kn32;       // diag(G^T K G)
  const float2 *mn32;      // diag(G^T M G)
  const float *msn32;      // [NN][C] diag(G^T S_c G)
  // vector-nodal space (npi = 3; 0 = off): per edge 3 weights, per (node,
  // component) diagonal components of K, M, MD and the side terms
  int32_t npi;
  const float *piw;        // [N][3]
  const float *kpn32;      // [NN][3]
  const float2 *mpn32;     // [NN][3]
  const float *mdpn32;     // [NN][3]
  const float *mspn32;     // [NN][3][C]
  // Debye region (has_md != 0): low words of MD (high words in nzlo.w),
  // its row and nodal diagonals, and kappa = k0_f^2 eps_D(f) per column
  int32_t has_md;
  const float *mdlo;
  const float *mdd32;      // diag(MD) per row
  const float *mnd32;      // diag(G^T MD G) per node
  const double2 *kappa64;  // [R]
  const float2 *kappa32;
  // per right-hand side / instance tables
  const float *k0sq32;     // [R]
  const double *k0sq64;    // [R]
  const float2 *scoef32;   // [B*C][R] side-term coefficients
  const double2 *scoef64;
  const double2 *rcoef64;  // [B*P][R] right-hand-side coefficients
  // vectors [N][R] (t: [NN][R]); complex64 engine
  float2 *xc, *r, *p, *q, *t;
  double2 *x64;
  // double-float engine: complex dd vectors (re_hi, re_lo, im_hi, im_lo)
  // and the low words of each stored nonzero (k_lo, m_re_lo, m_im_lo,
  // md_hi): K = k + k_lo, M = (m_re + m_re_lo) + j (m_im + m_im_lo),
  // MD = md_hi + mdlo
  float4 *xd, *rd, *pd, *qd, *td;  // td: [NN][1 + npi][R]
  const float4 *nzlo;
  // per (instance, rhs) scalars, index i = b*R + rhs
  double *rho;             // [2][B*R] complex (re, im interleaved)
  double *pq;              // [2][B*R] complex
  double *rr;              // [2][B*R]
  double *bb;              // [B*R]   |b|^2
  double *rmax;            // [B*R]   |r|^2 at the last residual replacement
  int32_t *status;         // [B*R] 0 running, 1 converged, 2 breakdown, 3 max iterations, 4 inactive
  int32_t *flag;           // [B*R] residual replacement requested at this checkpoint
  int32_t *iters;          // [B*R]
  int32_t *last_rep;       // [B*R] iteration of the last residual replacement
  int32_t *counters;       // [0] iterations done, [1] flagged count
  double *S_acc;           // [B][P][R] complex: c_j^H x
  double tol2;
  double delta2;           // replacement threshold (|r| < delta * |r_last|)^2
  int32_t stagnation;      // replace and restart after this many iterations without progress
  int32_t replace_on_progress;  // 1: replace at every factor-1/delta drop of |r|
  int32_t max_iters;
};
