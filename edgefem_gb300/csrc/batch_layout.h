// Device-side description of one batched eigenmode solve: B mesh instances
// stacked block-diagonally (N edge rows and NN nodes in total), R = F*P
// right-hand sides per row (frequency f, active port a at column f*P + a),
// vectors stored row-major [rows][R] so a row's right-hand sides are
// contiguous.
//
// The operator of instance b at frequency f is
//   A_bf = K_b - k0_f^2 M_b + sum_p coef[b,p,f] * Ms_{b,p}
// with K real (1/mu_r real), M complex (eps_r baked in) and the port
// surface masses Ms stored as a small side CSR over the port-face rows.
//
// Preconditioner per right-hand side: z = D^-1 r + G Dn^-1 G^T r with the
// Jacobi diagonal D and the nodal diagonal Dn = diag(G^T A_bf G), both
// formed on the fly from per-row / per-node components.
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
  int32_t B;          // instances
  // row chunks (never straddle instances); each block of a launch takes a
  // contiguous range of chunks
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
  const int32_t *scidx;    // coefficient row b*P + p of each entry
  const float *sdiag32;    // [n_srows][P]
  const double2 *cval;     // [n_srows][P] port overlap vector c_p = Ms_p e_p
  const int32_t *srow_inst;
  const int32_t *srow_row;
  int32_t n_srows;
  // gradient: per edge (tail, head) global node, (-1,-1) for PEC; per node
  // incident edges and signs; nodal diagonal components
  const int2 *enodes;
  const int32_t *nptr, *nedge;
  const signed char *nsign;
  const float *kn32;       // diag(G^T K G)
  const float2 *mn32;      // diag(G^T M G)
  const float *msn32;      // [NN][P] diag(G^T Ms_p G)
  // per right-hand side / instance tables
  const float *k0sq32;     // [R]
  const double *k0sq64;    // [R]
  const float2 *scoef32;   // [B*P][R]  j*alpha*beta_{b,p}(f)
  const double2 *scoef64;
  // vectors [N][R] (t: [NN][R]); complex64 engine
  float2 *xc, *r, *p, *q, *t;
  double2 *x64;
  // double-float engine: complex dd vectors (re_hi, re_lo, im_hi, im_lo)
  // and the low words of each stored nonzero (k_lo, m_re_lo, m_im_lo, 0):
  // K = k + k_lo, M = (m_re + m_re_lo) + j (m_im + m_im_lo)
  float4 *xd, *rd, *pd, *qd, *td;
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
  double *S_acc;           // [B][P][R] complex: e_j^H Ms_j x
  double tol2;
  double delta2;           // replacement threshold (|r| < delta * |r_last|)^2
  int32_t stagnation;      // force a replacement after this many iterations without one
  int32_t max_iters;
};
