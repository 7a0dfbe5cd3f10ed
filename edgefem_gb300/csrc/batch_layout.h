// Device-side description of one batched eigenmode solve: B mesh instances
// stacked block-diagonally (N rows in total), R = F*P right-hand sides per
// row (frequency f, active port a at column f*P + a), vectors stored
// row-major [N][R] so a row's right-hand sides are contiguous.
//
// The operator of instance b at frequency f is
//   A_bf = K_b - k0_f^2 M_b + sum_p coef[b,p,f] * Ms_{b,p}
// with K real (1/mu_r real), M complex (eps_r baked in) and the port
// surface masses Ms stored as a small side CSR over the port-face rows.
#pragma once

#include <stdint.h>

#ifdef __CUDACC__
#include <cuda_runtime.h>
#else
#include <vector_types.h>
#endif

struct EfgkBatch {
  int32_t N;          // total rows
  int32_t R;          // right-hand sides per row (padded)
  int32_t F, P;       // frequencies, ports (R >= F*P)
  int32_t B;          // instances
  int32_t n_chunks;   // row chunks (never straddle instances)
  // chunk table
  const int32_t *chunk_inst, *chunk_begin, *chunk_end;
  // matrix (global row/column numbering)
  const int32_t *rowptr, *colidx;
  const float *K32;
  const float2 *M32;
  const double *K64;
  const double2 *M64;
  const float *kd32;       // K diagonal per row
  const float2 *md32;      // M diagonal per row
  const double *kd64;
  const double2 *md64;
  // port-face side CSR: rows with sidx[row] >= 0 own entries sptr[s]..sptr[s+1]
  const int32_t *sidx;     // per row, -1 if none
  const int32_t *sptr;     // n_srows + 1
  const int32_t *scol;     // global column
  const float *sval32;
  const double *sval64;
  const int32_t *scidx;    // coefficient row b*P + p of each entry
  const float *sdiag32;    // [n_srows][P] diagonal of Ms_p on that row
  const double *sdiag64;
  const double2 *cval;     // [n_srows][P] port overlap vector c_p = Ms_p e_p
  const int32_t *srow_inst;// instance of each side row
  const int32_t *srow_row; // global row of each side row
  int32_t n_srows;
  // per right-hand side / instance tables
  const float *k0sq32;     // [R]
  const double *k0sq64;    // [R]
  const float2 *scoef32;   // [B*P][R]  j*alpha*beta_{b,p}(f)
  const double2 *scoef64;
  // vectors [N][R]
  float2 *xc, *r, *p, *q;
  double2 *x64;
  // per (instance, rhs) scalars, index b*R + rhs
  double *rho;             // [2][B*R] complex -> 4*B*R doubles (re, im interleaved per parity)
  double *pq;              // [2][B*R] complex
  double *rr;              // [2][B*R]
  double *bb;              // [B*R]
  int32_t *status;         // [B*R] 0 running, 1 converged, 2 breakdown, 3 max iterations
  int32_t *iters;          // [B*R]
  int32_t *it_count;       // [1] iterations done
  double *S_acc;           // [B][P (out port j)][R] complex: e_j^H Ms_j x
  double tol2;
  int32_t max_iters;
};
