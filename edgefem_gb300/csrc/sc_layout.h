// Device scalar-block layouts shared by the Krylov kernels and the host
// drivers (indices into a small double array).
#pragma once

// Status codes written to the status slot.
#define EFGK_RUNNING 0.0
#define EFGK_CONVERGED 1.0
#define EFGK_BREAKDOWN 2.0
#define EFGK_MAXIT 3.0

// COCG64: parity-buffered accumulators (P = iteration & 1).
#define SC_RHO 0      // rho[2] complex  -> [0..3]
#define SC_PQ 4       // pq[2] complex   -> [4..7]
#define SC_RR 8       // rr[2]           -> [8..9]
#define SC_BB 10      // |b|^2
#define SC_TOL2 11    // tol^2
#define SC_STATUS 12
#define SC_ITERS 13
#define SC_MAXIT 14
#define SC_LASTRR 15
#define SC_SIZE 16

// BiCGStab64
#define SB_RHO 0      // complex
#define SB_ALPHA 2    // complex
#define SB_OMEGA 4    // complex
#define SB_BETA 6     // complex
#define SB_RHR 8      // complex accumulator rhat^H r
#define SB_RV 10      // complex accumulator rhat^H v
#define SB_TS 12      // complex accumulator conj(s)^T t
#define SB_TT 14
#define SB_RR 15
#define SB_BB 16
#define SB_TOL2 17
#define SB_STATUS 18
#define SB_ITERS 19
#define SB_MAXIT 20
#define SB_LASTRR 21
#define SB_SIZE 24
