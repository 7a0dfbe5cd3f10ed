/* CPU complex128 COCG with the auxiliary-space preconditioner.
 *
 * TEST INFRASTRUCTURE ONLY: the oracle's iterative solver in C, for systems
 * too large for a direct factorisation on the CPU (the 580k-edge WR-90 slab
 * guide).  Tests, the smoke check and the benchmark's CPU legs call it (as
 * the checker and as the timed CPU baseline); the product never does.
 *
 * It restates edgefem_oracle.cocg_jacobi + aux_preconditioner exactly:
 *
 *   z = D^-1 r + G Dn^-1 G^T r + Pi Dp^-1 Pi^T r
 *
 * with D = diag(A); G the edge-node incidence without PEC edges (-1 at the
 * tail node, +1 at the head node), Dn = diag(G^T A G) (entries below 1e-12 of
 * the largest magnitude give 0); Pi[e, (k, d)] = (x_head - x_tail)_d / 2 at
 * both end nodes k of e, Dp = diag(Pi^T A Pi), Dp^-1 scaled by the weight
 * omega (0 switches the vector-nodal term off).  COCG (van der Vorst and
 * Melissen 1990) uses the unconjugated bilinear form of the complex
 * symmetric A:
 *
 *   q = A p; alpha = rho / p^T q; x += alpha p; r -= alpha q;
 *   stop when |r| / |b| < tol;  z = M r; rho' = r^T z; p = z + (rho'/rho) p.
 *
 * This is the preconditioned COCG of the GPU plain path; the reference's
 * solver (src/solver.cpp:35-193, Eigen BiCGSTAB + ILUT) does not build here
 * (Eigen is absent), and this C form lets the CPU side converge the
 * full-size systems in seconds instead of minutes (OpenMP over rows).
 *
 * Complex numbers are interleaved (re, im) doubles.  Loops are split into
 * static OpenMP chunks, so results are reproducible for a fixed thread
 * count.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef struct {
  double re, im;
} cx;

static inline cx cmul(cx a, cx b) { return (cx){a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re}; }
static inline cx cdiv(cx a, cx b) {
  const double d = b.re * b.re + b.im * b.im;
  return (cx){(a.re * b.re + a.im * b.im) / d, (a.im * b.re - a.re * b.im) / d};
}
static inline cx crecip_or(cx a, cx fallback) {
  const double d = a.re * a.re + a.im * a.im;
  if (!(d > 0.0) || !isfinite(d)) return fallback;
  return (cx){a.re / d, -a.im / d};
}

static double now_s(void) {
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

/* Aux-space data built from the matrix and the incidence lists. */
typedef struct {
  int n, nn, npi;
  const int32_t *enodes; /* 2n: tail, head node index; -1 for PEC edges */
  const double *piw;     /* 3n: (x_head - x_tail) / 2 */
  const int32_t *nptr;   /* nn + 1 */
  const int32_t *nedge;  /* incident non-PEC edges of each node */
  const int8_t *nsign;   /* -1 at the edge's tail, +1 at its head */
  cx *dinv, *dninv, *dpinv, *t, *tp;
} Aux;

/* Diagonal entry (e, f) lookup inside row e (sorted columns). */
static cx row_entry(const int64_t *rp, const int32_t *ci, const cx *v, int e, int f) {
  int64_t lo = rp[e], hi = rp[e + 1];
  while (lo < hi) {
    const int64_t mid = (lo + hi) / 2;
    if (ci[mid] < f)
      lo = mid + 1;
    else
      hi = mid;
  }
  if (lo < rp[e + 1] && ci[lo] == f) return v[lo];
  return (cx){0.0, 0.0};
}

static void aux_setup(Aux *a, const int64_t *rp, const int32_t *ci, const cx *v, double omega_vec) {
  const int n = a->n, nn = a->nn;
  cx *dn = (cx *)calloc((size_t)nn, sizeof(cx));
  cx *dp = (cx *)calloc((size_t)3 * nn, sizeof(cx));
#pragma omp parallel for schedule(static)
  for (int e = 0; e < n; ++e) {
    const cx d = row_entry(rp, ci, v, e, e);
    a->dinv[e] = crecip_or(d, (cx){1.0, 0.0});
  }
  /* Dn[k] = sum_{e,f at k} s_e s_f A_ef, Dp[k,d] = sum w_ed w_fd A_ef */
#pragma omp parallel for schedule(static)
  for (int k = 0; k < nn; ++k) {
    cx sn = {0.0, 0.0}, sp3[3] = {{0.0, 0.0}, {0.0, 0.0}, {0.0, 0.0}};
    for (int i = a->nptr[k]; i < a->nptr[k + 1]; ++i) {
      const int e = a->nedge[i];
      const double se = a->nsign[i];
      for (int j = a->nptr[k]; j < a->nptr[k + 1]; ++j) {
        const int f = a->nedge[j];
        const cx aef = row_entry(rp, ci, v, e, f);
        const double sf = a->nsign[j];
        sn.re += se * sf * aef.re;
        sn.im += se * sf * aef.im;
        for (int d = 0; d < 3; ++d) {
          const double w = a->piw[3 * (size_t)e + d] * a->piw[3 * (size_t)f + d];
          sp3[d].re += w * aef.re;
          sp3[d].im += w * aef.im;
        }
      }
    }
    dn[k] = sn;
    for (int d = 0; d < 3; ++d) dp[3 * (size_t)k + d] = sp3[d];
  }
  double mn = 0.0, mp = 0.0;
  for (int k = 0; k < nn; ++k) {
    const double m = hypot(dn[k].re, dn[k].im);
    if (m > mn) mn = m;
    for (int d = 0; d < 3; ++d) {
      const double q = hypot(dp[3 * (size_t)k + d].re, dp[3 * (size_t)k + d].im);
      if (q > mp) mp = q;
    }
  }
  for (int k = 0; k < nn; ++k) {
    const double m = hypot(dn[k].re, dn[k].im);
    a->dninv[k] = m > 1e-12 * mn ? cdiv((cx){1.0, 0.0}, dn[k]) : (cx){0.0, 0.0};
    for (int d = 0; d < 3; ++d) {
      const cx q = dp[3 * (size_t)k + d];
      const double mq = hypot(q.re, q.im);
      a->dpinv[3 * (size_t)k + d] =
          (a->npi && mq > 1e-12 * mp) ? cdiv((cx){omega_vec, 0.0}, q) : (cx){0.0, 0.0};
    }
  }
  free(dn);
  free(dp);
}

/* z = M r; returns r^T z. */
static cx aux_apply(const Aux *a, const cx *r, cx *z, int level) {
  const int n = a->n, nn = a->nn;
  if (level > 0) {
#pragma omp parallel for schedule(static)
    for (int k = 0; k < nn; ++k) {
      cx s = {0.0, 0.0}, sp3[3] = {{0.0, 0.0}, {0.0, 0.0}, {0.0, 0.0}};
      for (int i = a->nptr[k]; i < a->nptr[k + 1]; ++i) {
        const int e = a->nedge[i];
        const double se = a->nsign[i];
        s.re += se * r[e].re;
        s.im += se * r[e].im;
        if (level > 1)
          for (int d = 0; d < 3; ++d) {
            const double w = a->piw[3 * (size_t)e + d];
            sp3[d].re += w * r[e].re;
            sp3[d].im += w * r[e].im;
          }
      }
      a->t[k] = cmul(a->dninv[k], s);
      if (level > 1)
        for (int d = 0; d < 3; ++d) a->tp[3 * (size_t)k + d] = cmul(a->dpinv[3 * (size_t)k + d], sp3[d]);
    }
  }
  double rzr = 0.0, rzi = 0.0;
#pragma omp parallel for schedule(static) reduction(+ : rzr, rzi)
  for (int e = 0; e < n; ++e) {
    cx ze = cmul(a->dinv[e], r[e]);
    if (level > 0) {
      const int ta = a->enodes[2 * (size_t)e], hb = a->enodes[2 * (size_t)e + 1];
      if (ta >= 0) {
        ze.re += a->t[hb].re - a->t[ta].re;
        ze.im += a->t[hb].im - a->t[ta].im;
        if (level > 1)
          for (int d = 0; d < 3; ++d) {
            const double w = a->piw[3 * (size_t)e + d];
            ze.re += w * (a->tp[3 * (size_t)ta + d].re + a->tp[3 * (size_t)hb + d].re);
            ze.im += w * (a->tp[3 * (size_t)ta + d].im + a->tp[3 * (size_t)hb + d].im);
          }
      }
    }
    z[e] = ze;
    const cx rz = cmul(r[e], ze);
    rzr += rz.re;
    rzi += rz.im;
  }
  return (cx){rzr, rzi};
}

/* Solve A x = b from x = 0.  level: 0 Jacobi, 1 + gradient space, 2 + the
 * vector-nodal space (weight omega_vec).  Stops at |r|/|b| < tol2 (the
 * recurrence residual) or maxit; the wall time at which |r|/|b| first fell
 * below tol1 (<= 0: unused) is written to t_tol1 together with the
 * iteration count then.  Returns 0 when tol2 was reached, 1 otherwise, -1
 * on bad arguments or allocation failure. */
int oracle_cocg_aux(int n, const int64_t *rowptr, const int32_t *colidx, const double *vals, int nn,
                    const int32_t *enodes, const double *piw, const int32_t *nptr, const int32_t *nedge,
                    const int8_t *nsign, int level, double omega_vec, const double *b, double *x,
                    double tol1, double tol2, int maxit, int nthreads, int *iters_out, double *relres_out,
                    double *seconds_out, int *iters_tol1, double *seconds_tol1) {
  if (n <= 0 || !rowptr || !colidx || !vals || !b || !x || level < 0 || level > 2) return -1;
  if (level > 0 && (nn <= 0 || !enodes || !nptr || !nedge || !nsign || (level > 1 && !piw))) return -1;
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#else
  (void)nthreads;
#endif
  const cx *A = (const cx *)vals;
  const cx *bb = (const cx *)b;
  cx *xx = (cx *)x;
  Aux a;
  memset(&a, 0, sizeof(a));
  a.n = n;
  a.nn = level > 0 ? nn : 0;
  a.npi = level > 1;
  a.enodes = enodes;
  a.piw = piw;
  a.nptr = nptr;
  a.nedge = nedge;
  a.nsign = nsign;
  a.dinv = (cx *)malloc((size_t)n * sizeof(cx));
  if (level > 0) {
    a.dninv = (cx *)malloc((size_t)nn * sizeof(cx));
    a.dpinv = (cx *)malloc((size_t)3 * nn * sizeof(cx));
    a.t = (cx *)malloc((size_t)nn * sizeof(cx));
    a.tp = (cx *)malloc((size_t)3 * nn * sizeof(cx));
  }
  cx *r = (cx *)malloc((size_t)n * sizeof(cx));
  cx *z = (cx *)malloc((size_t)n * sizeof(cx));
  cx *p = (cx *)malloc((size_t)n * sizeof(cx));
  cx *q = (cx *)malloc((size_t)n * sizeof(cx));
  if (!a.dinv || !r || !z || !p || !q || (level > 0 && (!a.dninv || !a.dpinv || !a.t || !a.tp))) {
    free(a.dinv), free(a.dninv), free(a.dpinv), free(a.t), free(a.tp), free(r), free(z), free(p), free(q);
    return -1;
  }
  const double t0 = now_s();
  if (level > 0) {
    aux_setup(&a, rowptr, colidx, A, omega_vec);
  } else {
#pragma omp parallel for schedule(static)
    for (int e = 0; e < n; ++e) a.dinv[e] = crecip_or(row_entry(rowptr, colidx, A, e, e), (cx){1.0, 0.0});
  }
  double nb2 = 0.0;
#pragma omp parallel for schedule(static) reduction(+ : nb2)
  for (int e = 0; e < n; ++e) {
    xx[e] = (cx){0.0, 0.0};
    r[e] = bb[e];
    nb2 += bb[e].re * bb[e].re + bb[e].im * bb[e].im;
  }
  const double nb = sqrt(nb2);
  cx rho = aux_apply(&a, r, z, level);
#pragma omp parallel for schedule(static)
  for (int e = 0; e < n; ++e) p[e] = z[e];
  int it = 0, status = 1;
  double rel = 1.0;
  if (iters_tol1) *iters_tol1 = -1;
  if (seconds_tol1) *seconds_tol1 = -1.0;
  if (nb == 0.0) {
    rel = 0.0;
    status = 0;
  }
  while (status != 0 && it < maxit) {
    double pqr = 0.0, pqi = 0.0;
#pragma omp parallel for schedule(static) reduction(+ : pqr, pqi)
    for (int e = 0; e < n; ++e) {
      double sr = 0.0, si = 0.0;
      for (int64_t k = rowptr[e]; k < rowptr[e + 1]; ++k) {
        const cx av = A[k], pv = p[colidx[k]];
        sr += av.re * pv.re - av.im * pv.im;
        si += av.re * pv.im + av.im * pv.re;
      }
      q[e] = (cx){sr, si};
      pqr += p[e].re * sr - p[e].im * si;
      pqi += p[e].re * si + p[e].im * sr;
    }
    const cx alpha = cdiv(rho, (cx){pqr, pqi});
    double rr = 0.0;
#pragma omp parallel for schedule(static) reduction(+ : rr)
    for (int e = 0; e < n; ++e) {
      const cx ap = cmul(alpha, p[e]), aq = cmul(alpha, q[e]);
      xx[e].re += ap.re;
      xx[e].im += ap.im;
      r[e].re -= aq.re;
      r[e].im -= aq.im;
      rr += r[e].re * r[e].re + r[e].im * r[e].im;
    }
    ++it;
    rel = sqrt(rr) / nb;
    if (!isfinite(rel)) break;
    if (tol1 > 0.0 && iters_tol1 && *iters_tol1 < 0 && rel < tol1) {
      *iters_tol1 = it;
      if (seconds_tol1) *seconds_tol1 = now_s() - t0;
    }
    if (rel < tol2) {
      status = 0;
      break;
    }
    const cx rho_new = aux_apply(&a, r, z, level);
    const cx beta = cdiv(rho_new, rho);
#pragma omp parallel for schedule(static)
    for (int e = 0; e < n; ++e) {
      const cx bp = cmul(beta, p[e]);
      p[e] = (cx){z[e].re + bp.re, z[e].im + bp.im};
    }
    rho = rho_new;
  }
  if (iters_out) *iters_out = it;
  if (relres_out) *relres_out = rel;
  if (seconds_out) *seconds_out = now_s() - t0;
  free(a.dinv), free(a.dninv), free(a.dpinv), free(a.t), free(a.tp), free(r), free(z), free(p), free(q);
  return status;
}

/* y = A x (complex128 CSR, OpenMP over rows). */
void oracle_csr_matvec(int n, const int64_t *rowptr, const int32_t *colidx, const double *vals, const double *x,
                       double *y, int nthreads) {
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#else
  (void)nthreads;
#endif
  const cx *A = (const cx *)vals, *xx = (const cx *)x;
  cx *yy = (cx *)y;
#pragma omp parallel for schedule(static)
  for (int e = 0; e < n; ++e) {
    double sr = 0.0, si = 0.0;
    for (int64_t k = rowptr[e]; k < rowptr[e + 1]; ++k) {
      const cx av = A[k], pv = xx[colidx[k]];
      sr += av.re * pv.re - av.im * pv.im;
      si += av.re * pv.im + av.im * pv.re;
    }
    yy[e] = (cx){sr, si};
  }
}

int oracle_max_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}
