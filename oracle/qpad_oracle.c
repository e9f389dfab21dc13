/*
 * qpad_oracle.c -- CPU FP64 restatement of QPAD's per-xi-slice quasi-static loop.
 *
 * TEST INFRASTRUCTURE ONLY (the oracle and the timed CPU baseline).  Parity is
 * UNPINNED against the reference itself: the reference cannot be built here and its
 * tests hold no golden vectors.  It is pinned by the project's own known-answer
 * tests instead.  See qpad_oracle.h for the layouts.
 *
 * Each function names the reference routine (file:line within QPAD's source/) that it
 * restates, with single-rank semantics (noff = 0, idproc = 0 = nvp-1, no pipeline).
 * Operation order follows the Fortran expressions; compile with -ffp-contract=off.
 */
#include "qpad_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define NR2 (g->nr + 2)
/* slice-field element: part p, component c, node i (0..nr+1) */
#define F(f, nc, p, c, i) ((f)[((size_t)(p) * (nc) + (c)) * (size_t)NR2 + (size_t)(i)])
#define PRE(m) (2 * (m) - 1)  /* part holding Re of mode m >= 1 */
#define PIM(m) (2 * (m))      /* part holding Im of mode m >= 1 */

static const double ORC_PI = 3.141592653589793; /* 4*atan(1.0), param.f03:29 */

static int nparts(const orc_grid* g) { return 2 * g->max_mode + 1; }

/* =============================================================================
 * Tridiagonal operators: field_solver_class.f03:256-561 (set_struct_matrix)
 * ============================================================================= */
void orc_build_matrix(const orc_grid* g, int kind, int m, double* a, double* b, double* c) {
  const int nr = g->nr;
  const double dr = g->dr, dr2 = dr * dr, m2 = (double)(m * m), rf = g->relax_fac;
  /* rows 2..nr: j = row-1 (field_solver_class.f03:301-307, 335-342, 370-377) */
  for (int k = 2; k <= nr; ++k) {
    double j = (double)(k - 1);
    a[k - 1] = 1.0 - 0.5 / j;
    c[k - 1] = 1.0 + 0.5 / j;
    if (kind == ORC_FK_BPLUS) {
      double t = (double)(m + 1) / j;
      b[k - 1] = -2.0 - t * t - rf;
    } else if (kind == ORC_FK_BMINUS) {
      double t = (double)(m - 1) / j;
      b[k - 1] = -2.0 - t * t - rf;
    } else {
      b[k - 1] = -2.0 - m2 / (j * j);
    }
  }
  /* first row (axis) */
  int identity_axis = 1;
  if (kind == ORC_FK_BPLUS) {
    identity_axis = 1;                                   /* :346-356 */
  } else if (kind == ORC_FK_BMINUS) {
    if (m == 1) {                                        /* :383-389 */
      a[0] = 0.0; b[0] = -4.0 - rf; c[0] = 4.0; identity_axis = 0;
    }
  } else if (m == 0) {                                   /* :312-315 */
    a[0] = 0.0; b[0] = -4.0; c[0] = 4.0; identity_axis = 0;
  }
  if (identity_axis) {                                   /* :316-322 */
    a[0] = 0.0; b[0] = 1.0; c[0] = 0.0;
    if (nr >= 2) a[1] = 0.0;
  }
  /* outer boundary (:484-545) */
  if (g->bnd == ORC_BND_ZERO) {
    c[nr - 1] = 0.0;
  } else {
    double jmax = (double)nr;
    double fac;
    int dirichlet = 0;
    switch (kind) {
      case ORC_FK_PSI: case ORC_FK_EZ: case ORC_FK_BZ:
        if (m == 0) dirichlet = 1; else fac = 1.0 - (double)m / jmax;
        break;
      case ORC_FK_BT:
        if (m == 0) fac = 1.0 + 1.0 / (jmax * log(jmax * dr));
        else fac = 1.0 - (double)m / jmax;
        break;
      default: /* BPLUS, BMINUS both use (m+1) */
        fac = 1.0 - (double)(m + 1) / jmax;
        break;
    }
    if (!dirichlet) b[nr - 1] = b[nr - 1] + fac * c[nr - 1];
    c[nr - 1] = 0.0;
  }
  for (int k = 0; k < nr; ++k) { a[k] /= dr2; b[k] /= dr2; c[k] /= dr2; }  /* :552 */
}

void orc_thomas(int n, const double* a, const double* b, const double* c, double* d) {
  double* cp = (double*)malloc(sizeof(double) * (size_t)n);
  cp[0] = c[0] / b[0];
  d[0] = d[0] / b[0];
  for (int k = 1; k < n; ++k) {
    double den = b[k] - a[k] * cp[k - 1];
    cp[k] = c[k] / den;
    d[k] = (d[k] - a[k] * d[k - 1]) / den;
  }
  for (int k = n - 2; k >= 0; --k) d[k] = d[k] - cp[k] * d[k + 1];
  free(cp);
}

/* HYPRE StructCycRedSolve stand-in (field_solver_class.f03:145-196): solve in place.
 * buf is 1-based in the reference (buf(1..nr)); here buf[0..nr-1]. */
static void solve_sys(const orc_grid* g, int kind, int m, double* buf) {
  int nr = g->nr;
  double* a = (double*)malloc(sizeof(double) * 3 * (size_t)nr);
  double* b = a + nr;
  double* c = b + nr;
  orc_build_matrix(g, kind, m, a, b, c);
  orc_thomas(nr, a, b, c, buf);
  free(a);
}

/* =============================================================================
 * psi: field_psi_class.f03:131-254
 * ============================================================================= */
void orc_solve_psi(const orc_grid* g, const double* q, double* psi) {
  const int nr = g->nr, M = g->max_mode;
  double* bre = (double*)malloc(sizeof(double) * 2 * (size_t)nr);
  double* bim = bre + nr;
  for (int m = 0; m <= M; ++m) {
    int pr = m == 0 ? 0 : PRE(m), pi = m == 0 ? 0 : PIM(m);
    for (int i = 1; i <= nr; ++i) {                                  /* set_source 131-176 */
      bre[i - 1] = -1.0 * F(q, 1, pr, 0, i);
      if (m > 0) bim[i - 1] = -1.0 * F(q, 1, pi, 0, i);
    }
    solve_sys(g, ORC_FK_PSI, m, bre);
    if (m > 0) solve_sys(g, ORC_FK_PSI, m, bim);
    for (int i = 1; i <= nr; ++i) {                                  /* get_solution 178-216 */
      F(psi, 1, pr, 0, i) = bre[i - 1];
      if (m > 0) F(psi, 1, pi, 0, i) = bim[i - 1];
    }
    if (m > 0) { F(psi, 1, pr, 0, 1) = 0.0; F(psi, 1, pi, 0, 1) = 0.0; }
  }
  free(bre);
}

/* =============================================================================
 * Bz: field_b_class.f03:205-307 (set_source_bz), 508-543, 760-796
 * ============================================================================= */
void orc_solve_bz(const orc_grid* g, const double* cu, double* b) {
  const int nr = g->nr, M = g->max_mode;
  const double idr = 1.0 / g->dr, idrh = 0.5 * idr;
  double* bre = (double*)calloc(2 * (size_t)nr + 2, sizeof(double));
  double* bim = bre + nr + 1;   /* 1-based buffers: bre[1..nr] */
  for (int m = 0; m <= M; ++m) {
    memset(bre, 0, sizeof(double) * (2 * (size_t)nr + 2));
    if (m == 0) {
      for (int i = 2; i <= nr; ++i) {
        double ir = idr / (double)(i - 1);
        bre[i] = -idrh * (F(cu, 3, 0, 1, i + 1) - F(cu, 3, 0, 1, i - 1)) - ir * F(cu, 3, 0, 1, i);
      }
      bre[1] = -2.0 * idr * F(cu, 3, 0, 1, 2);
      {
        double ir = idr / (double)(nr - 1);
        bre[nr] = -idrh * (3.0 * F(cu, 3, 0, 1, nr) - 4.0 * F(cu, 3, 0, 1, nr - 1) + F(cu, 3, 0, 1, nr - 2))
                  - ir * F(cu, 3, 0, 1, nr);
      }
    } else {
      const int pr = PRE(m), pi = PIM(m);
      for (int i = 2; i <= nr; ++i) {
        double ir = idr / (double)(i - 1);
        bre[i] = -idrh * (F(cu, 3, pr, 1, i + 1) - F(cu, 3, pr, 1, i - 1)) - ir * F(cu, 3, pr, 1, i)
                 - m * ir * F(cu, 3, pi, 0, i);
        bim[i] = -idrh * (F(cu, 3, pi, 1, i + 1) - F(cu, 3, pi, 1, i - 1)) - ir * F(cu, 3, pi, 1, i)
                 + m * ir * F(cu, 3, pr, 0, i);
      }
      if (m % 2 == 0) {
        bre[1] = -2.0 * idr * F(cu, 3, pr, 1, 2) - m * idr * F(cu, 3, pi, 0, 2);
        bim[1] = -2.0 * idr * F(cu, 3, pi, 1, 2) + m * idr * F(cu, 3, pr, 0, 2);
      } else {
        bre[1] = 0.0;
        bim[1] = 0.0;
        if (m == 1) {
          double ir = idr;
          bre[2] = -idr * (F(cu, 3, pr, 1, 3) - F(cu, 3, pr, 1, 2)) - ir * F(cu, 3, pr, 1, 2)
                   - m * ir * F(cu, 3, pi, 0, 2);
          bim[2] = -idr * (F(cu, 3, pi, 1, 3) - F(cu, 3, pi, 1, 2)) - ir * F(cu, 3, pi, 1, 2)
                   + m * ir * F(cu, 3, pr, 0, 2);
        }
      }
      {
        double ir = idr / (double)(nr - 1);
        bre[nr] = -idrh * (3.0 * F(cu, 3, pr, 1, nr) - 4.0 * F(cu, 3, pr, 1, nr - 1) + F(cu, 3, pr, 1, nr - 2))
                  - ir * F(cu, 3, pr, 1, nr) - m * ir * F(cu, 3, pi, 0, nr);
        bim[nr] = -idrh * (3.0 * F(cu, 3, pi, 1, nr) - 4.0 * F(cu, 3, pi, 1, nr - 1) + F(cu, 3, pi, 1, nr - 2))
                  - ir * F(cu, 3, pi, 1, nr) + m * ir * F(cu, 3, pr, 0, nr);
      }
    }
    solve_sys(g, ORC_FK_BZ, m, bre + 1);
    if (m > 0) solve_sys(g, ORC_FK_BZ, m, bim + 1);
    int pr = m == 0 ? 0 : PRE(m), pi = m == 0 ? 0 : PIM(m);
    for (int i = 1; i <= nr; ++i) {
      F(b, 3, pr, 2, i) = bre[i];
      if (m > 0) F(b, 3, pi, 2, i) = bim[i];
    }
    if (m > 0) { F(b, 3, pr, 2, 1) = 0.0; F(b, 3, pi, 2, 1) = 0.0; }
  }
  free(bre);
}

/* =============================================================================
 * Beam B-perp: field_b_class.f03:309-358 (set_source_bt), 545-701, 798-834
 * ============================================================================= */
void orc_solve_bt_beam(const orc_grid* g, const double* q, double* b) {
  const int nr = g->nr, M = g->max_mode;
  const double idr = 1.0 / g->dr, idrh = 0.5 * idr;
  double* bre = (double*)calloc(2 * (size_t)nr + 2, sizeof(double));
  double* bim = bre + nr + 1;
  for (int m = 0; m <= M; ++m) {
    int pr = m == 0 ? 0 : PRE(m), pi = m == 0 ? 0 : PIM(m);
    for (int i = 1; i <= nr; ++i) {
      bre[i] = -1.0 * F(q, 1, pr, 0, i);
      if (m > 0) bim[i] = -1.0 * F(q, 1, pi, 0, i);
    }
    solve_sys(g, ORC_FK_BT, m, bre + 1);
    if (m > 0) solve_sys(g, ORC_FK_BT, m, bim + 1);
    if (m == 0) {
      for (int i = 2; i <= nr - 1; ++i) {
        F(b, 3, 0, 0, i) = 0.0;
        F(b, 3, 0, 1, i) = -idrh * (bre[i + 1] - bre[i - 1]);
      }
      F(b, 3, 0, 0, 1) = 0.0;
      F(b, 3, 0, 1, 1) = 0.0;
      F(b, 3, 0, 0, nr) = 0.0;
      F(b, 3, 0, 1, nr) = -idrh * (3.0 * bre[nr] - 4.0 * bre[nr - 1] + bre[nr - 2]);
    } else {
      for (int i = 2; i <= nr - 1; ++i) {
        double ir = idr / (double)(i - 1);
        F(b, 3, pr, 0, i) = -ir * m * bim[i];
        F(b, 3, pi, 0, i) = ir * m * bre[i];
        F(b, 3, pr, 1, i) = -idrh * (bre[i + 1] - bre[i - 1]);
        F(b, 3, pi, 1, i) = -idrh * (bim[i + 1] - bim[i - 1]);
      }
      if (m == 1) {
        F(b, 3, pr, 0, 1) = -idr * m * bim[2];
        F(b, 3, pi, 0, 1) = idr * m * bre[2];
        F(b, 3, pr, 1, 1) = -idr * bre[2];
        F(b, 3, pi, 1, 1) = -idr * bim[2];
      } else {
        F(b, 3, pr, 0, 1) = 0.0;
        F(b, 3, pi, 0, 1) = 0.0;
        F(b, 3, pr, 1, 1) = 0.0;
        F(b, 3, pi, 1, 1) = 0.0;
      }
      {
        double ir = idr / (double)(nr - 1);
        F(b, 3, pr, 0, nr) = -ir * m * bim[nr];
        F(b, 3, pi, 0, nr) = ir * m * bre[nr];
        F(b, 3, pr, 1, nr) = -idrh * (3.0 * bre[nr] - 4.0 * bre[nr - 1] + bre[nr - 2]);
        F(b, 3, pi, 1, nr) = -idrh * (3.0 * bim[nr] - 4.0 * bim[nr - 1] + bim[nr - 2]);
      }
    }
  }
  free(bre);
}

/* =============================================================================
 * Plasma B-perp predictor-corrector: field_b_class.f03:360-506, 703-758, 836-879
 * b holds B_old on entry (components 1:2), receives the new B_perp.
 * ============================================================================= */
void orc_solve_bt_iter(const orc_grid* g, const double* dcu, const double* cu, double* b) {
  const int nr = g->nr, M = g->max_mode;
  const double idr = 1.0 / g->dr, idrh = 0.5 * idr;
  const double relax_idr2 = g->relax_fac * (idr * idr);
  double* buf = (double*)calloc(4 * ((size_t)nr + 1), sizeof(double));
  double *b1re = buf, *b1im = buf + (nr + 1), *b2re = buf + 2 * (nr + 1), *b2im = buf + 3 * (nr + 1);
  for (int m = 0; m <= M; ++m) {
    memset(buf, 0, sizeof(double) * 4 * ((size_t)nr + 1));
    if (m == 0) {
      /* f1 = djdxi, f2 = jay, f3 = b (old) */
      for (int i = 2; i <= nr; ++i) {
        b1re[i] = -F(dcu, 2, 0, 1, i) - F(b, 3, 0, 0, i) * relax_idr2;
        b2re[i] = F(dcu, 2, 0, 0, i) + idrh * (F(cu, 3, 0, 2, i + 1) - F(cu, 3, 0, 2, i - 1))
                  - F(b, 3, 0, 1, i) * relax_idr2;
      }
      b1re[1] = 0.0;
      b2re[1] = 0.0;
      b2re[2] = F(dcu, 2, 0, 0, 2) + idr * (F(cu, 3, 0, 2, 3) - F(cu, 3, 0, 2, 2)) - F(b, 3, 0, 1, 2) * relax_idr2;
      b1re[nr] = -F(dcu, 2, 0, 1, nr) - F(b, 3, 0, 0, nr) * relax_idr2;
      b2re[nr] = F(dcu, 2, 0, 0, nr) + idrh * (3.0 * F(cu, 3, 0, 2, nr) - 4.0 * F(cu, 3, 0, 2, nr - 1) + F(cu, 3, 0, 2, nr - 2))
                 - F(b, 3, 0, 1, nr) * relax_idr2;
      solve_sys(g, ORC_FK_BPLUS, 0, b1re + 1);
      solve_sys(g, ORC_FK_BMINUS, 0, b2re + 1);
      for (int i = 1; i <= nr; ++i) {
        F(b, 3, 0, 0, i) = b1re[i];
        F(b, 3, 0, 1, i) = b2re[i];
      }
      F(b, 3, 0, 0, 1) = 0.0;
      F(b, 3, 0, 1, 1) = 0.0;
    } else {
      const int pr = PRE(m), pi = PIM(m);
      double s1re, s1im, s2re, s2im;
#define BT_ITER_FILL(I)                                                                           \
  b1re[I] = s1re - s2im - (F(b, 3, pr, 0, I) - F(b, 3, pi, 1, I)) * relax_idr2;                   \
  b1im[I] = s1im + s2re - (F(b, 3, pi, 0, I) + F(b, 3, pr, 1, I)) * relax_idr2;                   \
  b2re[I] = s1re + s2im - (F(b, 3, pr, 0, I) + F(b, 3, pi, 1, I)) * relax_idr2;                   \
  b2im[I] = s1im - s2re - (F(b, 3, pi, 0, I) - F(b, 3, pr, 1, I)) * relax_idr2;
      for (int i = 2; i <= nr; ++i) {
        double ir = idr / (double)(i - 1);
        s1re = -F(dcu, 2, pr, 1, i) + m * F(cu, 3, pi, 2, i) * ir;
        s1im = -F(dcu, 2, pi, 1, i) - m * F(cu, 3, pr, 2, i) * ir;
        s2re = F(dcu, 2, pr, 0, i) + idrh * (F(cu, 3, pr, 2, i + 1) - F(cu, 3, pr, 2, i - 1));
        s2im = F(dcu, 2, pi, 0, i) + idrh * (F(cu, 3, pi, 2, i + 1) - F(cu, 3, pi, 2, i - 1));
        BT_ITER_FILL(i)
      }
      if (m == 1) {
        s1re = -F(dcu, 2, pr, 1, 1) + idr * m * F(cu, 3, pi, 2, 2);
        s1im = -F(dcu, 2, pi, 1, 1) - idr * m * F(cu, 3, pr, 2, 2);
        s2re = F(dcu, 2, pr, 0, 1) + idr * F(cu, 3, pr, 2, 2);
        s2im = F(dcu, 2, pi, 0, 1) + idr * F(cu, 3, pi, 2, 2);
      } else if (m % 2 == 0) {
        s1re = 0.0; s1im = 0.0; s2re = 0.0; s2im = 0.0;
      } else {
        s1re = idr * m * F(cu, 3, pi, 2, 2);
        s1im = idr * m * F(cu, 3, pr, 2, 2);
        s2re = idr * F(cu, 3, pr, 2, 2);
        s2im = idr * F(cu, 3, pi, 2, 2);
      }
      BT_ITER_FILL(1)
      {
        double ir = idr / (double)(nr - 1);
        s1re = -F(dcu, 2, pr, 1, nr) + m * F(cu, 3, pi, 2, nr) * ir;
        s1im = -F(dcu, 2, pi, 1, nr) - m * F(cu, 3, pr, 2, nr) * ir;
        s2re = F(dcu, 2, pr, 0, nr) + idrh * (3.0 * F(cu, 3, pr, 2, nr) - 4.0 * F(cu, 3, pr, 2, nr - 1) + F(cu, 3, pr, 2, nr - 2));
        s2im = F(dcu, 2, pi, 0, nr) + idrh * (3.0 * F(cu, 3, pi, 2, nr) - 4.0 * F(cu, 3, pi, 2, nr - 1) + F(cu, 3, pi, 2, nr - 2));
        BT_ITER_FILL(nr)
      }
#undef BT_ITER_FILL
      solve_sys(g, ORC_FK_BPLUS, m, b1re + 1);
      solve_sys(g, ORC_FK_BPLUS, m, b1im + 1);
      solve_sys(g, ORC_FK_BMINUS, m, b2re + 1);
      solve_sys(g, ORC_FK_BMINUS, m, b2im + 1);
      for (int i = 1; i <= nr; ++i) {
        F(b, 3, pr, 0, i) = 0.5 * (b1re[i] + b2re[i]);
        F(b, 3, pi, 0, i) = 0.5 * (b1im[i] + b2im[i]);
        F(b, 3, pr, 1, i) = 0.5 * (b1im[i] - b2im[i]);
        F(b, 3, pi, 1, i) = 0.5 * (-b1re[i] + b2re[i]);
      }
      if (m != 1) {
        F(b, 3, pr, 0, 1) = 0.0; F(b, 3, pi, 0, 1) = 0.0;
        F(b, 3, pr, 1, 1) = 0.0; F(b, 3, pi, 1, 1) = 0.0;
      }
    }
  }
  free(buf);
}

/* =============================================================================
 * Ez: field_e_class.f03:148-259 (set_source_ez), 261-296, 298-334
 * ============================================================================= */
void orc_solve_ez(const orc_grid* g, const double* cu, double* e) {
  const int nr = g->nr, M = g->max_mode;
  const double idr = 1.0 / g->dr, idrh = 0.5 * idr;
  double* bre = (double*)calloc(2 * (size_t)nr + 2, sizeof(double));
  double* bim = bre + nr + 1;
  for (int m = 0; m <= M; ++m) {
    memset(bre, 0, sizeof(double) * (2 * (size_t)nr + 2));
    if (m == 0) {
      double div = 0.0;
      for (int i = 2; i <= nr - 2; ++i) {
        double ir = idr / (double)(i - 1);
        bre[i] = idrh * (F(cu, 3, 0, 0, i + 1) - F(cu, 3, 0, 0, i - 1)) + ir * F(cu, 3, 0, 0, i);
        div = div + bre[i] * (double)(i - 1);
      }
      {
        double ir = idr / (double)(nr - 2);
        bre[nr - 1] = idrh * (F(cu, 3, 0, 0, nr) - F(cu, 3, 0, 0, nr - 2)) + ir * F(cu, 3, 0, 0, nr - 1);
        ir = idr / (double)(nr - 1);
        bre[nr] = idr * (F(cu, 3, 0, 0, nr) - F(cu, 3, 0, 0, nr - 1)) + ir * F(cu, 3, 0, 0, nr);
        div = div - idrh * (F(cu, 3, 0, 0, nr - 2) + F(cu, 3, 0, 0, nr - 1)) * ((double)nr - 2.5);
      }
      bre[1] = div;                 /* MPI_REDUCE on one rank */
      bre[1] = -8.0 * bre[1];
    } else {
      const int pr = PRE(m), pi = PIM(m);
      for (int i = 2; i <= nr; ++i) {
        double ir = idr / (double)(i - 1);
        bre[i] = idrh * (F(cu, 3, pr, 0, i + 1) - F(cu, 3, pr, 0, i - 1)) + ir * F(cu, 3, pr, 0, i)
                 - m * ir * F(cu, 3, pi, 1, i);
        bim[i] = idrh * (F(cu, 3, pi, 0, i + 1) - F(cu, 3, pi, 0, i - 1)) + ir * F(cu, 3, pi, 0, i)
                 + m * ir * F(cu, 3, pr, 1, i);
      }
      if (m % 2 == 0) {
        bre[1] = 2.0 * idr * F(cu, 3, pr, 0, 2) - m * idr * F(cu, 3, pi, 1, 2);
        bim[1] = 2.0 * idr * F(cu, 3, pi, 0, 2) + m * idr * F(cu, 3, pr, 1, 2);
      } else {
        bre[1] = 0.0;
        bim[1] = 0.0;
        if (m == 1) {
          double ir = idr;
          bre[2] = idr * (F(cu, 3, pr, 0, 3) - F(cu, 3, pr, 0, 2)) + ir * F(cu, 3, pr, 0, 2) - m * ir * F(cu, 3, pi, 1, 2);
          bim[2] = idr * (F(cu, 3, pi, 0, 3) - F(cu, 3, pi, 0, 2)) + ir * F(cu, 3, pi, 0, 2) + m * ir * F(cu, 3, pr, 1, 2);
        }
      }
      {
        double ir = idr / (double)(nr - 1);
        bre[nr] = idrh * (3.0 * F(cu, 3, pr, 0, nr) - 4.0 * F(cu, 3, pr, 0, nr - 1) + F(cu, 3, pr, 0, nr - 2))
                  + ir * F(cu, 3, pr, 0, nr) - m * ir * F(cu, 3, pi, 1, nr);
        bim[nr] = idrh * (3.0 * F(cu, 3, pi, 0, nr) - 4.0 * F(cu, 3, pi, 0, nr - 1) + F(cu, 3, pi, 0, nr - 2))
                  + ir * F(cu, 3, pi, 0, nr) + m * ir * F(cu, 3, pr, 1, nr);
      }
    }
    solve_sys(g, ORC_FK_EZ, m, bre + 1);
    if (m > 0) solve_sys(g, ORC_FK_EZ, m, bim + 1);
    int pr = m == 0 ? 0 : PRE(m), pi = m == 0 ? 0 : PIM(m);
    for (int i = 1; i <= nr; ++i) {
      F(e, 3, pr, 2, i) = bre[i];
      if (m > 0) F(e, 3, pi, 2, i) = bim[i];
    }
    if (m > 0) { F(e, 3, pr, 2, 1) = 0.0; F(e, 3, pi, 2, 1) = 0.0; }
  }
  free(bre);
}

/* =============================================================================
 * E-perp from B and psi: field_e_class.f03:412-514
 * ============================================================================= */
void orc_solve_et(const orc_grid* g, const double* b, const double* psi, double* e) {
  const int nr = g->nr, M = g->max_mode;
  const double idr = 1.0 / g->dr, idrh = idr * 0.5;
  for (int i = 1; i <= nr; ++i) {
    F(e, 3, 0, 0, i) = F(b, 3, 0, 1, i) - idrh * (F(psi, 1, 0, 0, i + 1) - F(psi, 1, 0, 0, i - 1));
    F(e, 3, 0, 1, i) = -F(b, 3, 0, 0, i);
  }
  F(e, 3, 0, 0, 1) = 0.0;
  F(e, 3, 0, 1, 1) = 0.0;
  F(e, 3, 0, 0, nr) = F(b, 3, 0, 1, nr) + idrh * (4.0 * F(psi, 1, 0, 0, nr - 1) - F(psi, 1, 0, 0, nr - 2) - 3.0 * F(psi, 1, 0, 0, nr));
  for (int m = 1; m <= M; ++m) {
    const int pr = PRE(m), pi = PIM(m);
    for (int i = 2; i <= nr; ++i) {
      double ir = idr / (double)(i - 1);
      F(e, 3, pr, 0, i) = F(b, 3, pr, 1, i) - idrh * (F(psi, 1, pr, 0, i + 1) - F(psi, 1, pr, 0, i - 1));
      F(e, 3, pi, 0, i) = F(b, 3, pi, 1, i) - idrh * (F(psi, 1, pi, 0, i + 1) - F(psi, 1, pi, 0, i - 1));
      F(e, 3, pr, 1, i) = -F(b, 3, pr, 0, i) + ir * m * F(psi, 1, pi, 0, i);
      F(e, 3, pi, 1, i) = -F(b, 3, pi, 0, i) - ir * m * F(psi, 1, pr, 0, i);
    }
    if (m == 1) {
      F(e, 3, pr, 0, 1) = F(b, 3, pr, 1, 1) - idr * F(psi, 1, pr, 0, 2);
      F(e, 3, pi, 0, 1) = F(b, 3, pi, 1, 1) - idr * F(psi, 1, pi, 0, 2);
      F(e, 3, pr, 1, 1) = -F(b, 3, pr, 0, 1) + idr * F(psi, 1, pi, 0, 2);
      F(e, 3, pi, 1, 1) = -F(b, 3, pi, 0, 1) - idr * F(psi, 1, pr, 0, 2);
    } else {
      F(e, 3, pr, 0, 1) = 0.0; F(e, 3, pi, 0, 1) = 0.0;
      F(e, 3, pr, 1, 1) = 0.0; F(e, 3, pi, 1, 1) = 0.0;
    }
    F(e, 3, pr, 0, nr) = F(b, 3, pr, 1, nr) + idrh * (4.0 * F(psi, 1, pr, 0, nr - 1) - F(psi, 1, pr, 0, nr - 2) - 3.0 * F(psi, 1, pr, 0, nr));
    F(e, 3, pi, 0, nr) = F(b, 3, pi, 1, nr) + idrh * (4.0 * F(psi, 1, pi, 0, nr - 1) - F(psi, 1, pi, 0, nr - 2) - 3.0 * F(psi, 1, pi, 0, nr));
  }
}

/* =============================================================================
 * dJ_perp/dxi = acu - div(amu): field_src_class.f03:273-405
 * ============================================================================= */
void orc_solve_djdxi(const orc_grid* g, const double* acu, const double* amu, double* dcu) {
  const int nr = g->nr, M = g->max_mode;
  const double idr = 1.0 / g->dr, idrh = idr * 0.5;
#define A(p, c, i) F(acu, 2, p, c, i)
#define U(p, c, i) F(amu, 3, p, c, i)
#define D(p, c, i) F(dcu, 2, p, c, i)
  for (int i = 2; i <= nr; ++i) {
    double ir = idr / (double)(i - 1);
    D(0, 0, i) = A(0, 0, i) - idrh * (U(0, 0, i + 1) - U(0, 0, i - 1)) - ir * U(0, 0, i);
    D(0, 1, i) = A(0, 1, i) - idrh * (U(0, 1, i + 1) - U(0, 1, i - 1)) - ir * U(0, 1, i);
  }
  D(0, 0, 1) = 0.0;
  D(0, 1, 1) = 0.0;
  {
    double ir = idr / (double)(nr - 1);
    D(0, 0, nr) = A(0, 0, nr) + idrh * (4.0 * U(0, 0, nr - 1) - U(0, 0, nr - 2) - 3.0 * U(0, 0, nr)) - ir * U(0, 0, nr);
    D(0, 1, nr) = A(0, 1, nr) + idrh * (4.0 * U(0, 1, nr - 1) - U(0, 1, nr - 2) - 3.0 * U(0, 1, nr)) - ir * U(0, 1, nr);
  }
  for (int m = 1; m <= M; ++m) {
    const int r = PRE(m), s = PIM(m);
    for (int i = 2; i <= nr; ++i) {
      double ir = idr / (double)(i - 1);
      D(r, 0, i) = A(r, 0, i) - idrh * (U(r, 0, i + 1) - U(r, 0, i - 1)) - ir * U(r, 0, i) + m * ir * U(s, 1, i);
      D(r, 1, i) = A(r, 1, i) - idrh * (U(r, 1, i + 1) - U(r, 1, i - 1)) - ir * U(r, 1, i) + m * ir * U(s, 2, i);
      D(s, 0, i) = A(s, 0, i) - idrh * (U(s, 0, i + 1) - U(s, 0, i - 1)) - ir * U(s, 0, i) - m * ir * U(r, 1, i);
      D(s, 1, i) = A(s, 1, i) - idrh * (U(s, 1, i + 1) - U(s, 1, i - 1)) - ir * U(s, 1, i) - m * ir * U(r, 2, i);
    }
    if (m == 1) {
      D(r, 0, 1) = A(r, 0, 1) - 2.0 * idr * U(r, 0, 2) + m * idr * U(s, 1, 2);
      D(r, 1, 1) = A(r, 1, 1) - 2.0 * idr * U(r, 1, 2) + m * idr * U(s, 2, 2);
      D(s, 0, 1) = A(s, 0, 1) - 2.0 * idr * U(s, 0, 2) - m * idr * U(r, 1, 2);
      D(s, 1, 1) = A(s, 1, 1) - 2.0 * idr * U(s, 1, 2) - m * idr * U(r, 2, 2);
    } else {
      D(r, 0, 1) = 0.0; D(r, 1, 1) = 0.0; D(s, 0, 1) = 0.0; D(s, 1, 1) = 0.0;
      if (m == 2) {
        double ir = idr;
        D(r, 0, 2) = A(r, 0, 2) - idr * (U(r, 0, 3) - U(r, 0, 2)) - ir * U(r, 0, 2) + m * ir * U(s, 1, 2);
        D(r, 1, 2) = A(r, 1, 2) - idr * (U(r, 1, 3) - U(r, 1, 2)) - ir * U(r, 1, 2) + m * ir * U(s, 2, 2);
        D(s, 0, 2) = A(s, 0, 2) - idr * (U(s, 0, 3) - U(s, 0, 2)) - ir * U(s, 0, 2) - m * ir * U(r, 1, 2);
        D(s, 1, 2) = A(s, 1, 2) - idr * (U(s, 1, 3) - U(s, 1, 2)) - ir * U(s, 1, 2) - m * ir * U(r, 2, 2);
      }
    }
    {
      double ir = idr / (double)(nr - 1);
      D(r, 0, nr) = A(r, 0, nr) + idrh * (4.0 * U(r, 0, nr - 1) - U(r, 0, nr - 2) - 3.0 * U(r, 0, nr)) - ir * U(r, 0, nr) + m * ir * U(s, 1, nr);
      D(r, 1, nr) = A(r, 1, nr) + idrh * (4.0 * U(r, 1, nr - 1) - U(r, 1, nr - 2) - 3.0 * U(r, 1, nr)) - ir * U(r, 1, nr) + m * ir * U(s, 2, nr);
      D(s, 0, nr) = A(s, 0, nr) + idrh * (4.0 * U(s, 0, nr - 1) - U(s, 0, nr - 2) - 3.0 * U(s, 0, nr)) - ir * U(s, 0, nr) - m * ir * U(r, 1, nr);
      D(s, 1, nr) = A(s, 1, nr) + idrh * (4.0 * U(s, 1, nr - 1) - U(s, 1, nr - 2) - 3.0 * U(s, 1, nr)) - ir * U(s, 1, nr) - m * ir * U(r, 2, nr);
    }
  }
#undef A
#undef U
#undef D
}

/* =============================================================================
 * convergence_tester: simulation_class.f03:522-606 (dim = 2, infinity norm)
 * ============================================================================= */
void orc_conv_record(const orc_grid* g, const double* b, double* s_re, double* s_im) {
  const int nr = g->nr, M = g->max_mode;
  for (int i = 1; i <= nr; ++i) { s_re[i - 1] = 0.0; s_im[i - 1] = 0.0; }
  for (int m = 0; m <= M; ++m) {
    int pr = m == 0 ? 0 : PRE(m);
    for (int i = 1; i <= nr; ++i) s_re[i - 1] = s_re[i - 1] + fabs(F(b, 3, pr, 1, i));
    if (m == 0) continue;
    for (int i = 1; i <= nr; ++i) s_im[i - 1] = s_im[i - 1] + fabs(F(b, 3, PIM(m), 1, i));
  }
}

void orc_conv_compare(const orc_grid* g, const double* b, double* s_re, double* s_im,
                      double* rel_res, double* abs_res) {
  const int nr = g->nr, M = g->max_mode;
  double mx = 0.0;
  for (int i = 0; i < nr; ++i) {
    double v = s_re[i] * s_re[i] + s_im[i] * s_im[i];
    if (i == 0 || v > mx) mx = v;
  }
  double old_norm = sqrt(mx);
  for (int m = 0; m <= M; ++m) {
    int pr = m == 0 ? 0 : PRE(m);
    for (int i = 1; i <= nr; ++i) s_re[i - 1] = s_re[i - 1] - fabs(F(b, 3, pr, 1, i));
    if (m == 0) continue;
    for (int i = 1; i <= nr; ++i) s_im[i - 1] = s_im[i - 1] - fabs(F(b, 3, PIM(m), 1, i));
  }
  mx = 0.0;
  for (int i = 0; i < nr; ++i) {
    double v = s_re[i] * s_re[i] + s_im[i] * s_im[i];
    if (i == 0 || v > mx) mx = v;
  }
  *abs_res = sqrt(mx);
  if (old_norm > 2.220446049250313e-16) *rel_res = *abs_res / old_norm;   /* epsilon(1.0d0) */
  else *rel_res = 1.7976931348623157e308;                                 /* huge(1.0) */
}

/* =============================================================================
 * Plasma charge deposit: part2d_class.f03:231-359 (accumulates into qf)
 * ============================================================================= */
/* ufield::smooth_f1 (ufield_class.f03:274-339) on every mode part and component of a
 * deposit field, single rank (idproc = 0, noff = 0): kernel = stencil / sum(stencil) with
 * stencil (1, 2, 1); node 1 uses the axis form where ax_smooth is set for the mode and
 * component (else 0), node 2 the near-axis form, nodes j >= 3 the r-weighted form with
 * r_idx = j - 1; the guard nodes are left as they are.  The ax_smooth switches per mode are
 * those of field_rho / field_jay / field_djdxi::smooth (field_src_class.f03:114-118,
 * 181-193, 256-266). */
void orc_smooth(const orc_grid* g, int kind, double* f) {
  const int nc = kind == 0 ? 1 : (kind == 1 ? 3 : 2);
  const double st[3] = {1.0, 2.0, 1.0};
  const double sum = st[0] + st[1] + st[2];
  const double km = st[0] / sum, k0 = st[1] / sum, kp = st[2] / sum;
  double* tmp = (double*)malloc((size_t)(g->nr + 2) * sizeof(double));
  for (int p = 0; p < nparts(g); ++p) {
    const int m = (p + 1) / 2;
    for (int c = 0; c < nc; ++c) {
      int ax;
      if (kind == 0) ax = m == 0;
      else if (kind == 1) ax = m == 0 ? (c == 2) : (m == 1 ? (c < 2) : 0);
      else ax = m == 1;
      double* v = &F(f, nc, p, c, 0);
      tmp[1] = ax ? (k0 + kp) * v[1] + 8.0 * kp * v[2] : 0.0;
      tmp[2] = k0 * v[2] + 0.125 * km * v[1] + 2.0 * kp * v[3];
      for (int j = 3; j <= g->nr; ++j) {
        const double r = (double)(j - 1);
        tmp[j] = k0 * v[j] + (1.0 - 1.0 / r) * km * v[j - 1] + (1.0 + 1.0 / r) * kp * v[j + 1];
      }
      for (int j = 1; j <= g->nr; ++j) v[j] = tmp[j];
    }
  }
  free(tmp);
}

static void qdeposit_axis_scale(const orc_grid* g, double* qf) {
  const int nr = g->nr, M = g->max_mode;
  F(qf, 1, 0, 0, 0) = 0.0;
  F(qf, 1, 0, 0, 1) = 8.0 * F(qf, 1, 0, 0, 1);
  for (int j = 2; j <= nr + 1; ++j) {
    double ir = 1.0 / (double)(j - 1);
    F(qf, 1, 0, 0, j) = F(qf, 1, 0, 0, j) * ir;
  }
  for (int m = 1; m <= M; ++m) {
    F(qf, 1, PRE(m), 0, 0) = 0.0; F(qf, 1, PIM(m), 0, 0) = 0.0;
    F(qf, 1, PRE(m), 0, 1) = 0.0; F(qf, 1, PIM(m), 0, 1) = 0.0;
    for (int j = 2; j <= nr + 1; ++j) {
      double ir = 1.0 / (double)(j - 1);
      F(qf, 1, PRE(m), 0, j) = F(qf, 1, PRE(m), 0, j) * ir;
      F(qf, 1, PIM(m), 0, j) = F(qf, 1, PIM(m), 0, j) * ir;
    }
  }
}

void orc_qdeposit(const orc_grid* g, int64_t np, const double* x, const double* y,
                  const double* q, double* qf) {
  const int M = g->max_mode;
  const double idr = 1.0 / g->dr;
  for (int64_t pp = 0; pp < np; ++pp) {
    double pos = sqrt(x[pp] * x[pp] + y[pp] * y[pp]) * idr;
    double ph0r = x[pp] / pos * idr, ph0i = -y[pp] / pos * idr;
    if (!(pos >= 0.0 && pos < 1.0e9)) continue;
    int nn = (int)floor(pos);
    pos = pos - (double)nn;
    nn = nn + 1;
    if (nn < 1 || nn > g->nr) continue;  /* radius rounds onto/over the edge: nothing deposited */
    double wt0 = 1.0 - pos, wt1 = pos;
    double phr = 1.0 * q[pp], phi = 0.0 * q[pp];
    F(qf, 1, 0, 0, nn) = F(qf, 1, 0, 0, nn) + wt0 * phr;
    F(qf, 1, 0, 0, nn + 1) = F(qf, 1, 0, 0, nn + 1) + wt1 * phr;
    for (int m = 1; m <= M; ++m) {
      double t = phr * ph0r - phi * ph0i;
      phi = phr * ph0i + phi * ph0r;
      phr = t;
      F(qf, 1, PRE(m), 0, nn) = F(qf, 1, PRE(m), 0, nn) + wt0 * phr;
      F(qf, 1, PIM(m), 0, nn) = F(qf, 1, PIM(m), 0, nn) + wt0 * phi;
      F(qf, 1, PRE(m), 0, nn + 1) = F(qf, 1, PRE(m), 0, nn + 1) + wt1 * phr;
      F(qf, 1, PIM(m), 0, nn + 1) = F(qf, 1, PIM(m), 0, nn + 1) + wt1 * phi;
    }
  }
  qdeposit_axis_scale(g, qf);
}

/* =============================================================================
 * Field gather helpers: interp_part2d.f03:28-171
 * ============================================================================= */
/* idx outside 1..nr (a radius that rounds onto the outer edge, or a NaN) marks a
 * particle that gathers zero fields and deposits nothing: the reference would read
 * and write past the upper guard cell there. */
typedef struct { double w0, w1, pcos, psin; int idx; } interp_info;
#define II_OK(g, ii) ((ii).idx >= 1 && (ii).idx <= (g)->nr)

static inline interp_info gen_interp_info(double x, double y, double idr) {  /* :28-65 */
  interp_info ii;
  double pos = sqrt(x * x + y * y);
  ii.pcos = x / pos;
  ii.psin = y / pos;
  pos = pos * idr;
  if (!(pos >= 0.0 && pos < 1.0e9)) { ii.idx = 0; ii.w0 = ii.w1 = 0.0; return ii; }
  int ip = (int)pos;
  ii.idx = ip + 1;
  pos = pos - (double)ip;
  ii.w0 = 1.0 - pos;
  ii.w1 = pos;
  return ii;
}

/* vector gather of a 3-component field (:67-109) */
static inline void interp_vec(const orc_grid* g, const double* f, const interp_info* ii, double fp[3]) {
  const int M = g->max_mode;
  const int i0 = ii->idx, i1 = ii->idx + 1;
  if (!II_OK(g, *ii)) { fp[0] = fp[1] = fp[2] = 0.0; return; }
  for (int c = 0; c < 3; ++c) {
    fp[c] = 0.0;
    fp[c] = fp[c] + F(f, 3, 0, c, i0) * ii->w0;
    fp[c] = fp[c] + F(f, 3, 0, c, i1) * ii->w1;
  }
  double phr = 1.0, phi = 0.0;
  for (int m = 1; m <= M; ++m) {
    double t = phr * ii->pcos - phi * ii->psin;
    phi = phr * ii->psin + phi * ii->pcos;
    phr = t;
    double pre = 2.0 * phr, pim = 2.0 * phi;
    for (int c = 0; c < 3; ++c) {
      fp[c] = fp[c] + (F(f, 3, PRE(m), c, i0) * pre - F(f, 3, PIM(m), c, i0) * pim) * ii->w0;
      fp[c] = fp[c] + (F(f, 3, PRE(m), c, i1) * pre - F(f, 3, PIM(m), c, i1) * pim) * ii->w1;
    }
  }
}

static inline double interp_scalar(const orc_grid* g, const double* f, const interp_info* ii) {  /* :111-153 */
  const int M = g->max_mode;
  const int i0 = ii->idx, i1 = ii->idx + 1;
  double fp = 0.0;
  if (!II_OK(g, *ii)) return 0.0;
  fp = fp + F(f, 1, 0, 0, i0) * ii->w0;
  fp = fp + F(f, 1, 0, 0, i1) * ii->w1;
  double phr = 1.0, phi = 0.0;
  for (int m = 1; m <= M; ++m) {
    double t = phr * ii->pcos - phi * ii->psin;
    phi = phr * ii->psin + phi * ii->pcos;
    phr = t;
    double pre = 2.0 * phr, pim = 2.0 * phi;
    fp = fp + (F(f, 1, PRE(m), 0, i0) * pre - F(f, 1, PIM(m), 0, i0) * pim) * ii->w0;
    fp = fp + (F(f, 1, PRE(m), 0, i1) * pre - F(f, 1, PIM(m), 0, i1) * pim) * ii->w1;
  }
  return fp;
}

/* =============================================================================
 * Current / acceleration / momentum-flux deposit:
 *   amjdeposit_robust part2d_class.f03:746-1010, amjdeposit_std 478-744
 * cu (3 comps), amu (3), dcu (2) accumulate; the axis fix and 1/(j-1) scaling follow.
 * ============================================================================= */
static void amj_one(const orc_grid* g, int push_type, double qbm, double qtmh, double idt,
                    double idr, int64_t pp, const double* x, const double* y, const double* px,
                    const double* py, const double* pz, const double* q, double* gamma, double* psi,
                    const double* ef, const double* bf, double* cu, double* amu, double* dcu) {
  const int M = g->max_mode;
  interp_info ii = gen_interp_info(x[pp], y[pp], idr);
  double ep[3], bp[3], wp[3], u0[3], u[3], utmp[3], du[3], u2[3];
  interp_vec(g, ef, &ii, ep);
  interp_vec(g, bf, &ii, bp);
  wp[0] = ep[0] - bp[1];
  wp[1] = ep[1] + bp[0];
  wp[2] = ep[2];
  u0[0] = px[pp] * ii.pcos + py[pp] * ii.psin;
  u0[1] = py[pp] * ii.pcos - px[pp] * ii.psin;
  u0[2] = pz[pp];
  double ipsi;
  if (push_type == ORC_PUSH_ROBUST) {
    double gam = sqrt(1.0 + u0[0] * u0[0] + u0[1] * u0[1] + u0[2] * u0[2]);
    double qtmh1 = qtmh * gam / (gam - u0[2]);
    for (int c = 0; c < 3; ++c) { ep[c] = ep[c] * qtmh1; utmp[c] = u0[c] + ep[c]; }
    gam = sqrt(1.0 + utmp[0] * utmp[0] + utmp[1] * utmp[1] + utmp[2] * utmp[2]);
    double qtmh2 = qtmh / (gam - utmp[2]);
    for (int c = 0; c < 3; ++c) bp[c] = bp[c] * qtmh2;
  } else {
    double gam = sqrt(1.0 + u0[0] * u0[0] + u0[1] * u0[1] + u0[2] * u0[2]);
    double qtmh2 = qtmh / (1.0 - qbm * psi[pp]);
    double qtmh1 = qtmh2 * gam;
    for (int c = 0; c < 3; ++c) bp[c] = bp[c] * qtmh2;
    for (int c = 0; c < 3; ++c) utmp[c] = u0[c] + ep[c] * qtmh1;
  }
  u[0] = utmp[0] + utmp[1] * bp[2] - utmp[2] * bp[1];
  u[1] = utmp[1] + utmp[2] * bp[0] - utmp[0] * bp[2];
  u[2] = utmp[2] + utmp[0] * bp[1] - utmp[1] * bp[0];
  double ostq = 2.0 / (1.0 + bp[0] * bp[0] + bp[1] * bp[1] + bp[2] * bp[2]);
  for (int c = 0; c < 3; ++c) bp[c] = bp[c] * ostq;
  {
    double t0 = utmp[0] + u[1] * bp[2] - u[2] * bp[1];
    double t1 = utmp[1] + u[2] * bp[0] - u[0] * bp[2];
    double t2 = utmp[2] + u[0] * bp[1] - u[1] * bp[0];
    utmp[0] = t0; utmp[1] = t1; utmp[2] = t2;
  }
  if (push_type == ORC_PUSH_ROBUST) {
    for (int c = 0; c < 3; ++c) u[c] = utmp[c] + ep[c];
  } else {
    double gam = sqrt(1.0 + utmp[0] * utmp[0] + utmp[1] * utmp[1] + utmp[2] * utmp[2]);
    double qtmh2 = qtmh / (1.0 - qbm * psi[pp]);
    double qtmh1 = qtmh2 * gam;
    for (int c = 0; c < 3; ++c) u[c] = utmp[c] + ep[c] * qtmh1;
  }
  /* time-centred values and deposit (robust :857-909, std :602-662) */
  du[0] = idt * (u[0] - u0[0]);
  du[1] = idt * (u[1] - u0[1]);
  for (int c = 0; c < 3; ++c) u[c] = 0.5 * (u[c] + u0[c]);
  gamma[pp] = sqrt(1.0 + u[0] * u[0] + u[1] * u[1] + u[2] * u[2]);
  if (push_type == ORC_PUSH_ROBUST) {
    ipsi = 1.0 / (gamma[pp] - u[2]);
    psi[pp] = (1.0 - 1.0 / ipsi) / qbm;
  } else {
    ipsi = 1.0 / (1.0 - qbm * psi[pp]);
  }
  double dpsi = qbm * (wp[2] - (wp[0] * u[0] + wp[1] * u[1]) * ipsi);
  du[0] = du[0] + u[0] * dpsi * ipsi;
  du[1] = du[1] + u[1] * dpsi * ipsi;
  u2[0] = u[0] * u[0] * ipsi;
  u2[1] = u[0] * u[1] * ipsi;
  u2[2] = u[1] * u[1] * ipsi;
  double ph0r = ii.pcos, ph0i = -ii.psin;
  double phr = 1.0 * q[pp] * ipsi, phi = 0.0 * q[pp] * ipsi;
  const double wj[2] = {ii.w0, ii.w1};
  if (!II_OK(g, ii)) return;
  for (int j = 0; j < 2; ++j) {
    int n = ii.idx + j;
    double w = wj[j] * phr;
    for (int c = 0; c < 3; ++c) F(cu, 3, 0, c, n) = F(cu, 3, 0, c, n) + w * u[c];
    for (int c = 0; c < 2; ++c) F(dcu, 2, 0, c, n) = F(dcu, 2, 0, c, n) + w * du[c];
    for (int c = 0; c < 3; ++c) F(amu, 3, 0, c, n) = F(amu, 3, 0, c, n) + w * u2[c];
  }
  for (int m = 1; m <= M; ++m) {
    double t = phr * ph0r - phi * ph0i;
    phi = phr * ph0i + phi * ph0r;
    phr = t;
    const int r = PRE(m), s = PIM(m);
    for (int j = 0; j < 2; ++j) {
      int n = ii.idx + j;
      double w = wj[j] * phr;
      for (int c = 0; c < 3; ++c) F(cu, 3, r, c, n) = F(cu, 3, r, c, n) + w * u[c];
      for (int c = 0; c < 2; ++c) F(dcu, 2, r, c, n) = F(dcu, 2, r, c, n) + w * du[c];
      for (int c = 0; c < 3; ++c) F(amu, 3, r, c, n) = F(amu, 3, r, c, n) + w * u2[c];
      w = wj[j] * phi;
      for (int c = 0; c < 3; ++c) F(cu, 3, s, c, n) = F(cu, 3, s, c, n) + w * u[c];
      for (int c = 0; c < 2; ++c) F(dcu, 2, s, c, n) = F(dcu, 2, s, c, n) + w * du[c];
      for (int c = 0; c < 3; ++c) F(amu, 3, s, c, n) = F(amu, 3, s, c, n) + w * u2[c];
    }
  }
}

/* axis fixes and 1/(j-1) scaling: part2d_class.f03:914-1005 (robust), 658-740 (std) */
static void amj_axis_scale(const orc_grid* g, double* cu, double* amu, double* dcu) {
  const int nr = g->nr, M = g->max_mode;
  for (int c = 0; c < 3; ++c) { F(cu, 3, 0, c, 0) = 0.0; F(amu, 3, 0, c, 0) = 0.0; }
  for (int c = 0; c < 2; ++c) F(dcu, 2, 0, c, 0) = 0.0;
  F(cu, 3, 0, 0, 1) = 0.0; F(cu, 3, 0, 1, 1) = 0.0; F(cu, 3, 0, 2, 1) = 8.0 * F(cu, 3, 0, 2, 1);
  F(dcu, 2, 0, 0, 1) = 0.0; F(dcu, 2, 0, 1, 1) = 0.0;
  for (int c = 0; c < 3; ++c) F(amu, 3, 0, c, 1) = 0.0;
  for (int m = 1; m <= M; ++m) {
    for (int h = 0; h < 2; ++h) {
      int p = h == 0 ? PRE(m) : PIM(m);
      for (int c = 0; c < 3; ++c) { F(cu, 3, p, c, 0) = 0.0; F(amu, 3, p, c, 0) = 0.0; }
      for (int c = 0; c < 2; ++c) F(dcu, 2, p, c, 0) = 0.0;
      if (m == 1) {
        F(cu, 3, p, 0, 1) = 8.0 * F(cu, 3, p, 0, 1);
        F(cu, 3, p, 1, 1) = 8.0 * F(cu, 3, p, 1, 1);
        F(cu, 3, p, 2, 1) = 0.0;
        F(dcu, 2, p, 0, 1) = 8.0 * F(dcu, 2, p, 0, 1);
        F(dcu, 2, p, 1, 1) = 8.0 * F(dcu, 2, p, 1, 1);
        for (int c = 0; c < 3; ++c) F(amu, 3, p, c, 1) = 0.0;
      } else if (m == 2) {
        for (int c = 0; c < 3; ++c) F(cu, 3, p, c, 1) = 0.0;
        for (int c = 0; c < 2; ++c) F(dcu, 2, p, c, 1) = 0.0;
        for (int c = 0; c < 3; ++c) F(amu, 3, p, c, 1) = 8.0 * F(amu, 3, p, c, 1);
      } else {
        for (int c = 0; c < 3; ++c) F(cu, 3, p, c, 1) = 0.0;
        for (int c = 0; c < 2; ++c) F(dcu, 2, p, c, 1) = 0.0;
        for (int c = 0; c < 3; ++c) F(amu, 3, p, c, 1) = 0.0;
      }
    }
  }
  for (int p = 0; p < nparts(g); ++p) {
    for (int j = 2; j <= nr + 1; ++j) {
      double ir = 1.0 / (double)(j - 1);
      for (int c = 0; c < 3; ++c) F(cu, 3, p, c, j) = F(cu, 3, p, c, j) * ir;
      for (int c = 0; c < 2; ++c) F(dcu, 2, p, c, j) = F(dcu, 2, p, c, j) * ir;
      for (int c = 0; c < 3; ++c) F(amu, 3, p, c, j) = F(amu, 3, p, c, j) * ir;
    }
  }
}

void orc_amjdeposit(const orc_grid* g, int push_type, double qbm, double dt, int64_t np,
                    const double* x, const double* y, const double* px, const double* py,
                    const double* pz, const double* q, double* gamma, double* psi,
                    const double* ef, const double* bf, double* cu, double* amu, double* dcu,
                    int nthreads) {
  const double idt = 1.0 / dt, qtmh = 0.5 * qbm * dt, idr = 1.0 / g->dr;
  if (nthreads <= 1) {
    for (int64_t pp = 0; pp < np; ++pp)
      amj_one(g, push_type, qbm, qtmh, idt, idr, pp, x, y, px, py, pz, q, gamma, psi, ef, bf, cu, amu, dcu);
  } else {
    /* thread-private deposit arrays summed afterwards (CPU baseline only) */
    const size_t n3 = (size_t)nparts(g) * 3 * NR2, n2 = (size_t)nparts(g) * 2 * NR2;
    double* priv = (double*)calloc((size_t)nthreads * (2 * n3 + n2), sizeof(double));
#pragma omp parallel num_threads(nthreads)
    {
#ifdef _OPENMP
      int t = omp_get_thread_num();
#else
      int t = 0;
#endif
      double* pc = priv + (size_t)t * (2 * n3 + n2);
      double* pa = pc + n3;
      double* pd = pa + n3;
#pragma omp for schedule(static)
      for (int64_t pp = 0; pp < np; ++pp)
        amj_one(g, push_type, qbm, qtmh, idt, idr, pp, x, y, px, py, pz, q, gamma, psi, ef, bf, pc, pa, pd);
#pragma omp for schedule(static)
      for (int64_t k = 0; k < (int64_t)n3; ++k) {
        double sc = 0.0, sa = 0.0;
        for (int u = 0; u < nthreads; ++u) {
          sc += priv[(size_t)u * (2 * n3 + n2) + (size_t)k];
          sa += priv[(size_t)u * (2 * n3 + n2) + n3 + (size_t)k];
        }
        cu[k] += sc;
        amu[k] += sa;
      }
#pragma omp for schedule(static)
      for (int64_t k = 0; k < (int64_t)n2; ++k) {
        double sd = 0.0;
        for (int u = 0; u < nthreads; ++u) sd += priv[(size_t)u * (2 * n3 + n2) + 2 * n3 + (size_t)k];
        dcu[k] += sd;
      }
    }
    free(priv);
  }
  amj_axis_scale(g, cu, amu, dcu);
}

/* =============================================================================
 * Momentum push: push_u_robust part2d_class.f03:1879-1965, push_u_std 1790-1877
 * ============================================================================= */
static inline void push_u_one(const orc_grid* g, int push_type, double qbm, double qtmh, double idr,
                              int64_t pp, const double* x, const double* y, double* px, double* py,
                              double* pz, double* gamma, const double* psi, const double* ef,
                              const double* bf) {
  interp_info ii = gen_interp_info(x[pp], y[pp], idr);
  double ep[3], bp[3], utmp[3], p[3];
  interp_vec(g, ef, &ii, ep);
  interp_vec(g, bf, &ii, bp);
  /* transform_to_cartesian, interp_part2d.f03:155-171 */
  double t = ep[0] * ii.pcos - ep[1] * ii.psin;
  ep[1] = ep[0] * ii.psin + ep[1] * ii.pcos;
  ep[0] = t;
  t = bp[0] * ii.pcos - bp[1] * ii.psin;
  bp[1] = bp[0] * ii.psin + bp[1] * ii.pcos;
  bp[0] = t;
  p[0] = px[pp]; p[1] = py[pp]; p[2] = pz[pp];
  double qtmh1, qtmh2;
  if (push_type == ORC_PUSH_ROBUST) {
    double gam = sqrt(1.0 + p[0] * p[0] + p[1] * p[1] + p[2] * p[2]);
    qtmh1 = qtmh / (gam - p[2]);
    qtmh2 = qtmh1 * gam;
  } else {
    qtmh1 = qtmh / (1.0 - qbm * psi[pp]);
    qtmh2 = qtmh1 * gamma[pp];
  }
  for (int c = 0; c < 3; ++c) { ep[c] = ep[c] * qtmh2; bp[c] = bp[c] * qtmh1; }
  for (int c = 0; c < 3; ++c) utmp[c] = p[c] + ep[c];
  p[0] = utmp[0] + utmp[1] * bp[2] - utmp[2] * bp[1];
  p[1] = utmp[1] + utmp[2] * bp[0] - utmp[0] * bp[2];
  p[2] = utmp[2] + utmp[0] * bp[1] - utmp[1] * bp[0];
  double ostq = 2.0 / (1.0 + bp[0] * bp[0] + bp[1] * bp[1] + bp[2] * bp[2]);
  for (int c = 0; c < 3; ++c) bp[c] = bp[c] * ostq;
  {
    double t0 = utmp[0] + p[1] * bp[2] - p[2] * bp[1];
    double t1 = utmp[1] + p[2] * bp[0] - p[0] * bp[2];
    double t2 = utmp[2] + p[0] * bp[1] - p[1] * bp[0];
    utmp[0] = t0; utmp[1] = t1; utmp[2] = t2;
  }
  for (int c = 0; c < 3; ++c) p[c] = utmp[c] + ep[c];
  px[pp] = p[0]; py[pp] = p[1]; pz[pp] = p[2];
  gamma[pp] = sqrt(1.0 + p[0] * p[0] + p[1] * p[1] + p[2] * p[2]);
}

void orc_push_u(const orc_grid* g, int push_type, double qbm, double dt, int64_t np,
                const double* x, const double* y, double* px, double* py, double* pz,
                double* gamma, const double* psi, const double* ef, const double* bf, int nthreads) {
  const double qtmh = qbm * dt * 0.5, idr = 1.0 / g->dr;
  if (nthreads < 1) nthreads = 1;
#pragma omp parallel for schedule(static) num_threads(nthreads) if (nthreads > 1)
  for (int64_t pp = 0; pp < np; ++pp)
    push_u_one(g, push_type, qbm, qtmh, idr, pp, x, y, px, py, pz, gamma, psi, ef, bf);
}

/* =============================================================================
 * PGC (ponderomotive guiding centre) pushers, for species that see a laser envelope
 *   amjdeposit_robust_pgc part2d_class.f03:1310-1602, amjdeposit_std_pgc :1012-1308,
 *   push_u_robust_pgc / push_u_std_pgc :1967-2219 (the two push_u variants are the same).
 * The laser enters through a = a_r + i a_i and the gradients (r, phi, xi components) of
 * a_r and a_i, all gathered like any field; |a|^2 raises gamma, its gradient adds the
 * ponderomotive force to E.
 * ============================================================================= */
static void amj_one_pgc(const orc_grid* g, int push_type, double qbm, double qtmh, double idt,
                        double idr, int64_t pp, const double* x, const double* y, const double* px,
                        const double* py, const double* pz, const double* q, double* gamma, double* psi,
                        const double* ef, const double* bf, const orc_laser_f1* lf, double* cu,
                        double* amu, double* dcu) {
  const int M = g->max_mode;
  interp_info ii = gen_interp_info(x[pp], y[pp], idr);
  double ep[3], bp[3], wp[3], u0[3], u[3], utmp[3], du[2], u2[3], gr[3], gi[3];
  interp_vec(g, ef, &ii, ep);
  interp_vec(g, bf, &ii, bp);
  const double apr = interp_scalar(g, lf->ar, &ii), api = interp_scalar(g, lf->ai, &ii);
  interp_vec(g, lf->gr, &ii, gr);
  interp_vec(g, lf->gi, &ii, gi);
  const double gam_corr = 0.5 * (qbm * qbm) * (apr * apr + api * api);
  u0[0] = px[pp] * ii.pcos + py[pp] * ii.psin;
  u0[1] = py[pp] * ii.pcos - px[pp] * ii.psin;
  u0[2] = pz[pp];
  double gam = sqrt(1.0 + u0[0] * u0[0] + u0[1] * u0[1] + u0[2] * u0[2] + gam_corr);
  wp[0] = ep[0] - bp[1];
  wp[1] = ep[1] + bp[0];
  wp[2] = ep[2];
  const double tmp = 0.5 * qbm / gam;          /* effective E: the ponderomotive force */
  ep[0] = ep[0] - tmp * (apr * gr[0] + api * gi[0]);
  ep[1] = ep[1] - tmp * (apr * gr[1] + api * gi[1]);
  ep[2] = ep[2] + tmp * (apr * gr[2] + api * gi[2]);
  double qtmh_e, qtmh_b = 0.0;
  if (push_type == ORC_PUSH_ROBUST_PGC) {
    qtmh_e = qtmh * gam / (gam - u0[2]);
    for (int c = 0; c < 3; ++c) utmp[c] = u0[c] + ep[c] * qtmh_e;
    gam = sqrt(1.0 + utmp[0] * utmp[0] + utmp[1] * utmp[1] + utmp[2] * utmp[2] + gam_corr);
    qtmh_b = qtmh / (gam - utmp[2]);
    for (int c = 0; c < 3; ++c) bp[c] = bp[c] * qtmh_b;
  } else {
    qtmh_b = qtmh / (1.0 - qbm * psi[pp]);
    qtmh_e = qtmh_b * gam;
    for (int c = 0; c < 3; ++c) utmp[c] = u0[c] + ep[c] * qtmh_e;
    for (int c = 0; c < 3; ++c) bp[c] = bp[c] * qtmh_b;
  }
  u[0] = utmp[0] + utmp[1] * bp[2] - utmp[2] * bp[1];
  u[1] = utmp[1] + utmp[2] * bp[0] - utmp[0] * bp[2];
  u[2] = utmp[2] + utmp[0] * bp[1] - utmp[1] * bp[0];
  const double ostq = 2.0 / (1.0 + bp[0] * bp[0] + bp[1] * bp[1] + bp[2] * bp[2]);
  for (int c = 0; c < 3; ++c) bp[c] = bp[c] * ostq;
  {
    double t0 = utmp[0] + u[1] * bp[2] - u[2] * bp[1];
    double t1 = utmp[1] + u[2] * bp[0] - u[0] * bp[2];
    double t2 = utmp[2] + u[0] * bp[1] - u[1] * bp[0];
    utmp[0] = t0; utmp[1] = t1; utmp[2] = t2;
  }
  gam = sqrt(1.0 + utmp[0] * utmp[0] + utmp[1] * utmp[1] + utmp[2] * utmp[2] + gam_corr);
  qtmh_e = push_type == ORC_PUSH_ROBUST_PGC ? qtmh * gam / (gam - utmp[2]) : qtmh_b * gam;
  for (int c = 0; c < 3; ++c) u[c] = utmp[c] + ep[c] * qtmh_e;
  du[0] = idt * (u[0] - u0[0]);
  du[1] = idt * (u[1] - u0[1]);
  for (int c = 0; c < 3; ++c) u[c] = 0.5 * (u[c] + u0[c]);
  gamma[pp] = sqrt(1.0 + u[0] * u[0] + u[1] * u[1] + u[2] * u[2] + gam_corr);
  double ipsi;
  if (push_type == ORC_PUSH_ROBUST_PGC) {
    ipsi = 1.0 / (gamma[pp] - u[2]);
    psi[pp] = (1.0 - 1.0 / ipsi) / qbm;
  } else {
    ipsi = 1.0 / (1.0 - qbm * psi[pp]);
  }
  const double dpsi = qbm * (wp[2] - (wp[0] * u[0] + wp[1] * u[1]) * ipsi);
  du[0] = du[0] + u[0] * dpsi * ipsi;
  du[1] = du[1] + u[1] * dpsi * ipsi;
  u2[0] = u[0] * u[0] * ipsi;
  u2[1] = u[0] * u[1] * ipsi;
  u2[2] = u[1] * u[1] * ipsi;
  if (!II_OK(g, ii)) return;
  const double ph0r = ii.pcos, ph0i = -ii.psin;
  double phr = q[pp] * ipsi, phi = 0.0;
  const double wj[2] = {ii.w0, ii.w1};
  for (int j = 0; j < 2; ++j) {
    int n = ii.idx + j;
    double w = wj[j] * phr;
    for (int c = 0; c < 3; ++c) F(cu, 3, 0, c, n) = F(cu, 3, 0, c, n) + w * u[c];
    for (int c = 0; c < 2; ++c) F(dcu, 2, 0, c, n) = F(dcu, 2, 0, c, n) + w * du[c];
    for (int c = 0; c < 3; ++c) F(amu, 3, 0, c, n) = F(amu, 3, 0, c, n) + w * u2[c];
  }
  for (int m = 1; m <= M; ++m) {
    double t = phr * ph0r - phi * ph0i;
    phi = phr * ph0i + phi * ph0r;
    phr = t;
    const int r = PRE(m), s = PIM(m);
    for (int j = 0; j < 2; ++j) {
      int n = ii.idx + j;
      double w = wj[j] * phr;
      for (int c = 0; c < 3; ++c) F(cu, 3, r, c, n) = F(cu, 3, r, c, n) + w * u[c];
      for (int c = 0; c < 2; ++c) F(dcu, 2, r, c, n) = F(dcu, 2, r, c, n) + w * du[c];
      for (int c = 0; c < 3; ++c) F(amu, 3, r, c, n) = F(amu, 3, r, c, n) + w * u2[c];
      w = wj[j] * phi;
      for (int c = 0; c < 3; ++c) F(cu, 3, s, c, n) = F(cu, 3, s, c, n) + w * u[c];
      for (int c = 0; c < 2; ++c) F(dcu, 2, s, c, n) = F(dcu, 2, s, c, n) + w * du[c];
      for (int c = 0; c < 3; ++c) F(amu, 3, s, c, n) = F(amu, 3, s, c, n) + w * u2[c];
    }
  }
}

void orc_amjdeposit_pgc(const orc_grid* g, int push_type, double qbm, double dt, int64_t np,
                        const double* x, const double* y, const double* px, const double* py,
                        const double* pz, const double* q, double* gamma, double* psi, const double* ef,
                        const double* bf, const orc_laser_f1* lf, double* cu, double* amu, double* dcu) {
  const double idt = 1.0 / dt, qtmh = 0.5 * qbm * dt, idr = 1.0 / g->dr;
  for (int64_t pp = 0; pp < np; ++pp)
    amj_one_pgc(g, push_type, qbm, qtmh, idt, idr, pp, x, y, px, py, pz, q, gamma, psi, ef, bf, lf, cu, amu, dcu);
  amj_axis_scale(g, cu, amu, dcu);   /* the same finishing as the plain deposits */
}

void orc_push_u_pgc(const orc_grid* g, double qbm, double dt, int64_t np, const double* x, const double* y,
                    double* px, double* py, double* pz, double* gamma, const double* psi, const double* ef,
                    const double* bf, const orc_laser_f1* lf) {
  const double qtmh = qbm * dt * 0.5, qbm2_hf = (qbm * qbm) * 0.5, idr = 1.0 / g->dr;
  for (int64_t pp = 0; pp < np; ++pp) {
    interp_info ii = gen_interp_info(x[pp], y[pp], idr);
    double ep[3], bp[3], gr[3], gi[3], utmp[3], p[3];
    interp_vec(g, ef, &ii, ep);
    interp_vec(g, bf, &ii, bp);
    const double apr = interp_scalar(g, lf->ar, &ii), api = interp_scalar(g, lf->ai, &ii);
    interp_vec(g, lf->gr, &ii, gr);
    interp_vec(g, lf->gi, &ii, gi);
    double* vs[4] = {ep, bp, gr, gi};          /* transform_to_cartesian, interp_part2d.f03:155-171 */
    for (int k = 0; k < 4; ++k) {
      double t = vs[k][0] * ii.pcos - vs[k][1] * ii.psin;
      vs[k][1] = vs[k][0] * ii.psin + vs[k][1] * ii.pcos;
      vs[k][0] = t;
    }
    double gam_corr = qbm2_hf * (apr * apr + api * api);
    double tmp = 0.5 * qbm / gamma[pp];
    ep[0] = ep[0] - tmp * (apr * gr[0] + api * gi[0]);
    ep[1] = ep[1] - tmp * (apr * gr[1] + api * gi[1]);
    ep[2] = ep[2] + tmp * (apr * gr[2] + api * gi[2]);
    const double qtmh_b = qtmh / (1.0 - qbm * psi[pp]);
    const double qtmh_e = qtmh_b * gamma[pp];
    p[0] = px[pp]; p[1] = py[pp]; p[2] = pz[pp];
    for (int c = 0; c < 3; ++c) { ep[c] = ep[c] * qtmh_e; utmp[c] = p[c] + ep[c]; bp[c] = bp[c] * qtmh_b; }
    p[0] = utmp[0] + utmp[1] * bp[2] - utmp[2] * bp[1];
    p[1] = utmp[1] + utmp[2] * bp[0] - utmp[0] * bp[2];
    p[2] = utmp[2] + utmp[0] * bp[1] - utmp[1] * bp[0];
    const double ostq = 2.0 / (1.0 + bp[0] * bp[0] + bp[1] * bp[1] + bp[2] * bp[2]);
    for (int c = 0; c < 3; ++c) bp[c] = bp[c] * ostq;
    {
      double t0 = utmp[0] + p[1] * bp[2] - p[2] * bp[1];
      double t1 = utmp[1] + p[2] * bp[0] - p[0] * bp[2];
      double t2 = utmp[2] + p[0] * bp[1] - p[1] * bp[0];
      utmp[0] = t0; utmp[1] = t1; utmp[2] = t2;
    }
    for (int c = 0; c < 3; ++c) p[c] = utmp[c] + ep[c];
    /* time-centred gamma for the position push: |a|^2 advanced by half a step in xi */
    tmp = gr[2] * dt; gam_corr = gam_corr + qbm2_hf * (apr + 0.25 * tmp) * tmp;
    tmp = gi[2] * dt; gam_corr = gam_corr + qbm2_hf * (api + 0.25 * tmp) * tmp;
    px[pp] = p[0]; py[pp] = p[1]; pz[pp] = p[2];
    gamma[pp] = sqrt(1.0 + p[0] * p[0] + p[1] * p[1] + p[2] * p[2] + gam_corr);
  }
}

/* deposit_chi (part2d_class.f03:361-476): the plasma susceptibility -qbm q / (1 - qbm psi)
 * of each particle into the modes of chi, then the axis rule (m = 0 node 1 times
 * 12 ppc_r^2 / (1 + 2 ppc_r^2), get_deposit_ax_corr :2581-2586; m >= 1 node 1 zero) and
 * 1/(i-1) on nodes 2..nr+1.  The finishing scales the whole array, so a second species
 * finishes the first one's contribution again, as in the reference. */
void orc_deposit_chi(const orc_grid* g, double qbm, int ppc_r, int64_t np, const double* x, const double* y,
                     const double* q, const double* psi, double* chi) {
  const int M = g->max_mode, nr = g->nr;
  const double idr = 1.0 / g->dr;
  for (int64_t pp = 0; pp < np; ++pp) {
    double pos = sqrt(x[pp] * x[pp] + y[pp] * y[pp]) * idr;
    const double p0r = x[pp] / pos * idr, p0i = -y[pp] / pos * idr;
    if (!(pos >= 0.0 && pos < (double)nr)) continue;   /* beyond the outer edge: nothing */
    const int nn0 = (int)floor(pos);
    pos = pos - (double)nn0;
    const int nn = nn0 + 1;
    const double wt[2] = {1.0 - pos, pos};
    double phr = -(qbm * q[pp] / (1.0 - qbm * psi[pp])), phi = 0.0;
    for (int j = 0; j < 2; ++j) F(chi, 1, 0, 0, nn + j) = F(chi, 1, 0, 0, nn + j) + wt[j] * phr;
    for (int m = 1; m <= M; ++m) {
      const double t = phr * p0r - phi * p0i;
      phi = phr * p0i + phi * p0r;
      phr = t;
      for (int j = 0; j < 2; ++j) {
        F(chi, 1, PRE(m), 0, nn + j) = F(chi, 1, PRE(m), 0, nn + j) + wt[j] * phr;
        F(chi, 1, PIM(m), 0, nn + j) = F(chi, 1, PIM(m), 0, nn + j) + wt[j] * phi;
      }
    }
  }
  const double corr = (12.0 * (double)(ppc_r * ppc_r)) / (1.0 + 2.0 * (double)(ppc_r * ppc_r));
  for (int p = 0; p < nparts(g); ++p) {
    F(chi, 1, p, 0, 0) = 0.0;
    F(chi, 1, p, 0, 1) = p == 0 ? F(chi, 1, p, 0, 1) * corr : 0.0;
    for (int j = 2; j <= nr + 1; ++j) F(chi, 1, p, 0, j) = F(chi, 1, p, 0, j) * (1.0 / (double)(j - 1));
  }
}

void orc_push_x(int64_t np, double dt, double* x, double* y, const double* px, const double* py,
                const double* pz, const double* gamma) {                  /* :2221-2262 */
  for (int64_t pp = 0; pp < np; ++pp) {
    double dtc = dt / (gamma[pp] - pz[pp]);
    x[pp] = x[pp] + px[pp] * dtc;
    y[pp] = y[pp] + py[pp] * dtc;
  }
}

int64_t orc_update_bound(const orc_grid* g, int64_t np, double* x, double* y, double* px,
                         double* py, double* pz, double* gamma, double* psi, double* q) {  /* :2307-2353 */
  if (np == 0) return 0;
  const double edge = (double)g->nr * g->dr;
  int64_t i = 0, n = np;       /* 0-based: i < n-1 mirrors Fortran i < npp */
  while (i < n - 1) {
    double pos = sqrt(x[i] * x[i] + y[i] * y[i]);
    if (pos >= edge) {
      int64_t l = n - 1;
      x[i] = x[l]; y[i] = y[l]; px[i] = px[l]; py[i] = py[l]; pz[i] = pz[l];
      gamma[i] = gamma[l]; psi[i] = psi[l]; q[i] = q[l];
      n = n - 1;
      continue;
    }
    i = i + 1;
  }
  double pos = sqrt(x[n - 1] * x[n - 1] + y[n - 1] * y[n - 1]);
  if (pos >= edge) n = n - 1;
  return n;
}

void orc_interp_psi(const orc_grid* g, int64_t np, const double* x, const double* y,
                    const double* psif, double* psi) {                      /* :2264-2305 */
  const double idr = 1.0 / g->dr;
  for (int64_t pp = 0; pp < np; ++pp) {
    interp_info ii = gen_interp_info(x[pp], y[pp], idr);
    psi[pp] = interp_scalar(g, psif, &ii);
  }
}

/* counting sort: sort_module.f03:10-41, part2d_class.f03:2498-2579 */
void orc_sort(const orc_grid* g, int64_t np, double* x, double* y, double* px, double* py,
              double* pz, double* gamma, double* psi, double* q, int32_t* keys, int32_t* sort_idx) {
  const int nr = g->nr;
  const double idr = 1.0 / g->dr;
  for (int64_t i = 0; i < np; ++i) {
    double pos = sqrt(x[i] * x[i] + y[i] * y[i]) * idr;
    keys[i] = (int32_t)floor(pos) + 1;
  }
  int64_t* counter = (int64_t*)calloc((size_t)nr + 2, sizeof(int64_t));
  for (int64_t i = 0; i < np; ++i) counter[keys[i]] += 1;
  for (int k = 2; k <= nr; ++k) counter[k] += counter[k - 1];
  for (int64_t i = 0; i < np; ++i) {
    int k = keys[i];
    sort_idx[i] = (int32_t)counter[k];       /* 1-based destination */
    counter[k] -= 1;
  }
  free(counter);
  double* buf = (double*)malloc(sizeof(double) * (size_t)(np > 0 ? np : 1));
  double* arrs[8] = {x, y, px, py, pz, gamma, q, psi};
  for (int a = 0; a < 8; ++a) {
    memcpy(buf, arrs[a], sizeof(double) * (size_t)np);
    for (int64_t i = 0; i < np; ++i) arrs[a][sort_idx[i] - 1] = buf[i];
  }
  free(buf);
}

/* =============================================================================
 * Beam: part3d_class.f03
 * q2 and e2/b2 are f2 stores: slices 1..nz+1.
 * ============================================================================= */
#define F2(f, nc, s, p, c, i) \
  ((f)[((((size_t)(s) - 1) * (size_t)P + (size_t)(p)) * (nc) + (c)) * (size_t)NR2 + (size_t)(i)])

void orc_beam_qdeposit(const orc_grid* g, int64_t nb, const double* x, const double* y,
                       const double* z, const double* q, double* q2) {    /* :221-356 */
  const int M = g->max_mode, P = nparts(g), nr = g->nr, nz = g->nz;
  const double idr = 1.0 / g->dr, idz = 1.0 / g->dxi;
  for (int64_t pp = 0; pp < nb; ++pp) {
    double pr = sqrt(x[pp] * x[pp] + y[pp] * y[pp]) * idr;
    double pzs = z[pp] * idz;
    double ph0r = x[pp] / pr * idr, ph0i = -y[pp] / pr * idr;
    if (!(pr >= 0.0 && pr < 1.0e9 && pzs >= 0.0 && pzs < 1.0e9)) continue;
    int nn = (int)floor(pr), mm = (int)floor(pzs);
    pr = pr - (double)nn;
    pzs = pzs - (double)mm;
    nn = nn + 1;
    mm = mm + 1;
    if (mm < 1 || mm > nz || nn < 1 || nn > nr) continue;   /* outside the stored box */
    double wr[2] = {1.0 - pr, pr}, wz[2] = {1.0 - pzs, pzs};
    double phr = 1.0 * q[pp], phi = 0.0 * q[pp];
    for (int k = 0; k < 2; ++k)
      for (int j = 0; j < 2; ++j)
        F2(q2, 1, mm + k, 0, 0, nn + j) = F2(q2, 1, mm + k, 0, 0, nn + j) + wr[j] * wz[k] * phr;
    for (int m = 1; m <= M; ++m) {
      double t = phr * ph0r - phi * ph0i;
      phi = phr * ph0i + phi * ph0r;
      phr = t;
      for (int k = 0; k < 2; ++k)
        for (int j = 0; j < 2; ++j) {
          F2(q2, 1, mm + k, PRE(m), 0, nn + j) = F2(q2, 1, mm + k, PRE(m), 0, nn + j) + wr[j] * wz[k] * phr;
          F2(q2, 1, mm + k, PIM(m), 0, nn + j) = F2(q2, 1, mm + k, PIM(m), 0, nn + j) + wr[j] * wz[k] * phi;
        }
    }
  }
  for (int s = 1; s <= nz; ++s) {
    F2(q2, 1, s, 0, 0, 0) = 0.0;
    F2(q2, 1, s, 0, 0, 1) = 8.0 * F2(q2, 1, s, 0, 0, 1);
    for (int m = 1; m <= M; ++m) {
      F2(q2, 1, s, PRE(m), 0, 0) = 0.0; F2(q2, 1, s, PIM(m), 0, 0) = 0.0;
      F2(q2, 1, s, PRE(m), 0, 1) = 0.0; F2(q2, 1, s, PIM(m), 0, 1) = 0.0;
    }
    for (int j = 2; j <= nr + 1; ++j) {
      double ir = 1.0 / (double)(j - 1);
      for (int p = 0; p < P; ++p) F2(q2, 1, s, p, 0, j) = F2(q2, 1, s, p, 0, j) * ir;
    }
  }
}

/* interp_emf_part3d :691-790 */
static inline void beam_interp(const orc_grid* g, const double* e2, const double* b2, double x,
                               double y, double z, double ep[3], double bp[3]) {
  const int M = g->max_mode, P = nparts(g);
  const double idr = 1.0 / g->dr, idz = 1.0 / g->dxi;
  double pr = sqrt(x * x + y * y) * idr;
  double pzs = z * idz;
  double cc = x / pr * idr, ss = y / pr * idr;
  for (int c = 0; c < 3; ++c) { ep[c] = 0.0; bp[c] = 0.0; }
  if (!(pr >= 0.0 && pr < 1.0e9 && pzs > -1.0 && pzs < 1.0e9)) return;
  int nn = (int)pr, mm = (int)pzs;
  pr = pr - (double)nn;
  pzs = pzs - (double)mm;
  nn = nn + 1;
  mm = mm + 1;
  double wr[2] = {1.0 - pr, pr}, wz[2] = {1.0 - pzs, pzs};
  for (int c = 0; c < 3; ++c) { ep[c] = 0.0; bp[c] = 0.0; }
  if (nn < 1 || nn > g->nr || mm < 1 || mm > g->nz) return;  /* outside the stored box */
  for (int k = 0; k < 2; ++k)
    for (int j = 0; j < 2; ++j) {
      double wt = wr[j] * wz[k];
      for (int c = 0; c < 3; ++c) {
        ep[c] = ep[c] + F2(e2, 3, mm + k, 0, c, nn + j) * wt;
        bp[c] = bp[c] + F2(b2, 3, mm + k, 0, c, nn + j) * wt;
      }
    }
  double phr = 1.0, phi = 0.0;
  for (int m = 1; m <= M; ++m) {
    double t = phr * cc - phi * ss;
    phi = phr * ss + phi * cc;
    phr = t;
    double ph_r = 2.0 * phr, ph_i = 2.0 * phi;
    for (int k = 0; k < 2; ++k)
      for (int j = 0; j < 2; ++j) {
        double wt = wr[j] * wz[k];
        for (int c = 0; c < 3; ++c) {
          ep[c] = ep[c] + (F2(e2, 3, mm + k, PRE(m), c, nn + j) * ph_r - F2(e2, 3, mm + k, PIM(m), c, nn + j) * ph_i) * wt;
          bp[c] = bp[c] + (F2(b2, 3, mm + k, PRE(m), c, nn + j) * ph_r - F2(b2, 3, mm + k, PIM(m), c, nn + j) * ph_i) * wt;
        }
      }
  }
  double a = ep[0] * cc - ep[1] * ss, b = ep[0] * ss + ep[1] * cc;
  ep[0] = a; ep[1] = b;
  a = bp[0] * cc - bp[1] * ss; b = bp[0] * ss + bp[1] * cc;
  bp[0] = a; bp[1] = b;
}

void orc_beam_push(const orc_grid* g, int push_type, double qbm, double dt, int64_t nb,
                   double* x, double* y, double* z, double* px, double* py, double* pz,
                   const double* e2, const double* b2, int nthreads) {
  const double qtmh = qbm * dt * 0.5;
  if (nthreads < 1) nthreads = 1;
#pragma omp parallel for schedule(static) num_threads(nthreads) if (nthreads > 1)
  for (int64_t pp = 0; pp < nb; ++pp) {
    double ep[3], bp[3], p[3] = {px[pp], py[pp], pz[pp]};
    beam_interp(g, e2, b2, x[pp], y[pp], z[pp], ep, bp);
    if (push_type == ORC_PUSH3_REDUCED) {                     /* :477-576 */
      double wp[3];
      for (int c = 0; c < 3; ++c) { ep[c] = ep[c] * qtmh; bp[c] = bp[c] * qtmh; }
      wp[0] = ep[0] - bp[1];
      wp[1] = ep[1] + bp[0];
      wp[2] = ep[2];
      for (int c = 0; c < 3; ++c) p[c] = p[c] + wp[c];
      for (int c = 0; c < 3; ++c) p[c] = p[c] + wp[c];
    } else {                                                  /* :358-475 */
      double utmp[3];
      for (int c = 0; c < 3; ++c) { ep[c] = ep[c] * qtmh; utmp[c] = p[c] + ep[c]; }
      double u2 = utmp[0] * utmp[0] + utmp[1] * utmp[1] + utmp[2] * utmp[2];
      double gam = sqrt(1.0 + u2);
      double gq = qtmh / gam;
      for (int c = 0; c < 3; ++c) bp[c] = bp[c] * gq;
      p[0] = utmp[0] + utmp[1] * bp[2] - utmp[2] * bp[1];
      p[1] = utmp[1] + utmp[2] * bp[0] - utmp[0] * bp[2];
      p[2] = utmp[2] + utmp[0] * bp[1] - utmp[1] * bp[0];
      double ostq = 2.0 / (1.0 + bp[0] * bp[0] + bp[1] * bp[1] + bp[2] * bp[2]);
      for (int c = 0; c < 3; ++c) bp[c] = bp[c] * ostq;
      double t0 = utmp[0] + p[1] * bp[2] - p[2] * bp[1];
      double t1 = utmp[1] + p[2] * bp[0] - p[0] * bp[2];
      double t2 = utmp[2] + p[0] * bp[1] - p[1] * bp[0];
      p[0] = t0 + ep[0]; p[1] = t1 + ep[1]; p[2] = t2 + ep[2];
    }
    double dt_gam = dt / sqrt(1.0 + p[0] * p[0] + p[1] * p[1] + p[2] * p[2]);
    x[pp] = x[pp] + p[0] * dt_gam;
    y[pp] = y[pp] + p[1] * dt_gam;
    z[pp] = z[pp] - p[2] * dt_gam + dt;
    px[pp] = p[0]; py[pp] = p[1]; pz[pp] = p[2];
  }
}

int64_t orc_beam_update_bound(const orc_grid* g, int64_t nb, double* x, double* y, double* z,
                              double* px, double* py, double* pz, double* q) {  /* :640-689 */
  if (nb == 0) return 0;
  const double er = (double)g->nr * g->dr, ez = (double)g->nz * g->dxi;
  int64_t i = 0, n = nb;
  while (i < n - 1) {
    double pr = sqrt(x[i] * x[i] + y[i] * y[i]);
    if (pr >= er || z[i] >= ez) {
      int64_t l = n - 1;
      x[i] = x[l]; y[i] = y[l]; z[i] = z[l]; px[i] = px[l]; py[i] = py[l]; pz[i] = pz[l]; q[i] = q[l];
      n = n - 1;
      continue;
    }
    i = i + 1;
  }
  double pr = sqrt(x[n - 1] * x[n - 1] + y[n - 1] * y[n - 1]);
  if (pr >= er || z[n - 1] >= ez) n = n - 1;
  return n;
}

/* =============================================================================
 * Loaders.  The reference draws from gfortran's random_number through rand_norm
 * (math_module.f03:77-102), which cannot be reproduced without gfortran; the
 * project substitutes a SplitMix64 stream (Steele, Lea & Flood 2014) feeding the
 * same Box-Muller pairing.  Product and oracle implement the identical generator.
 * ============================================================================= */
void orc_rng_seed(orc_rng* r, uint64_t seed) { r->s = seed; r->have = 0; r->next = 0.0; }

static uint64_t splitmix64(uint64_t* s) {
  uint64_t z = (*s += 0x9E3779B97F4A7C15ULL);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}

double orc_rand_uniform(orc_rng* r) {
  return ((double)(splitmix64(&r->s) >> 11) + 0.5) * (1.0 / 9007199254740992.0);
}

double orc_rand_norm(orc_rng* r) {
  if (!r->have) {
    double u1 = orc_rand_uniform(r), u2 = orc_rand_uniform(r);
    double theta = 2.0 * ORC_PI * u1;
    double amp = sqrt(-2.0 * log(u2));
    r->next = amp * sin(theta);
    r->have = 1;
    return amp * cos(theta);
  }
  r->have = 0;
  double v = r->next;
  r->next = 0.0;
  return v;
}

int64_t orc_load_plasma(const orc_grid* g, orc_rng* r, int ppc1, int ppc2, int num_theta,
                        double qm, double density, const double uth[3], double* x, double* y,
                        double* px, double* py, double* pz, double* gamma, double* psi, double* q) {
  /* fdist2d_class.f03:289-357 with uniform transverse and longitudinal profiles */
  const int nr = g->nr;
  const double dr = g->dr, dtheta = 2.0 * ORC_PI / num_theta;
  const int ppc_tot = ppc1 * ppc2;
  const double coef = (qm >= 0.0 ? 1.0 : -1.0) / ((double)ppc_tot * (double)num_theta);
  const double den_lon = 1.0, den_perp = 1.0, den_min = 1.0e-10;
  int64_t ip = 0;
  for (int j = 1; j <= num_theta; ++j)
    for (int i = 1; i <= nr; ++i)
      for (int i1 = 1; i1 <= ppc1; ++i1) {
        double rn = (i1 - 0.5) / ppc1 + (double)(i - 1);
        for (int i2 = 1; i2 <= ppc2; ++i2) {
          double theta = ((i2 - 0.5) / ppc2 + j - 1.0) * dtheta;
          double xt = rn * dr * cos(theta), yt = rn * dr * sin(theta);
          if (den_lon * den_perp * density < den_min) continue;
          x[ip] = xt;
          y[ip] = yt;
          q[ip] = rn * den_perp * den_lon * density * coef;
          px[ip] = uth[0] * orc_rand_norm(r);
          py[ip] = uth[1] * orc_rand_norm(r);
          pz[ip] = uth[2] * orc_rand_norm(r);
          gamma[ip] = sqrt(1.0 + px[ip] * px[ip] + py[ip] * py[ip] + pz[ip] * pz[ip]);
          psi[ip] = (1.0 - gamma[ip] + pz[ip]) / qm;
          ++ip;
        }
      }
  return ip;
}

int64_t orc_load_beam(const orc_grid* g, orc_rng* r, const orc_beam_desc* d, double* x, double* y,
                      double* z, double* px, double* py, double* pz, double* q) {
  /* fdist3d_rnd_class.f03:360-514, Gaussian profiles, cartesian geometry */
  const double dr = g->dr, dz = g->dxi;
  const double er = (double)g->nr * dr, ez = (double)g->nz * dz;
  const double q_per_part = (d->qm >= 0.0 ? 1.0 : -1.0) * d->tot_charge /
                            (2.0 * ORC_PI * (double)d->tot_num * (dr * dr) * dz);
  /* an empty sampling range would make the rejection loop below endless */
  for (int k = 0; k < 3; ++k)
    if (!(d->range_lo[k] < d->range_hi[k]) || !(d->sigma[k] > 0.0)) return -1;
  int64_t n = 0;
  for (int64_t i = 0; i < d->tot_num; ++i) {
    double xt[3];
    for (;;) {
      xt[0] = orc_rand_norm(r) * d->sigma[0] + d->center[0];
      if (xt[0] < d->range_lo[0] || xt[0] >= d->range_hi[0]) continue;
      xt[1] = orc_rand_norm(r) * d->sigma[1] + d->center[1];
      if (xt[1] < d->range_lo[1] || xt[1] >= d->range_hi[1]) continue;
      xt[2] = orc_rand_norm(r) * d->sigma[2] + d->center[2];
      if (xt[2] < d->range_lo[2] || xt[2] >= d->range_hi[2]) continue;
      break;
    }
    double rt = sqrt(xt[0] * xt[0] + xt[1] * xt[1]);
    if (rt < 0.0 || rt >= er) continue;
    if (xt[2] < 0.0 || xt[2] >= ez) continue;
    x[n] = xt[0]; y[n] = xt[1]; z[n] = xt[2];
    q[n] = q_per_part;
    px[n] = d->uth[0] * orc_rand_norm(r);
    py[n] = d->uth[1] * orc_rand_norm(r);
    pz[n] = d->uth[2] * orc_rand_norm(r) + d->gamma;
    pz[n] = sqrt(pz[n] * pz[n] - px[n] * px[n] - py[n] * py[n] - 1);
    ++n;
  }
  if (d->quiet) {
    int64_t ip = n;
    for (int64_t i = 0; i < ip; ++i) {
      x[ip + i] = -x[i]; y[ip + i] = -y[i]; z[ip + i] = z[i];
      px[ip + i] = -px[i]; py[ip + i] = -py[i]; pz[ip + i] = pz[i];
      q[i] = 0.5 * q[i];
      q[ip + i] = q[i];
    }
    n *= 2;
  }
  return n;
}

/* =============================================================================
 * Whole-loop driver: simulation_class.f03:294-512 (one 3D step)
 * ============================================================================= */
struct orc_sim {
  orc_sim_desc d;
  int P;
  size_t n1, n2;  /* doubles per 1-component f1 / f2 */
  /* slice fields */
  double *psi, *e, *e_spe, *b, *b_spe, *b_beam, *cu, *amu, *acu, *dcu, *q_spe, *q_beam, *qsp, *qn;
  /* 3D stores */
  double *q_beam2, *e2, *b2, *psi2, *b_spe2, *e_spe2, *cu2, *q_spe2;
  double *q_beamk;  /* one beam's own charge store (beam3d%q), summed into q_beam2 */
  /* neutral gas (neutral_class.f03) */
  int64_t nnp, na;
  double *nx, *ny, *npx, *npy, *npz, *ngamma, *npsi, *nq;   /* its electrons */
  double *ax, *ay, *aq;                                      /* ions born in the last update */
  double *multi_ion, *ion_old;
  double *rho_ion, *rho_add, *qneut, *cun, *amun, *acun;
  /* plasma */
  int64_t np;
  double *x, *y, *px, *py, *pz, *gamma, *ppsi, *q;
  /* beams */
  int64_t nb[4];
  double *bx[4], *by[4], *bz[4], *bpx[4], *bpy[4], *bpz[4], *bq[4];
  double *s_re, *s_im;
  /* lasers */
  double *lr2[4], *li2[4], *lsr[4], *lsi[4];   /* envelope stores, explicit right-hand sides */
  double **lcoef[4];                           /* per mode: PCR tables */
  double *lgr, *lgi;                           /* one laser's gradients of a slice */
  double *la_r, *la_i, *la_gr, *la_gi;         /* all lasers' sum of a slice (laser_all) */
  double *chi, *chi2;
};

static double* zalloc(size_t n) { return (double*)calloc(n ? n : 1, sizeof(double)); }

orc_sim* orc_sim_create(const orc_sim_desc* d) {
  orc_sim* s = (orc_sim*)calloc(1, sizeof(orc_sim));
  s->d = *d;
  const orc_grid* g = &s->d.g;
  s->P = nparts(g);
  s->n1 = (size_t)s->P * NR2;
  s->n2 = s->n1 * (size_t)(g->nz + 1);
  s->psi = zalloc(s->n1); s->e = zalloc(3 * s->n1); s->e_spe = zalloc(3 * s->n1);
  s->b = zalloc(3 * s->n1); s->b_spe = zalloc(3 * s->n1); s->b_beam = zalloc(3 * s->n1);
  s->cu = zalloc(3 * s->n1); s->amu = zalloc(3 * s->n1); s->acu = zalloc(2 * s->n1);
  s->dcu = zalloc(2 * s->n1); s->q_spe = zalloc(s->n1); s->q_beam = zalloc(s->n1);
  s->qsp = zalloc(s->n1); s->qn = zalloc(s->n1);
  s->q_beam2 = zalloc(s->n2); s->e2 = zalloc(3 * s->n2); s->b2 = zalloc(3 * s->n2);
  s->psi2 = zalloc(s->n2); s->b_spe2 = zalloc(3 * s->n2); s->e_spe2 = zalloc(3 * s->n2);
  s->cu2 = zalloc(3 * s->n2); s->q_spe2 = zalloc(s->n2);
  s->q_beamk = d->nbeams > 1 ? zalloc(s->n2) : NULL;
  if (d->neut_levels > 0) {
    const int64_t nm = d->neut_npmax;
    s->nx = zalloc(nm); s->ny = zalloc(nm); s->npx = zalloc(nm); s->npy = zalloc(nm); s->npz = zalloc(nm);
    s->ngamma = zalloc(nm); s->npsi = zalloc(nm); s->nq = zalloc(nm);
    s->ax = zalloc(nm); s->ay = zalloc(nm); s->aq = zalloc(nm);
    s->multi_ion = zalloc((size_t)d->neut_num_theta * g->nr * (d->neut_levels + 2));
    s->ion_old = zalloc((size_t)d->neut_num_theta * g->nr);
    s->rho_ion = zalloc(s->n1); s->rho_add = zalloc(s->n1); s->qneut = zalloc(s->n1);
    s->cun = zalloc(3 * s->n1); s->amun = zalloc(3 * s->n1); s->acun = zalloc(2 * s->n1);
  }
  int64_t npm = d->sp_npmax;
  s->x = zalloc(npm); s->y = zalloc(npm); s->px = zalloc(npm); s->py = zalloc(npm);
  s->pz = zalloc(npm); s->gamma = zalloc(npm); s->ppsi = zalloc(npm); s->q = zalloc(npm);
  for (int k = 0; k < d->nbeams; ++k) {
    int64_t n = d->beam_npmax[k];
    s->bx[k] = zalloc(n); s->by[k] = zalloc(n); s->bz[k] = zalloc(n);
    s->bpx[k] = zalloc(n); s->bpy[k] = zalloc(n); s->bpz[k] = zalloc(n); s->bq[k] = zalloc(n);
  }
  s->s_re = zalloc((size_t)g->nr);
  s->s_im = zalloc((size_t)g->nr);
  if (d->nlasers > 0) {
    const size_t nls = (size_t)(g->nz + 3) * s->n1;
    const int n = 2 * g->nr;
    int steps = 0;
    while ((1 << steps) < n) ++steps;
    double* A = zalloc(5 * (size_t)n);
    for (int k = 0; k < d->nlasers; ++k) {
      s->lr2[k] = zalloc(nls); s->li2[k] = zalloc(nls);
      s->lsr[k] = zalloc(s->n2); s->lsi[k] = zalloc(s->n2);
      s->lcoef[k] = (double**)calloc((size_t)g->max_mode + 1, sizeof(double*));
      for (int m = 0; m <= g->max_mode; ++m) {
        double* c = zalloc((4 * (size_t)steps + 1) * n);
        orc_laser_matrix(g->nr, m, d->laser_k0[k], d->dt3d, g->dr, g->dxi, A, A + n, A + 2 * n, A + 3 * n, A + 4 * n);
        orc_pcr_coef(n, A, A + n, A + 2 * n, A + 3 * n, A + 4 * n, c, c + (size_t)steps * n, c + 2 * (size_t)steps * n,
                     c + 3 * (size_t)steps * n, c + 4 * (size_t)steps * n);
        s->lcoef[k][m] = c;
      }
    }
    free(A);
    s->lgr = zalloc(3 * s->n1); s->lgi = zalloc(3 * s->n1);
    s->la_r = zalloc(s->n1); s->la_i = zalloc(s->n1); s->la_gr = zalloc(3 * s->n1); s->la_gi = zalloc(3 * s->n1);
    s->chi = zalloc(s->n1); s->chi2 = zalloc(s->n2);
  }
  return s;
}

void orc_sim_destroy(orc_sim* s) {
  if (!s) return;
  double* all[] = {s->psi, s->e, s->e_spe, s->b, s->b_spe, s->b_beam, s->cu, s->amu, s->acu, s->dcu,
                   s->q_spe, s->q_beam, s->qsp, s->qn, s->q_beam2, s->e2, s->b2, s->psi2, s->b_spe2,
                   s->e_spe2, s->cu2, s->q_spe2, s->x, s->y, s->px, s->py, s->pz, s->gamma, s->ppsi,
                   s->q, s->s_re, s->s_im, s->q_beamk, s->nx, s->ny, s->npx, s->npy, s->npz, s->ngamma, s->npsi,
                   s->nq, s->ax, s->ay, s->aq, s->multi_ion, s->ion_old, s->rho_ion, s->rho_add, s->qneut,
                   s->cun, s->amun, s->acun};
  for (size_t i = 0; i < sizeof(all) / sizeof(all[0]); ++i) free(all[i]);
  for (int k = 0; k < s->d.nlasers; ++k) {
    free(s->lr2[k]); free(s->li2[k]); free(s->lsr[k]); free(s->lsi[k]);
    for (int m = 0; m <= s->d.g.max_mode; ++m) free(s->lcoef[k][m]);
    free(s->lcoef[k]);
  }
  free(s->lgr); free(s->lgi); free(s->la_r); free(s->la_i); free(s->la_gr); free(s->la_gi);
  free(s->chi); free(s->chi2);
  for (int k = 0; k < s->d.nbeams; ++k) {
    free(s->bx[k]); free(s->by[k]); free(s->bz[k]); free(s->bpx[k]); free(s->bpy[k]);
    free(s->bpz[k]); free(s->bq[k]);
  }
  free(s);
}

void orc_sim_set_plasma(orc_sim* s, int64_t np, const double* x, const double* y,
                        const double* px, const double* py, const double* pz,
                        const double* gamma, const double* psi, const double* q) {
  const orc_grid* g = &s->d.g;
  s->np = np;
  size_t b = sizeof(double) * (size_t)np;
  memcpy(s->x, x, b); memcpy(s->y, y, b); memcpy(s->px, px, b); memcpy(s->py, py, b);
  memcpy(s->pz, pz, b); memcpy(s->gamma, gamma, b); memcpy(s->ppsi, psi, b); memcpy(s->q, q, b);
  /* species2d_class.f03:114-129 / 171-180: qn = -(deposit of the fresh particles) */
  memset(s->qsp, 0, sizeof(double) * s->n1);
  orc_qdeposit(g, s->np, s->x, s->y, s->q, s->qsp);
  for (size_t i = 0; i < s->n1; ++i) s->qn[i] = s->qsp[i] * -1.0;
}

void orc_sim_set_beam(orc_sim* s, int k, int64_t nb, const double* x, const double* y,
                      const double* z, const double* px, const double* py, const double* pz,
                      const double* q) {
  s->nb[k] = nb;
  size_t b = sizeof(double) * (size_t)nb;
  memcpy(s->bx[k], x, b); memcpy(s->by[k], y, b); memcpy(s->bz[k], z, b);
  memcpy(s->bpx[k], px, b); memcpy(s->bpy[k], py, b); memcpy(s->bpz[k], pz, b);
  memcpy(s->bq[k], q, b);
}

static void copy_1to2(orc_sim* s, const double* f1, double* f2, int nc, int j) {
  size_t n = s->n1 * (size_t)nc;
  memcpy(f2 + (size_t)(j - 1) * n, f1, sizeof(double) * n);
}

void orc_sim_begin_3dstep(orc_sim* s) {
  const orc_grid* g = &s->d.g;
  const size_t n1 = s->n1;
  /* simulation_class.f03:309-317 */
  memset(s->q_beam2, 0, sizeof(double) * s->n2);
  memset(s->q_spe2, 0, sizeof(double) * s->n2);
  /* beam3d::qdp (beam3d_class.f03:193-221): each beam deposits into its own zeroed store,
     which part3d::qdeposit finishes (axis rule, 1/(i-1)), then add_f2 into q_beam */
  if (s->d.nbeams == 1) {
    orc_beam_qdeposit(g, s->nb[0], s->bx[0], s->by[0], s->bz[0], s->bq[0], s->q_beam2);
  } else {
    for (int k = 0; k < s->d.nbeams; ++k) {
      memset(s->q_beamk, 0, sizeof(double) * s->n2);
      orc_beam_qdeposit(g, s->nb[k], s->bx[k], s->by[k], s->bz[k], s->bq[k], s->q_beamk);
      for (size_t i = 0; i < s->n2; ++i) s->q_beam2[i] = s->q_beam2[i] + s->q_beamk[i];
    }
  }
  /* renew_neutral (neutral_class.f03:839-878): no electrons, no ions, all gas neutral */
  if (s->d.neut_levels > 0) {
    const int L = s->d.neut_levels, ncell = s->d.neut_num_theta * g->nr;
    s->nnp = 0;
    s->na = 0;
    for (int c = 0; c < ncell; ++c) {
      for (int l = 0; l < L + 2; ++l) s->multi_ion[(size_t)c * (L + 2) + l] = l == L ? 1.0 : 0.0;
      s->ion_old[c] = 0.0;
    }
    memset(s->rho_ion, 0, n1 * sizeof(double));
  }
  /* :332-341 */
  memset(s->b, 0, 3 * n1 * sizeof(double)); memset(s->e, 0, 3 * n1 * sizeof(double));
  memset(s->b_spe, 0, 3 * n1 * sizeof(double)); memset(s->e_spe, 0, 3 * n1 * sizeof(double));
  memset(s->psi, 0, n1 * sizeof(double)); memset(s->cu, 0, 3 * n1 * sizeof(double));
  memset(s->acu, 0, 2 * n1 * sizeof(double)); memset(s->amu, 0, 3 * n1 * sizeof(double));
}

/* ---- neutral gas: neutral_class.f03 ---------------------------------------------------
 * multi_ion[(k * nr + j) * (L + 2) + l]: angle k, cell j (0-based, cell j + 1 of the
 * reference), level l = 0..L-1 the ionisation levels 1..L, l = L the neutral fraction,
 * l = L + 1 the mean ionisation quantised to the particles per cell. */
static double* MI(orc_sim* s, int k, int j) {
  return s->multi_ion + ((size_t)k * s->d.g.nr + j) * (s->d.neut_levels + 2);
}

/* ionize_neutral (neutral_class.f03:600-753): ADK rates from |E| at the cell centres at the
 * angles 2 pi k / n_theta and the level cascade over one slice step.  The mode sum takes the
 * Re part of mode m for both its Re and its Im term, as the reference does (e_im => rf_re(m)). */
static void neutral_ionize(orc_sim* s) {
  const orc_grid* g = &s->d.g;
  const int L = s->d.neut_levels, nth = s->d.neut_num_theta, nr = g->nr, M = g->max_mode;
  const int ppc_tot = s->d.neut_ppc1 * s->d.neut_ppc2;
  const double wp = s->d.neut_wp, dt = g->dxi, pi = 3.14159265358979323846;
  const double* e = s->e;
  double w[16];
  for (int k = 0; k < nth; ++k) {
    const double theta = 2.0 * pi / (double)nth * (double)k;
    const double inc_r = cos(theta), inc_i = sin(theta);
    double ph_r = 1.0, ph_i = 0.0;
    double* e1 = (double*)malloc(sizeof(double) * 3 * (size_t)nr);
    for (int j = 1; j <= nr; ++j)
      for (int c = 0; c < 3; ++c) e1[3 * (j - 1) + c] = 0.5 * (F(e, 3, 0, c, j) + F(e, 3, 0, c, j + 1));
    for (int m = 1; m <= M; ++m) {
      const double t = ph_r * inc_r - ph_i * inc_i;
      ph_i = ph_r * inc_i + ph_i * inc_r;
      ph_r = t;
      for (int j = 1; j <= nr; ++j)
        for (int c = 0; c < 3; ++c) {
          const double er = F(e, 3, PRE(m), c, j) + F(e, 3, PRE(m), c, j + 1);
          const double ei = F(e, 3, PRE(m), c, j) + F(e, 3, PRE(m), c, j + 1);
          e1[3 * (j - 1) + c] = e1[3 * (j - 1) + c] + er * ph_r - ei * ph_i;
        }
    }
    for (int j = 0; j < nr; ++j) {
      double* mi = MI(s, k, j);
      const double* v = e1 + 3 * j;
      const double eij = sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]) * wp * 1.708e-12;
      if (!(eij > 1.0e-6) || !(mi[L + 1] < (double)L)) continue;
      for (int i = 0; i < L; ++i)
        w[i] = s->d.neut_adk[3 * i] * pow(eij, -s->d.neut_adk[3 * i + 2]) * exp(-s->d.neut_adk[3 * i + 1] / eij) / wp;
      int shoot = 0;
      double cons = mi[L] * w[0] * dt * (1.0 + 0.5 * w[0] * dt);
      if (cons > mi[L]) { shoot = 1; cons = mi[L]; }
      mi[L] = mi[L] - cons;
      for (int i = 1; i <= L - 1; ++i) {          /* levels i = 1 .. L-1 of the reference */
        const double inj = cons;
        double dens = 0.0;
        if (shoot) { dens = inj * 0.5; shoot = 0; }
        cons = (mi[i - 1] + dens) * w[i] * dt * (1.0 + 0.5 * w[i] * dt);
        if (cons > mi[i - 1] + dens) { shoot = 1; cons = mi[i - 1] + dens; }
        const double nv = mi[i - 1] - cons + inj;
        mi[i - 1] = nv < 1.0 ? nv : 1.0;
      }
      const double top = mi[L - 1] + cons;
      mi[L - 1] = top < 1.0 ? top : 1.0;
      double avg = 0.0;
      for (int i = 1; i <= L; ++i) avg = avg + (double)i * mi[i - 1];
      mi[L + 1] = (double)L / (double)ppc_tot * (double)(int)(avg * (double)ppc_tot / (double)L + 0.5);
    }
    free(e1);
  }
}

/* add_particles (neutral_class.f03:755-837): each (angle, cell) whose quantised ionisation
 * rose gives that many new electrons, evenly spaced in r across the cell at the angle, at
 * rest; their ions (opposite charge, same places) go to the ion buffer.  Uniform gas. */
static void neutral_inject(orc_sim* s) {
  const orc_grid* g = &s->d.g;
  const int L = s->d.neut_levels, nth = s->d.neut_num_theta, nr = g->nr;
  const int ppc_tot = s->d.neut_ppc1 * s->d.neut_ppc2;
  const double pi = 3.14159265358979323846, dth = 2.0 * pi / (double)nth;
  const double coef = (double)L * (s->d.neut_qm < 0.0 ? -1.0 : 1.0) / ((double)ppc_tot * (double)nth);
  s->na = 0;
  for (int k = 0; k < nth; ++k)
    for (int j = 0; j < nr; ++j) {
      const double* mi = MI(s, k, j);
      const int add = (int)((mi[L + 1] - s->ion_old[(size_t)k * nr + j]) / (double)L * (double)ppc_tot + 0.5);
      for (int i = 1; i <= add; ++i) {
        if (s->nnp >= s->d.neut_npmax) break;      /* capacity (the reference assumes enough room) */
        const double rn = (double)j + ((double)i - 0.5) / (double)add;   /* (j + 1) + noff - 1 */
        const double th = (double)k * dth;
        const int64_t p = s->nnp++, a = s->na++;
        s->nx[p] = rn * g->dr * cos(th);
        s->ny[p] = rn * g->dr * sin(th);
        s->nq[p] = rn * 1.0 * 1.0 * s->d.neut_density * coef;
        s->npx[p] = 0.0; s->npy[p] = 0.0; s->npz[p] = 0.0;
        s->ngamma[p] = 1.0; s->npsi[p] = 0.0;
        s->ax[a] = s->nx[p]; s->ay[a] = s->ny[p]; s->aq[a] = -s->nq[p];
      }
    }
}

/* update_neutral (neutral_class.f03:576-598) */
static void neutral_update(orc_sim* s) {
  const int L = s->d.neut_levels, ncell = s->d.neut_num_theta * s->d.g.nr;
  for (int c = 0; c < ncell; ++c) s->ion_old[c] = s->multi_ion[(size_t)c * (L + 2) + L + 1];
  neutral_ionize(s);
  neutral_inject(s);
}

/* =============================================================================
 * Laser envelope: field_laser_class.f03 (init_solver :269-391, set_rhs :393-635,
 * set_grad :637-750, solve :752-927, gather :929-946) and the parallel cyclic
 * reduction of its penta-diagonal systems (fpcr_penta_class.f03).
 *
 * Per laser the envelope a = a_r + i a_i is stored per xi slice like a 1-component field
 * (parts: m = 0, Re m, Im m), slices -1..nz+1 (the two slices ahead of the box stay zero):
 *   LS(f, j, p, i) = f[((j + 1) * P + p) * (nr + 2) + i].
 * In the reference's names, cfr_re(m) / cfr_im(m) are parts Re m / Im m of a_r and
 * cfi_re(m) / cfi_im(m) those of a_i.
 * ============================================================================= */
#define LS(f, j, p, i) ((f)[(((size_t)(j) + 1) * (size_t)P + (size_t)(p)) * (size_t)NR2 + (size_t)(i)])
#define SL(f, j, p, i) ((f)[(((size_t)(j) - 1) * (size_t)P + (size_t)(p)) * (size_t)NR2 + (size_t)(i)])

static inline int part_of(int m, int im) { return m == 0 ? 0 : (im ? PIM(m) : PRE(m)); }

/* generate_cr_coef (fpcr_penta_class.f03:288-527) on one rank: rows 1..n (index i-1) of a
 * penta-diagonal matrix, (a, b, c, d, e) multiplying x(i-2) .. x(i+2); steps = log2(n)
 * reductions with strides 1, 2, 4, ...; rows outside 1..n read as (0, 1, 2, 1, 0).  Writes
 * the coefficients cm1, cm2, cp1, cp2 [step][n] and the final diagonal cfin[n]. */
void orc_pcr_coef(int n, const double* a_in, const double* b_in, const double* c_in, const double* d_in,
                  const double* e_in, double* cm1, double* cm2, double* cp1, double* cp2, double* cfin) {
  int steps = 0;
  while ((1 << steps) < n) ++steps;
  double* A = (double*)malloc(sizeof(double) * 10 * (size_t)n);
  double *a = A, *b = A + n, *c = A + 2 * n, *d = A + 3 * n, *e = A + 4 * n;
  double *na = A + 5 * n, *nb = A + 6 * n, *nc = A + 7 * n, *nd = A + 8 * n, *ne = A + 9 * n;
  memcpy(a, a_in, sizeof(double) * n); memcpy(b, b_in, sizeof(double) * n); memcpy(c, c_in, sizeof(double) * n);
  memcpy(d, d_in, sizeof(double) * n); memcpy(e, e_in, sizeof(double) * n);
#define ROW(arr, k, pad) ((k) >= 1 && (k) <= n ? (arr)[(k) - 1] : (pad))
  for (int s = 1; s <= steps; ++s) {
    const int cs = 1 << (s - 1);
    double* m1 = cm1 + (size_t)(s - 1) * n;
    double* m2 = cm2 + (size_t)(s - 1) * n;
    double* p1 = cp1 + (size_t)(s - 1) * n;
    double* p2 = cp2 + (size_t)(s - 1) * n;
    for (int i = 1; i <= n; ++i) {
      const int im1 = i - cs, ip1 = i + cs, im2 = i - 2 * cs, ip2 = i + 2 * cs;
      const double am1 = ROW(a, im1, 0.0), bm1 = ROW(b, im1, 1.0), cm1v = ROW(c, im1, 2.0), dm1 = ROW(d, im1, 1.0),
                   em1 = ROW(e, im1, 0.0);
      const double am2 = ROW(a, im2, 0.0), bm2 = ROW(b, im2, 1.0), cm2v = ROW(c, im2, 2.0), dm2 = ROW(d, im2, 1.0),
                   em2 = ROW(e, im2, 0.0);
      const double ap1 = ROW(a, ip1, 0.0), bp1 = ROW(b, ip1, 1.0), cp1v = ROW(c, ip1, 2.0), dp1 = ROW(d, ip1, 1.0),
                   ep1 = ROW(e, ip1, 0.0);
      const double ap2 = ROW(a, ip2, 0.0), bp2 = ROW(b, ip2, 1.0), cp2v = ROW(c, ip2, 2.0), dp2 = ROW(d, ip2, 1.0),
                   ep2 = ROW(e, ip2, 0.0);
      const double a0 = a[i - 1], b0 = b[i - 1], c0 = c[i - 1], d0 = d[i - 1], e0 = e[i - 1];
      double tmp = am1 * cp1v * dm2 * dp2 - am1 * bp2 * dm2 * ep1 + ap1 * bm2 * dp2 * em1 + bm2 * bp2 * cm1v * ep1 -
                   bm2 * cm1v * cp1v * dp2;
      double km2 = 0.0, km1 = 0.0, kp1 = 0.0, kp2 = 0.0;
      if (fabs(tmp) > 1e-40) {
        tmp = 1.0 / tmp;
        km2 = am1 * (ap1 * d0 * dp2 + b0 * bp2 * ep1 - b0 * cp1v * dp2) * tmp;
        km1 = -(bm2 * (ap1 * d0 * dp2 + b0 * bp2 * ep1 - b0 * cp1v * dp2) * tmp);
        kp1 = -(dp2 * (am1 * d0 * dm2 + b0 * bm2 * em1 - d0 * bm2 * cm1v) * tmp);
        kp2 = ep1 * (am1 * d0 * dm2 + b0 * bm2 * em1 - d0 * bm2 * cm1v) * tmp;
      }
      m2[i - 1] = km2; m1[i - 1] = km1; p1[i - 1] = kp1; p2[i - 1] = kp2;
      na[i - 1] = km2 * am2;
      nb[i - 1] = km2 * cm2v + km1 * bm1 + a0;
      nc[i - 1] = km2 * em2 + km1 * dm1 + c0 + kp1 * bp1 + kp2 * ap2;
      nd[i - 1] = e0 + kp1 * dp1 + kp2 * cp2v;
      ne[i - 1] = kp2 * ep2;
    }
    memcpy(a, na, sizeof(double) * n); memcpy(b, nb, sizeof(double) * n); memcpy(c, nc, sizeof(double) * n);
    memcpy(d, nd, sizeof(double) * n); memcpy(e, ne, sizeof(double) * n);
  }
#undef ROW
  memcpy(cfin, c, sizeof(double) * n);
  free(A);
}

/* solve_fpcr_penta (:129-286) on one rank: rhs in, solution out (rows outside 1..n are 0) */
void orc_pcr_solve(int n, const double* cm1, const double* cm2, const double* cp1, const double* cp2,
                   const double* cfin, double* rhs) {
  int steps = 0;
  while ((1 << steps) < n) ++steps;
  double* x = (double*)malloc(sizeof(double) * (size_t)n);
  for (int s = 1; s <= steps; ++s) {
    const int cs = 1 << (s - 1);
    const size_t o = (size_t)(s - 1) * n;
    for (int i = 1; i <= n; ++i) {
      const int im1 = i - cs, ip1 = i + cs, im2 = i - 2 * cs, ip2 = i + 2 * cs;
      double v = rhs[i - 1];
      v = v + cm1[o + i - 1] * (im1 >= 1 ? rhs[im1 - 1] : 0.0);
      v = v + cm2[o + i - 1] * (im2 >= 1 ? rhs[im2 - 1] : 0.0);
      v = v + cp1[o + i - 1] * (ip1 <= n ? rhs[ip1 - 1] : 0.0);
      v = v + cp2[o + i - 1] * (ip2 <= n ? rhs[ip2 - 1] : 0.0);
      x[i - 1] = v;
    }
    memcpy(rhs, x, sizeof(double) * n);
  }
  for (int i = 0; i < n; ++i) rhs[i] = rhs[i] / cfin[i];
  free(x);
}

/* init_solver (field_laser_class.f03:269-391) on one rank: the 2 nr rows of mode m, rows
 * 2i-1 / 2i for a_r / a_i at node i, with set_values_matrix_byrow's boundary entries
 * (fpcr_penta_class.f03:570-595: a, b of row 1 and a of row 2, d, e of row n and e of row
 * n-1 set to the machine epsilon). */
void orc_laser_matrix(int nr, int m, double k0, double ds, double dr, double dz, double* a, double* b, double* c,
                      double* d, double* e) {
  const int n = 2 * nr;
  const double eps = 2.220446049250313e-16;     /* epsilon(1.0) of the 8-byte default real */
  const double ds_qtr = 0.25 * ds, dr2_idz_1hf = 1.5 * (dr * dr) / dz, kap = k0 * (dr * dr);
  const double m2 = (double)(m * m);
#define SETROW(r, A_, B_, C_, D_, E_)                       \
  do {                                                      \
    a[(r) - 1] = (A_); b[(r) - 1] = (B_); c[(r) - 1] = (C_); \
    d[(r) - 1] = (D_); e[(r) - 1] = (E_);                  \
    if ((r) == 1) { a[0] = eps; b[0] = eps; }               \
    else if ((r) == 2) a[1] = eps;                          \
    if ((r) == n) { e[n - 1] = eps; d[n - 1] = eps; }       \
    else if ((r) == n - 1) e[n - 2] = eps;                  \
  } while (0)
  for (int i = 3; i <= n - 1; i += 2) {          /* node j + 1 = (i + 1) / 2; row pair 1-2 is the axis */
    const int j = (i + 1) / 2 - 1;
    const double j2 = (double)(j * j);
    const double av = -(ds_qtr * (1.0 - 0.5 / (double)j));
    const double cv = ds_qtr * (2.0 + m2 / j2) + dr2_idz_1hf;
    const double ev = -(ds_qtr * (1.0 + 0.5 / (double)j));
    SETROW(i, av, 0.0, cv, -kap, ev);
    SETROW(i + 1, av, kap, cv, 0.0, ev);
  }
  if (m == 0) {
    SETROW(1, 0.0, eps, ds + dr2_idz_1hf, -kap, -ds);
    SETROW(2, eps, kap, ds + dr2_idz_1hf, 0.0, -ds);
  } else {
    SETROW(1, eps, eps, 1.0, eps, eps);
    SETROW(2, eps, eps, 1.0, eps, eps);
  }
  {
    const int j = nr - 1;
    const double j2 = (double)(j * j);
    const double av = -(ds_qtr * (1.0 - 0.5 / (double)j));
    const double cv = ds_qtr * (2.0 + m2 / j2) + dr2_idz_1hf;
    SETROW(n - 1, av, 0.0, cv, -kap, 0.0);
    SETROW(n, av, kap, cv, 0.0, 0.0);
  }
#undef SETROW
}

/* the plasma-susceptibility coupling of mode m at node i and slice j (set_rhs :558-631,
 * solve :795-862): t[0..3] += the terms of a_r Re, a_i Re, a_r Im, a_i Im */
static void laser_chi_terms(const orc_grid* g, const double* chi2, const double* lr, const double* li, int j, int m,
                            int i, double cq, double t[4]) {
  const int M = g->max_mode, P = nparts(g);
  for (int k = m - M; k <= M; ++k) {
    const int ak = abs(k), amk = abs(m - k);
    const double sg = (k >= 0 && k <= m) ? 1.0 : -1.0;
    const double cr = SL(chi2, j, part_of(ak, 0), i);
    t[0] = t[0] + cq * cr * LS(lr, j, part_of(amk, 0), i);
    t[1] = t[1] + cq * cr * LS(li, j, part_of(amk, 0), i);
    if (k == 0 || k == m) continue;
    const double ci = SL(chi2, j, PIM(ak), i);
    t[0] = t[0] - cq * sg * ci * LS(lr, j, PIM(amk), i);
    t[1] = t[1] - cq * sg * ci * LS(li, j, PIM(amk), i);
  }
  if (m == 0) return;
  for (int k = m - M; k <= M; ++k) {
    const int ak = abs(k), amk = abs(m - k);
    if (k != 0) {
      const double sg = k < 0 ? -1.0 : 1.0;
      const double ci = SL(chi2, j, PIM(ak), i);
      t[2] = t[2] + cq * sg * ci * LS(lr, j, part_of(amk, 0), i);
      t[3] = t[3] + cq * sg * ci * LS(li, j, part_of(amk, 0), i);
    }
    if (k != m) {
      const double sg = k > m ? -1.0 : 1.0;
      const double cr = SL(chi2, j, part_of(ak, 0), i);
      t[2] = t[2] + cq * sg * cr * LS(lr, j, PIM(amk), i);
      t[3] = t[3] + cq * sg * cr * LS(li, j, PIM(amk), i);
    }
  }
}

/* set_rhs (:393-635): for every slice the explicit half of the envelope equation from the
 * envelope before the step, plus the susceptibility coupling.  sr / si like chi2 (slices 1..nz). */
void orc_laser_rhs(const orc_grid* g, double k0, double ds, const double* chi2, const double* lr, const double* li,
                   double* sr, double* si) {
  const int M = g->max_mode, P = nparts(g), nr = g->nr;
  const double dr = g->dr, dz = g->dxi;
  const double dr2_idzh = 0.5 * (dr * dr) / dz, kap = k0 * (dr * dr), ds_qtr = 0.25 * ds,
               cq = ds_qtr * (dr * dr);
  for (int j = 1; j <= g->nz; ++j)
    for (int m = 0; m <= M; ++m) {
      const double m2 = (double)(m * m);
      for (int h = 0; h < (m == 0 ? 1 : 2); ++h) {
        const int p = part_of(m, h);
        for (int i = 1; i <= nr; ++i) {
          double bm, bp, al;
          if (i == 1) {
            if (m > 0) { SL(sr, j, p, i) = 0.0; SL(si, j, p, i) = 0.0; continue; }
            bm = 0.0; bp = ds; al = -ds;
          } else {
            const double ik = 1.0 / (double)(i - 1);
            bm = ds_qtr * (1.0 - 0.5 * ik);
            bp = i == nr ? 0.0 : ds_qtr * (1.0 + 0.5 * ik);
            al = m == 0 ? -ds_qtr * 2.0 : -(ds_qtr * (2.0 + m2 * ik * ik));
          }
          SL(sr, j, p, i) = dr2_idzh * (3.0 * LS(lr, j, p, i) - 4.0 * LS(lr, j - 1, p, i) + LS(lr, j - 2, p, i)) -
                            kap * LS(li, j, p, i) + bm * LS(lr, j, p, i - 1) + al * LS(lr, j, p, i) +
                            bp * LS(lr, j, p, i + 1);
          SL(si, j, p, i) = dr2_idzh * (3.0 * LS(li, j, p, i) - 4.0 * LS(li, j - 1, p, i) + LS(li, j - 2, p, i)) +
                            kap * LS(lr, j, p, i) + bm * LS(li, j, p, i - 1) + al * LS(li, j, p, i) +
                            bp * LS(li, j, p, i + 1);
        }
      }
      for (int i = 1; i <= nr; ++i) {
        double t[4] = {SL(sr, j, part_of(m, 0), i), SL(si, j, part_of(m, 0), i), 0.0, 0.0};
        if (m > 0) { t[2] = SL(sr, j, PIM(m), i); t[3] = SL(si, j, PIM(m), i); }
        laser_chi_terms(g, chi2, lr, li, j, m, i, cq, t);
        SL(sr, j, part_of(m, 0), i) = t[0];
        SL(si, j, part_of(m, 0), i) = t[1];
        if (m > 0) { SL(sr, j, PIM(m), i) = t[2]; SL(si, j, PIM(m), i) = t[3]; }
      }
    }
}

/* solve (:752-927): slice by slice from the front of the box, `iter` times each, the
 * implicit half: coupling with the current envelope, then one penta-diagonal solve per mode
 * and Re / Im part; m >= 1 axis values zero.  coef: per mode m the PCR tables
 * [cm1 | cm2 | cp1 | cp2 ([steps][2nr] each) | cfin (2nr)]. */
void orc_laser_solve(const orc_grid* g, int iter, double ds, const double* const* coef, const double* chi2,
                     const double* sr, const double* si, double* lr, double* li) {
  const int M = g->max_mode, P = nparts(g), nr = g->nr, n = 2 * nr;
  int steps = 0;
  while ((1 << steps) < n) ++steps;
  const double dr = g->dr, dz = g->dxi;
  const double dr2_idzh = 0.5 * (dr * dr) / dz, cq = 0.25 * ds * (dr * dr);
  double* t = (double*)malloc(sizeof(double) * 4 * (size_t)(M + 1) * nr);
  double* x = (double*)malloc(sizeof(double) * (size_t)n);
  for (int j = 1; j <= g->nz; ++j)
    for (int l = 1; l <= iter; ++l) {
      for (int m = 0; m <= M; ++m)
        for (int i = 1; i <= nr; ++i) {
          double* tt = t + 4 * ((size_t)m * nr + (i - 1));
          tt[0] = tt[1] = tt[2] = tt[3] = 0.0;
          laser_chi_terms(g, chi2, lr, li, j, m, i, cq, tt);
        }
      for (int m = 0; m <= M; ++m) {
        const double* cm1 = coef[m];
        const double* cm2 = cm1 + (size_t)steps * n;
        const double* cp1 = cm2 + (size_t)steps * n;
        const double* cp2 = cp1 + (size_t)steps * n;
        const double* cf = cp2 + (size_t)steps * n;
        for (int h = 0; h < (m == 0 ? 1 : 2); ++h) {
          const int p = part_of(m, h);
          for (int i = 1; i <= nr; ++i) {
            const double* tt = t + 4 * ((size_t)m * nr + (i - 1));
            x[2 * i - 2] = SL(sr, j, p, i) + tt[2 * h] + dr2_idzh * (4.0 * LS(lr, j - 1, p, i) - LS(lr, j - 2, p, i));
            x[2 * i - 1] = SL(si, j, p, i) + tt[2 * h + 1] + dr2_idzh * (4.0 * LS(li, j - 1, p, i) - LS(li, j - 2, p, i));
          }
          orc_pcr_solve(n, cm1, cm2, cp1, cp2, cf, x);
          for (int i = 1; i <= nr; ++i) {
            LS(lr, j, p, i) = x[2 * i - 2];
            LS(li, j, p, i) = x[2 * i - 1];
          }
        }
        if (m > 0) {
          LS(lr, j, PRE(m), 1) = 0.0; LS(li, j, PRE(m), 1) = 0.0;
          LS(lr, j, PIM(m), 1) = 0.0; LS(li, j, PIM(m), 1) = 0.0;
        }
      }
    }
  free(t);
  free(x);
}

/* set_grad (:637-750) for slice j: gradients [P][3][nr+2] (r, phi, xi) of a_r (gr) and a_i
 * (gi), every other entry zero (as left by the zeroing at the 3D step start).  For m >= 1 the
 * reference's axis branch runs with the loop index left at nr + 1 after its loop, so it
 * writes the upper guard node, not node 1 (node 1 keeps r and phi components zero);
 * kept for identical results. */
void orc_laser_grad(const orc_grid* g, const double* lr, const double* li, int j, double* gr, double* gi) {
  const int M = g->max_mode, P = nparts(g), nr = g->nr;
  const double idrh = 0.5 / g->dr, idzh = 0.5 / g->dxi;
  memset(gr, 0, sizeof(double) * 3 * (size_t)P * NR2);
  memset(gi, 0, sizeof(double) * 3 * (size_t)P * NR2);
  const double* src[2] = {lr, li};
  double* dst[2] = {gr, gi};
  for (int h = 0; h < 2; ++h) {
    const double* a = src[h];
    double* gg = dst[h];
    for (int p = 0; p < P; ++p)
      for (int i = 1; i <= nr; ++i)
        F(gg, 3, p, 2, i) = idzh * (3.0 * LS(a, j, p, i) - 4.0 * LS(a, j - 1, p, i) + LS(a, j - 2, p, i));
    for (int i = 2; i <= nr; ++i) {
      F(gg, 3, 0, 0, i) = idrh * (LS(a, j, 0, i + 1) - LS(a, j, 0, i - 1));
      F(gg, 3, 0, 1, i) = 0.0;
    }
    for (int m = 1; m <= M; ++m) {
      const int pr = PRE(m), pi = PIM(m);
      for (int i = 2; i <= nr; ++i) {
        const double ir = 1.0 / ((double)(i - 1) * g->dr);
        F(gg, 3, pr, 0, i) = idrh * (LS(a, j, pr, i + 1) - LS(a, j, pr, i - 1));
        F(gg, 3, pi, 0, i) = idrh * (LS(a, j, pi, i + 1) - LS(a, j, pi, i - 1));
        F(gg, 3, pr, 1, i) = -ir * (double)m * LS(a, j, pi, i);
        F(gg, 3, pi, 1, i) = ir * (double)m * LS(a, j, pr, i);
      }
      const int ig = nr + 1;
      if (m % 2 == 1) {
        F(gg, 3, pr, 0, ig) = 2.0 * idrh * LS(a, j, pr, 2);
        F(gg, 3, pi, 0, ig) = 2.0 * idrh * LS(a, j, pi, 2);
        F(gg, 3, pr, 1, ig) = -((double)m * F(gg, 3, pi, 0, ig));
        F(gg, 3, pi, 1, ig) = (double)m * F(gg, 3, pr, 0, ig);
      }
    }
  }
}

void orc_sim_set_laser(orc_sim* s, int k, const double* ar, const double* ai) {
  const orc_grid* g = &s->d.g;
  const int P = s->P, nr = g->nr;
  for (int j = 1; j <= g->nz; ++j)
    for (int p = 0; p < P; ++p)
      for (int i = 1; i <= nr; ++i) {
        const size_t o = ((size_t)(j - 1) * P + p) * nr + (i - 1);
        LS(s->lr2[k], j, p, i) = ar[o];
        LS(s->li2[k], j, p, i) = ai[o];
      }
}

void orc_sim_laser(orc_sim* s, int k, double** ar, double** ai) { *ar = s->lr2[k]; *ai = s->li2[k]; }

/* :362-367 laser_all = sum over the lasers of slice j's envelope (copy_slice) and gradients (set_grad) */
static void lasers_slice(orc_sim* s, int j) {
  const orc_grid* g = &s->d.g;
  const int P = s->P;
  const size_t n1 = s->n1;
  memset(s->la_r, 0, n1 * sizeof(double)); memset(s->la_i, 0, n1 * sizeof(double));
  memset(s->la_gr, 0, 3 * n1 * sizeof(double)); memset(s->la_gi, 0, 3 * n1 * sizeof(double));
  for (int k = 0; k < s->d.nlasers; ++k) {
    orc_laser_grad(g, s->lr2[k], s->li2[k], j, s->lgr, s->lgi);
    for (int p = 0; p < P; ++p)
      for (int i = 0; i < NR2; ++i) {
        F(s->la_r, 1, p, 0, i) = F(s->la_r, 1, p, 0, i) + LS(s->lr2[k], j, p, i);
        F(s->la_i, 1, p, 0, i) = F(s->la_i, 1, p, 0, i) + LS(s->li2[k], j, p, i);
      }
    for (size_t i = 0; i < 3 * n1; ++i) {
      s->la_gr[i] = s->la_gr[i] + s->lgr[i];
      s->la_gi[i] = s->la_gi[i] + s->lgi[i];
    }
  }
}

/* :485-486 lasers%advance (sim_lasers_class.f03:202-223): set_rhs, then solve */
static void lasers_advance(orc_sim* s) {
  const orc_grid* g = &s->d.g;
  for (int k = 0; k < s->d.nlasers; ++k) {
    orc_laser_rhs(g, s->d.laser_k0[k], s->d.dt3d, s->chi2, s->lr2[k], s->li2[k], s->lsr[k], s->lsi[k]);
    orc_laser_solve(g, s->d.laser_iter[k], s->d.dt3d, (const double* const*)s->lcoef[k], s->chi2, s->lsr[k],
                    s->lsi[k], s->lr2[k], s->li2[k]);
  }
}

static int is_pgc(int push_type) { return push_type == ORC_PUSH_STD_PGC || push_type == ORC_PUSH_ROBUST_PGC; }

/* one xi slice j: simulation_class.f03:342-469 */
void orc_sim_slice(orc_sim* s, int j, int* iters, double* rel) {
  const orc_grid* g = &s->d.g;
  const int nt = s->d.nthreads;
  const double dxi = g->dxi;
  const size_t n1 = s->n1;
  if (s->d.extrap > 0 && j > s->d.extrap + 1) {
    /* not in the reference, which carries B-perp(j-1) into slice j: the initial B-perp guess
       extrapolated from the stored slices j-1, j-2 (order 1) or j-1..j-3 (order 2), every
       mode part, nodes 1..nr */
    const int P = s->P;
    for (int p = 0; p < P; ++p)
      for (int c = 0; c < 2; ++c)
        for (int i = 1; i <= g->nr; ++i) {
          const double b1 = F2(s->b_spe2, 3, j - 1, p, c, i), b2 = F2(s->b_spe2, 3, j - 2, p, c, i);
          F(s->b_spe, 3, p, c, i) = s->d.extrap == 1 ? 2.0 * b1 - b2
                                                     : 3.0 * (b1 - b2) + F2(s->b_spe2, 3, j - 3, p, c, i);
        }
  }
  {
    /* :344-345 q_beam%copy_slice(j, 2->1); b_beam%solve(q_beam) */
    memcpy(s->q_beam, s->q_beam2 + (size_t)(j - 1) * n1, n1 * sizeof(double));
    orc_solve_bt_beam(g, s->q_beam, s->b_beam);
    /* :346-349 q_spe = 0; spe%qdp(q_spe) (species2d_class.f03:186-208) */
    memset(s->q_spe, 0, n1 * sizeof(double));
    memset(s->qsp, 0, n1 * sizeof(double));
    orc_qdeposit(g, s->np, s->x, s->y, s->q, s->qsp);
    for (int k = 0; k < s->d.smooth_order; ++k) orc_smooth(g, 0, s->qsp);   /* q%smooth(), :202 */
    for (size_t i = 0; i < n1; ++i) s->q_spe[i] = s->q_spe[i] + s->qsp[i];
    if (s->d.sp_neutralized) for (size_t i = 0; i < n1; ++i) s->q_spe[i] = s->q_spe[i] + s->qn[i];
    if (s->d.neut_levels > 0) {
      /* :351-354 neut%qdp (qdeposit_neutral :880-902) and neut%ion_deposit (:904-930) */
      memset(s->qneut, 0, n1 * sizeof(double));
      orc_qdeposit(g, s->nnp, s->nx, s->ny, s->nq, s->qneut);
      for (int k = 0; k < s->d.smooth_order; ++k) orc_smooth(g, 0, s->qneut);
      for (size_t i = 0; i < n1; ++i) s->q_spe[i] = s->q_spe[i] + s->qneut[i];
      memset(s->rho_add, 0, n1 * sizeof(double));
      orc_qdeposit(g, s->na, s->ax, s->ay, s->aq, s->rho_add);
      for (int k = 0; k < s->d.smooth_order; ++k) orc_smooth(g, 0, s->rho_add);
      for (size_t i = 0; i < n1; ++i) s->rho_ion[i] = s->rho_ion[i] + s->rho_add[i];
      for (size_t i = 0; i < n1; ++i) s->q_spe[i] = s->q_spe[i] + s->rho_ion[i];
      s->na = 0;
    }
    /* :356-360 */
    orc_solve_psi(g, s->q_spe, s->psi);
    if (s->d.sp_push_type == ORC_PUSH_STD || s->d.sp_push_type == ORC_PUSH_STD_PGC)
      orc_interp_psi(g, s->np, s->x, s->y, s->psi, s->ppsi);
    orc_solve_bz(g, s->cu, s->b_spe);
    if (s->d.nlasers > 0) lasers_slice(s, j);
    const orc_laser_f1 lf = {s->la_r, s->la_i, s->la_gr, s->la_gi};
    /* :370-398 predictor-corrector */
    int l;
    double rel_res = 0.0, abs_res = 0.0;
    for (l = 1; l <= s->d.iter_max; ++l) {
      orc_conv_record(g, s->b_spe, s->s_re, s->s_im);
      for (size_t i = 0; i < 3 * n1; ++i) s->b[i] = s->b_spe[i] + s->b_beam[i];
      orc_solve_ez(g, s->cu, s->e);
      orc_solve_et(g, s->b, s->psi, s->e);
      memset(s->cu, 0, 3 * n1 * sizeof(double));
      memset(s->acu, 0, 2 * n1 * sizeof(double));
      memset(s->amu, 0, 3 * n1 * sizeof(double));
      if (is_pgc(s->d.sp_push_type))
        orc_amjdeposit_pgc(g, s->d.sp_push_type, s->d.sp_qbm, dxi, s->np, s->x, s->y, s->px, s->py, s->pz,
                           s->q, s->gamma, s->ppsi, s->e, s->b, &lf, s->cu, s->amu, s->acu);
      else
        orc_amjdeposit(g, s->d.sp_push_type, s->d.sp_qbm, dxi, s->np, s->x, s->y, s->px, s->py, s->pz,
                       s->q, s->gamma, s->ppsi, s->e, s->b, s->cu, s->amu, s->acu, nt);
      for (int k = 0; k < s->d.smooth_order; ++k) {      /* cu, dcu, amu %smooth(), :270-272 */
        orc_smooth(g, 1, s->cu);
        orc_smooth(g, 2, s->acu);
        orc_smooth(g, 1, s->amu);
      }
      if (s->d.neut_levels > 0) {                      /* :384-386 neut%amjdp (:932-973), not smoothed */
        memset(s->cun, 0, 3 * n1 * sizeof(double));
        memset(s->acun, 0, 2 * n1 * sizeof(double));
        memset(s->amun, 0, 3 * n1 * sizeof(double));
        orc_amjdeposit(g, s->d.neut_push_type, s->d.neut_qbm, dxi, s->nnp, s->nx, s->ny, s->npx, s->npy, s->npz,
                       s->nq, s->ngamma, s->npsi, s->e, s->b, s->cun, s->amun, s->acun, nt);
        for (size_t i = 0; i < 3 * n1; ++i) { s->cu[i] = s->cu[i] + s->cun[i]; s->amu[i] = s->amu[i] + s->amun[i]; }
        for (size_t i = 0; i < 2 * n1; ++i) s->acu[i] = s->acu[i] + s->acun[i];
      }
      orc_solve_djdxi(g, s->acu, s->amu, s->dcu);
      orc_solve_bt_iter(g, s->dcu, s->cu, s->b_spe);
      orc_solve_bz(g, s->cu, s->b_spe);
      orc_conv_compare(g, s->b_spe, s->s_re, s->s_im, &rel_res, &abs_res);
      if (rel_res < s->d.iter_reltol || abs_res < s->d.iter_abstol) break;
    }
    if (iters) *iters = l > s->d.iter_max ? s->d.iter_max : l;
    if (rel) *rel = rel_res;
    /* :400-401 lasers%deposit_chi (sim_lasers_class.f03:176-200): chi of slice j into its store */
    if (s->d.nlasers > 0) {
      memset(s->chi, 0, n1 * sizeof(double));
      orc_deposit_chi(g, s->d.sp_qbm, s->d.sp_ppc_r, s->np, s->x, s->y, s->q, s->ppsi, s->chi);
      memcpy(s->chi2 + (size_t)(j - 1) * n1, s->chi, n1 * sizeof(double));
    }
    /* :403-416 cbq, stores */
    copy_1to2(s, s->cu, s->cu2, 3, j);
    for (int i = 0; i < NR2 * s->P; ++i) {
      int p = i / NR2, n = i % NR2;
      F(s->q_spe, 1, p, 0, n) = F(s->q_spe, 1, p, 0, n) + F(s->cu, 3, p, 2, n);
    }
    copy_1to2(s, s->q_spe, s->q_spe2, 1, j);
    for (size_t i = 0; i < 3 * n1; ++i) s->b[i] = s->b_spe[i] + s->b_beam[i];
    orc_solve_et(g, s->b_spe, s->psi, s->e_spe);
    orc_solve_ez(g, s->cu, s->e);
    orc_solve_et(g, s->b, s->psi, s->e);
    /* :425-426 dcu *= dxi; cu(1:2) += dcu(1:2) */
    for (size_t i = 0; i < 2 * n1; ++i) s->dcu[i] = s->dcu[i] * dxi;
    for (int p = 0; p < s->P; ++p)
      for (int c = 0; c < 2; ++c)
        for (int n = 0; n < NR2; ++n) F(s->cu, 3, p, c, n) = F(s->cu, 3, p, c, n) + F(s->dcu, 2, p, c, n);
    /* :437-441 push_u, push_x (+update_bound) */
    if (is_pgc(s->d.sp_push_type))
      orc_push_u_pgc(g, s->d.sp_qbm, dxi, s->np, s->x, s->y, s->px, s->py, s->pz, s->gamma, s->ppsi, s->e, s->b, &lf);
    else
      orc_push_u(g, s->d.sp_push_type, s->d.sp_qbm, dxi, s->np, s->x, s->y, s->px, s->py, s->pz,
                 s->gamma, s->ppsi, s->e, s->b, nt);
    orc_push_x(s->np, dxi, s->x, s->y, s->px, s->py, s->pz, s->gamma);
    s->np = orc_update_bound(g, s->np, s->x, s->y, s->px, s->py, s->pz, s->gamma, s->ppsi, s->q);
    if (s->d.neut_levels > 0) {                        /* :443-449 neut%update, push_u, push_x */
      neutral_update(s);
      orc_push_u(g, s->d.neut_push_type, s->d.neut_qbm, dxi, s->nnp, s->nx, s->ny, s->npx, s->npy, s->npz,
                 s->ngamma, s->npsi, s->e, s->b, nt);
      orc_push_x(s->nnp, dxi, s->nx, s->ny, s->npx, s->npy, s->npz, s->ngamma);
      s->nnp = orc_update_bound(g, s->nnp, s->nx, s->ny, s->npx, s->npy, s->npz, s->ngamma, s->npsi, s->nq);
    }
    /* :452-456 copy slices */
    copy_1to2(s, s->e, s->e2, 3, j);
    copy_1to2(s, s->b, s->b2, 3, j);
    copy_1to2(s, s->psi, s->psi2, 1, j);
    copy_1to2(s, s->b_spe, s->b_spe2, 3, j);
    copy_1to2(s, s->e_spe, s->e_spe2, 3, j);
  }
}

/* :487-492 beam push (slice nz+1 of e2/b2 stays zero on one stage) */
void orc_sim_end_3dstep(orc_sim* s, int push_beams) {
  const orc_grid* g = &s->d.g;
  const int nt = s->d.nthreads;
  if (s->d.nlasers > 0) lasers_advance(s);
  if (push_beams) {
    for (int k = 0; k < s->d.nbeams; ++k) {
      orc_beam_push(g, s->d.beam_push_type[k], s->d.beam_qbm[k], s->d.dt3d, s->nb[k], s->bx[k], s->by[k],
                    s->bz[k], s->bpx[k], s->bpy[k], s->bpz[k], s->e2, s->b2, nt);
      s->nb[k] = orc_beam_update_bound(g, s->nb[k], s->bx[k], s->by[k], s->bz[k], s->bpx[k], s->bpy[k],
                                       s->bpz[k], s->bq[k]);
    }
  }
}

void orc_sim_run_3dstep(orc_sim* s, int push_beams, int* iters, double* rel) {
  orc_sim_begin_3dstep(s);
  for (int j = 1; j <= s->d.g.nz; ++j) orc_sim_slice(s, j, iters ? iters + (j - 1) : NULL, rel ? rel + (j - 1) : NULL);
  orc_sim_end_3dstep(s, push_beams);
}

double* orc_sim_field(orc_sim* s, const char* name, int* nc) {
  struct { const char* n; double* p; int c; } t[] = {
      {"psi", s->psi, 1}, {"e", s->e, 3}, {"e_spe", s->e_spe, 3}, {"b", s->b, 3},
      {"b_spe", s->b_spe, 3}, {"b_beam", s->b_beam, 3}, {"cu", s->cu, 3}, {"amu", s->amu, 3},
      {"acu", s->acu, 2}, {"dcu", s->dcu, 2}, {"q_spe", s->q_spe, 1}, {"q_beam", s->q_beam, 1},
      {"qn", s->qn, 1}};
  for (size_t i = 0; i < sizeof(t) / sizeof(t[0]); ++i)
    if (!strcmp(t[i].n, name)) { if (nc) *nc = t[i].c; return t[i].p; }
  return NULL;
}

double* orc_sim_store(orc_sim* s, const char* name, int* nc) {
  struct { const char* n; double* p; int c; } t[] = {
      {"q_beam", s->q_beam2, 1}, {"e", s->e2, 3}, {"b", s->b2, 3}, {"psi", s->psi2, 1},
      {"b_spe", s->b_spe2, 3}, {"e_spe", s->e_spe2, 3}, {"cu", s->cu2, 3}, {"q_spe", s->q_spe2, 1}, {"chi", s->chi2, 1}};
  for (size_t i = 0; i < sizeof(t) / sizeof(t[0]); ++i)
    if (!strcmp(t[i].n, name)) { if (nc) *nc = t[i].c; return t[i].p; }
  return NULL;
}

int64_t orc_sim_neutral(orc_sim* s, double** x, double** y, double** px, double** py, double** pz,
                        double** gamma, double** psi, double** q) {
  *x = s->nx; *y = s->ny; *px = s->npx; *py = s->npy; *pz = s->npz; *gamma = s->ngamma; *psi = s->npsi; *q = s->nq;
  return s->nnp;
}

double* orc_sim_multi_ion(orc_sim* s) { return s->multi_ion; }

int64_t orc_sim_plasma(orc_sim* s, double** x, double** y, double** px, double** py, double** pz,
                       double** gamma, double** psi, double** q) {
  *x = s->x; *y = s->y; *px = s->px; *py = s->py; *pz = s->pz; *gamma = s->gamma; *psi = s->ppsi; *q = s->q;
  return s->np;
}

int64_t orc_sim_beam(orc_sim* s, int k, double** x, double** y, double** z, double** px, double** py,
                     double** pz, double** q) {
  *x = s->bx[k]; *y = s->by[k]; *z = s->bz[k]; *px = s->bpx[k]; *py = s->bpy[k]; *pz = s->bpz[k]; *q = s->bq[k];
  return s->nb[k];
}
