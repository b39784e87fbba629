/*
 * shl_limit.h -- Loop limit-surface evaluation at any (v, w) of a face, shared
 * bit for bit by the CUDA kernels and the host code (library set-up, CPU
 * oracle).
 *
 * Reference behaviour (file:line):
 *  - SubdivEvaluation::evaluate / evaluate_deriv (SubdivEvaluation.C:14-165):
 *    a regular patch (first vertex of valence 6) is evaluated with Stam's 12
 *    box splines; an irregular patch is subdivided n times around its
 *    irregular vertex, n = floor(1 - log2(v + w)) after clamping points closer
 *    than irregular_tol = 1e-10 to the vertex (rescale_irregular_coords,
 *    SubdivEvaluation.C:168-187), and evaluated in one of the three regular
 *    children of the n-th step: k = 0 for v > 1/2 with local (2v - 1, 2w),
 *    k = 2 for w > 1/2 with (2v, 2w - 1), else the middle child k = 1 with
 *    (1 - 2v, 1 - 2w).  The children's control points are fixed linear
 *    combinations of the patch nodes (the tables of shl_subdiv.h; the
 *    reference's PAnArray, SubdivEvaluation.h:14-96, holds the same matrices in
 *    libMesh's node order, at most max_A_exponent = 34 levels).
 *    Derivatives: d/dv of the local coordinates is 2^n for k = 0, 2 and -2^n
 *    for the middle child (chain rule through the n-1 rescalings by 2 and the
 *    child map).  SubdivEvaluation.C:125 uses (-2)^n for the middle child,
 *    whose sign differs for even n; this restatement follows the chain rule,
 *    so its tangents are the derivatives of its positions everywhere.
 *
 * Every floating-point operation is rounded on its own (SHL_MUL / SHL_ADD of
 * shl_distance.h) or is an explicit fused multiply-add (fma, IEEE on both sides);
 * frexp / ldexp are exact, so host and device agree bit for bit.
 */
#ifndef SHL_LIMIT_H_
#define SHL_LIMIT_H_

#include <stdint.h>

#include "shl_distance.h"

#ifndef __CUDACC__
#include <math.h>
#endif

#define SHL_SMOOTH_LEVELS 34        /* max_A_exponent = floor(1 - log2(irregular_tol)) */
#define SHL_IRREGULAR_TOL 1e-10
#define SHL_SMOOTH_MAX_SLOTS 18     /* patch nodes of the largest valence (12) */
/* Stam's box splines (J. Stam, "Evaluation of Loop subdivision surfaces",
 * SIGGRAPH'98 course notes) expanded into monomials of (v, w) with
 * u = 1 - v - w: basis s = (1/12) sum_m C[s][m] v^p w^q over the monomials
 * m = (p, q) in the order (0,0) (0,1) .. (0,4) (1,0) .. (1,3) (2,0) (2,1) (2,2)
 * (3,0) (3,1) (4,0).  Integer coefficients, exact in double. */
#define SHL_BOX_COEFFS                                                        \
  {{1, -4, 6, -4, 1, -2, 6, -6, 2, 0, 0, 0, 2, -2, -1},                       \
   {1, -2, 0, 2, -1, -4, 6, 0, -2, 6, -6, 0, -4, 2, 1},                       \
   {1, -2, 0, 2, -1, 2, -6, 6, -2, 0, 0, 0, -4, 4, 2},                        \
   {6, 0, -12, 8, -1, 0, -12, 12, -2, -12, 12, 0, 8, -2, -1},                 \
   {1, 2, 0, -4, 2, -2, -6, 0, 4, 0, 6, 0, 2, -2, -1},                        \
   {0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 2, -2, -1},                           \
   {1, 2, 0, -4, 2, 4, 6, -12, 4, 6, -6, 0, -4, -2, -1},                      \
   {1, 4, 6, -4, -1, 2, 6, -6, -2, 0, -12, 0, -4, 4, 2},                      \
   {0, 0, 0, 2, -1, 0, 0, 0, -2, 0, 0, 0, 0, 0, 0},                           \
   {0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 2, 1},                             \
   {0, 0, 0, 2, -1, 0, 0, 6, -2, 0, 6, 0, 2, -2, -1},                         \
   {0, 0, 0, 0, 1, 0, 0, 0, 2, 0, 0, 0, 0, 0, 0}}
#define SHL_BOX_P {0, 0, 0, 0, 0, 1, 1, 1, 1, 2, 2, 2, 3, 3, 4}
#define SHL_BOX_Q {0, 1, 2, 3, 4, 0, 1, 2, 3, 0, 1, 2, 0, 1, 0}
/* patch slot (this library's regular-patch order) of Stam node s */
#define SHL_STAM_SLOT {5, 4, 6, 0, 3, 9, 1, 2, 11, 8, 7, 10}

/* Device loops over the twelve splines and fifteen monomials unroll fully, so
 * that the tables fold into the code (no table loads, no dynamically indexed
 * arrays); the host runs the same loops, operation for operation. */
#ifdef __CUDA_ARCH__
#define SHL_UNROLL _Pragma("unroll")
#define SHL_TABLE const
#else
#define SHL_UNROLL
#define SHL_TABLE static const
#endif

/* rescale_irregular_coords (SubdivEvaluation.C:168-187): returns n and scales
 * (v, w) by 2^(n-1) so that v + w lies in (1/2, 1].  n = floor(1 - log2(v+w))
 * is computed exactly from the binary exponent. */
SHL_HD int shl_rescale_irregular(double* v, double* w)
{
  if (SHL_ADD(*v, *w) < SHL_IRREGULAR_TOL) {
    *v = fmax(*v, SHL_IRREGULAR_TOL);
    *w = fmax(*w, 0.0);
  }
  const double s = SHL_ADD(*v, *w);
  int e = 0;
  const double fr = frexp(s, &e);  /* s = fr 2^e, fr in [1/2, 1) */
  int m = -e + (fr == 0.5 ? 1 : 0);  /* floor(-log2 s) */
  /* n in [1, SHL_SMOOTH_LEVELS] for any input (v + w rounded above 1, NaN) */
  if (!(m >= 0)) m = 0;
  if (m > SHL_SMOOTH_LEVELS - 1) m = SHL_SMOOTH_LEVELS - 1;
  *v = ldexp(*v, m);
  *w = ldexp(*w, m);
  return m + 1;
}

/* A face's limit patch: its node positions in this library's patch order
 * (a, b, c, the remaining ring of a, d, b_far0, b_far1, c_far0, c_far1) as
 * base + 3 * ids[j * stride], the valence N of its first vertex, and for
 * N != 6 the subdivision table of valence N (shl_subdiv.h layout: [level n-1]
 * [child k][Stam node s][slot]). */
typedef struct {
  const double* base;
  const uint32_t* ids;
  uint32_t stride;
  int N;
  const double* tab;
} shl_limit_patch;

#define SHL_FMA(a, b, c) fma((a), (b), (c))
#define SHL_LIMIT_NCOEF 45  /* power-form coefficients of a regular patch: 15 monomials x 3 */

/* The limit surface of a regular (sub-)patch over its triangle is a quartic
 * polynomial: sum_s B_s(v, w) Q_s = sum_m P_m v^p w^q with the power-form
 * coefficients P_m = (1/12) sum_s C[s][m] Q_s of its twelve control points Q_s
 * (Stam node order; m in the monomial order of SHL_BOX_P / SHL_BOX_Q).
 * shl_limit_add_point adds control point s to the coefficients (s ascending,
 * fused multiply-adds from zero, so P_m's rounding does not depend on how
 * the points are formed); shl_limit_scale applies the 1/12. */
SHL_HD void shl_limit_add_point(double P[15][3], int s, double q0, double q1, double q2)
{
  SHL_TABLE signed char BC[12][15] = SHL_BOX_COEFFS;
  SHL_UNROLL
  for (int m = 0; m < 15; ++m) {
    const int c = BC[s][m];
    if (c == 0) continue;
    P[m][0] = SHL_FMA((double)c, q0, P[m][0]);
    P[m][1] = SHL_FMA((double)c, q1, P[m][1]);
    P[m][2] = SHL_FMA((double)c, q2, P[m][2]);
  }
}

SHL_HD void shl_limit_scale(double P[15][3])
{
  const double twelfth = 1.0 / 12.0;
  SHL_UNROLL
  for (int m = 0; m < 15; ++m) {
    P[m][0] = SHL_MUL(P[m][0], twelfth);
    P[m][1] = SHL_MUL(P[m][1], twelfth);
    P[m][2] = SHL_MUL(P[m][2], twelfth);
  }
}

/* Power-form coefficients of a regular patch (N = 6) from its nodes. */
SHL_HD void shl_limit_coeffs_regular(const shl_limit_patch* pt, double P[15][3])
{
  SHL_TABLE signed char SLOT[12] = SHL_STAM_SLOT;
  SHL_UNROLL
  for (int m = 0; m < 15; ++m) P[m][0] = P[m][1] = P[m][2] = 0.0;
  SHL_UNROLL
  for (int s = 0; s < 12; ++s) {
    const double* x = pt->base + 3 * (size_t)pt->ids[(size_t)SLOT[s] * pt->stride];
    shl_limit_add_point(P, s, x[0], x[1], x[2]);
  }
  shl_limit_scale(P);
}

/* Evaluation of the power form at (v, w) of the (sub-)patch's triangle:
 * out[0] the point, out[1] d/dv, out[2] d/dw (order >= 1), out[3] d2/dv2,
 * out[4] d2/dw2, out[5] d2/dvdw (order 2), the derivatives times j1 and j1^2
 * (the chain rule of an irregular patch's sub-patch map; j1 = 1 for a regular
 * patch, a power of two otherwise, so the scaling is exact).  Each sum runs
 * over the monomials in order; the integer factors of the derivatives scale
 * the monomials. */
SHL_HD void shl_limit_poly(const double P[15][3], double v, double w, int order, double j1, double out[6][3])
{
  SHL_TABLE signed char BP[15] = SHL_BOX_P;
  SHL_TABLE signed char BQ[15] = SHL_BOX_Q;
  double vp[5], wp[5];
  vp[0] = 1.0;
  wp[0] = 1.0;
  SHL_UNROLL
  for (int i = 1; i < 5; ++i) {
    vp[i] = SHL_MUL(vp[i - 1], v);
    wp[i] = SHL_MUL(wp[i - 1], w);
  }
  double a0 = 0.0, a1 = 0.0, a2 = 0.0;
  SHL_UNROLL
  for (int m = 0; m < 15; ++m) {
    const double t = SHL_MUL(vp[BP[m]], wp[BQ[m]]);
    a0 = SHL_FMA(P[m][0], t, a0);
    a1 = SHL_FMA(P[m][1], t, a1);
    a2 = SHL_FMA(P[m][2], t, a2);
  }
  out[0][0] = a0;
  out[0][1] = a1;
  out[0][2] = a2;
  if (order < 1) return;
  double d[5][3];
  SHL_UNROLL
  for (int q = 0; q < 5; ++q) d[q][0] = d[q][1] = d[q][2] = 0.0;
  SHL_UNROLL
  for (int m = 0; m < 15; ++m) {
    const int p = BP[m], q = BQ[m];
    if (p >= 1) {
      const double t = SHL_MUL((double)p, SHL_MUL(vp[p - 1], wp[q]));
      for (int c = 0; c < 3; ++c) d[0][c] = SHL_FMA(P[m][c], t, d[0][c]);
    }
    if (q >= 1) {
      const double t = SHL_MUL((double)q, SHL_MUL(vp[p], wp[q - 1]));
      for (int c = 0; c < 3; ++c) d[1][c] = SHL_FMA(P[m][c], t, d[1][c]);
    }
    if (order < 2) continue;
    if (p >= 2) {
      const double t = SHL_MUL((double)(p * (p - 1)), SHL_MUL(vp[p - 2], wp[q]));
      for (int c = 0; c < 3; ++c) d[2][c] = SHL_FMA(P[m][c], t, d[2][c]);
    }
    if (q >= 2) {
      const double t = SHL_MUL((double)(q * (q - 1)), SHL_MUL(vp[p], wp[q - 2]));
      for (int c = 0; c < 3; ++c) d[3][c] = SHL_FMA(P[m][c], t, d[3][c]);
    }
    if (p >= 1 && q >= 1) {
      const double t = SHL_MUL((double)(p * q), SHL_MUL(vp[p - 1], wp[q - 1]));
      for (int c = 0; c < 3; ++c) d[4][c] = SHL_FMA(P[m][c], t, d[4][c]);
    }
  }
  const double j2 = SHL_MUL(j1, j1);
  for (int c = 0; c < 3; ++c) {
    out[1][c] = SHL_MUL(d[0][c], j1);
    out[2][c] = SHL_MUL(d[1][c], j1);
  }
  if (order < 2) return;
  for (int c = 0; c < 3; ++c) {
    out[3][c] = SHL_MUL(d[2][c], j2);
    out[4][c] = SHL_MUL(d[3][c], j2);
    out[5][c] = SHL_MUL(d[4][c], j2);
  }
}

/* Limit surface of a patch at (v, w) (outputs as shl_limit_poly).  An
 * irregular patch is evaluated in the regular child of the n-th subdivision
 * step that holds (v, w), whose control points are table rows of the patch
 * nodes (each formed by fused multiply-adds over the nonzero weights). */
SHL_HD void shl_limit_eval(const shl_limit_patch* pt, double v, double w, int order, double out[6][3])
{
  double P[15][3];
  double j1 = 1.0;
  if (pt->N == 6) {
    shl_limit_coeffs_regular(pt, P);
  } else {
    const int n = shl_rescale_irregular(&v, &w);
    int k;
    if (v > 0.5) {
      k = 0;
      v = SHL_SUB(SHL_MUL(2.0, v), 1.0);
      w = SHL_MUL(2.0, w);
      j1 = ldexp(1.0, n);
    } else if (w > 0.5) {
      k = 2;
      v = SHL_MUL(2.0, v);
      w = SHL_SUB(SHL_MUL(2.0, w), 1.0);
      j1 = ldexp(1.0, n);
    } else {
      k = 1;
      v = SHL_SUB(1.0, SHL_MUL(2.0, v));
      w = SHL_SUB(1.0, SHL_MUL(2.0, w));
      j1 = -ldexp(1.0, n);
    }
    const int np = pt->N + 6;
    const double* T = pt->tab + (size_t)((n - 1) * 3 + k) * 12 * (size_t)np;
    for (int m = 0; m < 15; ++m) P[m][0] = P[m][1] = P[m][2] = 0.0;
    SHL_UNROLL
    for (int s = 0; s < 12; ++s) {
      double Q0 = 0.0, Q1 = 0.0, Q2 = 0.0;
      for (int j = 0; j < np; ++j) {
        const double t = T[s * np + j];
        if (t == 0.0) continue;
        const double* x = pt->base + 3 * (size_t)pt->ids[(size_t)j * pt->stride];
        Q0 = SHL_FMA(t, x[0], Q0);
        Q1 = SHL_FMA(t, x[1], Q1);
        Q2 = SHL_FMA(t, x[2], Q2);
      }
      shl_limit_add_point(P, s, Q0, Q1, Q2);
    }
    shl_limit_scale(P);
  }
  shl_limit_poly(P, v, w, order, j1, out);
}


#endif /* SHL_LIMIT_H_ */
