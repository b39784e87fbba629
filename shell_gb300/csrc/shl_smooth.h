/*
 * shl_smooth.h -- Loop limit-surface evaluation at any (v, w) of a face and the
 * closest points of two limit patches (SMOOTH self-contact), shared bit for
 * bit by the CUDA kernels and the host code (library set-up, CPU oracle).
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
 *  - SmoothShellShellContact::compute (SmoothShellShellContact.C:16-60):
 *    minimise f(x) = |p2(v2, w2) - p1(v1, w1)|^2 over x = (v1, w1, v2, w2)
 *    subject to v, w >= 0 and v + w <= 1 per element, starting from the
 *    previous solution of the pair (1/3 for a new pair).  The constraint hooks
 *    are kept: constraint activity within 100 eps (update_constraint_bitmap,
 *    :139-152), the largest feasible step along a direction (find_max_alpha,
 *    :96-136), and the projection back onto the triangles (apply_constraints,
 *    :155-179).  The minimiser itself (ConstrainedMinimizer.h) is not part of
 *    the reference's sources; it is restated here as an active-set projected
 *    Newton method: exact Hessian of f from the limit surface's second
 *    derivatives, shifted to positive definite on the free subspace (the
 *    line search then starts at the boundary, f being not convex there, and
 *    goes on from a step of length 0.05 if that is rejected), the
 *    working set from the first-order multipliers of the active constraints,
 *    an Armijo backtracking line search capped by find_max_alpha.  It stops
 *    when the gradient projected on the free directions of the working set
 *    is below 1e-9 of the gradient (first-order optimality), when the
 *    decrease the Newton step promises is below 1e-15 of f, after
 *    a full Newton step (convex model) shorter than 1e-6 (quadratic
 *    convergence: the next would be of order 1e-12), when a step no longer
 *    changes x by more than 1e-14, when the line search can no longer decrease
 *    f, or after SHL_SMOOTH_MAX_IT iterations.
 *
 * Every floating-point operation is rounded on its own (SHL_MUL / SHL_ADD of
 * shl_distance.h) or is an explicit fused multiply-add (fma, IEEE on both sides);
 * frexp / ldexp are exact, so host and device agree bit for bit.
 */
#ifndef SHL_SMOOTH_H_
#define SHL_SMOOTH_H_

#include <stdint.h>

#include "shl_distance.h"

#ifndef __CUDACC__
#include <math.h>
#endif

#define SHL_SMOOTH_LEVELS 34        /* max_A_exponent = floor(1 - log2(irregular_tol)) */
#define SHL_IRREGULAR_TOL 1e-10
#define SHL_SMOOTH_MAX_SLOTS 18     /* patch nodes of the largest valence (12) */
#define SHL_SMOOTH_MAX_IT 40
#define SHL_SMOOTH_CONSTRAINT_TOL (100 * 2.220446049250313e-16)
#define SHL_SMOOTH_STEP_TOL 1e-14
#define SHL_SMOOTH_DECREMENT_TOL 1e-15
#define SHL_SMOOTH_QUAD_TOL 1e-6
#define SHL_SMOOTH_KKT_TOL 1e-9
#define SHL_SMOOTH_MAX_HALVINGS 30

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

#ifdef __CUDACC__
static __constant__ signed char kShlBoxC_d[12][15] = SHL_BOX_COEFFS;
static __constant__ signed char kShlBoxP_d[15] = SHL_BOX_P;
static __constant__ signed char kShlBoxQ_d[15] = SHL_BOX_Q;
static __constant__ signed char kShlStamSlot_d[12] = SHL_STAM_SLOT;
#endif
static const signed char kShlBoxC_h[12][15] = SHL_BOX_COEFFS;
static const signed char kShlBoxP_h[15] = SHL_BOX_P;
static const signed char kShlBoxQ_h[15] = SHL_BOX_Q;
static const signed char kShlStamSlot_h[12] = SHL_STAM_SLOT;

#ifdef __CUDA_ARCH__
#define SHL_BOXC kShlBoxC_d
#define SHL_BOXP kShlBoxP_d
#define SHL_BOXQ kShlBoxQ_d
#define SHL_STAMSLOT kShlStamSlot_d
#else
#define SHL_BOXC kShlBoxC_h
#define SHL_BOXP kShlBoxP_h
#define SHL_BOXQ kShlBoxQ_h
#define SHL_STAMSLOT kShlStamSlot_h
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

/* Limit surface of a patch at (v, w): out[0] the point, out[1] d/dv, out[2]
 * d/dw (order >= 1), out[3] d2/dv2, out[4] d2/dw2, out[5] d2/dvdw (order 2).
 * The twelve control points of the regular (sub-)patch are formed one at a
 * time and contracted with the box splines as they are evaluated (12 times
 * the splines, scaled by 1/12 at the end), in fused multiply-adds; fma is
 * IEEE on host and device, so both round alike. */
SHL_HD void shl_limit_eval(const shl_limit_patch* pt, double v, double w, int order, double out[6][3])
{
  double j1 = 1.0;
  int n = 0, k = 0;
  if (pt->N != 6) {
    n = shl_rescale_irregular(&v, &w);
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
  }
  const int np = pt->N + 6;
  const double* T = pt->N == 6 ? 0 : pt->tab + (size_t)((n - 1) * 3 + k) * 12 * (size_t)np;
  double vp[5], wp[5];
  vp[0] = 1.0;
  wp[0] = 1.0;
  for (int i = 1; i < 5; ++i) {
    vp[i] = SHL_MUL(vp[i - 1], v);
    wp[i] = SHL_MUL(wp[i - 1], w);
  }
  const int nq = order >= 2 ? 6 : (order >= 1 ? 3 : 1);
  double acc[6][3];
  for (int q = 0; q < 6; ++q) acc[q][0] = acc[q][1] = acc[q][2] = 0.0;
  for (int s = 0; s < 12; ++s) {
    /* control point s */
    double Q0, Q1, Q2;
    if (T == 0) {
      const double* x = pt->base + 3 * (size_t)pt->ids[(size_t)SHL_STAMSLOT[s] * pt->stride];
      Q0 = x[0];
      Q1 = x[1];
      Q2 = x[2];
    } else {
      Q0 = Q1 = Q2 = 0.0;
      for (int j = 0; j < np; ++j) {
        const double t = T[s * np + j];
        if (t == 0.0) continue;
        const double* x = pt->base + 3 * (size_t)pt->ids[(size_t)j * pt->stride];
        Q0 = SHL_FMA(t, x[0], Q0);
        Q1 = SHL_FMA(t, x[1], Q1);
        Q2 = SHL_FMA(t, x[2], Q2);
      }
    }
    /* box spline s and its derivatives, times 12 */
    double bs[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
    for (int m = 0; m < 15; ++m) {
      const int c = SHL_BOXC[s][m];
      if (c == 0) continue;
      const int p = SHL_BOXP[m], q = SHL_BOXQ[m];
      bs[0] = SHL_FMA((double)c, SHL_MUL(vp[p], wp[q]), bs[0]);
      if (nq > 1) {
        if (p >= 1) bs[1] = SHL_FMA((double)(c * p), SHL_MUL(vp[p - 1], wp[q]), bs[1]);
        if (q >= 1) bs[2] = SHL_FMA((double)(c * q), SHL_MUL(vp[p], wp[q - 1]), bs[2]);
      }
      if (nq > 3) {
        if (p >= 2) bs[3] = SHL_FMA((double)(c * p * (p - 1)), SHL_MUL(vp[p - 2], wp[q]), bs[3]);
        if (q >= 2) bs[4] = SHL_FMA((double)(c * q * (q - 1)), SHL_MUL(vp[p], wp[q - 2]), bs[4]);
        if (p >= 1 && q >= 1) bs[5] = SHL_FMA((double)(c * p * q), SHL_MUL(vp[p - 1], wp[q - 1]), bs[5]);
      }
    }
    for (int q = 0; q < nq; ++q) {
      acc[q][0] = SHL_FMA(bs[q], Q0, acc[q][0]);
      acc[q][1] = SHL_FMA(bs[q], Q1, acc[q][1]);
      acc[q][2] = SHL_FMA(bs[q], Q2, acc[q][2]);
    }
  }
  const double twelfth = 1.0 / 12.0;
  for (int q = 0; q < nq; ++q) {
    const double sc = q == 0 ? twelfth : (q < 3 ? SHL_MUL(j1, twelfth) : SHL_MUL(SHL_MUL(j1, j1), twelfth));
    for (int c = 0; c < 3; ++c) out[q][c] = SHL_MUL(acc[q][c], sc);
  }
}

/* ---- closest points of two limit patches -------------------------------- */

/* apply_constraints (SmoothShellShellContact.C:155-179) */
SHL_HD void shl_smooth_apply_constraints(double* x)
{
  const double eps = 2.220446049250313e-16;
  for (int i = 0; i < 4; ++i) x[i] = fmax(x[i], 0.0);
  for (int t = 0; t < 2; ++t) {
    const double u = SHL_SUB(SHL_SUB(1.0, x[2 * t]), x[2 * t + 1]);
    if (u < 0.0) {
      if (x[2 * t] > x[2 * t + 1])
        x[2 * t] = SHL_ADD(x[2 * t], SHL_SUB(u, eps));
      else
        x[2 * t + 1] = SHL_ADD(x[2 * t + 1], SHL_SUB(u, eps));
    }
  }
}

/* update_constraint_bitmap (SmoothShellShellContact.C:139-152): bit 0..3
 * x_i at 0, bit 4 / 5 v + w at 1 for the first / second element. */
SHL_HD unsigned shl_smooth_bitmap(const double* x)
{
  const double tol = SHL_SMOOTH_CONSTRAINT_TOL;
  unsigned bm = 0;
  for (int i = 0; i < 4; ++i)
    if (x[i] < tol) bm |= 1u << i;
  if (SHL_ADD(x[0], x[1]) > SHL_SUB(1.0, tol)) bm |= 1u << 4;
  if (SHL_ADD(x[2], x[3]) > SHL_SUB(1.0, tol)) bm |= 1u << 5;
  return bm;
}

/* find_max_alpha (SmoothShellShellContact.C:96-136); SHL_DBL_MAX when no
 * constraint limits the step. */
SHL_HD double shl_smooth_max_alpha(const double* x, const double* d)
{
  double a = SHL_DBL_MAX;
  for (int i = 0; i < 4; ++i)
    if (d[i] < 0.0) a = fmin(a, SHL_DIV(-x[i], d[i]));
  for (int t = 0; t < 2; ++t) {
    const double ds = SHL_ADD(d[2 * t], d[2 * t + 1]);
    if (ds > 0.0) a = fmin(a, SHL_DIV(SHL_SUB(SHL_SUB(1.0, x[2 * t]), x[2 * t + 1]), ds));
  }
  return a;
}

/* Working constraints of one element from its active constraints and the
 * gradient (gv, gw): kept where the first-order multiplier is non-negative.
 * Bits: 1 v = 0, 2 w = 0, 4 v + w = 1. */
SHL_HD unsigned shl_smooth_working(unsigned act, double gv, double gw)
{
  const unsigned V = 1, W = 2, S = 4;
  /* single-constraint multipliers (up to a positive factor) */
  const double lv = gv, lw = gw, ls = -SHL_ADD(gv, gw);
  if (act == (V | W)) {
    if (lv >= 0.0 && lw >= 0.0) return V | W;
    if (lv >= 0.0) return V;
    if (lw >= 0.0) return W;
    return 0;
  }
  if (act == (V | S)) {  /* vertex (0, 1): g = lam_v (1,0) + lam_s (-1,-1) */
    const double lam_v = SHL_SUB(gv, gw), lam_s = -gw;
    if (lam_v >= 0.0 && lam_s >= 0.0) return V | S;
    if (lam_v >= 0.0) return lv >= 0.0 ? V : 0;
    if (lam_s >= 0.0) return ls >= 0.0 ? S : 0;
    return 0;
  }
  if (act == (W | S)) {  /* vertex (1, 0): g = lam_w (0,1) + lam_s (-1,-1) */
    const double lam_w = SHL_SUB(gw, gv), lam_s = -gv;
    if (lam_w >= 0.0 && lam_s >= 0.0) return W | S;
    if (lam_w >= 0.0) return lw >= 0.0 ? W : 0;
    if (lam_s >= 0.0) return ls >= 0.0 ? S : 0;
    return 0;
  }
  if (act == V) return lv >= 0.0 ? V : 0;
  if (act == W) return lw >= 0.0 ? W : 0;
  if (act == S) return ls >= 0.0 ? S : 0;
  return 0;
}

/* f, gradient and Hessian of |p2 - p1|^2 at x; p1, p2 the limit points. */
SHL_HD double shl_smooth_fgh(const shl_limit_patch* A, const shl_limit_patch* B, const double* x, double* g,
                             double H[4][4], double* p1, double* p2)
{
  double e1[6][3], e2[6][3];
  shl_limit_eval(A, x[0], x[1], 2, e1);
  shl_limit_eval(B, x[2], x[3], 2, e2);
  double r[3], ri[4][3];
  for (int c = 0; c < 3; ++c) {
    r[c] = SHL_SUB(e2[0][c], e1[0][c]);
    ri[0][c] = -e1[1][c];
    ri[1][c] = -e1[2][c];
    ri[2][c] = e2[1][c];
    ri[3][c] = e2[2][c];
    p1[c] = e1[0][c];
    p2[c] = e2[0][c];
  }
  for (int i = 0; i < 4; ++i) g[i] = SHL_MUL(2.0, shl_v3_dot(r, ri[i]));
  /* second derivatives of r: -p1_ij within element 1, p2_ij within element 2 */
  const double r00 = -shl_v3_dot(r, e1[3]), r11 = -shl_v3_dot(r, e1[4]), r01 = -shl_v3_dot(r, e1[5]);
  const double r22 = shl_v3_dot(r, e2[3]), r33 = shl_v3_dot(r, e2[4]), r23 = shl_v3_dot(r, e2[5]);
  for (int i = 0; i < 4; ++i)
    for (int j = i; j < 4; ++j) {
      double h = shl_v3_dot(ri[i], ri[j]);
      if (i == 0 && j == 0) h = SHL_ADD(h, r00);
      if (i == 1 && j == 1) h = SHL_ADD(h, r11);
      if (i == 0 && j == 1) h = SHL_ADD(h, r01);
      if (i == 2 && j == 2) h = SHL_ADD(h, r22);
      if (i == 3 && j == 3) h = SHL_ADD(h, r33);
      if (i == 2 && j == 3) h = SHL_ADD(h, r23);
      H[i][j] = SHL_MUL(2.0, h);
      H[j][i] = H[i][j];
    }
  return shl_v3_dot(r, r);
}

/* f only (positions) */
SHL_HD double shl_smooth_f(const shl_limit_patch* A, const shl_limit_patch* B, const double* x, double* p1,
                           double* p2)
{
  double e1[6][3], e2[6][3];
  shl_limit_eval(A, x[0], x[1], 0, e1);
  shl_limit_eval(B, x[2], x[3], 0, e2);
  double r[3];
  for (int c = 0; c < 3; ++c) {
    r[c] = SHL_SUB(e2[0][c], e1[0][c]);
    p1[c] = e1[0][c];
    p2[c] = e2[0][c];
  }
  return shl_v3_dot(r, r);
}

/* Newton direction on the free subspace of the working set (Z columns), the
 * reduced Hessian shifted by mu I until its Cholesky factorisation succeeds.
 * Returns 1 when a shift was needed (f is not convex on the free subspace). */
SHL_HD int shl_smooth_direction(const double* g, double H[4][4], const unsigned* work, double* d)
{
  double Z[4][4];
  int m = 0;
  for (int t = 0; t < 2; ++t) {
    const unsigned wk = work[t];
    double z0[4] = {0, 0, 0, 0}, z1[4] = {0, 0, 0, 0};
    int nz = 0;
    if (wk == 0) {
      z0[2 * t] = 1.0;
      z1[2 * t + 1] = 1.0;
      nz = 2;
    } else if (wk == 1u) {  /* v = 0: w free */
      z0[2 * t + 1] = 1.0;
      nz = 1;
    } else if (wk == 2u) {  /* w = 0: v free */
      z0[2 * t] = 1.0;
      nz = 1;
    } else if (wk == 4u) {  /* v + w = 1: along (1, -1) */
      z0[2 * t] = 1.0;
      z0[2 * t + 1] = -1.0;
      nz = 1;
    }
    if (nz >= 1) {
      for (int i = 0; i < 4; ++i) Z[m][i] = z0[i];
      ++m;
    }
    if (nz == 2) {
      for (int i = 0; i < 4; ++i) Z[m][i] = z1[i];
      ++m;
    }
  }
  for (int i = 0; i < 4; ++i) d[i] = 0.0;
  if (m == 0) return 0;
  double Hr[4][4], gr[4], HZ[4][4];
  for (int a = 0; a < m; ++a) {
    double s = 0.0;
    for (int i = 0; i < 4; ++i) s = SHL_ADD(s, SHL_MUL(Z[a][i], g[i]));
    gr[a] = s;
    for (int i = 0; i < 4; ++i) {
      double t = 0.0;
      for (int j = 0; j < 4; ++j) t = SHL_ADD(t, SHL_MUL(H[i][j], Z[a][j]));
      HZ[a][i] = t;
    }
  }
  for (int a = 0; a < m; ++a)
    for (int b = 0; b < m; ++b) {
      double s = 0.0;
      for (int i = 0; i < 4; ++i) s = SHL_ADD(s, SHL_MUL(Z[a][i], HZ[b][i]));
      Hr[a][b] = s;
    }
  /* Jacobi scaling: the free directions can differ in scale by many orders
   * (the limit surface's parametric derivatives grow like 2^n next to an
   * irregular vertex), so the system is solved for the unit-diagonal matrix
   * S Hr S, S = diag(|Hr_aa|^-1/2), and the shift mu is relative to 1 */
  double S[4];
  for (int a = 0; a < m; ++a) {
    const double h = fabs(Hr[a][a]);
    S[a] = h > 0.0 ? SHL_DIV(1.0, SHL_SQRT(h)) : 1.0;
  }
  for (int a = 0; a < m; ++a) {
    gr[a] = SHL_MUL(S[a], gr[a]);
    for (int b = 0; b < m; ++b) Hr[a][b] = SHL_MUL(SHL_MUL(S[a], Hr[a][b]), S[b]);
  }
  double mu = 0.0, L[4][4], y[4];
  for (int attempt = 0; attempt < 24; ++attempt) {
    bool ok = true;
    for (int a = 0; a < m && ok; ++a)
      for (int b = 0; b <= a; ++b) {
        double s = Hr[a][b];
        if (a == b) s = SHL_ADD(s, mu);
        for (int k = 0; k < b; ++k) s = SHL_SUB(s, SHL_MUL(L[a][k], L[b][k]));
        if (a == b) {
          if (!(s > 1e-14)) { ok = false; break; }
          L[a][a] = SHL_SQRT(s);
        } else {
          L[a][b] = SHL_DIV(s, L[b][b]);
        }
      }
    if (ok) {
      for (int a = 0; a < m; ++a) {  /* L z = -gr */
        double s = -gr[a];
        for (int k = 0; k < a; ++k) s = SHL_SUB(s, SHL_MUL(L[a][k], y[k]));
        y[a] = SHL_DIV(s, L[a][a]);
      }
      for (int a = m - 1; a >= 0; --a) {  /* L^T y = z */
        double s = y[a];
        for (int k = a + 1; k < m; ++k) s = SHL_SUB(s, SHL_MUL(L[k][a], y[k]));
        y[a] = SHL_DIV(s, L[a][a]);
      }
      for (int i = 0; i < 4; ++i) {
        double s = 0.0;
        for (int a = 0; a < m; ++a) s = SHL_ADD(s, SHL_MUL(Z[a][i], SHL_MUL(S[a], y[a])));
        d[i] = s;
      }
      return mu > 0.0 ? 1 : 0;
    }
    mu = mu == 0.0 ? 1e-10 : SHL_MUL(mu, 10.0);
  }
  /* not reached for finite input: scaled projected steepest descent */
  for (int i = 0; i < 4; ++i) {
    double s = 0.0;
    for (int a = 0; a < m; ++a) s = SHL_ADD(s, SHL_MUL(Z[a][i], SHL_MUL(S[a], -gr[a])));
    d[i] = s;
  }
  return 1;
}

/* Closest points of the limit patches A (element 1) and B (element 2).
 * x = (v1, w1, v2, w2): in the start point, out the minimiser.  Returns the
 * iterations taken; d2 = |p2 - p1|^2, dc = p2 - p1 (ShellShellContact's dc). */
SHL_HD int shl_smooth_closest(const shl_limit_patch* A, const shl_limit_patch* B, double* x, double* d2,
                              double* dc)
{
  shl_smooth_apply_constraints(x);
  double p1[3], p2[3], g[4], H[4][4];
  double f = shl_smooth_fgh(A, B, x, g, H, p1, p2);
  int it = 0;
  for (; it < SHL_SMOOTH_MAX_IT; ++it) {
    const unsigned bm = shl_smooth_bitmap(x);
    unsigned act[2], work[2];
    for (int t = 0; t < 2; ++t) {
      act[t] = ((bm >> (2 * t)) & 1u) | (((bm >> (2 * t + 1)) & 1u) << 1) | (((bm >> (4 + t)) & 1u) << 2);
      work[t] = shl_smooth_working(act[t], g[2 * t], g[2 * t + 1]);
    }
    /* first-order optimality on the working set (the KKT conditions of the
     * constrained minimum, the multipliers' signs being the working set's
     * condition): the projected gradient vanishes to 1e-9 of the gradient */
    {
      double pg = 0.0, gn = 0.0;
      for (int t = 0; t < 2; ++t) {
        const double gv = g[2 * t], gw = g[2 * t + 1];
        gn = fmax(gn, fmax(fabs(gv), fabs(gw)));
        if (work[t] == 0u) pg = fmax(pg, fmax(fabs(gv), fabs(gw)));
        else if (work[t] == 1u) pg = fmax(pg, fabs(gw));
        else if (work[t] == 2u) pg = fmax(pg, fabs(gv));
        else if (work[t] == 4u) pg = fmax(pg, SHL_MUL(0.5, fabs(SHL_SUB(gv, gw))));
      }
      if (pg <= SHL_MUL(SHL_SMOOTH_KKT_TOL, gn)) break;
    }
    double d[4];
    int shifted = 0;
    /* each round adds at least one of the (at most four) active constraints */
    for (int round = 0; round < 6; ++round) {
      shifted = shl_smooth_direction(g, H, work, d);
      /* an active constraint left out of the working set must not be violated */
      bool grown = false;
      for (int t = 0; t < 2; ++t) {
        const unsigned freed = act[t] & ~work[t];
        unsigned add = 0;
        if ((freed & 1u) && d[2 * t] < 0.0) add |= 1u;
        if ((freed & 2u) && d[2 * t + 1] < 0.0) add |= 2u;
        if ((freed & 4u) && SHL_ADD(d[2 * t], d[2 * t + 1]) > 0.0) add |= 4u;
        if (add) {
          work[t] |= add;
          grown = true;
        }
      }
      if (!grown) break;
    }
    double dn = 0.0, gd = 0.0;
    for (int i = 0; i < 4; ++i) {
      dn = fmax(dn, fabs(d[i]));
      gd = SHL_ADD(gd, SHL_MUL(g[i], d[i]));
    }
#ifdef SHL_SMOOTH_TRACE
    SHL_SMOOTH_TRACE(it, x, f, g, d, work);
#endif
    /* converged: the model decrease along the step (-g.d, the Newton
     * decrement) is below 1e-15 of f, the precision of f itself */
    if (!(dn > 0.0) || !(gd < 0.0) || -gd <= SHL_MUL(SHL_SMOOTH_DECREMENT_TOL, f)) break;
    const double amax = shl_smooth_max_alpha(x, d);
    /* a Newton step where f is convex on the free subspace; otherwise the step
     * to the boundary first (along a direction of negative curvature f keeps
     * falling), backtracked */
    double alpha = (shifted || amax < 1.0) ? amax : 1.0;
    if (!(alpha > 0.0)) break;
    bool accepted = false;
    double xt[4], q1[3], q2[3], ft = 0.0;
    for (int ls = 0; ls < SHL_SMOOTH_MAX_HALVINGS; ++ls) {
      for (int i = 0; i < 4; ++i) xt[i] = SHL_ADD(x[i], SHL_MUL(alpha, d[i]));
      shl_smooth_apply_constraints(xt);
      ft = shl_smooth_f(A, B, xt, q1, q2);
      if (ft <= SHL_ADD(f, SHL_MUL(SHL_MUL(1e-4, alpha), gd))) {
        accepted = true;
        break;
      }
      /* after a rejected step to the boundary along a direction of negative
       * curvature, go on from a step of length 0.05 (triangle units) */
      const double a_half = SHL_MUL(alpha, 0.5);
      alpha = (ls == 0 && shifted) ? fmin(a_half, SHL_DIV(0.05, dn)) : a_half;
    }
    if (!accepted) break;
    double step = 0.0;
    for (int i = 0; i < 4; ++i) {
      step = fmax(step, fabs(SHL_SUB(xt[i], x[i])));
      x[i] = xt[i];
    }
    /* done after a vanishing step, or after a full Newton step of a convex
     * model that was already short: the next one would be of its square */
    const int full_newton = !shifted && alpha == 1.0;
    if (step <= SHL_SMOOTH_STEP_TOL || (full_newton && step <= SHL_SMOOTH_QUAD_TOL)) {
      f = ft;
      for (int c = 0; c < 3; ++c) {
        p1[c] = q1[c];
        p2[c] = q2[c];
      }
      ++it;
      break;
    }
    f = shl_smooth_fgh(A, B, x, g, H, p1, p2);
  }
  *d2 = f;
  for (int c = 0; c < 3; ++c) dc[c] = SHL_SUB(p2[c], p1[c]);
  return it;
}

#endif /* SHL_SMOOTH_H_ */
