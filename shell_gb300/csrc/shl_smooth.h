/*
 * shl_smooth.h -- the closest points of two Loop limit patches (SMOOTH
 * self-contact), on the limit evaluation of shl_limit.h.
 *
 * Reference behaviour (file:line):
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
 * shl_distance.h), so host and device agree bit for bit.
 */
#ifndef SHL_SMOOTH_H_
#define SHL_SMOOTH_H_

#include "shl_limit.h"

#define SHL_SMOOTH_MAX_IT 40
#define SHL_SMOOTH_CONSTRAINT_TOL (100 * 2.220446049250313e-16)
#define SHL_SMOOTH_STEP_TOL 1e-14
#define SHL_SMOOTH_DECREMENT_TOL 1e-15
#define SHL_SMOOTH_QUAD_TOL 1e-6
#define SHL_SMOOTH_KKT_TOL 1e-9
#define SHL_SMOOTH_MAX_HALVINGS 30

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

/* f, gradient and Hessian of |p2 - p1|^2 from the limit evaluations e1 (of
 * element 1 at (x0, x1)) and e2 (of element 2 at (x2, x3)), order 2; p1, p2
 * the limit points. */
SHL_HD double shl_smooth_fgh_from(const double e1[6][3], const double e2[6][3], double* g, double H[4][4],
                                  double* p1, double* p2)
{
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

/* f only, from order-0 evaluations */
SHL_HD double shl_smooth_f_from(const double e1[6][3], const double e2[6][3], double* p1, double* p2)
{
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
 * Returns 1 when a shift was needed (f is not convex on the free subspace).
 * The columns of Z are unit vectors e_k (a free coordinate) or e_k - e_(k+1)
 * (along an active edge v + w = 1), so the reduced gradient Z^T g and Hessian
 * Z^T H Z are single entries or differences: each is formed as the sum over
 * the four coordinates from zero would round it (the zero products add
 * nothing; a zero result is +0). */
SHL_HD int shl_smooth_direction(const double* g, double H[4][4], const unsigned* work, double* d)
{
  int zk[4], zd[4];  /* column a of Z: e_zk, minus e_(zk+1) when zd */
  int m = 0;
  for (int t = 0; t < 2; ++t) {
    const unsigned wk = work[t];
    if (wk == 0) {
      zk[m] = 2 * t;
      zd[m++] = 0;
      zk[m] = 2 * t + 1;
      zd[m++] = 0;
    } else if (wk == 1u) {  /* v = 0: w free */
      zk[m] = 2 * t + 1;
      zd[m++] = 0;
    } else if (wk == 2u) {  /* w = 0: v free */
      zk[m] = 2 * t;
      zd[m++] = 0;
    } else if (wk == 4u) {  /* v + w = 1: along (1, -1) */
      zk[m] = 2 * t;
      zd[m++] = 1;
    }
  }
  for (int i = 0; i < 4; ++i) d[i] = 0.0;
  if (m == 0) return 0;
  double Hr[4][4], gr[4], HZ[4][4];
  for (int a = 0; a < m; ++a) {
    const int k = zk[a];
    gr[a] = SHL_ADD(0.0, g[k]);
    if (zd[a]) gr[a] = SHL_SUB(gr[a], g[k + 1]);
    for (int i = 0; i < 4; ++i) {
      HZ[a][i] = SHL_ADD(0.0, H[i][k]);
      if (zd[a]) HZ[a][i] = SHL_SUB(HZ[a][i], H[i][k + 1]);
    }
  }
  for (int a = 0; a < m; ++a)
    for (int b = 0; b < m; ++b) {
      const int k = zk[a];
      Hr[a][b] = SHL_ADD(0.0, HZ[b][k]);
      if (zd[a]) Hr[a][b] = SHL_SUB(Hr[a][b], HZ[b][k + 1]);
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
      /* d = Z S y: each coordinate is one column's share (or +0) */
      for (int a = 0; a < m; ++a) {
        const double sy = SHL_MUL(S[a], y[a]);
        d[zk[a]] = SHL_ADD(0.0, sy);
        if (zd[a]) d[zk[a] + 1] = SHL_ADD(0.0, -sy);
      }
      return mu > 0.0 ? 1 : 0;
    }
    mu = mu == 0.0 ? 1e-10 : SHL_MUL(mu, 10.0);
  }
  /* not reached for finite input: scaled projected steepest descent */
  for (int a = 0; a < m; ++a) {
    const double sg = SHL_MUL(S[a], -gr[a]);
    d[zk[a]] = SHL_ADD(0.0, sg);
    if (zd[a]) d[zk[a] + 1] = SHL_ADD(0.0, -sg);
  }
  return 1;
}

/* The search as a resumable state: each step consumes one limit evaluation of
 * both patches (order 2 at x for f, g, H; order 0 at the line search's trial
 * point xt for f), so that threads searching for different pairs evaluate in
 * step.  shl_smooth_closest runs it to the end; every decision and every
 * operation is that of the loop the reference's minimiser would run. */
enum { SHL_SMOOTH_EVAL_FGH = 0, SHL_SMOOTH_EVAL_TRIAL = 1, SHL_SMOOTH_DONE = 2 };
typedef struct {
  double x[4], f, g[4], H[4][4], p1[3], p2[3];  /* the iterate and its evaluation */
  double d[4], dn, gd, alpha, xt[4];            /* the step and the line search's trial point */
  int it, ls, shifted, phase, after_accept;
} shl_smooth_state;

SHL_HD void shl_smooth_start(shl_smooth_state* s, const double* x0)
{
  for (int i = 0; i < 4; ++i) s->x[i] = x0[i];
  shl_smooth_apply_constraints(s->x);
  s->it = 0;
  s->ls = 0;
  s->shifted = 0;
  s->after_accept = 0;
  s->phase = SHL_SMOOTH_EVAL_FGH;
}

/* the point and the derivative order of the state's next evaluation */
SHL_HD const double* shl_smooth_point(const shl_smooth_state* s) { return s->phase == SHL_SMOOTH_EVAL_FGH ? s->x : s->xt; }
SHL_HD int shl_smooth_order(const shl_smooth_state* s) { return s->phase == SHL_SMOOTH_EVAL_FGH ? 2 : 0; }

/* the line search's trial point x + alpha d, projected */
SHL_HD void shl_smooth_trial(shl_smooth_state* s)
{
  for (int i = 0; i < 4; ++i) s->xt[i] = SHL_ADD(s->x[i], SHL_MUL(s->alpha, s->d[i]));
  shl_smooth_apply_constraints(s->xt);
}

/* a new iterate's evaluation is in: optimality test, Newton direction, first trial */
SHL_HD void shl_smooth_direction_step(shl_smooth_state* s)
{
  if (s->after_accept) ++s->it;
  if (!(s->it < SHL_SMOOTH_MAX_IT)) {
    s->phase = SHL_SMOOTH_DONE;
    return;
  }
  const double* g = s->g;
  const unsigned bm = shl_smooth_bitmap(s->x);
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
    if (pg <= SHL_MUL(SHL_SMOOTH_KKT_TOL, gn)) {
      s->phase = SHL_SMOOTH_DONE;
      return;
    }
  }
  double* d = s->d;
  int shifted = 0;
  /* each round adds at least one of the (at most four) active constraints */
  for (int round = 0; round < 6; ++round) {
    shifted = shl_smooth_direction(g, s->H, work, d);
    /* an active constraint left out of the working set must not be violated */
    int grown = 0;
    for (int t = 0; t < 2; ++t) {
      const unsigned freed = act[t] & ~work[t];
      unsigned add = 0;
      if ((freed & 1u) && d[2 * t] < 0.0) add |= 1u;
      if ((freed & 2u) && d[2 * t + 1] < 0.0) add |= 2u;
      if ((freed & 4u) && SHL_ADD(d[2 * t], d[2 * t + 1]) > 0.0) add |= 4u;
      if (add) {
        work[t] |= add;
        grown = 1;
      }
    }
    if (!grown) break;
  }
  double dn = 0.0, gd = 0.0;
  for (int i = 0; i < 4; ++i) {
    dn = fmax(dn, fabs(d[i]));
    gd = SHL_ADD(gd, SHL_MUL(g[i], d[i]));
  }
  /* converged: the model decrease along the step (-g.d, the Newton
   * decrement) is below 1e-15 of f, the precision of f itself */
  if (!(dn > 0.0) || !(gd < 0.0) || -gd <= SHL_MUL(SHL_SMOOTH_DECREMENT_TOL, s->f)) {
    s->phase = SHL_SMOOTH_DONE;
    return;
  }
  const double amax = shl_smooth_max_alpha(s->x, d);
  /* a Newton step where f is convex on the free subspace; otherwise the step
   * to the boundary first (along a direction of negative curvature f keeps
   * falling), backtracked */
  const double alpha = (shifted || amax < 1.0) ? amax : 1.0;
  if (!(alpha > 0.0)) {
    s->phase = SHL_SMOOTH_DONE;
    return;
  }
  s->shifted = shifted;
  s->dn = dn;
  s->gd = gd;
  s->alpha = alpha;
  s->ls = 0;
  shl_smooth_trial(s);
  s->phase = SHL_SMOOTH_EVAL_TRIAL;
}

/* Consumes the evaluations e1, e2 of the state's next point and advances. */
SHL_HD void shl_smooth_take(shl_smooth_state* s, const double e1[6][3], const double e2[6][3])
{
  if (s->phase == SHL_SMOOTH_EVAL_FGH) {
    s->f = shl_smooth_fgh_from(e1, e2, s->g, s->H, s->p1, s->p2);
    shl_smooth_direction_step(s);
    return;
  }
  double q1[3], q2[3];
  const double ft = shl_smooth_f_from(e1, e2, q1, q2);
  if (ft <= SHL_ADD(s->f, SHL_MUL(SHL_MUL(1e-4, s->alpha), s->gd))) {
    double step = 0.0;
    for (int i = 0; i < 4; ++i) {
      step = fmax(step, fabs(SHL_SUB(s->xt[i], s->x[i])));
      s->x[i] = s->xt[i];
    }
    /* done after a vanishing step, or after a full Newton step of a convex
     * model that was already short: the next one would be of its square */
    const int full_newton = !s->shifted && s->alpha == 1.0;
    if (step <= SHL_SMOOTH_STEP_TOL || (full_newton && step <= SHL_SMOOTH_QUAD_TOL)) {
      s->f = ft;
      for (int c = 0; c < 3; ++c) {
        s->p1[c] = q1[c];
        s->p2[c] = q2[c];
      }
      ++s->it;
      s->phase = SHL_SMOOTH_DONE;
      return;
    }
    s->after_accept = 1;
    s->phase = SHL_SMOOTH_EVAL_FGH;
    return;
  }
  /* after a rejected step to the boundary along a direction of negative
   * curvature, go on from a step of length 0.05 (triangle units) */
  const double a_half = SHL_MUL(s->alpha, 0.5);
  s->alpha = (s->ls == 0 && s->shifted) ? fmin(a_half, SHL_DIV(0.05, s->dn)) : a_half;
  if (++s->ls == SHL_SMOOTH_MAX_HALVINGS) {
    s->phase = SHL_SMOOTH_DONE;
    return;
  }
  shl_smooth_trial(s);
}

/* Closest points of the limit patches A (element 1) and B (element 2).
 * x = (v1, w1, v2, w2): in the start point, out the minimiser.  Returns the
 * iterations taken; d2 = |p2 - p1|^2, dc = p2 - p1 (ShellShellContact's dc). */
SHL_HD int shl_smooth_closest(const shl_limit_patch* A, const shl_limit_patch* B, double* x, double* d2,
                              double* dc)
{
  shl_smooth_state s;
  shl_smooth_start(&s, x);
  while (s.phase != SHL_SMOOTH_DONE) {
    const double* pt = shl_smooth_point(&s);
    const int order = shl_smooth_order(&s);
    double e1[6][3], e2[6][3];
    shl_limit_eval(A, pt[0], pt[1], order, e1);
    shl_limit_eval(B, pt[2], pt[3], order, e2);
    shl_smooth_take(&s, e1, e2);
  }
  for (int i = 0; i < 4; ++i) x[i] = s.x[i];
  *d2 = s.f;
  for (int c = 0; c < 3; ++c) dc[c] = SHL_SUB(s.p2[c], s.p1[c]);
  return s.it;
}

#endif /* SHL_SMOOTH_H_ */
