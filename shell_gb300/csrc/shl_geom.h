/*
 * shl_geom.h -- contact geometry shared bit-for-bit by the CUDA kernels and the
 * host code (library set-up and the CPU oracle).
 *
 * The self-contact candidate list of the shell solver is decided by comparing
 * FP64 squared distances against a threshold (ShellSystem.C:2082, 2020).  For
 * the GPU list to be identical to the CPU list, every operation on that path
 * is rounded separately: on the device through __dmul_rn/__dadd_rn/__dsub_rn
 * (which the compiler never fuses into an FMA), on the host through plain
 * operators in translation units built with -ffp-contract=off.  Division and
 * square root are IEEE round-to-nearest on both sides.
 *
 * Contents
 *  - the distance routines of shl_distance.h (segment/segment and
 *    point/triangle closest points, in place of the reference's missing
 *    Contact.C);
 *  - shl_pair_compute(): ShellShellContact::compute() (ShellShellContact.C:35-57,
 *    89-145): minimum over 9 edge-edge and 6 vertex-face tests, edge tests
 *    first, strict '<' updates, dc from element 1 to element 2.
 *  - shl_friction_apply(): Margolis slip-stick law, Friction.C:4-60.
 *  - shl_fixed_order_sum(): the summation order used for avg_elem_size
 *    (ShellSystem.C:2572, 2584), which feeds the linked-cell size and therefore
 *    the candidate list; the reference leaves the order to OpenMP, here it is
 *    fixed so host and device agree exactly.
 */
#ifndef SHL_GEOM_H_
#define SHL_GEOM_H_

#include "shl_distance.h"

/* ---- one contact pair: ShellShellContact::compute() ----------------------- */
typedef struct shl_pair_geom {
  double d2;      /* squared minimum distance */
  double dc[3];   /* contact vector, element 1 -> element 2 */
  double v[2], w[2];  /* barycentric coordinates on elements 1 and 2 */
} shl_pair_geom;

/* p1[k], p2[k]: vertex k of element 1 / element 2 (3 doubles each). */
SHL_HD void shl_pair_compute(const double* const* p1, const double* const* p2, shl_pair_geom* g)
{
  g->d2 = SHL_DBL_MAX;
  g->dc[0] = g->dc[1] = g->dc[2] = 0.0;
  g->v[0] = g->v[1] = g->w[0] = g->w[1] = 0.0;
  /* edge-edge: edge i of element 1 runs from node i to node (i+1)%3 */
  for (int i = 0; i < 3; ++i) {
    const int i1 = (i == 2) ? 0 : i + 1;
    for (int j = 0; j < 3; ++j) {
      const int j1 = (j == 2) ? 0 : j + 1;
      double dc[3], st[2];
      shl_segment_segment(p1[i], p1[i1], p2[j], p2[j1], dc, st);
      const double d2 = shl_v3_dot(dc, dc);
      if (d2 < g->d2) {
        g->d2 = d2;
        g->dc[0] = dc[0]; g->dc[1] = dc[1]; g->dc[2] = dc[2];
        const double s0 = st[0], s1 = st[1];
        g->v[0] = (i == 0) ? s0 : ((i == 1) ? SHL_SUB(1.0, s0) : 0.0);
        g->w[0] = (i == 1) ? s0 : ((i == 2) ? SHL_SUB(1.0, s0) : 0.0);
        g->v[1] = (j == 0) ? s1 : ((j == 1) ? SHL_SUB(1.0, s1) : 0.0);
        g->w[1] = (j == 1) ? s1 : ((j == 2) ? SHL_SUB(1.0, s1) : 0.0);
      }
    }
  }
  /* vertex-face: vertex j of one element against the face of the other */
  for (int i = 0; i < 2; ++i) {
    const double* const* pv = (i == 0) ? p1 : p2;
    const double* const* pf = (i == 0) ? p2 : p1;
    for (int j = 0; j < 3; ++j) {
      double dc[3], vw[2];
      shl_point_triangle(pv[j], pf[0], pf[1], pf[2], dc, vw);
      const double d2 = shl_v3_dot(dc, dc);
      if (d2 < g->d2) {
        g->d2 = d2;
        if (i == 0) { g->dc[0] = dc[0]; g->dc[1] = dc[1]; g->dc[2] = dc[2]; }
        else { g->dc[0] = -dc[0]; g->dc[1] = -dc[1]; g->dc[2] = -dc[2]; }
        const double jv = (j == 1) ? 1.0 : 0.0, jw = (j == 2) ? 1.0 : 0.0;
        g->v[0] = (i == 0) ? jv : vw[0];
        g->w[0] = (i == 0) ? jw : vw[1];
        g->v[1] = (i == 1) ? jv : vw[0];
        g->w[1] = (i == 1) ? jw : vw[1];
      }
    }
  }
}

/* ---- Margolis slip-stick friction, Friction.C:4-60 ------------------------ */
/* Inputs as in Friction::apply; f_contact is both in (zero from the caller)
 * and out; stick/spring_origin are the persistent per-contact state. */
SHL_HD void shl_friction_apply(double* Efric, double* f_contact, double f_normal,
                               const double* n, const double* v, double abs_v_normal,
                               double v_stop, double k, double mu_s, double mu_d,
                               double damping, int* stick, double* spring_origin,
                               const double* contact_point)
{
  double vt[3];
  for (int c = 0; c < 3; ++c) vt[c] = SHL_SUB(v[c], SHL_MUL(abs_v_normal, n[c]));
  const double abs_vt = SHL_SQRT(shl_v3_dot(vt, vt));
  const double v_eps = SHL_MUL(1e-8, v_stop);
  if (mu_s > 0.0 && abs_vt <= v_stop) {
    if (!*stick) {
      *stick = 1;
      const double pre = SHL_SUB(SHL_DIV(SHL_MUL(mu_d, f_normal), SHL_MUL(k, SHL_ADD(abs_vt, v_eps))), damping);
      for (int c = 0; c < 3; ++c) spring_origin[c] = SHL_SUB(contact_point[c], SHL_MUL(pre, vt[c]));
    }
    double us[3];
    shl_v3_sub(contact_point, spring_origin, us);
    const double un = shl_v3_dot(us, n);
    for (int c = 0; c < 3; ++c) us[c] = SHL_SUB(us[c], SHL_MUL(un, n[c]));
    *Efric = SHL_MUL(SHL_MUL(0.5, k), shl_v3_dot(us, us));
    const double dk = SHL_MUL(damping, k);
    for (int c = 0; c < 3; ++c) {
      f_contact[c] = SHL_MUL(-k, us[c]);
      f_contact[c] = SHL_SUB(f_contact[c], SHL_MUL(dk, vt[c]));
    }
  }
  const double fs = SHL_MUL(mu_s, f_normal);
  if (abs_vt > v_stop || shl_v3_dot(f_contact, f_contact) >= SHL_MUL(fs, fs)) {
    spring_origin[0] = spring_origin[1] = spring_origin[2] = 0.0;
    *stick = 0;
    *Efric = 0.0;
    const double pre = SHL_DIV(SHL_MUL(-mu_d, f_normal), SHL_ADD(abs_vt, v_eps));
    for (int c = 0; c < 3; ++c) f_contact[c] = SHL_MUL(pre, vt[c]);
  }
}

/* ---- fixed-order sum -------------------------------------------------------
 * SHL_SUM_LANES partial sums, lane l adding x[l], x[l+LANES], ... in index
 * order; the lanes are then combined by a pairwise tree (stride LANES/2, /4,
 * ..., 1).  The CUDA reduction kernel uses one block of SHL_SUM_LANES threads
 * and performs exactly these additions. */
#define SHL_SUM_LANES 1024

/* host version (the device version lives in the AABB kernel) */
static inline double shl_fixed_order_sum(const double* x, unsigned n)
{
  double lane[SHL_SUM_LANES];
  for (unsigned l = 0; l < SHL_SUM_LANES; ++l) {
    double s = 0.0;
    for (unsigned i = l; i < n; i += SHL_SUM_LANES) s = SHL_ADD(s, x[i]);
    lane[l] = s;
  }
  for (unsigned stride = SHL_SUM_LANES / 2; stride > 0; stride /= 2)
    for (unsigned l = 0; l < stride; ++l) lane[l] = SHL_ADD(lane[l], lane[l + stride]);
  return lane[0];
}

#endif /* SHL_GEOM_H_ */
