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
 *  - shl_segment_segment(): closest points of two segments.  Replaces the
 *    declared-but-missing Contact::segment_segment_distance (Contact.h:22-27);
 *    semantics fixed by its call site ShellShellContact.C:98-111: st[0] is the
 *    parameter along p10->p11, st[1] along p20->p21, diffvec points from the
 *    point on segment 1 to the point on segment 2.
 *  - shl_point_triangle(): closest point of a triangle to a point.  Replaces
 *    Contact::point_triangle_distance (Contact.h:29-34); semantics from
 *    ShellShellContact.C:128-141: the closest point is (1-v-w)p1 + v p2 + w p3,
 *    diffvec points from p0 to it.
 *  - shl_pair_compute(): ShellShellContact::compute() (ShellShellContact.C:35-57,
 *    89-145): minimum over 9 edge-edge and 6 vertex-face tests, edge tests
 *    first, strict '<' updates, dc from element 1 to element 2.
 *  - shl_friction_apply(): Margolis slip-stick law, Friction.C:4-60.
 *  - shl_fixed_order_sum(): the summation order used for avg_elem_size
 *    (ShellSystem.C:2572, 2584), which feeds the linked-cell size and therefore
 *    the candidate list; the reference leaves the order to OpenMP, here it is
 *    fixed so host and device agree exactly.
 *
 * The closest-point constructions follow the standard Voronoi-region method
 * for point/triangle and the clamped-parameter method for segment/segment
 * (C. Ericson, Real-Time Collision Detection, 2005, sections 5.1.5 and 5.1.9).
 */
#ifndef SHL_GEOM_H_
#define SHL_GEOM_H_

#ifdef __CUDACC__
#define SHL_HD __host__ __device__ __forceinline__
#else
#define SHL_HD static inline
#endif

#ifdef __CUDA_ARCH__
#define SHL_MUL(a, b) __dmul_rn((a), (b))
#define SHL_ADD(a, b) __dadd_rn((a), (b))
#define SHL_SUB(a, b) __dsub_rn((a), (b))
#define SHL_DIV(a, b) __ddiv_rn((a), (b))
#define SHL_SQRT(a) __dsqrt_rn(a)
#else
#include <math.h>
#define SHL_MUL(a, b) ((a) * (b))
#define SHL_ADD(a, b) ((a) + (b))
#define SHL_SUB(a, b) ((a) - (b))
#define SHL_DIV(a, b) ((a) / (b))
#define SHL_SQRT(a) sqrt(a)
#endif

#define SHL_DBL_MAX 1.7976931348623157e308

/* ---- 3-vector helpers, each operation rounded on its own ---------------- */

SHL_HD void shl_v3_sub(const double* a, const double* b, double* r)
{
  r[0] = SHL_SUB(a[0], b[0]);
  r[1] = SHL_SUB(a[1], b[1]);
  r[2] = SHL_SUB(a[2], b[2]);
}

SHL_HD double shl_v3_dot(const double* a, const double* b)
{
  return SHL_ADD(SHL_ADD(SHL_MUL(a[0], b[0]), SHL_MUL(a[1], b[1])), SHL_MUL(a[2], b[2]));
}

/* r = a + s*b */
SHL_HD void shl_v3_axpy(const double* a, double s, const double* b, double* r)
{
  r[0] = SHL_ADD(a[0], SHL_MUL(s, b[0]));
  r[1] = SHL_ADD(a[1], SHL_MUL(s, b[1]));
  r[2] = SHL_ADD(a[2], SHL_MUL(s, b[2]));
}

SHL_HD double shl_clamp01(double x)
{
  return x < 0.0 ? 0.0 : (x > 1.0 ? 1.0 : x);
}

/* ---- closest points of segments [p10,p11] and [p20,p21] ------------------ */
SHL_HD void shl_segment_segment(const double* p10, const double* p11,
                                const double* p20, const double* p21,
                                double* diffvec, double* st)
{
  double d1[3], d2[3], r[3];
  shl_v3_sub(p11, p10, d1);
  shl_v3_sub(p21, p20, d2);
  shl_v3_sub(p10, p20, r);
  const double a = shl_v3_dot(d1, d1);
  const double e = shl_v3_dot(d2, d2);
  const double f = shl_v3_dot(d2, r);
  double s, t;
  if (a <= 0.0 && e <= 0.0) {
    s = 0.0;
    t = 0.0;
  } else if (a <= 0.0) {
    s = 0.0;
    t = shl_clamp01(SHL_DIV(f, e));
  } else {
    const double c = shl_v3_dot(d1, r);
    if (e <= 0.0) {
      t = 0.0;
      s = shl_clamp01(SHL_DIV(-c, a));
    } else {
      const double b = shl_v3_dot(d1, d2);
      const double denom = SHL_SUB(SHL_MUL(a, e), SHL_MUL(b, b));
      /* parallel segments: any s works, take the start of segment 1 */
      s = denom > 0.0 ? shl_clamp01(SHL_DIV(SHL_SUB(SHL_MUL(b, f), SHL_MUL(c, e)), denom)) : 0.0;
      const double tnom = SHL_ADD(SHL_MUL(b, s), f);
      if (tnom < 0.0) {
        t = 0.0;
        s = shl_clamp01(SHL_DIV(-c, a));
      } else if (tnom > e) {
        t = 1.0;
        s = shl_clamp01(SHL_DIV(SHL_SUB(b, c), a));
      } else {
        t = SHL_DIV(tnom, e);
      }
    }
  }
  double c1[3], c2[3];
  shl_v3_axpy(p10, s, d1, c1);
  shl_v3_axpy(p20, t, d2, c2);
  shl_v3_sub(c2, c1, diffvec);
  st[0] = s;
  st[1] = t;
}

/* ---- closest point of triangle (p1,p2,p3) to p0 -------------------------- */
SHL_HD void shl_point_triangle(const double* p0, const double* p1, const double* p2,
                               const double* p3, double* diffvec, double* vw)
{
  double ab[3], ac[3], ap[3];
  shl_v3_sub(p2, p1, ab);
  shl_v3_sub(p3, p1, ac);
  shl_v3_sub(p0, p1, ap);
  double v, w;
  const double d1 = shl_v3_dot(ab, ap);
  const double d2 = shl_v3_dot(ac, ap);
  double bp[3], cp[3];
  shl_v3_sub(p0, p2, bp);
  const double d3 = shl_v3_dot(ab, bp);
  const double d4 = shl_v3_dot(ac, bp);
  shl_v3_sub(p0, p3, cp);
  const double d5 = shl_v3_dot(ab, cp);
  const double d6 = shl_v3_dot(ac, cp);
  const double vc = SHL_SUB(SHL_MUL(d1, d4), SHL_MUL(d3, d2));
  const double vb = SHL_SUB(SHL_MUL(d5, d2), SHL_MUL(d1, d6));
  const double va = SHL_SUB(SHL_MUL(d3, d6), SHL_MUL(d5, d4));
  if (d1 <= 0.0 && d2 <= 0.0) {            /* vertex p1 */
    v = 0.0; w = 0.0;
  } else if (d3 >= 0.0 && d4 <= d3) {      /* vertex p2 */
    v = 1.0; w = 0.0;
  } else if (vc <= 0.0 && d1 >= 0.0 && d3 <= 0.0) {  /* edge p1-p2 */
    v = SHL_DIV(d1, SHL_SUB(d1, d3)); w = 0.0;
  } else if (d6 >= 0.0 && d5 <= d6) {      /* vertex p3 */
    v = 0.0; w = 1.0;
  } else if (vb <= 0.0 && d2 >= 0.0 && d6 <= 0.0) {  /* edge p1-p3 */
    v = 0.0; w = SHL_DIV(d2, SHL_SUB(d2, d6));
  } else if (va <= 0.0 && SHL_SUB(d4, d3) >= 0.0 && SHL_SUB(d5, d6) >= 0.0) {  /* edge p2-p3 */
    const double e43 = SHL_SUB(d4, d3);
    w = SHL_DIV(e43, SHL_ADD(e43, SHL_SUB(d5, d6)));
    v = SHL_SUB(1.0, w);
  } else {                                 /* interior */
    const double den = SHL_ADD(SHL_ADD(va, vb), vc);
    v = SHL_DIV(vb, den);
    w = SHL_DIV(vc, den);
  }
  const double u = SHL_SUB(SHL_SUB(1.0, v), w);
  double q[3];
  for (int k = 0; k < 3; ++k)
    q[k] = SHL_ADD(SHL_ADD(SHL_MUL(u, p1[k]), SHL_MUL(v, p2[k])), SHL_MUL(w, p3[k]));
  shl_v3_sub(q, p0, diffvec);
  vw[0] = v;
  vw[1] = w;
}

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
