/*
 * shl_distance.h -- closest points of segments and triangles, shared bit for
 * bit by the CUDA kernels and the host code (library set-up and the CPU
 * oracle).
 *
 * These are the two distance routines that the reference declares but whose
 * source is missing (Contact.h:22-34; Contact.C is not in the reference).
 * Their semantics are fixed by the call sites in ShellShellContact.C:
 *  - shl_segment_segment(): closest points of two segments; st[0] is the
 *    parameter along p10->p11, st[1] along p20->p21, diffvec points from the
 *    point on segment 1 to the point on segment 2 (ShellShellContact.C:98-111).
 *  - shl_point_triangle(): closest point of a triangle to a point; the closest
 *    point is (1-v-w)p1 + v p2 + w p3, diffvec points from p0 to it
 *    (ShellShellContact.C:128-141).
 * The constructions follow the standard Voronoi-region method for
 * point/triangle and the clamped-parameter method for segment/segment
 * (C. Ericson, Real-Time Collision Detection, 2005, sections 5.1.5 and 5.1.9).
 *
 * Every operation is rounded on its own: on the device through
 * __dmul_rn/__dadd_rn/__dsub_rn (which the compiler never fuses into an FMA),
 * on the host through plain operators in translation units built with
 * -ffp-contract=off.  Division and square root are IEEE round-to-nearest on
 * both sides.
 */
#ifndef SHL_DISTANCE_H_
#define SHL_DISTANCE_H_

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

#endif /* SHL_DISTANCE_H_ */
