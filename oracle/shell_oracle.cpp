/*
 * shell_oracle.cpp -- CPU oracle for the explicit shell time step.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a libMesh-free FP64 restatement of the
 * reference's hot path, kept in the reference's own structure (per-element
 * caches of arrays-of-structs, OpenMP element loops with critical-section
 * assembly, a std::vector of contact candidates with NULL-slot reuse).  It is
 * loaded by the tests, by the smoke check and by the CPU-baseline leg of the
 * benchmark, never by the library.
 *
 * Parity status: the reference cannot be built (it needs an unpublished libMesh
 * fork and muparser, and Contact.C / ConstrainedMinimizer.h are missing), and it
 * ships no tests, golden vectors or fixtures apart from the two icosphere OFF
 * files.  Force and state parity is therefore UNPINNED against reference
 * outputs; it is pinned by known-answer tests instead (basis against
 * explicit Loop subdivision, rigid-motion invariance, energy gradient by
 * finite differences, brute-force contact pairs, the reference's own
 * Friction.C compiled beside it).
 *
 * Followed reference code (file:line):
 *   set_newmark_parameters ShellSystem.C:744-759, advance 952-1122,
 *   prepare_next_step 924-949, subtract_internal_force 1125-1314,
 *   compute_reference_metrics 1317-1379, compute_deformed_metrics 1382-1464,
 *   compute_external_force 1467-1585, add_shell_shell_contact_force 1792-1907,
 *   compute_shell_shell_contact_candidates 1910-2135, compute_position
 *   2484-2502, compute_enclosed_volume 2505-2541, compute_bounding_box
 *   2544-2587, check_increment 2591-2652, reset/measure_properties 2686-2846,
 *   update_derived 421-487, build_cache 490-681, build_topological_neighborhood
 *   684-741, compute_mass_damping 762-852, apply_initial_conditions 855-905,
 *   reinit_mod 3321-3499, ShellSystem::inverse ShellSystem.h:437-455,
 *   shell_shell_contact_force/energy ShellSystem.h:387-401,
 *   BoundingBox::apart BoundingBox.h:64-69.
 * The subdivision basis (libMesh FESubdivision, not in the reference) is
 * restated from the published method: Stam's box-spline form of Loop's
 * regular patch (J. Stam, "Evaluation of Loop subdivision surfaces",
 * SIGGRAPH'98 course notes) and one explicit Loop subdivision step with
 * Loop's vertex weight beta(N) = (5/8 - (3/8 + cos(2 pi/N)/4)^2)/N for the
 * irregular patch (the quadrature point (1/3,1/3) lies in the middle
 * sub-triangle after one step, as in SubdivEvaluation.C:170-187, 110-135).
 *
 * The narrow phase (ShellShellContact::compute, ShellShellContact.C:35-145),
 * the friction law (Friction::apply, Friction.C:4-60) and the SMOOTH
 * closest-point search (SmoothShellShellContact.C:16-204, with the minimiser
 * the reference does not ship restated as the library documents it) are
 * restated here on the oracle's own code, in the reference's order of
 * operations.  The only contact code shared with the library is
 * shl_distance.h: the two closest-point routines that the reference declares
 * but does not ship (Contact.h:22-34, Contact.C missing); for SMOOTH contact
 * the limit-surface evaluation (shl_limit.h, SubdivEvaluation.C:14-187) and its
 * subdivision tables (shl_subdiv.h, the reference's PAnArray) are shared too,
 * pinned by explicit Loop subdivision in the tests.
 *
 * Build with -ffp-contract=off: every multiply and add is rounded on its own,
 * as the device code does (__dmul_rn/__dadd_rn), so candidate lists agree bit
 * for bit.
 */
#include "oracle.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <limits>
#include <list>
#include <set>
#include <string>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

#include "../shell_gb300/csrc/shl_expr.h"
#include "../shell_gb300/csrc/shl_limit.h"
#include "../shell_gb300/csrc/shl_subdiv.h"
#include "../shell_gb300/csrc/shl_distance.h"
#ifdef SHL_GEOM_H_
#error "the oracle restates the narrow phase and friction; it must not compile the library's versions"
#endif

namespace {

thread_local std::string g_err;

typedef double Real;

struct Point {
  Real x[3];
  Point() { x[0] = x[1] = x[2] = 0; }
  Point(Real a, Real b, Real c) { x[0] = a; x[1] = b; x[2] = c; }
  Real& operator()(int i) { return x[i]; }
  Real operator()(int i) const { return x[i]; }
  Point operator+(const Point& o) const { return Point(x[0] + o.x[0], x[1] + o.x[1], x[2] + o.x[2]); }
  Point operator-(const Point& o) const { return Point(x[0] - o.x[0], x[1] - o.x[1], x[2] - o.x[2]); }
  Point operator-() const { return Point(-x[0], -x[1], -x[2]); }
  Point operator*(Real s) const { return Point(x[0] * s, x[1] * s, x[2] * s); }
  Point operator/(Real s) const { return Point(x[0] / s, x[1] / s, x[2] / s); }
  Real operator*(const Point& o) const { return x[0] * o.x[0] + x[1] * o.x[1] + x[2] * o.x[2]; }
  Point& operator+=(const Point& o) { x[0] += o.x[0]; x[1] += o.x[1]; x[2] += o.x[2]; return *this; }
  Point& operator-=(const Point& o) { x[0] -= o.x[0]; x[1] -= o.x[1]; x[2] -= o.x[2]; return *this; }
  Point& operator*=(Real s) { x[0] *= s; x[1] *= s; x[2] *= s; return *this; }
  void add_scaled(const Point& o, Real s) { x[0] += o.x[0] * s; x[1] += o.x[1] * s; x[2] += o.x[2] * s; }
  Point cross(const Point& o) const {
    return Point(x[1] * o.x[2] - x[2] * o.x[1], x[2] * o.x[0] - x[0] * o.x[2], x[0] * o.x[1] - x[1] * o.x[0]);
  }
  Real size_sq() const { return x[0] * x[0] + x[1] * x[1] + x[2] * x[2]; }
  Real size() const { return std::sqrt(size_sq()); }
  void zero() { x[0] = x[1] = x[2] = 0; }
};
inline Point operator*(Real s, const Point& p) { return p * s; }
static_assert(sizeof(Point) == 3 * sizeof(Real), "positions are read as packed xyz");

// ---- narrow phase: ShellShellContact::compute (ShellShellContact.C:35-57) ----
// d2, the contact vector dc (element 1 -> element 2) and the barycentric
// coordinates (v, w) of the closest points on both elements.
struct PairGeom {
  Real d2;
  Point dc;
  Real v[2], w[2];
};

// edge_edge_test (ShellShellContact.C:89-113): each edge of element 1 against
// each edge of element 2, edge i running from node i to node mod3[i]; a pair of
// edges replaces the current minimum only when strictly closer.
void edge_edge_test(const Point* const p[2][3], PairGeom& c) {
  static const unsigned int mod3[3] = {1, 2, 0};
  Real st[2];
  Point this_dc;
  for (unsigned int i = 0; i < 3; ++i) {
    for (unsigned int j = 0; j < 3; ++j) {
      shl_segment_segment(p[0][i]->x, p[0][mod3[i]]->x, p[1][j]->x, p[1][mod3[j]]->x, this_dc.x, st);
      const Real this_d2 = this_dc.size_sq();
      if (this_d2 < c.d2) {
        c.d2 = this_d2;
        c.dc = this_dc;
        c.v[0] = (i == 0) * st[0] + (i == 1) * (1 - st[0]);
        c.w[0] = (i == 1) * st[0] + (i == 2) * (1 - st[0]);
        c.v[1] = (j == 0) * st[1] + (j == 1) * (1 - st[1]);
        c.w[1] = (j == 1) * st[1] + (j == 2) * (1 - st[1]);
      }
    }
  }
}

// vertex_face_test (ShellShellContact.C:115-145): each vertex of each element
// against the face of the other; dc is turned to point from element 1 to 2.
void vertex_face_test(const Point* const p[2][3], PairGeom& c) {
  Real vw[2];
  Point this_dc;
  for (unsigned int i = 0; i < 2; ++i) {
    for (unsigned int j = 0; j < 3; ++j) {
      shl_point_triangle(p[i][j]->x, p[1 - i][0]->x, p[1 - i][1]->x, p[1 - i][2]->x, this_dc.x, vw);
      const Real this_d2 = this_dc.size_sq();
      if (this_d2 < c.d2) {
        c.d2 = this_d2;
        c.dc = (i == 0 ? this_dc : -this_dc);
        c.v[0] = (i == 0) * (j == 1) + (i == 1) * vw[0];
        c.w[0] = (i == 0) * (j == 2) + (i == 1) * vw[1];
        c.v[1] = (i == 1) * (j == 1) + (i == 0) * vw[0];
        c.w[1] = (i == 1) * (j == 2) + (i == 0) * vw[1];
      }
    }
  }
}

void shell_shell_compute(const Point* const p[2][3], PairGeom& c) {
  c.d2 = std::numeric_limits<Real>::max();
  c.dc = Point();
  c.v[0] = c.v[1] = c.w[0] = c.w[1] = 0;
  edge_edge_test(p, c);
  vertex_face_test(p, c);
}

// ---- Friction::apply (Friction.C:4-60): Margolis slip-stick law -------------
// f_contact is zero on entry (the callers' fresh vector); stick and
// spring_origin are the contact's persistent state.
void friction_apply(Real& Efric, Point& f_contact, Real f_normal, const Point& n, const Point& v, Real abs_v_normal,
                    Real v_stop, Real spring_stiffness, Real mu_s, Real mu_d, Real damping, bool& stick,
                    Point& spring_origin, const Point& contact_point) {
  // tangential velocity
  const Point v_normal = abs_v_normal * n;
  const Point v_tangential = v - v_normal;
  const Real abs_v_tangential = v_tangential.size();
  const Real v_eps = 1e-8 * v_stop;
  // static part
  if (mu_s > 0 && abs_v_tangential <= v_stop) {
    if (!stick) {
      // a new spring, sized so that the force is continuous from dynamic to static
      stick = true;
      const Real prefactor = mu_d * f_normal / (spring_stiffness * (abs_v_tangential + v_eps)) - damping;
      spring_origin = contact_point - prefactor * v_tangential;
    }
    Point u_spring = contact_point - spring_origin;
    u_spring -= (u_spring * n) * n;  // tangential part of the spring
    Efric = 0.5 * spring_stiffness * u_spring.size_sq();
    f_contact = -spring_stiffness * u_spring;
    f_contact -= damping * spring_stiffness * v_tangential;
  }
  // dynamic part
  if (abs_v_tangential > v_stop || f_contact.size_sq() >= std::pow(mu_s * f_normal, 2)) {
    spring_origin.zero();
    stick = false;
    Efric = 0;
    f_contact = -mu_d * f_normal / (abs_v_tangential + v_eps) * v_tangential;
  }
}

// The summation order of avg_elem_size (ShellSystem.C:2572, 2584).  The
// reference leaves it to OpenMP; the library fixes it so that host and device
// agree: 1024 lanes, lane l adding x[l], x[l + 1024], ... in index order, then
// the lanes combined pairwise (strides 512, 256, ..., 1).
Real fixed_order_sum(const Real* x, unsigned n) {
  const unsigned lanes = 1024;
  std::vector<Real> lane(lanes, 0.0);
  for (unsigned l = 0; l < lanes; ++l) {
    Real s = 0;
    for (unsigned i = l; i < n; i += lanes) s = s + x[i];
    lane[l] = s;
  }
  for (unsigned stride = lanes / 2; stride > 0; stride /= 2)
    for (unsigned l = 0; l < stride; ++l) lane[l] = lane[l] + lane[l + stride];
  return lane[0];
}

struct Tensor {  // 3x3, row major
  Real a[3][3];
  Tensor() { std::memset(a, 0, sizeof(a)); }
  Real& operator()(int i, int j) { return a[i][j]; }
  Real operator()(int i, int j) const { return a[i][j]; }
  Tensor operator*(const Tensor& o) const {
    Tensor r;
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) {
        Real s = 0;
        for (int k = 0; k < 3; ++k) s += a[i][k] * o.a[k][j];
        r.a[i][j] = s;
      }
    return r;
  }
  Point operator*(const Point& p) const {
    return Point(a[0][0] * p(0) + a[0][1] * p(1) + a[0][2] * p(2), a[1][0] * p(0) + a[1][1] * p(1) + a[1][2] * p(2),
                 a[2][0] * p(0) + a[2][1] * p(1) + a[2][2] * p(2));
  }
};

// ShellSystem::inverse, ShellSystem.h:437-455
Tensor inverse3(const Tensor& A) {
  const Real det00 = A(1, 1) * A(2, 2) - A(1, 2) * A(2, 1);
  const Real det01 = A(1, 2) * A(2, 0) - A(1, 0) * A(2, 2);
  const Real det02 = A(1, 0) * A(2, 1) - A(1, 1) * A(2, 0);
  const Real det10 = A(0, 2) * A(2, 1) - A(0, 1) * A(2, 2);
  const Real det11 = A(0, 0) * A(2, 2) - A(0, 2) * A(2, 0);
  const Real det12 = A(0, 1) * A(2, 0) - A(0, 0) * A(2, 1);
  const Real det20 = A(0, 1) * A(1, 2) - A(0, 2) * A(1, 1);
  const Real det21 = A(0, 2) * A(1, 0) - A(0, 0) * A(1, 2);
  const Real det22 = A(0, 0) * A(1, 1) - A(0, 1) * A(1, 0);
  const Real inv_det = 1 / (A(0, 0) * det00 + A(0, 1) * det01 + A(0, 2) * det02);
  Tensor r;
  r(0, 0) = inv_det * det00; r(0, 1) = inv_det * det10; r(0, 2) = inv_det * det20;
  r(1, 0) = inv_det * det01; r(1, 1) = inv_det * det11; r(1, 2) = inv_det * det21;
  r(2, 0) = inv_det * det02; r(2, 1) = inv_det * det12; r(2, 2) = inv_det * det22;
  return r;
}

/* ------------------------------------------------------------------------
 * Loop box-spline basis of a regular 12-node patch (Stam's numbering).
 * Each function is (1/12) * sum coef * u^i v^j w^k with u = 1 - v - w.
 * Node s sits at lattice offset (sv[s], sw[s]) from the element origin;
 * the element is (s3, s6, s7) = origin, +v, +w.
 * ------------------------------------------------------------------------ */
struct Mono { int c, i, j, k; };
const Mono kN[12][15] = {
  {{1,4,0,0},{2,3,1,0}},
  {{1,4,0,0},{2,3,0,1}},
  {{1,4,0,0},{2,3,0,1},{6,3,1,0},{6,2,1,1},{12,2,2,0},{6,1,2,1},{6,1,3,0},{2,0,3,1},{1,0,4,0}},
  {{6,4,0,0},{24,3,0,1},{24,2,0,2},{8,1,0,3},{1,0,0,4},{24,3,1,0},{60,2,1,1},{36,1,1,2},{6,0,1,3},
   {24,2,2,0},{36,1,2,1},{12,0,2,2},{8,1,3,0},{6,0,3,1},{1,0,4,0}},
  {{1,4,0,0},{6,3,0,1},{12,2,0,2},{6,1,0,3},{1,0,0,4},{2,3,1,0},{6,2,1,1},{6,1,1,2},{2,0,1,3}},
  {{2,1,3,0},{1,0,4,0}},
  {{1,4,0,0},{6,3,0,1},{12,2,0,2},{6,1,0,3},{1,0,0,4},{8,3,1,0},{36,2,1,1},{36,1,1,2},{8,0,1,3},
   {24,2,2,0},{60,1,2,1},{24,0,2,2},{24,1,3,0},{24,0,3,1},{6,0,4,0}},
  {{1,4,0,0},{8,3,0,1},{24,2,0,2},{24,1,0,3},{6,0,0,4},{6,3,1,0},{36,2,1,1},{60,1,1,2},{24,0,1,3},
   {12,2,2,0},{36,1,2,1},{24,0,2,2},{6,1,3,0},{8,0,3,1},{1,0,4,0}},
  {{2,1,0,3},{1,0,0,4}},
  {{2,0,3,1},{1,0,4,0}},
  {{2,1,0,3},{1,0,0,4},{6,1,1,2},{6,0,1,3},{6,1,2,1},{12,0,2,2},{2,1,3,0},{6,0,3,1},{1,0,4,0}},
  {{1,0,0,4},{2,0,1,3}},
};

// monomial coefficients in (v,w): C[s][p][q] for v^p w^q, times 1/12
struct BoxSpline {
  double C[12][5][5];
  BoxSpline() {
    std::memset(C, 0, sizeof(C));
    const int fact[5] = {1, 1, 2, 6, 24};
    for (int s = 0; s < 12; ++s)
      for (int t = 0; t < 15; ++t) {
        const Mono& m = kN[s][t];
        if (m.c == 0) break;
        // u^i = (1 - v - w)^i = sum_{a+b+c=i} i!/(a!b!c!) (-v)^b (-w)^c
        for (int b = 0; b <= m.i; ++b)
          for (int c = 0; b + c <= m.i; ++c) {
            const int a = m.i - b - c;
            const int mult = fact[m.i] / (fact[a] * fact[b] * fact[c]);
            const int sgn = ((b + c) & 1) ? -1 : 1;
            C[s][m.j + b][m.k + c] += (double)(m.c * mult * sgn) / 12.0;
          }
      }
  }
  // out[6*s + k]: value, d/dv, d/dw, d2/dv2, d2/dw2, d2/dvdw
  void eval(double v, double w, double* out) const {
    double vp[5], wp[5];
    vp[0] = wp[0] = 1;
    for (int i = 1; i < 5; ++i) { vp[i] = vp[i - 1] * v; wp[i] = wp[i - 1] * w; }
    for (int s = 0; s < 12; ++s) {
      double f = 0, fv = 0, fw = 0, fvv = 0, fww = 0, fvw = 0;
      for (int p = 0; p < 5; ++p)
        for (int q = 0; p + q < 5; ++q) {
          const double c = C[s][p][q];
          if (c == 0) continue;
          f += c * vp[p] * wp[q];
          if (p >= 1) fv += c * p * vp[p - 1] * wp[q];
          if (q >= 1) fw += c * q * vp[p] * wp[q - 1];
          if (p >= 2) fvv += c * p * (p - 1) * vp[p - 2] * wp[q];
          if (q >= 2) fww += c * q * (q - 1) * vp[p] * wp[q - 2];
          if (p >= 1 && q >= 1) fvw += c * p * q * vp[p - 1] * wp[q - 1];
        }
      out[6 * s + 0] = f; out[6 * s + 1] = fv; out[6 * s + 2] = fw;
      out[6 * s + 3] = fvv; out[6 * s + 4] = fww; out[6 * s + 5] = fvw;
    }
  }
};
const BoxSpline g_box;

/* Patch order used here, for an element (a, b, c) whose vertex a has valence N
 * (b and c regular):
 *   0: a, 1: b, 2: c, 3..N: the remaining neighbours n2..n_{N-1} of a
 *   (counter-clockwise after c), N+1: d (across edge bc), N+2: (2,0),
 *   N+3: (2,-1), N+4: (0,2), N+5: (-1,2)   [lattice offsets for N = 6].
 * For N = 6 the Stam node s maps to patch index kStamToPatch[s]. */
const int kStamToPatch[12] = {5, 4, 6, 0, 3, 9, 1, 2, 11, 8, 7, 10};

double loop_beta(int N) {
  const double t = 3.0 / 8.0 + 0.25 * std::cos(2.0 * M_PI / N);
  return (5.0 / 8.0 - t * t) / N;
}

/* Stencil of the middle sub-triangle's 12 Stam nodes after one Loop step, as
 * weights over the N+6 patch nodes. S[s*(N+6) + p]. */
void irregular_stencil(int N, std::vector<double>& S) {
  const int np = N + 6;
  S.assign(12 * np, 0.0);
  const int a = 0, b = 1, c = 2, n2 = 3, n3 = 4, nl = N, nl2 = N - 1, d = N + 1, e2 = N + 2, e1 = N + 3,
            f1 = N + 4, f2 = N + 5;
  auto edge = [&](int s, int p, int q, int r, int t) {
    S[s * np + p] += 3.0 / 8.0; S[s * np + q] += 3.0 / 8.0;
    S[s * np + r] += 1.0 / 8.0; S[s * np + t] += 1.0 / 8.0;
  };
  auto vert6 = [&](int s, int center, const int* ring) {
    S[s * np + center] += 5.0 / 8.0;
    for (int k = 0; k < 6; ++k) S[s * np + ring[k]] += 1.0 / 16.0;
  };
  edge(0, c, d, b, f1);
  edge(1, b, d, c, e2);
  { const int ring[6] = {a, b, d, f1, f2, n2}; vert6(2, c, ring); }
  edge(3, b, c, a, d);
  { const int ring[6] = {c, a, nl, e1, e2, d}; vert6(4, b, ring); }
  edge(5, c, n2, a, f2);
  edge(6, a, c, b, n2);
  edge(7, a, b, c, nl);
  edge(8, b, nl, a, e1);
  edge(9, a, n2, c, n3);
  {  // vertex point of a
    const double beta = loop_beta(N);
    S[10 * np + a] += 1.0 - N * beta;
    S[10 * np + b] += beta;
    S[10 * np + c] += beta;
    for (int k = 2; k < N; ++k) S[10 * np + (k + 1)] += beta;
  }
  edge(11, a, nl, b, nl2);
}


/* ------------------------------------------------------------------------
 * SmoothShellShellContact::compute (SmoothShellShellContact.C:16-60): the
 * closest points of the limit surfaces of two faces, minimising
 * f(x) = |p2(v2, w2) - p1(v1, w1)|^2 over x = (v1, w1, v2, w2) subject to
 * v, w >= 0 and v + w <= 1 per face, from the pair's previous solution.  The
 * constraint hooks are the reference's: apply_constraints (:155-179),
 * update_constraint_bitmap (:139-152, activity within 100 eps) and
 * find_max_alpha (:96-136).  The minimiser (ConstrainedMinimizer.h) is not in
 * the reference's sources; it is restated here, on the oracle's own code, as
 * the active-set projected Newton method that the library documents: exact
 * Hessian from the limit surface's second derivatives, Jacobi-scaled and
 * shifted by mu I until its Cholesky factor exists on the free subspace of the
 * working set (multiplier signs of the active constraints), Armijo
 * backtracking capped by find_max_alpha; stops on a projected gradient below
 * 1e-9 of the gradient, a Newton decrement below 1e-15 of f, a short full
 * Newton step (1e-6), a vanishing step (1e-14), a failed line search or 40
 * iterations.  Only the limit evaluation (shl_limit.h) is shared with the
 * library.  Every operation is rounded on its own (-ffp-contract=off).
 * ------------------------------------------------------------------------ */
namespace smooth {

const double kEps = 2.220446049250313e-16;
const double kActiveTol = 100 * kEps;
const int kMaxIt = 40, kMaxHalvings = 30;
const double kStepTol = 1e-14, kDecrementTol = 1e-15, kQuadTol = 1e-6, kKktTol = 1e-9;

inline double dot(const double* a, const double* b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }

// apply_constraints: clip to v, w >= 0, then pull the larger coordinate back
// when v + w exceeds 1
void apply_constraints(double* x) {
  for (int i = 0; i < 4; ++i) x[i] = std::fmax(x[i], 0.0);
  for (int e = 0; e < 2; ++e) {
    const double u = (1.0 - x[2 * e]) - x[2 * e + 1];
    if (u < 0.0) {
      double& big = x[2 * e] > x[2 * e + 1] ? x[2 * e] : x[2 * e + 1];
      big = big + (u - kEps);
    }
  }
}

// update_constraint_bitmap: bits 0..3 coordinate i at 0, bits 4, 5 v + w at 1
unsigned bitmap(const double* x) {
  unsigned m = 0;
  for (int i = 0; i < 4; ++i)
    if (x[i] < kActiveTol) m |= 1u << i;
  if (x[0] + x[1] > 1.0 - kActiveTol) m |= 1u << 4;
  if (x[2] + x[3] > 1.0 - kActiveTol) m |= 1u << 5;
  return m;
}

// find_max_alpha: the longest feasible step along d (the largest double if none limits it)
double max_alpha(const double* x, const double* d) {
  double a = std::numeric_limits<double>::max();
  for (int i = 0; i < 4; ++i)
    if (d[i] < 0.0) a = std::fmin(a, -x[i] / d[i]);
  for (int e = 0; e < 2; ++e) {
    const double ds = d[2 * e] + d[2 * e + 1];
    if (ds > 0.0) a = std::fmin(a, ((1.0 - x[2 * e]) - x[2 * e + 1]) / ds);
  }
  return a;
}

// the working constraints of one face (1: v = 0, 2: w = 0, 4: v + w = 1) among
// its active ones, kept where the first-order multiplier is non-negative
unsigned working(unsigned act, double gv, double gw) {
  const double mu_v = gv, mu_w = gw, mu_s = -(gv + gw);
  switch (act) {
    case 3u:  // corner (0, 0)
      if (mu_v >= 0.0 && mu_w >= 0.0) return 3u;
      return mu_v >= 0.0 ? 1u : (mu_w >= 0.0 ? 2u : 0u);
    case 5u: {  // corner (0, 1): g = a (1, 0) + b (-1, -1)
      const double a = gv - gw, b = -gw;
      if (a >= 0.0 && b >= 0.0) return 5u;
      if (a >= 0.0) return mu_v >= 0.0 ? 1u : 0u;
      if (b >= 0.0) return mu_s >= 0.0 ? 4u : 0u;
      return 0u;
    }
    case 6u: {  // corner (1, 0): g = a (0, 1) + b (-1, -1)
      const double a = gw - gv, b = -gv;
      if (a >= 0.0 && b >= 0.0) return 6u;
      if (a >= 0.0) return mu_w >= 0.0 ? 2u : 0u;
      if (b >= 0.0) return mu_s >= 0.0 ? 4u : 0u;
      return 0u;
    }
    case 1u: return mu_v >= 0.0 ? 1u : 0u;
    case 2u: return mu_w >= 0.0 ? 2u : 0u;
    case 4u: return mu_s >= 0.0 ? 4u : 0u;
    default: return 0u;
  }
}

// f, its gradient and Hessian at x (limit points and derivatives of both faces)
double value_grad_hess(const shl_limit_patch* A, const shl_limit_patch* B, const double* x, double* g,
                       double H[4][4], double* p1, double* p2) {
  double a[6][3], b[6][3];
  shl_limit_eval(A, x[0], x[1], 2, a);
  shl_limit_eval(B, x[2], x[3], 2, b);
  double r[3], dr[4][3];  // r = p2 - p1 and its derivatives along x
  for (int c = 0; c < 3; ++c) {
    r[c] = b[0][c] - a[0][c];
    dr[0][c] = -a[1][c];
    dr[1][c] = -a[2][c];
    dr[2][c] = b[1][c];
    dr[3][c] = b[2][c];
    p1[c] = a[0][c];
    p2[c] = b[0][c];
  }
  for (int i = 0; i < 4; ++i) g[i] = 2.0 * dot(r, dr[i]);
  // r . (second derivatives of r): -p1's within face 1, p2's within face 2
  const double s00 = -dot(r, a[3]), s11 = -dot(r, a[4]), s01 = -dot(r, a[5]);
  const double s22 = dot(r, b[3]), s33 = dot(r, b[4]), s23 = dot(r, b[5]);
  for (int i = 0; i < 4; ++i)
    for (int j = i; j < 4; ++j) {
      double h = dot(dr[i], dr[j]);
      if (i == 0 && j == 0) h = h + s00;
      if (i == 1 && j == 1) h = h + s11;
      if (i == 0 && j == 1) h = h + s01;
      if (i == 2 && j == 2) h = h + s22;
      if (i == 3 && j == 3) h = h + s33;
      if (i == 2 && j == 3) h = h + s23;
      H[i][j] = 2.0 * h;
      H[j][i] = H[i][j];
    }
  return dot(r, r);
}

double value(const shl_limit_patch* A, const shl_limit_patch* B, const double* x, double* p1, double* p2) {
  double a[6][3], b[6][3];
  shl_limit_eval(A, x[0], x[1], 0, a);
  shl_limit_eval(B, x[2], x[3], 0, b);
  double r[3];
  for (int c = 0; c < 3; ++c) {
    r[c] = b[0][c] - a[0][c];
    p1[c] = a[0][c];
    p2[c] = b[0][c];
  }
  return dot(r, r);
}

// Newton direction on the free subspace of the working set; true when the
// reduced Hessian had to be shifted (f not convex there)
bool newton_direction(const double* g, double H[4][4], const unsigned* work, double* d) {
  // basis of the free subspace, face by face
  double Z[4][4];
  int m = 0;
  for (int e = 0; e < 2; ++e) {
    const int iv = 2 * e, iw = 2 * e + 1;
    auto push = [&](double zv, double zw) {
      for (int i = 0; i < 4; ++i) Z[m][i] = 0.0;
      Z[m][iv] = zv;
      Z[m][iw] = zw;
      ++m;
    };
    switch (work[e]) {
      case 0u: push(1.0, 0.0); push(0.0, 1.0); break;
      case 1u: push(0.0, 1.0); break;   // v = 0: w free
      case 2u: push(1.0, 0.0); break;   // w = 0: v free
      case 4u: push(1.0, -1.0); break;  // v + w = 1
      default: break;
    }
  }
  for (int i = 0; i < 4; ++i) d[i] = 0.0;
  if (m == 0) return false;
  double Hz[4][4], rg[4], rh[4][4];
  for (int a = 0; a < m; ++a) {
    double s = 0.0;
    for (int i = 0; i < 4; ++i) s = s + Z[a][i] * g[i];
    rg[a] = s;
    for (int i = 0; i < 4; ++i) {
      double t = 0.0;
      for (int j = 0; j < 4; ++j) t = t + H[i][j] * Z[a][j];
      Hz[a][i] = t;
    }
  }
  for (int a = 0; a < m; ++a)
    for (int c = 0; c < m; ++c) {
      double s = 0.0;
      for (int i = 0; i < 4; ++i) s = s + Z[a][i] * Hz[c][i];
      rh[a][c] = s;
    }
  // unit diagonal: the free directions' scales differ by powers of 2 next to an irregular vertex
  double sc[4];
  for (int a = 0; a < m; ++a) {
    const double h = std::fabs(rh[a][a]);
    sc[a] = h > 0.0 ? 1.0 / std::sqrt(h) : 1.0;
  }
  for (int a = 0; a < m; ++a) {
    rg[a] = sc[a] * rg[a];
    for (int c = 0; c < m; ++c) rh[a][c] = (sc[a] * rh[a][c]) * sc[c];
  }
  double shift = 0.0, L[4][4], y[4];
  for (int attempt = 0; attempt < 24; ++attempt) {
    bool factored = true;
    for (int a = 0; a < m && factored; ++a)
      for (int c = 0; c <= a; ++c) {
        double s = rh[a][c];
        if (a == c) s = s + shift;
        for (int k = 0; k < c; ++k) s = s - L[a][k] * L[c][k];
        if (a == c) {
          if (!(s > 1e-14)) {
            factored = false;
            break;
          }
          L[a][a] = std::sqrt(s);
        } else {
          L[a][c] = s / L[c][c];
        }
      }
    if (factored) {
      for (int a = 0; a < m; ++a) {  // forward: L y = -rg
        double s = -rg[a];
        for (int k = 0; k < a; ++k) s = s - L[a][k] * y[k];
        y[a] = s / L[a][a];
      }
      for (int a = m - 1; a >= 0; --a) {  // backward: L^T y = y
        double s = y[a];
        for (int k = a + 1; k < m; ++k) s = s - L[k][a] * y[k];
        y[a] = s / L[a][a];
      }
      for (int i = 0; i < 4; ++i) {
        double s = 0.0;
        for (int a = 0; a < m; ++a) s = s + Z[a][i] * (sc[a] * y[a]);
        d[i] = s;
      }
      return shift > 0.0;
    }
    shift = shift == 0.0 ? 1e-10 : shift * 10.0;
  }
  for (int i = 0; i < 4; ++i) {  // scaled projected steepest descent
    double s = 0.0;
    for (int a = 0; a < m; ++a) s = s + Z[a][i] * (sc[a] * -rg[a]);
    d[i] = s;
  }
  return true;
}

// the closest points of the limit patches A (face 1) and B (face 2) from x;
// x becomes the minimiser, d2 = |p2 - p1|^2 and dc = p2 - p1
int closest(const shl_limit_patch* A, const shl_limit_patch* B, double* x, double* d2, double* dc) {
  apply_constraints(x);
  double p1[3], p2[3], g[4], H[4][4];
  double f = value_grad_hess(A, B, x, g, H, p1, p2);
  int it = 0;
  for (; it < kMaxIt; ++it) {
    const unsigned bm = bitmap(x);
    unsigned act[2], work[2];
    for (int e = 0; e < 2; ++e) {
      act[e] = ((bm >> (2 * e)) & 1u) | (((bm >> (2 * e + 1)) & 1u) << 1) | (((bm >> (4 + e)) & 1u) << 2);
      work[e] = working(act[e], g[2 * e], g[2 * e + 1]);
    }
    // first-order optimality on the working set
    double pg = 0.0, gmax = 0.0;
    for (int e = 0; e < 2; ++e) {
      const double gv = g[2 * e], gw = g[2 * e + 1];
      gmax = std::fmax(gmax, std::fmax(std::fabs(gv), std::fabs(gw)));
      switch (work[e]) {
        case 0u: pg = std::fmax(pg, std::fmax(std::fabs(gv), std::fabs(gw))); break;
        case 1u: pg = std::fmax(pg, std::fabs(gw)); break;
        case 2u: pg = std::fmax(pg, std::fabs(gv)); break;
        case 4u: pg = std::fmax(pg, 0.5 * std::fabs(gv - gw)); break;
        default: break;
      }
    }
    if (pg <= kKktTol * gmax) break;
    double d[4];
    bool shifted = false;
    // a constraint left out of the working set must not be violated by the step:
    // each round adds one back
    for (int round = 0; round < 6; ++round) {
      shifted = newton_direction(g, H, work, d);
      bool added = false;
      for (int e = 0; e < 2; ++e) {
        const unsigned freed = act[e] & ~work[e];
        unsigned add = 0;
        if ((freed & 1u) && d[2 * e] < 0.0) add |= 1u;
        if ((freed & 2u) && d[2 * e + 1] < 0.0) add |= 2u;
        if ((freed & 4u) && d[2 * e] + d[2 * e + 1] > 0.0) add |= 4u;
        if (add) {
          work[e] |= add;
          added = true;
        }
      }
      if (!added) break;
    }
    double dmax = 0.0, gd = 0.0;
    for (int i = 0; i < 4; ++i) {
      dmax = std::fmax(dmax, std::fabs(d[i]));
      gd = gd + g[i] * d[i];
    }
    if (!(dmax > 0.0) || !(gd < 0.0) || -gd <= kDecrementTol * f) break;
    const double amax = max_alpha(x, d);
    double alpha = (shifted || amax < 1.0) ? amax : 1.0;
    if (!(alpha > 0.0)) break;
    double xt[4], q1[3], q2[3], ft = 0.0;
    bool accepted = false;
    for (int ls = 0; ls < kMaxHalvings; ++ls) {
      for (int i = 0; i < 4; ++i) xt[i] = x[i] + alpha * d[i];
      apply_constraints(xt);
      ft = value(A, B, xt, q1, q2);
      if (ft <= f + (1e-4 * alpha) * gd) {
        accepted = true;
        break;
      }
      const double half = alpha * 0.5;
      alpha = (ls == 0 && shifted) ? std::fmin(half, 0.05 / dmax) : half;
    }
    if (!accepted) break;
    double step = 0.0;
    for (int i = 0; i < 4; ++i) {
      step = std::fmax(step, std::fabs(xt[i] - x[i]));
      x[i] = xt[i];
    }
    const bool full_newton = !shifted && alpha == 1.0;
    if (step <= kStepTol || (full_newton && step <= kQuadTol)) {
      f = ft;
      for (int c = 0; c < 3; ++c) {
        p1[c] = q1[c];
        p2[c] = q2[c];
      }
      ++it;
      break;
    }
    f = value_grad_hess(A, B, x, g, H, p1, p2);
  }
  *d2 = f;
  for (int c = 0; c < 3; ++c) dc[c] = p2[c] - p1[c];
  return it;
}

}  // namespace smooth

/* ------------------------------------------------------------------------ */

struct SurfaceMetric {  // ShellSystem.h:56-63
  Point xyz;
  Point vec[3], dvec[3];
  Point ff1, ff2;
  Real jac;
};

struct ElemCache {  // ShellSystem.h:74-101 (single quadrature point)
  Real area = 0;
  std::vector<unsigned> patch;  // node ids
  Real JxW = 0;
  std::vector<Real> phi;
  std::vector<Point> dphi;   // (d/ds1, d/ds2, 0)
  std::vector<Point> d2phi;  // (11, 22, 12)
  SurfaceMetric a_ref, a_def;
  Tensor H;
  Point alpha, beta;
  Point qxyz;
  Real R[2][2];
  Real bmin[3], bmax[3];
  std::vector<unsigned> neighbor_elems;  // sorted
  std::vector<unsigned> close_elems;     // sorted
  std::list<unsigned> in_contact_with;
  Real kGauss = 0, kMean = 0, etens = 0, ebend = 0;
};

struct Contact {  // Contact.h:14-19, ShellShellContact.h:17-20
  unsigned eid[2];
  Real d2 = 0;
  bool stick = false;
  Point dc, spring_origin;
  Real v[2] = {0, 0}, w[2] = {0, 0};
  // SMOOTH: the minimiser's (v1, w1, v2, w2) in each face's patch frame (irregular
  // vertex first), kept from step to step; 1/3 for a new pair
  // (SmoothShellShellContact.C:9-14)
  Real x[4] = {1.0 / 3, 1.0 / 3, 1.0 / 3, 1.0 / 3};
};

}  // namespace

struct oracle {
  // mesh
  unsigned V = 0, F = 0;
  std::vector<Point> X;
  std::vector<unsigned> tri;
  std::vector<std::vector<unsigned>> nodes_to_elem;
  std::vector<ElemCache> ec;
  std::vector<int> valence;

  shl_params P;
  // derived (update_derived)
  Real K = 0, D = 0, stiff_density = 0, stiff_static_friction = 0, d2_touch = 0, d2_friction = 0;
  Real thickness0 = 0;
  Real qw = 0.5;  // one-point rule on the reference triangle

  // state
  std::vector<Real> u, v, a, f, Minv, C, u_pred, v_pred, a_pred;
  std::vector<Point> p;  // NodeCache::p
  Real time = 0;
  unsigned time_step = 0;
  Real dt = 0;
  Real newmark_a[10];
  Real pressure = 0;
  Real volume = 0, volume0 = 0, area = 0;

  // contact
  Real du_sum = 0, avg_elem_size = 0;
  Real bounds_min[3], bounds_max[3];
  Real last_cell_size = 0, last_d_max = 0;
  std::vector<std::vector<double>> subdiv_tab = std::vector<std::vector<double>>(13);  // SMOOTH: by valence
  uint64_t n_cells_max = 0;
  std::vector<Contact*> candidates;

  // measurement
  unsigned Nc = 0;
  Real Eself = 0, Efric = 0, Etens = 0, Ebend = 0, Ekin = 0, kGauss = 0, kMean = 0;
  // node_vectors ekin, eself, efric (ShellSystem.C:126-130), reset every step
  std::vector<Real> ekin_vec, eself_vec, efric_vec, ecav_vec;
  // cavity contact (ShellSystem.C:1600-1723): spring origins per node, measurements
  std::vector<Point> cav_origin;
  std::vector<std::vector<unsigned>> vertex_faces;  // faces of which each node is a vertex
  unsigned Nc_cav = 0;
  Real Ecav = 0, cavity_force = 0;
  Real cav_R[3] = {0, 0, 0};
  shl::expr::Expression rfun[3];
  bool has_rfun[3] = {false, false, false};
  void add_cavity_force();
  int current_problem = 0;

  ~oracle() {
    for (Contact* c : candidates) delete c;
  }

  unsigned dof(unsigned nid, int var) const { return 3 * nid + var; }

  void register_problem(int pr) {
    if (pr > current_problem) current_problem = pr;
  }

  /* ------------------------------ set-up -------------------------------- */
  bool build(const shl_mesh* m, const shl_params* prm);
  bool build_patch(unsigned eid, std::vector<unsigned>& patch, int& N);
  void basis_unrotated(unsigned eid, double v, double w, std::vector<double>& out);
  void update_derived();
  void reinit_mod_and_reference(unsigned eid);
  void compute_mass_damping();
  void build_topological_neighborhood();
  void set_newmark_parameters(Real new_dt);
  template <class PressureAt>
  bool advance(const PressureAt& p_at);
  Real dt_step = 0;       // dt of the last accepted step
  bool accepted = false;  // the last advance() accepted a step
  uint64_t rejections = 0;
  uint64_t n_rebuilds = 0;  // candidate-list rebuilds made (forced or triggered)
  shl::expr::Expression pfun;  // pressure as an expression of t, when set
  bool has_pfun = false;

  /* ------------------------------ step ---------------------------------- */
  void compute_position();
  void reset_properties();
  void prepare_next_step(Real p_now);
  void check_increment(bool require_change);
  void compute_bounding_box();
  void compute_deformed_metrics();
  void compute_external_force();
  void subtract_internal_force();
  void add_shell_shell_contact_force();
  void compute_shell_shell_contact_candidates(bool force);
  void compute_enclosed_volume();
  void measure_properties();
  bool elems_are_close(unsigned e1, unsigned e2) const {
    const std::vector<unsigned>& ce = ec[e1].close_elems;
    return std::binary_search(ce.begin(), ce.end(), e2);
  }
  // limit patch of face e at the current positions (SubdivEvaluation.C:14-77)
  void limit_patch(unsigned e, shl_limit_patch& lp) const {
    const std::vector<unsigned>& pt = ec[e].patch;
    lp.N = (int)pt.size() - 6;
    lp.base = p[0].x;  // Point is three packed doubles
    lp.ids = pt.data();
    lp.stride = 1;
    lp.tab = lp.N == 6 ? nullptr : subdiv_tab[lp.N].data();
  }
  // position of the patch's first vertex in the face's node list
  int patch_rotation(unsigned e) const {
    for (int k = 0; k < 3; ++k)
      if (tri[3 * e + k] == ec[e].patch[0]) return k;
    return 0;
  }
  // SmoothShellShellContact::compute (SmoothShellShellContact.C:16-60); the
  // minimiser's coordinates are handed to the force distribution in the face's
  // own node order (u, v, w of tri[0..2])
  void smooth_compute(Contact& c) const {
    shl_limit_patch A, B;
    limit_patch(c.eid[0], A);
    limit_patch(c.eid[1], B);
    double d2, dc[3];
    smooth::closest(&A, &B, c.x, &d2, dc);
    c.d2 = d2;
    c.dc = Point(dc[0], dc[1], dc[2]);
    for (int e = 0; e < 2; ++e) {
      const int r = patch_rotation(c.eid[e]);
      double lam[3];
      lam[r] = 1 - c.x[2 * e] - c.x[2 * e + 1];
      lam[(r + 1) % 3] = c.x[2 * e];
      lam[(r + 2) % 3] = c.x[2 * e + 1];
      c.v[e] = lam[1];
      c.w[e] = lam[2];
    }
  }
  void pair_compute(Contact& c, bool on_mesh) const {
    if (!on_mesh && P.shell_shell_contact == SHL_CONTACT_SMOOTH) {
      smooth_compute(c);
      return;
    }
    const Point* pp[2][3];
    for (int e = 0; e < 2; ++e)
      for (int n = 0; n < 3; ++n) pp[e][n] = on_mesh ? &X[tri[3 * c.eid[e] + n]] : &p[tri[3 * c.eid[e] + n]];
    PairGeom g;
    shell_shell_compute(pp, g);
    c.d2 = g.d2;
    c.dc = g.dc;
    c.v[0] = g.v[0]; c.v[1] = g.v[1]; c.w[0] = g.w[0]; c.w[1] = g.w[1];
  }
  Point contact_point(const Contact& c) const {  // ShellShellContact::point()
    const Point& p0 = p[tri[3 * c.eid[0]]];
    const Point& p1 = p[tri[3 * c.eid[0] + 1]];
    const Point& p2 = p[tri[3 * c.eid[0] + 2]];
    return (1 - c.v[0] - c.w[0]) * p0 + c.v[0] * p1 + c.w[0] * p2 + 0.5 * c.dc;
  }
};

bool oracle::build_patch(unsigned eid, std::vector<unsigned>& patch, int& N) {
  unsigned t[3] = {tri[3 * eid], tri[3 * eid + 1], tri[3 * eid + 2]};
  int irr = -1, n_irr = 0;
  for (int k = 0; k < 3; ++k)
    if (valence[t[k]] != 6) { irr = k; ++n_irr; }
  if (n_irr > 1) {
    g_err = "element " + std::to_string(eid) + " has more than one irregular vertex";
    return false;
  }
  const int r = irr < 0 ? 0 : irr;
  const unsigned A = t[r], B = t[(r + 1) % 3], Cc = t[(r + 2) % 3];
  // next-vertex around a vertex: for face (x,y,z) oriented, around x: y -> z
  auto next_around = [&](unsigned center, unsigned from) -> long {
    for (unsigned e : nodes_to_elem[center]) {
      for (int k = 0; k < 3; ++k)
        if (tri[3 * e + k] == center && tri[3 * e + (k + 1) % 3] == from) return tri[3 * e + (k + 2) % 3];
    }
    return -1;
  };
  auto ring = [&](unsigned center, unsigned start, std::vector<unsigned>& out) -> bool {
    out.clear();
    out.push_back(start);
    long x = next_around(center, start);
    while (x >= 0 && (unsigned)x != start) {
      out.push_back((unsigned)x);
      if (out.size() > 64) return false;
      x = next_around(center, (unsigned)x);
    }
    return x >= 0;
  };
  std::vector<unsigned> ra, rb, rc;
  if (!ring(A, B, ra) || !ring(B, Cc, rb) || !ring(Cc, A, rc) || rb.size() != 6 || rc.size() != 6) {
    g_err = "element " + std::to_string(eid) + ": open or non-manifold one-ring";
    return false;
  }
  N = (int)ra.size();
  patch.clear();
  patch.push_back(A);
  patch.push_back(B);
  patch.push_back(Cc);
  for (int k = 2; k < N; ++k) patch.push_back(ra[k]);
  // consistency of the rings: rb = [c, a, n_{N-1}, (2,-1), (2,0), d], rc = [a, b, d, (0,2), (-1,2), n2]
  if (rb[1] != A || rb[2] != ra[N - 1] || rc[1] != B || rc[5] != ra[2] || rb[5] != rc[2]) {
    g_err = "element " + std::to_string(eid) + ": inconsistent one-ring";
    return false;
  }
  patch.push_back(rb[5]);  // d
  patch.push_back(rb[4]);  // (2,0)
  patch.push_back(rb[3]);  // (2,-1)
  patch.push_back(rc[3]);  // (0,2)
  patch.push_back(rc[4]);  // (-1,2)
  return true;
}

void oracle::basis_unrotated(unsigned eid, double v, double w, std::vector<double>& out) {
  const int N = (int)ec[eid].patch.size() - 6;
  const int np = N + 6;
  out.assign(6 * np, 0.0);
  double B[72];
  if (N == 6) {
    g_box.eval(v, w, B);
    for (int s = 0; s < 12; ++s)
      for (int k = 0; k < 6; ++k) out[6 * kStamToPatch[s] + k] = B[6 * s + k];
    return;
  }
  // middle triangle of the first subdivision: local (1-2v, 1-2w), Jacobian -2
  g_box.eval(1 - 2 * v, 1 - 2 * w, B);
  std::vector<double> S;
  irregular_stencil(N, S);
  const double scale[6] = {1, -2, -2, 4, 4, 4};
  for (int s = 0; s < 12; ++s)
    for (int pidx = 0; pidx < np; ++pidx) {
      const double wgt = S[s * np + pidx];
      if (wgt == 0) continue;
      for (int k = 0; k < 6; ++k) out[6 * pidx + k] += wgt * (scale[k] * B[6 * s + k]);
    }
}

// ShellSystem::update_derived, ShellSystem.C:421-487 (terms of the time step)
void oracle::update_derived() {
  d2_touch = P.thickness * P.thickness;
  d2_friction = std::pow((1 + P.static_friction_tol) * P.thickness, 2);
  const Real nu2 = (P.shell_young_modulus2 * P.shell_poisson_ratio) / P.shell_young_modulus;
  const Real one_nu2 = 1 - P.shell_poisson_ratio * nu2;
  K = P.memb_stiff_mult * P.thickness / one_nu2;
  D = P.bend_stiff_mult * std::pow(P.thickness, 3) / (12 * one_nu2);
  const Real E_avg = (P.shell_young_modulus + P.shell_young_modulus2) * 0.5;
  stiff_density = 0.5 * E_avg / (one_nu2 * P.thickness);
  stiff_static_friction = P.fric_stiff_mult * E_avg * P.thickness / one_nu2;
}

// ShellSystem::reinit_mod (ShellSystem.C:3321-3499) followed by the libMesh map
// recomputation and compute_reference_metrics (ShellSystem.C:1317-1379)
void oracle::reinit_mod_and_reference(unsigned eid) {
  ElemCache& cache = ec[eid];
  const int np = (int)cache.patch.size();
  std::vector<double> B;
  basis_unrotated(eid, 1.0 / 3.0, 1.0 / 3.0, B);

  // first map (unrotated): xyz, dxyzdxi, dxyzdeta and JxW
  Point xyz, b1, b2;
  for (int i = 0; i < np; ++i) {
    const Point& Xi = X[cache.patch[i]];
    xyz.add_scaled(Xi, B[6 * i + 0]);
    b1.add_scaled(Xi, B[6 * i + 1]);
    b2.add_scaled(Xi, B[6 * i + 2]);
  }
  {
    const Real g11 = b1 * b1, g12 = b1 * b2, g22 = b2 * b2;
    cache.JxW = std::sqrt(g11 * g22 - g12 * g12) * qw;
  }
  cache.qxyz = xyz;

  Point n = b1.cross(b2);
  const Point normal = n;
  Point dir(0, 0, 100);
  dir = dir / dir.size();
  n = n / n.size();
  Point j = dir - (dir * n) * n;
  Point k = -n.cross(j);
  const Real anglejb1 = std::atan2((j.cross(b1)).size(), j * b1);
  const Real jfac = normal.size() / (b1.size() * std::sin(anglejb1));
  const Real kfac = normal.size() / jfac;
  j *= jfac / j.size();
  k *= kfac / k.size();

  const Point vz(0, 0, 1);
  const Point pivot = n.cross(vz);
  Tensor Rn;
  Rn(0, 0) = Rn(1, 1) = Rn(2, 2) = 1;
  if (pivot.size() > 0) {
    const Point pivotn = pivot / pivot.size();
    const Real angle = std::atan2(pivot.size(), n * vz);
    Tensor Rod;
    Rod(0, 1) = -pivotn(2); Rod(0, 2) = pivotn(1);
    Rod(1, 0) = pivotn(2); Rod(1, 2) = -pivotn(0);
    Rod(2, 0) = -pivotn(1); Rod(2, 1) = pivotn(0);
    const Tensor Rod2 = Rod * Rod;
    const Real s = std::sin(angle), c1 = 1 - std::cos(angle);
    for (int r = 0; r < 3; ++r)
      for (int q = 0; q < 3; ++q) Rn(r, q) = (r == q ? 1.0 : 0.0) + s * Rod(r, q) + c1 * Rod2(r, q);
  }
  Tensor A, Bm;
  for (int i = 0; i < 3; ++i) {
    A(i, 0) = b1(i); A(i, 1) = b2(i);
    Bm(i, 0) = k(i); Bm(i, 1) = j(i);
    A(i, 2) = Bm(i, 2) = normal(i);
  }
  A = Rn * A;
  Bm = Rn * Bm;
  const Tensor R = inverse3(A) * Bm;
  cache.R[0][0] = R(0, 0); cache.R[0][1] = R(0, 1); cache.R[1][0] = R(1, 0); cache.R[1][1] = R(1, 1);

  cache.phi.assign(np, 0);
  cache.dphi.assign(np, Point());
  cache.d2phi.assign(np, Point());
  for (int w = 0; w < np; ++w) {
    const Real dxi = B[6 * w + 1], deta = B[6 * w + 2];
    const Real d00 = B[6 * w + 3], d11 = B[6 * w + 4], d01 = B[6 * w + 5], d10 = d01;
    cache.phi[w] = B[6 * w + 0];
    cache.dphi[w](0) = dxi * R(0, 0) + deta * R(1, 0);
    cache.dphi[w](1) = dxi * R(0, 1) + deta * R(1, 1);
    cache.d2phi[w](0) = d00 * R(0, 0) * R(0, 0) + d11 * R(1, 0) * R(1, 0) + 2 * d10 * R(0, 0) * R(1, 0);
    cache.d2phi[w](1) = d00 * R(0, 1) * R(0, 1) + d11 * R(1, 1) * R(1, 1) + 2 * d01 * R(0, 1) * R(1, 1);
    cache.d2phi[w](2) = d00 * R(0, 0) * R(0, 1) + d11 * R(1, 0) * R(1, 1) + d01 * R(0, 1) * R(1, 0) +
                        d10 * R(0, 0) * R(1, 1);
  }

  // second map with the rotated derivatives, then the reference metric
  SurfaceMetric& ar = cache.a_ref;
  ar = SurfaceMetric();
  ar.xyz = cache.qxyz;
  for (int i = 0; i < np; ++i) {
    const Point& Xi = X[cache.patch[i]];
    ar.vec[0].add_scaled(Xi, cache.dphi[i](0));
    ar.vec[1].add_scaled(Xi, cache.dphi[i](1));
    ar.dvec[0].add_scaled(Xi, cache.d2phi[i](0));
    ar.dvec[1].add_scaled(Xi, cache.d2phi[i](1));
    ar.dvec[2].add_scaled(Xi, cache.d2phi[i](2));
  }
  ar.vec[2] = ar.vec[0].cross(ar.vec[1]);
  ar.jac = ar.vec[2].size();
  ar.vec[2] *= 1 / ar.jac;
  ar.ff1(0) = ar.vec[0] * ar.vec[0];
  ar.ff1(1) = ar.vec[1] * ar.vec[1];
  ar.ff1(2) = ar.vec[0] * ar.vec[1];
  ar.ff2(0) = ar.dvec[0] * ar.vec[2];
  ar.ff2(1) = ar.dvec[1] * ar.vec[2];
  ar.ff2(2) = ar.dvec[2] * ar.vec[2];
  cache.a_def = ar;
}

// ShellSystem::compute_mass_damping, ShellSystem.C:762-852
void oracle::compute_mass_damping() {
  std::fill(Minv.begin(), Minv.end(), 0.0);
  std::fill(C.begin(), C.end(), 0.0);
#pragma omp parallel
  {
    std::vector<Real> Me, Ce;
#pragma omp for
    for (int eid = 0; eid < (int)F; ++eid) {
      const ElemCache& cache = ec[eid];
      const unsigned n_var_dofs = (unsigned)cache.patch.size();
      Me.assign(3 * n_var_dofs, 0.0);
      Ce.assign(3 * n_var_dofs, 0.0);
      const Real JxW = cache.JxW;
      const Real avg_growth = 1;
      for (unsigned i = 0; i < n_var_dofs; ++i) {
        Real lumped_mass = 0;
        for (unsigned jj = 0; jj < n_var_dofs; ++jj) lumped_mass += cache.phi[jj];
        lumped_mass *= JxW * cache.phi[i];
        Me[i] += lumped_mass;
        Me[n_var_dofs + i] += lumped_mass;
        Me[2 * n_var_dofs + i] += lumped_mass;
      }
      for (Real& m : Me) m *= P.shell_mass_density * P.thickness;
      // Elem::hmin/hmax of the triangle (vertex distances)
      Real hmin = std::numeric_limits<Real>::max(), hmax = 0;
      for (int e = 0; e < 3; ++e) {
        const Real l = (X[tri[3 * eid + e]] - X[tri[3 * eid + (e + 1) % 3]]).size();
        hmin = std::min(hmin, l);
        hmax = std::max(hmax, l);
      }
      const Real avg_stiff = 2 * (K + D / (avg_growth * hmin * hmax)) / 3;
      for (unsigned i = 0; i < Me.size(); ++i) Ce[i] = P.damping_alpha * Me[i] + P.damping_beta * avg_stiff;
#pragma omp critical(oracle_assemble_MC)
      {
        for (int var = 0; var < 3; ++var)
          for (unsigned i = 0; i < n_var_dofs; ++i) {
            Minv[dof(cache.patch[i], var)] += Me[var * n_var_dofs + i];
            C[dof(cache.patch[i], var)] += Ce[var * n_var_dofs + i];
          }
      }
    }
  }
  for (Real& c : C) c += P.damping_gamma;
  for (Real& m : Minv) m = 1 / m;
}

// ShellSystem::build_topological_neighborhood, ShellSystem.C:684-741
void oracle::build_topological_neighborhood() {
  const Real cutoff = (1 + P.neighbor_margin) * P.thickness / std::min(1.0, 1.0);
  const Real cutoff2 = cutoff * cutoff;
#pragma omp parallel for schedule(dynamic, 16)
  for (int eid = 0; eid < (int)F; ++eid) {
    std::set<unsigned> close(ec[eid].neighbor_elems.begin(), ec[eid].neighbor_elems.end());
    std::set<unsigned> added = close;
    do {
      std::set<unsigned> cands;
      for (unsigned ad : added)
        for (unsigned nb : ec[ad].neighbor_elems)
          if (nb != (unsigned)eid) cands.insert(nb);
      added.clear();
      for (unsigned c : cands) {
        Contact ct;
        ct.eid[0] = eid;
        ct.eid[1] = c;
        pair_compute(ct, true);
        if (ct.d2 < cutoff2 && close.find(c) == close.end()) {
          added.insert(c);
          close.insert(c);
        }
      }
    } while (!added.empty());
    ec[eid].close_elems.assign(close.begin(), close.end());
  }
}

// ShellSystem::set_newmark_parameters, ShellSystem.C:744-759, with the bounds of
// ShellSystem.C:306-310 (dt_min at least the machine epsilon, dt_max 0 = none)
void oracle::set_newmark_parameters(Real new_dt) {
  const Real dt_min = std::max(P.dt_min, std::numeric_limits<Real>::epsilon());
  const Real dt_max = P.dt_max <= 0 ? std::numeric_limits<Real>::max() : P.dt_max;
  dt = std::max(new_dt, dt_min);
  dt = std::min(dt, dt_max);
  const Real beta = P.newmark_beta, gamma = P.newmark_gamma;
  newmark_a[0] = beta * dt * dt;
  newmark_a[1] = gamma / (beta * dt);
  newmark_a[2] = 1 / (beta * dt);
  newmark_a[3] = 1 / (2 * beta) - 1;
  newmark_a[4] = gamma / beta - 1;
  newmark_a[5] = dt * (gamma / (2 * beta) - 1);
  newmark_a[6] = (1 - gamma) * dt;
  newmark_a[7] = gamma * dt;
  newmark_a[8] = dt * dt * (0.5 - beta);
  newmark_a[9] = dt * dt * std::fabs(beta - 1. / 6);
}

bool oracle::build(const shl_mesh* m, const shl_params* prm) {
  if (!m || !prm || !m->xyz || !m->faces || m->n_nodes == 0 || m->n_faces == 0) {
    g_err = "empty mesh";
    return false;
  }
  P = *prm;
  V = m->n_nodes;
  F = m->n_faces;
  X.resize(V);
  for (unsigned i = 0; i < V; ++i) X[i] = Point(m->xyz[3 * i], m->xyz[3 * i + 1], m->xyz[3 * i + 2]);
  tri.assign(m->faces, m->faces + 3 * F);
  for (unsigned i = 0; i < 3 * F; ++i)
    if (tri[i] >= V) { g_err = "face index out of range"; return false; }
  nodes_to_elem.assign(V, {});
  for (unsigned e = 0; e < F; ++e)
    for (int k = 0; k < 3; ++k) nodes_to_elem[tri[3 * e + k]].push_back(e);
  valence.assign(V, 0);
  for (unsigned nid = 0; nid < V; ++nid) valence[nid] = (int)nodes_to_elem[nid].size();  // closed mesh
  ec.assign(F, ElemCache());

  const unsigned nd = 3 * V;
  for (auto* vec : {&u, &v, &a, &f, &Minv, &C, &u_pred, &v_pred, &a_pred}) vec->assign(nd, 0.0);
  p = X;

  thickness0 = P.thickness;
  // n_cells_max, ShellSystem.C:279-280 (in 64 bits)
  {
    const uint64_t nc = (uint64_t)std::ceil(std::sqrt((double)F) / P.cell_size_mult);
    n_cells_max = nc * nc * nc;
  }
  vertex_faces.assign(V, {});
  for (unsigned e = 0; e < F; ++e)
    for (int q = 0; q < 3; ++q) vertex_faces[tri[3 * e + q]].push_back(e);
  cav_origin.assign(V, Point());
  set_newmark_parameters(P.dt);
  update_derived();

  bool ok = true;
  for (unsigned e = 0; e < F && ok; ++e) {
    int N;
    ok = build_patch(e, ec[e].patch, N);
  }
  if (!ok) return false;
  if (P.shell_shell_contact == SHL_CONTACT_SMOOTH)
    for (unsigned e = 0; e < F; ++e) {
      const int N = (int)ec[e].patch.size() - 6;
      if (N != 6 && subdiv_tab[N].empty() && !shl_subdiv::build_table(N, subdiv_tab[N])) {
        g_err = "subdivision table of valence " + std::to_string(N);
        return false;
      }
    }
#pragma omp parallel for
  for (int e = 0; e < (int)F; ++e) reinit_mod_and_reference(e);

  if (P.shell_shell_contact != SHL_CONTACT_NONE) {
    for (unsigned e = 0; e < F; ++e) {
      std::set<unsigned> nb;
      for (int k = 0; k < 3; ++k)
        for (unsigned o : nodes_to_elem[tri[3 * e + k]])
          if (o != e) nb.insert(o);
      ec[e].neighbor_elems.assign(nb.begin(), nb.end());
    }
    build_topological_neighborhood();
  }
  compute_mass_damping();
  return true;
}

/* ------------------------------ the step --------------------------------- */

void oracle::compute_position() {
#pragma omp parallel for
  for (int nid = 0; nid < (int)V; ++nid) {
    p[nid] = X[nid];
    for (int var = 0; var < 3; ++var) p[nid](var) += u_pred[dof(nid, var)];
  }
}

void oracle::reset_properties() {
  for (ElemCache& c : ec) c.kGauss = c.kMean = c.etens = c.ebend = 0;
  Nc = 0;
  Eself = Efric = Etens = Ebend = 0;
  Nc_cav = 0;
  Ecav = cavity_force = 0;
  ecav_vec.assign(V, 0.0);
  ekin_vec.assign(V, 0.0);
  eself_vec.assign(V, 0.0);
  efric_vec.assign(V, 0.0);
}

// prepare_next_step, ShellSystem.C:924-949: the only time-dependent parameter
// here is the pressure, whose value at the new time the caller supplies.
void oracle::prepare_next_step(Real p_now) {
  reset_properties();
  time += dt;
  pressure = p_now;
}

void oracle::check_increment(bool require_change) {
  Real du_max = 0;
#pragma omp parallel
  {
    Real du_max_local = 0;
#pragma omp for nowait
    for (int nid = 0; nid < (int)V; ++nid) {
      const Real dx = u_pred[dof(nid, 0)] - u[dof(nid, 0)];
      const Real dy = u_pred[dof(nid, 1)] - u[dof(nid, 1)];
      const Real dz = u_pred[dof(nid, 2)] - u[dof(nid, 2)];
      const Real du = dx * dx + dy * dy + dz * dz;
      du_max_local = std::max(du_max_local, du);
    }
#pragma omp critical(oracle_du_max)
    du_max = std::max(du_max, du_max_local);
  }
  du_max = std::sqrt(du_max);
  if (std::isfinite(du_max)) {
    du_sum += 2 * du_max;
    if (require_change && du_max == 0)
      register_problem(SHL_NO_DISP_CHANGE);
    else if (P.shell_shell_contact != SHL_CONTACT_NONE && du_max > 0.5 * P.thickness)
      register_problem(SHL_LARGE_DISP);
  } else {
    register_problem(SHL_NOT_FINITE);
  }
}

void oracle::compute_bounding_box() {
  for (int c = 0; c < 3; ++c) {
    bounds_min[c] = std::numeric_limits<Real>::max();
    bounds_max[c] = -bounds_min[c];
  }
  std::vector<Real> sizes(F);
  for (unsigned eid = 0; eid < F; ++eid) {
    ElemCache& cache = ec[eid];
    for (int c = 0; c < 3; ++c) {
      cache.bmin[c] = std::numeric_limits<Real>::max();
      cache.bmax[c] = -cache.bmin[c];
    }
    for (int n = 0; n < 3; ++n) {
      const Point& q = p[tri[3 * eid + n]];
      for (int c = 0; c < 3; ++c) {
        if (q(c) < cache.bmin[c]) cache.bmin[c] = q(c);
        if (q(c) > cache.bmax[c]) cache.bmax[c] = q(c);
      }
    }
    for (int c = 0; c < 3; ++c) {
      if (cache.bmin[c] < bounds_min[c]) bounds_min[c] = cache.bmin[c];
      if (cache.bmax[c] > bounds_max[c]) bounds_max[c] = cache.bmax[c];
    }
    // BoundingBox::max_size
    Real dmax = cache.bmax[0] - cache.bmin[0];
    const Real d1 = cache.bmax[1] - cache.bmin[1], d2 = cache.bmax[2] - cache.bmin[2];
    if (d1 > dmax) dmax = d1;
    if (d2 > dmax) dmax = d2;
    sizes[eid] = dmax;
  }
  avg_elem_size = fixed_order_sum(sizes.data(), F) / F;
}

void oracle::compute_deformed_metrics() {
#pragma omp parallel for
  for (int eid = 0; eid < (int)F; ++eid) {
    ElemCache& cache = ec[eid];
    cache.area = 0;
    const SurfaceMetric& a_ref = cache.a_ref;
    SurfaceMetric& a_def = cache.a_def;
    Point uq, dudxi, dudeta, d2udxi2, d2udeta2, d2udxideta;
    for (unsigned i = 0; i < cache.patch.size(); ++i) {
      const unsigned nid = cache.patch[i];
      const Point u_qp(u_pred[dof(nid, 0)], u_pred[dof(nid, 1)], u_pred[dof(nid, 2)]);
      uq.add_scaled(u_qp, cache.phi[i]);
      dudxi.add_scaled(u_qp, cache.dphi[i](0));
      dudeta.add_scaled(u_qp, cache.dphi[i](1));
      d2udxi2.add_scaled(u_qp, cache.d2phi[i](0));
      d2udeta2.add_scaled(u_qp, cache.d2phi[i](1));
      d2udxideta.add_scaled(u_qp, cache.d2phi[i](2));
    }
    a_def.xyz = a_ref.xyz + uq;
    a_def.vec[0] = a_ref.vec[0] + dudxi;
    a_def.vec[1] = a_ref.vec[1] + dudeta;
    a_def.vec[2] = a_def.vec[0].cross(a_def.vec[1]);
    a_def.jac = a_def.vec[2].size();
    a_def.vec[2] *= 1 / a_def.jac;
    a_def.dvec[0] = a_ref.dvec[0] + d2udxi2;
    a_def.dvec[1] = a_ref.dvec[1] + d2udeta2;
    a_def.dvec[2] = a_ref.dvec[2] + d2udxideta;
    a_def.ff1(0) = a_def.vec[0] * a_def.vec[0];
    a_def.ff1(1) = a_def.vec[1] * a_def.vec[1];
    a_def.ff1(2) = a_def.vec[0] * a_def.vec[1];
    a_def.ff2(0) = a_def.dvec[0] * a_def.vec[2];
    a_def.ff2(1) = a_def.dvec[1] * a_def.vec[2];
    a_def.ff2(2) = a_def.dvec[2] * a_def.vec[2];
    cache.area += qw * a_def.jac;
  }
}

void oracle::compute_external_force() {
  std::fill(f.begin(), f.end(), 0.0);
  const Real volume_growth_red = std::max((1.0 - static_cast<int>(time * 5.0) * 0.01), 0.5);
  if (time_step == 2) volume0 = volume;
  const Real volume_pressure =
      (P.bulk_modulus == 0 ? 0 : P.bulk_modulus * (volume0 * volume_growth_red / volume - 1));
  if (P.compat_zero_pressure) pressure *= 0.0;  // ShellSystem.C:1480, fulltime == 0
  if (pressure != 0 || volume_pressure != 0) {
#pragma omp parallel
    {
      std::vector<Real> qe;
#pragma omp for
      for (int eid = 0; eid < (int)F; ++eid) {
        const ElemCache& cache = ec[eid];
        const unsigned n_var_dofs = (unsigned)cache.patch.size();
        qe.assign(3 * n_var_dofs, 0.0);
        const SurfaceMetric& a_def = cache.a_def;
        Point pressure_vec;
        if (pressure != 0) {
          switch (P.pressure_base) {
            case SHL_CS_LOCAL: pressure_vec = a_def.vec[2]; break;
            case SHL_CS_CARTESIAN: pressure_vec(P.pressure_dir) = 1; break;
            case SHL_CS_CYLINDRICAL:
              if (P.pressure_dir == 0)
                pressure_vec(0) = 1;
              else {
                const Real inv_r = 1 / std::sqrt(a_def.xyz(1) * a_def.xyz(1) + a_def.xyz(2) * a_def.xyz(2));
                if (std::isfinite(inv_r)) {
                  pressure_vec(1) = inv_r * a_def.xyz(1);
                  pressure_vec(2) = inv_r * a_def.xyz(2);
                }
              }
              break;
            case SHL_CS_SPHERICAL: {
              pressure_vec = a_def.xyz;
              const Real radius = pressure_vec.size();
              if (radius > 0)
                pressure_vec *= 1 / radius;
              else
                pressure_vec.zero();
              break;
            }
            default: break;
          }
          pressure_vec *= pressure;
        }
        if (volume_pressure != 0) pressure_vec.add_scaled(a_def.vec[2], volume_pressure);
        for (unsigned i = 0; i < n_var_dofs; ++i) {
          const Real prefactor = cache.JxW * cache.phi[i];
          qe[i] += prefactor * pressure_vec(0);
          qe[n_var_dofs + i] += prefactor * pressure_vec(1);
          qe[2 * n_var_dofs + i] += prefactor * pressure_vec(2);
        }
#pragma omp critical(oracle_assemble_vec)
        for (int var = 0; var < 3; ++var)
          for (unsigned i = 0; i < n_var_dofs; ++i) f[dof(cache.patch[i], var)] += qe[var * n_var_dofs + i];
      }
    }
  }
  if (P.shell_cavity_contact) add_cavity_force();
  if (P.shell_shell_contact != SHL_CONTACT_NONE) add_shell_shell_contact_force();
}

// interaction with the cavity, ShellSystem.C:1600-1723, with update_derived's
// cavity quantities (421-436) at the current semi-axes
void oracle::add_cavity_force() {
  for (int c = 0; c < 3; ++c)
    cav_R[c] = has_rfun[c] ? rfun[c].eval({{"t", time}, {"d", 0.0}}) : (c == 0 ? P.Rx : c == 1 ? P.Ry : P.Rz);
  const Real h_half = 0.5 * P.thickness;
  const Real Rx_eff = cav_R[0] - h_half, Ry_eff = cav_R[1] - h_half, Rz_eff = cav_R[2] - h_half;
  const Real avg_R_eff = (Rx_eff + Ry_eff + Rz_eff) / 3;
  const Real inv_R2_eff[3] = {1 / (Rx_eff * Rx_eff), 1 / (Ry_eff * Ry_eff), 1 / (Rz_eff * Rz_eff)};
  const Real one_plus_delta_friction = std::pow(1 - P.static_friction_tol * P.thickness / avg_R_eff, 2);
  const bool cavity_friction = P.mu_s_cavity != 0 || P.mu_d_cavity != 0;
  unsigned Nc_cav_sum = 0;
  Real Efric_sum = 0, Ecav_sum = 0, cavity_force_sum = 0;
  if (cav_origin.size() != V) cav_origin.assign(V, Point());
#pragma omp parallel for reduction(+ : Nc_cav_sum, Efric_sum, Ecav_sum, cavity_force_sum)
  for (int nid = 0; nid < (int)V; ++nid) {
    const Point& pp = p[nid];
    Real x_red = pp(0) / Rx_eff, y_red = pp(1) / Ry_eff, z_red = pp(2) / Rz_eff;
    x_red = x_red * x_red;
    y_red = y_red * y_red;
    z_red = z_red * z_red;
    Real one_plus_delta;  // cavity_isoparameter, ShellSystem.h:336-362
    if (P.cavity == SHL_CAVITY_BOX)
      one_plus_delta = std::max(x_red, std::max(y_red, z_red));
    else if (P.cavity == SHL_CAVITY_CYLINDER)
      one_plus_delta = std::max(x_red, y_red + z_red);
    else
      one_plus_delta = x_red + y_red + z_red;
    if (one_plus_delta > one_plus_delta_friction) {
      const Real depth = avg_R_eff * (std::sqrt(one_plus_delta) - 1);
      Real area_node = 0;  // avg_area_node, ShellSystem.C:2462-2481
      for (unsigned e : vertex_faces[nid]) area_node += ec[e].area;
      area_node /= vertex_faces[nid].size();
      const Real stiffness = stiff_density * area_node;
      Real f_normal = 0;
      if (depth > 0) {
        ++Nc_cav_sum;
        const Real Ecav_node = 0.5 * stiffness * depth * depth;
        Ecav_sum += Ecav_node;
        ecav_vec[nid] += Ecav_node / area_node;
        f_normal = stiffness * depth;
        cavity_force_sum += f_normal;
      }
      Point n;
      const Real xr = pp(0) * pp(0) * inv_R2_eff[0], yr = pp(1) * pp(1) * inv_R2_eff[1],
                 zr = pp(2) * pp(2) * inv_R2_eff[2];
      auto sgn = [](Real x) { return (Real)((x > 0) - (x < 0)); };
      if (P.cavity == SHL_CAVITY_BOX) {
        if (xr > yr && xr > zr)
          n(0) = sgn(pp(0));
        else if (yr > zr)
          n(1) = sgn(pp(1));
        else
          n(2) = sgn(pp(2));
      } else if (P.cavity == SHL_CAVITY_CYLINDER) {
        if (xr > yr + zr) {
          n(0) = sgn(pp(0));
        } else {
          n(1) = pp(1) * inv_R2_eff[1];
          n(2) = pp(2) * inv_R2_eff[2];
        }
      } else {
        n(0) = pp(0) * inv_R2_eff[0];
        n(1) = pp(1) * inv_R2_eff[1];
        n(2) = pp(2) * inv_R2_eff[2];
      }
      n = n * (1 / n.size());
      const Point vel(v[dof(nid, 0)], v[dof(nid, 1)], v[dof(nid, 2)]);
      const Real abs_v_normal = vel * n;
      Point f_contact;
      if (cavity_friction) {
        Real Efric_node = 0;
        bool stick = cav_origin[nid].size_sq() != 0;
        friction_apply(Efric_node, f_contact, f_normal, n, vel, abs_v_normal, P.friction_stop_velocity,
                       stiff_static_friction, P.mu_s_cavity, P.mu_d_cavity, P.cavity_friction_damping, stick,
                       cav_origin[nid], pp);
        Efric_sum += Efric_node;
        efric_vec[nid] += Efric_node / area_node;
      }
      f_normal += P.cavity_damping * stiffness * abs_v_normal;
      f_contact -= f_normal * n;
      f[dof(nid, 0)] += f_contact(0);
      f[dof(nid, 1)] += f_contact(1);
      f[dof(nid, 2)] += f_contact(2);
    } else {
      cav_origin[nid].zero();
    }
  }
  Nc_cav += Nc_cav_sum;
  Efric += Efric_sum;
  Ecav += Ecav_sum;
  cavity_force += cavity_force_sum;
}

void oracle::add_shell_shell_contact_force() {
  unsigned Nc_sum = 0;
  Real Efric_sum = 0, Eself_sum = 0;
  const bool self_friction = (P.mu_s != 0 || P.mu_d != 0);
  const Real h = P.thickness;
#pragma omp parallel for reduction(+ : Nc_sum, Efric_sum, Eself_sum)
  for (int i = 0; i < (int)candidates.size(); ++i) {
    Contact* contact = candidates[i];
    if (!contact) continue;
    pair_compute(*contact, false);
    if (contact->d2 <= 0) {
#pragma omp critical(oracle_problem)
      register_problem(SHL_CONTACT_PROBLEM);
    }
    if (contact->d2 < d2_friction) {
      const Real area1 = ec[contact->eid[0]].area, area2 = ec[contact->eid[1]].area;
      const Real area_min = std::min(area1, area2);
      const Real abs_dc = std::sqrt(contact->d2);
      const Real depth = h - abs_dc;
      const Point n = contact->dc / abs_dc;
      const Real stiffness = stiff_density * area_min;
      Real f_normal = 0;
      Real Eself_contact = 0, Efric_contact = 0;
      if (depth > 0) {
        ++Nc_sum;
        f_normal = stiffness * (h - abs_dc) * 0.5 * (1 + h / abs_dc);  // ShellSystem.h:387-393
        const Real dep = h - abs_dc;  // ShellSystem.h:396-401
        Eself_contact = 0.5 * stiffness * (0.5 * dep * dep - dep * h + h * h * std::log(h / abs_dc));
      }
      Eself_sum += Eself_contact;
      Point vn[2][3];
      for (int e = 0; e < 2; ++e)
        for (int k = 0; k < 3; ++k) {
          const unsigned nid = tri[3 * contact->eid[e] + k];
          vn[e][k] = Point(v[dof(nid, 0)], v[dof(nid, 1)], v[dof(nid, 2)]);
        }
      const Real uu[2] = {1 - contact->v[0] - contact->w[0], 1 - contact->v[1] - contact->w[1]};
      const Point v_rel = uu[1] * vn[1][0] + contact->v[1] * vn[1][1] + contact->w[1] * vn[1][2] -
                          (uu[0] * vn[0][0] + contact->v[0] * vn[0][1] + contact->w[0] * vn[0][2]);
      const Real abs_v_normal = v_rel * n;
      Point f_contact;
      if (self_friction) {
        bool stick = contact->stick;
        const Point cp = contact_point(*contact);
        friction_apply(Efric_contact, f_contact, f_normal, n, v_rel, abs_v_normal, P.friction_stop_velocity,
                       stiff_static_friction, P.mu_s, P.mu_d, P.self_friction_damping, stick,
                       contact->spring_origin, cp);
        contact->stick = stick;
        Efric_sum += Efric_contact;
      }
      f_normal -= P.self_damping * stiffness * abs_v_normal;
      f_contact += f_normal * n;
#pragma omp critical(oracle_assemble_vec)
      for (int e = 0; e < 2; ++e) {
        const Real vv = contact->v[e], ww = contact->w[e], u0 = 1 - vv - ww;
        // energy densities, ShellSystem.C:1862-1877
        const Real pre[3] = {0.5 * u0 / area_min, 0.5 * vv / area_min, 0.5 * ww / area_min};
        for (int k = 0; k < 3; ++k) {
          eself_vec[tri[3 * contact->eid[e] + k]] += pre[k] * Eself_contact;
          efric_vec[tri[3 * contact->eid[e] + k]] += pre[k] * Efric_contact;
        }
        const Real prefactor = (e == 0 ? -0.5 : 0.5);
        for (int var = 0; var < 3; ++var) {
          const Real fc = prefactor * f_contact(var);
          f[dof(tri[3 * contact->eid[e] + 0], var)] += u0 * fc;
          f[dof(tri[3 * contact->eid[e] + 1], var)] += vv * fc;
          f[dof(tri[3 * contact->eid[e] + 2], var)] += ww * fc;
        }
      }
    } else {
      contact->spring_origin.zero();
      contact->stick = false;
    }
  }
  Nc += Nc_sum;
  Efric += Efric_sum;
  Eself += Eself_sum;
}

void oracle::subtract_internal_force() {
  Real Etens_sum = 0, Ebend_sum = 0;
  const Real E1 = P.shell_young_modulus, E2 = P.shell_young_modulus2, nu = P.shell_poisson_ratio,
             G12 = P.shell_shear_modulus;
#pragma omp parallel reduction(+ : Etens_sum, Ebend_sum)
  {
    std::vector<Real> qe;
    Tensor BmT, BbT;
    Point n, m, p11, p21, p12, p22, p13, p23, column, a2xa3, a3xa1, fint_density;
#pragma omp for
    for (int eid = 0; eid < (int)F; ++eid) {
      ElemCache& cache = ec[eid];
      const unsigned n_var_dofs = (unsigned)cache.patch.size();
      qe.assign(3 * n_var_dofs, 0.0);
      Real Etens_elem = 0, Ebend_elem = 0;
      const Real JxW = cache.JxW;
      const SurfaceMetric& a_ref = cache.a_ref;
      const SurfaceMetric& a_def = cache.a_def;
      Point& alpha = cache.alpha;
      Point& beta = cache.beta;
      alpha = 0.5 * (a_def.ff1 - a_ref.ff1);
      beta = a_ref.ff2 - a_def.ff2;
      alpha(2) *= 2;
      beta(2) *= 2;
      Tensor& H = cache.H;
      const Real nu2 = (E1 * nu) / E2;  // ShellSystem.C:1199
      H(0, 0) = E1 * a_ref.ff1(1) * a_ref.ff1(1);
      H(0, 1) = H(1, 0) = E1 * (nu * a_ref.ff1(1) * a_ref.ff1(0) + (1 - nu) * a_ref.ff1(2) * a_ref.ff1(2));
      H(0, 2) = H(2, 0) = E1 * -a_ref.ff1(1) * a_ref.ff1(2);
      H(1, 1) = E2 * a_ref.ff1(0) * a_ref.ff1(0);
      H(1, 2) = H(2, 1) = E2 * -a_ref.ff1(0) * a_ref.ff1(2);
      H(2, 2) = G12 * ((1 - nu * nu2) * a_ref.ff1(1) * a_ref.ff1(0) +
                       (1 - nu * nu2) * ((1 + nu) / (1 - nu)) * a_ref.ff1(2) * a_ref.ff1(2));
      const Real invdet = 1 / (a_ref.ff1(0) * a_ref.ff1(1) - a_ref.ff1(2) * a_ref.ff1(2));
      for (int r = 0; r < 3; ++r)
        for (int q = 0; q < 3; ++q) H(r, q) *= invdet * invdet;
      n = K * (H * alpha);
      m = D * (H * beta);
      a2xa3 = a_def.vec[1].cross(a_def.vec[2]);
      a3xa1 = a_def.vec[2].cross(a_def.vec[0]);
      const Real invjac = 1 / a_def.jac;
      p11 = invjac * (a_def.dvec[0].cross(a_def.vec[1]) + a_def.ff2(0) * a2xa3);
      p12 = invjac * (a_def.dvec[1].cross(a_def.vec[1]) + a_def.ff2(1) * a2xa3);
      p13 = invjac * (a_def.dvec[2].cross(a_def.vec[1]) + a_def.ff2(2) * a2xa3);
      p21 = invjac * (a_def.vec[0].cross(a_def.dvec[0]) + a_def.ff2(0) * a3xa1);
      p22 = invjac * (a_def.vec[0].cross(a_def.dvec[1]) + a_def.ff2(1) * a3xa1);
      p23 = invjac * (a_def.vec[0].cross(a_def.dvec[2]) + a_def.ff2(2) * a3xa1);
      for (unsigned i = 0; i < n_var_dofs; ++i) {
        const Point& dphi = cache.dphi[i];
        const Point& d2phi = cache.d2phi[i];
        column = a_def.vec[0] * dphi(0);
        BmT(0, 0) = column(0); BmT(1, 0) = column(1); BmT(2, 0) = column(2);
        column = a_def.vec[1] * dphi(1);
        BmT(0, 1) = column(0); BmT(1, 1) = column(1); BmT(2, 1) = column(2);
        column = a_def.vec[0] * dphi(1) + a_def.vec[1] * dphi(0);
        BmT(0, 2) = column(0); BmT(1, 2) = column(1); BmT(2, 2) = column(2);
        column = a_def.vec[2] * -d2phi(0) + (dphi(0) * p11 + dphi(1) * p21);
        BbT(0, 0) = column(0); BbT(1, 0) = column(1); BbT(2, 0) = column(2);
        column = a_def.vec[2] * -d2phi(1) + (dphi(0) * p12 + dphi(1) * p22);
        BbT(0, 1) = column(0); BbT(1, 1) = column(1); BbT(2, 1) = column(2);
        column = 2 * (a_def.vec[2] * -d2phi(2) + (dphi(0) * p13 + dphi(1) * p23));
        BbT(0, 2) = column(0); BbT(1, 2) = column(1); BbT(2, 2) = column(2);
        fint_density = BmT * n + BbT * m;
        qe[i] += JxW * fint_density(0);
        qe[n_var_dofs + i] += JxW * fint_density(1);
        qe[2 * n_var_dofs + i] += JxW * fint_density(2);
      }
      Etens_elem += 0.5 * JxW * (n * alpha);
      Ebend_elem += 0.5 * JxW * (m * beta);
      Etens_sum += Etens_elem;
      Ebend_sum += Ebend_elem;
      cache.etens = Etens_elem / cache.area;
      cache.ebend = Ebend_elem / cache.area;
#pragma omp critical(oracle_assemble_vec)
      for (int var = 0; var < 3; ++var)
        for (unsigned i = 0; i < n_var_dofs; ++i) f[dof(cache.patch[i], var)] -= qe[var * n_var_dofs + i];
    }
  }
  Etens += Etens_sum;
  Ebend += Ebend_sum;
}

void oracle::compute_shell_shell_contact_candidates(bool force) {
  if (P.shell_shell_contact == SHL_CONTACT_NONE) return;
  Real cell_size = P.cell_size_mult * avg_elem_size;
  Real tolerance = P.cell_margin * cell_size;
  if (!(force || du_sum >= tolerance)) return;
  ++n_rebuilds;
  du_sum = 0;
  compute_bounding_box();
  cell_size = P.cell_size_mult * avg_elem_size;
  tolerance = P.cell_margin * cell_size;
  cell_size += tolerance;
  Real d_max = P.thickness + tolerance;
  // SMOOTH: the limit surfaces may be closer than the facets (ShellSystem.C:1940-1944)
  if (P.shell_shell_contact == SHL_CONTACT_SMOOTH) d_max += avg_elem_size;
  const Real d2_max = d_max * d_max;
  last_cell_size = cell_size;
  last_d_max = d_max;
  unsigned n_cells_dir[3];
  for (int c = 0; c < 3; ++c)
    n_cells_dir[c] = static_cast<int>(((bounds_max[c] - bounds_min[c]) + d_max) / cell_size + 1);
  const uint64_t n_cells = (uint64_t)n_cells_dir[0] * n_cells_dir[1] * n_cells_dir[2];
  if (n_cells > n_cells_max) {
    register_problem(SHL_TOO_MANY_CELLS);
    return;
  }
  std::vector<std::vector<unsigned>> elem_to_cell_map(F);
  std::vector<std::vector<unsigned>> cell_to_elem_map(n_cells);
  for (unsigned eid = 0; eid < F; ++eid) {
    const ElemCache& cache = ec[eid];
    int lo[3], hi[3];
    for (int var = 0; var < 3; ++var) {
      lo[var] = static_cast<int>((cache.bmin[var] - bounds_min[var]) / cell_size);
      hi[var] = static_cast<int>((cache.bmax[var] - bounds_min[var] + d_max) / cell_size);
    }
    for (int cx = lo[0]; cx <= hi[0]; ++cx)
      for (int cy = lo[1]; cy <= hi[1]; ++cy)
        for (int cz = lo[2]; cz <= hi[2]; ++cz) {
          const unsigned c = cx * n_cells_dir[1] * n_cells_dir[2] + cy * n_cells_dir[2] + cz;
          elem_to_cell_map[eid].push_back(c);
          cell_to_elem_map[c].push_back(eid);
        }
  }
  unsigned first_empty = (unsigned)candidates.size();
  for (unsigned i = 0; i < candidates.size(); ++i) {
    Contact* contact = candidates[i];
    if (contact && !contact->stick && contact->d2 > d2_max) {
      ec[contact->eid[0]].in_contact_with.remove(contact->eid[1]);
      delete contact;
      candidates[i] = nullptr;
      first_empty = std::min(first_empty, i);
    }
  }
  // candidates of each eid1 in discovery order (the searches are independent per
  // eid1; the reference runs this loop with OpenMP too), then added to the list
  // in eid1 order exactly as the serial loop would
  std::vector<std::vector<Contact*>> found(F);
#pragma omp parallel for schedule(dynamic, 8)
  for (int e1i = 0; e1i < (int)F; ++e1i) {
    const unsigned eid1 = (unsigned)e1i;
    const std::vector<unsigned>& cells = elem_to_cell_map[eid1];
    for (unsigned cidx = 0; cidx < cells.size(); ++cidx) {
      const std::vector<unsigned>& elems_in_cell = cell_to_elem_map[cells[cidx]];
      for (unsigned i = 0; i < elems_in_cell.size(); ++i) {
        const unsigned eid2 = elems_in_cell[i];
        if (eid1 >= eid2) continue;
        if (elems_are_close(eid1, eid2)) continue;
        const std::list<unsigned>& lst = ec[eid1].in_contact_with;
        if (std::find(lst.begin(), lst.end(), eid2) != lst.end()) continue;
        const ElemCache& c1 = ec[eid1];
        const ElemCache& c2 = ec[eid2];
        bool apart = false;
        for (int c = 0; c < 3; ++c)
          apart = apart || c1.bmin[c] > c2.bmax[c] + d_max || c2.bmin[c] > c1.bmax[c] + d_max;
        if (apart) continue;
        Contact* cand = new Contact;
        cand->eid[0] = eid1;
        cand->eid[1] = eid2;
        pair_compute(*cand, false);
        if (cand->d2 <= 0) {
#pragma omp critical(oracle_problem)
          register_problem(SHL_CONTACT_PROBLEM);
        }
        if (cand->d2 > d2_max) {
          delete cand;
          continue;
        }
        found[eid1].push_back(cand);
        ec[eid1].in_contact_with.push_back(eid2);
      }
    }
  }
  for (unsigned eid1 = 0; eid1 < F; ++eid1)
    for (Contact* cand : found[eid1]) {
      if (first_empty == candidates.size()) {
        ++first_empty;
        candidates.push_back(cand);
      } else {
        candidates[first_empty] = cand;
        auto it = std::find(candidates.begin() + first_empty + 1, candidates.end(), (Contact*)nullptr);
        first_empty = (unsigned)(it - candidates.begin());
      }
    }
}

void oracle::compute_enclosed_volume() {
  Real area_sum = 0, volume_sum = 0;
#pragma omp parallel for reduction(+ : area_sum, volume_sum)
  for (int eid = 0; eid < (int)F; ++eid) {
    const Point& q0 = p[tri[3 * eid]];
    const Point& q1 = p[tri[3 * eid + 1]];
    const Point& q2 = p[tri[3 * eid + 2]];
    // det of the triad with the node positions as columns (libMesh TypeTensor::det)
    const Real det = q0(0) * (q1(1) * q2(2) - q2(1) * q1(2)) - q1(0) * (q0(1) * q2(2) - q2(1) * q0(2)) +
                     q2(0) * (q0(1) * q1(2) - q1(1) * q0(2));
    area_sum += ec[eid].area;
    volume_sum += det;
  }
  area = area_sum;
  volume = std::fabs(volume_sum / 6) - area * 0.5 * P.thickness;
}

void oracle::measure_properties() {
  Real kG = 0, kM = 0, area_sum = 0;
#pragma omp parallel for reduction(+ : kG, kM, area_sum)
  for (int eid = 0; eid < (int)F; ++eid) {
    ElemCache& cache = ec[eid];
    const Point& ff1 = cache.a_def.ff1;
    const Point& ff2 = cache.a_def.ff2;
    const Real w = cache.a_def.jac * qw;
    const Real invdet = 1 / (ff1(0) * ff1(1) - ff1(2) * ff1(2));
    const Real kGauss_elem = w * invdet * (ff2(0) * ff2(1) - ff2(2) * ff2(2));
    const Real kMean_elem = w * invdet * 0.5 * (ff2(0) * ff1(1) + ff2(1) * ff1(0) - 2 * ff2(2) * ff1(2));
    kG += kGauss_elem;
    kM += kMean_elem;
    cache.kGauss = kGauss_elem / cache.area;
    cache.kMean = kMean_elem / cache.area;
    area_sum += cache.area;
  }
  kGauss = kG;
  kMean = kM;
  area = area_sum;
  // mean area of the faces around each node, avg_area_node (ShellSystem.C:2462-2481)
  std::vector<Real> node_area(V, 0.0);
  std::vector<unsigned> node_faces(V, 0);
  for (unsigned e = 0; e < F; ++e)
    for (int k = 0; k < 3; ++k) {
      node_area[tri[3 * e + k]] += ec[e].area;
      ++node_faces[tri[3 * e + k]];
    }
  if (ekin_vec.size() != V) ekin_vec.assign(V, 0.0);
  Real ek = 0;
#pragma omp parallel for reduction(+ : ek)
  for (int nid = 0; nid < (int)V; ++nid) {
    Real e = 0;
    for (int var = 0; var < 3; ++var) {
      const unsigned d = dof(nid, var);
      e += v[d] * v[d] / Minv[d];
    }
    ek += 0.5 * e;
    ekin_vec[nid] += 0.5 * e / (node_area[nid] / node_faces[nid]);
  }
  Ekin = ek;
  if (!std::isfinite(Ekin)) register_problem(SHL_NOT_FINITE);
  compute_enclosed_volume();
}

// advance(), ShellSystem.C:952-1122: predictor, forces, and with adaptive dt
// the local-error estimate (1010-1044) that repeats the step with a smaller dt
// (1104-1117).  p_at(time) gives the pressure of an attempt at its time.
// Returns true when the run must stop; dt_step is the dt of the accepted step.
template <class PressureAt>
bool oracle::advance(const PressureAt& p_at) {
  const bool adapt_now = P.adapt_dt_every && time_step % P.adapt_dt_every == 0;
  const Real target = std::sqrt(P.rel_loc_err_min * P.rel_loc_err_max);
  accepted = false;
  while (true) {
    prepare_next_step(p_at(time + dt));
    // predictor (972-989)
    for (unsigned i = 0; i < 3 * V; ++i) {
      u_pred[i] = u[i];
      u_pred[i] = dt * v[i] + u_pred[i];
      u_pred[i] = newmark_a[8] * a[i] + u_pred[i];
    }
    check_increment(false);
    compute_position();
    for (unsigned i = 0; i < 3 * V; ++i) {
      v_pred[i] = v[i];
      v_pred[i] = newmark_a[6] * a[i] + v_pred[i];
    }
    compute_shell_shell_contact_candidates(false);
    compute_deformed_metrics();
    compute_external_force();
    subtract_internal_force();
    for (unsigned i = 0; i < 3 * V; ++i) {
      a_pred[i] = C[i] * v_pred[i];
      f[i] -= a_pred[i];
      a_pred[i] = Minv[i] * f[i];
    }
    Real new_dt = dt;
    if (adapt_now) {
      // Zienkiewicz-Xie local error with the thickness as reference length (1010-1044)
      Real norm_a = 0, vmax = 0;
      for (unsigned i = 0; i < 3 * V; ++i) {
        norm_a = std::max(norm_a, std::fabs(a_pred[i] - a[i]));
        vmax = std::max(vmax, std::fabs(v_pred[i]));
      }
      Real rel_loc_err = target;
      if (std::isfinite(norm_a))
        rel_loc_err = newmark_a[9] * norm_a / P.thickness;
      else
        register_problem(SHL_NOT_FINITE);
      if (rel_loc_err == 0)
        new_dt = 2 * dt;
      else if (rel_loc_err > P.rel_loc_err_max || rel_loc_err < P.rel_loc_err_min)
        new_dt = dt * std::pow(target / rel_loc_err, 1. / 3);
      if (P.shell_shell_contact != SHL_CONTACT_NONE) {
        const unsigned contact_resolution = 10;
        if (new_dt * vmax * contact_resolution * 2 > P.thickness) new_dt = P.thickness / (2 * contact_resolution * vmax);
      }
    }
    if (new_dt >= dt) {
      // accept (1046-1101)
      for (unsigned i = 0; i < 3 * V; ++i) u_pred[i] = newmark_a[0] * a_pred[i] + u_pred[i];
      check_increment(true);
      compute_position();
      u.swap(u_pred);
      for (unsigned i = 0; i < 3 * V; ++i) v_pred[i] = newmark_a[7] * a_pred[i] + v_pred[i];
      v.swap(v_pred);
      a.swap(a_pred);
      compute_shell_shell_contact_candidates(false);
      measure_properties();
      dt_step = dt;
      accepted = true;
      set_newmark_parameters(new_dt);
      break;
    }
    // repeat the step (1104-1117)
    time -= dt;
    set_newmark_parameters(new_dt);
    ++rejections;
    if (dt <= std::numeric_limits<Real>::epsilon()) {
      register_problem(SHL_SMALL_TIMESTEP);
      break;
    }
  }
  return current_problem >= SHL_STOP_SIM || (P.stop_on_problem && current_problem > 0);
}

/* ------------------------------ C interface ------------------------------ */

extern "C" {

const char* oracle_error(void) { return g_err.c_str(); }

void oracle_set_threads(int n) {
#ifdef _OPENMP
  omp_set_num_threads(n > 0 ? n : 1);
#else
  (void)n;
#endif
}

oracle* oracle_create(const shl_mesh* mesh, const shl_params* params) {
  oracle* o = new oracle;
  if (!o->build(mesh, params)) {
    delete o;
    return nullptr;
  }
  return o;
}

void oracle_destroy(oracle* o) { delete o; }

int oracle_apply_initial_conditions(oracle* o, const double* u0, double t0, double pressure_next) {
  const unsigned nd = 3 * o->V;
  std::copy(u0, u0 + nd, o->u.begin());
  std::fill(o->v.begin(), o->v.end(), 0.0);
  std::fill(o->a.begin(), o->a.end(), 0.0);
  o->time = t0;
  o->u_pred = o->u;
  o->compute_position();
  o->reset_properties();
  o->compute_bounding_box();
  o->compute_deformed_metrics();
  o->compute_enclosed_volume();
  o->volume0 = o->volume;
  o->compute_shell_shell_contact_candidates(true);
  const Real old_time = o->time;
  const unsigned old_step = o->time_step;
  ++o->time_step;
  o->prepare_next_step(pressure_next);
  o->compute_external_force();
  o->subtract_internal_force();
  for (unsigned i = 0; i < nd; ++i) o->a[i] = o->Minv[i] * o->f[i];
  o->time = old_time;
  o->time_step = old_step;
  return o->current_problem;
}

int oracle_set_state(oracle* o, const double* u, const double* v, const double* a) {
  const unsigned nd = 3 * o->V;
  if (u) { std::copy(u, u + nd, o->u.begin()); std::copy(u, u + nd, o->u_pred.begin()); }
  if (v) std::copy(v, v + nd, o->v.begin());
  if (a) std::copy(a, a + nd, o->a.begin());
  o->compute_position();
  return 0;
}

int oracle_get_state(oracle* o, double* u, double* v, double* a) {
  if (u) std::copy(o->u.begin(), o->u.end(), u);
  if (v) std::copy(o->v.begin(), o->v.end(), v);
  if (a) std::copy(o->a.begin(), o->a.end(), a);
  return 0;
}

int oracle_set_time(oracle* o, double t, uint32_t step) {
  o->time = t;
  o->time_step = step;
  return 0;
}

int oracle_get_time(oracle* o, double* t, uint32_t* step) {
  if (t) *t = o->time;
  if (step) *step = o->time_step;
  return 0;
}

static void fill_energies(const oracle* o, shl_energies* e) {
  if (!e) return;
  e->Etens = o->Etens; e->Ebend = o->Ebend; e->Eself = o->Eself; e->Efric = o->Efric;
  e->Ekin = o->Ekin; e->area = o->area; e->volume = o->volume;
  e->kGauss = o->kGauss; e->kMean = o->kMean; e->Nc = o->Nc; e->Ecav = o->Ecav; e->cavity_force = o->cavity_force; e->Nc_cav = o->Nc_cav;
  unsigned n = 0;
  for (const Contact* c : o->candidates) n += c != nullptr;
  e->n_pairs = n;
}

int oracle_eval_forces(oracle* o, const double* u_pred, const double* v_pred, double pressure,
                       double* f_out, double* a_out, shl_energies* e) {
  const unsigned nd = 3 * o->V;
  o->current_problem = 0;
  std::copy(u_pred, u_pred + nd, o->u_pred.begin());
  std::copy(v_pred, v_pred + nd, o->v_pred.begin());
  o->reset_properties();
  o->pressure = pressure;
  o->compute_position();
  o->compute_shell_shell_contact_candidates(false);
  o->compute_deformed_metrics();
  o->compute_external_force();
  o->subtract_internal_force();
  if (f_out) std::copy(o->f.begin(), o->f.end(), f_out);
  if (a_out)
    for (unsigned i = 0; i < nd; ++i) a_out[i] = o->Minv[i] * (o->f[i] - o->C[i] * o->v_pred[i]);
  Real area = 0;
  for (const ElemCache& c : o->ec) area += c.area;
  o->area = area;
  fill_energies(o, e);
  return o->current_problem;
}

// cavity surface, ShellSystem.C:441-468
static Real cavity_surface(const Real* R, int type) {
  const Real Rx = R[0], Ry = R[1], Rz = R[2];
  const Real pi = 3.141592653589793238;
  if (type == SHL_CAVITY_BOX) return 8 * (Rx * Ry + Rx * Rz + Ry * Rz);
  if (type == SHL_CAVITY_CYLINDER) {
    const Real lambda = (Ry - Rz) / (Ry + Rz);
    const Real lambda32 = 3 * lambda * lambda;
    return 2 * pi * ((Ry + Rz) * (1 + lambda32 / (10 + std::sqrt(4 - lambda32))) + Ry * Rz);
  }
  return 4 * pi * std::pow((std::pow(Rx * Ry, 1.6) + std::pow(Rx * Rz, 1.6) + std::pow(Ry * Rz, 1.6)) / 3, 0.625);
}

int oracle_step(oracle* o, uint32_t n_steps, const double* pressure_table, shl_step_report* r) {
  shl_step_report rep;
  std::memset(&rep, 0, sizeof(rep));
  int worst = 0;
  uint32_t done = 0;
  const uint64_t rej0 = o->rejections, reb0 = o->n_rebuilds;
  for (uint32_t s = 0; s < n_steps; ++s) {
    o->current_problem = 0;
    ++o->time_step;
    // the pressure of an attempt: the expression at its time, else the step's table entry
    const double p_tab = pressure_table ? pressure_table[s] : o->P.pressure;
    const bool stop = o->advance([&](double t) {
      return o->has_pfun ? o->pfun.eval({{"t", t}, {"d", 0.0}}) : p_tab;
    });
    worst = std::max(worst, o->current_problem);
    if (o->accepted) {
      ++done;
      const Real dt = o->dt_step;
      rep.sum_dt += dt;
      rep.sum_area += dt * o->area;
      rep.sum_volume += dt * o->volume;
      rep.sum_Nc += dt * o->Nc;
      rep.sum_Ekin += dt * o->Ekin;
      rep.sum_Etens += dt * o->Etens;
      rep.sum_Ebend += dt * o->Ebend;
      rep.sum_Eself += dt * o->Eself;
      rep.sum_Efric += dt * o->Efric;
      rep.sum_kGauss += dt * o->kGauss;
      rep.sum_kMean += dt * o->kMean;
      if (o->P.shell_cavity_contact) {
        rep.sum_pcav += dt * o->cavity_force / cavity_surface(o->cav_R, o->P.cavity);
        rep.sum_Nc_cav += dt * o->Nc_cav;
        rep.sum_Ecav += dt * o->Ecav;
      }
    } else {
      --o->time_step;
    }
    if (stop) break;
  }
  rep.steps_done = done;
  rep.rejections = (uint32_t)(o->rejections - rej0);
  rep.n_rebuilds = (uint32_t)(o->n_rebuilds - reb0);
  rep.worst_problem = worst;
  rep.time = o->time;
  rep.du_sum = o->du_sum;
  fill_energies(o, &rep.last);
  if (r) *r = rep;
  return worst;
}

int oracle_set_pressure_function(oracle* o, const char* expr) {
  if (!expr || !*expr) {
    o->has_pfun = false;
    return 0;
  }
  try {
    o->pfun = shl::expr::Expression(expr);
  } catch (const std::exception& e) {
    g_err = e.what();
    return -1;
  }
  o->has_pfun = true;
  return 0;
}

int oracle_set_cavity_functions(oracle* o, const char* rx, const char* ry, const char* rz) {
  const char* ex[3] = {rx, ry, rz};
  for (int k = 0; k < 3; ++k) {
    o->has_rfun[k] = ex[k] && *ex[k];
    if (!o->has_rfun[k]) continue;
    try {
      o->rfun[k] = shl::expr::Expression(ex[k]);
    } catch (const std::exception& e) {
      g_err = e.what();
      return -1;
    }
  }
  return 0;
}

int oracle_get_cavity(oracle* o, double* origins, double* ecav, double* out3) {
  for (unsigned n = 0; n < o->V; ++n) {
    if (origins)
      for (int c = 0; c < 3; ++c) origins[3 * n + c] = n < o->cav_origin.size() ? o->cav_origin[n](c) : 0.0;
    if (ecav) ecav[n] = n < o->ecav_vec.size() ? o->ecav_vec[n] : 0.0;
  }
  if (out3) {
    out3[0] = o->Ecav;
    out3[1] = o->cavity_force;
    out3[2] = o->Nc_cav;
  }
  return 0;
}

double oracle_get_dt(oracle* o) { return o->dt; }
uint64_t oracle_get_rejections(oracle* o) { return o->rejections; }

size_t oracle_get_contact_state(oracle* o, uint32_t* pairs, uint8_t* stick, double* origin, double* d2,
                                size_t cap, double* du_sum) {
  std::vector<const Contact*> cs;
  for (const Contact* c : o->candidates)
    if (c) cs.push_back(c);
  std::sort(cs.begin(), cs.end(), [](const Contact* x, const Contact* y) {
    return x->eid[0] != y->eid[0] ? x->eid[0] < y->eid[0] : x->eid[1] < y->eid[1];
  });
  for (size_t i = 0; i < cs.size() && i < cap; ++i) {
    if (pairs) { pairs[2 * i] = cs[i]->eid[0]; pairs[2 * i + 1] = cs[i]->eid[1]; }
    if (stick) stick[i] = cs[i]->stick ? 1 : 0;
    if (origin) for (int c = 0; c < 3; ++c) origin[3 * i + c] = cs[i]->spring_origin(c);
    if (d2) d2[i] = cs[i]->d2;
  }
  if (du_sum) *du_sum = o->du_sum;
  return cs.size();
}

int oracle_set_contact_state(oracle* o, const uint32_t* pairs, const uint8_t* stick, const double* origin,
                             const double* d2, size_t n, double du_sum) {
  for (Contact* c : o->candidates) delete c;
  o->candidates.clear();
  for (ElemCache& c : o->ec) c.in_contact_with.clear();
  for (size_t i = 0; i < n; ++i) {
    Contact* c = new Contact;
    c->eid[0] = pairs[2 * i];
    c->eid[1] = pairs[2 * i + 1];
    if (c->eid[0] >= o->F || c->eid[1] >= o->F || c->eid[0] >= c->eid[1]) {
      delete c;
      g_err = "bad contact pair";
      return -1;
    }
    c->stick = stick ? stick[i] != 0 : false;
    if (origin) c->spring_origin = Point(origin[3 * i], origin[3 * i + 1], origin[3 * i + 2]);
    c->d2 = d2 ? d2[i] : 0.0;
    o->candidates.push_back(c);
    o->ec[c->eid[0]].in_contact_with.push_back(c->eid[1]);
  }
  o->du_sum = du_sum;
  return 0;
}

static std::vector<Contact*> sorted_contacts(oracle* o) {
  std::vector<Contact*> cs;
  for (Contact* c : o->candidates)
    if (c) cs.push_back(c);
  std::sort(cs.begin(), cs.end(), [](const Contact* x, const Contact* y) {
    return x->eid[0] != y->eid[0] ? x->eid[0] < y->eid[0] : x->eid[1] < y->eid[1];
  });
  return cs;
}

size_t oracle_get_contact_coords(oracle* o, double* x, size_t cap) {
  const std::vector<Contact*> cs = sorted_contacts(o);
  for (size_t i = 0; i < cs.size() && i < cap; ++i)
    for (int k = 0; k < 4; ++k) x[4 * i + k] = cs[i]->x[k];
  return cs.size();
}

int oracle_set_contact_coords(oracle* o, const double* x, size_t n) {
  const std::vector<Contact*> cs = sorted_contacts(o);
  if (n != cs.size()) { g_err = "contact count mismatch"; return -1; }
  for (size_t i = 0; i < n; ++i)
    for (int k = 0; k < 4; ++k) cs[i]->x[k] = x[4 * i + k];
  return 0;
}

int oracle_limit_eval(oracle* o, uint32_t eid, double v, double w, double* out) {
  if (eid >= o->F || o->P.shell_shell_contact != SHL_CONTACT_SMOOTH) { g_err = "limit evaluation needs SMOOTH"; return -1; }
  shl_limit_patch lp;
  o->limit_patch(eid, lp);
  double r[6][3];
  shl_limit_eval(&lp, v, w, 2, r);
  for (int k = 0; k < 6; ++k)
    for (int c = 0; c < 3; ++c) out[3 * k + c] = r[k][c];
  return 0;
}

int oracle_limit_basis(oracle* o, uint32_t eid, double v, double w, double* out) {
  if (eid >= o->F || o->P.shell_shell_contact != SHL_CONTACT_SMOOTH) { g_err = "limit evaluation needs SMOOTH"; return -1; }
  shl_limit_patch lp;
  o->limit_patch(eid, lp);
  const int np = lp.N + 6;
  std::vector<double> E(3 * (size_t)np, 0.0);
  std::vector<uint32_t> ids(np);
  for (int j = 0; j < np; ++j) ids[j] = (uint32_t)j;
  lp.base = E.data();
  lp.ids = ids.data();
  lp.stride = 1;
  for (int j0 = 0; j0 < np; j0 += 3) {
    std::fill(E.begin(), E.end(), 0.0);
    for (int c = 0; c < 3 && j0 + c < np; ++c) E[3 * (j0 + c) + c] = 1.0;
    double r[6][3];
    shl_limit_eval(&lp, v, w, 2, r);
    for (int c = 0; c < 3 && j0 + c < np; ++c)
      for (int k = 0; k < 6; ++k) out[6 * (j0 + c) + k] = r[k][c];
  }
  return 0;
}

int oracle_smooth_closest(oracle* o, uint32_t e1, uint32_t e2, double* x, double* d2, double* dc) {
  if (e1 >= o->F || e2 >= o->F || o->P.shell_shell_contact != SHL_CONTACT_SMOOTH) { g_err = "needs SMOOTH"; return -1; }
  shl_limit_patch A, B;
  o->limit_patch(e1, A);
  o->limit_patch(e2, B);
  return smooth::closest(&A, &B, x, d2, dc);
}

size_t oracle_subdiv_table(int N, double* out, size_t cap) {
  std::vector<double> tab;
  if (N < 3 || N > 12 || N == 6 || !shl_subdiv::build_table(N, tab)) return 0;
  for (size_t i = 0; i < tab.size() && i < cap; ++i) out[i] = tab[i];
  return tab.size();
}

int oracle_rebuild_contacts(oracle* o) {
  o->current_problem = 0;
  o->compute_shell_shell_contact_candidates(true);
  return o->current_problem;
}

int oracle_get_mass_damping(oracle* o, double* Minv, double* C) {
  if (Minv) std::copy(o->Minv.begin(), o->Minv.end(), Minv);
  if (C) std::copy(o->C.begin(), o->C.end(), C);
  return 0;
}

int oracle_get_element_fields(oracle* o, double* kG, double* kM, double* et, double* eb, double* ar) {
  for (unsigned e = 0; e < o->F; ++e) {
    if (kG) kG[e] = o->ec[e].kGauss;
    if (kM) kM[e] = o->ec[e].kMean;
    if (et) et[e] = o->ec[e].etens;
    if (eb) eb[e] = o->ec[e].ebend;
    if (ar) ar[e] = o->ec[e].area;
  }
  return 0;
}

int oracle_get_node_fields(oracle* o, double* ekin, double* eself, double* efric) {
  for (unsigned n = 0; n < o->V; ++n) {
    if (ekin) ekin[n] = n < o->ekin_vec.size() ? o->ekin_vec[n] : 0.0;
    if (eself) eself[n] = n < o->eself_vec.size() ? o->eself_vec[n] : 0.0;
    if (efric) efric[n] = n < o->efric_vec.size() ? o->efric_vec[n] : 0.0;
  }
  return 0;
}

int oracle_get_cell_info(oracle* o, double* out) {
  out[0] = o->avg_elem_size;
  out[1] = o->last_cell_size;
  out[2] = o->last_d_max;
  for (int c = 0; c < 3; ++c) { out[3 + c] = o->bounds_min[c]; out[6 + c] = o->bounds_max[c]; }
  return 0;
}

int oracle_patch(oracle* o, uint32_t eid, uint32_t* nodes, uint32_t* n) {
  if (eid >= o->F) return -1;
  const auto& pt = o->ec[eid].patch;
  for (size_t i = 0; i < pt.size(); ++i) nodes[i] = pt[i];
  *n = (uint32_t)pt.size();
  return 0;
}

int oracle_basis_at(oracle* o, uint32_t eid, double v, double w, double* out) {
  if (eid >= o->F) return -1;
  std::vector<double> B;
  o->basis_unrotated(eid, v, w, B);
  std::copy(B.begin(), B.end(), out);
  return 0;
}

int oracle_basis_cached(oracle* o, uint32_t eid, double* out, double* R) {
  if (eid >= o->F) return -1;
  const ElemCache& c = o->ec[eid];
  for (size_t i = 0; i < c.patch.size(); ++i) {
    out[6 * i + 0] = c.phi[i];
    out[6 * i + 1] = c.dphi[i](0);
    out[6 * i + 2] = c.dphi[i](1);
    out[6 * i + 3] = c.d2phi[i](0);
    out[6 * i + 4] = c.d2phi[i](1);
    out[6 * i + 5] = c.d2phi[i](2);
  }
  if (R) { R[0] = c.R[0][0]; R[1] = c.R[0][1]; R[2] = c.R[1][0]; R[3] = c.R[1][1]; }
  return 0;
}

int oracle_elem_metric(oracle* o, uint32_t eid, int which, double* out) {
  if (eid >= o->F) return -1;
  const SurfaceMetric& m = which ? o->ec[eid].a_def : o->ec[eid].a_ref;
  int k = 0;
  for (int c = 0; c < 3; ++c) out[k++] = m.xyz(c);
  for (int i = 0; i < 3; ++i) for (int c = 0; c < 3; ++c) out[k++] = m.vec[i](c);
  for (int i = 0; i < 3; ++i) for (int c = 0; c < 3; ++c) out[k++] = m.dvec[i](c);
  for (int c = 0; c < 3; ++c) out[k++] = m.ff1(c);
  for (int c = 0; c < 3; ++c) out[k++] = m.ff2(c);
  out[k++] = m.jac;
  out[k++] = o->ec[eid].JxW;
  return 0;
}

int oracle_close_elems(oracle* o, uint32_t eid, uint32_t* out, size_t cap, size_t* n) {
  if (eid >= o->F) return -1;
  const auto& ce = o->ec[eid].close_elems;
  for (size_t i = 0; i < ce.size() && i < cap; ++i) out[i] = ce[i];
  *n = ce.size();
  return 0;
}

void oracle_segment_segment(const double* p10, const double* p11, const double* p20, const double* p21,
                            double* diffvec, double* st) {
  shl_segment_segment(p10, p11, p20, p21, diffvec, st);
}

void oracle_point_triangle(const double* p0, const double* p1, const double* p2, const double* p3,
                           double* diffvec, double* vw) {
  shl_point_triangle(p0, p1, p2, p3, diffvec, vw);
}

void oracle_pair_compute(const double* p, double* out) {
  Point q[2][3];
  const Point* pp[2][3];
  for (int e = 0; e < 2; ++e)
    for (int n = 0; n < 3; ++n) {
      q[e][n] = Point(p[9 * e + 3 * n], p[9 * e + 3 * n + 1], p[9 * e + 3 * n + 2]);
      pp[e][n] = &q[e][n];
    }
  PairGeom g;
  shell_shell_compute(pp, g);
  out[0] = g.d2;
  out[1] = g.dc(0); out[2] = g.dc(1); out[3] = g.dc(2);
  out[4] = g.v[0]; out[5] = g.w[0]; out[6] = g.v[1]; out[7] = g.w[1];
}

void oracle_friction_apply(double* Efric, double* f_contact, double f_normal, const double* n, const double* v,
                           double abs_v_normal, double v_stop, double k, double mu_s, double mu_d,
                           double damping, int* stick, double* spring_origin, const double* contact_point) {
  Point fc(f_contact[0], f_contact[1], f_contact[2]), so(spring_origin[0], spring_origin[1], spring_origin[2]);
  bool st = *stick != 0;
  Real E = *Efric;
  friction_apply(E, fc, f_normal, Point(n[0], n[1], n[2]), Point(v[0], v[1], v[2]), abs_v_normal, v_stop, k, mu_s,
                 mu_d, damping, st, so, Point(contact_point[0], contact_point[1], contact_point[2]));
  *Efric = E;
  *stick = st ? 1 : 0;
  for (int c = 0; c < 3; ++c) {
    f_contact[c] = fc(c);
    spring_origin[c] = so(c);
  }
}

double oracle_fixed_order_sum(const double* x, uint32_t n) { return fixed_order_sum(x, n); }

int oracle_fp_contract_off(void) {
  volatile double x = 1.0 + 1.0 / (1 << 30);  // x*x = 1 + 2^-29 + 2^-60
  volatile double y = 1.0 + 1.0 / (1 << 29);
  const double r = x * x - y;  // 0 when rounded in two steps, 2^-60 when fused
  return r == 0.0 ? 1 : 0;
}

}  // extern "C"
