// shl_setup.cpp -- host-side set-up of the shell library.
//
// Restates ShellSystem::set_parameters / update_derived / build_cache /
// reinit_mod / compute_reference_metrics / compute_mass_damping /
// build_topological_neighborhood (ShellSystem.C:170-852, 1317-1379,
// 3321-3499) for a closed triangle mesh with one quadrature point per face.
//
// The Loop basis at the quadrature point (1/3,1/3) is evaluated from Stam's
// box-spline polynomials in barycentric form (J. Stam, "Evaluation of Loop
// subdivision surfaces", SIGGRAPH'98 course notes); a patch whose first vertex
// is irregular (valence N != 6) is evaluated after one Loop subdivision step,
// in the middle sub-triangle that contains the quadrature point (as
// SubdivEvaluation.C:110-135 does for n = 1, k = 1), with Loop's vertex weight
// beta(N) = (5/8 - (3/8 + cos(2 pi/N)/4)^2)/N.
//
// Compiled with -ffp-contract=off (the contact-geometry header is shared with
// the device and must round identically).
#include "shl_setup.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <limits>
#include <set>
#include <unordered_map>

#include "shl_geom.h"

namespace shl {
namespace {

// Stam's 12 box-spline functions: (1/12) sum c u^i v^j w^k, u = 1 - v - w.
// Node s is at lattice offset kLat[s] from the element origin; the element is
// (origin, +v, +w) = nodes (3, 6, 7).
struct Term { int c, i, j, k; };
const Term kBox[12][15] = {
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

// power with derivative helpers: x^n, n x^(n-1), n(n-1) x^(n-2)
inline double pw(double x, int n) { double r = 1; for (int i = 0; i < n; ++i) r *= x; return r; }
inline double dpw(double x, int n) { return n >= 1 ? n * pw(x, n - 1) : 0.0; }
inline double ddpw(double x, int n) { return n >= 2 ? n * (n - 1) * pw(x, n - 2) : 0.0; }

// Box spline s at (v, w): value and the 5 derivatives with respect to (v, w),
// through the partial derivatives in (u, v, w) and u = 1 - v - w.
void box_eval(int s, double v, double w, double* out) {
  const double u = 1.0 - v - w;
  double f = 0, fu = 0, fv = 0, fw = 0, fuu = 0, fvv = 0, fww = 0, fuv = 0, fuw = 0, fvw = 0;
  for (const Term& t : kBox[s]) {
    if (t.c == 0) break;
    const double c = t.c / 12.0;
    const double U = pw(u, t.i), Vv = pw(v, t.j), W = pw(w, t.k);
    const double dU = dpw(u, t.i), dV = dpw(v, t.j), dW = dpw(w, t.k);
    f += c * U * Vv * W;
    fu += c * dU * Vv * W;
    fv += c * U * dV * W;
    fw += c * U * Vv * dW;
    fuu += c * ddpw(u, t.i) * Vv * W;
    fvv += c * U * ddpw(v, t.j) * W;
    fww += c * U * Vv * ddpw(w, t.k);
    fuv += c * dU * dV * W;
    fuw += c * dU * Vv * dW;
    fvw += c * U * dV * dW;
  }
  out[0] = f;
  out[1] = fv - fu;
  out[2] = fw - fu;
  out[3] = fvv - 2 * fuv + fuu;
  out[4] = fww - 2 * fuw + fuu;
  out[5] = fvw - fuv - fuw + fuu;
}

// Patch roles.  For an element (a, b, c) with a of valence N (b, c regular),
// slots: a=0, b=1, c=2, ring of a after c: 3..N, then d (across bc), the two
// further neighbours of b, the two further neighbours of c.
struct Roles {
  int N;
  int a() const { return 0; }
  int b() const { return 1; }
  int c() const { return 2; }
  int n(int k) const { return k == 0 ? 1 : (k == 1 ? 2 : k + 1); }  // k-th neighbour of a
  int d() const { return N + 1; }
  int b_far0() const { return N + 2; }  // next to d around b
  int b_far1() const { return N + 3; }  // next to n_{N-1} around b
  int c_far0() const { return N + 4; }  // next to d around c
  int c_far1() const { return N + 5; }  // next to n_2 around c
};

// Lattice slot of a regular patch for Stam node s (N = 6).
int stam_slot_regular(int s) {
  // lattice offsets of Stam nodes: (0,-1) (-1,0) (1,-1) (0,0) (-1,1) (2,-1) (1,0) (0,1) (-1,2) (2,0) (1,1) (0,2)
  static const int slot[12] = {5, 4, 6, 0, 3, 9, 1, 2, 11, 8, 7, 10};
  return slot[s];
}

// weights of Stam node s of the middle sub-triangle after one Loop step
void middle_node_weights(const Roles& r, int s, std::vector<double>& wt) {
  const int np = r.N + 6;
  wt.assign(np, 0.0);
  auto edge_pt = [&](int p, int q, int o1, int o2) {
    wt[p] += 0.375; wt[q] += 0.375; wt[o1] += 0.125; wt[o2] += 0.125;
  };
  auto vertex6 = [&](int ctr, std::initializer_list<int> ring) {
    wt[ctr] += 0.625;
    for (int x : ring) wt[x] += 0.0625;
  };
  const int N = r.N;
  switch (s) {
    case 0: edge_pt(r.c(), r.d(), r.b(), r.c_far0()); break;
    case 1: edge_pt(r.b(), r.d(), r.c(), r.b_far0()); break;
    case 2: vertex6(r.c(), {r.a(), r.b(), r.d(), r.c_far0(), r.c_far1(), r.n(2)}); break;
    case 3: edge_pt(r.b(), r.c(), r.a(), r.d()); break;
    case 4: vertex6(r.b(), {r.c(), r.a(), r.n(N - 1), r.b_far1(), r.b_far0(), r.d()}); break;
    case 5: edge_pt(r.c(), r.n(2), r.a(), r.c_far1()); break;
    case 6: edge_pt(r.a(), r.c(), r.b(), r.n(2)); break;
    case 7: edge_pt(r.a(), r.b(), r.c(), r.n(N - 1)); break;
    case 8: edge_pt(r.b(), r.n(N - 1), r.a(), r.b_far1()); break;
    case 9: edge_pt(r.a(), r.n(2), r.c(), r.n(3)); break;
    case 10: {
      const double t = 0.375 + 0.25 * std::cos(2.0 * M_PI / N);
      const double beta = (0.625 - t * t) / N;
      wt[r.a()] += 1.0 - N * beta;
      for (int k = 0; k < N; ++k) wt[r.n(k)] += beta;
      break;
    }
    case 11: edge_pt(r.a(), r.n(N - 1), r.b(), r.n(N - 2)); break;
  }
}

struct V3 {
  double x, y, z;
};
inline V3 operator+(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline V3 operator-(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V3 operator*(double s, V3 a) { return {s * a.x, s * a.y, s * a.z}; }
inline double dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline V3 cross(V3 a, V3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
inline double norm(V3 a) { return std::sqrt(dot(a, a)); }

}  // namespace

void regular_basis(double v, double w, double* out) {
  for (int s = 0; s < 12; ++s) box_eval(s, v, w, out + 6 * stam_slot_regular(s));
}

void irregular_basis(int n, double v, double w, double* out) {
  const Roles r{n};
  const int np = n + 6;
  std::fill(out, out + 6 * np, 0.0);
  // middle sub-triangle: local coordinates (1-2v, 1-2w); d/dv = -2 d/dv_local
  const double jac[6] = {1, -2, -2, 4, 4, 4};
  std::vector<double> wt;
  for (int s = 0; s < 12; ++s) {
    double b[6];
    box_eval(s, 1 - 2 * v, 1 - 2 * w, b);
    middle_node_weights(r, s, wt);
    for (int p = 0; p < np; ++p) {
      if (wt[p] == 0) continue;
      for (int k = 0; k < 6; ++k) out[6 * p + k] += wt[p] * (jac[k] * b[k]);
    }
  }
}

namespace {

// Element-force slot layout: group after group, n_slots slots per face.
void layout_slots(Setup& S) {
  uint32_t base = 0, rows = 12;
  for (PatchGroup& g : S.groups) {
    g.slot_base = base;
    base += g.count * (uint32_t)g.n_slots;
    if ((uint32_t)g.n_slots > rows) rows = (uint32_t)g.n_slots;
  }
  S.n_slots_total = base;
  S.patch_rows = rows;
}

// Gather CSR (node -> element-force slots, ascending) and the node -> face
// CSR (faces of which a node is a vertex, ascending internal order).
void build_node_lists(Setup& S) {
  const uint32_t V = S.V, F = S.F;
  S.gather_ptr.assign(V + 1, 0);
  S.node_face_ptr.assign(V + 1, 0);
  for (const PatchGroup& g : S.groups)
    for (uint32_t i = g.first; i < g.first + g.count; ++i)
      for (int s = 0; s < g.n_slots; ++s) {
        const int32_t nd = S.patch[(size_t)s * F + i];
        if (nd < 0) continue;
        ++S.gather_ptr[nd + 1];
        if (s < 3) ++S.node_face_ptr[nd + 1];
      }
  for (uint32_t nd = 0; nd < V; ++nd) {
    S.gather_ptr[nd + 1] += S.gather_ptr[nd];
    S.node_face_ptr[nd + 1] += S.node_face_ptr[nd];
  }
  S.gather_ent.assign(S.gather_ptr[V], 0);
  S.node_face.assign(S.node_face_ptr[V], 0);
  std::vector<uint32_t> cur(S.gather_ptr.begin(), S.gather_ptr.end() - 1);
  std::vector<uint32_t> cur_f(S.node_face_ptr.begin(), S.node_face_ptr.end() - 1);
  for (const PatchGroup& g : S.groups)
    for (uint32_t i = g.first; i < g.first + g.count; ++i)
      for (int s = 0; s < g.n_slots; ++s) {
        const int32_t nd = S.patch[(size_t)s * F + i];
        if (nd < 0) continue;
        S.gather_ent[cur[nd]++] = g.slot_base + (i - g.first) * (uint32_t)g.n_slots + (uint32_t)s;
        if (s < 3) S.node_face[cur_f[nd]++] = S.perm[i];
      }
  S.slot_pos.assign(S.n_slots_total, 0);
  for (uint32_t k = 0; k < (uint32_t)S.gather_ent.size(); ++k) S.slot_pos[S.gather_ent[k]] = k;
}

}  // namespace

bool build_setup(const shl_mesh& mesh, const shl_params& prm, Setup& S, std::string& err) {
  const uint32_t V = mesh.n_nodes, F = mesh.n_faces;
  if (V < 4 || F < 4 || !mesh.xyz || !mesh.faces) { err = "empty mesh"; return false; }
  S.V = V;
  S.F = F;
  S.X.assign(mesh.xyz, mesh.xyz + 3 * (size_t)V);
  S.tri.assign(mesh.faces, mesh.faces + 3 * (size_t)F);
  for (uint32_t x : S.tri)
    if (x >= V) { err = "face index out of range"; return false; }

  // directed half-edge (from, to) -> opposite vertex of its face
  std::unordered_map<uint64_t, uint32_t> opp;
  opp.reserve(3 * (size_t)F * 2);
  auto key = [](uint32_t a, uint32_t b) { return ((uint64_t)a << 32) | b; };
  std::vector<int> valence(V, 0);
  for (uint32_t f = 0; f < F; ++f) {
    const uint32_t* t = &S.tri[3 * f];
    for (int k = 0; k < 3; ++k) {
      const uint32_t a = t[k], b = t[(k + 1) % 3], c = t[(k + 2) % 3];
      if (!opp.emplace(key(a, b), c).second) { err = "non-manifold or inconsistently oriented mesh"; return false; }
      ++valence[a];
    }
  }
  for (const auto& kv : opp)
    if (!opp.count(key((uint32_t)kv.first, (uint32_t)(kv.first >> 32)))) {
      err = "open mesh (boundary edges need ghost elements, which are not supported)";
      return false;
    }
  // the vertex after x when turning around `center` through the face with edge center->x
  auto turn = [&](uint32_t center, uint32_t x) -> uint32_t { return opp.at(key(center, x)); };

  // per face: rotated vertex order (irregular vertex first) and patch slots
  std::vector<std::vector<uint32_t>> patch_of(F);
  std::vector<int> val_of(F);
  for (uint32_t f = 0; f < F; ++f) {
    const uint32_t* t = &S.tri[3 * f];
    int first = 0, n_irr = 0;
    for (int k = 0; k < 3; ++k)
      if (valence[t[k]] != 6) { first = k; ++n_irr; }
    if (n_irr > 1) { err = "a face has more than one irregular vertex; refine the mesh"; return false; }
    const uint32_t a = t[first], b = t[(first + 1) % 3], c = t[(first + 2) % 3];
    const int N = valence[a];
    if (N < 3 || N > 12) { err = "unsupported vertex valence"; return false; }
    std::vector<uint32_t> ring_a{b};
    for (uint32_t x = turn(a, b); x != b; x = turn(a, x)) ring_a.push_back(x);
    if ((int)ring_a.size() != N) { err = "inconsistent vertex ring"; return false; }
    std::vector<uint32_t>& P = patch_of[f];
    P.assign(N + 6, 0);
    const Roles r{N};
    for (int k = 0; k < N; ++k) P[r.n(k)] = ring_a[k];
    P[r.a()] = a;
    // around b starting at c: c, a, n_{N-1}, b_far1, b_far0, d
    uint32_t x = turn(b, c);                 // a
    x = turn(b, x);                          // n_{N-1}
    if (x != ring_a[N - 1]) { err = "inconsistent ring around b"; return false; }
    P[r.b_far1()] = turn(b, x);
    P[r.b_far0()] = turn(b, P[r.b_far1()]);
    P[r.d()] = turn(b, P[r.b_far0()]);
    if (turn(b, P[r.d()]) != c) { err = "irregular vertex next to face (b)"; return false; }
    // around c starting at a: a, b, d, c_far0, c_far1, n_2
    if (turn(c, a) != b || turn(c, b) != P[r.d()]) { err = "inconsistent ring around c"; return false; }
    P[r.c_far0()] = turn(c, P[r.d()]);
    P[r.c_far1()] = turn(c, P[r.c_far0()]);
    if (turn(c, P[r.c_far1()]) != ring_a[2 % N] || turn(c, ring_a[2 % N]) != a) {
      err = "irregular vertex next to face (c)";
      return false;
    }
    val_of[f] = N;
  }

  // groups: regular first, then irregular by valence (original order inside)
  std::vector<int> vals;
  for (uint32_t f = 0; f < F; ++f) vals.push_back(val_of[f]);
  std::vector<int> distinct(vals.begin(), vals.end());
  std::sort(distinct.begin(), distinct.end());
  distinct.erase(std::unique(distinct.begin(), distinct.end()), distinct.end());
  std::stable_sort(distinct.begin(), distinct.end(), [](int x, int y) { return (x == 6) > (y == 6); });
  S.perm.clear();
  S.groups.clear();
  for (int N : distinct) {
    PatchGroup g;
    g.valence = N;
    g.n_slots = N + 6;
    g.first = (uint32_t)S.perm.size();
    for (uint32_t f = 0; f < F; ++f)
      if (val_of[f] == N) S.perm.push_back(f);
    g.count = (uint32_t)S.perm.size() - g.first;
    g.basis.assign(6 * g.n_slots, 0.0);
    if (N == 6)
      regular_basis(1.0 / 3.0, 1.0 / 3.0, g.basis.data());
    else
      irregular_basis(N, 1.0 / 3.0, 1.0 / 3.0, g.basis.data());
    S.groups.push_back(std::move(g));
  }
  if (S.groups.empty() || S.groups[0].valence != 6) {
    // meshes without regular faces: keep an empty regular group first
    PatchGroup g;
    g.valence = 6; g.n_slots = 12; g.first = 0; g.count = 0;
    g.basis.assign(72, 0.0);
    regular_basis(1.0 / 3.0, 1.0 / 3.0, g.basis.data());
    S.groups.insert(S.groups.begin(), g);
    for (size_t i = 1; i < S.groups.size(); ++i) S.groups[i].first = S.groups[i - 1].first + S.groups[i - 1].count;
  }
  S.inv_perm.assign(F, 0);
  for (uint32_t i = 0; i < F; ++i) S.inv_perm[S.perm[i]] = i;
  layout_slots(S);

  // derived constants, ShellSystem.C:472-486
  {
    const double nu2 = (prm.shell_young_modulus2 * prm.shell_poisson_ratio) / prm.shell_young_modulus;
    const double one_nu2 = 1 - prm.shell_poisson_ratio * nu2;
    S.K = prm.memb_stiff_mult * prm.thickness / one_nu2;
    S.D = prm.bend_stiff_mult * std::pow(prm.thickness, 3) / (12 * one_nu2);
    const double E_avg = (prm.shell_young_modulus + prm.shell_young_modulus2) * 0.5;
    S.stiff_density = 0.5 * E_avg / (one_nu2 * prm.thickness);
    S.stiff_static_friction = prm.fric_stiff_mult * E_avg * prm.thickness / one_nu2;
    S.d2_friction = std::pow((1 + prm.static_friction_tol) * prm.thickness, 2);
  }

  S.patch.assign((size_t)S.patch_rows * F, -1);
  S.face.assign((size_t)FF_COUNT * F, 0.0);
  std::vector<double> face_bal((size_t)FF_COUNT * F, 0.0);  // balanced-frame constants (FP32 path)
  S.Minv.assign(3 * (size_t)V, 0.0);
  S.C.assign(3 * (size_t)V, 0.0);
  auto Xn = [&](uint32_t n) { return V3{S.X[3 * n], S.X[3 * n + 1], S.X[3 * n + 2]}; };
  const double qw = 0.5;  // one-point Gauss rule on the reference triangle
  const double E1 = prm.shell_young_modulus, E2 = prm.shell_young_modulus2, nu = prm.shell_poisson_ratio,
               G12 = prm.shell_shear_modulus;

  for (const PatchGroup& g : S.groups) {
    const double* B = g.basis.data();
    for (uint32_t i = g.first; i < g.first + g.count; ++i) {
      const uint32_t f = S.perm[i];
      const std::vector<uint32_t>& P = patch_of[f];
      const int np = g.n_slots;
      for (int s = 0; s < np; ++s) S.patch[(size_t)s * F + i] = (int32_t)P[s];
      auto put = [&](int field, double x) { S.face[(size_t)field * F + i] = x; };

      // first map with the unrotated derivatives
      V3 xq{0, 0, 0}, b1{0, 0, 0}, b2{0, 0, 0};
      for (int s = 0; s < np; ++s) {
        const V3 x = Xn(P[s]);
        xq = xq + B[6 * s] * x;
        b1 = b1 + B[6 * s + 1] * x;
        b2 = b2 + B[6 * s + 2] * x;
      }
      const double g11 = dot(b1, b1), g12 = dot(b1, b2), g22 = dot(b2, b2);
      const double JxW = std::sqrt(g11 * g22 - g12 * g12) * qw;

      // material frame: j = projection of +z, k = -n x j, scaled as in reinit_mod
      const V3 normal = cross(b1, b2);
      const double nn = norm(normal);
      const V3 n = (1.0 / nn) * normal;
      const V3 ez{0, 0, 1};
      V3 j = ez - dot(ez, n) * n;
      V3 k = -1.0 * cross(n, j);
      if (norm(j) == 0) { err = "face normal parallel to z: material frame undefined"; return false; }
      const double ang = std::atan2(norm(cross(j, b1)), dot(j, b1));
      const double jfac = nn / (norm(b1) * std::sin(ang));
      const double kfac = nn / jfac;
      j = (jfac / norm(j)) * j;
      k = (kfac / norm(k)) * k;
      // R = [b1 b2 normal]^-1 [k j normal]; the rotation by Rn in reinit_mod
      // cancels mathematically and is not applied.  Solve the 2x2 block by
      // projecting onto the dual basis of (b1, b2).
      const double det = g11 * g22 - g12 * g12;
      auto coords = [&](V3 t, double& c1, double& c2) {
        const double t1 = dot(t, b1), t2 = dot(t, b2);
        c1 = (g22 * t1 - g12 * t2) / det;
        c2 = (g11 * t2 - g12 * t1) / det;
      };
      // constants of the frame (kk, jj): rotation, reference metric, H
      auto frame_constants = [&](V3 kk, V3 jj, double* out) {
        double R00, R10, R01, R11;
        coords(kk, R00, R10);  // kk = R00 b1 + R10 b2
        coords(jj, R01, R11);  // jj = R01 b1 + R11 b2
        out[FF_R00] = R00; out[FF_R01] = R01; out[FF_R10] = R10; out[FF_R11] = R11;
        out[FF_JXW] = JxW;
        out[FF_X0] = xq.x; out[FF_X1] = xq.y; out[FF_X2] = xq.z;
        // second map with the rotated derivatives
        V3 a1{0, 0, 0}, a2{0, 0, 0}, d11{0, 0, 0}, d22{0, 0, 0}, d12{0, 0, 0};
        for (int s = 0; s < np; ++s) {
          const double px = B[6 * s + 1], pe = B[6 * s + 2];
          const double pxx = B[6 * s + 3], pee = B[6 * s + 4], pxe = B[6 * s + 5];
          const double r1 = px * R00 + pe * R10;
          const double r2 = px * R01 + pe * R11;
          const double r11 = pxx * R00 * R00 + pee * R10 * R10 + 2 * pxe * R00 * R10;
          const double r22 = pxx * R01 * R01 + pee * R11 * R11 + 2 * pxe * R01 * R11;
          const double r12 = pxx * R00 * R01 + pee * R10 * R11 + pxe * (R01 * R10 + R00 * R11);
          const V3 x = Xn(P[s]);
          a1 = a1 + r1 * x;
          a2 = a2 + r2 * x;
          d11 = d11 + r11 * x;
          d22 = d22 + r22 * x;
          d12 = d12 + r12 * x;
        }
        const V3 a3u = cross(a1, a2);
        const V3 a3 = (1.0 / norm(a3u)) * a3u;
        const double ff1[3] = {dot(a1, a1), dot(a2, a2), dot(a1, a2)};
        const double ff2[3] = {dot(d11, a3), dot(d22, a3), dot(d12, a3)};
        out[FF_A10] = a1.x; out[FF_A11] = a1.y; out[FF_A12] = a1.z;
        out[FF_A20] = a2.x; out[FF_A21] = a2.y; out[FF_A22] = a2.z;
        out[FF_D10] = d11.x; out[FF_D11] = d11.y; out[FF_D12] = d11.z;
        out[FF_D20] = d22.x; out[FF_D21] = d22.y; out[FF_D22] = d22.z;
        out[FF_D30] = d12.x; out[FF_D31] = d12.y; out[FF_D32] = d12.z;
        out[FF_G0] = ff1[0]; out[FF_G1] = ff1[1]; out[FF_G2] = ff1[2];
        out[FF_B0] = ff2[0]; out[FF_B1] = ff2[1]; out[FF_B2] = ff2[2];
        // orthotropic H, ShellSystem.C:1199-1213 (constant for constant moduli)
        const double nu2 = (E1 * nu) / E2;
        const double g0 = ff1[0], g1 = ff1[1], g2 = ff1[2];
        const double id = 1 / (g0 * g1 - g2 * g2);
        const double s2 = id * id;
        out[FF_H00] = s2 * (E1 * g1 * g1);
        out[FF_H01] = s2 * (E1 * (nu * g1 * g0 + (1 - nu) * g2 * g2));
        out[FF_H02] = s2 * (E1 * -g1 * g2);
        out[FF_H11] = s2 * (E2 * g0 * g0);
        out[FF_H12] = s2 * (E2 * -g0 * g2);
        out[FF_H22] = s2 * (G12 * ((1 - nu * nu2) * g1 * g0 + (1 - nu * nu2) * ((1 + nu) / (1 - nu)) * g2 * g2));
        out[FF_K] = S.K;
        out[FF_D] = S.D;
      };
      double cref[FF_COUNT], cbal[FF_COUNT];
      frame_constants(k, j, cref);
      for (int fld = 0; fld < FF_COUNT; ++fld) put(fld, cref[fld]);
      // The scaling of reinit_mod (kfac, jfac) degenerates when b1 is nearly
      // parallel to the meridian j (kfac -> 0 and the constants span dozens of
      // decades).  The mechanics does not depend on the lengths of k and j, so
      // the FP32 path uses the same directions with |k| = |j| = sqrt(|b1 x b2|).
      {
        const double sq = std::sqrt(nn);
        frame_constants((sq / norm(k)) * k, (sq / norm(j)) * j, cbal);
        for (int fld = 0; fld < FF_COUNT; ++fld) face_bal[(size_t)fld * F + i] = cbal[fld];
      }

      // lumped mass and damping, ShellSystem.C:795-844
      double sum_phi = 0;
      for (int s = 0; s < np; ++s) sum_phi += B[6 * s];
      double hmin = std::numeric_limits<double>::max(), hmax = 0;
      for (int e = 0; e < 3; ++e) {
        const double l = norm(Xn(S.tri[3 * f + e]) - Xn(S.tri[3 * f + (e + 1) % 3]));
        hmin = std::min(hmin, l);
        hmax = std::max(hmax, l);
      }
      const double avg_stiff = 2 * (S.K + S.D / (hmin * hmax)) / 3;
      for (int s = 0; s < np; ++s) {
        const double m = (sum_phi * JxW * B[6 * s]) * (prm.shell_mass_density * prm.thickness);
        const double c = prm.damping_alpha * m + prm.damping_beta * avg_stiff;
        for (int cc = 0; cc < 3; ++cc) {
          S.Minv[3 * (size_t)P[s] + cc] += m;
          S.C[3 * (size_t)P[s] + cc] += c;
        }
      }
    }
  }
  // FP32 constants of the relative-displacement element path
  S.face32.assign((size_t)F32_COUNT * F, 0.0f);
  S.face_df.assign((size_t)2 * F32_COUNT * F, 0.0f);
  for (uint32_t i = 0; i < F; ++i) {
    auto get = [&](int fld) { return face_bal[(size_t)fld * F + i]; };
    auto put32 = [&](int fld, double x) {
      const float h = (float)x;
      S.face32[(size_t)fld * F + i] = h;
      S.face_df[(size_t)fld * F + i] = h;
      S.face_df[(size_t)(F32_COUNT + fld) * F + i] = (float)(x - (double)h);
    };
    const int map64[][2] = {{F32_R00, FF_R00}, {F32_R01, FF_R01}, {F32_R10, FF_R10}, {F32_R11, FF_R11},
                            {F32_JXW, FF_JXW}, {F32_X0, FF_X0}, {F32_X1, FF_X1}, {F32_X2, FF_X2},
                            {F32_A10, FF_A10}, {F32_A11, FF_A11}, {F32_A12, FF_A12}, {F32_A20, FF_A20},
                            {F32_A21, FF_A21}, {F32_A22, FF_A22}, {F32_D10, FF_D10}, {F32_D11, FF_D11},
                            {F32_D12, FF_D12}, {F32_D20, FF_D20}, {F32_D21, FF_D21}, {F32_D22, FF_D22},
                            {F32_D30, FF_D30}, {F32_D31, FF_D31}, {F32_D32, FF_D32}, {F32_G0, FF_G0},
                            {F32_G1, FF_G1}, {F32_G2, FF_G2}, {F32_H00, FF_H00}, {F32_H01, FF_H01},
                            {F32_H02, FF_H02}, {F32_H11, FF_H11}, {F32_H12, FF_H12}, {F32_H22, FF_H22},
                            {F32_K, FF_K}, {F32_D, FF_D}};
    for (const auto& m : map64) put32(m[0], get(m[1]));
    const V3 a1{get(FF_A10), get(FF_A11), get(FF_A12)}, a2{get(FF_A20), get(FF_A21), get(FF_A22)};
    const V3 n = cross(a1, a2);
    const double L = norm(n);
    put32(F32_N0, n.x / L);
    put32(F32_N1, n.y / L);
    put32(F32_N2, n.z / L);
    put32(F32_L0, L);
  }

  for (double& c : S.C) c += prm.damping_gamma;
  for (double& m : S.Minv) {
    if (!(m > 0)) { err = "non-positive lumped mass"; return false; }
    m = 1 / m;
  }

  build_node_lists(S);

  // topological exclusion set, ShellSystem.C:657-741 (original face ids)
  S.close_ptr.assign(F + 1, 0);
  S.close_list.clear();
  if (prm.shell_shell_contact != SHL_CONTACT_NONE) {
    std::vector<std::vector<uint32_t>> node_faces(V);
    for (uint32_t f = 0; f < F; ++f)
      for (int k = 0; k < 3; ++k) node_faces[S.tri[3 * f + k]].push_back(f);
    std::vector<std::vector<uint32_t>> nbrs(F);
    for (uint32_t f = 0; f < F; ++f) {
      std::vector<uint32_t>& nb = nbrs[f];
      for (int k = 0; k < 3; ++k)
        for (uint32_t o : node_faces[S.tri[3 * f + k]])
          if (o != f) nb.push_back(o);
      std::sort(nb.begin(), nb.end());
      nb.erase(std::unique(nb.begin(), nb.end()), nb.end());
    }
    const double cutoff = (1 + prm.neighbor_margin) * prm.thickness;
    const double cutoff2 = cutoff * cutoff;
    auto mesh_d2 = [&](uint32_t e1, uint32_t e2) {
      const double* p1[3] = {&S.X[3 * S.tri[3 * e1]], &S.X[3 * S.tri[3 * e1 + 1]], &S.X[3 * S.tri[3 * e1 + 2]]};
      const double* p2[3] = {&S.X[3 * S.tri[3 * e2]], &S.X[3 * S.tri[3 * e2 + 1]], &S.X[3 * S.tri[3 * e2 + 2]]};
      shl_pair_geom g;
      shl_pair_compute(p1, p2, &g);
      return g.d2;
    };
    std::vector<std::vector<uint32_t>> close(F);
#pragma omp parallel for schedule(dynamic, 64)
    for (int64_t fi = 0; fi < (int64_t)F; ++fi) {
      const uint32_t f = (uint32_t)fi;
      std::set<uint32_t> cl(nbrs[f].begin(), nbrs[f].end());
      std::vector<uint32_t> frontier(nbrs[f].begin(), nbrs[f].end());
      while (!frontier.empty()) {
        std::set<uint32_t> cand;
        for (uint32_t x : frontier)
          for (uint32_t y : nbrs[x])
            if (y != f) cand.insert(y);
        frontier.clear();
        for (uint32_t y : cand)
          if (!cl.count(y) && mesh_d2(f, y) < cutoff2) {
            cl.insert(y);
            frontier.push_back(y);
          }
      }
      close[f].assign(cl.begin(), cl.end());
    }
    for (uint32_t f = 0; f < F; ++f) {
      S.close_ptr[f + 1] = S.close_ptr[f] + (uint32_t)close[f].size();
      S.close_list.insert(S.close_list.end(), close[f].begin(), close[f].end());
    }
  }
  {
    const uint64_t nc = (uint64_t)std::ceil(std::sqrt((double)F) / prm.cell_size_mult);
    S.n_cells_max = nc * nc * nc;
  }
  return true;
}

bool merge_setups(std::vector<Setup>& shells, Setup& M, std::vector<uint32_t>& node_off,
                  std::vector<uint32_t>& face_off, std::vector<uint32_t>& face_shell, std::string& err) {
  const size_t n = shells.size();
  if (n == 0) { err = "no shells"; return false; }
  node_off.assign(n + 1, 0);
  face_off.assign(n + 1, 0);
  for (size_t k = 0; k < n; ++k) {
    node_off[k + 1] = node_off[k] + shells[k].V;
    face_off[k + 1] = face_off[k] + shells[k].F;
  }
  const uint32_t V = node_off[n], F = face_off[n];
  M = Setup();
  M.V = V;
  M.F = F;
  face_shell.assign(F, 0);
  // the distinct patch types, regular first
  std::vector<int> vals;
  for (const Setup& S : shells)
    for (const PatchGroup& g : S.groups)
      if (g.count && std::find(vals.begin(), vals.end(), g.valence) == vals.end()) vals.push_back(g.valence);
  std::sort(vals.begin(), vals.end());
  std::stable_sort(vals.begin(), vals.end(), [](int x, int y) { return (x == 6) > (y == 6); });
  if (vals.empty() || vals[0] != 6) vals.insert(vals.begin(), 6);
  M.X.reserve(3 * (size_t)V);
  M.tri.reserve(3 * (size_t)F);
  M.Minv.reserve(3 * (size_t)V);
  M.C.reserve(3 * (size_t)V);
  for (size_t k = 0; k < n; ++k) {
    const Setup& S = shells[k];
    M.X.insert(M.X.end(), S.X.begin(), S.X.end());
    for (uint32_t x : S.tri) M.tri.push_back(x + node_off[k]);
    M.Minv.insert(M.Minv.end(), S.Minv.begin(), S.Minv.end());
    M.C.insert(M.C.end(), S.C.begin(), S.C.end());
    for (uint32_t f = 0; f < S.F; ++f) face_shell[face_off[k] + f] = (uint32_t)k;
  }
  // regroup: for each patch type, the faces of every shell in shell order
  M.perm.clear();
  std::vector<std::pair<uint32_t, uint32_t>> src;  // (shell, internal face of the shell)
  for (int val : vals) {
    PatchGroup g;
    g.valence = val;
    g.n_slots = val + 6;
    g.first = (uint32_t)M.perm.size();
    for (size_t k = 0; k < n; ++k) {
      const Setup& S = shells[k];
      for (const PatchGroup& sg : S.groups) {
        if (sg.valence != val) continue;
        if (g.basis.empty()) g.basis = sg.basis;
        for (uint32_t i = sg.first; i < sg.first + sg.count; ++i) {
          M.perm.push_back(face_off[k] + S.perm[i]);
          src.emplace_back((uint32_t)k, i);
        }
      }
    }
    g.count = (uint32_t)M.perm.size() - g.first;
    if (g.basis.empty()) {
      g.basis.assign(6 * g.n_slots, 0.0);
      if (val == 6) regular_basis(1.0 / 3.0, 1.0 / 3.0, g.basis.data());
      else irregular_basis(val, 1.0 / 3.0, 1.0 / 3.0, g.basis.data());
    }
    M.groups.push_back(std::move(g));
  }
  if (M.perm.size() != F) { err = "face regrouping lost faces"; return false; }
  M.inv_perm.assign(F, 0);
  for (uint32_t i = 0; i < F; ++i) M.inv_perm[M.perm[i]] = i;
  layout_slots(M);
  M.patch.assign((size_t)M.patch_rows * F, -1);
  M.face.assign((size_t)FF_COUNT * F, 0.0);
  M.face32.assign((size_t)F32_COUNT * F, 0.0f);
  M.face_df.assign((size_t)2 * F32_COUNT * F, 0.0f);
  for (uint32_t i = 0; i < F; ++i) {
    const uint32_t k = src[i].first, si = src[i].second;
    const Setup& S = shells[k];
    for (uint32_t s = 0; s < S.patch_rows; ++s) {
      const int32_t nd = S.patch[(size_t)s * S.F + si];
      M.patch[(size_t)s * F + i] = nd < 0 ? -1 : nd + (int32_t)node_off[k];
    }
    for (int fld = 0; fld < FF_COUNT; ++fld) M.face[(size_t)fld * F + i] = S.face[(size_t)fld * S.F + si];
    for (int fld = 0; fld < F32_COUNT; ++fld) M.face32[(size_t)fld * F + i] = S.face32[(size_t)fld * S.F + si];
    for (int fld = 0; fld < 2 * F32_COUNT; ++fld) M.face_df[(size_t)fld * F + i] = S.face_df[(size_t)fld * S.F + si];
  }
  build_node_lists(M);
  // topological exclusion sets (self-contact), face ids offset shell by shell
  M.close_ptr.assign(F + 1, 0);
  M.close_list.clear();
  for (size_t k = 0; k < n; ++k) {
    const Setup& S = shells[k];
    for (uint32_t f = 0; f < S.F; ++f) {
      const uint32_t c0 = S.close_ptr.empty() ? 0 : S.close_ptr[f], c1 = S.close_ptr.empty() ? 0 : S.close_ptr[f + 1];
      for (uint32_t q = c0; q < c1; ++q) M.close_list.push_back(S.close_list[q] + face_off[k]);
      M.close_ptr[face_off[k] + f + 1] = (uint32_t)M.close_list.size();
    }
  }
  M.K = shells[0].K;
  M.D = shells[0].D;
  return true;
}

}  // namespace shl
