// shl_subdiv.h -- subdivision tables of the Loop limit-surface evaluation of
// irregular patches (host only; shared by the library set-up and the CPU oracle
// so that both evaluate with the same doubles).
//
// For a face (a, b, c) whose vertex a has valence N != 6 the patch holds N + 6
// nodes in this library's order: a = 0, b = 1, c = 2, the ring of a after c =
// 3 .. N, d (across bc) = N+1, then the two further neighbours of b (b_far0 next
// to d, b_far1) = N+2, N+3 and of c (c_far0 next to d, c_far1) = N+4, N+5.
// The table holds, for every level n = 1 .. 34 and child k = 0, 1, 2, the 12
// control points (Stam's node order) of the regular child patch reached after n
// Loop steps around a, as weights of the N + 6 patch nodes:
//   tab[((n - 1) * 3 + k) * 12 * (N + 6) + s * (N + 6) + j].
// Children (SubdivEvaluation.C:110-135): k = 0 is the corner at b, (m_ab, b,
// m_bc) with local (2v - 1, 2w); k = 2 the corner at c, (m_ca, m_bc, c) with
// (2v, 2w - 1); k = 1 the middle triangle (m_bc, m_ca, m_ab) with
// (1 - 2v, 1 - 2w); each listed as (origin, +v vertex, +w vertex).
//
// The tables are built by subdividing a small local mesh symbolically: the
// N + 7 faces of the patch carry their nodes as weight vectors over the N + 6
// patch nodes; one Loop step (Loop's vertex rule with beta(N) = (5/8 - (3/8 +
// cos(2 pi / N)/4)^2) / N, edge rule 3/8, 3/8, 1/8, 1/8) produces every vertex
// point whose one-ring is complete and every edge point with both faces
// present; the children's patches are then read off the subdivided mesh by
// walking the one-rings, exactly as the mesh set-up reads the patches of the
// mesh.  The corner child (a', m_ab, m_ca) is again an N + 6 patch of valence
// N, which carries the recursion to the next level.
#ifndef SHL_SUBDIV_H_
#define SHL_SUBDIV_H_

#include <array>
#include <cmath>
#include <map>
#include <utility>
#include <vector>

namespace shl_subdiv {

constexpr int kLevels = 34;

struct LocalMesh {
  std::vector<std::vector<double>> W;   // node weights over the original patch nodes
  std::vector<std::array<int, 3>> F;    // oriented faces
};

inline int slot_n(int N, int k) { (void)N; return k == 0 ? 1 : (k == 1 ? 2 : k + 1); }

// Local mesh of a patch given its N + 6 nodes' weights (patch order).
inline LocalMesh patch_mesh(int N, const std::vector<std::vector<double>>& nodes) {
  LocalMesh M;
  M.W = nodes;
  const int a = 0, b = 1, c = 2, d = N + 1, bf0 = N + 2, bf1 = N + 3, cf0 = N + 4, cf1 = N + 5;
  for (int k = 0; k < N; ++k) M.F.push_back({a, slot_n(N, k), slot_n(N, (k + 1) % N)});
  const int nl = slot_n(N, N - 1), n2 = slot_n(N, 2 % N);
  M.F.push_back({b, nl, bf1});
  M.F.push_back({b, bf1, bf0});
  M.F.push_back({b, bf0, d});
  M.F.push_back({b, d, c});
  M.F.push_back({c, d, cf0});
  M.F.push_back({c, cf0, cf1});
  M.F.push_back({c, cf1, n2});
  return M;
}

struct HalfEdges {
  std::map<std::pair<int, int>, int> opp;  // directed edge (x, y) -> third vertex of its face
  explicit HalfEdges(const LocalMesh& M) {
    for (const auto& f : M.F)
      for (int k = 0; k < 3; ++k) opp[{f[k], f[(k + 1) % 3]}] = f[(k + 2) % 3];
  }
  int turn(int center, int x) const {
    auto it = opp.find({center, x});
    return it == opp.end() ? -1 : it->second;
  }
  // closed one-ring of v starting at x (empty if open)
  std::vector<int> ring(int v, int x) const {
    std::vector<int> r{x};
    for (int y = turn(v, x); y != x; y = turn(v, y)) {
      if (y < 0 || r.size() > 64) return {};
      r.push_back(y);
    }
    return r;
  }
};

inline void axpy(std::vector<double>& acc, double s, const std::vector<double>& x) {
  for (size_t i = 0; i < acc.size(); ++i) acc[i] += s * x[i];
}

// One Loop step.  vmap[v] = vertex point of v (or -1); emap = edge points.
struct Subdivided {
  LocalMesh M;
  std::vector<int> vmap;
  std::map<std::pair<int, int>, int> emap;
  int edge(int x, int y) const {
    auto it = emap.find({std::min(x, y), std::max(x, y)});
    return it == emap.end() ? -1 : it->second;
  }
};

inline Subdivided loop_step(const LocalMesh& M) {
  const HalfEdges he(M);
  const size_t nw = M.W.empty() ? 0 : M.W[0].size();
  Subdivided S;
  S.vmap.assign(M.W.size(), -1);
  // vertex points (complete one-ring)
  for (int v = 0; v < (int)M.W.size(); ++v) {
    int start = -1;
    for (const auto& f : M.F)
      for (int k = 0; k < 3; ++k)
        if (f[k] == v) start = f[(k + 1) % 3];
    if (start < 0) continue;
    const std::vector<int> r = he.ring(v, start);
    if (r.empty()) continue;
    const int n = (int)r.size();
    double beta, self;
    if (n == 6) {
      beta = 0.0625;
      self = 0.625;
    } else {
      const double t = 0.375 + 0.25 * std::cos(2.0 * M_PI / n);
      beta = (0.625 - t * t) / n;
      self = 1.0 - n * beta;
    }
    std::vector<double> w(nw, 0.0);
    axpy(w, self, M.W[v]);
    for (int x : r) axpy(w, beta, M.W[x]);
    S.vmap[v] = (int)S.M.W.size();
    S.M.W.push_back(std::move(w));
  }
  // edge points (both faces present)
  for (const auto& f : M.F)
    for (int k = 0; k < 3; ++k) {
      const int x = f[k], y = f[(k + 1) % 3];
      const std::pair<int, int> key{std::min(x, y), std::max(x, y)};
      if (S.emap.count(key)) continue;
      const int r1 = he.turn(x, y), r2 = he.turn(y, x);
      if (r1 < 0 || r2 < 0) continue;
      std::vector<double> w(nw, 0.0);
      axpy(w, 0.375, M.W[x]);
      axpy(w, 0.375, M.W[y]);
      axpy(w, 0.125, M.W[r1]);
      axpy(w, 0.125, M.W[r2]);
      S.emap[key] = (int)S.M.W.size();
      S.M.W.push_back(std::move(w));
    }
  // children whose three nodes exist
  for (const auto& f : M.F) {
    const int x = f[0], y = f[1], z = f[2];
    const int mxy = S.edge(x, y), myz = S.edge(y, z), mzx = S.edge(z, x);
    const int X = S.vmap[x], Y = S.vmap[y], Z = S.vmap[z];
    if (X >= 0 && mxy >= 0 && mzx >= 0) S.M.F.push_back({X, mxy, mzx});
    if (Y >= 0 && myz >= 0 && mxy >= 0) S.M.F.push_back({Y, myz, mxy});
    if (Z >= 0 && mzx >= 0 && myz >= 0) S.M.F.push_back({Z, mzx, myz});
    if (mxy >= 0 && myz >= 0 && mzx >= 0) S.M.F.push_back({mxy, myz, mzx});
  }
  return S;
}

// Patch of the face (a, b, c) in patch order; empty when the mesh does not
// hold it or b / c are not regular.  N = valence of a.
inline std::vector<int> read_patch(const LocalMesh& M, int a, int b, int c, int& N) {
  const HalfEdges he(M);
  const std::vector<int> ra = he.ring(a, b);
  if (ra.size() < 3 || ra[1] != c) return {};
  N = (int)ra.size();
  const std::vector<int> rb = he.ring(b, c), rc = he.ring(c, a);
  if (rb.size() != 6 || rc.size() != 6) return {};
  std::vector<int> P(N + 6, -1);
  P[0] = a;
  for (int k = 0; k < N; ++k) P[slot_n(N, k)] = ra[k];
  // rb = c, a, n_{N-1}, b_far1, b_far0, d ; rc = a, b, d, c_far0, c_far1, n_2
  if (rb[1] != a || rb[2] != ra[N - 1] || rc[1] != b || rc[2] != rb[5] || rc[5] != ra[2 % N]) return {};
  P[N + 1] = rb[5];
  P[N + 2] = rb[4];
  P[N + 3] = rb[3];
  P[N + 4] = rc[3];
  P[N + 5] = rc[4];
  return P;
}

// Builds the table of valence N; false if a child patch could not be read.
inline bool build_table(int N, std::vector<double>& tab) {
  static const int kStamSlot[12] = {5, 4, 6, 0, 3, 9, 1, 2, 11, 8, 7, 10};
  const int np = N + 6;
  tab.assign((size_t)kLevels * 3 * 12 * np, 0.0);
  std::vector<std::vector<double>> cur(np, std::vector<double>(np, 0.0));
  for (int j = 0; j < np; ++j) cur[j][j] = 1.0;
  for (int n = 1; n <= kLevels; ++n) {
    const LocalMesh M = patch_mesh(N, cur);
    const Subdivided S = loop_step(M);
    const int a1 = S.vmap[0], b1 = S.vmap[1], c1 = S.vmap[2];
    const int mab = S.edge(0, 1), mbc = S.edge(1, 2), mca = S.edge(2, 0);
    if (a1 < 0 || b1 < 0 || c1 < 0 || mab < 0 || mbc < 0 || mca < 0) return false;
    const int kids[3][3] = {{mab, b1, mbc}, {mbc, mca, mab}, {mca, mbc, c1}};
    for (int k = 0; k < 3; ++k) {
      int Nk = 0;
      const std::vector<int> P = read_patch(S.M, kids[k][0], kids[k][1], kids[k][2], Nk);
      if (P.empty() || Nk != 6) return false;
      double* T = tab.data() + ((size_t)(n - 1) * 3 + k) * 12 * np;
      for (int s = 0; s < 12; ++s) {
        const std::vector<double>& w = S.M.W[P[kStamSlot[s]]];
        for (int j = 0; j < np; ++j) T[s * np + j] = w[j];
      }
    }
    int Nc = 0;
    const std::vector<int> C = read_patch(S.M, a1, mab, mca, Nc);
    if (C.empty() || Nc != N) return false;
    std::vector<std::vector<double>> next(np);
    for (int j = 0; j < np; ++j) next[j] = S.M.W[C[j]];
    cur.swap(next);
  }
  return true;
}

}  // namespace shl_subdiv

#endif  // SHL_SUBDIV_H_
