// shl_host.cpp -- host helpers of the C ABI: the icosphere generator, the OFF
// reader, the seeded imperfection, default parameters, version and status text.
//
// The icosphere rule reproduces the reference's icosasphere3.off and
// icosasphere4.off byte for byte: the 12 icosahedron vertices (+-1, +-phi, 0),
// (0, +-1, +-phi), (+-phi, 0, +-1) normalised, 20 faces, and per refinement
// each face (a,b,c) -> (a,ab,ca), (b,bc,ab), (c,ca,bc), (ab,bc,ca) with the
// edge midpoints appended on first use, pushed to the unit sphere; the result is
// written with "%g" and read back, so coordinates are those of the OFF text
// (as the reference reads them, shell.C:167).
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "../../include/shl.h"

namespace {

thread_local std::string g_host_err;

std::string icosphere_text(uint32_t level) {
  const double t = (1.0 + std::sqrt(5.0)) / 2.0;
  const double base[12][3] = {{-1, t, 0}, {1, t, 0}, {-1, -t, 0}, {1, -t, 0}, {0, -1, t}, {0, 1, t},
                              {0, -1, -t}, {0, 1, -t}, {t, 0, -1}, {t, 0, 1}, {-t, 0, -1}, {-t, 0, 1}};
  std::vector<double> V;
  auto push_unit = [&](double x, double y, double z) {
    const double l = std::sqrt(x * x + y * y + z * z);
    V.push_back(x / l);
    V.push_back(y / l);
    V.push_back(z / l);
  };
  for (auto& p : base) push_unit(p[0], p[1], p[2]);
  std::vector<uint32_t> Fc = {0, 11, 5, 0, 5, 1, 0, 1, 7, 0, 7, 10, 0, 10, 11, 1, 5, 9, 5, 11, 4, 11, 10, 2, 10, 7, 6,
                              7, 1, 8, 3, 9, 4, 3, 4, 2, 3, 2, 6, 3, 6, 8, 3, 8, 9, 4, 9, 5, 2, 4, 11, 6, 2, 10,
                              8, 6, 7, 9, 8, 1};
  for (uint32_t l = 0; l < level; ++l) {
    std::map<std::pair<uint32_t, uint32_t>, uint32_t> mid;
    auto midpoint = [&](uint32_t a, uint32_t b) {
      const auto key = std::make_pair(a < b ? a : b, a < b ? b : a);
      auto it = mid.find(key);
      if (it != mid.end()) return it->second;
      push_unit((V[3 * a] + V[3 * b]) / 2, (V[3 * a + 1] + V[3 * b + 1]) / 2, (V[3 * a + 2] + V[3 * b + 2]) / 2);
      const uint32_t id = (uint32_t)(V.size() / 3 - 1);
      mid[key] = id;
      return id;
    };
    std::vector<uint32_t> Fn;
    Fn.reserve(Fc.size() * 4);
    for (size_t f = 0; f < Fc.size(); f += 3) {
      const uint32_t a = Fc[f], b = Fc[f + 1], c = Fc[f + 2];
      const uint32_t ab = midpoint(a, b), bc = midpoint(b, c), ca = midpoint(c, a);
      const uint32_t add[12] = {a, ab, ca, b, bc, ab, c, ca, bc, ab, bc, ca};
      Fn.insert(Fn.end(), add, add + 12);
    }
    Fc.swap(Fn);
  }
  std::string s = "OFF\n" + std::to_string(V.size() / 3) + " " + std::to_string(Fc.size() / 3) + " 0\n";
  char buf[96];
  for (size_t i = 0; i < V.size(); i += 3) {
    std::snprintf(buf, sizeof(buf), "%g %g %g\n", V[i], V[i + 1], V[i + 2]);
    s += buf;
  }
  for (size_t f = 0; f < Fc.size(); f += 3) {
    std::snprintf(buf, sizeof(buf), "3 %u %u %u\n", Fc[f], Fc[f + 1], Fc[f + 2]);
    s += buf;
  }
  return s;
}

// parse OFF text (triangles only)
bool parse_off(const std::string& text, std::vector<double>& X, std::vector<uint32_t>& T) {
  const char* p = text.c_str();
  char* end = nullptr;
  while (*p == ' ' || *p == '\n' || *p == '\r' || *p == '\t') ++p;
  if (std::strncmp(p, "OFF", 3) != 0) { g_host_err = "not an OFF file"; return false; }
  p += 3;
  const long nv = std::strtol(p, &end, 10); p = end;
  const long nf = std::strtol(p, &end, 10); p = end;
  std::strtol(p, &end, 10); p = end;
  if (nv <= 0 || nf <= 0) { g_host_err = "bad OFF header"; return false; }
  X.resize(3 * (size_t)nv);
  for (long i = 0; i < 3 * nv; ++i) {
    X[i] = std::strtod(p, &end);
    if (end == p) { g_host_err = "truncated OFF vertices"; return false; }
    p = end;
  }
  T.resize(3 * (size_t)nf);
  for (long f = 0; f < nf; ++f) {
    const long k = std::strtol(p, &end, 10);
    if (end == p || k != 3) { g_host_err = "OFF face is not a triangle"; return false; }
    p = end;
    for (int j = 0; j < 3; ++j) {
      const long id = std::strtol(p, &end, 10);
      if (end == p || id < 0 || id >= nv) { g_host_err = "bad OFF face index"; return false; }
      T[3 * f + j] = (uint32_t)id;
      p = end;
    }
  }
  return true;
}

// Philox-4x32-10 (Salmon et al., "Parallel random numbers: as easy as 1, 2, 3", SC'11)
void philox4x32_10(uint32_t ctr[4], uint32_t key[2]) {
  const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u, W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
  uint32_t k0 = key[0], k1 = key[1];
  for (int r = 0; r < 10; ++r) {
    const uint64_t p0 = (uint64_t)M0 * ctr[0], p1 = (uint64_t)M1 * ctr[2];
    const uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0, hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
    const uint32_t n0 = hi1 ^ ctr[1] ^ k0, n2 = hi0 ^ ctr[3] ^ k1;
    ctr[0] = n0; ctr[1] = lo1; ctr[2] = n2; ctr[3] = lo0;
    k0 += W0;
    k1 += W1;
  }
}

}  // namespace

extern "C" {

shl_status shl_icosphere_off(uint32_t level, char* buf, size_t cap, size_t* len) {
  if (level > 9) return SHL_ERR_ARG;
  const std::string s = icosphere_text(level);
  if (len) *len = s.size();
  if (buf) {
    if (cap < s.size() + 1) return SHL_ERR_CAPACITY;
    std::memcpy(buf, s.c_str(), s.size() + 1);
  }
  return SHL_OK;
}

shl_status shl_icosphere(uint32_t level, double* xyz, size_t cap_nodes, uint32_t* faces, size_t cap_faces,
                         uint32_t* n_nodes, uint32_t* n_faces) {
  if (level > 9) return SHL_ERR_ARG;
  std::vector<double> X;
  std::vector<uint32_t> T;
  if (!parse_off(icosphere_text(level), X, T)) return SHL_ERR_ARG;
  if (n_nodes) *n_nodes = (uint32_t)(X.size() / 3);
  if (n_faces) *n_faces = (uint32_t)(T.size() / 3);
  if (xyz) {
    if (cap_nodes < X.size() / 3) return SHL_ERR_CAPACITY;
    std::memcpy(xyz, X.data(), X.size() * sizeof(double));
  }
  if (faces) {
    if (cap_faces < T.size() / 3) return SHL_ERR_CAPACITY;
    std::memcpy(faces, T.data(), T.size() * sizeof(uint32_t));
  }
  return SHL_OK;
}

shl_status shl_read_off(const char* path, double* xyz, size_t cap_nodes, uint32_t* faces, size_t cap_faces,
                        uint32_t* n_nodes, uint32_t* n_faces) {
  if (!path) return SHL_ERR_ARG;
  FILE* fp = std::fopen(path, "rb");
  if (!fp) { g_host_err = std::string("cannot open ") + path; return SHL_ERR_ARG; }
  std::string text;
  char chunk[65536];
  size_t n;
  while ((n = std::fread(chunk, 1, sizeof(chunk), fp)) > 0) text.append(chunk, n);
  std::fclose(fp);
  std::vector<double> X;
  std::vector<uint32_t> T;
  if (!parse_off(text, X, T)) return SHL_ERR_ARG;
  if (n_nodes) *n_nodes = (uint32_t)(X.size() / 3);
  if (n_faces) *n_faces = (uint32_t)(T.size() / 3);
  if (xyz) {
    if (cap_nodes < X.size() / 3) return SHL_ERR_CAPACITY;
    std::memcpy(xyz, X.data(), X.size() * sizeof(double));
  }
  if (faces) {
    if (cap_faces < T.size() / 3) return SHL_ERR_CAPACITY;
    std::memcpy(faces, T.data(), T.size() * sizeof(uint32_t));
  }
  return SHL_OK;
}

shl_status shl_gaussian_normal_imperfection(const double* xyz, uint32_t n_nodes, double amplitude, uint64_t seed,
                                            double* u_out) {
  if (!xyz || !u_out) return SHL_ERR_ARG;
  for (uint32_t i = 0; i < n_nodes; ++i) {
    uint32_t ctr[4] = {i, 0x5348454Cu, 0u, 0u};  // counter: node id, "SHEL"
    uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
    philox4x32_10(ctr, key);
    const double two53 = 9007199254740992.0;
    const double u1 = ((double)(((uint64_t)(ctr[0] >> 5) << 26) | (ctr[1] >> 6)) + 0.5) / two53;
    const double u2 = ((double)(((uint64_t)(ctr[2] >> 5) << 26) | (ctr[3] >> 6)) + 0.5) / two53;
    const double g = std::sqrt(-2.0 * std::log(u1)) * std::cos(2.0 * M_PI * u2);
    const double* x = xyz + 3 * (size_t)i;
    const double r = std::sqrt(x[0] * x[0] + x[1] * x[1] + x[2] * x[2]);
    for (int c = 0; c < 3; ++c) u_out[3 * (size_t)i + c] = r > 0 ? amplitude * g * x[c] / r : 0.0;
  }
  return SHL_OK;
}

void shl_params_default(shl_params* p) {
  if (!p) return;
  std::memset(p, 0, sizeof(*p));
  p->shell_mass_density = 1e3;
  p->shell_young_modulus = 1e9;
  p->shell_young_modulus2 = 1e9;
  p->shell_poisson_ratio = 1.0 / 3.0;
  p->shell_shear_modulus = 0.0;
  p->bulk_modulus = 0.0;
  p->memb_stiff_mult = 1.0;
  p->bend_stiff_mult = 1.0;
  p->thickness = 1e-3;
  p->pressure_base = SHL_CS_LOCAL;
  p->pressure_dir = 2;
  p->shell_shell_contact = SHL_CONTACT_NONE;
  p->fric_stiff_mult = 1.0;
  p->friction_stop_velocity = 0.03;
  p->static_friction_tol = 0.1;
  p->cell_size_mult = 4.0;
  p->cell_margin = 0.02;
  p->neighbor_margin = 0.4;
  p->dt = 1e-6;
  p->newmark_beta = 0.25;
  p->newmark_gamma = 0.5;
  p->precision = SHL_PREC_FP64;
  p->adapt_dt_every = 0;
  p->dt_min = 0.0;
  p->dt_max = 0.0;
  p->rel_loc_err_min = 5e-5;
  p->rel_loc_err_max = 5e-4;
  p->shell_cavity_contact = 0;
  p->cavity = SHL_CAVITY_ELLIPSOID;
  p->Rx = p->Ry = p->Rz = 0.1005;
  p->mu_s_cavity = p->mu_d_cavity = 0.0;
  p->cavity_damping = p->cavity_friction_damping = 0.0;
}

const char* shl_status_string(shl_status s) {
  switch (s) {
    case SHL_OK: return "OK";
    case SHL_NO_DISP_CHANGE: return "WARNING: No change in displacement";
    case SHL_LARGE_DISP: return "WARNING: A physical solution is not guaranteed, because the increment is too large";
    case SHL_STOP_SIM: return "STOP_SIM";
    case SHL_TOO_MANY_CELLS: return "ERROR: The number of linked cells seems to have exploded";
    case SHL_SMALL_TIMESTEP: return "ERROR: The timestep is too small";
    case SHL_CONTACT_PROBLEM: return "ERROR: Problem in shell-shell contact";
    case SHL_NOT_FINITE: return "ERROR: The solution is not finite";
    case SHL_ERR_ARG: return "invalid argument";
    case SHL_ERR_CUDA: return "CUDA error";
    case SHL_ERR_TIMEOUT: return "device wait timed out";
    case SHL_ERR_OOM: return "device out of memory";
    case SHL_ERR_CAPACITY: return "device buffer capacity exceeded";
  }
  return "unknown status";
}

const char* shl_host_error(void) { return g_host_err.c_str(); }

}  // extern "C"
