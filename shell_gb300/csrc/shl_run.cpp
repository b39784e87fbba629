// shl_run.cpp -- the command-line program of the library: the time loop of
// shell.C (shell.C:43-395) over the C ABI instead of ShellSystem::advance.
//
//   shl_run [-c configfile] [-l loadfile] [-m meshfile] [-d datadir] [-<name> <value> ...] [--dry-run]
//
// What it keeps from the reference:
//   * the config file format (name = value, '#' comments) and "-name value"
//     command-line overrides (macros.h:15-21), with the same warnings for
//     missing and unrecognised parameters (shell.C:241-256);
//   * "[function]" parameters as expressions of t (macros.h:51-60): the
//     pressure is evaluated by the host at every step's time and handed to the
//     device as a per-step table; the stopping criterion is tested before each
//     step (shell.C:314-318);
//   * mesh preparation: OFF file, uniform refinement, project, scale, rotate,
//     translate (shell.C:145-229); the initial distortion with srand48/drand48
//     (ShellSystem.C:316-317, 864-869);
//   * output: the property table (ShellSystem.h:454-464, ShellSystem.C:
//     2849-2893) every data_time, shell%010u.vtu every vtk_time, state files
//     shell_state%010u.dat every state_time wall seconds and at the end with
//     the shell_state_latest.dat link (shell.C:102-105, 343-392); exit codes
//     SUCCESS 0, TIME_LIMIT_REACHED 1, SIGNAL_CAUGHT 2, ERROR 3.
// Steps between two outputs run as one shl_step call on the device; the table
// line of an output averages the dt-weighted sums of the steps since the last
// line, as the MovingAverage accumulators do (MovingAverage.h:12-29).
//
// --dry-run parses everything, prints the resolved parameters and the first
// pressure values as one JSON line, and exits without touching a GPU.
#include <sys/stat.h>
#include <unistd.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <csignal>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <ctime>
#include <filesystem>
#include <fstream>
#include <iostream>
#include <limits>
#include <map>
#include <set>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/shl.h"
#include "shl_expr.h"

namespace {

enum ExitCode { UNFINISHED = -1, SUCCESS = 0, TIME_LIMIT_REACHED = 1, SIGNAL_CAUGHT = 2, ERROR = 3 };

volatile std::sig_atomic_t g_signal = 0;
void catch_signal(int sig) { g_signal = sig; }

std::string trim(const std::string& s) {
  size_t a = 0, b = s.size();
  while (a < b && std::isspace((unsigned char)s[a])) ++a;
  while (b > a && std::isspace((unsigned char)s[b - 1])) --b;
  return s.substr(a, b - a);
}

// The config file and command line (the GetPot calls of macros.h:15-21).
class Config {
 public:
  Config(int argc, char** argv) {
    for (int i = 1; i < argc; ++i) args_.push_back(argv[i]);
  }
  bool read(const std::string& path) {
    std::ifstream f(path);
    if (!f) return false;
    std::string line;
    while (std::getline(f, line)) {
      const size_t hash = line.find('#');
      if (hash != std::string::npos) line = line.substr(0, hash);
      const size_t eq = line.find('=');
      if (eq == std::string::npos) continue;
      const std::string name = trim(line.substr(0, eq));
      std::string value = trim(line.substr(eq + 1));
      if (value.size() >= 2 && value.front() == '\'' && value.back() == '\'') value = value.substr(1, value.size() - 2);
      if (!name.empty()) vars_[name] = value;
    }
    return true;
  }
  // command-line flag present (GetPot::search)
  bool search(const std::string& flag) {
    for (size_t i = 0; i < args_.size(); ++i)
      if (args_[i] == flag) {
        used_args_.insert(i);
        last_ = i;
        return true;
      }
    return false;
  }
  // the argument after the last searched flag (GetPot::next)
  std::string next(const std::string& def) {
    if (last_ + 1 < args_.size()) {
      used_args_.insert(last_ + 1);
      return args_[++last_];
    }
    return def;
  }
  // the text of a parameter: config value, overridden by "-name value"
  std::string text(const std::string& name, const std::string& def, bool warn = true) {
    const bool in_cfg = vars_.count(name) != 0;
    const bool in_cl = search("-" + name);
    if (!in_cfg && !in_cl && warn)
      std::cout << "WARNING: Parameter " << name << " is missing! Using default: " << def << std::endl;
    std::string v = in_cfg ? vars_[name] : def;
    used_.insert(name);
    if (in_cl) {
      search("-" + name);
      v = next(v);
    }
    return v;
  }
  double real(const std::string& name, double def) {
    std::ostringstream d;
    d << def;
    const std::string s = text(name, d.str());
    return std::strtod(s.c_str(), nullptr);
  }
  unsigned uint(const std::string& name, unsigned def) {
    const std::string s = text(name, std::to_string(def));
    return (unsigned)std::strtoul(s.c_str(), nullptr, 10);
  }
  bool boolean(const std::string& name, bool def, bool warn = true) {
    std::string s = text(name, def ? "true" : "false", warn);
    std::transform(s.begin(), s.end(), s.begin(), ::tolower);
    return s == "true" || s == "1" || s == "yes" || s == "on";
  }
  std::string upper(const std::string& name, const std::string& def, bool warn = true) {
    std::string s = text(name, def, warn);
    std::transform(s.begin(), s.end(), s.begin(), ::toupper);
    return s;
  }
  std::vector<std::string> unused_variables() const {
    std::vector<std::string> out;
    for (const auto& kv : vars_)
      if (!used_.count(kv.first)) out.push_back(kv.first);
    return out;
  }
  std::vector<std::string> unused_arguments() const {
    std::vector<std::string> out;
    for (size_t i = 0; i < args_.size(); ++i)
      if (!used_args_.count(i)) out.push_back(args_[i]);
    return out;
  }

 private:
  std::vector<std::string> args_;
  std::set<size_t> used_args_;
  size_t last_ = 0;
  std::map<std::string, std::string> vars_;
  std::set<std::string> used_;
};

struct Function {
  std::string name;
  shl::expr::Expression e;
  double value = 0;
};

struct Error : std::runtime_error {
  using std::runtime_error::runtime_error;
};

// [function] parameter: parse, evaluate at t = 0
Function function(Config& cfg, const std::string& name, const std::string& def) {
  Function f;
  f.name = name;
  try {
    f.e = shl::expr::Expression(cfg.text(name, def));
  } catch (const std::exception& ex) {
    throw Error("ERROR: " + std::string(ex.what()));
  }
  f.value = f.e.eval({{"t", 0.0}, {"d", 0.0}});
  return f;
}

std::vector<double> vector3(Config& cfg, const std::string& name, double def) {
  std::ostringstream d;
  d << def << "," << def << "," << def;
  shl::expr::Expression e(cfg.text(name, d.str()));
  if (e.size() != 3) throw Error("ERROR: " + name + " needs three components");
  return {e.eval({}, 0), e.eval({}, 1), e.eval({}, 2)};
}

// uniform refinement: every face (a,b,c) -> (a,ab,ca), (b,bc,ab), (c,ca,bc),
// (ab,bc,ca) with the edge midpoints appended on first use
void refine(std::vector<double>& X, std::vector<uint32_t>& T) {
  std::map<std::pair<uint32_t, uint32_t>, uint32_t> mid;
  auto midpoint = [&](uint32_t a, uint32_t b) {
    const auto key = std::make_pair(std::min(a, b), std::max(a, b));
    auto it = mid.find(key);
    if (it != mid.end()) return it->second;
    for (int c = 0; c < 3; ++c) X.push_back(0.5 * (X[3 * a + c] + X[3 * b + c]));
    const uint32_t id = (uint32_t)(X.size() / 3 - 1);
    mid[key] = id;
    return id;
  };
  std::vector<uint32_t> out;
  out.reserve(4 * T.size());
  for (size_t f = 0; f < T.size(); f += 3) {
    const uint32_t a = T[f], b = T[f + 1], c = T[f + 2];
    const uint32_t ab = midpoint(a, b), bc = midpoint(b, c), ca = midpoint(c, a);
    const uint32_t add[12] = {a, ab, ca, b, bc, ab, c, ca, bc, ab, bc, ca};
    out.insert(out.end(), add, add + 12);
  }
  T.swap(out);
}

// z-x-z Euler rotation by the angles (phi, theta, psi), given in turns
void rotate(std::vector<double>& X, double phi, double theta, double psi) {
  const double tau = 2.0 * 3.141592653589793238462643383279502884;
  auto rz = [](double a, double R[3][3]) {
    const double c = std::cos(a), s = std::sin(a);
    double M[3][3] = {{c, -s, 0}, {s, c, 0}, {0, 0, 1}};
    std::memcpy(R, M, sizeof(M));
  };
  double A[3][3], B[3][3], C[3][3], AB[3][3], R[3][3];
  rz(phi * tau, A);
  {
    const double c = std::cos(theta * tau), s = std::sin(theta * tau);
    double M[3][3] = {{1, 0, 0}, {0, c, -s}, {0, s, c}};
    std::memcpy(B, M, sizeof(M));
  }
  rz(psi * tau, C);
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      AB[i][j] = 0;
      for (int k = 0; k < 3; ++k) AB[i][j] += C[i][k] * B[k][j];
    }
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      R[i][j] = 0;
      for (int k = 0; k < 3; ++k) R[i][j] += AB[i][k] * A[k][j];
    }
  for (size_t n = 0; n < X.size(); n += 3) {
    const double x[3] = {X[n], X[n + 1], X[n + 2]};
    for (int i = 0; i < 3; ++i) X[n + i] = R[i][0] * x[0] + R[i][1] * x[1] + R[i][2] * x[2];
  }
}

std::string timestamp(const char* fmt) {
  char buf[32];
  std::time_t raw = std::time(nullptr);
  std::strftime(buf, sizeof(buf), fmt, std::localtime(&raw));
  return buf;
}

// the dt-weighted sums since the last table line (the MovingAverage state)
struct Averages {
  double n = 0;
  // dt, area, vol, pcav, Nc_cav, Nc, Ekin, Etens, Ebend, Ecav, Eself, Efric, kGauss, kMean
  double s[14] = {0};
  void add_report(const shl_step_report& r) {
    n += r.steps_done;
    const double v[14] = {r.sum_dt,    r.sum_area,  r.sum_volume, r.sum_pcav,  r.sum_Nc_cav, r.sum_Nc,     r.sum_Ekin,
                          r.sum_Etens, r.sum_Ebend, r.sum_Ecav,   r.sum_Eself, r.sum_Efric,  r.sum_kGauss, r.sum_kMean};
    for (int k = 0; k < 14; ++k) s[k] += v[k];
  }
  void add_sample(double dt, const shl_energies& e, double Ekin, double pcav) {
    n += 1;
    const double v[14] = {dt,         dt * e.area,  dt * e.volume, dt * pcav,   dt * e.Nc_cav, dt * e.Nc,
                          dt * Ekin,  dt * e.Etens, dt * e.Ebend,  dt * e.Ecav, dt * e.Eself,  dt * e.Efric,
                          dt * e.kGauss, dt * e.kMean};
    for (int k = 0; k < 14; ++k) s[k] += v[k];
  }
  // n rows of the mean sample: keeps both the sums and the count in a state file
  std::vector<double> rows() const {
    std::vector<double> out;
    for (int i = 0; i < (int)n; ++i)
      for (int k = 0; k < 14; ++k) out.push_back(s[k] / n);
    return out;
  }
  void load_rows(const std::vector<double>& r, uint32_t nr) {
    n = nr;
    for (uint32_t i = 0; i < nr; ++i)
      for (int k = 0; k < 14; ++k) s[k] += r[14 * i + k];
  }
};

void print_header() {
  std::cout << "  timestamp    step       dt          time        wall_time "
            << "area        volume      density     pressure    Nc_cav      Nc_self     "
            << "E_kin       E_tens      E_bend      E_cav       E_self      E_fric      kGauss      kMean      \n"
            << std::string(60 + 72 + 95, '-') << std::endl;
}

// cavity surface and volume, ShellSystem.C:441-468 (box; cylinder with axis x; ellipsoid)
void cavity_size(int type, const double* R, double* surface, double* volume) {
  const double Rx = R[0], Ry = R[1], Rz = R[2], pi = 3.141592653589793238;
  if (type == SHL_CAVITY_BOX) {
    *surface = 8 * (Rx * Ry + Rx * Rz + Ry * Rz);
    *volume = 8 * Rx * Ry * Rz;
  } else if (type == SHL_CAVITY_CYLINDER) {
    const double lambda = (Ry - Rz) / (Ry + Rz);
    const double lambda32 = 3 * lambda * lambda;
    *surface = 2 * pi * ((Ry + Rz) * (1 + lambda32 / (10 + std::sqrt(4 - lambda32))) + Ry * Rz);
    *volume = 2 * pi * Rx * Ry * Rz;
  } else {
    *surface = 4 * pi * std::pow((std::pow(Rx * Ry, 1.6) + std::pow(Rx * Rz, 1.6) + std::pow(Ry * Rz, 1.6)) / 3, 0.625);
    *volume = 4. / 3 * pi * Rx * Ry * Rz;
  }
}

// density: the packing density of the last measurement (area h / cavity volume), 0 without cavity
void print_properties(Averages& avg, uint32_t time_step, double time, double secs_running, double density) {
  if (avg.n == 0) return;
  const double adt = avg.s[0] / avg.n;
  if (secs_running < 1) secs_running = std::floor(secs_running * 1e7) * 1e-7;
  auto a = [&](int k) { return (avg.s[k] / avg.n) / adt; };
  char line[512];
  std::snprintf(line, sizeof(line),
                "%12s %10d %11.6g %11.6g %9.8g %11.6g %11.6g %11.6g %11.6g %11.6g %11.6g %11.6g %11.6g %11.6g "
                "%11.6g %11.6g %11.6g % 11.5g % 11.5g",
                timestamp("%y%m%d%H%M%S").c_str(), (int)time_step, adt, time, secs_running, a(1), a(2), density,
                a(3), a(4), a(5), a(6), a(7), a(8), a(9), a(10), a(11), a(12), a(13));
  std::cout << "# " << line << std::endl;
  avg = Averages();
}

const char* problem_text(int p) {
  switch (p) {
    case SHL_OK: return "CLEAR: Problem resolved";
    case SHL_NO_DISP_CHANGE: return "WARNING: No change in displacement";
    case SHL_LARGE_DISP: return "WARNING: A physical solution is not guaranteed, because the increment is too large";
    case SHL_SMALL_TIMESTEP: return "ERROR: The timestep is too small";
    case SHL_TOO_MANY_CELLS: return "ERROR: The number of linked cells seems to have exploded";
    case SHL_CONTACT_PROBLEM: return "ERROR: Problem in shell-shell contact";
    case SHL_NOT_FINITE: return "ERROR: The solution is not finite";
  }
  return "ERROR: An unknown problem occurred";
}

void json_kv(std::ostream& o, const char* k, double v, bool comma = true) {
  o << "\"" << k << "\": " << v << (comma ? ", " : "");
}

int run(int argc, char** argv) {
  const auto wall0 = std::chrono::steady_clock::now();
  auto elapsed = [&]() { return std::chrono::duration<double>(std::chrono::steady_clock::now() - wall0).count(); };
  Config cl(argc, argv);
  if (cl.search("-h") || cl.search("--help")) {
    std::cout << "Usage: " << argv[0] << " [-c configfile] [-l loadfile] [-m meshfile] [-d datadir] [options]\n";
    return SUCCESS;
  }
  const bool dry = cl.search("--dry-run");
  std::cout << "Invocation at " << timestamp("%Y-%m-%d %H:%M:%S") << ": " << argv[0];
  for (int i = 1; i < argc; ++i) std::cout << " " << argv[i];
  std::cout << "\n" << shl_version() << std::endl;

  std::signal(SIGHUP, SIG_IGN);
  std::signal(SIGQUIT, catch_signal);
  std::signal(SIGTERM, catch_signal);

  std::string cfgname = "config.cfg";
  if (cl.search("-c")) cfgname = cl.next(cfgname);
  if (!cl.read(cfgname)) {
    std::cout << "ERROR: Can't open config file \"" << cfgname << "\" for reading!\n";
    return ERROR;
  }
  std::string data_dir = "data";
  if (cl.search("-d")) data_dir = cl.next(data_dir);
  std::string load_filename;
  if (cl.search("-l")) load_filename = cl.next(load_filename);
  std::string mesh_filename;
  if (cl.search("-m")) mesh_filename = cl.next(mesh_filename);

  Config& cfg = cl;
  const unsigned time_steps = cfg.uint("time_steps", 0);
  const double walltime_limit = cfg.real("walltime_limit", 0);
  const double data_time = cfg.real("data_time", 0.01);
  const double vtk_time = cfg.real("vtk_time", 0.01);
  const double state_time = cfg.real("state_time", 0);
  if (walltime_limit < 0 || data_time < 0 || vtk_time < 0 || state_time < 0)
    throw Error("ERROR: output intervals and the wall-time limit must be >= 0");

  // ---- mesh (shell.C:145-229)
  const unsigned refinements = cfg.uint("refinements", 0);
  if (mesh_filename.empty())
    throw Error("ERROR: a closed mesh file (-m file.off) is required; the built-in open square of the "
                "reference needs boundary ghosts, which this library does not model");
  std::vector<double> X;
  std::vector<uint32_t> T;
  {
    uint32_t nv = 0, nf = 0;
    if (shl_read_off(mesh_filename.c_str(), nullptr, 0, nullptr, 0, &nv, &nf) != SHL_OK)
      throw Error("ERROR: Can't open mesh file \"" + mesh_filename + "\" for reading!");
    X.resize(3 * (size_t)nv);
    T.resize(3 * (size_t)nf);
    if (shl_read_off(mesh_filename.c_str(), X.data(), nv, T.data(), nf, &nv, &nf) != SHL_OK)
      throw Error(std::string("ERROR: ") + shl_last_error());
  }
  for (unsigned r = 0; r < refinements; ++r) refine(X, T);
  const double randomness = cfg.real("randomness", 0);
  if (randomness != 0) throw Error("ERROR: randomness != 0 (libMesh's random node distortion) is not supported");
  const std::vector<double> project = vector3(cfg, "project", 0);
  if (project[0] != 0 || project[1] != 0 || project[2] != 0)
    for (size_t n = 0; n < X.size(); n += 3) {
      double q[3] = {0, 0, 0}, l2 = 0;
      for (int c = 0; c < 3; ++c)
        if (project[c] != 0) q[c] = X[n + c] / project[c];
      for (int c = 0; c < 3; ++c) l2 += q[c] * q[c];
      const double factor = 1 / std::sqrt(l2);
      for (int c = 0; c < 3; ++c)
        if (project[c] != 0) X[n + c] *= factor;
    }
  const std::vector<double> scale = vector3(cfg, "scale", 1);
  if (scale[0] == 0 || scale[1] == 0 || scale[2] == 0) throw Error("ERROR: scale components must be nonzero");
  for (size_t n = 0; n < X.size(); n += 3)
    for (int c = 0; c < 3; ++c) X[n + c] *= scale[c];
  const std::vector<double> rot = vector3(cfg, "rotate", 0);
  if (std::fmod(rot[0], 1) != 0 || std::fmod(rot[1], 1) != 0 || std::fmod(rot[2], 1) != 0)
    rotate(X, rot[0], rot[1], rot[2]);
  const std::vector<double> translate = vector3(cfg, "translate", 0);
  for (size_t n = 0; n < X.size(); n += 3)
    for (int c = 0; c < 3; ++c) X[n + c] += translate[c];
  cfg.boolean("add_ghosts", true);  // closed meshes have no boundary, hence no ghosts
  const uint32_t V = (uint32_t)(X.size() / 3), F = (uint32_t)(T.size() / 3);

  // ---- system parameters (ShellSystem.C:170-418)
  shl_params P;
  shl_params_default(&P);
  if (cfg.uint("extra_order", 0) != 0) throw Error("ERROR: extra_order > 0 is not supported (one quadrature point)");
  std::vector<Function> fn;
  auto F_ = [&](const char* name, const char* def) -> double {
    fn.push_back(function(cfg, name, def));
    return fn.back().value;
  };
  P.shell_mass_density = F_("shell_mass_density", "1e3");
  P.shell_young_modulus = F_("shell_young_modulus", "1e9");
  P.shell_young_modulus2 = F_("shell_young_modulus2", "1e9");
  P.shell_poisson_ratio = F_("shell_poisson_ratio", "1/3");
  P.shell_shear_modulus = F_("shell_shear_modulus", "0");
  P.bulk_modulus = F_("bulk_modulus", "0");
  P.memb_stiff_mult = F_("memb_stiff_mult", "1");
  P.bend_stiff_mult = F_("bend_stiff_mult", "1");
  P.thickness = F_("thickness", "1e-3");
  const std::string cav = cfg.upper("cavity", "ELLIPSOID");
  P.cavity = cav == "BOX" ? SHL_CAVITY_BOX : cav == "CYLINDER" ? SHL_CAVITY_CYLINDER
             : cav == "ELLIPSOID" ? SHL_CAVITY_ELLIPSOID : -1;
  if (P.cavity < 0) throw Error("ERROR: unknown cavity " + cav);
  P.Rx = F_("Rx", "0.1005");
  P.Ry = F_("Ry", "0.1005");
  P.Rz = F_("Rz", "0.1005");
  cfg.upper("shell_boundary", "FREE");  // no boundary on a closed mesh
  cfg.uint("bc_coords", 7);
  cfg.uint("bc_every", 0);
  F_("bc_stiff_mult", "1");
  F_("bc_criterion", "1");
  P.damping_alpha = F_("damping_alpha", "0");
  P.damping_beta = F_("damping_beta", "0");
  P.damping_gamma = F_("damping_gamma", "0");
  const double damping_rotation = F_("damping_rotation", "0");
  const double perturbation_rate = F_("perturbation_rate", "0");
  F_("perturbation_energy", "0");
  const double gravity = F_("gravity", "0");
  cfg.uint("gravity_dir", 2);
  P.pressure = F_("pressure", "0");
  P.pressure_dir = (int32_t)cfg.uint("pressure_dir", 2);
  const double growth1 = F_("growth1", "1"), growth2 = F_("growth2", "1");
  const double mgr = F_("metric_growth_rate", "0"), cgr = F_("curvature_growth_rate", "0");
  cfg.boolean("grow_mass", true);
  const std::string pb = cfg.upper("pressure_base", "LOCAL");
  P.pressure_base = pb == "LOCAL" ? SHL_CS_LOCAL
                    : pb == "CARTESIAN" ? SHL_CS_CARTESIAN
                    : pb == "CYLINDRICAL" ? SHL_CS_CYLINDRICAL
                    : pb == "SPHERICAL" ? SHL_CS_SPHERICAL
                                        : -1;
  if (P.pressure_base < 0) throw Error("ERROR: unknown pressure_base " + pb);
  cfg.upper("growth_base", "LOCAL");
  cfg.uint("thickness_dir", 2);
  F_("volume_growth", "1");  // not read by the force evaluation (ShellSystem.C:1474-1476)
  const bool stand_still = cfg.boolean("stand_still", false);
  const std::string ssc = cfg.upper("shell_shell_contact", "NONE");
  P.shell_shell_contact = ssc == "NONE" ? SHL_CONTACT_NONE : ssc == "LINEAR" ? SHL_CONTACT_LINEAR
                                                             : ssc == "SMOOTH" ? SHL_CONTACT_SMOOTH : -1;
  if (P.shell_shell_contact < 0) throw Error("ERROR: unknown shell_shell_contact " + ssc);
  const bool cavity_contact = cfg.boolean("shell_cavity_contact", false);
  P.shell_cavity_contact = cavity_contact ? 1 : 0;
  P.mu_s = F_("mu_s", "0");
  P.mu_d = F_("mu_d", "0");
  P.mu_s_cavity = F_("mu_s_cavity", "0");
  P.mu_d_cavity = F_("mu_d_cavity", "0");
  P.self_damping = F_("self_damping", "0");
  P.cavity_damping = F_("cavity_damping", "0");
  P.self_friction_damping = F_("self_friction_damping", "0");
  P.cavity_friction_damping = F_("cavity_friction_damping", "0");
  P.fric_stiff_mult = F_("fric_stiff_mult", "1");
  P.friction_stop_velocity = cfg.real("friction_stop_velocity", P.friction_stop_velocity);
  P.static_friction_tol = cfg.real("static_friction_tol", P.static_friction_tol);
  P.cell_size_mult = cfg.real("cell_size_mult", P.cell_size_mult);
  P.cell_margin = cfg.real("cell_margin", P.cell_margin);
  P.neighbor_margin = cfg.real("neighbor_margin", P.neighbor_margin);
  P.dt = cfg.real("dt", P.dt);
  P.newmark_beta = cfg.real("newmark_beta", P.newmark_beta);
  P.newmark_gamma = cfg.real("newmark_gamma", P.newmark_gamma);
  Function stop = function(cfg, "stopping_criterion", "0");
  P.stop_on_problem = cfg.boolean("stop_on_problem", false) ? 1 : 0;
  const unsigned adapt_dt_every = cfg.uint("adapt_dt_every", 0);
  P.adapt_dt_every = adapt_dt_every;
  P.dt_min = cfg.real("dt_min", 0);
  P.dt_max = cfg.real("dt_max", 0);
  P.rel_loc_err_max = cfg.real("rel_loc_err_max", 5e-4);
  P.rel_loc_err_min = cfg.real("rel_loc_err_min", 5e-5);
  const unsigned random_seed = cfg.uint("random_seed", (unsigned)std::time(nullptr));
  const double distortion = cfg.real("distortion", 0);
  // parameters of this library only (no warning when absent)
  P.compat_zero_pressure = cfg.boolean("compat_zero_pressure", false, false) ? 1 : 0;
  const std::string prec = cfg.upper("precision", "FP64", false);
  P.precision = prec == "FP32" ? SHL_PREC_FP32 : SHL_PREC_FP64;

  // what the library does not model must be off
  auto need = [](bool ok, const std::string& what) {
    if (!ok) throw Error("ERROR: " + what + " is not supported by this library");
  };
  need(damping_rotation == 0 && perturbation_rate == 0 && gravity == 0 && !stand_still,
       "damping_rotation, perturbation_rate, gravity or stand_still");
  need(growth1 == 1 && growth2 == 1 && mgr == 0 && cgr == 0, "growth");
  for (const Function& f : fn) {
    if (f.name == "pressure" || f.name == "Rx" || f.name == "Ry" || f.name == "Rz" || f.name == "bc_stiff_mult" ||
        f.name == "bc_criterion")
      continue;
    if (!cavity_contact && f.name.find("cavity") != std::string::npos) continue;
    need(f.e.is_constant(), "a time-dependent " + f.name);
  }
  need(!stop.e.uses("x") && !stop.e.uses("y") && !stop.e.uses("z"), "a stopping criterion of x, y, z");

  auto eval_at = [](const Function& f, double t) { return f.e.eval({{"t", t}, {"d", 0.0}}); };

  for (const auto& u : cfg.unused_variables())
    std::cout << "WARNING: Unrecognized config file parameter: " << u << std::endl;
  {
    std::vector<std::string> ufo;
    for (const auto& a : cl.unused_arguments())
      if (a != "--dry-run") ufo.push_back(a);
    for (const auto& u : ufo) std::cout << "WARNING: Unrecognized command line argument: " << u << std::endl;
  }

  // element size distribution (shell.C:257-271): per face the shortest and longest edge
  double hmin = std::numeric_limits<double>::infinity(), hmax = 0, havg = 0;
  for (uint32_t f = 0; f < F; ++f) {
    double lo = std::numeric_limits<double>::infinity(), hi = 0;
    for (int k = 0; k < 3; ++k) {
      const uint32_t a = T[3 * f + k], b = T[3 * f + (k + 1) % 3];
      double l2 = 0;
      for (int c = 0; c < 3; ++c) l2 += (X[3 * a + c] - X[3 * b + c]) * (X[3 * a + c] - X[3 * b + c]);
      lo = std::min(lo, std::sqrt(l2));
      hi = std::max(hi, std::sqrt(l2));
    }
    hmin = std::min(hmin, lo);
    hmax = std::max(hmax, hi);
    havg += 0.5 * (lo + hi);
  }
  havg /= F;
  std::cout << "\nnodes   : " << V << "\nelements: " << F << "\nDOFs    : " << 3 * V << "\n"
            << "ELEMENT SIZE:\nmin: " << hmin << "\navg: " << havg << "\nmax: " << hmax << "\n" << std::endl;

  if (dry) {
    std::ostringstream o;
    o.precision(17);
    o << "{";
    json_kv(o, "nodes", V);
    json_kv(o, "faces", F);
    json_kv(o, "shell_mass_density", P.shell_mass_density);
    json_kv(o, "shell_young_modulus", P.shell_young_modulus);
    json_kv(o, "shell_young_modulus2", P.shell_young_modulus2);
    json_kv(o, "shell_poisson_ratio", P.shell_poisson_ratio);
    json_kv(o, "shell_shear_modulus", P.shell_shear_modulus);
    json_kv(o, "thickness", P.thickness);
    json_kv(o, "damping_alpha", P.damping_alpha);
    json_kv(o, "dt", P.dt);
    json_kv(o, "shell_shell_contact", P.shell_shell_contact);
    json_kv(o, "pressure_base", P.pressure_base);
    json_kv(o, "mu_s", P.mu_s);
    json_kv(o, "cell_size_mult", P.cell_size_mult);
    json_kv(o, "time_steps", time_steps);
    json_kv(o, "random_seed", random_seed);
    json_kv(o, "distortion", distortion);
    json_kv(o, "xsum", [&] { double s = 0; for (double x : X) s += x; return s; }());
    json_kv(o, "x0", X[0]);
    json_kv(o, "y0", X[1]);
    json_kv(o, "z0", X[2]);
    o << "\"pressure_at\": [";
    double t = 0;
    for (int k = 0; k < 4; ++k) {
      t += P.dt;
      o << eval_at(fn[std::find_if(fn.begin(), fn.end(), [](const Function& f) { return f.name == "pressure"; }) -
                      fn.begin()],
                   t)
        << (k < 3 ? ", " : "");
    }
    o << "], ";
    json_kv(o, "stop_at_0", eval_at(stop, 0.0), false);
    o << "}";
    std::cout << o.str() << std::endl;
    return SUCCESS;
  }
  const Function& pressure_fn = *std::find_if(fn.begin(), fn.end(), [](const Function& f) { return f.name == "pressure"; });

  // ---- output directory, copies of the inputs (shell.C:96-101, 162-163)
  std::filesystem::create_directories(data_dir);
  std::error_code ec;
  std::filesystem::copy_file(cfgname, data_dir + "/" + std::filesystem::path(cfgname).filename().string(),
                             std::filesystem::copy_options::overwrite_existing, ec);
  std::filesystem::copy_file(mesh_filename, data_dir + "/" + std::filesystem::path(mesh_filename).filename().string(),
                             std::filesystem::copy_options::overwrite_existing, ec);

  // ---- context
  shl_mesh mesh{V, F, X.data(), T.data()};
  shl_ctx* ctx = nullptr;
  shl_status st = shl_create(&mesh, &P, &ctx);
  if (st != SHL_OK) throw Error(std::string("ERROR: shl_create: ") + shl_status_string(st) + " " + shl_last_error());
  struct Guard {
    shl_ctx* c;
    ~Guard() { shl_destroy(c); }
  } guard{ctx};
  auto check = [&](shl_status s, const char* where) {
    if (s >= SHL_ERR_ARG) throw Error(std::string("ERROR: ") + where + ": " + shl_status_string(s) + " " + shl_last_error());
    return s;
  };

  uint32_t time_step = 0;
  double time = 0, wall_time = 0;
  Averages avg;
  bool loaded = false;
  if (!load_filename.empty()) {
    std::ifstream lf(load_filename);
    if (!lf) {
      std::cout << "WARNING: Can't open load file \"" << load_filename << "\" for reading! Starting new simulation.\n";
    } else {
      lf >> time_step;
      if (time_steps && time_step >= time_steps) {
        std::cout << "ERROR: Loaded state is already finished!\n";
        return SUCCESS;
      }
      std::vector<double> rows(14 * (size_t)(1u << 20));
      uint32_t nr = 0;
      double dt_loaded = 0;
      check(shl_load_state_file(ctx, load_filename.c_str(), &time_step, &dt_loaded, &wall_time, rows.data(),
                                1u << 20, &nr),
            "shl_load_state_file");
      avg.load_rows(rows, nr);
      check(shl_get_time(ctx, &time, nullptr), "shl_get_time");
      loaded = true;
      if (adapt_dt_every > 0 && dt_loaded != P.dt) {
        // with adaptive dt the saved step size is resumed (ShellSystem.C:3064-3067)
        shl_destroy(ctx);
        guard.c = nullptr;
        P.dt = dt_loaded;
        st = shl_create(&mesh, &P, &ctx);
        if (st != SHL_OK) throw Error(std::string("ERROR: shl_create: ") + shl_last_error());
        guard.c = ctx;
        check(shl_load_state_file(ctx, load_filename.c_str(), &time_step, &dt_loaded, &wall_time, nullptr, 0, &nr),
              "shl_load_state_file");
      }
    }
  }
  if (!loaded) {
    std::vector<double> u0(3 * (size_t)V, 0.0);
    srand48(random_seed);
    for (uint32_t n = 0; n < V; ++n)
      for (int c = 0; c < 3; ++c) u0[3 * n + c] += distortion * (2 * drand48() - 1) * P.thickness;
    check(shl_set_time(ctx, 0.0, 0), "shl_set_time");
    check(shl_apply_initial_conditions(ctx, u0.data(), 0.0, eval_at(pressure_fn, P.dt)),
          "shl_apply_initial_conditions");
  }
  auto fn_named = [&](const char* name) -> const Function& {
    return *std::find_if(fn.begin(), fn.end(), [&](const Function& f) { return f.name == name; });
  };
  // cavity semi-axes and packing density at time t (update_derived, measure_properties)
  auto cavity_R = [&](double t, double* R) {
    const char* names[3] = {"Rx", "Ry", "Rz"};
    for (int k = 0; k < 3; ++k) R[k] = eval_at(fn_named(names[k]), t);
  };
  auto density_at = [&](double t, double area) {
    if (!cavity_contact) return 0.0;
    double R[3], surface, volume;
    cavity_R(t, R);
    cavity_size(P.cavity, R, &surface, &volume);
    return area * P.thickness / volume;
  };
  if (cavity_contact) {
    const Function &rx = fn_named("Rx"), &ry = fn_named("Ry"), &rz = fn_named("Rz");
    if (!rx.e.is_constant() || !ry.e.is_constant() || !rz.e.is_constant())
      check(shl_set_cavity_functions(ctx, rx.e.text().c_str(), ry.e.text().c_str(), rz.e.text().c_str()),
            "shl_set_cavity_functions");
  }
  if (adapt_dt_every > 0) {
    // the step times are not known in advance: the device evaluates the
    // pressure at each attempt's time and tests the stopping criterion after each step
    check(shl_set_pressure_function(ctx, pressure_fn.e.text().c_str()), "shl_set_pressure_function");
    if (!stop.e.is_constant()) check(shl_set_stop_function(ctx, stop.e.text().c_str()), "shl_set_stop_function");
  }
  std::cout.precision(std::numeric_limits<double>::digits10 + 2);
  if (data_time > 0) print_header();
  char path[1024];
  if (!loaded) {
    if (data_time > 0) {
      shl_energies e{};
      check(shl_get_energies(ctx, &e), "shl_get_energies");
      double pcav = 0.0;
      if (cavity_contact) {
        double R[3], surface, volume;
        cavity_R(time + P.dt, R);  // the initial force evaluation's time (ShellSystem.C:892-904)
        cavity_size(P.cavity, R, &surface, &volume);
        pcav = e.cavity_force / surface;
      }
      avg.add_sample(P.dt, e, 0.0, pcav);
      print_properties(avg, time_step, time, wall_time + elapsed(), density_at(time + P.dt, e.area));
    }
    if (vtk_time > 0) {
      std::snprintf(path, sizeof(path), "%s/shell%010u.vtu", data_dir.c_str(), time_step);
      check(shl_write_vtu(ctx, path), "shl_write_vtu");
    }
  }

  int exit_code = UNFINISHED;
  int last_problem = 0;
  unsigned last_data = data_time > 0 ? (unsigned)(time / data_time) : 0;
  unsigned last_vtk = vtk_time > 0 ? (unsigned)(time / vtk_time) : 0;
  unsigned last_state = 0;
  constexpr uint32_t kMaxChunk = 4096;
  std::vector<double> table;
  while (true) {
    // plan the steps up to the next output, stop or check (the device runs them in one call)
    table.clear();
    double t = time;
    bool stop_now = false;
    if (eval_at(stop, t) != 0) {
      exit_code = SUCCESS;
      stop_now = true;
    } else if (walltime_limit > 0 && wall_time + elapsed() >= walltime_limit) {
      exit_code = TIME_LIMIT_REACHED;
      stop_now = true;
    } else if (g_signal) {
      std::cout << "Received signal " << (int)g_signal << ": " << strsignal(g_signal) << " ("
                << timestamp("%Y-%m-%d %H:%M:%S") << ")" << std::endl;
      exit_code = SIGNAL_CAUGHT;
      stop_now = true;
    }
    if (!stop_now) {
      shl_step_report rep{};
      if (adapt_dt_every > 0) {
        // steps of unknown size: run half the steps the current dt needs to the next
        // output time, so the step that crosses it is found one step at a time
        double dt_now = P.dt;
        check(shl_get_dt(ctx, &dt_now, nullptr), "shl_get_dt");
        double next_t = INFINITY;
        if (data_time > 0) next_t = std::min(next_t, (last_data + 1) * data_time);
        if (vtk_time > 0) next_t = std::min(next_t, (last_vtk + 1) * vtk_time);
        double k = std::isfinite(next_t) ? std::floor((next_t - time) / dt_now / 2) : (double)kMaxChunk;
        uint32_t n = (uint32_t)std::max(1.0, std::min(k, (double)kMaxChunk));
        if (time_steps) n = std::min<uint32_t>(n, time_steps - time_step);
        check(shl_step(ctx, n, nullptr, 1, &rep), "shl_step");
        if (rep.stopped) exit_code = SUCCESS;
      } else {
        while (table.size() < kMaxChunk) {
          if (!table.empty() && eval_at(stop, t) != 0) break;  // the next iteration stops before stepping
          t += P.dt;
          table.push_back(eval_at(pressure_fn, t));
          const uint32_t step_no = time_step + (uint32_t)table.size();
          if (data_time > 0 && (unsigned)(t / data_time) > last_data) break;
          if (vtk_time > 0 && (unsigned)(t / vtk_time) > last_vtk) break;
          if (time_steps && step_no >= time_steps) break;
        }
        check(shl_step(ctx, (uint32_t)table.size(), table.data(), 1, &rep), "shl_step");
      }
      time_step += rep.steps_done;
      time = rep.time;
      avg.add_report(rep);
      if (rep.worst_problem != last_problem) {
        std::cout << problem_text(rep.worst_problem) << " in time step " << time_step << "!" << std::endl;
        last_problem = rep.worst_problem;
      }
      const bool problem = rep.worst_problem >= SHL_STOP_SIM || (P.stop_on_problem && rep.worst_problem > 0);
      const unsigned dc = data_time > 0 ? (unsigned)(time / data_time) : 0;
      if (dc > last_data) {
        last_data = dc;
        print_properties(avg, time_step, time, wall_time + elapsed(), density_at(time, rep.last.area));
      }
      const unsigned vc = vtk_time > 0 ? (unsigned)(time / vtk_time) : 0;
      if (vc > last_vtk) {
        last_vtk = vc;
        std::snprintf(path, sizeof(path), "%s/shell%010u.vtu", data_dir.c_str(), time_step);
        check(shl_write_vtu(ctx, path), "shl_write_vtu");
      }
      if (time_steps && time_step >= time_steps) exit_code = SUCCESS;
      if (problem) exit_code = ERROR;
    }
    const unsigned sc = state_time > 0 ? (unsigned)(elapsed() / state_time) : 0;
    if (exit_code > UNFINISHED || sc > last_state) {
      last_state = sc;
      char name[64];
      std::snprintf(name, sizeof(name), "shell_state%010u.dat", time_step);
      const std::vector<double> rows = avg.rows();
      double dt_save = P.dt;
      check(shl_get_dt(ctx, &dt_save, nullptr), "shl_get_dt");
      check(shl_save_state_file(ctx, (data_dir + "/" + name).c_str(), time_step, dt_save, wall_time + elapsed(),
                                rows.empty() ? nullptr : rows.data(), (uint32_t)(rows.size() / 14)),
            "shl_save_state_file");
      const std::string latest = data_dir + "/shell_state_latest.dat";
      ::unlink(latest.c_str());
      if (::symlink(name, latest.c_str()) != 0) std::cout << "WARNING: cannot link " << latest << std::endl;
      if (exit_code > UNFINISHED) break;
    }
  }
  return exit_code;
}

}  // namespace

int main(int argc, char** argv) {
  try {
    return run(argc, argv);
  } catch (const std::exception& e) {
    std::cout << e.what() << std::endl;
    return ERROR;
  }
}
