// shl_io.cpp -- state files and VTU output of a context, on top of the C ABI.
//
// shl_save_state_file / shl_load_state_file keep the text layout of
// ShellSystem::save / load (ShellSystem.C:2956-3153) as shell.C writes it
// (time step first, shell.C:385-389; 17 significant digits): dt, time, wall
// time; per node "u v a" for x, y, z and the cavity spring origin; the
// dt-weighted measurement rows; the sticking self-contacts "eid1 eid2 origin".
// The reference's load reads the Nc column twice instead of Nc_cav
// (ShellSystem.C:3089-3090); here the 14 columns are read in the order they
// are written.  After a load the context is brought to the state the
// reference's apply_initial_conditions leaves with a load file
// (ShellSystem.C:872-888): volume0 = loaded volume, forced candidate list that
// keeps the loaded sticking contacts.
//
// shl_write_vtu writes the ASCII .vtu of ShellSystem::write_vtk
// (ShellSystem.C:3156-3320): reference node positions, point data ux uy uz
// and ecav efric ekin eself mass, cell data ebend etens kGauss kMean, a line
// break after every 256 values.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <iomanip>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/shl.h"
#include "shl_setup.h"

using shl::set_error;

extern "C" {

shl_status shl_save_state_file(shl_ctx* ctx, const char* path, uint32_t time_step, double dt, double wall_time,
                               const double* avg_rows, uint32_t n_rows) {
  if (!ctx || !path) return SHL_ERR_ARG;
  double t = 0;
  uint32_t step = 0;
  shl_status s = shl_get_time(ctx, &t, &step);
  if (s != SHL_OK) return s;
  // sizes through the contact query and the state (u has 3V entries)
  size_t n_pairs = 0;
  double du_sum = 0;
  s = shl_get_contact_state(ctx, nullptr, nullptr, nullptr, nullptr, 0, &n_pairs, &du_sum);
  if (s != SHL_OK) return s;
  std::vector<uint32_t> pairs(2 * n_pairs);
  std::vector<uint8_t> stick(n_pairs);
  std::vector<double> origin(3 * n_pairs);
  if (n_pairs) {
    s = shl_get_contact_state(ctx, pairs.data(), stick.data(), origin.data(), nullptr, n_pairs, &n_pairs, &du_sum);
    if (s != SHL_OK) return s;
  }
  uint32_t nv = 0;
  s = shl_context_size(ctx, &nv, nullptr);
  if (s != SHL_OK) return s;
  std::vector<double> u(3 * (size_t)nv), v(3 * (size_t)nv), a(3 * (size_t)nv), so(3 * (size_t)nv);
  s = shl_get_state(ctx, u.data(), v.data(), a.data());
  if (s != SHL_OK) return s;
  if ((s = shl_get_cavity_origins(ctx, so.data())) != SHL_OK) return s;
  std::ofstream f(path);
  if (!f) {
    set_error(std::string("cannot write ") + path);
    return SHL_ERR_ARG;
  }
  f << std::setprecision(17);
  f << time_step << "\n" << dt << "\n" << t << "\n" << wall_time << "\n";
  for (uint32_t n = 0; n < nv; ++n) {
    for (int c = 0; c < 3; ++c) f << u[3 * n + c] << "\t" << v[3 * n + c] << "\t" << a[3 * n + c] << "\t";
    f << so[3 * n] << "\t" << so[3 * n + 1] << "\t" << so[3 * n + 2] << "\n";  // cavity spring origin
  }
  f << n_rows << "\n";
  for (uint32_t r = 0; r < n_rows; ++r) {
    for (int c = 0; c < 14; ++c) f << avg_rows[14 * r + c] << (c == 13 ? "\n" : "\t");
  }
  uint32_t nc = 0;
  for (size_t k = 0; k < n_pairs; ++k) nc += stick[k] != 0;
  f << nc << "\n";
  for (size_t k = 0; k < n_pairs; ++k)
    if (stick[k])
      f << pairs[2 * k] << "\t" << pairs[2 * k + 1] << "\t" << origin[3 * k] << "\t" << origin[3 * k + 1] << "\t"
        << origin[3 * k + 2] << "\n";
  return f ? SHL_OK : SHL_ERR_ARG;
}

shl_status shl_load_state_file(shl_ctx* ctx, const char* path, uint32_t* time_step, double* dt, double* wall_time,
                               double* avg_rows, uint32_t cap_rows, uint32_t* n_rows) {
  if (!ctx || !path) return SHL_ERR_ARG;
  std::ifstream f(path);
  if (!f) {
    set_error(std::string("cannot read ") + path);
    return SHL_ERR_ARG;
  }
  uint32_t step = 0, nv = 0;
  double dtl = 0, t = 0, wt = 0;
  f >> step >> dtl >> t >> wt;
  shl_status s = shl_context_size(ctx, &nv, nullptr);
  if (s != SHL_OK) return s;
  std::vector<double> u(3 * (size_t)nv), v(3 * (size_t)nv), a(3 * (size_t)nv), so(3 * (size_t)nv);
  for (uint32_t n = 0; n < nv; ++n) {
    for (int c = 0; c < 3; ++c) f >> u[3 * n + c] >> v[3 * n + c] >> a[3 * n + c];
    f >> so[3 * n] >> so[3 * n + 1] >> so[3 * n + 2];
  }
  uint32_t rows = 0;
  f >> rows;
  for (uint32_t r = 0; r < rows; ++r)
    for (int c = 0; c < 14; ++c) {
      double x = 0;
      f >> x;
      if (avg_rows && r < cap_rows) avg_rows[14 * r + c] = x;
    }
  uint32_t nc = 0;
  f >> nc;
  std::vector<uint32_t> pairs(2 * (size_t)nc);
  std::vector<uint8_t> stick(nc, 1);
  std::vector<double> origin(3 * (size_t)nc), d2(nc, 0.0);
  for (uint32_t k = 0; k < nc; ++k) f >> pairs[2 * k] >> pairs[2 * k + 1] >> origin[3 * k] >> origin[3 * k + 1] >> origin[3 * k + 2];
  if (!f) {
    set_error(std::string("truncated state file ") + path);
    return SHL_ERR_ARG;
  }
  if (avg_rows && rows > cap_rows) {
    set_error("state file holds more measurement rows than cap_rows");
    return SHL_ERR_CAPACITY;
  }
  if ((s = shl_set_state(ctx, u.data(), v.data(), a.data())) != SHL_OK) return s;
  if ((s = shl_set_time(ctx, t, step)) != SHL_OK) return s;
  if ((s = shl_set_cavity_origins(ctx, so.data())) != SHL_OK) return s;
  if (nc) {
    if ((s = shl_set_contact_state(ctx, pairs.data(), stick.data(), origin.data(), d2.data(), nc, 0.0)) != SHL_OK)
      return s;
  }
  if ((s = shl_apply_loaded_state(ctx)) != SHL_OK) return s;
  if (time_step) *time_step = step;
  if (dt) *dt = dtl;
  if (wall_time) *wall_time = wt;
  if (n_rows) *n_rows = rows;
  return SHL_OK;
}

shl_status shl_write_vtu(shl_ctx* ctx, const char* path) {
  if (!ctx || !path) return SHL_ERR_ARG;
  uint32_t nv = 0, nf = 0;
  shl_status s = shl_context_size(ctx, &nv, &nf);
  if (s != SHL_OK) return s;
  std::vector<double> X(3 * (size_t)nv), u(3 * (size_t)nv);
  std::vector<uint32_t> T(3 * (size_t)nf);
  if ((s = shl_context_mesh(ctx, X.data(), T.data())) != SHL_OK) return s;
  if ((s = shl_get_state(ctx, u.data(), nullptr, nullptr)) != SHL_OK) return s;
  std::vector<double> kG(nf), kM(nf), et(nf), eb(nf);
  if ((s = shl_get_element_fields(ctx, kG.data(), kM.data(), et.data(), eb.data(), nullptr)) != SHL_OK) return s;
  std::vector<double> ekin(nv), ecav(nv), eself(nv), efric(nv), mass(nv);
  if ((s = shl_get_node_fields(ctx, ekin.data(), ecav.data(), eself.data(), efric.data(), mass.data())) != SHL_OK)
    return s;
  std::ofstream f(path);
  if (!f) {
    set_error(std::string("cannot write ") + path);
    return SHL_ERR_ARG;
  }
  auto array = [&](const char* type, const char* name, const std::vector<double>& vals, size_t stride, size_t off) {
    f << "        <DataArray type=\"" << type << "\" Name=\"" << name << "\" format=\"ascii\">\n";
    unsigned char count = 0;
    for (size_t i = off; i < vals.size(); i += stride) {
      f << vals[i] << " ";
      if (++count == 0) f << "\n";
    }
    f << "\n        </DataArray>\n";
  };
  f << "<?xml version=\"1.0\"?>\n";
  f << "<VTKFile type=\"UnstructuredGrid\" version=\"0.1\" byte_order=\"LittleEndian\">\n";
  f << "  <UnstructuredGrid>\n";
  f << "    <Piece NumberOfPoints=\"" << nv << "\" NumberOfCells=\"" << nf << "\">\n";
  f << "      <PointData>\n";
  array("Float64", "ux", u, 3, 0);
  array("Float64", "uy", u, 3, 1);
  array("Float64", "uz", u, 3, 2);
  array("Float64", "ecav", ecav, 1, 0);
  array("Float64", "efric", efric, 1, 0);
  array("Float64", "ekin", ekin, 1, 0);
  array("Float64", "eself", eself, 1, 0);
  array("Float64", "mass", mass, 1, 0);
  f << "      </PointData>\n";
  f << "      <CellData>\n";
  array("Float64", "ebend", eb, 1, 0);
  array("Float64", "etens", et, 1, 0);
  array("Float64", "kGauss", kG, 1, 0);
  array("Float64", "kMean", kM, 1, 0);
  f << "      </CellData>\n";
  f << "      <Points>\n";
  f << "        <DataArray type=\"Float64\" Name=\"Points\" NumberOfComponents=\"3\" format=\"ascii\">\n";
  {
    unsigned char count = 0;
    for (size_t i = 0; i < X.size(); ++i) {
      f << X[i] << " ";
      if (++count == 0) f << "\n";
    }
    f << "\n";
  }
  f << "        </DataArray>\n";
  f << "      </Points>\n";
  f << "      <Cells>\n";
  f << "        <DataArray type=\"Int64\" Name=\"connectivity\" format=\"ascii\">\n";
  {
    unsigned char count = 0;
    for (size_t i = 0; i < T.size(); ++i) {
      f << T[i] << " ";
      if (++count == 0) f << "\n";
    }
    f << "\n";
  }
  f << "        </DataArray>\n";
  f << "        <DataArray type=\"Int64\" Name=\"offsets\" format=\"ascii\">\n";
  {
    unsigned char count = 0;
    for (uint64_t i = 3; i <= 3 * (uint64_t)nf; i += 3) {
      f << i << " ";
      if (++count == 0) f << "\n";
    }
    f << "\n";
  }
  f << "        </DataArray>\n";
  f << "        <DataArray type=\"UInt8\" Name=\"types\" format=\"ascii\">\n";
  {
    unsigned char count = 0;
    for (uint32_t i = 0; i < nf; ++i) {
      f << "5 ";
      if (++count == 0) f << "\n";
    }
    f << "\n";
  }
  f << "        </DataArray>\n";
  f << "      </Cells>\n";
  f << "    </Piece>\n";
  f << "  </UnstructuredGrid>\n";
  f << "</VTKFile>\n";
  return f ? SHL_OK : SHL_ERR_ARG;
}

}  // extern "C"
