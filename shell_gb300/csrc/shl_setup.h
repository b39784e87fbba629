// shl_setup.h -- host-side set-up of the shell library (internal).
//
// Everything the reference computes once in ShellSystem::set_parameters /
// build_cache / compute_mass_damping (ShellSystem.C:170-852) is computed here on
// the host, laid out for the device kernels:
//   * faces reordered so that the regular 12-node patches come first and the
//     irregular (valence != 6) patches follow, grouped by valence;
//   * patch node ids slot-major (patch[slot * n_faces + face]) for coalesced loads;
//   * one universal table of unrotated basis values per patch type (the basis
//     at the quadrature point (1/3,1/3) is the same for every face of a type),
//     plus per face the 2x2 rotation R of reinit_mod (ShellSystem.C:3321-3499);
//   * per-face reference metric and orthotropic H, structure of arrays;
//   * lumped masses / damping, the gather CSR (node -> (face, slot) entries in
//     ascending order) and the topological exclusion CSR (close_elems).
#ifndef SHL_SETUP_H_
#define SHL_SETUP_H_

#include <cstdint>
#include <string>
#include <vector>

#include "../../include/shl.h"

namespace shl {

// Number of per-face FP64 constants (structure of arrays, field-major).
enum FaceField {
  FF_R00, FF_R01, FF_R10, FF_R11,  // rotation onto the material frame
  FF_JXW,                          // Jacobian x weight of the first map
  FF_X0, FF_X1, FF_X2,             // quadrature point, reference
  FF_A10, FF_A11, FF_A12,          // a_ref.vec[0]
  FF_A20, FF_A21, FF_A22,          // a_ref.vec[1]
  FF_D10, FF_D11, FF_D12,          // a_ref.dvec[0]  (d2x/ds1^2)
  FF_D20, FF_D21, FF_D22,          // a_ref.dvec[1]  (d2x/ds2^2)
  FF_D30, FF_D31, FF_D32,          // a_ref.dvec[2]  (d2x/ds1ds2)
  FF_G0, FF_G1, FF_G2,             // a_ref.ff1 (Voigt, no factor 2)
  FF_B0, FF_B1, FF_B2,             // a_ref.ff2
  FF_H00, FF_H01, FF_H02, FF_H11, FF_H12, FF_H22,  // orthotropic H incl. 1/det^2
  FF_K, FF_D,                      // membrane and bending stiffness of the face's shell
  FF_COUNT
};

// Per-face FP32 constants of the FP32 element path (structure of arrays).
// The strains are formed from the displacement relative to this reference
// geometry, so no difference of nearly equal metrics is taken.
enum FaceField32 {
  F32_R00, F32_R01, F32_R10, F32_R11, F32_JXW,
  F32_X0, F32_X1, F32_X2,
  F32_A10, F32_A11, F32_A12, F32_A20, F32_A21, F32_A22,
  F32_D10, F32_D11, F32_D12, F32_D20, F32_D21, F32_D22, F32_D30, F32_D31, F32_D32,
  F32_G0, F32_G1, F32_G2,          // a_ref.ff1
  F32_N0, F32_N1, F32_N2, F32_L0,  // unit normal and |a1 x a2| of the reference
  F32_H00, F32_H01, F32_H02, F32_H11, F32_H12, F32_H22,
  F32_K, F32_D,
  F32_COUNT
};

struct PatchGroup {
  int valence;        // valence of the first vertex (6 = regular)
  int n_slots;        // valence + 6
  uint32_t first;     // first internal face of the group
  uint32_t count;     // faces in the group
  uint32_t slot_base; // first element-force slot of the group: face i of the group owns
                      // slots slot_base + (i - first) * n_slots + [0, n_slots)
  std::vector<double> basis;  // n_slots x 6 (phi, d/dv, d/dw, d2/dv2, d2/dw2, d2/dvdw)
};

struct Setup {
  uint32_t V = 0, F = 0;
  std::vector<double> X;           // 3V node-major
  std::vector<uint32_t> tri;       // 3F original order
  std::vector<uint32_t> perm;      // internal face -> original face id
  std::vector<uint32_t> inv_perm;  // original -> internal
  std::vector<PatchGroup> groups;  // groups[0] = regular
  uint32_t patch_rows = 12;        // slot rows of `patch` (the largest n_slots, at least 12)
  uint32_t n_slots_total = 0;      // element-force slots of all faces (sum of n_slots)
  std::vector<int32_t> patch;      // [slot * F + internal face], -1 for unused slots
  std::vector<double> face;        // [field * F + internal face]
  std::vector<float> face32;       // [FaceField32 * F + internal face]
  std::vector<float> face_df;      // the same constants as float pairs: hi [fld * F + i], lo [(F32_COUNT + fld) * F + i]
  std::vector<double> Minv, C;     // 3V node-major
  std::vector<uint32_t> gather_ptr;  // V+1
  std::vector<uint32_t> gather_ent;  // element-force slot (PatchGroup::slot_base), ascending per node
  std::vector<uint32_t> slot_pos;    // per element-force slot: its position k in gather_ent (the inverse)
  std::vector<uint32_t> node_face_ptr;  // V+1: faces of which each node is a vertex
  std::vector<uint32_t> node_face;      // original face ids, ascending internal order
  std::vector<uint32_t> close_ptr;   // F+1 (original ids)
  std::vector<uint32_t> close_list;  // sorted original ids
  uint64_t n_cells_max = 0;
  // derived constants (update_derived, ShellSystem.C:421-487)
  double K = 0, D = 0, stiff_density = 0, stiff_static_friction = 0, d2_friction = 0;
};

// Builds everything; returns false with a message on unsupported input.
bool build_setup(const shl_mesh& mesh, const shl_params& p, Setup& out, std::string& err);

// Concatenates the set-ups of independent shells into one (node and face
// ids offset shell by shell, faces regrouped so that each patch group spans
// all shells).  node_off/face_off (n+1 entries) get the original-order
// offsets of each shell; face_shell gets the shell of every original face.
bool merge_setups(std::vector<Setup>& shells, Setup& out, std::vector<uint32_t>& node_off,
                  std::vector<uint32_t>& face_off, std::vector<uint32_t>& face_shell, std::string& err);

// Loop box-spline basis of a regular patch at (v, w) in this library's patch
// order; out[6*slot + k].  Exposed for tests through the C ABI helpers.
void regular_basis(double v, double w, double* out);
// Basis of a patch whose first vertex has valence n at the quadrature point
// of the middle sub-triangle; out[6*slot + k] for n + 6 slots.
void irregular_basis(int n, double v, double w, double* out);

// Sets the message returned by shl_last_error() on this thread.
void set_error(const std::string& msg);

}  // namespace shl

#endif
