// shl_internal.cuh -- device data layout and kernel launchers (internal).
//
// Layout in HBM (one context = one shell):
//   node vectors   u, v, a, u_pred, v_pred, p, X, Minv, C : node-major xyz, 3V doubles
//   face constants face[field * F + i], i = internal face index (regular
//                  patches first, then irregular groups), FaceField order
//   patch ids      patch[slot * F + i] (slot-major, coalesced per slot)
//   element forces qe[(i * 12 + slot) * 3 + c]: the per-(face, slot) share of
//                  f (internal minus external pressure), gathered per node
//                  through gather_ptr/gather_ent with no atomics
//   contact list   sorted by (eid1, eid2); per-pair state SoA; pair_ptr[F+1]
//                  gives each eid1's segment; per-node contact CSR for the gather
//   control block  Ctl: step scalars, problem flags, energy sums (device-resident,
//                  so a whole multi-step sequence runs without host round trips)
#ifndef SHL_INTERNAL_CUH_
#define SHL_INTERNAL_CUH_

#include <cuda_runtime.h>
#include <cstdint>

#include "shl_expr.h"
#include "shl_geom.h"
#include "shl_smooth.h"
#include <string>
#include <vector>

#include "../../include/shl.h"
#include "shl_setup.h"

namespace shl {

constexpr int kBlock = 256;          // threads per block for element / node kernels
constexpr int kMaxGroups = 8;        // patch groups (regular + irregular valences)
constexpr int kMaxSlots = 18;        // patch slots of the largest supported valence (12)
// doubles per contact pair written by the contact-force kernel
constexpr int kPairOut = 9;
constexpr int kScanTile = 2048;      // elements per block in the multi-block scan

// Patch-group description for the element kernel (in __constant__ memory).
struct GroupDesc {
  uint32_t first;       // first internal face
  uint32_t count;       // faces
  uint32_t block_start; // first block of the element launch for this group
  int32_t n_slots;
  int32_t basis_off;    // offset into the basis table (doubles)
  uint32_t slot_base;   // first element-force slot: face i owns slot_base + (i - first) * n_slots + [0, n_slots)
  uint32_t pad;
};

// All patch groups of one shell, passed by value to the element kernel; the
// basis tables live in device memory (per context).
struct ElemGroups {
  GroupDesc g[kMaxGroups];
  int32_t n;
  const double* basis;
  const float* basis32;
};

// An element-kernel variant: threads per block, arithmetic (0 FP64, 1 the
// displacement contraction as float pairs, 2 double-float throughout;
// FP32-path variants use 0) and a name for reports.
struct ElemVariant {
  int block;
  int pairs;
  const char* name;
};
constexpr int kNumElemVariants = SHL_ELEMENT_VARIANTS;
constexpr int kFirstFp32Variant = 11;
// the one-round double-float element kernel (variant kFlatVariant): one block
// of 544 threads (17 warps, 120 registers each) per SM, one face per thread
constexpr int kFlatVariant = 10;
constexpr int kFlatBlock = 544;
extern const ElemVariant kElemVariants[kNumElemVariants];

// The element launch of a context: variant, grid and patch-group block ranges for its block size.
struct ElemLaunch {
  int variant;
  uint32_t blocks;
  ElemGroups eg;
};

// Control block in device memory.
struct Ctl {
  // time stepping
  double time;
  double pressure;         // pressure of the current step
  double volume_pressure;  // bulk-modulus pressure of the current step
  double volume, volume0, area;
  uint32_t time_step;
  uint32_t table_pos;      // index into the per-step pressure table
  uint32_t table_len;      // entries uploaded (the last one repeats past the end)
  int32_t problem;         // worst problem of the current step
  int32_t worst_problem;   // worst problem since the last report reset
  int32_t halted;          // set at the end of a step whose problem stops the run
  uint32_t steps_done;
  int32_t error;           // library error (SHL_ERR_CAPACITY ...), halts the run
  uint32_t first_problem_step;
  // linked cells / contact
  double du_sum;
  double du2_pred;         // largest |u_pred - u|^2 of the prediction made ahead (fused steps)
  double avg_elem_size;
  double cell_size, d_max, d2_max;
  double bmin[3], bmax[3];
  uint32_t ncd[3];
  uint32_t rebuild;        // rebuild requested for the next rebuild pass
  uint32_t rebuild_pending; // fused steps: the corrector's pass, deferred to the next step's IF node
  uint32_t rebuild_b;       // fused steps: the predictor-side pass of the same IF node
  uint32_t n_cells;
  uint32_t n_entries;      // (cell, face) entries of the current rebuild
  uint32_t n_pairs;        // pairs in the current list
  uint32_t n_old;          // pairs in the previous list (during a rebuild)
  uint32_t n_new;          // new pairs found in the current rebuild
  uint32_t n_rebuilds;
  uint32_t n_csr;          // contact CSR entries
  uint32_t n_next;         // pairs in the list being assembled
  uint32_t csr_dirty;      // the contact CSR must be rebuilt
  uint32_t n_cand;         // candidates of the current rebuild
  // measurements of the current step
  double Etens, Ebend, Eself, Efric, Ekin, kGauss, kMean;
  uint32_t Nc;
  uint32_t pad;
  // adaptive time stepping (ShellSystem.C:1010-1044, 1104-1117)
  double dt_cur;            // time step of the next attempt
  double nm[10];            // newmark_a of dt_cur (ShellSystem.C:744-759)
  double new_dt;            // proposal of the current attempt
  uint32_t accept;          // the current attempt is accepted
  uint32_t rejections;      // repeated attempts since the last report reset
  uint32_t steps_target;    // pause once steps_done reaches it
  uint32_t paused;          // 1: steps_target reached, 2: stopping criterion true
  // cavity contact (ShellSystem.C:1600-1723)
  double cav_R[3];          // semi-axes of the current step
  double Ecav, cavity_force;
  uint32_t Nc_cav;
  uint32_t pad_cav;
  double sum_pcav, sum_Nc_cav, sum_Ecav;
  // dt-weighted sums (MovingAverage inputs)
  double sum_dt, sum_area, sum_volume, sum_Nc, sum_Ekin, sum_Etens, sum_Ebend, sum_Eself, sum_Efric,
      sum_kGauss, sum_kMean;
  // last-block counters
  uint32_t cnt[16];
};

// Per-shell linked-cell state of a batch with self-contact.  The shells of a
// batch are independent: each keeps the single-shell control block's
// linked-cell fields (its own rebuild trigger, bounds, cell size, d_max and
// cell grid) and its own contact constants, and the grids of all shells share
// one counting sort (shell s owns cells cell_base .. cell_base + n_cells).
// The control block's rebuild / rebuild_pending flags are the OR over shells.
struct ShellCell {
  // constants of the shell (ShellSystem.C:421-487 with its own thickness and moduli)
  double thickness, cell_size_mult, stiff_density, stiff_static_friction, d2_friction;
  uint64_t n_cells_max;
  uint32_t face_first, face_end;  // original face ids of the shell
  // linked-cell state (Ctl's fields of a single shell)
  double du_sum, du2_pred, avg_elem_size, cell_size, d_max, d2_max;
  double bmin[3], bmax[3];
  unsigned long long du2_acc, du2n_acc;  // largest |du|^2 of a node pass (bits of non-negative doubles)
  uint32_t ncd[3], cell_base, n_cells, n_rebuilds;
  uint32_t rebuild, rebuild_pending, rebuild_b, pad;
};

// Step constants (captured by value in each launch).
struct StepConst {
  double dt;
  double nm0, nm6, nm7, nm8;  // newmark_a[0], [6], [7], [8]
  double thickness;
  double K, D;
  double qw;
  double stiff_density, stiff_static_friction, d2_friction;
  double mu_s, mu_d, self_damping, self_friction_damping, v_stop;
  double cell_size_mult, cell_margin;
  double bulk_modulus;
  double pressure_default;
  const double* pressure_table;  // device, or null
  uint64_t n_cells_max;
  uint32_t n_cells_cap, entries_cap, pairs_cap, csr_cap, cand_cap;
  int32_t contact;   // 1 if self-contact is on (LINEAR or SMOOTH)
  int32_t smooth;    // 1 for SMOOTH (limit-surface) self-contact
  int32_t qe_df;     // element shares are double-float pairs (the FP64 variants of arithmetic 2)
  int32_t stab_off[13];  // SMOOTH: offset of the subdivision table of valence N in DevBuf::stab, or -1
  int32_t friction;  // 1 if mu_s or mu_d != 0
  int32_t pressure_base, pressure_dir;
  int32_t compat_zero_pressure;
  int32_t stop_on_problem;
  int32_t fp32;      // element forces in FP32 (relative-displacement form)
  uint32_t V, F;
  double internal_scale;  // 1, or 0 for the pressure-only force of a residual check
  const shl::expr::Op* pfun;  // pressure as a compiled expression of t (device), or null: use the table
  int32_t pfun_len;
  int32_t sfun_len;
  const shl::expr::Op* sfun;  // stopping criterion as a compiled expression of t, or null
  // adaptive time stepping: 0 = fixed dt
  uint32_t adapt_every;
  int32_t pad_adapt;
  double beta, gamma;
  double err_min, err_max, err_target;
  double dt_min_eff, dt_max_eff;
  // cavity contact
  int32_t cavity_contact, cavity_type, cavity_friction, pad_cav;
  double cav_R[3];
  double mu_s_cav, mu_d_cav, cav_damping, cav_fric_damping, static_friction_tol;
  const shl::expr::Op* rfun[3];  // semi-axes as compiled expressions of t, or null: cav_R
  int32_t rfun_len[3];
  // shells of a batch with self-contact (per-shell linked cells, DevBuf::shc);
  // 0 for a single shell, whose linked-cell state is the control block's
  uint32_t n_cs;
};

// Device buffers of one context.
struct DevBuf {
  double *X, *u, *v, *a, *up, *vp, *p, *Minv, *C;
  double* M;          // 3V lumped masses (1 / Minv), for the kinetic energy
  double* pn;         // 3V predicted positions of fused steps (written by the previous step's corrector)
  double* ap;         // 3V predicted acceleration of an adaptive attempt (adaptive dt only)
  double* cav_origin; // 3V static-friction spring origins of the cavity contacts (cavity contact only)
  double* cav_ecav;   // V cavity-contact energy density of the last step
  double* cav_efric;  // V cavity-friction energy density of the last step
  double* fcorr;      // 3V defect correction added to the FP32 force in a step, or null
  double* face;       // FF_COUNT * F
  double* pscale;     // F (internal order): factor on the step's pressure (per shell)
  int32_t* patch;     // patch_rows * F, slot-major
  double* qe;         // 3 per element-force slot, in gather order (slot_pos)
  float* face32;      // F32_COUNT * F (FP32 element path)
  float* face_df;     // 2 * F32_COUNT * F: the same constants as float pairs (double-float FP64 path)
  float* qe32;        // 3 per element-force slot, in gather order (FP32 element path)
  float4* up32;       // V, FP32 copy of u_pred (x, y, z, 0; FP32 element path)
  float4* upk;        // 2V, u_pred as float pairs: [2n] = hi (x, y, z, 0), [2n + 1] = lo (the FP64 path's contractions)
  // element force shares are stored in gather order (node by node, ascending
  // element-force slot): slot_pos maps a (face, slot) to its place, and node n's
  // shares are qe[gather_ptr[n] .. gather_ptr[n + 1])
  uint32_t *gather_ptr, *slot_pos;
  uint32_t *node_face_ptr, *node_face;  // V+1 / faces of each node (original ids; cavity contact only)
  uint32_t* tri;      // 3F original order
  uint32_t *perm;     // internal -> original
  double *area, *kG, *kM, *etens, *ebend;  // original order
  double* partial;    // per-block partial sums
  uint32_t *close_ptr, *close_list;
  // contact: per-face AABB (original order), size, cell ranges
  double *bmin, *bmax, *fsize;
  int32_t *cell_lo, *cell_hi;  // 3 per face
  uint32_t *cell_count, *cell_start, *cell_fill, *cell_items;
  uint32_t* scan_block;        // block sums for the scans
  // pair lists (double buffered: cur / old), sorted by (e1, e2)
  uint32_t *pe1[2], *pe2[2];
  uint8_t* pstick[2];
  double *pd2[2], *porig[2];   // porig: 3 per pair
  uint32_t* pair_ptr[2];       // F+1
  uint8_t* pkeep;              // keep flags of the old list
  uint32_t *new_e1, *new_e2;   // new pairs of a rebuild
  double* new_d2;
  uint32_t *new_off, *new_cnt, *new_fill;  // per face: offset, count, fill cursor of its new pairs
  uint32_t* entry_cell;        // cell of each (cell, face) entry
  float* p32;                  // 3V, FP32 copy of the positions for the candidate prefilter
  uint32_t *cand_e1, *cand_e2; // candidates that passed the cheap filters
  double* cand_d2;
  uint8_t* cand_ok;
  uint32_t* seg_count;         // per-face pair counts (F)
  double* pforce;              // kPairOut per pair: f_contact(3), v1, w1, v2, w2, Eself, Efric
  // SMOOTH contact
  double* pvw[2];              // 4 per pair: the closest-point search's (v1, w1, v2, w2), patch frames
  double* new_x;               // 4 per new pair of a rebuild
  double* cand_x;              // 4 per candidate
  double* sum_lanes;           // SHL_SUM_LANES lane sums of the face sizes (linked-cell pass)
  double* lcoef;               // per original face with a regular patch: the limit surface's power form
                               // (SHL_LIMIT_NCOEF), made before each search from the current positions
  uint32_t* inv_perm;          // original -> internal face
  int32_t* fsm;                // per original face: valence | (position of the patch's first vertex) << 8
  double* stab;                // subdivision tables of the valences present
  uint32_t *csr_count, *csr_ptr, *csr_ent, *csr_fill;  // per-node contact CSR
  // batch with self-contact: per-shell linked-cell state, shell of each
  // original face and of each node (null for a single shell)
  ShellCell* shc;
  uint32_t *face_shell, *node_shell;
  Ctl* ctl;
  double* ptable;              // per-step pressure table (capacity)
  uint32_t ptable_cap;
};

#ifdef __CUDACC__
// Limit patch of original face e at the current positions b.p (SMOOTH contact).
__device__ __forceinline__ void smooth_patch(const DevBuf& b, const StepConst& sc, uint32_t e, shl_limit_patch& lp) {
  const uint32_t i = b.inv_perm[e];
  const int N = b.fsm[e] & 0xff;
  lp.N = N;
  lp.base = b.p;
  lp.ids = reinterpret_cast<const uint32_t*>(b.patch) + i;
  lp.stride = sc.F;
  lp.tab = N == 6 ? nullptr : b.stab + sc.stab_off[N];
}

// The pair geometry's coordinates in each face's own node order (the force
// distribution's u, v, w of tri[0..2]) from the closest-point search's
// x = (v1, w1, v2, w2) in the patch frames.
__device__ __forceinline__ void smooth_coords(const DevBuf& b, uint32_t e1, uint32_t e2, const double* x,
                                              shl_pair_geom* g) {
  const uint32_t e[2] = {e1, e2};
  for (int t = 0; t < 2; ++t) {
    const int r = b.fsm[e[t]] >> 8;
    double lam[3];
    lam[r] = SHL_SUB(SHL_SUB(1.0, x[2 * t]), x[2 * t + 1]);
    lam[(r + 1) % 3] = x[2 * t];
    lam[(r + 2) % 3] = x[2 * t + 1];
    g->v[t] = lam[1];
    g->w[t] = lam[2];
  }
}
#endif

// ---- launchers (shl_kernels.cu) ----
// SMOOTH closest-point searches (shl_contact.cu): rebuild = the candidates of a
// linked-cell pass (then k_rb_narrow's acceptance), else the pairs of the list
// from their previous solution (x to pvw, d2 to pd2, dc to the pair's force
// slots 0-2, which k_contact_force reads and overwrites)
void launch_smooth_search(const DevBuf& b, const StepConst& sc, bool rebuild, cudaStream_t s);
// The condition of a graph IF node around a linked-cell pass, set to
// (ctl->rebuild && !ctl->halted) by the last block of the kernel that decides
// the rebuild (has = 0: launched outside a graph, or no IF node follows).
struct RebuildCond {
  cudaGraphConditionalHandle h;
  int has;
};
// nodes_only: the predicted state and its largest |du|^2 (ctl->du2_pred) without
// the step's scalar start, which k_begin_step then makes (fused steps)
void launch_predict(const DevBuf& b, const StepConst& sc, RebuildCond rc, cudaStream_t s, bool nodes_only = false);
void launch_begin_step(const DevBuf& b, const StepConst& sc, RebuildCond rc, cudaStream_t s);
// Fused steps make both linked-cell passes of a step boundary in one IF node:
// the corrector's (deferred, at the corrected positions) and then the
// predictor's; launch_rebuild_second sits between them.  launch_rebuild_first
// turns a deferred pass into a due one (before a direct launch_rebuild).
void launch_rebuild_second(const DevBuf& b, const StepConst& sc, cudaStream_t s);
void launch_rebuild_first(const DevBuf& b, const StepConst& sc, cudaStream_t s);
// batch with self-contact: the per-shell rebuild flags of a pass started by the
// host (mode 0: every shell, 1: the shells whose du_sum reached their tolerance,
// 2: none) and the control block's OR of them
void launch_batch_flags(const DevBuf& b, const StepConst& sc, int mode, cudaStream_t s);
// totals: also the fixed-order sums of the per-face measurements (k_elem_totals);
// k_volume_end forms them too, so launches followed by it pass false
void launch_elements(const DevBuf& b, const StepConst& sc, const ElemLaunch& el, cudaStream_t s, bool totals = true);
void launch_contact_force(const DevBuf& b, const StepConst& sc, int cur, cudaStream_t s);
// mode 2: adaptive attempt; mode 3: corrector fused with the next step's prediction
// (reads the step's predicted positions from b.pn and writes the next ones there);
// otherwise correct ? corrector : evaluation
void launch_gather_correct(const DevBuf& b, const StepConst& sc, int mode, bool correct, double* f_out,
                           double* a_out, cudaStream_t s, RebuildCond rc = {0, 0});
void launch_volume_end_step(const DevBuf& b, const StepConst& sc, bool end_step, cudaStream_t s);
void launch_positions(const DevBuf& b, const StepConst& sc, cudaStream_t s);
// u, v, a between the context and mapped page-locked host memory (device pointers of it)
void launch_state_host(const DevBuf& b, const StepConst& sc, double* hu, double* hv, double* ha, bool load,
                       cudaStream_t s);
cudaError_t init_element_kernels();
cudaError_t init_contact_kernels();
enum : uint32_t { kCtlReset = 1u, kCtlTable = 2u, kCtlArm = 4u };
void launch_ctl_begin(Ctl* ctl, uint32_t n, uint32_t flags, cudaStream_t s);
void launch_fp64_peak(double* out, int blocks, int iters, cudaStream_t s);
// allocation-free force evaluation (scratch in a static device array)
uint64_t noalloc_max_slots();
cudaError_t launch_force_noalloc(const DevBuf& ctx_b, const StepConst& sc, const ElemGroups& eg, uint32_t n_blocks,
                                 const double* u, double pressure, double* f_out, cudaStream_t s);
void launch_shell_norms(const double* f, const double* fext, const double* mass, const uint32_t* node_off,
                        uint32_t n_shells, double* out, cudaStream_t s);
void launch_defect(const double* f64, const double* f32, size_t n, double* out, cudaStream_t s);
void launch_eval_program(const void* prog, int n, const double* t, int m, double* out, cudaStream_t s);
void launch_correct_adapt(const DevBuf& b, const StepConst& sc, cudaStream_t s, RebuildCond rc = {0, 0});
void launch_flush(void* buf, size_t bytes, uint32_t tag, cudaStream_t s);

// ---- launchers (shl_contact.cu) ----
// One candidate-list update (compute_shell_shell_contact_candidates,
// ShellSystem.C:1910-2135).  Runs only when ctl->rebuild is set on the device
// (every kernel returns at once otherwise), so it can sit in a CUDA graph.
// The list lives in buffer 0; buffer 1 is scratch.
void launch_rebuild(const DevBuf& b, const StepConst& sc, cudaStream_t s);
// Rebuild the per-node contact CSR when ctl->csr_dirty is set.
void launch_contact_csr(const DevBuf& b, const StepConst& sc, cudaStream_t s);

}  // namespace shl

#endif
