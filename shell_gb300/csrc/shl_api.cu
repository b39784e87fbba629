// shl_api.cu -- the C ABI of include/shl.h on top of the device kernels.
//
// One context = one shell on the current CUDA device, with its own stream.
// shl_step() runs n Newmark steps without host synchronisation: the steps are
// captured once into a CUDA graph of kGraphSteps steps that is replayed; the
// per-step pressure comes from a device table, problems and energies are
// accumulated in the device control block and read back once at the end.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/shl.h"
#include "shl_geom.h"
#include "shl_internal.cuh"
#include "shl_subdiv.h"
#include "shl_setup.h"

using namespace shl;

namespace {

thread_local std::string g_err;
constexpr uint32_t kGraphSteps = 16;
constexpr uint32_t kTableCap = 1u << 16;

#define SHL_CUDA_TRY(expr)                                                 \
  do {                                                                     \
    cudaError_t e_ = (expr);                                               \
    if (e_ != cudaSuccess) {                                               \
      g_err = std::string(#expr) + ": " + cudaGetErrorString(e_);          \
      return e_ == cudaErrorMemoryAllocation ? SHL_ERR_OOM : SHL_ERR_CUDA; \
    }                                                                      \
  } while (0)

}  // namespace

namespace shl {
void set_error(const std::string& msg) { g_err = msg; }
}  // namespace shl

struct shl_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  cudaStream_t side = nullptr;      // captures the bodies of conditional graph nodes
  bool conditional_ok = true;       // the driver accepted conditional nodes
  shl_params P{};
  Setup S;
  DevBuf b{};
  StepConst sc{};
  uint32_t elem_blocks = 0;
  ElemGroups eg{};                 // 256-thread block ranges (the no-allocation path)
  ElemGroups eg_bs[3]{};           // block ranges for 64, 128, 256 threads per block
  uint32_t blocks_bs[3]{};
  int var64 = -1, var32 = kFirstFp32Variant;  // chosen element-kernel variants (-1: not set yet)
  float variant_ms[kNumElemVariants]{};      // tuning times (0: not timed)
  std::vector<void*> allocs;
  cudaGraphExec_t graph = nullptr;
  cudaGraphExec_t graph1 = nullptr;
  // The graphs run fused steps (fixed dt): each corrector also predicts the next
  // step.  pred_valid: the device holds that prediction for the current state
  // (set by graph steps, cleared by every entry point that may change the state)
  bool pred_valid = false;
  // fused graph steps ran since the last collect: a corrector-side linked-cell
  // pass may be pending on the device (made by the next step, or on host access)
  bool maybe_pending = false;
  double* h_pin = nullptr;  // pinned staging buffer, 3V doubles x 3
  Ctl* h_ctl = nullptr;     // pinned copy of the device control block
  double* h_table = nullptr;  // pinned staging of the pressure table (kTableCap doubles)
  double* d_fa = nullptr;   // device f and a of shl_eval_forces, 2 x 3V doubles
  void* d_flush = nullptr;  // L2 eviction buffer of shl_time_kernel
  size_t flush_bytes = 0;
  std::vector<uint32_t> node_off, face_off;  // shell offsets (original order) of a batch
  uint32_t* d_node_off = nullptr;            // device copy (shl_residual)
  double* d_norms = nullptr;                 // per-shell |f|^2, |f_ext|^2
  double* qe64 = nullptr;                    // FP64 element shares of an FP32 context (shl_residual)
  shl::expr::Op* d_pfun = nullptr;           // compiled pressure expression (device)
  shl::expr::Op* d_sfun = nullptr;           // compiled stopping criterion (device)
  shl::expr::Op* d_rfun = nullptr;           // compiled cavity semi-axes (device), 3 programs
  std::string rfun_text[3];                  // the same, for evaluations started by the host
  double* f32 = nullptr;                     // FP32 force at the checked state (defect correction)
  // batch with self-contact: per-shell constants (empty otherwise), the shell
  // of each original face, and the shells' summed linked-cell estimates
  std::vector<ShellCell> shc_host;
  std::vector<uint32_t> face_shell;
  uint64_t bc_cells = 0, bc_entries = 0, bc_cells_max = 0;
  double bc_pairs = 0;
};

namespace {

int bs_index(int block) { return block == 64 ? 0 : block == 128 ? 1 : 2; }

// the element launch of the context's current variant for the given step constants
ElemLaunch elem_launch(const shl_ctx* c, const StepConst& sc) {
  ElemLaunch el;
  el.variant = sc.fp32 ? c->var32 : c->var64;
  if (el.variant == kFlatVariant) {
    // one face per thread over the whole mesh; the groups are found by face index
    el.blocks = (sc.F + kFlatBlock - 1) / kFlatBlock;
    el.eg = c->eg_bs[0];
    return el;
  }
  const int k = bs_index(kElemVariants[el.variant].block);
  el.blocks = c->blocks_bs[k];
  el.eg = c->eg_bs[k];
  return el;
}

}  // namespace

namespace {

template <class T>
shl_status dev_alloc(shl_ctx* c, T** p, size_t n) {
  void* q = nullptr;
  const size_t bytes = std::max<size_t>(n, 1) * sizeof(T);
  cudaError_t e = cudaMalloc(&q, bytes);
  if (e != cudaSuccess) {
    g_err = "cudaMalloc(" + std::to_string(bytes) + "): " + cudaGetErrorString(e);
    return SHL_ERR_OOM;
  }
  // zero on the context stream: the stream is non-blocking, so a default-stream
  // memset would not be ordered before the uploads that follow
  e = cudaMemsetAsync(q, 0, bytes, c->stream);
  if (e != cudaSuccess) {
    cudaFree(q);
    g_err = std::string("cudaMemsetAsync: ") + cudaGetErrorString(e);
    return SHL_ERR_CUDA;
  }
  c->allocs.push_back(q);
  *p = (T*)q;
  return SHL_OK;
}

template <class T>
shl_status upload(shl_ctx* c, T* dst, const T* src, size_t n) {
  SHL_CUDA_TRY(cudaMemcpyAsync(dst, src, n * sizeof(T), cudaMemcpyHostToDevice, c->stream));
  return SHL_OK;
}

// the control block travels through a pinned host copy (one DMA, no staging)
shl_status ctl_get(shl_ctx* c, Ctl& h) {
  Ctl* dst = c->h_ctl ? c->h_ctl : &h;
  SHL_CUDA_TRY(cudaMemcpyAsync(dst, c->b.ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, c->stream));
  SHL_CUDA_TRY(cudaStreamSynchronize(c->stream));
  if (dst != &h) std::memcpy(&h, dst, sizeof(Ctl));
  return SHL_OK;
}

shl_status ctl_put(shl_ctx* c, const Ctl& h) {
  const Ctl* src = &h;
  if (c->h_ctl) {
    std::memcpy(c->h_ctl, &h, sizeof(Ctl));
    src = c->h_ctl;
  }
  SHL_CUDA_TRY(cudaMemcpyAsync(c->b.ctl, src, sizeof(Ctl), cudaMemcpyHostToDevice, c->stream));
  SHL_CUDA_TRY(cudaStreamSynchronize(c->stream));
  return SHL_OK;
}

shl_status check_launch(const char* where) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    g_err = std::string(where) + ": " + cudaGetErrorString(e);
    return SHL_ERR_CUDA;
  }
  return SHL_OK;
}



#define SHL_TRY(expr)             \
  do {                            \
    shl_status s_ = (expr);       \
    if (s_ != SHL_OK) return s_;  \
  } while (0)

// Makes the corrector-side linked-cell pass that fused steps may have left
// pending, so the candidate list and du_sum are those of the unfused sequence
// at this point (before the host reads or changes the state).
shl_status flush_deferred_rebuild(shl_ctx* c) {
  if (!c->maybe_pending) return SHL_OK;
  c->maybe_pending = false;
  if (!c->sc.contact) return SHL_OK;
  Ctl h;
  SHL_TRY(ctl_get(c, h));
  if (!h.rebuild_pending) return SHL_OK;
  launch_rebuild_first(c->b, c->sc, c->stream);
  launch_rebuild(c->b, c->sc, c->stream);
  SHL_CUDA_TRY(cudaStreamSynchronize(c->stream));
  return check_launch("deferred linked-cell pass");
}

// entry points that read the contact state or may change the step state
shl_status host_access(shl_ctx* c) {
  SHL_TRY(flush_deferred_rebuild(c));
  c->pred_valid = false;
  return SHL_OK;
}

bool validate(const shl_params& p, std::string& err) {
  if (!(p.shell_mass_density > 0)) { err = "shell_mass_density must be > 0"; return false; }
  if (!(p.shell_young_modulus > 0) || !(p.shell_young_modulus2 > 0)) { err = "Young's moduli must be > 0"; return false; }
  if (!(p.shell_shear_modulus > 0)) { err = "shell_shear_modulus must be > 0"; return false; }
  if (!(p.shell_poisson_ratio >= 0 && p.shell_poisson_ratio < 1)) { err = "shell_poisson_ratio must be in [0,1)"; return false; }
  if (!(p.thickness > 0)) { err = "thickness must be > 0"; return false; }
  if (!(p.dt > 0) || !(p.newmark_beta > 0)) { err = "dt and newmark_beta must be > 0"; return false; }
  if (p.damping_alpha < 0 || p.damping_beta < 0 || p.damping_gamma < 0) { err = "damping must be >= 0"; return false; }
  if (p.pressure_base < SHL_CS_LOCAL || p.pressure_base > SHL_CS_SPHERICAL) { err = "bad pressure_base"; return false; }
  if (p.pressure_dir < 0 || p.pressure_dir > 2) { err = "bad pressure_dir"; return false; }
  if (p.shell_shell_contact != SHL_CONTACT_LINEAR && p.shell_shell_contact != SHL_CONTACT_SMOOTH &&
      p.shell_shell_contact != SHL_CONTACT_NONE) {
    err = "bad shell_shell_contact";
    return false;
  }
  if (p.shell_shell_contact != SHL_CONTACT_NONE) {
    if (p.mu_s < 0 || p.mu_d < 0 || p.self_damping < 0 || p.self_friction_damping < 0) { err = "contact coefficients must be >= 0"; return false; }
    if (!(p.cell_size_mult > 0) || p.cell_margin < 0 || !(p.neighbor_margin > 0)) { err = "bad linked-cell parameters"; return false; }
    if (!(p.friction_stop_velocity > 0)) { err = "friction_stop_velocity must be > 0"; return false; }
  }
  if (p.precision != SHL_PREC_FP64 && p.precision != SHL_PREC_FP32) { err = "bad precision"; return false; }
  if (p.shell_cavity_contact) {
    // ShellSystem.C:373-380
    if (p.cavity < SHL_CAVITY_BOX || p.cavity > SHL_CAVITY_ELLIPSOID) { err = "bad cavity"; return false; }
    if (p.mu_s_cavity < 0 || p.mu_d_cavity < 0 || p.cavity_damping < 0 || p.cavity_friction_damping < 0 ||
        p.static_friction_tol < 0) {
      err = "cavity coefficients must be >= 0";
      return false;
    }
    if (!(p.Rx > 0.5 * p.thickness && p.Ry > 0.5 * p.thickness && p.Rz > 0.5 * p.thickness)) {
      err = "cavity semi-axes must exceed half the thickness";
      return false;
    }
    if (!(p.friction_stop_velocity > 0)) { err = "friction_stop_velocity must be > 0"; return false; }
  }
  if (p.adapt_dt_every > 0) {
    // ShellSystem.C:300-313
    if (!(p.rel_loc_err_min >= 0) || !(p.rel_loc_err_max > p.rel_loc_err_min)) {
      err = "adaptive dt needs 0 <= rel_loc_err_min < rel_loc_err_max";
      return false;
    }
    if (p.newmark_beta == 1.0 / 6) { err = "adaptive dt: no error estimate for newmark_beta = 1/6"; return false; }
    if (p.dt_min < 0 || p.dt_max < 0 || (p.dt_min > p.dt) || (p.dt_max > 0 && p.dt_max < p.dt)) {
      err = "adaptive dt needs dt_min <= dt <= dt_max";
      return false;
    }
  }
  return true;
}

// Host estimate of the first rebuild's cell grid, for buffer capacities.
// Linked-cell sizes at the reference configuration, and the pairs per face of a
// double layer in contact everywhere (pi (d_max + 2 avg)^2 / mean face area):
// the largest list a folded shell can need.
void estimate_cells(const Setup& S, const shl_params& p, uint64_t& n_cells, uint64_t& entries,
                    double& pairs_per_face) {
  std::vector<double> sizes(S.F);
  double bmin[3] = {SHL_DBL_MAX, SHL_DBL_MAX, SHL_DBL_MAX}, bmax[3] = {-SHL_DBL_MAX, -SHL_DBL_MAX, -SHL_DBL_MAX};
  std::vector<double> fmin(3 * (size_t)S.F), fmax(3 * (size_t)S.F);
  for (uint32_t f = 0; f < S.F; ++f) {
    double lo[3] = {SHL_DBL_MAX, SHL_DBL_MAX, SHL_DBL_MAX}, hi[3] = {-SHL_DBL_MAX, -SHL_DBL_MAX, -SHL_DBL_MAX};
    for (int k = 0; k < 3; ++k)
      for (int c = 0; c < 3; ++c) {
        const double x = S.X[3 * (size_t)S.tri[3 * f + k] + c];
        lo[c] = std::min(lo[c], x);
        hi[c] = std::max(hi[c], x);
      }
    double d = 0;
    for (int c = 0; c < 3; ++c) {
      d = std::max(d, hi[c] - lo[c]);
      bmin[c] = std::min(bmin[c], lo[c]);
      bmax[c] = std::max(bmax[c], hi[c]);
      fmin[3 * f + c] = lo[c];
      fmax[3 * f + c] = hi[c];
    }
    sizes[f] = d;
  }
  const double avg = shl_fixed_order_sum(sizes.data(), S.F) / S.F;
  double cs = p.cell_size_mult * avg;
  const double tol = p.cell_margin * cs;
  cs += tol;
  double dm = p.thickness + tol;
  if (p.shell_shell_contact == SHL_CONTACT_SMOOTH) dm += avg;
  double area = 0;
  for (uint32_t f = 0; f < S.F; ++f) {
    double e1[3], e2[3];
    for (int c = 0; c < 3; ++c) {
      e1[c] = S.X[3 * (size_t)S.tri[3 * f + 1] + c] - S.X[3 * (size_t)S.tri[3 * f] + c];
      e2[c] = S.X[3 * (size_t)S.tri[3 * f + 2] + c] - S.X[3 * (size_t)S.tri[3 * f] + c];
    }
    const double nx = e1[1] * e2[2] - e1[2] * e2[1], ny = e1[2] * e2[0] - e1[0] * e2[2],
                 nz = e1[0] * e2[1] - e1[1] * e2[0];
    area += 0.5 * std::sqrt(nx * nx + ny * ny + nz * nz);
  }
  const double af = area / S.F;
  pairs_per_face = af > 0 ? M_PI * (dm + 2 * avg) * (dm + 2 * avg) / af : 16.0;
  n_cells = 1;
  uint64_t ncd[3];
  for (int c = 0; c < 3; ++c) {
    ncd[c] = (uint64_t)((bmax[c] - bmin[c] + dm) / cs + 1);
    n_cells *= ncd[c];
  }
  entries = 0;
  for (uint32_t f = 0; f < S.F; ++f) {
    uint64_t e = 1;
    for (int c = 0; c < 3; ++c) {
      const int lo = (int)((fmin[3 * f + c] - bmin[c]) / cs);
      const int hi = (int)((fmax[3 * f + c] - bmin[c] + dm) / cs);
      e *= (uint64_t)(hi - lo + 1);
    }
    entries += e;
  }
}

// A linked-cell pass inside a graph capture: an IF node whose body is the
// rebuild pipeline.  Its condition handle is created first and handed to the
// kernel that decides the rebuild (predictor, corrector), whose last block sets
// it from ctl->rebuild, so steps without a rebuild launch no extra kernel.
cudaError_t rebuild_cond_create(shl_ctx* c, RebuildCond* rc) {
  cudaStreamCaptureStatus st;
  cudaGraph_t g = nullptr;
  const cudaGraphNode_t* deps = nullptr;
  const cudaGraphEdgeData* edges = nullptr;
  size_t nd = 0;
  cudaError_t e = cudaStreamGetCaptureInfo(c->stream, &st, nullptr, &g, &deps, &edges, &nd);
  if (e != cudaSuccess) return e;
  e = cudaGraphConditionalHandleCreate(&rc->h, g, 0, cudaGraphCondAssignDefault);
  if (e != cudaSuccess) return e;
  rc->has = 1;
  return cudaSuccess;
}

cudaError_t rebuild_if_node(shl_ctx* c, const RebuildCond& rc, const DevBuf& b, const DevBuf* second) {
  cudaStreamCaptureStatus st;
  cudaGraph_t g = nullptr;
  const cudaGraphNode_t* deps = nullptr;
  const cudaGraphEdgeData* edges = nullptr;
  size_t nd = 0;
  cudaError_t e = cudaStreamGetCaptureInfo(c->stream, &st, nullptr, &g, &deps, &edges, &nd);
  if (e != cudaSuccess) return e;
  cudaGraphNodeParams cp = {cudaGraphNodeTypeConditional};
  cp.conditional.handle = rc.h;
  cp.conditional.type = cudaGraphCondTypeIf;
  cp.conditional.size = 1;
  cudaGraphNode_t node;
  e = cudaGraphAddNode(&node, g, deps, edges, nd, &cp);
  if (e != cudaSuccess) return e;
  cudaGraph_t body = cp.conditional.phGraph_out[0];
  e = cudaStreamBeginCaptureToGraph(c->side, body, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed);
  if (e != cudaSuccess) return e;
  launch_rebuild(b, c->sc, c->side);
  if (second) {
    launch_rebuild_second(b, c->sc, c->side);
    launch_rebuild(*second, c->sc, c->side);
  }
  e = cudaStreamEndCapture(c->side, &body);
  if (e != cudaSuccess) return e;
  return cudaStreamUpdateCaptureDependencies(c->stream, &node, nullptr, 1, cudaStreamSetCaptureDependencies);
}

// the linked-cell pass after the kernel that decided it: an IF node in a graph
// with conditional nodes, else the pipeline itself (its kernels return at once
// when no rebuild is due); b.p = the positions it works on
// second: fused steps' pair of passes (b at the corrected positions, then
// *second at the predicted ones, k_rebuild_second between them)
cudaError_t enqueue_rebuild(shl_ctx* c, const RebuildCond& rc, const DevBuf& b, const DevBuf* second = nullptr) {
  if (rc.has) return rebuild_if_node(c, rc, b, second);
  launch_rebuild(b, c->sc, c->stream);
  if (second) {
    launch_rebuild_second(b, c->sc, c->stream);
    launch_rebuild(*second, c->sc, c->stream);
  }
  return cudaSuccess;
}

bool fused_steps(const shl_ctx* c) { return c->sc.adapt_every == 0; }

// One step.  fused (graphs, fixed dt): the step opens with k_begin_step, its
// nodes having been predicted by the previous corrector (or k_predict with
// nodes_only), reads the predicted positions from b.pn and predicts the next
// step in its corrector; otherwise the predictor opens the step.
cudaError_t enqueue_step(shl_ctx* c, bool capturing = false, bool fused = false) {
  const DevBuf& b = c->b;
  const StepConst& sc = c->sc;
  cudaStream_t s = c->stream;
  cudaError_t e = cudaSuccess;
  const bool cond = capturing && c->conditional_ok && sc.contact;
  DevBuf bp = b;  // the step's predicted positions
  if (fused) bp.p = b.pn;
  RebuildCond r1{0, 0}, r2{0, 0};
  if (cond && (e = rebuild_cond_create(c, &r1)) != cudaSuccess) return e;
  if (fused)
    launch_begin_step(b, sc, r1, s);
  else
    launch_predict(b, sc, r1, s);
  // fused: one IF node for the previous corrector's pass and this predictor's
  if (sc.contact && (e = enqueue_rebuild(c, r1, fused ? b : bp, fused ? &bp : nullptr)) != cudaSuccess) return e;
  launch_elements(b, sc, elem_launch(c, sc), s, false);  // totals in k_volume_end
  if (sc.contact) launch_contact_force(bp, sc, 0, s);
  if (cond && !fused && (e = rebuild_cond_create(c, &r2)) != cudaSuccess) return e;
  if (sc.adapt_every) {
    // one attempt: estimate, then correct only if accepted (ShellSystem.C:1010-1117)
    launch_gather_correct(b, sc, 2, false, nullptr, nullptr, s);
    launch_correct_adapt(b, sc, s, r2);
  } else {
    launch_gather_correct(b, sc, fused ? 3 : 0, true, nullptr, nullptr, s, r2);
  }
  if (sc.contact && !fused && (e = enqueue_rebuild(c, r2, b)) != cudaSuccess) return e;
  launch_volume_end_step(b, sc, true, s);
  return cudaSuccess;
}

shl_status build_graph(shl_ctx* c, uint32_t steps, cudaGraphExec_t* out) {
  for (int attempt = 0; attempt < 2; ++attempt) {
    cudaGraph_t g = nullptr;
    SHL_CUDA_TRY(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
    cudaError_t e = cudaSuccess;
    for (uint32_t i = 0; i < steps && e == cudaSuccess; ++i) e = enqueue_step(c, true, fused_steps(c));
    cudaError_t e2 = cudaStreamEndCapture(c->stream, &g);
    if (e == cudaSuccess) e = e2;
    if (e == cudaSuccess) e = cudaGraphInstantiate(out, g, 0);
    if (g) cudaGraphDestroy(g);
    if (e == cudaSuccess) return SHL_OK;
    cudaGetLastError();
    if (!c->conditional_ok) {
      g_err = std::string("graph capture: ") + cudaGetErrorString(e);
      return SHL_ERR_CUDA;
    }
    c->conditional_ok = false;  // retry with early-exit launches instead of IF nodes
  }
  return SHL_ERR_CUDA;
}

// cavity semi-axes at time t as the device computes them (functions or constants)
void cavity_axes_host(const shl_ctx* c, double t, double* R) {
  const double R0[3] = {c->P.Rx, c->P.Ry, c->P.Rz};
  for (int k = 0; k < 3; ++k) {
    R[k] = R0[k];
    if (!c->rfun_text[k].empty()) R[k] = shl::expr::Expression(c->rfun_text[k]).eval({{"t", t}, {"d", 0.0}});
  }
}

// newmark_a of dt (ShellSystem.C:744-759) into the control block
void set_newmark_host(Ctl& h, double dt, double beta, double gamma) {
  h.dt_cur = dt;
  h.nm[0] = beta * dt * dt;
  h.nm[1] = gamma / (beta * dt);
  h.nm[2] = 1 / (beta * dt);
  h.nm[3] = 1 / (2 * beta) - 1;
  h.nm[4] = gamma / beta - 1;
  h.nm[5] = dt * (gamma / (2 * beta) - 1);
  h.nm[6] = (1 - gamma) * dt;
  h.nm[7] = gamma * dt;
  h.nm[8] = dt * dt * (0.5 - beta);
  h.nm[9] = dt * dt * std::fabs(beta - 1. / 6);
}

void fill_energies(const Ctl& h, shl_energies* e) {
  if (!e) return;
  e->Etens = h.Etens; e->Ebend = h.Ebend; e->Eself = h.Eself; e->Efric = h.Efric; e->Ekin = h.Ekin;
  e->area = h.area; e->volume = h.volume; e->kGauss = h.kGauss; e->kMean = h.kMean;
  e->Nc = h.Nc; e->n_pairs = h.n_pairs;
  e->Ecav = h.Ecav; e->cavity_force = h.cavity_force; e->Nc_cav = h.Nc_cav;
}

}  // namespace

extern "C" {

const char* shl_version(void) { return "shl_gb300 0.1 sm_103a"; }
const char* shl_last_error(void) { return g_err.c_str(); }

void shl_destroy(shl_ctx* c) {
  if (!c) return;
  if (c->graph) cudaGraphExecDestroy(c->graph);
  if (c->graph1) cudaGraphExecDestroy(c->graph1);
  for (void* p : c->allocs) cudaFree(p);
  if (c->h_pin) cudaFreeHost(c->h_pin);
  if (c->h_ctl) cudaFreeHost(c->h_ctl);
  if (c->h_table) cudaFreeHost(c->h_table);
  if (c->d_flush) cudaFree(c->d_flush);
  if (c->stream) cudaStreamDestroy(c->stream);
  if (c->side) cudaStreamDestroy(c->side);
  delete c;
}

}  // extern "C"

namespace {

// Device allocation, uploads and step constants for a context whose set-up
// (c->S, one shell or a merged batch) is built; pscale: per original face.
// The FP64 path's arithmetic: 0 = both basis contractions in FP64, 1 = the
// displacement contraction as float pairs (24-26 % faster than 0 at levels 6
// and 7), 2 = double-float throughout: the relative-displacement formulation
// in float pairs on the FP32 pipe, shares kept as pairs and added in
// double-float by the gather (element kernel 14 % faster than 1 at level 6,
// 34 % at level 7; forces within 1e-14 of FP64).  Fixed for all contexts, so
// that results do not depend on which launch shape a context picks (the
// per-face arithmetic of a variant does not depend on its shape).
constexpr int kFp64Pairs = 2;

// step constants that follow the FP64 variant: its share format
void apply_variant(shl_ctx* c) { c->sc.qe_df = kElemVariants[c->var64].pairs == 2 ? 1 : 0; }

// first FP64 variant of the fixed arithmetic (the FP64 launch of FP32 contexts)
int default_var64() {
  for (int v = 0; v < kFirstFp32Variant; ++v)
    if (kElemVariants[v].pairs == kFp64Pairs) return v;
  return 0;
}


// Element-kernel autotuning: time every launch shape of the context's path on
// its own mesh (one warm-up and three timed launches each, CUDA events on the
// context stream) and keep the fastest.
shl_status tune_elements(shl_ctx* c) {
  cudaEvent_t e0, e1;
  SHL_CUDA_TRY(cudaEventCreate(&e0));
  SHL_CUDA_TRY(cudaEventCreate(&e1));
  const bool fp32 = c->sc.fp32 != 0;
  float best = 0.f;
  int best_v = -1;
  for (int v = 0; v < kNumElemVariants; ++v) {
    const bool v32 = v >= kFirstFp32Variant;
    if (v32 != fp32 || (!v32 && kElemVariants[v].pairs != kFp64Pairs)) continue;
    if (fp32) c->var32 = v; else c->var64 = v;
    const ElemLaunch el = elem_launch(c, c->sc);
    launch_elements(c->b, c->sc, el, c->stream);
    float total = 0.f;
    for (int r = 0; r < 3; ++r) {
      cudaEventRecord(e0, c->stream);
      launch_elements(c->b, c->sc, el, c->stream);
      cudaEventRecord(e1, c->stream);
      SHL_CUDA_TRY(cudaEventSynchronize(e1));
      float ms = 0.f;
      cudaEventElapsedTime(&ms, e0, e1);
      total += ms;
    }
    c->variant_ms[v] = total / 3;
    if (best_v < 0 || c->variant_ms[v] < best) {
      best = c->variant_ms[v];
      best_v = v;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (fp32) c->var32 = best_v; else c->var64 = best_v;
  apply_variant(c);
  return check_launch("element tuning");
}

shl_status create_common(shl_ctx* c, const std::vector<double>& pscale_orig, shl_ctx** out) {
  const shl_params* params = &c->P;
  std::string err;
  shl_status st = SHL_OK;
  auto fail = [&](shl_status s) { shl_destroy(c); return s; };
  if (cudaGetDevice(&c->device) != cudaSuccess || cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaStreamCreateWithFlags(&c->side, cudaStreamNonBlocking) != cudaSuccess) {
    g_err = "no CUDA device";
    return fail(SHL_ERR_CUDA);
  }
  if (cudaError_t e = init_element_kernels(); e != cudaSuccess) {
    g_err = std::string("element kernel attributes: ") + cudaGetErrorString(e);
    return fail(SHL_ERR_CUDA);
  }
  if (cudaError_t e = init_contact_kernels(); e != cudaSuccess) {
    g_err = std::string("contact kernel attributes: ") + cudaGetErrorString(e);
    return fail(SHL_ERR_CUDA);
  }
  const Setup& S = c->S;
  const uint32_t V = S.V, F = S.F;
  DevBuf& b = c->b;
  const size_t nd = 3 * (size_t)V;
#define ALLOC(ptr, n) do { if ((st = dev_alloc(c, &(ptr), (n))) != SHL_OK) return fail(st); } while (0)
  ALLOC(b.X, nd); ALLOC(b.u, nd); ALLOC(b.v, nd); ALLOC(b.a, nd); ALLOC(b.up, nd); ALLOC(b.vp, nd);
  ALLOC(b.p, nd); ALLOC(b.Minv, nd); ALLOC(b.C, nd); ALLOC(b.M, nd); ALLOC(b.pn, nd);
  ALLOC(b.upk, 2 * (size_t)S.V);
  if (params->adapt_dt_every) ALLOC(b.ap, nd);
  if (params->shell_cavity_contact) {
    ALLOC(b.cav_origin, nd);
    ALLOC(b.cav_ecav, V);
    ALLOC(b.cav_efric, V);
  }
  ALLOC(b.face, (size_t)FF_COUNT * F);
  ALLOC(b.patch, (size_t)S.patch_rows * F);
  const bool fp32 = params->precision == SHL_PREC_FP32;
  if (fp32) {
    ALLOC(b.qe32, 3 * (size_t)S.n_slots_total);
    ALLOC(b.up32, (size_t)V);
    ALLOC(b.face32, (size_t)F32_COUNT * F);
  } else {
    ALLOC(b.face_df, (size_t)2 * F32_COUNT * F);
  }
  ALLOC(b.qe, fp32 ? 1 : 3 * (size_t)S.n_slots_total);
  ALLOC(b.gather_ptr, V + 1);
  ALLOC(b.slot_pos, S.slot_pos.size());
  if (params->shell_cavity_contact) {
    ALLOC(b.node_face_ptr, V + 1);
    ALLOC(b.node_face, S.node_face.size());
  }
  ALLOC(b.tri, 3 * (size_t)F);
  ALLOC(b.perm, F);
  ALLOC(b.pscale, F);
  ALLOC(b.area, F); ALLOC(b.kG, F); ALLOC(b.kM, F); ALLOC(b.etens, F); ALLOC(b.ebend, F);
  // element launch: one block range per patch group
  std::vector<GroupDesc> gd;
  std::vector<double> basis;
  uint32_t blocks = 0;
  for (const PatchGroup& g : S.groups) {
    GroupDesc d;
    d.first = g.first;
    d.count = g.count;
    d.block_start = blocks;
    d.n_slots = g.n_slots;
    d.slot_base = g.slot_base;
    d.basis_off = (int32_t)basis.size();
    basis.insert(basis.end(), g.basis.begin(), g.basis.end());
    blocks += (g.count + kBlock - 1) / kBlock;
    gd.push_back(d);
  }
  if ((int)gd.size() > kMaxGroups) { g_err = "too many patch valences"; return fail(SHL_ERR_ARG); }
  if (blocks == 0) blocks = 1;
  c->elem_blocks = blocks;
  // block ranges of the other launch shapes
  const int bs_list[3] = {64, 128, 256};
  std::vector<GroupDesc> gd_bs[3];
  for (int k = 0; k < 3; ++k) {
    uint32_t nb = 0;
    for (GroupDesc d : gd) {
      d.block_start = nb;
      nb += (d.count + bs_list[k] - 1) / bs_list[k];
      gd_bs[k].push_back(d);
    }
    c->blocks_bs[k] = nb ? nb : 1;
  }
  const uint32_t max_blocks = std::max({blocks, (F + kBlock - 1) / kBlock, (V + kBlock - 1) / kBlock, 4u * 152u}) + 8;
  ALLOC(b.partial, 8 * (size_t)max_blocks);
  ALLOC(c->d_fa, 2 * nd);
  ALLOC(b.ctl, 1);
  ALLOC(b.ptable, kTableCap);
  b.ptable_cap = kTableCap;

  // contact buffers
  const bool contact = params->shell_shell_contact != SHL_CONTACT_NONE;
  const bool smooth = params->shell_shell_contact == SHL_CONTACT_SMOOTH;
  uint64_t n_cells0 = 0, entries0 = 0;
  uint32_t n_cells_cap = 1, entries_cap = 1, pairs_cap = 1, csr_cap = 1, cand_cap = 1;
  if (contact) {
    double ppf = 16.0;
    const bool batch_contact = !c->shc_host.empty();
    uint64_t cells_max = S.n_cells_max;
    if (batch_contact) {  // the shells' own estimates, summed
      n_cells0 = c->bc_cells;
      entries0 = c->bc_entries;
      cells_max = c->bc_cells_max;
    } else {
      estimate_cells(S, *params, n_cells0, entries0, ppf);
    }
    const uint64_t want_cells = std::min<uint64_t>(cells_max, 1ull << 28);
    n_cells_cap = (uint32_t)std::max<uint64_t>(std::min<uint64_t>(want_cells, std::max<uint64_t>(8 * n_cells0, 1u << 20)), 1);
    if (n_cells_cap < n_cells0) n_cells_cap = (uint32_t)std::min<uint64_t>(n_cells0, 1ull << 28);
    entries_cap = (uint32_t)std::min<uint64_t>(std::max<uint64_t>(8 * entries0, 1u << 20), 1ull << 30);
    // room for a shell folded onto itself everywhere (1.5 x the double-layer estimate);
    // csr entries hold pair * 8 + role, so at most 2^28 pairs
    const double per_face = std::max(16.0, 1.5 * ppf);
    const double pairs_want = batch_contact ? c->bc_pairs : per_face * F;
    pairs_cap = (uint32_t)std::min<double>(std::max<double>(pairs_want, 65536.0), (double)(1u << 28));
    csr_cap = (uint32_t)std::min<uint64_t>((uint64_t)6 * pairs_cap, 0xFFFFFFF0u);
    // candidates before the distance test (SMOOTH skips the facet prefilter)
    cand_cap = (uint32_t)std::min<uint64_t>(std::max<uint64_t>((uint64_t)(smooth ? 3 : 2) * pairs_cap, 1u << 18),
                                            1u << 30);
    ALLOC(b.close_ptr, F + 1);
    ALLOC(b.close_list, S.close_list.size());
    ALLOC(b.bmin, 3 * (size_t)F); ALLOC(b.bmax, 3 * (size_t)F); ALLOC(b.fsize, F); ALLOC(b.sum_lanes, SHL_SUM_LANES);
    ALLOC(b.cell_lo, 3 * (size_t)F); ALLOC(b.cell_hi, 3 * (size_t)F);
    ALLOC(b.cell_count, n_cells_cap); ALLOC(b.cell_start, n_cells_cap + 1); ALLOC(b.cell_fill, n_cells_cap);
    ALLOC(b.cell_items, entries_cap);
    ALLOC(b.entry_cell, entries_cap);
    ALLOC(b.p32, nd);
    const size_t scan_cap = std::max<size_t>({(size_t)n_cells_cap, (size_t)F + 1, (size_t)V + 1});
    ALLOC(b.scan_block, scan_cap / kScanTile + 2);
    for (int k = 0; k < 2; ++k) {
      ALLOC(b.pe1[k], pairs_cap); ALLOC(b.pe2[k], pairs_cap); ALLOC(b.pstick[k], pairs_cap);
      ALLOC(b.pd2[k], pairs_cap); ALLOC(b.porig[k], 3 * (size_t)pairs_cap); ALLOC(b.pair_ptr[k], F + 1);
    }
    ALLOC(b.pkeep, pairs_cap);
    ALLOC(b.new_e1, pairs_cap); ALLOC(b.new_e2, pairs_cap); ALLOC(b.new_d2, pairs_cap);
    ALLOC(b.new_off, F + 1); ALLOC(b.new_cnt, F); ALLOC(b.new_fill, F);
    ALLOC(b.cand_e1, cand_cap); ALLOC(b.cand_e2, cand_cap); ALLOC(b.cand_d2, cand_cap); ALLOC(b.cand_ok, cand_cap);
    ALLOC(b.seg_count, F);
    ALLOC(b.pforce, kPairOut * (size_t)pairs_cap);
    ALLOC(b.csr_count, V); ALLOC(b.csr_ptr, V + 1); ALLOC(b.csr_ent, csr_cap); ALLOC(b.csr_fill, V);
    if (smooth) {
      ALLOC(b.pvw[0], 4 * (size_t)pairs_cap); ALLOC(b.pvw[1], 4 * (size_t)pairs_cap);
      ALLOC(b.new_x, 4 * (size_t)pairs_cap); ALLOC(b.cand_x, 4 * (size_t)cand_cap);
      ALLOC(b.lcoef, SHL_LIMIT_NCOEF * (size_t)F);
      ALLOC(b.inv_perm, F); ALLOC(b.fsm, F);
    }
    if (batch_contact) {
      ALLOC(b.shc, c->shc_host.size());
      ALLOC(b.face_shell, F);
      ALLOC(b.node_shell, V);
    }
  }
#undef ALLOC

  // uploads
  if ((st = upload(c, b.X, S.X.data(), nd)) != SHL_OK) return fail(st);
  if ((st = upload(c, b.p, S.X.data(), nd)) != SHL_OK) return fail(st);
  if ((st = upload(c, b.Minv, S.Minv.data(), nd)) != SHL_OK) return fail(st);
  std::vector<double> mass(nd);
  for (size_t k = 0; k < nd; ++k) mass[k] = 1.0 / S.Minv[k];
  if ((st = upload(c, b.M, mass.data(), nd)) != SHL_OK) return fail(st);
  if ((st = upload(c, b.C, S.C.data(), nd)) != SHL_OK) return fail(st);
  if ((st = upload(c, b.face, S.face.data(), S.face.size())) != SHL_OK) return fail(st);
  if (fp32 && (st = upload(c, b.face32, S.face32.data(), S.face32.size())) != SHL_OK) return fail(st);
  if (!fp32 && (st = upload(c, b.face_df, S.face_df.data(), S.face_df.size())) != SHL_OK) return fail(st);
  if ((st = upload(c, b.patch, S.patch.data(), S.patch.size())) != SHL_OK) return fail(st);
  if ((st = upload(c, b.gather_ptr, S.gather_ptr.data(), S.gather_ptr.size())) != SHL_OK) return fail(st);
  if ((st = upload(c, b.slot_pos, S.slot_pos.data(), S.slot_pos.size())) != SHL_OK) return fail(st);
  if (params->shell_cavity_contact) {
    if ((st = upload(c, b.node_face_ptr, S.node_face_ptr.data(), S.node_face_ptr.size())) != SHL_OK) return fail(st);
    if ((st = upload(c, b.node_face, S.node_face.data(), S.node_face.size())) != SHL_OK) return fail(st);
  }
  if ((st = upload(c, b.tri, S.tri.data(), S.tri.size())) != SHL_OK) return fail(st);
  if ((st = upload(c, b.perm, S.perm.data(), S.perm.size())) != SHL_OK) return fail(st);
  std::vector<double> pscale(F);
  for (uint32_t i = 0; i < F; ++i) pscale[i] = pscale_orig[S.perm[i]];
  if ((st = upload(c, b.pscale, pscale.data(), F)) != SHL_OK) return fail(st);
  int32_t stab_off[13];
  for (int k = 0; k < 13; ++k) stab_off[k] = -1;
  if (smooth) {
    // per original face: valence of the patch's first vertex | (its position in the face) << 8
    std::vector<int32_t> fsm(F);
    std::vector<int> vals;
    for (const PatchGroup& g : S.groups)
      for (uint32_t i = g.first; i < g.first + g.count; ++i) {
        const uint32_t e = S.perm[i];
        int r = 0;
        for (int k = 0; k < 3; ++k)
          if ((int32_t)S.tri[3 * (size_t)e + k] == S.patch[i]) r = k;
        fsm[e] = g.valence | (r << 8);
        if (g.valence != 6 && std::find(vals.begin(), vals.end(), g.valence) == vals.end()) vals.push_back(g.valence);
      }
    std::vector<double> tabs;
    for (int N : vals) {
      std::vector<double> t;
      if (!shl_subdiv::build_table(N, t)) { g_err = "subdivision table of valence " + std::to_string(N); return fail(SHL_ERR_ARG); }
      stab_off[N] = (int32_t)tabs.size();
      tabs.insert(tabs.end(), t.begin(), t.end());
    }
    if (!tabs.empty()) {
      if ((st = dev_alloc(c, &b.stab, tabs.size())) != SHL_OK) return fail(st);
      if ((st = upload(c, b.stab, tabs.data(), tabs.size())) != SHL_OK) return fail(st);
    }
    if ((st = upload(c, b.fsm, fsm.data(), F)) != SHL_OK) return fail(st);
    if ((st = upload(c, b.inv_perm, S.inv_perm.data(), F)) != SHL_OK) return fail(st);
  }
  if (contact && !c->shc_host.empty()) {
    std::vector<uint32_t> node_shell(V);
    for (size_t k = 0; k + 1 < c->node_off.size(); ++k)
      for (uint32_t n = c->node_off[k]; n < c->node_off[k + 1]; ++n) node_shell[n] = (uint32_t)k;
    if ((st = upload(c, b.shc, c->shc_host.data(), c->shc_host.size())) != SHL_OK) return fail(st);
    if ((st = upload(c, b.face_shell, c->face_shell.data(), F)) != SHL_OK) return fail(st);
    if ((st = upload(c, b.node_shell, node_shell.data(), V)) != SHL_OK) return fail(st);
  }
  if (contact) {
    if ((st = upload(c, b.close_ptr, S.close_ptr.data(), S.close_ptr.size())) != SHL_OK) return fail(st);
    if (!S.close_list.empty() && (st = upload(c, b.close_list, S.close_list.data(), S.close_list.size())) != SHL_OK)
      return fail(st);
  }
  {
    double* d_basis = nullptr;
    if ((st = dev_alloc(c, &d_basis, basis.size())) != SHL_OK) return fail(st);
    if ((st = upload(c, d_basis, basis.data(), basis.size())) != SHL_OK) return fail(st);
    std::vector<float> basis32(basis.begin(), basis.end());
    float* d_basis32 = nullptr;
    if ((st = dev_alloc(c, &d_basis32, basis32.size())) != SHL_OK) return fail(st);
    if ((st = upload(c, d_basis32, basis32.data(), basis32.size())) != SHL_OK) return fail(st);
    c->eg.n = (int32_t)gd.size();
    for (size_t k = 0; k < gd.size(); ++k) c->eg.g[k] = gd[k];
    c->eg.basis = d_basis;
    c->eg.basis32 = d_basis32;
    for (int k = 0; k < 3; ++k) {
      c->eg_bs[k] = c->eg;
      for (size_t q = 0; q < gd_bs[k].size(); ++q) c->eg_bs[k].g[q] = gd_bs[k][q];
    }
  }

  // step constants
  StepConst& sc = c->sc;
  const shl_params& p = *params;
  sc.dt = p.dt;
  sc.nm0 = p.newmark_beta * p.dt * p.dt;
  sc.nm6 = (1 - p.newmark_gamma) * p.dt;
  sc.nm7 = p.newmark_gamma * p.dt;
  sc.nm8 = p.dt * p.dt * (0.5 - p.newmark_beta);
  sc.thickness = p.thickness;
  sc.K = S.K;
  sc.D = S.D;
  sc.qw = 0.5;
  sc.stiff_density = S.stiff_density;
  sc.stiff_static_friction = S.stiff_static_friction;
  sc.d2_friction = S.d2_friction;
  sc.mu_s = p.mu_s;
  sc.mu_d = p.mu_d;
  sc.self_damping = p.self_damping;
  sc.self_friction_damping = p.self_friction_damping;
  sc.v_stop = p.friction_stop_velocity;
  sc.cell_size_mult = p.cell_size_mult;
  sc.cell_margin = p.cell_margin;
  sc.bulk_modulus = p.bulk_modulus;
  sc.pressure_default = p.pressure;
  sc.pressure_table = b.ptable;
  sc.n_cells_max = S.n_cells_max;
  sc.n_cells_cap = n_cells_cap;
  sc.entries_cap = entries_cap;
  sc.pairs_cap = pairs_cap;
  sc.csr_cap = csr_cap;
  sc.cand_cap = cand_cap;
  sc.contact = contact ? 1 : 0;
  sc.smooth = smooth ? 1 : 0;
  c->var64 = default_var64();
  apply_variant(c);
  for (int k = 0; k < 13; ++k) sc.stab_off[k] = stab_off[k];
  sc.friction = (contact && (p.mu_s != 0 || p.mu_d != 0)) ? 1 : 0;
  sc.pressure_base = p.pressure_base;
  sc.pressure_dir = p.pressure_dir;
  sc.compat_zero_pressure = p.compat_zero_pressure;
  sc.stop_on_problem = p.stop_on_problem;
  sc.fp32 = fp32 ? 1 : 0;
  sc.V = V;
  sc.F = F;
  sc.internal_scale = 1.0;
  sc.adapt_every = p.adapt_dt_every;
  sc.beta = p.newmark_beta;
  sc.gamma = p.newmark_gamma;
  sc.err_min = p.rel_loc_err_min;
  sc.err_max = p.rel_loc_err_max;
  sc.err_target = std::sqrt(p.rel_loc_err_min * p.rel_loc_err_max);
  sc.dt_min_eff = std::max(p.dt_min, 2.220446049250313e-16);
  sc.dt_max_eff = p.dt_max <= 0 ? SHL_DBL_MAX : p.dt_max;
  sc.cavity_contact = p.shell_cavity_contact ? 1 : 0;
  sc.cavity_type = p.cavity;
  sc.cavity_friction = (p.shell_cavity_contact && (p.mu_s_cavity != 0 || p.mu_d_cavity != 0)) ? 1 : 0;
  sc.cav_R[0] = p.Rx;
  sc.cav_R[1] = p.Ry;
  sc.cav_R[2] = p.Rz;
  sc.mu_s_cav = p.mu_s_cavity;
  sc.mu_d_cav = p.mu_d_cavity;
  sc.cav_damping = p.cavity_damping;
  sc.cav_fric_damping = p.cavity_friction_damping;
  sc.static_friction_tol = p.static_friction_tol;
  sc.n_cs = contact ? (uint32_t)c->shc_host.size() : 0u;

  Ctl h;
  std::memset(&h, 0, sizeof(h));
  set_newmark_host(h, p.dt, p.newmark_beta, p.newmark_gamma);
  h.steps_target = ~0u;
  h.cav_R[0] = p.Rx;
  h.cav_R[1] = p.Ry;
  h.cav_R[2] = p.Rz;
  if (cudaMallocHost(&c->h_ctl, sizeof(Ctl)) != cudaSuccess) c->h_ctl = nullptr;
  if (cudaMallocHost(&c->h_table, kTableCap * sizeof(double)) != cudaSuccess) c->h_table = nullptr;
  if ((st = ctl_put(c, h)) != SHL_OK) return fail(st);
  if (cudaMallocHost(&c->h_pin, 3 * nd * sizeof(double)) != cudaSuccess) c->h_pin = nullptr;
  if ((st = check_launch("shl_create")) != SHL_OK) return fail(st);
  if (cudaStreamSynchronize(c->stream) != cudaSuccess) {
    g_err = "stream synchronisation failed in shl_create";
    return fail(SHL_ERR_CUDA);
  }
  if ((st = tune_elements(c)) != SHL_OK) return fail(st);
  *out = c;
  return SHL_OK;
}

}  // namespace

extern "C" {

shl_status shl_create(const shl_mesh* mesh, const shl_params* params, shl_ctx** out) {
  if (!mesh || !params || !out) { g_err = "null argument"; return SHL_ERR_ARG; }
  *out = nullptr;
  std::string err;
  if (!validate(*params, err)) { g_err = err; return SHL_ERR_ARG; }
  shl_ctx* c = new shl_ctx;
  c->P = *params;
  if (!build_setup(*mesh, *params, c->S, err)) {
    g_err = err;
    delete c;
    return SHL_ERR_ARG;
  }
  c->node_off = {0, c->S.V};
  c->face_off = {0, c->S.F};
  return create_common(c, std::vector<double>(c->S.F, 1.0), out);
}

shl_status shl_batch_create(const shl_mesh* meshes, const shl_params* params, const double* pressure_scale,
                            uint32_t n_shells, shl_ctx** out) {
  if (!meshes || !params || !out || n_shells == 0) { g_err = "null argument"; return SHL_ERR_ARG; }
  *out = nullptr;
  std::string err;
  const shl_params& p0 = params[0];
  for (uint32_t k = 0; k < n_shells; ++k) {
    const shl_params& p = params[k];
    if (!validate(p, err)) { g_err = "shell " + std::to_string(k) + ": " + err; return SHL_ERR_ARG; }
    if (p.bulk_modulus != 0.0) {
      g_err = "batched shells: bulk-modulus pressure is evaluated per single shell only";
      return SHL_ERR_ARG;
    }
    // self-contact: each shell's own linked cells; the friction law and the
    // cell margin are shared
    if (p.shell_shell_contact != p0.shell_shell_contact ||
        (p.shell_shell_contact != SHL_CONTACT_NONE &&
         (p.mu_s != p0.mu_s || p.mu_d != p0.mu_d || p.self_damping != p0.self_damping ||
          p.self_friction_damping != p0.self_friction_damping ||
          p.friction_stop_velocity != p0.friction_stop_velocity || p.cell_margin != p0.cell_margin ||
          p.adapt_dt_every != 0))) {
      g_err = "batched shells with self-contact must share the contact mode, friction, damping and cell margin, "
              "with a fixed dt";
      return SHL_ERR_ARG;
    }
    if (p.dt != p0.dt || p.newmark_beta != p0.newmark_beta || p.newmark_gamma != p0.newmark_gamma ||
        p.precision != p0.precision || p.pressure_base != p0.pressure_base || p.pressure_dir != p0.pressure_dir ||
        p.compat_zero_pressure != p0.compat_zero_pressure) {
      g_err = "batched shells must share dt, Newmark parameters, precision and pressure basis";
      return SHL_ERR_ARG;
    }
  }
  std::vector<Setup> shells(n_shells);
  std::vector<std::string> errs(n_shells);
  std::vector<char> ok(n_shells, 0);
#pragma omp parallel for schedule(dynamic, 1)
  for (int64_t k = 0; k < (int64_t)n_shells; ++k) ok[k] = build_setup(meshes[k], params[k], shells[k], errs[k]) ? 1 : 0;
  for (uint32_t k = 0; k < n_shells; ++k)
    if (!ok[k]) { g_err = "shell " + std::to_string(k) + ": " + errs[k]; return SHL_ERR_ARG; }
  shl_ctx* c = new shl_ctx;
  c->P = p0;
  if (p0.shell_shell_contact != SHL_CONTACT_NONE) {
    // per-shell constants and linked-cell estimates (before the merge moves the set-ups)
    uint32_t f0 = 0;
    for (uint32_t k = 0; k < n_shells; ++k) {
      const Setup& S = shells[k];
      ShellCell sc{};
      sc.thickness = params[k].thickness;
      sc.cell_size_mult = params[k].cell_size_mult;
      sc.stiff_density = S.stiff_density;
      sc.stiff_static_friction = S.stiff_static_friction;
      sc.d2_friction = S.d2_friction;
      sc.n_cells_max = S.n_cells_max;
      sc.face_first = f0;
      sc.face_end = f0 + S.F;
      f0 += S.F;
      c->shc_host.push_back(sc);
      uint64_t nc = 0, ne = 0;
      double ppf = 16.0;
      estimate_cells(S, params[k], nc, ne, ppf);
      c->bc_cells += nc;
      c->bc_entries += ne;
      c->bc_cells_max += S.n_cells_max;
      c->bc_pairs += std::max(16.0, 1.5 * ppf) * S.F;
    }
  }
  if (!merge_setups(shells, c->S, c->node_off, c->face_off, c->face_shell, err)) {
    g_err = err;
    delete c;
    return SHL_ERR_ARG;
  }
  std::vector<double> pscale(c->S.F);
  for (uint32_t f = 0; f < c->S.F; ++f) pscale[f] = pressure_scale ? pressure_scale[c->face_shell[f]] : 1.0;
  return create_common(c, pscale, out);
}

shl_status shl_batch_layout(shl_ctx* c, uint32_t* n_shells, uint32_t* node_offsets, uint32_t* face_offsets) {
  if (!c) return SHL_ERR_ARG;
  const uint32_t n = (uint32_t)c->node_off.size() - 1;
  if (n_shells) *n_shells = n;
  if (node_offsets) std::copy(c->node_off.begin(), c->node_off.end(), node_offsets);
  if (face_offsets) std::copy(c->face_off.begin(), c->face_off.end(), face_offsets);
  return SHL_OK;
}

shl_status shl_batch_contact_stats(shl_ctx* c, double* du_sum, uint32_t* n_rebuilds) {
  if (!c) return SHL_ERR_ARG;
  if (!c->sc.n_cs) { g_err = "not a batch with self-contact"; return SHL_ERR_ARG; }
  SHL_TRY(flush_deferred_rebuild(c));
  std::vector<ShellCell> h(c->sc.n_cs);
  SHL_CUDA_TRY(cudaMemcpyAsync(h.data(), c->b.shc, h.size() * sizeof(ShellCell), cudaMemcpyDeviceToHost, c->stream));
  SHL_CUDA_TRY(cudaStreamSynchronize(c->stream));
  for (size_t k = 0; k < h.size(); ++k) {
    if (du_sum) du_sum[k] = h[k].du_sum;
    if (n_rebuilds) n_rebuilds[k] = h[k].n_rebuilds;
  }
  return SHL_OK;
}

namespace {
// the device address of page-locked, mapped host memory, or null for any other pointer
double* mapped_host(const void* p) {
  if (!p) return nullptr;
  cudaPointerAttributes at;
  if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  if (at.type != cudaMemoryTypeHost || at.devicePointer == nullptr) return nullptr;
  return static_cast<double*>(at.devicePointer);
}
}  // namespace

shl_status shl_set_state(shl_ctx* c, const double* u, const double* v, const double* a) {
  if (!c) return SHL_ERR_ARG;
  SHL_TRY(host_access(c));  // pending linked-cell pass; the step prediction is rebuilt
  const size_t nd = 3 * (size_t)c->S.V;
  double *du = mapped_host(u), *dv = mapped_host(v), *da = mapped_host(a);
  if (du && dv && da) {
    // all three in mapped page-locked memory: one kernel reads them over the host link
    // and sets the positions
    launch_state_host(c->b, c->sc, du, dv, da, true, c->stream);
    SHL_CUDA_TRY(cudaStreamSynchronize(c->stream));
    return check_launch("shl_set_state");
  }
  if (u) {
    SHL_TRY(upload(c, c->b.u, u, nd));
    SHL_TRY(upload(c, c->b.up, u, nd));
    launch_positions(c->b, c->sc, c->stream);
  }
  if (v) SHL_TRY(upload(c, c->b.v, v, nd));
  if (a) SHL_TRY(upload(c, c->b.a, a, nd));
  SHL_CUDA_TRY(cudaStreamSynchronize(c->stream));
  return check_launch("shl_set_state");
}

shl_status shl_get_state(shl_ctx* c, double* u, double* v, double* a) {
  if (!c) return SHL_ERR_ARG;
  const size_t bytes = 3 * (size_t)c->S.V * sizeof(double);
  double *du = mapped_host(u), *dv = mapped_host(v), *da = mapped_host(a);
  if (du && dv && da) {
    launch_state_host(c->b, c->sc, du, dv, da, false, c->stream);
    SHL_CUDA_TRY(cudaStreamSynchronize(c->stream));
    return check_launch("shl_get_state");
  }
  if (u) SHL_CUDA_TRY(cudaMemcpyAsync(u, c->b.u, bytes, cudaMemcpyDeviceToHost, c->stream));
  if (v) SHL_CUDA_TRY(cudaMemcpyAsync(v, c->b.v, bytes, cudaMemcpyDeviceToHost, c->stream));
  if (a) SHL_CUDA_TRY(cudaMemcpyAsync(a, c->b.a, bytes, cudaMemcpyDeviceToHost, c->stream));
  SHL_CUDA_TRY(cudaStreamSynchronize(c->stream));
  return SHL_OK;
}

shl_status shl_set_time(shl_ctx* c, double t, uint32_t step) {
  if (!c) return SHL_ERR_ARG;
  SHL_TRY(host_access(c));  // pending linked-cell pass; the step prediction is rebuilt
  Ctl h;
  SHL_TRY(ctl_get(c, h));
  h.time = t;
  h.time_step = step;
  return ctl_put(c, h);
}

shl_status shl_get_time(shl_ctx* c, double* t, uint32_t* step) {
  if (!c) return SHL_ERR_ARG;
  Ctl h;
  SHL_TRY(ctl_get(c, h));
  if (t) *t = h.time;
  if (step) *step = h.time_step;
  return SHL_OK;
}

}  // extern "C"

namespace {

// scalar part of a force evaluation (pressure, volume pressure, problem reset)
shl_status begin_eval(shl_ctx* c, double pressure, bool allow_rebuild) {
  Ctl h;
  SHL_TRY(ctl_get(c, h));
  h.problem = 0;
  h.halted = 0;
  h.error = 0;
  h.pressure = c->P.compat_zero_pressure ? pressure * 0.0 : pressure;
  const double red = std::max((1.0 - static_cast<int>(h.time * 5.0) * 0.01), 0.5);
  if (h.time_step == 2) h.volume0 = h.volume;
  h.volume_pressure = (c->P.bulk_modulus == 0 ? 0 : c->P.bulk_modulus * (h.volume0 * red / h.volume - 1));
  cavity_axes_host(c, h.time, h.cav_R);
  if (allow_rebuild && c->sc.contact) {
    const double tol = c->P.cell_margin * (c->P.cell_size_mult * h.avg_elem_size);
    h.rebuild = h.du_sum >= tol ? 1u : 0u;
  } else {
    h.rebuild = 0;
  }
  SHL_TRY(ctl_put(c, h));
  // a batch: each shell's own test (the control block gets the OR)
  if (c->sc.n_cs) launch_batch_flags(c->b, c->sc, allow_rebuild ? 1 : 2, c->stream);
  return SHL_OK;
}

shl_status eval_into(shl_ctx* c, double* d_f, double* d_a) {
  const DevBuf& b = c->b;
  if (c->sc.contact) launch_rebuild(b, c->sc, c->stream);
  launch_elements(b, c->sc, elem_launch(c, c->sc), c->stream);
  if (c->sc.contact) launch_contact_force(b, c->sc, 0, c->stream);
  launch_gather_correct(b, c->sc, 0, false, d_f, d_a, c->stream);
  return check_launch("force evaluation");
}

shl_status finish_status(shl_ctx* c, Ctl& h) {
  SHL_TRY(ctl_get(c, h));
  if (h.error) {
    g_err = "device buffer capacity exceeded (contact pairs / linked cells)";
    return (shl_status)h.error;
  }
  return (shl_status)h.problem;
}

}  // namespace

extern "C" {

shl_status shl_eval_forces(shl_ctx* c, const double* u_pred, const double* v_pred, double pressure, double* f_out,
                           double* a_out, shl_energies* e) {
  if (!c || !u_pred || !v_pred) return SHL_ERR_ARG;
  SHL_TRY(host_access(c));  // pending linked-cell pass; the step prediction is rebuilt
  const size_t nd = 3 * (size_t)c->S.V;
  SHL_TRY(upload(c, c->b.up, u_pred, nd));
  SHL_TRY(upload(c, c->b.vp, v_pred, nd));
  launch_positions(c->b, c->sc, c->stream);
  SHL_TRY(begin_eval(c, pressure, true));
  double* d_f = c->d_fa;
  double* d_a = c->d_fa + nd;
  SHL_TRY(eval_into(c, d_f, d_a));
  if (f_out) SHL_CUDA_TRY(cudaMemcpyAsync(f_out, d_f, nd * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  if (a_out) SHL_CUDA_TRY(cudaMemcpyAsync(a_out, d_a, nd * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  Ctl h;
  const shl_status s = finish_status(c, h);
  fill_energies(h, e);
  return s;
}

namespace {

// the part of ShellSystem::apply_initial_conditions (ShellSystem.C:872-888)
// shared by a new start and a loaded state: positions, bounding boxes, the
// forced candidate-list build, deformed metrics and volume0 = volume
shl_status initial_state(shl_ctx* c, Ctl& h) {
  launch_positions(c->b, c->sc, c->stream);
  SHL_TRY(ctl_get(c, h));
  h.problem = 0;
  h.halted = 0;
  h.error = 0;
  h.pressure = 0;
  h.volume_pressure = 0;
  h.rebuild = c->sc.contact ? 1u : 0u;  // compute_shell_shell_contact_candidates(true)
  SHL_TRY(ctl_put(c, h));
  if (c->sc.n_cs) launch_batch_flags(c->b, c->sc, 0, c->stream);
  if (c->sc.contact) launch_rebuild(c->b, c->sc, c->stream);
  launch_elements(c->b, c->sc, elem_launch(c, c->sc), c->stream, false);
  launch_volume_end_step(c->b, c->sc, false, c->stream);
  SHL_TRY(check_launch("initial conditions"));
  SHL_TRY(ctl_get(c, h));
  h.volume0 = h.volume;
  return ctl_put(c, h);
}

}  // namespace

shl_status shl_apply_initial_conditions(shl_ctx* c, const double* u0, double t0, double pressure_next) {
  if (!c || !u0) return SHL_ERR_ARG;
  SHL_TRY(host_access(c));  // pending linked-cell pass; the step prediction is rebuilt
  const size_t nd = 3 * (size_t)c->S.V;
  SHL_TRY(upload(c, c->b.u, u0, nd));
  SHL_TRY(upload(c, c->b.up, u0, nd));
  SHL_CUDA_TRY(cudaMemsetAsync(c->b.v, 0, nd * sizeof(double), c->stream));
  SHL_CUDA_TRY(cudaMemsetAsync(c->b.vp, 0, nd * sizeof(double), c->stream));
  SHL_CUDA_TRY(cudaMemsetAsync(c->b.a, 0, nd * sizeof(double), c->stream));
  Ctl h;
  SHL_TRY(ctl_get(c, h));
  const uint32_t step0 = h.time_step;
  h.time = t0;
  SHL_TRY(ctl_put(c, h));
  SHL_TRY(initial_state(c, h));
  // one force evaluation at t0 + dt (ShellSystem.C:892-904)
  h.time = t0 + c->P.dt;
  h.time_step = step0 + 1;
  SHL_TRY(ctl_put(c, h));
  SHL_TRY(begin_eval(c, pressure_next, false));
  SHL_TRY(eval_into(c, nullptr, c->b.a));
  Ctl h2;
  const shl_status s = finish_status(c, h2);
  h2.time = t0;
  h2.time_step = step0;
  SHL_TRY(ctl_put(c, h2));
  return s;
}

shl_status shl_apply_loaded_state(shl_ctx* c) {
  if (!c) return SHL_ERR_ARG;
  SHL_TRY(host_access(c));  // pending linked-cell pass; the step prediction is rebuilt
  Ctl h;
  return initial_state(c, h);
}

namespace {

// clears the run report on the device, ordered on the context stream (no host round trip)
shl_status reset_report(shl_ctx* c) {
  launch_ctl_begin(c->b.ctl, 0, kCtlReset, c->stream);
  return check_launch("reset_report");
}

shl_status ensure_graphs(shl_ctx* c) {
  if (c->graph) return SHL_OK;
  SHL_TRY(build_graph(c, kGraphSteps, &c->graph));
  return build_graph(c, 1, &c->graph1);
}

shl_status enqueue_steps(shl_ctx* c, uint32_t n, bool use_graph) {
  if (n == 0) return SHL_OK;
  if (!use_graph || !fused_steps(c)) SHL_TRY(flush_deferred_rebuild(c));
  if (use_graph) {
    SHL_TRY(ensure_graphs(c));
    if (fused_steps(c) && !c->pred_valid) {
      DevBuf bp = c->b;
      bp.p = c->b.pn;
      launch_predict(bp, c->sc, RebuildCond{0, 0}, c->stream, true);
    }
    uint32_t k = 0;
    for (; k + kGraphSteps <= n; k += kGraphSteps) SHL_CUDA_TRY(cudaGraphLaunch(c->graph, c->stream));
    for (; k < n; ++k) SHL_CUDA_TRY(cudaGraphLaunch(c->graph1, c->stream));
    c->pred_valid = fused_steps(c);
    c->maybe_pending = c->maybe_pending || (fused_steps(c) && c->sc.contact);
  } else {
    for (uint32_t k = 0; k < n; ++k) enqueue_step(c);
    c->pred_valid = false;
  }
  return check_launch("step");
}

// Uploads n pressures and rewinds the device table to them; `flags` adds further
// control-block updates (kCtlReset, kCtlArm) to the same launch.  With the pinned
// staging buffer the copy is asynchronous: callers synchronise the stream before
// the buffer is written again (shl_step does at the end of every chunk).
shl_status upload_table(shl_ctx* c, const double* table, uint32_t n, uint32_t flags = 0, bool sync = true) {
  if (n > c->b.ptable_cap) { g_err = "pressure table longer than the device table"; return SHL_ERR_CAPACITY; }
  if (n) {
    const double* src = table;
    if (c->h_table && table != c->h_table) {
      std::memcpy(c->h_table, table, n * sizeof(double));
      src = c->h_table;
    }
    SHL_TRY(upload(c, c->b.ptable, src, n));
  }
  launch_ctl_begin(c->b.ctl, n, kCtlTable | flags, c->stream);
  SHL_TRY(check_launch("upload_table"));
  if (sync) SHL_CUDA_TRY(cudaStreamSynchronize(c->stream));
  return SHL_OK;
}

// `fresh`: the caller has just read the control block into `h` (no launch since)
shl_status collect(shl_ctx* c, shl_step_report* report, const Ctl* fresh = nullptr) {
  Ctl h;
  if (fresh)
    h = *fresh;
  else
    SHL_TRY(ctl_get(c, h));
  if (c->maybe_pending) {
    // a corrector-side linked-cell pass left pending by the last fused step
    c->maybe_pending = false;
    if (c->sc.contact && h.rebuild_pending) {
      launch_rebuild_first(c->b, c->sc, c->stream);
      launch_rebuild(c->b, c->sc, c->stream);
      SHL_TRY(check_launch("deferred linked-cell pass"));
      SHL_TRY(ctl_get(c, h));
    }
  }
  if (report) {
    std::memset(report, 0, sizeof(*report));
    report->steps_done = h.steps_done;
    report->worst_problem = h.worst_problem;
    report->time = h.time;
    report->du_sum = h.du_sum;
    report->n_rebuilds = h.n_rebuilds;
    report->rejections = h.rejections;
    report->sum_pcav = h.sum_pcav; report->sum_Nc_cav = h.sum_Nc_cav; report->sum_Ecav = h.sum_Ecav;
    report->stopped = (h.paused & 2u) ? 1u : 0u;
    fill_energies(h, &report->last);
    report->sum_dt = h.sum_dt; report->sum_area = h.sum_area; report->sum_volume = h.sum_volume;
    report->sum_Nc = h.sum_Nc; report->sum_Ekin = h.sum_Ekin; report->sum_Etens = h.sum_Etens;
    report->sum_Ebend = h.sum_Ebend; report->sum_Eself = h.sum_Eself; report->sum_Efric = h.sum_Efric;
    report->sum_kGauss = h.sum_kGauss; report->sum_kMean = h.sum_kMean;
  }
  const int err = h.error;
  const int worst = h.worst_problem;
  if (h.halted || h.error) c->pred_valid = false;  // the run stopped inside a step
  SHL_TRY(reset_report(c));
  if (err) {
    g_err = "device buffer capacity exceeded (contact pairs / linked cells)";
    return (shl_status)err;
  }
  return (shl_status)worst;
}

}  // namespace

shl_status shl_step(shl_ctx* c, uint32_t n_steps, const double* pressure_table, int use_graph,
                    shl_step_report* report) {
  if (!c) return SHL_ERR_ARG;
  std::vector<double> chunk;
  uint32_t done = 0, steps_before = 0;
  bool stop = false;
  Ctl hh;
  while (done < n_steps && !stop) {
    const uint32_t m = std::min<uint32_t>(n_steps - done, c->b.ptable_cap);
    double* t = c->h_table;
    if (!t) {
      chunk.resize(m);
      t = chunk.data();
    }
    for (uint32_t i = 0; i < m; ++i) t[i] = pressure_table ? pressure_table[done + i] : c->P.pressure;
    // one launch rewinds the table, arms the pause target (and clears the report before the first chunk)
    SHL_TRY(upload_table(c, t, m, kCtlArm | (done == 0 ? kCtlReset : 0u), false));
    const uint32_t target = steps_before + m;
    // one slot per attempt: with adaptive dt, repeated attempts leave steps to top up
    uint32_t attempts = m;
    for (int round = 0;; ++round) {
      SHL_TRY(enqueue_steps(c, attempts, use_graph != 0));
      SHL_TRY(ctl_get(c, hh));  // copy + stream synchronisation
      if (hh.halted || (hh.paused & 2u) || hh.steps_done >= target) break;
      if (round >= 100000) {
        g_err = "shl_step: steps were repeated without end (adaptive dt)";
        return SHL_ERR_TIMEOUT;
      }
      attempts = target - hh.steps_done;
    }
    done += m;
    steps_before = hh.steps_done;
    if (hh.halted) break;
    if (hh.paused & 2u) stop = true;
  }
  if (n_steps == 0) SHL_TRY(reset_report(c));
  return collect(c, report, n_steps ? &hh : nullptr);
}

shl_status shl_set_cavity_functions(shl_ctx* c, const char* rx, const char* ry, const char* rz) {
  if (!c) return SHL_ERR_ARG;
  if (!c->sc.cavity_contact) {
    g_err = "cavity contact is off";
    return SHL_ERR_ARG;
  }
  const char* ex[3] = {rx, ry, rz};
  std::vector<shl::expr::Op> prog[3];
  for (int k = 0; k < 3; ++k) {
    if (!ex[k] || !*ex[k]) continue;
    try {
      shl::expr::Expression e(ex[k]);
      if (e.size() != 1) throw std::runtime_error("one expression expected");
      if (e.uses("x") || e.uses("y") || e.uses("z")) throw std::runtime_error("semi-axes may depend on t and d only");
      prog[k] = e.compile();
    } catch (const std::exception& x) {
      g_err = x.what();
      return SHL_ERR_ARG;
    }
  }
  if (!c->d_rfun) SHL_TRY(dev_alloc(c, &c->d_rfun, 3 * (size_t)shl::expr::kMaxProgram));
  for (int k = 0; k < 3; ++k) {
    c->rfun_text[k] = prog[k].empty() ? std::string() : std::string(ex[k]);
    c->sc.rfun[k] = prog[k].empty() ? nullptr : c->d_rfun + k * shl::expr::kMaxProgram;
    c->sc.rfun_len[k] = (int32_t)prog[k].size();
    if (!prog[k].empty())
      SHL_CUDA_TRY(cudaMemcpyAsync(c->d_rfun + k * shl::expr::kMaxProgram, prog[k].data(),
                                   prog[k].size() * sizeof(shl::expr::Op), cudaMemcpyHostToDevice, c->stream));
  }
  SHL_CUDA_TRY(cudaStreamSynchronize(c->stream));
  if (c->graph) cudaGraphExecDestroy(c->graph);
  if (c->graph1) cudaGraphExecDestroy(c->graph1);
  c->graph = c->graph1 = nullptr;
  return SHL_OK;
}

shl_status shl_get_cavity_origins(shl_ctx* c, double* origins) {
  if (!c || !origins) return SHL_ERR_ARG;
  const size_t nd = 3 * (size_t)c->S.V;
  if (!c->b.cav_origin) {
    std::fill(origins, origins + nd, 0.0);
    return SHL_OK;
  }
  SHL_CUDA_TRY(cudaMemcpyAsync(origins, c->b.cav_origin, nd * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  SHL_CUDA_TRY(cudaStreamSynchronize(c->stream));
  return SHL_OK;
}

shl_status shl_set_cavity_origins(shl_ctx* c, const double* origins) {
  if (!c || !origins) return SHL_ERR_ARG;
  SHL_TRY(host_access(c));  // pending linked-cell pass; the step prediction is rebuilt
  if (!c->b.cav_origin) return SHL_OK;  // nothing to keep without cavity contact
  SHL_TRY(upload(c, c->b.cav_origin, origins, 3 * (size_t)c->S.V));
  SHL_CUDA_TRY(cudaStreamSynchronize(c->stream));
  return SHL_OK;
}

shl_status shl_get_dt(shl_ctx* c, double* dt, uint32_t* rejections) {
  if (!c) return SHL_ERR_ARG;
  Ctl h;
  SHL_TRY(ctl_get(c, h));
  if (dt) *dt = c->sc.adapt_every ? h.dt_cur : c->P.dt;
  if (rejections) *rejections = h.rejections;
  return SHL_OK;
}

shl_status shl_set_stop_function(shl_ctx* c, const char* expr) {
  if (!c) return SHL_ERR_ARG;
  if (!expr || !*expr) {
    c->sc.sfun = nullptr;
    c->sc.sfun_len = 0;
  } else {
    std::vector<shl::expr::Op> prog;
    try {
      shl::expr::Expression e(expr);
      if (e.size() != 1) throw std::runtime_error("one expression expected");
      if (e.uses("x") || e.uses("y") || e.uses("z")) throw std::runtime_error("the criterion may depend on t and d only");
      prog = e.compile();
    } catch (const std::exception& ex) {
      g_err = ex.what();
      return SHL_ERR_ARG;
    }
    if (!c->d_sfun) SHL_TRY(dev_alloc(c, &c->d_sfun, shl::expr::kMaxProgram));
    SHL_CUDA_TRY(cudaMemcpyAsync(c->d_sfun, prog.data(), prog.size() * sizeof(shl::expr::Op), cudaMemcpyHostToDevice,
                                 c->stream));
    SHL_CUDA_TRY(cudaStreamSynchronize(c->stream));
    c->sc.sfun = c->d_sfun;
    c->sc.sfun_len = (int32_t)prog.size();
  }
  if (c->graph) cudaGraphExecDestroy(c->graph);
  if (c->graph1) cudaGraphExecDestroy(c->graph1);
  c->graph = c->graph1 = nullptr;
  return SHL_OK;
}

shl_status shl_get_stream(shl_ctx* c, void** stream) {
  if (!c || !stream) return SHL_ERR_ARG;
  *stream = (void*)c->stream;
  return SHL_OK;
}

shl_status shl_upload_pressure_table(shl_ctx* c, const double* table, uint32_t n) {
  if (!c || (n && !table)) return SHL_ERR_ARG;
  return upload_table(c, table, n);
}

shl_status shl_step_enqueue(shl_ctx* c, uint32_t n_steps) {
  if (!c) return SHL_ERR_ARG;
  return enqueue_steps(c, n_steps, true);
}

shl_status shl_step_collect(shl_ctx* c, shl_step_report* report) {
  if (!c) return SHL_ERR_ARG;
  return collect(c, report);
}

shl_status shl_time_kernel(shl_ctx* c, int which, int reps, size_t flush_bytes, double* avg_ms) {
  if (!c || !avg_ms || reps <= 0 || (which != 0 && which != 1)) return SHL_ERR_ARG;
  if (flush_bytes > c->flush_bytes) {
    if (c->d_flush) cudaFree(c->d_flush);
    c->d_flush = nullptr;
    c->flush_bytes = 0;
    SHL_CUDA_TRY(cudaMalloc(&c->d_flush, flush_bytes));
    c->flush_bytes = flush_bytes;
  }
  Ctl h;
  SHL_TRY(ctl_get(c, h));
  const int32_t halted = h.halted;
  h.halted = 0;
  SHL_TRY(ctl_put(c, h));
  cudaEvent_t e0, e1;
  SHL_CUDA_TRY(cudaEventCreate(&e0));
  SHL_CUDA_TRY(cudaEventCreate(&e1));
  double total = 0.0;
  const size_t nd = 3 * (size_t)c->S.V;
  for (int r = 0; r < reps; ++r) {
    if (flush_bytes) launch_flush(c->d_flush, flush_bytes, (uint32_t)r, c->stream);
    cudaEventRecord(e0, c->stream);
    if (which == 0)
      launch_elements(c->b, c->sc, elem_launch(c, c->sc), c->stream, false);  // the element kernel alone
    else
      launch_gather_correct(c->b, c->sc, 0, false, c->d_fa, c->d_fa + nd, c->stream);
    cudaEventRecord(e1, c->stream);
    SHL_CUDA_TRY(cudaEventSynchronize(e1));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    total += ms;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  SHL_TRY(check_launch("shl_time_kernel"));
  SHL_TRY(ctl_get(c, h));
  h.halted = halted;
  SHL_TRY(ctl_put(c, h));
  *avg_ms = total / reps;
  return SHL_OK;
}

shl_status shl_profile_step(shl_ctx* c, double pressure, size_t flush_bytes, double* ms_out) {
  if (!c || !ms_out) return SHL_ERR_ARG;
  SHL_TRY(host_access(c));  // pending linked-cell pass; the step prediction is rebuilt
  if (flush_bytes > c->flush_bytes) {
    if (c->d_flush) cudaFree(c->d_flush);
    c->d_flush = nullptr;
    c->flush_bytes = 0;
    SHL_CUDA_TRY(cudaMalloc(&c->d_flush, flush_bytes));
    c->flush_bytes = flush_bytes;
  }
  SHL_TRY(upload_table(c, &pressure, 1));
  cudaEvent_t ev[8];
  for (auto& e : ev) SHL_CUDA_TRY(cudaEventCreate(&e));
  const DevBuf& b = c->b;
  const StepConst& sc = c->sc;
  cudaStream_t s = c->stream;
  if (flush_bytes) launch_flush(c->d_flush, flush_bytes, 7u, s);
  cudaEventRecord(ev[0], s);
  launch_predict(b, sc, RebuildCond{0, 0}, s);
  cudaEventRecord(ev[1], s);
  if (sc.contact) launch_rebuild(b, sc, s);
  cudaEventRecord(ev[2], s);
  launch_elements(b, sc, elem_launch(c, sc), s, false);
  cudaEventRecord(ev[3], s);
  if (sc.contact) launch_contact_force(b, sc, 0, s);
  cudaEventRecord(ev[4], s);
  launch_gather_correct(b, sc, 0, true, nullptr, nullptr, s);
  cudaEventRecord(ev[5], s);
  if (sc.contact) launch_rebuild(b, sc, s);
  cudaEventRecord(ev[6], s);
  launch_volume_end_step(b, sc, true, s);
  cudaEventRecord(ev[7], s);
  SHL_CUDA_TRY(cudaEventSynchronize(ev[7]));
  for (int k = 0; k < 7; ++k) {
    float ms = 0.f;
    cudaEventElapsedTime(&ms, ev[k], ev[k + 1]);
    ms_out[k] = ms;
  }
  for (auto& e : ev) cudaEventDestroy(e);
  return check_launch("shl_profile_step");
}

shl_status shl_measure_fp64_peak(double* tflops) {
  if (!tflops) return SHL_ERR_ARG;
  int dev = 0, sms = 0;
  SHL_CUDA_TRY(cudaGetDevice(&dev));
  SHL_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  cudaStream_t s;
  SHL_CUDA_TRY(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
  double* out = nullptr;
  SHL_CUDA_TRY(cudaMalloc(&out, 8 * 64 * 1024));
  const int blocks = 8 * sms, iters = 1 << 14;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  launch_fp64_peak(out, blocks, iters, s);  // warm-up
  float best = 1e30f;
  for (int r = 0; r < 5; ++r) {
    cudaEventRecord(e0, s);
    launch_fp64_peak(out, blocks, iters, s);
    cudaEventRecord(e1, s);
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    best = std::min(best, ms);
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  cudaStreamDestroy(s);
  SHL_TRY(check_launch("shl_measure_fp64_peak"));
  const double flops = 2.0 * 8.0 * iters * (double)blocks * 256.0;
  *tflops = flops / (best * 1e-3) / 1e12;
  return SHL_OK;
}

shl_status shl_get_contact_state(shl_ctx* c, uint32_t* pairs, uint8_t* stick, double* spring_origin, double* d2,
                                 size_t cap, size_t* n_pairs, double* du_sum) {
  if (!c) return SHL_ERR_ARG;
  SHL_TRY(flush_deferred_rebuild(c));
  Ctl h;
  SHL_TRY(ctl_get(c, h));
  if (n_pairs) *n_pairs = h.n_pairs;
  if (du_sum) *du_sum = h.du_sum;
  if (!c->sc.contact || h.n_pairs == 0) return SHL_OK;
  const size_t n = std::min<size_t>(cap, h.n_pairs);
  if (pairs && n) {
    std::vector<uint32_t> e1(n), e2(n);
    SHL_CUDA_TRY(cudaMemcpyAsync(e1.data(), c->b.pe1[0], n * 4, cudaMemcpyDeviceToHost, c->stream));
    SHL_CUDA_TRY(cudaMemcpyAsync(e2.data(), c->b.pe2[0], n * 4, cudaMemcpyDeviceToHost, c->stream));
    SHL_CUDA_TRY(cudaStreamSynchronize(c->stream));
    for (size_t i = 0; i < n; ++i) { pairs[2 * i] = e1[i]; pairs[2 * i + 1] = e2[i]; }
  }
  if (stick && n) SHL_CUDA_TRY(cudaMemcpyAsync(stick, c->b.pstick[0], n, cudaMemcpyDeviceToHost, c->stream));
  if (spring_origin && n)
    SHL_CUDA_TRY(cudaMemcpyAsync(spring_origin, c->b.porig[0], 3 * n * 8, cudaMemcpyDeviceToHost, c->stream));
  if (d2 && n) SHL_CUDA_TRY(cudaMemcpyAsync(d2, c->b.pd2[0], n * 8, cudaMemcpyDeviceToHost, c->stream));
  SHL_CUDA_TRY(cudaStreamSynchronize(c->stream));
  return SHL_OK;
}

shl_status shl_get_contact_pairs(shl_ctx* c, uint32_t* pairs, size_t cap, size_t* n_pairs) {
  return shl_get_contact_state(c, pairs, nullptr, nullptr, nullptr, cap, n_pairs, nullptr);
}

shl_status shl_get_contact_coords(shl_ctx* c, double* x, size_t cap, size_t* n_pairs) {
  if (!c) return SHL_ERR_ARG;
  SHL_TRY(flush_deferred_rebuild(c));
  SHL_TRY(flush_deferred_rebuild(c));
  Ctl h;
  SHL_TRY(ctl_get(c, h));
  if (n_pairs) *n_pairs = h.n_pairs;
  if (!c->sc.smooth) { g_err = "closest-point coordinates are kept for SMOOTH contact only"; return SHL_ERR_ARG; }
  const size_t n = std::min<size_t>(cap, h.n_pairs);
  if (x && n) {
    SHL_CUDA_TRY(cudaMemcpyAsync(x, c->b.pvw[0], 4 * n * 8, cudaMemcpyDeviceToHost, c->stream));
    SHL_CUDA_TRY(cudaStreamSynchronize(c->stream));
  }
  return SHL_OK;
}

shl_status shl_set_contact_coords(shl_ctx* c, const double* x, size_t n) {
  if (!c || (n && !x)) return SHL_ERR_ARG;
  SHL_TRY(host_access(c));  // pending linked-cell pass; the step prediction is rebuilt
  if (!c->sc.smooth) { g_err = "closest-point coordinates are kept for SMOOTH contact only"; return SHL_ERR_ARG; }
  Ctl h;
  SHL_TRY(ctl_get(c, h));
  if (n != h.n_pairs) { g_err = "coordinate count differs from the pair count"; return SHL_ERR_ARG; }
  if (n) SHL_TRY(upload(c, c->b.pvw[0], x, 4 * n));
  SHL_CUDA_TRY(cudaStreamSynchronize(c->stream));
  return SHL_OK;
}

shl_status shl_set_contact_state(shl_ctx* c, const uint32_t* pairs, const uint8_t* stick, const double* spring_origin,
                                 const double* d2, size_t n, double du_sum) {
  if (!c) return SHL_ERR_ARG;
  SHL_TRY(host_access(c));  // pending linked-cell pass; the step prediction is rebuilt
  if (!c->sc.contact) { g_err = "self-contact is off"; return SHL_ERR_ARG; }
  if (c->sc.n_cs) { g_err = "contact state files are written and read for single shells only"; return SHL_ERR_ARG; }
  if (n > c->sc.pairs_cap) { g_err = "too many pairs"; return SHL_ERR_CAPACITY; }
  const uint32_t F = c->S.F;
  std::vector<size_t> order(n);
  for (size_t i = 0; i < n; ++i) {
    order[i] = i;
    if (pairs[2 * i] >= F || pairs[2 * i + 1] >= F || pairs[2 * i] >= pairs[2 * i + 1]) {
      g_err = "pairs must satisfy eid1 < eid2 < n_faces";
      return SHL_ERR_ARG;
    }
  }
  std::sort(order.begin(), order.end(), [&](size_t x, size_t y) {
    return pairs[2 * x] != pairs[2 * y] ? pairs[2 * x] < pairs[2 * y] : pairs[2 * x + 1] < pairs[2 * y + 1];
  });
  std::vector<uint32_t> e1(n), e2(n), ptr(F + 1, 0);
  std::vector<uint8_t> st(n);
  std::vector<double> org(3 * n), dd(n);
  for (size_t k = 0; k < n; ++k) {
    const size_t i = order[k];
    e1[k] = pairs[2 * i];
    e2[k] = pairs[2 * i + 1];
    if (k > 0 && e1[k] == e1[k - 1] && e2[k] == e2[k - 1]) { g_err = "duplicate pair"; return SHL_ERR_ARG; }
    st[k] = stick ? (stick[i] ? 1 : 0) : 0;
    for (int q = 0; q < 3; ++q) org[3 * k + q] = spring_origin ? spring_origin[3 * i + q] : 0.0;
    dd[k] = d2 ? d2[i] : 0.0;
    ++ptr[e1[k] + 1];
  }
  for (uint32_t f = 0; f < F; ++f) ptr[f + 1] += ptr[f];
  if (n) {
    SHL_TRY(upload(c, c->b.pe1[0], e1.data(), n));
    SHL_TRY(upload(c, c->b.pe2[0], e2.data(), n));
    SHL_TRY(upload(c, c->b.pstick[0], st.data(), n));
    SHL_TRY(upload(c, c->b.porig[0], org.data(), 3 * n));
    SHL_TRY(upload(c, c->b.pd2[0], dd.data(), n));
    if (c->sc.smooth) {  // loaded pairs restart their closest-point search at 1/3
      std::vector<double> x(4 * n, 1.0 / 3.0);
      SHL_TRY(upload(c, c->b.pvw[0], x.data(), 4 * n));
    }
  }
  SHL_TRY(upload(c, c->b.pair_ptr[0], ptr.data(), F + 1));
  Ctl h;
  SHL_TRY(ctl_get(c, h));
  h.n_pairs = (uint32_t)n;
  h.du_sum = du_sum;
  h.csr_dirty = 1;
  SHL_TRY(ctl_put(c, h));
  launch_contact_csr(c->b, c->sc, c->stream);
  SHL_TRY(check_launch("shl_set_contact_state"));
  SHL_CUDA_TRY(cudaStreamSynchronize(c->stream));
  return SHL_OK;
}

shl_status shl_rebuild_contacts(shl_ctx* c) {
  if (!c) return SHL_ERR_ARG;
  SHL_TRY(host_access(c));  // pending linked-cell pass; the step prediction is rebuilt
  if (!c->sc.contact) return SHL_OK;
  Ctl h;
  SHL_TRY(ctl_get(c, h));
  h.rebuild = 1;
  h.problem = 0;
  h.halted = 0;
  h.error = 0;
  SHL_TRY(ctl_put(c, h));
  if (c->sc.n_cs) launch_batch_flags(c->b, c->sc, 0, c->stream);
  launch_rebuild(c->b, c->sc, c->stream);
  SHL_TRY(check_launch("shl_rebuild_contacts"));
  return finish_status(c, h);
}

shl_status shl_get_element_fields(shl_ctx* c, double* kG, double* kM, double* et, double* eb, double* area) {
  if (!c) return SHL_ERR_ARG;
  const size_t bytes = (size_t)c->S.F * sizeof(double);
  if (kG) SHL_CUDA_TRY(cudaMemcpyAsync(kG, c->b.kG, bytes, cudaMemcpyDeviceToHost, c->stream));
  if (kM) SHL_CUDA_TRY(cudaMemcpyAsync(kM, c->b.kM, bytes, cudaMemcpyDeviceToHost, c->stream));
  if (et) SHL_CUDA_TRY(cudaMemcpyAsync(et, c->b.etens, bytes, cudaMemcpyDeviceToHost, c->stream));
  if (eb) SHL_CUDA_TRY(cudaMemcpyAsync(eb, c->b.ebend, bytes, cudaMemcpyDeviceToHost, c->stream));
  if (area) SHL_CUDA_TRY(cudaMemcpyAsync(area, c->b.area, bytes, cudaMemcpyDeviceToHost, c->stream));
  SHL_CUDA_TRY(cudaStreamSynchronize(c->stream));
  return SHL_OK;
}

shl_status shl_residual(shl_ctx* c, double pressure, int flags, double* rel, double* f2, double* fext2) {
  if (!c) return SHL_ERR_ARG;
  SHL_TRY(host_access(c));  // pending linked-cell pass; the step prediction is rebuilt
  const size_t nd = 3 * (size_t)c->S.V;
  const uint32_t ns = (uint32_t)c->node_off.size() - 1;
  const bool ctx32 = c->sc.fp32 != 0;
  const bool fp64 = (flags & SHL_RESIDUAL_FP64) || !ctx32;
  const bool correct = (flags & SHL_RESIDUAL_CORRECT) && ctx32 && fp64;
  const bool with_contact = (flags & SHL_RESIDUAL_CONTACT) != 0;
  if (with_contact && (!c->sc.contact || c->sc.friction)) {
    g_err = "SHL_RESIDUAL_CONTACT needs self-contact without friction";
    return SHL_ERR_ARG;
  }
  if (!c->d_node_off) {
    SHL_TRY(dev_alloc(c, &c->d_node_off, ns + 1));
    SHL_TRY(dev_alloc(c, &c->d_norms, 2 * (size_t)ns));
    SHL_CUDA_TRY(cudaMemcpyAsync(c->d_node_off, c->node_off.data(), (ns + 1) * sizeof(uint32_t),
                                 cudaMemcpyHostToDevice, c->stream));
  }
  if (fp64 && ctx32 && !c->qe64) SHL_TRY(dev_alloc(c, &c->qe64, 3 * (size_t)c->S.n_slots_total));
  if (fp64 && ctx32 && !c->b.face_df) {  // the double-float FP64 path's constants
    SHL_TRY(dev_alloc(c, &c->b.face_df, c->S.face_df.size()));
    SHL_TRY(upload(c, c->b.face_df, c->S.face_df.data(), c->S.face_df.size()));
  }
  if (correct && !c->b.fcorr) {
    SHL_TRY(dev_alloc(c, &c->b.fcorr, nd));
    SHL_TRY(dev_alloc(c, &c->f32, nd));
    // the step graphs hold the buffer table by value: capture them again with the correction
    if (c->graph) cudaGraphExecDestroy(c->graph);
    if (c->graph1) cudaGraphExecDestroy(c->graph1);
    c->graph = c->graph1 = nullptr;
  }
  DevBuf b = c->b;
  b.fcorr = nullptr;
  SHL_CUDA_TRY(cudaMemcpyAsync(b.up, b.u, nd * sizeof(double), cudaMemcpyDeviceToDevice, c->stream));
  launch_positions(b, c->sc, c->stream);
  Ctl h;
  SHL_TRY(ctl_get(c, h));
  Ctl saved = h;
  h.halted = 0;
  h.pressure = c->P.compat_zero_pressure ? pressure * 0.0 : pressure;
  const double red = std::max((1.0 - static_cast<int>(h.time * 5.0) * 0.01), 0.5);
  h.volume_pressure = (c->P.bulk_modulus == 0 ? 0 : c->P.bulk_modulus * (h.volume0 * red / h.volume - 1));
  SHL_TRY(ctl_put(c, h));
  // f = pressure force - internal force (- the static self-contact force), then
  // the pressure force alone (no contact, no damping)
  StepConst sc = c->sc;
  sc.contact = 0;
  sc.cavity_contact = 0;
  DevBuf bf = b;
  if (fp64 && ctx32) {
    sc.fp32 = 0;
    bf.qe = c->qe64;
  }
  launch_elements(bf, sc, elem_launch(c, sc), c->stream);
  if (with_contact) {
    // the contact kernel at this state on copies of the per-pair state (the
    // list's scratch side), without contact damping
    StepConst scc = sc;
    scc.contact = 1;
    scc.self_damping = 0.0;
    DevBuf bc = bf;
    if (h.n_pairs) {
      SHL_CUDA_TRY(cudaMemcpyAsync(b.pd2[1], b.pd2[0], h.n_pairs * sizeof(double), cudaMemcpyDeviceToDevice, c->stream));
      SHL_CUDA_TRY(cudaMemcpyAsync(b.pstick[1], b.pstick[0], h.n_pairs, cudaMemcpyDeviceToDevice, c->stream));
      SHL_CUDA_TRY(cudaMemcpyAsync(b.porig[1], b.porig[0], 3 * h.n_pairs * sizeof(double), cudaMemcpyDeviceToDevice,
                                   c->stream));
      if (c->sc.smooth)
        SHL_CUDA_TRY(cudaMemcpyAsync(b.pvw[1], b.pvw[0], 4 * h.n_pairs * sizeof(double), cudaMemcpyDeviceToDevice,
                                     c->stream));
    }
    bc.pd2[0] = b.pd2[1];
    bc.pstick[0] = b.pstick[1];
    bc.porig[0] = b.porig[1];
    bc.pvw[0] = b.pvw[1];
    launch_contact_force(bc, scc, 0, c->stream);
    launch_gather_correct(bc, scc, 0, false, c->d_fa, nullptr, c->stream);
  } else {
    launch_gather_correct(bf, sc, 0, false, c->d_fa, nullptr, c->stream);
  }
  if (correct) {
    // the context's own FP32 force at the same state, and the defect the steps add to it
    StepConst s32 = c->sc;
    s32.contact = 0;
    s32.cavity_contact = 0;
    launch_elements(b, s32, elem_launch(c, s32), c->stream);
    launch_gather_correct(b, s32, 0, false, c->f32, nullptr, c->stream);
    launch_defect(c->d_fa, c->f32, nd, c->b.fcorr, c->stream);
  }
  if ((flags & SHL_RESIDUAL_CLEAR) && c->b.fcorr)
    SHL_CUDA_TRY(cudaMemsetAsync(c->b.fcorr, 0, nd * sizeof(double), c->stream));
  sc.internal_scale = 0.0;
  launch_elements(bf, sc, elem_launch(c, sc), c->stream);
  launch_gather_correct(bf, sc, 0, false, c->d_fa + nd, nullptr, c->stream);
  launch_shell_norms(c->d_fa, c->d_fa + nd, c->b.M, c->d_node_off, ns, c->d_norms, c->stream);
  SHL_TRY(check_launch("shl_residual"));
  std::vector<double> norms(2 * (size_t)ns);
  SHL_CUDA_TRY(cudaMemcpyAsync(norms.data(), c->d_norms, norms.size() * sizeof(double), cudaMemcpyDeviceToHost,
                               c->stream));
  SHL_CUDA_TRY(cudaStreamSynchronize(c->stream));
  // the step state is the stored one: restore the control block's step scalars
  Ctl h2;
  SHL_TRY(ctl_get(c, h2));
  h2.halted = saved.halted;
  h2.pressure = saved.pressure;
  h2.volume_pressure = saved.volume_pressure;
  SHL_TRY(ctl_put(c, h2));
  for (uint32_t k = 0; k < ns; ++k) {
    if (f2) f2[k] = norms[2 * k];
    if (fext2) fext2[k] = norms[2 * k + 1];
    if (rel) rel[k] = norms[2 * k + 1] > 0 ? std::sqrt(norms[2 * k] / norms[2 * k + 1]) : INFINITY;
  }
  return SHL_OK;
}

shl_status shl_set_pressure_function(shl_ctx* c, const char* expr) {
  if (!c) return SHL_ERR_ARG;
  if (!expr || !*expr) {
    c->sc.pfun = nullptr;
    c->sc.pfun_len = 0;
  } else {
    std::vector<shl::expr::Op> prog;
    try {
      shl::expr::Expression e(expr);
      if (e.size() != 1) throw std::runtime_error("one expression expected");
      if (e.uses("x") || e.uses("y") || e.uses("z")) throw std::runtime_error("the pressure may depend on t and d only");
      prog = e.compile();
    } catch (const std::exception& ex) {
      g_err = ex.what();
      return SHL_ERR_ARG;
    }
    if (!c->d_pfun) SHL_TRY(dev_alloc(c, &c->d_pfun, shl::expr::kMaxProgram));
    SHL_CUDA_TRY(cudaMemcpyAsync(c->d_pfun, prog.data(), prog.size() * sizeof(shl::expr::Op), cudaMemcpyHostToDevice,
                                 c->stream));
    SHL_CUDA_TRY(cudaStreamSynchronize(c->stream));
    c->sc.pfun = c->d_pfun;
    c->sc.pfun_len = (int32_t)prog.size();
  }
  // the step graphs hold the step constants by value
  if (c->graph) cudaGraphExecDestroy(c->graph);
  if (c->graph1) cudaGraphExecDestroy(c->graph1);
  c->graph = c->graph1 = nullptr;
  return SHL_OK;
}

shl_status shl_eval_pressure_function(shl_ctx* c, const double* t, uint32_t n, double* out) {
  if (!c || (n && (!t || !out))) return SHL_ERR_ARG;
  if (c->sc.pfun_len == 0) {
    g_err = "no pressure function set";
    return SHL_ERR_ARG;
  }
  if (n == 0) return SHL_OK;
  double* d = nullptr;
  SHL_CUDA_TRY(cudaMallocAsync((void**)&d, 2 * (size_t)n * sizeof(double), c->stream));
  SHL_CUDA_TRY(cudaMemcpyAsync(d, t, n * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  launch_eval_program(c->sc.pfun, c->sc.pfun_len, d, (int)n, d + n, c->stream);
  SHL_CUDA_TRY(cudaMemcpyAsync(out, d + n, n * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  SHL_CUDA_TRY(cudaFreeAsync(d, c->stream));
  SHL_CUDA_TRY(cudaStreamSynchronize(c->stream));
  return check_launch("shl_eval_pressure_function");
}

shl_status shl_get_energies(shl_ctx* c, shl_energies* e) {
  if (!c || !e) return SHL_ERR_ARG;
  Ctl h;
  SHL_TRY(ctl_get(c, h));
  fill_energies(h, e);
  return SHL_OK;
}

shl_status shl_context_size(shl_ctx* c, uint32_t* n_nodes, uint32_t* n_faces) {
  if (!c) return SHL_ERR_ARG;
  if (n_nodes) *n_nodes = c->S.V;
  if (n_faces) *n_faces = c->S.F;
  return SHL_OK;
}

shl_status shl_context_mesh(shl_ctx* c, double* xyz, uint32_t* faces) {
  if (!c) return SHL_ERR_ARG;
  if (xyz) std::memcpy(xyz, c->S.X.data(), c->S.X.size() * sizeof(double));
  if (faces) std::memcpy(faces, c->S.tri.data(), c->S.tri.size() * sizeof(uint32_t));
  return SHL_OK;
}

shl_status shl_get_node_fields(shl_ctx* c, double* ekin, double* ecav, double* eself, double* efric,
                               double* mass) {
  if (!c) return SHL_ERR_ARG;
  const uint32_t V = c->S.V, F = c->S.F;
  const std::vector<double>& Minv = c->S.Minv;
  if (ecav) {
    if (c->b.cav_ecav) {
      SHL_CUDA_TRY(cudaMemcpyAsync(ecav, c->b.cav_ecav, V * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
      SHL_CUDA_TRY(cudaStreamSynchronize(c->stream));
    } else {
      std::fill(ecav, ecav + V, 0.0);
    }
  }
  if (mass)
    for (uint32_t n = 0; n < V; ++n) mass[n] = 1.0 / Minv[3 * (size_t)n];
  if (!ekin && !eself && !efric) return SHL_OK;
  std::vector<double> area(F), v(3 * (size_t)V);
  SHL_CUDA_TRY(cudaMemcpyAsync(area.data(), c->b.area, F * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  SHL_CUDA_TRY(cudaMemcpyAsync(v.data(), c->b.v, v.size() * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  Ctl h;
  SHL_TRY(ctl_get(c, h));
  const std::vector<uint32_t>& T = c->S.tri;
  if (ekin) {
    // Ekin_node / avg_area_node (ShellSystem.C:2796-2812, 2462-2481)
    std::vector<double> asum(V, 0.0);
    std::vector<uint32_t> cnt(V, 0);
    for (uint32_t e = 0; e < F; ++e)
      for (int k = 0; k < 3; ++k) {
        asum[T[3 * (size_t)e + k]] += area[e];
        ++cnt[T[3 * (size_t)e + k]];
      }
    for (uint32_t n = 0; n < V; ++n) {
      double en = 0.0;
      for (int d = 0; d < 3; ++d) {
        const size_t k = 3 * (size_t)n + d;
        en += v[k] * v[k] / Minv[k];
      }
      ekin[n] = 0.5 * en / (asum[n] / cnt[n]);
    }
  }
  if (!eself && !efric) return SHL_OK;
  if (eself) std::fill(eself, eself + V, 0.0);
  if (efric) {
    if (c->b.cav_efric) {
      SHL_CUDA_TRY(cudaMemcpyAsync(efric, c->b.cav_efric, V * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
      SHL_CUDA_TRY(cudaStreamSynchronize(c->stream));
    } else {
      std::fill(efric, efric + V, 0.0);
    }
  }
  const uint32_t np = c->sc.contact ? h.n_pairs : 0u;
  if (np == 0) return SHL_OK;
  // per-pair energies spread over the six nodes with weights 0.5 (u, v, w) / area_min
  // (ShellSystem.C:1862-1877)
  std::vector<uint32_t> e1(np), e2(np);
  std::vector<double> pf((size_t)kPairOut * np);
  SHL_CUDA_TRY(cudaMemcpyAsync(e1.data(), c->b.pe1[0], np * 4, cudaMemcpyDeviceToHost, c->stream));
  SHL_CUDA_TRY(cudaMemcpyAsync(e2.data(), c->b.pe2[0], np * 4, cudaMemcpyDeviceToHost, c->stream));
  SHL_CUDA_TRY(cudaMemcpyAsync(pf.data(), c->b.pforce, pf.size() * 8, cudaMemcpyDeviceToHost, c->stream));
  SHL_CUDA_TRY(cudaStreamSynchronize(c->stream));
  for (uint32_t j = 0; j < np; ++j) {
    const double* o = &pf[(size_t)kPairOut * j];
    const double es = o[7], ef = o[8];
    if (es == 0.0 && ef == 0.0) continue;
    const uint32_t ee[2] = {e1[j], e2[j]};
    const double area_min = std::min(area[ee[0]], area[ee[1]]);
    for (int s = 0; s < 2; ++s) {
      const double vv = o[3 + 2 * s], ww = o[4 + 2 * s];
      const double w[3] = {0.5 * (1.0 - vv - ww) / area_min, 0.5 * vv / area_min, 0.5 * ww / area_min};
      for (int k = 0; k < 3; ++k) {
        const uint32_t n = T[3 * (size_t)ee[s] + k];
        if (eself) eself[n] += w[k] * es;
        if (efric) efric[n] += w[k] * ef;
      }
    }
  }
  return SHL_OK;
}

shl_status shl_set_element_variant(shl_ctx* c, int variant) {
  if (!c) return SHL_ERR_ARG;
  if (variant < 0) return tune_elements(c);
  if (variant >= kNumElemVariants || (variant >= kFirstFp32Variant) != (c->sc.fp32 != 0)) {
    g_err = "element variant does not exist for this precision";
    return SHL_ERR_ARG;
  }
  if (c->sc.fp32) c->var32 = variant; else c->var64 = variant;
  apply_variant(c);
  if (c->graph) cudaGraphExecDestroy(c->graph);
  if (c->graph1) cudaGraphExecDestroy(c->graph1);
  c->graph = c->graph1 = nullptr;
  return SHL_OK;
}

shl_status shl_get_element_variant(shl_ctx* c, int* variant, char* name, size_t cap, float* tuned_ms) {
  if (!c) return SHL_ERR_ARG;
  const int v = c->sc.fp32 ? c->var32 : c->var64;
  if (variant) *variant = v;
  if (name && cap) {
    std::strncpy(name, kElemVariants[v].name, cap - 1);
    name[cap - 1] = 0;
  }
  if (tuned_ms) std::memcpy(tuned_ms, c->variant_ms, sizeof(c->variant_ms));
  return SHL_OK;
}

shl_status shl_scale_damping(shl_ctx* c, double factor) {
  if (!c || !(factor >= 0)) return SHL_ERR_ARG;
  SHL_TRY(host_access(c));  // pending linked-cell pass; the step prediction is rebuilt
  const size_t nd = 3 * (size_t)c->S.V;
  std::vector<double> C(nd);
  for (size_t i = 0; i < nd; ++i) C[i] = factor * c->S.C[i];
  SHL_TRY(upload(c, c->b.C, C.data(), nd));
  SHL_CUDA_TRY(cudaStreamSynchronize(c->stream));
  return SHL_OK;
}

shl_status shl_get_mass_damping(shl_ctx* c, double* Minv, double* C) {
  if (!c) return SHL_ERR_ARG;
  const size_t nd = 3 * (size_t)c->S.V;
  if (Minv) std::memcpy(Minv, c->S.Minv.data(), nd * sizeof(double));
  if (C) std::memcpy(C, c->S.C.data(), nd * sizeof(double));
  return SHL_OK;
}

shl_status shl_internal_force_noalloc(shl_ctx* c, const double* u_dev, double pressure, double* f_dev,
                                      void* stream) {
  if (!c || !u_dev || !f_dev) { g_err = "null argument"; return SHL_ERR_ARG; }
  if (c->sc.contact || c->P.bulk_modulus != 0.0 || c->sc.fp32) {
    g_err = "shl_internal_force_noalloc: self-contact, bulk-modulus pressure and FP32 element forces are not "
            "evaluated here";
    return SHL_ERR_ARG;
  }
  if (c->S.n_slots_total > noalloc_max_slots()) {
    g_err = "shl_internal_force_noalloc: the shell has " + std::to_string(c->S.n_slots_total) +
            " (face, patch node) slots, above the scratch limit of " + std::to_string(noalloc_max_slots()) +
            " slots (32768 faces of 12-node patches)";
    return SHL_ERR_CAPACITY;
  }
  int dev = -1;
  SHL_CUDA_TRY(cudaGetDevice(&dev));
  if (dev != c->device) {
    g_err = "shl_internal_force_noalloc: the current device (" + std::to_string(dev) +
            ") is not the context's device (" + std::to_string(c->device) + ")";
    return SHL_ERR_ARG;
  }
  // Only the context's constant set-up data are read (patches, face constants,
  // basis, gather CSR): no step state, so a pending candidate-list pass or the
  // stored prediction are neither needed nor changed.
  const double p = c->P.compat_zero_pressure ? pressure * 0.0 : pressure;
  cudaError_t e = launch_force_noalloc(c->b, c->sc, c->eg, c->elem_blocks, u_dev, p, f_dev, (cudaStream_t)stream);
  if (e != cudaSuccess) {
    g_err = std::string("shl_internal_force_noalloc: ") + cudaGetErrorString(e);
    return SHL_ERR_CUDA;
  }
  return SHL_OK;
}

}  // extern "C"
