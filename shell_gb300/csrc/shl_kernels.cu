// shl_kernels.cu -- FP64 kernels of one explicit Newmark step.
//
//   k_predict        nodes  ShellSystem.C:972-989 (predictor), 2591-2652
//                           (check_increment), 2484-2502 (positions), and the
//                           scalar part of prepare_next_step (924-949)
//   k_elements       faces  1382-1464 (deformed metrics), 1125-1314 (internal
//                           force), 1474-1585 (pressure), 2737-2788 (curvatures)
//   k_contact_force  pairs  1792-1907 with Friction.C:4-60
//   k_gather_correct nodes  the per-node sum of element and contact shares
//                           (a deterministic gather, no atomics), 1006-1008
//                           (damping, M^-1), 1046-1090 (corrector, check_increment)
//   k_volume_end     faces  2505-2541 (enclosed volume), 2830-2843 (sums),
//                           2901-2953 (problem handling)
//
// Reductions are fixed-order (warp shuffles, then the last block to finish sums
// the per-block partials in block order), so results are bitwise reproducible
// run to run.  The predictor, positions and the contact path use separately
// rounded operations (no FMA) so the contact candidate list agrees bit for bit
// with the CPU path at the same state.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <mutex>

#include "shl_geom.h"
#include "shl_internal.cuh"
#include "shl_df.cuh"

namespace shl {


// ---------------------------------------------------------------- helpers --

__device__ __forceinline__ bool inactive(const Ctl* ctl) {
  return ctl->halted != 0 || ctl->paused != 0;
}

// the rebuild IF node's condition (one thread, after ctl->rebuild is final)
__device__ __forceinline__ void set_rebuild_cond(const RebuildCond& rc, const Ctl* ctl) {
  if (rc.has) cudaGraphSetConditional(rc.h, (ctl->rebuild != 0 && ctl->halted == 0) ? 1u : 0u);
}

// ShellSystem::set_newmark_parameters (ShellSystem.C:744-759) with the bounds
// of ShellSystem.C:306-310, into the control block (adaptive dt)
__device__ void set_newmark(Ctl* ctl, const StepConst& sc, double new_dt) {
  double dt = fmax(new_dt, sc.dt_min_eff);
  dt = fmin(dt, sc.dt_max_eff);
  const double beta = sc.beta, gamma = sc.gamma;
  ctl->dt_cur = dt;
  ctl->nm[0] = beta * dt * dt;
  ctl->nm[1] = gamma / (beta * dt);
  ctl->nm[2] = 1 / (beta * dt);
  ctl->nm[3] = 1 / (2 * beta) - 1;
  ctl->nm[4] = gamma / beta - 1;
  ctl->nm[5] = dt * (gamma / (2 * beta) - 1);
  ctl->nm[6] = (1 - gamma) * dt;
  ctl->nm[7] = gamma * dt;
  ctl->nm[8] = dt * dt * (0.5 - beta);
  ctl->nm[9] = dt * dt * fabs(beta - 1. / 6);
}

// fixed-order block sum; result valid in thread 0; sh needs blockDim/32 doubles
__device__ __forceinline__ double block_sum(double x, double* sh) {
  for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  __syncthreads();
  if (lane == 0) sh[warp] = x;
  __syncthreads();
  if (warp == 0) {
    x = (lane < (int)(blockDim.x >> 5)) ? sh[lane] : 0.0;
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
  }
  return x;
}

__device__ __forceinline__ double block_max(double x, double* sh) {
  for (int o = 16; o > 0; o >>= 1) x = fmax(x, __shfl_down_sync(0xffffffffu, x, o));
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  __syncthreads();
  if (lane == 0) sh[warp] = x;
  __syncthreads();
  if (warp == 0) {
    x = (lane < (int)(blockDim.x >> 5)) ? sh[lane] : 0.0;
    for (int o = 16; o > 0; o >>= 1) x = fmax(x, __shfl_down_sync(0xffffffffu, x, o));
  }
  return x;
}

// true in every thread of the block that finished last; resets the counter
__device__ __forceinline__ bool last_block(uint32_t* counter) {
  __shared__ bool is_last;
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) {
    const uint32_t t = atomicAdd(counter, 1u);
    is_last = (t == gridDim.x - 1);
    if (is_last) *counter = 0;
  }
  __syncthreads();
  return is_last;
}

// Block sums of N values per thread (kBlock threads), transposed through shared
// memory: warp k adds column k (its lane's 8 values in order, then a shuffle
// tree), so the FP64 adds and shuffles are N warps' worth instead of every
// warp's.  Fixed order; the sums land in thread 0's x.
struct TransposedSum {
  double v[8][kBlock];
  double res[8];
};
template <int N>
__device__ __forceinline__ void block_sum_t(double* x, TransposedSum& sh) {
  static_assert(N <= 8 && N * 32 <= kBlock, "one warp per value");
  const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
  __syncthreads();  // the shared buffer may still be read by a previous call
#pragma unroll
  for (int k = 0; k < N; ++k) sh.v[k][t] = x[k];
  __syncthreads();
  if (warp < N) {
    double a = sh.v[warp][lane];
#pragma unroll
    for (int i = 1; i < kBlock / 32; ++i) a += sh.v[warp][lane + 32 * i];
    for (int o = 16; o > 0; o >>= 1) a += __shfl_down_sync(0xffffffffu, a, o);
    if (lane == 0) sh.res[warp] = a;
  }
  __syncthreads();
  if (t == 0)
#pragma unroll
    for (int k = 0; k < N; ++k) x[k] = sh.res[k];
}
template <int N>
__device__ __forceinline__ void sum_partials_t(const double* partial, int nb, TransposedSum& sh, double* out) {
#pragma unroll
  for (int k = 0; k < N; ++k) out[k] = 0.0;
  for (int b = threadIdx.x; b < nb; b += blockDim.x)
#pragma unroll
    for (int k = 0; k < N; ++k) out[k] += __ldcg(&partial[(size_t)b * 8 + k]);
  block_sum_t<N>(out, sh);
}

// per-face measurement densities times area (E_tens, E_bend, kGauss, kMean) and the area
__device__ __forceinline__ void face_totals(const DevBuf& b, uint32_t e, double* v) {
  const double ar = b.area[e];
  v[0] = b.etens[e] * ar;
  v[1] = b.ebend[e] * ar;
  v[2] = b.kG[e] * ar;
  v[3] = b.kM[e] * ar;
  v[4] = ar;
}

// sum of partial[k * stride + b] over blocks b in fixed order (last block only)
__device__ __forceinline__ double sum_partials(const double* partial, int k, int nb, double* sh) {
  double s = 0.0;
  for (int b = threadIdx.x; b < nb; b += blockDim.x) s += __ldcg(&partial[(size_t)b * 8 + k]);
  return block_sum(s, sh);
}

__device__ __forceinline__ void register_problem(Ctl* ctl, int p) { atomicMax(&ctl->problem, p); }

// tolerance of the linked-cell rebuild test, ShellSystem.C:1917-1919
__device__ __forceinline__ double rebuild_tolerance(const StepConst& sc, const Ctl* ctl) {
  const double cs = __dmul_rn(sc.cell_size_mult, ctl->avg_elem_size);
  return __dmul_rn(sc.cell_margin, cs);
}

// ---- batch with self-contact: the linked-cell trigger of every shell ----
// (ShellCell; the same decisions as the single-shell code below, per shell)
__device__ __forceinline__ double shell_tolerance(const StepConst& sc, const ShellCell& S) {
  const double cs = __dmul_rn(S.cell_size_mult, S.avg_elem_size);
  return __dmul_rn(sc.cell_margin, cs);
}

// Largest |du|^2 of a node pass, per shell (which: 0 du2_acc, 1 du2n_acc).
// Called by every lane of a warp; a warp whose nodes belong to one shell makes
// one atomic.  NaNs are skipped, as fmax skips them in the single-shell maximum.
__device__ __forceinline__ void shell_max_acc(const DevBuf& b, const StepConst& sc, uint32_t n, double x, int which) {
  const uint32_t s = n < sc.V ? b.node_shell[n] : 0xffffffffu;
  const uint32_t s0 = __shfl_sync(0xffffffffu, s, 0);
  if (s0 == 0xffffffffu) return;  // the whole warp is past the last node
  const bool valid = n < sc.V && !isnan(x);
  if (__all_sync(0xffffffffu, s == s0 || n >= sc.V)) {
    double m = valid ? x : 0.0;
    for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) {
      ShellCell& S = b.shc[s0];
      atomicMax(which ? &S.du2n_acc : &S.du2_acc, (unsigned long long)__double_as_longlong(m));
    }
  } else if (valid) {
    ShellCell& S = b.shc[s];
    atomicMax(which ? &S.du2n_acc : &S.du2_acc, (unsigned long long)__double_as_longlong(x));
  }
}

// takes (and clears) a shell's accumulated maximum
__device__ __forceinline__ double shell_take_max(unsigned long long* acc) {
  return __longlong_as_double((long long)atomicExch(acc, 0ull));
}

// check_increment(false) of every shell (all threads of one block; thread t
// takes shells t, t + blockDim.x, ...): the largest |du|^2 of the pass that
// just ran (from_acc), or that the fused corrector predicted (du2_pred).  The
// control block gets the OR of the shells' flags and the IF condition, as
// begin_step sets them for one shell.
__device__ void batch_begin_check(const DevBuf& b, const StepConst& sc, const RebuildCond& rc, bool fused,
                                  bool from_acc) {
  Ctl* ctl = b.ctl;
  int r = 0, rb = 0;
  for (uint32_t s = threadIdx.x; s < sc.n_cs; s += blockDim.x) {
    ShellCell& S = b.shc[s];
    const double mm = from_acc ? shell_take_max(&S.du2_acc) : S.du2_pred;
    const double du_max = sqrt(mm);
    const bool finite = isfinite(du_max);
    if (finite) {
      if (du_max > 0.5 * S.thickness) register_problem(ctl, SHL_LARGE_DISP);
    } else {
      register_problem(ctl, SHL_NOT_FINITE);
    }
    if (fused && S.rebuild_pending) {  // the corrector's pass first; k_rebuild_second updates du_sum
      S.rebuild = 1u;
      r = 1;
      continue;
    }
    if (finite) S.du_sum = __dadd_rn(S.du_sum, __dmul_rn(2.0, du_max));
    const uint32_t flag = S.du_sum >= shell_tolerance(sc, S) ? 1u : 0u;
    if (fused) {
      S.rebuild = 0u;
      S.rebuild_b = flag;
      rb |= (int)flag;
    } else {
      S.rebuild = flag;
      r |= (int)flag;
    }
  }
  r = __syncthreads_or(r);
  rb = __syncthreads_or(rb);
  if (threadIdx.x != 0) return;
  ctl->rebuild = r ? 1u : 0u;
  if (fused) ctl->rebuild_b = rb ? 1u : 0u;
  if (rc.has) cudaGraphSetConditional(rc.h, ((r || rb) && ctl->halted == 0) ? 1u : 0u);
}

// check_increment(true) of every shell after a corrector (all threads of one
// block): fused (mode 3) leaves each shell's flag pending for the next step's
// IF node and keeps the next prediction's maximum in du2_pred
__device__ void batch_correct_check(const DevBuf& b, const StepConst& sc, const RebuildCond& rc, bool fused) {
  Ctl* ctl = b.ctl;
  int r = 0;
  for (uint32_t s = threadIdx.x; s < sc.n_cs; s += blockDim.x) {
    ShellCell& S = b.shc[s];
    const double du_max = sqrt(shell_take_max(&S.du2_acc));
    if (fused) S.du2_pred = shell_take_max(&S.du2n_acc);
    if (isfinite(du_max)) {
      S.du_sum = __dadd_rn(S.du_sum, __dmul_rn(2.0, du_max));
      if (du_max == 0.0)
        register_problem(ctl, SHL_NO_DISP_CHANGE);
      else if (du_max > 0.5 * S.thickness)
        register_problem(ctl, SHL_LARGE_DISP);
    } else {
      register_problem(ctl, SHL_NOT_FINITE);
    }
    const uint32_t flag = S.du_sum >= shell_tolerance(sc, S) ? 1u : 0u;
    if (fused)
      S.rebuild_pending = flag;
    else
      S.rebuild = flag;
    r |= (int)flag;
  }
  r = __syncthreads_or(r);
  if (threadIdx.x != 0) return;
  if (fused) {
    ctl->rebuild_pending = r ? 1u : 0u;
    return;
  }
  ctl->rebuild = r ? 1u : 0u;
  set_rebuild_cond(rc, ctl);
}

// ---- float-pair ("double-float") arithmetic for the FP64 path's two
// basis contractions.  GB300 issues 64 FP32 FMAs per FP64 FMA, so a product
// sum carried as an unevaluated pair hi + lo of floats (about 48 significant
// bits: TwoProd by FMA, TwoSum by Knuth, with the lo parts accumulated; the
// intrinsics keep the compiler from fusing the error terms) is several times
// cheaper than the same sum in FP64, and its error (~2^-48 of the summands)
// stays far below the path's 1e-12 budget: the contractions produce the
// displacement derivatives and the per-slot force shares, and the
// cancellation-prone steps (metric differences, the nodal gather) stay FP64.
__device__ __forceinline__ void df_madd(float& ah, float& al, float bh, float bl, float xh, float xl) {
  const float p = __fmul_rn(bh, xh);
  float e = __fmaf_rn(bh, xh, -p);
  e = __fmaf_rn(bh, xl, e);
  e = __fmaf_rn(bl, xh, e);
  const float s = __fadd_rn(ah, p);
  const float bb = __fsub_rn(s, ah);
  const float err = __fadd_rn(__fsub_rn(ah, __fsub_rn(s, bb)), __fsub_rn(p, bb));
  al = __fadd_rn(al, __fadd_rn(e, err));
  ah = s;
}

__device__ __forceinline__ void df_split(double x, float& h, float& l) {
  h = __double2float_rn(x);
  l = __double2float_rn(x - (double)h);
}

__device__ __forceinline__ double df_value(float h, float l) { return (double)h + (double)l; }

// 16-byte asynchronous global -> shared copy (LDGSTS; both addresses 16-byte
// aligned) and the wait for all of this thread's copies
__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
  const uint32_t d = (uint32_t)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 16;\n" ::"r"(d), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async4(void* smem, const void* gmem) {
  const uint32_t d = (uint32_t)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(d), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

// dynamic shared memory of the double-float element kernels: the displacements
// (hi and lo float4) of up to 12 patch slots per thread
constexpr int kDfStageSlots = 12;
constexpr size_t df_stage_bytes(int block) { return (size_t)kDfStageSlots * 2 * sizeof(float4) * block; }
// the one-round kernel: staging columns of its block plus the basis tables
// (hi and lo floats) of every patch group
constexpr size_t flat_smem_bytes() {
  return df_stage_bytes(kFlatBlock) + (size_t)kMaxGroups * 2 * kMaxSlots * 6 * sizeof(float);
}
static_assert(flat_smem_bytes() <= 232448, "the one-round element kernel exceeds the shared memory of a block");

// ---------------------------------------------------------------- cavity --
// effective semi-axes and friction scope (update_derived, ShellSystem.C:421-436)
struct CavityGeom {
  double R_eff[3], inv_R2[3], avg_R_eff, opd_friction;
};

__device__ __forceinline__ CavityGeom cavity_geom(const double* R, const StepConst& sc) {
  CavityGeom g;
  const double h_half = 0.5 * sc.thickness;
  for (int c = 0; c < 3; ++c) {
    g.R_eff[c] = R[c] - h_half;
    g.inv_R2[c] = 1 / (g.R_eff[c] * g.R_eff[c]);
  }
  g.avg_R_eff = (g.R_eff[0] + g.R_eff[1] + g.R_eff[2]) / 3;
  const double q = 1 - sc.static_friction_tol * sc.thickness / g.avg_R_eff;
  g.opd_friction = q * q;
  return g;
}

// cavity surface (Knud Thomsen's approximation for the ellipsoid, an ellipse
// circumference approximation for the cylinder), ShellSystem.C:441-468
__device__ double cavity_surface(const double* R, int type) {
  const double Rx = R[0], Ry = R[1], Rz = R[2];
  if (type == SHL_CAVITY_BOX) return 8 * (Rx * Ry + Rx * Rz + Ry * Rz);
  if (type == SHL_CAVITY_CYLINDER) {
    const double lambda = (Ry - Rz) / (Ry + Rz);
    const double lambda32 = 3 * lambda * lambda;
    return 2 * 3.141592653589793238 * ((Ry + Rz) * (1 + lambda32 / (10 + sqrt(4 - lambda32))) + Ry * Rz);
  }
  return 4 * 3.141592653589793238 *
         pow((pow(Rx * Ry, 1.6) + pow(Rx * Rz, 1.6) + pow(Ry * Rz, 1.6)) / 3, 0.625);
}

// ------------------------------------------------ config expressions --
// Stack-machine evaluation of a program compiled by shl_expr.h, one thread;
// bounded by the program length (at most shl::expr::kMaxProgram ops, each
// jump forward) and stack depth (checked when compiling).
__device__ double eval_program(const shl::expr::Op* prog, int n, double t, double d) {
  using namespace shl::expr;
  double st[kMaxStack];
  int sp = 0;
  const double vars[5] = {t, d, 0.0, 0.0, 0.0};
  for (int pc = 0; pc < n && pc < kMaxProgram;) {
    const Op op = prog[pc++];
    switch (op.code) {
      case OP_CONST: st[sp++] = op.value; break;
      case OP_VAR: st[sp++] = vars[op.arg]; break;
      case OP_NEG: st[sp - 1] = -st[sp - 1]; break;
      case OP_JZ: {
        const double c = st[--sp];
        if (c == 0.0) pc = op.arg;
        break;
      }
      case OP_JMP: pc = op.arg; break;
      case OP_FUN1: {
        const double x = st[sp - 1];
        double r = 0.0;
        switch (op.arg) {
          case F_SIN: r = sin(x); break;
          case F_COS: r = cos(x); break;
          case F_TAN: r = tan(x); break;
          case F_ASIN: r = asin(x); break;
          case F_ACOS: r = acos(x); break;
          case F_ATAN: r = atan(x); break;
          case F_SINH: r = sinh(x); break;
          case F_COSH: r = cosh(x); break;
          case F_TANH: r = tanh(x); break;
          case F_ASINH: r = asinh(x); break;
          case F_ACOSH: r = acosh(x); break;
          case F_ATANH: r = atanh(x); break;
          case F_EXP: r = exp(x); break;
          case F_LOG: r = log(x); break;
          case F_LOG2: r = log2(x); break;
          case F_LOG10: r = log10(x); break;
          case F_SQRT: r = sqrt(x); break;
          case F_SIGN: r = (double)((x > 0.0) - (x < 0.0)); break;
          case F_RINT: r = rint(x); break;
          case F_ABS: r = fabs(x); break;
        }
        st[sp - 1] = r;
        break;
      }
      case OP_MIN:
      case OP_MAX:
      case OP_SUM:
      case OP_AVG: {
        const int k = op.arg;
        double r = st[sp - k];
        if (op.code == OP_SUM || op.code == OP_AVG) r = 0.0;
        for (int i = sp - k; i < sp; ++i) {
          const double x = st[i];
          if (op.code == OP_MIN) r = x < r ? x : r;
          else if (op.code == OP_MAX) r = x > r ? x : r;
          else r += x;
        }
        if (op.code == OP_AVG) r /= (double)k;
        sp -= k;
        st[sp++] = r;
        break;
      }
      default: {
        const double b = st[--sp], a = st[sp - 1];
        double r = 0.0;
        switch (op.code) {
          case OP_ADD: r = a + b; break;
          case OP_SUB: r = a - b; break;
          case OP_MUL: r = a * b; break;
          case OP_DIV: r = a / b; break;
          case OP_POW: r = pow(a, b); break;
          case OP_LT: r = a < b; break;
          case OP_GT: r = a > b; break;
          case OP_LE: r = a <= b; break;
          case OP_GE: r = a >= b; break;
          case OP_EQ: r = a == b; break;
          case OP_NE: r = a != b; break;
          case OP_AND: r = (a != 0.0 && b != 0.0); break;
          case OP_OR: r = (a != 0.0 || b != 0.0); break;
        }
        st[sp - 1] = r;
      }
    }
  }
  return sp > 0 ? st[sp - 1] : 0.0;
}

__global__ void k_eval_program(const shl::expr::Op* prog, int n, const double* t, int m, double* out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < m) out[i] = eval_program(prog, n, t[i], 0.0);
}

void launch_eval_program(const void* prog, int n, const double* t, int m, double* out, cudaStream_t s) {
  k_eval_program<<<(m + 127) / 128, 128, 0, s>>>((const shl::expr::Op*)prog, n, t, m, out);
}

// ------------------------------------------------------------ predictor --
// One node's prediction (ShellSystem.C:972-989): u_pred = u + dt v + a8 a,
// v_pred = v + a6 a, positions X + u_pred into `pos`, the FP32 or float-pair
// copy of u_pred; returns |u_pred - u|^2.  Shared by k_predict and the fused
// corrector of k_gather_correct, so both give the same bits.
__device__ __forceinline__ double predict_node(const DevBuf& b, const StepConst& sc, uint32_t n, const double* u,
                                               const double* v, const double* a, double dt, double nm8, double nm6,
                                               double* pos) {
  double d[3];
  float uh[3], ul[3], u32[3];
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    const size_t k = 3 * (size_t)n + c;
    double up, vp;
    if (sc.contact) {
      // separately rounded, as the host does: positions feed the contact list
      up = __dadd_rn(__dmul_rn(dt, v[c]), u[c]);
      up = __dadd_rn(__dmul_rn(nm8, a[c]), up);
      vp = __dadd_rn(__dmul_rn(nm6, a[c]), v[c]);
    } else {
      up = fma(nm8, a[c], fma(dt, v[c], u[c]));
      vp = fma(nm6, a[c], v[c]);
    }
    b.up[k] = up;
    if (sc.fp32)
      u32[c] = (float)up;
    else
      df_split(up, uh[c], ul[c]);
    b.vp[k] = vp;
    pos[k] = __dadd_rn(b.X[k], up);
    d[c] = __dsub_rn(up, u[c]);
  }
  if (sc.fp32) {
    b.up32[n] = make_float4(u32[0], u32[1], u32[2], 0.f);
  } else {
    b.upk[2 * (size_t)n] = make_float4(uh[0], uh[1], uh[2], 0.f);
    b.upk[2 * (size_t)n + 1] = make_float4(ul[0], ul[1], ul[2], 0.f);
  }
  return __dadd_rn(__dadd_rn(__dmul_rn(d[0], d[0]), __dmul_rn(d[1], d[1])), __dmul_rn(d[2], d[2]));
}

// The scalar start of a step (one thread): prepare_next_step (time, the step's
// pressure, cavity semi-axes, volume pressure) and check_increment(false) with
// the predictor's largest |du|^2; sets the rebuild flag and the IF condition.
// fused: the IF node holds both passes of the step boundary.  With the previous
// corrector's pass pending, that pass runs first and this check's du_sum update
// follows it (k_rebuild_second); otherwise the second pass's flag is rebuild_b.
__device__ void begin_step_scalar(Ctl* ctl, const StepConst& sc, double dt) {
  ctl->time = __dadd_rn(ctl->time, dt);
  ctl->time_step += 1;
  double pr = sc.pressure_default;
  if (sc.pfun_len > 0)
    pr = eval_program(sc.pfun, sc.pfun_len, ctl->time, 0.0);
  else if (sc.pressure_table && ctl->table_len > 0)
    pr = sc.pressure_table[ctl->table_pos < ctl->table_len ? ctl->table_pos : ctl->table_len - 1];
  ctl->table_pos += 1;
  if (sc.compat_zero_pressure) pr = pr * 0.0;
  ctl->pressure = pr;
  if (sc.cavity_contact)
    for (int c = 0; c < 3; ++c)
      ctl->cav_R[c] = sc.rfun_len[c] > 0 ? eval_program(sc.rfun[c], sc.rfun_len[c], ctl->time, 0.0) : sc.cav_R[c];
  {
    const double red = fmax(1.0 - (double)((int)(ctl->time * 5.0)) * 0.01, 0.5);
    if (ctl->time_step == 2) ctl->volume0 = ctl->volume;
    ctl->volume_pressure = (sc.bulk_modulus == 0.0) ? 0.0 : sc.bulk_modulus * (ctl->volume0 * red / ctl->volume - 1.0);
  }
}

__device__ void begin_step(Ctl* ctl, const StepConst& sc, double dt, double mm, const RebuildCond& rc,
                           bool fused = false) {
  begin_step_scalar(ctl, sc, dt);
  // check_increment(false)
  const double du_max = sqrt(mm);
  const bool finite = isfinite(du_max);
  if (finite) {
    if (sc.contact && du_max > 0.5 * sc.thickness) register_problem(ctl, SHL_LARGE_DISP);
  } else {
    register_problem(ctl, SHL_NOT_FINITE);
  }
  if (fused && ctl->rebuild_pending) {
    ctl->rebuild = 1u;
    if (rc.has) cudaGraphSetConditional(rc.h, ctl->halted == 0 ? 1u : 0u);
    return;
  }
  if (finite) ctl->du_sum = __dadd_rn(ctl->du_sum, __dmul_rn(2.0, du_max));
  const uint32_t flag = (sc.contact && ctl->du_sum >= rebuild_tolerance(sc, ctl)) ? 1u : 0u;
  if (fused) {
    ctl->rebuild = 0u;
    ctl->rebuild_b = flag;
    if (rc.has) cudaGraphSetConditional(rc.h, (flag != 0 && ctl->halted == 0) ? 1u : 0u);
    return;
  }
  ctl->rebuild = flag;
  set_rebuild_cond(rc, ctl);
}

// between the two passes of a fused step's IF node (one thread): the deferred
// du_sum update of check_increment(false) (after the first pass reset du_sum
// and the element size), then the second pass's flag
__global__ void k_rebuild_second(DevBuf b, StepConst sc) {
  Ctl* ctl = b.ctl;
  if (blockIdx.x != 0 || ctl->halted != 0) return;
  if (sc.n_cs) {  // per shell of a batch
    int r = 0;
    for (uint32_t s = threadIdx.x; s < sc.n_cs; s += blockDim.x) {
      ShellCell& S = b.shc[s];
      if (S.rebuild_pending) {
        S.rebuild_pending = 0u;
        const double du_max = sqrt(S.du2_pred);
        if (isfinite(du_max)) S.du_sum = __dadd_rn(S.du_sum, __dmul_rn(2.0, du_max));
        S.rebuild_b = S.du_sum >= shell_tolerance(sc, S) ? 1u : 0u;
      }
      S.rebuild = S.rebuild_b;
      S.rebuild_b = 0u;
      r |= (int)S.rebuild;
    }
    r = __syncthreads_or(r);
    if (threadIdx.x == 0) {
      ctl->rebuild_pending = 0u;
      ctl->rebuild = r ? 1u : 0u;
      ctl->rebuild_b = 0u;
    }
    return;
  }
  if (threadIdx.x != 0) return;
  if (ctl->rebuild_pending) {
    ctl->rebuild_pending = 0u;
    const double du_max = sqrt(ctl->du2_pred);
    if (isfinite(du_max)) ctl->du_sum = __dadd_rn(ctl->du_sum, __dmul_rn(2.0, du_max));
    ctl->rebuild_b = (sc.contact && ctl->du_sum >= rebuild_tolerance(sc, ctl)) ? 1u : 0u;
  }
  ctl->rebuild = ctl->rebuild_b;
  ctl->rebuild_b = 0u;
}

// a deferred corrector pass made due for a direct launch_rebuild
__global__ void k_rebuild_first(DevBuf b, StepConst sc) {
  Ctl* ctl = b.ctl;
  if (blockIdx.x != 0) return;
  if (sc.n_cs) {
    int r = 0;
    for (uint32_t s = threadIdx.x; s < sc.n_cs; s += blockDim.x) {
      ShellCell& S = b.shc[s];
      S.rebuild = S.rebuild_pending;
      S.rebuild_pending = 0u;
      r |= (int)S.rebuild;
    }
    r = __syncthreads_or(r);
    if (threadIdx.x == 0) {
      ctl->rebuild = r ? 1u : 0u;
      ctl->rebuild_pending = 0u;
    }
    return;
  }
  if (threadIdx.x != 0) return;
  ctl->rebuild = ctl->rebuild_pending;
  ctl->rebuild_pending = 0u;
}

// rebuild flags of a pass started by the host (batch with self-contact):
// mode 0 every shell, 1 the shells whose du_sum reached their tolerance, 2 none
__global__ void k_batch_flags(DevBuf b, StepConst sc, int mode) {
  Ctl* ctl = b.ctl;
  int r = 0;
  for (uint32_t s = threadIdx.x; s < sc.n_cs; s += blockDim.x) {
    ShellCell& S = b.shc[s];
    S.rebuild = mode == 0 ? 1u : (mode == 1 && S.du_sum >= shell_tolerance(sc, S)) ? 1u : 0u;
    r |= (int)S.rebuild;
  }
  r = __syncthreads_or(r);
  if (threadIdx.x == 0) ctl->rebuild = r ? 1u : 0u;
}

// u_pred, v_pred, positions and du_max of every node, then the step's scalar
// start.  nodes_only: the predicted state alone, its largest |du|^2 left in
// ctl->du2_pred for k_begin_step (the start of a run of fused steps).
__global__ void __launch_bounds__(kBlock) k_predict(DevBuf b, StepConst sc, RebuildCond rc, int nodes_only) {
  Ctl* ctl = b.ctl;
  if (inactive(ctl)) {
    if (blockIdx.x == 0 && threadIdx.x == 0) set_rebuild_cond(rc, ctl);
    return;
  }
  __shared__ double sh[kBlock / 32];
  const uint32_t n = blockIdx.x * blockDim.x + threadIdx.x;
  const double dt = sc.adapt_every ? ctl->dt_cur : sc.dt;
  const double nm8 = sc.adapt_every ? ctl->nm[8] : sc.nm8, nm6 = sc.adapt_every ? ctl->nm[6] : sc.nm6;
  double du2 = 0.0;
  if (n < sc.V) {
    const size_t k3 = 3 * (size_t)n;
    const double u[3] = {b.u[k3], b.u[k3 + 1], b.u[k3 + 2]};
    const double v[3] = {b.v[k3], b.v[k3 + 1], b.v[k3 + 2]};
    const double a[3] = {b.a[k3], b.a[k3 + 1], b.a[k3 + 2]};
    du2 = predict_node(b, sc, n, u, v, a, dt, nm8, nm6, b.p);
  }
  if (sc.n_cs) shell_max_acc(b, sc, n, du2, 0);
  const double m = block_max(du2, sh);
  if (threadIdx.x == 0) b.partial[(size_t)blockIdx.x * 8] = m;
  if (!last_block(&ctl->cnt[0])) return;
  double mm = 0.0;
  for (int k = threadIdx.x; k < (int)gridDim.x; k += blockDim.x) mm = fmax(mm, __ldcg(&b.partial[(size_t)k * 8]));
  mm = block_max(mm, sh);
  if (sc.n_cs) {  // a batch: each shell's own check
    if (nodes_only) {
      for (uint32_t s = threadIdx.x; s < sc.n_cs; s += blockDim.x) b.shc[s].du2_pred = shell_take_max(&b.shc[s].du2_acc);
      return;
    }
    if (threadIdx.x == 0) begin_step_scalar(ctl, sc, dt);
    __syncthreads();
    batch_begin_check(b, sc, rc, false, true);
    return;
  }
  if (threadIdx.x != 0) return;
  if (nodes_only) {
    ctl->du2_pred = mm;
    return;
  }
  begin_step(ctl, sc, dt, mm, rc);
}

// the scalar start of a fused step: the nodes were predicted by the previous
// step's corrector (k_gather_correct mode 3) or by k_predict(nodes_only)
__global__ void k_begin_step(DevBuf b, StepConst sc, RebuildCond rc) {
  Ctl* ctl = b.ctl;
  if (blockIdx.x != 0) return;
  if (sc.n_cs) {  // a batch: each shell's own check (all threads of the block)
    if (inactive(ctl)) {
      if (threadIdx.x == 0) set_rebuild_cond(rc, ctl);
      return;
    }
    if (threadIdx.x == 0) begin_step_scalar(ctl, sc, sc.dt);
    __syncthreads();
    batch_begin_check(b, sc, rc, true, false);
    return;
  }
  if (threadIdx.x != 0) return;
  if (inactive(ctl)) {
    set_rebuild_cond(rc, ctl);
    return;
  }
  begin_step(ctl, sc, sc.dt, ctl->du2_pred, rc, true);
}

// positions p = X + u_pred of node n and the packed copies of u_pred that the
// element kernels read (float pairs; FP32 for the FP32 path)
__device__ __forceinline__ void set_positions(const DevBuf& b, const StepConst& sc, uint32_t n, const double* up) {
  float uh[3], ul[3];
  for (int c = 0; c < 3; ++c) {
    const size_t k = 3 * (size_t)n + c;
    b.p[k] = __dadd_rn(b.X[k], up[c]);
    df_split(up[c], uh[c], ul[c]);
  }
  if (sc.fp32) b.up32[n] = make_float4((float)up[0], (float)up[1], (float)up[2], 0.f);
  b.upk[2 * (size_t)n] = make_float4(uh[0], uh[1], uh[2], 0.f);
  b.upk[2 * (size_t)n + 1] = make_float4(ul[0], ul[1], ul[2], 0.f);
}

// The state from (hu, hv, ha) or to them: host memory that the device reads and
// writes directly (page-locked, mapped), one kernel instead of three copies each
// way.  Loading (one thread per node) also sets u_pred = u and the positions.
__global__ void k_state_host(DevBuf b, StepConst sc, double* hu, double* hv, double* ha, int load) {
  if (load) {
    const uint32_t n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= sc.V) return;
    double u[3];
    for (int c = 0; c < 3; ++c) {
      const size_t k = 3 * (size_t)n + c;
      u[c] = hu[k];
      b.u[k] = u[c];
      b.up[k] = u[c];
      b.v[k] = hv[k];
      b.a[k] = ha[k];
    }
    set_positions(b, sc, n, u);
    return;
  }
  const size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (k >= 3 * (size_t)sc.V) return;
  hu[k] = b.u[k];
  hv[k] = b.v[k];
  ha[k] = b.a[k];
}

// positions only (p = X + u_pred), for force evaluations at a given state
__global__ void k_positions(DevBuf b, StepConst sc) {
  const uint32_t n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= sc.V) return;
  const double up[3] = {b.up[3 * (size_t)n], b.up[3 * (size_t)n + 1], b.up[3 * (size_t)n + 2]};
  set_positions(b, sc, n, up);
}

// ------------------------------------------------------------- elements --
struct ElemOut {
  double etens, ebend, kg, km, area;
};

__device__ __forceinline__ void cross3(const double* a, const double* b, double* r) {
  r[0] = a[1] * b[2] - a[2] * b[1];
  r[1] = a[2] * b[0] - a[0] * b[2];
  r[2] = a[0] * b[1] - a[1] * b[0];
}
__device__ __forceinline__ double dot3(const double* a, const double* b) {
  return a[0] * b[0] + a[1] * b[1] + a[2] * b[2];
}

// One face: deformed metric, stress resultants, and the per-slot force
// share qe_s = sum_k B[s][k] Z_k (internal minus pressure), see the comments.
template <int NP, bool DFG = false, bool DFQ = false>
__device__ __forceinline__ ElemOut element_force(uint32_t i, int np_rt, uint32_t slot0, const double* __restrict__ B,
                                                 const DevBuf& b, const StepConst& sc, double pressure,
                                                 double vol_p) {
  const uint32_t F = sc.F;
  const int np = NP > 0 ? NP : np_rt;
  // G[k] = sum_s B[s][k] u_s  (unrotated value and derivatives of u at the qp)
  double G[6][3];
  if (DFG) {
    // B as float pairs in shared memory right after the FP64 table (Bh, then Bl)
    const float* Bh = reinterpret_cast<const float*>(B + kMaxSlots * 6);
    const float* Bl = Bh + kMaxSlots * 6;
    float gh[6][3], gl[6][3];
#pragma unroll
    for (int k = 0; k < 6; ++k)
#pragma unroll
      for (int c = 0; c < 3; ++c) gh[k][c] = gl[k][c] = 0.f;
#pragma unroll
    for (int s = 0; s < (NP > 0 ? NP : kMaxSlots); ++s) {
      if (NP == 0 && s >= np) break;
      const int nd = __ldg(&b.patch[(size_t)s * F + i]);
      const float4 h4 = __ldg(&b.upk[2 * (size_t)nd]), l4 = __ldg(&b.upk[2 * (size_t)nd + 1]);
      const float uh[3] = {h4.x, h4.y, h4.z}, ul[3] = {l4.x, l4.y, l4.z};
#pragma unroll
      for (int k = 0; k < 6; ++k) {
        const float wh = Bh[6 * s + k], wl = Bl[6 * s + k];
#pragma unroll
        for (int c = 0; c < 3; ++c) df_madd(gh[k][c], gl[k][c], wh, wl, uh[c], ul[c]);
      }
    }
#pragma unroll
    for (int k = 0; k < 6; ++k)
#pragma unroll
      for (int c = 0; c < 3; ++c) G[k][c] = df_value(gh[k][c], gl[k][c]);
  } else {
#pragma unroll
    for (int k = 0; k < 6; ++k) G[k][0] = G[k][1] = G[k][2] = 0.0;
#pragma unroll
    for (int s = 0; s < (NP > 0 ? NP : kMaxSlots); ++s) {
      if (NP == 0 && s >= np) break;
      const int nd = __ldg(&b.patch[(size_t)s * F + i]);
      const double ux = __ldg(&b.up[3 * (size_t)nd]);
      const double uy = __ldg(&b.up[3 * (size_t)nd + 1]);
      const double uz = __ldg(&b.up[3 * (size_t)nd + 2]);
#pragma unroll
      for (int k = 0; k < 6; ++k) {
        const double w = B[6 * s + k];
        G[k][0] = fma(w, ux, G[k][0]);
        G[k][1] = fma(w, uy, G[k][1]);
        G[k][2] = fma(w, uz, G[k][2]);
      }
    }
  }
  const double* fc = b.face;
#define FC(fld) __ldg(&fc[(size_t)(fld) * F + i])
  const double R00 = FC(FF_R00), R01 = FC(FF_R01), R10 = FC(FF_R10), R11 = FC(FF_R11);
  const double JxW = FC(FF_JXW);
  // rotation of derivatives onto the material frame (reinit_mod)
  const double c11a = R00 * R00, c11b = R10 * R10, c11c = 2.0 * R00 * R10;
  const double c22a = R01 * R01, c22b = R11 * R11, c22c = 2.0 * R01 * R11;
  const double c12a = R00 * R01, c12b = R10 * R11, c12c = R01 * R10 + R00 * R11;
  double a1[3], a2[3], v1[3], v2[3], v3[3], xq[3];
  {
    const double A1[3] = {FC(FF_A10), FC(FF_A11), FC(FF_A12)};
    const double A2[3] = {FC(FF_A20), FC(FF_A21), FC(FF_A22)};
    const double D1[3] = {FC(FF_D10), FC(FF_D11), FC(FF_D12)};
    const double D2[3] = {FC(FF_D20), FC(FF_D21), FC(FF_D22)};
    const double D3[3] = {FC(FF_D30), FC(FF_D31), FC(FF_D32)};
    const double X0[3] = {FC(FF_X0), FC(FF_X1), FC(FF_X2)};
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      a1[c] = A1[c] + (R00 * G[1][c] + R10 * G[2][c]);
      a2[c] = A2[c] + (R01 * G[1][c] + R11 * G[2][c]);
      v1[c] = D1[c] + (c11a * G[3][c] + c11b * G[4][c] + c11c * G[5][c]);
      v2[c] = D2[c] + (c22a * G[3][c] + c22b * G[4][c] + c22c * G[5][c]);
      v3[c] = D3[c] + (c12a * G[3][c] + c12b * G[4][c] + c12c * G[5][c]);
      xq[c] = X0[c] + G[0][c];
    }
  }
  double a3[3];
  cross3(a1, a2, a3);
  const double jac = sqrt(dot3(a3, a3));
  const double invjac = 1.0 / jac;
  a3[0] *= invjac; a3[1] *= invjac; a3[2] *= invjac;
  const double g0 = dot3(a1, a1), g1 = dot3(a2, a2), g2 = dot3(a1, a2);
  const double h0 = dot3(v1, a3), h1 = dot3(v2, a3), h2 = dot3(v3, a3);
  // strains (Voigt, shear doubled), ShellSystem.C:1190-1194
  const double al0 = 0.5 * (g0 - FC(FF_G0)), al1 = 0.5 * (g1 - FC(FF_G1)), al2 = g2 - FC(FF_G2);
  const double be0 = FC(FF_B0) - h0, be1 = FC(FF_B1) - h1, be2 = 2.0 * (FC(FF_B2) - h2);
  const double H00 = FC(FF_H00), H01 = FC(FF_H01), H02 = FC(FF_H02), H11 = FC(FF_H11), H12 = FC(FF_H12),
               H22 = FC(FF_H22);
  const double Kf = FC(FF_K) * sc.internal_scale, Df = FC(FF_D) * sc.internal_scale;
#undef FC
  const double n0 = Kf * (H00 * al0 + H01 * al1 + H02 * al2);
  const double n1 = Kf * (H01 * al0 + H11 * al1 + H12 * al2);
  const double n2 = Kf * (H02 * al0 + H12 * al1 + H22 * al2);
  const double m0 = Df * (H00 * be0 + H01 * be1 + H02 * be2);
  const double m1 = Df * (H01 * be0 + H11 * be1 + H12 * be2);
  const double m2 = Df * (H02 * be0 + H12 * be1 + H22 * be2);
  // sum_k m_k p_1k and sum_k m_k p_2k of eq. (A6) (ShellSystem.C:1223-1233)
  double M[3], a2xa3[3], a3xa1[3], Mxa2[3], a1xM[3];
#pragma unroll
  for (int c = 0; c < 3; ++c) M[c] = m0 * v1[c] + m1 * v2[c] + 2.0 * m2 * v3[c];
  const double sm = m0 * h0 + m1 * h1 + 2.0 * m2 * h2;
  cross3(a2, a3, a2xa3);
  cross3(a3, a1, a3xa1);
  cross3(M, a2, Mxa2);
  cross3(a1, M, a1xM);
  // pressure vector (ShellSystem.C:1509-1568)
  double pv[3] = {0.0, 0.0, 0.0};
  if (pressure != 0.0) {
    switch (sc.pressure_base) {
      case SHL_CS_LOCAL: pv[0] = a3[0]; pv[1] = a3[1]; pv[2] = a3[2]; break;
      case SHL_CS_CARTESIAN: pv[sc.pressure_dir] = 1.0; break;
      case SHL_CS_CYLINDRICAL:
        if (sc.pressure_dir == 0) {
          pv[0] = 1.0;
        } else {
          const double inv_r = 1.0 / sqrt(xq[1] * xq[1] + xq[2] * xq[2]);
          if (isfinite(inv_r)) { pv[1] = inv_r * xq[1]; pv[2] = inv_r * xq[2]; }
        }
        break;
      case SHL_CS_SPHERICAL: {
        const double r = sqrt(dot3(xq, xq));
        if (r > 0) { const double ir = 1.0 / r; pv[0] = xq[0] * ir; pv[1] = xq[1] * ir; pv[2] = xq[2] * ir; }
        break;
      }
      default: break;
    }
    pv[0] *= pressure; pv[1] *= pressure; pv[2] *= pressure;
  }
  if (vol_p != 0.0) {
    pv[0] += a3[0] * vol_p; pv[1] += a3[1] * vol_p; pv[2] += a3[2] * vol_p;
  }
  // Y: the qp vectors multiplying phi, phi_1, phi_2, phi_11, phi_22, phi_12;
  // Z = the same in the unrotated derivatives
  double Z[6][3];
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    const double Y1 = JxW * (n0 * a1[c] + n2 * a2[c] + invjac * (Mxa2[c] + sm * a2xa3[c]));
    const double Y2 = JxW * (n1 * a2[c] + n2 * a1[c] + invjac * (a1xM[c] + sm * a3xa1[c]));
    const double Y11 = -JxW * m0 * a3[c];
    const double Y22 = -JxW * m1 * a3[c];
    const double Y12 = -2.0 * JxW * m2 * a3[c];
    Z[0][c] = -JxW * pv[c];
    Z[1][c] = R00 * Y1 + R01 * Y2;
    Z[2][c] = R10 * Y1 + R11 * Y2;
    Z[3][c] = c11a * Y11 + c22a * Y22 + c12a * Y12;
    Z[4][c] = c11b * Y11 + c22b * Y22 + c12b * Y12;
    Z[5][c] = c11c * Y11 + c22c * Y22 + c12c * Y12;
  }
  // the measurements first: their inputs are then dead during the share contraction
  ElemOut o;
  o.etens = 0.5 * JxW * (n0 * al0 + n1 * al1 + n2 * al2);
  o.ebend = 0.5 * JxW * (m0 * be0 + m1 * be1 + m2 * be2);
  o.area = sc.qw * jac;
  {
    const double invdet = 1.0 / (g0 * g1 - g2 * g2);
    o.kg = o.area * invdet * (h0 * h1 - h2 * h2);
    o.km = o.area * invdet * 0.5 * (h0 * g1 + h1 * g0 - 2.0 * h2 * g2);
  }
  // shares go to their places in gather order (scattered writes, contiguous reads in the gather)
  const uint32_t* spos = b.slot_pos + slot0;
  if (DFQ) {
    const float* Bh = reinterpret_cast<const float*>(B + kMaxSlots * 6);
    const float* Bl = Bh + kMaxSlots * 6;
    float zh[6][3], zl[6][3];
#pragma unroll
    for (int k = 0; k < 6; ++k)
#pragma unroll
      for (int c = 0; c < 3; ++c) df_split(Z[k][c], zh[k][c], zl[k][c]);
#pragma unroll
    for (int s = 0; s < (NP > 0 ? NP : kMaxSlots); ++s) {
      if (NP == 0 && s >= np) break;
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        float th = 0.f, tl = 0.f;
#pragma unroll
        for (int k = 0; k < 6; ++k) df_madd(th, tl, Bh[6 * s + k], Bl[6 * s + k], zh[k][c], zl[k][c]);
        b.qe[3 * (size_t)__ldg(&spos[s]) + c] = df_value(th, tl);
      }
    }
  } else {
#pragma unroll
    for (int s = 0; s < (NP > 0 ? NP : kMaxSlots); ++s) {
      if (NP == 0 && s >= np) break;
      double q[3];
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        double t = B[6 * s] * Z[0][c];
#pragma unroll
        for (int k = 1; k < 6; ++k) t = fma(B[6 * s + k], Z[k][c], t);
        q[c] = t;
      }
      double* qe = b.qe + 3 * (size_t)__ldg(&spos[s]);
      qe[0] = q[0];
      qe[1] = q[1];
      qe[2] = q[2];
    }
  }
  return o;
}

// FP32 element force in relative-displacement form.  Same mechanics as
// element_force, but the strains are built from the displacement derivatives
// and the reference geometry without subtracting nearly equal metrics:
//   alpha_11 = A1.du1 + |du1|^2/2, alpha_22 = A2.du2 + |du2|^2/2,
//   alpha_12 = A1.du2 + du1.A2 + du1.du2 (Voigt, shear doubled)
//   beta_k   = -(D_k.(n - N) + d_k.n), with n - N formed from the change
//              of a1 x a2 (no cancellation), shear doubled.
// The per-slot shares are written in FP32.
template <int NP>
__device__ __forceinline__ ElemOut element_force32(uint32_t i, int np_rt, uint32_t slot0, const float* __restrict__ B,
                                                   const DevBuf& b, const StepConst& sc, float pressure,
                                                   float vol_p) {
  const uint32_t F = sc.F;
  const int np = NP > 0 ? NP : np_rt;
  float G[6][3];
#pragma unroll
  for (int k = 0; k < 6; ++k) G[k][0] = G[k][1] = G[k][2] = 0.f;
#pragma unroll
  for (int s = 0; s < (NP > 0 ? NP : kMaxSlots); ++s) {
    if (NP == 0 && s >= np) break;
    const int nd = __ldg(&b.patch[(size_t)s * F + i]);
    const float4 un = __ldg(&b.up32[nd]);
    const float ux = un.x, uy = un.y, uz = un.z;
#pragma unroll
    for (int k = 0; k < 6; ++k) {
      const float w = B[6 * s + k];
      G[k][0] = fmaf(w, ux, G[k][0]);
      G[k][1] = fmaf(w, uy, G[k][1]);
      G[k][2] = fmaf(w, uz, G[k][2]);
    }
  }
  const float* fc = b.face32;
#define FC(fld) __ldg(&fc[(size_t)(fld) * F + i])
  const float R00 = FC(F32_R00), R01 = FC(F32_R01), R10 = FC(F32_R10), R11 = FC(F32_R11);
  const float JxW = FC(F32_JXW);
  const float c11a = R00 * R00, c11b = R10 * R10, c11c = 2.f * R00 * R10;
  const float c22a = R01 * R01, c22b = R11 * R11, c22c = 2.f * R01 * R11;
  const float c12a = R00 * R01, c12b = R10 * R11, c12c = R01 * R10 + R00 * R11;
  float A1[3] = {FC(F32_A10), FC(F32_A11), FC(F32_A12)};
  float A2[3] = {FC(F32_A20), FC(F32_A21), FC(F32_A22)};
  float du1[3], du2[3], d1[3], d2[3], d3[3], xq[3];
  {
    const float X0[3] = {FC(F32_X0), FC(F32_X1), FC(F32_X2)};
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      du1[c] = R00 * G[1][c] + R10 * G[2][c];
      du2[c] = R01 * G[1][c] + R11 * G[2][c];
      d1[c] = c11a * G[3][c] + c11b * G[4][c] + c11c * G[5][c];
      d2[c] = c22a * G[3][c] + c22b * G[4][c] + c22c * G[5][c];
      d3[c] = c12a * G[3][c] + c12b * G[4][c] + c12c * G[5][c];
      xq[c] = X0[c] + G[0][c];
    }
  }
  auto dotf = [](const float* x, const float* y) { return x[0] * y[0] + x[1] * y[1] + x[2] * y[2]; };
  auto crossf = [](const float* x, const float* y, float* r) {
    r[0] = x[1] * y[2] - x[2] * y[1];
    r[1] = x[2] * y[0] - x[0] * y[2];
    r[2] = x[0] * y[1] - x[1] * y[0];
  };
  // membrane strains
  const float al0 = dotf(A1, du1) + 0.5f * dotf(du1, du1);
  const float al1 = dotf(A2, du2) + 0.5f * dotf(du2, du2);
  const float al2 = dotf(A1, du2) + dotf(du1, A2) + dotf(du1, du2);
  // deformed normal from the change of a1 x a2
  float Dn[3], t1[3], t2[3], t3[3];
  crossf(A1, du2, t1);
  crossf(du1, A2, t2);
  crossf(du1, du2, t3);
  Dn[0] = t1[0] + t2[0] + t3[0];
  Dn[1] = t1[1] + t2[1] + t3[1];
  Dn[2] = t1[2] + t2[2] + t3[2];
  const float N0[3] = {FC(F32_N0), FC(F32_N1), FC(F32_N2)};
  const float L0 = FC(F32_L0);
  const float dL2 = 2.f * L0 * dotf(N0, Dn) + dotf(Dn, Dn);  // |a1 x a2|^2 - L0^2
  const float jac = sqrtf(L0 * L0 + dL2);
  const float invjac = 1.f / jac;
  const float s_n = -dL2 / ((L0 + jac) * jac);  // L0/jac - 1
  float a3[3], dn[3], a1[3], a2[3], v1[3], v2[3], v3[3];
  {
    const float D1[3] = {FC(F32_D10), FC(F32_D11), FC(F32_D12)};
    const float D2[3] = {FC(F32_D20), FC(F32_D21), FC(F32_D22)};
    const float D3[3] = {FC(F32_D30), FC(F32_D31), FC(F32_D32)};
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      dn[c] = Dn[c] * invjac + N0[c] * s_n;
      a3[c] = N0[c] + dn[c];
      a1[c] = A1[c] + du1[c];
      a2[c] = A2[c] + du2[c];
      v1[c] = D1[c] + d1[c];
      v2[c] = D2[c] + d2[c];
      v3[c] = D3[c] + d3[c];
    }
    // bending strains beta_k = -(D_k.dn + d_k.a3)
    const float be0 = -(dotf(D1, dn) + dotf(d1, a3));
    const float be1 = -(dotf(D2, dn) + dotf(d2, a3));
    const float be2 = -2.f * (dotf(D3, dn) + dotf(d3, a3));
    const float H00 = FC(F32_H00), H01 = FC(F32_H01), H02 = FC(F32_H02), H11 = FC(F32_H11), H12 = FC(F32_H12),
                H22 = FC(F32_H22);
    const float K = FC(F32_K) * (float)sc.internal_scale, Dm = FC(F32_D) * (float)sc.internal_scale;
    const float n0 = K * (H00 * al0 + H01 * al1 + H02 * al2);
    const float n1 = K * (H01 * al0 + H11 * al1 + H12 * al2);
    const float n2 = K * (H02 * al0 + H12 * al1 + H22 * al2);
    const float m0 = Dm * (H00 * be0 + H01 * be1 + H02 * be2);
    const float m1 = Dm * (H01 * be0 + H11 * be1 + H12 * be2);
    const float m2 = Dm * (H02 * be0 + H12 * be1 + H22 * be2);
    const float h0 = dotf(v1, a3), h1 = dotf(v2, a3), h2 = dotf(v3, a3);
    float M[3], a2xa3[3], a3xa1[3], Mxa2[3], a1xM[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) M[c] = m0 * v1[c] + m1 * v2[c] + 2.f * m2 * v3[c];
    const float sm = m0 * h0 + m1 * h1 + 2.f * m2 * h2;
    crossf(a2, a3, a2xa3);
    crossf(a3, a1, a3xa1);
    crossf(M, a2, Mxa2);
    crossf(a1, M, a1xM);
    float pv[3] = {0.f, 0.f, 0.f};
    if (pressure != 0.f) {
      switch (sc.pressure_base) {
        case SHL_CS_LOCAL: pv[0] = a3[0]; pv[1] = a3[1]; pv[2] = a3[2]; break;
        case SHL_CS_CARTESIAN: pv[sc.pressure_dir] = 1.f; break;
        case SHL_CS_CYLINDRICAL:
          if (sc.pressure_dir == 0) {
            pv[0] = 1.f;
          } else {
            const float inv_r = 1.f / sqrtf(xq[1] * xq[1] + xq[2] * xq[2]);
            if (isfinite(inv_r)) { pv[1] = inv_r * xq[1]; pv[2] = inv_r * xq[2]; }
          }
          break;
        case SHL_CS_SPHERICAL: {
          const float r = sqrtf(dotf(xq, xq));
          if (r > 0.f) { const float ir = 1.f / r; pv[0] = xq[0] * ir; pv[1] = xq[1] * ir; pv[2] = xq[2] * ir; }
          break;
        }
        default: break;
      }
      pv[0] *= pressure; pv[1] *= pressure; pv[2] *= pressure;
    }
    if (vol_p != 0.f) {
      pv[0] += a3[0] * vol_p; pv[1] += a3[1] * vol_p; pv[2] += a3[2] * vol_p;
    }
    float Z[6][3];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const float Y1 = JxW * (n0 * a1[c] + n2 * a2[c] + invjac * (Mxa2[c] + sm * a2xa3[c]));
      const float Y2 = JxW * (n1 * a2[c] + n2 * a1[c] + invjac * (a1xM[c] + sm * a3xa1[c]));
      const float Y11 = -JxW * m0 * a3[c];
      const float Y22 = -JxW * m1 * a3[c];
      const float Y12 = -2.f * JxW * m2 * a3[c];
      Z[0][c] = -JxW * pv[c];
      Z[1][c] = R00 * Y1 + R01 * Y2;
      Z[2][c] = R10 * Y1 + R11 * Y2;
      Z[3][c] = c11a * Y11 + c22a * Y22 + c12a * Y12;
      Z[4][c] = c11b * Y11 + c22b * Y22 + c12b * Y12;
      Z[5][c] = c11c * Y11 + c22c * Y22 + c12c * Y12;
    }
    const uint32_t* spos = b.slot_pos + slot0;
#pragma unroll
    for (int s = 0; s < (NP > 0 ? NP : kMaxSlots); ++s) {
      if (NP == 0 && s >= np) break;
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        float t = B[6 * s] * Z[0][c];
#pragma unroll
        for (int k = 1; k < 6; ++k) t = fmaf(B[6 * s + k], Z[k][c], t);
        b.qe32[3 * (size_t)__ldg(&spos[s]) + c] = t;
      }
    }
    ElemOut o;
    const float area = 0.5f * jac;
    const float g0 = FC(F32_G0) + 2.f * al0, g1 = FC(F32_G1) + 2.f * al1, g2 = FC(F32_G2) + al2;
    const float w_invdet = area / (g0 * g1 - g2 * g2);
    o.etens = 0.5f * JxW * (n0 * al0 + n1 * al1 + n2 * al2);
    o.ebend = 0.5f * JxW * (m0 * be0 + m1 * be1 + m2 * be2);
    o.area = area;
    o.kg = w_invdet * (h0 * h1 - h2 * h2);
    o.km = w_invdet * 0.5f * (h0 * g1 + h1 * g0 - 2.f * h2 * g2);
    return o;
  }
#undef FC
}

// Element kernels are compiled in several launch shapes (threads per block,
// blocks per SM, hence registers per thread) -- and for the FP64 path with the
// two basis contractions in FP64 or as float pairs; set-up times them on the
// context's own mesh and keeps the fastest (shl_api.cu, tune_elements).  The
// per-face arithmetic of one path does not depend on the launch shape.  The
// totals of the per-face measurements are summed by k_elem_totals.
// FP64-class element force in double-float arithmetic on the FP32 pipe: the
// relative-displacement formulation of element_force32 with every quantity a
// float pair (about 48 significant bits), the constants from face_df (the
// same balanced-frame values as face32, kept to 48 bits), the displacement
// derivatives from the hi/lo copy of u_pred.  No step subtracts nearly equal
// quantities, so the forces carry a relative error of a few 1e-14 -- the
// class of the FP64 path -- at FP32 instruction rates.  Shares are written as
// float pairs; the measurements are returned as FP64, E_tens, E_bend, kGauss
// and kMean already divided by the area.
template <int NP>
__device__ __forceinline__ ElemOut element_force_df(uint32_t i, int np_rt, uint32_t slot0,
                                                    const float* __restrict__ Bh, const float* __restrict__ Bl,
                                                    const DevBuf& b, const StepConst& sc, double pressure_d,
                                                    double vol_p_d, float4* __restrict__ su) {
  const uint32_t F = sc.F;
  const int np = NP > 0 ? NP : np_rt;
  const uint32_t t = threadIdx.x, bs = blockDim.x;
  if (NP > 0) {
    // all patch ids, then all node displacements copied asynchronously into this
    // thread's shared-memory column ([2 s + hi/lo][thread], 16 B each): one
    // memory latency for the whole patch instead of one per slot of the loop below
    int nd[NP > 0 ? NP : 1];
#pragma unroll
    for (int s = 0; s < NP; ++s) nd[s] = __ldg(&b.patch[(size_t)s * F + i]);
#pragma unroll
    for (int s = 0; s < NP; ++s) {
      cp_async16(&su[(2 * s) * bs + t], &b.upk[2 * (size_t)nd[s]]);
      cp_async16(&su[(2 * s + 1) * bs + t], &b.upk[2 * (size_t)nd[s] + 1]);
    }
    cp_async_wait_all();
  }
  df2 G[6][3];
  {
    float gh[6][3], gl[6][3];
#pragma unroll
    for (int k = 0; k < 6; ++k)
#pragma unroll
      for (int c = 0; c < 3; ++c) gh[k][c] = gl[k][c] = 0.f;
    // slots in a rolled loop: the unrolled double-float code would not fit the instruction cache
#pragma unroll 1
    for (int s = 0; s < np; ++s) {
      float4 h4, l4;
      if (NP > 0) {
        h4 = su[(2 * s) * bs + t];
        l4 = su[(2 * s + 1) * bs + t];
      } else {
        const int nd = __ldg(&b.patch[(size_t)s * F + i]);
        h4 = __ldg(&b.upk[2 * (size_t)nd]);
        l4 = __ldg(&b.upk[2 * (size_t)nd + 1]);
      }
      const float uh[3] = {h4.x, h4.y, h4.z}, ul[3] = {l4.x, l4.y, l4.z};
#pragma unroll
      for (int k = 0; k < 6; ++k) {
        const float wh = Bh[6 * s + k], wl = Bl[6 * s + k];
#pragma unroll
        for (int c = 0; c < 3; ++c) df_madd(gh[k][c], gl[k][c], wh, wl, uh[c], ul[c]);
      }
    }
#pragma unroll
    for (int k = 0; k < 6; ++k)
#pragma unroll
      for (int c = 0; c < 3; ++c) df_quick_two_sum(gh[k][c], gl[k][c], G[k][c].h, G[k][c].l);
  }
  const float* fd = b.face_df;
  // constant row r (hi rows 0..37, lo rows 38..75) in component r % 4 of this
  // thread's float4 entry r / 4 -- the entries that held its displacements
  static_assert(2 * F32_COUNT <= 4 * 2 * kDfStageSlots, "face constants exceed the staging column");
  float* sf = reinterpret_cast<float*>(su);
  auto srow = [&](int r) -> float* { return &sf[4 * ((r >> 2) * bs + t) + (r & 3)]; };
  if (NP > 0) {
    // the displacements are consumed: the same entries now take the face's
    // constants, all 76 rows in flight at once
#pragma unroll
    for (int r = 0; r < 2 * F32_COUNT; ++r) cp_async4(srow(r), &fd[(size_t)r * F + i]);
    cp_async_wait_all();
  }
  auto FC = [&](int fld) -> df2 {
    if (NP > 0) return {*srow(fld), *srow(F32_COUNT + fld)};
    return {__ldg(&fd[(size_t)fld * F + i]), __ldg(&fd[(size_t)(F32_COUNT + fld) * F + i])};
  };
  const df2 R00 = FC(F32_R00), R01 = FC(F32_R01), R10 = FC(F32_R10), R11 = FC(F32_R11);
  const df2 JxW = FC(F32_JXW);
  const df2 c11a = R00 * R00, c11b = R10 * R10, c11c = 2.f * (R00 * R10);
  const df2 c22a = R01 * R01, c22b = R11 * R11, c22c = 2.f * (R01 * R11);
  const df2 c12a = R00 * R01, c12b = R10 * R11, c12c = R01 * R10 + R00 * R11;
  df2 A1[3] = {FC(F32_A10), FC(F32_A11), FC(F32_A12)};
  df2 A2[3] = {FC(F32_A20), FC(F32_A21), FC(F32_A22)};
  df2 du1[3], du2[3], d1[3], d2[3], d3[3], xq[3];
  {
    const df2 X0[3] = {FC(F32_X0), FC(F32_X1), FC(F32_X2)};
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      du1[c] = R00 * G[1][c] + R10 * G[2][c];
      du2[c] = R01 * G[1][c] + R11 * G[2][c];
      d1[c] = c11a * G[3][c] + c11b * G[4][c] + c11c * G[5][c];
      d2[c] = c22a * G[3][c] + c22b * G[4][c] + c22c * G[5][c];
      d3[c] = c12a * G[3][c] + c12b * G[4][c] + c12c * G[5][c];
      xq[c] = X0[c] + G[0][c];
    }
  }
  // membrane strains (Voigt, shear doubled), without metric differences
  const df2 al0 = dot3df(A1, du1) + 0.5f * dot3df(du1, du1);
  const df2 al1 = dot3df(A2, du2) + 0.5f * dot3df(du2, du2);
  const df2 al2 = dot3df(A1, du2) + dot3df(du1, A2) + dot3df(du1, du2);
  // deformed normal from the change of a1 x a2
  df2 Dn[3], t1[3], t2[3], t3[3];
  cross3df(A1, du2, t1);
  cross3df(du1, A2, t2);
  cross3df(du1, du2, t3);
#pragma unroll
  for (int c = 0; c < 3; ++c) Dn[c] = t1[c] + t2[c] + t3[c];
  const df2 N0[3] = {FC(F32_N0), FC(F32_N1), FC(F32_N2)};
  const df2 L0 = FC(F32_L0);
  const df2 dL2 = 2.f * (L0 * dot3df(N0, Dn)) + dot3df(Dn, Dn);  // |a1 x a2|^2 - L0^2
  const df2 jac = df_sqrt(L0 * L0 + dL2);
  const df2 invjac = df_recip(jac);
  const df2 s_n = -(dL2 * df_recip((L0 + jac) * jac));  // L0/jac - 1
  df2 a3[3], dn[3], a1[3], a2[3], v1[3], v2[3], v3[3];
  const df2 D1[3] = {FC(F32_D10), FC(F32_D11), FC(F32_D12)};
  const df2 D2[3] = {FC(F32_D20), FC(F32_D21), FC(F32_D22)};
  const df2 D3[3] = {FC(F32_D30), FC(F32_D31), FC(F32_D32)};
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    dn[c] = Dn[c] * invjac + N0[c] * s_n;
    a3[c] = N0[c] + dn[c];
    a1[c] = A1[c] + du1[c];
    a2[c] = A2[c] + du2[c];
    v1[c] = D1[c] + d1[c];
    v2[c] = D2[c] + d2[c];
    v3[c] = D3[c] + d3[c];
  }
  // bending strains beta_k = -(D_k.dn + d_k.a3), shear doubled
  const df2 be0 = -(dot3df(D1, dn) + dot3df(d1, a3));
  const df2 be1 = -(dot3df(D2, dn) + dot3df(d2, a3));
  const df2 be2 = -2.f * (dot3df(D3, dn) + dot3df(d3, a3));
  const df2 H00 = FC(F32_H00), H01 = FC(F32_H01), H02 = FC(F32_H02), H11 = FC(F32_H11), H12 = FC(F32_H12),
            H22 = FC(F32_H22);
  const float scale = (float)sc.internal_scale;  // 1, or 0 for the pressure-only force
  const df2 K = scale * FC(F32_K), Dm = scale * FC(F32_D);
  const df2 n0 = K * (H00 * al0 + H01 * al1 + H02 * al2);
  const df2 n1 = K * (H01 * al0 + H11 * al1 + H12 * al2);
  const df2 n2 = K * (H02 * al0 + H12 * al1 + H22 * al2);
  const df2 m0 = Dm * (H00 * be0 + H01 * be1 + H02 * be2);
  const df2 m1 = Dm * (H01 * be0 + H11 * be1 + H12 * be2);
  const df2 m2 = Dm * (H02 * be0 + H12 * be1 + H22 * be2);
  const df2 h0 = dot3df(v1, a3), h1 = dot3df(v2, a3), h2 = dot3df(v3, a3);
  df2 M[3], a2xa3[3], a3xa1[3], Mxa2[3], a1xM[3];
#pragma unroll
  for (int c = 0; c < 3; ++c) M[c] = m0 * v1[c] + m1 * v2[c] + 2.f * (m2 * v3[c]);
  const df2 sm = m0 * h0 + m1 * h1 + 2.f * (m2 * h2);
  cross3df(a2, a3, a2xa3);
  cross3df(a3, a1, a3xa1);
  cross3df(M, a2, Mxa2);
  cross3df(a1, M, a1xM);
  df2 pv[3] = {dfv(0.f), dfv(0.f), dfv(0.f)};
  if (pressure_d != 0.0) {
    const df2 pressure = df_from_double(pressure_d);
    switch (sc.pressure_base) {
      case SHL_CS_LOCAL: pv[0] = a3[0]; pv[1] = a3[1]; pv[2] = a3[2]; break;
      case SHL_CS_CARTESIAN: pv[sc.pressure_dir] = dfv(1.f); break;
      case SHL_CS_CYLINDRICAL:
        if (sc.pressure_dir == 0) {
          pv[0] = dfv(1.f);
        } else {
          const df2 r2 = xq[1] * xq[1] + xq[2] * xq[2];
          if (r2.h > 0.f) {
            const df2 inv_r = df_recip(df_sqrt(r2));
            pv[1] = inv_r * xq[1];
            pv[2] = inv_r * xq[2];
          }
        }
        break;
      case SHL_CS_SPHERICAL: {
        const df2 r2 = dot3df(xq, xq);
        if (r2.h > 0.f) {
          const df2 ir = df_recip(df_sqrt(r2));
          pv[0] = xq[0] * ir; pv[1] = xq[1] * ir; pv[2] = xq[2] * ir;
        }
        break;
      }
      default: break;
    }
    pv[0] = pv[0] * pressure; pv[1] = pv[1] * pressure; pv[2] = pv[2] * pressure;
  }
  if (vol_p_d != 0.0) {
    const df2 vol_p = df_from_double(vol_p_d);
    pv[0] += a3[0] * vol_p; pv[1] += a3[1] * vol_p; pv[2] += a3[2] * vol_p;
  }
  df2 Z[6][3];
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    const df2 Y1 = JxW * (n0 * a1[c] + n2 * a2[c] + invjac * (Mxa2[c] + sm * a2xa3[c]));
    const df2 Y2 = JxW * (n1 * a2[c] + n2 * a1[c] + invjac * (a1xM[c] + sm * a3xa1[c]));
    const df2 Y11 = -(JxW * m0 * a3[c]);
    const df2 Y22 = -(JxW * m1 * a3[c]);
    const df2 Y12 = -2.f * (JxW * m2 * a3[c]);
    Z[0][c] = -(JxW * pv[c]);
    Z[1][c] = R00 * Y1 + R01 * Y2;
    Z[2][c] = R10 * Y1 + R11 * Y2;
    Z[3][c] = c11a * Y11 + c22a * Y22 + c12a * Y12;
    Z[4][c] = c11b * Y11 + c22b * Y22 + c12b * Y12;
    Z[5][c] = c11c * Y11 + c22c * Y22 + c12c * Y12;
  }
  ElemOut o;
  {
    // per unit area, as stored (the area cancels from the curvatures): double-float
    // quotients instead of four FP64 divisions per face on GB300's narrow FP64 pipe
    const df2 area = 0.5f * jac;
    const df2 inv_area = df_recip(area);
    const df2 g0 = FC(F32_G0) + 2.f * al0, g1 = FC(F32_G1) + 2.f * al1, g2 = FC(F32_G2) + al2;
    const df2 invdet = df_recip(g0 * g1 - g2 * g2);
    o.etens = df_to_double((0.5f * (JxW * (n0 * al0 + n1 * al1 + n2 * al2))) * inv_area);
    o.ebend = df_to_double((0.5f * (JxW * (m0 * be0 + m1 * be1 + m2 * be2))) * inv_area);
    o.area = df_to_double(area);
    o.kg = df_to_double(invdet * (h0 * h1 - h2 * h2));
    o.km = df_to_double(invdet * (0.5f * (h0 * g1 + h1 * g0 - 2.f * (h2 * g2))));
  }
  const uint32_t* spos = b.slot_pos + slot0;
#pragma unroll 1
  for (int s = 0; s < np; ++s) {
    const df2 Bs[6] = {{Bh[6 * s], Bl[6 * s]},         {Bh[6 * s + 1], Bl[6 * s + 1]},
                       {Bh[6 * s + 2], Bl[6 * s + 2]}, {Bh[6 * s + 3], Bl[6 * s + 3]},
                       {Bh[6 * s + 4], Bl[6 * s + 4]}, {Bh[6 * s + 5], Bl[6 * s + 5]}};
    // the share stays a float pair in its 8 bytes; the gather adds the pairs and converts once per node
    float2* qe = reinterpret_cast<float2*>(b.qe) + 3 * (size_t)__ldg(&spos[s]);
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      df2 t = Bs[0] * Z[0][c];
#pragma unroll
      for (int k = 1; k < 6; ++k) t += Bs[k] * Z[k][c];
      qe[c] = make_float2(t.h, t.l);
    }
  }
  return o;
}

// the element kernel of the double-float path (block shapes as k_elements)
template <int BS, int MINB>
__global__ void __launch_bounds__(BS, MINB) k_elements_df(DevBuf b, StepConst sc, ElemGroups eg) {
  Ctl* ctl = b.ctl;
  if (inactive(ctl)) return;
  __shared__ double sB[kMaxSlots * 6 * 2];
  extern __shared__ float4 su[];  // kDfStageSlots x 2 x BS: the patch displacements of the block's faces
  int g = 0;
  while (g + 1 < eg.n && blockIdx.x >= eg.g[g + 1].block_start) ++g;
  const GroupDesc gd = eg.g[g];
  float* sBh = reinterpret_cast<float*>(sB + kMaxSlots * 6);
  float* sBl = sBh + kMaxSlots * 6;
  for (int k = threadIdx.x; k < gd.n_slots * 6; k += blockDim.x) {
    const double w = eg.basis[gd.basis_off + k];
    sB[k] = w;
    df_split(w, sBh[k], sBl[k]);
  }
  __syncthreads();
  const uint32_t li = (blockIdx.x - gd.block_start) * blockDim.x + threadIdx.x;
  if (li >= gd.count) return;
  const double pressure = ctl->pressure, vol_p = ctl->volume_pressure;
  const uint32_t i = gd.first + li;
  const uint32_t slot0 = gd.slot_base + li * (uint32_t)gd.n_slots;
  const double pr = pressure * __ldg(&b.pscale[i]);
  ElemOut o;
  if (gd.n_slots == 12)
    o = element_force_df<12>(i, 12, slot0, sBh, sBl, b, sc, pr, vol_p, su);
  else if (gd.n_slots == 11)
    o = element_force_df<11>(i, 11, slot0, sBh, sBl, b, sc, pr, vol_p, su);
  else
    o = element_force_df<0>(i, gd.n_slots, slot0, sBh, sBl, b, sc, pr, vol_p, su);
  const uint32_t e = __ldg(&b.perm[i]);
  b.area[e] = o.area;  // the other fields come per unit area
  b.kG[e] = o.kg;
  b.kM[e] = o.km;
  b.etens[e] = o.etens;
  b.ebend[e] = o.ebend;
}

// The double-float element kernel in one round of faces: thread t of block k
// takes face k * BS + t of the whole mesh (all patch groups), so with one
// 544-thread block per SM a level-6 shell (81,920 faces on 152 SMs) runs every
// face at once.  The shapes above run 1.4 rounds there, and since a face is a
// long dependent chain, the second, partly filled round costs as much as the
// first.  Each thread picks its patch group (groups are contiguous face
// ranges) and the basis tables of all groups sit in shared memory after the
// staging columns.  The per-face arithmetic is that of k_elements_df.
template <int BS>
__global__ void __launch_bounds__(BS, 1) k_elements_df_flat(DevBuf b, StepConst sc, ElemGroups eg) {
  Ctl* ctl = b.ctl;
  if (inactive(ctl)) return;
  extern __shared__ float4 su[];  // kDfStageSlots x 2 x BS staging, then per group the basis (hi, lo)
  float* sBall = reinterpret_cast<float*>(su + (size_t)kDfStageSlots * 2 * BS);
  for (int g = 0; g < eg.n; ++g) {
    float* h = sBall + g * (2 * kMaxSlots * 6);
    for (int k = threadIdx.x; k < eg.g[g].n_slots * 6; k += blockDim.x)
      df_split(eg.basis[eg.g[g].basis_off + k], h[k], h[kMaxSlots * 6 + k]);
  }
  __syncthreads();
  const uint32_t i = blockIdx.x * BS + threadIdx.x;
  if (i >= sc.F) return;
  int g = 0;
  while (g + 1 < eg.n && i >= eg.g[g + 1].first) ++g;
  const GroupDesc gd = eg.g[g];
  const float* Bh = sBall + g * (2 * kMaxSlots * 6);
  const float* Bl = Bh + kMaxSlots * 6;
  const double pressure = ctl->pressure, vol_p = ctl->volume_pressure;
  const uint32_t slot0 = gd.slot_base + (i - gd.first) * (uint32_t)gd.n_slots;
  const double pr = pressure * __ldg(&b.pscale[i]);
  ElemOut o;
  if (gd.n_slots == 12)
    o = element_force_df<12>(i, 12, slot0, Bh, Bl, b, sc, pr, vol_p, su);
  else if (gd.n_slots == 11)
    o = element_force_df<11>(i, 11, slot0, Bh, Bl, b, sc, pr, vol_p, su);
  else
    o = element_force_df<0>(i, gd.n_slots, slot0, Bh, Bl, b, sc, pr, vol_p, su);
  const uint32_t e = __ldg(&b.perm[i]);
  b.area[e] = o.area;
  b.kG[e] = o.kg;
  b.kM[e] = o.km;
  b.etens[e] = o.etens;
  b.ebend[e] = o.ebend;
}

template <int BS, int MINB>
__global__ void __launch_bounds__(BS, MINB) k_elements32(DevBuf b, StepConst sc, ElemGroups eg) {
  Ctl* ctl = b.ctl;
  if (inactive(ctl)) return;
  __shared__ float sB[kMaxSlots * 6];
  int g = 0;
  while (g + 1 < eg.n && blockIdx.x >= eg.g[g + 1].block_start) ++g;
  const GroupDesc gd = eg.g[g];
  for (int k = threadIdx.x; k < gd.n_slots * 6; k += blockDim.x) sB[k] = eg.basis32[gd.basis_off + k];
  __syncthreads();
  const uint32_t li = (blockIdx.x - gd.block_start) * blockDim.x + threadIdx.x;
  if (li >= gd.count) return;
  const double pressure = ctl->pressure;
  const float vol_p = (float)ctl->volume_pressure;
  const uint32_t i = gd.first + li;
  const uint32_t slot0 = gd.slot_base + li * (uint32_t)gd.n_slots;
  const float pr = (float)(pressure * __ldg(&b.pscale[i]));
  ElemOut o;
  if (gd.n_slots == 12)
    o = element_force32<12>(i, 12, slot0, sB, b, sc, pr, vol_p);
  else if (gd.n_slots == 11)
    o = element_force32<11>(i, 11, slot0, sB, b, sc, pr, vol_p);
  else
    o = element_force32<0>(i, gd.n_slots, slot0, sB, b, sc, pr, vol_p);
  const uint32_t e = __ldg(&b.perm[i]);
  const float ia = 1.f / (float)o.area;
  b.area[e] = o.area;
  b.kG[e] = (float)o.kg * ia;
  b.kM[e] = (float)o.km * ia;
  b.etens[e] = (float)o.etens * ia;
  b.ebend[e] = (float)o.ebend * ia;
}

template <int BS, int MINB, bool DFG, bool DFQ>
__global__ void __launch_bounds__(BS, MINB) k_elements(DevBuf b, StepConst sc, ElemGroups eg) {
  Ctl* ctl = b.ctl;
  if (inactive(ctl)) return;
  // FP64 basis table followed by its float pairs (hi, lo): kMaxSlots * 6 doubles + 2 x kMaxSlots * 6 floats
  __shared__ double sB[kMaxSlots * 6 * 2];
  int g = 0;
  while (g + 1 < eg.n && blockIdx.x >= eg.g[g + 1].block_start) ++g;
  const GroupDesc gd = eg.g[g];
  // the block's basis table (all threads of a block belong to one group)
  float* sBh = reinterpret_cast<float*>(sB + kMaxSlots * 6);
  float* sBl = sBh + kMaxSlots * 6;
  for (int k = threadIdx.x; k < gd.n_slots * 6; k += blockDim.x) {
    const double w = eg.basis[gd.basis_off + k];
    sB[k] = w;
    df_split(w, sBh[k], sBl[k]);
  }
  __syncthreads();
  const uint32_t li = (blockIdx.x - gd.block_start) * blockDim.x + threadIdx.x;
  if (li >= gd.count) return;
  const double pressure = ctl->pressure, vol_p = ctl->volume_pressure;
  const uint32_t i = gd.first + li;
  const uint32_t slot0 = gd.slot_base + li * (uint32_t)gd.n_slots;
  const double* B = sB;
  const double pr = pressure * __ldg(&b.pscale[i]);
  ElemOut o;
  if (gd.n_slots == 12)
    o = element_force<12, DFG, DFQ>(i, 12, slot0, B, b, sc, pr, vol_p);
  else if (gd.n_slots == 11)
    o = element_force<11, DFG, DFQ>(i, 11, slot0, B, b, sc, pr, vol_p);
  else
    o = element_force<0, DFG, DFQ>(i, gd.n_slots, slot0, B, b, sc, pr, vol_p);
  const uint32_t e = __ldg(&b.perm[i]);
  b.area[e] = o.area;
  b.kG[e] = o.kg / o.area;
  b.kM[e] = o.km / o.area;
  b.etens[e] = o.etens / o.area;
  b.ebend[e] = o.ebend / o.area;
}

// totals of the per-face measurements (original face order, fixed-order sums):
// E_tens, E_bend, kGauss, kMean and the area (ShellSystem.C:1285-1300, 2760-2786)
__global__ void __launch_bounds__(kBlock) k_elem_totals(DevBuf b, StepConst sc) {
  Ctl* ctl = b.ctl;
  if (inactive(ctl)) return;
  __shared__ TransposedSum sh;
  const uint32_t e = blockIdx.x * blockDim.x + threadIdx.x;
  double v[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
  if (e < sc.F) face_totals(b, e, v);
  block_sum_t<5>(v, sh);
  if (threadIdx.x == 0) {
    double* pp = b.partial + (size_t)blockIdx.x * 8;
    for (int k = 0; k < 5; ++k) pp[k] = v[k];
  }
  if (!last_block(&ctl->cnt[1])) return;
  double t[5];
  sum_partials_t<5>(b.partial, gridDim.x, sh, t);
  if (threadIdx.x == 0) {
    ctl->Etens = t[0]; ctl->Ebend = t[1]; ctl->kGauss = t[2]; ctl->kMean = t[3]; ctl->area = t[4];
  }
}

// -------------------------------------------------------- contact force --
// One candidate pair; ShellSystem.C:1803-1900.  Rounded operation by operation.
template <bool SMOOTH>
__global__ void __launch_bounds__(kBlock) k_contact_force(DevBuf b, StepConst sc) {
  Ctl* ctl = b.ctl;
  if (inactive(ctl)) return;
  __shared__ double sh[kBlock / 32];
  const uint32_t n_pairs = ctl->n_pairs;
  if (n_pairs == 0) {
    if (blockIdx.x == 0 && threadIdx.x == 0) {
      ctl->Eself = 0.0;
      ctl->Efric = 0.0;
      ctl->Nc = 0;
    }
    return;
  }
  double eself = 0.0, efric = 0.0, nc = 0.0;
  for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < n_pairs; j += gridDim.x * blockDim.x) {
    const uint32_t e[2] = {b.pe1[0][j], b.pe2[0][j]};
    // the shell's contact constants (a pair of a batch lies within one shell)
    const ShellCell* S = sc.n_cs ? &b.shc[b.face_shell[e[0]]] : nullptr;
    const double h = S ? S->thickness : sc.thickness;
    const double d2_friction = S ? S->d2_friction : sc.d2_friction;
    const double stiff_density = S ? S->stiff_density : sc.stiff_density;
    const double stiff_static_friction = S ? S->stiff_static_friction : sc.stiff_static_friction;
    const double* P1[3];
    const double* P2[3];
    uint32_t nid[2][3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      nid[0][k] = b.tri[3 * (size_t)e[0] + k];
      nid[1][k] = b.tri[3 * (size_t)e[1] + k];
      P1[k] = b.p + 3 * (size_t)nid[0][k];
      P2[k] = b.p + 3 * (size_t)nid[1][k];
    }
    shl_pair_geom g;
    double* out = b.pforce + kPairOut * (size_t)j;
    if (SMOOTH) {  // SmoothShellShellContact::compute: the search of k_smooth_search from the previous solution
      double x[4];
      for (int k = 0; k < 4; ++k) x[k] = b.pvw[0][4 * (size_t)j + k];
      g.d2 = b.pd2[0][j];
      for (int c = 0; c < 3; ++c) g.dc[c] = out[c];
      smooth_coords(b, e[0], e[1], x, &g);
    } else {
      shl_pair_compute(P1, P2, &g);
      b.pd2[0][j] = g.d2;
    }
    if (g.d2 <= 0.0) register_problem(ctl, SHL_CONTACT_PROBLEM);
    if (g.d2 < d2_friction) {
      const double area_min = fmin(b.area[e[0]], b.area[e[1]]);
      const double abs_dc = SHL_SQRT(g.d2);
      const double depth = SHL_SUB(h, abs_dc);
      double nrm[3];
      for (int c = 0; c < 3; ++c) nrm[c] = SHL_DIV(g.dc[c], abs_dc);
      const double stiffness = SHL_MUL(stiff_density, area_min);
      double f_normal = 0.0, es = 0.0, ef = 0.0;
      if (depth > 0.0) {
        nc += 1.0;
        f_normal = SHL_MUL(SHL_MUL(SHL_MUL(stiffness, SHL_SUB(h, abs_dc)), 0.5), SHL_ADD(1.0, SHL_DIV(h, abs_dc)));
        const double dep = SHL_SUB(h, abs_dc);
        es = SHL_MUL(SHL_MUL(0.5, stiffness),
                     SHL_ADD(SHL_SUB(SHL_MUL(SHL_MUL(0.5, dep), dep), SHL_MUL(dep, h)),
                             SHL_MUL(SHL_MUL(h, h), log(SHL_DIV(h, abs_dc)))));
      }
      eself += es;
      // relative velocity at the contact points (current velocity v)
      const double uu[2] = {SHL_SUB(SHL_SUB(1.0, g.v[0]), g.w[0]), SHL_SUB(SHL_SUB(1.0, g.v[1]), g.w[1])};
      double vrel[3];
      for (int c = 0; c < 3; ++c) {
        const double s2 = SHL_ADD(SHL_ADD(SHL_MUL(uu[1], b.v[3 * (size_t)nid[1][0] + c]),
                                          SHL_MUL(g.v[1], b.v[3 * (size_t)nid[1][1] + c])),
                                  SHL_MUL(g.w[1], b.v[3 * (size_t)nid[1][2] + c]));
        const double s1 = SHL_ADD(SHL_ADD(SHL_MUL(uu[0], b.v[3 * (size_t)nid[0][0] + c]),
                                          SHL_MUL(g.v[0], b.v[3 * (size_t)nid[0][1] + c])),
                                  SHL_MUL(g.w[0], b.v[3 * (size_t)nid[0][2] + c]));
        vrel[c] = SHL_SUB(s2, s1);
      }
      const double abs_v_normal = shl_v3_dot(vrel, nrm);
      double fcon[3] = {0.0, 0.0, 0.0};
      if (sc.friction) {
        double cp[3];
        for (int c = 0; c < 3; ++c)
          cp[c] = SHL_ADD(SHL_ADD(SHL_ADD(SHL_MUL(uu[0], P1[0][c]), SHL_MUL(g.v[0], P1[1][c])), SHL_MUL(g.w[0], P1[2][c])),
                          SHL_MUL(0.5, g.dc[c]));
        int stick = b.pstick[0][j];
        double orig[3] = {b.porig[0][3 * (size_t)j], b.porig[0][3 * (size_t)j + 1], b.porig[0][3 * (size_t)j + 2]};
        shl_friction_apply(&ef, fcon, f_normal, nrm, vrel, abs_v_normal, sc.v_stop, stiff_static_friction,
                           sc.mu_s, sc.mu_d, sc.self_friction_damping, &stick, orig, cp);
        b.pstick[0][j] = (uint8_t)stick;
        b.porig[0][3 * (size_t)j] = orig[0];
        b.porig[0][3 * (size_t)j + 1] = orig[1];
        b.porig[0][3 * (size_t)j + 2] = orig[2];
        efric += ef;
      }
      f_normal = SHL_SUB(f_normal, SHL_MUL(SHL_MUL(sc.self_damping, stiffness), abs_v_normal));
      for (int c = 0; c < 3; ++c) fcon[c] = SHL_ADD(fcon[c], SHL_MUL(f_normal, nrm[c]));
      out[0] = fcon[0]; out[1] = fcon[1]; out[2] = fcon[2];
      out[3] = g.v[0]; out[4] = g.w[0]; out[5] = g.v[1]; out[6] = g.w[1];
      out[7] = es; out[8] = ef;
    } else {
      b.porig[0][3 * (size_t)j] = 0.0;
      b.porig[0][3 * (size_t)j + 1] = 0.0;
      b.porig[0][3 * (size_t)j + 2] = 0.0;
      b.pstick[0][j] = 0;
      for (int c = 0; c < kPairOut; ++c) out[c] = 0.0;
    }
  }
  const double s0 = block_sum(eself, sh);
  const double s1 = block_sum(efric, sh);
  const double s2 = block_sum(nc, sh);
  if (threadIdx.x == 0) {
    double* pp = b.partial + (size_t)blockIdx.x * 8;
    pp[5] = s0; pp[6] = s1; pp[7] = s2;
  }
  if (!last_block(&ctl->cnt[2])) return;
  const int nb = gridDim.x;
  const double t0 = sum_partials(b.partial, 5, nb, sh);
  const double t1 = sum_partials(b.partial, 6, nb, sh);
  const double t2 = sum_partials(b.partial, 7, nb, sh);
  if (threadIdx.x == 0) {
    ctl->Eself = t0;
    ctl->Efric = t1;
    ctl->Nc = (uint32_t)t2;
  }
}

// ------------------------------------------------------ gather + correct --
// last block of the gather: the step's cavity totals (fixed order over blocks)
__device__ void cavity_totals(const DevBuf& b, const StepConst& sc, Ctl* ctl, double* sh) {
  const double nc = sum_partials(b.partial, 2, gridDim.x, sh);
  const double e = sum_partials(b.partial, 3, gridDim.x, sh);
  const double ef = sum_partials(b.partial, 4, gridDim.x, sh);
  const double fn = sum_partials(b.partial, 5, gridDim.x, sh);
  if (threadIdx.x == 0) {
    ctl->Nc_cav = (uint32_t)nc;
    ctl->Ecav = e;
    ctl->cavity_force = fn;
    ctl->Efric = (sc.contact ? ctl->Efric : 0.0) + ef;
  }
  __syncthreads();
}

__global__ void __launch_bounds__(kBlock) k_gather_correct(DevBuf b, StepConst sc, int mode, double* f_out,
                                                           double* a_out, RebuildCond rc) {
  // mode 0: eval (write f_out / a_out), mode 1: step corrector, mode 2: adaptive
  // attempt, mode 3: step corrector fused with the next step's prediction (fixed
  // dt): the step's predicted positions are read from b.pn and the next ones
  // written there, the corrected positions go to b.p
  Ctl* ctl = b.ctl;
  if (inactive(ctl)) {
    if (blockIdx.x == 0 && threadIdx.x == 0) set_rebuild_cond(rc, ctl);
    return;
  }
  __shared__ double sh[kBlock / 32];
  const uint32_t n = blockIdx.x * blockDim.x + threadIdx.x;
  double du2 = 0.0, ekin = 0.0, du2_next = 0.0;
  double c_nc = 0.0, c_e = 0.0, c_ef = 0.0, c_fn = 0.0;  // cavity: contacts, energy, friction energy, force
  if (n < sc.V) {
    double f[3] = {0.0, 0.0, 0.0};
    // the node's state, loaded ahead of (and independently of) the share sums
    const size_t k3n = 3 * (size_t)n;
    const bool corr = mode == 1 || mode == 3;
    double s_vp[3], s_minv[3], s_c[3], s_up[3], s_u[3], s_x[3], s_m[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      s_vp[c] = b.vp[k3n + c];
      s_minv[c] = b.Minv[k3n + c];
      s_c[c] = b.C[k3n + c];
      s_up[c] = corr ? b.up[k3n + c] : 0.0;
      s_u[c] = corr ? b.u[k3n + c] : 0.0;
      s_x[c] = corr ? b.X[k3n + c] : 0.0;
      s_m[c] = corr ? b.M[k3n + c] : 0.0;
    }
    if (sc.contact) {
      const uint32_t k0 = b.csr_ptr[n], k1 = b.csr_ptr[n + 1];
      // unrolled so that the loads of several entries are in flight; the
      // additions keep the list's order
#pragma unroll 4
      for (uint32_t k = k0; k < k1; ++k) {
        const uint32_t ent = b.csr_ent[k];
        const uint32_t j = ent >> 3, role = ent & 7u;
        const int e = role >= 3 ? 1 : 0, kk = role - 3 * e;
        const double* pf = b.pforce + kPairOut * (size_t)j;
        const double vv = pf[3 + 2 * e], ww = pf[4 + 2 * e];
        const double bary = kk == 0 ? (1.0 - vv - ww) : (kk == 1 ? vv : ww);
        const double pref = e == 0 ? -0.5 : 0.5;
        f[0] += bary * (pref * pf[0]);
        f[1] += bary * (pref * pf[1]);
        f[2] += bary * (pref * pf[2]);
      }
    }
    const uint32_t g0 = b.gather_ptr[n], g1 = b.gather_ptr[n + 1];
    if (sc.fp32) {
      float s0 = 0.f, s1 = 0.f, s2 = 0.f;
#pragma unroll 4
      for (uint32_t k = g0; k < g1; ++k) {
        const float* q = b.qe32 + 3 * (size_t)k;
        s0 += q[0];
        s1 += q[1];
        s2 += q[2];
      }
      f[0] -= (double)s0;
      f[1] -= (double)s1;
      f[2] -= (double)s2;
    } else if (sc.qe_df) {
      // double-float shares: added as pairs on the FP32 pipe, converted once
      const float2* q2 = reinterpret_cast<const float2*>(b.qe);
      df2 s0 = dfv(0.f), s1 = dfv(0.f), s2 = dfv(0.f);
#pragma unroll 8
      for (uint32_t k = g0; k < g1; ++k) {
        const float2 x = q2[3 * (size_t)k], y = q2[3 * (size_t)k + 1], z = q2[3 * (size_t)k + 2];
        s0 += df2{x.x, x.y};
        s1 += df2{y.x, y.y};
        s2 += df2{z.x, z.y};
      }
      f[0] -= df_to_double(s0);
      f[1] -= df_to_double(s1);
      f[2] -= df_to_double(s2);
    } else {
#pragma unroll 4
      for (uint32_t k = g0; k < g1; ++k) {
        const double* q = b.qe + 3 * (size_t)k;
        f[0] -= q[0];
        f[1] -= q[1];
        f[2] -= q[2];
      }
    }
    if (sc.cavity_contact) {
      // interaction with the cavity (ShellSystem.C:1600-1723)
      const CavityGeom cg = cavity_geom(ctl->cav_R, sc);
      const size_t k3 = 3 * (size_t)n;
      const double* pp = mode == 3 ? b.pn : b.p;
      const double p[3] = {pp[k3], pp[k3 + 1], pp[k3 + 2]};
      const double xr = (p[0] / cg.R_eff[0]) * (p[0] / cg.R_eff[0]);
      const double yr = (p[1] / cg.R_eff[1]) * (p[1] / cg.R_eff[1]);
      const double zr = (p[2] / cg.R_eff[2]) * (p[2] / cg.R_eff[2]);
      double opd;  // cavity_isoparameter, ShellSystem.h:336-362
      if (sc.cavity_type == SHL_CAVITY_BOX)
        opd = fmax(xr, fmax(yr, zr));
      else if (sc.cavity_type == SHL_CAVITY_CYLINDER)
        opd = fmax(xr, yr + zr);
      else
        opd = xr + yr + zr;
      double ecav_d = 0.0, efric_d = 0.0;
      if (opd > cg.opd_friction) {
        const double depth = cg.avg_R_eff * (sqrt(opd) - 1);
        // avg_area_node (ShellSystem.C:2462-2481): the faces of which the node is a vertex
        double area_sum = 0.0;
        uint32_t n_faces = 0;
        for (uint32_t k = __ldg(&b.node_face_ptr[n]); k < __ldg(&b.node_face_ptr[n + 1]); ++k) {
          area_sum += b.area[__ldg(&b.node_face[k])];
          ++n_faces;
        }
        const double area_node = area_sum / n_faces;
        const double stiffness = sc.stiff_density * area_node;
        double f_normal = 0.0;
        if (depth > 0) {
          c_nc += 1.0;
          const double e_node = 0.5 * stiffness * depth * depth;
          c_e += e_node;
          ecav_d = e_node / area_node;
          f_normal = stiffness * depth;
          c_fn += f_normal;
        }
        double nv[3] = {0.0, 0.0, 0.0};
        // the normal's case split uses p^2 / R_eff^2 (ShellSystem.C:1638-1660)
        const double xn = p[0] * p[0] * cg.inv_R2[0], yn = p[1] * p[1] * cg.inv_R2[1], zn = p[2] * p[2] * cg.inv_R2[2];
        if (sc.cavity_type == SHL_CAVITY_BOX) {
          const int c = (xn > yn && xn > zn) ? 0 : (yn > zn ? 1 : 2);
          nv[c] = (double)((p[c] > 0) - (p[c] < 0));
        } else if (sc.cavity_type == SHL_CAVITY_CYLINDER) {
          if (xn > yn + zn) {
            nv[0] = (double)((p[0] > 0) - (p[0] < 0));
          } else {
            nv[1] = p[1] * cg.inv_R2[1];
            nv[2] = p[2] * cg.inv_R2[2];
          }
        } else {
          for (int c = 0; c < 3; ++c) nv[c] = p[c] * cg.inv_R2[c];
        }
        const double inv_len = 1 / sqrt(nv[0] * nv[0] + nv[1] * nv[1] + nv[2] * nv[2]);
        for (int c = 0; c < 3; ++c) nv[c] *= inv_len;
        const double vel[3] = {b.v[k3], b.v[k3 + 1], b.v[k3 + 2]};
        const double abs_v_normal = vel[0] * nv[0] + vel[1] * nv[1] + vel[2] * nv[2];
        double fc[3] = {0.0, 0.0, 0.0};
        if (sc.cavity_friction) {
          double* so = b.cav_origin + k3;
          double orig[3] = {so[0], so[1], so[2]};
          int stick = (orig[0] * orig[0] + orig[1] * orig[1] + orig[2] * orig[2]) != 0.0;
          double ef = 0.0;
          shl_friction_apply(&ef, fc, f_normal, nv, vel, abs_v_normal, sc.v_stop, sc.stiff_static_friction,
                             sc.mu_s_cav, sc.mu_d_cav, sc.cav_fric_damping, &stick, orig, p);
          so[0] = orig[0];
          so[1] = orig[1];
          so[2] = orig[2];
          c_ef += ef;
          efric_d = ef / area_node;
        }
        f_normal += sc.cav_damping * stiffness * abs_v_normal;
        for (int c = 0; c < 3; ++c) {
          fc[c] -= f_normal * nv[c];
          f[c] += fc[c];
        }
      } else if (sc.cavity_friction) {
        // the spring is dropped only beyond the friction scope
        b.cav_origin[k3] = b.cav_origin[k3 + 1] = b.cav_origin[k3 + 2] = 0.0;
      }
      if (mode >= 1) {
        b.cav_ecav[n] = ecav_d;
        b.cav_efric[n] = efric_d;
      }
    }
    if (mode >= 1 && b.fcorr) {
      // FP64 defect of the FP32 force, refreshed at each residual check (shl_residual)
      f[0] += b.fcorr[3 * (size_t)n];
      f[1] += b.fcorr[3 * (size_t)n + 1];
      f[2] += b.fcorr[3 * (size_t)n + 2];
    }
    double d[3], un[3], vnn[3], an[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const size_t k = 3 * (size_t)n + c;
      const double vp = s_vp[c];
      const double ap = s_minv[c] * (f[c] - s_c[c] * vp);
      if (mode == 2) {
        // adaptive attempt: keep a_pred; local-error and velocity norms (ShellSystem.C:1017-1040)
        b.ap[k] = ap;
        du2 = fmax(du2, fabs(ap - b.a[k]));
        ekin = fmax(ekin, fabs(vp));
        continue;
      }
      if (mode == 0) {
        if (f_out) f_out[k] = f[c];
        if (a_out) a_out[k] = ap;
      } else {
        double up, vn;
        if (sc.contact) {
          up = __dadd_rn(__dmul_rn(sc.nm0, ap), s_up[c]);
          vn = __dadd_rn(__dmul_rn(sc.nm7, ap), vp);
        } else {
          up = fma(sc.nm0, ap, s_up[c]);
          vn = fma(sc.nm7, ap, vp);
        }
        d[c] = __dsub_rn(up, s_u[c]);
        b.u[k] = up;
        b.v[k] = vn;
        b.a[k] = ap;
        b.p[k] = __dadd_rn(s_x[c], up);
        ekin += vn * vn * s_m[c];
        un[c] = up;
        vnn[c] = vn;
        an[c] = ap;
      }
    }
    if (mode == 1 || mode == 3) du2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
    if (mode == 3) du2_next = predict_node(b, sc, n, un, vnn, an, sc.dt, sc.nm8, sc.nm6, b.pn);
  }
  if (mode == 0) return;
  if (sc.n_cs && (mode == 1 || mode == 3)) {
    shell_max_acc(b, sc, n, du2, 0);
    if (mode == 3) shell_max_acc(b, sc, n, du2_next, 1);
  }
  if (sc.cavity_contact) {
    const double r0 = block_sum(c_nc, sh), r1 = block_sum(c_e, sh), r2 = block_sum(c_ef, sh),
                 r3 = block_sum(c_fn, sh);
    if (threadIdx.x == 0) {
      double* pp = b.partial + (size_t)blockIdx.x * 8;
      pp[2] = r0; pp[3] = r1; pp[4] = r2; pp[5] = r3;
    }
  }
  if (mode == 2) {
    const double na = block_max(du2, sh);
    const double vm = block_max(ekin, sh);
    if (threadIdx.x == 0) {
      b.partial[(size_t)blockIdx.x * 8] = na;
      b.partial[(size_t)blockIdx.x * 8 + 1] = vm;
    }
    if (!last_block(&ctl->cnt[3])) return;
    if (sc.cavity_contact) cavity_totals(b, sc, ctl, sh);
    double m0 = 0.0, m1 = 0.0;
    for (int k = threadIdx.x; k < (int)gridDim.x; k += blockDim.x) {
      m0 = fmax(m0, __ldcg(&b.partial[(size_t)k * 8]));
      m1 = fmax(m1, __ldcg(&b.partial[(size_t)k * 8 + 1]));
    }
    const double norm_a = block_max(m0, sh);
    const double vmax = block_max(m1, sh);
    if (threadIdx.x != 0) return;
    const double dt = ctl->dt_cur;
    double new_dt = dt;
    if (ctl->time_step % sc.adapt_every == 0) {
      double rel_loc_err = sc.err_target;
      if (isfinite(norm_a))
        rel_loc_err = ctl->nm[9] * norm_a / sc.thickness;
      else
        register_problem(ctl, SHL_NOT_FINITE);
      if (rel_loc_err == 0.0)
        new_dt = 2 * dt;
      else if (rel_loc_err > sc.err_max || rel_loc_err < sc.err_min)
        new_dt = dt * pow(sc.err_target / rel_loc_err, 1. / 3);
      if (sc.contact || sc.cavity_contact) {
        // resolve the contact depth with at least 10 steps
        if (__dmul_rn(__dmul_rn(__dmul_rn(new_dt, vmax), 10.0), 2.0) > sc.thickness)
          new_dt = sc.thickness / (2.0 * 10.0 * vmax);
      }
    }
    ctl->new_dt = new_dt;
    ctl->accept = new_dt >= dt ? 1u : 0u;
    if (!ctl->accept) {
      // repeat the step with the smaller dt (ShellSystem.C:1104-1117)
      ctl->time = ctl->time - dt;
      ctl->time_step -= 1;
      if (ctl->table_pos > 0) ctl->table_pos -= 1;
      ctl->rejections += 1;
      set_newmark(ctl, sc, new_dt);
      if (ctl->dt_cur <= 2.220446049250313e-16) register_problem(ctl, SHL_SMALL_TIMESTEP);
    }
    return;
  }
  const double m = block_max(du2, sh);
  const double ek = block_sum(0.5 * ekin, sh);
  const double mn = mode == 3 ? block_max(du2_next, sh) : 0.0;
  if (threadIdx.x == 0) {
    b.partial[(size_t)blockIdx.x * 8] = m;
    b.partial[(size_t)blockIdx.x * 8 + 1] = ek;
    b.partial[(size_t)blockIdx.x * 8 + 6] = mn;
  }
  if (!last_block(&ctl->cnt[3])) return;
  if (sc.cavity_contact) cavity_totals(b, sc, ctl, sh);
  double mm = 0.0, mmn = 0.0;
  for (int k = threadIdx.x; k < (int)gridDim.x; k += blockDim.x) {
    mm = fmax(mm, __ldcg(&b.partial[(size_t)k * 8]));
    mmn = fmax(mmn, __ldcg(&b.partial[(size_t)k * 8 + 6]));
  }
  mm = block_max(mm, sh);
  if (mode == 3) mmn = block_max(mmn, sh);
  const double ekt = sum_partials(b.partial, 1, gridDim.x, sh);
  if (sc.n_cs) {  // a batch: each shell's own check_increment(true)
    if (threadIdx.x == 0) {
      ctl->Ekin = ekt;
      if (!isfinite(ekt)) register_problem(ctl, SHL_NOT_FINITE);
    }
    batch_correct_check(b, sc, rc, mode == 3);
    return;
  }
  if (threadIdx.x != 0) return;
  ctl->Ekin = ekt;
  if (mode == 3) ctl->du2_pred = mmn;  // check_increment(false) of the next step, in k_begin_step
  // check_increment(true)
  const double du_max = sqrt(mm);
  if (isfinite(du_max)) {
    ctl->du_sum = __dadd_rn(ctl->du_sum, __dmul_rn(2.0, du_max));
    if (du_max == 0.0)
      register_problem(ctl, SHL_NO_DISP_CHANGE);
    else if (sc.contact && du_max > 0.5 * sc.thickness)
      register_problem(ctl, SHL_LARGE_DISP);
  } else {
    register_problem(ctl, SHL_NOT_FINITE);
  }
  if (!isfinite(ekt)) register_problem(ctl, SHL_NOT_FINITE);
  const uint32_t flag = (sc.contact && ctl->du_sum >= rebuild_tolerance(sc, ctl)) ? 1u : 0u;
  if (mode == 3) {
    ctl->rebuild_pending = flag;  // made by the next step's IF node, before its own pass
    return;
  }
  ctl->rebuild = flag;
  set_rebuild_cond(rc, ctl);
}

// corrector of an accepted adaptive attempt (ShellSystem.C:1046-1101): u, v, a
// from the stored a_pred; check_increment(true); contact-list flag
__global__ void __launch_bounds__(kBlock) k_correct_adapt(DevBuf b, StepConst sc, RebuildCond rc) {
  Ctl* ctl = b.ctl;
  if (inactive(ctl) || !ctl->accept) {
    if (blockIdx.x == 0 && threadIdx.x == 0) set_rebuild_cond(rc, ctl);
    return;
  }
  __shared__ double sh[kBlock / 32];
  const uint32_t n = blockIdx.x * blockDim.x + threadIdx.x;
  const double nm0 = ctl->nm[0], nm7 = ctl->nm[7];
  double du2 = 0.0, ekin = 0.0;
  if (n < sc.V) {
    double d[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const size_t k = 3 * (size_t)n + c;
      const double ap = b.ap[k], vp = b.vp[k];
      double up, vn;
      if (sc.contact) {
        up = __dadd_rn(__dmul_rn(nm0, ap), b.up[k]);
        vn = __dadd_rn(__dmul_rn(nm7, ap), vp);
      } else {
        up = fma(nm0, ap, b.up[k]);
        vn = fma(nm7, ap, vp);
      }
      d[c] = __dsub_rn(up, b.u[k]);
      b.u[k] = up;
      b.v[k] = vn;
      b.a[k] = ap;
      b.p[k] = __dadd_rn(b.X[k], up);
      ekin += vn * vn * b.M[k];
    }
    du2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
  }
  const double m = block_max(du2, sh);
  const double ek = block_sum(0.5 * ekin, sh);
  if (threadIdx.x == 0) {
    b.partial[(size_t)blockIdx.x * 8] = m;
    b.partial[(size_t)blockIdx.x * 8 + 1] = ek;
  }
  if (!last_block(&ctl->cnt[6])) return;
  double mm = 0.0;
  for (int k = threadIdx.x; k < (int)gridDim.x; k += blockDim.x) mm = fmax(mm, __ldcg(&b.partial[(size_t)k * 8]));
  mm = block_max(mm, sh);
  const double ekt = sum_partials(b.partial, 1, gridDim.x, sh);
  if (threadIdx.x != 0) return;
  ctl->Ekin = ekt;
  const double du_max = sqrt(mm);
  if (isfinite(du_max)) {
    ctl->du_sum = __dadd_rn(ctl->du_sum, __dmul_rn(2.0, du_max));
    if (du_max == 0.0)
      register_problem(ctl, SHL_NO_DISP_CHANGE);
    else if (sc.contact && du_max > 0.5 * sc.thickness)
      register_problem(ctl, SHL_LARGE_DISP);
  } else {
    register_problem(ctl, SHL_NOT_FINITE);
  }
  if (!isfinite(ekt)) register_problem(ctl, SHL_NOT_FINITE);
  ctl->rebuild = (sc.contact && ctl->du_sum >= rebuild_tolerance(sc, ctl)) ? 1u : 0u;
  set_rebuild_cond(rc, ctl);
}

// ------------------------------------------------------ volume, end step --
__global__ void __launch_bounds__(kBlock) k_volume_end(DevBuf b, StepConst sc, int end_step) {
  Ctl* ctl = b.ctl;
  if (inactive(ctl)) return;
  if (end_step && sc.adapt_every && !ctl->accept) {
    // a repeated attempt ends no step; only a step size below the machine
    // precision (SHL_SMALL_TIMESTEP) ends the run (ShellSystem.C:1110-1117)
    if (blockIdx.x == 0 && threadIdx.x == 0) {
      const int pr = ctl->problem;
      if (pr >= SHL_STOP_SIM) {
        if (pr > ctl->worst_problem) ctl->worst_problem = pr;
        if (ctl->first_problem_step == 0) ctl->first_problem_step = ctl->time_step + 1;
        ctl->halted = 1;
        ctl->problem = 0;
      }
    }
    return;
  }
  // the element kernel's per-face measurement totals (as k_elem_totals forms
  // them, bit for bit) and the enclosed volume, in one pass over the faces
  __shared__ TransposedSum sh;
  const uint32_t f = blockIdx.x * blockDim.x + threadIdx.x;
  double v[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
  if (f < sc.F) {
    face_totals(b, f, v);
    const double* q0 = b.p + 3 * (size_t)b.tri[3 * (size_t)f];
    const double* q1 = b.p + 3 * (size_t)b.tri[3 * (size_t)f + 1];
    const double* q2 = b.p + 3 * (size_t)b.tri[3 * (size_t)f + 2];
    v[5] = q0[0] * (q1[1] * q2[2] - q2[1] * q1[2]) - q1[0] * (q0[1] * q2[2] - q2[1] * q0[2]) +
           q2[0] * (q0[1] * q1[2] - q1[1] * q0[2]);
  }
  block_sum_t<6>(v, sh);
  if (threadIdx.x == 0) {
    double* pp = b.partial + (size_t)blockIdx.x * 8;
    for (int k = 0; k < 6; ++k) pp[k] = v[k];
  }
  if (!last_block(&ctl->cnt[4])) return;
  double t[6];
  sum_partials_t<6>(b.partial, gridDim.x, sh, t);
  if (threadIdx.x != 0) return;
  ctl->Etens = t[0]; ctl->Ebend = t[1]; ctl->kGauss = t[2]; ctl->kMean = t[3]; ctl->area = t[4];
  ctl->volume = fabs(t[5] / 6.0) - ctl->area * 0.5 * sc.thickness;
  if (!end_step) return;
  const double dt = sc.adapt_every ? ctl->dt_cur : sc.dt;
  ctl->sum_dt += dt;
  ctl->sum_area += dt * ctl->area;
  ctl->sum_volume += dt * ctl->volume;
  ctl->sum_Nc += dt * (double)ctl->Nc;
  ctl->sum_Ekin += dt * ctl->Ekin;
  ctl->sum_Etens += dt * ctl->Etens;
  ctl->sum_Ebend += dt * ctl->Ebend;
  ctl->sum_Eself += dt * ctl->Eself;
  ctl->sum_Efric += dt * ctl->Efric;
  ctl->sum_kGauss += dt * ctl->kGauss;
  ctl->sum_kMean += dt * ctl->kMean;
  if (sc.cavity_contact) {
    ctl->sum_pcav += dt * ctl->cavity_force / cavity_surface(ctl->cav_R, sc.cavity_type);
    ctl->sum_Nc_cav += dt * (double)ctl->Nc_cav;
    ctl->sum_Ecav += dt * ctl->Ecav;
  }
  const int pr = ctl->problem;
  if (pr > ctl->worst_problem) ctl->worst_problem = pr;
  if (pr > 0 && ctl->first_problem_step == 0) ctl->first_problem_step = ctl->time_step;
  ctl->steps_done += 1;
  if (pr >= SHL_STOP_SIM || (sc.stop_on_problem && pr > 0) || ctl->error) ctl->halted = 1;
  ctl->problem = 0;
  // the next step's dt, after the measurement used this one (ShellSystem.C:1096-1098)
  if (sc.adapt_every) set_newmark(ctl, sc, ctl->new_dt);
  if (ctl->steps_done >= ctl->steps_target) ctl->paused |= 1u;
  // stopping criterion, tested before the next step (shell.C:314-318)
  if (sc.sfun_len > 0 && eval_program(sc.sfun, sc.sfun_len, ctl->time, 0.0) != 0.0) ctl->paused |= 2u;
}

// ------------------------------------------------------------ utilities --
// per shell s (nodes node_off[s] .. node_off[s+1]), one block per shell, fixed
// order: |f - m F/M|^2 and |f_ext - m F_ext/M|^2, where F is the resultant of f
// over the shell and m, M the nodal and total mass -- the residual without its
// rigid-translation part.  (A closed shell under uniform pressure carries a
// resultant of the order of the quadrature error, which a free shell answers
// with a steady drift, not with deformation.)
__global__ void __launch_bounds__(kBlock) k_shell_norms(const double* f, const double* fext, const double* mass,
                                                        const uint32_t* node_off, double* out) {
  __shared__ double sh[kBlock / 32];
  __shared__ double res[7];
  const uint32_t n0 = node_off[blockIdx.x], n1 = node_off[blockIdx.x + 1];
  double s[7] = {0, 0, 0, 0, 0, 0, 0};  // F (3), F_ext (3), M
  for (uint32_t n = n0 + threadIdx.x; n < n1; n += blockDim.x) {
    for (int c = 0; c < 3; ++c) {
      s[c] += f[3 * (size_t)n + c];
      s[3 + c] += fext[3 * (size_t)n + c];
    }
    s[6] += mass[3 * (size_t)n];
  }
  for (int k = 0; k < 7; ++k) {
    const double t = block_sum(s[k], sh);
    if (threadIdx.x == 0) res[k] = t;
  }
  __syncthreads();
  const double inv_m = 1.0 / res[6];
  double a = 0.0, e = 0.0;
  for (uint32_t n = n0 + threadIdx.x; n < n1; n += blockDim.x) {
    const double w = mass[3 * (size_t)n] * inv_m;
    for (int c = 0; c < 3; ++c) {
      const double x = f[3 * (size_t)n + c] - w * res[c];
      const double y = fext[3 * (size_t)n + c] - w * res[3 + c];
      a += x * x;
      e += y * y;
    }
  }
  a = block_sum(a, sh);
  e = block_sum(e, sh);
  if (threadIdx.x == 0) {
    out[2 * blockIdx.x] = a;
    out[2 * blockIdx.x + 1] = e;
  }
}

void launch_shell_norms(const double* f, const double* fext, const double* mass, const uint32_t* node_off,
                        uint32_t n_shells, double* out, cudaStream_t s) {
  k_shell_norms<<<n_shells, kBlock, 0, s>>>(f, fext, mass, node_off, out);
}

__global__ void k_defect(const double* f64, const double* f32, size_t n, double* out) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    out[i] = f64[i] - f32[i];
}

void launch_defect(const double* f64, const double* f32, size_t n, double* out, cudaStream_t s) {
  k_defect<<<(unsigned)std::min<size_t>((n + 255) / 256, 4096), 256, 0, s>>>(f64, f32, n, out);
}


// FP64 FMA throughput probe: 8 independent register chains per thread.
__global__ void __launch_bounds__(256) k_fp64_peak(double* out, int iters, double b, double c) {
  double a0 = threadIdx.x * 1e-9, a1 = a0 + 1e-3, a2 = a0 + 2e-3, a3 = a0 + 3e-3;
  double a4 = a0 + 4e-3, a5 = a0 + 5e-3, a6 = a0 + 6e-3, a7 = a0 + 7e-3;
  for (int i = 0; i < iters; ++i) {
    a0 = fma(a0, b, c); a1 = fma(a1, b, c); a2 = fma(a2, b, c); a3 = fma(a3, b, c);
    a4 = fma(a4, b, c); a5 = fma(a5, b, c); a6 = fma(a6, b, c); a7 = fma(a7, b, c);
  }
  const double s = ((a0 + a1) + (a2 + a3)) + ((a4 + a5) + (a6 + a7));
  if (s == 1.2345678) out[blockIdx.x] = s;  // never true; keeps the chains live
}

// write a buffer larger than L2 so that the next launch starts with a cold cache
__global__ void k_flush(uint4* buf, size_t n16, uint32_t tag) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n16; i += (size_t)gridDim.x * blockDim.x)
    buf[i] = make_uint4(tag, (uint32_t)i, tag, (uint32_t)(i >> 32));
}

void launch_fp64_peak(double* out, int blocks, int iters, cudaStream_t s) {
  k_fp64_peak<<<blocks, 256, 0, s>>>(out, iters, 0.9999999, 1e-9);
}
void launch_flush(void* buf, size_t bytes, uint32_t tag, cudaStream_t s) {
  k_flush<<<4 * 152, 512, 0, s>>>((uint4*)buf, bytes / 16, tag);
}

// --------------------------------------------------------------- launch --
static inline uint32_t nblk(uint32_t n) { return (n + kBlock - 1) / kBlock; }

void launch_predict(const DevBuf& b, const StepConst& sc, RebuildCond rc, cudaStream_t s, bool nodes_only) {
  k_predict<<<nblk(sc.V), kBlock, 0, s>>>(b, sc, rc, nodes_only ? 1 : 0);
}
void launch_begin_step(const DevBuf& b, const StepConst& sc, RebuildCond rc, cudaStream_t s) {
  k_begin_step<<<1, sc.n_cs ? kBlock : 32, 0, s>>>(b, sc, rc);
}
void launch_rebuild_second(const DevBuf& b, const StepConst& sc, cudaStream_t s) {
  k_rebuild_second<<<1, sc.n_cs ? kBlock : 32, 0, s>>>(b, sc);
}
void launch_rebuild_first(const DevBuf& b, const StepConst& sc, cudaStream_t s) {
  k_rebuild_first<<<1, sc.n_cs ? kBlock : 32, 0, s>>>(b, sc);
}
void launch_batch_flags(const DevBuf& b, const StepConst& sc, int mode, cudaStream_t s) {
  k_batch_flags<<<1, kBlock, 0, s>>>(b, sc, mode);
}
void launch_state_host(const DevBuf& b, const StepConst& sc, double* hu, double* hv, double* ha, bool load,
                       cudaStream_t s) {
  const size_t n = load ? (size_t)sc.V : 3 * (size_t)sc.V;  // load: one thread per node
  k_state_host<<<(unsigned)((n + kBlock - 1) / kBlock), kBlock, 0, s>>>(b, sc, hu, hv, ha, load ? 1 : 0);
}
void launch_positions(const DevBuf& b, const StepConst& sc, cudaStream_t s) {
  k_positions<<<nblk(sc.V), kBlock, 0, s>>>(b, sc);
}

// Control-block updates that the host would otherwise make by a read-modify-write
// round trip: kCtlReset clears the run report (worst problem, counters, sums),
// kCtlTable rewinds the pressure table to n entries, kCtlArm sets the pause
// target n steps past the steps done.
__global__ void k_ctl_begin(Ctl* ctl, uint32_t n, uint32_t flags) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  Ctl& h = *ctl;
  if (flags & kCtlReset) {
    h.steps_done = 0;
    h.worst_problem = 0;
    h.first_problem_step = 0;
    h.halted = 0;
    h.error = 0;
    h.problem = 0;
    h.n_rebuilds = 0;
    h.rejections = 0;
    h.paused = 0;
    h.sum_pcav = h.sum_Nc_cav = h.sum_Ecav = 0;
    h.steps_target = ~0u;
    h.sum_dt = h.sum_area = h.sum_volume = h.sum_Nc = h.sum_Ekin = h.sum_Etens = h.sum_Ebend = h.sum_Eself =
        h.sum_Efric = h.sum_kGauss = h.sum_kMean = 0;
  }
  if (flags & kCtlTable) {
    h.table_pos = 0;
    h.table_len = n;
  }
  if (flags & kCtlArm) {
    h.steps_target = h.steps_done + n;
    h.paused = 0;
  }
}
void launch_ctl_begin(Ctl* ctl, uint32_t n, uint32_t flags, cudaStream_t s) { k_ctl_begin<<<1, 32, 0, s>>>(ctl, n, flags); }
// launch shapes and arithmetic of the element kernels (see k_elements)
const ElemVariant kElemVariants[kNumElemVariants] = {
    {256, 0, "fp64 256x1"},        {256, 1, "fp64 256x1 pair-G"}, {128, 1, "fp64 128x3 pair-G"},
    {64, 1, "fp64 64x5 pair-G"},   {64, 1, "fp64 64x6 pair-G"},   {64, 0, "fp64 64x5"},
    {256, 2, "fp64 256x1 df"},     {128, 2, "fp64 128x3 df"},     {64, 2, "fp64 64x6 df"},
    {64, 2, "fp64 64x8 df"},       {kFlatBlock, 2, "fp64 544x1 df flat"},
    {256, 0, "fp32 256x2"},        {128, 0, "fp32 128x4"},        {64, 0, "fp32 64x8"}};

// the double-float kernels take more than the default 48 KB of shared memory
// (staging plus the basis table); called once per device before their first launch
cudaError_t init_element_kernels() {
  cudaError_t e = cudaSuccess;
  auto set = [&](const void* f, int block) {
    if (e != cudaSuccess) return;
    e = cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)df_stage_bytes(block));
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(f, cudaFuncAttributePreferredSharedMemoryCarveout, cudaSharedmemCarveoutMaxShared);
  };
  set((const void*)k_elements_df<256, 1>, 256);
  set((const void*)k_elements_df<128, 3>, 128);
  set((const void*)k_elements_df<64, 6>, 64);
  set((const void*)k_elements_df<64, 8>, 64);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute((const void*)k_elements_df_flat<kFlatBlock>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)flat_smem_bytes());
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute((const void*)k_elements_df_flat<kFlatBlock>,
                             cudaFuncAttributePreferredSharedMemoryCarveout, cudaSharedmemCarveoutMaxShared);
  return e;
}

void launch_elements(const DevBuf& b, const StepConst& sc, const ElemLaunch& el, cudaStream_t s, bool totals) {
  const uint32_t nb = el.blocks;
  const ElemGroups& eg = el.eg;
  switch (el.variant) {
    case 0: k_elements<256, 1, false, false><<<nb, 256, 0, s>>>(b, sc, eg); break;
    case 1: k_elements<256, 1, true, false><<<nb, 256, 0, s>>>(b, sc, eg); break;
    case 2: k_elements<128, 3, true, false><<<nb, 128, 0, s>>>(b, sc, eg); break;
    case 3: k_elements<64, 5, true, false><<<nb, 64, 0, s>>>(b, sc, eg); break;
    case 4: k_elements<64, 6, true, false><<<nb, 64, 0, s>>>(b, sc, eg); break;
    case 5: k_elements<64, 5, false, false><<<nb, 64, 0, s>>>(b, sc, eg); break;
    case 6: k_elements_df<256, 1><<<nb, 256, df_stage_bytes(256), s>>>(b, sc, eg); break;
    case 7: k_elements_df<128, 3><<<nb, 128, df_stage_bytes(128), s>>>(b, sc, eg); break;
    case 8: k_elements_df<64, 6><<<nb, 64, df_stage_bytes(64), s>>>(b, sc, eg); break;
    case 9: k_elements_df<64, 8><<<nb, 64, df_stage_bytes(64), s>>>(b, sc, eg); break;
    case 10: k_elements_df_flat<kFlatBlock><<<nb, kFlatBlock, flat_smem_bytes(), s>>>(b, sc, eg); break;
    case 11: k_elements32<256, 2><<<nb, 256, 0, s>>>(b, sc, eg); break;
    case 12: k_elements32<128, 4><<<nb, 128, 0, s>>>(b, sc, eg); break;
    default: k_elements32<64, 8><<<nb, 64, 0, s>>>(b, sc, eg); break;
  }
  if (totals) k_elem_totals<<<nblk(sc.F), kBlock, 0, s>>>(b, sc);
}
void launch_contact_force(const DevBuf& b, const StepConst& sc, int, cudaStream_t s) {
  uint32_t nb = nblk(sc.pairs_cap);
  if (nb > 4 * 152) nb = 4 * 152;
  if (nb == 0) nb = 1;
  if (sc.smooth) {
    launch_smooth_search(b, sc, false, s);
    k_contact_force<true><<<nb, kBlock, 0, s>>>(b, sc);
  } else
    k_contact_force<false><<<nb, kBlock, 0, s>>>(b, sc);
}
// mode 2: an adaptive attempt (a_pred and the error estimate); else correct ? step corrector : evaluation
void launch_gather_correct(const DevBuf& b, const StepConst& sc, int mode, bool correct, double* f_out, double* a_out,
                           cudaStream_t s, RebuildCond rc) {
  const int m = (mode == 2 || mode == 3) ? mode : (correct ? 1 : 0);
  k_gather_correct<<<nblk(sc.V), kBlock, 0, s>>>(b, sc, m, f_out, a_out, rc);
}
void launch_correct_adapt(const DevBuf& b, const StepConst& sc, cudaStream_t s, RebuildCond rc) {
  k_correct_adapt<<<(sc.V + kBlock - 1) / kBlock, kBlock, 0, s>>>(b, sc, rc);
}

void launch_volume_end_step(const DevBuf& b, const StepConst& sc, bool end_step, cudaStream_t s) {
  k_volume_end<<<nblk(sc.F), kBlock, 0, s>>>(b, sc, end_step ? 1 : 0);
}

// ================================================================ no-alloc --
// Force evaluation into caller-owned device memory with no device allocation:
// the per-(face, slot) force shares go to a file-scope scratch array instead of
// a buffer of the context.  See shl_internal_force_noalloc in include/shl.h.

// Largest shell this path accepts: 12 * 32768 (face, patch node) slots of 3
// doubles each, i.e. 32768 faces of regular 12-node patches (fewer where
// patches around vertices of valence above 6 have more nodes) -> 9 MiB,
// resident on every GPU that loads the library.
constexpr uint64_t kNoAllocMaxSlots = 12ull * 32768ull;
static __device__ __align__(256) double g_noalloc_scratch[kNoAllocMaxSlots * 3];

// Device address of the scratch array per device, looked up once per device
// (cudaGetSymbolAddress on the host side; the array name itself is only a
// host-side stand-in).  std::call_once orders first calls made by several
// host threads on one device.
constexpr int kNoAllocDevices = 64;
static std::once_flag g_noalloc_once[kNoAllocDevices];
static void* g_noalloc_ptr[kNoAllocDevices];
static cudaError_t g_noalloc_err[kNoAllocDevices];

uint64_t noalloc_max_slots() { return kNoAllocMaxSlots; }

cudaError_t noalloc_scratch(void** ptr) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= kNoAllocDevices) return cudaErrorInvalidDevice;
  std::call_once(g_noalloc_once[dev], [dev] {
    void* p = nullptr;
    g_noalloc_err[dev] = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    g_noalloc_ptr[dev] = p;
  });
  if (g_noalloc_err[dev] != cudaSuccess) return g_noalloc_err[dev];
  *ptr = g_noalloc_ptr[dev];
  return cudaSuccess;
}

// element shares at u (caller pointer in b.up) into the scratch (b.qe);
// touches neither the control block nor the context's buffers
__global__ void __launch_bounds__(kBlock) k_elements_noalloc(DevBuf b, StepConst sc, ElemGroups eg,
                                                             double pressure) {
  __shared__ double sB[kMaxSlots * 6];
  int g = 0;
  while (g + 1 < eg.n && blockIdx.x >= eg.g[g + 1].block_start) ++g;
  const GroupDesc gd = eg.g[g];
  for (int k = threadIdx.x; k < gd.n_slots * 6; k += blockDim.x) sB[k] = eg.basis[gd.basis_off + k];
  __syncthreads();
  const uint32_t li = (blockIdx.x - gd.block_start) * blockDim.x + threadIdx.x;
  if (li >= gd.count) return;
  const uint32_t i = gd.first + li;
  const uint32_t slot0 = gd.slot_base + li * (uint32_t)gd.n_slots;
  const double pr = pressure * __ldg(&b.pscale[i]);
  if (gd.n_slots == 12)
    element_force<12>(i, 12, slot0, sB, b, sc, pr, 0.0);
  else if (gd.n_slots == 11)
    element_force<11>(i, 11, slot0, sB, b, sc, pr, 0.0);
  else
    element_force<0>(i, gd.n_slots, slot0, sB, b, sc, pr, 0.0);
}

// f = -(sum of the node's shares), the same gather order as the step kernel
__global__ void __launch_bounds__(kBlock) k_gather_noalloc(DevBuf b, StepConst sc, double* f_out) {
  const uint32_t n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= sc.V) return;
  double f[3] = {0.0, 0.0, 0.0};
  const uint32_t g0 = b.gather_ptr[n], g1 = b.gather_ptr[n + 1];
  for (uint32_t k = g0; k < g1; ++k) {
    const double* q = b.qe + 3 * (size_t)k;
    f[0] -= q[0];
    f[1] -= q[1];
    f[2] -= q[2];
  }
  f_out[3 * (size_t)n] = f[0];
  f_out[3 * (size_t)n + 1] = f[1];
  f_out[3 * (size_t)n + 2] = f[2];
}

cudaError_t launch_force_noalloc(const DevBuf& ctx_b, const StepConst& sc, const ElemGroups& eg, uint32_t n_blocks,
                                 const double* u, double pressure, double* f_out, cudaStream_t s) {
  void* scratch = nullptr;
  cudaError_t e = noalloc_scratch(&scratch);
  if (e != cudaSuccess) return e;
  DevBuf b = ctx_b;
  b.up = const_cast<double*>(u);
  b.qe = (double*)scratch;
  k_elements_noalloc<<<n_blocks, kBlock, 0, s>>>(b, sc, eg, pressure);
  k_gather_noalloc<<<nblk(sc.V), kBlock, 0, s>>>(b, sc, f_out);
  return cudaGetLastError();
}

}  // namespace shl
