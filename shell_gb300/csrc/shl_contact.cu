// shl_contact.cu -- linked-cell self-contact candidate list on the device.
//
// compute_shell_shell_contact_candidates (ShellSystem.C:1910-2135) with
// compute_bounding_box (2544-2587), as a pipeline of kernels that all return
// immediately unless the device flag ctl->rebuild is set (so the pipeline can
// be captured into a CUDA graph and skipped on device):
//
//   k_rb_aabb      per-face AABBs and sizes, per-block bounds
//   k_rb_bounds    shell bounds, avg_elem_size (fixed-order sum), cell size,
//                  d_max, cell counts; TOO_MANY_CELLS check (k_rb_grids and
//                  k_rb_grid_scan per shell for a batch)
//   k_rb_clear     clear the cell histogram and the per-face counters
//   k_rb_count     cell ranges per face, cell histogram (counting sort, pass 1);
//                  keep flags of the old list (ShellSystem.C:2016-2027)
//   scan           cell_count -> cell_start
//   k_rb_fill      scatter faces into their cells (counting sort, pass 2)
//   k_rb_cand      per (cell, face e1) entry: faces e2 > e1 in the cell, emitted
//                  from the lowest shared cell only, not topologically close, not
//                  in the kept list, not AABB-apart by d_max, not certainly apart
//                  along the line of centroids (a conservative prefilter)
//   k_rb_narrow    per candidate: closest points, accept d2 <= d2_max (SMOOTH:
//                  k_limit_coeffs and k_smooth_search)
//   scan, k_rb_scatter_new  accepted pairs grouped by eid1 (counting sort)
//   scan           per-face pair counts -> segment offsets
//   k_rb_assemble  kept old pairs + new pairs of each face, merged in e2 order
//   k_rb_copyback  scratch list -> list
//
// The resulting list equals, as a set, the reference's list at the same state
// (the reference's cell-membership test is reproduced with the same rounded
// operations); it is stored sorted by (eid1, eid2), which fixes the order the
// per-node gather adds contact forces in.  The reference's slot order depends
// on OpenMP scheduling and is not reproduced.
#include <cuda_runtime.h>

#include <cstdint>

#include "shl_geom.h"
#include "shl_internal.cuh"

namespace shl {

namespace {

__device__ __forceinline__ bool rb_off(const Ctl* ctl) { return ctl->rebuild == 0 || ctl->halted != 0; }

__device__ __forceinline__ bool last_block_rb(uint32_t* counter) {
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

__device__ __forceinline__ void set_error(Ctl* ctl, int code) {
  atomicMax(&ctl->error, code);
  ctl->rebuild = 0;
}

// The cell grid that face f is binned in: the control block's for a single
// shell, its shell's for a batch with self-contact (ShellCell).
struct GridView {
  double cell_size, d_max, d2_max;
  const double* bmin;
  uint32_t ny, nz, base;
};
__device__ __forceinline__ GridView grid_of(const DevBuf& b, const StepConst& sc, uint32_t f) {
  GridView g;
  if (sc.n_cs) {
    const ShellCell& s = b.shc[b.face_shell[f]];
    g.cell_size = s.cell_size; g.d_max = s.d_max; g.d2_max = s.d2_max; g.bmin = s.bmin;
    g.ny = s.ncd[1]; g.nz = s.ncd[2]; g.base = s.cell_base;
  } else {
    const Ctl* ctl = b.ctl;
    g.cell_size = ctl->cell_size; g.d_max = ctl->d_max; g.d2_max = ctl->d2_max; g.bmin = ctl->bmin;
    g.ny = ctl->ncd[1]; g.nz = ctl->ncd[2]; g.base = 0;
  }
  return g;
}

// face f takes part in the current pass (a batch rebuilds only the shells whose trigger fired)
__device__ __forceinline__ bool face_in_pass(const DevBuf& b, const StepConst& sc, uint32_t f) {
  return sc.n_cs == 0 || b.shc[b.face_shell[f]].rebuild != 0;
}

// The lane sums of the fixed-order sum (shl_geom.h) of x[0..n): lane l adds
// x[l], x[l + LANES], ... in index order into lanes[l].  Each thread carries
// its LANES / blockDim lanes together so that the loads of several rounds are
// in flight at once; the additions of every lane keep their order.
template <int PER>
__device__ __forceinline__ void lane_sums(const double* x, uint32_t n, double* lanes) {
  double acc[PER];
#pragma unroll
  for (int k = 0; k < PER; ++k) acc[k] = 0.0;
#pragma unroll 4
  for (uint32_t i0 = 0; i0 < n; i0 += SHL_SUM_LANES) {
#pragma unroll
    for (int k = 0; k < PER; ++k) {
      const uint32_t i = i0 + threadIdx.x + (uint32_t)k * blockDim.x;
      if (i < n) acc[k] = __dadd_rn(acc[k], __ldcg(&x[i]));
    }
  }
#pragma unroll
  for (int k = 0; k < PER; ++k) lanes[threadIdx.x + (uint32_t)k * blockDim.x] = acc[k];
}

// Cell size, d_max and cell counts of a shell from its bounds and average
// element size (ShellSystem.C:1929-1969), rounded operation by operation.
// Returns the number of cells (0 with TOO_MANY_CELLS registered).
__device__ uint64_t grid_setup(const double* bmin, const double* bmax, double avg, double cell_size_mult,
                               double cell_margin, double thickness, int smooth, double* cell_size_out,
                               double* d_max_out, uint32_t* ncd) {
  double cell_size = __dmul_rn(cell_size_mult, avg);
  const double tolerance = __dmul_rn(cell_margin, cell_size);
  cell_size = __dadd_rn(cell_size, tolerance);
  double d_max = __dadd_rn(thickness, tolerance);
  // SMOOTH: the limit surfaces may be closer than the facets (ShellSystem.C:1940-1944)
  if (smooth) d_max = __dadd_rn(d_max, avg);
  *cell_size_out = cell_size;
  *d_max_out = d_max;
  uint64_t n_cells = 1;
  for (int c = 0; c < 3; ++c) {
    const double sz = __dsub_rn(bmax[c], bmin[c]);
    const double q = __dadd_rn(__ddiv_rn(__dadd_rn(sz, d_max), cell_size), 1.0);
    const int ncd_c = (q < 2147483647.0) ? (int)q : 2147483647;
    ncd[c] = (uint32_t)ncd_c;
    n_cells *= (uint64_t)(uint32_t)ncd_c;
  }
  return n_cells;
}

// ------------------------------------------------------------------ AABB --
__global__ void __launch_bounds__(kBlock) k_rb_aabb(DevBuf b, StepConst sc) {
  Ctl* ctl = b.ctl;
  if (rb_off(ctl)) return;
  __shared__ double sh_min[3][kBlock], sh_max[3][kBlock];
  const uint32_t f = blockIdx.x * blockDim.x + threadIdx.x;
  double lo[3] = {SHL_DBL_MAX, SHL_DBL_MAX, SHL_DBL_MAX}, hi[3] = {-SHL_DBL_MAX, -SHL_DBL_MAX, -SHL_DBL_MAX};
  if (f < sc.F) {
    for (int k = 0; k < 3; ++k) {
      const double* q = b.p + 3 * (size_t)b.tri[3 * (size_t)f + k];
      for (int c = 0; c < 3; ++c) {
        if (q[c] < lo[c]) lo[c] = q[c];
        if (q[c] > hi[c]) hi[c] = q[c];
      }
    }
    for (int c = 0; c < 3; ++c) {
      b.bmin[3 * (size_t)f + c] = lo[c];
      b.bmax[3 * (size_t)f + c] = hi[c];
    }
    // BoundingBox::max_size
    double dmax = __dsub_rn(hi[0], lo[0]);
    const double d1 = __dsub_rn(hi[1], lo[1]), d2 = __dsub_rn(hi[2], lo[2]);
    if (d1 > dmax) dmax = d1;
    if (d2 > dmax) dmax = d2;
    b.fsize[f] = dmax;
  }
  if (sc.n_cs) return;  // a batch: per-shell grids (k_rb_grids)
  for (int c = 0; c < 3; ++c) {
    sh_min[c][threadIdx.x] = lo[c];
    sh_max[c][threadIdx.x] = hi[c];
  }
  __syncthreads();
  for (int st = blockDim.x / 2; st > 0; st >>= 1) {
    if ((int)threadIdx.x < st)
      for (int c = 0; c < 3; ++c) {
        sh_min[c][threadIdx.x] = fmin(sh_min[c][threadIdx.x], sh_min[c][threadIdx.x + st]);
        sh_max[c][threadIdx.x] = fmax(sh_max[c][threadIdx.x], sh_max[c][threadIdx.x + st]);
      }
    __syncthreads();
  }
  if (threadIdx.x == 0)
    for (int c = 0; c < 3; ++c) {
      b.partial[(size_t)blockIdx.x * 8 + c] = sh_min[c][0];
      b.partial[(size_t)blockIdx.x * 8 + 3 + c] = sh_max[c][0];
    }
}

// The shell's bounds, average element size and cell grid (ShellSystem.C:1910-1969)
// from k_rb_aabb's per-block bounds and face sizes.  The 1024 lanes of the
// fixed-order sum of shl_geom.h are added on kBoundsBlocks SMs (a lane's sum
// is a chain of F / 1024 FP64 additions: on one SM the 1024 chains took most of
// a pass's bounds step); the last block adds the lanes in the fixed tree and
// makes the grid.
constexpr int kBoundsBlocks = 16;
__global__ void __launch_bounds__(kBlock) k_rb_bounds(DevBuf b, StepConst sc, uint32_t n_parts) {
  Ctl* ctl = b.ctl;
  if (rb_off(ctl) || sc.n_cs) return;  // a batch: per-shell grids (k_rb_grids)
  __shared__ double sh_min[3][kBlock], sh_max[3][kBlock];
  __shared__ double lanes[SHL_SUM_LANES];
  {
    constexpr uint32_t per_block = SHL_SUM_LANES / kBoundsBlocks;
    const uint32_t l = blockIdx.x * per_block + threadIdx.x;
    if (threadIdx.x < per_block) {
      double acc = 0.0;
#pragma unroll 4
      for (uint32_t i = l; i < sc.F; i += SHL_SUM_LANES) acc = __dadd_rn(acc, __ldcg(&b.fsize[i]));
      b.sum_lanes[l] = acc;
    }
  }
  if (!last_block_rb(&ctl->cnt[5])) return;
  // shell bounds (exact min/max)
  for (int c = 0; c < 3; ++c) {
    double mn = SHL_DBL_MAX, mx = -SHL_DBL_MAX;
    for (uint32_t k = threadIdx.x; k < n_parts; k += blockDim.x) {
      mn = fmin(mn, __ldcg(&b.partial[(size_t)k * 8 + c]));
      mx = fmax(mx, __ldcg(&b.partial[(size_t)k * 8 + 3 + c]));
    }
    sh_min[c][threadIdx.x] = mn;
    sh_max[c][threadIdx.x] = mx;
  }
  __syncthreads();
  for (int st = blockDim.x / 2; st > 0; st >>= 1) {
    if ((int)threadIdx.x < st)
      for (int c = 0; c < 3; ++c) {
        sh_min[c][threadIdx.x] = fmin(sh_min[c][threadIdx.x], sh_min[c][threadIdx.x + st]);
        sh_max[c][threadIdx.x] = fmax(sh_max[c][threadIdx.x], sh_max[c][threadIdx.x + st]);
      }
    __syncthreads();
  }
  // avg_elem_size: the fixed-order sum of shl_geom.h (1024 lanes, then a tree)
  for (uint32_t l = threadIdx.x; l < SHL_SUM_LANES; l += blockDim.x) lanes[l] = __ldcg(&b.sum_lanes[l]);
  __syncthreads();
  for (uint32_t st = SHL_SUM_LANES / 2; st > 0; st >>= 1) {
    for (uint32_t l = threadIdx.x; l < st; l += blockDim.x) lanes[l] = __dadd_rn(lanes[l], lanes[l + st]);
    __syncthreads();
  }
  if (threadIdx.x != 0) return;
  ctl->du_sum = 0.0;
  for (int c = 0; c < 3; ++c) {
    ctl->bmin[c] = sh_min[c][0];
    ctl->bmax[c] = sh_max[c][0];
  }
  const double avg = __ddiv_rn(lanes[0], (double)sc.F);
  ctl->avg_elem_size = avg;
  const uint64_t n_cells = grid_setup(ctl->bmin, ctl->bmax, avg, sc.cell_size_mult, sc.cell_margin, sc.thickness,
                                      sc.smooth, &ctl->cell_size, &ctl->d_max, ctl->ncd);
  ctl->d2_max = __dmul_rn(ctl->d_max, ctl->d_max);
  if (n_cells > sc.n_cells_max) {
    atomicMax(&ctl->problem, (int)SHL_TOO_MANY_CELLS);
    ctl->rebuild = 0;
    return;
  }
  if (n_cells > sc.n_cells_cap) {
    set_error(ctl, SHL_ERR_CAPACITY);
    return;
  }
  ctl->n_cells = (uint32_t)n_cells;
  ctl->n_old = ctl->n_pairs;
  ctl->n_new = 0;
  ctl->n_rebuilds += 1;
}

// ------------------------------------------------------- batch grids --
// One block per shell of a batch with self-contact: the shell's bounds and
// average element size (the fixed-order sum of shl_geom.h over the shell's own
// faces, so every value equals that of the shell run alone), its cell size,
// d_max and cell counts.  Shells whose trigger did not fire keep their list.
__global__ void __launch_bounds__(kBlock) k_rb_grids(DevBuf b, StepConst sc) {
  Ctl* ctl = b.ctl;
  if (rb_off(ctl)) return;
  ShellCell& S = b.shc[blockIdx.x];
  if (!S.rebuild) {
    if (threadIdx.x == 0) S.n_cells = 0;
    return;
  }
  __shared__ double sh_min[3][kBlock], sh_max[3][kBlock];
  __shared__ double lanes[SHL_SUM_LANES];
  const uint32_t f0 = S.face_first, nf = S.face_end - S.face_first;
  double lo[3] = {SHL_DBL_MAX, SHL_DBL_MAX, SHL_DBL_MAX}, hi[3] = {-SHL_DBL_MAX, -SHL_DBL_MAX, -SHL_DBL_MAX};
  for (uint32_t i = threadIdx.x; i < nf; i += blockDim.x)
    for (int c = 0; c < 3; ++c) {
      lo[c] = fmin(lo[c], b.bmin[3 * (size_t)(f0 + i) + c]);
      hi[c] = fmax(hi[c], b.bmax[3 * (size_t)(f0 + i) + c]);
    }
  for (int c = 0; c < 3; ++c) {
    sh_min[c][threadIdx.x] = lo[c];
    sh_max[c][threadIdx.x] = hi[c];
  }
  lane_sums<SHL_SUM_LANES / kBlock>(b.fsize + f0, nf, lanes);
  __syncthreads();
  for (int st = blockDim.x / 2; st > 0; st >>= 1) {
    if ((int)threadIdx.x < st)
      for (int c = 0; c < 3; ++c) {
        sh_min[c][threadIdx.x] = fmin(sh_min[c][threadIdx.x], sh_min[c][threadIdx.x + st]);
        sh_max[c][threadIdx.x] = fmax(sh_max[c][threadIdx.x], sh_max[c][threadIdx.x + st]);
      }
    __syncthreads();
  }
  for (uint32_t st = SHL_SUM_LANES / 2; st > 0; st >>= 1) {
    for (uint32_t l = threadIdx.x; l < st; l += blockDim.x) lanes[l] = __dadd_rn(lanes[l], lanes[l + st]);
    __syncthreads();
  }
  if (threadIdx.x != 0) return;
  S.du_sum = 0.0;
  for (int c = 0; c < 3; ++c) {
    S.bmin[c] = sh_min[c][0];
    S.bmax[c] = sh_max[c][0];
  }
  const double avg = __ddiv_rn(lanes[0], (double)nf);
  S.avg_elem_size = avg;
  const uint64_t n_cells = grid_setup(S.bmin, S.bmax, avg, S.cell_size_mult, sc.cell_margin, S.thickness, sc.smooth,
                                      &S.cell_size, &S.d_max, S.ncd);
  S.d2_max = __dmul_rn(S.d_max, S.d_max);
  S.n_rebuilds += 1;
  if (n_cells > S.n_cells_max) {
    atomicMax(&ctl->problem, (int)SHL_TOO_MANY_CELLS);
    ctl->rebuild = 0;
    S.n_cells = 0;
    return;
  }
  S.n_cells = n_cells > sc.n_cells_cap ? sc.n_cells_cap + 1u : (uint32_t)n_cells;
}

// first cell of each shell's grid (exclusive scan over the shells), the pass's
// cell count and the list counters (one block)
__global__ void __launch_bounds__(1024) k_rb_grid_scan(DevBuf b, StepConst sc) {
  Ctl* ctl = b.ctl;
  if (rb_off(ctl)) return;
  const uint32_t n = sc.n_cs;
  const uint32_t per = (n + blockDim.x - 1) / blockDim.x;
  const uint32_t s0 = threadIdx.x * per;
  uint64_t tot = 0;
  for (uint32_t k = 0; k < per; ++k)
    if (s0 + k < n) tot += b.shc[s0 + k].n_cells;
  __shared__ unsigned long long sh[1024];
  sh[threadIdx.x] = tot;
  __syncthreads();
  for (uint32_t o = 1; o < blockDim.x; o <<= 1) {
    const unsigned long long y = threadIdx.x >= o ? sh[threadIdx.x - o] : 0ull;
    __syncthreads();
    sh[threadIdx.x] += y;
    __syncthreads();
  }
  uint64_t run = sh[threadIdx.x] - tot;
  for (uint32_t k = 0; k < per; ++k)
    if (s0 + k < n) {
      ShellCell& S = b.shc[s0 + k];
      S.cell_base = run < 0xFFFFFFFFull ? (uint32_t)run : 0xFFFFFFFFu;
      run += S.n_cells;
    }
  if (threadIdx.x != blockDim.x - 1) return;
  const unsigned long long all = sh[blockDim.x - 1];
  if (all > sc.n_cells_cap) {
    set_error(ctl, SHL_ERR_CAPACITY);
    return;
  }
  ctl->n_cells = (uint32_t)all;
  ctl->n_old = ctl->n_pairs;
  ctl->n_new = 0;
  ctl->n_rebuilds += 1;
}

// ---------------------------------------------------------------- clear --
__global__ void k_rb_clear(DevBuf b, StepConst sc) {
  Ctl* ctl = b.ctl;
  if (rb_off(ctl)) return;
  const uint32_t n_cells = ctl->n_cells;
  const uint32_t stride = gridDim.x * blockDim.x;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n_cells; i += stride) {
    b.cell_count[i] = 0;
    b.cell_fill[i] = 0;
  }
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < sc.F; i += stride) {
    b.seg_count[i] = 0;
    b.new_cnt[i] = 0;
    b.new_fill[i] = 0;
  }
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < 3 * sc.V; i += stride) b.p32[i] = (float)b.p[i];
  if (blockIdx.x == 0 && threadIdx.x == 0) ctl->n_cand = 0;
}

// cell index range of face f on axis c (ShellSystem.C:1982-1983)
__device__ __forceinline__ void cell_range(const DevBuf& b, const GridView& g, uint32_t f, int* lo, int* hi) {
  const double cs = g.cell_size, dm = g.d_max;
  for (int c = 0; c < 3; ++c) {
    lo[c] = (int)__ddiv_rn(__dsub_rn(b.bmin[3 * (size_t)f + c], g.bmin[c]), cs);
    hi[c] = (int)__ddiv_rn(__dadd_rn(__dsub_rn(b.bmax[3 * (size_t)f + c], g.bmin[c]), dm), cs);
  }
}

// ---------------------------------------------------------------- count --
// one face t < F (cell ranges, histogram) or one old pair j = t - F (keep flag)
__device__ __forceinline__ void rb_count_one(const DevBuf& b, const StepConst& sc, const Ctl* ctl, uint32_t t) {
  if (t < sc.F) {
    if (!face_in_pass(b, sc, t)) return;
    const GridView g = grid_of(b, sc, t);
    int lo[3], hi[3];
    cell_range(b, g, t, lo, hi);
    for (int c = 0; c < 3; ++c) {
      b.cell_lo[3 * (size_t)t + c] = lo[c];
      b.cell_hi[3 * (size_t)t + c] = hi[c];
    }
    const uint32_t ny = g.ny, nz = g.nz;
    for (int cx = lo[0]; cx <= hi[0]; ++cx)
      for (int cy = lo[1]; cy <= hi[1]; ++cy)
        for (int cz = lo[2]; cz <= hi[2]; ++cz) {
          const uint32_t cell = g.base + (uint32_t)cx * ny * nz + (uint32_t)cy * nz + (uint32_t)cz;
          atomicAdd(&b.cell_count[cell], 1u);
        }
    return;
  }
  const uint32_t j = t - sc.F;
  if (j < ctl->n_old) {
    // ShellSystem.C:2020: drop unless sticking or still within d_max; a shell
    // of a batch that is not rebuilt keeps its whole list
    const uint32_t e1 = b.pe1[0][j];
    const bool keep = !face_in_pass(b, sc, e1) || b.pstick[0][j] != 0 || !(b.pd2[0][j] > grid_of(b, sc, e1).d2_max);
    b.pkeep[j] = keep ? 1 : 0;
    if (keep) atomicAdd(&b.seg_count[b.pe1[0][j]], 1u);
  }
}

__global__ void __launch_bounds__(kBlock) k_rb_count(DevBuf b, StepConst sc) {
  Ctl* ctl = b.ctl;
  if (rb_off(ctl)) return;
  const uint32_t n_all = sc.F + ctl->n_old;
  for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < n_all; t += gridDim.x * blockDim.x)
    rb_count_one(b, sc, ctl, t);
}

// ----------------------------------------------------------------- scan --
// Exclusive scan of in[0..n) into out[0..n) (+ out[n] = total if with_end),
// gated by *gate; two launches, fixed grids sized by capacity.
__global__ void __launch_bounds__(kBlock) k_scan_tiles(const uint32_t* gate, const Ctl* ctl, const uint32_t* in,
                                                       uint32_t* out, const uint32_t* n_ptr, uint32_t n_const,
                                                       uint32_t* tile_sums) {
  if (*gate == 0 || ctl->halted) return;
  const uint32_t n = n_ptr ? *n_ptr : n_const;
  const uint32_t base = blockIdx.x * kScanTile;
  if (base >= n) return;
  constexpr int PER = kScanTile / kBlock;
  uint32_t v[PER];
  uint32_t sum = 0;
  const uint32_t i0 = base + threadIdx.x * PER;
#pragma unroll
  for (int k = 0; k < PER; ++k) {
    const uint32_t x = (i0 + k < n) ? in[i0 + k] : 0u;
    v[k] = sum;
    sum += x;
  }
  // exclusive scan of the per-thread sums over the block
  __shared__ uint32_t wsum[kBlock / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t incl = sum;
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += y;
  }
  if (lane == 31) wsum[warp] = incl;
  __syncthreads();
  if (warp == 0) {
    uint32_t w = (lane < kBlock / 32) ? wsum[lane] : 0u;
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += y;
    }
    if (lane < kBlock / 32) wsum[lane] = w;
  }
  __syncthreads();
  const uint32_t excl = incl - sum + (warp > 0 ? wsum[warp - 1] : 0u);
#pragma unroll
  for (int k = 0; k < PER; ++k)
    if (i0 + k < n) out[i0 + k] = v[k] + excl;
  if (threadIdx.x == kBlock - 1) tile_sums[blockIdx.x] = excl + sum;
}

// Each tile's offset is the sum of the tiles before it, added up by the tile's
// own block (a few hundred tile sums at most); block 0 adds all of them: the
// total, out[n] and the capacity check.
__global__ void __launch_bounds__(kBlock) k_scan_add(const uint32_t* gate, Ctl* ctl, uint32_t* out,
                                                     const uint32_t* n_ptr, uint32_t n_const,
                                                     const uint32_t* tile_sums, uint32_t* total, int with_end,
                                                     uint32_t cap, int cap_error) {
  if (*gate == 0 || ctl->halted) return;
  const uint32_t n = n_ptr ? *n_ptr : n_const;
  const uint32_t base = blockIdx.x * kScanTile;
  if (blockIdx.x != 0 && base >= n) return;
  const uint32_t upto = blockIdx.x == 0 ? (n + kScanTile - 1) / kScanTile : blockIdx.x;
  uint32_t s = 0;
  for (uint32_t t = threadIdx.x; t < upto; t += blockDim.x) s += tile_sums[t];
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  __shared__ uint32_t wsum[kBlock / 32];
  __shared__ uint32_t offset;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) wsum[warp] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    uint32_t t = 0;
    for (int w = 0; w < kBlock / 32; ++w) t += wsum[w];
    offset = t;
  }
  __syncthreads();
  const uint32_t add = offset;
  if (blockIdx.x == 0) {
    if (threadIdx.x == 0) {
      *total = add;
      if (with_end) out[n] = add;
      if (cap_error && add > cap) {
        atomicMax(&ctl->error, (int)SHL_ERR_CAPACITY);
        ctl->rebuild = 0;
        ctl->csr_dirty = 0;
      }
    }
    return;
  }
  for (uint32_t i = base + threadIdx.x; i < base + kScanTile && i < n; i += blockDim.x) out[i] += add;
}

void launch_scan(const uint32_t* gate, Ctl* ctl, const uint32_t* in, uint32_t* out, const uint32_t* n_ptr,
                 uint32_t n_const, uint32_t n_cap, uint32_t* tile_sums, uint32_t* total, bool with_end,
                 uint32_t cap, bool cap_error, cudaStream_t s) {
  const uint32_t nt = (n_cap + kScanTile - 1) / kScanTile;
  const uint32_t grid = nt > 0 ? nt : 1;
  k_scan_tiles<<<grid, kBlock, 0, s>>>(gate, ctl, in, out, n_ptr, n_const, tile_sums);
  k_scan_add<<<grid, kBlock, 0, s>>>(gate, ctl, out, n_ptr, n_const, tile_sums, total, with_end ? 1 : 0, cap,
                                     cap_error ? 1 : 0);
}

// ----------------------------------------------------------------- fill --
__global__ void __launch_bounds__(kBlock) k_rb_fill(DevBuf b, StepConst sc) {
  Ctl* ctl = b.ctl;
  if (rb_off(ctl)) return;
  const uint32_t f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= sc.F || !face_in_pass(b, sc, f)) return;
  int lo[3], hi[3];
  for (int c = 0; c < 3; ++c) {
    lo[c] = b.cell_lo[3 * (size_t)f + c];
    hi[c] = b.cell_hi[3 * (size_t)f + c];
  }
  const GridView g = grid_of(b, sc, f);
  const uint32_t ny = g.ny, nz = g.nz;
  for (int cx = lo[0]; cx <= hi[0]; ++cx)
    for (int cy = lo[1]; cy <= hi[1]; ++cy)
      for (int cz = lo[2]; cz <= hi[2]; ++cz) {
        const uint32_t cell = g.base + (uint32_t)cx * ny * nz + (uint32_t)cy * nz + (uint32_t)cz;
        const uint32_t pos = b.cell_start[cell] + atomicAdd(&b.cell_fill[cell], 1u);
        b.cell_items[pos] = f;
        b.entry_cell[pos] = cell;
      }
}

__device__ __forceinline__ bool sorted_contains(const uint32_t* a, uint32_t lo, uint32_t hi, uint32_t x) {
  while (lo < hi) {
    const uint32_t mid = (lo + hi) >> 1;
    const uint32_t y = a[mid];
    if (y == x) return true;
    if (y < x) lo = mid + 1; else hi = mid;
  }
  return false;
}

// index of x in a[lo..hi), or hi if absent
__device__ __forceinline__ uint32_t sorted_find(const uint32_t* a, uint32_t lo, uint32_t hi, uint32_t x) {
  const uint32_t end = hi;
  while (lo < hi) {
    const uint32_t mid = (lo + hi) >> 1;
    const uint32_t y = a[mid];
    if (y == x) return mid;
    if (y < x) lo = mid + 1; else hi = mid;
  }
  return end;
}

// ---------------------------------------------------------------- pairs --
// Conservative separating-axis tests in FP32 on FP32 copies of the positions:
// true only when the triangles are certainly farther apart than d_max.  For an
// axis a (any vector, unnormalised, |a| = L) the projections of the two
// triangles onto a are separated by more than d_max L, allowing for the
// rounding of the FP32 projections (including the rounding of the positions to
// FP32): at most 32 eps32 L S with S the largest coordinate magnitude.  The
// remaining relative margin (1e-5) is far above the rounding of the FP64
// closest-point solve, so a pair rejected here is one the exact path would
// reject too (d^2 > d_max^2).  The axes: the line of centroids, the two face
// normals and the in-plane normals of the six edges (n x e), which separate
// neighbouring, nearly coplanar faces of a smooth surface.
__device__ __forceinline__ bool apart_on_axis(const float* a, const float* const* P1, const float* const* P2,
                                              float d_max, float S) {
  const float L2 = a[0] * a[0] + a[1] * a[1] + a[2] * a[2];
  if (!(L2 > 0.f)) return false;
  float mn1 = 3.0e38f, mx1 = -3.0e38f, mn2 = 3.0e38f, mx2 = -3.0e38f;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const float q1 = a[0] * P1[k][0] + a[1] * P1[k][1] + a[2] * P1[k][2];
    const float q2 = a[0] * P2[k][0] + a[1] * P2[k][1] + a[2] * P2[k][2];
    mn1 = fminf(mn1, q1);
    mx1 = fmaxf(mx1, q1);
    mn2 = fminf(mn2, q2);
    mx2 = fmaxf(mx2, q2);
  }
  const float L = sqrtf(L2);
  const float gap = fmaxf(mn2 - mx1, mn1 - mx2) - 32.f * 5.9604645e-8f * L * S;
  return gap > d_max * L * (1.f + 1e-5f);
}

// the line of centroids (S: the largest coordinate magnitude, for the next test)
__device__ __forceinline__ bool apart_centroids32(const float* const* P1, const float* const* P2, float d_max,
                                                  float& S) {
  float d[3];
  S = 0.f;
  for (int c = 0; c < 3; ++c) {
    d[c] = (P2[0][c] + P2[1][c] + P2[2][c]) - (P1[0][c] + P1[1][c] + P1[2][c]);
    for (int k = 0; k < 3; ++k) S = fmaxf(S, fmaxf(fabsf(P1[k][c]), fabsf(P2[k][c])));
  }
  return apart_on_axis(d, P1, P2, d_max, S);
}

// the face normals and the in-plane edge normals
__device__ __forceinline__ bool apart_faces32(const float* const* P1, const float* const* P2, float d_max, float S) {
  const float* const* T[2] = {P1, P2};
#pragma unroll
  for (int t = 0; t < 2; ++t) {
    const float* const* P = T[t];
    float e[3][3];
#pragma unroll
    for (int k = 0; k < 3; ++k)
#pragma unroll
      for (int c = 0; c < 3; ++c) e[k][c] = P[(k + 1) % 3][c] - P[k][c];
    const float n[3] = {e[0][1] * e[2][2] - e[0][2] * e[2][1], e[0][2] * e[2][0] - e[0][0] * e[2][2],
                        e[0][0] * e[2][1] - e[0][1] * e[2][0]};
    if (apart_on_axis(n, P1, P2, d_max, S)) return true;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      const float m[3] = {n[1] * e[k][2] - n[2] * e[k][1], n[2] * e[k][0] - n[0] * e[k][2],
                          n[0] * e[k][1] - n[1] * e[k][0]};
      if (apart_on_axis(m, P1, P2, d_max, S)) return true;
    }
  }
  return false;
}

// Candidate pairs of one (cell, face) entry: faces e2 > e1 in the cell, emitted
// from the lowest shared cell only, not topologically close, not in the kept
// list, not AABB-apart by d_max (ShellSystem.C:2047-2060), and not certainly
// apart by the separating-axis tests.  Buffered per thread, appended with one
// atomic per flush.
__global__ void __launch_bounds__(kBlock, 4) k_rb_cand(DevBuf b, StepConst sc) {
  Ctl* ctl = b.ctl;
  if (rb_off(ctl)) return;
  const uint32_t n_entries = ctl->n_entries;
  const uint32_t stride = gridDim.x * blockDim.x;
  constexpr int kBuf = 8;
  uint32_t buf1[kBuf], buf2[kBuf];
  int nb = 0;
  auto flush = [&]() {
    if (nb == 0) return;
    const uint32_t off = atomicAdd(&ctl->n_cand, (uint32_t)nb);
    if (off + nb > sc.cand_cap) {
      set_error(ctl, SHL_ERR_CAPACITY);
    } else {
      for (int q = 0; q < nb; ++q) {
        b.cand_e1[off + q] = buf1[q];
        b.cand_e2[off + q] = buf2[q];
      }
    }
    nb = 0;
  };
  for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < n_entries; j += stride) {
    const uint32_t e1 = b.cell_items[j];
    const GridView g = grid_of(b, sc, e1);
    const uint32_t ny = g.ny, nz = g.nz;
    const double d_max = g.d_max;
    const float d_max32 = (float)d_max;
    const uint32_t cell = b.entry_cell[j];
    const uint32_t local = cell - g.base;
    const uint32_t cz = local % nz, cy = (local / nz) % ny, cx = local / (nz * ny);
    const int* lo1 = b.cell_lo + 3 * (size_t)e1;
    const int l10 = lo1[0], l11 = lo1[1], l12 = lo1[2];
    const uint32_t c0 = b.close_ptr[e1], c1 = b.close_ptr[e1 + 1];
    const uint32_t o0 = b.pair_ptr[0][e1], o1 = b.pair_ptr[0][e1 + 1];
    double mn1[3], mx1[3];
    const float* Q1[3];
    uint32_t t1[3];
    for (int c = 0; c < 3; ++c) {
      mn1[c] = b.bmin[3 * (size_t)e1 + c];
      mx1[c] = b.bmax[3 * (size_t)e1 + c];
      t1[c] = b.tri[3 * (size_t)e1 + c];
      Q1[c] = b.p32 + 3 * (size_t)t1[c];
    }
    const uint32_t s0 = b.cell_start[cell], cnt = b.cell_count[cell];
    // The filters are conjunctive, so their order leaves the result unchanged;
    // the cheap and decisive ones come first.
    for (uint32_t k = 0; k < cnt; ++k) {
      const uint32_t e2 = b.cell_items[s0 + k];
      if (e2 <= e1) continue;
      const int* lo2 = b.cell_lo + 3 * (size_t)e2;
      if ((uint32_t)max(l10, lo2[0]) != cx || (uint32_t)max(l11, lo2[1]) != cy || (uint32_t)max(l12, lo2[2]) != cz)
        continue;
      // faces sharing a node are neighbours in the mesh, always in the close list (ShellSystem.C:657-678)
      uint32_t t2[3];
      for (int q = 0; q < 3; ++q) t2[q] = b.tri[3 * (size_t)e2 + q];
      bool shared = false;
      for (int q = 0; q < 3; ++q) shared = shared || t2[q] == t1[0] || t2[q] == t1[1] || t2[q] == t1[2];
      if (shared) continue;
      bool apart = false;
      for (int c = 0; c < 3; ++c) {
        const double mn2 = b.bmin[3 * (size_t)e2 + c], mx2 = b.bmax[3 * (size_t)e2 + c];
        apart = apart || mn1[c] > __dadd_rn(mx2, d_max) || mn2 > __dadd_rn(mx1[c], d_max);
      }
      if (apart) continue;
      const float* Q2[3];
      float S = 0.f;
      if (!sc.smooth) {  // facet bounds; SMOOTH distances are between limit surfaces
        for (int q = 0; q < 3; ++q) Q2[q] = b.p32 + 3 * (size_t)t2[q];
        if (apart_centroids32(Q1, Q2, d_max32, S)) continue;
      }
      if (!sc.smooth && apart_faces32(Q1, Q2, d_max32, S)) continue;
      if (sorted_contains(b.close_list, c0, c1, e2)) continue;
      const uint32_t at = sorted_find(b.pe2[0], o0, o1, e2);
      if (at < o1 && b.pkeep[at]) continue;
      buf1[nb] = e1;
      buf2[nb] = e2;
      if (++nb == kBuf) flush();
    }
  }
  flush();
}

// the acceptance of a candidate at squared distance d2 (ShellSystem.C:2082)
__device__ __forceinline__ void narrow_accept(const DevBuf& b, const StepConst& sc, Ctl* ctl, uint32_t i, uint32_t e1,
                                              double d2) {
  const double d2_max = sc.n_cs ? b.shc[b.face_shell[e1]].d2_max : ctl->d2_max;
  if (d2 <= 0.0) atomicMax(&ctl->problem, (int)SHL_CONTACT_PROBLEM);
  const bool ok = !(d2 > d2_max);
  b.cand_d2[i] = d2;
  b.cand_ok[i] = ok ? 1 : 0;
  if (ok) {
    atomicAdd(&b.new_cnt[e1], 1u);
    atomicAdd(&b.seg_count[e1], 1u);
  }
}

// closest-point test of each candidate (rounded operation by operation)
__global__ void __launch_bounds__(kBlock) k_rb_narrow(DevBuf b, StepConst sc) {
  Ctl* ctl = b.ctl;
  if (rb_off(ctl)) return;
  const uint32_t n = min(ctl->n_cand, sc.cand_cap);
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const uint32_t e1 = b.cand_e1[i], e2 = b.cand_e2[i];
    const double* P1[3];
    const double* P2[3];
    for (int q = 0; q < 3; ++q) {
      P1[q] = b.p + 3 * (size_t)b.tri[3 * (size_t)e1 + q];
      P2[q] = b.p + 3 * (size_t)b.tri[3 * (size_t)e2 + q];
    }
    shl_pair_geom g;
    shl_pair_compute(P1, P2, &g);
    narrow_accept(b, sc, ctl, i, e1, g.d2);
  }
}

// the power form of each regular patch at the current positions (irregular
// patches are evaluated from their subdivision tables in the search)
__global__ void __launch_bounds__(kBlock) k_limit_coeffs(DevBuf b, StepConst sc, bool rebuild) {
  const Ctl* ctl = b.ctl;
  if (rebuild ? rb_off(ctl) : (ctl->halted != 0 || ctl->paused != 0)) return;
  for (uint32_t e = blockIdx.x * blockDim.x + threadIdx.x; e < sc.F; e += gridDim.x * blockDim.x) {
    if ((b.fsm[e] & 0xff) != 6) continue;
    shl_limit_patch lp;
    smooth_patch(b, sc, e, lp);
    double P[15][3];
    shl_limit_coeffs_regular(&lp, P);
    double* out = b.lcoef + SHL_LIMIT_NCOEF * (size_t)e;
    for (int m = 0; m < 15; ++m)
      for (int c = 0; c < 3; ++c) out[3 * m + c] = P[m][c];
  }
}

// a patch's limit surface at (v, w): the stored power form of a regular patch
__device__ __forceinline__ void limit_at(const DevBuf& b, uint32_t e, const shl_limit_patch& lp, double v, double w,
                                         int order, double out[6][3]) {
  if (lp.N == 6)
    shl_limit_poly(reinterpret_cast<const double(*)[3]>(b.lcoef + SHL_LIMIT_NCOEF * (size_t)e), v, w, order, 1.0, out);
  else
    shl_limit_eval(&lp, v, w, order, out);
}

// SMOOTH closest-point searches with lane refill.  A search takes from one to
// several hundred limit evaluations (most of a squashed shell's pairs end after
// one to three, a few run the line search to its limit), so one thread per
// pair would hold each warp until its longest search ends.  Here each lane
// runs its search as a resumable state (shl_smooth_state): per trip a warp
// evaluates one point of both limit patches per lane and advances the
// searches, and a lane whose search has ended takes the next pair from a queue
// shared by the grid (ctl->cnt[7]; the last warp to leave resets it), so that
// the lanes stay busy until the queue is empty.  A search's result does not
// depend on the lane or the order that runs it.
//   REBUILD: the candidates of a linked-cell pass, each from (1/3, 1/3, 1/3,
//   1/3) as a new SmoothShellShellContact (SmoothShellShellContact.C:9-14),
//   then k_rb_narrow's acceptance;
//   else: the pairs of the list from their previous solution; x, d2 and
//   dc = p2 - p1 go to pvw, pd2 and the pair's force slots 0-2 for
//   k_contact_force.
constexpr int kSearchBlock = 128;
template <bool REBUILD>
__global__ void __launch_bounds__(kSearchBlock) k_smooth_search(DevBuf b, StepConst sc) {
  Ctl* ctl = b.ctl;
  uint32_t* queue = &ctl->cnt[7];
  uint32_t* left = &ctl->cnt[8];
  const bool off = REBUILD ? rb_off(ctl) : (ctl->halted != 0 || ctl->paused != 0);
  const uint32_t n = off ? 0u : (REBUILD ? min(ctl->n_cand, sc.cand_cap) : ctl->n_pairs);
  const unsigned lane = threadIdx.x & 31u;
  const unsigned below = (1u << lane) - 1u;
  bool busy = false, more = n > 0;
  uint32_t j = 0, e1 = 0, e2 = 0;
  shl_limit_patch A, B;
  shl_smooth_state st;
  for (;;) {
    const unsigned idle = __ballot_sync(0xffffffffu, !busy);
    if (more && idle) {
      const int leader = __ffs(idle) - 1;
      const uint32_t want = (uint32_t)__popc(idle);
      uint32_t base = 0;
      if ((int)lane == leader) base = atomicAdd(queue, want);
      base = __shfl_sync(0xffffffffu, base, leader);
      if (!(base + want < n)) more = false;  // the queue is empty for every warp
      if (!busy) {
        const uint32_t i = base + (uint32_t)__popc(idle & below);
        if (i < n) {
          busy = true;
          j = i;
          double x0[4];
          if (REBUILD) {
            e1 = b.cand_e1[i];
            e2 = b.cand_e2[i];
            for (int k = 0; k < 4; ++k) x0[k] = 1.0 / 3.0;
          } else {
            e1 = b.pe1[0][i];
            e2 = b.pe2[0][i];
            for (int k = 0; k < 4; ++k) x0[k] = b.pvw[0][4 * (size_t)i + k];
          }
          smooth_patch(b, sc, e1, A);
          smooth_patch(b, sc, e2, B);
          shl_smooth_start(&st, x0);
        }
      }
    }
    if (!__any_sync(0xffffffffu, busy)) break;
    if (busy) {
      const double* pt = shl_smooth_point(&st);
      const int order = shl_smooth_order(&st);
      double ev1[6][3], ev2[6][3];
      limit_at(b, e1, A, pt[0], pt[1], order, ev1);
      limit_at(b, e2, B, pt[2], pt[3], order, ev2);
      shl_smooth_take(&st, ev1, ev2);
      if (st.phase == SHL_SMOOTH_DONE) {
        busy = false;
        if (REBUILD) {
          for (int k = 0; k < 4; ++k) b.cand_x[4 * (size_t)j + k] = st.x[k];
          narrow_accept(b, sc, ctl, j, e1, st.f);
        } else {
          for (int k = 0; k < 4; ++k) b.pvw[0][4 * (size_t)j + k] = st.x[k];
          b.pd2[0][j] = st.f;
          double* out = b.pforce + kPairOut * (size_t)j;
          for (int c = 0; c < 3; ++c) out[c] = SHL_SUB(st.p2[c], st.p1[c]);
        }
      }
    }
  }
  if (lane == 0) {
    __threadfence();
    const uint32_t warps = gridDim.x * (kSearchBlock / 32);
    if (atomicAdd(left, 1u) == warps - 1) {
      atomicExch(queue, 0u);
      atomicExch(left, 0u);
    }
  }
}

// accepted candidates grouped by eid1 (counting sort; order inside a group is
// fixed later by the assembly)
__global__ void __launch_bounds__(kBlock) k_rb_scatter_new(DevBuf b, StepConst sc) {
  Ctl* ctl = b.ctl;
  if (rb_off(ctl)) return;
  const uint32_t n = min(ctl->n_cand, sc.cand_cap);
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    if (!b.cand_ok[i]) continue;
    const uint32_t e1 = b.cand_e1[i];
    const uint32_t pos = b.new_off[e1] + atomicAdd(&b.new_fill[e1], 1u);
    b.new_e2[pos] = b.cand_e2[i];
    b.new_d2[pos] = b.cand_d2[i];
    if (sc.smooth)
      for (int k = 0; k < 4; ++k) b.new_x[4 * (size_t)pos + k] = b.cand_x[4 * (size_t)i + k];
  }
}

// -------------------------------------------------------------- assemble --
// one face's segment of the new list, serially: the face's new pairs sorted
// by e2 in place (insertion sort), merged with its kept old pairs
__device__ void assemble_serial(const DevBuf& b, const StepConst& sc, uint32_t e1) {
  uint32_t dst = b.pair_ptr[1][e1];
  const uint32_t o0 = b.pair_ptr[0][e1], o1 = b.pair_ptr[0][e1 + 1];
  const uint32_t nn = b.new_cnt[e1];
  const uint32_t off = nn ? b.new_off[e1] : 0u;
  uint32_t* ne2 = b.new_e2 + off;
  double* nd2 = b.new_d2 + off;
  double* nx = sc.smooth ? b.new_x + 4 * (size_t)off : nullptr;
  for (uint32_t k = 1; k < nn; ++k) {
    const uint32_t x = ne2[k];
    const double d = nd2[k];
    double xs[4];
    if (nx)
      for (int c = 0; c < 4; ++c) xs[c] = nx[4 * k + c];
    uint32_t q = k;
    while (q > 0 && ne2[q - 1] > x) {
      ne2[q] = ne2[q - 1];
      nd2[q] = nd2[q - 1];
      if (nx)
        for (int c = 0; c < 4; ++c) nx[4 * q + c] = nx[4 * (q - 1) + c];
      --q;
    }
    ne2[q] = x;
    nd2[q] = d;
    if (nx)
      for (int c = 0; c < 4; ++c) nx[4 * q + c] = xs[c];
  }
  uint32_t io = o0, in = 0;
  for (;;) {
    while (io < o1 && !b.pkeep[io]) ++io;
    const bool have_old = io < o1, have_new = in < nn;
    if (!have_old && !have_new) break;
    const bool take_old = have_old && (!have_new || b.pe2[0][io] < ne2[in]);
    b.pe1[1][dst] = e1;
    if (take_old) {
      b.pe2[1][dst] = b.pe2[0][io];
      b.pstick[1][dst] = b.pstick[0][io];
      b.pd2[1][dst] = b.pd2[0][io];
      for (int c = 0; c < 3; ++c) b.porig[1][3 * (size_t)dst + c] = b.porig[0][3 * (size_t)io + c];
      if (nx)
        for (int c = 0; c < 4; ++c) b.pvw[1][4 * (size_t)dst + c] = b.pvw[0][4 * (size_t)io + c];
      ++io;
    } else {
      b.pe2[1][dst] = ne2[in];
      b.pstick[1][dst] = 0;
      b.pd2[1][dst] = nd2[in];
      for (int c = 0; c < 3; ++c) b.porig[1][3 * (size_t)dst + c] = 0.0;
      if (nx)
        for (int c = 0; c < 4; ++c) b.pvw[1][4 * (size_t)dst + c] = nx[4 * in + c];
      ++in;
    }
    ++dst;
  }
}

// The new list, face by face (segments of eid1): the kept old pairs (in e2
// order already) merged with the face's new pairs sorted by e2, a new pair
// before an old one of the same e2.  One warp per face: the new pairs' keys
// (e2, index) are sorted in shared memory (bitonic), and every pair's place
// follows from ranks, an old pair's = its rank among the kept old ones + the
// new pairs of e2 <= its e2, a new pair's = its rank among the new ones + the
// kept old pairs of e2 < its e2; the same list as the serial merge, which
// takes a face with more than kAsmCap old or new pairs.
constexpr int kAsmWarps = 4;
constexpr uint32_t kAsmCap = 512;
__global__ void __launch_bounds__(32 * kAsmWarps) k_rb_assemble(DevBuf b, StepConst sc) {
  Ctl* ctl = b.ctl;
  if (rb_off(ctl)) return;
  __shared__ unsigned long long skey[kAsmWarps][kAsmCap];
  __shared__ uint32_t skept[kAsmWarps][kAsmCap + 1];
  const uint32_t lane = threadIdx.x & 31u, w = threadIdx.x >> 5;
  unsigned long long* key = skey[w];
  uint32_t* kept = skept[w];
  // each warp reads the segments of 32 consecutive faces at once and merges
  // the faces that have old or new pairs, one after the other
  for (uint32_t fbase = (blockIdx.x * kAsmWarps + w) * 32; fbase < sc.F; fbase += gridDim.x * kAsmWarps * 32) {
    const uint32_t mine = fbase + lane;
    uint32_t my_o0 = 0, my_no = 0, my_nn = 0;
    if (mine < sc.F) {
      my_o0 = b.pair_ptr[0][mine];
      my_no = b.pair_ptr[0][mine + 1] - my_o0;
      my_nn = b.new_cnt[mine];
    }
    const bool big = my_nn > kAsmCap || my_no > kAsmCap;
    if (big) assemble_serial(b, sc, mine);
    unsigned todo = __ballot_sync(0xffffffffu, !big && (my_no > 0 || my_nn > 0));
    while (todo) {
      const int src = __ffs(todo) - 1;
      todo &= todo - 1;
      const uint32_t e1 = fbase + (uint32_t)src;
      const uint32_t o0 = __shfl_sync(0xffffffffu, my_o0, src);
      const uint32_t no = __shfl_sync(0xffffffffu, my_no, src);
      const uint32_t nn = __shfl_sync(0xffffffffu, my_nn, src);
      const uint32_t dst = b.pair_ptr[1][e1];
      const uint32_t off = nn ? b.new_off[e1] : 0u;
      // the new pairs' keys, sorted
      uint32_t P = 32;
      while (P < nn) P <<= 1;
      for (uint32_t i = lane; i < P; i += 32)
        key[i] = i < nn ? ((unsigned long long)b.new_e2[off + i] << 32) | i : ~0ull;
      __syncwarp();
      if (nn > 1)
        for (uint32_t k = 2; k <= P; k <<= 1)
          for (uint32_t j = k >> 1; j > 0; j >>= 1) {
            for (uint32_t t = lane; t < P / 2; t += 32) {
              const uint32_t i = ((t & ~(j - 1)) << 1) | (t & (j - 1));
              const unsigned long long x = key[i], y = key[i + j];
              if (((i & k) == 0) == (x > y)) {
                key[i] = y;
                key[i + j] = x;
              }
            }
            __syncwarp();
          }
      // kept old pairs before each old position (exclusive prefix count)
      uint32_t run = 0;
      for (uint32_t base = 0; base < no; base += 32) {
        const uint32_t i = base + lane;
        const bool kp = i < no && b.pkeep[o0 + i];
        const unsigned m = __ballot_sync(0xffffffffu, kp);
        if (i < no) kept[i] = run + (uint32_t)__popc(m & ((1u << lane) - 1u));
        run += (uint32_t)__popc(m);
      }
      if (lane == 0) kept[no] = run;
      __syncwarp();
      // kept old pairs
      for (uint32_t i = lane; i < no; i += 32) {
        const uint32_t io = o0 + i;
        if (!b.pkeep[io]) continue;
        const uint32_t x = b.pe2[0][io];
        uint32_t lo = 0, hi = nn;  // new pairs with e2 <= x
        while (lo < hi) {
          const uint32_t mid = (lo + hi) >> 1;
          if ((uint32_t)(key[mid] >> 32) <= x) lo = mid + 1;
          else hi = mid;
        }
        const uint32_t d = dst + kept[i] + lo;
        b.pe1[1][d] = e1;
        b.pe2[1][d] = x;
        b.pstick[1][d] = b.pstick[0][io];
        b.pd2[1][d] = b.pd2[0][io];
        for (int c = 0; c < 3; ++c) b.porig[1][3 * (size_t)d + c] = b.porig[0][3 * (size_t)io + c];
        if (sc.smooth)
          for (int c = 0; c < 4; ++c) b.pvw[1][4 * (size_t)d + c] = b.pvw[0][4 * (size_t)io + c];
      }
      // new pairs
      for (uint32_t r = lane; r < nn; r += 32) {
        const unsigned long long kr = key[r];
        const uint32_t x = (uint32_t)(kr >> 32), k = off + (uint32_t)(kr & 0xffffffffu);
        uint32_t lo = 0, hi = no;  // old pairs (kept or not) with e2 < x
        while (lo < hi) {
          const uint32_t mid = (lo + hi) >> 1;
          if (b.pe2[0][o0 + mid] < x) lo = mid + 1;
          else hi = mid;
        }
        const uint32_t d = dst + r + kept[lo];
        b.pe1[1][d] = e1;
        b.pe2[1][d] = x;
        b.pstick[1][d] = 0;
        b.pd2[1][d] = b.new_d2[k];
        for (int c = 0; c < 3; ++c) b.porig[1][3 * (size_t)d + c] = 0.0;
        if (sc.smooth)
          for (int c = 0; c < 4; ++c) b.pvw[1][4 * (size_t)d + c] = b.new_x[4 * (size_t)k + c];
      }
      __syncwarp();
    }
  }
}

__global__ void k_rb_copyback(DevBuf b, StepConst sc) {
  Ctl* ctl = b.ctl;
  if (rb_off(ctl)) return;
  const uint32_t n = ctl->n_next;
  const uint32_t stride = gridDim.x * blockDim.x;
  for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += stride) {
    b.pe1[0][j] = b.pe1[1][j];
    b.pe2[0][j] = b.pe2[1][j];
    b.pstick[0][j] = b.pstick[1][j];
    b.pd2[0][j] = b.pd2[1][j];
    for (int c = 0; c < 3; ++c) b.porig[0][3 * (size_t)j + c] = b.porig[1][3 * (size_t)j + c];
    if (sc.smooth)
      for (int c = 0; c < 4; ++c) b.pvw[0][4 * (size_t)j + c] = b.pvw[1][4 * (size_t)j + c];
  }
  for (uint32_t f = blockIdx.x * blockDim.x + threadIdx.x; f <= sc.F; f += stride) b.pair_ptr[0][f] = b.pair_ptr[1][f];
}

// flag flip after the copy-back (after all blocks are done); a batch also
// clears its shells' flags
__global__ void k_rb_finish(DevBuf b, StepConst sc) {
  Ctl* ctl = b.ctl;
  if (rb_off(ctl)) return;
  for (uint32_t s = threadIdx.x; s < sc.n_cs; s += blockDim.x) b.shc[s].rebuild = 0;
  __syncthreads();
  if (threadIdx.x != 0) return;
  ctl->n_pairs = ctl->n_next;
  ctl->rebuild = 0;
  ctl->csr_dirty = 1;
}

// ------------------------------------------------------------ contact CSR --
__device__ __forceinline__ bool csr_off(const Ctl* ctl) { return ctl->csr_dirty == 0 || ctl->halted != 0; }

__global__ void k_csr_clear(DevBuf b, StepConst sc) {
  if (csr_off(b.ctl)) return;
  if (blockIdx.x == 0 && threadIdx.x == 0) b.ctl->cnt[9] = 0;  // k_csr_sort's list of large nodes
  const uint32_t stride = gridDim.x * blockDim.x;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < sc.V; i += stride) {
    b.csr_count[i] = 0;
    b.csr_fill[i] = 0;
  }
}

__global__ void k_csr_count(DevBuf b, StepConst sc) {
  Ctl* ctl = b.ctl;
  if (csr_off(ctl)) return;
  const uint32_t n = ctl->n_pairs;
  const uint32_t stride = gridDim.x * blockDim.x;
  for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += stride) {
    const uint32_t e[2] = {b.pe1[0][j], b.pe2[0][j]};
    for (int r = 0; r < 6; ++r) atomicAdd(&b.csr_count[b.tri[3 * (size_t)e[r / 3] + r % 3]], 1u);
  }
}

__global__ void k_csr_fill(DevBuf b, StepConst sc) {
  Ctl* ctl = b.ctl;
  if (csr_off(ctl)) return;
  const uint32_t n = ctl->n_pairs;
  const uint32_t stride = gridDim.x * blockDim.x;
  for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += stride) {
    const uint32_t e[2] = {b.pe1[0][j], b.pe2[0][j]};
    for (int r = 0; r < 6; ++r) {
      const uint32_t nd = b.tri[3 * (size_t)e[r / 3] + r % 3];
      const uint32_t pos = b.csr_ptr[nd] + atomicAdd(&b.csr_fill[nd], 1u);
      b.csr_ent[pos] = j * 8u + (uint32_t)r;
    }
  }
}

// sort each node's entries (deterministic order for the gather): a bitonic
// sort of the entries padded to a power of two in shared memory, by one warp
// for a node of up to kCsrSortCap entries (a few hundred in a contact-heavy
// state, about a thousand with SMOOTH contact), by a block of k_csr_sort_big
// up to kCsrSortBigCap, in place by one thread beyond
constexpr int kCsrSortWarps = 4;
constexpr uint32_t kCsrSortCap = 2048;
constexpr uint32_t kCsrSortBigCap = 16384;
constexpr int kCsrSortBigBlock = 1024;

__device__ void csr_sort_serial(const DevBuf& b, uint32_t k0, uint32_t k1) {
  for (uint32_t k = k0 + 1; k < k1; ++k) {
    const uint32_t x = b.csr_ent[k];
    uint32_t q = k;
    while (q > k0 && b.csr_ent[q - 1] > x) {
      b.csr_ent[q] = b.csr_ent[q - 1];
      --q;
    }
    b.csr_ent[q] = x;
  }
}

// the nodes that k_csr_sort listed (in csr_fill, free after k_csr_fill; count in ctl->cnt[9])
__global__ void __launch_bounds__(kCsrSortBigBlock) k_csr_sort_big(DevBuf b, StepConst sc) {
  Ctl* ctl = b.ctl;
  if (csr_off(ctl)) return;
  extern __shared__ uint32_t big[];
  const uint32_t n_big = min(ctl->cnt[9], sc.V);
  for (uint32_t q = blockIdx.x; q < n_big; q += gridDim.x) {
    const uint32_t nd = b.csr_fill[q];
    const uint32_t k0 = b.csr_ptr[nd], k1 = b.csr_ptr[nd + 1];
    const uint32_t n = k1 - k0;
    if (n > kCsrSortBigCap) {
      if (threadIdx.x == 0) csr_sort_serial(b, k0, k1);
      __syncthreads();
      continue;
    }
    uint32_t P = kCsrSortCap;
    while (P < n) P <<= 1;
    for (uint32_t i = threadIdx.x; i < P; i += blockDim.x) big[i] = i < n ? b.csr_ent[k0 + i] : 0xffffffffu;
    __syncthreads();
    for (uint32_t k = 2; k <= P; k <<= 1)
      for (uint32_t j = k >> 1; j > 0; j >>= 1) {
        for (uint32_t t = threadIdx.x; t < P / 2; t += blockDim.x) {
          const uint32_t i = ((t & ~(j - 1)) << 1) | (t & (j - 1));
          const uint32_t x = big[i], y = big[i + j];
          if (((i & k) == 0) == (x > y)) {
            big[i] = y;
            big[i + j] = x;
          }
        }
        __syncthreads();
      }
    for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) b.csr_ent[k0 + i] = big[i];
    __syncthreads();
  }
}

__global__ void __launch_bounds__(32 * kCsrSortWarps) k_csr_sort(DevBuf b, StepConst sc) {
  Ctl* ctl = b.ctl;
  if (csr_off(ctl)) return;
  __shared__ uint32_t buf[kCsrSortWarps][kCsrSortCap];
  const uint32_t lane = threadIdx.x & 31u, w = threadIdx.x >> 5;
  uint32_t* sh = buf[w];
  // each warp reads the segments of 32 consecutive nodes at once and sorts the
  // ones with two or more entries; larger ones than the buffer go to the list
  for (uint32_t base = (blockIdx.x * kCsrSortWarps + w) * 32; base < sc.V; base += gridDim.x * kCsrSortWarps * 32) {
    const uint32_t me = base + lane;
    uint32_t k0 = 0, n = 0;
    if (me < sc.V) {
      k0 = b.csr_ptr[me];
      n = b.csr_ptr[me + 1] - k0;
    }
    if (n > kCsrSortCap) b.csr_fill[atomicAdd(&ctl->cnt[9], 1u)] = me;
    unsigned todo = __ballot_sync(0xffffffffu, n >= 2 && n <= kCsrSortCap);
    while (todo) {
      const int src = __ffs(todo) - 1;
      todo &= todo - 1;
      const uint32_t s0 = __shfl_sync(0xffffffffu, k0, src), sn = __shfl_sync(0xffffffffu, n, src);
      uint32_t P = 32;
      while (P < sn) P <<= 1;
      for (uint32_t i = lane; i < P; i += 32) sh[i] = i < sn ? b.csr_ent[s0 + i] : 0xffffffffu;
      __syncwarp();
      for (uint32_t k = 2; k <= P; k <<= 1)
        for (uint32_t j = k >> 1; j > 0; j >>= 1) {
          // compare-exchange t: the pair (i, i + j) with bit j of i clear
          for (uint32_t t = lane; t < P / 2; t += 32) {
            const uint32_t i = ((t & ~(j - 1)) << 1) | (t & (j - 1));
            const uint32_t x = sh[i], y = sh[i + j];
            if (((i & k) == 0) == (x > y)) {
              sh[i] = y;
              sh[i + j] = x;
            }
          }
          __syncwarp();
        }
      for (uint32_t i = lane; i < sn; i += 32) b.csr_ent[s0 + i] = sh[i];
      __syncwarp();
    }
  }
}

__global__ void k_csr_finish(DevBuf b) {
  if (csr_off(b.ctl)) return;
  b.ctl->csr_dirty = 0;
}

inline uint32_t nblk(uint32_t n, uint32_t bs = kBlock) { return n == 0 ? 1 : (n + bs - 1) / bs; }

}  // namespace

// a grid that the SMs hold at once (the queue hands out the pairs)
template <bool REBUILD>
static uint32_t search_grid() {
  static const uint32_t g = [] {
    int dev = 0, sms = 0, per_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_smooth_search<REBUILD>, kSearchBlock, 0);
    return (uint32_t)(sms > 0 ? sms : 152) * (uint32_t)(per_sm > 0 ? per_sm : 1);
  }();
  return g;
}

void launch_smooth_search(const DevBuf& b, const StepConst& sc, bool rebuild, cudaStream_t s) {
  uint32_t g = nblk(sc.F);
  if (g > 8 * 152) g = 8 * 152;
  k_limit_coeffs<<<g, kBlock, 0, s>>>(b, sc, rebuild);
  if (rebuild)
    k_smooth_search<true><<<search_grid<true>(), kSearchBlock, 0, s>>>(b, sc);
  else
    k_smooth_search<false><<<search_grid<false>(), kSearchBlock, 0, s>>>(b, sc);
}

// k_csr_sort_big takes more than the default 48 KB of shared memory; called
// once per device before its first launch
cudaError_t init_contact_kernels() {
  return cudaFuncSetAttribute((const void*)k_csr_sort_big, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)(kCsrSortBigCap * 4));
}

void launch_contact_csr(const DevBuf& b, const StepConst& sc, cudaStream_t s) {
  const uint32_t gV = nblk(sc.V);
  uint32_t gP = nblk(sc.pairs_cap);
  if (gP > 8 * 152) gP = 8 * 152;
  k_csr_clear<<<gV, kBlock, 0, s>>>(b, sc);
  k_csr_count<<<gP, kBlock, 0, s>>>(b, sc);
  launch_scan(&b.ctl->csr_dirty, b.ctl, b.csr_count, b.csr_ptr, nullptr, sc.V, sc.V, b.scan_block, &b.ctl->n_csr,
              true, sc.csr_cap, true, s);
  k_csr_fill<<<gP, kBlock, 0, s>>>(b, sc);
  {
    uint32_t g = (sc.V + 32 * kCsrSortWarps - 1) / (32 * kCsrSortWarps);
    if (g > 16 * 152) g = 16 * 152;
    k_csr_sort<<<g ? g : 1, 32 * kCsrSortWarps, 0, s>>>(b, sc);
    k_csr_sort_big<<<152, kCsrSortBigBlock, kCsrSortBigCap * 4, s>>>(b, sc);
  }
  k_csr_finish<<<1, 1, 0, s>>>(b);
}

void launch_rebuild(const DevBuf& b, const StepConst& sc, cudaStream_t s) {
  const uint32_t gF = nblk(sc.F);
  k_rb_aabb<<<gF, kBlock, 0, s>>>(b, sc);
  if (!sc.n_cs) k_rb_bounds<<<kBoundsBlocks, kBlock, 0, s>>>(b, sc, gF);
  if (sc.n_cs) {
    k_rb_grids<<<sc.n_cs, kBlock, 0, s>>>(b, sc);
    k_rb_grid_scan<<<1, 1024, 0, s>>>(b, sc);
  }
  {
    uint32_t g = nblk(sc.n_cells_cap > sc.F ? sc.n_cells_cap : sc.F);
    if (g > 16 * 152) g = 16 * 152;
    k_rb_clear<<<g, kBlock, 0, s>>>(b, sc);
  }
  {
    uint32_t g = nblk(sc.F + sc.pairs_cap);
    if (g > 16 * 152) g = 16 * 152;
    k_rb_count<<<g, kBlock, 0, s>>>(b, sc);
  }
  launch_scan(&b.ctl->rebuild, b.ctl, b.cell_count, b.cell_start, &b.ctl->n_cells, 0, sc.n_cells_cap, b.scan_block,
              &b.ctl->n_entries, false, sc.entries_cap, true, s);
  k_rb_fill<<<gF, kBlock, 0, s>>>(b, sc);
  {
    uint32_t g = nblk(sc.entries_cap);
    if (g > 16 * 152) g = 16 * 152;
    k_rb_cand<<<g, kBlock, 0, s>>>(b, sc);
    uint32_t gc = nblk(sc.cand_cap);
    if (gc > 16 * 152) gc = 16 * 152;
    if (sc.smooth)
      launch_smooth_search(b, sc, true, s);
    else
      k_rb_narrow<<<gc, kBlock, 0, s>>>(b, sc);
    launch_scan(&b.ctl->rebuild, b.ctl, b.new_cnt, b.new_off, nullptr, sc.F, sc.F, b.scan_block, &b.ctl->n_new,
                false, sc.pairs_cap, true, s);
    k_rb_scatter_new<<<gc, kBlock, 0, s>>>(b, sc);
  }
  launch_scan(&b.ctl->rebuild, b.ctl, b.seg_count, b.pair_ptr[1], nullptr, sc.F, sc.F, b.scan_block, &b.ctl->n_next,
              true, sc.pairs_cap, true, s);
  {
    uint32_t g = (sc.F + 32 * kAsmWarps - 1) / (32 * kAsmWarps);
    if (g > 16 * 152) g = 16 * 152;
    k_rb_assemble<<<g ? g : 1, 32 * kAsmWarps, 0, s>>>(b, sc);
  }
  {
    uint32_t g = nblk(sc.pairs_cap > sc.F + 1 ? sc.pairs_cap : sc.F + 1);
    if (g > 8 * 152) g = 8 * 152;
    k_rb_copyback<<<g, kBlock, 0, s>>>(b, sc);
  }
  k_rb_finish<<<1, sc.n_cs ? kBlock : 32, 0, s>>>(b, sc);
  launch_contact_csr(b, sc, s);
}

}  // namespace shl
