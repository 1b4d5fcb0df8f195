// Batched solves: hundreds of independent TeaLeaf problems of uneven size,
// each a single chunk, solved together with FP64 CG.
//
// Every problem keeps its own padded fields (one arena for the batch), its
// own reduction partials, completion counter and CG scalar state
// (ResState) in device memory.  One CG iteration of every still-active
// problem is three persistent grid-stride kernels over a flat work list of
// (problem, supertile) items, largest problems first:
//   k_b_calc_w   w = A p, p.w           (tea_leaf_cg_cl.cl:45-69)
//   k_b_calc_ur  u, r, z updates, r.z   (tea_leaf_cg_cl.cl:73-137)
//   k_b_calc_p   p = z + beta p         (tea_leaf_cg_cl.cl:141-160)
// The block that completes a problem's last supertile of a phase finishes
// that problem's sum in the fixed order of tea_device.cuh and, after
// calc_ur, takes its CG scalar step and exit test on the device
// (cg_scalar_step).  Items of problems that have stopped are skipped.  The
// phase boundaries are kernel boundaries, so no block ever waits for
// another.  Batches of iterations are replayed from a captured CUDA graph
// until no problem is active.
//
// Each problem's arithmetic, summation order and exit test are those of a
// single-chunk run of that problem, so its iteration counts and field
// summaries are bit-identical to it.  The autotuner (batch_autotune)
// chooses only the launch geometry, which does not change any result.
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <string>
#include <vector>

#include "../../include/tealeaf_gb300.h"
#include "tea_cg.cuh"

namespace tea {

// The batch's list of active problems, kept in device memory: plist holds
// the problems still iterating (largest first), ustart the prefix sums of
// their work units (ustart[j] = first unit of plist[j]), counts[0] the
// number of units and counts[1] the number of problems.  A work unit is a
// run of at most G consecutive supertiles of one problem.
struct WorkList {
  const int* plist;
  const int* ustart;
  const int* counts;
  int G;
};

// Minimum resident blocks per SM of the iteration kernels (a register cap).
// Measured on configuration 4: 2.59e10 cell-iterations/s without the bound,
// 2.70e10 / 2.63e10 / 2.56e10 with 4 / 6 / 8.
constexpr int kBatchMinBlocks = 4;

__device__ __forceinline__ int units_of(int ns, int G) { return (ns + G - 1) / G; }

// Position in the active list of the problem that owns unit u (every
// thread of the block computes the same value).
__device__ __forceinline__ int find_problem(const WorkList& wl, int np, int u) {
  int lo = 0, hi = np - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (__ldg(wl.ustart + mid) <= u)
      lo = mid;
    else
      hi = mid - 1;
  }
  return lo;
}

// Runs body(x, y0, xin, acc) for this warp's tile of supertile s of a
// problem and butterflies the NV sums (the inner part of tile_driver).
template <int NV, class Body>
__device__ __forceinline__ void run_supertile(const Dev& d, int s, double* acc,
                                              Body body) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int sy = s / d.nsx, sx = s - sy * d.nsx;
  const int tx = sx * kTilesPerSuper + warp;
#pragma unroll
  for (int v = 0; v < (NV > 0 ? NV : 1); v++) acc[v] = 0.0;
  if (tx < d.ntx) {
    const int x = tx * kTileW + lane;
    body(x, sy * d.th, x < d.x_max, acc);
    if (NV > 0) {
#pragma unroll
      for (int v = 0; v < NV; v++) acc[v] = bfly(acc[v]);
    }
  }
}

// The supertile partial sums of supertiles s0..s1-1 of a problem (one
// value), four supertiles at a time with the shared butterflies of
// tea_device.cuh (bfly4, supertile_partials4): the same sums as one
// run_supertile and supertile_partial per supertile.  sh holds 32 doubles.
template <class Body>
__device__ __forceinline__ void unit_partials(const Dev& d, const Red& red, int s0,
                                              int s1, double* sh, Body body) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int g = s0; g < s1; g += 4) {
    double tiles[4];
    int s_k[4];
#pragma unroll 1
    for (int k = 0; k < 4; k++) {
      double acc[1] = {0.0};
      const int s = g + k;
      if (s < s1) {
        const int sy = s / d.nsx, sx = s - sy * d.nsx;
        const int tx = sx * kTilesPerSuper + warp;
        if (tx < d.ntx) {
          const int x = tx * kTileW + lane;
          body(x, sy * d.th, x < d.x_max, acc);
        }
      }
#pragma unroll
      for (int q = 0; q < 4; q++)
        if (q == k) {
          tiles[q] = acc[0];
          s_k[q] = s < s1 ? s : d.ns;
        }
    }
    const double t = bfly4(tiles[0], tiles[1], tiles[2], tiles[3]);
    if ((lane & 7) == 0) sh[bfly4_slot(lane) * 8 + warp] = t;
    supertile_partials4<1>(red, s_k, d.ns, sh);
  }
}

// Counts one finished unit of a problem; true in the block that finished
// the problem's last one, which also resets the counter.
__device__ __forceinline__ bool unit_done(unsigned int* counter, int units,
                                          unsigned int* is_last) {
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) {
    const unsigned int t = atomicAdd(counter, 1u);
    *is_last = (t == (unsigned int)units - 1u) ? 1u : 0u;
    if (*is_last) *counter = 0u;
  }
  __syncthreads();
  if (*is_last) __threadfence();
  return *is_last != 0u;
}

// A double of the loop state written by another block of the same
// (persistent) launch is read through L2 (CG); plain otherwise.
template <bool CG>
__device__ __forceinline__ double st_load(const double* p) {
  return CG ? __ldcg(p) : *p;
}

// The three phases of one CG iteration over the block's work units.  The
// separate kernels below run one phase each; k_b_iterations runs them in
// turn with grid barriers between them (CG = true: fields and loop state
// written by other blocks in an earlier phase are read through L2).

// w = A p and p.w of every active problem (tea_leaf_cg_cl.cl:45-69); the
// finishing block stores pw in the problem's loop state.
template <int F, bool CG>
__device__ __forceinline__ void phase_w(const Dev* __restrict__ devs,
                                        const Red* __restrict__ reds, ResState* st,
                                        const WorkList& wl, int U, int np, double* sh,
                                        unsigned int* is_last) {
  for (int u = blockIdx.x; u < U; u += gridDim.x) {
    const int j = find_problem(wl, np, u);
    const int i = wl.plist[j];
    if (*(volatile int*)&st[i].stop) continue;
    const Dev d = devs[i];
    const Red red = reds[i];
    const int s0 = (u - wl.ustart[j]) * wl.G, s1 = min(s0 + wl.G, d.ns);
    unit_partials(d, red, s0, s1, sh, [&](int x, int y0, bool xin, double* a) {
      // the three-kernel mode takes the restrict-qualified bodies; the
      // persistent mode reads other blocks' writes through L2 (CG)
      if constexpr (CG) {
        if (d.th == 16)
          cg_w_tile<16, F, CG>(d, x, y0, xin, a);
        else
          cg_w_tile<4, F, CG>(d, x, y0, xin, a);
      } else {
        if (d.th == 16)
          cg_w_tile_r<16, F>(d, x, y0, xin, a);
        else
          cg_w_tile_r<4, F>(d, x, y0, xin, a);
      }
    });
    if (unit_done(red.counter, units_of(d.ns, wl.G), is_last)) {
      block_final_sum<1>(red.partials, red.stride, d.ns, red.result, sh);
      if (threadIdx.x == 0) {
        st[i].pw = red.result[0];
        __threadfence();
      }
      __syncthreads();
    }
  }
}

// u, r, z updates and r.z (tea_leaf_cg_cl.cl:73-137) with alpha = rro/pw;
// the finishing block takes the problem's scalar step and exit test.
template <int F, bool CG>
__device__ __forceinline__ void phase_ur(const Dev* __restrict__ devs,
                                         const Red* __restrict__ reds, ResState* st,
                                         const WorkList& wl, int U, int np, double* sh,
                                         unsigned int* is_last) {
  for (int u = blockIdx.x; u < U; u += gridDim.x) {
    const int j = find_problem(wl, np, u);
    const int i = wl.plist[j];
    if (*(volatile int*)&st[i].stop) continue;
    const Dev d = devs[i];
    const Red red = reds[i];
    const double alpha = st_load<CG>(&st[i].rro) / st_load<CG>(&st[i].pw);
    const int s0 = (u - wl.ustart[j]) * wl.G, s1 = min(s0 + wl.G, d.ns);
    unit_partials(d, red, s0, s1, sh, [&](int x, int y0, bool xin, double* a) {
      if constexpr (CG) {
        if (d.th == 16)
          cg_ur_tile<16, F, 1, CG>(d, x, y0, xin, a, alpha);
        else
          cg_ur_tile<4, F, 1, CG>(d, x, y0, xin, a, alpha);
      } else {
        if (d.th == 16)
          cg_ur_tile_r<16, F, 1>(d, x, y0, xin, a, alpha);
        else
          cg_ur_tile_r<4, F, 1>(d, x, y0, xin, a, alpha);
      }
    });
    if (unit_done(red.counter, units_of(d.ns, wl.G), is_last)) {
      block_final_sum<1>(red.partials, red.stride, d.ns, red.result, sh);
      if (threadIdx.x == 0) {
        cg_scalar_step<1>(&st[i], alpha, red.result);
        __threadfence();
      }
      __syncthreads();
    }
  }
}

// p = z + beta p (tea_leaf_cg_cl.cl:141-160) for every problem whose
// calc_ur has just run, including the iteration on which it stopped.
template <int F, bool CG>
__device__ __forceinline__ void phase_p(const Dev* __restrict__ devs,
                                        const Red* __restrict__ reds, ResState* st,
                                        const WorkList& wl, int U, int np,
                                        unsigned int* is_last) {
  for (int u = blockIdx.x; u < U; u += gridDim.x) {
    const int j = find_problem(wl, np, u);
    const int i = wl.plist[j];
    if (!*(volatile int*)&st[i].p_pending) continue;
    const Dev d = devs[i];
    const Red red = reds[i];
    const double beta = st_load<CG>(&st[i].beta);
    const int s0 = (u - wl.ustart[j]) * wl.G, s1 = min(s0 + wl.G, d.ns);
    for (int s = s0; s < s1; s++) {
      double acc[1];
      run_supertile<0>(d, s, acc, [&](int x, int y0, bool xin, double* a) {
        if (d.th == 16)
          cg_p_tile<16, F, CG>(d, x, y0, xin, beta);
        else
          cg_p_tile<4, F, CG>(d, x, y0, xin, beta);
      });
    }
    if (unit_done(red.counter, units_of(d.ns, wl.G), is_last)) {
      if (threadIdx.x == 0) {
        st[i].p_pending = 0;
        __threadfence();
      }
      __syncthreads();
    }
  }
}

template <int F>
__global__ void __launch_bounds__(kBlock, kBatchMinBlocks)
    k_b_calc_w(const Dev* __restrict__ devs, const Red* __restrict__ reds,
               ResState* st, WorkList wl) {
  __shared__ double sh[32];
  __shared__ unsigned int is_last;
  phase_w<F, false>(devs, reds, st, wl, wl.counts[0], wl.counts[1], sh, &is_last);
}

template <int F>
__global__ void __launch_bounds__(kBlock, kBatchMinBlocks)
    k_b_calc_ur(const Dev* __restrict__ devs, const Red* __restrict__ reds,
                ResState* st, WorkList wl) {
  __shared__ double sh[32];
  __shared__ unsigned int is_last;
  phase_ur<F, false>(devs, reds, st, wl, wl.counts[0], wl.counts[1], sh, &is_last);
}

template <int F>
__global__ void __launch_bounds__(kBlock, kBatchMinBlocks)
    k_b_calc_p(const Dev* __restrict__ devs, const Red* __restrict__ reds,
               ResState* st, WorkList wl) {
  __shared__ unsigned int is_last;
  phase_p<F, false>(devs, reds, st, wl, wl.counts[0], wl.counts[1], &is_last);
}

// `iters` CG iterations of every active problem in one cooperative launch:
// the three phases above with grid barriers between them (all blocks are
// resident).  The active list is fixed for the launch (problems that stop
// are skipped, as in the separate kernels); bar[0..1] is the barrier,
// bar[2] its error flag, set if a barrier times out, after which every
// block returns.  Results are those of the separate kernels.
template <int F>
__global__ void __launch_bounds__(kBlock, kBatchMinBlocks)
    k_b_iterations(const Dev* __restrict__ devs, const Red* __restrict__ reds,
                   ResState* st, WorkList wl, int iters, unsigned int* bar,
                   long long spin_limit) {
  __shared__ double sh[32];
  __shared__ unsigned int is_last;
  int* err = (int*)(bar + 2);
  const int U = wl.counts[0], np = wl.counts[1];
  for (int it = 0; it < iters; it++) {
    phase_w<F, true>(devs, reds, st, wl, U, np, sh, &is_last);
    if (!grid_barrier(bar, err, spin_limit)) return;
    phase_ur<F, true>(devs, reds, st, wl, U, np, sh, &is_last);
    if (!grid_barrier(bar, err, spin_limit)) return;
    phase_p<F, true>(devs, reds, st, wl, U, np, &is_last);
    if (!grid_barrier(bar, err, spin_limit)) return;
  }
}

// Exclusive prefix sum over a block of 1024 threads; *total gets the sum.
__device__ __forceinline__ int block_scan_1024(int v, int* total, int* sh32) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) sh32[warp] = x;
  __syncthreads();
  if (warp == 0) {
    int w = sh32[lane];
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += y;
    }
    sh32[lane] = w;  // inclusive sums of the warps
  }
  __syncthreads();
  const int before = warp > 0 ? sh32[warp - 1] : 0;
  *total = sh32[31];
  __syncthreads();
  return before + x - v;
}

// One block of 1024 threads, after every replay of the iteration kernels:
// drops the problems that have stopped from the active list (in place,
// keeping the order) and rebuilds the unit prefix sums and the counts.
__global__ void __launch_bounds__(1024)
    k_b_compact(const Dev* __restrict__ devs, const ResState* st, int* plist,
                int* ustart, int* counts, int G) {
  __shared__ int sh32[32];
  const int np = counts[1];
  int base_p = 0, base_u = 0;
  for (int c0 = 0; c0 < np; c0 += 1024) {
    const int j = c0 + (int)threadIdx.x;
    int i = -1, keep = 0, nu = 0;
    if (j < np) {
      i = plist[j];
      keep = st[i].stop ? 0 : 1;
      nu = keep ? units_of(devs[i].ns, G) : 0;
    }
    int tp = 0, tu = 0;
    const int ep = block_scan_1024(keep, &tp, sh32);
    const int eu = block_scan_1024(nu, &tu, sh32);
    // every read of this chunk happened before the first scan's barrier;
    // the writes land at positions below c0 + 1024
    if (keep) {
      plist[base_p + ep] = i;
      ustart[base_p + ep] = base_u + eu;
    }
    base_p += tp;
    base_u += tu;
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    ustart[base_p] = base_u;
    counts[0] = base_u;
    counts[1] = base_p;
  }
}

// Start of a solve: every problem active, in the given order, with its
// loop scalars as a single-chunk run has them at the top of its CG loop
// (tea_solve.f90:129-146): rro from cg_init, the exit threshold
// eps * sqrt(initial r.r) and iteration number 1.
__global__ void k_b_begin(ResState* st, const double* results, int n, double eps,
                          int loop_max, const int* order, const int* ustart_all,
                          int* plist, int* ustart, int* counts);

}  // namespace tea

namespace tea {

constexpr int kResults = 8;     // reduction results per problem
constexpr int kResInitial = 4;  // slot of the initial r.r

__global__ void k_b_begin(ResState* st, const double* results, int n, double eps,
                          int loop_max, const int* order, const int* ustart_all,
                          int* plist, int* ustart, int* counts) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j == 0) {
    ustart[n] = ustart_all[n];
    counts[0] = ustart_all[n];
    counts[1] = n;
  }
  if (j >= n) return;
  plist[j] = order[j];
  ustart[j] = ustart_all[j];
  const double* res = results + (long long)kResults * j;
  ResState s{};
  s.rro = res[0];
  s.eps_target = eps * sqrt(res[kResInitial]);
  s.n = 1;
  s.loop_max = loop_max;
  st[j] = s;
}

// Iterations of each problem in the step that just ended (the loop stops at
// iteration n whether it converged there or reached loop_max).
__global__ void k_b_record(const ResState* st, int n, int* out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = st[i].n;
}

}  // namespace tea

namespace {

using namespace tea;

constexpr int kBranches = 8;  // parallel graph branches of per-problem work

struct Problem {
  int x = 0, y = 0;
  Dev d;
  Red red;
};

struct Batch {
  bool ready = false;
  int n = 0;
  int prec = PREC_NONE, coef = 1;
  double xmin = 0, xmax = 0, ymin = 0, ymax = 0;
  int arith = 1;  // arithmetic form
  int device = 0, num_sms = 0;
  cudaStream_t stream = nullptr;
  cudaStream_t aux[kBranches] = {};
  cudaEvent_t fork = nullptr, join[kBranches] = {};
  cudaEvent_t t0 = nullptr, t1 = nullptr, s0 = nullptr, s1 = nullptr;
  cudaEvent_t replay[2] = {};
  double* arena = nullptr;
  double* partials = nullptr;
  unsigned int* counters = nullptr;
  double* results = nullptr;
  double* results_h = nullptr;  // pinned, n * kResults
  Dev* devs_d = nullptr;
  Red* reds_d = nullptr;
  ResState* st_d = nullptr;
  int* order_d = nullptr;       // problems, largest first
  int* ustart_all_d = nullptr;  // unit prefix sums over order (n + 1)
  int* plist_d = nullptr;       // active list (WorkList)
  int* ustart_d = nullptr;
  int* counts_d = nullptr;
  int* counts_h = nullptr;      // pinned copy of counts_d after a replay, and
                                // [2] the persistent launch's barrier error flag
  unsigned int* bar_d = nullptr;  // grid barrier of k_b_iterations [2] + error flag
  int* iters_d = nullptr;       // [iters_cap steps][n]
  int iters_cap = 0;
  std::vector<int> iters_h;     // [last_steps][n]
  int last_steps = 0;
  std::vector<Problem> probs;
  std::vector<int> order;       // problems, largest first
  std::vector<double> summary_h;
  bool summary_valid = false;
  tea_gb300_batch_launch launch{0, 16, 1, 0};
  int ustart_G = 0;             // G that ustart_all_d was built for
  int max_bps = 1;
  int occ[3][3] = {};  // [arithmetic form][w, ur, p]
  int occ_persistent[3] = {};  // [arithmetic form] k_b_iterations
  cudaGraphExec_t iter_graph = nullptr;
  int graph_bps = 0, graph_iters = 0, graph_G = 0, graph_persistent = 0;
};

Batch g_batch;

bool batch_ok(const char* who) {
  if (!g_batch.ready) {
    fail(50, "%s: no batch (call tea_gb300_batch_create first)", who);
    return false;
  }
  return true;
}

void release_batch() {
  Batch& b = g_batch;
  if (b.stream) cudaStreamSynchronize(b.stream);
  if (b.iter_graph) cudaGraphExecDestroy(b.iter_graph);
  cudaFree(b.arena);
  cudaFree(b.partials);
  cudaFree(b.counters);
  cudaFree(b.results);
  cudaFree(b.devs_d);
  cudaFree(b.reds_d);
  cudaFree(b.st_d);
  cudaFree(b.order_d);
  cudaFree(b.ustart_all_d);
  cudaFree(b.plist_d);
  cudaFree(b.ustart_d);
  cudaFree(b.counts_d);
  cudaFree(b.bar_d);
  cudaFree(b.iters_d);
  cudaFreeHost(b.results_h);
  cudaFreeHost(b.counts_h);
  for (int k = 0; k < kBranches; k++) {
    if (b.aux[k]) cudaStreamDestroy(b.aux[k]);
    if (b.join[k]) cudaEventDestroy(b.join[k]);
  }
  cudaEvent_t evs[] = {b.fork, b.t0, b.t1, b.s0, b.s1, b.replay[0], b.replay[1]};
  for (cudaEvent_t e : evs)
    if (e) cudaEventDestroy(e);
  if (b.stream) cudaStreamDestroy(b.stream);
  b = Batch();
}

// Doubles of one padded field of an x by y problem with halo 1, rounded up
// so that the next field's base stays 256-byte aligned.
size_t field_doubles(long long S, int y) {
  const long long rows = y + 2 + 1;
  const long long off = 31;  // column 1 of every row on a 256-byte boundary
  const long long n = off + rows * S + 32;
  return (size_t)((n + 31) / 32 * 32);
}

// Resident blocks per SM of a kernel at kBlock threads.
int occupancy(const void* k) {
  int v = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&v, k, kBlock, 0);
  return std::max(v, 1);
}

// Occupancy of the iteration kernels ([arithmetic form][w, ur, p]) and the
// largest of them (the upper end of blocks_per_sm).
int set_occupancy(Batch& b) {
  b.occ[0][0] = occupancy((const void*)k_b_calc_w<0>);
  b.occ[0][1] = occupancy((const void*)k_b_calc_ur<0>);
  b.occ[0][2] = occupancy((const void*)k_b_calc_p<0>);
  b.occ[1][0] = occupancy((const void*)k_b_calc_w<1>);
  b.occ[1][1] = occupancy((const void*)k_b_calc_ur<1>);
  b.occ[1][2] = occupancy((const void*)k_b_calc_p<1>);
  b.occ[2][0] = occupancy((const void*)k_b_calc_w<2>);
  b.occ[2][1] = occupancy((const void*)k_b_calc_ur<2>);
  b.occ[2][2] = occupancy((const void*)k_b_calc_p<2>);
  b.occ_persistent[0] = occupancy((const void*)k_b_iterations<0>);
  b.occ_persistent[1] = occupancy((const void*)k_b_iterations<1>);
  b.occ_persistent[2] = occupancy((const void*)k_b_iterations<2>);
  int m = 1;
  for (int f = 0; f < 3; f++)
    for (int k = 0; k < 3; k++) m = std::max(m, b.occ[f][k]);
  return std::min(m, 8);
}

}  // namespace

extern "C" int tea_gb300_batch_create(int n, const int* x_cells, const int* y_cells,
                                      double xmin, double xmax, double ymin,
                                      double ymax, int preconditioner,
                                      int coefficient) {
  release_batch();
  Batch& b = g_batch;
  if (n < 1 || !x_cells || !y_cells) {
    fail(51, "tea_gb300_batch_create: need n >= 1 problems (got %d)", n);
    return -1;
  }
  if (preconditioner != PREC_NONE && preconditioner != PREC_JAC_DIAG &&
      preconditioner != PREC_JAC_BLOCK) {
    fail(51, "tea_gb300_batch_create: unknown preconditioner %d", preconditioner);
    return -1;
  }
  if (coefficient != TEA_COEF_CONDUCTIVITY &&
      coefficient != TEA_COEF_RECIP_CONDUCTIVITY) {
    fail(51, "tea_gb300_batch_create: unknown coefficient %d", coefficient);
    return -1;
  }
  if (!(xmax > xmin) || !(ymax > ymin)) {
    fail(51, "tea_gb300_batch_create: empty domain");
    return -1;
  }
  for (int i = 0; i < n; i++) {
    if (x_cells[i] < 1 || y_cells[i] < 1 || x_cells[i] > (1 << 20) ||
        y_cells[i] > (1 << 20)) {
      fail(51, "tea_gb300_batch_create: problem %d has invalid size %d x %d", i,
           x_cells[i], y_cells[i]);
      return -1;
    }
  }
  b.n = n;
  b.prec = preconditioner;
  b.coef = coefficient;
  b.xmin = xmin;
  b.xmax = xmax;
  b.ymin = ymin;
  b.ymax = ymax;
  b.arith = tea_gb300_get_arithmetic();
  if (!check_cuda(cudaGetDevice(&b.device), "cudaGetDevice")) return -1;
  cudaDeviceGetAttribute(&b.num_sms, cudaDevAttrMultiProcessorCount, b.device);
  b.ready = true;  // from here on release_batch frees partial allocations
  if (!check_cuda(cudaStreamCreateWithFlags(&b.stream, cudaStreamNonBlocking),
                  "batch stream"))
    return -1;
  for (int k = 0; k < kBranches; k++) {
    if (!check_cuda(cudaStreamCreateWithFlags(&b.aux[k], cudaStreamNonBlocking),
                    "batch stream") ||
        !check_cuda(cudaEventCreateWithFlags(&b.join[k], cudaEventDisableTiming),
                    "batch event"))
      return -1;
  }
  cudaEventCreateWithFlags(&b.fork, cudaEventDisableTiming);
  cudaEventCreateWithFlags(&b.replay[0], cudaEventDisableTiming);
  cudaEventCreateWithFlags(&b.replay[1], cudaEventDisableTiming);
  cudaEventCreate(&b.t0);
  cudaEventCreate(&b.t1);
  cudaEventCreate(&b.s0);
  cudaEventCreate(&b.s1);

  // arena layout: problem after problem, each with its fields in turn
  const int nf = preconditioner == PREC_JAC_BLOCK ? 15 : 13;
  b.probs.resize(n);
  size_t total = 0, part_total = 0;
  std::vector<size_t> offs(n), part_offs(n);
  for (int i = 0; i < n; i++) {
    Problem& p = b.probs[i];
    p.x = x_cells[i];
    p.y = y_cells[i];
    const long long S = ((long long)(p.x + 2 + 1 + 31) / 32) * 32;
    offs[i] = total;
    total += nf * field_doubles(S, p.y);
    const long long ntx = (p.x + kTileW - 1) / kTileW;
    const long long nsx = (ntx + kTilesPerSuper - 1) / kTilesPerSuper;
    const long long stride = nsx * ((p.y + 3) / 4) + 1;
    part_offs[i] = part_total;
    part_total += (size_t)(4 * stride + 32) / 32 * 32;
    p.red.stride = stride;
    p.d.S = S;
  }
  if (!check_cuda(cudaMalloc(&b.arena, total * sizeof(double)), "cudaMalloc batch arena") ||
      !check_cuda(cudaMemsetAsync(b.arena, 0, total * sizeof(double), b.stream),
                  "cudaMemset batch arena") ||
      !check_cuda(cudaMalloc(&b.partials, part_total * sizeof(double)),
                  "cudaMalloc batch partials") ||
      !check_cuda(cudaMalloc(&b.counters, n * sizeof(unsigned int)),
                  "cudaMalloc batch counters") ||
      !check_cuda(cudaMemsetAsync(b.counters, 0, n * sizeof(unsigned int), b.stream),
                  "cudaMemset batch counters") ||
      !check_cuda(cudaMalloc(&b.results, (size_t)n * kResults * sizeof(double)),
                  "cudaMalloc batch results") ||
      !check_cuda(cudaMallocHost(&b.results_h, (size_t)n * kResults * sizeof(double)),
                  "cudaMallocHost batch results") ||
      !check_cuda(cudaMalloc(&b.order_d, n * sizeof(int)), "cudaMalloc batch order") ||
      !check_cuda(cudaMalloc(&b.ustart_all_d, (n + 1) * sizeof(int)), "cudaMalloc ustart") ||
      !check_cuda(cudaMalloc(&b.plist_d, n * sizeof(int)), "cudaMalloc plist") ||
      !check_cuda(cudaMalloc(&b.ustart_d, (n + 1) * sizeof(int)), "cudaMalloc ustart") ||
      !check_cuda(cudaMalloc(&b.counts_d, 2 * sizeof(int)), "cudaMalloc counts") ||
      !check_cuda(cudaMallocHost(&b.counts_h, 3 * sizeof(int)), "cudaMallocHost counts") ||
      !check_cuda(cudaMalloc(&b.bar_d, 3 * sizeof(unsigned int)), "cudaMalloc batch barrier") ||
      !check_cuda(cudaMemsetAsync(b.bar_d, 0, 3 * sizeof(unsigned int), b.stream),
                  "cudaMemset batch barrier") ||
      !check_cuda(cudaMalloc(&b.st_d, n * sizeof(ResState)), "cudaMalloc batch state")) {
    release_batch();
    return -1;
  }
  for (int i = 0; i < n; i++) {
    Problem& p = b.probs[i];
    Dev d;
    memset(&d, 0, sizeof(d));
    d.x_max = p.x;
    d.y_max = p.y;
    d.H = 1;
    d.S = p.d.S;
    d.prec = preconditioner;
    const size_t fd = field_doubles(d.S, p.y);
    double* base = b.arena + offs[i];
    int k = 0;
    auto next = [&]() { return base + (k++) * fd + 31; };
    d.density = next();
    d.energy1 = next();
    d.volume = next();
    d.u = next();
    d.u0 = next();
    d.p = next();
    d.r = next();
    d.w = next();
    d.Mi = next();
    d.Kx = next();
    d.Ky = next();
    d.z = next();
    d.diag = next();
    if (preconditioner == PREC_JAC_BLOCK) {
      d.cp = next();
      d.bfp = next();
    }
    d.un = d.Mi;
    p.d = make_dev_tiling(d);
    p.red.partials = b.partials + part_offs[i];
    p.red.counter = b.counters + i;
    p.red.result = b.results + (size_t)kResults * i;
  }
  // work order: largest problems first
  b.order.resize(n);
  for (int i = 0; i < n; i++) b.order[i] = i;
  std::stable_sort(b.order.begin(), b.order.end(), [&](int a, int c) {
    return (long long)b.probs[a].x * b.probs[a].y > (long long)b.probs[c].x * b.probs[c].y;
  });
  std::vector<Dev> devs(n);
  std::vector<Red> reds(n);
  for (int i = 0; i < n; i++) {
    devs[i] = b.probs[i].d;
    reds[i] = b.probs[i].red;
  }
  if (!check_cuda(cudaMalloc(&b.devs_d, n * sizeof(Dev)), "cudaMalloc devs") ||
      !check_cuda(cudaMalloc(&b.reds_d, n * sizeof(Red)), "cudaMalloc reds") ||
      !check_cuda(cudaMemcpyAsync(b.order_d, b.order.data(), n * sizeof(int),
                                  cudaMemcpyHostToDevice, b.stream), "order upload") ||
      !check_cuda(cudaMemcpyAsync(b.devs_d, devs.data(), n * sizeof(Dev),
                                  cudaMemcpyHostToDevice, b.stream), "devs upload") ||
      !check_cuda(cudaMemcpyAsync(b.reds_d, reds.data(), n * sizeof(Red),
                                  cudaMemcpyHostToDevice, b.stream), "reds upload")) {
    release_batch();
    return -1;
  }
  // cell volumes (initialise_chunk_kernel with dx, dy of each problem)
  LaunchCtx l{b.stream, b.num_sms, b.arith};
  for (int i = 0; i < n; i++) {
    const Problem& p = b.probs[i];
    const double dx = (xmax - xmin) / (double)(float)p.x;
    const double dy = (ymax - ymin) / (double)(float)p.y;
    dev_volume(l, p.d, dx * dy);
  }
  b.max_bps = set_occupancy(b);
  b.launch.blocks_per_sm = b.max_bps;
  b.launch.graph_iterations = 16;
  if (!check_cuda(cudaStreamSynchronize(b.stream), "batch create")) {
    release_batch();
    return -1;
  }
  b.summary_valid = false;
  return 0;
}

extern "C" void tea_gb300_batch_free(void) { release_batch(); }

static bool check_index(int i, const char* who) {
  if (!batch_ok(who)) return false;
  if (i < 0 || i >= g_batch.n) {
    fail(52, "%s: problem %d outside 0..%d", who, i, g_batch.n - 1);
    return false;
  }
  return true;
}

// interior of a padded field <-> a dense x-fastest host array
static bool copy_interior(const Problem& p, double* field, const double* host_in,
                          double* host_out, cudaStream_t s) {
  double* dst = field + p.d.S + 1;  // padded (1,1)
  const size_t pitch = (size_t)p.d.S * sizeof(double);
  const size_t row = (size_t)p.x * sizeof(double);
  if (host_in)
    return check_cuda(cudaMemcpy2DAsync(dst, pitch, host_in, row, row, p.y,
                                        cudaMemcpyHostToDevice, s),
                      "batch field upload");
  return check_cuda(cudaMemcpy2DAsync(host_out, row, dst, pitch, row, p.y,
                                      cudaMemcpyDeviceToHost, s),
                    "batch field download");
}

extern "C" int tea_gb300_batch_set_fields(int i, const double* density,
                                          const double* energy) {
  if (!check_index(i, "tea_gb300_batch_set_fields")) return -1;
  if (!density || !energy) {
    fail(52, "tea_gb300_batch_set_fields: null field");
    return -1;
  }
  Batch& b = g_batch;
  const Problem& p = b.probs[i];
  if (!copy_interior(p, p.d.density, density, nullptr, b.stream) ||
      !copy_interior(p, p.d.energy1, energy, nullptr, b.stream) ||
      !check_cuda(cudaStreamSynchronize(b.stream), "batch set fields"))
    return -1;
  b.summary_valid = false;
  return 0;
}

extern "C" int tea_gb300_batch_read_field(int i, int field, double* out) {
  if (!check_index(i, "tea_gb300_batch_read_field")) return -1;
  Batch& b = g_batch;
  const Problem& p = b.probs[i];
  double* f = field == TEA_FIELD_DENSITY ? p.d.density
              : field == TEA_FIELD_ENERGY1 ? p.d.energy1
              : field == TEA_FIELD_U       ? p.d.u
                                           : nullptr;
  if (!f || !out) {
    fail(52, "tea_gb300_batch_read_field: field %d not kept by a batch", field);
    return -1;
  }
  if (!copy_interior(p, f, nullptr, out, b.stream) ||
      !check_cuda(cudaStreamSynchronize(b.stream), "batch read field"))
    return -1;
  return 0;
}

// ---------------------------------------------------------------------------
// solve phases
// ---------------------------------------------------------------------------

namespace {

// Unit prefix sums over the work order for the current units size G.
bool upload_units(Batch& b) {
  const int G = b.launch.supertiles_per_unit;
  if (b.ustart_G == G) return true;
  std::vector<int> us(b.n + 1);
  long long acc = 0;
  for (int j = 0; j < b.n; j++) {
    us[j] = (int)acc;
    acc += (b.probs[b.order[j]].d.ns + G - 1) / G;
    if (acc > (1LL << 30)) {
      fail(54, "batch: %lld work units exceed the limit", acc);
      return false;
    }
  }
  us[b.n] = (int)acc;
  if (!check_cuda(cudaMemcpyAsync(b.ustart_all_d, us.data(), us.size() * sizeof(int),
                                  cudaMemcpyHostToDevice, b.stream),
                  "batch units upload") ||
      !check_cuda(cudaStreamSynchronize(b.stream), "batch units upload"))
    return false;
  b.ustart_G = G;
  return true;
}

// Queues per-problem work on kBranches streams forked from the batch
// stream (parallel branches when captured into a graph) and joins them.
template <class F>
void for_each_problem(Batch& b, F f) {
  cudaEventRecord(b.fork, b.stream);
  for (int k = 0; k < kBranches; k++) cudaStreamWaitEvent(b.aux[k], b.fork, 0);
  for (int j = 0; j < b.n; j++) {
    const int i = b.order[j];
    const LaunchCtx l{b.aux[j % kBranches], b.num_sms, b.arith};
    f(l, b.probs[i]);
  }
  for (int k = 0; k < kBranches; k++) {
    cudaEventRecord(b.join[k], b.aux[k]);
    cudaStreamWaitEvent(b.stream, b.join[k], 0);
  }
}

// The start of one timestep of every problem, as the single-chunk driver
// does it for tl_use_cg (tea_solve.f90:37-146 with all faces external):
// halo update of density and energy1, common_init (face coefficients,
// boundary faces zeroed, diagonal, u = u0 = energy1 density), residual,
// initial r.r, preconditioner set-up and cg_init (p, r.z), then the loop
// scalars of every problem.
void enqueue_prologue(Batch& b, double dt, double eps, int loop_max) {
  for_each_problem(b, [&](const LaunchCtx& l, const Problem& p) {
    const double dx = (b.xmax - b.xmin) / (double)(float)p.x;
    const double dy = (b.ymax - b.ymin) / (double)(float)p.y;
    const double rx = dt / (dx * dx), ry = dt / (dy * dy);
    const int zb[4] = {1, 1, 1, 1};
    dev_update_halo(l, p.d, 1 | 4, 1);
    dev_init_common(l, p.d, b.coef, rx, ry);
    dev_zero_boundary(l, p.d, zb);
    dev_init_diag(l, p.d, p.red);
    dev_init_u(l, p.d, p.d.energy1);
    dev_calc_residual(l, p.d, p.red);
    Red rdot = p.red;
    rdot.result = p.red.result + kResInitial;
    dev_dot(l, p.d, rdot, p.d.r, p.d.r);
    if (b.prec == PREC_JAC_BLOCK)
      dev_block_init(l, p.d);
    else if (b.prec == PREC_JAC_DIAG)
      dev_init_jac_diag(l, p.d);
    dev_cg_init_p(l, p.d, p.red);
  });
  k_b_begin<<<(b.n + 255) / 256, 256, 0, b.stream>>>(
      b.st_d, b.results, b.n, eps, loop_max, b.order_d, b.ustart_all_d, b.plist_d,
      b.ustart_d, b.counts_d);
  count_launch("batch_begin");
  check_cuda(cudaGetLastError(), "batch_begin");
}

// The end of a timestep: energy1 = u / density and its halo
// (tea_solve.f90:388-394).
void enqueue_epilogue(Batch& b) {
  for_each_problem(b, [&](const LaunchCtx& l, const Problem& p) {
    dev_finalise(l, p.d, p.red);
    dev_update_halo(l, p.d, 4, 1);
  });
}

WorkList work_list(const Batch& b) {
  return WorkList{b.plist_d, b.ustart_d, b.counts_d, b.launch.supertiles_per_unit};
}

// `iters` CG iterations of every active problem; with `compact` the active
// list is then rebuilt and its counts copied to the host.  Returns the
// number of kernels queued.
// One CG iteration; each kernel's grid is bps blocks per SM, capped by
// that kernel's own occupancy (b.occ).
template <int F>
void enqueue_iteration(Batch& b, const WorkList& wl, int bps) {
  const int* occ = b.occ[F];
  auto grid = [&](int k) { return std::max(1, b.num_sms * std::min(bps, occ[k])); };
  k_b_calc_w<F><<<grid(0), kBlock, 0, b.stream>>>(b.devs_d, b.reds_d, b.st_d, wl);
  k_b_calc_ur<F><<<grid(1), kBlock, 0, b.stream>>>(b.devs_d, b.reds_d, b.st_d, wl);
  k_b_calc_p<F><<<grid(2), kBlock, 0, b.stream>>>(b.devs_d, b.reds_d, b.st_d, wl);
}

// All `iters` iterations as one cooperative launch of k_b_iterations: as
// many blocks as are resident at once (bps per SM, capped by the kernel's
// occupancy), the barrier words cleared first.
template <int F>
void enqueue_persistent(Batch& b, const WorkList& wl, int iters, int bps) {
  const int grid = std::max(1, b.num_sms * std::min(bps, b.occ_persistent[F]));
  cudaMemsetAsync(b.bar_d, 0, 3 * sizeof(unsigned int), b.stream);
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(kBlock);
  cfg.stream = b.stream;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  const long long spin_limit = 1LL << 26;
  check_cuda(cudaLaunchKernelEx(&cfg, k_b_iterations<F>, (const Dev*)b.devs_d,
                                (const Red*)b.reds_d, b.st_d, wl, iters, b.bar_d, spin_limit),
             "batch persistent launch");
}

int enqueue_iterations(Batch& b, int iters, int bps, bool compact) {
  const WorkList wl = work_list(b);
  int launched = 0;
  if (b.launch.persistent) {
    if (b.arith == 2)
      enqueue_persistent<2>(b, wl, iters, bps);
    else if (b.arith == 1)
      enqueue_persistent<1>(b, wl, iters, bps);
    else
      enqueue_persistent<0>(b, wl, iters, bps);
    launched = 1;
  } else {
    for (int k = 0; k < iters; k++) {
      if (b.arith == 2)
        enqueue_iteration<2>(b, wl, bps);
      else if (b.arith == 1)
        enqueue_iteration<1>(b, wl, bps);
      else
        enqueue_iteration<0>(b, wl, bps);
    }
    launched = 3 * iters;
  }
  if (compact) {
    k_b_compact<<<1, 1024, 0, b.stream>>>(b.devs_d, b.st_d, b.plist_d, b.ustart_d,
                                          b.counts_d, wl.G);
    cudaMemcpyAsync(b.counts_h, b.counts_d, 2 * sizeof(int), cudaMemcpyDeviceToHost,
                    b.stream);
    // the persistent launch's barrier error flag, for the host's check
    if (b.launch.persistent)
      cudaMemcpyAsync(b.counts_h + 2, b.bar_d + 2, sizeof(int), cudaMemcpyDeviceToHost,
                      b.stream);
    launched++;
  }
  check_cuda(cudaGetLastError(), "batch iterations");
  return launched;
}

// Captures the queued work of `enqueue` into an executable graph.
template <class F>
cudaGraphExec_t capture(Batch& b, F enqueue) {
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  if (!check_cuda(cudaStreamBeginCapture(b.stream, cudaStreamCaptureModeThreadLocal),
                  "batch graph capture"))
    return nullptr;
  enqueue();
  if (!check_cuda(cudaStreamEndCapture(b.stream, &graph), "batch graph capture end"))
    return nullptr;
  const bool ok = check_cuda(cudaGraphInstantiate(&exec, graph, 0), "batch graph instantiate");
  cudaGraphDestroy(graph);
  return ok ? exec : nullptr;
}

}  // namespace

extern "C" int tea_gb300_batch_run(int steps, double dt, double eps, int max_iters,
                                   tea_gb300_batch_stats* stats) {
  if (stats) memset(stats, 0, sizeof(*stats));
  if (!batch_ok("tea_gb300_batch_run")) return -1;
  Batch& b = g_batch;
  if (steps < 1 || !(dt > 0.0) || !(eps >= 0.0) || max_iters < 1) {
    fail(53, "tea_gb300_batch_run: invalid steps %d, dt %g, eps %g or max_iters %d",
         steps, dt, eps, max_iters);
    return -1;
  }
  if (!upload_units(b)) return -1;
  const long long need = (long long)steps * b.n;
  if (need > b.iters_cap) {
    cudaFree(b.iters_d);
    b.iters_d = nullptr;
    b.iters_cap = 0;
    if (!check_cuda(cudaMalloc(&b.iters_d, need * sizeof(int)), "cudaMalloc batch iterations"))
      return -1;
    b.iters_cap = (int)need;
  }
  const int bps = std::min(std::max(b.launch.blocks_per_sm, 1), b.max_bps);
  const int gi = b.launch.graph_iterations;
  if (b.iter_graph && (b.graph_bps != bps || b.graph_iters != gi ||
                       b.graph_G != b.launch.supertiles_per_unit ||
                       b.graph_persistent != b.launch.persistent)) {
    cudaGraphExecDestroy(b.iter_graph);
    b.iter_graph = nullptr;
  }
  int per_replay = 0;
  if (!b.iter_graph) {
    b.iter_graph = capture(b, [&]() { per_replay = enqueue_iterations(b, gi, bps, true); });
    if (!b.iter_graph) return -1;
    b.graph_bps = bps;
    b.graph_iters = gi;
    b.graph_G = b.launch.supertiles_per_unit;
    b.graph_persistent = b.launch.persistent;
  }
  per_replay = b.launch.persistent ? 2 : 3 * gi + 1;
  b.counts_h[2] = 0;
  long long n0 = tea_gb300_kernel_launches();
  cudaGraphExec_t pro = capture(b, [&]() { enqueue_prologue(b, dt, eps, max_iters); });
  const long long pro_nodes = tea_gb300_kernel_launches() - n0;
  n0 = tea_gb300_kernel_launches();
  cudaGraphExec_t epi = capture(b, [&]() { enqueue_epilogue(b); });
  const long long epi_nodes = tea_gb300_kernel_launches() - n0;
  count_launches(-(pro_nodes + epi_nodes));  // counted again when they run
  auto done = [&](int rc) {
    if (pro) cudaGraphExecDestroy(pro);
    if (epi) cudaGraphExecDestroy(epi);
    return rc;
  };
  if (!pro || !epi) return done(-1);

  const long long max_replays = (long long)max_iters / gi + 3;
  long long replays = 0, kernels = 0;
  double solve_ms = 0.0;
  b.summary_valid = false;
  cudaEventRecord(b.t0, b.stream);
  for (int step = 0; step < steps; step++) {
    if (!check_cuda(cudaGraphLaunch(pro, b.stream), "batch prologue")) return done(-1);
    kernels += pro_nodes;
    cudaEventRecord(b.s0, b.stream);
    // one replay queued ahead of the one whose counts are read
    long long launched = 0;
    for (;;) {
      if (launched >= max_replays) {
        fail(53, "batch: the CG loops did not stop after %lld graph replays", launched);
        cudaStreamSynchronize(b.stream);
        return done(-1);
      }
      if (!check_cuda(cudaGraphLaunch(b.iter_graph, b.stream), "batch replay"))
        return done(-1);
      cudaEventRecord(b.replay[launched % 2], b.stream);
      launched++;
      if (launched < 2) continue;
      if (!check_cuda(cudaEventSynchronize(b.replay[(launched - 2) % 2]), "batch replay"))
        return done(-1);
      if (((volatile int*)b.counts_h)[2] != 0) {
        fail(57, "batch: a grid barrier of the persistent iterations timed out");
        cudaStreamSynchronize(b.stream);
        return done(-1);
      }
      if (((volatile int*)b.counts_h)[1] == 0) break;
    }
    replays += launched;
    kernels += launched * per_replay;
    cudaEventRecord(b.s1, b.stream);
    if (!check_cuda(cudaGraphLaunch(epi, b.stream), "batch epilogue")) return done(-1);
    kernels += epi_nodes;
    k_b_record<<<(b.n + 255) / 256, 256, 0, b.stream>>>(b.st_d, b.n,
                                                        b.iters_d + (long long)step * b.n);
    kernels++;
    float ms = 0.0f;
    if (!check_cuda(cudaEventSynchronize(b.s1), "batch step") ||
        !check_cuda(cudaEventElapsedTime(&ms, b.s0, b.s1), "batch step timing"))
      return done(-1);
    solve_ms += ms;
  }
  // field summaries of every problem (field_summary_kernel)
  n0 = tea_gb300_kernel_launches();
  for_each_problem(b, [&](const LaunchCtx& l, const Problem& p) {
    dev_field_summary(l, p.d, p.red);
  });
  const long long summary_kernels = tea_gb300_kernel_launches() - n0;
  kernels += summary_kernels;
  cudaMemcpyAsync(b.results_h, b.results, (size_t)b.n * kResults * sizeof(double),
                  cudaMemcpyDeviceToHost, b.stream);
  cudaEventRecord(b.t1, b.stream);
  b.iters_h.assign((size_t)need, 0);
  if (!check_cuda(cudaMemcpyAsync(b.iters_h.data(), b.iters_d, need * sizeof(int),
                                  cudaMemcpyDeviceToHost, b.stream),
                  "batch iterations") ||
      !check_cuda(cudaStreamSynchronize(b.stream), "batch run"))
    return done(-1);
  count_launches(kernels - summary_kernels);  // the rest ran from graphs
  b.last_steps = steps;
  b.summary_h.resize((size_t)b.n * 4);
  for (int i = 0; i < b.n; i++)
    for (int v = 0; v < 4; v++) b.summary_h[4 * i + v] = b.results_h[(size_t)kResults * i + v];
  b.summary_valid = true;
  if (stats) {
    float total = 0.0f;
    cudaEventElapsedTime(&total, b.t0, b.t1);
    stats->steps = steps;
    stats->graph_launches = (int)replays;
    stats->kernel_launches = kernels;
    stats->solve_ms = solve_ms;
    stats->total_ms = total;
    for (int s = 0; s < steps; s++)
      for (int i = 0; i < b.n; i++) {
        const int it = b.iters_h[(size_t)s * b.n + i];
        stats->max_iterations = std::max(stats->max_iterations, it);
        stats->iterations += it;
        stats->cell_iterations += (double)b.probs[i].x * b.probs[i].y * it;
      }
  }
  return done(0);
}

extern "C" int tea_gb300_batch_summary(int i, double summary[4]) {
  if (!check_index(i, "tea_gb300_batch_summary")) return -1;
  if (!g_batch.summary_valid) {
    fail(55, "tea_gb300_batch_summary: no run since the batch or its fields were set");
    return -1;
  }
  for (int v = 0; v < 4; v++) summary[v] = g_batch.summary_h[4 * (size_t)i + v];
  return 0;
}

extern "C" int tea_gb300_batch_iterations(int i, int* iterations, int steps) {
  if (!check_index(i, "tea_gb300_batch_iterations")) return -1;
  const Batch& b = g_batch;
  if (steps < 0 || steps > b.last_steps || (steps > 0 && !iterations)) {
    fail(55, "tea_gb300_batch_iterations: %d steps asked, the last run had %d", steps,
         b.last_steps);
    return -1;
  }
  for (int s = 0; s < steps; s++) iterations[s] = b.iters_h[(size_t)s * b.n + i];
  return 0;
}

extern "C" int tea_gb300_batch_get_launch(tea_gb300_batch_launch* launch) {
  if (!batch_ok("tea_gb300_batch_get_launch")) return -1;
  *launch = g_batch.launch;
  return 0;
}

extern "C" int tea_gb300_batch_set_launch(const tea_gb300_batch_launch* launch) {
  if (!batch_ok("tea_gb300_batch_set_launch")) return -1;
  Batch& b = g_batch;
  if (!launch || launch->blocks_per_sm < 1 || launch->blocks_per_sm > b.max_bps ||
      launch->graph_iterations < 1 || launch->graph_iterations > 64 ||
      launch->supertiles_per_unit < 1 || launch->supertiles_per_unit > 64 ||
      launch->persistent < 0 || launch->persistent > 1) {
    fail(56, "tea_gb300_batch_set_launch: blocks_per_sm must be 1..%d, "
             "graph_iterations 1..64, supertiles_per_unit 1..64, persistent 0 or 1",
         b.max_bps);
    return -1;
  }
  b.launch = *launch;
  return 0;
}

// Times CG iterations of the whole batch for each candidate geometry and
// keeps the fastest.  The iterations run on the solver work fields (u, r,
// p, w, z) from a fresh prologue with eps = 0, so that no problem stops
// while it is timed; density, energy1 and the results of every later
// batch_run, which starts with its own prologue, are unchanged.
extern "C" int tea_gb300_batch_autotune(tea_gb300_batch_launch* best) {
  if (!batch_ok("tea_gb300_batch_autotune")) return -1;
  Batch& b = g_batch;
  const tea_gb300_batch_launch keep = b.launch;
  const int units[] = {1, 2, 4, 8};
  const int timed = 4;
  float best_ms = 0.0f;
  tea_gb300_batch_launch choice = keep;
  bool have = false;
  for (int G : units) {
    b.launch.supertiles_per_unit = G;
    if (!upload_units(b)) {
      b.launch = keep;
      return -1;
    }
    enqueue_prologue(b, 0.004, 0.0, 1 << 30);
    // three kernels per iteration, or one persistent launch per replay
    for (int persistent = 0; persistent < 2; persistent++) {
      b.launch.persistent = persistent;
      const int top = persistent ? std::min(b.max_bps, b.occ_persistent[b.arith]) : b.max_bps;
      for (int bps = 1; bps <= top; bps++) {
        enqueue_iterations(b, 1, bps, false);  // warm-up
        float ms_min = 0.0f;
        for (int rep = 0; rep < 2; rep++) {
          cudaEventRecord(b.s0, b.stream);
          enqueue_iterations(b, timed, bps, false);
          cudaEventRecord(b.s1, b.stream);
          float ms = 0.0f;
          if (!check_cuda(cudaEventSynchronize(b.s1), "batch autotune") ||
              !check_cuda(cudaEventElapsedTime(&ms, b.s0, b.s1), "batch autotune")) {
            b.launch = keep;
            return -1;
          }
          count_launches(persistent ? 1 : 3 * timed);
          if (rep == 0 || ms < ms_min) ms_min = ms;
        }
        count_launches(persistent ? 1 : 3);
        if (persistent) {
          // a launch whose barrier timed out returned early: never a candidate
          unsigned int flag = 0;
          if (!check_cuda(cudaMemcpy(&flag, b.bar_d + 2, sizeof(flag), cudaMemcpyDeviceToHost),
                          "batch autotune barrier flag") ||
              flag != 0) {
            if (flag)
              fail(57, "batch autotune: a grid barrier of the persistent iterations timed out");
            b.launch = keep;
            return -1;
          }
        }
        if (!have || ms_min < best_ms) {
          have = true;
          best_ms = ms_min;
          choice.blocks_per_sm = bps;
          choice.supertiles_per_unit = G;
          choice.persistent = persistent;
        }
      }
    }
  }
  choice.graph_iterations = keep.graph_iterations;
  b.launch = choice;
  if (best) *best = choice;
  return 0;
}
