// Two PPCG inner steps in one pass over the grid, with the block-Jacobi
// preconditioner: tea_leaf_ppcg_solve_update_r and
// tea_leaf_ppcg_solve_calc_sd (tea_leaf_ppcg_cl.cl:62-155) for steps k and
// k+1 fused, the inputs staged through shared memory by TMA.
//
// Why.  On GB300 an inner step is bound by the FP64 pipe (about 8.5 FP64
// instructions per cell) and, close behind, by HBM (update_r and calc_sd
// move 112 B per cell between them).  Fusing two steps reads u, r, sd and
// the five coefficient fields once and writes u, r, sd once: 88 B per cell
// for two steps, so HBM drops well below the FP64 pipe and only the FP64
// pipe bounds the pass.  This is the matrix-powers schedule of the
// reference's halo depth 2 (tea_solve.f90:445-470, the bounds_extra of
// tea_leaf_kernel_ocl.cpp:352-411) kept on chip instead of in the halo.
//
// Work decomposition.  The interior is cut into column bands of at most
// kLanes - 2 columns (even band starts, for TMA's 16-byte rule) and each
// band into chunks of L four-row strips (the block-Jacobi strips).  A block
// takes (band, chunk) items in turn and marches up the chunk strip by strip.
// Per stage a TMA copy brings one strip (4 rows x the band plus two columns
// each side) of sd, r, u, Kx, Ky, diag, cp and bfp into a ring of five
// shared-memory slots.  Warp group A runs step k on strip a (columns band
// - 1 .. band + 1, the halo step B needs), warp group B runs step k+1 on
// strip a - 2 (the band itself), which needs A's results of strips a - 3 ..
// a - 1.  A chunk costs two extra strips of step k (its lower and upper
// halo) and a band two extra columns.
//
// Buffers.  A block reads r and sd around its items (other blocks' cells)
// while other blocks write theirs, so r and sd are written to a second
// buffer pair (the caller swaps); u is read and written only at a block's
// own cells and is updated in place.
//
// Arithmetic.  Every value is formed by the expressions of the two
// unfused kernels in the same order (bms_v, strip_solve_v; the same
// integer-pipe products), so the results are bit-identical to two calls of
// update_r + calc_sd in each of the three arithmetic forms.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <stdio.h>

#include <algorithm>
#include <utility>
#include <vector>

#include "tea_device.cuh"
#include "tea_tma.cuh"

namespace tea {

constexpr int kTbSlots = 5;
constexpr int kTbFields = 8;
enum { TB_SD = 0, TB_R, TB_U, TB_KX, TB_KY, TB_DIAG, TB_CP, TB_BFP };

template <int NWA>
struct TbShape {
  static constexpr int kLanes = 32 * NWA;  // columns of one warp group
  static constexpr int kWt = kLanes + 2;   // columns loaded: band <= kLanes - 2, two halo columns each side
  static constexpr int kFb = ((4 * kWt + 15) / 16) * 16;  // doubles per field strip (128-byte multiple)
  static constexpr int kSlot = kTbFields * kFb;
  static constexpr int kSd1 = 4 * kWt;    // one strip of sd after step k
  static constexpr int kRu = 4 * kLanes;  // one strip of r or u after step k
  static constexpr int kThreads = 2 * kLanes;
  static constexpr size_t kSmem =
      (size_t)(kTbSlots * kSlot + 4 * kSd1 + 6 * kRu) * sizeof(double) + kTbSlots * 8;
  static constexpr uint32_t kSlotBytes = (uint32_t)(kTbFields * 4 * kWt * sizeof(double));
};

struct TbMaps {
  CUtensorMap m[kTbFields];
};

struct TbArgs {
  int x_max, y_max, H, E;  // E: halo columns kept left of the tensor origin (H rounded up to even)
  long long S;
  double* u;  // padded element (0,0) of u, updated in place
  double* r_out;
  double* sd_out;
  int nb, half_x, ny, L, nchunks, block_top_check;
  double a0, b0, a1, b1;  // coefficients of steps k and k+1
  int* err;               // set when a copy does not arrive
  long long spin_limit;
  const ResState* st;     // resident loop: nothing to do once it has stopped
};

template <int F, int NWA>
__global__ void __launch_bounds__(TbShape<NWA>::kThreads)
    k_ppcg_inner_pair(const __grid_constant__ TbMaps maps, const TbArgs g) {
  using T = TbShape<NWA>;
  if (g.st && *(volatile const int*)&g.st->stop) return;
  extern __shared__ __align__(128) double smem[];
  double* slots = smem;
  double* sd1 = slots + kTbSlots * T::kSlot;
  double* r1 = sd1 + 4 * T::kSd1;
  double* u1 = r1 + 3 * T::kRu;
  uint64_t* bars = (uint64_t*)(u1 + 3 * T::kRu);
  const int tid = threadIdx.x;
  const bool grp_a = tid < T::kLanes;
  const int lane = grp_a ? tid : tid - T::kLanes;
  const int ci = lane + 1;  // shared-memory column of this thread's column
  // a TMA destination must be 128-byte aligned: every field strip is a
  // multiple of 128 bytes from the base, so the base decides
  if (smem_addr(smem) & 127u) {
    if (tid == 0) atomicExch(g.err, 2);
    return;
  }
  if (tid == 0) {
    for (int s = 0; s < kTbSlots; s++) mbar_init(&bars[s], 1);
    fence_barrier_init();
  }
  __syncthreads();
  // rows in the block-Jacobi strip starting at interior row y (strip_rows)
  auto rows_of = [&](int y) {
    if (!g.block_top_check) return 4;
    const int up = g.y_max - y + (g.H == 1 ? 1 : 0);
    return up < 4 ? up : 4;
  };
  long long issued = 0;  // copies this block has issued (load n: slot n % 5, parity (n / 5) & 1)
  bool failed = false;
  const int items = g.nb * g.nchunks;
  for (int item = blockIdx.x; item < items && !failed; item += gridDim.x) {
    const int band = item % g.nb, chunk = item / g.nb;
    const int x0 = 2 * (int)((long long)band * g.half_x / g.nb);
    const int x1 = band + 1 < g.nb ? 2 * (int)((long long)(band + 1) * g.half_x / g.nb) : g.x_max;
    const int j0 = chunk * g.L;
    const int nL = min(g.ny, j0 + g.L) - j0;
    const int nloads = nL + 4;  // strips j0-2 .. j0+nL+1
    const long long g0 = issued;
    issued += nloads;
    auto slot_of = [&](int k) { return slots + (int)((g0 + k) % kTbSlots) * T::kSlot; };
    auto issue = [&](int k) {  // thread 0
      const long long n = g0 + k;
      uint64_t* bar = &bars[n % kTbSlots];
      double* dst = slots + (int)(n % kTbSlots) * T::kSlot;
      fence_proxy_async_smem();
      mbar_arrive_expect_tx(bar, T::kSlotBytes);
      const int tx = x0 - 2 + g.E, ty = 4 * (j0 - 2 + k) + g.H;
#pragma unroll
      for (int f = 0; f < kTbFields; f++) tma_load_2d(dst + f * T::kFb, &maps.m[f], tx, ty, bar);
    };
    auto arrived = [&](int k) {
      const long long n = g0 + k;
      return mbar_wait_bounded(&bars[n % kTbSlots], (uint32_t)((n / kTbSlots) & 1), g.spin_limit);
    };
    if (tid == 0)
      for (int k = 0; k < 4 && k < nloads; k++) issue(k);
    for (int t = 0; t <= nL + 2; t++) {
      // the slot of load t + 3 held load t - 2, last read in stage t - 1
      if (t >= 1 && t + 3 < nloads && tid == 0) issue(t + 3);
      bool ok = true;
      if (t == 0) ok = arrived(0) && arrived(1);
      if (ok && t + 2 < nloads) ok = arrived(t + 2);
      if (ok && grp_a && t <= nL + 1) {
        // ---- step k on strip a, columns x0-1 .. x0+kLanes-2 ----
        const int a = j0 - 1 + t;
        const double* Lm = slot_of(t);      // strip a-1
        const double* L0 = slot_of(t + 1);  // strip a
        const double* Lp = slot_of(t + 2);  // strip a+1
        auto fld = [&](const double* L, int f, int i, int c) { return L[f * T::kFb + i * T::kWt + c]; };
        const int x = x0 - 1 + lane;
        const bool xs_in = x >= 0 && x < g.x_max && a >= 0 && a < g.ny;
        // Every row is computed (shared memory holds finite halo or fill
        // values everywhere) and the results outside the interior are
        // discarded by selection: no branch separates the four rows, so
        // their independent chains interleave.
        double rl[4], ul[4], sc[4];
        bool in[4];
#pragma unroll
        for (int i = 0; i < 4; i++) {
          in[i] = xs_in && 4 * a + i < g.y_max;
          sc[i] = fld(L0, TB_SD, i, ci);
          const double xn = i < 3 ? fld(L0, TB_SD, i + 1, ci) : fld(Lp, TB_SD, 0, ci);
          const double xs = i > 0 ? fld(L0, TB_SD, i - 1, ci) : fld(Lm, TB_SD, 3, ci);
          const double kyn = i < 3 ? fld(L0, TB_KY, i + 1, ci) : fld(Lp, TB_KY, 0, ci);
          const double rv = bms_v<F>(fld(L0, TB_R, i, ci), fld(L0, TB_DIAG, i, ci), kyn,
                                     fld(L0, TB_KY, i, ci), fld(L0, TB_KX, i, ci + 1),
                                     fld(L0, TB_KX, i, ci), sc[i], xn, xs,
                                     fld(L0, TB_SD, i, ci + 1), fld(L0, TB_SD, i, ci - 1));
          rl[i] = in[i] ? rv : 0.0;
          ul[i] = fld(L0, TB_U, i, ci) + sc[i];
        }
        double zl[4], bfp[4], ky[4], cp[4];
#pragma unroll
        for (int i = 0; i < 4; i++) {
          bfp[i] = fld(L0, TB_BFP, i, ci);
          ky[i] = fld(L0, TB_KY, i, ci);
          cp[i] = fld(L0, TB_CP, i, ci);
        }
        const int upper = xs_in ? rows_of(4 * a) : 4;
        if (upper == 4)
          strip_solve_v<F, true, true>(4, rl, bfp, ky, cp, fld(L0, TB_DIAG, 0, ci), zl);
        else
          strip_solve_v<F, true>(upper, rl, bfp, ky, cp, fld(L0, TB_DIAG, 0, ci), zl);
        double* s1 = sd1 + ((a + 4) & 3) * T::kSd1;
        double* rr = r1 + ((a + 3) % 3) * T::kRu;
        double* uu = u1 + ((a + 3) % 3) * T::kRu;
#pragma unroll
        for (int i = 0; i < 4; i++) {
          const double sn = F ? __fma_rn(g.a0, sc[i], emu_dmul(g.b0, zl[i]))
                              : g.a0 * sc[i] + emu_dmul(g.b0, zl[i]);
          // outside the interior sd keeps its stored (halo) value
          s1[i * T::kWt + ci] = in[i] ? sn : sc[i];
          rr[i * T::kLanes + lane] = rl[i];
          uu[i * T::kLanes + lane] = ul[i];
        }
      } else if (ok && !grp_a && t >= 3) {
        // ---- step k+1 on strip b = a-2, the band's own columns ----
        const int b = j0 - 3 + t;
        const double* L0 = slot_of(t - 1);  // strip b
        const double* Lp = slot_of(t);      // strip b+1
        auto fld = [&](const double* L, int f, int i, int c) { return L[f * T::kFb + i * T::kWt + c]; };
        const double* Sc = sd1 + ((b + 4) & 3) * T::kSd1;
        const double* Sm = sd1 + ((b + 3) & 3) * T::kSd1;
        const double* Sp = sd1 + ((b + 5) & 3) * T::kSd1;
        const double* rr = r1 + ((b + 3) % 3) * T::kRu;
        const double* uu = u1 + ((b + 3) % 3) * T::kRu;
        const int x = x0 - 1 + lane;
        const bool own = x >= x0 && x < x1 && x < g.x_max;
        // as in step k: every row and lane computes, the stores select
        double rl[4], sc[4], uv[4];
        bool in[4];
#pragma unroll
        for (int i = 0; i < 4; i++) {
          in[i] = own && 4 * b + i < g.y_max;
          sc[i] = Sc[i * T::kWt + ci];
          const double xn = i < 3 ? Sc[(i + 1) * T::kWt + ci] : Sp[ci];
          const double xs = i > 0 ? Sc[(i - 1) * T::kWt + ci] : Sm[3 * T::kWt + ci];
          const double kyn = i < 3 ? fld(L0, TB_KY, i + 1, ci) : fld(Lp, TB_KY, 0, ci);
          const double rv = bms_v<F>(rr[i * T::kLanes + lane], fld(L0, TB_DIAG, i, ci), kyn,
                                     fld(L0, TB_KY, i, ci), fld(L0, TB_KX, i, ci + 1),
                                     fld(L0, TB_KX, i, ci), sc[i], xn, xs,
                                     Sc[i * T::kWt + ci + 1], Sc[i * T::kWt + ci - 1]);
          rl[i] = in[i] ? rv : 0.0;
          uv[i] = uu[i * T::kLanes + lane] + sc[i];
        }
        double bfp[4], ky[4], cp[4], zl[4];
#pragma unroll
        for (int i = 0; i < 4; i++) {
          bfp[i] = fld(L0, TB_BFP, i, ci);
          ky[i] = fld(L0, TB_KY, i, ci);
          cp[i] = fld(L0, TB_CP, i, ci);
        }
        const int upper = rows_of(4 * b);
        if (upper == 4)
          strip_solve_v<F, true, true>(4, rl, bfp, ky, cp, fld(L0, TB_DIAG, 0, ci), zl);
        else
          strip_solve_v<F, true>(upper, rl, bfp, ky, cp, fld(L0, TB_DIAG, 0, ci), zl);
#pragma unroll
        for (int i = 0; i < 4; i++) {
          const double sn = F ? __fma_rn(g.a1, sc[i], emu_dmul(g.b1, zl[i]))
                              : g.a1 * sc[i] + emu_dmul(g.b1, zl[i]);
          if (in[i]) {
            const long long c = (long long)(4 * b + i + g.H) * g.S + (x + g.H);
            g.u[c] = uv[i];
            g.r_out[c] = rl[i];
            g.sd_out[c] = sn;
          }
        }
      }
      if (__syncthreads_or(!ok)) failed = true;
      if (failed) break;
    }
  }
  if (failed && tid == 0) {
    atomicExch(g.err, 1);
    // let the copies still in flight land before the block's shared memory
    // is given up (each wait bounded as well)
    for (long long n = issued > kTbSlots ? issued - kTbSlots : 0; n < issued; n++)
      mbar_wait_bounded(&bars[n % kTbSlots], (uint32_t)((n / kTbSlots) & 1), g.spin_limit);
  }
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------

constexpr int kTbNwa = 2;  // warps per group: 64-column bands, two blocks per SM

// Tensor map of one padded field: rows of S doubles, origin E - H columns
// left of element (0,0) so that interior column x is tensor column x + E
// and every copy starting at an even interior column is 16-byte aligned.
static bool encode_field_map(CUtensorMap* m, const Chunk& c, const double* f, int E) {
  using T = TbShape<kTbNwa>;
  // the driver function is looked up through the runtime, so the library
  // does not need the driver library to load (it is absent without a GPU)
  static PFN_cuTensorMapEncodeTiled_v12000 encode = nullptr;
  if (!encode) {
    void* fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (!check_cuda(cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000,
                                                     cudaEnableDefault, &q),
                    "cuTensorMapEncodeTiled lookup") ||
        q != cudaDriverEntryPointSuccess || !fn) {
      fail(80, "cuTensorMapEncodeTiled is not available");
      return false;
    }
    encode = (PFN_cuTensorMapEncodeTiled_v12000)fn;
  }
  const double* origin = f - (E - c.H);
  cuuint64_t dims[2] = {(cuuint64_t)c.S, (cuuint64_t)c.rows};
  cuuint64_t strides[1] = {(cuuint64_t)c.S * sizeof(double)};
  cuuint32_t box[2] = {(cuuint32_t)T::kWt, 4};
  cuuint32_t estr[2] = {1, 1};
  const CUresult rc = encode(
      m, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 2, (void*)origin, dims, strides, box, estr,
      CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
      CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (rc != CUDA_SUCCESS) {
    fail(80, "cuTensorMapEncodeTiled failed (%d)", (int)rc);
    return false;
  }
  return true;
}

// Bands, chunks and grid for the chunk's interior: bands of at most
// kLanes - 2 columns with even starts; chunk length L chosen so that the
// items fill whole waves of the grid with the fewest stages.
struct TbPlan {
  int nb, half_x, ny, L, nchunks, grid;
};

static TbPlan tb_plan(const Chunk& c, int blocks_per_sm) {
  using T = TbShape<kTbNwa>;
  TbPlan p;
  p.half_x = (c.x_max + 1) / 2;
  p.nb = (p.half_x + (T::kLanes - 2) / 2 - 1) / ((T::kLanes - 2) / 2);
  p.ny = (c.y_max + 3) / 4;
  p.grid = c.num_sms * blocks_per_sm;
  long long best = -1;
  p.L = p.ny;
  p.nchunks = 1;
  for (int n = 1; n <= p.ny; n++) {
    const int L = (p.ny + n - 1) / n;
    const int chunks = (p.ny + L - 1) / L;
    if (chunks != n) continue;
    const long long waves = ((long long)p.nb * chunks + p.grid - 1) / p.grid;
    const long long cost = waves * (L + 3);
    if (best < 0 || cost < best) {
      best = cost;
      p.L = L;
      p.nchunks = chunks;
    }
  }
  const long long items = (long long)p.nb * p.nchunks;
  p.grid = (int)std::min<long long>(p.grid, items);
  return p;
}

// The fused pair covers the block-Jacobi preconditioner on grids whose row
// stride holds a whole copy box (kWt columns); others keep the two kernels.
bool tb_applicable(const Chunk& c) {
  return c.inner_pairs && c.prec == PREC_JAC_BLOCK && c.S >= TbShape<kTbNwa>::kWt &&
         c.y_max >= 1;
}

// The launcher state of the current chunk: a tensor map per field buffer
// (looked up by its address, so swapping the r/sd buffers needs no new
// maps), the plan and the error word.  Released with the chunk.
struct TbState {
  bool ready = false;
  std::vector<std::pair<const double*, CUtensorMap>> maps;
  TbPlan plan;
  int* err = nullptr;
};
static TbState g_tb;

static const CUtensorMap* map_for(const Chunk& c, const double* f) {
  for (auto& kv : g_tb.maps)
    if (kv.first == f) return &kv.second;
  CUtensorMap m;
  if (!encode_field_map(&m, c, f, c.H + (c.H & 1))) return nullptr;
  g_tb.maps.emplace_back(f, m);
  return &g_tb.maps.back().second;
}

template <int F>
static void tb_set_attr() {
  static bool done = false;
  if (!done) {
    cudaFuncSetAttribute(k_ppcg_inner_pair<F, kTbNwa>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)TbShape<kTbNwa>::kSmem);
    done = true;
  }
}

// Once per chunk, outside any graph capture (it allocates): the error
// word, the kernels' shared-memory limit and the plan.
bool tb_prepare(Chunk& c) {
  if (g_tb.ready) return true;
  g_tb.maps.reserve(16);
  if (!g_tb.err && !check_cuda(cudaMalloc(&g_tb.err, sizeof(int)), "cudaMalloc tb error word"))
    return false;
  if (!check_cuda(cudaMemsetAsync(g_tb.err, 0, sizeof(int), c.stream), "tb error word reset"))
    return false;
  tb_set_attr<0>();
  tb_set_attr<1>();
  tb_set_attr<2>();
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_ppcg_inner_pair<2, kTbNwa>,
                                                    TbShape<kTbNwa>::kThreads,
                                                    TbShape<kTbNwa>::kSmem) != cudaSuccess ||
      per_sm < 1)
    per_sm = 1;
  g_tb.plan = tb_plan(c, per_sm);
  g_tb.ready = true;
  return true;
}

void tb_release() {
  cudaFree(g_tb.err);
  g_tb.err = nullptr;
  g_tb.maps.clear();
  g_tb.ready = false;
}

// Queues steps s and s+1 (0-based coefficient indices): reads r and sd
// from (r_in, sd_in), u and the coefficients from the chunk, writes u in
// place and r, sd to (r_out, sd_out).  st: resident-loop state or nullptr.
bool launch_ppcg_inner_pair(Chunk& c, int s, const ResState* st, double* r_in,
                            double* sd_in, double* r_out, double* sd_out) {
  if (!tb_prepare(c)) return false;
  const TbPlan& p = g_tb.plan;
  const double* fields[kTbFields] = {sd_in, r_in, c.u.f, c.Kx.f, c.Ky.f, c.diag.f, c.cp.f, c.bfp.f};
  TbMaps maps;
  for (int f = 0; f < kTbFields; f++) {
    const CUtensorMap* m = map_for(c, fields[f]);
    if (!m) return false;
    maps.m[f] = *m;
  }
  TbArgs a;
  a.x_max = c.x_max;
  a.y_max = c.y_max;
  a.H = c.H;
  a.E = c.H + (c.H & 1);
  a.S = c.S;
  a.u = c.u.f;
  a.r_out = r_out;
  a.sd_out = sd_out;
  a.nb = p.nb;
  a.half_x = p.half_x;
  a.ny = p.ny;
  a.L = p.L;
  a.nchunks = p.nchunks;
  a.block_top_check = (c.y_max % 4) != 0;
  a.a0 = c.ppcg_alpha_h[s];
  a.b0 = c.ppcg_beta_h[s];
  a.a1 = c.ppcg_alpha_h[s + 1];
  a.b1 = c.ppcg_beta_h[s + 1];
  a.err = g_tb.err;
  a.spin_limit = 1LL << 22;
  a.st = st;
  const char* name = "tea_leaf_ppcg_solve_inner_pair";
  // inside a graph capture (the resident loop) the caller counts launches
  // and no per-launch timing is taken
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  cudaStreamIsCapturing(c.stream, &cap);
  const bool direct = cap == cudaStreamCaptureStatusNone;
  if (direct) profile_begin(name);
  const size_t sm = TbShape<kTbNwa>::kSmem;
  const int threads = TbShape<kTbNwa>::kThreads;
  if (c.arith == 2)
    k_ppcg_inner_pair<2, kTbNwa><<<p.grid, threads, sm, c.stream>>>(maps, a);
  else if (c.arith == 1)
    k_ppcg_inner_pair<1, kTbNwa><<<p.grid, threads, sm, c.stream>>>(maps, a);
  else
    k_ppcg_inner_pair<0, kTbNwa><<<p.grid, threads, sm, c.stream>>>(maps, a);
  const bool ok = check_cuda(cudaGetLastError(), name);
  if (direct) {
    count_launch(name);
    profile_end(name);
  }
  return ok;
}

// Nonzero once a copy of the fused kernel did not arrive in time (read
// after the stream has been synchronised).
int tb_error() {
  if (!g_tb.err) return 0;
  int e = 0;
  cudaMemcpy(&e, g_tb.err, sizeof(int), cudaMemcpyDeviceToHost);
  return e;
}

}  // namespace tea
