// Device helpers shared by the tile kernels.
//
// Every interior kernel walks the grid in the same tiles: a tile is 32
// interior columns (one per lane of a warp) by TH rows; a supertile is 8
// tiles side by side (one per warp of a 256-thread block).  Blocks take
// supertiles s = blockIdx.x, blockIdx.x + gridDim.x, ...
//
// Fixed summation order of every global sum (the same order the CPU oracle
// implements in oracle_reduce):
//   1. a lane adds its TH rows bottom to top into an accumulator starting at
//      +0.0; rows past the interior add +0.0, lanes past it hold +0.0;
//   2. the 32 lane sums are combined by an xor butterfly (16,8,4,2,1): every
//      lane ends with the tile sum;
//   3. the 8 tile sums of a supertile (0.0 for tiles past the interior) go
//      through the same butterfly on lanes 0..7 of warp 0, lanes 8..31
//      holding 0.0, giving the supertile sum, stored at partials[s];
//   4. the last block to finish adds partials[t], partials[t+256], ... on
//      thread t from +0.0, butterflies each warp, and butterflies the 8 warp
//      sums as in 3.
// All arithmetic is compiled with --fmad=false, so every operation rounds
// exactly as written.
//
// Three arithmetic forms, chosen per chunk (template parameter F):
//   exact (F = 0): every expression of the reference kernels as written,
//     each multiply and add rounded separately;
//   fused (F = 1): the same expressions with each multiply feeding an add
//     contracted into one fused multiply-add (what OpenCL's default
//     FP_CONTRACT allows a GPU compiler to do), and the per-strip division of
//     the block-Jacobi solve replaced by a multiply with the reciprocal kept
//     in bfp at the strip's first row;
//   chain (F = 2): fused, except that the 5-point operator is one chain of
//     fused multiply-adds, A x = D x_c - Ky_n x_n - Ky_c x_s - Kx_e x_e -
//     Kx_c x_w evaluated left to right, and b - A x starts the chain from b.
//     That re-associates the reference's expression (no compiler contraction
//     does that), for the fewest FP64 instructions: 5 per operator
//     application against 6 (fused) and 9 (exact), and 5 per b - A x
//     against 7 and 10.
// The diagonal 1 + (Ky_n + Ky_c) + (Kx_e + Kx_c) is precomputed once per
// timestep into d.diag with the reference's association, so using it is
// bit-identical to recomputing it.  GB300's FP64 pipe, not HBM, bounds these
// kernels, and the fused form roughly halves their FP64 instruction count.
#pragma once

#include "tea_emu.cuh"
#include "tea_internal.h"

namespace tea {

__device__ __forceinline__ long long cidx(const Dev& d, int x, int y) {
  // interior coordinates (x,y) -> offset of padded (x+H, y+H)
  return (long long)(y + d.H) * d.S + (x + d.H);
}

__device__ __forceinline__ double bfly(double v) {
#pragma unroll
  for (int off = 16; off >= 1; off >>= 1)
    v = v + __shfl_xor_sync(0xffffffffu, v, off);
  return v;
}

// The 5-point operator in the association every reference kernel uses
// (e.g. tea_leaf_cg_cl.cl:59-63):
//   (1 + (Ky_n + Ky_c) + (Kx_e + Kx_c)) x_c - (Ky_n x_n + Ky_c x_s)
//                                           - (Kx_e x_e + Kx_c x_w)
// Load of a field value: plain, or with CG = true through L2 only
// (ld.global.cg), for fields that other blocks of a persistent kernel write
// while it runs (L1 is not coherent across SMs).
template <bool CG>
__device__ __forceinline__ double ldv(const double* p) {
  return CG ? __ldcg(p) : *p;
}

// a * b on the FP64 pipe or, with EMU, on the integer pipes (tea_emu.cuh):
// the same bits either way.
template <bool EMU>
__device__ __forceinline__ double mul_e(double a, double b) {
  return EMU ? emu_dmul(a, b) : a * b;
}

// A x at offset c.  With EMU some products run on the integer pipes (the
// one that starts the chain form, the two that feed no fused multiply-add
// in the fused form, two of the five in the exact form):
// GB300's FP64 pipe bounds the kernels that apply the operator, and moving
// those products off it took calc_w from 206 to 186 us (chain) and from 251
// to 214 us (fused) at 4096^2.  Kernels with high register pressure (the
// Chebyshev step) keep EMU off: the extra registers cost them more than the
// FP64 instructions saved.
// The operator on values: diagonal D, face coefficients Ky_n (Ky of the
// row above), Ky_c, Kx_e (Kx of the column to the right), Kx_c, and x at
// the cell and its north, south, east and west neighbours.
template <int F, bool EMU = true>
__device__ __forceinline__ double smvp_v(double D, double kyn, double kyc, double kxe,
                                         double kxc, double xc, double xn, double xs,
                                         double xe, double xw) {
  if (!F) return D * xc - (mul_e<EMU>(kyn, xn) + kyc * xs) - (mul_e<EMU>(kxe, xe) + kxc * xw);
  if (F == 2) {
    double t = mul_e<EMU>(D, xc);
    t = __fma_rn(-kyn, xn, t);
    t = __fma_rn(-kyc, xs, t);
    t = __fma_rn(-kxe, xe, t);
    return __fma_rn(-kxc, xw, t);
  }
  const double t1 = __fma_rn(kyc, xs, mul_e<EMU>(kyn, xn));
  const double t2 = __fma_rn(kxc, xw, mul_e<EMU>(kxe, xe));
  return __fma_rn(D, xc, -t1) - t2;
}

// b - A x on values: the reference's "b - smvp" (calc_residual,
// tea_leaf_common_cl.cl:17-36; ppcg update_r, tea_leaf_ppcg_cl.cl:62-88),
// or in the chain form the chain of fused multiply-adds started from b.
template <int F>
__device__ __forceinline__ double bms_v(double b, double D, double kyn, double kyc,
                                        double kxe, double kxc, double xc, double xn,
                                        double xs, double xe, double xw) {
  if (F != 2) return b - smvp_v<F>(D, kyn, kyc, kxe, kxc, xc, xn, xs, xe, xw);
  double t = __fma_rn(-D, xc, b);
  t = __fma_rn(kyn, xn, t);
  t = __fma_rn(kyc, xs, t);
  t = __fma_rn(kxe, xe, t);
  return __fma_rn(kxc, xw, t);
}

// The same operator at offset c of the padded fields, written out with the
// loads in place (the kernels' register budgets were tuned on this form);
// its arithmetic is smvp_v's.
template <int F, bool CG = false, bool EMU = true>
__device__ __forceinline__ double smvp(const Dev& d, const double* x,
                                       long long c) {
  const long long S = d.S;
  const double kyn = __ldg(d.Ky + c + S), kyc = __ldg(d.Ky + c);
  const double kxe = __ldg(d.Kx + c + 1), kxc = __ldg(d.Kx + c);
  const double D = __ldg(d.diag + c);
  if (!F)
    return D * ldv<CG>(x + c) -
           (mul_e<EMU>(kyn, ldv<CG>(x + c + S)) + kyc * ldv<CG>(x + c - S)) -
           (mul_e<EMU>(kxe, ldv<CG>(x + c + 1)) + kxc * ldv<CG>(x + c - 1));
  if (F == 2) {
    double t = mul_e<EMU>(D, ldv<CG>(x + c));
    t = __fma_rn(-kyn, ldv<CG>(x + c + S), t);
    t = __fma_rn(-kyc, ldv<CG>(x + c - S), t);
    t = __fma_rn(-kxe, ldv<CG>(x + c + 1), t);
    return __fma_rn(-kxc, ldv<CG>(x + c - 1), t);
  }
  const double t1 = __fma_rn(kyc, ldv<CG>(x + c - S), mul_e<EMU>(kyn, ldv<CG>(x + c + S)));
  const double t2 = __fma_rn(kxc, ldv<CG>(x + c - 1), mul_e<EMU>(kxe, ldv<CG>(x + c + 1)));
  return __fma_rn(D, ldv<CG>(x + c), -t1) - t2;
}

// b - A x at offset c (the arithmetic of bms_v)
template <int F>
__device__ __forceinline__ double b_minus_smvp(const Dev& d, const double* x,
                                               long long c, double b) {
  if (F != 2) return b - smvp<F>(d, x, c);
  const long long S = d.S;
  double t = __fma_rn(-__ldg(d.diag + c), x[c], b);
  t = __fma_rn(__ldg(d.Ky + c + S), x[c + S], t);
  t = __fma_rn(__ldg(d.Ky + c), x[c - S], t);
  t = __fma_rn(__ldg(d.Kx + c + 1), x[c + 1], t);
  return __fma_rn(__ldg(d.Kx + c), x[c - 1], t);
}

// acc + a*b of the per-lane dot-product accumulation
template <int F>
__device__ __forceinline__ double accum(double acc, double a, double b) {
  return F ? __fma_rn(a, b, acc) : acc + a * b;
}

// COEF_B of the block-Jacobi strip (tea_block_jacobi.cl:3) at offset c.
__device__ __forceinline__ double coef_b(const Dev& d, long long c) {
  return (1.0 + (__ldg(d.Ky + c + d.S) + __ldg(d.Ky + c)) +
          (__ldg(d.Kx + c + 1) + __ldg(d.Kx + c)));
}

// Rows in the strip starting at interior row y (BLOCK_TOP, macros_cl.cl:6-10;
// the reference's formula counts one halo row when H == 1 and is exact when
// H == 2; H >= 3 uses the exact count).
__device__ __forceinline__ int strip_rows(const Dev& d, int y) {
  if (!d.block_top_check) return 4;
  const int up = d.y_max - y + (d.H == 1 ? 1 : 0);
  return up < 4 ? up : 4;
}

// One forward step of the strip's Thomas algorithm:
// (r - COEF_A dp) * bfp with COEF_A = -Ky
template <int F, bool EMU = false>
__device__ __forceinline__ double fwd(double r, double ky, double dp,
                                      double bfp) {
  return mul_e<EMU>(F ? __fma_rn(ky, dp, r) : r - (-ky) * dp, bfp);
}

// One back-substitution step: dp - cp z
template <int F>
__device__ __forceinline__ double bwd(double dp, double cp, double z) {
  return F ? __fma_rn(-cp, z, dp) : dp - cp * z;
}

// block_solve_func (tea_block_jacobi.cl:6-42) for one column of one strip:
// z = M_block^-1 r for the strip whose first cell is at offset c0.  With
// EMU the multiplies by bfp run on the integer pipes (same bits).
// The strip solve on values: bfp, Ky and cp of the strip's rows 0..3 (Ky of
// row 0 and cp of row 3 unused), diag of row 0 (exact form only); entries of
// rows at or past `upper` are not read.  FULL: a whole strip (upper == 4),
// without the row tests.
template <int F, bool EMU = false, bool FULL = false>
__device__ __forceinline__ void strip_solve_v(int upper, const double rl[4],
                                              const double bfp[4], const double ky[4],
                                              const double cp[4], double diag0,
                                              double zl[4]) {
  double dp0, dp1 = 0.0, dp2 = 0.0, dp3 = 0.0;
  dp0 = F ? mul_e<EMU>(rl[0], bfp[0]) : emu_ddiv_var(rl[0], diag0);
  if (FULL || upper > 1) dp1 = fwd<F, EMU>(rl[1], ky[1], dp0, bfp[1]);
  if (FULL || upper > 2) dp2 = fwd<F, EMU>(rl[2], ky[2], dp1, bfp[2]);
  if (FULL || upper > 3) dp3 = fwd<F, EMU>(rl[3], ky[3], dp2, bfp[3]);
  double z0, z1 = 0.0, z2 = 0.0, z3 = 0.0;
  if (FULL || upper == 4) {
    z3 = dp3;
    z2 = bwd<F>(dp2, cp[2], z3);
    z1 = bwd<F>(dp1, cp[1], z2);
    z0 = bwd<F>(dp0, cp[0], z1);
  } else if (upper == 3) {
    z2 = dp2;
    z1 = bwd<F>(dp1, cp[1], z2);
    z0 = bwd<F>(dp0, cp[0], z1);
  } else if (upper == 2) {
    z1 = dp1;
    z0 = bwd<F>(dp0, cp[0], z1);
  } else {
    z0 = dp0;
  }
  zl[0] = z0;
  zl[1] = z1;
  zl[2] = z2;
  zl[3] = z3;
}

// The strip solve at offset c0 of the padded fields (the arithmetic of
// strip_solve_v, with the loads in place; only the rows the strip has are
// read, since a strip may end at the top of the allocation).
template <int F, bool EMU = false>
__device__ __forceinline__ void strip_solve(const Dev& d, long long c0,
                                            int upper, const double rl[4],
                                            double zl[4]) {
  const long long S = d.S;
  double dp0, dp1 = 0.0, dp2 = 0.0, dp3 = 0.0;
  dp0 = F ? mul_e<EMU>(rl[0], __ldg(d.bfp + c0)) : emu_ddiv_var(rl[0], __ldg(d.diag + c0));
  if (upper > 1)
    dp1 = fwd<F, EMU>(rl[1], __ldg(d.Ky + c0 + S), dp0, __ldg(d.bfp + c0 + S));
  if (upper > 2)
    dp2 = fwd<F, EMU>(rl[2], __ldg(d.Ky + c0 + 2 * S), dp1, __ldg(d.bfp + c0 + 2 * S));
  if (upper > 3)
    dp3 = fwd<F, EMU>(rl[3], __ldg(d.Ky + c0 + 3 * S), dp2, __ldg(d.bfp + c0 + 3 * S));
  double z0, z1 = 0.0, z2 = 0.0, z3 = 0.0;
  if (upper == 4) {
    z3 = dp3;
    z2 = bwd<F>(dp2, __ldg(d.cp + c0 + 2 * S), z3);
    z1 = bwd<F>(dp1, __ldg(d.cp + c0 + S), z2);
    z0 = bwd<F>(dp0, __ldg(d.cp + c0), z1);
  } else if (upper == 3) {
    z2 = dp2;
    z1 = bwd<F>(dp1, __ldg(d.cp + c0 + S), z2);
    z0 = bwd<F>(dp0, __ldg(d.cp + c0), z1);
  } else if (upper == 2) {
    z1 = dp1;
    z0 = bwd<F>(dp0, __ldg(d.cp + c0), z1);
  } else {
    z0 = dp0;
  }
  zl[0] = z0;
  zl[1] = z1;
  zl[2] = z2;
  zl[3] = z3;
}

// Sum the NV tile sums of the block into per-supertile partials.
template <int NV>
__device__ __forceinline__ void supertile_partial(const Red& red, int s,
                                                  const double* acc,
                                                  double* sh) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) {
#pragma unroll
    for (int v = 0; v < NV; v++) sh[v * 8 + warp] = acc[v];
  }
  __syncthreads();
  if (warp == 0) {
#pragma unroll
    for (int v = 0; v < NV; v++) {
      double t = lane < 8 ? sh[v * 8 + lane] : 0.0;
      t = bfly(t);
      if (lane == 0) red.partials[v * red.stride + s] = t;
    }
  }
  __syncthreads();
}

// Step 4 of the summation order, by one whole block: the ns partials of
// each of the NV sums (NV arrays, `stride` apart) reduced into result[v].
template <int NV>
__device__ __forceinline__ void block_final_sum(const double* partials,
                                                long long stride, int ns,
                                                double* result, double* sh) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll 1
  for (int v = 0; v < NV; v++) {
    double a = 0.0;
    for (int k = threadIdx.x; k < ns; k += kBlock)
      a = a + __ldcg(partials + v * stride + k);
    a = bfly(a);
    if (lane == 0) sh[warp] = a;
    __syncthreads();
    if (warp == 0) {
      double t = lane < 8 ? sh[lane] : 0.0;
      t = bfly(t);
      if (lane == 0) result[v] = t;
    }
    __syncthreads();
  }
}

// The same sum as block_final_sum for one value, handed to every thread of
// the block instead of stored (used by persistent kernels, in which every
// block forms the reduced value itself).  sh holds at least 9 doubles.
__device__ __forceinline__ double block_final_value(const double* partials, int ns,
                                                    double* sh) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  double a = 0.0;
  for (int k = threadIdx.x; k < ns; k += kBlock) a = a + __ldcg(partials + k);
  a = bfly(a);
  if (lane == 0) sh[warp] = a;
  __syncthreads();
  if (warp == 0) {
    double t = lane < 8 ? sh[lane] : 0.0;
    t = bfly(t);
    if (lane == 0) sh[8] = t;
  }
  __syncthreads();
  const double v = sh[8];
  __syncthreads();
  return v;
}

// Barrier across every block of a cooperative launch (all blocks resident).
// bar[0] counts arrivals, bar[1] is the generation.  Every thread's earlier
// global writes are visible to every block after it.  A block waits at most
// spin_limit polls (kBarrierSpins, about 4 s, unless the caller sets
// another); on time-out, or when another block has timed out, it sets *err
// and returns false, and the kernel must return.  The barrier opens when
// gridDim.x + extra blocks have arrived: extra is 0, except in the test that
// makes the wait run out (one arrival more than the grid has, so no block
// opens it).
constexpr long long kBarrierSpins = 1LL << 26;
__device__ __forceinline__ bool grid_barrier(unsigned int* bar, int* err,
                                             long long spin_limit = kBarrierSpins,
                                             unsigned int extra = 0) {
  __shared__ int ok;
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) {
    ok = 1;
    volatile unsigned int* gen = bar + 1;
    const unsigned int g = *gen;
    __threadfence();
    if (atomicAdd(bar, 1u) == gridDim.x - 1 + extra) {
      atomicExch(bar, 0u);
      __threadfence();
      atomicAdd(bar + 1, 1u);
    } else {
      long long spins = 0;
      while (*gen == g) {
        if (++spins > spin_limit || *(volatile int*)err) {
          atomicExch(err, 1);
          ok = 0;
          break;
        }
        __nanosleep(64);
      }
    }
    __threadfence();
  }
  __syncthreads();
  return ok != 0;
}

// Last-block-done finish of the reduction; returns true in the block that
// wrote the results.
template <int NV>
__device__ __forceinline__ bool finish_reduction(const Red& red, int ns,
                                                 double* sh) {
  __shared__ unsigned int is_last;
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) {
    const unsigned int t = atomicAdd(red.counter, 1u);
    is_last = (t == gridDim.x - 1) ? 1u : 0u;
  }
  __syncthreads();
  if (!is_last) return false;
  __threadfence();
  block_final_sum<NV>(red.partials, red.stride, ns, red.result, sh);
  if (threadIdx.x == 0) {
    *red.counter = 0u;
    if (red.host) {
      // thread 0 wrote red.result itself (block_final_sum)
#pragma unroll
      for (int v = 0; v < NV; v++)
        red.host[v] = (unsigned long long)__double_as_longlong(red.result[v]);
      __threadfence_system();
      *(volatile unsigned long long*)(red.host + 8) = 1ull;
    }
  }
  return true;
}

// Four xor butterflies (bfly) at once.  a0..a3 are this lane's values of
// four tiles.  Each stage adds exactly the pairs bfly adds, so every tile
// sum is bit-identical to bfly's; but the tiles share the instructions: 6
// FP64 additions for four tiles instead of 20.  On GB300 the FP64 pipe
// charges a whole warp instruction however few lanes are active, so the
// sharing is what saves time.  On return lanes 0-7 hold tile 0's sum,
// 16-23 tile 1's, 8-15 tile 2's and 24-31 tile 3's.
__device__ __forceinline__ double bfly4(double a0, double a1, double a2, double a3) {
  const int lane = threadIdx.x & 31;
  const bool hi16 = lane & 16, hi8 = lane & 8;
  // off 16: lanes 0-15 carry tiles 0 and 2, lanes 16-31 tiles 1 and 3
  const double r1 = (hi16 ? a1 : a0) +
                    __shfl_xor_sync(0xffffffffu, hi16 ? a0 : a1, 16);
  const double r2 = (hi16 ? a3 : a2) +
                    __shfl_xor_sync(0xffffffffu, hi16 ? a2 : a3, 16);
  // off 8: lanes with bit 8 clear keep r1's tile, lanes with it set r2's
  double r = (hi8 ? r2 : r1) + __shfl_xor_sync(0xffffffffu, hi8 ? r1 : r2, 8);
#pragma unroll
  for (int off = 4; off >= 1; off >>= 1) r = r + __shfl_xor_sync(0xffffffffu, r, off);
  return r;
}

// The slot (0-3) of the tile whose sum bfly4 leaves in this lane's group.
__device__ __forceinline__ int bfly4_slot(int lane) {
  return ((lane >> 4) & 1) | ((lane >> 2) & 2);
}

// Steps 3 of the summation order for four supertiles at once: sh[v*32 +
// k*8 + w] holds warp w's tile sum of value v in supertile k; warp 0 forms
// each supertile sum exactly as supertile_partial does (lanes 8-31 of that
// butterfly hold +0.0, so its first two stages add +0.0 and the last three
// add within lanes 0-7) and stores it at partials[v][s_k].  Called by the
// whole block.
template <int NV>
__device__ __forceinline__ void supertile_partials4(const Red& red, const int* s_k,
                                                    int ns, double* sh) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  __syncthreads();
  if (warp == 0) {
#pragma unroll
    for (int v = 0; v < NV; v++) {
      double t = sh[v * 32 + lane];
      t = t + 0.0;  // the two +0.0 stages: (t + 0) + 0 == t + 0
#pragma unroll
      for (int off = 4; off >= 1; off >>= 1) t = t + __shfl_xor_sync(0xffffffffu, t, off);
      const int k = lane >> 3;
      if ((lane & 7) == 0 && s_k[k] < ns) red.partials[v * red.stride + s_k[k]] = t;
    }
  }
  __syncthreads();
}

// Walks the block's supertiles (s = blockIdx.x + j*gridDim.x);
// body(x, y0, xin, acc) processes the TH rows of one lane's column x
// starting at interior row y0 and adds its contributions row by row into
// acc[0..NV).  With P = 4 the sums of four supertiles share their
// butterflies (bfly4, supertile_partials4); with P = 1 every supertile is
// summed on its own, which needs fewer registers (the FP32 kernels of the
// mixed solve, held to 32 registers for full occupancy, are faster so).
// Both give the same bits.  Returns true in the one block that finished
// the reduction (thread 0 of it holds red.result).
template <int TH, int NV, class Body, int P = 4>
__device__ __forceinline__ bool tile_driver(const Dev& d, const Red& red,
                                            Body body) {
  constexpr int NVV = NV > 0 ? NV : 1;
  __shared__ double sh[NVV * 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (NV > 0 && P == 1) {
    for (int s = blockIdx.x; s < d.ns; s += gridDim.x) {
      const int sy = s / d.nsx, sx = s - sy * d.nsx;
      const int tx = sx * kTilesPerSuper + warp;
      double acc[NVV];
#pragma unroll
      for (int v = 0; v < NVV; v++) acc[v] = 0.0;
      if (tx < d.ntx) {
        const int x = tx * kTileW + lane;
        body(x, sy * TH, x < d.x_max, acc);
#pragma unroll
        for (int v = 0; v < NVV; v++) acc[v] = bfly(acc[v]);
      }
      supertile_partial<NVV>(red, s, acc, sh);
    }
    return finish_reduction<NVV>(red, d.ns, sh);
  }
  if (NV == 0) {
    for (int s = blockIdx.x; s < d.ns; s += gridDim.x) {
      const int sy = s / d.nsx, sx = s - sy * d.nsx;
      const int tx = sx * kTilesPerSuper + warp;
      double acc[NVV] = {0.0};
      if (tx < d.ntx) {
        const int x = tx * kTileW + lane;
        body(x, sy * TH, x < d.x_max, acc);
      }
    }
    return false;
  }
  for (int s0 = blockIdx.x; s0 < d.ns; s0 += 4 * gridDim.x) {
    double tiles[4][NVV];
    int s_k[4];
#pragma unroll 1
    for (int k = 0; k < 4; k++) {
      double acc[NVV];
#pragma unroll
      for (int v = 0; v < NVV; v++) acc[v] = 0.0;
      const int s = s0 + k * gridDim.x;
      if (s < d.ns) {
        const int sy = s / d.nsx, sx = s - sy * d.nsx;
        const int tx = sx * kTilesPerSuper + warp;
        if (tx < d.ntx) {
          const int x = tx * kTileW + lane;
          body(x, sy * TH, x < d.x_max, acc);
        }
      }
      // keep the lane sums in registers (compile-time slots)
#pragma unroll
      for (int q = 0; q < 4; q++)
        if (q == k) {
          s_k[q] = s;
#pragma unroll
          for (int v = 0; v < NVV; v++) tiles[q][v] = acc[v];
        }
    }
#pragma unroll
    for (int v = 0; v < NVV; v++) {
      const double t = bfly4(tiles[0][v], tiles[1][v], tiles[2][v], tiles[3][v]);
      if ((lane & 7) == 0) sh[v * 32 + bfly4_slot(lane) * 8 + warp] = t;
    }
    supertile_partials4<NVV>(red, s_k, d.ns, sh);
  }
  return finish_reduction<NVV>(red, d.ns, sh);
}

// tile_driver summing one supertile at a time (P = 1).
template <int TH, int NV, class Body>
__device__ __forceinline__ bool tile_driver_p1(const Dev& d, const Red& red,
                                               Body body) {
  return tile_driver<TH, NV, Body, 1>(d, red, body);
}

// Copies the halo ring of a field (every padded cell outside the interior,
// depth H) from src to dst; grid-stride over all threads of the launch.
__device__ __forceinline__ void copy_halo_ring(const Dev& d, const double* src, double* dst) {
  const int H = d.H, xs = d.x_max + 2 * H;
  const long long band = (long long)H * xs;  // the rows above or below
  const long long n = 2 * band + 2LL * H * d.y_max;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    int row, col;
    if (i < 2 * band) {
      const long long j = i < band ? i : i - band;
      row = (int)(j / xs) + (i < band ? 0 : H + d.y_max);
      col = (int)(j % xs);
    } else {
      const long long j = i - 2 * band;
      const int k = (int)(j % (2 * H));
      row = H + (int)(j / (2 * H));
      col = k < H ? k : d.x_max + k;
    }
    const long long o = (long long)row * d.S + col;
    dst[o] = src[o];
  }
}

// True in the last block of the grid to get here (counter reset after).
__device__ __forceinline__ bool last_block(unsigned int* counter) {
  __shared__ unsigned int is_last;
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) {
    const unsigned int t = atomicAdd(counter, 1u);
    is_last = (t == gridDim.x - 1) ? 1u : 0u;
    if (is_last) *counter = 0u;
  }
  __syncthreads();
  return is_last != 0u;
}

}  // namespace tea
