// Mixed-precision implicit solve: FP32 inner CG inside an FP64
// defect-correction loop.
//
//   r = u0 - A u            FP64 (the outer residual, on the FP64 fields)
//   repeat until ||r||_2 <= tol * ||r_first||_2:
//     solve A d = r approximately with diagonally preconditioned CG in FP32
//       (FP32 copies of Kx, Ky, the diagonal and its inverse; FP32 vectors
//        d, r, p, w; every dot product summed exactly per lane, then in FP64)
//     u = u + d             FP64
//     r = u0 - A u          FP64
//
// On GB300 the FP64 pipe bounds the FP64 stencils while FP32 stencils run at
// HBM speed with half the bytes, so each inner iteration costs a fraction
// of an FP64 CG iteration; the few FP64 residual passes keep the answer an
// FP64 one.  The inner loop keeps its scalars on the device and runs in
// batches replayed from a CUDA graph, like the FP64 resident CG loop.
//
// Every sum uses the fixed tile order of tea_device.cuh.  Within a lane the
// (at most 16) products of an FP32 dot product are accumulated exactly as
// an unevaluated pair of floats (each product split exactly with a fused
// multiply-add, pairs added with an error-free two-sum), and the pair is
// converted to FP64 once per tile; everything above the lane is FP64.  This
// keeps the FP32 kernels off GB300's slow FP64 pipe.  Every FP32 expression
// is written out with explicit fused multiply-adds, so the CPU oracle
// (oracle_mixed_solve) reproduces the results bit for bit.
#include <math.h>
#include <string.h>

#include <algorithm>
#include <vector>

#include "../../include/tealeaf_gb300.h"
#include "tea_device.cuh"

namespace tea {

// FP32 fields of the mixed solve, padded like the FP64 ones (interior
// column H of each row 256-byte aligned).
struct MixDev {
  long long S;  // row stride in floats
  float *Kx, *Ky, *D, *Mi, *d, *r, *p, *w;
  float *z, *sd;  // PPCG: the kept M^-1 r and the inner direction
  float* p2;      // CG with calc_p folded into calc_w: the other p buffer
};

struct MixState {
  double rro, pw, rrn, alpha, beta, rz0;
  double eps2;  // (inner relative tolerance)^2 * rz0
  int n, max_iters, stop, p_pending;
  int done_iters, pad;
  double* alphas;  // CG alpha and beta by iteration number (PPCG presteps)
  double* betas;
};

struct MixChunk {
  bool ready = false;
  int x_max = 0, y_max = 0, H = 0;
  long long S = 0;
  float* base[11] = {nullptr};
  MixDev dev{};
  MixState* st = nullptr;    // device
  MixState* st_h = nullptr;  // pinned
  unsigned int* counter = nullptr;
  cudaGraphExec_t graph = nullptr;
  cudaGraphExec_t graph_fused = nullptr;  // CG with calc_p folded into calc_w
  int graph_batch = 0;
  int graph_epoch = 0;  // the chunk's field_epoch at capture
};

static MixChunk g_mix;

// Rows per load group of the one-column FP32 kernels (k_mix_calc_w and the
// PPCG kernels), and their minimum resident blocks per SM.  Measured at
// 4096^2 (ms per CG inner iteration, before the 4-column kernels below):
// groups of 1/2/4 rows at 8 blocks/SM (32 registers) 0.229/0.240/0.252,
// groups of 4 or 8 rows without the bound 0.277/0.303.
template <int TH>
constexpr int kGroup = 1;
constexpr int kMixMinBlocks = 8;

__device__ __forceinline__ long long cidx32(const Dev& d, const MixDev& m, int x,
                                            int y) {
  return (long long)(y + d.H) * m.S + (x + d.H);
}

// FP32 5-point operator with fused multiply-adds:
// D x_c - (Ky_n x_n + Ky_c x_s) - (Kx_e x_e + Kx_c x_w)
__device__ __forceinline__ float smvp32(const MixDev& m, const float* x,
                                        long long c) {
  const long long S = m.S;
  const float kyn = __ldg(m.Ky + c + S), kyc = __ldg(m.Ky + c);
  const float kxe = __ldg(m.Kx + c + 1), kxc = __ldg(m.Kx + c);
  const float t1 = __fmaf_rn(kyc, x[c - S], kyn * x[c + S]);
  const float t2 = __fmaf_rn(kxc, x[c - 1], kxe * x[c + 1]);
  return __fmaf_rn(__ldg(m.D + c), x[c], -t1) - t2;
}

// (hi, lo) += a*b, exactly up to the pair's rounding: the product is split
// into p + e with e = fma(a, b, -p), and p is added with a two-sum.
__device__ __forceinline__ void acc_pair(float& hi, float& lo, float a,
                                         float b) {
  const float p = a * b;
  const float e = __fmaf_rn(a, b, -p);
  const float s = hi + p;
  const float bb = s - hi;
  const float t = (hi - (s - bb)) + (p - bb);
  lo = lo + (t + e);
  hi = s;
}

__device__ __forceinline__ double pair_value(float hi, float lo) {
  return (double)hi + (double)lo;
}

// FP32 copies of the operator over the whole padded array:
// Kx, Ky rounded to nearest; D and Mi = 1/D from the FP64 diagonal.
__global__ void k_mix_convert(Dev d, MixDev m) {
  const int col = blockIdx.x * blockDim.x + threadIdx.x;
  const int row = blockIdx.y * blockDim.y + threadIdx.y;
  if (col > d.xs || row > d.ys) return;
  const long long c64 = (long long)row * d.S + col;
  const long long c32 = (long long)row * m.S + col;
  m.Kx[c32] = (float)d.Kx[c64];
  m.Ky[c32] = (float)d.Ky[c64];
  const bool in = col >= d.H && col < d.H + d.x_max && row >= d.H &&
                  row < d.H + d.y_max;
  const double D = in ? d.diag[c64] : 1.0;
  m.D[c32] = (float)D;
  m.Mi[c32] = (float)(1.0 / D);
}

// The outer step: r64 = u0 - A u (FP64, fused form), then the inner start
// r32 = (float)r64, d = 0, z = Mi r32, p = z.  Sums: r64.r64 and r32.z.
template <int TH>
__global__ void __launch_bounds__(kBlock)
    k_mix_residual(Dev d, MixDev m, Red red) {
  tile_driver_p1<TH, 2>(d, red, [&](int x, int y0, bool xin, double* acc) {
    float hi = 0.0f, lo = 0.0f;
#pragma unroll 1
    for (int g = y0; g < y0 + TH; g += 4) {
      double r64[4];
      float r32[4], z[4];
#pragma unroll
      for (int j = 0; j < 4; j++) {
        r64[j] = 0.0;
        r32[j] = z[j] = 0.0f;
        if (xin && g + j < d.y_max) {
          const long long c = cidx(d, x, g + j);
          r64[j] = d.u0[c] - smvp<1>(d, d.u, c);
          r32[j] = (float)r64[j];
          z[j] = m.Mi[cidx32(d, m, x, g + j)] * r32[j];
        }
      }
#pragma unroll
      for (int j = 0; j < 4; j++) {
        if (xin && g + j < d.y_max) {
          const long long c3 = cidx32(d, m, x, g + j);
          d.r[cidx(d, x, g + j)] = r64[j];
          m.r[c3] = r32[j];
          m.p[c3] = z[j];
          m.d[c3] = 0.0f;
        }
        acc[0] = __fma_rn(r64[j], r64[j], acc[0]);
        acc_pair(hi, lo, r32[j], z[j]);
      }
    }
    acc[1] = pair_value(hi, lo);
  });
}

// w = A p, sum p.w
template <int TH>
__global__ void __launch_bounds__(kBlock, kMixMinBlocks)
    k_mix_calc_w(Dev d, MixDev m, Red red, MixState* st) {
  if (*(volatile int*)&st->stop) return;
  const bool last = tile_driver_p1<TH, 1>(d, red, [&](int x, int y0, bool xin, double* acc) {
    float hi = 0.0f, lo = 0.0f;
    constexpr int GR = kGroup<TH>;
#pragma unroll 1
    for (int g = y0; g < y0 + TH; g += GR) {
      float pv[GR], wv[GR];
#pragma unroll
      for (int j = 0; j < GR; j++) {
        pv[j] = wv[j] = 0.0f;
        if (xin && g + j < d.y_max) {
          const long long c3 = cidx32(d, m, x, g + j);
          wv[j] = smvp32(m, m.p, c3);
          pv[j] = m.p[c3];
        }
      }
#pragma unroll
      for (int j = 0; j < GR; j++) {
        if (xin && g + j < d.y_max) m.w[cidx32(d, m, x, g + j)] = wv[j];
        acc_pair(hi, lo, pv[j], wv[j]);
      }
    }
    acc[0] = pair_value(hi, lo);
  });
  if (last && threadIdx.x == 0) st->pw = red.result[0];
}

// ---- FP32 iteration kernels with 16-byte accesses ----
//
// One-column FP32 kernels put 4 bytes per lane into every memory request,
// half of FP64's, and ran at about 70 % of HBM.  With float4 accesses the
// CG inner iteration at 4096^2 went from 0.229 ms to 0.217 ms (calc_p)
// and 0.197 ms (calc_w and calc_ur too); 4 blocks per SM measured best
// (5 and 6: 0.210 and 0.220 ms).
//
// Every thread takes 4 adjacent columns (one float4) of one tile; 8 threads
// cover a tile's 32 columns and 64 threads a supertile, so a 256-thread
// block works on 4 supertiles (s0 + k*gridDim.x, k = 0..3) at once.  Each
// column's lane sum is accumulated exactly as in the one-column kernels.
// The tile's xor butterfly over its 32 columns runs on 4 values per
// thread: the stages xor 16, 8, 4 become shuffles xor 4, 2, 1 between the
// tile's 8 threads, and the stages xor 2, 1 happen within a thread.  Every
// stage adds the same pairs, so the sums are bit-identical.

__device__ __forceinline__ float4 ld4(const float* p) {
  return *reinterpret_cast<const float4*>(p);
}
__device__ __forceinline__ float f4(const float4& v, int k) {
  return k == 0 ? v.x : k == 1 ? v.y : k == 2 ? v.z : v.w;
}

// Walks 4 supertiles per block and round; body(x, y0, v) gives v[k], the
// lane sum of interior column x+k of the tile rows y0..y0+TH-1 (0.0 for
// columns past the interior).  Forms the supertile partials and finishes
// the reduction in the last block (thread 0 of it holds red.result).
template <int TH, class Body>
__device__ __forceinline__ bool quad_driver(const Dev& d, const Red& red, Body body) {
  __shared__ double sh[32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int grp = warp >> 1;                       // supertile slot
  const int tile = 4 * (warp & 1) + (lane >> 3);   // tile within the supertile
  const int q = lane & 7;                          // column quad within the tile
  for (int s0 = blockIdx.x; s0 < d.ns; s0 += 4 * gridDim.x) {
    const int s = s0 + grp * gridDim.x;
    double v[4] = {0.0, 0.0, 0.0, 0.0};
    if (s < d.ns) {
      const int sy = s / d.nsx, sx = s - sy * d.nsx;
      const int tx = sx * kTilesPerSuper + tile;
      if (tx < d.ntx) body(tx * kTileW + 4 * q, sy * TH, v);
    }
#pragma unroll
    for (int off = 4; off >= 1; off >>= 1) {
#pragma unroll
      for (int k = 0; k < 4; k++) v[k] = v[k] + __shfl_xor_sync(0xffffffffu, v[k], off);
    }
    const double t = (v[0] + v[2]) + (v[1] + v[3]);
    if (q == 0) sh[grp * 8 + tile] = t;
    int s_k[4];
#pragma unroll
    for (int k = 0; k < 4; k++) s_k[k] = s0 + k * gridDim.x;
    supertile_partials4<1>(red, s_k, d.ns, sh);
  }
  return finish_reduction<1>(red, d.ns, sh);
}

// w = A p and p.w (k_mix_calc_w's values), 4 columns per thread
template <int TH>
__global__ void __launch_bounds__(kBlock, 4)
    k_mix_calc_w4(Dev d, MixDev m, Red red, MixState* st) {
  if (*(volatile int*)&st->stop) return;
  const bool last = quad_driver<TH>(d, red, [&](int x, int y0, double* v) {
    const long long S = m.S;
    float hi[4] = {0.0f, 0.0f, 0.0f, 0.0f}, lo[4] = {0.0f, 0.0f, 0.0f, 0.0f};
    const bool full = x + 4 <= d.x_max;
#pragma unroll 1
    for (int j = 0; j < TH; j++) {
      const int y = y0 + j;
      float pv[4] = {0.0f, 0.0f, 0.0f, 0.0f}, wv[4] = {0.0f, 0.0f, 0.0f, 0.0f};
      if (y < d.y_max) {
        const long long c = cidx32(d, m, x, y);
        if (full) {
          const float4 pc = ld4(m.p + c), pn = ld4(m.p + c + S), ps = ld4(m.p + c - S);
          const float4 kx = ld4(m.Kx + c), kyc = ld4(m.Ky + c), kyn = ld4(m.Ky + c + S);
          const float4 D = ld4(m.D + c);
          const float pwst = m.p[c - 1], peas = m.p[c + 4], kx4 = m.Kx[c + 4];
#pragma unroll
          for (int k = 0; k < 4; k++) {
            const float xw = k == 0 ? pwst : f4(pc, k - 1);
            const float xe = k == 3 ? peas : f4(pc, k + 1);
            const float ke = k == 3 ? kx4 : f4(kx, k + 1);
            const float t1 = __fmaf_rn(f4(kyc, k), f4(ps, k), f4(kyn, k) * f4(pn, k));
            const float t2 = __fmaf_rn(f4(kx, k), xw, ke * xe);
            wv[k] = __fmaf_rn(f4(D, k), f4(pc, k), -t1) - t2;
            pv[k] = f4(pc, k);
          }
          *reinterpret_cast<float4*>(m.w + c) = make_float4(wv[0], wv[1], wv[2], wv[3]);
        } else {
#pragma unroll
          for (int k = 0; k < 4; k++)
            if (x + k < d.x_max) {
              wv[k] = smvp32(m, m.p, c + k);
              pv[k] = m.p[c + k];
              m.w[c + k] = wv[k];
            }
        }
      }
#pragma unroll
      for (int k = 0; k < 4; k++) acc_pair(hi[k], lo[k], pv[k], wv[k]);
    }
#pragma unroll
    for (int k = 0; k < 4; k++) v[k] = pair_value(hi[k], lo[k]);
  });
  if (last && threadIdx.x == 0) st->pw = red.result[0];
}

// calc_p folded into calc_w (CG inner loop of the mixed solve): with the
// previous iteration's beta, p' = Mi r + beta p (k_mix_calc_p_v4's fused
// multiply-add per cell) is formed where w = A p' needs it, from the old p,
// Mi and r: each lane walks its 4 columns down the tile keeping p' of the
// rows above, at and below, and forms the columns either side itself.
// Halo cells keep the old p, as calc_p leaves them.  p' is written to pout
// (other blocks still read the old p for their operator), w and p'.w as
// k_mix_calc_w4.  On the first iteration of an inner solve (no calc_p
// pending) p' is p.  In FP32 the extra multiply-adds are cheap; the pass
// over p, Mi and r that calc_p made disappears with its launch.
template <int TH>
__global__ void __launch_bounds__(kBlock, 4)
    k_mix_calc_pw4(Dev d, MixDev m, float* pout, Red red, MixState* st) {
  if (*(volatile int*)&st->stop) return;
  const bool pend = *(volatile int*)&st->p_pending != 0;
  const float bf = (float)st->beta;
  const bool last = quad_driver<TH>(d, red, [&](int x, int y0, double* v) {
    const long long S = m.S;
    const float* __restrict__ pin = m.p;
    const float* __restrict__ mi = m.Mi;
    const float* __restrict__ rr = m.r;
    float* __restrict__ w = m.w;
    float* __restrict__ po = pout;
    // p' of one interior cell, or the old p elsewhere
    auto pn1 = [&](long long c, int xx, int y) -> float {
      const float pv = pin[c];
      if (!pend || xx < 0 || xx >= d.x_max || y < 0 || y >= d.y_max) return pv;
      return __fmaf_rn(bf, pv, mi[c] * rr[c]);
    };
    float hi[4] = {0.0f, 0.0f, 0.0f, 0.0f}, lo[4] = {0.0f, 0.0f, 0.0f, 0.0f};
    if (x + 4 <= d.x_max) {
      // p' of the 4 columns at row y (a halo row keeps the old p)
      auto pn4 = [&](long long c, int y) -> float4 {
        const float4 pv = ld4(pin + c);
        if (!pend || y < 0 || y >= d.y_max) return pv;
        const float4 m4 = ld4(mi + c), r4 = ld4(rr + c);
        return make_float4(__fmaf_rn(bf, pv.x, m4.x * r4.x), __fmaf_rn(bf, pv.y, m4.y * r4.y),
                           __fmaf_rn(bf, pv.z, m4.z * r4.z), __fmaf_rn(bf, pv.w, m4.w * r4.w));
      };
      const long long cb = cidx32(d, m, x, y0);
      float4 ps = pn4(cb - S, y0 - 1), pc = pn4(cb, y0);
#pragma unroll 1
      for (int j = 0; j < TH; j++) {
        const int y = y0 + j;
        float pv[4] = {0.0f, 0.0f, 0.0f, 0.0f}, wv[4] = {0.0f, 0.0f, 0.0f, 0.0f};
        if (y < d.y_max) {
          const long long c = cb + j * S;
          const float4 pnr = pn4(c + S, y + 1);
          const float4 kx = ld4(m.Kx + c), kyc = ld4(m.Ky + c), kyn = ld4(m.Ky + c + S);
          const float4 D = ld4(m.D + c);
          const float pwst = pn1(c - 1, x - 1, y), peas = pn1(c + 4, x + 4, y);
          const float kx4 = m.Kx[c + 4];
#pragma unroll
          for (int k = 0; k < 4; k++) {
            const float xw = k == 0 ? pwst : f4(pc, k - 1);
            const float xe = k == 3 ? peas : f4(pc, k + 1);
            const float ke = k == 3 ? kx4 : f4(kx, k + 1);
            const float t1 = __fmaf_rn(f4(kyc, k), f4(ps, k), f4(kyn, k) * f4(pnr, k));
            const float t2 = __fmaf_rn(f4(kx, k), xw, ke * xe);
            wv[k] = __fmaf_rn(f4(D, k), f4(pc, k), -t1) - t2;
            pv[k] = f4(pc, k);
          }
          *reinterpret_cast<float4*>(w + c) = make_float4(wv[0], wv[1], wv[2], wv[3]);
          *reinterpret_cast<float4*>(po + c) = pc;
          ps = pc;
          pc = pnr;
        }
#pragma unroll
        for (int k = 0; k < 4; k++) acc_pair(hi[k], lo[k], pv[k], wv[k]);
      }
    } else {
#pragma unroll 1
      for (int j = 0; j < TH; j++) {
        const int y = y0 + j;
        float pv[4] = {0.0f, 0.0f, 0.0f, 0.0f}, wv[4] = {0.0f, 0.0f, 0.0f, 0.0f};
        if (y < d.y_max) {
          const long long c = cidx32(d, m, x, y);
#pragma unroll
          for (int k = 0; k < 4; k++)
            if (x + k < d.x_max) {
              const long long ck = c + k;
              const float pc = pn1(ck, x + k, y);
              const float t1 = __fmaf_rn(__ldg(m.Ky + ck), pn1(ck - S, x + k, y - 1),
                                         __ldg(m.Ky + ck + S) * pn1(ck + S, x + k, y + 1));
              const float t2 = __fmaf_rn(__ldg(m.Kx + ck), pn1(ck - 1, x + k - 1, y),
                                         __ldg(m.Kx + ck + 1) * pn1(ck + 1, x + k + 1, y));
              wv[k] = __fmaf_rn(__ldg(m.D + ck), pc, -t1) - t2;
              pv[k] = pc;
              w[ck] = wv[k];
              po[ck] = pc;
            }
        }
#pragma unroll
        for (int k = 0; k < 4; k++) acc_pair(hi[k], lo[k], pv[k], wv[k]);
      }
    }
#pragma unroll
    for (int k = 0; k < 4; k++) v[k] = pair_value(hi[k], lo[k]);
  });
  if (last && threadIdx.x == 0) {
    st->pw = red.result[0];
    st->p_pending = 0;
    __threadfence();
  }
}

// d += alpha p; r -= alpha w; z = Mi r; r.z and the inner loop's scalar
// step (k_mix_calc_ur's values), 4 columns per thread
template <int TH>
__global__ void __launch_bounds__(kBlock, 4)
    k_mix_calc_ur4(Dev d, MixDev m, Red red, MixState* st) {
  if (*(volatile int*)&st->stop) return;
  const double alpha = st->rro / st->pw;
  const float af = (float)alpha;
  const bool last = quad_driver<TH>(d, red, [&](int x, int y0, double* v) {
    float hi[4] = {0.0f, 0.0f, 0.0f, 0.0f}, lo[4] = {0.0f, 0.0f, 0.0f, 0.0f};
    const bool full = x + 4 <= d.x_max;
#pragma unroll 1
    for (int j = 0; j < TH; j++) {
      const int y = y0 + j;
      float rv[4] = {0.0f, 0.0f, 0.0f, 0.0f}, zv[4] = {0.0f, 0.0f, 0.0f, 0.0f};
      if (y < d.y_max) {
        const long long c = cidx32(d, m, x, y);
        if (full) {
          const float4 p4 = ld4(m.p + c), d4 = ld4(m.d + c), w4 = ld4(m.w + c);
          const float4 r4 = ld4(m.r + c), mi4 = ld4(m.Mi + c);
          float dv[4];
#pragma unroll
          for (int k = 0; k < 4; k++) {
            dv[k] = __fmaf_rn(af, f4(p4, k), f4(d4, k));
            rv[k] = __fmaf_rn(-af, f4(w4, k), f4(r4, k));
            zv[k] = f4(mi4, k) * rv[k];
          }
          *reinterpret_cast<float4*>(m.d + c) = make_float4(dv[0], dv[1], dv[2], dv[3]);
          *reinterpret_cast<float4*>(m.r + c) = make_float4(rv[0], rv[1], rv[2], rv[3]);
        } else {
#pragma unroll
          for (int k = 0; k < 4; k++)
            if (x + k < d.x_max) {
              const long long ck = c + k;
              const float dk = __fmaf_rn(af, m.p[ck], m.d[ck]);
              rv[k] = __fmaf_rn(-af, m.w[ck], m.r[ck]);
              zv[k] = m.Mi[ck] * rv[k];
              m.d[ck] = dk;
              m.r[ck] = rv[k];
            }
        }
      }
#pragma unroll
      for (int k = 0; k < 4; k++) acc_pair(hi[k], lo[k], rv[k], zv[k]);
    }
#pragma unroll
    for (int k = 0; k < 4; k++) v[k] = pair_value(hi[k], lo[k]);
  });
  if (last && threadIdx.x == 0) {
    const double rrn = red.result[0];
    st->alpha = alpha;
    st->beta = rrn / st->rro;
    if (st->alphas) {
      st->alphas[st->n] = alpha;
      st->betas[st->n] = st->beta;
    }
    st->rrn = rrn;
    st->rro = rrn;
    st->p_pending = 1;
    st->done_iters = st->n;
    if (rrn <= st->eps2 || st->n >= st->max_iters)
      st->stop = 1;
    else
      st->n = st->n + 1;
    __threadfence();
  }
}

// p = Mi r + beta p with 16-byte loads: each thread updates 4 adjacent
// columns of 8 rows.  FP32 loads of 4 bytes per lane put half the bytes of
// FP64 into every memory request; float4 requests carry 16 bytes per lane.
// The values are those of k_mix_calc_p (the same fused multiply-add per
// cell).  Interior column 0 of every row is 256-byte aligned.
__global__ void __launch_bounds__(kBlock)
    k_mix_calc_p_v4(Dev d, MixDev m, MixState* st, unsigned int* counter) {
  if (!*(volatile int*)&st->p_pending) return;
  const float bf = (float)st->beta;
  const int nq = (d.x_max + 3) / 4, ng = (d.y_max + 7) / 8;
  const long long items = (long long)nq * ng;
  for (long long it = (long long)blockIdx.x * blockDim.x + threadIdx.x; it < items;
       it += (long long)gridDim.x * blockDim.x) {
    const int q = (int)(it % nq), g = (int)(it / nq);
    const int x = 4 * q, y0 = 8 * g;
    const int rows = min(8, d.y_max - y0);
    if (x + 4 <= d.x_max) {
      float4 pv[8];
#pragma unroll
      for (int j = 0; j < 8; j++) {
        if (j < rows) {
          const long long c3 = cidx32(d, m, x, y0 + j);
          const float4 p4 = *reinterpret_cast<const float4*>(m.p + c3);
          const float4 m4 = *reinterpret_cast<const float4*>(m.Mi + c3);
          const float4 r4 = *reinterpret_cast<const float4*>(m.r + c3);
          pv[j] = make_float4(__fmaf_rn(bf, p4.x, m4.x * r4.x), __fmaf_rn(bf, p4.y, m4.y * r4.y),
                              __fmaf_rn(bf, p4.z, m4.z * r4.z), __fmaf_rn(bf, p4.w, m4.w * r4.w));
        }
      }
#pragma unroll
      for (int j = 0; j < 8; j++)
        if (j < rows) *reinterpret_cast<float4*>(m.p + cidx32(d, m, x, y0 + j)) = pv[j];
    } else {
      for (int j = 0; j < rows; j++)
        for (int k = x; k < d.x_max; k++) {
          const long long c3 = cidx32(d, m, k, y0 + j);
          m.p[c3] = __fmaf_rn(bf, m.p[c3], m.Mi[c3] * m.r[c3]);
        }
    }
  }
  if (last_block(counter) && threadIdx.x == 0) {
    st->p_pending = 0;
    __threadfence();
  }
}

// ---- FP32 PPCG inner solve (the FP64 driver's tea_leaf PPCG branch,
// tea_solve.f90:240-268 and :422-475, restated in FP32 with diagonal
// Jacobi): after the CG presteps, one iteration is calc_w, the u/r update
// keeping z = M^-1 r, inner_steps Chebyshev steps on d and r, r.z with the
// kept z, and p = z + beta p.

// d += alpha p; r -= alpha w; z = Mi r (no sum: PPCG takes r.z after its
// inner steps)
template <int TH>
__global__ void __launch_bounds__(kBlock, kMixMinBlocks)
    k_mix_ppcg_ur(Dev d, MixDev m, Red red, MixState* st) {
  if (*(volatile int*)&st->stop) return;
  const double alpha = st->rro / st->pw;
  const float af = (float)alpha;
  tile_driver<TH, 0>(d, red, [&](int x, int y0, bool xin, double* acc) {
    if (!xin) return;
#pragma unroll 1
    for (int y = y0; y < y0 + TH && y < d.y_max; y++) {
      const long long c3 = cidx32(d, m, x, y);
      const float dv = __fmaf_rn(af, m.p[c3], m.d[c3]);
      const float rv = __fmaf_rn(-af, m.w[c3], m.r[c3]);
      m.d[c3] = dv;
      m.r[c3] = rv;
      m.z[c3] = m.Mi[c3] * rv;
    }
  });
}

// sd = (Mi r) / theta (tea_leaf_ppcg_solve_init_sd)
template <int TH>
__global__ void __launch_bounds__(kBlock, kMixMinBlocks)
    k_mix_ppcg_init_sd(Dev d, MixDev m, Red red, MixState* st, float theta) {
  if (*(volatile int*)&st->stop) return;
  tile_driver<TH, 0>(d, red, [&](int x, int y0, bool xin, double* acc) {
    if (!xin) return;
#pragma unroll 1
    for (int y = y0; y < y0 + TH && y < d.y_max; y++) {
      const long long c3 = cidx32(d, m, x, y);
      m.sd[c3] = (m.Mi[c3] * m.r[c3]) / theta;
    }
  });
}

// d += sd; r -= A sd (tea_leaf_ppcg_solve_update_r)
template <int TH>
__global__ void __launch_bounds__(kBlock, kMixMinBlocks)
    k_mix_ppcg_update_r(Dev d, MixDev m, Red red, MixState* st) {
  if (*(volatile int*)&st->stop) return;
  tile_driver<TH, 0>(d, red, [&](int x, int y0, bool xin, double* acc) {
    if (!xin) return;
#pragma unroll 1
    for (int y = y0; y < y0 + TH && y < d.y_max; y++) {
      const long long c3 = cidx32(d, m, x, y);
      const float dv = m.d[c3] + m.sd[c3];
      const float rv = m.r[c3] - smvp32(m, m.sd, c3);
      m.d[c3] = dv;
      m.r[c3] = rv;
    }
  });
}

// sd = a sd + b (Mi r) (tea_leaf_ppcg_solve_calc_sd)
template <int TH>
__global__ void __launch_bounds__(kBlock, kMixMinBlocks)
    k_mix_ppcg_calc_sd(Dev d, MixDev m, Red red, MixState* st, float a, float b) {
  if (*(volatile int*)&st->stop) return;
  tile_driver<TH, 0>(d, red, [&](int x, int y0, bool xin, double* acc) {
    if (!xin) return;
#pragma unroll 1
    for (int y = y0; y < y0 + TH && y < d.y_max; y++) {
      const long long c3 = cidx32(d, m, x, y);
      m.sd[c3] = __fmaf_rn(a, m.sd[c3], b * (m.Mi[c3] * m.r[c3]));
    }
  });
}

// r.z with the z kept by k_mix_ppcg_ur; the last block takes the scalar
// step and the exit test of the iteration
template <int TH>
__global__ void __launch_bounds__(kBlock, kMixMinBlocks)
    k_mix_ppcg_rz(Dev d, MixDev m, Red red, MixState* st) {
  if (*(volatile int*)&st->stop) return;
  const bool last = tile_driver_p1<TH, 1>(d, red, [&](int x, int y0, bool xin, double* acc) {
    float hi = 0.0f, lo = 0.0f;
#pragma unroll 4
    for (int j = 0; j < TH; j++) {
      const int y = y0 + j;
      float rv = 0.0f, zv = 0.0f;
      if (xin && y < d.y_max) {
        const long long c3 = cidx32(d, m, x, y);
        rv = m.r[c3];
        zv = m.z[c3];
      }
      acc_pair(hi, lo, rv, zv);
    }
    acc[0] = pair_value(hi, lo);
  });
  if (last && threadIdx.x == 0) {
    const double rrn = red.result[0];
    st->beta = rrn / st->rro;
    st->rrn = rrn;
    st->rro = rrn;
    st->p_pending = 1;
    st->done_iters = st->n;
    if (rrn <= st->eps2 || st->n >= st->max_iters)
      st->stop = 1;
    else
      st->n = st->n + 1;
    __threadfence();
  }
}

// p = z + beta p with the kept z
template <int TH>
__global__ void __launch_bounds__(kBlock, kMixMinBlocks)
    k_mix_ppcg_calc_p(Dev d, MixDev m, Red red, MixState* st, unsigned int* counter) {
  if (!*(volatile int*)&st->p_pending) return;
  const float bf = (float)st->beta;
  tile_driver<TH, 0>(d, red, [&](int x, int y0, bool xin, double* acc) {
    if (!xin) return;
#pragma unroll 1
    for (int y = y0; y < y0 + TH && y < d.y_max; y++) {
      const long long c3 = cidx32(d, m, x, y);
      m.p[c3] = __fmaf_rn(bf, m.p[c3], m.z[c3]);
    }
  });
  if (last_block(counter) && threadIdx.x == 0) {
    st->p_pending = 0;
    __threadfence();
  }
}

// u = u + d (FP64 accumulation of the FP32 correction)
template <int TH>
__global__ void __launch_bounds__(kBlock) k_mix_update_u(Dev d, MixDev m, Red red) {
  tile_driver<TH, 0>(d, red, [&](int x, int y0, bool xin, double* acc) {
    if (!xin) return;
#pragma unroll 1
    for (int g = y0; g < y0 + TH; g += 4) {
      double uv[4];
#pragma unroll
      for (int j = 0; j < 4; j++)
        if (g + j < d.y_max)
          uv[j] = d.u[cidx(d, x, g + j)] + (double)m.d[cidx32(d, m, x, g + j)];
#pragma unroll
      for (int j = 0; j < 4; j++)
        if (g + j < d.y_max) d.u[cidx(d, x, g + j)] = uv[j];
    }
  });
}

template <class... KArgs>
static int mix_grid(Chunk& c, void (*kernel)(KArgs...), int ns = 0) {
  int n = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, (const void*)kernel, kBlock, 0) !=
          cudaSuccess ||
      n < 1)
    n = 1;
  const long long cap = (long long)c.num_sms * n;
  return (int)std::max<long long>(1, std::min<long long>(ns > 0 ? ns : c.dev().ns, cap));
}

template <int TH>
static void enqueue_inner(Chunk& c, int iters) {
  const Dev d = c.dev();
  const Red red = c.red();
  const MixDev m = g_mix.dev;
  const int nblk4 = (d.ns + 3) / 4;  // 4 supertiles per block and round
  const int gw = mix_grid(c, k_mix_calc_w4<TH>, nblk4);
  const int gu = mix_grid(c, k_mix_calc_ur4<TH>, nblk4);
  const int gp = mix_grid(c, k_mix_calc_p_v4,
                          (int)std::min<long long>(1 << 30, ((long long)(d.x_max + 3) / 4 *
                                                             ((d.y_max + 7) / 8) + kBlock - 1) /
                                                                kBlock));
  for (int i = 0; i < iters; i++) {
    k_mix_calc_w4<TH><<<gw, kBlock, 0, c.stream>>>(d, m, red, g_mix.st);
    k_mix_calc_ur4<TH><<<gu, kBlock, 0, c.stream>>>(d, m, red, g_mix.st);
    k_mix_calc_p_v4<<<gp, kBlock, 0, c.stream>>>(d, m, g_mix.st, g_mix.counter);
  }
}

// The CG inner loop with calc_p folded into calc_w: iteration i reads p
// from one buffer and writes p' to the other, so an even count ends where
// it began.
template <int TH>
static void enqueue_inner_fused(Chunk& c, int iters) {
  const Dev d = c.dev();
  const Red red = c.red();
  MixDev m[2] = {g_mix.dev, g_mix.dev};
  m[1].p = g_mix.dev.p2;
  const int nblk4 = (d.ns + 3) / 4;
  const int gw = mix_grid(c, k_mix_calc_pw4<TH>, nblk4);
  const int gu = mix_grid(c, k_mix_calc_ur4<TH>, nblk4);
  for (int i = 0; i < iters; i++) {
    const int a = i & 1, b = a ^ 1;
    k_mix_calc_pw4<TH><<<gw, kBlock, 0, c.stream>>>(d, m[a], m[b].p, red, g_mix.st);
    k_mix_calc_ur4<TH><<<gu, kBlock, 0, c.stream>>>(d, m[b], red, g_mix.st);
  }
}

void mixed_release() {
  MixChunk& g = g_mix;
  if (g.graph) cudaGraphExecDestroy(g.graph);
  if (g.graph_fused) cudaGraphExecDestroy(g.graph_fused);
  for (float*& b : g.base) {
    cudaFree(b);
    b = nullptr;
  }
  cudaFree(g.st);
  cudaFree(g.counter);
  cudaFreeHost(g.st_h);
  g = MixChunk();
}

static bool mixed_alloc(Chunk& c) {
  MixChunk& g = g_mix;
  if (g.ready && g.x_max == c.x_max && g.y_max == c.y_max && g.H == c.H) return true;
  mixed_release();
  g.x_max = c.x_max;
  g.y_max = c.y_max;
  g.H = c.H;
  g.S = ((long long)(c.x_max + 2 * c.H + 1 + 63) / 64) * 64;
  const long long off = (64 - (c.H % 64)) % 64;
  const size_t n = (size_t)(off + (c.y_max + 2 * c.H + 1) * g.S + 64);
  float** f[11] = {&g.dev.Kx, &g.dev.Ky, &g.dev.D, &g.dev.Mi, &g.dev.d, &g.dev.r,
                   &g.dev.p,  &g.dev.w,  &g.dev.z, &g.dev.sd, &g.dev.p2};
  for (int i = 0; i < 11; i++) {
    if (!check_cuda(cudaMalloc(&g.base[i], n * sizeof(float)), "cudaMalloc mixed field"))
      return false;
    cudaMemsetAsync(g.base[i], 0, n * sizeof(float), c.stream);
    *f[i] = g.base[i] + off;
  }
  g.dev.S = g.S;
  if (!check_cuda(cudaMalloc(&g.st, sizeof(MixState)), "cudaMalloc mixed state") ||
      !check_cuda(cudaMallocHost(&g.st_h, sizeof(MixState)), "cudaMallocHost") ||
      !check_cuda(cudaMalloc(&g.counter, sizeof(unsigned int)), "cudaMalloc counter"))
    return false;
  cudaMemsetAsync(g.counter, 0, sizeof(unsigned int), c.stream);
  g.ready = true;
  return true;
}

template <int TH>
static void enqueue_ppcg(Chunk& c, int iters, float theta, const std::vector<float>& ca,
                         const std::vector<float>& cb) {
  const Dev d = c.dev();
  const Red red = c.red();
  const MixDev m = g_mix.dev;
  MixState* st = g_mix.st;
  const int gw = mix_grid(c, k_mix_calc_w<TH>);
  const int gu = mix_grid(c, k_mix_ppcg_ur<TH>);
  const int gs = mix_grid(c, k_mix_ppcg_init_sd<TH>);
  const int gr = mix_grid(c, k_mix_ppcg_update_r<TH>);
  const int gd = mix_grid(c, k_mix_ppcg_calc_sd<TH>);
  const int gz = mix_grid(c, k_mix_ppcg_rz<TH>);
  const int gp = mix_grid(c, k_mix_ppcg_calc_p<TH>);
  for (int i = 0; i < iters; i++) {
    k_mix_calc_w<TH><<<gw, kBlock, 0, c.stream>>>(d, m, red, st);
    k_mix_ppcg_ur<TH><<<gu, kBlock, 0, c.stream>>>(d, m, red, st);
    k_mix_ppcg_init_sd<TH><<<gs, kBlock, 0, c.stream>>>(d, m, red, st, theta);
    for (size_t k = 0; k < ca.size(); k++) {
      k_mix_ppcg_update_r<TH><<<gr, kBlock, 0, c.stream>>>(d, m, red, st);
      k_mix_ppcg_calc_sd<TH><<<gd, kBlock, 0, c.stream>>>(d, m, red, st, ca[k], cb[k]);
    }
    k_mix_ppcg_rz<TH><<<gz, kBlock, 0, c.stream>>>(d, m, red, st);
    k_mix_ppcg_calc_p<TH><<<gp, kBlock, 0, c.stream>>>(d, m, red, st, g_mix.counter);
  }
}

// Captures `enqueue` on the chunk's stream into an executable graph.
template <class F>
static cudaGraphExec_t mix_capture(Chunk& c, F enqueue) {
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  if (!check_cuda(cudaStreamBeginCapture(c.stream, cudaStreamCaptureModeThreadLocal),
                  "mixed graph capture"))
    return nullptr;
  enqueue();
  if (!check_cuda(cudaStreamEndCapture(c.stream, &graph), "mixed graph capture end"))
    return nullptr;
  const bool ok = check_cuda(cudaGraphInstantiate(&exec, graph, 0), "mixed graph instantiate");
  cudaGraphDestroy(graph);
  return ok ? exec : nullptr;
}

// Uploads h, replays `graph` (iters_per_replay iterations, `kernels`
// kernels each) until the inner loop has stopped, and reads h back.
static bool run_inner(Chunk& c, cudaGraphExec_t graph, int iters_per_replay, int kernels,
                      MixState& h, bool stop_only = false) {
  MixChunk& g = g_mix;
  if (!check_cuda(cudaMemcpyAsync(g.st, &h, sizeof(MixState), cudaMemcpyHostToDevice,
                                  c.stream),
                  "mixed state upload"))
    return false;
  const long long max_batches = (long long)(h.max_iters - h.n) / iters_per_replay + 3;
  for (long long nb = 0;; nb++) {
    if (nb >= max_batches) {
      fail(40, "mixed inner loop did not stop after %lld batches", nb);
      return false;
    }
    if (!check_cuda(cudaGraphLaunch(graph, c.stream), "mixed graph launch")) return false;
    count_launches(kernels);
    if (!check_cuda(cudaMemcpyAsync(&h, g.st, sizeof(MixState), cudaMemcpyDeviceToHost,
                                    c.stream),
                    "mixed state read") ||
        !check_cuda(cudaStreamSynchronize(c.stream), "mixed sync"))
      return false;
    // the loop with calc_p folded into calc_w leaves the last p' unformed:
    // a CG correction starts again from p = z
    if (h.stop && (stop_only || !h.p_pending)) return true;
  }
}

template <int TH>
static bool mixed_solve_t(Chunk& c, double tol, double inner_tol, int max_outer,
                          int max_inner, int solver, int presteps, int inner_steps,
                          tea_gb300_mixed_info* info) {
  MixChunk& g = g_mix;
  const Dev d = c.dev();
  const Red red = c.red();
  const int batch = 16, ppcg_batch = 4;
  {
    const dim3 block(32, 8), grid((d.xs + 1 + 31) / 32, (d.ys + 1 + 7) / 8);
    k_mix_convert<<<grid, block, 0, c.stream>>>(d, g.dev);
    count_launch("mixed_convert");
  }
  if (g.graph && g.graph_epoch != c.field_epoch) {
    cudaGraphExecDestroy(g.graph);  // the chunk's r/sd buffers have traded places
    g.graph = nullptr;
    if (g.graph_fused) cudaGraphExecDestroy(g.graph_fused);
    g.graph_fused = nullptr;
  }
  if (!g.graph) {
    g.graph = mix_capture(c, [&]() { enqueue_inner<TH>(c, batch); });
    if (!g.graph) return false;
    g.graph_batch = batch;
    g.graph_epoch = c.field_epoch;
  }
  if (!g.graph_fused) {
    g.graph_fused = mix_capture(c, [&]() { enqueue_inner_fused<TH>(c, batch); });
    if (!g.graph_fused) return false;
  }
  double res[2];
  auto outer_residual = [&](double* out) -> bool {
    k_mix_residual<TH><<<mix_grid(c, k_mix_residual<TH>), kBlock, 0, c.stream>>>(d, g.dev, red);
    count_launch("mixed_residual");
    if (!check_cuda(cudaMemcpyAsync(c.host_result, c.red_result, 2 * sizeof(double),
                                    cudaMemcpyDeviceToHost, c.stream),
                    "mixed residual read") ||
        !check_cuda(cudaStreamSynchronize(c.stream), "mixed residual sync"))
      return false;
    out[0] = c.host_result[0];
    out[1] = c.host_result[1];
    return true;
  };
  // PPCG: the first correction's CG presteps give the eigenvalue range
  // (tea_solve.f90:175-210), kept for the later corrections of this call
  const bool ppcg = solver == SOLVER_PPCG;
  bool have_eigs = false, eig_failed = false;
  double* coef_d = nullptr;
  cudaGraphExec_t ppcg_graph = nullptr;
  auto cleanup = [&](bool ok) {
    if (ppcg_graph) cudaGraphExecDestroy(ppcg_graph);
    cudaFree(coef_d);
    return ok;
  };
  if (ppcg && !check_cuda(cudaMalloc(&coef_d, 2 * sizeof(double) * (presteps + 2)),
                          "cudaMalloc mixed coefficients"))
    return false;
  if (!outer_residual(res)) return cleanup(false);
  const double rr_first = res[0];
  info->initial_residual = sqrt(rr_first);
  int outer = 0;
  long long inner_total = 0, cheby_total = 0;
  while (!(sqrt(res[0]) <= tol * sqrt(rr_first)) && outer < max_outer) {
    MixState h;
    memset(&h, 0, sizeof(h));
    h.rro = res[1];
    h.rz0 = res[1];
    // the last corrections only need the reduction still missing (with a
    // margin of 4), never less than inner_tol
    const double need = 0.25 * tol * sqrt(rr_first) / sqrt(res[0]);
    const double itol = need > inner_tol ? (need < 0.5 ? need : 0.5) : inner_tol;
    h.eps2 = itol * itol * res[1];
    h.n = 1;
    h.max_iters = max_inner;
    bool use_ppcg = ppcg && have_eigs;
    if (ppcg && !have_eigs && !eig_failed) {
      h.max_iters = std::min(presteps, max_inner);
      h.alphas = coef_d;
      h.betas = coef_d + presteps + 2;
      if (!run_inner(c, g.graph, batch, 3 * batch, h)) return cleanup(false);
      const bool converged = h.rrn <= h.eps2;
      if (!converged && h.done_iters < max_inner) {
        const int n = h.done_iters;
        std::vector<double> ab(2 * (presteps + 2));
        if (!check_cuda(cudaMemcpy(ab.data(), coef_d, ab.size() * sizeof(double),
                                   cudaMemcpyDeviceToHost),
                        "mixed coefficients read"))
          return cleanup(false);
        const std::vector<double> a(ab.begin() + 1, ab.begin() + 1 + n);
        const std::vector<double> b(ab.begin() + presteps + 3,
                                    ab.begin() + presteps + 3 + n);
        double eigmin = 0.0, eigmax = 0.0;
        if (eigenvalues_from_cg(a, b, n, &eigmin, &eigmax) != 0) {
          eig_failed = true;  // the rest of the solve stays CG
        } else {
          std::vector<double> cha, chb;
          double theta = 0.0;
          chebyshev_coefficients(cha, chb, eigmin * 0.95, eigmax * 1.05, &theta,
                                 inner_steps);
          std::vector<float> ca(inner_steps), cb(inner_steps);
          for (int k = 0; k < inner_steps; k++) {
            ca[k] = (float)cha[k];
            cb[k] = (float)chb[k];
          }
          const float tf = (float)theta;
          ppcg_graph = mix_capture(c, [&]() { enqueue_ppcg<TH>(c, ppcg_batch, tf, ca, cb); });
          if (!ppcg_graph) return cleanup(false);
          have_eigs = true;
          use_ppcg = true;
        }
        // continue this inner solve from where the presteps stopped
        h.stop = 0;
        h.n = n + 1;
        h.max_iters = max_inner;
      }
      h.alphas = h.betas = nullptr;
      if (h.stop) {
        inner_total += h.done_iters;
      } else {
        const int pre = h.done_iters;
        if (use_ppcg) {
          if (!run_inner(c, ppcg_graph, ppcg_batch, ppcg_batch * (5 + 2 * inner_steps), h))
            return cleanup(false);
          cheby_total += (long long)(h.done_iters - pre) * inner_steps;
        } else if (!run_inner(c, g.graph, batch, 3 * batch, h)) {
          return cleanup(false);
        }
        inner_total += h.done_iters;
      }
    } else {
      if (use_ppcg) {
        if (!run_inner(c, ppcg_graph, ppcg_batch, ppcg_batch * (5 + 2 * inner_steps), h))
          return cleanup(false);
        cheby_total += (long long)h.done_iters * inner_steps;
      } else if (!run_inner(c, g.graph_fused, batch, 2 * batch, h, true)) {
        return cleanup(false);
      }
      inner_total += h.done_iters;
    }
    k_mix_update_u<TH><<<mix_grid(c, k_mix_update_u<TH>), kBlock, 0, c.stream>>>(d, g.dev, red);
    count_launch("mixed_update_u");
    outer++;
    if (!outer_residual(res)) return cleanup(false);
  }
  info->outer_iterations = outer;
  info->inner_iterations = inner_total;
  info->ppcg_inner_steps = cheby_total;
  info->final_residual = sqrt(res[0]);
  info->relative_residual = sqrt(res[0]) / sqrt(rr_first);
  return cleanup(true);
}

}  // namespace tea

using namespace tea;

static int mixed_entry(double tol, double inner_tol, int max_outer, int max_inner,
                       int solver, int presteps, int inner_steps,
                       tea_gb300_mixed_info* info, const char* who) {
  Chunk& c = chunk();
  if (!c.ready) {
    fail(5, "%s called before initialise_ocl_", who);
    return -1;
  }
  if (!(tol > 0.0) || !(inner_tol > 0.0) || inner_tol >= 1.0 || max_outer < 1 ||
      max_inner < 1 || !info ||
      (solver == SOLVER_PPCG && (presteps < 1 || inner_steps < 1 || inner_steps > 1000))) {
    fail(41, "%s: invalid arguments", who);
    return -1;
  }
  memset(info, 0, sizeof(*info));
  if (!mixed_alloc(c)) return -1;
  const bool ok =
      c.TH == 16 ? mixed_solve_t<16>(c, tol, inner_tol, max_outer, max_inner, solver,
                                     presteps, inner_steps, info)
                 : mixed_solve_t<4>(c, tol, inner_tol, max_outer, max_inner, solver,
                                    presteps, inner_steps, info);
  return ok ? 0 : -1;
}

extern "C" int tea_gb300_mixed_solve(double tol, double inner_tol, int max_outer,
                                     int max_inner, tea_gb300_mixed_info* info) {
  return mixed_entry(tol, inner_tol, max_outer, max_inner, SOLVER_CG, 0, 0, info,
                     "tea_gb300_mixed_solve");
}

extern "C" int tea_gb300_mixed_solve_ppcg(double tol, double inner_tol, int max_outer,
                                          int max_inner, int presteps, int inner_steps,
                                          tea_gb300_mixed_info* info) {
  return mixed_entry(tol, inner_tol, max_outer, max_inner, SOLVER_PPCG, presteps,
                     inner_steps, info, "tea_gb300_mixed_solve_ppcg");
}
