// CUDA kernels of the per-call C ABI, one per reference kernel (or fused
// pair), each citing the OpenCL kernel whose arithmetic it reproduces.
// Interior kernels use the tile walk of tea_device.cuh; setup and
// whole-array kernels use plain 2-D grids.
#include <algorithm>
#include <unordered_map>

#include "tea_cg.cuh"
#include "tea_device.cuh"

namespace tea {

// ---------------------------------------------------------------------------
// launch helpers
// ---------------------------------------------------------------------------

static int blocks_per_sm(const void* fn) {
  static std::unordered_map<const void*, int> cache;
  auto it = cache.find(fn);
  if (it != cache.end()) return it->second;
  int n = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, fn, kBlock, 0) !=
          cudaSuccess ||
      n < 1)
    n = 1;
  cache[fn] = n;
  return n;
}

template <class... KArgs, class... Args>
static void launch_tile(Chunk& c, const char* name, void (*kernel)(KArgs...),
                        Args... args) {
  const Dev d = c.dev();
  const long long cap = (long long)c.num_sms * blocks_per_sm((const void*)kernel);
  const int grid = (int)std::max<long long>(1, std::min<long long>(d.ns, cap));
  profile_begin(name);
  kernel<<<grid, kBlock, 0, c.stream>>>(args...);
  count_launch(name);
  check_cuda(cudaGetLastError(), name);
  profile_end(name);
}

// A kernel that takes no sum computes the same values whatever its tile
// height, so it may run over 4-row tiles: four times as many, smaller work
// items as the 16-row tiles of the summing kernels, and no long last wave
// of blocks (4096 16-row supertiles at 4096^2 make 4.5 rounds of 912
// blocks).  Measured at 4096^2: update_r 194 -> 191 us, calc_sd 163 -> 159,
// calc_residual 161 -> 155, calc_p 64.5 -> 62.7, finalise 253 -> 245.
// Chebyshev calc_p (352 -> 362) and the FP32 calc_p of the mixed solve got
// slower, so they keep the 16-row tiles.
Dev rows4_tiling(Dev d) {
  d.th = 4;
  d.nty = (d.y_max + 3) / 4;
  d.ns = d.nsx * d.nty;
  return d;
}

static Dev dev4(const Chunk& c) { return rows4_tiling(c.dev()); }



template <class... KArgs, class... Args>
static void launch_tile_ns(Chunk& c, const char* name, int ns, void (*kernel)(KArgs...),
                           Args... args) {
  const long long cap = (long long)c.num_sms * blocks_per_sm((const void*)kernel);
  const int grid = (int)std::max<long long>(1, std::min<long long>(ns, cap));
  profile_begin(name);
  kernel<<<grid, kBlock, 0, c.stream>>>(args...);
  count_launch(name);
  check_cuda(cudaGetLastError(), name);
  profile_end(name);
}

// TH_DISPATCH for kernels that take no sum: 4-row tiles (dev4)
#define TH4_DISPATCH(c, name, kern, d4, ...)                           \
  do {                                                                 \
    if ((c).arith == 2)                                                \
      launch_tile_ns(c, name, (d4).ns, kern<4, 2>, d4, __VA_ARGS__);   \
    else if ((c).arith == 1)                                           \
      launch_tile_ns(c, name, (d4).ns, kern<4, 1>, d4, __VA_ARGS__);   \
    else                                                               \
      launch_tile_ns(c, name, (d4).ns, kern<4, 0>, d4, __VA_ARGS__);   \
  } while (0)

template <class... KArgs, class... Args>
static void launch_2d(Chunk& c, const char* name, int nx, int ny,
                      void (*kernel)(KArgs...), Args... args) {
  if (nx <= 0 || ny <= 0) return;
  const dim3 block(32, 8);
  const dim3 grid((nx + 31) / 32, (ny + 7) / 8);
  profile_begin(name);
  kernel<<<grid, block, 0, c.stream>>>(args...);
  count_launch(name);
  check_cuda(cudaGetLastError(), name);
  profile_end(name);
}

#define TH_DISPATCH(c, name, kern, ...)                  \
  do {                                                   \
    if ((c).TH == 16) {                                  \
      if ((c).arith == 2)                                \
        launch_tile(c, name, kern<16, 2>, __VA_ARGS__);  \
      else if ((c).arith == 1)                           \
        launch_tile(c, name, kern<16, 1>, __VA_ARGS__);  \
      else                                               \
        launch_tile(c, name, kern<16, 0>, __VA_ARGS__);  \
    } else {                                             \
      if ((c).arith == 2)                                \
        launch_tile(c, name, kern<4, 2>, __VA_ARGS__);   \
      else if ((c).arith == 1)                           \
        launch_tile(c, name, kern<4, 1>, __VA_ARGS__);   \
      else                                               \
        launch_tile(c, name, kern<4, 0>, __VA_ARGS__);   \
    }                                                    \
  } while (0)

// ---------------------------------------------------------------------------
// setup kernels
// ---------------------------------------------------------------------------

// initialise_chunk_first, initialise_chunk_cl.cl:3-49 (1-D arrays)
__global__ void k_init_chunk_1d(Dev d, double xmin, double ymin, double dx,
                                double dy) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int H = d.H;
  if (i <= d.x_max + H) {
    d.vertexx[i] = xmin + dx * (double)(((i)-1) - H + 1);
    d.vertexdx[i] = dx;
    const double plus1 = xmin + dx * (double)((i)-H + 1);
    d.cellx[i] = 0.5 * (d.vertexx[i] + plus1);
    d.celldx[i] = dx;
  }
  if (i <= d.y_max + H) {
    d.vertexy[i] = ymin + dy * (double)(((i)-1) - H + 1);
    d.vertexdy[i] = dy;
    const double plus1 = ymin + dy * (double)((i)-H + 1);
    d.celly[i] = 0.5 * (d.vertexy[i] + plus1);
    d.celldy[i] = dy;
  }
}

// initialise_chunk_second, initialise_chunk_cl.cl:51-68 (volume only; no
// kernel of the solve reads xarea/yarea)
__global__ void k_volume(Dev d, double vol) {
  const int col = d.H - 1 + blockIdx.x * blockDim.x + threadIdx.x;
  const int row = d.H - 1 + blockIdx.y * blockDim.y + threadIdx.y;
  if (col <= d.x_max + d.H && row <= d.y_max + d.H)
    d.volume[(long long)row * d.S + col] = vol;
}

// generate_chunk_init, generate_chunk_cl.cl:82-95
__global__ void k_gen_init(Dev d, double dens0, double en0) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  if (x < d.x_max && y < d.y_max) {
    const long long c = cidx(d, x, y);
    d.energy0[c] = en0;
    d.density[c] = dens0;
  }
}

// generate_chunk, generate_chunk_cl.cl:3-65, one state
__global__ void k_gen_state(Dev d, double dens, double en, double sxmin,
                            double sxmax, double symin, double symax,
                            double srad, int geom, int g_rect, int g_circ,
                            int g_point) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  if (x >= d.x_max || y >= d.y_max) return;
  const int col = x + d.H, row = y + d.H;
  const double x_cent = sxmin, y_cent = symin;
  bool hit = false;
  if (g_rect == geom) {
    hit = d.vertexx[1 + col] >= sxmin && d.vertexx[col] < sxmax &&
          d.vertexy[1 + row] >= symin && d.vertexy[row] < symax;
  } else if (geom == g_circ) {
    const double x_pos = d.cellx[col] - x_cent;
    const double y_pos = d.celly[row] - y_cent;
    const double radius = sqrt(x_pos * x_pos + y_pos * y_pos);
    hit = radius <= srad;
  } else if (geom == g_point) {
    hit = d.vertexx[col] == x_cent && d.vertexy[row] == y_cent;
  }
  if (hit) {
    const long long c = cidx(d, x, y);
    d.energy0[c] = en;
    d.density[c] = dens;
  }
}

// generate_chunk_init_u, generate_chunk_cl.cl:67-80
__global__ void k_init_u(Dev d, const double* __restrict__ energy) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  if (x < d.x_max && y < d.y_max) {
    const long long c = cidx(d, x, y);
    d.u[c] = energy[c] * d.density[c];
    d.u0[c] = energy[c] * d.density[c];
  }
}

// set_field, set_field_cl.cl:3-13
__global__ void k_set_field(Dev d) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  if (x < d.x_max && y < d.y_max) {
    const long long c = cidx(d, x, y);
    d.energy1[c] = d.energy0[c];
  }
}

// ---------------------------------------------------------------------------
// whole-array solver kernels
// ---------------------------------------------------------------------------

// tea_leaf_init_common, tea_leaf_common_cl.cl:56-90, over
// [1, x_max+2H) x [1, y_max+2H)
__global__ void k_init_common(Dev d, int coef, double rx, double ry) {
  const int col = 1 + blockIdx.x * blockDim.x + threadIdx.x;
  const int row = 1 + blockIdx.y * blockDim.y + threadIdx.y;
  if (col >= d.xs || row >= d.ys) return;
  const long long c = (long long)row * d.S + col;
  double dc = 0.0, dl = 0.0, dd = 0.0;
  if (coef == 1) {
    dc = d.density[c];
    dl = d.density[c - 1];
    dd = d.density[c - d.S];
  } else if (coef == 2) {
    dc = emu_ddiv_var(1.0, d.density[c]);
    dl = emu_ddiv_var(1.0, d.density[c - 1]);
    dd = emu_ddiv_var(1.0, d.density[c - d.S]);
  }
  double kx = emu_ddiv_var(dl + dc, 2.0 * dl * dc);
  kx = kx * rx;
  double ky = emu_ddiv_var(dd + dc, 2.0 * dd * dc);
  ky = ky * ry;
  d.Kx[c] = kx;
  d.Ky[c] = ky;
}

// tea_leaf_zero_boundary, tea_leaf_common_cl.cl:92-125, whole padded array
__global__ void k_zero_boundary(Dev d, int zl, int zr, int zb, int zt) {
  const int col = blockIdx.x * blockDim.x + threadIdx.x;
  const int row = blockIdx.y * blockDim.y + threadIdx.y;
  if (col >= d.xs || row >= d.ys) return;
  const long long c = (long long)row * d.S + col;
  const int H = d.H;
  if (zl && col <= H) {
    d.Kx[c] = 0;
    if (col < H) d.Ky[c] = 0;
  }
  if (zr && col > (d.x_max - 1) + H) {
    d.Kx[c] = 0;
    d.Ky[c] = 0;
  }
  if (zb && row <= H) {
    d.Ky[c] = 0;
    if (row < H) d.Kx[c] = 0;
  }
  if (zt && row > (d.y_max - 1) + H) {
    d.Ky[c] = 0;
    d.Kx[c] = 0;
  }
}

// tea_leaf_init_jac_diag, tea_leaf_common_cl.cl:127-142, whole padded array
__global__ void k_init_jac_diag(Dev d) {
  const int col = blockIdx.x * blockDim.x + threadIdx.x;
  const int row = blockIdx.y * blockDim.y + threadIdx.y;
  if (col >= d.xs || row >= d.ys) return;
  const long long c = (long long)row * d.S + col;
  const double diag = (1.0 + (d.Ky[c + d.S] + d.Ky[c]) + (d.Kx[c + 1] + d.Kx[c]));
  d.Mi[c] = emu_ddiv_var(1.0, diag);
}

// tea_leaf_block_init, tea_block_jacobi.cl:78-105: one thread per column of
// one 4-row strip
__global__ void k_block_init(Dev d, int fused) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int g = blockIdx.y * blockDim.y + threadIdx.y;
  if (x >= d.x_max || 4 * g >= d.y_max) return;
  const int upper = strip_rows(d, 4 * g);
  const long long S = d.S;
  const long long c0 = cidx(d, x, 4 * g);
  double cpv = emu_ddiv_var(-d.Ky[c0 + S], coef_b(d, c0));
  d.cp[c0] = cpv;
  // the fused form divides by COEF_B of the first row through its
  // reciprocal, kept in the otherwise unused bfp of that row
  if (fused) d.bfp[c0] = emu_ddiv_var(1.0, coef_b(d, c0));
  for (int k = 1; k < upper; k++) {
    const long long ck = c0 + k * S;
    const double b = emu_ddiv_var(1.0, coef_b(d, ck) - (-d.Ky[ck]) * cpv);
    d.bfp[ck] = b;
    cpv = (-d.Ky[ck + S]) * b;
    d.cp[ck] = cpv;
  }
}

// update_halo_{bottom,top,left,right} (update_halo_cl.cl:3-69) fused: every
// cell of the depth-wide ring takes the value of its mirror image in the
// interior; corners mirror in both directions, which is what the
// reference's bottom/top-then-left/right order produces.  Sources are
// interior cells only, so the single pass has no hazards.
__global__ void k_update_halo(Dev d, int mask, int depth) {
  const int H = d.H;
  const int col = H - depth + blockIdx.x * blockDim.x + threadIdx.x;
  const int row = H - depth + blockIdx.y * blockDim.y + threadIdx.y;
  const int ce = d.x_max + H, re = d.y_max + H;
  if (col >= ce + depth || row >= re + depth) return;
  const bool cin = col >= H && col < ce, rin = row >= H && row < re;
  if (cin && rin) return;
  const int mc = col < H ? 2 * H - 1 - col : (col >= ce ? 2 * ce - 1 - col : col);
  const int mr = row < H ? 2 * H - 1 - row : (row >= re ? 2 * re - 1 - row : row);
  const long long dst = (long long)row * d.S + col;
  const long long src = (long long)mr * d.S + mc;
  if (mask & 1) d.density[dst] = d.density[src];
  if (mask & 2) d.energy0[dst] = d.energy0[src];
  if (mask & 4) d.energy1[dst] = d.energy1[src];
}

// ---------------------------------------------------------------------------
// interior tile kernels (TH: reduction tile height, F: fused arithmetic)
//
// Launch bounds are chosen per kernel by measurement at 4096^2.  Writing the
// minimum of one block per SM explicitly changes ptxas's register budget:
// faster for update_r (48 -> 56 registers, 192 -> 182 us), dot (67 -> 61
// us), cheby calc_u (62.4 -> 59.5), field_summary (277 -> 267),
// calc_residual (155 -> 153) and cg calc_p (63.3 -> 62.0); slower for
// calc_ur (240 -> 289), cg init_p (139 -> 196), init_sd, calc_w (186 ->
// 308) and the Chebyshev step, which keep the plain bound.  calc_w, with
// its fields through restrict-qualified pointers (cg_w_tile_r), names 4
// blocks per SM instead: 64 registers with a 16-byte spill, 192.2 -> 174.4
// us on non-zero fields (92 registers and 3 blocks per SM without it).  So
// do calc_ur and PPCG's calc_ur + init_sd (cg_ur_tile_r): 246.4 -> 210.9
// and 223.7 -> 215.0 us.
// ---------------------------------------------------------------------------

// tea_leaf_calc_residual, tea_leaf_common_cl.cl:17-36
template <int TH, int F>
__global__ void __launch_bounds__(kBlock, 1) k_calc_residual(Dev d, Red red) {
  tile_driver<TH, 0>(d, red, [&](int x, int y0, bool xin, double* acc) {
    if (!xin) return;
#pragma unroll 1
    for (int g = y0; g < y0 + TH; g += 4) {
      const long long c0 = cidx(d, x, g);
      double rv[4];
#pragma unroll
      for (int j = 0; j < 4; j++)
        if (g + j < d.y_max) {
          const long long c = c0 + j * d.S;
          rv[j] = b_minus_smvp<F>(d, d.u, c, d.u0[c]);
        }
#pragma unroll
      for (int j = 0; j < 4; j++)
        if (g + j < d.y_max) d.r[c0 + j * d.S] = rv[j];
    }
  });
}

// tea_leaf_calc_2norm, tea_leaf_common_cl.cl:38-54
template <int TH, int F>
__global__ void __launch_bounds__(kBlock, 1)
    k_dot(Dev d, Red red, const double* a, const double* b) {
  tile_driver<TH, 1>(d, red, [&](int x, int y0, bool xin, double* acc) {
#pragma unroll 4
    for (int j = 0; j < TH; j++) {
      const int y = y0 + j;
      double av = 0.0, bv = 0.0;
      if (xin && y < d.y_max) {
        const long long c = cidx(d, x, y);
        av = a[c];
        bv = b[c];
      }
      acc[0] = accum<F>(acc[0], av, bv);
    }
  });
}

// tea_leaf_block_solve (tea_block_jacobi.cl:44-76) fused with
// tea_leaf_cg_solve_init_p (tea_leaf_cg_cl.cl:8-41): z = M^-1 r, p = z,
// sum r.p
template <int TH, int F>
__global__ void __launch_bounds__(kBlock) k_cg_init_p(Dev d, Red red) {
  tile_driver<TH, 1>(d, red, [&](int x, int y0, bool xin, double* acc) {
    if (d.prec == PREC_JAC_BLOCK) {
#pragma unroll 1
      for (int ys = y0; ys < y0 + TH; ys += 4) {
        double zl[4] = {0.0, 0.0, 0.0, 0.0}, rl[4] = {0.0, 0.0, 0.0, 0.0};
        const long long c0 = cidx(d, x, ys);
        if (xin && ys < d.y_max) {
#pragma unroll
          for (int i = 0; i < 4; i++)
            rl[i] = (ys + i < d.y_max) ? d.r[c0 + i * d.S] : 0.0;
          strip_solve<F>(d, c0, strip_rows(d, ys), rl, zl);
        }
#pragma unroll
        for (int i = 0; i < 4; i++) {
          double av = 0.0, bv = 0.0;
          if (xin && ys + i < d.y_max) {
            const long long c = c0 + i * d.S;
            d.z[c] = zl[i];
            d.p[c] = zl[i];
            av = rl[i];
            bv = zl[i];
          }
          acc[0] = accum<F>(acc[0], av, bv);
        }
      }
    } else {
#pragma unroll 1
      for (int g = y0; g < y0 + TH; g += 4) {
        const long long c0 = cidx(d, x, g);
        double rv[4], pv[4];
#pragma unroll
        for (int j = 0; j < 4; j++) {
          rv[j] = pv[j] = 0.0;
          if (xin && g + j < d.y_max) {
            rv[j] = d.r[c0 + j * d.S];
            pv[j] = d.prec == PREC_JAC_DIAG ? rv[j] * d.Mi[c0 + j * d.S] : rv[j];
          }
        }
#pragma unroll
        for (int j = 0; j < 4; j++)
          if (xin && g + j < d.y_max) {
            if (d.prec == PREC_JAC_DIAG) d.z[c0 + j * d.S] = pv[j];
            d.p[c0 + j * d.S] = pv[j];
          }
#pragma unroll
        for (int j = 0; j < 4; j++) acc[0] = accum<F>(acc[0], rv[j], pv[j]);
      }
    }
  });
}

// tea_leaf_cg_solve_calc_w, tea_leaf_cg_cl.cl:45-69.  With st != nullptr
// (device-resident loop) it does nothing once the loop has stopped and
// leaves pw in st.
template <int TH, int F>
__global__ void __launch_bounds__(kBlock, 4)
    k_cg_calc_w(Dev d, Red red, ResState* st) {
  if (st && *(volatile int*)&st->stop) return;
  const bool last = tile_driver<TH, 1>(d, red, [&](int x, int y0, bool xin, double* acc) {
    cg_w_tile_r<TH, F>(d, x, y0, xin, acc);
  });
  if (st && last && threadIdx.x == 0) st->pw = red.result[0];
}

// tea_leaf_cg_solve_calc_ur, tea_leaf_cg_cl.cl:73-137.  In the
// device-resident loop alpha = rro/pw is formed here, and the block that
// finishes the reduction carries out the host steps of one CG iteration
// (cg_scalar_step).  With NV = 2 it also sums r.r, for the resident loop's
// optional exit test on the unpreconditioned residual.
// With r.r as well (NV = 2) the restrict-qualified body needs more registers
// than 4 blocks per SM leave (202.5 against 188.7 us at 4096^2, diagonal
// Jacobi), so that variant keeps cg_ur_tile at 3 blocks per SM.
template <int TH, int F, int NV = 1>
__global__ void __launch_bounds__(kBlock, NV == 2 ? 3 : 4)
    k_cg_calc_ur(Dev d, Red red, double alpha, ResState* st) {
  if (st) {
    if (*(volatile int*)&st->stop) return;
    alpha = st->rro / st->pw;
  }
  const bool last = tile_driver<TH, NV>(d, red, [&](int x, int y0, bool xin, double* acc) {
    if constexpr (NV == 2)
      cg_ur_tile<TH, F, NV>(d, x, y0, xin, acc, alpha);
    else
      cg_ur_tile_r<TH, F, NV>(d, x, y0, xin, acc, alpha);
  });
  if (st && last && threadIdx.x == 0) {
    cg_scalar_step<NV>(st, alpha, red.result);
    __threadfence();
  }
}

// tea_leaf_cg_solve_calc_ur with its r.z, and PPCG's init_sd
// (tea_leaf_ppcg_cl.cl:4-60) from the z it forms, into d.sd (the spare
// buffer, so the current sd stays as it is until init_sd is called).
template <int TH, int F>
__global__ void __launch_bounds__(kBlock, 4)
    k_cg_calc_ur_sd(Dev d, Red red, double alpha, DivConst theta) {
  tile_driver<TH, 1>(d, red, [&](int x, int y0, bool xin, double* acc) {
    cg_ur_tile_r<TH, F, 1, true>(d, x, y0, xin, acc, alpha, theta);
  });
}

// tea_leaf_cg_solve_calc_p, tea_leaf_cg_cl.cl:141-160.  In the
// device-resident loop it runs once per calc_ur that ran, with that
// iteration's beta.
template <int TH, int F>
__global__ void __launch_bounds__(kBlock, 1)
    k_cg_calc_p(Dev d, Red red, double beta, ResState* st,
                unsigned int* counter) {
  if (st) {
    if (!*(volatile int*)&st->p_pending) return;
    beta = st->beta;
  }
  tile_driver<TH, 0>(d, red, [&](int x, int y0, bool xin, double* acc) {
    cg_p_tile<TH, F>(d, x, y0, xin, beta);
  });
  if (st && last_block(counter) && threadIdx.x == 0) {
    st->p_pending = 0;
    __threadfence();
  }
}

// a p + bl br: the Chebyshev / PPCG coefficient update
// alpha p + beta M^-1 r of tea_leaf_cheby_cl.cl:134-144 and
// tea_leaf_ppcg_cl.cl:137-152, with bl br = beta z, (beta Mi) r, beta r or
// (beta r) Mi as each reference expression groups it
template <int F>
__device__ __forceinline__ double cheby_update(double a, double p, double bl,
                                               double br) {
  return F ? __fma_rn(a, p, bl * br) : a * p + bl * br;
}

// One Chebyshev iteration with the block-Jacobi preconditioner alone, in
// one pass: tea_leaf_cheby_solve_calc_p (tea_leaf_cheby_cl.cl:78-145) and
// then tea_leaf_cheby_solve_calc_u (u = u + p, :66-76) on the p it has just
// formed.  Only this path compiled in (k_cheby_p's mode-1 block path alone
// took 72 registers against 80, 340 -> 326 us at 4096^2).  The product
// beta z runs on the integer pipes (tea_emu.cuh, bit-identical): on non-zero
// fields 340.2 -> 315.6 us; the operator's first product there as well was
// slower (367.0 us), and so were the sweep's multiplies by bfp (388 us),
// which sit on each strip's dependent chain.  The new u goes to un: other
// blocks still read this block's u for their operator, so u cannot be
// updated in place.  un then becomes u; the kernel also copies u's halo
// ring to un, so un is exactly the in-place result.  One FP64 add per cell
// more in this FP64-bound kernel against a separate pass over u and p:
// 373.6 -> 350.6 us per iteration at 4096^2 (non-zero fields).
template <int TH, int F, bool U>
__device__ __forceinline__ void cheby_block_body(const Dev& d, const Red& red, double alpha,
                                                 double beta, double* un) {
  tile_driver<TH, 0>(d, red, [&](int x, int y0, bool xin, double* acc) {
    if (!xin) return;
#pragma unroll 1
    for (int ys = y0; ys < y0 + TH && ys < d.y_max; ys += 4) {
      double zl[4], rl[4] = {0.0, 0.0, 0.0, 0.0}, wl[4], pl[4], ul[4];
      const long long c0 = cidx(d, x, ys);
#pragma unroll
      for (int i = 0; i < 4; i++) {
        if (ys + i < d.y_max) {
          const long long c = c0 + i * d.S;
          wl[i] = smvp<F, false, false>(d, d.u, c);
          if (U) ul[i] = d.u[c];
          rl[i] = d.u0[c] - wl[i];
          pl[i] = d.p[c];
        }
      }
#pragma unroll
      for (int i = 0; i < 4; i++) {
        if (ys + i < d.y_max) {
          d.w[c0 + i * d.S] = wl[i];
          d.r[c0 + i * d.S] = rl[i];
        }
      }
      strip_solve<F>(d, c0, strip_rows(d, ys), rl, zl);
#pragma unroll
      for (int i = 0; i < 4; i++)
        if (ys + i < d.y_max) {
          const double pn = F ? __fma_rn(alpha, pl[i], emu_dmul(beta, zl[i]))
                              : alpha * pl[i] + emu_dmul(beta, zl[i]);
          d.p[c0 + i * d.S] = pn;
          if (U) un[c0 + i * d.S] = ul[i] + pn;
        }
    }
  });
}

template <int TH, int F>
__global__ void __launch_bounds__(kBlock, 3)
    k_cheby_calc_pu_block(Dev d, Red red, double alpha, double beta, double* un) {
  cheby_block_body<TH, F, true>(d, red, alpha, beta, un);
  copy_halo_ring(d, d.u, un);
}

// The Chebyshev residual step shared by tea_leaf_cheby_solve_init_p and
// tea_leaf_cheby_solve_calc_p (tea_leaf_cheby_cl.cl:4-64, :78-145):
// w = A u, r = u0 - w, then p from M^-1 r.  mode 0: p = M^-1 r / theta;
// mode 1: p = alpha p + beta M^-1 r.
template <int TH, int F>
__global__ void __launch_bounds__(kBlock)
    k_cheby_p(Dev d, Red red, int mode, DivConst theta, double alpha,
              double beta) {
  tile_driver<TH, 0>(d, red, [&](int x, int y0, bool xin, double* acc) {
    if (!xin) return;
    if (d.prec == PREC_JAC_BLOCK) {
#pragma unroll 1
      for (int ys = y0; ys < y0 + TH && ys < d.y_max; ys += 4) {
        double zl[4], rl[4] = {0.0, 0.0, 0.0, 0.0}, wl[4], pl[4];
        const long long c0 = cidx(d, x, ys);
#pragma unroll
        for (int i = 0; i < 4; i++) {
          if (ys + i < d.y_max) {
            const long long c = c0 + i * d.S;
            wl[i] = smvp<F, false, false>(d, d.u, c);
            rl[i] = d.u0[c] - wl[i];
            if (mode != 0) pl[i] = d.p[c];
          }
        }
#pragma unroll
        for (int i = 0; i < 4; i++) {
          if (ys + i < d.y_max) {
            d.w[c0 + i * d.S] = wl[i];
            d.r[c0 + i * d.S] = rl[i];
          }
        }
        strip_solve<F>(d, c0, strip_rows(d, ys), rl, zl);
#pragma unroll
        for (int i = 0; i < 4; i++) {
          if (ys + i < d.y_max) {
            const long long c = c0 + i * d.S;
            if (mode == 0)
              d.p[c] = emu_ddiv(zl[i], theta);
            else
              d.p[c] = cheby_update<F>(alpha, pl[i], beta, zl[i]);
          }
        }
      }
    } else {
#pragma unroll 1
      for (int g = y0; g < y0 + TH; g += 4) {
        const long long c0 = cidx(d, x, g);
        double wl[4], rl[4], pl[4];
#pragma unroll
        for (int j = 0; j < 4; j++) {
          if (g + j < d.y_max) {
            const long long c = c0 + j * d.S;
            const double wv = smvp<F, false, false>(d, d.u, c);
            const double rv = d.u0[c] - wv;
            wl[j] = wv;
            rl[j] = rv;
            if (mode == 0) {
              if (d.prec == PREC_JAC_DIAG)
                pl[j] = emu_ddiv(d.Mi[c] * rv, theta);
              else
                pl[j] = emu_ddiv(rv, theta);
            } else {
              if (d.prec == PREC_JAC_DIAG)
                pl[j] = cheby_update<F>(alpha, d.p[c], beta * d.Mi[c], rv);
              else
                pl[j] = cheby_update<F>(alpha, d.p[c], beta, rv);
            }
          }
        }
#pragma unroll
        for (int j = 0; j < 4; j++) {
          if (g + j < d.y_max) {
            const long long c = c0 + j * d.S;
            d.w[c] = wl[j];
            d.r[c] = rl[j];
            d.p[c] = pl[j];
          }
        }
      }
    }
  });
}

// tea_leaf_cheby_solve_calc_u, tea_leaf_cheby_cl.cl:66-76
template <int TH, int F>
__global__ void __launch_bounds__(kBlock, 1) k_cheby_calc_u(Dev d, Red red) {
  tile_driver<TH, 0>(d, red, [&](int x, int y0, bool xin, double* acc) {
    if (!xin) return;
#pragma unroll 1
    for (int g = y0; g < y0 + TH; g += 4) {
      const long long c0 = cidx(d, x, g);
      double uv[4], pv[4];
#pragma unroll
      for (int j = 0; j < 4; j++)
        if (g + j < d.y_max) {
          uv[j] = d.u[c0 + j * d.S];
          pv[j] = d.p[c0 + j * d.S];
        }
#pragma unroll
      for (int j = 0; j < 4; j++)
        if (g + j < d.y_max) d.u[c0 + j * d.S] = uv[j] + pv[j];
    }
  });
}

// M^-1 r with the PPCG forms: tea_leaf_ppcg_solve_init_sd
// (tea_leaf_ppcg_cl.cl:4-60, mode 0: sd = M^-1 r / theta) and
// tea_leaf_ppcg_solve_calc_sd (:90-155, mode 1: sd = alpha sd + beta M^-1 r,
// diagonal case alpha sd + (beta r) Mi)
template <int TH, int F>
__global__ void __launch_bounds__(kBlock)
    k_ppcg_sd(Dev d, Red red, int mode, DivConst theta, double alpha,
              double beta, const ResState* st) {
  if (st && *(volatile const int*)&st->stop) return;
  tile_driver<TH, 0>(d, red, [&](int x, int y0, bool xin, double* acc) {
    if (!xin) return;
    if (d.prec == PREC_JAC_BLOCK) {
#pragma unroll 1
      for (int ys = y0; ys < y0 + TH && ys < d.y_max; ys += 4) {
        double zl[4], rl[4];
        const long long c0 = cidx(d, x, ys);
        double sv[4];
#pragma unroll
        for (int i = 0; i < 4; i++) {
          const bool in = ys + i < d.y_max;
          rl[i] = in ? d.r[c0 + i * d.S] : 0.0;
          sv[i] = (in && mode != 0) ? d.sd[c0 + i * d.S] : 0.0;
        }
        strip_solve<F>(d, c0, strip_rows(d, ys), rl, zl);
#pragma unroll
        for (int i = 0; i < 4; i++) {
          if (ys + i < d.y_max) {
            const long long c = c0 + i * d.S;
            if (mode == 0)
              d.sd[c] = emu_ddiv(zl[i], theta);
            else
              d.sd[c] = cheby_update<F>(alpha, sv[i], beta, zl[i]);
          }
        }
      }
    } else {
#pragma unroll 1
      for (int g = y0; g < y0 + TH; g += 4) {
        const long long c0 = cidx(d, x, g);
        double nv[4];
#pragma unroll
        for (int j = 0; j < 4; j++) {
          if (g + j < d.y_max) {
            const long long c = c0 + j * d.S;
            const double rv = d.r[c];
            if (mode == 0) {
              if (d.prec == PREC_JAC_DIAG)
                nv[j] = emu_ddiv(rv * d.Mi[c], theta);
              else
                nv[j] = emu_ddiv(rv, theta);
            } else {
              if (d.prec == PREC_JAC_DIAG)
                nv[j] = cheby_update<F>(alpha, d.sd[c], beta * rv, d.Mi[c]);
              else
                nv[j] = cheby_update<F>(alpha, d.sd[c], beta, rv);
            }
          }
        }
#pragma unroll
        for (int j = 0; j < 4; j++)
          if (g + j < d.y_max) d.sd[c0 + j * d.S] = nv[j];
      }
    }
  });
}

// tea_leaf_ppcg_solve_calc_sd for the block-Jacobi preconditioner alone
// (tea_leaf_ppcg_cl.cl:90-134, the strip solve of tea_block_jacobi.cl:44-76):
// z = M^-1 r strip by strip, sd = alpha sd + beta z.  It takes no sum, so
// its walk over the grid is free: a warp takes 64 columns of one 4-row strip
// and each lane two adjacent columns, with 16-byte loads (padded column H
// of every row is 256-byte aligned and the lane's first column is even).
// Strips cut by the top of the interior, a last odd column and the exact
// form (whose first-row division needs more registers) take the one-column
// path.  The product beta z runs on the integer pipes
// (tea_emu.cuh, bit-identical); the sweep's multiplies by bfp stay on the
// FP64 pipe, where they sit on the strip's dependent chain.  At 4096^2 on
// non-zero fields: 149.8 us for one column per lane with both products on
// the integer pipes, 137.4 with beta z alone there, 131.5 for two columns
// per lane (165.4 with beta z on the FP64 pipe too).
constexpr int kSdMinBlocks = 4;
constexpr int kSdColsPerWarp = 64;

// warp units (64 columns x one strip) of calc_sd, and the blocks they fill
__host__ __device__ inline long long sd_units(const Dev& d) {
  return (long long)((d.x_max + kSdColsPerWarp - 1) / kSdColsPerWarp) * ((d.y_max + 3) / 4);
}
static int sd_blocks(const Dev& d) {
  return (int)std::max<long long>(1, (sd_units(d) + kBlock / 32 - 1) / (kBlock / 32));
}

// the sd update of one cell from the strip's z
template <int F>
__device__ __forceinline__ double sd_update(double alpha, double s, double beta, double z) {
  return F ? __fma_rn(alpha, s, emu_dmul(beta, z)) : alpha * s + emu_dmul(beta, z);
}

template <int F>
__global__ void __launch_bounds__(kBlock, kSdMinBlocks)
    k_ppcg_calc_sd_block(Dev d, double alpha, double beta, const ResState* st) {
  if (st && *(volatile const int*)&st->stop) return;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int nux = (d.x_max + kSdColsPerWarp - 1) / kSdColsPerWarp;
  const long long units = sd_units(d);
  const long long S = d.S;
  const double* __restrict__ rp = d.r;
  double* __restrict__ sp = d.sd;
  for (long long u = (long long)blockIdx.x * (kBlock / 32) + warp; u < units;
       u += (long long)gridDim.x * (kBlock / 32)) {
    const int ty = (int)(u / nux), tx = (int)(u - (long long)ty * nux);
    const int x = tx * kSdColsPerWarp + 2 * lane, ys = ty * 4;
    if (x >= d.x_max) continue;
    const long long c0 = cidx(d, x, ys);
    const int upper = strip_rows(d, ys);
    if (F && upper == 4 && ys + 3 < d.y_max && x + 1 < d.x_max) {
      double ra[4], rb[4], ba[4], bb[4], ka[4], kb[4], ca[4], cb[4], za[4], zb[4];
#pragma unroll
      for (int i = 0; i < 4; i++) {
        const double2 rv = *(const double2*)(rp + c0 + i * S);
        const double2 bv = __ldg((const double2*)(d.bfp + c0 + i * S));
        const double2 kv =
            i > 0 ? __ldg((const double2*)(d.Ky + c0 + i * S)) : make_double2(0.0, 0.0);
        const double2 cv =
            i < 3 ? __ldg((const double2*)(d.cp + c0 + i * S)) : make_double2(0.0, 0.0);
        ra[i] = rv.x;
        rb[i] = rv.y;
        ba[i] = bv.x;
        bb[i] = bv.y;
        ka[i] = kv.x;
        kb[i] = kv.y;
        ca[i] = cv.x;
        cb[i] = cv.y;
      }
      strip_solve_v<F, false, true>(4, ra, ba, ka, ca, 0.0, za);
      strip_solve_v<F, false, true>(4, rb, bb, kb, cb, 0.0, zb);
#pragma unroll
      for (int i = 0; i < 4; i++) {
        const double2 s = *(const double2*)(sp + c0 + i * S);
        double2 o;
        o.x = sd_update<F>(alpha, s.x, beta, za[i]);
        o.y = sd_update<F>(alpha, s.y, beta, zb[i]);
        *(double2*)(sp + c0 + i * S) = o;
      }
    } else {
      for (int k = 0; k < 2 && x + k < d.x_max; k++) {
        const long long cc = c0 + k;
        double zl[4], rl[4], sv[4];
#pragma unroll
        for (int i = 0; i < 4; i++) {
          const bool in = ys + i < d.y_max;
          rl[i] = in ? rp[cc + i * S] : 0.0;
          sv[i] = in ? sp[cc + i * S] : 0.0;
        }
        strip_solve<F>(d, cc, upper, rl, zl);
#pragma unroll
        for (int i = 0; i < 4; i++)
          if (ys + i < d.y_max) sp[cc + i * S] = sd_update<F>(alpha, sv[i], beta, zl[i]);
      }
    }
  }
}

// One PPCG inner step with the block-Jacobi preconditioner in one pass:
// tea_leaf_ppcg_solve_update_r (tea_leaf_ppcg_cl.cl:62-88) and then
// tea_leaf_ppcg_solve_calc_sd (:90-134) on the r it has just formed.  A lane
// takes one column of one 4-row strip: u += sd and r -= A sd at its 4
// cells, then z = M^-1 r by the strip's sweep (the rows' Ky shared with the
// operator) and sd' = alpha sd + beta z.  Other blocks still read this
// block's sd for their operator, so sd' goes to sdo; u and r are read only
// at their own cells and are updated in place.  The arithmetic is that of
// the two kernels (bit-identical); 9.5 FP64 instructions and 112 algorithmic
// bytes per cell against 6 + 3.5 and 56 + 56 for the two passes.  At 4096^2
// on non-zero fields 302-305 us against 322.4 us for update_r + calc_sd, at
// 3 blocks per SM (80 registers; 4 blocks per SM with 64 registers 317-321
// us).
template <int F>
__global__ void __launch_bounds__(kBlock, 3)
    k_ppcg_step(Dev d, Red red, double alpha, double beta, const ResState* st,
                const double* sdi_, double* sdo_) {
  if (st && *(volatile const int*)&st->stop) return;
  tile_driver<4, 0>(d, red, [&](int x, int y0, bool xin, double* acc) {
    if (!xin) return;
    const double* __restrict__ sdi = sdi_;
    double* __restrict__ sdo = sdo_;
    const double* __restrict__ kx = d.Kx;
    const double* __restrict__ ky = d.Ky;
    const double* __restrict__ dg = d.diag;
    double* __restrict__ u = d.u;
    double* __restrict__ r = d.r;
    const long long S = d.S;
    const long long c0 = cidx(d, x, y0);
    const int upper = strip_rows(d, y0);
    if (upper == 4 && y0 + 3 < d.y_max) {
      const double* __restrict__ bfp = d.bfp;
      const double* __restrict__ cp = d.cp;
      double sv[6], kyv[5], rv[4], uv[4], bl[4], cl[4], z[4];
#pragma unroll
      for (int i = 0; i < 6; i++) sv[i] = sdi[c0 + (i - 1) * S];
#pragma unroll
      for (int i = 0; i < 5; i++) kyv[i] = __ldg(ky + c0 + i * S);
      const double d0 = __ldg(dg + c0);
#pragma unroll
      for (int j = 0; j < 4; j++) {
        const long long c = c0 + j * S;
        uv[j] = u[c] + sv[j + 1];
        rv[j] = bms_v<F>(r[c], j ? __ldg(dg + c) : d0, kyv[j + 1], kyv[j], __ldg(kx + c + 1),
                         __ldg(kx + c), sv[j + 1], sv[j + 2], sv[j], sdi[c + 1], sdi[c - 1]);
        bl[j] = __ldg(bfp + c);
        cl[j] = j < 3 ? __ldg(cp + c) : 0.0;
      }
#pragma unroll
      for (int j = 0; j < 4; j++) {
        u[c0 + j * S] = uv[j];
        r[c0 + j * S] = rv[j];
      }
      const double kl[4] = {0.0, kyv[1], kyv[2], kyv[3]};
      strip_solve_v<F, false, true>(4, rv, bl, kl, cl, d0, z);
#pragma unroll
      for (int j = 0; j < 4; j++) sdo[c0 + j * S] = sd_update<F>(alpha, sv[j + 1], beta, z[j]);
    } else {
      // a strip cut by the top of the interior: the two kernels' steps
      bool in[4];
      double sv[4], rv[4], zl[4];
#pragma unroll
      for (int j = 0; j < 4; j++) {
        in[j] = y0 + j < d.y_max;
        sv[j] = rv[j] = 0.0;
        if (in[j]) {
          const long long c = c0 + j * S;
          sv[j] = sdi[c];
          const double uv = u[c] + sv[j];
          rv[j] = bms_v<F>(r[c], __ldg(dg + c), __ldg(ky + c + S), __ldg(ky + c),
                           __ldg(kx + c + 1), __ldg(kx + c), sv[j], sdi[c + S], sdi[c - S],
                           sdi[c + 1], sdi[c - 1]);
          u[c] = uv;
          r[c] = rv[j];
        }
      }
      strip_solve<F>(d, c0, upper, rv, zl);
#pragma unroll
      for (int j = 0; j < 4; j++)
        if (in[j]) sdo[c0 + j * S] = sd_update<F>(alpha, sv[j], beta, zl[j]);
    }
  });
}

// tea_leaf_ppcg_solve_update_r, tea_leaf_ppcg_cl.cl:62-88
template <int TH, int F>
__global__ void __launch_bounds__(kBlock, 1)
    k_ppcg_update_r(Dev d, Red red, const ResState* st) {
  if (st && *(volatile const int*)&st->stop) return;
  tile_driver<TH, 0>(d, red, [&](int x, int y0, bool xin, double* acc) {
    if (!xin) return;
#pragma unroll 1
    for (int g = y0; g < y0 + TH; g += 4) {
      const long long c0 = cidx(d, x, g);
      double uv[4], rv[4];
#pragma unroll
      for (int j = 0; j < 4; j++)
        if (g + j < d.y_max) {
          const long long c = c0 + j * d.S;
          uv[j] = d.u[c] + d.sd[c];
          rv[j] = b_minus_smvp<F>(d, d.sd, c, d.r[c]);
        }
#pragma unroll
      for (int j = 0; j < 4; j++)
        if (g + j < d.y_max) {
          d.u[c0 + j * d.S] = uv[j];
          d.r[c0 + j * d.S] = rv[j];
        }
    }
  });
}

// tea_leaf_jacobi_copy_u, tea_leaf_jacobi_cl.cl:3-13 (un is vector_Mi, as
// in the reference, ocl_kernels.cpp:576-585)
template <int TH, int F>
__global__ void __launch_bounds__(kBlock) k_jacobi_copy_u(Dev d, Red red) {
  tile_driver<TH, 0>(d, red, [&](int x, int y0, bool xin, double* acc) {
    if (!xin) return;
#pragma unroll 1
    for (int g = y0; g < y0 + TH; g += 4) {
      const long long c0 = cidx(d, x, g);
      double uv[4];
#pragma unroll
      for (int j = 0; j < 4; j++)
        if (g + j < d.y_max) uv[j] = d.u[c0 + j * d.S];
#pragma unroll
      for (int j = 0; j < 4; j++)
        if (g + j < d.y_max) d.un[c0 + j * d.S] = uv[j];
    }
  });
}

// tea_leaf_jacobi_solve, tea_leaf_jacobi_cl.cl:15-42 (the same arithmetic in
// both forms; its denominator associates differently from the diagonal)
template <int TH, int F>
__global__ void __launch_bounds__(kBlock) k_jacobi_solve(Dev d, Red red) {
  tile_driver<TH, 1>(d, red, [&](int x, int y0, bool xin, double* acc) {
    const long long S = d.S;
#pragma unroll 1
    for (int g = y0; g < y0 + TH; g += 4) {
      const long long c0 = cidx(d, x, g);
      double uv[4], v[4] = {0.0, 0.0, 0.0, 0.0};
#pragma unroll
      for (int j = 0; j < 4; j++)
        if (xin && g + j < d.y_max) {
          const long long c = c0 + j * S;
          const double* un = d.un;
          const double kxc = d.Kx[c], kxe = d.Kx[c + 1];
          const double kyc = d.Ky[c], kyn = d.Ky[c + S];
          const double u1 = emu_ddiv_var(d.u0[c] + kxe * un[c + 1] + kxc * un[c - 1] +
                                             kyn * un[c + S] + kyc * un[c - S],
                                         1.0 + (kxc + kxe) + (kyc + kyn));
          uv[j] = u1;
          v[j] = fabs(u1 - un[c]);
        }
#pragma unroll
      for (int j = 0; j < 4; j++)
        if (xin && g + j < d.y_max) d.u[c0 + j * S] = uv[j];
#pragma unroll
      for (int j = 0; j < 4; j++) acc[0] = acc[0] + v[j];
    }
  });
}

// tea_leaf_finalise, tea_leaf_common_cl.cl:4-15
template <int TH, int F>
__global__ void __launch_bounds__(kBlock) k_finalise(Dev d, Red red) {
  tile_driver<TH, 0>(d, red, [&](int x, int y0, bool xin, double* acc) {
    if (!xin) return;
#pragma unroll 1
    for (int g = y0; g < y0 + TH; g += 4) {
      const long long c0 = cidx(d, x, g);
      double ev[4];
#pragma unroll
      for (int j = 0; j < 4; j++)
        if (g + j < d.y_max) ev[j] = emu_ddiv_var(d.u[c0 + j * d.S], d.density[c0 + j * d.S]);
#pragma unroll
      for (int j = 0; j < 4; j++)
        if (g + j < d.y_max) d.energy1[c0 + j * d.S] = ev[j];
    }
  });
}

// field_summary, field_summary_cl.cl:3-43 (energy argument bound to energy1,
// ocl_kernels.cpp:466-469); the same arithmetic in both forms.  (Its three
// products on the integer pipes measured slower: 266 -> 457 us at 4096^2,
// 80 -> 94 registers and three blocks per SM -> two.)
template <int TH, int F>
__global__ void __launch_bounds__(kBlock, 1) k_field_summary(Dev d, Red red) {
  tile_driver<TH, 4>(d, red, [&](int x, int y0, bool xin, double* acc) {
#pragma unroll 2
    for (int j = 0; j < TH; j++) {
      const int y = y0 + j;
      double v0 = 0.0, v1 = 0.0, v2 = 0.0, v3 = 0.0;
      if (xin && y < d.y_max) {
        const long long c = cidx(d, x, y);
        const double cell_vol = d.volume[c];
        const double cell_mass = cell_vol * d.density[c];
        v0 = cell_vol;
        v1 = cell_mass;
        v2 = cell_mass * d.energy1[c];
        v3 = cell_mass * d.u[c];
      }
      acc[0] = acc[0] + v0;
      acc[1] = acc[1] + v1;
      acc[2] = acc[2] + v2;
      acc[3] = acc[3] + v3;
    }
  });
}

// The diagonal 1 + (Ky_n + Ky_c) + (Kx_e + Kx_c) of every interior cell, in
// the association of the reference's inline expression
template <int TH, int F>
__global__ void __launch_bounds__(kBlock) k_init_diag(Dev d, Red red) {
  tile_driver<TH, 0>(d, red, [&](int x, int y0, bool xin, double* acc) {
    if (!xin) return;
    for (int j = 0; j < TH; j++) {
      const int y = y0 + j;
      if (y < d.y_max) {
        const long long c = cidx(d, x, y);
        d.diag[c] = (1.0 + (d.Ky[c + d.S] + d.Ky[c]) + (d.Kx[c + 1] + d.Kx[c]));
      }
    }
  });
}

// ---------------------------------------------------------------------------
// launch wrappers
// ---------------------------------------------------------------------------

void launch_initialise_chunk(Chunk& c, double xmin, double ymin, double dx,
                             double dy) {
  const Dev d = c.dev();
  const int n = std::max(d.x_max, d.y_max) + d.H + 1;
  profile_begin("initialise_chunk_first");
  k_init_chunk_1d<<<(n + 255) / 256, 256, 0, c.stream>>>(d, xmin, ymin, dx, dy);
  count_launch("initialise_chunk_first");
  check_cuda(cudaGetLastError(), "initialise_chunk_first");
  profile_end("initialise_chunk_first");
  launch_2d(c, "initialise_chunk_second", d.x_max + 2, d.y_max + 2, k_volume, d,
            dx * dy);
}

void launch_generate_init(Chunk& c, double dens0, double en0) {
  const Dev d = c.dev();
  launch_2d(c, "generate_chunk_init", d.x_max, d.y_max, k_gen_init, d, dens0, en0);
}

void launch_generate_state(Chunk& c, double dens, double en, double xmin,
                           double xmax, double ymin, double ymax,
                           double radius, int geom, int g_rect, int g_circ,
                           int g_point) {
  const Dev d = c.dev();
  launch_2d(c, "generate_chunk", d.x_max, d.y_max, k_gen_state, d, dens, en,
            xmin, xmax, ymin, ymax, radius, geom, g_rect, g_circ, g_point);
}

void launch_init_u(Chunk& c, const double* energy) {
  const Dev d = c.dev();
  launch_2d(c, "generate_chunk_init_u", d.x_max, d.y_max, k_init_u, d, energy);
}

void launch_set_field(Chunk& c) {
  const Dev d = c.dev();
  launch_2d(c, "set_field", d.x_max, d.y_max, k_set_field, d);
}

void launch_init_common(Chunk& c, int coef, double rx, double ry) {
  const Dev d = c.dev();
  launch_2d(c, "tea_leaf_init_common", d.xs - 1, d.ys - 1, k_init_common, d,
            coef, rx, ry);
}

void launch_zero_boundary(Chunk& c, const int* zb) {
  const Dev d = c.dev();
  launch_2d(c, "tea_leaf_zero_boundary", d.xs, d.ys, k_zero_boundary, d, zb[0],
            zb[1], zb[2], zb[3]);
}

void launch_calc_residual(Chunk& c) {
  TH4_DISPATCH(c, "tea_leaf_calc_residual", k_calc_residual, dev4(c), c.red());
}

void launch_dot(Chunk& c, const double* a, const double* b) {
  TH_DISPATCH(c, "tea_leaf_calc_2norm", k_dot, c.dev(), c.red(), a, b);
}

void launch_init_diag(Chunk& c) {
  TH_DISPATCH(c, "tea_leaf_init_diag", k_init_diag, c.dev(), c.red());
}

void launch_init_jac_diag(Chunk& c) {
  const Dev d = c.dev();
  launch_2d(c, "tea_leaf_init_jac_diag", d.xs, d.ys, k_init_jac_diag, d);
}

void launch_block_init(Chunk& c) {
  const Dev d = c.dev();
  launch_2d(c, "tea_leaf_block_init", d.x_max, (d.y_max + 3) / 4, k_block_init, d,
            c.arith != 0 ? 1 : 0);
}

void launch_cg_init_p(Chunk& c) {
  TH_DISPATCH(c, "tea_leaf_cg_solve_init_p", k_cg_init_p, c.dev(), c.red());
}

void launch_cg_calc_w(Chunk& c) {
  TH_DISPATCH(c, "tea_leaf_cg_solve_calc_w", k_cg_calc_w, c.dev(), c.red(),
              (ResState*)nullptr);
}

void launch_cg_calc_ur(Chunk& c, double alpha) {
  TH_DISPATCH(c, "tea_leaf_cg_solve_calc_ur", k_cg_calc_ur, c.dev(), c.red(),
              alpha, (ResState*)nullptr);
}

void launch_cg_calc_ur_sd(Chunk& c, double alpha, double theta, double* sd_out) {
  Dev d = c.dev();
  d.sd = sd_out;
  TH_DISPATCH(c, "tea_leaf_cg_solve_calc_ur", k_cg_calc_ur_sd, d, c.red(), alpha,
              div_const(theta));
}

void launch_cg_calc_p(Chunk& c, double beta) {
  TH4_DISPATCH(c, "tea_leaf_cg_solve_calc_p", k_cg_calc_p, dev4(c), c.red(), beta,
              (ResState*)nullptr, (unsigned int*)nullptr);
}

void launch_cheby_init_p(Chunk& c, double theta) {
  TH_DISPATCH(c, "tea_leaf_cheby_solve_init_p", k_cheby_p, c.dev(), c.red(), 0,
              div_const(theta), 0.0, 0.0);
}

// calc_p alone (block Jacobi takes k_cheby_calc_pu_block, with calc_u)
void launch_cheby_calc_p(Chunk& c, double alpha, double beta) {
  TH_DISPATCH(c, "tea_leaf_cheby_solve_calc_p", k_cheby_p, c.dev(), c.red(), 1,
              div_const(1.0), alpha, beta);
}

void launch_cheby_calc_pu(Chunk& c, double alpha, double beta, double* un) {
  TH_DISPATCH(c, "tea_leaf_cheby_solve_calc_p_u", k_cheby_calc_pu_block, c.dev(), c.red(),
              alpha, beta, un);
}

void launch_cheby_calc_u(Chunk& c) {
  TH4_DISPATCH(c, "tea_leaf_cheby_solve_calc_u", k_cheby_calc_u, dev4(c), c.red());
}

void launch_ppcg_init_sd(Chunk& c, double theta) {
  TH4_DISPATCH(c, "tea_leaf_ppcg_solve_init_sd", k_ppcg_sd, dev4(c), c.red(), 0,
              div_const(theta), 0.0, 0.0, (const ResState*)nullptr);
}

void launch_ppcg_step(Chunk& c, double alpha, double beta, const double* sdi, double* sdo) {
  const Dev d4 = dev4(c);
  const char* name = "tea_leaf_ppcg_solve_inner_step";
  const ResState* st = nullptr;
  if (c.arith == 2)
    launch_tile_ns(c, name, d4.ns, k_ppcg_step<2>, d4, c.red(), alpha, beta, st, sdi, sdo);
  else if (c.arith == 1)
    launch_tile_ns(c, name, d4.ns, k_ppcg_step<1>, d4, c.red(), alpha, beta, st, sdi, sdo);
  else
    launch_tile_ns(c, name, d4.ns, k_ppcg_step<0>, d4, c.red(), alpha, beta, st, sdi, sdo);
}

void launch_ppcg_update_r(Chunk& c) {
  TH4_DISPATCH(c, "tea_leaf_ppcg_solve_update_r", k_ppcg_update_r, dev4(c),
              c.red(), (const ResState*)nullptr);
}

void launch_ppcg_calc_sd(Chunk& c, double alpha, double beta) {
  if (c.prec == PREC_JAC_BLOCK) {
    const Dev d4 = dev4(c);
    const char* name = "tea_leaf_ppcg_solve_calc_sd";
    const int nb = sd_blocks(d4);
    if (c.arith == 2)
      launch_tile_ns(c, name, nb, k_ppcg_calc_sd_block<2>, d4, alpha, beta,
                     (const ResState*)nullptr);
    else if (c.arith == 1)
      launch_tile_ns(c, name, nb, k_ppcg_calc_sd_block<1>, d4, alpha, beta,
                     (const ResState*)nullptr);
    else
      launch_tile_ns(c, name, nb, k_ppcg_calc_sd_block<0>, d4, alpha, beta,
                     (const ResState*)nullptr);
    return;
  }
  TH4_DISPATCH(c, "tea_leaf_ppcg_solve_calc_sd", k_ppcg_sd, dev4(c), c.red(), 1,
              div_const(1.0), alpha, beta, (const ResState*)nullptr);
}

void launch_jacobi_copy_u(Chunk& c) {
  TH4_DISPATCH(c, "tea_leaf_jacobi_copy_u", k_jacobi_copy_u, dev4(c), c.red());
}

void launch_jacobi_solve(Chunk& c) {
  TH_DISPATCH(c, "tea_leaf_jacobi_solve", k_jacobi_solve, c.dev(), c.red());
}

void launch_finalise(Chunk& c) {
  TH4_DISPATCH(c, "tea_leaf_finalise", k_finalise, dev4(c), c.red());
}

void launch_field_summary(Chunk& c) {
  TH_DISPATCH(c, "field_summary", k_field_summary, c.dev(), c.red());
}

void launch_update_halo(Chunk& c, int mask, int depth) {
  const Dev d = c.dev();
  if (!mask || depth < 1) return;
  launch_2d(c, "update_halo", d.x_max + 2 * depth, d.y_max + 2 * depth,
            k_update_halo, d, mask, depth);
}

// ---------------------------------------------------------------------------
// launchers for an explicit field set (batched problems)
// ---------------------------------------------------------------------------

Dev make_dev_tiling(Dev d) {
  const int TH = reduction_rows(d.x_max, d.y_max);
  d.th = TH;
  d.xs = d.x_max + 2 * d.H;
  d.ys = d.y_max + 2 * d.H;
  d.block_top_check = (d.y_max % 4) != 0;
  d.ntx = (d.x_max + kTileW - 1) / kTileW;
  d.nsx = (d.ntx + kTilesPerSuper - 1) / kTilesPerSuper;
  d.nty = (d.y_max + TH - 1) / TH;
  d.ns = d.nsx * d.nty;
  return d;
}

template <class... KArgs, class... Args>
static void ctx_tile(const LaunchCtx& l, const Dev& d, const char* name,
                     void (*kernel)(KArgs...), Args... args) {
  const long long cap = (long long)l.num_sms * blocks_per_sm((const void*)kernel);
  const int grid = (int)std::max<long long>(1, std::min<long long>(d.ns, cap));
  kernel<<<grid, kBlock, 0, l.stream>>>(args...);
  count_launch(name);
  check_cuda(cudaGetLastError(), name);
}

template <class... KArgs, class... Args>
static void ctx_2d(const LaunchCtx& l, const char* name, int nx, int ny,
                   void (*kernel)(KArgs...), Args... args) {
  if (nx <= 0 || ny <= 0) return;
  kernel<<<dim3((nx + 31) / 32, (ny + 7) / 8), dim3(32, 8), 0, l.stream>>>(args...);
  count_launch(name);
  check_cuda(cudaGetLastError(), name);
}

#define CTX_DISPATCH(l, d, name, kern, ...)              \
  do {                                                   \
    if ((d).th == 16) {                                  \
      if ((l).arith == 2)                                \
        ctx_tile(l, d, name, kern<16, 2>, __VA_ARGS__);  \
      else if ((l).arith == 1)                           \
        ctx_tile(l, d, name, kern<16, 1>, __VA_ARGS__);  \
      else                                               \
        ctx_tile(l, d, name, kern<16, 0>, __VA_ARGS__);  \
    } else {                                             \
      if ((l).arith == 2)                                \
        ctx_tile(l, d, name, kern<4, 2>, __VA_ARGS__);   \
      else if ((l).arith == 1)                           \
        ctx_tile(l, d, name, kern<4, 1>, __VA_ARGS__);   \
      else                                               \
        ctx_tile(l, d, name, kern<4, 0>, __VA_ARGS__);   \
    }                                                    \
  } while (0)

void dev_volume(const LaunchCtx& l, const Dev& d, double vol) {
  ctx_2d(l, "initialise_chunk_second", d.x_max + 2, d.y_max + 2, k_volume, d, vol);
}
void dev_init_common(const LaunchCtx& l, const Dev& d, int coef, double rx,
                     double ry) {
  ctx_2d(l, "tea_leaf_init_common", d.xs - 1, d.ys - 1, k_init_common, d, coef, rx, ry);
}
void dev_zero_boundary(const LaunchCtx& l, const Dev& d, const int* zb) {
  ctx_2d(l, "tea_leaf_zero_boundary", d.xs, d.ys, k_zero_boundary, d, zb[0], zb[1],
         zb[2], zb[3]);
}
void dev_init_diag(const LaunchCtx& l, const Dev& d, const Red& r) {
  CTX_DISPATCH(l, d, "tea_leaf_init_diag", k_init_diag, d, r);
}
void dev_init_jac_diag(const LaunchCtx& l, const Dev& d) {
  ctx_2d(l, "tea_leaf_init_jac_diag", d.xs, d.ys, k_init_jac_diag, d);
}
void dev_init_u(const LaunchCtx& l, const Dev& d, const double* energy) {
  ctx_2d(l, "generate_chunk_init_u", d.x_max, d.y_max, k_init_u, d, energy);
}
void dev_calc_residual(const LaunchCtx& l, const Dev& d, const Red& r) {
  CTX_DISPATCH(l, d, "tea_leaf_calc_residual", k_calc_residual, d, r);
}
void dev_dot(const LaunchCtx& l, const Dev& d, const Red& r, const double* a,
             const double* b) {
  CTX_DISPATCH(l, d, "tea_leaf_calc_2norm", k_dot, d, r, a, b);
}
void dev_block_init(const LaunchCtx& l, const Dev& d) {
  ctx_2d(l, "tea_leaf_block_init", d.x_max, (d.y_max + 3) / 4, k_block_init, d,
         l.arith != 0 ? 1 : 0);
}
void dev_update_halo(const LaunchCtx& l, const Dev& d, int mask, int depth) {
  if (!mask || depth < 1) return;
  ctx_2d(l, "update_halo", d.x_max + 2 * depth, d.y_max + 2 * depth, k_update_halo,
         d, mask, depth);
}
void dev_cg_init_p(const LaunchCtx& l, const Dev& d, const Red& r) {
  CTX_DISPATCH(l, d, "tea_leaf_cg_solve_init_p", k_cg_init_p, d, r);
}
void dev_cg_iteration(const LaunchCtx& l, const Dev& d, const Red& r, ResState* st,
                      unsigned int* counter) {
  CTX_DISPATCH(l, d, "tea_leaf_cg_solve_calc_w", k_cg_calc_w, d, r, st);
  CTX_DISPATCH(l, d, "tea_leaf_cg_solve_calc_ur", k_cg_calc_ur, d, r, 0.0, st);
  CTX_DISPATCH(l, d, "tea_leaf_cg_solve_calc_p", k_cg_calc_p, d, r, 0.0, st, counter);
}
void dev_finalise(const LaunchCtx& l, const Dev& d, const Red& r) {
  CTX_DISPATCH(l, d, "tea_leaf_finalise", k_finalise, d, r);
}
void dev_field_summary(const LaunchCtx& l, const Dev& d, const Red& r) {
  CTX_DISPATCH(l, d, "field_summary", k_field_summary, d, r);
}

// ---------------------------------------------------------------------------
// device-resident CG loop
// ---------------------------------------------------------------------------

// Grid size of a tile kernel: every SM filled once, capped by the number of
// supertiles.
template <class... KArgs>
static int tile_grid(Chunk& c, void (*kernel)(KArgs...), int ns = 0) {
  const long long cap = (long long)c.num_sms * blocks_per_sm((const void*)kernel);
  return (int)std::max<long long>(1, std::min<long long>(ns > 0 ? ns : c.dev().ns, cap));
}

// The whole remaining CG loop as one cooperative launch, for grids whose
// iterations are short enough for kernel boundaries to dominate.  Every
// block keeps the same supertiles in all three phases; grid barriers
// separate w = A p, the u/r/z update and p = z + beta p.  After each
// reducing phase every block forms the reduced value itself from the
// supertile partials, in the fixed order of block_final_sum, so all blocks
// agree bit for bit and no extra barrier is needed; block 0 keeps the loop
// state (cg_scalar_step).  Fields written by other blocks are read through
// L2 (CG = true).  Results are those of the three-kernel loop.
template <int TH, int F>
__global__ void __launch_bounds__(kBlock)
    k_cg_persistent(Dev d, Red red, ResState* st, unsigned int* bar, int* err,
                    long long spin_limit, unsigned int extra_arrivals) {
  __shared__ double sh[16];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  Red rw = red, ru = red;
  ru.partials = red.partials + red.stride;  // p.w and r.z partials apart
  auto phase = [&](const Red& r, auto body, bool reduce) {
    for (int s = blockIdx.x; s < d.ns; s += gridDim.x) {
      const int sy = s / d.nsx, sx = s - sy * d.nsx;
      const int tx = sx * kTilesPerSuper + warp;
      double acc[1] = {0.0};
      if (tx < d.ntx) {
        const int x = tx * kTileW + lane;
        body(x, sy * TH, x < d.x_max, acc);
        if (reduce) acc[0] = bfly(acc[0]);
      }
      if (reduce) supertile_partial<1>(r, s, acc, sh);
    }
  };
  for (;;) {
    if (*(volatile int*)&st->stop) return;
    const double rro = *(volatile double*)&st->rro;
    phase(rw, [&](int x, int y0, bool xin, double* acc) {
      cg_w_tile<TH, F, true>(d, x, y0, xin, acc);
    }, true);
    if (!grid_barrier(bar, err, spin_limit, extra_arrivals)) return;
    const double pw = block_final_value(rw.partials, d.ns, sh);
    const double alpha = rro / pw;
    phase(ru, [&](int x, int y0, bool xin, double* acc) {
      cg_ur_tile<TH, F, 1, true>(d, x, y0, xin, acc, alpha);
    }, true);
    if (!grid_barrier(bar, err, spin_limit, extra_arrivals)) return;
    const double rrn = block_final_value(ru.partials, d.ns, sh);
    const double beta = rrn / rro;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
      st->pw = pw;
      cg_scalar_step<1>(st, alpha, &rrn);
      st->p_pending = 0;
    }
    phase(rw, [&](int x, int y0, bool xin, double* acc) {
      cg_p_tile<TH, F, true>(d, x, y0, xin, beta);
    }, false);
    if (!grid_barrier(bar, err, spin_limit, extra_arrivals)) return;
  }
}

// Cooperative launch of k_cg_persistent: as many blocks as can be resident
// at once, at most one per supertile.  Returns false if the launch fails.
template <int TH, int F>
static bool launch_cg_persistent_t(Chunk& c) {
  const void* fn = (const void*)k_cg_persistent<TH, F>;
  const long long cap = (long long)c.num_sms * blocks_per_sm(fn);
  const int grid = (int)std::max<long long>(1, std::min<long long>(c.dev().ns, cap));
  Dev d = c.dev();
  Red red = c.red();
  ResState* st = c.res_state;
  unsigned int* bar = c.res_bar;
  int* err = (int*)(c.res_bar + 2);
  long long spin_limit = c.barrier_spin_limit;
  unsigned int extra = (unsigned int)c.barrier_extra;
  void* args[] = {&d, &red, &st, &bar, &err, &spin_limit, &extra};
  return check_cuda(cudaLaunchCooperativeKernel(fn, dim3(grid), dim3(kBlock), args, 0,
                                                c.stream),
                    "persistent CG launch");
}

static bool launch_cg_persistent(Chunk& c) {
  if (c.TH == 16)
    return c.arith == 2 ? launch_cg_persistent_t<16, 2>(c)
           : c.arith == 1 ? launch_cg_persistent_t<16, 1>(c)
                          : launch_cg_persistent_t<16, 0>(c);
  return c.arith == 2 ? launch_cg_persistent_t<4, 2>(c)
         : c.arith == 1 ? launch_cg_persistent_t<4, 1>(c)
                        : launch_cg_persistent_t<4, 0>(c);
}

// ---- device-resident PPCG iterations (tea_solve.f90:231-268 after the
// switch from CG), scalars in the ResState as for CG ----

// tea_leaf_cg_calc_ur of a PPCG iteration with alpha = rro/pw from the loop
// state, fused with tea_leaf_ppcg_init_sd: PPCG discards this r.z, so no
// sum is taken, and sd = M^-1 r / theta comes from the z formed here.
template <int TH, int F>
__global__ void __launch_bounds__(kBlock, 4)
    k_ppcg_ur_sd(Dev d, Red red, ResState* st, DivConst theta) {
  if (*(volatile int*)&st->stop) return;
  const double alpha = st->rro / st->pw;
  tile_driver<TH, 0>(d, red, [&](int x, int y0, bool xin, double* acc) {
    cg_ur_tile_r<TH, F, 0, true>(d, x, y0, xin, acc, alpha, theta);
  });
  if (blockIdx.x == 0 && threadIdx.x == 0) st->alpha = alpha;
}

// tea_leaf_ppcg_calc_zrnorm (r.z with the z of the last calc_ur) with the
// host steps of the iteration: beta, rro = rrn, error, the exit test.
template <int TH, int F>
__global__ void __launch_bounds__(kBlock) k_ppcg_rz_step(Dev d, Red red, ResState* st) {
  if (*(volatile int*)&st->stop) return;
  const double* zz = d.prec != PREC_NONE ? d.z : d.r;
  const bool last = tile_driver<TH, 1>(d, red, [&](int x, int y0, bool xin, double* acc) {
#pragma unroll 4
    for (int j = 0; j < TH; j++) {
      const int y = y0 + j;
      double av = 0.0, bv = 0.0;
      if (xin && y < d.y_max) {
        const long long c = cidx(d, x, y);
        av = d.r[c];
        bv = zz[c];
      }
      acc[0] = accum<F>(acc[0], av, bv);
    }
  });
  if (last && threadIdx.x == 0) {
    cg_scalar_step<1>(st, st->alpha, red.result);
    __threadfence();
  }
}

// True when the resident PPCG loop runs its inner steps in fused pairs.
static bool resident_pairs(const Chunk& c) { return tb_applicable(c) && c.n_ppcg >= 2; }

template <int TH, int F>
static void enqueue_ppcg_iterations_t(Chunk& c, int iters) {
  if (resident_pairs(c)) {
    // Inner steps two at a time (tea_ppcg_tb.cu).  Each pair writes r and sd
    // to the other buffer pair, so the sequence alternates between the two
    // field sets; the host copies back if the loop stops on the other one.
    Dev dv[2] = {c.dev(), c.dev()};
    dv[1].r = c.r2.f;
    dv[1].sd = c.sd2.f;
    const Dev d4v[2] = {rows4_tiling(dv[0]), rows4_tiling(dv[1])};
    const Red red = c.red();
    ResState* st = c.res_state;
    const DivConst theta = div_const(c.ppcg_theta);
    const int gw = tile_grid(c, k_cg_calc_w<TH, F>);
    const int gu = tile_grid(c, k_ppcg_ur_sd<TH, F>);
    const int gr = tile_grid(c, k_ppcg_update_r<4, F>, d4v[0].ns);
    const int gs = tile_grid(c, k_ppcg_calc_sd_block<F>, sd_blocks(d4v[0]));
    const int gz = tile_grid(c, k_ppcg_rz_step<TH, F>);
    const int gp = tile_grid(c, k_cg_calc_p<4, F>, d4v[0].ns);
    int cur = 0;
    for (int i = 0; i < iters; i++) {
      k_cg_calc_w<TH, F><<<gw, kBlock, 0, c.stream>>>(dv[cur], red, st);
      k_ppcg_ur_sd<TH, F><<<gu, kBlock, 0, c.stream>>>(dv[cur], red, st, theta);
      int k = 0;
      for (; k + 1 < c.n_ppcg; k += 2) {
        launch_ppcg_inner_pair(c, k, st, dv[cur].r, dv[cur].sd, dv[cur ^ 1].r, dv[cur ^ 1].sd);
        cur ^= 1;
      }
      if (k < c.n_ppcg) {
        k_ppcg_update_r<4, F><<<gr, kBlock, 0, c.stream>>>(d4v[cur], red, st);
        k_ppcg_calc_sd_block<F><<<gs, kBlock, 0, c.stream>>>(
            d4v[cur], c.ppcg_alpha_h[k], c.ppcg_beta_h[k], st);
      }
      k_ppcg_rz_step<TH, F><<<gz, kBlock, 0, c.stream>>>(dv[cur], red, st);
      k_cg_calc_p<4, F><<<gp, kBlock, 0, c.stream>>>(d4v[cur], red, 0.0, st, c.res_counter);
    }
    return;
  }
  const Dev d = c.dev();
  const Dev d4 = dev4(c);  // the kernels that take no sum
  const Red red = c.red();
  ResState* st = c.res_state;
  const DivConst theta = div_const(c.ppcg_theta);
  const int gw = tile_grid(c, k_cg_calc_w<TH, F>);
  const int gu = tile_grid(c, k_ppcg_ur_sd<TH, F>);
  const int gr = tile_grid(c, k_ppcg_update_r<4, F>, d4.ns);
  const bool blk = c.prec == PREC_JAC_BLOCK;
  const int gs = blk ? tile_grid(c, k_ppcg_calc_sd_block<F>, sd_blocks(d4))
                     : tile_grid(c, k_ppcg_sd<4, F>, d4.ns);
  const int gst = tile_grid(c, k_ppcg_step<F>, d4.ns);
  // block Jacobi: inner steps two at a time through k_ppcg_step, the first
  // writing sd to the second buffer and the second back, so each outer
  // iteration ends with sd where it began
  double* const sd_a = d4.sd;
  double* const sd_b = c.sd2.f;
  const int gz = tile_grid(c, k_ppcg_rz_step<TH, F>);
  const int gp = tile_grid(c, k_cg_calc_p<4, F>, d4.ns);
  for (int i = 0; i < iters; i++) {
    k_cg_calc_w<TH, F><<<gw, kBlock, 0, c.stream>>>(d, red, st);
    k_ppcg_ur_sd<TH, F><<<gu, kBlock, 0, c.stream>>>(d, red, st, theta);
    for (int k = 0; k < c.n_ppcg; k++) {
      if (blk && sd_b && k + 1 < c.n_ppcg) {
        k_ppcg_step<F><<<gst, kBlock, 0, c.stream>>>(d4, red, c.ppcg_alpha_h[k],
                                                     c.ppcg_beta_h[k], st, sd_a, sd_b);
        k_ppcg_step<F><<<gst, kBlock, 0, c.stream>>>(d4, red, c.ppcg_alpha_h[k + 1],
                                                     c.ppcg_beta_h[k + 1], st, sd_b, sd_a);
        k++;
        continue;
      }
      k_ppcg_update_r<4, F><<<gr, kBlock, 0, c.stream>>>(d4, red, st);
      if (blk)
        k_ppcg_calc_sd_block<F><<<gs, kBlock, 0, c.stream>>>(
            d4, c.ppcg_alpha_h[k], c.ppcg_beta_h[k], st);
      else
        k_ppcg_sd<4, F><<<gs, kBlock, 0, c.stream>>>(d4, red, 1, div_const(1.0), c.ppcg_alpha_h[k],
                                                     c.ppcg_beta_h[k], st);
    }
    k_ppcg_rz_step<TH, F><<<gz, kBlock, 0, c.stream>>>(d, red, st);
    k_cg_calc_p<4, F><<<gp, kBlock, 0, c.stream>>>(d4, red, 0.0, st, c.res_counter);
  }
}

static void enqueue_ppcg_iterations(Chunk& c, int iters) {
  if (c.TH == 16) {
    if (c.arith == 2) enqueue_ppcg_iterations_t<16, 2>(c, iters);
    else if (c.arith == 1) enqueue_ppcg_iterations_t<16, 1>(c, iters);
    else enqueue_ppcg_iterations_t<16, 0>(c, iters);
  } else {
    if (c.arith == 2) enqueue_ppcg_iterations_t<4, 2>(c, iters);
    else if (c.arith == 1) enqueue_ppcg_iterations_t<4, 1>(c, iters);
    else enqueue_ppcg_iterations_t<4, 0>(c, iters);
  }
}

template <int TH, int F, int NV>
static void enqueue_resident_iterations_t(Chunk& c, int iters) {
  const Dev d = c.dev();
  const Dev d4 = dev4(c);  // calc_p takes no sum
  const Red red = c.red();
  const int gw = tile_grid(c, k_cg_calc_w<TH, F>);
  const int gu = tile_grid(c, k_cg_calc_ur<TH, F, NV>);
  const int gp = tile_grid(c, k_cg_calc_p<4, F>, d4.ns);
  for (int i = 0; i < iters; i++) {
    k_cg_calc_w<TH, F><<<gw, kBlock, 0, c.stream>>>(d, red, c.res_state);
    k_cg_calc_ur<TH, F, NV><<<gu, kBlock, 0, c.stream>>>(d, red, 0.0, c.res_state);
    k_cg_calc_p<4, F><<<gp, kBlock, 0, c.stream>>>(d4, red, 0.0, c.res_state,
                                                   c.res_counter);
  }
}

template <int TH, int NV>
static void enqueue_resident_iterations_th(Chunk& c, int iters) {
  if (c.arith == 2)
    enqueue_resident_iterations_t<TH, 2, NV>(c, iters);
  else if (c.arith == 1)
    enqueue_resident_iterations_t<TH, 1, NV>(c, iters);
  else
    enqueue_resident_iterations_t<TH, 0, NV>(c, iters);
}

template <int NV>
static void enqueue_resident_iterations_nv(Chunk& c, int iters) {
  if (c.TH == 16)
    enqueue_resident_iterations_th<16, NV>(c, iters);
  else
    enqueue_resident_iterations_th<4, NV>(c, iters);
}

static void enqueue_resident_iterations(Chunk& c, int iters, bool true_exit) {
  if (true_exit)
    enqueue_resident_iterations_nv<2>(c, iters);
  else
    enqueue_resident_iterations_nv<1>(c, iters);
}

void resident_release() {
  Chunk& c = chunk();
  if (c.res_graph) cudaGraphExecDestroy(c.res_graph);
  c.res_graph = nullptr;
  c.res_graph_iters = 0;
  cudaFree(c.res_state);
  cudaFree(c.res_coef);
  cudaFree(c.res_counter);
  cudaFree(c.res_bar);
  c.res_bar = nullptr;
  if (c.res_ppcg_graph) cudaGraphExecDestroy(c.res_ppcg_graph);
  c.res_ppcg_graph = nullptr;
  c.res_ppcg_key.clear();
  cudaFreeHost(c.res_state_h);
  c.res_state = nullptr;
  c.res_coef = nullptr;
  c.res_counter = nullptr;
  c.res_state_h = nullptr;
  c.res_coef_n = 0;
}

// CG iterations n_begin..loop_max of tea_solve.f90:147-332 with all scalars
// on the device.  The iterations are queued in batches replayed from a
// captured CUDA graph; after each batch the host reads the loop state once.
// Kernels queued after the loop has stopped return at once.  The arithmetic
// and the exit test are those of the per-call path, so the results are
// bit-identical to it.
// The persistent loop runs when asked for (resident_mode 2).  The default
// is the graph loop: measured per CG iteration (jac_diag, chain form), the
// graph loop took 24.3 / 51.7 / 150 / 455 us at 512^2 / 1024^2 / 2048^2 /
// 4096^2 and the persistent one 25.3 / 56.3 / 154 / 455 us.  At small grids
// every phase is latency-bound either way, and three grid barriers cost
// what three graph-replayed launches cost; removing the barrier's back-off
// or using one block per SM changed nothing.  The persistent loop keeps the
// r.z exit test only (the true-residual exit uses the graph loop).
static bool use_persistent(const Chunk& c, bool true_exit) {
  return !true_exit && !c.profiler_on && c.resident_mode == 2;
}

int resident_cg_iterations(int n_begin, int loop_max, double rro_in,
                           double eps_target, double* rro_out,
                           double* error_out, int* n_done, int* converged,
                           double* cg_alphas, double* cg_betas, bool true_exit) {
  Chunk& c = chunk();
  flush_pending_inner(c);
  if (c.res_graph &&
      (c.res_graph_true_exit != true_exit || c.res_graph_epoch != c.field_epoch)) {
    cudaGraphExecDestroy(c.res_graph);
    c.res_graph = nullptr;
  }
  const int batch = 16;
  if (c.res_coef_n < loop_max + 2) {
    cudaFree(c.res_coef);
    c.res_coef = nullptr;
    if (!check_cuda(cudaMalloc(&c.res_coef, 2 * sizeof(double) * (loop_max + 2)),
                    "cudaMalloc resident coefficients"))
      return -1;
    c.res_coef_n = loop_max + 2;
  }
  if (!c.res_state) {
    if (!check_cuda(cudaMalloc(&c.res_state, sizeof(ResState)), "cudaMalloc state") ||
        !check_cuda(cudaMallocHost(&c.res_state_h, sizeof(ResState)),
                    "cudaMallocHost state") ||
        !check_cuda(cudaMalloc(&c.res_counter, sizeof(unsigned int)),
                    "cudaMalloc counter") ||
        !check_cuda(cudaMalloc(&c.res_bar, 3 * sizeof(unsigned int)),
                    "cudaMalloc barrier"))
      return -1;
    cudaMemsetAsync(c.res_counter, 0, sizeof(unsigned int), c.stream);
  }
  ResState& h = *c.res_state_h;
  memset(&h, 0, sizeof(h));
  h.rro = rro_in;
  h.eps_target = eps_target;
  h.n = n_begin;
  h.loop_max = loop_max;
  h.check = c.solver_checks;
  h.alphas = c.res_coef;
  h.betas = c.res_coef + c.res_coef_n;
  if (!check_cuda(cudaMemcpyAsync(c.res_state, &h, sizeof(ResState),
                                  cudaMemcpyHostToDevice, c.stream),
                  "resident state upload"))
    return -1;
  if (use_persistent(c, true_exit)) {
    // one cooperative launch runs the loop to its end
    if (!check_cuda(cudaMemsetAsync(c.res_bar, 0, 3 * sizeof(unsigned int), c.stream),
                    "barrier reset") ||
        !launch_cg_persistent(c))
      return -1;
    count_launch("resident_cg_persistent");
    int err = 0;
    if (!check_cuda(cudaMemcpyAsync(&h, c.res_state, sizeof(ResState),
                                    cudaMemcpyDeviceToHost, c.stream),
                    "resident state read") ||
        !check_cuda(cudaMemcpyAsync(&err, c.res_bar + 2, sizeof(int),
                                    cudaMemcpyDeviceToHost, c.stream),
                    "barrier flag read") ||
        !check_cuda(cudaStreamSynchronize(c.stream), "persistent CG"))
      return -1;
    if (err) {
      fail(25, "persistent CG: a grid barrier timed out");
      return -1;
    }
    if (!h.stop) {
      fail(24, "persistent CG loop ended before its exit test");
      return -1;
    }
  } else {
  if (!c.res_graph && !c.profiler_on) {
    cudaGraph_t graph = nullptr;
    if (!check_cuda(cudaStreamBeginCapture(c.stream, cudaStreamCaptureModeThreadLocal),
                    "graph capture"))
      return -1;
    enqueue_resident_iterations(c, batch, true_exit);
    if (!check_cuda(cudaStreamEndCapture(c.stream, &graph), "graph capture end") ||
        !check_cuda(cudaGraphInstantiate(&c.res_graph, graph, 0), "graph instantiate"))
      return -1;
    cudaGraphDestroy(graph);
    c.res_graph_iters = batch;
    c.res_graph_true_exit = true_exit;
    c.res_graph_epoch = c.field_epoch;
  }
  // every batch runs at least one iteration until the loop stops, so the
  // loop needs at most this many batches; more means the state is corrupt
  const long long max_batches = (long long)(loop_max - n_begin) / batch + 3;
  for (long long nb = 0;; nb++) {
    if (nb >= max_batches) {
      fail(24, "resident CG loop did not stop after %lld batches", nb);
      return -1;
    }
    if (c.res_graph) {
      if (!check_cuda(cudaGraphLaunch(c.res_graph, c.stream), "graph launch"))
        return -1;
    } else {
      enqueue_resident_iterations(c, batch, true_exit);
      check_cuda(cudaGetLastError(), "resident launch");
    }
    for (int i = 0; i < 3 * batch; i++) count_launch("resident_cg");
    if (!check_cuda(cudaMemcpyAsync(&h, c.res_state, sizeof(ResState),
                                    cudaMemcpyDeviceToHost, c.stream),
                    "resident state read") ||
        !check_cuda(cudaStreamSynchronize(c.stream), "resident sync"))
      return -1;
    if (h.stop && !h.p_pending) break;
  }
  }
  *rro_out = h.rro;
  *error_out = h.error;
  c.res_last_rr_true = h.rr_true;
  *n_done = h.n;
  *converged = h.converged;
  c.res_breakdown = h.breakdown;
  c.res_breakdown_n = h.breakdown_n;
  if (cg_alphas && cg_betas) {
    const int n = h.n - n_begin + 1;
    cudaMemcpyAsync(cg_alphas + n_begin, c.res_coef + n_begin, n * sizeof(double),
                    cudaMemcpyDeviceToHost, c.stream);
    cudaMemcpyAsync(cg_betas + n_begin, c.res_coef + c.res_coef_n + n_begin,
                    n * sizeof(double), cudaMemcpyDeviceToHost, c.stream);
    if (!check_cuda(cudaStreamSynchronize(c.stream), "resident coefficients"))
      return -1;
  }
  return 0;
}

// PPCG iterations n_begin..loop_max with all scalars on the device, batches
// of 4 iterations replayed from a captured graph until the loop stops.  The
// kernels and the exit test are those of the per-call path (whose
// calc_ur + init_sd pair is fused here), so results are bit-identical.
int resident_ppcg_iterations(int n_begin, int loop_max, double rro_in,
                             double eps_target, double* rro_out, double* error_out,
                             int* n_done, int* converged) {
  Chunk& c = chunk();
  if (c.n_ppcg < 1) {
    fail(26, "resident PPCG: no coefficients (tea_leaf_ppcg_init_ocl_ first)");
    return -1;
  }
  const int batch = 4;
  if (!c.res_state) {
    if (!check_cuda(cudaMalloc(&c.res_state, sizeof(ResState)), "cudaMalloc state") ||
        !check_cuda(cudaMallocHost(&c.res_state_h, sizeof(ResState)),
                    "cudaMallocHost state") ||
        !check_cuda(cudaMalloc(&c.res_counter, sizeof(unsigned int)),
                    "cudaMalloc counter") ||
        !check_cuda(cudaMalloc(&c.res_bar, 3 * sizeof(unsigned int)),
                    "cudaMalloc barrier"))
      return -1;
    cudaMemsetAsync(c.res_counter, 0, sizeof(unsigned int), c.stream);
  }
  flush_pending_inner(c);
  const bool pairs = resident_pairs(c);
  if (pairs && (!ensure_alt_fields(c) || !tb_prepare(c))) return -1;
  // the one-pass inner steps (k_ppcg_step) write sd to the second buffer
  if (c.prec == PREC_JAC_BLOCK && !ensure_alt_fields(c)) return -1;
  std::vector<double> key = {c.ppcg_theta, (double)c.arith, (double)c.n_ppcg,
                             (double)c.field_epoch, pairs ? 1.0 : 0.0};
  key.insert(key.end(), c.ppcg_alpha_h, c.ppcg_alpha_h + c.n_ppcg);
  key.insert(key.end(), c.ppcg_beta_h, c.ppcg_beta_h + c.n_ppcg);
  if (c.res_ppcg_graph && key != c.res_ppcg_key) {
    cudaGraphExecDestroy(c.res_ppcg_graph);
    c.res_ppcg_graph = nullptr;
  }
  ResState& h = *c.res_state_h;
  memset(&h, 0, sizeof(h));
  h.rro = rro_in;
  h.eps_target = eps_target;
  h.n = n_begin;
  h.loop_max = loop_max;
  h.check = c.solver_checks;
  if (!check_cuda(cudaMemcpyAsync(c.res_state, &h, sizeof(ResState),
                                  cudaMemcpyHostToDevice, c.stream),
                  "resident state upload"))
    return -1;
  if (!c.res_ppcg_graph && !c.profiler_on) {
    cudaGraph_t graph = nullptr;
    if (!check_cuda(cudaStreamBeginCapture(c.stream, cudaStreamCaptureModeThreadLocal),
                    "graph capture"))
      return -1;
    enqueue_ppcg_iterations(c, batch);
    if (!check_cuda(cudaStreamEndCapture(c.stream, &graph), "graph capture end") ||
        !check_cuda(cudaGraphInstantiate(&c.res_ppcg_graph, graph, 0), "graph instantiate"))
      return -1;
    cudaGraphDestroy(graph);
    c.res_ppcg_key = key;
  }
  const int per_iter = pairs ? 4 + c.n_ppcg / 2 + 2 * (c.n_ppcg % 2)
                       : c.prec == PREC_JAC_BLOCK ? 4 + c.n_ppcg + c.n_ppcg % 2
                                                  : 4 + 2 * c.n_ppcg;
  const long long max_batches = (long long)(loop_max - n_begin) / batch + 3;
  for (long long nb = 0;; nb++) {
    if (nb >= max_batches) {
      fail(24, "resident PPCG loop did not stop after %lld batches", nb);
      return -1;
    }
    if (c.res_ppcg_graph) {
      if (!check_cuda(cudaGraphLaunch(c.res_ppcg_graph, c.stream), "graph launch"))
        return -1;
    } else {
      enqueue_ppcg_iterations(c, batch);
      check_cuda(cudaGetLastError(), "resident PPCG launch");
    }
    count_launches((long long)batch * per_iter);
    if (!check_cuda(cudaMemcpyAsync(&h, c.res_state, sizeof(ResState),
                                    cudaMemcpyDeviceToHost, c.stream),
                    "resident state read") ||
        !check_cuda(cudaStreamSynchronize(c.stream), "resident sync"))
      return -1;
    if (pairs && tb_error()) {
      fail(81, "fused PPCG inner steps: a shared-memory copy did not arrive");
      return -1;
    }
    if (h.stop && !h.p_pending) break;
  }
  if (pairs && ((long long)(h.n - n_begin + 1) * (c.n_ppcg / 2)) % 2 != 0) {
    // an odd number of fused pairs ran: the results are in r2/sd2
    const size_t n = (size_t)((32 - (c.H % 32)) % 32 + c.rows * c.S + 32) * sizeof(double);
    if (!check_cuda(cudaMemcpyAsync(c.r.base, c.r2.base, n, cudaMemcpyDeviceToDevice, c.stream),
                    "resident PPCG r copy back") ||
        !check_cuda(cudaMemcpyAsync(c.sd.base, c.sd2.base, n, cudaMemcpyDeviceToDevice,
                                    c.stream),
                    "resident PPCG sd copy back"))
      return -1;
  }
  *rro_out = h.rro;
  *error_out = h.error;
  *n_done = h.n;
  *converged = h.converged;
  c.res_breakdown = h.breakdown;
  c.res_breakdown_n = h.breakdown_n;
  return 0;
}

}  // namespace tea

namespace tea {

// FP64 pipe throughput probe: every thread runs 8 independent fused
// multiply-add chains, so the FP64 pipe, not latency, sets the time.
__global__ void k_fp64_rate(double* out, int iters, double b, double c) {
  double a0 = threadIdx.x, a1 = a0 + 1, a2 = a0 + 2, a3 = a0 + 3, a4 = a0 + 4,
         a5 = a0 + 5, a6 = a0 + 6, a7 = a0 + 7;
  for (int i = 0; i < iters; i++) {
    a0 = __fma_rn(a0, b, c);
    a1 = __fma_rn(a1, b, c);
    a2 = __fma_rn(a2, b, c);
    a3 = __fma_rn(a3, b, c);
    a4 = __fma_rn(a4, b, c);
    a5 = __fma_rn(a5, b, c);
    a6 = __fma_rn(a6, b, c);
    a7 = __fma_rn(a7, b, c);
  }
  const double s = ((a0 + a1) + (a2 + a3)) + ((a4 + a5) + (a6 + a7));
  if (s == 12345.678) out[0] = s;  // keeps the chains live
}

double measure_fp64_rate() {
  Chunk& c = chunk();
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  double* out = nullptr;
  if (!check_cuda(cudaMalloc(&out, sizeof(double)), "probe alloc")) return -1.0;
  cudaStream_t s = c.stream;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  const int blocks = sms * 8, threads = 256, iters = 4096;
  k_fp64_rate<<<blocks, threads, 0, s>>>(out, 64, 0.999, 1e-3);  // warm-up
  cudaEventRecord(e0, s);
  k_fp64_rate<<<blocks, threads, 0, s>>>(out, iters, 0.999, 1e-3);
  cudaEventRecord(e1, s);
  cudaEventSynchronize(e1);
  float ms = 0.0f;
  cudaEventElapsedTime(&ms, e0, e1);
  count_launch("fp64_rate");
  count_launch("fp64_rate");
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  const double instr = (double)blocks * threads * iters * 8.0;
  return instr / (ms * 1e-3);
}

}  // namespace tea
