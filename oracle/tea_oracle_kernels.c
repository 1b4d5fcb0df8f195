/*
 * TEST INFRASTRUCTURE ONLY -- CPU oracle, kernel half.
 *
 * One C function per OpenCL kernel of UK-MAC/TeaLeaf_OpenCL that the implicit
 * solve runs, with the kernel's arithmetic written in the kernel's own
 * operation order and over the kernel's own launch range.  Launch ranges come
 * from the KERNEL_{X,Y}_{MIN,MAX} bounds given to compileKernel
 * (ocl_kernels.cpp:51-114) combined with findPaddingSize
 * (ocl_kernels.cpp:123-134) and WITHIN_BOUNDS (macros_cl.cl:25-29):
 *   bounds (0,0)   -> interior  col in [H, H+x_max), row in [H, H+y_max)
 *   bounds (1-H,H) -> col in [1, x_max+2H), row in [1, y_max+2H)
 *   bounds (-H,H)  -> the whole padded array
 * Fields use the reference layout: element (col,row) at col + row*(x_max+2H)
 * (THARR2D, macros_cl.cl:20-22), each array holding (x_max+2H+1)*(y_max+2H+1)
 * zero-initialised doubles (ocl_buffers.cpp:6-69).
 *
 * Build with -ffp-contract=off: no multiply-add contraction, so every result
 * is the IEEE double result of the expression as written.
 */
#include "tea_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef struct {
  int x_max, y_max, H, solver, prec;
  int xs, ys;
  long n2;
  double *density, *energy0, *energy1, *volume;
  double *cellx, *celldx, *vertexx, *vertexdx;
  double *celly, *celldy, *vertexy, *vertexdy;
  double *p, *r, *w, *Mi, *Kx, *Ky, *sd, *u, *u0, *z, *cp, *bfp;
  double *ch_alphas, *ch_betas;
  double *ztmp; /* M^-1 r kept out of z where the reference keeps it local */
  int n_coefs;
  double theta_cheby, theta_ppcg;
  double *scratch[4];
  double *scratchb[4];
} OrcChunk;

static OrcChunk C;
static int C_ready = 0;

/* Arithmetic form, as in the CUDA library: 0 = every expression of the
 * reference kernels as written (each multiply and add rounded); 1 = the same
 * expressions with each multiply feeding an add contracted into one fused
 * multiply-add (C fma()), dot-product accumulation acc = fma(a,b,acc), and
 * the block-Jacobi first-row division done through a stored reciprocal;
 * 2 = as 1, with the 5-point operator as one left-to-right chain of fma()
 * (D x_c - Ky_n x_n - Ky_c x_s - Kx_e x_e - Kx_c x_w) and b - A x as the
 * chain started from b. */
static int FUSED = 1;

void oracle_set_arithmetic(int form) { FUSED = (form >= 0 && form <= 2) ? form : 1; }
int oracle_get_arithmetic(void) { return FUSED; }

#define IDX(col, row) ((long)(col) + (long)(row) * C.xs)

/* ------------------------------------------------------------------------ */
/* Canonical fixed-order summation                                          */
/* ------------------------------------------------------------------------ */
/*
 * Interior cells (x in [0,x_max), y in [0,y_max)) are cut into tiles of 32
 * columns x TH rows, and tiles into supertiles of 8 tiles along x
 * (256 columns x TH rows).
 *   1. lane l of a tile holds column 32*tx+l; it adds its TH rows bottom to
 *      top into an accumulator that starts at +0.0 (cells outside the
 *      interior add +0.0);
 *   2. the 32 lane sums are combined by a butterfly: for offset 16,8,4,2,1
 *      every lane l replaces a[l] by a[l] + a[l^offset]; the tile sum is a[0];
 *   3. a supertile sum is the same butterfly over 32 lanes whose first 8
 *      hold the tile sums (0.0 for tiles past the interior), the rest 0.0;
 *   4. supertile sums are numbered row-major (sy*nsx+sx); lane i of 256
 *      adds sums i, i+256, i+512, ... in order from +0.0; each group of 32
 *      lanes is butterflied, and the 8 group sums are butterflied as in 3.
 * TH is 16 when the grid has at least 1216 supertiles of 16 rows, else 4.
 */
int oracle_reduction_rows(int x_max, int y_max) {
  long nsx = (x_max + 255) / 256;
  long nsy16 = (y_max + 15) / 16;
  return (nsx * nsy16 >= 1216) ? 16 : 4;
}

static double butterfly32(const double* v) {
  double a[32], b[32];
  memcpy(a, v, sizeof(a));
  for (int off = 16; off >= 1; off >>= 1) {
    for (int l = 0; l < 32; l++) b[l] = a[l] + a[l ^ off];
    memcpy(a, b, sizeof(a));
  }
  return a[0];
}

static double sum8(const double* v8) {
  double a[32];
  for (int l = 0; l < 32; l++) a[l] = (l < 8) ? v8[l] : 0.0;
  return butterfly32(a);
}

/* Lane accumulation: acc + a*b, fused or not.  Plain sums pass b = 1.0,
 * for which both forms give acc + a exactly. */
static inline double lane_acc(double acc, double a, double b, int fused) {
  return fused ? fma(a, b, acc) : acc + a * b;
}

/* (hi, lo) += a*b for float a, b: the product split exactly into p + e
 * with e = fmaf(a, b, -p), p added with a two-sum (the mixed solve's lane
 * accumulation). */
static inline void acc_pair(float* hi, float* lo, float a, float b) {
  const float p = a * b;
  const float e = fmaf(a, b, -p);
  const float s = *hi + p;
  const float bb = s - *hi;
  const float t = (*hi - (s - bb)) + (p - bb);
  *lo = *lo + (t + e);
  *hi = s;
}

#define LANE_FLOAT_PAIR 2 /* reduce_pairs mode for FP32 products */

static double reduce_pairs(const double* A, const double* B, int X, int Y,
                           int fused) {
  const int TH = oracle_reduction_rows(X, Y);
  const long ntx = (X + 31) / 32;
  const long nty = (Y + TH - 1) / TH;
  const long nsx = (ntx + 7) / 8;
  const long ns = nsx * nty;
  double* S = (double*)malloc(sizeof(double) * (size_t)(ns > 0 ? ns : 1));
#pragma omp parallel for schedule(static)
  for (long s = 0; s < ns; s++) {
    const long sy = s / nsx, sx = s % nsx;
    double t8[8];
    for (int wv = 0; wv < 8; wv++) {
      const long tx = 8 * sx + wv;
      if (tx >= ntx) {
        t8[wv] = 0.0;
        continue;
      }
      double lanes[32];
      for (int l = 0; l < 32; l++) {
        const long col = 32 * tx + l;
        double acc = 0.0;
        float hi = 0.0f, lo = 0.0f;
        for (int j = 0; j < TH; j++) {
          const long row = (long)TH * sy + j;
          const int in = col < X && row < Y;
          const double a = in ? A[row * X + col] : 0.0;
          const double b = in ? (B ? B[row * X + col] : 1.0) : 0.0;
          if (fused == LANE_FLOAT_PAIR)
            acc_pair(&hi, &lo, (float)a, (float)b);
          else
            acc = lane_acc(acc, a, b, fused);
        }
        lanes[l] = fused == LANE_FLOAT_PAIR ? (double)hi + (double)lo : acc;
      }
      t8[wv] = butterfly32(lanes);
    }
    S[s] = sum8(t8);
  }
  double lanes256[256];
  for (int i = 0; i < 256; i++) {
    double acc = 0.0;
    for (long k = i; k < ns; k += 256) acc = acc + S[k];
    lanes256[i] = acc;
  }
  double w8[8];
  for (int wv = 0; wv < 8; wv++) w8[wv] = butterfly32(lanes256 + 32 * wv);
  free(S);
  return sum8(w8);
}

double oracle_reduce(const double* contrib, int X, int Y) {
  return reduce_pairs(contrib, NULL, X, Y, 0);
}

double oracle_reduce_pairs(const double* a, const double* b, int X, int Y,
                           int fused) {
  return reduce_pairs(a, b, X, Y, fused);
}

/* plain sum of an interior-indexed scratch array */
static double reduce_scratch(int k) {
  return reduce_pairs(C.scratch[k], NULL, C.x_max, C.y_max, 0);
}

/* dot-product sum of scratch pairs (a in scratch, b in scratchb) */
static double reduce_dot(int k) {
  return reduce_pairs(C.scratch[k], C.scratchb[k], C.x_max, C.y_max, FUSED != 0);
}

#define SCR(k, col, row) \
  C.scratch[k][(long)((row)-C.H) * C.x_max + ((col)-C.H)]
#define SCRB(k, col, row) \
  C.scratchb[k][(long)((row)-C.H) * C.x_max + ((col)-C.H)]
#define DOT(k, col, row, a, b) \
  do {                         \
    SCR(k, col, row) = (a);    \
    SCRB(k, col, row) = (b);   \
  } while (0)

/* ------------------------------------------------------------------------ */
/* Lifecycle                                                                */
/* ------------------------------------------------------------------------ */

static double* zalloc(long n) {
  double* p = (double*)calloc((size_t)n, sizeof(double));
  return p;
}

static void mix_free(void);

void oracle_finalise(void) {
  if (!C_ready) return;
  mix_free();
  double** all[] = {&C.density, &C.energy0, &C.energy1, &C.volume, &C.cellx,
                    &C.celldx,  &C.vertexx, &C.vertexdx, &C.celly, &C.celldy,
                    &C.vertexy, &C.vertexdy, &C.p, &C.r, &C.w, &C.Mi, &C.Kx,
                    &C.Ky, &C.sd, &C.u, &C.u0, &C.z, &C.cp, &C.bfp,
                    &C.ch_alphas, &C.ch_betas, &C.ztmp, &C.scratch[0], &C.scratch[1],
                    &C.scratch[2], &C.scratch[3], &C.scratchb[0], &C.scratchb[1],
                    &C.scratchb[2], &C.scratchb[3]};
  for (size_t i = 0; i < sizeof(all) / sizeof(all[0]); i++) {
    free(*all[i]);
    *all[i] = NULL;
  }
  C_ready = 0;
}

/* initialise_ocl_ (ocl_init.cpp:11-17) + initBuffers (ocl_buffers.cpp). */
int oracle_initialise(int x_max, int y_max, int H, int solver, int prec) {
  oracle_finalise();
  if (x_max < 1 || y_max < 1 || H < 1) return -1;
  memset(&C, 0, sizeof(C));
  C.x_max = x_max;
  C.y_max = y_max;
  C.H = H;
  C.solver = solver;
  C.prec = prec;
  C.xs = x_max + 2 * H;
  C.ys = y_max + 2 * H;
  C.n2 = (long)(C.xs + 1) * (C.ys + 1);
  double** f2[] = {&C.density, &C.energy0, &C.energy1, &C.volume, &C.p, &C.r,
                   &C.w,       &C.Mi,      &C.Kx,      &C.Ky,     &C.sd, &C.u,
                   &C.u0,      &C.z,       &C.cp,      &C.bfp,    &C.ztmp};
  for (size_t i = 0; i < sizeof(f2) / sizeof(f2[0]); i++) {
    *f2[i] = zalloc(C.n2);
    if (!*f2[i]) return -2;
  }
  double** f1[] = {&C.cellx, &C.celldx, &C.vertexx, &C.vertexdx,
                   &C.celly, &C.celldy, &C.vertexy, &C.vertexdy};
  for (size_t i = 0; i < sizeof(f1) / sizeof(f1[0]); i++) {
    *f1[i] = zalloc((C.xs > C.ys ? C.xs : C.ys) + 2);
    if (!*f1[i]) return -2;
  }
  for (int k = 0; k < 4; k++) {
    C.scratch[k] = zalloc((long)x_max * y_max);
    C.scratchb[k] = zalloc((long)x_max * y_max);
    if (!C.scratch[k] || !C.scratchb[k]) return -2;
  }
  C_ready = 1;
  return 0;
}

/* ------------------------------------------------------------------------ */
/* Setup kernels                                                            */
/* ------------------------------------------------------------------------ */

/* initialise_chunk_first / _second, initialise_chunk_cl.cl:3-68.  xarea and
 * yarea are not computed: no kernel of the solve or field summary reads
 * them. */
void oracle_initialise_chunk(double xmin, double ymin, double dx, double dy) {
  const int H = C.H;
  for (int col = 0; col <= C.x_max + H; col++) {
    C.vertexx[col] = xmin + dx * (double)(((col)-1) - H + 1);
    C.vertexdx[col] = dx;
    const double plus1 = xmin + dx * (double)((col)-H + 1);
    C.cellx[col] = 0.5 * (C.vertexx[col] + plus1);
    C.celldx[col] = dx;
  }
  for (int row = 0; row <= C.y_max + H; row++) {
    C.vertexy[row] = ymin + dy * (double)(((row)-1) - H + 1);
    C.vertexdy[row] = dy;
    const double plus1 = ymin + dy * (double)((row)-H + 1);
    C.celly[row] = 0.5 * (C.vertexy[row] + plus1);
    C.celldy[row] = dy;
  }
  for (int row = H - 1; row <= C.y_max + H; row++)
    for (int col = H - 1; col <= C.x_max + H; col++)
      C.volume[IDX(col, row)] = dx * dy;
}

/* generate_chunk_init, generate_chunk, generate_chunk_init_u
 * (generate_chunk_cl.cl:3-95), in the order of
 * generate_chunk_kernel_ocl.cpp:52-91.  Geometry codes: 1 rectangle,
 * 2 circle, 3 point (data.f90 g_rect/g_circ/g_point). */
void oracle_generate_chunk(int nstates, const double* sd, const double* se,
                           const double* sxmin, const double* sxmax,
                           const double* symin, const double* symax,
                           const double* sradius, const int* sgeom) {
  const int H = C.H;
#pragma omp parallel for schedule(static)
  for (int row = H; row < H + C.y_max; row++) {
    for (int col = H; col < H + C.x_max; col++) {
      C.energy0[IDX(col, row)] = se[0];
      C.density[IDX(col, row)] = sd[0];
    }
  }
  for (int s = 1; s < nstates; s++) {
#pragma omp parallel for schedule(static)
    for (int row = H; row < H + C.y_max; row++) {
      for (int col = H; col < H + C.x_max; col++) {
        const double x_cent = sxmin[s];
        const double y_cent = symin[s];
        int hit = 0;
        if (sgeom[s] == 1) {
          hit = C.vertexx[1 + col] >= sxmin[s] && C.vertexx[col] < sxmax[s] &&
                C.vertexy[1 + row] >= symin[s] && C.vertexy[row] < symax[s];
        } else if (sgeom[s] == 2) {
          const double x_pos = C.cellx[col] - x_cent;
          const double y_pos = C.celly[row] - y_cent;
          const double radius = sqrt(x_pos * x_pos + y_pos * y_pos);
          hit = radius <= sradius[s];
        } else if (sgeom[s] == 3) {
          hit = C.vertexx[col] == x_cent && C.vertexy[row] == y_cent;
        }
        if (hit) {
          C.energy0[IDX(col, row)] = se[s];
          C.density[IDX(col, row)] = sd[s];
        }
      }
    }
  }
#pragma omp parallel for schedule(static)
  for (int row = H; row < H + C.y_max; row++) {
    for (int col = H; col < H + C.x_max; col++) {
      const long c = IDX(col, row);
      C.u[c] = C.energy0[c] * C.density[c];
      C.u0[c] = C.energy0[c] * C.density[c];
    }
  }
}

/* set_field_cl.cl:3-13 */
void oracle_set_field(void) {
  const int H = C.H;
#pragma omp parallel for schedule(static)
  for (int row = H; row < H + C.y_max; row++)
    for (int col = H; col < H + C.x_max; col++)
      C.energy1[IDX(col, row)] = C.energy0[IDX(col, row)];
}

/* ------------------------------------------------------------------------ */
/* Solver kernels                                                           */
/* ------------------------------------------------------------------------ */

/* The 5-point operator exactly as written inline in every kernel, e.g.
 * tea_leaf_cg_cl.cl:59-63. */
static inline double smvp_at(const double* x, long c) {
  const long xs = C.xs;
  const double D = (1.0 + (C.Ky[c + xs] + C.Ky[c]) + (C.Kx[c + 1] + C.Kx[c]));
  if (!FUSED)
    return D * x[c] - (C.Ky[c + xs] * x[c + xs] + C.Ky[c] * x[c - xs]) -
           (C.Kx[c + 1] * x[c + 1] + C.Kx[c] * x[c - 1]);
  if (FUSED == 2) {
    double t = D * x[c];
    t = fma(-C.Ky[c + xs], x[c + xs], t);
    t = fma(-C.Ky[c], x[c - xs], t);
    t = fma(-C.Kx[c + 1], x[c + 1], t);
    return fma(-C.Kx[c], x[c - 1], t);
  }
  const double t1 = fma(C.Ky[c], x[c - xs], C.Ky[c + xs] * x[c + xs]);
  const double t2 = fma(C.Kx[c], x[c - 1], C.Kx[c + 1] * x[c + 1]);
  return fma(D, x[c], -t1) - t2;
}

/* b - A x: the reference's b - smvp, or the chain started from b */
static inline double b_minus_smvp(const double* x, long c, double b) {
  if (FUSED != 2) return b - smvp_at(x, c);
  const long xs = C.xs;
  const double D = (1.0 + (C.Ky[c + xs] + C.Ky[c]) + (C.Kx[c + 1] + C.Kx[c]));
  double t = fma(-D, x[c], b);
  t = fma(C.Ky[c + xs], x[c + xs], t);
  t = fma(C.Ky[c], x[c - xs], t);
  t = fma(C.Kx[c + 1], x[c + 1], t);
  return fma(C.Kx[c], x[c - 1], t);
}

/* a*p + bl*br, the Chebyshev/PPCG coefficient update */
static inline double coef_update(double a, double p, double bl, double br) {
  return FUSED ? fma(a, p, bl * br) : a * p + bl * br;
}

/* Rows in the 4-row block-Jacobi strip starting at interior row 4g:
 * BLOCK_TOP, macros_cl.cl:6-10, enabled when y_max % 4 != 0
 * (ocl_kernels.cpp:26-29).  The reference's formula min(y_max+2-row, 4)
 * (row = H+4g) counts one halo row too many when H = 1 and is exact when
 * H = 2; for H >= 3 it undercounts and reads unset local memory, so there the
 * strip is taken as the remaining interior rows. */
static inline int block_top(int g) {
  if (C.y_max % 4 == 0) return 4;
  int up = C.y_max - 4 * g + (C.H == 1 ? 1 : 0);
  return up < 4 ? up : 4;
}

#define COEF_A(rk) (-C.Ky[IDX(col, rk)])
#define COEF_B(rk)                                                 \
  (1.0 + (C.Ky[IDX(col, (rk) + 1)] + C.Ky[IDX(col, rk)]) +         \
   (C.Kx[IDX(col + 1, rk)] + C.Kx[IDX(col, rk)]))
#define COEF_C(rk) (-C.Ky[IDX(col, (rk) + 1)])

/* tea_leaf_block_init, tea_block_jacobi.cl:78-105 */
static void block_init(void) {
  const int H = C.H;
  const int ng = (C.y_max + 3) / 4;
#pragma omp parallel for schedule(static)
  for (int g = 0; g < ng; g++) {
    const int row0 = H + 4 * g;
    const int upper = block_top(g);
    for (int col = H; col < H + C.x_max; col++) {
      C.cp[IDX(col, row0)] = COEF_C(row0) / COEF_B(row0);
      if (FUSED) C.bfp[IDX(col, row0)] = 1.0 / COEF_B(row0);
      for (int k = 1; k < upper; k++) {
        const int rk = row0 + k;
        C.bfp[IDX(col, rk)] =
            1.0 / (COEF_B(rk) - COEF_A(rk) * C.cp[IDX(col, rk - 1)]);
        C.cp[IDX(col, rk)] = COEF_C(rk) * C.bfp[IDX(col, rk)];
      }
    }
  }
}

/* block_solve_func, tea_block_jacobi.cl:6-42, applied to every strip:
 * zout = M_block^-1 rin.  Rows of the strip beyond the interior read r = 0
 * (the kernels zero their local copy there); z is written on interior rows
 * only. */
static void block_solve(const double* rin, double* zout) {
  const int H = C.H;
  const int ng = (C.y_max + 3) / 4;
#pragma omp parallel for schedule(static)
  for (int g = 0; g < ng; g++) {
    const int row0 = H + 4 * g;
    const int upper = block_top(g);
    for (int col = H; col < H + C.x_max; col++) {
      double rl[4], dp[4], zl[4];
      for (int k = 0; k < 4; k++) {
        const int rk = row0 + k;
        rl[k] = (rk < H + C.y_max) ? rin[IDX(col, rk)] : 0.0;
      }
      dp[0] = FUSED ? rl[0] * C.bfp[IDX(col, row0)] : rl[0] / COEF_B(row0);
      for (int k = 1; k < upper; k++) {
        const int rk = row0 + k;
        if (FUSED)
          dp[k] = fma(C.Ky[IDX(col, rk)], dp[k - 1], rl[k]) * C.bfp[IDX(col, rk)];
        else
          dp[k] = (rl[k] - COEF_A(rk) * dp[k - 1]) * C.bfp[IDX(col, rk)];
      }
      zl[upper - 1] = dp[upper - 1];
      for (int k = upper - 2; k >= 0; k--)
        zl[k] = FUSED ? fma(-C.cp[IDX(col, row0 + k)], zl[k + 1], dp[k])
                      : dp[k] - C.cp[IDX(col, row0 + k)] * zl[k + 1];
      for (int k = 0; k < upper; k++) {
        const int rk = row0 + k;
        if (rk < H + C.y_max) zout[IDX(col, rk)] = zl[k];
      }
    }
  }
}

/* tea_leaf_init_common + tea_leaf_zero_boundary + generate_chunk_init_u with
 * energy1, as run by CloverChunk::tea_leaf_common_init
 * (tea_leaf_kernel_ocl.cpp:254-289); rx, ry from calcrxry (:8-32), which
 * reads celldx/celldy at index H+1. */
void oracle_common_init(int coef, double dt, double* rx, double* ry,
                        const int* zero_boundary, int reflective) {
  const int H = C.H;
  const double dx = C.celldx[1 + H];
  const double dy = C.celldy[1 + H];
  const double RX = dt / (dx * dx);
  const double RY = dt / (dy * dy);
  *rx = RX;
  *ry = RY;
  /* tea_leaf_common_cl.cl:56-90 over [1, x_max+2H) x [1, y_max+2H) */
#pragma omp parallel for schedule(static)
  for (int row = 1; row < C.ys; row++) {
    for (int col = 1; col < C.xs; col++) {
      const long c = IDX(col, row);
      double dc = 0.0, dl = 0.0, dd = 0.0;
      if (coef == ORC_COEF_CONDUCTIVITY) {
        dc = C.density[c];
        dl = C.density[c - 1];
        dd = C.density[c - C.xs];
      } else if (coef == ORC_COEF_RECIP_CONDUCTIVITY) {
        dc = 1.0 / C.density[c];
        dl = 1.0 / C.density[c - 1];
        dd = 1.0 / C.density[c - C.xs];
      }
      double kx = (dl + dc) / (2.0 * dl * dc);
      kx = kx * RX;
      double ky = (dd + dc) / (2.0 * dd * dc);
      ky = ky * RY;
      C.Kx[c] = kx;
      C.Ky[c] = ky;
    }
  }
  if (!reflective) {
    /* tea_leaf_common_cl.cl:92-125 over the whole padded array */
    const int zl = zero_boundary[0], zr = zero_boundary[1];
    const int zb = zero_boundary[2], zt = zero_boundary[3];
#pragma omp parallel for schedule(static)
    for (int row = 0; row < C.ys; row++) {
      for (int col = 0; col < C.xs; col++) {
        const long c = IDX(col, row);
        if (zl && col <= H) {
          C.Kx[c] = 0;
          if (col < H) C.Ky[c] = 0;
        }
        if (zr && col > (C.x_max - 1) + H) {
          C.Kx[c] = 0;
          C.Ky[c] = 0;
        }
        if (zb && row <= H) {
          C.Ky[c] = 0;
          if (row < H) C.Kx[c] = 0;
        }
        if (zt && row > (C.y_max - 1) + H) {
          C.Ky[c] = 0;
          C.Kx[c] = 0;
        }
      }
    }
  }
  /* generate_chunk_cl.cl:67-80 with energy1 */
#pragma omp parallel for schedule(static)
  for (int row = H; row < H + C.y_max; row++) {
    for (int col = H; col < H + C.x_max; col++) {
      const long c = IDX(col, row);
      C.u[c] = C.energy1[c] * C.density[c];
      C.u0[c] = C.energy1[c] * C.density[c];
    }
  }
}

/* tea_leaf_calc_residual, tea_leaf_common_cl.cl:17-36 */
void oracle_calc_residual(void) {
  const int H = C.H;
#pragma omp parallel for schedule(static)
  for (int row = H; row < H + C.y_max; row++)
    for (int col = H; col < H + C.x_max; col++) {
      const long c = IDX(col, row);
      C.r[c] = b_minus_smvp(C.u, c, C.u0[c]);
    }
}

/* tea_leaf_calc_2norm, tea_leaf_common_cl.cl:38-54, with the argument
 * binding of tea_leaf_kernel_ocl.cpp:56-96 */
void oracle_calc_2norm(int which, double* norm) {
  const double *a, *b;
  if (which == 0) {
    a = C.u0;
    b = C.u0;
  } else if (which == 1) {
    a = C.r;
    b = C.r;
  } else if (which == 2) {
    a = C.r;
    b = (C.prec == ORC_PREC_NONE) ? C.r : C.z;
  } else {
    *norm = NAN;
    return;
  }
  const int H = C.H;
#pragma omp parallel for schedule(static)
  for (int row = H; row < H + C.y_max; row++)
    for (int col = H; col < H + C.x_max; col++) {
      const long c = IDX(col, row);
      DOT(0, col, row, a[c], b[c]);
    }
  *norm = reduce_dot(0);
}

/* tea_leaf_init_jac_diag, tea_leaf_common_cl.cl:127-142, whole array */
static void init_jac_diag(void) {
#pragma omp parallel for schedule(static)
  for (int row = 0; row < C.ys; row++)
    for (int col = 0; col < C.xs; col++) {
      const long c = IDX(col, row);
      const double diag =
          (1.0 + (C.Ky[c + C.xs] + C.Ky[c]) + (C.Kx[c + 1] + C.Kx[c]));
      C.Mi[c] = 1.0 / diag;
    }
}

/* CloverChunk::tea_leaf_cg_init_kernel, tea_leaf_kernel_ocl.cpp:167-187;
 * tea_leaf_cg_solve_init_p, tea_leaf_cg_cl.cl:8-41 */
void oracle_cg_init(double* rro) {
  const int H = C.H;
  if (C.prec == ORC_PREC_JAC_BLOCK) {
    block_init();
    block_solve(C.r, C.z);
  } else if (C.prec == ORC_PREC_JAC_DIAG) {
    init_jac_diag();
  }
#pragma omp parallel for schedule(static)
  for (int row = H; row < H + C.y_max; row++)
    for (int col = H; col < H + C.x_max; col++) {
      const long c = IDX(col, row);
      if (C.prec == ORC_PREC_JAC_BLOCK) {
        C.p[c] = C.z[c];
      } else if (C.prec == ORC_PREC_JAC_DIAG) {
        C.z[c] = C.r[c] * C.Mi[c];
        C.p[c] = C.z[c];
      } else {
        C.p[c] = C.r[c];
      }
      DOT(0, col, row, C.r[c], C.p[c]);
    }
  *rro = reduce_dot(0);
}

/* tea_leaf_cg_solve_calc_w, tea_leaf_cg_cl.cl:45-69 */
void oracle_cg_calc_w(double* pw) {
  const int H = C.H;
#pragma omp parallel for schedule(static)
  for (int row = H; row < H + C.y_max; row++)
    for (int col = H; col < H + C.x_max; col++) {
      const long c = IDX(col, row);
      C.w[c] = smvp_at(C.p, c);
      DOT(0, col, row, C.p[c], C.w[c]);
    }
  *pw = reduce_dot(0);
}

/* tea_leaf_cg_solve_calc_ur, tea_leaf_cg_cl.cl:73-137 */
void oracle_cg_calc_ur(double alpha, double* rrn) {
  const int H = C.H;
#pragma omp parallel for schedule(static)
  for (int row = H; row < H + C.y_max; row++)
    for (int col = H; col < H + C.x_max; col++) {
      const long c = IDX(col, row);
      if (FUSED) {
        C.u[c] = fma(alpha, C.p[c], C.u[c]);
        C.r[c] = fma(-alpha, C.w[c], C.r[c]);
      } else {
        C.u[c] = C.u[c] + alpha * C.p[c];
        C.r[c] = C.r[c] - alpha * C.w[c];
      }
    }
  if (C.prec == ORC_PREC_JAC_BLOCK) block_solve(C.r, C.z);
#pragma omp parallel for schedule(static)
  for (int row = H; row < H + C.y_max; row++)
    for (int col = H; col < H + C.x_max; col++) {
      const long c = IDX(col, row);
      if (C.prec == ORC_PREC_JAC_BLOCK) {
        DOT(0, col, row, C.r[c], C.z[c]);
      } else if (C.prec == ORC_PREC_JAC_DIAG) {
        C.z[c] = C.r[c] * C.Mi[c];
        DOT(0, col, row, C.r[c], C.z[c]);
      } else {
        DOT(0, col, row, C.r[c], C.r[c]);
      }
    }
  *rrn = reduce_dot(0);
}

/* tea_leaf_cg_solve_calc_p, tea_leaf_cg_cl.cl:141-160 */
void oracle_cg_calc_p(double beta) {
  const int H = C.H;
#pragma omp parallel for schedule(static)
  for (int row = H; row < H + C.y_max; row++)
    for (int col = H; col < H + C.x_max; col++) {
      const long c = IDX(col, row);
      const double src = (C.prec != ORC_PREC_NONE) ? C.z[c] : C.r[c];
      C.p[c] = FUSED ? fma(beta, C.p[c], src) : src + beta * C.p[c];
    }
}

static void store_coefs(const double* a, const double* b, int n) {
  free(C.ch_alphas);
  free(C.ch_betas);
  C.ch_alphas = (double*)malloc(sizeof(double) * (size_t)(n > 0 ? n : 1));
  C.ch_betas = (double*)malloc(sizeof(double) * (size_t)(n > 0 ? n : 1));
  if (n > 0) {
    memcpy(C.ch_alphas, a, sizeof(double) * (size_t)n);
    memcpy(C.ch_betas, b, sizeof(double) * (size_t)n);
  }
  C.n_coefs = n;
}

/* w = A u; r = u0 - w (first half of tea_leaf_cheby_solve_init_p and
 * tea_leaf_cheby_solve_calc_p, tea_leaf_cheby_cl.cl:14-26, :88-100) */
static void cheby_residual(void) {
  const int H = C.H;
#pragma omp parallel for schedule(static)
  for (int row = H; row < H + C.y_max; row++)
    for (int col = H; col < H + C.x_max; col++) {
      const long c = IDX(col, row);
      C.w[c] = smvp_at(C.u, c);
      C.r[c] = C.u0[c] - C.w[c];
    }
}

/* tea_leaf_cheby_solve_calc_u, tea_leaf_cheby_cl.cl:66-76 */
static void cheby_calc_u(void) {
  const int H = C.H;
#pragma omp parallel for schedule(static)
  for (int row = H; row < H + C.y_max; row++)
    for (int col = H; col < H + C.x_max; col++) {
      const long c = IDX(col, row);
      C.u[c] = C.u[c] + C.p[c];
    }
}

/* CloverChunk::tea_leaf_cheby_init_kernel, tea_leaf_kernel_ocl.cpp:98-129:
 * store coefficients, run cheby_solve_init_p then cheby_solve_calc_u. */
void oracle_cheby_init(const double* alphas, const double* betas, int n,
                       double theta) {
  const int H = C.H;
  store_coefs(alphas, betas, n);
  C.theta_cheby = theta;
  cheby_residual();
  if (C.prec == ORC_PREC_JAC_BLOCK) block_solve(C.r, C.ztmp);
#pragma omp parallel for schedule(static)
  for (int row = H; row < H + C.y_max; row++)
    for (int col = H; col < H + C.x_max; col++) {
      const long c = IDX(col, row);
      if (C.prec == ORC_PREC_JAC_BLOCK)
        C.p[c] = C.ztmp[c] / theta;
      else if (C.prec == ORC_PREC_JAC_DIAG)
        C.p[c] = (C.Mi[c] * C.r[c]) / theta;
      else
        C.p[c] = C.r[c] / theta;
    }
  cheby_calc_u();
}

/* CloverChunk::tea_leaf_cheby_iterate_kernel (tea_leaf_kernel_ocl.cpp:131-138):
 * cheby_solve_calc_p (tea_leaf_cheby_cl.cl:78-145) with coefficient index
 * step-1, then cheby_solve_calc_u.  In the block-Jacobi case the reference
 * keeps M^-1 r in local memory only and leaves z untouched. */
void oracle_cheby_iterate(int step) {
  const int H = C.H;
  const int s = step - 1;
  const double a = C.ch_alphas[s], b = C.ch_betas[s];
  cheby_residual();
  if (C.prec == ORC_PREC_JAC_BLOCK) block_solve(C.r, C.ztmp);
#pragma omp parallel for schedule(static)
  for (int row = H; row < H + C.y_max; row++)
    for (int col = H; col < H + C.x_max; col++) {
      const long c = IDX(col, row);
      if (C.prec == ORC_PREC_JAC_BLOCK)
        C.p[c] = coef_update(a, C.p[c], b, C.ztmp[c]);
      else if (C.prec == ORC_PREC_JAC_DIAG)
        C.p[c] = coef_update(a, C.p[c], b * C.Mi[c], C.r[c]);
      else
        C.p[c] = coef_update(a, C.p[c], b, C.r[c]);
    }
  cheby_calc_u();
}

/* CloverChunk::ppcg_init, tea_leaf_kernel_ocl.cpp:327-344 */
void oracle_ppcg_init(const double* alphas, const double* betas, double theta,
                      int n) {
  store_coefs(alphas, betas, n);
  C.theta_ppcg = theta;
}

/* tea_leaf_ppcg_solve_init_sd, tea_leaf_ppcg_cl.cl:4-60 (z is not written) */
void oracle_ppcg_init_sd(void) {
  const int H = C.H;
  const double theta = C.theta_ppcg;
  double* zl = C.ztmp;
  if (C.prec == ORC_PREC_JAC_BLOCK) block_solve(C.r, zl);
#pragma omp parallel for schedule(static)
  for (int row = H; row < H + C.y_max; row++)
    for (int col = H; col < H + C.x_max; col++) {
      const long c = IDX(col, row);
      if (C.prec == ORC_PREC_JAC_BLOCK)
        C.sd[c] = zl[c] / theta;
      else if (C.prec == ORC_PREC_JAC_DIAG)
        C.sd[c] = C.r[c] * C.Mi[c] / theta;
      else
        C.sd[c] = C.r[c] / theta;
    }
}

/* One inner step on a single chunk: CloverChunk::tea_leaf_ppcg_inner_kernel
 * (tea_leaf_kernel_ocl.cpp:352-411) with every neighbour an external face,
 * i.e. both kernels over the interior: ppcg_solve_update_r then
 * ppcg_solve_calc_sd with coefficient index step-1
 * (tea_leaf_ppcg_cl.cl:62-155). */
void oracle_ppcg_inner(int step) {
  const int H = C.H;
  const int s = step - 1;
  const double a = C.ch_alphas[s], b = C.ch_betas[s];
#pragma omp parallel for schedule(static)
  for (int row = H; row < H + C.y_max; row++)
    for (int col = H; col < H + C.x_max; col++) {
      const long c = IDX(col, row);
      C.u[c] = C.u[c] + C.sd[c];
    }
  /* r -= A sd reads sd only, so a second sweep is equivalent */
#pragma omp parallel for schedule(static)
  for (int row = H; row < H + C.y_max; row++)
    for (int col = H; col < H + C.x_max; col++) {
      const long c = IDX(col, row);
      C.r[c] = b_minus_smvp(C.sd, c, C.r[c]);
    }
  double* zl = C.ztmp;
  if (C.prec == ORC_PREC_JAC_BLOCK) block_solve(C.r, zl);
#pragma omp parallel for schedule(static)
  for (int row = H; row < H + C.y_max; row++)
    for (int col = H; col < H + C.x_max; col++) {
      const long c = IDX(col, row);
      if (C.prec == ORC_PREC_JAC_BLOCK)
        C.sd[c] = coef_update(a, C.sd[c], b, zl[c]);
      else if (C.prec == ORC_PREC_JAC_DIAG)
        C.sd[c] = coef_update(a, C.sd[c], b * C.r[c], C.Mi[c]);
      else
        C.sd[c] = coef_update(a, C.sd[c], b, C.r[c]);
    }
}

/* CloverChunk::tea_leaf_jacobi_solve_kernel (tea_leaf_kernel_ocl.cpp:222-229):
 * jacobi_copy_u into Mi (the reference reuses vector_Mi as un,
 * ocl_kernels.cpp:576-585), then jacobi_solve (tea_leaf_jacobi_cl.cl:15-42). */
void oracle_jacobi_solve(double* error) {
  const int H = C.H;
  double* un = C.Mi;
#pragma omp parallel for schedule(static)
  for (int row = H; row < H + C.y_max; row++)
    for (int col = H; col < H + C.x_max; col++) un[IDX(col, row)] = C.u[IDX(col, row)];
#pragma omp parallel for schedule(static)
  for (int row = H; row < H + C.y_max; row++)
    for (int col = H; col < H + C.x_max; col++) {
      const long c = IDX(col, row);
      const long xs = C.xs;
      C.u[c] = (C.u0[c] + C.Kx[c + 1] * un[c + 1] + C.Kx[c] * un[c - 1] +
                C.Ky[c + xs] * un[c + xs] + C.Ky[c] * un[c - xs]) /
               (1.0 + (C.Kx[c] + C.Kx[c + 1]) + (C.Ky[c] + C.Ky[c + xs]));
      SCR(0, col, row) = fabs(C.u[c] - un[c]);
    }
  *error = reduce_scratch(0);
}

/* tea_leaf_finalise, tea_leaf_common_cl.cl:4-15 */
void oracle_finalise_kernel(void) {
  const int H = C.H;
#pragma omp parallel for schedule(static)
  for (int row = H; row < H + C.y_max; row++)
    for (int col = H; col < H + C.x_max; col++) {
      const long c = IDX(col, row);
      C.energy1[c] = C.u[c] / C.density[c];
    }
}

/* field_summary, field_summary_cl.cl:3-43, bound to volume, density,
 * energy1, u (ocl_kernels.cpp:466-469) */
void oracle_field_summary(double* vol, double* mass, double* ie, double* temp) {
  const int H = C.H;
#pragma omp parallel for schedule(static)
  for (int row = H; row < H + C.y_max; row++)
    for (int col = H; col < H + C.x_max; col++) {
      const long c = IDX(col, row);
      const double cell_vol = C.volume[c];
      const double cell_mass = cell_vol * C.density[c];
      SCR(0, col, row) = cell_vol;
      SCR(1, col, row) = cell_mass;
      SCR(2, col, row) = cell_mass * C.energy1[c];
      SCR(3, col, row) = cell_mass * C.u[c];
    }
  *vol = reduce_scratch(0);
  *mass = reduce_scratch(1);
  *ie = reduce_scratch(2);
  *temp = reduce_scratch(3);
}

/* update_halo_{bottom,top,left,right} (update_halo_cl.cl:3-69) in the order
 * of CloverChunk::update_array (update_halo_kernel_ocl.cpp:14-46), for
 * density, energy0, energy1 (update_halo_kernel_ocl.cpp:48-62); every face is
 * external on a single chunk. */
static void reflect(double* a, int depth) {
  const int H = C.H;
  for (int row = H - depth; row < H; row++)
    for (int col = H - depth; col <= C.x_max + H - 1 + depth; col++) {
      const int src = 1 + (H - row - 1) * 2;
      a[IDX(col, row)] = 1 * a[IDX(col, row + src)];
    }
  for (int row = H - depth; row < H; row++)
    for (int col = H - depth; col <= C.x_max + H - 1 + depth; col++) {
      const int src = C.y_max;
      const int dst = C.y_max + (H - row - 1) * 2 + 1;
      a[IDX(col, row + dst)] = a[IDX(col, row + src)];
    }
  for (int row = H - depth; row <= C.y_max + H - 1 + depth; row++)
    for (int col = H - depth; col < H; col++) {
      const int src = 1 + (H - col - 1) * 2;
      a[IDX(col, row)] = 1 * a[IDX(col + src, row)];
    }
  for (int row = H - depth; row <= C.y_max + H - 1 + depth; row++)
    for (int col = H - depth; col < H; col++) {
      const int src = C.x_max;
      const int dst = C.x_max + (H - col - 1) * 2 + 1;
      a[IDX(col + dst, row)] = a[IDX(col + src, row)];
    }
}

void oracle_update_halo(const int* fields, int depth) {
  if (depth < 1 || depth > C.H) return;
  if (fields[ORC_FIELD_DENSITY - 1] == 1) reflect(C.density, depth);
  if (fields[ORC_FIELD_ENERGY0 - 1] == 1) reflect(C.energy0, depth);
  if (fields[ORC_FIELD_ENERGY1 - 1] == 1) reflect(C.energy1, depth);
}

/* ------------------------------------------------------------------------ */
/* Field access                                                             */
/* ------------------------------------------------------------------------ */

static double* field_ptr(int f) {
  switch (f) {
    case ORC_FIELD_DENSITY: return C.density;
    case ORC_FIELD_ENERGY0: return C.energy0;
    case ORC_FIELD_ENERGY1: return C.energy1;
    case ORC_FIELD_U: return C.u;
    case ORC_FIELD_P: return C.p;
    case ORC_FIELD_SD: return C.sd;
    case ORC_FIELD_R: return C.r;
    case ORC_FIELD_U0: return C.u0;
    case ORC_FIELD_W: return C.w;
    case ORC_FIELD_Z: return C.z;
    case ORC_FIELD_MI: return C.Mi;
    case ORC_FIELD_KX: return C.Kx;
    case ORC_FIELD_KY: return C.Ky;
    case ORC_FIELD_CP: return C.cp;
    case ORC_FIELD_BFP: return C.bfp;
    case ORC_FIELD_VOLUME: return C.volume;
    default: return NULL;
  }
}

int oracle_read_field(int f, double* out) {
  double* a = field_ptr(f);
  if (!a || !C_ready) return -1;
  for (int y = 0; y < C.y_max; y++)
    for (int x = 0; x < C.x_max; x++)
      out[(long)y * C.x_max + x] = a[IDX(x + C.H, y + C.H)];
  return 0;
}

int oracle_write_field(int f, const double* in) {
  double* a = field_ptr(f);
  if (!a || !C_ready) return -1;
  for (int y = 0; y < C.y_max; y++)
    for (int x = 0; x < C.x_max; x++)
      a[IDX(x + C.H, y + C.H)] = in[(long)y * C.x_max + x];
  return 0;
}

int oracle_read_field_padded(int f, double* out, long n) {
  double* a = field_ptr(f);
  const long need = (long)C.xs * C.ys;
  if (!a || !C_ready || n < need) return -1;
  memcpy(out, a, sizeof(double) * (size_t)need);
  return 0;
}

int oracle_write_field_padded(int f, const double* in, long n) {
  double* a = field_ptr(f);
  const long need = (long)C.xs * C.ys;
  if (!a || !C_ready || n < need) return -1;
  memcpy(a, in, sizeof(double) * (size_t)need);
  return 0;
}

int oracle_num_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

/* ------------------------------------------------------------------------ */
/* Mixed precision: FP32 inner CG in FP64 defect correction                 */
/* ------------------------------------------------------------------------ */
/*
 * Restates tea_gb300_mixed_solve of the CUDA library (the oracle has no
 * reference counterpart for it: it is an addition to the reference's
 * solvers).  FP32 parts use float with fmaf where the CUDA code uses
 * __fmaf_rn; FP64 parts use the fused form; FP32 dot products accumulate
 * per lane as an exact float pair (acc_pair), FP64 ones with fma.
 */
typedef struct {
  float *Kx, *Ky, *D, *Mi, *d, *r, *p, *w, *z, *sd;
} OrcMix;
static OrcMix M;
static long M_n = 0;

static void mix_free(void) {
  float** f[10] = {&M.Kx, &M.Ky, &M.D, &M.Mi, &M.d, &M.r, &M.p, &M.w, &M.z, &M.sd};
  for (int i = 0; i < 10; i++) {
    free(*f[i]);
    *f[i] = NULL;
  }
  M_n = 0;
}

static int mix_alloc(void) {
  if (M_n == C.n2 && M.Kx) return 0;
  mix_free();
  float** f[10] = {&M.Kx, &M.Ky, &M.D, &M.Mi, &M.d, &M.r, &M.p, &M.w, &M.z, &M.sd};
  for (int i = 0; i < 10; i++) {
    *f[i] = (float*)calloc((size_t)C.n2, sizeof(float));
    if (!*f[i]) return -1;
  }
  M_n = C.n2;
  return 0;
}

static inline double smvp64_fused(const double* x, long c) {
  const long xs = C.xs;
  const double D = (1.0 + (C.Ky[c + xs] + C.Ky[c]) + (C.Kx[c + 1] + C.Kx[c]));
  const double t1 = fma(C.Ky[c], x[c - xs], C.Ky[c + xs] * x[c + xs]);
  const double t2 = fma(C.Kx[c], x[c - 1], C.Kx[c + 1] * x[c + 1]);
  return fma(D, x[c], -t1) - t2;
}

static inline float smvp32(const float* x, long c) {
  const long xs = C.xs;
  const float kyn = M.Ky[c + xs], kyc = M.Ky[c];
  const float kxe = M.Kx[c + 1], kxc = M.Kx[c];
  const float t1 = fmaf(kyc, x[c - xs], kyn * x[c + xs]);
  const float t2 = fmaf(kxc, x[c - 1], kxe * x[c + 1]);
  return fmaf(M.D[c], x[c], -t1) - t2;
}

/* r64 = u0 - A u; r32 = (float)r64; z = Mi r32; p = z; d = 0.
 * out[0] = r64.r64, out[1] = r32.z */
static void mix_residual(double* out) {
  const int H = C.H;
#pragma omp parallel for schedule(static)
  for (int row = H; row < H + C.y_max; row++)
    for (int col = H; col < H + C.x_max; col++) {
      const long c = IDX(col, row);
      const double r64 = C.u0[c] - smvp64_fused(C.u, c);
      C.r[c] = r64;
      const float r32 = (float)r64;
      const float z = M.Mi[c] * r32;
      M.r[c] = r32;
      M.p[c] = z;
      M.d[c] = 0.0f;
      DOT(0, col, row, r64, r64);
      DOT(1, col, row, (double)r32, (double)z);
    }
  out[0] = reduce_pairs(C.scratch[0], C.scratchb[0], C.x_max, C.y_max, 1);
  out[1] = reduce_pairs(C.scratch[1], C.scratchb[1], C.x_max, C.y_max,
                        LANE_FLOAT_PAIR);
}

/* ---- FP32 inner iterations (the kernels of tea_mixed.cu) ---- */

/* w = A p; returns p.w */
static double mix_calc_w(void) {
  const int H = C.H;
#pragma omp parallel for schedule(static)
  for (int row = H; row < H + C.y_max; row++)
    for (int col = H; col < H + C.x_max; col++) {
      const long c = IDX(col, row);
      const float wv = smvp32(M.p, c);
      M.w[c] = wv;
      DOT(0, col, row, (double)M.p[c], (double)wv);
    }
  return reduce_pairs(C.scratch[0], C.scratchb[0], C.x_max, C.y_max, LANE_FLOAT_PAIR);
}

/* CG: d += a p; r -= a w; returns r.(Mi r) */
static double mix_cg_ur(float af) {
  const int H = C.H;
#pragma omp parallel for schedule(static)
  for (int row = H; row < H + C.y_max; row++)
    for (int col = H; col < H + C.x_max; col++) {
      const long c = IDX(col, row);
      M.d[c] = fmaf(af, M.p[c], M.d[c]);
      const float rv = fmaf(-af, M.w[c], M.r[c]);
      M.r[c] = rv;
      const float zv = M.Mi[c] * rv;
      DOT(0, col, row, (double)rv, (double)zv);
    }
  return reduce_pairs(C.scratch[0], C.scratchb[0], C.x_max, C.y_max, LANE_FLOAT_PAIR);
}

/* CG: p = Mi r + b p */
static void mix_cg_p(float bf) {
  const int H = C.H;
#pragma omp parallel for schedule(static)
  for (int row = H; row < H + C.y_max; row++)
    for (int col = H; col < H + C.x_max; col++) {
      const long c = IDX(col, row);
      M.p[c] = fmaf(bf, M.p[c], M.Mi[c] * M.r[c]);
    }
}

/* PPCG: d += a p; r -= a w; z = Mi r */
static void mix_ppcg_ur(float af) {
  const int H = C.H;
#pragma omp parallel for schedule(static)
  for (int row = H; row < H + C.y_max; row++)
    for (int col = H; col < H + C.x_max; col++) {
      const long c = IDX(col, row);
      const float dv = fmaf(af, M.p[c], M.d[c]);
      const float rv = fmaf(-af, M.w[c], M.r[c]);
      M.d[c] = dv;
      M.r[c] = rv;
      M.z[c] = M.Mi[c] * rv;
    }
}

/* PPCG inner steps: sd = (Mi r)/theta, then per step d += sd, r -= A sd,
 * sd = a sd + b (Mi r) */
static void mix_ppcg_inner(float tf, const float* ca, const float* cb, int steps) {
  const int H = C.H;
#pragma omp parallel for schedule(static)
  for (int row = H; row < H + C.y_max; row++)
    for (int col = H; col < H + C.x_max; col++) {
      const long c = IDX(col, row);
      M.sd[c] = (M.Mi[c] * M.r[c]) / tf;
    }
  for (int k = 0; k < steps; k++) {
#pragma omp parallel for schedule(static)
    for (int row = H; row < H + C.y_max; row++)
      for (int col = H; col < H + C.x_max; col++) {
        const long c = IDX(col, row);
        const float dv = M.d[c] + M.sd[c];
        const float rv = M.r[c] - smvp32(M.sd, c);
        M.d[c] = dv;
        M.r[c] = rv;
      }
#pragma omp parallel for schedule(static)
    for (int row = H; row < H + C.y_max; row++)
      for (int col = H; col < H + C.x_max; col++) {
        const long c = IDX(col, row);
        M.sd[c] = fmaf(ca[k], M.sd[c], cb[k] * (M.Mi[c] * M.r[c]));
      }
  }
}

/* PPCG: r.z with the kept z */
static double mix_ppcg_rz(void) {
  const int H = C.H;
#pragma omp parallel for schedule(static)
  for (int row = H; row < H + C.y_max; row++)
    for (int col = H; col < H + C.x_max; col++) {
      const long c = IDX(col, row);
      DOT(0, col, row, (double)M.r[c], (double)M.z[c]);
    }
  return reduce_pairs(C.scratch[0], C.scratchb[0], C.x_max, C.y_max, LANE_FLOAT_PAIR);
}

/* PPCG: p = z + b p */
static void mix_ppcg_p(float bf) {
  const int H = C.H;
#pragma omp parallel for schedule(static)
  for (int row = H; row < H + C.y_max; row++)
    for (int col = H; col < H + C.x_max; col++) {
      const long c = IDX(col, row);
      M.p[c] = fmaf(bf, M.p[c], M.z[c]);
    }
}

/* The device loop state of one inner solve (MixState in tea_mixed.cu). */
typedef struct {
  double rro, rrn, eps2;
  int n, max_iters, stop, done;
  double* alphas; /* CG alpha/beta by iteration number, or NULL */
  double* betas;
} MixLoop;

/* CG iterations until the loop stops (k_mix_calc_w/ur/p with the scalar
 * step of k_mix_calc_ur's last block) */
static void mix_run_cg(MixLoop* L) {
  for (;;) {
    const double pw = mix_calc_w();
    const double alpha = L->rro / pw;
    const double rrn = mix_cg_ur((float)alpha);
    const double beta = rrn / L->rro;
    if (L->alphas) {
      L->alphas[L->n] = alpha;
      L->betas[L->n] = beta;
    }
    L->rrn = rrn;
    L->rro = rrn;
    L->done = L->n;
    L->stop = (rrn <= L->eps2 || L->n >= L->max_iters);
    mix_cg_p((float)beta);
    if (L->stop) return;
    L->n++;
  }
}

/* PPCG iterations until the loop stops (tea_mixed.cu enqueue_ppcg) */
static void mix_run_ppcg(MixLoop* L, float tf, const float* ca, const float* cb,
                         int steps) {
  for (;;) {
    const double pw = mix_calc_w();
    const double alpha = L->rro / pw;
    mix_ppcg_ur((float)alpha);
    mix_ppcg_inner(tf, ca, cb, steps);
    const double rrn = mix_ppcg_rz();
    const double beta = rrn / L->rro;
    L->rrn = rrn;
    L->rro = rrn;
    L->done = L->n;
    L->stop = (rrn <= L->eps2 || L->n >= L->max_iters);
    mix_ppcg_p((float)beta);
    if (L->stop) return;
    L->n++;
  }
}

static int mixed_solve(double tol, double inner_tol, int max_outer, int max_inner,
                       int ppcg, int presteps, int inner_steps,
                       oracle_mixed_info* info) {
  const int H = C.H;
  memset(info, 0, sizeof(*info));
  if (!C_ready || mix_alloc() != 0) return -1;
  /* FP32 copies of the operator */
  for (long i = 0; i < C.n2; i++) {
    M.Kx[i] = (float)C.Kx[i];
    M.Ky[i] = (float)C.Ky[i];
  }
  for (int row = H; row < H + C.y_max; row++)
    for (int col = H; col < H + C.x_max; col++) {
      const long c = IDX(col, row);
      const double D =
          (1.0 + (C.Ky[c + C.xs] + C.Ky[c]) + (C.Kx[c + 1] + C.Kx[c]));
      M.D[c] = (float)D;
      M.Mi[c] = (float)(1.0 / D);
    }
  double* ab = NULL;
  float *ca = NULL, *cb = NULL;
  float tf = 0.0f;
  int have_eigs = 0, eig_failed = 0;
  if (ppcg) {
    ab = (double*)calloc(2 * (size_t)(presteps + 2), sizeof(double));
    ca = (float*)calloc((size_t)inner_steps, sizeof(float));
    cb = (float*)calloc((size_t)inner_steps, sizeof(float));
  }
  double res[2];
  mix_residual(res);
  const double rr_first = res[0];
  info->initial_residual = sqrt(rr_first);
  int outer = 0;
  long long inner_total = 0, cheby_total = 0;
  while (!(sqrt(res[0]) <= tol * sqrt(rr_first)) && outer < max_outer) {
    MixLoop L;
    memset(&L, 0, sizeof(L));
    L.rro = res[1];
    const double need = 0.25 * tol * sqrt(rr_first) / sqrt(res[0]);
    const double itol = need > inner_tol ? (need < 0.5 ? need : 0.5) : inner_tol;
    L.eps2 = itol * itol * res[1];
    L.n = 1;
    L.max_iters = max_inner;
    int use_ppcg = ppcg && have_eigs;
    if (ppcg && !have_eigs && !eig_failed) {
      /* CG presteps, then the eigenvalue range (tea_solve.f90:175-210) */
      L.max_iters = presteps < max_inner ? presteps : max_inner;
      L.alphas = ab;
      L.betas = ab + presteps + 2;
      mix_run_cg(&L);
      const int converged = L.rrn <= L.eps2;
      L.alphas = L.betas = NULL;
      if (!converged && L.done < max_inner) {
        const int n = L.done;
        double eigmin = 0.0, eigmax = 0.0;
        if (oracle_calc_eigenvalues(ab + 1, ab + presteps + 3, n, &eigmin, &eigmax) != 0) {
          eig_failed = 1;
        } else {
          double* cha = (double*)calloc((size_t)inner_steps, sizeof(double));
          double* chb = (double*)calloc((size_t)inner_steps, sizeof(double));
          double theta = 0.0;
          oracle_calc_ch_coefs(cha, chb, eigmin * 0.95, eigmax * 1.05, &theta, inner_steps);
          for (int k = 0; k < inner_steps; k++) {
            ca[k] = (float)cha[k];
            cb[k] = (float)chb[k];
          }
          tf = (float)theta;
          free(cha);
          free(chb);
          have_eigs = 1;
          use_ppcg = 1;
        }
        L.stop = 0;
        L.n = n + 1;
        L.max_iters = max_inner;
        const int pre = L.done;
        if (use_ppcg) {
          mix_run_ppcg(&L, tf, ca, cb, inner_steps);
          cheby_total += (long long)(L.done - pre) * inner_steps;
        } else {
          mix_run_cg(&L);
        }
      }
    } else if (use_ppcg) {
      mix_run_ppcg(&L, tf, ca, cb, inner_steps);
      cheby_total += (long long)L.done * inner_steps;
    } else {
      mix_run_cg(&L);
    }
    inner_total += L.done;
#pragma omp parallel for schedule(static)
    for (int row = H; row < H + C.y_max; row++)
      for (int col = H; col < H + C.x_max; col++) {
        const long c = IDX(col, row);
        C.u[c] = C.u[c] + (double)M.d[c];
      }
    outer++;
    mix_residual(res);
  }
  free(ab);
  free(ca);
  free(cb);
  info->outer_iterations = outer;
  info->inner_iterations = inner_total;
  info->ppcg_inner_steps = cheby_total;
  info->final_residual = sqrt(res[0]);
  info->relative_residual = sqrt(res[0]) / sqrt(rr_first);
  return 0;
}

int oracle_mixed_solve(double tol, double inner_tol, int max_outer,
                       int max_inner, oracle_mixed_info* info) {
  return mixed_solve(tol, inner_tol, max_outer, max_inner, 0, 0, 0, info);
}

int oracle_mixed_solve_ppcg(double tol, double inner_tol, int max_outer, int max_inner,
                            int presteps, int inner_steps, oracle_mixed_info* info) {
  if (presteps < 1 || inner_steps < 1) return -1;
  return mixed_solve(tol, inner_tol, max_outer, max_inner, 1, presteps, inner_steps, info);
}
