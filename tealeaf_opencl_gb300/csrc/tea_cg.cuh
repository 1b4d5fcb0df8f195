// CG tile bodies shared by the single-chunk kernels (tea_kernels.cu) and
// the batched kernels (tea_batch.cu): one lane's column x of one tile,
// rows y0 .. y0+TH-1, with the arithmetic of the reference kernels.
#pragma once

#include "tea_device.cuh"

namespace tea {

// Every tile body below works in groups of 4 rows and, within a group,
// issues all of its loads before its first store.  The fields are reached
// through the members of Dev, which the compiler must assume may alias, so
// a load written after a store cannot move above it; loading the group
// first keeps 4 rows of loads in flight instead of one.  The arithmetic and
// the order of the per-lane sums are those of the row-by-row form.

// w = A p and the lane's share of p.w (tea_leaf_cg_cl.cl:45-69)
template <int TH, int F, bool CG = false>
__device__ __forceinline__ void cg_w_tile(const Dev& d, int x, int y0, bool xin,
                                          double* acc) {
#pragma unroll 1
  for (int g = y0; g < y0 + TH; g += 4) {
    const long long c0 = cidx(d, x, g);
    double pv[4], wv[4];
#pragma unroll
    for (int j = 0; j < 4; j++) {
      pv[j] = 0.0;
      wv[j] = 0.0;
      if (xin && g + j < d.y_max) {
        wv[j] = smvp<F, CG>(d, d.p, c0 + j * d.S);
        pv[j] = ldv<CG>(d.p + c0 + j * d.S);
      }
    }
#pragma unroll
    for (int j = 0; j < 4; j++)
      if (xin && g + j < d.y_max) d.w[c0 + j * d.S] = wv[j];
#pragma unroll
    for (int j = 0; j < 4; j++) acc[0] = accum<F>(acc[0], pv[j], wv[j]);
  }
}

// cg_w_tile for the single-chunk calc_w kernel, with the fields reached
// through restrict-qualified pointers: p and the coefficients are only
// read and w only written, so the compiler may issue a group's loads before
// the previous group's stores and keep more loads in flight.  Same
// arithmetic and per-lane summation order; with 4 blocks per SM (64
// registers) 192.2 -> 174.4 us at 4096^2 on non-zero fields.
template <int TH, int F>
__device__ __forceinline__ void cg_w_tile_r(const Dev& d, int x, int y0, bool xin,
                                            double* acc) {
  const double* __restrict__ p = d.p;
  const double* __restrict__ kx = d.Kx;
  const double* __restrict__ ky = d.Ky;
  const double* __restrict__ dg = d.diag;
  double* __restrict__ w = d.w;
  const long long S = d.S;
#pragma unroll 1
  for (int g = y0; g < y0 + TH; g += 4) {
    const long long c0 = cidx(d, x, g);
    double pv[4], wv[4];
#pragma unroll
    for (int j = 0; j < 4; j++) {
      pv[j] = 0.0;
      wv[j] = 0.0;
      if (xin && g + j < d.y_max) {
        const long long c = c0 + j * S;
        pv[j] = p[c];
        wv[j] = smvp_v<F>(__ldg(dg + c), __ldg(ky + c + S), __ldg(ky + c), __ldg(kx + c + 1),
                          __ldg(kx + c), pv[j], p[c + S], p[c - S], p[c + 1], p[c - 1]);
      }
    }
#pragma unroll
    for (int j = 0; j < 4; j++)
      if (xin && g + j < d.y_max) w[c0 + j * S] = wv[j];
#pragma unroll
    for (int j = 0; j < 4; j++) acc[0] = accum<F>(acc[0], pv[j], wv[j]);
  }
}

// u += alpha p; r -= alpha w (tea_leaf_cg_cl.cl:88-89) on loaded values
template <int F>
__device__ __forceinline__ void ur_values(double alpha, double& u, double p,
                                          double& r, double w) {
  if (F) {
    u = __fma_rn(alpha, p, u);
    r = __fma_rn(-alpha, w, r);
  } else {
    u = u + alpha * p;
    r = r - alpha * w;
  }
}

// u += alpha p, r -= alpha w, z = M^-1 r and the lane's share of r.z (and
// of r.r when NV == 2; no sum when NV == 0), tea_leaf_cg_cl.cl:73-137.
// With SD it also starts PPCG's inner steps, sd = M^-1 r / theta
// (tea_leaf_ppcg_cl.cl:4-60), from the z it has just formed: the same
// values tea_leaf_ppcg_solve_init_sd computes from the stored r.
template <int TH, int F, int NV, bool CG = false, bool SD = false>
__device__ __forceinline__ void cg_ur_tile(const Dev& d, int x, int y0, bool xin,
                                           double* acc, double alpha,
                                           const DivConst& theta = DivConst{}) {
#pragma unroll 1
  for (int g = y0; g < y0 + TH; g += 4) {
    const long long c0 = cidx(d, x, g);
    bool in[4];
    double uv[4], pv[4], rv[4], wv[4], mv[4];
#pragma unroll
    for (int j = 0; j < 4; j++) {
      in[j] = xin && g + j < d.y_max;
      uv[j] = pv[j] = rv[j] = wv[j] = mv[j] = 0.0;
      if (in[j]) {
        const long long c = c0 + j * d.S;
        uv[j] = ldv<CG>(d.u + c);
        pv[j] = ldv<CG>(d.p + c);
        rv[j] = ldv<CG>(d.r + c);
        wv[j] = ldv<CG>(d.w + c);
        if (d.prec == PREC_JAC_DIAG) mv[j] = d.Mi[c];
      }
    }
#pragma unroll
    for (int j = 0; j < 4; j++) {
      if (in[j]) {
        ur_values<F>(alpha, uv[j], pv[j], rv[j], wv[j]);
        d.u[c0 + j * d.S] = uv[j];
        d.r[c0 + j * d.S] = rv[j];
      }
    }
    double zv[4] = {0.0, 0.0, 0.0, 0.0};
    if (d.prec == PREC_JAC_BLOCK) {
      // one 4-row strip of the block-Jacobi solve (strips start at rows
      // that are multiples of 4)
      if (in[0]) strip_solve<F>(d, c0, strip_rows(d, g), rv, zv);
    } else if (d.prec == PREC_JAC_DIAG) {
#pragma unroll
      for (int j = 0; j < 4; j++) zv[j] = rv[j] * mv[j];
    }
#pragma unroll
    for (int j = 0; j < 4; j++) {
      double av = 0.0, bv = 0.0;
      if (in[j]) {
        if (d.prec != PREC_NONE) d.z[c0 + j * d.S] = zv[j];
        if (SD) d.sd[c0 + j * d.S] = emu_ddiv(d.prec != PREC_NONE ? zv[j] : rv[j], theta);
        av = rv[j];
        bv = d.prec != PREC_NONE ? zv[j] : rv[j];
      }
      if (NV > 0) acc[0] = accum<F>(acc[0], av, bv);
      if (NV > 1) acc[NV - 1] = accum<F>(acc[NV - 1], av, av);
    }
  }
}

// cg_ur_tile for the single-chunk kernels (CG calc_ur, PPCG's calc_ur +
// init_sd), with the fields reached through restrict-qualified pointers and
// the strip coefficients loaded with u, p, r and w, before the stores of u
// and r, so that more loads are in flight.  The strip solve reads exactly
// the rows strip_solve reads (a strip may end in the halo row).  Same
// arithmetic and per-lane summation order; with 4 blocks per SM (64
// registers), on non-zero fields at 4096^2 (block Jacobi): calc_ur 246.4 ->
// 210.9 us, calc_ur + init_sd 223.7 -> 215.0 us.
template <int TH, int F, int NV, bool SD = false>
__device__ __forceinline__ void cg_ur_tile_r(const Dev& d, int x, int y0, bool xin,
                                             double* acc, double alpha,
                                             const DivConst& theta = DivConst{}) {
  double* __restrict__ u = d.u;
  const double* __restrict__ p = d.p;
  double* __restrict__ r = d.r;
  const double* __restrict__ w = d.w;
  double* __restrict__ z = d.z;
  double* __restrict__ sd = d.sd;
  const long long S = d.S;
  // the lane's sums and the z / sd stores of one group of 4 rows
  auto finish = [&](long long c0, const bool in[4], const double rv[4], const double zv[4],
                    bool prec) {
#pragma unroll
    for (int j = 0; j < 4; j++) {
      double av = 0.0, bv = 0.0;
      if (in[j]) {
        if (prec) z[c0 + j * S] = zv[j];
        if (SD) sd[c0 + j * S] = emu_ddiv(prec ? zv[j] : rv[j], theta);
        av = rv[j];
        bv = prec ? zv[j] : rv[j];
      }
      if (NV > 0) acc[0] = accum<F>(acc[0], av, bv);
      if (NV > 1) acc[NV - 1] = accum<F>(acc[NV - 1], av, av);
    }
  };
  if (d.prec == PREC_JAC_BLOCK) {
    const double* __restrict__ bfp = d.bfp;
    const double* __restrict__ ky = d.Ky;
    const double* __restrict__ cp = d.cp;
#pragma unroll 1
    for (int g = y0; g < y0 + TH; g += 4) {
      const long long c0 = cidx(d, x, g);
      const int upper = xin && g < d.y_max ? strip_rows(d, g) : 0;
      bool in[4];
      double uv[4], rv[4], bl[4], kl[4], cl[4];
#pragma unroll
      for (int j = 0; j < 4; j++) {
        in[j] = xin && g + j < d.y_max;
        uv[j] = rv[j] = bl[j] = kl[j] = cl[j] = 0.0;
        const long long c = c0 + j * S;
        if (in[j]) {
          uv[j] = u[c];
          rv[j] = r[c];
          ur_values<F>(alpha, uv[j], p[c], rv[j], w[c]);
        }
        if (j < upper) {
          if (F || j > 0) bl[j] = __ldg(bfp + c);
          if (j > 0) kl[j] = __ldg(ky + c);
          if (j + 1 < upper) cl[j] = __ldg(cp + c);
        }
      }
      const double d0 = !F && upper > 0 ? __ldg(d.diag + c0) : 0.0;
#pragma unroll
      for (int j = 0; j < 4; j++)
        if (in[j]) {
          u[c0 + j * S] = uv[j];
          r[c0 + j * S] = rv[j];
        }
      double zv[4] = {0.0, 0.0, 0.0, 0.0};
      if (upper == 4)
        strip_solve_v<F, false, true>(4, rv, bl, kl, cl, d0, zv);
      else if (upper > 0)
        strip_solve_v<F, false>(upper, rv, bl, kl, cl, d0, zv);
      finish(c0, in, rv, zv, true);
    }
  } else {
    const bool dia = d.prec == PREC_JAC_DIAG;
    const double* __restrict__ mi = d.Mi;
#pragma unroll 1
    for (int g = y0; g < y0 + TH; g += 4) {
      const long long c0 = cidx(d, x, g);
      bool in[4];
      double uv[4], rv[4], zv[4];
#pragma unroll
      for (int j = 0; j < 4; j++) {
        in[j] = xin && g + j < d.y_max;
        uv[j] = rv[j] = zv[j] = 0.0;
        const long long c = c0 + j * S;
        if (in[j]) {
          uv[j] = u[c];
          rv[j] = r[c];
          ur_values<F>(alpha, uv[j], p[c], rv[j], w[c]);
          if (dia) zv[j] = rv[j] * mi[c];
        }
      }
#pragma unroll
      for (int j = 0; j < 4; j++)
        if (in[j]) {
          u[c0 + j * S] = uv[j];
          r[c0 + j * S] = rv[j];
        }
      finish(c0, in, rv, zv, dia);
    }
  }
}

// p = z + beta p, or r + beta p without a preconditioner
// (tea_leaf_cg_cl.cl:141-160)
template <int TH, int F, bool CG = false>
__device__ __forceinline__ void cg_p_tile(const Dev& d, int x, int y0, bool xin,
                                          double beta) {
  if (!xin) return;
  const double* src = d.prec != PREC_NONE ? d.z : d.r;
#pragma unroll 1
  for (int g = y0; g < y0 + TH; g += 4) {
    const long long c0 = cidx(d, x, g);
    double sv[4], pv[4];
#pragma unroll
    for (int j = 0; j < 4; j++) {
      sv[j] = pv[j] = 0.0;
      if (g + j < d.y_max) {
        sv[j] = ldv<CG>(src + c0 + j * d.S);
        pv[j] = ldv<CG>(d.p + c0 + j * d.S);
      }
    }
#pragma unroll
    for (int j = 0; j < 4; j++)
      if (g + j < d.y_max)
        d.p[c0 + j * d.S] = F ? __fma_rn(beta, pv[j], sv[j]) : sv[j] + beta * pv[j];
  }
}

// The host steps of one CG iteration (tea_solve.f90:282-330) after calc_ur,
// on the device: beta = rrn/rro, rro = rrn, error = sqrt(rrn), and the exit
// test (on sqrt(r.z), or on ||r||_2 when NV == 2).  result[] holds the
// reduced sums; run by one thread.
template <int NV>
__device__ __forceinline__ void cg_scalar_step(ResState* st, double alpha,
                                               const double* result) {
  const double rrn = result[0];
  const int n = st->n;
  if (st->check) {
    // breakdown (the caller asked for the check; the reference runs on)
    const double pw = st->pw;
    const int b = !(pw > 0.0) || isinf(pw) ? 1 : (isfinite(rrn) ? 0 : 2);
    if (b) {
      st->breakdown = b;
      st->breakdown_n = n;
      st->stop = 1;
      st->p_pending = 0;
      return;
    }
  }
  const double beta = rrn / st->rro;
  if (st->alphas) {
    st->alphas[n] = alpha;
    st->betas[n] = beta;
  }
  st->alpha = alpha;
  st->beta = beta;
  st->rrn = rrn;
  st->rro = rrn;
  const double err = sqrt(rrn);
  st->error = err;
  st->p_pending = 1;
  const bool done = NV > 1 ? sqrt(result[NV - 1]) < st->eps_target
                           : fabs(err) < st->eps_target;
  if (NV > 1) st->rr_true = result[NV - 1];
  if (done) {
    st->converged = 1;
    st->stop = 1;
  } else if (n >= st->loop_max) {
    st->stop = 1;
  } else {
    st->n = n + 1;
  }
}

}  // namespace tea
