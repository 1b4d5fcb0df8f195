/*
 * TEST INFRASTRUCTURE ONLY -- CPU oracle, driver half.
 *
 * Restates the reference's Fortran driver on top of the oracle kernels:
 *   deck parsing       read_input.f90:24-329, parse.f90:99-381
 *   problem setup      start.f90:24-115, initialise_chunk.f90, generate_chunk.f90
 *   timestep loop      diffuse.f90:23-163, timestep.f90, calc_dt.f90
 *   implicit solve     tea_solve.f90:37-521 (tea_leaf, PPCG inner steps,
 *                      Chebyshev first step)
 *   eigenvalue maths   tea_leaf_cheby.f90:44-172 (tqli, eigenvalues, coefs),
 *                      tea_leaf_ppcg.f90:62-73
 *   field summary      field_summary.f90:27-110 (print and test-problem check)
 * Single chunk, single tile: every chunk face is external.
 */
#define _POSIX_C_SOURCE 200809L
#include <ctype.h>
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include "tea_oracle.h"

#define MAX_STATES 256

typedef struct {
  double xmin, ymin, xmax, ymax;
  int x_cells, y_cells;
  double end_time;
  int end_step;
  int summary_frequency;
  double dtinit;
  int max_iters;
  double eps;
  int coefficient;
  int tl_ch_cg_presteps;
  double tl_ch_cg_epslim;
  int tl_check_result;
  int preconditioner;
  int reflective_boundary;
  int ppcg_inner_steps;
  int solver;
  int halo_depth;
  int test_problem;
  int verbose;
  int fused; /* tl_arithmetic: 0 exact, 1 fused (default), 2 chain */
  int mixed; /* tl_mixed_precision */
  double mixed_inner_eps;
  int mixed_max_outer;
  int number_of_states;
  double s_density[MAX_STATES], s_energy[MAX_STATES];
  double s_xmin[MAX_STATES], s_xmax[MAX_STATES], s_ymin[MAX_STATES],
      s_ymax[MAX_STATES], s_radius[MAX_STATES];
  int s_geometry[MAX_STATES];
  int s_defined[MAX_STATES];
} Deck;

/* ------------------------------------------------------------------------ */
/* deck parsing                                                             */
/* ------------------------------------------------------------------------ */

typedef struct {
  char** lines;
  int n;
} Lines;

/* parse_getline: keep the *tea ... *endtea block, drop comments after '!'
 * and ';', lower-case, and turn '=' and ',' into blanks. */
static Lines deck_lines(const char* text) {
  Lines L = {NULL, 0};
  int cap = 0;
  int inside = 0;
  const char* p = text;
  while (*p) {
    const char* e = strchr(p, '\n');
    size_t len = e ? (size_t)(e - p) : strlen(p);
    char* l = (char*)malloc(len + 1);
    memcpy(l, p, len);
    l[len] = 0;
    for (size_t i = 0; i < len; i++) {
      unsigned char ch = (unsigned char)l[i];
      if (ch < 32 || ch > 128) l[i] = ' ';
    }
    char* s = strchr(l, '!');
    if (s) *s = 0;
    s = strchr(l, ';');
    if (s) *s = 0;
    for (char* q = l; *q; q++) {
      *q = (char)tolower((unsigned char)*q);
      if (*q == '=' || *q == ',') *q = ' ';
    }
    char* t = l;
    while (*t == ' ') t++;
    if (strncmp(t, "*endtea", 7) == 0) {
      inside = 0;
    } else if (strncmp(t, "*tea", 4) == 0) {
      inside = 1;
    } else if (inside && *t) {
      if (L.n == cap) {
        cap = cap ? 2 * cap : 64;
        L.lines = (char**)realloc(L.lines, sizeof(char*) * (size_t)cap);
      }
      L.lines[L.n++] = strdup(t);
    }
    free(l);
    p = e ? e + 1 : p + len;
  }
  return L;
}

static void free_lines(Lines* L) {
  for (int i = 0; i < L->n; i++) free(L->lines[i]);
  free(L->lines);
}

typedef struct {
  char* words[128];
  int n, pos;
} Words;

static void split_words(char* line, Words* W) {
  W->n = 0;
  W->pos = 0;
  char* save = NULL;
  for (char* t = strtok_r(line, " \t", &save); t && W->n < 128;
       t = strtok_r(NULL, " \t", &save))
    W->words[W->n++] = t;
}

static const char* next_word(Words* W) {
  return W->pos < W->n ? W->words[W->pos++] : "";
}

/* parse_getival: READ(FMT="(I7)") */
static int getival(const char* w, int* ok) {
  char buf[8];
  strncpy(buf, w, 7);
  buf[7] = 0;
  char* end = NULL;
  long v = strtol(buf, &end, 10);
  *ok = (end != buf);
  return (int)v;
}

/* parse_getrval: integers get ".0" appended, then a formatted real read */
static double getrval(const char* w, int* ok) {
  char* end = NULL;
  double v = strtod(w, &end);
  *ok = (end != w);
  return v;
}

static int perr(char* err, int errlen, const char* fmt, ...) {
  if (err && errlen > 0) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(err, (size_t)errlen, fmt, ap);
    va_end(ap);
  }
  return -1;
}

static int parse_deck(const char* text, Deck* D, char* err, int errlen) {
  memset(D, 0, sizeof(*D));
  /* defaults, read_input.f90:38-91 (single-precision literals kept) */
  D->xmin = 0.0;
  D->ymin = 0.0;
  D->xmax = 100.0;
  D->ymax = 100.0;
  D->x_cells = 10;
  D->y_cells = 10;
  D->end_time = 10.0;
  D->end_step = 640000; /* g_ibig */
  D->summary_frequency = 10;
  D->dtinit = (double)0.1f;
  D->max_iters = 1000;
  D->eps = (double)1.0e-10f;
  D->coefficient = ORC_COEF_CONDUCTIVITY;
  D->tl_ch_cg_presteps = 25;
  D->tl_ch_cg_epslim = 1.0;
  D->tl_check_result = 0;
  D->preconditioner = ORC_PREC_NONE;
  D->reflective_boundary = 0;
  D->ppcg_inner_steps = -1;
  D->solver = ORC_SOLVER_JACOBI;
  D->halo_depth = 1;
  D->fused = 1;
  D->mixed = 0;
  D->mixed_inner_eps = 1e-4;
  D->mixed_max_outer = 50;

  Lines L = deck_lines(text);
  int state_max = 0, ok = 1;
  for (int i = 0; i < L.n; i++) {
    char* line = strdup(L.lines[i]);
    Words W;
    split_words(line, &W);
    for (;;) {
      const char* w = next_word(&W);
      if (!*w) break;
      if (!strcmp(w, "state")) {
        int s = getival(next_word(&W), &ok);
        if (s > state_max) state_max = s;
        break;
      }
    }
    free(line);
  }
  if (state_max < 1) {
    free_lines(&L);
    return perr(err, errlen, "read_input: No states defined.");
  }
  if (state_max > MAX_STATES) {
    free_lines(&L);
    return perr(err, errlen, "read_input: too many states (%d)", state_max);
  }
  D->number_of_states = state_max;

  for (int i = 0; i < L.n; i++) {
    char* line = strdup(L.lines[i]);
    Words W;
    split_words(line, &W);
    for (;;) {
      const char* w = next_word(&W);
      if (!*w) break;
#define RVAL(dst) dst = getrval(next_word(&W), &ok)
#define IVAL(dst) dst = getival(next_word(&W), &ok)
      if (!strcmp(w, "initial_timestep")) RVAL(D->dtinit);
      else if (!strcmp(w, "end_time")) RVAL(D->end_time);
      else if (!strcmp(w, "end_step")) IVAL(D->end_step);
      else if (!strcmp(w, "xmin")) RVAL(D->xmin);
      else if (!strcmp(w, "xmax")) RVAL(D->xmax);
      else if (!strcmp(w, "ymin")) RVAL(D->ymin);
      else if (!strcmp(w, "ymax")) RVAL(D->ymax);
      else if (!strcmp(w, "x_cells")) IVAL(D->x_cells);
      else if (!strcmp(w, "y_cells")) IVAL(D->y_cells);
      else if (!strcmp(w, "visit_frequency")) { int v; IVAL(v); (void)v; }
      else if (!strcmp(w, "summary_frequency")) IVAL(D->summary_frequency);
      else if (!strcmp(w, "tl_ch_cg_presteps")) IVAL(D->tl_ch_cg_presteps);
      else if (!strcmp(w, "tl_ppcg_inner_steps")) IVAL(D->ppcg_inner_steps);
      else if (!strcmp(w, "tl_ch_cg_epslim")) RVAL(D->tl_ch_cg_epslim);
      else if (!strcmp(w, "tl_check_result")) D->tl_check_result = 1;
      else if (!strcmp(w, "tl_preconditioner_type")) {
        for (;;) {
          const char* v = next_word(&W);
          if (!*v) break;
          if (!strcmp(v, "none")) D->preconditioner = ORC_PREC_NONE;
          else if (!strcmp(v, "jac_diag")) D->preconditioner = ORC_PREC_JAC_DIAG;
          else if (!strcmp(v, "jac_block")) D->preconditioner = ORC_PREC_JAC_BLOCK;
          else {
            free(line);
            free_lines(&L);
            return perr(err, errlen,
                        "read_input: Invalid preconditioner type specified: %s", v);
          }
        }
      }
      else if (!strcmp(w, "verbose_on")) D->verbose = 1;
      else if (!strcmp(w, "tl_mixed_precision")) D->mixed = 1;
      else if (!strcmp(w, "tl_mixed_inner_eps")) RVAL(D->mixed_inner_eps);
      else if (!strcmp(w, "tl_mixed_max_outer")) IVAL(D->mixed_max_outer);
      else if (!strcmp(w, "tl_arithmetic")) {
        /* not a reference key: which arithmetic form to use */
        const char* v = next_word(&W);
        if (!strcmp(v, "exact")) D->fused = 0;
        else if (!strcmp(v, "fused")) D->fused = 1;
        else if (!strcmp(v, "chain")) D->fused = 2;
        else {
          free(line);
          free_lines(&L);
          return perr(err, errlen,
                      "read_input: tl_arithmetic must be exact, fused or chain");
        }
      }
      else if (!strcmp(w, "tl_use_jacobi")) D->solver = ORC_SOLVER_JACOBI;
      else if (!strcmp(w, "tl_use_cg")) D->solver = ORC_SOLVER_CG;
      else if (!strcmp(w, "tl_use_ppcg")) D->solver = ORC_SOLVER_PPCG;
      else if (!strcmp(w, "tl_use_chebyshev")) D->solver = ORC_SOLVER_CHEBYSHEV;
      else if (!strcmp(w, "reflective_boundary")) D->reflective_boundary = 1;
      else if (!strcmp(w, "halo_depth")) {
        IVAL(D->halo_depth);
        if (D->halo_depth < 1) {
          free(line);
          free_lines(&L);
          return perr(err, errlen, "read_input: Invalid halo exchange depth specified");
        }
      }
      else if (!strcmp(w, "tl_max_iters")) IVAL(D->max_iters);
      else if (!strcmp(w, "tl_eps")) RVAL(D->eps);
      else if (!strcmp(w, "tl_coefficient_density")) D->coefficient = ORC_COEF_CONDUCTIVITY;
      else if (!strcmp(w, "tl_coefficient_inverse_density"))
        D->coefficient = ORC_COEF_RECIP_CONDUCTIVITY;
      else if (!strcmp(w, "test_problem")) IVAL(D->test_problem);
      else if (!strcmp(w, "state")) {
        int s = getival(next_word(&W), &ok) - 1;
        if (s < 0 || s >= MAX_STATES || D->s_defined[s]) {
          free(line);
          free_lines(&L);
          return perr(err, errlen, "read_input: State defined twice.");
        }
        D->s_defined[s] = 1;
        for (;;) {
          const char* k = next_word(&W);
          if (!*k) break;
          if (!strcmp(k, "xmin")) RVAL(D->s_xmin[s]);
          else if (!strcmp(k, "ymin")) RVAL(D->s_ymin[s]);
          else if (!strcmp(k, "xmax")) RVAL(D->s_xmax[s]);
          else if (!strcmp(k, "ymax")) RVAL(D->s_ymax[s]);
          else if (!strcmp(k, "radius")) RVAL(D->s_radius[s]);
          else if (!strcmp(k, "density")) RVAL(D->s_density[s]);
          else if (!strcmp(k, "energy")) RVAL(D->s_energy[s]);
          else if (!strcmp(k, "geometry")) {
            const char* g = next_word(&W);
            if (!strcmp(g, "rectangle")) D->s_geometry[s] = 1;
            else if (!strcmp(g, "circle")) D->s_geometry[s] = 2;
            else if (!strcmp(g, "point")) D->s_geometry[s] = 3;
          }
        }
      }
      /* any other word (opencl_*, profiler_on, use_opencl_kernels, ...) is
       * ignored here, as in the reference's SELECT CASE */
#undef RVAL
#undef IVAL
      if (!ok) {
        free(line);
        free_lines(&L);
        return perr(err, errlen, "parse: conversion error after '%s'", w);
      }
    }
    free(line);
  }
  free_lines(&L);

  if (D->ppcg_inner_steps == -1) {
    const float cells = (float)(D->x_cells * D->y_cells);
    D->ppcg_inner_steps = 4 * (int)sqrtf(sqrtf(cells));
  }
  /* read_input.f90:314-327: shrink state boxes by a hundredth of a cell */
  const double dx = (D->xmax - D->xmin) / (double)(float)D->x_cells;
  const double dy = (D->ymax - D->ymin) / (double)(float)D->y_cells;
  for (int n = 1; n < D->number_of_states; n++) {
    D->s_xmin[n] = D->s_xmin[n] + (dx / 100.0);
    D->s_ymin[n] = D->s_ymin[n] + (dy / 100.0);
    D->s_xmax[n] = D->s_xmax[n] - (dx / 100.0);
    D->s_ymax[n] = D->s_ymax[n] - (dy / 100.0);
  }
  return 0;
}

/* ------------------------------------------------------------------------ */
/* eigenvalue and coefficient maths, tea_leaf_cheby.f90:44-172               */
/* ------------------------------------------------------------------------ */

/* tqli: QL with implicit shifts on a symmetric tridiagonal matrix; d holds
 * the diagonal, e the sub-diagonal shifted by one (e(1) unused). */
static int tqli(double* d, double* e, int n) {
  for (int i = 0; i < n - 1; i++) e[i] = e[i + 1];
  if (n > 0) e[n - 1] = 0.0;
  for (int l = 0; l < n; l++) {
    int iter = 0;
    for (;;) {
      int m;
      for (m = l; m < n - 1; m++) {
        const double dd = fabs(d[m]) + fabs(d[m + 1]);
        if (fabs(e[m]) + dd == dd) break;
      }
      if (m == l) break;
      if (iter == 30) return 1;
      iter++;
      double g = (d[l + 1] - d[l]) / (2.0 * e[l]);
      double r = sqrt(g * g + 1.0);
      g = d[m] - d[l] + e[l] / (g + copysign(fabs(r), g));
      double s = 1.0, c = 1.0, p = 0.0;
      int restart = 0;
      for (int i = m - 1; i >= l; i--) {
        double f = s * e[i];
        double b = c * e[i];
        r = sqrt(f * f + g * g);
        e[i + 1] = r;
        if (r == 0.0) {
          d[i + 1] = d[i + 1] - p;
          e[m] = 0.0;
          restart = 1;
          break;
        }
        s = f / r;
        c = g / r;
        g = d[i + 1] - p;
        r = (d[i] - g) * s + 2.0 * c * b;
        p = s * r;
        d[i + 1] = g + p;
        g = c * r - b;
      }
      if (restart) continue;
      d[l] = d[l] - p;
      e[l] = g;
      e[m] = 0.0;
    }
  }
  return 0;
}

/* tea_calc_eigenvalues: Lanczos tridiagonal from the CG alphas/betas. */
static int calc_eigenvalues(const double* cg_alphas, const double* cg_betas,
                            int nsteps, double* eigmin, double* eigmax) {
  if (nsteps < 1) return 1;
  double* diag = (double*)calloc((size_t)nsteps, sizeof(double));
  double* offdiag = (double*)calloc((size_t)nsteps, sizeof(double));
  for (int n = 0; n < nsteps; n++) {
    diag[n] = 1.0 / cg_alphas[n];
    if (n > 0) diag[n] = diag[n] + cg_betas[n - 1] / cg_alphas[n - 1];
    if (n < nsteps - 1) offdiag[n + 1] = sqrt(cg_betas[n]) / cg_alphas[n];
  }
  int info = tqli(diag, offdiag, nsteps);
  if (info == 0) {
    double lo = diag[0], hi = diag[0];
    for (int n = 1; n < nsteps; n++) {
      if (diag[n] < lo) lo = diag[n];
      if (diag[n] > hi) hi = diag[n];
    }
    *eigmin = lo;
    *eigmax = hi;
    if (lo < 0.0 || hi < 0.0) info = 1;
  }
  free(diag);
  free(offdiag);
  return info;
}

/* tea_calc_ch_coefs (and tea_calc_ls_coefs, which calls it) */
static void calc_ch_coefs(double* alphas, double* betas, double eigmin,
                          double eigmax, double* theta_out, int n) {
  const double theta = (eigmax + eigmin) / 2;
  const double delta = (eigmax - eigmin) / 2;
  const double sigma = theta / delta;
  double rho_old = 1.0 / sigma;
  for (int i = 0; i < n; i++) {
    const double rho_new = 1.0 / (2.0 * sigma - rho_old);
    alphas[i] = rho_new * rho_old;
    betas[i] = 2.0 * rho_new / delta;
    rho_old = rho_new;
  }
  *theta_out = theta;
}

int oracle_calc_eigenvalues(const double* cg_alphas, const double* cg_betas, int nsteps,
                            double* eigmin, double* eigmax) {
  return calc_eigenvalues(cg_alphas, cg_betas, nsteps, eigmin, eigmax);
}

void oracle_calc_ch_coefs(double* alphas, double* betas, double eigmin, double eigmax,
                          double* theta, int n) {
  calc_ch_coefs(alphas, betas, eigmin, eigmax, theta, n);
}

/* ------------------------------------------------------------------------ */
/* driver                                                                   */
/* ------------------------------------------------------------------------ */

typedef struct {
  Deck* D;
  FILE* log;
  oracle_result* R;
  int first;
  double eigmin, eigmax, theta, cn;
  int step;
  double time;
  double dt;
  int complete;
  int max_iters_cap;
  int max_after_switch; /* > 0: outer iterations allowed after the switch */
} Run;

static double now_s(void) {
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

static void logf_(Run* R, const char* fmt, ...) {
  if (!R->log) return;
  va_list ap;
  va_start(ap, fmt);
  vfprintf(R->log, fmt, ap);
  va_end(ap);
}

static void update_halo(Run* R, const int* fields, int depth) {
  /* tea_exchange is a no-op on one chunk (tea.f90:310); update_boundary
   * reflects only when reflective_boundary is set (update_halo.f90:47-68) */
  if (R->D->reflective_boundary) oracle_update_halo(fields, depth);
}

static void field_summary(Run* R) {
  double vol, mass, ie, temp;
  oracle_field_summary(&vol, &mass, &ie, &temp);
  logf_(R, "\n Time %.15g\n", R->time);
  logf_(R, " step:%7d%26.17E%26.17E%26.17E%26.17E%26.17E\n", R->step, vol, mass,
        mass / vol, ie, temp);
  oracle_result* res = R->R;
  const int k = res->n_summaries % 64;
  res->summary[k][0] = R->step;
  res->summary[k][1] = vol;
  res->summary[k][2] = mass;
  res->summary[k][3] = mass / vol;
  res->summary[k][4] = ie;
  res->summary[k][5] = temp;
  res->n_summaries++;
  res->final_temp = temp;
  if (R->complete && R->D->test_problem >= 1) {
    static const double golden[7] = {0.0,
                                     157.550841832793,
                                     116.067951160930,
                                     95.4865103390698,
                                     166.838315378708,
                                     116.482111627676,
                                     103.88639125996923};
    const int tp = R->D->test_problem;
    if (tp <= 6) {
      const double qa = fabs((100.0 * (temp / golden[tp])) - 100.0);
      res->qa_diff = qa;
      res->qa_passed = qa < 0.001;
      logf_(R, "Test problem %4d is within %16.7E%% of the expected solution\n",
            tp, qa);
      logf_(R, " %s\n", qa < 0.001 ? "This test is considered PASSED"
                                   : "This test is considered NOT PASSED");
    }
  }
}

/* tea_leaf_run_ppcg_inner_steps, tea_solve.f90:422-475, single chunk */
static void ppcg_inner_steps(Run* R, int inner, int H) {
  int fu[7] = {0, 0, 0, 1, 0, 0, 0};
  update_halo(R, fu, 1);
  oracle_ppcg_init_sd();
  for (int cur = 1; cur <= inner; cur += H) {
    int fsr[7] = {0, 0, 0, 0, 0, 1, 1};
    update_halo(R, fsr, H);
    int inner_step = cur;
    for (int bounds_extra = H - 1; bounds_extra >= 0; bounds_extra--) {
      oracle_ppcg_inner(inner_step);
      inner_step++;
      if (inner_step > inner) break;
    }
  }
}

/* SUBROUTINE tea_leaf, tea_solve.f90:37-420 */
static int tea_leaf(Run* R, int step_index) {
  Deck* D = R->D;
  const int max_iters = D->max_iters;
  const int use_cg = D->solver == ORC_SOLVER_CG;
  const int use_cheby = D->solver == ORC_SOLVER_CHEBYSHEV;
  const int use_ppcg = D->solver == ORC_SOLVER_PPCG;
  const int use_jacobi = D->solver == ORC_SOLVER_JACOBI;
  const int cap = R->max_iters_cap > 0 ? R->max_iters_cap : max_iters;
  int loop_max = cap < max_iters ? cap : max_iters;
  int switch_n = 0;

  double *cg_alphas = (double*)calloc((size_t)max_iters + 1, sizeof(double));
  double *cg_betas = (double*)calloc((size_t)max_iters + 1, sizeof(double));
  const int n_ch = (max_iters > D->ppcg_inner_steps ? max_iters : D->ppcg_inner_steps) + 2;
  double *ch_alphas = (double*)calloc((size_t)n_ch, sizeof(double));
  double *ch_betas = (double*)calloc((size_t)n_ch, sizeof(double));

  int cheby_calc_steps = 0, cg_calc_steps = 0, ppcg_inner_iters = 0;
  int ch_switch_check = 0, est_itc = 0, max_cheby_iters = 0;
  double rro = 0, pw = 0, rrn = 0, alpha, beta;
  double old_error, error = 0.0, exact_error = 0.0, initial_residual;

  int fields[7] = {0};
  fields[ORC_FIELD_ENERGY1 - 1] = 1;
  fields[ORC_FIELD_DENSITY - 1] = 1;
  update_halo(R, fields, D->halo_depth);

  const int zero_boundary[4] = {1, 1, 1, 1};
  double rx, ry;
  oracle_common_init(D->coefficient, R->dt, &rx, &ry, zero_boundary,
                     D->reflective_boundary);

  oracle_calc_residual();
  oracle_calc_2norm(1, &initial_residual);
  old_error = initial_residual;
  initial_residual = sqrt(initial_residual);

  if (D->mixed) {
    oracle_mixed_info mi;
    const int ppcg = D->solver == ORC_SOLVER_PPCG;
    if (ppcg)
      oracle_mixed_solve_ppcg(D->eps, D->mixed_inner_eps, D->mixed_max_outer,
                              D->max_iters, D->tl_ch_cg_presteps, D->ppcg_inner_steps, &mi);
    else
      oracle_mixed_solve(D->eps, D->mixed_inner_eps, D->mixed_max_outer,
                         D->max_iters, &mi);
    logf_(R, "Mixed precision: %d FP64 corrections, %lld FP32 %s iterations, "
             "relative FP64 residual %14.7E\n",
          mi.outer_iterations, mi.inner_iterations, ppcg ? "PPCG" : "CG",
          mi.relative_residual);
    oracle_finalise_kernel();
    int fe[7] = {0, 0, 1, 0, 0, 0, 0};
    update_halo(R, fe, 1);
    oracle_result* res = R->R;
    if (step_index < 1024) {
      res->iterations[step_index] = (int)mi.inner_iterations;
      res->inner_iterations[step_index] = (int)mi.ppcg_inner_steps;
      res->outer_corrections[step_index] = mi.outer_iterations;
      res->relative_residual[step_index] = mi.relative_residual;
      res->conduction_error[step_index] = mi.final_residual / initial_residual;
      res->exact_error[step_index] = NAN;
    }
    res->total_outer_iterations += mi.inner_iterations;
    free(cg_alphas); free(cg_betas); free(ch_alphas); free(ch_betas);
    return 0;
  }

  if (use_cg || use_cheby || use_ppcg) oracle_cg_init(&rro);

  int n;
  int exited = 0;
  for (n = 1; n <= loop_max; n++) {
    if (!ch_switch_check) {
      if (cheby_calc_steps > 0)
        ch_switch_check = 1;
      else if (!R->first && use_ppcg && n > 1)
        ch_switch_check = 1;
      else if (fabs(old_error) <= D->tl_ch_cg_epslim && n >= D->tl_ch_cg_presteps)
        ch_switch_check = 1;
      else
        ch_switch_check = 0;
    }

    if ((use_cheby || use_ppcg) && ch_switch_check) {
      if (cheby_calc_steps == 0) {
        max_cheby_iters = max_iters - n + 2;
        if (R->first) {
          int info = calc_eigenvalues(cg_alphas + 1, cg_betas + 1, n - 1,
                                      &R->eigmin, &R->eigmax);
          R->first = 0;
          if (info != 0) {
            free(cg_alphas); free(cg_betas); free(ch_alphas); free(ch_betas);
            return -3;
          }
          R->eigmin = R->eigmin * 0.95;
          R->eigmax = R->eigmax * 1.05;
        }
        if (use_cheby) {
          calc_ch_coefs(ch_alphas, ch_betas, R->eigmin, R->eigmax, &R->theta,
                        max_cheby_iters);
        } else {
          calc_ch_coefs(ch_alphas, ch_betas, R->eigmin, R->eigmax, &R->theta,
                        D->ppcg_inner_steps);
        }
        R->cn = R->eigmax / R->eigmin;
        switch_n = n;
        /* a bounded sample: this and max_after_switch - 1 more iterations */
        if (R->max_after_switch > 0 && n - 1 + R->max_after_switch < loop_max)
          loop_max = n - 1 + R->max_after_switch;
        logf_(R, "Switching after %3d CG its, error %15.7E\n", n, rro);
        logf_(R, "Eigen min%14.6E Eigen max%14.6E Condition number%14.6f Error%14.6E\n",
              R->eigmin, R->eigmax, R->cn, old_error);
      }
      if (use_cheby) {
        if (cheby_calc_steps == 0) {
          /* tea_leaf_cheby_first_step, tea_solve.f90:477-521; its 'error'
           * argument is the caller's old_error */
          double bb;
          oracle_calc_2norm(0, &bb);
          oracle_cheby_init(ch_alphas, ch_betas, max_cheby_iters, R->theta);
          oracle_cheby_iterate(1);
          oracle_calc_2norm(1, &old_error);
          const double it_alpha = D->eps * bb / (4.0 * old_error);
          const double gamm = (sqrt(R->cn) - 1.0) / (sqrt(R->cn) + 1.0);
          const double q = log(it_alpha) / (2.0 * log(gamm));
          est_itc = isfinite(q) ? (int)lround(q) : 0;
          logf_(R, "est itc\n%11d\n", est_itc);
          cheby_calc_steps = 1;
        } else {
          oracle_cheby_iterate(cheby_calc_steps);
          if (n >= est_itc && n % 10 == 0) oracle_calc_2norm(1, &error);
        }
      } else {
        if (cheby_calc_steps == 0)
          oracle_ppcg_init(ch_alphas, ch_betas, R->theta, D->ppcg_inner_steps);
        oracle_cg_calc_w(&pw);
        alpha = rro / pw;
        oracle_cg_calc_ur(alpha, &rrn);
        ppcg_inner_steps(R, D->ppcg_inner_steps, D->halo_depth);
        ppcg_inner_iters += D->ppcg_inner_steps;
        oracle_calc_2norm(2, &rrn);
        beta = rrn / rro;
        oracle_cg_calc_p(beta);
        error = rrn;
        rro = rrn;
      }
      cheby_calc_steps++;
    } else if (use_cg || use_cheby || use_ppcg) {
      cg_calc_steps++;
      oracle_cg_calc_w(&pw);
      alpha = rro / pw;
      cg_alphas[n] = alpha;
      oracle_cg_calc_ur(alpha, &rrn);
      beta = rrn / rro;
      cg_betas[n] = beta;
      oracle_cg_calc_p(beta);
      error = rrn;
      rro = rrn;
    } else if (use_jacobi) {
      oracle_jacobi_solve(&error);
    }

    int fu[7] = {0, 0, 0, 1, 0, 0, 0};
    update_halo(R, fu, 1);

    error = sqrt(error);
    if (D->verbose) logf_(R, " Residual %.17E\n", error);
    if (fabs(error) < D->eps * initial_residual) {
      exited = 1;
      break;
    }
    old_error = error;
  }
  const int performed = exited ? n : loop_max;

  if (D->tl_check_result) {
    int fu[7] = {0, 0, 0, 1, 0, 0, 0};
    update_halo(R, fu, 1);
    oracle_calc_residual();
    oracle_calc_2norm(1, &exact_error);
    exact_error = sqrt(exact_error);
  }

  logf_(R, "Conduction error %14.7E\n", error / initial_residual);
  if (D->tl_check_result)
    logf_(R, "EXACT error calculated as%14.7E\n", exact_error / initial_residual);
  logf_(R, "Iteration count %8d\n", (exited ? n : loop_max + 1) - 1);
  if (use_ppcg)
    logf_(R, "PPCG Iteration count%8d (Total %8d)\n", ppcg_inner_iters,
          ppcg_inner_iters + (exited ? n : loop_max + 1) - 1);

  oracle_finalise_kernel();
  int fe[7] = {0, 0, 1, 0, 0, 0, 0};
  update_halo(R, fe, 1);

  oracle_result* res = R->R;
  if (step_index < 1024) {
    res->iterations[step_index] = performed;
    res->inner_iterations[step_index] = ppcg_inner_iters;
    res->switch_iteration[step_index] = switch_n;
    res->conduction_error[step_index] = error / initial_residual;
    res->exact_error[step_index] =
        D->tl_check_result ? exact_error / initial_residual : NAN;
  }
  res->total_outer_iterations += performed;
  res->total_inner_iterations += ppcg_inner_iters;
  (void)cg_calc_steps;
  free(cg_alphas);
  free(cg_betas);
  free(ch_alphas);
  free(ch_betas);
  return 0;
}

int oracle_run_deck(const char* deck_text, const char* log_path,
                    int max_solver_iters, int max_after_switch,
                    oracle_result* result, char* err, int errlen) {
  Deck* D = (Deck*)malloc(sizeof(Deck));
  if (parse_deck(deck_text, D, err, errlen) != 0) {
    free(D);
    return -1;
  }
  memset(result, 0, sizeof(*result));
  result->qa_passed = -1;
  Run R;
  memset(&R, 0, sizeof(R));
  R.D = D;
  R.R = result;
  R.first = 1;
  R.max_iters_cap = max_solver_iters;
  R.max_after_switch = max_after_switch;
  if (log_path) R.log = fopen(log_path, "w");

  oracle_set_arithmetic(D->fused);
  /* start.f90:24-115 */
  R.time = 0.0;
  R.step = 0;
  R.dt = D->dtinit;
  if (oracle_initialise(D->x_cells, D->y_cells, D->halo_depth, D->solver,
                        D->preconditioner) != 0) {
    if (R.log) fclose(R.log);
    free(D);
    return perr(err, errlen, "oracle_initialise failed");
  }
  const double dx = (D->xmax - D->xmin) / (double)(float)D->x_cells;
  const double dy = (D->ymax - D->ymin) / (double)(float)D->y_cells;
  oracle_initialise_chunk(D->xmin + dx * 0.0, D->ymin + dy * 0.0, dx, dy);
  oracle_generate_chunk(D->number_of_states, D->s_density, D->s_energy,
                        D->s_xmin, D->s_xmax, D->s_ymin, D->s_ymax,
                        D->s_radius, D->s_geometry);
  int prime[7] = {1, 1, 1, 0, 0, 0, 0};
  update_halo(&R, prime, D->halo_depth);
  oracle_set_field();
  field_summary(&R);

  /* diffuse.f90:23-163 */
  const double g_small = (double)1.0e-16f;
  int rc = 0;
  for (;;) {
    R.step++;
    /* timestep / calc_dt: dt stays at dtinit */
    if (D->dtinit <= R.dt) R.dt = D->dtinit;
    logf_(&R, " Step %7d time %11.7f timestep  %9.2E\n", R.step, R.time, R.dt);
    const double t0 = now_s();
    rc = tea_leaf(&R, R.step - 1);
    const double t1 = now_s();
    result->solve_seconds += t1 - t0;
    if (R.step - 1 < 1024) result->step_seconds[R.step - 1] = t1 - t0;
    if (rc != 0) {
      perr(err, errlen, "tea_leaf: Error in calculating eigenvalues");
      break;
    }
    R.time = R.time + R.dt;
    if (D->summary_frequency != 0 && R.step % D->summary_frequency == 0)
      field_summary(&R);
    if (R.time + g_small > D->end_time || R.step >= D->end_step) {
      R.complete = 1;
      field_summary(&R);
      break;
    }
  }
  result->n_steps = R.step;
  if (R.log) fclose(R.log);
  free(D);
  return rc;
}
