/*
 * TEST INFRASTRUCTURE ONLY -- CPU oracle for the TeaLeaf implicit solve.
 *
 * This library is the parity checker for the CUDA implementation in
 * tealeaf_opencl_gb300/.  Only tests/, __graft_entry__.smoke() and the
 * cpu_baseline / --impl reference legs of bench.py may load it.  It is never
 * part of the product path.
 *
 * It restates, in plain C with OpenMP, the arithmetic of the reference's
 * OpenCL kernels (UK-MAC/TeaLeaf_OpenCL kernel_files, the .cl files) and the control
 * flow of its Fortran driver (tea_solve.f90, tea_leaf_*.f90, diffuse.f90,
 * start.f90, read_input.f90, parse.f90, field_summary.f90), using the
 * reference's own padded field layout (row stride x_max+2*halo, x fastest,
 * ocl_buffers.cpp:36-69, macros_cl.cl:20-22).
 *
 * Parity pin: the oracle reproduces the reference's built-in test problems
 * (field_summary.f90:88-106) within the reference's own 0.001 % criterion;
 * see tests/test_oracle_golden.py.
 *
 * Summation order: every global sum (dot products, field summary) uses the
 * fixed tile order documented in oracle_reduce() below, which is the same
 * order the CUDA kernels use, so the two implementations agree bit-for-bit.
 * The reference's own order (a 128-lane work-group tree followed by staged
 * reduction kernels, macros_cl.cl:47-64, reduction_cl.cl:39-149) is a
 * different fixed order; the test problems pass with either.
 */
#ifndef TEA_ORACLE_H
#define TEA_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* Enumerations, same values as kernel_files/definitions.hpp:45-56 and
 * data.f90. */
#define ORC_PREC_NONE 1
#define ORC_PREC_JAC_DIAG 2
#define ORC_PREC_JAC_BLOCK 3

#define ORC_SOLVER_JACOBI 1
#define ORC_SOLVER_CG 2
#define ORC_SOLVER_CHEBYSHEV 3
#define ORC_SOLVER_PPCG 4

#define ORC_COEF_CONDUCTIVITY 1
#define ORC_COEF_RECIP_CONDUCTIVITY 2

#define ORC_FIELD_DENSITY 1
#define ORC_FIELD_ENERGY0 2
#define ORC_FIELD_ENERGY1 3
#define ORC_FIELD_U 4
#define ORC_FIELD_P 5
#define ORC_FIELD_SD 6
#define ORC_FIELD_R 7
/* fields beyond the reference's FIELD_* set, for read-back in tests */
#define ORC_FIELD_U0 8
#define ORC_FIELD_W 9
#define ORC_FIELD_Z 10
#define ORC_FIELD_MI 11
#define ORC_FIELD_KX 12
#define ORC_FIELD_KY 13
#define ORC_FIELD_CP 14
#define ORC_FIELD_BFP 15
#define ORC_FIELD_VOLUME 16

/* ---- chunk lifecycle (mirrors initialise_ocl_, ocl_init.cpp:11) ---- */
int oracle_initialise(int x_max, int y_max, int halo_depth, int solver,
                      int preconditioner);
void oracle_finalise(void);

/* ---- setup kernels (initialise_chunk_cl.cl, generate_chunk_cl.cl,
 *      set_field_cl.cl) ---- */
void oracle_initialise_chunk(double xmin, double ymin, double dx, double dy);
void oracle_generate_chunk(int number_of_states, const double* density,
                           const double* energy, const double* xmin,
                           const double* xmax, const double* ymin,
                           const double* ymax, const double* radius,
                           const int* geometry);
void oracle_set_field(void);

/* ---- solver entry points (tea_leaf_kernel_ocl.cpp) ---- */
void oracle_common_init(int coefficient, double dt, double* rx, double* ry,
                        const int* zero_boundary, int reflective);
void oracle_calc_residual(void);
void oracle_calc_2norm(int which, double* norm);
void oracle_cg_init(double* rro);
void oracle_cg_calc_w(double* pw);
void oracle_cg_calc_ur(double alpha, double* rrn);
void oracle_cg_calc_p(double beta);
void oracle_cheby_init(const double* alphas, const double* betas, int n,
                       double theta);
void oracle_cheby_iterate(int step);
void oracle_ppcg_init(const double* alphas, const double* betas, double theta,
                      int n);
void oracle_ppcg_init_sd(void);
void oracle_ppcg_inner(int step);
void oracle_jacobi_solve(double* error);
void oracle_finalise_kernel(void);
void oracle_field_summary(double* vol, double* mass, double* ie, double* temp);
void oracle_update_halo(const int* fields, int depth);

/* ---- field access for tests: interior only, x fastest ---- */
int oracle_read_field(int field, double* out);
int oracle_write_field(int field, const double* in);
/* whole padded array in the reference layout (stride x_max+2H) */
int oracle_read_field_padded(int field, double* out, long n);
int oracle_write_field_padded(int field, const double* in, long n);

/* the canonical fixed-order sum of an interior-sized array */
double oracle_reduce(const double* contrib, int x_max, int y_max);
/* the same order for a dot product: lanes accumulate acc + a*b
 * (fused: fma(a, b, acc)) */
double oracle_reduce_pairs(const double* a, const double* b, int x_max,
                           int y_max, int fused);

/* arithmetic form: 0 exact reference expressions, 1 fused multiply-adds */
void oracle_set_arithmetic(int fused);
int oracle_get_arithmetic(void);
int oracle_reduction_rows(int x_max, int y_max);

/* ---- mixed precision (restates tea_gb300_mixed_solve) ---- */
typedef struct {
  int outer_iterations;
  long long inner_iterations;
  double initial_residual;
  double final_residual;
  double relative_residual;
  long long ppcg_inner_steps;
} oracle_mixed_info;
int oracle_mixed_solve(double tol, double inner_tol, int max_outer,
                       int max_inner, oracle_mixed_info* info);
/* restates tea_gb300_mixed_solve_ppcg: FP32 PPCG inner solver */
int oracle_mixed_solve_ppcg(double tol, double inner_tol, int max_outer, int max_inner,
                            int presteps, int inner_steps, oracle_mixed_info* info);
/* eigenvalue range from CG alphas/betas and Chebyshev coefficients
 * (tea_leaf_cheby.f90:96-172; tea_oracle_driver.c) */
int oracle_calc_eigenvalues(const double* cg_alphas, const double* cg_betas, int nsteps,
                            double* eigmin, double* eigmax);
void oracle_calc_ch_coefs(double* alphas, double* betas, double eigmin, double eigmax,
                          double* theta, int n);

/* ---- whole runs (restatement of the Fortran driver) ---- */
typedef struct {
  int n_summaries;      /* field_summary calls made */
  int n_steps;          /* timesteps run */
  double summary[64][6]; /* step, vol, mass, mass/vol, ie, temp (last 64) */
  int iterations[1024];  /* outer iteration count per step (first 1024) */
  int inner_iterations[1024];
  double conduction_error[1024];
  double exact_error[1024];
  double final_temp;
  double solve_seconds;   /* wall time inside tea_leaf calls */
  double step_seconds[1024]; /* wall time of each tea_leaf call */
  long long total_outer_iterations;
  long long total_inner_iterations;
  int qa_passed;          /* 1 pass, 0 fail, -1 not a test problem */
  double qa_diff;
  int outer_corrections[1024]; /* mixed precision: FP64 corrections */
  double relative_residual[1024];
  int switch_iteration[1024]; /* iteration of the switch to Chebyshev/PPCG, 0 if none */
} oracle_result;

/* Parse tea.in text and run it.  log_path may be NULL; otherwise a tea.out
 * style log is written there.  max_solver_iters > 0 caps tl_max_iters (for
 * bounded timing samples).  max_after_switch > 0 ends a Chebyshev or PPCG
 * step after that many iterations from the switch on (the iteration of the
 * switch included), so a bounded sample still reaches the switch and then
 * runs the polynomial solver.  Returns 0 on success. */
int oracle_run_deck(const char* deck_text, const char* log_path,
                    int max_solver_iters, int max_after_switch,
                    oracle_result* result, char* err, int errlen);

int oracle_num_threads(void);

#ifdef __cplusplus
}
#endif
#endif
