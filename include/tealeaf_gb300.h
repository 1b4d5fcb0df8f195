/*
 * tealeaf_gb300.h -- C ABI of the GB300 (sm_103a) TeaLeaf implicit-solve
 * library, libtealeaf_gb300.so.
 *
 * Part 1 declares the entry points a TeaLeaf Fortran driver calls, with the
 * names, argument order and by-pointer convention of UK-MAC/TeaLeaf_OpenCL
 * (gfortran trailing underscore, implicit interfaces).  Each declaration
 * cites the reference definition it replaces.  The library keeps one
 * process-global chunk, as the reference does (ocl_init.cpp:9), so there is
 * no handle.  Calls that return a scalar return once the kernel that forms
 * it has written it to host memory; calls without an output may return
 * before the GPU finishes.  All work runs on one in-order CUDA stream, so
 * every call sees the effects of the calls before it.
 *
 * Errors: by default a fatal error prints a message and aborts the process,
 * like cloverDie (ocl_errors.cpp:175-194).  tea_gb300_set_abort_on_error(0)
 * switches to recording the error (tea_gb300_last_error) and returning, with
 * NaN written to any scalar output.
 *
 * Part 2 declares additions that have no counterpart in the reference:
 * configuration without a tea.in file, field access, error query, and the
 * whole-run driver.
 */
#ifndef TEALEAF_GB300_H
#define TEALEAF_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------------- */
/* Part 1: reference entry points                                          */
/* ---------------------------------------------------------------------- */

/* Enumerations (kernel_files/definitions.hpp:45-56, data.f90). */
#define TEA_PREC_NONE 1
#define TEA_PREC_JAC_DIAG 2
#define TEA_PREC_JAC_BLOCK 3
#define TEA_SOLVER_JACOBI 1
#define TEA_SOLVER_CG 2
#define TEA_SOLVER_CHEBYSHEV 3
#define TEA_SOLVER_PPCG 4
#define TEA_COEF_CONDUCTIVITY 1
#define TEA_COEF_RECIP_CONDUCTIVITY 2
#define TEA_EXTERNAL_FACE (-1)
/* field numbers of the fields[7] arrays (definitions.hpp:14-21) */
#define TEA_FIELD_DENSITY 1
#define TEA_FIELD_ENERGY0 2
#define TEA_FIELD_ENERGY1 3
#define TEA_FIELD_U 4
#define TEA_FIELD_P 5
#define TEA_FIELD_SD 6
#define TEA_FIELD_R 7

/* Replaces initialise_ocl_ (ocl_init.cpp:11-17).  Allocates the chunk of
 * (*x_max-*x_min+1) x (*y_max-*y_min+1) cells on the current CUDA device.
 * Halo depth, solver, preconditioner and profiler_on come from
 * tea_gb300_configure() if it was called, else from ./tea.in with the
 * reference's key matching (ocl_init.cpp:131-220, ocl_strings.cpp:7-37). */
void initialise_ocl_(int* x_min, int* x_max, int* y_min, int* y_max);

/* Replaces initialise_chunk_kernel_ocl_ (initialise_chunk_kernel_ocl.cpp:3-8):
 * cell/vertex coordinates and volume (initialise_chunk_cl.cl:3-68). */
void initialise_chunk_kernel_ocl_(double* d_xmin, double* d_ymin,
                                  double* d_dx, double* d_dy);

/* Replaces generate_chunk_kernel_ocl_ (generate_chunk_kernel_ocl.cpp:3-92):
 * paint states (rectangle/circle/point, last wins), then u = u0 =
 * energy0*density (generate_chunk_cl.cl:3-95). */
void generate_chunk_kernel_ocl_(const int* number_of_states,
                                const double* state_density,
                                const double* state_energy,
                                const double* state_xmin,
                                const double* state_xmax,
                                const double* state_ymin,
                                const double* state_ymax,
                                const double* state_radius,
                                const int* state_geometry, const int* g_rect,
                                const int* g_circ, const int* g_point);

/* Replaces set_field_kernel_ocl_ (set_field_kernel_ocl.cpp:3-7):
 * energy1 = energy0. */
void set_field_kernel_ocl_(void);

/* Replaces field_summary_kernel_ocl_ (field_summary_kernel_ocl.cpp:4-20):
 * sums of volume, mass, mass*energy1 and mass*u over the interior. */
void field_summary_kernel_ocl_(double* vol, double* mass, double* ie,
                               double* temp);

/* Replaces update_halo_kernel_ocl_ (update_halo_kernel_ocl.cpp:6-62):
 * reflective halo update of density, energy0, energy1 (fields[0..2] == 1)
 * to the given depth on every external face, as one fused launch. */
void update_halo_kernel_ocl_(const int* chunk_neighbours, const int* fields,
                             const int* depth);

/* Replaces tea_leaf_common_init_kernel_ocl_ (tea_leaf_kernel_ocl.cpp:233-239,
 * :254-289): rx = dt/dx^2, ry = dt/dy^2; face coefficients Kx, Ky; boundary
 * faces zeroed unless *reflective_boundary; u = u0 = energy1*density. */
void tea_leaf_common_init_kernel_ocl_(const int* coefficient, double* dt,
                                      double* rx, double* ry,
                                      int* zero_boundary,
                                      int* reflective_boundary);

/* Replaces tea_leaf_calc_residual_ocl_ (tea_leaf_kernel_ocl.cpp:248-252):
 * r = u0 - A u. */
void tea_leaf_calc_residual_ocl_(void);

/* Replaces tea_leaf_calc_2norm_kernel_ocl_ (tea_leaf_kernel_ocl.cpp:34-38,
 * :56-96): *norm_array 0 -> u0.u0, 1 -> r.r, 2 -> r.z (r.r without a
 * preconditioner). */
void tea_leaf_calc_2norm_kernel_ocl_(int* norm_array, double* norm);

/* Replaces tea_leaf_cg_init_kernel_ocl_ (tea_leaf_kernel_ocl.cpp:143-147,
 * :167-187): build the preconditioner, z = M^-1 r, p = z, *rro = r.p. */
void tea_leaf_cg_init_kernel_ocl_(double* rro);

/* Replaces tea_leaf_cg_calc_w_kernel_ocl_ (tea_leaf_kernel_ocl.cpp:149-153,
 * :189-194): w = A p, *pw = p.w. */
void tea_leaf_cg_calc_w_kernel_ocl_(double* pw);

/* Replaces tea_leaf_cg_calc_ur_kernel_ocl_ (tea_leaf_kernel_ocl.cpp:154-158,
 * :196-204): u += alpha p, r -= alpha w, z = M^-1 r, *rrn = r.z. */
void tea_leaf_cg_calc_ur_kernel_ocl_(double* alpha, double* rrn);

/* Replaces tea_leaf_cg_calc_p_kernel_ocl_ (tea_leaf_kernel_ocl.cpp:159-163,
 * :206-212): p = z + beta p. */
void tea_leaf_cg_calc_p_kernel_ocl_(double* beta);

/* Replaces tea_leaf_cheby_init_kernel_ocl_ (tea_leaf_kernel_ocl.cpp:42-48,
 * :98-129): keep *n_coefs Chebyshev coefficients, then w = A u,
 * r = u0 - w, p = M^-1 r / theta, u += p.  No size limit applies (the
 * reference is bounded by the device's constant-buffer size). */
void tea_leaf_cheby_init_kernel_ocl_(const double* ch_alphas,
                                     const double* ch_betas, int* n_coefs,
                                     const double* rx, const double* ry,
                                     const double* theta);

/* Replaces tea_leaf_cheby_iterate_kernel_ocl_ (tea_leaf_kernel_ocl.cpp:50-54,
 * :131-138): w = A u, r = u0 - w, p = alpha[s] p + beta[s] M^-1 r, u += p
 * with s = *cheby_calc_step - 1. */
void tea_leaf_cheby_iterate_kernel_ocl_(const int* cheby_calc_step);

/* Replaces tea_leaf_ppcg_init_ocl_ (tea_leaf_kernel_ocl.cpp:306-311,
 * :327-344): keep *n_inner_steps coefficients and theta. */
void tea_leaf_ppcg_init_ocl_(const double* ch_alphas, const double* ch_betas,
                             double* theta, int* n_inner_steps);

/* Replaces tea_leaf_ppcg_init_sd_kernel_ocl_ (tea_leaf_kernel_ocl.cpp:313-317,
 * :346-350): sd = M^-1 r / theta. */
void tea_leaf_ppcg_init_sd_kernel_ocl_(void);

/* Replaces tea_leaf_ppcg_inner_kernel_ocl_ (tea_leaf_kernel_ocl.cpp:319-325,
 * :352-411): u += sd, r -= A sd, sd = alpha[s] sd + beta[s] M^-1 r with
 * s = *inner_step - 1.  Single chunk: every neighbour must be
 * TEA_EXTERNAL_FACE, so *bounds_extra does not change the range. */
void tea_leaf_ppcg_inner_kernel_ocl_(int* inner_step, int* bounds_extra,
                                     const int* chunk_neighbours);

/* Replaces tea_leaf_jacobi_solve_kernel_ocl_ (tea_leaf_kernel_ocl.cpp:216-229):
 * un = u, one Jacobi sweep, *error = sum |u - un|. */
void tea_leaf_jacobi_solve_kernel_ocl_(double* error);

/* Replaces tea_leaf_common_finalise_kernel_ocl_
 * (tea_leaf_kernel_ocl.cpp:242-246, :292-296): energy1 = u / density. */
void tea_leaf_common_finalise_kernel_ocl_(void);

/* Replaces print_opencl_profiling_info_ (ocl_errors.cpp:196-232): per-kernel
 * call counts and times, collected when profiler_on is set. */
void print_opencl_profiling_info_(void);

/* Replace ocl_pack_buffers_ / ocl_unpack_buffers_ (ocl_pack.cpp:4-16).  MPI
 * halo exchange is out of scope for a single chunk: these accept only calls
 * that exchange no field and report an error otherwise. */
void ocl_pack_buffers_(int* fields, int* offsets, int* depth, int* face,
                       double* host_buffer);
void ocl_unpack_buffers_(int* fields, int* offsets, int* depth, int* face,
                         double* host_buffer);

/* ---------------------------------------------------------------------- */
/* Part 2: additions (no counterpart in the reference)                     */
/* ---------------------------------------------------------------------- */

/* Field numbers for tea_gb300_read_field / write_field: 1..7 as above, and */
#define TEA_FIELD_U0 8
#define TEA_FIELD_W 9
#define TEA_FIELD_Z 10
#define TEA_FIELD_MI 11
#define TEA_FIELD_KX 12
#define TEA_FIELD_KY 13
#define TEA_FIELD_CP 14
#define TEA_FIELD_BFP 15
#define TEA_FIELD_VOLUME 16

/* Sets what initialise_ocl_ would otherwise read from ./tea.in.  Returns 0,
 * or -1 for invalid values. */
int tea_gb300_configure(int halo_depth, int solver, int preconditioner,
                        int profiler_on);

/* Arithmetic form of the solver kernels.  1 (default): the reference's
 * expressions with each multiply feeding an add contracted into a fused
 * multiply-add, dot products accumulated with fused multiply-adds, and the
 * block-Jacobi strip's first division done with a stored reciprocal.
 * 0: every expression exactly as the reference writes it.  2: as 1, with
 * the 5-point operator (and b - A x) as one left-to-right chain of fused
 * multiply-adds, the fewest FP64 instructions.  Applies to the current
 * chunk and to chunks, batches and adjoint objects created later; set it
 * before tea_leaf_common_init_kernel_ocl_.  Returns 0, or -1 for another
 * value. */
int tea_gb300_set_arithmetic(int form);
/* How the driver's device-resident CG loop runs (TEA_DRIVER_RESIDENT):
 * 0 (default) and 1 replay batches of iterations, three kernels each, from a
 * CUDA graph; 2 runs the whole loop as one cooperative (persistent) launch
 * with grid barriers between its phases.  The results are identical; on
 * GB300 the persistent launch measured no faster at 512^2 to 4096^2.
 * Returns 0, or -1 for another value. */
int tea_gb300_set_resident_mode(int mode);
int tea_gb300_get_arithmetic(void);
/* With the block-Jacobi preconditioner, PPCG inner steps can run two at a
 * time in one pass whose inputs are staged in shared memory by TMA (1), or
 * one step per pass, update_r and then calc_sd on the r it has formed (0,
 * default: on GB300 measured faster, 586 against 818 us per two steps at
 * 4096^2).  With 1, tea_leaf_ppcg_inner_kernel_ocl_ holds back a step that a
 * next step may follow until that step (or any other call) arrives.
 * Results are identical either way.  Applies to the current chunk and later
 * ones.  Returns 0, or -1 for another value. */
int tea_gb300_set_inner_pairs(int on);
/* The persistent loop's grid barrier (mode 2 above): a block polls at most
 * spin_limit times (default 2^26, about 4 s) before it gives up, sets the
 * loop's error flag and returns; the call then fails with error 25.
 * extra_arrivals = 1 makes the barrier wait for one block more than the
 * grid has, so the wait always runs out: the test of that path uses it with
 * a short limit.  Use 2^26 and 0 for normal runs.  Returns 0 or -1. */
int tea_gb300_set_barrier_limits(long long spin_limit, int extra_arrivals);

/* 1 (default): fatal errors abort; 0: record and return. */
void tea_gb300_set_abort_on_error(int abort_on_error);

/* 0 if no error was recorded since the last call, else the code of the most
 * recent error; its message is copied to msg (may be NULL).  Clears the
 * recorded error. */
int tea_gb300_last_error(char* msg, int msg_len);

/* Frees the chunk's device memory. */
void tea_gb300_finalise(void);

/* Interior of a field (x fastest, y_max rows of x_max), host <-> device,
 * synchronous.  Return 0 or -1. */
int tea_gb300_read_field(int field, double* out);
int tea_gb300_write_field(int field, const double* in);
/* The padded field ((x_max+2H) x (y_max+2H), x fastest), as the reference
 * lays it out. */
int tea_gb300_read_field_padded(int field, double* out);
int tea_gb300_write_field_padded(int field, const double* in);

/* Rows per reduction tile for a grid (4 or 16); the summation order is
 * documented with the kernels. */
int tea_gb300_reduction_rows(int x_max, int y_max);

/* Number of kernel launches this library has made since load. */
long long tea_gb300_kernel_launches(void);

/* The cudaStream_t all work is queued on. */
void* tea_gb300_stream(void);

/* Chunk geometry: x_max, y_max, halo depth, row stride in doubles. */
int tea_gb300_chunk_info(int* x_max, int* y_max, int* halo, int* stride);

/* Timing on the library's stream: record CUDA event `slot` (0..15) now;
 * elapsed milliseconds between two recorded slots (waits for the second). */
int tea_gb300_event_record(int slot);
float tea_gb300_event_elapsed_ms(int start_slot, int end_slot);

/* Times every launch of the kernel with the given name (as listed by
 * print_opencl_profiling_info_), or of every kernel for "*", with CUDA
 * events on the library's stream, without serialising other work.
 * Selecting resets the totals; NULL or "" stops timing.  Read returns the
 * summed milliseconds and launch count of everything timed, or of one
 * kernel name. */
int tea_gb300_kernel_timer_select(const char* name);
int tea_gb300_kernel_timer_read(double* total_ms, long long* launches);
int tea_gb300_kernel_timer_read_name(const char* name, double* total_ms,
                                     long long* launches);

/* Measures the FP64 pipe: fused multiply-add instructions per second of the
 * current GPU (independent chains, all SMs).  Needs an initialised chunk. */
double tea_gb300_fp64_rate(void);

/* No counterpart in the reference; a check of this library's own
 * arithmetic.  The solver kernels compute some FP64 multiplies and
 * divisions from the operands' bit patterns with integer instructions,
 * correctly rounded.  This runs that device code on n operand pairs
 * (device pointers a, b) beside the GPU's own FP64 instruction and counts
 * the results whose bits differ (NaN counts as equal to NaN):
 *   TEA_EMU_MUL            a*b     against __dmul_rn
 *   TEA_EMU_DIV_INVARIANT  a/divisor, one divisor for all (b unused)
 *   TEA_EMU_DIV            a/b     against __ddiv_rn
 *   TEA_EMU_ADD            a+b     against __dadd_rn
 * *first_mismatch is the lowest index that differs, or -1.  Synchronous;
 * allocates two words of device memory.  Returns 0 or -1. */
#define TEA_EMU_MUL 0
#define TEA_EMU_DIV_INVARIANT 1
#define TEA_EMU_DIV 2
#define TEA_EMU_ADD 3
int tea_gb300_emu_check(int op, const double* a, const double* b, long long n,
                        double divisor, long long* mismatches, long long* first_mismatch);

/* No counterpart in the reference.  The dot product sum(a*b) over the
 * interior of two padded FP64 fields, for callers that cannot allocate GPU
 * memory (their device memory is held by another allocator, or they must
 * not call cudaMalloc on this path).  The caller passes device pointers to
 * the inputs and to one double for the result; nothing is allocated.  The
 * reduction's scratch is a fixed device array inside this library (512 KiB,
 * held on every GPU that loads the library until the process exits), which
 * holds 65536 partial sums, one per supertile of the fixed summation order:
 * ceil(ceil(x_max/32)/8) * ceil(y_max/TH) <= 65536, TH being
 * tea_gb300_reduction_rows(x_max, y_max).  16384 x 16384 cells fit; larger
 * interiors are rejected with an error.  Layout: element (col,row) at
 * a[row*stride + col], interior at [halo, halo+x_max) x [halo, halo+y_max).
 * The summation order is that of tea_leaf_calc_2norm_kernel_ocl_, and the
 * arithmetic form follows tea_gb300_set_arithmetic (default fused; the
 * chain form sums as fused does): equal inputs and equal forms give equal
 * bits.  Queued on `stream` (a cudaStream_t; NULL for the default stream)
 * and returns before the GPU finishes.  The first call on a device looks up
 * the scratch's device address; make that first call before any stream
 * capture, from one host thread.  All calls share the scratch: calls that
 * can overlap on the GPU (different streams, no ordering between them) race
 * and give wrong results.  Returns 0; an error aborts the process in the
 * library's default mode, and returns -1 (see tea_gb300_last_error) only
 * after tea_gb300_set_abort_on_error(0). */
int tea_gb300_dot_noalloc(const double* a, const double* b, int x_max,
                          int y_max, int halo, long long stride,
                          double* result, void* stream);

/* No counterpart in the reference.  Mixed-precision solve of the current
 * timestep's system (I + L_K) u = u0 on the chunk, after
 * tea_leaf_common_init_kernel_ocl_: FP32 diagonally preconditioned CG inner
 * solves inside an FP64 defect-correction loop.  The FP64 steps are the
 * residual u0 - A u, the accumulation u += d and every dot product; the
 * FP32 ones are the inner vectors and the operator copies.  Stops when
 * ||u0 - A u||_2 <= tol * (its value at entry), or after max_outer
 * corrections; each inner solve stops when its preconditioned residual has
 * fallen by inner_tol or after max_inner iterations.  u holds the FP64
 * solution on return.  Returns 0 or -1. */
typedef struct {
  int outer_iterations;          /* FP64 corrections made */
  long long inner_iterations;    /* FP32 CG iterations, all corrections */
  double initial_residual;       /* ||u0 - A u||_2 at entry */
  double final_residual;         /* ||u0 - A u||_2 at return, FP64 */
  double relative_residual;      /* their ratio */
  long long ppcg_inner_steps;    /* FP32 Chebyshev steps (PPCG inner solver) */
} tea_gb300_mixed_info;
int tea_gb300_mixed_solve(double tol, double inner_tol, int max_outer,
                          int max_inner, tea_gb300_mixed_info* info);
/* The same solve with FP32 PPCG as the inner solver, as the driver's PPCG
 * (tea_solve.f90:147-332, :422-475) in FP32 with diagonal Jacobi: the first
 * correction starts with up to `presteps` CG iterations, whose alphas and
 * betas give the eigenvalue range (x0.95, x1.05) and the Chebyshev
 * coefficients of `inner_steps` inner steps, and continues, like every
 * later correction, with PPCG iterations.  inner_iterations counts CG and
 * PPCG iterations; ppcg_inner_steps the Chebyshev steps.  If the eigenvalue
 * estimate fails the solve stays CG. */
int tea_gb300_mixed_solve_ppcg(double tol, double inner_tol, int max_outer,
                               int max_inner, int presteps, int inner_steps,
                               tea_gb300_mixed_info* info);

/* Waits for all work queued on the library's stream. */
int tea_gb300_synchronize(void);

/* Page-locked host memory for fast field copies. */
void* tea_gb300_host_alloc(size_t bytes);
void tea_gb300_host_free(void* p);

/* ---- whole-run driver (C++ restatement of the Fortran driver) ---- */

/* Solve-loop implementations the driver can use. */
#define TEA_DRIVER_PER_CALL 0  /* reference call sequence, host scalars */
#define TEA_DRIVER_RESIDENT 1  /* CG and PPCG iterations kept on the device */

typedef struct {
  int step;               /* timestep number */
  double time;            /* simulated time after the step */
  double dt;
  int iterations;         /* solver loop iterations run in this step */
  int inner_iterations;   /* PPCG inner steps run in this step */
  double conduction_error; /* final error / initial residual */
  double exact_error;     /* tl_check_result residual (NaN if not asked) */
  int summary_done;       /* 1 if a field summary ran in this step */
  double vol, mass, ie, temp; /* that field summary */
  int complete;           /* 1 after the last step of the deck */
  int qa_passed;          /* test problem check: 1, 0, or -1 (none) */
  double qa_diff;
  int outer_corrections;  /* mixed precision: FP64 corrections (else 0) */
  double relative_residual; /* mixed precision: final ||r||/||r0|| (FP64) */
  int switch_iteration;   /* iteration of the switch from CG to Chebyshev or
                             PPCG in this step (0: none) */
} tea_gb300_step_info;

/* Parses a tea.in deck (its text), sets up the problem on the GPU (as
 * start.f90 does, including the first field summary).  log_path may be
 * NULL, else a tea.out-style log is written.  max_iters_cap > 0 limits
 * solver iterations per step.  Returns 0 or -1 (see tea_gb300_last_error). */
int tea_gb300_driver_open(const char* deck_text, const char* log_path,
                          int mode, int max_iters_cap);
/* One timestep (timestep, tea_leaf, summaries).  Returns 0, 1 when the deck
 * had already completed, or -1 on error. */
int tea_gb300_driver_step(tea_gb300_step_info* info);
/* Closes the log; the chunk stays allocated for inspection. */
void tea_gb300_driver_close(void);

/* Checks the reference does not make (it runs on silently,
 * tea_solve.f90:270-330), off by default:
 *   TEA_CHECK_BREAKDOWN  p.w <= 0 or not finite (error 70), a non-finite
 *                        r.z, r.r or Jacobi error (71): the step fails;
 *   TEA_CHECK_MAX_ITERS  a step that used all tl_max_iters iterations
 *                        without meeting tl_eps fails (72). */
#define TEA_CHECK_BREAKDOWN 1
#define TEA_CHECK_MAX_ITERS 2
/* For the open driver: checks (TEA_CHECK_* flags), and cap_after_switch > 0
 * to end every Chebyshev or PPCG step that many iterations after its switch
 * from CG (the switch's own iteration counted; 0: no such limit), so that a
 * bounded sample still reaches the polynomial solver.  Returns 0 or -1. */
int tea_gb300_driver_set_limits(int cap_after_switch, int checks);

/* ---- batched solves (no counterpart in the reference) ----
 *
 * Many independent single-chunk problems of different sizes, solved
 * together on the GPU with FP64 CG.  Each problem follows, step for step,
 * what the driver above does for one chunk with tl_use_cg and reflective
 * boundaries (tea_solve.f90:37-420 with all faces external): its iteration
 * counts and field summaries are bit-identical to a single-chunk run of the
 * same problem with the same arithmetic form.  One batch exists per process,
 * independent of the chunk; it uses its own stream. */

typedef struct {
  int steps;                 /* timesteps run by the call */
  int max_iterations;        /* largest per-problem iteration count of a step */
  long long iterations;      /* sum of iterations over problems and steps */
  double cell_iterations;    /* sum of cells x iterations */
  int graph_launches;        /* graph replays of the iteration kernels */
  long long kernel_launches; /* kernels run by the call (graph nodes included) */
  double solve_ms;           /* GPU time of the iteration phase (all steps) */
  double total_ms;           /* GPU time of the whole call */
} tea_gb300_batch_stats;

/* Launch geometry of the iteration kernels.  None of it changes a result:
 * the summation order of every problem is fixed by its own size. */
typedef struct {
  int blocks_per_sm;         /* resident blocks per SM of each kernel (1..8) */
  int graph_iterations;      /* CG iterations per graph replay (1..64) */
  int supertiles_per_unit;   /* 256-column supertiles per work unit (1..64) */
  int persistent;            /* 0: three kernels per CG iteration, replayed from
                                a CUDA graph; 1: one persistent (cooperative)
                                kernel per replay running its iterations with
                                grid barriers between the phases */
} tea_gb300_batch_launch;

/* Creates a batch of n problems; problem i has x_cells[i] x y_cells[i]
 * cells on [xmin,xmax] x [ymin,ymax].  preconditioner: TEA_PREC_NONE,
 * TEA_PREC_JAC_DIAG or TEA_PREC_JAC_BLOCK; coefficient: TEA_COEF_*.  The
 * arithmetic form is the one set by tea_gb300_set_arithmetic.  Replaces any
 * earlier batch.  Returns 0 or -1. */
int tea_gb300_batch_create(int n, const int* x_cells, const int* y_cells,
                           double xmin, double xmax, double ymin, double ymax,
                           int preconditioner, int coefficient);
/* Sets problem i's density and energy (host arrays of x_cells*y_cells
 * values, x fastest), as generate_chunk and set_field leave them. */
int tea_gb300_batch_set_fields(int i, const double* density,
                               const double* energy);
/* Runs `steps` timesteps of length dt on every problem, each solved to
 * ||r|| < eps ||r0|| or max_iters iterations.  stats may be NULL. */
int tea_gb300_batch_run(int steps, double dt, double eps, int max_iters,
                        tea_gb300_batch_stats* stats);
/* Field summary of problem i (vol, mass, ie, temp; field_summary_kernel).  */
int tea_gb300_batch_summary(int i, double summary[4]);
/* Iteration count of problem i in each step of the last run
 * (steps values). */
int tea_gb300_batch_iterations(int i, int* iterations, int steps);
/* Copies problem i's interior field (TEA_FIELD_DENSITY, _ENERGY1 or _U) to
 * out (x_cells*y_cells values, x fastest). */
int tea_gb300_batch_read_field(int i, int field, double* out);
/* Sets / reads the launch geometry. */
int tea_gb300_batch_set_launch(const tea_gb300_batch_launch* launch);
int tea_gb300_batch_get_launch(tea_gb300_batch_launch* launch);
/* Times CG iterations per candidate geometry (three-kernel or persistent
 * launch, blocks per SM, supertiles per unit) on the batch's current state
 * (restored afterwards) and keeps the fastest; best gets the choice.  The
 * fields and every later result are unchanged by the search. */
int tea_gb300_batch_autotune(tea_gb300_batch_launch* best);
/* Releases the batch. */
void tea_gb300_batch_free(void);

/* ---- adjoint of the time-stepped solve (no counterpart in the reference) ----
 *
 * The forward model is `steps` TeaLeaf timesteps on one chunk with CG, all
 * faces external and zeroed boundary faces (tea_solve.f90:37-420): each step
 * u0 = energy*density, solve (I + dt L_K) u = u0 to eps*||r0||, energy =
 * u/density.  Its iteration counts and its final u are bit-identical to the
 * single-chunk driver's.  The loss is 0.5*||u_T - u_obs||^2.  The adjoint
 * gives d loss / d log(density) per cell: one CG solve with the same
 * (symmetric) operator per step, backwards, and one fused kernel per step that
 * turns the face-coefficient gradient -(mu_a - mu_b)(u_a - u_b) into the
 * per-cell log-density gradient.  Forward states are checkpointed every
 * `checkpoint_every` steps; the steps in between are recomputed.  One adjoint
 * object exists per process, with its own stream.  Field arguments are DEVICE
 * pointers to x_cells*y_cells doubles, x fastest. */

typedef struct {
  int steps;             /* timesteps */
  double dt;             /* timestep length */
  double eps;            /* relative CG tolerance of every solve */
  int max_iters;         /* CG iteration limit of every solve */
  int checkpoint_every;  /* steps between stored states (>= 1) */
} tea_gb300_adjoint_config;

typedef struct {
  long long forward_iterations;    /* CG iterations of the forward pass */
  long long recompute_iterations;  /* of the recomputed steps */
  long long adjoint_iterations;    /* of the adjoint solves */
  int checkpoints;                 /* states kept by the forward pass */
  double forward_ms;               /* GPU time of the last forward call */
  double backward_ms;              /* GPU time of the last backward call */
} tea_gb300_adjoint_stats;

/* Sets up an x_cells by y_cells problem on [xmin,xmax] x [ymin,ymax] with
 * the given coefficient (TEA_COEF_*) and preconditioner (TEA_PREC_NONE or
 * TEA_PREC_JAC_DIAG), in the arithmetic form set by
 * tea_gb300_set_arithmetic.  Replaces any earlier adjoint object. */
int tea_gb300_adjoint_create(int x_cells, int y_cells, double xmin, double xmax,
                             double ymin, double ymax, int coefficient,
                             int preconditioner);
/* Runs the forward model from density and energy0.  If u_obs is not NULL,
 * *loss gets 0.5*||u_T - u_obs||^2 and the pass is kept for
 * tea_gb300_adjoint_backward.  u_final (may be NULL) gets u_T. */
int tea_gb300_adjoint_forward(const double* density, const double* energy0,
                              const double* u_obs,
                              const tea_gb300_adjoint_config* config,
                              double* loss, double* u_final,
                              tea_gb300_adjoint_stats* stats);
/* d loss / d log(density) of the last forward pass into grad_log_density. */
int tea_gb300_adjoint_backward(double* grad_log_density,
                               tea_gb300_adjoint_stats* stats);
/* Releases the adjoint object. */
void tea_gb300_adjoint_free(void);

#ifdef __cplusplus
}
#endif
#endif
