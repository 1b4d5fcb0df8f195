// Internal declarations shared by the CUDA kernels, the C-ABI layer and the
// resident solver of libtealeaf_gb300.so.
//
// Field layout in HBM.  Every 2-D field is FP64, x fastest.  Padded
// coordinates (col,row) follow the reference (interior at
// [H, H+x_max) x [H, H+y_max), halo of depth H around it;
// THARR2D, macros_cl.cl:20-22) but the row stride S is rounded up to a
// multiple of 32 doubles (256 B) and the base is offset so that interior
// column H of every row starts on a 256-byte boundary.  Each field holds
// y_max+2H+1 rows of S doubles (the extra row and the columns past x_max+2H
// play the role of the reference's "+1" allocations, ocl_buffers.cpp:55-69)
// and is zero-filled at allocation, as the reference's buffers are.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

namespace tea {

constexpr int kBlock = 256;  // threads per block of every tile kernel
constexpr int kTileW = 32;   // columns per tile (one per lane)
constexpr int kTilesPerSuper = 8;  // tiles per supertile (one per warp)

enum Prec { PREC_NONE = 1, PREC_JAC_DIAG = 2, PREC_JAC_BLOCK = 3 };
enum Solver { SOLVER_JACOBI = 1, SOLVER_CG = 2, SOLVER_CHEBY = 3, SOLVER_PPCG = 4 };

// POD view of the chunk passed by value to every kernel.
struct Dev {
  int x_max, y_max, H;
  long long S;        // row stride in doubles
  int xs, ys;         // logical padded extents x_max+2H, y_max+2H
  int prec;
  int block_top_check;  // y_max % 4 != 0 (ocl_kernels.cpp:26-29)
  int ntx, nsx, nty, ns;  // tiling for the chunk's tile height
  int th;                 // the tile height itself (4 or 16)
  double *density, *energy0, *energy1, *volume;
  double *u, *u0, *p, *r, *w, *Mi, *Kx, *Ky, *sd, *z, *cp, *bfp, *un;
  double* diag;  // 1 + (Ky_n + Ky_c) + (Kx_e + Kx_c), set by common_init
  double *cellx, *celly, *celldx, *celldy, *vertexx, *vertexy, *vertexdx,
      *vertexdy;
};

// Scratch for the fixed-order reductions: per-supertile partial sums, a
// completion counter and the reduced values.
struct Red {
  double* partials;     // [nvals][stride]
  long long stride;     // >= number of supertiles
  unsigned int* counter;
  double* result;       // [nvals]
  // Optional copy of the result in mapped pinned host memory for a caller
  // waiting on the host: the bit patterns of the result values at
  // host[0..nvals), then a nonzero word at host[8] once they are visible
  // (see tea_abi.cu, fetch).
  unsigned long long* host = nullptr;
};

// Scalar state of the device-resident CG loop: the host scalars of
// tea_solve.f90:270-300 kept in device memory.
struct ResState {
  double rro, pw, rrn, alpha, beta, error;
  double eps_target;  // eps * initial_residual
  int n, loop_max;
  int stop;       // set when the loop has converged or reached loop_max
  int p_pending;  // calc_p of the current iteration still to run
  int converged;
  int check;       // stop on a breakdown (p.w <= 0 or not finite, r.z not finite)
  int breakdown;   // 0, or 1 (p.w) / 2 (r.z) with check set
  int breakdown_n; // the iteration it happened in
  double rr_true;  // r.r of the last iteration (true-residual exit only)
  double* alphas;  // indexed by iteration number n
  double* betas;
};

struct Field {
  double* base = nullptr;  // cudaMalloc'd allocation
  double* f = nullptr;     // element (0,0) of the padded layout
};

// Host-side chunk state (one per process, as CloverChunk in the reference).
struct Chunk {
  bool ready = false;
  int x_max = 0, y_max = 0, H = 1;
  int solver = SOLVER_JACOBI, prec = PREC_NONE;
  bool profiler_on = false;
  int TH = 4;  // reduction tile height
  long long S = 0;
  long long rows = 0;
  size_t field_doubles = 0;
  int device = 0, num_sms = 0;
  cudaStream_t stream = nullptr;
  Field density, energy0, energy1, volume, u, u0, p, r, w, Mi, Kx, Ky, sd, z,
      cp, bfp, diag;
  int arith = 1;  // arithmetic form: 0 exact, 1 fused, 2 chain (tea_device.cuh)
  double *cellx = nullptr, *celly = nullptr, *celldx = nullptr,
         *celldy = nullptr, *vertexx = nullptr, *vertexy = nullptr,
         *vertexdx = nullptr, *vertexdy = nullptr;
  // reductions
  double* red_partials = nullptr;
  long long red_stride = 0;
  unsigned int* red_counter = nullptr;
  double* red_result = nullptr;
  double* host_result = nullptr;  // pinned, 8 doubles
  unsigned long long* host_map = nullptr;      // mapped pinned: 8 results, ready word
  unsigned long long* host_map_dev = nullptr;  // its device address
  bool red_to_host = false;        // next c.red() copies its result to host_map
  // coefficients kept on the host (passed to kernels by value) and on device
  double* cheby_alpha_h = nullptr;
  double* cheby_beta_h = nullptr;
  int n_cheby = 0;
  double cheby_theta = 0.0;
  double* ppcg_alpha_h = nullptr;
  double* ppcg_beta_h = nullptr;
  int n_ppcg = 0;
  double ppcg_theta = 0.0;
  double celldx_h = 0.0, celldy_h = 0.0;
  // device-resident CG loop
  ResState* res_state = nullptr;       // device
  ResState* res_state_h = nullptr;     // pinned mirror
  double* res_coef = nullptr;          // device alphas/betas
  int res_coef_n = 0;
  unsigned int* res_counter = nullptr;
  unsigned int* res_bar = nullptr;     // grid barrier [2] + error flag
  cudaGraphExec_t res_ppcg_graph = nullptr;  // resident PPCG iterations
  std::vector<double> res_ppcg_key;          // theta, coefficients, form of it
  int resident_mode = 0;               // 0 auto, 1 graph replay, 2 persistent
  // second r and sd buffers for the fused pair of PPCG inner steps
  // (tea_ppcg_tb.cu), which writes r and sd to the pair it does not read;
  // allocated on first use, with the halos of the live pair
  Field r2, sd2;
  // second u buffer of the Chebyshev iteration with calc_u folded into
  // calc_p (block Jacobi), which writes the new u, halo included, to the
  // buffer it does not read; the two then trade places
  Field u2;
  int inner_pairs = 0;      // run PPCG inner steps in fused pairs where they apply
  int field_epoch = 0;      // bumped whenever r/sd and r2/sd2 trade places
  int pending_inner = -1;   // a per-call inner step (0-based) not launched yet
  // PPCG's sd formed ahead by calc_ur into sd2 (tea_abi.cu): valid for the
  // init_sd call that directly follows that calc_ur
  long long abi_calls = 0;       // entry-point calls on this chunk
  long long spec_sd_call = -1;   // abi_calls of that calc_ur, or -1
  double spec_sd_theta = 0.0;
  int spec_sd_arith = -1;
  int solver_checks = 0;               // next resident loop: stop on a breakdown
  // grid barrier of the persistent loop: polls before it gives up, and the
  // arrivals it waits for beyond the grid (nonzero only to test the time-out)
  long long barrier_spin_limit = 1LL << 26;
  int barrier_extra = 0;
  int res_breakdown = 0, res_breakdown_n = 0;  // what the last one found
  cudaGraphExec_t res_graph = nullptr;
  int res_graph_iters = 0;
  bool res_graph_true_exit = false;
  int res_graph_epoch = 0;  // field_epoch the CG graph was captured at
  double res_last_rr_true = 0.0;

  Dev dev() const;
  Red red() const;
};

Chunk& chunk();

// error handling (tea_abi.cu)
void fail(int code, const char* fmt, ...);
int error_code();
long long error_count();  // errors recorded so far (never reset)
bool check_cuda(cudaError_t e, const char* what);
void count_launch(const char* name);
void count_launches(long long n);  // n kernels run from a graph replay
void profile_begin(const char* name);
void profile_end(const char* name);

int reduction_rows(int x_max, int y_max);

// ---- kernel launch wrappers (tea_kernels.cu) ----
// setup
void launch_initialise_chunk(Chunk& c, double xmin, double ymin, double dx,
                             double dy);
void launch_generate_init(Chunk& c, double density0, double energy0);
void launch_generate_state(Chunk& c, double density, double energy,
                           double xmin, double xmax, double ymin, double ymax,
                           double radius, int geometry, int g_rect, int g_circ,
                           int g_point);
void launch_init_u(Chunk& c, const double* energy);
void launch_set_field(Chunk& c);
// solver
void launch_init_common(Chunk& c, int coef, double rx, double ry);
void launch_zero_boundary(Chunk& c, const int* zero_boundary);
void launch_calc_residual(Chunk& c);
void launch_dot(Chunk& c, const double* a, const double* b);
void launch_init_jac_diag(Chunk& c);
void launch_init_diag(Chunk& c);
void launch_block_init(Chunk& c);
void launch_cg_init_p(Chunk& c);
void launch_cg_calc_w(Chunk& c);
void launch_cg_calc_ur(Chunk& c, double alpha);
// calc_ur and, from its z, PPCG's sd = M^-1 r / theta into sd_out
void launch_cg_calc_ur_sd(Chunk& c, double alpha, double theta, double* sd_out);
void launch_cg_calc_p(Chunk& c, double beta);
void launch_cheby_init_p(Chunk& c, double theta);
void launch_cheby_calc_p(Chunk& c, double alpha, double beta);
void launch_cheby_calc_u(Chunk& c);
// calc_p and calc_u of one Chebyshev iteration in one pass (block Jacobi),
// the new u into un
void launch_cheby_calc_pu(Chunk& c, double alpha, double beta, double* un);
void launch_ppcg_init_sd(Chunk& c, double theta);
void launch_ppcg_update_r(Chunk& c);
// update_r and calc_sd of one inner step in one pass (block Jacobi), sd
// read from sdi and the new sd written to sdo
void launch_ppcg_step(Chunk& c, double alpha, double beta, const double* sdi, double* sdo);
void launch_ppcg_calc_sd(Chunk& c, double alpha, double beta);
void launch_jacobi_copy_u(Chunk& c);
void launch_jacobi_solve(Chunk& c);
void launch_finalise(Chunk& c);
void launch_field_summary(Chunk& c);
void launch_update_halo(Chunk& c, int mask, int depth);
// The same kernels for an explicit field set (a problem of a batch):
// launched on `stream` with grids sized for `num_sms` SMs.
struct LaunchCtx {
  cudaStream_t stream;
  int num_sms;
  int arith;  // arithmetic form
};
Dev make_dev_tiling(Dev d);  // fills th, ntx, nsx, nty, ns from x_max, y_max
Dev rows4_tiling(Dev d);     // the same field set tiled in 4-row tiles
void dev_volume(const LaunchCtx& l, const Dev& d, double vol);
void dev_init_common(const LaunchCtx& l, const Dev& d, int coef, double rx,
                     double ry);
void dev_zero_boundary(const LaunchCtx& l, const Dev& d, const int* zb);
void dev_init_diag(const LaunchCtx& l, const Dev& d, const Red& r);
void dev_init_jac_diag(const LaunchCtx& l, const Dev& d);
void dev_init_u(const LaunchCtx& l, const Dev& d, const double* energy);
void dev_calc_residual(const LaunchCtx& l, const Dev& d, const Red& r);
void dev_dot(const LaunchCtx& l, const Dev& d, const Red& r, const double* a,
             const double* b);
void dev_block_init(const LaunchCtx& l, const Dev& d);
void dev_update_halo(const LaunchCtx& l, const Dev& d, int mask, int depth);
void dev_cg_init_p(const LaunchCtx& l, const Dev& d, const Red& r);
// one iteration of the device-resident CG loop (loop scalars in *st; the
// kernels return at once after it has stopped)
void dev_cg_iteration(const LaunchCtx& l, const Dev& d, const Red& r, ResState* st,
                      unsigned int* counter);
void dev_finalise(const LaunchCtx& l, const Dev& d, const Red& r);
void dev_field_summary(const LaunchCtx& l, const Dev& d, const Red& r);
// device-resident CG loop (tea_kernels.cu)
// true_exit: stop on ||r||_2 < eps_target instead of sqrt(r.z)
int resident_cg_iterations(int n_begin, int loop_max, double rro_in,
                           double eps_target, double* rro_out,
                           double* error_out, int* n_done, int* converged,
                           double* cg_alphas, double* cg_betas,
                           bool true_exit = false);
// device-resident PPCG iterations n_begin..loop_max with the coefficients
// of the last tea_leaf_ppcg_init_ocl_ (tea_solve.f90:231-268); the fused
// calc_ur + init_sd kernel replaces the per-call pair
int resident_ppcg_iterations(int n_begin, int loop_max, double rro_in,
                             double eps_target, double* rro_out, double* error_out,
                             int* n_done, int* converged);
void resident_release();
// fused pair of PPCG inner steps (tea_ppcg_tb.cu)
bool tb_applicable(const Chunk& c);
bool tb_prepare(Chunk& c);  // before any graph capture that launches the pair
bool launch_ppcg_inner_pair(Chunk& c, int s, const ResState* st, double* r_in,
                            double* sd_in, double* r_out, double* sd_out);
int tb_error();
void tb_release();
// the second r/sd buffers (tea_abi.cu): allocated and given the live
// buffers' contents once; false on failure
bool ensure_alt_fields(Chunk& c);
// allocates u2 on first use
bool ensure_u_alt(Chunk& c);
// r/sd and r2/sd2 trade places (the fused pair has just written r2/sd2)
void swap_alt_fields(Chunk& c);
// launches a per-call PPCG inner step held back for pairing (tea_abi.cu)
void flush_pending_inner(Chunk& c);
// mixed-precision solve (tea_mixed.cu)
void mixed_release();
// eigenvalue range from CG alphas/betas (nsteps of each, iteration 1
// first) and Chebyshev coefficients (tea_driver.cpp; tea_leaf_cheby.f90)
int eigenvalues_from_cg(const std::vector<double>& alphas,
                        const std::vector<double>& betas, int nsteps,
                        double* eigmin, double* eigmax);
void chebyshev_coefficients(std::vector<double>& a, std::vector<double>& b,
                            double eigmin, double eigmax, double* theta, int n);
// FP64 fused-multiply-add instructions per second of this GPU
double measure_fp64_rate();

}  // namespace tea
