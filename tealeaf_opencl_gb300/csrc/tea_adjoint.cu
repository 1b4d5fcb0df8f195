// Adjoint of the time-stepped implicit solve with respect to per-cell
// log-density.
//
// Forward model: `steps` TeaLeaf timesteps on one chunk with CG and zeroed
// boundary faces, exactly as the single-chunk driver runs them
// (tea_solve.f90:37-420): u0 = energy*density (init_u), solve
// A u = u0 with A = I + dt L_K to eps*||r0||, energy = u/density (finalise).
// Density, and so A, does not change between steps, so mathematically
// u_{n+1} = A^-1 u_n with u_0 = density*energy_0.  Loss
// L = 0.5*||u_T - u_obs||^2.
//
// Adjoint.  A = I + sum_f K_f (e_a - e_b)(e_a - e_b)^T over the faces f
// between cells a and b, so A is symmetric and
//   lambda_T = u_T - u_obs;
//   for n = T-1 .. 0:  A mu = lambda_{n+1};
//                      dL/dK_f += -(mu_a - mu_b)(u_{n+1,a} - u_{n+1,b});
//                      lambda_n = mu;
//   dL/dlog(rho_c) = sum_f dL/dK_f dK_f/dlog(rho_c) + lambda_0,c u_0,c.
// The face coefficients of tea_leaf_common_cl.cl (init_common) are
// K_f = r (w_a + w_b)/(2 w_a w_b) = r/2 (1/w_a + 1/w_b) with w = rho
// (coefficient 1) or 1/rho (coefficient 2), so dK_f/dlog(rho_c) is
// -r/(2 rho_c) or r rho_c/2: it needs only the cell's own density, and one
// fused per-cell kernel (k_adj_face_grad) turns a step's face products into
// its log-density gradient.  Boundary faces are zeroed (zero_boundary) and
// do not depend on density.
//
// Checkpointing: the forward pass keeps energy at every checkpoint_every-th
// step and u_{n+1} of the steps of the last segment; the backward pass
// recomputes each earlier segment from its checkpoint before walking it
// backwards.  Every solve is the device-resident CG loop of the single-chunk
// path (dev_cg_iteration, graph-replayed), so the forward pass is
// bit-identical to the driver's.
#include <math.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <vector>

#include "../../include/tealeaf_gb300.h"
#include "tea_device.cuh"

namespace tea {

// lambda_T = u - u_obs (u_obs dense, x fastest)
__global__ void k_adj_residual(Dev d, const double* __restrict__ uobs,
                               double* __restrict__ lam) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  if (x >= d.x_max || y >= d.y_max) return;
  const long long c = cidx(d, x, y);
  lam[c] = d.u[c] - uobs[(long long)y * d.x_max + x];
}

// One step's contribution to dL/dlog(rho): the face gradients
// -(mu_a - mu_b)(u_a - u_b) of the cell's four faces (boundary faces
// excluded) times the cell's share of dK_f/dlog(rho).
__global__ void k_adj_face_grad(Dev d, const double* __restrict__ mu,
                                const double* __restrict__ U,
                                double* __restrict__ grad, int coef, double rx,
                                double ry) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  if (x >= d.x_max || y >= d.y_max) return;
  const long long S = d.S;
  const long long c = cidx(d, x, y);
  const double mc = mu[c], uc = U[c];
  double gx = 0.0, gy = 0.0;
  if (x > 0) gx -= (mu[c - 1] - mc) * (U[c - 1] - uc);
  if (x < d.x_max - 1) gx -= (mc - mu[c + 1]) * (uc - U[c + 1]);
  if (y > 0) gy -= (mu[c - S] - mc) * (U[c - S] - uc);
  if (y < d.y_max - 1) gy -= (mc - mu[c + S]) * (uc - U[c + S]);
  const double rho = d.density[c];
  const double sx = coef == 1 ? -rx / (2.0 * rho) : 0.5 * rx * rho;
  const double sy = coef == 1 ? -ry / (2.0 * rho) : 0.5 * ry * rho;
  grad[c] += sx * gx + sy * gy;
}

// The initial condition's term: u_0 = energy_0 * rho, so
// du_0/dlog(rho) = u_0 and the gradient gains lambda_0 * u_0.
__global__ void k_adj_initial(Dev d, const double* __restrict__ lam,
                              const double* __restrict__ e0,
                              double* __restrict__ grad) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  if (x >= d.x_max || y >= d.y_max) return;
  const long long c = cidx(d, x, y);
  grad[c] += lam[c] * (e0[c] * d.density[c]);
}

// Loop scalars at the top of a CG solve (tea_solve.f90:129-146): rro from
// cg_init in results[0], the threshold eps*sqrt(r.r) from results[4].
__global__ void k_adj_begin(ResState* st, const double* results, double eps,
                            int loop_max) {
  ResState s{};
  s.rro = results[0];
  s.eps_target = eps * sqrt(results[4]);
  s.n = 1;
  s.loop_max = loop_max;
  *st = s;
}

}  // namespace tea

namespace {

using namespace tea;

constexpr int kReplayIters = 16;  // CG iterations per graph replay

struct Adjoint {
  bool ready = false;
  int x = 0, y = 0, coef = 1, prec = PREC_JAC_DIAG;
  double xmin = 0, xmax = 0, ymin = 0, ymax = 0;
  int arith = 1;  // arithmetic form
  int num_sms = 0;
  cudaStream_t stream = nullptr;
  cudaEvent_t t0 = nullptr, t1 = nullptr;
  size_t fd = 0;                   // doubles per padded field
  double* arena = nullptr;         // solver fields, lambda, gradient
  double* states = nullptr;        // checkpoints and the segment's u's
  int n_states = 0;
  double* partials = nullptr;
  unsigned int* counters = nullptr;  // [0] reductions, [1] calc_p
  double* results = nullptr;
  ResState* st = nullptr;
  ResState* st_h = nullptr;        // pinned
  Dev d;
  Red red;
  double* lam = nullptr;
  double* grad = nullptr;
  cudaGraphExec_t graph = nullptr;
  // the last forward pass
  bool have_pass = false;
  tea_gb300_adjoint_config cfg{};
  double rx = 0, ry = 0;
  long long fwd_iters = 0;
  double fwd_ms = 0;
  int checkpoints = 0;
};

Adjoint g_adj;

void release_adjoint() {
  Adjoint& a = g_adj;
  if (a.stream) cudaStreamSynchronize(a.stream);
  if (a.graph) cudaGraphExecDestroy(a.graph);
  cudaFree(a.arena);
  cudaFree(a.states);
  cudaFree(a.partials);
  cudaFree(a.counters);
  cudaFree(a.results);
  cudaFree(a.st);
  cudaFreeHost(a.st_h);
  if (a.t0) cudaEventDestroy(a.t0);
  if (a.t1) cudaEventDestroy(a.t1);
  if (a.stream) cudaStreamDestroy(a.stream);
  a = Adjoint();
}

bool adj_ok(const char* who) {
  if (!g_adj.ready) {
    fail(60, "%s: no adjoint object (call tea_gb300_adjoint_create first)", who);
    return false;
  }
  return true;
}

LaunchCtx ctx(const Adjoint& a) { return LaunchCtx{a.stream, a.num_sms, a.arith}; }

template <class K, class... Args>
void launch_cells(const Adjoint& a, const char* name, K kernel, Args... args) {
  kernel<<<dim3((a.x + 31) / 32, (a.y + 7) / 8), dim3(32, 8), 0, a.stream>>>(args...);
  count_launch(name);
  check_cuda(cudaGetLastError(), name);
}

// dense x-fastest array <-> interior of a padded field, device to device
bool dense_to_field(const Adjoint& a, const double* src, double* field) {
  return check_cuda(cudaMemcpy2DAsync(field + a.d.S + 1, a.d.S * sizeof(double), src,
                                      a.x * sizeof(double), a.x * sizeof(double), a.y,
                                      cudaMemcpyDeviceToDevice, a.stream),
                    "adjoint field copy");
}
bool field_to_dense(const Adjoint& a, const double* field, double* dst) {
  return check_cuda(cudaMemcpy2DAsync(dst, a.x * sizeof(double), field + a.d.S + 1,
                                      a.d.S * sizeof(double), a.x * sizeof(double), a.y,
                                      cudaMemcpyDeviceToDevice, a.stream),
                    "adjoint field copy");
}
// whole padded field (halo included)
bool copy_field(const Adjoint& a, double* dst, const double* src) {
  return check_cuda(cudaMemcpyAsync(dst - 31, src - 31, a.fd * sizeof(double),
                                    cudaMemcpyDeviceToDevice, a.stream),
                    "adjoint field copy");
}

// Solves A u = u0 from the initial guess in u with the device-resident CG
// loop of the single-chunk path (the driver's exit test: eps*||r0|| or
// max_iters).  Returns the iteration count, or -1.
long long solve(Adjoint& a, double eps, int max_iters) {
  const LaunchCtx l = ctx(a);
  dev_calc_residual(l, a.d, a.red);
  Red rdot = a.red;
  rdot.result = a.red.result + 4;
  dev_dot(l, a.d, rdot, a.d.r, a.d.r);
  if (a.prec == PREC_JAC_DIAG) dev_init_jac_diag(l, a.d);
  dev_cg_init_p(l, a.d, a.red);
  k_adj_begin<<<1, 1, 0, a.stream>>>(a.st, a.red.result, eps, max_iters);
  count_launch("adjoint_begin");
  const long long max_replays = (long long)max_iters / kReplayIters + 3;
  for (long long nb = 0;; nb++) {
    if (nb >= max_replays) {
      fail(61, "adjoint: CG loop did not stop after %lld graph replays", nb);
      return -1;
    }
    if (!check_cuda(cudaGraphLaunch(a.graph, a.stream), "adjoint replay")) return -1;
    count_launches(3 * kReplayIters);
    if (!check_cuda(cudaMemcpyAsync(a.st_h, a.st, sizeof(ResState),
                                    cudaMemcpyDeviceToHost, a.stream),
                    "adjoint state read") ||
        !check_cuda(cudaStreamSynchronize(a.stream), "adjoint solve"))
      return -1;
    if (a.st_h->stop && !a.st_h->p_pending) break;
  }
  return a.st_h->n;
}

// One forward timestep from energy1: init_u, solve, finalise.
long long forward_step(Adjoint& a, double* keep_u) {
  const LaunchCtx l = ctx(a);
  dev_init_u(l, a.d, a.d.energy1);
  const long long it = solve(a, a.cfg.eps, a.cfg.max_iters);
  if (it < 0) return -1;
  if (keep_u && !copy_field(a, keep_u, a.d.u)) return -1;
  dev_finalise(l, a.d, a.red);
  return it;
}

double* state(Adjoint& a, int k) { return a.states + (size_t)k * a.fd + 31; }

}  // namespace

extern "C" int tea_gb300_adjoint_create(int x_cells, int y_cells, double xmin,
                                        double xmax, double ymin, double ymax,
                                        int coefficient, int preconditioner) {
  release_adjoint();
  Adjoint& a = g_adj;
  if (x_cells < 2 || y_cells < 2 || x_cells > (1 << 16) || y_cells > (1 << 16) ||
      !(xmax > xmin) || !(ymax > ymin)) {
    fail(62, "tea_gb300_adjoint_create: invalid problem %d x %d", x_cells, y_cells);
    return -1;
  }
  if ((coefficient != TEA_COEF_CONDUCTIVITY && coefficient != TEA_COEF_RECIP_CONDUCTIVITY) ||
      (preconditioner != PREC_NONE && preconditioner != PREC_JAC_DIAG)) {
    fail(62, "tea_gb300_adjoint_create: coefficient %d / preconditioner %d not supported",
         coefficient, preconditioner);
    return -1;
  }
  a.x = x_cells;
  a.y = y_cells;
  a.xmin = xmin;
  a.xmax = xmax;
  a.ymin = ymin;
  a.ymax = ymax;
  a.coef = coefficient;
  a.prec = preconditioner;
  a.arith = tea_gb300_get_arithmetic();
  int dev = 0;
  if (!check_cuda(cudaGetDevice(&dev), "cudaGetDevice")) return -1;
  cudaDeviceGetAttribute(&a.num_sms, cudaDevAttrMultiProcessorCount, dev);
  a.ready = true;
  if (!check_cuda(cudaStreamCreateWithFlags(&a.stream, cudaStreamNonBlocking),
                  "adjoint stream")) {
    release_adjoint();
    return -1;
  }
  cudaEventCreate(&a.t0);
  cudaEventCreate(&a.t1);
  // fields with halo 1 and 256-byte-aligned interior rows (as the chunk's)
  const long long S = ((long long)(x_cells + 2 + 1 + 31) / 32) * 32;
  const long long rows = y_cells + 2 + 1;
  a.fd = (size_t)((31 + rows * S + 32 + 31) / 32 * 32);
  const int nf = 14;  // 12 solver fields, lambda, gradient
  const long long ntx = (x_cells + kTileW - 1) / kTileW;
  const long long nsx = (ntx + kTilesPerSuper - 1) / kTilesPerSuper;
  const long long stride = nsx * ((y_cells + 3) / 4) + 1;
  if (!check_cuda(cudaMalloc(&a.arena, nf * a.fd * sizeof(double)), "cudaMalloc adjoint") ||
      !check_cuda(cudaMemsetAsync(a.arena, 0, nf * a.fd * sizeof(double), a.stream),
                  "cudaMemset adjoint") ||
      !check_cuda(cudaMalloc(&a.partials, 4 * stride * sizeof(double)), "cudaMalloc partials") ||
      !check_cuda(cudaMalloc(&a.counters, 2 * sizeof(unsigned int)), "cudaMalloc counters") ||
      !check_cuda(cudaMemsetAsync(a.counters, 0, 2 * sizeof(unsigned int), a.stream),
                  "cudaMemset counters") ||
      !check_cuda(cudaMalloc(&a.results, 8 * sizeof(double)), "cudaMalloc results") ||
      !check_cuda(cudaMalloc(&a.st, sizeof(ResState)), "cudaMalloc state") ||
      !check_cuda(cudaMallocHost(&a.st_h, sizeof(ResState)), "cudaMallocHost state")) {
    release_adjoint();
    return -1;
  }
  Dev d;
  memset(&d, 0, sizeof(d));
  d.x_max = x_cells;
  d.y_max = y_cells;
  d.H = 1;
  d.S = S;
  d.prec = preconditioner;
  int k = 0;
  auto next = [&]() { return a.arena + (k++) * a.fd + 31; };
  d.density = next();
  d.energy1 = next();
  d.u = next();
  d.u0 = next();
  d.p = next();
  d.r = next();
  d.w = next();
  d.Mi = next();
  d.Kx = next();
  d.Ky = next();
  d.z = next();
  d.diag = next();
  d.un = d.Mi;
  a.lam = next();
  a.grad = next();
  a.d = make_dev_tiling(d);
  a.red.partials = a.partials;
  a.red.stride = stride;
  a.red.counter = a.counters;
  a.red.result = a.results;
  // the graph of kReplayIters resident CG iterations on these fields
  const long long n0 = tea_gb300_kernel_launches();
  cudaGraph_t g = nullptr;
  if (!check_cuda(cudaStreamBeginCapture(a.stream, cudaStreamCaptureModeThreadLocal),
                  "adjoint capture")) {
    release_adjoint();
    return -1;
  }
  for (int i = 0; i < kReplayIters; i++)
    dev_cg_iteration(ctx(a), a.d, a.red, a.st, a.counters + 1);
  const bool ok = check_cuda(cudaStreamEndCapture(a.stream, &g), "adjoint capture end") &&
                  check_cuda(cudaGraphInstantiate(&a.graph, g, 0), "adjoint instantiate");
  if (g) cudaGraphDestroy(g);
  count_launches(-(tea_gb300_kernel_launches() - n0));
  if (!ok || !check_cuda(cudaStreamSynchronize(a.stream), "adjoint create")) {
    release_adjoint();
    return -1;
  }
  return 0;
}

extern "C" void tea_gb300_adjoint_free(void) { release_adjoint(); }

extern "C" int tea_gb300_adjoint_forward(const double* density, const double* energy0,
                                         const double* u_obs,
                                         const tea_gb300_adjoint_config* config,
                                         double* loss, double* u_final,
                                         tea_gb300_adjoint_stats* stats) {
  if (loss) *loss = NAN;
  if (stats) memset(stats, 0, sizeof(*stats));
  if (!adj_ok("tea_gb300_adjoint_forward")) return -1;
  Adjoint& a = g_adj;
  const long long errors = error_count();
  a.have_pass = false;
  if (!density || !energy0 || !config || config->steps < 1 || !(config->dt > 0.0) ||
      !(config->eps >= 0.0) || config->max_iters < 1 || config->checkpoint_every < 1) {
    fail(63, "tea_gb300_adjoint_forward: invalid arguments");
    return -1;
  }
  a.cfg = *config;
  const int T = a.cfg.steps, ce = std::min(a.cfg.checkpoint_every, T);
  const int nseg = (T + ce - 1) / ce;
  const int need = nseg + ce;  // checkpoints, then the last segment's u's
  if (need > a.n_states) {
    cudaFree(a.states);
    a.states = nullptr;
    a.n_states = 0;
    if (!check_cuda(cudaMalloc(&a.states, (size_t)need * a.fd * sizeof(double)),
                    "cudaMalloc adjoint states") ||
        !check_cuda(cudaMemsetAsync(a.states, 0, (size_t)need * a.fd * sizeof(double),
                                    a.stream),
                    "cudaMemset adjoint states"))
      return -1;
    a.n_states = need;
  }
  const LaunchCtx l = ctx(a);
  cudaEventRecord(a.t0, a.stream);
  if (!dense_to_field(a, density, a.d.density) || !dense_to_field(a, energy0, a.d.energy1))
    return -1;
  // common_init with all faces external (tea_leaf_kernel_ocl.cpp:233-289);
  // density does not change, so the operator is set up once
  const double dx = (a.xmax - a.xmin) / (double)(float)a.x;
  const double dy = (a.ymax - a.ymin) / (double)(float)a.y;
  a.rx = a.cfg.dt / (dx * dx);
  a.ry = a.cfg.dt / (dy * dy);
  const int zb[4] = {1, 1, 1, 1};
  dev_update_halo(l, a.d, 1 | 4, 1);
  dev_init_common(l, a.d, a.coef, a.rx, a.ry);
  dev_zero_boundary(l, a.d, zb);
  dev_init_diag(l, a.d, a.red);
  long long iters = 0;
  const int last_k0 = (nseg - 1) * ce;
  for (int n = 0; n < T; n++) {
    if (n % ce == 0 && !copy_field(a, state(a, n / ce), a.d.energy1)) return -1;
    const long long it = forward_step(a, n >= last_k0 ? state(a, nseg + n - last_k0) : nullptr);
    if (it < 0) return -1;
    iters += it;
  }
  if (u_final && !field_to_dense(a, a.d.u, u_final)) return -1;
  if (u_obs) {
    launch_cells(a, "adjoint_residual", k_adj_residual, a.d, u_obs, a.lam);
    Red rl = a.red;
    rl.result = a.red.result + 5;
    dev_dot(l, a.d, rl, a.lam, a.lam);
    double sum = NAN;
    if (!check_cuda(cudaMemcpyAsync(&sum, a.red.result + 5, sizeof(double),
                                    cudaMemcpyDeviceToHost, a.stream),
                    "adjoint loss"))
      return -1;
    cudaEventRecord(a.t1, a.stream);
    if (!check_cuda(cudaStreamSynchronize(a.stream), "adjoint forward")) return -1;
    if (loss) *loss = 0.5 * sum;
  } else {
    cudaEventRecord(a.t1, a.stream);
    if (!check_cuda(cudaStreamSynchronize(a.stream), "adjoint forward")) return -1;
  }
  float ms = 0.0f;
  cudaEventElapsedTime(&ms, a.t0, a.t1);
  a.fwd_iters = iters;
  a.fwd_ms = ms;
  a.checkpoints = nseg;
  a.have_pass = u_obs != nullptr && error_count() == errors;
  if (stats) {
    stats->forward_iterations = iters;
    stats->checkpoints = nseg;
    stats->forward_ms = ms;
  }
  return error_count() == errors ? 0 : -1;
}

extern "C" int tea_gb300_adjoint_backward(double* grad_log_density,
                                          tea_gb300_adjoint_stats* stats) {
  if (stats) memset(stats, 0, sizeof(*stats));
  if (!adj_ok("tea_gb300_adjoint_backward")) return -1;
  Adjoint& a = g_adj;
  if (!a.have_pass || !grad_log_density) {
    fail(64, "tea_gb300_adjoint_backward: needs a forward pass with u_obs first");
    return -1;
  }
  const long long errors = error_count();
  a.have_pass = false;  // lambda and the states are consumed below
  const int T = a.cfg.steps, ce = std::min(a.cfg.checkpoint_every, T);
  const int nseg = (T + ce - 1) / ce;
  const LaunchCtx l = ctx(a);
  long long rec_iters = 0, adj_iters = 0;
  cudaEventRecord(a.t0, a.stream);
  if (!check_cuda(cudaMemsetAsync(a.grad - 31, 0, a.fd * sizeof(double), a.stream),
                  "adjoint gradient clear"))
    return -1;
  for (int seg = nseg - 1; seg >= 0; seg--) {
    const int k0 = seg * ce, k1 = std::min(k0 + ce, T);
    if (seg != nseg - 1) {
      // recompute the segment from its checkpoint, keeping each u_{n+1}
      if (!copy_field(a, a.d.energy1, state(a, seg))) return -1;
      for (int n = k0; n < k1; n++) {
        const long long it = forward_step(a, state(a, nseg + n - k0));
        if (it < 0) return -1;
        rec_iters += it;
      }
    }
    for (int n = k1 - 1; n >= k0; n--) {
      // A mu = lambda_{n+1} from the initial guess lambda_{n+1}
      if (!copy_field(a, a.d.u0, a.lam) || !copy_field(a, a.d.u, a.lam)) return -1;
      const long long it = solve(a, a.cfg.eps, a.cfg.max_iters);
      if (it < 0) return -1;
      adj_iters += it;
      launch_cells(a, "adjoint_face_grad", k_adj_face_grad, a.d, (const double*)a.d.u,
                   (const double*)state(a, nseg + n - k0), a.grad, a.coef, a.rx, a.ry);
      if (!copy_field(a, a.lam, a.d.u)) return -1;
    }
  }
  launch_cells(a, "adjoint_initial", k_adj_initial, a.d, (const double*)a.lam,
               (const double*)state(a, 0), a.grad);
  if (!field_to_dense(a, a.grad, grad_log_density)) return -1;
  cudaEventRecord(a.t1, a.stream);
  if (!check_cuda(cudaStreamSynchronize(a.stream), "adjoint backward")) return -1;
  float ms = 0.0f;
  cudaEventElapsedTime(&ms, a.t0, a.t1);
  if (stats) {
    stats->forward_iterations = a.fwd_iters;
    stats->recompute_iterations = rec_iters;
    stats->adjoint_iterations = adj_iters;
    stats->checkpoints = a.checkpoints;
    stats->forward_ms = a.fwd_ms;
    stats->backward_ms = ms;
  }
  return error_count() == errors ? 0 : -1;
}
