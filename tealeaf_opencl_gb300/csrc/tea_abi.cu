// The C ABI of libtealeaf_gb300.so: the reference's extern "C" entry points
// (tea_leaf_kernel_ocl.cpp, field_summary_kernel_ocl.cpp,
// update_halo_kernel_ocl.cpp, ocl_init.cpp, initialise_chunk_kernel_ocl.cpp,
// generate_chunk_kernel_ocl.cpp, set_field_kernel_ocl.cpp, ocl_errors.cpp,
// ocl_pack.cpp) on top of the CUDA kernels, plus the chunk's lifecycle.
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <fstream>
#include <map>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/tealeaf_gb300.h"
#include "tea_internal.h"

namespace tea {

static Chunk g_chunk;
Chunk& chunk() { return g_chunk; }

// ---------------------------------------------------------------------------
// errors, launch accounting, profiling
// ---------------------------------------------------------------------------

static int g_abort_on_error = 1;
static int g_err_code = 0;
static long long g_err_count = 0;  // errors recorded since load
static std::string g_err_msg;
static long long g_launches = 0;

void fail(int code, const char* fmt, ...) {
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_err_count++;
  g_err_code = code;  // the most recent error is the one reported
  g_err_msg = buf;
  fprintf(stderr, "@@@@@\nFatal error in libtealeaf_gb300: %s\n", buf);
  if (g_abort_on_error) {
    fprintf(stderr, "Exiting\n");
    abort();
  }
}

int error_code() { return g_err_code; }
long long error_count() { return g_err_count; }

bool check_cuda(cudaError_t e, const char* what) {
  if (e == cudaSuccess) return true;
  fail(2, "CUDA error in %s: %s", what, cudaGetErrorString(e));
  return false;
}

void count_launch(const char*) { g_launches++; }
void count_launches(long long n) { g_launches += n; }

struct ProfEntry {
  long long calls = 0;
  double ms = 0.0;
};
static std::map<std::string, ProfEntry> g_prof;
static cudaEvent_t g_prof_ev[2] = {nullptr, nullptr};

// Optional timing of kernels inside a running workload: event pairs
// recorded around each launch on the library's stream and read back in
// batches, without serialising the other work.  The selection is one kernel
// name, or "*" for every kernel.
static std::string g_timed_name;
static std::vector<cudaEvent_t> g_timed_ev;
static std::vector<std::string> g_timed_names;
static size_t g_timed_used = 0;
static std::map<std::string, ProfEntry> g_timed;

static void timed_drain() {
  if (g_timed_used == 0) return;
  cudaEventSynchronize(g_timed_ev[2 * g_timed_used - 1]);
  for (size_t i = 0; i < g_timed_used; i++) {
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, g_timed_ev[2 * i], g_timed_ev[2 * i + 1]);
    ProfEntry& e = g_timed[g_timed_names[i]];
    e.ms += ms;
    e.calls++;
  }
  g_timed_used = 0;
}

static bool timed_match(const char* name) {
  return !g_timed_name.empty() && (g_timed_name == "*" || g_timed_name == name);
}

void profile_begin(const char* name) {
  Chunk& c = chunk();
  if (timed_match(name)) {
    if (g_timed_ev.empty()) {
      g_timed_ev.resize(2 * 1024);
      g_timed_names.resize(1024);
      for (auto& e : g_timed_ev) cudaEventCreate(&e);
    }
    if (2 * (g_timed_used + 1) > g_timed_ev.size()) timed_drain();
    g_timed_names[g_timed_used] = name;
    cudaEventRecord(g_timed_ev[2 * g_timed_used], c.stream);
  }
  if (!c.profiler_on) return;
  if (!g_prof_ev[0]) {
    cudaEventCreate(&g_prof_ev[0]);
    cudaEventCreate(&g_prof_ev[1]);
  }
  cudaEventRecord(g_prof_ev[0], c.stream);
}

// Waits for the kernel, as the reference's profiled enqueueKernel does
// (ocl_errors.cpp:75-122).
void profile_end(const char* name) {
  Chunk& c = chunk();
  if (timed_match(name)) {
    cudaEventRecord(g_timed_ev[2 * g_timed_used + 1], c.stream);
    g_timed_used++;
  }
  if (!c.profiler_on) return;
  cudaEventRecord(g_prof_ev[1], c.stream);
  cudaEventSynchronize(g_prof_ev[1]);
  float ms = 0.0f;
  cudaEventElapsedTime(&ms, g_prof_ev[0], g_prof_ev[1]);
  ProfEntry& e = g_prof[name];
  e.calls++;
  e.ms += ms;
}

// ---------------------------------------------------------------------------
// chunk
// ---------------------------------------------------------------------------

int reduction_rows(int x_max, int y_max) {
  const long long nsx = (x_max + 255) / 256;
  const long long nsy16 = (y_max + 15) / 16;
  return (nsx * nsy16 >= 1216) ? 16 : 4;
}

Dev Chunk::dev() const {
  Dev d;
  memset(&d, 0, sizeof(d));
  d.x_max = x_max;
  d.y_max = y_max;
  d.H = H;
  d.S = S;
  d.xs = x_max + 2 * H;
  d.ys = y_max + 2 * H;
  d.prec = prec;
  d.block_top_check = (y_max % 4) != 0;
  d.ntx = (x_max + kTileW - 1) / kTileW;
  d.nsx = (d.ntx + kTilesPerSuper - 1) / kTilesPerSuper;
  d.nty = (y_max + TH - 1) / TH;
  d.ns = d.nsx * d.nty;
  d.th = TH;
  d.density = density.f;
  d.energy0 = energy0.f;
  d.energy1 = energy1.f;
  d.volume = volume.f;
  d.u = u.f;
  d.u0 = u0.f;
  d.p = p.f;
  d.r = r.f;
  d.w = w.f;
  d.Mi = Mi.f;
  d.Kx = Kx.f;
  d.Ky = Ky.f;
  d.sd = sd.f;
  d.z = z.f;
  d.cp = cp.f;
  d.bfp = bfp.f;
  d.diag = diag.f;
  d.un = Mi.f;  // the reference reuses vector_Mi as Jacobi's un
  d.cellx = cellx;
  d.celly = celly;
  d.celldx = celldx;
  d.celldy = celldy;
  d.vertexx = vertexx;
  d.vertexy = vertexy;
  d.vertexdx = vertexdx;
  d.vertexdy = vertexdy;
  return d;
}

Red Chunk::red() const {
  Red rr;
  rr.partials = red_partials;
  rr.stride = red_stride;
  rr.counter = red_counter;
  rr.result = red_result;
  rr.host = red_to_host ? host_map_dev : nullptr;
  return rr;
}

static void free_chunk(Chunk& c) {
  if (!c.ready) return;
  resident_release();
  mixed_release();
  Field* l[] = {&c.density, &c.energy0, &c.energy1, &c.volume, &c.u, &c.u0,
                &c.p,       &c.r,       &c.w,       &c.Mi,     &c.Kx, &c.Ky,
                &c.sd,      &c.z,       &c.cp,      &c.bfp,    &c.diag};
  for (Field* f : l) {
    cudaFree(f->base);
    f->base = f->f = nullptr;
  }
  double** one[] = {&c.cellx,   &c.celly,   &c.celldx,   &c.celldy,
                    &c.vertexx, &c.vertexy, &c.vertexdx, &c.vertexdy,
                    &c.red_partials, &c.red_result};
  for (double** p : one) {
    cudaFree(*p);
    *p = nullptr;
  }
  cudaFree(c.red_counter);
  c.red_counter = nullptr;
  cudaFreeHost(c.host_result);
  c.host_result = nullptr;
  cudaFreeHost(c.host_map);
  c.host_map = c.host_map_dev = nullptr;
  c.red_to_host = false;
  free(c.cheby_alpha_h);
  free(c.cheby_beta_h);
  free(c.ppcg_alpha_h);
  free(c.ppcg_beta_h);
  c.cheby_alpha_h = c.cheby_beta_h = c.ppcg_alpha_h = c.ppcg_beta_h = nullptr;
  cudaFree(c.r2.base);
  cudaFree(c.sd2.base);
  cudaFree(c.u2.base);
  c.r2 = c.sd2 = c.u2 = Field();
  c.pending_inner = -1;
  tb_release();
  if (c.stream) cudaStreamDestroy(c.stream);
  c.stream = nullptr;
  c.ready = false;
}

static bool alloc_field(Chunk& c, Field& f) {
  // the offset makes padded column H of every row 256-byte aligned
  const long long off = (32 - (c.H % 32)) % 32;
  const size_t n = (size_t)(off + c.rows * c.S + 32);
  if (!check_cuda(cudaMalloc(&f.base, n * sizeof(double)), "cudaMalloc field"))
    return false;
  if (!check_cuda(cudaMemsetAsync(f.base, 0, n * sizeof(double), c.stream),
                  "cudaMemset field"))
    return false;
  f.f = f.base + off;
  return true;
}

struct Config {
  bool set = false;
  int halo = 1, solver = SOLVER_JACOBI, prec = PREC_NONE, profiler = 0;
  int arith = 1;  // arithmetic form
  int resident_mode = 0;
  long long barrier_spin_limit = 1LL << 26;  // persistent loop's grid barrier
  int barrier_extra = 0;
  int inner_pairs = 0;  // measured slower than one-pass steps on GB300 (tea_ppcg_tb.cu)
};
static Config g_config;

// matchParam / readInt / paramEnabled (ocl_strings.cpp:7-37, :53-75,
// :127-132): first line without '!' that contains the name; its value is
// the text after the first '='.
static std::string match_param(const std::string& text, const char* name) {
  std::istringstream in(text);
  std::string line;
  while (std::getline(in, line)) {
    if (line.find('!') != std::string::npos) continue;
    if (line.find(name) != std::string::npos) {
      const size_t eq = line.find('=');
      if (eq != std::string::npos) return line.substr(eq + 1);
      return std::string(name);
    }
  }
  return std::string();
}

static bool config_from_tea_in(Config* cfg) {
  std::ifstream f("tea.in");
  if (!f.is_open()) {
    fail(3, "Input file not found");
    return false;
  }
  std::stringstream ss;
  ss << f.rdbuf();
  const std::string text = ss.str();
  cfg->profiler = !match_param(text, "profiler_on").empty();
  {
    std::stringstream conv(match_param(text, "halo_depth"));
    int h = -1;
    if (!(conv >> h)) h = -1;
    cfg->halo = h;
    if (h < 1) {
      fail(3, "Halo exchange depth unspecified or was too small");
      return false;
    }
  }
  if (!match_param(text, "tl_use_ppcg").empty())
    cfg->solver = SOLVER_PPCG;
  else if (!match_param(text, "tl_use_chebyshev").empty())
    cfg->solver = SOLVER_CHEBY;
  else if (!match_param(text, "tl_use_cg").empty())
    cfg->solver = SOLVER_CG;
  else
    cfg->solver = SOLVER_JACOBI;
  std::string prec = match_param(text, "tl_preconditioner_type");
  std::transform(prec.begin(), prec.end(), prec.begin(), ::tolower);
  if (prec.find("jac_diag") != std::string::npos)
    cfg->prec = PREC_JAC_DIAG;
  else if (prec.find("jac_block") != std::string::npos)
    cfg->prec = PREC_JAC_BLOCK;
  else
    cfg->prec = PREC_NONE;
  return true;
}

static bool init_chunk(int x_max, int y_max, const Config& cfg) {
  Chunk& c = chunk();
  free_chunk(c);
  c = Chunk();
  if (x_max < 1 || y_max < 1) {
    fail(4, "invalid chunk size %d x %d", x_max, y_max);
    return false;
  }
  c.x_max = x_max;
  c.y_max = y_max;
  c.H = cfg.halo;
  c.solver = cfg.solver;
  c.prec = cfg.prec;
  c.profiler_on = cfg.profiler != 0;
  c.arith = cfg.arith;
  c.resident_mode = cfg.resident_mode;
  c.barrier_spin_limit = cfg.barrier_spin_limit;
  c.barrier_extra = cfg.barrier_extra;
  c.inner_pairs = cfg.inner_pairs;
  c.TH = reduction_rows(x_max, y_max);
  c.S = ((long long)(x_max + 2 * c.H + 1 + 31) / 32) * 32;
  c.rows = y_max + 2 * c.H + 1;
  if (!check_cuda(cudaGetDevice(&c.device), "cudaGetDevice")) return false;
  cudaDeviceGetAttribute(&c.num_sms, cudaDevAttrMultiProcessorCount, c.device);
  if (!check_cuda(cudaStreamCreateWithFlags(&c.stream, cudaStreamNonBlocking),
                  "cudaStreamCreate"))
    return false;
  c.ready = true;  // so that free_chunk releases partial allocations
  Field* l[] = {&c.density, &c.energy0, &c.energy1, &c.volume, &c.u, &c.u0,
                &c.p,       &c.r,       &c.w,       &c.Mi,     &c.Kx, &c.Ky,
                &c.sd,      &c.z,       &c.cp,      &c.bfp,    &c.diag};
  for (Field* f : l)
    if (!alloc_field(c, *f)) return false;
  const int n1 = std::max(x_max, y_max) + 2 * c.H + 2;
  double** one[] = {&c.cellx,   &c.celly,   &c.celldx,   &c.celldy,
                    &c.vertexx, &c.vertexy, &c.vertexdx, &c.vertexdy};
  for (double** p : one) {
    if (!check_cuda(cudaMalloc(p, n1 * sizeof(double)), "cudaMalloc 1d"))
      return false;
    cudaMemsetAsync(*p, 0, n1 * sizeof(double), c.stream);
  }
  // supertile count is largest for the smallest tile height
  const long long ntx = (x_max + kTileW - 1) / kTileW;
  const long long nsx = (ntx + kTilesPerSuper - 1) / kTilesPerSuper;
  c.red_stride = nsx * ((y_max + 3) / 4) + 1;
  if (!check_cuda(cudaMalloc(&c.red_partials, 8 * c.red_stride * sizeof(double)),
                  "cudaMalloc partials") ||
      !check_cuda(cudaMalloc(&c.red_result, 8 * sizeof(double)),
                  "cudaMalloc result") ||
      !check_cuda(cudaMalloc(&c.red_counter, 8 * sizeof(unsigned int)),
                  "cudaMalloc counter") ||
      !check_cuda(cudaMallocHost(&c.host_result, 8 * sizeof(double)),
                  "cudaMallocHost") ||
      !check_cuda(cudaHostAlloc(&c.host_map, 9 * sizeof(unsigned long long),
                                cudaHostAllocMapped),
                  "cudaHostAlloc mapped") ||
      !check_cuda(cudaHostGetDevicePointer(&c.host_map_dev, c.host_map, 0),
                  "cudaHostGetDevicePointer"))
    return false;
  cudaMemsetAsync(c.red_counter, 0, 8 * sizeof(unsigned int), c.stream);
  cudaMemsetAsync(c.red_result, 0, 8 * sizeof(double), c.stream);
  return check_cuda(cudaStreamSynchronize(c.stream), "chunk allocation");
}

// Every entry point that works on the chunk first launches a PPCG inner step
// held back for pairing (flush_pending_inner), so what any call sees is
// what the reference's call sequence would have produced by then.
static bool need_chunk(const char* who) {
  if (!chunk().ready) {
    fail(5, "%s called before initialise_ocl_", who);
    return false;
  }
  flush_pending_inner(chunk());
  chunk().abi_calls++;
  return true;
}

bool ensure_alt_fields(Chunk& c) {
  if (c.r2.base) return true;
  if (!alloc_field(c, c.r2) || !alloc_field(c, c.sd2)) return false;
  // the halos (never written by the solve) must match the live pair's
  const size_t n = (size_t)((32 - (c.H % 32)) % 32 + c.rows * c.S + 32) * sizeof(double);
  return check_cuda(cudaMemcpyAsync(c.r2.base, c.r.base, n, cudaMemcpyDeviceToDevice, c.stream),
                    "alt r copy") &&
         check_cuda(cudaMemcpyAsync(c.sd2.base, c.sd.base, n, cudaMemcpyDeviceToDevice, c.stream),
                    "alt sd copy");
}

bool ensure_u_alt(Chunk& c) { return c.u2.base || alloc_field(c, c.u2); }

void swap_alt_fields(Chunk& c) {
  std::swap(c.r, c.r2);
  std::swap(c.sd, c.sd2);
  c.field_epoch++;
}

void flush_pending_inner(Chunk& c) {
  const int s = c.pending_inner;
  if (s < 0) return;
  c.pending_inner = -1;
  launch_ppcg_update_r(c);
  launch_ppcg_calc_sd(c, c.ppcg_alpha_h[s], c.ppcg_beta_h[s]);
}

// The next reduction launched copies its result to mapped host memory and
// then sets the ready word there (finish_reduction), so fetch can wait on
// that word instead of a copy and a stream synchronisation.
static void arm_host_result(Chunk& c) {
  __atomic_store_n(c.host_map + 8, 0ull, __ATOMIC_RELEASE);
  c.red_to_host = true;
}

// Returns the reduced values: every scalar-returning call is synchronous,
// like reduceValue (ocl_reduction.hpp:6-35).  After arm_host_result the
// host waits for the ready word (checking the stream for errors while it
// waits, and synchronising it after a long wait); otherwise it copies the
// result back and synchronises.
static bool fetch(int nv, double* out) {
  Chunk& c = chunk();
  if (c.red_to_host) {
    c.red_to_host = false;
    const unsigned long long* ready = c.host_map + 8;
    bool got = false;
    for (long long spin = 0; spin < (1ll << 22); spin++) {
      if (__atomic_load_n(ready, __ATOMIC_ACQUIRE) != 0ull) {
        got = true;
        break;
      }
      if ((spin & 1023) == 1023) {
        const cudaError_t e = cudaStreamQuery(c.stream);
        if (e != cudaSuccess && e != cudaErrorNotReady) {
          check_cuda(e, "reduction wait");
          break;
        }
        if (e == cudaSuccess) {  // the stream is idle: the word must be there
          got = __atomic_load_n(ready, __ATOMIC_ACQUIRE) != 0ull;
          break;
        }
      }
    }
    if (!got && check_cuda(cudaStreamSynchronize(c.stream), "reduction sync"))
      got = __atomic_load_n(ready, __ATOMIC_ACQUIRE) != 0ull;
    if (got) {
      for (int i = 0; i < nv; i++) {
        const unsigned long long b = __atomic_load_n(c.host_map + i, __ATOMIC_RELAXED);
        memcpy(&out[i], &b, sizeof(double));
      }
      return true;
    }
    if (error_code() == 0) fail(27, "reduction result did not arrive");
    for (int i = 0; i < nv; i++) out[i] = NAN;
    return false;
  }
  if (!check_cuda(cudaMemcpyAsync(c.host_result, c.red_result,
                                  nv * sizeof(double), cudaMemcpyDeviceToHost,
                                  c.stream),
                  "reduction read-back") ||
      !check_cuda(cudaStreamSynchronize(c.stream), "reduction sync")) {
    for (int i = 0; i < nv; i++) out[i] = NAN;
    return false;
  }
  for (int i = 0; i < nv; i++) out[i] = c.host_result[i];
  return true;
}

static Field* field_by_id(Chunk& c, int id) {
  switch (id) {
    case 1: return &c.density;
    case 2: return &c.energy0;
    case 3: return &c.energy1;
    case 4: return &c.u;
    case 5: return &c.p;
    case 6: return &c.sd;
    case 7: return &c.r;
    case 8: return &c.u0;
    case 9: return &c.w;
    case 10: return &c.z;
    case 11: return &c.Mi;
    case 12: return &c.Kx;
    case 13: return &c.Ky;
    case 14: return &c.cp;
    case 15: return &c.bfp;
    case 16: return &c.volume;
    default: return nullptr;
  }
}

static bool store_coefs(const double* a, const double* b, int n, double** ah,
                        double** bh) {
  free(*ah);
  free(*bh);
  *ah = (double*)malloc(sizeof(double) * (size_t)std::max(n, 1));
  *bh = (double*)malloc(sizeof(double) * (size_t)std::max(n, 1));
  if (!*ah || !*bh) {
    fail(6, "out of host memory for %d coefficients", n);
    return false;
  }
  if (n > 0) {
    memcpy(*ah, a, sizeof(double) * (size_t)n);
    memcpy(*bh, b, sizeof(double) * (size_t)n);
  }
  return true;
}

}  // namespace tea

using namespace tea;

// ===========================================================================
// Part 1: reference entry points
// ===========================================================================

extern "C" void initialise_ocl_(int* x_min, int* x_max, int* y_min, int* y_max) {
  Config cfg = g_config;
  if (!cfg.set && !config_from_tea_in(&cfg)) return;
  init_chunk(*x_max - *x_min + 1, *y_max - *y_min + 1, cfg);
}

extern "C" void initialise_chunk_kernel_ocl_(double* d_xmin, double* d_ymin,
                                             double* d_dx, double* d_dy) {
  if (!need_chunk("initialise_chunk_kernel_ocl_")) return;
  Chunk& c = chunk();
  c.celldx_h = *d_dx;
  c.celldy_h = *d_dy;
  launch_initialise_chunk(c, *d_xmin, *d_ymin, *d_dx, *d_dy);
  check_cuda(cudaStreamSynchronize(c.stream), "initialise_chunk");
}

extern "C" void generate_chunk_kernel_ocl_(
    const int* number_of_states, const double* state_density,
    const double* state_energy, const double* state_xmin,
    const double* state_xmax, const double* state_ymin,
    const double* state_ymax, const double* state_radius,
    const int* state_geometry, const int* g_rect, const int* g_circ,
    const int* g_point) {
  if (!need_chunk("generate_chunk_kernel_ocl_")) return;
  Chunk& c = chunk();
  launch_generate_init(c, state_density[0], state_energy[0]);
  for (int s = 1; s < *number_of_states; s++)
    launch_generate_state(c, state_density[s], state_energy[s], state_xmin[s],
                          state_xmax[s], state_ymin[s], state_ymax[s],
                          state_radius[s], state_geometry[s], *g_rect, *g_circ,
                          *g_point);
  launch_init_u(c, c.energy0.f);
}

extern "C" void set_field_kernel_ocl_(void) {
  if (!need_chunk("set_field_kernel_ocl_")) return;
  launch_set_field(chunk());
}

extern "C" void field_summary_kernel_ocl_(double* vol, double* mass, double* ie,
                                          double* temp) {
  double out[4] = {NAN, NAN, NAN, NAN};
  if (need_chunk("field_summary_kernel_ocl_")) {
    arm_host_result(chunk());
    launch_field_summary(chunk());
    fetch(4, out);
  }
  *vol = out[0];
  *mass = out[1];
  *ie = out[2];
  *temp = out[3];
}

extern "C" void update_halo_kernel_ocl_(const int* chunk_neighbours,
                                        const int* fields, const int* depth) {
  if (!need_chunk("update_halo_kernel_ocl_")) return;
  Chunk& c = chunk();
  for (int f = 0; f < 4; f++) {
    if (chunk_neighbours[f] != TEA_EXTERNAL_FACE) {
      fail(7, "update_halo_kernel_ocl_: only a single chunk (all faces "
              "external) is supported");
      return;
    }
  }
  if (*depth < 1 || *depth > c.H) {
    fail(7, "update_halo_kernel_ocl_: depth %d outside 1..%d", *depth, c.H);
    return;
  }
  const int mask = (fields[TEA_FIELD_DENSITY - 1] == 1 ? 1 : 0) |
                   (fields[TEA_FIELD_ENERGY0 - 1] == 1 ? 2 : 0) |
                   (fields[TEA_FIELD_ENERGY1 - 1] == 1 ? 4 : 0);
  launch_update_halo(c, mask, *depth);
}

extern "C" void tea_leaf_common_init_kernel_ocl_(const int* coefficient,
                                                 double* dt, double* rx,
                                                 double* ry, int* zero_boundary,
                                                 int* reflective_boundary) {
  if (!need_chunk("tea_leaf_common_init_kernel_ocl_")) return;
  Chunk& c = chunk();
  if (*coefficient != TEA_COEF_CONDUCTIVITY &&
      *coefficient != TEA_COEF_RECIP_CONDUCTIVITY) {
    fail(8, "Unknown coefficient %d passed to tea leaf", *coefficient);
    return;
  }
  // calcrxry (tea_leaf_kernel_ocl.cpp:8-32): celldx/celldy never change, so
  // the host copies kept at initialise_chunk time are used.
  const double dx = c.celldx_h, dy = c.celldy_h;
  *rx = *dt / (dx * dx);
  *ry = *dt / (dy * dy);
  launch_init_common(c, *coefficient, *rx, *ry);
  if (!*reflective_boundary) launch_zero_boundary(c, zero_boundary);
  launch_init_diag(c);
  launch_init_u(c, c.energy1.f);
}

extern "C" void tea_leaf_calc_residual_ocl_(void) {
  if (!need_chunk("tea_leaf_calc_residual_ocl_")) return;
  launch_calc_residual(chunk());
}

extern "C" void tea_leaf_calc_2norm_kernel_ocl_(int* norm_array, double* norm) {
  *norm = NAN;
  if (!need_chunk("tea_leaf_calc_2norm_kernel_ocl_")) return;
  Chunk& c = chunk();
  const double *a, *b;
  if (*norm_array == 0) {
    a = b = c.u0.f;
  } else if (*norm_array == 1) {
    a = b = c.r.f;
  } else if (*norm_array == 2) {
    a = c.r.f;
    b = (c.prec == PREC_NONE) ? c.r.f : c.z.f;
  } else {
    fail(9, "Invalid value '%d' for norm_array passed, should be 0 for u0, 1 "
            "for r, 2 for r*z",
         *norm_array);
    return;
  }
  arm_host_result(c);
  launch_dot(c, a, b);
  fetch(1, norm);
}

extern "C" void tea_leaf_cg_init_kernel_ocl_(double* rro) {
  *rro = NAN;
  if (!need_chunk("tea_leaf_cg_init_kernel_ocl_")) return;
  Chunk& c = chunk();
  if (c.solver == SOLVER_JACOBI) {
    fail(10, "tea_leaf_cg_init_kernel_ocl_ called with the Jacobi solver");
    return;
  }
  if (c.prec == PREC_JAC_BLOCK)
    launch_block_init(c);
  else if (c.prec == PREC_JAC_DIAG)
    launch_init_jac_diag(c);
  arm_host_result(c);
  launch_cg_init_p(c);
  fetch(1, rro);
}

extern "C" void tea_leaf_cg_calc_w_kernel_ocl_(double* pw) {
  *pw = NAN;
  if (!need_chunk("tea_leaf_cg_calc_w_kernel_ocl_")) return;
  arm_host_result(chunk());
  launch_cg_calc_w(chunk());
  fetch(1, pw);
}

extern "C" void tea_leaf_cg_calc_ur_kernel_ocl_(double* alpha, double* rrn) {
  const double a = *alpha;
  *rrn = NAN;
  if (!need_chunk("tea_leaf_cg_calc_ur_kernel_ocl_")) return;
  Chunk& c = chunk();
  arm_host_result(c);
  // In a PPCG solve the next call is normally tea_leaf_ppcg_init_sd_kernel_ocl_
  // (tea_solve.f90:247-249, :422-475), which forms sd = M^-1 r / theta from
  // the r and z made here.  This pass forms it too, from its own z, into the
  // spare sd buffer; init_sd then only makes that buffer current, provided no
  // other call came in between (the current sd is untouched until then).
  if (c.solver == SOLVER_PPCG && c.n_ppcg > 0 && ensure_alt_fields(c)) {
    launch_cg_calc_ur_sd(c, a, c.ppcg_theta, c.sd2.f);
    c.spec_sd_call = c.abi_calls;
    c.spec_sd_theta = c.ppcg_theta;
    c.spec_sd_arith = c.arith;
  } else {
    launch_cg_calc_ur(c, a);
  }
  fetch(1, rrn);
}

extern "C" void tea_leaf_cg_calc_p_kernel_ocl_(double* beta) {
  if (!need_chunk("tea_leaf_cg_calc_p_kernel_ocl_")) return;
  launch_cg_calc_p(chunk(), *beta);
}

extern "C" void tea_leaf_cheby_init_kernel_ocl_(const double* ch_alphas,
                                                const double* ch_betas,
                                                int* n_coefs, const double* rx,
                                                const double* ry,
                                                const double* theta) {
  (void)rx;
  (void)ry;
  if (!need_chunk("tea_leaf_cheby_init_kernel_ocl_")) return;
  Chunk& c = chunk();
  if (!store_coefs(ch_alphas, ch_betas, *n_coefs, &c.cheby_alpha_h,
                   &c.cheby_beta_h))
    return;
  c.n_cheby = *n_coefs;
  c.cheby_theta = *theta;
  launch_cheby_init_p(c, *theta);
  launch_cheby_calc_u(c);
}

extern "C" void tea_leaf_cheby_iterate_kernel_ocl_(const int* cheby_calc_step) {
  if (!need_chunk("tea_leaf_cheby_iterate_kernel_ocl_")) return;
  Chunk& c = chunk();
  const int s = *cheby_calc_step - 1;
  if (s < 0 || s >= c.n_cheby) {
    fail(11, "Chebyshev step %d outside the %d stored coefficients",
         *cheby_calc_step, c.n_cheby);
    return;
  }
  if (c.prec == PREC_JAC_BLOCK) {
    // calc_u folded into calc_p: the new u goes to the second buffer,
    // which then becomes u
    if (!ensure_u_alt(c)) return;
    launch_cheby_calc_pu(c, c.cheby_alpha_h[s], c.cheby_beta_h[s], c.u2.f);
    std::swap(c.u, c.u2);
    c.field_epoch++;
    return;
  }
  launch_cheby_calc_p(c, c.cheby_alpha_h[s], c.cheby_beta_h[s]);
  launch_cheby_calc_u(c);
}

extern "C" void tea_leaf_ppcg_init_ocl_(const double* ch_alphas,
                                        const double* ch_betas, double* theta,
                                        int* n_inner_steps) {
  if (!need_chunk("tea_leaf_ppcg_init_ocl_")) return;
  Chunk& c = chunk();
  if (!store_coefs(ch_alphas, ch_betas, *n_inner_steps, &c.ppcg_alpha_h,
                   &c.ppcg_beta_h))
    return;
  c.n_ppcg = *n_inner_steps;
  c.ppcg_theta = *theta;
}

extern "C" void tea_leaf_ppcg_init_sd_kernel_ocl_(void) {
  if (!need_chunk("tea_leaf_ppcg_init_sd_kernel_ocl_")) return;
  Chunk& c = chunk();
  // the sd the last calc_ur formed, if this call directly follows it
  if (c.spec_sd_call >= 0 && c.abi_calls == c.spec_sd_call + 1 &&
      c.spec_sd_theta == c.ppcg_theta && c.spec_sd_arith == c.arith) {
    c.spec_sd_call = -1;
    std::swap(c.sd, c.sd2);
    c.field_epoch++;
    return;
  }
  launch_ppcg_init_sd(c, c.ppcg_theta);
}

extern "C" void tea_leaf_ppcg_inner_kernel_ocl_(int* inner_step,
                                                int* bounds_extra,
                                                const int* chunk_neighbours) {
  (void)bounds_extra;
  Chunk& c = chunk();
  if (!c.ready) {
    fail(5, "tea_leaf_ppcg_inner_kernel_ocl_ called before initialise_ocl_");
    return;
  }
  for (int f = 0; f < 4; f++) {
    if (chunk_neighbours[f] != TEA_EXTERNAL_FACE) {
      flush_pending_inner(c);
      fail(7, "tea_leaf_ppcg_inner_kernel_ocl_: only a single chunk (all "
              "faces external) is supported");
      return;
    }
  }
  const int s = *inner_step - 1;
  if (s < 0 || s >= c.n_ppcg) {
    flush_pending_inner(c);
    fail(11, "PPCG inner step %d outside the %d stored coefficients",
         *inner_step, c.n_ppcg);
    return;
  }
  // Steps are paired: a step that a later one may follow is held back, and
  // when the next step arrives the two run as one fused pass
  // (tea_ppcg_tb.cu); any other call launches a held step first.  The
  // results are those of one update_r + calc_sd per call.
  if (tb_applicable(c)) {
    if (c.pending_inner >= 0 && c.pending_inner == s - 1) {
      c.pending_inner = -1;
      if (!ensure_alt_fields(c) ||
          !launch_ppcg_inner_pair(c, s - 1, nullptr, c.r.f, c.sd.f, c.r2.f, c.sd2.f))
        return;
      swap_alt_fields(c);
      return;
    }
    flush_pending_inner(c);
    if (s + 1 < c.n_ppcg) {
      c.pending_inner = s;
      return;
    }
  }
  flush_pending_inner(c);
  if (c.prec == PREC_JAC_BLOCK) {
    // update_r and calc_sd in one pass (k_ppcg_step): the new sd goes to
    // the second buffer, which then becomes sd
    if (!ensure_alt_fields(c)) return;
    launch_ppcg_step(c, c.ppcg_alpha_h[s], c.ppcg_beta_h[s], c.sd.f, c.sd2.f);
    std::swap(c.sd, c.sd2);
    c.field_epoch++;
    return;
  }
  launch_ppcg_update_r(c);
  launch_ppcg_calc_sd(c, c.ppcg_alpha_h[s], c.ppcg_beta_h[s]);
}

extern "C" void tea_leaf_jacobi_solve_kernel_ocl_(double* error) {
  *error = NAN;
  if (!need_chunk("tea_leaf_jacobi_solve_kernel_ocl_")) return;
  Chunk& c = chunk();
  launch_jacobi_copy_u(c);
  arm_host_result(c);
  launch_jacobi_solve(c);
  fetch(1, error);
}

extern "C" void tea_leaf_common_finalise_kernel_ocl_(void) {
  if (!need_chunk("tea_leaf_common_finalise_kernel_ocl_")) return;
  launch_finalise(chunk());
}

extern "C" void print_opencl_profiling_info_(void) {
  Chunk& c = chunk();
  if (!c.profiler_on) return;
  // one row per kernel name, in name order, in the reference's layout
  // (ocl_errors.cpp:207-228)
  fprintf(stdout, "@@@@@ CUDA Profiling information @@@@@\n");
  for (auto& kv : g_prof) {
    if (kv.second.calls)
      fprintf(stdout, "%30s : %10.3f ms (%.2f \xce\xbcs avg. over %lld calls)\n",
              kv.first.c_str(), kv.second.ms,
              1e3 * kv.second.ms / (double)kv.second.calls, kv.second.calls);
  }
  fflush(stdout);
}

static void pack_unpack(int* fields, const char* who) {
  int n = 0;
  for (int i = 0; i < 7; i++) n += fields[i];
  if (n < 1) return;  // nothing exchanged, as ocl_pack.cpp:24-29
  fail(12, "%s: MPI halo exchange is not supported (single chunk)", who);
}

extern "C" void ocl_pack_buffers_(int* fields, int* offsets, int* depth,
                                  int* face, double* host_buffer) {
  (void)offsets;
  (void)depth;
  (void)face;
  (void)host_buffer;
  pack_unpack(fields, "ocl_pack_buffers_");
}

extern "C" void ocl_unpack_buffers_(int* fields, int* offsets, int* depth,
                                    int* face, double* host_buffer) {
  (void)offsets;
  (void)depth;
  (void)face;
  (void)host_buffer;
  pack_unpack(fields, "ocl_unpack_buffers_");
}

// ===========================================================================
// Part 2: additions
// ===========================================================================

extern "C" int tea_gb300_configure(int halo_depth, int solver,
                                   int preconditioner, int profiler_on) {
  if (halo_depth < 1 || solver < 1 || solver > 4 || preconditioner < 1 ||
      preconditioner > 3)
    return -1;
  g_config.set = true;
  g_config.halo = halo_depth;
  g_config.solver = solver;
  g_config.prec = preconditioner;
  g_config.profiler = profiler_on;
  return 0;
}

extern "C" void tea_gb300_set_abort_on_error(int a) { g_abort_on_error = a; }

extern "C" int tea_gb300_set_arithmetic(int form) {
  if (form < 0 || form > 2) {
    fail(3, "tea_gb300_set_arithmetic: form %d is not 0 (exact), 1 (fused) or 2 (chain)",
         form);
    return -1;
  }
  if (chunk().ready) flush_pending_inner(chunk());  // a held step keeps its form
  g_config.arith = form;
  chunk().arith = form;
  return 0;
}

extern "C" int tea_gb300_get_arithmetic(void) { return chunk().arith; }

extern "C" int tea_gb300_set_resident_mode(int mode) {
  if (mode < 0 || mode > 2) {
    fail(3, "tea_gb300_set_resident_mode: mode %d is not 0 (auto), 1 (graph) or 2 "
            "(persistent)", mode);
    return -1;
  }
  g_config.resident_mode = mode;
  chunk().resident_mode = mode;
  return 0;
}

extern "C" int tea_gb300_set_inner_pairs(int on) {
  if (on != 0 && on != 1) {
    fail(3, "tea_gb300_set_inner_pairs: %d is not 0 or 1", on);
    return -1;
  }
  if (chunk().ready) flush_pending_inner(chunk());
  g_config.inner_pairs = chunk().inner_pairs = on;
  return 0;
}

extern "C" int tea_gb300_set_barrier_limits(long long spin_limit, int extra_arrivals) {
  if (spin_limit < 1 || extra_arrivals < 0 || extra_arrivals > 1) {
    fail(3, "tea_gb300_set_barrier_limits: spin limit %lld, extra arrivals %d", spin_limit,
         extra_arrivals);
    return -1;
  }
  g_config.barrier_spin_limit = chunk().barrier_spin_limit = spin_limit;
  g_config.barrier_extra = chunk().barrier_extra = extra_arrivals;
  return 0;
}

extern "C" int tea_gb300_last_error(char* msg, int len) {
  const int code = g_err_code;
  if (msg && len > 0) {
    strncpy(msg, g_err_msg.c_str(), (size_t)len - 1);
    msg[len - 1] = 0;
  }
  g_err_code = 0;
  g_err_msg.clear();
  return code;
}

extern "C" void tea_gb300_finalise(void) { free_chunk(chunk()); }

static int copy_field(int id, double* host, const double* in, bool padded) {
  if (!need_chunk("field access")) return -1;
  Chunk& c = chunk();
  Field* f = field_by_id(c, id);
  if (!f) {
    fail(13, "unknown field %d", id);
    return -1;
  }
  const int off = padded ? 0 : c.H;
  const int w = padded ? c.x_max + 2 * c.H : c.x_max;
  const int h = padded ? c.y_max + 2 * c.H : c.y_max;
  double* dev = f->f + (long long)off * c.S + off;
  cudaError_t e;
  if (in)
    e = cudaMemcpy2DAsync(dev, c.S * sizeof(double), in, w * sizeof(double),
                          w * sizeof(double), h, cudaMemcpyHostToDevice,
                          c.stream);
  else
    e = cudaMemcpy2DAsync(host, w * sizeof(double), dev, c.S * sizeof(double),
                          w * sizeof(double), h, cudaMemcpyDeviceToHost,
                          c.stream);
  if (!check_cuda(e, "field copy")) return -1;
  // the second r/sd buffer keeps the same halo (the fused PPCG inner steps
  // read halos from whichever buffer is live)
  Field* alt = f == &c.r ? &c.r2 : f == &c.sd ? &c.sd2 : nullptr;
  if (in && padded && alt && alt->base &&
      !check_cuda(cudaMemcpy2DAsync(alt->f, c.S * sizeof(double), in, w * sizeof(double),
                                    w * sizeof(double), h, cudaMemcpyHostToDevice, c.stream),
                  "field copy (second buffer)"))
    return -1;
  // the stored diagonal follows the face coefficients
  if (in && (id == 12 || id == 13)) launch_init_diag(c);
  return check_cuda(cudaStreamSynchronize(c.stream), "field copy sync") ? 0 : -1;
}

extern "C" int tea_gb300_read_field(int field, double* out) {
  return copy_field(field, out, nullptr, false);
}
extern "C" int tea_gb300_write_field(int field, const double* in) {
  return copy_field(field, nullptr, in, false);
}
extern "C" int tea_gb300_read_field_padded(int field, double* out) {
  return copy_field(field, out, nullptr, true);
}
extern "C" int tea_gb300_write_field_padded(int field, const double* in) {
  return copy_field(field, nullptr, in, true);
}

extern "C" int tea_gb300_reduction_rows(int x_max, int y_max) {
  return reduction_rows(x_max, y_max);
}

extern "C" long long tea_gb300_kernel_launches(void) { return g_launches; }

extern "C" void* tea_gb300_stream(void) {
  if (chunk().ready) flush_pending_inner(chunk());
  return (void*)chunk().stream;
}

extern "C" int tea_gb300_chunk_info(int* x_max, int* y_max, int* halo,
                                    int* stride) {
  Chunk& c = chunk();
  if (!c.ready) return -1;
  *x_max = c.x_max;
  *y_max = c.y_max;
  *halo = c.H;
  *stride = (int)c.S;
  return 0;
}

static cudaEvent_t g_events[16] = {nullptr};

extern "C" int tea_gb300_event_record(int slot) {
  Chunk& c = chunk();
  if (slot < 0 || slot >= 16 || !c.ready) return -1;
  flush_pending_inner(c);
  if (!g_events[slot] && !check_cuda(cudaEventCreate(&g_events[slot]), "cudaEventCreate"))
    return -1;
  return check_cuda(cudaEventRecord(g_events[slot], c.stream), "cudaEventRecord") ? 0 : -1;
}

extern "C" float tea_gb300_event_elapsed_ms(int a, int b) {
  if (a < 0 || a >= 16 || b < 0 || b >= 16 || !g_events[a] || !g_events[b]) return -1.0f;
  if (!check_cuda(cudaEventSynchronize(g_events[b]), "cudaEventSynchronize")) return -1.0f;
  float ms = -1.0f;
  if (!check_cuda(cudaEventElapsedTime(&ms, g_events[a], g_events[b]), "cudaEventElapsedTime"))
    return -1.0f;
  return ms;
}

extern "C" int tea_gb300_synchronize(void) {
  Chunk& c = chunk();
  if (!c.ready) return -1;
  flush_pending_inner(c);
  return check_cuda(cudaStreamSynchronize(c.stream), "cudaStreamSynchronize") ? 0 : -1;
}

extern "C" void* tea_gb300_host_alloc(size_t bytes) {
  void* p = nullptr;
  if (!check_cuda(cudaMallocHost(&p, bytes), "cudaMallocHost")) return nullptr;
  return p;
}

extern "C" void tea_gb300_host_free(void* p) { cudaFreeHost(p); }

extern "C" int tea_gb300_kernel_timer_select(const char* name) {
  timed_drain();
  g_timed_name = name ? name : "";
  g_timed.clear();
  return 0;
}

extern "C" int tea_gb300_kernel_timer_read(double* total_ms, long long* launches) {
  timed_drain();
  double ms = 0.0;
  long long n = 0;
  for (auto& kv : g_timed) {
    ms += kv.second.ms;
    n += kv.second.calls;
  }
  *total_ms = ms;
  *launches = n;
  return 0;
}

extern "C" int tea_gb300_kernel_timer_read_name(const char* name, double* total_ms,
                                                long long* launches) {
  timed_drain();
  auto it = g_timed.find(name ? name : "");
  *total_ms = it == g_timed.end() ? 0.0 : it->second.ms;
  *launches = it == g_timed.end() ? 0 : it->second.calls;
  return 0;
}

extern "C" double tea_gb300_fp64_rate(void) { return measure_fp64_rate(); }
