// tea_gb300_dot_noalloc: the fixed-order dot product of two padded fields
// for callers that cannot allocate GPU memory.
//
// Who needs it: a host program whose GPU memory is already claimed by
// another allocator (a framework's caching pool, or a fixed budget handed
// out up front), or a code path that must not call cudaMalloc for latency
// or failure-handling reasons.  Such a caller owns its input and output
// buffers but cannot give the reduction its scratch (per-supertile partial
// sums and a completion counter).  Here that scratch is a file-scope
// device array, sized for at most kNoAllocMaxPartials supertiles (512 KiB),
// which every GPU that loads the library holds until the process exits.
//
// The summation order, the arithmetic form and the result are those of
// tea_leaf_calc_2norm_kernel_ocl_ (k_dot in tea_kernels.cu) for the same
// values: the same tile walk and the same last-block finish.
#include <stdio.h>
#include <string.h>

#include "../../include/tealeaf_gb300.h"
#include "tea_device.cuh"

namespace tea {

// Largest supported number of supertiles (8 x 32 columns by 16 or 4 rows):
// enough for a 16384 x 16384 interior.
constexpr long long kNoAllocMaxPartials = 65536;

// The scratch: partial sums in [0, kNoAllocMaxPartials), the completion
// counter in the element after them.  Shared by every call on a device.
static __device__ __align__(256) double g_noalloc_scratch[kNoAllocMaxPartials + 32];

template <int TH, int F>
__global__ void __launch_bounds__(kBlock)
    k_dot_noalloc(Dev d, Red red, const double* a, const double* b) {
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

// Device address of the scratch array, looked up once per device.  The
// array's name in host code is only a stand-in for the symbol, never a
// usable address.  The table is filled without locking: the first call on
// each device should come from one host thread (two threads racing there
// would both store the same address).
static double* g_scratch_addr[64] = {nullptr};

static double* scratch_for_current_device() {
  int dev = 0;
  if (!check_cuda(cudaGetDevice(&dev), "cudaGetDevice")) return nullptr;
  if (dev < 0 || dev >= 64) {
    fail(30, "tea_gb300_dot_noalloc: device ordinal %d not supported", dev);
    return nullptr;
  }
  if (!g_scratch_addr[dev]) {
    void* p = nullptr;
    if (!check_cuda(cudaGetSymbolAddress(&p, g_noalloc_scratch),
                    "cudaGetSymbolAddress (no-alloc scratch)"))
      return nullptr;
    g_scratch_addr[dev] = (double*)p;
  }
  return g_scratch_addr[dev];
}

template <int TH, int F>
static int launch_dot_noalloc(const Dev& d, const Red& red, const double* a,
                              const double* b, cudaStream_t s) {
  int dev = 0, sms = 0, per_sm = 0;
  if (!check_cuda(cudaGetDevice(&dev), "tea_gb300_dot_noalloc: cudaGetDevice") ||
      !check_cuda(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev),
                  "tea_gb300_dot_noalloc: SM count"))
    return -1;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(
          &per_sm, k_dot_noalloc<TH, F>, kBlock, 0) != cudaSuccess ||
      per_sm < 1)
    per_sm = 1;
  long long grid = (long long)sms * per_sm;
  if (grid > d.ns) grid = d.ns;
  if (grid < 1) grid = 1;
  k_dot_noalloc<TH, F><<<(int)grid, kBlock, 0, s>>>(d, red, a, b);
  count_launch("tea_gb300_dot_noalloc");
  return check_cuda(cudaGetLastError(), "tea_gb300_dot_noalloc launch") ? 0 : -1;
}

}  // namespace tea

using namespace tea;

extern "C" int tea_gb300_dot_noalloc(const double* a, const double* b,
                                     int x_max, int y_max, int halo,
                                     long long stride, double* result,
                                     void* stream) {
  if (!a || !b || !result || x_max < 1 || y_max < 1 || halo < 1 ||
      stride < (long long)x_max + 2 * halo) {
    fail(31, "tea_gb300_dot_noalloc: invalid arguments");
    return -1;
  }
  const int TH = reduction_rows(x_max, y_max);
  Dev d;
  memset(&d, 0, sizeof(d));
  d.x_max = x_max;
  d.y_max = y_max;
  d.H = halo;
  d.S = stride;
  d.ntx = (x_max + kTileW - 1) / kTileW;
  d.nsx = (d.ntx + kTilesPerSuper - 1) / kTilesPerSuper;
  d.nty = (y_max + TH - 1) / TH;
  d.ns = d.nsx * d.nty;
  if ((long long)d.nsx * d.nty > kNoAllocMaxPartials) {
    fail(32,
         "tea_gb300_dot_noalloc: a %d x %d interior has %lld supertiles "
         "(ceil(ceil(x/32)/8) x ceil(y/%d)), more than the %lld partial sums "
         "of the fixed scratch (16384 x 16384 cells fit)",
         x_max, y_max, (long long)d.nsx * d.nty, TH, kNoAllocMaxPartials);
    return -1;
  }
  double* scratch = scratch_for_current_device();
  if (!scratch) return -1;
  cudaStream_t s = (cudaStream_t)stream;
  // the completion counter must start at zero; the partials are all written
  // before they are read
  unsigned int* counter = (unsigned int*)(scratch + kNoAllocMaxPartials);
  if (!check_cuda(cudaMemsetAsync(counter, 0, sizeof(unsigned int), s),
                  "tea_gb300_dot_noalloc counter reset"))
    return -1;
  Red red;
  red.partials = scratch;
  red.stride = kNoAllocMaxPartials;
  red.counter = counter;
  red.result = result;
  const bool fused = tea_gb300_get_arithmetic() != 0;
  if (TH == 16)
    return fused ? launch_dot_noalloc<16, 1>(d, red, a, b, s)
                 : launch_dot_noalloc<16, 0>(d, red, a, b, s);
  return fused ? launch_dot_noalloc<4, 1>(d, red, a, b, s)
               : launch_dot_noalloc<4, 0>(d, red, a, b, s);
}
