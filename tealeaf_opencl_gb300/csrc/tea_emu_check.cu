// tea_gb300_emu_check: the integer-pipe FP64 arithmetic of tea_emu.cuh,
// built for the GPU exactly as the solver kernels build it, compared bit for
// bit with the GPU's own FP64 instructions on caller-supplied operands.
//
// Every FP64 stencil kernel of the solve takes some of its multiplies and
// divisions from tea_emu.cuh and is bit-exact against the oracle only if
// those give the correctly rounded result for every operand.  The host
// build of the header is checked against numpy; this entry point checks the
// device build against __dmul_rn, __ddiv_rn and __dadd_rn on the same GPU.
#include <stdio.h>

#include "../../include/tealeaf_gb300.h"
#include "tea_emu.cuh"
#include "tea_internal.h"

namespace tea {

__global__ void k_emu_check(int op, const double* __restrict__ a,
                            const double* __restrict__ b, long long n, DivConst k,
                            unsigned long long* count, long long* first) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const double x = a[i];
    double want, got;
    if (op == TEA_EMU_MUL) {
      const double y = b[i];
      want = __dmul_rn(x, y);
      got = emu_dmul(x, y);
    } else if (op == TEA_EMU_DIV_INVARIANT) {
      want = __ddiv_rn(x, k.y);
      got = emu_ddiv(x, k);
    } else if (op == TEA_EMU_DIV) {
      const double y = b[i];
      want = __ddiv_rn(x, y);
      got = emu_ddiv_var(x, y);
    } else {
      const double y = b[i];
      want = __dadd_rn(x, y);
      got = emu_dadd(x, y);
    }
    const unsigned long long wb = (unsigned long long)__double_as_longlong(want);
    const unsigned long long gb = (unsigned long long)__double_as_longlong(got);
    const bool both_nan = want != want && got != got;
    if (wb != gb && !both_nan) {
      atomicAdd(count, 1ull);
      atomicMin((unsigned long long*)first, (unsigned long long)i);
    }
  }
}

}  // namespace tea

using namespace tea;

extern "C" int tea_gb300_emu_check(int op, const double* a, const double* b,
                                   long long n, double divisor,
                                   long long* mismatches, long long* first_mismatch) {
  if (op < TEA_EMU_MUL || op > TEA_EMU_ADD || !a || n < 0 || !mismatches ||
      !first_mismatch || (op != TEA_EMU_DIV_INVARIANT && !b)) {
    fail(33, "tea_gb300_emu_check: invalid arguments");
    return -1;
  }
  *mismatches = 0;
  *first_mismatch = -1;
  if (n == 0) return 0;
  unsigned long long* dev = nullptr;  // [0] count, [1] first index
  if (!check_cuda(cudaMalloc(&dev, 2 * sizeof(unsigned long long)), "emu check alloc"))
    return -1;
  const unsigned long long init[2] = {0ull, ~0ull};
  int rc = -1;
  if (check_cuda(cudaMemcpy(dev, init, sizeof(init), cudaMemcpyHostToDevice),
                 "emu check init")) {
    int sms = 0, d = 0;
    cudaGetDevice(&d);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, d);
    long long blocks = (n + 255) / 256;
    const long long cap = (long long)(sms > 0 ? sms : 1) * 8;
    if (blocks > cap) blocks = cap;
    k_emu_check<<<(int)blocks, 256>>>(op, a, b, n, div_const(divisor), dev,
                                       (long long*)(dev + 1));
    count_launch("tea_gb300_emu_check");
    unsigned long long out[2];
    if (check_cuda(cudaGetLastError(), "emu check launch") &&
        check_cuda(cudaMemcpy(out, dev, sizeof(out), cudaMemcpyDeviceToHost),
                   "emu check result")) {
      *mismatches = (long long)out[0];
      *first_mismatch = out[0] ? (long long)out[1] : -1;
      rc = 0;
    }
  }
  cudaFree(dev);
  return rc;
}
