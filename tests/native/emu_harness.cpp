// Host build of the integer FP64 add and multiply of tea_emu.cuh, for
// checking them against the host's IEEE arithmetic on the CPU.  The CUDA
// intrinsics the header uses are given host definitions here; the
// hardware fallbacks become the host's own correctly rounded + and *
// (built with -ffp-contract=off).
#include <cstdint>
#include <cstring>

#define __device__
#define __forceinline__ inline
static inline long long __double_as_longlong(double d) {
  long long r;
  std::memcpy(&r, &d, 8);
  return r;
}
static inline double __longlong_as_double(long long v) {
  double r;
  std::memcpy(&r, &v, 8);
  return r;
}
static inline double __dadd_rn(double a, double b) { return a + b; }
static inline double __dmul_rn(double a, double b) { return a * b; }
static inline int __clzll(long long v) { return __builtin_clzll((unsigned long long)v); }
static inline float __frcp_rn(float v) { return 1.0f / v; }
static inline unsigned long long __float2ull_rz(float v) { return (unsigned long long)v; }
static inline unsigned long long __umul64hi(unsigned long long a, unsigned long long b) {
  return (unsigned long long)(((unsigned __int128)a * b) >> 64);
}

#include "tea_emu.cuh"

extern "C" void emu_add_n(const double* a, const double* b, double* o, long n) {
  for (long i = 0; i < n; i++) o[i] = tea::emu_dadd(a[i], b[i]);
}

extern "C" void emu_mul_n(const double* a, const double* b, double* o, long n) {
  for (long i = 0; i < n; i++) o[i] = tea::emu_dmul(a[i], b[i]);
}

extern "C" void emu_div_n(const double* a, double y, double* o, long n) {
  const tea::DivConst k = tea::div_const(y);
  for (long i = 0; i < n; i++) o[i] = tea::emu_ddiv(a[i], k);
}

extern "C" void emu_divv_n(const double* a, const double* b, double* o, long n) {
  for (long i = 0; i < n; i++) o[i] = tea::emu_ddiv_var(a[i], b[i]);
}
