// Shared device/host helpers for the ceviche GB300 Yee-stencil library.
#pragma once
#include <initializer_list>

#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <string>

#include "cevgpu.h"

namespace cev {

// ------------------------------------------------------------------ errors
void set_error(const char* fmt, ...);
int cuda_status(cudaError_t e, const char* where);

#define CEV_CUDA(call)                                                   \
  do {                                                                   \
    cudaError_t _e = (call);                                             \
    if (_e != cudaSuccess) return ::cev::cuda_status(_e, #call);         \
  } while (0)

#define CEV_CHECK_LAUNCH(where)                                          \
  do {                                                                   \
    cudaError_t _e = cudaGetLastError();                                 \
    if (_e != cudaSuccess) return ::cev::cuda_status(_e, where);         \
  } while (0)

#define CEV_REQUIRE(cond, ...)                                           \
  do {                                                                   \
    if (!(cond)) {                                                       \
      ::cev::set_error(__VA_ARGS__);                                     \
      return CEV_ERR_INVALID;                                            \
    }                                                                    \
  } while (0)

// ------------------------------------------------------------ complex math
template <typename R> struct CplxOf;
template <> struct CplxOf<float> { using T = float2; };
template <> struct CplxOf<double> { using T = double2; };
template <typename R> using Cplx = typename CplxOf<R>::T;

template <typename C> __host__ __device__ __forceinline__ C cmk(double re, double im) {
  C c;
  c.x = re;
  c.y = im;
  return c;
}
template <typename C> __host__ __device__ __forceinline__ C cadd(C a, C b) {
  C c; c.x = a.x + b.x; c.y = a.y + b.y; return c;
}
template <typename C> __host__ __device__ __forceinline__ C csub(C a, C b) {
  C c; c.x = a.x - b.x; c.y = a.y - b.y; return c;
}
template <typename C> __host__ __device__ __forceinline__ C cmul(C a, C b) {
  C c; c.x = a.x * b.x - a.y * b.y; c.y = a.x * b.y + a.y * b.x; return c;
}
// conj(a) * b
template <typename C> __host__ __device__ __forceinline__ C cmulc(C a, C b) {
  C c; c.x = a.x * b.x + a.y * b.y; c.y = a.x * b.y - a.y * b.x; return c;
}
template <typename C, typename R> __host__ __device__ __forceinline__ C cscale(C a, R s) {
  C c; c.x = a.x * s; c.y = a.y * s; return c;
}
template <typename C> __host__ __device__ __forceinline__ C cconj(C a) {
  C c; c.x = a.x; c.y = -a.y; return c;
}
// a + b*c
template <typename C> __host__ __device__ __forceinline__ C cfma(C b, C c, C a) {
  C r;
  r.x = a.x + b.x * c.x - b.y * c.y;
  r.y = a.y + b.x * c.y + b.y * c.x;
  return r;
}

__host__ __device__ __forceinline__ float2 to_f(double2 a) { return make_float2((float)a.x, (float)a.y); }
__host__ __device__ __forceinline__ double2 to_d(float2 a) { return make_double2(a.x, a.y); }

// -------------------------------------------------------- warp reductions
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ float warp_sumf(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Number of SMs of the current device (cached per device).
int sm_count();
// Allows `bytes` of dynamic shared memory for kernel `fn` on the current
// device (set once per device and kernel; thread-safe), and with carveout >= 0
// the preferred shared-memory carve-out in percent.
int allow_dynamic_smem(const void* fn, int bytes, int carveout = -1);
// Device memory from the current device's default stream-ordered pool, which
// keeps up to 256 MB of freed blocks for reuse: objects created and destroyed
// in a loop (an FDTD plan per design iteration) then allocate without a driver
// call.  Free with dev_free_all.
int dev_alloc(void** p, size_t bytes, cudaStream_t s);
// Waits for the device (as cudaFree does) and returns dev_alloc blocks to the pool.
void dev_free_all(std::initializer_list<void*> ps);

inline unsigned ceil_div(size_t a, size_t b) { return (unsigned)((a + b - 1) / b); }

}  // namespace cev
