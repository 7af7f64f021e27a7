// Probe accumulation for ceviche.utils.measure_fields (utils.py:316-332):
// measured[t, p] = sum over the probe's cells of field[t] * probe_p, on the
// device, so a time series of weighted field sums needs no per-step copy.
//
// Probes are given as a CSR of their non-zero cells (probe_ptr[p] ..
// probe_ptr[p+1] index cell[] / weight[]).  One CTA reduces one (row, probe)
// pair in FP64 with a fixed reduction tree, so the result does not depend on
// scheduling.
#include "common.cuh"
#include "reduce.cuh"

namespace cev {

template <typename R>
__global__ void __launch_bounds__(RED_THREADS) k_probe_dot(int n_probe, const int* __restrict__ pptr,
                                                         const int* __restrict__ cell,
                                                         const double* __restrict__ w,
                                                         const R* __restrict__ field,
                                                         long long fstride, double* __restrict__ out,
                                                         long long ostride) {
  const int p = blockIdx.x;
  const long long row = blockIdx.y;
  const R* f = field + row * fstride;
  double acc = 0.0;
  for (int q = pptr[p] + threadIdx.x; q < pptr[p + 1]; q += blockDim.x)
    acc += w[q] * (double)f[cell[q]];
  __shared__ double sm[32];
  double v[1] = {acc};
  block_sum<1>(v, sm);
  if (threadIdx.x == 0) out[row * ostride + p] = v[0];
}

}  // namespace cev

using namespace cev;

extern "C" {

int cev_probe_measure(int n_probe, const int* probe_ptr, const int* cell, const double* weight,
                      const void* field, int field_is_f64, int nrows, long long field_stride,
                      double* out, long long out_stride, cudaStream_t s) {
  CEV_REQUIRE(n_probe >= 0 && nrows >= 0, "bad sizes n_probe=%d nrows=%d", n_probe, nrows);
  if (n_probe == 0 || nrows == 0) return CEV_OK;
  CEV_REQUIRE(probe_ptr && cell && weight && field && out, "NULL argument");
  CEV_REQUIRE(nrows <= 65535, "at most 65535 rows per call (got %d)", nrows);
  CEV_REQUIRE(out_stride >= n_probe && field_stride >= 0, "bad strides");
  const dim3 g(n_probe, nrows);
  if (field_is_f64)
    k_probe_dot<double><<<g, RED_THREADS, 0, s>>>(n_probe, probe_ptr, cell, weight,
                                                  (const double*)field, field_stride, out, out_stride);
  else
    k_probe_dot<float><<<g, RED_THREADS, 0, s>>>(n_probe, probe_ptr, cell, weight,
                                                 (const float*)field, field_stride, out, out_stride);
  CEV_CHECK_LAUNCH("k_probe_dot");
  return CEV_OK;
}

}  // extern "C"
