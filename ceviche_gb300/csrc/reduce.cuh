// Deterministic block / grid reductions shared by the Krylov operators.
#pragma once

#include "krylov.hpp"

namespace cev {

static constexpr int RED_THREADS = 256;

// --------------------------------------------------------------- reductions
// Block-wide sum of NV doubles per thread into out (valid in thread 0).
template <int NV>
__device__ __forceinline__ void block_sum(double (&v)[NV], double* smem /* NV*32 */) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int nw = (blockDim.x * blockDim.y + 31) >> 5;
#pragma unroll
  for (int k = 0; k < NV; ++k) v[k] = warp_sum(v[k]);
  __syncthreads();
  if (lane == 0)
#pragma unroll
    for (int k = 0; k < NV; ++k) smem[k * 32 + warp] = v[k];
  __syncthreads();
  if (warp == 0) {
#pragma unroll
    for (int k = 0; k < NV; ++k) {
      double t = lane < nw ? smem[k * 32 + lane] : 0.0;
      v[k] = warp_sum(t);
    }
  }
}

// Block-wide sum of NV floats per thread: FP32 warp shuffles (the GB300 FP64
// pipe is narrow), then the per-warp sums combined in FP64 by thread k < NV.
// Result for value k in out[k] (valid in threads k < NV after the call).
template <int NV>
__device__ __forceinline__ void block_sum_f(float (&v)[NV], float* smem /* NV*32 */,
                                            double (&out)[1], int k_of_thread) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int nw = (blockDim.x + 31) >> 5;
#pragma unroll
  for (int k = 0; k < NV; ++k) v[k] = warp_sumf(v[k]);
  __syncthreads();
  if (lane == 0)
#pragma unroll
    for (int k = 0; k < NV; ++k) smem[k * 32 + warp] = v[k];
  __syncthreads();
  double t = 0.0;
  if (k_of_thread < NV)
    for (int w = 0; w < nw; ++w) t += (double)smem[k_of_thread * 32 + w];
  out[0] = t;
}

// Arrival counter: returns true in the whole block of the last block to
// arrive (after its partials are visible).  Resets the counter.
__device__ __forceinline__ bool last_block(unsigned* counter, unsigned nblocks) {
  __shared__ bool s_last;
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0 && threadIdx.y == 0) {
    const unsigned t = atomicAdd(counter, 1u);
    s_last = (t == nblocks - 1);
    if (s_last) *counter = 0u;
  }
  __syncthreads();
  if (s_last) __threadfence();
  return s_last;
}

// Block-wide FP64 completion of a residual kernel: every thread passes its
// sum of |r|^2; the last of the problem's nblk blocks sets the KState for the
// next Arnoldi cycle (beta, normalisation of V_0 stored / rscale, activity).
__device__ __forceinline__ void residual_finish(double acc, const KCtx& c, int b, int m,
                                                unsigned nblk, unsigned blk) {
  __shared__ double sm_rf[32];
  KState* st = c.st + b;
  double v[1] = {acc};
  block_sum<1>(v, sm_rf);
  double* part = c.partial + (size_t)b * c.part_stride;
  if (threadIdx.x == 0 && threadIdx.y == 0) part[blk] = v[0];
  if (!last_block(c.counter + 2 * b, nblk)) return;
  double s[1] = {0.0};
  for (unsigned k = threadIdx.x; k < nblk; k += blockDim.x) s[0] += __ldcg(part + k);
  block_sum<1>(s, sm_rf);
  if (threadIdx.x == 0 && threadIdx.y == 0) {
    const double beta = sqrt(s[0]);
    st->beta = beta;
    st->res_est = beta;
    st->ncols = 0;
    c.sc[(size_t)b * (m + 1)] = beta > 0 ? st->rscale / beta : 0.0;
    if (beta > 0) st->rscale = beta;
    c.gam[(size_t)b * (m + 1)] = make_double2(beta, 0.0);
    st->thresh = fmax(c.tol * st->bnorm * 0.5, c.inner_rtol * beta);
    const bool ok = isfinite(beta);
    if (!ok) st->nan = 1;
    st->active = (ok && beta > c.tol * st->bnorm && st->bnorm > 0) ? 1 : 0;
  }
}

}  // namespace cev
