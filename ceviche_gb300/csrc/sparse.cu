// Generic sparse systems: CSR SpMV and the Krylov solve of ceviche's
// entries/indices primitives (ceviche/primitives.py:58-148), for matrices
// that are not the Yee stencil.
//
// The caller converts COO entries/indices to CSR (duplicates summed, as
// scipy's coo->csr in ceviche/utils.py:13-25 does).  The solve runs on the
// uniformly scaled system (scale * A) x = scale * b, with scale ~ 1/max|A_ij|
// so complex64 Arnoldi vectors stay in range; the FP64 residual and the
// convergence test are scale-free.
#include <cmath>

#include "krylov.hpp"
#include "reduce.cuh"

namespace cev {

__global__ void k_csr_apply(int n, const int* __restrict__ rp, const int* __restrict__ col,
                            const double2* __restrict__ val, const double2* __restrict__ x,
                            double2* __restrict__ y) {
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) {
    double2 acc = make_double2(0.0, 0.0);
    for (int q = rp[r]; q < rp[r + 1]; ++q) acc = cfma(val[q], x[col[q]], acc);
    y[r] = acc;
  }
}

__global__ void k_csr_to_c64(int nnz, const double2* val, double scale, float2* out) {
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < nnz; q += gridDim.x * blockDim.x)
    out[q] = to_f(cscale(val[q], scale));
}

// FP64 residual of the scaled system; complex64 copy / rscale into V0
__global__ void __launch_bounds__(256) k_csr_residual(int n, const int* rp, const int* col,
                                                      const double2* val, double scale,
                                                      const double2* x, const double2* b,
                                                      float2* r, KCtx ctx, int m) {
  const KState* st = ctx.st;
  if (st->done) return;
  const double inv = 1.0 / st->rscale;
  double acc = 0.0;
  for (int row = blockIdx.x * blockDim.x + threadIdx.x; row < n;
       row += gridDim.x * blockDim.x) {
    double2 ax = make_double2(0.0, 0.0);
    for (int q = rp[row]; q < rp[row + 1]; ++q) ax = cfma(val[q], x[col[q]], ax);
    const double2 rv = cscale(csub(b[row], ax), scale);
    r[row] = to_f(cscale(rv, inv));
    acc += rv.x * rv.x + rv.y * rv.y;
  }
  residual_finish(acc, ctx, 0, m, gridDim.x, blockIdx.x);
}

__global__ void k_csr_mv(int n, const int* __restrict__ rp, const int* __restrict__ col,
                         const float2* __restrict__ val, const float2* __restrict__ x,
                         float2* __restrict__ y, KCtx ctx, int j, int use_scale) {
  if (!ctx.st[0].active) return;
  const float s = use_scale ? (float)ctx.sc[j] : 1.0f;
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) {
    float2 acc = make_float2(0.f, 0.f);
    for (int q = rp[r]; q < rp[r + 1]; ++q) acc = cfma(val[q], x[col[q]], acc);
    y[r] = cscale(acc, s);
  }
}

static unsigned csr_blocks(int n) {
  return std::max(1u, std::min(ceil_div((size_t)n, 256), 4u * sm_count()));
}

static KrylovProblem csr_problem(int n, int nnz) {
  KrylovProblem P;
  P.B = 1;
  P.n = (size_t)n;
  P.res_blocks = csr_blocks(n);
  P.extra_bytes = sizeof(float2) * (size_t)nnz;
  return P;
}

}  // namespace cev

using namespace cev;

extern "C" {

int cev_csr_apply(int n, int nnz, const int* row_ptr, const int* col, const void* val,
                  const void* x, void* y, cudaStream_t s) {
  CEV_REQUIRE(n >= 1 && nnz >= 0, "bad sizes n=%d nnz=%d", n, nnz);
  CEV_REQUIRE(row_ptr && (nnz == 0 || (col && val)) && x && y, "NULL argument");
  CEV_REQUIRE(x != y, "x and y must not alias");
  k_csr_apply<<<csr_blocks(n), 256, 0, s>>>(n, row_ptr, col, (const double2*)val,
                                            (const double2*)x, (double2*)y);
  CEV_CHECK_LAUNCH("k_csr_apply");
  return CEV_OK;
}

size_t cev_csr_solve_workspace_size(int n, int nnz, const cev_solve_opts* opts) {
  if (n < 1 || nnz < 0 || !opts || opts->restart < 1 || opts->restart > 64) return 0;
  return klayout(csr_problem(n, nnz), *opts, 0).total;
}

int cev_csr_solve(int n, int nnz, const int* row_ptr, const int* col, const void* val,
                  double scale, const void* bvec, void* xvec, const cev_solve_opts* opts,
                  cev_solve_info* info, void* ws, size_t ws_bytes, cudaStream_t s) {
  CEV_REQUIRE(n >= 1 && nnz >= 1, "bad sizes n=%d nnz=%d", n, nnz);
  CEV_REQUIRE(row_ptr && col && val && bvec && xvec && opts && info, "NULL argument");
  CEV_REQUIRE(scale > 0 && std::isfinite(scale), "scale must be positive");
  const cev_solve_opts& o = *opts;
  int rc = validate_opts(o);
  if (rc != CEV_OK) return rc;
  CEV_REQUIRE(o.precond == CEV_PRECOND_NONE, "the generic sparse solve has no preconditioner");
  CEV_REQUIRE(!o.transpose, "pass the transposed CSR arrays for A^T");
  const KrylovProblem P = csr_problem(n, nnz);
  const KLayout L = klayout(P, o, 0);
  CEV_REQUIRE(ws != nullptr && ws_bytes >= L.total,
              "workspace too small: need %zu bytes, got %zu", L.total, ws_bytes);
  CEV_REQUIRE(((uintptr_t)ws & 255) == 0, "workspace must be 256-byte aligned");
  float2* val32 = (float2*)((char*)ws + L.extra);
  k_csr_to_c64<<<csr_blocks(nnz), 256, 0, s>>>(nnz, (const double2*)val, scale, val32);
  CEV_CHECK_LAUNCH("k_csr_to_c64");
  const int m = o.restart;
  KrylovOps ops;
  ops.bscale = scale;
  ops.residual = [&](const KCtx& c, float2* V0, cudaStream_t st) -> int {
    k_csr_residual<<<csr_blocks(n), 256, 0, st>>>(n, row_ptr, col, (const double2*)val, scale,
                                                  (const double2*)xvec, (const double2*)bvec,
                                                  V0, c, m);
    CEV_CHECK_LAUNCH("k_csr_residual");
    return CEV_OK;
  };
  ops.matvec = [&](const KCtx& c, int j, const float2* in, int use_scale, float2* out,
                   cudaStream_t st) -> int {
    k_csr_mv<<<csr_blocks(n), 256, 0, st>>>(n, row_ptr, col, val32, in, out, c, j, use_scale);
    CEV_CHECK_LAUNCH("k_csr_mv");
    return CEV_OK;
  };
  return krylov_run(P, ops, o, (const double2*)bvec, (double2*)xvec, info, ws, ws_bytes, s);
}

}  // extern "C"
