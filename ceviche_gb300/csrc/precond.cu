// Right preconditioners for the flexible GMRES cycle.
//
// CEV_PRECOND_SEPARABLE: the exact inverse of the plan's stretched operator
// with eps replaced by a constant c per problem,
//   M^-1 = (Vx (x) Vy) diag(1/d) (Vx^-1 (x) Vy^-1),
// from the eigendecompositions of the plan's 1D axis operators (computed by
// the caller from cev_fdfd_axis_matrix).  A vector of the basis is the
// row-major (nx, ny) grid R, i.e. the column-major (ny x nx) matrix R^T, so
//   (M^-1 R)^T = Vy ((Vy^-1 R^T Vx^-T) ./ D^T) Vx^T
// is four complex GEMMs (cuBLAS, strided-batched over the problems; plain
// library GEMMs) around one scaling kernel that also applies the basis
// vector's scale sc_j.  The factors and GEMMs are complex128: with PML the
// 1D operators are far from normal (cond(V) ~ 1e6 for 20 PML cells on a
// 200-cell axis), and complex64 factors leave the preconditioner with O(0.1)
// errors.
#include <cublas_v2.h>

#include "krylov.hpp"

struct cev_sep_precond_s {
  int nx = 0, ny = 0, batch = 0, transpose = 0;
  const double2 *vx = nullptr, *vxi = nullptr, *vy = nullptr, *vyi = nullptr, *dinv = nullptr;
  cublasHandle_t blas = nullptr;
};

namespace cev {

static int blas_status(cublasStatus_t st, const char* where) {
  if (st == CUBLAS_STATUS_SUCCESS) return CEV_OK;
  set_error("%s: cuBLAS status %d", where, (int)st);
  return CEV_ERR_CUDA;
}

size_t precond_workspace_size(const cev_fdfd_plan_s* p, const cev_solve_opts& o) {
  if (o.precond != CEV_PRECOND_SEPARABLE || !p) return 0;
  return 2 * sizeof(double2) * p->n() * (size_t)p->batch + 256;  // two GEMM temporaries
}

struct SepState {
  cev_sep_precond_s* h = nullptr;
  double2* t1 = nullptr;
  double2* t2 = nullptr;
  size_t n = 0;
  int B = 0, m = 0;
};

// CEV_PRECOND_LEARNED: the network of csrc/learned.cu, z = sc_j * f(v_j)
struct LearnedState {
  cev_learned_precond_s* h;
  const cev_fdfd_plan_s* p;
  const float* eps;
  int eps_shared;
};

int precond_setup(Precond& pc, const cev_fdfd_plan_s* p, const cev_solve_opts& o, const float* eps32,
                  int eps_shared, void* ws, cudaStream_t) {
  pc.kind = o.precond;
  if (o.precond == CEV_PRECOND_NONE) return CEV_OK;
  if (o.precond == CEV_PRECOND_LEARNED) {
    auto* h = (cev_learned_precond_s*)o.learned;
    const int rc = nn::learned_check(h, p);
    if (rc != CEV_OK) return rc;
    static thread_local LearnedState ls;  // one Precond per solve call, as above
    ls = LearnedState{h, p, eps32, eps_shared};
    pc.impl = &ls;
    return CEV_OK;
  }
  if (o.precond == CEV_PRECOND_DIRECT || o.precond == CEV_PRECOND_SHIFTED_LAPLACIAN) {
    auto* h = (cev_nd_precond_s*)o.direct;
    const int rc = nd_check(h, p, o.precond, o.transpose ? 1 : 0);
    if (rc != CEV_OK) return rc;
    pc.impl = h;
    return CEV_OK;
  }
  CEV_REQUIRE(o.precond == CEV_PRECOND_SEPARABLE, "preconditioner %d is not available", o.precond);
  auto* h = (cev_sep_precond_s*)o.separable;
  CEV_REQUIRE(h != nullptr, "CEV_PRECOND_SEPARABLE needs opts.separable");
  CEV_REQUIRE(h->nx == p->nx && h->ny == p->ny && h->batch == p->batch,
              "separable preconditioner built for (%d, %d, batch %d), plan is (%d, %d, batch %d)",
              h->nx, h->ny, h->batch, p->nx, p->ny, p->batch);
  CEV_REQUIRE(h->transpose == (o.transpose ? 1 : 0),
              "separable preconditioner built for transpose=%d, solve has transpose=%d",
              h->transpose, o.transpose ? 1 : 0);
  static thread_local SepState st;  // the driver holds one Precond per solve call
  st.h = h;
  st.n = p->n();
  st.B = p->batch;
  st.m = o.restart;
  st.t1 = (double2*)ws;
  st.t2 = st.t1 + st.n * st.B;
  pc.impl = &st;
  return CEV_OK;
}

// out = (sc_j / d) .* t  (same layout: row-major (nx, ny) per problem)
__global__ void k_sep_scale(const double2* __restrict__ t, const double2* __restrict__ dinv,
                            const double* __restrict__ sc, int j, int m, size_t n, int B,
                            double2* __restrict__ out) {
  const size_t total = n * (size_t)B;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total;
       e += (size_t)gridDim.x * blockDim.x) {
    const int b = (int)(e / n);
    out[e] = cscale(cmul(t[e], dinv[e]), sc[(size_t)b * (m + 1) + j]);
  }
}

__global__ void k_c64_to_c128(const float2* __restrict__ in, double2* __restrict__ out, size_t n) {
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n;
       e += (size_t)gridDim.x * blockDim.x)
    out[e] = to_d(in[e]);
}

__global__ void k_c128_to_c64(const double2* __restrict__ in, float2* __restrict__ out, size_t n) {
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n;
       e += (size_t)gridDim.x * blockDim.x)
    out[e] = to_f(in[e]);
}

int precond_apply(Precond& pc, const KCtx& c, int j, int m, const float2* v, float2* z,
                  cudaStream_t s) {
  CEV_REQUIRE(pc.impl != nullptr, "no preconditioner configured");
  if (pc.kind == CEV_PRECOND_LEARNED) {
    const LearnedState& ls = *(const LearnedState*)pc.impl;
    return nn::learned_forward(ls.h, ls.p, ls.eps, ls.eps_shared, v, z, c.sc, m + 1, j, s);
  }
  if (pc.kind == CEV_PRECOND_DIRECT || pc.kind == CEV_PRECOND_SHIFTED_LAPLACIAN)
    return nd_apply((cev_nd_precond_s*)pc.impl, v, z, c.sc, m + 1, j, c.st, s);
  CEV_REQUIRE(pc.kind == CEV_PRECOND_SEPARABLE, "no preconditioner configured");
  SepState& st = *(SepState*)pc.impl;
  cev_sep_precond_s& h = *st.h;
  const int nx = h.nx, ny = h.ny, B = h.batch;
  const size_t total = st.n * (size_t)B;
  const long long sn = (long long)st.n, sx = (long long)nx * nx, sy = (long long)ny * ny;
  const cuDoubleComplex one = make_cuDoubleComplex(1.0, 0.0), zero = make_cuDoubleComplex(0.0, 0.0);
  int rc = blas_status(cublasSetStream(h.blas, s), "cublasSetStream");
  if (rc != CEV_OK) return rc;
  auto C = [](const double2* p) { return (const cuDoubleComplex*)p; };
  auto W = [](double2* p) { return (cuDoubleComplex*)p; };
  const unsigned g = std::max(1u, std::min(ceil_div(total, 256), 8u * sm_count()));
  k_c64_to_c128<<<g, 256, 0, s>>>(v, st.t1, total);
  CEV_CHECK_LAUNCH("k_c64_to_c128");
  // t2 = Vy^-1 R^T   (row-major Vy^-1 read transposed)
  rc = blas_status(cublasZgemmStridedBatched(h.blas, CUBLAS_OP_T, CUBLAS_OP_N, ny, nx, ny, &one,
                                             C(h.vyi), ny, sy, C(st.t1), ny, sn, &zero, W(st.t2),
                                             ny, sn, B),
                   "gemm 1");
  if (rc != CEV_OK) return rc;
  // t1 = t2 Vx^-T   (row-major Vx^-1 read as column-major is Vx^-T)
  rc = blas_status(cublasZgemmStridedBatched(h.blas, CUBLAS_OP_N, CUBLAS_OP_N, ny, nx, nx, &one,
                                             C(st.t2), ny, sn, C(h.vxi), nx, sx, &zero, W(st.t1),
                                             ny, sn, B),
                   "gemm 2");
  if (rc != CEV_OK) return rc;
  k_sep_scale<<<g, 256, 0, s>>>(st.t1, h.dinv, c.sc, j, m, st.n, B, st.t2);
  CEV_CHECK_LAUNCH("k_sep_scale");
  // t1 = Vy t2 ; t2 = t1 Vx^T ; z = complex64(t2)
  rc = blas_status(cublasZgemmStridedBatched(h.blas, CUBLAS_OP_T, CUBLAS_OP_N, ny, nx, ny, &one,
                                             C(h.vy), ny, sy, C(st.t2), ny, sn, &zero, W(st.t1),
                                             ny, sn, B),
                   "gemm 3");
  if (rc != CEV_OK) return rc;
  rc = blas_status(cublasZgemmStridedBatched(h.blas, CUBLAS_OP_N, CUBLAS_OP_N, ny, nx, nx, &one,
                                             C(st.t1), ny, sn, C(h.vx), nx, sx, &zero, W(st.t2),
                                             ny, sn, B),
                   "gemm 4");
  if (rc != CEV_OK) return rc;
  k_c128_to_c64<<<g, 256, 0, s>>>(st.t2, z, total);
  CEV_CHECK_LAUNCH("k_c128_to_c64");
  return CEV_OK;
}

}  // namespace cev

using namespace cev;

extern "C" {

int cev_sep_precond_create(cev_sep_precond* out, cev_fdfd_plan plan, int transpose,
                           const void* vx, const void* vxi, const void* vy, const void* vyi,
                           const void* dinv) {
  CEV_REQUIRE(out != nullptr && plan != nullptr, "NULL argument");
  *out = nullptr;
  CEV_REQUIRE(vx && vxi && vy && vyi && dinv, "NULL factor");
  CEV_REQUIRE(plan->mf_nsb < 0, "multi-frequency plans have no separable preconditioner");
  auto* h = new cev_sep_precond_s();
  h->nx = plan->nx;
  h->ny = plan->ny;
  h->batch = plan->batch;
  h->transpose = transpose ? 1 : 0;
  h->vx = (const double2*)vx;
  h->vxi = (const double2*)vxi;
  h->vy = (const double2*)vy;
  h->vyi = (const double2*)vyi;
  h->dinv = (const double2*)dinv;
  const cublasStatus_t st = cublasCreate(&h->blas);
  if (st != CUBLAS_STATUS_SUCCESS) {
    delete h;
    set_error("cublasCreate: status %d", (int)st);
    return CEV_ERR_CUDA;
  }
  *out = h;
  return CEV_OK;
}

int cev_sep_precond_destroy(cev_sep_precond h) {
  if (!h) return CEV_OK;
  if (h->blas) cublasDestroy(h->blas);
  delete h;
  return CEV_OK;
}

}  // extern "C"
