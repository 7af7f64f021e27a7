// Multi-frequency (time-modulated) FDFD Ez: ceviche/fdfd.py:247-359.
//
// Unknowns: M = 2 Nsb + 1 sideband fields [M][nx][ny] at W_m = w + m w_mod,
// m = -Nsb..Nsb.  Block operator (fdfd.py:289-326):
//   A_mm        = -(1/mu0)(Dxf Dxb + Dyf Dyb) - eps0 W_m^2 diag(eps)
//   A_m,m+k+1   = diag(-1/2 eps0 W_m^2 delta_k e^{+i phi_k})        (k = 0..Nfreq-1)
//   A_m,m-k-1   = diag(-1/2 eps0 W_m^2 delta_k e^{-i phi_k})
// with every derivative matrix built at the centre frequency w.  The
// modulation enters as c_k = delta_k e^{i phi_k} (complex128 [Nfreq][nx][ny]).
// The plan is an Ez plan with M problems sharing the centre-w PML tables and
// carrying k^2 = eps0 mu0 W_m^2 dL^2 and W_m per problem; the Krylov solve
// treats the M sidebands as ONE coupled system of M*nx*ny unknowns.
#include <cmath>
#include <vector>

#include "krylov.hpp"
#include "reduce.cuh"

namespace cev {

void launch_geometry(int nx, int ny, int batch, dim3& grid, dim3& block, int& rows);

// Coupling added to row block m (without the -1/2 factor):
//   forward:   k2_m c u_{m+k+1} + k2_m conj(c) u_{m-k-1}
//   transpose: k2_{m+k+1} conj(c) u_{m+k+1} + k2_{m-k-1} c u_{m-k-1}
template <typename R>
struct MfArgs {
  int nx, ny, rows, M, nfreq, transpose;
  const R* eps;       // [N]
  const Cplx<R>* cpl; // [nfreq][N]
  const Cplx<R>* x;   // [M][N]
  const Coef<R>* cx;  // [M][nx]
  const Coef<R>* cy;  // [M][ny]
  const R* k2;        // [M]
};

template <typename R>
__device__ __forceinline__ Cplx<R> mf_coupling(const MfArgs<R>& a, int m, size_t n) {
  using C = Cplx<R>;
  const size_t N = (size_t)a.nx * a.ny;
  C acc = cmk<C>(0.0, 0.0);
  for (int k = 0; k < a.nfreq; ++k) {
    const C c = a.cpl[(size_t)k * N + n];
    const int mp = m + k + 1, mm = m - k - 1;
    if (mp < a.M) {
      const R f = a.transpose ? a.k2[mp] : a.k2[m];
      const C cc = a.transpose ? cconj(c) : c;
      acc = cfma(cscale(cc, f), a.x[(size_t)mp * N + n], acc);
    }
    if (mm >= 0) {
      const R f = a.transpose ? a.k2[mm] : a.k2[m];
      const C cc = a.transpose ? c : cconj(c);
      acc = cfma(cscale(cc, f), a.x[(size_t)mm * N + n], acc);
    }
  }
  return cscale(acc, R(-0.5));
}

// y = oscale * A' x, one sideband per blockIdx.z
template <typename R>
__global__ void __launch_bounds__(128) k_mf_apply(MfArgs<R> a, Cplx<R>* y, R oscale) {
  using C = Cplx<R>;
  const int m = blockIdx.z;
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= a.ny) return;
  const int i0 = blockIdx.y * a.rows;
  const int i1 = min(i0 + a.rows, a.nx);
  const size_t N = (size_t)a.nx * a.ny;
  const Coef<R> cyj = a.cy[(size_t)m * a.ny + j];
  auto ep = [&](int i, C v, C) {
    const size_t n = (size_t)i * a.ny + j;
    y[(size_t)m * N + n] = cscale(cadd(v, mf_coupling(a, m, n)), oscale);
  };
  stencil_column<R, POL_EZ>(a.nx, a.ny, j, i0, i1, a.x + (size_t)m * N, a.eps,
                            a.cx + (size_t)m * a.nx, cyj, a.k2[m], ep);
}

// FP64 residual r = b' - A' x of the coupled system -> V0 (/ rscale), beta
__global__ void __launch_bounds__(128) k_mf_residual(MfArgs<double> a, const double2* b,
                                                     double bscale, float2* r, KCtx ctx, int mres) {
  const KState* st = ctx.st;
  if (st->done) return;
  const int m = blockIdx.z;
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  const size_t N = (size_t)a.nx * a.ny;
  const unsigned nblk = gridDim.x * gridDim.y * gridDim.z;
  const unsigned blk = (blockIdx.z * gridDim.y + blockIdx.y) * gridDim.x + blockIdx.x;
  double acc = 0.0;
  if (j < a.ny) {
    const int i0 = blockIdx.y * a.rows;
    const int i1 = min(i0 + a.rows, a.nx);
    const double inv = 1.0 / st->rscale;
    const Coef<double> cyj = a.cy[(size_t)m * a.ny + j];
    auto ep = [&](int i, double2 v, double2) {
      const size_t n = (size_t)i * a.ny + j;
      const double2 av = cadd(v, mf_coupling(a, m, n));
      const double2 rv = csub(cscale(b[(size_t)m * N + n], bscale), av);
      r[(size_t)m * N + n] = to_f(cscale(rv, inv));
      acc += rv.x * rv.x + rv.y * rv.y;
    };
    stencil_column<double, POL_EZ>(a.nx, a.ny, j, i0, i1, a.x + (size_t)m * N, a.eps,
                                   a.cx + (size_t)m * a.nx, cyj, a.k2[m], ep);
  }
  residual_finish(acc, ctx, 0, mres, nblk, blk);
}

// Arnoldi matvec of the coupled system; input scaled by sc[0][j_col]
__global__ void __launch_bounds__(128) k_mf_mv(MfArgs<float> a, float2* y, KCtx ctx, int j_col,
                                               int use_scale) {
  if (!ctx.st[0].active) return;
  const int m = blockIdx.z;
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= a.ny) return;
  const int i0 = blockIdx.y * a.rows;
  const int i1 = min(i0 + a.rows, a.nx);
  const size_t N = (size_t)a.nx * a.ny;
  const float s = use_scale ? (float)ctx.sc[j_col] : 1.0f;
  const Coef<float> cyj = a.cy[(size_t)m * a.ny + j];
  auto ep = [&](int i, float2 v, float2) {
    const size_t n = (size_t)i * a.ny + j;
    y[(size_t)m * N + n] = cscale(cadd(v, mf_coupling(a, m, n)), s);
  };
  stencil_column<float, POL_EZ>(a.nx, a.ny, j, i0, i1, a.x + (size_t)m * N, a.eps,
                                a.cx + (size_t)m * a.nx, cyj, a.k2[m], ep);
}

__global__ void k_mf_c128_to_c64(const double2* in, float2* out, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x)
    out[i] = to_f(in[i]);
}
__global__ void k_mf_f64_to_f32(const double* in, float* out, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x)
    out[i] = (float)in[i];
}

// Gradients of a real loss through A (SI), given x and mu = A^{-T} conj(g):
//   geps[n]   += sum_m Re(mu_m eps0 W_m^2 x_m)
//   gcpl_k[n] += conj(P) + Q,  P = sum_m a_m x_{m+k+1}, Q = sum_m a_m x_{m-k-1},
//                a_m = 1/2 eps0 W_m^2 mu_m   (PyTorch convention for complex c_k)
__global__ void k_mf_grad(int M, int nfreq, size_t N, const double* W, const double2* x,
                          const double2* mu, double* geps, double2* gcpl) {
  for (size_t n = blockIdx.x * (size_t)blockDim.x + threadIdx.x; n < N;
       n += (size_t)gridDim.x * blockDim.x) {
    double ge = 0.0;
    for (int m = 0; m < M; ++m) {
      const double2 p = cmul(mu[(size_t)m * N + n], x[(size_t)m * N + n]);
      ge += p.x * EPSILON_0 * W[m] * W[m];
    }
    geps[n] += ge;
    if (!gcpl) continue;
    for (int k = 0; k < nfreq; ++k) {
      double2 P = make_double2(0, 0), Q = make_double2(0, 0);
      for (int m = 0; m < M; ++m) {
        const double2 am = cscale(mu[(size_t)m * N + n], 0.5 * EPSILON_0 * W[m] * W[m]);
        if (m + k + 1 < M) P = cfma(am, x[(size_t)(m + k + 1) * N + n], P);
        if (m - k - 1 >= 0) Q = cfma(am, x[(size_t)(m - k - 1) * N + n], Q);
      }
      gcpl[(size_t)k * N + n] = cadd(gcpl[(size_t)k * N + n], cadd(cconj(P), Q));
    }
  }
}

static size_t mf_eps_bytes(size_t N) { return (sizeof(float) * N + 255) & ~(size_t)255; }

static KrylovProblem mf_problem(const cev_fdfd_plan_s* p, int nfreq) {
  KrylovProblem P;
  P.B = 1;
  P.n = p->n() * p->batch;
  dim3 g, bl;
  int rows;
  launch_geometry(p->nx, p->ny, p->batch, g, bl, rows);
  P.res_blocks = (size_t)g.x * g.y * g.z;
  P.extra_bytes = mf_eps_bytes(p->n()) + sizeof(float2) * p->n() * nfreq;
  return P;
}

static int check_mf(cev_fdfd_plan p, int nfreq) {
  CEV_REQUIRE(p != nullptr && p->mf_nsb >= 0 && p->pol == CEV_POL_EZ,
              "not a multi-frequency plan (use cev_fdfd_mf_plan_create)");
  CEV_REQUIRE(nfreq >= 0 && nfreq <= 2 * p->mf_nsb, "nfreq must be in [0, 2*Nsb]");
  return CEV_OK;
}

}  // namespace cev

using namespace cev;

extern "C" {

int cev_fdfd_mf_plan_create(cev_fdfd_plan* out, int nx, int ny, double dL, double omega,
                            double omega_mod, int nsb, int npml_x, int npml_y, double bloch_x,
                            double bloch_y) {
  CEV_REQUIRE(out != nullptr, "plan output pointer is NULL");
  CEV_REQUIRE(nsb >= 0 && nsb <= 64, "Nsb must be in [0, 64]");
  CEV_REQUIRE(std::isfinite(omega_mod), "omega_mod must be finite");
  const int M = 2 * nsb + 1;
  std::vector<double> W(M);
  for (int m = 0; m < M; ++m) {
    W[m] = omega + (m - nsb) * omega_mod;
    CEV_REQUIRE(W[m] > 0, "sideband frequency %d is not positive", m - nsb);
  }
  // every sideband uses the centre-frequency derivatives (fdfd.py:80-99)
  std::vector<double> centre(M, omega);
  int rc = cev_fdfd_plan_create(out, CEV_POL_EZ, nx, ny, M, dL, centre.data(), npml_x, npml_y,
                                bloch_x, bloch_y);
  if (rc != CEV_OK) return rc;
  cev_fdfd_plan p = *out;
  std::vector<double> k2(M);
  std::vector<float> k2f(M);
  for (int m = 0; m < M; ++m) {
    k2[m] = EPSILON_0 * MU_0 * W[m] * W[m] * dL * dL;
    k2f[m] = (float)k2[m];
  }
  p->omega = W;
  p->mf_nsb = nsb;
  p->omega_mod = omega_mod;
  cudaError_t e = cudaMemcpy(p->k2_64, k2.data(), sizeof(double) * M, cudaMemcpyHostToDevice);
  if (e == cudaSuccess)
    e = cudaMemcpy(p->k2_32, k2f.data(), sizeof(float) * M, cudaMemcpyHostToDevice);
  if (e == cudaSuccess)
    e = cudaMemcpy(p->omega_d, W.data(), sizeof(double) * M, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    cev_fdfd_plan_destroy(p);
    *out = nullptr;
    return cuda_status(e, "cev_fdfd_mf_plan_create");
  }
  return CEV_OK;
}

int cev_fdfd_mf_apply(cev_fdfd_plan p, const double* eps, int nfreq, const void* coupling,
                      const void* x, void* y, int transpose, cudaStream_t s) {
  int rc = check_mf(p, nfreq);
  if (rc != CEV_OK) return rc;
  CEV_REQUIRE(eps && x && y && (nfreq == 0 || coupling), "NULL argument");
  const int tr = transpose ? 1 : 0;
  MfArgs<double> a{};
  dim3 g, bl;
  launch_geometry(p->nx, p->ny, p->batch, g, bl, a.rows);
  a.nx = p->nx;
  a.ny = p->ny;
  a.M = p->batch;
  a.nfreq = nfreq;
  a.transpose = tr;
  a.eps = eps;
  a.cpl = (const double2*)coupling;
  a.x = (const double2*)x;
  a.cx = p->cx64[tr];
  a.cy = p->cy64[tr];
  a.k2 = p->k2_64;
  k_mf_apply<double><<<g, bl, 0, s>>>(a, (double2*)y, 1.0 / p->scale);
  CEV_CHECK_LAUNCH("k_mf_apply");
  return CEV_OK;
}

size_t cev_fdfd_mf_solve_workspace_size(cev_fdfd_plan p, int nfreq, const cev_solve_opts* opts) {
  if (!p || !opts || opts->restart < 1 || opts->restart > 64 || nfreq < 0) return 0;
  return klayout(mf_problem(p, nfreq), *opts, 0).total;
}

int cev_fdfd_mf_solve(cev_fdfd_plan p, const double* eps, int nfreq, const void* coupling,
                      const void* bvec, void* xvec, const cev_solve_opts* opts,
                      cev_solve_info* info, void* ws, size_t ws_bytes, cudaStream_t s) {
  int rc = check_mf(p, nfreq);
  if (rc != CEV_OK) return rc;
  CEV_REQUIRE(opts != nullptr, "opts is NULL");
  CEV_REQUIRE(eps && bvec && xvec && info && (nfreq == 0 || coupling), "NULL argument");
  const cev_solve_opts& o = *opts;
  rc = validate_opts(o);
  if (rc != CEV_OK) return rc;
  CEV_REQUIRE(o.precond == CEV_PRECOND_NONE, "the multi-frequency solve has no preconditioner");
  const KrylovProblem P = mf_problem(p, nfreq);
  const KLayout L = klayout(P, o, 0);
  CEV_REQUIRE(ws != nullptr && ws_bytes >= L.total,
              "workspace too small: need %zu bytes, got %zu", L.total, ws_bytes);
  CEV_REQUIRE(((uintptr_t)ws & 255) == 0, "workspace must be 256-byte aligned");
  const size_t N = p->n();
  const int tr = o.transpose ? 1 : 0;
  float* eps32 = (float*)((char*)ws + L.extra);
  float2* cpl32 = (float2*)((char*)ws + L.extra + mf_eps_bytes(N));
  const unsigned gb = std::max(1u, std::min(ceil_div(N * std::max(1, nfreq), 256), 8u * sm_count()));
  k_mf_f64_to_f32<<<gb, 256, 0, s>>>(eps, eps32, N);
  if (nfreq > 0) k_mf_c128_to_c64<<<gb, 256, 0, s>>>((const double2*)coupling, cpl32, N * nfreq);
  CEV_CHECK_LAUNCH("mf conversions");
  dim3 g, bl;
  int rows;
  launch_geometry(p->nx, p->ny, p->batch, g, bl, rows);
  const int m = o.restart;
  KrylovOps ops;
  ops.bscale = p->scale;
  ops.residual = [&](const KCtx& c, float2* V0, cudaStream_t st) -> int {
    MfArgs<double> a{p->nx, p->ny, rows, p->batch, nfreq, tr, eps, (const double2*)coupling,
                     (const double2*)xvec, p->cx64[tr], p->cy64[tr], p->k2_64};
    k_mf_residual<<<g, bl, 0, st>>>(a, (const double2*)bvec, p->scale, V0, c, m);
    CEV_CHECK_LAUNCH("k_mf_residual");
    return CEV_OK;
  };
  ops.matvec = [&](const KCtx& c, int j, const float2* in, int use_scale, float2* out,
                   cudaStream_t st) -> int {
    MfArgs<float> a{p->nx, p->ny, rows, p->batch, nfreq, tr, eps32, cpl32, in,
                    p->cx32[tr], p->cy32[tr], p->k2_32};
    k_mf_mv<<<g, bl, 0, st>>>(a, out, c, j, use_scale);
    CEV_CHECK_LAUNCH("k_mf_mv");
    return CEV_OK;
  };
  return krylov_run(P, ops, o, (const double2*)bvec, (double2*)xvec, info, ws, ws_bytes, s);
}

int cev_fdfd_mf_grad(cev_fdfd_plan p, int nfreq, const void* x, const void* mu, double* geps,
                     void* gcoupling, cudaStream_t s) {
  int rc = check_mf(p, nfreq);
  if (rc != CEV_OK) return rc;
  CEV_REQUIRE(x && mu && geps, "NULL argument");
  const size_t N = p->n();
  const unsigned gb = std::max(1u, std::min(ceil_div(N, 256), 8u * sm_count()));
  k_mf_grad<<<gb, 256, 0, s>>>(p->batch, nfreq, N, p->omega_d, (const double2*)x,
                               (const double2*)mu, geps,
                               (nfreq > 0 && gcoupling) ? (double2*)gcoupling : nullptr);
  CEV_CHECK_LAUNCH("k_mf_grad");
  return CEV_OK;
}

}  // extern "C"
