// Right preconditioners for the flexible GMRES cycle.
//
// CEV_PRECOND_SEPARABLE: the exact inverse of the plan's stretched operator
// with eps replaced by a constant c per problem,
//   M^-1 = (Vx (x) Vy) diag(1/d) (Vx^-1 (x) Vy^-1),
// from the eigendecompositions of the plan's 1D axis operators (computed by
// the caller from cev_fdfd_axis_matrix).  A vector of the basis is the
// row-major (nx, ny) grid R, i.e. the column-major (ny x nx) matrix R^T, so
//   (M^-1 R)^T = Vy ((Vy^-1 R^T Vx^-T) ./ D^T) Vx^T
// is four complex GEMMs (k_zgemm, strided-batched over the problems) around
// one scaling kernel that also applies the basis vector's scale sc_j.  The
// factors and GEMMs are complex128: with PML the 1D operators are far from
// normal (cond(V) ~ 1e6 for 20 PML cells on a 200-cell axis), and complex64
// factors leave the preconditioner with O(0.1) errors.
#include "krylov.hpp"

struct cev_sep_precond_s {
  int nx = 0, ny = 0, batch = 0, transpose = 0;
  const double2 *vx = nullptr, *vxi = nullptr, *vy = nullptr, *vyi = nullptr, *dinv = nullptr;
};

namespace cev {

// Batched complex128 GEMM, column-major: C_b = op(A_b) B_b, op(A) = A^T when
// TA (m x n result, inner dimension k; leading dimensions and per-problem
// strides as given).  A T x T output tile per CTA of (T/U)^2 threads, each a
// U x U block, 16-deep k chunks staged in shared memory.  On GB300 the FP64
// FMA pipe is the bound, so what matters is occupying every SM: 64 x 64 tiles
// for large or batched products, 16 x 16 tiles when those would leave SMs idle
// (a single 200 x 200 product has 16 tiles of 64 but 169 of 16).
constexpr int ZG_K = 16;
template <bool TA, int T, int U>
__global__ void __launch_bounds__((T / U) * (T / U)) k_zgemm(
    int m, int n, int k, const double2* __restrict__ A, int lda, long long sa,
    const double2* __restrict__ B, int ldb, long long sb, double2* __restrict__ C, int ldc,
    long long sc) {
  constexpr int TP = T / U, NT = TP * TP;
  __shared__ double2 As[ZG_K][T + 1];  // [l][i] = op(A)[i][l]
  __shared__ double2 Bs[ZG_K][T + 1];  // [l][j] = B[l][j]
  const int bz = blockIdx.z;
  A += bz * sa;
  B += bz * sb;
  C += bz * sc;
  const int i0 = blockIdx.x * T, j0 = blockIdx.y * T;
  const int tx = threadIdx.x % TP, ty = threadIdx.x / TP;
  double2 acc[U][U];
#pragma unroll
  for (int u = 0; u < U; ++u)
#pragma unroll
    for (int v = 0; v < U; ++v) acc[u][v] = make_double2(0.0, 0.0);
  for (int k0 = 0; k0 < k; k0 += ZG_K) {
    for (int e = threadIdx.x; e < T * ZG_K; e += NT) {
      // op(A): element (i, l) is A[l + i lda] (TA) or A[i + l lda]; read along the contiguous index
      int i, l;
      if (TA) {
        i = e / ZG_K;
        l = e - i * ZG_K;
      } else {
        l = e / T;
        i = e - l * T;
      }
      const int gi = i0 + i, gl = k0 + l;
      As[l][i] = (gi < m && gl < k) ? (TA ? A[gl + (size_t)gi * lda] : A[gi + (size_t)gl * lda])
                                    : make_double2(0.0, 0.0);
      const int j = e / ZG_K, lb = e - j * ZG_K;
      const int gj = j0 + j, glb = k0 + lb;
      Bs[lb][j] = (gj < n && glb < k) ? B[glb + (size_t)gj * ldb] : make_double2(0.0, 0.0);
    }
    __syncthreads();
#pragma unroll 4
    for (int l = 0; l < ZG_K; ++l) {
      double2 a[U], bv[U];
#pragma unroll
      for (int u = 0; u < U; ++u) a[u] = As[l][tx + TP * u];
#pragma unroll
      for (int v = 0; v < U; ++v) bv[v] = Bs[l][ty + TP * v];
#pragma unroll
      for (int u = 0; u < U; ++u)
#pragma unroll
        for (int v = 0; v < U; ++v) {
          acc[u][v].x = fma(a[u].x, bv[v].x, acc[u][v].x);
          acc[u][v].x = fma(-a[u].y, bv[v].y, acc[u][v].x);
          acc[u][v].y = fma(a[u].x, bv[v].y, acc[u][v].y);
          acc[u][v].y = fma(a[u].y, bv[v].x, acc[u][v].y);
        }
    }
    __syncthreads();
  }
#pragma unroll
  for (int u = 0; u < U; ++u)
#pragma unroll
    for (int v = 0; v < U; ++v) {
      const int gi = i0 + tx + TP * u, gj = j0 + ty + TP * v;
      if (gi < m && gj < n) C[gi + (size_t)gj * ldc] = acc[u][v];
    }
}

template <bool TA>
static int zgemm(int m, int n, int k, const double2* A, int lda, long long sa, const double2* B,
                 int ldb, long long sb, double2* C, int ldc, long long sc, int batch,
                 cudaStream_t s) {
  const long long big = (long long)((m + 63) / 64) * ((n + 63) / 64) * batch;
  if (big >= 2LL * sm_count()) {
    const dim3 g((m + 63) / 64, (n + 63) / 64, batch);
    k_zgemm<TA, 64, 4><<<g, 256, 0, s>>>(m, n, k, A, lda, sa, B, ldb, sb, C, ldc, sc);
  } else {
    const dim3 g((m + 15) / 16, (n + 15) / 16, batch);
    k_zgemm<TA, 16, 2><<<g, 64, 0, s>>>(m, n, k, A, lda, sa, B, ldb, sb, C, ldc, sc);
  }
  CEV_CHECK_LAUNCH("k_zgemm");
  return CEV_OK;
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
  const unsigned g = std::max(1u, std::min(ceil_div(total, 256), 8u * sm_count()));
  k_c64_to_c128<<<g, 256, 0, s>>>(v, st.t1, total);
  CEV_CHECK_LAUNCH("k_c64_to_c128");
  // t2 = Vy^-1 R^T   (row-major Vy^-1 read transposed)
  int rc = zgemm<true>(ny, nx, ny, h.vyi, ny, sy, st.t1, ny, sn, st.t2, ny, sn, B, s);
  if (rc != CEV_OK) return rc;
  // t1 = t2 Vx^-T   (row-major Vx^-1 read as column-major is Vx^-T)
  rc = zgemm<false>(ny, nx, nx, st.t2, ny, sn, h.vxi, nx, sx, st.t1, ny, sn, B, s);
  if (rc != CEV_OK) return rc;
  k_sep_scale<<<g, 256, 0, s>>>(st.t1, h.dinv, c.sc, j, m, st.n, B, st.t2);
  CEV_CHECK_LAUNCH("k_sep_scale");
  // t1 = Vy t2 ; t2 = t1 Vx^T ; z = complex64(t2)
  rc = zgemm<true>(ny, nx, ny, h.vy, ny, sy, st.t2, ny, sn, st.t1, ny, sn, B, s);
  if (rc != CEV_OK) return rc;
  rc = zgemm<false>(ny, nx, nx, st.t1, ny, sn, h.vx, nx, sx, st.t2, ny, sn, B, s);
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
  *out = h;
  return CEV_OK;
}

int cev_sep_precond_destroy(cev_sep_precond h) {
  if (!h) return CEV_OK;
  delete h;
  return CEV_OK;
}

}  // extern "C"
