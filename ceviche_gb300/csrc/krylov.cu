// Restarted (flexible) GMRES on the matrix-free SC-PML stencil.
//
// Precision split: Arnoldi vectors, the stencil inside the cycle and the
// orthogonalisation run in complex64; inner products are reduced across
// threads and blocks in FP64 in a fixed order (deterministic); the
// Hessenberg matrix, Givens rotations and the small triangular solve are
// FP64 on the device; every restart recomputes the true residual
// b - A x in FP64 from the complex128 iterate and adds the cycle's
// correction to x in FP64 (mixed-precision iterative refinement).
//
// Device-side control: each problem of the batch carries a KState; the last
// block of a reduction (threadfence + counter) finalises the per-problem
// scalars, so a whole cycle is enqueued without host round trips.  The host
// reads the FP64 residuals once per cycle.
#include <algorithm>
#include <cstdlib>
#include <cmath>
#include <functional>
#include <type_traits>
#include <vector>

#include "fdfd_plan.hpp"
#include "krylov.hpp"
#include "reduce.cuh"

namespace cev {

void launch_geometry(int nx, int ny, int batch, dim3& grid, dim3& block, int& rows);

static constexpr int DOT_GROUP = 16;
// Largest batch (cells over all problems) solved with the fused cycle; above
// it the per-iteration launches are bandwidth-bound and their overhead small.
static constexpr size_t FUSED_MAX_CELLS = (size_t)1 << 21;

// --------------------------------------------------------------- residual
template <int POL, typename E = double>
struct ResArgs {
  int nx, ny, rows, first, m;
  const E* eps;
  size_t eps_bs;
  const double2* x;
  const double2* b;
  double bscale;
  const Coef<double>* cx;
  const Coef<double>* cy;
  const double* k2;
  float2* r;  // V_0 slot of each problem (stride n)
  size_t r_bs;
  KCtx ctx;
};

template <int POL, typename E>
__global__ void __launch_bounds__(128) k_residual(ResArgs<POL, E> a) {
  const int b = blockIdx.z;
  KState* st = a.ctx.st + b;
  if (st->done) return;
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  const size_t N = (size_t)a.nx * a.ny;
  const unsigned nblk = gridDim.x * gridDim.y;
  const unsigned blk = blockIdx.y * gridDim.x + blockIdx.x;
  double acc[1] = {0.0};
  if (j < a.ny) {
    const int i0 = blockIdx.y * a.rows;
    const int i1 = min(i0 + a.rows, a.nx);
    const double2* x = a.x + b * N;
    const double2* bb = a.b + b * N;
    float2* r = a.r + b * a.r_bs;
    const Coef<double> cyj = a.cy[(size_t)b * a.ny + j];
    const double bs = a.bscale;
    // keep the complex64 copy O(1): a tiny right-hand side (e.g. an adjoint
    // cotangent) would otherwise underflow float32
    const double inv = 1.0 / st->rscale;
    auto ep = [&](int i, double2 v, double2) {
      const size_t n = (size_t)i * a.ny + j;
      const double2 bv = cscale(bb[n], bs);
      const double2 rv = csub(bv, v);
      r[n] = to_f(cscale(rv, inv));
      acc[0] += rv.x * rv.x + rv.y * rv.y;
    };
    stencil_column<double, POL, decltype(ep), false, E>(a.nx, a.ny, j, i0, i1, x,
                                                         a.eps + b * a.eps_bs,
                                a.cx + (size_t)b * a.nx, cyj, a.k2[b], ep);
  }
  residual_finish(acc[0], a.ctx, b, a.m, nblk, blk);
}

// ||scale*b|| in FP64 before the first residual; seeds rscale
__global__ void __launch_bounds__(RED_THREADS) k_bnorm(const double2* bvec, double bscale, size_t n,
                                                       KCtx c) {
  const int b = blockIdx.y;
  const unsigned nblk = gridDim.x;
  const double2* bb = bvec + b * n;
  double acc[1] = {0.0};
  for (size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x; q < n;
       q += (size_t)gridDim.x * blockDim.x) {
    const double2 v = cscale(bb[q], bscale);
    acc[0] += v.x * v.x + v.y * v.y;
  }
  __shared__ double sm[32];
  block_sum<1>(acc, sm);
  double* part = c.partial + (size_t)b * c.part_stride;
  if (threadIdx.x == 0) part[blockIdx.x] = acc[0];
  if (!last_block(c.counter + 2 * b, nblk)) return;
  double s[1] = {0.0};
  for (unsigned q = threadIdx.x; q < nblk; q += blockDim.x) s[0] += __ldcg(part + q);
  block_sum<1>(s, sm);
  if (threadIdx.x == 0) {
    const double bn = sqrt(s[0]);
    c.st[b].bnorm = bn;
    c.st[b].rscale = bn > 0 ? bn : 1.0;
  }
}

// ------------------------------------------------------- Arnoldi matvec
template <int POL, typename E = float>
struct MvArgs {
  int nx, ny, rows, m, j;
  const E* eps;
  size_t eps_bs;
  const float2* in;  // [B][N] with stride in_bs
  size_t in_bs;
  int use_scale;     // multiply by sc[b][j]
  float2* out;
  size_t out_bs;
  const Coef<float>* cx;
  const Coef<float>* cy;
  const float* k2;
  KCtx ctx;
};

template <int POL, typename E>
__global__ void __launch_bounds__(128) k_arnoldi_mv(MvArgs<POL, E> a) {
  const int b = blockIdx.z;
  if (!a.ctx.st[b].active) return;
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= a.ny) return;
  const int i0 = blockIdx.y * a.rows;
  const int i1 = min(i0 + a.rows, a.nx);
  const float2* x = a.in + b * a.in_bs;
  float2* y = a.out + b * a.out_bs;
  const float s = a.use_scale ? (float)a.ctx.sc[(size_t)b * (a.m + 1) + a.j] : 1.0f;
  const Coef<float> cyj = a.cy[(size_t)b * a.ny + j];
  auto ep = [&](int i, float2 v, float2) { y[(size_t)i * a.ny + j] = cscale(v, s); };
  stencil_column<float, POL, decltype(ep), false, E>(a.nx, a.ny, j, i0, i1, x,
                                                    a.eps + b * a.eps_bs,
                             a.cx + (size_t)b * a.nx, cyj, a.k2[b], ep);
}

// The exact (FP64) operator on a complex64 input, complex64 output: the
// matvec of a flexible cycle whose preconditioner is a factorisation.  There
// z = M^-1 v is larger than A z ~ v by up to cond(A), so a float32 stencil
// (float tables, float eps, float products) would lose cond(A) * 6e-8 of the
// Arnoldi relation to cancellation.
template <int POL, typename E>
struct Mv64Args {
  int nx, ny, rows;
  const E* eps;
  size_t eps_bs;
  const float2* in;
  float2* out;
  size_t bs;
  const Coef<double>* cx;
  const Coef<double>* cy;
  const double* k2;
  const KState* st;
};

template <int POL, typename E>
__global__ void __launch_bounds__(128) k_arnoldi_mv64(Mv64Args<POL, E> a) {
  const int b = blockIdx.z;
  if (!a.st[b].active) return;
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= a.ny) return;
  const int i0 = blockIdx.y * a.rows;
  const int i1 = min(i0 + a.rows, a.nx);
  const float2* x = a.in + b * a.bs;
  float2* y = a.out + b * a.bs;
  const Coef<double> cyj = a.cy[(size_t)b * a.ny + j];
  auto ep = [&](int i, double2 v, double2) { y[(size_t)i * a.ny + j] = to_f(v); };
  stencil_column<double, POL, decltype(ep), false, E, float2>(
      a.nx, a.ny, j, i0, i1, x, a.eps + b * a.eps_bs, a.cx + (size_t)b * a.nx, cyj, a.k2[b], ep);
}

// ----------------------------------------------------------- multi-dot
// d_k = sum_n conj(V_k[n]) w[n], k = 0..j ; H[j][k] (+)= sc_k d_k
struct DotArgs {
  size_t n;
  int B, m, j, accumulate;
  const float2* V;  // V_k of problem b at V + (k*B + b)*n
  KCtx ctx;
};

__global__ void __launch_bounds__(RED_THREADS) k_multidot(DotArgs a) {
  const int b = blockIdx.y;
  KState* st = a.ctx.st + b;
  if (!st->active) return;
  const int nv = a.j + 1;
  const unsigned nblk = gridDim.x;
  const float2* w = a.V + ((size_t)(a.j + 1) * a.B + b) * a.n;
  __shared__ float smf[2 * DOT_GROUP * 32];
  double* part = a.ctx.partial + (size_t)b * a.ctx.part_stride;
  const size_t stride = (size_t)nblk * blockDim.x;
  for (int g0 = 0; g0 < nv; g0 += DOT_GROUP) {
    float2 acc[DOT_GROUP];
    const float2* vp[DOT_GROUP];  // vector bases, computed once per group
#pragma unroll
    for (int k = 0; k < DOT_GROUP; ++k) {
      acc[k] = make_float2(0.f, 0.f);
      vp[k] = a.V + ((size_t)(g0 + k) * a.B + b) * a.n;
    }
    if ((a.n & 1) == 0) {
      // two cells per load (16-byte aligned: every vector starts at an even cell)
      const float4* w4 = (const float4*)w;
      for (size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x; q < (a.n >> 1); q += stride) {
        const float4 wv = w4[q];
#pragma unroll
        for (int k = 0; k < DOT_GROUP; ++k) {
          if (g0 + k < nv) {
            const float4 v = ((const float4*)vp[k])[q];
            acc[k].x += v.x * wv.x + v.y * wv.y + v.z * wv.z + v.w * wv.w;
            acc[k].y += v.x * wv.y - v.y * wv.x + v.z * wv.w - v.w * wv.z;
          }
        }
      }
    } else {
      for (size_t n = (size_t)blockIdx.x * blockDim.x + threadIdx.x; n < a.n; n += stride) {
        const float2 wv = w[n];
#pragma unroll
        for (int k = 0; k < DOT_GROUP; ++k) {
          if (g0 + k < nv) {
            const float2 v = vp[k][n];
            acc[k].x += v.x * wv.x + v.y * wv.y;
            acc[k].y += v.x * wv.y - v.y * wv.x;
          }
        }
      }
    }
    float fv[2 * DOT_GROUP];
#pragma unroll
    for (int k = 0; k < DOT_GROUP; ++k) {
      fv[2 * k] = acc[k].x;
      fv[2 * k + 1] = acc[k].y;
    }
    double tot[1];
    block_sum_f<2 * DOT_GROUP>(fv, smf, tot, threadIdx.x);
    const int kk = threadIdx.x >> 1;
    if (threadIdx.x < 2 * DOT_GROUP && g0 + kk < nv)
      part[(size_t)blockIdx.x * 2 * (a.m + 1) + 2 * g0 + threadIdx.x] = tot[0];
    __syncthreads();
  }
  if (!last_block(a.ctx.counter + 2 * b, nblk)) return;
  // fixed-order reduction over blocks: one warp per vector, lanes stride the
  // partials, then a shuffle tree (deterministic)
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const size_t ps = 2 * (size_t)(a.m + 1);
  for (int k = warp; k < nv; k += nw) {
    double re = 0.0, im = 0.0;
    for (unsigned q = lane; q < nblk; q += 32) {
      re += __ldcg(part + q * ps + 2 * k);
      im += __ldcg(part + q * ps + 2 * k + 1);
    }
    re = warp_sum(re);
    im = warp_sum(im);
    if (lane == 0) {
      const double s = a.ctx.sc[(size_t)b * (a.m + 1) + k];
      const double2 h = make_double2(s * re, s * im);
      double2* Hc = a.ctx.H + ((size_t)b * a.m + a.j) * (a.m + 1);  // column j
      a.ctx.hpass[(size_t)b * (a.m + 1) + k] = h;
      Hc[k] = a.accumulate ? cadd(Hc[k], h) : h;
    }
  }
}

// ------------------------------------------------------------ update
// w -= sum_k V_k (sc_k h_k); final pass: ||w|| -> Givens -> residual estimate
struct UpdArgs {
  size_t n;
  int B, m, j, final_pass;
  float2* V;
  KCtx ctx;
};

// Givens update of Hessenberg column j (FP64), run by the whole last block:
// the column and the previous rotations are staged in shared memory so the
// serial part touches no global memory.
__device__ void givens_finish(const UpdArgs& a, int b, double hn) {
  KCtx& c = const_cast<KCtx&>(a.ctx);
  KState* st = c.st + b;
  const int m = a.m, j = a.j;
  double2* Hc = c.H + ((size_t)b * m + j) * (m + 1);
  double* cs = c.cs + (size_t)b * m;
  double2* sn = c.sn + (size_t)b * m;
  double2* gam = c.gam + (size_t)b * (m + 1);
  __shared__ double2 sH[66];
  __shared__ double2 sSn[64];
  __shared__ double sCs[64];
  for (int k = threadIdx.x; k <= j; k += blockDim.x) {
    sH[k] = Hc[k];
    if (k < j) {
      sCs[k] = cs[k];
      sSn[k] = sn[k];
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    sH[j + 1] = make_double2(hn, 0.0);
    for (int k = 0; k < j; ++k) {
      const double2 h0 = sH[k], h1 = sH[k + 1];
      // [c s; -conj(s) c] [h0; h1]
      sH[k] = cadd(cscale(h0, sCs[k]), cmul(sSn[k], h1));
      sH[k + 1] = csub(cscale(h1, sCs[k]), cmulc(sSn[k], h0));
    }
    const double2 av = sH[j];
    const double aa = sqrt(av.x * av.x + av.y * av.y);
    double cj;
    double2 sj, rj;
    if (aa == 0.0) {
      cj = 0.0;
      sj = make_double2(1.0, 0.0);
      rj = make_double2(hn, 0.0);
    } else {
      const double t = sqrt(aa * aa + hn * hn);
      cj = aa / t;
      const double2 ph = make_double2(av.x / aa, av.y / aa);
      sj = cscale(ph, hn / t);  // (a/|a|) conj(b)/t with b = hn real
      rj = cscale(ph, t);
    }
    cs[j] = cj;
    sn[j] = sj;
    sH[j] = rj;
    sH[j + 1] = make_double2(0.0, 0.0);
    const double2 g = gam[j];
    gam[j + 1] = cscale(cmulc(sj, g), -1.0);
    gam[j] = cscale(g, cj);
    const double2 gn = gam[j + 1];
    const double res = sqrt(gn.x * gn.x + gn.y * gn.y);
    st->res_est = res;
    st->ncols = j + 1;
    st->iters += 1;
    const bool breakdown = !(hn > 1e-30);  // basis vectors have unit norm
    c.sc[(size_t)b * (m + 1) + j + 1] = breakdown ? 0.0 : 1.0 / hn;
    if (!isfinite(res) || !isfinite(hn)) {
      st->nan = 1;
      st->active = 0;
    } else if (res <= st->thresh || breakdown || j + 1 >= m || st->iters >= c.max_iters) {
      st->active = 0;
    }
  }
  __syncthreads();
  for (int k = threadIdx.x; k <= j + 1; k += blockDim.x) Hc[k] = sH[k];
}

__global__ void __launch_bounds__(RED_THREADS) k_update(UpdArgs a) {
  const int b = blockIdx.y;
  KState* st = a.ctx.st + b;
  if (!st->active) return;
  const int nv = a.j + 1;
  __shared__ float2 u[65];
  for (int k = threadIdx.x; k < nv; k += blockDim.x) {
    const double s = a.ctx.sc[(size_t)b * (a.m + 1) + k];
    const double2 h = a.ctx.hpass[(size_t)b * (a.m + 1) + k];
    u[k] = make_float2((float)(s * h.x), (float)(s * h.y));
  }
  __syncthreads();
  float2* w = a.V + ((size_t)(a.j + 1) * a.B + b) * a.n;
  const unsigned nblk = gridDim.x;
  const size_t stride = (size_t)nblk * blockDim.x;
  float nrm = 0.f;
  constexpr int G = 8;  // basis vectors loaded together (predicated) per group
  const float2* vb = a.V + (size_t)b * a.n;  // vector k at vb + k * B * n
  const size_t vs = (size_t)a.B * a.n;
  if ((a.n & 1) == 0) {
    // two cells per load (16-byte aligned: every vector starts at an even cell)
    float4* w4 = (float4*)w;
    for (size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x; q < (a.n >> 1); q += stride) {
      float4 wv = w4[q];
      for (int g0 = 0; g0 < nv; g0 += G) {
        float4 v[G];
#pragma unroll
        for (int k = 0; k < G; ++k)
          v[k] = (g0 + k < nv) ? ((const float4*)(vb + (size_t)(g0 + k) * vs))[q]
                               : make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
        for (int k = 0; k < G; ++k) {
          const float2 c = u[g0 + k < nv ? g0 + k : 0];
          if (g0 + k < nv) {
            wv.x -= v[k].x * c.x - v[k].y * c.y;
            wv.y -= v[k].x * c.y + v[k].y * c.x;
            wv.z -= v[k].z * c.x - v[k].w * c.y;
            wv.w -= v[k].z * c.y + v[k].w * c.x;
          }
        }
      }
      w4[q] = wv;
      nrm += wv.x * wv.x + wv.y * wv.y + wv.z * wv.z + wv.w * wv.w;
    }
  } else {
    for (size_t n = (size_t)blockIdx.x * blockDim.x + threadIdx.x; n < a.n; n += stride) {
      float2 wv = w[n];
      for (int g0 = 0; g0 < nv; g0 += G) {
        float2 v[G];
#pragma unroll
        for (int k = 0; k < G; ++k)
          v[k] = (g0 + k < nv) ? vb[(size_t)(g0 + k) * vs + n] : make_float2(0.f, 0.f);
#pragma unroll
        for (int k = 0; k < G; ++k) {
          const float2 c = u[g0 + k < nv ? g0 + k : 0];
          if (g0 + k < nv) {
            wv.x -= v[k].x * c.x - v[k].y * c.y;
            wv.y -= v[k].x * c.y + v[k].y * c.x;
          }
        }
      }
      w[n] = wv;
      nrm += wv.x * wv.x + wv.y * wv.y;
    }
  }
  if (!a.final_pass) return;
  __shared__ double sm[32];
  __shared__ float smf[32];
  float accf[1] = {nrm};
  double tot[1];
  block_sum_f<1>(accf, smf, tot, threadIdx.x);
  double* part = a.ctx.partial + (size_t)b * a.ctx.part_stride;
  if (threadIdx.x == 0) part[blockIdx.x] = tot[0];
  if (!last_block(a.ctx.counter + 2 * b + 1, nblk)) return;
  double s[1] = {0.0};
  for (unsigned q = threadIdx.x; q < nblk; q += blockDim.x) s[0] += __ldcg(part + q);
  block_sum<1>(s, sm);
  __shared__ double s_hn;
  if (threadIdx.x == 0) s_hn = sqrt(s[0]);
  __syncthreads();
  givens_finish(a, b, s_hn);
}

// ------------------------------------------------- triangular solve + update
// y = R^{-1} gamma for the k columns of this cycle, one block per problem:
// R staged in shared memory, column-oriented back substitution.
__global__ void k_trisolve(KCtx c, int B, int m) {
  const int b = blockIdx.x;
  const KState* st = c.st + b;
  const int k = st->ncols;
  if (k == 0) return;
  // packed upper triangle: R[row][col] (row <= col) at col*(col+1)/2 + row
  __shared__ double2 sR[64 * 65 / 2];
  __shared__ double2 sT[64];
  for (int col = 0; col < k; ++col)
    for (int row = threadIdx.x; row <= col; row += blockDim.x)
      sR[col * (col + 1) / 2 + row] = c.H[((size_t)b * m + col) * (m + 1) + row];
  for (int r = threadIdx.x; r < k; r += blockDim.x) sT[r] = c.gam[(size_t)b * (m + 1) + r];
  __syncthreads();
  double2* y = c.y + (size_t)b * m;
  for (int r = k - 1; r >= 0; --r) {
    const double2 d = sR[r * (r + 1) / 2 + r];
    const double dd = d.x * d.x + d.y * d.y;
    const double2 yr = dd > 0 ? cscale(cmulc(d, sT[r]), 1.0 / dd) : make_double2(0.0, 0.0);
    for (int q = threadIdx.x; q < r; q += blockDim.x)
      sT[q] = csub(sT[q], cmul(sR[r * (r + 1) / 2 + q], yr));
    if (threadIdx.x == 0) y[r] = yr;
    __syncthreads();
  }
}

struct XupArgs {
  size_t n;
  int B, m, flexible;
  const float2* V;  // basis (unscaled)
  const float2* Z;  // preconditioned basis (flexible)
  double2* x;
  double xscale;    // 1/scale: corrections of the non-dimensional system
  KCtx ctx;
};

// S + E += (h + l) * v with h*v exact (FMA TwoProd) and the sum by Knuth's
// TwoSum: a float-float accumulation on the FP32 pipe (GB300's FP64 rate
// would make a double accumulation of 30+ terms per cell the bottleneck of
// this otherwise bandwidth-bound kernel).
__device__ __forceinline__ void ff_acc(float& S, float& E, float h, float l, float v) {
  const float p = __fmul_rn(h, v);
  const float e = __fadd_rn(__fmaf_rn(h, v, -p), __fmul_rn(l, v));
  const float t = __fadd_rn(S, p);
  const float bb = __fsub_rn(t, S);
  const float err = __fadd_rn(__fsub_rn(S, __fsub_rn(t, bb)), __fsub_rn(p, bb));
  S = t;
  E = __fadd_rn(E, __fadd_rn(err, e));
}

__global__ void __launch_bounds__(RED_THREADS) k_xupdate(XupArgs a) {
  const int b = blockIdx.y;
  const KState* st = a.ctx.st + b;
  const int k = st->ncols;
  if (k == 0 || st->done) return;
  // y_q (times the basis scale) can lie far outside the float range (tiny or
  // huge right-hand sides), so the float-float sum runs on y_q / ymax and
  // the FP64 result is scaled back by ymax.
  __shared__ double2 yd[64];
  __shared__ float4 cy[64];  // (re hi, re lo, im hi, im lo) of y_q / ymax
  __shared__ double ymax;
  for (int q = threadIdx.x; q < k; q += blockDim.x) {
    double2 yy = a.ctx.y[(size_t)b * a.m + q];
    if (!a.flexible) yy = cscale(yy, a.ctx.sc[(size_t)b * (a.m + 1) + q]);
    yd[q] = yy;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double mx = 0.0;
    for (int q = 0; q < k; ++q) mx = fmax(mx, fmax(fabs(yd[q].x), fabs(yd[q].y)));
    ymax = (mx > 0.0 && mx < INFINITY) ? mx : 1.0;
  }
  __syncthreads();
  for (int q = threadIdx.x; q < k; q += blockDim.x) {
    const double yr = yd[q].x / ymax, yi = yd[q].y / ymax;
    const float rh = (float)yr, ih = (float)yi;
    cy[q] = make_float4(rh, (float)(yr - (double)rh), ih, (float)(yi - (double)ih));
  }
  __syncthreads();
  const double ys = ymax;
  const float2* base = a.flexible ? a.Z : a.V;
  double2* x = a.x + b * a.n;
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  for (size_t n = (size_t)blockIdx.x * blockDim.x + threadIdx.x; n < a.n; n += stride) {
    float sr = 0.f, er = 0.f, si = 0.f, ei = 0.f;
    constexpr int G = 8;
    for (int q0 = 0; q0 < k; q0 += G) {
      float2 v[G];
#pragma unroll
      for (int q = 0; q < G; ++q)
        v[q] = (q0 + q < k) ? base[((size_t)(q0 + q) * a.B + b) * a.n + n] : make_float2(0.f, 0.f);
#pragma unroll
      for (int q = 0; q < G; ++q) {
        if (q0 + q >= k) break;
        const float4 y = cy[q0 + q];
        ff_acc(sr, er, y.x, y.y, v[q].x);    // + Re y Re v
        ff_acc(sr, er, -y.z, -y.w, v[q].y);  // - Im y Im v
        ff_acc(si, ei, y.x, y.y, v[q].y);    // + Re y Im v
        ff_acc(si, ei, y.z, y.w, v[q].x);    // + Im y Re v
      }
    }
    // The cycle solved A' d = r with A' = scale*A and r the residual of
    // A' x = scale*b, so d is already a correction of x in SI units.
    const double2 xo = x[n];
    x[n] = make_double2(xo.x + ys * ((double)sr + (double)er), xo.y + ys * ((double)si + (double)ei));
  }
}

__global__ void k_to_f32(const double* in, float* out, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x)
    out[i] = (float)in[i];
}

__global__ void k_zero_c128(double2* x, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x)
    x[i] = make_double2(0.0, 0.0);
}

// ----------------------------------------------------------- workspace
static size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

int fused_max_blocks() { return 2 * sm_count(); }

int reduction_blocks(size_t n, int B) {
  const long target = 8L * sm_count();
  long nb = (target + B - 1) / B;
  long cap = (long)((n + RED_THREADS - 1) / RED_THREADS);
  return (int)std::max(1L, std::min(nb, cap));
}

KLayout klayout(const KrylovProblem& P, const cev_solve_opts& o, size_t pc_bytes) {
  KLayout L{};
  const size_t N = P.n;
  const int B = P.B, m = o.restart;
  L.nblk = reduction_blocks(N, B);
  L.part_stride = std::max((size_t)L.nblk * 2 * (m + 1), P.res_blocks);
  size_t off = 0;
  auto take = [&](size_t bytes) {
    size_t at = off;
    off = align256(off + bytes);
    return at;
  };
  L.extra = take(P.extra_bytes);
  L.V = take(sizeof(float2) * N * B * (m + 1));
  L.Z = take(o.precond != CEV_PRECOND_NONE ? sizeof(float2) * N * B * m : 0);
  L.partial = take(sizeof(double) * L.part_stride * B);
  L.counter = take(sizeof(unsigned) * (2 * B + 4 * B));  // + fused-cycle barrier words
  L.st = take(sizeof(KState) * B);
  L.H = take(sizeof(double2) * (size_t)B * m * (m + 1));
  L.cs = take(sizeof(double) * (size_t)B * m);
  L.sn = take(sizeof(double2) * (size_t)B * m);
  L.gam = take(sizeof(double2) * (size_t)B * (m + 1));
  L.sc = take(sizeof(double) * (size_t)B * (m + 1));
  L.y = take(sizeof(double2) * (size_t)B * m);
  L.hpass = take(sizeof(double2) * (size_t)B * (m + 1));
  // fused cycle (<= FUSED_MAX_BATCH problems): per problem two dot-pass
  // regions and the norm partials, then one stage per problem
  L.fpart = take(B <= FUSED_MAX_BATCH
                     ? sizeof(double) * (size_t)fused_max_blocks() * (4 * (m + 1) + 1) +
                           (size_t)B * cycle_stage_bytes()
                     : 0);
  L.pc = off;
  off = align256(off + pc_bytes);
  L.total = off;
  return L;
}

static KrylovProblem stencil_problem(const cev_fdfd_plan_s* p) {
  KrylovProblem P;
  P.B = p->batch;
  P.n = p->n();
  dim3 g, bl;
  int rows;
  launch_geometry(p->nx, p->ny, p->batch, g, bl, rows);
  P.res_blocks = (size_t)g.x * g.y;
  P.extra_bytes = sizeof(float2) * p->n() * p->batch;  // float copy of (complex) eps
  return P;
}

// ------------------------------------------------------------ the driver
int krylov_run(const KrylovProblem& P, const KrylovOps& ops, const cev_solve_opts& o,
               const double2* bvec, double2* xvec, cev_solve_info* info, void* ws,
               size_t ws_bytes, cudaStream_t s) {
  const size_t N = P.n;
  const int B = P.B, m = o.restart;
  const bool flexible = o.precond != CEV_PRECOND_NONE;
  const KLayout L = klayout(P, o, 0);
  CEV_REQUIRE(ws_bytes >= L.pc, "workspace too small");
  char* w = (char*)ws;
  KCtx c;
  c.st = (KState*)(w + L.st);
  c.partial = (double*)(w + L.partial);
  c.part_stride = L.part_stride;
  c.counter = (unsigned*)(w + L.counter);
  c.H = (double2*)(w + L.H);
  c.cs = (double*)(w + L.cs);
  c.sn = (double2*)(w + L.sn);
  c.gam = (double2*)(w + L.gam);
  c.sc = (double*)(w + L.sc);
  c.y = (double2*)(w + L.y);
  c.hpass = (double2*)(w + L.hpass);
  c.fpart = (double*)(w + L.fpart);
  c.bar = c.counter + 2 * B;
  c.tol = o.tol;
  c.inner_rtol = o.inner_rtol;
  c.max_iters = o.max_iters;
  float2* V = (float2*)(w + L.V);
  float2* Z = (float2*)(w + L.Z);
  CEV_REQUIRE(!flexible || ops.precond, "preconditioner not available for this operator");

  CEV_CUDA(cudaMemsetAsync(c.counter, 0, sizeof(unsigned) * (2 * B + 4 * B), s));
  const bool fused = ops.cycle && !flexible && B <= FUSED_MAX_BATCH;
  CEV_CUDA(cudaMemsetAsync(c.st, 0, sizeof(KState) * B, s));
  if (!o.use_x0)
    k_zero_c128<<<std::min(ceil_div(N * B, 256), 8u * sm_count()), 256, 0, s>>>(xvec, N * B);
  const dim3 rg(L.nblk, B, 1);
  k_bnorm<<<rg, RED_THREADS, 0, s>>>(bvec, ops.bscale, N, c);
  CEV_CHECK_LAUNCH("k_bnorm");
  int rc = ops.residual(c, V, s);
  if (rc != CEV_OK) return rc;

  std::vector<KState> hst(B);
  std::vector<double> best(B, INFINITY);
  std::vector<int> stall(B, 0), status(B, CEV_NOT_CONVERGED), cycles(B, 0);
  for (int cyc = 0;; ++cyc) {
    CEV_CUDA(cudaMemcpyAsync(hst.data(), c.st, sizeof(KState) * B, cudaMemcpyDeviceToHost, s));
    CEV_CUDA(cudaStreamSynchronize(s));
    bool any = false, changed = false;
    for (int b = 0; b < B; ++b) {
      KState& q = hst[b];
      if (q.fault) {
        set_error("a bounded device wait (fused GMRES cycle or TMA matvec) timed out");
        return CEV_ERR_CUDA;
      }
      if (q.done) continue;
      cycles[b] = cyc;
      const double rel = q.bnorm > 0 ? q.beta / q.bnorm : 0.0;
      int stt = -100;
      if (q.nan || !std::isfinite(rel)) stt = CEV_ERR_NUMERIC;
      else if (q.bnorm == 0 || rel <= o.tol) stt = CEV_OK;
      else if (q.iters >= o.max_iters) stt = CEV_NOT_CONVERGED;
      else {
        if (rel < 0.9 * best[b]) {
          best[b] = rel;
          stall[b] = 0;
        } else if (++stall[b] > o.max_stall) {
          stt = CEV_STAGNATED;
        }
      }
      if (stt != -100) {
        status[b] = stt;
        q.done = 1;
        q.active = 0;
        changed = true;
      } else {
        any = true;
      }
    }
    if (changed)
      CEV_CUDA(cudaMemcpyAsync(c.st, hst.data(), sizeof(KState) * B, cudaMemcpyHostToDevice, s));
    if (!any) break;
    if (fused) {
      CEV_CUDA(cudaMemsetAsync(c.bar, 0, sizeof(unsigned) * 4 * B, s));
      if ((rc = ops.cycle(c, V, s)) != CEV_OK) return rc;
    }
    for (int j = 0; j < (fused ? 0 : m); ++j) {
      const float2* vin = V + (size_t)j * B * N;
      float2* vout = V + (size_t)(j + 1) * B * N;
      if (flexible) {
        float2* zj = Z + (size_t)j * B * N;
        if ((rc = ops.precond(c, j, vin, zj, s)) != CEV_OK) return rc;
        if ((rc = ops.matvec(c, j, zj, 0, vout, s)) != CEV_OK) return rc;
      } else {
        if ((rc = ops.matvec(c, j, vin, 1, vout, s)) != CEV_OK) return rc;
      }
      for (int pass = 0; pass < (o.reorth ? 2 : 1); ++pass) {
        const bool final_pass = pass == (o.reorth ? 1 : 0);
        DotArgs da{N, B, m, j, pass, V, c};
        k_multidot<<<rg, RED_THREADS, 0, s>>>(da);
        UpdArgs ua{N, B, m, j, final_pass ? 1 : 0, V, c};
        k_update<<<rg, RED_THREADS, 0, s>>>(ua);
      }
      CEV_CHECK_LAUNCH("arnoldi step");
      if (ops.check_each_step && j + 1 < m) {
        CEV_CUDA(cudaMemcpyAsync(hst.data(), c.st, sizeof(KState) * B, cudaMemcpyDeviceToHost, s));
        CEV_CUDA(cudaStreamSynchronize(s));
        bool left = false;
        for (int b = 0; b < B; ++b) left = left || hst[b].active;
        if (!left) break;
      }
    }
    k_trisolve<<<B, 64, 0, s>>>(c, B, m);
    XupArgs xa{N, B, m, flexible ? 1 : 0, V, Z, xvec, 1.0, c};
    k_xupdate<<<rg, RED_THREADS, 0, s>>>(xa);
    CEV_CHECK_LAUNCH("cycle finish");
    if ((rc = ops.residual(c, V, s)) != CEV_OK) return rc;
  }
  int worst = CEV_OK;
  for (int b = 0; b < B; ++b) {
    info[b].status = status[b];
    info[b].iterations = hst[b].iters;
    info[b].cycles = cycles[b];
    info[b].reserved = 0;
    info[b].bnorm = hst[b].bnorm / ops.bscale;
    info[b].residual = hst[b].bnorm > 0 ? hst[b].beta / hst[b].bnorm : 0.0;
    if (status[b] < 0) worst = std::min(worst, status[b]);
    else if (worst >= 0) worst = std::max(worst, status[b]);
  }
  return worst;
}

int validate_opts(const cev_solve_opts& o) {
  CEV_REQUIRE(o.restart >= 1 && o.restart <= 64, "restart must be in [1, 64], got %d", o.restart);
  CEV_REQUIRE(o.tol > 0 && o.tol < 1, "tol must be in (0, 1)");
  CEV_REQUIRE(o.max_iters >= 1, "max_iters must be >= 1");
  CEV_REQUIRE(o.precond == CEV_PRECOND_NONE || o.precond == CEV_PRECOND_SHIFTED_LAPLACIAN ||
                  o.precond == CEV_PRECOND_LEARNED || o.precond == CEV_PRECOND_SEPARABLE ||
                  o.precond == CEV_PRECOND_DIRECT,
              "unknown preconditioner %d", o.precond);
  return CEV_OK;
}

}  // namespace cev

using namespace cev;

extern "C" {

void cev_solve_opts_default(cev_solve_opts* o) {
  if (!o) return;
  o->tol = 1e-6;
  o->inner_rtol = 1e-4;
  o->max_iters = 20000;
  o->restart = 30;
  o->precond = CEV_PRECOND_NONE;
  o->transpose = 0;
  o->use_x0 = 0;
  o->reorth = 0;
  o->max_stall = 20;
  o->mg_levels = 0;
  o->mg_shift = 0.5;
  o->learned = nullptr;
  o->separable = nullptr;
  o->direct = nullptr;
}

size_t cev_fdfd_solve_workspace_size(cev_fdfd_plan p, const cev_solve_opts* opts) {
  if (!p || !opts || opts->restart < 1 || opts->restart > 64) return 0;
  return klayout(stencil_problem(p), *opts, precond_workspace_size(p, *opts)).total;
}

int cev_fdfd_solve(cev_fdfd_plan p, const double* eps, int eps_shared, const void* bvec, void* xvec,
                   const cev_solve_opts* opts, cev_solve_info* info, void* ws, size_t ws_bytes,
                   cudaStream_t s) {
  CEV_REQUIRE(p != nullptr, "plan is NULL");
  CEV_REQUIRE(opts != nullptr, "opts is NULL");
  CEV_REQUIRE(eps && bvec && xvec && info, "NULL argument");
  const cev_solve_opts& o = *opts;
  int rc = validate_opts(o);
  if (rc != CEV_OK) return rc;
  const KrylovProblem P = stencil_problem(p);
  const KLayout L = klayout(P, o, precond_workspace_size(p, o));
  CEV_REQUIRE(ws != nullptr && ws_bytes >= L.total,
              "workspace too small: need %zu bytes, got %zu", L.total, ws_bytes);
  CEV_REQUIRE(((uintptr_t)ws & 255) == 0, "workspace must be 256-byte aligned");
  const size_t N = p->n();
  const int B = p->batch, m = o.restart;
  const int tr = o.transpose ? 1 : 0;
  float* eps32 = (float*)((char*)ws + L.extra);
  const bool ce = p->eps_complex != 0;
  const size_t ne = (eps_shared ? N : N * B) * (ce ? 2 : 1);
  k_to_f32<<<std::min(ceil_div(ne, 256), 8u * sm_count()), 256, 0, s>>>(eps, eps32, ne);
  CEV_CHECK_LAUNCH("k_to_f32");
  dim3 sg, sb;
  int rows;
  launch_geometry(p->nx, p->ny, B, sg, sb, rows);

  KrylovOps ops;
  ops.bscale = p->scale;
  const size_t ebs = eps_shared ? 0 : N;
  ops.residual = [&](const KCtx& c, float2* V0, cudaStream_t st) -> int {
    auto go = [&](auto pol_tag, auto e_tag) {
      constexpr int POL = decltype(pol_tag)::value;
      using E = decltype(e_tag);
      ResArgs<POL, E> a{p->nx, p->ny, rows, 0, m, (const E*)eps, ebs, (const double2*)xvec,
                        (const double2*)bvec, p->scale, p->cx64[tr], p->cy64[tr], p->k2_64, V0, N,
                        c};
      k_residual<POL, E><<<sg, sb, 0, st>>>(a);
    };
    if (p->pol == POL_EZ) {
      if (ce) go(std::integral_constant<int, POL_EZ>{}, double2{});
      else go(std::integral_constant<int, POL_EZ>{}, double{});
    } else {
      if (ce) go(std::integral_constant<int, POL_HZ>{}, double2{});
      else go(std::integral_constant<int, POL_HZ>{}, double{});
    }
    CEV_CHECK_LAUNCH("k_residual");
    return CEV_OK;
  };
  const bool tma_mv = tma_matvec_usable(p, ce);
  const bool exact_mv =
      o.precond == CEV_PRECOND_DIRECT || o.precond == CEV_PRECOND_SHIFTED_LAPLACIAN;
  ops.matvec = [&](const KCtx& c, int j, const float2* in, int use_scale, float2* out,
                   cudaStream_t st) -> int {
    if (exact_mv && !use_scale) {
      auto go = [&](auto pol_tag, auto e_tag) {
        constexpr int POL = decltype(pol_tag)::value;
        using E = decltype(e_tag);
        Mv64Args<POL, E> a{p->nx, p->ny, rows, (const E*)eps, ebs, in, out, N,
                           p->cx64[tr], p->cy64[tr], p->k2_64, c.st};
        k_arnoldi_mv64<POL, E><<<sg, sb, 0, st>>>(a);
      };
      if (p->pol == POL_EZ) {
        if (ce) go(std::integral_constant<int, POL_EZ>{}, double2{});
        else go(std::integral_constant<int, POL_EZ>{}, double{});
      } else {
        if (ce) go(std::integral_constant<int, POL_HZ>{}, double2{});
        else go(std::integral_constant<int, POL_HZ>{}, double{});
      }
      CEV_CHECK_LAUNCH("k_arnoldi_mv64");
      return CEV_OK;
    }
    // TMA needs 16-byte aligned operands; anything else takes the column sweep
    if (tma_mv && (((uintptr_t)in | (uintptr_t)eps32) & 15) == 0)
      return tma_matvec(p, tr, eps32, eps_shared, in, out, c, m, j, use_scale, st);
    auto go = [&](auto pol_tag, auto e_tag) {
      constexpr int POL = decltype(pol_tag)::value;
      using E = decltype(e_tag);
      MvArgs<POL, E> a{p->nx, p->ny, rows, m, j, (const E*)eps32, ebs, in, N, use_scale,
                       out, N, p->cx32[tr], p->cy32[tr], p->k2_32, c};
      k_arnoldi_mv<POL, E><<<sg, sb, 0, st>>>(a);
    };
    if (p->pol == POL_EZ) {
      if (ce) go(std::integral_constant<int, POL_EZ>{}, float2{});
      else go(std::integral_constant<int, POL_EZ>{}, float{});
    } else {
      if (ce) go(std::integral_constant<int, POL_HZ>{}, float2{});
      else go(std::integral_constant<int, POL_HZ>{}, float{});
    }
    CEV_CHECK_LAUNCH("k_arnoldi_mv");
    return CEV_OK;
  };
  // One launch per restart cycle for a small batch (the per-iteration
  // launches are latency-bound there).  CEV_FUSED_CYCLE=0 disables
  // it; CEV_FUSED_BLOCKS=<n> caps its blocks (testing the multi-unit loop).
  int cyc_rows = 0, cyc_tiles = 0, cyc_units = 0, cyc_gp = 0, cyc_blocks = 0;
  const char* fenv = std::getenv("CEV_FUSED_CYCLE");
  const char* benv = std::getenv("CEV_FUSED_BLOCKS");
  if (!(fenv && fenv[0] == '0') && B <= FUSED_MAX_BATCH && o.precond == CEV_PRECOND_NONE &&
      N * B <= FUSED_MAX_CELLS)
    cyc_blocks = cycle_plan(p->nx, p->ny, p->pol, ce ? 1 : 0, B, benv ? std::atoi(benv) : 0,
                            cyc_rows, cyc_tiles, cyc_units, cyc_gp);
  if (cyc_blocks > 0) {
    ops.cycle = [&](const KCtx& c, float2* V, cudaStream_t st) -> int {
      CycArgs a{p->nx, p->ny, cyc_rows, m, o.reorth, cyc_tiles, cyc_units, B, cyc_gp, N,
                ebs, eps32, p->cx32[tr], p->cy32[tr], p->k2_32, V, c};
      return cycle_launch(p->pol, ce ? 1 : 0, cyc_blocks, a, st);
    };
  }
  Precond pc;
  if (o.precond != CEV_PRECOND_NONE) {
    rc = precond_setup(pc, p, o, eps32, eps_shared, (char*)ws + L.pc, s);
    if (rc != CEV_OK) return rc;
    ops.precond = [&](const KCtx& c, int j, const float2* v, float2* z, cudaStream_t st) {
      return precond_apply(pc, c, j, m, v, z, st);
    };
    ops.check_each_step =
        o.precond == CEV_PRECOND_DIRECT || o.precond == CEV_PRECOND_SHIFTED_LAPLACIAN;
  }
  return krylov_run(P, ops, o, (const double2*)bvec, (double2*)xvec, info, ws, ws_bytes, s);
}

}  // extern "C"
