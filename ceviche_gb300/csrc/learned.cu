// Learned right preconditioner for flexible GMRES (CEV_PRECOND_LEARNED).
//
// The network has no counterpart in ceviche: it is the solver add-on that
// acts as an approximate inverse of the non-dimensional Ez operator A'.
//   z = |r| * sc * f(r / |r|, eps, k2)
// (|r| the per-problem RMS of the basis vector, sc the basis vector's scale),
// where f is a 4-level convolutional encoder-decoder on the (nx, ny) grid,
// base width c0 (32 -> 64 -> 128 -> 256 channels), additive skips:
//
//   L0  conv3(8 -> c0)       @1     s1 = A1
//   pool; L1 conv3(c0 -> 2c0) @1/2  s2 = A2
//   pool; L2 conv3(2c0->4c0) @1/4   s3 = A3
//   pool; L3 conv3(4c0->8c0), L4 conv3(8c0->8c0), L5 conv3(8c0->4c0) @1/8
//   U3 = up(A6) + A3;  L6 conv3(4c0->4c0), L7 conv3(4c0->2c0) @1/4
//   U2 = up(A8) + A2;  L8 conv3(2c0->2c0), L9 conv3(2c0->c0)  @1/2
//   U1 = up(A10) + A1; L10 conv3(c0->c0) @1; head 1x1 (c0 -> 2) = (Re z, Im z)
//
// Every conv is followed by ReLU; pooling is 2x2 average, upsampling nearest.
// Input features per cell: Re r, Im r (normalised), k2*eps, a PML indicator,
// sqrt(k2), three zero channels.
//
// Data layout: activations are bf16 NHWC ([batch][nx][ny][C], channels
// contiguous), the grid's own (i, j) order.  Parameters are one fp32 vector:
// per conv layer W[cout][cin][3][3] then b[cout]; then the head W[2][c0], b[2].
//
// Tensor-core paths: the 3x3 convs are implicit GEMMs (bf16 in, fp32
// accumulate).  By default they run on tcgen05 with TMEM accumulators
// (k_conv3_tc, and k_conv3_tcp for single-slab layers).  k_conv3 is the
// mma.sync m16n8k16 alternative: cp.async staging, ldmatrix operands.  The
// data gradient is the same conv with the weights flipped and transposed.
// The weight gradient (k_wgrad3, mma.sync) is a second GEMM that reduces
// over pixels, split over blocks, with fp32 atomics.
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "krylov.hpp"

namespace cev {
namespace nn {

using bf16 = __nv_bfloat16;

constexpr int CIN0 = 8;    // input feature channels (5 used)
constexpr int NLAYER = 11;

struct LayerSpec {
  int cin, cout, level;
};

static void layer_specs(int c0, LayerSpec* s) {
  const int c1 = c0, c2 = 2 * c0, c3 = 4 * c0, c4 = 8 * c0;
  const LayerSpec t[NLAYER] = {{CIN0, c1, 0}, {c1, c2, 1}, {c2, c3, 2}, {c3, c4, 3},
                               {c4, c4, 3},   {c4, c3, 3}, {c3, c3, 2}, {c3, c2, 2},
                               {c2, c2, 1},   {c2, c1, 1}, {c1, c1, 0}};
  for (int l = 0; l < NLAYER; ++l) s[l] = t[l];
}

static inline int round_up(int a, int b) { return (a + b - 1) / b * b; }

static size_t param_count(int c0) {
  LayerSpec s[NLAYER];
  layer_specs(c0, s);
  size_t n = 0;
  for (int l = 0; l < NLAYER; ++l) n += (size_t)s[l].cout * s[l].cin * 9 + s[l].cout;
  return n + 2 * (size_t)c0 + 2;
}

// ------------------------------------------------------------------ PTX helpers
__device__ __forceinline__ void cp_async16(void* smem, const void* gmem, bool valid) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  const int sz = valid ? 16 : 0;  // 0: the 16 bytes are zero-filled, nothing is read
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(s), "l"(gmem), "r"(sz));
}
__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;\n" ::); }
__device__ __forceinline__ void cp_wait_all() { asm volatile("cp.async.wait_group 0;\n" ::); }

__device__ __forceinline__ void ldsm_x4(unsigned (&r)[4], const void* p) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(p);
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];\n"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
               : "r"(s));
}
__device__ __forceinline__ void ldsm_x4_t(unsigned (&r)[4], const void* p) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(p);
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0,%1,%2,%3}, [%4];\n"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
               : "r"(s));
}
// d += a (16x16, row) * b (16x8, col); bf16 inputs, fp32 accumulators
__device__ __forceinline__ void mma16816(float (&d)[4], const unsigned (&a)[4], unsigned b0,
                                         unsigned b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, "
      "{%8,%9}, {%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// ------------------------------------------------------------ 3x3 conv (fwd / dgrad)
// out[p][co] = act(bias[co] + sum_{tap, ci} in[p + off(tap)][ci] * w[tap][co][ci])
// (+ the old out when accumulating).  Zero padding at the grid edges.
struct ConvArgs {
  const bf16* in;
  int cin, in_cs;      // channels used, channel stride (multiple of 8)
  const bf16* w;       // [9][cout][cinp], zero beyond cin
  int cinp;            // multiple of 32
  const float* bias;   // [cout] or null
  bf16* out;
  int cout, out_cs;    // cout multiple of 8
  int H, W;
  long long npix;      // batch * H * W
  int relu, accumulate;
};

constexpr int CBM = 128, CBK = 32, CPAD = 40;  // smem rows of 32 bf16 + 8 pad (80 B)

template <int BN>
__global__ void __launch_bounds__(128) k_conv3(ConvArgs a) {
  __shared__ __align__(16) bf16 sA[2][CBM * CPAD];
  __shared__ __align__(16) bf16 sB[2][BN * CPAD];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const long long m0 = (long long)blockIdx.x * CBM;
  const int n0 = blockIdx.y * BN;
  const long long HW = (long long)a.H * a.W;
  // each thread stages one pixel row of the A tile (4 chunks of 8 channels)
  const long long p = m0 + tid;
  const bool prow = p < a.npix;
  long long pb = 0;
  int pi = 0, pj = 0;
  if (prow) {
    pb = p / HW;
    const long long rem = p - pb * HW;
    pi = (int)(rem / a.W);
    pj = (int)(rem - (long long)pi * a.W);
  }
  const int nck = a.cinp / CBK;
  const int ksteps = 9 * nck;
  auto load = [&](int ks, int buf) {
    const int tap = ks / nck, c0 = (ks - tap * nck) * CBK;
    const int ii = pi + tap / 3 - 1, jj = pj + tap % 3 - 1;
    const bool pv = prow && ii >= 0 && ii < a.H && jj >= 0 && jj < a.W;
    const long long q = pb * HW + (long long)ii * a.W + jj;
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      const int ch = c0 + c * 8;
      const bool v = pv && ch < a.cin;
      const void* src = v ? (const void*)(a.in + q * a.in_cs + ch) : (const void*)a.in;
      cp_async16(&sA[buf][tid * CPAD + c * 8], src, v);
    }
#pragma unroll
    for (int t = 0; t < BN / 32; ++t) {
      const int idx = tid + t * 128;
      const int row = idx >> 2, c = idx & 3;
      const int co = n0 + row;
      const bool v = co < a.cout;
      const void* src =
          v ? (const void*)(a.w + ((size_t)tap * a.cout + co) * a.cinp + c0 + c * 8) : (const void*)a.w;
      cp_async16(&sB[buf][row * CPAD + c * 8], src, v);
    }
    cp_commit();
  };
  float acc[2][BN / 8][4];
#pragma unroll
  for (int mi = 0; mi < 2; ++mi)
#pragma unroll
    for (int ni = 0; ni < BN / 8; ++ni)
#pragma unroll
      for (int e = 0; e < 4; ++e) acc[mi][ni][e] = 0.f;
  load(0, 0);
  for (int ks = 0; ks < ksteps; ++ks) {
    const int buf = ks & 1;
    cp_wait_all();
    __syncthreads();
    if (ks + 1 < ksteps) load(ks + 1, buf ^ 1);
    const bf16* As = sA[buf];
    const bf16* Bs = sB[buf];
#pragma unroll
    for (int kk = 0; kk < CBK; kk += 16) {
      unsigned af[2][4];
#pragma unroll
      for (int mi = 0; mi < 2; ++mi) {
        const int row = warp * 32 + mi * 16 + (lane & 7) + ((lane >> 3) & 1) * 8;
        const int col = kk + (lane >> 4) * 8;
        ldsm_x4(af[mi], &As[row * CPAD + col]);
      }
#pragma unroll
      for (int nj = 0; nj < BN / 16; ++nj) {
        unsigned bfr[4];
        const int q = lane >> 3;
        const int row = nj * 16 + (lane & 7) + (q >> 1) * 8;
        const int col = kk + (q & 1) * 8;
        ldsm_x4(bfr, &Bs[row * CPAD + col]);
#pragma unroll
        for (int mi = 0; mi < 2; ++mi) {
          mma16816(acc[mi][2 * nj], af[mi], bfr[0], bfr[1]);
          mma16816(acc[mi][2 * nj + 1], af[mi], bfr[2], bfr[3]);
        }
      }
    }
  }
#pragma unroll
  for (int mi = 0; mi < 2; ++mi)
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const long long pp = m0 + warp * 32 + mi * 16 + (lane >> 2) + h * 8;
      if (pp >= a.npix) continue;
      bf16* o = a.out + pp * a.out_cs;
#pragma unroll
      for (int ni = 0; ni < BN / 8; ++ni) {
        const int co = n0 + ni * 8 + (lane & 3) * 2;
        if (co >= a.cout) continue;
        float v0 = acc[mi][ni][2 * h], v1 = acc[mi][ni][2 * h + 1];
        if (a.bias) {
          v0 += a.bias[co];
          v1 += a.bias[co + 1];
        }
        if (a.accumulate) {
          const __nv_bfloat162 old = *(const __nv_bfloat162*)(o + co);
          v0 += __low2float(old);
          v1 += __high2float(old);
        }
        if (a.relu) {
          v0 = fmaxf(v0, 0.f);
          v1 = fmaxf(v1, 0.f);
        }
        *(__nv_bfloat162*)(o + co) = __floats2bfloat162_rn(v0, v1);
      }
    }
}

// ------------------------------------------------------------ 3x3 conv weight gradient
// dw[co][ci][tap] += sum_p g[p][co] * in[p + off(tap)][ci]
struct WgradArgs {
  const bf16* g;
  int cout, g_cs;
  const bf16* in;
  int cin, in_cs;
  float* dw;
  int H, W;
  long long npix;
  long long chunk;  // pixels per block, multiple of 32
};

constexpr int WPAD = 72;  // smem rows of 64 bf16 + 8 pad (144 B)

__global__ void __launch_bounds__(128) k_wgrad3(WgradArgs a) {
  __shared__ __align__(16) bf16 sG[2][32 * WPAD];
  __shared__ __align__(16) bf16 sX[2][32 * WPAD];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int tap = blockIdx.y;
  const int dy = tap / 3 - 1, dx = tap % 3 - 1;
  const int ntci = (a.cin + 63) / 64;
  const int co0 = (blockIdx.z / ntci) * 64, ci0 = (blockIdx.z % ntci) * 64;
  const long long pbeg = (long long)blockIdx.x * a.chunk;
  const long long pend = pbeg + a.chunk < a.npix ? pbeg + a.chunk : a.npix;
  if (pbeg >= pend) return;  // uniform over the block
  const long long HW = (long long)a.H * a.W;
  auto load = [&](long long pk, int buf) {
#pragma unroll
    for (int t = 0; t < 2; ++t) {
      const int idx = tid + t * 128;
      const int row = idx >> 3, c = idx & 7;
      const long long p = pk + row;
      const bool pv = p < pend;
      const int co = co0 + c * 8;
      const bool vg = pv && co < a.cout;
      cp_async16(&sG[buf][row * WPAD + c * 8], vg ? (const void*)(a.g + p * a.g_cs + co) : (const void*)a.g,
                 vg);
      bool vx = false;
      long long q = 0;
      if (pv) {
        const long long b = p / HW;
        const long long rem = p - b * HW;
        const int i = (int)(rem / a.W) + dy, j = (int)(rem % a.W) + dx;
        vx = i >= 0 && i < a.H && j >= 0 && j < a.W && ci0 + c * 8 < a.cin;
        q = b * HW + (long long)i * a.W + j;
      }
      cp_async16(&sX[buf][row * WPAD + c * 8],
                 vx ? (const void*)(a.in + q * a.in_cs + ci0 + c * 8) : (const void*)a.in, vx);
    }
    cp_commit();
  };
  float acc[2][4][4];
#pragma unroll
  for (int mi = 0; mi < 2; ++mi)
#pragma unroll
    for (int ni = 0; ni < 4; ++ni)
#pragma unroll
      for (int e = 0; e < 4; ++e) acc[mi][ni][e] = 0.f;
  const int wm = (warp >> 1) * 32, wn = (warp & 1) * 32;
  const int nsteps = (int)((pend - pbeg + 31) / 32);
  load(pbeg, 0);
  for (int s = 0; s < nsteps; ++s) {
    const int buf = s & 1;
    cp_wait_all();
    __syncthreads();
    if (s + 1 < nsteps) load(pbeg + (long long)(s + 1) * 32, buf ^ 1);
    const bf16* G = sG[buf];
    const bf16* X = sX[buf];
#pragma unroll
    for (int kk = 0; kk < 32; kk += 16) {
      const int q = lane >> 3;
      unsigned af[2][4];
#pragma unroll
      for (int mi = 0; mi < 2; ++mi) {
        const int krow = kk + (lane & 7) + (q >> 1) * 8;
        const int mcol = wm + mi * 16 + (q & 1) * 8;
        ldsm_x4_t(af[mi], &G[krow * WPAD + mcol]);
      }
#pragma unroll
      for (int nj = 0; nj < 2; ++nj) {
        unsigned bfr[4];
        const int krow = kk + (lane & 7) + (q & 1) * 8;
        const int ncol = wn + nj * 16 + (q >> 1) * 8;
        ldsm_x4_t(bfr, &X[krow * WPAD + ncol]);
#pragma unroll
        for (int mi = 0; mi < 2; ++mi) {
          mma16816(acc[mi][2 * nj], af[mi], bfr[0], bfr[1]);
          mma16816(acc[mi][2 * nj + 1], af[mi], bfr[2], bfr[3]);
        }
      }
    }
  }
#pragma unroll
  for (int mi = 0; mi < 2; ++mi)
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int co = co0 + wm + mi * 16 + (lane >> 2) + h * 8;
      if (co >= a.cout) continue;
#pragma unroll
      for (int ni = 0; ni < 4; ++ni) {
        const int ci = ci0 + wn + ni * 8 + (lane & 3) * 2;
        if (ci < a.cin) atomicAdd(&a.dw[((size_t)co * a.cin + ci) * 9 + tap], acc[mi][ni][2 * h]);
        if (ci + 1 < a.cin)
          atomicAdd(&a.dw[((size_t)co * a.cin + ci + 1) * 9 + tap], acc[mi][ni][2 * h + 1]);
      }
    }
}

// ------------------------------------------------------------ elementwise kernels
union V8 {
  uint4 u;
  __nv_bfloat162 h[4];
};

// g = g * (a > 0), n8 vectors of 8 channels
__global__ void k_relu_mask(bf16* __restrict__ g, const bf16* __restrict__ a, size_t n8) {
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n8;
       e += (size_t)gridDim.x * blockDim.x) {
    V8 gv, av;
    gv.u = ((const uint4*)g)[e];
    av.u = ((const uint4*)a)[e];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const float2 gg = __bfloat1622float2(gv.h[k]), aa = __bfloat1622float2(av.h[k]);
      gv.h[k] = __floats2bfloat162_rn(aa.x > 0.f ? gg.x : 0.f, aa.y > 0.f ? gg.y : 0.f);
    }
    ((uint4*)g)[e] = gv.u;
  }
}

// out[b][i][j] = scale * sum of the 2x2 block of in (out is (Ho, Wo), in (2Ho, 2Wo))
__global__ void k_pool2(const bf16* __restrict__ in, bf16* __restrict__ out, long long nout, int Ho,
                        int Wo, int C, float scale) {
  const int c8n = C / 8;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < nout * c8n;
       e += (long long)gridDim.x * blockDim.x) {
    const long long po = e / c8n;
    const int c8 = (int)(e - po * c8n);
    const long long b = po / ((long long)Ho * Wo);
    const long long rem = po - b * Ho * Wo;
    const int i = (int)(rem / Wo), j = (int)(rem % Wo);
    const long long Wi = 2LL * Wo;
    const long long p00 = (b * 2 * Ho + 2 * i) * Wi + 2 * j;
    const long long src[4] = {p00, p00 + 1, p00 + Wi, p00 + Wi + 1};
    float s[8] = {0, 0, 0, 0, 0, 0, 0, 0};
#pragma unroll
    for (int t = 0; t < 4; ++t) {
      V8 v;
      v.u = *(const uint4*)(in + src[t] * C + c8 * 8);
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        const float2 f = __bfloat1622float2(v.h[k]);
        s[2 * k] += f.x;
        s[2 * k + 1] += f.y;
      }
    }
    V8 o;
#pragma unroll
    for (int k = 0; k < 4; ++k) o.h[k] = __floats2bfloat162_rn(scale * s[2 * k], scale * s[2 * k + 1]);
    *(uint4*)(out + po * C + c8 * 8) = o.u;
  }
}

// out[b][i][j] = scale * in[b][i/2][j/2] (+ add[b][i][j]) (+ out[b][i][j] when accumulating)
__global__ void k_up2(const bf16* __restrict__ in, const bf16* __restrict__ add, bf16* out,
                      long long nout, int Ho, int Wo, int C, float scale, int accumulate) {
  const int c8n = C / 8;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < nout * c8n;
       e += (long long)gridDim.x * blockDim.x) {
    const long long po = e / c8n;
    const int c8 = (int)(e - po * c8n);
    const long long b = po / ((long long)Ho * Wo);
    const long long rem = po - b * Ho * Wo;
    const int i = (int)(rem / Wo), j = (int)(rem % Wo);
    const long long pi = (b * (Ho / 2) + i / 2) * (Wo / 2) + j / 2;
    V8 v, o;
    v.u = *(const uint4*)(in + pi * C + c8 * 8);
    float s[8];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const float2 f = __bfloat1622float2(v.h[k]);
      s[2 * k] = scale * f.x;
      s[2 * k + 1] = scale * f.y;
    }
    if (add) {
      V8 w;
      w.u = *(const uint4*)(add + po * C + c8 * 8);
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        const float2 f = __bfloat1622float2(w.h[k]);
        s[2 * k] += f.x;
        s[2 * k + 1] += f.y;
      }
    }
    if (accumulate) {
      V8 w;
      w.u = *(const uint4*)(out + po * C + c8 * 8);
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        const float2 f = __bfloat1622float2(w.h[k]);
        s[2 * k] += f.x;
        s[2 * k + 1] += f.y;
      }
    }
#pragma unroll
    for (int k = 0; k < 4; ++k) o.h[k] = __floats2bfloat162_rn(s[2 * k], s[2 * k + 1]);
    *(uint4*)(out + po * C + c8 * 8) = o.u;
  }
}

// db[c] += sum_p g[p][c]; C divides 256
__global__ void __launch_bounds__(256) k_bias_grad(const bf16* __restrict__ g, float* db, long long npix,
                                                   int C) {
  __shared__ float s[256];
  const int per = 256 / C;
  const int c = threadIdx.x % C, sub = threadIdx.x / C;
  float acc = 0.f;
  for (long long p = blockIdx.x * (long long)per + sub; p < npix; p += (long long)gridDim.x * per)
    acc += __bfloat162float(g[p * C + c]);
  s[threadIdx.x] = acc;
  __syncthreads();
  if (threadIdx.x < C) {
    float t = 0.f;
    for (int k = 0; k < per; ++k) t += s[k * C + threadIdx.x];
    atomicAdd(&db[threadIdx.x], t);
  }
}

// per-problem RMS of r: nrm[b] = sqrt(mean |r|^2), two passes: RMS_PARTS
// blocks per problem write partial sums, then one thread per problem adds them
constexpr int RMS_PARTS = 32;

__global__ void __launch_bounds__(256) k_rms_part(const float2* __restrict__ r, size_t n,
                                                  double* __restrict__ part) {
  const int b = blockIdx.y;
  const float2* rb = r + (size_t)b * n;
  double acc = 0.0;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n;
       e += (size_t)gridDim.x * blockDim.x) {
    const float2 v = rb[e];
    acc += (double)v.x * v.x + (double)v.y * v.y;
  }
  __shared__ double s[256];
  s[threadIdx.x] = acc;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if (threadIdx.x < w) s[threadIdx.x] += s[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[(size_t)b * RMS_PARTS + blockIdx.x] = s[0];
}

__global__ void k_rms_final(const double* __restrict__ part, size_t n, int B, float* nrm) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= B) return;
  double t = 0.0;
  for (int k = 0; k < RMS_PARTS; ++k) t += part[(size_t)b * RMS_PARTS + k];
  nrm[b] = (float)sqrt(t / (double)n);
}

// input features, bf16 [npix][8]
__global__ void k_prep(const float2* __restrict__ r, const float* __restrict__ eps, int eps_shared,
                       const float* __restrict__ k2, const float* __restrict__ nrm, int B, int H,
                       int W, int npml_x, int npml_y, bf16* __restrict__ x0) {
  const long long HW = (long long)H * W;
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < B * HW;
       p += (long long)gridDim.x * blockDim.x) {
    const int b = (int)(p / HW);
    const long long cell = p - b * HW;
    const int i = (int)(cell / W), j = (int)(cell % W);
    const float s = nrm[b];
    const float inv = s > 0.f ? 1.f / s : 0.f;
    const float2 v = r[p];
    const float e = eps[eps_shared ? cell : p];
    const bool pml = i < npml_x || i >= H - npml_x || j < npml_y || j >= W - npml_y;
    V8 o;
    o.h[0] = __floats2bfloat162_rn(v.x * inv, v.y * inv);
    o.h[1] = __floats2bfloat162_rn(k2[b] * e, pml ? 1.f : 0.f);
    o.h[2] = __floats2bfloat162_rn(sqrtf(k2[b]), 0.f);
    o.h[3] = __floats2bfloat162_rn(0.f, 0.f);
    *(uint4*)(x0 + p * CIN0) = o.u;
  }
}

// z[p] = nrm[b] * mult_b * (bh + Wh a[p]); mult_b = sc[b*sc_stride + sc_index] or 1
template <int C>
__global__ void k_head_fwd(const bf16* __restrict__ a, const float* __restrict__ wh,
                           const float* __restrict__ nrm, const double* __restrict__ sc, int sc_stride,
                           int sc_index, long long npix, long long HW, float2* __restrict__ z) {
  __shared__ float w[2 * C + 2];
  for (int t = threadIdx.x; t < 2 * C + 2; t += blockDim.x) w[t] = wh[t];
  __syncthreads();
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < npix;
       p += (long long)gridDim.x * blockDim.x) {
    const int b = (int)(p / HW);
    float o0 = w[2 * C], o1 = w[2 * C + 1];
#pragma unroll
    for (int c8 = 0; c8 < C / 8; ++c8) {
      V8 v;
      v.u = *(const uint4*)(a + p * C + c8 * 8);
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        const float2 f = __bfloat1622float2(v.h[k]);
        const int c = c8 * 8 + 2 * k;
        o0 += w[c] * f.x + w[c + 1] * f.y;
        o1 += w[C + c] * f.x + w[C + c + 1] * f.y;
      }
    }
    float m = nrm[b];
    if (sc) m *= (float)sc[(size_t)b * sc_stride + sc_index];
    z[p] = make_float2(m * o0, m * o1);
  }
}

// head backward: go = nrm_b * gz; ga[p][c] = go . Wh[:, c]; dWh, dbh accumulated
template <int C>
__global__ void __launch_bounds__(256) k_head_bwd(const bf16* __restrict__ a, const float* __restrict__ wh,
                                                  const float* __restrict__ nrm,
                                                  const float2* __restrict__ gz, long long npix,
                                                  long long HW, bf16* __restrict__ ga,
                                                  float* __restrict__ dwh) {
  __shared__ float w[2 * C];
  __shared__ float red[8][2 * C + 2];
  for (int t = threadIdx.x; t < 2 * C; t += blockDim.x) w[t] = wh[t];
  __syncthreads();
  float dw[2 * C + 2];
#pragma unroll
  for (int t = 0; t < 2 * C + 2; ++t) dw[t] = 0.f;
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < npix;
       p += (long long)gridDim.x * blockDim.x) {
    const int b = (int)(p / HW);
    const float2 g = gz[p];
    const float g0 = nrm[b] * g.x, g1 = nrm[b] * g.y;
    dw[2 * C] += g0;
    dw[2 * C + 1] += g1;
#pragma unroll
    for (int c8 = 0; c8 < C / 8; ++c8) {
      V8 v, o;
      v.u = *(const uint4*)(a + p * C + c8 * 8);
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        const float2 f = __bfloat1622float2(v.h[k]);
        const int c = c8 * 8 + 2 * k;
        dw[c] += g0 * f.x;
        dw[c + 1] += g0 * f.y;
        dw[C + c] += g1 * f.x;
        dw[C + c + 1] += g1 * f.y;
        o.h[k] = __floats2bfloat162_rn(g0 * w[c] + g1 * w[C + c], g0 * w[c + 1] + g1 * w[C + c + 1]);
      }
      *(uint4*)(ga + p * C + c8 * 8) = o.u;
    }
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int t = 0; t < 2 * C + 2; ++t) {
    float v = dw[t];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (lane == 0) red[warp][t] = v;
  }
  __syncthreads();
  for (int t = threadIdx.x; t < 2 * C + 2; t += blockDim.x) {
    float v = 0.f;
    for (int k = 0; k < 8; ++k) v += red[k][t];
    atomicAdd(&dwh[t], v);
  }
}

// packed forward weights wf[tap][co][cip] and data-gradient weights
// wd[tap][ci][cop] = W[co][ci][8 - tap] (flipped, transposed)
__global__ void k_pack(const float* __restrict__ W, int cin, int cout, int cip, int cop,
                       bf16* __restrict__ wf, bf16* __restrict__ wd) {
  const size_t nf = (size_t)9 * cout * cip, nd = (size_t)9 * cin * cop;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < nf + nd;
       e += (size_t)gridDim.x * blockDim.x) {
    if (e < nf) {
      const int ci = (int)(e % cip);
      const size_t r = e / cip;
      const int co = (int)(r % cout), tap = (int)(r / cout);
      wf[e] = __float2bfloat16(ci < cin ? W[((size_t)co * cin + ci) * 9 + tap] : 0.f);
    } else {
      const size_t f = e - nf;
      const int co = (int)(f % cop);
      const size_t r = f / cop;
      const int ci = (int)(r % cin), tap = (int)(r / cin);
      wd[f] = __float2bfloat16(co < cout ? W[((size_t)co * cin + ci) * 9 + (8 - tap)] : 0.f);
    }
  }
}

__global__ void k_adam(float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m,
                       float* __restrict__ v, size_t n, float lr, float b1, float b2, float eps,
                       float bc1, float bc2) {
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n;
       e += (size_t)gridDim.x * blockDim.x) {
    const float gg = g[e];
    const float mm = b1 * m[e] + (1.f - b1) * gg;
    const float vv = b2 * v[e] + (1.f - b2) * gg * gg;
    m[e] = mm;
    v[e] = vv;
    p[e] -= lr * (mm / bc1) / (sqrtf(vv / bc2) + eps);
  }
}

// ------------------------------------------------ 3x3 conv on tcgen05 (TMEM accumulators)
// The conv as an implicit GEMM on the 5th-generation tensor cores.  A CTA
// owns a 16 x 8 pixel tile (M = 128) and BN output channels; one thread
// issues tcgen05.mma (K = 16 per instruction) from shared-memory
// descriptors and the fp32 accumulator tile lives in TMEM (BN columns x 128
// lanes), read back by tcgen05.ld for the fused bias/ReLU epilogue.
//
// Operand layout: K-major, no swizzle, core matrices of 8 rows x 16 B.
//  * A: for each 32-channel slab the 18 x 10 halo tile of the input is
//    staged once as 180 pixel lines of 16 B (8 channels) per 8-channel chunk.
//    An output row of the tile is one 8-row core-matrix group, so the
//    stride-dimension offset is one halo row (160 B) and the leading-
//    dimension offset one channel chunk (2880 B).  Tap (dy, dx) is the same
//    descriptor with its start moved by ((1+dy)*10 + 1+dx) lines: the 9 taps
//    reuse one staged tile instead of nine.
//  * B: the slab's weights for all 9 taps, [tap][BN rows][32 channels] as
//    core matrices (leading offset 128 B, stride offset 512 B).
// Two slabs are in flight when the layer has more than one; an mbarrier per
// stage, armed by tcgen05.commit, tells the loaders when the MMAs reading a
// stage are done.  Every wait is bounded: on timeout the kernel records the
// fault, waits (bounded) for its own MMAs, frees TMEM and returns.

constexpr int HX_TI = 16, HX_TJ = 8;                 // output tile (rows i, columns j)
constexpr int HX_HJ = HX_TJ + 2;                     // halo width
constexpr int HX_LINES = (HX_TI + 2) * HX_HJ;        // 180 pixel lines per channel chunk
constexpr int HX_LBO = HX_LINES * 16;                // 2880 B between 8-channel chunks
constexpr int HX_SBO = HX_HJ * 16;                   // 160 B between output rows
constexpr int HX_SLAB_A = (CBK / 8) * HX_LBO;        // 11520 B per 32-channel slab
constexpr long long TC_SPIN = 1LL << 22;

__device__ int g_tc_fault = 0;

__device__ __forceinline__ unsigned smem_u32(const void* p) {
  return (unsigned)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ bool mbar_wait(unsigned addr, unsigned parity) {
  for (long long i = 0; i < TC_SPIN; ++i) {
    unsigned ok;
    asm volatile(
        "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        "selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(addr), "r"(parity)
        : "memory");
    if (ok) return true;
  }
  return false;
}

// shared-memory matrix descriptor: K-major, no swizzle
__device__ __forceinline__ unsigned long long tc_desc(unsigned saddr, unsigned lbo, unsigned sbo) {
  return (unsigned long long)((saddr >> 4) & 0x3FFFu) |
         ((unsigned long long)((lbo >> 4) & 0x3FFFu) << 16) |
         ((unsigned long long)((sbo >> 4) & 0x3FFFu) << 32) | (1ULL << 46);
}

template <int BN> struct TcGeom {
  static constexpr int TAP_B = BN * CBK * 2;       // one tap's weights: BN x 32 channels
  static constexpr int SLAB = HX_SLAB_A + 9 * TAP_B;
};

template <int BN>
__global__ void __launch_bounds__(128) k_conv3_tc(ConvArgs a) {
  extern __shared__ __align__(128) unsigned char tc_smem[];
  __shared__ __align__(8) unsigned long long mbar[2];
  __shared__ unsigned tslot;
  constexpr int SLAB = TcGeom<BN>::SLAB, TAP_B = TcGeom<BN>::TAP_B;
  // instruction descriptor: f32 accumulate, bf16 A and B, both K-major, N = BN, M = 128
  constexpr unsigned IDESC = (1u << 4) | (1u << 7) | (1u << 10) | ((unsigned)(BN >> 3) << 17) |
                             ((unsigned)(CBM >> 4) << 24);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int tiles_j = (a.W + HX_TJ - 1) / HX_TJ, tiles_i = (a.H + HX_TI - 1) / HX_TI;
  int t = blockIdx.x;
  const int tj = t % tiles_j;
  t /= tiles_j;
  const int ti = t % tiles_i;
  const int b = t / tiles_i;
  const int i0 = ti * HX_TI, j0 = tj * HX_TJ;
  const int n0 = blockIdx.y * BN;
  const long long img = (long long)b * a.H * a.W;
  const int nslab = a.cinp / CBK;
  const unsigned sbase = smem_u32(tc_smem);
  if (tid == 0) {
    for (int q = 0; q < 2; ++q)
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_u32(&mbar[q])));
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(
                     smem_u32(&tslot)),
                 "r"(BN));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n");
  }
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
  const unsigned tmem = tslot;

  auto load = [&](int sl, int st) {
    unsigned char* sa = tc_smem + (size_t)st * SLAB;
    unsigned char* sb = sa + HX_SLAB_A;
    const int c0 = sl * CBK;
    for (int e = tid; e < (CBK / 8) * HX_LINES; e += 128) {
      const int c = e / HX_LINES, L = e - c * HX_LINES;
      const int hr = L / HX_HJ, hc = L - hr * HX_HJ;
      const int i = i0 - 1 + hr, j = j0 - 1 + hc, ch = c0 + c * 8;
      const bool v = i >= 0 && i < a.H && j >= 0 && j < a.W && ch < a.cin;
      const void* src =
          v ? (const void*)(a.in + (img + (long long)i * a.W + j) * a.in_cs + ch) : (const void*)a.in;
      cp_async16(sa + c * HX_LBO + L * 16, src, v);
    }
    for (int e = tid; e < 9 * BN * (CBK / 8); e += 128) {
      const int c = e & 3, rt = e >> 2;
      const int row = rt % BN, tap = rt / BN;
      const int co = n0 + row;
      const bool v = co < a.cout;
      const void* src =
          v ? (const void*)(a.w + ((size_t)tap * a.cout + co) * a.cinp + c0 + c * 8) : (const void*)a.w;
      cp_async16(sb + tap * TAP_B + (row >> 3) * 512 + (row & 7) * 16 + c * 128, src, v);
    }
    cp_commit();
  };

  bool ok = true;
  int issued = -1;
  load(0, 0);
  for (int sl = 0; sl < nslab && ok; ++sl) {
    const int st = sl & 1;
    cp_wait_all();
    asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
    __syncthreads();
    if (tid == 0) {
      asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
      const unsigned sa = sbase + (unsigned)(st * SLAB), sb = sa + HX_SLAB_A;
#pragma unroll
      for (int tap = 0; tap < 9; ++tap) {
        const unsigned aoff = (unsigned)(((tap / 3) * HX_HJ + (tap % 3)) * 16);
#pragma unroll
        for (int kk = 0; kk < CBK / 16; ++kk) {
          const unsigned long long ad = tc_desc(sa + kk * 2 * HX_LBO + aoff, HX_LBO, HX_SBO);
          const unsigned long long bd = tc_desc(sb + tap * TAP_B + kk * 256, 128, 512);
          const unsigned acc = (sl > 0 || tap > 0 || kk > 0) ? 1u : 0u;
          asm volatile(
              "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
              "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
              "l"(ad), "l"(bd), "r"(IDESC), "r"(acc));
        }
      }
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
                       smem_u32(&mbar[st]))
                   : "memory");
    }
    issued = sl;
    if (sl + 1 < nslab) {
      // stage (sl + 1) & 1 was last read by the MMAs of slab sl - 1
      bool w = true;
      if (sl >= 1) w = mbar_wait(smem_u32(&mbar[(sl - 1) & 1]), (unsigned)(((sl - 1) >> 1) & 1));
      ok = __syncthreads_and(w ? 1 : 0) != 0;  // block-uniform, so the loop exits together
      if (ok) load(sl + 1, (sl + 1) & 1);
    }
  }
  // the last commit covers every earlier tcgen05.mma of the issuing thread
  if (issued >= 0) {
    const bool done = mbar_wait(smem_u32(&mbar[issued & 1]), (unsigned)((issued >> 1) & 1));
    ok = ok && done;
  }
  cp_wait_all();
  if (!ok) atomicExch(&g_tc_fault, 1);
  const int all_ok = __syncthreads_and(ok ? 1 : 0);
  asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
  if (all_ok) {
    // TMEM lane m = 8 * (tile row) + (tile column); warp w owns lanes 32w..32w+31
    const int m = warp * 32 + lane;
    const int i = i0 + m / HX_TJ, j = j0 + m % HX_TJ;
    const bool in_grid = i < a.H && j < a.W;
    const unsigned lane_base = tmem + ((unsigned)(warp * 32) << 16);
#pragma unroll
    for (int ch = 0; ch < BN / 16; ++ch) {
      unsigned r[16];
      asm volatile(
          "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, "
          "[%16];\n"
          : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
            "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
            "=r"(r[14]), "=r"(r[15])
          : "r"(lane_base + (unsigned)(ch * 16)));
      asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
      if (!in_grid) continue;
      bf16* o = a.out + (img + (long long)i * a.W + j) * a.out_cs;
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int co = n0 + ch * 16 + h * 8;
        if (co + 8 > a.cout) continue;
        V8 prev, res;
        if (a.accumulate) prev.u = *(const uint4*)(o + co);
#pragma unroll
        for (int k = 0; k < 4; ++k) {
          float v0 = __uint_as_float(r[h * 8 + 2 * k]), v1 = __uint_as_float(r[h * 8 + 2 * k + 1]);
          if (a.bias) {
            v0 += a.bias[co + 2 * k];
            v1 += a.bias[co + 2 * k + 1];
          }
          if (a.accumulate) {
            const float2 f = __bfloat1622float2(prev.h[k]);
            v0 += f.x;
            v1 += f.y;
          }
          if (a.relu) {
            v0 = fmaxf(v0, 0.f);
            v1 = fmaxf(v1, 0.f);
          }
          res.h[k] = __floats2bfloat162_rn(v0, v1);
        }
        *(uint4*)(o + co) = res.u;
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(BN));
}

// Persistent variant for single-slab layers (input channels <= 32): the
// 9-tap weights stay resident in shared memory, halo tiles are double-
// buffered and so are the TMEM accumulators (2 x BN columns), so while the
// tensor cores run tile n the CTA stages tile n+1 and writes out tile n-1.
template <int BN>
__global__ void __launch_bounds__(128) k_conv3_tcp(ConvArgs a, int ntiles) {
  extern __shared__ __align__(128) unsigned char tc_smem[];
  __shared__ __align__(8) unsigned long long mbar[2];
  __shared__ unsigned tslot;
  constexpr int TAP_B = TcGeom<BN>::TAP_B, SLAB_B = 9 * TAP_B;
  constexpr unsigned IDESC = (1u << 4) | (1u << 7) | (1u << 10) | ((unsigned)(BN >> 3) << 17) |
                             ((unsigned)(CBM >> 4) << 24);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int tiles_j = (a.W + HX_TJ - 1) / HX_TJ, tiles_i = (a.H + HX_TI - 1) / HX_TI;
  const int n0 = blockIdx.y * BN;
  unsigned char* sbw = tc_smem;                // resident weights
  unsigned char* sa0 = tc_smem + SLAB_B;       // two halo stages
  const unsigned sbase = smem_u32(tc_smem);
  if (tid == 0) {
    for (int q = 0; q < 2; ++q)
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_u32(&mbar[q])));
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(
                     smem_u32(&tslot)),
                 "r"(2 * BN));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n");
  }
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
  const unsigned tmem = tslot;

  auto tile_origin = [&](int t, long long& img, int& i0, int& j0) {
    const int tj = t % tiles_j;
    t /= tiles_j;
    const int ti = t % tiles_i;
    img = (long long)(t / tiles_i) * a.H * a.W;
    i0 = ti * HX_TI;
    j0 = tj * HX_TJ;
  };
  auto load_a = [&](int t, int st) {
    long long img;
    int i0, j0;
    tile_origin(t, img, i0, j0);
    unsigned char* sa = sa0 + st * HX_SLAB_A;
    for (int e = tid; e < (CBK / 8) * HX_LINES; e += 128) {
      const int c = e / HX_LINES, L = e - c * HX_LINES;
      const int hr = L / HX_HJ, hc = L - hr * HX_HJ;
      const int i = i0 - 1 + hr, j = j0 - 1 + hc, ch = c * 8;
      const bool v = i >= 0 && i < a.H && j >= 0 && j < a.W && ch < a.cin;
      const void* src =
          v ? (const void*)(a.in + (img + (long long)i * a.W + j) * a.in_cs + ch) : (const void*)a.in;
      cp_async16(sa + c * HX_LBO + L * 16, src, v);
    }
  };
  auto epilogue = [&](int t, int buf) {
    long long img;
    int i0, j0;
    tile_origin(t, img, i0, j0);
    const int m = warp * 32 + lane;
    const int i = i0 + m / HX_TJ, j = j0 + m % HX_TJ;
    const bool in_grid = i < a.H && j < a.W;
    const unsigned lane_base = tmem + ((unsigned)(warp * 32) << 16) + (unsigned)(buf * BN);
#pragma unroll
    for (int ch = 0; ch < BN / 16; ++ch) {
      unsigned r[16];
      asm volatile(
          "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, "
          "[%16];\n"
          : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
            "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
            "=r"(r[14]), "=r"(r[15])
          : "r"(lane_base + (unsigned)(ch * 16)));
      asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
      if (!in_grid) continue;
      bf16* o = a.out + (img + (long long)i * a.W + j) * a.out_cs;
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int co = n0 + ch * 16 + h * 8;
        if (co + 8 > a.cout) continue;
        V8 prev, res;
        if (a.accumulate) prev.u = *(const uint4*)(o + co);
#pragma unroll
        for (int k = 0; k < 4; ++k) {
          float v0 = __uint_as_float(r[h * 8 + 2 * k]), v1 = __uint_as_float(r[h * 8 + 2 * k + 1]);
          if (a.bias) {
            v0 += a.bias[co + 2 * k];
            v1 += a.bias[co + 2 * k + 1];
          }
          if (a.accumulate) {
            const float2 f = __bfloat1622float2(prev.h[k]);
            v0 += f.x;
            v1 += f.y;
          }
          if (a.relu) {
            v0 = fmaxf(v0, 0.f);
            v1 = fmaxf(v1, 0.f);
          }
          res.h[k] = __floats2bfloat162_rn(v0, v1);
        }
        *(uint4*)(o + co) = res.u;
      }
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
  };

  // resident weights + the first tile, one cp.async group
  for (int e = tid; e < 9 * BN * (CBK / 8); e += 128) {
    const int c = e & 3, rt = e >> 2;
    const int row = rt % BN, tap = rt / BN;
    const int co = n0 + row;
    const bool v = co < a.cout;
    const void* src = v ? (const void*)(a.w + ((size_t)tap * a.cout + co) * a.cinp + c * 8) : (const void*)a.w;
    cp_async16(sbw + tap * TAP_B + (row >> 3) * 512 + (row & 7) * 16 + c * 128, src, v);
  }
  const int first = blockIdx.x;
  if (first < ntiles) load_a(first, 0);
  cp_commit();

  bool ok = true;
  int n = 0, issued = -1;
  for (int t = first; t < ntiles && ok; t += gridDim.x, ++n) {
    const int st = n & 1;
    cp_wait_all();
    asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
    __syncthreads();
    if (tid == 0) {
      asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
      const unsigned sa = sbase + (unsigned)(SLAB_B + st * HX_SLAB_A), sb = sbase;
      const unsigned dcol = tmem + (unsigned)(st * BN);
#pragma unroll
      for (int tap = 0; tap < 9; ++tap) {
        const unsigned aoff = (unsigned)(((tap / 3) * HX_HJ + (tap % 3)) * 16);
#pragma unroll
        for (int kk = 0; kk < CBK / 16; ++kk) {
          const unsigned long long ad = tc_desc(sa + kk * 2 * HX_LBO + aoff, HX_LBO, HX_SBO);
          const unsigned long long bd = tc_desc(sb + tap * TAP_B + kk * 256, 128, 512);
          const unsigned acc = (tap > 0 || kk > 0) ? 1u : 0u;
          asm volatile(
              "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
              "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(dcol),
              "l"(ad), "l"(bd), "r"(IDESC), "r"(acc));
        }
      }
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
                       smem_u32(&mbar[st]))
                   : "memory");
    }
    issued = n;
    // tile n-1: its MMAs read stage st^1 and wrote TMEM buffer st^1
    bool w = true;
    if (n >= 1) w = mbar_wait(smem_u32(&mbar[st ^ 1]), (unsigned)(((n - 1) >> 1) & 1));
    ok = __syncthreads_and(w ? 1 : 0) != 0;
    if (!ok) break;
    const int next = t + gridDim.x;
    if (next < ntiles) load_a(next, st ^ 1);
    cp_commit();
    if (n >= 1) {
      asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
      epilogue(t - gridDim.x, st ^ 1);
    }
  }
  // the last committed tile; its commit also covers every earlier MMA, so
  // after a timeout this waits (bounded) for whatever is still in flight
  if (issued >= 0) {
    const bool done = mbar_wait(smem_u32(&mbar[issued & 1]), (unsigned)((issued >> 1) & 1));
    ok = ok && done;
    const int all_ok = __syncthreads_and(ok ? 1 : 0);
    if (all_ok) {
      asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
      epilogue(first + issued * (int)gridDim.x, issued & 1);
    }
  }
  cp_wait_all();
  if (!ok) atomicExch(&g_tc_fault, 1);
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(2 * BN));
}

static int g_conv_impl = 1;  // 1: tcgen05 (k_conv3_tc, default), 0: mma.sync (k_conv3)
static int g_conv_nonpersistent = 0;  // 1: single-slab layers also use k_conv3_tc

template <int BN>
static int launch_conv_tcp(const ConvArgs& a, cudaStream_t s) {
  constexpr int smem = 9 * TcGeom<BN>::TAP_B + 2 * HX_SLAB_A;
  {
    const int rc = allow_dynamic_smem((const void*)k_conv3_tcp<BN>, smem, 100);
    if (rc != CEV_OK) return rc;
  }
  // resident CTAs per SM: shared memory (227 KB usable, 1 KB reserved per
  // CTA) and TMEM (2*BN of 512 columns per CTA)
  const int per_sm = std::max(1, std::min((227 * 1024) / (smem + 128 + 1024), 512 / (2 * BN)));
  const long long tiles = (long long)((a.H + HX_TI - 1) / HX_TI) * ((a.W + HX_TJ - 1) / HX_TJ) *
                          (a.npix / ((long long)a.H * a.W));
  const int ny = (a.cout + BN - 1) / BN;
  const long long cap = std::max(1LL, (long long)per_sm * sm_count() / ny);
  const unsigned gx = (unsigned)std::min(tiles, cap);
  k_conv3_tcp<BN><<<dim3(gx, ny), 128, smem, s>>>(a, (int)tiles);
  CEV_CHECK_LAUNCH("k_conv3_tcp");
  return CEV_OK;
}

template <int BN>
static int launch_conv_tc(const ConvArgs& a, cudaStream_t s) {
  if (a.cinp == CBK && !g_conv_nonpersistent) return launch_conv_tcp<BN>(a, s);
  constexpr int slab = TcGeom<BN>::SLAB;
  {
    const int rc = allow_dynamic_smem((const void*)k_conv3_tc<BN>, 2 * slab);
    if (rc != CEV_OK) return rc;
  }
  const int smem = (a.cinp > CBK ? 2 : 1) * slab;
  const long long tiles = (long long)((a.H + HX_TI - 1) / HX_TI) * ((a.W + HX_TJ - 1) / HX_TJ) *
                          (a.npix / ((long long)a.H * a.W));
  k_conv3_tc<BN><<<dim3((unsigned)tiles, (a.cout + BN - 1) / BN), 128, smem, s>>>(a);
  CEV_CHECK_LAUNCH("k_conv3_tc");
  return CEV_OK;
}

static unsigned grid_for(long long n, int threads) {
  const long long want = (n + threads - 1) / threads;
  const long long cap = 16LL * sm_count();
  return (unsigned)std::max(1LL, std::min(want, cap));
}

}  // namespace nn
}  // namespace cev

using namespace cev;
using namespace cev::nn;

struct cev_learned_precond_s {
  int nx = 0, ny = 0, maxb = 0, c0 = 0;
  LayerSpec L[NLAYER];
  size_t nparam = 0;
  size_t woff[NLAYER], boff[NLAYER], hoff = 0;  // offsets into params
  float* params = nullptr;                        // device fp32 copy
  bf16* wf[NLAYER] = {};
  bf16* wd[NLAYER] = {};
  int cinp[NLAYER], coutp[NLAYER];
  float* nrm = nullptr;
  double* rms_part = nullptr;  // [max_batch][RMS_PARTS]
  // activations (forward) and their gradients (backward, allocated on first use)
  enum { X0, A1, P1, A2, P2, A3, P3, A4, A5, A6, U3, A7, A8, U2, A9, A10, U1, A11, NACT };
  bf16* act[NACT] = {};
  int act_c[NACT], act_lv[NACT];
  bf16* grad[NACT] = {};
  bf16* gtmp[4] = {};  // per-level scratch for the pooled-branch gradients
  int batch = 0;       // of the last forward
  int H[4], W[4];
  std::vector<void*> allocs;
  ~cev_learned_precond_s() {
    for (void* p : allocs) cudaFree(p);
  }
  template <typename T> int alloc(T** p, size_t count) {
    void* q = nullptr;
    if (cudaMalloc(&q, std::max<size_t>(count * sizeof(T), 16)) != cudaSuccess) {
      cudaGetLastError();
      set_error("learned preconditioner: out of device memory (%zu bytes)", count * sizeof(T));
      return CEV_ERR_CUDA;
    }
    allocs.push_back(q);
    *p = (T*)q;
    return CEV_OK;
  }
  long long npix(int lv, int b) const { return (long long)b * H[lv] * W[lv]; }
};

namespace cev {
namespace nn {

using Net = cev_learned_precond_s;

static int conv(Net& n, int l, const bf16* in, bf16* out, bool dgrad, int accumulate, int b,
                cudaStream_t s) {
  const LayerSpec& sp = n.L[l];
  ConvArgs a;
  a.in = in;
  a.cin = dgrad ? sp.cout : sp.cin;
  a.in_cs = a.cin;
  a.w = dgrad ? n.wd[l] : n.wf[l];
  a.cinp = dgrad ? n.coutp[l] : n.cinp[l];
  a.bias = dgrad ? nullptr : n.params + n.boff[l];
  a.out = out;
  a.cout = dgrad ? sp.cin : sp.cout;
  a.out_cs = a.cout;
  a.H = n.H[sp.level];
  a.W = n.W[sp.level];
  a.npix = n.npix(sp.level, b);
  a.relu = dgrad ? 0 : 1;
  a.accumulate = accumulate;
  const unsigned gx = (unsigned)((a.npix + CBM - 1) / CBM);
  if (g_conv_impl == 1) {
    if (a.cout <= 32) return launch_conv_tc<32>(a, s);
    return launch_conv_tc<64>(a, s);
  }
  if (a.cout <= 32) {
    k_conv3<32><<<dim3(gx, (a.cout + 31) / 32), 128, 0, s>>>(a);
  } else {
    k_conv3<64><<<dim3(gx, (a.cout + 63) / 64), 128, 0, s>>>(a);
  }
  CEV_CHECK_LAUNCH("k_conv3");
  return CEV_OK;
}

static int wgrad(Net& n, int l, const bf16* g, const bf16* in, float* gparams, int b, cudaStream_t s) {
  const LayerSpec& sp = n.L[l];
  WgradArgs a;
  a.g = g;
  a.cout = sp.cout;
  a.g_cs = sp.cout;
  a.in = in;
  a.cin = sp.cin;
  a.in_cs = sp.cin;
  a.dw = gparams + n.woff[l];
  a.H = n.H[sp.level];
  a.W = n.W[sp.level];
  a.npix = n.npix(sp.level, b);
  const int tiles = ((sp.cout + 63) / 64) * ((sp.cin + 63) / 64);
  const long long target = std::max(1LL, (long long)(8 * sm_count()) / (9LL * tiles));
  long long chunk = (a.npix + target - 1) / target;
  chunk = std::max(256LL, (chunk + 31) / 32 * 32);
  a.chunk = chunk;
  const unsigned gx = (unsigned)((a.npix + chunk - 1) / chunk);
  k_wgrad3<<<dim3(gx, 9, tiles), 128, 0, s>>>(a);
  CEV_CHECK_LAUNCH("k_wgrad3");
  const int C = sp.cout;
  k_bias_grad<<<grid_for(a.npix, 256), 256, 0, s>>>(g, gparams + n.boff[l], a.npix, C);
  CEV_CHECK_LAUNCH("k_bias_grad");
  return CEV_OK;
}

static int pool(Net& n, const bf16* in, bf16* out, int lv_out, int C, int b, float scale,
                cudaStream_t s) {
  const long long no = n.npix(lv_out, b);
  k_pool2<<<grid_for(no * (C / 8), 256), 256, 0, s>>>(in, out, no, n.H[lv_out], n.W[lv_out], C, scale);
  CEV_CHECK_LAUNCH("k_pool2");
  return CEV_OK;
}

static int up(Net& n, const bf16* in, const bf16* add, bf16* out, int lv_out, int C, int b, float scale,
              int accumulate, cudaStream_t s) {
  const long long no = n.npix(lv_out, b);
  k_up2<<<grid_for(no * (C / 8), 256), 256, 0, s>>>(in, add, out, no, n.H[lv_out], n.W[lv_out], C, scale,
                                                    accumulate);
  CEV_CHECK_LAUNCH("k_up2");
  return CEV_OK;
}

static int mask(Net& n, bf16* g, const bf16* a, int lv, int C, int b, cudaStream_t s) {
  const size_t n8 = (size_t)n.npix(lv, b) * C / 8;
  k_relu_mask<<<grid_for((long long)n8, 256), 256, 0, s>>>(g, a, n8);
  CEV_CHECK_LAUNCH("k_relu_mask");
  return CEV_OK;
}

int learned_check(const cev_learned_precond_s* h, const cev_fdfd_plan_s* p) {
  CEV_REQUIRE(h != nullptr, "CEV_PRECOND_LEARNED needs opts.learned");
  CEV_REQUIRE(p->pol == CEV_POL_EZ && p->mf_nsb < 0 && !p->eps_complex,
              "the learned preconditioner serves single-frequency Ez plans with real eps");
  CEV_REQUIRE(p->nx == h->nx && p->ny == h->ny, "learned preconditioner built for %dx%d, plan is %dx%d",
              h->nx, h->ny, p->nx, p->ny);
  CEV_REQUIRE(p->batch <= h->maxb, "plan batch %d exceeds the network's max batch %d", p->batch,
              h->maxb);
  return CEV_OK;
}

#define CEV_TRY(x)                   \
  do {                               \
    const int _rc = (x);             \
    if (_rc != CEV_OK) return _rc;   \
  } while (0)

int learned_forward(cev_learned_precond_s* hp, const cev_fdfd_plan_s* p, const float* eps,
                    int eps_shared, const float2* r, float2* z, const double* sc, int sc_stride,
                    int sc_index, cudaStream_t s) {
  CEV_TRY(learned_check(hp, p));
  Net& n = *hp;
  const int b = p->batch;
  n.batch = b;
  auto& A = n.act;
  k_rms_part<<<dim3(RMS_PARTS, b), 256, 0, s>>>(r, p->n(), n.rms_part);
  k_rms_final<<<(b + 127) / 128, 128, 0, s>>>(n.rms_part, p->n(), b, n.nrm);
  CEV_CHECK_LAUNCH("k_rms");
  k_prep<<<grid_for(n.npix(0, b), 256), 256, 0, s>>>(r, eps, eps_shared, p->k2_32, n.nrm, b, n.H[0],
                                                     n.W[0], p->npml_x, p->npml_y, A[Net::X0]);
  CEV_CHECK_LAUNCH("k_prep");
  const int c1 = n.c0, c2 = 2 * n.c0, c3 = 4 * n.c0;
  CEV_TRY(conv(n, 0, A[Net::X0], A[Net::A1], false, 0, b, s));
  CEV_TRY(pool(n, A[Net::A1], A[Net::P1], 1, c1, b, 0.25f, s));
  CEV_TRY(conv(n, 1, A[Net::P1], A[Net::A2], false, 0, b, s));
  CEV_TRY(pool(n, A[Net::A2], A[Net::P2], 2, c2, b, 0.25f, s));
  CEV_TRY(conv(n, 2, A[Net::P2], A[Net::A3], false, 0, b, s));
  CEV_TRY(pool(n, A[Net::A3], A[Net::P3], 3, c3, b, 0.25f, s));
  CEV_TRY(conv(n, 3, A[Net::P3], A[Net::A4], false, 0, b, s));
  CEV_TRY(conv(n, 4, A[Net::A4], A[Net::A5], false, 0, b, s));
  CEV_TRY(conv(n, 5, A[Net::A5], A[Net::A6], false, 0, b, s));
  CEV_TRY(up(n, A[Net::A6], A[Net::A3], A[Net::U3], 2, c3, b, 1.f, 0, s));
  CEV_TRY(conv(n, 6, A[Net::U3], A[Net::A7], false, 0, b, s));
  CEV_TRY(conv(n, 7, A[Net::A7], A[Net::A8], false, 0, b, s));
  CEV_TRY(up(n, A[Net::A8], A[Net::A2], A[Net::U2], 1, c2, b, 1.f, 0, s));
  CEV_TRY(conv(n, 8, A[Net::U2], A[Net::A9], false, 0, b, s));
  CEV_TRY(conv(n, 9, A[Net::A9], A[Net::A10], false, 0, b, s));
  CEV_TRY(up(n, A[Net::A10], A[Net::A1], A[Net::U1], 0, c1, b, 1.f, 0, s));
  CEV_TRY(conv(n, 10, A[Net::U1], A[Net::A11], false, 0, b, s));
  const long long np = n.npix(0, b), HW = (long long)n.H[0] * n.W[0];
  const float* wh = n.params + n.hoff;
  const unsigned g = grid_for(np, 256);
  switch (n.c0) {
    case 8: k_head_fwd<8><<<g, 256, 0, s>>>(A[Net::A11], wh, n.nrm, sc, sc_stride, sc_index, np, HW, z); break;
    case 16: k_head_fwd<16><<<g, 256, 0, s>>>(A[Net::A11], wh, n.nrm, sc, sc_stride, sc_index, np, HW, z); break;
    default: k_head_fwd<32><<<g, 256, 0, s>>>(A[Net::A11], wh, n.nrm, sc, sc_stride, sc_index, np, HW, z); break;
  }
  CEV_CHECK_LAUNCH("k_head_fwd");
  return CEV_OK;
}

static int learned_backward(Net& n, const float2* gz, float* gp, cudaStream_t s) {
  const int b = n.batch;
  auto& A = n.act;
  auto& G = n.grad;
  const int c1 = n.c0, c2 = 2 * n.c0, c3 = 4 * n.c0, c4 = 8 * n.c0;
  const long long np = n.npix(0, b), HW = (long long)n.H[0] * n.W[0];
  const unsigned g = std::min(grid_for(np, 256), 2u * sm_count());
  const float* wh = n.params + n.hoff;
  switch (n.c0) {
    case 8: k_head_bwd<8><<<g, 256, 0, s>>>(A[Net::A11], wh, n.nrm, gz, np, HW, G[Net::A11], gp + n.hoff); break;
    case 16: k_head_bwd<16><<<g, 256, 0, s>>>(A[Net::A11], wh, n.nrm, gz, np, HW, G[Net::A11], gp + n.hoff); break;
    default: k_head_bwd<32><<<g, 256, 0, s>>>(A[Net::A11], wh, n.nrm, gz, np, HW, G[Net::A11], gp + n.hoff); break;
  }
  CEV_CHECK_LAUNCH("k_head_bwd");
  // L10: U1 -> A11
  CEV_TRY(mask(n, G[Net::A11], A[Net::A11], 0, c1, b, s));
  CEV_TRY(wgrad(n, 10, G[Net::A11], A[Net::U1], gp, b, s));
  CEV_TRY(conv(n, 10, G[Net::A11], G[Net::U1], true, 0, b, s));  // dU1 = dA1 (skip part)
  // U1 = up(A10) + A1
  CEV_TRY(pool(n, G[Net::U1], G[Net::A10], 1, c1, b, 1.f, s));
  CEV_TRY(mask(n, G[Net::A10], A[Net::A10], 1, c1, b, s));
  CEV_TRY(wgrad(n, 9, G[Net::A10], A[Net::A9], gp, b, s));
  CEV_TRY(conv(n, 9, G[Net::A10], G[Net::A9], true, 0, b, s));
  CEV_TRY(mask(n, G[Net::A9], A[Net::A9], 1, c2, b, s));
  CEV_TRY(wgrad(n, 8, G[Net::A9], A[Net::U2], gp, b, s));
  CEV_TRY(conv(n, 8, G[Net::A9], G[Net::U2], true, 0, b, s));
  // U2 = up(A8) + A2
  CEV_TRY(pool(n, G[Net::U2], G[Net::A8], 2, c2, b, 1.f, s));
  CEV_TRY(mask(n, G[Net::A8], A[Net::A8], 2, c2, b, s));
  CEV_TRY(wgrad(n, 7, G[Net::A8], A[Net::A7], gp, b, s));
  CEV_TRY(conv(n, 7, G[Net::A8], G[Net::A7], true, 0, b, s));
  CEV_TRY(mask(n, G[Net::A7], A[Net::A7], 2, c3, b, s));
  CEV_TRY(wgrad(n, 6, G[Net::A7], A[Net::U3], gp, b, s));
  CEV_TRY(conv(n, 6, G[Net::A7], G[Net::U3], true, 0, b, s));
  // U3 = up(A6) + A3
  CEV_TRY(pool(n, G[Net::U3], G[Net::A6], 3, c3, b, 1.f, s));
  CEV_TRY(mask(n, G[Net::A6], A[Net::A6], 3, c3, b, s));
  CEV_TRY(wgrad(n, 5, G[Net::A6], A[Net::A5], gp, b, s));
  CEV_TRY(conv(n, 5, G[Net::A6], G[Net::A5], true, 0, b, s));
  CEV_TRY(mask(n, G[Net::A5], A[Net::A5], 3, c4, b, s));
  CEV_TRY(wgrad(n, 4, G[Net::A5], A[Net::A4], gp, b, s));
  CEV_TRY(conv(n, 4, G[Net::A5], G[Net::A4], true, 0, b, s));
  CEV_TRY(mask(n, G[Net::A4], A[Net::A4], 3, c4, b, s));
  CEV_TRY(wgrad(n, 3, G[Net::A4], A[Net::P3], gp, b, s));
  CEV_TRY(conv(n, 3, G[Net::A4], G[Net::P3], true, 0, b, s));
  // P3 = pool(A3): dA3 = dU3 + up(dP3)/4
  CEV_TRY(up(n, G[Net::P3], nullptr, G[Net::U3], 2, c3, b, 0.25f, 1, s));
  CEV_TRY(mask(n, G[Net::U3], A[Net::A3], 2, c3, b, s));
  CEV_TRY(wgrad(n, 2, G[Net::U3], A[Net::P2], gp, b, s));
  CEV_TRY(conv(n, 2, G[Net::U3], G[Net::P2], true, 0, b, s));
  CEV_TRY(up(n, G[Net::P2], nullptr, G[Net::U2], 1, c2, b, 0.25f, 1, s));
  CEV_TRY(mask(n, G[Net::U2], A[Net::A2], 1, c2, b, s));
  CEV_TRY(wgrad(n, 1, G[Net::U2], A[Net::P1], gp, b, s));
  CEV_TRY(conv(n, 1, G[Net::U2], G[Net::P1], true, 0, b, s));
  CEV_TRY(up(n, G[Net::P1], nullptr, G[Net::U1], 0, c1, b, 0.25f, 1, s));
  CEV_TRY(mask(n, G[Net::U1], A[Net::A1], 0, c1, b, s));
  CEV_TRY(wgrad(n, 0, G[Net::U1], A[Net::X0], gp, b, s));
  return CEV_OK;
}

}  // namespace nn
}  // namespace cev

extern "C" {

int cev_learned_param_count(int c0, size_t* count) {
  CEV_REQUIRE(count != nullptr, "NULL argument");
  CEV_REQUIRE(c0 == 8 || c0 == 16 || c0 == 32, "base width must be 8, 16 or 32");
  *count = param_count(c0);
  return CEV_OK;
}

int cev_learned_create(cev_learned_precond* out, int nx, int ny, int max_batch, int c0) {
  CEV_REQUIRE(out != nullptr, "NULL argument");
  *out = nullptr;
  CEV_REQUIRE(c0 == 8 || c0 == 16 || c0 == 32, "base width must be 8, 16 or 32");
  CEV_REQUIRE(nx >= 16 && ny >= 16 && nx % 8 == 0 && ny % 8 == 0,
              "the network needs nx, ny >= 16 and divisible by 8 (got %d x %d)", nx, ny);
  CEV_REQUIRE(max_batch >= 1, "max_batch must be >= 1");
  auto* n = new cev_learned_precond_s();
  n->nx = nx;
  n->ny = ny;
  n->maxb = max_batch;
  n->c0 = c0;
  layer_specs(c0, n->L);
  size_t off = 0;
  for (int l = 0; l < NLAYER; ++l) {
    n->woff[l] = off;
    off += (size_t)n->L[l].cout * n->L[l].cin * 9;
    n->boff[l] = off;
    off += n->L[l].cout;
    n->cinp[l] = round_up(n->L[l].cin, 32);
    n->coutp[l] = round_up(n->L[l].cout, 32);
  }
  n->hoff = off;
  n->nparam = off + 2 * (size_t)c0 + 2;
  for (int lv = 0; lv < 4; ++lv) {
    n->H[lv] = nx >> lv;
    n->W[lv] = ny >> lv;
  }
  const int c1 = c0, c2 = 2 * c0, c3 = 4 * c0, c4 = 8 * c0;
  using N = cev_learned_precond_s;
  const int spec[N::NACT][2] = {{CIN0, 0}, {c1, 0}, {c1, 1}, {c2, 1}, {c2, 2}, {c3, 2},
                                {c3, 3},   {c4, 3}, {c4, 3}, {c3, 3}, {c3, 2}, {c3, 2},
                                {c2, 2},   {c2, 1}, {c2, 1}, {c1, 1}, {c1, 0}, {c1, 0}};
  int rc = n->alloc(&n->params, n->nparam);
  for (int l = 0; l < NLAYER && rc == CEV_OK; ++l) {
    rc = n->alloc(&n->wf[l], (size_t)9 * n->L[l].cout * n->cinp[l]);
    if (rc == CEV_OK) rc = n->alloc(&n->wd[l], (size_t)9 * n->L[l].cin * n->coutp[l]);
  }
  if (rc == CEV_OK) rc = n->alloc(&n->nrm, (size_t)max_batch);
  if (rc == CEV_OK) rc = n->alloc(&n->rms_part, (size_t)max_batch * RMS_PARTS);
  for (int k = 0; k < N::NACT && rc == CEV_OK; ++k) {
    n->act_c[k] = spec[k][0];
    n->act_lv[k] = spec[k][1];
    rc = n->alloc(&n->act[k], (size_t)n->npix(spec[k][1], max_batch) * spec[k][0]);
  }
  if (rc != CEV_OK) {
    delete n;
    return rc;
  }
  if (cudaMemset(n->params, 0, n->nparam * sizeof(float)) != cudaSuccess) {
    delete n;
    return cuda_status(cudaGetLastError(), "cudaMemset");
  }
  *out = n;
  return CEV_OK;
}

int cev_learned_set_params(cev_learned_precond h, const float* params, cudaStream_t s) {
  CEV_REQUIRE(h != nullptr && params != nullptr, "NULL argument");
  CEV_CUDA(cudaMemcpyAsync(h->params, params, h->nparam * sizeof(float), cudaMemcpyDeviceToDevice, s));
  for (int l = 0; l < NLAYER; ++l) {
    const size_t tot = (size_t)9 * h->L[l].cout * h->cinp[l] + (size_t)9 * h->L[l].cin * h->coutp[l];
    k_pack<<<grid_for((long long)tot, 256), 256, 0, s>>>(h->params + h->woff[l], h->L[l].cin,
                                                          h->L[l].cout, h->cinp[l], h->coutp[l],
                                                          h->wf[l], h->wd[l]);
    CEV_CHECK_LAUNCH("k_pack");
  }
  return CEV_OK;
}

int cev_learned_forward(cev_learned_precond h, cev_fdfd_plan plan, const float* eps, int eps_shared,
                        const void* r, void* z, cudaStream_t s) {
  CEV_REQUIRE(h != nullptr && plan != nullptr && eps && r && z, "NULL argument");
  return learned_forward(h, plan, eps, eps_shared, (const float2*)r, (float2*)z, nullptr, 0, 0, s);
}

int cev_learned_backward(cev_learned_precond h, const void* gz, float* grad, cudaStream_t s) {
  CEV_REQUIRE(h != nullptr && gz && grad, "NULL argument");
  CEV_REQUIRE(h->batch > 0, "backward needs a forward first");
  using N = cev_learned_precond_s;
  if (!h->grad[N::A11]) {
    for (int k = 1; k < N::NACT; ++k) {
      const int rc = h->alloc(&h->grad[k], (size_t)h->npix(h->act_lv[k], h->maxb) * h->act_c[k]);
      if (rc != CEV_OK) return rc;
    }
  }
  return learned_backward(*h, (const float2*)gz, grad, s);
}

int cev_adam_step(float* p, const float* g, float* m, float* v, size_t n, float lr, float beta1,
                  float beta2, float eps, int step, cudaStream_t s) {
  CEV_REQUIRE(p && g && m && v, "NULL argument");
  CEV_REQUIRE(step >= 1, "step counts from 1");
  const float bc1 = 1.f - powf(beta1, (float)step), bc2 = 1.f - powf(beta2, (float)step);
  k_adam<<<grid_for((long long)n, 256), 256, 0, s>>>(p, g, m, v, n, lr, beta1, beta2, eps, bc1, bc2);
  CEV_CHECK_LAUNCH("k_adam");
  return CEV_OK;
}

int cev_learned_set_conv_impl(int impl) {
  CEV_REQUIRE(impl >= 0 && impl <= 2,
              "conv implementation must be 0 (mma.sync), 1 (tcgen05) or 2 (tcgen05, not persistent)");
  g_conv_impl = impl == 0 ? 0 : 1;
  g_conv_nonpersistent = impl == 2 ? 1 : 0;
  return CEV_OK;
}

int cev_learned_tc_fault(int* fault) {
  CEV_REQUIRE(fault != nullptr, "NULL argument");
  int zero = 0;
  CEV_CUDA(cudaMemcpyFromSymbol(fault, g_tc_fault, sizeof(int)));
  CEV_CUDA(cudaMemcpyToSymbol(g_tc_fault, &zero, sizeof(int)));
  return CEV_OK;
}

int cev_learned_destroy(cev_learned_precond h) {
  delete h;
  return CEV_OK;
}

}  // extern "C"
