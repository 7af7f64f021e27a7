// Fused restart cycle of the stencil GMRES for small problems and batches.
//
// The multi-kernel cycle (krylov.cu) issues a matvec, a multi-dot and an
// update launch per Arnoldi iteration, each ending in a last-block reduction
// tail; at 200x200 (40k cells) that is launch- and latency-bound (~40 us per
// iteration for < 1 us of memory traffic).  Here one cooperative launch runs
// the whole cycle for up to 16 problems, each on its own group of blocks
// with its own barrier: every block owns a fixed set of (column tile, row
// chunk) units of its problem for all iterations, so
//   * the matvec of iteration j and the projections onto V_0..V_j run on the
//     block's own cells with no barrier in between (each thread reads back
//     only cells it wrote itself; the stencil halo of V_j, written by other
//     blocks, is read through L2 with ld.global.cg);
//   * one grid barrier per Gram-Schmidt pass and one for the norm; after each
//     barrier every block reduces all blocks' partials itself, in the same
//     fixed order, so all blocks hold bitwise-identical projections, norms and
//     Givens rotations and no broadcast step is needed; block 0 writes the
//     Hessenberg column, rotations and KState for the triangular solve;
//   * the arithmetic follows the multi-kernel path: complex64 vectors, FP32
//     warp sums combined in FP64 per block, FP64 Givens.  The cross-block sums,
//     which every block repeats, use compensated float-float arithmetic
//     (Knuth's TwoSum on (hi, lo) FP32 pairs, ~48-bit significand) instead of
//     FP64: GB300's FP64 pipe is narrow, and 200 blocks each summing 200
//     partials per vector in FP64 kept it ~25% busy and dominated the
//     iteration.  Each block's FP64 partial is split exactly enough into
//     hi = fl32(d), lo = fl32(d - hi); the fixed summation order keeps the
//     result identical in every block and from run to run.
// The grid barrier spins on a generation word with a bounded wait (about a
// second); on timeout the block records a fault in KState and every block
// leaves at its next barrier, so the host reports an error instead of the
// kernel hanging.  The cooperative launch guarantees all blocks are resident.
#include <algorithm>
#include <cstdlib>

#include "fdfd_plan.hpp"
#include "krylov.hpp"
#include "reduce.cuh"

namespace cev {

static constexpr int CYC_THREADS = 256;
static constexpr int CYC_GROUP = 16;
static constexpr unsigned CYC_SPIN_LIMIT = 1u << 24;  // x ~64 ns sleep: about a second

// ---------------------------------------------------------- float-float
// (hi, lo) FP32 pairs, |lo| <= ulp(hi)/2: ~48-bit significands on the FP32
// pipe.  Sums by Knuth's TwoSum, products by the FMA-exact TwoProd; division
// and square root by one Newton correction of the FP32 result.
__device__ __forceinline__ float2 ff(float a) { return make_float2(a, 0.f); }
__device__ __forceinline__ float2 ff_split(double d) {
  const float hi = (float)d;
  return make_float2(hi, (float)(d - (double)hi));
}
__device__ __forceinline__ double ff_d(float2 a) { return (double)a.x + (double)a.y; }
__device__ __forceinline__ float2 ff_norm(float s, float e) {
  const float hi = __fadd_rn(s, e);
  return make_float2(hi, __fsub_rn(e, __fsub_rn(hi, s)));
}
__device__ __forceinline__ float2 ff_add(float2 a, float2 b) {
  const float s = __fadd_rn(a.x, b.x);
  const float bb = __fsub_rn(s, a.x);
  const float e = __fadd_rn(__fsub_rn(a.x, __fsub_rn(s, bb)), __fsub_rn(b.x, bb));
  return ff_norm(s, __fadd_rn(e, __fadd_rn(a.y, b.y)));
}
__device__ __forceinline__ float2 ff_neg(float2 a) { return make_float2(-a.x, -a.y); }
__device__ __forceinline__ float2 ff_sub(float2 a, float2 b) { return ff_add(a, ff_neg(b)); }
__device__ __forceinline__ float2 ff_mul(float2 a, float2 b) {
  const float p = __fmul_rn(a.x, b.x);
  float e = __fmaf_rn(a.x, b.x, -p);
  e = __fmaf_rn(a.x, b.y, e);
  e = __fmaf_rn(a.y, b.x, e);
  return ff_norm(p, e);
}
__device__ __forceinline__ float2 ff_div(float2 a, float2 b) {
  const float q1 = __fdiv_rn(a.x, b.x);
  const float2 r = ff_sub(a, ff_mul(b, ff(q1)));
  return ff_norm(q1, __fdiv_rn(r.x, b.x));
}
__device__ __forceinline__ float2 ff_sqrt(float2 a) {
  if (!(a.x > 0.f)) return ff(0.f);
  const float s = __fsqrt_rn(a.x);
  const float2 r = ff_sub(a, ff_mul(ff(s), ff(s)));
  return ff_norm(s, __fdiv_rn(r.x, 2.f * s));
}
__device__ __forceinline__ bool ff_le(float2 a, float2 b) {
  return a.x < b.x || (a.x == b.x && a.y <= b.y);
}
// complex float-float
struct cff {
  float2 re, im;
};
__device__ __forceinline__ cff cff_mul(cff a, cff b) {
  return {ff_sub(ff_mul(a.re, b.re), ff_mul(a.im, b.im)),
          ff_add(ff_mul(a.re, b.im), ff_mul(a.im, b.re))};
}
__device__ __forceinline__ cff cff_mulc(cff a, cff b) {  // conj(a) b
  return {ff_add(ff_mul(a.re, b.re), ff_mul(a.im, b.im)),
          ff_sub(ff_mul(a.re, b.im), ff_mul(a.im, b.re))};
}
__device__ __forceinline__ cff cff_add(cff a, cff b) { return {ff_add(a.re, b.re), ff_add(a.im, b.im)}; }
__device__ __forceinline__ cff cff_sub(cff a, cff b) { return {ff_sub(a.re, b.re), ff_sub(a.im, b.im)}; }
__device__ __forceinline__ cff cff_scale(cff a, float2 s) { return {ff_mul(a.re, s), ff_mul(a.im, s)}; }
__device__ __forceinline__ float2 ff_warp_sum(float2 v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    float2 t;
    t.x = __shfl_xor_sync(0xffffffffu, v.x, o);
    t.y = __shfl_xor_sync(0xffffffffu, v.y, o);
    // order the operands by lane so both partners compute the same sum
    v = (threadIdx.x & o) ? ff_add(t, v) : ff_add(v, t);
  }
  return v;
}
// Block sum of NV floats per thread: FP32 warp sums, then the per-warp sums
// combined in float-float by thread k (valid in threads k < NV).
template <int NV>
__device__ __forceinline__ float2 block_sum_ff(float (&v)[NV], float* smem /* NV*32 */) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int nw = (blockDim.x + 31) >> 5;
#pragma unroll
  for (int k = 0; k < NV; ++k) v[k] = warp_sumf(v[k]);
  __syncthreads();
  if (lane == 0)
#pragma unroll
    for (int k = 0; k < NV; ++k) smem[k * 32 + warp] = v[k];
  __syncthreads();
  float2 t = ff(0.f);
  if ((int)threadIdx.x < NV)
    for (int q = 0; q < nw; ++q) t = ff_add(t, ff(smem[threadIdx.x * 32 + q]));
  return t;
}

__device__ __forceinline__ unsigned ld_volatile(const unsigned* p) {
  return *(const volatile unsigned*)p;
}

// Grid barrier (thread 0 of each block arrives; the last one releases).
// Returns false if the wait timed out here or a fault was recorded elsewhere.
__device__ __forceinline__ bool grid_sync(unsigned* bar, unsigned nblk, unsigned& gen,
                                          int* s_ok, KState* st) {
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    const unsigned arrived = atomicAdd(bar, 1u);
    if (arrived == nblk - 1) {
      atomicExch(bar, 0u);
      __threadfence();
      atomicAdd(bar + 1, 1u);
    } else {
      unsigned spins = 0;
      while (ld_volatile(bar + 1) == gen) {
        if (ld_volatile(bar + 2) != 0u) break;
        if (++spins > CYC_SPIN_LIMIT) {
          atomicExch(bar + 2, 1u);
          st->fault = 1;
          break;
        }
        __nanosleep(64);
      }
    }
    __threadfence();
    gen += 1;
    *s_ok = ld_volatile(bar + 2) == 0u;
  }
  __syncthreads();
  return *s_ok != 0;
}

// Staged cycle results (float-float), converted to the FP64 Krylov arrays
// by k_cycle_publish after the cycle: Hessenberg columns, Givens cosines and
// sines, gamma / beta, 1/||v_k|| and the residual estimate / beta.
struct CycStage {
  float2 H[64 * 65 * 2];  // [col][row][re, im]
  float2 cs[64];
  float2 sn[64 * 2];
  float2 gam[65 * 2];
  float2 sc[65];
  float2 res;
};

size_t cycle_stage_bytes() { return sizeof(CycStage); }

// float2 slots (8 bytes, counted as doubles) of the partials ahead of the stage
__host__ __device__ inline size_t fused_part_doubles(unsigned G, int m) {
  return 2 * (size_t)G * 2 * (size_t)(m + 1) + G;
}

template <int POL, typename E>
__global__ void __launch_bounds__(CYC_THREADS) k_cycle(CycArgs a) {
  // problem b of the batch runs on its own group of gp blocks (own barrier,
  // partials and stage); lb is the block's index within the group
  const int b = blockIdx.x / a.gp;
  const unsigned lb = blockIdx.x % a.gp;
  KState* st = a.ctx.st + b;
  if (!st->active) return;
  const int m = a.m, ny = a.ny, nx = a.nx;
  const unsigned G = a.gp;
  // partials as float-float pairs, [value][block] (value = 2k + re/im)
  const size_t ps = 2 * (size_t)(m + 1);
  float2* dpart0 = (float2*)(a.ctx.fpart + (size_t)b * fused_part_doubles(G, m));
  float2* dpart1 = dpart0 + (size_t)G * ps;
  float2* npart = dpart1 + (size_t)G * ps;
  CycStage* stage = (CycStage*)(a.ctx.fpart + (size_t)a.B * fused_part_doubles(G, m)) + b;
  unsigned* bar = a.ctx.bar + 4 * b;
  double* gsc = a.ctx.sc + (size_t)b * (m + 1);
  const E* eps = (const E*)a.eps + (size_t)b * a.eps_bs;
  const Coef<float>* cx = a.cx + (size_t)b * nx;
  const Coef<float>* cy = a.cy + (size_t)b * ny;

  __shared__ float2 sCs[64], sSnR[64], sSnI[64], sGR[65], sGI[65], sHR[66], sHI[66], sSc[65];
  __shared__ float2 sU[65];
  __shared__ float smf[2 * CYC_GROUP * 32];
  __shared__ int s_ok, s_active;
  __shared__ float2 s_hn;
  unsigned gen = 0;
  const double beta = st->beta;  // > 0 when active
  if (threadIdx.x == 0) {
    gen = ld_volatile(bar + 1);
    sGR[0] = ff(1.f);
    sGI[0] = ff(0.f);
    sSc[0] = ff_split(gsc[0]);
    s_ok = 1;
  }
  int iters = st->iters;
  const float2 thr = ff_split(st->thresh / beta);
  const float k2 = a.k2[b];
  __syncthreads();

  for (int j = 0; j < m; ++j) {
    float2* w = a.V + ((size_t)(j + 1) * a.B + b) * a.N;
    const float2* vj = a.V + ((size_t)j * a.B + b) * a.N;
    // 1. w = A' (sc_j V_j) on the block's own cells
    const float s = sSc[j].x + sSc[j].y;
    for (int u = lb; u < a.units; u += G) {
      const int col = (u % a.tiles_y) * CYC_THREADS + threadIdx.x;
      if (col < ny) {
        const int i0 = (u / a.tiles_y) * a.rows, i1 = min(i0 + a.rows, nx);
        auto ep = [&](int i, float2 v, float2) { w[(size_t)i * ny + col] = cscale(v, s); };
        stencil_column<float, POL, decltype(ep), true, E>(nx, ny, col, i0, i1, vj, eps, cx,
                                                          cy[col], k2, ep);
      }
    }
    // 2. Gram-Schmidt passes
    float nrm = 0.f;
    const int npass = a.reorth ? 2 : 1;
    const int nv = j + 1;
    for (int pass = 0; pass < npass; ++pass) {
      float2* dpart = pass == 0 ? dpart0 : dpart1;
      for (int g0 = 0; g0 < nv; g0 += CYC_GROUP) {
        float2 acc[CYC_GROUP];
#pragma unroll
        for (int k = 0; k < CYC_GROUP; ++k) acc[k] = make_float2(0.f, 0.f);
        for (int u = lb; u < a.units; u += G) {
          const int col = (u % a.tiles_y) * CYC_THREADS + threadIdx.x;
          if (col >= ny) continue;
          const int i0 = (u / a.tiles_y) * a.rows, i1 = min(i0 + a.rows, nx);
          for (int i = i0; i < i1; ++i) {
            const size_t n = (size_t)i * ny + col;
            const float2 wv = w[n];
            float2 v[CYC_GROUP];
#pragma unroll
            for (int k = 0; k < CYC_GROUP; ++k)
              v[k] = (g0 + k < nv) ? a.V[((size_t)(g0 + k) * a.B + b) * a.N + n]
                                   : make_float2(0.f, 0.f);
#pragma unroll
            for (int k = 0; k < CYC_GROUP; ++k) {
              acc[k].x += v[k].x * wv.x + v[k].y * wv.y;
              acc[k].y += v[k].x * wv.y - v[k].y * wv.x;
            }
          }
        }
        float fv[2 * CYC_GROUP];
#pragma unroll
        for (int k = 0; k < CYC_GROUP; ++k) {
          fv[2 * k] = acc[k].x;
          fv[2 * k + 1] = acc[k].y;
        }
        const float2 tot = block_sum_ff<2 * CYC_GROUP>(fv, smf);
        if (threadIdx.x < 2 * CYC_GROUP && g0 + (int)(threadIdx.x >> 1) < nv)
          dpart[(size_t)(2 * g0 + threadIdx.x) * G + lb] = tot;
        __syncthreads();
      }
      if (!grid_sync(bar, G, gen, &s_ok, st)) return;
      // every block: fixed-order float-float sum over blocks, one warp per vector
      const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
      for (int k = warp; k < nv; k += nw) {
        float2 fre = ff(0.f), fim = ff(0.f);
        for (unsigned q = lane; q < G; q += 32) {
          fre = ff_add(fre, __ldcg(dpart + (size_t)(2 * k) * G + q));
          fim = ff_add(fim, __ldcg(dpart + (size_t)(2 * k + 1) * G + q));
        }
        fre = ff_warp_sum(fre);
        fim = ff_warp_sum(fim);
        if (lane == 0) {
          const float2 sk = sSc[k];
          const float2 hre = ff_mul(sk, fre), him = ff_mul(sk, fim);
          sHR[k] = pass == 0 ? hre : ff_add(sHR[k], hre);
          sHI[k] = pass == 0 ? him : ff_add(sHI[k], him);
          const float2 ure = ff_mul(sk, hre), uim = ff_mul(sk, him);
          sU[k] = make_float2(ure.x + ure.y, uim.x + uim.y);
        }
      }
      __syncthreads();
      // w -= sum_k V_k u_k on the block's own cells
      const bool last = pass == npass - 1;
      for (int u = lb; u < a.units; u += G) {
        const int col = (u % a.tiles_y) * CYC_THREADS + threadIdx.x;
        if (col >= ny) continue;
        const int i0 = (u / a.tiles_y) * a.rows, i1 = min(i0 + a.rows, nx);
        for (int i = i0; i < i1; ++i) {
          const size_t n = (size_t)i * ny + col;
          float2 wv = w[n];
          constexpr int GL = 16;
          for (int k0 = 0; k0 < nv; k0 += GL) {
            float2 v[GL];
#pragma unroll
            for (int k = 0; k < GL; ++k)
              v[k] = (k0 + k < nv) ? a.V[((size_t)(k0 + k) * a.B + b) * a.N + n]
                                   : make_float2(0.f, 0.f);
#pragma unroll
            for (int k = 0; k < GL; ++k) {
              const float2 c = (k0 + k < nv) ? sU[k0 + k] : make_float2(0.f, 0.f);
              wv.x -= v[k].x * c.x - v[k].y * c.y;
              wv.y -= v[k].x * c.y + v[k].y * c.x;
            }
          }
          w[n] = wv;
          if (last) nrm += wv.x * wv.x + wv.y * wv.y;
        }
      }
    }
    // 3. ||w||
    {
      float accf[1] = {nrm};
      const float2 tot = block_sum_ff<1>(accf, smf);
      if (threadIdx.x == 0) npart[lb] = tot;
    }
    if (!grid_sync(bar, G, gen, &s_ok, st)) return;
    if (threadIdx.x < 32) {
      float2 f = ff(0.f);
      for (unsigned q = threadIdx.x; q < G; q += 32) f = ff_add(f, __ldcg(npart + q));
      f = ff_warp_sum(f);
      if (threadIdx.x == 0) s_hn = ff_sqrt(f);
    }
    __syncthreads();
    // 4. Givens in float-float (identical in every block)
    if (threadIdx.x == 0) {
      const float2 hn = s_hn;
      sHR[j + 1] = hn;
      sHI[j + 1] = ff(0.f);
      for (int k = 0; k < j; ++k) {
        const cff h0{sHR[k], sHI[k]}, h1{sHR[k + 1], sHI[k + 1]}, sk{sSnR[k], sSnI[k]};
        const float2 ck = sCs[k];
        const cff n0 = cff_add(cff_scale(h0, ck), cff_mul(sk, h1));
        const cff n1 = cff_sub(cff_scale(h1, ck), cff_mulc(sk, h0));
        sHR[k] = n0.re;
        sHI[k] = n0.im;
        sHR[k + 1] = n1.re;
        sHI[k + 1] = n1.im;
      }
      const cff av{sHR[j], sHI[j]};
      const float2 aa2 = ff_add(ff_mul(av.re, av.re), ff_mul(av.im, av.im));
      float2 cj;
      cff sj, rj;
      if (!(aa2.x > 0.f)) {
        cj = ff(0.f);
        sj = {ff(1.f), ff(0.f)};
        rj = {hn, ff(0.f)};
      } else {
        const float2 aa = ff_sqrt(aa2);
        const float2 t = ff_sqrt(ff_add(aa2, ff_mul(hn, hn)));
        cj = ff_div(aa, t);
        const cff ph{ff_div(av.re, aa), ff_div(av.im, aa)};
        sj = cff_scale(ph, ff_div(hn, t));
        rj = cff_scale(ph, t);
      }
      sCs[j] = cj;
      sSnR[j] = sj.re;
      sSnI[j] = sj.im;
      sHR[j] = rj.re;
      sHI[j] = rj.im;
      sHR[j + 1] = ff(0.f);
      const cff g{sGR[j], sGI[j]};
      const cff gn = cff_mulc(sj, g);
      sGR[j + 1] = ff_neg(gn.re);
      sGI[j + 1] = ff_neg(gn.im);
      sGR[j] = ff_mul(g.re, cj);
      sGI[j] = ff_mul(g.im, cj);
      const float2 res = ff_sqrt(ff_add(ff_mul(gn.re, gn.re), ff_mul(gn.im, gn.im)));
      const bool breakdown = !(hn.x > 1e-30f);
      sSc[j + 1] = breakdown ? ff(0.f) : ff_div(ff(1.f), hn);
      iters += 1;
      const bool bad = !isfinite(res.x) || !isfinite(hn.x);
      const bool stop = bad || ff_le(res, thr) || breakdown || j + 1 >= m || iters >= a.ctx.max_iters;
      s_active = stop ? 0 : 1;
      if (lb == 0) {
        stage->res = res;
        st->ncols = j + 1;
        st->iters = iters;
        if (bad) st->nan = 1;
        if (stop) st->active = 0;
      }
    }
    __syncthreads();
    if (lb == 0) {  // stage column j and the rotation (parallel stores)
      for (int k = threadIdx.x; k <= j + 1; k += blockDim.x) {
        stage->H[((size_t)j * 65 + k) * 2] = sHR[k];
        stage->H[((size_t)j * 65 + k) * 2 + 1] = sHI[k];
      }
      if (threadIdx.x == 64) {
        stage->cs[j] = sCs[j];
        stage->sn[2 * j] = sSnR[j];
        stage->sn[2 * j + 1] = sSnI[j];
        stage->gam[2 * j] = sGR[j];
        stage->gam[2 * j + 1] = sGI[j];
        stage->gam[2 * j + 2] = sGR[j + 1];
        stage->gam[2 * j + 3] = sGI[j + 1];
        stage->sc[j + 1] = sSc[j + 1];
      }
    }
    if (!s_active) break;
  }
}

// FP64 Krylov arrays from the staged float-float results (one block per
// problem).
__global__ void k_cycle_publish(KCtx c, int m, const CycStage* stages) {
  const int b = blockIdx.x;
  const KState* st = c.st + b;
  const CycStage* stage = stages + b;
  const int nc = st->ncols;
  if (nc == 0) return;
  c.H += (size_t)b * m * (m + 1);
  c.cs += (size_t)b * m;
  c.sn += (size_t)b * m;
  c.gam += (size_t)b * (m + 1);
  c.sc += (size_t)b * (m + 1);
  const double beta = st->beta;
  for (int e = threadIdx.x; e < nc * (m + 1); e += blockDim.x) {
    const int col = e / (m + 1), k = e % (m + 1);
    if (k > col + 1) continue;
    c.H[(size_t)col * (m + 1) + k] =
        make_double2(ff_d(stage->H[((size_t)col * 65 + k) * 2]), ff_d(stage->H[((size_t)col * 65 + k) * 2 + 1]));
  }
  for (int k = threadIdx.x; k <= nc; k += blockDim.x) {
    if (k < nc) {
      c.cs[k] = ff_d(stage->cs[k]);
      c.sn[k] = make_double2(ff_d(stage->sn[2 * k]), ff_d(stage->sn[2 * k + 1]));
    }
    c.gam[k] = make_double2(beta * ff_d(stage->gam[2 * k]), beta * ff_d(stage->gam[2 * k + 1]));
    if (k > 0) c.sc[k] = ff_d(stage->sc[k]);
  }
  if (threadIdx.x == 0) c.st[b].res_est = beta * ff_d(stage->res);
}

// Grid of the fused cycle for a batch of B problems: a group of gp blocks per
// problem, each block a set of units of CYC_THREADS columns x rows rows, all
// groups together about as many blocks as are co-resident (at most 2 per SM).
// limit > 0 caps gp (blocks then loop over several units).  Returns the total
// number of blocks, 0 if the fused cycle is not available.
template <int POL, typename E>
static int cycle_occupancy() {
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_cycle<POL, E>, CYC_THREADS, 0);
  return per_sm;
}

int cycle_plan(int nx, int ny, int pol, int ceps, int B, int limit, int& rows, int& tiles_y,
               int& units, int& gp) {
  static int coop = -1;
  if (coop < 0) {
    int dev = 0, v = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&v, cudaDevAttrCooperativeLaunch, dev);
    coop = v;
  }
  if (!coop || B < 1) return 0;
  const int per_sm = pol == POL_EZ ? (ceps ? cycle_occupancy<POL_EZ, float2>()
                                             : cycle_occupancy<POL_EZ, float>())
                                   : (ceps ? cycle_occupancy<POL_HZ, float2>()
                                           : cycle_occupancy<POL_HZ, float>());
  if (per_sm < 1) return 0;
  const int cap = std::min(fused_max_blocks(), std::min(per_sm, 2) * sm_count());
  const int per = cap / B;  // blocks per problem
  if (per < 1) return 0;
  tiles_y = (ny + CYC_THREADS - 1) / CYC_THREADS;
  rows = std::max(1, (int)(((long)nx * tiles_y + per - 1) / per));
  units = tiles_y * ((nx + rows - 1) / rows);
  gp = std::min(units, per);
  if (limit > 0) gp = std::min(gp, limit);
  return gp * B;
}

int cycle_launch(int pol, int ceps, int blocks, const CycArgs& a, cudaStream_t s) {
  void* args[] = {(void*)&a};
  const void* fn = pol == POL_EZ ? (ceps ? (const void*)k_cycle<POL_EZ, float2>
                                         : (const void*)k_cycle<POL_EZ, float>)
                                 : (ceps ? (const void*)k_cycle<POL_HZ, float2>
                                         : (const void*)k_cycle<POL_HZ, float>);
  const cudaError_t e =
      cudaLaunchCooperativeKernel(fn, dim3(blocks), dim3(CYC_THREADS), args, 0, s);
  if (e != cudaSuccess) return cuda_status(e, "k_cycle");
  const CycStage* stages =
      (const CycStage*)(a.ctx.fpart + (size_t)a.B * fused_part_doubles(a.gp, a.m));
  k_cycle_publish<<<a.B, 256, 0, s>>>(a.ctx, a.m, stages);
  CEV_CHECK_LAUNCH("k_cycle_publish");
  return CEV_OK;
}

}  // namespace cev
