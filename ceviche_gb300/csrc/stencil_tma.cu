// TMA-staged Arnoldi matvec for real eps, Ez and Hz: the batched
// w = s * A' v of the multi-kernel GMRES iteration (fdfd.py:172-185 and
// 200-233 applied matrix-free).
//
// A CTA owns a 16 x 128 cell tile of one problem.  One elected thread arms
// an mbarrier with the expected byte count and issues two tiled TMA copies
// (cp.async.bulk.tensor): the complex64 input with a one-cell halo, and the
// tile's eps.  The halo box starts two cells left of the tile so that its
// innermost coordinate stays on a 16-byte boundary (complex64 = 8 B), and it
// is 132 cells wide.  Cells outside the grid arrive zero-filled.  The
// periodic (Bloch) wrap needs the values from the opposite edge; edge tiles
// patch those halo cells with plain loads after the copy lands (the Bloch
// phasors live in the coefficient tables, as in stencil_column).  Each
// thread then evaluates its cells from shared memory: the five-point
// stencil, PML tables per row (cx, broadcast) and column (cy, in registers).
// Hz averages eps with its i-1, i-2 and j-1, j-2 neighbours, so its eps box
// has a two-cell halo on the low side: 18 x 132 floats starting two rows up
// and four columns left (16-byte aligned), wrap cells patched the same way.
//
// The wait on the mbarrier is bounded; a timeout records a fault in the
// problem's KState and the block waits (bounded) again before it exits.
#include <mutex>
#include <cuda.h>
#include <cudaTypedefs.h>

#include <cstdlib>

#include "krylov.hpp"
#include "stencil.cuh"

namespace cev {

namespace {

constexpr int TT_I = 16, TT_J = 128;         // tile
constexpr int TT_HI = TT_I + 2;              // halo rows
constexpr int TT_HJ = TT_J + 4;              // halo columns (start 2 left: 16-B aligned)
constexpr int TT_THREADS = 256;
// eps box: Ez the tile itself; Hz two rows up and four columns left
template <int POL> struct EpsBox {
  static constexpr int RI = POL == CEV_POL_EZ ? TT_I : TT_I + 2;
  static constexpr int RJ = POL == CEV_POL_EZ ? TT_J : TT_J + 4;
  static constexpr int OI = POL == CEV_POL_EZ ? 0 : 2;  // rows above the tile
  static constexpr int OJ = POL == CEV_POL_EZ ? 0 : 4;  // columns left of the tile
  static constexpr unsigned BYTES = TT_HI * TT_HJ * 8 + RI * RJ * 4;
};
constexpr long long TT_SPIN = 1LL << 22;

struct TmaMvArgs {
  int nx, ny, m, j, use_scale;
  float2* out;
  size_t out_bs;
  const float2* in;  // for the wrap patches
  size_t in_bs;
  const float* eps;  // for the Hz eps wrap patches
  const Coef<float>* cx;
  const Coef<float>* cy;
  const float* k2;
  KCtx ctx;
};

__device__ __forceinline__ unsigned su32(const void* p) {
  return (unsigned)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ bool tt_wait(unsigned bar) {
  for (long long i = 0; i < TT_SPIN; ++i) {
    unsigned ok;
    asm volatile(
        "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        "selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(bar), "r"(0u)
        : "memory");
    if (ok) return true;
  }
  return false;
}

template <int POL>
__global__ void __launch_bounds__(TT_THREADS) k_arnoldi_mv_tma(const __grid_constant__ CUtensorMap tx,
                                                               const __grid_constant__ CUtensorMap te,
                                                               int eps_shared, TmaMvArgs a) {
  using EB = EpsBox<POL>;
  __shared__ __align__(128) float2 sx[TT_HI * TT_HJ];
  __shared__ __align__(128) float se[EB::RI * EB::RJ];
  __shared__ __align__(8) unsigned long long bar;
  const int b = blockIdx.z;
  if (!a.ctx.st[b].active) return;  // uniform over the block
  const int j0 = blockIdx.x * TT_J, i0 = blockIdx.y * TT_I;
  const int tid = threadIdx.x;
  const unsigned sbar = su32(&bar);
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(sbar));
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  }
  __syncthreads();
  if (tid == 0) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(sbar), "r"(EB::BYTES)
                 : "memory");
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, "
        "%4}], [%5];\n" ::"r"(su32(sx)),
        "l"(&tx), "r"(j0 - 2), "r"(i0 - 1), "r"(b), "r"(sbar)
        : "memory");
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, "
        "%4}], [%5];\n" ::"r"(su32(se)),
        "l"(&te), "r"(j0 - EB::OJ), "r"(i0 - EB::OI), "r"(eps_shared ? 0 : b), "r"(sbar)
        : "memory");
  }
  // per-column data while the copies are in flight
  const int jj = tid % TT_J, ii0 = tid / TT_J;
  const int j = j0 + jj;
  const bool jv = j < a.ny;
  const Coef<float> cyj = a.cy[(size_t)b * a.ny + (jv ? j : 0)];
  const float s = a.use_scale ? (float)a.ctx.sc[(size_t)b * (a.m + 1) + a.j] : 1.0f;
  const float k2 = a.k2[b];
  const Coef<float>* cx = a.cx + (size_t)b * a.nx;
  if (!__syncthreads_and(tt_wait(sbar) ? 1 : 0)) {  // block-uniform decision
    if (tid == 0) a.ctx.st[b].fault = 1;
    tt_wait(sbar);  // bounded: let the copy land before the block exits
    return;
  }
  // periodic wrap: halo cells from the opposite edge (zero-filled by the copy)
  const float2* x = a.in + (size_t)b * a.in_bs;
  bool patched = false;
  if (i0 == 0) {
    for (int q = tid; q < TT_J; q += TT_THREADS)
      if (j0 + q < a.ny) sx[q + 2] = x[(size_t)(a.nx - 1) * a.ny + j0 + q];
    patched = true;
  }
  if (i0 + TT_I >= a.nx) {
    const int rs = a.nx - i0 + 1;
    for (int q = tid; q < TT_J; q += TT_THREADS)
      if (j0 + q < a.ny) sx[rs * TT_HJ + q + 2] = x[j0 + q];
    patched = true;
  }
  if (j0 == 0) {
    for (int q = tid; q < TT_I; q += TT_THREADS)
      if (i0 + q < a.nx) sx[(q + 1) * TT_HJ + 1] = x[(size_t)(i0 + q) * a.ny + a.ny - 1];
    patched = true;
  }
  if (j0 + TT_J >= a.ny) {
    const int cs = a.ny - j0 + 2;
    for (int q = tid; q < TT_I; q += TT_THREADS)
      if (i0 + q < a.nx) sx[(q + 1) * TT_HJ + cs] = x[(size_t)(i0 + q) * a.ny];
    patched = true;
  }
  if (POL == CEV_POL_HZ) {
    // eps rows i0-2, i0-1 and columns j0-2, j0-1 wrap at the low edges
    const float* ep = a.eps + (eps_shared ? 0 : (size_t)b * a.nx * a.ny);
    if (i0 == 0) {
      for (int q = tid; q < 2 * TT_J; q += TT_THREADS) {
        const int r = q / TT_J, jq = j0 + q % TT_J;  // r = 0: row nx-2, r = 1: row nx-1
        if (jq < a.ny) se[r * EB::RJ + EB::OJ + q % TT_J] = ep[(size_t)((a.nx - 2 + r + a.nx) % a.nx) * a.ny + jq];
      }
      patched = true;
    }
    if (j0 == 0) {
      for (int q = tid; q < 2 * TT_I; q += TT_THREADS) {
        const int c = q / TT_I, iq = i0 + q % TT_I;  // c = 0: column ny-2, c = 1: column ny-1
        if (iq < a.nx) se[(EB::OI + q % TT_I) * EB::RJ + 2 + c] = ep[(size_t)iq * a.ny + (a.ny - 2 + c)];
      }
      patched = true;
    }
  }
  if (patched) __syncthreads();  // patched is uniform over the block
  if (!jv) return;
  float2* y = a.out + (size_t)b * a.out_bs;
  const float2 ym_c = cyj.cm, yp_c = cyj.cp;
  const float2 ya = cadd(cyj.am, cyj.ap);
  for (int ii = ii0; ii < TT_I; ii += TT_THREADS / TT_J) {
    const int i = i0 + ii;
    if (i >= a.nx) break;
    const float2* r = sx + (ii + 1) * TT_HJ + jj + 2;
    const float2 u_c = r[0], u_l = r[-1], u_r = r[1];
    const float2 u_m = r[-TT_HJ], u_p = r[TT_HJ];
    const Coef<float> c = cx[i];
    float2 acc;
    if constexpr (POL == CEV_POL_EZ) {
      const float e = se[ii * TT_J + jj];
      const float2 d0 = cadd(cadd(c.am, c.ap), ya);
      acc = cmul(c.cm, u_m);
      acc = cfma(c.cp, u_p, acc);
      acc = cfma(ym_c, u_l, acc);
      acc = cfma(yp_c, u_r, acc);
      acc = csub(acc, cmul(d0, u_c));
      acc.x = -acc.x - k2 * e * u_c.x;
      acc.y = -acc.y - k2 * e * u_c.y;
    } else {
      // the column sweep's Hz expression (stencil_column), eps from the box
      const float* er = se + (ii + EB::OI) * EB::RJ + jj + EB::OJ;
      const float e = er[0], e_m = er[-EB::RJ], e_mm = er[-2 * EB::RJ], el = er[-1], ell = er[-2];
      const float dyy_p = hz_d(e, e_m), dyy_m = hz_d(e_m, e_mm);
      const float dxx_p = hz_d(e, el), dxx_m = hz_d(el, ell);
      float2 d0;
      d0.x = c.am.x * dyy_m + c.ap.x * dyy_p + cyj.am.x * dxx_m + cyj.ap.x * dxx_p;
      d0.y = c.am.y * dyy_m + c.ap.y * dyy_p + cyj.am.y * dxx_m + cyj.ap.y * dxx_p;
      acc = emul(cmul(c.cm, u_m), dyy_m);
      acc = cadd(acc, emul(cmul(c.cp, u_p), dyy_p));
      acc = cadd(acc, emul(cmul(ym_c, u_l), dxx_m));
      acc = cadd(acc, emul(cmul(yp_c, u_r), dxx_p));
      acc = csub(acc, cmul(d0, u_c));
      acc.x += k2 * u_c.x;
      acc.y += k2 * u_c.y;
    }
    y[(size_t)i * a.ny + j] = cscale(acc, s);
  }
}

PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  // a driver entry point is the same for every device: look it up once
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = (PFN_cuTensorMapEncodeTiled_v12000)p;
    else
      cudaGetLastError();
  });
  return fn;
}

bool encode3d(CUtensorMap* map, CUtensorMapDataType type, size_t esize, const void* base, int ny, int nx,
              int nb, unsigned box0, unsigned box1) {
  auto fn = encode_fn();
  if (!fn) return false;
  const cuuint64_t dims[3] = {(cuuint64_t)ny, (cuuint64_t)nx, (cuuint64_t)nb};
  const cuuint64_t strides[2] = {(cuuint64_t)ny * esize, (cuuint64_t)ny * nx * esize};
  const cuuint32_t box[3] = {box0, box1, 1};
  const cuuint32_t es[3] = {1, 1, 1};
  return fn(map, type, 3, const_cast<void*>(base), dims, strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
            CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

}  // namespace

bool tma_matvec_usable(const cev_fdfd_plan_s* p, bool eps_complex) {
  const char* env = std::getenv("CEV_TMA_MATVEC");  // "0": column-sweep kernel instead
  const bool off = env && env[0] == '0';
  return !off && !eps_complex && p->mf_nsb < 0 && p->ny % 4 == 0 && p->nx >= 2 && p->ny >= 4 &&
         encode_fn() != nullptr;
}

int tma_matvec(const cev_fdfd_plan_s* p, int tr, const float* eps32, int eps_shared,
               const float2* in, float2* out, const KCtx& c, int m, int j, int use_scale,
               cudaStream_t s) {
  const bool hz = p->pol == CEV_POL_HZ;
  const size_t N = p->n();
  CUtensorMap tx, te;
  if (!encode3d(&tx, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 8, in, p->ny, p->nx, p->batch, TT_HJ, TT_HI) ||
      !encode3d(&te, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, eps32, p->ny, p->nx, eps_shared ? 1 : p->batch,
                hz ? EpsBox<CEV_POL_HZ>::RJ : EpsBox<CEV_POL_EZ>::RJ,
                hz ? EpsBox<CEV_POL_HZ>::RI : EpsBox<CEV_POL_EZ>::RI)) {
    set_error("cuTensorMapEncodeTiled failed for the matvec operands");
    return CEV_ERR_CUDA;
  }
  TmaMvArgs a{p->nx, p->ny, m, j, use_scale, out, N, in, N, eps32, p->cx32[tr], p->cy32[tr],
              p->k2_32, c};
  const dim3 grid((p->ny + TT_J - 1) / TT_J, (p->nx + TT_I - 1) / TT_I, p->batch);
  if (hz)
    k_arnoldi_mv_tma<CEV_POL_HZ><<<grid, TT_THREADS, 0, s>>>(tx, te, eps_shared, a);
  else
    k_arnoldi_mv_tma<CEV_POL_EZ><<<grid, TT_THREADS, 0, s>>>(tx, te, eps_shared, a);
  CEV_CHECK_LAUNCH("k_arnoldi_mv_tma");
  return CEV_OK;
}

}  // namespace cev
