// 2D Yee FDTD with ceviche's integrated-sigma PML, forward and adjoint.
//
// Update form (TM; Nz = 1, sigma_z = 0).  With a = sigma*dt/(2 eps0) on the
// H and D sub-grids and S = C0 dt / dL, the coefficients of
// ceviche/fdtd.py:265-316 become
//   mHx1 = (1-aHy)/(1+aHy),  mHx2*CEx = -S/(1+aHy) dEy,
//   mHx3*ICEx = -S/(1+aHy) (2 aHx) sum(dEy)          (same for y with x<->y)
//   mDz0*dt = (1+aDx)(1+aDy), mDz1 = (1-aDx-aDy-aDx aDy)/((1+aDx)(1+aDy)),
//   mDz2*CHz = S/((1+aDx)(1+aDy)) CH',  mDz4 = -4 aDx aDy/((1+aDx)(1+aDy))
// with dEy = Ez[i,j+1]-Ez, dEx' = -(Ez[i+1,j]-Ez), CH' = (Hy-Hy[i-1])-(Hx-Hx[i,j-1])
// (the curls of ceviche/derivatives.py:16-30 without the 1/dL factor, which
// sits in S).  mHx4, mHy4 and mDz3 carry sigma_z and are exactly zero, so the
// IHx, IHy and ICHz integrals never reach a field.  The PML integrals are
// accumulated only where their coefficient is non-zero; elsewhere they are
// multiplied by an exact zero in the reference.
// TE (Hz, Dx, Dy) is the dual: mHz has the (1+aHx)(1+aHy) form and
// Dx, Dy the single-axis form.
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <mutex>
#include <vector>

#include "common.cuh"

namespace cev {

constexpr double F_EPSILON_0 = 8.85418782e-12;
constexpr double F_MU_0 = 1.25663706e-6;

template <typename R>
struct AxisCoef {
  R aH, f1H, f2H, pH;  // H sub-grid: a, (1-a)/(1+a), S/(1+a), 1/(1+a)
  R aD, f1D, f2D, pD;  // D sub-grid
};

}  // namespace cev

struct cev_fdtd_plan_s {
  int nx = 0, ny = 0, npml_x = 0, npml_y = 0, prec = 0;
  double dL = 0, dt = 0, S = 0;
  void* ax = nullptr;   // AxisCoef<R>[nx]
  void* ay = nullptr;   // AxisCoef<R>[ny]
  void* iez = nullptr;  // 1/eps_zz, 1/eps_xx, 1/eps_yy (R[N])
  void* iexx = nullptr;
  void* ieyy = nullptr;
  void* shadow = nullptr;  // second TM state for the time-blocked run (6 N R)
  // Device pointers borrowed from elsewhere (the allocation-free runner's
  // static scratch): run_tm_impl then never allocates, and nothing frees them
  // (cev_fdtd_plan_destroy is never called on such a plan).
  bool borrowed = false;
  // persistent runner: neighbour lists of its tile grid, tile flags, fault word
  int pcfg = -1, ptiles = 0;
  int* pnbr = nullptr;
  int* pflags = nullptr;  // [ptiles] flags, then the fault word
  std::vector<double> aHx, aDx, aHy, aDy;
  size_t n() const { return (size_t)nx * ny; }
  size_t rs() const { return prec == CEV_PREC_C128 ? sizeof(double) : sizeof(float); }
};

namespace cev {

// ceviche/fdtd.py:213-222
static double fdtd_dt(double dL) {
  const double C_0 = 1.0 / std::sqrt(F_EPSILON_0 * F_MU_0);
  const double dL_sum = 3.0 / (dL * dL);
  const double dL_avg = 1.0 / std::sqrt(dL_sum);
  return dL_avg / C_0 * 0.5;
}

// sigma on the 2X grid (ceviche/fdtd.py:224-263), returned as a = sigma dt/(2 eps0)
static void sigma_profile(int N, int npml, double dt, std::vector<double>& aH,
                          std::vector<double>& aD) {
  std::vector<double> s2(2 * (size_t)N, 0.0);
  for (int k = 0; k < 2 * npml; ++k) {
    const int k1 = 2 * npml - k + 1;
    const int k2 = 2 * N - 2 * npml + k;
    const double v = (0.5 * F_EPSILON_0 / dt) * std::pow((double)k / 2 / npml, 3);
    if (k1 >= 0 && k1 < 2 * N) s2[k1] = v;
    if (k2 >= 0 && k2 < 2 * N) s2[k2] = v;
  }
  aH.resize(N);
  aD.resize(N);
  for (int i = 0; i < N; ++i) {
    aH[i] = s2[2 * i + 1] * dt / (2 * F_EPSILON_0);  // sigH = sig2[1::2]
    aD[i] = s2[2 * i] * dt / (2 * F_EPSILON_0);      // sigD = sig2[::2]
  }
}

template <typename R>
static std::vector<AxisCoef<R>> axis_coefs(const std::vector<double>& aH,
                                           const std::vector<double>& aD, double S) {
  std::vector<AxisCoef<R>> c(aH.size());
  for (size_t i = 0; i < aH.size(); ++i) {
    const double h = aH[i], d = aD[i];
    c[i].aH = (R)h;
    c[i].f1H = (R)((1 - h) / (1 + h));
    c[i].f2H = (R)(S / (1 + h));
    c[i].pH = (R)(1 / (1 + h));
    c[i].aD = (R)d;
    c[i].f1D = (R)((1 - d) / (1 + d));
    c[i].f2D = (R)(S / (1 + d));
    c[i].pD = (R)(1 / (1 + d));
  }
  return c;
}

template <typename R>
__global__ void k_inv_eps(const double* eps, R* iez, R* iexx, R* ieyy, int nx, int ny) {
  const size_t N = (size_t)nx * ny;
  for (size_t n = blockIdx.x * (size_t)blockDim.x + threadIdx.x; n < N;
       n += (size_t)gridDim.x * blockDim.x) {
    const int i = (int)(n / ny), j = (int)(n % ny);
    const double e = eps[n];
    // ceviche/utils.py:153-176: xx averages with roll(+1) along axis 0, yy along axis 1
    const double exx = (e + eps[(size_t)((i + nx - 1) % nx) * ny + j]) / 2;
    const double eyy = (e + eps[(size_t)i * ny + (j + ny - 1) % ny]) / 2;
    const double ezz = (e + e) / 2;
    iez[n] = (R)(1.0 / ezz);
    iexx[n] = (R)(1.0 / exx);
    ieyy[n] = (R)(1.0 / eyy);
  }
}

// ------------------------------------------------------------ per-step TM
template <typename R>
struct TMArgs {
  int nx, ny;
  R* hx; R* hy; R* dz; R* icex; R* icey; R* idz;
  const R* iez;
  const AxisCoef<R>* ax;
  const AxisCoef<R>* ay;
  R S;
  const R* jz;
};

template <typename R>
__global__ void k_tm_h(TMArgs<R> a) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  const int i = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= a.nx || j >= a.ny) return;
  const size_t n = (size_t)i * a.ny + j;
  const int ip = i + 1 == a.nx ? 0 : i + 1, jp = j + 1 == a.ny ? 0 : j + 1;
  const R ez = a.dz[n] * a.iez[n];
  const size_t nr = (size_t)i * a.ny + jp, nd = (size_t)ip * a.ny + j;
  const R ezr = a.dz[nr] * a.iez[nr];
  const R ezd = a.dz[nd] * a.iez[nd];
  const R dEy = ezr - ez;
  const R dEx = -(ezd - ez);
  const AxisCoef<R> cx = a.ax[i], cy = a.ay[j];
  R icx = R(0), icy = R(0);
  if (cx.aH != R(0)) { icx = a.icex[n] + dEy; a.icex[n] = icx; }
  if (cy.aH != R(0)) { icy = a.icey[n] + dEx; a.icey[n] = icy; }
  a.hx[n] = cy.f1H * a.hx[n] - cy.f2H * (dEy + R(2) * cx.aH * icx);
  a.hy[n] = cx.f1H * a.hy[n] - cx.f2H * (dEx + R(2) * cy.aH * icy);
}

template <typename R>
__device__ __forceinline__ void dz_coefs(const AxisCoef<R>& cx, const AxisCoef<R>& cy, R S, R& m1,
                                         R& m2, R& m4) {
  const R ax = cx.aD, ay = cy.aD;
  const R pd = cx.pD * cy.pD;
  m1 = (R(1) - ax - ay - ax * ay) * pd;
  m2 = S * pd;
  m4 = R(-4) * ax * ay * pd;
}

template <typename R>
__global__ void k_tm_d(TMArgs<R> a) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  const int i = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= a.nx || j >= a.ny) return;
  const size_t n = (size_t)i * a.ny + j;
  const int im = i == 0 ? a.nx - 1 : i - 1, jm = j == 0 ? a.ny - 1 : j - 1;
  const R hy = a.hy[n], hx = a.hx[n];
  const R ch = (hy - a.hy[(size_t)im * a.ny + j]) - (hx - a.hx[(size_t)i * a.ny + jm]);
  const AxisCoef<R> cx = a.ax[i], cy = a.ay[j];
  R m1, m2, m4;
  dz_coefs(cx, cy, a.S, m1, m2, m4);
  const R dz = a.dz[n];
  R id = R(0);
  if (m4 != R(0)) { id = a.idz[n] + dz; a.idz[n] = id; }
  R v = m1 * dz + m2 * ch + m4 * id;
  if (a.jz) v += a.jz[n];
  a.dz[n] = v;
}

// ------------------------------------------------------------ per-step TE
template <typename R>
struct TEArgs {
  int nx, ny;
  R* hz; R* dx; R* dy; R* ihz; R* ichx; R* ichy;
  const R* iexx;
  const R* ieyy;
  const AxisCoef<R>* ax;
  const AxisCoef<R>* ay;
  R S;
  const R* jx;
  const R* jy;
};

template <typename R>
__global__ void k_te_h(TEArgs<R> a) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  const int i = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= a.nx || j >= a.ny) return;
  const size_t n = (size_t)i * a.ny + j;
  const int ip = i + 1 == a.nx ? 0 : i + 1, jp = j + 1 == a.ny ? 0 : j + 1;
  const size_t nr = (size_t)i * a.ny + jp, nd = (size_t)ip * a.ny + j;
  const R ex = a.dx[n] * a.iexx[n], exr = a.dx[nr] * a.iexx[nr];
  const R ey = a.dy[n] * a.ieyy[n], eyd = a.dy[nd] * a.ieyy[nd];
  const R ce = (eyd - ey) - (exr - ex);
  const AxisCoef<R> cx = a.ax[i], cy = a.ay[j];
  const R ph = cx.pH * cy.pH;
  const R m1 = fma(-cx.aH, cy.aH, (R(1) - cx.aH) - cy.aH) * ph;
  const R m2 = -a.S * ph;
  const R m4 = R(-4) * cx.aH * cy.aH * ph;
  const R hz = a.hz[n];
  R ih = R(0);
  if (m4 != R(0)) { ih = a.ihz[n] + hz; a.ihz[n] = ih; }
  // explicit fused multiply-adds: the time-blocked TE kernel rounds the same way
  a.hz[n] = fma(m4, ih, fma(m2, ce, m1 * hz));
}

template <typename R>
__global__ void k_te_d(TEArgs<R> a) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  const int i = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= a.nx || j >= a.ny) return;
  const size_t n = (size_t)i * a.ny + j;
  const int im = i == 0 ? a.nx - 1 : i - 1, jm = j == 0 ? a.ny - 1 : j - 1;
  const R hz = a.hz[n];
  const R chx = hz - a.hz[(size_t)i * a.ny + jm];
  const R chy = -(hz - a.hz[(size_t)im * a.ny + j]);
  const AxisCoef<R> cx = a.ax[i], cy = a.ay[j];
  R icx = R(0), icy = R(0);
  if (cx.aD != R(0)) { icx = a.ichx[n] + chx; a.ichx[n] = icx; }
  if (cy.aD != R(0)) { icy = a.ichy[n] + chy; a.ichy[n] = icy; }
  R vx = fma(cy.f2D, fma(R(2) * cx.aD, icx, chx), cy.f1D * a.dx[n]);
  R vy = fma(cx.f2D, fma(R(2) * cy.aD, icy, chy), cx.f1D * a.dy[n]);
  if (a.jx) vx += a.jx[n];
  if (a.jy) vy += a.jy[n];
  a.dx[n] = vx;
  a.dy[n] = vy;
}

template <typename R>
__global__ void k_e_fields(int N, const R* dx, const R* dy, const R* dz, const R* iexx,
                           const R* ieyy, const R* iez, R* ex, R* ey, R* ez) {
  for (size_t n = blockIdx.x * (size_t)blockDim.x + threadIdx.x; n < (size_t)N;
       n += (size_t)gridDim.x * blockDim.x) {
    if (ez) ez[n] = iez[n] * dz[n];
    if (ex) ex[n] = iexx[n] * dx[n];
    if (ey) ey[n] = ieyy[n] * dy[n];
  }
}

// sparse source injection Dz[idx] += w * amps[t]
template <typename R>
__global__ void k_add_src(R* dz, int ns, const int* idx, const R* w, const R* amps, int t) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < ns) dz[idx[k]] += w[k] * amps[t];
}

template <typename R>
__global__ void k_probe(const R* dz, const R* iez, int np, const int* idx, R* out) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < np) out[k] = dz[idx[k]] * iez[idx[k]];
}

// ------------------------------------------------------- time-blocked TM
// One CTA advances a TI x TJ tile by up to K steps.  It loads the tile plus a
// halo of K cells; each cell's state (Hx, Hy, Dz, 1/eps, PML integrals,
// source weight) stays in registers of its owning thread for the whole
// launch, and only Ez (after the D phase) and Hx, Hy (after the H phase) go
// through shared memory.  The halo's valid zone shrinks by one cell per step
// (H needs Ez at i+1, j+1; D needs H at i-1, j-1), so after K steps the
// interior is exact.  At the region's edge the missing neighbour is replaced
// by the cell itself: those cells are outside the valid zone and never reach
// the interior.  The state is double-buffered in global memory.
template <typename R>
struct TBArgs {
  int nx, ny, K, t0;
  const R* hx_i; const R* hy_i; const R* dz_i; const R* icex_i; const R* icey_i; const R* idz_i;
  R* hx_o; R* hy_o; R* dz_o; R* icex_o; R* icey_o; R* idz_o;
  const R* iez;
  const AxisCoef<R>* ax;
  const AxisCoef<R>* ay;
  R S;
  int ns;
  const int* src_idx;
  const R* src_w;
  const R* amps;  // amps[t]
  int np;
  const int* probe_idx;
  R* probe_out;   // [t][np]
  R* dz_hist;     // HIST kernels: Dz after step t0+st goes to dz_hist[(t0+st+1)*N]
  // PERSIST kernels: the whole run in one launch (see k_tm_tile)
  int nsteps;           // steps of the run
  R* xb[2][6];          // exchange buffers (hx, hy, dz, icex, icey, idz); block m uses xb[m & 1]
  int* flags;           // [tiles] blocks published by each tile (zeroed before the launch)
  const int* nbr;       // [tiles][NBR_MAX] tiles this tile exchanges with (-1 ends a list)
  int* fault;           // set when a neighbour wait ran out
};

// Most tiles one persistent tile exchanges its ring with.
constexpr int NBR_MAX = 16;
// Tile flags sit one 128-byte line apart (no two tiles' flags share a line).
constexpr int FLAG_STRIDE = 32;

__device__ __forceinline__ int ld_acquire_gpu(const int* p) {
  int v;
  asm volatile("ld.acquire.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ int ld_relaxed_gpu(const int* p) {
  int v;
  asm volatile("ld.relaxed.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void fence_acq_rel_gpu() { asm volatile("fence.acq_rel.gpu;" ::: "memory"); }
__device__ __forceinline__ void st_release_gpu(int* p, int v) {
  asm volatile("st.release.gpu.global.s32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

template <typename R, int TI, int TJ, int K, int NT>
struct Tile {
  static constexpr int RI = TI + 2 * K, RJ = TJ + 2 * K, RN = RI * RJ;
  static constexpr int CPT = (RN + NT - 1) / NT;
  // sEz, sHx, sHy, sW (source weights), sIx, sIy, sId (PML integrals) [RN];
  // per-row x tables (5 x RI) and per-column y tables (5 x RJ); amps [K]
  static constexpr size_t smem =
      7 * (size_t)RN * sizeof(R) + 5 * (size_t)(RI + RJ) * sizeof(R) + (size_t)K * sizeof(R);
};

// PERSIST: one cooperative launch runs all a.nsteps steps.  Each CTA keeps its
// region resident; after every block of K steps its interior is exact and its
// K-wide ring is stale, so it publishes its interior to the exchange buffer
// xb[m & 1], releases flags[tile] = m + 1, waits (bounded) until every tile of
// its neighbour list has published block m, and reloads the ring from the same
// buffer.  Neighbour lists are symmetric, so a tile two blocks ahead can never
// overwrite a buffer a neighbour is still reading.
template <typename R, int TI, int TJ, int K, int NT, bool HIST = false, bool PERSIST = false>
__global__ void __launch_bounds__(NT, 1) k_tm_tile(TBArgs<R> a) {
  using T = Tile<R, TI, TJ, K, NT>;
  constexpr int RI = T::RI, RJ = T::RJ, RN = T::RN, CPT = T::CPT;
  extern __shared__ __align__(16) unsigned char smraw[];
  R* sEz = (R*)smraw;
  R* sHx = sEz + RN;
  R* sHy = sHx + RN;
  R* sW = sHy + RN;   // source weight per region cell
  R* sIx = sW + RN;   // ICEx' (PML tiles only)
  R* sIy = sIx + RN;  // ICEy'
  R* sId = sIy + RN;  // IDz
  // structure-of-arrays coefficient tables (conflict-free column access)
  R* xf1 = sId + RN;  // f1H along x (rows)
  R* xf2 = xf1 + RI;  // f2H
  R* xg3 = xf2 + RI;  // 2 aH
  R* xaD = xg3 + RI;  // aD
  R* xpD = xaD + RI;  // pD
  R* yf1 = xpD + RI;
  R* yf2 = yf1 + RJ;
  R* yg3 = yf2 + RJ;
  R* yaD = yg3 + RJ;
  R* ypD = yaD + RJ;
  R* sAmp = ypD + RJ;
  const int nst = a.K;  // steps of this launch, <= K
  const int gi0 = blockIdx.y * TI - K, gj0 = blockIdx.x * TJ - K;
  const int tid = threadIdx.x;
  auto gi = [&](int r) { int v = (gi0 + r) % a.nx; return v < 0 ? v + a.nx : v; };
  auto gj = [&](int c) { int v = (gj0 + c) % a.ny; return v < 0 ? v + a.ny : v; };
  int pl = 0;
  for (int r = tid; r < RI; r += NT) {
    const AxisCoef<R> c = a.ax[gi(r)];
    xf1[r] = c.f1H; xf2[r] = c.f2H; xg3[r] = R(2) * c.aH; xaD[r] = c.aD; xpD[r] = c.pD;
    pl |= (c.aH != R(0)) | (c.aD != R(0));
  }
  for (int q = tid; q < RJ; q += NT) {
    const AxisCoef<R> c = a.ay[gj(q)];
    yf1[q] = c.f1H; yf2[q] = c.f2H; yg3[q] = R(2) * c.aH; yaD[q] = c.aD; ypD[q] = c.pD;
    pl |= (c.aH != R(0)) | (c.aD != R(0));
  }
  if (!PERSIST)
    for (int st = tid; st < nst; st += NT) sAmp[st] = a.ns > 0 ? a.amps[a.t0 + st] : R(0);
  for (int q = tid; q < RN; q += NT) sW[q] = R(0);
  const bool pml = __syncthreads_or(pl);
  for (int k = tid; k < a.ns; k += NT) {
    const int n = a.src_idx[k];
    const int ii = n / a.ny, jj = n - ii * a.ny;
    int r = (ii - gi0) % a.nx;
    if (r < 0) r += a.nx;
    int c = (jj - gj0) % a.ny;
    if (c < 0) c += a.ny;
    if (r < RI && c < RJ) atomicAdd(&sW[r * RJ + c], a.src_w[k]);
  }
  __syncthreads();
  R hx[CPT], hy[CPT], dz[CPT], ie[CPT];
  // PML integrals of the owned cells: private to the cell, so in registers
  // when the register budget allows (float, <= 512 threads), else in shared
  // memory
  constexpr bool REG_INT = NT <= 512 && sizeof(R) == 4;
  // every owned cell lies in the same region column when NT is a multiple
  // of the region width: its column coefficients then live in registers
  constexpr bool COLC = (NT % RJ) == 0;
  R ixr[REG_INT ? CPT : 1], iyr[REG_INT ? CPT : 1], idr[REG_INT ? CPT : 1];
  // D-phase PML coefficients of the owned cells (same budget condition)
  R dm1[REG_INT ? CPT : 1], dm2[REG_INT ? CPT : 1], dm4[REG_INT ? CPT : 1];
  unsigned srcmask = 0;  // bit k: owned cell k has a source
  unsigned pmlmask = 0;  // bit k: some cell of this warp's slot k lies on a PML row/column
#pragma unroll
  for (int k = 0; k < CPT; ++k) {
    const int q = tid + k * NT;
    hx[k] = hy[k] = dz[k] = ie[k] = R(0);
    bool cell_pml = false;
    if (q < RN) {
      const int r = q / RJ, c = q - r * RJ;
      const size_t n = (size_t)gi(r) * a.ny + gj(c);
      hx[k] = a.hx_i[n];
      hy[k] = a.hy_i[n];
      dz[k] = a.dz_i[n];
      ie[k] = a.iez[n];
      cell_pml = (xg3[r] != R(0)) | (yg3[c] != R(0)) | (xaD[r] != R(0)) | (yaD[c] != R(0));
      if constexpr (REG_INT) {
        ixr[k] = pml ? a.icex_i[n] : R(0);
        iyr[k] = pml ? a.icey_i[n] : R(0);
        idr[k] = pml ? a.idz_i[n] : R(0);
      } else if (pml) {
        sIx[q] = a.icex_i[n];
        sIy[q] = a.icey_i[n];
        sId[q] = a.idz_i[n];
      }
      if (sW[q] != R(0)) srcmask |= 1u << k;
      sEz[q] = dz[k] * ie[k];
    }
    if (__any_sync(0xffffffffu, cell_pml)) pmlmask |= 1u << k;
  }
  __syncthreads();
  const R S = a.S;
  R cf1 = R(0), cf2 = R(0), cg3 = R(0), caD = R(0), cpD = R(0);
  if constexpr (COLC) {
    const int c0 = tid % RJ;
    cf1 = yf1[c0]; cf2 = yf2[c0]; cg3 = yg3[c0]; caD = yaD[c0]; cpD = ypD[c0];
  }
  if constexpr (REG_INT) {
#pragma unroll
    for (int k = 0; k < CPT; ++k) {
      const int q = tid + k * NT;
      const int r = q < RN ? q / RJ : 0, c = q < RN ? q - r * RJ : 0;
      const R ax = xaD[r], ay = yaD[c];
      const R pd = xpD[r] * ypD[c];
      dm1[k] = (R(1) - ax - ay - ax * ay) * pd;
      dm2[k] = S * pd;
      dm4[k] = R(-4) * ax * ay * pd;
    }
  }
  // interior cells owned by this tile (inside the grid) -> 6 field arrays
  auto publish = [&](R* const* o) {
#pragma unroll
    for (int k = 0; k < CPT; ++k) {
      const int q = tid + k * NT;
      if (q < RN) {
        const int r = q / RJ, c = q - r * RJ;
        const int ii = gi0 + r, jj = gj0 + c;
        if (r >= K && r < K + TI && c >= K && c < K + TJ && ii < a.nx && jj < a.ny) {
          const size_t n = (size_t)ii * a.ny + jj;
          o[0][n] = hx[k];
          o[1][n] = hy[k];
          o[2][n] = dz[k];
          if (pml) {
            if constexpr (REG_INT) {
              o[3][n] = ixr[k];
              o[4][n] = iyr[k];
              o[5][n] = idr[k];
            } else {
              o[3][n] = sIx[q];
              o[4][n] = sIy[q];
              o[5][n] = sId[q];
            }
          }
        }
      }
    }
  };
  const int nblk = PERSIST ? (a.nsteps + K - 1) / K : 1;
  const int tile = blockIdx.y * gridDim.x + blockIdx.x;
  for (int blk = 0; blk < nblk; ++blk) {
  const int t0 = PERSIST ? blk * K : a.t0;
  const int bst = PERSIST ? min(K, a.nsteps - t0) : nst;
  if (PERSIST) {
    for (int st = tid; st < bst; st += NT) sAmp[st] = a.ns > 0 ? a.amps[t0 + st] : R(0);
    __syncthreads();
  }
  for (int st = 0; st < bst; ++st) {
    const R amp = sAmp[st];
    if (!pml) {
      // no PML cell in the region: a = 0, so f1 = 1, f2 = S, mDz1 = 1,
      // mDz2 = S, mDz4 = 0 and no integral is accumulated
#pragma unroll
      for (int k = 0; k < CPT; ++k) {
        const int q = tid + k * NT;
        if (q < RN) {
          const int r = q / RJ, c = q - r * RJ;
          const R ez = sEz[q];
          const R ezr = (c < RJ - 1) ? sEz[q + 1] : ez;
          const R ezd = (r < RI - 1) ? sEz[q + RJ] : ez;
          hx[k] = hx[k] - S * (ezr - ez);
          hy[k] = hy[k] - S * (-(ezd - ez));
          sHx[q] = hx[k];
          sHy[q] = hy[k];
        }
      }
      __syncthreads();
#pragma unroll
      for (int k = 0; k < CPT; ++k) {
        const int q = tid + k * NT;
        if (q < RN) {
          const int r = q / RJ, c = q - r * RJ;
          const R hyu = (r > 0) ? sHy[q - RJ] : hy[k];
          const R hxl = (c > 0) ? sHx[q - 1] : hx[k];
          R v = dz[k] + S * ((hy[k] - hyu) - (hx[k] - hxl));
          if (srcmask & (1u << k)) v += sW[q] * amp;
          dz[k] = v;
          sEz[q] = v * ie[k];
        }
      }
    } else {
      // PML tile: warp slots without a PML cell still take the a = 0 form
#pragma unroll
      for (int k = 0; k < CPT; ++k) {
        const int q = tid + k * NT;
        if (q < RN) {
          const int r = q / RJ, c = q - r * RJ;
          const R ez = sEz[q];
          const R ezr = (c < RJ - 1) ? sEz[q + 1] : ez;
          const R ezd = (r < RI - 1) ? sEz[q + RJ] : ez;
          const R dEy = ezr - ez;
          const R dEx = -(ezd - ez);
          if (!(pmlmask & (1u << k))) {
            hx[k] = hx[k] - S * dEy;
            hy[k] = hy[k] - S * dEx;
          } else {
            const R gx = xg3[r], gy = COLC ? cg3 : yg3[c];
            R ix = R(0), iy = R(0);
            if constexpr (REG_INT) {
              if (gx != R(0)) { ixr[k] += dEy; ix = ixr[k]; }
              if (gy != R(0)) { iyr[k] += dEx; iy = iyr[k]; }
            } else {
              if (gx != R(0)) { ix = sIx[q] + dEy; sIx[q] = ix; }
              if (gy != R(0)) { iy = sIy[q] + dEx; sIy[q] = iy; }
            }
            const R f1c = COLC ? cf1 : yf1[c], f2c = COLC ? cf2 : yf2[c];
            hx[k] = f1c * hx[k] - f2c * (dEy + gx * ix);
            hy[k] = xf1[r] * hy[k] - xf2[r] * (dEx + gy * iy);
          }
          sHx[q] = hx[k];
          sHy[q] = hy[k];
        }
      }
      __syncthreads();
#pragma unroll
      for (int k = 0; k < CPT; ++k) {
        const int q = tid + k * NT;
        if (q < RN) {
          const int r = q / RJ, c = q - r * RJ;
          const R hyu = (r > 0) ? sHy[q - RJ] : hy[k];
          const R hxl = (c > 0) ? sHx[q - 1] : hx[k];
          const R ch = (hy[k] - hyu) - (hx[k] - hxl);
          R v;
          if (!(pmlmask & (1u << k))) {
            v = dz[k] + S * ch;
          } else {
            R m1, m2, m4;
            if constexpr (REG_INT) {
              m1 = dm1[k];
              m2 = dm2[k];
              m4 = dm4[k];
            } else {
              const R ax = xaD[r], ay = COLC ? caD : yaD[c];
              const R pd = xpD[r] * (COLC ? cpD : ypD[c]);
              m1 = (R(1) - ax - ay - ax * ay) * pd;
              m2 = S * pd;
              m4 = R(-4) * ax * ay * pd;
            }
            R id = R(0);
            if (m4 != R(0)) {
              if constexpr (REG_INT) {
                idr[k] += dz[k];
                id = idr[k];
              } else {
                id = sId[q] + dz[k];
                sId[q] = id;
              }
            }
            v = m1 * dz[k] + m2 * ch + m4 * id;
          }
          if (srcmask & (1u << k)) v += sW[q] * amp;
          dz[k] = v;
          sEz[q] = v * ie[k];
        }
      }
    }
    __syncthreads();
    if constexpr (HIST) {  // Dz after this step, interior cells (adjoint recompute)
#pragma unroll
      for (int k = 0; k < CPT; ++k) {
        const int q = tid + k * NT;
        if (q < RN) {
          const int r = q / RJ, c = q - r * RJ;
          const int ii = gi0 + r, jj = gj0 + c;
          if (r >= K && r < K + TI && c >= K && c < K + TJ && ii < a.nx && jj < a.ny)
            a.dz_hist[(size_t)(a.t0 + st + 1) * a.nx * a.ny + (size_t)ii * a.ny + jj] = dz[k];
        }
      }
    }
    // probes of interior cells: Ez after this step
    for (int k = tid; k < a.np; k += NT) {
      const int n = a.probe_idx[k];
      const int ii = n / a.ny, jj = n - ii * a.ny;
      const int r = ii - gi0, c = jj - gj0;
      if (r >= K && r < K + TI && c >= K && c < K + TJ)
        a.probe_out[(size_t)(t0 + st) * a.np + k] = sEz[r * RJ + c];
    }
  }
  if constexpr (PERSIST) {
    if (blk + 1 < nblk) {
      R* const* xb = a.xb[blk & 1];
      publish(xb);
      __syncthreads();
      // bar.sync orders the CTA's stores before thread 0's release
      if (tid == 0) st_release_gpu(a.flags + tile * FLAG_STRIDE, blk + 1);
      // bounded busy wait for the neighbours' block (about 2^24 L2 round
      // trips at most, well under a minute)
      bool late = false;
      if (tid < NBR_MAX) {
        const int nb = a.nbr[tile * NBR_MAX + tid];
        if (nb >= 0) {
          int spins = 0;
          while (ld_acquire_gpu(a.flags + nb * FLAG_STRIDE) < blk + 1) {
            if (++spins > (1 << 24) || ((spins & 1023) == 0 && ld_acquire_gpu(a.fault) != 0)) {
              late = true;
              break;
            }
          }
        }
      }
      if (__syncthreads_or(late)) {
        if (tid == 0) atomicExch(a.fault, 1);
        return;
      }
      // ring cells: the neighbours' published values (through L2)
#pragma unroll
      for (int k = 0; k < CPT; ++k) {
        const int q = tid + k * NT;
        if (q < RN) {
          const int r = q / RJ, c = q - r * RJ;
          if (!(r >= K && r < K + TI && c >= K && c < K + TJ)) {
            const size_t n = (size_t)gi(r) * a.ny + gj(c);
            hx[k] = __ldcg(xb[0] + n);
            hy[k] = __ldcg(xb[1] + n);
            dz[k] = __ldcg(xb[2] + n);
            if (pml) {
              if constexpr (REG_INT) {
                ixr[k] = __ldcg(xb[3] + n);
                iyr[k] = __ldcg(xb[4] + n);
                idr[k] = __ldcg(xb[5] + n);
              } else {
                sIx[q] = __ldcg(xb[3] + n);
                sIy[q] = __ldcg(xb[4] + n);
                sId[q] = __ldcg(xb[5] + n);
              }
            }
            sEz[q] = dz[k] * ie[k];
          }
        }
      }
      __syncthreads();
    }
  }
  }  // blocks of K steps
  // write back the tile interior
  if constexpr (PERSIST) {
    publish(a.xb[(nblk - 1) & 1]);
  } else {
    R* const o[6] = {a.hx_o, a.hy_o, a.dz_o, a.icex_o, a.icey_o, a.idz_o};
    publish(o);
  }
}

// ------------------------------------------------- register-strip TM kernel
// The same K-step time-blocked recurrence as k_tm_tile with the state in
// registers: lane l of warp w owns columns 2l and 2l+1 of rows w*S .. w*S+S-1
// of a (W*S) x 64 region (interior (W*S - 2K) x (64 - 2K)).  Left and right
// neighbours come by warp shuffle, up and down neighbours from the thread's
// own rows; only the first Ez row and the last Hy row of each warp cross
// shared memory, once per phase.  The PML form is evaluated for every cell of
// a PML region (for a = 0 it reduces exactly to the interior form), and the
// integrals are accumulated only where their coefficient is non-zero, as in
// k_tm_tile.  PERSIST: the whole run in one cooperative launch with the ring
// exchange of k_tm_tile.
constexpr int STRIP_PROBE_MAX = 2048;

template <int W, int S, int K>
struct Strip {
  static constexpr int RI = W * S, RJ = 64, TI = RI - 2 * K, TJ = RJ - 2 * K, NT = 32 * W;
  static constexpr int RN = RI * RJ;
  template <typename R>
  static constexpr size_t smem(int np) {
    return (size_t)RN * sizeof(R) + 2 * (size_t)W * RJ * sizeof(R) + 2 * (size_t)K * sizeof(R) +
           (np > 0 ? (size_t)(RN + np) * sizeof(int) : 0);
  }
};

template <typename R, int W, int S, int K, bool PERSIST>
__global__ void __launch_bounds__(32 * W, 1) k_tm_strip(TBArgs<R> a) {
  using G = Strip<W, S, K>;
  constexpr int RI = G::RI, RJ = G::RJ, TI = G::TI, TJ = G::TJ, NT = G::NT, RN = G::RN;
  extern __shared__ __align__(16) unsigned char smraw[];
  R* sW = (R*)smraw;             // [RN] source weight per region cell
  R* ezTop = sW + RN;            // [W][RJ] first Ez row of each warp
  R* hyBot = ezTop + W * RJ;     // [W][RJ] last Hy row of each warp
  R* sAmp = hyBot + W * RJ;      // [2][K]: this block's and the next block's amplitudes
  int* sPid = (int*)(sAmp + 2 * K);  // [RN] first probe at a region cell (-1: none)
  int* sPnext = sPid + RN;       // [np] next probe at the same cell
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int gi0 = blockIdx.y * TI - K, gj0 = blockIdx.x * TJ - K;
  auto gi = [&](int r) { int v = (gi0 + r) % a.nx; return v < 0 ? v + a.nx : v; };
  auto gj = [&](int c) { int v = (gj0 + c) % a.ny; return v < 0 ? v + a.ny : v; };
  const int c0 = 2 * lane;
  // coefficients: rows (x tables) and the thread's two columns (y tables)
  R xf1[S], xf2[S], xg3[S], yf1[2], yf2[2], yg3[2];
  R m1[S][2], m2[S][2], m4[S][2];
  int pl = 0;
  {
    R xaD[S], xpD[S], yaD[2], ypD[2];
#pragma unroll
    for (int s = 0; s < S; ++s) {
      const AxisCoef<R> c = a.ax[gi(warp * S + s)];
      xf1[s] = c.f1H; xf2[s] = c.f2H; xg3[s] = R(2) * c.aH; xaD[s] = c.aD; xpD[s] = c.pD;
      pl |= (c.aH != R(0)) | (c.aD != R(0));
    }
#pragma unroll
    for (int q = 0; q < 2; ++q) {
      const AxisCoef<R> c = a.ay[gj(c0 + q)];
      yf1[q] = c.f1H; yf2[q] = c.f2H; yg3[q] = R(2) * c.aH; yaD[q] = c.aD; ypD[q] = c.pD;
      pl |= (c.aH != R(0)) | (c.aD != R(0));
    }
#pragma unroll
    for (int s = 0; s < S; ++s)
#pragma unroll
      for (int q = 0; q < 2; ++q) {
        const R ax = xaD[s], ay = yaD[q], pd = xpD[s] * ypD[q];
        m1[s][q] = (R(1) - ax - ay - ax * ay) * pd;
        m2[s][q] = a.S * pd;
        m4[s][q] = R(-4) * ax * ay * pd;
      }
  }
  for (int q = tid; q < RN; q += NT) sW[q] = R(0);
  if (a.np > 0)
    for (int q = tid; q < RN; q += NT) sPid[q] = -1;
  const bool pml = __syncthreads_or(pl);
  for (int k = tid; k < a.ns; k += NT) {
    const int n = a.src_idx[k];
    const int ii = n / a.ny, jj = n - ii * a.ny;
    int r = (ii - gi0) % a.nx;
    if (r < 0) r += a.nx;
    int c = (jj - gj0) % a.ny;
    if (c < 0) c += a.ny;
    if (r < RI && c < RJ) atomicAdd(&sW[r * RJ + c], a.src_w[k]);
  }
  for (int k = tid; k < a.np; k += NT) {
    const int n = a.probe_idx[k];
    const int ii = n / a.ny, jj = n - ii * a.ny;
    const int r = ii - gi0, c = jj - gj0;
    if (r >= K && r < K + TI && c >= K && c < K + TJ) sPnext[k] = atomicExch(&sPid[r * RJ + c], k);
  }
  R hx[S][2], hy[S][2], dz[S][2], ie[S][2], ez[S][2], ix[S][2], iy[S][2], id[S][2];
  // flat grid index of each owned cell (wrapped), and which of them this
  // tile owns (interior, inside the grid) and publishes
  int gofs[S][2];
  unsigned srcmask = 0, probemask = 0, ownmask = 0, bandmask = 0;
  __syncthreads();
#pragma unroll
  for (int s = 0; s < S; ++s)
#pragma unroll
    for (int q = 0; q < 2; ++q) {
      const int r = warp * S + s, c = c0 + q;
      gofs[s][q] = gi(r) * a.ny + gj(c);
      if (r >= K && r < K + TI && c >= K && c < K + TJ && gi0 + r < a.nx && gj0 + c < a.ny) {
        ownmask |= 1u << (2 * s + q);
        // published at an exchange only if it lies in the ring of some
        // neighbour (partial tiles at the grid edge wrap, so this is more
        // than the K-wide band of the interior)
        if (PERSIST) {
          const int ii = gi0 + r, jj = gj0 + c;
          const int gx = gridDim.x;
          for (int k = 0; k < NBR_MAX; ++k) {
            const int nb = a.nbr[(blockIdx.y * gx + blockIdx.x) * NBR_MAX + k];
            if (nb < 0) break;
            const int by = nb / gx, bx = nb - (nb / gx) * gx;
            int dr = (ii - (by * TI - K)) % a.nx, dc = (jj - (bx * TJ - K)) % a.ny;
            if (dr < 0) dr += a.nx;
            if (dc < 0) dc += a.ny;
            if (dr < RI && dc < RJ && !(dr >= K && dr < K + TI && dc >= K && dc < K + TJ))
              bandmask |= 1u << (2 * s + q);
          }
        }
      }
      const size_t n = (size_t)gofs[s][q];
      hx[s][q] = a.hx_i[n];
      hy[s][q] = a.hy_i[n];
      dz[s][q] = a.dz_i[n];
      ie[s][q] = a.iez[n];
      ix[s][q] = pml ? a.icex_i[n] : R(0);
      iy[s][q] = pml ? a.icey_i[n] : R(0);
      id[s][q] = pml ? a.idz_i[n] : R(0);
      ez[s][q] = dz[s][q] * ie[s][q];
      if (sW[r * RJ + c] != R(0)) srcmask |= 1u << (2 * s + q);
      if (a.np > 0 && sPid[r * RJ + c] >= 0) probemask |= 1u << (2 * s + q);
    }
  const R Sc = a.S;
  // warps without any PML coefficient take the interior form (for a = 0 the
  // PML form gives the same numbers)
  bool cell_pml = false;
#pragma unroll
  for (int s = 0; s < S; ++s)
#pragma unroll
    for (int q = 0; q < 2; ++q)
      cell_pml |= (xg3[s] != R(0)) | (yg3[q] != R(0)) | (m4[s][q] != R(0)) |
                  (m1[s][q] != R(1)) | (m2[s][q] != Sc) | (xf1[s] != R(1)) | (yf1[q] != R(1)) |
                  (xf2[s] != Sc) | (yf2[q] != Sc);
  const bool wpml = pml && __any_sync(0xffffffffu, cell_pml);
  const int wn = warp + 1 < W ? warp + 1 : warp;  // warp below (the last warp reads its own row)
  const int wp = warp > 0 ? warp - 1 : warp;      // warp above
  auto publish = [&](R* const* o, unsigned mask) {
#pragma unroll
    for (int s = 0; s < S; ++s)
#pragma unroll
      for (int q = 0; q < 2; ++q) {
        if (mask & (1u << (2 * s + q))) {
          const size_t n = (size_t)gofs[s][q];
          o[0][n] = hx[s][q];
          o[1][n] = hy[s][q];
          o[2][n] = dz[s][q];
          if (pml) {
            o[3][n] = ix[s][q];
            o[4][n] = iy[s][q];
            o[5][n] = id[s][q];
          }
        }
      }
  };
  ezTop[warp * RJ + c0] = ez[0][0];
  ezTop[warp * RJ + c0 + 1] = ez[0][1];
  __syncthreads();
  const int nblk = PERSIST ? (a.nsteps + K - 1) / K : 1;
  const int tile = blockIdx.y * gridDim.x + blockIdx.x;
  // amplitudes of a block's steps; the next block's are fetched before the
  // neighbour wait, so no load latency sits between two blocks
  auto load_amps = [&](int blk_) {
    const int t0_ = PERSIST ? blk_ * K : a.t0;
    const int n_ = PERSIST ? min(K, a.nsteps - t0_) : a.K;
    for (int st = tid; st < n_; st += NT) sAmp[(blk_ & 1) * K + st] = a.ns > 0 ? a.amps[t0_ + st] : R(0);
  };
  load_amps(0);
  __syncthreads();
  for (int blk = 0; blk < nblk; ++blk) {
    const int t0 = PERSIST ? blk * K : a.t0;
    const int bst = PERSIST ? min(K, a.nsteps - t0) : a.K;
    const R* amps = sAmp + (blk & 1) * K;
    for (int st = 0; st < bst; ++st) {
      // ---- H phase: Ez at (i, j+1) by shuffle, at (i+1, j) from the next row
#pragma unroll
      for (int s = 0; s < S; ++s) {
        const R ezr = __shfl_down_sync(0xffffffffu, ez[s][0], 1);  // lane 31: its own (region edge)
        const R right[2] = {ez[s][1], ezr};
        R below[2];
        if (s + 1 < S) {
          below[0] = ez[s + 1][0];
          below[1] = ez[s + 1][1];
        } else {
          below[0] = ezTop[wn * RJ + c0];
          below[1] = ezTop[wn * RJ + c0 + 1];
        }
#pragma unroll
        for (int q = 0; q < 2; ++q) {
          const R dEy = right[q] - ez[s][q];
          const R dEx = -(below[q] - ez[s][q]);
          if (!wpml) {
            hx[s][q] = hx[s][q] - Sc * dEy;
            hy[s][q] = hy[s][q] - Sc * dEx;
          } else {
            const R gx = xg3[s], gy = yg3[q];
            R vx = R(0), vy = R(0);
            if (gx != R(0)) { ix[s][q] += dEy; vx = ix[s][q]; }
            if (gy != R(0)) { iy[s][q] += dEx; vy = iy[s][q]; }
            hx[s][q] = yf1[q] * hx[s][q] - yf2[q] * (dEy + gx * vx);
            hy[s][q] = xf1[s] * hy[s][q] - xf2[s] * (dEx + gy * vy);
          }
        }
      }
      hyBot[warp * RJ + c0] = hy[S - 1][0];
      hyBot[warp * RJ + c0 + 1] = hy[S - 1][1];
      __syncthreads();
      // ---- D phase: Hx at (i, j-1) by shuffle, Hy at (i-1, j) from the row above
      const R amp = amps[st];
#pragma unroll
      for (int s = 0; s < S; ++s) {
        const R hxl0 = __shfl_up_sync(0xffffffffu, hx[s][1], 1);  // lane 0: its own (region edge)
        const R left[2] = {hxl0, hx[s][0]};
        R up[2];
        if (s > 0) {
          up[0] = hy[s - 1][0];
          up[1] = hy[s - 1][1];
        } else {
          up[0] = hyBot[wp * RJ + c0];
          up[1] = hyBot[wp * RJ + c0 + 1];
        }
#pragma unroll
        for (int q = 0; q < 2; ++q) {
          const R ch = (hy[s][q] - up[q]) - (hx[s][q] - left[q]);
          R v;
          if (!wpml) {
            v = dz[s][q] + Sc * ch;
          } else {
            R vd = R(0);
            if (m4[s][q] != R(0)) {
              id[s][q] += dz[s][q];
              vd = id[s][q];
            }
            v = m1[s][q] * dz[s][q] + m2[s][q] * ch + m4[s][q] * vd;
          }
          if (srcmask & (1u << (2 * s + q))) v += sW[(warp * S + s) * RJ + c0 + q] * amp;
          dz[s][q] = v;
          ez[s][q] = v * ie[s][q];
        }
      }
      ezTop[warp * RJ + c0] = ez[0][0];
      ezTop[warp * RJ + c0 + 1] = ez[0][1];
      if (probemask) {
#pragma unroll
        for (int s = 0; s < S; ++s)
#pragma unroll
          for (int q = 0; q < 2; ++q)
            if (probemask & (1u << (2 * s + q)))
              for (int k = sPid[(warp * S + s) * RJ + c0 + q]; k >= 0; k = sPnext[k])
                a.probe_out[(size_t)(t0 + st) * a.np + k] = ez[s][q];
      }
      __syncthreads();
    }
    if constexpr (PERSIST) {
      if (blk + 1 < nblk) {
        R* const* xb = a.xb[blk & 1];
        publish(xb, bandmask);
        load_amps(blk + 1);
        __syncthreads();
        // bar.sync orders the CTA's stores before thread 0's release
        if (tid == 0) st_release_gpu(a.flags + tile * FLAG_STRIDE, blk + 1);
        bool late = false;
        if (tid < NBR_MAX) {
          const int nb = a.nbr[tile * NBR_MAX + tid];
          if (nb >= 0) {
            int spins = 0;
            // busy poll (a sleep's granularity costs more than the wait);
            // bounded: about 2^24 L2 round trips, well under a minute
            // relaxed polls, one acquire fence once the flag is seen
            while (ld_relaxed_gpu(a.flags + nb * FLAG_STRIDE) < blk + 1) {
              if (++spins > (1 << 24) || ((spins & 1023) == 0 && ld_relaxed_gpu(a.fault) != 0)) {
                late = true;
                break;
              }
            }
            fence_acq_rel_gpu();
          }
        }
        if (__syncthreads_or(late)) {
          if (tid == 0) atomicExch(a.fault, 1);
          return;
        }
#pragma unroll
        for (int s = 0; s < S; ++s)
#pragma unroll
          for (int q = 0; q < 2; ++q) {
            const int r = warp * S + s, c = c0 + q;
            if (!(r >= K && r < K + TI && c >= K && c < K + TJ)) {
              const size_t n = (size_t)gofs[s][q];
              hx[s][q] = __ldcg(xb[0] + n);
              hy[s][q] = __ldcg(xb[1] + n);
              dz[s][q] = __ldcg(xb[2] + n);
              if (pml) {
                ix[s][q] = __ldcg(xb[3] + n);
                iy[s][q] = __ldcg(xb[4] + n);
                id[s][q] = __ldcg(xb[5] + n);
              }
              ez[s][q] = dz[s][q] * ie[s][q];
            }
          }
        ezTop[warp * RJ + c0] = ez[0][0];
        ezTop[warp * RJ + c0 + 1] = ez[0][1];
        __syncthreads();
      }
    }
  }
  if constexpr (PERSIST) {
    publish(a.xb[(nblk - 1) & 1], ownmask);
  } else {
    R* const o[6] = {a.hx_o, a.hy_o, a.dz_o, a.icex_o, a.icey_o, a.idz_o};
    publish(o, ownmask);
  }
}

// Tile configurations (TI, TJ, K, threads); the launcher picks one per grid.
struct TileCfg {
  int ti, tj, k, nt;
};
constexpr TileCfg TILE_CFGS[] = {{48, 48, 8, 1024}, {48, 48, 8, 512}, {32, 48, 8, 512},
                                 {26, 48, 8, 512},  {25, 50, 8, 512}, {16, 48, 8, 512}};
constexpr int N_TILE_CFGS = sizeof(TILE_CFGS) / sizeof(TILE_CFGS[0]);

template <typename R, int I>
struct TileLauncher {
  static constexpr TileCfg c = TILE_CFGS[I];
  using T = Tile<R, c.ti, c.tj, c.k, c.nt>;
  static int prepare() {
    return allow_dynamic_smem((const void*)k_tm_tile<R, c.ti, c.tj, c.k, c.nt>, (int)T::smem);
  }
  static void launch(dim3 g, const TBArgs<R>& a, cudaStream_t s) {
    k_tm_tile<R, c.ti, c.tj, c.k, c.nt><<<g, c.nt, T::smem, s>>>(a);
  }
  static constexpr size_t smem_bytes = T::smem;
  static int per_sm() {
    int n = 0;
    if (prepare() != CEV_OK) return 1;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_tm_tile<R, c.ti, c.tj, c.k, c.nt>,
                                                      c.nt, T::smem) != cudaSuccess || n < 1)
      n = 1;
    return n;
  }
};

template <typename R, int I = 0>
size_t tile_smem(int cfg) {
  if constexpr (I < N_TILE_CFGS) {
    if (cfg == I) return TileLauncher<R, I>::smem_bytes;
    return tile_smem<R, I + 1>(cfg);
  } else {
    return 0;
  }
}

template <typename R, int I = 0>
int tile_per_sm(int cfg) {
  if constexpr (I < N_TILE_CFGS) {
    if (cfg == I) return TileLauncher<R, I>::per_sm();
    return tile_per_sm<R, I + 1>(cfg);
  } else {
    return 1;
  }
}

template <typename R, int I = 0>
int tile_dispatch(int cfg, bool prepare, dim3 g, const TBArgs<R>& a, cudaStream_t s) {
  if constexpr (I < N_TILE_CFGS) {
    if (cfg == I) {
      if (prepare) return TileLauncher<R, I>::prepare();
      TileLauncher<R, I>::launch(g, a, s);
      return CEV_OK;
    }
    return tile_dispatch<R, I + 1>(cfg, prepare, g, a, s);
  } else {
    set_error("bad tile configuration %d", cfg);
    return CEV_ERR_INVALID;
  }
}

// Tile choice: CEV_FDTD_TILE=<index> overrides.  Otherwise 48x48 tiles with
// 512 threads (measured best from 1024^2 to 4096^2 once the PML integrals
// and coefficients moved to registers), or 32x48 tiles with 512 threads when
// 48x48 tiles would not fill the GPU once (measured best at 400^2).
template <typename R>
static int pick_tile(int nx, int ny) {
  auto fits = [&](int v) {
    const TileCfg c = TILE_CFGS[v];
    return nx >= c.ti + 2 * c.k && ny >= c.tj + 2 * c.k && tile_smem<R>(v) <= 227 * 1024;
  };
  if (const char* e = std::getenv("CEV_FDTD_TILE")) {
    const int v = std::atoi(e);
    if (v >= 0 && v < N_TILE_CFGS && fits(v)) return v;
  }
  const long tiles0 = (long)((nx + 47) / 48) * ((ny + 47) / 48);
  const int order_big[] = {1, 0, 2, 5};
  const int order_small[] = {2, 3, 5, 0};
  const int* order = tiles0 >= sm_count() ? order_big : order_small;
  for (int k = 0; k < 4; ++k)
    if (fits(order[k])) return order[k];
  return -1;
}

// ------------------------------------------------------------ TM adjoint
// Reverse of one TM step n (see header comment for the forward form):
//   aCH = m2 aDz ; aIDz += m4 aDz ; aDz_prev = m1 aDz + aIDz
//   aHy_t = aHy + aCH - aCH[i+1,j] ; aHx_t = aHx - (aCH - aCH[i,j+1])
//   aHx = f1Hy aHx_t ; t = -f2Hy aHx_t ; aICEx += 2aHx t ; adEy = t + aICEx  (same for y)
//   aEz^{n-1} = w_{n-1} p + adEy[i,j-1] - adEy + adEx - adEx[i-1,j]
//   aDz^{n-1} = aDz_prev + aEz^{n-1}/eps ; geps += aEz^{n-1} (-Dz^{n-1}/eps^2)
template <typename R>
struct AdjArgs {
  int nx, ny;
  R* ahx; R* ahy; R* adz; R* aicex; R* aicey; R* aidz;
  R* ach; R* adey; R* adex; R* adzp;
  const R* iez;
  const AxisCoef<R>* ax;
  const AxisCoef<R>* ay;
  R S;
};

template <typename R>
__global__ void k_adj_a(AdjArgs<R> a) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  const int i = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= a.nx || j >= a.ny) return;
  const size_t n = (size_t)i * a.ny + j;
  R m1, m2, m4;
  dz_coefs(a.ax[i], a.ay[j], a.S, m1, m2, m4);
  const R adz = a.adz[n];
  a.ach[n] = m2 * adz;
  R aid = a.aidz[n];
  if (m4 != R(0)) { aid += m4 * adz; a.aidz[n] = aid; }
  a.adzp[n] = m1 * adz + aid;
}

template <typename R>
__global__ void k_adj_b(AdjArgs<R> a) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  const int i = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= a.nx || j >= a.ny) return;
  const size_t n = (size_t)i * a.ny + j;
  const int ip = i + 1 == a.nx ? 0 : i + 1, jp = j + 1 == a.ny ? 0 : j + 1;
  const R ach = a.ach[n];
  const R ahy_t = a.ahy[n] + ach - a.ach[(size_t)ip * a.ny + j];
  const R ahx_t = a.ahx[n] - (ach - a.ach[(size_t)i * a.ny + jp]);
  const AxisCoef<R> cx = a.ax[i], cy = a.ay[j];
  a.ahx[n] = cy.f1H * ahx_t;
  R t = -cy.f2H * ahx_t;
  R ai = R(0);
  if (cx.aH != R(0)) { ai = a.aicex[n] + R(2) * cx.aH * t; a.aicex[n] = ai; }
  a.adey[n] = t + ai;
  a.ahy[n] = cx.f1H * ahy_t;
  t = -cx.f2H * ahy_t;
  ai = R(0);
  if (cy.aH != R(0)) { ai = a.aicey[n] + R(2) * cy.aH * t; a.aicey[n] = ai; }
  a.adex[n] = t + ai;
}

// finishes the step: aDz for Ez^{n-1}; gradient term with Dz^{n-1}
template <typename R>
__global__ void k_adj_c(AdjArgs<R> a, const R* dz_prev, double* geps, int np, const int* pidx,
                        const R* wrow) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  const int i = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= a.nx || j >= a.ny) return;
  const size_t n = (size_t)i * a.ny + j;
  const int im = i == 0 ? a.nx - 1 : i - 1, jm = j == 0 ? a.ny - 1 : j - 1;
  R aez = a.adey[(size_t)i * a.ny + jm] - a.adey[n] + a.adex[n] - a.adex[(size_t)im * a.ny + j];
  if (wrow) {
    for (int k = 0; k < np; ++k)
      if (pidx[k] == (int)n) aez += wrow[k];
  }
  const R ie = a.iez[n];
  a.adz[n] = a.adzp[n] + aez * ie;
  if (dz_prev) geps[n] += (double)aez * (double)(-dz_prev[n] * ie * ie);
}

// gradient of an output Ez^n = Dz^n / eps: aDz^n += g iez ; geps += g (-Dz^n iez^2)
template <typename R>
__global__ void k_adj_out_ez(int N, R* adz, const R* gez, const R* dz, const R* iez, double* geps) {
  for (size_t n = blockIdx.x * (size_t)blockDim.x + threadIdx.x; n < (size_t)N;
       n += (size_t)gridDim.x * blockDim.x) {
    const R g = gez[n], ie = iez[n];
    adz[n] += g * ie;
    geps[n] += (double)g * (double)(-dz[n] * ie * ie);
  }
}

// initial adjoint for the last output step T: aEz^T = w_T p
template <typename R>
__global__ void k_adj_init(int N, R* adz, const R* iez, double* geps, const R* dz_T, int np,
                           const int* pidx, const R* wrow) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= np) return;
  const int n = pidx[k];
  const R ie = iez[n];
  atomicAdd(&adz[n], wrow[k] * ie);
  atomicAdd(&geps[n], (double)wrow[k] * (double)(-dz_T[n] * ie * ie));
}

dim3 grid2(int nx, int ny, dim3 blk) { return dim3((ny + blk.x - 1) / blk.x, (nx + blk.y - 1) / blk.y, 1); }

template <typename R>
TMArgs<R> tm_args(cev_fdtd_plan p, const cev_fdtd_state* st, const R* jz) {
  TMArgs<R> a;
  a.nx = p->nx;
  a.ny = p->ny;
  a.hx = (R*)st->hx; a.hy = (R*)st->hy; a.dz = (R*)st->dz;
  a.icex = (R*)st->icex; a.icey = (R*)st->icey; a.idz = (R*)st->idz;
  a.iez = (const R*)p->iez;
  a.ax = (const AxisCoef<R>*)p->ax;
  a.ay = (const AxisCoef<R>*)p->ay;
  a.S = (R)p->S;
  a.jz = jz;
  return a;
}

template <typename R>
int step_impl(cev_fdtd_plan p, const cev_fdtd_state* st, const R* jx, const R* jy, const R* jz,
              int te, cudaStream_t s) {
  const dim3 blk(32, 8);
  const dim3 g = grid2(p->nx, p->ny, blk);
  TMArgs<R> a = tm_args<R>(p, st, jz);
  k_tm_h<R><<<g, blk, 0, s>>>(a);
  if (te) {
    TEArgs<R> e;
    e.nx = p->nx; e.ny = p->ny;
    e.hz = (R*)st->hz; e.dx = (R*)st->dx; e.dy = (R*)st->dy;
    e.ihz = (R*)st->ihz; e.ichx = (R*)st->ichx; e.ichy = (R*)st->ichy;
    e.iexx = (const R*)p->iexx; e.ieyy = (const R*)p->ieyy;
    e.ax = a.ax; e.ay = a.ay; e.S = a.S; e.jx = jx; e.jy = jy;
    k_te_h<R><<<g, blk, 0, s>>>(e);
    k_te_d<R><<<g, blk, 0, s>>>(e);
  }
  k_tm_d<R><<<g, blk, 0, s>>>(a);
  CEV_CHECK_LAUNCH("fdtd step");
  return CEV_OK;
}


template <typename R>
int step_adjoint_impl(cev_fdtd_plan p, const R* dz_in, const R* dz_out, const R* gez,
                      const cev_fdtd_state* adj, R* scratch, double* geps, cudaStream_t s) {
  const size_t N = p->n();
  AdjArgs<R> a;
  a.nx = p->nx; a.ny = p->ny;
  a.ahx = (R*)adj->hx; a.ahy = (R*)adj->hy; a.adz = (R*)adj->dz;
  a.aicex = (R*)adj->icex; a.aicey = (R*)adj->icey; a.aidz = (R*)adj->idz;
  a.ach = scratch; a.adey = scratch + N; a.adex = scratch + 2 * N; a.adzp = scratch + 3 * N;
  a.iez = (const R*)p->iez;
  a.ax = (const AxisCoef<R>*)p->ax;
  a.ay = (const AxisCoef<R>*)p->ay;
  a.S = (R)p->S;
  if (gez) {
    const unsigned g1 = std::max(1u, std::min(ceil_div(N, 256), 8u * sm_count()));
    k_adj_out_ez<R><<<g1, 256, 0, s>>>((int)N, a.adz, gez, dz_out, a.iez, geps);
  }
  const dim3 blk(32, 8);
  const dim3 g = grid2(p->nx, p->ny, blk);
  k_adj_a<R><<<g, blk, 0, s>>>(a);
  k_adj_b<R><<<g, blk, 0, s>>>(a);
  k_adj_c<R><<<g, blk, 0, s>>>(a, dz_in, geps, 0, nullptr, nullptr);
  CEV_CHECK_LAUNCH("fdtd step adjoint");
  return CEV_OK;
}

// Tile shape of the Dz-history runner (adjoint recompute): 32x48 tiles, 512
// threads -- one extra kernel instantiation per precision.
constexpr int HIST_CFG = 2;

template <typename R>
static int hist_launch(bool prepare, dim3 g, const TBArgs<R>& a, cudaStream_t s) {
  constexpr TileCfg c = TILE_CFGS[HIST_CFG];
  using T = Tile<R, c.ti, c.tj, c.k, c.nt>;
  if (prepare)
    return allow_dynamic_smem((const void*)k_tm_tile<R, c.ti, c.tj, c.k, c.nt, true>, (int)T::smem);
  k_tm_tile<R, c.ti, c.tj, c.k, c.nt, true><<<g, c.nt, T::smem, s>>>(a);
  return CEV_OK;
}

// ------------------------------------------------ persistent TM runner
// Tile shapes of the single-launch runner: every tile's CTA must be resident
// at once (cooperative launch), so the runner serves grids whose tile count
// fits the GPU (about 600 x 600 cells); larger grids take the launch-per-K
// path, where launch overhead is a small share.
constexpr TileCfg PERSIST_CFGS[] = {{34, 34, 8, 512}, {42, 42, 8, 512}, {50, 50, 8, 512},
                                    {34, 34, 4, 512}};
constexpr int N_PERSIST_CFGS = sizeof(PERSIST_CFGS) / sizeof(PERSIST_CFGS[0]);

template <typename R, int I>
struct PersistLauncher {
  static constexpr TileCfg c = PERSIST_CFGS[I];
  using T = Tile<R, c.ti, c.tj, c.k, c.nt>;
  static const void* fn() { return (const void*)k_tm_tile<R, c.ti, c.tj, c.k, c.nt, false, true>; }
  static int capacity() {
    if (T::smem > 227 * 1024 || allow_dynamic_smem(fn(), (int)T::smem) != CEV_OK) {
      cudaGetLastError();
      return 0;
    }
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_tm_tile<R, c.ti, c.tj, c.k, c.nt, false, true>,
                                                      c.nt, T::smem) != cudaSuccess) {
      cudaGetLastError();
      return 0;
    }
    return n * sm_count();
  }
  static int launch(dim3 g, TBArgs<R>& a, cudaStream_t s) {
    void* args[] = {&a};
    CEV_CUDA(cudaLaunchCooperativeKernel(fn(), g, dim3(c.nt), args, T::smem, s));
    return CEV_OK;
  }
};

template <typename R, int I = 0>
static int persist_capacity(int cfg) {
  if constexpr (I < N_PERSIST_CFGS) {
    return cfg == I ? PersistLauncher<R, I>::capacity() : persist_capacity<R, I + 1>(cfg);
  } else {
    return 0;
  }
}

template <typename R, int I = 0>
static int persist_launch(int cfg, dim3 g, TBArgs<R>& a, cudaStream_t s) {
  if constexpr (I < N_PERSIST_CFGS) {
    return cfg == I ? PersistLauncher<R, I>::launch(g, a, s) : persist_launch<R, I + 1>(cfg, g, a, s);
  } else {
    set_error("bad persistent tile configuration %d", cfg);
    return CEV_ERR_INVALID;
  }
}

// Symmetric neighbour lists of the tile grid: tile T exchanges with every
// tile owning a cell of T's region (the tile rows its region rows fall in
// times the tile columns its region columns fall in), and each of those with
// T.  Returns false when some tile has more than NBR_MAX neighbours.
static bool persist_neighbours(int nx, int ny, const TileCfg& c, std::vector<int>& out) {
  const int gy = (nx + c.ti - 1) / c.ti, gx = (ny + c.tj - 1) / c.tj, tiles = gx * gy;
  const int RI = c.ti + 2 * c.k, RJ = c.tj + 2 * c.k;
  std::vector<std::vector<int>> nb(tiles);
  auto add = [&](int a, int b) {
    if (std::find(nb[a].begin(), nb[a].end(), b) == nb[a].end()) nb[a].push_back(b);
  };
  auto touched = [](int g0, int len, int n, int t, std::vector<int>& v) {
    v.clear();
    for (int r = 0; r < len; ++r) {
      const int q = (((g0 + r) % n + n) % n) / t;
      if (std::find(v.begin(), v.end(), q) == v.end()) v.push_back(q);
    }
  };
  std::vector<int> rows, cols;
  for (int ty = 0; ty < gy; ++ty)
    for (int tx = 0; tx < gx; ++tx) {
      const int t = ty * gx + tx;
      touched(ty * c.ti - c.k, RI, nx, c.ti, rows);
      touched(tx * c.tj - c.k, RJ, ny, c.tj, cols);
      for (int r : rows)
        for (int q : cols) {
          const int o = r * gx + q;
          if (o == t) continue;
          add(t, o);
          add(o, t);
        }
    }
  out.assign((size_t)tiles * NBR_MAX, -1);
  for (int t = 0; t < tiles; ++t) {
    if ((int)nb[t].size() > NBR_MAX) return false;
    for (size_t k = 0; k < nb[t].size(); ++k) out[(size_t)t * NBR_MAX + k] = nb[t][k];
  }
  return true;
}

// Persistent configuration for this grid, or -1.  CEV_FDTD_PERSIST=0 turns
// the runner off; CEV_FDTD_PERSIST=<i+1> forces configuration i.
template <typename R>
static int pick_persist(int nx, int ny) {
  const char* e = std::getenv("CEV_FDTD_PERSIST");
  int forced = -1;
  if (std::getenv("CEV_FDTD_TILE") && !e) return -1;  // a forced launch-per-K tile shape
  if (e) {
    if (e[0] == '0') return -1;
    forced = std::atoi(e) - 1;
  }
  for (int v = 0; v < N_PERSIST_CFGS; ++v) {
    if (forced >= 0 && v != forced) continue;
    const TileCfg c = PERSIST_CFGS[v];
    if (forced < 0 && c.k != 8) continue;  // K = 8 by default; K = 4 on request
    if (nx < c.ti + 2 * c.k || ny < c.tj + 2 * c.k) continue;
    const int tiles = ((nx + c.ti - 1) / c.ti) * ((ny + c.tj - 1) / c.tj);
    if (tiles <= persist_capacity<R>(v)) return v;
  }
  return -1;
}

// Register-strip configurations (warps, rows per thread, K); float32 only.
struct StripCfg {
  int w, s, k;
};
constexpr StripCfg STRIP_CFGS[] = {{16, 3, 8}, {16, 2, 4}, {16, 3, 4}, {32, 2, 8},
                                   {14, 3, 8}, {21, 2, 8}};
constexpr int N_STRIP_CFGS = sizeof(STRIP_CFGS) / sizeof(STRIP_CFGS[0]);

static TileCfg strip_tile(const StripCfg& c) {
  return TileCfg{c.w * c.s - 2 * c.k, 64 - 2 * c.k, c.k, 32 * c.w};
}

template <int I, bool P>
struct StripLauncher {
  static constexpr StripCfg c = STRIP_CFGS[I];
  using G = Strip<c.w, c.s, c.k>;
  static const void* fn() { return (const void*)k_tm_strip<float, c.w, c.s, c.k, P>; }
  static int capacity(int np) {
    const size_t smem = G::template smem<float>(np);
    if (smem > 227 * 1024 || allow_dynamic_smem(fn(), (int)smem) != CEV_OK) {
      cudaGetLastError();
      return 0;
    }
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_tm_strip<float, c.w, c.s, c.k, P>, G::NT,
                                                      smem) != cudaSuccess) {
      cudaGetLastError();
      return 0;
    }
    return n * sm_count();
  }
  static int launch(dim3 g, TBArgs<float>& a, int np, cudaStream_t s) {
    const size_t smem = G::template smem<float>(np);
    int rc = allow_dynamic_smem(fn(), (int)smem);
    if (rc != CEV_OK) return rc;
    if (P) {
      void* args[] = {&a};
      CEV_CUDA(cudaLaunchCooperativeKernel(fn(), g, dim3(G::NT), args, smem, s));
    } else {
      k_tm_strip<float, c.w, c.s, c.k, P><<<g, G::NT, smem, s>>>(a);
      CEV_CHECK_LAUNCH("k_tm_strip");
    }
    return CEV_OK;
  }
};

template <int I = 0>
static int strip_capacity(int cfg, int np) {
  if constexpr (I < N_STRIP_CFGS) {
    return cfg == I ? StripLauncher<I, true>::capacity(np) : strip_capacity<I + 1>(cfg, np);
  } else {
    return 0;
  }
}

template <int I = 0>
static int strip_launch(int cfg, bool persist, dim3 g, TBArgs<float>& a, int np, cudaStream_t s) {
  if constexpr (I < N_STRIP_CFGS) {
    if (cfg == I)
      return persist ? StripLauncher<I, true>::launch(g, a, np, s)
                     : StripLauncher<I, false>::launch(g, a, np, s);
    return strip_launch<I + 1>(cfg, persist, g, a, np, s);
  } else {
    set_error("bad strip configuration %d", cfg);
    return CEV_ERR_INVALID;
  }
}

// Register-strip configuration of the single-launch runner for this grid, or
// -1.  CEV_FDTD_STRIP=0 turns it off, CEV_FDTD_STRIP=<i+1> forces
// configuration i; a forced tile (CEV_FDTD_TILE) or persistent-tile
// (CEV_FDTD_PERSIST) choice also turns it off.
template <typename R>
static int pick_strip(int nx, int ny, int np) {
  if (sizeof(R) != sizeof(float)) return -1;
  const char* e = std::getenv("CEV_FDTD_STRIP");
  int forced = -1;
  if (!e && (std::getenv("CEV_FDTD_TILE") || std::getenv("CEV_FDTD_PERSIST"))) return -1;
  if (e) {
    if (e[0] == '0') return -1;
    forced = std::atoi(e) - 1;
  }
  if (np > STRIP_PROBE_MAX) return -1;
  // by default (14, 3, 8), then (16, 3, 8): the smaller tile spreads a grid
  // over more SMs (400 x 400: 144 tiles of 26 x 48 instead of 117 of 32 x 48)
  const int order[] = {4, 0};
  const int n_try = forced >= 0 ? 1 : 2;
  for (int i = 0; i < n_try; ++i) {
    const int v = forced >= 0 ? forced : order[i];
    if (v < 0 || v >= N_STRIP_CFGS) return -1;
    const TileCfg c = strip_tile(STRIP_CFGS[v]);
    if (nx < c.ti + 2 * c.k || ny < c.tj + 2 * c.k) continue;
    const int tiles = ((nx + c.ti - 1) / c.ti) * ((ny + c.tj - 1) / c.tj);
    if (tiles <= strip_capacity(v, np)) return v;
  }
  return -1;
}

template <typename R>
int run_tm_impl(cev_fdtd_plan p, const cev_fdtd_state* st, int nsteps, const cev_fdtd_io* io,
                cudaStream_t s, R* dz_hist = nullptr) {
  const size_t N = p->n();
  const int ns = io ? io->n_src : 0, np = io ? io->n_probe : 0;
  int cfg = pick_tile<R>(p->nx, p->ny);
  if (dz_hist) {  // Dz after every step: the history kernel's tile shape, if it fits
    const TileCfg h = TILE_CFGS[HIST_CFG];
    cfg = (p->nx >= h.ti + 2 * h.k && p->ny >= h.tj + 2 * h.k) ? HIST_CFG : -1;
  }
  if (cfg < 0) {
    // grids smaller than one tile region: per-step kernels
    for (int t = 0; t < nsteps; ++t) {
      int rc = step_impl<R>(p, st, nullptr, nullptr, nullptr, 0, s);
      if (rc != CEV_OK) return rc;
      if (ns > 0)
        k_add_src<R><<<(ns + 127) / 128, 128, 0, s>>>((R*)st->dz, ns, io->src_idx,
                                                       (const R*)io->src_w, (const R*)io->amps, t);
      if (np > 0)
        k_probe<R><<<(np + 127) / 128, 128, 0, s>>>((const R*)st->dz, (const R*)p->iez, np,
                                                     io->probe_idx, (R*)io->probe_out + (size_t)t * np);
      if (dz_hist)
        CEV_CUDA(cudaMemcpyAsync(dz_hist + (size_t)(t + 1) * N, st->dz, N * sizeof(R),
                                 cudaMemcpyDeviceToDevice, s));
    }
    CEV_CHECK_LAUNCH("fdtd run (per step)");
    return CEV_OK;
  }
  if (!p->shadow) {
    CEV_REQUIRE(!p->borrowed, "borrowed FDTD plan without a shadow state");
    int rc = dev_alloc(&p->shadow, 6 * N * sizeof(R), s);
    if (rc != CEV_OK) return rc;
  }
  R* sh = (R*)p->shadow;
  R* bufA[6] = {(R*)st->hx, (R*)st->hy, (R*)st->dz, (R*)st->icex, (R*)st->icey, (R*)st->idz};
  R* bufB[6] = {sh, sh + N, sh + 2 * N, sh + 3 * N, sh + 4 * N, sh + 5 * N};
  // the shadow's PML integrals must match the state outside tiles that skip them
  CEV_CUDA(cudaMemcpyAsync(bufB[3], bufA[3], N * sizeof(R), cudaMemcpyDeviceToDevice, s));
  CEV_CUDA(cudaMemcpyAsync(bufB[4], bufA[4], N * sizeof(R), cudaMemcpyDeviceToDevice, s));
  CEV_CUDA(cudaMemcpyAsync(bufB[5], bufA[5], N * sizeof(R), cudaMemcpyDeviceToDevice, s));
  // single launch for grids whose tiles all fit on the GPU at once: the
  // register-strip kernel (float32), else the persistent tile kernel
  int pc = -1, key = -1;
  TileCfg c{};
  if (!dz_hist && !p->borrowed) {
    const int si = pick_strip<R>(p->nx, p->ny, np);
    if (si >= 0) {
      pc = si;
      key = 100 + si;
      c = strip_tile(STRIP_CFGS[si]);
    } else if ((pc = pick_persist<R>(p->nx, p->ny)) >= 0) {
      key = pc;
      c = PERSIST_CFGS[pc];
    }
  }
  if (pc >= 0 && nsteps > c.k) {
    const int gy = (p->nx + c.ti - 1) / c.ti, gx = (p->ny + c.tj - 1) / c.tj;
    if (p->pcfg != key) {
      std::vector<int> nbr;
      if (persist_neighbours(p->nx, p->ny, c, nbr)) {
        dev_free_all({p->pnbr, p->pflags});
        p->pnbr = nullptr;
        p->pflags = nullptr;
        p->pcfg = -1;
        int rc = dev_alloc((void**)&p->pnbr, sizeof(int) * nbr.size(), s);
        if (rc == CEV_OK)
          rc = dev_alloc((void**)&p->pflags, sizeof(int) * FLAG_STRIDE * (gx * gy + 1), s);
        if (rc != CEV_OK) return rc;
        // pageable source: the copy is staged before the call returns
        CEV_CUDA(cudaMemcpyAsync(p->pnbr, nbr.data(), sizeof(int) * nbr.size(),
                                 cudaMemcpyHostToDevice, s));
        p->pcfg = key;
        p->ptiles = gx * gy;
      }
    }
    if (p->pcfg == key) {
      TBArgs<R> a{};
      a.nx = p->nx; a.ny = p->ny; a.K = c.k; a.t0 = 0;
      a.hx_i = bufA[0]; a.hy_i = bufA[1]; a.dz_i = bufA[2];
      a.icex_i = bufA[3]; a.icey_i = bufA[4]; a.idz_i = bufA[5];
      a.iez = (const R*)p->iez;
      a.ax = (const AxisCoef<R>*)p->ax;
      a.ay = (const AxisCoef<R>*)p->ay;
      a.S = (R)p->S;
      a.ns = ns;
      a.src_idx = ns ? io->src_idx : nullptr;
      a.src_w = ns ? (const R*)io->src_w : nullptr;
      a.amps = ns ? (const R*)io->amps : nullptr;
      a.np = np;
      a.probe_idx = np ? io->probe_idx : nullptr;
      a.probe_out = np ? (R*)io->probe_out : nullptr;
      a.nsteps = nsteps;
      for (int f = 0; f < 6; ++f) {
        a.xb[0][f] = bufB[f];
        a.xb[1][f] = bufA[f];
      }
      a.flags = p->pflags;
      a.fault = p->pflags + (size_t)p->ptiles * FLAG_STRIDE;
      a.nbr = p->pnbr;
      CEV_CUDA(cudaMemsetAsync(p->pflags, 0, sizeof(int) * FLAG_STRIDE * (p->ptiles + 1), s));
      int rc;
      if (key >= 100) {
        if constexpr (sizeof(R) == sizeof(float))
          rc = strip_launch(pc, true, dim3(gx, gy, 1), a, np, s);
        else
          rc = CEV_ERR_INVALID;
      } else {
        rc = persist_launch<R>(pc, dim3(gx, gy, 1), a, s);
      }
      if (rc != CEV_OK) return rc;
      const int nblk = (nsteps + c.k - 1) / c.k;
      if (((nblk - 1) & 1) == 0)  // the last block went to the shadow buffer
        for (int f = 0; f < 6; ++f)
          CEV_CUDA(cudaMemcpyAsync(bufA[f], bufB[f], N * sizeof(R), cudaMemcpyDeviceToDevice, s));
      int fault = 0;
      CEV_CUDA(cudaMemcpyAsync(&fault, a.fault, sizeof(int), cudaMemcpyDeviceToHost, s));
      CEV_CUDA(cudaStreamSynchronize(s));
      if (fault) {
        set_error("persistent FDTD runner: a tile's neighbour wait ran out (exchange fault)");
        return CEV_ERR_CUDA;
      }
      return CEV_OK;
    }
  }
  TBArgs<R> a{};
  {
    // per device and kernel, thread-safe (allow_dynamic_smem)
    int rc = dz_hist ? hist_launch<R>(true, dim3(), a, s) : tile_dispatch<R>(cfg, true, dim3(), a, s);
    if (rc != CEV_OK) return rc;
  }
  const TileCfg tc = TILE_CFGS[cfg];
  const int K = tc.k;
  const dim3 g((p->ny + tc.tj - 1) / tc.tj, (p->nx + tc.ti - 1) / tc.ti, 1);
  R** in = bufA;
  R** out = bufB;
  int t = 0;
  while (t < nsteps) {
    const int k = std::min(K, nsteps - t);
    a.nx = p->nx; a.ny = p->ny; a.K = k; a.t0 = t;
    a.hx_i = in[0]; a.hy_i = in[1]; a.dz_i = in[2]; a.icex_i = in[3]; a.icey_i = in[4]; a.idz_i = in[5];
    a.hx_o = out[0]; a.hy_o = out[1]; a.dz_o = out[2]; a.icex_o = out[3]; a.icey_o = out[4]; a.idz_o = out[5];
    a.iez = (const R*)p->iez;
    a.ax = (const AxisCoef<R>*)p->ax;
    a.ay = (const AxisCoef<R>*)p->ay;
    a.S = (R)p->S;
    a.ns = ns;
    a.src_idx = ns ? io->src_idx : nullptr;
    a.src_w = ns ? (const R*)io->src_w : nullptr;
    a.amps = ns ? (const R*)io->amps : nullptr;
    a.np = np;
    a.probe_idx = np ? io->probe_idx : nullptr;
    a.probe_out = np ? (R*)io->probe_out : nullptr;
    a.dz_hist = dz_hist;
    if (dz_hist)
      hist_launch<R>(false, g, a, s);
    else
      tile_dispatch<R>(cfg, false, g, a, s);
    CEV_CHECK_LAUNCH("k_tm_tile");
    std::swap(in, out);
    t += k;
  }
  if (in != bufA)
    for (int f = 0; f < 6; ++f)
      CEV_CUDA(cudaMemcpyAsync(bufA[f], in[f], N * sizeof(R), cudaMemcpyDeviceToDevice, s));
  return CEV_OK;
}

// ------------------------------------------------------ time-blocked TE
// The TE recurrence of k_te_h / k_te_d (ceviche/fdtd.py:79-137 with
// Nz = 1: Hz from the curl of (Ex, Ey), then Dx, Dy from the curl of Hz, with
// the Jx, Jy sources added to Dx, Dy) advanced K steps per launch on a
// (TI + 2K) x (TJ + 2K) region in shared memory, as k_tm_tile does for TM:
// the H phase needs E at i+1, j+1 and the D phase H at i-1, j-1, so the
// interior is exact after K steps.  Sources: Jx(t) = wx * amps[t],
// Jy(t) = wy * amps[t] at sparse cells; probes record Hz after each step.
template <typename R>
struct TEBArgs {
  int nx, ny, K, t0;
  const R* hz_i; const R* dx_i; const R* dy_i; const R* ih_i; const R* icx_i; const R* icy_i;
  R* hz_o; R* dx_o; R* dy_o; R* ih_o; R* icx_o; R* icy_o;
  const R* iexx;
  const R* ieyy;
  const AxisCoef<R>* ax;
  const AxisCoef<R>* ay;
  R S;
  int ns;
  const int* src_idx;
  const R* src_wx;
  const R* src_wy;
  const R* amps;
  int np;
  const int* probe_idx;
  R* probe_out;  // [t][np]
};

// a * b rounded on its own (no contraction into a following add)
__device__ __forceinline__ float mul_rn(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double mul_rn(double a, double b) { return __dmul_rn(a, b); }

template <typename R, int TI, int TJ, int K, int NT>
struct TeTile {
  static constexpr int RI = TI + 2 * K, RJ = TJ + 2 * K, RN = RI * RJ;
  static constexpr int CPT = (RN + NT - 1) / NT;
  // sEx, sEy, sHz, sWx, sWy [RN]; x tables aH, pH, aD, f1D, f2D [RI]; y the same [RJ]; amps [K]
  static constexpr size_t smem =
      5 * (size_t)RN * sizeof(R) + 5 * (size_t)(RI + RJ) * sizeof(R) + (size_t)K * sizeof(R);
};

template <typename R, int TI, int TJ, int K, int NT>
__global__ void __launch_bounds__(NT, 1) k_te_tile(TEBArgs<R> a) {
  using T = TeTile<R, TI, TJ, K, NT>;
  constexpr int RI = T::RI, RJ = T::RJ, RN = T::RN, CPT = T::CPT;
  extern __shared__ __align__(16) unsigned char smraw[];
  R* sEx = (R*)smraw;
  R* sEy = sEx + RN;
  R* sHz = sEy + RN;
  R* sWx = sHz + RN;
  R* sWy = sWx + RN;
  R* xaH = sWy + RN;
  R* xpH = xaH + RI;
  R* xaD = xpH + RI;
  R* xf1 = xaD + RI;
  R* xf2 = xf1 + RI;
  R* yaH = xf2 + RI;
  R* ypH = yaH + RJ;
  R* yaD = ypH + RJ;
  R* yf1 = yaD + RJ;
  R* yf2 = yf1 + RJ;
  R* sAmp = yf2 + RJ;
  const int nst = a.K;
  const int gi0 = blockIdx.y * TI - K, gj0 = blockIdx.x * TJ - K;
  const int tid = threadIdx.x;
  auto gi = [&](int r) { int v = (gi0 + r) % a.nx; return v < 0 ? v + a.nx : v; };
  auto gj = [&](int c) { int v = (gj0 + c) % a.ny; return v < 0 ? v + a.ny : v; };
  int pl = 0;
  for (int r = tid; r < RI; r += NT) {
    const AxisCoef<R> c = a.ax[gi(r)];
    xaH[r] = c.aH; xpH[r] = c.pH; xaD[r] = c.aD; xf1[r] = c.f1D; xf2[r] = c.f2D;
    pl |= (c.aH != R(0)) | (c.aD != R(0));
  }
  for (int q = tid; q < RJ; q += NT) {
    const AxisCoef<R> c = a.ay[gj(q)];
    yaH[q] = c.aH; ypH[q] = c.pH; yaD[q] = c.aD; yf1[q] = c.f1D; yf2[q] = c.f2D;
    pl |= (c.aH != R(0)) | (c.aD != R(0));
  }
  for (int st = tid; st < nst; st += NT) sAmp[st] = a.ns > 0 ? a.amps[a.t0 + st] : R(0);
  for (int q = tid; q < RN; q += NT) {
    sWx[q] = R(0);
    sWy[q] = R(0);
  }
  const bool pml = __syncthreads_or(pl);
  for (int k = tid; k < a.ns; k += NT) {
    const int n = a.src_idx[k];
    const int ii = n / a.ny, jj = n - ii * a.ny;
    int r = (ii - gi0) % a.nx;
    if (r < 0) r += a.nx;
    int c = (jj - gj0) % a.ny;
    if (c < 0) c += a.ny;
    if (r < RI && c < RJ) {
      atomicAdd(&sWx[r * RJ + c], a.src_wx[k]);
      atomicAdd(&sWy[r * RJ + c], a.src_wy[k]);
    }
  }
  __syncthreads();
  R hz[CPT], dx[CPT], dy[CPT], iex[CPT], iey[CPT], ih[CPT], icx[CPT], icy[CPT];
  unsigned srcmask = 0;
#pragma unroll
  for (int k = 0; k < CPT; ++k) {
    const int q = tid + k * NT;
    hz[k] = dx[k] = dy[k] = iex[k] = iey[k] = ih[k] = icx[k] = icy[k] = R(0);
    if (q < RN) {
      const int r = q / RJ, c = q - r * RJ;
      const size_t n = (size_t)gi(r) * a.ny + gj(c);
      hz[k] = a.hz_i[n];
      dx[k] = a.dx_i[n];
      dy[k] = a.dy_i[n];
      iex[k] = a.iexx[n];
      iey[k] = a.ieyy[n];
      if (pml) {
        ih[k] = a.ih_i[n];
        icx[k] = a.icx_i[n];
        icy[k] = a.icy_i[n];
      }
      if (sWx[q] != R(0) || sWy[q] != R(0)) srcmask |= 1u << k;
      sEx[q] = dx[k] * iex[k];
      sEy[q] = dy[k] * iey[k];
    }
  }
  __syncthreads();
  const R S = a.S;
  for (int st = 0; st < nst; ++st) {
    const R amp = sAmp[st];
    // ---- H phase: Hz from the curl of (Ex, Ey)
#pragma unroll
    for (int k = 0; k < CPT; ++k) {
      const int q = tid + k * NT;
      if (q < RN) {
        const int r = q / RJ, c = q - r * RJ;
        const R ex = sEx[q], ey = sEy[q];
        const R exr = (c < RJ - 1) ? sEx[q + 1] : ex;
        const R eyd = (r < RI - 1) ? sEy[q + RJ] : ey;
        const R ce = (eyd - ey) - (exr - ex);
        if (!pml) {
          hz[k] = fma(-S, ce, hz[k]);
        } else {
          const R ax = xaH[r], ay = yaH[c];
          const R ph = xpH[r] * ypH[c];
          const R m1 = fma(-ax, ay, (R(1) - ax) - ay) * ph;
          const R m2 = -S * ph;
          const R m4 = R(-4) * ax * ay * ph;
          R v = R(0);
          if (m4 != R(0)) { ih[k] += hz[k]; v = ih[k]; }
          hz[k] = fma(m4, v, fma(m2, ce, m1 * hz[k]));  // as k_te_h
        }
        sHz[q] = hz[k];
      }
    }
    __syncthreads();
    // ---- D phase: Dx, Dy from the curl of Hz, plus the sources
#pragma unroll
    for (int k = 0; k < CPT; ++k) {
      const int q = tid + k * NT;
      if (q < RN) {
        const int r = q / RJ, c = q - r * RJ;
        const R hzl = (c > 0) ? sHz[q - 1] : hz[k];
        const R hzu = (r > 0) ? sHz[q - RJ] : hz[k];
        const R chx = hz[k] - hzl;
        const R chy = -(hz[k] - hzu);
        R vx, vy;
        if (!pml) {
          vx = fma(S, chx, dx[k]);
          vy = fma(S, chy, dy[k]);
        } else {
          const R ax = xaD[r], ay = yaD[c];
          R wx = R(0), wy = R(0);
          if (ax != R(0)) { icx[k] += chx; wx = icx[k]; }
          if (ay != R(0)) { icy[k] += chy; wy = icy[k]; }
          vx = fma(yf2[c], fma(R(2) * ax, wx, chx), yf1[c] * dx[k]);  // as k_te_d
          vy = fma(xf2[r], fma(R(2) * ay, wy, chy), xf1[r] * dy[k]);
        }
        if (srcmask & (1u << k)) {  // the product rounded, then added, as a dense J
          vx += mul_rn(sWx[q], amp);
          vy += mul_rn(sWy[q], amp);
        }
        dx[k] = vx;
        dy[k] = vy;
        sEx[q] = vx * iex[k];
        sEy[q] = vy * iey[k];
      }
    }
    __syncthreads();
    for (int k = tid; k < a.np; k += NT) {
      const int n = a.probe_idx[k];
      const int ii = n / a.ny, jj = n - ii * a.ny;
      const int r = ii - gi0, c = jj - gj0;
      if (r >= K && r < K + TI && c >= K && c < K + TJ)
        a.probe_out[(size_t)(a.t0 + st) * a.np + k] = sHz[r * RJ + c];
    }
    // the next H phase writes sHz: every probe read must be done first
    if (a.np > 0) __syncthreads();
  }
#pragma unroll
  for (int k = 0; k < CPT; ++k) {
    const int q = tid + k * NT;
    if (q < RN) {
      const int r = q / RJ, c = q - r * RJ;
      const int ii = gi0 + r, jj = gj0 + c;
      if (r >= K && r < K + TI && c >= K && c < K + TJ && ii < a.nx && jj < a.ny) {
        const size_t n = (size_t)ii * a.ny + jj;
        a.hz_o[n] = hz[k];
        a.dx_o[n] = dx[k];
        a.dy_o[n] = dy[k];
        if (pml) {
          a.ih_o[n] = ih[k];
          a.icx_o[n] = icx[k];
          a.icy_o[n] = icy[k];
        }
      }
    }
  }
}

// per-step TE extras of the fallback: sparse Jx/Jy sources and Hz probes
template <typename R>
__global__ void k_add_src_te(R* dx, R* dy, int ns, const int* idx, const R* wx, const R* wy,
                             const R* amps, int t) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= ns) return;
  dx[idx[k]] += wx[k] * amps[t];
  dy[idx[k]] += wy[k] * amps[t];
}

template <typename R>
__global__ void k_probe_hz(const R* hz, int np, const int* idx, R* out) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < np) out[k] = hz[idx[k]];
}

// TE tile shape: 32 x 48 interior, K = 8, 512 threads (the TM choice at 400^2)
constexpr int TE_TI = 32, TE_TJ = 48, TE_K = 8, TE_NT = 512;

template <typename R>
int run_te_impl(cev_fdtd_plan p, const cev_fdtd_state* st, int nsteps, const cev_fdtd_io_te* io,
                cudaStream_t s) {
  const size_t N = p->n();
  const int ns = io ? io->n_src : 0, np = io ? io->n_probe : 0;
  if (p->nx < TE_TI + 2 * TE_K || p->ny < TE_TJ + 2 * TE_K) {
    // grids smaller than one tile region: per-step kernels
    for (int t = 0; t < nsteps; ++t) {
      int rc = step_impl<R>(p, st, nullptr, nullptr, nullptr, 1, s);
      if (rc != CEV_OK) return rc;
      if (ns > 0)
        k_add_src_te<R><<<(ns + 127) / 128, 128, 0, s>>>(
            (R*)st->dx, (R*)st->dy, ns, io->src_idx, (const R*)io->src_wx, (const R*)io->src_wy,
            (const R*)io->amps, t);
      if (np > 0)
        k_probe_hz<R><<<(np + 127) / 128, 128, 0, s>>>((const R*)st->hz, np, io->probe_idx,
                                                        (R*)io->probe_out + (size_t)t * np);
    }
    CEV_CHECK_LAUNCH("fdtd run te (per step)");
    return CEV_OK;
  }
  if (!p->shadow) {
    CEV_REQUIRE(!p->borrowed, "borrowed FDTD plan without a shadow state");
    int rc = dev_alloc(&p->shadow, 6 * N * sizeof(R), s);
    if (rc != CEV_OK) return rc;
  }
  R* sh = (R*)p->shadow;
  R* bufA[6] = {(R*)st->hz, (R*)st->dx, (R*)st->dy, (R*)st->ihz, (R*)st->ichx, (R*)st->ichy};
  R* bufB[6] = {sh, sh + N, sh + 2 * N, sh + 3 * N, sh + 4 * N, sh + 5 * N};
  // the shadow's PML integrals must match the state outside tiles that skip them
  for (int f = 3; f < 6; ++f)
    CEV_CUDA(cudaMemcpyAsync(bufB[f], bufA[f], N * sizeof(R), cudaMemcpyDeviceToDevice, s));
  using T = TeTile<R, TE_TI, TE_TJ, TE_K, TE_NT>;
  int rc = allow_dynamic_smem((const void*)k_te_tile<R, TE_TI, TE_TJ, TE_K, TE_NT>, (int)T::smem);
  if (rc != CEV_OK) return rc;
  const dim3 g((p->ny + TE_TJ - 1) / TE_TJ, (p->nx + TE_TI - 1) / TE_TI, 1);
  R** in = bufA;
  R** out = bufB;
  TEBArgs<R> a{};
  for (int t = 0; t < nsteps; t += TE_K) {
    a.nx = p->nx; a.ny = p->ny; a.K = std::min(TE_K, nsteps - t); a.t0 = t;
    a.hz_i = in[0]; a.dx_i = in[1]; a.dy_i = in[2]; a.ih_i = in[3]; a.icx_i = in[4]; a.icy_i = in[5];
    a.hz_o = out[0]; a.dx_o = out[1]; a.dy_o = out[2]; a.ih_o = out[3]; a.icx_o = out[4]; a.icy_o = out[5];
    a.iexx = (const R*)p->iexx;
    a.ieyy = (const R*)p->ieyy;
    a.ax = (const AxisCoef<R>*)p->ax;
    a.ay = (const AxisCoef<R>*)p->ay;
    a.S = (R)p->S;
    a.ns = ns;
    a.src_idx = ns ? io->src_idx : nullptr;
    a.src_wx = ns ? (const R*)io->src_wx : nullptr;
    a.src_wy = ns ? (const R*)io->src_wy : nullptr;
    a.amps = ns ? (const R*)io->amps : nullptr;
    a.np = np;
    a.probe_idx = np ? io->probe_idx : nullptr;
    a.probe_out = np ? (R*)io->probe_out : nullptr;
    k_te_tile<R, TE_TI, TE_TJ, TE_K, TE_NT><<<g, TE_NT, T::smem, s>>>(a);
    CEV_CHECK_LAUNCH("k_te_tile");
    std::swap(in, out);
  }
  if (in != bufA)
    for (int f = 0; f < 6; ++f)
      CEV_CUDA(cudaMemcpyAsync(bufA[f], in[f], N * sizeof(R), cudaMemcpyDeviceToDevice, s));
  return CEV_OK;
}

template <typename R>
int adjoint_impl(cev_fdtd_plan p, int T, int C, const cev_fdtd_io* io, const R* w, double* geps,
                 void* ws, cudaStream_t s) {
  const size_t N = p->n();
  const int nck = (T + C - 1) / C + 1;
  R* base = (R*)ws;
  R* cur[6];
  for (int f = 0; f < 6; ++f) cur[f] = base + f * N;
  R* ck = base + 6 * N;                    // nck checkpoints of 6 fields
  R* seg = ck + (size_t)nck * 6 * N;       // (C+1) Dz snapshots
  R* adj = seg + (size_t)(C + 1) * N;      // 10 adjoint arrays
  const int ns = io->n_src, np = io->n_probe;
  cev_fdtd_state st{};
  st.hx = cur[0]; st.hy = cur[1]; st.dz = cur[2]; st.icex = cur[3]; st.icey = cur[4]; st.idz = cur[5];
  CEV_CUDA(cudaMemsetAsync(base, 0, 6 * N * sizeof(R), s));
  CEV_CUDA(cudaMemsetAsync(adj, 0, 10 * N * sizeof(R), s));
  // forward sweep with checkpoints of the state before steps 0, C, 2C, ...,
  // each stretch of C steps in the time-blocked runner (sources only)
  auto seg_io = [&](int t0) {
    cev_fdtd_io f{};
    f.n_src = ns;
    f.src_idx = io->src_idx;
    f.src_w = io->src_w;
    f.amps = ns ? (const void*)((const R*)io->amps + t0) : nullptr;
    return f;
  };
  for (int t0 = 0; t0 < T; t0 += C) {
    CEV_CUDA(cudaMemcpyAsync(ck + (size_t)(t0 / C) * 6 * N, base, 6 * N * sizeof(R),
                             cudaMemcpyDeviceToDevice, s));
    const cev_fdtd_io f = seg_io(t0);
    int rc = run_tm_impl<R>(p, &st, std::min(C, T - t0), &f, s);
    if (rc != CEV_OK) return rc;
  }
  AdjArgs<R> a;
  a.nx = p->nx; a.ny = p->ny;
  a.ahx = adj; a.ahy = adj + N; a.adz = adj + 2 * N; a.aicex = adj + 3 * N; a.aicey = adj + 4 * N;
  a.aidz = adj + 5 * N; a.ach = adj + 6 * N; a.adey = adj + 7 * N; a.adex = adj + 8 * N;
  a.adzp = adj + 9 * N;
  a.iez = (const R*)p->iez;
  a.ax = (const AxisCoef<R>*)p->ax;
  a.ay = (const AxisCoef<R>*)p->ay;
  a.S = (R)p->S;
  const dim3 blk(32, 8);
  const dim3 g = grid2(p->nx, p->ny, blk);
  bool first = true;
  for (int seg0 = ((T - 1) / C) * C; seg0 >= 0; seg0 -= C) {
    const int seg1 = std::min(T, seg0 + C);
    // recompute Dz^{seg0} .. Dz^{seg1} (Dz^t = Dz after step t; index t - seg0)
    CEV_CUDA(cudaMemcpyAsync(base, ck + (size_t)(seg0 / C) * 6 * N, 6 * N * sizeof(R),
                             cudaMemcpyDeviceToDevice, s));
    CEV_CUDA(cudaMemcpyAsync(seg, cur[2], N * sizeof(R), cudaMemcpyDeviceToDevice, s));
    {
      const cev_fdtd_io f = seg_io(seg0);
      int rc = run_tm_impl<R>(p, &st, seg1 - seg0, &f, s, seg);
      if (rc != CEV_OK) return rc;
    }
    if (first) {
      // output step T (after the last step): aEz^T = w[T-1] p
      k_adj_init<R><<<(np + 127) / 128, 128, 0, s>>>((int)N, a.adz, a.iez, geps,
                                                       seg + (size_t)(T - seg0) * N, np,
                                                       io->probe_idx, w + (size_t)(T - 1) * np);
      first = false;
    }
    // reverse steps n = seg1 .. seg0+1 (step n maps state n-1 -> n)
    for (int n = seg1; n > seg0; --n) {
      k_adj_a<R><<<g, blk, 0, s>>>(a);
      k_adj_b<R><<<g, blk, 0, s>>>(a);
      // Ez^{n-1}: output of step n-1 (weights w[n-2]); n-1 == 0 is the initial field
      const R* wrow = (n - 1 >= 1) ? w + (size_t)(n - 2) * np : nullptr;
      const R* dzp = (n - 1 >= 1) ? seg + (size_t)(n - 1 - seg0) * N : nullptr;
      k_adj_c<R><<<g, blk, 0, s>>>(a, dzp, geps, np, io->probe_idx, wrow);
    }
    CEV_CHECK_LAUNCH("fdtd adjoint segment");
  }
  return CEV_OK;
}

}  // namespace cev

using namespace cev;

extern "C" {

int cev_fdtd_plan_create(cev_fdtd_plan* out, int nx, int ny, double dL, int npml_x, int npml_y,
                         int precision, const double* eps, cudaStream_t s) {
  CEV_REQUIRE(out != nullptr, "plan output pointer is NULL");
  *out = nullptr;
  CEV_REQUIRE(nx >= 2 && ny >= 2, "grid (%d, %d) must be at least 2x2", nx, ny);
  CEV_REQUIRE((long)nx * ny <= (1L << 31) - 1, "grid too large");
  CEV_REQUIRE(dL > 0 && std::isfinite(dL), "dL must be positive");
  CEV_REQUIRE(npml_x >= 0 && npml_y >= 0 && 2 * npml_x <= nx && 2 * npml_y <= ny,
              "npml (%d, %d) must be >= 0 and fit twice in the grid", npml_x, npml_y);
  CEV_REQUIRE(precision == CEV_PREC_C64 || precision == CEV_PREC_C128, "bad precision");
  CEV_REQUIRE(eps != nullptr, "eps is NULL");
  auto* p = new cev_fdtd_plan_s();
  p->nx = nx; p->ny = ny; p->npml_x = npml_x; p->npml_y = npml_y; p->prec = precision;
  p->dL = dL;
  p->dt = fdtd_dt(dL);
  const double C_0 = 1.0 / std::sqrt(F_EPSILON_0 * F_MU_0);
  p->S = C_0 * p->dt / dL;
  sigma_profile(nx, npml_x, p->dt, p->aHx, p->aDx);
  sigma_profile(ny, npml_y, p->dt, p->aHy, p->aDy);
  cudaError_t e = cudaSuccess;
  int arc = CEV_OK;
  auto up = [&](void** dst, const void* src, size_t bytes) {
    if (e != cudaSuccess || arc != CEV_OK) return;
    arc = dev_alloc(dst, bytes, s);
    // pageable source: the copy is staged before the call returns
    if (arc == CEV_OK) e = cudaMemcpyAsync(*dst, src, bytes, cudaMemcpyHostToDevice, s);
  };
  if (precision == CEV_PREC_C128) {
    auto cx = axis_coefs<double>(p->aHx, p->aDx, p->S), cy = axis_coefs<double>(p->aHy, p->aDy, p->S);
    up(&p->ax, cx.data(), cx.size() * sizeof(cx[0]));
    up(&p->ay, cy.data(), cy.size() * sizeof(cy[0]));
  } else {
    auto cx = axis_coefs<float>(p->aHx, p->aDx, p->S), cy = axis_coefs<float>(p->aHy, p->aDy, p->S);
    up(&p->ax, cx.data(), cx.size() * sizeof(cx[0]));
    up(&p->ay, cy.data(), cy.size() * sizeof(cy[0]));
  }
  const size_t N = p->n();
  if (arc == CEV_OK && e == cudaSuccess) arc = dev_alloc(&p->iez, N * p->rs(), s);
  if (arc == CEV_OK && e == cudaSuccess) arc = dev_alloc(&p->iexx, N * p->rs(), s);
  if (arc == CEV_OK && e == cudaSuccess) arc = dev_alloc(&p->ieyy, N * p->rs(), s);
  if (arc != CEV_OK) {
    cev_fdtd_plan_destroy(p);
    return arc;
  }
  if (e != cudaSuccess) {
    cev_fdtd_plan_destroy(p);
    return cuda_status(e, "cev_fdtd_plan_create");
  }
  int rc = cev_fdtd_set_eps(p, eps, s);
  if (rc != CEV_OK) {
    cev_fdtd_plan_destroy(p);
    return rc;
  }
  *out = p;
  return CEV_OK;
}

int cev_fdtd_plan_destroy(cev_fdtd_plan p) {
  if (!p) return CEV_OK;
  dev_free_all({p->pnbr, p->pflags, p->ax, p->ay, p->iez, p->iexx, p->ieyy, p->shadow});
  delete p;
  return CEV_OK;
}

int cev_fdtd_set_eps(cev_fdtd_plan p, const double* eps, cudaStream_t s) {
  CEV_REQUIRE(p && eps, "NULL argument");
  const size_t N = p->n();
  const unsigned g = std::max(1u, std::min(ceil_div(N, 256), 8u * sm_count()));
  if (p->prec == CEV_PREC_C128)
    k_inv_eps<double><<<g, 256, 0, s>>>(eps, (double*)p->iez, (double*)p->iexx, (double*)p->ieyy,
                                        p->nx, p->ny);
  else
    k_inv_eps<float><<<g, 256, 0, s>>>(eps, (float*)p->iez, (float*)p->iexx, (float*)p->ieyy,
                                       p->nx, p->ny);
  CEV_CHECK_LAUNCH("k_inv_eps");
  return CEV_OK;
}

double cev_fdtd_dt(cev_fdtd_plan p) { return p ? p->dt : 0.0; }

int cev_fdtd_step(cev_fdtd_plan p, const cev_fdtd_state* st, const void* jx, const void* jy,
                  const void* jz, int te, cudaStream_t s) {
  CEV_REQUIRE(p && st, "NULL argument");
  CEV_REQUIRE(st->hx && st->hy && st->dz && st->icex && st->icey && st->idz, "TM state incomplete");
  if (te || jx || jy) {
    CEV_REQUIRE(st->hz && st->dx && st->dy && st->ihz && st->ichx && st->ichy,
                "TE state incomplete");
    te = 1;
  }
  if (p->prec == CEV_PREC_C128)
    return step_impl<double>(p, st, (const double*)jx, (const double*)jy, (const double*)jz, te, s);
  return step_impl<float>(p, st, (const float*)jx, (const float*)jy, (const float*)jz, te, s);
}

int cev_fdtd_e_fields(cev_fdtd_plan p, const cev_fdtd_state* st, void* ex, void* ey, void* ez,
                      cudaStream_t s) {
  CEV_REQUIRE(p && st, "NULL argument");
  CEV_REQUIRE(!ez || st->dz, "ez needs st->dz");
  CEV_REQUIRE(!(ex || ey) || (st->dx && st->dy), "ex/ey need st->dx, st->dy");
  const size_t N = p->n();
  const unsigned g = std::max(1u, std::min(ceil_div(N, 256), 8u * sm_count()));
  if (p->prec == CEV_PREC_C128)
    k_e_fields<double><<<g, 256, 0, s>>>((int)N, (const double*)st->dx, (const double*)st->dy,
                                         (const double*)st->dz, (const double*)p->iexx,
                                         (const double*)p->ieyy, (const double*)p->iez,
                                         (double*)ex, (double*)ey, (double*)ez);
  else
    k_e_fields<float><<<g, 256, 0, s>>>((int)N, (const float*)st->dx, (const float*)st->dy,
                                        (const float*)st->dz, (const float*)p->iexx,
                                        (const float*)p->ieyy, (const float*)p->iez, (float*)ex,
                                        (float*)ey, (float*)ez);
  CEV_CHECK_LAUNCH("k_e_fields");
  return CEV_OK;
}

int cev_fdtd_run_tm(cev_fdtd_plan p, const cev_fdtd_state* st, int nsteps, const cev_fdtd_io* io,
                    cudaStream_t s) {
  CEV_REQUIRE(p && st, "NULL argument");
  CEV_REQUIRE(nsteps >= 0, "nsteps must be >= 0");
  CEV_REQUIRE(st->hx && st->hy && st->dz && st->icex && st->icey && st->idz, "TM state incomplete");
  if (io) {
    CEV_REQUIRE(io->n_src >= 0 && io->n_probe >= 0, "negative source/probe count");
    CEV_REQUIRE(io->n_src == 0 || (io->src_idx && io->src_w && io->amps), "source arrays missing");
    CEV_REQUIRE(io->n_probe == 0 || (io->probe_idx && io->probe_out), "probe arrays missing");
  }
  if (nsteps == 0) return CEV_OK;
  if (p->prec == CEV_PREC_C128) return run_tm_impl<double>(p, st, nsteps, io, s);
  return run_tm_impl<float>(p, st, nsteps, io, s);
}

int cev_fdtd_run_te(cev_fdtd_plan p, const cev_fdtd_state* st, int nsteps,
                    const cev_fdtd_io_te* io, cudaStream_t s) {
  CEV_REQUIRE(p && st, "NULL argument");
  CEV_REQUIRE(nsteps >= 0, "nsteps must be >= 0");
  CEV_REQUIRE(st->hz && st->dx && st->dy && st->ihz && st->ichx && st->ichy, "TE state incomplete");
  if (io) {
    CEV_REQUIRE(io->n_src >= 0 && io->n_probe >= 0, "negative source/probe count");
    CEV_REQUIRE(io->n_src == 0 || (io->src_idx && io->src_wx && io->src_wy && io->amps),
                "source arrays missing");
    CEV_REQUIRE(io->n_probe == 0 || (io->probe_idx && io->probe_out), "probe arrays missing");
  }
  if (nsteps == 0) return CEV_OK;
  if (p->prec == CEV_PREC_C128) return run_te_impl<double>(p, st, nsteps, io, s);
  return run_te_impl<float>(p, st, nsteps, io, s);
}

int cev_fdtd_step_adjoint_tm(cev_fdtd_plan p, const void* dz_in, const void* dz_out,
                             const void* g_ez, const cev_fdtd_state* adj, void* scratch,
                             double* geps, cudaStream_t s) {
  CEV_REQUIRE(p && dz_in && adj && scratch && geps, "NULL argument");
  CEV_REQUIRE(adj->hx && adj->hy && adj->dz && adj->icex && adj->icey && adj->idz,
              "adjoint state incomplete");
  CEV_REQUIRE(!g_ez || dz_out, "g_ez needs dz_out");
  if (p->prec == CEV_PREC_C128)
    return step_adjoint_impl<double>(p, (const double*)dz_in, (const double*)dz_out,
                                     (const double*)g_ez, adj, (double*)scratch, geps, s);
  return step_adjoint_impl<float>(p, (const float*)dz_in, (const float*)dz_out, (const float*)g_ez,
                                  adj, (float*)scratch, geps, s);
}

size_t cev_fdtd_adjoint_workspace_size(cev_fdtd_plan p, int nsteps, int C) {
  if (!p || nsteps < 1 || C < 1) return 0;
  const size_t N = p->n();
  const size_t nck = (nsteps + C - 1) / C + 1;
  return (6 + nck * 6 + (size_t)(C + 1) + 10) * N * p->rs();
}

int cev_fdtd_adjoint_tm(cev_fdtd_plan p, int nsteps, int C, const cev_fdtd_io* io, const void* w,
                        double* geps, void* ws, size_t ws_bytes, cudaStream_t s) {
  CEV_REQUIRE(p && io && w && geps && ws, "NULL argument");
  CEV_REQUIRE(nsteps >= 1 && C >= 1, "nsteps and ckpt_every must be >= 1");
  CEV_REQUIRE(io->n_probe >= 1 && io->probe_idx, "adjoint needs probes");
  CEV_REQUIRE(io->n_src == 0 || (io->src_idx && io->src_w && io->amps), "source arrays missing");
  const size_t need = cev_fdtd_adjoint_workspace_size(p, nsteps, C);
  CEV_REQUIRE(ws_bytes >= need, "workspace too small: need %zu bytes, got %zu", need, ws_bytes);
  if (p->prec == CEV_PREC_C128)
    return adjoint_impl<double>(p, nsteps, C, io, (const double*)w, geps, ws, s);
  return adjoint_impl<float>(p, nsteps, C, io, (const float*)w, geps, ws, s);
}

}  // extern "C"

// ====================================================================
// Allocation-free TM runner.
//
// For callers that must not allocate device memory themselves -- e.g. code
// running inside a host framework that owns every device allocation, or a
// real-time loop where cudaMalloc/cudaFree (which can synchronise the
// device) are forbidden.  It runs the same time-blocked TM kernels as
// cev_fdtd_run_tm, but the plan's tables, 1/eps and the second (shadow)
// copy of the state live in the file-scope arrays below, which every GPU
// that loads this library keeps for the life of the process.
//
// Limits: float32 only; nx*ny <= NOALLOC_MAX_CELLS (2^18 cells, e.g.
// 512x512), nx, ny <= NOALLOC_MAX_DIM.  Scratch: 7 * 2^18 floats (7 MiB)
// plus 2 * 8192 axis-coefficient records (512 KiB) per device.
// ====================================================================
namespace cev {
namespace {
constexpr size_t NOALLOC_MAX_CELLS = size_t(1) << 18;
constexpr int NOALLOC_MAX_DIM = 8192;
// [0, 6N): shadow TM state for the double-buffered blocked kernel; [6N, 7N): 1/eps_zz
static __device__ __align__(256) float g_noalloc_scratch[7 * NOALLOC_MAX_CELLS];
static __device__ __align__(256) AxisCoef<float> g_noalloc_axis[2 * NOALLOC_MAX_DIM];

struct NoAllocPtrs {
  float* scratch = nullptr;
  AxisCoef<float>* axis = nullptr;
};
constexpr int NOALLOC_MAX_DEVICES = 64;
static NoAllocPtrs g_noalloc_ptrs[NOALLOC_MAX_DEVICES];
static std::mutex g_noalloc_mu;

// Device addresses of the static arrays for the current device, looked up
// once per device (the host-side names are not device addresses).
int noalloc_setup(NoAllocPtrs& out) {
  int dev = 0;
  CEV_CUDA(cudaGetDevice(&dev));
  CEV_REQUIRE(dev >= 0 && dev < NOALLOC_MAX_DEVICES, "device index %d out of range", dev);
  std::lock_guard<std::mutex> lk(g_noalloc_mu);
  NoAllocPtrs& p = g_noalloc_ptrs[dev];
  if (!p.scratch) {
    void* s = nullptr;
    void* a = nullptr;
    CEV_CUDA(cudaGetSymbolAddress(&s, g_noalloc_scratch));
    CEV_CUDA(cudaGetSymbolAddress(&a, g_noalloc_axis));
    p.scratch = (float*)s;
    p.axis = (AxisCoef<float>*)a;
  }
  out = p;
  return CEV_OK;
}

__global__ void k_inv_ezz_f32(const double* eps, float* iez, size_t N) {
  for (size_t n = blockIdx.x * (size_t)blockDim.x + threadIdx.x; n < N;
       n += (size_t)gridDim.x * blockDim.x)
    iez[n] = (float)(1.0 / ((eps[n] + eps[n]) / 2));
}
}  // namespace
}  // namespace cev

namespace cev {
// AxisCoef<float>[N] of one axis computed on the device from (N, npml, dt, S):
// the sigma loop of ceviche/fdtd.py:224-263 keeps, for every 2X-grid index, the
// value of its last write (the largest loop index n that writes it), then the
// coefficients of axis_coefs.  Lets the allocation-free runner build its
// tables without host-to-device copies.
__global__ void k_axis_coef_f32(AxisCoef<float>* out, int N, int npml, double dt, double S) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  auto s2 = [&](int k) -> double {
    int n = -1;
    const int n1 = 2 * npml + 1 - k;       // written as k1 = 2 npml - n + 1
    const int n2 = k - 2 * N + 2 * npml;   // written as k2 = 2N - 2 npml + n
    if (n1 >= 0 && n1 < 2 * npml) n = n1;
    if (n2 >= 0 && n2 < 2 * npml && n2 >= n) n = n2;
    if (n < 0) return 0.0;
    const double x = (double)n / 2 / npml;
    return (0.5 * F_EPSILON_0 / dt) * (x * x * x);
  };
  const double h = s2(2 * i + 1) * dt / (2 * F_EPSILON_0);
  const double d = s2(2 * i) * dt / (2 * F_EPSILON_0);
  AxisCoef<float> c;
  c.aH = (float)h;
  c.f1H = (float)((1 - h) / (1 + h));
  c.f2H = (float)(S / (1 + h));
  c.pH = (float)(1 / (1 + h));
  c.aD = (float)d;
  c.f1D = (float)((1 - d) / (1 + d));
  c.f2D = (float)(S / (1 + d));
  c.pD = (float)(1 / (1 + d));
  out[i] = c;
}
}  // namespace cev

extern "C" CEV_API int cev_fdtd_run_tm_noalloc(int nx, int ny, double dL, int npml_x, int npml_y,
                                               const double* eps, const cev_fdtd_state* st,
                                               int nsteps, const cev_fdtd_io* io,
                                               cudaStream_t s) {
  using namespace cev;
  CEV_REQUIRE(st && eps, "NULL argument");
  CEV_REQUIRE(nx >= 2 && ny >= 2, "grid (%d, %d) must be at least 2x2", nx, ny);
  CEV_REQUIRE(nx <= NOALLOC_MAX_DIM && ny <= NOALLOC_MAX_DIM &&
                  (size_t)nx * (size_t)ny <= NOALLOC_MAX_CELLS,
              "grid (%d, %d) exceeds the allocation-free runner's limit of %zu cells "
              "(and %d per dimension); use cev_fdtd_run_tm",
              nx, ny, NOALLOC_MAX_CELLS, NOALLOC_MAX_DIM);
  CEV_REQUIRE(dL > 0 && std::isfinite(dL), "dL must be positive");
  CEV_REQUIRE(npml_x >= 0 && npml_y >= 0 && 2 * npml_x <= nx && 2 * npml_y <= ny,
              "npml (%d, %d) must be >= 0 and fit twice in the grid", npml_x, npml_y);
  CEV_REQUIRE(nsteps >= 0, "nsteps must be >= 0");
  CEV_REQUIRE(st->hx && st->hy && st->dz && st->icex && st->icey && st->idz, "TM state incomplete");
  if (io) {
    CEV_REQUIRE(io->n_src >= 0 && io->n_probe >= 0, "negative source/probe count");
    CEV_REQUIRE(io->n_src == 0 || (io->src_idx && io->src_w && io->amps), "source arrays missing");
    CEV_REQUIRE(io->n_probe == 0 || (io->probe_idx && io->probe_out), "probe arrays missing");
  }
  NoAllocPtrs sp;
  int rc = noalloc_setup(sp);
  if (rc != CEV_OK) return rc;
  if (nsteps == 0) return CEV_OK;
  // a plan whose device tables point into the static scratch (host struct only)
  cev_fdtd_plan_s p;
  p.nx = nx;
  p.ny = ny;
  p.npml_x = npml_x;
  p.npml_y = npml_y;
  p.prec = CEV_PREC_C64;
  p.dL = dL;
  p.dt = fdtd_dt(dL);
  const double C_0 = 1.0 / std::sqrt(F_EPSILON_0 * F_MU_0);
  p.S = C_0 * p.dt / dL;
  const size_t N = (size_t)nx * ny;
  AxisCoef<float>* ax = sp.axis;
  AxisCoef<float>* ay = sp.axis + NOALLOC_MAX_DIM;
  // tables built on the device: the call issues no host-to-device copy
  k_axis_coef_f32<<<ceil_div(nx, 256), 256, 0, s>>>(ax, nx, npml_x, p.dt, p.S);
  k_axis_coef_f32<<<ceil_div(ny, 256), 256, 0, s>>>(ay, ny, npml_y, p.dt, p.S);
  CEV_CHECK_LAUNCH("k_axis_coef_f32");
  float* iez = sp.scratch + 6 * NOALLOC_MAX_CELLS;
  k_inv_ezz_f32<<<std::max(1u, std::min(ceil_div(N, 256), 8u * sm_count())), 256, 0, s>>>(eps, iez,
                                                                                          N);
  CEV_CHECK_LAUNCH("k_inv_ezz_f32");
  p.ax = ax;
  p.ay = ay;
  p.iez = iez;
  p.shadow = sp.scratch;  // run_tm_impl uses 6N floats from here
  p.borrowed = true;      // ... and, for a borrowed plan, never allocates
  rc = run_tm_impl<float>(&p, st, nsteps, io, s);
  p.ax = p.ay = p.iez = p.shadow = nullptr;  // not owned: nothing for the host struct to free
  return rc;
}
