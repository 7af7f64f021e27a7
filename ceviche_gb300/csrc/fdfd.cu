// FDFD plan, matrix-free operator, field conversions and eps gradients.
#include <atomic>
#include <cmath>
#include <cstdarg>
#include <cstring>
#include <map>
#include <mutex>
#include <utility>

#include "fdfd_plan.hpp"

namespace cev {

// ------------------------------------------------------------------ errors
static thread_local char g_err[512] = "";

void set_error(const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
}

int cuda_status(cudaError_t e, const char* where) {
  set_error("CUDA error %d (%s) at %s", (int)e, cudaGetErrorString(e), where);
  return CEV_ERR_CUDA;
}

int sm_count() {
  static std::atomic<int> cache[64];
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 0 || dev >= 64) dev = 0;
  int v = cache[dev].load(std::memory_order_relaxed);
  if (v == 0) {
    int n = 0;
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0)
      n = 148;
    cache[dev].store(n, std::memory_order_relaxed);
    v = n;
  }
  return v;
}

// The dynamic shared-memory limit is an attribute of a kernel on the current
// device: record, per (device, kernel), the largest size already allowed.
int allow_dynamic_smem(const void* fn, int bytes, int carveout) {
  static std::mutex mu;
  static std::map<std::pair<int, const void*>, int> done;
  int dev = 0;
  CEV_CUDA(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lk(mu);
  int& have = done[std::make_pair(dev, fn)];
  if (have >= bytes) return CEV_OK;
  CEV_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
  if (carveout >= 0)
    CEV_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributePreferredSharedMemoryCarveout, carveout));
  have = bytes;
  return CEV_OK;
}

int dev_alloc(void** p, size_t bytes, cudaStream_t s) {
  static std::mutex mu;
  static std::map<int, bool> pooled;
  int dev = 0;
  CEV_CUDA(cudaGetDevice(&dev));
  {
    std::lock_guard<std::mutex> lk(mu);
    if (!pooled[dev]) {
      cudaMemPool_t pool;
      if (cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
        unsigned long long keep = 256ull << 20;
        cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
      }
      cudaGetLastError();
      pooled[dev] = true;
    }
  }
  *p = nullptr;
  CEV_CUDA(cudaMallocAsync(p, bytes, s));
  return CEV_OK;
}

void dev_free_all(std::initializer_list<void*> ps) {
  bool any = false;
  for (void* q : ps) any |= q != nullptr;
  if (!any) return;
  cudaDeviceSynchronize();
  for (void* q : ps)
    if (q) cudaFreeAsync(q, 0);
  cudaGetLastError();
}

// ------------------------------------------------------------ PML profiles
// sig_w / s_value of ceviche/derivatives.py:209-216 (m = 3, lnR = -30)
static zd s_value(double l, double dw, double omega) {
  const double ETA_0 = std::sqrt(MU_0 / EPSILON_0);
  const double m = 3.0, lnR = -30.0;
  const double sig_max = -(m + 1) * lnR / (2 * ETA_0 * dw);
  const double sig = sig_max * std::pow(l / dw, m);
  return zd(1.0, 0.0) - zd(0.0, 1.0) * (sig / (omega * EPSILON_0));
}

std::vector<zd> sfactor(bool forward, double omega, double dL, int N, int npml) {
  std::vector<zd> s(N, zd(1.0, 0.0));
  if (npml == 0) return s;
  const double dw = npml * dL;
  const double off = forward ? 0.5 : 1.0;
  for (int i = 0; i < N; ++i) {
    if (i <= npml)
      s[i] = s_value(dL * (npml - i + off), dw, omega);
    else if (i > N - npml)
      s[i] = s_value(dL * (i - (N - npml) - off), dw, omega);
  }
  return s;
}

void axis_tables(int pol, int N, int npml, double dL, double omega, double phase, bool transpose,
                 std::vector<Coef<double>>& out) {
  std::vector<zd> sf = sfactor(true, omega, dL, N, npml);
  std::vector<zd> sb = sfactor(false, omega, dL, N, npml);
  std::vector<zd> P(N), E(N), R(N, zd(1.0, 0.0));
  for (int i = 0; i < N; ++i) {
    if (pol == POL_EZ) {
      P[i] = 1.0 / sf[i];
      E[i] = 1.0 / sb[(i + 1) % N];  // W_{i+1/2} = 1/s_b[i+1]
    } else {
      P[i] = 1.0 / sb[i];
      E[i] = 1.0 / sf[i];  // W_{i+1/2} = (1/s_f[i]) * d[i]
    }
  }
  zd ph = std::exp(zd(0.0, phase));
  if (transpose) {
    std::swap(P, R);
    ph = std::conj(ph);
  }
  out.resize(N);
  for (int i = 0; i < N; ++i) {
    const int im = (i + N - 1) % N, ip = (i + 1) % N;
    zd cm = P[i] * E[im] * R[im];
    zd cp = P[i] * E[i] * R[ip];
    if (i == 0) cm *= std::conj(ph);
    if (i == N - 1) cp *= ph;
    const zd am = P[i] * E[im] * R[i];
    const zd ap = P[i] * E[i] * R[i];
    out[i].cm = make_double2(cm.real(), cm.imag());
    out[i].cp = make_double2(cp.real(), cp.imag());
    out[i].am = make_double2(am.real(), am.imag());
    out[i].ap = make_double2(ap.real(), ap.imag());
  }
}

// ------------------------------------------------------------ apply kernel
template <typename R, typename E = R>
struct ApplyArgs {
  int nx, ny, batch, rows;
  const E* eps;
  size_t eps_bs;
  const Cplx<R>* x;
  Cplx<R>* y;
  const Coef<R>* cx;
  const Coef<R>* cy;
  const R* k2;
  R oscale;
};

template <typename R, int POL, typename E>
__global__ void __launch_bounds__(128) k_apply(ApplyArgs<R, E> a) {
  using C = Cplx<R>;
  const int b = blockIdx.z;
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= a.ny) return;
  const int i0 = blockIdx.y * a.rows;
  const int i1 = min(i0 + a.rows, a.nx);
  const size_t N = (size_t)a.nx * a.ny;
  const C* x = a.x + b * N;
  C* y = a.y + b * N;
  const E* eps = a.eps + b * a.eps_bs;
  const Coef<R> cyj = a.cy[(size_t)b * a.ny + j];
  const R os = a.oscale;
  auto ep = [&](int i, C v, C) { y[(size_t)i * a.ny + j] = cscale(v, os); };
  stencil_column<R, POL, decltype(ep), false, E>(a.nx, a.ny, j, i0, i1, x, eps,
                                                 a.cx + (size_t)b * a.nx, cyj, a.k2[b], ep);
}

void launch_geometry(int nx, int ny, int batch, dim3& grid, dim3& block, int& rows) {
  int bx = ny >= 128 ? 128 : ((ny + 31) / 32) * 32;
  block = dim3(bx, 1, 1);
  const int cols = (ny + bx - 1) / bx;
  // about 64 blocks per SM: short row chunks keep many independent row
  // loads in flight (a column sweep waits on each row's loads)
  const long target = 64L * sm_count();
  long per = (long)cols * batch;
  rows = (int)std::max(2L, std::min(16L, (long)nx * per / std::max(1L, target)));
  grid = dim3(cols, (nx + rows - 1) / rows, batch);
}

template <typename R, typename E>
static int apply_impl(cev_fdfd_plan p, const E* eps, int eps_shared, const Cplx<R>* x, Cplx<R>* y,
                      int transpose, const Coef<R>* cx, const Coef<R>* cy, const R* k2, R oscale,
                      cudaStream_t s) {
  ApplyArgs<R, E> a;
  a.nx = p->nx;
  a.ny = p->ny;
  a.batch = p->batch;
  a.eps = eps;
  a.eps_bs = eps_shared ? 0 : p->n();
  a.x = x;
  a.y = y;
  a.cx = cx;
  a.cy = cy;
  a.k2 = k2;
  a.oscale = oscale;
  dim3 grid, block;
  launch_geometry(p->nx, p->ny, p->batch, grid, block, a.rows);
  if (p->pol == POL_EZ)
    k_apply<R, POL_EZ, E><<<grid, block, 0, s>>>(a);
  else
    k_apply<R, POL_HZ, E><<<grid, block, 0, s>>>(a);
  CEV_CHECK_LAUNCH("k_apply");
  return CEV_OK;
}

// -------------------------------------------------------- field conversion
// Permittivity elements: E = double (real eps) or double2 (complex eps,
// lossy media, interleaved).  The field and gradient kernels below compute in
// complex arithmetic throughout; for real eps every imaginary part is an
// exact zero, so the results equal the real-arithmetic ones.
__device__ __forceinline__ double2 ldE(const double* e, size_t i) { return make_double2(e[i], 0.0); }
__device__ __forceinline__ double2 ldE(const double2* e, size_t i) { return e[i]; }
// geps accumulation of a complex sensitivity c = dL-linear coefficient of
// d eps: real eps takes Re(c); complex eps (PyTorch convention
// dL/dRe + i dL/dIm) takes conj(c).
__device__ __forceinline__ void gacc(double* g, size_t i, double2 c) { g[i] += c.x; }
__device__ __forceinline__ void gacc(double2* g, size_t i, double2 c) { g[i] = cadd(g[i], cconj(c)); }
// 1 / ((a + b)/2 + 1e-5) in complex arithmetic
__device__ __forceinline__ double2 hz_dc(double2 a, double2 b) { return hz_d(a, b); }

struct FieldArgs {
  int nx, ny, batch;
  const void* eps;
  size_t eps_bs;
  const double2* fz;
  double2* f1;
  double2* f2;
  const double2 *sfx, *sbx, *sfy, *sby;
  double2 phx, phy;
  const double* omega;
  double dL;
};

// Ez -> (Hx, Hy) = (-Dyb Ez, Dxb Ez) / (1j w mu0)
__global__ void k_fields_ez(FieldArgs a) {
  const size_t N = (size_t)a.nx * a.ny;
  const int b = blockIdx.y;
  for (size_t n = blockIdx.x * (size_t)blockDim.x + threadIdx.x; n < N;
       n += (size_t)gridDim.x * blockDim.x) {
    const int i = (int)(n / a.ny), j = (int)(n % a.ny);
    const double2* u = a.fz + b * N;
    const double2 uc = u[n];
    double2 um_x = u[(size_t)((i + a.nx - 1) % a.nx) * a.ny + j];
    double2 um_y = u[(size_t)i * a.ny + (j + a.ny - 1) % a.ny];
    if (i == 0) um_x = cmul(cconj(a.phx), um_x);
    if (j == 0) um_y = cmul(cconj(a.phy), um_y);
    // Dxb u = (1/s_b[i]) (u_i - u_{i-1}) / dL
    const double2 dxb = cscale(cmul(a.sbx[(size_t)b * a.nx + i], csub(uc, um_x)), 1.0 / a.dL);
    const double2 dyb = cscale(cmul(a.sby[(size_t)b * a.ny + j], csub(uc, um_y)), 1.0 / a.dL);
    // 1/(1j w mu0) = -1j/(w mu0)
    const double c = 1.0 / (a.omega[b] * MU_0);
    // Hx = -(-1j c) Dyb = 1j c Dyb ; Hy = -1j c Dxb
    a.f1[b * N + n] = make_double2(-c * dyb.y, c * dyb.x);
    a.f2[b * N + n] = make_double2(c * dxb.y, -c * dxb.x);
  }
}

// Hz -> (Ex, Ey) = (Dyf Hz / (eps_xx+1e-5), -Dxf Hz / (eps_yy+1e-5)) / (1j w eps0)
template <typename E>
__global__ void k_fields_hz(FieldArgs a) {
  const size_t N = (size_t)a.nx * a.ny;
  const int b = blockIdx.y;
  for (size_t n = blockIdx.x * (size_t)blockDim.x + threadIdx.x; n < N;
       n += (size_t)gridDim.x * blockDim.x) {
    const int i = (int)(n / a.ny), j = (int)(n % a.ny);
    const double2* u = a.fz + b * N;
    const E* e = (const E*)a.eps + b * a.eps_bs;
    const double2 uc = u[n];
    double2 up_x = u[(size_t)((i + 1) % a.nx) * a.ny + j];
    double2 up_y = u[(size_t)i * a.ny + (j + 1) % a.ny];
    if (i == a.nx - 1) up_x = cmul(a.phx, up_x);
    if (j == a.ny - 1) up_y = cmul(a.phy, up_y);
    const double2 dxf = cscale(cmul(a.sfx[(size_t)b * a.nx + i], csub(up_x, uc)), 1.0 / a.dL);
    const double2 dyf = cscale(cmul(a.sfy[(size_t)b * a.ny + j], csub(up_y, uc)), 1.0 / a.dL);
    const double2 ec = ldE(e, n);
    const double2 dxx = hz_dc(ec, ldE(e, (size_t)i * a.ny + (j + a.ny - 1) % a.ny));
    const double2 dyy = hz_dc(ec, ldE(e, (size_t)((i + a.nx - 1) % a.nx) * a.ny + j));
    const double c = 1.0 / (a.omega[b] * EPSILON_0);
    // 1/(1j w eps0) = -1j c
    a.f1[b * N + n] = cmul(make_double2(c * dyf.y, -c * dyf.x), dxx);
    a.f2[b * N + n] = cmul(make_double2(-c * dxf.y, c * dxf.x), dyy);
  }
}

// ------------------------------------------------- field conversion adjoint
struct FieldAdjArgs {
  int nx, ny, batch, eps_shared;
  const void* eps;
  const double2* fz;
  const double2* g1;
  const double2* g2;
  double2* gz;
  void* geps;
  const double2 *sfx, *sbx, *sfy, *sby;
  double2 phx, phy;
  const double* omega;
  double dL;
};

// Ez: Hx = a1 Dyb Ez, Hy = a2 Dxb Ez with a1 = 1j c, a2 = -1j c, c = 1/(w mu0)
// gz += conj(a1) Dyb^H g1 + conj(a2) Dxb^H g2
__global__ void k_fields_adj_ez(FieldAdjArgs a) {
  const size_t N = (size_t)a.nx * a.ny;
  const int b = blockIdx.y;
  for (size_t n = blockIdx.x * (size_t)blockDim.x + threadIdx.x; n < N;
       n += (size_t)gridDim.x * blockDim.x) {
    const int i = (int)(n / a.ny), j = (int)(n % a.ny);
    const int ip = (i + 1) % a.nx, jp = (j + 1) % a.ny;
    const double2* g1 = a.g1 + b * N;
    const double2* g2 = a.g2 + b * N;
    // (Dxb^H v)_k = conj(sb_k) v_k/dL - conj(sb_{k+1}) v_{k+1} [ph at k=N-1] / dL
    const double2* sbx = a.sbx + (size_t)b * a.nx;
    const double2* sby = a.sby + (size_t)b * a.ny;
    double2 t2 = cmulc(sbx[i], g2[n]);
    double2 q2 = cmulc(sbx[ip], g2[(size_t)ip * a.ny + j]);
    if (i == a.nx - 1) q2 = cmul(a.phx, q2);
    t2 = cscale(csub(t2, q2), 1.0 / a.dL);
    double2 t1 = cmulc(sby[j], g1[n]);
    double2 q1 = cmulc(sby[jp], g1[(size_t)i * a.ny + jp]);
    if (j == a.ny - 1) q1 = cmul(a.phy, q1);
    t1 = cscale(csub(t1, q1), 1.0 / a.dL);
    const double c = 1.0 / (a.omega[b] * MU_0);
    // conj(1j c) = -1j c ; conj(-1j c) = 1j c
    const double2 r1 = make_double2(c * t1.y, -c * t1.x);
    const double2 r2 = make_double2(-c * t2.y, c * t2.x);
    double2 g = a.gz[b * N + n];
    g = cadd(g, cadd(r1, r2));
    a.gz[b * N + n] = g;
  }
}

// Hz: Ex = be*dxx*Dyf Hz, Ey = -be*dyy*Dxf Hz, be = -1j c, c = 1/(w eps0);
// gz += Dyf^H conj(be dxx) g1 + Dxf^H conj(-be dyy) g2
template <typename E>
__global__ void k_fields_adj_hz(FieldAdjArgs a) {
  const size_t N = (size_t)a.nx * a.ny;
  const int b = blockIdx.y;
  const size_t ebs = a.eps_shared ? 0 : N;
  for (size_t n = blockIdx.x * (size_t)blockDim.x + threadIdx.x; n < N;
       n += (size_t)gridDim.x * blockDim.x) {
    const int i = (int)(n / a.ny), j = (int)(n % a.ny);
    const int im = (i + a.nx - 1) % a.nx, jm = (j + a.ny - 1) % a.ny;
    const E* e = (const E*)a.eps + b * ebs;
    const double c = 1.0 / (a.omega[b] * EPSILON_0);
    const double2* g1 = a.g1 + b * N;
    const double2* g2 = a.g2 + b * N;
    const double2* sfx = a.sfx + (size_t)b * a.nx;
    const double2* sfy = a.sfy + (size_t)b * a.ny;
    // v1 = conj(be) conj(dxx) g1 = 1j c conj(dxx) g1 ; v2 = -1j c conj(dyy) g2
    auto v1 = [&](int ii, int jj) {
      const double2 d = hz_dc(ldE(e, (size_t)ii * a.ny + jj),
                              ldE(e, (size_t)ii * a.ny + (jj + a.ny - 1) % a.ny));
      const double2 g = cmulc(d, g1[(size_t)ii * a.ny + jj]);
      return make_double2(-c * g.y, c * g.x);
    };
    auto v2 = [&](int ii, int jj) {
      const double2 d = hz_dc(ldE(e, (size_t)ii * a.ny + jj),
                              ldE(e, (size_t)((ii + a.nx - 1) % a.nx) * a.ny + jj));
      const double2 g = cmulc(d, g2[(size_t)ii * a.ny + jj]);
      return make_double2(c * g.y, -c * g.x);
    };
    // (Dyf^H v)_k = (-conj(sf_k) v_k + conj(sf_{k-1}) v_{k-1} [conj(ph) at k=0]) / dL
    double2 q = cmulc(sfy[jm], v1(i, jm));
    if (j == 0) q = cmul(cconj(a.phy), q);
    double2 t1 = csub(q, cmulc(sfy[j], v1(i, j)));
    double2 r = cmulc(sfx[im], v2(im, j));
    if (i == 0) r = cmul(cconj(a.phx), r);
    double2 t2 = csub(r, cmulc(sfx[i], v2(i, j)));
    double2 g = a.gz[b * N + n];
    g = cadd(g, cscale(cadd(t1, t2), 1.0 / a.dL));
    a.gz[b * N + n] = g;
  }
}

// Direct eps dependence of (Ex, Ey): sensitivity of L to d is conj(g) * coef
// * Df Hz; d = 1/(avg + 1e-5) so d d = -d^2 d avg; avg^T spreads it to eps.
template <typename E, typename G>
__global__ void k_fields_adj_hz_eps(FieldAdjArgs a) {
  const size_t N = (size_t)a.nx * a.ny;
  const int nb = a.eps_shared ? a.batch : 1;
  const int b0 = a.eps_shared ? 0 : blockIdx.y;
  for (size_t n = blockIdx.x * (size_t)blockDim.x + threadIdx.x; n < N;
       n += (size_t)gridDim.x * blockDim.x) {
    const int i = (int)(n / a.ny), j = (int)(n % a.ny);
    const int ip = (i + 1) % a.nx, jp = (j + 1) % a.ny;
    double2 acc = make_double2(0.0, 0.0);
    for (int bb = 0; bb < nb; ++bb) {
      const int b = b0 + bb;
      const E* e = (const E*)a.eps + (a.eps_shared ? 0 : b * N);
      const double2* u = a.fz + b * N;
      const double c = 1.0 / (a.omega[b] * EPSILON_0);
      const double2* sfx = a.sfx + (size_t)b * a.nx;
      const double2* sfy = a.sfy + (size_t)b * a.ny;
      auto txx = [&](int ii, int jj) {
        const size_t m = (size_t)ii * a.ny + jj;
        const int jj1 = (jj + 1) % a.ny;
        double2 up = u[(size_t)ii * a.ny + jj1];
        if (jj == a.ny - 1) up = cmul(a.phy, up);
        const double2 df = cscale(cmul(sfy[jj], csub(up, u[m])), 1.0 / a.dL);
        const double2 ex_c = make_double2(c * df.y, -c * df.x);  // (-1j c) df
        const double2 d = hz_dc(ldE(e, m), ldE(e, (size_t)ii * a.ny + (jj + a.ny - 1) % a.ny));
        return cscale(cmul(cmul(d, d), cmulc(a.g1[b * N + m], ex_c)), -1.0);
      };
      auto tyy = [&](int ii, int jj) {
        const size_t m = (size_t)ii * a.ny + jj;
        const int ii1 = (ii + 1) % a.nx;
        double2 up = u[(size_t)ii1 * a.ny + jj];
        if (ii == a.nx - 1) up = cmul(a.phx, up);
        const double2 df = cscale(cmul(sfx[ii], csub(up, u[m])), 1.0 / a.dL);
        const double2 ey_c = make_double2(-c * df.y, c * df.x);  // (1j c) df
        const double2 d = hz_dc(ldE(e, m), ldE(e, (size_t)((ii + a.nx - 1) % a.nx) * a.ny + jj));
        return cscale(cmul(cmul(d, d), cmulc(a.g2[b * N + m], ey_c)), -1.0);
      };
      acc = cadd(acc, cscale(cadd(txx(i, j), txx(i, jp)), 0.5));
      acc = cadd(acc, cscale(cadd(tyy(i, j), tyy(ip, j)), 0.5));
    }
    gacc((G*)a.geps, (a.eps_shared ? 0 : (size_t)b0 * N) + n, acc);
  }
}

// ------------------------------------------------------------- eps gradient
// Sensitivities c of L to d eps (geps += Re(c), or conj(c) for complex eps):
// Ez: c = mu * x * eps0 w^2
// Hz: c_dyy = -(1/eps0) (Dxb^T mu)(Dxf x), c_dxx likewise along y;
//     c = avg^T(-d^2 c_d)
struct GradArgs {
  int nx, ny, batch, eps_shared, pol;
  const void* eps;
  const double2* x;
  const double2* mu;
  void* geps;
  const double2 *sfx, *sbx, *sfy, *sby;
  double2 phx, phy;
  const double* omega;
  double dL;
};

template <typename E, typename G>
__global__ void k_grad_eps(GradArgs a) {
  const size_t N = (size_t)a.nx * a.ny;
  const int nb = a.eps_shared ? a.batch : 1;
  const int b0 = a.eps_shared ? 0 : blockIdx.y;
  for (size_t n = blockIdx.x * (size_t)blockDim.x + threadIdx.x; n < N;
       n += (size_t)gridDim.x * blockDim.x) {
    const int i = (int)(n / a.ny), j = (int)(n % a.ny);
    double2 acc = make_double2(0.0, 0.0);
    for (int bb = 0; bb < nb; ++bb) {
      const int b = b0 + bb;
      const double2* x = a.x + b * N;
      const double2* mu = a.mu + b * N;
      if (a.pol == POL_EZ) {
        const double2 p = cmul(mu[n], x[n]);
        acc = cadd(acc, cscale(p, EPSILON_0 * a.omega[b] * a.omega[b]));
      } else {
        const E* e = (const E*)a.eps + (a.eps_shared ? 0 : b * N);
        const double2 *sfx = a.sfx + (size_t)b * a.nx, *sbx = a.sbx + (size_t)b * a.nx;
        const double2 *sfy = a.sfy + (size_t)b * a.ny, *sby = a.sby + (size_t)b * a.ny;
        auto gyy = [&](int ii, int jj) {
          const size_t m = (size_t)ii * a.ny + jj;
          const int ii1 = (ii + 1) % a.nx;
          double2 xp = x[(size_t)ii1 * a.ny + jj];
          if (ii == a.nx - 1) xp = cmul(a.phx, xp);
          const double2 dxf = cmul(sfx[ii], csub(xp, x[m]));
          // (Dxb^T mu)_k = sb_k mu_k - sb_{k+1} mu_{k+1} [conj(ph) at k = N-1]
          double2 q = cmul(sbx[ii1], mu[(size_t)ii1 * a.ny + jj]);
          if (ii == a.nx - 1) q = cmul(cconj(a.phx), q);
          const double2 dbt = csub(cmul(sbx[ii], mu[m]), q);
          const double2 cd = cscale(cmul(dbt, dxf), -(1.0 / EPSILON_0) / (a.dL * a.dL));
          const double2 d = hz_dc(ldE(e, m), ldE(e, (size_t)((ii + a.nx - 1) % a.nx) * a.ny + jj));
          return cscale(cmul(cmul(d, d), cd), -1.0);
        };
        auto gxx = [&](int ii, int jj) {
          const size_t m = (size_t)ii * a.ny + jj;
          const int jj1 = (jj + 1) % a.ny;
          double2 xp = x[(size_t)ii * a.ny + jj1];
          if (jj == a.ny - 1) xp = cmul(a.phy, xp);
          const double2 dyf = cmul(sfy[jj], csub(xp, x[m]));
          double2 q = cmul(sby[jj1], mu[(size_t)ii * a.ny + jj1]);
          if (jj == a.ny - 1) q = cmul(cconj(a.phy), q);
          const double2 dbt = csub(cmul(sby[jj], mu[m]), q);
          const double2 cd = cscale(cmul(dbt, dyf), -(1.0 / EPSILON_0) / (a.dL * a.dL));
          const double2 d = hz_dc(ldE(e, m), ldE(e, (size_t)ii * a.ny + (jj + a.ny - 1) % a.ny));
          return cscale(cmul(cmul(d, d), cd), -1.0);
        };
        const int ip = (i + 1) % a.nx, jp = (j + 1) % a.ny;
        acc = cadd(acc, cscale(cadd(gxx(i, j), gxx(i, jp)), 0.5));
        acc = cadd(acc, cscale(cadd(gyy(i, j), gyy(ip, j)), 0.5));
      }
    }
    gacc((G*)a.geps, (a.eps_shared ? 0 : (size_t)b0 * N) + n, acc);
  }
}


// --------------------------------------------------------- forward mode
// Tangent right-hand side rhs += -(dA/d eps . deps) x  (SI units):
//   Ez: +eps0 w^2 deps x
//   Hz: -(1/eps0)(Dxb (d'yy Dxf x) + Dyb (d'xx Dyf x)),
//       d'yy = -dyy^2 (deps + deps[i-1,j])/2, d'xx = -dxx^2 (deps + deps[i,j-1])/2
// (complex products for complex eps / deps).  Restates
// grad_sp_solve_entries_forward (ceviche/primitives.py:139-142), whose
// sp_mult(g, indices, x) is dA.x for the entries tangent g, chained from eps.
struct JvpArgs {
  int nx, ny, batch, eps_shared, pol;
  const void* eps;
  const void* deps;
  const double2* x;
  double2* out;
  const double2 *sfx, *sbx, *sfy, *sby;
  double2 phx, phy;
  const double* omega;
  double dL;
};

template <typename E>
__global__ void k_jvp_rhs(JvpArgs a) {
  const size_t N = (size_t)a.nx * a.ny;
  const int b = blockIdx.y;
  const size_t ebs = a.eps_shared ? 0 : N;
  const E* e = (const E*)a.eps + b * ebs;
  const E* de = (const E*)a.deps + b * ebs;
  const double2* x = a.x + b * N;
  for (size_t n = blockIdx.x * (size_t)blockDim.x + threadIdx.x; n < N;
       n += (size_t)gridDim.x * blockDim.x) {
    const int i = (int)(n / a.ny), j = (int)(n % a.ny);
    double2 v;
    if (a.pol == POL_EZ) {
      const double w = a.omega[b];
      v = cscale(cmul(x[n], ldE(de, n)), EPSILON_0 * w * w);
    } else {
      const double2 *sfx = a.sfx + (size_t)b * a.nx, *sbx = a.sbx + (size_t)b * a.nx;
      const double2 *sfy = a.sfy + (size_t)b * a.ny, *sby = a.sby + (size_t)b * a.ny;
      auto gx = [&](int ii) {
        const size_t m = (size_t)ii * a.ny + j;
        const int ip = (ii + 1) % a.nx, im = (ii + a.nx - 1) % a.nx;
        double2 xp = x[(size_t)ip * a.ny + j];
        if (ii == a.nx - 1) xp = cmul(a.phx, xp);
        const double2 df = cscale(cmul(sfx[ii], csub(xp, x[m])), 1.0 / a.dL);
        const double2 d = hz_dc(ldE(e, m), ldE(e, (size_t)im * a.ny + j));
        const double2 dd = cscale(cmul(cmul(d, d), cadd(ldE(de, m), ldE(de, (size_t)im * a.ny + j))), -0.5);
        return cmul(df, dd);
      };
      auto gy = [&](int jj) {
        const size_t m = (size_t)i * a.ny + jj;
        const int jp = (jj + 1) % a.ny, jm = (jj + a.ny - 1) % a.ny;
        double2 xp = x[(size_t)i * a.ny + jp];
        if (jj == a.ny - 1) xp = cmul(a.phy, xp);
        const double2 df = cscale(cmul(sfy[jj], csub(xp, x[m])), 1.0 / a.dL);
        const double2 d = hz_dc(ldE(e, m), ldE(e, (size_t)i * a.ny + jm));
        const double2 dd = cscale(cmul(cmul(d, d), cadd(ldE(de, m), ldE(de, (size_t)i * a.ny + jm))), -0.5);
        return cmul(df, dd);
      };
      const int im = (i + a.nx - 1) % a.nx, jm = (j + a.ny - 1) % a.ny;
      double2 gxm = gx(im), gym = gy(jm);
      if (i == 0) gxm = cmul(cconj(a.phx), gxm);
      if (j == 0) gym = cmul(cconj(a.phy), gym);
      const double2 tx = cscale(cmul(sbx[i], csub(gx(i), gxm)), 1.0 / a.dL);
      const double2 ty = cscale(cmul(sby[j], csub(gy(j), gym)), 1.0 / a.dL);
      v = cscale(cadd(tx, ty), -1.0 / EPSILON_0);
    }
    a.out[b * N + n] = cadd(a.out[b * N + n], v);
  }
}

// Direct eps tangent of the Hz field conversion (fdfd.py:150-162):
// dEx += (-1j c) d'xx Dyf Hz ; dEy += (1j c) d'yy Dxf Hz, c = 1/(w eps0)
template <typename E>
__global__ void k_fields_jvp_hz(JvpArgs a, double2* df2) {
  const size_t N = (size_t)a.nx * a.ny;
  const int b = blockIdx.y;
  const size_t ebs = a.eps_shared ? 0 : N;
  const E* e = (const E*)a.eps + b * ebs;
  const E* de = (const E*)a.deps + b * ebs;
  const double2* u = a.x + b * N;
  const double2* sfx = a.sfx + (size_t)b * a.nx;
  const double2* sfy = a.sfy + (size_t)b * a.ny;
  const double c = 1.0 / (a.omega[b] * EPSILON_0);
  for (size_t n = blockIdx.x * (size_t)blockDim.x + threadIdx.x; n < N;
       n += (size_t)gridDim.x * blockDim.x) {
    const int i = (int)(n / a.ny), j = (int)(n % a.ny);
    const int ip = (i + 1) % a.nx, im = (i + a.nx - 1) % a.nx;
    const int jp = (j + 1) % a.ny, jm = (j + a.ny - 1) % a.ny;
    double2 upx = u[(size_t)ip * a.ny + j], upy = u[(size_t)i * a.ny + jp];
    if (i == a.nx - 1) upx = cmul(a.phx, upx);
    if (j == a.ny - 1) upy = cmul(a.phy, upy);
    const double2 dxf = cscale(cmul(sfx[i], csub(upx, u[n])), 1.0 / a.dL);
    const double2 dyf = cscale(cmul(sfy[j], csub(upy, u[n])), 1.0 / a.dL);
    const double2 dxx = hz_dc(ldE(e, n), ldE(e, (size_t)i * a.ny + jm));
    const double2 dyy = hz_dc(ldE(e, n), ldE(e, (size_t)im * a.ny + j));
    const double2 pxx = cscale(cmul(cmul(dxx, dxx), cadd(ldE(de, n), ldE(de, (size_t)i * a.ny + jm))), -0.5);
    const double2 pyy = cscale(cmul(cmul(dyy, dyy), cadd(ldE(de, n), ldE(de, (size_t)im * a.ny + j))), -0.5);
    // (-1j c) pxx dyf ; (1j c) pyy dxf
    const double2 t1 = cmul(pxx, dyf), t2 = cmul(pyy, dxf);
    const double2 ex = make_double2(c * t1.y, -c * t1.x);
    const double2 ey = make_double2(-c * t2.y, c * t2.x);
    a.out[b * N + n] = cadd(a.out[b * N + n], ex);
    df2[b * N + n] = cadd(df2[b * N + n], ey);
  }
}

static dim3 grid_1d(size_t N, int batch) {
  const unsigned blocks = std::max(1u, std::min(ceil_div(N, 256), (unsigned)(8 * sm_count())));
  return dim3(blocks, batch, 1);
}

}  // namespace cev

using namespace cev;

// =============================================================== C ABI
extern "C" {

const char* cev_last_error_string(void) { return g_err; }

int cev_version(void) { return 100; }

int cev_fdfd_plan_create(cev_fdfd_plan* out, int pol, int nx, int ny, int batch, double dL,
                         const double* omegas, int npml_x, int npml_y, double bloch_x,
                         double bloch_y) {
  CEV_REQUIRE(out != nullptr, "plan output pointer is NULL");
  *out = nullptr;
  CEV_REQUIRE(pol == CEV_POL_EZ || pol == CEV_POL_HZ, "pol must be CEV_POL_EZ or CEV_POL_HZ");
  CEV_REQUIRE(nx >= 2 && ny >= 2,
              "grid (%d, %d): both dimensions must be >= 2 (1D grids fail in the reference solve)",
              nx, ny);
  CEV_REQUIRE((long)nx * ny <= (1L << 31) - 1, "grid too large");
  CEV_REQUIRE(batch >= 1 && batch <= 65535, "batch must be in [1, 65535]");
  CEV_REQUIRE(dL > 0 && std::isfinite(dL), "dL must be positive");
  CEV_REQUIRE(omegas != nullptr, "omegas is NULL");
  CEV_REQUIRE(npml_x >= 0 && npml_y >= 0 && 2 * npml_x <= nx && 2 * npml_y <= ny,
              "npml (%d, %d) must be >= 0 and fit twice in the grid", npml_x, npml_y);
  for (int b = 0; b < batch; ++b)
    CEV_REQUIRE(std::isfinite(omegas[b]) && omegas[b] > 0, "omega[%d] must be positive", b);

  auto* p = new cev_fdfd_plan_s();
  p->pol = pol;
  p->nx = nx;
  p->ny = ny;
  p->batch = batch;
  p->dL = dL;
  p->npml_x = npml_x;
  p->npml_y = npml_y;
  p->bloch_x = bloch_x;
  p->bloch_y = bloch_y;
  p->omega.assign(omegas, omegas + batch);
  p->scale = (pol == CEV_POL_EZ ? MU_0 : EPSILON_0) * dL * dL;
  p->phx = make_double2(std::cos(bloch_x), std::sin(bloch_x));
  p->phy = make_double2(std::cos(bloch_y), std::sin(bloch_y));
  cudaGetDevice(&p->device);

  std::vector<Coef<double>> hx[2], hy[2], t;
  std::vector<double> k2(batch);
  std::vector<double2> sfx(batch * (size_t)nx), sbx(batch * (size_t)nx), sfy(batch * (size_t)ny),
      sby(batch * (size_t)ny);
  for (int b = 0; b < batch; ++b) {
    const double w = omegas[b];
    k2[b] = EPSILON_0 * MU_0 * w * w * dL * dL;
    for (int tr = 0; tr < 2; ++tr) {
      axis_tables(pol, nx, npml_x, dL, w, bloch_x, tr, t);
      hx[tr].insert(hx[tr].end(), t.begin(), t.end());
      axis_tables(pol, ny, npml_y, dL, w, bloch_y, tr, t);
      hy[tr].insert(hy[tr].end(), t.begin(), t.end());
    }
    auto fx = sfactor(true, w, dL, nx, npml_x), bx = sfactor(false, w, dL, nx, npml_x);
    auto fy = sfactor(true, w, dL, ny, npml_y), by = sfactor(false, w, dL, ny, npml_y);
    for (int i = 0; i < nx; ++i) {
      zd a = 1.0 / fx[i], c = 1.0 / bx[i];
      sfx[b * (size_t)nx + i] = make_double2(a.real(), a.imag());
      sbx[b * (size_t)nx + i] = make_double2(c.real(), c.imag());
    }
    for (int j = 0; j < ny; ++j) {
      zd a = 1.0 / fy[j], c = 1.0 / by[j];
      sfy[b * (size_t)ny + j] = make_double2(a.real(), a.imag());
      sby[b * (size_t)ny + j] = make_double2(c.real(), c.imag());
    }
  }
  auto up = [&](auto** dst, const auto& src) -> cudaError_t {
    using T = std::remove_reference_t<decltype(src[0])>;
    cudaError_t e = cudaMalloc((void**)dst, src.size() * sizeof(T));
    if (e != cudaSuccess) return e;
    return cudaMemcpy(*dst, src.data(), src.size() * sizeof(T), cudaMemcpyHostToDevice);
  };
  cudaError_t e = cudaSuccess;
  for (int tr = 0; tr < 2 && e == cudaSuccess; ++tr) {
    std::vector<Coef<float>> fx(hx[tr].size()), fy(hy[tr].size());
    for (size_t k = 0; k < fx.size(); ++k)
      fx[k] = {to_f(hx[tr][k].cm), to_f(hx[tr][k].cp), to_f(hx[tr][k].am), to_f(hx[tr][k].ap)};
    for (size_t k = 0; k < fy.size(); ++k)
      fy[k] = {to_f(hy[tr][k].cm), to_f(hy[tr][k].cp), to_f(hy[tr][k].am), to_f(hy[tr][k].ap)};
    if (e == cudaSuccess) e = up(&p->cx64[tr], hx[tr]);
    if (e == cudaSuccess) e = up(&p->cy64[tr], hy[tr]);
    if (e == cudaSuccess) e = up(&p->cx32[tr], fx);
    if (e == cudaSuccess) e = up(&p->cy32[tr], fy);
  }
  std::vector<float> k2f(k2.begin(), k2.end());
  if (e == cudaSuccess) e = up(&p->k2_64, k2);
  if (e == cudaSuccess) e = up(&p->k2_32, k2f);
  if (e == cudaSuccess) e = up(&p->omega_d, p->omega);
  if (e == cudaSuccess) e = up(&p->ft.sfx, sfx);
  if (e == cudaSuccess) e = up(&p->ft.sbx, sbx);
  if (e == cudaSuccess) e = up(&p->ft.sfy, sfy);
  if (e == cudaSuccess) e = up(&p->ft.sby, sby);
  if (e != cudaSuccess) {
    cev_fdfd_plan_destroy(p);
    return cuda_status(e, "cev_fdfd_plan_create upload");
  }
  *out = p;
  return CEV_OK;
}

int cev_fdfd_axis_matrix(cev_fdfd_plan p, int b, int axis, int transpose, double* out) {
  CEV_REQUIRE(p != nullptr && out != nullptr, "NULL argument");
  CEV_REQUIRE(b >= 0 && b < p->batch, "problem %d out of range", b);
  CEV_REQUIRE(axis == 0 || axis == 1, "axis must be 0 (x) or 1 (y)");
  const int n = axis == 0 ? p->nx : p->ny;
  std::vector<Coef<double>> t;
  axis_tables(p->pol, n, axis == 0 ? p->npml_x : p->npml_y, p->dL, p->omega[b],
              axis == 0 ? p->bloch_x : p->bloch_y, transpose != 0, t);
  std::fill(out, out + 2 * (size_t)n * n, 0.0);
  auto add = [&](int r, int c, double2 v) {
    out[2 * ((size_t)r * n + c)] += v.x;
    out[2 * ((size_t)r * n + c) + 1] += v.y;
  };
  for (int i = 0; i < n; ++i) {
    add(i, (i + n - 1) % n, t[i].cm);
    add(i, (i + 1) % n, t[i].cp);
    add(i, i, make_double2(-(t[i].am.x + t[i].ap.x), -(t[i].am.y + t[i].ap.y)));
  }
  return CEV_OK;
}

int cev_fdfd_plan_set_eps_complex(cev_fdfd_plan p, int on) {
  CEV_REQUIRE(p != nullptr, "plan is NULL");
  CEV_REQUIRE(p->mf_nsb < 0 || !on, "multi-frequency plans take a real eps");
  p->eps_complex = on ? 1 : 0;
  return CEV_OK;
}

int cev_fdfd_plan_destroy(cev_fdfd_plan p) {
  if (!p) return CEV_OK;
  for (int tr = 0; tr < 2; ++tr) {
    cudaFree(p->cx64[tr]);
    cudaFree(p->cy64[tr]);
    cudaFree(p->cx32[tr]);
    cudaFree(p->cy32[tr]);
  }
  cudaFree(p->k2_64);
  cudaFree(p->k2_32);
  cudaFree(p->omega_d);
  cudaFree(p->ft.sfx);
  cudaFree(p->ft.sbx);
  cudaFree(p->ft.sfy);
  cudaFree(p->ft.sby);
  delete p;
  return CEV_OK;
}

double cev_fdfd_plan_scale(cev_fdfd_plan p) { return p ? p->scale : 0.0; }

int cev_fdfd_apply(cev_fdfd_plan p, const void* eps, int eps_shared, const void* x, void* y,
                   int transpose, int precision, int si_units, cudaStream_t s) {
  CEV_REQUIRE(p != nullptr, "plan is NULL");
  CEV_REQUIRE(eps && x && y, "eps/x/y must be non-NULL");
  CEV_REQUIRE(x != y, "x and y must not alias");
  const int tr = transpose ? 1 : 0;
  const bool ce = p->eps_complex != 0;
  if (precision == CEV_PREC_C128) {
    const double os = si_units ? 1.0 / p->scale : 1.0;
    if (ce)
      return apply_impl<double>(p, (const double2*)eps, eps_shared, (const double2*)x,
                                (double2*)y, tr, p->cx64[tr], p->cy64[tr], p->k2_64, os, s);
    return apply_impl<double>(p, (const double*)eps, eps_shared, (const double2*)x, (double2*)y, tr,
                              p->cx64[tr], p->cy64[tr], p->k2_64, os, s);
  }
  CEV_REQUIRE(precision == CEV_PREC_C64, "precision must be CEV_PREC_C64 or CEV_PREC_C128");
  const float os = si_units ? (float)(1.0 / p->scale) : 1.0f;
  if (ce)
    return apply_impl<float>(p, (const float2*)eps, eps_shared, (const float2*)x, (float2*)y, tr,
                             p->cx32[tr], p->cy32[tr], p->k2_32, os, s);
  return apply_impl<float>(p, (const float*)eps, eps_shared, (const float2*)x, (float2*)y, tr,
                           p->cx32[tr], p->cy32[tr], p->k2_32, os, s);
}

int cev_fdfd_fields(cev_fdfd_plan p, const double* eps, int eps_shared, const void* fz, void* f1,
                    void* f2, cudaStream_t s) {
  CEV_REQUIRE(p != nullptr, "plan is NULL");
  CEV_REQUIRE(eps && fz && f1 && f2, "NULL argument");
  FieldArgs a;
  a.nx = p->nx;
  a.ny = p->ny;
  a.batch = p->batch;
  a.eps = eps;
  a.eps_bs = eps_shared ? 0 : p->n();
  a.fz = (const double2*)fz;
  a.f1 = (double2*)f1;
  a.f2 = (double2*)f2;
  a.sfx = p->ft.sfx;
  a.sbx = p->ft.sbx;
  a.sfy = p->ft.sfy;
  a.sby = p->ft.sby;
  a.phx = p->phx;
  a.phy = p->phy;
  a.omega = p->omega_d;
  a.dL = p->dL;
  if (p->pol == CEV_POL_EZ)
    k_fields_ez<<<grid_1d(p->n(), p->batch), 256, 0, s>>>(a);
  else if (p->eps_complex)
    k_fields_hz<double2><<<grid_1d(p->n(), p->batch), 256, 0, s>>>(a);
  else
    k_fields_hz<double><<<grid_1d(p->n(), p->batch), 256, 0, s>>>(a);
  CEV_CHECK_LAUNCH("k_fields");
  return CEV_OK;
}

int cev_fdfd_fields_adjoint(cev_fdfd_plan p, const double* eps, int eps_shared, const void* fz,
                            const void* g1, const void* g2, void* gz, double* geps,
                            cudaStream_t s) {
  const bool ce = p && p->eps_complex;
  CEV_REQUIRE(p != nullptr, "plan is NULL");
  CEV_REQUIRE(eps && g1 && g2 && gz, "NULL argument");
  FieldAdjArgs a;
  a.nx = p->nx;
  a.ny = p->ny;
  a.batch = p->batch;
  a.eps_shared = eps_shared ? 1 : 0;
  a.eps = eps;
  a.fz = (const double2*)fz;
  a.g1 = (const double2*)g1;
  a.g2 = (const double2*)g2;
  a.gz = (double2*)gz;
  a.geps = geps;
  a.sfx = p->ft.sfx;
  a.sbx = p->ft.sbx;
  a.sfy = p->ft.sfy;
  a.sby = p->ft.sby;
  a.phx = p->phx;
  a.phy = p->phy;
  a.omega = p->omega_d;
  a.dL = p->dL;
  if (p->pol == CEV_POL_EZ) {
    k_fields_adj_ez<<<grid_1d(p->n(), p->batch), 256, 0, s>>>(a);
  } else {
    if (ce)
      k_fields_adj_hz<double2><<<grid_1d(p->n(), p->batch), 256, 0, s>>>(a);
    else
      k_fields_adj_hz<double><<<grid_1d(p->n(), p->batch), 256, 0, s>>>(a);
    CEV_CHECK_LAUNCH("k_fields_adj_hz");
    if (geps) {
      CEV_REQUIRE(fz != nullptr, "Hz field adjoint with geps needs fz");
      const dim3 g = grid_1d(p->n(), eps_shared ? 1 : p->batch);
      if (ce)
        k_fields_adj_hz_eps<double2, double2><<<g, 256, 0, s>>>(a);
      else
        k_fields_adj_hz_eps<double, double><<<g, 256, 0, s>>>(a);
    }
  }
  CEV_CHECK_LAUNCH("k_fields_adj");
  return CEV_OK;
}

int cev_fdfd_grad_eps(cev_fdfd_plan p, const double* eps, int eps_shared, const void* x,
                      const void* mu, double* geps, cudaStream_t s) {
  CEV_REQUIRE(p != nullptr, "plan is NULL");
  CEV_REQUIRE(eps && x && mu && geps, "NULL argument");
  GradArgs a;
  a.nx = p->nx;
  a.ny = p->ny;
  a.batch = p->batch;
  a.eps_shared = eps_shared ? 1 : 0;
  a.pol = p->pol;
  a.eps = eps;
  a.x = (const double2*)x;
  a.mu = (const double2*)mu;
  a.geps = geps;
  a.sfx = p->ft.sfx;
  a.sbx = p->ft.sbx;
  a.sfy = p->ft.sfy;
  a.sby = p->ft.sby;
  a.phx = p->phx;
  a.phy = p->phy;
  a.omega = p->omega_d;
  a.dL = p->dL;
  const dim3 g = grid_1d(p->n(), eps_shared ? 1 : p->batch);
  if (p->eps_complex)
    k_grad_eps<double2, double2><<<g, 256, 0, s>>>(a);
  else
    k_grad_eps<double, double><<<g, 256, 0, s>>>(a);
  CEV_CHECK_LAUNCH("k_grad_eps");
  return CEV_OK;
}

int cev_fdfd_jvp_rhs(cev_fdfd_plan p, const double* eps, int eps_shared, const double* deps,
                     const void* x, void* rhs, cudaStream_t s) {
  CEV_REQUIRE(p != nullptr, "plan is NULL");
  CEV_REQUIRE(eps && deps && x && rhs, "NULL argument");
  JvpArgs a{p->nx, p->ny, p->batch, eps_shared ? 1 : 0, p->pol, eps, deps, (const double2*)x,
            (double2*)rhs, p->ft.sfx, p->ft.sbx, p->ft.sfy, p->ft.sby, p->phx, p->phy, p->omega_d,
            p->dL};
  if (p->eps_complex)
    k_jvp_rhs<double2><<<grid_1d(p->n(), p->batch), 256, 0, s>>>(a);
  else
    k_jvp_rhs<double><<<grid_1d(p->n(), p->batch), 256, 0, s>>>(a);
  CEV_CHECK_LAUNCH("k_jvp_rhs");
  return CEV_OK;
}

int cev_fdfd_fields_jvp(cev_fdfd_plan p, const double* eps, int eps_shared, const double* deps,
                        const void* fz, void* df1, void* df2, cudaStream_t s) {
  CEV_REQUIRE(p != nullptr, "plan is NULL");
  CEV_REQUIRE(eps && deps && fz && df1 && df2, "NULL argument");
  if (p->pol == CEV_POL_EZ) return CEV_OK;  // Hx, Hy do not depend on eps directly
  JvpArgs a{p->nx, p->ny, p->batch, eps_shared ? 1 : 0, p->pol, eps, deps, (const double2*)fz,
            (double2*)df1, p->ft.sfx, p->ft.sbx, p->ft.sfy, p->ft.sby, p->phx, p->phy, p->omega_d,
            p->dL};
  if (p->eps_complex)
    k_fields_jvp_hz<double2><<<grid_1d(p->n(), p->batch), 256, 0, s>>>(a, (double2*)df2);
  else
    k_fields_jvp_hz<double><<<grid_1d(p->n(), p->batch), 256, 0, s>>>(a, (double2*)df2);
  CEV_CHECK_LAUNCH("k_fields_jvp_hz");
  return CEV_OK;
}

}  // extern "C"
