// Waveguide modes for ceviche.modes.get_modes / insert_mode
// (ceviche/modes.py:10-65): the m eigenpairs of
//     A = diag(eps) + Dxf Dxb / k0^2,   k0 = omega / C_0,
// nearest sigma = max(eps) -- the reference's shift-invert ARPACK call
// (modes.py:68-78, scipy eigs with sigma = n_max^2, which='LM') -- for a
// batch of 1D cross sections, one CTA per section.
//
// Dxf Dxb is the 1D second difference of ceviche/derivatives.py with its
// SC-PML stretch (sfactor, derivatives.py:173-216) and the periodic wrap of
// the (N, 1) grid: row i holds up_i at column i+1, dn_i at column i-1
// (indices mod N) and -(up_i + dn_i) on the diagonal, with
// up_i = 1 / (s_f[i] s_b[i+1] (k0 dL)^2) and dn_i = 1 / (s_f[i] s_b[i] (k0 dL)^2).
//
// Method (own design, FP64 complex throughout):
//   * M = A - sigma I is cyclic tridiagonal.  M = B + u v^T with B
//     tridiagonal (Sherman-Morrison for the two corner entries); B is
//     factored once by Gaussian elimination with partial pivoting
//     (one thread, O(N)).
//   * Orthogonal iteration Q <- qr(M^{-1} Q) on k = min(N, max(m + 4, 2m), 24)
//     vectors (k threads solve one column each; modified Gram-Schmidt with
//     block reductions).
//   * Every iteration a Rayleigh-Ritz step: G = Q^H A Q (k x k), its
//     eigenpairs by small_eig, Ritz values ordered by |theta - sigma|
//     (nearest first, the order the reference returns); converged when the
//     m leading Ritz residuals ||A x - theta x|| / ||x|| are <= tol max(1, |sigma|).
//   * Output vectors have unit 2-norm and their largest-magnitude entry
//     (first one on ties) real and positive.  The reference's phase is that
//     of ARPACK's random start vector, i.e. arbitrary.
#include <cmath>
#include <vector>

#include "fdfd_plan.hpp"
#include "reduce.cuh"
#include "small_eig.cuh"

namespace cev {

static constexpr int MODE_THREADS = 256;
static constexpr int MODE_KMAX = 24;

struct ModeArgs {
  int n, m, k, max_iters;
  double tol;
  const double* eps;   // [B][n]
  const double2* up;   // [n] coefficient to column i+1 (mod n)
  const double2* dn;   // [n] coefficient to column i-1 (mod n)
  double2* vals;       // [B][m]
  double2* vecs;       // [B][m][n]
  int* iters;          // [B]
  int* status;         // [B]
  char* ws;            // per problem ws_stride bytes
  size_t ws_stride;
};

struct ModeWs {
  double2 *u0, *u1, *u2, *lm, *z, *Q, *Y, *AQ;
  unsigned char* piv;
};

__host__ __device__ inline size_t mode_ws_stride(int n, int k) {
  const size_t c = sizeof(double2) * (size_t)n;
  size_t s = c * (5 + 3 * (size_t)k) + (size_t)n;
  return (s + 255) & ~(size_t)255;
}

__device__ inline ModeWs mode_ws(char* base, int n, int k) {
  ModeWs w;
  double2* p = (double2*)base;
  w.u0 = p; p += n;
  w.u1 = p; p += n;
  w.u2 = p; p += n;
  w.lm = p; p += n;
  w.z = p; p += n;
  w.Q = p; p += (size_t)k * n;
  w.Y = p; p += (size_t)k * n;
  w.AQ = p; p += (size_t)k * n;
  w.piv = (unsigned char*)p;
  return w;
}

// Solve B y = x in place with the pivoted LU (u0 diag, u1 / u2 first and
// second super-diagonals, lm multipliers, piv row swaps).
__device__ inline void lu_solve(const ModeWs& w, int n, double2* x) {
  for (int i = 0; i + 1 < n; ++i) {
    if (w.piv[i]) {
      const double2 t = x[i];
      x[i] = x[i + 1];
      x[i + 1] = t;
    }
    x[i + 1] = csub(x[i + 1], cmul(w.lm[i], x[i]));
  }
  for (int i = n - 1; i >= 0; --i) {
    double2 s = x[i];
    if (i + 1 < n) s = csub(s, cmul(w.u1[i], x[i + 1]));
    if (i + 2 < n) s = csub(s, cmul(w.u2[i], x[i + 2]));
    x[i] = cdivd(s, w.u0[i]);
  }
}

__device__ inline double2 block_cdot(const double2* a, const double2* b, int n, double* sm) {
  double v[2] = {0.0, 0.0};
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const double2 t = cmulc(a[i], b[i]);
    v[0] += t.x;
    v[1] += t.y;
  }
  block_sum<2>(v, sm);
  __shared__ double2 res;
  if (threadIdx.x == 0) res = make_double2(v[0], v[1]);
  __syncthreads();
  const double2 r = res;
  __syncthreads();
  return r;
}

__device__ inline double2 hash_c(unsigned i, unsigned j) {
  unsigned h = i * 0x9E3779B1u ^ (j + 0x7F4A7C15u) * 0x85EBCA77u;
  h ^= h >> 15; h *= 0x2C1B3C6Du; h ^= h >> 12; h *= 0x297A2D39u; h ^= h >> 15;
  const unsigned g = h * 0x165667B1u + 0x27D4EB2Fu;
  return make_double2((h & 0xFFFFFF) / 16777216.0 - 0.5, (g & 0xFFFFFF) / 16777216.0 - 0.5);
}

// Orthonormalise the k columns of X in place (modified Gram-Schmidt, twice
// for the columns whose norm dropped); returns false on a zero column.
__device__ bool mgs(double2* X, int n, int k, double* sm) {
  bool ok = true;
  for (int j = 0; j < k; ++j) {
    double2* xj = X + (size_t)j * n;
    double before = 0.0;
    {
      const double2 t = block_cdot(xj, xj, n, sm);
      before = t.x;
    }
    for (int pass = 0; pass < 2; ++pass) {
      for (int l = 0; l < j; ++l) {
        const double2* ql = X + (size_t)l * n;
        const double2 r = block_cdot(ql, xj, n, sm);
        for (int i = threadIdx.x; i < n; i += blockDim.x) xj[i] = csub(xj[i], cmul(r, ql[i]));
        __syncthreads();
      }
      const double2 t = block_cdot(xj, xj, n, sm);
      if (pass == 0 && t.x > 0.25 * before) {
        before = t.x;
        break;
      }
      before = t.x;
    }
    const double nrm = sqrt(before);
    if (!(nrm > 0.0)) {
      ok = false;
      break;
    }
    for (int i = threadIdx.x; i < n; i += blockDim.x) xj[i] = cscale(xj[i], 1.0 / nrm);
    __syncthreads();
  }
  return ok;
}

__global__ void __launch_bounds__(MODE_THREADS) k_modes(ModeArgs a) {
  const int b = blockIdx.x, n = a.n, k = a.k, m = a.m;
  const double* eps = a.eps + (size_t)b * n;
  ModeWs w = mode_ws(a.ws + (size_t)b * a.ws_stride, n, k);
  __shared__ double sm[64];
  __shared__ double2 G[MODE_KMAX * MODE_KMAX], Zs[MODE_KMAX * MODE_KMAX],
      S[MODE_KMAX * MODE_KMAX], th[MODE_KMAX];
  __shared__ int order[MODE_KMAX], s_flag;
  __shared__ double s_sigma, s_res[MODE_KMAX];
  __shared__ double2 s_alpha, s_den;

  // sigma = max(eps)
  double mx = -INFINITY;
  for (int i = threadIdx.x; i < n; i += blockDim.x) mx = fmax(mx, eps[i]);
  for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = mx;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = sm[0];
    for (int q = 1; q < (int)(blockDim.x >> 5); ++q) t = fmax(t, sm[q]);
    s_sigma = t;
  }
  __syncthreads();
  const double sigma = s_sigma;

  // Factor B = M - u v^T (thread 0): u = [gamma, 0.., beta], v = [1, 0.., alpha/gamma]
  if (threadIdx.x == 0) {
    int flag = 0;
    auto diag = [&](int i) {
      return make_double2(eps[i] - sigma - a.up[i].x - a.dn[i].x, -a.up[i].y - a.dn[i].y);
    };
    const double2 alpha = a.dn[0];     // M[0][n-1]
    const double2 beta = a.up[n - 1];  // M[n-1][0]
    double2 d0 = diag(0);
    double2 gamma = cabsd(d0) > 0 ? make_double2(-d0.x, -d0.y) : make_double2(1.0, 0.0);
    // working rows: diagonal bd (current row), super sup (current row)
    double2 bd = csub(d0, gamma);
    double2 sup = a.up[0];
    for (int i = 0; i + 1 < n; ++i) {
      const double2 sub = a.dn[i + 1];  // M[i+1][i]
      double2 nd = diag(i + 1);
      if (i + 1 == n - 1) nd = csub(nd, cdivd(cmul(alpha, beta), gamma));
      const double2 nsup = (i + 2 < n) ? a.up[i + 1] : make_double2(0.0, 0.0);
      if (cabs2(bd) >= cabs2(sub)) {
        if (cabs2(bd) == 0.0) { flag = 1; bd = make_double2(1e-300, 0.0); }
        const double2 l = cdivd(sub, bd);
        w.piv[i] = 0;
        w.lm[i] = l;
        w.u0[i] = bd;
        w.u1[i] = sup;
        w.u2[i] = make_double2(0.0, 0.0);
        bd = csub(nd, cmul(l, sup));
        sup = nsup;
      } else {
        const double2 l = cdivd(bd, sub);
        w.piv[i] = 1;
        w.lm[i] = l;
        w.u0[i] = sub;
        w.u1[i] = nd;
        w.u2[i] = nsup;
        const double2 nbd = csub(sup, cmul(l, nd));
        sup = make_double2(-(l.x * nsup.x - l.y * nsup.y), -(l.x * nsup.y + l.y * nsup.x));
        bd = nbd;
      }
    }
    if (cabs2(bd) == 0.0) { flag = 1; bd = make_double2(1e-300, 0.0); }
    w.u0[n - 1] = bd;
    // B z = u
    for (int i = 0; i < n; ++i) w.z[i] = make_double2(0.0, 0.0);
    w.z[0] = gamma;
    w.z[n - 1] = cadd(w.z[n - 1], beta);
    lu_solve(w, n, w.z);
    const double2 ag = cdivd(alpha, gamma);
    const double2 vz = cadd(w.z[0], cmul(ag, w.z[n - 1]));
    s_den = cadd(make_double2(1.0, 0.0), vz);
    s_alpha = ag;
    if (cabs2(s_den) == 0.0) flag = 1;
    s_flag = flag;
  }
  __syncthreads();
  if (s_flag) {
    if (threadIdx.x == 0) { a.status[b] = 2; a.iters[b] = 0; }
    return;
  }

  // start vectors
  double2 *Q = w.Q, *Y = w.Y;
  for (int j = 0; j < k; ++j)
    for (int i = threadIdx.x; i < n; i += blockDim.x) Q[(size_t)j * n + i] = hash_c(i, j + 977 * b);
  __syncthreads();
  mgs(Q, n, k, sm);

  if (threadIdx.x == 0) {
    for (int j = 0; j < k; ++j) {
      order[j] = j;
      th[j] = make_double2(0.0, 0.0);
      for (int l = 0; l < k; ++l) S[l * k + j] = make_double2(l == j ? 1.0 : 0.0, 0.0);
    }
  }
  __syncthreads();
  int it = 0, conv = 0;
  for (it = 1; it <= a.max_iters; ++it) {
    // Y = M^{-1} Q (one column per thread, Sherman-Morrison correction)
    if ((int)threadIdx.x < k) {
      const int j = threadIdx.x;
      double2* y = Y + (size_t)j * n;
      const double2* q = Q + (size_t)j * n;
      for (int i = 0; i < n; ++i) y[i] = q[i];
      lu_solve(w, n, y);
      const double2 vy = cadd(y[0], cmul(s_alpha, y[n - 1]));
      const double2 f = cdivd(vy, s_den);
      for (int i = 0; i < n; ++i) y[i] = csub(y[i], cmul(f, w.z[i]));
    }
    __syncthreads();
    if (!mgs(Y, n, k, sm)) break;
    double2* t = Q;
    Q = Y;
    Y = t;

    // AQ = A Q
    for (size_t e = threadIdx.x; e < (size_t)k * n; e += blockDim.x) {
      const int j = (int)(e / n), i = (int)(e % n);
      const double2* q = Q + (size_t)j * n;
      const int ip = i + 1 == n ? 0 : i + 1, im = i == 0 ? n - 1 : i - 1;
      double2 v = cscale(q[i], eps[i]);
      v = cfma(a.up[i], csub(q[ip], q[i]), v);
      v = cfma(a.dn[i], csub(q[im], q[i]), v);
      w.AQ[e] = v;
    }
    __syncthreads();
    // G = Q^H A Q
    for (int r = 0; r < k; ++r)
      for (int c = 0; c < k; ++c) {
        const double2 g = block_cdot(Q + (size_t)r * n, w.AQ + (size_t)c * n, n, sm);
        if (threadIdx.x == 0) G[r * k + c] = g;
      }
    if (threadIdx.x == 0) {
      const int rc = small_eig(k, G, Zs, th, S);
      s_flag = rc;
      // order Ritz values by distance to sigma (insertion sort, stable)
      for (int j = 0; j < k; ++j) order[j] = j;
      for (int j = 1; j < k; ++j) {
        const int o = order[j];
        const double dj = cabs2(make_double2(th[o].x - sigma, th[o].y));
        int q = j - 1;
        while (q >= 0 && cabs2(make_double2(th[order[q]].x - sigma, th[order[q]].y)) > dj) {
          order[q + 1] = order[q];
          --q;
        }
        order[q + 1] = o;
      }
    }
    __syncthreads();
    if (s_flag) break;
    // Ritz residuals of the m leading pairs: r = (AQ - theta Q) s
    for (int j = 0; j < m; ++j) {
      const int o = order[j];
      double v[2] = {0.0, 0.0};
      for (int i = threadIdx.x; i < n; i += blockDim.x) {
        double2 x = make_double2(0.0, 0.0), r = make_double2(0.0, 0.0);
        for (int l = 0; l < k; ++l) {
          const double2 s = S[l * k + o];
          x = cfma(Q[(size_t)l * n + i], s, x);
          r = cfma(w.AQ[(size_t)l * n + i], s, r);
        }
        r = csub(r, cmul(th[o], x));
        v[0] += cabs2(r);
        v[1] += cabs2(x);
      }
      block_sum<2>(v, sm);
      if (threadIdx.x == 0) s_res[j] = v[1] > 0 ? sqrt(v[0] / v[1]) : INFINITY;
      __syncthreads();
    }
    if (threadIdx.x == 0) {
      int ok = 1;
      for (int j = 0; j < m; ++j) ok &= s_res[j] <= a.tol * fmax(1.0, fabs(sigma));
      s_flag = ok;
    }
    __syncthreads();
    conv = s_flag;
    __syncthreads();
    if (conv) break;
  }

  // outputs (the last Ritz pairs, converged or not)
  for (int j = 0; j < m; ++j) {
    const int o = order[j];
    double2* out = a.vecs + ((size_t)b * m + j) * n;
    double v[2] = {0.0, 0.0};
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
      double2 x = make_double2(0.0, 0.0);
      for (int l = 0; l < k; ++l) x = cfma(Q[(size_t)l * n + i], S[l * k + o], x);
      out[i] = x;
      v[0] += cabs2(x);
    }
    block_sum<2>(v, sm);
    __shared__ double s_nrm;
    if (threadIdx.x == 0) s_nrm = v[0];
    __syncthreads();
    // largest-magnitude entry (first index on ties)
    double best = -1.0;
    int bi = 0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
      const double t = cabs2(out[i]);
      if (t > best) { best = t; bi = i; }
    }
    for (int o2 = 16; o2 > 0; o2 >>= 1) {
      const double ob = __shfl_xor_sync(0xffffffffu, best, o2);
      const int oi = __shfl_xor_sync(0xffffffffu, bi, o2);
      if (ob > best || (ob == best && oi < bi)) { best = ob; bi = oi; }
    }
    __shared__ double s_best[MODE_THREADS / 32];
    __shared__ int s_bi[MODE_THREADS / 32];
    __shared__ double2 s_ph;
    if ((threadIdx.x & 31) == 0) { s_best[threadIdx.x >> 5] = best; s_bi[threadIdx.x >> 5] = bi; }
    __syncthreads();
    if (threadIdx.x == 0) {
      for (int q = 1; q < (int)(blockDim.x >> 5); ++q)
        if (s_best[q] > best || (s_best[q] == best && s_bi[q] < bi)) { best = s_best[q]; bi = s_bi[q]; }
      const double2 p = out[bi];
      const double ap = cabsd(p);
      const double sc = 1.0 / sqrt(s_nrm);
      s_ph = ap > 0 ? make_double2(p.x / ap * sc, -p.y / ap * sc) : make_double2(sc, 0.0);
      a.vals[(size_t)b * m + j] = th[o];
    }
    __syncthreads();
    const double2 ph = s_ph;
    for (int i = threadIdx.x; i < n; i += blockDim.x) out[i] = cmul(out[i], ph);
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    a.iters[b] = it > a.max_iters ? a.max_iters : it;
    a.status[b] = conv ? 0 : 1;
  }
}

static int mode_k(int n, int m) {
  int k = std::max(m + 4, 2 * m);
  k = std::min(k, MODE_KMAX);
  return std::min(k, n);
}

}  // namespace cev

using namespace cev;

extern "C" {

static size_t mode_table_bytes(int n) {
  return (2 * sizeof(double2) * (size_t)n + 255) & ~(size_t)255;
}

size_t cev_mode_workspace_size(int batch, int n, int m) {
  if (batch < 1 || n < 3 || m < 1 || m > n || m > MODE_KMAX) return 0;
  return mode_table_bytes(n) + (size_t)batch * mode_ws_stride(n, mode_k(n, m));
}

int cev_mode_solve(int batch, int n, const double* eps, double omega, double dL, int npml, int m,
                   double tol, int max_iters, void* vals, void* vecs, int* iters, int* status,
                   void* ws, size_t ws_bytes, cudaStream_t s) {
  CEV_REQUIRE(batch >= 1 && n >= 3, "bad sizes batch=%d n=%d (n >= 3)", batch, n);
  CEV_REQUIRE(m >= 1 && m <= n && m <= MODE_KMAX, "m=%d must be in [1, min(n, %d)]", m, MODE_KMAX);
  CEV_REQUIRE(npml >= 0 && 2 * npml <= n, "npml=%d out of range for n=%d", npml, n);
  CEV_REQUIRE(omega > 0 && dL > 0 && tol > 0 && max_iters >= 1, "bad omega/dL/tol/max_iters");
  CEV_REQUIRE(eps && vals && vecs && iters && status && ws, "NULL argument");
  CEV_REQUIRE(((uintptr_t)ws & 255) == 0, "workspace must be 256-byte aligned");
  const size_t need = cev_mode_workspace_size(batch, n, m);
  CEV_REQUIRE(ws_bytes >= need, "workspace too small: need %zu bytes, got %zu", need, ws_bytes);
  const std::vector<zd> sf = sfactor(true, omega, dL, n, npml);
  const std::vector<zd> sb = sfactor(false, omega, dL, n, npml);
  const double C_0 = 1.0 / std::sqrt(EPSILON_0 * MU_0);  // ceviche/constants.py
  const double k0dl = omega / C_0 * dL, f = 1.0 / (k0dl * k0dl);
  std::vector<double2> tab(2 * (size_t)n);
  for (int i = 0; i < n; ++i) {
    const zd up = f / (sf[i] * sb[(i + 1) % n]);
    const zd dn = f / (sf[i] * sb[i]);
    tab[i] = make_double2(up.real(), up.imag());
    tab[n + i] = make_double2(dn.real(), dn.imag());
  }
  char* w = (char*)ws;
  double2* dtab = (double2*)w;
  CEV_CUDA(cudaMemcpyAsync(dtab, tab.data(), sizeof(double2) * 2 * n, cudaMemcpyHostToDevice, s));
  const size_t off = mode_table_bytes(n);
  ModeArgs a;
  a.n = n;
  a.m = m;
  a.k = mode_k(n, m);
  a.max_iters = max_iters;
  a.tol = tol;
  a.eps = eps;
  a.up = dtab;
  a.dn = dtab + n;
  a.vals = (double2*)vals;
  a.vecs = (double2*)vecs;
  a.iters = iters;
  a.status = status;
  a.ws = w + off;
  a.ws_stride = mode_ws_stride(n, a.k);
  k_modes<<<batch, MODE_THREADS, 0, s>>>(a);
  CEV_CHECK_LAUNCH("k_modes");
  // the host table must outlive the copy: wait for it before returning
  CEV_CUDA(cudaStreamSynchronize(s));
  return CEV_OK;
}

int cev_dense_eig(int k, const double* h, double* w, double* v) {
  CEV_REQUIRE(k >= 1 && k <= MODE_KMAX, "k=%d must be in [1, %d]", k, MODE_KMAX);
  CEV_REQUIRE(h && w && v, "NULL argument");
  std::vector<double2> H(k * k), Z(k * k), V(k * k), W(k);
  for (int i = 0; i < k * k; ++i) H[i] = make_double2(h[2 * i], h[2 * i + 1]);
  const int rc = small_eig(k, H.data(), Z.data(), W.data(), V.data());
  for (int i = 0; i < k; ++i) { w[2 * i] = W[i].x; w[2 * i + 1] = W[i].y; }
  for (int i = 0; i < k * k; ++i) { v[2 * i] = V[i].x; v[2 * i + 1] = V[i].y; }
  if (rc != 0) {
    set_error("QR iteration did not converge");
    return CEV_ERR_NUMERIC;
  }
  return CEV_OK;
}

}  // extern "C"
