// Matrix-free 5-point SC-PML Yee stencil of ceviche's FDFD system matrices.
//
// Along one axis (x = axis 0, index i; the same along y with index j) both
// polarisations have the form
//     (A_axis u)_i = P_i [ W_{i+1/2} (R_{i+1} f+ u_{i+1} - R_i u_i)
//                         - W_{i-1/2} (R_i u_i - R_{i-1} f- u_{i-1}) ]
// with the periodic wrap carrying the Bloch phasor f+ = ph at i = N-1 and
// f- = conj(ph) at i = 0 (ceviche/derivatives.py:94-124):
//   Ez: P = 1/s_f, W_{i+1/2} = 1/s_b[i+1], R = 1, overall sign -1
//       (-(1/mu0) Dxf Dxb, ceviche/fdfd.py:174-175)
//   Hz: P = 1/s_b, W_{i+1/2} = (1/s_f[i]) * d[i], R = 1, sign +1, where d is
//       1/(eps_yy + 1e-5) along x and 1/(eps_xx + 1e-5) along y
//       ((1/eps0) Dxb diag(d) Dxf, ceviche/fdfd.py:211-226)
// and A^T swaps P and R and conjugates the phasor.  The host folds P, W, R
// and the phasors into four complex coefficients per row (Coef):
//   cm = P_i W_{i-1/2} R_{i-1} f-,  cp = P_i W_{i+1/2} R_{i+1} f+,
//   am = P_i W_{i-1/2} R_i,         ap = P_i W_{i+1/2} R_i
// so one row costs   cm dm u_{i-1} + cp dp u_{i+1} - (am dm + ap dp) u_i
// with dm, dp the 2D factors (1 for Ez).  The system is non-dimensionalised:
// rows are scaled by mu0 dL^2 (Ez) or eps0 dL^2 (Hz), so the coefficients are
// O(1) and the diagonal is -k^2 eps (Ez) or +k^2 (Hz), k^2 = eps0 mu0 w^2 dL^2.
#pragma once

#include <type_traits>

#include "common.cuh"

namespace cev {

template <typename R>
struct Coef {
  Cplx<R> cm, cp, am, ap;
};

// Ez/Hz selector
enum { POL_EZ = 0, POL_HZ = 1 };

template <typename R>
__device__ __forceinline__ R hz_d(R a, R b) {
  // 1 / ((a + b)/2 + 1e-5), the ordering of fdfd.py:203-204, 214-215
  return R(1) / (R(0.5) * (a + b) + R(1e-5));
}

// Complex permittivity (lossy media): the same factor in complex arithmetic.
__device__ __forceinline__ float2 hz_d(float2 a, float2 b) {
  const float2 den = make_float2(0.5f * (a.x + b.x) + 1e-5f, 0.5f * (a.y + b.y));
  const float q = 1.0f / (den.x * den.x + den.y * den.y);
  return make_float2(den.x * q, -den.y * q);
}
__device__ __forceinline__ double2 hz_d(double2 a, double2 b) {
  const double2 den = make_double2(0.5 * (a.x + b.x) + 1e-5, 0.5 * (a.y + b.y));
  const double q = 1.0 / (den.x * den.x + den.y * den.y);
  return make_double2(den.x * q, -den.y * q);
}

// v * e for a real or complex permittivity-derived factor e
template <typename C, typename R>
__device__ __forceinline__ C emul(C v, R e) { return cscale(v, e); }
__device__ __forceinline__ float2 emul(float2 v, float2 e) { return cmul(v, e); }
__device__ __forceinline__ double2 emul(double2 v, double2 e) { return cmul(v, e); }

// Loads of the stencil input: the read-only path (the input is not written
// during the launch), or with CG = true through L2 only (ld.global.cg), for
// kernels that read vectors other blocks wrote earlier in the same launch.
template <bool CG, typename T>
__device__ __forceinline__ T ldx(const T* p) {
  if constexpr (CG)
    return __ldcg(p);
  else
    return __ldg(p);
}

// Input conversion of the stencil: a complex64 vector may feed the FP64
// stencil (the exact operator applied to a complex64 preconditioned vector).
template <typename C, typename X>
struct CvtIn;
template <typename C>
struct CvtIn<C, C> {
  static __device__ __forceinline__ C go(C v) { return v; }
};
template <>
struct CvtIn<double2, float2> {
  static __device__ __forceinline__ double2 go(float2 v) { return to_d(v); }
};

// Sliding-window row iterator over one column j for rows [i0, i1).
// Calls ep(i, Au, u_c) for every row with Au the stencil (without output
// scaling) and u_c the centre value.  E is the permittivity element: R (real
// eps) or Cplx<R> (complex eps, lossy media).
template <typename R, int POL, typename Epi, bool CG = false, typename E = R,
          typename X = Cplx<R>>
__device__ __forceinline__ void stencil_column(int nx, int ny, int j, int i0, int i1,
                                               const X* x,
                                               const E* __restrict__ eps,
                                               const Coef<R>* __restrict__ cx,
                                               const Coef<R>& cyj, R k2, Epi& ep) {
  using C = Cplx<R>;
  const int jm = (j == 0) ? ny - 1 : j - 1;
  const int jp = (j == ny - 1) ? 0 : j + 1;
  const int jmm = (jm == 0) ? ny - 1 : jm - 1;
  const int im0 = (i0 == 0) ? nx - 1 : i0 - 1;
  C u_m = CvtIn<C, X>::go(ldx<CG>(x + (size_t)im0 * ny + j));
  C u_c = CvtIn<C, X>::go(ldx<CG>(x + (size_t)i0 * ny + j));
  // Hz: eps window along i (for d_yy) ; Ez: unused
  E e_m{}, dyy_m{};
  if (POL == POL_HZ) {
    const int imm = (im0 == 0) ? nx - 1 : im0 - 1;
    e_m = eps[(size_t)im0 * ny + j];
    dyy_m = hz_d(e_m, eps[(size_t)imm * ny + j]);
  }
  const C ym_c = cyj.cm, yp_c = cyj.cp, ym_a = cyj.am, yp_a = cyj.ap;
  for (int i = i0; i < i1; ++i) {
    const int ip = (i == nx - 1) ? 0 : i + 1;
    const size_t row = (size_t)i * ny;
    const C u_p = CvtIn<C, X>::go(ldx<CG>(x + (size_t)ip * ny + j));
    const C u_l = CvtIn<C, X>::go(ldx<CG>(x + row + jm));
    const C u_r = CvtIn<C, X>::go(ldx<CG>(x + row + jp));
    const Coef<R> c = cx[i];
    C acc;
    if (POL == POL_EZ) {
      const E e = eps[row + j];
      // x part
      C d0 = cadd(c.am, c.ap);
      d0 = cadd(d0, cadd(ym_a, yp_a));
      acc = cmul(c.cm, u_m);
      acc = cfma(c.cp, u_p, acc);
      acc = cfma(ym_c, u_l, acc);
      acc = cfma(yp_c, u_r, acc);
      acc = csub(acc, cmul(d0, u_c));
      // A' u = -(...) - k2 eps u
      if constexpr (std::is_same<E, R>::value) {
        acc.x = -acc.x - k2 * e * u_c.x;
        acc.y = -acc.y - k2 * e * u_c.y;
      } else {
        const C eu = cmul(e, u_c);
        acc.x = -acc.x - k2 * eu.x;
        acc.y = -acc.y - k2 * eu.y;
      }
    } else {
      const E e = eps[row + j];
      const E el = eps[row + jm];
      const E ell = eps[row + jmm];
      const E dyy_p = hz_d(e, e_m);     // d_yy[i]   (edge i+1/2 along x)
      const E dxx_p = hz_d(e, el);      // d_xx[i,j] (edge j+1/2 along y)
      const E dxx_m = hz_d(el, ell);    // d_xx[i,j-1]
      C d0;
      if constexpr (std::is_same<E, R>::value) {
        d0.x = c.am.x * dyy_m + c.ap.x * dyy_p + ym_a.x * dxx_m + yp_a.x * dxx_p;
        d0.y = c.am.y * dyy_m + c.ap.y * dyy_p + ym_a.y * dxx_m + yp_a.y * dxx_p;
      } else {
        d0 = cadd(cadd(emul(c.am, dyy_m), emul(c.ap, dyy_p)),
                  cadd(emul(ym_a, dxx_m), emul(yp_a, dxx_p)));
      }
      acc = emul(cmul(c.cm, u_m), dyy_m);
      acc = cadd(acc, emul(cmul(c.cp, u_p), dyy_p));
      acc = cadd(acc, emul(cmul(ym_c, u_l), dxx_m));
      acc = cadd(acc, emul(cmul(yp_c, u_r), dxx_p));
      acc = csub(acc, cmul(d0, u_c));
      acc.x += k2 * u_c.x;
      acc.y += k2 * u_c.y;
      e_m = e;
      dyy_m = dyy_p;
    }
    ep(i, acc, u_c);
    u_m = u_c;
    u_c = u_p;
  }
}

}  // namespace cev
