// Eigen-decomposition of a small dense complex matrix (k <= 32), host and
// device: Householder reduction to Hessenberg form, implicit single-shift QR
// with Wilkinson shifts and deflation to the complex Schur form T = Z^H H Z,
// then eigenvectors of T by back substitution, mapped back by Z.  FP64.
// Used by the mode solver's Rayleigh-Ritz step; one thread runs it.
#pragma once

#include "common.cuh"

namespace cev {

__host__ __device__ inline double cabs2(double2 a) { return a.x * a.x + a.y * a.y; }
__host__ __device__ inline double cabsd(double2 a) { return hypot(a.x, a.y); }
__host__ __device__ inline double2 cdivd(double2 a, double2 b) {
  // Smith's algorithm (avoids overflow in |b|^2)
  if (fabs(b.x) >= fabs(b.y)) {
    const double r = b.y / b.x, d = b.x + b.y * r;
    return make_double2((a.x + a.y * r) / d, (a.y - a.x * r) / d);
  }
  const double r = b.x / b.y, d = b.y + b.x * r;
  return make_double2((a.x * r + a.y) / d, (a.y * r - a.x) / d);
}
__host__ __device__ inline double2 csqrtd(double2 a) {
  const double r = cabsd(a);
  if (r == 0.0) return make_double2(0.0, 0.0);
  double re = sqrt(0.5 * (r + fabs(a.x))), im = a.y / (2.0 * re);
  if (a.x < 0) {
    const double t = re;
    re = fabs(im);
    im = a.y < 0 ? -t : t;
  }
  return make_double2(re, im);
}

// Row-major k x k.  On return w[j] are the eigenvalues and column j of V
// (V[i*k + j]) the matching eigenvector (unit 2-norm).  H is destroyed; Z is
// k x k scratch.  Returns 0, or -1 if QR did not converge in 60 k sweeps.
__host__ __device__ inline int small_eig(int k, double2* H, double2* Z, double2* w, double2* V) {
  const double2 zero = make_double2(0.0, 0.0), one = make_double2(1.0, 0.0);
  for (int i = 0; i < k; ++i)
    for (int j = 0; j < k; ++j) Z[i * k + j] = i == j ? one : zero;
  double hnorm = 0.0;
  for (int i = 0; i < k * k; ++i) hnorm = fmax(hnorm, cabsd(H[i]));
  if (hnorm == 0.0) hnorm = 1.0;
  const double eps = 2.220446049250313e-16;

  // Householder reduction to Hessenberg form; Z accumulates the reflectors.
  for (int c = 0; c + 2 < k; ++c) {
    double xn = 0.0;
    for (int i = c + 1; i < k; ++i) xn += cabs2(H[i * k + c]);
    xn = sqrt(xn);
    if (xn == 0.0) continue;
    const double2 x0 = H[(c + 1) * k + c];
    const double a0 = cabsd(x0);
    const double2 ph = a0 > 0 ? cscale(x0, 1.0 / a0) : one;
    const double2 alpha = cscale(ph, -xn);  // P x = alpha e1
    double2 v[32];
    double vn = 0.0;
    for (int i = c + 1; i < k; ++i) {
      v[i] = H[i * k + c];
      if (i == c + 1) v[i] = csub(v[i], alpha);
      vn += cabs2(v[i]);
    }
    if (vn == 0.0) continue;
    const double f = 2.0 / vn;  // P = I - f v v^H
    for (int j = 0; j < k; ++j) {  // H <- P H (rows c+1..k-1)
      double2 s = zero;
      for (int i = c + 1; i < k; ++i) s = cfma(cconj(v[i]), H[i * k + j], s);
      s = cscale(s, f);
      for (int i = c + 1; i < k; ++i) H[i * k + j] = csub(H[i * k + j], cmul(v[i], s));
    }
    for (int i = 0; i < k; ++i) {  // H <- H P, Z <- Z P (columns c+1..k-1)
      double2 s = zero, t = zero;
      for (int j = c + 1; j < k; ++j) {
        s = cfma(H[i * k + j], v[j], s);
        t = cfma(Z[i * k + j], v[j], t);
      }
      s = cscale(s, f);
      t = cscale(t, f);
      for (int j = c + 1; j < k; ++j) {
        H[i * k + j] = csub(H[i * k + j], cmul(s, cconj(v[j])));
        Z[i * k + j] = csub(Z[i * k + j], cmul(t, cconj(v[j])));
      }
    }
    for (int i = c + 2; i < k; ++i) H[i * k + c] = zero;
  }

  // Shifted QR on the Hessenberg matrix, Givens rotations G = [c s; -s* c].
  int hi = k - 1, it = 0, total = 0;
  while (hi > 0) {
    if (++total > 60 * k) return -1;
    int l = hi;
    for (; l > 0; --l) {
      const double sub = cabsd(H[l * k + l - 1]);
      double scale = cabsd(H[l * k + l]) + cabsd(H[(l - 1) * k + l - 1]);
      if (scale == 0.0) scale = hnorm;
      if (sub <= eps * scale) {
        H[l * k + l - 1] = zero;
        break;
      }
    }
    if (l == hi) {
      --hi;
      it = 0;
      continue;
    }
    ++it;
    // Wilkinson shift: eigenvalue of the trailing 2x2 closest to H[hi][hi]
    const double2 a = H[(hi - 1) * k + hi - 1], b = H[(hi - 1) * k + hi];
    const double2 c = H[hi * k + hi - 1], d = H[hi * k + hi];
    double2 mu;
    if (it % 11 == 10) {  // exceptional shift
      mu = cadd(d, make_double2(cabsd(c), 0.0));
    } else {
      const double2 half = cscale(csub(a, d), 0.5);
      const double2 disc = csqrtd(cadd(cmul(half, half), cmul(b, c)));
      const double2 m0 = cscale(cadd(a, d), 0.5);
      const double2 e1 = cadd(m0, disc), e2 = csub(m0, disc);
      mu = cabs2(csub(e1, d)) <= cabs2(csub(e2, d)) ? e1 : e2;
    }
    double2 x = csub(H[l * k + l], mu), y = H[(l + 1) * k + l];
    for (int i = l; i < hi; ++i) {
      if (i > l) {
        x = H[i * k + i - 1];
        y = H[(i + 1) * k + i - 1];
      }
      const double ax = cabsd(x), r = hypot(ax, cabsd(y));
      double cr;
      double2 s;
      if (r == 0.0) {
        cr = 1.0;
        s = zero;
      } else if (ax == 0.0) {
        cr = 0.0;
        s = cscale(cconj(y), 1.0 / cabsd(y));
      } else {
        cr = ax / r;
        s = cscale(cmul(cscale(x, 1.0 / ax), cconj(y)), 1.0 / r);
      }
      // rows i, i+1 (left multiply by G)
      for (int j = (i > l ? i - 1 : l); j < k; ++j) {
        const double2 p = H[i * k + j], q = H[(i + 1) * k + j];
        H[i * k + j] = cadd(cscale(p, cr), cmul(s, q));
        H[(i + 1) * k + j] = csub(cscale(q, cr), cmul(cconj(s), p));
      }
      if (i > l) H[(i + 1) * k + i - 1] = zero;
      // columns i, i+1 (right multiply by G^H), and Z
      const int rmax = i + 2 < hi ? i + 2 : hi;
      for (int r2 = 0; r2 <= rmax; ++r2) {
        const double2 p = H[r2 * k + i], q = H[r2 * k + i + 1];
        H[r2 * k + i] = cadd(cscale(p, cr), cmul(cconj(s), q));
        H[r2 * k + i + 1] = csub(cscale(q, cr), cmul(s, p));
      }
      for (int r2 = 0; r2 < k; ++r2) {
        const double2 p = Z[r2 * k + i], q = Z[r2 * k + i + 1];
        Z[r2 * k + i] = cadd(cscale(p, cr), cmul(cconj(s), q));
        Z[r2 * k + i + 1] = csub(cscale(q, cr), cmul(s, p));
      }
    }
  }

  // Eigenvectors of the triangular T = H, then V = Z y.
  for (int j = 0; j < k; ++j) w[j] = H[j * k + j];
  double2 y[32];
  for (int j = 0; j < k; ++j) {
    for (int i = 0; i < k; ++i) y[i] = zero;
    y[j] = one;
    for (int i = j - 1; i >= 0; --i) {
      double2 s = zero;
      for (int l2 = i + 1; l2 <= j; ++l2) s = cfma(H[i * k + l2], y[l2], s);
      double2 den = csub(H[i * k + i], w[j]);
      if (cabsd(den) < eps * hnorm) den = make_double2(eps * hnorm, 0.0);
      y[i] = cdivd(make_double2(-s.x, -s.y), den);
    }
    double nrm = 0.0;
    for (int i = 0; i < k; ++i) {
      double2 s = zero;
      for (int l2 = 0; l2 <= j; ++l2) s = cfma(Z[i * k + l2], y[l2], s);
      V[i * k + j] = s;
      nrm += cabs2(s);
    }
    nrm = nrm > 0 ? 1.0 / sqrt(nrm) : 1.0;
    for (int i = 0; i < k; ++i) V[i * k + j] = cscale(V[i * k + j], nrm);
  }
  return 0;
}

}  // namespace cev
