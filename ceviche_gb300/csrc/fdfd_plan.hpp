// FDFD plan: per-problem SC-PML coefficient tables on the device.
#pragma once

#include <complex>
#include <vector>

#include "stencil.cuh"

namespace cev {

using zd = std::complex<double>;

// SI constants, ceviche/constants.py:7-11
constexpr double EPSILON_0 = 8.85418782e-12;
constexpr double MU_0 = 1.25663706e-6;

// 1D stretch profile s(i) of ceviche/derivatives.py:173-216 ('f': offset 0.5,
// 'b': offset 1); returns s itself (not 1/s).
std::vector<zd> sfactor(bool forward, double omega, double dL, int N, int npml);

// Row coefficients (cm, cp, am, ap) along one axis, see stencil.cuh.
void axis_tables(int pol, int N, int npml, double dL, double omega, double phase, bool transpose,
                 std::vector<Coef<double>>& out);

struct FieldTab {
  // per axis, per problem: 1/s_f and 1/s_b (complex128)
  double2* sfx = nullptr;
  double2* sbx = nullptr;
  double2* sfy = nullptr;
  double2* sby = nullptr;
};

}  // namespace cev

struct cev_fdfd_plan_s {
  int pol = 0, nx = 0, ny = 0, batch = 0;
  int eps_complex = 0;  // eps arrays are interleaved complex (lossy media)
  int npml_x = 0, npml_y = 0;
  double dL = 0, scale = 1, bloch_x = 0, bloch_y = 0;
  std::vector<double> omega;
  int device = 0;
  // [transpose] -> [batch][n]
  cev::Coef<double>* cx64[2] = {nullptr, nullptr};
  cev::Coef<double>* cy64[2] = {nullptr, nullptr};
  cev::Coef<float>* cx32[2] = {nullptr, nullptr};
  cev::Coef<float>* cy32[2] = {nullptr, nullptr};
  double* k2_64 = nullptr;  // [batch]
  float* k2_32 = nullptr;
  double* omega_d = nullptr;  // [batch]
  cev::FieldTab ft;
  double2 phx, phy;  // Bloch phasors exp(1j*bloch)
  int mf_nsb = -1;      // multi-frequency plan: sidebands on each side (-1: not one)
  double omega_mod = 0;
  size_t n() const { return (size_t)nx * ny; }
};
