// Host-side workspace setup shared by both precisions: grid constants, spin
// matrices, Clebsch-Gordan / 6j tables, tensor-path activation and the DDI
// convolution geometry.  Everything here runs once in sbec_ws_create.
#pragma once

#include <complex>
#include <string>
#include <vector>

#include "sbec.h"

namespace sbec {

struct SbecError {
  sbec_status status;
  std::string msg;
};

[[noreturn]] inline void fail(sbec_status s, const std::string& m) { throw SbecError{s, m}; }

struct Setup {
  sbec_config cfg;
  int ndim = 1;
  int n[3] = {1, 1, 1};
  double L[3] = {1, 1, 1};
  long long N = 1;     // spatial points
  bool pow2 = true;    // every axis a power of two (else the general path with Bluestein axes)
  int F = 0, D = 1;
  double dx[3] = {1, 1, 1};
  double dV = 1;
  double kmult[3] = {0, 0, 0};  // k(m) = fftfreq index * kmult (src/grid.jl:12-17)
  // effective interactions after tensor activation (src/initialization.jl:164-185)
  double c0 = 0, c1 = 0, c_lhy = 0, c2 = 0;
  bool tensor = false;
  std::vector<int> chS;          // active channels S
  std::vector<double> chG;       // g_S
  std::vector<double> G;         // (4F+1)*D*D regrouped h-build coefficients
  double bound_coef = 0;         // sum_S |g_S| (2S+1)/(2F+1)
  // pair amplitudes for the tensor energy: rows (a_idx, c1, c2), cg, and g per a_idx
  std::vector<int> pair_a, pair_c1, pair_c2;
  std::vector<double> pair_cg, gA;
  // spin tables
  std::vector<std::complex<double>> FyV, FyVt;  // D*D row-major
  std::vector<double> fp, m;
  // Raman coupling H_R = delta Fz + (Omega/2)(e^{ik.r} F+ + h.c.) (src/raman.jl:1-31)
  bool raman = false;
  double raman_omega = 0, raman_delta = 0, raman_k[3] = {0, 0, 0};
  double x0[3] = {0, 0, 0};  // first grid coordinate per axis, -L/2 + dx/2 (src/grid.jl:2-7)
  // density-dependent losses: rate_c = gamma_m + L3 per component (src/losses.jl:25-97)
  bool loss = false;
  std::vector<double> loss_rates;
  // DDI
  bool ddi = false, secular = false, padded = false;
  double c_dd = 0;
  // convolution grids: [0] periodic (n), [1] padded (2n)
  int conv_M[2][3] = {{1, 1, 1}, {1, 1, 1}};
  double conv_kmult[2][3] = {{0, 0, 0}, {0, 0, 0}};
};

Setup build_setup(const sbec_config& cfg);

// Exposed for tests through the C ABI helpers.
double wigner_3j(int j1, int j2, int j3, int m1, int m2, int m3);
double clebsch_gordan(int j1, int m1, int j2, int m2, int J, int M);
double wigner_6j(int j1, int j2, int j3, int j4, int j5, int j6);

}  // namespace sbec
