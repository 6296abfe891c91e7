// Host-side setup: grid constants, Clebsch-Gordan and Wigner 6j symbols
// (log-space Racah formulas, src/clebsch_gordan.jl:1-180), channel couplings and
// tensor-path activation (src/interactions.jl:123-155, src/initialization.jl:164-185),
// spin matrices and the Fy eigen-decomposition (src/spin_matrices.jl:1-50).
#include "sbec_setup.h"

#include <algorithm>
#include <cmath>
#include <map>
#include <tuple>

namespace sbec {

namespace {

double log_factorial(int n) {
  if (n < 0) return -INFINITY;
  double s = 0.0;
  for (int i = 2; i <= n; ++i) s += std::log((double)i);
  return s;
}

double log_triangle(int a, int b, int c) {
  const int ab = a + b - c, ac = a - b + c, bc = -a + b + c;
  if (ab < 0 || ac < 0 || bc < 0) return -INFINITY;
  return log_factorial(ab) + log_factorial(ac) + log_factorial(bc) - log_factorial(a + b + c + 1);
}

bool is_pow2(int n) { return n >= 2 && (n & (n - 1)) == 0; }

// Real symmetric cyclic Jacobi eigen-solver (n <= 26); returns eigenvalues and
// column eigenvectors in `vec` (row-major n*n).
void jacobi_sym(std::vector<double>& a, int n, std::vector<double>& val, std::vector<double>& vec) {
  vec.assign((size_t)n * n, 0.0);
  for (int i = 0; i < n; ++i) vec[(size_t)i * n + i] = 1.0;
  for (int sweep = 0; sweep < 100; ++sweep) {
    double off = 0.0;
    for (int p = 0; p < n; ++p)
      for (int q = p + 1; q < n; ++q) off += a[(size_t)p * n + q] * a[(size_t)p * n + q];
    if (off < 1e-300) break;
    for (int p = 0; p < n; ++p) {
      for (int q = p + 1; q < n; ++q) {
        const double apq = a[(size_t)p * n + q];
        if (std::fabs(apq) < 1e-300) continue;
        const double app = a[(size_t)p * n + p], aqq = a[(size_t)q * n + q];
        const double theta = (aqq - app) / (2.0 * apq);
        const double t = (theta >= 0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
        const double c = 1.0 / std::sqrt(t * t + 1.0), s = t * c;
        for (int k = 0; k < n; ++k) {
          const double akp = a[(size_t)k * n + p], akq = a[(size_t)k * n + q];
          a[(size_t)k * n + p] = c * akp - s * akq;
          a[(size_t)k * n + q] = s * akp + c * akq;
        }
        for (int k = 0; k < n; ++k) {
          const double apk = a[(size_t)p * n + k], aqk = a[(size_t)q * n + k];
          a[(size_t)p * n + k] = c * apk - s * aqk;
          a[(size_t)q * n + k] = s * apk + c * aqk;
        }
        for (int k = 0; k < n; ++k) {
          const double vkp = vec[(size_t)k * n + p], vkq = vec[(size_t)k * n + q];
          vec[(size_t)k * n + p] = c * vkp - s * vkq;
          vec[(size_t)k * n + q] = s * vkp + c * vkq;
        }
      }
    }
  }
  val.resize(n);
  for (int i = 0; i < n; ++i) val[i] = a[(size_t)i * n + i];
}

std::map<std::tuple<int, int, int, int>, double> cg_table(int F) {
  std::map<std::tuple<int, int, int, int>, double> t;
  for (int l = 0; l <= 2 * F; l += 2)
    for (int M = -l; M <= l; ++M)
      for (int m1 = -F; m1 <= F; ++m1) {
        const int m2 = M - m1;
        if (std::abs(m2) > F) continue;
        const double v = clebsch_gordan(F, m1, F, m2, l, M);
        if (std::fabs(v) < 1e-15) continue;
        t[{l, M, m1, m2}] = v;
      }
  return t;
}

// g_S = sum_k (2k+1) {F F k; F F S} c_k over even k (src/clebsch_gordan.jl:118-141).
std::map<int, double> cn_to_gS(int F, const std::map<int, double>& c) {
  std::map<int, double> g;
  for (int S = 0; S <= 2 * F; S += 2) {
    double s = 0.0;
    for (int k = 0; k <= 2 * F; k += 2) {
      auto it = c.find(k);
      const double ck = it == c.end() ? 0.0 : it->second;
      s += (2 * k + 1) * wigner_6j(F, F, k, F, F, S) * ck;
    }
    g[S] = s;
  }
  return g;
}

}  // namespace

double wigner_3j(int j1, int j2, int j3, int m1, int m2, int m3) {
  if (m1 + m2 + m3 != 0) return 0.0;
  const double lt = log_triangle(j1, j2, j3);
  if (lt == -INFINITY) return 0.0;
  const double ln = log_factorial(j1 + m1) + log_factorial(j1 - m1) + log_factorial(j2 + m2) +
                    log_factorial(j2 - m2) + log_factorial(j3 + m3) + log_factorial(j3 - m3);
  const int tmin = std::max({0, j2 - j3 - m1, j1 - j3 + m2});
  const int tmax = std::min({j1 + j2 - j3, j1 - m1, j2 + m2});
  if (tmin > tmax) return 0.0;
  double s = 0.0;
  for (int t = tmin; t <= tmax; ++t) {
    const double ld = log_factorial(t) + log_factorial(j1 + j2 - j3 - t) + log_factorial(j1 - m1 - t) +
                      log_factorial(j2 + m2 - t) + log_factorial(j3 - j2 + m1 + t) +
                      log_factorial(j3 - j1 - m2 + t);
    s += ((t % 2 == 0) ? 1.0 : -1.0) * std::exp(-ld);
  }
  const double phase = (((j1 - j2 - m3) % 2) == 0) ? 1.0 : -1.0;
  return phase * std::exp(0.5 * (lt + ln)) * s;
}

double clebsch_gordan(int j1, int m1, int j2, int m2, int J, int M) {
  if (m1 + m2 != M) return 0.0;
  const double phase = (((j1 - j2 + M) % 2) == 0) ? 1.0 : -1.0;
  return phase * std::sqrt(2.0 * J + 1.0) * wigner_3j(j1, j2, J, m1, m2, -M);
}

double wigner_6j(int j1, int j2, int j3, int j4, int j5, int j6) {
  const double t1 = log_triangle(j1, j2, j3), t2 = log_triangle(j1, j5, j6), t3 = log_triangle(j4, j2, j6),
               t4 = log_triangle(j4, j5, j3);
  if (t1 == -INFINITY || t2 == -INFINITY || t3 == -INFINITY || t4 == -INFINITY) return 0.0;
  const double lts = 0.5 * (t1 + t2 + t3 + t4);
  const int tmin = std::max({j1 + j2 + j3, j1 + j5 + j6, j4 + j2 + j6, j4 + j5 + j3});
  const int tmax = std::min({j1 + j2 + j4 + j5, j2 + j3 + j5 + j6, j1 + j3 + j4 + j6});
  if (tmin > tmax) return 0.0;
  double s = 0.0;
  for (int t = tmin; t <= tmax; ++t) {
    const double ln = log_factorial(t + 1);
    const double ld = log_factorial(t - j1 - j2 - j3) + log_factorial(t - j1 - j5 - j6) +
                      log_factorial(t - j4 - j2 - j6) + log_factorial(t - j4 - j5 - j3) +
                      log_factorial(j1 + j2 + j4 + j5 - t) + log_factorial(j2 + j3 + j5 + j6 - t) +
                      log_factorial(j1 + j3 + j4 + j6 - t);
    s += ((t % 2 == 0) ? 1.0 : -1.0) * std::exp(ln - ld);
  }
  return std::exp(lts) * s;
}

Setup build_setup(const sbec_config& cfg) {
  Setup s;
  s.cfg = cfg;
  if (cfg.ndim < 1 || cfg.ndim > 3) fail(SBEC_ERR_INVALID, "ndim must be 1, 2 or 3");
  s.ndim = cfg.ndim;
  s.N = 1;
  for (int d = 0; d < 3; ++d) {
    s.n[d] = 1;
    s.L[d] = 1.0;
  }
  for (int d = 0; d < s.ndim; ++d) {
    if (cfg.n[d] <= 0 || cfg.n[d] % 2 != 0) fail(SBEC_ERR_INVALID, "n_points must be positive even integers");
    if (!(cfg.L[d] > 0)) fail(SBEC_ERR_INVALID, "box_size must be positive");
    // power-of-two axes run the line kernels directly; other even sizes (up to 2048) run the
    // Bluestein transform on power-of-two lines of length >= 2n - 1
    const bool p2 = is_pow2(cfg.n[d]);
    if ((p2 && (cfg.n[d] > 4096 || (s.ndim > 1 && cfg.n[d] > 1024))) || (!p2 && cfg.n[d] > (d == 0 ? 2048 : 512)))
      fail(SBEC_ERR_UNSUPPORTED,
           "grid size " + std::to_string(cfg.n[d]) +
               " unsupported: the GPU path handles power-of-two n <= 4096 in 1-D and <= 1024 per axis in 2-D/3-D, "
               "and other even n <= 2048 on the first axis, <= 512 on the others");
    if (!p2) s.pow2 = false;
    s.n[d] = cfg.n[d];
    s.L[d] = cfg.L[d];
    s.N *= cfg.n[d];
    s.dx[d] = cfg.L[d] / cfg.n[d];
    const double dk = 2.0 * M_PI / cfg.L[d];
    s.kmult[d] = ((double)cfg.n[d] * dk) / (double)cfg.n[d];
  }
  s.dV = 1.0;
  for (int d = 0; d < s.ndim; ++d) s.dV *= s.dx[d];
  for (int d = 0; d < s.ndim; ++d) s.x0[d] = -cfg.L[d] / 2 + s.dx[d] / 2;
  if (cfg.F < 0) fail(SBEC_ERR_INVALID, "F must be non-negative");
  if (cfg.F > 6) fail(SBEC_ERR_UNSUPPORTED, "spin F > 6 is not supported by the GPU path");
  s.F = cfg.F;
  s.D = 2 * cfg.F + 1;
  if (!(cfg.dt > 0)) fail(SBEC_ERR_INVALID, "dt must be positive");
  if (cfg.precision != SBEC_FP64 && cfg.precision != SBEC_FP32_BULK) fail(SBEC_ERR_INVALID, "unknown precision");
  if (cfg.n_c_extra < 0 || cfg.n_c_extra > SBEC_MAX_C_EXTRA) fail(SBEC_ERR_INVALID, "n_c_extra out of range");
  const int F = s.F, D = s.D;

  // --- Raman coupling and losses
  if (cfg.raman) {
    if (!std::isfinite(cfg.raman_omega) || !std::isfinite(cfg.raman_delta))
      fail(SBEC_ERR_INVALID, "Raman Omega_R and delta must be finite");
    s.raman = true;
    s.raman_omega = cfg.raman_omega;
    s.raman_delta = cfg.raman_delta;
    for (int d = 0; d < 3; ++d) s.raman_k[d] = d < s.ndim ? cfg.raman_k[d] : 0.0;
  }
  if (!(cfg.loss_gamma_dr < 1e-30 && cfg.loss_L3 < 1e-30)) {
    // _dipolar_relaxation_rates (src/losses.jl:68-97): gamma_m = gamma_dr raw_m / (sum raw / D)
    // with raw_m = sum over q in {-1,-2}, |m+q| <= F, of CG(F,m; 2,q | F,m+q)^2
    std::vector<double> raw(D, 0.0);
    double raw_sum = 0.0;
    for (int c = 0; c < D; ++c) {
      const int m = F - c;
      double acc = 0.0;
      for (int q : {-1, -2}) {
        const int mp = m + q;
        if (mp < -F || mp > F) continue;
        const double cg = clebsch_gordan(F, m, 2, q, F, mp);
        acc += cg * cg;
      }
      raw[c] = acc;
      raw_sum += acc;
    }
    s.loss = true;
    s.loss_rates.assign(D, 0.0);
    for (int c = 0; c < D; ++c) {
      const double g = raw_sum < 1e-30 ? 0.0 : cfg.loss_gamma_dr * raw[c] / (raw_sum / D);
      s.loss_rates[c] = g + cfg.loss_L3;
    }
  }

  // --- interactions and tensor activation (src/initialization.jl:164-185)
  auto get_cn = [&](int k) -> double {
    if (k == 0) return cfg.c0;
    if (k == 1) return cfg.c1;
    const int idx = k - 1;  // 1-based c_extra index
    return idx <= cfg.n_c_extra ? cfg.c_extra[idx - 1] : 0.0;
  };
  std::map<int, double> g_total;
  bool tensor = false;
  s.c0 = cfg.c0;
  s.c1 = cfg.c1;
  s.c_lhy = cfg.c_lhy;
  if (cfg.gS_direct) {
    for (int S = 0; S <= 2 * F; S += 2) g_total[S] = cfg.gS[S / 2];
    tensor = true;
    s.c0 = s.c1 = 0.0;
  } else {
    bool has_higher = false;
    for (int i = 1; i <= cfg.n_c_extra; ++i) {
      const int k = i + 1;
      if (k % 2 == 0 && k >= 4 && k <= 2 * F && std::fabs(cfg.c_extra[i - 1]) > 1e-30) has_higher = true;
    }
    if (has_higher) {
      // g_base = c0 + c1 (S(S+1) - 2F(F+1))/2 (src/interactions.jl:123-128)
      for (int S = 0; S <= 2 * F; S += 2) g_total[S] = cfg.c0 + cfg.c1 * (S * (S + 1) - 2 * F * (F + 1)) / 2.0;
      std::map<int, double> cd;
      for (int i = 1; i <= cfg.n_c_extra; ++i) {
        const int k = i + 1;
        const double v = cfg.c_extra[i - 1];
        if (std::fabs(v) > 1e-30 && k % 2 == 0 && k <= 2 * F) cd[k] = v;
      }
      if (!cd.empty()) {
        auto gd = cn_to_gS(F, cd);
        for (auto& kv : gd) g_total[kv.first] += kv.second;
      }
      tensor = true;
      s.c0 = s.c1 = 0.0;
    } else {
      // make_tensor_interaction_cache(F, interactions) (src/tensor_interaction.jl:61-99)
      std::map<int, double> cd;
      for (int k = 0; k <= 2 * F; k += 2) {
        const double ck = get_cn(k);
        if (std::fabs(ck) > 1e-30) cd[k] = ck;
      }
      bool higher = false;
      for (auto& kv : cd)
        if (kv.first > 2) higher = true;
      if (!cd.empty() && higher) {
        g_total = cn_to_gS(F, cd);
        tensor = true;
        if (std::fabs(cfg.c0) > 1e-30 || std::fabs(cfg.c1) > 1e-30)
          fail(SBEC_ERR_INVALID,
               "tensor_cache active with non-zero c0/c1. When tensor_cache handles all channels, set c0=c1=0 "
               "in InteractionParams to avoid double-counting");
      }
    }
  }
  if (tensor) {
    for (int S = 0; S <= 2 * F; S += 2) {
      const double g = g_total.count(S) ? g_total[S] : 0.0;
      if (std::fabs(g) > 1e-30) {
        s.chS.push_back(S);
        s.chG.push_back(g);
      }
    }
    tensor = !s.chS.empty();
  }
  s.tensor = tensor;
  if (!tensor) s.c2 = get_cn(2);  // the singlet-pair (nematic) step (src/nematic.jl:34-51)

  if (tensor) {
    auto tab = cg_table(F);
    auto cg = [&](int S, int M, int m1, int m2) {
      auto it = tab.find({S, M, m1, m2});
      return it == tab.end() ? 0.0 : it->second;
    };
    const int NJ = 4 * F + 1;
    s.G.assign((size_t)NJ * D * D, 0.0);
    for (size_t si = 0; si < s.chS.size(); ++si) {
      const int S = s.chS[si];
      const double g = s.chG[si];
      for (int J = 0; J < NJ; ++J) {
        const int M = 2 * F - J;
        if (std::abs(M) > S) continue;
        for (int c = 0; c < D; ++c) {
          const int a = J - c;
          if (a < 0 || a >= D) continue;
          const int m = F - c, mu = F - a;
          const double c1v = cg(S, M, m, mu);
          if (std::fabs(c1v) < 1e-15) continue;
          for (int cp = 0; cp < D; ++cp) {
            const int b = J - cp;
            if (b < 0 || b >= D) continue;
            const int mp = F - cp, nu = F - b;
            const double c2v = cg(S, M, mp, nu);
            if (std::fabs(c2v) < 1e-15) continue;
            s.G[((size_t)J * D + c) * D + cp] += g * (c1v * c2v);
          }
        }
      }
      s.bound_coef += std::fabs(g) * (2.0 * S + 1.0) / (2.0 * F + 1.0);
    }
    // pair amplitudes (src/tensor_interaction.jl:285-305)
    int offset = 0;
    for (size_t si = 0; si < s.chS.size(); ++si) {
      const int S = s.chS[si];
      for (int M = -S; M <= S; ++M) {
        const int a_idx = offset + M + S;
        for (int m1 = -F; m1 <= F; ++m1) {
          const int m2 = M - m1;
          if (std::abs(m2) > F) continue;
          const double v = cg(S, M, m1, m2);
          if (std::fabs(v) < 1e-15) continue;
          s.pair_a.push_back(a_idx);
          s.pair_c1.push_back(F - m1);
          s.pair_c2.push_back(F - m2);
          s.pair_cg.push_back(v);
        }
        s.gA.push_back(s.chG[si]);
      }
      offset += 2 * S + 1;
    }
  }

  // --- spin matrices (src/spin_matrices.jl:1-50)
  s.fp.assign(D, 0.0);
  s.m.assign(D, 0.0);
  for (int c = 0; c < D; ++c) s.m[c] = (double)(F - c);
  for (int c = 1; c < D; ++c) {
    const double mc = (double)(F - c);
    s.fp[c] = std::sqrt((double)(F * (F + 1)) - mc * (mc + 1.0));
  }
  // Fy = (F+ - F-)/(2i): Fy[c][c+1] = -i fp[c+1]/2, Fy[c+1][c] = +i fp[c+1]/2.
  // Real embedding [[A,-B],[B,A]] of Fy = A + iB (A = 0).
  {
    const int n2 = 2 * D;
    std::vector<double> emb((size_t)n2 * n2, 0.0);
    for (int c = 0; c + 1 < D; ++c) {
      const double b = -0.5 * s.fp[c + 1];  // B[c][c+1] = Im Fy[c][c+1]
      // -B block (top right) and B block (bottom left)
      emb[(size_t)c * n2 + (D + c + 1)] = -b;
      emb[(size_t)(c + 1) * n2 + (D + c)] = b;        // B[c+1][c] = -b -> -B = b
      emb[(size_t)(D + c) * n2 + (c + 1)] = b;
      emb[(size_t)(D + c + 1) * n2 + c] = -b;
    }
    std::vector<double> val, vec;
    jacobi_sym(emb, n2, val, vec);
    std::vector<int> order(n2);
    for (int i = 0; i < n2; ++i) order[i] = i;
    std::sort(order.begin(), order.end(), [&](int a, int b) { return val[a] < val[b]; });
    s.FyV.assign((size_t)D * D, 0.0);
    s.FyVt.assign((size_t)D * D, 0.0);
    for (int k = 0; k < D; ++k) {
      const int col = order[2 * k];
      const double lam = val[col];
      if (std::fabs(lam - (double)(k - F)) > 1e-9)
        fail(SBEC_ERR_INVALID, "Fy eigenvalues not uniformly spaced (internal eigensolver failure)");
      double nrm = 0.0;
      for (int i = 0; i < D; ++i) {
        const double x = vec[(size_t)i * n2 + col], y = vec[(size_t)(D + i) * n2 + col];
        nrm += x * x + y * y;
      }
      nrm = std::sqrt(nrm);
      for (int i = 0; i < D; ++i) {
        const std::complex<double> z(vec[(size_t)i * n2 + col] / nrm, vec[(size_t)(D + i) * n2 + col] / nrm);
        s.FyV[(size_t)i * D + k] = z;
        s.FyVt[(size_t)k * D + i] = std::conj(z);
      }
    }
  }

  // --- DDI (src/ddi.jl:51-82, src/ddi_padded.jl:6-49)
  s.ddi = cfg.enable_ddi != 0;
  if (s.ddi && !s.pow2)
    fail(SBEC_ERR_UNSUPPORTED, "the dipolar convolution on the GPU path needs power-of-two grid sizes");
  s.secular = cfg.secular_ddi != 0;
  s.padded = s.ddi && cfg.ddi_padding != 0;
  s.c_dd = std::isnan(cfg.c_dd) ? 0.0 : cfg.c_dd;
  for (int d = 0; d < 3; ++d) {
    const int nd = d < s.ndim ? s.n[d] : 1;
    s.conv_M[0][d] = nd;
    s.conv_M[1][d] = d < s.ndim ? 2 * nd : 1;
    if (d < s.ndim) {
      const double dk = 2.0 * M_PI / s.L[d];
      s.conv_kmult[0][d] = ((double)nd * dk) / (double)nd;
      const int Mp = 2 * nd;
      const double fs = (double)Mp * (2.0 * M_PI / ((double)Mp * s.dx[d]));
      s.conv_kmult[1][d] = fs / (double)Mp;
    }
  }
  if (s.ddi && s.padded && s.ndim > 1) {
    for (int d = 0; d < s.ndim; ++d)
      if (2 * s.n[d] > 1024) fail(SBEC_ERR_UNSUPPORTED, "zero-padded DDI needs 2n <= 1024 per axis");
  }
  return s;
}

}  // namespace sbec
