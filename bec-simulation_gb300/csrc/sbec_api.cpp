// C ABI (include/sbec.h) and the host-side drivers that loop over the device
// operators: split_step!, the leapfrog / standard run_simulation! loops, the
// adaptive Strang and Yoshida loops and the find_ground_state ITP loop.  Each
// driver restates the control flow of the reference file:line it cites; the
// per-step arithmetic runs in the device kernels (sbec_kernels.cuh).
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <memory>
#include <string>
#include <thread>
#include <vector>

#include "sbec.h"
#include "sbec_engine.h"
#include "sbec_setup.h"

namespace sbec {

void cuda_check(cudaError_t e, const char* what) {
  if (e == cudaSuccess) return;
  cudaGetLastError();
  const sbec_status st = (e == cudaErrorMemoryAllocation) ? SBEC_ERR_OOM : SBEC_ERR_DEVICE;
  throw SbecError{st, std::string(what) + ": " + cudaGetErrorString(e)};
}

}  // namespace sbec

using namespace sbec;

// A batch: solves grouped by grid, one engine (device buffers, stream) per group; solve i
// lives in group grp[i] at local index loc[i].  Groups advance concurrently.
struct sbec_batch {
  std::vector<std::unique_ptr<EngineBase>> groups;
  std::vector<int> grp, loc;
  int n() const { return (int)grp.size(); }
};

struct sbec_ws {
  std::unique_ptr<EngineBase> eng;
  double kin_dt = 0.0;    // parameters of the current kinetic phase (the batched kinetic cache)
  bool kin_itp = false;
  bool pipelined_snapshots = false;  // sbec_set_snapshot_mode
  std::vector<double> host_psi;
  sbec_zeeman_fn zfn = nullptr;      // sbec_set_zeeman_fn (TimeDependentZeeman)
  void* zuser = nullptr;
};

namespace {

thread_local std::string g_err;

}  // namespace

namespace sbec {
void set_last_error(const std::string& msg) { g_err = msg; }

std::mutex& tune_table_mutex() {
  static std::mutex m;
  return m;
}
std::map<std::string, int>& tune_table_map() {
  static std::map<std::string, int> t;
  return t;
}

std::atomic<bool>& tune_frozen() {
  static std::atomic<bool> f{false};
  return f;
}
}  // namespace sbec

namespace {

#define SBEC_API_BEGIN try {
#define SBEC_API_END                                      \
  }                                                       \
  catch (const SbecError& e) {                            \
    g_err = e.msg;                                        \
    return e.status;                                      \
  }                                                       \
  catch (const std::bad_alloc&) {                         \
    g_err = "host allocation failed";                     \
    return SBEC_ERR_OOM;                                  \
  }                                                       \
  catch (const std::exception& e) {                       \
    g_err = e.what();                                     \
    return SBEC_ERR_DEVICE;                               \
  }                                                       \
  return SBEC_OK;

void need(const void* p, const char* what) {
  if (!p) fail(SBEC_ERR_INVALID, std::string(what) + " must not be NULL");
}

EngineBase& E(sbec_ws* ws) {
  need(ws, "workspace");
  return *ws->eng;
}

// ---- operator sequences shared by the drivers -----------------------------

// zeeman_at(ws.zeeman, ws.state.t) (src/zeeman.jl:20-21) when a time-dependent Zeeman
// function is set; a no-op for the static (p, q).
void zee(sbec_ws* ws) {
  if (!ws->zfn) return;
  EngineBase& e = *ws->eng;
  double p = e.zeeman_p, q = e.zeeman_q;
  ws->zfn(ws->zuser, e.t, &p, &q);
  if (!std::isfinite(p) || !std::isfinite(q)) fail(SBEC_ERR_INVALID, "Zeeman function returned a non-finite p or q");
  e.zeeman_p = p;
  e.zeeman_q = q;
}

void kinetic(sbec_ws* ws, double dt, bool itp) {
  ws->kin_dt = dt;
  ws->kin_itp = itp;
  ws->eng->kinetic(dt, itp);
}

// split_step! x n through the fused row passes when the workspace allows it
// (no DDI / tensor, renormalisation every step or never); else operator by operator,
// replayed from graph chunks when renormalisation is every step or never.
void split_steps(sbec_ws* ws, long long n);

// split_step! (src/split_step.jl:10-35)
void split_step_once(sbec_ws* ws) {
  EngineBase& e = *ws->eng;
  const double dt = e.dt;
  const bool it = e.itp;
  e.half_potential(dt / 2, it);
  e.kinetic(ws->kin_dt, ws->kin_itp);
  e.half_potential(dt / 2, it);
  if (!it) e.apply_loss(dt);  // src/split_step.jl:21-23
  e.t += it ? 0.0 : dt;
  e.step += 1;
  if (it && e.normalize_every > 0 && e.step % e.normalize_every == 0) e.normalize();
}

void split_steps(sbec_ws* ws, long long n) {
  EngineBase& e = *ws->eng;
  if (ws->zfn) {
    // the Zeeman factors change with t: one step at a time, launched eagerly
    for (long long i = 0; i < n; ++i) {
      zee(ws);
      split_step_once(ws);
    }
    return;
  }
  const bool it = e.itp;
  const bool norm_each = it && e.normalize_every == 1;
  const bool no_norm = !it || e.normalize_every <= 0;
  if (n > 0 && e.fused_path() && (norm_each || no_norm)) {
    e.fused_split_steps(n, e.dt, ws->kin_dt, ws->kin_itp, it, norm_each);
    for (long long i = 0; i < n; ++i) {
      e.t += it ? 0.0 : e.dt;
      e.step += 1;
    }
    return;
  }
  if (n > 1 && (norm_each || no_norm)) {
    e.unfused_split_steps(n, e.dt, ws->kin_dt, ws->kin_itp, it, norm_each);
    for (long long i = 0; i < n; ++i) {
      e.t += it ? 0.0 : e.dt;
      e.step += 1;
    }
    return;
  }
  for (long long i = 0; i < n; ++i) split_step_once(ws);
}

// _strang_core! (src/split_step.jl:146-152)
void strang_core(sbec_ws* ws, double dt) {
  zee(ws);
  ws->eng->half_potential(dt / 2, false);
  kinetic(ws, dt, false);
  ws->eng->half_potential(dt / 2, false);
}

const double kW1 = 1.0 / (2.0 - std::pow(2.0, 1.0 / 3.0));
const double kW0 = 1.0 - 2.0 * kW1;

// _yoshida_core! (src/split_step.jl:161-183)
void yoshida_core(sbec_ws* ws, double dt) {
  const double w1 = kW1, w0 = kW0, wm = (w1 + w0) / 2;
  EngineBase& e = *ws->eng;
  zee(ws);
  e.half_potential(w1 * dt / 2, false);
  kinetic(ws, w1 * dt, false);
  e.half_potential(wm * dt, false);
  kinetic(ws, w0 * dt, false);
  e.half_potential(wm * dt, false);
  kinetic(ws, w1 * dt, false);
  e.half_potential(w1 * dt / 2, false);
}

double total_energy(EngineBase& e) {
  const sbec_energy_terms t = e.energy_terms();
  return t.kinetic + t.trap + t.zeeman + t.c0 + t.c1 + t.ddi + t.lhy + t.tensor + t.raman;
}

void norm_and_mz(EngineBase& e, double* norm, double* mz) {
  const Setup& s = e.setup();
  std::vector<double> sums(s.D);
  double nan = 0;
  e.comp_norms(sums.data(), &nan);
  double n = 0.0, m = 0.0;
  for (int c = 0; c < s.D; ++c) {
    n += sums[c];
    m += (double)(s.F - c) * sums[c] * s.dV;
  }
  *norm = n * s.dV;
  *mz = m;
}

// _record_snapshot! (src/simulation_utils.jl:9-15) delivered to the callback.
int snapshot(sbec_ws* ws, sbec_callback cb, void* user) {
  if (!cb) return 0;
  zee(ws);  // total_energy evaluates zeeman_at(ws.zeeman, ws.state.t) (src/energy.jl:15)
  EngineBase& e = *ws->eng;
  sbec_snapshot sn{};
  sn.t = e.t;
  sn.step = e.step;
  const Setup& s = e.setup();
  std::vector<double> sums(s.D);
  const sbec_energy_terms t = e.energy_terms_and_norms(sums.data());
  sn.energy = t.kinetic + t.trap + t.zeeman + t.c0 + t.c1 + t.ddi + t.lhy + t.tensor + t.raman;
  double n = 0.0, m = 0.0;
  for (int c = 0; c < s.D; ++c) {
    n += sums[c];
    m += (double)(s.F - c) * sums[c] * s.dV;
  }
  sn.norm = n * s.dV;
  sn.magnetization = m;
  sn.psi = e.psi_to_pinned();
  return cb(user, &sn);
}

void check_cb(int rc) {
  if (rc != 0) fail(SBEC_ERR_CALLBACK, "callback requested stop");
}

// Leapfrog run with pipelined save points: the snapshot of save point j (energy
// sums and FP64 psi into pinned slot j & 1) is enqueued behind segment j, segment
// j + 1 is enqueued, and only then is save point j handed to the callback, so the
// host-side callback overlaps the device work of the next segment.  A stop request
// restores psi, t and step from the snapshot of that save point.
void run_leapfrog_pipelined(sbec_ws* ws, int64_t n_steps, int64_t save_every, sbec_callback cb, void* user) {
  EngineBase& e = *ws->eng;
  const double dt = e.dt;
  const Setup& s = e.setup();
  struct Meta {
    double t;
    int64_t step;
  } meta[2] = {};
  auto deliver = [&](int k) {
    sbec_snapshot sn{};
    std::vector<double> sums(s.D);
    sbec_energy_terms t{};
    sn.psi = e.snapshot_wait(k, &t, sums.data());
    sn.t = meta[k & 1].t;
    sn.step = meta[k & 1].step;
    sn.energy = t.kinetic + t.trap + t.zeeman + t.c0 + t.c1 + t.ddi + t.lhy + t.tensor + t.raman;
    double n = 0.0, m = 0.0;
    for (int c = 0; c < s.D; ++c) {
      n += sums[c];
      m += (double)(s.F - c) * sums[c] * s.dV;
    }
    sn.norm = n * s.dV;
    sn.magnetization = m;
    if (cb(user, &sn) != 0) {
      e.restore_snapshot(k);
      e.t = meta[k & 1].t;
      e.step = meta[k & 1].step;
      fail(SBEC_ERR_CALLBACK, "callback requested stop");
    }
  };
  e.lf_open(dt);  // the caller has delivered the step-0 snapshot
  int64_t step = 0;
  int pending = -1, k = 0;
  while (step < n_steps) {
    const int64_t seg_end = std::min(n_steps, (step / save_every + 1) * save_every);
    const int64_t nseg = seg_end - step;
    e.lf_steps(nseg - 1, dt);
    e.lf_close(dt);
    for (int64_t i = 0; i < nseg; ++i) {
      e.t += dt;
      e.step += 1;
    }
    step = seg_end;
    if (pending >= 0) {
      deliver(pending);
      pending = -1;
    }
    if (step % save_every == 0) {
      e.snapshot_enqueue(k);
      meta[k & 1] = {e.t, e.step};
      pending = k++;
    }
    if (step < n_steps) e.lf_open(dt);
  }
  if (pending >= 0) deliver(pending);
  e.check_segments();
}

// _normalize_psi_constrained! (src/ground_state.jl:279-320)
void normalize_constrained(EngineBase& e, double target) {
  const Setup& s = e.setup();
  const int D = s.D, F = s.F;
  e.normalize();
  std::vector<double> raw(D);
  double nan = 0;
  e.comp_norms(raw.data(), &nan);
  double lambda = 0.0;
  std::vector<double> norms(D);
  for (int it = 0; it < 20; ++it) {
    for (int c = 0; c < D; ++c) {
      const int m = F - c;
      const double w = std::exp(lambda * m);
      norms[c] = raw[c] * s.dV * (w * w);
    }
    double total = 0.0;
    for (int c = 0; c < D; ++c) total += norms[c];
    if (total < 1e-30) break;
    double Mz = 0.0;
    for (int c = 0; c < D; ++c) Mz += (double)(F - c) * norms[c];
    Mz /= total;
    if (std::fabs(Mz - target) < 1e-12) break;
    double dMz = 0.0;
    for (int c = 0; c < D; ++c) {
      const double m = (double)(F - c);
      dMz += 2 * m * (m - Mz) * norms[c] / total;
    }
    if (std::fabs(dMz) < 1e-30) break;
    lambda -= (Mz - target) / dMz;
    lambda = std::min(10.0, std::max(-10.0, lambda));
  }
  std::vector<double> w(D);
  for (int c = 0; c < D; ++c) w[c] = std::exp(lambda * (double)(F - c));
  e.scale_components(w.data());
  e.normalize();
}

// classify_phase (src/diagnostics.jl:166-206) from the device grid sums.
void classify_phase(EngineBase& e, int solve, sbec_phase_info* out) {
  const Setup& s = e.setup();
  double r[kPhaseSums];
  e.phase_sums(solve, r);
  *out = sbec_phase_info{};
  const int F = s.F, D = s.D;
  const double dV = s.dV;
  out->n_channels = F + 1;
  const double n_sum = r[0] * dV, n_sq = r[1] * dV;
  if (n_sum < 1e-30) {
    out->phase = SBEC_PHASE_VACUUM;
    return;
  }
  out->spin_order = F > 0 ? r[2] * dV / ((double)F * F * n_sq) : 0.0;
  double total = 0.0;
  for (int k = 0; k <= F; ++k) {
    out->raw_channel_weights[k] = r[4 + k] * dV;
    total += out->raw_channel_weights[k];
  }
  for (int k = 0; k <= F; ++k) out->channel_weights[k] = total > 0 ? out->raw_channel_weights[k] / total : 0.0;
  out->nematic_order = out->raw_channel_weights[0] / (n_sq / D);
  out->magnetization_density = r[3] * dV / n_sum;
  if (out->spin_order > 0.9)
    out->phase = SBEC_PHASE_FERROMAGNETIC;
  else if (out->nematic_order > 0.9)
    out->phase = F == 1 ? SBEC_PHASE_POLAR : SBEC_PHASE_NEMATIC;
  else if (out->channel_weights[F] > 0.5)
    out->phase = SBEC_PHASE_CYCLIC;
  else
    out->phase = SBEC_PHASE_MIXED;
}

// _check_itp_overflow (src/ground_state.jl:4-29)
void check_itp_overflow(EngineBase& e, long long step) {
  const Setup& s = e.setup();
  std::vector<double> sums(s.D);
  double nan = 0;
  e.comp_norms(sums.data(), &nan);
  if (nan > 0)
    fail(SBEC_ERR_NUMERIC, "NaN detected in ITP at step " + std::to_string(step) +
                               ". Likely DDI potential overflow. Reduce dt.");
  if (!s.ddi) return;
  const double phi_max = e.ddi_phi_max();
  const double exponent = phi_max * e.dt / 2;
  if (exponent > 50.0)
    fail(SBEC_ERR_NUMERIC, "DDI potential overflow in ITP at step " + std::to_string(step) + ": exponent=" +
                               std::to_string(exponent) + " > 50. Reduce dt.");
}

}  // namespace

// ============================================================================
extern "C" {

const char* sbec_last_error(void) { return g_err.c_str(); }

const char* sbec_version(void) { return "sbec-gb300 0.1 (sm_103a)"; }

int sbec_device_count(void) {
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return n;
}

sbec_status sbec_ws_create(const sbec_config* cfg, const double* psi, const double* V, sbec_ws** out) {
  SBEC_API_BEGIN
  need(cfg, "config");
  need(psi, "psi");
  need(out, "out");
  *out = nullptr;
  Setup s = build_setup(*cfg);
  if (sbec_device_count() < 1) fail(SBEC_ERR_DEVICE, "no CUDA device available (the GPU path has no CPU fallback)");
  auto ws = std::make_unique<sbec_ws>();
  ws->eng = cfg->precision == SBEC_FP32_BULK ? make_engine_f32(s) : make_engine_f64(s);
  EngineBase& e = *ws->eng;
  e.zeeman_p = cfg->zeeman_p;
  e.zeeman_q = cfg->zeeman_q;
  e.dt = cfg->dt;
  e.itp = cfg->imaginary_time != 0;
  e.normalize_every = cfg->normalize_every;
  ws->kin_dt = cfg->dt;
  ws->kin_itp = e.itp;
  e.set_psi(psi);
  if (V) e.set_potential(V);
  e.sync();
  *out = ws.release();
  SBEC_API_END
}

sbec_status sbec_ws_destroy(sbec_ws* ws) {
  SBEC_API_BEGIN
  delete ws;
  SBEC_API_END
}

sbec_status sbec_set_psi(sbec_ws* ws, const double* psi) {
  SBEC_API_BEGIN
  need(psi, "psi");
  E(ws).set_psi(psi);
  E(ws).sync();
  SBEC_API_END
}

sbec_status sbec_get_psi(sbec_ws* ws, double* psi) {
  SBEC_API_BEGIN
  need(psi, "psi");
  E(ws).get_psi(psi);
  SBEC_API_END
}

sbec_status sbec_set_time(sbec_ws* ws, double t, int64_t step) {
  SBEC_API_BEGIN
  E(ws).t = t;
  E(ws).step = step;
  SBEC_API_END
}

sbec_status sbec_get_time(sbec_ws* ws, double* t, int64_t* step) {
  SBEC_API_BEGIN
  if (t) *t = E(ws).t;
  if (step) *step = E(ws).step;
  SBEC_API_END
}

sbec_status sbec_set_zeeman(sbec_ws* ws, double p, double q) {
  SBEC_API_BEGIN
  E(ws).zeeman_p = p;
  E(ws).zeeman_q = q;
  SBEC_API_END
}

sbec_status sbec_set_zeeman_fn(sbec_ws* ws, sbec_zeeman_fn fn, void* user) {
  SBEC_API_BEGIN
  E(ws);
  ws->zfn = fn;
  ws->zuser = fn ? user : nullptr;
  SBEC_API_END
}

sbec_status sbec_set_potential(sbec_ws* ws, const double* V) {
  SBEC_API_BEGIN
  need(V, "V");
  E(ws).set_potential(V);
  SBEC_API_END
}

sbec_status sbec_set_dt(sbec_ws* ws, double dt) {
  SBEC_API_BEGIN
  if (!(dt > 0)) fail(SBEC_ERR_INVALID, "dt must be positive");
  E(ws).dt = dt;
  ws->kin_dt = dt;
  ws->kin_itp = E(ws).itp;
  SBEC_API_END
}

sbec_status sbec_tensor_channels(sbec_ws* ws, int32_t* active, int32_t* n_channels, int32_t* S, double* gS) {
  SBEC_API_BEGIN
  const Setup& s = E(ws).setup();
  if (active) *active = s.tensor ? 1 : 0;
  if (n_channels) *n_channels = (int32_t)s.chS.size();
  for (size_t i = 0; i < s.chS.size(); ++i) {
    if (S) S[i] = s.chS[i];
    if (gS) gS[i] = s.chG[i];
  }
  SBEC_API_END
}

sbec_status sbec_half_potential(sbec_ws* ws, double dt_half, int32_t imaginary_time) {
  SBEC_API_BEGIN
  E(ws);
  zee(ws);
  E(ws).half_potential(dt_half, imaginary_time != 0);
  E(ws).sync();
  SBEC_API_END
}

sbec_status sbec_kinetic(sbec_ws* ws, double dt, int32_t imaginary_time) {
  SBEC_API_BEGIN
  E(ws);
  kinetic(ws, dt, imaginary_time != 0);
  ws->eng->sync();
  SBEC_API_END
}

sbec_status sbec_normalize(sbec_ws* ws) {
  SBEC_API_BEGIN
  E(ws).normalize();
  E(ws).sync();
  SBEC_API_END
}

sbec_status sbec_normalize_constrained(sbec_ws* ws, double target_Mz) {
  SBEC_API_BEGIN
  normalize_constrained(E(ws), target_Mz);
  E(ws).sync();
  SBEC_API_END
}

sbec_status sbec_split_step(sbec_ws* ws, int64_t n) {
  SBEC_API_BEGIN
  E(ws);
  split_steps(ws, n);
  ws->eng->sync();
  SBEC_API_END
}

sbec_status sbec_strang_core(sbec_ws* ws, double dt) {
  SBEC_API_BEGIN
  E(ws);
  strang_core(ws, dt);
  ws->eng->sync();
  SBEC_API_END
}

sbec_status sbec_yoshida_core(sbec_ws* ws, double dt) {
  SBEC_API_BEGIN
  E(ws);
  yoshida_core(ws, dt);
  ws->eng->sync();
  SBEC_API_END
}

// run_simulation! (src/simulation.jl:1-94)
sbec_status sbec_run_simulation(sbec_ws* ws, int64_t n_steps, int64_t save_every, sbec_callback cb, void* user) {
  SBEC_API_BEGIN
  EngineBase& e = E(ws);
  if (n_steps <= 0) fail(SBEC_ERR_INVALID, "n_steps must be positive");
  if (save_every <= 0) fail(SBEC_ERR_INVALID, "save_every must be positive");
  check_cb(snapshot(ws, cb, user));
  if (e.itp) {
    int64_t step = 0;
    while (step < n_steps) {
      const int64_t nxt = std::min(n_steps, (step / save_every + 1) * save_every);
      split_steps(ws, nxt - step);
      step = nxt;
      if (step % save_every == 0) check_cb(snapshot(ws, cb, user));
    }
  } else if (ws->zfn) {
    // the leapfrog with the Zeeman term evaluated at the state time before every potential
    // step (src/simulation.jl:49-94), one step at a time
    const double dt = e.dt;
    zee(ws);
    e.half_potential(dt / 2, false);
    for (int64_t step = 1; step <= n_steps; ++step) {
      e.kinetic(ws->kin_dt, ws->kin_itp);
      const bool is_save = step % save_every == 0, is_last = step == n_steps;
      zee(ws);
      e.half_potential(is_save || is_last ? dt / 2 : dt, false);
      e.apply_loss(dt);
      e.t += dt;
      e.step += 1;
      if (is_save) check_cb(snapshot(ws, cb, user));
      if ((is_save || is_last) && !is_last) {
        zee(ws);
        e.half_potential(dt / 2, false);
      }
    }
  } else if (e.fused_path() && !ws->kin_itp && ws->kin_dt == e.dt && ws->pipelined_snapshots && cb) {
    run_leapfrog_pipelined(ws, n_steps, save_every, cb, user);
  } else if (e.fused_path() && !ws->kin_itp && ws->kin_dt == e.dt) {
    // leapfrog with the fused row passes: identical operator sequence
    const double dt = e.dt;
    e.lf_open(dt);
    int64_t step = 0;
    while (step < n_steps) {
      const int64_t seg_end = std::min(n_steps, (step / save_every + 1) * save_every);
      const int64_t nseg = seg_end - step;
      e.lf_steps(nseg - 1, dt);
      e.lf_close(dt);
      for (int64_t i = 0; i < nseg; ++i) {
        e.t += dt;
        e.step += 1;
      }
      step = seg_end;
      if (step % save_every == 0) check_cb(snapshot(ws, cb, user));
      if (step < n_steps) e.lf_open(dt);
    }
    e.check_segments();
  } else {
    // the same leapfrog on the general path: V(dt/2), then per save segment
    // (n-1) x [K, V(dt)] from graph chunks, K, V(dt/2), the save point, V(dt/2)
    const double dt = e.dt;
    e.half_potential(dt / 2, false);
    int64_t step = 0;
    while (step < n_steps) {
      const int64_t seg_end = std::min(n_steps, (step / save_every + 1) * save_every);
      const int64_t nseg = seg_end - step;
      e.unfused_lf_steps(nseg - 1, dt, ws->kin_dt, ws->kin_itp);
      e.kinetic(ws->kin_dt, ws->kin_itp);
      e.half_potential(dt / 2, false);
      e.apply_loss(dt);  // src/simulation.jl:74-76
      for (int64_t i = 0; i < nseg; ++i) {
        e.t += dt;
        e.step += 1;
      }
      step = seg_end;
      if (step % save_every == 0) check_cb(snapshot(ws, cb, user));
      if (step < n_steps) e.half_potential(dt / 2, false);
    }
  }
  e.sync();
  SBEC_API_END
}

// run_simulation_adaptive! (src/adaptive.jl:57-296)
sbec_status sbec_run_adaptive(sbec_ws* ws, const sbec_adaptive_params* p, double t_end, double save_interval,
                              sbec_callback cb, void* user, sbec_adaptive_result* out) {
  SBEC_API_BEGIN
  EngineBase& e = E(ws);
  need(p, "params");
  if (!(p->dt_init > 0) || !(p->dt_min > 0) || !(p->dt_max >= p->dt_min) || !(p->tol > 0))
    fail(SBEC_ERR_INVALID, "invalid AdaptiveDtParams");
  double dt = std::min(std::max(p->dt_init, p->dt_min), p->dt_max);
  long long n_acc = 0, n_rej = 0;
  check_cb(snapshot(ws, cb, user));
  double next_save = e.t + save_interval;
  if (p->error_mode == 0) {
    // _adaptive_step_change_loop! (src/adaptive.jl:69-195)
    double current_kinetic_dt = NAN;
    bool fsal_deferred = false;
    double fsal_dt = 0.0;
    while (e.t < t_end - 1e-14) {
      zee(ws);
      double dt_step = std::min(dt, t_end - e.t);
      const double rem = next_save - e.t;
      if (rem > 1e-14 && rem < dt_step) dt_step = rem;
      dt_step = std::max(dt_step, p->dt_min);
      const bool is_clamped = dt_step < dt * 0.99;
      const bool may_reject = !is_clamped && dt_step > p->dt_min * 1.01;
      if (dt_step != current_kinetic_dt) current_kinetic_dt = dt_step;
      if (!is_clamped) e.copy_slot(kSlotA, kPsi);
      const bool prev_fd = fsal_deferred;
      const double prev_fdt = fsal_dt;
      if (fsal_deferred && std::fabs(fsal_dt - dt_step) < 1e-14) {
        e.half_potential(dt_step, false);
      } else if (fsal_deferred) {
        e.half_potential(fsal_dt / 2, false);
        e.half_potential(dt_step / 2, false);
      } else {
        e.half_potential(dt_step / 2, false);
      }
      fsal_deferred = false;
      kinetic(ws, current_kinetic_dt, false);
      double rel = 0.0;
      if (may_reject) {
        rel = e.l2_change(kPsi, kSlotA);
        if (rel > p->tol) {
          e.copy_slot(kPsi, kSlotA);
          fsal_deferred = prev_fd;
          fsal_dt = prev_fdt;
          const double factor = std::max(0.5, 0.9 * std::sqrt(p->tol / rel));
          dt = std::max(dt_step * factor, p->dt_min);
          current_kinetic_dt = NAN;
          ++n_rej;
          continue;
        }
      }
      fsal_deferred = true;
      fsal_dt = dt_step;
      e.apply_loss(dt_step);  // src/adaptive.jl:151-153
      e.t += dt_step;
      e.step += 1;
      ++n_acc;
      if (!is_clamped) {
        if (!may_reject) rel = e.l2_change(kPsi, kSlotA);
        const double factor = rel > 1e-300 ? std::min(2.0, 0.9 * std::sqrt(p->tol / rel)) : 2.0;
        dt = std::min(std::max(dt * factor, p->dt_min), p->dt_max);
      }
      if (e.t >= next_save - 1e-14) {
        zee(ws);
        e.half_potential(fsal_dt / 2, false);
        fsal_deferred = false;
        check_cb(snapshot(ws, cb, user));
        next_save += save_interval;
      }
    }
    if (fsal_deferred) {
      zee(ws);
      e.half_potential(fsal_dt / 2, false);
    }
  } else {
    // _adaptive_richardson_loop! (src/adaptive.jl:204-296)
    while (e.t < t_end - 1e-14) {
      double dt_step = std::min(dt, t_end - e.t);
      const double rem = next_save - e.t;
      if (rem > 1e-14 && rem < dt_step) dt_step = rem;
      dt_step = std::max(dt_step, p->dt_min);
      const bool is_clamped = dt_step < dt * 0.99;
      const bool may_reject = !is_clamped && dt_step > p->dt_min * 1.01;
      zee(ws);
      e.copy_slot(kSlotA, kPsi);
      e.half_potential(dt_step / 2, false);
      kinetic(ws, dt_step, false);
      e.half_potential(dt_step / 2, false);
      e.copy_slot(kSlotB, kPsi);
      e.copy_slot(kPsi, kSlotA);
      const double dt_half = dt_step / 2;
      for (int r = 0; r < 2; ++r) {
        e.half_potential(dt_half / 2, false);
        kinetic(ws, dt_half, false);
        e.half_potential(dt_half / 2, false);
      }
      const double err = e.l2_change(kSlotB, kPsi);
      if (may_reject && err > p->tol) {
        e.copy_slot(kPsi, kSlotA);
        const double factor = std::max(0.5, 0.9 * std::cbrt(p->tol / err));
        dt = std::max(dt_step * factor, p->dt_min);
        ++n_rej;
        continue;
      }
      e.apply_loss(dt_step);  // src/adaptive.jl:262-264
      e.t += dt_step;
      e.step += 1;
      ++n_acc;
      if (!is_clamped) {
        const double factor = err > 1e-300 ? std::min(2.0, 0.9 * std::cbrt(p->tol / err)) : 2.0;
        dt = std::min(std::max(dt * factor, p->dt_min), p->dt_max);
      }
      if (e.t >= next_save - 1e-14) {
        check_cb(snapshot(ws, cb, user));
        next_save += save_interval;
      }
    }
  }
  e.sync();
  if (out) {
    out->n_accepted = n_acc;
    out->n_rejected = n_rej;
    out->final_dt = dt;
  }
  SBEC_API_END
}

// run_simulation_yoshida! (src/yoshida.jl:11-98)
sbec_status sbec_run_yoshida(sbec_ws* ws, const sbec_adaptive_params* p, double t_end, double save_interval,
                             int64_t max_accepted, sbec_callback cb, void* user, sbec_adaptive_result* out) {
  SBEC_API_BEGIN
  EngineBase& e = E(ws);
  need(p, "params");
  if (!(p->dt_init > 0) || !(p->dt_min > 0) || !(p->dt_max >= p->dt_min) || !(p->tol > 0))
    fail(SBEC_ERR_INVALID, "invalid AdaptiveDtParams");
  double dt = std::min(std::max(p->dt_init, p->dt_min), p->dt_max);
  long long n_acc = 0, n_rej = 0;
  check_cb(snapshot(ws, cb, user));
  double next_save = e.t + save_interval;
  while (e.t < t_end - 1e-14) {
    if (max_accepted > 0 && n_acc >= max_accepted) break;
    double dt_step = std::min(dt, t_end - e.t);
    const double rem = next_save - e.t;
    if (rem > 1e-14 && rem < dt_step) dt_step = rem;
    dt_step = std::max(dt_step, p->dt_min);
    const bool is_clamped = dt_step < dt * 0.99;
    e.copy_slot(kSlotA, kPsi);
    strang_core(ws, dt_step);
    e.copy_slot(kSlotB, kPsi);
    e.copy_slot(kPsi, kSlotA);
    yoshida_core(ws, dt_step);
    const double err = e.l2_change(kPsi, kSlotB);
    if (!is_clamped && err > p->tol && dt_step > p->dt_min * 1.01) {
      e.copy_slot(kPsi, kSlotA);
      const double factor = std::max(0.3, 0.9 * std::pow(p->tol / err, 0.2));
      dt = std::max(dt_step * factor, p->dt_min);
      ++n_rej;
      continue;
    }
    e.apply_loss(dt_step);  // src/yoshida.jl:64-66
    e.t += dt_step;
    e.step += 1;
    ++n_acc;
    if (!is_clamped) {
      const double factor = err > 1e-300 ? std::min(3.0, 0.9 * std::pow(p->tol / err, 0.2)) : 3.0;
      dt = std::min(std::max(dt * factor, p->dt_min), p->dt_max);
    }
    if (e.t >= next_save - 1e-14) {
      check_cb(snapshot(ws, cb, user));
      next_save += save_interval;
    }
  }
  e.sync();
  if (out) {
    out->n_accepted = n_acc;
    out->n_rejected = n_rej;
    out->final_dt = dt;
  }
  SBEC_API_END
}

// find_ground_state ITP loop (src/ground_state.jl:116-169)
sbec_status sbec_ground_state(sbec_ws* ws, int64_t n_steps, double tol, int64_t check_every, double target_Mz,
                              sbec_gs_result* out) {
  SBEC_API_BEGIN
  EngineBase& e = E(ws);
  if (!e.itp) fail(SBEC_ERR_INVALID, "sbec_ground_state needs an imaginary-time workspace");
  if (n_steps <= 0 || check_every <= 0) fail(SBEC_ERR_INVALID, "n_steps and check_every must be positive");
  const bool use_c = !std::isnan(target_Mz);
  if (use_c) normalize_constrained(e, target_Mz);
  double E_prev = total_energy(e);
  bool converged = false;
  e.copy_slot(kSlotA, kPsi);
  double final_dE = NAN, final_dpsi = NAN;
  int64_t steps = 0;
  for (int64_t step = 1; step <= n_steps; ++step) {
    if (!use_c && step > 10 && step % check_every != 0) {
      // run steps step..nxt in one fused block: up to the step before the next
      // convergence check, or to n_steps when no check remains
      const int64_t nxt = std::min(n_steps, (step / check_every + 1) * check_every - 1);
      split_steps(ws, nxt - step + 1);
      step = nxt;
      steps = step;
      if (step == n_steps) break;
      continue;
    }
    split_steps(ws, 1);
    steps = step;
    if (step <= 10) check_itp_overflow(e, step);
    if (use_c) normalize_constrained(e, target_Mz);
    if (step % check_every == 0) {
      const double En = total_energy(e);
      const double dE = std::fabs(En - E_prev);
      double pmax = 0, dmax = 0;
      e.max_abs(kPsi, kSlotA, &pmax, &dmax);
      const double dpsi = pmax > 0 ? dmax / pmax : 0.0;
      final_dE = dE;
      final_dpsi = dpsi;
      if (dE < std::max(tol, 0.5 * e.psi_resolution() * std::fabs(En)) &&
          dpsi < std::max(tol, e.psi_resolution())) {
        converged = true;
        break;
      }
      E_prev = En;
      e.copy_slot(kSlotA, kPsi);
    }
  }
  const double Efin = total_energy(e);
  if (out) {
    out->converged = converged ? 1 : 0;
    out->energy = Efin;
    out->dE = final_dE;
    out->dpsi = final_dpsi;
    out->steps = steps;
  }
  SBEC_API_END
}

// _find_ground_state_adaptive (src/ground_state.jl:172-237): blocks of check_every
// split steps; the block is kept when the energy did not rise (dt grows by 10 %, capped
// at dt_max), otherwise psi returns to the block's start and dt halves (floor 1e-8).
// The NaN / DDI-overflow guard runs once, after the very first step (:193).  The
// backup of psi stays on the device (slot A); _rebuild_workspace_with_dt (:380-392) is
// a new dt for the ITP kinetic phase.
sbec_status sbec_ground_state_adaptive(sbec_ws* ws, int64_t n_steps, double tol, double dt_max,
                                       sbec_gs_result* out, double* final_dt) {
  SBEC_API_BEGIN
  EngineBase& e = E(ws);
  if (!e.itp || e.normalize_every != 1)
    fail(SBEC_ERR_INVALID, "sbec_ground_state_adaptive needs an imaginary-time workspace with normalize_every=1");
  if (n_steps <= 0) fail(SBEC_ERR_INVALID, "n_steps must be positive");
  if (!(dt_max > 0)) fail(SBEC_ERR_INVALID, "dt_max must be positive");
  const int64_t check_every = std::max<int64_t>(1, n_steps / 100);
  auto set_dt = [&](double dt) {
    e.dt = dt;
    ws->kin_dt = dt;
    ws->kin_itp = true;
  };
  double current_dt = e.dt;
  double E_prev = total_energy(e);
  bool converged = false;
  int64_t total = 0;
  double final_dE = NAN, final_dpsi = NAN;
  while (total < n_steps) {
    e.copy_slot(kSlotA, kPsi);
    if (total == 0) {
      split_steps(ws, 1);
      check_itp_overflow(e, 1);
      if (check_every > 1) split_steps(ws, check_every - 1);
    } else {
      split_steps(ws, check_every);
    }
    total += check_every;
    const double En = total_energy(e);
    if (std::isnan(En) || En > E_prev) {
      e.copy_slot(kPsi, kSlotA);
      current_dt = std::max(current_dt * 0.5, 1e-8);
      set_dt(current_dt);
    } else {
      const double dE = std::fabs(En - E_prev);
      double pmax = 0, dmax = 0;
      e.max_abs(kPsi, kSlotA, &pmax, &dmax);
      const double dpsi = pmax > 0 ? dmax / pmax : 0.0;
      final_dE = dE;
      final_dpsi = dpsi;
      if (dE < std::max(tol, 0.5 * e.psi_resolution() * std::fabs(En)) &&
          dpsi < std::max(tol, e.psi_resolution())) {
        converged = true;
        break;
      }
      E_prev = En;
      const double new_dt = std::min(current_dt * 1.1, dt_max);
      if (new_dt != current_dt) {
        current_dt = new_dt;
        set_dt(current_dt);
      }
    }
  }
  const double Efin = total_energy(e);
  if (out) {
    out->converged = converged ? 1 : 0;
    out->energy = Efin;
    out->dE = final_dE;
    out->dpsi = final_dpsi;
    out->steps = total;
  }
  if (final_dt) *final_dt = current_dt;
  SBEC_API_END
}

sbec_status sbec_total_energy(sbec_ws* ws, double* Eout) {
  SBEC_API_BEGIN
  need(Eout, "E");
  E(ws);
  zee(ws);
  *Eout = total_energy(E(ws));
  SBEC_API_END
}

sbec_status sbec_energy_breakdown(sbec_ws* ws, sbec_energy_terms* out) {
  SBEC_API_BEGIN
  need(out, "out");
  E(ws);
  zee(ws);
  *out = E(ws).energy_terms();
  SBEC_API_END
}

// estimate_splitting_error (src/diagnostics.jl:214-251): one split step of dt against two of
// dt/2 (kinetic phase and potential steps at dt/2) from the same state; returns
// max|psi_1 - psi_2| / max|psi|.  psi, t and step are restored (the saved psi stays on the
// device, slot A).
sbec_status sbec_estimate_splitting_error(sbec_ws* ws, double* err) {
  SBEC_API_BEGIN
  need(err, "err");
  EngineBase& e = E(ws);
  const double t0 = e.t, dt = e.dt, kdt = ws->kin_dt;
  const long long s0 = e.step;
  const bool kit = ws->kin_itp;
  e.copy_slot(kSlotA, kPsi);
  split_steps(ws, 1);
  e.copy_slot(kSlotB, kPsi);
  e.copy_slot(kPsi, kSlotA);
  e.t = t0;
  e.step = s0;
  e.dt = dt / 2;
  ws->kin_dt = dt / 2;
  ws->kin_itp = e.itp;
  try {
    split_steps(ws, 2);
  } catch (...) {
    e.dt = dt;
    ws->kin_dt = kdt;
    ws->kin_itp = kit;
    throw;
  }
  e.dt = dt;
  ws->kin_dt = kdt;
  ws->kin_itp = kit;
  double p1, d1, p0, d0;
  e.max_abs(kPsi, kSlotB, &p1, &d1);  // max |psi_half - psi_full|
  e.max_abs(kSlotA, kSlotA, &p0, &d0);  // max |psi| of the saved state
  e.copy_slot(kPsi, kSlotA);
  e.t = t0;
  e.step = s0;
  *err = d1 / p0;
  SBEC_API_END
}

// validate_conservation's measurement (src/diagnostics.jl:259-293): the relative drifts of the
// norm, the energy and Mz over n split steps (Mz relative to max(|Mz0|, 1e-10)); psi, t and step
// are restored.  The tolerance test stays with the caller.
sbec_status sbec_conservation_drift(sbec_ws* ws, int64_t n_steps, double* norm_drift, double* energy_drift,
                                    double* mag_drift) {
  SBEC_API_BEGIN
  need(norm_drift, "norm_drift");
  need(energy_drift, "energy_drift");
  need(mag_drift, "mag_drift");
  if (n_steps < 0) fail(SBEC_ERR_INVALID, "n_steps must be non-negative");
  EngineBase& e = E(ws);
  const double t0 = e.t;
  const long long s0 = e.step;
  e.copy_slot(kSlotA, kPsi);
  double N0, M0, N1, M1;
  norm_and_mz(e, &N0, &M0);
  zee(ws);
  const double E0 = total_energy(e);
  split_steps(ws, n_steps);
  norm_and_mz(e, &N1, &M1);
  zee(ws);
  const double E1 = total_energy(e);
  e.copy_slot(kPsi, kSlotA);
  e.t = t0;
  e.step = s0;
  zee(ws);
  *norm_drift = std::fabs(N1 - N0) / std::max(N0, 1e-30);
  *energy_drift = std::fabs(E1 - E0) / std::max(std::fabs(E0), 1e-30);
  *mag_drift = std::fabs(M1 - M0) / std::max(std::fabs(M0), 1e-10);
  SBEC_API_END
}

sbec_status sbec_total_norm(sbec_ws* ws, double* norm) {
  SBEC_API_BEGIN
  need(norm, "norm");
  double mz;
  norm_and_mz(E(ws), norm, &mz);
  SBEC_API_END
}

sbec_status sbec_magnetization(sbec_ws* ws, double* Mz) {
  SBEC_API_BEGIN
  need(Mz, "Mz");
  double n;
  norm_and_mz(E(ws), &n, Mz);
  SBEC_API_END
}

sbec_status sbec_spin_density(sbec_ws* ws, double* out) {
  SBEC_API_BEGIN
  need(out, "out");
  E(ws).spin_density(out);
  SBEC_API_END
}

sbec_status sbec_ddi_potential(sbec_ws* ws, int32_t padded, double* out) {
  SBEC_API_BEGIN
  need(out, "out");
  E(ws).ddi_potential(padded != 0, out);
  SBEC_API_END
}

sbec_status sbec_classify_phase(sbec_ws* ws, sbec_phase_info* out) {
  SBEC_API_BEGIN
  need(out, "out");
  classify_phase(E(ws), -1, out);
  SBEC_API_END
}

// ---- batches of independent ITP solves (find_ground_state per solve, one schedule)
namespace {

// Options a batch takes (the same for every group of a batch).
void check_batch_options(const sbec_config* cfg) {
  if (!cfg->imaginary_time || cfg->normalize_every != 1)
    fail(SBEC_ERR_INVALID, "batched ground states need imaginary_time=1 and normalize_every=1");
  if (cfg->gS_direct || cfg->enable_ddi || cfg->raman || !(cfg->loss_gamma_dr < 1e-30 && cfg->loss_L3 < 1e-30))
    fail(SBEC_ERR_UNSUPPORTED,
         "batched ground states support contact c0/c1 (+LHY, nematic c2) couplings without DDI, Raman or losses");
}

// One group's grid and spin: argument errors, then the fused passes the batch runs on (no
// tensor step — c_extra may carry the nematic c2, shared by every solve, but not an even c_k
// with k >= 4 — D in {1, 3, 5}, power-of-two axes), all before any device work (the same test
// as sbec_batch_supported).
void check_batch_group(const sbec_config* cfg) {
  const Setup s = build_setup(*cfg);
  if (!fused_path_supported(s, cfg->precision == SBEC_FP32_BULK))
    fail(SBEC_ERR_UNSUPPORTED,
         "batched ground states need the fused passes: no tensor step, D in {1, 3, 5}, power-of-two axes "
         "and a row pass that fits the first axis");
}

std::unique_ptr<EngineBase> make_batch_group(const sbec_config& cfg, int n, const double* c0, const double* c1,
                                             const double* psi, const double* V) {
  Setup s = build_setup(cfg);
  auto e = cfg.precision == SBEC_FP32_BULK ? make_engine_f32(s) : make_engine_f64(s);
  e->zeeman_p = cfg.zeeman_p;
  e->zeeman_q = cfg.zeeman_q;
  e->dt = cfg.dt;
  e->itp = true;
  e->normalize_every = 1;
  if (V) e->set_potential(V);
  e->batch_init(n, c0, c1, psi);
  return e;
}

// The find_ground_state ITP loop (src/ground_state.jl:116-169) for every solve of one group;
// a solve leaves the active set at the check where it converges.  The NaN guard of steps
// 1-10 (src/ground_state.jl:4-29) is evaluated once, at step 10.  out: the group's solves.
// find_ground_state's loop (src/ground_state.jl:116-169) for every solve of one group: solve s
// runs up to n_steps[s] steps with its convergence test every check_every[s] steps (the
// previous psi and energy are those of its own last check).  The active solves advance
// together in blocks that end at the next step where some solve checks or stops; a solve
// leaves the batch when it converges or reaches its step limit.
void batch_ground_state(EngineBase& e, const int64_t* n_steps, double tol, const int64_t* check_every,
                        sbec_gs_result* out) {
  const int n = e.n_solves();
  std::vector<int> active;
  int64_t max_steps = 0;
  for (int i = 0; i < n; ++i) {
    active.push_back(i);
    max_steps = std::max(max_steps, n_steps[i]);
  }
  e.batch_set_active(active);
  std::vector<double> E_prev(n), E(n), pmax(n), dmax(n);
  e.batch_energies(E_prev.data());
  e.batch_save_prev();
  for (int i = 0; i < n; ++i) out[i] = sbec_gs_result{0, NAN, NAN, NAN, n_steps[i]};
  const int64_t nan_step = std::min<int64_t>(10, max_steps);
  int64_t step = 0;
  while (!active.empty()) {
    int64_t nxt = INT64_MAX;
    for (int s : active) nxt = std::min(nxt, std::min(n_steps[s], (step / check_every[s] + 1) * check_every[s]));
    if (step < nan_step) nxt = std::min(nxt, nan_step);
    e.batch_itp_steps(nxt - step, e.dt);
    step = nxt;
    if (step == nan_step && e.batch_has_nan())
      fail(SBEC_ERR_NUMERIC, "NaN detected in ITP within the first 10 steps. Likely potential overflow. Reduce dt.");
    bool any_check = false, any_end = false;
    for (int s : active) {
      any_check = any_check || step % check_every[s] == 0;
      any_end = any_end || step == n_steps[s];
    }
    if (!any_check && !any_end) continue;
    e.batch_energies(E.data());
    if (any_check) e.batch_max_abs(pmax.data(), dmax.data());
    std::vector<int> keep;
    for (int s : active) {
      bool leave = false;
      if (step % check_every[s] == 0) {
        const double dE = std::fabs(E[s] - E_prev[s]);
        const double dpsi = pmax[s] > 0 ? dmax[s] / pmax[s] : 0.0;
        out[s].dE = dE;
        out[s].dpsi = dpsi;
        if (dE < std::max(tol, 0.5 * e.psi_resolution() * std::fabs(E[s])) &&
            dpsi < std::max(tol, e.psi_resolution())) {
          out[s].converged = 1;
          leave = true;
        } else {
          E_prev[s] = E[s];
          e.batch_save_prev_solve(s);
        }
      }
      if (leave || step == n_steps[s]) {
        out[s].energy = E[s];
        out[s].steps = step;
      } else {
        keep.push_back(s);
      }
    }
    if (keep.size() != active.size()) {
      active = keep;
      e.batch_set_active(active);
    }
  }
  e.sync();
}

EngineBase& batch_solve(sbec_batch* b, int32_t solve, int* local) {
  need(b, "batch");
  if (solve < 0 || solve >= b->n()) fail(SBEC_ERR_INVALID, "solve index out of range");
  *local = b->loc[solve];
  return *b->groups[b->grp[solve]];
}

}  // namespace

sbec_status sbec_batch_create(const sbec_config* cfg, int32_t n_solves, const double* c0, const double* c1,
                              const double* psi, const double* V, sbec_batch** out) {
  SBEC_API_BEGIN
  need(cfg, "config");
  need(c0, "c0");
  need(c1, "c1");
  need(psi, "psi");
  need(out, "out");
  *out = nullptr;
  check_batch_options(cfg);  // argument and support errors before the device check
  check_batch_group(cfg);
  if (sbec_device_count() < 1) fail(SBEC_ERR_DEVICE, "no CUDA device available (the GPU path has no CPU fallback)");
  auto b = std::make_unique<sbec_batch>();
  b->groups.push_back(make_batch_group(*cfg, n_solves, c0, c1, psi, V));
  for (int i = 0; i < n_solves; ++i) {
    b->grp.push_back(0);
    b->loc.push_back(i);
  }
  *out = b.release();
  SBEC_API_END
}

namespace {

// Solves grouped by grid and spin F (first appearance order): one engine per group, all solves
// of a group sharing its potential.  F = null: every solve has cfg->F.
sbec_batch* batch_create_grouped(const sbec_config* cfg, int32_t n_solves, const int32_t* F, const int32_t* n,
                                 const double* L, const double* c0, const double* c1, const double* const* psi,
                                 const double* const* V) {
  need(cfg, "config");
  need(n, "n");
  need(L, "L");
  need(c0, "c0");
  need(c1, "c1");
  need(psi, "psi");
  if (n_solves < 1) fail(SBEC_ERR_INVALID, "n_solves must be >= 1");
  check_batch_options(cfg);
  std::vector<sbec_config> gcfg;
  std::vector<std::vector<int>> members;
  std::vector<int> grp(n_solves), loc(n_solves);
  for (int i = 0; i < n_solves; ++i) {
    sbec_config c = *cfg;
    if (F) c.F = F[i];
    for (int d = 0; d < 3; ++d) {
      c.n[d] = d < cfg->ndim ? n[3 * i + d] : 1;
      c.L[d] = d < cfg->ndim ? L[3 * i + d] : 1.0;
    }
    int g = -1;
    for (size_t k = 0; k < gcfg.size(); ++k) {
      bool same = gcfg[k].F == c.F;
      for (int d = 0; d < cfg->ndim; ++d) same = same && gcfg[k].n[d] == c.n[d] && gcfg[k].L[d] == c.L[d];
      if (same) g = (int)k;
    }
    if (g < 0) {
      check_batch_group(&c);  // argument and support errors of this grid and F before any device work
      g = (int)gcfg.size();
      gcfg.push_back(c);
      members.emplace_back();
    }
    need(psi[i], "psi[i]");
    if (V && !members[g].empty()) {
      const double* v0 = V[members[g][0]];
      long long N = 1;
      for (int d = 0; d < cfg->ndim; ++d) N *= c.n[d];
      const bool same = (V[i] == v0) || (V[i] && v0 && std::memcmp(V[i], v0, sizeof(double) * N) == 0);
      if (!same) fail(SBEC_ERR_INVALID, "solves on the same grid must share one potential");
    }
    grp[i] = g;
    loc[i] = (int)members[g].size();
    members[g].push_back(i);
  }
  if (sbec_device_count() < 1) fail(SBEC_ERR_DEVICE, "no CUDA device available (the GPU path has no CPU fallback)");
  auto b = std::make_unique<sbec_batch>();
  b->grp = grp;
  b->loc = loc;
  for (size_t g = 0; g < gcfg.size(); ++g) {
    const auto& m = members[g];
    long long N = 1;
    for (int d = 0; d < cfg->ndim; ++d) N *= gcfg[g].n[d];
    const size_t per = (size_t)2 * N * (2 * gcfg[g].F + 1);
    std::vector<double> gc0, gc1, gpsi(per * m.size());
    for (size_t k = 0; k < m.size(); ++k) {
      gc0.push_back(c0[m[k]]);
      gc1.push_back(c1[m[k]]);
      std::memcpy(gpsi.data() + k * per, psi[m[k]], sizeof(double) * per);
    }
    b->groups.push_back(make_batch_group(gcfg[g], (int)m.size(), gc0.data(), gc1.data(), gpsi.data(),
                                         V ? V[m[0]] : nullptr));
  }
  return b.release();
}

}  // namespace

sbec_status sbec_batch_create_grids(const sbec_config* cfg, int32_t n_solves, const int32_t* n, const double* L,
                                    const double* c0, const double* c1, const double* const* psi,
                                    const double* const* V, sbec_batch** out) {
  SBEC_API_BEGIN
  need(out, "out");
  *out = nullptr;
  *out = batch_create_grouped(cfg, n_solves, nullptr, n, L, c0, c1, psi, V);
  SBEC_API_END
}

sbec_status sbec_batch_create_mixed(const sbec_config* cfg, int32_t n_solves, const int32_t* F, const int32_t* n,
                                    const double* L, const double* c0, const double* c1,
                                    const double* const* psi, const double* const* V, sbec_batch** out) {
  SBEC_API_BEGIN
  need(out, "out");
  need(F, "F");
  *out = nullptr;
  *out = batch_create_grouped(cfg, n_solves, F, n, L, c0, c1, psi, V);
  SBEC_API_END
}

sbec_status sbec_batch_supported(const sbec_config* cfg, int32_t* supported) {
  SBEC_API_BEGIN
  need(cfg, "config");
  need(supported, "supported");
  *supported = 0;
  const Setup s = build_setup(*cfg);  // argument errors are errors
  const bool contact = !s.tensor && !cfg->gS_direct && !cfg->enable_ddi && !cfg->raman &&
                       cfg->loss_gamma_dr < 1e-30 && cfg->loss_L3 < 1e-30;
  *supported = cfg->imaginary_time && cfg->normalize_every == 1 && contact &&
               fused_path_supported(s, cfg->precision == SBEC_FP32_BULK);
  SBEC_API_END
}

sbec_status sbec_batch_destroy(sbec_batch* b) {
  SBEC_API_BEGIN
  delete b;
  SBEC_API_END
}

sbec_status sbec_batch_get_psi(sbec_batch* b, int32_t solve, double* psi) {
  SBEC_API_BEGIN
  need(psi, "psi");
  int l = 0;
  EngineBase& e = batch_solve(b, solve, &l);
  e.batch_get_psi(l, psi);
  SBEC_API_END
}

sbec_status sbec_batch_classify_phase(sbec_batch* b, int32_t solve, sbec_phase_info* out) {
  SBEC_API_BEGIN
  need(out, "out");
  int l = 0;
  EngineBase& e = batch_solve(b, solve, &l);
  classify_phase(e, l, out);
  SBEC_API_END
}

sbec_status sbec_batch_energies(sbec_batch* b, double* E) {
  SBEC_API_BEGIN
  need(b, "batch");
  need(E, "E");
  for (size_t g = 0; g < b->groups.size(); ++g) {
    EngineBase& e = *b->groups[g];
    std::vector<int> all(e.n_solves());
    for (int i = 0; i < e.n_solves(); ++i) all[i] = i;
    e.batch_set_active(all);
    std::vector<double> Eg(e.n_solves());
    e.batch_energies(Eg.data());
    for (int i = 0; i < b->n(); ++i)
      if (b->grp[i] == (int)g) E[i] = Eg[b->loc[i]];
  }
  SBEC_API_END
}

namespace {
void batch_ground_state_all(sbec_batch* b, const int64_t* n_steps, double tol, const int64_t* check_every,
                            sbec_gs_result* out);
}  // namespace

// The groups' ITP loops run concurrently, one host thread per group (each group has its own
// stream, buffers and graphs); results in the caller's solve order.
sbec_status sbec_batch_ground_state(sbec_batch* b, int64_t n_steps, double tol, int64_t check_every,
                                    sbec_gs_result* out) {
  SBEC_API_BEGIN
  need(b, "batch");
  need(out, "out");
  if (n_steps <= 0 || check_every <= 0) fail(SBEC_ERR_INVALID, "n_steps and check_every must be positive");
  std::vector<int64_t> ns((size_t)b->n(), n_steps), ce((size_t)b->n(), check_every);
  batch_ground_state_all(b, ns.data(), tol, ce.data(), out);
  SBEC_API_END
}

sbec_status sbec_batch_ground_state_each(sbec_batch* b, const int64_t* n_steps, double tol,
                                         const int64_t* check_every, sbec_gs_result* out) {
  SBEC_API_BEGIN
  need(b, "batch");
  need(n_steps, "n_steps");
  need(check_every, "check_every");
  need(out, "out");
  for (int i = 0; i < b->n(); ++i)
    if (n_steps[i] <= 0 || check_every[i] <= 0) fail(SBEC_ERR_INVALID, "n_steps and check_every must be positive");
  batch_ground_state_all(b, n_steps, tol, check_every, out);
  SBEC_API_END
}

sbec_status sbec_batch_set_graph_mode(sbec_batch* b, int32_t graphs) {
  SBEC_API_BEGIN
  need(b, "batch");
  for (auto& g : b->groups) g->set_graphs(graphs != 0);
  SBEC_API_END
}

namespace {

// Every group of the batch (its solves' entries of the per-solve arrays); groups on their
// own threads (and streams) when there are several.
void batch_ground_state_all(sbec_batch* b, const int64_t* n_steps, double tol, const int64_t* check_every,
                            sbec_gs_result* out) {
  const size_t G = b->groups.size();
  std::vector<std::vector<sbec_gs_result>> res(G);
  std::vector<std::vector<int64_t>> gn(G), gc(G);
  for (size_t g = 0; g < G; ++g) {
    res[g].resize(b->groups[g]->n_solves());
    gn[g].resize(b->groups[g]->n_solves());
    gc[g].resize(b->groups[g]->n_solves());
  }
  for (int i = 0; i < b->n(); ++i) {
    gn[b->grp[i]][b->loc[i]] = n_steps[i];
    gc[b->grp[i]][b->loc[i]] = check_every[i];
  }
  if (G == 1) {
    batch_ground_state(*b->groups[0], gn[0].data(), tol, gc[0].data(), res[0].data());
  } else {
    int dev = 0;
    cuda_check(cudaGetDevice(&dev), "cudaGetDevice");
    std::vector<std::thread> th;
    std::vector<SbecError> err(G, SbecError{SBEC_OK, ""});
    for (size_t g = 0; g < G; ++g)
      th.emplace_back([&, g] {
        try {
          cuda_check(cudaSetDevice(dev), "cudaSetDevice");
          batch_ground_state(*b->groups[g], gn[g].data(), tol, gc[g].data(), res[g].data());
        } catch (const SbecError& e) {
          err[g] = e;
        } catch (const std::exception& e) {
          err[g] = SbecError{SBEC_ERR_DEVICE, e.what()};
        }
      });
    for (auto& t : th) t.join();
    for (const auto& e : err)
      if (e.status != SBEC_OK) throw e;
  }
  for (int i = 0; i < b->n(); ++i) out[i] = res[b->grp[i]][b->loc[i]];
}

}  // namespace

sbec_status sbec_profile_enable(sbec_ws* ws, int32_t enable) {
  SBEC_API_BEGIN
  E(ws).sync();
  E(ws).prof.enable(enable != 0);
  SBEC_API_END
}

sbec_status sbec_profile_read(sbec_ws* ws, sbec_kernel_stat* out, int32_t max, int32_t* n) {
  SBEC_API_BEGIN
  const auto& st = E(ws).prof.read();
  int32_t i = 0;
  for (const auto& kv : st) {
    if (out && i < max) {
      std::memset(out[i].name, 0, sizeof(out[i].name));
      std::strncpy(out[i].name, kv.first.c_str(), sizeof(out[i].name) - 1);
      out[i].launches = kv.second.launches;
      out[i].ms = kv.second.ms;
      out[i].bytes = kv.second.bytes;
    }
    ++i;
  }
  if (n) *n = i;
  SBEC_API_END
}

sbec_status sbec_launch_count(sbec_ws* ws, int64_t* n) {
  SBEC_API_BEGIN
  need(n, "n");
  *n = E(ws).prof.total_launches();
  SBEC_API_END
}

sbec_status sbec_ws_stream(sbec_ws* ws, void** stream) {
  SBEC_API_BEGIN
  need(stream, "stream");
  *stream = (void*)E(ws).stream();
  SBEC_API_END
}

static void copy_report(const std::string& r, char* buf, int64_t cap, int64_t* len) {
  if (len) *len = (int64_t)r.size();
  if (buf && cap > 0) {
    const size_t n = std::min<size_t>(r.size(), (size_t)cap - 1);
    std::memcpy(buf, r.data(), n);
    buf[n] = 0;
  }
}

sbec_status sbec_set_snapshot_mode(sbec_ws* ws, int32_t pipelined) {
  SBEC_API_BEGIN
  need(ws, "workspace");
  ws->pipelined_snapshots = pipelined != 0;
  SBEC_API_END
}

sbec_status sbec_set_graph_mode(sbec_ws* ws, int32_t graphs) {
  SBEC_API_BEGIN
  need(ws, "workspace");
  ws->eng->set_graphs(graphs != 0);
  SBEC_API_END
}

sbec_status sbec_tuning_report(sbec_ws* ws, char* buf, int64_t cap, int64_t* len) {
  SBEC_API_BEGIN
  copy_report(E(ws).tuning_report(), buf, cap, len);
  SBEC_API_END
}

sbec_status sbec_tune_table_export(char* buf, int64_t cap, int64_t* len) {
  SBEC_API_BEGIN
  std::string r;
  {
    std::lock_guard<std::mutex> lock(tune_table_mutex());
    for (const auto& kv : tune_table_map()) r += kv.first + "\t" + std::to_string(kv.second) + "\n";
  }
  copy_report(r, buf, cap, len);
  SBEC_API_END
}

sbec_status sbec_tune_freeze(int32_t frozen) {
  SBEC_API_BEGIN
  tune_frozen().store(frozen != 0);
  SBEC_API_END
}

sbec_status sbec_tune_table_import(const char* text) {
  SBEC_API_BEGIN
  need(text, "text");
  std::map<std::string, int> add;
  const std::string t(text);
  size_t pos = 0;
  while (pos < t.size()) {
    size_t eol = t.find('\n', pos);
    if (eol == std::string::npos) eol = t.size();
    const std::string line = t.substr(pos, eol - pos);
    pos = eol + 1;
    if (line.empty()) continue;
    const size_t tab = line.rfind('\t');
    if (tab == std::string::npos || tab == 0) fail(SBEC_ERR_INVALID, "tune table line without a tab: " + line);
    char* end = nullptr;
    const long v = std::strtol(line.c_str() + tab + 1, &end, 10);
    if (end == line.c_str() + tab + 1 || *end != 0 || v < 0 || v > 255)
      fail(SBEC_ERR_INVALID, "tune table line with a bad variant: " + line);
    add[line.substr(0, tab)] = (int)v;
  }
  std::lock_guard<std::mutex> lock(tune_table_mutex());
  for (const auto& kv : add) tune_table_map()[kv.first] = kv.second;
  SBEC_API_END
}

sbec_status sbec_batch_tuning_report(sbec_batch* b, char* buf, int64_t cap, int64_t* len) {
  SBEC_API_BEGIN
  need(b, "batch");
  std::string r;
  for (const auto& g : b->groups) r += g->tuning_report() + "\n";
  copy_report(r, buf, cap, len);
  SBEC_API_END
}

}  // extern "C"
