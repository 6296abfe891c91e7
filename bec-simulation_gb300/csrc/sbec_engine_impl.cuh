// Engine<R>: device buffers of one workspace and the launch sequences of the
// split-step operators.  Included once per precision (sbec_engine_f64.cu,
// sbec_engine_f32.cu).
#pragma once

#include <cmath>
#include <complex>
#include <cstdlib>
#include <cstring>
#include <algorithm>
#include <map>
#include <mutex>
#include <tuple>
#include <type_traits>
#include <string>
#include <vector>

#include "sbec_engine.h"
#include "sbec_kernels.cuh"
#include "sbec_lines.h"

namespace sbec {

// ---------------------------------------------------------------------------
// Tile shapes
// ---------------------------------------------------------------------------
// Tiles are kept small (about 64 threads) so that the 2-D grids of a single solve
// (e.g. 768 lines of 256) still spread over all 152 SMs; strided tiles are at
// least one 32-byte sector wide so every global access moves whole sectors.
template <typename R, int MH>
constexpr int ddi_x_rows_per_block() {
  constexpr int tpl = MH / PlanOf<R, MH>::E;
  int lpb = 64 / (3 * tpl);
  if (lpb < 1) lpb = 1;
  while (lpb > 1 && (long)3 * lpb * (2 * MH + 1) * (int)sizeof(cplx<R>) > 96 * 1024) lpb /= 2;
  return lpb;
}

template <typename R, int M>
constexpr int ddi_last_width() {
  constexpr int tpl = M / PlanOf<R, M>::E;
  constexpr int sector = 32 / (int)sizeof(cplx<R>);
  int w = 64 / (3 * tpl);
  if (w < sector) w = sector;
  while (w > 1 && (3 * w * tpl > 1024 || (long)3 * w * M * (int)sizeof(cplx<R>) > 100 * 1024)) w /= 2;
  return w;
}

template <typename K>
inline void set_smem(K kernel, size_t bytes) {
  // opt in above 40 KB: dynamic plus the kernels' static shared arrays must fit the limit
  if (bytes > 40 * 1024) cuda_check(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes),
                                    "cudaFuncSetAttribute");
}

#define SBEC_SWITCH_POW2(n, FN, ...)                                 \
  switch (n) {                                                       \
    case 2: FN<2>(__VA_ARGS__); break;                               \
    case 4: FN<4>(__VA_ARGS__); break;                               \
    case 8: FN<8>(__VA_ARGS__); break;                               \
    case 16: FN<16>(__VA_ARGS__); break;                             \
    case 32: FN<32>(__VA_ARGS__); break;                             \
    case 64: FN<64>(__VA_ARGS__); break;                             \
    case 128: FN<128>(__VA_ARGS__); break;                           \
    case 256: FN<256>(__VA_ARGS__); break;                           \
    case 512: FN<512>(__VA_ARGS__); break;                           \
    case 1024: FN<1024>(__VA_ARGS__); break;                         \
    case 2048: FN<2048>(__VA_ARGS__); break;                         \
    case 4096: FN<4096>(__VA_ARGS__); break;                         \
    default: fail(SBEC_ERR_UNSUPPORTED, "unsupported FFT length " + std::to_string(n)); \
  }

#define SBEC_SWITCH_POW2_STRIDED(n, FN, ...)                         \
  switch (n) {                                                       \
    case 2: FN<2>(__VA_ARGS__); break;                               \
    case 4: FN<4>(__VA_ARGS__); break;                               \
    case 8: FN<8>(__VA_ARGS__); break;                               \
    case 16: FN<16>(__VA_ARGS__); break;                             \
    case 32: FN<32>(__VA_ARGS__); break;                             \
    case 64: FN<64>(__VA_ARGS__); break;                             \
    case 128: FN<128>(__VA_ARGS__); break;                           \
    case 256: FN<256>(__VA_ARGS__); break;                           \
    case 512: FN<512>(__VA_ARGS__); break;                           \
    case 1024: FN<1024>(__VA_ARGS__); break;                         \
    default: fail(SBEC_ERR_UNSUPPORTED, "unsupported FFT length " + std::to_string(n)); \
  }

#define SBEC_SWITCH_D(D, FN, ...)                                    \
  switch (D) {                                                       \
    case 1: FN<1>(__VA_ARGS__); break;                               \
    case 3: FN<3>(__VA_ARGS__); break;                               \
    case 5: FN<5>(__VA_ARGS__); break;                               \
    case 7: FN<7>(__VA_ARGS__); break;                               \
    case 9: FN<9>(__VA_ARGS__); break;                               \
    case 11: FN<11>(__VA_ARGS__); break;                             \
    case 13: FN<13>(__VA_ARGS__); break;                             \
    default: fail(SBEC_ERR_UNSUPPORTED, "unsupported component count"); \
  }

// ---------------------------------------------------------------------------
template <typename R>
class Engine final : public EngineBase {
 public:
  explicit Engine(const Setup& s) : EngineBase(s) {
    cuda_check(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking), "cudaStreamCreate");
    // SBEC_GRAPHS=0 / SBEC_PDL=0 turn off graph replay / programmatic dependent launch.
    if (const char* g = std::getenv("SBEC_GRAPHS")) use_graphs_ = std::atoi(g) != 0;
    if (const char* p = std::getenv("SBEC_PDL")) use_pdl_ = std::atoi(p) != 0;
    if (const char* t = std::getenv("SBEC_TUNE")) tune_on_ = std::atoi(t) != 0;
    if (const char* f = std::getenv("SBEC_TUNE_FORCE")) tune_force_ = std::atoi(f);
    if (const char* m = std::getenv("SBEC_BATCH_MERGED")) merged_itp_ = std::atoi(m) != 0;
    if (const char* t = std::getenv("SBEC_TENSOR_LANES")) tensor_mode_ = std::atoi(t);
    if (const char* g = std::getenv("SBEC_SEGMENT")) segment_on_ = std::atoi(g) != 0;
    if (const char* g = std::getenv("SBEC_ITP_STEPS")) use_itp_steps_ = std::atoi(g) != 0;
    // host-side fault injection for the tests: the segment barrier's arrival counter starts
    // beyond the block count, so no block is ever the last arriver and every wait runs out
    if (const char* f = std::getenv("SBEC_FAULT_SEGMENT_STALL")) segment_stall_ = std::atoi(f) != 0;
    const int D = s_.D;
    N_ = s_.N;
    nc_ = N_ * D;
    psi_[kPsi] = alloc<cplx<R>>(nc_);
    V_ = alloc<R>(N_);
    cuda_check(cudaMemsetAsync(V_, 0, sizeof(R) * N_, stream_), "memset V");
    for (int a = 0; a < s_.ndim; ++a) {
      ptab_[a] = alloc<cplx<R>>((size_t)s_.n[a] * (sizeof(R) == 4 ? 2 : 1));
      ptab_lo_[a] = nullptr;
    }
    for (int a = 0; a < s_.ndim; ++a) twiddle(s_.n[a]);
    partials_n_ = (size_t)kMaxBlocks * 16;
    partials_ = alloc<double>(partials_n_);
    results_ = alloc<double>(64);
    cuda_check(cudaMallocHost(&host_res_, 64 * sizeof(double)), "cudaMallocHost");
    cuda_check(cudaMallocHost(&host_psi_, sizeof(double) * 2 * nc_), "cudaMallocHost psi");
    if (sizeof(R) != 8) stage_ = alloc<double2>(nc_);
    // spin tables
    std::memset(&st_, 0, sizeof(st_));
    for (int i = 0; i < D; ++i)
      for (int j = 0; j < D; ++j) {
        const auto v = s_.FyV[(size_t)i * D + j], vt = s_.FyVt[(size_t)i * D + j];
        st_.V[i * D + j] = mk<R>((R)v.real(), (R)v.imag());
        st_.Vt[i * D + j] = mk<R>((R)vt.real(), (R)vt.imag());
      }
    for (int c = 0; c < D; ++c) {
      st_.fp[c] = (R)s_.fp[c];
      st_.m[c] = (R)s_.m[c];
    }
    if (s_.tensor) {
      G_ = alloc<double>(s_.G.size());
      upload(G_, s_.G.data(), s_.G.size());
      std::vector<float> g32(s_.G.begin(), s_.G.end());
      G32_ = alloc<float>(g32.size());
      upload(G32_, g32.data(), g32.size());
      const int np = (int)s_.pair_a.size();
      std::vector<int4> pairs(np);
      for (int q = 0; q < np; ++q) pairs[q] = make_int4(s_.pair_a[q], s_.pair_c1[q], s_.pair_c2[q], 0);
      pairs_ = alloc<int4>(std::max(np, 1));
      pcg_ = alloc<double>(std::max(np, 1));
      gA_ = alloc<double>(std::max((int)s_.gA.size(), 1));
      upload(pairs_, pairs.data(), np);
      upload(pcg_, s_.pair_cg.data(), np);
      upload(gA_, s_.gA.data(), s_.gA.size());
    }
    if (s_.ddi) {
      spin3_ = alloc<R>(3 * N_);
      phi3_ = alloc<R>(3 * N_);
      phi_per_ = alloc<R>(3 * N_);
      for (int kind = 0; kind < (s_.padded ? 2 : 1); ++kind) {
        DdiGeom g = geom(kind);
        spec_[kind] = alloc<cplx<R>>((size_t)3 * g.field_stride);
        twiddle(g.Mx / 2);
        twiddle(g.Mx);
        if (s_.ndim >= 2) twiddle(g.My);
        if (s_.ndim >= 3) twiddle(g.Mz);
      }
    }
    sync();
  }

  ~Engine() override {
    cudaStreamSynchronize(stream_);
    if (side_) {
      cudaStreamSynchronize(side_);
      cudaStreamDestroy(side_);
      for (auto& ev : copied_ev_)
        if (ev) cudaEventDestroy(ev);
    }
    for (auto& kv : graphs_)
      if (kv.second.exec) cudaGraphExecDestroy(kv.second.exec);
    for (void* p : allocs_) cudaFree(p);
    if (host_res_) cudaFreeHost(host_res_);
    if (bar_host_) cudaFreeHost(bar_host_);
    if (host_psi_) cudaFreeHost(host_psi_);
    for (int k = 0; k < 2; ++k) {
      if (snap_res_[k]) cudaFreeHost(snap_res_[k]);
      if (snap_psi_[k]) cudaFreeHost(snap_psi_[k]);
      if (snap_ev_[k]) cudaEventDestroy(snap_ev_[k]);
    }
    cudaStreamDestroy(stream_);
  }

  // ---------------- state ----------------
  void set_psi(const double* host) override {
    std::memcpy(host_psi_, host, sizeof(double) * 2 * nc_);
    upload_psi_from_pinned();
  }

  void get_psi(double* host) override {
    download_psi_to_pinned();
    sync();
    std::memcpy(host, host_psi_, sizeof(double) * 2 * nc_);
  }

  void set_potential(const double* host) override {
    if (sizeof(R) == 8) {
      cuda_check(cudaMemcpyAsync(V_, host, sizeof(double) * N_, cudaMemcpyHostToDevice, stream_), "V upload");
    } else {
      double* tmp = reinterpret_cast<double*>(stage_);
      cuda_check(cudaMemcpyAsync(tmp, host, sizeof(double) * N_, cudaMemcpyHostToDevice, stream_), "V upload");
      pb();
      k_real_from_f64<R><<<grid_for(N_), 256, 0, stream_>>>(tmp, V_, N_);
      done("convert", 12.0 * N_);
    }
    sync();
  }

  // ---------------- operators ----------------
  void half_potential(double dt_half, bool imaginary_time) override {
    const double tau_d = dt_half / 2;
    const double tau_s = dt_half / 2;
    const bool sm = !s_.tensor && std::fabs(s_.c1) >= 1e-30 && s_.D > 1;
    PotArgs<R> a = pot_args(tau_d, imaginary_time);
    a.tau_s = (R)tau_s;
    a.tau_ddi = (R)dt_half;
    a.tau_r = (R)(dt_half / 2);
    const int rm = s_.raman ? 1 : 0;
    if (s_.tensor && rm) {
      // tensor(tau/2), Raman(tau/2), [DDI(tau)], Raman(tau/2), tensor(tau/2) (src/split_step.jl:58-131)
      TensorArgs<R> ta = tensor_args(tau_d, tau_s, imaginary_time);
      ta.pre_diag = 1;
      ta.post_diag = 0;
      ta.n_apply = 1;
      launch_tensor(ta);
      PotArgs<R> r1 = a;
      r1.raman_a = 1;
      if (s_.ddi) {
        r1.spin_out = spin3_;
        launch_potential(r1);
        ddi_conv(s_.padded ? 1 : 0, spin3_, phi3_);
        PotArgs<R> r2 = a;
        r2.ddi_rot = 1;
        r2.phi = phi3_;
        r2.raman_b = 1;
        launch_potential(r2);
      } else {
        r1.raman_b = 1;
        launch_potential(r1);
      }
      ta.pre_diag = 0;
      ta.post_diag = 1;
      launch_tensor(ta);
      return;
    }
    if (s_.tensor) {
      TensorArgs<R> ta = tensor_args(tau_d, tau_s, imaginary_time);
      ta.pre_diag = 1;
      ta.post_diag = s_.ddi ? 0 : 1;
      ta.n_apply = s_.ddi ? 1 : 2;
      launch_tensor(ta);
      if (s_.ddi) {
        SBEC_SWITCH_D(s_.D, launch_spin_density_d, spin3_);
        ddi_conv(s_.padded ? 1 : 0, spin3_, phi3_);
        PotArgs<R> b = a;
        b.pre_diag = 0;
        b.rot_a = 0;
        b.rot_b = 0;
        b.post_diag = 0;
        b.ddi_rot = 1;
        b.phi = phi3_;
        launch_potential(b);
        ta.pre_diag = 0;
        ta.post_diag = 1;
        ta.n_apply = 1;
        launch_tensor(ta);
      }
      return;
    }
    if (!s_.ddi) {
      a.pre_diag = 1;
      a.rot_a = sm;
      a.nem_a = a.nem_b = nematic();
      a.raman_a = a.raman_b = rm;
      a.rot_b = sm;
      a.post_diag = 1;
      launch_potential(a);
      return;
    }
    PotArgs<R> first = a;
    first.pre_diag = 1;
    first.rot_a = sm;
    first.nem_a = nematic();
    first.raman_a = rm;
    first.spin_out = spin3_;
    launch_potential(first);
    ddi_conv(s_.padded ? 1 : 0, spin3_, phi3_);
    PotArgs<R> second = a;
    second.ddi_rot = 1;
    second.phi = phi3_;
    second.raman_b = rm;
    second.nem_b = nematic();
    second.rot_b = sm;
    second.post_diag = 1;
    launch_potential(second);
  }

  // apply_loss_step! (src/losses.jl:25-45) for a step of dt; no-op without losses.
  void apply_loss(double dt) override {
    if (!s_.loss) return;
    LossRates<R> lr{};
    for (int c = 0; c < s_.D; ++c) lr.r[c] = (R)s_.loss_rates[c];
    SBEC_SWITCH_D(s_.D, launch_loss_d, lr, (R)(dt / 2));
  }

  void kinetic(double dt_k, bool imaginary_time) override {
    update_phase(dt_k, imaginary_time);
    fft_full(psi_[kPsi], /*kinetic=*/true);
  }

  void normalize() override {
    comp_norms_async(psi_[kPsi]);
    pb();
    k_normalize_apply<R><<<grid_for(nc_), 256, 0, stream_>>>(psi_[kPsi], N_, s_.D, results_ + 1, s_.dV);
    done("normalize", 2.0 * (double)sizeof(cplx<R>) * nc_);
  }

  void scale_components(const double* w) override {
    std::memcpy(host_res_, w, sizeof(double) * s_.D);
    cuda_check(cudaMemcpyAsync(results_ + 32, host_res_, sizeof(double) * s_.D, cudaMemcpyHostToDevice, stream_),
               "weights");
    pb();
    k_scale_comp<R><<<grid_for(nc_), 256, 0, stream_>>>(psi_[kPsi], N_, s_.D, results_ + 32);
    done("elementwise", 2.0 * (double)sizeof(cplx<R>) * nc_);
    sync();
  }

  void copy_slot(int dst, int src) override {
    cuda_check(cudaMemcpyAsync(slot(dst), slot(src), sizeof(cplx<R>) * nc_, cudaMemcpyDeviceToDevice, stream_),
               "slot copy");
  }

  // ---------------- reductions ----------------
  void comp_norms(double* sums, double* nan_count) override {
    comp_norms_async(psi_[kPsi]);
    fetch(s_.D + 2);
    for (int c = 0; c < s_.D; ++c) sums[c] = host_res_[1 + c];
    if (nan_count) *nan_count = host_res_[1 + s_.D];
  }

  sbec_energy_terms energy_terms() override { return energy_terms_and_norms(nullptr); }

  const double* psi_to_pinned() override {
    download_psi_to_pinned();
    sync();
    return host_psi_;
  }

  // ---- pipelined snapshots: two pinned slots, each receiving the reduction sums and
  // the FP64 psi of one save point in stream order, with an event marking completion.
  // The host reads slot k while the stream already runs the next segment.
  void snapshot_enqueue(int k) override {
    k &= 1;
    if (!snap_res_[k]) {
      cuda_check(cudaMallocHost(&snap_res_[k], 32 * sizeof(double)), "cudaMallocHost");
      cuda_check(cudaMallocHost(&snap_psi_[k], sizeof(double) * 2 * nc_), "cudaMallocHost");
      cuda_check(cudaEventCreateWithFlags(&snap_ev_[k], cudaEventDisableTiming), "cudaEventCreate");
    }
    if (s_.ddi) {  // the dipolar energy shares the step's spin-density fields: stay on the step stream
      energy_enqueue();
      snapshot_copy_out(k, psi_[kPsi]);
      return;
    }
    // The step stream only copies psi (device to device); the reductions, the FP64
    // conversion and the host copies run on a second stream from that copy, so they
    // overlap the next segment instead of delaying it.
    if (!side_) {
      cuda_check(cudaStreamCreateWithFlags(&side_, cudaStreamNonBlocking), "cudaStreamCreate");
      for (int i = 0; i < 2; ++i) {
        cuda_check(cudaEventCreateWithFlags(&copied_ev_[i], cudaEventDisableTiming), "cudaEventCreate");
        snap_copy_[i] = alloc<cplx<R>>(nc_);
        if (sizeof(R) != 8) snap_stage_[i] = alloc<double2>(nc_);
      }
      side_partials_n_ = partials_n_;
      side_partials_ = alloc<double>(side_partials_n_);
      side_results_ = alloc<double>(64);
      side_scratch_ = alloc<cplx<R>>(nc_);
    }
    cuda_check(cudaMemcpyAsync(snap_copy_[k], psi_[kPsi], sizeof(cplx<R>) * nc_, cudaMemcpyDeviceToDevice, stream_),
               "snapshot copy");
    cuda_check(cudaEventRecord(copied_ev_[k], stream_), "cudaEventRecord");
    cuda_check(cudaStreamWaitEvent(side_, copied_ev_[k], 0), "cudaStreamWaitEvent");
    struct Redirect {  // the energy launches address these members; point them at the side set
      Engine* e;
      cplx<R>* psi;
      cudaStream_t st;
      double *part, *res;
      size_t part_n;
      cplx<R>* scr;
      double2* stage;
      Redirect(Engine* en, int slot) : e(en) {
        psi = e->psi_[kPsi];
        st = e->stream_;
        part = e->partials_;
        part_n = e->partials_n_;
        res = e->results_;
        scr = e->scratch_;
        stage = e->stage_;
        e->psi_[kPsi] = e->snap_copy_[slot];
        e->stream_ = e->side_;
        e->partials_ = e->side_partials_;
        e->partials_n_ = e->side_partials_n_;
        e->results_ = e->side_results_;
        e->scratch_ = e->side_scratch_;
        if (e->snap_stage_[slot]) e->stage_ = e->snap_stage_[slot];
      }
      ~Redirect() {
        e->psi_[kPsi] = psi;
        e->stream_ = st;
        e->partials_ = part;
        e->partials_n_ = part_n;
        e->results_ = res;
        e->scratch_ = scr;
        e->stage_ = stage;
      }
    } redirect(this, k);
    energy_enqueue();
    snapshot_copy_out(k, psi_[kPsi]);
  }

  // results_[0..31] and psi (as FP64) of the current stream into pinned slot k, then its event.
  void snapshot_copy_out(int k, const cplx<R>* src_psi) {
    cuda_check(cudaMemcpyAsync(snap_res_[k], results_, 32 * sizeof(double), cudaMemcpyDeviceToHost, stream_),
               "snapshot sums");
    const void* src = src_psi;
    if (sizeof(R) != 8) {
      pb();
      k_to_f64<R><<<grid_for(nc_), 256, 0, stream_>>>(src_psi, stage_, nc_);
      done("convert", (16.0 + (double)sizeof(cplx<R>)) * nc_);
      src = stage_;
    }
    cuda_check(cudaMemcpyAsync(snap_psi_[k], src, sizeof(double) * 2 * nc_, cudaMemcpyDeviceToHost, stream_),
               "snapshot psi");
    cuda_check(cudaEventRecord(snap_ev_[k], stream_), "cudaEventRecord");
  }

  const double* snapshot_wait(int k, sbec_energy_terms* terms, double* comp_sums) override {
    k &= 1;
    if (!snap_ev_[k]) fail(SBEC_ERR_INVALID, "no snapshot in flight");
    cuda_check(cudaEventSynchronize(snap_ev_[k]), "cudaEventSynchronize");
    *terms = energy_from(snap_res_[k], comp_sums);
    return snap_psi_[k];
  }

  void restore_snapshot(int k) override {
    sync();
    if (side_) cuda_check(cudaStreamSynchronize(side_), "cudaStreamSynchronize");
    set_psi(snap_psi_[k & 1]);
  }

  sbec_energy_terms energy_terms_and_norms(double* comp_sums) override {
    energy_enqueue();
    fetch(32);
    return energy_from(host_res_, comp_sums);
  }

  // Launch every reduction of the energy and the component norms; the sums land
  // in results_[0..31] (no host synchronisation).
  void energy_enqueue() {
    // kinetic: forward FFT of a copy, sum k^2 |psi_hat|^2 dV / N (src/energy.jl:56-65)
    cplx<R>* scr = slot_scratch();
    cuda_check(cudaMemcpyAsync(scr, psi_[kPsi], sizeof(cplx<R>) * nc_, cudaMemcpyDeviceToDevice, stream_), "copy");
    fft_full(scr, false);
    {
      PhaseTableArgs g = phase_geom(0.0, false);
      const int nb = red_blocks(nc_);
      pb();
      k_kinetic_sum<R><<<nb, kRedThreads, 0, stream_>>>(scr, N_, s_.D, g, partials_);
      done("reduce", (double)sizeof(cplx<R>) * nc_);
      finish<1>(nb, false, 0);
    }
    comp_norms_async(psi_[kPsi]);  // -> results_[1 .. D+1]
    {
      const int nb = red_blocks(N_);
      SBEC_SWITCH_D(s_.D, launch_energy_local_d, nb);
      finish<4>(nb, false, 20);
    }
    if (s_.tensor) {
      const int nb = red_blocks(N_);
      SBEC_SWITCH_D(s_.D, launch_tensor_energy_d, nb);
      finish<1>(nb, false, 30);
    }
    if (nematic()) {
      const int nb = red_blocks(N_);
      SBEC_SWITCH_D(s_.D, launch_pair_energy_d, nb);
      finish<1>(nb, false, 29);
    }
    if (s_.raman) {
      const int nb = red_blocks(N_);
      SBEC_SWITCH_D(s_.D, launch_raman_energy_d, nb);
      finish<1>(nb, false, 24);
    }
    if (s_.ddi) {
      SBEC_SWITCH_D(s_.D, launch_spin_density_d, spin3_);
      ddi_conv(0, spin3_, phi_per_);
      const int nb = red_blocks(N_);
      pb();
      k_dot3<R><<<nb, kRedThreads, 0, stream_>>>(phi_per_, spin3_, N_, partials_);
      done("reduce", 6.0 * (double)sizeof(R) * N_);
      finish<1>(nb, false, 31);
    }
  }

  // Energy terms and component sums from a host copy of results_[0..31].
  sbec_energy_terms energy_from(const double* res, double* comp_sums) const {
    sbec_energy_terms e{};
    const double dV = s_.dV;
    const double N = (double)N_;
    e.kinetic = 0.5 * (res[0] * dV / N);
    e.trap = res[20] * dV;
    double ez = 0.0;
    for (int c = 0; c < s_.D; ++c) {
      const double mc = (double)(s_.F - c);
      const double Ec = -zeeman_p * mc + zeeman_q * mc * mc;
      ez += Ec * res[1 + c] * dV;
    }
    e.zeeman = ez;
    if (!s_.tensor) {
      e.c0 = 0.5 * s_.c0 * res[21] * dV;
      e.c1 = 0.5 * s_.c1 * res[22] * dV;
    }
    if (s_.ddi) e.ddi = 0.5 * res[31] * dV;
    if (s_.c_lhy != 0.0) e.lhy = (2.0 / 5.0) * s_.c_lhy * res[23] * dV;
    if (s_.tensor) e.tensor = res[30] * dV;
    if (nematic()) e.tensor = 0.5 * s_.c2 * res[29] * dV;  // _nematic_energy (src/energy.jl:106-109)
    if (s_.raman) e.raman = res[24] * dV;                    // _raman_energy (src/energy.jl:123-135)
    if (comp_sums)
      for (int c = 0; c < s_.D; ++c) comp_sums[c] = res[1 + c];
    return e;
  }

  double l2_change(int a, int b) override {
    const int nb = red_blocks(nc_);
    pb();
    k_l2_change<R><<<nb, kRedThreads, 0, stream_>>>(slot(a), slot(b), nc_, partials_);
    done("reduce", 2.0 * (double)sizeof(cplx<R>) * nc_);
    finish<2>(nb, false, 0);
    fetch(2);
    return host_res_[0] / std::max(host_res_[1], 1e-300);
  }

  void max_abs(int a, int b, double* max_a, double* max_diff) override {
    const int nb = red_blocks(nc_);
    pb();
    k_max_abs<R><<<nb, kRedThreads, 0, stream_>>>(slot(a), b >= 0 ? slot(b) : nullptr, nc_, partials_);
    done("reduce", (b >= 0 ? 2.0 : 1.0) * (double)sizeof(cplx<R>) * nc_);
    finish<2>(nb, true, 0);
    fetch(2);
    *max_a = host_res_[0];
    *max_diff = host_res_[1];
  }

  double ddi_phi_max() override {
    if (!s_.ddi) return 0.0;
    const int nb = red_blocks(3 * N_);
    pb();
    k_max_abs_real<R><<<nb, kRedThreads, 0, stream_>>>(s_.padded ? phi_per_ : phi3_, 3 * N_, partials_);
    done("reduce", 3.0 * (double)sizeof(R) * N_);
    finish<1>(nb, true, 0);
    fetch(1);
    return host_res_[0];
  }

  void spin_density(double* host3N) override {
    R* out = s_.ddi ? spin3_ : alloc_tmp_real3();
    SBEC_SWITCH_D(s_.D, launch_spin_density_d, out);
    download_real3(out, host3N);
  }

  void phase_sums(int solve, double* out) override {
    const cplx<R>* src = psi_[kPsi];
    if (solve >= 0) {
      if (!bpsi_ || solve >= nsolve_) fail(SBEC_ERR_INVALID, "solve index out of range");
      src = bpsi_ + (size_t)solve * nc_;
    }
    if (!phase_pairs_) {
      // pair table of every even channel S <= 2F: rows (S/2, (S,M) index, c1, c2) and CG
      std::vector<int4> rows;
      std::vector<double> cgs;
      const int F = s_.F;
      int a = 0;
      for (int S = 0; S <= 2 * F; S += 2)
        for (int M = -S; M <= S; ++M, ++a)
          for (int m1 = -F; m1 <= F; ++m1) {
            const int m2 = M - m1;
            if (m2 < -F || m2 > F) continue;
            const double cg = clebsch_gordan(F, m1, F, m2, S, M);
            if (std::fabs(cg) < 1e-15) continue;
            rows.push_back(make_int4(S / 2, a, F - m1, F - m2));
            cgs.push_back(cg);
          }
      n_phase_pairs_ = (int)rows.size();
      phase_pairs_ = alloc<int4>(std::max<size_t>(rows.size(), 1));
      phase_cg_ = alloc<double>(std::max<size_t>(cgs.size(), 1));
      upload(phase_pairs_, rows.data(), rows.size());
      upload(phase_cg_, cgs.data(), cgs.size());
    }
    const int nb = red_blocks(N_);
    SBEC_SWITCH_D(s_.D, launch_phase_sums_d, src, nb);
    finish<kPhaseSums>(nb, false, 0);
    fetch(kPhaseSums);
    for (int k = 0; k < kPhaseSums; ++k) out[k] = host_res_[k];
  }

  void ddi_potential(bool padded, double* host3N) override {
    if (!s_.ddi) fail(SBEC_ERR_INVALID, "DDI is not enabled on this workspace");
    if (padded && !s_.padded) fail(SBEC_ERR_INVALID, "zero-padded DDI is not enabled on this workspace");
    SBEC_SWITCH_D(s_.D, launch_spin_density_d, spin3_);
    ddi_conv(padded ? 1 : 0, spin3_, phi_per_);
    download_real3(phi_per_, host3N);
  }

  double psi_resolution() const override { return sizeof(R) == 4 ? std::ldexp(1.0, -21) : 0.0; }

  // ---------------- fused paths ----------------
  bool fused_path() const override { return fused_path_supported(s_, sizeof(R) == 4); }

  void lf_open(double dtv) override {
    update_phase(dtv, false);
    ensure_row_tuned(dtv, false, false);
    RowArgs<R> a = row_args(false);
    a.p1 = pot_full(dtv / 2, false);
    a.flags = RP_POT1 | (s_.ndim > 1 ? RP_FWD_X : 0);
    launch_row(a);
  }

  void lf_steps(long long n, double dtv) override {
    update_phase(dtv, false);
    ensure_row_tuned(dtv, false, false);
    if (n <= 0) return;
    if (segment_ok()) {
      lf_segment(n, dtv);
      return;
    }
    const GraphKey key{1, n, dtv, 0.0, zeeman_p, zeeman_q, 0};
    if (graph_replay(key)) return;
    graph_begin(key);
    for (long long i = 0; i < n; ++i) {
      if (s_.ndim == 1) {
        RowArgs<R> a = row_args(false);
        a.p2 = pot_full(dtv, false);
        a.flags = RP_KIN_X | RP_POT2;
        launch_row(a);
      } else {
        last_axes_kinetic();
        RowArgs<R> a = row_args(false);
        a.p1 = pot_full(dtv, false);
        a.flags = RP_INV_X | RP_POT1 | RP_FWD_X;
        launch_row(a);
      }
    }
    graph_end(key);
  }

  // ---- persistent leapfrog segments (k_lf_segment): one cooperative launch per run of
  // merged steps, for the 2-D FP32 shapes it is compiled for.  Opt-in (SBEC_SEGMENT=1):
  // on the 256² spin-1 step it measured 17.9 µs per step against 13.7 µs for the graph
  // of row and column kernels with programmatic dependent launch, whose launch overlap
  // already hides what the segment saves, while its two grid barriers per step do not.
  bool segment_ok() const {
    if constexpr (sizeof(R) != 4) {
      return false;
    } else {
      return segment_on_ && s_.ndim == 2 && lf_segment_supported(true, s_.n[0], s_.n[1], s_.D) && !capturing();
    }
  }

  void lf_segment(long long n, double dtv) {
    if constexpr (sizeof(R) == 4) {
      if (!bar_) {
        bar_ = alloc<GridBarrier>(1);
        cuda_check(cudaMemsetAsync(bar_, 0, sizeof(GridBarrier), stream_), "memset barrier");
        cuda_check(cudaMallocHost(&bar_host_, sizeof(GridBarrier)), "cudaMallocHost");
      }
      if (segment_stall_) {
        bar_host_->count = 1u << 30;
        bar_host_->gen = 0;
        bar_host_->err = 0;
        cuda_check(cudaMemcpyAsync(bar_, bar_host_, sizeof(GridBarrier), cudaMemcpyHostToDevice, stream_),
                   "barrier");
        sync();
        segment_stall_ = false;  // one injected stall per workspace
      }
      RowArgs<R> a = row_args(false);
      a.p1 = pot_full(dtv, false);
      a.flags = RP_INV_X | RP_POT1 | RP_FWD_X;
      pb();
      lf_segment_launch(line_ctx(), twiddle(s_.n[0]), twiddle(s_.n[1]), a, s_.n[0], s_.D, n, bar_);
      done("lf_segment", (double)n * (4.0 * sizeof(cplx<R>) * nc_ + sizeof(R) * (double)N_));
      segment_used_ = true;
    }
  }

  // A grid barrier of a segment launch that ran out of time leaves an error flag in
  // device memory; read it once per run and report it (the state is then invalid).
  void check_segments() override {
    if (!segment_used_) return;
    segment_used_ = false;
    cuda_check(cudaMemcpyAsync(bar_host_, bar_, sizeof(GridBarrier), cudaMemcpyDeviceToHost, stream_), "barrier");
    sync();
    if (bar_host_->err != 0) {
      cuda_check(cudaMemsetAsync(bar_, 0, sizeof(GridBarrier), stream_), "memset barrier");
      sync();
      fail(SBEC_ERR_DEVICE, "leapfrog segment: a grid barrier wait ran out; the state is invalid");
    }
  }

  void lf_close(double dtv) override {
    update_phase(dtv, false);
    ensure_row_tuned(dtv, false, false);
    RowArgs<R> a = row_args(false);
    if (s_.ndim == 1) {
      a.p2 = pot_full(dtv / 2, false);
      a.flags = RP_KIN_X | RP_POT2;
    } else {
      last_axes_kinetic();
      a.p1 = pot_full(dtv / 2, false);
      a.flags = RP_INV_X | RP_POT1;
    }
    launch_row(a);
  }

  // split_step! x n (src/split_step.jl:10-35) as row passes; with `normalize` the
  // renormalisation of step k is applied at the start of step k+1 (and flushed at
  // the end), using the |psi|^2 sums the closing pass of step k accumulated.
  // The steps run as graph chunks of up to kGraphChunk steps (small graphs, captured once
  // and shared by blocks of any length); a chunk that follows another starts with the
  // previous step's renormalisation pending (key bit 8), and the last one is flushed
  // after the chunks, so the operator sequence is that of one uninterrupted loop.
  void fused_split_steps(long long n, double dtv, double kin_dt, bool kin_itp, bool it, bool normalize) override {
    update_phase(kin_dt, kin_itp);
    ensure_row_tuned(dtv, it, false);
    if (n <= 0) return;
    const int flags = (kin_itp ? 1 : 0) | (it ? 2 : 0) | (normalize ? 4 : 0);
    bool pending = false;
    if (s_.ndim == 1 && it && normalize && s_.n[0] >= 32 && s_.n[0] <= kItpStepsMaxLine && use_itp_steps_) {
      // one launch for all n steps (k_row_itp_steps): the 1-D solve is one row-pass block
      RowArgs<R> a = row_args(false);
      a.p1 = pot_full(dtv / 2, it);
      a.p2 = pot_full(dtv / 2, it);
      a.flags |= RP_POT1 | RP_KIN_X | RP_POT2 | RP_NORM;
      const LineCtx<R> c = line_ctx();
      const Tw<R> tw = twiddle(s_.n[0]);
      pb();
      row_itp_steps<R>(c, tw, s_.n[0], s_.D, a, n, 0, results_ + 40);
      done("row_pass", (double)n * (2.0 * (double)sizeof(cplx<R>) * nc_ + (double)sizeof(R) * N_));
      pending = true;
      n = 0;
    }
    for (long long done_steps = 0; done_steps < n;) {
      const long long m = std::min(kGraphChunk, n - done_steps);
      const GraphKey key{2, m, dtv, kin_dt, zeeman_p, zeeman_q, flags | (pending ? 8 : 0)};
      if (!graph_replay(key)) {
        graph_begin(key);
        fused_steps_body(m, dtv, it, normalize, pending);
        graph_end(key);
      }
      pending = normalize;
      done_steps += m;
    }
    if (pending) {
      pb();
      launch_pdl(k_normalize_apply<R>, dim3(grid_for(nc_)), dim3(256), 0, psi_[kPsi], (int64_t)(N_ * s_.D), 1,
                 (const double*)(results_ + 40), s_.dV);
      done("normalize", 2.0 * (double)sizeof(cplx<R>) * nc_);
    }
  }

  // n fused split steps; `pending`: the renormalisation of the step before is still to apply.
  void fused_steps_body(long long n, double dtv, bool it, bool normalize, bool pending) {
    for (long long i = 0; i < n; ++i) {
      if (s_.ndim == 1) {
        RowArgs<R> a = row_args(pending);
        a.p1 = pot_full(dtv / 2, it);
        a.p2 = pot_full(dtv / 2, it);
        a.flags |= RP_POT1 | RP_KIN_X | RP_POT2 | (normalize ? RP_NORM : 0);
        const int nb = launch_row(a);
        if (normalize) finish_row_norm(nb);
      } else {
        RowArgs<R> a = row_args(pending);
        a.p1 = pot_full(dtv / 2, it);
        a.flags |= RP_POT1 | RP_FWD_X;
        launch_row(a);
        last_axes_kinetic();
        RowArgs<R> b = row_args(false);
        b.p1 = pot_full(dtv / 2, it);
        b.flags = RP_INV_X | RP_POT1 | (normalize ? RP_NORM : 0);
        const int nb = launch_row(b);
        if (normalize) finish_row_norm(nb);
      }
      pending = normalize;
    }
  }

  // ---- the general path in graph chunks of kGraphChunk steps (the last chunk shorter);
  // the kinetic tables are made current before a replay, since a replay does not
  // rebuild them.
  static constexpr long long kGraphChunk = 16;

  template <typename Body>
  void graph_chunks(int kind, long long n, double dtv, double kin_dt, bool kin_itp, int flags, Body&& body) {
    update_phase(kin_dt, kin_itp);
    for (long long done_steps = 0; done_steps < n;) {
      const long long m = std::min(kGraphChunk, n - done_steps);
      const GraphKey key{kind, m, dtv, kin_dt, zeeman_p, zeeman_q, flags};
      if (!graph_replay(key)) {
        graph_begin(key);
        for (long long i = 0; i < m; ++i) body();
        graph_end(key);
      }
      done_steps += m;
    }
  }

  void unfused_split_steps(long long n, double dtv, double kin_dt, bool kin_itp, bool it, bool normalize) override {
    const int flags = (kin_itp ? 1 : 0) | (it ? 2 : 0) | (normalize ? 4 : 0);
    graph_chunks(5, n, dtv, kin_dt, kin_itp, flags, [&] {
      half_potential(dtv / 2, it);
      kinetic(kin_dt, kin_itp);
      half_potential(dtv / 2, it);
      if (!it) apply_loss(dtv);  // src/split_step.jl:21-23
      if (normalize) this->normalize();
    });
  }

  void unfused_lf_steps(long long n, double dtv, double kin_dt, bool kin_itp) override {
    graph_chunks(6, n, dtv, kin_dt, kin_itp, kin_itp ? 1 : 0, [&] {
      kinetic(kin_dt, kin_itp);
      half_potential(dtv, false);
      apply_loss(dtv);  // src/simulation.jl:74-76
    });
  }

  // ---- CUDA graphs of repeated step blocks.  A block runs eagerly the first
  // time a key is seen (creating lazily built tables), is captured on the
  // second and replayed from then on; profiling runs stay eager so every
  // launch keeps its own events.
  struct GraphKey {
    int kind;
    long long n;
    double dt, kin_dt, zp, zq;
    int flags;
    bool operator<(const GraphKey& o) const {
      return std::tie(kind, n, dt, kin_dt, zp, zq, flags) < std::tie(o.kind, o.n, o.dt, o.kin_dt, o.zp, o.zq, o.flags);
    }
  };
  struct GraphEntry {
    cudaGraphExec_t exec = nullptr;
    long long launches = 0;
  };

  void set_graphs(bool on) override { use_graphs_ = on; }

  bool graph_replay(const GraphKey& k) {
    if (prof.enabled() || !use_graphs_) return false;
    auto it = graphs_.find(k);
    if (it == graphs_.end() || !it->second.exec) return false;
    cuda_check(cudaGraphLaunch(it->second.exec, stream_), "cudaGraphLaunch");
    prof.add_launches(it->second.launches);
    return true;
  }

  // At most kMaxGraphs instantiated graphs and kMaxGraphKeys remembered keys per engine:
  // keys that change every call (a Zeeman field set before each step) run eagerly and stop
  // being recorded once the table is full.
  static constexpr size_t kMaxGraphs = 64;
  static constexpr size_t kMaxGraphKeys = 1024;

  void graph_begin(const GraphKey& k) {
    capturing_ = false;
    if (prof.enabled() || !use_graphs_) return;
    auto it = graphs_.find(k);
    if (it == graphs_.end()) {  // first use: eager
      if (graphs_.size() < kMaxGraphKeys) graphs_.emplace(k, GraphEntry{});
      return;
    }
    if (it->second.exec || n_graphs_ >= kMaxGraphs) return;
    cuda_check(cudaStreamBeginCapture(stream_, cudaStreamCaptureModeThreadLocal), "cudaStreamBeginCapture");
    capturing_ = true;
    cap_launch0_ = prof.total_launches();
  }

  void graph_end(const GraphKey& k) {
    if (!capturing_) return;
    capturing_ = false;
    cudaGraph_t graph = nullptr;
    cuda_check(cudaStreamEndCapture(stream_, &graph), "cudaStreamEndCapture");
    GraphEntry& g = graphs_[k];
    cuda_check(cudaGraphInstantiate(&g.exec, graph, 0), "cudaGraphInstantiate");
    cudaGraphDestroy(graph);
    ++n_graphs_;
    g.launches = prof.total_launches() - cap_launch0_;
    prof.add_launches(-g.launches);  // counted again on each replay
    cuda_check(cudaGraphLaunch(g.exec, stream_), "cudaGraphLaunch");
    prof.add_launches(g.launches);
  }

  // ---------------- batches of independent solves ----------------
  int n_solves() const override { return nsolve_; }

  void batch_init(int n, const double* c0, const double* c1, const double* psi_all) override {
    if (!fused_path()) fail(SBEC_ERR_UNSUPPORTED, "batched solves need the fused path (no DDI / tensor, D in {1,3,5})");
    if (n < 1) fail(SBEC_ERR_INVALID, "n_solves must be >= 1");
    nsolve_ = n;
    const size_t tot = (size_t)n * nc_;
    bpsi_ = alloc<cplx<R>>(tot);
    bprev_ = alloc<cplx<R>>(tot);
    c0s_ = alloc<R>(n);
    c1s_ = alloc<R>(n);
    active_ = alloc<int>(n);
    bnorm_ = alloc<double>(n);
    bres_ = alloc<double>((size_t)n * 16);
    std::vector<R> h0(n), h1(n);
    for (int i = 0; i < n; ++i) {
      h0[i] = (R)c0[i];
      h1[i] = (R)c1[i];
    }
    upload(c0s_, h0.data(), n);
    upload(c1s_, h1.data(), n);
    // predicted renormalisation of the merged FP32 ITP step: corr, pred, and a row of ones
    bcorr_ = alloc<R>(n);
    bpred_ = alloc<R>(n);
    bones_ = alloc<R>(n);
    std::vector<R> ones(n, (R)1);
    upload(bpred_, ones.data(), n);
    upload(bones_, ones.data(), n);
    // psi: host doubles -> device (converted per solve through the staging buffer)
    for (int i = 0; i < n; ++i) {
      std::memcpy(host_psi_, psi_all + (size_t)i * 2 * nc_, sizeof(double) * 2 * nc_);
      if (sizeof(R) == 8) {
        cuda_check(cudaMemcpyAsync(bpsi_ + (size_t)i * nc_, host_psi_, sizeof(double) * 2 * nc_,
                                   cudaMemcpyHostToDevice, stream_), "batch psi upload");
      } else {
        cuda_check(cudaMemcpyAsync(stage_, host_psi_, sizeof(double) * 2 * nc_, cudaMemcpyHostToDevice, stream_),
                   "batch psi upload");
        pb();
        k_from_f64<R><<<grid_for(nc_), 256, 0, stream_>>>(stage_, bpsi_ + (size_t)i * nc_, nc_);
        done("convert", (16.0 + sizeof(cplx<R>)) * nc_);
      }
      sync();
    }
    const int bps = row_blocks_per_solve();
    const size_t need = std::max((size_t)n * bps, (size_t)n * 64 * 16) + 64;
    if (need > partials_n_) {
      partials_n_ = need;
      partials_ = alloc<double>(partials_n_);
    }
    std::vector<int> all(n);
    for (int i = 0; i < n; ++i) all[i] = i;
    batch_set_active(all);
  }

  void batch_set_active(const std::vector<int>& act) override {
    n_active_ = (int)act.size();
    if (n_active_ > 0) upload(active_, act.data(), act.size());
  }

  // FP32 batched ITP, n steps with two passes per step.  The reference order per step is
  // V/2, K, V/2, renormalise (src/split_step.jl:10-35, src/ground_state.jl:130-140).  Here
  // the closing V/2 of step i, the renormalisation and the opening V/2 of step i+1 share
  // one row pass: the scale is not known inside that pass (it needs the norm of every row
  // of the solve), so the opening V/2 sees the state scaled by the previous step's scale
  // (pred) and the exact factor actual/pred is applied on the next pass's load (the
  // kinetic pass between is linear).  Only the density inside that one V/2 differs from
  // the reference, by the change of scale between consecutive steps; at convergence the
  // prediction is exact, so the ground state is the same fixed point.  The last step of
  // the block closes as in the reference and the block ends renormalised.  Opt-in
  // (SBEC_BATCH_MERGED=1): from random starts the transient differs from the reference
  // order by up to ~2e-6 in energy (FP64 emulation, 64^2 spin-1), from polar or
  // ferromagnetic starts by 1e-8 after 250 steps and 1e-12 after 1000.
  void batch_itp_merged(long long n, double dtv) {
    PotArgs<R> pot = pot_full(dtv / 2, true);
    pot.rot_a = pot.rot_b = s_.D > 1;
    cuda_check(cudaMemcpyAsync(bcorr_, bones_, sizeof(R) * nsolve_, cudaMemcpyDeviceToDevice, stream_), "corr reset");
    RowArgs<R> a = batch_row_args(false);
    a.p1 = pot;
    a.flags |= RP_POT1 | RP_FWD_X;
    launch_row(a);
    for (long long i = 0; i < n; ++i) {
      last_axes_kinetic_on(bpsi_, n_active_);
      RowArgs<R> m = batch_row_args(false);
      m.corr = bcorr_;
      m.pred = bpred_;
      m.p1 = pot;
      m.p2 = pot;
      if (i + 1 < n) {
        m.flags |= RP_CORR | RP_INV_X | RP_POT1 | RP_MID | RP_FWD_X;
        launch_row(m);
        pb();
        launch_pdl(k_seg_pred<R>, dim3((n_active_ + 127) / 128), dim3(128), 0, (const double*)partials_,
                   row_blocks_per_solve(), n_active_, (const int*)active_, s_.dV, bcorr_, bpred_);
        done("reduce_finish", 8.0 * row_blocks_per_solve() * n_active_);
      } else {
        m.flags |= RP_CORR | RP_INV_X | RP_POT1 | RP_NORM;
        launch_row(m);
        pb();
        launch_pdl(k_seg_finish_rows<R>, dim3((n_active_ + 127) / 128), dim3(128), 0, (const double*)partials_,
                   row_blocks_per_solve(), n_active_, (const int*)active_, bnorm_);
        done("reduce_finish", 8.0 * row_blocks_per_solve() * n_active_);
      }
    }
  }

  // Batched ITP in the reference order: per step one row pass (1-D) or row, column,
  // row passes, each step renormalised at the start of the next (deferred scale).
  void batch_itp_exact(long long n, double dtv) {
    bool pending = false;
    for (long long i = 0; i < n; ++i) {
      // spin mixing is decided per solve from c1[b] inside the pass
      PotArgs<R> pot = pot_full(dtv / 2, true);
      pot.rot_a = pot.rot_b = s_.D > 1;
      if (s_.ndim == 1) {
        RowArgs<R> a = batch_row_args(pending);
        a.p1 = pot;
        a.p2 = pot;
        a.flags |= RP_POT1 | RP_KIN_X | RP_POT2 | RP_NORM;
        launch_row(a);
      } else {
        RowArgs<R> a = batch_row_args(pending);
        a.p1 = pot;
        a.flags |= RP_POT1 | RP_FWD_X;
        launch_row(a);
        last_axes_kinetic_on(bpsi_, n_active_);
        RowArgs<R> b = batch_row_args(false);
        b.p1 = pot;
        b.flags |= RP_INV_X | RP_POT1 | RP_NORM;
        launch_row(b);
      }
      pb();
      launch_pdl(k_seg_finish_rows<R>, dim3((n_active_ + 127) / 128), dim3(128), 0, (const double*)partials_,
                 row_blocks_per_solve(), n_active_, (const int*)active_, bnorm_);
      done("reduce_finish", 8.0 * row_blocks_per_solve() * n_active_);
      pending = true;
    }
  }

  void batch_itp_steps(long long n, double dtv) override {
    if (n <= 0 || n_active_ == 0) return;
    update_phase(dtv, true);
    ensure_row_tuned(dtv, true, true);
    const GraphKey key{3, n, dtv, (double)n_active_, zeeman_p, zeeman_q, active_version_};
    if (graph_replay(key)) return;
    graph_begin(key);
    omap_ = active_;
    oper_ = s_.D;
    if (sizeof(R) == 4 && s_.ndim >= 2 && merged_itp_)
      batch_itp_merged(n, dtv);
    else
      batch_itp_exact(n, dtv);
    pb();
    launch_pdl(k_batch_normalize<R>, dim3(grid_for(nc_ * n_active_)), dim3(256), 0, bpsi_, (int64_t)nc_,
               (const int*)active_, n_active_, (const double*)bnorm_, s_.dV);
    done("normalize", 2.0 * sizeof(cplx<R>) * nc_ * n_active_);
    omap_ = nullptr;
    oper_ = 1;
    graph_end(key);
  }

  void batch_energies(double* E) override {
    const int na = n_active_;
    for (int i = 0; i < nsolve_; ++i) E[i] = NAN;
    if (na == 0) return;
    cplx<R>* scr = batch_scratch();
    pb();
    k_batch_gather<R><<<grid_for(nc_ * na), 256, 0, stream_>>>(bpsi_, scr, nc_, active_, na, 1);
    done("elementwise", 2.0 * sizeof(cplx<R>) * nc_ * na);
    fft_forward_batch(scr, na);
    const int bpe = (int)std::min<int64_t>(64, (N_ + kRedThreads - 1) / kRedThreads);
    PhaseTableArgs g = phase_geom(0.0, false);
    pb();
    k_batch_kinetic_sum<R><<<dim3(bpe, na), kRedThreads, 0, stream_>>>(scr, N_, s_.D, g, partials_);
    done("reduce", sizeof(cplx<R>) * (double)nc_ * na);
    pb();
    k_seg_finish<1><<<(na + 127) / 128, 128, 0, stream_>>>(partials_, bpe, na, active_, 0, bres_, 16);
    done("reduce_finish", 8.0 * bpe * na);
    SBEC_SWITCH_D(s_.D, launch_batch_energy_local_d, bpe, na);
    if (nematic()) SBEC_SWITCH_D(s_.D, launch_batch_pair_energy_d, bpe, na);
    std::vector<double> h((size_t)nsolve_ * 16);
    cuda_check(cudaMemcpyAsync(h.data(), bres_, sizeof(double) * h.size(), cudaMemcpyDeviceToHost, stream_), "fetch");
    sync();
    std::vector<int> act(na);
    cuda_check(cudaMemcpy(act.data(), active_, sizeof(int) * na, cudaMemcpyDeviceToHost), "active");
    std::vector<R> c0h(nsolve_), c1h(nsolve_);
    cuda_check(cudaMemcpy(c0h.data(), c0s_, sizeof(R) * nsolve_, cudaMemcpyDeviceToHost), "c0");
    cuda_check(cudaMemcpy(c1h.data(), c1s_, sizeof(R) * nsolve_, cudaMemcpyDeviceToHost), "c1");
    const double dV = s_.dV, N = (double)N_;
    for (int b : act) {
      const double* r = &h[(size_t)b * 16];
      double ez = 0.0;
      for (int c = 0; c < s_.D; ++c) {
        const double m = (double)(s_.F - c);
        ez += (-zeeman_p * m + zeeman_q * m * m) * r[1 + c] * dV;
      }
      const int o = 1 + s_.D;
      double e = 0.5 * (r[0] * dV / N) + r[o] * dV + ez + 0.5 * (double)c0h[b] * r[o + 1] * dV +
                 0.5 * (double)c1h[b] * r[o + 2] * dV;
      if (s_.c_lhy != 0.0) e += (2.0 / 5.0) * s_.c_lhy * r[o + 3] * dV;
      if (nematic()) e += 0.5 * s_.c2 * r[o + 4] * dV;  // _nematic_energy (src/energy.jl:106-109)
      E[b] = e;
    }
  }

  void batch_max_abs(double* pmax, double* dmax) override {
    const int na = n_active_;
    if (na == 0) return;
    const int bpe = (int)std::min<int64_t>(64, (nc_ + kRedThreads - 1) / kRedThreads);
    pb();
    k_batch_max_abs<R><<<dim3(bpe, na), kRedThreads, 0, stream_>>>(bpsi_, bprev_, nc_, nc_, active_, partials_);
    done("reduce", 2.0 * sizeof(cplx<R>) * (double)nc_ * na);
    pb();
    k_seg_finish<2><<<(na + 127) / 128, 128, 0, stream_>>>(partials_, bpe, na, active_, 1, bres_, 16);
    done("reduce_finish", 16.0 * bpe * na);
    std::vector<double> h((size_t)nsolve_ * 16);
    cuda_check(cudaMemcpyAsync(h.data(), bres_, sizeof(double) * h.size(), cudaMemcpyDeviceToHost, stream_), "fetch");
    sync();
    for (int b = 0; b < nsolve_; ++b) {
      pmax[b] = h[(size_t)b * 16];
      dmax[b] = h[(size_t)b * 16 + 1];
    }
  }

  void batch_save_prev() override {
    cuda_check(cudaMemcpyAsync(bprev_, bpsi_, sizeof(cplx<R>) * nc_ * nsolve_, cudaMemcpyDeviceToDevice, stream_),
               "prev copy");
  }

  void batch_save_prev_solve(int solve) override {
    const size_t off = (size_t)solve * nc_;
    cuda_check(cudaMemcpyAsync(bprev_ + off, bpsi_ + off, sizeof(cplx<R>) * nc_, cudaMemcpyDeviceToDevice, stream_),
               "prev copy");
  }

  bool batch_has_nan() override {
    const int nb = red_blocks(nc_ * nsolve_);
    pb();
    k_comp_norms<R, 1><<<nb, kRedThreads, 0, stream_>>>(bpsi_, nc_ * nsolve_, partials_);
    done("reduce", sizeof(cplx<R>) * (double)nc_ * nsolve_);
    finish<2>(nb, false, 1);
    fetch(3);
    return host_res_[2] > 0;
  }

  void batch_get_psi(int solve, double* host) override {
    if (solve < 0 || solve >= nsolve_) fail(SBEC_ERR_INVALID, "solve index out of range");
    const cplx<R>* src = bpsi_ + (size_t)solve * nc_;
    if (sizeof(R) == 8) {
      cuda_check(cudaMemcpyAsync(host_psi_, src, sizeof(double) * 2 * nc_, cudaMemcpyDeviceToHost, stream_), "get");
    } else {
      pb();
      k_to_f64<R><<<grid_for(nc_), 256, 0, stream_>>>(src, stage_, nc_);
      done("convert", (16.0 + sizeof(cplx<R>)) * nc_);
      cuda_check(cudaMemcpyAsync(host_psi_, stage_, sizeof(double) * 2 * nc_, cudaMemcpyDeviceToHost, stream_), "get");
    }
    sync();
    std::memcpy(host, host_psi_, sizeof(double) * 2 * nc_);
  }

  void sync() override { cuda_check(cudaStreamSynchronize(stream_), "stream sync"); }

 private:
  static constexpr int kMaxBlocks = 2048;

  template <typename T>
  T* alloc(size_t n) {
    void* p = nullptr;
    const cudaError_t e = cudaMalloc(&p, sizeof(T) * std::max<size_t>(n, 1));
    if (e != cudaSuccess) {
      cudaGetLastError();
      fail(SBEC_ERR_OOM, std::string("device allocation failed: ") + cudaGetErrorString(e));
    }
    allocs_.push_back(p);
    return static_cast<T*>(p);
  }

  template <typename T>
  void upload(T* dst, const T* src, size_t n) {
    if (n == 0) return;
    cuda_check(cudaMemcpy(dst, src, sizeof(T) * n, cudaMemcpyHostToDevice), "upload");
  }

  void launch_check(const char* what) { cuda_check(cudaGetLastError(), what); }

  // Launch with programmatic stream serialisation (the kernel waits in pdl_wait()).
  template <typename... KArgs, typename... Args>
  void launch_pdl(void (*kern)(KArgs...), dim3 grid, dim3 block, size_t smem, Args... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = stream_;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = use_pdl_ ? 1 : 0;
    cuda_check(cudaLaunchKernelEx(&cfg, kern, args...), "cudaLaunchKernelEx");
  }
  void pb() { prof.begin(stream_); }
  void done(const char* name, double bytes) {
    cuda_check(cudaGetLastError(), name);
    prof.end(stream_, name, bytes);
  }

  int grid_for(int64_t n) const {
    const int64_t b = (n + 255) / 256;
    return (int)std::min<int64_t>(std::max<int64_t>(b, 1), 152 * 16);
  }
  int red_blocks(int64_t n) const {
    const int64_t b = (n + kRedThreads - 1) / kRedThreads;
    return (int)std::min<int64_t>(std::max<int64_t>(b, 1), kMaxBlocks);
  }

  template <int K>
  void finish(int nb, bool is_max, int out_off) {
    pb();
    launch_pdl(k_reduce_finish<K>, dim3(1), dim3(32), 0, (const double*)partials_, nb, is_max ? 1 : 0,
               results_ + out_off);
    done("reduce_finish", 8.0 * K * nb);
  }

  void fetch(int n) {
    cuda_check(cudaMemcpyAsync(host_res_, results_, sizeof(double) * n, cudaMemcpyDeviceToHost, stream_), "fetch");
    sync();
  }

  cplx<R>* slot(int i) {
    if (i < 0 || i >= kNumSlots) fail(SBEC_ERR_INVALID, "bad slot");
    if (!psi_[i]) psi_[i] = alloc<cplx<R>>(nc_);
    return psi_[i];
  }
  cplx<R>* slot_scratch() {
    if (!scratch_) scratch_ = alloc<cplx<R>>(nc_);
    return scratch_;
  }
  R* alloc_tmp_real3() {
    if (!tmp3_) tmp3_ = alloc<R>(3 * N_);
    return tmp3_;
  }

  void upload_psi_from_pinned() {
    if (sizeof(R) == 8) {
      cuda_check(cudaMemcpyAsync(psi_[kPsi], host_psi_, sizeof(double) * 2 * nc_, cudaMemcpyHostToDevice, stream_),
                 "psi upload");
    } else {
      cuda_check(cudaMemcpyAsync(stage_, host_psi_, sizeof(double) * 2 * nc_, cudaMemcpyHostToDevice, stream_),
                 "psi upload");
      pb();
      k_from_f64<R><<<grid_for(nc_), 256, 0, stream_>>>(stage_, psi_[kPsi], nc_);
      done("convert", (16.0 + (double)sizeof(cplx<R>)) * nc_);
    }
  }

  void download_psi_to_pinned() {
    if (sizeof(R) == 8) {
      cuda_check(cudaMemcpyAsync(host_psi_, psi_[kPsi], sizeof(double) * 2 * nc_, cudaMemcpyDeviceToHost, stream_),
                 "psi download");
    } else {
      pb();
      k_to_f64<R><<<grid_for(nc_), 256, 0, stream_>>>(psi_[kPsi], stage_, nc_);
      done("convert", (16.0 + (double)sizeof(cplx<R>)) * nc_);
      cuda_check(cudaMemcpyAsync(host_psi_, stage_, sizeof(double) * 2 * nc_, cudaMemcpyDeviceToHost, stream_),
                 "psi download");
    }
  }

  void download_real3(const R* src, double* host) {
    double* tmp = alloc_host_tmp(3 * N_);
    if (sizeof(R) == 8) {
      cuda_check(cudaMemcpyAsync(tmp, src, sizeof(double) * 3 * N_, cudaMemcpyDeviceToHost, stream_), "download");
    } else {
      double* dtmp = reinterpret_cast<double*>(stage_);
      if (3 * N_ > 2 * nc_) fail(SBEC_ERR_INVALID, "staging buffer too small");
      pb();
      k_real_to_f64<R><<<grid_for(3 * N_), 256, 0, stream_>>>(src, dtmp, 3 * N_);
      done("convert", (8.0 + (double)sizeof(R)) * 3 * N_);
      cuda_check(cudaMemcpyAsync(tmp, dtmp, sizeof(double) * 3 * N_, cudaMemcpyDeviceToHost, stream_), "download");
    }
    sync();
    std::memcpy(host, tmp, sizeof(double) * 3 * N_);
  }

  double* alloc_host_tmp(int64_t n) {
    if (host_tmp_n_ < n) {
      if (host_tmp_) cudaFreeHost(host_tmp_);
      cuda_check(cudaMallocHost(&host_tmp_, sizeof(double) * n), "cudaMallocHost");
      host_tmp_n_ = n;
    }
    return host_tmp_;
  }

  // twiddle table W_n^e = exp(-2 pi i e/n), e = 0..n-1 (computed in long double);
  // FP32 tables carry the tail (value - rounded head) for compensated products.
  Tw<R> twiddle(int n) {
    auto it = tw_.find(n);
    if (it != tw_.end()) return it->second;
    std::vector<cplx<R>> h(n), l(n);
    const int per = sizeof(R) == 4 ? 2 : 1;  // FP32: (head, tail) interleaved
    std::vector<cplx<R>> tab((size_t)n * per);
    for (int e = 0; e < n; ++e) {
      const long double ang = -2.0L * 3.141592653589793238462643383279502884L * (long double)e / (long double)n;
      const long double c = std::cos(ang), sn = std::sin(ang);
      h[e] = mk<R>((R)c, (R)sn);
      tab[(size_t)e * per] = h[e];
      if (per == 2) tab[(size_t)e * 2 + 1] = mk<R>((R)(c - (long double)h[e].x), (R)(sn - (long double)h[e].y));
    }
    (void)l;
    Tw<R> t{};
    cplx<R>* dh = alloc<cplx<R>>(tab.size());
    upload(dh, tab.data(), tab.size());
    t.hi = dh;
    t.lo = nullptr;
    tw_[n] = t;
    return t;
  }

  PhaseTableArgs phase_geom(double dtv, bool it) const {
    PhaseTableArgs g{};
    g.ndim = s_.ndim;
    for (int a = 0; a < 3; ++a) {
      g.n[a] = s_.n[a];
      g.kmult[a] = s_.kmult[a];
    }
    g.dt = dtv;
    g.itp = it ? 1 : 0;
    g.scale = 1.0 / (double)N_;
    return g;
  }

  void update_phase(double dtv, bool it) {
    if (dtv == phase_dt_ && (it ? 1 : 0) == phase_itp_) return;
    PhaseTableArgs g = phase_geom(dtv, it);
    dim3 grid(8, s_.ndim);
    PhaseOut<R> po{};
    for (int a = 0; a < 3; ++a) {
      po.hi[a] = ptab_[a];
      po.lo[a] = ptab_lo_[a];
    }
    pb();
    k_phase_tables<R><<<grid, 256, 0, stream_>>>(po, g);
    done("phase_tables", 0.0);
    phase_dt_ = dtv;
    phase_itp_ = it ? 1 : 0;
  }

  PhaseRef<R> phase_ref() const {
    PhaseRef<R> p{};
    p.ndim = s_.ndim;
    for (int a = 0; a < 3; ++a) {
      p.tab[a].hi = ptab_[a];
      p.tab[a].lo = ptab_lo_[a];
      p.n[a] = s_.n[a];
    }
    p.scale0 = (R)(1.0 / (double)N_);  // exact when N_ is a power of two
    // FP32 real time: the unbiased rotation (the line kernels of power-of-two grids, where
    // scale0 is exact; k_kinetic_apply of other grids, which carries the rounding of x scale0)
    p.unbiased = (sizeof(R) == 4 && phase_itp_ == 0) ? 1 : 0;
    return p;
  }

  // ---- FFT launchers
  LineCtx<R> line_ctx() const { return LineCtx<R>{stream_, use_pdl_, phase_ref(), st_}; }

  // Calls f(std::integral_constant<int, V>) for the compiled variant V of a line kind.
  template <typename F>
  void with_variant(int n, int v, F&& f) {
    if constexpr (sizeof(R) == 8) {
      (void)n;
      (void)v;
      f(std::integral_constant<int, 0>{});
    } else {
      switch (line_variant(true, n, v)) {
        case 1: f(std::integral_constant<int, 1>{}); break;
        case 2: f(std::integral_constant<int, 2>{}); break;
        case 3: f(std::integral_constant<int, 3>{}); break;
        case 4: f(std::integral_constant<int, 4>{}); break;
        case 5: f(std::integral_constant<int, 5>{}); break;
        case 6: f(std::integral_constant<int, 6>{}); break;
        case 7: f(std::integral_constant<int, 7>{}); break;
        default: f(std::integral_constant<int, 0>{}); break;
      }
    }
  }

  // ---- autotuner.  The first time a line-kernel call shape is met (outside a graph
  // capture) every compiled variant is timed on a copy of the data it would touch:
  // one warm-up launch, then the median of three CUDA-event timings, each on a
  // fresh copy (of 8 back-to-back launches for data up to 32 MB).  The fastest is kept in a table shared by all workspaces of the
  // process, so every solve of one shape runs the same kernels (the variants agree
  // to FP32 rounding, not bit for bit).
  static std::mutex& tune_mutex() { return tune_table_mutex(); }
  static std::map<std::string, int>& tune_table() { return tune_table_map(); }

  bool capturing() const {
    cudaStreamCaptureStatus st = cudaStreamCaptureStatusNone;
    cuda_check(cudaStreamIsCapturing(stream_, &st), "cudaStreamIsCapturing");
    return st != cudaStreamCaptureStatusNone;
  }

  // Candidates of a call shape: row passes (row), strided lines (reg, not row: tile and
  // register forms) or x lines (tile forms).
  std::vector<int> line_candidates(int n, bool row, bool reg) const {
    std::vector<int> c;
    for (int v = 0; v < (reg ? kRowVariants : kLineVariants); ++v) {
      if (line_variant(sizeof(R) == 4, n, v) != v || !row_variant_compiled(v)) continue;
      if (row && !row_variant_ok(sizeof(R) == 4, n, s_.D, v)) continue;
      if (!row && v >= kLineVariants && n > 1024) continue;  // register strided lines up to 1024 points
      c.push_back(v);
    }
    return c;
  }

  // Runs strided-line variant v (tile forms 0-7, register forms 12-15).
  void strided_variant_launch(int v, const LineCtx<R>& c, const Tw<R>& tw, int n, cplx<R>* data, int64_t S,
                              int64_t inner, int64_t outer, int64_t outer_stride, int n_in, int n_out, int mode,
                              const int* om, int op) {
    if constexpr (sizeof(R) == 4) {
      switch (line_variant(true, n, v)) {
        case 12: RegKernels<R, 12>::fft_strided(c, tw, n, data, S, inner, outer, outer_stride, n_in, n_out, mode, om, op); return;
        case 13: RegKernels<R, 13>::fft_strided(c, tw, n, data, S, inner, outer, outer_stride, n_in, n_out, mode, om, op); return;
        case 14: RegKernels<R, 14>::fft_strided(c, tw, n, data, S, inner, outer, outer_stride, n_in, n_out, mode, om, op); return;
        case 15: RegKernels<R, 15>::fft_strided(c, tw, n, data, S, inner, outer, outer_stride, n_in, n_out, mode, om, op); return;
        default: break;
      }
    }
    with_variant(n, v, [&](auto vv) {
      LineKernels<R, decltype(vv)::value>::fft_strided(c, tw, n, data, S, inner, outer, outer_stride, n_in, n_out,
                                                       mode, om, op);
    });
  }

  // Runs row-pass variant v (tile forms 0-7 through LineKernels, register forms 12-15).
  void row_variant_launch(int v, const LineCtx<R>& c, const Tw<R>& tw, int nx, int D, const RowArgs<R>& a, int nb) {
    if constexpr (sizeof(R) == 4) {
      switch (line_variant(true, nx, v)) {
        case 12: RegKernels<R, 12>::row(c, tw, nx, D, a, nb); return;
        case 13: RegKernels<R, 13>::row(c, tw, nx, D, a, nb); return;
        case 14: RegKernels<R, 14>::row(c, tw, nx, D, a, nb); return;
        case 15: RegKernels<R, 15>::row(c, tw, nx, D, a, nb); return;
        default: break;
      }
    }
    with_variant(nx, v, [&](auto vv) { LineKernels<R, decltype(vv)::value>::row(c, tw, nx, D, a, nb); });
  }

  // Variant for a call shape: forced, cached, or measured now.  launch(v, buf)
  // runs variant v on buf, a copy of the `extent` elements at src.
  template <typename Launch>
  int line_tune(const std::string& shape, int n, bool row, const cplx<R>* src, size_t extent, Launch&& launch,
                bool reg = false) {
    reg = reg || row;
    const std::vector<int> cands = line_candidates(n, row, reg);
    if (cands.empty()) return 0;
    if (tune_force_ >= 0) {
      // a forced register form (12-15) runs the x-line kernels of its plan and tile scale
      const int f = reg ? tune_force_ : (tune_force_ & (kLineVariants - 1));
      for (int v : cands)
        if (v == f) return v;
      return 0;
    }
    if (!tune_on_ || cands.size() == 1) return cands[0];
    const std::string key = std::string(sizeof(R) == 4 ? "fp32 " : "fp64 ") + shape + " D=" + std::to_string(s_.D) +
                            " grid=" + std::to_string(s_.n[0]) + "x" + std::to_string(s_.n[1]) + "x" +
                            std::to_string(s_.n[2]) + " solves=" + std::to_string(std::max(nsolve_, 1));
    auto mine = tuned_.find(key);
    if (mine != tuned_.end()) return mine->second;
    std::lock_guard<std::mutex> lock(tune_mutex());
    auto it = tune_table().find(key);
    if (it != tune_table().end() && std::find(cands.begin(), cands.end(), it->second) != cands.end()) {
      tune_log_.push_back(key + " -> v" + std::to_string(it->second) + " (from the process table)");
      return tuned_[key] = it->second;
    }
    if (tune_frozen().load()) {
      tune_log_.push_back(key + " -> v" + std::to_string(cands[0]) + " (frozen table: default)");
      tune_table()[key] = cands[0];
      return tuned_[key] = cands[0];
    }
    if (capturing()) return 0;  // never reached: shapes are first met in an eager run
    if (extent > tune_buf_n_) {
      tune_buf_ = alloc<cplx<R>>(extent);
      tune_buf_n_ = extent;
    }
    cudaEvent_t e0, e1;
    cuda_check(cudaEventCreate(&e0), "cudaEventCreate");
    cuda_check(cudaEventCreate(&e1), "cudaEventCreate");
    const size_t bytes = sizeof(cplx<R>) * extent;
    // Small (latency-bound) shapes are timed as a burst of back-to-back launches, the way
    // they run inside a step graph; one launch there is mostly launch latency, which is
    // the same for every variant.
    const int reps = bytes <= ((size_t)32 << 20) ? 8 : 1;
    std::string line = key + " ->";
    float best = 0.0f;
    int bv = cands[0];
    for (int v : cands) {
      cuda_check(cudaMemcpyAsync(tune_buf_, src, bytes, cudaMemcpyDeviceToDevice, stream_), "cudaMemcpyAsync");
      launch(v, tune_buf_);
      float t[3];
      for (float& ti : t) {
        cuda_check(cudaMemcpyAsync(tune_buf_, src, bytes, cudaMemcpyDeviceToDevice, stream_), "cudaMemcpyAsync");
        cuda_check(cudaEventRecord(e0, stream_), "cudaEventRecord");
        for (int r = 0; r < reps; ++r) launch(v, tune_buf_);
        cuda_check(cudaEventRecord(e1, stream_), "cudaEventRecord");
        cuda_check(cudaEventSynchronize(e1), "cudaEventSynchronize");
        cuda_check(cudaEventElapsedTime(&ti, e0, e1), "cudaEventElapsedTime");
        ti /= (float)reps;
      }
      std::sort(t, t + 3);
      line += " v" + std::to_string(v) + "=" + std::to_string(t[1] * 1000.0f).substr(0, 7) + "us";
      if (v == cands[0] || t[1] < best) {
        best = t[1];
        bv = v;
      }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cuda_check(cudaGetLastError(), "autotune");
    tune_log_.push_back(line + " chosen v" + std::to_string(bv));
    tune_table()[key] = bv;
    return tuned_[key] = bv;
  }

  // Row-pass variant, fixed once per engine before any row arguments are built
  // (the tile height sets how many norm partials a pass writes).
  void ensure_row_tuned(double dtv, bool itp, bool batch) {
    if (row_tuned_ || !fused_path()) return;
    row_tuned_ = true;
    const int nx = s_.n[0];
    RowArgs<R> a = batch ? batch_row_args(false) : row_args(false);
    PotArgs<R> pot = pot_full(dtv / 2, itp);
    if (batch) pot.rot_a = pot.rot_b = s_.D > 1;
    a.p1 = pot;
    a.p2 = pot;
    a.flags = s_.ndim > 1 ? (RP_INV_X | RP_POT1 | RP_FWD_X) : (RP_POT1 | RP_KIN_X);
    const LineCtx<R> c = line_ctx();
    const Tw<R> tw = twiddle(nx);
    const int D = s_.D;
    const size_t extent = batch ? (size_t)nc_ * nsolve_ : (size_t)nc_;
    const cplx<R>* src = batch ? bpsi_ : psi_[kPsi];
    v_row_ = line_tune("row flags=" + std::to_string(a.flags) + (batch ? " batched" : ""), nx, true, src, extent,
                       [&](int v, cplx<R>* buf) {
                         RowArgs<R> b = a;
                         b.psi = buf;
                         const int rpb = row_rpb_host(sizeof(R) == 4, nx, D, v);
                         const int bps = (int)((a.n_rows + rpb - 1) / rpb);
                         b.blocks_per_solve = bps;
                         const int nb = b.active ? bps * b.n_slots : bps;
                         row_variant_launch(v, c, tw, nx, D, b, nb);
                       });
  }

  std::string tuning_report() const override {
    std::string r;
    for (const auto& l : tune_log_) r += l + "\n";
    r += "row variant " + std::to_string(v_row_) + (tune_force_ >= 0 ? " (forced)" : (tune_on_ ? "" : " (tuning off)"));
    return r;
  }

  void fft_x_n(int n, cplx<R>* data, int64_t n_lines, int mode) {
    const LineCtx<R> c = line_ctx();
    const Tw<R> tw = twiddle(n);
    const int vx = line_tune(
        "x n=" + std::to_string(n) + " lines=" + std::to_string(n_lines) + " mode=" + std::to_string(mode), n,
        false, data, (size_t)n_lines * n, [&](int v, cplx<R>* buf) {
          with_variant(n, v, [&](auto vv) { LineKernels<R, decltype(vv)::value>::fft_x(c, tw, n, buf, n_lines, mode); });
        });
    pb();
    with_variant(n, vx, [&](auto v) { LineKernels<R, decltype(v)::value>::fft_x(c, tw, n, data, n_lines, mode); });
    done(mode == 2 ? "fft_x_kinetic" : "fft_x", 2.0 * (double)sizeof(cplx<R>) * (double)n_lines * n);
  }

  void fft_strided_n(int n, cplx<R>* data, int64_t S, int64_t inner, int64_t outer, int64_t outer_stride, int n_in,
                     int n_out, int mode) {
    const LineCtx<R> c = line_ctx();
    const Tw<R> tw = twiddle(n);
    const int* om = omap_;
    const int op = oper_;
    // elements the launch touches from `data`: all outer lines, or every solve slot through omap
    const size_t extent = (size_t)(om ? (int64_t)std::max(nsolve_, 1) * op : outer) * (size_t)outer_stride;
    const int vs = line_tune("strided n=" + std::to_string(n) + " S=" + std::to_string(S) + " inner=" +
                                 std::to_string(inner) + " outer=" + std::to_string(outer) + " in/out=" +
                                 std::to_string(n_in) + "/" + std::to_string(n_out) + " mode=" + std::to_string(mode) +
                                 (om ? " batched" : ""),
                             n, false, data, extent, [&](int v, cplx<R>* buf) {
                               strided_variant_launch(v, c, tw, n, buf, S, inner, outer, outer_stride, n_in, n_out,
                                                      mode, om, op);
                             }, true);
    pb();
    strided_variant_launch(vs, c, tw, n, data, S, inner, outer, outer_stride, n_in, n_out, mode, om, op);
    done(mode == 2 ? "fft_last_kinetic" : "fft_strided",
         (double)sizeof(cplx<R>) * (double)(n_in + n_out) * (double)inner * (double)outer);
  }

  // ---- axes of non-power-of-two length (Bluestein, k_blue_*): per (n, direction) the chirp
  // w_j = exp(sign i pi (j^2 mod 2n) / n) and the M-point FFT of conj(w) placed at m and M - m.
  struct BlueTab {
    int M = 0;
    cplx<R>* chirp = nullptr;  // head values
    cplx<R>* chirp_lo = nullptr;  // tails (FP32; zero in FP64)
    cplx<R>* bhat = nullptr;
    cplx<R>* bhat_lo = nullptr;
  };

  const BlueTab& blue_tab(int n, int sign) {
    const int key = sign > 0 ? n : -n;
    auto it = blue_.find(key);
    if (it != blue_.end()) return it->second;
    int M = 1;
    while (M < 2 * n - 1) M *= 2;
    const long double pi = 3.141592653589793238462643383279502884L;
    using cld = std::complex<long double>;
    std::vector<cplx<R>> w(n), wl(n), bh((size_t)M), bl((size_t)M);
    std::vector<cld> b((size_t)M, cld(0, 0));
    // head (rounded to R) and tail (the remainder, rounded to R; zero in FP64)
    auto split = [](cld v, cplx<R>& hi, cplx<R>& lo) {
      hi = mk<R>((R)v.real(), (R)v.imag());
      lo = sizeof(R) == 4 ? mk<R>((R)(v.real() - (long double)hi.x), (R)(v.imag() - (long double)hi.y)) : mk<R>(0, 0);
    };
    for (int j = 0; j < n; ++j) {
      const long long jj = ((long long)j * j) % (2LL * n);
      const long double ang = (long double)sign * pi * (long double)jj / (long double)n;
      split(cld(std::cos(ang), std::sin(ang)), w[j], wl[j]);
      const cld cw(std::cos(ang), -std::sin(ang));
      b[j] = cw;
      if (j > 0) b[(size_t)M - j] = cw;
    }
    // The M-point forward transform of the chirp on the host in long double (radix 2, in
    // place), rounded once to R: the table enters every transform of the axis, so its error
    // must not be that of an R-precision FFT.
    for (int i = 1, j = 0; i < M; ++i) {
      int bit = M >> 1;
      for (; j & bit; bit >>= 1) j ^= bit;
      j ^= bit;
      if (i < j) std::swap(b[(size_t)i], b[(size_t)j]);
    }
    for (int len = 2; len <= M; len <<= 1) {
      const int h = len / 2;
      for (int k = 0; k < h; ++k) {
        const long double a = -2.0L * pi * (long double)k / (long double)len;
        const cld tw(std::cos(a), std::sin(a));
        for (int s0 = 0; s0 < M; s0 += len) {
          const cld u = b[(size_t)(s0 + k)], v = b[(size_t)(s0 + k + h)] * tw;
          b[(size_t)(s0 + k)] = u + v;
          b[(size_t)(s0 + k + h)] = u - v;
        }
      }
    }
    for (int k = 0; k < M; ++k) split(b[(size_t)k], bh[(size_t)k], bl[(size_t)k]);
    BlueTab t;
    t.M = M;
    t.chirp = alloc<cplx<R>>(n);
    t.chirp_lo = alloc<cplx<R>>(n);
    t.bhat = alloc<cplx<R>>(M);
    t.bhat_lo = alloc<cplx<R>>(M);
    upload(t.chirp, w.data(), w.size());
    upload(t.chirp_lo, wl.data(), wl.size());
    upload(t.bhat, bh.data(), bh.size());
    upload(t.bhat_lo, bl.data(), bl.size());
    return blue_[key] = t;
  }

  // Unnormalised transform of every line of axis `axis` (sign -1 forward, +1 inverse) for an
  // axis whose length is not a power of two.
  void blue_axis(cplx<R>* buf, int axis, int sign) {
    const int n = s_.n[axis];
    int64_t inner = 1;
    for (int a = 0; a < axis; ++a) inner *= s_.n[a];
    const int64_t outer = nc_ / (inner * n);
    const BlueTab& t = blue_tab(n, sign);
    const int M = t.M;
    const size_t need = (size_t)outer * M * inner;
    if (need > blue_scr_n_) {
      blue_scr_ = alloc<cplx<R>>(need);
      blue_scr_n_ = need;
    }
    pb();
    k_blue_pre<R><<<grid_for((int64_t)need), 256, 0, stream_>>>(buf, blue_scr_, n, M, inner, (int64_t)need, t.chirp,
                                                                  t.chirp_lo);
    done("blue", (double)sizeof(cplx<R>) * ((double)nc_ + (double)need));
    auto line_fft = [&](int mode) {
      if (inner == 1)
        fft_x_n(M, blue_scr_, outer, mode);
      else
        fft_strided_n(M, blue_scr_, inner, inner, outer, (int64_t)M * inner, M, M, mode);
    };
    line_fft(0);
    pb();
    k_blue_mid<R><<<grid_for((int64_t)need), 256, 0, stream_>>>(blue_scr_, M, inner, (int64_t)need, t.bhat,
                                                                  t.bhat_lo);
    done("blue", 2.0 * (double)sizeof(cplx<R>) * (double)need);
    line_fft(1);
    pb();
    k_blue_post<R><<<grid_for(nc_), 256, 0, stream_>>>(blue_scr_, buf, n, M, inner, nc_, t.chirp, t.chirp_lo,
                                                         (R)(1.0 / M));
    done("blue", (double)sizeof(cplx<R>) * 2.0 * (double)nc_);
  }

  // One axis of the unnormalised transform: the line kernels for a power-of-two length,
  // Bluestein otherwise.
  void fft_axis(cplx<R>* buf, int axis, int sign) {
    const int n = s_.n[axis];
    if (n & (n - 1)) {
      blue_axis(buf, axis, sign);
      return;
    }
    const int mode = sign < 0 ? 0 : 1;
    if (axis == 0) {
      fft_x_n(n, buf, nc_ / n, mode);
      return;
    }
    int64_t inner = 1;
    for (int a = 0; a < axis; ++a) inner *= s_.n[a];
    fft_strided_n(n, buf, inner, inner, nc_ / (inner * n), inner * n, n, n, mode);
  }

  // Full spatial FFT of a D-component buffer: forward only (kinetic=false), or the
  // kinetic step fwd -> phase -> inv (kinetic=true).
  void fft_full(cplx<R>* buf, bool kinetic) {
    if (!s_.pow2) {
      // a non-power-of-two axis: forward on every axis, the kinetic phase, inverse on every axis
      for (int a = 0; a < s_.ndim; ++a) fft_axis(buf, a, -1);
      if (!kinetic) return;
      pb();
      k_kinetic_apply<R><<<grid_for(nc_), 256, 0, stream_>>>(buf, N_, nc_, phase_ref());
      done("kinetic_phase", 2.0 * (double)sizeof(cplx<R>) * (double)nc_);
      for (int a = s_.ndim - 1; a >= 0; --a) fft_axis(buf, a, +1);
      return;
    }
    const int nd = s_.ndim;
    const int nx = s_.n[0], ny = s_.n[1], nz = s_.n[2];
    const int64_t D = s_.D;
    if (nd == 1) {
      fft_x_n(nx, buf, D, kinetic ? 2 : 0);
      return;
    }
    fft_x_n(nx, buf, (int64_t)ny * nz * D, 0);
    if (nd == 2) {
      fft_strided_n(ny, buf, (int64_t)nx, (int64_t)nx, D, N_, ny, ny, kinetic ? 2 : 0);
    } else {
      fft_strided_n(ny, buf, (int64_t)nx, (int64_t)nx, (int64_t)nz * D,
                               (int64_t)nx * ny, ny, ny, 0);
      fft_strided_n(nz, buf, (int64_t)nx * ny, (int64_t)nx * ny, D, N_, nz, nz,
                               kinetic ? 2 : 0);
      if (kinetic)
        fft_strided_n(ny, buf, (int64_t)nx, (int64_t)nx, (int64_t)nz * D,
                                 (int64_t)nx * ny, ny, ny, 1);
    }
    if (kinetic) fft_x_n(nx, buf, (int64_t)ny * nz * D, 1);
  }

  // ---- batch helpers
  int row_blocks_per_solve() const {
    const int nx = s_.n[0];
    const int rpb = row_rpb_host(sizeof(R) == 4, nx, s_.D, v_row_);
    const int64_t rows = N_ / nx;
    return (int)((rows + rpb - 1) / rpb);
  }

  RowArgs<R> batch_row_args(bool scale) {
    RowArgs<R> a = row_args(scale);
    a.psi = bpsi_;
    a.active = active_;
    a.blocks_per_solve = row_blocks_per_solve();
    a.solve_stride = nc_;
    a.c0s = c0s_;
    a.c1s = c1s_;
    a.n_slots = n_active_;
    a.norm_total = bnorm_;
    return a;
  }

  cplx<R>* batch_scratch() {
    if (!bscratch_) bscratch_ = alloc<cplx<R>>((size_t)nc_ * nsolve_);
    return bscratch_;
  }

  // kinetic passes above x for n_slots solves addressed through omap_
  void last_axes_kinetic_on(cplx<R>* buf, int n_slots) {
    const int nx = s_.n[0], ny = s_.n[1], nz = s_.n[2];
    const int64_t D = s_.D;
    if (s_.ndim == 2) {
      oper_ = (int)D;
      fft_strided_n(ny, buf, (int64_t)nx, (int64_t)nx, D * n_slots, N_, ny, ny, 2);
    } else {
      oper_ = (int)(nz * D);
      fft_strided_n(ny, buf, (int64_t)nx, (int64_t)nx, (int64_t)nz * D * n_slots,
                               (int64_t)nx * ny, ny, ny, 0);
      oper_ = (int)D;
      fft_strided_n(nz, buf, (int64_t)nx * ny, (int64_t)nx * ny, D * n_slots, N_, nz,
                               nz, 2);
      oper_ = (int)(nz * D);
      fft_strided_n(ny, buf, (int64_t)nx, (int64_t)nx, (int64_t)nz * D * n_slots,
                               (int64_t)nx * ny, ny, ny, 1);
      oper_ = (int)D;
    }
  }

  // forward FFT of n_slots compact solves (energy)
  void fft_forward_batch(cplx<R>* buf, int n_slots) {
    const int nx = s_.n[0], ny = s_.n[1], nz = s_.n[2];
    const int64_t D = s_.D;
    fft_x_n(nx, buf, (int64_t)ny * nz * D * n_slots, 0);
    if (s_.ndim >= 2)
      fft_strided_n(ny, buf, (int64_t)nx, (int64_t)nx, (int64_t)nz * D * n_slots,
                               (int64_t)nx * ny, ny, ny, 0);
    if (s_.ndim >= 3)
      fft_strided_n(nz, buf, (int64_t)nx * ny, (int64_t)nx * ny, D * n_slots, N_, nz,
                               nz, 0);
  }

  // per-solve sum |A00|^2 -> bres_[16 b + 1 + D + 4]
  template <int D>
  void launch_batch_pair_energy_d(int bpe, int na) {
    pb();
    k_batch_pair_energy<R, D><<<dim3(bpe, na), kRedThreads, 0, stream_>>>(bpsi_, N_, nc_, active_, partials_);
    done("reduce", sizeof(cplx<R>) * D * (double)N_ * na);
    pb();
    k_seg_finish<1><<<(na + 127) / 128, 128, 0, stream_>>>(partials_, bpe, na, active_, 0, bres_ + 1 + D + 4, 16);
    done("reduce_finish", 8.0 * bpe * na);
  }

  template <int D>
  void launch_batch_energy_local_d(int bpe, int na) {
    pb();
    k_batch_energy_local<R, D><<<dim3(bpe, na), kRedThreads, 0, stream_>>>(bpsi_, N_, nc_, active_, V_, st_, partials_);
    done("reduce", (sizeof(cplx<R>) * D + sizeof(R)) * (double)N_ * na);
    pb();
    k_seg_finish<D + 4><<<(na + 127) / 128, 128, 0, stream_>>>(partials_, bpe, na, active_, 0, bres_ + 1, 16);
    done("reduce_finish", 8.0 * (D + 4) * bpe * na);
  }

  // ---- fused row pass
  PotArgs<R> pot_full(double tau_half, bool it) const {
    // the half-potential stage without DDI/tensor: diag(tau/2) SM(tau/2) SM(tau/2) diag(tau/2)
    PotArgs<R> a = pot_args(tau_half / 2, it);
    const bool sm = std::fabs(s_.c1) >= 1e-30 && s_.D > 1;
    a.pre_diag = 1;
    a.rot_a = sm;
    a.nem_a = a.nem_b = nematic();
    a.rot_b = sm;
    a.post_diag = 1;
    a.tau_s = (R)(tau_half / 2);
    return a;
  }

  RowArgs<R> row_args(bool scale) const {
    RowArgs<R> a{};
    a.psi = psi_[kPsi];
    a.N = N_;
    a.n_rows = N_ / s_.n[0];
    a.flags = scale ? RP_SCALE : 0;
    a.norm_total = results_ + 40;
    a.dV = s_.dV;
    a.partials = partials_;
    return a;
  }

  int launch_row(const RowArgs<R>& a) {
    if (a.flags & RP_NORM) {
      if ((size_t)a.n_rows * std::max(a.n_slots, 1) > partials_n_) fail(SBEC_ERR_UNSUPPORTED, "too many rows for the norm partials");
    }
    const int nx = s_.n[0];
    const int rpb = row_rpb_host(sizeof(R) == 4, nx, s_.D, v_row_);
    const int bps = (int)((a.n_rows + rpb - 1) / rpb);
    const int nb = a.active ? bps * a.n_slots : bps;
    if (a.active && a.blocks_per_solve != bps) fail(SBEC_ERR_INVALID, "row pass blocks per solve mismatch");
    const LineCtx<R> c = line_ctx();
    const Tw<R> tw = twiddle(nx);
    const int D = s_.D;
    pb();
    row_variant_launch(v_row_, c, tw, nx, D, a, nb);
    done("row_pass", 2.0 * (double)sizeof(cplx<R>) * nc_ + (double)sizeof(R) * N_ * ((a.flags & RP_POT1) ? 1 : 0));
    return nb;
  }

  void finish_row_norm(int nb) {
    if ((size_t)nb > partials_n_) fail(SBEC_ERR_UNSUPPORTED, "too many row blocks");
    pb();
    launch_pdl(k_reduce_finish<1>, dim3(1), dim3(32), 0, (const double*)partials_, nb, 0, results_ + 40);
    done("reduce_finish", 8.0 * nb);
  }

  // The kinetic passes over the axes above x: 2-D: y fwd*phase*inv;
  // 3-D: y fwd, z fwd*phase*inv, y inv.
  void last_axes_kinetic() {
    const int nx = s_.n[0], ny = s_.n[1], nz = s_.n[2];
    const int64_t D = s_.D;
    if (s_.ndim == 2) {
      fft_strided_n(ny, psi_[kPsi], (int64_t)nx, (int64_t)nx, D, N_, ny, ny, 2);
    } else {
      fft_strided_n(ny, psi_[kPsi], (int64_t)nx, (int64_t)nx, (int64_t)nz * D,
                               (int64_t)nx * ny, ny, ny, 0);
      fft_strided_n(nz, psi_[kPsi], (int64_t)nx * ny, (int64_t)nx * ny, D, N_, nz, nz, 2);
      fft_strided_n(ny, psi_[kPsi], (int64_t)nx, (int64_t)nx, (int64_t)nz * D,
                               (int64_t)nx * ny, ny, ny, 1);
    }
  }

  // ---- DDI
  DdiGeom geom(int kind) const {
    DdiGeom g{};
    g.ndim = s_.ndim;
    g.nx = s_.n[0];
    g.ny = s_.ndim >= 2 ? s_.n[1] : 1;
    g.nz = s_.ndim >= 3 ? s_.n[2] : 1;
    g.Mx = s_.conv_M[kind][0];
    g.My = s_.conv_M[kind][1];
    g.Mz = s_.conv_M[kind][2];
    g.Hx = g.Mx / 2 + 1;
    g.field_stride = (int64_t)g.Hx * g.My * g.nz;
    g.kmx = s_.conv_kmult[kind][0];
    g.kmy = s_.conv_kmult[kind][1];
    g.kmz = s_.conv_kmult[kind][2];
    g.C = s_.c_dd / ((double)g.Mx * g.My * g.Mz);
    g.secular = s_.secular ? 1 : 0;
    return g;
  }

  template <int MH>
  void launch_ddi_r2c(const R* f3, cplx<R>* spec, const DdiGeom& g, R* phi3) {
    constexpr int LPB = ddi_x_rows_per_block<R, MH>();
    constexpr int TPL = MH / PlanOf<R, MH>::E;
    const size_t smem = sizeof(cplx<R>) * 3 * LPB * (2 * MH + 1);
    auto kern = k_ddi_r2c_x<R, MH, LPB>;
    static const bool once = (set_smem(kern, smem), true);
    (void)once;
    const int64_t rows = (int64_t)g.ny * g.nz;
    pb();
    kern<<<(unsigned)((rows + LPB - 1) / LPB), 3 * LPB * TPL, smem, stream_>>>(f3, N_, spec, g, phi3, twiddle(MH),
                                                                               twiddle(2 * MH));
    done("ddi_r2c_x", (3.0 * (double)sizeof(R) * g.nx + 3.0 * (double)sizeof(cplx<R>) * g.Hx) * (double)rows);
  }

  template <int MH>
  void launch_ddi_c2r(const cplx<R>* spec, const DdiGeom& g, R* phi3) {
    constexpr int LPB = ddi_x_rows_per_block<R, MH>();
    constexpr int TPL = MH / PlanOf<R, MH>::E;
    const size_t smem = sizeof(cplx<R>) * 3 * LPB * (2 * MH + 1);
    auto kern = k_ddi_c2r_x<R, MH, LPB>;
    static const bool once = (set_smem(kern, smem), true);
    (void)once;
    const int64_t rows = (int64_t)g.ny * g.nz;
    pb();
    kern<<<(unsigned)((rows + LPB - 1) / LPB), 3 * LPB * TPL, smem, stream_>>>(spec, g, phi3, N_, twiddle(MH),
                                                                               twiddle(2 * MH));
    done("ddi_c2r_x", (3.0 * (double)sizeof(R) * g.nx + 3.0 * (double)sizeof(cplx<R>) * g.Hx) * (double)rows);
  }

  template <int M>
  void launch_ddi_last(cplx<R>* spec, const DdiGeom& g, int64_t S, int64_t inner, int n_in, int n_out) {
    constexpr int W = ddi_last_width<R, M>();
    constexpr int TPL = M / PlanOf<R, M>::E;
    const size_t smem = sizeof(cplx<R>) * 3 * W * M;
    auto kern = k_ddi_last<R, M, W>;
    static const bool once = (set_smem(kern, smem), true);
    (void)once;
    pb();
    kern<<<(unsigned)((inner + W - 1) / W), 3 * W * TPL, smem, stream_>>>(spec, g, S, inner, n_in, n_out,
                                                                         twiddle(M));
    done("ddi_last", 3.0 * (double)sizeof(cplx<R>) * (double)(n_in + n_out) * (double)inner);
  }

  // Φ = C_dd Q * F on convolution grid `kind` (0 periodic, 1 zero padded).
  void ddi_conv(int kind, const R* f3, R* phi3) {
    const DdiGeom g = geom(kind);
    cplx<R>* spec = spec_[kind];
    if (!spec) fail(SBEC_ERR_INVALID, "DDI convolution buffers missing");
    const int MH = g.Mx / 2;
    if (MH < 2) fail(SBEC_ERR_UNSUPPORTED, "DDI needs at least 4 points along x");
    SBEC_SWITCH_POW2(MH, launch_ddi_r2c, f3, spec, g, phi3);
    if (g.ndim == 1) return;
    if (g.ndim == 2) {
      SBEC_SWITCH_POW2_STRIDED(g.My, launch_ddi_last, spec, g, (int64_t)g.Hx, (int64_t)g.Hx, g.ny, g.ny);
    } else {
      const int64_t plane = (int64_t)g.Hx * g.My;
      fft_strided_n(g.My, spec, (int64_t)g.Hx, (int64_t)g.Hx, (int64_t)3 * g.nz,
                               plane, g.ny, g.My, 0);
      SBEC_SWITCH_POW2_STRIDED(g.Mz, launch_ddi_last, spec, g, plane, plane, g.nz, g.nz);
      fft_strided_n(g.My, spec, (int64_t)g.Hx, (int64_t)g.Hx, (int64_t)3 * g.nz,
                               plane, g.My, g.ny, 1);
    }
    SBEC_SWITCH_POW2(MH, launch_ddi_c2r, spec, g, phi3);
  }

  // ---- pointwise launchers
  // The singlet-pair (nematic) step runs when c2 is set and the tensor path is off
  // (src/split_step.jl:60-75, src/nematic.jl:44).
  int nematic() const { return (!s_.tensor && std::fabs(s_.c2) >= 1e-30) ? 1 : 0; }

  PotArgs<R> pot_args(double tau_d, bool it) const {
    PotArgs<R> a{};
    a.psi = psi_[kPsi];
    a.N = N_;
    a.V = V_;
    a.itp = it ? 1 : 0;
    a.tau_d = (R)tau_d;
    a.c0 = (R)s_.c0;
    a.c1 = (R)s_.c1;
    a.c_lhy = (R)s_.c_lhy;
    a.c2 = (R)s_.c2;
    zeeman_factors(tau_d, it, a.zee, a.zee_lo);
    a.rg = raman_geom();
    return a;
  }

  RamanGeom raman_geom() const {
    RamanGeom g{};
    g.omega = s_.raman_omega;
    g.delta = s_.raman_delta;
    for (int d = 0; d < 3; ++d) {
      g.k[d] = s_.raman_k[d];
      g.x0[d] = s_.x0[d];
      g.dx[d] = s_.dx[d];
    }
    g.n0 = s_.n[0];
    g.n1 = s_.n[1];
    return g;
  }

  // Zeeman factors (src/propagators.jl:95-116): cis(-E_c tau) or exp(-(E_c - min E) tau).
  void zeeman_factors(double tau, bool it, cplx<R>* out, cplx<R>* out_lo) const {
    const int D = s_.D, F = s_.F;
    double E[kMaxD];
    double emin = INFINITY;
    for (int c = 0; c < D; ++c) {
      const double m = (double)(F - c);
      E[c] = -zeeman_p * m + zeeman_q * (m * m);
      emin = std::min(emin, E[c]);
    }
    for (int c = 0; c < D; ++c) {
      double re, im;
      if (it) {
        re = std::exp(-((E[c] - emin) * tau));
        im = 0.0;
      } else {
        const double arg = -(E[c] * tau);
        re = std::cos(arg);
        im = std::sin(arg);
      }
      out[c] = mk<R>((R)re, (R)im);
      out_lo[c] = mk<R>((R)(re - (double)out[c].x), (R)(im - (double)out[c].y));
      if (sizeof(R) == 4 && !it) {
        // the FP32 real-time diagonal step turns by e^{i arg} in small quantities
        // (rot_small_zee): cos arg - 1 = -2 sin^2(arg / 2) without cancellation, and sin arg
        const double s2 = std::sin(-(E[c] * tau) / 2);
        out_lo[c] = mk<R>((R)(-2.0 * s2 * s2), (R)im);
      }
    }
  }

  TensorArgs<R> tensor_args(double tau_d, double tau_t, bool it) const {
    TensorArgs<R> a{};
    a.psi = psi_[kPsi];
    a.N = N_;
    a.V = V_;
    a.G = G_;
    a.G32 = G32_;
    a.bound_coef = s_.bound_coef;
    a.itp = it ? 1 : 0;
    a.tau = (R)tau_t;
    a.tau_d = (R)tau_d;
    a.c0 = (R)s_.c0;
    a.c_lhy = (R)s_.c_lhy;
    a.eps = sizeof(R) == 8 ? 1e-17 : 1e-13;  // FP32: keep the norm change of the truncated series far below the FP32 rounding
    zeeman_factors(tau_d, it, a.zee, a.zee_lo);
    return a;
  }

  template <int D>
  void launch_potential_d(const PotArgs<R>& a) {
    pb();
    k_potential<R, D><<<(unsigned)((N_ + 255) / 256), 256, 0, stream_>>>(a, st_);
    done("potential", (2.0 * (double)sizeof(cplx<R>) * D + (double)sizeof(R) * (1 + (a.phi ? 3 : 0) + (a.spin_out ? 3 : 0))) * (double)N_);
  }
  void launch_potential(const PotArgs<R>& a) { SBEC_SWITCH_D(s_.D, launch_potential_d, a); }

  template <int D, int RL>
  void launch_tensor_lanes(const TensorArgs<R>& a) {
    if constexpr (sizeof(R) == 4) {
      using TL = TensorLanes<D, RL>;
      const size_t smem = TL::smem_bytes();
      auto kern = k_tensor_lanes<D, RL>;
      static const bool once = (set_smem(kern, smem), true);
      (void)once;
      pb();
      kern<<<(unsigned)((N_ + TL::PPB - 1) / TL::PPB), 256, smem, stream_>>>(a);
      done("tensor", (2.0 * (double)sizeof(cplx<R>) * D + (double)sizeof(R)) * (double)N_);
    }
  }

  template <int D>
  void launch_tensor_d(const TensorArgs<R>& a) {
    if constexpr (sizeof(R) == 4) {
      // default: rows of h in registers up to D = 5, lane groups with two rows per lane above
      // (ms per call on a 128^3 grid, modes 1 / 2 / 3: D = 5 1.38 / 0.69 / 0.85, D = 7 1.58 /
      // 1.42 / 1.20, D = 9 3.23 / 3.01 / 2.25, D = 11 3.76 / 6.34 / 3.49, D = 13 2.91 / 9.04 /
      // 2.46; the rows kernel's registers grow with D: 255 at D = 13, 7 warps per SM)
      const int mode = tensor_mode_ >= 0 ? tensor_mode_ : (D <= 5 ? 2 : 3);
      if (mode == 2) {
        constexpr int NW = (D + 1) / 2;
        pb();
        k_tensor_rows<D, NW><<<(unsigned)((N_ + 31) / 32), 32 * NW, 0, stream_>>>(a);
        done("tensor", (2.0 * (double)sizeof(cplx<R>) * D + (double)sizeof(R)) * (double)N_);
        return;
      }
      if (mode == 1) {
        launch_tensor_lanes<D, 1>(a);
        return;
      }
      if (mode == 3) {
        launch_tensor_lanes<D, 2>(a);
        return;
      }
    }
    constexpr int T = 64;
    const size_t smem = sizeof(cplx<R>) * T * (D * (D + 1) / 2);
    auto kern = k_tensor<R, D>;
    static const bool once = (set_smem(kern, smem), true);
    (void)once;
    pb();
    kern<<<(unsigned)((N_ + T - 1) / T), T, smem, stream_>>>(a);
    done("tensor", (2.0 * (double)sizeof(cplx<R>) * D + (double)sizeof(R)) * (double)N_);
  }
  void launch_tensor(const TensorArgs<R>& a) { SBEC_SWITCH_D(s_.D, launch_tensor_d, a); }

  template <int D>
  void launch_spin_density_d(R* out) {
    pb();
    k_spin_density<R, D><<<(unsigned)((N_ + 255) / 256), 256, 0, stream_>>>(psi_[kPsi], N_, st_, out);
    done("spin_density", ((double)sizeof(cplx<R>) * D + 3.0 * (double)sizeof(R)) * (double)N_);
  }

  template <int D>
  void launch_energy_local_d(int nb) {
    pb();
    k_energy_local<R, D><<<nb, kRedThreads, 0, stream_>>>(psi_[kPsi], N_, V_, st_, partials_);
    done("reduce", ((double)sizeof(cplx<R>) * D + (double)sizeof(R)) * (double)N_);
  }

  template <int D>
  void launch_pair_energy_d(int nb) {
    pb();
    k_pair_energy<R, D><<<nb, kRedThreads, 0, stream_>>>(psi_[kPsi], N_, partials_);
    done("reduce", (double)sizeof(cplx<R>) * D * (double)N_);
  }

  template <int D>
  void launch_tensor_energy_d(int nb) {
    pb();
    k_tensor_energy<R, D><<<nb, kRedThreads, 0, stream_>>>(psi_[kPsi], N_, pairs_, pcg_, (int)s_.pair_a.size(), gA_,
                                                          (int)s_.gA.size(), partials_);
    done("reduce", (double)sizeof(cplx<R>) * D * (double)N_);
  }

  template <int D>
  void launch_loss_d(LossRates<R> lr, R half_dt) {
    pb();
    k_loss<R, D><<<(unsigned)((N_ + 255) / 256), 256, 0, stream_>>>(psi_[kPsi], N_, lr, half_dt);
    done("loss", 2.0 * (double)sizeof(cplx<R>) * D * (double)N_);
  }

  template <int D>
  void launch_raman_energy_d(int nb) {
    pb();
    k_raman_energy<R, D><<<nb, kRedThreads, 0, stream_>>>(psi_[kPsi], N_, st_, raman_geom(), partials_);
    done("reduce", (double)sizeof(cplx<R>) * D * (double)N_);
  }

  template <int D>
  void launch_phase_sums_d(const cplx<R>* buf, int nb) {
    pb();
    k_phase_sums<R, D><<<nb, kRedThreads, 0, stream_>>>(buf, N_, st_, phase_pairs_, phase_cg_, n_phase_pairs_,
                                                       partials_);
    done("reduce", (double)sizeof(cplx<R>) * D * (double)N_);
  }

  template <int D>
  void launch_comp_norms_d(const cplx<R>* buf, int nb) {
    pb();
    k_comp_norms<R, D><<<nb, kRedThreads, 0, stream_>>>(buf, N_, partials_);
    done("reduce", (double)sizeof(cplx<R>) * D * (double)N_);
  }

  // per-component sums into results_[1..D], NaN count into results_[D+1]
  void comp_norms_async(const cplx<R>* buf) {
    const int nb = red_blocks(N_);
    SBEC_SWITCH_D(s_.D, launch_comp_norms_d, buf, nb);
    switch (s_.D) {
      case 1: finish<2>(nb, false, 1); break;
      case 3: finish<4>(nb, false, 1); break;
      case 5: finish<6>(nb, false, 1); break;
      case 7: finish<8>(nb, false, 1); break;
      case 9: finish<10>(nb, false, 1); break;
      case 11: finish<12>(nb, false, 1); break;
      case 13: finish<14>(nb, false, 1); break;
    }
  }

  int64_t N_ = 0, nc_ = 0;
  cplx<R>* psi_[kNumSlots] = {nullptr, nullptr, nullptr, nullptr};
  cplx<R>* scratch_ = nullptr;
  R* V_ = nullptr;
  R* tmp3_ = nullptr;
  cplx<R>* ptab_[3] = {nullptr, nullptr, nullptr};
  cplx<R>* ptab_lo_[3] = {nullptr, nullptr, nullptr};
  std::map<int, Tw<R>> tw_;
  std::map<int, BlueTab> blue_;  // Bluestein tables by +-n
  cplx<R>* blue_scr_ = nullptr;
  size_t blue_scr_n_ = 0;
  double* partials_ = nullptr;
  size_t partials_n_ = 0;
  double* results_ = nullptr;
  double* host_res_ = nullptr;
  double* host_psi_ = nullptr;
  double* host_tmp_ = nullptr;
  int64_t host_tmp_n_ = 0;
  double2* stage_ = nullptr;
  SpinTabs<R> st_;
  double* G_ = nullptr;
  int4* pairs_ = nullptr;
  int4* phase_pairs_ = nullptr;  // classify_phase pair table (built on first use)
  double* phase_cg_ = nullptr;
  int n_phase_pairs_ = 0;
  double* pcg_ = nullptr;
  double* gA_ = nullptr;
  R* spin3_ = nullptr;
  R* phi3_ = nullptr;
  R* phi_per_ = nullptr;
  cplx<R>* spec_[2] = {nullptr, nullptr};
  std::map<GraphKey, GraphEntry> graphs_;
  size_t n_graphs_ = 0;  // instantiated graphs in graphs_
  const int* omap_ = nullptr;  // outer-index map for batched strided passes (null: identity)
  int nsolve_ = 1, n_active_ = 0, active_version_ = 0;
  cplx<R>* bpsi_ = nullptr;
  cplx<R>* bprev_ = nullptr;
  cplx<R>* bscratch_ = nullptr;
  R* c0s_ = nullptr;
  R* c1s_ = nullptr;
  int* active_ = nullptr;
  double* bnorm_ = nullptr;
  double* bres_ = nullptr;
  int oper_ = 1;
  bool use_graphs_ = true;
  bool use_pdl_ = true;  // programmatic dependent launch (SBEC_PDL=0 disables)
  bool segment_on_ = false;     // persistent leapfrog segments (SBEC_SEGMENT=1 enables)
  bool segment_used_ = false;   // a segment ran since the last check_segments()
  bool segment_stall_ = false;  // SBEC_FAULT_SEGMENT_STALL: one injected barrier stall (tests)
  GridBarrier* bar_ = nullptr;  // grid barrier of the segment kernel
  GridBarrier* bar_host_ = nullptr;
  // line-kernel variants in use (see sbec_lines.h); chosen by the autotuner
  int v_row_ = 0, v_str_ = 0, v_x_ = 0;
  bool merged_itp_ = false;  // SBEC_BATCH_MERGED=1: two-pass FP32 batched ITP step (predicted scale)
  // FP32 tensor kernel (SBEC_TENSOR_LANES): 0 one thread per point, 1 a lane group per point
  // (one row of h per lane), 2 rows of h in registers ((D + 1) / 2 warps per 32 points), 3 a
  // lane group with two rows per lane; -1 (default) by D
  int tensor_mode_ = -1;
  // 1-D fused ITP steps in one launch (k_row_itp_steps); SBEC_ITP_STEPS=0: one launch per step
  bool use_itp_steps_ = true;
  float* G32_ = nullptr;
  R* bcorr_ = nullptr;  // merged FP32 batched ITP: per-solve correction, prediction, ones
  R* bpred_ = nullptr;
  R* bones_ = nullptr;
  cudaStream_t side_ = nullptr;  // pipelined snapshots: reductions and copies of the save points
  cudaEvent_t copied_ev_[2] = {nullptr, nullptr};
  cplx<R>* snap_copy_[2] = {nullptr, nullptr};
  double2* snap_stage_[2] = {nullptr, nullptr};
  double* side_partials_ = nullptr;
  size_t side_partials_n_ = 0;
  double* side_results_ = nullptr;
  cplx<R>* side_scratch_ = nullptr;
  double* snap_res_[2] = {nullptr, nullptr};  // pinned snapshot slots
  double* snap_psi_[2] = {nullptr, nullptr};
  cudaEvent_t snap_ev_[2] = {nullptr, nullptr};
  bool tune_on_ = true;       // SBEC_TUNE=0: variant 0 everywhere
  int tune_force_ = -1;       // SBEC_TUNE_FORCE=v: variant v wherever it is compiled (line kernels: v & 7)
  bool row_tuned_ = false;
  std::map<std::string, int> tuned_;  // this engine's strided / x decisions by call shape
  std::vector<std::string> tune_log_;
  cplx<R>* tune_buf_ = nullptr;
  size_t tune_buf_n_ = 0;
  bool capturing_ = false;
  long long cap_launch0_ = 0;
  double phase_dt_ = NAN;
  int phase_itp_ = -1;
  std::vector<void*> allocs_;
};

}  // namespace sbec
