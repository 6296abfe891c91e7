// Precision-independent engine interface used by the C ABI and the drivers.
#pragma once

#include <cuda_runtime.h>

#include <atomic>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "sbec_setup.h"

namespace sbec {

void cuda_check(cudaError_t e, const char* what);
// Message returned by sbec_last_error() on the calling thread.
void set_last_error(const std::string& msg);

// Per-kernel-category launch counts and (when enabled) CUDA-event durations on
// the workspace stream; the counterpart of the reference's @timeit_debug
// substep timers (src/split_step.jl:15-131, src/SpinorBEC.jl:175-186).
class Profiler {
 public:
  struct Stat {
    long long launches = 0;
    double ms = 0.0;
    double bytes = 0.0;  // algorithmic bytes summed over timed launches
  };
  ~Profiler() { release(); }
  void enable(bool on) {
    drain();
    enabled_ = on;
    stats_.clear();
  }
  bool enabled() const { return enabled_; }
  long long total_launches() const { return total_; }
  void add_launches(long long n) { total_ += n; }
  void begin(cudaStream_t s) {
    if (!enabled_) return;
    cur_ = get_event();
    cuda_check(cudaEventRecord(cur_, s), "cudaEventRecord");
  }
  void end(cudaStream_t s, const char* name, double bytes) {
    ++total_;
    if (!enabled_) return;
    cudaEvent_t stop = get_event();
    cuda_check(cudaEventRecord(stop, s), "cudaEventRecord");
    pending_.push_back({name, cur_, stop, bytes});
    if (pending_.size() > 4000) drain();
  }
  const std::map<std::string, Stat>& read() {
    drain();
    return stats_;
  }

 private:
  struct Pending {
    std::string name;
    cudaEvent_t a, b;
    double bytes;
  };
  cudaEvent_t get_event() {
    if (free_.empty()) {
      cudaEvent_t e;
      cuda_check(cudaEventCreate(&e), "cudaEventCreate");
      all_.push_back(e);
      return e;
    }
    cudaEvent_t e = free_.back();
    free_.pop_back();
    return e;
  }
  void drain() {
    for (auto& p : pending_) {
      cuda_check(cudaEventSynchronize(p.b), "cudaEventSynchronize");
      float ms = 0.f;
      cuda_check(cudaEventElapsedTime(&ms, p.a, p.b), "cudaEventElapsedTime");
      Stat& st = stats_[p.name];
      st.launches += 1;
      st.ms += ms;
      st.bytes += p.bytes;
      free_.push_back(p.a);
      free_.push_back(p.b);
    }
    pending_.clear();
  }
  void release() {
    for (auto e : all_) cudaEventDestroy(e);
    all_.clear();
  }
  bool enabled_ = false;
  long long total_ = 0;
  cudaEvent_t cur_ = nullptr;
  std::vector<Pending> pending_;
  std::vector<cudaEvent_t> free_, all_;
  std::map<std::string, Stat> stats_;
};

// Grid sums of classify_phase: n, n^2, |<F>|^2, m|psi|^2 and F_max + 1 = 7 channel weights.
constexpr int kPhaseSums = 11;

// Buffers a driver can save psi into (adaptive loops, convergence checks).
enum Slot { kPsi = 0, kSlotA = 1, kSlotB = 2, kSlotC = 3, kNumSlots = 4 };

class EngineBase {
 public:
  explicit EngineBase(Setup s) : s_(std::move(s)) {}
  virtual ~EngineBase() = default;
  const Setup& setup() const { return s_; }
  cudaStream_t stream() const { return stream_; }
  Profiler prof;

  double zeeman_p = 0.0, zeeman_q = 0.0;
  double t = 0.0;
  long long step = 0;
  double dt = 0.0;         // SimParams.dt (split_step!)
  bool itp = false;        // SimParams.imaginary_time
  int normalize_every = 0;

  virtual void set_psi(const double* host) = 0;
  virtual void get_psi(double* host) = 0;
  virtual void set_potential(const double* host) = 0;

  // operators (stream ordered, no host synchronisation)
  virtual void half_potential(double dt_half, bool imaginary_time) = 0;
  virtual void kinetic(double dt, bool imaginary_time) = 0;
  virtual void normalize() = 0;                         // device-side _normalize_psi!
  virtual void apply_loss(double dt) = 0;               // apply_loss_step! (no-op without losses)
  virtual void scale_components(const double* w) = 0;   // host weights, D values
  virtual void copy_slot(int dst, int src) = 0;

  // reductions (synchronise the stream)
  virtual void comp_norms(double* sums, double* nan_count) = 0;  // sum |psi_c|^2 per component
  virtual sbec_energy_terms energy_terms() = 0;
  // total_energy terms plus the component sums of the same psi (one device->host fetch)
  virtual sbec_energy_terms energy_terms_and_norms(double* comp_sums) = 0;
  // psi downloaded into the workspace's pinned staging buffer (valid until the next call)
  virtual const double* psi_to_pinned() = 0;
  // Pipelined snapshots (two slots, k & 1): enqueue energy sums and the FP64 psi into
  // pinned slot k; wait for slot k and read it; restore psi from slot k.
  virtual void snapshot_enqueue(int k) = 0;
  virtual const double* snapshot_wait(int k, sbec_energy_terms* terms, double* comp_sums) = 0;
  virtual void restore_snapshot(int k) = 0;
  virtual double l2_change(int a, int b) = 0;                      // ||a-b||^2/||b||^2
  virtual void max_abs(int a, int b, double* max_a, double* max_diff) = 0;
  virtual double ddi_phi_max() = 0;                                // last periodic Φ (ITP check)
  virtual void spin_density(double* host3N) = 0;
  // classify_phase grid sums (k_phase_sums): [n, n^2, |<F>|^2, m|psi|^2, W_0, W_2, ..., W_2F]
  // of the workspace psi (solve < 0) or of one solve of a batch; kPhaseSums doubles.
  virtual void phase_sums(int solve, double* out) = 0;
  virtual void ddi_potential(bool padded, double* host3N) = 0;
  virtual void sync() = 0;

  // Fused paths (no DDI, no tensor, supported line length / D): a leapfrog step is a
  // row pass plus the last-axis pass; an ITP split_step defers its renormalisation
  // into the next row pass.
  virtual bool fused_path() const = 0;
  // Smallest relative change of psi the form can resolve: 0 in FP64; in FP32 eight units in
  // the last place (2^-21), below which max|psi - psi_prev| / max|psi| is rounding noise.
  virtual double psi_resolution() const = 0;
  virtual std::string tuning_report() const = 0;  // autotuner decisions of this engine
  virtual void lf_open(double dt) = 0;               // V(dt/2), forward x
  virtual void lf_steps(long long n, double dt) = 0;  // n x [K(dt) with merged V(dt)]
  virtual void lf_close(double dt) = 0;              // K(dt), V(dt/2)
  virtual void check_segments() {}                   // report a failed persistent segment
  virtual void set_graphs(bool on) = 0;               // sbec_set_graph_mode
  virtual void fused_split_steps(long long n, double dt, double kin_dt, bool kin_itp, bool itp,
                                 bool normalize) = 0;
  // The same operator sequences on the general path (DDI, tensor, any D), replayed from
  // CUDA graphs of a few steps: n x split_step! and n x [K(kin_dt), V(dt)].
  virtual void unfused_split_steps(long long n, double dt, double kin_dt, bool kin_itp, bool itp,
                                   bool normalize) = 0;
  virtual void unfused_lf_steps(long long n, double dt, double kin_dt, bool kin_itp) = 0;

  // Batches of independent solves sharing grid, F, V, dt and Zeeman (per-solve c0, c1, psi).
  virtual int n_solves() const = 0;
  virtual void batch_init(int n, const double* c0, const double* c1, const double* psi_all) = 0;
  virtual void batch_set_active(const std::vector<int>& active) = 0;
  virtual void batch_itp_steps(long long n, double dt) = 0;    // fused ITP split_step! x n, renormalised
  virtual void batch_energies(double* E) = 0;                  // total_energy per solve (all solves)
  virtual void batch_max_abs(double* pmax, double* dmax) = 0;  // vs the saved previous psi (active solves)
  virtual void batch_save_prev() = 0;
  virtual void batch_save_prev_solve(int solve) = 0;  // the same for one solve
  virtual bool batch_has_nan() = 0;
  virtual void batch_get_psi(int solve, double* host) = 0;

 protected:
  Setup s_;
  cudaStream_t stream_ = nullptr;
};

// Process-wide autotuner decisions (line-kernel call shape -> variant), shared by both
// precisions and every workspace and batch; guarded by tune_table_mutex().
std::mutex& tune_table_mutex();
std::map<std::string, int>& tune_table_map();
// sbec_tune_freeze: shapes missing from the table take the default variant (untimed)
std::atomic<bool>& tune_frozen();

// Whether a grid takes the fused row / column passes (the batch and leapfrog fast path):
// power-of-two axes, no DDI / tensor / Raman / losses, D in {1, 3, 5}, a row-pass variant that
// fits (threads, shared memory) for the first axis.  Host-only; defined with the FP32 engine.
bool fused_path_supported(const Setup& s, bool fp32);

std::unique_ptr<EngineBase> make_engine_f64(const Setup& s);
std::unique_ptr<EngineBase> make_engine_f32(const Setup& s);

}  // namespace sbec
