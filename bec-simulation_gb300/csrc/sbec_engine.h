// Precision-independent engine interface used by the C ABI and the drivers.
#pragma once

#include <cuda_runtime.h>

#include <memory>

#include "sbec_setup.h"

namespace sbec {

// Buffers a driver can save psi into (adaptive loops, convergence checks).
enum Slot { kPsi = 0, kSlotA = 1, kSlotB = 2, kSlotC = 3, kNumSlots = 4 };

class EngineBase {
 public:
  explicit EngineBase(Setup s) : s_(std::move(s)) {}
  virtual ~EngineBase() = default;
  const Setup& setup() const { return s_; }
  cudaStream_t stream() const { return stream_; }

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
  virtual void scale_components(const double* w) = 0;   // host weights, D values
  virtual void copy_slot(int dst, int src) = 0;

  // reductions (synchronise the stream)
  virtual void comp_norms(double* sums, double* nan_count) = 0;  // sum |psi_c|^2 per component
  virtual sbec_energy_terms energy_terms() = 0;
  virtual double l2_change(int a, int b) = 0;                      // ||a-b||^2/||b||^2
  virtual void max_abs(int a, int b, double* max_a, double* max_diff) = 0;
  virtual double ddi_phi_max() = 0;                                // last periodic Φ (ITP check)
  virtual void spin_density(double* host3N) = 0;
  virtual void ddi_potential(bool padded, double* host3N) = 0;
  virtual void sync() = 0;

 protected:
  Setup s_;
  cudaStream_t stream_ = nullptr;
};

std::unique_ptr<EngineBase> make_engine_f64(const Setup& s);
std::unique_ptr<EngineBase> make_engine_f32(const Setup& s);

void cuda_check(cudaError_t e, const char* what);

}  // namespace sbec
