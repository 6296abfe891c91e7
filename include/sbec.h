/*
 * sbec.h — C ABI of the GB300-native split-step engine for SpinorBEC.jl.
 *
 * The library replaces the Julia hot path of SpinorBEC.jl (anko9801/BEC-simulation):
 * the per-step operators, the integrators and the drivers that loop over them.
 * A Julia shim keeps the reference API (make_workspace, split_step!, run_simulation!,
 * run_simulation_adaptive!, run_simulation_yoshida!, find_ground_state, ...) and
 * forwards to these entry points with `ccall`; the Python package `spinorbec` in
 * this repository mirrors the same API over ctypes.
 *
 * Conventions
 *  - Wavefunction buffers on the host are the reference's own layout
 *    (src/types.jl:239-244): complex Float64, interleaved re/im, column-major
 *    psi[x,(y,(z,))c], x fastest, one planar block of prod(n) points per
 *    component; component c (0-based) carries m = F - c.
 *  - The library copies host buffers; it never keeps a caller pointer after a call returns.
 *  - Every entry point returns an sbec_status.  On failure, sbec_last_error() returns a
 *    message for the calling thread (valid until that thread's next call).
 *  - A workspace owns all its device memory and one CUDA stream.  Distinct workspaces are
 *    independent; one workspace must be used from one host thread at a time.
 *  - There is no CPU fallback: without a usable CUDA device every entry point that needs
 *    one returns SBEC_ERR_DEVICE.
 */
#ifndef SBEC_H
#define SBEC_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum sbec_status {
  SBEC_OK = 0,
  SBEC_ERR_INVALID = 1,      /* invalid argument / configuration (ArgumentError in the reference) */
  SBEC_ERR_UNSUPPORTED = 2,  /* option outside the GPU path (non power-of-two n, F > 6, ...) */
  SBEC_ERR_OOM = 3,          /* device allocation failed */
  SBEC_ERR_NUMERIC = 4,      /* NaN / ITP overflow detected (src/ground_state.jl:4-29) */
  SBEC_ERR_DEVICE = 5,       /* CUDA error or no device */
  SBEC_ERR_CALLBACK = 6      /* a host callback returned non-zero (the run stops) */
} sbec_status;

typedef enum sbec_precision {
  SBEC_FP64 = 0,             /* plain form: complex FP64 everywhere */
  SBEC_FP32_BULK = 1         /* FFTs and pointwise phases in FP32; reductions, norm, energy, errors in FP64 */
} sbec_precision;

#define SBEC_MAX_C_EXTRA 32
#define SBEC_MAX_CHANNELS 32

/* Workspace configuration: the arguments of `make_workspace`
 * (src/initialization.jl:86-101) that reach the hot path. */
typedef struct sbec_config {
  int32_t ndim;              /* 1, 2 or 3 */
  int32_t n[3];              /* points per axis (GridConfig.n_points, src/types.jl:7-20) */
  double L[3];               /* box size per axis (GridConfig.box_size) */
  int32_t F;                 /* spin (atom.F) */
  double c0, c1, c_lhy;      /* InteractionParams (src/types.jl:145-162) */
  int32_t n_c_extra;         /* InteractionParams.c_extra: c_extra[i] = c_{i+2} */
  double c_extra[SBEC_MAX_C_EXTRA];
  int32_t gS_direct;         /* 1: use gS[] below as channel couplings g_S (S = 0,2,...,2F), bypassing
                                the c0/c1/c_extra activation rule (_make_tensor_cache_from_channels) */
  double gS[SBEC_MAX_CHANNELS];
  double zeeman_p, zeeman_q; /* ZeemanParams (src/types.jl:172-178); time-dependent: sbec_set_zeeman */
  int32_t enable_ddi;
  double c_dd;
  int32_t secular_ddi;
  int32_t ddi_padding;
  double dt;                 /* SimParams.dt */
  int32_t imaginary_time;    /* SimParams.imaginary_time */
  int32_t normalize_every;   /* SimParams.normalize_every (ITP renormalisation period) */
  int32_t precision;         /* sbec_precision */
  int32_t raman;             /* 1: RamanCoupling (src/types.jl:179-183) on the half potential */
  double raman_omega, raman_delta;  /* Omega_R, delta */
  double raman_k[3];         /* k_eff per axis */
  double loss_gamma_dr, loss_L3;  /* LossParams (src/types.jl:291-296); both < 1e-30: no loss */
} sbec_config;

typedef struct sbec_ws sbec_ws;

/* Observables recorded at save points: `_record_snapshot!` (src/simulation_utils.jl:9-15). */
typedef struct sbec_snapshot {
  double t;
  int64_t step;
  double energy, norm, magnetization;
  const double* psi;         /* host copy (interleaved, reference layout), valid during the callback only */
} sbec_snapshot;

/* Save-point callback; return non-zero to stop the run (sbec returns SBEC_ERR_CALLBACK). */
typedef int (*sbec_callback)(void* user, const sbec_snapshot* snap);

/* AdaptiveDtParams (src/types.jl:343-361); error_mode 0 = :step_change, 1 = :richardson. */
typedef struct sbec_adaptive_params {
  double dt_init, dt_min, dt_max, tol;
  int32_t error_mode;
} sbec_adaptive_params;

typedef struct sbec_adaptive_result {
  int64_t n_accepted, n_rejected;
  double final_dt;
} sbec_adaptive_result;

/* find_ground_state result tuple (src/ground_state.jl:165-169). */
typedef struct sbec_gs_result {
  int32_t converged;
  double energy, dE, dpsi;
  int64_t steps;
} sbec_gs_result;

/* Terms of total_energy (src/energy.jl:6-54); `tensor` also carries the singlet-pair
 * (nematic) energy of a c2 workspace, `raman` the Raman term (src/energy.jl:123-135). */
typedef struct sbec_energy_terms {
  double kinetic, trap, zeeman, c0, c1, ddi, lhy, tensor, raman;
} sbec_energy_terms;

/* ---- diagnostics ------------------------------------------------------- */
const char* sbec_last_error(void);
const char* sbec_version(void);
/* Number of usable CUDA devices (0 when none); never fails. */
int sbec_device_count(void);

/* ---- lifecycle ----------------------------------------------------------
 * sbec_ws_create replaces make_workspace (src/initialization.jl:86-191): builds the
 * device-resident psi, potential, kinetic-phase tables, spin-matrix tables, the
 * tensor-interaction tables (activated as in src/initialization.jl:164-185) and the
 * DDI buffers (src/ddi.jl:51-102, src/ddi_padded.jl:6-49).
 * psi: n_total*D complex (2*n_total*D doubles); V: n_total doubles or NULL (NoPotential). */
sbec_status sbec_ws_create(const sbec_config* cfg, const double* psi, const double* V, sbec_ws** out);
sbec_status sbec_ws_destroy(sbec_ws* ws);

/* ---- state -------------------------------------------------------------
 * ws.state.psi / t / step (src/types.jl:239-244). */
sbec_status sbec_set_psi(sbec_ws* ws, const double* psi);
sbec_status sbec_get_psi(sbec_ws* ws, double* psi);
sbec_status sbec_set_time(sbec_ws* ws, double t, int64_t step);
sbec_status sbec_get_time(sbec_ws* ws, double* t, int64_t* step);
/* zeeman_at(z, t) evaluated by the host for TimeDependentZeeman (src/zeeman.jl:20-21). */
sbec_status sbec_set_zeeman(sbec_ws* ws, double p, double q);
/* TimeDependentZeeman (src/types.jl:172-178) for every entry point that steps: fn(user, t, &p, &q)
 * is called with the state time before each half potential, as _half_potential_step! evaluates
 * zeeman_at(ws.zeeman, ws.state.t) (src/split_step.jl:49); the leapfrog's merged V(dt) uses the
 * time at the start of its step, as in src/simulation.jl:66-72.  fn = NULL restores the static
 * (p, q) of sbec_set_zeeman.  While a function is set, steps launch eagerly (the Zeeman factors
 * change from step to step).  fn runs on the calling thread and must not call into this workspace. */
typedef void (*sbec_zeeman_fn)(void* user, double t, double* p, double* q);
sbec_status sbec_set_zeeman_fn(sbec_ws* ws, sbec_zeeman_fn fn, void* user);
/* Replaces the potential values (evaluate_potential, src/potentials.jl:1-32). */
sbec_status sbec_set_potential(sbec_ws* ws, const double* V);
/* _rebuild_workspace_with_dt (src/ground_state.jl:380-392): new dt for split_step!. */
sbec_status sbec_set_dt(sbec_ws* ws, double dt);
/* Query: whether the tensor path is active and the channel couplings g_S it uses. */
sbec_status sbec_tensor_channels(sbec_ws* ws, int32_t* active, int32_t* n_channels, int32_t* S, double* gS);

/* ---- operators ---------------------------------------------------------- */
/* _half_potential_step!(ws, dt_half, ...) (src/split_step.jl:48-133). */
sbec_status sbec_half_potential(sbec_ws* ws, double dt_half, int32_t imaginary_time);
/* apply_kinetic_step_batched! with the phase for `dt` (src/propagators.jl:130-145);
 * imaginary_time selects exp(-k^2 dt/2) instead of cis(-k^2 dt/2). */
sbec_status sbec_kinetic(sbec_ws* ws, double dt, int32_t imaginary_time);
/* _normalize_psi! (src/split_step.jl:185-195). */
sbec_status sbec_normalize(sbec_ws* ws);
/* _normalize_psi_constrained! (src/ground_state.jl:279-320). */
sbec_status sbec_normalize_constrained(sbec_ws* ws, double target_Mz);

/* ---- integrators -------------------------------------------------------- */
/* split_step!(ws) repeated n times (src/split_step.jl:10-35). */
sbec_status sbec_split_step(sbec_ws* ws, int64_t n);
/* _strang_core! / _yoshida_core! (src/split_step.jl:146-183). */
sbec_status sbec_strang_core(sbec_ws* ws, double dt);
sbec_status sbec_yoshida_core(sbec_ws* ws, double dt);

/* ---- drivers ------------------------------------------------------------ */
/* run_simulation!(ws; callback) (src/simulation.jl:1-94): leapfrog-fused real time or the
 * standard ITP loop; the callback receives each save point (initial state included). */
sbec_status sbec_run_simulation(sbec_ws* ws, int64_t n_steps, int64_t save_every,
                                sbec_callback cb, void* user);
/* run_simulation_adaptive! (src/adaptive.jl:57-296). */
sbec_status sbec_run_adaptive(sbec_ws* ws, const sbec_adaptive_params* p, double t_end,
                              double save_interval, sbec_callback cb, void* user,
                              sbec_adaptive_result* out);
/* run_simulation_yoshida! (src/yoshida.jl:11-98); max_accepted <= 0 means no cap. */
sbec_status sbec_run_yoshida(sbec_ws* ws, const sbec_adaptive_params* p, double t_end,
                             double save_interval, int64_t max_accepted, sbec_callback cb,
                             void* user, sbec_adaptive_result* out);
/* The ITP loop of find_ground_state on an existing ITP workspace (src/ground_state.jl:116-169):
 * convergence checked every check_every steps; target_Mz = NaN disables the constraint.
 * Convergence (here, in sbec_ground_state_adaptive and in batches) is the reference's
 * dE < tol && dpsi < tol, evaluated in FP64; in the FP32-bulk form the tests use
 * dE < max(tol, 2^-22 |E|) and dpsi < max(tol, 2^-21), the resolution of an FP32 wavefunction
 * and of its energy, since smaller changes are rounding noise that never settles. */
sbec_status sbec_ground_state(sbec_ws* ws, int64_t n_steps, double tol, int64_t check_every,
                              double target_Mz, sbec_gs_result* out);
/* _find_ground_state_adaptive (src/ground_state.jl:172-237) on an existing ITP workspace with
 * normalize_every = 1: blocks of max(1, n_steps/100) steps; a block whose energy rose (or is NaN)
 * is undone and dt halves (floor 1e-8), otherwise dt grows by 10 % up to dt_max.  The NaN /
 * DDI-overflow guard runs after the first step (SBEC_ERR_NUMERIC).  *final_dt receives the dt
 * the workspace ends with (may be NULL). */
sbec_status sbec_ground_state_adaptive(sbec_ws* ws, int64_t n_steps, double tol, double dt_max,
                                       sbec_gs_result* out, double* final_dt);

/* ---- reductions --------------------------------------------------------- */
/* total_energy (src/energy.jl:6-54) and its terms. */
sbec_status sbec_total_energy(sbec_ws* ws, double* E);
sbec_status sbec_energy_breakdown(sbec_ws* ws, sbec_energy_terms* out);
/* total_norm, magnetization (src/observables.jl:13-31). */
/* estimate_splitting_error (src/diagnostics.jl:214-251): max|psi_dt - psi_{2 x dt/2}| / max|psi|
 * from the current state, which is restored. */
sbec_status sbec_estimate_splitting_error(sbec_ws* ws, double* err);
/* validate_conservation's drifts (src/diagnostics.jl:259-293) over n_steps split steps: |dN|/N,
 * |dE|/|E|, |dMz|/max(|Mz|, 1e-10); the state is restored. */
sbec_status sbec_conservation_drift(sbec_ws* ws, int64_t n_steps, double* norm_drift, double* energy_drift,
                                    double* mag_drift);
sbec_status sbec_total_norm(sbec_ws* ws, double* norm);
sbec_status sbec_magnetization(sbec_ws* ws, double* Mz);
/* Spin density (Fx, Fy, Fz) on the grid (src/observables.jl:61-86); 3*n_total doubles. */
sbec_status sbec_spin_density(sbec_ws* ws, double* out);
/* Dipolar potential (Φx, Φy, Φz) on the grid for the current psi (src/ddi.jl:108-163,
 * src/ddi_padded.jl:55-85); padded selects the zero-padded convolution. */
sbec_status sbec_ddi_potential(sbec_ws* ws, int32_t padded, double* out);

/* classify_phase (src/diagnostics.jl:166-206) on the device-resident psi: FP64 grid sums of
 * n, n^2, |<F>|^2, m|psi_m|^2 and the pair-amplitude channel weights sum_M int |A_SM|^2 dV
 * (pair_amplitude_spectrum, src/observables.jl:227-246), then the reference's labelling. */
typedef enum sbec_phase_label {
  SBEC_PHASE_VACUUM = 0,
  SBEC_PHASE_FERROMAGNETIC = 1,
  SBEC_PHASE_POLAR = 2,
  SBEC_PHASE_NEMATIC = 3,
  SBEC_PHASE_CYCLIC = 4,
  SBEC_PHASE_MIXED = 5
} sbec_phase_label;
typedef struct sbec_phase_info {
  double spin_order;             /* int |<F>|^2 / (F^2 int n^2) */
  double nematic_order;          /* W_0 / (int n^2 / (2F+1)) */
  double magnetization_density;  /* Mz / N */
  int32_t phase;                 /* sbec_phase_label */
  int32_t n_channels;            /* F + 1: S = 0, 2, ..., 2F */
  double channel_weights[SBEC_MAX_CHANNELS];  /* W_S / sum W, index S/2 */
  double raw_channel_weights[SBEC_MAX_CHANNELS];  /* W_S = sum_M int |A_SM|^2 dV */
} sbec_phase_info;
sbec_status sbec_classify_phase(sbec_ws* ws, sbec_phase_info* out);

/* ---- batches of independent ground-state solves ---------------------------
 * The multistart / continuation / phase-boundary callers of find_ground_state
 * (src/ground_state.jl:239-378, src/phase_boundary.jl:9) run many independent ITP
 * solves; a batch steps all solves that share grid, F, V, dt and Zeeman in the same
 * kernels (per-solve c0, c1 and psi), each with the find_ground_state convergence
 * test of src/ground_state.jl:138-159.  cfg: imaginary_time=1, normalize_every=1,
 * contact couplings: per-solve c0/c1 (cfg->c0/c1 are ignored), a shared c_lhy and a shared
 * nematic c2 (cfg->c_extra[0], src/nematic.jl:34-51); no DDI, Raman, losses or couplings
 * that switch on the tensor step.
 * psi: n_solves consecutive host psi buffers (reference layout). */
typedef struct sbec_batch sbec_batch;
sbec_status sbec_batch_create(const sbec_config* cfg, int32_t n_solves, const double* c0, const double* c1,
                              const double* psi, const double* V, sbec_batch** out);
/* A batch of solves on different grids (cfg->ndim axes each): solve i has n[3i..3i+2] points and
 * box L[3i..3i+2], couplings c0[i], c1[i], host psi[i] (reference layout of its grid) and potential
 * V[i] (n points, or V = NULL for none).  Solves are grouped by grid inside the batch; solves of one
 * grid must pass the same potential values.  The groups advance concurrently (own stream each) in
 * sbec_batch_ground_state; every other batch call addresses solves by their index i. */
sbec_status sbec_batch_create_grids(const sbec_config* cfg, int32_t n_solves, const int32_t* n, const double* L,
                                    const double* c0, const double* c1, const double* const* psi,
                                    const double* const* V, sbec_batch** out);
/* *supported = 1 when sbec_batch_create would take cfg (contact couplings, the nematic c2
 * included, without DDI, Raman, losses or the tensor step; grids that take the fused passes:
 * power-of-two axes, D in {1, 3, 5} and a row pass that fits the first axis), else 0.  Needs
 * no device. */
sbec_status sbec_batch_supported(const sbec_config* cfg, int32_t* supported);
/* The same with a spin F per solve (F[i]; cfg->F is ignored): solves are grouped by grid and F,
 * and psi[i] holds 2F[i]+1 components.  No counterpart in the reference, whose callers loop
 * over the solves one at a time. */
sbec_status sbec_batch_create_mixed(const sbec_config* cfg, int32_t n_solves, const int32_t* F, const int32_t* n,
                                    const double* L, const double* c0, const double* c1,
                                    const double* const* psi, const double* const* V, sbec_batch** out);
sbec_status sbec_batch_destroy(sbec_batch* b);
sbec_status sbec_batch_ground_state(sbec_batch* b, int64_t n_steps, double tol, int64_t check_every,
                                    sbec_gs_result* out);
/* The same with a step limit and check interval per solve (n_steps[i], check_every[i]): solve i
 * follows find_ground_state(n_steps = n_steps[i]) with its convergence test every check_every[i]
 * steps; the batch advances in blocks up to the next step where some solve checks or stops. */
sbec_status sbec_batch_ground_state_each(sbec_batch* b, const int64_t* n_steps, double tol,
                                         const int64_t* check_every, sbec_gs_result* out);
/* As sbec_set_graph_mode, for every group of the batch. */
sbec_status sbec_batch_set_graph_mode(sbec_batch* b, int32_t graphs);
sbec_status sbec_batch_get_psi(sbec_batch* b, int32_t solve, double* psi);
sbec_status sbec_batch_energies(sbec_batch* b, double* E);
/* classify_phase of one solve of the batch (as sbec_classify_phase). */
sbec_status sbec_batch_classify_phase(sbec_batch* b, int32_t solve, sbec_phase_info* out);

/* ---- tracing (the reference's @timeit_debug substep timers, src/split_step.jl:15-131) ---- */
typedef struct sbec_kernel_stat {
  char name[32];             /* kernel category: fft_x, fft_last_kinetic, potential, tensor, ddi_*, reduce, ... */
  int64_t launches;          /* timed launches since profiling was enabled */
  double ms;                 /* summed CUDA-event durations on the workspace stream */
  double bytes;              /* summed algorithmic bytes (one read + one write of each array touched) */
} sbec_kernel_stat;
/* Enable (1) or disable (0) per-launch CUDA-event timing; either call resets the statistics. */
sbec_status sbec_profile_enable(sbec_ws* ws, int32_t enable);
/* Copy up to max statistics into out; *n receives the number of categories. */
sbec_status sbec_profile_read(sbec_ws* ws, sbec_kernel_stat* out, int32_t max, int32_t* n);
/* Number of kernels this workspace has launched since creation. */
sbec_status sbec_launch_count(sbec_ws* ws, int64_t* n);
/* The workspace's CUDA stream (cudaStream_t), for callers that order or time work on it. */
sbec_status sbec_ws_stream(sbec_ws* ws, void** stream);
/* Save-point delivery of sbec_run_simulation: 0 (default) synchronous; 1 pipelined — each
 * snapshot is copied to a pinned slot in stream order and handed to the callback while the
 * device already runs the next segment (leapfrog path).  Only for callbacks that read the
 * snapshot and do not call back into this workspace; a stop request still leaves psi, t and
 * step at the save point.  No counterpart in the reference. */
sbec_status sbec_set_snapshot_mode(sbec_ws* ws, int32_t pipelined);
/* graphs = 1 (default): repeated step blocks are captured once as CUDA graphs and replayed;
 * 0: every kernel is launched eagerly.  Same kernels, same results.  Eager suits workspaces
 * that live for one short solve among many running concurrently (each would capture and
 * instantiate its own graphs).  No counterpart in the reference. */
sbec_status sbec_set_graph_mode(sbec_ws* ws, int32_t graphs);
/* Autotuner decisions of a workspace / batch (FFT line-kernel variant per call shape, with
 * the measured time of every variant), as text; *len receives the full length.  No
 * counterpart in the reference (FFTW plans are chosen inside FFTW). */
sbec_status sbec_tuning_report(sbec_ws* ws, char* buf, int64_t cap, int64_t* len);
sbec_status sbec_batch_tuning_report(sbec_batch* b, char* buf, int64_t cap, int64_t* len);
/* The autotuner's process-wide decisions as text, one "shape<TAB>variant" line each; *len
 * receives the full length.  No counterpart in the reference. */
sbec_status sbec_tune_table_export(char* buf, int64_t cap, int64_t* len);
/* Loads decisions in the export format.  A shape found in the table is never timed again, so
 * processes that load the same table run the same line kernels and give bit-identical FP32
 * results; without it, the variant of a shape is the fastest in a timing of this process, and
 * FP32 results may differ between processes at the level of FP32 rounding.  Entries whose
 * variant is not compiled for a shape are ignored there.  No counterpart in the reference. */
sbec_status sbec_tune_table_import(const char* text);
/* frozen = 1: a shape missing from the table is no longer timed; it takes its default variant
 * (recorded in the table), so results cannot depend on a timing race.  0 (default): timed on
 * first contact.  No counterpart in the reference. */
sbec_status sbec_tune_freeze(int32_t frozen);

/* Measured FMA throughput of the current device in TFLOP/s (2 flops per FMA), FP32
 * (precision = SBEC_FP32_BULK) or FP64 (SBEC_FP64): eight register-resident FMA chains per
 * thread, 2048 threads per SM, best of three CUDA-event timings.  The denominators of the
 * compute rooflines; no counterpart in the reference. */
sbec_status sbec_measure_fma_peak(int32_t precision, double* tflops);

/* ---- allocation-free reduction --------------------------------------------
 * No counterpart in the reference: an extra entry point for callers that cannot
 * allocate GPU memory at the time of the call -- code running while a stream is
 * captured into a CUDA graph, or hosts whose device memory belongs to another
 * allocator (e.g. a Julia CUDA.jl pool) that must not see cudaMalloc/cudaFree.
 * Computes sums_dev[c] = sum_x |psi_c(x)|^2 for c < n_components and writes the
 * number of NaN entries to sums_dev[n_components], for a device wavefunction in
 * the reference layout (interleaved complex FP64, planar per component).  The
 * norm and <Fz> of total_norm / magnetization follow as dV*sum_c sums_dev[c] and
 * dV*sum_c (F-c)*sums_dev[c].  psi_dev and sums_dev are device pointers owned by
 * the caller; the work is queued on `stream` (a cudaStream_t, NULL = default).
 * Scratch lives in a fixed device array (256 KiB per device, kept until exit), so
 * the call performs no allocation.  The first call on a device resolves that
 * array's address (no allocation, but make it before any stream capture).  All
 * calls on a device share the array: calls whose kernels overlap on the GPU race.
 * Limits: 1 <= n_components <= SBEC_NOALLOC_MAX_COMPONENTS,
 * 1 <= n_points <= SBEC_NOALLOC_MAX_POINTS, psi_dev 16-byte aligned (whole complex
 * entries) and sums_dev 8-byte aligned; otherwise SBEC_ERR_INVALID. */
#define SBEC_NOALLOC_MAX_COMPONENTS 16
#define SBEC_NOALLOC_MAX_POINTS (1LL << 31)
sbec_status sbec_component_norms_noalloc(const double* psi_dev, int64_t n_points, int32_t n_components,
                                         double* sums_dev, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* SBEC_H */
