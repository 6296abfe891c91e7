#!/usr/bin/env python
"""Benchmark of the split-step hot path on the 2-D spin-1 real-time workload.

Workload (one bench step): a 256x256 spin-1 (3 components) real-time Strang
run, box 30x30, c0=10, c1=0.5, harmonic trap omega=(1,1), q=0.1, p=0,
dt=1e-3, 5000 leapfrog-fused steps, starting from the polar ground state plus
seeded complex noise of amplitude 1e-3 on m=+-1.

* value: pts*comps*steps/s of the chosen form (FP32 bulk, FP64 reductions)
  with psi resident on the device, no host traffic, L2 flushed between runs.
* e2e: the same run through the C ABI as a caller makes it: psi copied in from
  host memory, 100 save points (energy, norm, magnetisation and a host copy of
  psi each, as run_simulation! records them), final psi copied out.
* plain_fp64: the plain complex-FP64 form on the same workload.
* roofline: the dominant kernel's algorithmic bytes per launch over its mean
  CUDA-event duration (profiled pass on the engine stream), against the measured
  HBM copy bandwidth.
* cpu_baseline: the CPU FP64 restatement (numpy + scipy.fft, all host threads)
  on a bounded sample of the same run.

--impl reference times that CPU restatement alone (the reference itself is
Julia and cannot run on these hosts).
"""

from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
for _p in (str(ROOT), str(ROOT / "bec-simulation_gb300")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

N_GRID = (256, 256)
BOX = (30.0, 30.0)
F = 1
C0, C1 = 10.0, 0.5
OMEGA = (1.0, 1.0)
ZP, ZQ = 0.0, 0.1
DT = 1e-3
RUN_STEPS = 5000
SAVE_EVERY = 50
METRIC = "split-step pts·comps/s"
UNIT = "pts·comps·steps/s"
WORKLOAD = "2D spin-1 256x256 real-time Strang (leapfrog), 5000 steps, dt=1e-3, save_every=50"


def units_per_run(steps: int) -> float:
    return float(N_GRID[0] * N_GRID[1] * (2 * F + 1) * steps)


def noisy_polar(psi_gs: np.ndarray, dV: float) -> np.ndarray:
    rng = np.random.Generator(np.random.PCG64(20261203))
    psi = np.array(psi_gs, dtype=np.complex128, order="F", copy=True)
    for c in (0, 2):  # m = +1, -1
        noise = (rng.standard_normal(N_GRID) + 1j * rng.standard_normal(N_GRID)) / math.sqrt(2.0)
        psi[..., c] += 1e-3 * noise
    psi /= math.sqrt(float(np.sum(np.abs(psi) ** 2)) * dV)
    return psi


# ----------------------------------------------------------------------------- clocks
class ClockSampler:
    """nvidia-smi sampling of SM clocks and throttle reasons during the timed region."""

    def __init__(self):
        self.samples = []
        self._stop = threading.Event()
        self._th = None

    def start(self):
        self._th = threading.Thread(target=self._run, daemon=True)
        self._th.start()

    def _run(self):
        q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        while not self._stop.is_set():
            try:
                out = subprocess.run(["nvidia-smi", f"--query-gpu={q}", "--format=csv,noheader,nounits", "-i",
                                      os.environ.get("LOCAL_RANK", "0")], capture_output=True, text=True,
                                     timeout=5).stdout.strip().splitlines()
                if out:
                    self.samples.append([v.strip() for v in out[0].split(",")])
            except Exception:
                pass
            self._stop.wait(0.2)

    def stop(self) -> dict:
        self._stop.set()
        if self._th:
            self._th.join(timeout=5)
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        smax = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in self.samples for i in range(4) if "Active" in s[3 + i]
                          and not s[3 + i].startswith("Not")})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": reasons, "samples": len(self.samples)}


# ----------------------------------------------------------------------------- dist
def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class Dist:
    def __init__(self):
        self.world, self.rank, self.local = dist_env()
        self.pg = None
        if self.world > 1:
            import torch.distributed as td

            backend = "nccl" if self._cuda() else "gloo"
            td.init_process_group(backend=backend)
            self.td = td

    @staticmethod
    def _cuda():
        try:
            import torch

            return torch.cuda.is_available()
        except Exception:
            return False

    def barrier(self):
        if self.world > 1:
            self.td.barrier()

    def max(self, x: float) -> float:
        if self.world == 1:
            return x
        import torch

        dev = torch.device("cuda", self.local) if self._cuda() else torch.device("cpu")
        t = torch.tensor([x], dtype=torch.float64, device=dev)
        self.td.all_reduce(t, op=self.td.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.world > 1:
            self.td.destroy_process_group()


# ----------------------------------------------------------------------------- CPU arm
def cpu_leapfrog_sample(n_steps: int, threads: int) -> tuple:
    """Time n_steps leapfrog-fused real-time steps of the CPU restatement (oracle)."""
    import oracle as O

    O.set_fft_workers(threads)
    g = O.make_grid(O.GridConfig(N_GRID, BOX))
    psi0 = noisy_polar(O.init_psi(g, F, "polar"), O.cell_volume(g))
    ws = O.make_workspace(grid=g, atom=O.Na23, interactions=O.InteractionParams(C0, C1),
                          zeeman=O.ZeemanParams(ZP, ZQ), V=O.harmonic_potential(g, OMEGA),
                          sim_params=O.SimParams(DT, n_steps, False, None, n_steps + 1), psi_init=psi0)
    t0 = time.perf_counter()
    O.run_simulation(ws, keep_psi=False)
    return time.perf_counter() - t0, units_per_run(n_steps)


def cpu_calibrated(target_s: float, threads: int) -> dict:
    dt1, _ = cpu_leapfrog_sample(5, threads)
    n = max(5, min(5000, int(target_s / max(dt1 / 5, 1e-6))))
    secs, units = cpu_leapfrog_sample(n, threads)
    return {"value": units / secs, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{n} of the {RUN_STEPS} leapfrog steps of the workload ({secs:.1f} s), CPU FP64 "
                      "restatement (numpy + scipy.fft), not the reference Julia (not runnable on this host)"}


def run_reference(args) -> None:
    world, rank, _ = dist_env()
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    import oracle as O

    O.set_fft_workers(threads)
    dt1, _ = cpu_leapfrog_sample(3, threads)
    per_step = dt1 / 3
    n = max(3, min(RUN_STEPS, int(6.0 / max(per_step, 1e-6))))
    for _ in range(args.warmup):
        cpu_leapfrog_sample(max(1, n // 10), threads)
    tot_s = 0.0
    tot_u = 0.0
    for _ in range(args.steps):
        s, u = cpu_leapfrog_sample(n, threads)
        tot_s += s
        tot_u += u
    value = tot_u / tot_s
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * tot_s / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "fp64", "data": "synthetic",
        "config": {"workload": WORKLOAD, "sample_steps_per_bench_step": n, "cpu_threads": threads},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": f"{n} leapfrog steps per bench step; CPU FP64 restatement of the reference "
                                   "(numpy + scipy.fft); the Julia reference cannot run on this host"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# ----------------------------------------------------------------------------- batched ground states
def batched_workload(S, n_solves: int = 512, seed: int = 4242):
    """The 512-solve batch: c1 on 64 values in [-1, 1] x 8 starts (polar, ferromagnetic,
    uniform, antiferromagnetic, 4 seeded random), grid 64^2 / 128^2 / 256^2 drawn per solve."""
    rng = np.random.Generator(np.random.PCG64(seed))
    c1s = np.linspace(-1.0, 1.0, 64)
    starts = ["polar", "ferromagnetic", "uniform", "antiferromagnetic", "random", "random", "random", "random"]
    sizes = rng.choice([64, 128, 256], size=n_solves)
    jobs = []
    for i in range(n_solves):
        c1 = float(c1s[i // 8 % 64])
        st = starts[i % 8]
        jobs.append(dict(idx=i, n=int(sizes[i]), c1=c1, state=st, seed=1000 + i))
    return jobs


def run_batched(S, jobs, precision: str, n_steps: int, tol: float) -> tuple:
    """Runs every job through GroundStateBatch grouped by grid size; returns (seconds, results by idx)."""
    import time as _t
    res = {}
    tune = {}
    total = 0.0
    for n in sorted({j["n"] for j in jobs}):
        group = [j for j in jobs if j["n"] == n]
        g = S.make_grid(S.GridConfig((n, n), (20.0, 20.0)))
        psis = [S.init_psi(g, 1, j["state"], seed=j["seed"]) for j in group]
        b = S.GroundStateBatch(grid=g, atom=S.Rb87, c0s=[10.0] * len(group), c1s=[j["c1"] for j in group],
                               psi_inits=psis, potential=S.HarmonicTrap(1.0, 1.0), dt=0.005, precision=precision)
        t0 = _t.perf_counter()
        r = b.ground_state(n_steps, tol, max(1, n_steps // 10))
        total += _t.perf_counter() - t0
        log(f"batched {precision} {len(group)} x {n}^2: {_t.perf_counter() - t0:.2f} s")
        tune[n] = b.tuning_report.splitlines()
        b.close()
        for j, x in zip(group, r):
            res[j["idx"]] = x
    res["autotune"] = tune
    return total, res


def batched_row_roofline(tune: dict) -> dict:
    """HBM roofline of the batched ITP row pass of the largest grid group, from the autotuner's
    own CUDA-event timing of the variant it chose (median of three launches on the live batch).
    Algorithmic bytes: read + write of every active solve's psi (3 x n^2 complex FP32) plus V
    once (all solves share it)."""
    import re
    n = max(tune)
    for line in tune[n]:
        m = re.match(r"fp32 row flags=\S+ batched D=(\d+) grid=\S+ solves=(\d+) -> (.*) chosen v(\d+)", line)
        if not m:
            continue
        D, solves, times, chosen = int(m.group(1)), int(m.group(2)), m.group(3), m.group(4)
        us = float(re.search(rf"v{chosen}=([0-9.]+)us", times).group(1))
        N = n * n
        nbytes = solves * 2.0 * D * N * 8 + N * 4
        peaks = measured_peaks()
        hbm = float(peaks.get("hbm_gbs", 6800.0))
        achieved = nbytes / (us * 1e-6) / 1e9
        return {"kernel": f"row_pass (batched ITP, {solves} x {n}^2 spin-1, variant {chosen})", "bound": "hbm",
                "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm, "us_per_launch": us,
                "bytes_per_launch": nbytes,
                "peak_source": "MEASURED_PEAKS.json hbm_gbs (of measured)" if "hbm_gbs" in peaks else "fallback",
                "timing": "autotuner CUDA events, median of three launches of the chosen variant"}
    return None


def bench_batched(S, sample: int = 6, n_steps: int = 10000, tol: float = 1e-8) -> dict:
    jobs = batched_workload(S)
    secs32, r32 = run_batched(S, jobs, "fp32", n_steps, tol)
    # plain FP64 form, one solve at a time (find_ground_state per solve), on a seeded sample
    rng = np.random.Generator(np.random.PCG64(7))
    pick = [int(i) for i in rng.choice(len(jobs), size=sample, replace=False)]
    secs64 = 0.0
    errs = []
    by_size = {}
    for i in pick:
        j = jobs[i]
        g = S.make_grid(S.GridConfig((j["n"], j["n"]), (20.0, 20.0)))
        psi0 = S.init_psi(g, 1, j["state"], seed=j["seed"])
        t0 = time.perf_counter()
        r = S.find_ground_state(grid=g, atom=S.Rb87, interactions=S.InteractionParams(10.0, j["c1"]),
                                potential=S.HarmonicTrap(1.0, 1.0), dt=0.005, n_steps=n_steps, tol=tol,
                                psi_init=psi0, precision="fp64")
        dt = time.perf_counter() - t0
        r["workspace"].close()
        secs64 += dt
        by_size.setdefault(j["n"], []).append(dt)
        errs.append(abs(r32[i]["energy"] - r["energy"]) / abs(r["energy"]))
    # one-at-a-time FP64 time for all 512 solves, from the per-size mean of the sample
    mean = {n: float(np.mean(v)) for n, v in by_size.items()}
    overall = float(np.mean([x for v in by_size.values() for x in v]))
    est64 = sum(mean.get(j["n"], overall) for j in jobs)
    tune = r32.pop("autotune")
    conv = sum(1 for x in r32.values() if x["converged"])
    return {"workload": "512 ITP solves, 2D spin-1, c1 in 64 values of [-1,1] x 8 starts, grids 64^2/128^2/256^2, "
                        "dt=0.005, tol=1e-8, check every 1000 of 10000 steps",
            "fp32_batched_solves_per_s": len(jobs) / secs32, "fp32_batched_seconds": secs32,
            "fp64_one_at_a_time_solves_per_s": len(jobs) / est64,
            "fp64_sample": f"{sample} solves timed one at a time ({secs64:.2f} s), extrapolated per grid size",
            "speedup_vs_fp64_one_at_a_time": est64 / secs32,
            "energy_rel_err_fp32_vs_fp64_max": max(errs), "converged": conv,
            "row_pass_roofline": batched_row_roofline(tune), "autotune": tune}


_T0 = time.perf_counter()


def log(msg: str) -> None:
    """Progress line on stderr (the JSON result stays alone on stdout)."""
    print(f"[bench {time.perf_counter() - _T0:8.1f}s] {msg}", file=sys.stderr, flush=True)


# ----------------------------------------------------------------------------- 1-D quickstart
def bench_quickstart(S, reps: int = 3) -> dict:
    """The reference's own CPU-runnable case: 1-D spin-1 Rb87 ground state, 64 points, box 20,
    c0=10, c1=-0.5, trap 1, dt=0.005, up to 5000 steps, tol 1e-10, polar start; solves/s of the
    plain FP64 and FP32-bulk forms on the GPU and of the CPU restatement (one solve)."""
    import oracle as O

    out = {"workload": "1D spin-1 64-pt ITP ground state (quickstart), tol 1e-10, up to 5000 steps"}
    g = S.make_grid(S.GridConfig((64,), (20.0,)))
    for prec in ("fp64", "fp32"):
        kw = dict(grid=g, atom=S.Rb87, interactions=S.InteractionParams(10.0, -0.5), potential=S.HarmonicTrap(1.0),
                  dt=0.005, n_steps=5000, tol=1e-10, initial_state="polar", precision=prec)
        S.find_ground_state(**kw)["workspace"].close()
        t0 = time.perf_counter()
        for _ in range(reps):
            r = S.find_ground_state(**kw)
            r["workspace"].close()
        secs = (time.perf_counter() - t0) / reps
        out[prec] = {"solves_per_s": 1.0 / secs, "seconds": secs, "steps": r["steps"], "energy": r["energy"],
                     "converged": r["converged"]}
    og = O.make_grid(O.GridConfig((64,), (20.0,)))
    t0 = time.perf_counter()
    ro = O.find_ground_state(grid=og, atom=O.Rb87, interactions=O.InteractionParams(10.0, -0.5),
                             V=O.harmonic_potential(og, (1.0,)), dt=0.005, n_steps=5000, tol=1e-10)
    secs = time.perf_counter() - t0
    out["cpu_port"] = {"solves_per_s": 1.0 / secs, "seconds": secs, "steps": ro["steps"], "energy": ro["energy"],
                       "kind": "port"}
    out["fp64_energy_rel_err_vs_oracle"] = abs(out["fp64"]["energy"] - ro["energy"]) / abs(ro["energy"])
    out["fp32_energy_rel_err_vs_oracle"] = abs(out["fp32"]["energy"] - ro["energy"]) / abs(ro["energy"])
    return out


# ----------------------------------------------------------------------------- serving
def bench_serving(S, n_requests: int, fp64_probe_steps: int = 20, check_budget_s: float = 45.0) -> dict:
    """Poisson request stream (seeded, mean 200 req/s) served with continuous batching in the
    FP32-bulk form under a 150 GB HBM budget, after the autotuner's decisions are fixed for
    every call shape of the stream.  The plain FP64 form one request at a time is estimated
    per request from a timed probe of the same grid (per-step time x the steps the served solve
    took, plus its measured setup).  Served energies are checked against the FP64 form by
    rerunning requests in FP64, cheapest first, within a time budget."""
    from spinorbec import serve

    reqs = serve.poisson_requests(n_requests, rate=200.0, seed=5)
    window = 0.25
    policy = "sjf"  # shortest estimated work first among the units waiting for admission
    n_shapes = serve.pretune(reqs, merge_window_s=window)
    log(f"serving: autotuner fixed for {n_shapes} shapes")
    srv = serve.Server(hbm_budget_bytes=150e9, max_slots=32, runner=_logged(serve.run_request),
                       merge_window_s=window, policy=policy)
    try:
        out = srv.run(reqs, realtime=True)
    finally:
        S.tune_freeze(False)
    log(f"serving: {len(reqs)} requests in {out['wall_s']:.1f} s ({srv.merged_requests} in {srv.merged_units} "
        "merged batches)")
    est64 = 0.0
    probes = {}
    cost = {}
    for r, res in zip(reqs, out["results"]):
        key = (r.n_points, r.F, r.enable_ddi, r.kind)
        if key not in probes:
            probes[key] = fp64_probe(S, r, fp64_probe_steps)
        setup, per_step = probes[key]
        cost[r.rid] = setup + per_step * res.steps
        est64 += cost[r.rid]
    # accuracy of served energies against the plain FP64 form (same request, same steps / tol).
    # Ground states: the 1e-6 energy bar.  Real-time runs: the FP32 - FP64 difference of the final
    # energy, split by whether the FP64 run itself conserves energy to the 1e-6 bar over the run
    # (where it does not, the time discretisation moves the energy by more than the bar and the
    # two roundings of the dynamics part ways), with each form's own energy drift beside it.
    t0 = time.perf_counter()
    errs, dyn_ok, dyn_bad, drift32, drift64 = [], [], [], [], []
    for r in sorted(reqs, key=lambda q: cost[q.rid]):
        if time.perf_counter() - t0 + cost[r.rid] > check_budget_s:
            break
        o64 = serve.run_request(serve.SolveRequest(**{**r.__dict__, "precision": "fp64"}))
        e32 = out["results"][r.rid].energy
        rel = abs(e32 - o64["energy"]) / abs(o64["energy"])
        if r.kind == "ground_state":
            errs.append(rel)
        else:
            drift = abs(o64["energy"] - o64["energy0"]) / abs(o64["energy0"])
            drift64.append(drift)
            drift32.append(abs(e32 - o64["energy0"]) / abs(o64["energy0"]))
            (dyn_ok if drift < 1e-6 else dyn_bad).append(rel)
    lat = sorted(x.latency for x in out["results"])
    return {"workload": f"{n_requests} requests of the seeded Poisson stream (mean 200 req/s): 1-D 256..4096, "
                        "2-D 64^2..512^2, 3-D 32^3..128^3, F in {1,2,6}, DDI for F=6, 500-5000 steps, "
                        "half ground states (tol 1e-8) half real-time runs",
            "hbm_budget_gb": 150, "max_slots": 32, "peak_concurrent": srv.peak_active,
            "admission": f"{policy}: by HBM footprint and slots, waiting units in order of estimated work "
                         "(points x components x steps, x4 with DDI)",
            "merging": {"window_s": window, "merged_units": srv.merged_units,
                        "merged_requests": srv.merged_requests,
                        "rule": "ground states of one grid/F/dt/tol/trap (contact couplings) arriving in the same "
                                "window run as one GroundStateBatch, per-solve step limits"},
            "peak_admitted_gb": srv.peak_used / 1e9, "tuned_shapes_before_serving": n_shapes,
            "fp32_served_solves_per_s": out["solves_per_s"], "wall_s": out["wall_s"],
            "p50_latency_s": out["p50_latency_s"], "p99_latency_s": out["p99_latency_s"],
            "max_latency_s": lat[-1] if lat else None,
            "fp64_one_at_a_time_solves_per_s": len(reqs) / est64,
            "fp64_estimate": f"per grid/F/kind: setup + {fp64_probe_steps}-step timed probe x steps of the served solve",
            "speedup_vs_fp64_one_at_a_time": est64 / out["wall_s"],
            "accuracy_vs_fp64": {
                "selection": f"cheapest FP64 reruns first within {check_budget_s:.0f} s",
                "ground_states": {"checked": len(errs), "of": sum(1 for r in reqs if r.kind == "ground_state"),
                                  "max_energy_rel_err": max(errs) if errs else None,
                                  "above_1e-6": sum(1 for e in errs if e > 1e-6)},
                "dynamics_fp64_conserves_to_1e-6": {"checked": len(dyn_ok),
                                                    "max_energy_rel_err": max(dyn_ok) if dyn_ok else None,
                                                    "above_1e-6": sum(1 for e in dyn_ok if e > 1e-6)},
                "dynamics_fp64_drift_above_1e-6": {"checked": len(dyn_bad),
                                                   "max_energy_rel_err": max(dyn_bad) if dyn_bad else None},
                "dynamics_energy_drift_over_run": {
                    "fp64_median": float(np.median(drift64)) if drift64 else None,
                    "fp32_median": float(np.median(drift32)) if drift32 else None,
                    "fp64_max": max(drift64) if drift64 else None, "fp32_max": max(drift32) if drift32 else None,
                    "how": "|E(T) - E(0)| / |E(0)| of each form, E(0) of the FP64 run"}}}


def _logged(runner):
    def run(req):
        t0 = time.perf_counter()
        out = runner(req)
        log(f"  request {req.rid}: {req.kind} {req.n_points} F={req.F} ddi={req.enable_ddi} {out['steps']} steps "
            f"{time.perf_counter() - t0:.2f} s")
        return out
    return run


def fp64_probe(S, r, k: int) -> tuple:
    """(setup seconds, seconds per step) of request r's grid in the plain FP64 form."""
    from spinorbec import serve

    g = S.make_grid(S.GridConfig(r.n_points, r.box_size))
    t0 = time.perf_counter()
    ws = S.make_workspace(grid=g, atom=S.AtomSpecies("req", r.F), interactions=S.InteractionParams(r.c0, r.c1),
                          potential=S.HarmonicTrap(*([r.omega] * len(r.n_points))), zeeman=S.ZeemanParams(0.0, 0.1),
                          sim_params=S.SimParams(r.dt, k, r.kind == "ground_state", 1 if r.kind == "ground_state"
                                                 else None, k),
                          psi_init=S.init_psi(g, r.F, "polar"), enable_ddi=r.enable_ddi, c_dd=r.c_dd,
                          precision="fp64")
    S.split_step(ws, 2)
    S.total_energy(ws)
    setup = time.perf_counter() - t0
    t0 = time.perf_counter()
    S.split_step(ws, k)
    S.total_energy(ws)
    per_step = (time.perf_counter() - t0) / k
    ws.close()
    del serve
    return setup, per_step


# ----------------------------------------------------------------------------- 3D spin-6 dipolar
def bench_3d_f6(S, n: int = 128, steps32: int = 200, steps64: int = 20, fp32_peak: float = None) -> dict:
    """3D spin-6 Eu151 (c_total 4689, c1/c0 1/36, tensor c_extra (0,0,50)), zero-padded DDI
    c_dd=100, trap (1,1,1.2), polarised m=+6 with 0.01 rad seeded phase noise; adaptive
    Yoshida from dt=1e-3.  The first 200 (FP32) / 20 (FP64) accepted steps of the 2000-step
    run, measured with their rejections; the FP32 energy against the FP64 one after fixed-dt
    steps; the tensor step's time share and FLOP rate (the reference's operation count)."""
    ip = S.interaction_params_from_constraint(c_total=4689.0, c1_ratio=1 / 36, F=6, c_extra=(0.0, 0.0, 50.0))
    g = S.make_grid(S.GridConfig((n, n, n), (24.0, 24.0, 24.0)))
    rng = np.random.Generator(np.random.PCG64(11))
    psi = S.init_psi(g, 6, "ferromagnetic")
    psi = psi * np.exp(1j * 0.01 * rng.standard_normal(psi.shape))
    out = {"workload": f"3D spin-6 {n}^3, 13 components, tensor + zero-padded {2 * n}^3 DDI, adaptive Yoshida "
                       "dt0=1e-3 (sample of the 2000-step run)"}

    def make(prec):
        return S.make_workspace(grid=g, atom=S.AtomSpecies("151Eu", 6), interactions=ip,
                                potential=S.HarmonicTrap(1.0, 1.0, 1.2), sim_params=S.SimParams(1e-3, 10),
                                psi_init=psi, enable_ddi=True, c_dd=100.0, ddi_padding=True, precision=prec)

    units = n ** 3 * 13
    for prec, k in (("fp32", steps32), ("fp64", steps64)):
        ws = make(prec)
        S.run_simulation_yoshida(ws, S.AdaptiveDtParams(dt_init=1e-3), t_end=1.0, save_interval=1.0,
                                 keep_psi=False, max_accepted=1)
        ws.close()
        ws = make(prec)
        t0 = time.perf_counter()
        r = S.run_simulation_yoshida(ws, S.AdaptiveDtParams(dt_init=1e-3), t_end=100.0, save_interval=100.0,
                                     keep_psi=False, max_accepted=k)
        secs = time.perf_counter() - t0
        acc = int(r["n_accepted"])
        log(f"3d f6 {prec}: {acc} accepted, {int(r['n_rejected'])} rejected in {secs:.2f} s")
        ws.close()
        out[prec] = {"seconds": secs, "accepted_steps": acc, "rejected_steps": int(r["n_rejected"]),
                     "steps_per_s": acc / secs, "value": units * acc / secs, "unit": UNIT,
                     "accepted_per_attempt": acc / max(acc + int(r["n_rejected"]), 1)}
    out["speedup_fp32_vs_fp64"] = out["fp32"]["steps_per_s"] / out["fp64"]["steps_per_s"]
    # tensor step: per-call time from one profiled fixed-dt Yoshida step (12 tensor calls:
    # 6 half potentials, each tensor(tau/2) before and after the DDI), against the FP32 peak at
    # the reference's count of h-build work (HFEntry terms x 10 flops per point and call)
    wp = make("fp32")
    S.yoshida_core(wp, 1e-3)
    wp.profile(True)
    S.yoshida_core(wp, 1e-3)
    prof = wp.profile_read()
    wp.profile(False)
    wp.close()
    tot = sum(v["ms"] for v in prof.values())
    ten = prof.get("tensor", {"ms": 0.0, "launches": 0})
    hf_terms = 7497  # _precompute_hf_entries for F=6 with all seven channels active
    if ten["launches"]:
        per_call_s = ten["ms"] / 1e3 / ten["launches"]
        tflops = hf_terms * 10.0 * n ** 3 / per_call_s / 1e12
        out["tensor_step"] = {"calls_per_step": ten["launches"], "ms_per_call": per_call_s * 1e3,
                              "share_of_step": ten["ms"] / tot if tot else None,
                              "reference_flops_per_point_call": hf_terms * 10,
                              "achieved_tflops_reference_count": tflops, "fp32_peak_tflops_measured": fp32_peak,
                              "frac_of_fp32_peak": tflops / fp32_peak if fp32_peak else None,
                              "timing": "per-launch CUDA events, one profiled Yoshida step"}
        out["kernel_time_share"] = {k: round(v["ms"] / tot, 4) for k, v in prof.items()} if tot else None
    # accuracy: same fixed-dt Yoshida steps in both forms
    w32, w64 = make("fp32"), make("fp64")
    for _ in range(steps64):
        S.yoshida_core(w32, 1e-3)
        S.yoshida_core(w64, 1e-3)
    e32, e64 = S.total_energy(w32), S.total_energy(w64)
    n32, n64 = S.total_norm(w32), S.total_norm(w64)
    out["energy_rel_err_fp32_vs_fp64"] = abs(e32 - e64) / abs(e64)
    out["norm_rel_err_fp32_vs_fp64"] = abs(n32 - n64) / abs(n64)
    w32.close()
    w64.close()
    return out


# ----------------------------------------------------------------------------- GPU arm
def tuned_launch_us(report: list, kind: str):
    """The autotuner's burst time (us per launch) of the variant it chose for the first call
    shape of the given kind ("row" or "strided"), or None when the shape was not timed."""
    import re
    for line in report:
        if not line.startswith(("fp32 " + kind, "fp64 " + kind)) or " chosen v" not in line:
            continue
        chosen = line.rsplit(" chosen v", 1)[1].strip()
        m = re.search(rf" v{chosen}=([0-9.]+)us", line)
        if m:
            return float(m.group(1))
    return None


def measured_peaks() -> dict:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        try:
            return json.loads(p.read_text())
        except Exception:
            pass
    return {}


def main_gpu(args) -> None:
    import torch

    import __graft_entry__

    dist = Dist()
    torch.cuda.set_device(dist.local)
    __graft_entry__.build()
    import spinorbec as S

    grid = S.make_grid(S.GridConfig(N_GRID, BOX))
    dV = S.cell_volume(grid)
    atom = S.Na23
    inter = S.InteractionParams(C0, C1)
    trap = S.HarmonicTrap(*OMEGA)
    zee = S.ZeemanParams(ZP, ZQ)

    # initial state: polar ground state (FP64 ITP on the GPU, setup only) + seeded noise
    gs = S.find_ground_state(grid=grid, atom=atom, interactions=inter, zeeman=zee, potential=trap, dt=0.005,
                             n_steps=args.gs_steps, tol=1e-8, initial_state="polar")
    psi0 = noisy_polar(gs["workspace"].psi, dV)
    gs["workspace"].close()
    log("initial state ready")

    flush = torch.empty(int(256e6) // 4, dtype=torch.float32, device="cuda")

    def make(precision: str, steps: int, save_every: int):
        return S.make_workspace(grid=grid, atom=atom, interactions=inter, zeeman=zee, potential=trap,
                                sim_params=S.SimParams(DT, steps, False, None, save_every), psi_init=psi0,
                                precision=precision)

    lib = S._lib.load()
    noop = S._lib.CALLBACK(lambda user, snap: 0)  # save points are produced; the caller keeps none

    def timed_runs(ws, n_runs: int, warm: int) -> tuple:
        """Full runs with their save points: at each one the energy, norm and Mz reductions and a
        copy of psi into pinned host memory (pipelined behind the next segment)."""
        ext = torch.cuda.ExternalStream(ws.stream_ptr)
        S._lib.check(lib.sbec_set_snapshot_mode(ws.handle, 1))
        run = lambda: S._lib.check(lib.sbec_run_simulation(ws.handle, ws.sim_params.n_steps,  # noqa: E731
                                                           ws.sim_params.save_every, noop, None))
        for _ in range(warm):
            ws.set_time(0.0, 0)
            run()
        total_ms = 0.0
        l0 = ws.launch_count
        for _ in range(n_runs):
            ws.set_time(0.0, 0)
            flush.fill_(1.0)
            torch.cuda.synchronize()
            dist.barrier()
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            a.record(ext)
            run()
            b.record(ext)
            b.synchronize()
            total_ms += a.elapsed_time(b)
        launches = ws.launch_count - l0
        return total_ms, launches

    # ---- chosen form, device resident: the run as the workload names it (save every 50)
    steps = args.run_steps
    ws32 = make("fp32", steps, SAVE_EVERY)
    clocks = ClockSampler()
    clocks.start()
    ms32, launches = timed_runs(ws32, args.steps, args.warmup)
    clk = clocks.stop()
    ms32 = dist.max(ms32)
    value = dist.world * units_per_run(steps) * args.steps / (ms32 / 1e3)

    # ---- roofline of the dominant kernel.  Bytes per launch from the engine's counters (one
    # profiled run, CUDA events around every launch on the engine stream); the duration of a
    # launch from the autotuner's burst timing of the chosen variant (eight back-to-back
    # launches, median of three), which keeps the launch overlap of the step graph that
    # per-launch events take away.  The profiled (perturbed) duration is kept beside it.
    ws32.set_time(0.0, 0)
    ws32.profile(True)
    S._lib.check(lib.sbec_run_simulation(ws32.handle, steps, SAVE_EVERY, noop, None))
    prof = ws32.profile_read()
    ws32.profile(False)
    dom_name, dom = max(prof.items(), key=lambda kv: kv[1]["ms"])
    peaks = measured_peaks()
    hbm = float(peaks.get("hbm_gbs", 6800.0))
    peak_src = "MEASURED_PEAKS.json hbm_gbs (of measured)" if "hbm_gbs" in peaks else "fallback 6800 GB/s"
    per_launch_bytes = dom["bytes"] / max(dom["launches"], 1)
    profiled_s = dom["ms"] / 1e3 / max(dom["launches"], 1)
    burst_us = tuned_launch_us(ws32.tuning_report.splitlines(), "row" if dom_name == "row_pass" else "strided")
    per_launch_s = burst_us * 1e-6 if burst_us else profiled_s
    achieved = per_launch_bytes / per_launch_s / 1e9
    run_bytes = sum(v["bytes"] for v in prof.values())  # algorithmic bytes of every launch of one run
    traffic = None
    tfile = ROOT / "profiles" / "traffic_2d_256_fp32.json"
    if tfile.exists():
        try:
            traffic = json.loads(tfile.read_text()).get(dom_name)
        except Exception:
            traffic = None
    kernel_share = {k: round(v["ms"] / sum(x["ms"] for x in prof.values()), 4) for k, v in prof.items()}
    autotune = ws32.tuning_report.splitlines()
    ws32.close()

    # ---- e2e through the C ABI: host psi in, 100 save points with host copies, psi out
    ws_e = make("fp32", RUN_STEPS, SAVE_EVERY)
    host_psi = np.asfortranarray(psi0)
    e2e_ms = 0.0
    n_snap = RUN_STEPS // SAVE_EVERY
    for i in range(args.warmup + args.steps):
        flush.fill_(1.0)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        ws_e.psi = host_psi
        ws_e.set_time(0.0, 0)
        res = S.run_simulation(ws_e, keep_psi=True)
        out = ws_e.psi
        t1 = time.perf_counter()
        if i >= args.warmup:
            e2e_ms += (t1 - t0) * 1e3
    assert len(res.psi_snapshots) == n_snap + 1 and out.shape == host_psi.shape
    ws_e.close()
    e2e_ms = dist.max(e2e_ms)
    psi_bytes = host_psi.size * 16
    e2e = {"value": dist.world * units_per_run(RUN_STEPS) * args.steps / (e2e_ms / 1e3), "unit": UNIT,
           "h2d_bytes_per_step": psi_bytes, "d2h_bytes_per_step": psi_bytes * (n_snap + 2),
           "includes": "psi H2D, 5000 steps, 101 save points (energy, norm, Mz, psi D2H), final psi D2H"}

    # ---- measured FMA peaks (the compute-roofline denominators)
    fp_peaks = {}
    for prec, key in ((1, "fp32_tflops"), (0, "fp64_tflops")):
        v = __import__("ctypes").c_double()
        S._lib.check(lib.sbec_measure_fma_peak(prec, __import__("ctypes").byref(v)))
        fp_peaks[key] = v.value
    fp_peaks["how"] = "sbec_measure_fma_peak: register-resident FMA chains, 2048 threads/SM, CUDA events"

    # ---- plain FP64 form on the same workload
    plain = None
    if not args.no_plain:
        p_steps = max(50, steps // 5)
        ws64 = make("fp64", p_steps, SAVE_EVERY)
        ms64, _ = timed_runs(ws64, max(1, args.steps // 2), 1)
        ws64.close()
        ms64 = dist.max(ms64)
        v64 = dist.world * units_per_run(p_steps) * max(1, args.steps // 2) / (ms64 / 1e3)
        steps_per_s = p_steps * max(1, args.steps // 2) / (ms64 / 1e3)
        # FFT flops per step by the 5 N log2 N convention: a forward and an inverse 2-D
        # transform of each component (the pointwise stages are not counted)
        npts = N_GRID[0] * N_GRID[1]
        fft_flops = 2 * 5.0 * (2 * F + 1) * npts * math.log2(npts)
        plain = {"value": v64, "unit": UNIT, "steps_per_run": p_steps,
                 "fft_tflops": fft_flops * steps_per_s / 1e12,
                 "fp64_peak_tflops_measured": fp_peaks.get("fp64_tflops"),
                 "fft_frac_of_fp64_peak": (fft_flops * steps_per_s / 1e12 / fp_peaks["fp64_tflops"])
                 if fp_peaks.get("fp64_tflops") else None}

    # ---- error of the FP32-bulk run against the plain FP64 form (itself within 1e-10 of
    # the oracle in the parity tests) after the full 5000-step run
    accuracy = None
    if not args.no_plain:
        finals = {}
        for prec in ("fp32", "fp64"):
            w = make(prec, steps, steps + 1)
            S.run_simulation(w, keep_psi=False)
            finals[prec] = (w.psi, S.total_energy(w), S.total_norm(w), S.magnetization(w))
            w.close()
        (p32, e32, n32, m32), (p64, e64, n64, m64) = finals["fp32"], finals["fp64"]
        accuracy = {"steps": steps, "psi_max_rel": float(np.max(np.abs(p32 - p64)) / np.max(np.abs(p64))),
                    "energy_rel": abs(e32 - e64) / abs(e64), "norm_rel": abs(n32 - n64) / abs(n64),
                    "magnetization_abs": abs(m32 - m64)}

    log("main workload done")
    quick = None
    if not args.no_quickstart:
        quick = bench_quickstart(S)
        log("quickstart done")
    batched = None
    if not args.no_batched:
        batched = bench_batched(S)
        log("batched done")
    serving = None
    if not args.no_serving:
        serving = bench_serving(S, args.serve_requests)
        log("serving done")
    dipolar = None
    if not args.no_3d:
        dipolar = bench_3d_f6(S, n=args.grid_3d, fp32_peak=fp_peaks.get("fp32_tflops"))
        log("3d f6 done")

    cpu = None
    if dist.rank == 0 and not args.no_cpu:
        cpu = cpu_calibrated(args.cpu_seconds, os.cpu_count() or 1)

    if dist.rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": dist.world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms32 / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "fp32", "data": "synthetic",
            "config": {"workload": WORKLOAD, "grid": list(N_GRID), "components": 2 * F + 1, "steps_per_run": steps,
                       "save_every": SAVE_EVERY,
                       "save_points": "energy, norm, Mz and a pinned host copy of psi at each (pipelined)",
                       "precision": "fp32 bulk (FFTs, phases), fp64 reductions", "parallelism": "replicas",
                       "l2": "flushed (256 MB write) between timed runs; psi (1.5 MB) stays L2-resident within a run"},
            "e2e": e2e,
            "autotune": autotune,
            "plain_fp64": plain,
            "fp32_vs_fp64": accuracy,
            "quickstart_1d": quick,
            "batched_ground_states": batched,
            "serving": serving,
            "dipolar_3d_f6": dipolar,
            "vs_plain_fp64": (value / plain["value"]) if plain else None,
            "roofline": {"bound": "hbm", "kernel": dom_name, "achieved": achieved, "peak": hbm, "unit": "GB/s",
                         "frac": achieved / hbm, "traffic": traffic, "peak_source": peak_src,
                         "bytes_per_launch": per_launch_bytes, "us_per_launch": per_launch_s * 1e6,
                         "timing": "autotuner burst: 8 back-to-back launches of the chosen variant, median of 3"
                                   if burst_us else "per-launch CUDA events (profiled run)",
                         "us_per_launch_profiled": profiled_s * 1e6,
                         "run_algorithmic_bytes": run_bytes,
                         "step_algorithmic_gbs": run_bytes / (ms32 / args.steps / 1e3) / 1e9,
                         "step_frac": run_bytes / (ms32 / args.steps / 1e3) / 1e9 / hbm,
                         "kernel_time_share": kernel_share,
                         "note": "the 1.5 MB state is L2-resident within a run: a latency figure, not HBM"},
            "roofline_batched": batched["row_pass_roofline"] if batched else None,
            "fp_peaks_measured": fp_peaks,
            "cpu_baseline": cpu,
            "clocks": clk,
            "gpu_launches": launches,
        }
        print(json.dumps(line), flush=True)
    dist.close()


def ncu_case(args) -> None:
    """Short runs of each workload for ncu captures (a few steps; no timing)."""
    import __graft_entry__

    __graft_entry__.build()
    import spinorbec as S

    k = args.ncu_steps
    case = args.ncu_case
    if args.ncu_tune_table:
        # the tuned variants of an earlier run: no autotuner trial launches in the capture
        with open(args.ncu_tune_table) as f:
            S.tune_table_import(f.read())
    if case in ("2d256_fp32", "2d256_fp64"):
        g = S.make_grid(S.GridConfig(N_GRID, BOX))
        ws = S.make_workspace(grid=g, atom=S.Na23, interactions=S.InteractionParams(C0, C1), zeeman=S.ZeemanParams(ZP, ZQ),
                              potential=S.HarmonicTrap(*OMEGA), sim_params=S.SimParams(DT, k, False, None, k + 1),
                              precision=case.split("_")[1])
        S.run_simulation(ws, keep_psi=False)
        print(ws.tuning_report)
    elif case == "batch256_fp32":
        g = S.make_grid(S.GridConfig((256, 256), (20.0, 20.0)))
        nb = args.ncu_batch
        psis = [S.init_psi(g, 1, "polar") for _ in range(nb)]
        b = S.GroundStateBatch(grid=g, atom=S.Rb87, c0s=[10.0] * nb, c1s=list(np.linspace(-1, 1, nb)), psi_inits=psis,
                               potential=S.HarmonicTrap(1.0, 1.0), dt=0.005, precision="fp32")
        b.ground_state(k, 1e-30, k)
        print(b.tuning_report)
    elif case in ("3d_f6_fp32", "3d_f6_fp64"):
        ip = S.interaction_params_from_constraint(c_total=4689.0, c1_ratio=1 / 36, F=6, c_extra=(0.0, 0.0, 50.0))
        n = args.ncu_grid
        g = S.make_grid(S.GridConfig((n, n, n), (24.0, 24.0, 24.0)))
        psi = S.init_psi(g, 6, "ferromagnetic")
        ws = S.make_workspace(grid=g, atom=S.AtomSpecies("151Eu", 6), interactions=ip, potential=S.HarmonicTrap(1.0, 1.0, 1.2),
                              sim_params=S.SimParams(1e-3, k, False, None, k + 1), psi_init=psi, enable_ddi=True,
                              c_dd=100.0, ddi_padding=True, precision=case.split("_")[2])
        S.split_step(ws, k)
    else:
        raise SystemExit(f"unknown --ncu-case {case}")
    if args.ncu_export_table:
        with open(args.ncu_export_table, "w") as f:
            f.write(S.tune_table_export())
    print(f"ncu case {case}: {k} steps done")


def only_section(args) -> None:
    """One optional section on its own (its JSON object on stdout)."""
    import __graft_entry__

    __graft_entry__.build()
    import spinorbec as S

    if args.only == "batched":
        out = bench_batched(S)
    elif args.only == "quickstart":
        out = bench_quickstart(S)
    elif args.only == "serving":
        out = bench_serving(S, args.serve_requests)
    else:
        out = bench_3d_f6(S, n=args.grid_3d)
    print(json.dumps({args.only: out}), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--run-steps", type=int, default=RUN_STEPS)
    ap.add_argument("--gs-steps", type=int, default=3000)
    ap.add_argument("--cpu-seconds", type=float, default=15.0)  # the sample lands in ~10-20 s
    ap.add_argument("--no-plain", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-batched", action="store_true")
    ap.add_argument("--no-serving", action="store_true")
    ap.add_argument("--no-quickstart", action="store_true")
    ap.add_argument("--no-3d", action="store_true")
    ap.add_argument("--serve-requests", type=int, default=200)
    ap.add_argument("--only", default=None, choices=["batched", "serving", "3d", "quickstart"],
                    help="run one optional section alone and print its JSON")
    ap.add_argument("--grid-3d", type=int, default=128)
    ap.add_argument("--ncu-case", default=None, help="short run for profiling: 2d256_fp32|2d256_fp64|batch256_fp32|3d_f6_fp32|3d_f6_fp64")
    ap.add_argument("--ncu-steps", type=int, default=4)
    ap.add_argument("--ncu-grid", type=int, default=32)
    ap.add_argument("--ncu-tune-table", default=None, help="import this tune table first (no autotuner trials)")
    ap.add_argument("--ncu-export-table", default=None, help="write the tune table after the run")
    ap.add_argument("--ncu-batch", type=int, default=170, help="solves in the batch256_fp32 case (the 256^2 group)")
    args = ap.parse_args()
    if args.only:
        only_section(args)
        return
    if args.ncu_case:
        ncu_case(args)
        return
    if args.impl == "reference":
        run_reference(args)
    else:
        main_gpu(args)


if __name__ == "__main__":
    main()
