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


# ----------------------------------------------------------------------------- GPU arm
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

    flush = torch.empty(int(256e6) // 4, dtype=torch.float32, device="cuda")

    def make(precision: str, steps: int, save_every: int):
        return S.make_workspace(grid=grid, atom=atom, interactions=inter, zeeman=zee, potential=trap,
                                sim_params=S.SimParams(DT, steps, False, None, save_every), psi_init=psi0,
                                precision=precision)

    def timed_runs(ws, n_runs: int, warm: int) -> tuple:
        ext = torch.cuda.ExternalStream(ws.stream_ptr)
        for _ in range(warm):
            S.run_simulation(ws, keep_psi=False)
        total_ms = 0.0
        l0 = ws.launch_count
        for _ in range(n_runs):
            flush.fill_(1.0)
            torch.cuda.synchronize()
            dist.barrier()
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            a.record(ext)
            st = S._lib.load().sbec_run_simulation(ws.handle, ws.sim_params.n_steps, ws.sim_params.save_every,
                                                   S._lib.CALLBACK(), None)
            S._lib.check(st)
            b.record(ext)
            b.synchronize()
            total_ms += a.elapsed_time(b)
        launches = ws.launch_count - l0
        return total_ms, launches

    # ---- chosen form, device resident
    steps = args.run_steps
    ws32 = make("fp32", steps, steps + 1)
    clocks = ClockSampler()
    clocks.start()
    ms32, launches = timed_runs(ws32, args.steps, args.warmup)
    clk = clocks.stop()
    ms32 = dist.max(ms32)
    value = dist.world * units_per_run(steps) * args.steps / (ms32 / 1e3)

    # ---- roofline of the dominant kernel (profiled pass, CUDA events on the engine stream)
    ws32.profile(True)
    S.run_simulation(ws32, keep_psi=False)
    prof = ws32.profile_read()
    ws32.profile(False)
    dom_name, dom = max(prof.items(), key=lambda kv: kv[1]["ms"])
    peaks = measured_peaks()
    hbm = float(peaks.get("hbm_gbs", 6800.0))
    peak_src = "MEASURED_PEAKS.json hbm_gbs (of measured)" if "hbm_gbs" in peaks else "fallback 6800 GB/s"
    per_launch_bytes = dom["bytes"] / max(dom["launches"], 1)
    per_launch_s = dom["ms"] / 1e3 / max(dom["launches"], 1)
    achieved = per_launch_bytes / per_launch_s / 1e9
    traffic = None
    tfile = ROOT / "profiles" / "traffic_2d_256_fp32.json"
    if tfile.exists():
        try:
            traffic = json.loads(tfile.read_text()).get(dom_name)
        except Exception:
            traffic = None
    kernel_share = {k: round(v["ms"] / sum(x["ms"] for x in prof.values()), 4) for k, v in prof.items()}
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

    # ---- plain FP64 form on the same workload
    plain = None
    if not args.no_plain:
        p_steps = max(50, steps // 5)
        ws64 = make("fp64", p_steps, p_steps + 1)
        ms64, _ = timed_runs(ws64, max(1, args.steps // 2), 1)
        ws64.close()
        ms64 = dist.max(ms64)
        v64 = dist.world * units_per_run(p_steps) * max(1, args.steps // 2) / (ms64 / 1e3)
        plain = {"value": v64, "unit": UNIT, "steps_per_run": p_steps}

    cpu = None
    if dist.rank == 0 and not args.no_cpu:
        cpu = cpu_calibrated(args.cpu_seconds, os.cpu_count() or 1)

    if dist.rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": dist.world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms32 / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "fp32", "data": "synthetic",
            "config": {"workload": WORKLOAD, "grid": list(N_GRID), "components": 2 * F + 1, "steps_per_run": steps,
                       "precision": "fp32 bulk (FFTs, phases), fp64 reductions", "parallelism": "replicas",
                       "l2": "flushed (256 MB write) between timed runs; psi (1.5 MB) stays L2-resident within a run"},
            "e2e": e2e,
            "plain_fp64": plain,
            "vs_plain_fp64": (value / plain["value"]) if plain else None,
            "roofline": {"bound": "hbm", "kernel": dom_name, "achieved": achieved, "peak": hbm, "unit": "GB/s",
                         "frac": achieved / hbm, "traffic": traffic, "peak_source": peak_src,
                         "bytes_per_launch": per_launch_bytes, "us_per_launch": per_launch_s * 1e6,
                         "step_algorithmic_gbs": value * 49.3 / 1e9, "kernel_time_share": kernel_share},
            "cpu_baseline": cpu,
            "clocks": clk,
            "gpu_launches": launches,
        }
        print(json.dumps(line), flush=True)
    dist.close()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--run-steps", type=int, default=RUN_STEPS)
    ap.add_argument("--gs-steps", type=int, default=3000)
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--no-plain", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
    else:
        main_gpu(args)


if __name__ == "__main__":
    main()
