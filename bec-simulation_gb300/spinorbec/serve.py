"""Continuous-batching request server for ground-state and dynamics solves.

Requests arrive over time (e.g. a seeded Poisson stream).  A request is admitted
as soon as its device footprint fits the HBM budget and a slot is free; each
admitted request gets a resident workspace with its own CUDA stream and runs in a
worker thread (the C calls release the GIL), so the work of requests that are in
flight together overlaps on the GPU.  When a request finishes, its workspace is
freed and the next waiting requests are admitted.  Every kernel and reduction of
the engine is deterministic, so a request's result does not depend on what else
is in flight.

Per request the server records queueing, service and end-to-end latency; run()
returns them with throughput and p50/p99.

Request workspaces launch their kernels eagerly (graphs off): each lives for one short
solve, and capturing and instantiating CUDA graphs in two dozen concurrent workspaces
cost more than the replays saved (24-request stream: 8.9 solves/s eager against
4.9-6.6 with graphs).

Ground-state requests that can share kernels (merge_key: contact couplings, no DDI, same
grid, F, dt, tol, trap and precision) are merged when the server is given a merge window:
the requests of one key that arrive in the same window [k w, (k + 1) w) run as one
GroundStateBatch (per-solve c0, c1 and step limit, each solve with find_ground_state's loop
and convergence test), dispatched at the window's end.  The grouping depends only on the
arrival times, so which requests share a batch is the same in every run.
"""

from __future__ import annotations

import math
import threading
import time
from concurrent.futures import ThreadPoolExecutor
from dataclasses import dataclass
from typing import Callable, Optional

import numpy as np

from . import api
from .host import (AtomSpecies, GridConfig, HarmonicTrap, InteractionParams, SimParams, ZeemanParams, init_psi,
                   make_grid)


@dataclass
class SolveRequest:
    """One solve: a ground state (find_ground_state) or a real-time run (run_simulation!)."""

    rid: int
    kind: str                 # "ground_state" | "dynamics"
    n_points: tuple
    box_size: tuple
    F: int
    c0: float
    c1: float
    steps: int
    dt: float = 0.005
    enable_ddi: bool = False
    c_dd: float = 0.0
    tol: float = 1e-8
    arrival: float = 0.0      # seconds after the start of the stream
    precision: str = "fp32"
    omega: float = 1.0


@dataclass
class SolveResult:
    rid: int
    kind: str
    energy: float
    norm: float
    converged: Optional[bool]
    steps: int
    arrival: float
    admitted: float
    finished: float
    footprint: int

    @property
    def latency(self) -> float:
        return self.finished - self.arrival

    @property
    def queueing(self) -> float:
        return self.admitted - self.arrival


def footprint_bytes(req: SolveRequest, ddi_padding: bool = False) -> int:
    """Upper bound of the device memory one request's workspace allocates: four psi slots
    and a scratch copy, V and a 3-field temporary, the FP64 staging buffer of the FP32 form,
    and for DDI the spin density, two phi fields and the half-spectrum of three fields
    (periodic, plus the zero-padded one when enabled); 10 % and 8 MiB on top for tables,
    reduction partials and allocation granularity."""
    N = int(np.prod(req.n_points))
    nc = N * (2 * req.F + 1)
    s = 8 if req.precision.startswith("fp32") else 16   # bytes per complex element
    r = s // 2
    total = 5 * nc * s + 4 * N * r
    if s == 8:
        total += nc * 16
    if req.enable_ddi:
        total += 9 * N * r + (3 * N * s) // 2
        if ddi_padding:
            total += 6 * N * s
    return int(total * 1.1) + (8 << 20)


def run_request(req: SolveRequest) -> dict:
    """Run one request to completion on its own workspace (and stream); returns its results."""
    grid = make_grid(GridConfig(req.n_points, req.box_size))
    atom = AtomSpecies("req", req.F)
    inter = InteractionParams(req.c0, req.c1)
    trap = HarmonicTrap(*([req.omega] * len(req.n_points)))
    if req.kind == "ground_state":
        r = api.find_ground_state(grid=grid, atom=atom, interactions=inter, potential=trap, dt=req.dt,
                                  n_steps=req.steps, tol=req.tol, initial_state="polar",
                                  enable_ddi=req.enable_ddi, c_dd=req.c_dd if req.enable_ddi else float("nan"),
                                  precision=req.precision, graphs=False)
        ws = r["workspace"]
        out = dict(energy=r["energy"], norm=api.total_norm(ws), converged=r["converged"], steps=r["steps"])
        ws.close()
        return out
    psi = init_psi(grid, req.F, "ferromagnetic" if req.F > 1 else "polar")
    ws = api.make_workspace(grid=grid, atom=atom, interactions=inter, potential=trap,
                            zeeman=ZeemanParams(0.0, 0.1),
                            sim_params=SimParams(req.dt, req.steps, False, None, req.steps), psi_init=psi,
                            enable_ddi=req.enable_ddi, c_dd=req.c_dd, precision=req.precision, graphs=False)
    res = api.run_simulation(ws, keep_psi=False)
    out = dict(energy=res.energies[-1], norm=res.norms[-1], converged=None, steps=req.steps,
               energy0=res.energies[0])
    ws.close()
    return out


def merge_key(req: SolveRequest) -> Optional[tuple]:
    """The key of the requests that may run as one GroundStateBatch, or None: ground states
    with contact couplings (F <= 2, no DDI) on a grid the batch takes (api.batch_supported),
    with the same grid, dt, tol, trap and precision (the batch's shared terms; c0, c1 and the
    step limit are per solve)."""
    if req.kind != "ground_state" or req.enable_ddi or req.F > 2:
        return None
    if not api.batch_supported(make_grid(GridConfig(req.n_points, req.box_size)), req.F, req.precision):
        return None
    return (tuple(req.n_points), tuple(req.box_size), req.F, req.dt, req.tol, req.omega, req.precision)


def run_batch(reqs: list) -> list:
    """Run requests of one merge_key as one GroundStateBatch from the polar state (as
    run_request); returns one result dict per request, in order."""
    r0 = reqs[0]
    grid = make_grid(GridConfig(r0.n_points, r0.box_size))
    psi0 = init_psi(grid, r0.F, "polar")
    b = api.GroundStateBatch(grid=grid, atom=AtomSpecies("req", r0.F), c0s=[r.c0 for r in reqs],
                             c1s=[r.c1 for r in reqs], psi_inits=[psi0] * len(reqs),
                             potential=HarmonicTrap(*([r0.omega] * len(r0.n_points))), dt=r0.dt,
                             precision=r0.precision)
    try:
        b.set_graph_mode(False)
        res = b.ground_state([r.steps for r in reqs], r0.tol)
        dV = float(np.prod([L / n for L, n in zip(r0.box_size, r0.n_points)]))
        outs = []
        for i, r in enumerate(res):
            norm = float(np.sum(np.abs(b.psi(i)) ** 2) * dV)
            outs.append(dict(energy=r["energy"], norm=norm, converged=r["converged"], steps=r["steps"]))
        return outs
    finally:
        b.close()


def dispatch_units(requests: list, merge_window_s: float = 0.0, max_merge: int = 32,
                   budget_bytes: float = float("inf")) -> list:
    """Split `requests` into dispatch units [(time, [requests])], sorted by time.  Without a
    window every request is its own unit at its arrival; with one, the requests of a
    merge_key that arrive in the same window form units of up to max_merge requests (and at
    most budget_bytes of summed footprint), dispatched at the window's end."""
    order = sorted(requests, key=lambda r: r.arrival)
    units = []
    groups: dict = {}
    for r in order:
        k = merge_key(r) if merge_window_s > 0 else None
        if k is None:
            units.append((r.arrival, [r]))
        else:
            groups.setdefault((k, int(r.arrival // merge_window_s)), []).append(r)
    for (_, w), rs in groups.items():
        t = (w + 1) * merge_window_s
        cur, fp = [], 0
        for r in rs:
            f = footprint_bytes(r)
            if cur and (len(cur) >= max_merge or fp + f > budget_bytes):
                units.append((t, cur))
                cur, fp = [], 0
            cur.append(r)
            fp += f
        units.append((t, cur))
    units.sort(key=lambda u: (u[0], u[1][0].rid))
    return units


def pretune(requests: list, merge_window_s: float = 0.0, max_merge: int = 32) -> int:
    """Fix the autotuner's decisions before any request is served: one two-step run per
    distinct (grid, F, DDI, kind, precision) and per merged batch size, then the table is
    frozen (api.tune_freeze), so shapes met later (a batch whose solves have left) take
    their default variant untimed.  Served results then do not depend on which request met a
    shape first; returns the number of shapes run."""
    seen = set()
    for _, rs in dispatch_units(requests, merge_window_s, max_merge):
        r = rs[0]
        key = (tuple(r.n_points), r.F, r.enable_ddi, r.kind, r.precision, len(rs) if len(rs) > 1 else 0)
        if key in seen:
            continue
        seen.add(key)
        if len(rs) > 1:
            run_batch([SolveRequest(**{**q.__dict__, "steps": 2, "tol": 0.0}) for q in rs])
        else:
            run_request(SolveRequest(**{**r.__dict__, "steps": 2, "tol": 0.0}))
    api.tune_freeze(True)
    return len(seen)


def work_estimate(req: SolveRequest) -> float:
    """Relative cost of a request for admission order: points x components x steps, four
    times that with the dipolar convolution (its six FFTs on the padded grid)."""
    w = float(np.prod(req.n_points)) * (2 * req.F + 1) * req.steps
    return 4.0 * w if req.enable_ddi else w


class Server:
    """Admission by HBM budget and slots; concurrent resident workspaces.

    policy "fifo" admits waiting units in the order they were dispatched; "sjf" admits the
    waiting unit with the least estimated work (work_estimate, summed over a merged unit)
    first, ties by dispatch order — the same solves and results, shorter queueing for short
    requests."""

    def __init__(self, hbm_budget_bytes: float = 150e9, max_slots: int = 32,
                 runner: Callable[[SolveRequest], dict] = run_request,
                 batch_runner: Callable[[list], list] = run_batch, merge_window_s: float = 0.0,
                 max_merge: int = 32, policy: str = "fifo"):
        if policy not in ("fifo", "sjf"):
            raise ValueError("policy must be 'fifo' or 'sjf'")
        self.budget = float(hbm_budget_bytes)
        self.max_slots = int(max_slots)
        self.runner = runner
        self.batch_runner = batch_runner
        self.merge_window_s = float(merge_window_s)
        self.max_merge = int(max_merge)
        self.policy = policy
        self.merged_units = 0
        self.merged_requests = 0
        self._used = 0.0
        self._active = 0
        self._waiting: dict = {}  # ticket -> (priority key, footprint)
        self._tickets = 0
        self.peak_used = 0.0
        self.peak_active = 0
        self._cv = threading.Condition()

    def _fits(self, fp: int) -> bool:
        return self._active < self.max_slots and (self._used + fp <= self.budget or self._active == 0)

    def _admit(self, fp: int, work: float = 0.0, seq: Optional[int] = None) -> None:
        with self._cv:
            ticket = self._tickets
            self._tickets += 1
            order = ticket if seq is None else seq  # dispatch order
            key = (work, order) if self.policy == "sjf" else (0.0, order)
            self._waiting[ticket] = (key, fp)
            # admitted when it fits and no waiting unit ahead of it in the policy's order fits
            while not (self._fits(fp) and
                       all(not (k < key and self._fits(f)) for k, f in self._waiting.values())):
                self._cv.wait()
            del self._waiting[ticket]
            self._used += fp
            self._active += 1
            self.peak_used = max(self.peak_used, self._used)
            self.peak_active = max(self.peak_active, self._active)
            self._cv.notify_all()

    def _release(self, fp: int) -> None:
        with self._cv:
            self._used -= fp
            self._active -= 1
            self._cv.notify_all()

    def run(self, requests: list, realtime: bool = True) -> dict:
        """Serve `requests`; returns per-request results and stats.

        With realtime=True each request is submitted at its arrival time (seconds from
        the call); otherwise all are submitted at once and queue by arrival order."""
        t0 = time.perf_counter()
        results: list = []
        lock = threading.Lock()

        def serve(seq: int, reqs: list):
            fps = [footprint_bytes(r) for r in reqs]
            fp = sum(fps)
            if fp > self.budget:
                raise MemoryError(f"request {reqs[0].rid} needs {fp / 1e9:.1f} GB > budget")
            self._admit(fp, sum(work_estimate(r) for r in reqs), seq)
            admitted = time.perf_counter() - t0
            try:
                outs = [self.runner(reqs[0])] if len(reqs) == 1 else self.batch_runner(reqs)
            finally:
                self._release(fp)
            fin = time.perf_counter() - t0
            with lock:
                for req, out, f in zip(reqs, outs, fps):
                    results.append(SolveResult(req.rid, req.kind, out["energy"], out["norm"], out["converged"],
                                               out["steps"], req.arrival, admitted, fin, f))

        units = dispatch_units(requests, self.merge_window_s, self.max_merge, self.budget)
        for _, rs in units:
            if len(rs) > 1:
                self.merged_units += 1
                self.merged_requests += len(rs)
        # one thread per dispatched unit: every unit that has arrived waits in _admit, so the
        # admission policy chooses among all of them
        with ThreadPoolExecutor(max_workers=max(self.max_slots + 4, len(units))) as ex:
            futs = []
            for seq, (t_disp, rs) in enumerate(units):
                if realtime:
                    wait = t_disp - (time.perf_counter() - t0)
                    if wait > 0:
                        time.sleep(wait)
                futs.append(ex.submit(serve, seq, rs))
            for f in futs:
                f.result()
        wall = time.perf_counter() - t0
        lat = np.array([r.latency for r in results])
        return dict(results=sorted(results, key=lambda r: r.rid), wall_s=wall,
                    solves_per_s=len(results) / wall if wall > 0 else float("nan"),
                    p50_latency_s=float(np.percentile(lat, 50)) if len(lat) else float("nan"),
                    p99_latency_s=float(np.percentile(lat, 99)) if len(lat) else float("nan"))


def poisson_requests(n: int, rate: float = 200.0, seed: int = 5, *, max_points_3d: int = 128,
                     max_steps: int = 5000, min_steps: int = 500, precision: str = "fp32") -> list:
    """Seeded request stream: dimension uniform over 1-D/2-D/3-D with power-of-two sizes drawn
    log-uniformly (1-D 256..4096, 2-D 64^2..512^2, 3-D 32^3..max^3), F in {1, 2, 6}, c0 ~ U[5, 20],
    c1 ~ U[-1, 1], DDI on for F = 6, steps ~ U{min..max}, half ground states, half dynamics."""
    rng = np.random.Generator(np.random.PCG64(seed))
    t = 0.0
    reqs = []
    for i in range(n):
        t += rng.exponential(1.0 / rate)
        dim = int(rng.integers(1, 4))
        if dim == 1:
            e = int(rng.integers(8, 13))
            npts = (2 ** e,)
            box = (40.0,)
        elif dim == 2:
            e = int(rng.integers(6, 10))
            npts = (2 ** e, 2 ** e)
            box = (20.0, 20.0)
        else:
            hi = int(round(math.log2(max_points_3d)))
            e = int(rng.integers(5, hi + 1))
            npts = (2 ** e,) * 3
            box = (16.0,) * 3
        F = int(rng.choice([1, 2, 6]))
        kind = "ground_state" if rng.random() < 0.5 else "dynamics"
        reqs.append(SolveRequest(rid=i, kind=kind, n_points=npts, box_size=box, F=F,
                                 c0=float(rng.uniform(5.0, 20.0)), c1=float(rng.uniform(-1.0, 1.0)),
                                 steps=int(rng.integers(min_steps, max_steps + 1)),
                                 dt=0.005 if kind == "ground_state" else 1e-3,
                                 enable_ddi=(F == 6), c_dd=20.0 if F == 6 else 0.0, arrival=t, precision=precision))
    return reqs
