"""Index algebra of the shared-memory Stockham transforms (csrc/sbec_fft.cuh), emulated in
numpy: every radix plan of every line length gives numpy's FFT, and the register-resident
forms' slot map holds — the first stage of a plan reads, and its last stage writes, thread t's
positions x = t + k*TPL with k = b + r*(E/RAD) (reg_slot), so a transform can start from and end
in registers.  The plans are read from the header, so a changed plan is checked too."""

import re
from pathlib import Path

import numpy as np
import pytest

HDR = Path(__file__).resolve().parent.parent / "bec-simulation_gb300" / "csrc" / "sbec_fft.cuh"


def _plans():
    out = []
    for m in re.finditer(r"SBEC_PLAN\((FftPlan32|FftPlan), (\d+), (\d+), ([\d, ]+)\)", HDR.read_text()):
        fam, n, e = m.group(1), int(m.group(2)), int(m.group(3))
        rads = [int(x) for x in m.group(4).split(",")]
        out.append((fam, n, e, rads))
    return out


PLANS = _plans()


def _stockham(x, N, E, rads, sign):
    """One line through the plan's stages with the kernels' index formulas; records the
    positions each thread reads in the first stage and writes in the last."""
    TPL = N // E
    s = x.astype(np.complex128).copy()
    Ns = 1
    first_reads, last_writes = {}, {}
    for si, R in enumerate(rads):
        NBT = E // R
        STRIDE = N // R
        out = np.empty_like(s)
        for t in range(TPL):
            for b in range(NBT):
                j = t + b * TPL
                jm = j & (Ns - 1)
                v = np.array([s[j + r * STRIDE] for r in range(R)])
                if si == 0:
                    for r in range(R):
                        first_reads[(t, b * R + r)] = j + r * STRIDE
                if Ns > 1:
                    step = jm * (N // (Ns * R))
                    v = v * np.exp(sign * 2j * np.pi * np.arange(R) * step / N)
                v = np.array([np.sum(v * np.exp(sign * 2j * np.pi * np.arange(R) * q / R)) for q in range(R)])
                base = (j - jm) * R + jm
                for r in range(R):
                    out[base + r * Ns] = v[r]
                    if si == len(rads) - 1:
                        last_writes[(t, b * R + r)] = base + r * Ns
        s = out
        Ns *= R
    return s, first_reads, last_writes


def test_plans_are_parsed():
    assert len(PLANS) >= 20
    for fam, n, e, rads in PLANS:
        assert int(np.prod(rads)) == n and max(rads) == e and all(e % r == 0 for r in rads), (fam, n)


@pytest.mark.parametrize("plan", PLANS, ids=lambda p: f"{p[0]}-{p[1]}")
def test_stockham_plan_matches_fft_and_register_slots(plan):
    fam, N, E, rads = plan
    rng = np.random.default_rng(N)
    x = rng.standard_normal(N) + 1j * rng.standard_normal(N)
    fwd, first, last = _stockham(x, N, E, rads, -1)
    assert np.allclose(fwd, np.fft.fft(x), atol=1e-9 * N)
    inv, _, _ = _stockham(x, N, E, rads, +1)
    assert np.allclose(inv, np.fft.ifft(x) * N, atol=1e-9 * N)
    if len(rads) < 2:
        return
    TPL = N // E
    for (t, e), pos in first.items():
        R = rads[0]
        k = e // R + (e % R) * (E // R)  # reg_slot<E, RAD0>(e)
        assert pos == t + k * TPL
    for (t, e), pos in last.items():
        R = rads[-1]
        k = e // R + (e % R) * (E // R)  # reg_slot<E, RAD_last>(e)
        assert pos == t + k * TPL
    # every position of the line is covered exactly once by the threads' slots
    assert sorted(first.values()) == list(range(N)) and sorted(last.values()) == list(range(N))
