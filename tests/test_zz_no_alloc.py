"""The allocation-free reduction entry point, sbec_component_norms_noalloc.

It serves callers that cannot allocate GPU memory at call time (work being
captured into a CUDA graph, or hosts whose device memory belongs to another
allocator).  Its scratch is a fixed device array shared by all calls, so the test
calls it twice in a row on different wavefunctions and checks each result against
the workspace entry points sbec_total_norm / sbec_magnetization for the same psi.
This file is collected last so that a failure here leaves every other test run.
"""

import ctypes

import numpy as np
import pytest

import oracle as O
import spinorbec as S

pytestmark = pytest.mark.gpu


def _noalloc_sums(psi: np.ndarray, D: int) -> np.ndarray:
    torch = pytest.importorskip("torch")
    n_points = psi.size // D
    dev_psi = torch.from_numpy(S.to_interleaved(psi).copy()).to("cuda")
    out = torch.full((D + 1,), -1.0, dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    st = S.load().sbec_component_norms_noalloc(ctypes.c_void_p(dev_psi.data_ptr()), n_points, D,
                                               ctypes.c_void_p(out.data_ptr()), ctypes.c_void_p(stream))
    S._lib.check(st)
    torch.cuda.synchronize()
    return out.cpu().numpy()


def test_noalloc_matches_workspace_on_two_calls(gpu):
    cases = [((32, 32), (10.0, 10.0), 1, 1), ((16, 8, 8), (6.0, 6.0, 6.0), 2, 2)]
    for n, L, F, seed in cases:
        D = 2 * F + 1
        og = O.make_grid(O.GridConfig(n, L))
        psi = O.init_psi(og, F, "random", seed=seed)
        ws = S.make_workspace(grid=S.make_grid(S.GridConfig(n, L)), atom=S.AtomSpecies("x", F),
                              interactions=S.InteractionParams(1.0, 0.0), sim_params=S.SimParams(1e-3, 1),
                              psi_init=psi, precision="fp64")
        sums = _noalloc_sums(psi, D)
        dV = O.cell_volume(og)
        norm = float(np.sum(sums[:D])) * dV
        mz = float(sum((F - c) * sums[c] for c in range(D))) * dV
        assert sums[D] == 0.0  # no NaN entries
        assert abs(norm - S.total_norm(ws)) <= 1e-13 * abs(S.total_norm(ws))
        assert abs(mz - S.magnetization(ws)) <= 1e-12 * max(1.0, abs(S.magnetization(ws)))
        ws.close()


def test_noalloc_counts_planted_nan(gpu):
    """One NaN entry in psi: the component sums of the other entries are unaffected in the
    NaN-free components and the NaN count slot reads 1."""
    og = O.make_grid(O.GridConfig((32, 32), (10.0, 10.0)))
    psi = O.init_psi(og, 1, "random", seed=3)
    clean = _noalloc_sums(psi, 3)
    psi[5, 7, 1] = complex(np.nan, 0.0)
    sums = _noalloc_sums(psi, 3)
    assert sums[3] == 1.0
    assert sums[0] == clean[0] and sums[2] == clean[2]
    assert np.isnan(sums[1])


def test_noalloc_rejects_sizes_beyond_limits(gpu):
    torch = pytest.importorskip("torch")
    buf = torch.zeros(64, dtype=torch.float64, device="cuda")
    lib = S.load()
    st = lib.sbec_component_norms_noalloc(ctypes.c_void_p(buf.data_ptr()), 1, 17, ctypes.c_void_p(buf.data_ptr()),
                                          None)
    with pytest.raises(S.ArgumentError):
        S._lib.check(st)
    st = lib.sbec_component_norms_noalloc(ctypes.c_void_p(buf.data_ptr()), (1 << 31) + 1, 3,
                                          ctypes.c_void_p(buf.data_ptr()), None)
    with pytest.raises(S.ArgumentError):
        S._lib.check(st)
    # psi at an odd double offset (a view that splits a complex entry) is refused
    st = lib.sbec_component_norms_noalloc(ctypes.c_void_p(buf.data_ptr() + 8), 4, 3,
                                          ctypes.c_void_p(buf.data_ptr()), None)
    with pytest.raises(S.ArgumentError):
        S._lib.check(st)
