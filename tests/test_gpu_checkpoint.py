"""run_simulation_checkpointed (src/simulation.jl:96-148) over the device drivers: a run that
stops half way and resumes from its latest checkpoint ends where the continuous run ends
(test/test_checkpoint.jl:21-54, there to 1e-10), the checkpoint files carry the reference's
fields, and the state in a checkpoint equals the oracle's state at that step."""

import os

import numpy as np
import pytest

import oracle as O
import spinorbec as S
from parity_util import PSI_TOL_FP64, make_pair, rel_psi_err

pytestmark = pytest.mark.gpu


def _pair(n_steps):
    ws_o, ws_g = make_pair((32, 32), (12.0, 12.0), 1, c0=10.0, c1=0.5, omega=(1.0, 1.0), zeeman=(0.0, 0.1),
                           dt=1e-3, state="random")
    ws_o.sim_params = O.SimParams(1e-3, n_steps, False, None, 10)
    ws_g.sim_params = S.SimParams(1e-3, n_steps, False, None, 10)
    return ws_o, ws_g


def test_checkpoint_resume_equals_continuous(gpu, tmp_path):
    ws_o, full = _pair(100)
    psi0 = full.psi
    S.run_simulation(full, keep_psi=False)
    # first half: checkpoints at steps 20 and 40 (save points every 10)
    d = str(tmp_path / "ck")
    _, half = _pair(50)
    half.psi = psi0
    S.run_simulation_checkpointed(half, checkpoint_dir=d, checkpoint_every=20)
    files = sorted(os.listdir(d))
    assert files == ["step_00000020.npz", "step_00000040.npz"]
    data = S.load_state(os.path.join(d, files[-1]))
    assert data["step"] == 40 and abs(data["t"] - 0.04) < 1e-14
    assert set(data) >= {"psi", "t", "step", "grid_n_points", "grid_box_size", "c0", "c1", "zeeman_q", "dt"}
    # the state at step 40 is the oracle's state at step 40
    ws_o.sim_params = O.SimParams(1e-3, 40, False, None, 10)
    O.run_simulation(ws_o, keep_psi=False)
    assert rel_psi_err(data["psi"], ws_o.psi) < PSI_TOL_FP64
    # resume a fresh 100-step workspace from the latest checkpoint (step 40) and finish
    _, rest = _pair(100)
    steps = []
    S.run_simulation_checkpointed(rest, checkpoint_dir=d, checkpoint_every=20, resume=True,
                                  callback=lambda ws, step: steps.append(step))
    assert steps == [10, 20, 30, 40, 50, 60]   # save points of the 60 remaining steps
    assert rest.step == 100 and abs(rest.t - full.t) < 1e-12
    assert float(np.max(np.abs(rest.psi - full.psi))) < 1e-10
    assert sorted(os.listdir(d))[-1] == "step_00000100.npz"
    for w in (full, half, rest):
        w.close()
