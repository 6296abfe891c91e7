"""CPU FP64 oracle for the SpinorBEC.jl split-step hot path.

TEST INFRASTRUCTURE ONLY.  This package is the checker: only ``tests/``,
``__graft_entry__.smoke()`` and the ``cpu_baseline`` / ``--impl reference``
legs of ``bench.py`` may import it.  The product path (the CUDA library behind
``include/sbec.h`` and the ``spinorbec`` host package) never calls into it.

The reference (anko9801/BEC-simulation, a pure-Julia package) cannot be run in
this container (no ``julia`` binary).  The oracle is a numpy / scipy.fft
restatement of its algorithm, function by function, each citing the Julia
file:line it follows.  Its third-party numerics are FFTW (via FFTW.jl, compat
"1", unpinned: no Manifest.toml) and LAPACK ``eigen(Hermitian)`` (Julia
stdlib); the oracle restates them with pocketfft (scipy.fft) and
``numpy.linalg.eigh``, both accurate FP64 implementations of the same
mathematical maps (the DFT, and the Hermitian eigen-decomposition, whose
exponential ``V e^{-iΛτ} V^†`` is basis independent).

Pinning: the reference stores no golden vectors.  The oracle is pinned by
ports of the reference's own known-answer and invariant tests
(``tests/test_oracle_*.py``: Wigner 3j/6j/CG known values from
test/test_clebsch_gordan.jl, the g_S identities of
test/test_interactions_constraint.jl, the conservation and order tests of
test/test_split_step.jl, test/test_physics_level1.jl, test/test_ddi.jl,
test/test_tensor_interaction.jl, test/test_analytical_validation.jl, the
singlet-pair (nematic) tests of test/test_nematic.jl, the loss tests of
test/test_losses.jl, the Raman tests of test/test_raman.jl and the ground-state tests of
test/test_simulation.jl).
"""

from .spinorbec_oracle import *  # noqa: F401,F403
