"""Pins the oracle's angular-momentum algebra and coupling transforms to the
known answers and identities of the reference's own tests:
test/test_clebsch_gordan.jl, test/test_interactions_constraint.jl,
test/test_tensor_interaction.jl:1-62, test/test_analytical_validation.jl:243-258."""

import math

import numpy as np
import pytest

import oracle as O


def test_wigner_3j_known_values():  # test/test_clebsch_gordan.jl:3-23
    assert O.wigner_3j(1, 1, 0, 0, 0, 0) == pytest.approx(-1 / math.sqrt(3), abs=1e-12)
    assert O.wigner_3j(1, 1, 0, 1, -1, 0) == pytest.approx(1 / math.sqrt(3), abs=1e-12)
    assert O.wigner_3j(1, 1, 1, 1, 1, 0) == 0.0
    assert O.wigner_3j(1, 1, 2, 0, 0, 0) == pytest.approx(math.sqrt(2 / 15), abs=1e-12)
    assert O.wigner_3j(1, 1, 5, 0, 0, 0) == 0.0
    assert O.wigner_3j(1, 1, 1, 0, 1, -1) != 0.0


def test_cg_known_values_f1():  # :25-40
    assert O.clebsch_gordan(1, 1, 1, -1, 0, 0) == pytest.approx(1 / math.sqrt(3), abs=1e-12)
    assert O.clebsch_gordan(1, 0, 1, 0, 0, 0) == pytest.approx(-1 / math.sqrt(3), abs=1e-12)
    assert O.clebsch_gordan(1, -1, 1, 1, 0, 0) == pytest.approx(1 / math.sqrt(3), abs=1e-12)
    assert O.clebsch_gordan(1, 1, 1, 1, 0, 0) == 0.0
    assert O.clebsch_gordan(2, 2, 2, 2, 4, 4) == pytest.approx(1.0, abs=1e-10)


@pytest.mark.parametrize("F", [1, 2, 3])
def test_cg_orthogonality_and_completeness(F):  # :42-71
    for l in range(0, 2 * F + 1):
        for M in range(-l, l + 1):
            s = sum(O.clebsch_gordan(F, m1, F, M - m1, l, M) ** 2 for m1 in range(-F, F + 1) if abs(M - m1) <= F)
            assert s == pytest.approx(1.0, abs=1e-10)
    if F <= 2:
        for m1 in range(-F, F + 1):
            for m2 in range(-F, F + 1):
                M = m1 + m2
                s = sum(O.clebsch_gordan(F, m1, F, m2, l, M) ** 2 for l in range(0, 2 * F + 1) if abs(M) <= l)
                assert s == pytest.approx(1.0, abs=1e-10)


def test_wigner_6j_known_values_and_orthogonality():  # :73-90
    assert O.wigner_6j(1, 1, 0, 1, 1, 0) == pytest.approx(1 / 3, abs=1e-12)
    assert O.wigner_6j(1, 1, 0, 1, 1, 2) == pytest.approx(1 / 3, abs=1e-12)
    for S1 in range(3):
        for S2 in range(3):
            s = sum((2 * l + 1) * O.wigner_6j(1, 1, l, 1, 1, S1) * O.wigner_6j(1, 1, l, 1, 1, S2) for l in range(3))
            assert s == pytest.approx(1.0 / (2 * S1 + 1) if S1 == S2 else 0.0, abs=1e-10)


def _pair_energy(F, g, sp, table):
    E = 0.0
    for S, gS in g.items():
        for M in range(-S, S + 1):
            A = 0j
            for m1 in range(-F, F + 1):
                m2 = M - m1
                if abs(m2) > F:
                    continue
                A += table.get((S, M, m1, m2), 0.0) * sp[F - m1] * sp[F - m2]
            E += gS * abs(A) ** 2
    return E


def test_f1_pair_amplitude_consistency():  # :92-120
    a0, a2 = 5.0, 10.0
    c0, c1 = (a0 + 2 * a2) / 3, (a2 - a0) / 3
    psi = np.array([0.5 + 0.1j, 0.3 - 0.2j, 0.4 + 0.3j])
    sm = O.spin_matrices(1)
    n = float(np.sum(np.abs(psi) ** 2))
    f = [float(np.real(psi.conj() @ M @ psi)) for M in (sm.Fx, sm.Fy, sm.Fz)]
    V_std = c0 * n ** 2 + c1 * sum(x * x for x in f)
    tab = {}
    for S in (0, 2):
        for M in range(-S, S + 1):
            for m1 in (-1, 0, 1):
                if abs(M - m1) <= 1:
                    tab[(S, M, m1, M - m1)] = O.clebsch_gordan(1, m1, 1, M - m1, S, M)
    V_pair = _pair_energy(1, {0: a0, 2: a2}, psi, tab)
    assert V_pair == pytest.approx(V_std, rel=1e-10)


@pytest.mark.parametrize("F", [1, 2, 3, 6])
def test_ck_gS_roundtrip(F):  # :122-131 (seeded draws instead of randn)
    rng = np.random.default_rng(F)
    c = {k: float(rng.standard_normal()) for k in range(0, 2 * F + 1, 2)}
    back = O.gS_to_cn(F, O.cn_to_gS(F, c))
    for k in c:
        assert back[k] == pytest.approx(c[k], abs=1e-10)


def test_f1_analytic_ck_to_gS():  # :133-143
    g = O.cn_to_gS(1, {0: 8.0, 2: 5.0})
    assert g[0] == pytest.approx(8.0 / 3 + 5 * 5.0 / 3, abs=1e-10)
    assert g[2] == pytest.approx(8.0 / 3 + 5.0 / 6, abs=1e-10)


@pytest.mark.parametrize("F", [1, 2, 3])
def test_precompute_cg_table(F):  # :145-160
    t = O.precompute_cg_table(F)
    assert t
    for (l, M, m1, m2), v in t.items():
        assert m1 + m2 == M and abs(m1) <= F and abs(m2) <= F and l % 2 == 0 and 0 <= l <= 2 * F
        assert v == pytest.approx(O.clebsch_gordan(F, m1, F, m2, l, M), abs=1e-14)


def test_interaction_params_from_constraint():  # test/test_interactions_constraint.jl:3-26
    ip = O.interaction_params_from_constraint(c_total=4689.0, c1_ratio=0.0, F=6)
    assert ip.c0 == pytest.approx(4689.0) and ip.c1 == pytest.approx(0.0)
    ip2 = O.interaction_params_from_constraint(c_total=4689.0, c1_ratio=1.0 / 36, F=6)
    assert ip2.c0 + 36 * ip2.c1 == pytest.approx(4689.0, rel=1e-12)
    assert ip2.c1 / ip2.c0 == pytest.approx(1 / 36, rel=1e-12)
    ip3 = O.interaction_params_from_constraint(c_total=4689.0, c1_ratio=-1.0 / 72, F=6)
    assert ip3.c0 + 36 * ip3.c1 == pytest.approx(4689.0, rel=1e-12) and ip3.c1 < 0
    ip4 = O.interaction_params_from_constraint(c_total=100.0, c1_ratio=-0.1, F=1)
    assert ip4.c0 + ip4.c1 == pytest.approx(100.0, rel=1e-12)


def test_c0c1_to_gS_analytic_f1():  # test/test_interactions_constraint.jl:130-135
    g = O.c0c1_to_gS(1, 100.0, -5.0)
    assert g[0] == pytest.approx(100.0 - 2 * -5.0)
    assert g[2] == pytest.approx(100.0 + -5.0)


@pytest.mark.parametrize("F", [1, 2, 6])
def test_c0c1_pair_amplitude_identity(F):  # test/test_interactions_constraint.jl:137-171
    c0, c1 = 100.0, -3.0
    g = O.c0c1_to_gS(F, c0, c1)
    tab = O.precompute_cg_table(F)
    sm = O.spin_matrices(F)
    rng = np.random.default_rng(10 + F)
    for _ in range(5):
        sp = rng.standard_normal(2 * F + 1) + 1j * rng.standard_normal(2 * F + 1)
        n = float(np.sum(np.abs(sp) ** 2))
        Fv = [sp.conj() @ M @ sp for M in (sm.Fx, sm.Fy, sm.Fz)]
        Fsq = float(np.real(sum(abs(x) ** 2 for x in Fv)))
        assert _pair_energy(F, g, sp, tab) == pytest.approx(c0 * n ** 2 + c1 * Fsq, rel=1e-10)


def test_c_extra_to_delta_gS():  # test/test_interactions_constraint.jl:173-182
    assert O.c_extra_to_delta_gS(2, [0.0, 0.0, 5.0])
    assert O.c_extra_to_delta_gS(2, []) == {}
    assert O.c_extra_to_delta_gS(2, [0.0, 3.0]) == {}


def test_tensor_cache_activation():  # test/test_tensor_interaction.jl:3-23, 165-217
    assert O.make_tensor_interaction_cache(1, O.InteractionParams(100.0, 10.0, 0.0, (5.0,))) is None
    assert O.make_tensor_interaction_cache(2, O.InteractionParams(100.0, 10.0, 0.0, ())) is None
    c = O.make_tensor_interaction_cache(2, O.InteractionParams(100.0, 10.0, 0.0, (5.0, 0.0, 3.0)))
    assert c is not None and c.F == 2 and c.D == 5 and 4 in c.active_channels
    cc = O.make_tensor_interaction_cache(2, O.InteractionParams(0.0, 0.0, 0.0, (5.0, 0.0, 3.0)), basis="channel")
    assert cc.g_values[cc.active_channels.index(2)] == pytest.approx(5.0)
    assert cc.g_values[cc.active_channels.index(4)] == pytest.approx(3.0)
    assert 0 not in cc.active_channels
    d = O.make_tensor_cache_from_channels(2, {0: 100.0, 2: 0.0, 4: 25.0})
    assert set(d.active_channels) == {0, 4} and d.g_values[d.active_channels.index(4)] == pytest.approx(25.0)
    assert O.make_tensor_cache_from_channels(2, {}) is None
    assert O.make_tensor_interaction_cache(2, O.InteractionParams(0.0, 0.0)) is None


@pytest.mark.parametrize("F,expected", [(1, 28), (2, 185), (6, 7497)])
def test_hf_entry_counts(F, expected):
    """Number of h-build terms with every channel active (the CG sparsity rule of
    src/tensor_interaction.jl:165-193)."""
    c = O.make_tensor_cache_from_channels(F, {S: 1.0 for S in range(0, 2 * F + 1, 2)})
    assert len(O.precompute_hf_entries(c)[0]) == expected


def test_f1_pair_amplitudes_complete():  # test/test_tensor_interaction.jl:25-62
    rng = np.random.default_rng(3)
    tab = O.precompute_cg_table(1)
    for _ in range(16):
        sp = rng.standard_normal(3) + 1j * rng.standard_normal(3)
        n = float(np.sum(np.abs(sp) ** 2))
        assert _pair_energy(1, {0: 1.0, 2: 1.0}, sp, tab) == pytest.approx(n ** 2, rel=1e-10)


def test_spin_matrices_fy_eigen():  # src/spin_matrices.jl:38-45
    for F in (1, 2, 6):
        sm = O.spin_matrices(F)
        assert np.allclose(sm.Fy_eigvals, np.arange(-F, F + 1), atol=1e-12)
        assert np.allclose(sm.Fy @ sm.Fy_eigvecs, sm.Fy_eigvecs * sm.Fy_eigvals, atol=1e-12)
