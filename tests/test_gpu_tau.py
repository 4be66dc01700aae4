"""Time-displaced Green functions (TAU_M + CGR2_2) and the measurement callbacks
(ham%Obser / ham%ObserT) against the CPU oracle on the same fields and draws.

Every callback of one sweep is compared: the equal-time G at each time slice of both
passes, and the quartet [GT0, G0T, G00, GTT] at NT = 0..Ltrot.  Propagated matrices
carry rounding drift, so the bound is the oracle's own propagation-vs-CGR2_2 deviation
(Control_Precision_tau) times ten, floored at 1e-10.
"""
import numpy as np
import pytest

import oracle
from alf_gb300 import model as mdl, rng
from alf_gb300.sweep import Chains

pytestmark = pytest.mark.gpu


def _run(m, seed, ltau=1):
    f0 = rng.initial_fields(seed, 0, m.n_op, m.ltrot)
    u = rng.sweep_uniforms(seed, 0, m.n_op, m.ltrot, 0)
    o = oracle.Oracle(m, ltau=ltau)
    o.set_fields(f0)
    o.init_state()
    eq_o, tau_o = o.collect_measurements()
    o.sweep(u)
    g = Chains(m, ltau=ltau)
    g.set_fields(0, f0)
    g.init_state()
    eq_g, tau_g = g.sweep(u[None, :], measure=True)
    np.testing.assert_array_equal(g.fields(0), o.fields())
    return o, g, eq_o, tau_o, eq_g, tau_g


@pytest.mark.parametrize("shape", [(2, 2, 0.5, 5), (3, 3, 1.0, 5)])
def test_tau_m_quartets_match_oracle(shape):
    l1, l2, beta, nwrap = shape
    m = mdl.hubbard("honeycomb", l1, l2, U=5.0, beta=beta, dtau=0.05, nwrap=nwrap)
    o, g, eq_o, tau_o, eq_g, tau_g = _run(m, seed=3)
    so, sg = o.stats(), g.stats(0)
    assert sg.ncg_tau == so.ncg_tau > 0
    band = max(1e-10, 10.0 * so.xmax_tau)
    assert sg.xmax_tau <= band and so.xmax_tau <= max(1e-10, 10.0 * sg.xmax_tau)
    assert [t[1] for t in tau_g] == [t[0] for t in tau_o] == list(range(m.ltrot + 1))
    for (c, nt, qg, phg), (nt_o, qo, pho) in zip(tau_g, tau_o):
        assert c == 0
        assert abs(phg - pho) < 1e-10
        for k in range(4):
            assert np.max(np.abs(qg[k] - qo[k])) <= band, (nt, k)


def test_equal_time_measurements_match_oracle():
    m = mdl.config("hubbard4x4")
    o, g, eq_o, tau_o, eq_g, tau_g = _run(m, seed=11, ltau=0)
    assert not tau_g and not tau_o
    assert [e[1] for e in eq_g] == [e[0] for e in eq_o]
    assert len(eq_g) == 2 * m.ltrot - 1
    so = o.stats()
    band = max(1e-10, 10.0 * so.xmaxG)
    for (c, nt, Gg, phg), (nt_o, Go, pho) in zip(eq_g, eq_o):
        assert np.max(np.abs(Gg - Go)) <= band, nt
        assert abs(phg - pho) < 1e-10


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_tau_m_with_checkerboard_hopping(precision):
    # TAU_M's PROPR / PROPRM1 with the bond operators (both forms: the bonds are O(N^2) passes)
    m = mdl.hubbard("honeycomb", 2, 2, U=5.0, beta=0.5, dtau=0.05, nwrap=5, checkerboard=True)
    f0 = rng.initial_fields(3, 0, m.n_op, m.ltrot)
    u = rng.sweep_uniforms(3, 0, m.n_op, m.ltrot, 0)
    o = oracle.Oracle(m, ltau=1)
    o.set_fields(f0)
    o.init_state()
    _, tau_o = o.collect_measurements()
    o.sweep(u)
    g = Chains(m, ltau=1, precision=precision)
    g.set_fields(0, f0)
    g.init_state()
    _, tau_g = g.sweep(u[None, :], measure=True)
    np.testing.assert_array_equal(g.fields(0), o.fields())
    band = max(1e-10, 10.0 * o.stats().xmax_tau) if precision == "fp64" else 1e-5
    assert len(tau_g) == len(tau_o) == m.ltrot + 1
    for (c, nt, qg, _), (nt_o, qo, _) in zip(tau_g, tau_o):
        for k in range(4):
            assert np.max(np.abs(qg[k] - qo[k])) <= band, (nt, k)
