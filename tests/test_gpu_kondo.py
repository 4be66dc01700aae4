"""Kondo lattice (two-site J_K vertices, N_op = 2, non-diagonal) against the CPU oracle.

The GPU runs the sweep in the eigenbasis shared by all J_K vertices (one 2x2 rotation
per c-f pair); the oracle rotates around every vertex update as Op_Wrapup / Op_Wrapdo
do.  Ratios, the accept sequence, fields, G at every stabilisation point (rotated back)
and the time-displaced quartets are compared as in the Hubbard parity tests.
"""
import numpy as np
import pytest

import oracle
from alf_gb300 import _lib, model as mdl, rng
from alf_gb300.sweep import Chains
from tests.test_gpu_parity import _run_pair

pytestmark = pytest.mark.gpu


def _kondo(L=2, beta=1.0, nwrap=5, Uf=0.0):
    return mdl.kondo(L, L, JK=1.5, Uf=Uf, beta=beta, dtau=0.1, nwrap=nwrap)


def test_kondo_bilayer_2x2_parity():
    _run_pair(_kondo(2), seed=5, sweeps=3)


def test_kondo_bilayer_4x4_parity():
    _run_pair(_kondo(4, beta=2.0, nwrap=10), seed=8, sweeps=2)


def test_kondo_tau_m_matches_oracle():
    m = _kondo(2)
    f0 = rng.initial_fields(6, 0, m.n_op, m.ltrot)
    u = rng.sweep_uniforms(6, 0, m.n_op, m.ltrot, 0)
    o = oracle.Oracle(m, ltau=1)
    o.set_fields(f0)
    o.init_state()
    _, tau_o = o.collect_measurements()
    o.sweep(u)
    g = Chains(m, ltau=1)
    g.set_fields(0, f0)
    g.init_state()
    _, tau_g = g.sweep(u[None, :], measure=True)
    so = o.stats()
    band = max(1e-10, 10.0 * so.xmax_tau)
    assert len(tau_g) == len(tau_o) == m.ltrot + 1
    for (c, nt, qg, _), (nt_o, qo, _) in zip(tau_g, tau_o):
        for k in range(4):
            assert np.max(np.abs(qg[k] - qo[k])) <= band, (nt, k)


def test_kondo_with_f_interaction_parity():
    # ham_Uf = 2 (the reference default): the U_f vertex of each f orbital is a rank-one vector
    # vertex on its c-f pair in the J_K eigenbasis; the sweep runs its phases (all U_f vertices,
    # then all J_K vertices) with explicit wraps.  Against the oracle, which rotates around
    # every vertex as Op_Wrapup / Op_Wrapdo do.
    _run_pair(_kondo(2, Uf=2.0), seed=5, sweeps=3)
    _run_pair(_kondo(4, beta=2.0, nwrap=10, Uf=2.0), seed=8, sweeps=2)


def test_kondo_with_f_interaction_tau_m_and_mixed_form():
    m = _kondo(2, Uf=2.0)
    f0 = rng.initial_fields(6, 0, m.n_op, m.ltrot)
    u = rng.sweep_uniforms(6, 0, m.n_op, m.ltrot, 0)
    o = oracle.Oracle(m, ltau=1)
    o.set_fields(f0)
    o.init_state()
    _, tau_o = o.collect_measurements()
    o.sweep(u)
    so = o.stats()
    for precision, tol in (("fp64", max(1e-10, 10.0 * so.xmax_tau)), ("mixed", 1e-5)):
        g = Chains(m, ltau=1, precision=precision)
        g.set_fields(0, f0)
        g.init_state()
        _, tau_g = g.sweep(u[None, :], measure=True)
        np.testing.assert_array_equal(g.fields(0), o.fields())
        assert abs(g.phase()[0] - o.phase()) < (1e-10 if precision == "fp64" else 1e-6)
        assert len(tau_g) == len(tau_o) == m.ltrot + 1
        for (c, nt, qg, _), (nt_o, qo, _) in zip(tau_g, tau_o):
            for k in range(4):
                assert np.max(np.abs(qg[k] - qo[k])) <= tol, (precision, nt, k)
        g.close()
