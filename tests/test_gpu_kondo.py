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


def test_kondo_with_f_interaction_is_rejected():
    # U_f vertices act on single f orbitals, which are not diagonal in the J_K eigenbasis
    with pytest.raises(_lib.AlfGpuError):
        Chains(_kondo(2, Uf=2.0))
