"""Device-side lattice-resolved observables (alfgpu_set_lattice_obs) against the host
restatement of the predefined measurements (alf_gb300.lattice_obs: EqualTimeObs and
TimeDisplacedObs, which follow Predefined_Obs_mod.F90:137-600) fed the same sweep's
ham%Obser / ham%ObserT callbacks.  Same G, different summation order: the bins agree to
1e-10 relative to their largest entry."""
import numpy as np
import pytest

from alf_gb300 import lattice_obs as lo, model as mdl, rng
from alf_gb300.sweep import Chains

pytestmark = pytest.mark.gpu

TOL = 1e-10


def _close(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return np.max(np.abs(a - b)) <= TOL * max(1.0, np.max(np.abs(b)))


def _compare(m, latt, ltau, precision="fp64", seed=3, sweeps=2):
    g = Chains(m, ltau=ltau, precision=precision)
    g.set_fields(0, rng.initial_fields(seed, 0, m.n_op, m.ltrot))
    g.init_state()
    g.set_lattice_obs(latt)
    eq_h = lo.EqualTimeObs(latt, n_sun=m.n_sun, n_fl=m.n_fl)
    tau_h = lo.TimeDisplacedObs(latt, n_sun=m.n_sun, ntau=m.ltrot + 1, n_fl=m.n_fl) if ltau else None
    for s in range(sweeps):
        eq, tau = g.sweep(rng.sweep_uniforms(seed, 0, m.n_op, m.ltrot, s)[None, :], measure=True)
        for c, nt, G, ph in eq:
            eq_h.measure(G, ph)
        for c, nt, q, ph in tau:
            tau_h.measure(nt, *q, ph)
    bd, bh = g.lattice_bin(0, 0), eq_h.bin()
    assert set(bd) == set(bh) == set(lo.names_for(m.n_fl))
    for k in bh:
        assert bd[k]["latt"].shape == bh[k]["latt"].shape
        assert _close(bd[k]["latt"], bh[k]["latt"]), k
        assert _close(bd[k]["latt0"], bh[k]["latt0"]), k
        assert bd[k]["sign"] == bh[k]["sign"]
    assert g.lattice_obs(0, 0)["count"] == sweeps * (2 * m.ltrot - 1)
    if ltau:
        td, th = g.lattice_bin(0, 1), tau_h.bin()
        for k in th:
            assert td[k]["latt"].shape == th[k]["latt"].shape == (latt.N, m.ltrot + 1, latt.norb, latt.norb)
            assert _close(td[k]["latt"], th[k]["latt"]), k
            assert _close(td[k]["latt0"], th[k]["latt0"]), k
        assert g.lattice_obs(0, 1)["count"] == sweeps
    return g


def test_square_hubbard_equal_time():
    m = mdl.hubbard("square", 4, 4, U=4.0, beta=1.0, dtau=0.1, nwrap=5)
    g = _compare(m, lo.Lattice("square", 4, 4), ltau=0)
    # without a callback the sweep replays its CUDA graph: the device still measures every slice
    g.reset_lattice_obs()
    g.set_rng(0, 7, rng.sweep_counter_base(m.n_op, m.ltrot, 5))
    g.sweep(None)
    assert g.lattice_obs(0, 0)["count"] == 2 * m.ltrot - 1


def test_honeycomb_hubbard_equal_time_and_tau():
    m = mdl.hubbard("honeycomb", 3, 3, U=5.0, beta=0.5, dtau=0.05, nwrap=5)
    _compare(m, lo.Lattice("honeycomb", 3, 3), ltau=1)


def test_honeycomb_hubbard_mixed_form():
    m = mdl.hubbard("honeycomb", 3, 3, U=5.0, beta=0.5, dtau=0.05, nwrap=5)
    _compare(m, lo.Lattice("honeycomb", 3, 3), ltau=1, precision="mixed")


def test_kondo_bilayer_single_flavour():
    m = mdl.kondo(2, 2, JK=1.5, Uf=0.0, beta=1.0, dtau=0.1, nwrap=5)
    _compare(m, lo.Lattice("bilayer_square", 2, 2), ltau=1)
