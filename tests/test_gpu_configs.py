"""GPU parity at the benchmark configurations' own sizes, through the C ABI, against the
CPU oracle on the same fields and draws.

* 4x4 Hubbard, beta = 4 (the small configuration exactly): identical accept sequence
  over 20 sweeps; 10 bins x 20 sweeps of the scalar observables equal to the oracle's on
  the same draws, and within jackknife error bars of an independent oracle chain.
* the batch of Hubbard chains: one handle per (N_dim, Ltrot) group, the N_dim = 36 and
  N_dim = 256 groups at the Nwrap the drift control chose, mixed form.
* 12x12 honeycomb, beta = 20, dtau = 0.05, Nwrap = 5 (N_dim = 288, 80 stabilisations,
  TAU_M with CGR2_2 on 2N = 576): one sweep in both forms.
* Kondo bilayer 12x12 (N_dim = 288, N_FL = 1, N_SUN = 2, ham_Uf = 0, TAU_M): two chains of
  a 32-chain handle, each against its own oracle run, in both forms.

Tolerances: FP64 form as tests/test_gpu_parity.py (G at every stabilisation point and the
phase within 1e-10 relative, ratios median <= 1e-12 and max <= max(1e-10, 10 S) with S the
oracle's own build-to-build spread, identical accept sequence); TAU_M quartets within
max(1e-10, 10 x the oracle's Control_Precision_tau).  Mixed form: |G_mixed - G_oracle|
<= 1e-5 at every stabilisation point before the accept sequences part (they may part
only at a draw within rounding of its weight, and at least one point must be
compared), Precision Green <= 1e-5, quartets within 1e-5 when the sequences agree.
"""
import os

import numpy as np
import pytest

import oracle
from alf_gb300 import bins, model as mdl, replicas, rng
from alf_gb300.sweep import Chains
from parity_util import compare_record, relmax
from test_gpu_parity import _run_pair

pytestmark = pytest.mark.gpu

THREADS = os.cpu_count() or 1
RTOL = 1e-10
BOUND = 1e-5


# ---------------------------------------------------------------------------------------------
# 4x4 Hubbard, beta = 4: 20 sweeps, and 10 bins x 20 sweeps of observables
# ---------------------------------------------------------------------------------------------
def test_small_config_twenty_sweeps_identical_accept_sequence():
    g, o = _run_pair(mdl.config("hubbard4x4"), seed=17, sweeps=20)
    assert g.stats(0).n_acc > 0


def _scalar_bins(run_sweep, get_sums, reset, nbins, nsweeps):
    out = []
    for _ in range(nbins):
        for _ in range(nsweeps):
            run_sweep()
        out.append(bins.walker_mean([bins.bin_from_sums(get_sums())]))
        reset()
    return np.array([b[0] for b in out]), np.array([b[1] for b in out])


def test_small_config_observables_ten_bins_of_twenty_sweeps():
    m = mdl.config("hubbard4x4")
    H = mdl.hopping_matrix("square", 4, 4).real
    Hs, U = np.stack([H, H]), np.full(m.ndim, 4.0)
    nb, ns = 10, 20
    # same fields and draws on both sides: the bins agree to rounding
    seed = 790789
    o = oracle.Oracle(m)
    o.set_fields(rng.initial_fields(seed, 0, m.n_op, m.ltrot))
    o.init_state()
    o.set_scalar_obs(Hs, U)
    g = Chains(m)
    g.set_fields(0, rng.initial_fields(seed, 0, m.n_op, m.ltrot))
    g.init_state()
    g.set_scalar_obs(Hs, U)
    k = {"o": 0, "g": 0}

    def step_o():
        o.sweep(rng.sweep_uniforms(seed, 0, m.n_op, m.ltrot, k["o"]))
        k["o"] += 1

    def step_g():
        g.sweep(rng.sweep_uniforms(seed, 0, m.n_op, m.ltrot, k["g"])[None, :])
        k["g"] += 1

    bo, so = _scalar_bins(step_o, lambda: o.scalar_obs(reset=False), lambda: o.scalar_obs(reset=True), nb, ns)
    bg, sg = _scalar_bins(step_g, lambda: g.scalar_obs(0), g.reset_scalar_obs, nb, ns)
    np.testing.assert_array_equal(g.fields(0), o.fields())
    assert np.max(np.abs(bg - bo)) <= 1e-9 * np.max(np.abs(bo)), np.max(np.abs(bg - bo))
    np.testing.assert_allclose(sg, so, rtol=0, atol=1e-12)
    rg, _ = bins.ana_vec(bg, sg)
    ro, _ = bins.ana_vec(bo, so)
    for (mg, eg), (mo, eo) in zip(rg, ro):
        # Part is exactly N at half filling: its jackknife error is itself rounding
        floor = 1e-9 * max(1.0, abs(mo))
        assert abs(mg - mo) <= floor and abs(eg - eo) <= 1e-7 * eo + floor, (mg, mo, eg, eo)
    # an independent chain (the GPU's own device draw stream, another seed) against the
    # oracle's bins: the jackknife means agree within the combined error bars
    g2 = Chains(m)
    seed2 = 452938
    g2.set_fields(0, rng.initial_fields(seed2, 0, m.n_op, m.ltrot))
    g2.init_state()
    g2.set_rng(0, seed2, rng.sweep_counter_base(m.n_op, m.ltrot, 0))
    g2.set_scalar_obs(Hs, U)
    b2, s2 = _scalar_bins(lambda: g2.sweep(None), lambda: g2.scalar_obs(0), g2.reset_scalar_obs, nb, ns)
    r2, _ = bins.ana_vec(b2, s2)
    for name, (m2, e2), (mo, eo) in zip(bins.HUBBARD_SCALARS, r2, ro):
        # Part is exactly N at half filling: its error bar is rounding, so floor it there
        z = abs(m2 - mo) / max(np.hypot(e2, eo), 1e-9 * max(1.0, abs(mo)))
        print(f"{name}: GPU {m2:.4f} +- {e2:.4f}, oracle {mo:.4f} +- {eo:.4f}, z = {z:.2f}")
        assert z < 4.0, (name, m2, e2, mo, eo)
    for h in (g, g2):
        h.close()


# ---------------------------------------------------------------------------------------------
# the batched Hubbard chains: two (N_dim, Ltrot) groups at their adapted Nwrap
# ---------------------------------------------------------------------------------------------
def test_batched_groups_at_adapted_nwrap_mixed():
    groups = mdl.batch_groups(replicas.replica_seed(1, 0))
    picked = [min((k for k in groups if k[0] == 6), key=lambda k: -len(groups[k])),
              min((k for k in groups if k[0] == 16), key=lambda k: -len(groups[k]))]
    for (L, beta) in picked:
        members = groups[(L, beta)]
        models = [mdl.hubbard("square", L, L, U=U, beta=beta, dtau=0.1, nwrap=10) for _, U in members]
        C = len(members)
        g = Chains(models[0], n_chains=C, precision="mixed", models=models)
        seeds = [replicas.replica_seed(1, 0, c) for c, _ in members]
        for k in range(C):
            g.set_fields(k, rng.initial_fields(seeds[k], k, models[0].n_op, models[0].ltrot))
        g.init_state()
        for k in range(C):
            g.set_rng(k, seeds[k], rng.sweep_counter_base(models[0].n_op, models[0].ltrot, 0))
        nw, worst = g.adapt_nwrap(bound=BOUND)
        assert worst <= BOUND, (L, beta, nw, worst)
        # from the adapted chains' fields: one sweep on host draws, recorded
        g.init_state()
        g.set_recording(True)
        us = np.stack([rng.sweep_uniforms(seeds[k], k, models[0].n_op, models[0].ltrot, 99) for k in range(C)])
        fields = [g.fields(k) for k in range(C)]
        g.sweep(us)
        for k in sorted({0, C - 1}):
            mk = mdl.hubbard("square", L, L, U=members[k][1], beta=beta, dtau=0.1, nwrap=nw)
            o = oracle.Oracle(mk, threads=THREADS)
            o.set_fields(fields[k])
            o.init_state()
            o.record(1)
            o.sweep(us[k])
            res = compare_record(g.record(k), o.recorded(), us[k], mk.n_op, mk.ltrot, nw, g_tol=BOUND,
                                 relative=False, exact_sequence=False, ratio_median=1e-5)
            print(f"L={L} beta={beta} chains={C} Nwrap={nw} chain {k}: {res}")
            assert g.stats(k).xmaxG <= BOUND
        g.close()


# ---------------------------------------------------------------------------------------------
# 12x12 honeycomb, beta = 20, TAU_M every sweep
# ---------------------------------------------------------------------------------------------
def _keep_every(step, last):
    pts = set(range(0, last + 1, step)) | {1, last}
    return lambda nt: nt in pts


class _OracleSweep:
    """One recorded oracle sweep (G at every stabilisation point, ratios, accept bits) with
    a subset of its measurement callbacks, and the ratio spread S of a second build."""

    def __init__(self, m, f0, u, ltau, keep_eq, keep_tau, spread=True):
        if spread:
            oracle.set_variant(1)
            try:
                ov = oracle.Oracle(m, ltau=0, threads=THREADS)
                ov.set_fields(f0)
                ov.init_state()
                ov.record(1, green=False)
                ov.sweep(u)
                rv = ov.recorded()["ratio"].copy()
                del ov
            finally:
                oracle.set_variant(0)
        o = oracle.Oracle(m, ltau=ltau, threads=THREADS)
        o.set_fields(f0)
        self.phase0 = o.init_state()
        self.G0 = o.green()
        self.eq, self.tau = o.collect_measurements(
            keep=lambda kind, nt: keep_eq(nt) if kind == 0 else keep_tau(nt))
        o.record(1)
        o.sweep(u)
        self.rec = o.recorded()
        self.fields = o.fields()
        self.green = o.green()
        self.phase = o.phase()
        self.stats = o.stats()
        r = self.rec["ratio"]
        prop = np.abs(r) > 0
        self.spread = float(np.max(np.abs(rv[prop] - r[prop]) / np.abs(r[prop]))) if spread else None
        del o


def _check_tau(tau_g, tau_o, tol):
    assert [t[1] for t in tau_g] == [t[0] for t in tau_o] and tau_o
    worst = 0.0
    for (c, nt, qg, _), (nt_o, qo, _) in zip(tau_g, tau_o):
        for k in range(4):
            d = float(np.max(np.abs(qg[k] - qo[k])))
            worst = max(worst, d)
            assert d <= tol, (nt, k, d, tol)
    return worst


@pytest.fixture(scope="module")
def honeycomb_run():
    m = mdl.config("honeycomb12x12")
    seed = 3
    f0 = rng.initial_fields(seed, 0, m.n_op, m.ltrot)
    u = rng.sweep_uniforms(seed, 0, m.n_op, m.ltrot, 0)
    keep_eq = _keep_every(100, m.ltrot)
    keep_tau = _keep_every(40, m.ltrot)
    return m, f0, u, keep_eq, keep_tau, _OracleSweep(m, f0, u, 1, keep_eq, keep_tau)


def test_honeycomb12x12_beta20_fp64_parity_with_tau_m(honeycomb_run):
    m, f0, u, keep_eq, keep_tau, ro = honeycomb_run
    g = Chains(m, ltau=1)
    g.set_fields(0, f0)
    assert abs(g.init_state()[0] - ro.phase0) < 1e-10
    assert relmax(g.green(0), ro.G0) < RTOL
    g.set_recording(True)
    eq_g, tau_g = g.sweep(u[None, :], measure=True,
                          keep=lambda kind, c, nt: keep_eq(nt) if kind == 0 else keep_tau(nt))
    res = compare_record(g.record(0), ro.rec, u, m.n_op, m.ltrot, m.nwrap, g_tol=RTOL, relative=True,
                         exact_sequence=True, ratio_median=1e-12, ratio_tol=max(RTOL, 10.0 * ro.spread))
    np.testing.assert_array_equal(g.fields(0), ro.fields)
    assert relmax(g.green(0), ro.green) < RTOL
    assert abs(g.phase()[0] - ro.phase) < 1e-10
    sg, so = g.stats(0), ro.stats
    # Control_Precision_tau compares four blocks per flavour at each of the Nstm CGR2_2 points
    assert sg.n_acc == so.n_acc and sg.ncg_tau == so.ncg_tau == 4 * m.n_fl * m.nstm
    band = max(1e-10, 10.0 * so.xmax_tau)
    assert sg.xmax_tau <= band
    wq = _check_tau(tau_g, ro.tau, band)
    band_eq = max(1e-10, 10.0 * so.xmaxG)
    assert [e[1] for e in eq_g] == [e[0] for e in ro.eq]
    for (c, nt, Gg, phg), (nt_o, Go, pho) in zip(eq_g, ro.eq):
        assert np.max(np.abs(Gg - Go)) <= band_eq, nt
        assert abs(phg - pho) < 1e-10
    print(f"honeycomb 12x12 beta 20 FP64: {res}; ratio spread S = {ro.spread:.2e}; oracle Precision Green "
          f"{so.xmaxG:.2e}, Precision_tau {so.xmax_tau:.2e}; worst quartet deviation {wq:.2e}")
    g.close()


def test_honeycomb12x12_beta20_mixed_vs_fp64_oracle(honeycomb_run):
    m, f0, u, keep_eq, keep_tau, ro = honeycomb_run
    g = Chains(m, ltau=1, precision="mixed")
    g.set_fields(0, f0)
    g.init_state()
    assert np.max(np.abs(g.green(0) - ro.G0)) < BOUND
    g.set_recording(True)
    _, tau_g = g.sweep(u[None, :], measure=True, keep=lambda kind, c, nt: kind == 1 and keep_tau(nt))
    res = compare_record(g.record(0), ro.rec, u, m.n_op, m.ltrot, m.nwrap, g_tol=BOUND, relative=False,
                         exact_sequence=False, ratio_median=1e-6)
    st = g.stats(0)
    assert st.xmaxG <= BOUND, st.xmaxG
    wq = None
    if res["parting_visit"] is None:
        np.testing.assert_array_equal(g.fields(0), ro.fields)
        wq = _check_tau(tau_g, ro.tau, BOUND)
        assert st.xmax_tau <= BOUND
    print(f"honeycomb 12x12 beta 20 mixed: {res}; Precision Green {st.xmaxG:.2e}, Precision_tau "
          f"{st.xmax_tau:.2e}; worst quartet deviation {wq}")
    g.close()


# ---------------------------------------------------------------------------------------------
# Kondo bilayer 12x12: two chains of a 32-chain handle
# ---------------------------------------------------------------------------------------------
KONDO_CHAINS = 32
KONDO_PICK = (0, 31)


@pytest.fixture(scope="module")
def kondo_runs():
    m = mdl.kondo(12, 12, JK=1.5, Uf=0.0, beta=10.0, dtau=0.1, nwrap=10)
    seeds = [replicas.replica_seed(5, 0, c) for c in range(KONDO_CHAINS)]
    fs = [rng.initial_fields(seeds[c], c, m.n_op, m.ltrot) for c in range(KONDO_CHAINS)]
    us = np.stack([rng.sweep_uniforms(seeds[c], c, m.n_op, m.ltrot, 0) for c in range(KONDO_CHAINS)])
    keep_eq = _keep_every(50, m.ltrot)
    keep_tau = _keep_every(20, m.ltrot)
    ors = {c: _OracleSweep(m, fs[c], us[c], 1, keep_eq, keep_tau) for c in KONDO_PICK}
    return m, fs, us, keep_eq, keep_tau, ors


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_kondo12x12_two_chains_of_a_32_chain_handle(kondo_runs, precision):
    m, fs, us, keep_eq, keep_tau, ors = kondo_runs
    g = Chains(m, n_chains=KONDO_CHAINS, ltau=1, precision=precision)
    for c in range(KONDO_CHAINS):
        g.set_fields(c, fs[c])
    g.init_state()
    g.set_recording(True)
    _, tau_g = g.sweep(us, measure=True, keep=lambda kind, c, nt: kind == 1 and c in KONDO_PICK and keep_tau(nt))
    for c in KONDO_PICK:
        ro = ors[c]
        tq = [t for t in tau_g if t[0] == c]
        if precision == "fp64":
            res = compare_record(g.record(c), ro.rec, us[c], m.n_op, m.ltrot, m.nwrap, g_tol=RTOL, relative=True,
                                 exact_sequence=True, ratio_median=1e-12,
                                 ratio_tol=max(RTOL, 10.0 * ro.spread))
            np.testing.assert_array_equal(g.fields(c), ro.fields)
            assert relmax(g.green(c), ro.green) < RTOL
            band = max(1e-10, 10.0 * ro.stats.xmax_tau)
            wq = _check_tau(tq, ro.tau, band)
        else:
            res = compare_record(g.record(c), ro.rec, us[c], m.n_op, m.ltrot, m.nwrap, g_tol=BOUND,
                                 relative=False, exact_sequence=False, ratio_median=1e-6)
            assert g.stats(c).xmaxG <= BOUND
            wq = None
            if res["parting_visit"] is None:
                wq = _check_tau(tq, ro.tau, BOUND)
        print(f"Kondo 12x12 {precision} chain {c}: {res}; ratio spread S = {ro.spread:.2e}; worst quartet "
              f"deviation {wq}")
    g.close()
