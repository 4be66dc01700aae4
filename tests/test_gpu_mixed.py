"""Mixed-precision form against the FP64 CPU oracle on the same fields and draws.  The form:
complex128 storage; G wraps, UDV propagation and the stabilisation's complex products as
digit-sliced BF16 tensor-core products (FP64-accurate); on grids of several chains the
delayed-update flush and the explicit Q on the tensor cores too; the per-visit Metropolis
arithmetic in double-float with the ratio and phase accumulated in FP64; pivoted QRs,
triangular solves and phases in FP64.

Acceptance bound: max |G_mixed - G_fp64| <= 1e-5 at every stabilisation point
(the freshly computed CGR result) while the accept/reject sequences agree, and
the mixed form's own Precision Green (max |G_wrapped - G_fresh|) <= 1e-5.
"""
import numpy as np
import pytest

import oracle
from alf_gb300 import model as mdl, rng
from alf_gb300.sweep import (FLAG_DF_FLUSH, FLAG_FP64_VISITS, FLAG_OZ_DEEP_RING, FLAG_OZ_FLUSH_RESIDENT,
                             FLAG_OZ_FLUSH_SINGLE, FLAG_TENSOR_WIDE, Chains)
from parity_util import compare_record

pytestmark = pytest.mark.gpu

BOUND = 1e-5


def _compare(m, seed, sweeps, flags=0):
    """Worst |G_mixed - G_oracle| over the stabilisation points of `sweeps` sweeps; stops at
    the sweep where the accept sequences part (only at a draw within rounding of its
    weight), after comparing the points before the parting visit.  At least one point must
    be compared."""
    f0 = rng.initial_fields(seed, 0, m.n_op, m.ltrot)
    o = oracle.Oracle(m)
    o.set_fields(f0)
    o.init_state()
    g = Chains(m, precision="mixed", flags=flags)
    g.set_fields(0, f0)
    g.init_state()
    assert np.max(np.abs(g.green(0) - o.green())) < BOUND
    g.set_recording(True)
    worst, compared, parted = 0.0, 0, False
    for s in range(sweeps):
        u = rng.sweep_uniforms(seed, 0, m.n_op, m.ltrot, s)
        o.record(1)
        o.sweep(u)
        g.sweep(u[None, :])
        res = compare_record(g.record(0), o.recorded(), u, m.n_op, m.ltrot, m.nwrap, g_tol=BOUND, relative=False,
                             exact_sequence=False, ratio_median=1e-5)
        worst = max(worst, res["worst_dG"])
        compared += res["points_compared"]
        if res["parting_visit"] is not None:
            parted = True
            break
    assert compared >= 1
    st = g.stats(0)
    assert st.xmaxG <= BOUND
    if not parted:
        assert np.array_equal(g.fields(0), o.fields())
    return worst


def test_mixed_hubbard_4x4_vs_fp64_oracle():
    w = _compare(mdl.config("hubbard4x4"), seed=5, sweeps=3)
    assert w < BOUND


def test_mixed_hubbard_8x8_vs_fp64_oracle():
    m = mdl.hubbard("square", 8, 8, U=4.0, beta=4.0, dtau=0.1, nwrap=10)
    w = _compare(m, seed=2, sweeps=1)
    assert w < BOUND


def test_mixed_honeycomb_vs_fp64_oracle():
    m = mdl.hubbard("honeycomb", 3, 3, U=5.0, beta=2.0, dtau=0.05, nwrap=5)
    w = _compare(m, seed=3, sweeps=2)
    assert w < BOUND


def test_mixed_hubbard_16x16_vs_fp64_oracle():
    # the 16x16 (N_dim = 256) beta = 10 configuration, one sweep: 20 stabilisation points
    w = _compare(mdl.config("hubbard16x16"), seed=1, sweeps=1)
    assert w < BOUND


def test_mixed_double_float_stabilisation_small():
    # opt-in double-float QR and stabilisation products (scale-free column factoring)
    from alf_gb300.sweep import FLAG_DF_STAB
    w = _compare(mdl.hubbard("square", 8, 8, U=4.0, beta=4.0, dtau=0.1, nwrap=10), seed=2, sweeps=1,
                 flags=FLAG_DF_STAB)
    assert w < BOUND


def test_mixed_double_float_wraps_small():
    # the double-float G wraps and flushes on the FP32 pipes (instead of the tensor-core GEMM)
    from alf_gb300.sweep import FLAG_NO_TENSOR_GEMM
    w = _compare(mdl.hubbard("square", 8, 8, U=4.0, beta=4.0, dtau=0.1, nwrap=10), seed=2, sweeps=1,
                 flags=FLAG_NO_TENSOR_GEMM)
    assert w < BOUND


def test_mixed_kondo_bilayer_vs_fp64_oracle():
    # two-site J_K vertices in their shared eigenbasis, tensor-core wraps in that basis
    m = mdl.kondo(4, 4, JK=1.5, Uf=0.0, beta=2.0, dtau=0.1, nwrap=10)
    w = _compare(m, seed=8, sweeps=1)
    assert w < BOUND


def test_mixed_tau_m_quartets_vs_fp64_oracle():
    # TAU_M propagation in the mixed form (tensor-core hopping products): every quartet
    # [GT0, G0T, G00, GTT] within 1e-5 of the FP64 oracle's.  TAU_M runs after the sweep, so
    # it is compared on a draw stream whose accept sequence agrees with the oracle's (a
    # sequence may part only at a draw within rounding of its weight; then the next seed is
    # taken); at least one sweep must be compared.
    m = mdl.hubbard("honeycomb", 3, 3, U=5.0, beta=1.0, dtau=0.05, nwrap=5)
    compared = 0
    for seed in (3, 4, 5, 6):
        f0 = rng.initial_fields(seed, 0, m.n_op, m.ltrot)
        u = rng.sweep_uniforms(seed, 0, m.n_op, m.ltrot, 0)
        o = oracle.Oracle(m, ltau=1)
        o.set_fields(f0)
        o.init_state()
        _, tau_o = o.collect_measurements()
        o.record(1, green=False)
        o.sweep(u)
        g = Chains(m, precision="mixed", ltau=1)
        g.set_fields(0, f0)
        g.init_state()
        g.set_recording(True)
        _, tau_g = g.sweep(u[None, :], measure=True)
        rg, ro = g.record(0), o.recorded()
        if not np.array_equal(rg["acc"], ro["acc"]):
            v = int(np.argmax(rg["acc"] != ro["acc"]))
            w = abs(ro["ratio"][v])
            assert abs(w - u[3 * v + 2]) < 1e-4 * max(w, 1.0), (seed, v)
            continue
        assert np.array_equal(g.fields(0), o.fields())
        assert len(tau_g) == len(tau_o) == m.ltrot + 1
        for (c, nt, qg, _), (nt_o, qo, _) in zip(tau_g, tau_o):
            for k in range(4):
                assert np.max(np.abs(qg[k] - qo[k])) <= BOUND, (nt, k)
        compared += 1
        break
    assert compared == 1


@pytest.mark.parametrize("flags", [0, FLAG_TENSOR_WIDE, FLAG_TENSOR_WIDE | FLAG_DF_FLUSH,
                                   FLAG_TENSOR_WIDE | FLAG_OZ_FLUSH_SINGLE, FLAG_TENSOR_WIDE | FLAG_FP64_VISITS,
                                   FLAG_TENSOR_WIDE | FLAG_OZ_DEEP_RING],
                         ids=["default", "wide", "wide-df-flush", "wide-flush-single", "wide-fp64-visits",
                              "wide-deep-ring"])
def test_mixed_batched_chains_with_own_couplings_vs_oracle(flags):
    # one handle, two chains with different U (per-chain vertex tables): each within 1e-5 of
    # its own FP64 oracle run; "wide": the grid takes the batched-grid choices (flush on the
    # tensor cores, compact-WY explicit Q); "wide-df-flush": the same with the double-float flush;
    # "wide-flush-single": the K = 64 products on 16-wide tiles, two CTAs per SM; "wide-fp64-visits":
    # the visits, block updates and flush operands in FP64; "wide-deep-ring": the K = N products on
    # 16-wide tiles with the deeper A ring
    ms = [mdl.hubbard("square", 6, 6, U=U, beta=2.0, dtau=0.1, nwrap=10) for U in (3.0, 7.0)]
    seeds = (12, 13)
    g = Chains(ms[0], n_chains=2, precision="mixed", models=ms, flags=flags)
    for c in range(2):
        g.set_fields(c, rng.initial_fields(seeds[c], c, ms[c].n_op, ms[c].ltrot))
    g.init_state()
    us = np.stack([rng.sweep_uniforms(seeds[c], c, ms[c].n_op, ms[c].ltrot, 0) for c in range(2)])
    g.set_recording(True)
    g.sweep(us)
    for c in range(2):
        o = oracle.Oracle(ms[c])
        o.set_fields(rng.initial_fields(seeds[c], c, ms[c].n_op, ms[c].ltrot))
        o.init_state()
        o.record(1)
        o.sweep(us[c])
        res = compare_record(g.record(c), o.recorded(), us[c], ms[c].n_op, ms[c].ltrot, ms[c].nwrap, g_tol=BOUND,
                             relative=False, exact_sequence=False, ratio_median=1e-5)
        if res["parting_visit"] is None:
            np.testing.assert_array_equal(g.fields(c), o.fields())
            assert np.max(np.abs(g.green(c) - o.green())) < BOUND, c


def test_mixed_wide_grid_paths_vs_fp64_oracle():
    # the batched-grid choices on one chain: 32-wide tiles, the flush on the tensor cores and
    # the explicit Q in compact-WY form (Gram matrix, ZLARFT, rank-32 digit-sliced updates)
    from alf_gb300.sweep import FLAG_TENSOR_WIDE
    w = _compare(mdl.hubbard("square", 8, 8, U=4.0, beta=4.0, dtau=0.1, nwrap=10), seed=2, sweeps=2,
                 flags=FLAG_TENSOR_WIDE)
    assert w < BOUND
    w = _compare(mdl.config("hubbard16x16"), seed=1, sweeps=1, flags=FLAG_TENSOR_WIDE)
    assert w < BOUND


@pytest.mark.parametrize("flags", [0, FLAG_OZ_FLUSH_RESIDENT], ids=["paired-tiles", "resident-a"])
def test_mixed_persistent_k64_products_vs_oracle(flags):
    # four 16x16 chains: the flush and the compact-WY updates (K = 64) have more output tiles than
    # the persistent grid, so each CTA loops over tiles (paired 16-wide tiles by default; with
    # the resident option one CTA per SM keeps a tile's A slices for the next tiles)
    m = mdl.hubbard("square", 16, 16, U=4.0, beta=2.0, dtau=0.1, nwrap=10)
    C, seed = 4, 21
    g = Chains(m, n_chains=C, precision="mixed", flags=flags)
    fs = [rng.initial_fields(seed + c, c, m.n_op, m.ltrot) for c in range(C)]
    for c in range(C):
        g.set_fields(c, fs[c])
    g.init_state()
    us = np.stack([rng.sweep_uniforms(seed + c, c, m.n_op, m.ltrot, 0) for c in range(C)])
    g.set_recording(True)
    g.sweep(us)
    compared = 0
    for c in range(C):
        o = oracle.Oracle(m)
        o.set_fields(fs[c])
        o.init_state()
        o.record(1)
        o.sweep(us[c])
        res = compare_record(g.record(c), o.recorded(), us[c], m.n_op, m.ltrot, m.nwrap, g_tol=BOUND,
                             relative=False, exact_sequence=False, ratio_median=1e-5)
        compared += res["points_compared"]
        if res["parting_visit"] is None:
            np.testing.assert_array_equal(g.fields(c), o.fields())
            assert np.max(np.abs(g.green(c) - o.green())) < BOUND, c
    assert compared >= C
