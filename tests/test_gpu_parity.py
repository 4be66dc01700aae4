"""GPU parity tests: the CUDA path (called through the C ABI) against the CPU oracle.

Tolerances for the plain complex128 form:
* identical accept/reject sequence and final fields from the same draws;
* G at every stabilisation point (the freshly computed CGR result) and the
  phase within 1e-10 relative;
* Metropolis ratios: median relative deviation <= 1e-12, and the maximum
  within max(1e-10, 10 x S), where S is the largest ratio deviation between two
  valid builds of the reference itself (the oracle with OpenBLAS vs. the oracle
  with another summation order of the hopping products), measured in the same
  test on the same draws.  Ratios are computed from the wrapped G, whose
  rounding drift between stabilisations (ALF's "Precision Green", ~1e-8 here)
  amplifies reordered roundings at ill-conditioned visits, so a fixed 1e-10 is
  below the reference's own build-to-build reproducibility (1.9e-9 measured on
  the 4x4 configuration).
All tests run on cuda:0.
"""
import numpy as np
import pytest

import oracle
from alf_gb300 import model as mdl, rng
from alf_gb300.sweep import FLAG_QR_GLOBAL_ROWS, FLAG_QR_HALF_CLUSTER, FLAG_QR_TWO_PASS, Chains, cgr as gpu_cgr, decompose as gpu_decompose

pytestmark = pytest.mark.gpu

RTOL = 1e-10


def _relmax(a, b):
    return np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300)


def test_decompose_matches_oracle_and_reconstructs():
    rs = np.random.default_rng(4782347)
    N = 32
    for side in ("r", "l"):
        U, D, V = np.eye(N, dtype=complex), np.ones(N, complex), np.eye(N, dtype=complex)
        Uo, Do, Vo = U.copy(), D.copy(), V.copy()
        P = np.eye(N, dtype=complex)
        for _ in range(6):
            X = rs.standard_normal((N, N)) + 1j * rs.standard_normal((N, N))
            U, Uo, P = X @ U, X @ Uo, X @ P
            U, D, V = gpu_decompose(side, U, D, V)
            Uo, Do, Vo = oracle.decompose(side, Uo, Do, Vo)
            R = U @ np.diag(D) @ (V if side == "r" else V.conj().T)
            assert _relmax(R, P) < 1e-10
            assert np.max(np.abs(U.conj().T @ U - np.eye(N))) < 1e-12
            assert _relmax(D, Do) < 1e-10


def test_cgr_matches_naive_15cgr_and_oracle():
    N = 5
    for nvar in (1, 2):
        UR = np.eye(N, dtype=complex)
        UL = np.eye(N, dtype=complex)
        VR = np.array([[complex(i, j) for j in range(1, N + 1)] for i in range(1, N + 1)])
        VL = np.array([[complex(i + j, 0) for j in range(1, N + 1)] for i in range(1, N + 1)])
        for i in range(N):
            VR[i, i] = 1 + 1j
            VL[i, i] = 1 + 1j
        DL = np.ones(N, complex)
        DR = np.arange(1, N + 1).astype(complex)
        G, ph = gpu_cgr(nvar, UR, DR, VR, UL, DL, VL)
        M = np.eye(N) + UR @ np.diag(DR) @ VR @ VL @ np.diag(DL) @ UL.conj().T
        assert _relmax(G, np.linalg.inv(M)) < 1e-10
        d = np.linalg.det(M)
        assert abs(ph - d / abs(d)) < 1e-13
    # random unitary U's and graded D's, against the oracle
    rs = np.random.default_rng(7)
    N = 48
    q = lambda: np.linalg.qr(rs.standard_normal((N, N)) + 1j * rs.standard_normal((N, N)))[0]
    UR, UL = q(), q()
    VR = rs.standard_normal((N, N)) + 1j * rs.standard_normal((N, N))
    VL = rs.standard_normal((N, N)) + 1j * rs.standard_normal((N, N))
    DR = np.exp(np.linspace(8, -8, N)).astype(complex)
    DL = np.exp(np.linspace(6, -6, N)).astype(complex)
    for nvar in (1, 2):
        G, ph = gpu_cgr(nvar, UR, DR, VR, UL, DL, VL)
        Go, pho = oracle.cgr(nvar, UR, DR, VR, UL, DL, VL)
        assert _relmax(G, Go) < 1e-10
        assert abs(ph - pho) < 1e-10


def test_decompose_and_cgr_with_rows_beyond_shared_memory():
    # N_dim = 480: the exact pivoted QR keeps each CTA's 30 rows x 480 columns in a global
    # workspace (they do not fit a 16-CTA cluster's shared memory); same results as the oracle
    rs = np.random.default_rng(480)
    N = 480
    for side in ("r", "l"):
        U, D, V = np.eye(N, dtype=complex), np.ones(N, complex), np.eye(N, dtype=complex)
        Uo, Do, Vo = U.copy(), D.copy(), V.copy()
        P = np.eye(N, dtype=complex)
        for _ in range(2):
            X = rs.standard_normal((N, N)) + 1j * rs.standard_normal((N, N))
            U, Uo, P = X @ U, X @ Uo, X @ P
            U, D, V = gpu_decompose(side, U, D, V)
            Uo, Do, Vo = oracle.decompose(side, Uo, Do, Vo)
            R = U @ np.diag(D) @ (V if side == "r" else V.conj().T)
            assert _relmax(R, P) < 1e-10
            assert np.max(np.abs(U.conj().T @ U - np.eye(N))) < 1e-12
            assert _relmax(D, Do) < 1e-10
    q = lambda: np.linalg.qr(rs.standard_normal((N, N)) + 1j * rs.standard_normal((N, N)))[0]
    UR, UL = q(), q()
    VR = rs.standard_normal((N, N)) + 1j * rs.standard_normal((N, N))
    VL = rs.standard_normal((N, N)) + 1j * rs.standard_normal((N, N))
    DR = np.exp(np.linspace(8, -8, N)).astype(complex)
    DL = np.exp(np.linspace(6, -6, N)).astype(complex)
    for nvar in (1, 2):
        G, ph = gpu_cgr(nvar, UR, DR, VR, UL, DL, VL)
        Go, pho = oracle.cgr(nvar, UR, DR, VR, UL, DL, VL)
        assert _relmax(G, Go) < 1e-10
        assert abs(ph - pho) < 1e-10


def _variant_ratios(m, f0, seed, sweeps, chain):
    oracle.set_variant(1)
    try:
        o = oracle.Oracle(m)
        o.set_fields(f0)
        o.init_state()
        out = []
        for s in range(sweeps):
            o.record(1)
            o.sweep(rng.sweep_uniforms(seed, chain, m.n_op, m.ltrot, s))
            out.append(o.recorded()["ratio"].copy())
        return out
    finally:
        oracle.set_variant(0)


def _run_pair(m, seed=5, sweeps=1, chain=0, pivoting="default", flags=0):
    f0 = rng.initial_fields(seed, chain, m.n_op, m.ltrot)
    var = _variant_ratios(m, f0, seed, sweeps, chain)
    o = oracle.Oracle(m)
    o.set_fields(f0)
    ph_o = o.init_state()
    g = Chains(m, n_chains=1, pivoting=pivoting, flags=flags)
    g.set_fields(0, f0)
    ph_g = g.init_state()[0]
    assert abs(ph_g - ph_o) < 1e-10
    assert _relmax(g.green(0), o.green()) < RTOL
    g.set_recording(True)
    for s in range(sweeps):
        u = rng.sweep_uniforms(seed, chain, m.n_op, m.ltrot, s)
        o.record(1)
        o.sweep(u)
        ro = o.recorded()
        g.sweep(u[None, :])
        rg = g.record(0)
        np.testing.assert_array_equal(rg["acc"], ro["acc"])
        acc = ro["acc"].astype(bool)
        r_o, r_g = ro["ratio"], rg["ratio"]
        rel = np.abs(r_g - r_o) / np.maximum(np.abs(r_o), 1e-300)
        spread = np.max(np.abs(var[s] - r_o) / np.maximum(np.abs(r_o), 1e-300))
        assert np.median(rel) <= 1e-12, np.median(rel)
        assert rel.max() <= max(RTOL, 10.0 * spread), (rel.max(), spread)
        # wrapped G just before each stabilisation: within 10x the oracle's own drift
        drift = max(np.max(np.abs(ro["Gwrap"][p] - ro["G"][p])) for p in range(ro["G"].shape[0]))
        for p in range(ro["G"].shape[0]):
            assert _relmax(rg["G"][p], ro["G"][p]) < RTOL, (s, p, _relmax(rg["G"][p], ro["G"][p]))
            assert np.max(np.abs(rg["Gwrap"][p] - ro["Gwrap"][p])) <= 10.0 * drift + 1e-12, (s, p)
        np.testing.assert_array_equal(g.fields(0), o.fields())
        assert _relmax(g.green(0), o.green()) < RTOL
        assert abs(g.phase()[0] - o.phase()) < 1e-10
    so, sg = o.stats(), g.stats(0)
    assert sg.n_acc == so.n_acc and sg.n_prop == so.n_prop
    # Precision Green (max |G_wrapped - G_fresh|) is rounding drift: same band as above
    assert sg.xmaxG <= 10.0 * so.xmaxG + 1e-12 and so.xmaxG <= 10.0 * sg.xmaxG + 1e-12
    return g, o


@pytest.mark.parametrize("pivoting", ["default", "norms"])
def test_init_and_sweep_hubbard_4x4_parity(pivoting):
    # the small reference configuration: 4x4 square Hubbard, U=4, beta=4, dtau=0.1, Nwrap=10;
    # the oracle pivots like ZGEQP3: with "norms" only G (not the UDV factors) is comparable
    _run_pair(mdl.config("hubbard4x4"), sweeps=3, pivoting=pivoting)


@pytest.mark.parametrize("pivoting", ["default", "norms"])
def test_sweep_hubbard_8x8_parity(pivoting):
    # 8x8 (N_dim = 64): exact pivoting on a 4-CTA cluster; norm pivoting runs the
    # blocked QR (two panels)
    m = mdl.hubbard("square", 8, 8, U=4.0, beta=2.0, dtau=0.1, nwrap=10)
    _run_pair(m, seed=4, sweeps=1, pivoting=pivoting)


def test_sweep_hubbard_8x8_half_cluster_qr_parity():
    # the exact pivoted QR on clusters of half the default size (2 CTAs of 32 rows each at
    # N_dim = 64), the shape batched grids take when it saves waves
    m = mdl.hubbard("square", 8, 8, U=4.0, beta=2.0, dtau=0.1, nwrap=10)
    _run_pair(m, seed=4, sweeps=1, flags=FLAG_QR_HALF_CLUSTER)


@pytest.mark.parametrize("flags", [FLAG_QR_GLOBAL_ROWS, FLAG_QR_GLOBAL_ROWS | FLAG_QR_HALF_CLUSTER,
                                   FLAG_QR_TWO_PASS, FLAG_QR_GLOBAL_ROWS | FLAG_QR_TWO_PASS],
                         ids=["global-rows", "global-rows-half", "two-pass", "global-rows-two-pass"])
def test_sweep_hubbard_8x8_global_rows_qr_parity(flags):
    # the exact pivoted QR with every CTA's rows in the global workspace although they fit in
    # shared memory (the same arithmetic and order as the shared-memory rows), and with the update
    # and the next step's partial sums in separate passes
    m = mdl.hubbard("square", 8, 8, U=4.0, beta=2.0, dtau=0.1, nwrap=10)
    _run_pair(m, seed=4, sweeps=1, flags=flags)


def test_complex_fields_entry_matches_the_int8_entry():
    # nsigma%f as the Fortran side holds it (complex) gives the same state as the int8 form;
    # a value that is not a discrete field is rejected (ALFGPU_ERROR_FIELDS)
    m = mdl.config("hubbard4x4")
    f0 = rng.initial_fields(3, 0, m.n_op, m.ltrot)
    u = rng.sweep_uniforms(3, 0, m.n_op, m.ltrot, 0)[None, :]
    a, b = Chains(m), Chains(m)
    a.set_fields(0, f0)
    b.set_fields_c128(0, f0.astype(np.complex128))
    for g in (a, b):
        g.init_state()
        g.sweep(u)
    np.testing.assert_array_equal(a.fields(0), b.fields(0))
    assert _relmax(a.green(0), b.green(0)) == 0.0
    bad = f0.astype(np.complex128)
    bad[0, 0] = 1.5
    with pytest.raises(RuntimeError):
        b.set_fields_c128(0, bad)
    a.close()
    b.close()


def test_sweep_hubbard_odd_sizes_parity():
    # ragged blocks (M not a multiple of the delay block), odd Nwrap remainder
    m = mdl.hubbard("square", 6, 4, U=6.0, beta=1.3, dtau=0.1, nwrap=4)
    _run_pair(m, seed=9, sweeps=2)


def test_sweep_honeycomb_parity():
    m = mdl.hubbard("honeycomb", 3, 3, U=5.0, beta=1.0, dtau=0.05, nwrap=5)
    _run_pair(m, seed=3, sweeps=2)


def test_twenty_sweeps_identical_accept_sequence():
    m = mdl.hubbard("square", 4, 4, U=4.0, beta=2.0, dtau=0.1, nwrap=10)
    _run_pair(m, seed=17, sweeps=20)


def test_device_stream_matches_host_draws():
    m = mdl.config("hubbard4x4")
    seed = 23
    f0 = rng.initial_fields(seed, 0, m.n_op, m.ltrot)
    a = Chains(m)
    a.set_fields(0, f0)
    a.init_state()
    a.set_rng(0, seed, rng.sweep_counter_base(m.n_op, m.ltrot, 0))
    a.sweep(None)
    b = Chains(m)
    b.set_fields(0, f0)
    b.init_state()
    b.sweep(rng.sweep_uniforms(seed, 0, m.n_op, m.ltrot, 0)[None, :])
    np.testing.assert_array_equal(a.fields(0), b.fields(0))
    assert _relmax(a.green(0), b.green(0)) == 0.0


def test_batched_chains_match_single_chains():
    m = mdl.config("hubbard4x4")
    C = 3
    g = Chains(m, n_chains=C)
    fs = [rng.initial_fields(100 + c, c, m.n_op, m.ltrot) for c in range(C)]
    for c in range(C):
        g.set_fields(c, fs[c])
    g.init_state()
    u = np.stack([rng.sweep_uniforms(100 + c, c, m.n_op, m.ltrot, 0) for c in range(C)])
    g.sweep(u)
    for c in range(C):
        o = oracle.Oracle(m)
        o.set_fields(fs[c])
        o.init_state()
        o.sweep(u[c])
        np.testing.assert_array_equal(g.fields(c), o.fields())
        assert _relmax(g.green(c), o.green()) < RTOL


def test_graph_replay_matches_stream_path():
    # alfgpu_sweep replays a captured CUDA graph; the stream path must give identical state
    from alf_gb300.sweep import FLAG_NO_GRAPH
    m = mdl.hubbard("square", 6, 6, U=4.0, beta=2.0, dtau=0.1, nwrap=10)
    seed = 31
    f0 = rng.initial_fields(seed, 0, m.n_op, m.ltrot)
    out = []
    for flags in (0, FLAG_NO_GRAPH):
        g = Chains(m, flags=flags)
        g.set_fields(0, f0)
        g.init_state()
        g.set_rng(0, seed, rng.sweep_counter_base(m.n_op, m.ltrot, 0))
        for s in range(3):
            g.sweep(None)
        g.sweep(rng.sweep_uniforms(seed, 0, m.n_op, m.ltrot, 7)[None, :])
        out.append((g.fields(0), g.green(0), g.phase()[0], g.stats(0).n_acc))
    np.testing.assert_array_equal(out[0][0], out[1][0])
    assert _relmax(out[0][1], out[1][1]) == 0.0
    assert out[0][2] == out[1][2] and out[0][3] == out[1][3]


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_overlapped_blocks_match_the_serial_order(precision):
    # a block's visits start from its submatrix staged while the previous block's flush runs
    # (second stream); the serial order reads it from the flushed G.  Same Woodbury updates in
    # another summation order: identical decisions, G equal to rounding.
    from alf_gb300.sweep import FLAG_NO_OVERLAP
    m = mdl.hubbard("square", 8, 8, U=4.0, beta=2.0, dtau=0.1, nwrap=10)
    C, seed = 2, 41
    out = []
    for flags in (0, FLAG_NO_OVERLAP):
        g = Chains(m, n_chains=C, precision=precision, flags=flags)
        for c in range(C):
            g.set_fields(c, rng.initial_fields(seed + c, c, m.n_op, m.ltrot))
        g.init_state()
        for s in range(2):
            g.sweep(np.stack([rng.sweep_uniforms(seed + c, c, m.n_op, m.ltrot, s) for c in range(C)]))
        out.append([(g.fields(c), g.green(c), g.stats(c).n_acc) for c in range(C)])
    for c in range(C):
        np.testing.assert_array_equal(out[0][c][0], out[1][c][0])
        assert out[0][c][2] == out[1][c][2]
        assert _relmax(out[0][c][1], out[1][c][1]) < (RTOL if precision == "fp64" else 1e-8)


def test_delay_depth_changes_only_rounding_and_autotuner_picks_a_candidate():
    # the delay depth regroups the same Sherman-Morrison sequence; results agree to rounding
    m = mdl.hubbard("square", 6, 6, U=4.0, beta=2.0, dtau=0.1, nwrap=10)
    seed = 41
    f0 = rng.initial_fields(seed, 0, m.n_op, m.ltrot)
    u = rng.sweep_uniforms(seed, 0, m.n_op, m.ltrot, 0)[None, :]
    res = []
    for k in (8, 32):
        g = Chains(m)
        g.set_delay(k)
        assert g.delay() == k
        g.set_fields(0, f0)
        g.init_state()
        g.sweep(u)
        res.append((g.fields(0), g.green(0)))
    np.testing.assert_array_equal(res[0][0], res[1][0])
    assert _relmax(res[0][1], res[1][1]) < RTOL
    g = Chains(m)
    g.set_fields(0, f0)
    g.init_state()
    g.set_rng(0, seed, rng.sweep_counter_base(m.n_op, m.ltrot, 0))
    assert g.tune_delay(1) in (8, 16, 24, 32)


@pytest.mark.parametrize("pivoting", ["default", "norms-cgr"])
def test_sweep_hubbard_16x16_beta10_parity(pivoting):
    # the benchmark configuration itself (N_dim = 256, Ltrot = 100, 20 stabilisation points):
    # fresh G at every stabilisation point and every ratio against the oracle on one sweep
    _run_pair(mdl.config("hubbard16x16"), seed=3, sweeps=1, pivoting=pivoting)


def test_set_nwrap_matches_oracle_with_that_nwrap():
    # a handle built with Nwrap = 10, switched to Nwrap = 3 (ragged: Ltrot = 40 -> 14 points)
    # and re-initialised from its fields, sweeps like the oracle built with Nwrap = 3
    m10 = mdl.config("hubbard4x4")
    m3 = mdl.hubbard("square", 4, 4, U=4.0, beta=4.0, dtau=0.1, nwrap=3)
    seed = 31
    f0 = rng.initial_fields(seed, 0, m10.n_op, m10.ltrot)
    g = Chains(m10, n_chains=1)
    g.set_fields(0, f0)
    g.init_state()
    g.set_nwrap(3)
    assert g.nwrap() == 3
    g.init_state()
    o = oracle.Oracle(m3)
    o.set_fields(f0)
    o.init_state()
    assert _relmax(g.green(0), o.green()) < RTOL
    g.set_recording(True)
    for s in range(2):
        u = rng.sweep_uniforms(seed, 0, m3.n_op, m3.ltrot, s)
        o.record(1)
        o.sweep(u)
        ro = o.recorded()
        g.sweep(u[None, :])
        rg = g.record(0)
        np.testing.assert_array_equal(rg["acc"], ro["acc"])
        assert rg["G"].shape[0] == ro["G"].shape[0] == 2 * 14
        for p in range(ro["G"].shape[0]):
            assert _relmax(rg["G"][p], ro["G"][p]) < RTOL, (s, p)
    np.testing.assert_array_equal(g.fields(0), o.fields())


def test_adapt_nwrap_shortens_until_the_drift_bound_holds():
    # U = 8 at beta = 4 with Nwrap = 20: the wrap drift is far above 1e-12; halving Nwrap
    # until Precision Green <= 1e-12 ends at a shorter interval that meets it (or at 1)
    m = mdl.hubbard("square", 4, 4, U=8.0, beta=4.0, dtau=0.1, nwrap=20)
    g = Chains(m, n_chains=2)
    for c in range(2):
        g.set_fields(c, rng.initial_fields(40 + c, c, m.n_op, m.ltrot))
    g.init_state()
    for c in range(2):
        g.set_rng(c, 40 + c, rng.sweep_counter_base(m.n_op, m.ltrot, 0))
    nw, worst = g.adapt_nwrap(bound=1e-12)
    assert nw < 20 and (worst <= 1e-12 or nw == 1)
    g.sweep(None)
    assert max(g.stats(c).xmaxG for c in range(2)) < 1e-9


def test_checkpoint_resume_continues_on_the_same_draws(tmp_path):
    # confout-style restart: fields + draw-stream state (+ Nwrap, delay depth) written after two
    # sweeps; a new handle restored from it and the original both run two more sweeps
    m = mdl.config("hubbard4x4")
    g = Chains(m, n_chains=2)
    for c in range(2):
        g.set_fields(c, rng.initial_fields(50 + c, c, m.n_op, m.ltrot))
        g.set_rng(c, 50 + c, rng.sweep_counter_base(m.n_op, m.ltrot, 0))
    g.init_state()
    g.set_nwrap(5)
    g.init_state()
    for _ in range(2):
        g.sweep(None)
    path = str(tmp_path / "confout.npz")
    g.checkpoint(path)
    for _ in range(2):
        g.sweep(None)
    h = Chains(m, n_chains=2)
    h.restore(path)
    assert h.nwrap() == 5
    for _ in range(2):
        h.sweep(None)
    for c in range(2):
        np.testing.assert_array_equal(h.fields(c), g.fields(c))
        assert _relmax(h.green(c), g.green(c)) < 1e-8


@pytest.mark.parametrize("lattice,L1,L2", [("square", 4, 4), ("honeycomb", 3, 3)])
def test_checkerboard_hopping_parity(lattice, L1, L2):
    # Checkerboard = .T.: the hopping products are the bond operators of each family, applied in
    # the order of each Hop_mod routine (the oracle restates that order bond by bond)
    m = mdl.hubbard(lattice, L1, L2, U=4.0, chem=0.2, beta=1.0, dtau=0.1, nwrap=5, checkerboard=True)
    _run_pair(m, seed=12, sweeps=2)
