"""Pins the CPU oracle against the reference's own known-answer identities.

* ``testsuite/Prog.tests/15-cgr.F90``: CGR against a naive inverse on the 5x5
  inputs of that test, G to 1e-10 relative, phase to 1e-13, both NVAR.
* ``testsuite/Prog.tests/20-qdrp.F90``: QDRP + ZUNGQR + ZTRMM reconstruct the
  Hilbert matrix, N = 2..50, to 1e-14 (here 1e-13 relative to |A|).
* ``testsuite/Prog.tests/24-udv.F90``: ten random products decomposed on the R
  and L sides reconstruct U D V (resp. U D V^H).
* Whole-sweep identities: G at every stabilisation point equals the dense
  ``(1 + B(tau,0) B(beta,tau))^-1`` of the current fields, and every recorded
  Metropolis ratio equals the ratio of dense weights.
"""
import numpy as np
import pytest

import oracle
from alf_gb300 import model as mdl, rng
from tests import naive


def test_cgr_matches_naive_inverse_15cgr():
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
        G, ph = oracle.cgr(nvar, UR, DR, VR, UL, DL, VL)
        M = np.eye(N) + UR @ np.diag(DR) @ VR @ VL @ np.diag(DL) @ UL.conj().T
        Gn = np.linalg.inv(M)
        assert np.max(np.abs(G - Gn)) <= 1e-10 * np.max(np.abs(Gn))
        d = np.linalg.det(M)
        assert abs(ph - d / abs(d)) < 1e-13


def test_qdrp_reconstructs_hilbert_20qdrp():
    for N in range(2, 51):
        A = np.array([[1.0 / (i + j + 1) for j in range(N)] for i in range(N)], dtype=complex)
        U, D, V = oracle.decompose("r", A, np.ones(N, complex), np.eye(N, dtype=complex))
        R = U @ np.diag(D) @ V
        assert np.max(np.abs(R - A)) <= 1e-13 * np.max(np.abs(A)), N


def test_udv_products_24udv():
    rs = np.random.default_rng(4782347)
    N = 16
    for side in ("r", "l"):
        U, D, V = np.eye(N, dtype=complex), np.ones(N, complex), np.eye(N, dtype=complex)
        P = np.eye(N, dtype=complex)
        for _ in range(10):
            X = rs.standard_normal((N, N)) + 1j * rs.standard_normal((N, N))
            U = X @ U
            P = X @ P
            U, D, V = oracle.decompose(side, U, D, V)
            R = U @ np.diag(D) @ (V if side == "r" else V.conj().T)
            assert np.max(np.abs(R - P)) <= 1e-10 * np.max(np.abs(P))
            # U is unitary and D is real positive, sorted by the pivoting
            assert np.max(np.abs(U.conj().T @ U - np.eye(N))) < 1e-12
            assert np.all(D.real > 0) and np.all(np.abs(D.imag) == 0)


def _small_hubbard(lattice="square", L1=4, L2=2, beta=1.0, nwrap=5, U=4.0):
    return mdl.hubbard(lattice, L1, L2, U=U, beta=beta, dtau=0.1, nwrap=nwrap)


@pytest.mark.parametrize("kind", ["hubbard", "kondo", "checkerboard", "checkerboard-honeycomb"])
def test_sweep_identities(kind):
    # checkerboard: the oracle applies the bond operators one by one in the order of each
    # Hop_mod routine; the dense formulas use their product B_T = E_1 ... E_Ncheck (and B_T^T
    # where the left UDV state propagates), so a wrong order or a missing transpose shows
    if kind == "hubbard":
        m = _small_hubbard()
    elif kind == "checkerboard":
        m = mdl.hubbard("square", 4, 4, U=4.0, chem=0.2, beta=1.0, dtau=0.1, nwrap=5, checkerboard=True)
    elif kind == "checkerboard-honeycomb":
        m = mdl.hubbard("honeycomb", 2, 2, U=4.0, beta=1.0, dtau=0.1, nwrap=5, checkerboard=True)
    else:
        m = mdl.kondo(2, 2, JK=1.5, Uf=2.0, beta=1.0, dtau=0.1, nwrap=5)
    seed, chain = 11, 0
    f0 = rng.initial_fields(seed, chain, m.n_op, m.ltrot)
    o = oracle.Oracle(m)
    o.set_fields(f0)
    ph0 = o.init_state()
    G0 = o.green()
    for nf in range(m.n_fl):
        Gn = naive.green(m, f0, 0, nf)
        assert np.max(np.abs(G0[nf] - Gn)) < 1e-10
    w0 = naive.full_weight(m, f0)
    assert abs(ph0 - w0 / abs(w0)) < 1e-10
    rec = o.record(1)
    u = rng.sweep_uniforms(seed, chain, m.n_op, m.ltrot, 0)
    o.sweep(u)
    # replay the field history and check every ratio against dense weights
    f = f0.copy()
    visits = naive.visit_order(m)
    w_old = naive.full_weight(m, f)
    checked = 0
    for v, (nt1, n) in enumerate(visits):
        s_old = int(f[nt1 - 1, n])
        s_new = mdl.FLIP_TYPE2[s_old][naive.nranf3(u[3 * v]) - 1]
        fn = f.copy()
        fn[nt1 - 1, n] = s_new
        if v % 7 == 0:  # dense weights are expensive; sample the visits
            w_new = naive.full_weight(m, fn)
            r = rec["ratio"][v]
            assert abs(r - w_new / w_old) <= 1e-9 * abs(w_new / w_old), (v, r, w_new / w_old)
            checked += 1
        if rec["acc"][v]:
            f = fn
            w_old = naive.full_weight(m, f) if v % 7 != 6 else w_old
        if v % 7 == 6 and rec["acc"][v]:
            w_old = naive.full_weight(m, f)
    assert checked > 10
    assert np.array_equal(f, o.fields())
    # stabilisation points: recorded fresh G equals the dense formula for the fields at that time
    Gend = o.green()
    for nf in range(m.n_fl):
        Gn = naive.green(m, f, 0, nf)
        assert np.max(np.abs(Gend[nf] - Gn)) < 1e-9
    st = o.stats()
    assert st.n_prop == len(visits) and 0 < st.n_acc < st.n_prop
    assert st.xmaxG < 1e-8


def test_oracle_tau_m_propagation_matches_cgr2_2():
    # TAU_M's propagated GT0/G0T/GTT/G00 against the fresh CGR2_2 blocks every Nwrap slices
    # (Control_Precision_tau): two independent computations of the same matrices
    from alf_gb300 import model as mdl, rng
    m = mdl.hubbard("honeycomb", 2, 2, U=5.0, beta=1.0, dtau=0.05, nwrap=5)
    o = oracle.Oracle(m, ltau=1)
    o.set_fields(rng.initial_fields(7, 0, m.n_op, m.ltrot))
    o.init_state()
    eq, tau = o.collect_measurements()
    o.sweep(rng.sweep_uniforms(7, 0, m.n_op, m.ltrot, 0))
    s = o.stats()
    assert s.ncg_tau == 4 * m.n_fl * m.nstm
    assert s.xmax_tau < 1e-9
    # at NT = 0: G00 = GT0 = GTT = G and G0T = G - 1
    nt, (gt0, g0t, g00, gtt), _ = tau[0]
    assert nt == 0
    np.testing.assert_array_equal(gt0, g00)
    np.testing.assert_array_equal(gtt, g00)
    np.testing.assert_allclose(g0t, g00 - np.eye(m.ndim)[None], atol=1e-15)


def test_checkerboard_families_follow_the_reference():
    # test_checkerboard_decomposition (Predefined_Hop_mod.F90:171-246): the bonds of a family are
    # disjoint, and together the families hold every nearest-neighbour bond of the dense Op_T once
    for lat, L1, L2, nfam in (("square", 4, 4, 4), ("square", 6, 4, 4), ("honeycomb", 3, 3, 3)):
        cb = mdl.checkerboard_ops(lat, L1, L2, 0.1)
        assert len(cb["fam"]) == nfam + 1
        for f in range(nfam):
            sites = cb["P"][cb["fam"][f]:cb["fam"][f + 1]].ravel()
            assert len(set(sites.tolist())) == len(sites)
        O = mdl.hopping_matrix(lat, L1, L2)
        dense = {tuple(sorted((i, j))) for i, j in zip(*np.nonzero(np.triu(O, 1)))}
        bonds = [tuple(sorted(p)) for p in cb["P"].tolist()]
        assert sorted(bonds) == sorted(dense)
        # the product of the bond exponentials is exp(-dtau T) up to the Trotter error O(dtau^2)
        for dt in (0.1, 0.05):
            c = mdl.checkerboard_ops(lat, L1, L2, dt, chem=0.3)
            B = mdl.checkerboard_product(c, O.shape[0])
            w, Z = np.linalg.eigh(mdl.hopping_matrix(lat, L1, L2, chem=0.3))
            ex = (Z * np.exp(-dt * w)[None, :]) @ Z.conj().T
            assert np.max(np.abs(B - ex)) < 1.2 * dt ** 2


def test_solve_extended_system_17():
    # testsuite/Prog.tests/17-solve-extended-system.F90: for LQ = 1, 2, 3 the QDRP of the 2LQ Hilbert
    # matrix, UCT = ones, VINV(i, j) = i + j (1-based); solve_extended_System must equal
    # U3 conj(1/D3) (V3^H)^-1 blockdiag(UCT, VINV).  The reference accepts 10% per entry; the
    # restatement agrees to rounding.
    for LQ in (1, 2, 3):
        n2 = 2 * LQ
        inp = np.array([[1.0 / (i + j) for j in range(1, n2 + 1)] for i in range(1, n2 + 1)], np.complex128)
        UCT = np.ones((LQ, LQ), np.complex128)
        VINV = np.array([[float(i + j) for j in range(1, LQ + 1)] for i in range(1, LQ + 1)], np.complex128)
        H, U3, V3, D3 = oracle.solve_extended_case(inp, UCT, VINV)
        B1 = np.zeros((n2, n2), np.complex128)
        B1[:LQ, :LQ] = UCT
        B1[LQ:, LQ:] = VINV
        X = np.linalg.solve(V3.conj().T, B1)
        X = np.conj(1.0 / D3)[:, None] * X
        Ho = U3 @ X
        assert np.max(np.abs(H - Ho)) <= 1e-8 * np.max(np.abs(Ho)), LQ
        # and the pieces reconstruct the input: Q diag(D3) V3 = inp
        assert np.max(np.abs(U3 @ (D3[:, None] * V3) - inp)) < 1e-13
