"""Physics known answers for the sweep: the 4-site Hubbard ring and a small Kondo bilayer.

The reference's test suite checks ALF's finite-temperature sweep against exact
diagonalisation on the N_leg_ladder lattice with L1 = 4, L2 = 1 (a periodic 4-site
chain), t = 1, U = 4, beta = 2, Mz decoupling and dense hopping, with
E_ED = -1.47261997 (testsuite/test_vs_ed/test_specs.yaml:25-47; Ener_scal0 extrapolated
in dtau^2 by testsuite/test_vs_ed/analysis.py). Here this is pinned in three layers:

* Exact diagonalisation in the 256-state Fock space of the model this package builds
  gives that number. The ensemble is the Mz form K - U/2 sum (n_up - n_do)^2. The
  estimator is Ener = Kin + U sum <n_up n_do> (Hamiltonian_Hubbard_smod.F90:695-801).
* The Trotterized ensemble, with the HS field summed out exactly per site and slice using
  the package's vertices and four-point tables, is the exact expectation of the Monte
  Carlo estimator at finite dtau. Its dtau -> 0 extrapolation gives the ED number.
* The oracle's Monte Carlo at dtau = 0.1 agrees with that exact finite-dtau value within
  its jackknife error bar. The oracle accumulates the Obs_scal part of ham%Obser at every
  measurement point; bins are analysed with alf_gb300.analysis.
* With Ltau = 1, TAU_M's time-displaced Green functions agree at every tau with the exact
  Trotterized <c(tau) c+(0)> of the same transfer matrix.
* The Kondo model's two-site vertices get the same exact Trotterized check, on one- and
  two-body observables of a 2 x 1 bilayer.
"""
import json
import os

import numpy as np
import pytest
import scipy.linalg as sl

import oracle
from alf_gb300 import model as mdl, rng
from alf_gb300.analysis import jackknife

# the reference's ED test case, extracted from testsuite/test_vs_ed/test_specs.yaml by
# tests/golden/make_golden.py
_GOLD = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "hubbard_finT_chain.json")))
_P = _GOLD["parameters"]
E_ED = _GOLD["ed_energy"]
L_SITES, T_HOP, U_INT, BETA = _P["L1"], _P["ham_T"], _P["ham_U"], _P["beta"]


def test_golden_case_is_the_model_built_here():
    # the fixture's lattice and ensemble are the ones the tests below build.  The reference's runs
    # of this case use the symmetric Trotter split (Symm = true), this package the plain one: the
    # finite-dtau energies differ, their dtau -> 0 limit (the ED energy) does not.
    assert _P["Lattice_type"] == "N_leg_ladder" and _P["L2"] == 1 and _P["Mz"] and not _P["Checkerboard"]
    assert _P["ham_Tperp"] == 0.0 and _P["Ltau"] == 0
    assert abs(E_ED - (-1.47261997)) < 1e-12 and _GOLD["max_delta"] == 0.001


def _ring(dtau, nwrap):
    return mdl.hubbard("n_leg_ladder", L_SITES, 1, t=T_HOP, U=U_INT, beta=BETA, dtau=dtau, nwrap=nwrap)


class _Fock:
    """Dense many-body operators of F flavours x N sites (Jordan-Wigner, orbital f*N + i)."""

    def __init__(self, N, F=2):
        self.N, self.F = N, F
        no = N * F
        self.dim = 1 << no
        states = np.arange(self.dim)
        self.occ = (states[:, None] >> np.arange(no)[None, :]) & 1
        self.c = []
        for k in range(no):
            m = np.zeros((self.dim, self.dim))
            src = states[self.occ[:, k] == 1]
            below = self.occ[src, :k].sum(axis=1)
            m[src ^ (1 << k), src] = np.where(below % 2 == 0, 1.0, -1.0)
            self.c.append(m)

    def n(self, f, i):
        return np.diag(self.occ[:, f * self.N + i].astype(np.float64))

    def one_body(self, H, f):
        """sum_ij H(i,j) c+_{i,f} c_{j,f}"""
        N = self.N
        out = np.zeros((self.dim, self.dim))
        for i in range(N):
            for j in range(N):
                if H[i, j] != 0.0:
                    out += H[i, j] * self.c[f * N + i].T @ self.c[f * N + j]
        return out


def _operators(m):
    fk = _Fock(m.ndim)
    H = mdl.hopping_matrix("n_leg_ladder", L_SITES, 1, t=T_HOP).real
    K = sum(m.n_sun * fk.one_body(H, f) for f in range(2))
    D = sum(fk.n(0, i) @ fk.n(1, i) for i in range(m.ndim))
    return fk, K, D, K + U_INT * D


def _transfer(dtau):
    """(model, Fock space, energy operator, B) with B = W e^{-dtau K}: one slice of the
    Trotterized ensemble with the HS field summed out, W = prod_i sum_s gamma(s) prod_f
    exp(g_f phi(s) (n_{i,f} - alpha_f)) from the model's own vertices (as Upgrade2 weighs a
    field: the vertex exponentials times gamma).  B is scaled to max |B| = 1."""
    m = _ring(dtau, 10)
    fk, K, _, O = _operators(m)
    w = np.ones(fk.dim)
    for i in range(m.ndim):
        wi = np.zeros(fk.dim)
        for s in (-2, -1, 1, 2):
            e = np.zeros(fk.dim)
            for f in range(2):
                v = m.vertices[f][i]
                assert v.P == [i] and v.op_type == 2
                e = e + (v.g * mdl.phi(s, 2) * (fk.occ[:, f * m.ndim + i] - v.alpha)).real
            wi += mdl.GAMA_TYPE2[s] * np.exp(e)
        w *= wi
    B = w[:, None] * sl.expm(-dtau * K)
    return m, fk, O, B / np.abs(B).max()


def _trotter_energy(dtau):
    """Tr[O B^L] / Tr[B^L]: the expectation of Ener over the HS fields, measured (as
    ham%Obser is) after a slice's vertex exponentials."""
    m, _, O, B = _transfer(dtau)
    P = np.linalg.matrix_power(B, m.ltrot)
    return float(np.trace(O @ P) / np.trace(P))


def _trotter_green(dtau):
    """Time-displaced Green functions of the Trotterized ensemble at tau = 0..L (orbital 0
    and its neighbour 1 of flavour 0): [<c_0(tau) c+_0>, <c_0(tau) c+_1>, -<c+_0(tau) c_0>]
    with c(tau) = U(tau,0)^-1 c U(tau,0), U(tau,0) = B^tau, i.e. the expectations of TAU_M's
    GT0(0,0), GT0(0,1) and G0T(0,0)."""
    m, fk, _, B = _transfer(dtau)
    L = m.ltrot
    A = [np.eye(fk.dim)]
    for _ in range(L):
        A.append(B @ A[-1])
    Z = np.trace(A[L])
    c0, c1 = fk.c[0], fk.c[1]
    return m, np.array([[np.trace(A[L - k] @ c0 @ A[k] @ c0.T) / Z for k in range(L + 1)],
                        [np.trace(A[L - k] @ c0 @ A[k] @ c1.T) / Z for k in range(L + 1)],
                        [-np.trace(A[L - k] @ c0.T @ A[k] @ c0) / Z for k in range(L + 1)]]).real


def test_exact_diagonalisation_gives_the_reference_energy():
    m = _ring(0.1, 10)
    fk, K, D, O = _operators(m)
    mz = sum((fk.n(0, i) - fk.n(1, i)) @ (fk.n(0, i) - fk.n(1, i)) for i in range(m.ndim))
    w, V = np.linalg.eigh(K - 0.5 * U_INT * mz)
    p = np.exp(-BETA * (w - w.min()))
    p /= p.sum()
    e = float(np.sum(p * np.einsum("ki,kl,li->i", V, O, V)))
    assert abs(e - E_ED) < 5e-9, e


def test_trotterized_energy_extrapolates_to_the_exact_diagonalisation():
    dt = np.array([0.05, 0.1, 0.2])
    e = np.array([_trotter_energy(x) for x in dt])
    # finite dtau moves the energy by O(dtau^2); the HS sum is exact to higher order
    A = np.stack([np.ones_like(dt), dt ** 2, dt ** 4], axis=1)
    y0 = np.linalg.solve(A, e)[0]
    assert abs(y0 - E_ED) < 2e-4, (y0, e)
    assert abs(e[1] - E_ED) > 0.02  # the Trotter shift at dtau = 0.1 is far above the MC error below


def test_oracle_monte_carlo_energy_matches_the_trotterized_value():
    dtau, nwrap = 0.1, 15  # test_specs.yaml:42-43
    m = _ring(dtau, nwrap)
    seed = 790789
    o = oracle.Oracle(m)
    o.set_fields(rng.initial_fields(seed, 0, m.n_op, m.ltrot))
    o.init_state()
    n_warm, n_bins, n_per_bin = 200, 40, 500
    for s in range(n_warm):
        o.sweep(rng.sweep_uniforms(seed, 0, m.n_op, m.ltrot, s))
    H = mdl.hopping_matrix("n_leg_ladder", L_SITES, 1, t=T_HOP).real
    o.set_scalar_obs(np.stack([H, H]), np.full(m.ndim, U_INT))
    en, si = [], []
    sweep = n_warm
    for b in range(n_bins):
        for _ in range(n_per_bin):
            o.sweep(rng.sweep_uniforms(seed, 0, m.n_op, m.ltrot, sweep))
            sweep += 1
        d = o.scalar_obs(reset=True)
        assert d["count"] == n_per_bin * (2 * m.ltrot - 1)
        en.append(d["ener"].real / d["count"])
        si.append(d["sign"] / d["count"])
    e_mc, err = jackknife(np.array(en), np.array(si))
    e_ex = _trotter_energy(dtau)
    assert err < 0.01, err
    assert abs(e_mc - e_ex) < 3.5 * err, (e_mc, err, e_ex)


@pytest.mark.parametrize("L1", [3, 5])
def test_n_leg_ladder_needs_even_length(L1):
    with pytest.raises(ValueError):
        mdl.hopping_matrix("n_leg_ladder", L1, 1)


def test_oracle_time_displaced_green_functions_match_the_trotterized_values():
    # TAU_M (PROPR / PROPRM1 and the CGR2_2 refreshes) on the same ring, Ltau = 1: the site-
    # and spin-averaged GT0(i,i), GT0(i,i+1) and G0T(i,i) at every tau against the exact
    # Trotterized curves; at tau = 0 and beta particle-hole symmetry makes the local values
    # exact per configuration (zero error bar)
    m, ex = _trotter_green(0.1)
    L = m.ltrot
    o = oracle.Oracle(m, ltau=1)
    seed = 1048
    o.set_fields(rng.initial_fields(seed, 0, m.n_op, m.ltrot))
    o.init_state()
    for s in range(100):
        o.sweep(rng.sweep_uniforms(seed, 0, m.n_op, m.ltrot, s))
    _, tau = o.collect_measurements()
    n_bins, n_per_bin = 20, 100
    rows = []
    for s in range(100, 100 + n_bins * n_per_bin):
        tau.clear()
        o.sweep(rng.sweep_uniforms(seed, 0, m.n_op, m.ltrot, s))
        row = np.zeros((3, L + 1))
        for nt, (gt0, g0t, _, _), ph in tau:
            assert ph.real > 0 and abs(ph.imag) < 1e-10  # Mz at half filling: no sign problem
            nn = [0.5 * (gt0[f][i, (i + 1) % 4] + gt0[f][(i + 1) % 4, i]).real for f in range(2) for i in range(4)]
            row[0, nt] = np.mean([gt0[f][i, i].real for f in range(2) for i in range(4)])
            row[1, nt] = np.mean(nn)
            row[2, nt] = np.mean([g0t[f][i, i].real for f in range(2) for i in range(4)])
        rows.append(row)
        assert len(tau) == L + 1
    a = np.array(rows).reshape(n_bins, n_per_bin, 3, L + 1).mean(axis=1)
    mean = a.mean(axis=0)
    err = a.std(axis=0, ddof=1) / np.sqrt(n_bins)
    dev = np.abs(mean - ex)
    assert np.all(dev <= 4.0 * err + 1e-9), np.max(dev / (err + 1e-300))
    z = (mean - ex)[:, 1:L] / err[:, 1:L]
    assert np.mean(z ** 2) < 2.0, np.mean(z ** 2)
    assert np.max(err[:, 1:L]) < 0.01


def test_kondo_two_site_vertices_match_the_trotterized_values():
    # config 5's vertex algebra (two-site V_SUN vertices, N_FL = 1, N_SUN = 2, ham_Uf = 0) on a
    # bilayer of 2 x 1 cells (c0 f0 c1 f1): the c kinetic energy and the J_K correlator
    # sum_i <D_i^2>, D_i = sum_sigma (c+_i f_i + f+_i c_i), from the oracle's ham%Obser G
    # (Wick per configuration, two identical species) against Tr[O B^L] / Tr[B^L] with the
    # HS field summed out per c-f pair
    dtau = 0.1
    m = mdl.kondo(2, 1, JK=1.5, Uf=0.0, beta=BETA, dtau=dtau, nwrap=10)
    N = m.ndim
    H = mdl.hopping_matrix("BILAYER_SQUARE", 2, 1, t=1.0).real
    fk = _Fock(N, F=2)  # the two SU(2) species of the single flavour

    def ob(A):
        return sum(fk.one_body(A, sp) for sp in range(2))

    pairs = [(2 * i, 2 * i + 1) for i in range(N // 2)]
    W = np.eye(fk.dim)
    for v in m.vertices[0]:
        Ov = np.zeros((N, N))
        for a, pa in enumerate(v.P):
            for b, pb in enumerate(v.P):
                Ov[pa, pb] = v.O[a, b].real
        w, Z = np.linalg.eigh(ob(Ov))
        W = sum(mdl.GAMA_TYPE2[s] * (Z * np.exp((v.g * mdl.phi(s, 2)).real * (w - m.n_sun * v.alpha.real))) @ Z.T
                for s in (-2, -1, 1, 2)) @ W
    B = W @ sl.expm(-dtau * ob(H))
    P = np.linalg.matrix_power(B / np.abs(B).max(), m.ltrot)
    DD = np.zeros((fk.dim, fk.dim))
    for c, f in pairs:
        Oi = np.zeros((N, N))
        Oi[c, f] = Oi[f, c] = 1.0
        Di = ob(Oi)
        DD += Di @ Di
    ex = np.array([np.trace(ob(H) @ P), np.trace(DD @ P)]) / np.trace(P)
    # the lattice density correlation of the bilayer (N_FL = 1 Den, alf_gb300.lattice_obs):
    # Den(r, no, no1) = sum over cell pairs with imj = r of <n_{I,no} n_{J,no1}>, both species
    from alf_gb300 import lattice_obs as lo
    latt = lo.Lattice("bilayer_square", 2, 1)
    nop = [fk.n(0, i) + fk.n(1, i) for i in range(N)]
    den_ex = np.zeros((latt.N, 2, 2))
    for i1 in range(N):
        for j1 in range(N):
            rr = latt.imj[latt.site_cell[i1], latt.site_cell[j1]]
            den_ex[rr, latt.site_orb[i1], latt.site_orb[j1]] += (np.trace(nop[i1] @ nop[j1] @ P) / np.trace(P)).real

    o = oracle.Oracle(m)
    seed = 2024
    o.set_fields(rng.initial_fields(seed, 0, m.n_op, m.ltrot))
    o.init_state()
    for s in range(100):
        o.sweep(rng.sweep_uniforms(seed, 0, m.n_op, m.ltrot, s))
    eq, _ = o.collect_measurements()
    n_bins, n_per_bin = 20, 100
    vals = []
    den_obs = lo.EqualTimeObs(latt, n_sun=m.n_sun, n_fl=1)
    den_bins = []
    sel = np.zeros((N, N))
    for c, f in pairs:
        sel[c, f] = sel[f, c] = 1.0
    for s in range(100, 100 + n_bins * n_per_bin):
        eq.clear()
        o.sweep(rng.sweep_uniforms(seed, 0, m.n_op, m.ltrot, s))
        kin = dd = 0.0
        for _, G, ph in eq:
            assert ph.real > 0 and abs(ph.imag) < 1e-10  # N_SUN = 2, real couplings: no sign problem
            g = G[0]
            grc = np.eye(N) - g.T  # <c+_a c_b>
            kin += m.n_sun * np.sum(H * grc).real
            for c, f in pairs:
                idx = [(c, f), (f, c)]
                d = sum(grc[a, b] for a, b in idx)
                w2 = sum(grc[a, b] * grc[p, q] + grc[a, q] * g[b, p] for a, b in idx for p, q in idx)
                dd += (2.0 * w2 + 2.0 * d * d).real
            den_obs.measure(G, ph)
        vals.append((kin / len(eq), dd / len(eq)))
        if (s - 99) % n_per_bin == 0:
            den_bins.append(den_obs.bin()["Den"]["latt"][:, 0].real)
    a = np.array(vals).reshape(n_bins, n_per_bin, 2).mean(axis=1)
    mean, err = a.mean(axis=0), a.std(axis=0, ddof=1) / np.sqrt(n_bins)
    assert np.all(err < 0.05), err
    assert np.all(np.abs(mean - ex) < 4.0 * err), (mean, err, ex)
    db = np.array(den_bins)
    dm, de = db.mean(axis=0), db.std(axis=0, ddof=1) / np.sqrt(len(db))
    assert len(db) == n_bins and np.all(np.abs(dm - den_ex) < 4.0 * de + 1e-9), (dm, de, den_ex)


def test_lattice_correlations_of_the_ring_match_the_trotterized_values():
    # the SpinZ and Den lattice observables (Predefined_Obs measurements on the oracle's
    # ham%Obser G, alf_gb300.lattice_obs) against N <m_r m_0> and N <n_r n_0> of the exact
    # Trotterized ensemble, m = n_up - n_do, n = n_up + n_do, r over Make_lattice's list
    from alf_gb300 import lattice_obs as lo

    m, fk, _, B = _transfer(0.1)
    P = np.linalg.matrix_power(B, m.ltrot)
    Z = np.trace(P)
    L = lo.Lattice("n_leg_ladder", L_SITES, 1)
    mz = [fk.n(0, i) - fk.n(1, i) for i in range(L_SITES)]
    nn = [fk.n(0, i) + fk.n(1, i) for i in range(L_SITES)]
    ex = {"SpinZ": np.array([L_SITES * np.trace(mz[i1 % L_SITES] @ mz[0] @ P) / Z for i1, _ in L.list]).real,
          "Den": np.array([L_SITES * np.trace(nn[i1 % L_SITES] @ nn[0] @ P) / Z for i1, _ in L.list]).real}
    o = oracle.Oracle(m)
    seed = 31
    o.set_fields(rng.initial_fields(seed, 0, m.n_op, m.ltrot))
    o.init_state()
    for s in range(100):
        o.sweep(rng.sweep_uniforms(seed, 0, m.n_op, m.ltrot, s))
    eq, _ = o.collect_measurements()
    obs = lo.EqualTimeObs(L, n_sun=m.n_sun)
    bins = []
    for b in range(20):
        for s in range(100):
            eq.clear()
            o.sweep(rng.sweep_uniforms(seed, 0, m.n_op, m.ltrot, 100 + 100 * b + s))
            for _, G, ph in eq:
                obs.measure(G, ph)
        bins.append(obs.bin())
    for k in ("SpinZ", "Den"):
        a = np.array([bb[k]["latt"][:, 0, 0, 0].real for bb in bins])
        mean, err = a.mean(axis=0), a.std(axis=0, ddof=1) / np.sqrt(len(bins))
        assert np.all(np.abs(mean - ex[k]) < 4.0 * err + 1e-12), (k, mean, err, ex[k])
    # backgrounds: <m> = 0 and <n> = 1 per site at half filling
    assert abs(np.mean([bb["Den"]["latt0"][0].real for bb in bins]) - 1.0) < 1e-9
    # the same bins through the legacy files and ana_eq: real-space results are the connected
    # per-site correlations <O_r O_0> - <O>^2
    import tempfile
    with tempfile.TemporaryDirectory() as d:
        for bb in bins:
            for k in ("SpinZ", "Den"):
                lo.write_eq_bin(d, k, bb[k], L, dtau=m.dtau)
        for k, bgk in (("SpinZ", 0.0), ("Den", 1.0)):
            _, jr = lo.ana_eq(lo.read_eq(f"{d}/{k}_eq"), L, n_skip=1)
            mean, err = jr[:, 0, 0, 0].real, jr[:, 0, 0, 1].real
            want = ex[k] / L_SITES - bgk ** 2
            assert np.all(np.abs(mean - want) < 4.0 * err + 1e-9), (k, mean, err, want)


def test_time_displaced_lattice_correlations_of_the_ring_match_the_trotterized_values():
    # SpinZ(r, tau) and Den(r, tau) from the oracle's TAU_M quartets (Predefined_Obs_tau_*
    # measurements, alf_gb300.lattice_obs) against N <O_r(tau) O_0(0)> of the exact
    # Trotterized ensemble at every tau
    from alf_gb300 import lattice_obs as lo

    m, fk, _, B = _transfer(0.1)
    Lt = m.ltrot
    A = [np.eye(fk.dim)]
    for _ in range(Lt):
        A.append(B @ A[-1])
    Z = np.trace(A[Lt])
    L = lo.Lattice("n_leg_ladder", L_SITES, 1)
    mz = [fk.n(0, i) - fk.n(1, i) for i in range(L_SITES)]
    nn = [fk.n(0, i) + fk.n(1, i) for i in range(L_SITES)]
    ex = {k: np.array([[L_SITES * np.trace(A[Lt - t] @ ops[i1 % L_SITES] @ A[t] @ ops[0]) / Z
                        for t in range(Lt + 1)] for i1, _ in L.list]).real
          for k, ops in (("SpinZ", mz), ("Den", nn))}
    o = oracle.Oracle(m, ltau=1)
    seed = 77
    o.set_fields(rng.initial_fields(seed, 0, m.n_op, m.ltrot))
    o.init_state()
    for s in range(100):
        o.sweep(rng.sweep_uniforms(seed, 0, m.n_op, m.ltrot, s))
    _, tau = o.collect_measurements()
    obs = lo.TimeDisplacedObs(L, n_sun=m.n_sun, ntau=Lt + 1)
    bins = []
    for b in range(20):
        for s in range(100):
            tau.clear()
            o.sweep(rng.sweep_uniforms(seed, 0, m.n_op, m.ltrot, 100 + 100 * b + s))
            for nt, (gt0, g0t, g00, gtt), ph in tau:
                obs.measure(nt, gt0, g0t, g00, gtt, ph)
        bins.append(obs.bin())
    for k in ("SpinZ", "Den"):
        a = np.array([bb[k]["latt"][:, :, 0, 0].real for bb in bins])
        mean, err = a.mean(axis=0), a.std(axis=0, ddof=1) / np.sqrt(len(bins))
        assert np.all(np.abs(mean - ex[k]) < 4.0 * err + 1e-9), (k, np.max(np.abs(mean - ex[k]) / (err + 1e-300)))
