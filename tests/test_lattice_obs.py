"""Lattice-resolved observables on the host (alf_gb300.lattice_obs): Make_lattice's walks and
imj, the R -> K transform, the equal-time and time-displaced Predefined_Obs measurements
against plain per-site loops, and the legacy ``*_eq`` / ``*_tau`` files.  Their physics (spin
and density correlations of the 4-site ring against exact Trotterized values) is tested in
test_ed_energy.py."""
import math
import os

import numpy as np
import pytest

from alf_gb300 import lattice_obs as lo, model as mdl


@pytest.mark.parametrize("lat,L1,L2", [("square", 4, 4), ("square", 6, 4), ("honeycomb", 6, 6),
                                       ("bilayer_square", 4, 4), ("n_leg_ladder", 4, 2), ("n_leg_ladder", 4, 1)])
def test_walks_tile_and_imj_is_the_folded_difference(lat, L1, L2):
    L = lo.Lattice(lat, L1, L2)
    A = np.array([L.L1p, L.L2p]).T  # columns: the periods
    for i in range(L.N):
        for j in range(L.N):
            d = L.R[i] - L.R[j] - L.R[L.imj[i, j]]
            n = np.linalg.solve(A, d)  # integer multiples of the periods
            assert np.allclose(n, np.round(n), atol=1e-9), (i, j)
    # the k points are distinct modulo the reciprocal periods
    B = np.array([L.b1 * L.L1, L.b2 * L.n2]).T
    fr = np.linalg.solve(B, L.K.T).T
    keys = {tuple(np.round(np.mod(f, 1.0) * 1e6).astype(int) % 1000000) for f in fr}
    assert len(keys) == L.N
    # the list is the one model.alf_cell_order walks
    assert [(i1 % L1) + L1 * (i2 % L.n2) for i1, i2 in L.list] == mdl.alf_cell_order(lat, L1, L2)


def test_square_walk_order():
    L = lo.Lattice("square", 4, 4)
    assert L.list == [(i1, i2) for i1 in (-1, 0, 1, 2) for i2 in (-1, 0, 1, 2)]
    np.testing.assert_allclose(L.b1, [math.pi / 2, 0.0], atol=1e-15)
    np.testing.assert_allclose(L.b2, [0.0, math.pi / 2], atol=1e-15)


def test_fourier_of_a_delta_and_of_a_plane_wave():
    L = lo.Lattice("honeycomb", 3, 3)
    x = np.zeros(L.N, complex)
    x[L.list.index((0, 0))] = 1.0
    np.testing.assert_allclose(L.fourier_r_to_k(x), np.full(L.N, 1.0 / L.N), atol=1e-15)
    k0 = 4
    wave = np.exp(1j * (L.R @ L.K[k0]))
    xk = L.fourier_r_to_k(wave)
    e = np.zeros(L.N)
    e[k0] = 1.0
    np.testing.assert_allclose(xk, e, atol=1e-12)


def _loop_measure(L, G, phase, n_sun):
    """Predefined_Obs_eq_{Green,SpinMz,Den}_measure written out per site pair."""
    nd = G.shape[1]
    GR = lambda i, j, f: G[f][i, j]
    GRC = lambda i, j, f: (1.0 if i == j else 0.0) - G[f][j, i]
    zp, zs = phase / phase.real, np.sign(phase.real)
    no = L.norb
    obs = {k: np.zeros((L.N, no, no), complex) for k in lo.EQ_NAMES}
    obs0 = {k: np.zeros(no, complex) for k in lo.EQ_NAMES}
    for i1 in range(nd):
        I, oi = L.site_cell[i1], L.site_orb[i1]
        zi = n_sun * (GRC(i1, i1, 0) + GRC(i1, i1, 1))
        for j1 in range(nd):
            J, oj = L.site_cell[j1], L.site_orb[j1]
            r = L.imj[I, J]
            obs["Green"][r, oi, oj] += n_sun * (GRC(i1, j1, 0) + GRC(i1, j1, 1)) * zp * zs
            zxy = GRC(i1, j1, 0) * GR(i1, j1, 1) + GRC(i1, j1, 1) * GR(i1, j1, 0)
            zz = (GRC(i1, j1, 0) * GR(i1, j1, 0) + GRC(i1, j1, 1) * GR(i1, j1, 1)
                  + (GRC(i1, i1, 1) - GRC(i1, i1, 0)) * (GRC(j1, j1, 1) - GRC(j1, j1, 0)))
            obs["SpinZ"][r, oi, oj] += zz * zp * zs
            obs["SpinXY"][r, oi, oj] += zxy * zp * zs
            obs["SpinT"][r, oi, oj] += (2 * zxy + zz) * zp * zs / 3.0
            zj = n_sun * (GRC(j1, j1, 0) + GRC(j1, j1, 1))
            z = n_sun * (GRC(i1, j1, 0) * GR(i1, j1, 0) + GRC(i1, j1, 1) * GR(i1, j1, 1))
            obs["Den"][r, oi, oj] += (zi * zj + z) * zp * zs
        dz = GRC(i1, i1, 1) - GRC(i1, i1, 0)
        obs0["SpinZ"][oi] += dz * zp * zs
        obs0["SpinT"][oi] += dz * zp * zs / math.sqrt(3.0)
        obs0["Den"][oi] += zi * zp * zs
    return obs, obs0


@pytest.mark.parametrize("order", ["natural", "alf"])
def test_measurements_equal_the_per_site_loops(order):
    L = lo.Lattice("honeycomb", 2, 3, site_order=order)
    nd = L.N * L.norb
    r = np.random.default_rng(11)
    G = r.standard_normal((2, nd, nd)) + 1j * r.standard_normal((2, nd, nd))
    ph = complex(0.8, 0.3)
    m = lo.EqualTimeObs(L, n_sun=1)
    m.measure(G, ph)
    m.measure(G, ph)
    b = m.bin()
    ref, ref0 = _loop_measure(L, G, ph, 1)
    for k in lo.EQ_NAMES:
        np.testing.assert_allclose(b[k]["latt"][:, 0], ref[k], rtol=1e-13, atol=1e-13)
        np.testing.assert_allclose(b[k]["latt0"], ref0[k] / L.N, rtol=1e-13, atol=1e-13)
        assert b[k]["sign"] == 1.0
    assert m.count == 0


def test_eq_files_round_trip(tmp_path):
    L = lo.Lattice("honeycomb", 2, 2)
    nd = L.N * L.norb
    r = np.random.default_rng(2)
    m = lo.EqualTimeObs(L, n_sun=1)
    bins = []
    for _ in range(2):
        G = r.standard_normal((2, nd, nd)) * 0.3 + 0.5 * np.eye(nd)[None]
        m.measure(G.astype(complex), complex(1.0, 0.0))
        bins.append(m.bin())
        lo.write_eq_bin(str(tmp_path), "SpinZ", bins[-1]["SpinZ"], L, dtau=0.1)
    back = lo.read_eq(str(tmp_path / "SpinZ_eq"))
    assert len(back) == 2
    for b, rd in zip(bins, back):
        assert rd["sign"] == b["SpinZ"]["sign"]
        np.testing.assert_array_equal(rd["latt0"], b["SpinZ"]["latt0"])
        np.testing.assert_array_equal(rd["k"], L.K)
        want = np.stack([L.fourier_r_to_k(b["SpinZ"]["latt"][:, 0, a, c]) for a in range(2) for c in range(2)], axis=1)
        np.testing.assert_array_equal(rd["values"].reshape(L.N, 4), want)
    info = open(tmp_path / "SpinZ_eq_info").read().splitlines()
    assert info[0] == "          Observable: SpinZ_eq" and info[2].endswith(" 1") and "Bravais" in info[4]
    assert os.path.getsize(tmp_path / "SpinZ_eq_info") > 0


def _loop_measure_tau(L, nt, GT0, G0T, G00, GTT, phase, n_sun):
    """Predefined_Obs_tau_{Green,SpinMz,Den}_measure written out per site pair."""
    nd = GT0.shape[1]
    w = phase / phase.real * np.sign(phase.real)
    no = L.norb
    obs = {k: np.zeros((L.N, no, no), complex) for k in lo.EQ_NAMES}
    obs0 = {k: np.zeros(no, complex) for k in lo.EQ_NAMES}
    for i1 in range(nd):
        I, oi = L.site_cell[i1], L.site_orb[i1]
        zi = n_sun * sum(1.0 - GTT[f][i1, i1] for f in range(2))
        for j1 in range(nd):
            J, oj = L.site_cell[j1], L.site_orb[j1]
            r = L.imj[I, J]
            obs["Green"][r, oi, oj] += (GT0[0][i1, j1] + GT0[1][i1, j1]) / 2.0 * w
            zz = ((GTT[0][i1, i1] - GTT[1][i1, i1]) * (G00[0][j1, j1] - G00[1][j1, j1])
                  - G0T[0][j1, i1] * GT0[0][i1, j1] - G0T[1][j1, i1] * GT0[1][i1, j1])
            zxy = -G0T[0][j1, i1] * GT0[1][i1, j1] - G0T[1][j1, i1] * GT0[0][i1, j1]
            obs["SpinZ"][r, oi, oj] += zz * w
            obs["SpinXY"][r, oi, oj] += zxy * w
            obs["SpinT"][r, oi, oj] += (2 * zxy + zz) / 3.0 * w
            zj = n_sun * sum(1.0 - G00[f][j1, j1] for f in range(2))
            z = -n_sun * sum(G0T[f][j1, i1] * GT0[f][i1, j1] for f in range(2))
            obs["Den"][r, oi, oj] += (zi * zj + z) * w
        d = GTT[1][i1, i1] - GTT[0][i1, i1]
        obs0["SpinZ"][oi] += d * w
        obs0["SpinT"][oi] += d * w / math.sqrt(3.0)
        obs0["Den"][oi] += zi * w
    return obs, obs0


def test_time_displaced_measurements_equal_the_per_site_loops_and_round_trip(tmp_path):
    L = lo.Lattice("square", 2, 3, site_order="alf")
    nd = L.N * L.norb
    r = np.random.default_rng(4)
    ntau = 3
    m = lo.TimeDisplacedObs(L, n_sun=1, ntau=ntau)
    ref = {k: np.zeros((L.N, ntau, 1, 1), complex) for k in lo.EQ_NAMES}
    ref0 = {k: np.zeros(1, complex) for k in lo.EQ_NAMES}
    ph = complex(-0.7, 0.2)
    for nt in range(ntau):
        q = [r.standard_normal((2, nd, nd)) + 1j * r.standard_normal((2, nd, nd)) for _ in range(4)]
        m.measure(nt, *q, ph)
        o, o0 = _loop_measure_tau(L, nt, *q, ph, 1)
        for k in lo.EQ_NAMES:
            ref[k][:, nt] += o[k]
            ref0[k] += o0[k]
    b = m.bin()
    for k in lo.EQ_NAMES:
        np.testing.assert_allclose(b[k]["latt"], ref[k], rtol=1e-13, atol=1e-13)
        np.testing.assert_allclose(b[k]["latt0"], ref0[k] / (L.N * ntau), rtol=1e-13, atol=1e-13)
        assert b[k]["sign"] == -1.0
    lo.write_latt_bin(str(tmp_path), "Den", b["Den"], L, dtau=0.05)
    back = lo.read_eq(str(tmp_path / "Den_tau"))
    assert len(back) == 1 and back[0]["dtau"] == 0.05 and back[0]["values"].shape == (L.N, ntau, 1, 1)
    for nt in range(ntau):
        np.testing.assert_array_equal(back[0]["values"][:, nt, 0, 0], L.fourier_r_to_k(b["Den"]["latt"][:, nt, 0, 0]))
    assert open(tmp_path / "Den_tau_info").readline().rstrip() == "          Observable: Den_tau"


def test_ana_eq_subtracts_the_background_at_k0_and_in_real_space(tmp_path):
    from alf_gb300.analysis import jackknife_vec
    L = lo.Lattice("square", 4, 2)
    r = np.random.default_rng(6)
    bins = []
    for _ in range(9):
        b = {"latt": (r.standard_normal((L.N, 1, 1, 1)) + 1j * r.standard_normal((L.N, 1, 1, 1))),
             "latt0": np.array([0.3 + 0.1 * r.standard_normal()], complex), "sign": 0.9 + 0.05 * r.random()}
        lo.write_eq_bin(str(tmp_path), "Den", b, L, dtau=0.1)
    back = lo.read_eq(str(tmp_path / "Den_eq"))
    jk, jr = lo.ana_eq(back, L, n_skip=1)
    use = back[1:]
    sg = np.array([x["sign"] for x in use])
    bg = np.array([x["latt0"][0] for x in use])
    k0 = int(np.argmin(np.hypot(L.K[:, 0], L.K[:, 1])))
    for k in range(L.N):
        v = np.array([x["values"][k, 0, 0] for x in use])
        if k == k0:
            want = jackknife_vec(np.stack([v, bg * L.N, bg]), sg, lambda X: X[0] - X[1] * X[2])
        else:
            want = jackknife_vec(v[None, :], sg, lambda X: X[0])
        np.testing.assert_allclose(jk[k, 0, 0], want, rtol=1e-12, atol=1e-14)
    vr = np.array([L.fourier_k_to_r(x["values"][:, 0, 0]) for x in use])  # [nb][R]
    for R in range(L.N):
        want = jackknife_vec(np.stack([vr[:, R], bg, bg]), sg, lambda X: X[0] - X[1] * X[2])
        np.testing.assert_allclose(jr[R, 0, 0], want, rtol=1e-12, atol=1e-14)
    lo.write_ana_eq(str(tmp_path), "Den", jk, jr, L)
    lines = open(tmp_path / "DenJK").read().splitlines()
    assert len(lines) == 2 * L.N and lines[1].split()[:2] == ["1", "1"]
    assert float(lines[1].split()[2]) == float(jk[0, 0, 0, 0].real)  # 17 digits: the double itself


def test_single_flavour_measurements_equal_the_per_site_loops():
    # N_FL = 1 (SU(N) models, Kondo): Green, SpinZ by SpinSUN, Den; equal time and tau
    L = lo.Lattice("bilayer_square", 2, 2)
    nd = L.N * L.norb
    r = np.random.default_rng(13)
    ns = 2
    G = r.standard_normal((1, nd, nd)) + 1j * r.standard_normal((1, nd, nd))
    ph = complex(1.2, -0.1)
    w = ph / ph.real
    m = lo.EqualTimeObs(L, n_sun=ns, n_fl=1)
    m.measure(G, ph)
    b = m.bin()
    assert tuple(b) == lo.EQ_NAMES_SUN
    GR = G[0]
    GRC = np.eye(nd) - GR.T
    ref = {k: np.zeros((L.N, 2, 2), complex) for k in lo.EQ_NAMES_SUN}
    ref0 = np.zeros(2, complex)
    for i1 in range(nd):
        for j1 in range(nd):
            rr, a, c = L.imj[L.site_cell[i1], L.site_cell[j1]], L.site_orb[i1], L.site_orb[j1]
            ref["Green"][rr, a, c] += ns * GRC[i1, j1] * w
            ref["SpinZ"][rr, a, c] += ns * GRC[i1, j1] * GR[i1, j1] * w
            ref["Den"][rr, a, c] += (ns * GRC[i1, i1] * ns * GRC[j1, j1] + ns * GRC[i1, j1] * GR[i1, j1]) * w
        ref0[L.site_orb[i1]] += ns * GRC[i1, i1] * w
    for k in lo.EQ_NAMES_SUN:
        np.testing.assert_allclose(b[k]["latt"][:, 0], ref[k], rtol=1e-13, atol=1e-13)
    np.testing.assert_allclose(b["Den"]["latt0"], ref0 / L.N, rtol=1e-13)
    t = lo.TimeDisplacedObs(L, n_sun=ns, ntau=2, n_fl=1)
    q = [r.standard_normal((1, nd, nd)) + 1j * r.standard_normal((1, nd, nd)) for _ in range(4)]
    t.measure(0, *q, ph)
    t.measure(1, *q, ph)
    bt = t.bin()
    gt0, g0t, g00, gtt = (x[0] for x in q)
    refs = np.zeros((L.N, 2, 2), complex)
    refd = np.zeros((L.N, 2, 2), complex)
    for i1 in range(nd):
        for j1 in range(nd):
            rr, a, c = L.imj[L.site_cell[i1], L.site_cell[j1]], L.site_orb[i1], L.site_orb[j1]
            refs[rr, a, c] += -ns * g0t[j1, i1] * gt0[i1, j1] * w
            refd[rr, a, c] += (ns * (1 - gtt[i1, i1]) * ns * (1 - g00[j1, j1]) - ns * g0t[j1, i1] * gt0[i1, j1]) * w
    for nt in range(2):
        np.testing.assert_allclose(bt["SpinZ"]["latt"][:, nt], refs, rtol=1e-13, atol=1e-13)
        np.testing.assert_allclose(bt["Den"]["latt"][:, nt], refd, rtol=1e-13, atol=1e-13)
    with pytest.raises(ValueError):
        m.measure(np.zeros((2, nd, nd)), ph)
