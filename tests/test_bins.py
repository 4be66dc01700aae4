"""Scalar observable bins on the host: the legacy ``*_scal`` text format, its reader, the
walker / rank reduction (two gloo ranks) and ana_vec's jackknife, end to end on oracle
bins (Prog/observables_mod.F90:815-866, Analysis/ana_mod.F90:104-127, 1750-1797)."""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

import oracle
from alf_gb300 import bins, model as mdl, rng
from alf_gb300.analysis import jackknife, jackknife_plain


def test_scal_line_has_the_fixed_width_legacy_layout():
    line = bins.scal_line([complex(-1.5240558190394764, 0.0), complex(2.5, -1e-300)], 1.0)
    assert line == ("         3"
                    " (-0.15240558190394764E+001, 0.00000000000000000E+000)"
                    " ( 0.25000000000000000E+001,-0.10000000000000000E-299)"
                    "  0.10000000000000000E+001")
    assert bins.fortran_e(0.5, 26, 17) == "  0.50000000000000000E+000"
    assert bins.fortran_e(-123456.0, 25, 17) == "-0.12345600000000000E+006"


def test_write_then_read_returns_the_same_doubles(tmp_path):
    r = np.random.default_rng(3)
    vals = (r.standard_normal((30, 2)) + 1j * r.standard_normal((30, 2))) * 10.0 ** r.integers(-8, 8, (30, 2))
    sgn = r.choice([-1.0, 1.0], 30) * r.random(30)
    p = str(tmp_path / "X_scal")
    for v, s in zip(vals, sgn):
        bins.write_scal(p, v, s)
    b, s = bins.read_scal(p)
    np.testing.assert_array_equal(b, vals)  # 17 significant digits round-trip a double
    np.testing.assert_array_equal(s, sgn)


def test_reader_stops_at_a_truncated_line(tmp_path):
    p = str(tmp_path / "Y_scal")
    for k in range(3):
        bins.write_scal(p, [complex(k, 0)], 1.0)
    with open(p, "a") as f:
        f.write("         2 ( 0.1E+001,")  # a bin cut off mid-write
    b, s = bins.read_scal(p)
    assert b.shape == (3, 1) and s.shape == (3,)


def test_ana_vec_skips_rebins_and_uses_the_signed_jackknife(tmp_path):
    r = np.random.default_rng(5)
    nb = 41
    b = r.standard_normal((nb, 3)) + 0.1j
    s = 0.8 + 0.1 * r.random(nb)
    res, sres = bins.ana_vec(b, s, n_skip=1, n_rebin=2)
    for i in range(3):
        assert res[i] == jackknife(b[1:, i].real, s[1:], nrebin=2)
    assert sres == jackknife_plain(s[1:], nrebin=2)
    # ALF's plain jackknife error is the standard error of the mean times sqrt(n / (n - 1))
    x = s[1:].reshape(-1, 2).mean(axis=1)
    n = x.size
    assert abs(sres[1] - np.std(x, ddof=1) / np.sqrt(n) * np.sqrt(n / (n - 1))) < 1e-14
    p = str(tmp_path / "ZJ")
    bins.write_ana(p, b, s, n_skip=1, n_rebin=2)
    rows = bins.read_ana(p)
    assert len(rows) == 4
    for (m, e), (m2, e2) in zip(res + [sres], rows):
        assert abs(m - m2) <= 1e-16 * max(1.0, abs(m)) and abs(e - e2) <= 1e-16 * max(1.0, abs(e))
    with pytest.raises(ValueError):
        bins.ana_vec(b[:3], s[:3], n_skip=1, n_rebin=2)


def test_walker_mean_divides_by_the_count():
    a = {"kin": 4 + 2j, "pot": 2.0, "part": 8.0, "ener": 6 + 2j, "sign": 2.0, "count": 2}
    b = {"kin": 0.0, "pot": 6.0, "part": 4.0, "ener": 6.0, "sign": -1.0, "count": 1}
    ov, sg = bins.walker_mean([bins.bin_from_sums(a), bins.bin_from_sums(b)])
    np.testing.assert_allclose(ov, [1 + 0.5j, 3.5, 4.0, 4.5 + 0.5j])
    assert sg == 0.0
    with pytest.raises(ValueError):
        bins.bin_from_sums(dict(a, count=0))


def _free_port() -> int:
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank(rank, world, port, out):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ov, sg = bins.mean_over_ranks(np.array([1.0 + rank, 2j * rank]), 1.0 - 2 * rank)
        out[rank] = (list(ov), sg)
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_average_their_bins():
    mgr = mp.Manager()
    out = mgr.dict()
    mp.spawn(_rank, args=(2, _free_port(), out), nprocs=2, join=True)
    for r in range(2):
        ov, sg = out[r]
        np.testing.assert_allclose(ov, [1.5, 1j])
        assert sg == 0.0


def test_oracle_bins_through_the_files_give_the_direct_jackknife(tmp_path):
    m = mdl.hubbard("n_leg_ladder", 4, 1, U=4.0, beta=2.0, dtau=0.1, nwrap=10)
    seed = 452938
    o = oracle.Oracle(m)
    o.set_fields(rng.initial_fields(seed, 0, m.n_op, m.ltrot))
    o.init_state()
    H = mdl.hopping_matrix("n_leg_ladder", 4, 1).real
    o.set_scalar_obs(np.stack([H, H]), np.full(m.ndim, 4.0))
    direct = []
    sweep = 0
    for _ in range(12):
        for _ in range(20):
            o.sweep(rng.sweep_uniforms(seed, 0, m.n_op, m.ltrot, sweep))
            sweep += 1
        ov, sg = bins.walker_mean([bins.bin_from_sums(o.scalar_obs(reset=True))])
        bins.write_hubbard_bin(str(tmp_path), ov, sg)
        direct.append((ov, sg))
    b, s = bins.read_scal(str(tmp_path / "Ener_scal"))
    assert b.shape == (12, 1)
    np.testing.assert_array_equal(b[:, 0], [d[0][3] for d in direct])
    res, _ = bins.ana_vec(b, s)
    assert res[0] == jackknife(np.array([d[0][3].real for d in direct[1:]]), np.array([d[1] for d in direct[1:]]))
    for name in bins.HUBBARD_SCALARS:
        assert os.path.exists(tmp_path / f"{name}_scal")
