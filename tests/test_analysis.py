"""Jackknife bin analysis (alf_gb300.analysis) against direct restatements of
errors_mod.F90's formulas."""
import numpy as np

from alf_gb300 import analysis


def test_errcalc_is_mean_and_standard_error():
    x = np.array([1.0, 2.0, 4.0, 7.0])
    m, e = analysis.errcalc(x)
    assert m == 3.5
    assert np.isclose(e, np.sqrt(np.mean((x - 3.5) ** 2) / 4))


def test_jackknife_without_sign_equals_error_of_the_mean_scaled():
    # with s = 1 the jackknife values are the leave-one-out means (S - x_n) / (n - 1); the
    # error is sqrt(sum_n (loo_n - mean)^2)
    r = np.random.default_rng(0)
    x = r.standard_normal(20)
    m, e = analysis.jackknife(x)
    n = x.size
    loo = (x.sum() - x) / (n - 1)
    assert np.isclose(m, x.mean())
    assert np.isclose(e, np.sqrt(((loo - loo.mean()) ** 2).sum()))


def test_jackknife_with_sign_and_function_and_rebinning():
    r = np.random.default_rng(1)
    s = 0.8 + 0.1 * r.standard_normal(30)
    o = s * (2.0 + 0.3 * r.standard_normal(30))
    m, e = analysis.jackknife(o, s, nrebin=3, f=lambda v: v * v)
    ob, sb = o.reshape(10, 3).mean(1), s.reshape(10, 3).mean(1)
    x = ((ob.sum() - ob) / (sb.sum() - sb)) ** 2
    assert np.isclose(m, x.mean())
    assert np.isclose(e, np.sqrt(((x - x.mean()) ** 2).sum()))


def test_complex_observables_are_analysed_part_by_part():
    r = np.random.default_rng(2)
    z = r.standard_normal(12) + 1j * r.standard_normal(12)
    m, e = analysis.jackknife(z)
    mr, er = analysis.jackknife(z.real)
    mi, ei = analysis.jackknife(z.imag)
    assert m == complex(mr, mi) and e == complex(er, ei)


def test_vector_jackknife_reduces_to_the_signed_scalar_one():
    from alf_gb300.analysis import jackknife, jackknife_vec
    r = np.random.default_rng(8)
    en = r.standard_normal(30)
    si = 0.7 + 0.2 * r.random(30)
    m, e = jackknife_vec(en[None, :], si, lambda X: X[0])
    m2, e2 = jackknife(en, si)
    assert abs(m.real - m2) < 1e-14 and abs(e.real - e2) < 1e-14 and m.imag == 0.0 and e.imag == 0.0
    # with rebinning, and a non-linear function of two observables
    en2 = np.stack([en + 1j * r.standard_normal(30), 1.0 + 0.1 * r.standard_normal(30)])
    m3, e3 = jackknife_vec(en2, si, lambda X: X[0] / X[1], nrebin=3)
    a, s = en2.reshape(2, 10, 3).mean(axis=2), si.reshape(10, 3).mean(axis=1)
    x = [((a[0].sum() - a[0][n]) / (s.sum() - s[n])) / ((a[1].sum() - a[1][n]) / (s.sum() - s[n])) for n in range(10)]
    x = np.array(x)
    assert abs(m3 - x.mean()) < 1e-13
    assert abs(e3.real - np.sqrt(np.sum((x.real - x.real.mean()) ** 2) / 10 / 10) * 10) < 1e-13


def test_jack_is_the_unsigned_vector_jackknife_after_skip_and_rebin():
    from alf_gb300.analysis import jack, jackknife_plain, jackknife_vec
    r = np.random.default_rng(9)
    d = r.standard_normal((2, 25)) + 1j * r.standard_normal((2, 25))
    m, e = jack(lambda X: X[0] * X[1], d, n_skip=1, n_rebin=4)
    # the same as the signed form with unit signs (leave-one-out sums over n - 1 bins)
    m2, e2 = jackknife_vec(d[:, 1:], np.ones(24), lambda X: X[0] * X[1], nrebin=4)
    assert abs(m - m2) < 1e-13 and abs(e - e2) < 1e-13
    m3, e3 = jack(lambda X: X[0], d[:1].real, n_skip=0, n_rebin=1)
    m4, e4 = jackknife_plain(d[0].real)
    assert abs(m3.real - m4) < 1e-14 and abs(e3.real - e4) < 1e-14
