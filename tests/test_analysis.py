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
