"""Bin analysis of Monte Carlo observables: ALF's jackknife with the sign.

Restates the published algorithm of Libraries/Modules/errors_mod.F90 (ERRCALC :98-126,
ERRCALC_C :128-158, ERRCALC_J :160-190, ERRCALC_J_REBIN :257-287, ERRCALC_JS :290-327,
ERRCALC_JS_F :338-388, ERRCALC_JS_C_F :432-476, ERRCALC_JS_REBIN :481-516,
ERRCALC_JS_C_REBIN_F :599-) and Analysis/ana_mod.F90:862-933 (jack).  ana_mod applies them
(ERRCALCJ calls, e.g. :1380, :1587, :1783) to the per-bin averages of <O s> and <s> written
by the observables module:

* rebin: consecutive groups of ``nrebin`` bins are averaged (a trailing remainder is
  dropped, like the reference's integer division);
* jackknife: leave-one-out ratios x_n = (sum_b O_b - O_n) / (sum_b s_b - s_n), optionally
  mapped by f;
* mean and error: the mean of the x_n, and sqrt(sum_n (x_n - mean)^2) (the reference's
  ERRCALC standard error times the number of bins, without the (n - 1)/n factor of the
  textbook jackknife).

Complex observables are analysed part by part (ERRCALC_C): real and imaginary errors.
"""
from __future__ import annotations

from typing import Callable, Optional, Tuple

import numpy as np


def errcalc(en) -> Tuple[float, float]:
    """Mean and standard error of the mean of the samples (ERRCALC)."""
    en = np.asarray(en, dtype=np.float64)
    n = en.size
    xm = en.sum() / n
    xsq = ((en - xm) ** 2).sum() / n
    xerr = xsq / n
    return float(xm), float(np.sqrt(xerr)) if xerr > 0 else 0.0


def rebin(x, nrebin: int) -> np.ndarray:
    """Averages of consecutive groups of nrebin bins (the remainder is dropped)."""
    x = np.asarray(x)
    n = x.shape[0] // nrebin
    return x[: n * nrebin].reshape((n, nrebin) + x.shape[1:]).mean(axis=1)


def _js_real(en, si, f):
    en = np.asarray(en, dtype=np.float64)
    si = np.asarray(si, dtype=np.float64)
    if en.shape != si.shape:
        raise ValueError("jackknife: observable and sign bins differ in number")
    x = (en.sum() - en) / (si.sum() - si)
    if f is not None:
        x = np.array([f(v) for v in x], dtype=np.float64)
    xm, xerr = errcalc(x)
    return xm, xerr * en.size


def jackknife(en, si=None, nrebin: int = 1, f: Optional[Callable[[float], float]] = None):
    """Sign-weighted jackknife of per-bin averages ``en`` (of O s) and ``si`` (of s):
    mean and error of <O s>/<s> (or of f of it).  si = None: no sign (all ones).  Complex
    en: (mean, error) with real and imaginary parts analysed separately."""
    en = np.asarray(en)
    si = np.ones(en.shape[0]) if si is None else np.asarray(si, dtype=np.float64)
    if nrebin > 1:
        en, si = rebin(en, nrebin), rebin(si, nrebin)
    if np.iscomplexobj(en):
        mr, er = _js_real(en.real, si, f)
        mi, ei = _js_real(en.imag, si, f)
        return complex(mr, mi), complex(er, ei)
    return _js_real(en, si, f)


def jackknife_plain(en, nrebin: int = 1):
    """Jackknife without a sign (ERRCALC_J, ERRCALC_J_REBIN): leave-one-out means
    (sum - x_n) / (n - 1) of the (rebinned) samples; mean and ERRCALC error times n."""
    en = np.asarray(en, dtype=np.float64)
    if nrebin > 1:
        en = rebin(en, nrebin)
    n = en.size
    if n < 2:
        raise ValueError("jackknife: fewer than two bins")
    xm, xerr = errcalc((en.sum() - en) / (n - 1))
    return xm, xerr * n


def jackknife_vec(en, si, f: Callable, nrebin: int = 1):
    """ERRCALC_JS_C_F / ERRCALC_JS_C_REBIN_F: en [n_obs][n_bins] (complex) and the sign bins
    si [n_bins]; f maps the leave-one-out ratio vector (sum_b en_b - en_n) / (sum_b si_b -
    si_n) to a complex number.  Mean and error of the f values, real and imaginary parts
    separately (ERRCALC_C), the error times the number of (rebinned) bins."""
    en = np.asarray(en, dtype=np.complex128)
    si = np.asarray(si, dtype=np.complex128)
    if en.shape[1] != si.shape[0]:
        raise ValueError("jackknife: observable and sign bins differ in number")
    if nrebin > 1:
        en = rebin(en.T, nrebin).T
        si = rebin(si, nrebin)
    n = si.size
    if n < 2:
        raise ValueError("jackknife: fewer than two bins")
    X = (en.sum(axis=1)[:, None] - en) / (si.sum() - si)[None, :]
    vals = np.array([complex(f(X[:, b])) for b in range(n)])
    mr, er = errcalc(vals.real)
    mi, ei = errcalc(vals.imag)
    return complex(mr, mi), complex(er, ei) * n


def jack(func: Callable, data, n_skip: int = 0, n_rebin: int = 1):
    """Analysis/ana_mod.F90:862-933 (jack): data [n_obs][n_bins]; bins after the first n_skip
    are rebinned by n_rebin (remainder dropped), func maps each leave-one-out mean vector
    (sum - x_n) / (n - 1) to a complex number; mean and error of those values, real and
    imaginary parts separately, the error times n.  No sign weighting."""
    data = np.asarray(data, dtype=np.complex128)[:, n_skip:]
    nr = data.shape[1] // n_rebin
    if nr < 2:
        raise ValueError("jack: fewer than two rebinned bins")
    d = data[:, : nr * n_rebin].reshape(data.shape[0], nr, n_rebin).mean(axis=2)
    X = (d.sum(axis=1)[:, None] - d) / (nr - 1)
    vals = np.array([complex(func(X[:, n])) for n in range(nr)])
    mr, er = errcalc(vals.real)
    mi, ei = errcalc(vals.imag)
    return complex(mr, mi), complex(er, ei) * nr
