"""Scalar observable bins: formation, reduction over walkers and the legacy text files.

Restates the host side of ALF's scalar observables for the accumulators the sweep library
fills (alfgpu_get_scalar_obs: sums of ZP ZS O, of ZS, and the count of measurements):

* a bin is Obs_vec / N and Ave_sign / N (Prog/observables_mod.F90:815-816);
* walkers are averaged: the MPI_REDUCE(SUM) / Isize_g over a group of ranks
  (observables_mod.F90:824-834).  Here the chains of one handle are walkers, and
  ranks (one per GPU) reduce with torch.distributed (gloo or nccl);
* rank 0 appends one line per bin to ``<name>_scal`` in the legacy text format
  (observables_mod.F90:848-866): ``(I10)`` entries + 1, then `` (re,im)`` as
  ``E25.17E3`` pairs, then the sign as ``E26.17E3``;
* the analysis reads those lines back (Analysis/ana_mod.F90:104-127 read_vec), drops
  N_skip bins, rebins and takes ALF's jackknife of <O s>/<s> per entry and of the sign
  alone, written as ``<name>J`` (ana_mod.F90:1750-1797 ana_vec, identity mode).
"""
from __future__ import annotations

import math
import os
import re
from typing import Dict, Iterable, List, Sequence, Tuple

import numpy as np

from .analysis import jackknife, jackknife_plain

# the Hubbard Obs_scal entries in ham%Obser order (Hamiltonian_Hubbard_smod.F90:695-801)
HUBBARD_SCALARS = ("Kin", "Pot", "Part", "Ener")


def fortran_e(x: float, w: int, d: int, e: int = 3) -> str:
    """Fortran ``Ew.dEe`` edit descriptor: ``0.<d digits>E<sign><e digits>``, right
    justified in w columns (the optional leading zero kept when it fits)."""
    x = float(x)
    if math.isnan(x) or math.isinf(x):
        return ("NaN" if math.isnan(x) else ("-Infinity" if x < 0 else "Infinity")).rjust(w)
    if x == 0.0:
        mant, exp = "0" * d, 0
        neg = math.copysign(1.0, x) < 0
    else:
        s = f"{abs(x):.{d - 1}e}"  # d significant digits, rounded once
        digits, ex = s.split("e")
        mant = digits.replace(".", "")
        exp = int(ex) + 1  # 0.ddd x 10^(k+1) == d.dd x 10^k
        neg = x < 0
    body = f"0.{mant}E{'-' if exp < 0 else '+'}{abs(exp):0{e}d}"
    if neg:
        body = "-" + body
    if len(body) > w and body.startswith(("0.", "-0.")):
        body = body.replace("0.", ".", 1)
    if len(body) > w:
        return "*" * w
    return body.rjust(w)


def scal_line(obs_vec: Sequence[complex], sign: float) -> str:
    """One bin of a ``*_scal`` file (observables_mod.F90:862-866)."""
    parts = [f"{len(obs_vec) + 1:10d}"]
    for z in obs_vec:
        z = complex(z)
        parts.append(f" ({fortran_e(z.real, 25, 17)},{fortran_e(z.imag, 25, 17)})")
    parts.append(fortran_e(sign, 26, 17))
    return "".join(parts)


def write_scal(path: str, obs_vec: Sequence[complex], sign: float) -> None:
    """Append one bin to the ``*_scal`` file at path (created when absent)."""
    with open(path, "a") as f:
        f.write(scal_line(obs_vec, sign) + "\n")


_NUM = r"[-+]?(?:\d+\.?\d*|\.\d+)(?:[EeDd][-+]?\d+)?"
_CPLX = re.compile(r"\(\s*(" + _NUM + r")\s*,\s*(" + _NUM + r")\s*\)")


def read_scal(path: str) -> Tuple[np.ndarray, np.ndarray]:
    """All bins of a ``*_scal`` file: (bins [n_bins][n_obs] complex, sign [n_bins]).  A
    line that does not hold the declared number of entries ends the read, as the
    reference's iostat loop does."""
    rows, sgn = [], []
    with open(path) as f:
        nobs = None
        for line in f:
            line = line.strip()
            if not line:
                break
            head = line.split(None, 1)
            try:
                n1 = int(head[0])
            except ValueError:
                break
            if nobs is None:
                nobs = n1 - 1
            zs = _CPLX.findall(line)
            tail = line[line.rfind(")") + 1:].split() if zs else head[1:]
            if len(zs) != nobs or len(tail) != 1:
                break
            rows.append([complex(float(a.replace("D", "E").replace("d", "e")),
                                 float(b.replace("D", "E").replace("d", "e"))) for a, b in zs])
            sgn.append(float(tail[0].replace("D", "E").replace("d", "e")))
    return np.array(rows, dtype=np.complex128).reshape(len(rows), -1), np.array(sgn, dtype=np.float64)


def bin_from_sums(sums: Dict, names: Sequence[str] = ("kin", "pot", "part", "ener")) -> Tuple[np.ndarray, float]:
    """Obs_vec / N and Ave_sign / N of one walker's accumulators (the dictionary
    ``Chains.scalar_obs`` returns): (entries in ``names`` order, sign)."""
    n = int(sums["count"])
    if n <= 0:
        raise ValueError("an empty bin (no measurement since the last reset)")
    return np.array([complex(sums[k]) / n for k in names]), float(sums["sign"]) / n


def walker_mean(bins: Iterable[Tuple[np.ndarray, float]]) -> Tuple[np.ndarray, float]:
    """Mean over walkers of (Obs_vec, Ave_sign): the group reduction SUM / Isize_g."""
    bins = list(bins)
    if not bins:
        raise ValueError("no walkers")
    ov = np.mean(np.stack([np.asarray(b[0], np.complex128) for b in bins]), axis=0)
    return ov, float(np.mean([b[1] for b in bins]))


def mean_over_ranks(obs_vec: np.ndarray, sign: float) -> Tuple[np.ndarray, float]:
    """The same reduction over the ranks of the initialised process group (each rank
    passes its own walker mean; equal walker counts per rank).  Without a process group,
    returns the input."""
    import torch
    import torch.distributed as dist
    obs_vec = np.asarray(obs_vec, np.complex128)
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return obs_vec, float(sign)
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor(np.concatenate([obs_vec.view(np.float64), [sign]]), dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    a = t.cpu().numpy() / dist.get_world_size()
    return a[:-1].copy().view(np.complex128), float(a[-1])


def write_hubbard_bin(directory: str, obs_vec: Sequence[complex], sign: float,
                      names: Sequence[str] = HUBBARD_SCALARS) -> None:
    """One bin of the Hubbard scalars: each entry is its own observable with a
    one-element vector (``Kin_scal``, ``Pot_scal``, ``Part_scal``, ``Ener_scal``)."""
    os.makedirs(directory, exist_ok=True)
    for name, z in zip(names, obs_vec):
        write_scal(os.path.join(directory, f"{name}_scal"), [z], sign)


def ana_vec(bins: np.ndarray, sgn: np.ndarray, n_skip: int = 1, n_rebin: int = 1) -> Tuple[List, Tuple]:
    """ana_vec in identity mode: per entry the sign-weighted jackknife of the real part
    over bins n_skip.., rebinned by n_rebin; then the jackknife of the sign alone.
    Returns ([(mean, err) per entry], (sign mean, sign err))."""
    bins = np.asarray(bins)
    sgn = np.asarray(sgn, np.float64)
    b, s = bins[n_skip:], sgn[n_skip:]
    if b.shape[0] // n_rebin < 2:
        raise ValueError("effective number of bins smaller than 2")
    out = [jackknife(b[:, i].real, s, nrebin=n_rebin) for i in range(b.shape[1])]
    return out, jackknife_plain(s, nrebin=n_rebin)


def write_ana(path: str, bins: np.ndarray, sgn: np.ndarray, n_skip: int = 1, n_rebin: int = 1) -> None:
    """The ``<name>J`` file of ana_vec: effective and raw bin counts, then per entry and
    for the sign ``(I11, 2(E26.17E3))`` index, mean, error, each after a blank line."""
    res, sres = ana_vec(bins, sgn, n_skip, n_rebin)
    nb = np.asarray(bins).shape[0]
    with open(path, "w") as f:
        f.write(f" Effective number of bins, and bins: {(nb - n_skip) // n_rebin:11d} {nb:11d}\n")
        for i, (m, e) in enumerate(res + [sres], start=1):
            f.write("\n")
            f.write(f"{i:11d}{fortran_e(m, 26, 17)}{fortran_e(e, 26, 17)}\n")


def read_ana(path: str) -> List[Tuple[float, float]]:
    """(mean, error) rows of a ``<name>J`` file, the sign last."""
    rows = []
    with open(path) as f:
        next(f)
        for line in f:
            p = line.split()
            if len(p) == 3:
                rows.append((float(p[1]), float(p[2])))
    return rows
