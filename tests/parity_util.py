"""Helpers of the GPU parity tests: where a sweep's recorded stabilisation points sit in
its visit sequence, and comparisons of a GPU chain's record with the oracle's that stop
at the first visit where the two accept sequences part.

Visit order (Prog/Wrapgr_mod.F90, Prog/main.F90:714-887): the up pass visits slices
nt = 1..Ltrot, M vertices each; the down pass nt = Ltrot..1.  A stabilisation point of
the up pass at slice Stab_nt(n) comes after the updates of slice Stab_nt(n); one of the
down pass at ntau1 = Stab_nt(n) after the updates of slice ntau1 + 1; the last point
(G on slice 0) after the whole sweep.
"""
from __future__ import annotations

from typing import Optional

import numpy as np


def stab_nt(ltrot: int, nwrap: int) -> list:
    nstm = -(-ltrot // nwrap)
    return [0] + [nwrap * n for n in range(1, nstm)] + [ltrot]


def point_visits(n_op: int, ltrot: int, nwrap: int) -> np.ndarray:
    """Visits completed when each of the 2 Nstm recorded stabilisation points is taken."""
    st = stab_nt(ltrot, nwrap)
    nstm = len(st) - 1
    up = [st[n] * n_op for n in range(1, nstm + 1)]
    down = [ltrot * n_op + (ltrot - st[n]) * n_op for n in range(nstm - 1, 0, -1)]
    return np.array(up + down + [2 * ltrot * n_op], dtype=np.int64)


def parting_visit(acc_a: np.ndarray, acc_b: np.ndarray) -> Optional[int]:
    """Index of the first visit whose accept bits differ, or None."""
    d = np.flatnonzero(np.asarray(acc_a) != np.asarray(acc_b))
    return int(d[0]) if d.size else None


def relmax(a, b) -> float:
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def compare_record(rg: dict, ro: dict, u: np.ndarray, n_op: int, ltrot: int, nwrap: int, *,
                   g_tol: float, relative: bool, exact_sequence: bool, ratio_tol: Optional[float] = None,
                   ratio_median: Optional[float] = None) -> dict:
    """Compare one sweep's GPU record with the oracle's.

    With exact_sequence the accept sequences must agree visit for visit.  Otherwise they
    may part, but only at a visit whose Metropolis weight lies within rounding of its draw
    (|W - r| < 1e-4 max(W, 1)); the points taken before that visit are compared and at
    least one must be.  G at every compared point within g_tol (relative to max|G| when
    relative, else absolute); ratios of the agreeing visits: median relative deviation
    <= ratio_median and maximum <= ratio_tol when given.  Returns the counts and worst
    deviations."""
    v = parting_visit(rg["acc"], ro["acc"])
    if exact_sequence:
        assert v is None, f"accept sequences part at visit {v}"
    nvis = len(ro["acc"])
    upto = nvis if v is None else v
    if v is not None:
        w = abs(ro["ratio"][v])
        assert abs(w - u[3 * v + 2]) < 1e-4 * max(w, 1.0), (v, w, u[3 * v + 2])
    pv = point_visits(n_op, ltrot, nwrap)
    npts = ro["G"].shape[0]
    assert len(pv) == npts
    worst = 0.0
    compared = 0
    for p in range(npts):
        if pv[p] > upto:
            break
        d = relmax(rg["G"][p], ro["G"][p]) if relative else float(np.max(np.abs(rg["G"][p] - ro["G"][p])))
        worst = max(worst, d)
        assert d <= g_tol, (p, d)
        compared += 1
    assert compared >= 1, "no stabilisation point before the accept sequences part"
    n = upto + 1 if v is not None else upto  # the parting visit's ratio still comes from equal state
    r_o, r_g = ro["ratio"][:n], rg["ratio"][:n]
    prop = np.abs(r_o) > 0
    rel = np.abs(r_g[prop] - r_o[prop]) / np.abs(r_o[prop])
    if ratio_median is not None:
        assert np.median(rel) <= ratio_median, np.median(rel)
    if ratio_tol is not None:
        assert rel.max() <= ratio_tol, (rel.max(), ratio_tol)
    return {"parting_visit": v, "points_compared": compared, "points": npts, "worst_dG": worst,
            "ratio_rel_max": float(rel.max()) if rel.size else 0.0,
            "ratio_rel_median": float(np.median(rel)) if rel.size else 0.0}
