"""Uniform-draw streams for the sweep.

ALF draws with the Fortran intrinsic ``RANDOM_NUMBER`` through ``ranf_wrap``
(Libraries/Modules/random_wrap_mod.F90:135-141).  The sweep consumes, per
vertex visit, three draws in this order (Prog/Wrapgr_mod.F90:125,133 and
Prog/upgrade_mod.F90:222):

  slot 0: the type-2 flip choice ``nranf(3)`` (Prog/Fields_mod.F90:184)
  slot 1: the ``T0_proposal`` test (always passes for ``Propose_S0 = .F.``)
  slot 2: the Metropolis test ``Weight > ranf``

Visits run ``nt = 1..Ltrot, n = 1..M`` on the up pass and ``nt = Ltrot..1,
n = M..1`` on the down pass, so one sweep consumes ``3 * 2 * M * Ltrot`` draws.
The library accepts those draws from the caller (a Fortran host passes
``ranf_wrap`` values) or generates them on the device from the counter-based
stream defined here, which both the GPU library and the oracle implement
bit-identically: ``u = (splitmix64(key(seed, chain) + counter) >> 11) * 2**-53``.
"""
from __future__ import annotations

import numpy as np

_GOLD = np.uint64(0x9E3779B97F4A7C15)
_M1 = np.uint64(0xBF58476D1CE4E5B9)
_M2 = np.uint64(0x94D049BB133111EB)
_CHAIN = np.uint64(0xD1B54A32D192ED03)


def _mix(z: np.ndarray) -> np.ndarray:
    z = z.astype(np.uint64)
    with np.errstate(over="ignore"):
        z = (z ^ (z >> np.uint64(30))) * _M1
        z = (z ^ (z >> np.uint64(27))) * _M2
    return z ^ (z >> np.uint64(31))


def chain_key(seed: int, chain: int) -> np.uint64:
    with np.errstate(over="ignore"):
        k = np.uint64(seed & 0xFFFFFFFFFFFFFFFF) ^ (np.uint64(chain) * _CHAIN)
        return _mix(np.array([k + _GOLD], dtype=np.uint64))[0]


def uniforms(seed: int, chain: int, start: int, count: int) -> np.ndarray:
    """Draws ``counter = start .. start+count-1`` of chain ``chain``."""
    key = chain_key(seed, chain)
    ctr = np.arange(start, start + count, dtype=np.uint64)
    with np.errstate(over="ignore"):
        z = _mix(key + (ctr + np.uint64(1)) * _GOLD)
    return (z >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)


def draws_per_sweep(n_op: int, ltrot: int) -> int:
    return 3 * 2 * n_op * ltrot


def sweep_counter_base(n_op: int, ltrot: int, sweep: int) -> int:
    """Counter of the first draw of sweep ``sweep`` (0-based).

    Counters ``0 .. M*Ltrot-1`` are reserved for the initial fields.
    """
    return n_op * ltrot + sweep * draws_per_sweep(n_op, ltrot)


def sweep_uniforms(seed: int, chain: int, n_op: int, ltrot: int, sweep: int) -> np.ndarray:
    return uniforms(seed, chain, sweep_counter_base(n_op, ltrot, sweep), draws_per_sweep(n_op, ltrot))


def initial_fields(seed: int, chain: int, n_op: int, ltrot: int) -> np.ndarray:
    """``Fields_set`` (Prog/Fields_mod.F90:588-610): +1, or -1 when r > 0.5.

    Returns int8 ``f[nt][n]`` (the Fortran ``f(n, nt)`` array, column-major).
    """
    r = uniforms(seed, chain, 0, n_op * ltrot).reshape(ltrot, n_op)
    return np.where(r > 0.5, -1, 1).astype(np.int8)
