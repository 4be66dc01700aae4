"""Lattice-resolved equal-time and time-displaced observables and their legacy bins, on the host.

The sweep hands every equal-time Green function to ``ham%Obser`` (the library's observable
callback).  For callers without ALF's Fortran driver, this module restates what the Hubbard
models do there with the lattice:

* the Bravais lattice exactly as Make_lattice builds it
  (Libraries/Modules/lattices_v3_mod.F90:88-336): the real-space cells and the k points as
  centred walks (i1 / m outer, i2 / n inner), the k grid vectors b1, b2, and imj(I, J), the
  cell of R_I - R_J folded back into the list; unit cells and orbital positions of
  Prog/Predefined_Latt_mod.F90:100-262;
* the measurements Predefined_Obs_eq_Green_measure, _SpinMz_measure and _Den_measure
  (Prog/Predefined_Obs_mod.F90:137-330) as Hamiltonian_Hubbard_smod.F90:776-790 calls them
  for N_FL = 2: Green, SpinZ, SpinXY, SpinT, Den; and their time-displaced versions
  Predefined_Obs_tau_*_measure (Predefined_Obs_mod.F90:330-600) on the TAU_M quartets, as
  ham%ObserT calls them (Hamiltonian_Hubbard_smod.F90:847-850);
* Print_bin_Latt's legacy output (Prog/observables_mod.F90:355-500): Obs_Latt / N,
  Obs_Latt0 / (N Ns Ntau), Ave_sign / N, the transform to k space
  X(k) = 1/Ns sum_R exp(-i k.R) X(R) (FT_R_to_K_C, lattices_v3_mod.F90:847-872), one
  ``<name>_eq_info`` (``_tau_info``) file and one block per bin appended to ``<name>_eq``
  (``<name>_tau``).

Sites are numbered as the model numbers them (``model.hopping_matrix``'s ``site_order``):
site = cell * Norb + orbital, cells in natural order or in Make_lattice's order.
"""
from __future__ import annotations

import math
import os
import re
from typing import Dict, List, Sequence, Tuple

import numpy as np

from . import model as mdl
from .bins import fortran_e

EQ_NAMES = ("Green", "SpinZ", "SpinXY", "SpinT", "Den")  # N_FL = 2 (Mz Hubbard)
EQ_NAMES_SUN = ("Green", "SpinZ", "Den")                   # N_FL = 1 (SU(N) models, Kondo): SpinZ by SpinSUN


def names_for(n_fl: int):
    """The Obs_eq / Obs_tau files of the predefined measurements for N_FL flavours."""
    return EQ_NAMES if n_fl == 2 else EQ_NAMES_SUN


def _walk(v1: np.ndarray, v2: np.ndarray, tests: Sequence[np.ndarray], L: int) -> List[Tuple[int, int]]:
    """Make_lattice's centred walk: x = i1 v1 + i2 v2 (i1 outer) kept when
    -|a|^2/2 + eps <= x.a <= |a|^2/2 + eps for every a in tests."""
    out = []
    for i1 in range(-L, L + 1):
        for i2 in range(-L, L + 1):
            x = i1 * v1 + i2 * v2
            if all(-float(a @ a) / 2.0 + mdl.EPS_SMALL <= float(x @ a) <= float(a @ a) / 2.0 + mdl.EPS_SMALL
                   for a in tests):
                out.append((i1, i2))
    return out


class Lattice:
    """Bravais lattice, unit cell and site map of one of the model's lattices."""

    def __init__(self, lattice: str, L1: int, L2: int, site_order: str = "natural"):
        lat = lattice.upper()
        a1, a2 = (np.array(v, dtype=np.float64) for v in mdl._PRIMITIVE[lat])
        if lat == "SQUARE":
            norb, n2c, ncoord, orb = 1, L2, (1 if L2 == 1 else 2), [(0.0, 0.0)]
        elif lat == "HONEYCOMB":
            norb, n2c, ncoord = 2, L2, 3
            orb = [(0.0, 0.0), tuple((a2 - 0.5 * a1) * 2.0 / 3.0)]
        elif lat == "BILAYER_SQUARE":
            norb, n2c, ncoord, orb = 2, L2, 2, [(0.0, 0.0, 0.0), (0.0, 0.0, -1.0)]
        elif lat == "N_LEG_LADDER":
            norb, n2c, ncoord, orb = L2, 1, 1, [(0.0, float(no)) for no in range(L2)]
        else:
            raise ValueError(f"lattice {lattice!r} not supported")
        self.name, self.L1, self.n2 = lat, L1, n2c
        self.a1, self.a2, self.norb, self.n_coord, self.orb_pos = a1, a2, norb, ncoord, orb
        self.L1p, self.L2p = L1 * a1, n2c * a2
        Minv = np.linalg.inv(np.array([a1, a2]))
        bz1, bz2 = 2.0 * math.pi * Minv[:, 0], 2.0 * math.pi * Minv[:, 1]
        L = max(abs(int(round(float(b @ v) / (2.0 * math.pi)))) for b in (bz1, bz2) for v in (self.L1p, self.L2p))
        self.list = _walk(a1, a2, [self.L2p, self.L1p, self.L2p - self.L1p, self.L2p + self.L1p], L)
        X = abs(2.0 * math.pi / (float(bz1 @ self.L1p) * float(bz2 @ self.L2p)
                                 - float(bz2 @ self.L1p) * float(bz1 @ self.L2p)))
        self.b1 = X * (float(bz2 @ self.L2p) * bz1 - float(bz1 @ self.L2p) * bz2)
        self.b2 = X * (float(bz1 @ self.L1p) * bz2 - float(bz2 @ self.L1p) * bz1)
        self.listk = _walk(self.b1, self.b2, [bz2, bz1, bz2 - bz1, bz2 + bz1], L)
        self.N = L1 * n2c
        if len(self.list) != self.N or len(self.listk) != self.N:
            raise ValueError(f"{lattice} {L1}x{L2}: the centred walks do not tile the lattice")
        cls = {(i1 % L1, i2 % n2c): k for k, (i1, i2) in enumerate(self.list)}
        if len(cls) != self.N:
            raise ValueError(f"{lattice} {L1}x{L2}: two cells of the walk are equivalent")
        li = np.array(self.list)
        self.imj = np.array([[cls[((li[i, 0] - li[j, 0]) % L1, (li[i, 1] - li[j, 1]) % n2c)]
                              for j in range(self.N)] for i in range(self.N)])
        self.R = li[:, :1] * a1[None, :] + li[:, 1:] * a2[None, :]
        lk = np.array(self.listk)
        self.K = lk[:, :1] * self.b1[None, :] + lk[:, 1:] * self.b2[None, :]
        ndim = self.N * norb
        if site_order == "alf":
            cell = np.arange(ndim) // norb
        elif site_order == "natural":
            nat = np.arange(ndim) // norb
            cell = np.array([cls[(c % L1, c // L1)] for c in nat])
        else:
            raise ValueError(f"site_order {site_order!r}: 'natural' or 'alf'")
        self.site_cell, self.site_orb = cell, np.arange(ndim) % norb

    def fourier_r_to_k(self, x_r: np.ndarray) -> np.ndarray:
        """X(k) = 1/Ns sum_R exp(-i k.R) X(R) over the first axis (FT_R_to_K_C)."""
        ph = np.exp(-1j * (self.K @ self.R.T))  # [k][R]
        return np.tensordot(ph, np.asarray(x_r, dtype=np.complex128), axes=(1, 0)) / self.N

    def fourier_k_to_r(self, x_k: np.ndarray) -> np.ndarray:
        """X(R) = 1/Ns sum_k exp(i k.R) X(k) over the first axis (FT_K_to_R_Mat_C,
        lattices_v3_mod.F90:672-709; with the 1/Ns of both directions a round trip divides
        by Ns, so ana_eq's real-space results are per-site correlations)."""
        ph = np.exp(1j * (self.R @ self.K.T))  # [R][k]
        return np.tensordot(ph, np.asarray(x_k, dtype=np.complex128), axes=(1, 0)) / self.N


class EqualTimeObs:
    """Obs_eq of the predefined measurements, accumulated as Obs_Latt(imj, 1, no_I, no_J),
    Obs_Latt0(no), N and Ave_sign: for N_FL = 2 (Hubbard Mz) Green, SpinZ, SpinXY, SpinT,
    Den; for N_FL = 1 (SU(N) Hubbard, Kondo) Green, SpinZ (SpinSUN), Den."""

    def __init__(self, latt: Lattice, n_sun: int, n_fl: int = 2):
        if n_fl not in (1, 2):
            raise ValueError("N_FL is 1 or 2")
        self.latt, self.n_sun, self.n_fl = latt, n_sun, n_fl
        self.names = names_for(n_fl)
        self.reset()

    def reset(self):
        no, N = self.latt.norb, self.latt.N
        self.obs = {k: np.zeros((N, 1, no, no), np.complex128) for k in self.names}
        self.obs0 = {k: np.zeros(no, np.complex128) for k in self.names}
        self.count, self.sign = 0, 0.0

    def measure(self, G: np.ndarray, phase: complex):
        """One ham%Obser call: G [n_fl][row][col] (the callback's frame), phase."""
        G = np.asarray(G)
        if G.shape[0] != self.n_fl:
            raise ValueError(f"G has {G.shape[0]} flavours, expected {self.n_fl}")
        if self.n_fl == 1:
            return self._measure_sun(G, phase)
        zp = phase / phase.real
        zs = float(np.sign(phase.real))
        w = zp * zs
        nd = G.shape[1]
        eye = np.eye(nd)
        GR = G
        GRC = np.stack([eye - G[f].T for f in range(2)])  # GRC(i,j) = delta_ij - G(j,i)
        L = self.latt
        rows = L.imj[np.ix_(L.site_cell, L.site_cell)]  # [I1][J1] -> imj
        oi = np.broadcast_to(L.site_orb[:, None], (nd, nd))
        oj = np.broadcast_to(L.site_orb[None, :], (nd, nd))
        ns = self.n_sun

        def add(name, val):
            np.add.at(self.obs[name][:, 0], (rows, oi, oj), val * w)

        add("Green", ns * (GRC[0] + GRC[1]))
        if ns == 1:
            dz = np.diag(GRC[1]) - np.diag(GRC[0])
            zxy = GRC[0] * GR[1] + GRC[1] * GR[0]
            zz = GRC[0] * GR[0] + GRC[1] * GR[1] + dz[:, None] * dz[None, :]
            add("SpinZ", zz)
            add("SpinXY", zxy)
            add("SpinT", (2.0 * zxy + zz) / 3.0)
            np.add.at(self.obs0["SpinZ"], L.site_orb, dz * w)
            np.add.at(self.obs0["SpinT"], L.site_orb, dz * w / math.sqrt(3.0))
        zi = ns * (np.diag(GRC[0]) + np.diag(GRC[1]))
        z = ns * (GRC[0] * GR[0] + GRC[1] * GR[1])
        add("Den", zi[:, None] * zi[None, :] + z)
        np.add.at(self.obs0["Den"], L.site_orb, zi * w)
        self.count += 1
        self.sign += zs

    def _measure_sun(self, G: np.ndarray, phase: complex):
        """N_FL = 1: Green and Den as above with one flavour, SpinZ by
        Predefined_Obs_eq_SpinSUN_measure (N_SUN GRC(I,J) GR(I,J), no background)."""
        w = phase / phase.real * float(np.sign(phase.real))
        nd = G.shape[1]
        GR, GRC = G[0], np.eye(nd) - G[0].T
        L = self.latt
        rows = L.imj[np.ix_(L.site_cell, L.site_cell)]
        oi = np.broadcast_to(L.site_orb[:, None], (nd, nd))
        oj = np.broadcast_to(L.site_orb[None, :], (nd, nd))
        ns = self.n_sun

        def add(name, val):
            np.add.at(self.obs[name][:, 0], (rows, oi, oj), val * w)

        add("Green", ns * GRC)
        add("SpinZ", ns * GRC * GR)
        zi = ns * np.diag(GRC)
        add("Den", zi[:, None] * zi[None, :] + ns * GRC * GR)
        np.add.at(self.obs0["Den"], L.site_orb, zi * w)
        self.count += 1
        self.sign += float(np.sign(phase.real))

    def bin(self, reset: bool = True) -> Dict[str, dict]:
        """Print_bin_Latt's normalisation: per observable Obs_Latt / N, Obs_Latt0 / (N Ns Ntau)
        and Ave_sign / N (Ntau = 1)."""
        if self.count == 0:
            raise ValueError("an empty bin")
        n, ns = self.count, self.latt.N
        out = {k: {"latt": self.obs[k] / n, "latt0": self.obs0[k] / (n * ns), "sign": self.sign / n}
               for k in self.names}
        if reset:
            self.reset()
        return out


class TimeDisplacedObs:
    """Obs_tau of the predefined measurements on the quartets of ham%ObserT at NT = 0..Ltrot:
    Obs_Latt(imj, NT + 1, no_I, no_J), Obs_Latt0(no); N and Ave_sign count the NT = 0 calls.
    Files as EqualTimeObs (N_FL = 1: SpinZ by Predefined_Obs_tau_SpinSUN_measure)."""

    def __init__(self, latt: Lattice, n_sun: int, ntau: int, n_fl: int = 2):
        if n_fl not in (1, 2):
            raise ValueError("N_FL is 1 or 2")
        self.latt, self.n_sun, self.ntau, self.n_fl = latt, n_sun, ntau, n_fl
        self.names = names_for(n_fl)
        self.reset()

    def reset(self):
        no, N = self.latt.norb, self.latt.N
        self.obs = {k: np.zeros((N, self.ntau, no, no), np.complex128) for k in self.names}
        self.obs0 = {k: np.zeros(no, np.complex128) for k in self.names}
        self.count, self.sign = 0, 0.0

    def measure(self, nt: int, GT0, G0T, G00, GTT, phase: complex):
        """One ham%ObserT call: NT and the quartet, each [n_fl][row][col]."""
        GT0, G0T, G00, GTT = (np.asarray(x) for x in (GT0, G0T, G00, GTT))
        if GT0.shape[0] != self.n_fl:
            raise ValueError(f"the quartet has {GT0.shape[0]} flavours, expected {self.n_fl}")
        zp = phase / phase.real
        zs = float(np.sign(phase.real))
        w = zp * zs
        if nt == 0:
            self.count += 1
            self.sign += zs
        if self.n_fl == 1:
            return self._measure_sun(nt, GT0[0], G0T[0], G00[0], GTT[0], w)
        L = self.latt
        nd = GT0.shape[1]
        rows = L.imj[np.ix_(L.site_cell, L.site_cell)]
        oi = np.broadcast_to(L.site_orb[:, None], (nd, nd))
        oj = np.broadcast_to(L.site_orb[None, :], (nd, nd))
        ns = self.n_sun
        g0t = [G0T[f].T for f in range(2)]  # g0t[f][I1][J1] = G0T(J1, I1, f)

        def add(name, val):
            np.add.at(self.obs[name][:, nt], (rows, oi, oj), val * w)

        add("Green", (GT0[0] + GT0[1]) / 2.0)
        dtt = np.diag(GTT[0]) - np.diag(GTT[1])
        d00 = np.diag(G00[0]) - np.diag(G00[1])
        zz = dtt[:, None] * d00[None, :] - g0t[0] * GT0[0] - g0t[1] * GT0[1]
        zxy = -g0t[0] * GT0[1] - g0t[1] * GT0[0]
        add("SpinZ", zz)
        add("SpinXY", zxy)
        add("SpinT", (2.0 * zxy + zz) / 3.0)
        np.add.at(self.obs0["SpinZ"], L.site_orb, -dtt * w)
        np.add.at(self.obs0["SpinT"], L.site_orb, -dtt * w / math.sqrt(3.0))
        zi = ns * ((1.0 - np.diag(GTT[0])) + (1.0 - np.diag(GTT[1])))
        zj = ns * ((1.0 - np.diag(G00[0])) + (1.0 - np.diag(G00[1])))
        z = -ns * (g0t[0] * GT0[0] + g0t[1] * GT0[1])
        add("Den", zi[:, None] * zj[None, :] + z)
        np.add.at(self.obs0["Den"], L.site_orb, zi * w)

    def _measure_sun(self, nt, gt0, g0t, g00, gtt, w):
        """N_FL = 1: Green (GT0 / N_FL), SpinZ (-N_SUN G0T(J,I) GT0(I,J)) and Den."""
        L = self.latt
        nd = gt0.shape[0]
        rows = L.imj[np.ix_(L.site_cell, L.site_cell)]
        oi = np.broadcast_to(L.site_orb[:, None], (nd, nd))
        oj = np.broadcast_to(L.site_orb[None, :], (nd, nd))
        ns = self.n_sun

        def add(name, val):
            np.add.at(self.obs[name][:, nt], (rows, oi, oj), val * w)

        add("Green", gt0)
        conn = g0t.T * gt0
        add("SpinZ", -ns * conn)
        zi, zj = ns * (1.0 - np.diag(gtt)), ns * (1.0 - np.diag(g00))
        add("Den", zi[:, None] * zj[None, :] - ns * conn)
        np.add.at(self.obs0["Den"], L.site_orb, zi * w)

    def bin(self, reset: bool = True) -> Dict[str, dict]:
        """Obs_Latt / N, Obs_Latt0 / (N Ns Ntau), Ave_sign / N."""
        if self.count == 0:
            raise ValueError("an empty bin")
        n, ns = self.count, self.latt.N
        out = {k: {"latt": self.obs[k] / n, "latt0": self.obs0[k] / (n * ns * self.ntau), "sign": self.sign / n}
               for k in self.names}
        if reset:
            self.reset()
        return out


def _a20(label: str) -> str:
    return label.rjust(20) + ": "


def write_eq_bin(directory: str, name: str, b: dict, latt: Lattice, dtau: float, channel: str = "--") -> None:
    """Append one bin to ``<name>_eq`` (and write ``<name>_eq_info`` once), as the legacy
    branch of Print_bin_Latt does for Ntau = 1."""
    write_latt_bin(directory, name, b, latt, dtau, channel)


def write_latt_bin(directory: str, name: str, b: dict, latt: Lattice, dtau: float, channel: str = "--") -> None:
    """Append one bin to ``<name>_eq`` (Ntau = 1) or ``<name>_tau`` (Ntau > 1, the time
    slices taken from the bin) and write the ``_info`` file once (Print_bin_Latt)."""
    ntau = b["latt"].shape[1]
    suff = "_eq" if ntau == 1 else "_tau"
    os.makedirs(directory, exist_ok=True)
    base = os.path.join(directory, f"{name}{suff}")
    if not os.path.exists(base + "_info"):
        with open(base + "_info", "w") as f:
            f.write(_a20("Observable") + f"{name}{suff}\n")
            f.write(_a20("Channel") + f"{channel}\n")
            f.write(_a20("Ntau") + f"{ntau:10d}\n")
            f.write(_a20("dtau") + fortran_e(dtau, 26, 17) + "\n")
            f.write("       ====== Bravais Lattice ======\n")
            f.write(_a20("Unit cells") + f"{latt.N:10d}\n")
            for lab, v in (("L1", latt.L1p), ("L2", latt.L2p), ("a1", latt.a1), ("a2", latt.a2)):
                f.write(_a20(lab) + "".join(fortran_e(x, 26, 17) for x in v) + "\n")
            f.write("       ========= Unit cell =========\n")
            f.write(_a20("Coordination number") + f"{latt.n_coord:10d}\n")
            f.write(_a20("Number of orbitals") + f"{latt.norb:10d}\n")
            f.write(_a20("Ndim") + f"{len(latt.orb_pos[0]):10d}\n")
            for no, pos in enumerate(latt.orb_pos, start=1):
                f.write(_a20(f"Orbital {no}") + "".join(fortran_e(x, 26, 17) for x in pos) + "\n")
    xk = np.stack([latt.fourier_r_to_k(b["latt"][:, nt, no, no1]) for nt in range(ntau) for no in range(latt.norb)
                   for no1 in range(latt.norb)], axis=1)  # [k][(nt * norb + no) * norb + no1]

    def cz(z):
        z = complex(z)
        return f"({fortran_e(z.real, 25, 17)},{fortran_e(z.imag, 25, 17)})"

    with open(base, "a") as f:
        if ntau == 1:
            f.write(f"{fortran_e(b['sign'], 25, 17)}{latt.norb:11d}{latt.N:11d}\n")
        else:
            f.write(f"{fortran_e(b['sign'], 25, 17)}{latt.norb:11d}{latt.N:11d}{ntau:11d}{fortran_e(dtau, 26, 17)}\n")
        for no in range(latt.norb):
            f.write(cz(b["latt0"][no]) + "\n")
        for k in range(latt.N):
            f.write(f"{fortran_e(latt.K[k, 0], 25, 17)} {fortran_e(latt.K[k, 1], 25, 17)}\n")
            for v in xk[k]:
                f.write(cz(v) + "\n")


_NUM = r"[-+]?(?:\d+\.?\d*|\.\d+)(?:[EeDd][-+]?\d+)?"
_CPLX = re.compile(r"^\(\s*(" + _NUM + r")\s*,\s*(" + _NUM + r")\s*\)$")


def read_eq(path: str) -> List[dict]:
    """All bins of a legacy ``<name>_eq`` or ``<name>_tau`` file: per bin the sign, the
    background [norb], the k points [Ns][2] and the k-space values [Ns][Ntau][norb][norb]
    ([Ns][norb][norb] for ``_eq``)."""
    with open(path) as f:
        lines = [ln.strip() for ln in f if ln.strip()]

    def z(s):
        m = _CPLX.match(s)
        if not m:
            raise ValueError(f"not a complex value: {s!r}")
        return complex(float(m.group(1)), float(m.group(2)))

    out, p = [], 0
    while p < len(lines):
        head = lines[p].split()
        sign, norb, ns = float(head[0]), int(head[1]), int(head[2])
        ntau = int(head[3]) if len(head) > 3 else 1
        p += 1
        back = np.array([z(lines[p + i]) for i in range(norb)])
        p += norb
        ks, vals = np.zeros((ns, 2)), np.zeros((ns, ntau, norb, norb), np.complex128)
        for k in range(ns):
            ks[k] = [float(x) for x in lines[p].split()]
            p += 1
            for i in range(ntau * norb * norb):
                vals[k, i // (norb * norb), (i // norb) % norb, i % norb] = z(lines[p + i])
            p += ntau * norb * norb
        out.append({"sign": sign, "latt0": back, "k": ks, "values": vals[:, 0] if len(head) <= 3 else vals,
                    **({"dtau": float(head[4])} if len(head) > 4 else {})})
    return out


EPS_CONVERGENCE = 1.0e-6  # Natural_Constants Eps_convergence: the k = 0 test of ana_eq


def ana_eq(bins: Sequence[dict], latt: Lattice, n_skip: int = 1, n_rebin: int = 1):
    """ana_eq (Analysis/ana_mod.F90:1427-1648, default zone) on the bins read_eq returns:
    per k point and orbital pair the signed jackknife (analysis.jackknife_vec) of
    f(X) = X1 - X2 X3 with X1 the bin's value, and at k = 0 only X2 = Ns <O_no>, X3 = <O_no1>
    (the background), else 0; in real space (FT_K_to_R of the k-space bins) X2 = <O_no>,
    X3 = <O_no1> at every R.  Returns (jk, jr): complex arrays [Ns][norb][norb][2] of
    (mean, error)."""
    from .analysis import jackknife_vec
    b = list(bins)[n_skip:]
    if len(b) // n_rebin < 2:
        raise ValueError("effective number of bins smaller than 2")
    sgn = np.array([x["sign"] for x in b], dtype=np.complex128)
    vk = np.stack([x["values"] for x in b], axis=-1)  # [Ns][no][no1][nb]
    bg = np.stack([x["latt0"] for x in b], axis=-1)   # [no][nb]
    vr = np.stack([latt.fourier_k_to_r(x["values"]) for x in b], axis=-1)
    f = lambda X: X[0] - X[1] * X[2]
    ns, no = latt.N, latt.norb
    jk = np.zeros((ns, no, no, 2), np.complex128)
    jr = np.zeros((ns, no, no, 2), np.complex128)
    zero = np.zeros(len(b), np.complex128)
    for k in range(ns):
        at0 = float(np.hypot(*latt.K[k])) < EPS_CONVERGENCE
        for a in range(no):
            for c in range(no):
                V = np.stack([vk[k, a, c], bg[a] * ns if at0 else zero, bg[c] if at0 else zero])
                jk[k, a, c] = jackknife_vec(V, sgn, f, n_rebin)
                VR = np.stack([vr[k, a, c], bg[a], bg[c]])
                jr[k, a, c] = jackknife_vec(VR, sgn, f, n_rebin)
    return jk, jr


def write_ana_eq(directory: str, name: str, jk: np.ndarray, jr: np.ndarray, latt: Lattice) -> None:
    """``<name>JK`` and ``<name>JR`` as ana_eq writes them: per k point (R point) its
    coordinates as ``2(E26.17E3)``, then per orbital pair ``(2(I11), 4(E26.17E3))`` no, no1,
    Re mean, Re error, Im mean, Im error."""
    for suffix, arr, pts in (("JK", jk, latt.K), ("JR", jr, latt.R)):
        with open(os.path.join(directory, f"{name}{suffix}"), "w") as f:
            for n in range(latt.N):
                f.write(fortran_e(pts[n, 0], 26, 17) + fortran_e(pts[n, 1], 26, 17) + "\n")
                for a in range(latt.norb):
                    for c in range(latt.norb):
                        m, e = arr[n, a, c]
                        f.write(f"{a + 1:11d}{c + 1:11d}" + fortran_e(m.real, 26, 17) + fortran_e(e.real, 26, 17)
                                + fortran_e(m.imag, 26, 17) + fortran_e(e.imag, 26, 17) + "\n")
