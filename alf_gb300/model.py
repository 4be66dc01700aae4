"""Model tables for the finite-temperature AFQMC sweep (host side, built once).

This module produces exactly the inputs ALF's Fortran ``Ham_Set`` hands to the
sweep: the dense hopping exponentials of ``Op_T`` and the interaction vertices
``Op_V`` with their exponential tables.  The GPU library and the CPU oracle both
consume the packed arrays built here, so the field-update arithmetic sees the
same numbers on both sides.

Reference files followed (paths inside the ALF tree):

* lattices / site numbering: ``Prog/Predefined_Latt_mod.F90:100-262``
  (``Invlist(I,no)`` = orbital-fastest numbering of unit cells)
* hopping matrices: ``Prog/Predefined_Hop_mod.F90:257-362`` (square),
  ``:827-906`` (honeycomb), ``:918-1216`` (bilayer square),
  dense ``Op_T`` assembly ``:1718-1772`` with ``g = -Dtau``
* exponentials of ``Op_T``: ``Prog/OpTTypes_mod.F90:92-133``
  (real storage, upper triangle symmetrised in place)
* ``Op_set``/``Op_exp``: ``Prog/Operator_mod.F90:259-529``
* Mz Hubbard vertices: ``Prog/Predefined_Int_mod.F90:121-148``; SU(N) Hubbard
  ``:59-76``; Kondo ``V_SUN`` ``:200-219``
* Hubbard ``Ham_V`` ordering: ``Prog/Hamiltonians/Hamiltonian_Hubbard_smod.F90:477-542``
* Kondo ``Ham_V`` ordering: ``Prog/Hamiltonians/Hamiltonian_Kondo_smod.F90:464-530``
* type-2 field tables: ``Prog/Fields_mod.F90:270-301``
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field
from typing import List, Optional

import numpy as np

# Fields_init (Prog/Fields_mod.F90:270-301): Gauss-Hermite 4-point HS tables.
SQ6 = math.sqrt(6.0)
PHI_TYPE2 = {-2: -math.sqrt(2.0 * (3.0 + SQ6)), -1: -math.sqrt(2.0 * (3.0 - SQ6)),
             1: math.sqrt(2.0 * (3.0 - SQ6)), 2: math.sqrt(2.0 * (3.0 + SQ6))}
GAMA_TYPE2 = {-2: 1.0 - SQ6 / 3.0, -1: 1.0 + SQ6 / 3.0, 1: 1.0 + SQ6 / 3.0, 2: 1.0 - SQ6 / 3.0}
FLIP_TYPE2 = {-2: (-1, 1, 2), -1: (1, 2, -2), 1: (2, -2, -1), 2: (-2, -1, 1)}

EPS_SMALL = 1.0e-10  # Natural_Constants Eps_small (threshold for zero eigenvalues)


def phi(s: int, op_type: int) -> float:
    """``Fields_Phi`` for discrete fields (Prog/Fields_mod.F90:112-133)."""
    if op_type == 1:
        return float(s)
    return PHI_TYPE2[s]


@dataclass
class Vertex:
    """One interaction operator ``Op_V(n,nf)`` after ``Op_set``.

    ``P`` are 0-based site indices; ``E_exp[m, s+2] = exp(g*E[m]*phi(s))`` for
    the first ``n_non_zero`` eigenvalues (1 otherwise); ``M_exp[s+2]`` is
    ``exp(g*phi(s)*O)`` in the original basis.
    """
    P: List[int]
    O: np.ndarray
    g: complex
    alpha: complex
    op_type: int = 2
    n_non_zero: int = 0
    diag: bool = True
    E: np.ndarray = field(default_factory=lambda: np.zeros(1))
    U: np.ndarray = field(default_factory=lambda: np.eye(1, dtype=complex))
    E_exp: np.ndarray = field(default_factory=lambda: np.ones((1, 5), dtype=complex))
    M_exp: np.ndarray = field(default_factory=lambda: np.ones((5, 1, 1), dtype=complex))

    @property
    def n(self) -> int:
        return len(self.P)


def op_set(v: Vertex) -> Vertex:
    """Eigen-decompose the operator and fill the exponential tables.

    Follows ``Op_set`` (Prog/Operator_mod.F90:259-472): diagonal operators keep
    ``U = 1`` and ``E = diag(O)``; otherwise the Hermitian eigenproblem is
    solved, eigenvectors with |E| > Eps_small are moved to the front, and the
    first column of ``U`` is divided by ``det(U)`` so that ``U`` is in SU(N).
    """
    n = v.n
    O = np.asarray(v.O, dtype=complex)
    if n == 1:
        v.diag = True
    else:
        off = O - np.diag(np.diag(O))
        v.diag = not np.any(off != 0)
    if v.diag:
        E = np.real(np.diag(O)).astype(float)
        U = np.eye(n, dtype=complex)
        nz = n
    else:
        w, Z = np.linalg.eigh(O)
        order_nz = [i for i in range(n) if abs(w[i]) > EPS_SMALL]
        order_z = [i for i in range(n) if abs(w[i]) <= EPS_SMALL]
        E = np.zeros(n)
        U = np.zeros((n, n), dtype=complex)
        for k, i in enumerate(order_nz):
            E[k] = w[i]
            U[:, k] = Z[:, i]
        for k, i in enumerate(order_z):
            E[n - 1 - k] = w[i]
            U[:, n - 1 - k] = Z[:, i]
        nz = len(order_nz)
        det = np.linalg.det(U)
        U[:, 0] = U[:, 0] / det
    v.E, v.U, v.n_non_zero = E, U, nz
    if v.op_type in (1, 2):
        t = v.op_type
        E_exp = np.ones((n, 5), dtype=complex)
        M_exp = np.zeros((5, n, n), dtype=complex)
        for I in range(1, t + 1):
            ph = phi(I, t)
            for m in range(n):
                if m < nz:
                    E_exp[m, I + 2] = np.exp(v.g * E[m] * ph)
                    E_exp[m, -I + 2] = 1.0 / E_exp[m, I + 2]
            M_exp[I + 2] = op_exp(v.g * ph, v)
            M_exp[-I + 2] = op_exp(-v.g * ph, v)
        if t == 1:
            M_exp[2] = np.eye(n)
            M_exp[0] = np.eye(n)
            M_exp[4] = np.eye(n)
        else:
            M_exp[2] = np.eye(n)
        v.E_exp, v.M_exp = E_exp, M_exp
    return v


def op_exp(g: complex, v: Vertex) -> np.ndarray:
    """``Op_exp`` (Prog/Operator_mod.F90:491-529): ``exp(g*O) = U exp(gE) U^H``."""
    if v.diag:
        return np.diag(np.exp(g * v.E)).astype(complex)
    return (v.U * np.exp(g * v.E)[None, :]) @ v.U.conj().T


# ----------------------------------------------------------------------------
# Lattices (Predefined_Latt_mod.F90) and hopping (Predefined_Hop_mod.F90)
# ----------------------------------------------------------------------------

def _cell(n1: int, n2: int, L1: int, L2: int) -> int:
    return (n1 % L1) + L1 * (n2 % L2)


# primitive vectors a1, a2 of the unit cells (Predefined_Latt_mod.F90:100-265)
_PRIMITIVE = {"SQUARE": ((1.0, 0.0), (0.0, 1.0)), "BILAYER_SQUARE": ((1.0, 0.0), (0.0, 1.0)),
              "HONEYCOMB": ((1.0, 0.0), (0.5, math.sqrt(3.0) / 2.0)), "N_LEG_LADDER": ((1.0, 0.0), (0.0, 1.0))}


def alf_cell_order(lattice: str, L1: int, L2: int) -> List[int]:
    """The unit cells in the order of ALF's Make_lattice (lattices_v3_mod.F90:88-336), as
    indices of this module's natural numbering (n1 fastest).

    Make_lattice walks i1 (outer) and i2 (inner) over -L..L, L the largest
    |BZ_i . L_j / 2 pi|, and keeps x = i1 a1 + i2 a2 when -|a|^2/2 < x . a <= |a|^2/2
    (within Eps_small) for a in {L2, L1, L2 - L1, L2 + L1}: one representative per
    periodic class, centred on the origin.  Here L1 = L1 a1 and L2 = L2 a2 (one cell
    along a2 for the N_leg_ladder, whose legs are orbitals), so (i1, i2) is the cell
    (i1 mod L1, i2 mod L2)."""
    lat = lattice.upper()
    a1, a2 = (np.array(v) for v in _PRIMITIVE[lat])
    n2c = 1 if lat == "N_LEG_LADDER" else L2
    L1p, L2p = L1 * a1, n2c * a2
    Minv = np.linalg.inv(np.array([a1, a2]))
    bz = [2.0 * math.pi * Minv[:, 0], 2.0 * math.pi * Minv[:, 1]]
    L = max(abs(int(round(float(b @ v) / (2.0 * math.pi)))) for b in bz for v in (L1p, L2p))
    tests = [L2p, L1p, L2p - L1p, L2p + L1p]
    order = []
    for i1 in range(-L, L + 1):
        for i2 in range(-L, L + 1):
            x = i1 * a1 + i2 * a2
            if all(float(x @ a) <= float(a @ a) / 2.0 + EPS_SMALL and float(x @ a) >= -float(a @ a) / 2.0 + EPS_SMALL
                   for a in tests):
                order.append(_cell(i1, i2, L1, n2c))
    if sorted(order) != list(range(L1 * n2c)):
        raise ValueError(f"{lattice} {L1}x{L2}: the centred cell does not tile the lattice")
    return order


def _site_permutation(lattice: str, L1: int, L2: int, norb: int, site_order: str) -> Optional[np.ndarray]:
    if site_order == "natural":
        return None
    if site_order != "alf":
        raise ValueError(f"site_order {site_order!r}: 'natural' or 'alf'")
    cells = alf_cell_order(lattice, L1, L2)
    return np.array([I * norb + o for I in cells for o in range(norb)])


def hopping_matrix(lattice: str, L1: int, L2: int, t: float = 1.0, chem: float = 0.0,
                   t2: float = 0.0, tperp: float = 0.0, site_order: str = "natural") -> np.ndarray:
    """Dense Hermitian hopping ``Op_T(1,nf)%O`` (no flux, no checkerboard).

    Bond tables follow ``Set_Default_hopping_parameters_*``; the assembly
    ``O(I1,J1) = T; O(J1,I1) = conj(T); O(I1,I1) = T_loc`` follows
    Prog/Predefined_Hop_mod.F90:1730-1761.  Sites are ``cell * norb + orbital``; cells
    are numbered n1 fastest (``site_order="natural"``) or in Make_lattice's order
    (``"alf"``, see alf_cell_order), which is ALF's Invlist and vertex order.
    """
    lat0, L1_0, L2_0 = lattice, L1, L2
    lat = lattice.upper()
    if lat == "SQUARE":
        norb = 1
        bonds = [(0, 0, 0, 1, -t), (0, 0, 1, 0, -t)]
        tloc = [-chem]
    elif lat == "HONEYCOMB":
        norb = 2
        bonds = [(0, 1, 0, 0, -t), (1, 0, 0, 1, -t), (0, 1, 1, -1, -t)]
        tloc = [-chem, -chem]
    elif lat == "BILAYER_SQUARE":
        norb = 2
        bonds = [(0, 0, 1, 0, -t), (0, 0, 0, 1, -t), (1, 1, 1, 0, -t2), (1, 1, 0, 1, -t2),
                 (0, 1, 0, 0, -tperp)]
        tloc = [-chem, -chem]
    elif lat == "N_LEG_LADDER":
        # Predefined_Latt_mod.F90:133-146 and Predefined_Hop_mod.F90:631-812: L1 cells along
        # the legs (periodic), the L2 legs are the orbitals of one cell (open across legs)
        if L1 != 1 and L1 % 2 != 0:
            raise ValueError("the N_leg_ladder hopping needs L1 = 1 or L1 even")
        norb = L2
        bonds = [(n, n, 1, 0, -t) for n in range(L2)] + [(n, n + 1, 0, 0, -tperp) for n in range(L2 - 1)]
        tloc = [-chem] * L2
        L2 = 1
    else:
        raise ValueError(f"lattice {lattice!r} not supported")
    ncell = L1 * L2
    N = ncell * norb
    O = np.zeros((N, N), dtype=complex)
    for n2 in range(L2):
        for n1 in range(L1):
            I = _cell(n1, n2, L1, L2)
            for (oi, oj, d1, d2, tb) in bonds:
                J = _cell(n1 + d1, n2 + d2, L1, L2)
                i1 = I * norb + oi
                j1 = J * norb + oj
                O[i1, j1] = tb
                O[j1, i1] = np.conj(tb)
            for o in range(norb):
                O[I * norb + o, I * norb + o] = tloc[o]
    p = _site_permutation(lat0, L1_0, L2_0, norb, site_order)
    return O if p is None else O[np.ix_(p, p)]


def exp_hopping(O: np.ndarray, dtau: float):
    """``RealExpOpT_init`` (Prog/OpTTypes_mod.F90:92-133).

    Returns ``(mat, invmat)`` = real parts of ``exp(-dtau*O)`` and
    ``exp(+dtau*O)``, with the upper triangle replaced in place by the
    symmetrised value ``(a_ij + a_ji)/2`` (the lower triangle keeps the raw
    value, as the Fortran loop leaves it).
    """
    w, Z = np.linalg.eigh(O)
    mats = []
    for g in (-dtau, dtau):
        m = np.real((Z * np.exp(g * w)[None, :]) @ Z.conj().T).copy()
        iu = np.triu_indices(m.shape[0])
        sym = 0.5 * (m + m.T)
        m[iu] = sym[iu]
        mats.append(m)
    return mats[0], mats[1]


def checkerboard_ops(lattice: str, L1: int, L2: int, dtau: float, t: float = 1.0, chem: float = 0.0,
                     site_order: str = "natural") -> dict:
    """Checkerboard ``Op_T`` of the square and honeycomb lattices: one two-site operator per
    bond, in ALF's family order (Predefined_Hop_mod.F90:331-361 square: four families, the a2
    and a1 bonds of the cells with even i1 + i2, then those of the odd cells (even L1, L2);
    :893-904 honeycomb: three families, one per bond of the unit cell).  Each operator is
    ``O = [[T_loc(no_I)/m(no_I), T], [conj T, T_loc(no_J)/m(no_J)]]`` on (I1, J1) with the
    orbital multiplicities m of the bond table and ``g = -dtau`` (Predefined_Hop_mod.F90:
    1780-1835).  Returns P [Ncheck][2] (0-based sites), mat = exp(g O), inv = exp(-g O)
    [Ncheck][2][2], and fam: the first operator of each family and Ncheck."""
    lat = lattice.upper()
    if lat == "SQUARE":
        if L1 % 2 or L2 % 2:
            raise ValueError("the square-lattice checkerboard decomposition needs even L1 and L2")
        norb, bonds = 1, [(0, 0, 0, 1), (0, 0, 1, 0)]
        fam_of = lambda n1, n2: [(0 if (n1 + n2) % 2 == 0 else 2) + b for b in range(2)]
        nfam = 4
    elif lat == "HONEYCOMB":
        norb, bonds = 2, [(0, 1, 0, 0), (1, 0, 0, 1), (0, 1, 1, -1)]
        fam_of = lambda n1, n2: [0, 1, 2]
        nfam = 3
    else:
        raise ValueError(f"no checkerboard decomposition for {lattice!r}")
    mult = [0] * norb
    for (oi, oj, _, _) in bonds:
        mult[oi] += 1
        mult[oj] += 1
    perm = _site_permutation(lattice, L1, L2, norb, site_order)
    new_of = np.arange(L1 * L2 * norb) if perm is None else np.argsort(perm)
    fams = [[] for _ in range(nfam)]
    for I in alf_cell_order(lattice, L1, L2):  # the cells in Latt%List order
        n1, n2 = I % L1, I // L1
        for b, f in enumerate(fam_of(n1, n2)):
            oi, oj, d1, d2 = bonds[b]
            J = _cell(n1 + d1, n2 + d2, L1, L2)
            fams[f].append((int(new_of[I * norb + oi]), int(new_of[J * norb + oj]),
                            np.array([[-chem / mult[oi], -t], [-t, -chem / mult[oj]]])))
    P, mats, invs, fam = [], [], [], []
    for ops in fams:
        fam.append(len(P))
        for i, j, O in ops:
            m, mi = exp_hopping(O, dtau)
            P.append((i, j))
            mats.append(m)
            invs.append(mi)
    fam.append(len(P))
    return {"P": np.array(P, np.int32), "mat": np.array(mats), "inv": np.array(invs), "fam": fam}


def checkerboard_product(cb: dict, N: int, inverse: bool = False) -> np.ndarray:
    """Dense B_T = E_1 E_2 ... E_Ncheck (or its inverse E_Ncheck^-1 ... E_1^-1) of the bond
    operators, the matrix Hop_mod_mmthr applies."""
    B = np.eye(N)
    seq = range(len(cb["P"])) if not inverse else range(len(cb["P"]) - 1, -1, -1)
    for nc in seq:
        i, j = cb["P"][nc]
        E = np.eye(N)
        E[np.ix_([i, j], [i, j])] = cb["inv" if inverse else "mat"][nc]
        B = B @ E
    return B


# ----------------------------------------------------------------------------
# Model container
# ----------------------------------------------------------------------------

@dataclass
class Model:
    """Everything the sweep needs, in the layout of the C ABI.

    ``vertices[nf][n]`` is ``Op_V(n+1, nf+1)``; ``expT[nf]``/``expTinv[nf]`` are
    the real ``mat``/``invmat`` of the single dense ``Op_T(1,nf)``.
    """
    name: str
    ndim: int
    n_fl: int
    n_sun: int
    ltrot: int
    nwrap: int
    dtau: float
    beta: float
    expT: np.ndarray
    expTinv: np.ndarray
    vertices: List[List[Vertex]]
    params: dict = field(default_factory=dict)
    checkerboard: Optional[dict] = None  # checkerboard_ops of each flavour's Op_T, or None (dense)

    @property
    def n_op(self) -> int:
        return len(self.vertices[0])

    @property
    def nstm(self) -> int:
        return -(-self.ltrot // self.nwrap)

    def stab_nt(self) -> List[int]:
        """``Stab_nt(0:Nstm)`` (Prog/main.F90:446-457)."""
        nstm = self.nstm
        s = [0] + [self.nwrap * n for n in range(1, nstm)] + [self.ltrot]
        return s

    def pack(self) -> dict:
        """Struct-of-arrays vertex tables, index ``k = nf*M + n``."""
        F, M = self.n_fl, self.n_op
        K = F * M
        out = {
            "op_n": np.zeros(K, np.int32), "op_nz": np.zeros(K, np.int32),
            "op_diag": np.zeros(K, np.int32), "op_type": np.zeros(K, np.int32),
            "op_P": np.zeros((K, 2), np.int32), "op_g": np.zeros(K, np.complex128),
            "op_alpha": np.zeros(K, np.complex128), "op_E": np.zeros((K, 2), np.float64),
            "op_U": np.zeros((K, 2, 2), np.complex128),      # [k][col][row]
            "op_Eexp": np.ones((K, 2, 5), np.complex128),    # [k][m][s+2]
            "op_Mexp": np.zeros((K, 5, 2, 2), np.complex128),  # [k][s+2][col][row]
        }
        for nf in range(F):
            for n in range(M):
                v = self.vertices[nf][n]
                k = nf * M + n
                nn = v.n
                if nn > 2:
                    raise ValueError("operators with more than 2 sites are not supported")
                out["op_n"][k] = nn
                out["op_nz"][k] = v.n_non_zero
                out["op_diag"][k] = int(v.diag)
                out["op_type"][k] = v.op_type
                out["op_P"][k, :nn] = v.P
                out["op_g"][k] = v.g
                out["op_alpha"][k] = v.alpha
                out["op_E"][k, :nn] = v.E
                out["op_U"][k, :nn, :nn] = v.U.T  # column-major storage
                out["op_Eexp"][k, :nn, :] = v.E_exp
                for s in range(5):
                    out["op_Mexp"][k, s, :nn, :nn] = v.M_exp[s].T
        out["expT"] = np.ascontiguousarray(np.stack([m.T for m in self.expT]))   # col-major per flavour
        out["expTinv"] = np.ascontiguousarray(np.stack([m.T for m in self.expTinv]))
        if self.checkerboard is not None:  # [F][Ncheck][2] sites, [F][Ncheck][4] column-major 2 x 2
            out["cb_P"] = np.ascontiguousarray(np.stack([c["P"] for c in self.checkerboard]), dtype=np.int32)
            out["cb_mat"] = np.ascontiguousarray(np.stack([np.transpose(c["mat"], (0, 2, 1)).reshape(-1, 4)
                                                           for c in self.checkerboard]))
            out["cb_inv"] = np.ascontiguousarray(np.stack([np.transpose(c["inv"], (0, 2, 1)).reshape(-1, 4)
                                                           for c in self.checkerboard]))
            out["cb_fam"] = np.ascontiguousarray(self.checkerboard[0]["fam"], dtype=np.int32)
        return out


def _mz_pair(site: int, dtau: float, U: float):
    """``Predefined_Int_U_MZ`` (Prog/Predefined_Int_mod.F90:121-148)."""
    g = complex(math.sqrt(dtau * U / 2.0), 0.0)
    up = op_set(Vertex(P=[site], O=np.ones((1, 1), complex), g=g, alpha=-0.5, op_type=2))
    do = op_set(Vertex(P=[site], O=np.ones((1, 1), complex), g=-g, alpha=-0.5, op_type=2))
    return up, do


def hubbard(lattice: str = "square", L1: int = 4, L2: int = 4, t: float = 1.0, U: float = 4.0,
            chem: float = 0.0, beta: float = 4.0, dtau: float = 0.1, nwrap: int = 10,
            n_sun_input: int = 2, tperp: float = 0.0, site_order: str = "natural",
            checkerboard: bool = False) -> Model:
    """Mz Hubbard model with dense hopping, as ``Ham_Set`` builds it.

    ``N_FL = 2`` and ``N_SUN`` is halved (Hamiltonian_Hubbard_smod.F90:264-266);
    the interaction strength per vertex is ``U/N_SUN`` (``:503``) and one
    vertex per site is created in ``Invlist`` order (``:505-517``).
    """
    ltrot = int(round(beta / dtau))
    n_sun = n_sun_input // 2
    O = hopping_matrix(lattice, L1, L2, t=t, chem=chem, tperp=tperp, site_order=site_order)
    N = O.shape[0]
    cb = None
    if checkerboard:  # Checkerboard = .T.: the product of the bond exponentials replaces exp(-dtau T)
        cb = checkerboard_ops(lattice, L1, L2, dtau, t=t, chem=chem, site_order=site_order)
        mat, inv = checkerboard_product(cb, N), checkerboard_product(cb, N, inverse=True)
    else:
        mat, inv = exp_hopping(O, dtau)
    up, do = [], []
    u_eff = U / n_sun
    for i in range(N):
        a, b = _mz_pair(i, dtau, u_eff)
        up.append(a)
        do.append(b)
    return Model(name=f"hubbard_{lattice.lower()}_{L1}x{L2}", ndim=N, n_fl=2, n_sun=n_sun,
                 ltrot=ltrot, nwrap=nwrap, dtau=dtau, beta=beta, expT=[mat, mat.copy()],
                 expTinv=[inv, inv.copy()], vertices=[up, do],
                 params=dict(lattice=lattice, L1=L1, L2=L2, t=t, U=U, chem=chem, tperp=tperp,
                             site_order=site_order, checkerboard=checkerboard),
                 checkerboard=None if cb is None else [cb, cb])


def kondo(L1: int = 12, L2: int = 12, t: float = 1.0, JK: float = 1.5, Uf: float = 2.0,
          chem: float = 0.0, beta: float = 10.0, dtau: float = 0.1, nwrap: int = 10,
          n_sun: int = 2, site_order: str = "natural") -> Model:
    """SU(N) Kondo lattice on the bilayer square lattice (N_FL = 1).

    Vertex order follows Hamiltonian_Kondo_smod.F90:464-530: first the ``Uf``
    vertices on f orbitals (``Predefined_Int_U_SUN``, imaginary ``g``), then
    one ``V_SUN`` vertex per c-f pair with ``JK/2`` (N_SUN = 2 branch).
    """
    ltrot = int(round(beta / dtau))
    O = hopping_matrix("BILAYER_SQUARE", L1, L2, t=t, chem=chem, t2=0.0, tperp=0.0, site_order=site_order)
    N = O.shape[0]
    mat, inv = exp_hopping(O, dtau)
    verts = []
    ncell = L1 * L2
    if abs(Uf) > EPS_SMALL:
        g = np.sqrt(complex(-dtau * Uf / n_sun, 0.0))
        for I in range(ncell):
            f = I * 2 + 1
            verts.append(op_set(Vertex(P=[f], O=np.ones((1, 1), complex), g=g, alpha=-0.5, op_type=2)))
    if abs(JK) > EPS_SMALL:
        if n_sun != 2:
            raise ValueError("only the N_SUN = 2 Kondo coupling is built here")
        g = complex(math.sqrt(dtau * (JK / 2.0) / n_sun), 0.0)
        Oj = np.array([[0, 1], [1, 0]], dtype=complex)
        for I in range(ncell):
            c, f = I * 2, I * 2 + 1
            verts.append(op_set(Vertex(P=[c, f], O=Oj, g=g, alpha=0.0, op_type=2)))
    return Model(name=f"kondo_bilayer_{L1}x{L2}", ndim=N, n_fl=1, n_sun=n_sun, ltrot=ltrot,
                 nwrap=nwrap, dtau=dtau, beta=beta, expT=[mat], expTinv=[inv], vertices=[verts],
                 params=dict(lattice="bilayer_square", L1=L1, L2=L2, t=t, JK=JK, Uf=Uf, chem=chem,
                             site_order=site_order))


# Named workloads (sizes as quoted in the project's benchmark configurations).
def config(name: str, **over) -> Model:
    name = name.lower()
    if name == "hubbard4x4":
        return hubbard("square", 4, 4, U=4.0, beta=4.0, dtau=0.1, nwrap=10, **over)
    if name == "hubbard16x16":
        return hubbard("square", 16, 16, U=4.0, beta=10.0, dtau=0.1, nwrap=10, **over)
    if name == "honeycomb12x12":
        return hubbard("honeycomb", 12, 12, U=5.0, beta=20.0, dtau=0.05, nwrap=5, **over)
    if name == "kondo12x12":
        return kondo(12, 12, JK=1.5, Uf=2.0, beta=10.0, dtau=0.1, nwrap=10, **over)
    raise KeyError(name)


def batch_groups(seed: int, n: int = 128) -> dict:
    """The batched Hubbard workload: chain c in [0, n) draws from its own generator
    (numpy's default_rng([seed, c])) a square L in {6, 8, 10, 12, 14, 16}, beta in
    {4, 6, 8, 10} (dtau 0.1, so Ltrot 40..100) and U uniform in [2, 8].  Returns
    {(L, beta): [(chain, U), ...]}: the chains grouped by (N_dim, Ltrot), one handle each."""
    groups = {}
    for c in range(n):
        r = np.random.default_rng([seed, c])
        L = int(r.choice([6, 8, 10, 12, 14, 16]))
        beta = float(r.choice([4.0, 6.0, 8.0, 10.0]))
        U = float(r.uniform(2.0, 8.0))
        groups.setdefault((L, beta), []).append((c, U))
    return groups
