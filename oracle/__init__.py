"""CPU oracle for the AFQMC sweep -- test infrastructure, not product code.

``alf_oracle.cpp`` restates ALF's default-STAB sequential sweep (see its
header for the reference file:line list) and calls the same LAPACK routines the
Fortran calls, resolved at run time from the OpenBLAS that ships inside SciPy.
Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline
leg use this package: as the reference results are compared with, and as the
reported CPU baseline.
"""
from __future__ import annotations

import ctypes
import glob
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "liboracle.so")
SRC = os.path.join(HERE, "alf_oracle.cpp")

_c = ctypes
_p = _c.c_void_p


def build(force: bool = False) -> str:
    """Compile the oracle with g++ (no cmake, no reference build system)."""
    os.makedirs(BUILD, exist_ok=True)
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(SRC):
        cmd = ["g++", "-O3", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", "-fcx-limited-range",
               SRC, "-o", LIB + ".tmp", "-ldl"]
        subprocess.check_call(cmd)
        os.replace(LIB + ".tmp", LIB)
    return LIB


def openblas_path() -> str:
    import scipy
    d = os.path.join(os.path.dirname(os.path.dirname(scipy.__file__)), "scipy.libs")
    cands = [p for p in glob.glob(os.path.join(d, "libscipy_openblas*.so*")) if "64_" not in os.path.basename(p)]
    if not cands:
        raise RuntimeError("no LP64 OpenBLAS found next to scipy")
    return sorted(cands)[0]


_lib = None


def lib():
    global _lib
    if _lib is not None:
        return _lib
    build()
    L = _c.CDLL(LIB)
    path = openblas_path().encode()
    rc = L.oracle_load_lapack(path, b"scipy_")
    if rc != 0:
        raise RuntimeError(f"oracle could not load LAPACK from {path!r} (rc={rc})")
    rc = L.oracle_load_getri(path, b"scipy_")
    if rc != 0:
        raise RuntimeError("oracle could not load zgetri")
    L.oracle_create.restype = _p
    L.oracle_create.argtypes = [_c.c_int] * 7
    L.oracle_destroy.argtypes = [_p]
    L.oracle_sweep_chunk.argtypes = [_p, _p, _c.c_int]
    L.oracle_sweep_chunk.restype = _c.c_int
    for name in ("oracle_init_state", "oracle_sweep", "oracle_get_green", "oracle_set_green",
                 "oracle_set_fields", "oracle_get_fields", "oracle_wrapgrup", "oracle_wrapgrdo"):
        getattr(L, name).restype = _c.c_int
    L.oracle_set_threads.argtypes = [_c.c_int]
    L.oracle_set_variant.argtypes = [_c.c_int]
    L.oracle_set_eq_callback.argtypes = [_p, EQ_CB, _p]
    L.oracle_set_tau_callback.argtypes = [_p, TAU_CB, _p]
    L.oracle_set_scalar_obs.argtypes = [_p, _p, _p]
    L.oracle_get_scalar_obs.argtypes = [_p, _p, _c.c_int]
    _lib = L
    return L


class _Z(_c.Structure):
    _fields_ = [("re", _c.c_double), ("im", _c.c_double)]


_PD = _c.POINTER(_c.c_double)
# ham%Obser: (ctx, ntau, G[F][N][N] col-major, phase); ham%ObserT: (ctx, ntau, GT0, G0T, G00, GTT, phase)
EQ_CB = _c.CFUNCTYPE(None, _p, _c.c_int, _PD, _Z)
TAU_CB = _c.CFUNCTYPE(None, _p, _c.c_int, _PD, _PD, _PD, _PD, _Z)


def set_variant(v: int) -> None:
    """Summation order of the hopping products: 0 = OpenBLAS (as linked by the
    reference), 1 = plain loops (what another BLAS build of the reference gives)."""
    lib().oracle_set_variant(v)


class OracleStats(_c.Structure):
    _fields_ = [("n_prop", _c.c_int64), ("n_acc", _c.c_int64), ("n_prop_eff", _c.c_int64),
                ("n_acc_eff", _c.c_int64), ("ncg", _c.c_int64), ("xmeanG_sum", _c.c_double),
                ("xmaxG", _c.c_double), ("xmaxP", _c.c_double), ("ncg_tau", _c.c_int64),
                ("xmean_tau_sum", _c.c_double), ("xmax_tau", _c.c_double)]


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(_p)


class Oracle:
    """One Markov chain on the CPU (``main.F90`` state: G, UDV stacks, fields)."""

    def __init__(self, model, ltau: int = 0, threads: int = 1):
        L = lib()
        L.oracle_set_threads(threads)
        self.model = model
        self.N, self.F, self.M, self.L = model.ndim, model.n_fl, model.n_op, model.ltrot
        self.h = L.oracle_create(model.ndim, model.n_fl, model.n_sun, model.n_op, model.ltrot, model.nwrap, ltau)
        if not self.h:
            raise RuntimeError("oracle_create failed")
        pk = model.pack()
        self._pk = pk  # keep alive
        rc = L.oracle_set_model(self.h, _ptr(pk["expT"]), _ptr(pk["expTinv"]), _ptr(pk["op_n"]), _ptr(pk["op_nz"]),
                                _ptr(pk["op_diag"]), _ptr(pk["op_type"]), _ptr(pk["op_P"]), _ptr(pk["op_g"]),
                                _ptr(pk["op_alpha"]), _ptr(pk["op_E"]), _ptr(pk["op_U"]), _ptr(pk["op_Eexp"]),
                                _ptr(pk["op_Mexp"]))
        if rc:
            raise RuntimeError(f"oracle_set_model rc={rc}")
        if "cb_P" in pk:  # checkerboard Op_T: the bond operators replace the dense exponentials
            ncheck = pk["cb_P"].shape[1]
            rc = L.oracle_set_checkerboard(self.h, ncheck, _ptr(pk["cb_P"]), _ptr(pk["cb_mat"]), _ptr(pk["cb_inv"]))
            if rc:
                raise RuntimeError(f"oracle_set_checkerboard rc={rc}")
        self._rec = None

    def __del__(self):
        if getattr(self, "h", None):
            lib().oracle_destroy(self.h)
            self.h = None

    def set_fields(self, f: np.ndarray):
        f = np.ascontiguousarray(f, dtype=np.int8)
        rc = lib().oracle_set_fields(self.h, _ptr(f))
        if rc:
            raise RuntimeError(f"oracle_set_fields rc={rc}")

    def fields(self) -> np.ndarray:
        f = np.zeros((self.L, self.M), np.int8)
        lib().oracle_get_fields(self.h, _ptr(f))
        return f

    def init_state(self) -> complex:
        ph = np.zeros(1, np.complex128)
        rc = lib().oracle_init_state(self.h, _ptr(ph))
        if rc:
            raise RuntimeError(f"oracle_init_state rc={rc}")
        return complex(ph[0])

    def record(self, n_sweeps: int = 1, green: bool = True):
        """Arm recording of accept bits, ratios and G at every stabilisation point."""
        nst = self.model.nstm
        nv = 2 * self.M * self.L * n_sweeps
        ns = 2 * nst * n_sweeps
        self._rec = dict(acc=np.zeros(nv, np.int8), ratio=np.zeros(nv, np.complex128),
                         G=np.zeros((ns, self.F, self.N, self.N), np.complex128) if green else None,
                         Gwrap=np.zeros((ns, self.F, self.N, self.N), np.complex128) if green else None,
                         phase=np.zeros(ns, np.complex128))
        r = self._rec
        lib().oracle_set_recording(self.h, _ptr(r["acc"]), _ptr(r["ratio"]),
                                   _ptr(r["G"]) if green else None, _ptr(r["Gwrap"]) if green else None,
                                   _ptr(r["phase"]))
        return r

    def recorded(self) -> dict:
        """Recorded data of the armed sweeps; G arrays as [point][nf][row][col]."""
        r = dict(self._rec)
        for k in ("G", "Gwrap"):
            if r[k] is not None:
                r[k] = np.transpose(r[k], (0, 1, 3, 2)).copy()
        return r

    def sweep(self, u: np.ndarray) -> None:
        u = np.ascontiguousarray(u, dtype=np.float64)
        assert u.size == 6 * self.M * self.L
        rc = lib().oracle_sweep(self.h, _ptr(u))
        if rc:
            raise RuntimeError(f"oracle_sweep rc={rc}")

    def sweep_chunk(self, u: np.ndarray, nslices: int) -> bool:
        """Advance the current sweep by nslices time slices (with their stabilisations).
        Returns True once the sweep is complete."""
        rc = lib().oracle_sweep_chunk(self.h, u.ctypes.data_as(_p), nslices)
        if rc < 0:
            raise RuntimeError(f"oracle_sweep_chunk rc={-rc}")
        return rc == 1

    def _mats(self, ptr) -> np.ndarray:
        a = np.ctypeslib.as_array(ptr, shape=(2 * self.F * self.N * self.N,)).view(np.complex128)
        return np.transpose(a.reshape(self.F, self.N, self.N), (0, 2, 1)).copy()  # -> [nf][row][col]

    def collect_measurements(self, keep=None):
        """Collect the equal-time (ham%Obser) and time-displaced (ham%ObserT) callbacks of
        the following sweeps: lists of (ntau, G, phase) and (ntau, [GT0, G0T, G00, GTT], phase).
        ``keep`` (kind, ntau) -> bool, kind 0 = equal-time and 1 = time-displaced, selects the
        callbacks that are copied (all by default)."""
        eq, tau = [], []

        def on_eq(ctx, ntau, G, ph):
            if keep is None or keep(0, ntau):
                eq.append((ntau, self._mats(G), complex(ph.re, ph.im)))

        def on_tau(ctx, ntau, a, b, c, d, ph):
            if keep is None or keep(1, ntau):
                tau.append((ntau, [self._mats(x) for x in (a, b, c, d)], complex(ph.re, ph.im)))

        self._cbs = (EQ_CB(on_eq), TAU_CB(on_tau))
        lib().oracle_set_eq_callback(self.h, self._cbs[0], None)
        lib().oracle_set_tau_callback(self.h, self._cbs[1], None)
        return eq, tau

    def set_scalar_obs(self, H=None, U=None):
        """Accumulate ZP ZS {Kin, Pot, Part, Ener}, ZS and the count at every ham%Obser point
        (the Hubbard Obs_scal, the same sums alfgpu_set_scalar_obs forms on the device).
        H: [n_fl][N][N] real hopping Hamiltonian (row index first); U: [N].  No arguments: off."""
        if H is None:
            lib().oracle_set_scalar_obs(self.h, None, None)
            return
        self._obs = (np.ascontiguousarray(np.transpose(np.asarray(H, np.float64).reshape(self.F, self.N, self.N),
                                                       (0, 2, 1))),
                     np.ascontiguousarray(np.asarray(U, np.float64).reshape(self.N)))
        lib().oracle_set_scalar_obs(self.h, _ptr(self._obs[0]), _ptr(self._obs[1]))

    def scalar_obs(self, reset: bool = False) -> dict:
        """Accumulators since the last reset: sums of ZP ZS {kin, pot, part, ener}, sum of ZS, count."""
        a = np.zeros(10, np.float64)
        lib().oracle_get_scalar_obs(self.h, _ptr(a), int(reset))
        return {"kin": complex(a[0], a[1]), "pot": complex(a[2], a[3]), "part": complex(a[4], a[5]),
                "ener": complex(a[6], a[7]), "sign": a[8], "count": int(a[9])}

    def green(self) -> np.ndarray:
        G = np.zeros((self.F, self.N, self.N), np.complex128)  # [nf][col][row] memory = col-major per flavour
        lib().oracle_get_green(self.h, _ptr(G))
        return np.transpose(G, (0, 2, 1)).copy()  # -> [nf][row][col]

    def set_green(self, G: np.ndarray):
        Gc = np.ascontiguousarray(np.transpose(G, (0, 2, 1)))
        lib().oracle_set_green(self.h, _ptr(Gc))

    def phase(self) -> complex:
        ph = np.zeros(1, np.complex128)
        lib().oracle_get_phase(self.h, _ptr(ph))
        return complex(ph[0])

    def stats(self) -> OracleStats:
        s = OracleStats()
        lib().oracle_get_stats(self.h, _c.byref(s))
        return s

    def wrapgrup(self, ntau: int, u3: np.ndarray):
        u3 = np.ascontiguousarray(u3, dtype=np.float64)
        lib().oracle_wrapgrup(self.h, ntau, _ptr(u3))

    def wrapgrdo(self, ntau: int, u3: np.ndarray):
        u3 = np.ascontiguousarray(u3, dtype=np.float64)
        lib().oracle_wrapgrdo(self.h, ntau, _ptr(u3))


def cgr(nvar, UR, DR, VR, UL, DL, VL):
    """``CGR`` on explicit UDV factors (row-major numpy in, row-major G out)."""
    N = UR.shape[0]
    cm = lambda A: np.ascontiguousarray(np.asarray(A, np.complex128).T)
    args = [cm(UR), np.ascontiguousarray(DR, np.complex128), cm(VR), cm(UL), np.ascontiguousarray(DL, np.complex128), cm(VL)]
    G = np.zeros((N, N), np.complex128)
    ph = np.zeros(1, np.complex128)
    lib().oracle_cgr(N, nvar, *[_ptr(a) for a in args], _ptr(G), _ptr(ph))
    return G.T.copy(), complex(ph[0])


def decompose(side: str, U, D, V):
    """``decompose_UDV_state`` on explicit factors; returns new (U, D, V)."""
    N = U.shape[0]
    Uc = np.ascontiguousarray(np.asarray(U, np.complex128).T)
    Vc = np.ascontiguousarray(np.asarray(V, np.complex128).T)
    Dc = np.ascontiguousarray(D, np.complex128).copy()
    lib().oracle_decompose(N, _c.c_char(side.encode()), _ptr(Uc), _ptr(Dc), _ptr(Vc))
    return Uc.T.copy(), Dc, Vc.T.copy()


def solve_extended_case(inp, UCT, VINV):
    """The reference's solve_extended_System test case (testsuite/Prog.tests/
    17-solve-extended-system.F90) on the oracle: QDRP of the 2N x 2N ``inp``, U3 = Q, V3 = the
    normalised R with its columns moved back by the pivots, D3, and
    HLP = solve_extended_System(UCT, VINV) (row-major numpy in and out)."""
    N = UCT.shape[0]
    N2 = 2 * N
    cm = lambda A: np.ascontiguousarray(np.asarray(A, np.complex128).T)
    A = cm(inp)
    U, V = np.zeros((N2, N2), np.complex128), np.zeros((N2, N2), np.complex128)
    H = np.zeros((N2, N2), np.complex128)
    D = np.zeros(N2, np.complex128)
    uct, vinv = cm(UCT), cm(VINV)
    rc = lib().oracle_solve_extended_case(N, _ptr(A), _ptr(uct), _ptr(vinv), _ptr(H), _ptr(U), _ptr(V), _ptr(D))
    if rc:
        raise RuntimeError(f"oracle_solve_extended_case: info {rc}")
    return H.T.copy(), U.T.copy(), V.T.copy(), D
