"""Host-side API over the GPU library, mirroring ALF's sweep interface.

``Chains`` owns one library handle (``alfgpu_create``) for ``n_chains``
Markov chains that share lattice size, Ltrot and Nwrap.  Its methods map onto
the Fortran driver's steps:

=========================  =============================================
``Chains.init_state()``    Prog/main.F90:589-631 (WRAPUL chain + CGR)
``Chains.sweep()``         Prog/main.F90:714-887 (up pass, down pass,
                           stabilisations, TAU_M when enabled)
``Chains.green(c)``        GR(:,:,:) of chain c
``Chains.stats(c)``        Control_upgrade / Control_Precision* counters
=========================  =============================================
"""
from __future__ import annotations

import ctypes as C
from typing import Optional, Sequence

import numpy as np

from . import _lib
from .model import Model

PRECISIONS = {"fp64": 0, "mixed": 1}
# dims.reserved[0] flags (include/alfgpu.h)
FLAG_DF_PROPAGATION = 1
FLAG_EXACT_QRP = 2
FLAG_NORM_PIVOT_CGR = 4
FLAG_NORM_PIVOT_DECOMPOSE = 8
FLAG_NORM_PIVOT = 12
FLAG_DF_STAB_QR = 16
FLAG_DF_STAB_GEMM = 32
FLAG_DF_STAB = 48
FLAG_NO_GRAPH = 64
FLAG_NO_TENSOR_GEMM = 128
FLAG_FP64_STAB_GEMM = 256
FLAG_TENSOR_WIDE = 512
FLAG_QR_HALF_CLUSTER = 1024
FLAG_QR_FULL_CLUSTER = 2048
FLAG_DF_FLUSH = 4096
FLAG_QR_GLOBAL_ROWS = 8192
FLAG_NO_OVERLAP = 16384
FLAG_OZ_FLUSH_SINGLE = 32768
FLAG_FP64_VISITS = 65536
FLAG_OZ_DEEP_RING = 131072
FLAG_OZ_FLUSH_RESIDENT = 262144
FLAG_QR_TWO_PASS = 524288
# "default": ZGEQP3 everywhere in the FP64 form; norm-pivoted CGR in the mixed form
PIVOTING = {"default": 0, "exact": FLAG_EXACT_QRP, "norms": FLAG_NORM_PIVOT,
            "norms-cgr": FLAG_NORM_PIVOT_CGR, "norms-decompose": FLAG_NORM_PIVOT_DECOMPOSE}


def _p(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


class Chains:
    def __init__(self, model: Model, n_chains: int = 1, precision: str = "fp64", delay_k: int = 0,
                 device: int = 0, ltau: int = 0, models: Optional[Sequence[Model]] = None,
                 pivoting: str = "default", flags: int = 0, wrap_bits: int = 0, propagate_bits: int = 0):
        """``pivoting``: "exact" uses ZGEQP3's dynamic column pivoting (ALF's default branch)
        for every stabilisation QR; "norms" orders the columns once by their norms (ALF's
        STABLOG pivoting) and factors them with the blocked QR; "norms-cgr" /
        "norms-decompose" do so at one call site; "default" is "exact".  ``wrap_bits`` / ``propagate_bits`` (mixed form): target
        bits of the digit-sliced tensor-core products of the G wraps (and TAU_M) / of the UDV
        propagation (dims.reserved[1] / [2]; 0 = the full ~54)."""
        self.L = _lib.lib()
        self.model = model
        self.C = n_chains
        self.N, self.F, self.M, self.Lt = model.ndim, model.n_fl, model.n_op, model.ltrot
        d = _lib.Dims(model.ndim, model.n_fl, model.n_sun, model.n_op, model.ltrot, model.nwrap, n_chains,
                      PRECISIONS[precision], delay_k, ltau, device)
        d.reserved[0] = PIVOTING[pivoting] | flags
        d.reserved[1] = wrap_bits
        d.reserved[2] = propagate_bits
        h = C.c_void_p()
        _lib.check(self.L.alfgpu_create(C.byref(h), C.byref(d)), "alfgpu_create")
        self.h = h
        self._keep = []
        pk = model.pack()
        _lib.check(self.L.alfgpu_upload_hopping(self.h, _p(pk["expT"]), _p(pk["expTinv"])), "alfgpu_upload_hopping")
        if "cb_P" in pk:  # checkerboard Op_T: the bond operators replace the dense products
            self._keep.append(pk)
            _lib.check(self.L.alfgpu_upload_checkerboard(self.h, pk["cb_P"].shape[1], len(pk["cb_fam"]) - 1,
                                                         _p(pk["cb_fam"]), _p(pk["cb_P"]), _p(pk["cb_mat"]),
                                                         _p(pk["cb_inv"])), "alfgpu_upload_checkerboard")
        if models is None:
            self._upload_vertices(-1, pk)
        else:
            if len(models) != n_chains:
                raise ValueError(f"{len(models)} models for {n_chains} chains")
            for c, m in enumerate(models):
                self._upload_vertices(c, m.pack())

    def _upload_vertices(self, chain: int, pk: dict):
        v = _lib.Vertices(*[_p(np.ascontiguousarray(pk[k])).value for k in
                            ("op_n", "op_nz", "op_diag", "op_type", "op_P", "op_g", "op_alpha", "op_E",
                             "op_U", "op_Eexp", "op_Mexp")])
        self._keep.append(pk)
        _lib.check(self.L.alfgpu_upload_vertices(self.h, chain, C.byref(v)), "alfgpu_upload_vertices")

    def close(self):
        if getattr(self, "h", None):
            self.L.alfgpu_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    # --- fields and draws -------------------------------------------------------------------
    def set_fields(self, chain: int, f: np.ndarray):
        f = np.ascontiguousarray(f, dtype=np.int8)
        if f.shape != (self.Lt, self.M):
            raise ValueError(f"fields of shape {f.shape}, expected {(self.Lt, self.M)}")
        _lib.check(self.L.alfgpu_set_fields(self.h, chain, _p(f)), "alfgpu_set_fields")

    def set_fields_c128(self, chain: int, f: np.ndarray):
        """The fields as ALF stores them (nsigma%f: complex, values +-1 / +-2), [Ltrot][M]."""
        z = np.ascontiguousarray(f, dtype=np.complex128)
        if z.shape != (self.Lt, self.M):
            raise ValueError(f"fields of shape {z.shape}, expected {(self.Lt, self.M)}")
        _lib.check(self.L.alfgpu_set_fields_c128(self.h, chain, _p(z)), "alfgpu_set_fields_c128")

    def fields(self, chain: int) -> np.ndarray:
        f = np.zeros((self.Lt, self.M), np.int8)
        _lib.check(self.L.alfgpu_get_fields(self.h, chain, _p(f)), "alfgpu_get_fields")
        return f

    def set_rng(self, chain: int, seed: int, counter: int):
        _lib.check(self.L.alfgpu_set_rng(self.h, chain, seed, counter), "alfgpu_set_rng")

    # --- the sweep -----------------------------------------------------------------------------
    def init_state(self) -> np.ndarray:
        ph = np.zeros(self.C, np.complex128)
        _lib.check(self.L.alfgpu_init_state(self.h, _p(ph)), "alfgpu_init_state")
        return ph

    def sweep(self, uniforms: Optional[np.ndarray] = None, measure: bool = False, keep=None):
        """One sweep on every chain.  With ``measure``, the library's ham%Obser / ham%ObserT
        callbacks are collected: returns (eq, tau), lists of (chain, ntau, G, phase) and
        (chain, ntau, [GT0, G0T, G00, GTT], phase), matrices as [nf][row][col].  ``keep``
        (kind, chain, ntau) -> bool, kind 0 = equal-time and 1 = time-displaced, selects the
        callbacks that are copied (all by default)."""
        eq, tau = [], []
        NN = self.N * self.N

        def mats(ptr, k):
            a = np.ctypeslib.as_array(ptr, shape=(2 * k * self.F * NN,)).view(np.complex128)
            return np.transpose(a.reshape(k, self.F, self.N, self.N), (0, 1, 3, 2)).copy()

        def on_obs(ctx, chain, ntau, kind, G, ph):
            if keep is not None and not keep(kind, chain, ntau):
                return
            phase = complex(ph[0], ph[1])
            if kind == 0:
                eq.append((chain, ntau, mats(G, 1)[0], phase))
            else:
                tau.append((chain, ntau, list(mats(G, 4)), phase))

        cb = _lib.OBS_CB(on_obs) if measure else _lib.OBS_CB()
        if uniforms is not None:
            u = np.ascontiguousarray(uniforms, dtype=np.float64)
            if u.size != self.C * 6 * self.M * self.Lt:
                raise ValueError(f"{u.size} draws, expected {self.C * 6 * self.M * self.Lt} (chains x 6 M Ltrot)")
            rc = self.L.alfgpu_sweep(self.h, _p(u), cb, None)
        else:
            rc = self.L.alfgpu_sweep(self.h, None, cb, None)
        _lib.check(rc, "alfgpu_sweep" + (f" ({self.L.alfgpu_last_error(self.h).decode()})" if rc == 100 else ""))
        return (eq, tau) if measure else None

    # --- delay depth ---------------------------------------------------------------------------
    def set_delay(self, k: int):
        _lib.check(self.L.alfgpu_set_delay(self.h, k), "alfgpu_set_delay")

    def delay(self) -> int:
        k = C.c_int32()
        _lib.check(self.L.alfgpu_get_delay(self.h, C.byref(k)), "alfgpu_get_delay")
        return k.value

    def tune_delay(self, nsweeps: int = 1) -> int:
        """Autotune the delay depth on nsweeps device-stream sweeps per candidate (these
        sweeps advance the chains: use them as thermalisation)."""
        k = C.c_int32()
        _lib.check(self.L.alfgpu_tune_delay(self.h, nsweeps, C.byref(k)), "alfgpu_tune_delay")
        return k.value

    # --- device-side scalar observables ----------------------------------------------------------
    def set_scalar_obs(self, H: Optional[np.ndarray] = None, U: Optional[np.ndarray] = None):
        """Accumulate Kin, Pot, Part, Ener on the device at every ham%Obser point (see
        alfgpu_set_scalar_obs).  H: [n_fl][N][N] real hopping Hamiltonian (row index first);
        U: [N].  No arguments: off."""
        if H is None:
            _lib.check(self.L.alfgpu_set_scalar_obs(self.h, None, None), "alfgpu_set_scalar_obs")
            return
        Hc = np.ascontiguousarray(np.transpose(np.asarray(H, np.float64).reshape(self.F, self.N, self.N),
                                               (0, 2, 1)))  # column-major per flavour
        Uc = np.ascontiguousarray(np.asarray(U, np.float64).reshape(self.N))
        self._keep.append((Hc, Uc))
        _lib.check(self.L.alfgpu_set_scalar_obs(self.h, _p(Hc), _p(Uc)), "alfgpu_set_scalar_obs")

    def scalar_obs(self, chain: int = 0) -> dict:
        """Accumulators of one chain: sums of ZP ZS {kin, pot, part, ener}, sum of ZS (sign), count."""
        a = np.zeros(10, np.float64)
        _lib.check(self.L.alfgpu_get_scalar_obs(self.h, chain, _p(a)), "alfgpu_get_scalar_obs")
        return {"kin": complex(a[0], a[1]), "pot": complex(a[2], a[3]), "part": complex(a[4], a[5]),
                "ener": complex(a[6], a[7]), "sign": a[8], "count": int(a[9])}

    def reset_scalar_obs(self):
        _lib.check(self.L.alfgpu_reset_scalar_obs(self.h), "alfgpu_reset_scalar_obs")

    def scalar_bin(self, reset: bool = True):
        """One bin of the scalar observables: per chain Obs_vec / N and Ave_sign / N, averaged
        over the handle's chains as ALF averages walkers (alf_gb300.bins); then, with reset,
        the accumulators are cleared for the next bin.  Returns (Kin, Pot, Part, Ener), sign."""
        from . import bins
        b = bins.walker_mean(bins.bin_from_sums(self.scalar_obs(c)) for c in range(self.C))
        if reset:
            self.reset_scalar_obs()
        return b

    # --- device-side lattice-resolved observables ------------------------------------------------
    def set_lattice_obs(self, latt=None):
        """Accumulate the predefined lattice observables (lattice_obs.EQ_NAMES / EQ_NAMES_SUN, as
        lattice_obs.EqualTimeObs and TimeDisplacedObs form them on the host) on the device at
        every ham%Obser point and, with TAU_M, every ham%ObserT slice.  latt: a
        lattice_obs.Lattice of the model's lattice and site order; None switches it off."""
        if latt is None:
            _lib.check(self.L.alfgpu_set_lattice_obs(self.h, 0, 0, None, None), "alfgpu_set_lattice_obs")
            return
        site_of = np.zeros((latt.N, latt.norb), np.int32)
        site_of[latt.site_cell, latt.site_orb] = np.arange(latt.N * latt.norb)
        jof = np.zeros((latt.N, latt.N), np.int32)
        I = np.repeat(np.arange(latt.N), latt.N)
        J = np.tile(np.arange(latt.N), latt.N)
        jof[I, latt.imj[I, J]] = J
        self._latt = latt
        self._keep.append((site_of, jof))
        _lib.check(self.L.alfgpu_set_lattice_obs(self.h, latt.N, latt.norb, _p(site_of), _p(jof)),
                   "alfgpu_set_lattice_obs")

    def reset_lattice_obs(self):
        _lib.check(self.L.alfgpu_reset_lattice_obs(self.h), "alfgpu_reset_lattice_obs")

    def lattice_obs(self, chain: int = 0, kind: int = 0) -> dict:
        """Accumulators of one chain (kind 0: equal time, 1: time displaced): per observable
        Obs_Latt [R][nt][no][no] and Obs_Latt0 [no] (complex), with the count and sign sum."""
        from .lattice_obs import names_for
        latt = self._latt
        names = names_for(self.F)
        nt = 1 if kind == 0 else self.Lt + 1
        a = np.zeros((len(names), latt.N, nt, latt.norb, latt.norb), np.complex128)
        a0 = np.zeros((len(names), latt.norb), np.complex128)
        cs = np.zeros(2, np.float64)
        _lib.check(self.L.alfgpu_get_lattice_obs(self.h, chain, kind, _p(a), _p(a0), _p(cs)),
                   "alfgpu_get_lattice_obs")
        return {"obs": {k: a[i] for i, k in enumerate(names)}, "obs0": {k: a0[i] for i, k in enumerate(names)},
                "count": int(cs[0]), "sign": float(cs[1])}

    def lattice_bin(self, chain: int = 0, kind: int = 0, reset: bool = False) -> dict:
        """Print_bin_Latt's normalisation of one chain's accumulators, as EqualTimeObs.bin()
        (kind 0) or TimeDisplacedObs.bin() (kind 1) returns it: Obs_Latt / N,
        Obs_Latt0 / (N Ns Ntau), Ave_sign / N."""
        d = self.lattice_obs(chain, kind)
        n, ns = d["count"], self._latt.N
        if n == 0:
            raise ValueError("an empty bin")
        ntau = 1 if kind == 0 else self.Lt + 1
        out = {k: {"latt": d["obs"][k] / n, "latt0": d["obs0"][k] / (n * ns * ntau), "sign": d["sign"] / n}
               for k in d["obs"]}
        if reset:
            self.reset_lattice_obs()
        return out

    # --- checkpoint / resume (the reference's confout files) ------------------------------------
    def checkpoint(self, path: str):
        """Write every chain's fields and draw-stream state, the stabilisation interval and the
        delay depth to an .npz file."""
        keys = np.zeros(self.C, np.uint64)
        ctrs = np.zeros(self.C, np.uint64)
        for c in range(self.C):
            k, n = C.c_uint64(), C.c_uint64()
            _lib.check(self.L.alfgpu_get_rng_state(self.h, c, C.byref(k), C.byref(n)), "alfgpu_get_rng_state")
            keys[c], ctrs[c] = k.value, n.value
        np.savez(path, fields=np.stack([self.fields(c) for c in range(self.C)]), keys=keys, counters=ctrs,
                 nwrap=self.nwrap(), delay=self.delay(), ndim=self.N, ltrot=self.Lt, n_op=self.M)

    def restore(self, path: str) -> np.ndarray:
        """Resume from checkpoint(): fields, draw streams, Nwrap and delay depth; G and the UDV
        stack are rebuilt from the fields (init_state), as the reference does on restart."""
        z = np.load(path)
        if (int(z["ndim"]), int(z["ltrot"]), int(z["n_op"])) != (self.N, self.Lt, self.M) or \
                z["fields"].shape[0] != self.C:
            raise ValueError("checkpoint does not match this handle's sizes")
        for c in range(self.C):
            self.set_fields(c, z["fields"][c])
            _lib.check(self.L.alfgpu_set_rng_state(self.h, c, int(z["keys"][c]), int(z["counters"][c])),
                       "alfgpu_set_rng_state")
        if int(z["nwrap"]) != self.nwrap():
            self.set_nwrap(int(z["nwrap"]))
        self.set_delay(int(z["delay"]))
        return self.init_state()

    # --- stabilisation interval --------------------------------------------------------------
    def set_nwrap(self, nwrap: int):
        """New stabilisation interval; call init_state before the next sweep."""
        _lib.check(self.L.alfgpu_set_nwrap(self.h, nwrap), "alfgpu_set_nwrap")

    def nwrap(self) -> int:
        k = C.c_int32()
        _lib.check(self.L.alfgpu_get_nwrap(self.h, C.byref(k)), "alfgpu_get_nwrap")
        return k.value

    def adapt_nwrap(self, bound: float = 1e-5, sweeps: int = 1):
        """Shorten Nwrap while the drift is too large: run `sweeps` device-draw sweeps, and if
        any chain's Precision Green (max |G_wrapped - G_fresh|) exceeds `bound` (or the sweep
        stops with ALF's ERROR_UNSTABLE_MATRIX or a NaN in G), halve Nwrap, rebuild G and the
        UDV stack from the current fields and try again.  The sweeps advance the chains (use them as
        thermalisation).  Returns (nwrap, worst Precision Green)."""
        while True:
            self.reset_stats()
            try:
                for _ in range(sweeps):
                    self.sweep(None)
                worst = max(self.stats(c).xmaxG for c in range(self.C))
            except _lib.AlfGpuError as e:
                # ERROR_UNSTABLE_MATRIX (ALF's abort at Precision Green > 10) or a NaN in G (the
                # same instability past the point where the comparison is defined)
                if e.code not in (3, 103):
                    raise
                worst = float("inf")
            nw = self.nwrap()
            if worst <= bound or nw == 1:
                return nw, worst
            self.set_nwrap(max(1, nw // 2))
            self.init_state()

    # --- readback --------------------------------------------------------------------------------
    def green(self, chain: int = 0) -> np.ndarray:
        G = np.zeros((self.F, self.N, self.N), np.complex128)
        _lib.check(self.L.alfgpu_get_green(self.h, chain, _p(G)), "alfgpu_get_green")
        return np.transpose(G, (0, 2, 1)).copy()

    def phase(self) -> np.ndarray:
        ph = np.zeros(self.C, np.complex128)
        _lib.check(self.L.alfgpu_get_phase(self.h, _p(ph)), "alfgpu_get_phase")
        return ph

    def stats(self, chain: int = 0) -> _lib.Stats:
        s = _lib.Stats()
        _lib.check(self.L.alfgpu_get_stats(self.h, chain, C.byref(s)), "alfgpu_get_stats")
        return s

    def reset_stats(self):
        _lib.check(self.L.alfgpu_reset_stats(self.h), "alfgpu_reset_stats")

    def set_profiling(self, enable: bool = True):
        _lib.check(self.L.alfgpu_set_profiling(self.h, int(enable)), "alfgpu_set_profiling")

    def profile(self) -> dict:
        """Per-phase device time (ms) and launch-group counts since profiling was enabled."""
        n = len(_lib.PROF_PHASES)
        ms = np.zeros(n, np.float64)
        cnt = np.zeros(n, np.int64)
        _lib.check(self.L.alfgpu_get_profile(self.h, _p(ms), _p(cnt)), "alfgpu_get_profile")
        return {k: (float(ms[i]), int(cnt[i])) for i, k in enumerate(_lib.PROF_PHASES)}

    def set_recording(self, enable: bool = True):
        _lib.check(self.L.alfgpu_set_recording(self.h, int(enable)), "alfgpu_set_recording")

    def record_sizes(self) -> tuple:
        """(visits, stabilisation points) of one sweep's record at the handle's current Nwrap
        (alfgpu_set_nwrap may have changed it since the model was built): 2 M Ltrot visits and
        2 Nstm points, Nstm = ceil(Ltrot / Nwrap)."""
        nw = self.nwrap()
        return 2 * self.M * self.Lt, 2 * ((self.Lt + nw - 1) // nw)

    def record(self, chain: int = 0) -> dict:
        V, P = self.record_sizes()
        acc = np.zeros(V, np.int8)
        ratio = np.zeros(V, np.complex128)
        G = np.zeros((P, self.F, self.N, self.N), np.complex128)
        Gw = np.zeros((P, self.F, self.N, self.N), np.complex128)
        ph = np.zeros(P, np.complex128)
        _lib.check(self.L.alfgpu_get_record(self.h, chain, _p(acc), _p(ratio), _p(G), _p(Gw), _p(ph)),
                   "alfgpu_get_record")
        return dict(acc=acc, ratio=ratio, G=np.transpose(G, (0, 1, 3, 2)).copy(),
                    Gwrap=np.transpose(Gw, (0, 1, 3, 2)).copy(), phase=ph)


def cgr(nvar: int, UR, DR, VR, UL, DL, VL):
    """GPU ``CGR`` on explicit UDV factors (row-major numpy in/out)."""
    L = _lib.lib()
    N = UR.shape[0]
    cm = lambda A: np.ascontiguousarray(np.asarray(A, np.complex128).T)
    args = [cm(UR), np.ascontiguousarray(DR, np.complex128), cm(VR), cm(UL), np.ascontiguousarray(DL, np.complex128),
            cm(VL)]
    G = np.zeros((N, N), np.complex128)
    ph = np.zeros(1, np.complex128)
    _lib.check(L.alfgpu_cgr(N, nvar, *[_p(a) for a in args], _p(G), _p(ph)), "alfgpu_cgr")
    return G.T.copy(), complex(ph[0])


def decompose(side: str, U, D, V):
    """GPU ``decompose_UDV_state`` on explicit factors (row-major numpy in/out)."""
    L = _lib.lib()
    N = U.shape[0]
    Uc = np.ascontiguousarray(np.asarray(U, np.complex128).T)
    Vc = np.ascontiguousarray(np.asarray(V, np.complex128).T)
    Dc = np.ascontiguousarray(D, np.complex128).copy()
    _lib.check(L.alfgpu_decompose(N, C.c_char(side.encode()), _p(Uc), _p(Dc), _p(Vc)), "alfgpu_decompose")
    return Uc.T.copy(), Dc, Vc.T.copy()


def sweep_many(handles: Sequence["Chains"], uniforms: Optional[Sequence[Optional[np.ndarray]]] = None) -> None:
    """One sweep on each of several handles through alfgpu_sweep_many: every handle's launches
    are issued from this thread first, each on its own stream, then each handle is waited for,
    so handles of different sizes sweep concurrently without host threads.  uniforms: None (the
    device streams) or one host array (or None) per handle, as for Chains.sweep."""
    n = len(handles)
    if n == 0:
        return
    L = handles[0].L
    hs = (C.c_void_p * n)(*[h.h for h in handles])
    status = np.zeros(n, np.int32)
    keep = []
    if uniforms is None:
        up = None
    else:
        ptrs = []
        for h, u in zip(handles, uniforms):
            if u is None:
                ptrs.append(None)
                continue
            a = np.ascontiguousarray(u, dtype=np.float64)
            if a.size != h.C * 6 * h.M * h.Lt:
                raise ValueError(f"{a.size} draws, expected {h.C * 6 * h.M * h.Lt} (chains x 6 M Ltrot)")
            keep.append(a)
            ptrs.append(a.ctypes.data_as(C.c_void_p))
        up = (C.c_void_p * n)(*ptrs)
    rc = L.alfgpu_sweep_many(hs, n, up, status.ctypes.data_as(C.c_void_p))
    for k in range(n):
        if status[k]:
            h = handles[k]
            _lib.check(int(status[k]), f"alfgpu_sweep_many (handle {k})" +
                       (f" ({h.L.alfgpu_last_error(h.h).decode()})" if status[k] == 100 else ""))
    _lib.check(rc, "alfgpu_sweep_many")
