"""Host-side policies of the Python mirror (alf_gb300.sweep.Chains, sweep_many) on the CPU, driven by a
stand-in for the C library: the drift-control loop (adapt_nwrap), the sizing of the record
buffers from the handle's current Nwrap, checkpoint / restore, the layouts of the observable
callback and the scalar accumulators.  The library calls are the ones include/alfgpu.h
declares; the stand-in keeps their state in Python."""
import ctypes as C

import numpy as np
import pytest

from alf_gb300 import _lib, model as mdl, sweep


class FakeLib:
    """The entry points Chains uses, with the handle's state held in Python.  drift(nwrap)
    gives each sweep's Precision Green; unstable(nwrap) makes the sweep stop with ALF's
    ERROR_UNSTABLE_MATRIX (3)."""

    def __init__(self, drift=lambda nw: 1e-7, unstable=lambda nw: False, sweep_rc=0, unstable_rc=3):
        self.drift, self.unstable, self.sweep_rc, self.unstable_rc = drift, unstable, sweep_rc, unstable_rc
        self.log = []

    def alfgpu_create(self, hp, dp):
        d = dp._obj
        self.nw, self.Lt, self.M, self.C, self.delay = d.nwrap, d.ltrot, d.n_op, d.n_chains, 32
        self.fields = np.ones((self.C, self.Lt, self.M), np.int8)
        self.rng = [(0, 0)] * self.C
        hp._obj.value = 0x1000
        return 0

    def alfgpu_upload_hopping(self, h, a, b):
        return 0

    def alfgpu_upload_vertices(self, h, c, v):
        return 0

    def alfgpu_destroy(self, h):
        self.log.append("destroy")

    def alfgpu_set_fields(self, h, c, p):
        buf = np.zeros((self.Lt, self.M), np.int8)
        C.memmove(buf.ctypes.data, p.value, buf.nbytes)
        self.fields[c] = buf
        return 0

    def alfgpu_get_fields(self, h, c, p):
        C.memmove(p.value, np.ascontiguousarray(self.fields[c]).ctypes.data, self.fields[c].nbytes)
        return 0

    def alfgpu_get_rng_state(self, h, c, kp, np_):
        kp._obj.value, np_._obj.value = self.rng[c]
        return 0

    def alfgpu_set_rng_state(self, h, c, k, n):
        self.rng[c] = (k, n)
        return 0

    def alfgpu_get_nwrap(self, h, kp):
        kp._obj.value = self.nw
        return 0

    def alfgpu_set_nwrap(self, h, nw):
        self.nw = nw
        self.log.append(("set_nwrap", nw))
        return 0

    def alfgpu_get_delay(self, h, kp):
        kp._obj.value = self.delay
        return 0

    def alfgpu_set_delay(self, h, k):
        self.delay = k
        return 0

    def alfgpu_init_state(self, h, p):
        self.log.append(("init", self.nw))
        return 0

    def alfgpu_reset_stats(self, h):
        return 0

    def alfgpu_sweep(self, h, u, cb, ctx):
        self.log.append(("sweep", self.nw))
        if self.sweep_rc:
            return self.sweep_rc
        return self.unstable_rc if self.unstable(self.nw) else 0

    def alfgpu_last_error(self, h):
        return b"cudaLaunchKernelEx at alfgpu.cu:1"

    def alfgpu_get_stats(self, h, c, sp):
        sp._obj.xmaxG = self.drift(self.nw)
        return 0


@pytest.fixture
def fake(monkeypatch):
    holder = {}

    def use(**kw):
        f = FakeLib(**kw)
        monkeypatch.setattr(_lib, "lib", lambda *a, **k: f)
        holder["f"] = f
        return f
    return use


def _chains(n_chains=2, nwrap=10):
    m = mdl.hubbard("square", 2, 2, beta=2.0, dtau=0.1, nwrap=nwrap)
    return sweep.Chains(m, n_chains=n_chains)


def test_adapt_nwrap_halves_until_the_drift_bound_holds(fake):
    f = fake(drift=lambda nw: 1e-7 * nw ** 3, unstable=lambda nw: nw >= 10)
    ch = _chains()
    nw, worst = ch.adapt_nwrap(bound=2e-5)
    # 10: unstable -> 5: 1.25e-5 <= 2e-5
    assert nw == 5 and abs(worst - 1.25e-5) < 1e-12
    assert [e for e in f.log if e[0] in ("set_nwrap", "init")] == [("set_nwrap", 5), ("init", 5)]
    f.log.clear()
    nw, worst = ch.adapt_nwrap(bound=1e-7)  # 5 -> 2 -> 1 (Nwrap 1 ends the search)
    assert nw == 1 and [e for e in f.log if e[0] == "set_nwrap"] == [("set_nwrap", 2), ("set_nwrap", 1)]
    ch.close()


def test_adapt_nwrap_treats_a_nan_in_g_as_instability(fake):
    # ERROR_NAN (103) is the same instability past the point where Precision Green is defined
    f = fake(drift=lambda nw: 1e-7 * nw ** 3, unstable=lambda nw: nw >= 10, unstable_rc=103)
    ch = _chains()
    nw, worst = ch.adapt_nwrap(bound=2e-5)
    assert nw == 5 and abs(worst - 1.25e-5) < 1e-12
    ch.close()


def test_adapt_nwrap_passes_other_errors_through(fake):
    fake(sweep_rc=100)
    ch = _chains()
    with pytest.raises(_lib.AlfGpuError) as e:
        ch.adapt_nwrap()
    assert e.value.code == 100 and "cudaLaunchKernelEx" in str(e.value)
    ch.close()


def test_record_buffers_follow_the_handle_nwrap(fake):
    fake()
    ch = _chains(nwrap=10)
    m = ch.model
    assert ch.record_sizes() == (2 * m.n_op * m.ltrot, 2 * 2)  # Ltrot 20, Nwrap 10
    ch.set_nwrap(3)
    assert ch.record_sizes() == (2 * m.n_op * m.ltrot, 2 * 7)  # ceil(20 / 3) = 7 stabilisation points
    ch.close()


def test_checkpoint_restore_round_trip_and_size_check(fake, tmp_path):
    f = fake()
    ch = _chains(n_chains=2)
    r = np.random.default_rng(0)
    for c in range(2):
        ch.set_fields(c, r.choice(np.array([-2, -1, 1, 2], np.int8), size=(ch.Lt, ch.M)))
    f.rng = [(11, 500), (12, 700)]
    ch.set_nwrap(5)
    ch.set_delay(16)
    p = str(tmp_path / "conf.npz")
    ch.checkpoint(p)
    saved = f.fields.copy()
    ch.close()
    g = fake()
    ch2 = _chains(n_chains=2)
    ch2.restore(p)
    np.testing.assert_array_equal(g.fields, saved)
    assert g.rng == [(11, 500), (12, 700)] and g.nw == 5 and g.delay == 16
    assert g.log[-1] == ("init", 5)  # G and the UDV stack rebuilt from the fields
    ch2.close()
    fake()
    ch3 = _chains(n_chains=3)
    with pytest.raises(ValueError):
        ch3.restore(p)
    ch3.close()


class FakeObsLib(FakeLib):
    """Adds the observable callback (ham%Obser G and ham%ObserT quartets in the library's
    column-major layout) and the scalar accumulators."""

    def __init__(self, G, quartet, sums):
        super().__init__()
        self.G, self.quartet, self.sums = G, quartet, sums

    def alfgpu_sweep(self, h, u, cb, ctx):
        def colmajor(mats):  # [k][nf][row][col] -> column-major per matrix, interleaved re/im
            a = np.ascontiguousarray(np.transpose(np.asarray(mats, np.complex128), (0, 1, 3, 2)))
            return a.view(np.float64)
        ph = np.array([0.8, -0.6])
        g = colmajor(self.G[None])
        cb(None, 1, 7, 0, g.ctypes.data_as(C.POINTER(C.c_double)), ph.ctypes.data_as(C.POINTER(C.c_double)))
        q = colmajor(self.quartet)
        cb(None, 0, 3, 1, q.ctypes.data_as(C.POINTER(C.c_double)), ph.ctypes.data_as(C.POINTER(C.c_double)))
        return 0

    def alfgpu_set_scalar_obs(self, h, Hp, Up):
        n = self.N
        self.H = np.zeros((self.F, n, n))
        C.memmove(self.H.ctypes.data, Hp.value, self.H.nbytes)
        self.U = np.zeros(n)
        C.memmove(self.U.ctypes.data, Up.value, self.U.nbytes)
        return 0

    def alfgpu_get_scalar_obs(self, h, c, p):
        C.memmove(p.value, np.ascontiguousarray(self.sums[c], np.float64).ctypes.data, 80)
        return 0

    def alfgpu_reset_scalar_obs(self, h):
        self.log.append("reset_obs")
        return 0


def test_callback_matrices_arrive_row_major_and_scalar_layouts(monkeypatch):
    m = mdl.hubbard("square", 2, 2, beta=2.0, dtau=0.1, nwrap=10)
    N, F = m.ndim, m.n_fl
    r = np.random.default_rng(3)
    G = r.standard_normal((F, N, N)) + 1j * r.standard_normal((F, N, N))
    quartet = r.standard_normal((4, F, N, N)) + 1j * r.standard_normal((4, F, N, N))
    sums = [np.array([4, 0, 2, 0, 8, 0, 6, 0, 2, 2], float), np.array([0, 0, 6, 0, 4, 0, 6, 0, -1, 1], float)]
    f = FakeObsLib(G, quartet, sums)
    f.N, f.F = N, F
    monkeypatch.setattr(_lib, "lib", lambda *a, **k: f)
    ch = sweep.Chains(m, n_chains=2)
    eq, tau = ch.sweep(None, measure=True)
    (c, nt, Gr, ph), = eq
    assert (c, nt, ph) == (1, 7, complex(0.8, -0.6))
    np.testing.assert_array_equal(Gr, G)  # [nf][row][col], the matrix itself
    (c, nt, q, _), = tau
    assert (c, nt) == (0, 3) and len(q) == 4
    for a, b in zip(q, quartet):
        np.testing.assert_array_equal(a, b)
    H = r.standard_normal((F, N, N))
    ch.set_scalar_obs(H, np.arange(N, dtype=float))
    np.testing.assert_array_equal(f.H, np.transpose(H, (0, 2, 1)))  # column-major per flavour
    np.testing.assert_array_equal(f.U, np.arange(N))
    ov, sign = ch.scalar_bin()
    # per chain sums / count, then the mean over the two chains
    # chain 0: (4, 2, 8, 6) / 2 = (2, 1, 4, 3), sign 1; chain 1: (0, 6, 4, 6) / 1, sign -1
    np.testing.assert_allclose(ov, [1.0, 3.5, 4.0, 4.5])
    assert sign == (1.0 + (-1.0)) / 2 and f.log[-1] == "reset_obs"
    ch.close()


def test_sweep_many_passes_handles_draws_and_per_handle_status(fake):
    # alfgpu_sweep_many gets the handles, the count, one draw pointer per handle (NULL: device
    # stream) and a status array; a non-zero status of one handle is raised for that handle
    f = fake()
    seen = {}

    def sweep_many(hs, n, up, st):
        hv = C.cast(hs, C.POINTER(C.c_void_p))
        seen["handles"] = [hv[k] for k in range(n)]
        seen["draws"] = None if up is None else [C.cast(up, C.POINTER(C.c_void_p))[k] for k in range(n)]
        status = C.cast(st, C.POINTER(C.c_int32))
        for k in range(n):
            status[k] = f.many_status[k]
        return next((s for s in f.many_status if s), 0)

    f.alfgpu_sweep_many = sweep_many
    a, b = _chains(), _chains()
    f.many_status = [0, 0]
    sweep.sweep_many([a, b])
    assert seen["handles"] == [a.h.value, b.h.value] and seen["draws"] is None
    u = np.zeros((a.C, 6 * a.M * a.Lt))
    sweep.sweep_many([a, b], [u, None])
    assert seen["draws"][0] == u.ctypes.data and seen["draws"][1] is None
    with pytest.raises(ValueError):
        sweep.sweep_many([a, b], [np.zeros(3), None])
    f.many_status = [0, 3]
    with pytest.raises(_lib.AlfGpuError) as e:
        sweep.sweep_many([a, b])
    assert e.value.code == 3 and "handle 1" in str(e.value)
