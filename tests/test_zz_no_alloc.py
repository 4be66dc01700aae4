"""The no-allocation decompose entry point (alfgpu_decompose_noalloc).

Callers whose device memory belongs to another allocator, or that must not
trigger the device synchronisation of cudaMalloc/cudaFree, pass their own
device buffers; the entry point keeps its scratch in a static device array.
This test drives it through the C ABI on buffers the test allocates with
torch, twice in a row with different sizes and sides, and checks each result
against the allocating entry point alfgpu_decompose on the same inputs, within
the 1e-10 relative tolerance of the other decompose tests.  It also checks that
sizes above the static maximum are rejected without touching the buffers.
"""
import ctypes

import numpy as np
import pytest

from alf_gb300 import _lib
from alf_gb300.sweep import decompose as gpu_decompose

pytestmark = pytest.mark.gpu

RTOL = 1e-10


def _relmax(a, b):
    return np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300)


def _inputs(N, seed):
    rs = np.random.default_rng(seed)
    X = rs.standard_normal((N, N)) + 1j * rs.standard_normal((N, N))
    Y = rs.standard_normal((N, N)) + 1j * rs.standard_normal((N, N))
    U = X @ np.linalg.qr(Y)[0]
    D = np.exp(np.linspace(3.0, -3.0, N))
    V = np.eye(N, dtype=complex) + 0.1 * (rs.standard_normal((N, N)) + 1j * rs.standard_normal((N, N)))
    return U, D, V


def _noalloc(N, side, U, D, V):
    torch = pytest.importorskip("torch")
    dev = torch.device("cuda:0")
    tU = torch.from_numpy(np.ascontiguousarray(U.T)).to(dev)  # column-major complex128
    tV = torch.from_numpy(np.ascontiguousarray(V.T)).to(dev)
    tD = torch.from_numpy(np.ascontiguousarray(D, dtype=np.float64)).to(dev)
    tdet = torch.zeros(1, dtype=torch.complex128, device=dev)
    stream = torch.cuda.current_stream(dev)
    rc = _lib.lib().alfgpu_decompose_noalloc(N, ctypes.c_char(side.encode()), ctypes.c_void_p(tU.data_ptr()),
                                              ctypes.c_void_p(tD.data_ptr()), ctypes.c_void_p(tV.data_ptr()),
                                              ctypes.c_void_p(tdet.data_ptr()), ctypes.c_void_p(stream.cuda_stream))
    torch.cuda.synchronize(dev)
    return rc, tU.cpu().numpy().T, tD.cpu().numpy(), tV.cpu().numpy().T, complex(tdet.cpu().numpy()[0])


def test_noalloc_decompose_matches_allocating_entry_point_twice():
    for N, side, seed in ((64, "r", 11), (256, "l", 12)):
        U, D, V = _inputs(N, seed)
        rc, Un, Dn, Vn, det = _noalloc(N, side, U, D, V)
        assert rc == 0, _lib.ERRORS.get(rc, rc)
        Ua, Da, Va = gpu_decompose(side, U, D.astype(complex), V)
        assert _relmax(Un, Ua) < RTOL
        assert _relmax(Dn, Da.real) < RTOL
        assert _relmax(Vn, Va) < RTOL
        assert abs(det - np.linalg.det(Un)) < 1e-10
        # U D V (side r) or U D V^H (side l) reproduces the input product
        P = U @ np.diag(D) @ (V if side == "r" else V.conj().T)
        R = Un @ np.diag(Dn) @ (Vn if side == "r" else Vn.conj().T)
        assert _relmax(R, P) < RTOL


def test_noalloc_rejects_sizes_above_the_static_maximum():
    torch = pytest.importorskip("torch")
    N = 257
    buf = torch.full((N * N * 2,), 7.0, dtype=torch.float64, device="cuda:0")
    rc = _lib.lib().alfgpu_decompose_noalloc(N, ctypes.c_char(b"r"), ctypes.c_void_p(buf.data_ptr()),
                                              ctypes.c_void_p(buf.data_ptr()), ctypes.c_void_p(buf.data_ptr()),
                                              None, None)
    assert rc == 105
    assert _lib.lib().alfgpu_error_string(105).startswith(b"Ndim exceeds")
    assert bool(torch.all(buf == 7.0))
