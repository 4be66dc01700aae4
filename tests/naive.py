"""Naive dense formulas used to pin the oracle (small sizes only).

B(tau) for one slice is ``prod_n exp(g phi O_n) . exp(-dtau T)`` applied from
the left in the order of ``WRAPUR`` (Prog/wrapur_mod.F90:114-119), and the
equal-time Green function is ``(1 + B(tau,0) B(beta,tau))^-1``
(Prog/cgr1_mod.F90 header).
"""
import numpy as np

from alf_gb300 import model as mdl


def vertex_matrix(v, s, N):
    X = np.eye(N, dtype=complex)
    E = v.M_exp[s + 2]
    for a in range(v.n):
        for b in range(v.n):
            X[v.P[a], v.P[b]] = E[a, b]
    return X


def slice_B(m, f, nt1, nf):
    """B(nt1) (1-based slice index) for flavour nf."""
    N = m.ndim
    B = m.expT[nf].astype(complex)
    for n in range(m.n_op):
        B = vertex_matrix(m.vertices[nf][n], int(f[nt1 - 1, n]), N) @ B
    return B


def B_range(m, f, t2, t1, nf):
    """B(t2, t1) = B_{t2} ... B_{t1+1}."""
    N = m.ndim
    X = np.eye(N, dtype=complex)
    for t in range(t1 + 1, t2 + 1):
        X = slice_B(m, f, t, nf) @ X
    return X


def green(m, f, tau, nf):
    N = m.ndim
    A = B_range(m, f, tau, 0, nf) @ B_range(m, f, m.ltrot, tau, nf)
    return np.linalg.inv(np.eye(N) + A)


def weight_det(m, f, nf):
    N = m.ndim
    return np.linalg.det(np.eye(N) + B_range(m, f, m.ltrot, 0, nf))


def boson_factor(m, f):
    """prod exp(g alpha phi) over flavours (complex), and prod gamma."""
    z = 1.0 + 0j
    gam = 1.0
    for nf in range(m.n_fl):
        for n in range(m.n_op):
            v = m.vertices[nf][n]
            for nt in range(m.ltrot):
                z *= np.exp(v.g * v.alpha * mdl.phi(int(f[nt, n]), v.op_type))
    for n in range(m.n_op):
        v = m.vertices[0][n]
        for nt in range(m.ltrot):
            gam *= mdl.GAMA_TYPE2[int(f[nt, n])] if v.op_type == 2 else 1.0
    return z, gam


def full_weight(m, f):
    d = 1.0 + 0j
    z, gam = boson_factor(m, f)
    for nf in range(m.n_fl):
        d *= weight_det(m, f, nf)
    return (d * z) ** m.n_sun * gam


def nranf3(r):
    y = r * 3.0 + 0.5
    v = int(np.floor(y + 0.5)) if y >= 0 else int(np.ceil(y - 0.5))
    return min(max(v, 1), 3)


def visit_order(m):
    """(nt1, n) for every visit of one sweep, in draw order."""
    out = []
    for nt in range(1, m.ltrot + 1):
        for n in range(m.n_op):
            out.append((nt, n))
    for nt in range(m.ltrot, 0, -1):
        for n in range(m.n_op - 1, -1, -1):
            out.append((nt, n))
    return out
