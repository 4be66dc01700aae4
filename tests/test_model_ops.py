"""The vertex tables both the GPU library and the oracle consume (Op_set / Op_exp of
Prog/Operator_mod.F90:259-529), checked on the operators of the reference's own unit tests
against the dense matrix exponential: testsuite/Prog.tests/21-Op-make.F90 (Op_exp of
O(i,n) = (n+i, i-n), g = 2) and 10-Op-mmultL.F90 / 11-Op-mmultR.F90 (O(i,n) = (n+i, n-i),
g = 0.02, discrete fields of type 1 and 2; the continuous types 3 and 4 are outside the
sweep this package implements)."""
import numpy as np
import pytest
import scipy.linalg as sl

from alf_gb300 import model as mdl


def _op(opn, f):
    return np.array([[f(i, n) for n in range(1, opn + 1)] for i in range(1, opn + 1)], dtype=complex)


@pytest.mark.parametrize("opn", range(1, 9))  # larger O overflow exp (as the reference test notes)
def test_op_exp_matches_the_dense_exponential(opn):
    O = _op(opn, lambda i, n: complex(n + i, i - n))
    v = mdl.op_set(mdl.Vertex(P=list(range(opn)), O=O, g=2.0, alpha=0.0, op_type=2))
    ref = sl.expm(2.0 * O)
    got = mdl.op_exp(2.0, v)
    assert np.max(np.abs(got - ref)) <= 1e-12 * np.max(np.abs(ref))
    # Op_set's normalisation: U unitary with det 1, non-zero eigenvalues first
    np.testing.assert_allclose(v.U.conj().T @ v.U, np.eye(opn), atol=1e-13)
    if not v.diag:
        assert abs(np.linalg.det(v.U) - 1.0) < 1e-12
    nz = v.n_non_zero
    assert np.all(np.abs(v.E[:nz]) > mdl.EPS_SMALL) and np.all(np.abs(v.E[nz:]) <= mdl.EPS_SMALL)


@pytest.mark.parametrize("op_type", [1, 2])
@pytest.mark.parametrize("opn", [1, 2, 3, 4])
def test_exponential_tables_of_every_field_value(opn, op_type):
    O = _op(opn, lambda i, n: complex(n + i, n - i))
    g = 0.02
    v = mdl.op_set(mdl.Vertex(P=list(range(opn)), O=O, g=g, alpha=0.0, op_type=op_type))
    values = (-1, 1) if op_type == 1 else (-2, -1, 1, 2)
    for s in values:
        ref = sl.expm(g * mdl.phi(s, op_type) * O)
        np.testing.assert_allclose(v.M_exp[s + 2], ref, rtol=0, atol=1e-13 * np.max(np.abs(ref)))
        # the eigenvalue table the per-visit ratio uses: exp(g E phi) on the non-zero eigenvalues
        nz = v.n_non_zero
        np.testing.assert_allclose(v.E_exp[:nz, s + 2], np.exp(g * v.E[:nz] * mdl.phi(s, op_type)), rtol=1e-14)
        if nz == opn:
            np.testing.assert_allclose((v.U * v.E_exp[:, s + 2]) @ v.U.conj().T, ref, rtol=0,
                                       atol=1e-13 * np.max(np.abs(ref)))
    # the field tables: phi and gamma of type 2 are the four-point Gauss-Hermite rule
    if op_type == 2:
        w = np.array([mdl.GAMA_TYPE2[s] for s in values])
        x = np.array([mdl.PHI_TYPE2[s] for s in values])
        # sum_s gamma(s) exp(a phi(s)) / sum gamma = exp(a^2) up to O(a^8): the HS identity
        for a in (0.05, 0.1, 0.2):
            assert abs(np.sum(w * np.exp(a * x)) / np.sum(w) - np.exp(a * a)) < 5.0 * a ** 8
