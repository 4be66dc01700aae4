"""alfgpu_sweep_many: several handles (different N_dim and Ltrot) swept from one host thread,
their launches issued first on their own streams, then waited for.  The result of every handle
must be bit for bit the result of sweeping it alone with alfgpu_sweep on the same draws (the
same launches on the same stream), for device and host draws; a wrong draw count is rejected
before anything is launched."""
import numpy as np
import pytest

from alf_gb300 import model as mdl, rng
from alf_gb300.sweep import Chains, sweep_many

pytestmark = pytest.mark.gpu


def _handles(precision):
    ms = [mdl.hubbard("square", 6, 6, U=4.0, beta=2.0, dtau=0.1, nwrap=10),
          mdl.hubbard("square", 8, 8, U=3.0, beta=1.0, dtau=0.1, nwrap=5)]
    out = []
    for k, m in enumerate(ms):
        C = 2
        g = Chains(m, n_chains=C, precision=precision)
        for c in range(C):
            g.set_fields(c, rng.initial_fields(50 + 10 * k + c, c, m.n_op, m.ltrot))
            g.set_rng(c, 50 + 10 * k + c, rng.sweep_counter_base(m.n_op, m.ltrot, 0))
        g.init_state()
        out.append(g)
    return out


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_sweep_many_equals_single_sweeps(precision):
    a, b = _handles(precision), _handles(precision)
    for s in range(2):  # device draws (graph replay after the first sweep)
        sweep_many(a)
        for g in b:
            g.sweep(None)
    us = [np.stack([rng.sweep_uniforms(70 + c, c, g.model.n_op, g.model.ltrot, 9) for c in range(g.C)]) for g in a]
    sweep_many(a, us)  # host draws
    for g, u in zip(b, us):
        g.sweep(u)
    for ga, gb in zip(a, b):
        for c in range(ga.C):
            np.testing.assert_array_equal(ga.fields(c), gb.fields(c))
            assert np.array_equal(ga.green(c), gb.green(c))
            assert ga.stats(c).n_acc == gb.stats(c).n_acc
    for g in a + b:
        g.close()


def test_sweep_many_rejects_a_wrong_draw_count():
    a = _handles("fp64")
    with pytest.raises(Exception):
        sweep_many(a, [np.zeros(5), None])  # wrong draw count for handle 0: rejected on the host
    for g in a:
        g.close()
