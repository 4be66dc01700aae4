"""Several handles of different sizes in one process: per-kernel launch settings are process
wide, so a handle created later (here with a smaller exact-QR row block) must not break the
launches of an earlier one."""
import numpy as np
import pytest

from alf_gb300 import model as mdl, rng
from alf_gb300.sweep import Chains

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_handles_of_different_sizes(precision):
    ms = [mdl.hubbard("square", 14, 14, U=4.0, beta=1.0, dtau=0.1, nwrap=10),
          mdl.hubbard("square", 16, 16, U=4.0, beta=1.0, dtau=0.1, nwrap=10),
          mdl.hubbard("square", 6, 6, U=4.0, beta=1.0, dtau=0.1, nwrap=10)]
    hs = []
    for m in ms:
        ch = Chains(m, n_chains=2, precision=precision)
        for c in range(2):
            ch.set_fields(c, rng.initial_fields(3 + c, c, m.n_op, m.ltrot))
        hs.append((ch, m))
    for ch, m in hs:  # the first handle runs after the later ones were created
        ch.init_state()
        ch.sweep(None)
        G = ch.green(0)
        assert np.all(np.isfinite(G))
        assert ch.stats(0).xmaxG < 1e-5
        ch.close()
