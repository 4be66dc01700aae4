"""ALF's site numbering (Make_lattice, Libraries/Modules/lattices_v3_mod.F90:88-336) as an
option of the model setup: the centred cell walked i1-outer / i2-inner, one representative
per periodic class; Invlist numbers orbitals fastest within a cell."""
import numpy as np
import pytest

from alf_gb300 import model as mdl


def test_square_4x4_order_follows_the_centred_walk():
    # i1, i2 in {-1, 0, 1, 2} (the other points fall outside |x.a| <= |a|^2/2), i1 outer;
    # (i1, i2) is the natural cell (i1 mod 4) + 4 (i2 mod 4)
    expect = [(i1 % 4) + 4 * (i2 % 4) for i1 in (-1, 0, 1, 2) for i2 in (-1, 0, 1, 2)]
    assert mdl.alf_cell_order("square", 4, 4) == expect
    assert mdl.alf_cell_order("n_leg_ladder", 4, 1) == [3, 0, 1, 2]


@pytest.mark.parametrize("lat,L1,L2", [("square", 16, 16), ("square", 6, 4), ("honeycomb", 12, 12),
                                       ("honeycomb", 3, 3), ("bilayer_square", 12, 12), ("n_leg_ladder", 4, 3)])
def test_alf_order_relabels_the_same_lattice(lat, L1, L2):
    a = mdl.hopping_matrix(lat, L1, L2)
    b = mdl.hopping_matrix(lat, L1, L2, site_order="alf")
    norb = a.shape[0] // len(mdl.alf_cell_order(lat, L1, L2))
    p = np.array([I * norb + o for I in mdl.alf_cell_order(lat, L1, L2) for o in range(norb)])
    assert sorted(p) == list(range(a.shape[0]))
    np.testing.assert_array_equal(b, a[np.ix_(p, p)])


def test_models_take_the_order_and_keep_the_vertex_layout():
    m = mdl.hubbard("square", 4, 4, site_order="alf")
    assert [v.P for v in m.vertices[0]] == [[i] for i in range(16)]  # one vertex per site, Invlist order
    assert m.params["site_order"] == "alf"
    k = mdl.kondo(2, 2, Uf=0.0, site_order="alf")
    assert [v.P for v in k.vertices[0]] == [[2 * i, 2 * i + 1] for i in range(4)]
    with pytest.raises(ValueError):
        mdl.hopping_matrix("square", 4, 4, site_order="rows")
