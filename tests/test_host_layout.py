"""Host-side logic of the Python mirror (no GPU): the per-box fab split of whole-domain arrays
(valid region, ghosts by periodic wrap or clamping, face arrays with their extra entry), the
physical-to-elliptic boundary mapping, and the synthetic case generators' shapes."""
import numpy as np
import pytest

from maestro_gb300.inputs import (BC_DIR, BC_NEU, BC_PER, config_case, make_case,
                                  make_spherical_case)
from maestro_gb300.macproject import BcTower, Layout


@pytest.mark.parametrize("n,box", [((16, 8), (8, 4)), ((8, 8, 8), (4, 4, 8)), ((12, 6, 4), (4, 3, 2))])
@pytest.mark.parametrize("ng", [0, 1, 2])
@pytest.mark.parametrize("face_dir", [None, 0, 1])
def test_fab_split_round_trip(n, box, ng, face_dir):
    lay = Layout.tiled(n, box)
    shape = list(n)
    if face_dir is not None:
        shape[face_dir] += 1
    a = np.asfortranarray(np.random.default_rng(1).standard_normal(shape))
    fabs = lay.to_fabs(a, ng=ng, face_dir=face_dir, periodic=[True] * len(n))
    assert len(fabs) == int(np.prod([n[d] // box[d] for d in range(len(n))]))
    for (lo, hi), f in zip(lay.boxes, fabs):
        assert f.flags.f_contiguous and f.dtype == np.float64
        for d in range(len(n)):
            assert f.shape[d] == hi[d] - lo[d] + 1 + 2 * ng + (1 if face_dir == d else 0)
    np.testing.assert_array_equal(lay.from_fabs(fabs, ng=ng, face_dir=face_dir), a)


def test_fab_ghosts_wrap_or_clamp():
    n = (8, 8)
    lay = Layout.tiled(n, (4, 8))
    a = np.asfortranarray(np.arange(64, dtype=np.float64).reshape(n, order="F"))
    per = lay.to_fabs(a, ng=1, periodic=[True, True])
    cl = lay.to_fabs(a, ng=1, periodic=[False, False])
    # box 0 covers i = 0..3: its low ghost column is i = 7 (periodic) or i = 0 (clamped)
    np.testing.assert_array_equal(per[0][0, 1:-1], a[7, :])
    np.testing.assert_array_equal(cl[0][0, 1:-1], a[0, :])
    # the high ghost row j = 8 wraps to j = 0, or clamps to j = 7
    np.testing.assert_array_equal(per[0][1:-1, -1], a[0:4, 0])
    np.testing.assert_array_equal(cl[0][1:-1, -1], a[0:4, 7])


def test_physical_boundaries_map_to_elliptic_ones():
    bc = BcTower.from_phys(["periodic", "slip wall", "outlet"], ["periodic", "inlet", "no slip wall"])
    assert bc.lo == (BC_PER, BC_NEU, BC_DIR) and bc.hi == (BC_PER, BC_NEU, BC_NEU)
    assert BcTower.from_phys(["symmetry"], ["outlet"]).lo == (BC_NEU,)


def test_case_generators():
    c = config_case("3d_256", seed=1, scale=8)
    assert c.n == (32, 32, 32) and c.box == (16, 16, 16)
    assert all(u.shape[d] == c.n[d] + 1 for d, u in enumerate(c.umac))
    assert c.beta0.shape == (32,) and c.beta0_edge.shape == (33,)
    # macrhs is compatible with the singular periodic/Neumann problem: zero mean per layer
    assert np.abs(c.macrhs.mean(axis=(0, 1))).max() <= 1e-12 * np.abs(c.macrhs).max()
    s = make_spherical_case(n=(16, 16, 16), box=(8, 8, 8))
    assert s.bc_lo == (BC_DIR,) * 3 and s.beta0 is None
    for d in range(3):
        assert s.b0c[d].shape[d] == 17 and (s.b0c[d] > 0).all()
    # beta0 falls off from the centre: a corner face carries less than a central one
    assert s.b0c[0][8, 8, 8] > s.b0c[0][0, 0, 0]
    p = make_spherical_case(n=(16, 16, 16), box=(8, 8, 8), bc="periodic")
    assert p.bc_lo == (BC_PER,) * 3 and p.bc_hi == (BC_PER,) * 3
    m = make_case(dm=2, n=(16, 8), kmax=2)
    assert m.umac[0].shape == (17, 8) and m.umac[1].shape == (16, 9)
