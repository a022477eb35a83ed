"""Host-pointer paths of mac_macproject: fabs in page-locked host memory are read and written in
place by the gather/scatter kernels; pageable fabs go through device staging copies.  Both must
give bitwise the same fabs (valid entries, ghost entries the projection fills and ghost entries
outside non-periodic walls that it leaves alone), for one box or several and with a mix of the
two kinds of memory.
"""
import numpy as np
import pytest

from maestro_gb300.inputs import BC_DIR, BC_NEU, BC_PER, make_case
from maestro_gb300.macproject import BcTower, Layout, MacProjector

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def _pinned_like(a):
    t = torch.empty(a.size, dtype=torch.float64, pin_memory=True)
    v = t.numpy().reshape(a.shape, order="F")
    v[...] = a
    return t, v


def _fab_sets(c, lay, pinned_boxes):
    per = [c.bc_lo[d] == BC_PER for d in range(c.dm)]
    keep = []

    def conv(lst):
        out = []
        for b, f in enumerate(lst):
            if b in pinned_boxes:
                t, v = _pinned_like(f)
                keep.append(t)
                out.append(v)
            else:
                out.append(np.asfortranarray(f.copy()))
        return out

    fu = [conv(lay.to_fabs(c.umac[d], ng=1, face_dir=d, periodic=per)) for d in range(c.dm)]
    frho = conv(lay.to_fabs(c.rho, ng=1, periodic=per))
    fphi = conv(lay.to_fabs(c.phi0, ng=1, periodic=per))
    for f in fphi:
        # shift ghost and valid entries alike: ghosts outside the non-periodic z walls must keep
        # the shifted value, valid ones are overwritten by the solution
        f[...] += 7.0
    frhs = conv(lay.to_fabs(c.macrhs, ng=0))
    return keep, fu, frho, fphi, frhs


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("mix", ["pageable", "pinned", "mixed"])
def test_pinned_and_pageable_fabs_agree(cuda_lib, precision, mix):
    c = make_case(name="hostpaths", dm=3, n=(32, 32, 32), box=(16, 16, 16), H_frac=0.25,
                  noise=0.01, kmax=4, seed=21)
    c.bc_lo, c.bc_hi = (BC_PER, BC_PER, BC_NEU), (BC_PER, BC_PER, BC_DIR)
    lay = Layout.tiled(c.n, c.box)
    nb = len(lay.boxes)
    pinned = {"pageable": set(), "pinned": set(range(nb)), "mixed": set(range(0, nb, 2))}[mix]
    ref = _fab_sets(c, lay, set())
    run = _fab_sets(c, lay, pinned)
    outs = []
    for keep, fu, frho, fphi, frhs in (ref, run):
        P = MacProjector(lay, c.dx, BcTower(c.bc_lo, c.bc_hi), precision=precision)
        try:
            st = P.macproject(fu, fphi, frho, frhs, c.beta0, c.beta0_edge, strict=True)
        finally:
            P.close()
        assert st["status"] == 0 and st["rel_resid"] <= 1e-10
        outs.append((fu, fphi, frho))
    (fu0, fphi0, frho0), (fu1, fphi1, frho1) = outs
    for d in range(c.dm):
        for a, b in zip(fu0[d], fu1[d]):
            np.testing.assert_array_equal(a, b)
    for a, b in zip(fphi0, fphi1):
        np.testing.assert_array_equal(a, b)
    for a, b in zip(frho0, frho1):
        np.testing.assert_array_equal(a, b)
