"""Producers of the projection's inputs: make_macrhs and make_at_halftime (planar).

CPU: the oracle's restatement against values written out by hand from
Source/make_macrhs.f90:184-240.  GPU: the device kernels (per-box host fabs and the dense device
form) against the oracle, predictor and corrector calls, with and without the dpdt term and with
a base cutoff inside the domain.
"""
import numpy as np
import pytest

import oracle as O
from maestro_gb300.inputs import BC_NEU, BC_PER
from maestro_gb300.macproject import BcTower, Layout, MacProjector


def _fields(n, seed):
    rng = np.random.default_rng(seed)
    nr = n[-1]
    f = lambda: np.asfortranarray(rng.standard_normal(n))  # noqa: E731
    base = dict(Sbar=rng.standard_normal(nr), beta0=1.0 + rng.random(nr),
                gamma1bar=1.4 + 0.1 * rng.random(nr), p0=1e5 * (1.0 + rng.random(nr)))
    return f(), f(), f(), f(), base


def test_oracle_make_macrhs_by_hand():
    S = np.asfortranarray(np.arange(8.0).reshape(2, 2, 2, order="F"))
    dg = np.full_like(S, 0.5)
    Sbar = np.array([1.0, 2.0])
    beta0 = np.array([3.0, 4.0])
    rhs, _ = O.make_macrhs(S, dg, Sbar, beta0)
    expect = np.empty_like(S)
    for k in range(2):
        expect[:, :, k] = beta0[k] * (S[:, :, k] - Sbar[k] + 0.5)
    np.testing.assert_array_equal(rhs, expect)
    # dpdt term below the cutoff (k = 0 only), predictor zeroes delta_chi first
    dp = np.full_like(S, 2.0)
    chi0 = np.full_like(S, 9.0)
    rhs2, chi = O.make_macrhs(S, dg, Sbar, beta0, gamma1bar=np.array([2.0, 2.0]),
                              p0=np.array([5.0, 5.0]), delta_p_term=dp, delta_chi=chi0, dt=0.5,
                              dpdt_factor=0.25, base_cutoff_density_coord=1, is_predictor=True)
    inc = 0.25 * 2.0 / (0.5 * 2.0 * 5.0)
    np.testing.assert_allclose(chi[:, :, 0], inc)
    np.testing.assert_array_equal(chi[:, :, 1], 0.0)
    np.testing.assert_allclose(rhs2[:, :, 0], expect[:, :, 0] + beta0[0] * inc)
    np.testing.assert_array_equal(rhs2[:, :, 1], expect[:, :, 1])
    # corrector keeps delta_chi and adds to it
    _, chi_c = O.make_macrhs(S, dg, Sbar, beta0, gamma1bar=np.array([2.0, 2.0]),
                             p0=np.array([5.0, 5.0]), delta_p_term=dp, delta_chi=chi0, dt=0.5,
                             dpdt_factor=0.25, base_cutoff_density_coord=1, is_predictor=False)
    np.testing.assert_allclose(chi_c[:, :, 0], 9.0 + inc)
    np.testing.assert_array_equal(chi_c[:, :, 1], 9.0)


@pytest.mark.gpu
@pytest.mark.parametrize("dm", [2, 3])
@pytest.mark.parametrize("mode", ["plain", "predictor", "corrector"])
def test_make_macrhs_matches_oracle(cuda_lib, dm, mode):
    n = (32, 24, 16) if dm == 3 else (48, 32)
    box = (16, 12, 8) if dm == 3 else (16, 16)
    S, dg, dp, chi0, base = _fields(n, 11 + dm)
    dpdt = 0.0 if mode == "plain" else 0.3
    pred = mode == "predictor"
    cut = n[-1] - 5
    rhs_o, chi_o = O.make_macrhs(S, dg, base["Sbar"], base["beta0"], base["gamma1bar"], base["p0"],
                                 dp, chi0, dt=0.01, dpdt_factor=dpdt,
                                 base_cutoff_density_coord=cut, is_predictor=pred)
    lay = Layout.tiled(n, box)
    bc = BcTower((BC_PER,) * (dm - 1) + (BC_NEU,), (BC_PER,) * (dm - 1) + (BC_NEU,))
    P = MacProjector(lay, [1.0 / v for v in n], bc)
    try:
        f_rhs = [np.asfortranarray(np.zeros_like(f)) for f in lay.to_fabs(S, ng=0)]
        f_chi = lay.to_fabs(chi0, ng=1)
        P.make_macrhs(f_rhs, lay.to_fabs(S, ng=0), lay.to_fabs(dg, ng=0), base["Sbar"],
                      base["beta0"], base["gamma1bar"], base["p0"], lay.to_fabs(dp, ng=0), f_chi,
                      dt=0.01, dpdt_factor=dpdt, base_cutoff_density_coord=cut, is_predictor=pred,
                      ng_d=1)
    finally:
        P.close()
    rhs = lay.from_fabs(f_rhs, ng=0)
    scale = np.abs(rhs_o).max()
    assert np.abs(rhs - rhs_o).max() <= 1e-14 * scale
    if dpdt > 0:
        chi = lay.from_fabs(f_chi, ng=1)
        assert np.abs(chi - chi_o).max() <= 1e-14 * np.abs(chi_o).max()


@pytest.mark.gpu
def test_make_macrhs_dense_matches_oracle(cuda_lib):
    torch = pytest.importorskip("torch")
    n = (32, 32, 24)
    S, dg, dp, chi0, base = _fields(n, 5)
    rhs_o, chi_o = O.make_macrhs(S, dg, base["Sbar"], base["beta0"], base["gamma1bar"], base["p0"],
                                 dp, chi0, dt=0.02, dpdt_factor=0.5, base_cutoff_density_coord=17,
                                 is_predictor=False)
    dev = torch.device("cuda", 0)
    t = lambda a: torch.from_numpy(np.ascontiguousarray(np.asarray(a).transpose())).to(dev)  # noqa: E731
    v = lambda a: torch.from_numpy(np.asarray(a, dtype=np.float64)).to(dev)  # noqa: E731
    rhs = torch.zeros_like(t(S))
    chi = t(chi0)
    lay = Layout.tiled(n, n)
    P = MacProjector(lay, [1.0 / x for x in n], BcTower((BC_PER, BC_PER, BC_NEU),
                                                        (BC_PER, BC_PER, BC_NEU)))
    from maestro_gb300 import capi
    try:
        keep = [t(S), t(dg), v(base["Sbar"]), v(base["beta0"]), v(base["gamma1bar"]),
                v(base["p0"]), t(dp)]
        rc = capi.lib().mac_make_macrhs_dense(
            P.ctx, rhs.data_ptr(), keep[0].data_ptr(), keep[1].data_ptr(), keep[2].data_ptr(),
            keep[3].data_ptr(), keep[4].data_ptr(), keep[5].data_ptr(), keep[6].data_ptr(),
            chi.data_ptr(), 0.02, 0.5, 17, 0)
        assert rc == 0
    finally:
        P.close()
    back = lambda x: np.asfortranarray(x.cpu().numpy().transpose())  # noqa: E731
    assert np.abs(back(rhs) - rhs_o).max() <= 1e-14 * np.abs(rhs_o).max()
    assert np.abs(back(chi) - chi_o).max() <= 1e-14 * np.abs(chi_o).max()


@pytest.mark.gpu
def test_make_at_halftime_matches_oracle(cuda_lib):
    n = (24, 16, 16)
    rng = np.random.default_rng(3)
    ncomp = 3
    so = np.asfortranarray(rng.standard_normal(n + (ncomp,)))
    sn = np.asfortranarray(rng.standard_normal(n + (ncomp,)))
    lay = Layout.tiled(n, (12, 8, 8))
    bc = BcTower((BC_PER, BC_PER, BC_NEU), (BC_PER, BC_PER, BC_NEU))
    P = MacProjector(lay, [1.0 / v for v in n], bc)

    def fabs_nc(a):
        return lay.to_fabs(a, ng=1, periodic=[True, True, False], ncomp=ncomp)
    try:
        half = [np.asfortranarray(np.zeros_like(f)) for f in lay.to_fabs(so[..., 1], ng=1)]
        P.make_at_halftime(half, fabs_nc(so), fabs_nc(sn), in_comp=1, s_ncomp=ncomp)
    finally:
        P.close()
    got = lay.from_fabs(half, ng=1)
    np.testing.assert_array_equal(got, O.make_at_halftime(so[..., 1], sn[..., 1]))
