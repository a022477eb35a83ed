"""Seeded synthetic inputs for the MAC projection: a stratified, planar atmosphere.

No public dataset exists for this path; the workloads are the stratified-atmosphere cases of the
MAC projection benchmark (2D 128^2, 3D 256^3 / 384^3 / 512^3 in 128^3 boxes), generated here:

* domain [0,1]^dm, vertical direction = the last one (MAESTRO planar geometry), cell-centred
  heights z_k = (k + 1/2) dz;
* base density rho0(z) = 1e7 exp(-z / H), H a fraction of the domain height;
* cell density rho = rho0 (1 + sigma N(0,1)) ("linear" noise) or rho0 exp(sigma N(0,1))
  ("lognormal" noise);
* beta0 = rho0^(1/1.4) at cell centres, beta0 at edges by the limited fourth-order rule of
  Source/cell_to_edge.f90:14-70 (`cell_to_edge` below);
* U_edge: a sum of random Fourier modes with |k| <= kmax, amplitude 1e6 cm/s; horizontal
  directions periodic (e^{2 pi i k x}), vertical direction a slip wall: the wall-normal
  component goes like sin(k pi z), the tangential ones like cos(k pi z), so U.n = 0 on the walls;
  the field is divergent;
* S - Sbar: Gaussian noise of amplitude 1e-3 s^-1 with the mean of every horizontal layer
  removed, so macrhs = beta0 (S - Sbar) (Source/make_macrhs.f90:228-229) is compatible with the
  singular periodic/Neumann problem;
* w: N(0,1) face weights for the adjoint loss L = sum(w . U_proj).

Arrays are float64, Fortran order, indexed like MAESTRO's fabs: cells (nx, ny[, nz]); faces with one
extra entry along their own direction.
"""
from __future__ import annotations

import dataclasses

import numpy as np

BC_PER, BC_INT, BC_DIR, BC_NEU = -1, 0, 1, 2


def cell_to_edge(s0_cell: np.ndarray) -> np.ndarray:
    """Edge values of a 1D base-state array (Source/cell_to_edge.f90:14-70, one level).

    Copies at the two domain ends, arithmetic means one cell in, limited fourth-order
    7/12 (a+b) - 1/12 (c+d) clipped to [min(a,b), max(a,b)] elsewhere.
    """
    c = np.asarray(s0_cell, dtype=np.float64)
    nr = c.size
    e = np.empty(nr + 1)
    for r in range(nr + 1):
        if r == 0:
            e[r] = c[0]
        elif r == 1:
            e[r] = 0.5 * (c[0] + c[1])
        elif r == nr:
            e[r] = c[nr - 1]
        elif r == nr - 1:
            e[r] = 0.5 * (c[r] + c[r - 1])
        else:
            tmp = 7.0 / 12.0 * (c[r] + c[r - 1]) - 1.0 / 12.0 * (c[r + 1] + c[r - 2])
            e[r] = min(max(tmp, min(c[r], c[r - 1])), max(c[r], c[r - 1]))
    return e


@dataclasses.dataclass
class MacCase:
    """One MAC-projection input set on the whole domain (single level)."""

    name: str
    dm: int
    n: tuple
    box: tuple                 # box extent (cells per direction); boxes tile the domain
    dx: tuple
    bc_lo: tuple
    bc_hi: tuple
    rho: np.ndarray
    beta0: np.ndarray
    beta0_edge: np.ndarray
    umac: list
    macrhs: np.ndarray
    phi0: np.ndarray
    w: list | None = None
    seed: int = 0

    @property
    def ncell(self) -> int:
        return int(np.prod(self.n))

    def boxes(self):
        """(lo, hi) inclusive cell bounds of every box, x fastest (FBoxLib box list order)."""
        nb = [self.n[d] // self.box[d] for d in range(self.dm)]
        out = []
        for idx in np.ndindex(*reversed(nb)):
            idx = tuple(reversed(idx))
            lo = tuple(idx[d] * self.box[d] for d in range(self.dm))
            hi = tuple(lo[d] + self.box[d] - 1 for d in range(self.dm))
            out.append((lo, hi))
        return out


def _modes(kmax: int, dm: int):
    """Integer wave vectors with |k| <= kmax: horizontal in [-kmax, kmax], vertical in [0, kmax]."""
    ks = []
    r = range(-kmax, kmax + 1)
    if dm == 2:
        for kx in r:
            for kz in range(0, kmax + 1):
                if kx * kx + kz * kz <= kmax * kmax and (kx, kz) != (0, 0):
                    ks.append((kx, kz))
    else:
        for kx in r:
            for ky in r:
                for kz in range(0, kmax + 1):
                    if kx * kx + ky * ky + kz * kz <= kmax * kmax and (kx, ky, kz) != (0, 0, 0):
                        ks.append((kx, ky, kz))
    return np.array(ks, dtype=np.int64)


def _fourier_component(rng, n, dm, d, kmax, dtype=np.float64):
    """Random real field on the faces normal to direction d (see module docstring)."""
    modes = _modes(kmax, dm)
    coef = rng.standard_normal(len(modes)) + 1j * rng.standard_normal(len(modes))
    K = 2 * kmax + 1
    kz_n = kmax + 1
    if dm == 2:
        C = np.zeros((K, kz_n), dtype=np.complex128)
        C[modes[:, 0] + kmax, modes[:, 1]] = coef
    else:
        C = np.zeros((K, K, kz_n), dtype=np.complex128)
        C[modes[:, 0] + kmax, modes[:, 1] + kmax, modes[:, 2]] = coef
    shape = list(n)
    shape[d] += 1
    pos = []
    for e in range(dm):
        m = shape[e]
        if e == d:
            pos.append(np.arange(m) / n[e])            # faces
        else:
            pos.append((np.arange(m) + 0.5) / n[e])    # cell centres
    kh = np.arange(-kmax, kmax + 1)
    kv = np.arange(0, kmax + 1)
    # vertical basis: sin for the wall-normal component, cos for the tangential ones
    zv = pos[dm - 1]
    Z = np.sin(np.pi * np.outer(kv, zv)) if d == dm - 1 else np.cos(np.pi * np.outer(kv, zv))
    Ex = np.exp(2j * np.pi * np.outer(kh, pos[0]))           # (K, mx)
    if dm == 2:
        T = C @ Z                                            # (K, mz)
        u = np.real(Ex.T @ T)                                # (mx, mz)
    else:
        Ey = np.exp(2j * np.pi * np.outer(kh, pos[1]))       # (K, my)
        T1 = np.tensordot(C, Z, axes=([2], [0]))             # (K, K, mz)
        T2 = np.tensordot(T1, Ey, axes=([1], [0]))           # (K, mz, my)
        T2 = np.transpose(T2, (0, 2, 1)).reshape(K, -1)      # (K, my*mz)
        u = np.real(Ex.T @ T2).reshape(shape[0], shape[1], shape[2], order="C")
    u = np.asfortranarray(u.astype(dtype))
    return u


def make_case(name: str = "custom", dm: int = 3, n=(64, 64, 64), box=None, H_frac: float = 0.25,
              noise: float = 0.01, noise_kind: str = "lognormal", kmax: int = 8, seed: int = 1234,
              u_amp: float = 1e6, s_amp: float = 1e-3, with_w: bool = False) -> MacCase:
    """Build a seeded stratified-atmosphere MAC case (see module docstring)."""
    n = tuple(int(v) for v in n)
    assert len(n) == dm
    box = tuple(box) if box is not None else n
    rng = np.random.default_rng(seed)
    dx = tuple(1.0 / n[d] for d in range(dm))
    nz = n[dm - 1]
    z = (np.arange(nz) + 0.5) / nz
    H = H_frac * 1.0
    rho0 = 1e7 * np.exp(-z / H)
    bshape = [1] * dm
    bshape[dm - 1] = nz
    rho0_b = rho0.reshape(bshape)
    g = rng.standard_normal(n)
    if noise_kind == "linear":
        rho = rho0_b * (1.0 + noise * g)
    else:
        rho = rho0_b * np.exp(noise * g)
    rho = np.asfortranarray(rho)
    beta0 = rho0 ** (1.0 / 1.4)
    beta0_edge = cell_to_edge(beta0)
    umac = []
    for d in range(dm):
        u = _fourier_component(rng, n, dm, d, kmax)
        m = np.max(np.abs(u))
        umac.append(np.asfortranarray(u * (u_amp / m if m > 0 else 1.0)))
    s = rng.standard_normal(n) * s_amp
    axes = tuple(range(dm - 1))
    s = s - s.mean(axis=axes, keepdims=True)
    macrhs = np.asfortranarray(beta0.reshape(bshape) * s)
    w = None
    if with_w:
        w = []
        for d in range(dm):
            shp = list(n)
            shp[d] += 1
            w.append(np.asfortranarray(rng.standard_normal(shp)))
    bc_lo = tuple([BC_PER] * (dm - 1) + [BC_NEU])
    bc_hi = tuple([BC_PER] * (dm - 1) + [BC_NEU])
    return MacCase(name=name, dm=dm, n=n, box=box, dx=dx, bc_lo=bc_lo, bc_hi=bc_hi, rho=rho,
                   beta0=beta0, beta0_edge=beta0_edge, umac=umac, macrhs=macrhs,
                   phi0=np.zeros(n, order="F"), w=w, seed=seed)


def make_spherical_case(name: str = "spherical", n=(64, 64, 64), box=None, H_frac: float = 0.2,
                        noise: float = 0.01, kmax: int = 6, seed: int = 4321, u_amp: float = 1e6,
                        s_amp: float = 1e-3, bc: str = "outflow") -> MacCase:
    """A 3-D star-like case for the spherical form of the projection (beta0 on every face).

    MAESTRO's spherical geometry keeps a Cartesian grid and hands macproject beta0 as a 3-D face
    multifab (beta0_cart_edge) instead of 1-D arrays.  Here rho0(r) = 1e7 exp(-r / H) with r the
    distance from the domain centre, cell rho = rho0(r_cell) exp(sigma N(0,1)), beta0 =
    rho0^(1/1.4) evaluated at every face centre (returned as ``case.b0c``, one array per
    direction), macrhs = beta0(r_cell) (S - Sbar) with S Gaussian noise, U_edge a random
    divergent Fourier field.  ``bc``: "outflow" (Dirichlet phi on every face, the usual spherical
    setup) or "periodic".  ``beta0``/``beta0_edge`` are None.
    """
    dm = 3
    n = tuple(int(v) for v in n)
    box = tuple(box) if box is not None else n
    rng = np.random.default_rng(seed)
    dx = tuple(1.0 / n[d] for d in range(dm))
    H = H_frac

    def rho0(x, y, z):
        r = np.sqrt((x - 0.5) ** 2 + (y - 0.5) ** 2 + (z - 0.5) ** 2)
        return 1e7 * np.exp(-r / H)

    xc = [(np.arange(n[d]) + 0.5) / n[d] for d in range(dm)]
    X, Y, Z = np.meshgrid(*xc, indexing="ij")
    r0c = rho0(X, Y, Z)
    rho = np.asfortranarray(r0c * np.exp(noise * rng.standard_normal(n)))
    b0c = []
    for d in range(dm):
        pos = [xc[e] if e != d else np.arange(n[d] + 1) / n[d] for e in range(dm)]
        F = np.meshgrid(*pos, indexing="ij")
        b0c.append(np.asfortranarray(rho0(*F) ** (1.0 / 1.4)))
    umac = []
    for d in range(dm):
        u = _fourier_component(rng, n, dm, d, kmax)
        m = np.max(np.abs(u))
        umac.append(np.asfortranarray(u * (u_amp / m if m > 0 else 1.0)))
    s = rng.standard_normal(n) * s_amp
    if bc == "periodic":
        s = s - s.mean()
        bc_lo = bc_hi = (BC_PER, BC_PER, BC_PER)
    else:
        bc_lo = bc_hi = (BC_DIR, BC_DIR, BC_DIR)
    macrhs = np.asfortranarray(r0c ** (1.0 / 1.4) * s)
    c = MacCase(name=name, dm=dm, n=n, box=box, dx=dx, bc_lo=bc_lo, bc_hi=bc_hi, rho=rho,
                beta0=None, beta0_edge=None, umac=umac, macrhs=macrhs,
                phi0=np.zeros(n, order="F"), seed=seed)
    c.b0c = b0c
    return c


# The five MAC-projection workloads (sizes, boxes, stratification, noise, spectrum).
CONFIGS = {
    "2d_128": dict(dm=2, n=(128, 128), box=(128, 128), H_frac=0.25, noise=0.01,
                   noise_kind="linear", kmax=8),
    "3d_256": dict(dm=3, n=(256, 256, 256), box=(128, 128, 128), H_frac=0.25, noise=0.01,
                   noise_kind="lognormal", kmax=16),
    "3d_512_mixed": dict(dm=3, n=(512, 512, 512), box=(128, 128, 128), H_frac=0.15, noise=0.01,
                         noise_kind="lognormal", kmax=32),
    "3d_256_adjoint": dict(dm=3, n=(256, 256, 256), box=(128, 128, 128), H_frac=0.25,
                           noise=0.01, noise_kind="lognormal", kmax=16, with_w=True),
    "3d_384_stiff": dict(dm=3, n=(384, 384, 384), box=(128, 128, 128), H_frac=0.072,
                         noise=0.05, noise_kind="lognormal", kmax=16),
}


def config_case(key: str, seed: int = 1234, scale: int = 1) -> MacCase:
    """One of CONFIGS; `scale` > 1 divides every extent (and the box) by it for small tests."""
    kw = dict(CONFIGS[key])
    if scale > 1:
        kw["n"] = tuple(v // scale for v in kw["n"])
        kw["box"] = tuple(max(2, v // scale) for v in kw["box"])
        kw["kmax"] = max(2, kw["kmax"] // scale)
    return make_case(name=key, seed=seed, **kw)


# ------------------------------------------------------------------ multi-level (AMR) inputs

@dataclasses.dataclass
class AmrCase:
    """A MAC-projection input set on an AMR hierarchy with refinement ratio 2.

    Level l spans the whole level domain (n0 << l cells per direction) as dense arrays; only the
    cells of its boxes (`boxes[l]`, (lo, hi) inclusive in level-l indices; level 0 is the
    domain) carry data.  rho, macrhs, phi0: cell arrays per level; umac: dm face arrays per
    level; beta0 / beta0_edge: the planar base state of every level."""

    name: str
    dm: int
    n0: tuple
    dx0: tuple
    bc_lo: tuple
    bc_hi: tuple
    boxes: list
    rho: list
    beta0: list
    beta0_edge: list
    umac: list
    macrhs: list
    phi0: list
    seed: int = 0

    @property
    def nlev(self) -> int:
        return len(self.boxes)

    def shape(self, l: int) -> tuple:
        return tuple(int(v) << l for v in self.n0)

    def dx(self, l: int) -> tuple:
        return tuple(h / (1 << l) for h in self.dx0)


def _smooth_cell_field(seed: int, n, dm: int, kmax: int):
    """Seeded smooth cell-centred field of unit max: cosine modes, periodic horizontally,
    cos(k pi z) vertically, so every resolution samples the same function."""
    rng = np.random.default_rng(seed)
    pos = [(np.arange(n[e]) + 0.5) / n[e] for e in range(dm)]
    X = np.meshgrid(*pos, indexing="ij")
    f = np.zeros(tuple(n))
    for _ in range(4 * kmax):
        k = rng.integers(-kmax, kmax + 1, size=dm)
        k[dm - 1] = abs(k[dm - 1])
        ph = rng.uniform(0, 2 * np.pi, size=dm)
        a = rng.standard_normal() / (1.0 + float(np.sum(k * k)))
        t = a * np.cos(np.pi * k[dm - 1] * X[dm - 1] + ph[dm - 1])
        for e in range(dm - 1):
            t = t * np.cos(2 * np.pi * k[e] * X[e] + ph[e])
        f += t
    m = np.max(np.abs(f))
    return f / (m if m > 0 else 1.0)


def average_down(fine: np.ndarray) -> np.ndarray:
    """Mean of the 2^dm children of every coarse cell."""
    dm = fine.ndim
    out = 0.0
    for a in range(1 << dm):
        out = out + fine[tuple(slice((a >> e) & 1, None, 2) for e in range(dm))]
    return out / (1 << dm)


def region_mask(shape, boxes) -> np.ndarray:
    m = np.zeros(shape, dtype=bool)
    for lo, hi in boxes:
        m[tuple(slice(lo[e], hi[e] + 1) for e in range(len(shape)))] = True
    return m


def make_amr_case(name: str = "amr", dm: int = 2, n0=(32, 32), boxes=None, H_frac: float = 0.25,
                  noise: float = 0.05, kmax: int = 4, seed: int = 2024, u_amp: float = 1e6,
                  s_amp: float = 1e-3, bc: str = "wall") -> AmrCase:
    """Seeded stratified-atmosphere MAC case on an AMR hierarchy (the planar workload of
    `make_case`, smooth so that every level samples the same fields).

    rho = rho0(z) exp(noise P(x)) with P a smooth unit-max field, beta0 = rho0^(1/1.4) per level
    with cell_to_edge edges, U the Fourier field of `make_case` sampled on each level's faces,
    macrhs = beta0 (S - Sbar) with S smooth and Sbar its layer mean on each level.  The density of
    covered cells is the mean of their children (the state after MAESTRO's average-down).
    bc: "wall" (periodic horizontally, slip walls vertically), "periodic", or "outflow" (periodic
    horizontally, a slip wall below and an outflow face, phi = 0, above)."""
    n0 = tuple(int(v) for v in n0)
    assert len(n0) == dm
    boxes = [[]] + [list(b) for b in (boxes or [])[1:]] if boxes else [[]]
    nlev = len(boxes)
    dx0 = tuple(1.0 / n0[0] for _ in range(dm))
    bc_v = BC_PER if bc == "periodic" else BC_NEU
    bc_lo = tuple([BC_PER] * (dm - 1) + [bc_v])
    bc_hi = tuple([BC_PER] * (dm - 1) + [BC_DIR]) if bc == "outflow" else bc_lo
    rho, b0, b0e, umac, macrhs, phi0 = [], [], [], [], [], []
    # U normalisation from level 0 so all levels carry the same field
    norms = []
    for d in range(dm):
        u0 = _fourier_component(np.random.default_rng(seed + 10 + d), n0, dm, d, kmax)
        m = float(np.max(np.abs(u0)))
        norms.append(u_amp / m if m > 0 else 1.0)
    for l in range(nlev):
        n = tuple(v << l for v in n0)
        nz = n[dm - 1]
        z = (np.arange(nz) + 0.5) / nz
        rho0 = 1e7 * np.exp(-z / H_frac)
        shp = [1] * dm
        shp[dm - 1] = nz
        P = _smooth_cell_field(seed, n, dm, kmax)
        rho.append(rho0.reshape(shp) * np.exp(noise * P))
        beta0 = rho0 ** (1.0 / 1.4)
        b0.append(beta0)
        b0e.append(cell_to_edge(beta0))
        umac.append([np.asfortranarray(
            _fourier_component(np.random.default_rng(seed + 10 + d), n, dm, d, kmax) * norms[d])
            for d in range(dm)])
        S = s_amp * _smooth_cell_field(seed + 1, n, dm, kmax)
        S = S - S.mean(axis=tuple(range(dm - 1)), keepdims=True)
        macrhs.append(np.asfortranarray(beta0.reshape(shp) * S))
        phi0.append(np.zeros(n, order="F"))
    for l in range(nlev - 1, 0, -1):
        cov = region_mask(tuple(v << (l - 1) for v in n0),
                          [(tuple(a // 2 for a in lo), tuple(b // 2 for b in hi)) for lo, hi in boxes[l]])
        rho[l - 1] = np.where(cov, average_down(rho[l]), rho[l - 1])
    rho = [np.asfortranarray(r) for r in rho]
    return AmrCase(name=name, dm=dm, n0=n0, dx0=dx0, bc_lo=bc_lo, bc_hi=bc_hi, boxes=boxes,
                   rho=rho, beta0=b0, beta0_edge=b0e, umac=umac, macrhs=macrhs, phi0=phi0,
                   seed=seed)


AMR_CASES = {
    # two levels, a fine patch in the middle of a 2-D atmosphere
    "amr2d_32": dict(dm=2, n0=(32, 32), boxes=[[], [((16, 8), (47, 39))]]),
    # two fine boxes, one wrapping the periodic x boundary, one on the bottom wall
    "amr2d_wrap": dict(dm=2, n0=(32, 32), boxes=[[], [((0, 16), (11, 47)), ((52, 16), (63, 47)),
                                                       ((24, 0), (39, 15))]]),
    # three levels
    "amr2d_3lev": dict(dm=2, n0=(32, 32), boxes=[[], [((8, 8), (55, 55))], [((32, 32), (79, 79))]]),
    # 3-D, two levels, two boxes
    "amr3d_16": dict(dm=3, n0=(16, 16, 16), boxes=[[], [((8, 8, 8), (23, 23, 23)),
                                                          ((0, 0, 24), (7, 31, 31))]]),
    # outflow (Dirichlet) top with a fine box against it, three levels
    "amr2d_outflow": dict(dm=2, n0=(32, 16), bc="outflow",
                          boxes=[[], [((16, 8), (47, 31))], [((40, 24), (79, 63))]]),
    # 3-D, three levels, the finest box against the bottom wall
    "amr3d_3lev": dict(dm=3, n0=(8, 8, 8), boxes=[[], [((2, 2, 0), (13, 13, 9))],
                                                   [((8, 8, 0), (19, 19, 11))]]),
}


def amr_case(key: str, seed: int = 2024) -> AmrCase:
    return make_amr_case(name=key, seed=seed, **AMR_CASES[key])
