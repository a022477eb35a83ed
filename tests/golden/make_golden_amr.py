"""Golden fixtures that pin the multi-level (AMR) MAC-projection oracle.

The reference's composite solve lives in the un-vendored FBoxLib (ml_cc_solve) and its repository
holds no numeric outputs for it, so the fixtures come from an MG-independent computation of the
same discrete composite problem, written here with numpy/scipy and sharing no code with the C++
oracle (oracle/mac_oracle_ml.cpp) or the CUDA library:

  * unknowns       the valid cells of every level (level-l cells not under level l+1); a covered
                   cell's value is the mean of its children (recursively)
  * fine arms      beta_f (u_c - u_nb) / h^2; at a coarse-fine face the neighbour is the ghost
                   u_c / 3 + 2/3 u_crse, u_crse the coarse cell across the face corrected along
                   each tangential direction by the quadratic through its tangential neighbours
                   at the ghost's offset +-1/4 (one-sided linear at a non-periodic domain face)
  * coarse arms    next to a covered cell: the mean of the 2^(dm-1) fine fluxes
                   beta_f (ghost - u_fine) / h_fine through the fine faces tiling the face
  * physical faces Neumann dropped, periodic wrapped, Dirichlet with the ghost -u_c
  * MAC steps      Source/macproject.f90:51-328 with nlevs > 1: beta0 U, ml_edge_restriction of
                   the fine faces onto the coarse faces they tile, rh = -(div(beta0 U) - macrhs)
                   per level, coarse rh under a fine level = mean of the fine rh, beta_f =
                   beta0 * 2 / (rho_L + rho_R) per level, the composite solve (sparse LU with the
                   volume-weighted mean of phi pinned to zero for the singular problem), mkumac on
                   every level with the composite ghosts at coarse-fine faces, edge restriction,
                   division by beta0, edge restriction again.

Run from the repository root:  python tests/golden/make_golden_amr.py
"""
from __future__ import annotations

import itertools
import os
import sys

import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spl

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
sys.path.insert(0, HERE)

from maestro_gb300.inputs import (BC_DIR, BC_PER, AMR_CASES, amr_case, average_down,  # noqa: E402
                                  region_mask)
from make_golden import face_coeffs  # noqa: E402


class Hierarchy:
    """Masks, unknown numbering and the covered-value maps of an AMR layout."""

    def __init__(self, n0, dx0, bc_lo, bc_hi, boxes):
        self.dm = len(n0)
        self.n0 = tuple(n0)
        self.L = len(boxes)
        self.bc_lo, self.bc_hi = tuple(bc_lo), tuple(bc_hi)
        self.shape = [tuple(v << l for v in n0) for l in range(self.L)]
        self.h = [tuple(x / (1 << l) for x in dx0) for l in range(self.L)]
        self.inm = [np.ones(self.shape[0], dtype=bool)] + [
            region_mask(self.shape[l], boxes[l]) for l in range(1, self.L)]
        self.cov = []
        for l in range(self.L):
            if l + 1 < self.L:
                f = self.inm[l + 1]
                c = np.zeros(self.shape[l], dtype=bool)
                for a in range(1 << self.dm):
                    c |= f[tuple(slice((a >> e) & 1, None, 2) for e in range(self.dm))]
                self.cov.append(c)
            else:
                self.cov.append(np.zeros(self.shape[l], dtype=bool))
        self.valid = [self.inm[l] & ~self.cov[l] for l in range(self.L)]
        self.uid = []
        base = 0
        for l in range(self.L):
            flat = np.flatnonzero(self.valid[l].ravel(order="F"))
            uf = -np.ones(int(np.prod(self.shape[l])), dtype=np.int64)
            uf[flat] = base + np.arange(flat.size)
            u = np.asfortranarray(uf.reshape(self.shape[l], order="F"))
            self.uid.append(u)
            base += flat.size
        self.nunk = base
        self.vol = np.concatenate([
            np.full(int(self.valid[l].sum()), float(np.prod(self.h[l]))) for l in range(self.L)])
        # value maps: level-l cell values (Fortran flat order) from the unknowns
        self.V = [None] * self.L
        for l in range(self.L - 1, -1, -1):
            nc = int(np.prod(self.shape[l]))
            vf = self.valid[l].ravel(order="F")
            rows = np.flatnonzero(vf)
            sel = sp.csr_matrix((np.ones(rows.size), (rows, self.uid[l].ravel(order="F")[rows])),
                                shape=(nc, self.nunk))
            if l + 1 < self.L:
                sel = sel + self._avg_matrix(l) @ self.V[l + 1]
            self.V[l] = sel.tocsr()

    def _avg_matrix(self, l):
        """Covered level-l cells <- mean of their level-(l+1) children."""
        nc = int(np.prod(self.shape[l]))
        nf = int(np.prod(self.shape[l + 1]))
        rows, cols = [], []
        idx = np.argwhere(self.cov[l])
        for a in range(1 << self.dm):
            ch = idx * 2 + np.array([(a >> e) & 1 for e in range(self.dm)])
            rows.append(np.ravel_multi_index(idx.T, self.shape[l], order="F"))
            cols.append(np.ravel_multi_index(ch.T, self.shape[l + 1], order="F"))
        rows = np.concatenate(rows)
        cols = np.concatenate(cols)
        return sp.csr_matrix((np.full(rows.size, 1.0 / (1 << self.dm)), (rows, cols)),
                             shape=(nc, nf))

    def wrap(self, l, d, q):
        n = self.shape[l][d]
        if 0 <= q < n:
            return q
        per = (self.bc_lo[d] if q < 0 else self.bc_hi[d]) == BC_PER
        return q % n if per else None

    def flat(self, l, c):
        return int(np.ravel_multi_index(tuple(c), self.shape[l], order="F"))

    def coarse_weights(self, l, q, d):
        """Weights over level-(l-1) cells of the coarse value at the fine ghost q (level l)."""
        K = [v // 2 for v in q]
        w = {tuple(K): 1.0}

        def add(key, v):
            w[key] = w.get(key, 0.0) + v

        for t in range(self.dm):
            if t == d:
                continue
            dl = 0.25 if q[t] % 2 else -0.25
            km = self.wrap(l - 1, t, K[t] - 1)
            kp = self.wrap(l - 1, t, K[t] + 1)
            Km = list(K)
            Kp = list(K)
            if km is not None:
                Km[t] = km
            if kp is not None:
                Kp[t] = kp
            if km is not None and kp is not None:
                add(tuple(Kp), dl / 2 + dl * dl / 2)
                add(tuple(Km), -dl / 2 + dl * dl / 2)
                add(tuple(K), -dl * dl)
            elif kp is not None:
                add(tuple(Kp), dl)
                add(tuple(K), -dl)
            elif km is not None:
                add(tuple(K), dl)
                add(tuple(Km), -dl)
        return w


def composite_matrix(H: Hierarchy, beta):
    """The composite operator (rows: valid cells, columns: unknowns)."""
    dm = H.dm
    trip = [([], [], []) for _ in range(H.L)]

    def put(l, r, c, v):
        trip[l][0].append(r)
        trip[l][1].append(H.flat(l, c))
        trip[l][2].append(v)

    for l in range(H.L):
        for c in np.argwhere(H.valid[l]):
            c = [int(v) for v in c]
            row = int(H.uid[l][tuple(c)])
            for d in range(dm):
                ih2 = 1.0 / H.h[l][d] ** 2
                for s in (-1, 1):
                    fidx = list(c)
                    fidx[d] += 1 if s > 0 else 0
                    w = beta[l][d][tuple(fidx)] * ih2
                    qd = H.wrap(l, d, c[d] + s)
                    if qd is None:
                        bc = H.bc_lo[d] if s < 0 else H.bc_hi[d]
                        if bc == BC_DIR:
                            put(l, row, c, 2.0 * w)
                        continue
                    q = list(c)
                    q[d] = qd
                    if H.inm[l][tuple(q)]:
                        if H.cov[l][tuple(q)]:
                            # reflux: the mean of the fine fluxes through the face
                            nf = 1 << (dm - 1)
                            tdirs = [e for e in range(dm) if e != d]
                            for bits in itertools.product((0, 1), repeat=dm - 1):
                                fc = [0] * dm
                                gq = [0] * dm
                                fc[d] = 2 * qd if s > 0 else 2 * qd + 1
                                gq[d] = 2 * c[d] + 1 if s > 0 else 2 * c[d]
                                for e, b in zip(tdirs, bits):
                                    fc[e] = gq[e] = 2 * c[e] + b
                                ff = list(fc)
                                ff[d] += 0 if s > 0 else 1
                                bf = beta[l + 1][d][tuple(ff)]
                                k = bf / (H.h[l + 1][d] * H.h[l][d] * nf)
                                put(l + 1, row, fc, -(2.0 / 3.0) * k)
                                for K, wk in H.coarse_weights(l + 1, gq, d).items():
                                    put(l, row, K, (2.0 / 3.0) * k * wk)
                        else:
                            put(l, row, c, w)
                            put(l, row, q, -w)
                    else:
                        put(l, row, c, (2.0 / 3.0) * w)
                        for K, wk in H.coarse_weights(l, q, d).items():
                            put(l - 1, row, K, -(2.0 / 3.0) * w * wk)
    A = sp.csr_matrix((H.nunk, H.nunk))
    for l in range(H.L):
        r, cidx, v = trip[l]
        if not r:
            continue
        T = sp.csr_matrix((v, (r, cidx)), shape=(H.nunk, int(np.prod(H.shape[l]))))
        A = A + T @ H.V[l]
    return A.tocsr()


def singular(bc_lo, bc_hi):
    return BC_DIR not in tuple(bc_lo) + tuple(bc_hi)


def composite_solve(H: Hierarchy, beta, rh):
    """phi per level (covered = mean of children, outside a level's region 0)."""
    A = composite_matrix(H, beta)
    f = np.concatenate([rh[l].ravel(order="F")[np.flatnonzero(H.valid[l].ravel(order="F"))]
                        for l in range(H.L)])
    if singular(H.bc_lo, H.bc_hi):
        f = f - np.dot(H.vol, f) / H.vol.sum()
        w = H.vol[:, None]
        B = sp.bmat([[A, sp.csr_matrix(w)], [sp.csr_matrix(w.T), None]]).tocsc()
        x = spl.spsolve(B, np.concatenate([f, [0.0]]))[:-1]
    else:
        x = spl.spsolve(A.tocsc(), f)
    return [np.asfortranarray((H.V[l] @ x).reshape(H.shape[l], order="F")) for l in range(H.L)]


def face_member(H: Hierarchy, l, d):
    """Faces of level l that border a cell of its region (natural face layout)."""
    m = H.inm[l]
    n = H.shape[l][d]
    lo_idx = np.arange(-1, n)
    hi_idx = np.arange(0, n + 1)
    per = H.bc_lo[d] == BC_PER
    pad = np.zeros_like(np.take(m, [0], axis=d))
    lo = np.take(m, lo_idx % n, axis=d)
    hi = np.take(m, hi_idx % n, axis=d)
    if not per:
        sl0 = [slice(None)] * H.dm
        sl0[d] = slice(0, 1)
        lo[tuple(sl0)] = pad
        sl1 = [slice(None)] * H.dm
        sl1[d] = slice(n, n + 1)
        hi[tuple(sl1)] = pad
    return lo | hi


def edge_restrict(H: Hierarchy, uc, uf, l):
    """ml_edge_restriction of level l onto level l-1 (in place on uc)."""
    for d in range(H.dm):
        mem = face_member(H, l, d)
        sl = [slice(None)] * H.dm
        sl[d] = slice(None, None, 2)
        f = uf[d][tuple(sl)]
        mm = mem[tuple(sl)]
        acc = 0.0
        cnt = 0
        msk = None
        for bits in itertools.product((0, 1), repeat=H.dm - 1):
            s2 = [slice(None)] * H.dm
            for e, b in zip([e for e in range(H.dm) if e != d], bits):
                s2[e] = slice(b, None, 2)
            acc = acc + f[tuple(s2)]
            cnt += 1
            msk = mm[tuple(s2)] if msk is None else msk
        uc[d][msk] = (acc / cnt)[msk]


def beta0_face(case, l, d, shape):
    dm = case.dm
    shp = [1] * dm
    if d == dm - 1:
        shp[dm - 1] = shape[dm - 1] + 1
        return case.beta0_edge[l].reshape(shp)
    shp[dm - 1] = shape[dm - 1]
    return case.beta0[l].reshape(shp)


def reference_projection_amr(case, p=1):
    H = Hierarchy(case.n0, case.dx0, case.bc_lo, case.bc_hi, case.boxes)
    dm = case.dm
    L = H.L
    u = [[np.array(x, dtype=np.float64, order="F") for x in case.umac[l]] for l in range(L)]
    for l in range(L):
        for d in range(dm):
            u[l][d] *= beta0_face(case, l, d, H.shape[l])
    for l in range(L - 1, 0, -1):
        edge_restrict(H, u[l - 1], u[l], l)
    rh = []
    for l in range(L):
        dv = np.zeros(H.shape[l])
        for d in range(dm):
            dv += np.diff(u[l][d], axis=d) / H.h[l][d]
        r = -(dv - case.macrhs[l])
        rh.append(np.where(H.inm[l], r, 0.0))
    for l in range(L - 1, 0, -1):
        rh[l - 1] = np.where(H.cov[l - 1], average_down(rh[l]), rh[l - 1])
    beta = [face_coeffs(case.rho[l], case.beta0[l], case.beta0_edge[l], case.bc_lo, case.bc_hi, p)
            for l in range(L)]
    phi = composite_solve(H, beta, rh)
    # mkumac
    for l in range(L):
        for d in range(dm):
            mem = face_member(H, l, d)
            n = H.shape[l][d]
            for f in np.argwhere(mem):
                f = [int(v) for v in f]
                lo = list(f)
                hi = list(f)
                lo[d] = H.wrap(l, d, f[d] - 1)
                hi[d] = H.wrap(l, d, f[d]) if f[d] < n else H.wrap(l, d, f[d])
                lin = lo[d] is not None and H.inm[l][tuple(lo)]
                hin = hi[d] is not None and H.inm[l][tuple(hi)]
                hh = H.h[l][d]
                if lin and hin:
                    g = (phi[l][tuple(hi)] - phi[l][tuple(lo)]) / hh
                elif hin and lo[d] is None:
                    g = 2.0 * phi[l][tuple(hi)] / hh if case.bc_lo[d] == BC_DIR else 0.0
                elif lin and hi[d] is None:
                    g = -2.0 * phi[l][tuple(lo)] / hh if case.bc_hi[d] == BC_DIR else 0.0
                else:
                    own, gh = (hi, lo) if hin else (lo, hi)
                    pv = phi[l][tuple(own)]
                    pc = sum(wk * phi[l - 1][K] for K, wk in H.coarse_weights(l, gh, d).items())
                    gv = pv / 3.0 + 2.0 / 3.0 * pc
                    g = (pv - gv) / hh if hin else (gv - pv) / hh
                u[l][d][tuple(f)] -= beta[l][d][tuple(f)] * g
    for l in range(L - 1, 0, -1):
        edge_restrict(H, u[l - 1], u[l], l)
    for l in range(L):
        for d in range(dm):
            u[l][d] /= beta0_face(case, l, d, H.shape[l])
    for l in range(L - 1, 0, -1):
        edge_restrict(H, u[l - 1], u[l], l)
    return u, phi, rh, beta, H


def main():
    for name in AMR_CASES:
        case = amr_case(name)
        u, phi, rh, beta, H = reference_projection_amr(case)
        out = {"n0": np.array(case.n0), "dx0": np.array(case.dx0), "bc_lo": np.array(case.bc_lo),
               "bc_hi": np.array(case.bc_hi), "nlev": np.array(H.L), "seed": np.array(case.seed)}
        for l in range(H.L):
            # only what a level's region uses is stored (zeros elsewhere compress away): its
            # cells, its faces, and for rho one ghost cell around it
            grown = H.inm[l].copy()
            for d in range(case.dm):
                grown |= np.roll(H.inm[l], 1, axis=d) | np.roll(H.inm[l], -1, axis=d)
            out[f"boxes{l}"] = np.array([list(lo) + list(hi) for lo, hi in case.boxes[l]],
                                        dtype=np.int64).reshape(-1, 2 * case.dm)
            out[f"rho{l}"] = np.where(grown, case.rho[l], 0.0)
            out[f"macrhs{l}"] = np.where(H.inm[l], case.macrhs[l], 0.0)
            out[f"beta0_{l}"] = case.beta0[l]
            out[f"beta0e_{l}"] = case.beta0_edge[l]
            out[f"phi{l}"] = phi[l]
            for d in range(case.dm):
                m = face_member(H, l, d)
                out[f"u{l}_{d}"] = np.where(m, case.umac[l][d], 0.0)
                out[f"unew{l}_{d}"] = np.where(m, u[l][d], 0.0)
        path = os.path.join(HERE, f"{name}.npz")
        np.savez_compressed(path, **out)
        print(path, H.nunk, "unknowns")


if __name__ == "__main__":
    main()
