// Per-cell pieces of the finest-level FP32 operator with face coefficients computed on the fly
// from rho32 (shared by the half-sweeps and defect kernels of mac_otf.cu and the Krylov kernels
// of mac_krylov.cu):  beta'_f = fac_d[layer] / (rho_a + rho_b).
#pragma once
#include "mac_internal.cuh"

namespace mac {
namespace {

// Single-precision reciprocal estimate (relative error <= 2^-23; the inner V-cycle only needs
// an FP32-accurate operator).
__device__ __forceinline__ float rcp_approx(float s) {
    float y;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(s));
    return y;
}

struct Nb {
    int xm, xp, ym, yp, zm, zp;
};

__device__ __forceinline__ void nbrs(const Dims& d, int colour, int h, int j, int k, Nb& nb) {
    const int s = (colour + j + k) & 1;
    int hm = h - 1 + s;
    hm += (hm < 0) ? d.hn0 : 0;
    int hp = h + s;
    hp -= (hp >= d.hn0) ? d.hn0 : 0;
    const int jm = (j == 0) ? d.n1 - 1 : j - 1;
    const int jp = (j == d.n1 - 1) ? 0 : j + 1;
    const int km = (k == 0) ? d.n2 - 1 : k - 1;
    const int kp = (k == d.n2 - 1) ? 0 : k + 1;
    const int row = (j + d.n1 * k) * d.hn0;
    nb.xm = row + hm;
    nb.xp = row + hp;
    nb.ym = (jm + d.n1 * k) * d.hn0 + h;
    nb.yp = (jp + d.n1 * k) * d.hn0 + h;
    nb.zm = (j + d.n1 * km) * d.hn0 + h;
    nb.zp = (j + d.n1 * kp) * d.hn0 + h;
}

// Adds sum_arms beta'_f e_n to acc and returns the diagonal of cell (i, j, k) (colour half
// index via nb; ro/eo = the other colour's rho and e, rc = own rho).  Branch-free: a face on a
// non-periodic wall gets a zero factor (horizontal walls by position, vertical walls through the
// wall-zeroed layer tables), and its wrapped neighbour index stays a valid address.
template <int DM>
__device__ __forceinline__ void otf_cell(const OtfParams& P, const Nb& nb, int i, int j, int k,
                                         float rc, const float* __restrict__ ro,
                                         const float* __restrict__ eo, float& acc, float& diag) {
    const int r = DM == 3 ? k : j;
    const int st = P.n[DM - 1] + 1;   // the vertical direction is the last one
    const float fx = P.fac[r];
    const float fxl = (i > 0 || P.per[0]) ? fx : 0.f;
    const float fxh = (i < P.n[0] - 1 || P.per[0]) ? fx : 0.f;
    float fyl, fyh, fzl = 0.f, fzh = 0.f;
    if (DM == 3) {
        const float fy = P.fac[st + r];
        fyl = (j > 0 || P.per[1]) ? fy : 0.f;
        fyh = (j < P.n[1] - 1 || P.per[1]) ? fy : 0.f;
        fzl = P.fac[2 * st + r];
        fzh = P.fac[3 * st + r];
    } else {
        fyl = P.fac[2 * st + r];
        fyh = P.fac[3 * st + r];
    }
    float b = fxl * rcp_approx(rc + ro[nb.xm]);
    acc = fmaf(b, eo[nb.xm], acc);
    float dg = b;
    b = fxh * rcp_approx(rc + ro[nb.xp]);
    acc = fmaf(b, eo[nb.xp], acc);
    dg += b;
    b = fyl * rcp_approx(rc + ro[nb.ym]);
    acc = fmaf(b, eo[nb.ym], acc);
    dg += b;
    b = fyh * rcp_approx(rc + ro[nb.yp]);
    acc = fmaf(b, eo[nb.yp], acc);
    dg += b;
    if (DM == 3) {
        b = fzl * rcp_approx(rc + ro[nb.zm]);
        acc = fmaf(b, eo[nb.zm], acc);
        dg += b;
        b = fzh * rcp_approx(rc + ro[nb.zp]);
        acc = fmaf(b, eo[nb.zp], acc);
        dg += b;
    }
    if (P.has_dir) {   // Dirichlet walls add fac / rho to the diagonal
        float w = P.fac[4 * st + r];
        if (DM == 3) {
            w += (i == 0 && P.dlo[0]) || (i == P.n[0] - 1 && P.dhi[0]) ? fx : 0.f;
            w += (j == 0 && P.dlo[1]) || (j == P.n[1] - 1 && P.dhi[1]) ? P.fac[st + r] : 0.f;
        } else {
            w += (i == 0 && P.dlo[0]) || (i == P.n[0] - 1 && P.dhi[0]) ? fx : 0.f;
        }
        dg += w * rcp_approx(rc);
    }
    diag = dg;
}

}  // namespace
}  // namespace mac
