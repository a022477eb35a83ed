// Finest-level FP32 kernels of the mixed-precision solve with the face coefficients computed on
// the fly from an FP32 copy of the density, instead of reading stored coefficient arrays:
//   beta'_f = fac_d[layer] / (rho_a + rho_b),   fac_d = beta0_f^p * 2 / h_d^2
// (the coefficient of Source/macproject.f90:698-738 times beta0 of :184-203, divided by h^2).
// A red/black half-sweep then reads the other colour's e and rho, its own r and rho and writes
// its own e: 10 bytes per cell of the level instead of 20 with stored FP32 coefficients.  Only the
// inner (FP32) V-cycle uses these; the FP64 refinement residual keeps the stored FP64 operator.
#include "mac_internal.cuh"

namespace mac {
namespace {

constexpr int kB = 256;

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

template <int DM>
__global__ void __launch_bounds__(kB)
k_gsrb_otf(Dims d, OtfParams P, int colour, float* __restrict__ es, const float* __restrict__ eo,
           const float* __restrict__ rs, const float* __restrict__ rhos,
           const float* __restrict__ rhoo) {
    const int h = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z;
    if (h >= d.hn0 || j >= d.n1) return;
    const int q = (j + d.n1 * k) * d.hn0 + h;
    const int i = 2 * h + ((colour + j + k) & 1);
    Nb nb;
    nbrs(d, colour, h, j, k, nb);
    float acc = rs[q], diag;
    otf_cell<DM>(P, nb, i, j, k, rhos[q], rhoo, eo, acc, diag);
    es[q] = acc * rcp_approx(diag);
}

template <int DM, bool RED_ONLY>
__global__ void __launch_bounds__(kB)
k_resid_restrict_otf(Dims F, Dims C, OtfParams P, const float* __restrict__ e,
                     const float* __restrict__ r, float* __restrict__ fc) {
    const int I = blockIdx.x * blockDim.x + threadIdx.x;
    const int J = blockIdx.y * blockDim.y + threadIdx.y;
    const int K = blockIdx.z;
    if (I >= C.n0 || J >= C.n1) return;
    const int rz = DM == 3 ? 2 : 1;
    float sum = 0.f;
#pragma unroll
    for (int b = 0; b < rz; ++b) {
#pragma unroll
        for (int a = 0; a < 2; ++a) {
            const int j = 2 * J + a;
            const int k = DM == 3 ? 2 * K + b : K;
#pragma unroll
            for (int colour = 0; colour < (RED_ONLY ? 1 : 2); ++colour) {
                const int off = colour * F.half, oth = (colour ^ 1) * F.half;
                const int i = 2 * I + ((colour + j + k) & 1);
                Nb nb;
                nbrs(F, colour, I, j, k, nb);
                const int me = (j + F.n1 * k) * F.hn0 + I;
                float acc = r[off + me], diag;
                otf_cell<DM>(P, nb, i, j, k, P.rho[off + me], P.rho + oth, e + oth, acc, diag);
                sum += fmaf(-diag, e[off + me], acc);
            }
        }
    }
    int ci;
    if (C.split)
        ci = ((I + J + K) & 1) * C.half + (J + C.n1 * K) * C.hn0 + (I >> 1);
    else
        ci = I + C.n0 * (J + C.n1 * K);
    fc[ci] = sum * (DM == 3 ? 0.125f : 0.25f);
}

}  // namespace

void launch_gsrb_otf(const Dims& d, const OtfParams& P, int colour, float* e, const float* r,
                     cudaStream_t s) {
    const int own = colour * d.half, oth = (colour ^ 1) * d.half;
    const Grid3 g = grid3(d.hn0, d.n1, d.n2);
    if (P.dm == 3)
        k_gsrb_otf<3><<<g.grid, g.block, 0, s>>>(d, P, colour, e + own, e + oth, r + own,
                                                 P.rho + own, P.rho + oth);
    else
        k_gsrb_otf<2><<<g.grid, g.block, 0, s>>>(d, P, colour, e + own, e + oth, r + own,
                                                 P.rho + own, P.rho + oth);
}

void launch_resid_restrict_otf(const Dims& fine, const Dims& coarse, const OtfParams& P,
                               const float* e, const float* r, float* fc, bool red_only,
                               cudaStream_t s) {
    const Grid3 g = grid3(coarse.n0, coarse.n1, coarse.n2);
    if (P.dm == 3) {
        if (red_only)
            k_resid_restrict_otf<3, true><<<g.grid, g.block, 0, s>>>(fine, coarse, P, e, r, fc);
        else
            k_resid_restrict_otf<3, false><<<g.grid, g.block, 0, s>>>(fine, coarse, P, e, r, fc);
    } else {
        if (red_only)
            k_resid_restrict_otf<2, true><<<g.grid, g.block, 0, s>>>(fine, coarse, P, e, r, fc);
        else
            k_resid_restrict_otf<2, false><<<g.grid, g.block, 0, s>>>(fine, coarse, P, e, r, fc);
    }
}

}  // namespace mac
