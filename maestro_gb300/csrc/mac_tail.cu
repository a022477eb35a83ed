// Single-CTA "tail" of the V-cycle: every level from the first one small enough to live in
// shared memory down to the bottom solve runs inside one kernel, so the smallest levels no
// longer pay one kernel launch per half-sweep.  The arithmetic is the multi-kernel V-cycle's,
// operation for operation (same fused-multiply-add order per cell, same child order in the
// restriction, same separable trilinear prolongation, the same single-warp bottom solve), so the
// result is bitwise the same; only the data lives in shared memory in natural layout.
#include "mac_internal.cuh"
#include "mac_bottom.cuh"

namespace mac {
namespace {

constexpr int kTailThreads = 1024;

__device__ __forceinline__ double fmaT2(double a, double b, double c) { return fma(a, b, c); }
__device__ __forceinline__ float fmaT2(float a, float b, float c) { return fmaf(a, b, c); }

template <typename T>
struct TailLevel {
    int n0, n1, n2, N, rz;
    T *e, *f, *bx, *by, *bz, *dg, *idg;   // shared memory, natural layout
};

template <typename T>
__device__ __forceinline__ T arms_nat(T acc, const TailLevel<T>& L, const T* __restrict__ u, int i,
                                      int j, int k, int c) {
    const int im = i == 0 ? L.n0 - 1 : i - 1, ip = i == L.n0 - 1 ? 0 : i + 1;
    const int jm = j == 0 ? L.n1 - 1 : j - 1, jp = j == L.n1 - 1 ? 0 : j + 1;
    const int km = k == 0 ? L.n2 - 1 : k - 1, kp = k == L.n2 - 1 ? 0 : k + 1;
    const int cxm = im + L.n0 * (j + L.n1 * k), cxp = ip + L.n0 * (j + L.n1 * k);
    const int cym = i + L.n0 * (jm + L.n1 * k), cyp = i + L.n0 * (jp + L.n1 * k);
    const int czm = i + L.n0 * (j + L.n1 * km), czp = i + L.n0 * (j + L.n1 * kp);
    acc = fmaT2(L.bx[c], u[cxm], acc);
    acc = fmaT2(L.bx[cxp], u[cxp], acc);
    acc = fmaT2(L.by[c], u[cym], acc);
    acc = fmaT2(L.by[cyp], u[cyp], acc);
    acc = fmaT2(L.bz[c], u[czm], acc);
    acc = fmaT2(L.bz[czp], u[czp], acc);
    return acc;
}

// Thread layout over an (nx, rows) index space: tx strides x, ty strides the rows (row =
// j + n1 k, decoded incrementally), so no per-cell integer division.
struct Lanes {
    int tx, ty, TX, RY;
};
__device__ __forceinline__ Lanes lanes(int nx) {
    Lanes q;
    q.TX = nx < 32 ? nx : 32;
    q.tx = threadIdx.x % q.TX;
    q.ty = threadIdx.x / q.TX;
    q.RY = blockDim.x / q.TX;
    return q;
}

template <typename T>
__device__ __noinline__ void tail_sweep(const TailLevel<T>& L, T omega) {
    const int hn0 = L.n0 >> 1, rows = L.n1 * L.n2;
    const Lanes q = lanes(hn0);
    for (int colour = 0; colour < 2; ++colour) {
        if (q.ty < q.RY) {
            int j = q.ty % L.n1, k = q.ty / L.n1;
            const int dj = q.RY % L.n1, dk = q.RY / L.n1;
            for (int row = q.ty; row < rows; row += q.RY) {
                const int s = (colour + j + k) & 1;
                for (int h = q.tx; h < hn0; h += q.TX) {
                    const int i = 2 * h + s;
                    const int c = i + L.n0 * row;
                    const T acc = arms_nat<T>(L.f[c], L, L.e, i, j, k, c);
                    if (omega != T(1))
                        L.e[c] = fmaT2(omega, acc * L.idg[c] - L.e[c], L.e[c]);
                    else
                        L.e[c] = acc * L.idg[c];
                }
                j += dj;
                k += dk;
                if (j >= L.n1) {
                    j -= L.n1;
                    ++k;
                }
            }
        }
        __syncthreads();
    }
}

// defect of level F restricted into out[coarse natural index] (as T, then converted to To)
template <typename T, typename To>
__device__ __noinline__ void tail_restrict(const TailLevel<T>& F, int cn0, int cn1, int cn2, To* out,
                              bool red_only) {
    const Lanes ln = lanes(cn0);
    const int rows = cn1 * cn2;
    for (int crow = ln.ty; ln.ty < ln.RY && crow < rows; crow += ln.RY)
    for (int I = ln.tx; I < cn0; I += ln.TX) {
        const int J = crow % cn1, K = crow / cn1;
        const int q = I + cn0 * crow;
        T sum = T(0);
        for (int b = 0; b < F.rz; ++b) {
            for (int a = 0; a < 2; ++a) {
                const int j = 2 * J + a;
                const int k = F.rz == 2 ? 2 * K + b : K;
                for (int colour = 0; colour < (red_only ? 1 : 2); ++colour) {
                    const int i = 2 * I + ((colour + j + k) & 1);
                    const int c = i + F.n0 * (j + F.n1 * k);
                    T r = fmaT2(-F.dg[c], F.e[c], F.f[c]);
                    r = arms_nat<T>(r, F, F.e, i, j, k, c);
                    sum += r;
                }
            }
        }
        out[q] = (To)(sum * (T)(1.0 / (4 * F.rz)));
    }
    __syncthreads();
}

template <typename T>
__device__ __forceinline__ void nb_w(int q, int n, int blo, int bhi, int& qm, int& qp, T& wm, T& wp) {
    wm = T(0.25);
    wp = T(0.25);
    if (q > 0) qm = q - 1;
    else if (blo == MAC_BC_PER) qm = n - 1;
    else {
        qm = 0;
        if (blo == MAC_BC_DIR) wm = T(-0.25);
    }
    if (q < n - 1) qp = q + 1;
    else if (bhi == MAC_BC_PER) qp = 0;
    else {
        qp = n - 1;
        if (bhi == MAC_BC_DIR) wp = T(-0.25);
    }
}

// e_fine += trilinear interpolation of the coarse correction ec (natural, cn0 x cn1 x cn2)
// black_only: colour-1 children only (post-smoothing follows; see k_prolong_add)
template <typename T>
__device__ __noinline__ void tail_prolong(const TailLevel<T>& F, const T* ec, int cn0, int cn1, int cn2,
                             const BcDesc& bc, bool black_only) {
    const bool z2 = F.rz == 2;
    const Lanes ln = lanes(cn0);
    const int rows = cn1 * cn2;
    for (int crow = ln.ty; ln.ty < ln.RY && crow < rows; crow += ln.RY)
    for (int I = ln.tx; I < cn0; I += ln.TX) {
        const int J = crow % cn1, K = crow / cn1;
        int xs[3], ys[3], zs[3];
        T wxm, wxp, wym, wyp, wzm = T(0), wzp = T(0);
        xs[1] = I;
        ys[1] = J;
        zs[1] = K;
        nb_w<T>(I, cn0, bc.lo[0], bc.hi[0], xs[0], xs[2], wxm, wxp);
        nb_w<T>(J, cn1, bc.lo[1], bc.hi[1], ys[0], ys[2], wym, wyp);
        if (z2) nb_w<T>(K, cn2, bc.lo[2], bc.hi[2], zs[0], zs[2], wzm, wzp);
        T Yv[3][2][2];
        for (int a = 0; a < 3; ++a) {
            const int X = xs[a];
            T Zv[3][2];
            for (int b = 0; b < 3; ++b) {
                const int Y = ys[b];
                const T c0 = ec[X + cn0 * (Y + cn1 * K)];
                if (z2) {
                    const T t = T(0.75) * c0;
                    Zv[b][0] = fmaT2(wzm, ec[X + cn0 * (Y + cn1 * zs[0])], t);
                    Zv[b][1] = fmaT2(wzp, ec[X + cn0 * (Y + cn1 * zs[2])], t);
                } else {
                    Zv[b][0] = c0;
                    Zv[b][1] = c0;
                }
            }
            for (int zc = 0; zc < 2; ++zc) {
                const T t = T(0.75) * Zv[1][zc];
                Yv[a][0][zc] = fmaT2(wym, Zv[0][zc], t);
                Yv[a][1][zc] = fmaT2(wyp, Zv[2][zc], t);
            }
        }
        for (int zc = 0; zc < (z2 ? 2 : 1); ++zc) {
            for (int yc = 0; yc < 2; ++yc) {
                const T t = T(0.75) * Yv[1][yc][zc];
                const int j = 2 * J + yc;
                const int k = z2 ? 2 * K + zc : K;
                const int base = F.n0 * (j + F.n1 * k) + 2 * I;
                const int c0 = (yc + zc) & 1;   // colour of child 2I
                if (!black_only || c0) F.e[base] += fmaT2(wxm, Yv[0][yc][zc], t);
                if (!black_only || !c0) F.e[base + 1] += fmaT2(wxp, Yv[2][yc][zc], t);
            }
        }
    }
    __syncthreads();
}

// Asynchronous 4/8-byte global -> shared copy (cp.async); completed by cp_async_wait().
template <typename T>
__device__ __forceinline__ void cp_async(T* dst, const T* src) {
    static_assert(sizeof(T) == 4 || sizeof(T) == 8, "4 or 8 bytes");
    asm volatile("cp.async.ca.shared.global [%0], [%1], %2;" ::"r"(
                     (unsigned)__cvta_generic_to_shared(dst)),
                 "l"(src), "n"(sizeof(T))
                 : "memory");
}
__device__ __forceinline__ void cp_async_wait() {
    asm volatile("cp.async.commit_group;\ncp.async.wait_all;" ::: "memory");
}

// Visit every cell of a checkerboard-split level once: fn(g, c) with g the split-layout
// (global) index and c the natural (shared-memory) index; rows decoded incrementally, no
// per-cell integer division.
template <class Fn>
__device__ __forceinline__ void for_split_cells(const Dims& D, Fn fn) {
    const Lanes q = lanes(D.hn0);
    if (q.ty >= q.RY) return;
    const int rows = D.n1 * D.n2;
    int j = q.ty % D.n1, k = q.ty / D.n1;
    const int dj = q.RY % D.n1, dk = q.RY / D.n1;
    for (int row = q.ty; row < rows; row += q.RY) {
        for (int colour = 0; colour < 2; ++colour) {
            const int s = (colour + j + k) & 1;
            for (int h = q.tx; h < D.hn0; h += q.TX)
                fn(colour * D.half + row * D.hn0 + h, 2 * h + s + D.n0 * row);
        }
        j += dj;
        k += dk;
        if (j >= D.n1) {
            j -= D.n1;
            ++k;
        }
    }
}

}  // namespace

template <typename T>
__global__ void __launch_bounds__(kTailThreads)
k_tail(TailParams<T> P) {
    extern __shared__ __align__(16) unsigned char tail_smem[];
    const int tid = threadIdx.x, nt = blockDim.x;
    const int nl = P.nlev;   // non-bottom tail levels
    TailLevel<T> L[kTailMaxLevels];
    // carve shared memory: per non-bottom level 7 arrays of T, then the bottom's operator (5 N),
    // x, f and scratch (kBotScrPerCell N) doubles
    size_t off = 0;
    for (int l = 0; l < nl; ++l) {
        const int N = P.lev[l].ncell;
        T* base = reinterpret_cast<T*>(tail_smem + off);
        L[l].n0 = P.lev[l].n0;
        L[l].n1 = P.lev[l].n1;
        L[l].n2 = P.lev[l].n2;
        L[l].N = N;
        L[l].rz = P.lev[l].rz;
        L[l].e = base;
        L[l].f = base + N;
        L[l].bx = base + 2 * N;
        L[l].by = base + 3 * N;
        L[l].bz = base + 4 * N;
        L[l].dg = base + 5 * N;
        L[l].idg = base + 6 * N;
        off += ((size_t)7 * N * sizeof(T) + 15) & ~(size_t)15;
    }
    double* bsm = reinterpret_cast<double*>(tail_smem + off);
    const Dims BD = P.bottom;
    const int NB = BD.ncell;
    // load the operators (split layout in global memory -> natural in shared memory).  They are
    // built before the solve starts (and the host waits for that), so their copies are issued
    // before the wait on the preceding kernel and overlap its last part; only the restricted
    // defect f0 comes from that kernel.
    for (int l = 0; l < nl; ++l) {
        const TailLevel<T>& Ll = L[l];
        const T *gbx = P.bx[l], *gby = P.by[l], *gbz = P.bz[l], *gdg = P.dg[l], *gidg = P.idg[l];
        for_split_cells(P.lev[l], [&](int g, int c) {
            cp_async(Ll.bx + c, gbx + g);
            cp_async(Ll.by + c, gby + g);
            cp_async(Ll.bz + c, gbz + g);
            cp_async(Ll.dg + c, gdg + g);
            cp_async(Ll.idg + c, gidg + g);
            Ll.e[c] = T(0);
        });
    }
    BotView v;
    v.n0 = BD.n0;
    v.n1 = BD.n1;
    v.n2 = BD.n2;
    v.N = NB;
    double* ops = bsm;
    for (int c = tid; c < NB; c += nt) {
        cp_async(ops + c, P.bbx + c);
        cp_async(ops + NB + c, P.bby + c);
        cp_async(ops + 2 * NB + c, P.bbz + c);
        cp_async(ops + 3 * NB + c, P.bdg + c);
        cp_async(ops + 4 * NB + c, P.bidg + c);
    }
    pdl_wait();
    pdl_trigger();
    {
        const T* gf = P.f0;
        T* sf = L[0].f;
        for_split_cells(P.lev[0], [&](int g, int c) { cp_async(sf + c, gf + g); });
    }
    cp_async_wait();
    v.bx = ops;
    v.by = ops + NB;
    v.bz = ops + 2 * NB;
    v.dg = ops + 3 * NB;
    v.idg = ops + 4 * NB;
    double* xb = bsm + 5 * NB;
    double* fb = bsm + 6 * NB;
    double* wb = bsm + 7 * NB;
    __syncthreads();
    // down the V
    for (int l = 0; l < nl; ++l) {
        for (int s = 0; s < P.nu1; ++s) tail_sweep<T>(L[l], P.omega);
        // red-only defect / black-only prolongation rest on plain Gauss-Seidel half-sweeps
        const bool gs = P.omega == T(1);
        if (l + 1 < nl) {
            tail_restrict<T, T>(L[l], L[l + 1].n0, L[l + 1].n1, L[l + 1].n2, L[l + 1].f,
                                gs && P.nu1 > 0);
        } else {
            tail_restrict<T, double>(L[l], BD.n0, BD.n1, BD.n2, fb, gs && P.nu1 > 0);
        }
    }
    // bottom, FP64 (input rhs rounded through T as in the multi-kernel path)
    int count = 0;
    __shared__ double sm_red[33];
    if (P.binv) {
        // exact solve by the precomputed (pseudo-)inverse: x = B^-1 (f - mean f) (the mean comes
        // off for a singular operator, whose constant mode B^-1 only scales)
        if (P.singular) {
            if (tid < 32) {
                double s = 0.0;
                for (int c = tid; c < NB; c += 32) s += fb[c];
                for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
                if (tid == 0) sm_red[32] = s / NB;
            }
            __syncthreads();
            const double mean = sm_red[32];
            for (int c = tid; c < NB; c += nt) fb[c] -= mean;
            __syncthreads();
        }
        // row r of B^-1 by kDenseSeg lanes of one warp (NB <= kDenseBottomMax: one pass)
        const int r = tid / kDenseSeg, sg = tid % kDenseSeg;
        double acc = 0.0;
        if (r < NB)
            for (int c = sg; c < NB; c += kDenseSeg) acc = fma(__ldg(P.binv + (size_t)r * NB + c), fb[c], acc);
        for (int o = kDenseSeg / 2; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
        if (r < NB && sg == 0) xb[r] = acc;
    } else {
        for (int c = tid; c < NB; c += nt) xb[c] = 0.0;
        __syncthreads();
        if (tid < 128)
            count = bottom_body<Sync128<true>>(v, xb, fb, wb, sm_red, P.singular, P.nub,
                                               P.bottom_eps, P.bottom_max_iter);
    }
    __syncthreads();
    // the bottom solution is handed up as T, like the multi-kernel path's bottom output
    T* eb = reinterpret_cast<T*>(wb);
    for (int c = tid; c < NB; c += nt) eb[c] = (T)xb[c];
    __syncthreads();
    // up the V
    for (int l = nl - 1; l >= 0; --l) {
        const bool gs = P.omega == T(1);
        if (l + 1 < nl)
            tail_prolong<T>(L[l], L[l + 1].e, L[l + 1].n0, L[l + 1].n1, L[l + 1].n2, P.bc,
                            gs && P.nu2 > 0);
        else
            tail_prolong<T>(L[l], eb, BD.n0, BD.n1, BD.n2, P.bc, gs && P.nu2 > 0);
        for (int s = 0; s < P.nu2; ++s) tail_sweep<T>(L[l], P.omega);
    }
    // hand the correction of the first tail level back (its split layout)
    {
        const T* e = L[0].e;
        T* ge = P.e0;
        for_split_cells(P.lev[0], [&](int g, int c) { ge[g] = e[c]; });
    }
    if (tid == 0 && P.iters) atomicAdd(P.iters, count);
}

// (Pseudo-)inverse of the bottom operator for the exact bottom solve of the FP32 V-cycle: the
// dense N x N matrix of A x = diag x - sum_n a_n x_n (N <= kDenseBottomMax, natural layout; a
// periodic arm that wraps onto the same neighbour twice adds up), plus sigma 1 1^T with sigma =
// mean(diag) / N when A is singular (constant null space: B^-1 f = A^+ f for f of zero mean).
// B is symmetric positive definite, so it is inverted by the symmetric sweep operator (Gauss-
// Jordan elimination without pivoting that keeps the matrix symmetric; after sweeping every
// pivot the matrix holds -B^-1), updating only the upper triangle: N (N + 1) / 2 FMAs a pivot,
// each thread owning fixed elements of the packed triangle so that warps stay full (GB300 issues
// FP64 instructions per warp, whatever the number of active lanes).  FP64, shared memory, one
// CTA, once per solve (on a side stream, overlapping the right-hand-side setup).
constexpr int kInvPerThread = (kDenseBottomMax * (kDenseBottomMax + 1) / 2 + kTailThreads - 1) / kTailThreads;

__global__ void __launch_bounds__(kTailThreads)
k_bottom_inverse(Dims D, const double* __restrict__ bx, const double* __restrict__ by,
                 const double* __restrict__ bz, const double* __restrict__ dg, int singular,
                 double* __restrict__ out) {
    __shared__ double M[kDenseBottomMax * kDenseBottomMax];
    __shared__ double row[kDenseBottomMax], sk[kDenseBottomMax];
    __shared__ double sdiag, sip;
    const int N = D.ncell, tid = threadIdx.x, nt = blockDim.x;
    if (tid < 32) {
        double s = 0.0;
        for (int c = tid; c < N; c += 32) s += dg[c];
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if (tid == 0) sdiag = singular ? s / ((double)N * N) : 0.0;
    }
    __syncthreads();
    for (int q = tid; q < N * N; q += nt) M[q] = sdiag;
    __syncthreads();
    // row c by thread c (its six arms load in parallel with the other rows')
    if (tid < N) {
        const int c = tid;
        const int i = c % D.n0, rw = c / D.n0, j = rw % D.n1, k = rw / D.n1;
        const int im = i == 0 ? D.n0 - 1 : i - 1, ip = i == D.n0 - 1 ? 0 : i + 1;
        const int jm = j == 0 ? D.n1 - 1 : j - 1, jp = j == D.n1 - 1 ? 0 : j + 1;
        const int km = k == 0 ? D.n2 - 1 : k - 1, kp = k == D.n2 - 1 ? 0 : k + 1;
        const int nbr[6] = {im + D.n0 * (j + D.n1 * k), ip + D.n0 * (j + D.n1 * k),
                            i + D.n0 * (jm + D.n1 * k), i + D.n0 * (jp + D.n1 * k),
                            i + D.n0 * (j + D.n1 * km), i + D.n0 * (j + D.n1 * kp)};
        const double a[6] = {bx[c], bx[nbr[1]], by[c], by[nbr[3]], bz[c], bz[nbr[5]]};
        M[c * N + c] += dg[c];
        for (int n = 0; n < 6; ++n) M[c * N + nbr[n]] -= a[n];
    }
    // the upper-triangle elements (i <= j) this thread updates: packed indices tid + m nt
    int ei[kInvPerThread], ej[kInvPerThread];
    const int npk = N * (N + 1) / 2;
#pragma unroll
    for (int m = 0; m < kInvPerThread; ++m) {
        int p = tid + m * nt, i = 0;
        ei[m] = -1;
        ej[m] = 0;
        if (p < npk) {
            while (p >= N - i) {
                p -= N - i;
                ++i;
            }
            ei[m] = i;
            ej[m] = i + p;
        }
    }
    __syncthreads();
    for (int k = 0; k < N; ++k) {
        // row k of the symmetric matrix (upper-triangle storage) and the pivot's reciprocal
        if (tid < N) row[tid] = tid < k ? M[tid * N + k] : M[k * N + tid];
        if (tid == 0) sip = recip_nr(M[k * N + k]);
        __syncthreads();
        if (tid < N) sk[tid] = row[tid] * sip;
        __syncthreads();
#pragma unroll
        for (int m = 0; m < kInvPerThread; ++m) {
            const int i = ei[m], j = ej[m];
            if (i < 0) continue;
            double& v = M[i * N + j];
            if (i == k)
                v = j == k ? -sip : sk[j];
            else if (j == k)
                v = sk[i];
            else
                v = fma(-row[i], sk[j], v);
        }
        __syncthreads();
    }
    for (int q = tid; q < N * N; q += nt) {
        const int i = q / N, j = q - i * N;
        out[q] = -(i <= j ? M[i * N + j] : M[j * N + i]);
    }
}

void launch_bottom_inverse(const Dims& d, const double* bx, const double* by, const double* bz,
                           const double* dg, bool singular, double* out, cudaStream_t s) {
    k_bottom_inverse<<<1, kTailThreads, 0, s>>>(d, bx, by, bz, dg, singular ? 1 : 0, out);
}

template <typename T>
size_t tail_smem_bytes(const Dims* lev, int nl, const Dims& bottom) {
    size_t off = 0;
    for (int l = 0; l < nl; ++l) off += ((size_t)7 * lev[l].ncell * sizeof(T) + 15) & ~(size_t)15;
    return off + (size_t)(7 + kBotScrPerCell) * bottom.ncell * sizeof(double);
}

template <typename T>
void launch_tail(const TailParams<T>& P, size_t smem, cudaStream_t s) {
    launch_chain(k_tail<T>, dim3(1), dim3(kTailThreads), smem, s, P);
}

int prepare_tail_kernels() {
    if (cudaFuncSetAttribute(k_tail<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, kTailSmemMax) != cudaSuccess ||
        cudaFuncSetAttribute(k_tail<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, kTailSmemMax) != cudaSuccess) {
        cudaGetLastError();
        return MAC_ERR_CUDA;
    }
    return MAC_OK;
}

template size_t tail_smem_bytes<float>(const Dims*, int, const Dims&);
template size_t tail_smem_bytes<double>(const Dims*, int, const Dims&);
template void launch_tail<float>(const TailParams<float>&, size_t, cudaStream_t);
template void launch_tail<double>(const TailParams<double>&, size_t, cudaStream_t);

}  // namespace mac
