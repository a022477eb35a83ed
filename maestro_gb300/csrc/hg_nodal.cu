// Nodal (HG) projection on the GPU: the node / cell functions of hg_nodal.cuh as kernels, the
// executor of hg::project on device arrays, and the C ABI entry mac_hgproject_dense.
//
// One thread per node or cell, FP64, natural layout; the nodal hierarchy (coarse sigma and the
// node arrays of every multigrid level) lives in the context and is allocated on first use.  All
// launches go to the context's stream; the host reads one residual norm per V-cycle.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <vector>

#include "mac_internal.cuh"   // (first: hg_nodal.cuh's device code calls recip_nr)
#include "hg_nodal.cuh"

namespace mac {

namespace {

constexpr int kThreads = 256;
constexpr int kReduceBlocks = 1024;
constexpr int kMixedInner = 3;   // FP32 V-cycles per FP64 refinement step of the mixed solve

#define HG_LOOP(N) for (long idx = (long)blockIdx.x * blockDim.x + threadIdx.x; idx < (N); \
                        idx += (long)gridDim.x * blockDim.x)

template <typename T>
__global__ void k_hg_defect(hg::Geo G, hg::LevT<T> L, const T* phi, const T* f, T* r, long N) {
    HG_LOOP(N) hg::defect_node(G, L, idx, phi, f, r);
}
template <typename T>
__global__ void k_hg_gs(hg::Geo G, hg::LevT<T> L, int colour, T* phi, const T* f, long N) {
    HG_LOOP(N) hg::gs_node(G, L, idx, colour, phi, f);
}
template <typename T>
__global__ void k_hg_restrict(hg::Geo G, hg::LevT<T> F, hg::LevT<T> K, const T* rF, T* fK, long N) {
    HG_LOOP(N) hg::restrict_node(G, F, K, idx, rF, fK);
}
template <typename T>
__global__ void k_hg_prolong(hg::Geo G, hg::LevT<T> K, hg::LevT<T> F, const T* eK, T* phiF, long N) {
    HG_LOOP(N) hg::prolong_node(G, K, F, idx, eK, phiF);
}
// The same prolongation in 3-D by coarse nodes (N = the coarse level's nodes): the thread of
// coarse node P loads the 8 coarse values P + c, c in {0,1}^3 (folded through the periodic wrap)
// once and adds to each fine node 2P + a, a in {0,1}^3, that exists and is an unknown the
// interpolation prolong_node gives it -- the terms c <= a with weight 2^-(a0+a1+a2), in its
// order, so the result is bitwise the same -- instead of one thread per fine node gathering its
// own 1 to 8 parents (27 loads for the 8 fine nodes of a coarse cell instead of 8).
template <typename T>
__global__ void k_hg_prolong3(hg::Geo G, hg::LevT<T> K, hg::LevT<T> F, const T* __restrict__ eK,
                              T* __restrict__ phiF, long N) {
    HG_LOOP(N) {
        int P[3];
        hg::node_coords(K, idx, P);
        int q1[3];
#pragma unroll
        for (int d = 0; d < 3; ++d) q1[d] = hg::node_wrap(G, K, d, P[d] + 1);
        // the 8 parents (one beyond a non-periodic face is never used: its children do not exist)
        T e[2][2][2];
#pragma unroll
        for (int c2 = 0; c2 < 2; ++c2)
#pragma unroll
            for (int c1 = 0; c1 < 2; ++c1)
#pragma unroll
                for (int c0 = 0; c0 < 2; ++c0) {
                    const int i0 = c0 ? q1[0] : P[0], i1 = c1 ? q1[1] : P[1], i2 = c2 ? q1[2] : P[2];
                    e[c2][c1][c0] = (i0 >= 0 && i1 >= 0 && i2 >= 0) ? eK[hg::nix(K, i0, i1, i2)] : T(0);
                }
#pragma unroll
        for (int a2 = 0; a2 < 2; ++a2)
#pragma unroll
            for (int a1 = 0; a1 < 2; ++a1)
#pragma unroll
                for (int a0 = 0; a0 < 2; ++a0) {
                    const int p[3] = {2 * P[0] + a0, 2 * P[1] + a1, 2 * P[2] + a2};
                    if (p[0] > F.n[0] || p[1] > F.n[1] || p[2] > F.n[2]) continue;
                    if (!hg::is_unknown(G, F, p)) continue;
                    T w = 1;
                    if (a0) w *= (T)0.5;
                    if (a1) w *= (T)0.5;
                    if (a2) w *= (T)0.5;
                    T s = 0;
#pragma unroll
                    for (int b2 = 0; b2 < 2; ++b2)
#pragma unroll
                        for (int b1 = 0; b1 < 2; ++b1)
#pragma unroll
                            for (int b0 = 0; b0 < 2; ++b0) {
                                if (b2 > a2 || b1 > a1 || b0 > a0) continue;
                                s += w * e[b2][b1][b0];
                            }
                    phiF[hg::nix(F, p[0], p[1], p[2])] += s;
                }
    }
}
__global__ void k_hg_coarsen(hg::Geo G, hg::Lev F, hg::Lev K, double* sK, long N) {
    HG_LOOP(N) hg::coarsen_sig_cell(G, F, K, idx, sK);
}
template <typename T>
__global__ void k_hg_finish(hg::Geo G, hg::LevT<T> L, T* x, long N) {
    HG_LOOP(N) hg::finish_node(G, L, idx, x);
}
__global__ void k_hg_uvec(hg::Geo G, long nc, int proj_type, double dt, double idt, double* unew,
                          const double* uold, const double* gpi, const double* rhohalf,
                          const double* b0, int alt, double* sig) {
    HG_LOOP(nc) hg::uvec_cell(G, idx, nc, proj_type, dt, idt, unew, uold, gpi, rhohalf, b0, alt, sig);
}
__global__ void k_hg_divu(hg::Geo G, hg::Lev L, const double* u, const double* b0,
                          const double* nodalrhs, hg::Wall W, double* rh, long N) {
    HG_LOOP(N) hg::divu_node(G, L, idx, u, b0, nodalrhs, W, rh);
}
__global__ void k_hg_update(hg::Geo G, hg::Lev L, int proj_type, double dt, double idt,
                            const double* phi,
                            double* unew, const double* uold, double* gpi, const double* rhohalf,
                            const double* b0, int alt, long N) {
    HG_LOOP(N) hg::update_cell(G, L, idx, proj_type, dt, idt, phi, unew, uold, gpi, rhohalf, b0, alt);
}
__global__ void k_hg_update_pi(hg::Lev L, int proj_type, double dt, const double* phi, double* pi,
                               long N) {
    HG_LOOP(N) hg::update_pi_node(L, idx, proj_type, dt, phi, pi);
}

// ---- dense 3-D stencil, interior nodes --------------------------------------------------------
// For a node p and a neighbour offset o in {-1,0,1}^3 the dense finite-element weight is
// kw[mask(o)] * (the sum of sigma over the cells p and p + o share), mask(o) = the directions
// with o_d != 0: the weight table entry does not depend on which shared cell contributes.  A node
// one or more nodes away from every domain face (no wrap, no missing cell, no image node) takes
// this path: its 8 cell coefficients, 26 partial sums of them and 27 loads, all unrolled; the
// others (and 2-D, cross stencils) take node_op.  The sums are formed in a fixed order, so the
// result does not depend on the launch; it differs from node_op's only in rounding.
template <typename T>
__device__ __forceinline__ bool interior3(const hg::LevT<T>& L, const int p[3]) {
    return p[0] >= 1 && p[0] <= L.n[0] - 2 && p[1] >= 1 && p[1] <= L.n[1] - 2 && p[2] >= 1 &&
           p[2] <= L.n[2] - 2;
}
// ISO: the level's spacing is isotropic, so the weight of the 6 neighbours along one axis is
// exactly 0 (kw[1] = kw[2] = kw[4] = 0, checked by the caller) and those terms are left out:
// fma(0, a, acc) = acc for finite a, so the result is bitwise that of the full stencil.
template <typename T, bool ISO = false>
__device__ __forceinline__ void node_op_dense3(const hg::LevT<T>& L, const int p[3],
                                               const T* __restrict__ phi, T& diag, T& off) {
    const int n0 = L.n[0], n1 = L.n[1], m0 = L.nn[0], m1 = L.nn[1];
    // s[z][y][x]: the cell whose low corner is p + (x - 1, y - 1, z - 1)
    T s[2][2][2];
    const T* sg = L.sig + (p[0] - 1) + (long)n0 * ((p[1] - 1) + (long)n1 * (p[2] - 1));
#pragma unroll
    for (int z = 0; z < 2; ++z)
#pragma unroll
        for (int y = 0; y < 2; ++y)
#pragma unroll
            for (int x = 0; x < 2; ++x) s[z][y][x] = sg[x + (long)n0 * (y + (long)n1 * z)];
    // sums over the cells along x (index by the x offset of the neighbour: 0 -> -1, 1 -> 0, 2 -> +1)
    T sx[2][2][3];
#pragma unroll
    for (int z = 0; z < 2; ++z)
#pragma unroll
        for (int y = 0; y < 2; ++y) {
            sx[z][y][0] = s[z][y][0];
            sx[z][y][1] = s[z][y][0] + s[z][y][1];
            sx[z][y][2] = s[z][y][1];
        }
    T sxy[2][3][3];
#pragma unroll
    for (int z = 0; z < 2; ++z)
#pragma unroll
        for (int ox = 0; ox < 3; ++ox) {
            sxy[z][0][ox] = sx[z][0][ox];
            sxy[z][1][ox] = sx[z][0][ox] + sx[z][1][ox];
            sxy[z][2][ox] = sx[z][1][ox];
        }
    const T* ph = phi + (p[0] - 1) + (long)m0 * ((p[1] - 1) + (long)m1 * (p[2] - 1));
    // the neighbours grouped by weight class mask(o) (7 classes): sum S_o phi_o per class, then
    // one multiplication by kw per class (26 fewer multiplications than weighting each term)
    T am[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    T centre = 0;
#pragma unroll
    for (int oz = 0; oz < 3; ++oz)
#pragma unroll
        for (int oy = 0; oy < 3; ++oy)
#pragma unroll
            for (int ox = 0; ox < 3; ++ox) {
                const T S = oz == 0 ? sxy[0][oy][ox]
                                    : (oz == 2 ? sxy[1][oy][ox] : sxy[0][oy][ox] + sxy[1][oy][ox]);
                const int mask = (ox != 1 ? 1 : 0) | (oy != 1 ? 2 : 0) | (oz != 1 ? 4 : 0);
                if (mask == 0) {
                    centre = S;
                } else if (!(ISO && (mask == 1 || mask == 2 || mask == 4))) {
                    am[mask] = fma(S, ph[ox + (long)m0 * (oy + (long)m1 * oz)], am[mask]);
                }
            }
    T acc = 0;
#pragma unroll
    for (int m = 1; m < 8; ++m)
        if (!(ISO && (m == 1 || m == 2 || m == 4))) acc = fma(L.kw[m], am[m], acc);
    diag = -L.kw[0] * centre;
    off = acc;
}

// The same stencil for a node next to (or on) a domain face: cell and node indices folded through
// the periodic wrap, a missing cell (outside a non-periodic face) contributing sigma = 0 and its
// nodes read at a clamped index with weight 0, a neighbour that folds onto p itself (a periodic
// extent of 1) moved to the diagonal.  Branch-free (selects instead of branches), so all 35
// loads issue together; the terms are node_op's, grouped by neighbour.
template <typename T>
__device__ __forceinline__ void node_op_dense3_face(const hg::Geo& G, const hg::LevT<T>& L,
                                                    const int p[3], const T* __restrict__ phi,
                                                    T& diag, T& off) {
    int cw[3][2], nw[3][3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
#pragma unroll
        for (int x = 0; x < 2; ++x) cw[d][x] = hg::cell_wrap(G, L, d, p[d] - 1 + x);
#pragma unroll
        for (int o = 0; o < 3; ++o) nw[d][o] = hg::node_wrap(G, L, d, p[d] - 1 + o);
    }
    T s[2][2][2];
#pragma unroll
    for (int z = 0; z < 2; ++z)
#pragma unroll
        for (int y = 0; y < 2; ++y)
#pragma unroll
            for (int x = 0; x < 2; ++x) {
                const bool ok = cw[0][x] >= 0 && cw[1][y] >= 0 && cw[2][z] >= 0;
                const T v = L.sig[hg::cix(L, max(cw[0][x], 0), max(cw[1][y], 0), max(cw[2][z], 0))];
                s[z][y][x] = ok ? v : T(0);
            }
    T sx[2][2][3];
#pragma unroll
    for (int z = 0; z < 2; ++z)
#pragma unroll
        for (int y = 0; y < 2; ++y) {
            sx[z][y][0] = s[z][y][0];
            sx[z][y][1] = s[z][y][0] + s[z][y][1];
            sx[z][y][2] = s[z][y][1];
        }
    T sxy[2][3][3];
#pragma unroll
    for (int z = 0; z < 2; ++z)
#pragma unroll
        for (int ox = 0; ox < 3; ++ox) {
            sxy[z][0][ox] = sx[z][0][ox];
            sxy[z][1][ox] = sx[z][0][ox] + sx[z][1][ox];
            sxy[z][2][ox] = sx[z][1][ox];
        }
    const long pi = hg::nix(L, p[0], p[1], p[2]);
    T acc = 0, dsum = 0, centre = 0;
#pragma unroll
    for (int oz = 0; oz < 3; ++oz)
#pragma unroll
        for (int oy = 0; oy < 3; ++oy)
#pragma unroll
            for (int ox = 0; ox < 3; ++ox) {
                const T S = oz == 0 ? sxy[0][oy][ox]
                                    : (oz == 2 ? sxy[1][oy][ox] : sxy[0][oy][ox] + sxy[1][oy][ox]);
                const int mask = (ox != 1 ? 1 : 0) | (oy != 1 ? 2 : 0) | (oz != 1 ? 4 : 0);
                if (mask == 0) {
                    centre = S;
                } else {
                    const long m = hg::nix(L, max(nw[0][ox], 0), max(nw[1][oy], 0), max(nw[2][oz], 0));
                    const T w = L.kw[mask] * S;
                    const T v = phi[m];
                    const bool self = m == pi;
                    dsum += self ? w : T(0);
                    acc = fma(self ? T(0) : w, v, acc);
                }
            }
    diag = -(L.kw[0] * centre + dsum);
    off = acc;
}

// One half of a colour-ordered Gauss-Seidel sweep, by slabs.  The colours are the node-parity
// patterns, colour = p_0 + 2 p_1 (+ 4 p_2), updated in that order; the slab direction is the last
// active one (z in 3-D, y in 2-D).  A node's neighbours along the slab direction have the other
// slab parity, so while the colours of one slab parity are updated those neighbours stay as they
// are: the slabs of that parity are independent, and each only has to run its 2^(dm-1) in-slab
// colours in order.  Block b owns slab 2 b + sp and runs them with a block barrier between them
// (global writes of a block are visible to the block after the barrier): bitwise the update
// sequence of the 2^(dm-1) global colour launches it replaces, reading the level's phi and sigma
// about once per half instead of once per colour.
// ---- tiled Gauss-Seidel of the fine 3-D dense levels -------------------------------------------
// A sweep in two launches (slab parity sp = 0, then 1) instead of eight colour launches.  The
// colours p_0 + 2 p_1 + 4 p_2 of one slab parity are the four in-slab colours of the slabs of that
// parity, and a node's z-neighbours lie in slabs of the other parity, which the launch does not
// change.  A block owns a kTileX x kTileY tile of one slab: it stages in shared memory the slab
// and its two neighbour slabs over the tile grown by kTileH nodes, the cell coefficients of the
// two cell layers around the slab and the right-hand side, then runs the four colours in order
// on the tile grown by 3, 2, 1, 0 nodes (recomputing its neighbours' share of the ring, so the
// tile's nodes see exactly the values the global colour order gives them) and writes the tile.
// Reads come from src (the slab itself and, in the first launch, its neighbours) and srcnb (the
// neighbour slabs), writes go to dst != src: the caller alternates two arrays (the first launch
// reads and leaves src, the second reads the new even slabs from dst).  Node and cell indices
// fold through the periodic wrap when staged; outside a non-periodic face the staged values are
// 0, so every node, next to a face or not, takes node_op_dense3's arithmetic on the staged
// values: the missing neighbours of a face node carry weight 0 (a single formula keeps the
// warps of the tiles along a face from running two; the slab sweeps of the coarser levels take
// node_op_dense3_face there, the same terms summed in another order).

// One element global -> shared without passing through registers (cp.async, 4 or 8 bytes);
// inside = false writes 0 (zero-fill: nothing is read from src).
template <typename T>
__device__ __forceinline__ void stage_elem(T* dst, const T* src, bool inside) {
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
    if (sizeof(T) == 8)
        asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;" ::"r"(d), "l"(src),
                     "r"(inside ? 8 : 0) : "memory");
    else
        asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;" ::"r"(d), "l"(src),
                     "r"(inside ? 4 : 0) : "memory");
}
__device__ __forceinline__ void stage_wait() { asm volatile("cp.async.wait_all;" ::: "memory"); }

// node_op_dense3's formula on staged arrays, for every node of a tile: the staged values are
// folded through the periodic wrap and 0 outside a non-periodic face (sigma and phi), so the
// missing neighbours of a face node carry weight 0 here as well.  ss: the node's cell (-1,-1,-1)
// in a cell array of row pitch CX and layer pitch CP; ph: its node (-1,-1,-1) in a node array of
// row pitch RX and plane pitch RP.
template <typename T, bool ISO, int RX, int RP, int CX, int CP>
__device__ __forceinline__ void staged_node_op(const hg::LevT<T>& L, const T* ss, const T* ph, T& dg,
                                               T& off) {
    T s[2][2][2];
#pragma unroll
    for (int zz = 0; zz < 2; ++zz)
#pragma unroll
        for (int yy = 0; yy < 2; ++yy)
#pragma unroll
            for (int xx = 0; xx < 2; ++xx) s[zz][yy][xx] = ss[xx + CX * yy + CP * zz];
    T sx[2][2][3];
#pragma unroll
    for (int zz = 0; zz < 2; ++zz)
#pragma unroll
        for (int yy = 0; yy < 2; ++yy) {
            sx[zz][yy][0] = s[zz][yy][0];
            sx[zz][yy][1] = s[zz][yy][0] + s[zz][yy][1];
            sx[zz][yy][2] = s[zz][yy][1];
        }
    T sxy[2][3][3];
#pragma unroll
    for (int zz = 0; zz < 2; ++zz)
#pragma unroll
        for (int ox = 0; ox < 3; ++ox) {
            sxy[zz][0][ox] = sx[zz][0][ox];
            sxy[zz][1][ox] = sx[zz][0][ox] + sx[zz][1][ox];
            sxy[zz][2][ox] = sx[zz][1][ox];
        }
    T am[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    T centre = 0;
#pragma unroll
    for (int oz = 0; oz < 3; ++oz)
#pragma unroll
        for (int oy = 0; oy < 3; ++oy)
#pragma unroll
            for (int ox = 0; ox < 3; ++ox) {
                const T S = oz == 0 ? sxy[0][oy][ox]
                                    : (oz == 2 ? sxy[1][oy][ox] : sxy[0][oy][ox] + sxy[1][oy][ox]);
                const int mask = (ox != 1 ? 1 : 0) | (oy != 1 ? 2 : 0) | (oz != 1 ? 4 : 0);
                if (mask == 0)
                    centre = S;
                else if (!(ISO && (mask == 1 || mask == 2 || mask == 4)))
                    am[mask] = fma(S, ph[ox + RX * oy + RP * oz], am[mask]);
            }
    T acc = 0;
#pragma unroll
    for (int m = 1; m < 8; ++m)
        if (!(ISO && (m == 1 || m == 2 || m == 4))) acc = fma(L.kw[m], am[m], acc);
    dg = -L.kw[0] * centre;
    off = acc;
}

constexpr int kTileX = 32, kTileY = 32, kTileH = 4, kTileThreads = 384;
constexpr int kTRX = kTileX + 2 * kTileH, kTRY = kTileY + 2 * kTileH;           // staged nodes
constexpr int kTCX = kTileX + 2 * kTileH - 1, kTCY = kTileY + 2 * kTileH - 1;   // staged cells
constexpr int kTFX = kTileX + 2 * kTileH - 2, kTFY = kTileY + 2 * kTileH - 2;   // right-hand side
template <typename T>
constexpr size_t tile_smem() {
    return sizeof(T) * (3 * kTRX * kTRY + 2 * kTCX * kTCY + kTFX * kTFY);
}

// (FP32: five blocks an SM, registers capped for it; FP64: two, the staged tile being twice as large)
template <typename T, bool ISO>
__global__ void __launch_bounds__(kTileThreads, sizeof(T) == 4 ? 5 : 2)
k_hg_gs_tile(hg::Geo G, hg::LevT<T> L, int sp, int ntx, const T* __restrict__ src,
             const T* __restrict__ srcnb, T* __restrict__ dst, const T* __restrict__ f) {
    extern __shared__ __align__(16) unsigned char hg_tile_smem[];
    T* sphi = reinterpret_cast<T*>(hg_tile_smem);   // [3][kTRY][kTRX], slabs z-1, z, z+1
    T* ssig = sphi + 3 * kTRX * kTRY;                // [2][kTCY][kTCX], cell layers z-1, z
    T* sf = ssig + 2 * kTCX * kTCY;                  // [kTFY][kTFX]
    const int z = 2 * (int)blockIdx.y + sp;
    const int nzu = G.per[2] ? L.n[2] : L.n[2] + 1;  // slabs with unknown nodes
    if (z >= nzu) return;
    const int x0 = kTileX * ((int)blockIdx.x % ntx), y0 = kTileY * ((int)blockIdx.x / ntx);
    const int t = threadIdx.x;
    // per staged column / row: folded node and cell coordinates (-1: outside a non-periodic
    // face), whether the folded node is an unknown along that direction
    __shared__ int sqx[kTRX], sqy[kTRY], scx[kTCX], scy[kTCY];
    __shared__ unsigned char sux[kTRX], suy[kTRY];
    if (t < kTRX) {
        const int raw = x0 - kTileH + t;
        const int q = hg::node_wrap(G, L, 0, raw);
        sqx[t] = q;
        sux[t] = q >= 0 && !(G.per[0] ? q == L.n[0] : ((q == 0 && G.dlo[0]) || (q == L.n[0] && G.dhi[0])));
        if (t < kTCX) scx[t] = hg::cell_wrap(G, L, 0, raw);
    } else if (t >= 64 && t < 64 + kTRY) {
        const int u = t - 64, raw = y0 - kTileH + u;
        const int q = hg::node_wrap(G, L, 1, raw);
        sqy[u] = q;
        suy[u] = q >= 0 && !(G.per[1] ? q == L.n[1] : ((q == 0 && G.dlo[1]) || (q == L.n[1] && G.dhi[1])));
        if (u < kTCY) scy[u] = hg::cell_wrap(G, L, 1, raw);
    }
    // (scalars, not arrays: a dynamically indexed array would live in local memory)
    const int qz0 = hg::node_wrap(G, L, 2, z - 1), qz1 = hg::node_wrap(G, L, 2, z),
              qz2 = hg::node_wrap(G, L, 2, z + 1);
    const int cz0 = hg::cell_wrap(G, L, 2, z - 1), cz1 = hg::cell_wrap(G, L, 2, z);
    const bool uz = qz1 >= 0 &&
                    !(G.per[2] ? qz1 == L.n[2] : ((qz1 == 0 && G.dlo[2]) || (qz1 == L.n[2] && G.dhi[2])));
    __syncthreads();
    const long m01 = (long)L.nn[0] * L.nn[1], c01 = (long)L.n[0] * L.n[1];
    // stage: nodes x0 - kTileH .. x0 + kTileX + kTileH - 1 (same in y), slabs z - 1 .. z + 1,
    // the two cell layers and the right-hand side, all copies in flight at once.  A thread keeps
    // one staged column (its folded x in a register) and walks the rows kPR apart.
    constexpr int kPR = kTileThreads / kTRX;
    if (t < kPR * kTRX) {
        const int lx = t % kTRX, r0 = t / kTRX;
        const int q0 = sqx[lx];
        const int im0 = L.nn[0], ic0 = L.n[0];
#pragma unroll 1
        for (int lz = 0; lz < 3; ++lz) {
            const int q2 = lz == 0 ? qz0 : (lz == 1 ? qz1 : qz2);
            const T* from = lz == 1 ? src : srcnb;
            const bool zin = q0 >= 0 && q2 >= 0;
            const T* pb = from + (zin ? q0 + q2 * m01 : 0);
            T* dst_col = sphi + lz * (kTRX * kTRY) + lx;
            for (int ly = r0; ly < kTRY; ly += kPR) {
                const int q1 = sqy[ly];
                const bool in = zin && q1 >= 0;
                stage_elem(dst_col + ly * kTRX, in ? pb + (long)q1 * im0 : from, in);
            }
        }
        if (lx < kTCX) {
            const int c0 = scx[lx];
#pragma unroll 1
            for (int lz = 0; lz < 2; ++lz) {
                const int c2 = lz == 0 ? cz0 : cz1;
                const bool zin = c0 >= 0 && c2 >= 0;
                const T* pb = L.sig + (zin ? c0 + c2 * c01 : 0);
                T* dst_col = ssig + lz * (kTCX * kTCY) + lx;
                for (int ly = r0; ly < kTCY; ly += kPR) {
                    const int c1 = scy[ly];
                    const bool in = zin && c1 >= 0;
                    stage_elem(dst_col + ly * kTCX, in ? pb + (long)c1 * ic0 : L.sig, in);
                }
            }
        }
        if (lx >= 1 && lx <= kTFX) {
            const bool zin = q0 >= 0 && qz1 >= 0;
            const T* pb = f + (zin ? q0 + qz1 * m01 : 0);
            T* dst_col = sf + (lx - 1);
            for (int ly = r0; ly < kTFY; ly += kPR) {
                const int q1 = sqy[ly + 1];
                const bool in = zin && q1 >= 0;
                stage_elem(dst_col + ly * kTFX, in ? pb + (long)q1 * im0 : f, in);
            }
        }
    }
    stage_wait();
    __syncthreads();
    // the four in-slab colours, on the tile grown by 3, 2, 1, 0 nodes
#pragma unroll 1
    for (int k = 0; k < 4; ++k) {
        const int h = 3 - k, px = k & 1, py = k >> 1;
        const int xs = x0 - h + ((px - (x0 - h)) & 1), ys = y0 - h + ((py - (y0 - h)) & 1);
        const int nx = (x0 + kTileX - 1 + h - xs) / 2 + 1, ny = (y0 + kTileY - 1 + h - ys) / 2 + 1;
        for (int e = t; e < nx * ny; e += kTileThreads) {
            const int lx = xs - (x0 - kTileH) + 2 * (e % nx), ly = ys - (y0 - kTileH) + 2 * (e / nx);
            if (!(sux[lx] && suy[ly] && uz)) continue;
            T dg, off;
            staged_node_op<T, ISO, kTRX, kTRX * kTRY, kTCX, kTCX * kTCY>(
                L, ssig + (lx - 1) + kTCX * (ly - 1), sphi + (lx - 1) + kTRX * (ly - 1), dg, off);
            const int fi = (lx - 1) + kTFX * (ly - 1);
            sphi[lx + kTRX * (ly + kTRY)] = (sf[fi] + off) / dg;
        }
        __syncthreads();
    }
    // the tile's own unknown nodes
    for (int e = t; e < kTileX * kTileY; e += kTileThreads) {
        const int p[3] = {x0 + e % kTileX, y0 + e / kTileX, z};
        if (p[0] > L.n[0] - (G.per[0] ? 1 : 0) || p[1] > L.n[1] - (G.per[1] ? 1 : 0)) continue;
        if (!hg::is_unknown(G, L, p)) continue;
        dst[hg::nix(L, p[0], p[1], p[2])] =
            sphi[(p[0] - x0 + kTileH) + kTRX * ((p[1] - y0 + kTileH) + kTRY)];
    }
}

// ---- tiled defect of the fine 3-D dense levels ---------------------------------------------
// r = f - L phi on the unknown nodes, 0 on the other nodes of the domain (periodic images are
// left as they are: nothing reads them).  A block owns a kDefX x kDefY tile of one slab: it stages
// the slab and its two neighbour slabs over the tile grown by one node and the two cell layers
// (folded through the periodic wrap, 0 outside the domain) and forms each node's defect with
// staged_node_op -- the arithmetic of node_op_dense3 for every node, so interior nodes get
// k_hg_defect3's result bitwise and nodes next to a face its terms in another order -- instead
// of one thread per node reading its 35 operands through the cache.
constexpr int kDefX = 32, kDefY = 32, kDefThreads = 256;
constexpr int kDRX = kDefX + 2, kDRY = kDefY + 2;   // staged nodes
constexpr int kDCX = kDefX + 1, kDCY = kDefY + 1;   // staged cells
template <typename T>
constexpr size_t deftile_smem() {
    return sizeof(T) * (3 * kDRX * kDRY + 2 * kDCX * kDCY);
}

template <typename T, bool ISO>
__global__ void __launch_bounds__(kDefThreads)
k_hg_defect_tile(hg::Geo G, hg::LevT<T> L, int ntx, const T* __restrict__ phi,
                 const T* __restrict__ f, T* __restrict__ r) {
    extern __shared__ __align__(16) unsigned char hg_deftile_smem[];
    T* sphi = reinterpret_cast<T*>(hg_deftile_smem);   // [3][kDRY][kDRX], slabs z-1, z, z+1
    T* ssig = sphi + 3 * kDRX * kDRY;                   // [2][kDCY][kDCX], cell layers z-1, z
    const int z = (int)blockIdx.y;                      // 0 .. the slabs with unknown nodes - 1
    const int x0 = kDefX * ((int)blockIdx.x % ntx), y0 = kDefY * ((int)blockIdx.x / ntx);
    const int t = threadIdx.x;
    __shared__ int sqx[kDRX], sqy[kDRY], scx[kDCX], scy[kDCY];
    if (t < kDRX) {
        const int raw = x0 - 1 + t;
        sqx[t] = hg::node_wrap(G, L, 0, raw);
        if (t < kDCX) scx[t] = hg::cell_wrap(G, L, 0, raw);
    } else if (t >= 64 && t < 64 + kDRY) {
        const int u = t - 64, raw = y0 - 1 + u;
        sqy[u] = hg::node_wrap(G, L, 1, raw);
        if (u < kDCY) scy[u] = hg::cell_wrap(G, L, 1, raw);
    }
    const int qz0 = hg::node_wrap(G, L, 2, z - 1), qz1 = hg::node_wrap(G, L, 2, z),
              qz2 = hg::node_wrap(G, L, 2, z + 1);
    const int cz0 = hg::cell_wrap(G, L, 2, z - 1), cz1 = hg::cell_wrap(G, L, 2, z);
    __syncthreads();
    const long m01 = (long)L.nn[0] * L.nn[1], c01 = (long)L.n[0] * L.n[1];
    // stage, one column a thread (its folded x in a register), rows kPR apart
    constexpr int kPR = kDefThreads / kDRX;
    if (t < kPR * kDRX) {
        const int lx = t % kDRX, r0 = t / kDRX;
        const int q0 = sqx[lx];
        const int im0 = L.nn[0], ic0 = L.n[0];
#pragma unroll 1
        for (int lz = 0; lz < 3; ++lz) {
            const int q2 = lz == 0 ? qz0 : (lz == 1 ? qz1 : qz2);
            const bool zin = q0 >= 0 && q2 >= 0;
            const T* pb = phi + (zin ? q0 + q2 * m01 : 0);
            T* dst_col = sphi + lz * (kDRX * kDRY) + lx;
            for (int ly = r0; ly < kDRY; ly += kPR) {
                const int q1 = sqy[ly];
                const bool in = zin && q1 >= 0;
                stage_elem(dst_col + ly * kDRX, in ? pb + (long)q1 * im0 : phi, in);
            }
        }
        if (lx < kDCX) {
            const int c0 = scx[lx];
#pragma unroll 1
            for (int lz = 0; lz < 2; ++lz) {
                const int c2 = lz == 0 ? cz0 : cz1;
                const bool zin = c0 >= 0 && c2 >= 0;
                const T* pb = L.sig + (zin ? c0 + c2 * c01 : 0);
                T* dst_col = ssig + lz * (kDCX * kDCY) + lx;
                for (int ly = r0; ly < kDCY; ly += kPR) {
                    const int c1 = scy[ly];
                    const bool in = zin && c1 >= 0;
                    stage_elem(dst_col + ly * kDCX, in ? pb + (long)c1 * ic0 : L.sig, in);
                }
            }
        }
    }
    stage_wait();
    __syncthreads();
    for (int e = t; e < kDefX * kDefY; e += kDefThreads) {
        const int lx = 1 + e % kDefX, ly = 1 + e / kDefX;
        const int p[3] = {x0 + lx - 1, y0 + ly - 1, z};
        if (p[0] > L.n[0] - (G.per[0] ? 1 : 0) || p[1] > L.n[1] - (G.per[1] ? 1 : 0)) continue;
        const long i = hg::nix(L, p[0], p[1], p[2]);
        if (!hg::is_unknown(G, L, p)) {
            r[i] = 0;
            continue;
        }
        T dg, off;
        staged_node_op<T, ISO, kDRX, kDRX * kDRY, kDCX, kDCX * kDCY>(
            L, ssig + (lx - 1) + kDCX * (ly - 1), sphi + (lx - 1) + kDRX * (ly - 1), dg, off);
        r[i] = f[i] - (dg * sphi[lx + kDRX * (ly + kDRY)] - off);
    }
}

constexpr int kSlabThreads = 512;   // most threads of a slab block
template <typename T, bool DENSE3>
__global__ void __launch_bounds__(kSlabThreads)
k_hg_gs_slab(hg::Geo G, hg::LevT<T> L, int sp, T* phi, const T* f) {
    const int dm = G.dm, sd = dm - 1;
    const int slab = 2 * (int)blockIdx.x + sp;
    if (slab >= (sd == 2 ? L.nn[2] : L.nn[1])) return;   // (a select: no dynamic index)
    for (int cq = 0; cq < (1 << sd); ++cq) {
        const int px = cq & 1, py = sd == 2 ? (cq >> 1) & 1 : 0;
        const int mx = (L.nn[0] - px + 1) / 2;
        const int my = sd == 2 ? (L.nn[1] - py + 1) / 2 : 1;
        const int cnt = mx * my;
        for (int t = threadIdx.x; t < cnt; t += blockDim.x) {
            const int ty = t / mx;
            int p[3] = {2 * (t - ty * mx) + px, 0, 0};
            if (sd == 2) {
                p[1] = 2 * ty + py;
                p[2] = slab;
            } else {
                p[1] = slab;
            }
            if (!hg::is_unknown(G, L, p)) continue;
            T dg, off;
            if (DENSE3) {
                if (interior3(L, p))
                    node_op_dense3(L, p, phi, dg, off);
                else
                    node_op_dense3_face(G, L, p, phi, dg, off);
            } else {
                hg::node_op(G, L, p, phi, dg, off);
            }
            const long i = hg::nix(L, p[0], p[1], p[2]);
            phi[i] = (f[i] + off) / dg;
        }
        __syncthreads();
    }
}

template <typename T, bool ISO>
__global__ void k_hg_defect3(hg::Geo G, hg::LevT<T> L, const T* phi, const T* f, T* r, long N) {
    HG_LOOP(N) {
        int p[3];
        hg::node_coords(L, idx, p);
        if (!hg::is_unknown(G, L, p)) {
            r[idx] = 0;
            continue;
        }
        T dg, off;
        if (interior3(L, p))
            node_op_dense3<T, ISO>(L, p, phi, dg, off);
        else
            node_op_dense3_face(G, L, p, phi, dg, off);
        r[idx] = f[idx] - (dg * phi[idx] - off);
    }
}

// ---- exact coarsest-level solve --------------------------------------------------------------
constexpr int kExactMax = 128;   // unknown nodes of a coarsest level solved by its dense inverse
constexpr int kExactThreads = 256;

// One block: the operator of the coarsest level (FP64, rows by node_row) on its M unknown
// nodes, plus sigma 1 1^T for the singular problem (sigma = mean diagonal / M: B^-1 f = A^+ f
// for a mean-free f), inverted in place by Gauss-Jordan elimination without pivoting (B is
// definite).  A: M x M, row-major.
__global__ void __launch_bounds__(kExactThreads)
k_hg_bottom_inverse(hg::Geo G, hg::Lev L, int M, const int* __restrict__ node,
                    const int* __restrict__ map, int singular, double* __restrict__ A) {
    __shared__ double col[kExactMax];
    __shared__ double piv;
    const int t = threadIdx.x;
    for (int e = t; e < M * M; e += kExactThreads) A[e] = 0.0;
    __syncthreads();
    for (int u = t; u < M; u += kExactThreads) {
        int p[3];
        hg::node_coords(L, node[u], p);
        double* row = A + (long)u * M;
        hg::node_row(G, L, p, [&](long m, double w) {
            const int v = map[m];
            if (v >= 0) row[v] += w;
        });
    }
    __syncthreads();
    if (singular) {
        if (t == 0) {
            double s = 0.0;
            for (int u = 0; u < M; ++u) s += A[(long)u * M + u];
            piv = s / M / M;
        }
        __syncthreads();
        const double sg = piv;
        for (int e = t; e < M * M; e += kExactThreads) A[e] += sg;
        __syncthreads();
    }
    for (int k = 0; k < M; ++k) {
        if (t == 0) {
            piv = 1.0 / A[(long)k * M + k];
            A[(long)k * M + k] = 1.0;
        }
        __syncthreads();
        const double ip = piv;
        for (int j = t; j < M; j += kExactThreads) A[(long)k * M + j] *= ip;
        for (int i = t; i < M; i += kExactThreads) {
            if (i == k) continue;
            col[i] = A[(long)i * M + k];
            A[(long)i * M + k] = 0.0;
        }
        __syncthreads();
        for (int e = t; e < M * M; e += kExactThreads) {
            const int i = e / M, j = e - i * M;
            if (i != k) A[e] -= col[i] * A[(long)k * M + j];
        }
        __syncthreads();
    }
}

// phi = B^-1 f on the unknown nodes of the coarsest level (FP64 arithmetic; phi elsewhere
// untouched).
template <typename T>
__global__ void __launch_bounds__(kExactThreads)
k_hg_bottom_exact(int M, const int* __restrict__ node, const double* __restrict__ Binv,
                  const T* __restrict__ f, T* __restrict__ phi) {
    __shared__ double fs[kExactMax];
    for (int v = threadIdx.x; v < M; v += kExactThreads) fs[v] = (double)f[node[v]];
    __syncthreads();
    for (int u = threadIdx.x; u < M; u += kExactThreads) {
        const double* row = Binv + (long)u * M;
        double x = 0.0;
        for (int v = 0; v < M; ++v) x = fma(row[v], fs[v], x);
        phi[node[u]] = (T)x;
    }
}

// nu colour-ordered Gauss-Seidel sweeps of the coarsest level in one block.  An odd periodic
// extent couples nodes of one colour across the wrap: then one thread sweeps in order.
template <typename T>
__global__ void k_hg_bottom(hg::Geo G, hg::LevT<T> L, T* phi, const T* f, int nu, long N) {
    bool serial = false;
    for (int d = 0; d < G.dm; ++d) serial = serial || (G.per[d] && (L.n[d] & 1));
    const long start = serial ? 0 : threadIdx.x;
    const long step = serial ? 1 : blockDim.x;
    const bool active = !serial || threadIdx.x == 0;
    for (int s = 0; s < nu; ++s)
        for (int colour = 0; colour < (1 << G.dm); ++colour) {
            if (active)
                for (long idx = start; idx < hg::colour_count(G, L, colour); idx += step)
                    hg::gs_node(G, L, idx, colour, phi, f);
            __syncthreads();
        }
}

__global__ void k_hg_to_single(const double* r, float* r32, long N) {
    HG_LOOP(N) hg::to_single_node(idx, r, r32);
}
__global__ void k_hg_accumulate(hg::Geo G, hg::Lev L, double* phi, const float* e, long N) {
    HG_LOOP(N) hg::accumulate_node(G, L, idx, phi, e);
}
__global__ void k_hg_sig_single(const double* s, float* s32, long N) {
    HG_LOOP(N) s32[idx] = (float)s[idx];
}

// Per-block partials over the unknown nodes: [0] sum, [1] max |x|, [2] NaN count, [3] count.
// Only the sum is FP64 arithmetic: the NaN test, |x| and its maximum work on the IEEE bit
// pattern (for non-negative doubles the unsigned order of the bits is the numeric order) and
// the counts are integers, as GB300's FP64 pipe is the narrow one.
template <typename T>
__global__ void k_hg_reduce(hg::Geo G, hg::LevT<T> L, const T* x, double* part, long N) {
    __shared__ double s[kThreads / 32];
    __shared__ unsigned long long smax[kThreads / 32], snan[kThreads / 32], scnt[kThreads / 32];
    double sum = 0.0;
    unsigned long long amax = 0, nnan = 0, cnt = 0;
    HG_LOOP(N) {
        int p[3];
        hg::node_coords(L, idx, p);
        if (!hg::is_unknown(G, L, p)) continue;
        const double v = (double)x[idx];
        const unsigned long long b = (unsigned long long)__double_as_longlong(v) & 0x7fffffffffffffffull;
        if (b > 0x7ff0000000000000ull) {
            ++nnan;
            continue;
        }
        sum += v;
        amax = b > amax ? b : amax;
        ++cnt;
    }
    for (int o = 16; o > 0; o >>= 1) {
        sum += __shfl_down_sync(0xffffffffu, sum, o);
        const unsigned long long m = __shfl_down_sync(0xffffffffu, amax, o);
        amax = m > amax ? m : amax;
        nnan += __shfl_down_sync(0xffffffffu, nnan, o);
        cnt += __shfl_down_sync(0xffffffffu, cnt, o);
    }
    const int w = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0) {
        s[w] = sum;
        smax[w] = amax;
        snan[w] = nnan;
        scnt[w] = cnt;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int q = 1; q < kThreads / 32; ++q) {
            sum += s[q];
            amax = smax[q] > amax ? smax[q] : amax;
            nnan += snan[q];
            cnt += scnt[q];
        }
        part[4 * blockIdx.x] = sum;
        part[4 * blockIdx.x + 1] = __longlong_as_double((long long)amax);
        part[4 * blockIdx.x + 2] = (double)nnan;
        part[4 * blockIdx.x + 3] = (double)cnt;
    }
}

// out[0] sum, [1] max, [2] NaN count, [3] count, [4] mean; one block, fixed order.
__global__ void k_hg_reduce_finish(const double* part, int nparts, double* out) {
    __shared__ double s[4][kThreads];
    double a[4] = {0.0, 0.0, 0.0, 0.0};
    for (int q = threadIdx.x; q < nparts; q += blockDim.x) {
        a[0] += part[4 * q];
        a[1] = fmax(a[1], part[4 * q + 1]);
        a[2] += part[4 * q + 2];
        a[3] += part[4 * q + 3];
    }
    for (int k = 0; k < 4; ++k) s[k][threadIdx.x] = a[k];
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) {
            s[0][threadIdx.x] += s[0][threadIdx.x + w];
            s[1][threadIdx.x] = fmax(s[1][threadIdx.x], s[1][threadIdx.x + w]);
            s[2][threadIdx.x] += s[2][threadIdx.x + w];
            s[3][threadIdx.x] += s[3][threadIdx.x + w];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        for (int k = 0; k < 4; ++k) out[k] = s[k][0];
        out[4] = s[3][0] > 0.0 ? s[0][0] / s[3][0] : 0.0;
    }
}

template <typename T>
__global__ void k_hg_sub_mean(hg::Geo G, hg::LevT<T> L, T* x, const double* m, long N) {
    const T v = (T)*m;
    HG_LOOP(N) {
        int p[3];
        hg::node_coords(L, idx, p);
        if (hg::is_unknown(G, L, p)) x[idx] -= v;
    }
}

// A rhohalf that is not positive and finite, or a beta0 that is not, raises flag[0].
__global__ void k_hg_check(const double* rhohalf, const double* b0, int* flag, long N) {
    HG_LOOP(N) {
        const double r = rhohalf[idx];
        const double b = b0 ? b0[idx] : 1.0;
        if (!(r > 0.0) || !(r < INFINITY) || !(b > 0.0) || !(b < INFINITY)) atomicExch(flag, 1);
    }
}

// Caller fabs <-> whole-domain arrays, ncomp components (component stride `stride` in the
// array, B.count in the fab); blockIdx.y is the fab.
__global__ void k_hg_fabs_gather(hg::Geo G, hg::Lev L, const hg::Fab* T, int ncomp, long stride,
                                 double* arr) {
    const hg::Fab B = T[blockIdx.y];
    for (long e = (long)blockIdx.x * blockDim.x + threadIdx.x; e < B.count;
         e += (long)gridDim.x * blockDim.x) {
        const long t = hg::fab_target(G, L, B, e);
        if (t < 0) continue;
        for (int q = 0; q < ncomp; ++q) arr[q * stride + t] = B.src[q * B.count + e];
    }
}
__global__ void k_hg_fabs_scatter(hg::Geo G, hg::Lev L, const hg::Fab* T, int ncomp, long stride,
                                  const double* arr) {
    const hg::Fab B = T[blockIdx.y];
    for (long e = (long)blockIdx.x * blockDim.x + threadIdx.x; e < B.count;
         e += (long)gridDim.x * blockDim.x) {
        const long t = hg::fab_target(G, L, B, e);
        if (t < 0) continue;
        for (int q = 0; q < ncomp; ++q) B.dst[q * B.count + e] = arr[q * stride + t];
    }
}

// Wall values of the inflow faces from the ghost cells just outside them (per-box entry), as the
// divergence takes them: create_uvec_for_projection leaves an inlet face's ghost velocity as the
// caller filled it (the inflow velocity on the wall), except that the pressure iterations project
// (U - Uold) / dt there too (Source/hgproject.f90:461-474, the loops include the first ghost
// layer); U is then scaled by beta0_cart on the ghost layers beta0_cart has
// (Source/hgproject.f90:140-143, multifab_mult_mult_c over nghost(beta0_cart)).  One thread per
// cell of a face that a box touches; blockIdx.y = box, blockIdx.z = face 2 d + side.  TU / TUO /
// TB: the unew / uold / beta0_cart fab tables (TUO null unless pressure iterations; TB null, or
// b0_ghost 0: no beta0 scaling of the ghost).
__global__ void k_hg_fabs_wall(int dm, hg::Lev L, hg::Wall W, const hg::Fab* TU,
                               const hg::Fab* TUO, const hg::Fab* TB, int b0_ghost, double dt,
                               double* wall) {
    const int f = blockIdx.z;
    const int d = f >> 1, side = f & 1;
    if (d >= dm || W.off[f] < 0) return;
    const hg::Fab U = TU[blockIdx.y];
    if (side == 0 ? U.lo[d] != 0 : U.hi[d] != L.n[d] - 1) return;   // not on this face
    const int e1 = d == 0 ? 1 : 0;
    const int e2 = d == 2 ? 1 : 2;
    const int t1 = U.hi[e1] - U.lo[e1] + 1;
    const int t2 = dm == 3 ? U.hi[e2] - U.lo[e2] + 1 : 1;
    for (long e = (long)blockIdx.x * blockDim.x + threadIdx.x; e < (long)t1 * t2;
         e += (long)gridDim.x * blockDim.x) {
        const int i1 = (int)(e % t1), i2 = (int)(e / t1);
        // fab-local position of the ghost cell (valid cells start at ng)
        auto at = [&](const hg::Fab& B) {
            int a[3] = {0, 0, 0};
            a[d] = side == 0 ? B.ng - 1 : B.ng + (B.hi[d] - B.lo[d] + 1);
            a[e1] = B.ng + i1;
            if (dm == 3) a[e2] = B.ng + i2;
            return (long)a[0] + (long)B.ext[0] * (a[1] + (long)B.ext[1] * a[2]);
        };
        double w = U.src[(long)d * U.count + at(U)];
        if (TUO) {
            const hg::Fab O = TUO[blockIdx.y];
            w = (w - O.src[(long)d * O.count + at(O)]) / dt;
        }
        if (TB && b0_ghost) {
            const hg::Fab B = TB[blockIdx.y];
            w *= B.src[at(B)];
        }
        const long t = (long)(U.lo[e1] + i1) + (dm == 3 ? (long)L.n[e1] * (U.lo[e2] + i2) : 0L);
        wall[W.off[f] + t] = w;
    }
}

inline int blocks_for(long n, int sms) {
    const long b = (n + kThreads - 1) / kThreads;
    const long cap = (long)std::max(1, sms) * 16;
    return (int)std::max(1L, std::min(b, cap));
}

}  // namespace

struct HgState {
    hg::Geo geo{};
    struct Level {
        hg::Lev lev{};
        double* sig = nullptr;
        double* buf[hg::kNumBufs] = {};
        hg::LevT<float> lev32{};          // FP32 copy of the level (mixed precision)
        float* sig32 = nullptr;
        float* buf32[hg::kNumBufs] = {};
        // the second phi array of the tiled Gauss-Seidel (first use; zero, so that the
        // outflow nodes it never writes read 0)
        double* alt = nullptr;
        float* alt32 = nullptr;
        long nn = 0, nc = 0;
    };
    std::vector<Level> L;
    // exact solve of the coarsest level (at most kExactMax unknown nodes): its unknown nodes
    // (storage indices), node -> unknown number (-1: not an unknown), and the dense inverse of
    // its operator (B = A + sigma 1 1^T when singular), rebuilt with the coefficients each call
    // captured V-cycles (per precision: [0] FP64, [1] FP32), replayed while the key matches
    struct Graph {
        cudaGraphExec_t exec = nullptr;
        int key[4] = {-1, -1, -1, -1};   // count, nu1, nu2, dense stencil
        long long kernels = 0;
    } graph[2];
    int bM = 0;
    int* bnode = nullptr;
    int* bmap = nullptr;
    double* binv = nullptr;
    double* part = nullptr;
    double* out = nullptr;
    double* h_out = nullptr;
    int* flag = nullptr;
    int* h_flag = nullptr;
    std::vector<void*> allocs;
    // per-box calls: whole-domain copies of the fields, fab tables, host staging
    double* fu = nullptr;     // unew (dm components)
    double* fuo = nullptr;    // uold
    double* fg = nullptr;     // gpi
    double* frho = nullptr;
    double* fpi = nullptr;    // nodes
    double* fb0 = nullptr;
    double* fnr = nullptr;    // nodes
    hg::Fab* h_tab = nullptr;
    hg::Fab* d_tab = nullptr;
    size_t tab_cap = 0;
    double* staging = nullptr;
    size_t staging_cap = 0;
    double* fwall = nullptr;   // per-box calls: wall values of the inflow faces (hg::Wall)
    size_t fwall_cap = 0;
    // kernel-class timing (mac_opts.timing): CUDA events around level-0 launches, read after
    // the call; the cycles run uncaptured then
    struct Span {
        int cls, launches;
        cudaEvent_t a, b;
    };
    std::vector<cudaEvent_t> ev_pool;
    size_t ev_used = 0;
    std::vector<Span> spans;
};

void hg_release(mac_ctx* c) {
    HgState* H = c->hgs;
    if (!H) return;
    if (c->stream) cudaStreamSynchronize(c->stream);
    for (auto& g : H->graph)
        if (g.exec) cudaGraphExecDestroy(g.exec);
    for (void* p : H->allocs) cudaFree(p);
    if (H->d_tab) cudaFree(H->d_tab);
    if (H->staging) cudaFree(H->staging);
    if (H->fwall) cudaFree(H->fwall);
    for (cudaEvent_t e : H->ev_pool) cudaEventDestroy(e);
    if (H->h_tab) cudaFreeHost(H->h_tab);
    if (H->h_out) cudaFreeHost(H->h_out);
    if (H->h_flag) cudaFreeHost(H->h_flag);
    delete H;
    c->hgs = nullptr;
}

namespace {

template <typename T>
int hg_alloc(HgState* H, T** p, size_t n) {
    void* q = nullptr;
    if (cudaMalloc(&q, std::max<size_t>(n, 1) * sizeof(T)) != cudaSuccess) {
        cudaGetLastError();
        return MAC_ERR_ALLOC;
    }
    H->allocs.push_back(q);
    *p = static_cast<T*>(q);
    return MAC_OK;
}

// The nodal hierarchy of the context's geometry: level 0 at the context's cells, coarsened by 2
// while every active extent is even and at least 4.
int hg_ensure(mac_ctx* c) {
    if (c->hgs) return MAC_OK;
    HgState* H = new HgState();
    c->hgs = H;
    hg::Geo& G = H->geo;
    G.dm = c->dm;
    for (int d = 0; d < 3; ++d) {
        G.per[d] = d < c->dm && c->bc_lo[d] == MAC_BC_PER;
        G.dlo[d] = d < c->dm && c->bc_lo[d] == MAC_BC_DIR;
        G.dhi[d] = d < c->dm && c->bc_hi[d] == MAC_BC_DIR;
    }
    int n[3], rc = MAC_OK;
    double h[3];
    for (int d = 0; d < 3; ++d) {
        n[d] = d < c->dm ? c->n[d] : 1;
        h[d] = c->dx[d];
    }
    while (true) {
        HgState::Level S;
        for (int d = 0; d < 3; ++d) {
            S.lev.n[d] = n[d];
            S.lev.nn[d] = d < c->dm ? n[d] + 1 : 1;
            S.lev.h[d] = h[d];
        }
        S.nn = hg::nnodes(S.lev);
        S.nc = hg::ncells(S.lev);
        rc = hg_alloc(H, &S.sig, (size_t)S.nc);
        for (int b = 0; b < hg::kNumBufs && !rc; ++b) rc = hg_alloc(H, &S.buf[b], (size_t)S.nn);
        if (rc) break;
        S.lev.sig = S.sig;
        hg::set_dense_weights(c->dm, S.lev);
        H->L.push_back(S);
        bool more = (int)H->L.size() < hg::kMaxLevels;
        for (int d = 0; d < c->dm; ++d) more = more && n[d] % 2 == 0 && n[d] >= 4;
        if (!more) break;
        for (int d = 0; d < c->dm; ++d) {
            n[d] /= 2;
            h[d] *= 2;
        }
    }
    // the coarsest level's unknown nodes, for its exact solve when there are few
    if (!rc && !H->L.empty()) {
        const hg::Lev& B = H->L.back().lev;
        const long nnb = hg::nnodes(B);
        std::vector<int> map((size_t)nnb, -1), nodes;
        for (long idx = 0; idx < nnb; ++idx) {
            int p[3];
            hg::node_coords(B, idx, p);
            if (!hg::is_unknown(G, B, p)) continue;
            map[(size_t)idx] = (int)nodes.size();
            nodes.push_back((int)idx);
        }
        if (!nodes.empty() && (int)nodes.size() <= kExactMax) {
            H->bM = (int)nodes.size();
            rc = hg_alloc(H, &H->bnode, nodes.size());
            if (!rc) rc = hg_alloc(H, &H->bmap, map.size());
            if (!rc) rc = hg_alloc(H, &H->binv, nodes.size() * nodes.size());
            if (!rc && (cudaMemcpy(H->bnode, nodes.data(), nodes.size() * sizeof(int),
                                   cudaMemcpyHostToDevice) != cudaSuccess ||
                        cudaMemcpy(H->bmap, map.data(), map.size() * sizeof(int),
                                   cudaMemcpyHostToDevice) != cudaSuccess)) {
                cudaGetLastError();
                rc = MAC_ERR_CUDA;
            }
        }
    }
    if (!rc) rc = hg_alloc(H, &H->part, (size_t)4 * kReduceBlocks);
    if (!rc) rc = hg_alloc(H, &H->out, 8);
    if (!rc) rc = hg_alloc(H, &H->flag, 1);
    if (!rc && (cudaMallocHost((void**)&H->h_out, 8 * sizeof(double)) != cudaSuccess ||
                cudaMallocHost((void**)&H->h_flag, sizeof(int)) != cudaSuccess)) {
        cudaGetLastError();
        rc = MAC_ERR_ALLOC;
    }
    if (rc) hg_release(c);
    return rc;
}

// Level accessors per precision.
template <typename T> struct HgAccess;
template <> struct HgAccess<double> {
    static hg::LevT<double> lev(const HgState::Level& S) { return S.lev; }
    static double* buf(const HgState::Level& S, int w) { return S.buf[w]; }
    static double*& alt(HgState::Level& S) { return S.alt; }
};
template <> struct HgAccess<float> {
    static hg::LevT<float> lev(const HgState::Level& S) { return S.lev32; }
    static float* buf(const HgState::Level& S, int w) { return S.buf32[w]; }
    static float*& alt(HgState::Level& S) { return S.alt32; }
};

// The multigrid half of the executor in precision T on the context's stream.
template <typename T>
struct HgMg {
    mac_ctx* c;
    HgState* H;
    int nlev;
    hg::Geo geo;
    bool singular;
    int err = MAC_OK;

    hg::LevT<T> lev(int l) const { return HgAccess<T>::lev(H->L[l]); }
    T* buf(int l, int w) const { return HgAccess<T>::buf(H->L[l], w); }
    long nn(int l) const { return H->L[l].nn; }
    long nc(int l) const { return H->L[l].nc; }
    int blocks(long n) const { return blocks_for(n, c->sms); }
    int error() const { return err; }
    void launched() {
        ++c->issued;
        if (!err && cudaPeekAtLastError() != cudaSuccess) {
            set_last_cuda_error(cudaGetLastError(), "hg kernel launch", __FILE__, __LINE__);
            err = MAC_ERR_CUDA;
        }
    }
    bool dense3() const { return geo.dense && geo.dm == 3; }
    // isotropic level spacing: the dense 3-D weights of the axis neighbours are exactly 0
    bool iso(int l) const {
        const hg::LevT<T>& L = lev(l);
        return dense3() && L.kw[1] == T(0) && L.kw[2] == T(0) && L.kw[4] == T(0);
    }
    // count V-cycles from level 0, captured once into a CUDA graph per (count, nu1, nu2,
    // stencil) and replayed: the cycle issues one launch per colour, level and kernel kind,
    // most of them small, and needs no host value inside
    void run_cycles(int count, int nu1, int nu2) {
        prepare_tiles();
        if (err) return;
        if (c->o.timing) {   // events around the level-0 launches: no capture
            for (int v = 0; v < count; ++v) hg::vcycle(*this, 0, nu1, nu2);
            return;
        }
        HgState::Graph& g = H->graph[std::is_same<T, float>::value ? 1 : 0];
        const int key[4] = {count, nu1, nu2, geo.dense};
        if (!g.exec || std::memcmp(g.key, key, sizeof(key)) != 0) {
            if (g.exec) cudaGraphExecDestroy(g.exec);
            g.exec = nullptr;
            const long long before = c->issued;
            cudaGraph_t gr = nullptr;
            if (cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
                set_last_cuda_error(cudaGetLastError(), "cudaStreamBeginCapture", __FILE__, __LINE__);
                err = MAC_ERR_CUDA;
                return;
            }
            for (int v = 0; v < count; ++v) hg::vcycle(*this, 0, nu1, nu2);
            const cudaError_t ec = cudaStreamEndCapture(c->stream, &gr);
            if (ec != cudaSuccess || err ||
                cudaGraphInstantiate(&g.exec, gr, 0) != cudaSuccess) {
                set_last_cuda_error(cudaGetLastError(), "hg V-cycle graph", __FILE__, __LINE__);
                if (gr) cudaGraphDestroy(gr);
                g.exec = nullptr;
                if (!err) err = MAC_ERR_CUDA;
                return;
            }
            cudaGraphDestroy(gr);
            std::memcpy(g.key, key, sizeof(key));
            g.kernels = c->issued - before;
            c->issued = before;   // captured, not launched yet
        }
        if (cudaGraphLaunch(g.exec, c->stream) != cudaSuccess) {
            set_last_cuda_error(cudaGetLastError(), "cudaGraphLaunch", __FILE__, __LINE__);
            err = MAC_ERR_CUDA;
            return;
        }
        c->issued += g.kernels;
    }
    // timing spans (level 0 only)
    cudaEvent_t next_event() {
        if (H->ev_used < H->ev_pool.size()) return H->ev_pool[H->ev_used++];
        cudaEvent_t e = nullptr;
        if (cudaEventCreate(&e) != cudaSuccess) {
            set_last_cuda_error(cudaGetLastError(), "cudaEventCreate", __FILE__, __LINE__);
            err = MAC_ERR_CUDA;
            return nullptr;
        }
        H->ev_pool.push_back(e);
        ++H->ev_used;
        return e;
    }
    bool span_on(int l) const { return c->o.timing && l == 0 && !err; }
    cudaEvent_t span_begin() {
        cudaEvent_t a = next_event();
        if (a) cudaEventRecord(a, c->stream);
        return a;
    }
    void span_end(cudaEvent_t a, int cls, long long issued_before) {
        cudaEvent_t b = next_event();
        if (!a || !b) return;
        cudaEventRecord(b, c->stream);
        H->spans.push_back(HgState::Span{cls, (int)(c->issued - issued_before), a, b});
    }
    void defect(int l, const T* phi, const T* f, T* r) {
        const bool tm = span_on(l) && std::is_same<T, double>::value;
        const long long before = c->issued;
        cudaEvent_t a = tm ? span_begin() : nullptr;
        defect_launch(l, phi, f, r);
        if (tm) span_end(a, MAC_KT_RESID, before);
    }
    void defect_launch(int l, const T* phi, const T* f, T* r) {
        const hg::LevT<T>& L = lev(l);
        if (dense3() && (L.nn[0] + 1) / 2 * ((L.nn[1] + 1) / 2) > kSlabThreads) {
            // the fine levels (those the Gauss-Seidel sweeps by tiles): by tiles
            const int ntx = (L.n[0] + (geo.per[0] ? 0 : 1) + kDefX - 1) / kDefX;
            const int nty = (L.n[1] + (geo.per[1] ? 0 : 1) + kDefY - 1) / kDefY;
            const int nzu = L.n[2] + (geo.per[2] ? 0 : 1);
            const dim3 grid((unsigned)(ntx * nty), (unsigned)nzu);
            auto kern = iso(l) ? k_hg_defect_tile<T, true> : k_hg_defect_tile<T, false>;
            kern<<<grid, kDefThreads, deftile_smem<T>(), c->stream>>>(geo, L, ntx, phi, f, r);
        } else if (dense3() && iso(l))
            k_hg_defect3<T, true><<<blocks(nn(l)), kThreads, 0, c->stream>>>(geo, lev(l), phi, f, r, nn(l));
        else if (dense3())
            k_hg_defect3<T, false><<<blocks(nn(l)), kThreads, 0, c->stream>>>(geo, lev(l), phi, f, r, nn(l));
        else
            k_hg_defect<T><<<blocks(nn(l)), kThreads, 0, c->stream>>>(geo, lev(l), phi, f, r, nn(l));
        launched();
    }
    // nu Gauss-Seidel sweeps in the colour order.  Levels whose in-slab colours fit one block
    // (one node per thread, at most kSlabThreads) sweep by slabs (k_hg_gs_slab, two launches a
    // sweep, one block per slab); finer 3-D dense levels by tiles (k_hg_gs_tile, two launches
    // a sweep: one block per slab would leave most SMs idle there, 128 blocks at 256^3);
    // others (cross stencil, fine 2-D levels) one launch per colour.  All three are the same
    // update sequence.
    void gs(int l, T* phi, const T* f, int nu) {
        const bool tm = span_on(l);
        const long long before = c->issued;
        cudaEvent_t a = tm ? span_begin() : nullptr;
        gs_launch(l, phi, f, nu);
        if (tm) span_end(a, MAC_KT_SMOOTH, before);
    }
    void gs_launch(int l, T* phi, const T* f, int nu) {
        const int dm = geo.dm;
        const hg::LevT<T>& L = lev(l);
        const int ns = L.nn[dm - 1];
        const int per_slab = (L.nn[0] + 1) / 2 * (dm == 3 ? (L.nn[1] + 1) / 2 : 1);
        if (per_slab > kSlabThreads && dense3()) {
            gs_tiled(l, phi, f, nu);
            return;
        }
        if (per_slab > kSlabThreads) {
            for (int s = 0; s < nu; ++s)
                for (int colour = 0; colour < (1 << dm); ++colour) {
                    const long m = hg::colour_count(geo, L, colour);
                    k_hg_gs<T><<<blocks(m), kThreads, 0, c->stream>>>(geo, L, colour, phi, f, m);
                    launched();
                }
            return;
        }
        int threads = 32;
        while (threads < per_slab) threads <<= 1;
        for (int s = 0; s < nu; ++s)
            for (int sp = 0; sp < 2; ++sp) {
                const int nb = (ns - sp + 1) / 2;
                if (nb <= 0) continue;
                if (dense3())
                    k_hg_gs_slab<T, true><<<nb, threads, 0, c->stream>>>(geo, L, sp, phi, f);
                else
                    k_hg_gs_slab<T, false><<<nb, threads, 0, c->stream>>>(geo, L, sp, phi, f);
                launched();
            }
    }
    // nu sweeps of the tiled Gauss-Seidel (fine 3-D dense levels), two launches a sweep,
    // alternating between phi and the level's second array (a copy back after an odd count)
    void gs_tiled(int l, T* phi, const T* f, int nu) {
        const hg::LevT<T>& L = lev(l);
        T* alt = HgAccess<T>::alt(H->L[l]);
        if (!alt) {   // prepare_tiles runs before the cycles are captured
            err = MAC_ERR_CUDA;
            return;
        }
        const int ntx = (L.n[0] + (geo.per[0] ? 0 : 1) + kTileX - 1) / kTileX;
        const int nty = (L.n[1] + (geo.per[1] ? 0 : 1) + kTileY - 1) / kTileY;
        const int nzu = L.n[2] + (geo.per[2] ? 0 : 1);
        const dim3 grid((unsigned)(ntx * nty), (unsigned)((nzu + 1) / 2));
        T* cur = phi;
        T* nxt = alt;
        auto kern = iso(l) ? k_hg_gs_tile<T, true> : k_hg_gs_tile<T, false>;
        for (int s = 0; s < nu; ++s) {
            kern<<<grid, kTileThreads, tile_smem<T>(), c->stream>>>(geo, L, 0, ntx, cur, cur, nxt, f);
            launched();
            kern<<<grid, kTileThreads, tile_smem<T>(), c->stream>>>(geo, L, 1, ntx, cur, nxt, nxt, f);
            launched();
            T* tmp = cur;
            cur = nxt;
            nxt = tmp;
        }
        if (cur != phi &&
            cudaMemcpyAsync(phi, cur, (size_t)nn(l) * sizeof(T), cudaMemcpyDeviceToDevice, c->stream) !=
                cudaSuccess)
            err = MAC_ERR_CUDA;
    }
    // Levels that sweep with the tiled kernel: their second phi array (zeroed) and the kernel's
    // shared-memory limit, set up outside any stream capture.
    void prepare_tiles() {
        if (err || !dense3()) return;
        {   // (per call, a few host calls: a process-wide flag would skip a second device)
            // the largest shared-memory carveout (a hint; the kernel runs with any)
            cudaFuncSetAttribute(k_hg_gs_tile<T, false>, cudaFuncAttributePreferredSharedMemoryCarveout,
                                 (int)cudaSharedmemCarveoutMaxShared);
            cudaFuncSetAttribute(k_hg_gs_tile<T, true>, cudaFuncAttributePreferredSharedMemoryCarveout,
                                 (int)cudaSharedmemCarveoutMaxShared);
            (void)cudaGetLastError();   // (a refused hint leaves no error behind)
            if (cudaFuncSetAttribute(k_hg_gs_tile<T, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)tile_smem<T>()) != cudaSuccess ||
                cudaFuncSetAttribute(k_hg_gs_tile<T, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)tile_smem<T>()) != cudaSuccess) {
                set_last_cuda_error(cudaGetLastError(), "cudaFuncSetAttribute", __FILE__, __LINE__);
                err = MAC_ERR_CUDA;
                return;
            }
        }
        for (int l = 0; l < nlev; ++l) {
            const hg::LevT<T>& L = lev(l);
            if ((L.nn[0] + 1) / 2 * ((L.nn[1] + 1) / 2) <= kSlabThreads) continue;
            T*& alt = HgAccess<T>::alt(H->L[l]);
            if (alt) continue;
            if (hg_alloc(H, &alt, (size_t)nn(l)) ||
                cudaMemsetAsync(alt, 0, (size_t)nn(l) * sizeof(T), c->stream) != cudaSuccess) {
                alt = nullptr;
                err = MAC_ERR_ALLOC;
                return;
            }
        }
    }
    void bottom_gs(int l, T* phi, const T* f, int nu) {
        if (H->binv && l == (int)H->L.size() - 1) {
            // the exact solve replaces the sweeps (the inverse is built with the coefficients)
            k_hg_bottom_exact<T><<<1, kExactThreads, 0, c->stream>>>(H->bM, H->bnode, H->binv, f, phi);
        } else {
            k_hg_bottom<T><<<1, 1024, 0, c->stream>>>(geo, lev(l), phi, f, nu, nn(l));
        }
        launched();
    }
    void restrict_to(int lc, const T* rF, T* fK) {
        k_hg_restrict<T><<<blocks(nn(lc)), kThreads, 0, c->stream>>>(geo, lev(lc - 1), lev(lc), rF, fK, nn(lc));
        launched();
    }
    void prolong(int lc, const T* eK, T* phiF) {
        if (geo.dm == 3)
            k_hg_prolong3<T><<<blocks(nn(lc)), kThreads, 0, c->stream>>>(geo, lev(lc), lev(lc - 1), eK, phiF, nn(lc));
        else
            k_hg_prolong<T><<<blocks(nn(lc - 1)), kThreads, 0, c->stream>>>(geo, lev(lc), lev(lc - 1), eK, phiF,
                                                                              nn(lc - 1));
        launched();
    }
    void zero(int l, T* x) {
        if (!err && cudaMemsetAsync(x, 0, sizeof(T) * nn(l), c->stream) != cudaSuccess) {
            set_last_cuda_error(cudaGetLastError(), "cudaMemsetAsync", __FILE__, __LINE__);
            err = MAC_ERR_CUDA;
        }
    }
    void finish(int l, T* x) {
        k_hg_finish<T><<<blocks(nn(l)), kThreads, 0, c->stream>>>(geo, lev(l), x, nn(l));
        launched();
    }
    void reduce(int l, const T* x) {
        const int nb = std::min(kReduceBlocks, blocks(nn(l)));
        k_hg_reduce<T><<<nb, kThreads, 0, c->stream>>>(geo, lev(l), x, H->part, nn(l));
        launched();
        k_hg_reduce_finish<<<1, kThreads, 0, c->stream>>>(H->part, nb, H->out);
        launched();
    }
    double unknown_max(int l, const T* x) {
        reduce(l, x);
        if (err) return NAN;
        if (cudaMemcpyAsync(H->h_out, H->out, 5 * sizeof(double), cudaMemcpyDeviceToHost, c->stream) != cudaSuccess ||
            cudaStreamSynchronize(c->stream) != cudaSuccess) {
            set_last_cuda_error(cudaGetLastError(), "hg reduction", __FILE__, __LINE__);
            err = MAC_ERR_CUDA;
            return NAN;
        }
        return H->h_out[2] > 0.0 ? NAN : H->h_out[1];
    }
    void sub_unknown_mean(int l, T* x) {
        reduce(l, x);
        k_hg_sub_mean<T><<<blocks(nn(l)), kThreads, 0, c->stream>>>(geo, lev(l), x, H->out + 4, nn(l));
        launched();
    }
};

// FP64 executor: the multigrid, the projection steps and the hand-over to the FP32 cycles.
struct HgExec : HgMg<double> {
    int proj_type = hg::kRegular;
    double dt = 1.0;
    double* unew = nullptr;
    const double* uold = nullptr;
    double* gpi = nullptr;
    const double* rhohalf = nullptr;
    double* pi = nullptr;
    const double* b0 = nullptr;
    const double* nodalrhs = nullptr;
    hg::Wall wall{nullptr, {-1, -1, -1, -1, -1, -1}};
    int alt = 0;

    void uvec() {
        k_hg_uvec<<<blocks(nc(0)), kThreads, 0, c->stream>>>(geo, nc(0), proj_type, dt, 1.0 / dt, unew,
                                                            uold, gpi, rhohalf, b0, alt, H->L[0].sig);
        launched();
    }
    int build_levels() {
        for (size_t l = 1; l < H->L.size(); ++l) {
            k_hg_coarsen<<<blocks(nc((int)l)), kThreads, 0, c->stream>>>(geo, lev((int)l - 1), lev((int)l),
                                                                       H->L[l].sig, nc((int)l));
            launched();
        }
        if (H->binv) {
            k_hg_bottom_inverse<<<1, kExactThreads, 0, c->stream>>>(
                geo, lev((int)H->L.size() - 1), H->bM, H->bnode, H->bmap, singular ? 1 : 0, H->binv);
            launched();
        }
        return err;
    }
    void sig_to_single() {
        for (size_t l = 0; l < H->L.size(); ++l) {
            k_hg_sig_single<<<blocks(nc((int)l)), kThreads, 0, c->stream>>>(H->L[l].sig, H->L[l].sig32,
                                                                          nc((int)l));
            launched();
        }
    }
    void to_single(const double* r, float* r32) {
        k_hg_to_single<<<blocks(nn(0)), kThreads, 0, c->stream>>>(r, r32, nn(0));
        launched();
    }
    void accumulate(double* phi, const float* e) {
        k_hg_accumulate<<<blocks(nn(0)), kThreads, 0, c->stream>>>(geo, lev(0), phi, e, nn(0));
        launched();
    }
    void divu() {
        k_hg_divu<<<blocks(nn(0)), kThreads, 0, c->stream>>>(geo, lev(0), unew, b0, nodalrhs, wall,
                                                            buf(0, hg::kF), nn(0));
        launched();
    }
    void update() {
        k_hg_update<<<blocks(nc(0)), kThreads, 0, c->stream>>>(geo, lev(0), proj_type, dt, 1.0 / dt,
                                                              buf(0, hg::kPhi), unew, uold, gpi, rhohalf,
                                                              b0, alt, nc(0));
        launched();
        k_hg_update_pi<<<blocks(nn(0)), kThreads, 0, c->stream>>>(lev(0), proj_type, dt, buf(0, hg::kPhi),
                                                                 pi, nn(0));
        launched();
    }
};

// FP32 copies of the hierarchy for the mixed-precision solve (allocated on first use).
int hg_ensure_single(mac_ctx* c) {
    HgState* H = c->hgs;
    if (H->L[0].sig32) return MAC_OK;
    for (HgState::Level& S : H->L) {
        int rc = hg_alloc(H, &S.sig32, (size_t)S.nc);
        for (int b = 0; b < hg::kNumBufs && !rc; ++b) rc = hg_alloc(H, &S.buf32[b], (size_t)S.nn);
        if (rc) return rc;
        for (int d = 0; d < 3; ++d) {
            S.lev32.n[d] = S.lev.n[d];
            S.lev32.nn[d] = S.lev.nn[d];
            S.lev32.h[d] = S.lev.h[d];
        }
        S.lev32.sig = S.sig32;
        hg::set_dense_weights(H->geo.dm, S.lev32);
    }
    return MAC_OK;
}

}  // namespace

// The nodal projection on whole-domain device arrays (arguments validated by the caller); fills
// the solve fields of *st and returns the status code.
// Offsets of the context's inflow faces in a wall array (hg::Wall): face f = 2 d + side in that
// order, each holding its cells (the face's other directions, Fortran order); returns the total
// length (0: no inflow face).
long hg_wall_layout(const mac_ctx* c, long off[6]) {
    long tot = 0;
    for (int f = 0; f < 6; ++f) {
        off[f] = -1;
        const int d = f >> 1;
        if (d >= c->dm || !((f & 1) ? c->inflow_hi[d] : c->inflow_lo[d])) continue;
        long m = 1;
        for (int e = 0; e < c->dm; ++e)
            if (e != d) m *= c->n[e];
        off[f] = tot;
        tot += m;
    }
    return tot;
}

int hg_core(mac_ctx* c, int proj_type, double dt, int dense_stencil, double rel_eps,
            double* unew, const double* uold, double* gpi, const double* rhohalf, double* pi,
            const double* beta0_cart, const double* nodalrhs, const double* wall, mac_stats* st) {
    int rc = MAC_OK;
    HgState* H = c->hgs;
    H->geo.dense = dense_stencil ? 1 : 0;
    const bool singular = !(H->geo.dlo[0] || H->geo.dhi[0] || H->geo.dlo[1] || H->geo.dhi[1] ||
                            H->geo.dlo[2] || H->geo.dhi[2]);
    HgExec ex;
    ex.c = c;
    ex.H = H;
    ex.nlev = (int)H->L.size();
    ex.geo = H->geo;
    ex.singular = singular;
    ex.proj_type = proj_type;
    ex.dt = dt;
    ex.unew = unew;
    ex.uold = uold;
    ex.gpi = gpi;
    ex.rhohalf = rhohalf;
    ex.pi = pi;
    ex.b0 = beta0_cart;
    ex.nodalrhs = nodalrhs;
    if (hg_wall_layout(c, ex.wall.off) > 0) {
        if (!wall) return MAC_ERR_INVALID;
        ex.wall.w = wall;
    }
    ex.alt = (proj_type != hg::kInitial && proj_type != hg::kDivuIters && c->o.use_alt_energy_fix) ? 1 : 0;
    // rhohalf and beta0 must be positive and finite
    if (cudaMemsetAsync(H->flag, 0, sizeof(int), c->stream) != cudaSuccess) rc = MAC_ERR_CUDA;
    if (!rc) {
        k_hg_check<<<blocks_for(H->L[0].nc, c->sms), kThreads, 0, c->stream>>>(rhohalf, beta0_cart, H->flag,
                                                                            H->L[0].nc);
        ex.launched();
        if (cudaMemcpyAsync(H->h_flag, H->flag, sizeof(int), cudaMemcpyDeviceToHost, c->stream) != cudaSuccess ||
            cudaStreamSynchronize(c->stream) != cudaSuccess) {
            set_last_cuda_error(cudaGetLastError(), "hg density check", __FILE__, __LINE__);
            rc = MAC_ERR_CUDA;
        }
        if (!rc && ex.err) rc = ex.err;
        if (!rc && *H->h_flag) rc = MAC_ERR_BAD_DENSITY;
    }
    hg::SolveStats S{};
    H->spans.clear();
    H->ev_used = 0;
    cudaEventRecord(c->ev[0], c->stream);
    const double eps = rel_eps > 0.0 ? rel_eps : 1e-12;
    const bool mixed = c->o.precision == MAC_PREC_MIXED;
    if (!rc && mixed) rc = hg_ensure_single(c);
    if (!rc) {
        if (mixed) {
            // FP32 V-cycles (kMixedInner per FP64 refinement step) under FP64 refinement
            HgMg<float> ex32;
            ex32.c = c;
            ex32.H = H;
            ex32.nlev = ex.nlev;
            ex32.geo = ex.geo;
            ex32.singular = singular;
            rc = hg::project_mixed(ex, ex32, eps, c->o.max_vcycles, c->o.nu1, c->o.nu2,
                                   kMixedInner, &S);
        } else {
            rc = hg::project(ex, eps, c->o.max_vcycles, c->o.nu1, c->o.nu2, &S);
        }
        if (rc == 1) rc = MAC_ERR_NOT_CONVERGED;
        if (rc == -1) rc = MAC_ERR_NONFINITE;
    }
    cudaEventRecord(c->ev[2], c->stream);
    if (cudaStreamSynchronize(c->stream) != cudaSuccess && !rc) {
        set_last_cuda_error(cudaGetLastError(), "cudaStreamSynchronize", __FILE__, __LINE__);
        rc = MAC_ERR_CUDA;
    }
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, c->ev[0], c->ev[2]) == cudaSuccess) st->solve_ms = ms;
    for (const HgState::Span& sp : H->spans) {   // timing: the level-0 launch classes
        float t = 0.f;
        if (cudaEventElapsedTime(&t, sp.a, sp.b) != cudaSuccess) continue;
        c->ktime_ms[sp.cls] += t;
        c->ktime_launches[sp.cls] += sp.launches;
    }
    H->spans.clear();
    cudaGetLastError();
    st->vcycles = S.cycles;
    st->nlevels = (int)H->L.size();
    st->fnorm = S.fnorm;
    st->resid0 = S.resid0;
    st->rel_resid = S.rel_resid;
    st->nhist = S.nhist;
    for (int q = 0; q < S.nhist && q < 64; ++q) st->hist[q] = S.hist[q];
    return rc;
}


namespace {

int hg_check_args(const mac_ctx* c, int proj_type, double dt, bool have_uold) {
    if (proj_type < hg::kInitial || proj_type > hg::kRegular) return MAC_ERR_INVALID;
    if (proj_type == hg::kPressureIters && !have_uold) return MAC_ERR_INVALID;
    if ((proj_type == hg::kPressureIters || proj_type == hg::kRegular) && !(dt > 0.0))
        return MAC_ERR_INVALID;
    // the colour-parallel sweeps need even periodic extents (same-colour nodes uncoupled)
    for (int d = 0; d < c->dm; ++d)
        if (c->bc_lo[d] == MAC_BC_PER && (c->n[d] & 1)) return MAC_ERR_UNSUPPORTED;
    // node and cell coordinates are formed in 32-bit arithmetic
    long nodes = 1;
    for (int d = 0; d < c->dm; ++d) nodes *= (long)c->n[d] + 1;
    if (nodes >= (1L << 31)) return MAC_ERR_TOO_LARGE;
    return MAC_OK;
}

// Descriptor of box b of the context's layout as a fab with ng ghosts, cell- or node-centred.
hg::Fab hg_fab(const mac_ctx* c, int b, int ng, int nodal) {
    hg::Fab F{};
    long cnt = 1;
    for (int d = 0; d < 3; ++d) {
        if (d >= c->dm) {
            F.ext[d] = 1;
            continue;
        }
        F.lo[d] = c->box_lo[3 * b + d] - c->g.domain_lo[d];
        F.hi[d] = c->box_hi[3 * b + d] - c->g.domain_lo[d];
        F.ext[d] = F.hi[d] - F.lo[d] + 1 + nodal + 2 * ng;
        cnt *= F.ext[d];
    }
    F.ng = ng;
    F.nodal = nodal;
    F.count = cnt;
    return F;
}

template <typename T>
int hg_grow(T** p, size_t* cap, size_t need, bool pinned) {
    if (need <= *cap) return MAC_OK;
    if (*p) {
        if (pinned)
            cudaFreeHost(*p);
        else
            cudaFree(*p);
    }
    *p = nullptr;
    *cap = 0;
    const cudaError_t e = pinned ? cudaMallocHost((void**)p, need * sizeof(T))
                                 : cudaMalloc((void**)p, need * sizeof(T));
    if (e != cudaSuccess) {
        cudaGetLastError();
        return MAC_ERR_ALLOC;
    }
    *cap = need;
    return MAC_OK;
}

// Per-box entry: gather the fabs into whole-domain arrays, project, scatter unew, gpi and pi.
int hg_fabs(mac_ctx* c, int ptr_kind, int proj_type, double dt, int dense_stencil, double rel_eps,
            double* const* unew, int ng_u, const double* const* uold, int ng_uo,
            double* const* gpi, int ng_gp, const double* const* rhohalf, int ng_rho,
            double* const* pi, int ng_pi, const double* const* beta0_cart, int ng_b0,
            const double* const* nodalrhs, int ng_nr, mac_stats* st) {
    HgState* H = c->hgs;
    const int dm = c->dm;
    const int nb = c->g.nboxes;
    const bool host = ptr_kind == MAC_PTR_HOST;
    const long nc = H->L[0].nc, nn = H->L[0].nn;
    int rc = MAC_OK;
    if (!H->fu) {
        rc = hg_alloc(H, &H->fu, (size_t)dm * nc);
        if (!rc) rc = hg_alloc(H, &H->fuo, (size_t)dm * nc);
        if (!rc) rc = hg_alloc(H, &H->fg, (size_t)dm * nc);
        if (!rc) rc = hg_alloc(H, &H->frho, (size_t)nc);
        if (!rc) rc = hg_alloc(H, &H->fpi, (size_t)nn);
        if (!rc) rc = hg_alloc(H, &H->fb0, (size_t)nc);
        if (!rc) rc = hg_alloc(H, &H->fnr, (size_t)nn);
        if (rc) return rc;
    }
    // arrays of this call: (fabs, ng, nodal, ncomp, whole-domain array, scattered back)
    struct Arr {
        const double* const* fabs;
        int ng, nodal, ncomp;
        double* dst;
        bool back;
    };
    Arr arrs[7] = {{(const double* const*)unew, ng_u, 0, dm, H->fu, true},
                   {uold, ng_uo, 0, dm, H->fuo, false},
                   {(const double* const*)gpi, ng_gp, 0, dm, H->fg, true},
                   {rhohalf, ng_rho, 0, 1, H->frho, false},
                   {(const double* const*)pi, ng_pi, 1, 1, H->fpi, true},
                   {beta0_cart, ng_b0, 0, 1, H->fb0, false},
                   {nodalrhs, ng_nr, 1, 1, H->fnr, false}};
    size_t ntab = 0, nstage = 0;
    for (const Arr& A : arrs) {
        if (!A.fabs) continue;
        ntab += nb;
        for (int b = 0; b < nb; ++b) nstage += (size_t)hg_fab(c, b, A.ng, A.nodal).count * A.ncomp;
    }
    if (ntab > H->tab_cap) {
        MAC_CUDA_TRY(cudaStreamSynchronize(c->stream));
        size_t cap = H->tab_cap;
        rc = hg_grow(&H->h_tab, &cap, ntab, true);
        if (!rc) {
            size_t cap2 = H->tab_cap;
            rc = hg_grow(&H->d_tab, &cap2, ntab, false);
        }
        if (rc) {
            H->tab_cap = 0;   // one of the two tables may be gone: regrow both next call
            return rc;
        }
        H->tab_cap = ntab;
    }
    if (host) {
        MAC_CUDA_TRY(cudaStreamSynchronize(c->stream));
        rc = hg_grow(&H->staging, &H->staging_cap, std::max<size_t>(nstage, 1), false);
        if (rc) return rc;
    }
    size_t tcur = 0, scur = 0;
    size_t tab_at[7] = {0, 0, 0, 0, 0, 0, 0};
    const hg::Lev L0 = H->L[0].lev;
    for (int k = 0; k < 7; ++k) {
        const Arr& A = arrs[k];
        if (!A.fabs) continue;
        hg::Fab* T = H->h_tab + tcur;
        long maxc = 1;
        for (int b = 0; b < nb; ++b) {
            hg::Fab F = hg_fab(c, b, A.ng, A.nodal);
            const size_t elems = (size_t)F.count * A.ncomp;
            if (host) {
                double* region = H->staging + scur;
                scur += elems;
                MAC_CUDA_TRY(cudaMemcpyAsync(region, A.fabs[b], elems * sizeof(double),
                                             cudaMemcpyHostToDevice, c->stream));
                F.src = region;
                F.dst = region;
            } else {
                F.src = A.fabs[b];
                F.dst = const_cast<double*>(A.fabs[b]);
            }
            T[b] = F;
            maxc = std::max(maxc, F.count);
        }
        MAC_CUDA_TRY(cudaMemcpyAsync(H->d_tab + tcur, T, (size_t)nb * sizeof(hg::Fab),
                                     cudaMemcpyHostToDevice, c->stream));
        const dim3 grid((unsigned)std::min<long>((maxc + kThreads - 1) / kThreads, 1024), (unsigned)nb);
        k_hg_fabs_gather<<<grid, kThreads, 0, c->stream>>>(H->geo, L0, H->d_tab + tcur, A.ncomp,
                                                           A.nodal ? nn : nc, A.dst);
        MAC_CUDA_TRY(cudaGetLastError());
        ++c->issued;
        tab_at[k] = tcur;
        tcur += (size_t)nb;
    }
    long woff[6];
    const long nwall = hg_wall_layout(c, woff);
    if (nwall > 0) {
        MAC_CUDA_TRY(cudaStreamSynchronize(c->stream));   // (the buffer may be regrown)
        rc = hg_grow(&H->fwall, &H->fwall_cap, (size_t)nwall, false);
        if (rc) return rc;
        hg::Wall W{H->fwall, {woff[0], woff[1], woff[2], woff[3], woff[4], woff[5]}};
        long maxf = 1;
        for (int b = 0; b < nb; ++b)
            for (int d = 0; d < dm; ++d) {
                long m = 1;
                for (int e = 0; e < dm; ++e)
                    if (e != d) m *= (long)c->box_hi[3 * b + e] - c->box_lo[3 * b + e] + 1;
                maxf = std::max(maxf, m);
            }
        const dim3 grid((unsigned)std::min<long>((maxf + kThreads - 1) / kThreads, 1024), (unsigned)nb,
                        (unsigned)(2 * dm));
        k_hg_fabs_wall<<<grid, kThreads, 0, c->stream>>>(
            dm, L0, W, H->d_tab + tab_at[0],
            proj_type == hg::kPressureIters ? H->d_tab + tab_at[1] : nullptr,
            beta0_cart ? H->d_tab + tab_at[5] : nullptr, ng_b0 >= 1 ? 1 : 0, dt, H->fwall);
        MAC_CUDA_TRY(cudaGetLastError());
        ++c->issued;
    }
    const int solve_rc = hg_core(c, proj_type, dt, dense_stencil, rel_eps, H->fu,
                                 uold ? H->fuo : nullptr, H->fg, H->frho, H->fpi,
                                 beta0_cart ? H->fb0 : nullptr, nodalrhs ? H->fnr : nullptr,
                                 nwall > 0 ? H->fwall : nullptr, st);
    if (solve_rc != MAC_OK && solve_rc != MAC_ERR_NOT_CONVERGED) return solve_rc;
    for (int k = 0; k < 7; ++k) {
        const Arr& A = arrs[k];
        if (!A.fabs || !A.back) continue;
        long maxc = 1;
        for (int b = 0; b < nb; ++b) maxc = std::max(maxc, H->h_tab[tab_at[k] + b].count);
        const dim3 grid((unsigned)std::min<long>((maxc + kThreads - 1) / kThreads, 1024), (unsigned)nb);
        k_hg_fabs_scatter<<<grid, kThreads, 0, c->stream>>>(H->geo, L0, H->d_tab + tab_at[k], A.ncomp,
                                                            A.nodal ? nn : nc, A.dst);
        MAC_CUDA_TRY(cudaGetLastError());
        ++c->issued;
        if (host)
            for (int b = 0; b < nb; ++b) {
                const hg::Fab& F = H->h_tab[tab_at[k] + b];
                MAC_CUDA_TRY(cudaMemcpyAsync(const_cast<double*>(A.fabs[b]), F.src,
                                             (size_t)F.count * A.ncomp * sizeof(double),
                                             cudaMemcpyDeviceToHost, c->stream));
            }
    }
    MAC_CUDA_TRY(cudaStreamSynchronize(c->stream));
    return solve_rc;
}

}  // namespace

}  // namespace mac

using namespace mac;

extern "C" {

int mac_hgproject_dense(mac_ctx* c, int proj_type, double dt, int dense_stencil, double rel_eps,
                        double* unew, const double* uold, double* gpi, const double* rhohalf,
                        double* pi, const double* beta0_cart, const double* nodalrhs,
                        mac_stats* stats) {
    return mac_hgproject_dense_inflow(c, proj_type, dt, dense_stencil, rel_eps, unew, uold, gpi,
                                      rhohalf, pi, beta0_cart, nodalrhs, nullptr, stats);
}

int mac_hgproject_dense_inflow(mac_ctx* c, int proj_type, double dt, int dense_stencil,
                               double rel_eps, double* unew, const double* uold, double* gpi,
                               const double* rhohalf, double* pi, const double* beta0_cart,
                               const double* nodalrhs, const double* inflow_wall,
                               mac_stats* stats) {
    mac_stats local;
    mac_stats* st = stats ? stats : &local;
    std::memset(st, 0, sizeof(*st));
    if (!c || !unew || !gpi || !rhohalf || !pi) return st->status = MAC_ERR_INVALID;
    long woff[6];
    if ((hg_wall_layout(c, woff) > 0) != (inflow_wall != nullptr)) return st->status = MAC_ERR_INVALID;
    int rc = hg_check_args(c, proj_type, dt, uold != nullptr);
    if (rc) return st->status = rc;
    const auto t0 = std::chrono::steady_clock::now();
    begin_call_stats(c, st);
    rc = hg_ensure(c);
    if (!rc)
        rc = hg_core(c, proj_type, dt, dense_stencil, rel_eps, unew, uold, gpi, rhohalf, pi,
                     beta0_cart, nodalrhs, inflow_wall, st);
    st->status = rc;
    st->total_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    end_call_stats(c, st);
    report_call(c, "hgproject_dense", st);
    return rc;
}


int mac_hgproject(mac_ctx* c, int ptr_kind, int proj_type, double dt, int dense_stencil,
                  double rel_eps, double* const* unew, int ng_u, const double* const* uold,
                  int ng_uo, double* const* gpi, int ng_gp, const double* const* rhohalf,
                  int ng_rho, double* const* pi, int ng_pi, const double* const* beta0_cart,
                  int ng_b0, const double* const* nodalrhs, int ng_nr, mac_stats* stats) {
    mac_stats local;
    mac_stats* st = stats ? stats : &local;
    std::memset(st, 0, sizeof(*st));
    if (!c || !unew || !gpi || !rhohalf || !pi) return st->status = MAC_ERR_INVALID;
    if (ptr_kind != MAC_PTR_HOST && ptr_kind != MAC_PTR_DEVICE) return st->status = MAC_ERR_INVALID;
    if (ng_u < 0 || ng_uo < 0 || ng_gp < 0 || ng_rho < 0 || ng_pi < 0 || ng_b0 < 0 || ng_nr < 0)
        return st->status = MAC_ERR_INVALID;
    for (int b = 0; b < c->g.nboxes; ++b)
        if (!unew[b] || !gpi[b] || !rhohalf[b] || !pi[b] || (uold && !uold[b]) ||
            (beta0_cart && !beta0_cart[b]) || (nodalrhs && !nodalrhs[b]))
            return st->status = MAC_ERR_INVALID;
    int rc = hg_check_args(c, proj_type, dt, uold != nullptr);
    if (rc) return st->status = rc;
    // inflow faces take their wall values from the first ghost layer outside them
    long woff[6];
    if (hg_wall_layout(c, woff) > 0 &&
        (ng_u < 1 || (proj_type == hg::kPressureIters && ng_uo < 1)))
        return st->status = MAC_ERR_INVALID;
    const auto t0 = std::chrono::steady_clock::now();
    begin_call_stats(c, st);
    rc = hg_ensure(c);
    if (!rc)
        rc = hg_fabs(c, ptr_kind, proj_type, dt, dense_stencil, rel_eps, unew, ng_u, uold, ng_uo,
                     gpi, ng_gp, rhohalf, ng_rho, pi, ng_pi, beta0_cart, ng_b0, nodalrhs, ng_nr, st);
    st->status = rc;
    st->total_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    end_call_stats(c, st);
    report_call(c, "hgproject", st);
    return rc;
}

int mac_ctx_set_inflow(mac_ctx* c, const int* lo_inflow, const int* hi_inflow) {
    if (!c) return MAC_ERR_INVALID;
    int lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};
    for (int d = 0; d < c->dm; ++d) {
        lo[d] = lo_inflow ? lo_inflow[d] : 0;
        hi[d] = hi_inflow ? hi_inflow[d] : 0;
        if (lo[d] < 0 || lo[d] > 1 || hi[d] < 0 || hi[d] > 1) return MAC_ERR_INVALID;
        // an inlet is a Neumann face of the pressure (Source/define_bc_tower.f90:329-392)
        if ((lo[d] && c->bc_lo[d] != MAC_BC_NEU) || (hi[d] && c->bc_hi[d] != MAC_BC_NEU))
            return MAC_ERR_INVALID;
    }
    for (int d = 0; d < 3; ++d) {
        c->inflow_lo[d] = lo[d];
        c->inflow_hi[d] = hi[d];
    }
    return MAC_OK;
}

}  // extern "C"
