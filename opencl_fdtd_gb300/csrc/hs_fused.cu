// H update and Poynting vector in one pass (the multi-step path of fdtd_run).
//
// The drop-in update_H writes the six Poynting products oS (24 B per cell) and update_S reads
// them back with their minus neighbours (36 B per cell). Here the H update reads H from one
// buffer and writes it to another (ping-pong, with the H-side CPML arrays), so every value it
// reads is read-only for the whole launch; S is then formed in the same launch:
//   * a block owns whole z rows [y0, y0 + rows) and marches a chunk of x planes; it also
//     evaluates the row y0 - 1, owned by another block, without writing it (its inputs are
//     read-only, so the values are the owner's); after each plane's H update the products go
//     to shared memory;
//   * S at (x, y, z) takes the products of its own cell, of z-1 (same row), of y-1 (the row
//     before, in the block) and of x-1 (the thread's previous plane, kept in registers).
// With update_E in place this gives a step of 96 B per cell plus 32 B per CPML face-cell,
// the algorithmic figure of the two-pass accounting (84 + 12). Per-cell arithmetic and its
// order are those of update_H and update_S (compiled with --fmad=false), so fields and S are
// bit-identical to the per-call loop. Bloch boundaries are handled by the per-update path.
#include "yee_common.cuh"
#include "yee_device.cuh"
#include "hs_fused.h"

namespace fdtd {

// CPML face of one axis for a cell: depth ir (-1 outside) and side (0 = 'n', 1 = 'p').
// Thickness and psi pointers are read from the launch parameters on use; the coefficients of
// a thread's y and z faces, fixed for its march, are loaded once into registers (cy, cz),
// those of the x face on use.
struct HSF {
    int ir, side;
};

template <typename R>
__device__ __forceinline__ HSF hs_face(const HSAxis<R> &a, uint32_t s, uint32_t c)
{
    HSF f;
    f.ir = -1;
    f.side = 0;
    if (c < (uint32_t)a.Tn) {
        f.ir = (int)c;
    } else if (a.Tp && c >= s - (uint32_t)a.Tp) {
        f.ir = (int)(s - 1u - c);
        f.side = 1;
    }
    return f;
}

template <typename R>
__device__ __forceinline__ uint32_t hs_T(const HSAxis<R> &a, const HSF &f)
{
    return (uint32_t)(f.side ? a.Tp : a.Tn);
}

template <typename R>
__device__ __forceinline__ const R *hs_tab(const HSAxis<R> &a, const HSF &f, int c)
{
    return f.side ? a.tab[1][c] : a.tab[0][c];
}

template <typename R>
__device__ __forceinline__ const R *hs_A(const HSAxis<R> &a, const HSF &f, int c)
{
    return f.side ? a.A[1][c] : a.A[0][c];
}

template <typename R>
__device__ __forceinline__ R *hs_B(const HSAxis<R> &a, const HSF &f, int c)
{
    return f.side ? a.B[1][c] : a.B[0][c];
}

// Everything one H evaluation at (x, y, z) reads.
template <typename R>
struct HSLoad {
    R ex, ey, ez;                 // E at the cell
    R ey1, ez1;                   // E_y, E_z at x+1 (wrapped)
    R rxy, rzy;                   // E_x, E_z at y+1 (wrapped)
    R rxz, ryz;                   // E_x, E_y at z+1 (wrapped)
    R hx, hy, hz;                 // old H at the cell
    R cx, cy, cz;                 // dt/mu at the cell
    R xu, xv, yu, yv, zu, zv;     // old psi_H of the faces the cell is in
};

template <typename R, bool MU>
__device__ __forceinline__ void hs_load(const HSK<R> &k, uint32_t x, uint32_t i, uint32_t dpy,
                                        uint32_t dpz, const HSF &fx, const HSF &fy,
                                        const HSF &fz, uint32_t y, uint32_t z, HSLoad<R> &v)
{
    const uint64_t N = k.N;
    const uint32_t sx = k.sx, syz = k.syz;
    const R *Ex = k.E, *Ey = k.E + N, *Ez = k.E + 2 * N;
    const uint32_t i1 = (x + 1u < sx) ? i + syz : i - (sx - 1u) * syz;
    const uint32_t ipy = i + dpy, ipz = i + dpz;   // 32-bit wrap arithmetic
    v.ex = ldg(Ex + i); v.ey = ldg(Ey + i); v.ez = ldg(Ez + i);
    v.ey1 = ldg(Ey + i1); v.ez1 = ldg(Ez + i1);
    v.rxy = ldg(Ex + ipy); v.rzy = ldg(Ez + ipy);
    v.rxz = ldg(Ex + ipz); v.ryz = ldg(Ey + ipz);
    v.hx = ldg(k.HA + i); v.hy = ldg(k.HA + N + i); v.hz = ldg(k.HA + 2 * N + i);
    v.cx = v.cy = v.cz = R(0);
    if (MU) { v.cx = ldg(k.cm + i); v.cy = ldg(k.cm + N + i); v.cz = ldg(k.cm + 2 * N + i); }
    v.xu = v.xv = v.yu = v.yv = v.zu = v.zv = R(0);
    if (fx.ir >= 0) {
        const uint32_t ip = psi_index<0>((uint32_t)fx.ir, hs_T(k.ax[0], fx), x, y, z, k.sy, k.sz);
        v.xu = ldg(hs_A(k.ax[0], fx, 0) + ip); v.xv = ldg(hs_A(k.ax[0], fx, 1) + ip);
    }
    if (fy.ir >= 0) {
        const uint32_t ip = psi_index<1>((uint32_t)fy.ir, hs_T(k.ax[1], fy), x, y, z, k.sy, k.sz);
        v.yu = ldg(hs_A(k.ax[1], fy, 0) + ip); v.yv = ldg(hs_A(k.ax[1], fy, 1) + ip);
    }
    if (fz.ir >= 0) {
        const uint32_t ip = psi_index<2>((uint32_t)fz.ir, hs_T(k.ax[2], fz), x, y, z, k.sy, k.sz);
        v.zu = ldg(hs_A(k.ax[2], fz, 0) + ip); v.zv = ldg(hs_A(k.ax[2], fz, 1) + ip);
    }
}

// H_new and the six products from loaded values (update_h.cl:36-43, 63-70, 80-155).
// wr: write H_new and the advanced psi to the B buffers.
template <typename R, int DX, bool MU>
__device__ __forceinline__ void hs_math(const HSK<R> &k, uint32_t x, uint32_t y, uint32_t z,
                                        uint32_t i, const HSF &fx, const HSF &fy,
                                        const HSF &fz, const HSLoad<R> &v, bool wr, R *os,
                                        const R *cy, const R *cz)
{
    R d_xy = v.rxy - v.ex;
    R d_xz = v.rxz - v.ex;
    R d_yx = v.ey1 - v.ey;
    R d_yz = v.ryz - v.ey;
    R d_zx = v.ez1 - v.ez;
    R d_zy = v.rzy - v.ez;
    if (DX != 0) {
        R ix = k.inv_d, iy = k.inv_d, iz = k.inv_d;
        if (DX == 2) { ix = ldg(k.inv_de[0] + x); iy = ldg(k.inv_de[1] + y); iz = ldg(k.inv_de[2] + z); }
        d_xy = d_xy * iy; d_xz = d_xz * iz; d_yx = d_yx * ix;
        d_yz = d_yz * iz; d_zx = d_zx * ix; d_zy = d_zy * iy;
    }
    R px = R(0), py = R(0), pz = R(0);
    if (fx.ir >= 0) {
        const HSAxis<R> &a = k.ax[0];
        R su, sv;
        face_update<R, false, 0>(ldg(hs_tab(a, fx, 0) + fx.ir), ldg(hs_tab(a, fx, 1) + fx.ir),
                                  ldg(hs_tab(a, fx, 2) + fx.ir), v.xu, v.xv, su, sv,
                                  d_xy, d_xz, d_yx, d_yz, d_zx, d_zy, px, py, pz);
        if (wr) {
            const uint32_t ip = psi_index<0>((uint32_t)fx.ir, hs_T(a, fx), x, y, z, k.sy, k.sz);
            hs_B(a, fx, 0)[ip] = su;
            hs_B(a, fx, 1)[ip] = sv;
        }
    }
    if (fy.ir >= 0) {
        const HSAxis<R> &a = k.ax[1];
        R su, sv;
        face_update<R, false, 1>(cy[0], cy[1], cy[2], v.yu, v.yv, su, sv,
                                  d_xy, d_xz, d_yx, d_yz, d_zx, d_zy, px, py, pz);
        if (wr) {
            const uint32_t ip = psi_index<1>((uint32_t)fy.ir, hs_T(a, fy), x, y, z, k.sy, k.sz);
            hs_B(a, fy, 0)[ip] = su;
            hs_B(a, fy, 1)[ip] = sv;
        }
    }
    if (fz.ir >= 0) {
        const HSAxis<R> &a = k.ax[2];
        R su, sv;
        face_update<R, false, 2>(cz[0], cz[1], cz[2], v.zu, v.zv, su, sv,
                                  d_xy, d_xz, d_yx, d_yz, d_zx, d_zy, px, py, pz);
        if (wr) {
            const uint32_t ip = psi_index<2>((uint32_t)fz.ir, hs_T(a, fz), x, y, z, k.sy, k.sz);
            hs_B(a, fz, 0)[ip] = su;
            hs_B(a, fz, 1)[ip] = sv;
        }
    }
    R hx, hy, hz;
    if (MU) {
        hx = v.hx - v.cx * ((d_zy - d_yz) - px);
        hy = v.hy - v.cy * ((d_xz - d_zx) - py);
        hz = v.hz - v.cz * ((d_yx - d_xy) - pz);
    } else {
        hx = v.hx - k.dt * ((d_zy - d_yz) - px);
        hy = v.hy - k.dt * ((d_xz - d_zx) - py);
        hz = v.hz - k.dt * ((d_yx - d_xy) - pz);
    }
    if (wr) {
        const uint64_t N = k.N;
        k.HB[i] = hx;
        k.HB[N + i] = hy;
        k.HB[2 * N + i] = hz;
    }
    const R ahx = hx + v.hx, ahy = hy + v.hy, ahz = hz + v.hz;
    os[0] = (v.ey1 + v.ey) * ahz;
    os[3] = (-(v.ez1 + v.ez)) * ahy;
    os[1] = (v.rzy + v.ez) * ahx;
    os[4] = (-(v.rxy + v.ex)) * ahz;
    os[2] = (v.rxz + v.ex) * ahy;
    os[5] = (-(v.ryz + v.ey)) * ahx;
}

// S at the cell of thread t from the products of one plane in shared memory (six planes of
// HS_THREADS values: xy, yz, zx, xz, yx, zy) and the thread's x-1 products (update_s.cl:33-36);
// the x-1 products become this plane's.
template <typename R>
__device__ __forceinline__ void hs_s(const HSK<R> &k, const R *q, uint32_t t, uint32_t z,
                                     uint32_t i, R &prev_yx, R &prev_zx)
{
    const uint64_t N = k.N;
    const uint32_t sz = k.sz;
    const uint32_t tz = z ? t - 1u : t + sz - 1u;  // z-1, wrapped within the row
    const R a_xy = q[t], a_yz = q[HS_THREADS + t], a_zx = q[2 * HS_THREADS + t];
    const R a_xz = q[3 * HS_THREADS + t], a_yx = q[4 * HS_THREADS + t], a_zy = q[5 * HS_THREADS + t];
    const R xy_y = q[t - sz], zy_y = q[5 * HS_THREADS + t - sz];
    const R xz_z = q[3 * HS_THREADS + tz], yz_z = q[HS_THREADS + tz];
    k.S[i] = (((a_xy + a_xz) + xy_y) + xz_z) * k.sf;
    k.S[N + i] = (((a_yz + a_yx) + yz_z) + prev_yx) * k.sf;
    k.S[2 * N + i] = (((a_zx + a_zy) + prev_zx) + zy_y) * k.sf;
    prev_yx = a_yx;
    prev_zx = a_zx;
}

// Thread t of a block works on window row w = t / sz (cell z = t % sz): row 0 is the halo row
// y0 - 1 (wrapped), whose products only feed S of row y0; rows 1..rows are the block's own
// rows y0 .. y0 + rows - 1. Every thread evaluates exactly one cell per plane, so a barrier
// waits for no extra work. The products go to shared memory slots that alternate by plane,
// which is what lets one barrier per plane suffice.
// PF: issue the next plane's loads before the current plane's arithmetic (one block per SM
// with room for both sets of registers); otherwise (two blocks per SM) they are issued after
// the products are stored, so that the last plane's are in flight during the barrier and the
// S assembly.
// The grid is one-dimensional: block b takes row block b % nrowblk and x chunk b / nrowblk (row
// blocks fastest). With dft_on one more block (the last) takes the step's DFT monitor sample
// of E, which this launch leaves unchanged; a single block keeps a grid that fills whole
// waves of resident blocks doing so.
template <typename R, int DX, bool MU, bool PF>
__global__ void __launch_bounds__(HS_THREADS, PF ? 1 : 2) k_bulk_hs(const HSK<R> k)
{
    __shared__ R sS[2][6][HS_THREADS];
    grid_dependency_sync();
    const uint32_t t = threadIdx.x;
    const uint32_t chunk = blockIdx.x / k.nrowblk;
    if (chunk >= k.nchunk) {
        const int nq = k.dft.npoint * (k.dft.nfreq > 0 ? k.dft.nfreq : 1);
        for (int q = (int)t; q < nq; q += HS_THREADS) dft_sample(k.dft, q);
        return;
    }
    const uint32_t sx = k.sx, sy = k.sy, sz = k.sz, syz = k.syz;
    const uint64_t N = k.N;
    const uint32_t y0 = (blockIdx.x - chunk * k.nrowblk) * k.rows;
    const uint32_t nrow = min(k.rows, sy - y0);
    const bool act = t < (nrow + 1u) * sz;
    const uint32_t w = act ? k.dsz.div(t) : 0u;
    const uint32_t z = act ? t - w * sz : 0u;
    const uint32_t y = w ? y0 + w - 1u : (y0 ? y0 - 1u : sy - 1u);
    const bool own = act && w > 0;
    const uint32_t j = y * sz + z;
    // chunks in descending x order start where the preceding update_E (ascending) finished, on
    // planes still in L2
    const uint32_t xa = (k.reverse ? k.nchunk - 1u - chunk : chunk) * k.xchunk;
    const uint32_t xb = min(xa + k.xchunk, sx);
    // plus neighbours (common.cl:82-84) in 32-bit wrap arithmetic
    const uint32_t dpy = (y + 1u < sy) ? sz : 0u - (sy - 1u) * sz;
    const uint32_t dpz = (z + 1u < sz) ? 1u : 0u - (sz - 1u);
    const HSF fy = hs_face<R>(k.ax[1], sy, y);
    const HSF fz = hs_face<R>(k.ax[2], sz, z);
    // CPML coefficients of the thread's y and z faces, fixed for the march
    R cy[3] = {R(0), R(0), R(0)}, cz[3] = {R(0), R(0), R(0)};
    if (fy.ir >= 0)
        for (int c = 0; c < 3; ++c) cy[c] = ldg(hs_tab(k.ax[1], fy, c) + fy.ir);
    if (fz.ir >= 0)
        for (int c = 0; c < 3; ++c) cz[c] = ldg(hs_tab(k.ax[2], fz, c) + fz.ir);

    R prev_yx = R(0), prev_zx = R(0);
    if (own) {
        // products yx, zx of plane xa - 1 (the x-1 neighbour of the chunk's first S)
        const uint32_t xp = xa ? xa - 1u : sx - 1u;
        const uint32_t ip = xp * syz + j;
        const HSF fx = hs_face<R>(k.ax[0], sx, xp);
        HSLoad<R> v;
        hs_load<R, MU>(k, xp, ip, dpy, dpz, fx, fy, fz, y, z, v);
        R os[6];
        hs_math<R, DX, MU>(k, xp, y, z, ip, fx, fy, fz, v, false, os, cy, cz);
        prev_yx = os[4];
        prev_zx = os[2];
    }
    HSLoad<R> cur;
    uint32_t i = xa * syz + j;
    if (act) hs_load<R, MU>(k, xa, i, dpy, dpz, hs_face<R>(k.ax[0], sx, xa), fy, fz, y, z, cur);
    for (uint32_t x = xa; x < xb; ++x, i += syz) {
        const HSF fx = hs_face<R>(k.ax[0], sx, x);
        const int slot = (int)(x & 1u);
        HSLoad<R> nxt;
        if (act) {
            if (PF && x + 1u < xb) hs_load<R, MU>(k, x + 1u, i + syz, dpy, dpz, hs_face<R>(k.ax[0], sx, x + 1u), fy, fz, y, z, nxt);
            R os[6];
            hs_math<R, DX, MU>(k, x, y, z, i, fx, fy, fz, cur, own, os, cy, cz);
#pragma unroll
            for (int c = 0; c < 6; ++c) sS[slot][c][t] = os[c];
            if (own && k.write_oS) {
#pragma unroll
                for (int c = 0; c < 6; ++c) k.oS[(uint64_t)c * N + i] = os[c];
            }
            // the next plane's loads fly during the barrier and the S assembly
            if (!PF && x + 1u < xb)
                hs_load<R, MU>(k, x + 1u, i + syz, dpy, dpz, hs_face<R>(k.ax[0], sx, x + 1u), fy, fz, y, z, cur);
        }
        __syncthreads();
        if (own) hs_s<R>(k, sS[slot][0], t, z, i, prev_yx, prev_zx);
        if (PF && act) cur = nxt;
    }
}

template <typename R, int DX, bool PF>
static cudaError_t launch_hs_dx(const HSK<R> &k, bool mu, dim3 g, bool pdl, cudaStream_t st)
{
    if (mu) return launch_dependent(k_bulk_hs<R, DX, true, PF>, g, HS_THREADS, st, pdl, k);
    return launch_dependent(k_bulk_hs<R, DX, false, PF>, g, HS_THREADS, st, pdl, k);
}

template <typename R, bool PF>
static cudaError_t launch_hs_pf(const HSK<R> &k, bool mu, int dxmode, dim3 g, bool pdl, cudaStream_t st)
{
    if (dxmode == 0) return launch_hs_dx<R, 0, PF>(k, mu, g, pdl, st);
    if (dxmode == 1) return launch_hs_dx<R, 1, PF>(k, mu, g, pdl, st);
    return launch_hs_dx<R, 2, PF>(k, mu, g, pdl, st);
}

template <typename R>
cudaError_t launch_hs(const HSK<R> &k, bool mu, int dxmode, bool prefetch, bool pdl, cudaStream_t st)
{
    const dim3 g(k.nrowblk * k.nchunk + (k.dft_on ? 1u : 0u), 1, 1);
    if (prefetch) return launch_hs_pf<R, true>(k, mu, dxmode, g, pdl, st);
    return launch_hs_pf<R, false>(k, mu, dxmode, g, pdl, st);
}

template cudaError_t launch_hs<float>(const HSK<float> &, bool, int, bool, bool, cudaStream_t);
template cudaError_t launch_hs<double>(const HSK<double> &, bool, int, bool, bool, cudaStream_t);

}  // namespace fdtd
