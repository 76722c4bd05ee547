// Yee kernels behind update_E/H/S/F/G/J (the drop-in path).
//
// Bulk kernels (the normal path): thread (y, z) of the plane marches a chunk of consecutive
// x planes. The x-neighbour plane is carried in registers (the E update's x-1 values are the
// previous iteration's own loads; the H update's x+1 loads become the next iteration's own),
// and every load of iteration x+1 (fields, neighbours, dt/eps, CPML psi) is issued before
// iteration x computes and stores, so each warp keeps a full iteration of loads in flight.
// Consecutive threads walk consecutive z, so a warp's loads are contiguous runs. CPML faces
// are handled per axis: x-faces are uniform for a whole iteration, y- and z-face membership
// is fixed for a thread, so the depth index and the coefficients of y/z faces are looked up
// once per thread. One thread advances all three components of a cell, where the reference
// launches 3N work-items and idles two thirds of them (opencl_fdtd/kernels/common.cl:21-25).
//
// Generic kernels: one thread per cell with the faces applied in list order; used only when
// two CPML faces of one axis overlap (the order of their terms then matters).
//
// This translation unit is compiled with --fmad=false and every expression keeps the
// reference's operation order, so results match the reference kernel text bit for bit in
// float32 and float64.
#include "yee_common.cuh"
#include "yee_device.cuh"
#include "yee_launch.h"

namespace fdtd {



// ---- CPML contribution of one face ---------------------------------------------------------
template <typename R, bool ETYPE, int AX>
__device__ __forceinline__ void pml_face(const FaceK<R> &f, int ir, uint32_t x, uint32_t y,
                                         uint32_t z, uint32_t sy, uint32_t sz,
                                         R &d_xy, R &d_xz, R &d_yx, R &d_yz, R &d_zx, R &d_zy,
                                         R &px, R &py, R &pz)
{
    const uint32_t ip = psi_index<AX>((uint32_t)ir, (uint32_t)f.T, x, y, z, sy, sz);
    R su, sv;
    face_update<R, ETYPE, AX>(f.p0[ir], f.p1[ir], f.p2[ir], f.psi_u[ip], f.psi_v[ip], su, sv,
                              d_xy, d_xz, d_yx, d_yz, d_zx, d_zy, px, py, pz);
    f.psi_u[ip] = su;
    f.psi_v[ip] = sv;
}

template <typename R, bool ETYPE>
__device__ __forceinline__ void pml_all(const YeeK<R> &k, uint32_t x, uint32_t y, uint32_t z,
                                        R &d_xy, R &d_xz, R &d_yx, R &d_yz, R &d_zx, R &d_zy,
                                        R &px, R &py, R &pz)
{
#pragma unroll
    for (int f = 0; f < 6; ++f) {
        if (f >= k.nface) break;
        const FaceK<R> &fc = k.face[f];
        if (fc.axis == 0) {
            const int ir = pml_ir(fc.pol, fc.T, k.sx, x);
            if (ir >= 0)
                pml_face<R, ETYPE, 0>(fc, ir, x, y, z, k.sy, k.sz, d_xy, d_xz, d_yx, d_yz, d_zx, d_zy, px, py, pz);
        } else if (fc.axis == 1) {
            const int ir = pml_ir(fc.pol, fc.T, k.sy, y);
            if (ir >= 0)
                pml_face<R, ETYPE, 1>(fc, ir, x, y, z, k.sy, k.sz, d_xy, d_xz, d_yx, d_yz, d_zx, d_zy, px, py, pz);
        } else {
            const int ir = pml_ir(fc.pol, fc.T, k.sz, z);
            if (ir >= 0)
                pml_face<R, ETYPE, 2>(fc, ir, x, y, z, k.sy, k.sz, d_xy, d_xz, d_yx, d_yz, d_zx, d_zy, px, py, pz);
        }
    }
}

// ---- generic E-type cell: update_E / update_F (update_e.cl) --------------------------------
template <typename R>
__device__ __forceinline__ void cell_e(const YeeK<R> &k, uint32_t x, uint32_t y, uint32_t z)
{
    const uint32_t i = (x * k.sy + y) * k.sz + z;
    const uint64_t N = k.N;
    const R *__restrict__ Qx = k.Q;
    const R *__restrict__ Qy = k.Q + N;
    const R *__restrict__ Qz = k.Q + 2 * N;
    // minus neighbours with periodic wrap (common.cl:75-81)
    const uint32_t imx = x ? i - k.syz : i + (k.sx - 1u) * k.syz;
    const uint32_t imy = y ? i - k.sz : i + (k.sy - 1u) * k.sz;
    const uint32_t imz = z ? i - 1u : i + (k.sz - 1u);

    const R qx = Qx[i], qy = Qy[i], qz = Qz[i];
    R n_xy = Qx[imy], n_xz = Qx[imz];
    R n_yx = Qy[imx], n_yz = Qy[imz];
    R n_zx = Qz[imx], n_zy = Qz[imy];
    if (k.bloch_mask) {
        // wrapped neighbour of the complex pair times conj(beta)
        const R *Rx = k.Rp, *Ry = k.Rp + N, *Rz = k.Rp + 2 * N;
        if ((k.bloch_mask & 1) && x == 0) {
            n_yx = n_yx * k.br[0] + Ry[imx] * k.bi[0];
            n_zx = n_zx * k.br[0] + Rz[imx] * k.bi[0];
        }
        if ((k.bloch_mask & 2) && y == 0) {
            n_xy = n_xy * k.br[1] + Rx[imy] * k.bi[1];
            n_zy = n_zy * k.br[1] + Rz[imy] * k.bi[1];
        }
        if ((k.bloch_mask & 4) && z == 0) {
            n_xz = n_xz * k.br[2] + Rx[imz] * k.bi[2];
            n_yz = n_yz * k.br[2] + Ry[imz] * k.bi[2];
        }
    }
    R ix = k.inv_d, iy = k.inv_d, iz = k.inv_d;
    if (k.inv_tab[0]) { ix = k.inv_tab[0][x]; iy = k.inv_tab[1][y]; iz = k.inv_tab[2][z]; }
    // backward differences (update_e.cl:39-46)
    R d_xy = (qx - n_xy) * iy;
    R d_xz = (qx - n_xz) * iz;
    R d_yx = (qy - n_yx) * ix;
    R d_yz = (qy - n_yz) * iz;
    R d_zx = (qz - n_zx) * ix;
    R d_zy = (qz - n_zy) * iy;

    R px = R(0), py = R(0), pz = R(0);
    if (k.nface) pml_all<R, true>(k, x, y, z, d_xy, d_xz, d_yx, d_yz, d_zx, d_zy, px, py, pz);

    R *Px = k.P, *Py = k.P + N, *Pz = k.P + 2 * N;
    R cx, cy, cz;
    if (k.coef) {
        cx = k.coef[i]; cy = k.coef[N + i]; cz = k.coef[2 * N + i];
    } else {
        cx = k.dt / k.mat[i]; cy = k.dt / k.mat[N + i]; cz = k.dt / k.mat[2 * N + i];
    }
    // update_e.cl:105-107
    Px[i] = Px[i] + cx * ((d_zy - d_yz) + px);
    Py[i] = Py[i] + cy * ((d_xz - d_zx) + py);
    Pz[i] = Pz[i] + cz * ((d_yx - d_xy) + pz);
}

// ---- generic H-type cell: update_H / update_G (update_h.cl) --------------------------------
template <typename R, bool MU, bool POYNT>
__device__ __forceinline__ void cell_h(const YeeK<R> &k, uint32_t x, uint32_t y, uint32_t z)
{
    const uint32_t i = (x * k.sy + y) * k.sz + z;
    const uint64_t N = k.N;
    const R *__restrict__ Qx = k.Q;
    const R *__restrict__ Qy = k.Q + N;
    const R *__restrict__ Qz = k.Q + 2 * N;
    // plus neighbours with periodic wrap (common.cl:82-84)
    const uint32_t ipx = (x + 1u < k.sx) ? i + k.syz : i - (k.sx - 1u) * k.syz;
    const uint32_t ipy = (y + 1u < k.sy) ? i + k.sz : i - (k.sy - 1u) * k.sz;
    const uint32_t ipz = (z + 1u < k.sz) ? i + 1u : i - (k.sz - 1u);

    const R qx = Qx[i], qy = Qy[i], qz = Qz[i];
    const R r_xy = Qx[ipy], r_xz = Qx[ipz];
    const R r_yx = Qy[ipx], r_yz = Qy[ipz];
    const R r_zx = Qz[ipx], r_zy = Qz[ipy];
    R n_xy = r_xy, n_xz = r_xz, n_yx = r_yx, n_yz = r_yz, n_zx = r_zx, n_zy = r_zy;
    if (k.bloch_mask) {
        // wrapped neighbour of the complex pair times beta
        const R *Rx = k.Rp, *Ry = k.Rp + N, *Rz = k.Rp + 2 * N;
        if ((k.bloch_mask & 1) && x + 1u == k.sx) {
            n_yx = r_yx * k.br[0] + Ry[ipx] * k.bi[0];
            n_zx = r_zx * k.br[0] + Rz[ipx] * k.bi[0];
        }
        if ((k.bloch_mask & 2) && y + 1u == k.sy) {
            n_xy = r_xy * k.br[1] + Rx[ipy] * k.bi[1];
            n_zy = r_zy * k.br[1] + Rz[ipy] * k.bi[1];
        }
        if ((k.bloch_mask & 4) && z + 1u == k.sz) {
            n_xz = r_xz * k.br[2] + Rx[ipz] * k.bi[2];
            n_yz = r_yz * k.br[2] + Ry[ipz] * k.bi[2];
        }
    }
    R ix = k.inv_d, iy = k.inv_d, iz = k.inv_d;
    if (k.inv_tab[0]) { ix = k.inv_tab[0][x]; iy = k.inv_tab[1][y]; iz = k.inv_tab[2][z]; }
    // forward differences (update_h.cl:36-43)
    R d_xy = (n_xy - qx) * iy;
    R d_xz = (n_xz - qx) * iz;
    R d_yx = (n_yx - qy) * ix;
    R d_yz = (n_yz - qy) * iz;
    R d_zx = (n_zx - qz) * ix;
    R d_zy = (n_zy - qz) * iy;

    R px = R(0), py = R(0), pz = R(0);
    if (k.nface) pml_all<R, false>(k, x, y, z, d_xy, d_xz, d_yx, d_yz, d_zx, d_zy, px, py, pz);

    R *Px = k.P, *Py = k.P + N, *Pz = k.P + 2 * N;
    const R ox = Px[i], oy = Py[i], oz = Pz[i];
    R hx, hy, hz;
    if (MU) {
        R cx, cy, cz;
        if (k.coef) {
            cx = k.coef[i]; cy = k.coef[N + i]; cz = k.coef[2 * N + i];
        } else {
            cx = k.dt / k.mat[i]; cy = k.dt / k.mat[N + i]; cz = k.dt / k.mat[2 * N + i];
        }
        hx = ox - cx * ((d_zy - d_yz) - px);
        hy = oy - cy * ((d_xz - d_zx) - py);
        hz = oz - cz * ((d_yx - d_xy) - pz);
    } else {
        // update_h.cl:129-131
        hx = ox - k.dt * ((d_zy - d_yz) - px);
        hy = oy - k.dt * ((d_xz - d_zx) - py);
        hz = oz - k.dt * ((d_yx - d_xy) - pz);
    }
    Px[i] = hx;
    Py[i] = hy;
    Pz[i] = hz;
    if (POYNT) {
        // E averaged in space, H in time (update_h.cl:63-70, 135-137), six products in plane
        // order xy, yz, zx, xz, yx, zy (update_h.cl:142-154)
        const R ahx = hx + ox, ahy = hy + oy, ahz = hz + oz;
        R *o = k.oS;
        o[0 * N + i] = (r_yx + qy) * ahz;
        o[3 * N + i] = (-(r_zx + qz)) * ahy;
        o[1 * N + i] = (r_zy + qz) * ahx;
        o[4 * N + i] = (-(r_xy + qx)) * ahz;
        o[2 * N + i] = (r_xz + qx) * ahy;
        o[5 * N + i] = (-(r_yz + qy)) * ahx;
    }
}

// ---- generic full-grid kernels (overlapping CPML faces) ------------------------------------
template <typename R>
__global__ void __launch_bounds__(BLOCK) k_generic_e(const YeeK<R> k)
{
    const uint32_t j = blockIdx.x * BLOCK + threadIdx.x;
    if (j >= k.syz) return;
    const uint32_t y = k.dsz.div(j);
    cell_e<R>(k, k.xbeg + blockIdx.y, y, j - y * k.sz);
}

template <typename R, bool MU, bool POYNT>
__global__ void __launch_bounds__(BLOCK) k_generic_h(const YeeK<R> k)
{
    const uint32_t j = blockIdx.x * BLOCK + threadIdx.x;
    if (j >= k.syz) return;
    const uint32_t y = k.dsz.div(j);
    cell_h<R, MU, POYNT>(k, k.xbeg + blockIdx.y, y, j - y * k.sz);
}

// ---- bulk kernels ----------------------------------------------------------------------------
// Values one E-type iteration reads, loaded one iteration ahead.
template <typename R>
struct ELoad {
    R hx, hy, hz;                 // Q at x
    R nxy, nxz, nyz, nzy;         // Q_x(y-1), Q_x(z-1), Q_y(z-1), Q_z(y-1)
    R bxy, bzy, bxz, byz;         // Bloch partner at the wrapped y / z neighbour
    R ex, ey, ez;                 // P at x
    R cx, cy, cz;                 // dt/eps at x
    R xu, xv, yu, yv, zu, zv;     // psi of the faces the cell is in
};

// block shape of the bulk E kernel: EBLOCK threads, at least EMINB blocks per SM
constexpr int EBLOCK = 256, EMINB = 3;

// Forms of the bulk E kernel (FDTD_TUNE_E_FORM): 0 loads the next plane one iteration ahead
// (80 registers, three blocks per SM); 1 (the default) loads each plane when it is updated, at
// four blocks per SM (64 registers). Same arithmetic in both. On the 395x345x73 grid: 0.110
// and 0.105 ms (a per-plane form at five blocks per SM spilled 80 B and took 0.131 ms).
template <int FORM>
struct EForm {
    static constexpr bool prefetch = FORM == 0;
    static constexpr int min_blocks = FORM == 0 ? EMINB : 4;
};

template <typename R, int DX, bool BLOCH, int FORM>
__global__ void __launch_bounds__(EBLOCK, EForm<FORM>::min_blocks) k_bulk_e(const YeeK<R> k)
{
    constexpr bool PF = EForm<FORM>::prefetch;
    grid_dependency_sync();
    const uint32_t j = blockIdx.x * EBLOCK + threadIdx.x;
    if (j >= k.syz) return;
    const uint32_t sx = k.sx, sy = k.sy, sz = k.sz, syz = k.syz;
    const uint32_t y = k.dsz.div(j);
    const uint32_t z = j - y * sz;
    const uint32_t xa = k.xbeg + blockIdx.y * (uint32_t)k.xchunk;
    const uint32_t xb = min(xa + (uint32_t)k.xchunk, k.xend);
    const uint64_t N = k.N;
    const R *__restrict__ Qx = k.Q;
    const R *__restrict__ Qy = k.Q + N;
    const R *__restrict__ Qz = k.Q + 2 * N;
    const R *__restrict__ Cx = k.coef;
    const R *__restrict__ Cy = k.coef + N;
    const R *__restrict__ Cz = k.coef + 2 * N;
    R *__restrict__ Px = k.P;
    R *__restrict__ Py = k.P + N;
    R *__restrict__ Pz = k.P + 2 * N;
    // y/z minus neighbours with periodic wrap (common.cl:75-81), fixed for the thread
    const uint32_t dmy = y ? 0u - sz : (sy - 1u) * sz;
    const uint32_t dmz = z ? 0xffffffffu : sz - 1u;
    const bool by = BLOCH && (k.bloch_mask & 2) && y == 0;
    const bool bz = BLOCH && (k.bloch_mask & 4) && z == 0;
    const FixedFace<R> fy = fixed_face<R, true>(k.ax[1], sy, y);
    const FixedFace<R> fz = fixed_face<R, true>(k.ax[2], sz, z);
    R iy = k.inv_d, iz = k.inv_d;
    if (DX == 2) { iy = ldg(k.inv_tab[1] + y); iz = ldg(k.inv_tab[2] + z); }
    // a point source in this block's cells and planes (block-uniform)
    bool srcs = false;
    for (int s = 0; s < k.nsrc; ++s)
        srcs |= k.src_j[s] / (uint32_t)EBLOCK == blockIdx.x &&
                (k.src_x[s] - k.xbeg) / (uint32_t)k.xchunk == blockIdx.y;

    auto load = [&](uint32_t x, uint32_t i) {
        ELoad<R> v;
        v.hx = ldg(Qx + i); v.hy = ldg(Qy + i); v.hz = ldg(Qz + i);
        // neighbour indices in 32-bit arithmetic (dmy / dmz may be wrapped negatives)
        const uint32_t imy = i + dmy, imz = i + dmz;
        v.nxy = ldg(Qx + imy); v.nxz = ldg(Qx + imz);
        v.nyz = ldg(Qy + imz); v.nzy = ldg(Qz + imy);
        v.bxy = v.bzy = v.bxz = v.byz = R(0);
        if (by) { v.bxy = ldg(k.Rp + imy); v.bzy = ldg(k.Rp + 2 * N + imy); }
        if (bz) { v.bxz = ldg(k.Rp + imz); v.byz = ldg(k.Rp + N + imz); }
        v.ex = Px[i]; v.ey = Py[i]; v.ez = Pz[i];
        v.cx = ldg(Cx + i); v.cy = ldg(Cy + i); v.cz = ldg(Cz + i);
        v.xu = v.xv = v.yu = v.yv = v.zu = v.zv = R(0);
        const XFace<R> fx = x_face<R>(k.ax[0], sx, x);
        if (fx.ir >= 0) {
            const uint32_t ip = psi_index<0>((uint32_t)fx.ir, fx.T, x, y, z, sy, sz);
            v.xu = fx.pu[ip]; v.xv = fx.pv[ip];
        }
        if (fy.ir >= 0) {
            const uint32_t ip = psi_index<1>((uint32_t)fy.ir, fy.T, x, y, z, sy, sz);
            v.yu = fy.pu[ip]; v.yv = fy.pv[ip];
        }
        if (fz.ir >= 0) {
            const uint32_t ip = psi_index<2>((uint32_t)fz.ir, fz.T, x, y, z, sy, sz);
            v.zu = fz.pu[ip]; v.zv = fz.pv[ip];
        }
        return v;
    };

    uint32_t i = xa * syz + j;
    // x-1 plane of the first iteration, wrapped and Bloch-coupled at x = 0
    const uint32_t im = xa ? i - syz : i + (sx - 1u) * syz;
    R hy_m = ldg(Qy + im), hz_m = ldg(Qz + im);
    if (BLOCH && xa == 0 && (k.bloch_mask & 1)) {
        hy_m = hy_m * k.br[0] + ldg(k.Rp + N + im) * k.bi[0];
        hz_m = hz_m * k.br[0] + ldg(k.Rp + 2 * N + im) * k.bi[0];
    }
    ELoad<R> cur;
    if (PF) cur = load(xa, i);
    for (uint32_t x = xa; x < xb; ++x, i += syz) {
        ELoad<R> nxt;
        if (PF) {
            if (x + 1u < xb) nxt = load(x + 1u, i + syz);
        } else {
            cur = load(x, i);
        }
        R n_xy = cur.nxy, n_zy = cur.nzy, n_xz = cur.nxz, n_yz = cur.nyz;
        if (by) { n_xy = n_xy * k.br[1] + cur.bxy * k.bi[1]; n_zy = n_zy * k.br[1] + cur.bzy * k.bi[1]; }
        if (bz) { n_xz = n_xz * k.br[2] + cur.bxz * k.bi[2]; n_yz = n_yz * k.br[2] + cur.byz * k.bi[2]; }
        // backward differences (update_e.cl:39-46)
        R d_xy = cur.hx - n_xy;
        R d_xz = cur.hx - n_xz;
        R d_yx = cur.hy - hy_m;
        R d_yz = cur.hy - n_yz;
        R d_zx = cur.hz - hz_m;
        R d_zy = cur.hz - n_zy;
        if (DX != 0) {
            const R ix = (DX == 2) ? ldg(k.inv_tab[0] + x) : k.inv_d;
            d_xy = d_xy * iy; d_xz = d_xz * iz; d_yx = d_yx * ix;
            d_yz = d_yz * iz; d_zx = d_zx * ix; d_zy = d_zy * iy;
        }
        // CPML (update_e.cl:64-100): at most one face per axis
        R px = R(0), py = R(0), pz = R(0);
        const XFace<R> fx = x_face<R>(k.ax[0], sx, x);
        if (fx.ir >= 0) {
            R su, sv;
            face_update<R, true, 0>(ldg(fx.t0 + fx.ir), ldg(fx.t1 + fx.ir), ldg(fx.t2 + fx.ir),
                                    cur.xu, cur.xv, su, sv, d_xy, d_xz, d_yx, d_yz, d_zx, d_zy, px, py, pz);
            const uint32_t ip = psi_index<0>((uint32_t)fx.ir, fx.T, x, y, z, sy, sz);
            fx.pu[ip] = su; fx.pv[ip] = sv;
        }
        if (fy.ir >= 0) {
            R su, sv;
            face_update<R, true, 1>(fy.p0, fy.p1, fy.p2, cur.yu, cur.yv, su, sv,
                                    d_xy, d_xz, d_yx, d_yz, d_zx, d_zy, px, py, pz);
            const uint32_t ip = psi_index<1>((uint32_t)fy.ir, fy.T, x, y, z, sy, sz);
            fy.pu[ip] = su; fy.pv[ip] = sv;
        }
        if (fz.ir >= 0) {
            R su, sv;
            face_update<R, true, 2>(fz.p0, fz.p1, fz.p2, cur.zu, cur.zv, su, sv,
                                    d_xy, d_xz, d_yx, d_yz, d_zx, d_zy, px, py, pz);
            const uint32_t ip = psi_index<2>((uint32_t)fz.ir, fz.T, x, y, z, sy, sz);
            fz.pu[ip] = su; fz.pv[ip] = sv;
        }
        // update_e.cl:105-107
        R ex = cur.ex + cur.cx * ((d_zy - d_yz) + px);
        R ey = cur.ey + cur.cy * ((d_xz - d_zx) + py);
        R ez = cur.ez + cur.cz * ((d_yx - d_xy) + pz);
        if (srcs) {
            // the same additions, in list order, as a separate launch after the update
            for (int s = 0; s < k.nsrc; ++s) {
                if (k.src_x[s] != x || k.src_j[s] != j) continue;
                const R val = k.src_values[(int64_t)k.src_t * k.src_stride + k.src_col[s]];
                if (k.src_c[s] == 0) ex = ex + val;
                else if (k.src_c[s] == 1) ey = ey + val;
                else ez = ez + val;
            }
        }
        Px[i] = ex;
        Py[i] = ey;
        Pz[i] = ez;
        hy_m = cur.hy;
        hz_m = cur.hz;
        if (PF) cur = nxt;
    }
}

// Values one H-type iteration reads, loaded one iteration ahead.
template <typename R>
struct HLoad {
    R ex1, ey1, ez1;              // Q at x+1 (wrapped)
    R rxy, rxz, ryz, rzy;         // Q_x(y+1), Q_x(z+1), Q_y(z+1), Q_z(y+1) at x
    R bxy, bzy, bxz, byz;         // Bloch partner at the wrapped y / z neighbour
    R byx, bzx;                   // Bloch partner at the wrapped x neighbour
    R hx, hy, hz;                 // P at x
    R cx, cy, cz;                 // dt/mu at x
    R xu, xv, yu, yv, zu, zv;     // psi of the faces the cell is in
};

template <typename R, int DX, bool MU, bool POYNT, bool BLOCH>
__global__ void __launch_bounds__(BLOCK, 3) k_bulk_h(const YeeK<R> k)
{
    const uint32_t j = blockIdx.x * BLOCK + threadIdx.x;
    if (j >= k.syz) return;
    const uint32_t sx = k.sx, sy = k.sy, sz = k.sz, syz = k.syz;
    const uint32_t y = k.dsz.div(j);
    const uint32_t z = j - y * sz;
    const uint32_t xa = k.xbeg + blockIdx.y * (uint32_t)k.xchunk;
    const uint32_t xb = min(xa + (uint32_t)k.xchunk, k.xend);
    const uint64_t N = k.N;
    const R *__restrict__ Qx = k.Q;
    const R *__restrict__ Qy = k.Q + N;
    const R *__restrict__ Qz = k.Q + 2 * N;
    R *__restrict__ Px = k.P;
    R *__restrict__ Py = k.P + N;
    R *__restrict__ Pz = k.P + 2 * N;
    // y/z plus neighbours with periodic wrap (common.cl:82-84), fixed for the thread
    const uint32_t dpy = (y + 1u < sy) ? sz : 0u - (sy - 1u) * sz;
    const uint32_t dpz = (z + 1u < sz) ? 1u : 0u - (sz - 1u);
    const bool bx = BLOCH && (k.bloch_mask & 1) != 0;
    const bool by = BLOCH && (k.bloch_mask & 2) && y + 1u == sy;
    const bool bz = BLOCH && (k.bloch_mask & 4) && z + 1u == sz;
    const FixedFace<R> fy = fixed_face<R, false>(k.ax[1], sy, y);
    const FixedFace<R> fz = fixed_face<R, false>(k.ax[2], sz, z);
    R iy = k.inv_d, iz = k.inv_d;
    if (DX == 2) { iy = ldg(k.inv_tab[1] + y); iz = ldg(k.inv_tab[2] + z); }
    const R dt = k.dt;

    auto load = [&](uint32_t x, uint32_t i) {
        HLoad<R> v;
        const uint32_t i1 = (x + 1u < sx) ? i + syz : i - (sx - 1u) * syz;
        v.ex1 = ldg(Qx + i1); v.ey1 = ldg(Qy + i1); v.ez1 = ldg(Qz + i1);
        // neighbour indices in 32-bit arithmetic (dpy / dpz may be wrapped negatives)
        const uint32_t ipy = i + dpy, ipz = i + dpz;
        v.rxy = ldg(Qx + ipy); v.rxz = ldg(Qx + ipz);
        v.ryz = ldg(Qy + ipz); v.rzy = ldg(Qz + ipy);
        v.bxy = v.bzy = v.bxz = v.byz = v.byx = v.bzx = R(0);
        if (bx && x + 1u == sx) { v.byx = ldg(k.Rp + N + i1); v.bzx = ldg(k.Rp + 2 * N + i1); }
        if (by) { v.bxy = ldg(k.Rp + ipy); v.bzy = ldg(k.Rp + 2 * N + ipy); }
        if (bz) { v.bxz = ldg(k.Rp + ipz); v.byz = ldg(k.Rp + N + ipz); }
        v.hx = Px[i]; v.hy = Py[i]; v.hz = Pz[i];
        v.cx = v.cy = v.cz = R(0);
        if (MU) { v.cx = ldg(k.coef + i); v.cy = ldg(k.coef + N + i); v.cz = ldg(k.coef + 2 * N + i); }
        v.xu = v.xv = v.yu = v.yv = v.zu = v.zv = R(0);
        const XFace<R> fx = x_face<R>(k.ax[0], sx, x);
        if (fx.ir >= 0) {
            const uint32_t ip = psi_index<0>((uint32_t)fx.ir, fx.T, x, y, z, sy, sz);
            v.xu = fx.pu[ip]; v.xv = fx.pv[ip];
        }
        if (fy.ir >= 0) {
            const uint32_t ip = psi_index<1>((uint32_t)fy.ir, fy.T, x, y, z, sy, sz);
            v.yu = fy.pu[ip]; v.yv = fy.pv[ip];
        }
        if (fz.ir >= 0) {
            const uint32_t ip = psi_index<2>((uint32_t)fz.ir, fz.T, x, y, z, sy, sz);
            v.zu = fz.pu[ip]; v.zv = fz.pv[ip];
        }
        return v;
    };

    uint32_t i = xa * syz + j;
    R ex = ldg(Qx + i), ey = ldg(Qy + i), ez = ldg(Qz + i);
    HLoad<R> cur = load(xa, i);
    for (uint32_t x = xa; x < xb; ++x, i += syz) {
        HLoad<R> nxt;
        if (x + 1u < xb) nxt = load(x + 1u, i + syz);
        R n_yx = cur.ey1, n_zx = cur.ez1, n_xy = cur.rxy, n_zy = cur.rzy, n_xz = cur.rxz, n_yz = cur.ryz;
        if (bx && x + 1u == sx) { n_yx = n_yx * k.br[0] + cur.byx * k.bi[0]; n_zx = n_zx * k.br[0] + cur.bzx * k.bi[0]; }
        if (by) { n_xy = n_xy * k.br[1] + cur.bxy * k.bi[1]; n_zy = n_zy * k.br[1] + cur.bzy * k.bi[1]; }
        if (bz) { n_xz = n_xz * k.br[2] + cur.bxz * k.bi[2]; n_yz = n_yz * k.br[2] + cur.byz * k.bi[2]; }
        // forward differences (update_h.cl:36-43)
        R d_xy = n_xy - ex;
        R d_xz = n_xz - ex;
        R d_yx = n_yx - ey;
        R d_yz = n_yz - ey;
        R d_zx = n_zx - ez;
        R d_zy = n_zy - ez;
        if (DX != 0) {
            const R ix = (DX == 2) ? ldg(k.inv_tab[0] + x) : k.inv_d;
            d_xy = d_xy * iy; d_xz = d_xz * iz; d_yx = d_yx * ix;
            d_yz = d_yz * iz; d_zx = d_zx * ix; d_zy = d_zy * iy;
        }
        // CPML (update_h.cl:80-116): at most one face per axis
        R px = R(0), py = R(0), pz = R(0);
        const XFace<R> fx = x_face<R>(k.ax[0], sx, x);
        if (fx.ir >= 0) {
            R su, sv;
            face_update<R, false, 0>(ldg(fx.t0 + fx.ir), ldg(fx.t1 + fx.ir), ldg(fx.t2 + fx.ir),
                                     cur.xu, cur.xv, su, sv, d_xy, d_xz, d_yx, d_yz, d_zx, d_zy, px, py, pz);
            const uint32_t ip = psi_index<0>((uint32_t)fx.ir, fx.T, x, y, z, sy, sz);
            fx.pu[ip] = su; fx.pv[ip] = sv;
        }
        if (fy.ir >= 0) {
            R su, sv;
            face_update<R, false, 1>(fy.p0, fy.p1, fy.p2, cur.yu, cur.yv, su, sv,
                                     d_xy, d_xz, d_yx, d_yz, d_zx, d_zy, px, py, pz);
            const uint32_t ip = psi_index<1>((uint32_t)fy.ir, fy.T, x, y, z, sy, sz);
            fy.pu[ip] = su; fy.pv[ip] = sv;
        }
        if (fz.ir >= 0) {
            R su, sv;
            face_update<R, false, 2>(fz.p0, fz.p1, fz.p2, cur.zu, cur.zv, su, sv,
                                     d_xy, d_xz, d_yx, d_yz, d_zx, d_zy, px, py, pz);
            const uint32_t ip = psi_index<2>((uint32_t)fz.ir, fz.T, x, y, z, sy, sz);
            fz.pu[ip] = su; fz.pv[ip] = sv;
        }
        R hx, hy, hz;
        if (MU) {
            hx = cur.hx - cur.cx * ((d_zy - d_yz) - px);
            hy = cur.hy - cur.cy * ((d_xz - d_zx) - py);
            hz = cur.hz - cur.cz * ((d_yx - d_xy) - pz);
        } else {
            // update_h.cl:129-131
            hx = cur.hx - dt * ((d_zy - d_yz) - px);
            hy = cur.hy - dt * ((d_xz - d_zx) - py);
            hz = cur.hz - dt * ((d_yx - d_xy) - pz);
        }
        Px[i] = hx;
        Py[i] = hy;
        Pz[i] = hz;
        if (POYNT) {
            // E averaged in space with the plain wrapped neighbours, H in time
            // (update_h.cl:63-70, 135-137); planes xy, yz, zx, xz, yx, zy (update_h.cl:142-154)
            const R ahx = hx + cur.hx, ahy = hy + cur.hy, ahz = hz + cur.hz;
            R *o = k.oS;
            o[0 * N + i] = (cur.ey1 + ey) * ahz;
            o[3 * N + i] = (-(cur.ez1 + ez)) * ahy;
            o[1 * N + i] = (cur.rzy + ez) * ahx;
            o[4 * N + i] = (-(cur.rxy + ex)) * ahz;
            o[2 * N + i] = (cur.rxz + ex) * ahy;
            o[5 * N + i] = (-(cur.ryz + ey)) * ahx;
        }
        ex = cur.ex1;
        ey = cur.ey1;
        ez = cur.ez1;
        cur = nxt;
    }
}

// ---- update_S (update_s.cl:33-36) ----------------------------------------------------------
template <typename R>
struct SLoad {
    R xy, yz, zx, xz, yx, zy;     // oS planes at x
    R xy_y, xz_z, yz_z, zy_y;     // oS_xy(y-1), oS_xz(z-1), oS_yz(z-1), oS_zy(y-1)
};

template <typename R>
__global__ void __launch_bounds__(BLOCK) k_bulk_s(const SK<R> k)
{
    const uint32_t j = blockIdx.x * BLOCK + threadIdx.x;
    if (j >= k.syz) return;
    const uint32_t sx = k.sx, sy = k.sy, sz = k.sz, syz = k.syz;
    const uint32_t y = k.dsz.div(j);
    const uint32_t z = j - y * sz;
    const uint32_t xa = k.xbeg + blockIdx.y * (uint32_t)k.xchunk;
    const uint32_t xb = min(xa + (uint32_t)k.xchunk, k.xend);
    const uint64_t N = k.N;
    const R *__restrict__ oxy = k.oS;
    const R *__restrict__ oyz = k.oS + N;
    const R *__restrict__ ozx = k.oS + 2 * N;
    const R *__restrict__ oxz = k.oS + 3 * N;
    const R *__restrict__ oyx = k.oS + 4 * N;
    const R *__restrict__ ozy = k.oS + 5 * N;
    R *__restrict__ Sx = k.S;
    R *__restrict__ Sy = k.S + N;
    R *__restrict__ Sz = k.S + 2 * N;
    const uint32_t dmy = y ? 0u - sz : (sy - 1u) * sz;
    const uint32_t dmz = z ? 0xffffffffu : sz - 1u;
    auto load = [&](uint32_t i) {
        SLoad<R> v;
        v.xy = ldg(oxy + i); v.yz = ldg(oyz + i); v.zx = ldg(ozx + i);
        v.xz = ldg(oxz + i); v.yx = ldg(oyx + i); v.zy = ldg(ozy + i);
        const uint32_t imy = i + dmy, imz = i + dmz;   // 32-bit wrap arithmetic
        v.xy_y = ldg(oxy + imy); v.xz_z = ldg(oxz + imz);
        v.yz_z = ldg(oyz + imz); v.zy_y = ldg(ozy + imy);
        return v;
    };
    uint32_t i = xa * syz + j;
    const uint32_t im = xa ? i - syz : i + (sx - 1u) * syz;
    R yx_m = ldg(oyx + im), zx_m = ldg(ozx + im);
    const R sf = k.sf;
    SLoad<R> cur = load(i);
    for (uint32_t x = xa; x < xb; ++x, i += syz) {
        SLoad<R> nxt;
        if (x + 1u < xb) nxt = load(i + syz);
        Sx[i] = (((cur.xy + cur.xz) + cur.xy_y) + cur.xz_z) * sf;
        Sy[i] = (((cur.yz + cur.yx) + cur.yz_z) + yx_m) * sf;
        Sz[i] = (((cur.zx + cur.zy) + zx_m) + cur.zy_y) * sf;
        yx_m = cur.yx;
        zx_m = cur.zx;
        cur = nxt;
    }
}

// ---- dt / material coefficients (the quotient update_e.cl:105-107 forms per cell) ----------
template <typename R>
__global__ void __launch_bounds__(BLOCK) k_prepare(const PrepK<R> k)
{
    for (uint64_t i = (uint64_t)blockIdx.x * BLOCK + threadIdx.x; i < k.n;
         i += (uint64_t)gridDim.x * BLOCK)
        k.out[i] = k.dt / k.mat[i];
}

// ---- update_J (update_j.cl:23-32), launched over the box only -------------------------------
template <typename R>
__global__ void __launch_bounds__(BLOCK) k_fieldsrc(const JK<R> k)
{
    const uint32_t t = blockIdx.x * BLOCK + threadIdx.x;
    const uint32_t nbox = k.nx * k.ny * k.nz;
    if (t >= nbox) return;
    const uint32_t bx = k.dnyz.div(t);
    const uint32_t rem = t - bx * (k.ny * k.nz);
    const uint32_t by = k.dnz.div(rem);
    const uint32_t bz = rem - by * k.nz;
    const uint32_t i = ((k.x0 + bx) * k.sy + (k.y0 + by)) * k.sz + (k.z0 + bz);
#pragma unroll
    for (int q = 0; q < 3; ++q) {
        const uint64_t o = (uint64_t)q * k.N + i;
        k.E[o] = k.E[o] + (k.c * k.Jr[o] + k.s * k.Ji[o]);
    }
}

// ---- point sources of fdtd_run: E[index] += value (fdtd.py:168-169) ------------------------
// One thread adds every source in list order, so sources sharing a cell accumulate in the
// same order as successive host-side additions.
template <typename R>
__global__ void k_point_sources(const PointK<R> k)
{
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    for (int s = 0; s < k.n; ++s) {
        const int64_t ind = k.index[s];
        k.E[ind] = k.E[ind] + k.values[(int64_t)k.t * k.stride + k.col[s]];
    }
}

// ---- launchers ------------------------------------------------------------------------------
static inline dim3 bulk_grid(uint32_t syz, uint32_t nx, int xchunk, uint32_t block = BLOCK)
{
    return dim3((syz + block - 1) / block, (nx + (uint32_t)xchunk - 1) / (uint32_t)xchunk, 1);
}

static inline dim3 plane_grid(uint32_t syz, uint32_t nx)
{
    return dim3((syz + BLOCK - 1) / BLOCK, nx, 1);
}

template <typename R, bool BLOCH, int DX>
static void (*bulk_e_form(int form))(YeeK<R>)
{
    if (form == 1) return k_bulk_e<R, DX, BLOCH, 1>;
    return k_bulk_e<R, DX, BLOCH, 0>;
}

template <typename R, bool BLOCH>
static void (*bulk_e_kernel(int dxmode, int form))(YeeK<R>)
{
    if (dxmode == 0) return bulk_e_form<R, BLOCH, 0>(form);
    if (dxmode == 1) return bulk_e_form<R, BLOCH, 1>(form);
    return bulk_e_form<R, BLOCH, 2>(form);
}

template <typename R>
cudaError_t launch_yee_e(const YeeK<R> &k, cudaStream_t st, bool pdl)
{
    if (k.xend <= k.xbeg) return cudaSuccess;
    if (!k.bulk) {
        k_generic_e<R><<<plane_grid(k.syz, k.xend - k.xbeg), BLOCK, 0, st>>>(k);
        return cudaGetLastError();
    }
    const dim3 g = bulk_grid(k.syz, k.xend - k.xbeg, k.xchunk, EBLOCK);
    const int f = k.eform;
    return launch_dependent(k.bloch_mask ? bulk_e_kernel<R, true>(k.dxmode, f) : bulk_e_kernel<R, false>(k.dxmode, f),
                            g, EBLOCK, st, pdl, k);
}

template <typename R, int DX, bool BLOCH>
static void bulk_h(const YeeK<R> &k, bool mu, bool poynting, cudaStream_t st)
{
    const dim3 g = bulk_grid(k.syz, k.xend - k.xbeg, k.xchunk);
    if (mu) {
        if (poynting) k_bulk_h<R, DX, true, true, BLOCH><<<g, BLOCK, 0, st>>>(k);
        else k_bulk_h<R, DX, true, false, BLOCH><<<g, BLOCK, 0, st>>>(k);
    } else {
        if (poynting) k_bulk_h<R, DX, false, true, BLOCH><<<g, BLOCK, 0, st>>>(k);
        else k_bulk_h<R, DX, false, false, BLOCH><<<g, BLOCK, 0, st>>>(k);
    }
}

template <typename R, int DX>
static void bulk_h_dispatch(const YeeK<R> &k, bool mu, bool poynting, cudaStream_t st)
{
    if (k.bloch_mask) bulk_h<R, DX, true>(k, mu, poynting, st);
    else bulk_h<R, DX, false>(k, mu, poynting, st);
}

template <typename R>
cudaError_t launch_yee_h(const YeeK<R> &k, bool mu, bool poynting, cudaStream_t st)
{
    if (k.xend <= k.xbeg) return cudaSuccess;
    if (!k.bulk) {
        const dim3 g = plane_grid(k.syz, k.xend - k.xbeg);
        if (mu) {
            if (poynting) k_generic_h<R, true, true><<<g, BLOCK, 0, st>>>(k);
            else k_generic_h<R, true, false><<<g, BLOCK, 0, st>>>(k);
        } else {
            if (poynting) k_generic_h<R, false, true><<<g, BLOCK, 0, st>>>(k);
            else k_generic_h<R, false, false><<<g, BLOCK, 0, st>>>(k);
        }
        return cudaGetLastError();
    }
    if (k.dxmode == 0) bulk_h_dispatch<R, 0>(k, mu, poynting, st);
    else if (k.dxmode == 1) bulk_h_dispatch<R, 1>(k, mu, poynting, st);
    else bulk_h_dispatch<R, 2>(k, mu, poynting, st);
    return cudaGetLastError();
}

template <typename R>
cudaError_t launch_poynting(const SK<R> &k, cudaStream_t st)
{
    if (k.xend <= k.xbeg) return cudaSuccess;
    k_bulk_s<R><<<bulk_grid(k.syz, k.xend - k.xbeg, k.xchunk), BLOCK, 0, st>>>(k);
    return cudaGetLastError();
}

template <typename R>
cudaError_t launch_prepare(const PrepK<R> &k, cudaStream_t st)
{
    if (k.n == 0) return cudaSuccess;
    const uint64_t want = (k.n + BLOCK - 1) / BLOCK;
    const unsigned g = (unsigned)(want < 65535ull * 16 ? want : 65535ull * 16);
    k_prepare<R><<<g, BLOCK, 0, st>>>(k);
    return cudaGetLastError();
}

template <typename R>
cudaError_t launch_fieldsrc(const JK<R> &k, cudaStream_t st)
{
    const uint32_t n = k.nx * k.ny * k.nz;
    if (n == 0) return cudaSuccess;
    k_fieldsrc<R><<<(n + BLOCK - 1) / BLOCK, BLOCK, 0, st>>>(k);
    return cudaGetLastError();
}

template <typename R>
cudaError_t launch_point_sources(const PointK<R> &k, cudaStream_t st)
{
    if (k.n <= 0) return cudaSuccess;
    k_point_sources<R><<<1, 32, 0, st>>>(k);
    return cudaGetLastError();
}

#define FDTD_INSTANTIATE(R)                                                              \
    template cudaError_t launch_yee_e<R>(const YeeK<R> &, cudaStream_t, bool);         \
    template cudaError_t launch_yee_h<R>(const YeeK<R> &, bool, bool, cudaStream_t);   \
    template cudaError_t launch_poynting<R>(const SK<R> &, cudaStream_t);              \
    template cudaError_t launch_prepare<R>(const PrepK<R> &, cudaStream_t);            \
    template cudaError_t launch_fieldsrc<R>(const JK<R> &, cudaStream_t);              \
    template cudaError_t launch_point_sources<R>(const PointK<R> &, cudaStream_t);

FDTD_INSTANTIATE(float)
FDTD_INSTANTIATE(double)

}  // namespace fdtd
