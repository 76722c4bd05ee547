// Two-pass Yee kernels behind update_E/H/S/F/G/J (the drop-in path).
//
// One thread advances one cell (all three components), so each launch covers N threads,
// where the reference launches 3N work-items and idles two thirds of them
// (opencl_fdtd/kernels/common.cl:21-25). The grid is (ceil(sy*sz / 256), sx): blockIdx.y is
// the x plane, so x-face CPML branches are uniform per block, and consecutive threads walk
// consecutive z, so every field load of a warp is one contiguous 128-byte run. Neighbour
// re-reads (z-1 and y-1 rows in L1, the x-1 plane in L2) cost no extra HBM traffic.
//
// This translation unit is compiled with --fmad=false and every expression keeps the
// reference's operation order, so results match the reference kernel text bit for bit in
// float32 and float64.
#include "yee_common.cuh"
#include "yee_launch.h"

namespace fdtd {

// ---- CPML contribution of one face ---------------------------------------------------------
// Depth index of the cell inside the face's slab, or -1 (update_e.cl:81-90). A 'p' face
// thicker than its axis never applies (the reference's unsigned s - T wraps).
__device__ __forceinline__ int pml_ir(int pol, int T, uint32_t s, uint32_t c)
{
    if (pol == 0) return (c < (uint32_t)T) ? (int)c : -1;
    if ((uint32_t)T <= s && c >= s - (uint32_t)T) return (int)(s - 1u - c);
    return -1;
}

// psi_u advances with the derivative of the v component along r and psi_v with that of the
// u component (update_e.cl:93-96); both derivatives along r are first scaled by p2 = 1/kappa.
// E-type kernels fold (psi_u, psi_v) into (P_u, P_v) with signs (-, +) for r in {x, z} and
// (+, -) for r = y (update_e.cl:73-77, 97-98); H-type kernels use the mirrored signs
// (update_h.cl:113-114).
template <typename R, bool ETYPE, int AX>
__device__ __forceinline__ void pml_face(const FaceK<R> &f, int ir, uint32_t x, uint32_t y,
                                         uint32_t z, uint32_t sy, uint32_t sz,
                                         R &d_xy, R &d_xz, R &d_yx, R &d_yz, R &d_zx, R &d_zy,
                                         R &px, R &py, R &pz)
{
    const R p0 = f.p0[ir], p1 = f.p1[ir], p2 = f.p2[ir];
    uint32_t ip;
    if (AX == 0) ip = ((uint32_t)ir * sy + y) * sz + z;
    else if (AX == 1) ip = (x * (uint32_t)f.T + (uint32_t)ir) * sz + z;
    else ip = (x * sy + y) * (uint32_t)f.T + (uint32_t)ir;
    // (dv_r, du_r): derivative along AX of the v and the u component
    R &dv = (AX == 0) ? d_zx : (AX == 1) ? d_zy : d_yz;
    R &du = (AX == 0) ? d_yx : (AX == 1) ? d_xy : d_xz;
    dv = dv * p2;
    du = du * p2;
    const R su = p0 * f.psi_u[ip] + p1 * dv;
    const R sv = p0 * f.psi_v[ip] + p1 * du;
    f.psi_u[ip] = su;
    f.psi_v[ip] = sv;
    R &pu = (AX == 0) ? py : px;
    R &pv = (AX == 2) ? py : pz;
    const bool plus_u = ETYPE ? (AX == 1) : (AX != 1);
    if (plus_u) { pu = pu + su; pv = pv - sv; }
    else        { pu = pu - su; pv = pv + sv; }
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

// ---- E-type: update_E / update_F (update_e.cl) ---------------------------------------------
template <typename R>
__global__ void __launch_bounds__(256) k_yee_e(const YeeK<R> k)
{
    const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= k.syz) return;
    const uint32_t x = blockIdx.y;
    const uint32_t y = k.dsz.div(j);
    const uint32_t z = j - y * k.sz;
    const uint32_t i = x * k.syz + j;
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
    const R *ex = k.mat, *ey = k.mat + N, *ez = k.mat + 2 * N;
    Px[i] = Px[i] + (k.dt / ex[i]) * ((d_zy - d_yz) + px);
    Py[i] = Py[i] + (k.dt / ey[i]) * ((d_xz - d_zx) + py);
    Pz[i] = Pz[i] + (k.dt / ez[i]) * ((d_yx - d_xy) + pz);
}

// ---- H-type: update_H / update_G (update_h.cl) ---------------------------------------------
template <typename R, bool MU, bool POYNT>
__global__ void __launch_bounds__(256) k_yee_h(const YeeK<R> k)
{
    const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= k.syz) return;
    const uint32_t x = blockIdx.y;
    const uint32_t y = k.dsz.div(j);
    const uint32_t z = j - y * k.sz;
    const uint32_t i = x * k.syz + j;
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
        const R *mx = k.mat, *my = k.mat + N, *mz = k.mat + 2 * N;
        hx = ox - (k.dt / mx[i]) * ((d_zy - d_yz) - px);
        hy = oy - (k.dt / my[i]) * ((d_xz - d_zx) - py);
        hz = oz - (k.dt / mz[i]) * ((d_yx - d_xy) - pz);
    } else {
        hx = ox - k.dt * ((d_zy - d_yz) - px);
        hy = oy - k.dt * ((d_xz - d_zx) - py);
        hz = oz - k.dt * ((d_yx - d_xy) - pz);
    }
    Px[i] = hx;
    Py[i] = hy;
    Pz[i] = hz;
    if (POYNT) {
        // E averaged in space, H in time (update_h.cl:63-70, 135-137), six products
        // in plane order xy, yz, zx, xz, yx, zy (update_h.cl:142-154)
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

// ---- update_S (update_s.cl:33-36) ----------------------------------------------------------
template <typename R>
__global__ void __launch_bounds__(256) k_poynting(const SK<R> k)
{
    const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= k.syz) return;
    const uint32_t x = blockIdx.y;
    const uint32_t y = k.dsz.div(j);
    const uint32_t z = j - y * k.sz;
    const uint32_t i = x * k.syz + j;
    const uint64_t N = k.N;
    const uint32_t imx = x ? i - k.syz : i + (k.sx - 1u) * k.syz;
    const uint32_t imy = y ? i - k.sz : i + (k.sy - 1u) * k.sz;
    const uint32_t imz = z ? i - 1u : i + (k.sz - 1u);
    const R *oxy = k.oS, *oyz = k.oS + N, *ozx = k.oS + 2 * N;
    const R *oxz = k.oS + 3 * N, *oyx = k.oS + 4 * N, *ozy = k.oS + 5 * N;
    k.S[i] = (((oxy[i] + oxz[i]) + oxy[imy]) + oxz[imz]) * k.sf;
    k.S[N + i] = (((oyz[i] + oyx[i]) + oyz[imz]) + oyx[imx]) * k.sf;
    k.S[2 * N + i] = (((ozx[i] + ozy[i]) + ozx[imx]) + ozy[imy]) * k.sf;
}

// ---- update_J (update_j.cl:23-32), launched over the box only -------------------------------
template <typename R>
__global__ void __launch_bounds__(256) k_fieldsrc(const JK<R> k)
{
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
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
template <typename R>
__global__ void k_point_sources(const PointK<R> k)
{
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= k.n) return;
    const int64_t ind = k.index[s];
    k.E[ind] = k.E[ind] + k.values[(int64_t)k.t * k.n + s];
}

// ---- launchers ------------------------------------------------------------------------------
static inline dim3 plane_grid(uint32_t syz, uint32_t sx)
{
    return dim3((syz + 255u) / 256u, sx, 1);
}

template <typename R>
cudaError_t launch_yee_e(const YeeK<R> &k, cudaStream_t st)
{
    k_yee_e<R><<<plane_grid(k.syz, k.sx), 256, 0, st>>>(k);
    return cudaGetLastError();
}

template <typename R>
cudaError_t launch_yee_h(const YeeK<R> &k, bool mu, bool poynting, cudaStream_t st)
{
    const dim3 g = plane_grid(k.syz, k.sx);
    if (mu) {
        if (poynting) k_yee_h<R, true, true><<<g, 256, 0, st>>>(k);
        else k_yee_h<R, true, false><<<g, 256, 0, st>>>(k);
    } else {
        if (poynting) k_yee_h<R, false, true><<<g, 256, 0, st>>>(k);
        else k_yee_h<R, false, false><<<g, 256, 0, st>>>(k);
    }
    return cudaGetLastError();
}

template <typename R>
cudaError_t launch_poynting(const SK<R> &k, cudaStream_t st)
{
    k_poynting<R><<<plane_grid(k.syz, k.sx), 256, 0, st>>>(k);
    return cudaGetLastError();
}

template <typename R>
cudaError_t launch_fieldsrc(const JK<R> &k, cudaStream_t st)
{
    const uint32_t n = k.nx * k.ny * k.nz;
    if (n == 0) return cudaSuccess;
    k_fieldsrc<R><<<(n + 255u) / 256u, 256, 0, st>>>(k);
    return cudaGetLastError();
}

template <typename R>
cudaError_t launch_point_sources(const PointK<R> &k, cudaStream_t st)
{
    if (k.n <= 0) return cudaSuccess;
    k_point_sources<R><<<(k.n + 127) / 128, 128, 0, st>>>(k);
    return cudaGetLastError();
}

#define FDTD_INSTANTIATE(R)                                                              \
    template cudaError_t launch_yee_e<R>(const YeeK<R> &, cudaStream_t);               \
    template cudaError_t launch_yee_h<R>(const YeeK<R> &, bool, bool, cudaStream_t);   \
    template cudaError_t launch_poynting<R>(const SK<R> &, cudaStream_t);              \
    template cudaError_t launch_fieldsrc<R>(const JK<R> &, cudaStream_t);              \
    template cudaError_t launch_point_sources<R>(const PointK<R> &, cudaStream_t);

FDTD_INSTANTIATE(float)
FDTD_INSTANTIATE(double)

}  // namespace fdtd
