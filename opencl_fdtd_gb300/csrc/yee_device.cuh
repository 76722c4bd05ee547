// Device helpers shared by the per-update kernels (yee_kernels.cu) and the H+S kernel
// (hs_fused.cu): read-only loads, CPML depth lookup and the per-face CPML arithmetic.
#pragma once

#include "yee_common.cuh"

namespace fdtd {

template <typename T>
__device__ __forceinline__ T ldg(const T *p) { return __ldg(p); }

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
// (update_h.cl:113-114). Returns the new (psi_u, psi_v).
template <typename R, bool ETYPE, int AX>
__device__ __forceinline__ void face_update(R p0, R p1, R p2, R su_old, R sv_old, R &su, R &sv,
                                            R &d_xy, R &d_xz, R &d_yx, R &d_yz, R &d_zx, R &d_zy,
                                            R &px, R &py, R &pz)
{
    R &dv = (AX == 0) ? d_zx : (AX == 1) ? d_zy : d_yz;
    R &du = (AX == 0) ? d_yx : (AX == 1) ? d_xy : d_xz;
    dv = dv * p2;
    du = du * p2;
    su = p0 * su_old + p1 * dv;
    sv = p0 * sv_old + p1 * du;
    R &pu = (AX == 0) ? py : px;
    R &pv = (AX == 2) ? py : pz;
    const bool plus_u = ETYPE ? (AX == 1) : (AX != 1);
    if (plus_u) { pu = pu + su; pv = pv - sv; }
    else        { pu = pu - su; pv = pv + sv; }
}

// psi index of cell (x, y, z) at depth ir of a face of axis AX with thickness T
template <int AX>
__device__ __forceinline__ uint32_t psi_index(uint32_t ir, uint32_t T, uint32_t x, uint32_t y,
                                              uint32_t z, uint32_t sy, uint32_t sz)
{
    if (AX == 0) return (ir * sy + y) * sz + z;
    if (AX == 1) return (x * T + ir) * sz + z;
    return (x * sy + y) * T + ir;
}

// Per-thread view of one axis's CPML faces for a coordinate that stays fixed during the march
// (y or z): depth index, thickness and coefficients, or ir < 0 outside both faces.
template <typename R>
struct FixedFace {
    int ir;
    uint32_t T;
    R p0, p1, p2;
    R *pu, *pv;
};

template <typename R, bool ETYPE>
__device__ __forceinline__ FixedFace<R> fixed_face(const AxisK<R> &a, uint32_t s, uint32_t c)
{
    FixedFace<R> f;
    f.ir = -1;
    f.T = 0;
    f.p0 = f.p1 = f.p2 = R(0);
    f.pu = f.pv = nullptr;
    if (c < (uint32_t)a.Tn) {
        f.ir = (int)c;
        f.T = (uint32_t)a.Tn;
        f.p0 = ldg(a.n0 + c); f.p1 = ldg(a.n1 + c); f.p2 = ldg(a.n2 + c);
        f.pu = a.nu;
        f.pv = a.nv;
    } else if (a.Tp && c >= s - (uint32_t)a.Tp) {
        const uint32_t ir = s - 1u - c;
        f.ir = (int)ir;
        f.T = (uint32_t)a.Tp;
        f.p0 = ldg(a.p0 + ir); f.p1 = ldg(a.p1 + ir); f.p2 = ldg(a.p2 + ir);
        f.pu = a.pu;
        f.pv = a.pv;
    }
    return f;
}

// x-face of plane x (uniform across the block): depth, thickness and psi arrays
template <typename R>
struct XFace {
    int ir;
    uint32_t T;
    const R *t0, *t1, *t2;
    R *pu, *pv;
};

template <typename R>
__device__ __forceinline__ XFace<R> x_face(const AxisK<R> &a, uint32_t sx, uint32_t x)
{
    XFace<R> f;
    f.ir = -1;
    f.T = 0;
    f.t0 = f.t1 = f.t2 = nullptr;
    f.pu = f.pv = nullptr;
    if (x < (uint32_t)a.Tn) {
        f.ir = (int)x; f.T = (uint32_t)a.Tn;
        f.t0 = a.n0; f.t1 = a.n1; f.t2 = a.n2; f.pu = a.nu; f.pv = a.nv;
    } else if (a.Tp && x >= sx - (uint32_t)a.Tp) {
        f.ir = (int)(sx - 1u - x); f.T = (uint32_t)a.Tp;
        f.t0 = a.p0; f.t1 = a.p1; f.t2 = a.p2; f.pu = a.pu; f.pv = a.pv;
    }
    return f;
}

}  // namespace fdtd
