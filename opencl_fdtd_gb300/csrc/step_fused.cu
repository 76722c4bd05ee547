// Fused time step: E update, point sources, H update and Poynting vector in one launch.
//
// The two-pass drop-in path (update_E, update_H, update_S) moves E, H, eps and the six oS
// planes through HBM several times per step (about 144 B per cell in float32). One step only
// needs to read E, H and dt/eps once and write E, H and S once (72 B per cell). This kernel
// gets there by temporal blocking inside a tile:
//
//   * Fields are double-buffered: every read comes from the old buffers (A: E, H, CPML psi),
//     every write goes to the new ones (B). No block ever reads a value another block
//     writes, so halo cells can be recomputed freely.
//   * A block owns J consecutive cells j = y*sz + z of a plane and a chunk of x planes. It
//     marches x, one plane behind for H and two for S:
//       phase A  E_new at plane x over its cells plus one row (sz cells) of halo on each side,
//                into shared memory (and to E_B for its own cells);
//       phase B  H_new and the six Poynting products at plane x-1 over its cells plus the
//                row before, reading E_new of planes x-1 and x from shared memory;
//       phase C  S at plane x-1 for its own cells, from the products of planes x-1 and x-2.
//     The march starts one plane before the chunk and ends one plane after it, with x taken
//     modulo sx, so the periodic wrap in x needs no special case.
//   * Wrap-around neighbours in y and z that fall outside the block's window (row 0 seen
//     from row sy-1 and the like) are recomputed from the old buffers on the spot.
//
// Every cell value goes through the same arithmetic, in the same order, as the two-pass
// kernels (this translation unit is also compiled with --fmad=false), so a fused step gives
// bit-identical fields. CPML faces are handled per axis (faces of one axis must not overlap)
// and Bloch boundaries are not supported here; the plan falls back to the two-pass path for
// those cases.
#include "yee_common.cuh"
#include "fused.h"

namespace fdtd {

template <typename T>
__device__ __forceinline__ T ldgf(const T *p) { return __ldg(p); }

// depth index of coordinate c in the faces of one axis (-1: none); hi = high ('p') face
__device__ __forceinline__ int axis_face(int Tn, int Tp, uint32_t s, uint32_t c, bool &hi)
{
    if (c < (uint32_t)Tn) { hi = false; return (int)c; }
    if (Tp && c >= s - (uint32_t)Tp) { hi = true; return (int)(s - 1u - c); }
    hi = false;
    return -1;
}

template <int AX>
__device__ __forceinline__ uint32_t fpsi_index(uint32_t ir, uint32_t T, uint32_t x, uint32_t y,
                                               uint32_t z, uint32_t sy, uint32_t sz)
{
    if (AX == 0) return (ir * sy + y) * sz + z;
    if (AX == 1) return (x * T + ir) * sz + z;
    return (x * sy + y) * T + ir;
}

// Old CPML values of one cell for one update type, per axis (u, v); zero outside the slabs.
template <typename R>
struct PsiOld {
    R v[3][2];
};

template <typename R, bool ETYPE, int AX>
__device__ __forceinline__ void psi_load_axis(const FusedK<R> &k, uint32_t s, uint32_t x, uint32_t y,
                                              uint32_t z, PsiOld<R> &p)
{
    const FAxis<R> &a = k.ax[AX];
    const uint32_t c = (AX == 0) ? x : (AX == 1) ? y : z;
    bool hi;
    const int ir = axis_face(a.Tn, a.Tp, s, c, hi);
    p.v[AX][0] = p.v[AX][1] = R(0);
    if (ir < 0) return;
    const uint32_t T = (uint32_t)(hi ? a.Tp : a.Tn);
    const int side = hi ? 1 : 0, ty = ETYPE ? 0 : 1;
    const uint32_t ip = fpsi_index<AX>((uint32_t)ir, T, x, y, z, k.sy, k.sz);
    p.v[AX][0] = ldgf(a.psiA[ty][side][0] + ip);
    p.v[AX][1] = ldgf(a.psiA[ty][side][1] + ip);
}

template <typename R, bool ETYPE>
__device__ __forceinline__ void psi_load(const FusedK<R> &k, uint32_t x, uint32_t y, uint32_t z,
                                         PsiOld<R> &p)
{
    psi_load_axis<R, ETYPE, 0>(k, k.sx, x, y, z, p);
    psi_load_axis<R, ETYPE, 1>(k, k.sy, x, y, z, p);
    psi_load_axis<R, ETYPE, 2>(k, k.sz, x, y, z, p);
}

// CPML term of one axis for one cell (update_e.cl:64-100, update_h.cl:80-116), from the old
// psi values; identical arithmetic to face_update in yee_kernels.cu.
template <typename R, bool ETYPE, int AX>
__device__ __forceinline__ void fface(const FAxis<R> &a, uint32_t s, uint32_t x, uint32_t y,
                                      uint32_t z, uint32_t sy, uint32_t sz, bool wr, R so_u, R so_v,
                                      R &d_xy, R &d_xz, R &d_yx, R &d_yz, R &d_zx, R &d_zy,
                                      R &px, R &py, R &pz)
{
    const uint32_t c = (AX == 0) ? x : (AX == 1) ? y : z;
    bool hi;
    const int ir = axis_face(a.Tn, a.Tp, s, c, hi);
    if (ir < 0) return;
    const int side = hi ? 1 : 0;
    const int ty = ETYPE ? 0 : 1;
    const R p0 = ldgf(a.tab[ty][side][0] + ir);
    const R p1 = ldgf(a.tab[ty][side][1] + ir);
    const R p2 = ldgf(a.tab[ty][side][2] + ir);
    R &dv = (AX == 0) ? d_zx : (AX == 1) ? d_zy : d_yz;
    R &du = (AX == 0) ? d_yx : (AX == 1) ? d_xy : d_xz;
    dv = dv * p2;
    du = du * p2;
    const R su = p0 * so_u + p1 * dv;
    const R sv = p0 * so_v + p1 * du;
    if (wr) {
        const uint32_t T = (uint32_t)(hi ? a.Tp : a.Tn);
        const uint32_t ip = fpsi_index<AX>((uint32_t)ir, T, x, y, z, sy, sz);
        a.psiB[ty][side][0][ip] = su;
        a.psiB[ty][side][1][ip] = sv;
    }
    R &pu = (AX == 0) ? py : px;
    R &pv = (AX == 2) ? py : pz;
    const bool plus_u = ETYPE ? (AX == 1) : (AX != 1);
    if (plus_u) { pu = pu + su; pv = pv - sv; }
    else        { pu = pu - su; pv = pv + sv; }
}

// Inputs of one E_new evaluation.
template <typename R>
struct ELd {
    R hx, hy, hz;              // H_A at the cell
    R nxy, nxz, nyz, nzy;      // H_A: x comp at y-1 and z-1, y comp at z-1, z comp at y-1
    R ex, ey, ez;              // E_A at the cell
    R cx, cy, cz;              // dt/eps at the cell
    PsiOld<R> ps;              // psi_E_A at the cell
};

template <typename R>
__device__ __forceinline__ void e_load(const FusedK<R> &k, uint32_t x, uint32_t y, uint32_t z, ELd<R> &v)
{
    const uint32_t sz = k.sz, syz = k.syz;
    const uint64_t N = k.N;
    const uint32_t i = x * syz + y * sz + z;
    const uint32_t imy = y ? i - sz : i + (k.sy - 1u) * sz;
    const uint32_t imz = z ? i - 1u : i + (sz - 1u);
    const R *Hx = k.HA, *Hy = k.HA + N, *Hz = k.HA + 2 * N;
    v.hx = ldgf(Hx + i); v.hy = ldgf(Hy + i); v.hz = ldgf(Hz + i);
    v.nxy = ldgf(Hx + imy); v.nxz = ldgf(Hx + imz);
    v.nyz = ldgf(Hy + imz); v.nzy = ldgf(Hz + imy);
    v.ex = ldgf(k.EA + i); v.ey = ldgf(k.EA + N + i); v.ez = ldgf(k.EA + 2 * N + i);
    v.cx = ldgf(k.ce + i); v.cy = ldgf(k.ce + N + i); v.cz = ldgf(k.ce + 2 * N + i);
    psi_load<R, true>(k, x, y, z, v.ps);
}

// E_new from loaded inputs and the x-1 plane's H_y, H_z (update_e.cl:39-107), point sources
// added after the update (fdtd.py:168-169). wr: write the advanced psi to the B buffers.
template <typename R, int DX>
__device__ __forceinline__ void e_math(const FusedK<R> &k, uint32_t x, uint32_t y, uint32_t z,
                                       bool wr, const ELd<R> &v, R hym, R hzm,
                                       R &ox, R &oy, R &oz)
{
    R d_xy = v.hx - v.nxy;
    R d_xz = v.hx - v.nxz;
    R d_yx = v.hy - hym;
    R d_yz = v.hy - v.nyz;
    R d_zx = v.hz - hzm;
    R d_zy = v.hz - v.nzy;
    if (DX != 0) {
        R ix = k.inv_d, iy = k.inv_d, iz = k.inv_d;
        if (DX == 2) { ix = ldgf(k.inv_dh[0] + x); iy = ldgf(k.inv_dh[1] + y); iz = ldgf(k.inv_dh[2] + z); }
        d_xy = d_xy * iy; d_xz = d_xz * iz; d_yx = d_yx * ix;
        d_yz = d_yz * iz; d_zx = d_zx * ix; d_zy = d_zy * iy;
    }
    R px = R(0), py = R(0), pz = R(0);
    fface<R, true, 0>(k.ax[0], k.sx, x, y, z, k.sy, k.sz, wr, v.ps.v[0][0], v.ps.v[0][1], d_xy, d_xz, d_yx, d_yz, d_zx, d_zy, px, py, pz);
    fface<R, true, 1>(k.ax[1], k.sy, x, y, z, k.sy, k.sz, wr, v.ps.v[1][0], v.ps.v[1][1], d_xy, d_xz, d_yx, d_yz, d_zx, d_zy, px, py, pz);
    fface<R, true, 2>(k.ax[2], k.sz, x, y, z, k.sy, k.sz, wr, v.ps.v[2][0], v.ps.v[2][1], d_xy, d_xz, d_yx, d_yz, d_zx, d_zy, px, py, pz);
    ox = v.ex + v.cx * ((d_zy - d_yz) + px);
    oy = v.ey + v.cy * ((d_xz - d_zx) + py);
    oz = v.ez + v.cz * ((d_yx - d_xy) + pz);
    if (k.nsrc) {
#pragma unroll
        for (int s = 0; s < FUSED_MAX_SRC; ++s) {
            if (s >= k.nsrc) break;
            if (x == k.src_x[s] && y == k.src_y[s] && z == k.src_z[s]) {
                const R val = ldgf(k.src_values + (uint64_t)k.t * k.nsrc + s);
                if (k.src_c[s] == 0) ox = ox + val;
                else if (k.src_c[s] == 1) oy = oy + val;
                else oz = oz + val;
            }
        }
    }
}

// E_new at any cell from the old buffers (the wrap-around recomputation path).
template <typename R, int DX>
__device__ __forceinline__ void e_cell(const FusedK<R> &k, uint32_t x, uint32_t y, uint32_t z,
                                       R &ox, R &oy, R &oz)
{
    ELd<R> v;
    e_load<R>(k, x, y, z, v);
    const uint32_t i = x * k.syz + y * k.sz + z;
    const uint32_t imx = x ? i - k.syz : i + (k.sx - 1u) * k.syz;
    const R hym = ldgf(k.HA + k.N + imx), hzm = ldgf(k.HA + 2 * k.N + imx);
    e_math<R, DX>(k, x, y, z, false, v, hym, hzm, ox, oy, oz);
}

// H_new and the Poynting products at (x, y, z) from E_new of the cell and its plus
// neighbours, the old H and psi_H of the cell (update_h.cl:36-155).
template <typename R, int DX, bool MU>
__device__ __forceinline__ void h_math(const FusedK<R> &k, uint32_t x, uint32_t y, uint32_t z,
                                       bool wr, R ex, R ey, R ez, R ey_xp, R ez_xp, R ex_yp,
                                       R ez_yp, R ex_zp, R ey_zp, R ox, R oy, R oz,
                                       const PsiOld<R> &ps, R &hx, R &hy, R &hz, R *os)
{
    R d_xy = ex_yp - ex;
    R d_xz = ex_zp - ex;
    R d_yx = ey_xp - ey;
    R d_yz = ey_zp - ey;
    R d_zx = ez_xp - ez;
    R d_zy = ez_yp - ez;
    if (DX != 0) {
        R ix = k.inv_d, iy = k.inv_d, iz = k.inv_d;
        if (DX == 2) { ix = ldgf(k.inv_de[0] + x); iy = ldgf(k.inv_de[1] + y); iz = ldgf(k.inv_de[2] + z); }
        d_xy = d_xy * iy; d_xz = d_xz * iz; d_yx = d_yx * ix;
        d_yz = d_yz * iz; d_zx = d_zx * ix; d_zy = d_zy * iy;
    }
    R px = R(0), py = R(0), pz = R(0);
    fface<R, false, 0>(k.ax[0], k.sx, x, y, z, k.sy, k.sz, wr, ps.v[0][0], ps.v[0][1], d_xy, d_xz, d_yx, d_yz, d_zx, d_zy, px, py, pz);
    fface<R, false, 1>(k.ax[1], k.sy, x, y, z, k.sy, k.sz, wr, ps.v[1][0], ps.v[1][1], d_xy, d_xz, d_yx, d_yz, d_zx, d_zy, px, py, pz);
    fface<R, false, 2>(k.ax[2], k.sz, x, y, z, k.sy, k.sz, wr, ps.v[2][0], ps.v[2][1], d_xy, d_xz, d_yx, d_yz, d_zx, d_zy, px, py, pz);
    if (MU) {
        const uint64_t N = k.N;
        const uint32_t i = x * k.syz + y * k.sz + z;
        hx = ox - ldgf(k.cm + i) * ((d_zy - d_yz) - px);
        hy = oy - ldgf(k.cm + N + i) * ((d_xz - d_zx) - py);
        hz = oz - ldgf(k.cm + 2 * N + i) * ((d_yx - d_xy) - pz);
    } else {
        hx = ox - k.dt * ((d_zy - d_yz) - px);
        hy = oy - k.dt * ((d_xz - d_zx) - py);
        hz = oz - k.dt * ((d_yx - d_xy) - pz);
    }
    if (os) {
        const R ahx = hx + ox, ahy = hy + oy, ahz = hz + oz;
        os[0] = (ey_xp + ey) * ahz;
        os[3] = (-(ez_xp + ez)) * ahy;
        os[1] = (ez_yp + ez) * ahx;
        os[4] = (-(ex_yp + ex)) * ahz;
        os[2] = (ex_zp + ex) * ahy;
        os[5] = (-(ey_zp + ey)) * ahx;
    }
}

// Window bookkeeping of one block.
struct Win {
    uint32_t j0, j1, w0, wE1;   // own cells [j0, j1), E window [w0, wE1), H window [w0, j1)
    uint32_t nE, nH, ldE, ldH;  // window sizes and shared-memory leading dimensions
};

// E_new of plane px (stored in slot sEs when the cell is in the E window) or recomputed.
template <typename R, int DX>
__device__ __forceinline__ void enew_at(const FusedK<R> &k, const Win &w, const R *sEs,
                                        uint32_t px, uint32_t y, uint32_t z, R &ex, R &ey, R &ez)
{
    const uint32_t j = y * k.sz + z;
    if (j >= w.w0 && j < w.wE1) {
        const uint32_t o = j - w.w0;
        ex = sEs[o];
        ey = sEs[w.ldE + o];
        ez = sEs[2 * w.ldE + o];
    } else {
        e_cell<R, DX>(k, px, y, z, ex, ey, ez);
    }
}

// Poynting products at (xm, y, z), recomputing whatever is not in shared memory.
template <typename R, int DX, bool MU>
__device__ __forceinline__ void os_recompute(const FusedK<R> &k, const Win &w, const R *sEprev,
                                          const R *sEcur, uint32_t xm, uint32_t xp, uint32_t y,
                                          uint32_t z, R *os)
{
    R ex, ey, ez, ex1, ey1, ez1, exy, eyy, ezy, exz, eyz, ezz;
    enew_at<R, DX>(k, w, sEprev, xm, y, z, ex, ey, ez);
    enew_at<R, DX>(k, w, sEcur, xp, y, z, ex1, ey1, ez1);
    enew_at<R, DX>(k, w, sEprev, xm, y + 1u < k.sy ? y + 1u : 0u, z, exy, eyy, ezy);
    enew_at<R, DX>(k, w, sEprev, xm, y, z + 1u < k.sz ? z + 1u : 0u, exz, eyz, ezz);
    const uint64_t N = k.N;
    const uint32_t i = xm * k.syz + y * k.sz + z;
    PsiOld<R> ps;
    psi_load<R, false>(k, xm, y, z, ps);
    R hx, hy, hz;
    h_math<R, DX, MU>(k, xm, y, z, false, ex, ey, ez, ey1, ez1, exy, ezy, exz, eyz,
                      ldgf(k.HA + i), ldgf(k.HA + N + i), ldgf(k.HA + 2 * N + i), ps, hx, hy, hz, os);
}

// One thread per cell of the E window. Each thread keeps, across the x march: the inputs
// of its next E evaluation (loaded right after the current one, so they are in flight
// through phases B and C), the old H of the previous plane (the x-1 neighbour of phase A and
// the old value of phase B) and its cell's old psi_H.
template <typename R, int DX, bool MU, bool POYNT>
__global__ void __launch_bounds__(FUSED_THREADS, 1) k_fused_step(const FusedK<R> k)
{
    extern __shared__ __align__(16) unsigned char fsm[];
    R *sm = reinterpret_cast<R *>(fsm);
    const uint32_t sx = k.sx, sy = k.sy, sz = k.sz, syz = k.syz;
    const uint64_t N = k.N;
    Win w;
    w.j0 = blockIdx.x * k.J;
    w.j1 = min(w.j0 + k.J, syz);
    w.w0 = w.j0 >= sz ? w.j0 - sz : 0u;
    w.wE1 = min(w.j1 + sz, syz);
    w.nE = w.wE1 - w.w0;
    w.nH = w.j1 - w.w0;
    w.ldE = k.ldE;
    w.ldH = k.ldH;
    R *sE0 = sm;                        // slot 0: [3][ldE]
    R *sE1 = sm + 3 * k.ldE;            // slot 1
    R *sS = sm + 6 * k.ldE;             // [6][ldH] products of plane x-1
    const uint32_t t = threadIdx.x;
    const bool act = t < w.nE;
    const bool hact = t < w.nH;
    const uint32_t j = w.w0 + (act ? t : 0u);
    const uint32_t y = k.dsz.div(j);
    const uint32_t z = j - y * sz;
    const bool own = act && j >= w.j0 && j < w.j1;
    const uint32_t xa = blockIdx.y * k.xchunk;
    const uint32_t xb = min(xa + k.xchunk, sx);
    const int nst = (int)(xb - xa);
    auto plane = [&](int xi) -> uint32_t {
        if (xi < 0) xi += (int)sx;
        if (xi >= (int)sx) xi -= (int)sx;
        return (uint32_t)xi;
    };

    ELd<R> v;                           // inputs of the E evaluation of the current plane
    R pH0 = R(0), pH1 = R(0), pH2 = R(0);   // H_A of the previous plane at this cell
    PsiOld<R> phB;                      // psi_H_A of the previous plane at this cell
#pragma unroll
    for (int a = 0; a < 3; ++a) phB.v[a][0] = phB.v[a][1] = R(0);
    R prev_yx = R(0), prev_zx = R(0);   // products yx, zx of plane x-2 at this cell
    if (act) {
        const uint32_t xp0 = plane((int)xa - 2);
        const uint32_t i = xp0 * syz + j;
        pH0 = ldgf(k.HA + i); pH1 = ldgf(k.HA + N + i); pH2 = ldgf(k.HA + 2 * N + i);
        e_load<R>(k, plane((int)xa - 1), y, z, v);
    }

    for (int st = -1; st <= nst; ++st) {
        const uint32_t x = plane((int)xa + st);
        R *sEc = ((st + 2) & 1) ? sE1 : sE0;
        R *sEp = ((st + 2) & 1) ? sE0 : sE1;
        const bool inE = st >= 0 && st < nst;
        // phase A: E_new at plane x for this thread's window cell
        R nH0 = R(0), nH1 = R(0), nH2 = R(0);
        PsiOld<R> phN;
#pragma unroll
        for (int a = 0; a < 3; ++a) phN.v[a][0] = phN.v[a][1] = R(0);
        if (act) {
            R ex, ey, ez;
            e_math<R, DX>(k, x, y, z, own && inE, v, pH1, pH2, ex, ey, ez);
            sEc[t] = ex;
            sEc[w.ldE + t] = ey;
            sEc[2 * w.ldE + t] = ez;
            if (own && inE) {
                const uint32_t i = x * syz + j;
                k.EB[i] = ex;
                k.EB[N + i] = ey;
                k.EB[2 * N + i] = ez;
            }
            nH0 = v.hx; nH1 = v.hy; nH2 = v.hz;
            if (hact && st < nst) psi_load<R, false>(k, x, y, z, phN);
            if (st < nst) e_load<R>(k, plane((int)xa + st + 1), y, z, v);
        }
        __syncthreads();
        if (st >= 0) {
            // phase B: H_new and products at plane xm = x - 1 for this thread's H-window cell
            const uint32_t xm = x ? x - 1u : sx - 1u;
            const bool inH = st >= 1;
            if (hact) {
                R os[6];
                const R ex = sEp[t], ey = sEp[w.ldE + t], ez = sEp[2 * w.ldE + t];
                const R ey1 = sEc[w.ldE + t], ez1 = sEc[2 * w.ldE + t];
                R exy, ezy, exz, eyz, dummy;
                if (y + 1u < sy) {
                    exy = sEp[t + sz];
                    ezy = sEp[2 * w.ldE + t + sz];
                } else {
                    enew_at<R, DX>(k, w, sEp, xm, 0u, z, exy, dummy, ezy);
                }
                if (z + 1u < sz) {
                    exz = sEp[t + 1];
                    eyz = sEp[w.ldE + t + 1];
                } else {
                    enew_at<R, DX>(k, w, sEp, xm, y, 0u, exz, eyz, dummy);
                }
                R hx, hy, hz;
                const bool wr = own && inH;
                h_math<R, DX, MU>(k, xm, y, z, wr, ex, ey, ez, ey1, ez1, exy, ezy, exz, eyz,
                                  pH0, pH1, pH2, phB, hx, hy, hz, POYNT ? os : nullptr);
                if (wr) {
                    const uint32_t i = xm * syz + j;
                    k.HB[i] = hx;
                    k.HB[N + i] = hy;
                    k.HB[2 * N + i] = hz;
                    if (POYNT && k.write_oS) {
#pragma unroll
                        for (int c = 0; c < 6; ++c) k.oS[(uint64_t)c * N + i] = os[c];
                    }
                }
                if (POYNT) {
#pragma unroll
                    for (int c = 0; c < 6; ++c) sS[c * w.ldH + t] = os[c];
                }
            }
            __syncthreads();
            if (POYNT && own) {
                // phase C: S at plane xm (update_s.cl:33-36)
                if (inH) {
                    R xy_y, zy_y, xz_z, yz_z;
                    if (y) {
                        xy_y = sS[0 * w.ldH + t - sz];
                        zy_y = sS[5 * w.ldH + t - sz];
                    } else {
                        R o2[6];
                        os_recompute<R, DX, MU>(k, w, sEp, sEc, xm, x, sy - 1u, z, o2);
                        xy_y = o2[0];
                        zy_y = o2[5];
                    }
                    if (z) {
                        xz_z = sS[3 * w.ldH + t - 1];
                        yz_z = sS[1 * w.ldH + t - 1];
                    } else if (j + sz - 1u < w.j1) {
                        xz_z = sS[3 * w.ldH + t + sz - 1];
                        yz_z = sS[1 * w.ldH + t + sz - 1];
                    } else {
                        R o2[6];
                        os_recompute<R, DX, MU>(k, w, sEp, sEc, xm, x, y, sz - 1u, o2);
                        xz_z = o2[3];
                        yz_z = o2[1];
                    }
                    const uint32_t i = xm * syz + j;
                    k.S[i] = (((sS[t] + sS[3 * w.ldH + t]) + xy_y) + xz_z) * k.sf;
                    k.S[N + i] = (((sS[w.ldH + t] + sS[4 * w.ldH + t]) + yz_z) + prev_yx) * k.sf;
                    k.S[2 * N + i] = (((sS[2 * w.ldH + t] + sS[5 * w.ldH + t]) + prev_zx) + zy_y) * k.sf;
                }
                prev_yx = sS[4 * w.ldH + t];
                prev_zx = sS[2 * w.ldH + t];
            }
        }
        __syncthreads();
        pH0 = nH0; pH1 = nH1; pH2 = nH2;
        phB = phN;
    }
}

// ---- launcher ---------------------------------------------------------------------------------
template <typename R>
size_t fused_smem_bytes(const FusedK<R> &k)
{
    return (6 * (size_t)k.ldE + 6 * (size_t)k.ldH) * sizeof(R);
}

template <typename R, int DX, bool MU, bool POYNT>
static cudaError_t launch_one(const FusedK<R> &k, cudaStream_t st)
{
    const size_t smem = fused_smem_bytes(k);
    if (smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(k_fused_step<R, DX, MU, POYNT>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
    }
    const dim3 g((k.syz + k.J - 1) / k.J, (k.sx + k.xchunk - 1) / k.xchunk, 1);
    k_fused_step<R, DX, MU, POYNT><<<g, FUSED_THREADS, smem, st>>>(k);
    return cudaGetLastError();
}

template <typename R, int DX>
static cudaError_t launch_dx(const FusedK<R> &k, bool mu, bool poynting, cudaStream_t st)
{
    if (mu) return poynting ? launch_one<R, DX, true, true>(k, st) : launch_one<R, DX, true, false>(k, st);
    return poynting ? launch_one<R, DX, false, true>(k, st) : launch_one<R, DX, false, false>(k, st);
}

template <typename R>
cudaError_t launch_fused(const FusedK<R> &k, bool mu, bool poynting, int dxmode, cudaStream_t st)
{
    if (dxmode == 0) return launch_dx<R, 0>(k, mu, poynting, st);
    if (dxmode == 1) return launch_dx<R, 1>(k, mu, poynting, st);
    return launch_dx<R, 2>(k, mu, poynting, st);
}

template cudaError_t launch_fused<float>(const FusedK<float> &, bool, bool, int, cudaStream_t);
template cudaError_t launch_fused<double>(const FusedK<double> &, bool, bool, int, cudaStream_t);
template size_t fused_smem_bytes<float>(const FusedK<float> &);
template size_t fused_smem_bytes<double>(const FusedK<double> &);

}  // namespace fdtd
