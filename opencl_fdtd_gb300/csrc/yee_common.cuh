// Shared device-side definitions of the Yee time-stepping kernels.
//
// Grid and field layout follow opencl_fdtd/kernels/common.cl:34-52: a field is [X | Y | Z],
// each component C-ordered (x, y, z) with z fastest, so cell (x, y, z) is flat index
// i = (x*sy + y)*sz + z and the component offsets are 0, N, 2N.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace fdtd {

// Unsigned 32-bit division by a runtime constant (round-up magic number with an add step;
// Granlund & Montgomery 1994, "Division by invariant integers using multiplication", Thm 4.2).
struct FastDiv {
    uint32_t d, m, l;
    static FastDiv make(uint32_t dd)
    {
        FastDiv f;
        f.d = dd;
        uint32_t l = 0;
        while ((1ull << l) < dd) ++l;
        f.l = l;
        f.m = (uint32_t)((((1ull << 32) * ((1ull << l) - dd)) / dd) + 1);
        return f;
    }
    __device__ __forceinline__ uint32_t div(uint32_t n) const
    {
        const uint32_t t = __umulhi(m, n);
        return (uint32_t)(((uint64_t)t + n) >> l);
    }
};

// One CPML face as one update kernel sees it (E tables for E-type kernels, H tables for
// H-type ones). psi layout: C order of the grid shape with the face axis replaced by T,
// indexed by the depth ir from the outer face.
template <typename R>
struct FaceK {
    int32_t axis, pol, T, _pad;
    const R *p0, *p1, *p2;
    R *psi_u, *psi_v;
};

// Arguments of one E-type or H-type launch.
//   E-type: P += dt/mat * (curl Q + psi)         (update_e.cl:105-107)
//   H-type: P -= dt[/mat] * (curl Q - psi)       (update_h.cl:129-131)
// Rp is the other half of Q's complex pair for Bloch boundaries.
template <typename R>
struct YeeK {
    R *P;
    const R *Q;
    const R *Rp;
    const R *mat;
    R *oS;
    uint32_t sx, sy, sz, syz;
    uint64_t N;
    FastDiv dsz;
    R dt, inv_d;
    const R *inv_tab[3];
    int32_t nface, bloch_mask;
    R br[3], bi[3];
    FaceK<R> face[6];
};

template <typename R>
struct SK {
    R *S;
    const R *oS;
    uint32_t sx, sy, sz, syz;
    uint64_t N;
    FastDiv dsz;
    R sf;
};

template <typename R>
struct JK {
    R *E;
    const R *Jr, *Ji;
    uint32_t sy, sz;
    uint64_t N;
    uint32_t x0, y0, z0, nx, ny, nz;
    FastDiv dnz, dnyz;
    R c, s;
};

template <typename R>
struct PointK {
    R *E;
    const int64_t *index;
    const R *values;
    int32_t n, t;
};

}  // namespace fdtd
