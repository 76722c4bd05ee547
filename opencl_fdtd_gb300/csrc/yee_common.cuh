// Shared device-side definitions of the Yee time-stepping kernels.
//
// Grid and field layout follow opencl_fdtd/kernels/common.cl:34-52: a field is [X | Y | Z],
// each component C-ordered (x, y, z) with z fastest, so cell (x, y, z) is flat index
// i = (x*sy + y)*sz + z and the component offsets are 0, N, 2N.
//
// Every update is one "bulk" launch: thread (y, z) of a plane marches a chunk of
// consecutive x planes. The generic per-cell kernels (faces applied in list order) remain
// for the one case the bulk kernels exclude: two CPML faces of one axis that overlap.
// Both apply the same per-cell arithmetic.
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
        f.d = dd ? dd : 1u;
        uint32_t l = 0;
        while ((1ull << l) < f.d) ++l;
        f.l = l;
        f.m = (uint32_t)((((1ull << 32) * ((1ull << l) - f.d)) / f.d) + 1);
        return f;
    }
    __device__ __forceinline__ uint32_t div(uint32_t n) const
    {
        const uint32_t t = __umulhi(m, n);
        return (uint32_t)(((uint64_t)t + n) >> l);
    }
};

// Programmatic dependent launch (fdtd_run's H+S path, FDTD_TUNE_PDL): a kernel launched with
// programmatic stream serialization may be scheduled while the kernel before it in the stream
// still runs; it waits here, before its first global memory access, until that kernel has
// completed and its writes are visible, and then lets the next kernel of the stream be
// scheduled. Without the launch attribute both instructions have no effect.
__device__ __forceinline__ void grid_dependency_sync()
{
    asm volatile("griddepcontrol.wait;" ::: "memory");
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

// Launches kern<<<g, block, 0, st>>>(arg), with programmatic stream serialization when pdl.
template <typename K>
inline cudaError_t launch_dependent(void (*kern)(K), dim3 g, unsigned block, cudaStream_t st,
                                    bool pdl, const K &arg)
{
    if (!pdl) {
        kern<<<g, block, 0, st>>>(arg);
        return cudaGetLastError();
    }
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = g;
    cfg.blockDim = dim3(block, 1, 1);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = st;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kern, arg);
}

// CPML faces of one axis as the bulk kernels see them: the low ('n') face covers
// c < Tn, the high ('p') face c >= s - Tp (Tp = 0 when the face never applies). Faces of one
// axis never overlap in a bulk launch (the plan falls back to the generic kernels then), so
// every cell sees at most one face per axis and the order of faces cannot change a result.
template <typename R>
struct AxisK {
    int32_t Tn, Tp;
    const R *n0, *n1, *n2, *p0, *p1, *p2;
    R *nu, *nv, *pu, *pv;
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

// Arguments of one E-type or H-type update.
//   E-type: P += dt/eps * (curl Q + psi)         (update_e.cl:105-107)
//   H-type: P -= dt[/mu] * (curl Q - psi)       (update_h.cl:129-131)
// coef holds dt/mat precomputed (the same rounded quotient the reference forms per cell);
// when it is NULL the shell kernels divide. Rp is the other half of Q's complex pair.
constexpr int YEE_SRC = 8;       // point sources the bulk E kernel can add itself

template <typename R>
struct YeeK {
    R *P;
    const R *Q;
    const R *Rp;
    const R *mat;
    const R *coef;
    R *oS;
    uint32_t sx, sy, sz, syz;
    uint64_t N;
    R dt, inv_d;
    const R *inv_tab[3];
    int32_t nface, bloch_mask, dxmode;
    int32_t eform;              // form of the bulk E kernel (0 next plane ahead, 1 per-plane loads)
    R br[3], bi[3];
    FaceK<R> face[6];
    AxisK<R> ax[3];
    FastDiv dsz;
    int32_t xchunk, bulk;
    uint32_t xbeg, xend;        // planes [xbeg, xend) this launch updates
    // point sources the bulk E kernel adds after the update, in list order (fdtd.py:168-169):
    // E[c][x, j] += src_values[src_t * src_stride + src_col] for each of nsrc sources
    int32_t nsrc, src_t, src_stride, _pad2;
    const R *src_values;
    uint32_t src_x[YEE_SRC], src_j[YEE_SRC];
    int32_t src_c[YEE_SRC], src_col[YEE_SRC];
};

template <typename R>
struct SK {
    R *S;
    const R *oS;
    uint32_t sx, sy, sz, syz;
    uint64_t N;
    R sf;
    FastDiv dsz;
    int32_t xchunk, _pad;
    uint32_t xbeg, xend;        // planes [xbeg, xend) this launch updates
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

constexpr int MAX_POINT_SOURCES = 64;

template <typename R>
struct PointK {
    R *E;
    const R *values;            // [nsteps][stride]
    int32_t n, t, stride, _pad;
    int64_t index[MAX_POINT_SOURCES];
    int32_t col[MAX_POINT_SOURCES];   // column of each source in values
};

template <typename R>
struct PrepK {
    R *out;
    const R *mat;
    uint64_t n;
    R dt;
};

constexpr int BLOCK = 256;

}  // namespace fdtd
