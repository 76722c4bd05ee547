// Arguments and launcher of the fused time-step kernel (step_fused.cu).
#pragma once

#include "yee_common.cuh"

namespace fdtd {

constexpr int FUSED_MAX_SRC = 8;
// threads of a fused-step block: one per cell of its E window (own cells + one row each side)
constexpr int FUSED_THREADS = 768;

// CPML faces of one axis for the fused step: tables [E/H][n/p][p0,p1,p2] and the auxiliary
// arrays read (A) and written (B) [E/H][n/p][u/v]. Tp = 0 when the 'p' face never applies.
template <typename R>
struct FAxis {
    int32_t Tn, Tp;
    const R *tab[2][2][3];
    const R *psiA[2][2][2];
    R *psiB[2][2][2];
};

template <typename R>
struct FusedK {
    const R *EA, *HA;           // fields at the start of the step
    R *EB, *HB;                 // fields at the end of the step
    const R *ce, *cm;           // dt/eps, dt/mu (cm NULL without mu)
    R *S, *oS;                  // S every step; oS only when write_oS
    uint32_t sx, sy, sz, syz;
    uint64_t N;
    FastDiv dsz;
    R dt, inv_d, sf;
    const R *inv_de[3], *inv_dh[3];
    FAxis<R> ax[3];
    int32_t nsrc, t;            // point sources, step index into src_values
    uint32_t src_x[FUSED_MAX_SRC], src_y[FUSED_MAX_SRC], src_z[FUSED_MAX_SRC];
    int32_t src_c[FUSED_MAX_SRC];
    const R *src_values;        // device, [nsteps][nsrc]
    uint32_t J, xchunk, ldE, ldH;
    int32_t write_oS, _pad;
};

template <typename R> size_t fused_smem_bytes(const FusedK<R> &k);
template <typename R>
cudaError_t launch_fused(const FusedK<R> &k, bool mu, bool poynting, int dxmode, cudaStream_t st);

}  // namespace fdtd
