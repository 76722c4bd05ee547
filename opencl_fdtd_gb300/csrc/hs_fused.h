// Arguments and launcher of the H+S kernel (hs_fused.cu).
#pragma once

#include "yee_common.cuh"
#include "monitors.h"

namespace fdtd {

// threads of an H+S block: whole z rows, the block's own rows plus one halo row,
// rows = HS_THREADS / sz - 1 (z rows of at most HS_THREADS / 2 cells). Two blocks per SM of
// 448 threads leave 72 registers a thread; 512 threads (64 registers, more spilled) ran 5%
// slower on 73-cell rows, 384 threads (4 own rows per halo row) 1% slower.
constexpr int HS_THREADS = 448;

// H-side CPML faces of one axis: tables [n/p][p0,p1,p2], old (A) and new (B) psi [n/p][u/v].
// Tp = 0 when the 'p' face never applies.
template <typename R>
struct HSAxis {
    int32_t Tn, Tp;
    const R *tab[2][3];
    const R *A[2][2];
    R *B[2][2];
};

template <typename R>
struct HSK {
    const R *E;            // E after this step's update and sources (read-only here)
    const R *HA;           // H before the update
    R *HB;                 // H after the update
    R *S, *oS;             // S every launch; oS only when write_oS
    const R *cm;           // dt/mu, NULL without mu
    uint32_t sx, sy, sz, syz;
    uint64_t N;
    R dt, inv_d, sf;
    const R *inv_de[3];
    HSAxis<R> ax[3];
    FastDiv dsz;
    uint32_t rows, xchunk;
    uint32_t nrowblk, nchunk;  // row blocks (ceil(sy / rows)) and x chunks (ceil(sx / xchunk))
    int32_t write_oS;
    int32_t reverse;       // 1: block row b of the grid takes the x chunk gridDim.y - 1 - b
    int32_t dft_on;        // 1: one extra block (the last) takes the step's DFT sample of E
    DftK<R> dft;
};

// pdl: launched with programmatic stream serialization
template <typename R>
cudaError_t launch_hs(const HSK<R> &k, bool mu, int dxmode, bool prefetch, bool pdl, cudaStream_t st);

}  // namespace fdtd
