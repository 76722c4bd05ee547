// Batched stepping of many independent cavity variants (batch.cu): device-side descriptors.
#pragma once

#include <cstdint>

#include "yee_common.cuh"

namespace fdtd {

// One block covers BATCH_THREADS consecutive (y, z) cells of a plane. In 16-bit storage each
// warp's run of BATCH_TILE of those cells (one component, one x plane) carries one scale.
constexpr int BATCH_THREADS = 256;
constexpr int BATCH_TILE = 32;
constexpr int BATCH_MAX_SRC = 4;
constexpr int BATCH_MAX_MON = 8;

// storage of E, H and dt/eps (arithmetic is float32 in every case)
constexpr int BATCH_F32 = 0;
constexpr int BATCH_BF16 = 1;
constexpr int BATCH_F16 = 2;
constexpr int BATCH_BF16U = 3;     // bfloat16 without tile exponents (its exponent range is float32's)

// CPML faces of one axis of one variant: tables [E/H][n/p][p0,p1,p2], psi [E/H][n/p][u/v]
// (float32, updated in place). Tp = 0 when the 'p' face never applies.
struct BAxis {
    int32_t Tn, Tp;
    const float *tab[2][2][3];
    float *psi[2][2][2];
};

struct BVar {
    uint32_t sx, sy, sz, syz;
    uint64_t N;
    uint32_t njb;               // blocks per plane: ceil(syz / BATCH_THREADS)
    uint32_t ntl;               // exponent tiles per plane: ceil(syz / BATCH_TILE)
    int32_t dxmode;             // 0: dx = 1, 1: uniform dx != 1
    int32_t _pad1;
    FastDiv dsz;
    float dt, inv_d;
    void *E, *H;                // 3N each in the storage type
    const void *ce;             // 3N dt/eps in the storage type (never scaled)
    int32_t *eexp, *hexp;       // [sx][ntl] packed exponents of the tiles (16-bit storage)
    BAxis ax[3];
    int32_t nsrc, nmon;
    uint32_t src_x[BATCH_MAX_SRC], src_j[BATCH_MAX_SRC];
    int32_t src_c[BATCH_MAX_SRC], _pad0;
    const float *src_values;    // [rows][nsrc]: row = step number
    uint32_t mon_x[BATCH_MAX_MON], mon_j[BATCH_MAX_MON];
    int32_t mon_c[BATCH_MAX_MON];
    double *series;             // [rows][nmon] or NULL: E after the step's sources
};

struct BatchK {
    const BVar *vars;
    const int4 *tiles;          // (variant, first x, end x, tile column jb)
    uint32_t ntiles;
    int32_t nsteps;
    int64_t *step;              // device step counter: read at start, advanced by nsteps at end
    int64_t rows;               // rows of the source and series arrays
    uint32_t *work;             // persistent schedule: tiles handed out so far in the current
                                // half-step, two counters used alternately (zero between launches)
};

template <int ST>
cudaError_t launch_batch(const BatchK &k, int blocks, cudaStream_t st);
template <int ST>
int batch_max_blocks_per_sm();
// nsteps x (one launch of every tile's E update, one of every tile's H update)
template <int ST>
cudaError_t launch_batch_steps(const BatchK &k, cudaStream_t st);

// f32 <-> storage of one field of one variant, choosing the tile exponents (encode)
cudaError_t launch_batch_encode(int store, const BVar &v, int field, const float *src, cudaStream_t st);
cudaError_t launch_batch_decode(int store, const BVar &v, int field, float *dst, cudaStream_t st);

}  // namespace fdtd
