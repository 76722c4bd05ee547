// Arguments and launcher of the one-pass time step (step_kernel.cu): E update, point sources,
// H update and Poynting vector of one step in a single launch, with every field row a block
// needs staged in shared memory by bulk asynchronous copies.
#pragma once

#include "yee_common.cuh"

namespace fdtd {

constexpr int STEP_MAX_SRC = 8;
constexpr int STEP_MAX_STAGES = 6;

// Staged arrays of one x plane of a tile, in stage order. Field slots hold component c of
// H, E, dt/eps and (with mu) dt/mu at slot kind * 3 + c; the eight z-face CPML slots follow,
// four per side: (type * 2 + uv) with type 0 = E, 1 = H.
enum : int { SG_H = 0, SG_E = 3, SG_C = 6, SG_M = 9, SG_NF = 12, SG_NZ = 8, SG_N = SG_NF + SG_NZ };

// Block shapes: at most MAXT threads (one per cell of the E window), STR elements per field
// slot (every slot starts at a compile-time offset of its stage) and at least MINB resident
// blocks per SM. Float32 has a large shape (one block per SM, up to 1024 threads) and a small
// one (two blocks per SM, so one block's barrier and copy waits overlap the other's work);
// float64 has one shape.
struct StepBig {
    static constexpr int MAXT = 1024, STR = 1028, MINB = 1;
};
struct StepSmall {
    static constexpr int MAXT = 512, STR = 592, MINB = 2;
};
struct StepF64 {
    static constexpr int MAXT = 512, STR = 516, MINB = 1;
};
enum : int { STEP_SHAPE_BIG = 1, STEP_SHAPE_SMALL = 2 };

// CPML coefficient tables staged per block (all faces' six tables, FdtdPlan::coef order)
constexpr int STEP_MAX_COEF = 2048;

// CPML faces of one axis: thickness of the low ('n') and high ('p') face (0: none) and the
// auxiliary arrays read (A) and written (B), [E/H][n/p][u/v]. Faces of one axis never overlap
// here.
template <typename R>
struct StepAxis {
    int32_t Tn, Tp;
    const R *psiA[2][2][2];
    R *psiB[2][2][2];
};

template <typename R>
struct StepK {
    const R *EA, *HA;           // fields at the start of the step
    R *EB, *HB;                 // fields at the end of the step
    const R *ce, *cm;           // dt/eps, dt/mu (cm NULL without mu)
    R *S, *oS;                  // S every step (Poynting on); oS when write_oS
    uint32_t sx, sy, sz, syz;
    uint64_t N;
    R dt, inv_d, sf;
    const R *inv_de[3], *inv_dh[3];
    StepAxis<R> ax[3];
    uint32_t ntile;             // tiles along y (tile t owns rows [t*sy/ntile, (t+1)*sy/ntile))
    uint32_t xchunk;            // x planes per block
    uint32_t nstage;            // planes in the stage ring
    uint32_t stage_elems;       // elements of one stage (field slots, then the z slots)
    uint32_t zoff[2];           // offset of the z slots of side n / p in a stage: slot
    uint32_t zsz[2];            // (type * 2 + uv) at zoff[side] + (type * 2 + uv) * zsz[side]
    const R *coef;              // every face's six coefficient tables (p0e p1e p2e p0h p1h p2h)
    uint32_t ncoef;             // elements of coef (<= STEP_MAX_COEF)
    int32_t coff[3][2];         // offset of the tables of the face of axis / side in coef
    uint64_t len[SG_N];         // elements of each staged array (tail rule of the bulk copies)
    int32_t tma;                // 1: tiles whose rows do not wrap stage by bulk copies
    int32_t poynt, write_oS;
    int32_t nsrc, t;            // point sources; t: row of src_values for this step
    uint32_t src_x[STEP_MAX_SRC], src_j[STEP_MAX_SRC];   // plane and in-plane offset
    int32_t src_c[STEP_MAX_SRC];
    const R *src_values;        // device, [nsteps][nsrc]
    int32_t *status;            // device word: STEP_STATUS_* bits
    uint32_t wait_ns;           // bound of every wait on a stage
};

// A wait for staged data that ran out (the block stops; the host reads the bit).
constexpr int32_t STEP_STATUS_TIMEOUT = 4;

// Rows of a tile for the plan's z extent: the most that fit the block shape (0: sz too long).
template <typename R> uint32_t step_max_rows(int shape, uint32_t sz);
// Dynamic shared memory of a launch with `nstage` stages of `stage_elems` elements and `ncoef`
// CPML coefficients.
template <typename R> size_t step_smem_bytes(int shape, uint32_t nstage, uint32_t stage_elems, uint32_t ncoef);
// Threads of a block for tiles of at most `rows` own rows.
uint32_t step_threads(uint32_t rows, uint32_t sz);
template <typename R>
cudaError_t launch_step(const StepK<R> &k, int shape, int dxmode, bool mu, uint32_t threads, size_t smem,
                        cudaStream_t st);

}  // namespace fdtd
