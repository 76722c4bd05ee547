// Host-side plan object behind the opaque FdtdPlan of include/fdtd_gb300.h.
#pragma once

#include <cstddef>
#include <cstdint>

#include "fdtd_gb300.h"

struct FdtdPlan {
    FdtdDesc d;                 // copy of the caller's description
    uint32_t sx, sy, sz, syz;
    uint64_t N;
    size_t elem;                // bytes per element of the plan's dtype
    int device;                 // device that was current at creation
    int32_t xchunk;             // x planes a bulk-kernel thread marches
    int32_t eform;              // form of the bulk E kernel (FDTD_TUNE_E_FORM)
    uint32_t slab;              // x planes per L2-resident slab in fdtd_run (0: whole grid)
    uint32_t fused_rows;        // own rows of a one-pass step tile (0: the most that fit)
    uint32_t fused_xchunk;      // x planes one block of the one-pass step marches (0: automatic)
    uint32_t fused_stages;      // stages of the one-pass step's ring (0: 4, or as many as fit)
    int32_t fused_tma;          // one-pass step stages non-wrapping tiles by bulk copies
    int32_t fused_shape;        // one-pass block shape: 0 automatic, 1 large, 2 small
    int32_t last_run_path;      // FDTD_PATH_* of the last fdtd_run
    int32_t step_cfg[5];        // last one-pass launch: rows, xchunk, stages, threads, shape
    uint32_t hs_xchunk;         // x planes one block of the H+S kernel marches
    int32_t hs_prefetch;        // H+S kernel issues the next plane's loads early
    int32_t hs_reverse;         // H+S kernel takes its x chunks in descending order
    int32_t hs_xchunk_used;     // x chunk of the last H+S launch (hs_xchunk or the automatic one)
    int32_t hs_dft;             // H+S path: the DFT sample in the H+S launch, not a side stream
    int32_t pdl;                // H+S path: programmatic dependent launches of E and H+S
    int32_t timing;             // fdtd_run's H+S path records per-kernel CUDA events
    int32_t *status = nullptr;  // device word: bits of bounded waits inside kernels that ran out
    // side stream of fdtd_run's H+S path when hs_dft is off: the step's DFT monitor sample runs
    // there, beside the H+S launch (which leaves E unchanged); created on first use
    cudaStream_t side = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    double kernel_ms[2];        // last timed run: mean update_E and H+S launch times (ms)
    int32_t kernel_samples;     // launches each mean is over
    void *coef = nullptr;       // device copy of every face's six coefficient tables
    const void *tab[6][6];      // per face: p0e p1e p2e p0h p1h p2h (device pointers)
    // learned boundary attached with fdtd_lbc_attach (lbc_mask 0: none)
    int32_t lbc_mask = 0;       // faces, bit 2 * axis + side
    int32_t lbc_precision = 0;  // FDTD_LBC_F32 / BF16 / BF16X2
    float lbc_memory = 0.f;     // weight of the previous step's ghosts
    const void *lbc_w = nullptr;
    float *lbc_pred = nullptr;  // [columns][6] predictions of the current step
};

namespace fdtd {
int set_error(int code, const char *msg);
int check_cuda(cudaError_t e, const char *what);
// learned boundary around one step (no-ops when none is attached; lbc_abi.cu): the ghosts of
// every face from the pre-step state, the E fix-up after the E update, the H fix-up after the
// H update
int lbc_before_e(const FdtdPlan *p, const FdtdBuffers *b, const void *H, cudaStream_t st);
int lbc_after_e(const FdtdPlan *p, const FdtdBuffers *b, const void *H, cudaStream_t st);
int lbc_after_h(const FdtdPlan *p, const FdtdBuffers *b, void *H, cudaStream_t st);
}  // namespace fdtd
