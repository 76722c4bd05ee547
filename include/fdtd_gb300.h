/*
 * fdtd_gb300.h — C ABI of the GB300 (sm_103a) FDTD time-stepping library.
 *
 * The reference (opencl_fdtd) reaches its kernels through pyopencl: Simulation.__init__
 * renders jinja2 templates into OpenCL C (opencl_fdtd/simulation.py:198-245), wraps each in an
 * ElementwiseKernel (simulation.py:321-326) and hands back closures update_E/H/S/F/G/J that
 * enqueue one kernel on the context's queue. This header is the boundary that replaces that
 * FFI: a plan takes the role of the rendered, specialised kernel set, and one entry point per
 * closure enqueues the same update on a CUDA stream.
 *
 * Conventions
 *   - Every field is a flat device array of 3*N elements, components [X | Y | Z], each in C
 *     order (x, y, z) with z fastest (opencl_fdtd/kernels/common.cl:34-52). oS holds 6*N
 *     elements in the plane order xy, yz, zx, xz, yx, zy (update_h.cl:142-147).
 *   - Device buffers belong to the caller (torch tensors in the Python layer) and are passed
 *     as raw pointers on every call. A plan owns only its small coefficient tables.
 *   - Calls are asynchronous on the given stream (a cudaStream_t passed as void*; NULL is the
 *     legacy default stream). One plan serves one host thread at a time, as the reference's
 *     single queue does (simulation.py:328-338).
 *   - Every entry point returns FDTD_OK (0) or a negative status; no exception crosses the
 *     ABI. fdtd_last_error() returns the calling thread's last message.
 */
#ifndef FDTD_GB300_H
#define FDTD_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define FDTD_ABI_VERSION 1

/* status codes */
#define FDTD_OK 0
#define FDTD_ERR_INVALID (-1)      /* bad shape, size, pointer or option */
#define FDTD_ERR_UNSUPPORTED (-2)  /* dtype or option combination not built */
#define FDTD_ERR_CUDA (-3)         /* a CUDA runtime call or launch failed */
#define FDTD_ERR_WATCHDOG (-4)     /* a bounded device-side wait gave up */
#define FDTD_ERR_NONFINITE (-5)    /* a field watchdog found NaN/Inf */

/* storage / arithmetic types (simulation.py:360-376 maps numpy float16/32/64) */
#define FDTD_F32 0
#define FDTD_F64 1

typedef struct FdtdPmlDesc {
    int32_t axis;        /* 0, 1, 2 for 'x', 'y', 'z' */
    int32_t polarity;    /* 0 = 'n' (low side), 1 = 'p' (high side) */
    int32_t thickness;   /* T cells */
    int32_t _pad;
    /* Host pointers to the six coefficient tables p{0,1,2}e and p{0,1,2}h (simulation.py:
     * 284-307), each `thickness` long, indexed by depth ir (0 = outermost cell), in the
     * plan's dtype. The plan copies them to the device. */
    const void *p0e, *p1e, *p2e, *p0h, *p1h, *p2h;
} FdtdPmlDesc;

typedef struct FdtdBlochDesc {
    int32_t axis;        /* 0, 1, 2 */
    int32_t _pad;
    double real, imag;   /* beta = real + i*imag: field(r + L) = beta * field(r) */
} FdtdBlochDesc;

typedef struct FdtdDesc {
    int64_t shape[3];    /* (sx, sy, sz); N = sx*sy*sz must be < 2^32 */
    int32_t dtype;       /* FDTD_F32 or FDTD_F64 */
    int32_t uniform;     /* 1: uniform spacing dx; 0: per-axis tables in FdtdBuffers */
    double dt;           /* rounded to dtype, as the reference's `ftype dt` argument */
    double dx;           /* uniform spacing; the kernels use (dtype)(1.0/dx) */
    int32_t n_pml;       /* 0..6 faces, applied in list order */
    int32_t n_bloch;     /* 0..3 */
    FdtdPmlDesc pml[6];
    FdtdBlochDesc bloch[3];
    int32_t do_poynting; /* update_H writes oS; update_S is available */
    int32_t do_fieldsrc; /* update_J is available */
    int32_t has_mu;      /* H updates divide dt by mu (absent in the reference) */
    int32_t _pad;
} FdtdDesc;

typedef struct FdtdBuffers {
    void *E, *H;             /* 3N each */
    void *F, *G;             /* imaginary parts with Bloch boundaries, else NULL */
    const void *eps;         /* 3N relative permittivity; +inf marks PEC */
    const void *mu;          /* 3N relative permeability when has_mu, else NULL */
    void *S;                 /* 3N Poynting vector when do_poynting */
    void *oS;                /* 6N Poynting products when do_poynting */
    const void *Jr, *Ji;     /* 3N current-source phasor when do_fieldsrc */
    /* CPML auxiliary fields, per face in plan order, two components (u, v) each: the two
     * axes other than the face's, in xyz order. Layout: C order of the grid shape with the
     * face axis replaced by T, indexed by depth ir along that axis. */
    void *psi_e[6][2], *psi_h[6][2], *psi_f[6][2], *psi_g[6][2];
    /* non-uniform spacing: 1/dx on the E grid (H updates read these) and on the H grid
     * (E updates read these), lengths sx, sy, sz; NULL when uniform */
    const void *inv_de[3], *inv_dh[3];
    /* Optional 3N caches of dt/eps and dt/mu (the per-cell quotient of update_e.cl:105-107),
     * filled by fdtd_prepare. When set they must be current; when NULL every cell divides,
     * which is slower but gives the same result. */
    void *ce, *cm;
    /* Optional second copies for fdtd_run (same sizes as E, H, psi_e, psi_h). With H2 and every
     * psi_h2 set (E2 NULL), steps run update_E in place and H and S in one launch that reads
     * one copy of H and writes the other (z rows of at most 224 cells; longer rows, Bloch
     * boundaries or overlapping CPML faces use the per-update kernels). With E2, H2 and every psi_e2 / psi_h2 set, each step
     * is one launch of the one-pass kernel, which reads one copy of everything and writes the
     * other. At the end the result is always back in E, H, psi_e, psi_h. When NULL, fdtd_run
     * uses the per-update kernels. Results are identical either way. */
    void *E2, *H2;
    void *psi_e2[6][2], *psi_h2[6][2];
} FdtdBuffers;

typedef struct FdtdPlan FdtdPlan;

/* Returns FDTD_ABI_VERSION. */
int fdtd_abi_version(void);

/* Last error message of the calling thread ("" if none). */
const char *fdtd_last_error(void);

/* Build a plan: validates the description and uploads the coefficient tables.
 * Replaces Simulation.__init__'s kernel generation (simulation.py:170-271). */
int fdtd_plan_create(const FdtdDesc *desc, FdtdPlan **out);
int fdtd_plan_destroy(FdtdPlan *plan);

/* Tuning keys of fdtd_plan_tune. Any values give the same results.
 *   XCHUNK        consecutive x planes one thread of the update kernels advances (default 8)
 *   SLAB          x planes per L2-resident slab of fdtd_run's per-update schedule
 *                 (default 0 = whole grid)
 *   FUSED_ROWS    own y rows of a tile of the one-pass step (default 0: the most that fit a
 *                 block, 11 for sz = 73 in float32)
 *   FUSED_XCHUNK  x planes one block of the one-pass step marches (default 0: whole waves of
 *                 one block per SM)
 *   FUSED_STAGES  planes in the one-pass step's shared-memory ring, 2..6 (default 0: 4); fewer
 *                 when the shared memory of a block cannot hold that many
 *   FUSED_TMA     1 (default): the one-pass step stages the rows of tiles that do not wrap around
 *                 the y boundary with bulk asynchronous copies when every staged buffer is
 *                 16-byte aligned; 0: per-element asynchronous copies everywhere
 *   FUSED_SHAPE   block shape of the one-pass step: 1 large (up to 1024 threads, one block per
 *                 SM), 2 small (up to 512 threads, two blocks per SM; float32 only), 0
 *                 (default) small when its tiles hold at least 3 own rows
 *   HS_XCHUNK     x planes one block of the H+S kernel of fdtd_run marches; 0 (default): chosen
 *                 per launch among 14..24 so that the grid best fills whole waves of resident
 *                 blocks (18 on the 395x345x73 grid of a 152-SM GPU)
 *   HS_PREFETCH   1: the H+S kernel loads the next plane ahead (one block per SM); 0: not
 *                 (two blocks per SM, the default)
 *   HS_REVERSE    1 (default): the H+S kernel takes its x chunks in descending order, so that it
 *                 starts on the planes update_E wrote last (still in L2); 0: ascending
 *   HS_DFT        1 (default): on the H+S path the step's DFT monitor sample is taken by one extra
 *                 block of the H+S launch; 0: by the monitor kernel on a side stream beside it
 *   PDL           1 (default): on the H+S path the E and H+S kernels are launched with
 *                 programmatic stream serialization (each may be scheduled while the kernel
 *                 before it finishes, and waits for it before touching memory); 0: plain stream
 *                 order
 *   E_FORM        form of the bulk E kernel: 0 loads the next x plane one iteration ahead at
 *                 three blocks of 256 threads per SM; 1 (default) loads each plane when it is
 *                 updated, at four blocks per SM (both give the same results)
 *   TIMING        1: fdtd_run records CUDA events around its kernels on up to 64 steps spread
 *                 over the call (update_E and H+S on the H+S path, the step kernel on the
 *                 one-pass path) and waits for the stream before it returns (profiling; read
 *                 with fdtd_run_kernel_ms); 0 (default) */
#define FDTD_TUNE_XCHUNK 1
#define FDTD_TUNE_SLAB 2
#define FDTD_TUNE_FUSED_ROWS 3
#define FDTD_TUNE_FUSED_XCHUNK 4
#define FDTD_TUNE_HS_XCHUNK 5
#define FDTD_TUNE_HS_PREFETCH 6
#define FDTD_TUNE_TIMING 7
#define FDTD_TUNE_FUSED_STAGES 8
#define FDTD_TUNE_FUSED_TMA 9
#define FDTD_TUNE_FUSED_SHAPE 10
#define FDTD_TUNE_HS_REVERSE 11
#define FDTD_TUNE_HS_DFT 13
#define FDTD_TUNE_PDL 14
#define FDTD_TUNE_E_FORM 15
/* Read-only keys of fdtd_plan_get: the path of the last fdtd_run (FDTD_PATH_*), the tiling
 * of its last one-pass launch (own rows per tile, x chunk, stages, threads per block, shape)
 * and the x chunk of its last H+S launch. */
#define FDTD_GET_LAST_RUN_PATH 100
#define FDTD_GET_STEP_ROWS 101
#define FDTD_GET_STEP_XCHUNK 102
#define FDTD_GET_STEP_STAGES 103
#define FDTD_GET_STEP_THREADS 104
#define FDTD_GET_STEP_SHAPE 105
#define FDTD_GET_HS_XCHUNK_USED 106
#define FDTD_PATH_NONE 0
#define FDTD_PATH_PER_UPDATE 1     /* update_E, sources, update_H, update_S launches */
#define FDTD_PATH_HS 2             /* update_E in place, sources, H and S in one launch */
#define FDTD_PATH_ONEPASS 3        /* E, sources, H and S of a step in one launch */
int fdtd_plan_tune(FdtdPlan *plan, int32_t key, int32_t value);
/* Current value of a tuning key. */
int fdtd_plan_get(const FdtdPlan *plan, int32_t key, int32_t *value);

/* Fill buf->ce = dt/eps and, with has_mu, buf->cm = dt/mu (IEEE division, the quotient
 * the reference computes per cell). Call after creating or changing eps/mu. */
int fdtd_prepare(FdtdPlan *plan, const FdtdBuffers *buf, void *stream);

/* update_E (simulation.py:254; opencl_fdtd/kernels/update_e.cl): E += dt/eps * (curl H + psi),
 * advancing psi_e. With Bloch boundaries it reads G at the wrapped faces. */
int fdtd_update_e(FdtdPlan *plan, const FdtdBuffers *buf, void *stream);
/* update_H (simulation.py:255; update_h.cl): H -= dt[/mu] * (curl E - psi), advancing psi_h,
 * and writes oS when do_poynting. With Bloch boundaries it reads F at the wrapped faces. */
int fdtd_update_h(FdtdPlan *plan, const FdtdBuffers *buf, void *stream);
/* update_S (simulation.py:256-257; update_s.cl): S = dt/8 * (sum of four oS terms). */
int fdtd_update_s(FdtdPlan *plan, const FdtdBuffers *buf, void *stream);
/* update_F / update_G (simulation.py:258-264): the imaginary halves of a Bloch pair,
 * advancing psi_f / psi_g. */
int fdtd_update_f(FdtdPlan *plan, const FdtdBuffers *buf, void *stream);
int fdtd_update_g(FdtdPlan *plan, const FdtdBuffers *buf, void *stream);
/* update_J (simulation.py:265-271; update_j.cl): E += c*Jr + s*Ji for
 * box = {xmin, xmax, ymin, ymax, zmin, zmax} (half-open, clipped to the grid). */
int fdtd_update_j(FdtdPlan *plan, const FdtdBuffers *buf, void *stream, double c, double s,
                  const int64_t box[6]);

/* Point sources for fdtd_run: after the E update of step t, E[index[k]] += values[t*n + k]
 * (the host-side `sim.E[ind] += field_source(t)` of opencl_fdtd's fdtd.py:168-169, moved on
 * the device; sources on one cell are added in list order). index holds flat indices into
 * the 3N E array in HOST memory (n <= 64); values is a DEVICE array of nsteps*n elements in
 * the plan's dtype. */
typedef struct FdtdPointSources {
    int32_t n;
    int32_t _pad;
    const int64_t *index;    /* host, n entries */
    const void *values;      /* device, nsteps * n entries */
} FdtdPointSources;

/* FP64 DFT point monitor. After each step (E fully updated, point sources included) the
 * sample x = E[index[p]] is taken at time (step + 1) * dt and accum[p][f] += x *
 * exp(-i omega[f] (step + 1) dt) in double; with series set, x is also stored in row
 * series_row of series ([rows][n_points] doubles). All pointers are device pointers. */
typedef struct FdtdDftMonitor {
    int32_t n_points, n_freq;
    const int64_t *index;    /* n_points flat indices into the 3N E array */
    const double *omega;     /* n_freq angular frequencies, radians per unit time */
    double *accum;           /* n_points * n_freq * 2 doubles (re, im) */
    double *series;          /* NULL or rows * n_points doubles */
    int64_t step;            /* step index of the next sample */
    int64_t series_row;      /* series row of the next sample */
} FdtdDftMonitor;

/* Take one sample of a monitor (for per-call loops); advance mon->step and mon->series_row
 * yourself. */
int fdtd_monitor_sample(FdtdPlan *plan, const FdtdBuffers *buf, void *stream,
                        const FdtdDftMonitor *mon);

/* Deterministic FP64 sum over one plane of one component of a 3N field (field = E, H, S or
 * any caller array of that layout): component 0..2, axis 0..2 normal to the plane, plane
 * index along that axis. Two stages: per-block partial sums into scratch (scratch_len
 * doubles, device; more gives more parallelism, the result does not depend on it beyond
 * rounding of a fixed order), then one block folds them into *out (device double). */
int fdtd_plane_sum(FdtdPlan *plan, const void *field, int32_t component, int32_t axis,
                   int64_t plane, double *scratch, int32_t scratch_len, double *out, void *stream);

/* fdtd_plane_sum without allocation — no counterpart in the reference, which has no
 * monitors. For callers that must not allocate device memory between steps (a host driver
 * that has given the device memory to its own pool, or a callback between queued steps where
 * cudaMalloc/cudaFree would synchronize the device): the nblocks per-block partial sums go to
 * a static device array of this library (at most 1024 doubles, 8 KB, held on every GPU that
 * loads the library until exit) instead of caller scratch. nblocks must be in [1, 1024];
 * larger values are rejected with FDTD_ERR_INVALID. The first call on a device resolves the
 * array's device address (cudaGetSymbolAddress), so make it before any stream capture. Every
 * call writes the partials it reads (nothing needs clearing; the array keeps the last call's
 * values); calls share the array, so calls whose kernels overlap on the GPU race. */
int fdtd_plane_sum_noalloc(FdtdPlan *plan, const void *field, int32_t component, int32_t axis,
                           int64_t plane, int32_t nblocks, double *out, void *stream);

/* Deterministic FP64 total field energy 1/2 sum(eps E^2 + mu H^2) (mu = 1 without mu; PEC
 * cells hold none), with the same two-stage scheme into *out (device double). */
int fdtd_energy(FdtdPlan *plan, const FdtdBuffers *buf, double *scratch, int32_t scratch_len,
                double *out, void *stream);

/* Field watchdog: *count (a device uint32, cleared here) receives the number of NaN / Inf
 * values in E and H (and F, G with Bloch boundaries), on the stream; a caller that finds it
 * nonzero reports FDTD_ERR_NONFINITE. No trap, no host wait inside. */
int fdtd_count_nonfinite(FdtdPlan *plan, const FdtdBuffers *buf, uint32_t *count, void *stream);

/* Run nsteps canonical steps (fdtd.py:162-175: E, F, point sources, H, G, S) on the stream
 * with no host round trip. src and mon may be NULL; mon is sampled after every step and its
 * step / series_row advance by nsteps. With the second copies of FdtdBuffers set (and no
 * Bloch boundaries, at most 8 sources, no overlapping CPML faces) each step is two launches
 * (H2 and psi_h2: update_E in place, then H and S) or one (E2, H2 and every psi copy: the
 * one-pass step); oS is then written on the last step only. The path taken is read back with
 * fdtd_plan_get(FDTD_GET_LAST_RUN_PATH). On the H+S path the E kernel adds up to 8 point
 * sources itself (without a learned boundary), the monitor sample of each step is taken by
 * one extra block of the H+S launch (FDTD_TUNE_HS_DFT; 0: by the monitor kernel on a stream of
 * the plan beside the H+S launch, joined back into `stream` before the call returns), and the
 * two kernels use programmatic dependent launch (FDTD_TUNE_PDL). */
int fdtd_run(FdtdPlan *plan, const FdtdBuffers *buf, void *stream, int32_t nsteps,
             const FdtdPointSources *src, FdtdDftMonitor *mon);

/* Mean launch time in ms over the sampled steps of the last fdtd_run made with FDTD_TUNE_TIMING
 * on: update_E (ms[0]) and the H+S kernel (ms[1]) on the H+S path, the step kernel (ms[0]; ms[1]
 * = 0) on the one-pass path; and the number of samples (0 if none). Profiling aid; no
 * counterpart in the reference. */
int fdtd_run_kernel_ms(const FdtdPlan *plan, double ms[2], int32_t *samples);

/* Device status of the plan's kernels: every wait for staged data inside the one-pass step is
 * bounded, and one that runs out sets a bit here (4) and ends its block. Waits for the stream,
 * stores the bits in *bits, clears them and returns FDTD_ERR_WATCHDOG when any was set. No
 * counterpart in the reference. */
int fdtd_device_status(FdtdPlan *plan, void *stream, int32_t *bits);

/* ---- batched stepping of many independent variants (one persistent launch) ---------------
 * No counterpart in the reference, which steps one grid per Simulation. Each variant is a
 * grid with diagonal eps (no mu, no Bloch boundaries, no Poynting, uniform dx) whose E, H and
 * dt/eps arrays are stored in float32, bfloat16 or float16 (arithmetic is float32 in every
 * case); the CPML psi arrays are float32. With float32 storage the results are bit-identical
 * to stepping each variant on its own with fdtd_run. In 16-bit storage every run of 32
 * consecutive (y, z) cells of one component in one x plane carries a power-of-two exponent e
 * (stored = value * 2^-e), chosen when the run is written. e_exp / h_exp are int32
 * [sx][ceil(sy*sz/32)]: one word per run holds the three components' exponents as the bytes
 * e_c + 128 at bits 8c .. 8c + 7. FDTD_STORE_BF16U stores bfloat16 without exponents
 * (bfloat16 has float32's exponent range, so a tile exponent changes none of its roundings
 * short of the subnormal range) and takes no e_exp / h_exp. */
#define FDTD_STORE_F32 0
#define FDTD_STORE_BF16 1
#define FDTD_STORE_F16 2
#define FDTD_STORE_BF16U 3
#define FDTD_BATCH_MAX_SRC 4
#define FDTD_BATCH_MAX_MON 8

typedef struct FdtdBatchFace {
    int32_t axis, polarity, thickness, _pad;
    const float *tab_e[3], *tab_h[3];  /* device p0 p1 p2 of the E and H updates, T each */
    float *psi_e[2], *psi_h[2];        /* device psi (u, v) of the face, layout of FdtdBuffers */
} FdtdBatchFace;

typedef struct FdtdBatchVariant {
    int32_t shape[3], n_pml;
    double dt, dx;
    FdtdBatchFace pml[6];
    void *E, *H;                       /* device 3N each, storage type */
    const void *ce;                    /* device 3N dt/eps, storage type */
    int32_t *e_exp, *h_exp;            /* device tile exponents (16-bit storage), else NULL */
    int32_t n_src, n_mon;
    int64_t src_index[FDTD_BATCH_MAX_SRC];   /* flat indices into E (c*N + cell) */
    const float *src_values;           /* device [rows][n_src]: row = step number */
    int64_t mon_index[FDTD_BATCH_MAX_MON];   /* flat indices into E */
    double *series;                    /* device [rows][n_mon] or NULL: E after each step */
} FdtdBatchVariant;

typedef struct FdtdBatch FdtdBatch;

/* Validate n variants and build the tile list (x chunks of xchunk planes, default 8). rows:
 * rows of every variant's src_values / series (steps past it add no source, record nothing). */
int fdtd_batch_create(const FdtdBatchVariant *vars, int32_t n, int32_t storage, int64_t rows,
                      FdtdBatch **out);
int fdtd_batch_destroy(FdtdBatch *batch);
/* Tile shape and grid: x planes per tile (>= 1) and resident blocks per SM (0: the most that
 * fit). Rebuilds the tile list. */
int fdtd_batch_tune(FdtdBatch *batch, int32_t xchunk, int32_t blocks_per_sm);
/* Advance every variant by nsteps steps (E, sources, H per step) on the stream: with the
 * FDTD_BATCH_LAUNCHES schedule (default) as two launches per step, each covering the tiles of
 * every variant; with FDTD_BATCH_PERSISTENT as one cooperative launch for all nsteps steps.
 * The step counter lives on the device (read and advanced by the launches), so captured
 * launches keep counting when a CUDA graph replays them. */
#define FDTD_BATCH_PERSISTENT 0
#define FDTD_BATCH_LAUNCHES 1
int fdtd_batch_schedule(FdtdBatch *batch, int32_t schedule);
int fdtd_batch_run(FdtdBatch *batch, void *stream, int32_t nsteps);
/* Read / set the batch's device step counter (waits for the device). */
int fdtd_batch_get_step(FdtdBatch *batch, int64_t *step);
int fdtd_batch_set_step(FdtdBatch *batch, int64_t step);
/* 16-bit storage: float32 field (0 = E, 1 = H) of variant v -> storage with fresh tile
 * exponents, and back. */
int fdtd_batch_encode(FdtdBatch *batch, int32_t v, int32_t field, const float *src, void *stream);
int fdtd_batch_decode(FdtdBatch *batch, int32_t v, int32_t field, float *dst, void *stream);

/* ---- learned thin absorbing boundary ------------------------------------------------------
 * Replaces the CPML of selected faces (bit 2 * axis + side of face_mask; side 0 = index 0) by
 * a per-face MLP. Every column of a face (one cell of the face's plane) reads the six field
 * components (Ex Ey Ez Hx Hy Hz) on a 3 x 3 tangential patch two cells deep,
 * [depth][du + 1][dv + 1][component], with tangential neighbours past the grid clamped to its
 * edge. x = stencil / r with r its RMS; the network 108 -> 64 -> 64 -> 6 (GELU) maps x to the
 * six components of the ghost cell one step outside the face, divided by r. The grid's edges wrap; a boundary step is: the ghosts of every face from the
 * pre-step state E^n, H^{n+1/2} (H^{n+1/2} outside side-0 faces, E^{n+1} outside side-1
 * faces); E update; E fix-up; sources; H update; H fix-up (fdtd_lbc_fix). Edge cells get one
 * term per face they lie on.
 * Parameters: float32 [LBC_NPARAM] per face, W1 [108][64], b1 [64], W2 [64][64], b2 [64],
 * W3 [64][6], b3 [6] (row-major [in][out]); 6 faces in order 2 * axis + side. No reference
 * interface is replaced: opencl_fdtd absorbs only with CPML (simulation.py:274-319). */
#define FDTD_LBC_IN 108
#define FDTD_LBC_HID 64
#define FDTD_LBC_OUT 6
#define FDTD_LBC_NPARAM 11526
#define FDTD_LBC_PACK_WORDS 6024   /* bfloat16 tensor-core layout of one face, 32-bit words */
#define FDTD_LBC_F32 0              /* float32 weights, CUDA cores */
#define FDTD_LBC_BF16 1             /* bfloat16 weights and activations, tensor cores */
#define FDTD_LBC_BF16X2 2           /* bfloat16 weights, activations as two bfloat16 parts */
#define FDTD_LBC_LINEAR 3           /* an exactly linear layer: float32 [6][109][6], rows = the
                                       108 inputs then the bias; ghost = A^T stencil + r bias */

/* Columns of the faces in face_mask (whole planes); face_offsets[f] (f = 2 * axis + side) is
 * the first column of face f (-1 when absent), face_offsets[6] the total. face_offsets may be
 * NULL. Columns of a face run over its plane row-major in (u, v), the other axes in xyz order. */
int fdtd_lbc_columns(const int32_t shape[3], int32_t face_mask, int32_t *ncol, int32_t face_offsets[7]);
/* Training data of one state: X [ncol][108] = stencil / r, R [ncol] = r, C [ncol][6] = the
 * outermost cell's components (any of X, R, C may be NULL). */
int fdtd_lbc_gather(const int32_t shape[3], int32_t face_mask, const float *E, const float *H, float *X,
                    float *R, float *C, void *stream);
/* Training, float32, one network: forward of a batch keeps the pre-activations A1, A2 and
 * activations H1, H2 ([batch][64] each); backward gives the gradient of the mean over
 * batch x 6 of w_o (Y - T)^2 (out_weights: 6 device floats w_o, NULL = all 1) with respect to
 * the parameters (grad [LBC_NPARAM]), deterministic for a given batch; workspace floats from
 * fdtd_mlp_backward_workspace. */
int fdtd_mlp_forward(const float *params, const float *X, int32_t batch, float *Y, float *A1, float *A2,
                     float *H1, float *H2, void *stream);
int fdtd_mlp_backward_workspace(int32_t batch, int64_t *floats);
int fdtd_mlp_backward(const float *params, const float *X, const float *Y, const float *T,
                      const float *out_weights, int32_t batch, const float *A1, const float *A2, const float *H1,
                      const float *H2, float *grad, float *workspace, int64_t workspace_floats, void *stream);
/* out [(K + 1) x N] float32: A^T B in rows 0..K-1 and the column sums of B in row K, for
 * A [rows][K], B [rows][N] (the least-squares normal equations of the linear start of
 * training); deterministic (fixed partition of the rows, fixed folding order). (K + 1) N <=
 * 7168. Workspace floats from fdtd_gram_workspace. */
int fdtd_gram_workspace(int32_t rows, int32_t K, int32_t N, int64_t *floats);
int fdtd_gram(const float *A, int32_t rows, int32_t K, const float *B, int32_t N, float *out, float *workspace,
              int64_t workspace_floats, void *stream);
/* One Adam step (Kingma and Ba 2015, bias-corrected; step counts from 1) on n parameters. */
int fdtd_adam(float *params, const float *grad, float *m, float *v, int32_t n, float lr, float beta1,
              float beta2, float eps, int32_t step, void *stream);
/* float32 parameters [6][LBC_NPARAM] -> bfloat16 tensor-core layout [6][LBC_PACK_WORDS]. */
int fdtd_lbc_pack(const float *params, void *packed, void *stream);
/* Ghost values [ncol][6] of the faces of side `side` (-1: all): pred = r * (network output)
 * + memory * pred, pred holding the previous step's ghosts (zero before the first step);
 * weights: float32 parameters (FDTD_LBC_F32), the packed layout (BF16, BF16X2) or the linear
 * map of a layer that is exactly linear (FDTD_LBC_LINEAR). memory =
 * (1 - c dt) / (1 + c dt) makes room for Mur's first-order condition (its other terms are
 * linear in the stencil); memory = 0: ghosts from the current stencil alone. */
int fdtd_lbc_predict(const int32_t shape[3], int32_t face_mask, int32_t side, int32_t precision, float memory,
                     const void *weights, const float *E, const float *H, float *pred, int64_t pred_floats,
                     void *stream);
/* Replace, in the updates of the outermost cells, the wrapped neighbour by the ghost:
 * FDTD_LBC_FIX_E right after the E update, E_q += -e_qap ce_q (ghost H_p - wrapped H_p) for
 * every learned side-0 face of axis a through the cell (q, a, p distinct, e the Levi-Civita
 * sign, ce = dt / eps: 3N floats); FDTD_LBC_FIX_H after the H update, H_q += -e_qap ch_q
 * (ghost E_p - wrapped E_p) for every learned side-1 face (ch = cm, 3N floats dt / mu, or dt
 * when cm is NULL). Unit cells. One of the two per call. */
#define FDTD_LBC_FIX_E 1
#define FDTD_LBC_FIX_H 2
int fdtd_lbc_fix(const int32_t shape[3], int32_t face_mask, int32_t fields, const float *pred, float *E, float *H,
                 const float *ce, const float *cm, double dt, void *stream);
/* Make fdtd_run step the plan with the learned boundary (float32 plans with unit cells and no
 * Bloch boundaries; face_mask 0 detaches). weights and pred (ncol x 6 floats) stay owned by
 * the caller and must outlive the attachment. The faces in face_mask should carry no CPML;
 * columns of a learned face that lie inside the plan's other CPML faces get zero ghosts in
 * fdtd_run (fdtd_lbc_predict, which has no plan, predicts every column: a caller stepping by
 * hand zeroes those rows itself). */
int fdtd_lbc_attach(FdtdPlan *plan, int32_t face_mask, int32_t precision, float memory, const void *weights,
                    float *pred, int64_t pred_floats);

#ifdef __cplusplus
}
#endif

#endif /* FDTD_GB300_H */
