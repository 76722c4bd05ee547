// C ABI of the batched stepping path (fdtd_batch_*): validation, the device copy of the
// variant descriptors, the tile list and the cooperative launch.
#include <cstring>
#include <string>
#include <vector>

#include "fdtd_gb300.h"
#include "fdtd_plan.h"
#include "batch.h"

static_assert(FDTD_STORE_F32 == fdtd::BATCH_F32 && FDTD_STORE_BF16 == fdtd::BATCH_BF16 &&
                  FDTD_STORE_F16 == fdtd::BATCH_F16 && FDTD_STORE_BF16U == fdtd::BATCH_BF16U,
              "storage codes");

using namespace fdtd;

struct FdtdBatch {
    int storage;
    int device;
    int64_t rows;
    uint32_t xchunk;
    int blocks_per_sm;
    int schedule;                // FDTD_BATCH_PERSISTENT or FDTD_BATCH_LAUNCHES
    std::vector<BVar> host;      // descriptors as uploaded
    BVar *vars = nullptr;        // device copy
    int4 *tiles = nullptr;       // device tile list
    uint32_t ntiles = 0;
    int64_t *step = nullptr;     // device step counter
    uint32_t *work = nullptr;    // persistent schedule's two tile counters
};

namespace {

int fail(int code, const std::string &msg) { return set_error(code, msg.c_str()); }

int build_tiles(FdtdBatch *b)
{
    std::vector<int4> t;
    for (size_t v = 0; v < b->host.size(); ++v) {
        const BVar &h = b->host[v];
        for (uint32_t x0 = 0; x0 < h.sx; x0 += b->xchunk)
            for (uint32_t jb = 0; jb < h.njb; ++jb)
                t.push_back(make_int4((int)v, (int)x0, (int)(x0 + b->xchunk < h.sx ? x0 + b->xchunk : h.sx), (int)jb));
    }
    if (b->tiles) cudaFree(b->tiles);
    b->tiles = nullptr;
    int rc = check_cuda(cudaMalloc(&b->tiles, t.size() * sizeof(int4)), "cudaMalloc(batch tiles)");
    if (rc) return rc;
    rc = check_cuda(cudaMemcpy(b->tiles, t.data(), t.size() * sizeof(int4), cudaMemcpyHostToDevice), "copy batch tiles");
    if (rc) return rc;
    b->ntiles = (uint32_t)t.size();
    return FDTD_OK;
}

int make_var(const FdtdBatchVariant &d, int storage, BVar &v, int idx)
{
    const std::string who = "batch variant " + std::to_string(idx) + ": ";
    std::memset(&v, 0, sizeof(v));
    for (int r = 0; r < 3; ++r)
        if (d.shape[r] < 1) return fail(FDTD_ERR_INVALID, who + "shape must be positive");
    v.sx = (uint32_t)d.shape[0];
    v.sy = (uint32_t)d.shape[1];
    v.sz = (uint32_t)d.shape[2];
    const uint64_t syz = (uint64_t)v.sy * v.sz, N = syz * v.sx;
    if (3 * N >= (1ull << 32)) return fail(FDTD_ERR_UNSUPPORTED, who + "grid too large for 32-bit cell indices");
    v.syz = (uint32_t)syz;
    v.N = N;
    v.njb = (uint32_t)((syz + BATCH_THREADS - 1) / BATCH_THREADS);
    v.ntl = (uint32_t)((syz + BATCH_TILE - 1) / BATCH_TILE);
    v.dsz = FastDiv::make(v.sz);
    if (!(d.dt > 0.0) || !(d.dx > 0.0)) return fail(FDTD_ERR_INVALID, who + "dt and dx must be positive");
    v.dt = (float)d.dt;
    v.inv_d = (float)(1.0 / d.dx);
    v.dxmode = v.inv_d == 1.0f ? 0 : 1;
    if (!d.E || !d.H || !d.ce) return fail(FDTD_ERR_INVALID, who + "E, H and ce are required");
    v.E = d.E;
    v.H = d.H;
    v.ce = d.ce;
    const bool scaled = storage == BATCH_BF16 || storage == BATCH_F16;
    if (scaled && (!d.e_exp || !d.h_exp))
        return fail(FDTD_ERR_INVALID, who + "16-bit storage with tile exponents needs e_exp and h_exp");
    v.eexp = scaled ? d.e_exp : nullptr;
    v.hexp = scaled ? d.h_exp : nullptr;
    if (d.n_pml < 0 || d.n_pml > 6) return fail(FDTD_ERR_INVALID, who + "n_pml must be in [0, 6]");
    int seen = 0;
    uint32_t tn[3] = {0, 0, 0}, tp[3] = {0, 0, 0};
    const uint32_t s[3] = {v.sx, v.sy, v.sz};
    for (int f = 0; f < d.n_pml; ++f) {
        const FdtdBatchFace &pf = d.pml[f];
        if (pf.axis < 0 || pf.axis > 2 || pf.polarity < 0 || pf.polarity > 1 || pf.thickness < 0)
            return fail(FDTD_ERR_INVALID, who + "bad pml face");
        const int bit = 1 << (2 * pf.axis + pf.polarity);
        if (seen & bit) return fail(FDTD_ERR_INVALID, who + "duplicate pml face");
        seen |= bit;
        if (pf.thickness == 0) continue;
        const uint32_t T = (uint32_t)pf.thickness, a = (uint32_t)pf.axis;
        if (pf.polarity == 1 && T > s[a]) continue;   // never applies (the reference's s - T wraps)
        for (int c = 0; c < 3; ++c)
            if (!pf.tab_e[c] || !pf.tab_h[c]) return fail(FDTD_ERR_INVALID, who + "pml table pointer is NULL");
        for (int c = 0; c < 2; ++c)
            if (!pf.psi_e[c] || !pf.psi_h[c]) return fail(FDTD_ERR_INVALID, who + "psi pointer is NULL");
        BAxis &ax = v.ax[a];
        if (pf.polarity == 0) { ax.Tn = (int32_t)T; tn[a] = T; }
        else { ax.Tp = (int32_t)T; tp[a] = T; }
        for (int c = 0; c < 3; ++c) {
            ax.tab[0][pf.polarity][c] = pf.tab_e[c];
            ax.tab[1][pf.polarity][c] = pf.tab_h[c];
        }
        for (int c = 0; c < 2; ++c) {
            ax.psi[0][pf.polarity][c] = pf.psi_e[c];
            ax.psi[1][pf.polarity][c] = pf.psi_h[c];
        }
    }
    for (int r = 0; r < 3; ++r)
        if (tn[r] + tp[r] > s[r])
            return fail(FDTD_ERR_UNSUPPORTED, who + "CPML faces of one axis overlap (not supported in a batch)");
    if (d.n_src < 0 || d.n_src > BATCH_MAX_SRC) return fail(FDTD_ERR_INVALID, who + "at most 4 point sources");
    if (d.n_mon < 0 || d.n_mon > BATCH_MAX_MON) return fail(FDTD_ERR_INVALID, who + "at most 8 monitor points");
    if (d.n_src && !d.src_values) return fail(FDTD_ERR_INVALID, who + "src_values is NULL");
    if (d.n_mon && !d.series) return fail(FDTD_ERR_INVALID, who + "series is NULL");
    v.nsrc = d.n_src;
    v.nmon = d.n_mon;
    v.src_values = d.src_values;
    v.series = d.series;
    for (int k = 0; k < d.n_src; ++k) {
        const int64_t i = d.src_index[k];
        if (i < 0 || (uint64_t)i >= 3 * N) return fail(FDTD_ERR_INVALID, who + "source index out of range");
        v.src_c[k] = (int32_t)((uint64_t)i / N);
        const uint64_t cell = (uint64_t)i % N;
        v.src_x[k] = (uint32_t)(cell / syz);
        v.src_j[k] = (uint32_t)(cell % syz);
    }
    for (int k = 0; k < d.n_mon; ++k) {
        const int64_t i = d.mon_index[k];
        if (i < 0 || (uint64_t)i >= 3 * N) return fail(FDTD_ERR_INVALID, who + "monitor index out of range");
        v.mon_c[k] = (int32_t)((uint64_t)i / N);
        const uint64_t cell = (uint64_t)i % N;
        v.mon_x[k] = (uint32_t)(cell / syz);
        v.mon_j[k] = (uint32_t)(cell % syz);
    }
    return FDTD_OK;
}

int max_blocks(int storage)
{
    if (storage == BATCH_BF16) return batch_max_blocks_per_sm<BATCH_BF16>();
    if (storage == BATCH_F16) return batch_max_blocks_per_sm<BATCH_F16>();
    if (storage == BATCH_BF16U) return batch_max_blocks_per_sm<BATCH_BF16U>();
    return batch_max_blocks_per_sm<BATCH_F32>();
}

}  // namespace

extern "C" {

int fdtd_batch_create(const FdtdBatchVariant *vars, int32_t n, int32_t storage, int64_t rows,
                      FdtdBatch **out)
{
    if (!out) return fail(FDTD_ERR_INVALID, "fdtd_batch_create: out is NULL");
    *out = nullptr;
    if (!vars || n < 1) return fail(FDTD_ERR_INVALID, "fdtd_batch_create: no variants");
    if (storage != BATCH_F32 && storage != BATCH_BF16 && storage != BATCH_F16 && storage != BATCH_BF16U)
        return fail(FDTD_ERR_INVALID, "fdtd_batch_create: storage must be FDTD_STORE_F32, _BF16, _F16 or _BF16U");
    if (rows < 0) return fail(FDTD_ERR_INVALID, "fdtd_batch_create: rows must be >= 0");
    FdtdBatch *b = new FdtdBatch();
    b->storage = storage;
    b->rows = rows;
    b->xchunk = 8;
    b->blocks_per_sm = 0;
    b->schedule = FDTD_BATCH_LAUNCHES;
    cudaGetDevice(&b->device);
    b->host.resize((size_t)n);
    int rc = FDTD_OK;
    for (int v = 0; v < n && !rc; ++v) rc = make_var(vars[v], storage, b->host[v], v);
    if (!rc) rc = check_cuda(cudaMalloc(&b->vars, b->host.size() * sizeof(BVar)), "cudaMalloc(batch variants)");
    if (!rc)
        rc = check_cuda(cudaMemcpy(b->vars, b->host.data(), b->host.size() * sizeof(BVar), cudaMemcpyHostToDevice),
                        "copy batch variants");
    if (!rc) rc = check_cuda(cudaMalloc(&b->step, sizeof(int64_t)), "cudaMalloc(batch step)");
    if (!rc) rc = check_cuda(cudaMemset(b->step, 0, sizeof(int64_t)), "clear batch step");
    if (!rc) rc = check_cuda(cudaMalloc(&b->work, 2 * sizeof(uint32_t)), "cudaMalloc(batch work counters)");
    if (!rc) rc = check_cuda(cudaMemset(b->work, 0, 2 * sizeof(uint32_t)), "clear batch work counters");
    if (!rc) rc = build_tiles(b);
    if (rc) {
        fdtd_batch_destroy(b);
        return rc;
    }
    *out = b;
    return FDTD_OK;
}

int fdtd_batch_destroy(FdtdBatch *b)
{
    if (!b) return FDTD_OK;
    if (b->vars) cudaFree(b->vars);
    if (b->tiles) cudaFree(b->tiles);
    if (b->step) cudaFree(b->step);
    if (b->work) cudaFree(b->work);
    delete b;
    return FDTD_OK;
}

int fdtd_batch_tune(FdtdBatch *b, int32_t xchunk, int32_t blocks_per_sm)
{
    if (!b) return fail(FDTD_ERR_INVALID, "batch is NULL");
    if (xchunk < 1 || xchunk > 4096) return fail(FDTD_ERR_INVALID, "xchunk must be in [1, 4096]");
    if (blocks_per_sm < 0 || blocks_per_sm > 32) return fail(FDTD_ERR_INVALID, "blocks_per_sm must be in [0, 32]");
    b->blocks_per_sm = blocks_per_sm;
    if ((uint32_t)xchunk != b->xchunk) {
        b->xchunk = (uint32_t)xchunk;
        return build_tiles(b);
    }
    return FDTD_OK;
}

int fdtd_batch_run(FdtdBatch *b, void *stream, int32_t nsteps)
{
    if (!b) return fail(FDTD_ERR_INVALID, "batch is NULL");
    if (nsteps < 0) return fail(FDTD_ERR_INVALID, "nsteps must be >= 0");
    if (nsteps == 0) return FDTD_OK;
    int nsm = 0;
    int rc = check_cuda(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, b->device), "SM count");
    if (rc) return rc;
    const int fit = max_blocks(b->storage);
    if (fit < 1) return fail(FDTD_ERR_CUDA, "batch kernel does not fit on an SM");
    const int per = b->blocks_per_sm > 0 && b->blocks_per_sm < fit ? b->blocks_per_sm : fit;
    BatchK k;
    k.vars = b->vars;
    k.tiles = b->tiles;
    k.ntiles = b->ntiles;
    k.nsteps = nsteps;
    k.step = b->step;
    k.rows = b->rows;
    k.work = b->work;
    cudaStream_t st = (cudaStream_t)stream;
    cudaError_t e;
    if (b->schedule == FDTD_BATCH_LAUNCHES) {
        if (b->storage == BATCH_BF16) e = launch_batch_steps<BATCH_BF16>(k, st);
        else if (b->storage == BATCH_F16) e = launch_batch_steps<BATCH_F16>(k, st);
        else if (b->storage == BATCH_BF16U) e = launch_batch_steps<BATCH_BF16U>(k, st);
        else e = launch_batch_steps<BATCH_F32>(k, st);
        return check_cuda(e, "batch launch");
    }
    if (b->storage == BATCH_BF16) e = launch_batch<BATCH_BF16>(k, per * nsm, st);
    else if (b->storage == BATCH_F16) e = launch_batch<BATCH_F16>(k, per * nsm, st);
    else if (b->storage == BATCH_BF16U) e = launch_batch<BATCH_BF16U>(k, per * nsm, st);
    else e = launch_batch<BATCH_F32>(k, per * nsm, st);
    return check_cuda(e, "batch launch");
}

int fdtd_batch_schedule(FdtdBatch *b, int32_t schedule)
{
    if (!b) return fail(FDTD_ERR_INVALID, "batch is NULL");
    if (schedule != FDTD_BATCH_PERSISTENT && schedule != FDTD_BATCH_LAUNCHES)
        return fail(FDTD_ERR_INVALID, "schedule must be FDTD_BATCH_PERSISTENT or FDTD_BATCH_LAUNCHES");
    b->schedule = schedule;
    return FDTD_OK;
}

int fdtd_batch_get_step(FdtdBatch *b, int64_t *step)
{
    if (!b || !step) return fail(FDTD_ERR_INVALID, "fdtd_batch_get_step: NULL pointer");
    return check_cuda(cudaMemcpy(step, b->step, sizeof(int64_t), cudaMemcpyDeviceToHost), "read batch step");
}

int fdtd_batch_set_step(FdtdBatch *b, int64_t step)
{
    if (!b) return fail(FDTD_ERR_INVALID, "batch is NULL");
    if (step < 0) return fail(FDTD_ERR_INVALID, "step must be >= 0");
    return check_cuda(cudaMemcpy(b->step, &step, sizeof(int64_t), cudaMemcpyHostToDevice), "set batch step");
}

int fdtd_batch_encode(FdtdBatch *b, int32_t v, int32_t field, const float *src, void *stream)
{
    if (!b || !src) return fail(FDTD_ERR_INVALID, "fdtd_batch_encode: NULL pointer");
    if (b->storage == BATCH_F32) return fail(FDTD_ERR_INVALID, "fdtd_batch_encode: float32 storage has no encoding");
    if (v < 0 || (size_t)v >= b->host.size() || field < 0 || field > 1)
        return fail(FDTD_ERR_INVALID, "fdtd_batch_encode: bad variant or field");
    return check_cuda(launch_batch_encode(b->storage, b->host[(size_t)v], field, src, (cudaStream_t)stream), "batch encode");
}

int fdtd_batch_decode(FdtdBatch *b, int32_t v, int32_t field, float *dst, void *stream)
{
    if (!b || !dst) return fail(FDTD_ERR_INVALID, "fdtd_batch_decode: NULL pointer");
    if (b->storage == BATCH_F32) return fail(FDTD_ERR_INVALID, "fdtd_batch_decode: float32 storage has no encoding");
    if (v < 0 || (size_t)v >= b->host.size() || field < 0 || field > 1)
        return fail(FDTD_ERR_INVALID, "fdtd_batch_decode: bad variant or field");
    return check_cuda(launch_batch_decode(b->storage, b->host[(size_t)v], field, dst, (cudaStream_t)stream), "batch decode");
}

}  // extern "C"
