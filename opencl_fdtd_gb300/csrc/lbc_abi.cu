// C ABI of the learned boundary (fdtd_lbc_*, fdtd_mlp_*): argument checks around lbc.cu.
#include <cstdint>
#include <string>

#include "fdtd_gb300.h"
#include "fdtd_plan.h"
#include "lbc.h"

using namespace fdtd;

static_assert(FDTD_LBC_IN == LBC_IN && FDTD_LBC_HID == LBC_HID && FDTD_LBC_OUT == LBC_OUT, "stencil sizes");
static_assert(FDTD_LBC_NPARAM == LBC_NPARAM && FDTD_LBC_PACK_WORDS == LBC_PACK_WORDS, "parameter layout");
static_assert(FDTD_LBC_FIX_E == LBC_FIX_E && FDTD_LBC_FIX_H == LBC_FIX_H, "fix-up fields");
static_assert(FDTD_LBC_F32 == LBC_F32 && FDTD_LBC_BF16 == LBC_BF16 && FDTD_LBC_BF16X2 == LBC_BF16X2 &&
                  FDTD_LBC_LINEAR == LBC_LINEAR, "precision");

namespace {

int bad(const char *msg) { return set_error(FDTD_ERR_INVALID, msg); }

bool shape_ok(const int32_t shape[3])
{
    if (!shape) return false;
    for (int r = 0; r < 3; ++r)
        if (shape[r] < 2) return false;
    return (uint64_t)shape[0] * shape[1] * shape[2] * 3 < (1ull << 32);
}

LGrid grid_of(const int32_t shape[3], int32_t mask)
{
    const uint32_t s[3] = {(uint32_t)shape[0], (uint32_t)shape[1], (uint32_t)shape[2]};
    return lbc_grid(s, mask);
}

}  // namespace

namespace fdtd {

// the plan's learned faces, with the columns inside its CPML faces left to zero ghosts
static LGrid plan_grid(const FdtdPlan *p)
{
    const uint32_t s[3] = {p->sx, p->sy, p->sz};
    uint32_t lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};
    for (int f = 0; f < p->d.n_pml; ++f) {
        const FdtdPmlDesc &pd = p->d.pml[f];
        if (pd.thickness <= 0) continue;
        if (pd.polarity == 0) lo[pd.axis] = (uint32_t)pd.thickness;
        else hi[pd.axis] = (uint32_t)pd.thickness;
    }
    return lbc_grid_window(s, p->lbc_mask, lo, hi);
}

int lbc_before_e(const FdtdPlan *p, const FdtdBuffers *b, const void *H, cudaStream_t st)
{
    if (!p->lbc_mask) return FDTD_OK;
    return check_cuda(launch_lbc_predict(plan_grid(p), -1, p->lbc_precision, p->lbc_memory, p->lbc_w,
                                         (const float *)b->E, (const float *)H, p->lbc_pred, st),
                      "lbc predict launch");
}

int lbc_after_e(const FdtdPlan *p, const FdtdBuffers *b, const void *H, cudaStream_t st)
{
    if (!p->lbc_mask) return FDTD_OK;
    return check_cuda(launch_lbc_fix(plan_grid(p), LBC_FIX_E, p->lbc_pred, (float *)b->E, (float *)H,
                                     (const float *)b->ce, nullptr, (float)p->d.dt, st), "lbc fix launch");
}

int lbc_after_h(const FdtdPlan *p, const FdtdBuffers *b, void *H, cudaStream_t st)
{
    if (!p->lbc_mask) return FDTD_OK;
    return check_cuda(launch_lbc_fix(plan_grid(p), LBC_FIX_H, p->lbc_pred, (float *)b->E, (float *)H, nullptr,
                                     p->d.has_mu ? (const float *)b->cm : nullptr, (float)p->d.dt, st),
                      "lbc fix launch");
}

}  // namespace fdtd

extern "C" {

int fdtd_lbc_columns(const int32_t shape[3], int32_t face_mask, int32_t *ncol, int32_t face_offsets[7])
{
    if (!shape_ok(shape)) return bad("fdtd_lbc_columns: every extent must be >= 2");
    if (face_mask < 0 || face_mask > 63) return bad("fdtd_lbc_columns: face_mask must be in [0, 63]");
    if (!ncol) return bad("fdtd_lbc_columns: ncol is NULL");
    const LGrid g = grid_of(shape, face_mask);
    *ncol = (int32_t)g.ncol;
    if (face_offsets) {
        // offsets of the columns of face f = 2 * axis + side (-1 when the face is not in the mask)
        for (int f = 0; f < 7; ++f) face_offsets[f] = -1;
        for (int i = 0; i < g.nface; ++i) face_offsets[2 * g.face[i].axis + g.face[i].side] = (int32_t)g.face[i].col0;
        face_offsets[6] = (int32_t)g.ncol;
    }
    return FDTD_OK;
}

int fdtd_lbc_gather(const int32_t shape[3], int32_t face_mask, const float *E, const float *H, float *X,
                    float *R, float *C, void *stream)
{
    if (!shape_ok(shape)) return bad("fdtd_lbc_gather: every extent must be >= 2");
    if (!E || !H) return bad("fdtd_lbc_gather: E and H are required");
    return check_cuda(launch_lbc_gather(grid_of(shape, face_mask), E, H, X, R, C, (cudaStream_t)stream),
                      "lbc gather launch");
}

int fdtd_mlp_forward(const float *params, const float *X, int32_t batch, float *Y, float *A1, float *A2,
                     float *H1, float *H2, void *stream)
{
    if (!params || !X || !Y || !A1 || !A2 || !H1 || !H2) return bad("fdtd_mlp_forward: NULL pointer");
    if (batch < 0) return bad("fdtd_mlp_forward: batch must be >= 0");
    return check_cuda(launch_mlp_fwd(params, X, batch, Y, A1, A2, H1, H2, (cudaStream_t)stream), "mlp forward launch");
}

int fdtd_mlp_backward_workspace(int32_t batch, int64_t *floats)
{
    if (batch < 0 || !floats) return bad("fdtd_mlp_backward_workspace: bad argument");
    *floats = (int64_t)mlp_bwd_workspace(batch);
    return FDTD_OK;
}

int fdtd_mlp_backward(const float *params, const float *X, const float *Y, const float *T,
                      const float *out_weights, int32_t batch, const float *A1, const float *A2, const float *H1,
                      const float *H2, float *grad, float *workspace, int64_t workspace_floats, void *stream)
{
    if (!params || !X || !Y || !T || !A1 || !A2 || !H1 || !H2 || !grad || !workspace)
        return bad("fdtd_mlp_backward: NULL pointer");
    if (batch < 1) return bad("fdtd_mlp_backward: batch must be >= 1");
    if (workspace_floats < (int64_t)mlp_bwd_workspace(batch)) return bad("fdtd_mlp_backward: workspace too small");
    return check_cuda(launch_mlp_bwd(params, X, Y, T, out_weights, batch, A1, A2, H1, H2, grad, workspace,
                                     (cudaStream_t)stream),
                      "mlp backward launch");
}

int fdtd_gram_workspace(int32_t rows, int32_t K, int32_t N, int64_t *floats)
{
    if (rows < 0 || K < 1 || N < 1 || !floats) return bad("fdtd_gram_workspace: bad argument");
    *floats = (int64_t)gram_workspace(rows, K, N);
    return FDTD_OK;
}

int fdtd_gram(const float *A, int32_t rows, int32_t K, const float *B, int32_t N, float *out, float *workspace,
              int64_t workspace_floats, void *stream)
{
    if (!A || !B || !out || !workspace) return bad("fdtd_gram: NULL pointer");
    if (rows < 1 || K < 1 || N < 1) return bad("fdtd_gram: rows, K and N must be >= 1");
    if ((int64_t)(K + 1) * N > 28 * 256) return bad("fdtd_gram: (K + 1) * N must be <= 7168");
    if ((int64_t)32 * (K + N) * 4 > 48 * 1024) return bad("fdtd_gram: K + N too large");
    if (workspace_floats < (int64_t)gram_workspace(rows, K, N)) return bad("fdtd_gram: workspace too small");
    return check_cuda(launch_gram(A, rows, K, B, N, out, workspace, (cudaStream_t)stream), "gram launch");
}

int fdtd_adam(float *params, const float *grad, float *m, float *v, int32_t n, float lr, float beta1, float beta2,
              float eps, int32_t step, void *stream)
{
    if (!params || !grad || !m || !v) return bad("fdtd_adam: NULL pointer");
    if (n < 0 || step < 1) return bad("fdtd_adam: n must be >= 0 and step >= 1");
    return check_cuda(launch_adam(params, grad, m, v, n, lr, beta1, beta2, eps, step, (cudaStream_t)stream),
                      "adam launch");
}

int fdtd_lbc_pack(const float *params, void *packed, void *stream)
{
    if (!params || !packed) return bad("fdtd_lbc_pack: NULL pointer");
    if ((uintptr_t)packed % 16) return bad("fdtd_lbc_pack: packed must be 16-byte aligned");
    return check_cuda(launch_lbc_pack(params, (uint32_t *)packed, (cudaStream_t)stream), "lbc pack launch");
}

static int check_weights(int32_t precision, const void *weights, const char *what)
{
    if (precision != FDTD_LBC_F32 && precision != FDTD_LBC_BF16 && precision != FDTD_LBC_BF16X2 &&
        precision != FDTD_LBC_LINEAR)
        return bad((std::string(what) + ": unknown precision").c_str());
    if (!weights) return bad((std::string(what) + ": weights is NULL").c_str());
    if ((precision == FDTD_LBC_BF16 || precision == FDTD_LBC_BF16X2) && (uintptr_t)weights % 16)
        return bad((std::string(what) + ": packed weights must be 16-byte aligned").c_str());
    return FDTD_OK;
}

int fdtd_lbc_predict(const int32_t shape[3], int32_t face_mask, int32_t side, int32_t precision, float memory,
                     const void *weights, const float *E, const float *H, float *pred, int64_t pred_floats,
                     void *stream)
{
    if (!shape_ok(shape)) return bad("fdtd_lbc_predict: every extent must be >= 2");
    if (face_mask < 0 || face_mask > 63) return bad("fdtd_lbc_predict: face_mask must be in [0, 63]");
    int rc = check_weights(precision, weights, "fdtd_lbc_predict");
    if (rc) return rc;
    if (!E || !H || !pred) return bad("fdtd_lbc_predict: NULL pointer");
    if (side < -1 || side > 1) return bad("fdtd_lbc_predict: side must be -1, 0 or 1");
    if (!(memory >= 0.f && memory < 1.f)) return bad("fdtd_lbc_predict: memory must be in [0, 1)");
    const LGrid g = grid_of(shape, face_mask);
    if (pred_floats < (int64_t)g.ncol * LBC_OUT) return bad("fdtd_lbc_predict: pred too small");
    return check_cuda(launch_lbc_predict(g, side, precision, memory, weights, E, H, pred, (cudaStream_t)stream),
                      "lbc predict launch");
}

int fdtd_lbc_fix(const int32_t shape[3], int32_t face_mask, int32_t fields, const float *pred, float *E, float *H,
                 const float *ce, const float *cm, double dt, void *stream)
{
    if (!shape_ok(shape)) return bad("fdtd_lbc_fix: every extent must be >= 2");
    if (face_mask < 0 || face_mask > 63) return bad("fdtd_lbc_fix: face_mask must be in [0, 63]");
    // one field at a time: the E fix-up reads H and the H fix-up reads E at other cells
    if (fields != LBC_FIX_E && fields != LBC_FIX_H) return bad("fdtd_lbc_fix: fields must be FDTD_LBC_FIX_E or _H");
    if (!pred || !E || !H) return bad("fdtd_lbc_fix: NULL pointer");
    if ((fields & LBC_FIX_E) && !ce) return bad("fdtd_lbc_fix: ce is required for the E fix-up");
    return check_cuda(launch_lbc_fix(grid_of(shape, face_mask), fields, pred, E, H, ce, cm, (float)dt,
                                     (cudaStream_t)stream), "lbc fix launch");
}

int fdtd_lbc_attach(FdtdPlan *plan, int32_t face_mask, int32_t precision, float memory, const void *weights,
                    float *pred, int64_t pred_floats)
{
    if (!plan) return bad("fdtd_lbc_attach: plan is NULL");
    if (face_mask < 0 || face_mask > 63) return bad("fdtd_lbc_attach: face_mask must be in [0, 63]");
    if (face_mask == 0) {
        plan->lbc_mask = 0;
        plan->lbc_w = nullptr;
        plan->lbc_pred = nullptr;
        return FDTD_OK;
    }
    if (plan->d.dtype != FDTD_F32) return bad("fdtd_lbc_attach: the learned boundary needs a float32 plan");
    if (plan->d.n_bloch) return bad("fdtd_lbc_attach: the learned boundary does not combine with Bloch boundaries");
    if (!plan->d.uniform || plan->d.dx != 1.0) return bad("fdtd_lbc_attach: the learned boundary needs unit cells (dx = 1)");
    int rc = check_weights(precision, weights, "fdtd_lbc_attach");
    if (rc) return rc;
    if (!pred) return bad("fdtd_lbc_attach: pred is NULL");
    if (!(memory >= 0.f && memory < 1.f)) return bad("fdtd_lbc_attach: memory must be in [0, 1)");
    const int32_t shape[3] = {(int32_t)plan->sx, (int32_t)plan->sy, (int32_t)plan->sz};
    if (!shape_ok(shape)) return bad("fdtd_lbc_attach: every extent must be >= 2");
    const LGrid g = grid_of(shape, face_mask);
    if (pred_floats < (int64_t)g.ncol * LBC_OUT) return bad("fdtd_lbc_attach: pred too small");
    plan->lbc_mask = face_mask;
    plan->lbc_precision = precision;
    plan->lbc_memory = memory;
    plan->lbc_w = weights;
    plan->lbc_pred = pred;
    return FDTD_OK;
}

}  // extern "C"
