// Learned thin absorbing boundary: stencil gather, the boundary MLP's training kernels
// (forward, backward, Adam), its inference kernels and the boundary fix-up of the Yee updates.
//
// The boundary model: on every face with the learned layer, each column (one cell of the face's
// plane) reads the six field components on a 3 x 3 tangential patch two cells deep, scales
// them by their RMS r (Maxwell's equations are linear, so scaling the fields by a scales the
// answer by a: dividing by r makes the network's job amplitude-free), and a 108 -> 64 -> 64 -> 6
// MLP with GELU returns the fields of the ghost cell just outside the face, times r. The grid's
// own edges wrap; the fix-up replaces, in the updates of the outermost cells, the wrapped
// neighbour by the ghost (H ghosts outside side-0 faces for the E update, E ghosts outside
// side-1 faces for the H update), which is what a wave leaving the grid needs from the CPML
// layers that the learned layer replaces.
//
// Training runs in float32 with one thread per sample for the per-sample passes (weights in
// shared memory, broadcast reads) and a split reduction over samples for the weight gradients
// (deterministic: fixed partition, fixed folding order). Inference uses bfloat16 weights on
// the tensor cores (mma.sync, float32 accumulation) or float32 weights on the CUDA cores.
#include <cuda_bf16.h>

#include "lbc.h"

namespace fdtd {

namespace {

constexpr int T_FWD = 128;
constexpr int WG_ROWS = 32;      // rows staged per pass of the weight-gradient kernel
constexpr int WG_THREADS = 256;

__device__ __forceinline__ float gelu(float x) { return 0.5f * x * (1.0f + erff(x * 0.70710678118654752f)); }

__device__ __forceinline__ float gelu_d(float x)
{
    return 0.5f * (1.0f + erff(x * 0.70710678118654752f)) + x * 0.39894228040143268f * expf(-0.5f * x * x);
}

__device__ __forceinline__ uint32_t clampu(int v, uint32_t n) { return (uint32_t)(v < 0 ? 0 : (v >= (int)n ? (int)n - 1 : v)); }

// cell coordinates of column (u, v) of face f at depth d with tangential offset (du, dv)
__device__ __forceinline__ uint64_t cell_of(const LGrid &g, const LFace &f, uint32_t u, uint32_t v, int d,
                                            int du, int dv)
{
    const int a = f.axis, ua = a == 0 ? 1 : 0, va = a == 2 ? 1 : 2;
    uint32_t c[3];
    c[a] = f.side ? g.s[a] - 1u - (uint32_t)d : (uint32_t)d;
    c[ua] = clampu((int)u + du, g.s[ua]);
    c[va] = clampu((int)v + dv, g.s[va]);
    return ((uint64_t)c[0] * g.s[1] + c[1]) * g.s[2] + c[2];
}

__device__ __forceinline__ bool in_window(const LGrid &g, int fi, uint32_t u, uint32_t v)
{
    return u >= g.win[fi][0] && u < g.win[fi][1] && v >= g.win[fi][2] && v < g.win[fi][3];
}

__device__ __forceinline__ int face_of(const LGrid &g, uint32_t col)
{
    int f = 0;
    while (f + 1 < g.nface && col >= g.face[f + 1].col0) ++f;
    return f;
}

// the 108 stencil values of a column; returns their RMS
__device__ __forceinline__ float gather(const LGrid &g, const LFace &f, uint32_t u, uint32_t v, const float *E,
                                        const float *H, float *x)
{
    float ss = 0.f;
    int k = 0;
#pragma unroll
    for (int d = 0; d < 2; ++d)
#pragma unroll
        for (int du = -1; du <= 1; ++du)
#pragma unroll
            for (int dv = -1; dv <= 1; ++dv) {
                const uint64_t i = cell_of(g, f, u, v, d, du, dv);
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    const float e = E[c * g.N + i], h = H[c * g.N + i];
                    x[k + c] = e;
                    x[k + 3 + c] = h;
                    ss += e * e + h * h;
                }
                k += 6;
            }
    return sqrtf(ss * (1.0f / LBC_IN));
}

// ---- stencil gather: normalised inputs, their scale, the depth-0 centre values -----------------
__global__ void k_lbc_gather(const LGrid g, const float *E, const float *H, float *X, float *R, float *C)
{
    const uint32_t col = blockIdx.x * blockDim.x + threadIdx.x;
    if (col >= g.ncol) return;
    const LFace &f = g.face[face_of(g, col)];
    const uint32_t c = col - f.col0;
    const uint32_t u = f.u0 + c / f.nv, v = f.v0 + c % f.nv;
    float x[LBC_IN];
    const float r = gather(g, f, u, v, E, H, x);
    const float inv = r > 0.f ? 1.0f / r : 0.f;
    if (X)
        for (int k = 0; k < LBC_IN; ++k) X[(uint64_t)col * LBC_IN + k] = x[k] * inv;
    if (R) R[col] = r;
    if (C) {
        // depth 0, du = dv = 0: stencil entry ((0 * 3 + 1) * 3 + 1) * 6
        for (int k = 0; k < LBC_OUT; ++k) C[(uint64_t)col * LBC_OUT + k] = x[24 + k];
    }
}

// ---- training: forward (float32), one thread per sample ---------------------------------------
// Dynamic shared memory of the float32 MLP kernels: the parameters, then one column of 64
// hidden activations per thread, stored k-major (hs[k * T + t]) so that the runtime loops over
// k read them without bank conflicts and every register array keeps compile-time indices (a
// hidden vector indexed by the runtime k would live in local memory).
constexpr size_t MLP32_SMEM = ((size_t)LBC_NPARAM + (size_t)LBC_HID * 128) * sizeof(float);
static_assert(T_FWD == 128, "MLP32_SMEM holds 128 hidden columns");

__global__ void __launch_bounds__(T_FWD) k_mlp_fwd(const float *P, const float *X, int B, float *Y, float *A1,
                                                    float *A2, float *H1, float *H2)
{
    extern __shared__ float mlp_smem[];
    float *const w = mlp_smem;
    float *const hs = mlp_smem + LBC_NPARAM + threadIdx.x;   // hs[k * T_FWD]: this thread's column
    for (int i = threadIdx.x; i < LBC_NPARAM; i += blockDim.x) w[i] = P[i];
    __syncthreads();
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= B) return;
    float a[LBC_HID];
#pragma unroll
    for (int j = 0; j < LBC_HID; ++j) a[j] = w[LBC_B1 + j];
    for (int k = 0; k < LBC_IN; ++k) {
        const float xk = X[(uint64_t)r * LBC_IN + k];
#pragma unroll
        for (int j = 0; j < LBC_HID; ++j) a[j] += xk * w[LBC_W1 + k * LBC_HID + j];
    }
#pragma unroll
    for (int j = 0; j < LBC_HID; ++j) {
        A1[(uint64_t)r * LBC_HID + j] = a[j];
        const float hj = gelu(a[j]);
        hs[j * T_FWD] = hj;
        H1[(uint64_t)r * LBC_HID + j] = hj;
    }
#pragma unroll
    for (int j = 0; j < LBC_HID; ++j) a[j] = w[LBC_B2 + j];
    for (int k = 0; k < LBC_HID; ++k) {
        const float hk = hs[k * T_FWD];
#pragma unroll
        for (int j = 0; j < LBC_HID; ++j) a[j] += hk * w[LBC_W2 + k * LBC_HID + j];
    }
#pragma unroll
    for (int j = 0; j < LBC_HID; ++j) {
        A2[(uint64_t)r * LBC_HID + j] = a[j];
        const float hj = gelu(a[j]);
        hs[j * T_FWD] = hj;
        H2[(uint64_t)r * LBC_HID + j] = hj;
    }
    float y[LBC_OUT];
#pragma unroll
    for (int o = 0; o < LBC_OUT; ++o) y[o] = w[LBC_B3 + o];
    for (int k = 0; k < LBC_HID; ++k) {
        const float hk = hs[k * T_FWD];
#pragma unroll
        for (int o = 0; o < LBC_OUT; ++o) y[o] += hk * w[LBC_W3 + k * LBC_OUT + o];
    }
#pragma unroll
    for (int o = 0; o < LBC_OUT; ++o) Y[(uint64_t)r * LBC_OUT + o] = y[o];
}

// ---- training: backward through the activations, one thread per sample ------------------------
// loss = scale * sum over the batch and the outputs of w_o (Y - T)^2 (scale = 1 / (B * 6) for the
// mean, w_o = 1 without wout): DY, and the pre-activation gradients D2 (layer 2) and D1 (layer 1)
__global__ void __launch_bounds__(T_FWD) k_mlp_bwd_rows(const float *P, const float *Y, const float *T,
                                                         const float *wout, int B, float scale, const float *A1,
                                                         const float *A2, float *DY, float *D2, float *D1)
{
    __shared__ float w[LBC_NPARAM];
    for (int i = threadIdx.x; i < LBC_NPARAM; i += blockDim.x) w[i] = P[i];
    __syncthreads();
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= B) return;
    float dy[LBC_OUT];
#pragma unroll
    for (int o = 0; o < LBC_OUT; ++o) {
        const float wo = wout ? wout[o] : 1.0f;
        dy[o] = 2.0f * scale * wo * (Y[(uint64_t)r * LBC_OUT + o] - T[(uint64_t)r * LBC_OUT + o]);
        DY[(uint64_t)r * LBC_OUT + o] = dy[o];
    }
    float d2[LBC_HID];
#pragma unroll
    for (int j = 0; j < LBC_HID; ++j) {
        float s = 0.f;
#pragma unroll
        for (int o = 0; o < LBC_OUT; ++o) s += dy[o] * w[LBC_W3 + j * LBC_OUT + o];
        d2[j] = s * gelu_d(A2[(uint64_t)r * LBC_HID + j]);
        D2[(uint64_t)r * LBC_HID + j] = d2[j];
    }
    for (int i = 0; i < LBC_HID; ++i) {
        float s = 0.f;
#pragma unroll
        for (int j = 0; j < LBC_HID; ++j) s += d2[j] * w[LBC_W2 + i * LBC_HID + j];
        D1[(uint64_t)r * LBC_HID + i] = s * gelu_d(A1[(uint64_t)r * LBC_HID + i]);
    }
}

// ---- training: weight gradients dW[k][n] = sum_r In[r][k] D[r][n], bias row k = K ------------
// Block b sums rows b*rpb .. (b+1)*rpb - 1 into partial[b][(K + 1) * N]; the fold kernel then
// adds the partials in block order (same partition, same order: deterministic).
__global__ void __launch_bounds__(WG_THREADS) k_mlp_wgrad(const float *In, const float *D, int B, int K, int N,
                                                          int rpb, float *partial)
{
    extern __shared__ float sh[];
    float *si = sh;                       // [WG_ROWS][K]
    float *sd = sh + WG_ROWS * K;         // [WG_ROWS][N]
    const int KN = (K + 1) * N;
    const int r0 = blockIdx.x * rpb, r1 = min(B, r0 + rpb);
    float acc[28];
#pragma unroll
    for (int q = 0; q < 28; ++q) acc[q] = 0.f;
    for (int rb = r0; rb < r1; rb += WG_ROWS) {
        const int nr = min(WG_ROWS, r1 - rb);
        __syncthreads();
        for (int i = threadIdx.x; i < WG_ROWS * K; i += WG_THREADS) {
            const int rr = i / K;
            si[i] = rr < nr ? In[(uint64_t)(rb + rr) * K + (i - rr * K)] : 0.f;
        }
        for (int i = threadIdx.x; i < WG_ROWS * N; i += WG_THREADS) {
            const int rr = i / N;
            sd[i] = rr < nr ? D[(uint64_t)(rb + rr) * N + (i - rr * N)] : 0.f;
        }
        __syncthreads();
#pragma unroll
        for (int q = 0; q < 28; ++q) {
            const int e = threadIdx.x + q * WG_THREADS;
            if (e >= KN) break;
            const int k = e / N, n = e - k * N;
            float s = acc[q];
            if (k < K) {
                for (int rr = 0; rr < WG_ROWS; ++rr) s += si[rr * K + k] * sd[rr * N + n];
            } else {
                for (int rr = 0; rr < WG_ROWS; ++rr) s += sd[rr * N + n];
            }
            acc[q] = s;
        }
    }
#pragma unroll
    for (int q = 0; q < 28; ++q) {
        const int e = threadIdx.x + q * WG_THREADS;
        if (e < KN) partial[(uint64_t)blockIdx.x * KN + e] = acc[q];
    }
}

// grad[w_off + k*N + n] (k < K) and grad[b_off + n] (bias) from the partials, blocks in order
__global__ void k_mlp_wgrad_fold(const float *partial, int G, int K, int N, float *grad, int w_off, int b_off)
{
    const int KN = (K + 1) * N;
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= KN) return;
    float s = 0.f;
    for (int b = 0; b < G; ++b) s += partial[(uint64_t)b * KN + e];
    const int k = e / N, n = e - k * N;
    if (k < K) grad[w_off + k * N + n] = s;
    else grad[b_off + n] = s;
}

// ---- Adam (Kingma & Ba 2015) with bias correction ---------------------------------------------
__global__ void k_adam(float *P, const float *G, float *M, float *V, int n, float lr, float b1, float b2,
                       float eps, float c1, float c2)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float g = G[i];
    const float m = b1 * M[i] + (1.f - b1) * g;
    const float v = b2 * V[i] + (1.f - b2) * g * g;
    M[i] = m;
    V[i] = v;
    P[i] -= lr * (m / c1) / (sqrtf(v / c2) + eps);
}

// ---- inference ---------------------------------------------------------------------------------
// A boundary step: every face's columns predict their ghosts from E^n, H^{n+1/2}, as
// r * MLP(stencil / r) + memory * (the previous step's ghost): H^{n+1/2} outside side-0 faces,
// E^{n+1} outside side-1 faces; the E update; the E fix-up; sources; the H update; the H fix-up
// (k_lbc_fix). With memory = (1 - c dt) / (1 + c dt) the form contains Mur's first-order
// absorbing condition written for the ghost (the rest of Mur's update is linear in the stencil).
constexpr int T_APPLY = 128;

// float32 weights [6 faces][LBC_NPARAM] on the CUDA cores (the checker of the bfloat16 kernel)
static_assert(T_APPLY == 128, "MLP32_SMEM holds 128 hidden columns");

__global__ void __launch_bounds__(T_APPLY) k_lbc_predict32(const LGrid g, int side, float memory, const float *W,
                                                           const float *E, const float *H, float *pred)
{
    extern __shared__ float mlp_smem[];
    float *const w = mlp_smem;
    float *const hs = mlp_smem + LBC_NPARAM + threadIdx.x;   // hs[k * T_APPLY]: this thread's column
    // blockIdx.y: face; its columns: blockIdx.x * T_APPLY + threadIdx.x
    const int fi = blockIdx.y;
    const LFace &f = g.face[fi];
    if (side >= 0 && f.side != side) return;                 // block-uniform
    const float *Wf = W + (uint64_t)(f.axis * 2 + f.side) * LBC_NPARAM;
    for (int i = threadIdx.x; i < LBC_NPARAM; i += blockDim.x) w[i] = Wf[i];
    __syncthreads();
    const uint32_t c = blockIdx.x * T_APPLY + threadIdx.x;
    if (c >= f.ncol) return;
    const uint32_t u = f.u0 + c / f.nv, v = f.v0 + c % f.nv;
    float *out = pred + (uint64_t)(f.col0 + c) * LBC_OUT;
    if (!in_window(g, fi, u, v)) {
#pragma unroll
        for (int o = 0; o < LBC_OUT; ++o) out[o] = memory * out[o];
        return;
    }
    // layer 1 is linear in the inputs: accumulate W1^T x on the raw stencil while summing its
    // squares, then scale by 1/r (the normalisation) and add the bias
    float a[LBC_HID];
#pragma unroll
    for (int j = 0; j < LBC_HID; ++j) a[j] = 0.f;
    float ss = 0.f;
    // the 18 stencil cells as a runtime loop (unrolling them with the 64-wide inner products
    // multiplies the code and the compile time for a kernel that only checks the others)
#pragma unroll 1
    for (int d = 0; d < 2; ++d)
#pragma unroll 1
        for (int du = -1; du <= 1; ++du)
#pragma unroll 1
            for (int dv = -1; dv <= 1; ++dv) {
                const uint64_t i = cell_of(g, f, u, v, d, du, dv);
                const int k0 = ((d * 3 + (du + 1)) * 3 + (dv + 1)) * 6;
#pragma unroll
                for (int q = 0; q < 6; ++q) {
                    const float xv = q < 3 ? E[q * g.N + i] : H[(q - 3) * g.N + i];
                    ss += xv * xv;
#pragma unroll
                    for (int j = 0; j < LBC_HID; ++j) a[j] += xv * w[LBC_W1 + (k0 + q) * LBC_HID + j];
                }
            }
    const float r = sqrtf(ss * (1.0f / LBC_IN));
    if (!(r > 0.f)) {
#pragma unroll
        for (int o = 0; o < LBC_OUT; ++o) out[o] = memory * out[o];
        return;
    }
    const float inv = 1.0f / r;
#pragma unroll
    for (int j = 0; j < LBC_HID; ++j) a[j] = w[LBC_B1 + j] + a[j] * inv;
#pragma unroll
    for (int j = 0; j < LBC_HID; ++j) hs[j * T_APPLY] = gelu(a[j]);
#pragma unroll
    for (int j = 0; j < LBC_HID; ++j) a[j] = w[LBC_B2 + j];
    for (int k = 0; k < LBC_HID; ++k) {
        const float hk = hs[k * T_APPLY];
#pragma unroll
        for (int j = 0; j < LBC_HID; ++j) a[j] += hk * w[LBC_W2 + k * LBC_HID + j];
    }
#pragma unroll
    for (int j = 0; j < LBC_HID; ++j) hs[j * T_APPLY] = gelu(a[j]);
    float y[LBC_OUT];
#pragma unroll
    for (int o = 0; o < LBC_OUT; ++o) y[o] = w[LBC_B3 + o];
    for (int k = 0; k < LBC_HID; ++k) {
        const float hk = hs[k * T_APPLY];
#pragma unroll
        for (int o = 0; o < LBC_OUT; ++o) y[o] += hk * w[LBC_W3 + k * LBC_OUT + o];
    }
#pragma unroll
    for (int o = 0; o < LBC_OUT; ++o) out[o] = y[o] * r + memory * out[o];
}

// ---- stencil tiles staged per warp (the linear and the tensor-core inference) ------------------
// A warp's job: a tile of MMA_TU x 16 columns of one face (MMA_TU rows along u, 16 columns along
// v). The cells its stencils read, (MMA_TU + 2) x 18 positions x 2 depths x 6 components, are
// staged once in shared memory, plane (component q, depth d) by plane with a stride of
// MMA_PL floats (MMA_PL = 16 mod 32, so the two depths a lane pair reads fall in different
// banks), before the columns are evaluated 16 at a time. The loads follow the memory order:
// along z (v) on x and y faces, over the depth pair z = 0, 1 (or s - 1, s - 2) first on z faces.
constexpr int MMA_TU = 4;
constexpr int MMA_SU = MMA_TU + 2, MMA_SV = 16 + 2;
constexpr int MMA_PL = 112;
static_assert(MMA_SU * MMA_SV <= MMA_PL && MMA_PL % 32 == 16, "stage plane layout");
constexpr int MMA_STAGE = 12 * MMA_PL;                                   // floats per warp

// Stage the cells of the tile whose first (face-local) column is (cu0, cv0) into st.
__device__ __forceinline__ void stage_tile(const LGrid &g, const LFace &f, uint32_t cu0, uint32_t cv0,
                                           const float *E, const float *H, float *st, int lane)
{
        // stage: cells (u0 + cu0 - 1 + su, v0 + cv0 - 1 + sv), clamped to the grid like cell_of.
        // Per (component, su) row of the stage a lane loads the pairs (sv, d) number lane and
        // lane + 32 of 36, ordered (sv, d) on z faces (the depth pair is contiguous in memory)
        // and (d, sv) on x and y faces (v = z is contiguous).
        const int a = f.axis, ua = a == 0 ? 1 : 0, va = a == 2 ? 1 : 2;
        const uint64_t syz = (uint64_t)g.s[1] * g.s[2];
        const uint64_t sd = a == 0 ? syz : a == 1 ? (uint64_t)g.s[2] : 1u;     // strides of the depth,
        const uint64_t sua = ua == 0 ? syz : (uint64_t)g.s[2];                 // u and v axes
        const uint64_t sva = va == 1 ? (uint64_t)g.s[2] : 1u;
        uint64_t off[2];
        int soff[2];
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int e = lane + 32 * h < 2 * MMA_SV ? lane + 32 * h : 0;
            const int d = a == 2 ? (e & 1) : e / MMA_SV;
            const int sv = a == 2 ? (e >> 1) : e % MMA_SV;
            const uint32_t cd = f.side ? g.s[a] - 1u - (uint32_t)d : (uint32_t)d;
            const uint32_t cv = clampu((int)(f.v0 + cv0) - 1 + sv, g.s[va]);
            off[h] = cd * sd + cv * sva;
            soff[h] = d * MMA_PL + sv;
        }
        const bool second = lane + 32 < 2 * MMA_SV;
#pragma unroll 1
        for (int su = 0; su < MMA_SU; ++su) {
            const uint64_t ou = clampu((int)(f.u0 + cu0) - 1 + su, g.s[ua]) * sua;
#pragma unroll
            for (int q = 0; q < 6; ++q) {
                const float *src = q < 3 ? E + q * g.N : H + (q - 3) * g.N;
                float *dst = st + q * 2 * MMA_PL + su * MMA_SV;
                dst[soff[0]] = src[ou + off[0]];
                if (second) dst[soff[1]] = src[ou + off[1]];
            }
        }
}

constexpr int MMA_WARPS = 4;                      // warps of a block of the staged kernels

// an exactly linear layer (LBC_LINEAR), weights [6][IN + 1][OUT] float32 in shared memory: a
// warp stages a tile of 4 x 16 columns (stage_tile) and each lane forms the 108 x 6 products of
// two of them (column lane % 16 of the tile's rows lane / 16 and lane / 16 + 2), in the order
// of the stencil
__global__ void __launch_bounds__(MMA_WARPS * 32) k_lbc_predict_lin(const LGrid g, int side, float memory,
                                                                    const float *W, const float *E,
                                                                    const float *H, float *pred)
{
    __shared__ float w[(LBC_IN + 1) * LBC_OUT];
    __shared__ float stage[MMA_WARPS][MMA_STAGE];
    const LFace &f = g.face[blockIdx.y];
    if (side >= 0 && f.side != side) return;                 // block-uniform
    const float *Wf = W + (uint64_t)(f.axis * 2 + f.side) * (LBC_IN + 1) * LBC_OUT;
    for (int i = threadIdx.x; i < (LBC_IN + 1) * LBC_OUT; i += blockDim.x) w[i] = Wf[i];
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t ntv = (f.nv + 15u) / 16u, ntu = (f.nu + MMA_TU - 1u) / MMA_TU;
    const uint32_t job = blockIdx.x * MMA_WARPS + warp;
    if (job >= ntu * ntv) return;                            // warp-uniform; no block barrier below
    const uint32_t cu0 = (job / ntv) * MMA_TU, cv0 = (job % ntv) * 16u;
    float *st = stage[warp];
    stage_tile(g, f, cu0, cv0, E, H, st, lane);
    __syncwarp();
    const int jv = lane & 15;
#pragma unroll 1
    for (int h = 0; h < 2; ++h) {
        const int tr = (lane >> 4) + 2 * h;
        const uint32_t cu = cu0 + (uint32_t)tr, cv = cv0 + (uint32_t)jv;
        if (cu >= f.nu || cv >= f.nv) continue;
        const uint32_t c = cu * f.nv + cv;
        float *out = pred + (uint64_t)(f.col0 + c) * LBC_OUT;
        if (!in_window(g, blockIdx.y, f.u0 + cu, f.v0 + cv)) {
#pragma unroll
            for (int o = 0; o < LBC_OUT; ++o) out[o] = memory * out[o];
            continue;
        }
        float acc[LBC_OUT];
#pragma unroll
        for (int o = 0; o < LBC_OUT; ++o) acc[o] = 0.f;
        float ss = 0.f;
#pragma unroll
        for (int d = 0; d < 2; ++d)
#pragma unroll
            for (int du = -1; du <= 1; ++du)
#pragma unroll
                for (int dv = -1; dv <= 1; ++dv) {
                    const int k0 = ((d * 3 + (du + 1)) * 3 + (dv + 1)) * 6;
                    const float *sp = st + d * MMA_PL + (tr + 1 + du) * MMA_SV + (jv + 1 + dv);
#pragma unroll
                    for (int q = 0; q < 6; ++q) {
                        const float xv = sp[q * 2 * MMA_PL];
                        ss += xv * xv;
#pragma unroll
                        for (int o = 0; o < LBC_OUT; ++o) acc[o] += xv * w[(k0 + q) * LBC_OUT + o];
                    }
                }
        const float r = sqrtf(ss * (1.0f / LBC_IN));
#pragma unroll
        for (int o = 0; o < LBC_OUT; ++o) out[o] = acc[o] + r * w[LBC_IN * LBC_OUT + o] + memory * out[o];
    }
}

// ---- bfloat16 tensor-core inference (mma.sync m16n8k16, float32 accumulation) ------------------
// Weights are packed once per face into the B-fragment order of mma.m16n8k16 (PTX ISA, "Matrix
// fragments for mma.m16n8k16"): for k-step ks and n-tile nt, lane (g = lane / 4, t = lane % 4)
// holds B[16 ks + 2t + {0, 1}][8 nt + g] in word 0 and B[16 ks + 2t + 8 + {0, 1}][8 nt + g] in
// word 1, the lower k in the low half. Layer 1's K = 108 is padded to 112 with zero rows,
// layer 3's N = 6 to 8 with zero columns. Biases stay float32.
constexpr int PK_W1 = 0;                          // [7][8][32][2] words
constexpr int PK_W2 = PK_W1 + 7 * 8 * 64;         // [4][8][32][2]
constexpr int PK_W3 = PK_W2 + 4 * 8 * 64;         // [4][1][32][2]
constexpr int PK_B1 = PK_W3 + 4 * 64;             // float [64]
constexpr int PK_B2 = PK_B1 + LBC_HID;            // float [64]
constexpr int PK_B3 = PK_B2 + LBC_HID;            // float [8]
static_assert(PK_B3 + 8 == LBC_PACK_WORDS, "packed layout size");

constexpr int XS = 120;                           // float row stride of a warp's stencil tile

// two floats rounded to bfloat16 in one conversion (lo in the low half)
__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi)
{
    const __nv_bfloat162 p = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<const uint32_t *>(&p);
}

// x = hi + lo with hi = bf16(x), lo = bf16(x - hi): about 16 significant bits in two bf16 parts
__device__ __forceinline__ void split_bf16(float x0, float x1, uint32_t &hi, uint32_t &lo)
{
    hi = pack_bf16(x0, x1);
    const float h0 = __uint_as_float(hi << 16), h1 = __uint_as_float(hi & 0xffff0000u);
    lo = pack_bf16(x0 - h0, x1 - h1);
}

// GELU of the tensor-core inference: erf by Abramowitz & Stegun, Handbook of Mathematical
// Functions, formula 7.1.26 (Hastings' rational approximation, |error| <= 1.5e-7 for all x),
// with the exponential and reciprocal on the special-function unit; well inside the bfloat16
// (and split-bfloat16) precision of the layer inputs it feeds. Training and the float32 checker
// use erff.
__device__ __forceinline__ float rcp_approx(float x)
{
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

__device__ __forceinline__ float ex2_approx(float x)
{
    float r;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

// PTX: the reciprocal and 2^x by rcp.approx / ex2.approx and the last step as one fma;
// otherwise the __fdividef / __expf intrinsics. Same approximation either way; each form
// measured faster in one of the two kernels (bf16x2: PTX, bf16: intrinsics).
template <bool PTX>
__device__ __forceinline__ float gelu_mma(float x)
{
    const float z = x * 0.70710678118654752f;                 // x / sqrt(2)
    const float az = fabsf(z);
    const float den = fmaf(0.3275911f, az, 1.0f);
    const float t = PTX ? rcp_approx(den) : __fdividef(1.0f, den);
    const float poly = t * fmaf(t, fmaf(t, fmaf(t, fmaf(t, 1.061405429f, -1.453152027f), 1.421413741f),
                                        -0.284496736f), 0.254829592f);
    if (PTX) {
        // exp(-z^2) = 2^(-z^2 log2(e))
        const float e = copysignf(fmaf(-poly, ex2_approx((az * az) * -1.4426950408889634f), 1.0f), z);
        const float h = 0.5f * x;
        return fmaf(h, e, h);                                 // x (1 + erf(z)) / 2
    }
    const float e = copysignf(1.0f - poly * __expf(-az * az), z);
    return 0.5f * x * (1.0f + e);
}

__device__ __forceinline__ void mma_bf16(float c[4], const uint32_t a[4], uint32_t b0, uint32_t b1)
{
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0, %1, %2, %3}, {%4, %5, %6, %7}, {%8, %9}, "
        "{%0, %1, %2, %3};\n"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

__global__ void k_lbc_pack(const float *P, uint32_t *out)
{
    const int face = blockIdx.y;
    const float *w = P + (uint64_t)face * LBC_NPARAM;
    uint32_t *o = out + (uint64_t)face * LBC_PACK_WORDS;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < LBC_PACK_WORDS; e += gridDim.x * blockDim.x) {
        uint32_t word;
        if (e >= PK_B1) {
            const int j = e - PK_B1;
            const float b = j < LBC_HID ? w[LBC_B1 + j] : j < 2 * LBC_HID ? w[LBC_B2 + j - LBC_HID]
                                                         : (j - 2 * LBC_HID < LBC_OUT ? w[LBC_B3 + j - 2 * LBC_HID] : 0.f);
            word = __float_as_uint(b);
        } else {
            int base, K, N, nt_count, off;
            if (e < PK_W2) { off = e - PK_W1; base = LBC_W1; K = LBC_IN; N = LBC_HID; nt_count = 8; }
            else if (e < PK_W3) { off = e - PK_W2; base = LBC_W2; K = LBC_HID; N = LBC_HID; nt_count = 8; }
            else { off = e - PK_W3; base = LBC_W3; K = LBC_HID; N = LBC_OUT; nt_count = 1; }
            const int reg = off & 1, lane = (off >> 1) & 31, nt = (off >> 6) % nt_count, ks = (off >> 6) / nt_count;
            const int g = lane >> 2, t = lane & 3;
            const int k = 16 * ks + 2 * t + 8 * reg, n = 8 * nt + g;
            const float v0 = (k < K && n < N) ? w[base + k * N + n] : 0.f;
            const float v1 = (k + 1 < K && n < N) ? w[base + (k + 1) * N + n] : 0.f;
            word = pack_bf16(v0, v1);
        }
        o[e] = word;
    }
}

// GELU of a layer's accumulators, re-cut into the A fragments of the next layer: n-tiles 2 ks and
// 2 ks + 1 of a 16 x 64 output are the k-step ks A fragment (rows g / g + 8, cols 2t / 2t + 8).
template <bool SPLIT>
__device__ __forceinline__ void act_to_a(const float acc[8][4], uint32_t ah[4][4], uint32_t al[4][4])
{
#pragma unroll
    for (int ks = 0; ks < 4; ++ks)
#pragma unroll
        for (int half = 0; half < 2; ++half) {
            const float *c = acc[2 * ks + half];
            const float g0 = gelu_mma<SPLIT>(c[0]), g1 = gelu_mma<SPLIT>(c[1]);
            const float g2 = gelu_mma<SPLIT>(c[2]), g3 = gelu_mma<SPLIT>(c[3]);
            if (SPLIT) {
                split_bf16(g0, g1, ah[ks][2 * half], al[ks][2 * half]);
                split_bf16(g2, g3, ah[ks][2 * half + 1], al[ks][2 * half + 1]);
            } else {
                ah[ks][2 * half] = pack_bf16(g0, g1);
                ah[ks][2 * half + 1] = pack_bf16(g2, g3);
            }
        }
}


template <bool SPLIT>
__global__ void __launch_bounds__(MMA_WARPS * 32) k_lbc_predict_mma(const LGrid g, int side, float memory,
                                                                     const uint32_t *Wp, const float *E,
                                                                     const float *H, float *pred)
{
    extern __shared__ __align__(16) float smem_f[];
    const LFace &f = g.face[blockIdx.y];
    if (side >= 0 && f.side != side) return;                             // block-uniform
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int gq = lane >> 2, tq = lane & 3;
    float *st = smem_f + warp * (MMA_STAGE + 16 * XS + 16);
    float *xs = st + MMA_STAGE;                                           // [16][XS] network inputs
    float *rr = xs + 16 * XS;                                             // [16] RMS of each row
    // packed weights of the face (read through L1: every warp of the face reads the same 24 KB)
    const uint32_t *w = Wp + (uint64_t)(f.axis * 2 + f.side) * LBC_PACK_WORDS;
    const float *wb = reinterpret_cast<const float *>(w);
    const uint2 *w1 = reinterpret_cast<const uint2 *>(w + PK_W1);
    const uint2 *w2 = reinterpret_cast<const uint2 *>(w + PK_W2);
    const uint2 *w3 = reinterpret_cast<const uint2 *>(w + PK_W3);

    const uint32_t ntv = (f.nv + 15u) / 16u, ntu = (f.nu + MMA_TU - 1u) / MMA_TU;
    const uint32_t job = blockIdx.x * MMA_WARPS + warp;
    if (job >= ntu * ntv) return;                                         // warp-uniform; no block barrier below
    const uint32_t tu = job / ntv, tv = job % ntv;
    const uint32_t cu0 = tu * MMA_TU, cv0 = tv * 16u;                     // first column of the tile (face-local)
    stage_tile(g, f, cu0, cv0, E, H, st, lane);
    __syncwarp();
    for (int tr = 0; tr < MMA_TU; ++tr) {
        const uint32_t cu = cu0 + (uint32_t)tr;
        if (cu >= f.nu) break;                                            // warp-uniform
        // gather: lane pair (row = lane / 2) reads depth (lane & 1) of its column's stencil
        {
            const int row = lane >> 1, d = lane & 1;
            const uint32_t cv = cv0 + (uint32_t)row;
            const uint32_t u = f.u0 + cu, v = f.v0 + cv;
            // columns outside the window read nothing: r = 0, no network term
            const bool ok = cv < f.nv && in_window(g, blockIdx.y, u, v);
            float x[54];
            float ss = 0.f;
#pragma unroll
            for (int du = -1; du <= 1; ++du)
#pragma unroll
                for (int dv = -1; dv <= 1; ++dv) {
                    const int k0 = ((du + 1) * 3 + (dv + 1)) * 6;
                    const float *sp = st + d * MMA_PL + (tr + 1 + du) * MMA_SV + (row + 1 + dv);
#pragma unroll
                    for (int q = 0; q < 6; ++q) {
                        const float xv = ok ? sp[q * 2 * MMA_PL] : 0.f;
                        x[k0 + q] = xv;
                        ss += xv * xv;
                    }
                }
            ss += __shfl_xor_sync(0xffffffffu, ss, 1);
            const float r = sqrtf(ss * (1.0f / LBC_IN));
            const float inv = r > 0.f ? 1.0f / r : 0.f;
            float2 *xr = reinterpret_cast<float2 *>(xs + row * XS + d * 54);   // 8-byte aligned
#pragma unroll
            for (int k = 0; k < 27; ++k) xr[k] = make_float2(x[2 * k] * inv, x[2 * k + 1] * inv);
            if (d == 1) {
                xr[27] = make_float2(0.f, 0.f);                           // K padding 108..111
                xr[28] = make_float2(0.f, 0.f);
            } else {
                rr[row] = r;
            }
        }
        __syncwarp();
        // layer 1: [16 x 112] x [112 x 64]
        float acc[8][4];
#pragma unroll
        for (int nt = 0; nt < 8; ++nt) {
            const float b0 = __ldg(wb + PK_B1 + 8 * nt + 2 * tq), b1 = __ldg(wb + PK_B1 + 8 * nt + 2 * tq + 1);
            acc[nt][0] = b0; acc[nt][1] = b1; acc[nt][2] = b0; acc[nt][3] = b1;
        }
#pragma unroll
        for (int ks = 0; ks < 7; ++ks) {
            const float2 p0 = *reinterpret_cast<const float2 *>(xs + gq * XS + 16 * ks + 2 * tq);
            const float2 p1 = *reinterpret_cast<const float2 *>(xs + (gq + 8) * XS + 16 * ks + 2 * tq);
            const float2 p2 = *reinterpret_cast<const float2 *>(xs + gq * XS + 16 * ks + 8 + 2 * tq);
            const float2 p3 = *reinterpret_cast<const float2 *>(xs + (gq + 8) * XS + 16 * ks + 8 + 2 * tq);
            uint32_t ah[4], al[4];
            if (SPLIT) {
                split_bf16(p0.x, p0.y, ah[0], al[0]);
                split_bf16(p1.x, p1.y, ah[1], al[1]);
                split_bf16(p2.x, p2.y, ah[2], al[2]);
                split_bf16(p3.x, p3.y, ah[3], al[3]);
            } else {
                ah[0] = pack_bf16(p0.x, p0.y);
                ah[1] = pack_bf16(p1.x, p1.y);
                ah[2] = pack_bf16(p2.x, p2.y);
                ah[3] = pack_bf16(p3.x, p3.y);
            }
#pragma unroll
            for (int nt = 0; nt < 8; ++nt) {
                const uint2 b = __ldg(w1 + (ks * 8 + nt) * 32 + lane);
                mma_bf16(acc[nt], ah, b.x, b.y);
                if (SPLIT) mma_bf16(acc[nt], al, b.x, b.y);
            }
        }
        uint32_t ah2[4][4], al2[4][4];
        act_to_a<SPLIT>(acc, ah2, al2);
        // layer 2: [16 x 64] x [64 x 64]
#pragma unroll
        for (int nt = 0; nt < 8; ++nt) {
            const float b0 = __ldg(wb + PK_B2 + 8 * nt + 2 * tq), b1 = __ldg(wb + PK_B2 + 8 * nt + 2 * tq + 1);
            acc[nt][0] = b0; acc[nt][1] = b1; acc[nt][2] = b0; acc[nt][3] = b1;
        }
#pragma unroll
        for (int ks = 0; ks < 4; ++ks)
#pragma unroll
            for (int nt = 0; nt < 8; ++nt) {
                const uint2 b = __ldg(w2 + (ks * 8 + nt) * 32 + lane);
                mma_bf16(acc[nt], ah2[ks], b.x, b.y);
                if (SPLIT) mma_bf16(acc[nt], al2[ks], b.x, b.y);
            }
        act_to_a<SPLIT>(acc, ah2, al2);
        // layer 3: [16 x 64] x [64 x 8]
        float y[4];
        {
            const float b0 = __ldg(wb + PK_B3 + 2 * tq), b1 = __ldg(wb + PK_B3 + 2 * tq + 1);
            y[0] = b0; y[1] = b1; y[2] = b0; y[3] = b1;
        }
#pragma unroll
        for (int ks = 0; ks < 4; ++ks) {
            const uint2 b = __ldg(w3 + ks * 32 + lane);
            mma_bf16(y, ah2[ks], b.x, b.y);
            if (SPLIT) mma_bf16(y, al2[ks], b.x, b.y);
        }
        // rows gq and gq + 8, output components 2 tq and 2 tq + 1 (< 6)
        if (tq < 3) {
#pragma unroll
            for (int hr = 0; hr < 2; ++hr) {
                const int row = gq + 8 * hr;
                const uint32_t cv = cv0 + (uint32_t)row;
                if (cv < f.nv) {
                    const uint32_t c = cu * f.nv + cv;
                    const float r = rr[row];
                    float *out = pred + (uint64_t)(f.col0 + c) * LBC_OUT + 2 * tq;
                    out[0] = (r > 0.f ? y[2 * hr] * r : 0.f) + memory * out[0];
                    out[1] = (r > 0.f ? y[2 * hr + 1] * r : 0.f) + memory * out[1];
                }
            }
        }
        __syncwarp();
    }
}

constexpr size_t MMA_SMEM = (size_t)MMA_WARPS * (MMA_STAGE + 16 * XS + 16) * 4;

// Levi-Civita sign of distinct (q, a, p): +1 for the cyclic orders of (0, 1, 2)
__device__ __forceinline__ float lc(int q, int a) { return ((a - q + 3) % 3) == 1 ? 1.f : -1.f; }

__device__ __forceinline__ int own_of(const LGrid &g, uint32_t col)
{
    int f = 0;
    while (f + 1 < g.nface && col >= g.own[f + 1].col0) ++f;
    return f;
}

// one thread per outer cell: every learned face through the cell adds its term, faces in order
__global__ void k_lbc_fix(const LGrid g, int fields, const float *pred, float *E, float *H, const float *ce,
                          const float *cm, float dt)
{
    const uint32_t col = blockIdx.x * blockDim.x + threadIdx.x;
    if (col >= g.nown) return;
    const LFace &o = g.own[own_of(g, col)];
    const uint32_t k = col - o.col0;
    uint32_t c[3];
    {
        const int a = o.axis, ua = a == 0 ? 1 : 0, va = a == 2 ? 1 : 2;
        c[a] = o.side ? g.s[a] - 1u : 0u;
        c[ua] = o.u0 + k / o.nv;
        c[va] = o.v0 + k % o.nv;
    }
    const uint64_t st[3] = {(uint64_t)g.s[1] * g.s[2], g.s[2], 1};
    const uint64_t i = c[0] * st[0] + c[1] * st[1] + c[2];
    float dE[3] = {0.f, 0.f, 0.f}, dH[3] = {0.f, 0.f, 0.f};
    for (int fi = 0; fi < g.nface; ++fi) {
        const LFace &f = g.face[fi];
        const int a = f.axis, ua = a == 0 ? 1 : 0, va = a == 2 ? 1 : 2;
        if (c[a] != (f.side ? g.s[a] - 1u : 0u)) continue;
        const float *gp = pred + ((uint64_t)f.col0 + (uint64_t)c[ua] * f.nv + c[va]) * LBC_OUT;
        // the wrapped neighbour: index s_a - 1 (side 0) or 0 (side 1) along a
        const uint64_t j = f.side ? i - (uint64_t)(g.s[a] - 1u) * st[a] : i + (uint64_t)(g.s[a] - 1u) * st[a];
#pragma unroll
        for (int q = 0; q < 3; ++q) {
            if (q == a) continue;
            const int p = 3 - a - q;
            if (f.side == 0 && (fields & LBC_FIX_E)) dE[q] -= lc(q, a) * (gp[3 + p] - H[p * g.N + j]);
            if (f.side == 1 && (fields & LBC_FIX_H)) dH[q] -= lc(q, a) * (gp[p] - E[p * g.N + j]);
        }
    }
#pragma unroll
    for (int q = 0; q < 3; ++q) {
        if ((fields & LBC_FIX_E) && dE[q] != 0.f) E[q * g.N + i] += ce[q * g.N + i] * dE[q];
        if ((fields & LBC_FIX_H) && dH[q] != 0.f) H[q * g.N + i] += (cm ? cm[q * g.N + i] : dt) * dH[q];
    }
}

}  // namespace

// the column grids of the faces in face_mask (bit 2a + side): whole planes, and owned cells
LGrid lbc_grid(const uint32_t s[3], int face_mask)
{
    LGrid g;
    g.s[0] = s[0];
    g.s[1] = s[1];
    g.s[2] = s[2];
    g.N = (uint64_t)s[0] * s[1] * s[2];
    g.mask = face_mask;
    g.nface = 0;
    g.ncol = 0;
    g.nown = 0;
    bool owned[3][2] = {{false, false}, {false, false}, {false, false}};
    for (int a = 0; a < 3; ++a)
        for (int side = 0; side < 2; ++side) {
            if (!(face_mask & (1 << (2 * a + side)))) continue;
            const int ua = a == 0 ? 1 : 0, va = a == 2 ? 1 : 2;
            LFace f;
            f.axis = a;
            f.side = side;
            f.u0 = 0;
            f.v0 = 0;
            f.nu = s[ua];
            f.nv = s[va];
            f.ncol = f.nu * f.nv;
            f.col0 = g.ncol;
            g.ncol += f.ncol;
            // owned: skip the cells of an earlier face's plane (lower axes own the edges)
            LFace o = f;
            uint32_t u0 = 0, u1 = s[ua], v0 = 0, v1 = s[va];
            if (owned[ua][0]) u0 = 1;
            if (owned[ua][1] && u1 > 0) u1 -= 1;
            if (owned[va][0]) v0 = 1;
            if (owned[va][1] && v1 > 0) v1 -= 1;
            o.u0 = u0;
            o.v0 = v0;
            o.nu = u1 > u0 ? u1 - u0 : 0;
            o.nv = v1 > v0 ? v1 - v0 : 0;
            o.ncol = o.nu * o.nv;
            o.col0 = g.nown;
            g.nown += o.ncol;
            g.face[g.nface] = f;
            g.own[g.nface] = o;
            g.win[g.nface][0] = 0;
            g.win[g.nface][1] = s[ua];
            g.win[g.nface][2] = 0;
            g.win[g.nface][3] = s[va];
            ++g.nface;
            owned[a][side] = true;
        }
    return g;
}

LGrid lbc_grid_window(const uint32_t s[3], int face_mask, const uint32_t lo[3], const uint32_t hi[3])
{
    LGrid g = lbc_grid(s, face_mask);
    for (int i = 0; i < g.nface; ++i) {
        const int a = g.face[i].axis, ua = a == 0 ? 1 : 0, va = a == 2 ? 1 : 2;
        g.win[i][0] = lo[ua] < s[ua] ? lo[ua] : s[ua];
        g.win[i][1] = hi[ua] < s[ua] ? s[ua] - hi[ua] : 0;
        g.win[i][2] = lo[va] < s[va] ? lo[va] : s[va];
        g.win[i][3] = hi[va] < s[va] ? s[va] - hi[va] : 0;
    }
    return g;
}

cudaError_t launch_lbc_gather(const LGrid &g, const float *E, const float *H, float *X, float *R, float *C,
                              cudaStream_t st)
{
    if (!g.ncol) return cudaSuccess;
    k_lbc_gather<<<(g.ncol + 127) / 128, 128, 0, st>>>(g, E, H, X, R, C);
    return cudaGetLastError();
}

// The shared-memory opt-in above 48 KB is a per-device function attribute: set it once per device
// and kernel slot (setting it twice from two threads is harmless).
enum : int { SMEM_MLP_FWD = 0, SMEM_PREDICT32 = 1, SMEM_MMA = 2, SMEM_MMA_SPLIT = 3, SMEM_SLOTS = 4 };

static cudaError_t smem_opt_in(const void *fn, int slot, size_t bytes)
{
    constexpr int MAX_DEV = 64;
    static bool set[MAX_DEV][SMEM_SLOTS] = {};
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev >= 0 && dev < MAX_DEV && set[dev][slot]) return cudaSuccess;
    e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
    if (e != cudaSuccess) return e;
    if (dev >= 0 && dev < MAX_DEV) set[dev][slot] = true;
    return cudaSuccess;
}

cudaError_t launch_mlp_fwd(const float *P, const float *X, int B, float *Y, float *A1, float *A2, float *H1,
                           float *H2, cudaStream_t st)
{
    if (B <= 0) return cudaSuccess;
    const cudaError_t e = smem_opt_in((const void *)k_mlp_fwd, SMEM_MLP_FWD, MLP32_SMEM);
    if (e != cudaSuccess) return e;
    k_mlp_fwd<<<(B + T_FWD - 1) / T_FWD, T_FWD, MLP32_SMEM, st>>>(P, X, B, Y, A1, A2, H1, H2);
    return cudaGetLastError();
}

// workspace floats needed by launch_mlp_bwd for a batch of B
size_t mlp_bwd_workspace(int B)
{
    const int G = (B + 255) / 256;
    return (size_t)B * (LBC_OUT + 2 * LBC_HID) + (size_t)G * (LBC_IN + 1) * LBC_HID;
}

cudaError_t launch_mlp_bwd(const float *P, const float *X, const float *Y, const float *T, const float *wout,
                           int B, const float *A1, const float *A2, const float *H1, const float *H2,
                           float *grad, float *ws, cudaStream_t st)
{
    if (B <= 0) return cudaSuccess;
    float *DY = ws, *D2 = DY + (size_t)B * LBC_OUT, *D1 = D2 + (size_t)B * LBC_HID;
    float *part = D1 + (size_t)B * LBC_HID;
    k_mlp_bwd_rows<<<(B + T_FWD - 1) / T_FWD, T_FWD, 0, st>>>(P, Y, T, wout, B, 1.0f / ((float)B * LBC_OUT),
                                                              A1, A2, DY, D2, D1);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    const int rpb = 256, G = (B + rpb - 1) / rpb;
    struct L { const float *in; const float *d; int K, N, w, b; } layers[3] = {
        {X, D1, LBC_IN, LBC_HID, LBC_W1, LBC_B1},
        {H1, D2, LBC_HID, LBC_HID, LBC_W2, LBC_B2},
        {H2, DY, LBC_HID, LBC_OUT, LBC_W3, LBC_B3}};
    for (const L &l : layers) {
        const size_t smem = (size_t)WG_ROWS * (l.K + l.N) * sizeof(float);
        k_mlp_wgrad<<<G, WG_THREADS, smem, st>>>(l.in, l.d, B, l.K, l.N, rpb, part);
        const int KN = (l.K + 1) * l.N;
        k_mlp_wgrad_fold<<<(KN + 255) / 256, 256, 0, st>>>(part, G, l.K, l.N, grad, l.w, l.b);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
    }
    return cudaSuccess;
}

// out[(K + 1) x N]: A^T B (rows k < K) and the column sums of B (row K), A [rows][K], B [rows][N]
// (K, N with (K + 1) N <= 28 * WG_THREADS); ws: ceil(rows / 256) * (K + 1) * N floats
size_t gram_workspace(int rows, int K, int N) { return (size_t)((rows + 255) / 256) * (K + 1) * N; }

cudaError_t launch_gram(const float *A, int rows, int K, const float *B, int N, float *out, float *ws,
                        cudaStream_t st)
{
    if (rows <= 0) return cudaSuccess;
    const int rpb = 256, G = (rows + rpb - 1) / rpb;
    const size_t smem = (size_t)WG_ROWS * (K + N) * sizeof(float);
    k_mlp_wgrad<<<G, WG_THREADS, smem, st>>>(A, B, rows, K, N, rpb, ws);
    const int KN = (K + 1) * N;
    k_mlp_wgrad_fold<<<(KN + 255) / 256, 256, 0, st>>>(ws, G, K, N, out, 0, K * N);
    return cudaGetLastError();
}

cudaError_t launch_adam(float *P, const float *G, float *M, float *V, int n, float lr, float b1, float b2,
                        float eps, int step, cudaStream_t st)
{
    if (n <= 0) return cudaSuccess;
    const float c1 = 1.f - powf(b1, (float)step), c2 = 1.f - powf(b2, (float)step);
    k_adam<<<(n + 255) / 256, 256, 0, st>>>(P, G, M, V, n, lr, b1, b2, eps, c1, c2);
    return cudaGetLastError();
}

cudaError_t launch_lbc_pack(const float *P, uint32_t *out, cudaStream_t st)
{
    k_lbc_pack<<<dim3((LBC_PACK_WORDS + 255) / 256, 6, 1), 256, 0, st>>>(P, out);
    return cudaGetLastError();
}

cudaError_t launch_lbc_predict(const LGrid &g, int side, int precision, float memory, const void *W, const float *E,
                               const float *H, float *pred, cudaStream_t st)
{
    if (!g.ncol) return cudaSuccess;
    uint32_t maxc = 0;
    for (int f = 0; f < g.nface; ++f) maxc = g.face[f].ncol > maxc ? g.face[f].ncol : maxc;
    if (precision == LBC_F32 || precision == LBC_LINEAR) {
        const dim3 gi((maxc + T_APPLY - 1) / T_APPLY, (unsigned)g.nface, 1);
        uint32_t maxj = 0;
        for (int f = 0; f < g.nface; ++f) {
            const uint32_t nj = ((g.face[f].nu + MMA_TU - 1) / MMA_TU) * ((g.face[f].nv + 15) / 16);
            maxj = nj > maxj ? nj : maxj;
        }
        if (precision == LBC_F32) {
            const cudaError_t e = smem_opt_in((const void *)k_lbc_predict32, SMEM_PREDICT32, MLP32_SMEM);
            if (e != cudaSuccess) return e;
            k_lbc_predict32<<<gi, T_APPLY, MLP32_SMEM, st>>>(g, side, memory, (const float *)W, E, H, pred);
        } else {
            const dim3 gl((maxj + MMA_WARPS - 1) / MMA_WARPS, (unsigned)g.nface, 1);
            k_lbc_predict_lin<<<gl, MMA_WARPS * 32, 0, st>>>(g, side, memory, (const float *)W, E, H, pred);
        }
        return cudaGetLastError();
    }
    const int split = precision == LBC_BF16X2 ? 1 : 0;
    const cudaError_t e = split ? smem_opt_in((const void *)k_lbc_predict_mma<true>, SMEM_MMA_SPLIT, MMA_SMEM)
                                : smem_opt_in((const void *)k_lbc_predict_mma<false>, SMEM_MMA, MMA_SMEM);
    if (e != cudaSuccess) return e;
    uint32_t maxj = 0;
    for (int f = 0; f < g.nface; ++f) {
        const uint32_t nj = ((g.face[f].nu + MMA_TU - 1) / MMA_TU) * ((g.face[f].nv + 15) / 16);
        maxj = nj > maxj ? nj : maxj;
    }
    const dim3 gi((maxj + MMA_WARPS - 1) / MMA_WARPS, (unsigned)g.nface, 1);
    if (split)
        k_lbc_predict_mma<true><<<gi, MMA_WARPS * 32, MMA_SMEM, st>>>(g, side, memory, (const uint32_t *)W, E, H, pred);
    else
        k_lbc_predict_mma<false><<<gi, MMA_WARPS * 32, MMA_SMEM, st>>>(g, side, memory, (const uint32_t *)W, E, H, pred);
    return cudaGetLastError();
}

cudaError_t launch_lbc_fix(const LGrid &g, int fields, const float *pred, float *E, float *H, const float *ce,
                           const float *cm, float dt, cudaStream_t st)
{
    if (!g.nown) return cudaSuccess;
    k_lbc_fix<<<(g.nown + 127) / 128, 128, 0, st>>>(g, fields, pred, E, H, ce, cm, dt);
    return cudaGetLastError();
}

}  // namespace fdtd
