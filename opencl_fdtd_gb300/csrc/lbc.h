// Learned thin absorbing boundary (lbc.cu): stencil layout and the MLP's parameter layout.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace fdtd {

// Per boundary column (a cell of a learned face's plane): the six field components (Ex Ey Ez
// Hx Hy Hz) on a 3 x 3 tangential patch x 2 cells deep (depth 0 = the outermost cell, depth 1
// next to it), in the order [depth][du + 1][dv + 1][component], tangential neighbours past the
// grid clamped to its edge; the network returns the six components of the ghost cell one step
// outside the face.
constexpr int LBC_IN = 108;
constexpr int LBC_HID = 64;
constexpr int LBC_OUT = 6;
// parameter vector: W1 [IN][HID], b1 [HID], W2 [HID][HID], b2 [HID], W3 [HID][OUT], b3 [OUT]
constexpr int LBC_W1 = 0;
constexpr int LBC_B1 = LBC_W1 + LBC_IN * LBC_HID;
constexpr int LBC_W2 = LBC_B1 + LBC_HID;
constexpr int LBC_B2 = LBC_W2 + LBC_HID * LBC_HID;
constexpr int LBC_W3 = LBC_B2 + LBC_HID;
constexpr int LBC_B3 = LBC_W3 + LBC_HID * LBC_OUT;
constexpr int LBC_NPARAM = LBC_B3 + LBC_OUT;   // 11526
// bfloat16 weights of one face in mma.m16n8k16 B-fragment order, float32 biases (32-bit words)
constexpr int LBC_PACK_WORDS = 7 * 8 * 64 + 4 * 8 * 64 + 4 * 64 + 64 + 64 + 8;   // 6024
// inference precision: float32 weights on the CUDA cores; bfloat16 weights and activations on
// the tensor cores; bfloat16 weights with activations split into two bfloat16 parts
constexpr int LBC_F32 = 0;
constexpr int LBC_BF16 = 1;
constexpr int LBC_BF16X2 = 2;
// an exactly linear layer, float32 [6 faces][LBC_IN + 1][LBC_OUT] (rows: inputs, then the bias):
// ghost = sum_k A[k][o] stencil_k + r A[IN][o] (the normalisation cancels)
constexpr int LBC_LINEAR = 3;

// one face of a grid as the boundary kernels see it
struct LFace {
    int32_t axis, side;          // side 0: index 0, 1: index s - 1
    uint32_t nu, nv;             // extent of the column grid (u, v: the other axes in xyz order)
    uint32_t u0, v0;             // first column
    uint32_t ncol;               // nu * nv
    uint32_t col0;               // offset of this face's columns in the concatenated list
};

// face[]: every cell of each learned face's plane (the predictions; edge cells appear once per
// face they lie on); own[]: the same planes with the rows of earlier faces removed, so that
// every outer cell appears once (the corrections, which sum every face's term for a cell)
struct LGrid {
    uint32_t s[3];
    uint64_t N;
    int32_t mask;                // learned faces, bit 2 * axis + side
    int32_t nface;
    LFace face[6];
    LFace own[6];
    uint32_t ncol;               // columns of all faces
    uint32_t nown;               // outer cells
    // per face (order of face[]): the columns the network predicts, u in [win[f][0], win[f][1])
    // and v in [win[f][2], win[f][3]); outside (inside another face's CPML) the ghost is zero
    uint32_t win[6][4];
};

LGrid lbc_grid(const uint32_t s[3], int face_mask);
// the same with the columns that lie inside the CPML of other faces (thickness lo[a] / hi[a] at
// index 0 / s - 1 of axis a) left to zero ghosts
LGrid lbc_grid_window(const uint32_t s[3], int face_mask, const uint32_t lo[3], const uint32_t hi[3]);
cudaError_t launch_lbc_gather(const LGrid &g, const float *E, const float *H, float *X, float *R, float *C,
                              cudaStream_t st);
cudaError_t launch_mlp_fwd(const float *P, const float *X, int B, float *Y, float *A1, float *A2, float *H1,
                           float *H2, cudaStream_t st);
size_t mlp_bwd_workspace(int B);
// gradient of mean over B x 6 of w_o (Y - T)^2 (wout: 6 device floats, NULL = all ones)
cudaError_t launch_mlp_bwd(const float *P, const float *X, const float *Y, const float *T, const float *wout,
                           int B, const float *A1, const float *A2, const float *H1, const float *H2,
                           float *grad, float *ws, cudaStream_t st);
size_t gram_workspace(int rows, int K, int N);
cudaError_t launch_gram(const float *A, int rows, int K, const float *B, int N, float *out, float *ws,
                        cudaStream_t st);
cudaError_t launch_adam(float *P, const float *G, float *M, float *V, int n, float lr, float b1, float b2,
                        float eps, int step, cudaStream_t st);
// float32 parameters [6 faces][LBC_NPARAM] -> packed [6][LBC_PACK_WORDS]
cudaError_t launch_lbc_pack(const float *P, uint32_t *out, cudaStream_t st);
// ghost values [ncol][6] of the faces of side `side` (-1: all faces): pred = r * net + memory *
// pred (the previous ghosts); W: float32 parameters [6][LBC_NPARAM] (LBC_F32) or packed words
// [6][LBC_PACK_WORDS] (LBC_BF16, LBC_BF16X2), face = 2 * axis + side
cudaError_t launch_lbc_predict(const LGrid &g, int side, int precision, float memory, const void *W, const float *E,
                               const float *H, float *pred, cudaStream_t st);
// The plain update of a grid whose edges wrap reads, across a learned side-0 face of axis a,
// H_p at index s_a - 1 for E_q at index 0 (q, a, p distinct), and across a learned side-1 face
// E_p at index 0 for H_q at index s_a - 1. k_lbc_fix replaces those neighbours by the predicted
// ghost values: E_q += -eps_qap ce (ghost H_p - wrapped H_p) right after the E update
// (LBC_FIX_E), H_q += -eps_qap ch (ghost E_p - wrapped E_p) after the H update (LBC_FIX_H),
// eps_qap the Levi-Civita sign, ce = dt / eps, ch = dt / mu (dt without mu), unit cells.
constexpr int LBC_FIX_E = 1;
constexpr int LBC_FIX_H = 2;
cudaError_t launch_lbc_fix(const LGrid &g, int fields, const float *pred, float *E, float *H, const float *ce,
                           const float *cm, float dt, cudaStream_t st);

}  // namespace fdtd
