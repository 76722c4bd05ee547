// One-pass time step: E update, point sources, H update and Poynting vector of a whole step in
// one launch (the multi-step path of fdtd_run when second copies of every array are given).
//
// The two-pass form (update_E, then H and S) reads E twice and moves H, E and S through HBM in
// two launches: 96 B per cell per step in float32. One step only needs to read E, H and dt/eps
// once and write E, H and S once: 72 B per cell. Here:
//
//   * Fields are double-buffered: every read comes from the buffers of the old step (A: E, H
//     and every CPML psi), every write goes to the new ones (B), so a block may evaluate cells
//     another block owns (halo cells) from the same inputs and get the owner's values.
//   * A block owns the rows [y0, y0 + nown) of all z (a tile) and marches a chunk of x planes.
//     Its E window is the rows [y0 - 1, y0 + nown], one thread per cell (the cells outside the
//     z faces on the first warps, the z-face cells on the last ones); the H window is
//     [y0 - 1, y0 + nown), S is formed on the own rows. Row y0 - 1 exists only to give S the
//     products of its y - 1 neighbours, row y0 + nown only to give H its y + 1 neighbours.
//   * Iteration x: E_new at plane x (H of plane x and x - 1); H_new and the six Poynting products
//     at plane x - 1 (E_new of planes x - 1 and x); S at plane x - 1 (products of planes x - 1
//     and x - 2). The old H of plane x - 1 stays in registers; E_new and the products of a plane
//     go to two double-buffered shared arrays, so one barrier per plane orders everything.
//   * Inputs arrive through a ring of shared-memory stages. For each plane the block stages
//     the rows [y0 - 2, y0 + nown] of H, E, dt/eps (and dt/mu), and of the z-face CPML arrays,
//     each a contiguous range in the reference's layout (opencl_fdtd/kernels/common.cl:34-52).
//     Tiles whose rows do not wrap around the y boundary copy them with bulk asynchronous copies
//     (cp.async.bulk, completion on an mbarrier per stage), issued by the lanes of warp 0 right
//     after the barrier that frees the stage, nstage - 1 planes ahead. A bulk copy moves whole
//     16-byte units from 16-byte aligned addresses, so a range that starts inside a unit lands
//     `lead` elements into its slot; lead depends only on the range's first element index and
//     every thread computes it. The two tiles whose rows wrap (and any launch whose buffers are
//     not 16-byte aligned) fill the same stages with per-element cp.async instead.
//   * CPML arrays of the x and y faces are read with ordinary loads one plane ahead.
//   * Every wait for a stage is bounded (%globaltimer): a wait that runs out sets a bit in the
//     plan's status word, the block stops at the next barrier and first waits, again bounded,
//     for the copies it has issued.
//
// Per-cell arithmetic and its order are those of update_E, update_H and update_S
// (opencl_fdtd/kernels/update_e.cl:39-107, update_h.cl:36-155, update_s.cl:33-36), compiled
// with --fmad=false, so fields, psi and S are bit-identical to the per-call kernels.
#include "yee_common.cuh"
#include "yee_device.cuh"
#include "step.h"

namespace fdtd {

// ---- PTX wrappers ------------------------------------------------------------------------------
__device__ __forceinline__ uint32_t sh_addr(const void *p)
{
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(sh_addr(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_fence_init()
{
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_tx(uint64_t *bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(sh_addr(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ bool mbar_test(uint64_t *bar, uint32_t parity)
{
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(sh_addr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

__device__ __forceinline__ uint64_t timer_ns()
{
    uint64_t v;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(v));
    return v;
}

__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, uint32_t bytes, uint64_t *bar)
{
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            sh_addr(dst)),
        "l"(src), "r"(bytes), "r"(sh_addr(bar))
        : "memory");
}

template <typename R>
__device__ __forceinline__ void async_elem(R *dst, const R *src)
{
    if (sizeof(R) == 4)
        asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(sh_addr(dst)), "l"(src) : "memory");
    else
        asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(sh_addr(dst)), "l"(src) : "memory");
}

__device__ __forceinline__ void async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }

template <int N>
__device__ __forceinline__ void async_wait() { asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory"); }

// wait until at most n groups of this thread are pending (n < STEP_MAX_STAGES)
__device__ __forceinline__ void async_wait_n(int n)
{
    switch (n) {
    case 0: async_wait<0>(); break;
    case 1: async_wait<1>(); break;
    case 2: async_wait<2>(); break;
    case 3: async_wait<3>(); break;
    case 4: async_wait<4>(); break;
    default: async_wait<5>(); break;
    }
}

// Bounded wait for phase `parity` of a stage's barrier; false (and the status bit) when it ran out.
__device__ __noinline__ bool stage_wait_slow(uint64_t *bar, uint32_t parity, uint32_t wait_ns, int32_t *status)
{
    const uint64_t t0 = timer_ns();
    for (uint32_t it = 1;; ++it) {
        if (mbar_test(bar, parity)) return true;
        if ((it & 63u) == 0 && timer_ns() - t0 > wait_ns) {
            atomicOr(status, STEP_STATUS_TIMEOUT);
            return false;
        }
    }
}

__device__ __forceinline__ bool stage_wait(uint64_t *bar, uint32_t parity, uint32_t wait_ns, int32_t *status)
{
    return mbar_test(bar, parity) || stage_wait_slow(bar, parity, wait_ns, status);
}

// ---- stage fills -----------------------------------------------------------------------------
// Geometry of a block's staged ranges for one plane.
struct StageGeo {
    uint32_t x, yH, rows;       // plane, first staged row, staged rows
    uint32_t lead[3];           // lead of component c of every field slot
    uint32_t zlead[2];          // lead of the z slots of side n / p
};

// Bulk copies of one plane, issued by the 32 lanes of warp 0 (one range per lane), completing
// on `bar`. A range's tail that is not a whole 16-byte unit of its array is copied with
// ordinary stores before the arrive that publishes it.
template <typename R, int STR, bool MU>
__device__ __forceinline__ void fill_bulk(const StepK<R> &k, R *st, uint64_t *bar, const StageGeo &g, uint32_t lane)
{
    constexpr uint64_t V = 16 / sizeof(R);
    const R *src = nullptr;
    uint64_t first = 0, count = 0;
    R *dst = nullptr;
    if (lane < (uint32_t)SG_NF) {
        const int kind = (int)lane / 3, c = (int)lane % 3;
        if (kind < 3 || MU) {
            src = kind == 0 ? k.HA : kind == 1 ? k.EA : kind == 2 ? k.ce : k.cm;
            first = (uint64_t)c * k.N + (uint64_t)g.x * k.syz + (uint64_t)g.yH * k.sz;
            count = (uint64_t)g.rows * k.sz;
            dst = st + lane * STR;
        }
    } else if (lane < (uint32_t)SG_N) {
        const int q = (int)lane - SG_NF, side = q >> 2, slot = q & 3;
        const uint32_t T = (uint32_t)(side ? k.ax[2].Tp : k.ax[2].Tn);
        if (T) {
            src = k.ax[2].psiA[slot >> 1][side][slot & 1];
            first = ((uint64_t)g.x * k.sy + g.yH) * T;
            count = (uint64_t)g.rows * T;
            dst = st + k.zoff[side] + slot * k.zsz[side];
        }
    }
    uint32_t bytes = 0;
    const R *csrc = nullptr;
    if (src) {
        const uint64_t a = first & ~(V - 1), e = first + count;
        uint64_t b = (e + V - 1) & ~(V - 1);
        const uint64_t lim = k.len[lane] & ~(V - 1);
        if (b > lim) {
            for (uint64_t q = lim > first ? lim : first; q < e; ++q) dst[q - a] = src[q];
            b = lim;
        }
        if (b > a) {
            bytes = (uint32_t)((b - a) * sizeof(R));
            csrc = src + a;
        }
    }
    const uint32_t total = __reduce_add_sync(0xffffffffu, bytes);
    __syncwarp();
    if (lane == 0) mbar_arrive_tx(bar, total);
    __syncwarp();
    if (bytes) bulk_g2s(dst, csrc, bytes, bar);
}

// The same ranges copied element by element (cp.async) by every thread, rows taken modulo sy;
// commits one group per call (an empty one when `live` is false).
template <typename R, int STR, bool MU>
__device__ __forceinline__ void fill_async(const StepK<R> &k, R *st, const StageGeo &g, bool live, uint32_t t,
                                           uint32_t nt)
{
    if (live) {
        const uint32_t sz = k.sz, sy = k.sy;
        const uint32_t n = g.rows * sz;
        const uint64_t xo = (uint64_t)g.x * k.syz;
        for (uint32_t q = t; q < n; q += nt) {
            const uint32_t rq = q / sz, zq = q - rq * sz;
            const uint64_t off = xo + (uint64_t)((g.yH + rq) % sy) * sz + zq;
#pragma unroll
            for (int kind = 0; kind < (MU ? 4 : 3); ++kind) {
                const R *src = kind == 0 ? k.HA : kind == 1 ? k.EA : kind == 2 ? k.ce : k.cm;
#pragma unroll
                for (int c = 0; c < 3; ++c)
                    async_elem(st + (kind * 3 + c) * STR + g.lead[c] + q, src + (uint64_t)c * k.N + off);
            }
        }
        for (int side = 0; side < 2; ++side) {
            const uint32_t T = (uint32_t)(side ? k.ax[2].Tp : k.ax[2].Tn);
            if (!T) continue;
            const uint32_t m = g.rows * T;
            R *const zb = st + k.zoff[side] + g.zlead[side];
            for (uint32_t q = t; q < m; q += nt) {
                const uint32_t rq = q / T, ir = q - rq * T;
                const uint64_t off = ((uint64_t)g.x * sy + (g.yH + rq) % sy) * T + ir;
#pragma unroll
                for (int slot = 0; slot < 4; ++slot)
                    async_elem(zb + slot * k.zsz[side] + q, k.ax[2].psiA[slot >> 1][side][slot & 1] + off);
            }
        }
    }
    async_commit();
}

// ---- the kernel --------------------------------------------------------------------------------
// CPML face of an axis for coordinate c: depth (-1 outside) and side
__device__ __forceinline__ int step_face(int Tn, int Tp, uint32_t s, uint32_t c, int &side)
{
    side = 0;
    if (c < (uint32_t)Tn) return (int)c;
    if (Tp && c >= s - (uint32_t)Tp) {
        side = 1;
        return (int)(s - 1u - c);
    }
    return -1;
}

// psi of the x face (u, v) and of the y face (u, v) of one cell and type, zero outside
template <typename R>
struct PsiXY {
    R xu, xv, yu, yv;
};

template <typename R, typename C, int DX, bool MU>
__global__ void __launch_bounds__(C::MAXT, C::MINB) k_step(const __grid_constant__ StepK<R> k)
{
    constexpr int MAXT = C::MAXT;
    constexpr int STR = C::STR;
    constexpr uint32_t V = 16 / sizeof(R);
    extern __shared__ __align__(128) unsigned char step_smem[];
    R *const stages = reinterpret_cast<R *>(step_smem);
    R *const XE = stages + (size_t)k.nstage * k.stage_elems;     // [2][3][MAXT] E_new of a plane
    R *const PB = XE + 6 * MAXT;                                 // [2][6][MAXT] products of a plane
    R *const SC = PB + 12 * MAXT;                                // coefficient tables
    uint64_t *const full = reinterpret_cast<uint64_t *>(SC + ((k.ncoef + 3u) & ~3u));

    const uint32_t sx = k.sx, sy = k.sy, sz = k.sz, syz = k.syz;
    const uint64_t N = k.N;
    const int NS = (int)k.nstage;
    const uint32_t nt = blockDim.x;
    const uint32_t y0 = (uint32_t)(((uint64_t)blockIdx.x * sy) / k.ntile);
    const uint32_t nown = (uint32_t)(((uint64_t)(blockIdx.x + 1) * sy) / k.ntile) - y0;
    const uint32_t rows = nown + 3u;                     // staged rows y0 - 2 .. y0 + nown
    const uint32_t yH = (y0 + 2u * sy - 2u) % sy;
    const bool tma = k.tma && y0 >= 2u && y0 + nown < sy;
    const uint32_t xa = blockIdx.y * k.xchunk;
    const uint32_t xb = min(xa + k.xchunk, sx);
    const int nit = (int)(xb - xa) + 2;                  // planes xa - 1 .. xb

    // Thread t takes one cell of the E window. The cells outside the z faces come first (row by
    // row), the z-face cells after them, so that the z-face work falls on as few warps as
    // possible; q is the cell's position in the window (row r - 1, column z).
    const uint32_t t = threadIdx.x;
    const uint32_t nrw = nown + 2u;                      // rows of the E window
    const bool act = t < nrw * sz;
    uint32_t rr = 0u, z = 0u;
    if (act) {
        const uint32_t zi0 = (uint32_t)k.ax[2].Tn, wi = sz - zi0 - (uint32_t)k.ax[2].Tp;
        if (t < nrw * wi) {
            rr = t / wi;
            z = zi0 + (t - rr * wi);
        } else {
            const uint32_t f = t - nrw * wi, wf = sz - wi;
            rr = f / wf;
            const uint32_t zf = f - rr * wf;
            z = zf < zi0 ? zf : zf + wi;
        }
    }
    const uint32_t q = rr * sz + z;
    const uint32_t r = rr + 1u;                          // window row (0 is staged only)
    const bool hrow = act && r <= nown + 1u;
    const bool own = act && r >= 2u && r <= nown + 1u;
    const uint32_t y = (yH + r) % sy;
    const uint32_t j = y * sz + z;
    const int dmz = z ? -1 : (int)sz - 1;                // z - 1 / z + 1 within the row (periodic)
    const int dpz = (z + 1u < sz) ? 1 : 1 - (int)sz;
    int fy_side, fz_side;
    const int fy_ir = step_face(k.ax[1].Tn, k.ax[1].Tp, sy, y, fy_side);
    const int fz_ir = step_face(k.ax[2].Tn, k.ax[2].Tp, sz, z, fz_side);
    // thickness and coefficient table index (E p0 p1 p2, H p0 p1 p2, T apart) of the cell's y / z
    // face, the stride of its z slots, and its position in a field slot (before the lead):
    // recomputed on use
#define FY_T ((uint32_t)(fy_side ? k.ax[1].Tp : k.ax[1].Tn))
#define FZ_T ((uint32_t)(fz_side ? k.ax[2].Tp : k.ax[2].Tn))
#define CY ((uint32_t)(k.coff[1][fy_side] + fy_ir))
#define CZ ((uint32_t)(k.coff[2][fz_side] + fz_ir))
#define ZS (k.zsz[fz_side])
#define P_WIN (q + sz)
    // low bits of the first staged element index of component 0 at plane 0, and of N
    const uint32_t kc0 = yH * sz, nlo = (uint32_t)N;
    auto plane = [&](int q) -> uint32_t {               // plane of iteration q (x taken mod sx)
        int xi = (int)xa - 1 + q;
        if (xi < 0) xi += (int)sx;
        if (xi >= (int)sx) xi -= (int)sx;
        return (uint32_t)xi;
    };
    auto geo = [&](int q) -> StageGeo {
        StageGeo g;
        g.x = plane(q);
        g.yH = yH;
        g.rows = rows;
        const uint32_t xs = g.x * syz;
        g.lead[0] = (kc0 + xs) & (V - 1);
        g.lead[1] = (kc0 + xs + nlo) & (V - 1);
        g.lead[2] = (kc0 + xs + 2u * nlo) & (V - 1);
        g.zlead[0] = ((g.x * sy + yH) * (uint32_t)k.ax[2].Tn) & (V - 1);
        g.zlead[1] = ((g.x * sy + yH) * (uint32_t)k.ax[2].Tp) & (V - 1);
        return g;
    };
    // psi of the x and y faces of type ty (0: E, 1: H) at plane x, from the A buffers
    auto psi_xy = [&](int ty, uint32_t x) -> PsiXY<R> {
        PsiXY<R> v;
        v.xu = v.xv = v.yu = v.yv = R(0);
        int xs_;
        const int xi = step_face(k.ax[0].Tn, k.ax[0].Tp, sx, x, xs_);
        if (xi >= 0) {
            const uint64_t ip = (uint64_t)xi * syz + j;
            v.xu = ldg(k.ax[0].psiA[ty][xs_][0] + ip);
            v.xv = ldg(k.ax[0].psiA[ty][xs_][1] + ip);
        }
        if (fy_ir >= 0) {
            const uint64_t ip = ((uint64_t)x * FY_T + (uint32_t)fy_ir) * sz + z;
            v.yu = ldg(k.ax[1].psiA[ty][fy_side][0] + ip);
            v.yv = ldg(k.ax[1].psiA[ty][fy_side][1] + ip);
        }
        return v;
    };

    for (uint32_t q = t; q < k.ncoef; q += nt) SC[q] = k.coef[q];
    if (t == 0) {
        for (int s = 0; s < NS; ++s) mbar_init(&full[s], 1);
        mbar_fence_init();
    }
    __syncthreads();

    // x-1 values of the first E evaluation: H_A of plane xa - 2 at the thread's cell
    R hx_m = R(0), hy_m = R(0), hz_m = R(0);
    if (act) {
        const uint32_t xm2 = (xa + 2u * sx - 2u) % sx;
        const uint64_t i = (uint64_t)xm2 * syz + j;
        hy_m = ldg(k.HA + N + i);
        hz_m = ldg(k.HA + 2 * N + i);
    }
    // psi_E of the x and y faces for the next E evaluation; psi_H (x, y, z faces) for the next
    // H evaluation
    PsiXY<R> pe = {R(0), R(0), R(0), R(0)}, ph = {R(0), R(0), R(0), R(0)};
    R phzu = R(0), phzv = R(0);
    if (act) pe = psi_xy(0, plane(0));

    // first stages
    const int npre = NS < nit ? NS : nit;
    if (tma) {
        if (t < 32)
            for (int q = 0; q < npre; ++q)
                fill_bulk<R, STR, MU>(k, stages + (size_t)q * k.stage_elems, &full[q], geo(q), t);
    } else {
        for (int q = 0; q < NS; ++q)
            fill_async<R, STR, MU>(k, stages + (size_t)q * k.stage_elems, geo(q), q < nit, t, nt);
        async_wait_n(NS - 1);
        __syncthreads();
    }

    R cx_m = R(0), cy_m = R(0), cz_m = R(0);            // dt/mu of plane x - 1
    // the cell's 32-bit index at the planes x and x - 1 (the written arrays are addressed from
    // their per-component bases, which the kernel parameters give block-uniformly)
    uint32_t x = plane(0);
    int it = 0;
    uint32_t sp = 0;                                     // stage slot (bits 1..) and its parity (bit 0)
    bool abort = false;
    for (; it < nit; ++it) {
        const uint32_t slot = sp >> 1;
        R *const st = stages + (size_t)slot * k.stage_elems;
        bool failed = false;
        if (tma) failed = !stage_wait(&full[slot], sp & 1u, k.wait_ns, k.status);
        const uint32_t xs = x * syz;
        const uint32_t xm = x ? x - 1u : sx - 1u;
        const uint32_t ic = xs + j, im = xm * syz + j;  // the cell at planes x and x - 1
        const uint32_t xo = (uint32_t)(it & 1) * (uint32_t)MAXT;   // this plane's XE / PB halves
        const R *const b0 = st + ((kc0 + xs) & (V - 1)) + P_WIN;
        const R *const b1 = st + ((kc0 + xs + nlo) & (V - 1)) + P_WIN;
        const R *const b2 = st + ((kc0 + xs + 2u * nlo) & (V - 1)) + P_WIN;
        const bool ein = it >= 1 && it <= nit - 2;       // plane x is in the block's chunk
        const bool hin = it >= 2;                        // plane x - 1 is in the block's chunk
        int xf_side;
        const int xf_ir = step_face(k.ax[0].Tn, k.ax[0].Tp, sx, x, xf_side);
        R *const xe_c = XE + xo * 3u + q;                // E_new of plane x
        const R *const xe_p = XE + (xo ^ (uint32_t)MAXT) * 3u + q;   // of plane x - 1
        R *const pb_c = PB + xo * 6u + q;                // products of plane x - 1
        const R *const pb_p = PB + (xo ^ (uint32_t)MAXT) * 6u + q;   // of plane x - 2

        // ---- E_new at plane x (update_e.cl:39-107) ----
        R hx = R(0), hy = R(0), hz = R(0), ex = R(0), ey = R(0), ez = R(0);
        if (act && !failed) {
            hx = b0[SG_H * STR];
            hy = b1[(SG_H + 1) * STR];
            hz = b2[(SG_H + 2) * STR];
            const R nxy = b0[SG_H * STR - (int)sz], nzy = b2[(SG_H + 2) * STR - (int)sz];
            const R nxz = b0[SG_H * STR + dmz], nyz = b1[(SG_H + 1) * STR + dmz];
            R d_xy = hx - nxy;
            R d_xz = hx - nxz;
            R d_yx = hy - hy_m;
            R d_yz = hy - nyz;
            R d_zx = hz - hz_m;
            R d_zy = hz - nzy;
            if (DX != 0) {
                R ix = k.inv_d, iy = k.inv_d, iz = k.inv_d;
                if (DX == 2) { ix = ldg(k.inv_dh[0] + x); iy = ldg(k.inv_dh[1] + y); iz = ldg(k.inv_dh[2] + z); }
                d_xy = d_xy * iy; d_xz = d_xz * iz; d_yx = d_yx * ix;
                d_yz = d_yz * iz; d_zx = d_zx * ix; d_zy = d_zy * iy;
            }
            R px = R(0), py = R(0), pz = R(0);
            const bool wr = own && ein;
            if (xf_ir >= 0) {
                const uint32_t T = (uint32_t)(xf_side ? k.ax[0].Tp : k.ax[0].Tn);
                const uint32_t c = (uint32_t)(k.coff[0][xf_side] + xf_ir);
                R su, sv;
                face_update<R, true, 0>(SC[c], SC[c + T], SC[c + 2 * T], pe.xu, pe.xv,
                                        su, sv, d_xy, d_xz, d_yx, d_yz, d_zx, d_zy, px, py, pz);
                if (wr) {
                    const uint32_t ip = (uint32_t)xf_ir * syz + j;
                    k.ax[0].psiB[0][xf_side][0][ip] = su;
                    k.ax[0].psiB[0][xf_side][1][ip] = sv;
                }
            }
            if (fy_ir >= 0) {
                const uint32_t c = CY, T = FY_T;
                R su, sv;
                face_update<R, true, 1>(SC[c], SC[c + T], SC[c + 2 * T], pe.yu, pe.yv,
                                        su, sv, d_xy, d_xz, d_yx, d_yz, d_zx, d_zy, px, py, pz);
                if (wr) {
                    const uint32_t ip = (x * T + (uint32_t)fy_ir) * sz + z;
                    k.ax[1].psiB[0][fy_side][0][ip] = su;
                    k.ax[1].psiB[0][fy_side][1][ip] = sv;
                }
            }
            if (fz_ir >= 0) {
                const uint32_t c = CZ, T = FZ_T;
                const R *const zb = st + k.zoff[fz_side] + r * T + (uint32_t)fz_ir + (((x * sy + yH) * T) & (V - 1));
                R su, sv;
                face_update<R, true, 2>(SC[c], SC[c + T], SC[c + 2 * T], zb[0], zb[ZS],
                                        su, sv, d_xy, d_xz, d_yx, d_yz, d_zx, d_zy, px, py, pz);
                if (wr) {
                    const uint32_t ip = (x * sy + y) * T + (uint32_t)fz_ir;
                    k.ax[2].psiB[0][fz_side][0][ip] = su;
                    k.ax[2].psiB[0][fz_side][1][ip] = sv;
                }
            }
            ex = b0[SG_E * STR] + b0[SG_C * STR] * ((d_zy - d_yz) + px);
            ey = b1[(SG_E + 1) * STR] + b1[(SG_C + 1) * STR] * ((d_xz - d_zx) + py);
            ez = b2[(SG_E + 2) * STR] + b2[(SG_C + 2) * STR] * ((d_yx - d_xy) + pz);
            // point sources after the E update (fdtd.py:168-169), in list order
            if (k.nsrc) {
#pragma unroll 1
                for (int s = 0; s < k.nsrc; ++s) {
                    if (x == k.src_x[s] && j == k.src_j[s]) {
                        const R v = ldg(k.src_values + (uint64_t)k.t * k.nsrc + s);
                        if (k.src_c[s] == 0) ex = ex + v;
                        else if (k.src_c[s] == 1) ey = ey + v;
                        else ez = ez + v;
                    }
                }
            }
            if (wr) {
                k.EB[ic] = ex;
                (k.EB + N)[ic] = ey;
                (k.EB + 2 * N)[ic] = ez;
            }
            xe_c[0] = ex;
            xe_c[MAXT] = ey;
            xe_c[2 * MAXT] = ez;
        }
        const uint32_t xn = x + 1u == sx ? 0u : x + 1u;
        if (act && it + 1 < nit) pe = psi_xy(0, xn);

        // ---- H_new and the products at plane x - 1 (update_h.cl:36-155) ----
        if (hrow && it >= 1 && !failed) {
            // E_new of plane x - 1: the cell and its y + 1, z + 1 neighbours
            const R ex_m = xe_p[0], ey_m = xe_p[MAXT], ez_m = xe_p[2 * MAXT];
            const R rxy = xe_p[sz], rzy = xe_p[2 * MAXT + sz];
            const R rxz = xe_p[dpz], ryz = xe_p[MAXT + dpz];
            R d_xy = rxy - ex_m;
            R d_xz = rxz - ex_m;
            R d_yx = ey - ey_m;
            R d_yz = ryz - ey_m;
            R d_zx = ez - ez_m;
            R d_zy = rzy - ez_m;
            if (DX != 0) {
                R ix = k.inv_d, iy = k.inv_d, iz = k.inv_d;
                if (DX == 2) {
                    ix = ldg(k.inv_de[0] + xm);
                    iy = ldg(k.inv_de[1] + y);
                    iz = ldg(k.inv_de[2] + z);
                }
                d_xy = d_xy * iy; d_xz = d_xz * iz; d_yx = d_yx * ix;
                d_yz = d_yz * iz; d_zx = d_zx * ix; d_zy = d_zy * iy;
            }
            R px = R(0), py = R(0), pz = R(0);
            const bool wr = own && hin;
            int mf_side;
            const int mf_ir = step_face(k.ax[0].Tn, k.ax[0].Tp, sx, xm, mf_side);
            if (mf_ir >= 0) {
                const uint32_t T = (uint32_t)(mf_side ? k.ax[0].Tp : k.ax[0].Tn);
                const uint32_t c = (uint32_t)(k.coff[0][mf_side] + mf_ir) + 3u * T;
                R su, sv;
                face_update<R, false, 0>(SC[c], SC[c + T], SC[c + 2 * T], ph.xu, ph.xv,
                                         su, sv, d_xy, d_xz, d_yx, d_yz, d_zx, d_zy, px, py, pz);
                if (wr) {
                    const uint32_t ip = (uint32_t)mf_ir * syz + j;
                    k.ax[0].psiB[1][mf_side][0][ip] = su;
                    k.ax[0].psiB[1][mf_side][1][ip] = sv;
                }
            }
            if (fy_ir >= 0) {
                const uint32_t T = FY_T, c = CY + 3u * T;
                R su, sv;
                face_update<R, false, 1>(SC[c], SC[c + T], SC[c + 2 * T], ph.yu, ph.yv,
                                         su, sv, d_xy, d_xz, d_yx, d_yz, d_zx, d_zy, px, py, pz);
                if (wr) {
                    const uint32_t ip = (xm * T + (uint32_t)fy_ir) * sz + z;
                    k.ax[1].psiB[1][fy_side][0][ip] = su;
                    k.ax[1].psiB[1][fy_side][1][ip] = sv;
                }
            }
            if (fz_ir >= 0) {
                const uint32_t T = FZ_T, c = CZ + 3u * T;
                R su, sv;
                face_update<R, false, 2>(SC[c], SC[c + T], SC[c + 2 * T], phzu, phzv,
                                         su, sv, d_xy, d_xz, d_yx, d_yz, d_zx, d_zy, px, py, pz);
                if (wr) {
                    const uint32_t ip = (xm * sy + y) * T + (uint32_t)fz_ir;
                    k.ax[2].psiB[1][fz_side][0][ip] = su;
                    k.ax[2].psiB[1][fz_side][1][ip] = sv;
                }
            }
            R hxn, hyn, hzn;
            if (MU) {
                hxn = hx_m - cx_m * ((d_zy - d_yz) - px);
                hyn = hy_m - cy_m * ((d_xz - d_zx) - py);
                hzn = hz_m - cz_m * ((d_yx - d_xy) - pz);
            } else {
                hxn = hx_m - k.dt * ((d_zy - d_yz) - px);
                hyn = hy_m - k.dt * ((d_xz - d_zx) - py);
                hzn = hz_m - k.dt * ((d_yx - d_xy) - pz);
            }
            if (wr) {
                k.HB[im] = hxn;
                (k.HB + N)[im] = hyn;
                (k.HB + 2 * N)[im] = hzn;
            }
            if (k.poynt) {
                const R ahx = hxn + hx_m, ahy = hyn + hy_m, ahz = hzn + hz_m;
                const R os0 = (ey + ey_m) * ahz;
                const R os3 = (-(ez + ez_m)) * ahy;
                const R os1 = (rzy + ez_m) * ahx;
                const R os4 = (-(rxy + ex_m)) * ahz;
                const R os2 = (rxz + ex_m) * ahy;
                const R os5 = (-(ryz + ey_m)) * ahx;
                if (wr && k.write_oS) {
                    k.oS[im] = os0;
                    (k.oS + N)[im] = os1;
                    (k.oS + 2 * N)[im] = os2;
                    (k.oS + 3 * N)[im] = os3;
                    (k.oS + 4 * N)[im] = os4;
                    (k.oS + 5 * N)[im] = os5;
                }
                // the products in the reference's order xy, yz, zx, xz, yx, zy (update_h.cl:142-147)
                pb_c[0] = os0;
                pb_c[MAXT] = os1;
                pb_c[2 * MAXT] = os2;
                pb_c[3 * MAXT] = os3;
                pb_c[4 * MAXT] = os4;
                pb_c[5 * MAXT] = os5;
            }
        }
        // what the next H evaluation (plane x) needs from this plane
        if (act && !failed) {
            ph = psi_xy(1, x);
            if (fz_ir >= 0) {
                const uint32_t T = FZ_T;
                const R *const zb = st + k.zoff[fz_side] + r * T + (uint32_t)fz_ir + (((x * sy + yH) * T) & (V - 1));
                phzu = zb[2 * ZS];
                phzv = zb[3 * ZS];
            }
            if (MU) {
                cx_m = b0[SG_M * STR];
                cy_m = b1[(SG_M + 1) * STR];
                cz_m = b2[(SG_M + 2) * STR];
            }
        }
        hx_m = hx;
        hy_m = hy;
        hz_m = hz;
        if (!tma) async_wait_n(NS - 2);
        abort = __syncthreads_or(failed) != 0;
        if (abort) break;
        // this stage is free: stage the plane of iteration it + NS into it
        if (tma) {
            if (t < 32 && it + NS < nit) fill_bulk<R, STR, MU>(k, st, &full[slot], geo(it + NS), t);
        } else {
            fill_async<R, STR, MU>(k, st, geo(it + NS), it + NS < nit, t, nt);
        }

        // ---- S at plane x - 1 (update_s.cl:33-36): products of planes x - 1 (this iteration's
        // buffer) and x - 2 (the previous one) ----
        if (k.poynt && own && hin) {
            k.S[im] = (((pb_c[0] + pb_c[3 * MAXT]) + pb_c[-(int)sz]) + pb_c[3 * MAXT + dmz]) * k.sf;
            (k.S + N)[im] = (((pb_c[MAXT] + pb_c[4 * MAXT]) + pb_c[MAXT + dmz]) + pb_p[4 * MAXT]) * k.sf;
            (k.S + 2 * N)[im] = (((pb_c[2 * MAXT] + pb_c[5 * MAXT]) + pb_p[2 * MAXT]) + pb_c[5 * MAXT - (int)sz]) * k.sf;
        }
        x = xn;
        sp = (slot + 1u == (uint32_t)NS) ? ((sp & 1u) ^ 1u) : sp + 2u;
    }
#undef FY_T
#undef FZ_T
#undef CY
#undef CZ
#undef ZS
#undef P_WIN
    if (abort) {
        // wait (bounded) for the copies still in flight before the block's memory is released
        if (tma) {
            if (t == 0) {
                const int issued = it + NS < nit ? it + NS : nit;
                for (int q = it; q < issued; ++q) {
                    uint64_t *bar = &full[q % NS];
                    const uint32_t par = (uint32_t)(q / NS) & 1u;
                    const uint64_t t0 = timer_ns();
                    while (!mbar_test(bar, par))
                        if (timer_ns() - t0 > k.wait_ns) break;
                }
            }
        } else {
            async_wait<0>();
        }
    }
}

// ---- host side -------------------------------------------------------------------------------
template <typename C>
static uint32_t max_rows_of(uint32_t sz, uint32_t V)
{
    const uint32_t cap = (uint32_t)C::STR - 2u * (V - 1u);   // staged elements per slot
    if (!sz || 4u * sz > cap || 3u * sz > (uint32_t)C::MAXT) return 0;
    const uint32_t by_slot = cap / sz - 3u, by_threads = (uint32_t)C::MAXT / sz - 2u;
    return by_slot < by_threads ? by_slot : by_threads;
}

template <typename R>
uint32_t step_max_rows(int shape, uint32_t sz)
{
    constexpr uint32_t V = 16 / sizeof(R);
    if (sizeof(R) == 8) return max_rows_of<StepF64>(sz, V);
    return shape == STEP_SHAPE_SMALL ? max_rows_of<StepSmall>(sz, V) : max_rows_of<StepBig>(sz, V);
}

template <typename R>
size_t step_smem_bytes(int shape, uint32_t nstage, uint32_t stage_elems, uint32_t ncoef)
{
    const size_t maxt = sizeof(R) == 8 ? StepF64::MAXT : shape == STEP_SHAPE_SMALL ? StepSmall::MAXT : StepBig::MAXT;
    return ((size_t)nstage * stage_elems + 18u * maxt + ((ncoef + 3u) & ~3u)) * sizeof(R) +
           (size_t)STEP_MAX_STAGES * sizeof(uint64_t);
}

uint32_t step_threads(uint32_t rows, uint32_t sz)
{
    const uint32_t n = (rows + 2u) * sz;
    return (n + 31u) / 32u * 32u;
}

template <typename R, typename C, int DX, bool MU>
static cudaError_t launch_one(const StepK<R> &k, uint32_t threads, size_t smem, cudaStream_t st)
{
    static int configured[64];
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
    if (configured[dev] < (int)smem) {
        e = cudaFuncSetAttribute(k_step<R, C, DX, MU>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        configured[dev] = (int)smem;
    }
    const dim3 g(k.ntile, (k.sx + k.xchunk - 1) / k.xchunk, 1);
    k_step<R, C, DX, MU><<<g, threads, smem, st>>>(k);
    return cudaGetLastError();
}

template <typename R, typename C>
static cudaError_t launch_shape(const StepK<R> &k, int dxmode, bool mu, uint32_t threads, size_t smem,
                                cudaStream_t st)
{
    if (mu) {
        if (dxmode == 0) return launch_one<R, C, 0, true>(k, threads, smem, st);
        if (dxmode == 1) return launch_one<R, C, 1, true>(k, threads, smem, st);
        return launch_one<R, C, 2, true>(k, threads, smem, st);
    }
    if (dxmode == 0) return launch_one<R, C, 0, false>(k, threads, smem, st);
    if (dxmode == 1) return launch_one<R, C, 1, false>(k, threads, smem, st);
    return launch_one<R, C, 2, false>(k, threads, smem, st);
}

template <>
cudaError_t launch_step<float>(const StepK<float> &k, int shape, int dxmode, bool mu, uint32_t threads,
                               size_t smem, cudaStream_t st)
{
    if (shape == STEP_SHAPE_SMALL) return launch_shape<float, StepSmall>(k, dxmode, mu, threads, smem, st);
    return launch_shape<float, StepBig>(k, dxmode, mu, threads, smem, st);
}

template <>
cudaError_t launch_step<double>(const StepK<double> &k, int, int dxmode, bool mu, uint32_t threads, size_t smem,
                                cudaStream_t st)
{
    return launch_shape<double, StepF64>(k, dxmode, mu, threads, smem, st);
}

template uint32_t step_max_rows<float>(int, uint32_t);
template uint32_t step_max_rows<double>(int, uint32_t);
template size_t step_smem_bytes<float>(int, uint32_t, uint32_t, uint32_t);
template size_t step_smem_bytes<double>(int, uint32_t, uint32_t, uint32_t);

}  // namespace fdtd
