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
//     Its E window is the rows [y0 - 1, y0 + nown], one thread per cell; the H window is
//     [y0 - 1, y0 + nown), S is formed on the own rows. Row y0 - 1 exists only to give S the
//     products of its y - 1 neighbours, row y0 + nown only to give H its y + 1 neighbours.
//   * Iteration x: E_new at plane x (H of plane x and x - 1); H_new and the six Poynting products
//     at plane x - 1 (E_new of planes x - 1 and x); S at plane x - 1 (products of planes x - 1
//     and x - 2). The x - 1 values a cell needs from itself stay in registers; E_new of plane
//     x - 1 and the products go to two small double-buffered shared arrays, so one barrier per
//     plane orders everything.
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
template <typename R, bool MU>
__device__ __forceinline__ void fill_bulk(const StepK<R> &k, R *st, uint64_t *bar, const StageGeo &g, uint32_t lane)
{
    constexpr uint64_t V = 16 / sizeof(R);
    constexpr int STR = StepCfg<R>::STR;
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
        const int q = (int)lane - SG_NF, type = q >> 2, side = (q >> 1) & 1, uv = q & 1;
        const uint32_t T = (uint32_t)(side ? k.ax[2].Tp : k.ax[2].Tn);
        if (T) {
            src = k.ax[2].psiA[type][side][uv];
            first = ((uint64_t)g.x * k.sy + g.yH) * T;
            count = (uint64_t)g.rows * T;
            dst = st + k.zoff[q];
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
template <typename R, bool MU>
__device__ __forceinline__ void fill_async(const StepK<R> &k, R *st, const StageGeo &g, bool live, uint32_t t,
                                           uint32_t nt)
{
    constexpr int STR = StepCfg<R>::STR;
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
            for (uint32_t q = t; q < m; q += nt) {
                const uint32_t rq = q / T, ir = q - rq * T;
                const uint64_t off = ((uint64_t)g.x * sy + (g.yH + rq) % sy) * T + ir;
#pragma unroll
                for (int type = 0; type < 2; ++type)
#pragma unroll
                    for (int uv = 0; uv < 2; ++uv) {
                        const int zq = (type * 2 + side) * 2 + uv;
                        async_elem(st + k.zoff[zq] + g.zlead[side] + q, k.ax[2].psiA[type][side][uv] + off);
                    }
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

template <typename R, int DX, bool MU>
__global__ void __launch_bounds__(StepCfg<R>::MAXT, 1) k_step(const __grid_constant__ StepK<R> k)
{
    constexpr int MAXT = StepCfg<R>::MAXT;
    constexpr int STR = StepCfg<R>::STR;
    constexpr uint32_t V = 16 / sizeof(R);
    extern __shared__ __align__(128) unsigned char step_smem[];
    R *const stages = reinterpret_cast<R *>(step_smem);
    R *const XE = stages + (size_t)k.nstage * k.stage_elems;     // [2][3][MAXT] E_new of a plane
    R *const PB = XE + 6 * MAXT;                                 // [2][4][MAXT] products of a plane
    uint64_t *const full = reinterpret_cast<uint64_t *>(PB + 8 * MAXT);

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

    const uint32_t t = threadIdx.x;
    const bool act = t < (nown + 2u) * sz;
    const uint32_t rr = act ? t / sz : 0u;
    const uint32_t z = act ? t - rr * sz : 0u;
    const uint32_t r = rr + 1u;                          // window row (0 is staged only)
    const uint32_t p = r * sz + z;                       // position in a field slot (before lead)
    const bool hrow = act && r <= nown + 1u;
    const bool own = act && r >= 2u && r <= nown + 1u;
    const uint32_t y = (yH + r) % sy;
    const uint32_t j = y * sz + z;
    const int dmz = z ? -1 : (int)sz - 1;                // z - 1 / z + 1 within the row (periodic)
    const int dpz = (z + 1u < sz) ? 1 : 1 - (int)sz;
    int fy_side, fz_side;
    const int fy_ir = step_face(k.ax[1].Tn, k.ax[1].Tp, sy, y, fy_side);
    const int fz_ir = step_face(k.ax[2].Tn, k.ax[2].Tp, sz, z, fz_side);
    const uint32_t fy_T = (uint32_t)(fy_side ? k.ax[1].Tp : k.ax[1].Tn);
    const uint32_t fz_T = (uint32_t)(fz_side ? k.ax[2].Tp : k.ax[2].Tn);
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
    // psi_E of the x and y faces for the next E evaluation, psi_H (x, y, z faces) for the next
    // H evaluation
    R pe[4] = {R(0), R(0), R(0), R(0)};
    R ph[6] = {R(0), R(0), R(0), R(0), R(0), R(0)};
    auto load_pe = [&](uint32_t x) {
        int xs_;
        const int xi = step_face(k.ax[0].Tn, k.ax[0].Tp, sx, x, xs_);
        pe[0] = pe[1] = pe[2] = pe[3] = R(0);
        if (xi >= 0) {
            const uint64_t ip = (uint64_t)xi * syz + j;
            pe[0] = ldg(k.ax[0].psiA[0][xs_][0] + ip);
            pe[1] = ldg(k.ax[0].psiA[0][xs_][1] + ip);
        }
        if (fy_ir >= 0) {
            const uint64_t ip = ((uint64_t)x * fy_T + fy_ir) * sz + z;
            pe[2] = ldg(k.ax[1].psiA[0][fy_side][0] + ip);
            pe[3] = ldg(k.ax[1].psiA[0][fy_side][1] + ip);
        }
    };
    if (act) load_pe(plane(0));

    // first stages
    const int npre = NS < nit ? NS : nit;
    if (tma) {
        if (t < 32)
            for (int q = 0; q < npre; ++q) fill_bulk<R, MU>(k, stages + (size_t)q * k.stage_elems, &full[q], geo(q), t);
    } else {
        for (int q = 0; q < NS; ++q) fill_async<R, MU>(k, stages + (size_t)q * k.stage_elems, geo(q), q < nit, t, nt);
        async_wait_n(NS - 1);
        __syncthreads();
    }

    R ex_m = R(0), ey_m = R(0), ez_m = R(0);            // E_new of plane x - 1 at the cell
    R cx_m = R(0), cy_m = R(0), cz_m = R(0);            // dt/mu of plane x - 1
    R p_yx = R(0), p_zx = R(0);                          // products yx, zx of plane x - 2
    int it = 0;
    bool abort = false;
    for (; it < nit; ++it) {
        const uint32_t x = plane(it);
        const int slot = it % NS;
        R *const st = stages + (size_t)slot * k.stage_elems;
        bool failed = false;
        if (tma) failed = !stage_wait(&full[slot], (uint32_t)(it / NS) & 1u, k.wait_ns, k.status);
        const uint32_t xs = x * syz;
        const R *const b0 = st + ((kc0 + xs) & (V - 1)) + p;
        const R *const b1 = st + ((kc0 + xs + nlo) & (V - 1)) + p;
        const R *const b2 = st + ((kc0 + xs + 2u * nlo) & (V - 1)) + p;
        const bool ein = it >= 1 && it <= nit - 2;       // plane x is in the block's chunk
        const bool hin = it >= 2;                        // plane x - 1 is in the block's chunk
        int xf_side;
        const int xf_ir = step_face(k.ax[0].Tn, k.ax[0].Tp, sx, x, xf_side);
        const uint32_t zrow = ((x * sy + yH) * fz_T) & (V - 1);   // lead of this cell's z slots

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
                const R *const *tb = k.ax[0].tab[0][xf_side];
                R su, sv;
                face_update<R, true, 0>(ldg(tb[0] + xf_ir), ldg(tb[1] + xf_ir), ldg(tb[2] + xf_ir), pe[0], pe[1],
                                        su, sv, d_xy, d_xz, d_yx, d_yz, d_zx, d_zy, px, py, pz);
                if (wr) {
                    const uint64_t ip = (uint64_t)xf_ir * syz + j;
                    k.ax[0].psiB[0][xf_side][0][ip] = su;
                    k.ax[0].psiB[0][xf_side][1][ip] = sv;
                }
            }
            if (fy_ir >= 0) {
                const R *const *tb = k.ax[1].tab[0][fy_side];
                R su, sv;
                face_update<R, true, 1>(ldg(tb[0] + fy_ir), ldg(tb[1] + fy_ir), ldg(tb[2] + fy_ir), pe[2], pe[3],
                                        su, sv, d_xy, d_xz, d_yx, d_yz, d_zx, d_zy, px, py, pz);
                if (wr) {
                    const uint64_t ip = ((uint64_t)x * fy_T + fy_ir) * sz + z;
                    k.ax[1].psiB[0][fy_side][0][ip] = su;
                    k.ax[1].psiB[0][fy_side][1][ip] = sv;
                }
            }
            if (fz_ir >= 0) {
                const R *const *tb = k.ax[2].tab[0][fz_side];
                const uint32_t zq = zrow + r * fz_T + (uint32_t)fz_ir;
                const R ou = st[k.zoff[fz_side * 2 + 0] + zq], ov = st[k.zoff[fz_side * 2 + 1] + zq];
                R su, sv;
                face_update<R, true, 2>(ldg(tb[0] + fz_ir), ldg(tb[1] + fz_ir), ldg(tb[2] + fz_ir), ou, ov,
                                        su, sv, d_xy, d_xz, d_yx, d_yz, d_zx, d_zy, px, py, pz);
                if (wr) {
                    const uint64_t ip = ((uint64_t)x * sy + y) * fz_T + fz_ir;
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
                R *const e = k.EB + ((uint64_t)xs + j);
                e[0] = ex;
                e[N] = ey;
                e[2 * N] = ez;
            }
            R *const xe = XE + (it & 1) * 3 * MAXT + t;
            xe[0] = ex;
            xe[MAXT] = ey;
            xe[2 * MAXT] = ez;
        }
        if (act && it + 1 < nit) load_pe(plane(it + 1));

        // ---- H_new and the products at plane xm = x - 1 (update_h.cl:36-155) ----
        R os0 = R(0), os1 = R(0), os2 = R(0), os3 = R(0), os4 = R(0), os5 = R(0);
        if (hrow && it >= 1 && !failed) {
            const uint32_t xm = x ? x - 1u : sx - 1u;
            const R *const xe = XE + ((it - 1) & 1) * 3 * MAXT;
            const R rxy = xe[t + sz], rzy = xe[2 * MAXT + t + sz];
            const R rxz = xe[(int)t + dpz], ryz = xe[MAXT + (int)t + dpz];
            R d_xy = rxy - ex_m;
            R d_xz = rxz - ex_m;
            R d_yx = ey - ey_m;
            R d_yz = ryz - ey_m;
            R d_zx = ez - ez_m;
            R d_zy = rzy - ez_m;
            if (DX != 0) {
                R ix = k.inv_d, iy = k.inv_d, iz = k.inv_d;
                if (DX == 2) { ix = ldg(k.inv_de[0] + xm); iy = ldg(k.inv_de[1] + y); iz = ldg(k.inv_de[2] + z); }
                d_xy = d_xy * iy; d_xz = d_xz * iz; d_yx = d_yx * ix;
                d_yz = d_yz * iz; d_zx = d_zx * ix; d_zy = d_zy * iy;
            }
            R px = R(0), py = R(0), pz = R(0);
            const bool wr = own && hin;
            int mf_side;
            const int mf_ir = step_face(k.ax[0].Tn, k.ax[0].Tp, sx, xm, mf_side);
            if (mf_ir >= 0) {
                const R *const *tb = k.ax[0].tab[1][mf_side];
                R su, sv;
                face_update<R, false, 0>(ldg(tb[0] + mf_ir), ldg(tb[1] + mf_ir), ldg(tb[2] + mf_ir), ph[0], ph[1],
                                         su, sv, d_xy, d_xz, d_yx, d_yz, d_zx, d_zy, px, py, pz);
                if (wr) {
                    const uint64_t ip = (uint64_t)mf_ir * syz + j;
                    k.ax[0].psiB[1][mf_side][0][ip] = su;
                    k.ax[0].psiB[1][mf_side][1][ip] = sv;
                }
            }
            if (fy_ir >= 0) {
                const R *const *tb = k.ax[1].tab[1][fy_side];
                R su, sv;
                face_update<R, false, 1>(ldg(tb[0] + fy_ir), ldg(tb[1] + fy_ir), ldg(tb[2] + fy_ir), ph[2], ph[3],
                                         su, sv, d_xy, d_xz, d_yx, d_yz, d_zx, d_zy, px, py, pz);
                if (wr) {
                    const uint64_t ip = ((uint64_t)xm * fy_T + fy_ir) * sz + z;
                    k.ax[1].psiB[1][fy_side][0][ip] = su;
                    k.ax[1].psiB[1][fy_side][1][ip] = sv;
                }
            }
            if (fz_ir >= 0) {
                const R *const *tb = k.ax[2].tab[1][fz_side];
                R su, sv;
                face_update<R, false, 2>(ldg(tb[0] + fz_ir), ldg(tb[1] + fz_ir), ldg(tb[2] + fz_ir), ph[4], ph[5],
                                         su, sv, d_xy, d_xz, d_yx, d_yz, d_zx, d_zy, px, py, pz);
                if (wr) {
                    const uint64_t ip = ((uint64_t)xm * sy + y) * fz_T + fz_ir;
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
            const uint64_t i = (uint64_t)xm * syz + j;
            if (wr) {
                R *const h = k.HB + i;
                h[0] = hxn;
                h[N] = hyn;
                h[2 * N] = hzn;
            }
            if (k.poynt) {
                const R ahx = hxn + hx_m, ahy = hyn + hy_m, ahz = hzn + hz_m;
                os0 = (ey + ey_m) * ahz;
                os3 = (-(ez + ez_m)) * ahy;
                os1 = (rzy + ez_m) * ahx;
                os4 = (-(rxy + ex_m)) * ahz;
                os2 = (rxz + ex_m) * ahy;
                os5 = (-(ryz + ey_m)) * ahx;
                if (wr && k.write_oS) {
                    R *const o = k.oS + i;
                    o[0] = os0;
                    o[N] = os1;
                    o[2 * N] = os2;
                    o[3 * N] = os3;
                    o[4 * N] = os4;
                    o[5 * N] = os5;
                }
                R *const pb = PB + (it & 1) * 4 * MAXT + t;
                pb[0] = os0;
                pb[MAXT] = os3;
                pb[2 * MAXT] = os1;
                pb[3 * MAXT] = os5;
            }
        }
        // what the next H evaluation (plane x) needs from this plane
        if (act && !failed) {
            ph[0] = ph[1] = ph[2] = ph[3] = R(0);
            if (xf_ir >= 0) {
                const uint64_t ip = (uint64_t)xf_ir * syz + j;
                ph[0] = ldg(k.ax[0].psiA[1][xf_side][0] + ip);
                ph[1] = ldg(k.ax[0].psiA[1][xf_side][1] + ip);
            }
            if (fy_ir >= 0) {
                const uint64_t ip = ((uint64_t)x * fy_T + fy_ir) * sz + z;
                ph[2] = ldg(k.ax[1].psiA[1][fy_side][0] + ip);
                ph[3] = ldg(k.ax[1].psiA[1][fy_side][1] + ip);
            }
            if (fz_ir >= 0) {
                const uint32_t zq = zrow + r * fz_T + (uint32_t)fz_ir;
                ph[4] = st[k.zoff[(2 + fz_side) * 2 + 0] + zq];
                ph[5] = st[k.zoff[(2 + fz_side) * 2 + 1] + zq];
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
            if (t < 32 && it + NS < nit) fill_bulk<R, MU>(k, st, &full[slot], geo(it + NS), t);
        } else {
            fill_async<R, MU>(k, st, geo(it + NS), it + NS < nit, t, nt);
        }

        // ---- S at plane x - 1 (update_s.cl:33-36) ----
        if (k.poynt && own && hin) {
            const R *const pb = PB + (it & 1) * 4 * MAXT;
            const R xy_y = pb[t - sz], zy_y = pb[3 * MAXT + t - sz];
            const R xz_z = pb[MAXT + (int)t + dmz], yz_z = pb[2 * MAXT + (int)t + dmz];
            const uint32_t xm = x ? x - 1u : sx - 1u;
            R *const s = k.S + ((uint64_t)xm * syz + j);
            s[0] = (((os0 + os3) + xy_y) + xz_z) * k.sf;
            s[N] = (((os1 + os4) + yz_z) + p_yx) * k.sf;
            s[2 * N] = (((os2 + os5) + p_zx) + zy_y) * k.sf;
        }
        p_yx = os4;
        p_zx = os2;
        ex_m = ex;
        ey_m = ey;
        ez_m = ez;
    }
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
template <typename R>
uint32_t step_max_rows(uint32_t sz)
{
    constexpr uint32_t V = 16 / sizeof(R);
    const uint32_t cap = (uint32_t)StepCfg<R>::STR - 2u * (V - 1u);   // staged elements per slot
    if (!sz || 4u * sz > cap || 3u * sz > (uint32_t)StepCfg<R>::MAXT) return 0;
    const uint32_t by_slot = cap / sz - 3u, by_threads = (uint32_t)StepCfg<R>::MAXT / sz - 2u;
    return by_slot < by_threads ? by_slot : by_threads;
}

template <typename R>
size_t step_smem_bytes(uint32_t nstage, uint32_t stage_elems)
{
    return ((size_t)nstage * stage_elems + 14u * (size_t)StepCfg<R>::MAXT) * sizeof(R) +
           (size_t)STEP_MAX_STAGES * sizeof(uint64_t);
}

uint32_t step_threads(uint32_t rows, uint32_t sz)
{
    const uint32_t n = (rows + 2u) * sz;
    return (n + 31u) / 32u * 32u;
}

template <typename R, int DX, bool MU>
static cudaError_t launch_one(const StepK<R> &k, uint32_t threads, size_t smem, cudaStream_t st)
{
    static int configured[64];
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
    if (configured[dev] < (int)smem) {
        e = cudaFuncSetAttribute(k_step<R, DX, MU>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        configured[dev] = (int)smem;
    }
    const dim3 g(k.ntile, (k.sx + k.xchunk - 1) / k.xchunk, 1);
    k_step<R, DX, MU><<<g, threads, smem, st>>>(k);
    return cudaGetLastError();
}

template <typename R>
cudaError_t launch_step(const StepK<R> &k, int dxmode, bool mu, uint32_t threads, size_t smem, cudaStream_t st)
{
    if (mu) {
        if (dxmode == 0) return launch_one<R, 0, true>(k, threads, smem, st);
        if (dxmode == 1) return launch_one<R, 1, true>(k, threads, smem, st);
        return launch_one<R, 2, true>(k, threads, smem, st);
    }
    if (dxmode == 0) return launch_one<R, 0, false>(k, threads, smem, st);
    if (dxmode == 1) return launch_one<R, 1, false>(k, threads, smem, st);
    return launch_one<R, 2, false>(k, threads, smem, st);
}

template uint32_t step_max_rows<float>(uint32_t);
template uint32_t step_max_rows<double>(uint32_t);
template size_t step_smem_bytes<float>(uint32_t, uint32_t);
template size_t step_smem_bytes<double>(uint32_t, uint32_t);
template cudaError_t launch_step<float>(const StepK<float> &, int, bool, uint32_t, size_t, cudaStream_t);
template cudaError_t launch_step<double>(const StepK<double> &, int, bool, uint32_t, size_t, cudaStream_t);

}  // namespace fdtd
