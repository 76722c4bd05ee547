// Batched stepping of many independent cavity variants in one persistent launch.
//
// All variants' work is cut into tiles of BATCH_THREADS consecutive (y, z) cells times a chunk
// of x planes. Two schedules run the same tile code:
//   * persistent: a cooperative grid of two blocks per SM takes the tiles of every variant
//     from a device work counter for the E half-step, synchronises the grid, does the same for
//     the H half-step, synchronises again, and repeats -- one launch advances the whole sweep by
//     nsteps steps (two blocks: the E and H tile bodies together need 128 registers without
//     spilling; at three blocks per SM they spill and run slower);
//   * per half-step: one launch of one block per tile for E, one for H, per step (captured in
//     a CUDA graph by the caller); the hardware scheduler then overlaps blocks.
// Either way there is no per-variant launch or tail. Point sources are added and monitor
// points recorded by the thread that updates the cell.
//
// Storage: E, H and dt/eps in float32, or in bfloat16 / float16 with float32 arithmetic. In
// 16-bit storage every tile (one component of the BATCH_TILE cells one warp updates in one x
// plane) carries a power-of-two exponent e: stored value = value * 2^-e, chosen when the tile
// is written so that the tile's largest magnitude lands in [2^13, 2^14) -- inside float16's
// normal range with headroom, whatever the field's absolute level (a ringdown decays through
// many decades). The warp reduces the new values' maximum with shuffles before it stores them
// (no barrier); tiles of a field are only rewritten in that field's half-step, when no other
// tile reads them.
//
// The float32 arithmetic and its order are those of the per-update kernels (this translation
// unit is compiled with --fmad=false), so float32 storage gives results bit-identical to
// stepping each variant on its own.
#include <cooperative_groups.h>
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include "batch.h"
#include "yee_device.cuh"

namespace cg = cooperative_groups;

namespace fdtd {

namespace {

template <int ST>
struct Store;

template <>
struct Store<BATCH_F32> {
    using T = float;
    static constexpr bool scaled = false;
    __device__ static float dec(T v) { return v; }
    __device__ static T enc(float v) { return v; }
};

template <>
struct Store<BATCH_BF16> {
    using T = __nv_bfloat16;
    static constexpr bool scaled = true;
    __device__ static float dec(T v) { return __bfloat162float(v); }
    __device__ static T enc(float v) { return __float2bfloat16_rn(v); }
};

template <>
struct Store<BATCH_F16> {
    using T = __half;
    static constexpr bool scaled = true;
    __device__ static float dec(T v) { return __half2float(v); }
    __device__ static T enc(float v) { return __float2half_rn(v); }
};

template <>
struct Store<BATCH_BF16U> {
    using T = __nv_bfloat16;
    static constexpr bool scaled = false;
    __device__ static float dec(T v) { return __bfloat162float(v); }
    __device__ static T enc(float v) { return __float2bfloat16_rn(v); }
};

// 2^e for e in [-126, 127] (exact)
__device__ __forceinline__ float pow2(int e) { return __int_as_float((e + 127) << 23); }

// exponent of a tile whose largest magnitude is m: m * 2^-e in [2^13, 2^14)
__device__ __forceinline__ int tile_exp(float m)
{
    if (!(m > 0.f) || !isfinite(m)) return 0;
    int E;
    frexpf(m, &E);
    return max(-100, min(100, E - 14));
}

// exponent word of plane x, tile jt (= cell j / BATCH_TILE): the three components' exponents
// e_c as bytes e_c + 128 in bits 8c .. 8c + 7
__device__ __forceinline__ uint32_t texp_index(const BVar &v, uint32_t x, uint32_t jt)
{
    return x * v.ntl + jt;
}

__device__ __forceinline__ int xe(int32_t word, int c) { return (int)(((uint32_t)word >> (8 * c)) & 0xffu) - 128; }

__device__ __forceinline__ int32_t xpack(int e0, int e1, int e2)
{
    return (int32_t)((uint32_t)(e0 + 128) | ((uint32_t)(e1 + 128) << 8) | ((uint32_t)(e2 + 128) << 16));
}

// Largest magnitude of each of three values over the warp (all 32 lanes take part; idle lanes
// pass 0): the tile exponents, identical in every lane. The bit patterns of non-negative floats
// order like the values, so one integer warp reduction per component finds the maximum.
__device__ __forceinline__ void warp_exps(float a, float b, float c, int &ea, int &eb, int &ec)
{
    const uint32_t ma = __reduce_max_sync(0xffffffffu, __float_as_uint(fabsf(a)));
    const uint32_t mb = __reduce_max_sync(0xffffffffu, __float_as_uint(fabsf(b)));
    const uint32_t mc = __reduce_max_sync(0xffffffffu, __float_as_uint(fabsf(c)));
    ea = tile_exp(__uint_as_float(ma));
    eb = tile_exp(__uint_as_float(mb));
    ec = tile_exp(__uint_as_float(mc));
}

// CPML face of one axis fixed for the thread (y or z): depth, side, coefficients
struct BFix {
    int ir, side;
    float p0, p1, p2;
};

__device__ __forceinline__ BFix bfix(const BAxis &a, int h, uint32_t s, uint32_t c, bool act)
{
    BFix f;
    f.ir = -1;
    f.side = 0;
    f.p0 = f.p1 = f.p2 = 0.f;
    if (!act) return f;
    if (c < (uint32_t)a.Tn) {
        f.ir = (int)c;
    } else if (a.Tp && c >= s - (uint32_t)a.Tp) {
        f.ir = (int)(s - 1u - c);
        f.side = 1;
    }
    if (f.ir >= 0) {
        f.p0 = ldg(a.tab[h][f.side][0] + f.ir);
        f.p1 = ldg(a.tab[h][f.side][1] + f.ir);
        f.p2 = ldg(a.tab[h][f.side][2] + f.ir);
    }
    return f;
}

__device__ __forceinline__ int bx_face(const BAxis &a, uint32_t sx, uint32_t x, int &side)
{
    side = 0;
    if (x < (uint32_t)a.Tn) return (int)x;
    if (a.Tp && x >= sx - (uint32_t)a.Tp) {
        side = 1;
        return (int)(sx - 1u - x);
    }
    return -1;
}

// decode of a stored value with its tile exponent (no scaling at all in float32 storage)
template <int ST>
__device__ __forceinline__ float dv(typename Store<ST>::T v, int e)
{
    return Store<ST>::scaled ? Store<ST>::dec(v) * pow2(e) : Store<ST>::dec(v);
}

template <typename T>
__device__ __forceinline__ T ldr(const T *p) { return __ldg(p); }

// ---- E half-step of one tile (update_e.cl:39-107 per cell) ------------------------------------
// Values one E plane reads (stored form and tile exponents), loaded one plane ahead as in the
// per-update kernels.
template <typename T>
struct BELoad {
    T hx, hy, hz, nxy, nxz, nyz, nzy, ex, ey, ez, cx, cy, cz;
    int32_t gh, gy, gz, ge;        // exponent words: own H tile, H at y-1, H at z-1, own E tile
    float xu, xv, yu, yv, zu, zv;
};

// PF: the next plane's loads are issued before the current plane's arithmetic (latency hidden
// by instruction-level parallelism, twice the registers for loaded values); without, latency
// is hidden by more resident warps.
template <int ST, bool PF = true>
__device__ void batch_e_tile(const BVar &v, int4 tl, int64_t step, int64_t rows)
{
    using SS = Store<ST>;
    using T = typename SS::T;
    const uint32_t sx = v.sx, sy = v.sy, sz = v.sz, syz = v.syz;
    const uint64_t N = v.N;
    const uint32_t xa = (uint32_t)tl.y, xb = (uint32_t)tl.z, jb = (uint32_t)tl.w;
    const uint32_t j = jb * BATCH_THREADS + threadIdx.x;
    const bool act = j < syz;
    const uint32_t y = act ? v.dsz.div(j) : 0u;
    const uint32_t z = act ? j - y * sz : 0u;
    const T *Hx = (const T *)v.H, *Hy = Hx + N, *Hz = Hx + 2 * N;
    T *Ex = (T *)v.E, *Ey = Ex + N, *Ez = Ex + 2 * N;
    const T *C = (const T *)v.ce;
    const int32_t *hexp = v.hexp;
    int32_t *eexp = v.eexp;
    // minus neighbours with periodic wrap (common.cl:75-81), 32-bit modular offsets
    const uint32_t dmy = y ? 0u - sz : (sy - 1u) * sz;
    const uint32_t dmz = z ? 0xffffffffu : sz - 1u;
    const uint32_t jt = j / BATCH_TILE;                          // own exponent tile
    const uint32_t jby = (j + dmy) / BATCH_TILE, jbz = (j + dmz) / BATCH_TILE;
    const BFix fy = bfix(v.ax[1], 0, sy, y, act);
    const BFix fz = bfix(v.ax[2], 0, sz, z, act);
    const float inv = v.inv_d;
    const BAxis &ax0 = v.ax[0], &ax1 = v.ax[1], &ax2 = v.ax[2];

    auto load = [&](uint32_t x) {
        BELoad<T> q;
        const uint32_t i = x * syz + j;
        const uint32_t imy = i + dmy, imz = i + dmz;   // 32-bit wrap arithmetic
        q.hx = ldr(Hx + i); q.hy = ldr(Hy + i); q.hz = ldr(Hz + i);
        q.nxy = ldr(Hx + imy); q.nzy = ldr(Hz + imy);
        q.nxz = ldr(Hx + imz); q.nyz = ldr(Hy + imz);
        q.ex = Ex[i]; q.ey = Ey[i]; q.ez = Ez[i];
        q.cx = ldr(C + i); q.cy = ldr(C + N + i); q.cz = ldr(C + 2 * N + i);
        if (SS::scaled) {
            q.gh = hexp[texp_index(v, x, jt)];
            q.gy = hexp[texp_index(v, x, jby)];
            q.gz = hexp[texp_index(v, x, jbz)];
            q.ge = eexp[texp_index(v, x, jt)];
        }
        q.xu = q.xv = q.yu = q.yv = q.zu = q.zv = 0.f;
        int side;
        const int irx = bx_face(ax0, sx, x, side);
        if (irx >= 0) {
            const uint32_t ip = ((uint32_t)irx * sy + y) * sz + z;
            q.xu = ax0.psi[0][side][0][ip]; q.xv = ax0.psi[0][side][1][ip];
        }
        if (fy.ir >= 0) {
            const uint32_t ip = (x * (uint32_t)(fy.side ? ax1.Tp : ax1.Tn) + (uint32_t)fy.ir) * sz + z;
            q.yu = ax1.psi[0][fy.side][0][ip]; q.yv = ax1.psi[0][fy.side][1][ip];
        }
        if (fz.ir >= 0) {
            const uint32_t ip = (x * sy + y) * (uint32_t)(fz.side ? ax2.Tp : ax2.Tn) + (uint32_t)fz.ir;
            q.zu = ax2.psi[0][fz.side][0][ip]; q.zv = ax2.psi[0][fz.side][1][ip];
        }
        return q;
    };

    float hy_m = 0.f, hz_m = 0.f;
    BELoad<T> cur;
    if (act) {
        const uint32_t xm = xa ? xa - 1u : sx - 1u;
        const uint32_t im = xm * syz + j;
        const int32_t wm = SS::scaled ? hexp[texp_index(v, xm, jt)] : 0;
        hy_m = dv<ST>(ldr(Hy + im), xe(wm, 1));
        hz_m = dv<ST>(ldr(Hz + im), xe(wm, 2));
        if (PF) cur = load(xa);
    }
    for (uint32_t x = xa; x < xb; ++x) {
        const uint32_t i = x * syz + j;
        BELoad<T> nxt;
        float nx = 0.f, ny = 0.f, nz = 0.f, hy = 0.f, hz = 0.f;
        if (act) {
            if (!PF) cur = load(x);
            else if (x + 1u < xb) nxt = load(x + 1u);
            const float hx = dv<ST>(cur.hx, xe(cur.gh, 0));
            hy = dv<ST>(cur.hy, xe(cur.gh, 1));
            hz = dv<ST>(cur.hz, xe(cur.gh, 2));
            // backward differences (update_e.cl:39-46), times 1/dx (exact for dx = 1)
            float d_xy = (hx - dv<ST>(cur.nxy, xe(cur.gy, 0))) * inv;
            float d_xz = (hx - dv<ST>(cur.nxz, xe(cur.gz, 0))) * inv;
            float d_yx = (hy - hy_m) * inv;
            float d_yz = (hy - dv<ST>(cur.nyz, xe(cur.gz, 1))) * inv;
            float d_zx = (hz - hz_m) * inv;
            float d_zy = (hz - dv<ST>(cur.nzy, xe(cur.gy, 2))) * inv;
            // CPML (update_e.cl:64-100): at most one face per axis
            float px = 0.f, py = 0.f, pz = 0.f;
            int side;
            const int irx = bx_face(ax0, sx, x, side);
            if (irx >= 0) {
                const uint32_t ip = ((uint32_t)irx * sy + y) * sz + z;
                float su, sv;
                face_update<float, true, 0>(ldg(ax0.tab[0][side][0] + irx), ldg(ax0.tab[0][side][1] + irx),
                                            ldg(ax0.tab[0][side][2] + irx), cur.xu, cur.xv, su, sv,
                                            d_xy, d_xz, d_yx, d_yz, d_zx, d_zy, px, py, pz);
                ax0.psi[0][side][0][ip] = su;
                ax0.psi[0][side][1][ip] = sv;
            }
            if (fy.ir >= 0) {
                const uint32_t ip = (x * (uint32_t)(fy.side ? ax1.Tp : ax1.Tn) + (uint32_t)fy.ir) * sz + z;
                float su, sv;
                face_update<float, true, 1>(fy.p0, fy.p1, fy.p2, cur.yu, cur.yv, su, sv,
                                            d_xy, d_xz, d_yx, d_yz, d_zx, d_zy, px, py, pz);
                ax1.psi[0][fy.side][0][ip] = su;
                ax1.psi[0][fy.side][1][ip] = sv;
            }
            if (fz.ir >= 0) {
                const uint32_t ip = (x * sy + y) * (uint32_t)(fz.side ? ax2.Tp : ax2.Tn) + (uint32_t)fz.ir;
                float su, sv;
                face_update<float, true, 2>(fz.p0, fz.p1, fz.p2, cur.zu, cur.zv, su, sv,
                                            d_xy, d_xz, d_yx, d_yz, d_zx, d_zy, px, py, pz);
                ax2.psi[0][fz.side][0][ip] = su;
                ax2.psi[0][fz.side][1][ip] = sv;
            }
            // update_e.cl:105-107
            nx = dv<ST>(cur.ex, xe(cur.ge, 0)) + SS::dec(cur.cx) * ((d_zy - d_yz) + px);
            ny = dv<ST>(cur.ey, xe(cur.ge, 1)) + SS::dec(cur.cy) * ((d_xz - d_zx) + py);
            nz = dv<ST>(cur.ez, xe(cur.ge, 2)) + SS::dec(cur.cz) * ((d_yx - d_xy) + pz);
            // point sources after the update (fdtd.py:168-169: E[ind] += value)
            if (v.nsrc > 0 && step < rows) {
                for (int s = 0; s < v.nsrc; ++s) {
                    if (v.src_x[s] != x || v.src_j[s] != j) continue;
                    const float val = v.src_values[step * v.nsrc + s];
                    if (v.src_c[s] == 0) nx = nx + val;
                    else if (v.src_c[s] == 1) ny = ny + val;
                    else nz = nz + val;
                }
            }
        }
        int e0 = 0, e1 = 0, e2 = 0;
        if (SS::scaled) {
            warp_exps(nx, ny, nz, e0, e1, e2);
            if ((threadIdx.x & 31u) == 0 && jt < v.ntl) eexp[texp_index(v, x, jt)] = xpack(e0, e1, e2);
        }
        if (act) {
            const T wx = SS::enc(SS::scaled ? nx * pow2(-e0) : nx);
            const T wy = SS::enc(SS::scaled ? ny * pow2(-e1) : ny);
            const T wz = SS::enc(SS::scaled ? nz * pow2(-e2) : nz);
            Ex[i] = wx;
            Ey[i] = wy;
            Ez[i] = wz;
            if (v.nmon > 0 && step < rows) {
                for (int m = 0; m < v.nmon; ++m) {
                    if (v.mon_x[m] != x || v.mon_j[m] != j) continue;
                    const int c = v.mon_c[m];
                    const T w = c == 0 ? wx : c == 1 ? wy : wz;
                    v.series[step * v.nmon + m] = (double)dv<ST>(w, c == 0 ? e0 : c == 1 ? e1 : e2);
                }
            }
            hy_m = hy;
            hz_m = hz;
            if (PF) cur = nxt;
        }
    }
}

// ---- H half-step of one tile (update_h.cl:36-131 per cell; Poynting off) ----------------------
template <typename T>
struct BHLoad {
    T ex1, ey1, ez1, rxy, rxz, ryz, rzy, hx, hy, hz;
    int32_t ge, gy, gz, gh;        // exponent words: E at x+1, E at y+1, E at z+1, own H tile
    float xu, xv, yu, yv, zu, zv;
};

template <int ST, bool PF = true>
__device__ void batch_h_tile(const BVar &v, int4 tl)
{
    using SS = Store<ST>;
    using T = typename SS::T;
    const uint32_t sx = v.sx, sy = v.sy, sz = v.sz, syz = v.syz;
    const uint64_t N = v.N;
    const uint32_t xa = (uint32_t)tl.y, xb = (uint32_t)tl.z, jb = (uint32_t)tl.w;
    const uint32_t j = jb * BATCH_THREADS + threadIdx.x;
    const bool act = j < syz;
    const uint32_t y = act ? v.dsz.div(j) : 0u;
    const uint32_t z = act ? j - y * sz : 0u;
    const T *Ex = (const T *)v.E, *Ey = Ex + N, *Ez = Ex + 2 * N;
    T *Hx = (T *)v.H, *Hy = Hx + N, *Hz = Hx + 2 * N;
    int32_t *hexp = v.hexp;
    const int32_t *eexp = v.eexp;
    // plus neighbours with periodic wrap (common.cl:82-84)
    const uint32_t dpy = (y + 1u < sy) ? sz : 0u - (sy - 1u) * sz;
    const uint32_t dpz = (z + 1u < sz) ? 1u : 0u - (sz - 1u);
    const uint32_t jt = j / BATCH_TILE;
    const uint32_t jby = (j + dpy) / BATCH_TILE, jbz = (j + dpz) / BATCH_TILE;
    const BFix fy = bfix(v.ax[1], 1, sy, y, act);
    const BFix fz = bfix(v.ax[2], 1, sz, z, act);
    const float inv = v.inv_d, dt = v.dt;
    const BAxis &ax0 = v.ax[0], &ax1 = v.ax[1], &ax2 = v.ax[2];

    auto load = [&](uint32_t x) {
        BHLoad<T> q;
        const uint32_t i = x * syz + j;
        const uint32_t x1 = (x + 1u < sx) ? x + 1u : 0u;
        const uint32_t i1 = x1 * syz + j;
        const uint32_t ipy = i + dpy, ipz = i + dpz;   // 32-bit wrap arithmetic
        q.ex1 = ldr(Ex + i1); q.ey1 = ldr(Ey + i1); q.ez1 = ldr(Ez + i1);
        q.rxy = ldr(Ex + ipy); q.rzy = ldr(Ez + ipy);
        q.rxz = ldr(Ex + ipz); q.ryz = ldr(Ey + ipz);
        q.hx = Hx[i]; q.hy = Hy[i]; q.hz = Hz[i];
        if (SS::scaled) {
            q.ge = eexp[texp_index(v, x1, jt)];
            q.gy = eexp[texp_index(v, x, jby)];
            q.gz = eexp[texp_index(v, x, jbz)];
            q.gh = hexp[texp_index(v, x, jt)];
        }
        q.xu = q.xv = q.yu = q.yv = q.zu = q.zv = 0.f;
        int side;
        const int irx = bx_face(ax0, sx, x, side);
        if (irx >= 0) {
            const uint32_t ip = ((uint32_t)irx * sy + y) * sz + z;
            q.xu = ax0.psi[1][side][0][ip]; q.xv = ax0.psi[1][side][1][ip];
        }
        if (fy.ir >= 0) {
            const uint32_t ip = (x * (uint32_t)(fy.side ? ax1.Tp : ax1.Tn) + (uint32_t)fy.ir) * sz + z;
            q.yu = ax1.psi[1][fy.side][0][ip]; q.yv = ax1.psi[1][fy.side][1][ip];
        }
        if (fz.ir >= 0) {
            const uint32_t ip = (x * sy + y) * (uint32_t)(fz.side ? ax2.Tp : ax2.Tn) + (uint32_t)fz.ir;
            q.zu = ax2.psi[1][fz.side][0][ip]; q.zv = ax2.psi[1][fz.side][1][ip];
        }
        return q;
    };

    float ex = 0.f, ey = 0.f, ez = 0.f;
    BHLoad<T> cur;
    if (act) {
        const uint32_t i = xa * syz + j;
        const int32_t wa = SS::scaled ? eexp[texp_index(v, xa, jt)] : 0;
        ex = dv<ST>(ldr(Ex + i), xe(wa, 0));
        ey = dv<ST>(ldr(Ey + i), xe(wa, 1));
        ez = dv<ST>(ldr(Ez + i), xe(wa, 2));
        if (PF) cur = load(xa);
    }
    for (uint32_t x = xa; x < xb; ++x) {
        const uint32_t i = x * syz + j;
        BHLoad<T> nxt;
        float nx = 0.f, ny = 0.f, nz = 0.f, ex1 = 0.f, ey1 = 0.f, ez1 = 0.f;
        if (act) {
            if (!PF) cur = load(x);
            else if (x + 1u < xb) nxt = load(x + 1u);
            ex1 = dv<ST>(cur.ex1, xe(cur.ge, 0));
            ey1 = dv<ST>(cur.ey1, xe(cur.ge, 1));
            ez1 = dv<ST>(cur.ez1, xe(cur.ge, 2));
            // forward differences (update_h.cl:36-43), times 1/dx
            float d_xy = (dv<ST>(cur.rxy, xe(cur.gy, 0)) - ex) * inv;
            float d_xz = (dv<ST>(cur.rxz, xe(cur.gz, 0)) - ex) * inv;
            float d_yx = (ey1 - ey) * inv;
            float d_yz = (dv<ST>(cur.ryz, xe(cur.gz, 1)) - ey) * inv;
            float d_zx = (ez1 - ez) * inv;
            float d_zy = (dv<ST>(cur.rzy, xe(cur.gy, 2)) - ez) * inv;
            float px = 0.f, py = 0.f, pz = 0.f;
            int side;
            const int irx = bx_face(ax0, sx, x, side);
            if (irx >= 0) {
                const uint32_t ip = ((uint32_t)irx * sy + y) * sz + z;
                float su, sv;
                face_update<float, false, 0>(ldg(ax0.tab[1][side][0] + irx), ldg(ax0.tab[1][side][1] + irx),
                                             ldg(ax0.tab[1][side][2] + irx), cur.xu, cur.xv, su, sv,
                                             d_xy, d_xz, d_yx, d_yz, d_zx, d_zy, px, py, pz);
                ax0.psi[1][side][0][ip] = su;
                ax0.psi[1][side][1][ip] = sv;
            }
            if (fy.ir >= 0) {
                const uint32_t ip = (x * (uint32_t)(fy.side ? ax1.Tp : ax1.Tn) + (uint32_t)fy.ir) * sz + z;
                float su, sv;
                face_update<float, false, 1>(fy.p0, fy.p1, fy.p2, cur.yu, cur.yv, su, sv,
                                             d_xy, d_xz, d_yx, d_yz, d_zx, d_zy, px, py, pz);
                ax1.psi[1][fy.side][0][ip] = su;
                ax1.psi[1][fy.side][1][ip] = sv;
            }
            if (fz.ir >= 0) {
                const uint32_t ip = (x * sy + y) * (uint32_t)(fz.side ? ax2.Tp : ax2.Tn) + (uint32_t)fz.ir;
                float su, sv;
                face_update<float, false, 2>(fz.p0, fz.p1, fz.p2, cur.zu, cur.zv, su, sv,
                                             d_xy, d_xz, d_yx, d_yz, d_zx, d_zy, px, py, pz);
                ax2.psi[1][fz.side][0][ip] = su;
                ax2.psi[1][fz.side][1][ip] = sv;
            }
            // update_h.cl:129-131
            nx = dv<ST>(cur.hx, xe(cur.gh, 0)) - dt * ((d_zy - d_yz) - px);
            ny = dv<ST>(cur.hy, xe(cur.gh, 1)) - dt * ((d_xz - d_zx) - py);
            nz = dv<ST>(cur.hz, xe(cur.gh, 2)) - dt * ((d_yx - d_xy) - pz);
        }
        int e0 = 0, e1 = 0, e2 = 0;
        if (SS::scaled) {
            warp_exps(nx, ny, nz, e0, e1, e2);
            if ((threadIdx.x & 31u) == 0 && jt < v.ntl) hexp[texp_index(v, x, jt)] = xpack(e0, e1, e2);
        }
        if (act) {
            Hx[i] = SS::enc(SS::scaled ? nx * pow2(-e0) : nx);
            Hy[i] = SS::enc(SS::scaled ? ny * pow2(-e1) : ny);
            Hz[i] = SS::enc(SS::scaled ? nz * pow2(-e2) : nz);
            ex = ex1;
            ey = ey1;
            ez = ez1;
            if (PF) cur = nxt;
        }
    }
}

template <int ST, bool PF>
__device__ __forceinline__ void batch_e_item(const BatchK &k, uint32_t ti, int64_t step)
{
    const int4 tl = k.tiles[ti];
    batch_e_tile<ST, PF>(k.vars[tl.x], tl, step, k.rows);
}

template <int ST, bool PF>
__device__ __forceinline__ void batch_h_item(const BatchK &k, uint32_t ti)
{
    const int4 tl = k.tiles[ti];
    batch_h_tile<ST, PF>(k.vars[tl.x], tl);
}

// next tile of the half-step whose counter is `ctr` (>= ntiles: none left)
__device__ __forceinline__ uint32_t next_tile(uint32_t *ctr, uint32_t *slot)
{
    __syncthreads();                                     // every thread has read the last one
    if (threadIdx.x == 0) *slot = atomicAdd(ctr, 1u);
    __syncthreads();
    return *slot;
}

// Persistent form: without the register prefetch (PF false) the E and H tile bodies together
// fit BATCH_PERSIST_BLOCKS resident blocks per SM (64 registers), whose warps hide the load
// latency; with it they need 128 registers and two blocks per SM, 1.3x slower.
constexpr int BATCH_PERSIST_BLOCKS = 4;

template <int ST>
__global__ void __launch_bounds__(BATCH_THREADS, BATCH_PERSIST_BLOCKS) k_batch(const BatchK k)
{
    __shared__ uint32_t item;
    cg::grid_group grid = cg::this_grid();
    const int64_t step0 = *k.step;
    for (int t = 0; t < k.nsteps; ++t) {
        const int64_t step = step0 + t;
        // half-step 2t uses counter 0, 2t + 1 counter 1; a counter is cleared right after the
        // grid barrier that ends its half-step, two barriers before its next use
        for (uint32_t ti = next_tile(&k.work[0], &item); ti < k.ntiles; ti = next_tile(&k.work[0], &item))
            batch_e_item<ST, false>(k, ti, step);
        grid.sync();
        if (blockIdx.x == 0 && threadIdx.x == 0) k.work[0] = 0u;
        for (uint32_t ti = next_tile(&k.work[1], &item); ti < k.ntiles; ti = next_tile(&k.work[1], &item))
            batch_h_item<ST, false>(k, ti);
        grid.sync();
        if (blockIdx.x == 0 && threadIdx.x == 0) k.work[1] = 0u;
    }
    // every block read the step counter before its first grid barrier
    if (blockIdx.x == 0 && threadIdx.x == 0) *k.step = step0 + k.nsteps;
}

// One tile per block, all variants' tiles in one launch per half-step: three blocks per SM,
// each warp with two planes of loads in flight (the register prefetch), about 1.5x the loads
// in flight of the persistent form. The H launch advances the step counter.
template <int ST>
__global__ void __launch_bounds__(BATCH_THREADS, 3) k_batch_e(const BatchK k)
{
    const int4 tl = k.tiles[blockIdx.x];
    batch_e_tile<ST>(k.vars[tl.x], tl, *k.step, k.rows);
}

template <int ST>
__global__ void __launch_bounds__(BATCH_THREADS, 3) k_batch_h(const BatchK k)
{
    const int4 tl = k.tiles[blockIdx.x];
    batch_h_tile<ST>(k.vars[tl.x], tl);
    // the E launch of this step, which reads the counter, has completed
    if (blockIdx.x == 0 && threadIdx.x == 0) *k.step += 1;
}

// one block per (column jb of BATCH_THREADS cells, plane x): float32 <-> storage, all three
// components of a cell per thread, one exponent word per warp tile
template <int ST>
__global__ void __launch_bounds__(BATCH_THREADS) k_batch_encode(const BVar v, int field, const float *src)
{
    using SS = Store<ST>;
    using T = typename SS::T;
    const uint32_t jb = blockIdx.x, x = blockIdx.y;
    const uint32_t j = jb * BATCH_THREADS + threadIdx.x;
    const bool act = j < v.syz;
    const uint64_t i = (uint64_t)x * v.syz + j;
    float val[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) val[c] = act ? src[(uint64_t)c * v.N + i] : 0.f;
    int e[3] = {0, 0, 0};
    if (SS::scaled) warp_exps(val[0], val[1], val[2], e[0], e[1], e[2]);
    T *dst = (T *)(field ? v.H : v.E);
    if (act) {
#pragma unroll
        for (int c = 0; c < 3; ++c) dst[(uint64_t)c * v.N + i] = SS::enc(SS::scaled ? val[c] * pow2(-e[c]) : val[c]);
    }
    const uint32_t jt = j / BATCH_TILE;
    if (SS::scaled && (threadIdx.x & 31u) == 0 && jt < v.ntl)
        (field ? v.hexp : v.eexp)[texp_index(v, x, jt)] = xpack(e[0], e[1], e[2]);
}

template <int ST>
__global__ void __launch_bounds__(BATCH_THREADS) k_batch_decode(const BVar v, int field, float *dst)
{
    using SS = Store<ST>;
    using T = typename SS::T;
    const uint32_t jb = blockIdx.x, x = blockIdx.y;
    const uint32_t j = jb * BATCH_THREADS + threadIdx.x;
    if (j >= v.syz) return;
    const uint64_t i = (uint64_t)x * v.syz + j;
    const T *src = (const T *)(field ? v.H : v.E);
    const int32_t w = SS::scaled ? (field ? v.hexp : v.eexp)[texp_index(v, x, j / BATCH_TILE)] : 0;
#pragma unroll
    for (int c = 0; c < 3; ++c) dst[(uint64_t)c * v.N + i] = dv<ST>(src[(uint64_t)c * v.N + i], xe(w, c));
}

}  // namespace

template <int ST>
int batch_max_blocks_per_sm()
{
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_batch<ST>, BATCH_THREADS, 0) != cudaSuccess) return 0;
    return n;
}

template <int ST>
cudaError_t launch_batch(const BatchK &k, int blocks, cudaStream_t st)
{
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)blocks, 1, 1);
    cfg.blockDim = dim3(BATCH_THREADS, 1, 1);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, k_batch<ST>, k);
}

template <int ST>
cudaError_t launch_batch_steps(const BatchK &k, cudaStream_t st)
{
    for (int t = 0; t < k.nsteps; ++t) {
        k_batch_e<ST><<<k.ntiles, BATCH_THREADS, 0, st>>>(k);
        k_batch_h<ST><<<k.ntiles, BATCH_THREADS, 0, st>>>(k);
    }
    return cudaGetLastError();
}

cudaError_t launch_batch_encode(int store, const BVar &v, int field, const float *src, cudaStream_t st)
{
    const dim3 g(v.njb, v.sx, 1);
    if (store == BATCH_BF16) k_batch_encode<BATCH_BF16><<<g, BATCH_THREADS, 0, st>>>(v, field, src);
    else if (store == BATCH_F16) k_batch_encode<BATCH_F16><<<g, BATCH_THREADS, 0, st>>>(v, field, src);
    else if (store == BATCH_BF16U) k_batch_encode<BATCH_BF16U><<<g, BATCH_THREADS, 0, st>>>(v, field, src);
    else return cudaErrorInvalidValue;
    return cudaGetLastError();
}

cudaError_t launch_batch_decode(int store, const BVar &v, int field, float *dst, cudaStream_t st)
{
    const dim3 g(v.njb, v.sx, 1);
    if (store == BATCH_BF16) k_batch_decode<BATCH_BF16><<<g, BATCH_THREADS, 0, st>>>(v, field, dst);
    else if (store == BATCH_F16) k_batch_decode<BATCH_F16><<<g, BATCH_THREADS, 0, st>>>(v, field, dst);
    else if (store == BATCH_BF16U) k_batch_decode<BATCH_BF16U><<<g, BATCH_THREADS, 0, st>>>(v, field, dst);
    else return cudaErrorInvalidValue;
    return cudaGetLastError();
}

template cudaError_t launch_batch<BATCH_F32>(const BatchK &, int, cudaStream_t);
template cudaError_t launch_batch<BATCH_BF16>(const BatchK &, int, cudaStream_t);
template cudaError_t launch_batch<BATCH_F16>(const BatchK &, int, cudaStream_t);
template cudaError_t launch_batch_steps<BATCH_F32>(const BatchK &, cudaStream_t);
template cudaError_t launch_batch_steps<BATCH_BF16>(const BatchK &, cudaStream_t);
template cudaError_t launch_batch_steps<BATCH_F16>(const BatchK &, cudaStream_t);
template int batch_max_blocks_per_sm<BATCH_F32>();
template int batch_max_blocks_per_sm<BATCH_BF16>();
template int batch_max_blocks_per_sm<BATCH_F16>();
template cudaError_t launch_batch<BATCH_BF16U>(const BatchK &, int, cudaStream_t);
template cudaError_t launch_batch_steps<BATCH_BF16U>(const BatchK &, cudaStream_t);
template int batch_max_blocks_per_sm<BATCH_BF16U>();

}  // namespace fdtd
