// Arguments and launchers of the FP64 monitor kernels (monitors.cu).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace fdtd {

constexpr int RED_THREADS = 256;

template <typename R>
struct DftK {
    const R *field;          // 3N field the points index into
    const int64_t *index;    // device, npoint flat indices
    const double *omega;     // device, nfreq angular frequencies
    double *accum;           // device, [npoint][nfreq][re, im]
    double *series;          // device or NULL, [rows][npoint]
    int32_t npoint, nfreq;
    int64_t step;            // the sample is taken at time (step + 1) * dt
    int64_t series_row;
    double dt;
};

// Sample q = point * nfreq + f of a DFT monitor: adds x(t) * exp(-i w t dt) in double to the
// point's accumulator and stores x(t) in the time series (f == 0). One body for the monitor's
// own kernel (monitors.cu) and the H+S kernel's in-launch sample (hs_fused.cu); both units are
// compiled without FMA contraction, so the two give the same bits.
template <typename R>
__device__ __forceinline__ void dft_sample(const DftK<R> &k, int q)
{
    const int nf = k.nfreq > 0 ? k.nfreq : 1;
    const int p = q / nf, f = q - p * nf;
    const double v = (double)k.field[k.index[p]];
    if (k.nfreq > 0) {
        const double ph = k.omega[f] * ((double)(k.step + 1) * k.dt);
        double s, c;
        sincos(ph, &s, &c);
        double *a = k.accum + 2 * (int64_t)q;
        a[0] += v * c;
        a[1] -= v * s;
    }
    if (f == 0 && k.series) k.series[(int64_t)k.series_row * k.npoint + p] = v;
}

template <typename R>
struct PlaneRedK {
    const R *src;            // one component of a field
    double *partial;         // per-block partial sums
    uint64_t ncell, inner, base, stride_a, stride_b;
};

// Arguments of the plane sum of component ``comp`` of a 3N field over the plane ``plane``
// normal to ``axis`` on an (sx, sy, sz) grid; the one mapping both plane-sum entry points use.
template <typename R>
inline PlaneRedK<R> plane_red_args(const void *field, int comp, int axis, int64_t plane,
                                   uint64_t sx, uint64_t sy, uint64_t sz, double *partial)
{
    PlaneRedK<R> k;
    const uint64_t syz = sy * sz;
    k.src = (const R *)field + (uint64_t)comp * sx * syz;
    k.partial = partial;
    if (axis == 0) { k.base = plane * syz; k.stride_a = sz; k.stride_b = 1; k.inner = sz; k.ncell = syz; }
    else if (axis == 1) { k.base = plane * sz; k.stride_a = syz; k.stride_b = 1; k.inner = sz; k.ncell = sx * sz; }
    else { k.base = plane; k.stride_a = syz; k.stride_b = sz; k.inner = sy; k.ncell = sx * sy; }
    return k;
}

template <typename R>
struct EnergyK {
    const R *E, *H, *eps, *mu;
    double *partial;
    uint64_t n;              // 3N
};

template <typename R> cudaError_t launch_dft(const DftK<R> &k, cudaStream_t st);
template <typename R>
cudaError_t launch_plane_sum(const PlaneRedK<R> &k, int nblocks, double *out, cudaStream_t st);
template <typename R>
cudaError_t launch_energy(const EnergyK<R> &k, int nblocks, double *out, cudaStream_t st);
// adds the number of NaN / Inf values among a[0 .. n) to *count (device)
template <typename R>
cudaError_t launch_count_nonfinite(const R *a, uint64_t n, unsigned int *count, cudaStream_t st);

}  // namespace fdtd
