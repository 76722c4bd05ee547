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

template <typename R>
struct PlaneRedK {
    const R *src;            // one component of a field
    double *partial;         // per-block partial sums
    uint64_t ncell, inner, base, stride_a, stride_b;
};

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
