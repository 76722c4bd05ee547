// FP64 monitors of a running simulation: DFT point monitors, Poynting-flux plane integrals
// and the total field energy.
//
// The reference itself only saves the final fields (opencl_fdtd fdtd.py:181-191); its
// driver's purpose is a cavity ringdown (fdtd.py:84-179), whose analysis needs the field at a
// few points over thousands of steps and energy / flux balances. Accumulating those in the
// field dtype (float32) loses the small late-time ringdown signal, so everything here
// accumulates in double:
//   * k_dft: one thread per (point, frequency) adds x(t) * exp(-i w t dt) in double each step
//     and optionally stores x(t) in a time-series buffer;
//   * k_reduce_*: deterministic two-stage reductions (fixed grid, fixed order) of an S
//     component over one plane, or of 1/2 (eps E^2 + mu H^2) over the grid, into a caller
//     scratch array of per-block partial sums, then one block folds the partials.
#include <cstdint>
#include <cuda_runtime.h>

#include "monitors.h"

namespace fdtd {

template <typename R>
__global__ void k_dft(const DftK<R> k)
{
    const int nf = k.nfreq > 0 ? k.nfreq : 1;
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= k.npoint * nf) return;
    dft_sample(k, q);
}

// stage 1: block b sums cells b, b + G, b + 2G ... of the selection (G = grid size) in a
// fixed order, then folds the block in a fixed tree
template <typename R>
__global__ void __launch_bounds__(RED_THREADS) k_reduce_plane(const PlaneRedK<R> k)
{
    __shared__ double sh[RED_THREADS];
    double acc = 0.0;
    for (uint64_t c = (uint64_t)blockIdx.x * RED_THREADS + threadIdx.x; c < k.ncell;
         c += (uint64_t)gridDim.x * RED_THREADS) {
        // plane cell c -> flat index
        const uint64_t a = c / k.inner, b = c - a * k.inner;
        const uint64_t i = k.base + a * k.stride_a + b * k.stride_b;
        acc += (double)k.src[i];
    }
    sh[threadIdx.x] = acc;
    __syncthreads();
    for (int s = RED_THREADS / 2; s > 0; s >>= 1) {
        if ((int)threadIdx.x < s) sh[threadIdx.x] += sh[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) k.partial[blockIdx.x] = sh[0];
}

template <typename R>
__global__ void __launch_bounds__(RED_THREADS) k_reduce_energy(const EnergyK<R> k)
{
    __shared__ double sh[RED_THREADS];
    double acc = 0.0;
    for (uint64_t i = (uint64_t)blockIdx.x * RED_THREADS + threadIdx.x; i < k.n;
         i += (uint64_t)gridDim.x * RED_THREADS) {
        const double e = (double)k.E[i], h = (double)k.H[i];
        const double eps = (double)k.eps[i];
        const double mu = k.mu ? (double)k.mu[i] : 1.0;
        // a perfect conductor (eps = inf) holds E = 0 and no energy
        if (e != 0.0 && !isinf(eps)) acc += eps * e * e;
        acc += mu * h * h;
    }
    sh[threadIdx.x] = acc;
    __syncthreads();
    for (int s = RED_THREADS / 2; s > 0; s >>= 1) {
        if ((int)threadIdx.x < s) sh[threadIdx.x] += sh[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) k.partial[blockIdx.x] = 0.5 * sh[0];
}

// stage 2: one block folds n partials in a fixed order
__global__ void __launch_bounds__(RED_THREADS) k_fold(const double *partial, int n, double *out)
{
    __shared__ double sh[RED_THREADS];
    double acc = 0.0;
    for (int i = threadIdx.x; i < n; i += RED_THREADS) acc += partial[i];
    sh[threadIdx.x] = acc;
    __syncthreads();
    for (int s = RED_THREADS / 2; s > 0; s >>= 1) {
        if ((int)threadIdx.x < s) sh[threadIdx.x] += sh[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) *out = sh[0];
}

template <typename R>
cudaError_t launch_dft(const DftK<R> &k, cudaStream_t st)
{
    const int n = k.npoint * (k.nfreq > 0 ? k.nfreq : 1);
    if (n <= 0) return cudaSuccess;
    k_dft<R><<<(n + 127) / 128, 128, 0, st>>>(k);
    return cudaGetLastError();
}

template <typename R>
cudaError_t launch_plane_sum(const PlaneRedK<R> &k, int nblocks, double *out, cudaStream_t st)
{
    k_reduce_plane<R><<<nblocks, RED_THREADS, 0, st>>>(k);
    k_fold<<<1, RED_THREADS, 0, st>>>(k.partial, nblocks, out);
    return cudaGetLastError();
}

template <typename R>
cudaError_t launch_energy(const EnergyK<R> &k, int nblocks, double *out, cudaStream_t st)
{
    k_reduce_energy<R><<<nblocks, RED_THREADS, 0, st>>>(k);
    k_fold<<<1, RED_THREADS, 0, st>>>(k.partial, nblocks, out);
    return cudaGetLastError();
}

// field watchdog: every thread counts the non-finite values of its grid-stride slice, the warp
// sums its lanes' counts, one atomic per warp that found any
template <typename R>
__global__ void __launch_bounds__(RED_THREADS) k_count_nonfinite(const R *a, uint64_t n, unsigned int *count)
{
    unsigned int local = 0;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
        local += isfinite(a[i]) ? 0u : 1u;
    local = __reduce_add_sync(0xffffffffu, local);
    if ((threadIdx.x & 31u) == 0 && local) atomicAdd(count, local);
}

template <typename R>
cudaError_t launch_count_nonfinite(const R *a, uint64_t n, unsigned int *count, cudaStream_t st)
{
    if (!n) return cudaSuccess;
    const uint64_t want = (n + RED_THREADS - 1) / RED_THREADS;
    const int blocks = (int)(want < 2048 ? want : 2048);
    k_count_nonfinite<R><<<blocks, RED_THREADS, 0, st>>>(a, n, count);
    return cudaGetLastError();
}

template cudaError_t launch_count_nonfinite<float>(const float *, uint64_t, unsigned int *, cudaStream_t);
template cudaError_t launch_count_nonfinite<double>(const double *, uint64_t, unsigned int *, cudaStream_t);
template cudaError_t launch_dft<float>(const DftK<float> &, cudaStream_t);
template cudaError_t launch_dft<double>(const DftK<double> &, cudaStream_t);
template cudaError_t launch_plane_sum<float>(const PlaneRedK<float> &, int, double *, cudaStream_t);
template cudaError_t launch_plane_sum<double>(const PlaneRedK<double> &, int, double *, cudaStream_t);
template cudaError_t launch_energy<float>(const EnergyK<float> &, int, double *, cudaStream_t);
template cudaError_t launch_energy<double>(const EnergyK<double> &, int, double *, cudaStream_t);

}  // namespace fdtd
