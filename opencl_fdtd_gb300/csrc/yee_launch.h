// Host-side launchers of the Yee kernels (defined in yee_kernels.cu).
#pragma once

#include "yee_common.cuh"

namespace fdtd {

// pdl: the bulk E kernel is launched with programmatic stream serialization (fdtd_run's H+S path)
template <typename R> cudaError_t launch_yee_e(const YeeK<R> &k, cudaStream_t st, bool pdl = false);
template <typename R> cudaError_t launch_yee_h(const YeeK<R> &k, bool mu, bool poynting, cudaStream_t st);
template <typename R> cudaError_t launch_poynting(const SK<R> &k, cudaStream_t st);
template <typename R> cudaError_t launch_prepare(const PrepK<R> &k, cudaStream_t st);
template <typename R> cudaError_t launch_fieldsrc(const JK<R> &k, cudaStream_t st);
template <typename R> cudaError_t launch_point_sources(const PointK<R> &k, cudaStream_t st);

}  // namespace fdtd
