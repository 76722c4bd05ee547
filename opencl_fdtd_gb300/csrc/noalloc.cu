// fdtd_plane_sum_noalloc: the FP64 plane sum of fdtd_plane_sum without any device allocation.
//
// Who needs it: programs that drive the simulation from a time-stepping loop that must not
// allocate device memory, e.g. a C or Fortran host code that has given the device's memory
// to its own pool (a cudaMalloc there fails or fragments that pool), or a monitoring callback
// between queued steps, where cudaMalloc / cudaFree may synchronize the device and stall the
// work already queued. fdtd_plane_sum needs a caller-provided scratch array for its
// per-block partial sums; this variant keeps them in a static device array of this library
// instead, so the caller passes only the field and the output.
//
// The array holds at most NOALLOC_MAX_PARTIALS doubles (8 KB), allocated with the module on
// every GPU that loads the library and held until the process exits. Every call writes the
// nblocks partials it then reads, so nothing needs clearing between calls; the array keeps
// the last call's partials. Calls share the array: two calls whose kernels overlap on the GPU
// (different streams without ordering) race on it.
#include <cstdint>
#include <mutex>
#include <string>

#include "fdtd_gb300.h"
#include "fdtd_plan.h"
#include "monitors.h"

namespace {

constexpr int NOALLOC_MAX_PARTIALS = 1024;

// per-block partial sums of every fdtd_plane_sum_noalloc call on this device
static __device__ __align__(256) double g_plane_partials[NOALLOC_MAX_PARTIALS];

// device address of g_plane_partials per device, resolved on the first call on that device
constexpr int MAX_DEVICES = 64;
std::mutex g_addr_mutex;
double *g_addr[MAX_DEVICES] = {};

int partials_address(double **out)
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess)
        return fdtd::set_error(FDTD_ERR_CUDA, (std::string("cudaGetDevice: ") + cudaGetErrorString(e)).c_str());
    std::lock_guard<std::mutex> lock(g_addr_mutex);
    if (dev >= 0 && dev < MAX_DEVICES && g_addr[dev]) {
        *out = g_addr[dev];
        return FDTD_OK;
    }
    void *ptr = nullptr;
    e = cudaGetSymbolAddress(&ptr, g_plane_partials);
    if (e != cudaSuccess || !ptr)
        return fdtd::set_error(FDTD_ERR_CUDA, (std::string("cudaGetSymbolAddress(plane partials): ") +
                                               cudaGetErrorString(e)).c_str());
    if (dev >= 0 && dev < MAX_DEVICES) g_addr[dev] = (double *)ptr;
    *out = (double *)ptr;
    return FDTD_OK;
}

template <typename R>
int plane_sum_static(const FdtdPlan *p, const void *field, int comp, int axis, int64_t plane,
                     double *partials, int nblocks, double *out, cudaStream_t st)
{
    const fdtd::PlaneRedK<R> k =
        fdtd::plane_red_args<R>(field, comp, axis, plane, p->sx, p->sy, p->sz, partials);
    return fdtd::check_cuda(fdtd::launch_plane_sum<R>(k, nblocks, out, st), "plane sum (no-alloc) launch");
}

}  // namespace

extern "C" int fdtd_plane_sum_noalloc(FdtdPlan *p, const void *field, int32_t component,
                                      int32_t axis, int64_t plane, int32_t nblocks, double *out,
                                      void *stream)
{
    if (!p) return fdtd::set_error(FDTD_ERR_INVALID, "plan is NULL");
    if (!field || !out) return fdtd::set_error(FDTD_ERR_INVALID, "plane sum (no-alloc): NULL pointer");
    if (component < 0 || component > 2 || axis < 0 || axis > 2)
        return fdtd::set_error(FDTD_ERR_INVALID, "plane sum (no-alloc): component and axis must be 0..2");
    const int64_t s = axis == 0 ? p->sx : axis == 1 ? p->sy : p->sz;
    if (plane < 0 || plane >= s)
        return fdtd::set_error(FDTD_ERR_INVALID, "plane sum (no-alloc): plane index out of range");
    if (nblocks < 1 || nblocks > NOALLOC_MAX_PARTIALS)
        return fdtd::set_error(FDTD_ERR_INVALID,
                               "plane sum (no-alloc): nblocks must be in [1, 1024], the size of the "
                               "static partial-sum array");
    double *partials = nullptr;
    int rc = partials_address(&partials);
    if (rc) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    return p->d.dtype == FDTD_F64
               ? plane_sum_static<double>(p, field, component, axis, plane, partials, nblocks, out, st)
               : plane_sum_static<float>(p, field, component, axis, plane, partials, nblocks, out, st);
}
