/*
 * TEST INFRASTRUCTURE — the oracle for the FDTD time-stepping path.
 *
 * A plain-C restatement of opencl_fdtd's kernels (opencl_fdtd/kernels/*.cl), compiled with
 * gcc -O3 -fopenmp -ffp-contract=off into oracle/_build/libfdtd_port.so. Only tests/,
 * __graft_entry__.smoke() and bench.py's CPU-baseline leg load it; the product path never does.
 */
#include <stdint.h>

/* Grid, spacing, PML and Bloch description shared by both precisions. */
typedef struct PortDesc {
    int64_t sx, sy, sz;
    double dt;
    int32_t uniform;            /* 1: uniform spacing dx */
    double dx;
    const void *inv_de[3];      /* non-uniform: 1/dx tables on the E grid (used by H updates) */
    const void *inv_dh[3];      /* non-uniform: 1/dx tables on the H grid (used by E updates) */
    int32_t npml;
    int32_t axis[6], pol[6];    /* axis 0..2; polarity 0 = 'n', 1 = 'p' */
    int64_t thick[6];
    const void *pe[6][3];       /* p0, p1, p2 for the E update of each face */
    const void *ph[6][3];       /* p0, p1, p2 for the H update of each face */
    int32_t nbloch;
    int32_t baxis[3];
    double bre[3], bim[3];
    int32_t nthreads;
} PortDesc;

/* Depth index into a face's coefficient tables, or -1 when the cell is outside the slab
 * (update_e.cl:81-90; a 'p' face thicker than the axis never applies there, because the
 * reference's unsigned s - T wraps). */
static inline int64_t port_pml_ir(int pol, int64_t T, int64_t s, int64_t c)
{
    if (pol == 0) return (c < T) ? c : -1;
    if (T <= s && c >= s - T) return (s - 1) - c;
    return -1;
}

#define REAL float
#define SFX f32
#include "fdtd_port_body.h"
#undef REAL
#undef SFX

#define REAL double
#define SFX f64
#include "fdtd_port_body.h"
#undef REAL
#undef SFX

int port_abi_version(void) { return 1; }
