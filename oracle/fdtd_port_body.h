/*
 * CPU restatement of opencl_fdtd's Yee time-stepping kernels (TEST INFRASTRUCTURE).
 *
 * This file is the oracle: it exists only to check the CUDA product path. It is included
 * twice by fdtd_port.c, once with REAL=float (SFX=f32) and once with REAL=double (SFX=f64).
 * Nothing under opencl_fdtd_gb300/ may include, link or call it.
 *
 * Every per-cell expression keeps the reference's operation order so that, compiled with
 * -ffp-contract=off, the float instance reproduces the reference kernel text bit for bit:
 *
 *   index decode / periodic wrap ........ opencl_fdtd/kernels/common.cl:34-42, 75-85
 *   E curl + update ..................... opencl_fdtd/kernels/update_e.cl:25-46, 64-107
 *   H curl + update + Poynting products . opencl_fdtd/kernels/update_h.cl:25-43, 57-155
 *   Poynting assemble ................... opencl_fdtd/kernels/update_s.cl:21-36
 *   field (current) source .............. opencl_fdtd/kernels/update_j.cl:15-32
 *
 * Two extensions the reference lacks are restated from the physics, not from code:
 *   - diagonal mu in the H update (the reference has none, update_h.cl:129-131): the update
 *     becomes H -= (dt/mu) * (curl E - psi), the mirror of update_e.cl:105-107;
 *   - Bloch-phase coupling of split complex fields (the reference's template code for it is
 *     never rendered, simulation.py:206 vs update_e.cl:48): with beta = real + i*imag the
 *     phase across one period, the E-type update reads its wrapped minus-neighbour as
 *     (Q + iR)(s-1) * conj(beta) and the H-type update reads its wrapped plus-neighbour as
 *     (Q + iR)(0) * beta, taking the real or imaginary part as the updated field requires.
 *
 * PML psi arrays use the reference's layout, ip = v + u*s_v + ir*s_v*s_u
 * (update_e.cl:92), with ir the depth counted from the outer face.
 */

#define PCAT_(a, b) a##_##b
#define PCAT(a, b) PCAT_(a, b)
#define PFN(name) PCAT(name, SFX)

/* Per-axis inverse spacing at coordinate c: uniform (REAL)(1.0/dx) (update_e.cl:26-28), else
 * the table value (update_e.cl:30-32 for E, update_h.cl:30-32 for H). */
static inline REAL PFN(port_inv)(const PortDesc *d, const void *const *tab, int r, int64_t c)
{
    if (d->uniform) return (REAL)(1.0 / d->dx);
    return ((const REAL *)tab[r])[c];
}

/*
 * E-type update (update_e.cl): P += dt/eps * (curl Q + psi).
 * P/Q = (E, H) for the real part, (F, G) for the imaginary part of a Bloch pair;
 * R is the other half of Q's complex pair (NULL when there are no Bloch boundaries).
 * imag_part selects the sign of the coupling term (see the header).
 * psi holds 2 arrays per PML face, in the order of d->axis[]: [face0_u, face0_v, face1_u, ...].
 */
void PFN(port_update_e)(const PortDesc *d, REAL *P, const REAL *Q, const REAL *R,
                        int imag_part, const REAL *eps, REAL *const *psi)
{
    const int64_t sx = d->sx, sy = d->sy, sz = d->sz;
    const int64_t N = sx * sy * sz;
    const int64_t st[3] = {sy * sz, sz, 1};
    const int64_t sh[3] = {sx, sy, sz};
    const REAL dt = (REAL)d->dt;
    REAL br[3] = {1, 1, 1}, bi[3] = {0, 0, 0};
    int bl[3] = {0, 0, 0};
    for (int b = 0; b < d->nbloch; ++b) {
        int a = d->baxis[b];
        bl[a] = (R != 0);
        br[a] = (REAL)d->bre[b];
        bi[a] = (REAL)(imag_part ? -d->bim[b] : d->bim[b]);
    }

#pragma omp parallel for schedule(static) num_threads(d->nthreads > 0 ? d->nthreads : 1)
    for (int64_t x = 0; x < sx; ++x)
        for (int64_t y = 0; y < sy; ++y)
            for (int64_t z = 0; z < sz; ++z) {
                const int64_t i = (x * sy + y) * sz + z;
                const int64_t c[3] = {x, y, z};
                REAL inv[3];
                for (int r = 0; r < 3; ++r) inv[r] = PFN(port_inv)(d, d->inv_dh, r, c[r]);

                /* dQ[q][r]: backward difference of component q along axis r (update_e.cl:39-46) */
                REAL dQ[3][3] = {{0}};
                for (int q = 0; q < 3; ++q)
                    for (int r = 0; r < 3; ++r) {
                        if (q == r) continue;
                        REAL nb;
                        if (c[r] == 0) {
                            const int64_t j = i + (sh[r] - 1) * st[r];   /* common.cl:79-81 */
                            if (bl[r])
                                nb = Q[q * N + j] * br[r] + R[q * N + j] * bi[r];
                            else
                                nb = Q[q * N + j];
                        } else {
                            nb = Q[q * N + i - st[r]];
                        }
                        dQ[q][r] = (Q[q * N + i] - nb) * inv[r];
                    }

                /* CPML (update_e.cl:64-100), faces in list order */
                REAL pE[3] = {0, 0, 0};
                for (int f = 0; f < d->npml; ++f) {
                    const int r = d->axis[f];
                    const int u = (r == 0) ? 1 : 0;
                    const int v = (r == 2) ? 1 : 2;
                    const int64_t ir = port_pml_ir(d->pol[f], d->thick[f], sh[r], c[r]);
                    if (ir < 0) continue;
                    const REAL p0 = ((const REAL *)d->pe[f][0])[ir];
                    const REAL p1 = ((const REAL *)d->pe[f][1])[ir];
                    const REAL p2 = ((const REAL *)d->pe[f][2])[ir];
                    const int64_t ip = c[v] + c[u] * sh[v] + ir * sh[v] * sh[u];
                    REAL *pu = psi[2 * f], *pv = psi[2 * f + 1];
                    dQ[v][r] *= p2;
                    dQ[u][r] *= p2;
                    pu[ip] = p0 * pu[ip] + p1 * dQ[v][r];
                    pv[ip] = p0 * pv[ip] + p1 * dQ[u][r];
                    if (r != 1) { pE[u] -= pu[ip]; pE[v] += pv[ip]; }
                    else        { pE[u] += pu[ip]; pE[v] -= pv[ip]; }
                }

                /* update_e.cl:105-107 */
                P[0 * N + i] += dt / eps[0 * N + i] * (dQ[2][1] - dQ[1][2] + pE[0]);
                P[1 * N + i] += dt / eps[1 * N + i] * (dQ[0][2] - dQ[2][0] + pE[1]);
                P[2 * N + i] += dt / eps[2 * N + i] * (dQ[1][0] - dQ[0][1] + pE[2]);
            }
}

/*
 * H-type update (update_h.cl): P -= dt * (curl Q - psi), or (dt/mu) * (...) when mu != NULL.
 * When oS != NULL the six Poynting products are written to oS (update_h.cl:57-71, 121-155).
 */
void PFN(port_update_h)(const PortDesc *d, REAL *P, const REAL *Q, const REAL *R,
                        int imag_part, const REAL *mu, REAL *const *psi, REAL *oS)
{
    const int64_t sx = d->sx, sy = d->sy, sz = d->sz;
    const int64_t N = sx * sy * sz;
    const int64_t st[3] = {sy * sz, sz, 1};
    const int64_t sh[3] = {sx, sy, sz};
    const REAL dt = (REAL)d->dt;
    REAL br[3] = {1, 1, 1}, bi[3] = {0, 0, 0};
    int bl[3] = {0, 0, 0};
    for (int b = 0; b < d->nbloch; ++b) {
        int a = d->baxis[b];
        bl[a] = (R != 0);
        br[a] = (REAL)d->bre[b];
        bi[a] = (REAL)(imag_part ? d->bim[b] : -d->bim[b]);
    }

#pragma omp parallel for schedule(static) num_threads(d->nthreads > 0 ? d->nthreads : 1)
    for (int64_t x = 0; x < sx; ++x)
        for (int64_t y = 0; y < sy; ++y)
            for (int64_t z = 0; z < sz; ++z) {
                const int64_t i = (x * sy + y) * sz + z;
                const int64_t c[3] = {x, y, z};
                REAL inv[3];
                for (int r = 0; r < 3; ++r) inv[r] = PFN(port_inv)(d, d->inv_de, r, c[r]);

                /* dQ[q][r]: forward difference (update_h.cl:36-43); aE[q][r]: sum of the pair
                 * (update_h.cl:63-70), which always uses the plain wrapped neighbour. */
                REAL dQ[3][3] = {{0}}, aE[3][3] = {{0}};
                for (int q = 0; q < 3; ++q)
                    for (int r = 0; r < 3; ++r) {
                        if (q == r) continue;
                        REAL nb, raw;
                        if (c[r] == sh[r] - 1) {
                            const int64_t j = i - (sh[r] - 1) * st[r];   /* common.cl:82-84 */
                            raw = Q[q * N + j];
                            if (bl[r])
                                nb = Q[q * N + j] * br[r] + R[q * N + j] * bi[r];
                            else
                                nb = raw;
                        } else {
                            raw = nb = Q[q * N + i + st[r]];
                        }
                        dQ[q][r] = (nb - Q[q * N + i]) * inv[r];
                        aE[q][r] = raw + Q[q * N + i];
                    }

                /* CPML (update_h.cl:80-116) */
                REAL pH[3] = {0, 0, 0};
                for (int f = 0; f < d->npml; ++f) {
                    const int r = d->axis[f];
                    const int u = (r == 0) ? 1 : 0;
                    const int v = (r == 2) ? 1 : 2;
                    const int64_t ir = port_pml_ir(d->pol[f], d->thick[f], sh[r], c[r]);
                    if (ir < 0) continue;
                    const REAL p0 = ((const REAL *)d->ph[f][0])[ir];
                    const REAL p1 = ((const REAL *)d->ph[f][1])[ir];
                    const REAL p2 = ((const REAL *)d->ph[f][2])[ir];
                    const int64_t ip = c[v] + c[u] * sh[v] + ir * sh[v] * sh[u];
                    REAL *pu = psi[2 * f], *pv = psi[2 * f + 1];
                    dQ[v][r] *= p2;
                    dQ[u][r] *= p2;
                    pu[ip] = p0 * pu[ip] + p1 * dQ[v][r];
                    pv[ip] = p0 * pv[ip] + p1 * dQ[u][r];
                    if (r != 1) { pH[u] += pu[ip]; pH[v] -= pv[ip]; }
                    else        { pH[u] -= pu[ip]; pH[v] += pv[ip]; }
                }

                const REAL old0 = P[0 * N + i], old1 = P[1 * N + i], old2 = P[2 * N + i];
                if (mu) {
                    P[0 * N + i] -= dt / mu[0 * N + i] * (dQ[2][1] - dQ[1][2] - pH[0]);
                    P[1 * N + i] -= dt / mu[1 * N + i] * (dQ[0][2] - dQ[2][0] - pH[1]);
                    P[2 * N + i] -= dt / mu[2 * N + i] * (dQ[1][0] - dQ[0][1] - pH[2]);
                } else {
                    /* update_h.cl:129-131 */
                    P[0 * N + i] -= dt * (dQ[2][1] - dQ[1][2] - pH[0]);
                    P[1 * N + i] -= dt * (dQ[0][2] - dQ[2][0] - pH[1]);
                    P[2 * N + i] -= dt * (dQ[1][0] - dQ[0][1] - pH[2]);
                }

                if (oS) {
                    const REAL aHx = P[0 * N + i] + old0;
                    const REAL aHy = P[1 * N + i] + old1;
                    const REAL aHz = P[2 * N + i] + old2;
                    /* plane order xy, yz, zx, xz, yx, zy (update_h.cl:142-154) */
                    oS[0 * N + i] = aE[1][0] * aHz;
                    oS[3 * N + i] = -aE[2][0] * aHy;
                    oS[1 * N + i] = aE[2][1] * aHx;
                    oS[4 * N + i] = -aE[0][1] * aHz;
                    oS[2 * N + i] = aE[0][2] * aHy;
                    oS[5 * N + i] = -aE[1][2] * aHx;
                }
            }
}

/* Poynting assemble (update_s.cl:33-36). */
void PFN(port_update_s)(const PortDesc *d, REAL *S, const REAL *oS)
{
    const int64_t sx = d->sx, sy = d->sy, sz = d->sz;
    const int64_t N = sx * sy * sz;
    const REAL dt = (REAL)d->dt;
    const REAL sf = (REAL)((double)dt * 0.125);
#pragma omp parallel for schedule(static) num_threads(d->nthreads > 0 ? d->nthreads : 1)
    for (int64_t x = 0; x < sx; ++x)
        for (int64_t y = 0; y < sy; ++y)
            for (int64_t z = 0; z < sz; ++z) {
                const int64_t i = (x * sy + y) * sz + z;
                const int64_t mx = (x == 0) ? (sx - 1) * sy * sz : -sy * sz;
                const int64_t my = (y == 0) ? (sy - 1) * sz : -sz;
                const int64_t mz = (z == 0) ? (sz - 1) : -1;
                const REAL *Sxy = oS, *Syz = oS + N, *Szx = oS + 2 * N;
                const REAL *Sxz = oS + 3 * N, *Syx = oS + 4 * N, *Szy = oS + 5 * N;
                S[0 * N + i] = (Sxy[i] + Sxz[i] + Sxy[i + my] + Sxz[i + mz]) * sf;
                S[1 * N + i] = (Syz[i] + Syx[i] + Syz[i + mz] + Syx[i + mx]) * sf;
                S[2 * N + i] = (Szx[i] + Szy[i] + Szx[i + mx] + Szy[i + my]) * sf;
            }
}

/* Field source (update_j.cl:23-32): E += c*Jr + s*Ji inside [min, max) on every axis. */
void PFN(port_update_j)(const PortDesc *d, REAL *E, const REAL *Jr, const REAL *Ji,
                        double cc, double ss, const int64_t *box)
{
    const int64_t sx = d->sx, sy = d->sy, sz = d->sz;
    const int64_t N = sx * sy * sz;
    const REAL c = (REAL)cc, s = (REAL)ss;
#pragma omp parallel for schedule(static) num_threads(d->nthreads > 0 ? d->nthreads : 1)
    for (int64_t x = 0; x < sx; ++x)
        for (int64_t y = 0; y < sy; ++y)
            for (int64_t z = 0; z < sz; ++z) {
                if (x < box[0] || y < box[2] || z < box[4]) continue;
                if (x >= box[1] || y >= box[3] || z >= box[5]) continue;
                const int64_t i = (x * sy + y) * sz + z;
                for (int q = 0; q < 3; ++q)
                    E[q * N + i] += c * Jr[q * N + i] + s * Ji[q * N + i];
            }
}

#undef PFN
#undef PCAT
#undef PCAT_
