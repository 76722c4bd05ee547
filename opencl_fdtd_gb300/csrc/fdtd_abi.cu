// C ABI of the FDTD library (include/fdtd_gb300.h): plans, validation and launch dispatch.
//
// A plan stands in for what opencl_fdtd's Simulation.__init__ bakes into its rendered kernel
// sources (opencl_fdtd/simulation.py:170-271): grid shape, dtype, spacing, the CPML face list
// with its coefficient tables (simulation.py:274-319), Bloch phases and the Poynting/field-
// source switches. The kernels are compiled once for every combination instead of being
// rendered per simulation; the plan only fills their argument blocks.
#include <cstdio>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "fdtd_gb300.h"
#include "yee_common.cuh"
#include "yee_launch.h"
#include "fdtd_plan.h"
#include "step.h"
#include "monitors.h"
#include "hs_fused.h"

using namespace fdtd;

namespace {

thread_local std::string g_err;

int fail(int code, const std::string &msg)
{
    g_err = msg;
    return code;
}

int cuda_fail(cudaError_t e, const char *what)
{
    g_err = std::string(what) + ": " + cudaGetErrorString(e);
    return FDTD_ERR_CUDA;
}

}  // namespace

namespace fdtd {

int set_error(int code, const char *msg)
{
    return fail(code, msg);
}

int check_cuda(cudaError_t e, const char *what)
{
    if (e == cudaSuccess) return FDTD_OK;
    return cuda_fail(e, what);
}

// True when no two CPML faces of one axis share a cell, so every cell sees at most one face
// per axis and the bulk kernels (which apply faces per axis) match the list order exactly.
bool faces_disjoint(const FdtdPlan *p)
{
    const uint32_t s[3] = {p->sx, p->sy, p->sz};
    uint32_t tn[3] = {0, 0, 0}, tp[3] = {0, 0, 0};
    for (int f = 0; f < p->d.n_pml; ++f) {
        const FdtdPmlDesc &pd = p->d.pml[f];
        const uint32_t T = (uint32_t)pd.thickness, a = (uint32_t)pd.axis;
        if (pd.polarity == 0) tn[a] = T;
        else if (T <= s[a]) tp[a] = T;
    }
    for (int r = 0; r < 3; ++r)
        if ((uint64_t)tn[r] + tp[r] > s[r]) return false;
    return true;
}

// Bloch factors as each update reads them (see cell_e / cell_h in yee_kernels.cu): E-type real part uses
// +imag, imaginary part -imag; H-type real part -imag, imaginary part +imag.
template <typename R>
YeeK<R> make_yee(const FdtdPlan *p, bool etype, bool imag, R *P, const R *Q, const R *Rp,
                 const R *mat, const R *coef, R *oS, void *const psi[6][2],
                 const void *const inv_tab[3])
{
    YeeK<R> k;
    std::memset(&k, 0, sizeof(k));
    k.P = P;
    k.Q = Q;
    k.Rp = Rp;
    k.mat = mat;
    k.coef = coef;
    k.oS = oS;
    k.dxmode = !p->d.uniform ? 2 : ((R)(1.0 / p->d.dx) == R(1) ? 0 : 1);
    const bool coef_ok = etype ? coef != nullptr : (mat == nullptr || coef != nullptr);
    k.bulk = coef_ok && faces_disjoint(p);
    k.xchunk = p->xchunk;
    k.eform = p->eform;
    k.dsz = FastDiv::make(p->sz);
    k.sx = p->sx;
    k.sy = p->sy;
    k.sz = p->sz;
    k.syz = p->syz;
    k.N = p->N;
    k.dt = (R)p->d.dt;
    k.inv_d = (R)(1.0 / p->d.dx);
    for (int r = 0; r < 3; ++r) k.inv_tab[r] = p->d.uniform ? nullptr : (const R *)inv_tab[r];
    k.nface = p->d.n_pml;
    for (int f = 0; f < p->d.n_pml; ++f) {
        const FdtdPmlDesc &pd = p->d.pml[f];
        FaceK<R> &fk = k.face[f];
        fk.axis = pd.axis;
        fk.pol = pd.polarity;
        fk.T = pd.thickness;
        const int base = etype ? 0 : 3;
        fk.p0 = (const R *)p->tab[f][base + 0];
        fk.p1 = (const R *)p->tab[f][base + 1];
        fk.p2 = (const R *)p->tab[f][base + 2];
        fk.psi_u = (R *)psi[f][0];
        fk.psi_v = (R *)psi[f][1];
        AxisK<R> &ak = k.ax[pd.axis];
        const uint32_t sa = pd.axis == 0 ? p->sx : pd.axis == 1 ? p->sy : p->sz;
        if (pd.polarity == 0) {
            ak.Tn = pd.thickness;
            ak.n0 = fk.p0; ak.n1 = fk.p1; ak.n2 = fk.p2;
            ak.nu = fk.psi_u; ak.nv = fk.psi_v;
        } else if ((uint32_t)pd.thickness <= sa) {
            ak.Tp = pd.thickness;
            ak.p0 = fk.p0; ak.p1 = fk.p1; ak.p2 = fk.p2;
            ak.pu = fk.psi_u; ak.pv = fk.psi_v;
        }
    }
    k.bloch_mask = 0;
    for (int r = 0; r < 3; ++r) {
        k.br[r] = R(1);
        k.bi[r] = R(0);
    }
    if (Rp) {
        for (int b = 0; b < p->d.n_bloch; ++b) {
            const FdtdBlochDesc &bd = p->d.bloch[b];
            k.bloch_mask |= 1 << bd.axis;
            k.br[bd.axis] = (R)bd.real;
            const bool plus = etype ? !imag : imag;
            k.bi[bd.axis] = (R)(plus ? bd.imag : -bd.imag);
        }
    }
    return k;
}

// With `src` (E only, all planes): the bulk kernel adds the step's point sources itself after
// the update, when there are at most YEE_SRC of them; *added tells the caller.
template <typename R>
int run_update_e(FdtdPlan *p, const FdtdBuffers *b, cudaStream_t st, bool imag,
                 uint32_t xbeg = 0, uint32_t xend = 0xffffffffu,
                 const FdtdPointSources *src = nullptr, int t = 0, bool *added = nullptr,
                 bool pdl = false)
{
    R *P = (R *)(imag ? b->F : b->E);
    const R *Q = (const R *)(imag ? b->G : b->H);
    const R *Rp = p->d.n_bloch ? (const R *)(imag ? b->H : b->G) : nullptr;
    void *const(*psi)[2] = imag ? b->psi_f : b->psi_e;
    YeeK<R> k = make_yee<R>(p, true, imag, P, Q, Rp, (const R *)b->eps, (const R *)b->ce, nullptr,
                            psi, b->inv_dh);
    k.xbeg = xbeg;
    k.xend = xend < p->sx ? xend : p->sx;
    if (added) *added = false;
    if (src && added && !imag && k.bulk && src->n > 0 && src->n <= YEE_SRC && k.xbeg == 0 && k.xend == p->sx) {
        k.nsrc = src->n;
        k.src_t = t;
        k.src_stride = src->n;
        k.src_values = (const R *)src->values;
        for (int s = 0; s < src->n; ++s) {
            const uint64_t ind = (uint64_t)src->index[s], cell = ind % p->N;
            k.src_c[s] = (int32_t)(ind / p->N);
            k.src_x[s] = (uint32_t)(cell / p->syz);
            k.src_j[s] = (uint32_t)(cell % p->syz);
            k.src_col[s] = s;
        }
        *added = true;
    }
    return check_cuda(launch_yee_e<R>(k, st, pdl), imag ? "update_F launch" : "update_E launch");
}

template <typename R>
int run_update_h(FdtdPlan *p, const FdtdBuffers *b, cudaStream_t st, bool imag,
                 uint32_t xbeg = 0, uint32_t xend = 0xffffffffu)
{
    R *P = (R *)(imag ? b->G : b->H);
    const R *Q = (const R *)(imag ? b->F : b->E);
    const R *Rp = p->d.n_bloch ? (const R *)(imag ? b->E : b->F) : nullptr;
    void *const(*psi)[2] = imag ? b->psi_g : b->psi_h;
    const bool poynt = p->d.do_poynting && !imag;
    YeeK<R> k = make_yee<R>(p, false, imag, P, Q, Rp, p->d.has_mu ? (const R *)b->mu : nullptr,
                            p->d.has_mu ? (const R *)b->cm : nullptr,
                            poynt ? (R *)b->oS : nullptr, psi, b->inv_de);
    k.xbeg = xbeg;
    k.xend = xend < p->sx ? xend : p->sx;
    return check_cuda(launch_yee_h<R>(k, p->d.has_mu != 0, poynt, st),
                      imag ? "update_G launch" : "update_H launch");
}

template <typename R>
int run_update_s(FdtdPlan *p, const FdtdBuffers *b, cudaStream_t st,
                 uint32_t xbeg = 0, uint32_t xend = 0xffffffffu)
{
    SK<R> k;
    std::memset(&k, 0, sizeof(k));
    k.S = (R *)b->S;
    k.oS = (const R *)b->oS;
    k.sx = p->sx;
    k.sy = p->sy;
    k.sz = p->sz;
    k.syz = p->syz;
    k.N = p->N;
    k.dsz = FastDiv::make(p->sz);
    k.xchunk = p->xchunk;
    k.xbeg = xbeg;
    k.xend = xend < p->sx ? xend : p->sx;
    const R dt = (R)p->d.dt;
    k.sf = (R)((double)dt * 0.125);  // update_s.cl:33
    return check_cuda(launch_poynting<R>(k, st), "update_S launch");
}

template <typename R>
int run_prepare(FdtdPlan *p, const FdtdBuffers *b, cudaStream_t st)
{
    PrepK<R> k;
    k.n = 3 * p->N;
    k.dt = (R)p->d.dt;
    if (b->ce) {
        k.out = (R *)b->ce;
        k.mat = (const R *)b->eps;
        int rc = check_cuda(launch_prepare<R>(k, st), "prepare(dt/eps) launch");
        if (rc) return rc;
    }
    if (p->d.has_mu && b->cm) {
        k.out = (R *)b->cm;
        k.mat = (const R *)b->mu;
        return check_cuda(launch_prepare<R>(k, st), "prepare(dt/mu) launch");
    }
    return FDTD_OK;
}

template <typename R>
int run_update_j(FdtdPlan *p, const FdtdBuffers *b, cudaStream_t st, double c, double s,
                 const uint32_t lo[3], const uint32_t n[3])
{
    JK<R> k;
    k.E = (R *)b->E;
    k.Jr = (const R *)b->Jr;
    k.Ji = (const R *)b->Ji;
    k.sy = p->sy;
    k.sz = p->sz;
    k.N = p->N;
    k.x0 = lo[0];
    k.y0 = lo[1];
    k.z0 = lo[2];
    k.nx = n[0];
    k.ny = n[1];
    k.nz = n[2];
    k.dnz = FastDiv::make(n[2] ? n[2] : 1);
    k.dnyz = FastDiv::make(n[1] * n[2] ? n[1] * n[2] : 1);
    k.c = (R)c;
    k.s = (R)s;
    return check_cuda(launch_fieldsrc<R>(k, st), "update_J launch");
}

template <typename R>
DftK<R> dft_args(FdtdPlan *p, const void *field, const FdtdDftMonitor *m, int64_t t)
{
    DftK<R> k;
    k.field = (const R *)field;
    k.index = m->index;
    k.omega = m->omega;
    k.accum = m->accum;
    k.series = m->series;
    k.npoint = m->n_points;
    k.nfreq = m->n_freq;
    k.step = m->step + t;
    k.series_row = m->series_row + t;
    k.dt = p->d.dt;
    return k;
}

template <typename R>
int run_dft(FdtdPlan *p, const void *field, cudaStream_t st, const FdtdDftMonitor *m, int64_t t)
{
    return check_cuda(launch_dft<R>(dft_args<R>(p, field, m, t), st), "DFT monitor launch");
}

// Arguments of the sources whose x plane lies in [xbeg, xend) (all when the range is the grid).
template <typename R>
PointK<R> source_args(FdtdPlan *p, const FdtdBuffers *b, const FdtdPointSources *src, int t,
                      uint32_t xbeg = 0, uint32_t xend = 0xffffffffu)
{
    PointK<R> k;
    std::memset(&k, 0, sizeof(k));
    k.E = (R *)b->E;
    k.values = (const R *)src->values;
    k.t = t;
    k.stride = src->n;
    int n = 0;
    for (int s = 0; s < src->n; ++s) {
        const uint32_t plane = (uint32_t)(((uint64_t)src->index[s] % p->N) / p->syz);
        if (plane < xbeg || plane >= xend) continue;
        k.index[n] = src->index[s];
        k.col[n] = s;
        ++n;
    }
    k.n = n;
    return k;
}

template <typename R>
int run_point_sources(FdtdPlan *p, const FdtdBuffers *b, cudaStream_t st,
                      const FdtdPointSources *src, int t, uint32_t xbeg = 0,
                      uint32_t xend = 0xffffffffu)
{
    const PointK<R> k = source_args<R>(p, b, src, t, xbeg, xend);
    if (!k.n) return FDTD_OK;
    return check_cuda(launch_point_sources<R>(k, st), "point source launch");
}

// Profiling aid of fdtd_run (FDTD_TUNE_TIMING): CUDA events on the launching stream around the
// two kernels of up to 64 steps spread over the call; finish() waits for the stream and stores
// the mean launch times in the plan. Inactive (no events, no waiting) when timing is off.
class KernelTimer {
  public:
    static constexpr int MAX_SAMPLES = 64;
    KernelTimer(FdtdPlan *p, int nsteps, cudaStream_t st) : p_(p), st_(st), n_(0), stride_(0)
    {
        if (p->timing && nsteps > 0) stride_ = (nsteps + MAX_SAMPLES - 1) / MAX_SAMPLES;
        nsteps_ = nsteps;
    }
    ~KernelTimer()
    {
        for (int s = 0; s < n_; ++s)
            for (int c = 0; c < 4; ++c) cudaEventDestroy(ev_[s][c]);
    }
    int init()
    {
        if (!stride_) return FDTD_OK;
        for (int s = 0; s < MAX_SAMPLES && s * stride_ < nsteps_; ++s) {
            for (int c = 0; c < 4; ++c) {
                const cudaError_t e = cudaEventCreate(&ev_[s][c]);
                if (e != cudaSuccess) {
                    for (int q = 0; q < c; ++q) cudaEventDestroy(ev_[s][q]);
                    return check_cuda(e, "timing event");
                }
            }
            ++n_;
        }
        return FDTD_OK;
    }
    // c: 0/1 around update_E, 2/3 around the H+S kernel
    int mark(int t, int c)
    {
        if (!stride_ || t % stride_) return FDTD_OK;
        return check_cuda(cudaEventRecord(ev_[t / stride_][c], st_), "timing event");
    }
    int finish()
    {
        if (!n_) return FDTD_OK;
        int rc = check_cuda(cudaStreamSynchronize(st_), "timing sync");
        if (rc) return rc;
        double se = 0.0, sh = 0.0;
        for (int s = 0; s < n_; ++s) {
            float me = 0.f, mh = 0.f;
            if ((rc = check_cuda(cudaEventElapsedTime(&me, ev_[s][0], ev_[s][1]), "timing read"))) return rc;
            if ((rc = check_cuda(cudaEventElapsedTime(&mh, ev_[s][2], ev_[s][3]), "timing read"))) return rc;
            se += me;
            sh += mh;
        }
        p_->kernel_ms[0] = se / n_;
        p_->kernel_ms[1] = sh / n_;
        p_->kernel_samples = n_;
        return FDTD_OK;
    }

  private:
    FdtdPlan *p_;
    cudaStream_t st_;
    int n_, stride_, nsteps_;
    cudaEvent_t ev_[MAX_SAMPLES][4];
};

// The plan's side stream and its two events, created on first use.
static int side_stream(FdtdPlan *p)
{
    if (p->side) return FDTD_OK;
    int rc;
    if ((rc = check_cuda(cudaStreamCreateWithFlags(&p->side, cudaStreamNonBlocking), "side stream"))) return rc;
    if ((rc = check_cuda(cudaEventCreateWithFlags(&p->ev_fork, cudaEventDisableTiming), "fork event"))) return rc;
    return check_cuda(cudaEventCreateWithFlags(&p->ev_join, cudaEventDisableTiming), "join event");
}

// x chunk of the H+S kernel when none is set: among 14..24 planes, the one whose grid (plus
// the extra blocks) best fills whole waves of resident blocks, two per SM; the smallest such
// chunk on a tie. On the 395x345x73 grid (69 row blocks, 152 SMs) it is 18: 1518 blocks, 4.99
// waves, which ran 2% faster per step than 16 planes (5.67 waves).
static uint32_t hs_auto_xchunk(const FdtdPlan *p, uint32_t nrowblk, uint32_t extra)
{
    int nsm = 0;
    if (cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, p->device) != cudaSuccess || nsm <= 0)
        nsm = 1;
    const double slots = 2.0 * nsm;
    uint32_t best = 16;
    double best_eff = -1.0;
    for (uint32_t xc = 14; xc <= 24; ++xc) {
        const double waves = (double)(nrowblk * ((p->sx + xc - 1u) / xc) + extra) / slots;
        const double eff = waves / std::ceil(waves);
        if (eff > best_eff + 1e-12) {
            best_eff = eff;
            best = xc;
        }
    }
    return best;
}

// Multi-step path with the H+S kernel: update_E in place, point sources, then H and S in one
// launch that reads H (and the H-side psi) from one copy and writes the other; the copies
// swap every step and the state is brought home after an odd number of steps.
template <typename R>
int run_hs(FdtdPlan *p, const FdtdBuffers *b, cudaStream_t st, int nsteps,
           const FdtdPointSources *src, const FdtdDftMonitor *mon)
{
    HSK<R> k;
    std::memset(&k, 0, sizeof(k));
    k.sx = p->sx;
    k.sy = p->sy;
    k.sz = p->sz;
    k.syz = p->syz;
    k.N = p->N;
    k.dt = (R)p->d.dt;
    k.inv_d = (R)(1.0 / p->d.dx);
    k.sf = (R)((double)k.dt * 0.125);
    for (int r = 0; r < 3; ++r) k.inv_de[r] = p->d.uniform ? nullptr : (const R *)b->inv_de[r];
    const int dxmode = !p->d.uniform ? 2 : ((R)(1.0 / p->d.dx) == R(1) ? 0 : 1);
    k.cm = p->d.has_mu ? (const R *)b->cm : nullptr;
    k.S = (R *)b->S;
    k.oS = (R *)b->oS;
    k.dsz = FastDiv::make(p->sz);
    k.rows = (uint32_t)HS_THREADS / p->sz - 1u;
    k.reverse = p->hs_reverse;
    k.nrowblk = (k.sy + k.rows - 1u) / k.rows;
    k.xchunk = p->hs_xchunk ? p->hs_xchunk : hs_auto_xchunk(p, k.nrowblk, mon && p->hs_dft ? 1u : 0u);
    k.nchunk = (k.sx + k.xchunk - 1u) / k.xchunk;
    p->hs_xchunk_used = (int32_t)k.xchunk;
    int fidx[3][2] = {{-1, -1}, {-1, -1}, {-1, -1}};
    for (int f = 0; f < p->d.n_pml; ++f) {
        const FdtdPmlDesc &pd = p->d.pml[f];
        const uint32_t sa = pd.axis == 0 ? p->sx : pd.axis == 1 ? p->sy : p->sz;
        if (pd.polarity == 1 && (uint32_t)pd.thickness > sa) continue;
        HSAxis<R> &a = k.ax[pd.axis];
        if (pd.polarity == 0) a.Tn = pd.thickness;
        else a.Tp = pd.thickness;
        for (int c = 0; c < 3; ++c) a.tab[pd.polarity][c] = (const R *)p->tab[f][3 + c];
        fidx[pd.axis][pd.polarity] = f;
    }
    FdtdBuffers bb = *b;
    void *H[2] = {b->H, b->H2};
    int rc;
    KernelTimer timer(p, nsteps, st);
    if ((rc = timer.init())) return rc;
    // the step's DFT sample: in the H+S launch (one extra block) or on the side stream beside it
    const bool dft_in = mon && p->hs_dft;
    const bool dft_side = mon && !p->hs_dft;
    const bool pdl = p->pdl != 0;
    if (dft_side && (rc = side_stream(p))) return rc;
    for (int t = 0; t < nsteps; ++t) {
        const int a = t & 1, o = a ^ 1;
        bb.H = H[a];
        // the previous step's DFT sample has read E
        if (dft_side && t > 0 && (rc = check_cuda(cudaStreamWaitEvent(st, p->ev_join, 0), "join wait"))) return rc;
        if ((rc = lbc_before_e(p, b, H[a], st))) return rc;
        if ((rc = timer.mark(t, 0))) return rc;
        // without a learned boundary (whose E fix-up comes before the sources) the E kernel
        // adds the point sources itself
        bool added = false;
        if ((rc = run_update_e<R>(p, &bb, st, false, 0, 0xffffffffu, p->lbc_mask ? nullptr : src, t, &added, pdl))) return rc;
        if ((rc = timer.mark(t, 1))) return rc;
        if ((rc = lbc_after_e(p, b, H[a], st))) return rc;
        if (!added && src && src->n > 0 && (rc = run_point_sources<R>(p, &bb, st, src, t))) return rc;
        // the H+S launch leaves E unchanged, so the step's DFT sample of E is taken by its last
        // block, or (hs_dft off) runs on the side stream beside it and the next step's E update
        // waits for it (above)
        k.dft_on = dft_in ? 1 : 0;
        if (dft_in) k.dft = dft_args<R>(p, b->E, mon, t);
        if (dft_side) {
            if ((rc = check_cuda(cudaEventRecord(p->ev_fork, st), "fork event"))) return rc;
            if ((rc = check_cuda(cudaStreamWaitEvent(p->side, p->ev_fork, 0), "side stream wait"))) return rc;
            if ((rc = run_dft<R>(p, b->E, p->side, mon, t))) return rc;
            if ((rc = check_cuda(cudaEventRecord(p->ev_join, p->side), "join event"))) return rc;
        }
        k.E = (const R *)b->E;
        k.HA = (const R *)H[a];
        k.HB = (R *)H[o];
        for (int r = 0; r < 3; ++r)
            for (int side = 0; side < 2; ++side) {
                const int f = fidx[r][side];
                if (f < 0) continue;
                void *const *pa = a ? b->psi_h2[f] : b->psi_h[f];
                void *const *po = o ? b->psi_h2[f] : b->psi_h[f];
                for (int c = 0; c < 2; ++c) {
                    k.ax[r].A[side][c] = (const R *)pa[c];
                    k.ax[r].B[side][c] = (R *)po[c];
                }
            }
        k.write_oS = t == nsteps - 1;
        if ((rc = timer.mark(t, 2))) return rc;
        if ((rc = check_cuda(launch_hs<R>(k, p->d.has_mu != 0, dxmode, p->hs_prefetch != 0, pdl, st), "H+S launch"))) return rc;
        if ((rc = timer.mark(t, 3))) return rc;
        if ((rc = lbc_after_h(p, b, H[o], st))) return rc;
    }
    // the caller's stream sees the last DFT sample
    if (dft_side && nsteps > 0 && (rc = check_cuda(cudaStreamWaitEvent(st, p->ev_join, 0), "join wait"))) return rc;
    if ((rc = timer.finish())) return rc;
    if (nsteps & 1) {
        const size_t fb = 3 * (size_t)p->N * p->elem;
        rc = check_cuda(cudaMemcpyAsync(b->H, b->H2, fb, cudaMemcpyDeviceToDevice, st), "copy H");
        for (int f = 0; !rc && f < p->d.n_pml; ++f) {
            const FdtdPmlDesc &pd = p->d.pml[f];
            const size_t cells = (size_t)p->N / (pd.axis == 0 ? p->sx : pd.axis == 1 ? p->sy : p->sz);
            const size_t pb = cells * (size_t)pd.thickness * p->elem;
            for (int c = 0; !rc && c < 2 && pb; ++c)
                rc = check_cuda(cudaMemcpyAsync(b->psi_h[f][c], b->psi_h2[f][c], pb, cudaMemcpyDeviceToDevice, st), "copy psi_h");
        }
        if (rc) return rc;
    }
    return FDTD_OK;
}

// Per-update kernels over x slabs small enough to stay resident in L2: E on slab s, then H
// one plane behind (H at x needs E_new at x+1; E at x needs H_old at x-1), then S one plane
// behind H. Within a step each update's reads of the previous update's output hit L2 while
// the slab is still there. Every cell is updated by the same kernels as a full-grid launch,
// so results do not depend on the slab size.
template <typename R>
int run_slabs(FdtdPlan *p, const FdtdBuffers *b, cudaStream_t st, int nsteps,
              const FdtdPointSources *src, const FdtdDftMonitor *mon)
{
    const uint32_t sx = p->sx;
    // the learned boundary's E corrections must land before any H update reads them: whole grid
    const uint32_t W = p->slab && !p->lbc_mask ? p->slab : sx;
    const bool bloch = p->d.n_bloch != 0, poynt = p->d.do_poynting != 0;
    int rc;
    if (W >= sx) {
        // one slab: the plain whole-grid sequence
        for (int t = 0; t < nsteps; ++t) {
            if ((rc = lbc_before_e(p, b, b->H, st))) return rc;
            if ((rc = run_update_e<R>(p, b, st, false))) return rc;
            if (bloch && (rc = run_update_e<R>(p, b, st, true))) return rc;
            if ((rc = lbc_after_e(p, b, b->H, st))) return rc;
            if (src && src->n > 0 && (rc = run_point_sources<R>(p, b, st, src, t))) return rc;
            if ((rc = run_update_h<R>(p, b, st, false))) return rc;
            if (bloch && (rc = run_update_h<R>(p, b, st, true))) return rc;
            if ((rc = lbc_after_h(p, b, b->H, st))) return rc;
            if (poynt && (rc = run_update_s<R>(p, b, st))) return rc;
            if (mon && (rc = run_dft<R>(p, b->E, st, mon, t))) return rc;
        }
        return FDTD_OK;
    }
    for (int t = 0; t < nsteps; ++t) {
        for (uint32_t a = 0; a < sx; a += W) {
            const uint32_t e = a + W < sx ? a + W : sx;
            if ((rc = run_update_e<R>(p, b, st, false, a, e))) return rc;
            if (bloch && (rc = run_update_e<R>(p, b, st, true, a, e))) return rc;
            if (src && src->n > 0 && (rc = run_point_sources<R>(p, b, st, src, t, a, e))) return rc;
            const uint32_t h0 = a ? a - 1 : 0, h1 = e - 1;
            if ((rc = run_update_h<R>(p, b, st, false, h0, h1))) return rc;
            if (bloch && (rc = run_update_h<R>(p, b, st, true, h0, h1))) return rc;
            if (poynt && (rc = run_update_s<R>(p, b, st, h0 ? h0 : 1, h1))) return rc;
        }
        if ((rc = run_update_h<R>(p, b, st, false, sx - 1, sx))) return rc;
        if (bloch && (rc = run_update_h<R>(p, b, st, true, sx - 1, sx))) return rc;
        if (poynt) {
            if ((rc = run_update_s<R>(p, b, st, sx - 1, sx))) return rc;
            if (sx > 1 && (rc = run_update_s<R>(p, b, st, 0, 1))) return rc;
        }
        if (mon && (rc = run_dft<R>(p, b->E, st, mon, t))) return rc;
    }
    return FDTD_OK;
}

// ---- one-pass step (step_kernel.cu) -------------------------------------------------------
bool aligned16(const void *q) { return ((uintptr_t)q & 15u) == 0; }

// CPML faces of the one-pass step (a 'p' face thicker than its axis never applies), the offset
// of each face's six coefficient tables in the plan's table block, and the plan's face index per
// axis and side (-1: none).
template <typename R>
void step_faces(const FdtdPlan *p, StepK<R> &k, int fidx[3][2])
{
    const uint32_t sa[3] = {p->sx, p->sy, p->sz};
    for (int r = 0; r < 3; ++r) fidx[r][0] = fidx[r][1] = -1;
    size_t off = 0;
    for (int f = 0; f < p->d.n_pml; ++f) {
        const FdtdPmlDesc &pd = p->d.pml[f];
        const size_t here = off;
        off += 6 * (size_t)(pd.thickness > 0 ? pd.thickness : 0);
        if (pd.thickness <= 0 || (pd.polarity == 1 && (uint32_t)pd.thickness > sa[pd.axis])) continue;
        StepAxis<R> &a = k.ax[pd.axis];
        const int side = pd.polarity;
        if (side == 0) a.Tn = pd.thickness;
        else a.Tp = pd.thickness;
        k.coff[pd.axis][side] = (int32_t)here;
        fidx[pd.axis][side] = f;
    }
    k.coef = (const R *)p->coef;
    k.ncoef = (uint32_t)off;
}

// Tiling of the one-pass step for a plan: block shape, own rows per tile, tiles, x chunk, stages,
// threads and the stage layout. False when the kernel does not apply (z rows too long, too many
// CPML coefficients, or too little shared memory for two stages).
template <typename R>
bool step_layout(const FdtdPlan *p, StepK<R> &k, int &shape, uint32_t &threads, size_t &smem)
{
    constexpr uint32_t V = 16 / sizeof(R);
    if (k.ncoef > (uint32_t)STEP_MAX_COEF) return false;
    int optin = 0;
    cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, p->device);
    int smsm = 0;
    cudaDeviceGetAttribute(&smsm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, p->device);
    // block shape: the two-blocks-per-SM shape when a tile of it holds at least 3 own rows
    shape = STEP_SHAPE_BIG;
    if (sizeof(R) == 4) {
        if (p->fused_shape == STEP_SHAPE_SMALL) shape = STEP_SHAPE_SMALL;
        else if (!p->fused_shape && step_max_rows<R>(STEP_SHAPE_SMALL, p->sz) >= 3) shape = STEP_SHAPE_SMALL;
    }
    const uint32_t maxr = step_max_rows<R>(shape, p->sz);
    if (!maxr) return false;
    uint32_t rows = p->fused_rows ? (p->fused_rows < maxr ? p->fused_rows : maxr) : maxr;
    if (rows > p->sy) rows = p->sy;
    k.ntile = (p->sy + rows - 1) / rows;
    const uint32_t own = (p->sy + k.ntile - 1) / k.ntile;   // most own rows of any tile
    threads = step_threads(own, p->sz);
    // stage: the field slots, then the z-face CPML slots (four per side) for own + 3 staged rows
    const uint32_t nf = p->d.has_mu ? 12u : 9u;
    const uint32_t str = sizeof(R) == 8 ? (uint32_t)StepF64::STR
                       : shape == STEP_SHAPE_SMALL ? (uint32_t)StepSmall::STR : (uint32_t)StepBig::STR;
    uint32_t off = nf * str;
    for (int side = 0; side < 2; ++side) {
        const uint32_t T = (uint32_t)(side ? k.ax[2].Tp : k.ax[2].Tn);
        k.zoff[side] = off;
        k.zsz[side] = T ? ((own + 3u) * T + 2u * (V - 1u) + V - 1u) / V * V : 0u;
        off += 4u * k.zsz[side];
    }
    k.stage_elems = off;
    // shared memory per block: all of it for the large shape, half an SM for the small one
    size_t cap = (size_t)optin;
    if (shape == STEP_SHAPE_SMALL) {
        const size_t half = (size_t)smsm / 2 - 1024;
        if (half < cap) cap = half;
    }
    uint32_t ns = p->fused_stages ? p->fused_stages : 4u;
    while (ns >= 2 && step_smem_bytes<R>(shape, ns, k.stage_elems, k.ncoef) > cap) --ns;
    if (ns < 2) return false;
    k.nstage = ns;
    smem = step_smem_bytes<R>(shape, ns, k.stage_elems, k.ncoef);
    // x chunk: as many chunks as give whole waves of the resident blocks
    uint32_t xc = p->fused_xchunk;
    if (!xc) {
        int nsm = 0;
        cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, p->device);
        if (nsm < 1) nsm = 1;
        const uint32_t slots = (uint32_t)nsm * (shape == STEP_SHAPE_SMALL ? 2u : 1u);
        const uint32_t waves = (k.ntile + slots - 1) / slots;
        uint32_t nchunk = waves * slots / k.ntile;
        if (nchunk < 1) nchunk = 1;
        if (nchunk > p->sx) nchunk = p->sx;
        xc = (p->sx + nchunk - 1) / nchunk;
    }
    k.xchunk = xc;
    return true;
}

// One-pass multi-step path: one launch per step, reading A and writing B, then swapping; the
// state is brought home after an odd number of steps.
template <typename R>
int run_fused(FdtdPlan *p, const FdtdBuffers *b, cudaStream_t st, int nsteps,
              const FdtdPointSources *src, const FdtdDftMonitor *mon)
{
    StepK<R> k;
    std::memset(&k, 0, sizeof(k));
    k.sx = p->sx;
    k.sy = p->sy;
    k.sz = p->sz;
    k.syz = p->syz;
    k.N = p->N;
    k.dt = (R)p->d.dt;
    k.inv_d = (R)(1.0 / p->d.dx);
    k.sf = (R)((double)k.dt * 0.125);
    for (int r = 0; r < 3; ++r) {
        k.inv_de[r] = p->d.uniform ? nullptr : (const R *)b->inv_de[r];
        k.inv_dh[r] = p->d.uniform ? nullptr : (const R *)b->inv_dh[r];
    }
    const int dxmode = !p->d.uniform ? 2 : ((R)(1.0 / p->d.dx) == R(1) ? 0 : 1);
    const bool mu = p->d.has_mu != 0;
    k.ce = (const R *)b->ce;
    k.cm = mu ? (const R *)b->cm : nullptr;
    k.S = (R *)b->S;
    k.oS = (R *)b->oS;
    k.poynt = p->d.do_poynting ? 1 : 0;
    k.status = p->status;
    k.wait_ns = 2000000000u;
    if (src && src->n > 0) {
        k.nsrc = src->n;
        k.src_values = (const R *)src->values;
        for (int s = 0; s < src->n; ++s) {
            const uint64_t ind = (uint64_t)src->index[s];
            const uint64_t cell = ind % p->N;
            k.src_c[s] = (int32_t)(ind / p->N);
            k.src_x[s] = (uint32_t)(cell / p->syz);
            k.src_j[s] = (uint32_t)(cell % p->syz);
        }
    }
    int fidx[3][2];
    step_faces<R>(p, k, fidx);
    uint32_t threads = 0;
    size_t smem = 0;
    int shape = 0;
    if (!step_layout<R>(p, k, shape, threads, smem))
        return fail(FDTD_ERR_UNSUPPORTED, "fdtd_run: one-pass step does not fit");
    for (int c = 0; c < SG_NF; ++c) k.len[c] = 3 * p->N;
    for (int q = 0; q < SG_NZ; ++q) {
        const int side = q >> 2;
        k.len[SG_NF + q] = (uint64_t)p->sx * p->sy * (uint64_t)(side ? k.ax[2].Tp : k.ax[2].Tn);
    }
    // bulk copies need 16-byte aligned bases for every staged array of both parities
    bool al = p->fused_tma && aligned16(b->E) && aligned16(b->E2) && aligned16(b->H) && aligned16(b->H2) &&
              aligned16(b->ce) && (!mu || aligned16(b->cm));
    for (int side = 0; side < 2 && al; ++side) {
        const int f = fidx[2][side];
        if (f < 0) continue;
        for (int c = 0; c < 2; ++c)
            al = al && aligned16(b->psi_e[f][c]) && aligned16(b->psi_e2[f][c]) && aligned16(b->psi_h[f][c]) &&
                 aligned16(b->psi_h2[f][c]);
    }
    k.tma = al ? 1 : 0;
    p->step_cfg[0] = (int32_t)((p->sy + k.ntile - 1) / k.ntile);
    p->step_cfg[1] = (int32_t)k.xchunk;
    p->step_cfg[2] = (int32_t)k.nstage;
    p->step_cfg[3] = (int32_t)threads;
    p->step_cfg[4] = shape;
    void *E[2] = {b->E, b->E2}, *H[2] = {b->H, b->H2};
    KernelTimer timer(p, nsteps, st);
    int rc;
    if ((rc = timer.init())) return rc;
    for (int t = 0; t < nsteps; ++t) {
        const int a = t & 1, o = a ^ 1;
        k.EA = (const R *)E[a];
        k.HA = (const R *)H[a];
        k.EB = (R *)E[o];
        k.HB = (R *)H[o];
        for (int r = 0; r < 3; ++r)
            for (int side = 0; side < 2; ++side) {
                const int f = fidx[r][side];
                if (f < 0) continue;
                void *const *pe_a = a ? b->psi_e2[f] : b->psi_e[f];
                void *const *ph_a = a ? b->psi_h2[f] : b->psi_h[f];
                void *const *pe_o = o ? b->psi_e2[f] : b->psi_e[f];
                void *const *ph_o = o ? b->psi_h2[f] : b->psi_h[f];
                for (int c = 0; c < 2; ++c) {
                    k.ax[r].psiA[0][side][c] = (const R *)pe_a[c];
                    k.ax[r].psiA[1][side][c] = (const R *)ph_a[c];
                    k.ax[r].psiB[0][side][c] = (R *)pe_o[c];
                    k.ax[r].psiB[1][side][c] = (R *)ph_o[c];
                }
            }
        k.t = t;
        k.write_oS = k.poynt && t == nsteps - 1;
        if ((rc = timer.mark(t, 0))) return rc;
        if ((rc = check_cuda(launch_step<R>(k, shape, dxmode, mu, threads, smem, st), "one-pass step launch"))) return rc;
        if ((rc = timer.mark(t, 1))) return rc;
        if ((rc = timer.mark(t, 2))) return rc;
        if ((rc = timer.mark(t, 3))) return rc;
        if (mon && (rc = run_dft<R>(p, E[o], st, mon, t))) return rc;
    }
    if ((rc = timer.finish())) return rc;
    if (nsteps & 1) {
        // the last step wrote the second copies: bring the state home
        const size_t fb = 3 * (size_t)p->N * p->elem;
        rc = check_cuda(cudaMemcpyAsync(b->E, b->E2, fb, cudaMemcpyDeviceToDevice, st), "copy E");
        if (!rc) rc = check_cuda(cudaMemcpyAsync(b->H, b->H2, fb, cudaMemcpyDeviceToDevice, st), "copy H");
        for (int f = 0; !rc && f < p->d.n_pml; ++f) {
            const FdtdPmlDesc &pd = p->d.pml[f];
            size_t cells = (size_t)p->N / (pd.axis == 0 ? p->sx : pd.axis == 1 ? p->sy : p->sz);
            const size_t pb = cells * (size_t)pd.thickness * p->elem;
            for (int c = 0; !rc && c < 2 && pb; ++c) {
                rc = check_cuda(cudaMemcpyAsync(b->psi_e[f][c], b->psi_e2[f][c], pb, cudaMemcpyDeviceToDevice, st), "copy psi_e");
                if (!rc) rc = check_cuda(cudaMemcpyAsync(b->psi_h[f][c], b->psi_h2[f][c], pb, cudaMemcpyDeviceToDevice, st), "copy psi_h");
            }
        }
        if (rc) return rc;
    }
    return FDTD_OK;
}

}  // namespace fdtd

// ---------------------------------------------------------------------------------------------
// validation
// ---------------------------------------------------------------------------------------------
namespace {

int validate_desc(const FdtdDesc *d)
{
    if (!d) return fail(FDTD_ERR_INVALID, "desc is NULL");
    for (int r = 0; r < 3; ++r)
        if (d->shape[r] < 1) return fail(FDTD_ERR_INVALID, "shape entries must be >= 1");
    const unsigned long long N = (unsigned long long)d->shape[0] * d->shape[1] * d->shape[2];
    if (N >= (1ull << 32)) return fail(FDTD_ERR_INVALID, "grid too large: N must be < 2^32 cells");
    if (d->shape[0] > 65535) return fail(FDTD_ERR_INVALID, "sx must be <= 65535");
    if (d->dtype != FDTD_F32 && d->dtype != FDTD_F64)
        return fail(FDTD_ERR_UNSUPPORTED, "dtype must be FDTD_F32 or FDTD_F64");
    if (!(d->dt > 0)) return fail(FDTD_ERR_INVALID, "dt must be > 0");
    if (d->uniform && !(d->dx > 0)) return fail(FDTD_ERR_INVALID, "dx must be > 0");
    if (d->n_pml < 0 || d->n_pml > 6) return fail(FDTD_ERR_INVALID, "n_pml must be in [0, 6]");
    int seen = 0;
    for (int f = 0; f < d->n_pml; ++f) {
        const FdtdPmlDesc &p = d->pml[f];
        if (p.axis < 0 || p.axis > 2) return fail(FDTD_ERR_INVALID, "pml axis must be 0, 1 or 2");
        if (p.polarity != 0 && p.polarity != 1)
            return fail(FDTD_ERR_INVALID, "pml polarity must be 0 ('n') or 1 ('p')");
        if (p.thickness < 0 || p.thickness > 65535)
            return fail(FDTD_ERR_INVALID, "pml thickness must be in [0, 65535]");
        const int bit = 1 << (2 * p.axis + p.polarity);
        if (seen & bit) return fail(FDTD_ERR_INVALID, "duplicate pml face");
        seen |= bit;
        if (p.thickness > 0 && (!p.p0e || !p.p1e || !p.p2e || !p.p0h || !p.p1h || !p.p2h))
            return fail(FDTD_ERR_INVALID, "pml coefficient table pointer is NULL");
    }
    if (d->n_bloch < 0 || d->n_bloch > 3) return fail(FDTD_ERR_INVALID, "n_bloch must be in [0, 3]");
    int bseen = 0;
    for (int b = 0; b < d->n_bloch; ++b) {
        const int a = d->bloch[b].axis;
        if (a < 0 || a > 2) return fail(FDTD_ERR_INVALID, "bloch axis must be 0, 1 or 2");
        if (bseen & (1 << a)) return fail(FDTD_ERR_INVALID, "duplicate bloch axis");
        bseen |= 1 << a;
    }
    return FDTD_OK;
}

int check_common(const FdtdPlan *p, const FdtdBuffers *b)
{
    if (!p) return fail(FDTD_ERR_INVALID, "plan is NULL");
    if (!b) return fail(FDTD_ERR_INVALID, "buffers is NULL");
    return FDTD_OK;
}

int check_psi(const FdtdPlan *p, void *const psi[6][2], const char *what)
{
    for (int f = 0; f < p->d.n_pml; ++f)
        if (p->d.pml[f].thickness > 0 && (!psi[f][0] || !psi[f][1]))
            return fail(FDTD_ERR_INVALID, std::string(what) + ": psi pointer is NULL");
    return FDTD_OK;
}

// The fused step covers the common case: no Bloch boundaries, CPML faces of one axis
// disjoint, dt/eps (and dt/mu) caches and every scratch buffer present, few point sources,
// and a per-block window that fits in shared memory.
bool fused_eligible(const FdtdPlan *p, const FdtdBuffers *b, const FdtdPointSources *src)
{
    if (p->d.n_bloch || !faces_disjoint(p)) return false;
    if (!b->ce || (p->d.has_mu && !b->cm)) return false;
    if (!b->E2 || !b->H2) return false;
    if (p->d.do_poynting && (!b->S || !b->oS)) return false;
    if (!p->d.uniform && (!b->inv_de[0] || !b->inv_dh[0])) return false;
    for (int f = 0; f < p->d.n_pml; ++f)
        if (p->d.pml[f].thickness > 0 &&
            (!b->psi_e2[f][0] || !b->psi_e2[f][1] || !b->psi_h2[f][0] || !b->psi_h2[f][1]))
            return false;
    if (src && src->n > STEP_MAX_SRC) return false;
    uint32_t threads = 0;
    size_t smem = 0;
    int fidx[3][2], shape = 0;
    if (p->d.dtype == FDTD_F64) {
        StepK<double> k;
        std::memset(&k, 0, sizeof(k));
        step_faces<double>(p, k, fidx);
        return step_layout<double>(p, k, shape, threads, smem);
    }
    StepK<float> k;
    std::memset(&k, 0, sizeof(k));
    step_faces<float>(p, k, fidx);
    return step_layout<float>(p, k, shape, threads, smem);
}

// The H+S path: Poynting on, no Bloch boundaries, CPML faces of one axis disjoint, dt/eps
// (and dt/mu) caches and the H scratch copies present, and a z row that fits a block.
bool hs_eligible(const FdtdPlan *p, const FdtdBuffers *b)
{
    if (!p->d.do_poynting || p->d.n_bloch || !faces_disjoint(p)) return false;
    if (!b->ce || (p->d.has_mu && !b->cm) || !b->H2 || !b->S || !b->oS) return false;
    if (2 * p->sz > (uint32_t)HS_THREADS) return false;   // at least one own row plus the halo row
    for (int f = 0; f < p->d.n_pml; ++f)
        if (p->d.pml[f].thickness > 0 && (!b->psi_h2[f][0] || !b->psi_h2[f][1])) return false;
    return true;
}

int check_inv(const FdtdPlan *p, const void *const inv[3], const char *what)
{
    if (p->d.uniform) return FDTD_OK;
    for (int r = 0; r < 3; ++r)
        if (!inv[r]) return fail(FDTD_ERR_INVALID, std::string(what) + ": spacing table is NULL");
    return FDTD_OK;
}

}  // namespace

// ---------------------------------------------------------------------------------------------
// extern "C" entry points
// ---------------------------------------------------------------------------------------------
extern "C" {

int fdtd_abi_version(void) { return FDTD_ABI_VERSION; }

const char *fdtd_last_error(void) { return g_err.c_str(); }

int fdtd_plan_create(const FdtdDesc *desc, FdtdPlan **out)
{
    if (!out) return fail(FDTD_ERR_INVALID, "out is NULL");
    *out = nullptr;
    int rc = validate_desc(desc);
    if (rc) return rc;
    FdtdPlan *p = new FdtdPlan();
    p->d = *desc;
    p->sx = (uint32_t)desc->shape[0];
    p->sy = (uint32_t)desc->shape[1];
    p->sz = (uint32_t)desc->shape[2];
    p->syz = p->sy * p->sz;
    p->N = (uint64_t)p->sx * p->syz;
    p->elem = desc->dtype == FDTD_F64 ? 8 : 4;
    p->xchunk = 8;
    // Whole-grid launches measured fastest on GB300 for the 395x345x73 workload (0.33 ms per
    // step against 0.43-0.86 ms for 48- to 8-plane slabs), so slabs are opt-in.
    p->slab = 0;
    p->fused_rows = 0;
    p->fused_stages = 0;
    p->fused_tma = 1;
    p->fused_shape = 0;
    p->last_run_path = FDTD_PATH_NONE;
    std::memset(p->step_cfg, 0, sizeof(p->step_cfg));
    p->hs_xchunk = 0;
    p->hs_prefetch = 0;
    p->hs_reverse = 1;
    // per-plane loads at four blocks per SM: update_E 0.110 -> 0.105 ms on the 395x345x73 grid
    p->eform = 1;
    p->hs_xchunk_used = 0;
    p->hs_dft = 1;
    p->pdl = 1;
    p->timing = 0;
    p->kernel_ms[0] = p->kernel_ms[1] = 0.0;
    p->kernel_samples = 0;
    p->fused_xchunk = 0;
    cudaGetDevice(&p->device);
    {
        cudaError_t e = cudaMalloc(&p->status, sizeof(int32_t));
        if (e == cudaSuccess) e = cudaMemset(p->status, 0, sizeof(int32_t));
        if (e != cudaSuccess) {
            if (p->status) cudaFree(p->status);
            delete p;
            return cuda_fail(e, "cudaMalloc(status word)");
        }
    }
    size_t total = 0;
    for (int f = 0; f < desc->n_pml; ++f) total += 6 * (size_t)desc->pml[f].thickness;
    std::memset(p->tab, 0, sizeof(p->tab));
    if (total) {
        cudaError_t e = cudaMalloc(&p->coef, total * p->elem);
        if (e != cudaSuccess) {
            cudaFree(p->status);
            delete p;
            return cuda_fail(e, "cudaMalloc(coefficient tables)");
        }
        std::vector<char> host(total * p->elem);
        size_t off = 0;
        for (int f = 0; f < desc->n_pml; ++f) {
            const FdtdPmlDesc &pd = desc->pml[f];
            const size_t bytes = (size_t)pd.thickness * p->elem;
            const void *src[6] = {pd.p0e, pd.p1e, pd.p2e, pd.p0h, pd.p1h, pd.p2h};
            for (int t = 0; t < 6; ++t) {
                if (bytes) std::memcpy(host.data() + off, src[t], bytes);
                p->tab[f][t] = (char *)p->coef + off;
                off += bytes;
            }
        }
        e = cudaMemcpy(p->coef, host.data(), host.size(), cudaMemcpyHostToDevice);
        if (e != cudaSuccess) {
            cudaFree(p->coef);
            cudaFree(p->status);
            delete p;
            return cuda_fail(e, "cudaMemcpy(coefficient tables)");
        }
    }
    *out = p;
    g_err.clear();
    return FDTD_OK;
}

int fdtd_plan_destroy(FdtdPlan *plan)
{
    if (!plan) return FDTD_OK;
    if (plan->coef) cudaFree(plan->coef);
    if (plan->status) cudaFree(plan->status);
    if (plan->ev_fork) cudaEventDestroy(plan->ev_fork);
    if (plan->ev_join) cudaEventDestroy(plan->ev_join);
    if (plan->side) cudaStreamDestroy(plan->side);
    delete plan;
    return FDTD_OK;
}

int fdtd_plan_tune(FdtdPlan *p, int32_t key, int32_t value)
{
    if (!p) return fail(FDTD_ERR_INVALID, "plan is NULL");
    switch (key) {
    case FDTD_TUNE_XCHUNK:
        if (value < 1 || value > 4096) return fail(FDTD_ERR_INVALID, "xchunk must be in [1, 4096]");
        p->xchunk = value;
        return FDTD_OK;
    case FDTD_TUNE_SLAB:
        if (value < 0) return fail(FDTD_ERR_INVALID, "slab must be >= 0 (0: whole grid)");
        p->slab = (uint32_t)value;
        return FDTD_OK;
    case FDTD_TUNE_FUSED_ROWS:
        if (value < 0 || value > 1024) return fail(FDTD_ERR_INVALID, "fused_rows must be in [0, 1024]");
        p->fused_rows = (uint32_t)value;
        return FDTD_OK;
    case FDTD_TUNE_FUSED_XCHUNK:
        if (value < 0 || value > 65536) return fail(FDTD_ERR_INVALID, "fused_xchunk must be in [0, 65536]");
        p->fused_xchunk = (uint32_t)value;
        return FDTD_OK;
    case FDTD_TUNE_FUSED_STAGES:
        if (value != 0 && (value < 2 || value > STEP_MAX_STAGES))
            return fail(FDTD_ERR_INVALID, "fused_stages must be 0 or in [2, 6]");
        p->fused_stages = (uint32_t)value;
        return FDTD_OK;
    case FDTD_TUNE_FUSED_TMA:
        if (value != 0 && value != 1) return fail(FDTD_ERR_INVALID, "fused_tma must be 0 or 1");
        p->fused_tma = value;
        return FDTD_OK;
    case FDTD_TUNE_HS_REVERSE:
        if (value != 0 && value != 1) return fail(FDTD_ERR_INVALID, "hs_reverse must be 0 or 1");
        p->hs_reverse = value;
        return FDTD_OK;
    case FDTD_TUNE_FUSED_SHAPE:
        if (value < 0 || value > 2) return fail(FDTD_ERR_INVALID, "fused_shape must be 0, 1 or 2");
        p->fused_shape = value;
        return FDTD_OK;
    case FDTD_TUNE_HS_XCHUNK:
        if (value < 0 || value > 4096) return fail(FDTD_ERR_INVALID, "hs_xchunk must be in [0, 4096] (0: automatic)");
        p->hs_xchunk = (uint32_t)value;
        return FDTD_OK;
    case FDTD_TUNE_TIMING:
        if (value != 0 && value != 1) return fail(FDTD_ERR_INVALID, "timing must be 0 or 1");
        p->timing = value;
        return FDTD_OK;
    case FDTD_TUNE_HS_PREFETCH:
        if (value != 0 && value != 1) return fail(FDTD_ERR_INVALID, "hs_prefetch must be 0 or 1");
        p->hs_prefetch = value;
        return FDTD_OK;
    case FDTD_TUNE_HS_DFT:
        if (value != 0 && value != 1) return fail(FDTD_ERR_INVALID, "hs_dft must be 0 or 1");
        p->hs_dft = value;
        return FDTD_OK;
    case FDTD_TUNE_PDL:
        if (value != 0 && value != 1) return fail(FDTD_ERR_INVALID, "pdl must be 0 or 1");
        p->pdl = value;
        return FDTD_OK;
    case FDTD_TUNE_E_FORM:
        if (value != 0 && value != 1) return fail(FDTD_ERR_INVALID, "e_form must be 0 or 1");
        p->eform = value;
        return FDTD_OK;
    default:
        return fail(FDTD_ERR_INVALID, "unknown tuning key");
    }
}

int fdtd_plan_get(const FdtdPlan *p, int32_t key, int32_t *value)
{
    if (!p || !value) return fail(FDTD_ERR_INVALID, "plan or value is NULL");
    switch (key) {
    case FDTD_TUNE_XCHUNK: *value = p->xchunk; return FDTD_OK;
    case FDTD_TUNE_SLAB: *value = (int32_t)p->slab; return FDTD_OK;
    case FDTD_TUNE_FUSED_ROWS: *value = (int32_t)p->fused_rows; return FDTD_OK;
    case FDTD_TUNE_FUSED_XCHUNK: *value = (int32_t)p->fused_xchunk; return FDTD_OK;
    case FDTD_TUNE_FUSED_STAGES: *value = (int32_t)p->fused_stages; return FDTD_OK;
    case FDTD_TUNE_FUSED_TMA: *value = p->fused_tma; return FDTD_OK;
    case FDTD_TUNE_FUSED_SHAPE: *value = p->fused_shape; return FDTD_OK;
    case FDTD_TUNE_HS_REVERSE: *value = p->hs_reverse; return FDTD_OK;
    case FDTD_GET_STEP_SHAPE: *value = p->step_cfg[4]; return FDTD_OK;
    case FDTD_GET_LAST_RUN_PATH: *value = p->last_run_path; return FDTD_OK;
    case FDTD_GET_STEP_ROWS: *value = p->step_cfg[0]; return FDTD_OK;
    case FDTD_GET_STEP_XCHUNK: *value = p->step_cfg[1]; return FDTD_OK;
    case FDTD_GET_STEP_STAGES: *value = p->step_cfg[2]; return FDTD_OK;
    case FDTD_GET_STEP_THREADS: *value = p->step_cfg[3]; return FDTD_OK;
    case FDTD_TUNE_HS_XCHUNK: *value = (int32_t)p->hs_xchunk; return FDTD_OK;
    case FDTD_TUNE_HS_PREFETCH: *value = p->hs_prefetch; return FDTD_OK;
    case FDTD_GET_HS_XCHUNK_USED: *value = p->hs_xchunk_used; return FDTD_OK;
    case FDTD_TUNE_HS_DFT: *value = p->hs_dft; return FDTD_OK;
    case FDTD_TUNE_PDL: *value = p->pdl; return FDTD_OK;
    case FDTD_TUNE_E_FORM: *value = p->eform; return FDTD_OK;
    case FDTD_TUNE_TIMING: *value = p->timing; return FDTD_OK;
    default: return fail(FDTD_ERR_INVALID, "unknown tuning key");
    }
}

int fdtd_prepare(FdtdPlan *p, const FdtdBuffers *b, void *stream)
{
    int rc = check_common(p, b);
    if (rc) return rc;
    if (b->ce && !b->eps) return fail(FDTD_ERR_INVALID, "prepare: eps is required to fill ce");
    if (p->d.has_mu && b->cm && !b->mu) return fail(FDTD_ERR_INVALID, "prepare: mu is required to fill cm");
    cudaStream_t st = (cudaStream_t)stream;
    return p->d.dtype == FDTD_F64 ? run_prepare<double>(p, b, st) : run_prepare<float>(p, b, st);
}

// The buffer checks of every update fdtd_run performs.
static int check_run_buffers(FdtdPlan *p, const FdtdBuffers *b)
{
    int rc;
    if (!b->E || !b->H || !b->eps) return fail(FDTD_ERR_INVALID, "fdtd_run: E, H and eps are required");
    if (p->d.n_bloch && (!b->F || !b->G)) return fail(FDTD_ERR_INVALID, "fdtd_run: F and G are required with Bloch boundaries");
    if (p->d.has_mu && !b->mu) return fail(FDTD_ERR_INVALID, "fdtd_run: mu is required");
    if (p->d.do_poynting && (!b->S || !b->oS)) return fail(FDTD_ERR_INVALID, "fdtd_run: S and oS are required with Poynting");
    if ((rc = check_psi(p, b->psi_e, "fdtd_run")) || (rc = check_psi(p, b->psi_h, "fdtd_run"))) return rc;
    if (p->d.n_bloch && ((rc = check_psi(p, b->psi_f, "fdtd_run")) || (rc = check_psi(p, b->psi_g, "fdtd_run")))) return rc;
    if ((rc = check_inv(p, b->inv_dh, "fdtd_run")) || (rc = check_inv(p, b->inv_de, "fdtd_run"))) return rc;
    return FDTD_OK;
}

int fdtd_update_e(FdtdPlan *p, const FdtdBuffers *b, void *stream)
{
    int rc = check_common(p, b);
    if (rc) return rc;
    if (!b->E || !b->H || !b->eps) return fail(FDTD_ERR_INVALID, "update_E: E, H and eps are required");
    if (p->d.n_bloch && !b->G) return fail(FDTD_ERR_INVALID, "update_E: G is required with Bloch boundaries");
    if ((rc = check_psi(p, b->psi_e, "update_E"))) return rc;
    if ((rc = check_inv(p, b->inv_dh, "update_E"))) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    return p->d.dtype == FDTD_F64 ? run_update_e<double>(p, b, st, false)
                                  : run_update_e<float>(p, b, st, false);
}

int fdtd_update_f(FdtdPlan *p, const FdtdBuffers *b, void *stream)
{
    int rc = check_common(p, b);
    if (rc) return rc;
    if (!p->d.n_bloch) return fail(FDTD_ERR_INVALID, "update_F: the plan has no Bloch boundaries");
    if (!b->F || !b->G || !b->H || !b->eps)
        return fail(FDTD_ERR_INVALID, "update_F: F, G, H and eps are required");
    if ((rc = check_psi(p, b->psi_f, "update_F"))) return rc;
    if ((rc = check_inv(p, b->inv_dh, "update_F"))) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    return p->d.dtype == FDTD_F64 ? run_update_e<double>(p, b, st, true)
                                  : run_update_e<float>(p, b, st, true);
}

int fdtd_update_h(FdtdPlan *p, const FdtdBuffers *b, void *stream)
{
    int rc = check_common(p, b);
    if (rc) return rc;
    if (!b->E || !b->H) return fail(FDTD_ERR_INVALID, "update_H: E and H are required");
    if (p->d.n_bloch && !b->F) return fail(FDTD_ERR_INVALID, "update_H: F is required with Bloch boundaries");
    if (p->d.has_mu && !b->mu) return fail(FDTD_ERR_INVALID, "update_H: mu is required");
    if (p->d.do_poynting && !b->oS) return fail(FDTD_ERR_INVALID, "update_H: oS is required with Poynting");
    if ((rc = check_psi(p, b->psi_h, "update_H"))) return rc;
    if ((rc = check_inv(p, b->inv_de, "update_H"))) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    return p->d.dtype == FDTD_F64 ? run_update_h<double>(p, b, st, false)
                                  : run_update_h<float>(p, b, st, false);
}

int fdtd_update_g(FdtdPlan *p, const FdtdBuffers *b, void *stream)
{
    int rc = check_common(p, b);
    if (rc) return rc;
    if (!p->d.n_bloch) return fail(FDTD_ERR_INVALID, "update_G: the plan has no Bloch boundaries");
    if (!b->F || !b->G || !b->E) return fail(FDTD_ERR_INVALID, "update_G: E, F and G are required");
    if (p->d.has_mu && !b->mu) return fail(FDTD_ERR_INVALID, "update_G: mu is required");
    if ((rc = check_psi(p, b->psi_g, "update_G"))) return rc;
    if ((rc = check_inv(p, b->inv_de, "update_G"))) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    return p->d.dtype == FDTD_F64 ? run_update_h<double>(p, b, st, true)
                                  : run_update_h<float>(p, b, st, true);
}

int fdtd_update_s(FdtdPlan *p, const FdtdBuffers *b, void *stream)
{
    int rc = check_common(p, b);
    if (rc) return rc;
    if (!p->d.do_poynting) return fail(FDTD_ERR_INVALID, "update_S: the plan has Poynting off");
    if (!b->S || !b->oS) return fail(FDTD_ERR_INVALID, "update_S: S and oS are required");
    cudaStream_t st = (cudaStream_t)stream;
    return p->d.dtype == FDTD_F64 ? run_update_s<double>(p, b, st) : run_update_s<float>(p, b, st);
}

int fdtd_update_j(FdtdPlan *p, const FdtdBuffers *b, void *stream, double c, double s,
                  const int64_t box[6])
{
    int rc = check_common(p, b);
    if (rc) return rc;
    if (!p->d.do_fieldsrc) return fail(FDTD_ERR_INVALID, "update_J: the plan has the field source off");
    if (!b->E || !b->Jr || !b->Ji) return fail(FDTD_ERR_INVALID, "update_J: E, Jr and Ji are required");
    if (!box) return fail(FDTD_ERR_INVALID, "update_J: box is NULL");
    const int64_t s3[3] = {(int64_t)p->sx, (int64_t)p->sy, (int64_t)p->sz};
    uint32_t lo[3], n[3];
    for (int r = 0; r < 3; ++r) {
        const int64_t a = box[2 * r], e = box[2 * r + 1];
        if (a < 0 || e < 0 || a > 0xffffffffll || e > 0xffffffffll)
            return fail(FDTD_ERR_INVALID, "update_J: box bounds must be unsigned 32-bit values");
        const int64_t ec = e < s3[r] ? e : s3[r];
        lo[r] = (uint32_t)a;
        n[r] = ec > a ? (uint32_t)(ec - a) : 0u;
    }
    cudaStream_t st = (cudaStream_t)stream;
    return p->d.dtype == FDTD_F64 ? run_update_j<double>(p, b, st, c, s, lo, n)
                                  : run_update_j<float>(p, b, st, c, s, lo, n);
}

static int check_monitor(const FdtdPlan *p, const FdtdDftMonitor *m)
{
    if (!m) return FDTD_OK;
    if (m->n_points < 0 || m->n_freq < 0) return fail(FDTD_ERR_INVALID, "monitor: negative sizes");
    if (m->n_points && (!m->index || (m->n_freq && (!m->omega || !m->accum))))
        return fail(FDTD_ERR_INVALID, "monitor: index, omega and accum are required");
    if (m->n_points && !m->n_freq && !m->series)
        return fail(FDTD_ERR_INVALID, "monitor: no frequency and no series");
    if (m->n_freq == 0 && m->series) {
        // series only: the kernel runs one thread per point with frequency slot 0 unused
    }
    return FDTD_OK;
}

int fdtd_monitor_sample(FdtdPlan *p, const FdtdBuffers *b, void *stream, const FdtdDftMonitor *m)
{
    int rc = check_common(p, b);
    if (rc) return rc;
    if (!m) return fail(FDTD_ERR_INVALID, "monitor is NULL");
    if ((rc = check_monitor(p, m))) return rc;
    if (!b->E) return fail(FDTD_ERR_INVALID, "monitor: E is required");
    cudaStream_t st = (cudaStream_t)stream;
    return p->d.dtype == FDTD_F64 ? run_dft<double>(p, b->E, st, m, 0) : run_dft<float>(p, b->E, st, m, 0);
}

}  // extern "C"

template <typename R>
static int plane_sum_t(FdtdPlan *p, const void *field, int comp, int axis, int64_t plane,
                       double *scratch, int nblk, double *out, cudaStream_t st)
{
    const PlaneRedK<R> k = plane_red_args<R>(field, comp, axis, plane, p->sx, p->sy, p->sz, scratch);
    return check_cuda(launch_plane_sum<R>(k, nblk, out, st), "plane sum launch");
}

extern "C" int fdtd_plane_sum(FdtdPlan *p, const void *field, int32_t comp, int32_t axis, int64_t plane,
                   double *scratch, int32_t scratch_len, double *out, void *stream)
{
    if (!p) return fail(FDTD_ERR_INVALID, "plan is NULL");
    if (!field || !scratch || !out) return fail(FDTD_ERR_INVALID, "plane sum: NULL pointer");
    if (comp < 0 || comp > 2 || axis < 0 || axis > 2) return fail(FDTD_ERR_INVALID, "plane sum: component and axis must be 0..2");
    const int64_t s = axis == 0 ? p->sx : axis == 1 ? p->sy : p->sz;
    if (plane < 0 || plane >= s) return fail(FDTD_ERR_INVALID, "plane sum: plane index out of range");
    if (scratch_len < 1) return fail(FDTD_ERR_INVALID, "plane sum: scratch_len must be >= 1");
    const int nblk = scratch_len < 1024 ? scratch_len : 1024;
    cudaStream_t st = (cudaStream_t)stream;
    return p->d.dtype == FDTD_F64 ? plane_sum_t<double>(p, field, comp, axis, plane, scratch, nblk, out, st)
                                  : plane_sum_t<float>(p, field, comp, axis, plane, scratch, nblk, out, st);
}

template <typename R>
static int energy_t(FdtdPlan *p, const FdtdBuffers *b, double *scratch, int nblk, double *out,
                    cudaStream_t st)
{
    EnergyK<R> k;
    k.E = (const R *)b->E;
    k.H = (const R *)b->H;
    k.eps = (const R *)b->eps;
    k.mu = p->d.has_mu ? (const R *)b->mu : nullptr;
    k.partial = scratch;
    k.n = 3 * p->N;
    return check_cuda(launch_energy<R>(k, nblk, out, st), "energy launch");
}

extern "C" {

int fdtd_energy(FdtdPlan *p, const FdtdBuffers *b, double *scratch, int32_t scratch_len,
                double *out, void *stream)
{
    int rc = check_common(p, b);
    if (rc) return rc;
    if (!b->E || !b->H || !b->eps) return fail(FDTD_ERR_INVALID, "energy: E, H and eps are required");
    if (p->d.has_mu && !b->mu) return fail(FDTD_ERR_INVALID, "energy: mu is required");
    if (!scratch || !out || scratch_len < 1) return fail(FDTD_ERR_INVALID, "energy: scratch and out are required");
    const int nblk = scratch_len < 1024 ? scratch_len : 1024;
    cudaStream_t st = (cudaStream_t)stream;
    return p->d.dtype == FDTD_F64 ? energy_t<double>(p, b, scratch, nblk, out, st)
                                  : energy_t<float>(p, b, scratch, nblk, out, st);
}

}  // extern "C"

template <typename R>
static int count_nonfinite_t(FdtdPlan *p, const FdtdBuffers *b, uint32_t *count, cudaStream_t st)
{
    int rc = check_cuda(cudaMemsetAsync(count, 0, sizeof(uint32_t), st), "watchdog clear");
    const void *fields[4] = {b->E, b->H, p->d.n_bloch ? b->F : nullptr, p->d.n_bloch ? b->G : nullptr};
    for (int f = 0; !rc && f < 4; ++f)
        if (fields[f])
            rc = check_cuda(launch_count_nonfinite<R>((const R *)fields[f], 3 * p->N, (unsigned int *)count, st),
                            "watchdog launch");
    return rc;
}

extern "C" {

int fdtd_count_nonfinite(FdtdPlan *p, const FdtdBuffers *b, uint32_t *count, void *stream)
{
    int rc = check_common(p, b);
    if (rc) return rc;
    if (!b->E || !b->H) return fail(FDTD_ERR_INVALID, "count_nonfinite: E and H are required");
    if (p->d.n_bloch && (!b->F || !b->G)) return fail(FDTD_ERR_INVALID, "count_nonfinite: F and G are required");
    if (!count) return fail(FDTD_ERR_INVALID, "count_nonfinite: count is NULL");
    cudaStream_t st = (cudaStream_t)stream;
    return p->d.dtype == FDTD_F64 ? count_nonfinite_t<double>(p, b, count, st) : count_nonfinite_t<float>(p, b, count, st);
}

int fdtd_run(FdtdPlan *p, const FdtdBuffers *b, void *stream, int32_t nsteps,
             const FdtdPointSources *src, FdtdDftMonitor *mon)
{
    int rc = check_common(p, b);
    if (rc) return rc;
    if (nsteps < 0) return fail(FDTD_ERR_INVALID, "fdtd_run: nsteps must be >= 0");
    if (src && src->n > 0 && (!src->index || !src->values))
        return fail(FDTD_ERR_INVALID, "fdtd_run: source index/values pointer is NULL");
    if (src && src->n > MAX_POINT_SOURCES)
        return fail(FDTD_ERR_INVALID, "fdtd_run: at most 64 point sources");
    for (int s = 0; src && s < src->n; ++s)
        if (src->index[s] < 0 || (uint64_t)src->index[s] >= 3 * p->N)
            return fail(FDTD_ERR_INVALID, "fdtd_run: point source index out of range");
    if ((rc = check_monitor(p, mon))) return rc;
    const bool f64 = p->d.dtype == FDTD_F64;
    if (!b->E2 && hs_eligible(p, b)) {
        if ((rc = check_run_buffers(p, b))) return rc;
        cudaStream_t st = (cudaStream_t)stream;
        p->last_run_path = FDTD_PATH_HS;
        rc = f64 ? run_hs<double>(p, b, st, nsteps, src, mon) : run_hs<float>(p, b, st, nsteps, src, mon);
        if (!rc && mon) { mon->step += nsteps; mon->series_row += nsteps; }
        return rc;
    }
    if (!p->lbc_mask && fused_eligible(p, b, src)) {
        if ((rc = check_psi(p, b->psi_e, "fdtd_run")) || (rc = check_psi(p, b->psi_h, "fdtd_run")))
            return rc;
        cudaStream_t st = (cudaStream_t)stream;
        p->last_run_path = FDTD_PATH_ONEPASS;
        rc = f64 ? run_fused<double>(p, b, st, nsteps, src, mon) : run_fused<float>(p, b, st, nsteps, src, mon);
        if (!rc && mon) { mon->step += nsteps; mon->series_row += nsteps; }
        return rc;
    }
    // validate once with the per-update entry points' checks, then run the slab schedule
    if ((rc = check_run_buffers(p, b))) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    p->last_run_path = FDTD_PATH_PER_UPDATE;
    rc = f64 ? run_slabs<double>(p, b, st, nsteps, src, mon) : run_slabs<float>(p, b, st, nsteps, src, mon);
    if (!rc && mon) { mon->step += nsteps; mon->series_row += nsteps; }
    return rc;
}

int fdtd_device_status(FdtdPlan *p, void *stream, int32_t *bits)
{
    if (!p || !bits) return fail(FDTD_ERR_INVALID, "fdtd_device_status: NULL pointer");
    cudaStream_t st = (cudaStream_t)stream;
    int32_t v = 0;
    int rc = check_cuda(cudaMemcpyAsync(&v, p->status, sizeof(v), cudaMemcpyDeviceToHost, st), "status read");
    if (!rc) rc = check_cuda(cudaMemsetAsync(p->status, 0, sizeof(v), st), "status clear");
    if (!rc) rc = check_cuda(cudaStreamSynchronize(st), "status sync");
    if (rc) return rc;
    *bits = v;
    if (v)
        return fail(FDTD_ERR_WATCHDOG, "a bounded wait inside a kernel ran out (status bits " + std::to_string(v) + ")");
    return FDTD_OK;
}

int fdtd_run_kernel_ms(const FdtdPlan *p, double ms[2], int32_t *samples)
{
    if (!p || !ms || !samples) return fail(FDTD_ERR_INVALID, "fdtd_run_kernel_ms: NULL pointer");
    ms[0] = p->kernel_ms[0];
    ms[1] = p->kernel_ms[1];
    *samples = p->kernel_samples;
    return FDTD_OK;
}

}  // extern "C"
