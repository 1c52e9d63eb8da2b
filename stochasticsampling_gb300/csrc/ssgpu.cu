// ssgpu.cu -- the simulation context and the C ABI declared in include/ssgpu.h.
//
// ss_ctx mirrors the reference's Simulation (src/bin/simulation/mod.rs:60-77):
// it owns the particle state, the distribution (as an integer histogram), the
// spectral solvers (cuFFT plans + k-space kernel) and the per-cell field table,
// all resident in HBM.  Host code here only validates, allocates, launches and
// copies; every arithmetic stage runs in kernels.cu.
#include <cufft.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "../../include/ssgpu.h"
#include "kernels.cuh"
#include "denoiser.cuh"
#include "mixed.cuh"

using namespace ss;

namespace {

constexpr int kLutN = 4096;

thread_local std::string g_last_error;

struct Timing {
    bool on = false;
    cudaEvent_t ev[SS_NUM_STAGES + 1] = {};
    double ms[SS_NUM_STAGES] = {};
    uint64_t steps = 0;
};

}  // namespace

namespace ss {
// context-free error text for entry points outside this file
void record_error(const char *msg) { g_last_error = msg; }
}  // namespace ss

// ss_step_host splits the update and the read-back into this many chunks
constexpr int kHostChunks = 16;

struct ss_ctx {
    ss_grid grid{};
    ss_box box{};
    ss_params prm{};
    uint32_t flags = 0;
    DevParams P{};
    int device = 0;
    int sms = 1;  // multiprocessors of the device
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    bool q2d = false, mag_step = false, sort = true, use_graph = true;
    uint32_t resort_every = 0;  // re-sort by cell every this many steps (0: never; ss_set_resort)
    uint64_t launches_graph[2] = {};  // kernel launches of a captured step without / with the re-sort
    bool initialized = false;
    uint64_t timestep = 0;
    int pcur = 0, ccur = 0, dist_idx = 0;
    bool fields_mag_valid = false;  // inverse buffer holds B of the last solve
    bool solved = false;            // a step ran since the last init
    double screening_last = 0.0;    // the screening of the last flow solve (for the complex getters)

    double *px[2][5] = {};
    uint32_t *key[2] = {}, *pid[2] = {};
    uint32_t *counts[2] = {};
    // FP64 field solve: real fields -> half spectra -> real fields
    double *fr = nullptr;                   // contraction output, [12][ncell] real
    double2 *fwd = nullptr, *invh = nullptr;  // half spectra [12][nhalf], [24][nhalf]
    double *ir = nullptr;                   // the step's real fields [24][ncell] (the table's input)
    double2 *inv = nullptr;  // complex fields [24][ncell] for the getters (FP64: on demand; mixed: widened)
    double *table = nullptr;
    double *ctab = nullptr;  // canonical quasi-2-D rows (CT_*), FP64 quasi2d contexts
    uint32_t *cellcount = nullptr, *cursor = nullptr;
    double *kern = nullptr, *lut = nullptr;
    float *kslice = nullptr;    // the angle kernels as 12-bit integer slices (FP64 contraction)
    double *kfactor = nullptr;  // per component: 2^(E_j - 48) * measure * V / D
    double *staging = nullptr, *noise_dev = nullptr, *dist_dev = nullptr, *realbuf = nullptr;
    double *staging_sorted = nullptr;  // the rows in cell order before the ingest
    unsigned long long *d_step = nullptr;
    uint32_t *d_err = nullptr;
    unsigned long long *d_scan = nullptr;  // row validation: first non-finite particle, non-canonical flag
    double *d_halfpi = nullptr;

    // FP32 mixed-precision mode (SS_FLAG_MIXED)
    bool mixed = false;
    bool fixed = false;  // positions in 64-bit fixed point (SS_FLAG_FIXED64)
    // learned denoiser between the histogram and the stress contraction (mixed quasi2d only)
    ss_dn *dn = nullptr;
    float *dn_x = nullptr, *dn_y = nullptr;
    float dn_inv_mean = 0.f, dn_fscale = 0.f;
    bool canon = false;  // quasi2d: z == 0 and theta == pi/2 hold for every particle
    MixedParams M{};
    float *pa[2][2] = {};  // phi, theta (FP32)
    float *fr_f = nullptr, *ir_f = nullptr, *ii_f = nullptr;  // real fields [12][ncell], [24][ncell], imaginary parts
    float2 *fwd_f = nullptr, *inv_f = nullptr;               // half spectra [12][nhalf], [24][nhalf]
    float *table_f = nullptr, *kern_f = nullptr;
    double *sums = nullptr;  // FP64 per-component sums for the mean handling
    float2 *partials = nullptr;  // per-block float-pair component sums of the FP32 contraction (+ its counter)
    unsigned *partials_done = nullptr;
    // the TMA-staged FP32 contraction: tensor maps of both histograms and of
    // the denoised distribution, and the angle kernels as [angle][12]
    CUtensorMap tmap_counts[2];
    CUtensorMap tmap_dist;
    bool tma = false, tma_dist = false;
    float *kern_t = nullptr;
    bool wide_valid = false;  // inv (FP64) holds the widened mixed fields
    std::map<int, cufftHandle> plans_c;  // key: batch * 4 + kind (1 R2C, 2 C2R)

    std::map<int, cufftHandle> plans;  // key: batch * 4 + kind (0 Z2Z, 1 D2Z, 2 Z2D)
    int fft_rank = 0;
    int fft_n[3] = {1, 1, 1};

    cudaGraphExec_t graph[2][2][2] = {};  // [particle buffer][histogram][the step re-sorts]
    // ss_step_host: a copy stream and one event per chunk of the read-back
    cudaStream_t copy_stream = nullptr;
    cudaEvent_t chunk_ev[kHostChunks + 1] = {};
    uint64_t h_step = 0;  // host source of the step counter copy
    uint32_t *counts_in = nullptr;  // histogram of rows being loaded, until they are accepted
    // ss_output_begin / ss_output_wait: two device slots, each a copy of one
    // step's outputs, drained into host buffers on the output stream
    struct OutSlot {
        double *dist = nullptr, *fields = nullptr, *rows = nullptr;  // [nbins], [6][ncell] (flow, B), [n][5]
        cudaEvent_t ready = nullptr, done = nullptr;  // taken on the step stream, landed on the output stream
        uint32_t *h_err = nullptr;  // page-locked copy of the device error word at the snapshot
        bool pending = false;
    } out[2];
    cudaStream_t out_stream = nullptr;
    uint64_t launches = 0;
    uint64_t launches_per_step = 0;
    Timing timing;
    std::string err;
};

// the FP32 contraction's per-block component sums and, after them, its counter
static size_t partials_bytes(uint64_t ncell, int sms) {
    return (12ull * contract_m_blocks((int)ncell, sms) + 1) * sizeof(float2);
}

// ---------------------------------------------------------------------------
// error helpers
// ---------------------------------------------------------------------------
static int fail(ss_ctx *c, int code, const char *fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    if (c) c->err = buf;
    g_last_error = buf;
    return code;
}

#define CK(call)                                                                                    \
    do {                                                                                            \
        cudaError_t e_ = (call);                                                                    \
        if (e_ != cudaSuccess) return fail(c, SS_ERR_CUDA, "%s: %s", #call, cudaGetErrorString(e_)); \
    } while (0)
#define CKF(call)                                                                     \
    do {                                                                              \
        cufftResult r_ = (call);                                                      \
        if (r_ != CUFFT_SUCCESS) return fail(c, SS_ERR_CUFFT, "%s: cufft error %d", #call, (int)r_); \
    } while (0)
#define CKR(expr)                   \
    do {                            \
        int rc_ = (expr);           \
        if (rc_ != SS_OK) return rc_; \
    } while (0)

static int check_launch(ss_ctx *c, const char *what) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail(c, SS_ERR_CUDA, "launch of %s: %s", what, cudaGetErrorString(e));
    return SS_OK;
}

// ---------------------------------------------------------------------------
// angle kernels (init only): stress_kernel (src/flowfield/stress.rs:29-56)
// with the closure of src/bin/simulation/mod.rs:100-104, and
// orientation_kernel (src/polarization/director.rs:69-92).  Angles at cell
// centres by ndarray's linspace: start + step * i, step = (end-start)/(n-1).
// ---------------------------------------------------------------------------
static double linspace_at(double a, double b, uint64_t n, uint64_t i) {
    double step = (n > 1) ? (b - a) / ((double)n - 1.0) : 0.0;
    return a + step * (double)i;
}

static double host_modulo(double f, double m) {
    double r = std::fmod(f, m);
    return r < 0.0 ? r + std::fabs(m) : r;
}

void ss::build_angle_kernels(const ss_grid &grid, const ss_params &prm, std::vector<double> &K) {
    const uint64_t gp = grid.phi, gt = grid.theta, na = gp * gt;
    const double gwp = kTwoPi / (double)gp, gwt = kPi / (double)gt;
    const double hp = gwp / 2., ht = gwt / 2.;
    K.assign(12 * na, 0.0);
    for (uint64_t i = 0; i < gp; ++i) {
        double phi = linspace_at(0. + hp, kTwoPi - hp, gp, i);
        for (uint64_t j = 0; j < gt; ++j) {
            double theta = linspace_at(0. + ht, kPi - ht, gt, j);
            double cp = std::cos(phi), sp = std::sin(phi), ct = std::cos(theta), st = std::sin(theta);
            // stress_active (stress.rs:103-119)
            double sa[9] = {-(1. / 3.) + cp * cp * st * st, cp * st * st * sp, ct * cp * st,
                            cp * st * st * sp, -(1. / 3.) + st * st * sp * sp, ct * st * sp,
                            ct * cp * st, ct * st * sp, -(1. / 3.) + ct * ct};
            // stress_magnetic (stress.rs:125-141), field along y
            double sm[9] = {0., cp * st, 0., -cp * st, 0., -ct, 0., ct, 0.};
            // stress_magnetic_rods (stress.rs:144-159)
            double c2p = std::cos(2. * phi), c2t = std::cos(2. * theta), s2t = std::sin(2. * theta);
            double sr[9] = {2. * ct * (cp * cp) * (st * st), ct * (st * st) * c2p, c2t * cp * st,
                            ct * (st * st) * c2p, st * s2t * (sp * sp), c2t * st * sp,
                            c2t * cp * st, c2t * st * sp, -2. * ct * (st * st)};
            for (int k = 0; k < 9; ++k) {
                sm[k] = sm[k] * 0.5;
                sr[k] = sr[k] * 0.5;
                K[k * na + i * gt + j] =
                    prm.stress_active * sa[k] + prm.stress_magnetic * sm[k] + prm.shape * sr[k];
            }
            // orientation kernel: Orientation::new (ang_pbc) then to_vector
            double th = host_modulo(theta, kTwoPi), ph;
            if (th > kPi) {
                ph = host_modulo(phi + kPi, kTwoPi);
                th = kTwoPi - th;
            } else {
                ph = host_modulo(phi, kTwoPi);
            }
            double ocp = std::cos(ph), osp = std::sin(ph), oct = std::cos(th), ost = std::sin(th);
            K[9 * na + i * gt + j] = ost * ocp;
            K[10 * na + i * gt + j] = ost * osp;
            K[11 * na + i * gt + j] = oct;
        }
    }
}

// ---------------------------------------------------------------------------
// cuFFT plans (c2c Z2Z, unnormalised; the FFTW plans of
// spectral_solver.rs:44-68 and magnetic_solver.rs:38-52).  Axes of length 1
// are dropped: they do not change the memory layout of [comp][x][y][z].
// ---------------------------------------------------------------------------
// real-to-complex (D2Z) and complex-to-real (Z2D) plans, out of place: the
// real fields [batch][ncell] and their half spectra [batch][nhalf]
static int get_plan(ss_ctx *c, int batch, int kind, cufftHandle *out) {
    const int key = batch * 4 + kind;
    auto it = c->plans.find(key);
    if (it != c->plans.end()) {
        *out = it->second;
        return SS_OK;
    }
    cufftHandle h;
    const int nc = c->P.ncell, nh = c->P.nhalf, cs = c->P.cstride;
    int rn[3], hn[3];  // the real and the half-spectrum shapes
    for (int k = 0; k < c->fft_rank; ++k) rn[k] = hn[k] = c->fft_n[k];
    hn[c->fft_rank - 1] = c->fft_n[c->fft_rank - 1] / 2 + 1;
    if (kind == 1)  // input components cstride apart (16-byte aligned starts)
        CKF(cufftPlanMany(&h, c->fft_rank, c->fft_n, rn, 1, cs, hn, 1, nh, CUFFT_D2Z, batch));
    else
        CKF(cufftPlanMany(&h, c->fft_rank, c->fft_n, hn, 1, nh, rn, 1, nc, CUFFT_Z2D, batch));
    CKF(cufftSetStream(h, c->stream));
    c->plans[key] = h;
    *out = h;
    return SS_OK;
}

// forward: real fields src [batch][ncell] -> half spectra dst [batch][nhalf]
static int fft_r2c(ss_ctx *c, const double *src, double2 *dst, int batch) {
    if (batch == 0) return SS_OK;
    if (c->fft_rank == 0) {  // 1-cell grid: the DFT is the identity
        launch_real_to_complex(c->stream, src, batch, c->P.cstride, dst);
        return check_launch(c, "real_to_complex");
    }
    cufftHandle h = 0;
    CKR(get_plan(c, batch, 1, &h));
    CKF(cufftExecD2Z(h, const_cast<cufftDoubleReal *>(src), reinterpret_cast<cufftDoubleComplex *>(dst)));
    return SS_OK;
}

// inverse: half spectra src [batch][nhalf] (overwritten) -> real fields dst [batch][ncell]
static int fft_c2r(ss_ctx *c, double2 *src, double *dst, int batch) {
    if (batch == 0) return SS_OK;
    if (c->fft_rank == 0) {
        launch_complex_to_real(c->stream, src, batch, dst);
        return check_launch(c, "complex_to_real");
    }
    cufftHandle h = 0;
    CKR(get_plan(c, batch, 2, &h));
    CKF(cufftExecZ2D(h, reinterpret_cast<cufftDoubleComplex *>(src), dst));
    return SS_OK;
}

// the FP32 real-to-complex (R2C) and complex-to-real (C2R) plans of the mixed path
static int get_plan_c(ss_ctx *c, int batch, int kind, cufftHandle *out) {
    const int key = batch * 4 + kind;
    auto it = c->plans_c.find(key);
    if (it != c->plans_c.end()) {
        *out = it->second;
        return SS_OK;
    }
    cufftHandle h;
    const int nc = c->P.ncell, nh = c->P.nhalf, cs = c->P.cstride;
    int rn[3], hn[3];
    for (int k = 0; k < c->fft_rank; ++k) rn[k] = hn[k] = c->fft_n[k];
    hn[c->fft_rank - 1] = c->fft_n[c->fft_rank - 1] / 2 + 1;
    if (kind == 1)
        CKF(cufftPlanMany(&h, c->fft_rank, c->fft_n, rn, 1, cs, hn, 1, nh, CUFFT_R2C, batch));
    else
        CKF(cufftPlanMany(&h, c->fft_rank, c->fft_n, hn, 1, nh, rn, 1, nc, CUFFT_C2R, batch));
    CKF(cufftSetStream(h, c->stream));
    c->plans_c[key] = h;
    *out = h;
    return SS_OK;
}

static int fft_r2c_f(ss_ctx *c, const float *src, float2 *dst, int batch) {
    if (batch == 0) return SS_OK;
    if (c->fft_rank == 0) {
        launch_real_to_complex_f(c->stream, src, batch, c->P.cstride, dst);
        return check_launch(c, "real_to_complex (mixed)");
    }
    cufftHandle h = 0;
    CKR(get_plan_c(c, batch, 1, &h));
    CKF(cufftExecR2C(h, const_cast<cufftReal *>(src), reinterpret_cast<cufftComplex *>(dst)));
    return SS_OK;
}

static int fft_c2r_f(ss_ctx *c, float2 *src, float *dst, int batch) {
    if (batch == 0) return SS_OK;
    if (c->fft_rank == 0) {
        launch_complex_to_real_f(c->stream, src, batch, dst);
        return check_launch(c, "complex_to_real (mixed)");
    }
    cufftHandle h = 0;
    CKR(get_plan_c(c, batch, 2, &h));
    CKF(cufftExecC2R(h, reinterpret_cast<cufftComplex *>(src), dst));
    return SS_OK;
}

// ---------------------------------------------------------------------------
// timing helpers
// ---------------------------------------------------------------------------
static void mark(ss_ctx *c, int stage) {
    if (c->timing.on) cudaEventRecord(c->timing.ev[stage], c->stream);
}

// ---------------------------------------------------------------------------
// the field solve: contraction -> FFT -> k space -> inverse FFT -> table
// ---------------------------------------------------------------------------
static int enqueue_solve(ss_ctx *c, bool flow, bool mag, const uint32_t *counts, const double *dist, double screening,
                         int pcur, bool sort_now, uint64_t *nl) {
    const int ts = (c->mag_step || c->P.gather) ? TABLE_STRIDE_MAG : TABLE_STRIDE;
    mark(c, 0);
    if (dist)
        launch_contract(c->stream, flow, mag, counts, dist, c->lut, kLutN, c->kern, c->P, c->fr, c->table, ts,
                        c->cellcount);
    else
        launch_contract_x(c->stream, flow, mag, counts, c->kslice, c->kfactor, c->kern, c->lut, kLutN, c->P, c->fr,
                          c->table, ts, c->cellcount);
    ++*nl;
    CKR(check_launch(c, "contract"));
    mark(c, 6);
    if (sort_now) {
        launch_scan(c->stream, c->cellcount, c->P.ncell, c->cursor);
        launch_scatter(c->stream, c->P.n, c->px[pcur], c->key[pcur], c->pid[pcur], c->px[1 - pcur],
                       c->key[1 - pcur], c->pid[1 - pcur], c->cursor);
        *nl += 2;
        CKR(check_launch(c, "sort"));
    }
    mark(c, 1);
    const long long nc = c->P.ncell, nh = c->P.nhalf;
    if (flow && mag) CKR(fft_r2c(c, c->fr, c->fwd, 12));
    else if (flow) CKR(fft_r2c(c, c->fr, c->fwd, 9));
    else CKR(fft_r2c(c, c->fr + 9ll * c->P.cstride, c->fwd + 9 * nh, 3));
    mark(c, 2);
    launch_kspace(c->stream, flow, mag, false, c->fwd, c->invh, c->P, screening);
    ++*nl;
    CKR(check_launch(c, "kspace"));
    mark(c, 3);
    if (flow && mag) CKR(fft_c2r(c, c->invh, c->ir, 24));
    else if (flow) CKR(fft_c2r(c, c->invh, c->ir, 12));
    else CKR(fft_c2r(c, c->invh + 12 * nh, c->ir + 12 * nc, 12));
    if (flow) c->screening_last = screening;
    mark(c, 4);
    // the table has rows for the dipolar terms only when the step uses them
    const bool table_mag = mag && c->mag_step;
    if (flow || table_mag) {
        launch_table(c->stream, flow, table_mag, c->ir, c->P, c->table, ts,
                     (flow && !table_mag && !c->P.gather) ? c->ctab : nullptr);
        ++*nl;
        CKR(check_launch(c, "table"));
    }
    return SS_OK;
}

// The mixed-precision field solve (mixed.cu): FP32 contraction with FP64
// component sums, means removed in FP64, C2C FP32 transforms, FP32 k space.
// sort_pcur >= 0: the step also re-sorts the particles of buffer set
// sort_pcur into the other set (between the contraction and the transforms,
// where the per-stage timing puts the FP64 path's sort)
static int enqueue_solve_m(ss_ctx *c, bool flow, bool mag, const uint32_t *counts, double screening, uint64_t *nl,
                           int sort_pcur = -1) {
    const int ts = c->mag_step ? TABLE_STRIDE_MAG : TABLE_STRIDE;
    const int nc = c->P.ncell;
    mark(c, 0);
    if (c->dn && flow) {
        // the denoised histogram replaces the counts in the contraction
        launch_counts_to_unit(c->stream, counts, c->P.nbins, c->dn_inv_mean, c->dn_x);
        *nl += 1 + dn_enqueue_forward(c->dn, c->dn_x, c->dn_y, c->stream);
        launch_contract_m(c->stream, flow, mag, counts, c->kern_f, c->M, c->fr_f, c->table_f, ts, c->partials,
                          c->partials_done, c->sums, c->sms, c->dn_y, c->dn_fscale,
                          c->tma_dist ? &c->tmap_dist : nullptr, c->kern_t, c->d_err);
    } else {
        const CUtensorMap *tm = !c->tma ? nullptr : (counts == c->counts[0] ? &c->tmap_counts[0]
                                                   : counts == c->counts[1] ? &c->tmap_counts[1] : nullptr);
        launch_contract_m(c->stream, flow, mag, counts, c->kern_f, c->M, c->fr_f, c->table_f, ts, c->partials,
                          c->partials_done, c->sums, c->sms, nullptr, 0.f, tm, c->kern_t, c->d_err);
    }
    if (flow) launch_center_m(c->stream, c->fr_f, 0, 9, nc, c->P.cstride, c->sums);
    if (mag) launch_center_m(c->stream, c->fr_f, 9, 12, nc, c->P.cstride, c->sums);
    *nl += 1 + (flow ? 1 : 0) + (mag ? 1 : 0);
    CKR(check_launch(c, "contract (mixed)"));
    mark(c, 6);
    if (sort_pcur >= 0) {
        const int a = sort_pcur, b = 1 - sort_pcur;
        launch_resort_m(c->stream, c->M, c->px[a], c->pa[a], c->key[a], c->pid[a], c->px[b], c->pa[b], c->key[b],
                        c->pid[b], c->cellcount, c->cursor);
        *nl += 4;
        CKR(check_launch(c, "re-sort (mixed)"));
    }
    mark(c, 1);
    const long long nh = c->P.nhalf;
    if (flow && mag) CKR(fft_r2c_f(c, c->fr_f, c->fwd_f, 12));
    else if (flow) CKR(fft_r2c_f(c, c->fr_f, c->fwd_f, 9));
    else CKR(fft_r2c_f(c, c->fr_f + 9ll * c->P.cstride, c->fwd_f + 9 * nh, 3));
    mark(c, 2);
    launch_kspace_m(c->stream, flow, mag, false, c->fwd_f, c->inv_f, c->M, (float)screening);
    ++*nl;
    CKR(check_launch(c, "kspace (mixed)"));
    mark(c, 3);
    if (flow && mag) CKR(fft_c2r_f(c, c->inv_f, c->ir_f, 24));
    else if (flow) CKR(fft_c2r_f(c, c->inv_f, c->ir_f, 12));
    else CKR(fft_c2r_f(c, c->inv_f + 12 * nh, c->ir_f + 12ll * nc, 12));
    if (flow) c->screening_last = screening;
    mark(c, 4);
    const bool table_mag = mag && c->mag_step;
    if (flow || table_mag) {
        launch_table_m(c->stream, flow, table_mag, c->ir_f, c->M, c->table_f, ts, c->sums);
        ++*nl;
        CKR(check_launch(c, "table (mixed)"));
    }
    c->wide_valid = false;
    return SS_OK;
}

static int enqueue_step_m(ss_ctx *c, int pcur, int ccur, bool host_noise, bool sort_now, uint64_t *nl) {
    CKR(enqueue_solve_m(c, true, c->mag_step, c->counts[ccur], c->prm.hydro_screening, nl, sort_now ? pcur : -1));
    const int p = sort_now ? 1 - pcur : pcur;
    mark(c, 5);
    launch_zero_u32(c->stream, c->counts[1 - ccur], c->P.nbins);
    launch_update_m(c->stream, c->fixed, c->q2d, c->canon, c->mag_step, host_noise, c->M, c->px[p], c->pa[p],
                    c->key[p], c->pid[p], c->table_f, c->noise_dev, c->d_step, c->counts[1 - ccur]);
    launch_step_inc(c->stream, c->d_step);
    *nl += 3;
    CKR(check_launch(c, "update (mixed)"));
    mark(c, 7);
    return SS_OK;
}

// One do_timestep for the state (pcur, ccur); does not touch host-side state.
static int enqueue_step(ss_ctx *c, int pcur, int ccur, bool host_noise, bool sort_now, uint64_t *nl) {
    if (c->mixed) return enqueue_step_m(c, pcur, ccur, host_noise, sort_now, nl);
    CKR(enqueue_solve(c, true, c->mag_step, c->counts[ccur], nullptr, c->prm.hydro_screening, pcur, sort_now, nl));
    const int p = sort_now ? 1 - pcur : pcur;
    mark(c, 5);
    launch_zero_u32(c->stream, c->counts[1 - ccur], c->P.nbins);
    launch_update(c->stream, c->q2d, c->canon, c->mag_step, host_noise, c->P, c->px[p], c->key[p], c->pid[p], c->table,
                  c->ctab, c->noise_dev, c->d_step, c->counts[1 - ccur], c->d_err);
    launch_step_inc(c->stream, c->d_step);
    *nl += 3;
    CKR(check_launch(c, "update"));
    mark(c, 7);
    return SS_OK;
}

static void advance(ss_ctx *c, bool sorted) {
    // a replayed graph does not run the host side of enqueue_solve_m: the
    // widened FP64 copy of the mixed fields is stale after every step
    c->wide_valid = false;
    if (sorted) c->pcur ^= 1;
    c->dist_idx = c->ccur;
    c->ccur ^= 1;
    c->timestep += 1;
    c->fields_mag_valid = c->mag_step;
    c->solved = true;
    // the first quasi2d step sets z = 0 and theta = pi/2 everywhere
    if (c->q2d) c->canon = true;
}

static void accumulate_timing(ss_ctx *c) {
    if (!c->timing.on) return;
    cudaEventSynchronize(c->timing.ev[7]);
    // stage intervals: 0->6 contract, 6->1 sort, 1->2 fft fwd, 2->3 kspace, 3->4 fft inv, 4->5 table, 5->7 update
    const int from[7] = {0, 6, 1, 2, 3, 4, 5};
    const int to[7] = {6, 1, 2, 3, 4, 5, 7};
    const int slot[7] = {0, 6, 1, 2, 3, 4, 5};
    for (int k = 0; k < 7; ++k) {
        float ms = 0.f;
        cudaEventElapsedTime(&ms, c->timing.ev[from[k]], c->timing.ev[to[k]]);
        c->timing.ms[slot[k]] += ms;
    }
    c->timing.steps += 1;
}

// whether this step counting-sorts the particles by cell before its update:
// every step for an FP64 context made with sorting, and every resort_every-th
// step (ss_set_resort) for the others
static bool sorts_now(const ss_ctx *c) {
    if (c->sort) return true;
    return c->resort_every > 0 && (c->timestep + 1) % c->resort_every == 0;
}

static int direct_step(ss_ctx *c, bool host_noise) {
    uint64_t nl = 0;
    const bool sort_now = sorts_now(c);
    CKR(enqueue_step(c, c->pcur, c->ccur, host_noise, sort_now, &nl));
    c->launches += nl;
    c->launches_per_step = nl;
    accumulate_timing(c);
    advance(c, sort_now);
    return SS_OK;
}

static int graph_step(ss_ctx *c) {
    // the step after non-canonical quasi2d rows runs directly (graphs hold the canonical update)
    if (c->q2d && !c->canon) return direct_step(c, false);
    const bool sort_now = sorts_now(c);
    cudaGraphExec_t &g = c->graph[c->pcur][c->ccur][sort_now];
    if (!g) {
        cudaGraph_t graph;
        uint64_t nl = 0;
        CK(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
        int rc = enqueue_step(c, c->pcur, c->ccur, false, sort_now, &nl);
        cudaError_t e = cudaStreamEndCapture(c->stream, &graph);
        if (rc != SS_OK) return rc;
        if (e != cudaSuccess) return fail(c, SS_ERR_CUDA, "graph capture: %s", cudaGetErrorString(e));
        e = cudaGraphInstantiate(&g, graph, 0);
        cudaGraphDestroy(graph);
        if (e != cudaSuccess) return fail(c, SS_ERR_CUDA, "graph instantiate: %s", cudaGetErrorString(e));
        c->launches_graph[sort_now] = nl;
    }
    CK(cudaGraphLaunch(g, c->stream));
    c->launches_per_step = c->launches_graph[sort_now];
    c->launches += c->launches_per_step;
    advance(c, sort_now);
    return SS_OK;
}

static int read_device_error(ss_ctx *c) {
    uint32_t e = 0;
    CK(cudaMemcpyAsync(&e, c->d_err, sizeof e, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    if (e & 0x100u) {
        CK(cudaMemsetAsync(c->d_err, 0, sizeof(uint32_t), c->stream));
        return fail(c, SS_ERR_CUDA, "a tensor-memory-accelerator copy of the contraction did not complete in time");
    }
    if (e) {
        return fail(c, SS_ERR_RANGE,
                    "device bounds check fired (flags %u): a particle coordinate was non-finite or outside the "
                    "box after wrapping",
                    e);
    }
    return SS_OK;
}

static bool is_finite(double v) { return std::isfinite(v); }

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------
extern "C" {

const char *ss_version(void) { return "ssgpu 0.1 (sm_103a)"; }

int ss_last_error(ss_ctx *ctx, char *buf, size_t len) {
    if (!buf || len == 0) return SS_ERR_INVALID_ARGUMENT;
    const std::string &s = ctx ? ctx->err : g_last_error;
    std::snprintf(buf, len, "%s", s.c_str());
    return SS_OK;
}

static void destroy_impl(ss_ctx *c) {
    if (!c) return;
    cudaSetDevice(c->device);
    if (c->stream) cudaStreamSynchronize(c->stream);
    for (auto &kv : c->plans) cufftDestroy(kv.second);
    for (auto &ga : c->graph)
        for (auto &gb : ga)
            for (auto &g : gb)
                if (g) cudaGraphExecDestroy(g);
    for (int b = 0; b < 2; ++b) {
        for (int k = 0; k < 5; ++k) cudaFree(c->px[b][k]);
        cudaFree(c->key[b]);
        cudaFree(c->pid[b]);
        cudaFree(c->counts[b]);
    }
    cudaFree(c->fr); cudaFree(c->fwd); cudaFree(c->invh); cudaFree(c->ir); cudaFree(c->inv); cudaFree(c->table); cudaFree(c->ctab); cudaFree(c->cellcount); cudaFree(c->cursor);
    cudaFree(c->kern); cudaFree(c->lut); cudaFree(c->staging); cudaFree(c->noise_dev); cudaFree(c->dist_dev);
    cudaFree(c->realbuf); cudaFree(c->staging_sorted); cudaFree(c->d_step); cudaFree(c->d_err); cudaFree(c->d_scan); cudaFree(c->d_halfpi);
    for (auto &kv : c->plans_c) cufftDestroy(kv.second);
    for (int b = 0; b < 2; ++b)
        for (int k = 0; k < 2; ++k) cudaFree(c->pa[b][k]);
    cudaFree(c->fr_f); cudaFree(c->ir_f); cudaFree(c->ii_f); cudaFree(c->fwd_f); cudaFree(c->inv_f); cudaFree(c->table_f); cudaFree(c->kern_f); cudaFree(c->partials); cudaFree(c->kern_t);
    cudaFree(c->kslice); cudaFree(c->kfactor);
    cudaFree(c->dn_x); cudaFree(c->dn_y);
    cudaFree(c->sums);
    for (auto &e : c->timing.ev)
        if (e) cudaEventDestroy(e);
    for (auto &e : c->chunk_ev)
        if (e) cudaEventDestroy(e);
    if (c->copy_stream) cudaStreamDestroy(c->copy_stream);
    cudaFree(c->counts_in);
    if (c->out_stream) cudaStreamSynchronize(c->out_stream);
    for (auto &o : c->out) {
        cudaFree(o.dist); cudaFree(o.fields); cudaFree(o.rows);
        if (o.ready) cudaEventDestroy(o.ready);
        if (o.done) cudaEventDestroy(o.done);
        if (o.h_err) cudaFreeHost(o.h_err);
    }
    if (c->out_stream) cudaStreamDestroy(c->out_stream);
    if (c->own_stream && c->stream) cudaStreamDestroy(c->stream);
    delete c;
}

int ss_destroy(ss_ctx *ctx) {
    destroy_impl(ctx);
    return SS_OK;
}

int ss_create(const ss_grid *grid, const ss_box *box, const ss_params *params, uint32_t flags, void *stream,
              ss_ctx **out) {
    ss_ctx *c = nullptr;
    if (!grid || !box || !params || !out) return fail(nullptr, SS_ERR_INVALID_ARGUMENT, "ss_create: null argument");
    *out = nullptr;
    const uint64_t lim = 1ull << 20;
    if (grid->x < 1 || grid->y < 1 || grid->z < 1 || grid->phi < 1 || grid->theta < 1 || grid->x > lim ||
        grid->y > lim || grid->z > lim || grid->phi > lim || grid->theta > lim)
        return fail(nullptr, SS_ERR_INVALID_ARGUMENT, "grid sizes must lie in [1, 2^20]");
    const uint64_t ncell = grid->x * grid->y * grid->z, nang = grid->phi * grid->theta;
    if (ncell > 0x7fffffffull || nang > 0x7fffffffull || ncell * nang > (1ull << 36))
        return fail(nullptr, SS_ERR_INVALID_ARGUMENT, "grid too large (cells %llu, angle bins %llu)",
                    (unsigned long long)ncell, (unsigned long long)nang);
    // check_settings (settings/mod.rs:185-205)
    if (!(box->x > 0.) || !(box->y > 0.) || !(box->z > 0.) || !is_finite(box->x) || !is_finite(box->y) ||
        !is_finite(box->z))
        return fail(nullptr, SS_ERR_INVALID_ARGUMENT, "Box size is invalid. Must be bigger than 0: (%g, %g, %g)",
                    box->x, box->y, box->z);
    if ((flags & SS_FLAG_QUASI2D) && grid->z != 1)
        return fail(nullptr, SS_ERR_INVALID_ARGUMENT,
                    "z-direction must only contain 1 cell if feature 'quasi2d' is activated.");
    if (params->number_of_particles < 1 || params->number_of_particles > 0xffffffffull)
        return fail(nullptr, SS_ERR_INVALID_ARGUMENT, "number_of_particles must lie in [1, 2^32-1]");
    const double vals[] = {params->timestep, params->trans_diffusion, params->rot_diffusion, params->stress_active,
                           params->stress_magnetic, params->shape, params->magnetic_drag, params->hydro_screening,
                           params->volume_exclusion, params->magnetic_reorientation,
                           params->magnetic_dipole_dipole};
    for (double v : vals)
        if (!is_finite(v)) return fail(nullptr, SS_ERR_INVALID_ARGUMENT, "parameters must be finite");
    if (params->rot_diffusion * params->timestep < 0.0)
        return fail(nullptr, SS_ERR_INVALID_ARGUMENT, "2 * rotational diffusion * timestep must be >= 0");

    c = new ss_ctx();
    c->grid = *grid;
    c->box = *box;
    c->prm = *params;
    c->flags = flags;
    c->q2d = (flags & SS_FLAG_QUASI2D) != 0;
    c->sort = (flags & SS_FLAG_NO_SORT) == 0;
    c->use_graph = (flags & SS_FLAG_NO_GRAPH) == 0;
    c->fixed = (flags & SS_FLAG_FIXED64) != 0;
    c->mixed = (flags & (SS_FLAG_MIXED | SS_FLAG_FIXED64)) != 0;
    if (c->mixed && (flags & (SS_FLAG_TRILINEAR | SS_FLAG_TRILINEAR_ZFROMY))) {
        destroy_impl(c);
        return fail(nullptr, SS_ERR_INVALID_ARGUMENT, "the trilinear gather is available in the FP64 mode only");
    }
    if (c->mixed && nang > 1024) {  // the FP32 contraction keeps 12 angle kernels in 48 KB of shared memory
        destroy_impl(c);
        return fail(nullptr, SS_ERR_INVALID_ARGUMENT, "the mixed-precision mode supports at most 1024 angle bins");
    }
    if (c->mixed && (flags & SS_FLAG_F32X2)) {
        destroy_impl(c);
        return fail(nullptr, SS_ERR_INVALID_ARGUMENT, "SS_FLAG_F32X2 applies to the FP64 mode only");
    }
    if (c->mixed) c->sort = false;
    c->mag_step = (flags & SS_FLAG_ALWAYS_MAGNETIC) || params->magnetic_dipole_dipole != 0.0 ||
                  params->magnetic_drag != 0.0;
    cudaError_t e = cudaGetDevice(&c->device);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&c->sms, cudaDevAttrMultiProcessorCount, c->device);
    if (e != cudaSuccess) {
        destroy_impl(c);
        return fail(nullptr, SS_ERR_CUDA, "cudaGetDevice: %s", cudaGetErrorString(e));
    }
    if (c->sms < 1) c->sms = 1;
    if (stream) {
        c->stream = (cudaStream_t)stream;
    } else {
        e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
        if (e != cudaSuccess) {
            destroy_impl(c);
            return fail(nullptr, SS_ERR_CUDA, "cudaStreamCreate: %s", cudaGetErrorString(e));
        }
        c->own_stream = true;
    }

    DevParams &P = c->P;
    P.gx = (int)grid->x; P.gy = (int)grid->y; P.gz = (int)grid->z; P.gphi = (int)grid->phi;
    P.gtheta = (int)grid->theta;
    P.ncell = (int)ncell;
    P.nang = (int)nang;
    P.nbins = (long long)(ncell * nang);
    P.n = params->number_of_particles;
    P.bx = box->x; P.by = box->y; P.bz = box->z;
    // GridWidth::new (src/mesh/grid_width.rs:23-31)
    P.gw[0] = box->x / (double)grid->x;
    P.gw[1] = box->y / (double)grid->y;
    P.gw[2] = box->z / (double)grid->z;
    P.gw[3] = kTwoPi / (double)grid->phi;
    P.gw[4] = kPi / (double)grid->theta;
    for (int k = 0; k < 5; ++k) P.igw[k] = 1.0 / P.gw[k];
    {  // FP32 first estimate of the bin index: the band where FP64 decides (ref_bin_f)
        const int nk[5] = {P.gx, P.gy, P.gz, P.gphi, P.gtheta};
        for (int k = 0; k < 5; ++k) {
            P.igwf[k] = (float)P.igw[k];
            P.bintol[k] = (float)(8.0 * 0x1p-24 * ((double)nk[k] + 1.0));
        }
    }
    P.dt = params->timestep;
    P.Dt = params->trans_diffusion;
    P.Dr = params->rot_diffusion;
    P.shape = params->shape;
    P.drag = params->magnetic_drag;
    P.reorient = params->magnetic_reorientation;
    P.shape_dt = params->shape * params->timestep;
    P.reorient_dt = params->magnetic_reorientation * params->timestep;
    P.mdd = params->magnetic_dipole_dipole;
    P.volex = params->volume_exclusion;
    P.dist_den = P.gw[0] * P.gw[1] * P.gw[2] * P.gw[3] * P.gw[4] * (double)P.n;
    P.volume = box->x * box->y * box->z;
    P.measure = P.gw[3] * P.gw[4];
    P.dthph = P.gw[4] * P.gw[3];
    P.sigma_rot = std::sqrt(2. * params->rot_diffusion * params->timestep);
    {  // float pairs (hi, lo) of the constants of the two-float chain
        const double v[6] = {P.dt, P.reorient_dt, P.sigma_rot, P.reorient, P.shape, P.drag};
        float *out[6] = {P.dt2, P.reorient2, P.sigma2, P.reorient_f2, P.shape2, P.drag2};
        for (int k = 0; k < 6; ++k) {
            out[k][0] = (float)v[k];
            out[k][1] = (float)(v[k] - (double)out[k][0]);
        }
    }
    P.f32x2 = (flags & SS_FLAG_F32X2) ? 1 : 0;
    P.seed = params->seed;
    P.quasi2d = c->q2d ? 1 : 0;
    {  // floor((pi/2) / gw_theta) with the n -> n-1 clamp: the bin ref_bin gives pi/2
        const double f = std::floor(kPiHalf / P.gw[4]);
        P.bin_theta_half = f >= (double)P.gtheta ? P.gtheta - 1 : (int)f;
    }
    P.gather = (flags & SS_FLAG_TRILINEAR_ZFROMY) ? 2 : (flags & SS_FLAG_TRILINEAR) ? 1 : 0;
    uint32_t mask = M_ALL;
    if (params->magnetic_reorientation == 0.0) mask &= ~M_EXTERNAL_FIELD;
    if (params->shape == 0.0) mask &= ~M_JEFFREY_STRAIN;
    if (!c->mag_step || params->magnetic_drag == 0.0) mask &= ~M_MDD_FORCE;
    if (!c->mag_step || params->magnetic_dipole_dipole == 0.0) mask &= ~M_MDD_ROTATION;
    P.mask = mask;
    if (c->mixed) {
        MixedParams &M = c->M;
        M.gx = P.gx; M.gy = P.gy; M.gz = P.gz; M.gphi = P.gphi; M.gtheta = P.gtheta;
        M.ncell = P.ncell; M.nang = P.nang; M.n = P.n;
        M.bx = P.bx; M.by = P.by; M.bz = P.bz;
        M.bx2 = 2.0 * P.bx; M.by2 = 2.0 * P.by; M.bz2 = 2.0 * P.bz;
        for (int k = 0; k < 5; ++k) M.igwf[k] = (float)(1.0 / P.gw[k]);
        const double L[3] = {P.bx, P.by, P.bz};
        for (int k = 0; k < 3; ++k) {
            M.gwf[k] = (float)P.gw[k];
            M.s32[k] = (float)(0x1p32 / L[k]);
            M.unit[k] = L[k] * 0x1p-64;
        }
        M.dist_den = P.dist_den; M.volume = P.volume;
        M.measure = (float)P.measure; M.dthph = (float)P.dthph; M.two_dt = (float)(2.0 * P.dt);
        M.Dt = (float)P.Dt; M.volex = (float)P.volex; M.dt = (float)P.dt;
        M.drag = (float)P.drag; M.reorient = (float)P.reorient; M.shape = (float)P.shape; M.mdd = (float)P.mdd;
        M.sigma_rot = (float)P.sigma_rot;
        M.seed = P.seed;
        M.mask = mask;
    }

    // FFT geometry: drop axes of length 1; the real-to-complex transforms
    // halve the last remaining axis
    {
        int dims[3] = {P.gx, P.gy, P.gz}, r = 0;
        for (int k = 0; k < 3; ++k)
            if (dims[k] > 1) c->fft_n[r++] = dims[k];
        c->fft_rank = r;
        for (int k = 2; k >= 0; --k)
            if (dims[k] > 1) {
                dims[k] = dims[k] / 2 + 1;
                break;
            }
        for (int k = 0; k < 3; ++k) P.hdim[k] = c->M.hdim[k] = dims[k];
        P.nhalf = c->M.nhalf = dims[0] * dims[1] * dims[2];
        P.cstride = c->M.cstride = P.ncell + (P.ncell & 1);
    }

    auto alloc = [&](void **p, size_t bytes) -> int {
        cudaError_t err = cudaMalloc(p, bytes ? bytes : 16);
        if (err != cudaSuccess)
            return fail(c, SS_ERR_CUDA, "cudaMalloc(%zu bytes): %s", bytes, cudaGetErrorString(err));
        return SS_OK;
    };
    int rc = SS_OK;
    const size_t N = (size_t)P.n;
    const int nbuf = c->sort ? 2 : 1;
    for (int b = 0; b < nbuf && rc == SS_OK; ++b) {
        const int nd = c->mixed ? 3 : 5;  // mixed: x, y, z in FP64, phi, theta in FP32
        for (int k = 0; k < nd && rc == SS_OK; ++k) rc = alloc((void **)&c->px[b][k], N * sizeof(double));
        for (int k = 0; c->mixed && k < 2 && rc == SS_OK; ++k) rc = alloc((void **)&c->pa[b][k], N * sizeof(float));
        if (rc == SS_OK) rc = alloc((void **)&c->key[b], N * sizeof(uint32_t));
        if (rc == SS_OK) rc = alloc((void **)&c->pid[b], N * sizeof(uint32_t));
    }
    for (int b = 0; b < 2 && rc == SS_OK; ++b) rc = alloc((void **)&c->counts[b], (size_t)P.nbins * sizeof(uint32_t));
    const size_t nhalf = (size_t)P.nhalf;
    if (!c->mixed) {
        if (rc == SS_OK) rc = alloc((void **)&c->fr, 12 * (size_t)P.cstride * sizeof(double));
        if (rc == SS_OK) rc = alloc((void **)&c->fwd, 12 * nhalf * sizeof(double2));
        if (rc == SS_OK) rc = alloc((void **)&c->invh, 24 * nhalf * sizeof(double2));
        if (rc == SS_OK) rc = alloc((void **)&c->ir, 24 * ncell * sizeof(double));
    }
    if (rc == SS_OK) rc = alloc((void **)&c->inv, 24 * ncell * sizeof(double2));
    if (rc == SS_OK) rc = alloc((void **)&c->table, ncell * TABLE_STRIDE_MAG * sizeof(double));
    if (rc == SS_OK && c->q2d && !c->mixed) rc = alloc((void **)&c->ctab, ncell * CTAB_STRIDE * sizeof(double));
    if (rc == SS_OK) rc = alloc((void **)&c->cellcount, ncell * sizeof(uint32_t));
    if (rc == SS_OK) rc = alloc((void **)&c->cursor, ncell * sizeof(uint32_t));
    if (rc == SS_OK) rc = alloc((void **)&c->kern, 12 * nang * sizeof(double));
    if (rc == SS_OK) rc = alloc((void **)&c->lut, kLutN * sizeof(double));
    if (rc == SS_OK) rc = alloc((void **)&c->kslice, 48 * nang * sizeof(float));
    if (rc == SS_OK) rc = alloc((void **)&c->kfactor, 12 * sizeof(double));
    if (rc == SS_OK) rc = alloc((void **)&c->staging, 5 * N * sizeof(double));
    if (rc == SS_OK) rc = alloc((void **)&c->d_step, sizeof(unsigned long long));
    if (rc == SS_OK) rc = alloc((void **)&c->d_err, sizeof(uint32_t));
    if (rc == SS_OK) rc = alloc((void **)&c->d_scan, 2 * sizeof(unsigned long long));
    if (rc == SS_OK) rc = alloc((void **)&c->d_halfpi, 2 * sizeof(double));
    if (c->mixed) {
        if (rc == SS_OK) rc = alloc((void **)&c->fr_f, 12 * (size_t)P.cstride * sizeof(float));
        if (rc == SS_OK) rc = alloc((void **)&c->ir_f, 24 * ncell * sizeof(float));
        if (rc == SS_OK) rc = alloc((void **)&c->fwd_f, 12 * nhalf * sizeof(float2));
        if (rc == SS_OK) rc = alloc((void **)&c->inv_f, 24 * nhalf * sizeof(float2));
        if (rc == SS_OK) rc = alloc((void **)&c->table_f, ncell * TABLE_STRIDE_MAG * sizeof(float));
        if (rc == SS_OK) rc = alloc((void **)&c->kern_f, 12 * nang * sizeof(float));
        if (rc == SS_OK) rc = alloc((void **)&c->sums, 12 * sizeof(double));
        if (rc == SS_OK) rc = alloc((void **)&c->partials, partials_bytes(ncell, c->sms));
        if (rc == SS_OK) rc = alloc((void **)&c->kern_t, ((nang + 31) / 32 * 32) * 12 * sizeof(float));
    }
    if (rc != SS_OK) {
        std::string m = c->err;
        destroy_impl(c);
        return fail(nullptr, rc, "%s", m.c_str());
    }
#define CKC(call)                                                                                     \
    do {                                                                                              \
        cudaError_t e_ = (call);                                                                      \
        if (e_ != cudaSuccess) {                                                                      \
            std::string m_ = std::string(#call) + ": " + cudaGetErrorString(e_);                      \
            destroy_impl(c);                                                                          \
            return fail(nullptr, SS_ERR_CUDA, "%s", m_.c_str());                                      \
        }                                                                                             \
    } while (0)
    if (!c->mixed) {
        CKC(cudaMemsetAsync(c->fr, 0, 12 * (size_t)P.cstride * sizeof(double), c->stream));
        CKC(cudaMemsetAsync(c->fwd, 0, 12 * nhalf * sizeof(double2), c->stream));
        CKC(cudaMemsetAsync(c->ir, 0, 24 * ncell * sizeof(double), c->stream));
    }
    CKC(cudaMemsetAsync(c->inv, 0, 24 * ncell * sizeof(double2), c->stream));
    CKC(cudaMemsetAsync(c->table, 0, ncell * TABLE_STRIDE_MAG * sizeof(double), c->stream));
    CKC(cudaMemsetAsync(c->counts[0], 0, (size_t)P.nbins * sizeof(uint32_t), c->stream));
    CKC(cudaMemsetAsync(c->counts[1], 0, (size_t)P.nbins * sizeof(uint32_t), c->stream));
    CKC(cudaMemsetAsync(c->d_step, 0, sizeof(unsigned long long), c->stream));
    CKC(cudaMemsetAsync(c->d_err, 0, sizeof(uint32_t), c->stream));

    std::vector<double> K;
    build_angle_kernels(c->grid, c->prm, K);
    std::vector<double> lut(kLutN);
    for (int i = 0; i < kLutN; ++i) lut[i] = ((double)i / P.dist_den) * P.volume;
    CKC(cudaMemcpyAsync(c->kern, K.data(), K.size() * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    CKC(cudaMemcpyAsync(c->lut, lut.data(), lut.size() * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    std::vector<float> slices;
    std::vector<double> factor;
    kernel_slices(K, (int)nang, P.measure * (P.volume / P.dist_den), slices, factor);
    CKC(cudaMemcpyAsync(c->kslice, slices.data(), slices.size() * sizeof(float), cudaMemcpyHostToDevice, c->stream));
    CKC(cudaMemcpyAsync(c->kfactor, factor.data(), factor.size() * sizeof(double), cudaMemcpyHostToDevice,
                        c->stream));
    std::vector<float> Kf(K.begin(), K.end());
    if (c->mixed) {
        CKC(cudaMemsetAsync(c->ir_f, 0, 24 * ncell * sizeof(float), c->stream));
        CKC(cudaMemsetAsync(c->sums, 0, 12 * sizeof(double), c->stream));
        CKC(cudaMemsetAsync(c->partials, 0, partials_bytes(ncell, c->sms), c->stream));
        c->partials_done = reinterpret_cast<unsigned *>(c->partials + 12ull * contract_m_blocks((int)ncell, c->sms));
        CKC(cudaMemcpyAsync(c->kern_f, Kf.data(), Kf.size() * sizeof(float), cudaMemcpyHostToDevice, c->stream));
        std::vector<float> Kt;
        kernel_transposed(K, (int)nang, Kt);
        CKC(cudaMemcpyAsync(c->kern_t, Kt.data(), Kt.size() * sizeof(float), cudaMemcpyHostToDevice, c->stream));
        c->tma = contract_tma_fits((int)nang) &&
                 make_bins_tmap(&c->tmap_counts[0], c->counts[0], (int)ncell, (int)nang) &&
                 make_bins_tmap(&c->tmap_counts[1], c->counts[1], (int)ncell, (int)nang);
    }
    CKC(contract_prepare());
    launch_half_pi(c->stream, c->d_halfpi);
    double hp[2];
    CKC(cudaMemcpyAsync(hp, c->d_halfpi, sizeof hp, cudaMemcpyDeviceToHost, c->stream));
    CKC(cudaStreamSynchronize(c->stream));
    P.cos_half_pi = hp[0];
    P.sin_half_pi = hp[1];
    for (auto &ev : c->timing.ev) CKC(cudaEventCreate(&ev));
#undef CKC
    // plans for the step
    {
        cufftHandle h;
        int r1 = SS_OK, r2 = SS_OK;
        if (c->fft_rank > 0) {
            r1 = c->mixed ? get_plan_c(c, c->mag_step ? 12 : 9, 1, &h) : get_plan(c, c->mag_step ? 12 : 9, 1, &h);
            r2 = (r1 == SS_OK) ? (c->mixed ? get_plan_c(c, c->mag_step ? 24 : 12, 2, &h)
                                           : get_plan(c, c->mag_step ? 24 : 12, 2, &h))
                               : r1;
        }
        if (r1 != SS_OK || r2 != SS_OK) {
            std::string m = c->err;
            destroy_impl(c);
            return fail(nullptr, SS_ERR_CUFFT, "%s", m.c_str());
        }
    }
    *out = c;
    return SS_OK;
}

static int ingest_staging(ss_ctx *c, uint64_t n, bool canon);

static int load_particles(ss_ctx *c, const double *particles, uint64_t n) {
    if (!particles) return fail(c, SS_ERR_INVALID_ARGUMENT, "particles is NULL");
    if (n != c->P.n)
        return fail(c, SS_ERR_PARTICLE_COUNT,
                    "Given initial condition has not the same number of particles (%llu) as given in the "
                    "parameter file (%llu).",
                    (unsigned long long)n, (unsigned long long)c->P.n);
    CK(cudaSetDevice(c->device));
    CK(cudaMemcpyAsync(c->staging, particles, 5 * n * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    // the rows are checked on the device (finite; canonical quasi2d state)
    // before they replace the particle state
    static const unsigned long long scan_init[2] = {~0ull, 0ull};
    unsigned long long scan[2];
    CK(cudaMemcpyAsync(c->d_scan, scan_init, sizeof scan_init, cudaMemcpyHostToDevice, c->stream));
    launch_scan_rows(c->stream, c->staging, n, c->d_scan);
    CKR(check_launch(c, "scan_rows"));
    CK(cudaMemcpyAsync(scan, c->d_scan, sizeof scan, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    if (scan[0] != ~0ull)
        return fail(c, SS_ERR_INVALID_ARGUMENT, "particle %llu has a non-finite coordinate", scan[0]);
    return ingest_staging(c, n, c->q2d && scan[1] == 0ull);
}

// the rows in `staging` become the particle state: Particle::new, then the
// first histogram (Simulation::init, src/bin/simulation/mod.rs:163-196)
static int ingest_staging(ss_ctx *c, uint64_t n, bool canon) {
    c->pcur = 0;
    c->ccur = 0;
    // Rows in cell order (locality of the update's gathers and atomics); pid gets their caller
    // indices.  Every mixed context sorts; an FP64 context sorts only on a 3-D grid, whose
    // histogram outgrows L2 (the 2-D FP64 update is bound by the FP64 pipe, not by those
    // accesses, and the sort would only slow ss_resume).
    const bool sort_rows = c->mixed || c->P.gz > 1;
    if (sort_rows) {
        if (!c->staging_sorted) CK(cudaMalloc((void **)&c->staging_sorted, 5 * (size_t)n * sizeof(double)));
        launch_sort_rows(c->stream, c->staging, n, c->P, c->key[0], c->cellcount, c->cursor, c->staging_sorted,
                         c->pid[0]);
        c->launches += 4;
    }
    const double *rows = sort_rows ? c->staging_sorted : c->staging;
    if (c->mixed) {
        launch_ingest_m(c->stream, c->fixed, rows, n, c->P, c->M, c->px[0], c->pa[0], nullptr);
        launch_zero_u32(c->stream, c->counts[0], c->P.nbins);
        launch_bin_m(c->stream, c->fixed, n, c->M, c->px[0], c->pa[0], c->key[0], c->counts[0]);
        // quasi2d: the canonical state (z = 0, theta = pi/2) lets the update skip z and theta
        c->canon = canon;
        c->launches += 3;
    } else {
        launch_zero_u32(c->stream, c->counts[0], c->P.nbins);
        launch_ingest_bin(c->stream, canon, rows, n, c->P, c->px[0], sort_rows ? nullptr : c->pid[0], c->key[0],
                          c->counts[0], c->d_err);
        c->canon = canon;
        c->launches += 2;
    }
    CKR(check_launch(c, "init"));
    c->dist_idx = 0;
    c->fields_mag_valid = false;
    c->solved = false;
    c->initialized = true;
    CK(cudaStreamSynchronize(c->stream));
    return SS_OK;
}

int ss_init(ss_ctx *c, const double *particles, uint64_t n) {
    if (!c) return fail(nullptr, SS_ERR_INVALID_ARGUMENT, "null context");
    CKR(load_particles(c, particles, n));
    c->timestep = 0;
    CK(cudaMemsetAsync(c->d_step, 0, sizeof(unsigned long long), c->stream));
    CK(cudaStreamSynchronize(c->stream));
    return SS_OK;
}

int ss_resume(ss_ctx *c, const double *particles, uint64_t n, uint64_t timestep) {
    if (!c) return fail(nullptr, SS_ERR_INVALID_ARGUMENT, "null context");
    CKR(load_particles(c, particles, n));
    c->timestep = timestep;
    unsigned long long t = timestep;
    CK(cudaMemcpyAsync(c->d_step, &t, sizeof t, cudaMemcpyHostToDevice, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    return SS_OK;
}

int ss_init_distribution(ss_ctx *c, uint32_t kind) {
    if (!c) return fail(nullptr, SS_ERR_INVALID_ARGUMENT, "null context");
    if (kind > 1) return fail(c, SS_ERR_INVALID_ARGUMENT, "unknown initial distribution %u", kind);
    double kappa = 0.0;
    if (kind == 1) {
        // init.rs:103-110: kappa = magnetic_reorientation / rotational diffusion
        kappa = c->prm.magnetic_reorientation / c->prm.rot_diffusion;
        if (kappa == 0.0)
            return fail(c, SS_ERR_INVALID_ARGUMENT,
                        "Alignment of zero is the isotropic state. Please use that instead.");
        if (!is_finite(kappa)) return fail(c, SS_ERR_INVALID_ARGUMENT, "alignment kappa is not finite");
    }
    CK(cudaSetDevice(c->device));
    CK(cudaMemsetAsync(c->d_err, 0, sizeof(uint32_t), c->stream));
    launch_sample_initial(c->stream, kind == 1, c->P, kappa, c->staging, c->d_err);
    c->launches += 1;
    CKR(check_launch(c, "sample_initial"));
    uint32_t e = 0;
    CK(cudaMemcpyAsync(&e, c->d_err, sizeof e, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    if (e) return fail(c, SS_ERR_RANGE, "Caution, the alignment parameter is too high for the given precision.");
    CKR(ingest_staging(c, c->P.n, false));
    c->timestep = 0;
    CK(cudaMemsetAsync(c->d_step, 0, sizeof(unsigned long long), c->stream));
    CK(cudaStreamSynchronize(c->stream));
    return SS_OK;
}

int ss_do_timestep(ss_ctx *c, const double *noise, uint64_t *timestep_out) {
    if (!c) return fail(nullptr, SS_ERR_INVALID_ARGUMENT, "null context");
    if (!c->initialized) return fail(c, SS_ERR_STATE, "ss_do_timestep before ss_init");
    CK(cudaSetDevice(c->device));
    if (noise) {
        if (!c->noise_dev) CK(cudaMalloc((void **)&c->noise_dev, 5 * (size_t)c->P.n * sizeof(double)));
        CK(cudaMemcpyAsync(c->noise_dev, noise, 5 * (size_t)c->P.n * sizeof(double), cudaMemcpyHostToDevice,
                           c->stream));
        CKR(direct_step(c, true));
        // the caller may reuse its noise buffer once this returns
        CK(cudaStreamSynchronize(c->stream));
    } else if (c->use_graph && !c->timing.on) {
        CKR(graph_step(c));
    } else {
        CKR(direct_step(c, false));
    }
    if (timestep_out) *timestep_out = c->timestep;
    return SS_OK;
}

int ss_run(ss_ctx *c, uint64_t steps, uint64_t *timestep_out) {
    if (!c) return fail(nullptr, SS_ERR_INVALID_ARGUMENT, "null context");
    if (!c->initialized) return fail(c, SS_ERR_STATE, "ss_run before ss_init");
    CK(cudaSetDevice(c->device));
    for (uint64_t s = 0; s < steps; ++s) {
        if (c->use_graph && !c->timing.on) CKR(graph_step(c));
        else CKR(direct_step(c, false));
    }
    if (timestep_out) *timestep_out = c->timestep;
    return SS_OK;
}

int ss_noise(ss_ctx *c, uint64_t timestep, double *out) {
    if (!c || !out) return fail(c, SS_ERR_INVALID_ARGUMENT, "null argument");
    CK(cudaSetDevice(c->device));
    if (c->mixed) launch_noise_m(c->stream, c->q2d, c->M, timestep, c->staging);
    else launch_noise(c->stream, c->q2d, c->P, timestep, c->staging);
    c->launches += 1;
    CKR(check_launch(c, "noise"));
    CK(cudaMemcpyAsync(out, c->staging, 5 * (size_t)c->P.n * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    return SS_OK;
}

int ss_synchronize(ss_ctx *c) {
    if (!c) return fail(nullptr, SS_ERR_INVALID_ARGUMENT, "null context");
    CK(cudaStreamSynchronize(c->stream));
    if (c->dn) CKR(dn_status(c->dn, c->stream));
    return read_device_error(c);
}

int ss_set_denoiser(ss_ctx *c, ss_dn *dn) {
    if (!c) return fail(nullptr, SS_ERR_INVALID_ARGUMENT, "null context");
    CK(cudaSetDevice(c->device));
    CK(cudaStreamSynchronize(c->stream));
    if (dn) {
        int nx, ny, np;
        dn_shape(dn, &nx, &ny, &np);
        if (!c->mixed || !c->q2d || c->P.gz != 1 || c->P.gtheta != 1)
            return fail(c, SS_ERR_INVALID_ARGUMENT, "the denoiser needs a quasi2d mixed-precision context");
        if (nx != c->P.gx || ny != c->P.gy || np != c->P.gphi)
            return fail(c, SS_ERR_INVALID_ARGUMENT, "denoiser grid %dx%dx%d differs from the histogram's %dx%dx%d", nx,
                        ny, np, c->P.gx, c->P.gy, c->P.gphi);
        if (!c->dn_x) {
            CK(cudaMalloc((void **)&c->dn_x, (size_t)c->P.nbins * sizeof(float)));
            CK(cudaMalloc((void **)&c->dn_y, (size_t)c->P.nbins * sizeof(float)));
            c->tma_dist = c->tma && make_bins_tmap(&c->tmap_dist, c->dn_y, c->P.ncell, c->P.nang);
        }
        const double mean = (double)c->P.n / (double)c->P.nbins;  // counts per bin
        c->dn_inv_mean = (float)(1.0 / mean);
        c->dn_fscale = (float)(mean / c->P.dist_den * c->P.volume);
    }
    c->dn = dn;
    // the captured steps change: recapture on the next step
    for (auto &ga : c->graph)
        for (auto &gb : ga)
            for (auto &g : gb)
                if (g) {
                    cudaGraphExecDestroy(g);
                    g = nullptr;
                }
    return SS_OK;
}

int ss_get_particles(ss_ctx *c, double *out, uint64_t n) {
    if (!c || !out) return fail(c, SS_ERR_INVALID_ARGUMENT, "null argument");
    if (!c->initialized) return fail(c, SS_ERR_STATE, "no particles before ss_init");
    if (n > c->P.n) return fail(c, SS_ERR_INVALID_ARGUMENT, "asked for %llu of %llu particles",
                                (unsigned long long)n, (unsigned long long)c->P.n);
    CK(cudaSetDevice(c->device));
    if (c->mixed)
        launch_egest_m(c->stream, c->fixed, c->P.n, c->M, c->px[c->pcur], c->pa[c->pcur], c->pid[c->pcur], c->staging);
    else launch_egest(c->stream, c->P.n, c->px[c->pcur], c->pid[c->pcur], c->staging);
    c->launches += 1;
    CKR(check_launch(c, "egest"));
    CK(cudaMemcpyAsync(out, c->staging, 5 * n * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    return read_device_error(c);
}

static int ensure_host_pipeline(ss_ctx *c);

// One step of host-resident particles: the rows of `in` replace the state
// (ss_resume at the current step), one do_timestep, the new state into
// `out`.  The update runs in chunks; each chunk is laid out as rows and
// copied back on a second stream while the next chunk updates, so the
// read-back hides behind the update.  The step does not sort (sorting
// changes no result): the particles stay in the caller's order.
static int step_host_fp64(ss_ctx *c, double *out) {
    CKR(ensure_host_pipeline(c));
    uint64_t nl = 0;
    const int p = c->pcur, cc = c->ccur;
    CKR(enqueue_solve(c, true, c->mag_step, c->counts[cc], nullptr, c->prm.hydro_screening, p, false, &nl));
    launch_zero_u32(c->stream, c->counts[1 - cc], c->P.nbins);
    ++nl;
    const unsigned long long n = c->P.n;
    const unsigned long long chunk = ((n + kHostChunks - 1) / kHostChunks + 255) / 256 * 256;
    for (int k = 0; k < kHostChunks; ++k) {
        const unsigned long long off = (unsigned long long)k * chunk;
        if (off >= n) break;
        const unsigned long long cnt = (n - off < chunk) ? n - off : chunk;
        DevParams Pk = c->P;
        Pk.n = cnt;
        double *xs[5];
        for (int d = 0; d < 5; ++d) xs[d] = c->px[p][d] + off;
        launch_update(c->stream, c->q2d, c->canon, c->mag_step, false, Pk, xs, c->key[p] + off, c->pid[p] + off,
                      c->table, c->ctab, c->noise_dev, c->d_step, c->counts[1 - cc], c->d_err);
        // the ids are the identity after the ingest: chunk k fills rows off .. off + cnt
        launch_egest(c->stream, cnt, xs, c->pid[p] + off, c->staging);
        nl += 2;
        CKR(check_launch(c, "update (host step)"));
        CK(cudaEventRecord(c->chunk_ev[k], c->stream));
        CK(cudaStreamWaitEvent(c->copy_stream, c->chunk_ev[k], 0));
        CK(cudaMemcpyAsync(out + 5 * off, c->staging + 5 * off, 5 * cnt * sizeof(double), cudaMemcpyDeviceToHost,
                           c->copy_stream));
    }
    launch_step_inc(c->stream, c->d_step);
    ++nl;
    CK(cudaEventRecord(c->chunk_ev[kHostChunks], c->copy_stream));
    CK(cudaStreamWaitEvent(c->stream, c->chunk_ev[kHostChunks], 0));
    CK(cudaStreamSynchronize(c->stream));
    c->launches += nl;
    advance(c, false);
    return read_device_error(c);
}

static int ensure_host_pipeline(ss_ctx *c) {
    if (!c->copy_stream) CK(cudaStreamCreateWithFlags(&c->copy_stream, cudaStreamNonBlocking));
    for (auto &e : c->chunk_ev)
        if (!e) CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    return SS_OK;
}

// ss_resume's load for ss_step_host (FP64 path): the upload runs in chunks
// on the copy stream and each chunk is checked, sanitised and binned as soon
// as it lands, into the particle buffer the state does not use and a
// separate histogram.  Only when every row is finite do they become the
// state, so rejected rows leave it untouched, as in ss_resume.
static int load_host_fp64(ss_ctx *c, const double *in, uint64_t n) {
    if (!in) return fail(c, SS_ERR_INVALID_ARGUMENT, "particles is NULL");
    if (n != c->P.n)
        return fail(c, SS_ERR_PARTICLE_COUNT,
                    "Given initial condition has not the same number of particles (%llu) as given in the "
                    "parameter file (%llu).",
                    (unsigned long long)n, (unsigned long long)c->P.n);
    CKR(ensure_host_pipeline(c));
    const int alt = 1 - c->pcur;
    const size_t N = (size_t)n;
    // each missing buffer on its own, so that a failed call leaves nothing half-made for the next
    for (int k = 0; k < 5; ++k)
        if (!c->px[alt][k]) CK(cudaMalloc((void **)&c->px[alt][k], N * sizeof(double)));
    if (!c->key[alt]) CK(cudaMalloc((void **)&c->key[alt], N * sizeof(uint32_t)));
    if (!c->pid[alt]) CK(cudaMalloc((void **)&c->pid[alt], N * sizeof(uint32_t)));
    if (!c->counts_in) CK(cudaMalloc((void **)&c->counts_in, (size_t)c->P.nbins * sizeof(uint32_t)));
    static const unsigned long long scan_init[2] = {~0ull, 0ull};
    unsigned long long scan[2];
    CK(cudaMemcpyAsync(c->d_scan, scan_init, sizeof scan_init, cudaMemcpyHostToDevice, c->stream));
    launch_zero_u32(c->stream, c->counts_in, c->P.nbins);
    // the upload must not overwrite the staging rows before earlier work on the stream is done
    CK(cudaEventRecord(c->chunk_ev[kHostChunks], c->stream));
    CK(cudaStreamWaitEvent(c->copy_stream, c->chunk_ev[kHostChunks], 0));
    const unsigned long long chunk = ((N + kHostChunks - 1) / kHostChunks + 255) / 256 * 256;
    uint64_t nl = 1;
    for (int k = 0; k < kHostChunks; ++k) {
        const unsigned long long off = (unsigned long long)k * chunk;
        if (off >= N) break;
        const unsigned long long cnt = (N - off < chunk) ? N - off : chunk;
        CK(cudaMemcpyAsync(c->staging + 5 * off, in + 5 * off, 5 * cnt * sizeof(double), cudaMemcpyHostToDevice,
                           c->copy_stream));
        CK(cudaEventRecord(c->chunk_ev[k], c->copy_stream));
        CK(cudaStreamWaitEvent(c->stream, c->chunk_ev[k], 0));
        double *xs[5];
        for (int d = 0; d < 5; ++d) xs[d] = c->px[alt][d] + off;
        launch_ingest_bin_check(c->stream, c->staging + 5 * off, cnt, off, c->P, xs, c->pid[alt] + off,
                                c->key[alt] + off, c->counts_in, c->d_scan, c->d_err);
        ++nl;
        CKR(check_launch(c, "ingest (host step)"));
    }
    CK(cudaMemcpyAsync(scan, c->d_scan, sizeof scan, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    c->launches += nl;
    if (scan[0] != ~0ull)
        return fail(c, SS_ERR_INVALID_ARGUMENT, "particle %llu has a non-finite coordinate", scan[0]);
    // accept: the loaded rows are the state, their histogram the first one (Simulation::init)
    CK(cudaMemcpyAsync(c->counts[0], c->counts_in, (size_t)c->P.nbins * sizeof(uint32_t), cudaMemcpyDeviceToDevice,
                       c->stream));
    c->pcur = alt;
    c->ccur = 0;
    c->dist_idx = 0;
    c->canon = c->q2d && scan[1] == 0ull;
    c->fields_mag_valid = false;
    c->solved = false;
    c->initialized = true;
    return SS_OK;
}

int ss_step_host(ss_ctx *c, const double *in, double *out, uint64_t n, uint64_t *timestep_out) {
    if (!c) return fail(nullptr, SS_ERR_INVALID_ARGUMENT, "null context");
    if (!out) return fail(c, SS_ERR_INVALID_ARGUMENT, "out is NULL");
    CK(cudaSetDevice(c->device));
    // the pipelined form for the FP64 path; the mixed path, and a context recording per-stage
    // times (whose stage events the chunked step does not set), run the three calls in sequence
    const bool fused = !c->mixed && !c->timing.on;
    if (fused) CKR(load_host_fp64(c, in, n));
    else CKR(load_particles(c, in, n));
    c->h_step = c->timestep;
    CK(cudaMemcpyAsync(c->d_step, &c->h_step, sizeof c->h_step, cudaMemcpyHostToDevice, c->stream));
    if (!fused) {
        CKR(direct_step(c, false));
        CKR(ss_get_particles(c, out, n));
    } else {
        CKR(step_host_fp64(c, out));
    }
    if (timestep_out) *timestep_out = c->timestep;
    return SS_OK;
}

int ss_get_counts(ss_ctx *c, uint32_t *out) {
    if (!c || !out) return fail(c, SS_ERR_INVALID_ARGUMENT, "null argument");
    CK(cudaSetDevice(c->device));
    CK(cudaMemcpyAsync(out, c->counts[c->dist_idx], (size_t)c->P.nbins * sizeof(uint32_t), cudaMemcpyDeviceToHost,
                       c->stream));
    CK(cudaStreamSynchronize(c->stream));
    return read_device_error(c);
}

int ss_get_distribution(ss_ctx *c, double *out) {
    if (!c || !out) return fail(c, SS_ERR_INVALID_ARGUMENT, "null argument");
    CK(cudaSetDevice(c->device));
    if (!c->dist_dev) CK(cudaMalloc((void **)&c->dist_dev, (size_t)c->P.nbins * sizeof(double)));
    launch_counts_to_dist(c->stream, c->counts[c->dist_idx], c->P, c->dist_dev);
    c->launches += 1;
    CKR(check_launch(c, "counts_to_dist"));
    CK(cudaMemcpyAsync(out, c->dist_dev, (size_t)c->P.nbins * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    return read_device_error(c);
}

// the real fields of the last solve, components comp0 .. comp0 + comps, to
// host memory (the mixed path's widened fields, or the FP64 solve's own)
static int widen_fields(ss_ctx *c);
static int copy_real(ss_ctx *c, int comp0, int comps, double *out) {
    const long long nc = c->P.ncell, cnt = (long long)comps * nc;
    if (c->mixed) {
        CKR(widen_fields(c));
        if (!c->realbuf) CK(cudaMalloc((void **)&c->realbuf, 24ull * c->P.ncell * sizeof(double)));
        launch_real_parts(c->stream, c->inv + comp0 * nc, cnt, c->realbuf);
        c->launches += 1;
        CKR(check_launch(c, "real_parts"));
        CK(cudaMemcpyAsync(out, c->realbuf, cnt * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    } else {
        CK(cudaMemcpyAsync(out, c->ir + comp0 * nc, cnt * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    }
    CK(cudaStreamSynchronize(c->stream));
    return SS_OK;
}

// FP64 contexts: the complex fields of the last solve, as the reference's
// complex inverse gives them, into inv [comp][cell]: the real parts are the
// solve's own; the imaginary parts are the complex-to-real transform of the
// operators' anti-Hermitian part (zero away from Nyquist bins), from the
// half spectra that are still resident.
static int complex_fields(ss_ctx *c, bool flow) {
    if (c->mixed) return widen_fields(c);
    const long long nc = c->P.ncell, nh = c->P.nhalf;
    const int c0 = flow ? 0 : 12;
    if (!c->realbuf) CK(cudaMalloc((void **)&c->realbuf, 24ull * c->P.ncell * sizeof(double)));
    launch_kspace(c->stream, flow, !flow, true, c->fwd, c->invh, c->P, flow ? c->screening_last : 0.0);
    CKR(check_launch(c, "kspace (imaginary parts)"));
    CKR(fft_c2r(c, c->invh + c0 * nh, c->realbuf + c0 * nc, 12));
    launch_combine_complex(c->stream, c->ir + c0 * nc, c->realbuf + c0 * nc, 12 * nc, c->inv + c0 * nc);
    c->launches += 2;
    return check_launch(c, "combine_complex");
}

// The dipolar field of the last solve, computed on demand when the step
// skipped it (its couplings are zero).  The histogram it is built from is
// still resident, so the result equals what the step would have produced.
static int ensure_magnetic(ss_ctx *c) {
    if (c->fields_mag_valid) return SS_OK;
    if (!c->initialized || !c->solved) return SS_OK;  // nothing solved yet: zeros, like the reference
    uint64_t nl = 0;
    int pc = c->pcur;
    if (c->mixed) CKR(enqueue_solve_m(c, false, true, c->counts[c->dist_idx], 0.0, &nl));
    else CKR(enqueue_solve(c, false, true, c->counts[c->dist_idx], nullptr, 0.0, pc, false, &nl));
    c->launches += nl;
    c->fields_mag_valid = true;
    return SS_OK;
}

// mixed mode: the FP32 fields widened into the FP64 buffer the getters read,
// with the FP64 mean dipolar field added back; the imaginary parts (the
// reference's complex inverse) from the anti-Hermitian part of the operators,
// as for the FP64 path
static int widen_fields(ss_ctx *c) {
    if (!c->mixed || c->wide_valid) return SS_OK;
    const long long nc = c->P.ncell, nh = c->P.nhalf;
    if (!c->ii_f) CK(cudaMalloc((void **)&c->ii_f, 24ull * c->P.ncell * sizeof(float)));
    launch_kspace_m(c->stream, true, false, true, c->fwd_f, c->inv_f, c->M, (float)c->screening_last);
    CKR(check_launch(c, "kspace (mixed, imaginary parts)"));
    CKR(fft_c2r_f(c, c->inv_f, c->ii_f, 12));
    if (c->mag_step || c->fields_mag_valid) {
        launch_kspace_m(c->stream, false, true, true, c->fwd_f, c->inv_f, c->M, 0.f);
        CKR(check_launch(c, "kspace (mixed, imaginary parts)"));
        CKR(fft_c2r_f(c, c->inv_f + 12 * nh, c->ii_f + 12 * nc, 12));
    } else {
        CK(cudaMemsetAsync(c->ii_f + 12 * nc, 0, 12 * nc * sizeof(float), c->stream));
    }
    launch_widen_m(c->stream, c->ir_f, c->ii_f, 24ll * nc, (int)nc, 0, 21, 24, c->sums, c->inv);
    c->launches += 3;
    CKR(check_launch(c, "widen"));
    c->wide_valid = true;
    return SS_OK;
}

int ss_get_flow_field(ss_ctx *c, double *out) {
    if (!c || !out) return fail(c, SS_ERR_INVALID_ARGUMENT, "null argument");
    CK(cudaSetDevice(c->device));
    return copy_real(c, 9, 3, out);
}

int ss_get_magnetic_field(ss_ctx *c, double *out) {
    if (!c || !out) return fail(c, SS_ERR_INVALID_ARGUMENT, "null argument");
    CK(cudaSetDevice(c->device));
    CKR(ensure_magnetic(c));
    return copy_real(c, 21, 3, out);
}

int ss_get_flow_complex(ss_ctx *c, double *u, double *grad) {
    if (!c) return fail(nullptr, SS_ERR_INVALID_ARGUMENT, "null context");
    CK(cudaSetDevice(c->device));
    CKR(complex_fields(c, true));
    const size_t nc = c->P.ncell;
    if (u) CK(cudaMemcpyAsync(u, c->inv + 9 * nc, 3 * nc * sizeof(double2), cudaMemcpyDeviceToHost, c->stream));
    if (grad) CK(cudaMemcpyAsync(grad, c->inv, 9 * nc * sizeof(double2), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    return SS_OK;
}

int ss_get_magnetic_complex(ss_ctx *c, double *b, double *gradb) {
    if (!c) return fail(nullptr, SS_ERR_INVALID_ARGUMENT, "null context");
    CK(cudaSetDevice(c->device));
    CKR(ensure_magnetic(c));
    CKR(complex_fields(c, false));
    const size_t nc = c->P.ncell;
    if (b) CK(cudaMemcpyAsync(b, c->inv + 21 * nc, 3 * nc * sizeof(double2), cudaMemcpyDeviceToHost, c->stream));
    if (gradb) CK(cudaMemcpyAsync(gradb, c->inv + 12 * nc, 9 * nc * sizeof(double2), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    return SS_OK;
}

int ss_get_timestep(ss_ctx *c, uint64_t *out) {
    if (!c || !out) return fail(c, SS_ERR_INVALID_ARGUMENT, "null argument");
    *out = c->timestep;
    return SS_OK;
}

// the device error word as read_device_error reports it, from a copy taken
// without waiting for the step stream
static int report_error_word(ss_ctx *c, uint32_t e) {
    if (e & 0x100u)
        return fail(c, SS_ERR_CUDA, "a tensor-memory-accelerator copy of the contraction did not complete in time");
    if (e)
        return fail(c, SS_ERR_RANGE,
                    "device bounds check fired (flags %u): a particle coordinate was non-finite or outside the "
                    "box after wrapping",
                    e);
    return SS_OK;
}

int ss_output_begin(ss_ctx *c, int slot, double *dist, double *flow, double *mag, double *particles, uint64_t n) {
    if (!c) return fail(nullptr, SS_ERR_INVALID_ARGUMENT, "null context");
    if (slot < 0 || slot > 1) return fail(c, SS_ERR_INVALID_ARGUMENT, "output slot %d is not 0 or 1", slot);
    if (!c->initialized) return fail(c, SS_ERR_STATE, "no outputs before ss_init");
    if (particles && n > c->P.n)
        return fail(c, SS_ERR_INVALID_ARGUMENT, "asked for %llu of %llu particles", (unsigned long long)n,
                    (unsigned long long)c->P.n);
    ss_ctx::OutSlot &o = c->out[slot];
    if (o.pending) return fail(c, SS_ERR_STATE, "output slot %d is still in flight: ss_output_wait first", slot);
    CK(cudaSetDevice(c->device));
    if (!c->out_stream) CK(cudaStreamCreateWithFlags(&c->out_stream, cudaStreamNonBlocking));
    if (!o.ready) CK(cudaEventCreateWithFlags(&o.ready, cudaEventDisableTiming));
    if (!o.done) CK(cudaEventCreateWithFlags(&o.done, cudaEventDisableTiming));
    if (!o.h_err) CK(cudaHostAlloc((void **)&o.h_err, sizeof(uint32_t), cudaHostAllocDefault));
    const size_t nc = c->P.ncell;
    // the snapshot, on the step stream: after the steps queued so far, before any queued later
    if (dist) {
        if (!o.dist) CK(cudaMalloc((void **)&o.dist, (size_t)c->P.nbins * sizeof(double)));
        launch_counts_to_dist(c->stream, c->counts[c->dist_idx], c->P, o.dist);
        c->launches += 1;
        CKR(check_launch(c, "counts_to_dist"));
    }
    if (flow || mag) {
        if (!o.fields) CK(cudaMalloc((void **)&o.fields, 6 * nc * sizeof(double)));
        if (mag) CKR(ensure_magnetic(c));
        if (c->mixed) CKR(widen_fields(c));
        for (int f = 0; f < 2; ++f) {
            if (!(f == 0 ? flow : mag)) continue;
            const size_t comp0 = f == 0 ? 9 : 21;
            if (c->mixed) {
                launch_real_parts(c->stream, c->inv + comp0 * nc, 3ll * (long long)nc, o.fields + 3 * f * nc);
                c->launches += 1;
                CKR(check_launch(c, "real_parts"));
            } else {
                CK(cudaMemcpyAsync(o.fields + 3 * f * nc, c->ir + comp0 * nc, 3 * nc * sizeof(double),
                                   cudaMemcpyDeviceToDevice, c->stream));
            }
        }
    }
    if (particles && n) {
        if (!o.rows) CK(cudaMalloc((void **)&o.rows, 5 * (size_t)c->P.n * sizeof(double)));
        if (c->mixed)
            launch_egest_m(c->stream, c->fixed, c->P.n, c->M, c->px[c->pcur], c->pa[c->pcur], c->pid[c->pcur],
                           o.rows);
        else launch_egest(c->stream, c->P.n, c->px[c->pcur], c->pid[c->pcur], o.rows);
        c->launches += 1;
        CKR(check_launch(c, "egest"));
    }
    CK(cudaEventRecord(o.ready, c->stream));
    // the transfer, on the output stream
    CK(cudaStreamWaitEvent(c->out_stream, o.ready, 0));
    if (dist)
        CK(cudaMemcpyAsync(dist, o.dist, (size_t)c->P.nbins * sizeof(double), cudaMemcpyDeviceToHost,
                           c->out_stream));
    if (flow)
        CK(cudaMemcpyAsync(flow, o.fields, 3 * nc * sizeof(double), cudaMemcpyDeviceToHost, c->out_stream));
    if (mag)
        CK(cudaMemcpyAsync(mag, o.fields + 3 * nc, 3 * nc * sizeof(double), cudaMemcpyDeviceToHost,
                           c->out_stream));
    if (particles && n)
        CK(cudaMemcpyAsync(particles, o.rows, 5 * n * sizeof(double), cudaMemcpyDeviceToHost, c->out_stream));
    CK(cudaMemcpyAsync(o.h_err, c->d_err, sizeof(uint32_t), cudaMemcpyDeviceToHost, c->out_stream));
    CK(cudaEventRecord(o.done, c->out_stream));
    o.pending = true;
    return SS_OK;
}

int ss_output_wait(ss_ctx *c, int slot) {
    if (!c) return fail(nullptr, SS_ERR_INVALID_ARGUMENT, "null context");
    if (slot < 0 || slot > 1) return fail(c, SS_ERR_INVALID_ARGUMENT, "output slot %d is not 0 or 1", slot);
    ss_ctx::OutSlot &o = c->out[slot];
    if (!o.pending) return SS_OK;
    CK(cudaSetDevice(c->device));
    CK(cudaEventSynchronize(o.done));
    o.pending = false;
    return report_error_word(c, *o.h_err);
}

int ss_output_query(ss_ctx *c, int slot, int *ready) {
    if (!c || !ready) return fail(c, SS_ERR_INVALID_ARGUMENT, "null argument");
    if (slot < 0 || slot > 1) return fail(c, SS_ERR_INVALID_ARGUMENT, "output slot %d is not 0 or 1", slot);
    ss_ctx::OutSlot &o = c->out[slot];
    if (!o.pending) {
        *ready = 1;
        return SS_OK;
    }
    CK(cudaSetDevice(c->device));
    const cudaError_t e = cudaEventQuery(o.done);
    if (e == cudaErrorNotReady) {
        *ready = 0;
        return SS_OK;
    }
    CK(e);
    *ready = 1;
    return SS_OK;
}

int ss_host_alloc(uint64_t bytes, void **out) {
    ss_ctx *c = nullptr;
    if (!out) return fail(nullptr, SS_ERR_INVALID_ARGUMENT, "null argument");
    *out = nullptr;
    if (bytes == 0) return fail(nullptr, SS_ERR_INVALID_ARGUMENT, "ss_host_alloc of 0 bytes");
    CK(cudaHostAlloc(out, (size_t)bytes, cudaHostAllocDefault));
    return SS_OK;
}

int ss_host_free(void *p) {
    ss_ctx *c = nullptr;
    if (!p) return SS_OK;
    CK(cudaFreeHost(p));
    return SS_OK;
}

static int seam_solve(ss_ctx *c, bool flow, bool mag, double screening, const double *dist) {
    if (!dist) return fail(c, SS_ERR_INVALID_ARGUMENT, "dist is NULL");
    if (c->mixed)
        return fail(c, SS_ERR_INVALID_ARGUMENT,
                    "the solver seams on an explicit distribution need a context without SS_FLAG_MIXED");
    CK(cudaSetDevice(c->device));
    if (!c->dist_dev) CK(cudaMalloc((void **)&c->dist_dev, (size_t)c->P.nbins * sizeof(double)));
    CK(cudaMemcpyAsync(c->dist_dev, dist, (size_t)c->P.nbins * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    uint64_t nl = 0;
    CKR(enqueue_solve(c, flow, mag, nullptr, c->dist_dev, screening, c->pcur, false, &nl));
    c->launches += nl;
    if (mag) c->fields_mag_valid = true;
    return SS_OK;
}

int ss_mean_flow_field(ss_ctx *c, double screening, const double *dist, double *u, double *grad) {
    if (!c) return fail(nullptr, SS_ERR_INVALID_ARGUMENT, "null context");
    if (!is_finite(screening)) return fail(c, SS_ERR_INVALID_ARGUMENT, "screening must be finite");
    CKR(seam_solve(c, true, false, screening, dist));
    return ss_get_flow_complex(c, u, grad);
}

int ss_mean_magnetic_field(ss_ctx *c, const double *dist, double *b, double *gradb) {
    if (!c) return fail(nullptr, SS_ERR_INVALID_ARGUMENT, "null context");
    CKR(seam_solve(c, false, true, 0.0, dist));
    return ss_get_magnetic_complex(c, b, gradb);
}

int ss_langevin(const double *particles, uint64_t n, uint32_t mask, const ss_langevin_args *args, double *out) {
    ss_ctx *c = nullptr;
    if (!particles || !args || !out) return fail(nullptr, SS_ERR_INVALID_ARGUMENT, "ss_langevin: null argument");
    if (n == 0) return SS_OK;
    static_assert(sizeof(ss_langevin_args) == 46 * sizeof(double), "ss_langevin_args layout");
    double *d_in = nullptr, *d_out = nullptr, *d_args = nullptr;
    CK(cudaMalloc((void **)&d_in, 5 * n * sizeof(double)));
    CK(cudaMalloc((void **)&d_out, 5 * n * sizeof(double)));
    CK(cudaMalloc((void **)&d_args, sizeof(ss_langevin_args)));
    CK(cudaMemcpy(d_in, particles, 5 * n * sizeof(double), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(d_args, args, sizeof(ss_langevin_args), cudaMemcpyHostToDevice));
    launch_langevin_args(nullptr, d_in, n, mask & M_ALL, d_args, d_out);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpy(out, d_out, 5 * n * sizeof(double), cudaMemcpyDeviceToHost);
    cudaFree(d_in);
    cudaFree(d_out);
    cudaFree(d_args);
    if (e != cudaSuccess) return fail(nullptr, SS_ERR_CUDA, "ss_langevin: %s", cudaGetErrorString(e));
    return SS_OK;
}

int ss_set_resort(ss_ctx *c, uint32_t every_steps) {
    if (!c) return fail(nullptr, SS_ERR_INVALID_ARGUMENT, "null context");
    CK(cudaSetDevice(c->device));
    if (every_steps > 0) {
        // the re-sort writes into the second particle buffer set, which a context made without
        // the per-step sort has not allocated; each missing buffer on its own
        const size_t N = (size_t)c->P.n;
        const int nd = c->mixed ? 3 : 5;
        for (int b = 0; b < 2; ++b) {
            for (int k = 0; k < nd; ++k)
                if (!c->px[b][k]) CK(cudaMalloc((void **)&c->px[b][k], (N ? N : 1) * sizeof(double)));
            for (int k = 0; c->mixed && k < 2; ++k)
                if (!c->pa[b][k]) CK(cudaMalloc((void **)&c->pa[b][k], (N ? N : 1) * sizeof(float)));
            if (!c->key[b]) CK(cudaMalloc((void **)&c->key[b], (N ? N : 1) * sizeof(uint32_t)));
            if (!c->pid[b]) CK(cudaMalloc((void **)&c->pid[b], (N ? N : 1) * sizeof(uint32_t)));
        }
        if (!c->cursor) CK(cudaMalloc((void **)&c->cursor, (size_t)c->P.ncell * sizeof(uint32_t)));
    }
    c->resort_every = every_steps;
    return SS_OK;
}

int ss_profile_enable(ss_ctx *c, int enable) {
    if (!c) return fail(nullptr, SS_ERR_INVALID_ARGUMENT, "null context");
    CK(cudaStreamSynchronize(c->stream));
    c->timing.on = enable != 0;
    for (double &m : c->timing.ms) m = 0.0;
    c->timing.steps = 0;
    return SS_OK;
}

int ss_profile_read(ss_ctx *c, double *ms, uint64_t *count) {
    if (!c || !ms) return fail(c, SS_ERR_INVALID_ARGUMENT, "null argument");
    for (int k = 0; k < SS_NUM_STAGES; ++k) ms[k] = c->timing.ms[k];
    if (count) *count = c->timing.steps;
    return SS_OK;
}

int ss_launch_count(ss_ctx *c, uint64_t *out) {
    if (!c || !out) return fail(c, SS_ERR_INVALID_ARGUMENT, "null argument");
    *out = c->launches;
    return SS_OK;
}

int ss_fp64_rate(double *fma_per_second) {
    if (!fma_per_second) return fail(nullptr, SS_ERR_INVALID_ARGUMENT, "null argument");
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms <= 0)
        return fail(nullptr, SS_ERR_CUDA, "no CUDA device");
    const unsigned blocks = (unsigned)sms * 8u;  // 2048 threads per SM
    const int iters = 4096;
    double *d_out = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    cudaStream_t s = nullptr;
    float best = 0.0f;
    cudaError_t st = cudaMalloc(&d_out, sizeof(double) * blocks * 256);
    if (st == cudaSuccess) st = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
    if (st == cudaSuccess) st = cudaEventCreate(&e0);
    if (st == cudaSuccess) st = cudaEventCreate(&e1);
    for (int rep = 0; rep < 4 && st == cudaSuccess; ++rep) {  // the first launch warms up
        cudaEventRecord(e0, s);
        ss::launch_fp64_rate(s, blocks, iters, d_out);
        cudaEventRecord(e1, s);
        st = cudaEventSynchronize(e1);
        float ms = 0.0f;
        if (st == cudaSuccess) st = cudaEventElapsedTime(&ms, e0, e1);
        if (st == cudaSuccess && rep > 0 && (best == 0.0f || ms < best)) best = ms;
    }
    if (st == cudaSuccess) st = cudaGetLastError();
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (s) cudaStreamDestroy(s);
    if (d_out) cudaFree(d_out);
    if (st != cudaSuccess || best <= 0.0f) return fail(nullptr, SS_ERR_CUDA, "fp64 rate probe: %s", cudaGetErrorString(st));
    *fma_per_second = (double)blocks * 256.0 * 8.0 * iters / (best * 1e-3);
    return SS_OK;
}

}  // extern "C"
