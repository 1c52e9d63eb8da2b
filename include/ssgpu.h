/*
 * ssgpu.h -- C ABI of the GB300 (sm_103a) timestep for stochasticsampling.
 *
 * One context (ss_ctx) holds one simulation on one GPU: the particle state in
 * HBM, the histogram, the spectral solvers (cuFFT plans) and the per-cell
 * field table.  Every entry point returns an int status (SS_OK = 0); no C++
 * exception or CUDA error crosses the ABI.  ss_last_error() returns the text
 * of the last failure on a context.  A context is used by one host thread at
 * a time; its GPU work runs in order on its stream.
 *
 * All particle arrays at this boundary use the reference's serialised layout,
 * [n][5] doubles (x, y, z, phi, theta) -- src/particle.rs:363-395 -- in HOST
 * memory (pageable or pinned).  Fields use the reference's ndarray C order.
 * Complex arrays are interleaved (re, im) doubles, the layout of
 * num_complex::Complex<f64> and of cufftDoubleComplex.
 */
#ifndef SSGPU_H
#define SSGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define SS_OK 0
#define SS_ERR_INVALID_ARGUMENT 1 /* bad pointer, size or parameter (host-side check) */
#define SS_ERR_CUDA 2             /* a CUDA runtime call failed */
#define SS_ERR_CUFFT 3            /* a cuFFT call failed */
#define SS_ERR_STATE 4            /* call out of order (e.g. a step before ss_init) */
#define SS_ERR_PARTICLE_COUNT 5   /* n differs from number_of_particles */
#define SS_ERR_RANGE 6            /* a device bounds check fired (non-finite state) */

/* GridSize, src/lib.rs:52-61 */
typedef struct {
    uint64_t x, y, z, phi, theta;
} ss_grid;

/* BoxSize, src/lib.rs:44-51 */
typedef struct {
    double x, y, z;
} ss_box;

/* The numeric part of Settings (src/bin/simulation/settings/mod.rs:24-118)
 * that the timestep reads. */
typedef struct {
    double timestep;               /* simulation.timestep */
    double trans_diffusion;        /* parameters.diffusion.translational */
    double rot_diffusion;          /* parameters.diffusion.rotational */
    double stress_active;          /* parameters.stress.active */
    double stress_magnetic;        /* parameters.stress.magnetic */
    double shape;                  /* parameters.shape */
    double magnetic_drag;          /* parameters.magnetic_drag */
    double hydro_screening;        /* parameters.hydro_screening */
    double volume_exclusion;       /* parameters.volume_exclusion */
    double magnetic_reorientation; /* parameters.magnetic_reorientation */
    double magnetic_dipole_dipole; /* parameters.magnetic_dipole.magnetic_dipole_dipole */
    uint64_t number_of_particles;  /* simulation.number_of_particles */
    uint64_t seed;                 /* simulation.seed (Philox key) */
} ss_params;

/* flags for ss_create */
#define SS_FLAG_QUASI2D 1u         /* cargo feature quasi2d: grid z = 1, after each step z = 0, theta = pi/2 */
#define SS_FLAG_ALWAYS_MAGNETIC 2u /* run the dipolar solver even when its couplings are zero */
#define SS_FLAG_NO_SORT 4u         /* keep particles in input order (no counting sort by cell) */
#define SS_FLAG_NO_GRAPH 8u        /* launch kernels directly instead of replaying a CUDA graph */
#define SS_FLAG_MIXED 16u          /* FP32 mixed precision: FP64 positions and k = 0 / mean handling, FP32
                                      angles, binning, contraction, FFTs, fields and Langevin arithmetic
                                      (no sort; the library seams ss_mean_* need the FP64 mode) */
#define SS_FLAG_FIXED64 128u       /* as SS_FLAG_MIXED, with positions accumulated in 64-bit fixed point
                                      (units of L / 2^64: periodic wrap by integer overflow, exact binning by
                                      a 64-bit high multiply, no FP64 instruction in the step) */
#define SS_FLAG_F32X2 256u         /* FP64 mode: the update computes each step's increments (position,
                                      and the angle changes) in two-float (FP32 pair) arithmetic, about
                                      2^-46 relative, and adds them to the FP64 state in FP64; the field
                                      table is then kept as float pairs.  Needs the nearest-cell gather
                                      (no effect with SS_FLAG_TRILINEAR*); not with SS_FLAG_MIXED or
                                      SS_FLAG_FIXED64 */
#define SS_FLAG_TRILINEAR 32u      /* gather every field by trilinear interpolation at the particle position
                                      (src/mesh/interpolate.rs:11-119) instead of the nearest cell that
                                      do_timestep uses (FP64 mode) */
#define SS_FLAG_TRILINEAR_ZFROMY 64u /* as SS_FLAG_TRILINEAR, with the reference's z fraction computed from
                                        y (interpolate.rs:22), for comparisons with that code */

typedef struct ss_ctx ss_ctx;

/* Simulation::new, src/bin/simulation/mod.rs:91-160.  Builds the stress kernel
 * (closure :100-104), the k meshes and the cuFFT plans, allocates HBM.
 * stream: a cudaStream_t to run on, or NULL for a stream owned by the context. */
int ss_create(const ss_grid *grid, const ss_box *box, const ss_params *params, uint32_t flags,
              void *stream, ss_ctx **out);
/* Drop for Simulation, src/bin/simulation/mod.rs:377-381 */
int ss_destroy(ss_ctx *ctx);

/* Simulation::init, src/bin/simulation/mod.rs:163-196: sanitises every
 * particle with Particle::new (src/particle.rs:186-201) and samples the
 * distribution (x box volume).  n must equal number_of_particles. */
int ss_init(ss_ctx *ctx, const double *particles, uint64_t n);
/* Simulation::resume, src/bin/simulation/mod.rs:199-207.  The noise stream is
 * counter based (Philox4x32-10 keyed by seed, counter = (particle, timestep)),
 * so restoring the timestep restores the noise exactly. */
int ss_resume(ss_ctx *ctx, const double *particles, uint64_t n, uint64_t timestep);

/* init_simulation with InitType::Distribution (src/bin/init.rs:93-116):
 * samples the initial particles on the device and then behaves like ss_init.
 * kind 0 = Isotropic (Particle::create_isotropic, src/particle.rs:241-256),
 * kind 1 = Homogeneous (Particle::create_homogeneous, :280-295, with
 * kappa = magnetic_reorientation / rotational diffusion).  The draws come from
 * Philox keyed by seed (the reference uses Pcg64Mcg). */
int ss_init_distribution(ss_ctx *ctx, uint32_t kind);

/* Simulation::do_timestep, src/bin/simulation/mod.rs:251-374.
 * noise: NULL -> on-device Philox noise; otherwise [n][5] host doubles
 * (x, y, z, axis_angle, rotate_angle) = RandomVector (:51-57), the
 * verification mode that takes the reference's host-generated noise.
 * timestep_out (may be NULL) receives the incremented step counter. */
int ss_do_timestep(ss_ctx *ctx, const double *noise, uint64_t *timestep_out);
/* `steps` calls of do_timestep with Philox noise (the driver loop,
 * src/bin/main.rs:182-262, without IO); replays a captured CUDA graph. */
int ss_run(ss_ctx *ctx, uint64_t steps, uint64_t *timestep_out);
/* The on-device noise of step `timestep` as the RandomVector array the
 * verification mode takes: out[n][5] host doubles (x, y, z, axis_angle,
 * rotate_angle) in the caller's particle order (src/bin/simulation/mod.rs:
 * 272-286).  The step uses the axis as its sine and cosine (the sine is the
 * FP32 sine as an exact double, the cosine sqrt(1 - sine^2) in FP64 with the
 * FP32 cosine's sign: a unit pair); axis_angle is reported as their atan2 in
 * [0, 2 pi), whose sine and cosine give them back to FP64 rounding. */
int ss_noise(ss_ctx *ctx, uint64_t timestep, double *out);
/* One do_timestep on host-resident particles: the rows of `in` ([n][5] host
 * doubles) replace the state as in ss_resume at the current step (the same
 * checks), the step runs with on-device noise, and the new state is written
 * to `out` ([n][5]) -- ss_resume + ss_do_timestep + ss_get_particles in one
 * call, with the read-back of each chunk of updated particles overlapping
 * the update of the next (a second stream).  The particles stay in the
 * caller's order (no sort this step).  Mixed-precision contexts, and
 * contexts recording per-stage times, run it as those three calls.  `in` and `out` may be the same
 * buffer; pinned host memory gives the full copy bandwidth.  The drop-in
 * form of Simulation::do_timestep (src/bin/simulation/mod.rs:251-374) for a
 * caller that keeps the particles in host memory. */
int ss_step_host(ss_ctx *ctx, const double *in, double *out, uint64_t n, uint64_t *timestep_out);
/* Wait for the context's stream. */
int ss_synchronize(ss_ctx *ctx);

/* Simulation::get_particles / get_particles_head (:221-228): [n][5] */
int ss_get_particles(ss_ctx *ctx, double *out, uint64_t n);
/* Simulation::get_distribution (:231-233): dist[x][y][z][phi][theta] as
 * sampled at the start of the last step (after init: the initial sample),
 * normalised like Distribution::sample_from x box volume. */
int ss_get_distribution(ss_ctx *ctx, double *out);
/* the integer histogram behind ss_get_distribution (bit-exact counts) */
int ss_get_counts(ss_ctx *ctx, uint32_t *out);
/* Simulation::get_flow_field (:236-238): Re(u), [3][x][y][z] */
int ss_get_flow_field(ss_ctx *ctx, double *out);
/* Simulation::get_magnetic_field (:241-243): Re(B), [3][x][y][z].  When the
 * step skipped the dipolar solve (both couplings zero), it is computed here on
 * demand from the histogram of the last step, which is still resident. */
int ss_get_magnetic_field(ss_ctx *ctx, double *out);
/* the complex views returned by SpectralSolver::mean_flow_field
 * (src/flowfield/spectral_solver.rs:233-254): u [3][x][y][z], grad [3][3][x][y][z] */
int ss_get_flow_complex(ss_ctx *ctx, double *u, double *grad);
/* the complex views returned by MagneticSolver::mean_magnetic_field
 * (src/magnetic_interaction/magnetic_solver.rs:139-161) */
int ss_get_magnetic_complex(ss_ctx *ctx, double *b, double *gradb);
/* Simulation::get_timestep (:246-248) */
int ss_get_timestep(ss_ctx *ctx, uint64_t *out);

/* Output that overlaps the steps.  The reference's main loop hands each due
 * output to its IO worker thread, which serialises and compresses it while
 * the simulation steps on (src/bin/main.rs:182-262, src/bin/output/
 * worker.rs:130-248).  ss_output_begin is the device half of that hand-off:
 * on the context's stream it copies the requested outputs of the current
 * state into device slot `slot` (0 or 1) -- in HBM, so the next step may
 * overwrite the state at once -- and then starts their transfer into the
 * caller's host buffers on the context's output stream.  It returns without
 * waiting for either, so further ss_do_timestep / ss_run calls queue behind
 * it and the transfer runs while they execute.  Any buffer may be NULL:
 *   dist       [nbins] doubles, as ss_get_distribution
 *   flow       [3][cells] doubles, as ss_get_flow_field
 *   mag        [3][cells] doubles, as ss_get_magnetic_field
 *   particles  the first n rows, [n][5], as ss_get_particles
 * The transfer is asynchronous from page-locked memory (ss_host_alloc, or
 * cudaHostRegister'ed); from pageable memory the CUDA runtime stages it and
 * the call may wait for it.  The host buffers hold the outputs once
 * ss_output_wait(ctx, slot) has returned SS_OK and must not be touched
 * before.  A slot still in flight cannot begin again (SS_ERR_STATE). */
int ss_output_begin(ss_ctx *ctx, int slot, double *dist, double *flow, double *mag, double *particles,
                    uint64_t n);
/* Block until slot's transfer has landed (SS_OK at once when none is in
 * flight).  Reports the device's bounds-check flags as they stood when the
 * outputs were taken (SS_ERR_RANGE), as the synchronous getters do. */
int ss_output_wait(ss_ctx *ctx, int slot);
/* *ready = 1 when slot has no transfer in flight (ss_output_wait would not
 * block), else 0. */
int ss_output_query(ss_ctx *ctx, int slot, int *ready);
/* Page-locked host memory (cudaHostAlloc) for the output buffers, and its
 * release. */
int ss_host_alloc(uint64_t bytes, void **out);
int ss_host_free(void *p);

/* Library seams on an explicit distribution dist[x][y][z][phi][theta] (host):
 * SpectralSolver::mean_flow_field(screening, &Distribution) and
 * MagneticSolver::mean_magnetic_field(&Distribution).  Outputs as
 * ss_get_flow_complex / ss_get_magnetic_complex.  They overwrite the
 * context's field buffers; the particle state is untouched. */
int ss_mean_flow_field(ss_ctx *ctx, double screening, const double *dist, double *u, double *grad);
int ss_mean_magnetic_field(ss_ctx *ctx, const double *dist, double *b, double *gradb);

/* LangevinBuilder chain (src/integrators/langevin_builder/mod.rs:25-125,
 * modifiers.rs:39-231) on n independent particles with shared arguments,
 * run by the same device code as the timestep.  mask selects modifiers
 * (bit k = k-th modifier of the chain in do_timestep order:
 * self_propulsion, convection, magnetic_dipole_dipole_force,
 * external_field_alignment, magnetic_dipole_dipole_rotation,
 * jeffrey_vorticity, jeffrey_strain, step, translational_diffusion,
 * rotational_diffusion).  particles/out: host [n][5]. */
typedef struct {
    double flow[3];
    double drag;
    double gradb[9];
    double reorientation;
    double b[3]; /* magnetic field already times magnetic_dipole_dipole */
    double vort[9];
    double shape;
    double strain[9];
    double dt;
    double xi[3];
    double diff;
    double axis_angle, rotate_angle;
    double box_x, box_y, box_z;
} ss_langevin_args;
int ss_langevin(const double *particles, uint64_t n, uint32_t mask, const ss_langevin_args *args,
                double *out);

/* Counting-sort the particles by cell before the update of every
 * every_steps-th step (0: never, the default).  The FP32 paths and 3-D FP64
 * contexts sort their rows by cell once, at ingest; particles drift away from
 * that order over long runs (on the 3-D workload the FP32 update is 10 %
 * slower after 3,000 steps), which a re-sort every few hundred steps undoes.
 * A context made without SS_FLAG_NO_SORT already sorts every step.  No
 * result changes: the particles keep their caller order on every read-back.
 * Allocates the second particle buffer set on first use.  The stage is timed
 * as stage 6 (sort). */
int ss_set_resort(ss_ctx *ctx, uint32_t every_steps);

/* Per-stage timing (CUDA events on the context stream).  enable != 0 starts
 * recording; ss_profile_read fills ms[SS_NUM_STAGES] with the summed time of
 * each stage since enabling and count with the number of steps. */
#define SS_NUM_STAGES 8
/* stage order: 0 contract, 1 fft forward, 2 k-space, 3 fft inverse, 4 field table,
 * 5 particle update, 6 sort, 7 other */
int ss_profile_enable(ss_ctx *ctx, int enable);
int ss_profile_read(ss_ctx *ctx, double *ms, uint64_t *count);
/* number of this library's kernels launched on the context so far
 * (cuFFT's own kernels excluded) */
int ss_launch_count(ss_ctx *ctx, uint64_t *out);
/* FP64 FMA throughput of the current device (thread-FMAs per second) from a
 * probe kernel of independent FMA chains on every SM: the FP64 roofline of
 * the particle update, whose bound on GB300 is the FP64 pipe.  Diagnostic; no
 * counterpart in the reference. */
int ss_fp64_rate(double *fma_per_second);

/* The normalised distribution of a particle list, computed without any
 * allocation.  This entry point has no counterpart in the reference.
 *
 * It is for callers that cannot call cudaMalloc or cudaFree where they need
 * the histogram: a hook inside another library's loop, where the device-wide
 * synchronisation of cudaFree would stall or deadlock that loop, or an
 * application that reserves a fixed device-memory budget at start-up and may
 * not grow it.  It gives the same result as ss_init + ss_get_distribution on
 * a context, without creating one:
 * dist[b] = (count_b / (gw_x gw_y gw_z gw_phi gw_theta n)) * (L_x L_y L_z),
 * after applying Particle::new (src/particle.rs:186-201) to every row.
 *
 *   particles: DEVICE pointer, [n][5] doubles (x, y, z, phi, theta),
 *              1 <= n <= 2^32 - 1 (the limit of ss_create)
 *   dist:      DEVICE pointer, [x][y][z][phi][theta] doubles, written in full
 *   stream:    cudaStream_t to run on (NULL: the legacy default stream)
 *
 * Rows must be finite.  ss_init refuses a non-finite row on the host; here
 * the rows are only seen on the device, so such a row is not counted and
 * every bin of dist is written as NaN instead, which the caller finds in the
 * result when it reads it.
 *
 * Scratch: one file-scope device array of SS_NOALLOC_MAX_BINS u32 counts
 * plus an error word (8 MiB), which every GPU that loads this library holds
 * until the process exits.  Grids with more bins are rejected
 * (SS_ERR_INVALID_ARGUMENT).  Every call shares that array and clears it
 * first, so calls whose kernels overlap on the GPU (two streams, two threads)
 * race and corrupt each other's counts: order them on one stream.  The first
 * call on a device looks up the array's device address
 * (cudaGetSymbolAddress, with that device current) and the device's
 * multiprocessor count; make that first call before any stream capture.  The
 * call is asynchronous: it only enqueues kernels.  Errors are reported by
 * ss_last_error(NULL, ...). */
#define SS_NOALLOC_MAX_BINS 2097152u
int ss_sample_distribution_noalloc(const ss_grid *grid, const ss_box *box, const double *particles, uint64_t n,
                                   double *dist, void *stream);

/* ---- batched ensembles ---------------------------------------------------
 * Many independent quasi-2-D simulations stepped together on one GPU, the
 * batched form of running the reference binary once per parameter set
 * (src/bin/simulation/main.rs) -- a parameter scan or an ensemble average.
 * Member m has its own grid, box and parameters (particle count, seed,
 * activity, diffusion, ...).  Every member is stepped with the arithmetic of
 * a single context created with SS_FLAG_QUASI2D | SS_FLAG_MIXED and the same
 * grid, box and parameters, with the same Philox stream, so member m follows
 * that context's trajectory up to the round-off of the differently batched
 * FP32 FFTs.  Members of one grid shape share one batched cuFFT plan; each
 * step is one CUDA graph of 6 kernels plus 2 FFT calls per grid shape.
 * Dipolar coupling is not supported (magnetic_dipole_dipole and
 * magnetic_drag must be 0).  Errors are reported by ss_last_error(NULL, ...). */
typedef struct ss_ens ss_ens;

/* count members; grids[m].z == grids[m].theta == 1; flags: SS_FLAG_QUASI2D,
 * optionally | SS_FLAG_MIXED (implied).  stream as in ss_create. */
int ss_ensemble_create(const ss_grid *grids, const ss_box *boxes, const ss_params *params, uint32_t count,
                       uint32_t flags, void *stream, ss_ens **out);
int ss_ensemble_destroy(ss_ens *ens);
/* Simulation::init for every member: particles holds the members' rows one
 * after the other ([sum n_m][5] doubles, host memory); every row must have
 * z = 0 and theta = pi/2.  Resets every member's timestep to 0. */
int ss_ensemble_init(ss_ens *ens, const double *particles, uint64_t total);
/* times the particle update's launch shapes on the ensemble's own data and
 * keeps the fastest; config (optional, 4 entries) receives threads per
 * block, resident blocks per SM, particles per work unit and the register
 * plan (1: 72, 2: 64, 3: 40 registers per thread).  ss_ensemble_run calls it
 * before its first step when neither it nor ss_ensemble_set_config has run. */
int ss_ensemble_autotune(ss_ens *ens, uint32_t *config);
/* sets the update's launch shape (the 4 entries ss_ensemble_autotune
 * reports), e.g. one tuned earlier for the same ensemble shape */
int ss_ensemble_set_config(ss_ens *ens, const uint32_t *config);
/* steps do_timestep calls of every member (asynchronous) */
int ss_ensemble_run(ss_ens *ens, uint64_t steps);
int ss_ensemble_synchronize(ss_ens *ens);
/* member's particles, [n_m][5] doubles (x, y, 0, phi, pi/2), host memory */
int ss_ensemble_get_particles(ss_ens *ens, uint32_t member, double *out);
/* member's histogram the last step solved from (after init: the initial
 * one), as ss_get_counts */
int ss_ensemble_get_counts(ss_ens *ens, uint32_t member, uint32_t *out);
/* member's flow field of the last step, [3][x][y] doubles, as ss_get_flow_field */
int ss_ensemble_get_flow_field(ss_ens *ens, uint32_t member, double *out);
/* total particles, grid-shape groups and kernel launches so far (each optional) */
int ss_ensemble_info(ss_ens *ens, uint64_t *particles, uint32_t *groups, uint64_t *launches);

/* ---- learned histogram denoiser ------------------------------------------
 * One 3x3x3 periodic convolution of 32 -> 32 channels on the tensor cores
 * (tcgen05, BF16 operands, FP32 accumulation): the building block of the
 * denoiser, exposed for tests.  x: DEVICE bf16 in the activation layout
 * [nx][np][4][ny][8] (channel c of voxel (x, y, p) in chunk c / 8, lane
 * c % 8: each line's 128-row segment of one 8-channel chunk is one
 * contiguous 2 KB block), 16-byte aligned; w: DEVICE float [27][32
 * out][32 in], tap = 9 (dx+1) + 3 (dy+1) + (dp+1) (the torch conv3d weight
 * [out][in][dx+1][dy+1][dp+1] reordered);
 * bias: DEVICE float[32].  mode 0: y = bf16 ReLU(conv(x) + bias); mode 1:
 * y = float conv(x) + bias; mode 2: y = bf16 conv^T(x) * (ref > 0), the
 * backward-data step through a ReLU (ref: DEVICE bf16, bias unused); y and
 * ref in the same layout as x (float for mode 1), 16-byte aligned.
 * ny must be a positive multiple of 128.  Returns after completion. */
int ss_dn_conv32(const void *x, const float *w, const float *bias, const void *ref, void *y, uint32_t nx,
                 uint32_t ny, uint32_t np, uint32_t mode, void *stream);

/* The denoiser network: input x (the histogram divided by its mean count,
 * DEVICE float [nx][ny][np]) -> conv 1->32 + ReLU -> conv 32->32 + ReLU ->
 * conv 32->32 + ReLU -> conv 32->1 -> y = x + that (DEVICE float).  All
 * convolutions 3x3x3 with periodic padding, all on the tensor cores with
 * BF16 weights, BF16 inputs and activations and FP32 accumulation (the
 * residual x and the biases stay FP32).  57,121 FP32 parameters: w_in[27][32], b_in[32],
 * w2[27][32][32], b2[32], w3[27][32][32], b3[32], w_out[27][32], b_out
 * (w[tap][out][in], tap as for ss_dn_conv32).  Trained with Adam on the
 * mean-square error against a target distribution. */
typedef struct ss_dn ss_dn;
/* He-initialised from seed (the output layer near zero: y ~ x at start);
 * ny a positive multiple of 128.  stream as in ss_create. */
int ss_dn_create(uint32_t nx, uint32_t ny, uint32_t np, uint64_t seed, void *stream, ss_dn **out);
int ss_dn_destroy(ss_dn *dn);
/* parameter count (57121) and kernel launches so far (each optional) */
int ss_dn_info(ss_dn *dn, uint64_t *nparams, uint64_t *launches);
int ss_dn_get_params(ss_dn *dn, float *host, uint64_t count);
int ss_dn_set_params(ss_dn *dn, const float *host, uint64_t count);
/* y = network(x), DEVICE arrays; returns after completion */
int ss_dn_forward(ss_dn *dn, const float *x, float *y);
/* batch samples x[batch][V], t[batch][V] (DEVICE): loss = mean over the batch
 * of mean_v (y - t)^2 (plus the moment term of ss_dn_set_loss); with lr > 0 one Adam step (beta 0.9 / 0.999) on the
 * batch-mean gradient, with lr = 0 the loss only */
int ss_dn_train(ss_dn *dn, const float *x, const float *t, uint32_t batch, float lr, double *loss);
/* The training loss: w = 0 (the default) is the mean-square error above.
 * w > 0 adds, per cell (x, y), w times the squared second angular harmonic
 * of the residual r = y - t over phi, summed over cells and divided by the
 * voxel count: mean_v r^2 + w sum_cells (c2^2 + s2^2) / V with c2 = sum_k r_k
 * cos 2 phi_k, s2 = sum_k r_k sin 2 phi_k at the phi bin centres.  In the
 * plane the flow depends on a cell's orientation distribution only through
 * that harmonic (the Oseen projection removes the density's part), so the
 * term weights the error that reaches the flow.  No counterpart in the
 * reference (the denoiser is an extension). */
int ss_dn_set_loss(ss_dn *dn, float moment_weight);
/* the batch-mean gradient of that loss (host float[count]) without an update */
int ss_dn_gradients(ss_dn *dn, const float *x, const float *t, uint32_t batch, float *grads, uint64_t count,
                    double *loss);

/* Training data for the denoiser: adds to hist (DEVICE float [nx][ny][np])
 * the normalised histogram (nx ny np / n per particle, mean 1) of n particles
 * drawn with density 1 + amp sin(2 pi s + phase) along axis (0: x, 1: y; s =
 * position / box edge), uniform along the other axis and in phi -- the
 * production workload's initial-condition family.  Philox keyed by seed.
 * Asynchronous on stream. */
int ss_dn_sample_histogram(uint32_t nx, uint32_t ny, uint32_t np, uint64_t n, double amp, double phase,
                           uint32_t axis, uint64_t seed, float *hist, void *stream);

/* Put the denoiser between the histogram and the stress contraction of a
 * quasi2d SS_FLAG_MIXED / SS_FLAG_FIXED64 context whose grid (x, y, phi)
 * equals the network's: every step then contracts network(counts / mean
 * count) * mean count instead of the counts (the binning, the particles and
 * ss_get_counts are unchanged).  dn = NULL removes it.  The context does not
 * own dn; keep it alive while it is set. */
int ss_set_denoiser(ss_ctx *ctx, ss_dn *dn);

/* copy the last error message of ctx (or the last context-free error when
 * ctx is NULL) into buf, NUL terminated */
int ss_last_error(ss_ctx *ctx, char *buf, size_t len);
/* library version string */
const char *ss_version(void);

#ifdef __cplusplus
}
#endif
#endif
