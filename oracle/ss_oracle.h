/*
 * ss_oracle.h -- CPU FP64 restatement of the stochasticsampling timestep.
 *
 * TEST INFRASTRUCTURE, NOT PRODUCT.  Only the parity tests, the smoke check
 * and the CPU-baseline leg of the benchmark may load this library, and only
 * as the checker / the timed CPU reference.  The CUDA library never calls it.
 *
 * Every function restates the reference's arithmetic in the same operation
 * order (FP contraction disabled at build time), citing the reference file
 * and line it follows.  Third-party arithmetic on the path whose sources are
 * not in the reference tree is restated from its published algorithm:
 *   - ndarray 0.12.1   : linspace (start + step*i), eight-way unrolled dot,
 *                        sequential sum_axis
 *   - num-complex 0.2.3: real / complex division  (x*re / |z|^2)
 *   - quaternion 0.3.1 + vecmath 0.3.1 : axis_angle, rotate_vector = q v q*
 *   - FFTW 3.x         : unnormalised c2c DFT (sign -1 forward, +1 backward);
 *                        restated as an own mixed-radix FFT.
 *   - rand 0.7 / rand_distr 0.2.1 / rand_pcg 0.2.0 noise: not restated (not
 *     pinned by any reference test); the step takes an explicit noise array,
 *     and the timed baseline draws its own PCG32 noise.
 *
 * Particle layout is the reference's serialised one: [n][5] doubles
 * (x, y, z, phi, theta), src/particle.rs:363-395.
 * Complex arrays are interleaved (re, im) doubles, component-major, C order
 * [comp][x][y][z], like ndarray Array<Complex<f64>, Ix4/Ix5>.
 */
#ifndef SS_ORACLE_H
#define SS_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
    uint64_t gx, gy, gz, gphi, gtheta;   /* GridSize, src/lib.rs:40-54 */
    double bx, by, bz;                   /* BoxSize */
    double timestep;                     /* simulation.timestep */
    double trans_diff, rot_diff;         /* parameters.diffusion */
    double stress_active, stress_magnetic; /* parameters.stress */
    double shape;                        /* parameters.shape */
    double magnetic_drag;                /* parameters.magnetic_drag */
    double hydro_screening;              /* parameters.hydro_screening */
    double volume_exclusion;             /* parameters.volume_exclusion */
    double magnetic_reorientation;       /* parameters.magnetic_reorientation */
    double magnetic_dipole_dipole;       /* parameters.magnetic_dipole.magnetic_dipole_dipole */
    int32_t quasi2d;                     /* cargo feature quasi2d as a runtime flag */
    int32_t gather;                      /* 0 nearest cell (the step), 1 trilinear
                                            (src/mesh/interpolate.rs), 2 trilinear with
                                            the reference's z fraction from y (:22) */
    uint64_t seed;                       /* simulation.seed */
} orc_settings;

/* ---- particle.rs ------------------------------------------------------ */
double orc_modulo(double f, double m);
void orc_ang_pbc(double phi, double theta, double out[2]);
void orc_particle_new(const orc_settings *s, const double in[5], double out[5]);
void orc_from_vector(const double v[3], double out_phi_theta[2]);

/* ---- mesh / distribution --------------------------------------------- */
void orc_grid_width(const orc_settings *s, double gw[5]);
void orc_coord_to_grid(const orc_settings *s, const double p[5], uint64_t out[5]);
void orc_cell_index(const orc_settings *s, const double p[5], uint64_t out[3]);
void orc_k_sampling(uint64_t n, double box, double *out);
void orc_k_mesh(const orc_settings *s, double *out /* [3][gx][gy][gz] */);
void orc_norm_k_mesh(const orc_settings *s, double *out /* [3][gx][gy][gz] */);
void orc_inverse_norm_squared(const orc_settings *s, double *out /* [gx][gy][gz] */);
/* histogram_from: raw counts (as doubles) into dist[gx][gy][gz][gphi][gtheta] */
void orc_histogram(const orc_settings *s, const double *particles, uint64_t n, double *dist);
/* sample_from: counts / (gx*gy*gz*gphi*gtheta*n) (no box-volume factor) */
void orc_sample_from(const orc_settings *s, const double *particles, uint64_t n, double *dist);

/* ---- kernels over the angle grid ------------------------------------- */
void orc_stress_kernel(const orc_settings *s, double *out /* [3][3][gphi][gtheta] */);
void orc_orientation_kernel(const orc_settings *s, double *out /* [3][gphi][gtheta] */);
void orc_stress_active(double phi, double theta, double out[9]);
void orc_stress_magnetic(double phi, double theta, double out[9]);
void orc_stress_magnetic_rods(double phi, double theta, double out[9]);

/* ---- FFT (own restatement of an unnormalised c2c DFT) ---------------- */
void orc_fft3d(double *data, uint64_t nx, uint64_t ny, uint64_t nz, int sign);

/* ---- field solvers ---------------------------------------------------- */
/* average_stress over dist (already scaled by box volume as in do_timestep) */
void orc_average_stress(const orc_settings *s, const double *kernel, const double *dist,
                        double *stress /* cplx [9][ncell] */);
void orc_director_field(const orc_settings *s, const double *dist, double *p /* cplx [3][ncell] */);
void orc_flow_field(const orc_settings *s, const double *dist, double screening,
                    double *u /* cplx [3][ncell] */, double *grad /* cplx [3][3][ncell] */,
                    int nthreads);
void orc_magnetic_field(const orc_settings *s, const double *dist,
                        double *b /* cplx [3][ncell] */, double *gradb /* cplx [3][3][ncell] */,
                        int nthreads);
/* MagneticSolver::update_gradient on a given k-space field (no inverse of b) */
void orc_vector_gradient(const orc_settings *s, const double *bk /* cplx [3][ncell] */,
                         double *grad /* cplx [3][3][ncell], inverse-transformed */);

/* interpolate_vector_field (src/mesh/interpolate.rs:11-40) of `ncomp`
 * real fields [ncomp][gx][gy][gz] at position p; zbug != 0 keeps the
 * reference's z fraction computed from p.y (:22) */
void orc_interpolate(const orc_settings *s, const double *field, int ncomp, const double p[3], int zbug,
                     double *out);

/* ---- Langevin builder ------------------------------------------------- */
enum {
    ORC_SELF_PROPULSION = 1 << 0,
    ORC_CONVECTION = 1 << 1,
    ORC_MDD_FORCE = 1 << 2,
    ORC_EXTERNAL_FIELD = 1 << 3,
    ORC_MDD_ROTATION = 1 << 4,
    ORC_JEFFREY_VORTICITY = 1 << 5,
    ORC_JEFFREY_STRAIN = 1 << 6,
    ORC_STEP = 1 << 7,
    ORC_TRANS_DIFFUSION = 1 << 8,
    ORC_ROT_DIFFUSION = 1 << 9,
    ORC_ALL = (1 << 10) - 1
};

typedef struct {
    double flow[3];
    double drag;
    double gradb[9];
    double reorientation;
    double b[3];          /* already multiplied by magnetic_dipole_dipole */
    double vort[9];
    double shape;
    double strain[9];
    double dt;
    double xi[3];
    double diff;
    double axis_angle, rotate_angle;
    double bx, by, bz;
} orc_langevin_args;

void orc_langevin(const double p[5], uint32_t mask, const orc_langevin_args *a, double out[5]);

/* ---- whole simulation ------------------------------------------------- */
typedef struct orc_sim orc_sim;
orc_sim *orc_sim_new(const orc_settings *s, uint64_t n, int nthreads);
void orc_sim_free(orc_sim *sim);
int orc_sim_init(orc_sim *sim, const double *particles, uint64_t n);
/* noise: [n][5] (x, y, z, axis_angle, rotate_angle) or NULL for own PCG32 noise */
uint64_t orc_sim_step(orc_sim *sim, const double *noise);
double *orc_sim_particles(orc_sim *sim);
double *orc_sim_distribution(orc_sim *sim);
double *orc_sim_flow(orc_sim *sim);       /* cplx [3][ncell]    (after the step's solve) */
double *orc_sim_flow_grad(orc_sim *sim);  /* cplx [3][3][ncell] */
double *orc_sim_mag(orc_sim *sim);        /* cplx [3][ncell] */
double *orc_sim_mag_grad(orc_sim *sim);   /* cplx [3][3][ncell] */
double *orc_sim_density(orc_sim *sim);    /* [ncell] */
double *orc_sim_noise(orc_sim *sim);      /* [n][5] noise used by the last step */
uint64_t orc_sim_timestep(const orc_sim *sim);
void orc_sim_set_timestep(orc_sim *sim, uint64_t t);
int orc_max_threads(void);

#ifdef __cplusplus
}
#endif
#endif
