// CPU build of the two-float arithmetic of the FP64 update
// (stochasticsampling_gb300/csrc/f32x2.cuh) for test_f32x2.py:
//   g++ -O2 -std=c++17 -ffp-contract=off -shared -fPIC -I<csrc> f32x2_host.cpp
// Pairs cross this boundary as two floats (h, l); results come back as the
// same pairs widened to double.
#include "f32x2.cuh"

using namespace ss::xf;

static void put(double *o, f2 v) {
    o[0] = v.h;
    o[1] = v.l;
}

extern "C" {

void xf_split(int n, const double *d, float *out) {
    for (int i = 0; i < n; ++i) {
        const f2 v = split(d[i]);
        out[2 * i] = v.h;
        out[2 * i + 1] = v.l;
    }
}

void xf_to_double(int n, const float *f, double *out) {
    for (int i = 0; i < n; ++i) out[i] = to_double(f[i]);
}

void xf_sincos_d(int n, const double *a, double *out) {
    for (int i = 0; i < n; ++i) {
        f2 s, c;
        sincos_d(a[i], s, c);
        put(out + 4 * i, s);
        put(out + 4 * i + 2, c);
    }
}

void xf_sincos_f2(int n, const float *r, double *out) {
    for (int i = 0; i < n; ++i) {
        f2 s, c;
        sincos_f2(f2{r[2 * i], r[2 * i + 1]}, s, c);
        put(out + 4 * i, s);
        put(out + 4 * i + 2, c);
    }
}

void xf_atan2(int n, const float *y, const float *x, double *out) {
    for (int i = 0; i < n; ++i) put(out + 2 * i, atan2_f2(f2{y[2 * i], y[2 * i + 1]}, f2{x[2 * i], x[2 * i + 1]}));
}

// terms: bits 0..6 = self propulsion, convection, translational diffusion,
// rotational diffusion, external field, vorticity, strain; bit 7: the noise
// xi0, xi1, sa as floats (their h; the on-device noise), else as pairs.  ct: 16 floats a
// particle; xi: (xi0 h, l, xi1 h, l); sa, rot: pairs; dt, reorient_dt: one
// pair each.  out: dx, dy, dphi as pairs.
void xf_canon(int n, const double *phi, const float *ct, const float *xi, const float *sa, const float *rot,
              unsigned terms, const float *dt, const float *reorient_dt, double *out) {
    CanonTerms T;
    T.self_propulsion = terms & 1u;
    T.convection = terms & 2u;
    T.trans_diffusion = terms & 4u;
    T.rot_diffusion = terms & 8u;
    T.external_field = terms & 16u;
    T.vorticity = terms & 32u;
    T.strain = terms & 64u;
    for (int i = 0; i < n; ++i) {
        float4 row[4];
        for (int k = 0; k < 4; ++k)
            row[k] = float4{ct[16 * i + 4 * k], ct[16 * i + 4 * k + 1], ct[16 * i + 4 * k + 2], ct[16 * i + 4 * k + 3]};
        f2 dx, dy, dph;
        const f2 r = {rot[2 * i], rot[2 * i + 1]}, d = {dt[0], dt[1]}, re = {reorient_dt[0], reorient_dt[1]};
        if (terms & 128u)
            canon_increments(phi[i], row, xi[4 * i], xi[4 * i + 2], sa[2 * i], r, T, d, re, dx, dy, dph);
        else
            canon_increments(phi[i], row, f2{xi[4 * i], xi[4 * i + 1]}, f2{xi[4 * i + 2], xi[4 * i + 3]},
                             f2{sa[2 * i], sa[2 * i + 1]}, r, T, d, re, dx, dy, dph);
        put(out + 6 * i, dx);
        put(out + 6 * i + 2, dy);
        put(out + 6 * i + 4, dph);
    }
}
}

// The full chain.  terms: bits 0..9 = self propulsion, convection, dipolar
// force, external field, dipolar rotation, vorticity, strain, step,
// translational diffusion, rotational diffusion; bit 10: the noise as
// floats (xi h, sa h, ca from axis_cos(sa h, ca h)), else as pairs.
// row: 32 pairs a particle; xi: 3 pairs; sa, ca, rot: pairs; prm: dt,
// reorient, shape, drag as pairs.  out: dp (3 pairs), a, b (pairs), direct.
extern "C" void xf_full(int n, const double *phi, const double *theta, const float *row, const float *xi,
                        const float *sa, const float *ca, const float *rot, unsigned terms, const float *prm,
                        double *out) {
    FullTerms T;
    T.self_propulsion = terms & 1u;
    T.convection = terms & 2u;
    T.mdd_force = terms & 4u;
    T.external_field = terms & 8u;
    T.mdd_rotation = terms & 16u;
    T.vorticity = terms & 32u;
    T.strain = terms & 64u;
    T.step = terms & 128u;
    T.trans_diffusion = terms & 256u;
    T.rot_diffusion = terms & 512u;
    const f2 dt = {prm[0], prm[1]}, re = {prm[2], prm[3]}, sh = {prm[4], prm[5]}, dr = {prm[6], prm[7]};
    for (int i = 0; i < n; ++i) {
        const float2 *r = reinterpret_cast<const float2 *>(row + 64 * i);
        const float *x = xi + 6 * i;
        const f2 ro = {rot[2 * i], rot[2 * i + 1]};
        FullOut o;
        if (terms & 1024u)
            full_increments(phi[i], theta[i], r, x[0], x[2], x[4], sa[2 * i], axis_cos(sa[2 * i], ca[2 * i]), ro, T,
                            dt, re, sh, dr, o);
        else
            full_increments(phi[i], theta[i], r, f2{x[0], x[1]}, f2{x[2], x[3]}, f2{x[4], x[5]},
                            f2{sa[2 * i], sa[2 * i + 1]}, f2{ca[2 * i], ca[2 * i + 1]}, ro, T, dt, re, sh, dr, o);
        double *d = out + 11 * i;
        for (int k = 0; k < 3; ++k) put(d + 2 * k, o.dp[k]);
        put(d + 6, o.a);
        put(d + 8, o.b);
        d[10] = o.direct ? 1.0 : 0.0;
    }
}

// the pair helpers of the full chain: op 0 sqrt_f2(a), 1 div_f2(a, b),
// 2 sin_cosm1_f2(a) (two pairs out), 3 axis_cos(a.h, b.h); a, b: pairs,
// out: 4 doubles a row
extern "C" void xf_helpers(int n, int op, const float *a, const float *b, double *out) {
    for (int i = 0; i < n; ++i) {
        const f2 x = {a[2 * i], a[2 * i + 1]}, y = {b[2 * i], b[2 * i + 1]};
        f2 r0 = {0.0f, 0.0f}, r1 = {0.0f, 0.0f};
        if (op == 0) r0 = sqrt_f2(x);
        else if (op == 1) r0 = div_f2(x, y);
        else if (op == 2) sin_cosm1_f2(x, r0, r1);
        else r0 = axis_cos(x.h, y.h);
        put(out + 4 * i, r0);
        put(out + 4 * i + 2, r1);
    }
}
