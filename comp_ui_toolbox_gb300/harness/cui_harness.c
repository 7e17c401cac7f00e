/*
 * cui_harness.c -- plain C driver of libcui_born through its C-ABI only.
 *
 * Builds a small 2D Born operator from the setup form (tables computed on the
 * GPU), applies forward and adjoint to host FP64 buffers (the MEX gateway's
 * semantics, cui_born_combined_host), checks the dot-product identity
 * <Phi x, y> = <x, Phi^H y> and the VJP, and prints one JSON line.
 *
 *   cc -O2 -I include cui_harness.c -L comp_ui_toolbox_gb300 -lcui_born -lm -o cui_harness
 *   ./cui_harness [n_x n_z n_elements n_frequencies]
 *
 * Exit status 0 when every check passes.
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "cui_born.h"

#define CHECK(call)                                                                        \
    do {                                                                                   \
        cui_status s_ = (call);                                                            \
        if (s_ != CUI_OK) {                                                                \
            fprintf(stderr, "%s failed: %s (%s)\n", #call, cui_status_string(s_), cui_last_error()); \
            return 2;                                                                      \
        }                                                                                  \
    } while (0)

static double urand(unsigned long long* state) { /* xorshift64*, uniform in [-1, 1) */
    *state ^= *state >> 12;
    *state ^= *state << 25;
    *state ^= *state >> 27;
    return (double)((*state * 2685821657736338717ULL) >> 11) / 4503599627370496.0 - 1.0;
}

int main(int argc, char** argv) {
    const int nx = argc > 1 ? atoi(argv[1]) : 96;
    const int nz = argc > 2 ? atoi(argv[2]) : 64;
    const int ne = argc > 3 ? atoi(argv[3]) : 16;
    const int nf = argc > 4 ? atoi(argv[4]) : 8;
    const double dx = 76.2e-6, pitch = 4 * 76.2e-6, c = 1500.0;
    const double pi = 3.14159265358979323846;

    double* f = malloc(sizeof(double) * nf);
    int32_t* fidx = malloc(sizeof(int32_t) * nf);
    for (int i = 0; i < nf; ++i) {
        f[i] = 2.5e6 + 3.0e6 * i / (nf > 1 ? nf - 1 : 1);
        fidx[i] = i + 1;
    }
    /* one quasi-plane wave steered 10 degrees, delays quantised to the 80 MHz clock */
    cui_complex64* vd = malloc(sizeof(cui_complex64) * nf * ne);
    double tmin = 1e30;
    double* tau = malloc(sizeof(double) * ne);
    for (int e = 0; e < ne; ++e) {
        tau[e] = (e - 0.5 * (ne - 1)) * pitch * sin(10.0 * pi / 180.0) / c;
        if (tau[e] < tmin) tmin = tau[e];
    }
    for (int e = 0; e < ne; ++e) {
        const double t = round((tau[e] - tmin) * 80e6) / 80e6;
        for (int i = 0; i < nf; ++i) {
            vd[e * nf + i].re = cos(-2 * pi * f[i] * t);
            vd[e * nf + i].im = sin(-2 * pi * f[i] * t);
        }
    }
    /* identity receive mixing: one mix per element, unit response */
    cui_mix_desc* mixes = malloc(sizeof(cui_mix_desc) * ne);
    int32_t* act = malloc(sizeof(int32_t) * ne);
    cui_complex64* resp = malloc(sizeof(cui_complex64) * nf);
    for (int i = 0; i < nf; ++i) {
        resp[i].re = 1.0;
        resp[i].im = 0.0;
    }
    for (int e = 0; e < ne; ++e) {
        act[e] = e + 1;
        mixes[e].n_f = nf;
        mixes[e].indices_f_to_unique = fidx;
        mixes[e].n_active = 1;
        mixes[e].indices_active = &act[e];
        mixes[e].prefactors = resp;
    }
    cui_wave_desc wave = {nf, fidx, vd, ne, mixes};
    cui_born_setup_desc d;
    memset(&d, 0, sizeof(d));
    d.n_dims = 2;
    d.n_points_axis[0] = nx;
    d.n_points_axis[1] = nz;
    d.delta_axis[0] = dx;
    d.delta_axis[1] = dx;
    d.z_start = 5e-3;
    d.n_elements_axis[0] = ne;
    d.pitch_axis[0] = pitch;
    d.width_axis[0] = 279.8e-6;
    d.n_face_axis[0] = 1;
    d.absorption.kind = CUI_ABSORPTION_TIME_CAUSAL;
    d.absorption.c = c;
    d.absorption.slope_db = 0.5;
    d.absorption.exponent = 1.0;
    d.absorption.f_ref = 4e6;
    d.absorption.dispersion = 1;
    d.aa_tx_beta = 0.5;
    d.aa_rx_beta = 0.5;
    d.n_f_unique = nf;
    d.f_unique = f;
    d.n_measurements = 1;
    d.waves = &wave;
    d.device = 0;

    cui_born_plan* plan = NULL;
    CHECK(cui_born_plan_create_setup(&d, 1, &plan));
    int64_t n_obs = 0, n_pts = 0;
    CHECK(cui_born_size(plan, &n_obs, &n_pts));

    cui_complex64* x = malloc(sizeof(cui_complex64) * n_pts);
    cui_complex64* ax = malloc(sizeof(cui_complex64) * n_obs);
    cui_complex64* y = malloc(sizeof(cui_complex64) * n_obs);
    cui_complex64* ahy = malloc(sizeof(cui_complex64) * n_pts);
    cui_complex64* grad = malloc(sizeof(cui_complex64) * n_pts);
    unsigned long long st = 88172645463325252ULL;
    for (int64_t i = 0; i < n_pts; ++i) {
        x[i].re = urand(&st);
        x[i].im = urand(&st);
    }
    for (int64_t i = 0; i < n_obs; ++i) {
        y[i].re = urand(&st);
        y[i].im = urand(&st);
    }
    CHECK(cui_born_combined_host(plan, 1, x, n_pts, 1, ax, n_obs));
    CHECK(cui_born_combined_host(plan, 2, y, n_obs, 1, ahy, n_pts));
    /* <Phi x, y> = sum conj(y) Phi x ;  <x, Phi^H y> = sum conj(Phi^H y) x */
    double lr = 0, li = 0, rr = 0, ri = 0, nax = 0, ny = 0;
    for (int64_t i = 0; i < n_obs; ++i) {
        lr += y[i].re * ax[i].re + y[i].im * ax[i].im;
        li += y[i].re * ax[i].im - y[i].im * ax[i].re;
        nax += ax[i].re * ax[i].re + ax[i].im * ax[i].im;
        ny += y[i].re * y[i].re + y[i].im * y[i].im;
    }
    for (int64_t i = 0; i < n_pts; ++i) {
        rr += ahy[i].re * x[i].re + ahy[i].im * x[i].im;
        ri += ahy[i].re * x[i].im - ahy[i].im * x[i].re;
    }
    const double dot_err = hypot(lr - rr, li - ri) / (sqrt(nax) * sqrt(ny));
    /* VJP at x with data Phi x: the residual vanishes, so loss and gradient are zero */
    double loss = -1.0;
    CHECK(cui_born_vjp_host(plan, x, n_pts, ax, n_obs, 1, grad, n_pts, &loss));
    double gn = 0.0;
    for (int64_t i = 0; i < n_pts; ++i) gn += grad[i].re * grad[i].re + grad[i].im * grad[i].im;
    const int ok = dot_err < 1e-6 && loss == 0.0 && gn == 0.0 && nax > 0.0;
    printf("{\"n_points\": %lld, \"n_observations\": %lld, \"dot_product_rel_err\": %.3e, \"vjp_loss_at_solution\": %.3e, "
           "\"launches\": %lld, \"ok\": %s}\n",
           (long long)n_pts, (long long)n_obs, dot_err, loss, (long long)cui_launch_count(), ok ? "true" : "false");
    CHECK(cui_born_plan_destroy(plan));
    free(f); free(fidx); free(vd); free(tau); free(mixes); free(act); free(resp);
    free(x); free(ax); free(y); free(ahy); free(grad);
    return ok ? 0 : 1;
}
