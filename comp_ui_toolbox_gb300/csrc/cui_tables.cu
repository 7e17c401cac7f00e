// Device-side construction of the operator's tables from physical parameters.
//
// The reference computes its tables once per operator on the host in FP64
// (+scattering/operator.m:76-88): the reference element's transfer function
// (+scattering/+sequences/+setups/setup.m:1216-1281 with the Green's function
// of +processing/greens_function.m:88/103 and the anti-aliasing window of
// +scattering/+anti_aliasing_filters/on.m:64-70, raised_cosine.m:106-119), the
// incident fields (+scattering/+sequences/sequence.m:813-844) and the
// prefactors (setup.m:759, sequence.m:623).  cui_born_plan_create_setup does
// the same on the GPU:
//   * the lateral-offset table (one thread per entry), stored in FP32:
//     distances and phases in FP64, the rest in FP32; the 2D Green's function
//     needs H0^(2) of a complex argument, evaluated here from its power series
//     (DLMF 10.8.2, FP64) for |z| < 16 and from Hankel's asymptotic expansion
//     (DLMF 10.17.4, FP32 on the FP64-reduced phase) above;
//   * the incident field of every (wave, frequency) as the sum over transmit
//     elements of table rows shifted by the element offset, weighted by the
//     normal velocities v_d;
//   * the prefactors -dV k~(f)^2 times the caller's receive responses.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <string>
#include <vector>

#include "cui_internal.cuh"

namespace cui {
namespace {

// ---- complex FP64 helpers -----------------------------------------------------
__host__ __device__ inline double2 cadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__host__ __device__ inline double2 cmul(double2 a, double2 b) {
    return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__host__ __device__ inline double2 cscale(double2 a, double s) { return make_double2(a.x * s, a.y * s); }
__device__ inline double2 cinv(double2 a) {
    const double d = a.x * a.x + a.y * a.y;
    return make_double2(a.x / d, -a.y / d);
}
__device__ inline double cabsd(double2 a) { return hypot(a.x, a.y); }
// principal square root
__device__ inline double2 csqrt(double2 a) {
    const double r = hypot(a.x, a.y);
    double re = sqrt(0.5 * (r + fabs(a.x)));
    double im = (re > 0.0) ? 0.5 * a.y / re : 0.0;
    if (a.x < 0.0) {  // rotate into the right half-plane
        const double t = re;
        re = fabs(im);
        im = copysign(t, a.y);
    }
    return make_double2(re, im);
}
// exp(-i z) for z = x + i y  ->  exp(y) (cos x - i sin x)
__device__ inline double2 cexp_minus_i(double2 z) {
    double s, c;
    sincos(z.x, &s, &c);
    const double m = exp(z.y);
    return make_double2(m * c, -m * s);
}
__device__ inline double2 clog(double2 z) { return make_double2(log(hypot(z.x, z.y)), atan2(z.y, z.x)); }

constexpr double kPi = 3.14159265358979323846;
constexpr double kEulerGamma = 0.57721566490153286061;
constexpr double kHankelSwitch = 16.0;

// H0^(2)(z) for Re z > 0, Im z <= 0 (absorbing media).
__device__ double2 hankel2_0(double2 z) {
    if (cabsd(z) >= kHankelSwitch) {
        // DLMF 10.17.4: H0^(2)(z) ~ sqrt(2/(pi z)) exp(-i(z - pi/4)) sum_k (-i)^k a_k(0) / z^k,
        // a_k(0)/a_{k-1}(0) = -(2k-1)^2/(8k); the sum is truncated at its smallest term.
        const double2 w = cinv(z);
        double2 term = make_double2(1.0, 0.0), sum = term;
        double prev = 1.0;
        for (int k = 1; k < 64; ++k) {
            const double c = (2.0 * k - 1.0) * (2.0 * k - 1.0) / (8.0 * k);
            const double2 next = cmul(cmul(term, make_double2(0.0, c)), w);  // * (-i) * (-(2k-1)^2/(8k)) / z
            const double mag = cabsd(next);
            if (mag >= prev) break;
            term = next;
            sum = cadd(sum, term);
            prev = mag;
            if (mag < 1e-17 * cabsd(sum)) break;
        }
        const double2 pre = csqrt(cscale(cinv(z), 2.0 / kPi));
        const double2 ph = cmul(cexp_minus_i(z), make_double2(0.70710678118654752440, 0.70710678118654752440));
        return cmul(cmul(pre, ph), sum);
    }
    // DLMF 10.2.2 / 10.8.2: J0 = sum (-q)^k/(k!)^2, Y0 = (2/pi)(ln(z/2)+gamma) J0 + (2/pi) sum_{k>=1} (-1)^{k+1} H_k q^k/(k!)^2,
    // q = z^2/4, H_k the harmonic numbers; H0^(2) = J0 - i Y0.
    const double2 q = cscale(cmul(z, z), 0.25);
    double2 t = make_double2(1.0, 0.0), J = t, Ys = make_double2(0.0, 0.0);
    double H = 0.0;
    for (int k = 1; k < 80; ++k) {
        t = cscale(cmul(t, make_double2(-q.x, -q.y)), 1.0 / (static_cast<double>(k) * k));
        H += 1.0 / k;
        J = cadd(J, t);
        Ys = cadd(Ys, cscale(t, -H));
        if (k > 4 && cabsd(t) < 1e-18 * cabsd(J)) break;
    }
    const double2 L = clog(cscale(z, 0.5));
    const double2 Y = cadd(cscale(cmul(make_double2(L.x + kEulerGamma, L.y), J), 2.0 / kPi), cscale(Ys, 2.0 / kPi));
    return make_double2(J.x + Y.y, J.y - Y.x);  // J - i Y
}

// raised-cosine roll-off (raised_cosine.m:106-119); the cosine of the transition band in FP32
__device__ inline double raised_cosine(double flag, double beta) {
    const double lb = kPi * (1.0 - beta);
    if (flag <= lb) return 1.0;
    if (flag >= kPi) return 0.0;
    return 0.5 * (1.0 + static_cast<double>(cosf(static_cast<float>(kPi * (flag - lb) / (kPi - lb)))));
}

// ---- table entries: FP64 where FP32 cannot carry the accuracy, FP32 elsewhere ------------------
// The table is stored in FP32.  Its entries need the distance D and the phase k~ D in FP64 (k~ D
// reaches 10^3-10^4 rad); once the phase is reduced modulo 2 pi in FP64, its sine and cosine, the
// attenuation, the prefactor and the asymptotic series of the Hankel function are FP32 work.
// This GPU's FP64 rate is a small fraction of its FP32 rate, and the all-FP64 entry cost about a
// thousand FP64 operations.
constexpr double kTwoPi = 6.283185307179586476925;

__device__ inline float2 cmulf(float2 a, float2 b) { return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x); }

// principal square root, FP32
__device__ inline float2 csqrtf_principal(float2 a) {
    const float r = hypotf(a.x, a.y);
    float re = sqrtf(0.5f * (r + fabsf(a.x)));
    float im = (re > 0.f) ? 0.5f * a.y / re : 0.f;
    if (a.x < 0.f) {
        const float t = re;
        re = fabsf(im);
        im = copysignf(t, a.y);
    }
    return make_float2(re, im);
}

// exp(y) (cos x - i sin x) for a phase x of any size: x - n 2 pi with n = rint(x / 2 pi) by one FP64
// FMA (its error, |n| times that of fl(2 pi), stays below 1e-11 rad for |x| < 1e5), then FP32 sine
// and cosine of the reduced phase in [-pi, pi]
__device__ inline float2 exp_minus_i_f32(double x, double y) {
    const double n = rint(x * (1.0 / kTwoPi));
    const float r = static_cast<float>(fma(-n, kTwoPi, x));
    float sn, cs;
    sincosf(r, &sn, &cs);
    const float m = expf(static_cast<float>(y));
    return make_float2(m * cs, -m * sn);
}

// H0^(2)(z) of a table entry: for |z| >= 16 Hankel's expansion (DLMF 10.17.4) in FP32 with the
// phase reduced in FP64; nearer the array the FP64 power series of hankel2_0 (its terms cancel).
__device__ inline double2 hankel2_0_entry(double2 z) {
    if (z.x * z.x + z.y * z.y < kHankelSwitch * kHankelSwitch) return hankel2_0(z);
    const float2 zf = make_float2(static_cast<float>(z.x), static_cast<float>(z.y));
    const float d = zf.x * zf.x + zf.y * zf.y;
    const float2 w = make_float2(zf.x / d, -zf.y / d);  // 1/z
    float2 term = make_float2(1.f, 0.f), sum = term;
    float prev = 1.f;  // squared magnitude of the last term
    for (int k = 1; k < 32; ++k) {
        const float c = (2.f * k - 1.f) * (2.f * k - 1.f) / (8.f * k);
        const float2 next = cmulf(cmulf(term, make_float2(0.f, c)), w);  // * (-i) * (-(2k-1)^2/(8k)) / z
        const float mag = next.x * next.x + next.y * next.y;
        if (mag >= prev) break;  // truncated at the smallest term
        term = next;
        sum.x += term.x;
        sum.y += term.y;
        prev = mag;
        if (mag < 1e-15f) break;  // below FP32 resolution of a sum close to 1
    }
    const float2 pre = csqrtf_principal(make_float2(w.x * static_cast<float>(2.0 / kPi), w.y * static_cast<float>(2.0 / kPi)));
    const float2 r = cmulf(cmulf(pre, exp_minus_i_f32(z.x - 0.25 * kPi, z.y)), sum);
    return make_double2(r.x, r.y);
}

struct TableArgs {
    int n_dims, F, Nz, Noy, Nox, Ex, Ey, Qx, Qy;
    double dx, dy, dz, z_start, pitch_x, pitch_y, wx, wy, dA, beta;
    const double2* k;   // [F]
    const double2* w;   // [F][Qy * Qx] face weights, or nullptr (uniform)
    float2* out;        // [F][Nz][Noy][Nox]
    int* bad;           // set when an entry is not finite
};

// one thread per entry (f, z, oy, ox); distances and phases in FP64, the rest in FP32 (see above),
// FP32 store
__global__ void table_kernel(const TableArgs a) {
    const int64_t n = static_cast<int64_t>(a.F) * a.Nz * a.Noy * a.Nox;
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const int ox = static_cast<int>(i % a.Nox);
        int64_t t = i / a.Nox;
        const int oy = static_cast<int>(t % a.Noy);
        t /= a.Noy;
        const int z = static_cast<int>(t % a.Nz);
        const int f = static_cast<int>(t / a.Nz);
        const double X = (ox - 0.5 * (a.Nox - 1)) * a.dx;
        const double Y = (a.n_dims == 3) ? (oy - 0.5 * (a.Noy - 1)) * a.dy : 0.0;
        const double Z = a.z_start + (z + 0.5) * a.dz;
        const double2 k = a.k[f];
        double2 sum = make_double2(0.0, 0.0);
        for (int qy = 0; qy < a.Qy; ++qy) {
            const double fy = (a.n_dims == 3) ? (qy - 0.5 * (a.Qy - 1)) * (a.wy / a.Qy) : 0.0;
            for (int qx = 0; qx < a.Qx; ++qx) {
                const double fx = (qx - 0.5 * (a.Qx - 1)) * (a.wx / a.Qx);
                const double D = sqrt((X - fx) * (X - fx) + (Y - fy) * (Y - fy) + Z * Z);
                const double2 kD = cscale(k, D);
                double2 G;
                if (a.n_dims == 2) {
                    const double2 h = hankel2_0_entry(kD);
                    G = make_double2(-0.25 * h.y, 0.25 * h.x);  // 0.25j * H0^(2)(kD)
                } else {                                         // -exp(-j k D)/(4 pi D)
                    const float2 e = exp_minus_i_f32(kD.x, kD.y);
                    G = cscale(make_double2(e.x, e.y), -1.0 / (4.0 * kPi * D));
                }
                if (a.w) G = cmul(G, a.w[(static_cast<int64_t>(f) * a.Qy + qy) * a.Qx + qx]);
                sum = cadd(sum, G);
            }
        }
        double w = 1.0;
        if (a.beta >= 0.0) {
            const double dist = sqrt(X * X + Y * Y + Z * Z);
            if (a.Ex > 1) w *= raised_cosine(k.x * a.pitch_x * fabs(X) / dist, a.beta);
            if (a.n_dims == 3 && a.Ey > 1) w *= raised_cosine(k.x * a.pitch_y * fabs(Y) / dist, a.beta);
        }
        const double2 v = cscale(sum, -2.0 * a.dA * w);
        if (!isfinite(v.x) || !isfinite(v.y)) *a.bad = 1;
        a.out[i] = make_float2(static_cast<float>(v.x), static_cast<float>(v.y));
    }
}

struct PinArgs {
    int Nx, Ny, Nz, Ex, Ey, ppx, ppy, Nox, Noy;
    int64_t P;
    const float2* table;   // transmit table of frequencies f0 .. f0+nf-1: [nf][Nz][Noy][Nox]
    const float2* vd;      // [S][E]
    const int* slot_f;     // [S]
    int f0, nf;
    float2* p_in;          // [S][P]
};

// p_in[s][p] = sum_e T_tx[f_s][z][o(p, e)] * v_d[s][e]; block = (line, slot, x chunk), thread = x
__global__ void __launch_bounds__(256) incident_kernel(const PinArgs a) {
    extern __shared__ float2 sm[];
    float2* srow = sm;             // [Nox]
    float2* svd = sm + a.Nox;      // [Ex]
    const int line = blockIdx.x, s = blockIdx.y;
    const int iy = line % a.Ny, z = line / a.Ny;
    const int f = a.slot_f[s] - a.f0;
    if (f < 0 || f >= a.nf) return;  // slot of another frequency chunk (uniform over the block)
    const int64_t pt0 = (static_cast<int64_t>(z) * a.Ny + iy) * a.Nx;
    const int x = blockIdx.z * blockDim.x + threadIdx.x;
    float2 acc = make_float2(0.f, 0.f);
    for (int ey = 0; ey < a.Ey; ++ey) {
        const int oy = iy - ey * a.ppy + (a.Ey - 1) * a.ppy;
        const float2* row = a.table + ((static_cast<int64_t>(f) * a.Nz + z) * a.Noy + oy) * a.Nox;
        __syncthreads();
        for (int i = threadIdx.x; i < a.Nox; i += blockDim.x) srow[i] = row[i];
        for (int i = threadIdx.x; i < a.Ex; i += blockDim.x) svd[i] = a.vd[static_cast<int64_t>(s) * a.Ex * a.Ey + i + a.Ex * ey];
        __syncthreads();
        if (x < a.Nx) {
            const int o0 = x + (a.Ex - 1) * a.ppx;
            for (int ex = 0; ex < a.Ex; ++ex) {
                const float2 h = srow[o0 - ex * a.ppx];
                const float2 v = svd[ex];
                acc.x = fmaf(h.x, v.x, fmaf(-h.y, v.y, acc.x));
                acc.y = fmaf(h.x, v.y, fmaf(h.y, v.x, acc.y));
            }
        }
    }
    if (x < a.Nx) a.p_in[static_cast<int64_t>(s) * a.P + pt0 + x] = acc;
}

// complex wavenumbers k~(f): +scattering/+sequences/+setups/+materials/+absorption_models/
// none.m:83 and time_causal.m:82-83, :118-147
std::vector<double2> wavenumbers(const cui_absorption_desc& a, const double* f, int F, cui_status* st) {
    std::vector<double2> k(F);
    *st = CUI_OK;
    if (!(a.c > 0.0)) {
        *st = set_error(CUI_ERR_INVALID_ARG, "absorption.c must be positive");
        return k;
    }
    if (a.kind == CUI_ABSORPTION_NONE) {
        for (int i = 0; i < F; ++i) k[i] = make_double2(2.0 * kPi * f[i] / a.c, 0.0);
        return k;
    }
    if (a.kind != CUI_ABSORPTION_TIME_CAUSAL) {
        *st = set_error(CUI_ERR_INVALID_ARG, "unknown absorption model");
        return k;
    }
    const double alpha_0 = a.constant_db * std::log(10.0) / (20.0 * 0.01);
    const double alpha_1 = a.slope_db * std::log(10.0) / (20.0 * 0.01 * std::pow(1e6, a.exponent));
    const double y = a.exponent;
    for (int i = 0; i < F; ++i) {
        const double fi = f[i];
        const double k_ref = 2.0 * kPi * fi / a.c;
        const double k_imag = -alpha_0 - alpha_1 * std::pow(std::fabs(fi), y);
        double k_real = k_ref;
        if (a.dispersion) {
            if (std::fmod(y, 2.0) == 0.0 || std::floor(y) != y)
                k_real = k_ref + alpha_1 * std::tan(y * kPi / 2.0) * fi *
                                     (std::pow(std::fabs(fi), y - 1.0) - std::pow(std::fabs(a.f_ref), y - 1.0));
            else
                k_real = k_ref - 2.0 * alpha_1 * std::pow(fi, y) * std::log(std::fabs(fi / a.f_ref)) / kPi;
        }
        if (std::fabs(fi) < 2.220446049250313e-16) k_real = 0.0;
        k[i] = make_double2(k_real, k_imag);
    }
    return k;
}

int points_per_pitch(double pitch, double delta, bool* ok) {
    const double r = pitch / delta;
    const double n = std::round(r);
    *ok = (n >= 1.0) && std::fabs(r - n) <= 1e-9 * n;
    return static_cast<int>(n);
}

#define CUI_TRY(x) do { cudaError_t e_ = (x); if (e_ != cudaSuccess) return check_cuda(e_, #x); } while (0)

// Face weights w[f][q] = a_q exp(-j k_lens(f) t_q) of every frequency and face point
// (face.m:359-376 compute_weights_scalar), q = qy * Qx + qx.  The lens thickness restates
// thickness/focus_axial.m at the face point's normalised position rho = 2 (r_q - r_c) / width =
// (2 q_a - Q_a + 1) / Q_a along each axis: t = sum over the focused axes of
// (sqrt(1 + F^2) - sqrt(rho^2 + F^2)) width / 2 with F = 2 focus / width; the lens is lossless,
// k_lens = 2 pi f / c_lens (lens.m).  Empty for uniform weights (no apodization, no focus).
std::vector<double2> face_weights(const cui_born_setup_desc* d, int F, cui_status* st) {
    *st = CUI_OK;
    const int nl = d->n_dims - 1;
    const int Qx = std::max(1, d->n_face_axis[0]), Qy = (nl == 2) ? std::max(1, d->n_face_axis[1]) : 1;
    bool focused = false;
    for (int a = 0; a < nl; ++a) {
        const double fa = d->lens_focus_axis[a];
        if (std::isnan(fa) || fa < 0.0) {
            *st = set_error(CUI_ERR_INVALID_ARG, "lens focus must be 0, +inf or positive");
            return {};
        }
        focused = focused || (fa > 0.0 && std::isfinite(fa));
    }
    if (!d->face_apodization && !focused) return {};
    if (d->lens_c < 0.0 || std::isnan(d->lens_c)) {
        *st = set_error(CUI_ERR_INVALID_ARG, "lens speed of sound must be 0 (1540 m/s) or positive");
        return {};
    }
    const double c_lens = d->lens_c > 0.0 ? d->lens_c : 1540.0;
    const int Q = Qx * Qy;
    std::vector<double> amp(Q, 1.0), thick(Q, 0.0);
    for (int qy = 0; qy < Qy; ++qy)
        for (int qx = 0; qx < Qx; ++qx) {
            const int q = qy * Qx + qx;
            if (d->face_apodization) {
                amp[q] = d->face_apodization[q];
                if (!std::isfinite(amp[q])) {
                    *st = set_error(CUI_ERR_NUMERIC, "non-finite face apodization");
                    return {};
                }
            }
            const int qa[2] = {qx, qy}, Qa[2] = {Qx, Qy};
            for (int a = 0; a < nl; ++a) {
                const double fa = d->lens_focus_axis[a];
                if (!(fa > 0.0 && std::isfinite(fa))) continue;
                const double wa = d->width_axis[a];
                const double rho = (2.0 * qa[a] - Qa[a] + 1.0) / Qa[a];
                const double Fn = 2.0 * fa / wa;
                thick[q] += (std::sqrt(1.0 + Fn * Fn) - std::sqrt(rho * rho + Fn * Fn)) * wa / 2.0;
            }
        }
    std::vector<double2> w(static_cast<size_t>(F) * Q);
    for (int f = 0; f < F; ++f) {
        const double k_lens = 2.0 * kPi * d->f_unique[f] / c_lens;
        for (int q = 0; q < Q; ++q) {
            const double ph = k_lens * thick[q];
            w[static_cast<size_t>(f) * Q + q] = make_double2(amp[q] * std::cos(ph), -amp[q] * std::sin(ph));
        }
    }
    return w;
}

// table entries of the nf frequencies whose wavenumbers start at dk (face weights at dw, or
// nullptr for uniform ones), into out [nf][Nz][Noy][Nox]
cui_status launch_table(Plan& p, const cui_born_setup_desc* d, const double2* dk, const double2* dw, int nf,
                        double beta, float2* out, int* dbad) {
    TableArgs a;
    a.n_dims = p.n_dims; a.F = nf; a.Nz = p.Nz; a.Noy = p.Noy; a.Nox = p.Nox; a.Ex = p.Ex; a.Ey = p.Ey;
    a.Qx = std::max(1, d->n_face_axis[0]);
    a.Qy = (p.n_dims == 3) ? std::max(1, d->n_face_axis[1]) : 1;
    a.dx = d->delta_axis[0];
    a.dy = (p.n_dims == 3) ? d->delta_axis[1] : 0.0;
    a.dz = d->delta_axis[p.n_dims - 1];
    a.z_start = d->z_start;
    a.pitch_x = d->pitch_axis[0];
    a.pitch_y = (p.n_dims == 3) ? d->pitch_axis[1] : 0.0;
    a.wx = d->width_axis[0];
    a.wy = (p.n_dims == 3) ? d->width_axis[1] : 0.0;
    a.dA = (a.wx / a.Qx) * ((p.n_dims == 3) ? a.wy / a.Qy : 1.0);
    a.beta = beta;
    a.k = dk;
    a.w = dw;
    a.out = out;
    a.bad = dbad;
    const int64_t n = static_cast<int64_t>(nf) * p.Nz * p.Noy * p.Nox;
    const int blocks = static_cast<int>(std::min<int64_t>((n + 255) / 256, 152 * 64));
    table_kernel<<<blocks, 256>>>(a);
    count_launch();
    CUI_TRY(cudaGetLastError());
    return CUI_OK;
}

// Parameters of the generated table (cui_gen.cuh): per frequency the wavenumber with its real part
// split into an FP32 pair; per lateral offset and face quadrature point the squared distance, and per
// row the squared depth, computed in FP64 like table_kernel and split into FP32 pairs.
cui_status build_generator(Plan& p, const cui_born_setup_desc* d, const std::vector<double2>& k,
                           const std::vector<double2>& wq) {
    const int Qx = std::max(1, d->n_face_axis[0]), Qy = std::max(1, d->n_face_axis[1]);
    const double dx = d->delta_axis[0], dy = d->delta_axis[1], dz = d->delta_axis[2];
    const double wx = d->width_axis[0], wy = d->width_axis[1];
    auto split = [](double v) {
        const float hi = static_cast<float>(v);
        return make_float2(hi, static_cast<float>(v - static_cast<double>(hi)));
    };
    std::vector<float4> fk(p.F);
    for (int f = 0; f < p.F; ++f) {
        const float2 kr = split(k[f].x);
        fk[f] = make_float4(kr.x, kr.y, static_cast<float>(k[f].y), kr.x);
    }
    std::vector<float2> sx2(static_cast<size_t>(Qx) * p.Nox), sy2(static_cast<size_t>(Qy) * p.Noy), sz2(p.Nz);
    std::vector<float> ax(p.Nox), ay(p.Noy);
    for (int ox = 0; ox < p.Nox; ++ox) {
        const double X = (ox - 0.5 * (p.Nox - 1)) * dx;
        ax[ox] = static_cast<float>(std::fabs(X));
        for (int q = 0; q < Qx; ++q) {
            const double fx = (q - 0.5 * (Qx - 1)) * (wx / Qx);
            sx2[static_cast<size_t>(q) * p.Nox + ox] = split((X - fx) * (X - fx));
        }
    }
    for (int oy = 0; oy < p.Noy; ++oy) {
        const double Y = (oy - 0.5 * (p.Noy - 1)) * dy;
        ay[oy] = static_cast<float>(std::fabs(Y));
        for (int q = 0; q < Qy; ++q) {
            const double fy = (q - 0.5 * (Qy - 1)) * (wy / Qy);
            sy2[static_cast<size_t>(q) * p.Noy + oy] = split((Y - fy) * (Y - fy));
        }
    }
    for (int z = 0; z < p.Nz; ++z) {
        const double Z = d->z_start + (z + 0.5) * dz;
        sz2[z] = split(Z * Z);
    }
    cui_status st;
    auto up = [&](void** dst, const void* src, size_t bytes) -> cui_status {
        cui_status s2 = device_alloc(p, dst, bytes);
        if (s2 != CUI_OK) return s2;
        return check_cuda(cudaMemcpy(*dst, src, bytes, cudaMemcpyHostToDevice), "generated table parameters");
    };
    float4* dfk = nullptr;
    float2 *dsx = nullptr, *dsy = nullptr, *dsz = nullptr;
    float *dax = nullptr, *day = nullptr;
    if ((st = up(reinterpret_cast<void**>(&dfk), fk.data(), sizeof(float4) * fk.size())) != CUI_OK ||
        (st = up(reinterpret_cast<void**>(&dsx), sx2.data(), sizeof(float2) * sx2.size())) != CUI_OK ||
        (st = up(reinterpret_cast<void**>(&dsy), sy2.data(), sizeof(float2) * sy2.size())) != CUI_OK ||
        (st = up(reinterpret_cast<void**>(&dsz), sz2.data(), sizeof(float2) * sz2.size())) != CUI_OK ||
        (st = up(reinterpret_cast<void**>(&dax), ax.data(), sizeof(float) * ax.size())) != CUI_OK ||
        (st = up(reinterpret_cast<void**>(&day), ay.data(), sizeof(float) * ay.size())) != CUI_OK)
        return st;
    float2* dwq = nullptr;
    if (!wq.empty()) {  // face weights [F][Q] in FP32
        std::vector<float2> wf(wq.size());
        for (size_t i = 0; i < wq.size(); ++i) wf[i] = make_float2(static_cast<float>(wq[i].x), static_cast<float>(wq[i].y));
        if ((st = up(reinterpret_cast<void**>(&dwq), wf.data(), sizeof(float2) * wf.size())) != CUI_OK) return st;
    }
    TableGen& t = p.gen;
    t.fk = dfk; t.sx2 = dsx; t.sy2 = dsy; t.sz2 = dsz; t.ax = dax; t.ay = day; t.wq = dwq;
    t.Nox = p.Nox; t.Noy = p.Noy; t.Qx = Qx; t.Qy = Qy;
    t.scale = static_cast<float>((wx / Qx) * (wy / Qy) / (2.0 * kPi));  // -2 dA * (-1 / (4 pi))
    t.pitch_x = static_cast<float>(d->pitch_axis[0]);
    t.pitch_y = static_cast<float>(d->pitch_axis[1]);
    const double beta = d->aa_rx_beta;
    t.win_x = (beta >= 0.0 && p.Ex > 1) ? 1 : 0;
    t.win_y = (beta >= 0.0 && p.Ey > 1) ? 1 : 0;
    t.lb = static_cast<float>(kPi * (1.0 - beta));
    t.inv_span = beta > 0.0 ? static_cast<float>(1.0 / (kPi * beta)) : 0.f;  // beta = 0: no transition band
    return CUI_OK;
}

// transmit-table chunks of a plan whose table is not stored (and of a stored plan whose two
// filters differ)
constexpr size_t kTxChunkBytes = size_t(1) << 30;
// chunk buffer of a streamed table, and the adjoint partial sums that its frequency chunks need
constexpr size_t kStreamBytes = size_t(512) << 20;
constexpr size_t kStreamPartBytes = size_t(1) << 30;

// Frequencies per streamed chunk: what fits the chunk buffer, capped by CUI_BORN_STREAM_FREQUENCIES,
// but no more chunks than the adjoint's partial sums (one slab of max_objects x P per chunk) allow;
// and no more frequencies than the adjoint already takes per block.  The adjoint's frequency chunks
// become the streamed chunks.
int stream_frequencies(const Plan& p, size_t fbytes) {
    int nf = static_cast<int>(std::max<size_t>(1, std::min<size_t>(p.F, kStreamBytes / fbytes)));
    if (const char* env = std::getenv("CUI_BORN_STREAM_FREQUENCIES")) {
        const int cap = std::atoi(env);
        if (cap > 0) nf = std::min(nf, cap);
    }
    const size_t slab = sizeof(float2) * static_cast<size_t>(p.max_objects) * p.P;
    const int max_chunks = static_cast<int>(std::max<size_t>(1, kStreamPartBytes / slab));
    nf = std::max(nf, (p.F + max_chunks - 1) / max_chunks);
    return std::max(1, std::min(nf, p.adj_fchunk));
}

cui_status create_setup(const cui_born_setup_desc* d, int32_t max_objects, int32_t storage, Plan& p,
                        const char* cache_dir, int32_t* loaded) {
    if (!d) return set_error(CUI_ERR_INVALID_ARG, "desc is NULL");
    if (d->n_dims != 2 && d->n_dims != 3) return set_error(CUI_ERR_INVALID_ARG, "n_dims must be 2 or 3");
    const int nl = d->n_dims - 1;
    int32_t ppp[2] = {1, 1};
    for (int k = 0; k < nl; ++k) {
        if (!(d->delta_axis[k] > 0.0) || !(d->pitch_axis[k] > 0.0) || !(d->width_axis[k] > 0.0))
            return set_error(CUI_ERR_INVALID_ARG, "delta, pitch and width must be positive");
        bool ok = false;
        ppp[k] = points_per_pitch(d->pitch_axis[k], d->delta_axis[k], &ok);
        if (!ok)
            return set_error(CUI_ERR_UNSUPPORTED_SETUP,
                             "element pitch is not an integer multiple of the lateral grid spacing (setup.m:1176-1178)");
    }
    if (!(d->delta_axis[nl] > 0.0) || !(d->z_start >= 0.0))
        return set_error(CUI_ERR_INVALID_ARG, "axial spacing must be positive and z_start non-negative");
    if (!d->f_unique || !d->waves) return set_error(CUI_ERR_INVALID_ARG, "f_unique or waves is NULL");
    cui_status st = init_geometry(p, d->n_dims, d->n_points_axis, d->n_elements_axis, ppp, d->n_f_unique,
                                  d->n_measurements, max_objects);
    if (st != CUI_OK) return st;
    std::vector<double2> k = wavenumbers(d->absorption, d->f_unique, p.F, &st);
    if (st != CUI_OK) return st;
    const std::vector<double2> wq = face_weights(d, p.F, &st);
    if (st != CUI_OK) return st;
    const int Qf = std::max(1, d->n_face_axis[0]) * ((d->n_dims == 3) ? std::max(1, d->n_face_axis[1]) : 1);
    double dV = 1.0;
    for (int a = 0; a < d->n_dims; ++a) dV *= d->delta_axis[a];
    std::vector<double2> scale(p.F);
    for (int f = 0; f < p.F; ++f) scale[f] = cscale(cmul(k[f], k[f]), -dV);  // -dV k~^2 (setup.m:759)
    std::vector<MeasIn> ms(p.W);
    for (int w = 0; w < p.W; ++w) {
        const cui_wave_desc& wd = d->waves[w];
        if (!wd.v_d) return set_error(CUI_ERR_INVALID_ARG, "wave " + std::to_string(w) + " has no v_d");
        ms[w] = MeasIn{wd.n_f, wd.indices_f_to_unique, wd.n_mixes, wd.mixes};
    }
    std::vector<int> slot0;
    if ((st = build_metadata(p, ms, &scale, slot0)) != CUI_OK) return st;
    if ((st = select_device_and_shapes(p, d->device)) != CUI_OK) return st;

    // v_d of every slot, FP32 [S][E]
    std::vector<float2> vd(static_cast<size_t>(p.S) * p.E);
    for (int w = 0; w < p.W; ++w) {
        const cui_wave_desc& wd = d->waves[w];
        for (int e = 0; e < p.E; ++e)
            for (int i = 0; i < wd.n_f; ++i) {
                const cui_complex64 c = wd.v_d[static_cast<int64_t>(e) * wd.n_f + i];
                if (!std::isfinite(c.re) || !std::isfinite(c.im)) return set_error(CUI_ERR_NUMERIC, "non-finite v_d");
                vd[static_cast<size_t>(slot0[w] + i) * p.E + e] = make_float2(static_cast<float>(c.re), static_cast<float>(c.im));
            }
    }

    // scratch for the build (released before returning)
    double2* dk = nullptr;
    double2* dw = nullptr;
    float2* dvd = nullptr;
    int* dslot = nullptr;
    int* dbad = nullptr;
    float2* dtx = nullptr;
    std::vector<void*> tmp;
    auto release = [&]() {
        for (void* v : tmp) cudaFree(v);
        tmp.clear();
    };
    auto talloc = [&](void** ptr, size_t bytes) -> cudaError_t {
        if (injected_alloc_failure(p)) return cudaErrorMemoryAllocation;
        cudaError_t e = cudaMalloc(ptr, std::max<size_t>(bytes, 1));
        if (e == cudaSuccess) tmp.push_back(*ptr);
        return e;
    };
    cudaError_t ce;
    const size_t fbytes = sizeof(float2) * static_cast<size_t>(p.Nz) * p.Noy * p.Nox;  // one frequency
    const size_t tbytes = fbytes * p.F;
    const size_t ibytes = sizeof(float2) * static_cast<size_t>(p.S) * p.P;
    int mode = storage;
    const int stream_nf = stream_frequencies(p, fbytes);
    if (mode == CUI_STORAGE_AUTO) {
        mode = CUI_STORAGE_STORED;
        size_t free_b = 0, total_b = 0;
        if (p.n_dims == 3 && cudaMemGetInfo(&free_b, &total_b) == cudaSuccess && tbytes + ibytes > free_b / 10 * 9)
            mode = (fbytes * stream_nf + ibytes <= free_b / 10 * 9) ? CUI_STORAGE_STREAMED : CUI_STORAGE_GENERATED;
    } else if (mode != CUI_STORAGE_STORED && mode != CUI_STORAGE_GENERATED && mode != CUI_STORAGE_STREAMED) {
        return set_error(CUI_ERR_INVALID_ARG, "unknown table storage");
    }
    if (mode != CUI_STORAGE_STORED && p.n_dims != 3)
        return set_error(CUI_ERR_UNSUPPORTED_SETUP, "a streamed or generated table needs a 3D setup (2D entries are "
                                                    "Hankel functions: too costly to recompute per apply)");
    p.table_mode = mode;
    if (mode == CUI_STORAGE_STORED) {
        if ((st = device_alloc(p, reinterpret_cast<void**>(&p.table), tbytes)) != CUI_OK) return st;
        p.table_bytes = tbytes;
    } else {
        if ((st = build_generator(p, d, k, wq)) != CUI_OK) return st;
        p.table_bytes = 0;
        if (mode == CUI_STORAGE_STREAMED) {
            p.stream_nf = stream_nf;
            p.adj_fchunk = stream_nf;  // the adjoint's frequency chunks are the streamed chunks
            p.adj_nfc = (p.F + stream_nf - 1) / stream_nf;
            p.table_bytes = fbytes * stream_nf;
            if ((st = device_alloc(p, reinterpret_cast<void**>(&p.stream_buf), p.table_bytes)) != CUI_OK) return st;
        }
    }
    if ((st = device_alloc(p, reinterpret_cast<void**>(&p.p_in), ibytes)) != CUI_OK) return st;
    p.incident_bytes = ibytes;
    // compute_or_load_hash.m:65-185: load the arrays from the cache file of this setup if it exists
    // (a generated plan keeps only the incident fields, in a file of its own)
    std::vector<unsigned char> key;
    std::string path;
    if (cache_dir) {
        if ((st = setup_key(d, key)) != CUI_OK) return st;
        path = cache_path(cache_dir, key, mode != CUI_STORAGE_STORED);
        bool hit = false;
        if ((st = cache_load(path, key, p, &hit)) != CUI_OK) return st;
        if (hit) {
            if (loaded) *loaded = 1;
            return upload_metadata_and_workspace(p);
        }
    }
    const bool same_filter = (d->aa_tx_beta < 0.0 && d->aa_rx_beta < 0.0) || (d->aa_tx_beta == d->aa_rx_beta);
    // the transmit table is the stored table itself when both filters agree; else it is built in
    // chunks of frequencies into scratch, each chunk consumed by the incident-field kernel
    const bool own_tx = mode != CUI_STORAGE_STORED || !same_filter;
    const int fchunk = own_tx ? static_cast<int>(std::max<size_t>(1, std::min<size_t>(p.F, kTxChunkBytes / fbytes))) : p.F;
    if ((ce = talloc(reinterpret_cast<void**>(&dk), sizeof(double2) * p.F)) != cudaSuccess ||
        (ce = talloc(reinterpret_cast<void**>(&dvd), sizeof(float2) * vd.size())) != cudaSuccess ||
        (ce = talloc(reinterpret_cast<void**>(&dslot), sizeof(int) * p.S)) != cudaSuccess ||
        (ce = talloc(reinterpret_cast<void**>(&dbad), sizeof(int))) != cudaSuccess ||
        (own_tx && (ce = talloc(reinterpret_cast<void**>(&dtx), fbytes * fchunk)) != cudaSuccess) ||
        (!wq.empty() && (ce = talloc(reinterpret_cast<void**>(&dw), sizeof(double2) * wq.size())) != cudaSuccess)) {
        release();
        return check_cuda(ce, "table build scratch");
    }
    if (!wq.empty() && (ce = cudaMemcpy(dw, wq.data(), sizeof(double2) * wq.size(), cudaMemcpyHostToDevice)) != cudaSuccess) {
        release();
        return check_cuda(ce, "face weights upload");
    }
    if ((ce = cudaMemcpy(dk, k.data(), sizeof(double2) * p.F, cudaMemcpyHostToDevice)) != cudaSuccess ||
        (ce = cudaMemcpy(dvd, vd.data(), sizeof(float2) * vd.size(), cudaMemcpyHostToDevice)) != cudaSuccess ||
        (ce = cudaMemcpy(dslot, p.h_slot_f.data(), sizeof(int) * p.S, cudaMemcpyHostToDevice)) != cudaSuccess ||
        (ce = cudaMemset(dbad, 0, sizeof(int))) != cudaSuccess) {
        release();
        return check_cuda(ce, "table build upload");
    }
    std::vector<float2>().swap(vd);
    if (mode == CUI_STORAGE_STORED) st = launch_table(p, d, dk, dw, p.F, d->aa_rx_beta, p.table, dbad);
    for (int f0 = 0; st == CUI_OK && f0 < p.F; f0 += fchunk) {
        const int nf = std::min(fchunk, p.F - f0);
        if (own_tx) st = launch_table(p, d, dk + f0, dw ? dw + static_cast<size_t>(f0) * Qf : nullptr, nf, d->aa_tx_beta,
                                      dtx, dbad);
        if (st != CUI_OK) break;
        PinArgs a;
        a.Nx = p.Nx; a.Ny = p.Ny; a.Nz = p.Nz; a.Ex = p.Ex; a.Ey = p.Ey; a.ppx = p.ppx; a.ppy = p.ppy;
        a.Nox = p.Nox; a.Noy = p.Noy; a.P = p.P;
        a.table = own_tx ? dtx : p.table;
        a.vd = dvd; a.slot_f = dslot; a.f0 = f0; a.nf = nf; a.p_in = p.p_in;
        const size_t smem = sizeof(float2) * (p.Nox + p.Ex);
        const int tpb = 256;
        dim3 grid(p.Ny * p.Nz, p.S, (p.Nx + tpb - 1) / tpb);
        if (smem > 48 * 1024) cudaFuncSetAttribute(incident_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
        incident_kernel<<<grid, tpb, smem>>>(a);
        count_launch();
        if ((ce = cudaGetLastError()) != cudaSuccess) st = check_cuda(ce, "incident field");
    }
    int bad = 0;
    if (st == CUI_OK) {
        if ((ce = cudaMemcpy(&bad, dbad, sizeof(int), cudaMemcpyDeviceToHost)) != cudaSuccess)
            st = check_cuda(ce, "table build");
        else if (bad)
            st = set_error(CUI_ERR_NUMERIC, "non-finite transfer-function table entry");
    }
    release();
    if (st != CUI_OK) return st;
    if (cache_dir) {  // a failed store keeps the plan: *loaded = -1, the reason in cui_last_error()
        const cui_status cs = cache_store(path, key, p);
        if (loaded) *loaded = cs == CUI_OK ? 0 : -1;
    }
    return upload_metadata_and_workspace(p);
}
#undef CUI_TRY

}  // namespace
}  // namespace cui

namespace {
cui_status create_setup_plan(const cui_born_setup_desc* desc, int32_t max_objects, int32_t storage,
                             const char* cache_dir, int32_t* loaded, cui_born_plan** plan) {
    if (!plan) return cui::set_error(CUI_ERR_INVALID_ARG, "plan is NULL");
    *plan = nullptr;
    cui_born_plan* h = new (std::nothrow) cui_born_plan();
    if (!h) return cui::set_error(CUI_ERR_OOM, "host allocation failed");
    cui_status s;
    try {
        s = cui::create_setup(desc, max_objects, storage, h->p, cache_dir, loaded);
    } catch (const std::bad_alloc&) {
        s = cui::set_error(CUI_ERR_OOM, "host allocation failed");
    }
    if (s != CUI_OK) {
        cui_born_plan_destroy(h);
        return s;
    }
    *plan = h;
    return CUI_OK;
}
}  // namespace

extern "C" cui_status cui_born_plan_create_setup(const cui_born_setup_desc* desc, int32_t max_objects,
                                                 cui_born_plan** plan) {
    const cui::NvtxRange nvtx_range("cui_born_plan_create_setup");
    const cui::DeviceGuard restore(-1);  // the caller's current device is restored on return
    return create_setup_plan(desc, max_objects, CUI_STORAGE_AUTO, nullptr, nullptr, plan);
}

extern "C" cui_status cui_born_plan_create_setup_ex(const cui_born_setup_desc* desc, int32_t max_objects,
                                                    int32_t storage, const char* cache_dir, cui_born_plan** plan,
                                                    int32_t* loaded) {
    const cui::NvtxRange nvtx_range("cui_born_plan_create_setup_ex");
    if (loaded) *loaded = 0;
    const cui::DeviceGuard restore(-1);  // the caller's current device is restored on return
    return create_setup_plan(desc, max_objects, storage, cache_dir, loaded, plan);
}

extern "C" cui_status cui_born_plan_table_storage(const cui_born_plan* plan, int32_t* storage) {
    if (!plan || !storage) return cui::set_error(CUI_ERR_INVALID_ARG, "plan or storage is NULL");
    *storage = plan->p.table_mode;
    return CUI_OK;
}

extern "C" cui_status cui_born_plan_create_setup_cached(const cui_born_setup_desc* desc, int32_t max_objects,
                                                        const char* cache_dir, cui_born_plan** plan, int32_t* loaded) {
    const cui::NvtxRange nvtx_range("cui_born_plan_create_setup_cached");
    if (!cache_dir) return cui::set_error(CUI_ERR_INVALID_ARG, "cache_dir is NULL");
    if (loaded) *loaded = 0;
    const cui::DeviceGuard restore(-1);  // the caller's current device is restored on return
    return create_setup_plan(desc, max_objects, CUI_STORAGE_AUTO, cache_dir, loaded, plan);
}
