// Generated lateral-offset table: the 3D transfer function computed where it is
// consumed instead of read from a stored [F][Nz][Noy][Nox] array.
//
// An entry of the stored table (cui_tables.cu: table_kernel, after setup.m:1216-1281
// with the 3D Green's function of +processing/greens_function.m:103 and the
// anti-aliasing window of +scattering/+anti_aliasing_filters/on.m:64-70) is
//
//   T(f; z, oy, ox) = dA w / (2 pi) * sum_{qy, qx} exp(-j k~ D_q) / D_q,
//   D_q = sqrt((X - fx_q)^2 + (Y - fy_q)^2 + Z^2),
//
// with X, Y the lateral offsets of (ox, oy), Z the depth of row z, (fx_q, fy_q)
// the face quadrature points, k~ = kr + j ki the complex wavenumber and w the
// raised-cosine window of the centre offsets.  Here the same value is formed in
// FP32 with the two steps whose accuracy FP32 alone cannot carry done in FP32
// pairs (hi + lo, about 48 bits):
//   * D^2 = (X - fx)^2 + (Y - fy)^2 + Z^2: the squares come from the host in
//     FP64, split into pairs; the sum is a pair sum (Knuth's two-sum) and
//     D = sqrt(D^2) is refined by one Newton step on the pair;
//   * the phase kr D: the product's rounding error is kept exactly with an FMA
//     (Dekker's two-product), and the reduction modulo 2 pi subtracts n 2 pi in
//     two parts (Cody and Waite) where n * fl(2 pi) is exact inside the FMA, so
//     the reduced argument carries only its own FP32 rounding (about 1e-7 rad)
//     for any kr D.
// The reduced phase then goes through FP32 sin/cos, the attenuation through
// expf.  FP64 arithmetic would do the same at 1/64 of the FP32 issue rate on
// this GPU; the pair arithmetic keeps the generation cost a small fraction of
// the contraction that consumes each entry.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>

namespace cui {

// Per-plan parameters of the generated table (device pointers to small arrays).
struct TableGen {
    const float4* fk;   // [F] (kr_hi, kr_lo, ki, kr) of each global frequency
    const float2* sx2;  // [Qx][Nox] (X(ox) - fx(qx))^2 as a (hi, lo) pair
    const float2* sy2;  // [Qy][Noy] (Y(oy) - fy(qy))^2
    const float2* sz2;  // [Nz] Z(z)^2
    const float* ax;    // [Nox] |X(ox)|
    const float* ay;    // [Noy] |Y(oy)|
    const float2* wq;   // [F][Qy * Qx] face weights, or nullptr (uniform)
    int Nox, Noy, Qx, Qy;
    float scale;        // dA / (2 pi)
    float pitch_x, pitch_y;
    int win_x, win_y;   // raised-cosine window on the axis (array longer than one element, beta >= 0)
    float lb, inv_span; // window: pi (1 - beta) and 1 / (pi - lb)
};

// Constant part of one table row (f, z, oy).
struct GenRow {
    float kr_hi, kr_lo, ki, kw;  // kw = kr for the window flags
    float2 z2;                   // Z^2 pair
    float ay2c;                  // |Y|^2 + Z^2 of the centre offsets (window distance), FP32
    float ay;                    // |Y|
    int oy;
    int f;
};

__device__ __forceinline__ float2 pair_add(float2 a, float2 b) {
    const float s = a.x + b.x;
    const float bb = s - a.x;
    const float e = ((a.x - (s - bb)) + (b.x - bb)) + (a.y + b.y);
    const float hi = s + e;
    return make_float2(hi, e - (hi - s));
}

__device__ __forceinline__ GenRow gen_row(const TableGen& t, int f, int z, int oy) {
    GenRow r;
    const float4 k = __ldg(t.fk + f);
    r.kr_hi = k.x; r.kr_lo = k.y; r.ki = k.z; r.kw = k.w;
    r.z2 = __ldg(t.sz2 + z);
    r.ay = __ldg(t.ay + oy);
    r.ay2c = fmaf(r.ay, r.ay, r.z2.x);
    r.oy = oy;
    r.f = f;
    return r;
}

__device__ __forceinline__ float raised_cosine_f(float flag, const TableGen& t) {
    if (flag <= t.lb) return 1.f;
    if (flag >= 3.14159265358979f) return 0.f;
    return 0.5f * (1.f + __cosf(3.14159265358979f * (flag - t.lb) * t.inv_span));
}

// fl(2 pi) and the FP32 rounding of 2 pi - fl(2 pi)
constexpr double kTwoPiD = 6.283185307179586476925;
constexpr float kTwoPiHi = static_cast<float>(kTwoPiD);
constexpr float kTwoPiLo = static_cast<float>(kTwoPiD - static_cast<double>(kTwoPiHi));
constexpr float kInvTwoPi = static_cast<float>(1.0 / kTwoPiD);

// exp(-j k~ D) / D for the squared distance d2 (pair).  d = d2 rsqrt(d2) is within a few ulp of
// the square root; the Newton step on the pair removes that error from D = d + dl (the residual
// d2 - d^2 is exact in the FMA), and 1/D carries the reciprocal square root's ~1e-7.
__device__ __forceinline__ float2 gen_green(const GenRow& r, float2 d2) {
    const float inv = rsqrtf(d2.x);
    const float d = d2.x * inv;
    const float dl = 0.5f * (fmaf(-d, d, d2.x) + d2.y) * inv;  // D = d + dl
    const float p = r.kr_hi * d;
    const float pe = fmaf(r.kr_hi, d, -p);                      // exact: kr_hi d = p + pe
    const float small = fmaf(r.kr_hi, dl, fmaf(r.kr_lo, d, pe));
    const float n = rintf(p * kInvTwoPi);
    const float ph = fmaf(-n, kTwoPiLo, fmaf(-n, kTwoPiHi, p)) + small;  // kr D - 2 pi n
    float s, c;
    __sincosf(ph, &s, &c);
    const float m = expf(r.ki * (d + dl)) * inv;
    return make_float2(m * c, -m * s);
}

// One entry T(f; z, oy, ox) of the row described by r.
__device__ __forceinline__ float2 gen_entry(const TableGen& t, const GenRow& r, int ox) {
    float2 acc = make_float2(0.f, 0.f);
    for (int qy = 0; qy < t.Qy; ++qy) {
        const float2 yz = pair_add(__ldg(t.sy2 + static_cast<int64_t>(qy) * t.Noy + r.oy), r.z2);
        for (int qx = 0; qx < t.Qx; ++qx) {
            float2 g = gen_green(r, pair_add(__ldg(t.sx2 + static_cast<int64_t>(qx) * t.Nox + ox), yz));
            if (t.wq) {  // face weight w_q(f) (warp-uniform branch)
                const float2 wv = __ldg(t.wq + (static_cast<int64_t>(r.f) * t.Qy + qy) * t.Qx + qx);
                g = make_float2(g.x * wv.x - g.y * wv.y, g.x * wv.y + g.y * wv.x);
            }
            acc.x += g.x;
            acc.y += g.y;
        }
    }
    float w = t.scale;
    if (t.win_x | t.win_y) {
        const float axv = __ldg(t.ax + ox);
        const float rinv = rsqrtf(fmaf(axv, axv, r.ay2c));
        if (t.win_x) w *= raised_cosine_f(r.kw * t.pitch_x * axv * rinv, t);
        if (t.win_y) w *= raised_cosine_f(r.kw * t.pitch_y * r.ay * rinv, t);
    }
    return make_float2(acc.x * w, acc.y * w);
}

}  // namespace cui
