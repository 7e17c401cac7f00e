// Split-BF16 tensor-core (tcgen05) adjoint of the Born operator.
//
// The adjoint contraction of one grid line z, residue r (x = r + ppp*j) and
// frequency f is
//     Z[j][c] = sum_e conj(h(f; o(x, e), z)) V[e][c],   o = r + ppp*(j - e + E - 1)
// i.e. a GEMM with M = points j, K = elements, N = wave columns c.  The
// operand A[j][e'] (e' = E-1-e) is the band entry T_r[j + e'] -- a Toeplitz
// matrix whose rows shift by one complex entry.  It is never materialised:
// shared memory holds "spread chunks" (chunk i = band entries i..i+3, 16 B of
// interleaved bf16 re/im), and a no-swizzle K-major descriptor with LBO = 64 B
// and SBO = 128 B makes the tensor core read row j, K-group g from chunk
// j + 4g.  K interleaves real and imaginary parts and A = (T_re, T_im) serves
// both parts of the result: B1 = (V_re, V_im) gives Re(conj(T) V) and
// B2 = (V_im, -V_re) gives Im(conj(T) V).
//
// Precision: every operand is split into bf16 hi + lo (x = hi + lo + O(2^-18 x));
// the products hi*hi + hi*lo + lo*hi accumulate in FP32 in tensor memory.  B is
// stacked along N as [B1 hi | B2 hi | B1 lo | B2 lo] (16 columns each), so one
// N=64 MMA with A hi and one N=32 MMA with A lo cover all six products of a K
// step while A is read from shared memory only twice.  The epilogue multiplies
// by conj(p_in) in FP32 and sums the wave columns.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <string>

#include "cui_internal.cuh"
#include "cui_tc.cuh"

namespace cui {
namespace {

constexpr int kTcThreads = 128;  // 4 warps: one per TMEM lane quadrant; 4 CTAs per SM overlap staging with MMA

__device__ __forceinline__ uint32_t pack_bf16(float a, float b) {
    __nv_bfloat162 v = __floats2bfloat162_rn(a, b);
    return *reinterpret_cast<uint32_t*>(&v);
}

__device__ __forceinline__ float2 unpack_bf16(uint32_t w) {
    return make_float2(__uint_as_float(w << 16), __uint_as_float(w & 0xFFFF0000u));
}

// hi/lo split of a complex value into two packed bf16x2 words
__device__ __forceinline__ void split2(float a, float b, uint32_t& hi, uint32_t& lo) {
    hi = pack_bf16(a, b);
    const float2 h = unpack_bf16(hi);
    lo = pack_bf16(a - h.x, b - h.y);
}

// ---------------------------------------------------------------------------
// band arrays: tb[v][f][z][oy][r][i], v = {hi, lo} of (T_re, T_im) for table
// entry o = r + ppp*i
// ---------------------------------------------------------------------------
struct BandArgs {
    const float2* table;
    uint32_t* tb;
    int F, Nz, Noy, Nox, ppx, Nb;
    int64_t vstride;  // elements per variant
};

__global__ void band_kernel(const BandArgs a) {
    for (int64_t idx = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; idx < a.vstride;
         idx += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const int i = static_cast<int>(idx % a.Nb);
        int64_t t = idx / a.Nb;
        const int r = static_cast<int>(t % a.ppx);
        const int64_t row = t / a.ppx;  // (f, z, oy)
        const int o = r + a.ppx * i;
        const float2 v = (o < a.Nox) ? a.table[row * a.Nox + o] : make_float2(0.f, 0.f);
        uint32_t h1, l1;
        split2(v.x, v.y, h1, l1);
        a.tb[idx] = h1;
        a.tb[a.vstride + idx] = l1;
    }
}

// ---------------------------------------------------------------------------
// Shared pieces of the two contraction kernels.
//
// A "unit" is one (grid line, residue) of the forward or one (frequency,
// column pass, residue) of the adjoint.  Per unit the 4 band variants are
// expanded into spread chunks in shared memory (entry i of the band lands in
// chunks i-3..i), the MMAs run, and their result is read out of tensor memory
// into FP32 registers, so no tensor-core accumulation chain is longer than one
// unit (<= 768 products).  While the MMAs of unit u run, every thread already
// loads the band entries of unit u+1 (and, in the adjoint, the incident field
// its epilogue needs) into registers.
// ---------------------------------------------------------------------------
constexpr int kCols16 = 16;            // wave columns per pass
constexpr uint32_t kTmemCols = 128;    // D1 (64 columns) + D2 (32 columns), rounded to a power of two
constexpr int kMaxBandPerThread = 5;   // 2 variants x (NCH + 3) entries <= 5 per thread (NCH <= 256)

__device__ __forceinline__ void fetch_band(uint32_t (&be)[kMaxBandPerThread], const uint32_t* band, int64_t vstride,
                                           int Nb, int NCH, int tid) {
    const int n = 2 * (NCH + 3);
#pragma unroll
    for (int m = 0; m < kMaxBandPerThread; ++m) {
        const int idx = tid + kTcThreads * m;
        uint32_t w = 0u;
        if (idx < n) {
            const int v = idx >= NCH + 3 ? 1 : 0, i = idx - v * (NCH + 3);
            if (i < Nb) w = __ldg(band + static_cast<int64_t>(v) * vstride + i);
        }
        be[m] = w;
    }
}

// chunk ch of variant v holds band entries ch..ch+3 (16 B at sA + (v*NCH + ch)*16).
// A warp's 32 entries are written in 4 passes; in pass q lane l stores word
// l%4 of entry 8q + l/4 (taken from that lane by a shuffle), which puts the 32
// stores of a pass into 32 distinct banks.
__device__ __forceinline__ void store_chunks(unsigned char* sA, const uint32_t (&be)[kMaxBandPerThread], int NCH, int tid) {
    const int n = 2 * (NCH + 3);
    const int lane = tid & 31, wbase = tid - lane;
#pragma unroll
    for (int m = 0; m < kMaxBandPerThread; ++m) {
        if (wbase + kTcThreads * m >= n) break;  // uniform over the warp
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const int src = 8 * q + (lane >> 2), t = lane & 3;
            const uint32_t w = __shfl_sync(0xffffffffu, be[m], src);
            const int idx = wbase + kTcThreads * m + src;
            if (idx < n) {
                const int v = idx >= NCH + 3 ? 1 : 0, i = idx - v * (NCH + 3);
                const int ch = i - t;
                if (ch >= 0 && ch < NCH) *reinterpret_cast<uint32_t*>(sA + (static_cast<size_t>(v) * NCH + ch) * 16 + 4 * t) = w;
            }
        }
    }
}

// byte offset of the first stacked B row of column c at K index kk; the rows of
// B2 hi, B1 lo, B2 lo follow at +2, +4, +6 SBO (16 rows = two 8-row groups)
__device__ __forceinline__ int b_base(int c, int kk, int SBO) {
    return (c >> 3) * SBO + (kk >> 3) * 128 + (c & 7) * 16 + (kk & 7) * 2;
}

// Stores B1 = (x, y) and B2 = (-y, x) (hi and lo) at byte offset off:
// B2's bf16 words are B1's with the halves swapped and the new low half negated,
// because rounding to bf16 commutes with negation.
__device__ __forceinline__ void store_b_rot(unsigned char* sB, int off, int SBO, float x, float y) {
    uint32_t h1, l1;
    split2(x, y, h1, l1);
    const uint32_t h2 = __byte_perm(h1, 0, 0x1032) ^ 0x00008000u;
    const uint32_t l2 = __byte_perm(l1, 0, 0x1032) ^ 0x00008000u;
    *reinterpret_cast<uint32_t*>(sB + off) = h1;
    *reinterpret_cast<uint32_t*>(sB + off + 2 * SBO) = h2;
    *reinterpret_cast<uint32_t*>(sB + off + 4 * SBO) = l1;
    *reinterpret_cast<uint32_t*>(sB + off + 6 * SBO) = l2;
}

// Per K step: D1 (+)= A_hi x B[0:64) and D2 (+)= A_lo x B[0:32).  A K step
// advances A by 8 chunks (128 B) and B by two K-groups (256 B); descriptor
// address fields count 16-byte units, so the steps are +8 and +16.
__device__ __forceinline__ void issue_unit(uint32_t t_d1, uint32_t t_d2, uint32_t a0, int NCH, uint32_t b0, int SBO,
                                           int ks) {
    constexpr uint32_t id64 = tc::idesc_bf16(128, 64);
    constexpr uint32_t id32 = tc::idesc_bf16(128, 32);
    const uint64_t ah = tc::smem_desc(a0, 64, 128);
    const uint64_t al = tc::smem_desc(a0 + NCH * 16, 64, 128);
    const uint64_t db = tc::smem_desc(b0, 128, SBO);
    tc::mma_bf16(t_d1, ah, db, id64, 0u);
    tc::mma_bf16(t_d2, al, db, id32, 0u);
    for (int k = 1; k < ks; ++k) {
        tc::mma_bf16(t_d1, ah + 8ull * k, db + 16ull * k, id64, 1u);
        tc::mma_bf16(t_d2, al + 8ull * k, db + 16ull * k, id32, 1u);
    }
}

// adds the unit's result (re/im of the 16 columns) for the calling thread's lane:
// re = A_hi B1_hi + A_hi B1_lo + A_lo B1_hi, im likewise with B2 (two TMEM waits)
__device__ __forceinline__ void add_unit(uint32_t t_d1, uint32_t t_d2, uint32_t lane_base, float (&re)[kCols16],
                                         float (&im)[kCols16]) {
    float a[16], b[16], c[16];
    tc::tmem_ld16(t_d1 + lane_base, a);
    tc::tmem_ld16(t_d1 + lane_base + 32, b);
    tc::tmem_ld16(t_d2 + lane_base, c);
    tc::tmem_wait_ld();
#pragma unroll
    for (int u = 0; u < 16; ++u) re[u] += (a[u] + b[u]) + c[u];
    tc::tmem_ld16(t_d1 + lane_base + 16, a);
    tc::tmem_ld16(t_d1 + lane_base + 48, b);
    tc::tmem_ld16(t_d2 + lane_base + 16, c);
    tc::tmem_wait_ld();
#pragma unroll
    for (int u = 0; u < 16; ++u) im[u] += (a[u] + b[u]) + c[u];
}

// ---------------------------------------------------------------------------
// Adjoint
// ---------------------------------------------------------------------------
struct AdjTcArgs {
    const uint32_t* tb;
    int64_t vstride;
    const float2* p_in;
    const float2* V;        // [S][B][E]
    const int* f_slot_ptr;
    const int* f_slot_list;
    int Nx, Nz, Ex, ppx, Nb, F, E, Epad;
    int64_t P;
    int fchunk, B;
    float2* part;           // [nfc][B][P]
    int* status;
};

// dynamic shared memory layout (bytes):
//   [0, SBB)             stacked B (SBB = 64 rows x 2*Epad bf16 = 256*Epad)
//   [SBB, +2*NCH*16)     spread chunks of A hi, A lo (NCH = 128 + Epad)
//   then sG [Nx] float2, then bar (8 B), tslot (4 B), slots [16] int
__global__ void __launch_bounds__(kTcThreads, 3) adj_tc_kernel(const AdjTcArgs a) {
    extern __shared__ __align__(1024) unsigned char smem[];
    const int SBB = 256 * a.Epad;
    const int NCH = 128 + a.Epad;
    unsigned char* sB = smem;
    unsigned char* sA = smem + SBB;
    float2* sG = reinterpret_cast<float2*>(sA + 2 * NCH * 16);
    unsigned char* tail = reinterpret_cast<unsigned char*>(sG + a.Nx);
    uint64_t* barp = reinterpret_cast<uint64_t*>((reinterpret_cast<uintptr_t>(tail) + 7) & ~uintptr_t(7));
    uint32_t* tslot = reinterpret_cast<uint32_t*>(barp + 1);
    int* sSlot = reinterpret_cast<int*>(tslot + 1);

    const int tid = threadIdx.x, warp = tid >> 5;
    const int z = blockIdx.x, fc = blockIdx.y, b = blockIdx.z;
    const int64_t pt0 = static_cast<int64_t>(z) * a.Nx;
    const uint32_t bar = tc::smem_u32(barp);
    const int SBO = 32 * a.Epad;
    const int ksteps = a.Epad / 8;

    for (int x = tid; x < a.Nx; x += kTcThreads) sG[x] = make_float2(0.f, 0.f);
    if (tid == 0) tc::bar_init(bar, 1);
    if (warp == 0) tc::tmem_alloc(tc::smem_u32(tslot), kTmemCols);
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = *tslot;
    const uint32_t t_d1 = tmem, t_d2 = tmem + 64;
    const uint32_t lane_base = static_cast<uint32_t>(warp * 32) << 16;
    uint32_t phase = 0;
    bool failed = false;

    const int f_lo = fc * a.fchunk, f_hi = min(f_lo + a.fchunk, a.F);
    int f = f_lo, c0 = 0, r = 0;  // unit cursor; the first unit of a (f, c0) stages B
    auto band_of = [&](int ff, int rr) {
        return a.tb + ((static_cast<int64_t>(ff) * a.Nz + z) * a.ppx + rr) * a.Nb;
    };
    auto advance = [&](int& ff, int& cc, int& rr) {
        if (++rr < a.ppx) return;
        rr = 0;
        cc += kCols16;
        if (cc < a.f_slot_ptr[ff + 1] - a.f_slot_ptr[ff]) return;
        cc = 0;
        ++ff;
    };
    while (f < f_hi && a.f_slot_ptr[f + 1] == a.f_slot_ptr[f]) ++f;
    uint32_t be[kMaxBandPerThread];
    if (f < f_hi) fetch_band(be, band_of(f, r), a.vstride, a.Nb, NCH, tid);
    while (f < f_hi && !failed) {
        const int s0 = a.f_slot_ptr[f];
        const int nc = min(kCols16, a.f_slot_ptr[f + 1] - s0 - c0);
        const int Nj_r = (r < a.Nx) ? (a.Nx - r + a.ppx - 1) / a.ppx : 0;
        if (r == 0) {
            if (tid < kCols16) sSlot[tid] = (tid < nc) ? a.f_slot_list[s0 + c0 + tid] : 0;
            __syncthreads();
            // ---- B: V columns, element order reversed, complex interleaved along K ----
            // lanes -> (column mod 8, element mod 4): the 32 stores of a warp hit 32 banks
            for (int idx = tid; idx < kCols16 * a.Epad; idx += kTcThreads) {
                const int t = idx & 31, w = idx >> 5;
                const int c = ((t >> 2) & 7) + 8 * (w & 1), ep = 4 * (w >> 1) + (t & 3);
                const int e = a.Ex - 1 - ep;
                float2 v = make_float2(0.f, 0.f);
                if (c < nc && e >= 0) v = __ldg(a.V + (static_cast<int64_t>(sSlot[c]) * a.B + b) * a.E + e);
                store_b_rot(sB, b_base(c, 2 * ep, SBO), SBO, v.x, v.y);  // imaginary part comes out negated
            }
        }
        store_chunks(sA, be, NCH, tid);
        tc::fence_async_smem();
        __syncthreads();
        if (tid == 0) {
            tc::fence_after_sync();
            issue_unit(t_d1, t_d2, tc::smem_u32(sA), NCH, tc::smem_u32(sB), SBO, ksteps);
            tc::commit(bar);
        }
        // while the MMAs run: this unit's incident field, next unit's band
        const int x = r + a.ppx * tid;
        float2 pq[kCols16];
#pragma unroll
        for (int c = 0; c < kCols16; ++c)
            pq[c] = (c < nc && tid < Nj_r) ? __ldg(a.p_in + static_cast<int64_t>(sSlot[c]) * a.P + pt0 + x)
                                           : make_float2(0.f, 0.f);
        int fn = f, cn = c0, rn = r;
        advance(fn, cn, rn);
        while (fn < f_hi && a.f_slot_ptr[fn + 1] == a.f_slot_ptr[fn]) ++fn;
        if (fn < f_hi) fetch_band(be, band_of(fn, rn), a.vstride, a.Nb, NCH, tid);
        const bool ok = (tid == 0) ? tc::bar_wait(bar, phase) : true;  // one poller; the rest park at the barrier
        phase ^= 1u;
        if (__syncthreads_or(!ok)) {
            failed = true;
            break;
        }
        tc::fence_after_sync();
        // ---- epilogue: gamma_hat(x) += sum_c conj(p_in[slot_c][x]) Z[j][c] ----
        float zr[kCols16], zi[kCols16];
#pragma unroll
        for (int c = 0; c < kCols16; ++c) zr[c] = zi[c] = 0.f;
        add_unit(t_d1, t_d2, lane_base, zr, zi);
        float2 acc = make_float2(0.f, 0.f);
#pragma unroll
        for (int c = 0; c < kCols16; ++c) {  // Z = zr - i*zi
            const float2 p = pq[c];
            acc.x = fmaf(p.x, zr[c], fmaf(-p.y, zi[c], acc.x));
            acc.y = fmaf(-p.x, zi[c], fmaf(-p.y, zr[c], acc.y));
        }
        if (tid < Nj_r) {
            float2 g = sG[x];
            g.x += acc.x;
            g.y += acc.y;
            sG[x] = g;
        }
        tc::fence_before_sync();
        __syncthreads();
        f = fn;
        c0 = cn;
        r = rn;
    }
    if (failed && tid == 0) atomicOr(a.status, 1);
    __syncthreads();
    float2* out = a.part + (static_cast<int64_t>(fc) * a.B + b) * a.P + pt0;
    for (int xx = tid; xx < a.Nx; xx += kTcThreads) out[xx] = sG[xx];
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tmem, kTmemCols);
}

// ---------------------------------------------------------------------------
// Forward: Y[e][c] = sum_j T_r[j + e'] q_c(x_j), e' = E-1-e, summed over the
// block's grid lines and residues.  The same band chunks serve as A (rows =
// elements e', K = points j); B1 = conj(q) = (q_re, -q_im) gives Re(T q) and
// B2 = (q_im, q_re) gives Im(T q).
// ---------------------------------------------------------------------------
struct FwdTcArgs {
    const uint32_t* tb;
    int64_t vstride;
    const float2* p_in;
    const float2* gamma;
    int64_t ldg;
    const int* f_slot_ptr;
    const int* f_slot_list;
    int Nx, Nz, Ex, ppx, Nb, F, E, S, Jpad;
    int64_t P;
    int lines_per_group, n_lines, B, npass;
    float2* part;  // [groups][S][B][E]
    int* status;
};

// Two-stage pipeline: shared-memory stages and TMEM accumulators alternate, so
// the MMAs of unit u+1 run while unit u is read out and unit u+2 is staged.
// dynamic shared memory (bytes): 2 stages x [stacked B (256*Jpad), A chunks hi/lo
// (2 x NCH x 16, NCH = 128 + Jpad)], 2 mbarriers, tslot, slots[16]
constexpr uint32_t kFwdTmemCols = 256;  // 2 stages x (D1 64 + D2 32), stage stride 128 columns

__global__ void __launch_bounds__(kTcThreads, 2) fwd_tc_kernel(const FwdTcArgs a) {
    extern __shared__ __align__(1024) unsigned char smem[];
    const int SBB = 256 * a.Jpad;
    const int NCH = 128 + a.Jpad;
    const int STAGE = SBB + 2 * NCH * 16;
    unsigned char* tail = smem + 2 * STAGE;
    uint64_t* barp = reinterpret_cast<uint64_t*>(tail);  // [2]
    uint32_t* tslot = reinterpret_cast<uint32_t*>(barp + 2);
    int* sSlot = reinterpret_cast<int*>(tslot + 1);

    const int grp = blockIdx.x, f = blockIdx.y;
    const int b = blockIdx.z / a.npass, cp = blockIdx.z - b * a.npass;
    const int s0 = a.f_slot_ptr[f];
    const int ns = a.f_slot_ptr[f + 1] - s0;
    const int c0 = cp * kCols16;
    if (c0 >= ns) return;  // uniform over the block
    const int nc = min(kCols16, ns - c0);
    const int tid = threadIdx.x, warp = tid >> 5;
    if (tid < kCols16) sSlot[tid] = (tid < nc) ? a.f_slot_list[s0 + c0 + tid] : 0;
    const int SBO = 32 * a.Jpad;
    if (tid == 0) {
        tc::bar_init(tc::smem_u32(barp), 1);
        tc::bar_init(tc::smem_u32(barp + 1), 1);
    }
    if (warp == 0) tc::tmem_alloc(tc::smem_u32(tslot), kFwdTmemCols);
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = *tslot;
    const uint32_t lane_base = static_cast<uint32_t>(warp * 32) << 16;
    uint32_t phase0 = 0, phase1 = 0;
    bool failed = false;
    const float2* gam = a.gamma + static_cast<int64_t>(b) * a.ldg;

    // each thread owns one point j of every unit and the columns c = ct0 + cstride*((m + g) mod ncol);
    // the rotation by the lane group g spreads a warp's B stores over all banks
    const int jt = tid % a.Jpad, ct0 = tid / a.Jpad, cstride = kTcThreads / a.Jpad;
    const int ncol = (kCols16 + cstride - 1) / cstride;  // columns per thread (<= 16), a power of two
    const int g = (tid >> 2) & 7;
    auto col = [&](int m) { return ct0 + cstride * ((m + g) & (ncol - 1)); };
    float accr[kCols16], acci[kCols16];
#pragma unroll
    for (int c = 0; c < kCols16; ++c) accr[c] = acci[c] = 0.f;

    const int line0 = grp * a.lines_per_group, line1 = min(line0 + a.lines_per_group, a.n_lines);
    const int U = max(0, line1 - line0) * a.ppx;
    uint32_t be[kMaxBandPerThread];
    float2 pq[kCols16];
    float2 gq = make_float2(0.f, 0.f);
    auto nj_of = [&](int u) {
        const int r = u % a.ppx;
        return (r < a.Nx) ? (a.Nx - r + a.ppx - 1) / a.ppx : 0;
    };
    auto fetch = [&](int u) {
        const int z = line0 + u / a.ppx, r = u % a.ppx;
        const int Nj_r = nj_of(u);
        const int64_t pt = static_cast<int64_t>(z) * a.Nx + r + static_cast<int64_t>(a.ppx) * jt;
        fetch_band(be, a.tb + ((static_cast<int64_t>(f) * a.Nz + z) * a.ppx + r) * a.Nb, a.vstride, a.Nb, NCH, tid);
        gq = (jt < Nj_r) ? __ldg(gam + pt) : make_float2(0.f, 0.f);
#pragma unroll
        for (int m = 0; m < kCols16; ++m) {
            const int c = col(m);
            pq[m] = (m < ncol && c < nc && jt < Nj_r) ? __ldg(a.p_in + static_cast<int64_t>(sSlot[c]) * a.P + pt)
                                                      : make_float2(0.f, 0.f);
        }
    };
    auto store = [&](int st) {
        unsigned char* sB = smem + st * STAGE;
        store_chunks(sB + SBB, be, NCH, tid);
#pragma unroll
        for (int m = 0; m < kCols16; ++m) {
            const int c = col(m);
            if (m < ncol && c < kCols16) {
                const float2 p = pq[m];
                const float qx = p.x * gq.x - p.y * gq.y, qy = p.x * gq.y + p.y * gq.x;
                store_b_rot(sB, b_base(c, 2 * jt, SBO), SBO, qx, -qy);
            }
        }
    };
    auto issue = [&](int u, int st) {  // thread 0
        tc::fence_after_sync();
        const uint32_t base = tc::smem_u32(smem + st * STAGE);
        const uint32_t td = tmem + 128u * st;
        issue_unit(td, td + 64, base + SBB, NCH, base, SBO, (nj_of(u) + 7) / 8);
        tc::commit(tc::smem_u32(barp + st));
    };

    if (U > 0) {
        fetch(0);
        store(0);
        tc::fence_async_smem();
        __syncthreads();
        if (tid == 0) issue(0, 0);
        if (U > 1) fetch(1);
    }
    for (int u = 0; u < U; ++u) {
        const int st = u & 1;
        if (u + 1 < U) store(st ^ 1);  // overlaps MMA(u); stage st^1 was released when MMA(u-1) completed
        tc::fence_async_smem();
        bool ok = true;
        if (tid == 0) {
            ok = tc::bar_wait(tc::smem_u32(barp + st), st ? phase1 : phase0);
        }
        if (st) phase1 ^= 1u; else phase0 ^= 1u;
        if (__syncthreads_or(!ok)) {
            failed = true;
            break;
        }
        if (tid == 0 && u + 1 < U) issue(u + 1, st ^ 1);
        if (u + 2 < U) fetch(u + 2);
        tc::fence_after_sync();
        add_unit(tmem + 128u * st, tmem + 128u * st + 64, lane_base, accr, acci);
        tc::fence_before_sync();
    }
    if (failed && tid == 0) atomicOr(a.status, 1);
    // ---- epilogue: lanes = elements e' ----
    const int e = a.Ex - 1 - tid;
    if (e >= 0) {
#pragma unroll
        for (int c = 0; c < kCols16; ++c)
            if (c < nc)
                a.part[((static_cast<int64_t>(grp) * a.S + sSlot[c]) * a.B + b) * a.E + e] = make_float2(accr[c], acci[c]);
    }
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tmem, kFwdTmemCols);
}

size_t fwd_tc_smem(const Plan* p) {
    const size_t Jpad = static_cast<size_t>(p->Jpad);
    return 2 * (256 * Jpad + 2 * (128 + Jpad) * 16) + 16 + 8 + 4 * kCols16 + 64;
}

size_t adj_tc_smem(const Plan* p) {
    const size_t Epad = static_cast<size_t>(p->Epad);
    return 256 * Epad + 2 * (128 + Epad) * 16 + sizeof(float2) * p->Nx + 8 + 8 + 4 * kCols16 + 64;
}

}  // namespace

cudaError_t launch_fwd_tc(Plan* p, const float2* gamma, int64_t ldg, int B, cudaStream_t st) {
    FwdTcArgs a;
    a.tb = p->tb; a.vstride = p->tb_vstride; a.p_in = p->p_in; a.gamma = gamma; a.ldg = ldg;
    a.f_slot_ptr = p->f_slot_ptr; a.f_slot_list = p->f_slot_list;
    a.Nx = p->Nx; a.Nz = p->Nz; a.Ex = p->Ex; a.ppx = p->ppx; a.Nb = p->Nb; a.F = p->F; a.E = p->E; a.S = p->S;
    a.Jpad = p->Jpad; a.P = p->P;
    a.lines_per_group = p->fwd_lines_per_group; a.n_lines = p->Ny * p->Nz; a.B = B;
    a.npass = (p->max_slots_per_f + kCols16 - 1) / kCols16;
    a.part = p->ws_part; a.status = p->ws_status;
    const size_t smem = fwd_tc_smem(p);
    cudaError_t e = cudaFuncSetAttribute(fwd_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         static_cast<int>(smem));
    if (e != cudaSuccess) return e;
    dim3 grid(p->fwd_groups, p->F, B * a.npass);
    if ((e = timing_begin(p, 0, st)) != cudaSuccess) return e;
    fwd_tc_kernel<<<grid, kTcThreads, smem, st>>>(a);
    count_launch();
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    return timing_end(p, st);
}

cudaError_t launch_adj_tc(Plan* p, int B, cudaStream_t st) {
    AdjTcArgs a;
    a.tb = p->tb; a.vstride = p->tb_vstride; a.p_in = p->p_in; a.V = p->ws_G;
    a.f_slot_ptr = p->f_slot_ptr; a.f_slot_list = p->f_slot_list;
    a.Nx = p->Nx; a.Nz = p->Nz; a.Ex = p->Ex; a.ppx = p->ppx; a.Nb = p->Nb; a.F = p->F; a.E = p->E; a.Epad = p->Epad;
    a.P = p->P; a.fchunk = p->adj_fchunk; a.B = B; a.part = p->ws_part; a.status = p->ws_status;
    const size_t smem = adj_tc_smem(p);
    cudaError_t e = cudaFuncSetAttribute(adj_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         static_cast<int>(smem));
    if (e != cudaSuccess) return e;
    dim3 grid(p->Nz, p->adj_nfc, B);
    if ((e = timing_begin(p, 1, st)) != cudaSuccess) return e;
    adj_tc_kernel<<<grid, kTcThreads, smem, st>>>(a);
    count_launch();
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    return timing_end(p, st);
}

bool tc_supported(const Plan* p, std::string* why) {
    if (p->n_dims != 2) { *why = "the tensor-core path covers 2D setups"; return false; }
    if (p->Ex > 128) { *why = "the tensor-core path covers up to 128 elements"; return false; }
    if (p->Nj_max > 128 || p->Nx < p->ppx) { *why = "the tensor-core path covers 1..128 grid points per residue"; return false; }
    return true;
}

cui_status tc_build(Plan& p) {
    p.Epad = (p.Ex + 7) / 8 * 8;
    p.Jpad = 8;
    while (p.Jpad < p.Nj_max) p.Jpad *= 2;  // power of two <= 128: one point per thread for every column
    p.Nb = (p.Nox + p.ppx - 1) / p.ppx;
    p.tb_vstride = static_cast<int64_t>(p.F) * p.Nz * p.Noy * p.ppx * p.Nb;
    cui_status st = device_alloc(p, reinterpret_cast<void**>(&p.tb), sizeof(uint32_t) * 2 * p.tb_vstride);
    if (st != CUI_OK) return st;
    int smem_optin = 0;
    cudaError_t e = cudaDeviceGetAttribute(&smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, p.device);
    if (e != cudaSuccess) return check_cuda(e, "cudaDeviceGetAttribute");
    if (adj_tc_smem(&p) > static_cast<size_t>(smem_optin) || fwd_tc_smem(&p) > static_cast<size_t>(smem_optin))
        return set_error(CUI_ERR_UNSUPPORTED_SETUP, "grid line too long for the tensor-core staging");
    BandArgs b;
    b.table = p.table; b.tb = p.tb; b.F = p.F; b.Nz = p.Nz; b.Noy = p.Noy; b.Nox = p.Nox; b.ppx = p.ppx; b.Nb = p.Nb;
    b.vstride = p.tb_vstride;
    const int blocks = static_cast<int>(std::min<int64_t>((p.tb_vstride + 255) / 256, 152 * 32));
    band_kernel<<<blocks, 256>>>(b);
    count_launch();
    if ((e = cudaGetLastError()) != cudaSuccess) return check_cuda(e, "band table");
    if ((e = cudaDeviceSynchronize()) != cudaSuccess) return check_cuda(e, "band table");
    p.tc_bytes = sizeof(uint32_t) * 2 * static_cast<size_t>(p.tb_vstride);
    return CUI_OK;
}

// Residue-unit split tables, built once; a build that fails frees what it allocated and leaves the
// plan as it was (the next switch starts over).
cui_status tc_prepare(Plan& p) {
    std::string why;
    if (!tc_supported(&p, &why)) return set_error(CUI_ERR_UNSUPPORTED_SETUP, why);
    if (p.tb) return CUI_OK;
    if (!p.ws_status) {
        cui_status st = device_alloc(p, reinterpret_cast<void**>(&p.ws_status), sizeof(int));
        if (st != CUI_OK) return st;
        cudaError_t e = cudaMemset(p.ws_status, 0, sizeof(int));
        if (e != cudaSuccess) return check_cuda(e, "cudaMemset");
    }
    const size_t mark = p.allocations.size();
    const cui_status s = tc_build(p);
    if (s != CUI_OK) {
        release_since(p, mark);
        p.tb = nullptr;
    }
    return s;
}


}  // namespace cui

extern "C" cui_status cui_born_set_precision(cui_born_plan* plan, int32_t precision) {
    const cui::NvtxRange nvtx_range("cui_born_set_precision");
    using namespace cui;
    if (!plan) return set_error(CUI_ERR_INVALID_ARG, "plan is NULL");
    if (precision == CUI_PRECISION_FP32) {
        plan->p.precision = 0;
        return CUI_OK;
    }
    if (precision != CUI_PRECISION_BF16X3 && precision != CUI_PRECISION_BF16X3_FOLDED)
        return set_error(CUI_ERR_INVALID_ARG, "unknown precision");
    const DeviceGuard dev_guard(plan->p.device);
    cudaError_t e = dev_guard.err;
    if (e != cudaSuccess) return check_cuda(e, "cudaSetDevice");
    Plan& p = plan->p;
    if (precision == CUI_PRECISION_BF16X3_FOLDED) {
        cui_status s = phi_prepare(p);
        if (s != CUI_OK) return s;
        p.precision = 2;
        return CUI_OK;
    }
    if (!p.ws_status) {
        cui_status s = device_alloc(p, reinterpret_cast<void**>(&p.ws_status), sizeof(int));
        if (s != CUI_OK) return s;
        if ((e = cudaMemset(p.ws_status, 0, sizeof(int))) != cudaSuccess) return check_cuda(e, "cudaMemset");
    }
    std::string why;
    // line-unit kernels where the geometry allows them, else the residue-unit kernels
    cui_status s = (!p.tc2 && !p.tb && tc2_supported(&p, &why)) ? tc2_prepare(p) : (p.tc2 ? CUI_OK : tc_prepare(p));
    if (s != CUI_OK) return s;
    plan->p.precision = 1;
    return CUI_OK;
}

extern "C" cui_status cui_born_set_wait_limit(cui_born_plan* plan, int64_t nanoseconds) {
    using namespace cui;
    if (!plan) return set_error(CUI_ERR_INVALID_ARG, "plan is NULL");
    if (nanoseconds < 0 || nanoseconds > 60000000000ll)
        return set_error(CUI_ERR_INVALID_ARG, "wait limit must be 0 (default) or 1 ns to 60 s");
    plan->p.wait_limit_ns = nanoseconds == 0 ? 1000000000ull : static_cast<uint64_t>(nanoseconds);
    return CUI_OK;
}

extern "C" cui_status cui_born_set_occupancy_limit(cui_born_plan* plan, int64_t max_points) {
    using namespace cui;
    if (!plan) return set_error(CUI_ERR_INVALID_ARG, "plan is NULL");
    if (max_points < -1) return set_error(CUI_ERR_INVALID_ARG, "max_points must be -1 (default), 0 (off) or > 0");
    plan->p.occ_limit = max_points;
    return CUI_OK;
}

extern "C" cui_status cui_born_plan_status(cui_born_plan* plan, int32_t* device_status) {
    using namespace cui;
    if (!plan || !device_status) return set_error(CUI_ERR_INVALID_ARG, "NULL argument");
    *device_status = 0;
    if (!plan->p.ws_status) return CUI_OK;
    const DeviceGuard dev_guard(plan->p.device);
    cudaError_t e = dev_guard.err;
    if (e == cudaSuccess) e = cudaMemcpy(device_status, plan->p.ws_status, sizeof(int), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemset(plan->p.ws_status, 0, sizeof(int));
    if (e != cudaSuccess) return check_cuda(e, "status");
    return (*device_status != 0) ? set_error(CUI_ERR_TIMEOUT, "a bounded device-side wait gave up") : CUI_OK;
}
