// Folded operator: the Born operator's observation x grid-point matrix, stored
// in HBM as split bf16 and applied by tcgen05 GEMMs (the batched split-BF16 path
// for plans whose receive mixes are fewer than their active elements).
//
// The reference builds, per (measurement w, mix m, active element e), the matrix
//     Phi_{w,m,e}[f, p] = h_ref[f, shift(p, e)] * p_in_w[f, p] * pref_{w,m}[f, e]
// and accumulates u_{w,m} += Phi_{w,m,e} gamma over e (combined_quick_gpu.cu:
// 807-937, compute_matrix_kernel :1099-1124; operator_born.m:428-452).  Summing
// over the active elements first gives one row per observation (w, m, f):
//     Phi[r, p] = p_in[slot(r), p] * sum_{a in act(m)} pref[m, f, a] * h(f; o(p, e_a), z_p)
// so the forward is u = Phi gamma and the adjoint gamma^ = Phi^H u, two plain
// GEMMs over (observation rows) x (grid points) x (objects).  Against the element
// contraction this does min(M, E_act) / E_act of the multiply-adds (32 / 128 for
// 16 waves x 32 mixes of 128 elements) at 8 bytes of HBM per matrix entry and
// apply direction.  Rows whose frequency and mix (active elements and
// prefactors) agree share their element sum ("representatives"), so the build
// forms each sum once and multiplies it by every slot's incident field.
//
// Storage: 16-byte pieces of 8 bf16, one per (row r, point block pb = p/8,
// component c (re/im), half hl (hi/lo)), eight rows r%8 of a piece group forming
// one 128-byte core matrix (8 rows x 8 points):
//     byte offset = (((r/256 * NPB + pb) * 32 + (r/8)%32) * 512) + c*256 + hl*128 + (r%8)*16
// The same core matrix is a K-major A tile of the forward (M = rows, K = points)
// and an MN-major A tile of the adjoint (M = points, K = rows), so one copy of
// the matrix serves both directions:
//   forward, per 8-point K step: 256 rows x (c, hl) are one contiguous 16 KB;
//   adjoint, per 8-row K step: 256 points are 32 pieces of 512 B, 16 KB apart, so an
//   adjoint stage of KS row octets is one 4D tensor copy (box: 32 point blocks x KS
//   row octets x 512 B) whose shared-memory order is the MN-major A tile.
// K steps take the two components as two 8-element halves: K = [8 x re | 8 x im].
// The other operand is written once per apply in its shared-memory layout
// (K-major, N rows = [B1 hi | B2 hi | B1 lo | B2 lo] x 64 objects):
//   forward  B1 = (g, -h), B2 = (h, g) for gamma = g + ih  -> Re, Im of Phi gamma
//   adjoint  B1 = (c, d),  B2 = (d, -c) for u = c + id     -> Re, Im of conj(Phi) u
// Per K step and 128-row tile three N = 128 MMAs (A hi x B hi, A hi x B lo,
// A lo x B hi) accumulate hi*hi + hi*lo + lo*hi into the same 128 FP32 columns
// [Re 64 | Im 64] of tensor memory.
//
// Block: 10 warps.  Warp 9 issues the bulk and tensor copies, lane 0 of warp 8 the MMAs
// (warp 8 also owns the tensor memory: 2 tiles x 2 buffers x 128 columns), and
// warps 0-7 read the accumulators out: the tensor cores' FP32 accumulation loses
// precision over long chains, so every 32 K steps a chain's accumulator is
// handed over and added into FP32 registers while the MMAs continue in the
// tile's other buffer.  Every wait has a wall-clock limit after which the block
// drains its copies and MMAs, raises the plan's status word and returns.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <cstring>
#include <string>
#include <unordered_map>
#include <vector>

#include "cui_internal.cuh"
#include "cui_tc.cuh"

namespace cui {
namespace {

constexpr int kPhiObj = 64;          // objects per GEMM pass
constexpr int kPieceGroup = 512;     // bytes of (c, hl) x 8 rows for one row octet and point block
constexpr int kPbPad = 0;            // bytes between the 16 KB chunks of consecutive point blocks
constexpr int64_t kPbStride = 32 * kPieceGroup + kPbPad;  // bytes per (256-row block, point block) chunk
constexpr int kKStepA = 16384;       // A bytes per K step: 32 octets (256 rows or 256 points) x 512 B
constexpr int kKStepB = 8192;        // B bytes per K step: 256 N rows x 16 K x 2 B
constexpr uint64_t kDrainNs = 1000000000ull;
constexpr int kEpiWarps = 8;                       // warps 0-7: read-out (tile = warp / 4, lane quadrant = warp % 4)
constexpr int kPhiThreads = 32 * (kEpiWarps + 2);  // + warp 8 (MMA issue, TMEM owner) + warp 9 (bulk copies)
constexpr int kChain = 32;                         // K steps per accumulation chain (256 points or rows)

template <int KS, int NS>
struct PhiCfg {
    static constexpr int A_BYTES = KS * kKStepA;
    static constexpr int B_BYTES = KS * kKStepB;
    static constexpr int STAGE = A_BYTES + B_BYTES;
    static constexpr int BAR = NS * STAGE;  // barriers: FULL[NS], EMPTY[NS], ACCF[2], ACCE[2], DRAIN; tmem slot, abort
    static constexpr size_t SMEM = static_cast<size_t>(BAR) + 8 * (2 * NS + 5) + 16 + 1024;
};

__device__ __forceinline__ uint32_t bf16_bits(float x) {
    return static_cast<uint32_t>(__bfloat16_as_ushort(__float2bfloat16_rn(x)));
}

// split x = hi + lo (both bf16); returns the two 16-bit patterns
__device__ __forceinline__ void split1(float x, uint32_t& hi, uint32_t& lo) {
    const __nv_bfloat16 h = __float2bfloat16_rn(x);
    hi = static_cast<uint32_t>(__bfloat16_as_ushort(h));
    lo = bf16_bits(x - __bfloat162float(h));
}

__device__ __forceinline__ uint4 pack8(const uint32_t (&v)[8]) {
    return make_uint4(v[0] | (v[1] << 16), v[2] | (v[3] << 16), v[4] | (v[5] << 16), v[6] | (v[7] << 16));
}

// ---------------------------------------------------------------------------
// build: element sums of the representatives, then the split rows
// ---------------------------------------------------------------------------
struct KmixArgs {
    const float2* table;
    int Nx, Ny, Nz, Ex, Ey, ppx, ppy, Nox, Noy;
    int64_t P, ldk;
    const int* rep_f;
    const int* rep_mix;
    const int* rep_fl;
    const int* mix_nact;
    const int* mix_nf;
    const int64_t* mix_pref_off;
    const int* mix_act_off;
    const int* act;
    const float2* pref;
    float2* K;  // [n_rep][ldk]
};

// block per (grid line (z, y), representative); threads over x.  K[q][p] =
// sum_a pref[m, fl, a] * table[f, z, oy(a), x + ox(a)], the column_kernel sum of
// the OMP path for every point of the line.
__global__ void __launch_bounds__(256) kmix_kernel(const KmixArgs a) {
    extern __shared__ float2 sh_terms[];
    const int q = blockIdx.y, line = blockIdx.x;
    const int iy = line % a.Ny, iz = line / a.Ny;
    const int m = a.rep_mix[q], fl = a.rep_fl[q], f = a.rep_f[q];
    const int nact = a.mix_nact[m], nf = a.mix_nf[m];
    int64_t* off = reinterpret_cast<int64_t*>(sh_terms + nact);
    for (int i = threadIdx.x; i < nact; i += blockDim.x) {
        const int e = a.act[a.mix_act_off[m] + i];
        const int ey = e / a.Ex, ex = e - ey * a.Ex;
        const int oy = iy + (a.Ey - 1 - ey) * a.ppy;
        sh_terms[i] = a.pref[a.mix_pref_off[m] + static_cast<int64_t>(i) * nf + fl];
        off[i] = ((static_cast<int64_t>(f) * a.Nz + iz) * a.Noy + oy) * a.Nox + (a.Ex - 1 - ex) * a.ppx;
    }
    __syncthreads();
    float2* out = a.K + static_cast<int64_t>(q) * a.ldk + static_cast<int64_t>(line) * a.Nx;
    for (int x = threadIdx.x; x < a.Nx; x += blockDim.x) {
        float2 acc = make_float2(0.f, 0.f);
        for (int i = 0; i < nact; ++i) {
            const float2 w = sh_terms[i];
            const float2 h = __ldg(a.table + off[i] + x);
            acc.x = fmaf(w.x, h.x, fmaf(-w.y, h.y, acc.x));
            acc.y = fmaf(w.x, h.y, fmaf(w.y, h.x, acc.y));
        }
        out[x] = acc;
    }
}

struct PackArgs {
    const float2* K;
    int64_t ldk;
    const int* row_lrep;  // [rows of the chunk] representative (local index) or -1
    const int* row_slot;  // [n_obs]
    const float2* p_in;
    int64_t P, npb;
    int64_t r0, nrows;    // chunk rows [r0, r0 + nrows), both multiples of 256
    int64_t n_obs;
    uint8_t* phi;
};

// thread per (row, point block), rows of a 256-row block and point block adjacent,
// so that a warp writes 2 KB of whole core matrices
__global__ void __launch_bounds__(256) pack_kernel(const PackArgs a) {
    const int64_t n = a.nrows * a.npb;
    for (int64_t idx = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; idx < n;
         idx += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const int rr = static_cast<int>(idx & 7), rbl = static_cast<int>((idx >> 3) & 31);
        const int64_t t = idx >> 8;
        const int64_t pb = t % a.npb, RBl = t / a.npb;
        const int64_t rl = RBl * 256 + rbl * 8 + rr, r = a.r0 + rl;
        uint32_t v[4][8];
        const int q = (r < a.n_obs) ? a.row_lrep[rl] : -1;
        const int s = (q >= 0) ? a.row_slot[r] : 0;
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            const int64_t pt = pb * 8 + k;
            float2 ph = make_float2(0.f, 0.f);
            if (q >= 0 && pt < a.P) {
                const float2 kv = a.K[static_cast<int64_t>(q) * a.ldk + pt];
                const float2 pv = a.p_in[static_cast<int64_t>(s) * a.P + pt];
                ph = make_float2(pv.x * kv.x - pv.y * kv.y, pv.x * kv.y + pv.y * kv.x);
            }
            split1(ph.x, v[0][k], v[1][k]);
            split1(ph.y, v[2][k], v[3][k]);
        }
        uint8_t* dst = a.phi + (((a.r0 >> 8) + RBl) * a.npb + pb) * kPbStride + rbl * kPieceGroup + rr * 16;
        *reinterpret_cast<uint4*>(dst) = pack8(v[0]);        // re hi
        *reinterpret_cast<uint4*>(dst + 128) = pack8(v[1]);  // re lo
        *reinterpret_cast<uint4*>(dst + 256) = pack8(v[2]);  // im hi
        *reinterpret_cast<uint4*>(dst + 384) = pack8(v[3]);  // im lo
    }
}

// ---------------------------------------------------------------------------
// per-apply operands: B forms of gamma (forward) and of u (adjoint)
// ---------------------------------------------------------------------------
// forms[k8][nb 32][c 2][8 n][8 k] bf16 with n = form * 64 + b; k runs over the 8 points
// (gamma) or 8 rows (u) of K step k8.  A block takes 8 K steps (64 points or rows) at a time: it
// stages the 64 objects x 64 entries of x in shared memory with coalesced loads (one object's 64
// consecutive entries per pass of 64 threads), then writes the 8 x 512 pieces of 16 bytes, one
// per (k8, n, c), each from 8 staged entries.
constexpr int kFormsK8 = 8;  // K steps per block pass
template <bool ADJ>
__global__ void __launch_bounds__(256) forms_kernel(const float2* __restrict__ x, int64_t ldx, int B, int64_t n_in,
                                                    int64_t n_k8, uint4* __restrict__ out) {
    __shared__ float2 tile[kPhiObj][kFormsK8 * 8 + 1];  // [object][entry], padded against bank conflicts
    for (int64_t blk = blockIdx.x; blk * kFormsK8 < n_k8; blk += gridDim.x) {
        const int64_t k80 = blk * kFormsK8, i0 = k80 * 8;
        for (int e = threadIdx.x; e < kPhiObj * kFormsK8 * 8; e += blockDim.x) {
            const int b = e / (kFormsK8 * 8), kk = e % (kFormsK8 * 8);
            const int64_t i = i0 + kk;
            tile[b][kk] = (b < B && i < n_in) ? x[static_cast<int64_t>(b) * ldx + i] : make_float2(0.f, 0.f);
        }
        __syncthreads();
        for (int e = threadIdx.x; e < kFormsK8 * 512; e += blockDim.x) {
            const int k8l = e >> 9, w = e & 511;
            if (k80 + k8l >= n_k8) break;
            const int nrow = (w >> 4) * 8 + (w & 7), c = (w >> 3) & 1;
            const int form = nrow >> 6, b = nrow & 63;
            uint32_t v[8];
#pragma unroll
            for (int k = 0; k < 8; ++k) {
                const float2 z = tile[b][k8l * 8 + k];
                float val;
                if (!ADJ)  // gamma = g + ih: B1 = (g, -h), B2 = (h, g)
                    val = (form & 1) ? (c ? z.x : z.y) : (c ? -z.y : z.x);
                else       // u = c + id: B1 = (c, d), B2 = (d, -c)
                    val = (form & 1) ? (c ? -z.x : z.y) : (c ? z.y : z.x);
                uint32_t hi, lo;
                split1(val, hi, lo);
                v[k] = (form >= 2) ? lo : hi;
            }
            out[(k80 + k8l) * 512 + w] = pack8(v);
        }
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------
// GEMM kernels
// ---------------------------------------------------------------------------
struct PhiGemmArgs {
    const uint8_t* phi;
    const uint8_t* bf;      // B forms of this pass
    int64_t npb;            // point blocks of 8 (points padded to 256)
    int64_t nrb8;           // row octets (rows padded to 256)
    int n_kc;               // K chunks (gridDim.x of the forward, gridDim.y of the adjoint)
    int B;                  // objects of this pass (<= 64)
    int64_t n_out;          // valid output rows (forward: observations) or points (adjoint)
    float2* part;           // [n_kc][B][n_out]
    double2* host_out;      // adjoint with one K chunk: the caller's FP64 host columns (16-byte aligned,
    int64_t host_ld;        // leading dimension host_ld), written instead of part; else nullptr
    int* status;
    uint64_t wait_ns;
};

__device__ __forceinline__ bool wait_warp(uint32_t bar, uint32_t parity, volatile int* abort_flag, uint64_t ns) {
    return __all_sync(0xffffffffu, tc::bar_wait_abortable(bar, parity, abort_flag, ns));
}

// ADJ = false: block (kc, row block RB) contracts its 256 rows over the point range of chunk kc.
// ADJ = true: block (point block PS, kc) contracts its 256 points over the row range of chunk kc.
// HOST (adjoint with one K chunk): the epilogue writes the caller's FP64 host columns instead of
// the partials; a separate instantiation, so the device-resident kernel carries no branch for it
template <bool ADJ, int KS, int NS, bool HOST = false>
__global__ void __launch_bounds__(kPhiThreads, 1) phi_gemm_kernel(const PhiGemmArgs a,
                                                                  const __grid_constant__ CUtensorMap tmap) {
    using C = PhiCfg<KS, NS>;
    static_assert(kChain % KS == 0, "chains end on stage boundaries");
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    unsigned char* smem = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    // a block of an earlier launch gave up (status not yet read): skip the work, keep the error
    if (__syncthreads_or(tid == 0 && (*reinterpret_cast<volatile int*>(a.status) & 6) != 0)) return;
    const int kc = ADJ ? blockIdx.y : blockIdx.x;
    const int64_t tile = ADJ ? blockIdx.x : blockIdx.y;     // row block (forward) or point block of 256 (adjoint)
    const int64_t nk8 = ADJ ? a.nrb8 : a.npb;              // K steps over the whole K range
    const int64_t nst = nk8 / KS;
    const int64_t q0 = nst * kc / a.n_kc, q1 = nst * (kc + 1) / a.n_kc;
    const int nq = static_cast<int>(q1 - q0);
    const int nK = nq * KS, nch = (nK + kChain - 1) / kChain;

    const uint32_t s0 = tc::smem_u32(smem);
    const uint32_t FULL = s0 + C::BAR, EMPTY = FULL + 8 * NS, ACCF = EMPTY + 8 * NS, ACCE = ACCF + 16,
                   DRAIN = ACCE + 16;
    uint32_t* tslot = reinterpret_cast<uint32_t*>(smem + C::BAR + 8 * (2 * NS + 5));
    volatile int* abort_flag = reinterpret_cast<volatile int*>(tslot + 1);
    if (tid == 0) {
        for (int s = 0; s < NS; ++s) {
            tc::bar_init(FULL + 8 * s, 1);
            tc::bar_init(EMPTY + 8 * s, 1);
        }
        for (int b = 0; b < 2; ++b) {
            tc::bar_init(ACCF + 8 * b, 1);
            tc::bar_init(ACCE + 8 * b, 32 * kEpiWarps);
        }
        tc::bar_init(DRAIN, 1);
        *abort_flag = 0;
    }
    if (warp == 8) tc::tmem_alloc(tc::smem_u32(tslot), 512);
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = *tslot;
    int zero = 0;

    if (warp == 9) {  // ---- bulk copies ----
        bool ok = true;
        int last[NS];
#pragma unroll
        for (int s = 0; s < NS; ++s) last[s] = -1;
        for (int q = 0; q < nq; ++q) {
            const int s = q % NS;
            if (q >= NS && !(ok = wait_warp(EMPTY + 8 * s, ((q / NS) - 1) & 1, abort_flag, a.wait_ns))) break;
            const int64_t k0 = (q0 + q) * KS;  // first K step of the stage
            const uint32_t sa = s0 + s * C::STAGE, sb = sa + C::A_BYTES;
            if (lane == 0) tc::bar_expect_tx(FULL + 8 * s, C::STAGE);
            __syncwarp();
            if (!ADJ) {
                if (kPbPad == 0) {  // the stage's KS point-block chunks are one contiguous run
                    if (lane == 0) tc::bulk_g2s(sa, a.phi + (tile * a.npb + k0) * kPbStride, C::A_BYTES, FULL + 8 * s);
                } else if (lane < KS) {
                    tc::bulk_g2s(sa + lane * kKStepA, a.phi + (tile * a.npb + k0 + lane) * kPbStride, kKStepA,
                                 FULL + 8 * s);
                }
                if (lane == 0) tc::bulk_g2s(sb, a.bf + k0 * kKStepB, C::B_BYTES, FULL + 8 * s);
            } else {
                // K steps k0..k0+KS-1 are row octets of one 256-row block (KS divides 32): one tensor copy
                // of the box [point block 32][row octet KS][512 B] lands as the MN-major A stage
                if (lane == 0) {
                    const int RB = static_cast<int>(k0 >> 5), rbl0 = static_cast<int>(k0 & 31);
                    tc::tma_load_4d(sa, &tmap, 0, rbl0, static_cast<int>(tile * 32), RB, FULL + 8 * s);
                    tc::bulk_g2s(sb, a.bf + k0 * kKStepB, C::B_BYTES, FULL + 8 * s);
                }
            }
            last[s] = q / NS;
        }
        // every copy issued must have landed before the block may exit
        if (lane == 0)
            for (int s = 0; s < NS; ++s)
                if (last[s] >= 0) tc::bar_wait_abortable(FULL + 8 * s, last[s] & 1, &zero, kDrainNs);
        if (!ok && lane == 0) atomicOr(a.status, 2);
        __syncwarp();
    } else if (warp == 8) {
        if (lane == 0) {  // ---- MMA issue ----
            bool ok = true;
            // A descriptors, no swizzle: LBO is the byte step between core matrices along K (the next
            // component, 256 B) and SBO the step along M -- the next row octet (forward, K-major) or the
            // next point block (adjoint, MN-major: the point blocks sit KS pieces apart in the stage).
            // For MN-major operands the same two roles hold; a one-MMA probe against a host product
            // fixed this reading before the kernel first ran.
            constexpr uint32_t lbo = 256, sbo = ADJ ? KS * kPieceGroup : kPieceGroup;
            constexpr uint32_t tile_a = ADJ ? 16 * KS * kPieceGroup : 16 * kPieceGroup;  // 128-row/point tile
            constexpr uint32_t kstep_a = ADJ ? kPieceGroup : kKStepA;
            constexpr uint32_t tr = ADJ ? (1u << 15) : 0u;  // A MN-major in the adjoint
            constexpr uint32_t idesc = tc::idesc_bf16(128, 128) | tr;
            for (int q = 0; q < nq && ok; ++q) {
                const int s = q % NS;
                if (!(ok = tc::bar_wait_abortable(FULL + 8 * s, (q / NS) & 1, abort_flag, a.wait_ns))) break;
                tc::fence_after_sync();
                const uint32_t sa = s0 + s * C::STAGE, sb = sa + C::A_BYTES;
#pragma unroll
                for (int ks = 0; ks < KS; ++ks) {
                    const int kk = q * KS + ks, c = kk / kChain, buf = c & 1;
                    const bool first = kk % kChain == 0;
                    if (first && c >= 2 &&
                        !(ok = tc::bar_wait_abortable(ACCE + 8 * buf, ((c >> 1) - 1) & 1, abort_flag, a.wait_ns)))
                        break;
                    if (first) tc::fence_after_sync();
                    const uint64_t bh = tc::smem_desc(sb + ks * kKStepB, 128, 256);          // B1 hi | B2 hi
                    const uint64_t bl = tc::smem_desc(sb + ks * kKStepB + 4096, 128, 256);   // B1 lo | B2 lo
#pragma unroll
                    for (int t = 0; t < 2; ++t) {
                        const uint32_t ah = sa + t * tile_a + ks * kstep_a;
                        const uint64_t dh = tc::smem_desc(ah, lbo, sbo), dl = tc::smem_desc(ah + 128, lbo, sbo);
                        const uint32_t td = tmem + static_cast<uint32_t>((2 * t + buf) * 128);
                        tc::mma_bf16(td, dh, bh, idesc, first ? 0u : 1u);
                        tc::mma_bf16(td, dh, bl, idesc, 1u);
                        tc::mma_bf16(td, dl, bh, idesc, 1u);
                    }
                    if (kk % kChain == kChain - 1 || kk == nK - 1) tc::commit(ACCF + 8 * buf);
                }
                if (ok) tc::commit(EMPTY + 8 * s);
            }
            tc::commit(DRAIN);
            tc::bar_wait_abortable(DRAIN, 0, &zero, kDrainNs);
            if (!ok) atomicOr(a.status, 2);
        }
        __syncwarp();
    } else {  // ---- read-out: warp (tile t, lane quadrant qd) sums each chain into FP32 registers ----
        const int t = warp >> 2, qd = warp & 3;
        float acc[128];
#pragma unroll
        for (int i = 0; i < 128; ++i) acc[i] = 0.f;
        bool ok = true;
        for (int c = 0; c < nch; ++c) {
            const int buf = c & 1;
            if (!(ok = wait_warp(ACCF + 8 * buf, (c >> 1) & 1, abort_flag, a.wait_ns))) break;
            tc::fence_after_sync();
            const uint32_t ta = tmem + static_cast<uint32_t>((2 * t + buf) * 128) + (static_cast<uint32_t>(qd * 32) << 16);
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                float v[16];
                tc::tmem_ld16(ta + 16 * j, v);
                tc::tmem_wait_ld();
#pragma unroll
                for (int i = 0; i < 16; ++i) acc[16 * j + i] += v[i];
            }
            tc::fence_before_sync();
            tc::bar_arrive(ACCE + 8 * buf);
        }
        if (ok && nch > 0) {
            const int64_t row = tile * 256 + t * 128 + qd * 32 + lane;
            if (HOST && row < a.n_out) {
                // the finished gradient straight into the caller's host array (through the host page
                // tables), with streaming stores: 32 lanes write 512 contiguous bytes per object
                double2* out = a.host_out + row;
                const int64_t ld = a.host_ld;
#pragma unroll
                for (int b = 0; b < 64; ++b) {
                    // widened to FP64 inside the store so that no FP64 pairs stay live across stores
                    if (b < a.B)
                        asm volatile("{\n\t.reg .f64 re, im;\n\tcvt.f64.f32 re, %1;\n\tcvt.f64.f32 im, %2;\n\t"
                                     "st.global.cs.v2.f64 [%0], {re, im};\n\t}"
                                     :: "l"(out), "f"(acc[b]), "f"(acc[64 + b]) : "memory");
                    out += ld;
                }
            } else if (!HOST && row < a.n_out) {
                float2* out = a.part + static_cast<int64_t>(kc) * a.B * a.n_out + row;
#pragma unroll
                for (int b = 0; b < 64; ++b)
                    if (b < a.B) out[static_cast<int64_t>(b) * a.n_out] = make_float2(acc[b], acc[64 + b]);
            }
        } else if (!ok && lane == 0) {
            atomicOr(a.status, 2);
        }
    }
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 8) tc::tmem_dealloc(tmem, 512);
}

// Stage shapes (K steps per stage, stages), measured on the batched workload at 64 frequencies
// (68.7 GB matrix): the forward streams 6.76 TB/s with 4 x 2, 6.55 with 2 x 4 and 5.59 with 1 x 8.
// The adjoint's stage is 32 point-block pieces of KS x 512 B.  Issued as 32 bulk copies its rate
// followed the piece size (5.39 TB/s at 2 KB pieces, 4.06 at 1 KB, 2.13 at 512 B; padding the
// 16 KB stride changed nothing): the copies' issue, not DRAM, bounded it.  As one tensor copy per
// stage it streams 6.38 TB/s at 2 x 4, 5.97 at 4 x 2 and 5.25 at 1 x 8; 8 x 1 (one 192 KB stage,
// no overlap of copy and MMA) falls to 3.90.
constexpr int kFwdKS = 4, kFwdNS = 2;
constexpr int kAdjKS = 2, kAdjNS = 4;

int grid_1d(int64_t n, int threads) {
    const int64_t b = (n + threads - 1) / threads;
    return static_cast<int>(std::min<int64_t>(std::max<int64_t>(b, 1), 152 * 32));
}

// K chunks so that the grid covers the SMs several times over (at least two stages per chunk)
int pick_chunks(int64_t tiles, int64_t stages) {
    int64_t c = 1;
    while (c < 16 && tiles * c < 4 * 152 && 2 * c <= stages) c *= 2;
    return static_cast<int>(c);
}

template <typename T>
cui_status copy_back(std::vector<T>& h, const T* d, size_t n) {
    h.resize(n);
    if (n == 0) return CUI_OK;
    return check_cuda(cudaMemcpy(h.data(), d, n * sizeof(T), cudaMemcpyDeviceToHost), "folded operator metadata");
}

}  // namespace

// The adjoint's tensor map over the folded matrix, a 4D tensor of 16-bit elements, innermost first:
// 256 (the 512 B of one row octet and point block), 32 row octets of a 256-row block (stride
// 512 B), the point blocks (stride kPbStride) and the 256-row blocks (stride NPB x kPbStride).  A
// box of [256, KS, 32, 1] at (0, row octet, first point block, row block) is one adjoint stage:
// 32 point blocks x KS row octets x 512 B, in shared memory in the order the MN-major descriptor
// reads.  Every box lies inside the tensor (row octets + KS <= 32, point blocks padded to 256).
static cui_status encode_adjoint_map(Plan& p) {
    using Encode = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
    static Encode encode = nullptr;
    if (!encode) {
        void* fn = nullptr;
        cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
        const cudaError_t e = cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q);
        if (e != cudaSuccess || q != cudaDriverEntryPointSuccess || !fn)
            return set_error(CUI_ERR_CUDA, "cuTensorMapEncodeTiled is not available from the driver");
        encode = reinterpret_cast<Encode>(fn);
    }
    static_assert(sizeof(CUtensorMap) == sizeof(p.phi_tmap), "tensor map storage");
    const cuuint64_t dims[4] = {static_cast<cuuint64_t>(kPieceGroup / 2), 32, static_cast<cuuint64_t>(p.phi_npb),
                                static_cast<cuuint64_t>(p.phi_rows_pad / 256)};
    const cuuint64_t strides[3] = {static_cast<cuuint64_t>(kPieceGroup), static_cast<cuuint64_t>(kPbStride),
                                   static_cast<cuuint64_t>(p.phi_npb) * static_cast<cuuint64_t>(kPbStride)};
    const cuuint32_t box[4] = {static_cast<cuuint32_t>(kPieceGroup / 2), static_cast<cuuint32_t>(kAdjKS), 32, 1};
    const cuuint32_t estr[4] = {1, 1, 1, 1};
    if (p.phi_npb % 32 != 0 || 32 % kAdjKS != 0 || (reinterpret_cast<uintptr_t>(p.phi) & 15) != 0)
        return set_error(CUI_ERR_UNSUPPORTED_SETUP, "folded matrix layout does not tile into adjoint stages");
    CUtensorMap m;
    const CUresult r = encode(&m, CU_TENSOR_MAP_DATA_TYPE_UINT16, 4, p.phi, dims, strides, box, estr,
                              CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                              CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS)
        return set_error(CUI_ERR_CUDA, "cuTensorMapEncodeTiled failed for the folded matrix (" + std::to_string(r) + ")");
    std::memcpy(p.phi_tmap, &m, sizeof m);
    return CUI_OK;
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
size_t phi_matrix_bytes(const Plan* p) {
    const int64_t rows = (p->n_obs + 255) / 256 * 256, pts = (p->P + 255) / 256 * 256;
    return static_cast<size_t>(rows / 256) * static_cast<size_t>(pts / 8) * static_cast<size_t>(kPbStride);
}

bool phi_supported(const Plan* p, std::string* why) {
    if (p->table_mode != CUI_STORAGE_STORED || p->table == nullptr) {
        *why = "the folded operator is built from a stored transfer-function table";
        return false;
    }
    size_t free_b = 0, total_b = 0;
    if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) {
        *why = "cudaMemGetInfo failed";
        return false;
    }
    const size_t need = phi_matrix_bytes(p) + (static_cast<size_t>(1) << 30);
    if (need > free_b / 10 * 9) {
        *why = "the folded operator (" + std::to_string(phi_matrix_bytes(p) >> 20) + " MiB) does not fit in device memory";
        return false;
    }
    return true;
}

namespace {

cui_status phi_build(Plan& p) {
    std::string why;
    if (!phi_supported(&p, &why)) return set_error(CUI_ERR_UNSUPPORTED_SETUP, why);
    const int64_t n_obs = p.n_obs;
    // host copies of the row and mix metadata
    std::vector<int> row_slot, row_mix, row_fl, slot_f, mix_nact, mix_nf, mix_act_off, act;
    std::vector<int64_t> mix_pref_off;
    std::vector<float2> pref;
    cui_status st;
    if ((st = copy_back(row_slot, p.row_slot, n_obs)) != CUI_OK || (st = copy_back(row_mix, p.row_mix, n_obs)) != CUI_OK ||
        (st = copy_back(row_fl, p.row_fl, n_obs)) != CUI_OK || (st = copy_back(slot_f, p.slot_f, p.S)) != CUI_OK ||
        (st = copy_back(mix_nact, p.mix_nact, p.n_mix)) != CUI_OK || (st = copy_back(mix_nf, p.mix_nf, p.n_mix)) != CUI_OK ||
        (st = copy_back(mix_act_off, p.mix_act_off, p.n_mix)) != CUI_OK ||
        (st = copy_back(mix_pref_off, p.mix_pref_off, p.n_mix)) != CUI_OK)
        return st;
    size_t n_act = 0, n_pref = 0;
    for (int m = 0; m < p.n_mix; ++m) {
        n_act = std::max<size_t>(n_act, static_cast<size_t>(mix_act_off[m]) + mix_nact[m]);
        n_pref = std::max<size_t>(n_pref, static_cast<size_t>(mix_pref_off[m]) + static_cast<size_t>(mix_nact[m]) * mix_nf[m]);
    }
    if ((st = copy_back(act, p.act, n_act)) != CUI_OK || (st = copy_back(pref, p.pref, n_pref)) != CUI_OK) return st;

    // representatives: rows of one frequency whose mixes carry the same active elements and
    // prefactors (bitwise) share their element sum
    std::vector<int> row_rep(n_obs);
    std::vector<int> rep_row;  // first row of each representative
    {
        std::unordered_map<uint64_t, std::vector<int>> buckets;
        auto same = [&](int64_t r1, int64_t r2) {
            const int m1 = row_mix[r1], m2 = row_mix[r2];
            if (slot_f[row_slot[r1]] != slot_f[row_slot[r2]] || mix_nact[m1] != mix_nact[m2]) return false;
            const int na = mix_nact[m1];
            if (std::memcmp(&act[mix_act_off[m1]], &act[mix_act_off[m2]], sizeof(int) * na) != 0) return false;
            for (int i = 0; i < na; ++i) {
                const float2 a1 = pref[mix_pref_off[m1] + static_cast<int64_t>(i) * mix_nf[m1] + row_fl[r1]];
                const float2 a2 = pref[mix_pref_off[m2] + static_cast<int64_t>(i) * mix_nf[m2] + row_fl[r2]];
                if (std::memcmp(&a1, &a2, sizeof(float2)) != 0) return false;
            }
            return true;
        };
        for (int64_t r = 0; r < n_obs; ++r) {
            const int m = row_mix[r];
            uint64_t h = 1469598103934665603ull;
            auto mixin = [&h](const void* d, size_t n) {
                const unsigned char* c = static_cast<const unsigned char*>(d);
                for (size_t i = 0; i < n; ++i) h = (h ^ c[i]) * 1099511628211ull;
            };
            const int f = slot_f[row_slot[r]];
            mixin(&f, sizeof(f));
            mixin(&act[mix_act_off[m]], sizeof(int) * mix_nact[m]);
            for (int i = 0; i < mix_nact[m]; ++i)
                mixin(&pref[mix_pref_off[m] + static_cast<int64_t>(i) * mix_nf[m] + row_fl[r]], sizeof(float2));
            auto& b = buckets[h];
            int found = -1;
            for (int q : b)
                if (same(rep_row[q], r)) { found = q; break; }
            if (found < 0) {
                found = static_cast<int>(rep_row.size());
                rep_row.push_back(static_cast<int>(r));
                b.push_back(found);
            }
            row_rep[r] = found;
        }
    }

    const int64_t rows_pad = (n_obs + 255) / 256 * 256, pts_pad = (p.P + 255) / 256 * 256;
    p.phi_rows_pad = rows_pad;
    p.phi_npb = pts_pad / 8;
    p.phi_bytes = phi_matrix_bytes(&p);
    cudaError_t e = cudaSuccess;
    if ((st = device_alloc(p, reinterpret_cast<void**>(&p.phi), p.phi_bytes)) != CUI_OK) return st;
    if ((st = encode_adjoint_map(p)) != CUI_OK) return st;

    // element sums per chunk of 256-row blocks, as many representatives at a time as fit a
    // temporary of at most 16 GiB (every representative at once for the benchmark plans)
    const int64_t ldk = pts_pad;
    size_t free_b = 0, total_b = 0;
    if ((e = cudaMemGetInfo(&free_b, &total_b)) != cudaSuccess) return check_cuda(e, "cudaMemGetInfo");
    const size_t budget = std::min<size_t>(size_t(16) << 30, free_b / 2);
    const int64_t max_reps = std::max<int64_t>(256, static_cast<int64_t>(budget / (8 * ldk)));
    float2* dK = nullptr;
    int *d_rep_f = nullptr, *d_rep_mix = nullptr, *d_rep_fl = nullptr, *d_row_lrep = nullptr;
    const int64_t nreps_total = static_cast<int64_t>(rep_row.size());
    const int64_t kcap = std::min<int64_t>(max_reps, nreps_total);
    auto cleanup = [&]() {
        cudaFree(dK); cudaFree(d_rep_f); cudaFree(d_rep_mix); cudaFree(d_rep_fl); cudaFree(d_row_lrep);
    };
    // a chunk of rows needs at most one representative per row: chunks of kcap rows fit the temporary
    int64_t chunk_rows = rows_pad;
    if (kcap < nreps_total) chunk_rows = std::max<int64_t>(256, kcap / 256 * 256);
    if (injected_alloc_failure(p)) e = cudaErrorMemoryAllocation;
    if (e != cudaSuccess ||
        (e = cudaMalloc(&dK, 8 * static_cast<size_t>(std::max<int64_t>(kcap, 256)) * ldk)) != cudaSuccess ||
        (e = cudaMalloc(&d_rep_f, sizeof(int) * std::max<int64_t>(kcap, 256))) != cudaSuccess ||
        (e = cudaMalloc(&d_rep_mix, sizeof(int) * std::max<int64_t>(kcap, 256))) != cudaSuccess ||
        (e = cudaMalloc(&d_rep_fl, sizeof(int) * std::max<int64_t>(kcap, 256))) != cudaSuccess ||
        (e = cudaMalloc(&d_row_lrep, sizeof(int) * chunk_rows)) != cudaSuccess) {
        cleanup();
        return check_cuda(e, "folded operator build buffers");
    }
    std::vector<int> lrep_of(nreps_total, -1), h_rf, h_rm, h_rl, h_lrep;
    for (int64_t r0 = 0; r0 < rows_pad; r0 += chunk_rows) {
        const int64_t nr = std::min<int64_t>(chunk_rows, rows_pad - r0);
        h_rf.clear(); h_rm.clear(); h_rl.clear();
        h_lrep.assign(nr, -1);
        std::fill(lrep_of.begin(), lrep_of.end(), -1);
        for (int64_t i = 0; i < nr && r0 + i < n_obs; ++i) {
            const int q = row_rep[r0 + i];
            if (lrep_of[q] < 0) {
                lrep_of[q] = static_cast<int>(h_rf.size());
                const int r = rep_row[q];
                h_rf.push_back(slot_f[row_slot[r]]);
                h_rm.push_back(row_mix[r]);
                h_rl.push_back(row_fl[r]);
            }
            h_lrep[i] = lrep_of[q];
        }
        const int nq = static_cast<int>(h_rf.size());
        if ((e = cudaMemcpy(d_row_lrep, h_lrep.data(), sizeof(int) * nr, cudaMemcpyHostToDevice)) != cudaSuccess) break;
        if (nq > 0) {
            if ((e = cudaMemcpy(d_rep_f, h_rf.data(), sizeof(int) * nq, cudaMemcpyHostToDevice)) != cudaSuccess ||
                (e = cudaMemcpy(d_rep_mix, h_rm.data(), sizeof(int) * nq, cudaMemcpyHostToDevice)) != cudaSuccess ||
                (e = cudaMemcpy(d_rep_fl, h_rl.data(), sizeof(int) * nq, cudaMemcpyHostToDevice)) != cudaSuccess)
                break;
            KmixArgs k;
            k.table = p.table; k.Nx = p.Nx; k.Ny = p.Ny; k.Nz = p.Nz; k.Ex = p.Ex; k.Ey = p.Ey; k.ppx = p.ppx;
            k.ppy = p.ppy; k.Nox = p.Nox; k.Noy = p.Noy; k.P = p.P; k.ldk = ldk;
            k.rep_f = d_rep_f; k.rep_mix = d_rep_mix; k.rep_fl = d_rep_fl;
            k.mix_nact = p.mix_nact; k.mix_nf = p.mix_nf; k.mix_pref_off = p.mix_pref_off; k.mix_act_off = p.mix_act_off;
            k.act = p.act; k.pref = p.pref; k.K = dK;
            const size_t sm = (sizeof(float2) + sizeof(int64_t)) * static_cast<size_t>(p.E);
            kmix_kernel<<<dim3(p.Ny * p.Nz, nq), 256, sm>>>(k);
            count_launch();
            if ((e = cudaGetLastError()) != cudaSuccess) break;
        }
        PackArgs pa;
        pa.K = dK; pa.ldk = ldk; pa.row_lrep = d_row_lrep; pa.row_slot = p.row_slot; pa.p_in = p.p_in; pa.P = p.P;
        pa.npb = p.phi_npb; pa.r0 = r0; pa.nrows = nr; pa.n_obs = n_obs; pa.phi = p.phi;
        pack_kernel<<<grid_1d(nr * p.phi_npb, 256), 256>>>(pa);
        count_launch();
        if ((e = cudaGetLastError()) != cudaSuccess) break;
        if ((e = cudaDeviceSynchronize()) != cudaSuccess) break;
    }
    cleanup();
    if (e != cudaSuccess) return check_cuda(e, "folded operator build");
    p.phi_reps = nreps_total;

    // per-apply buffers: B forms of one 64-object pass (gamma, u) and the chunk partials
    p.phi_fwd_kc = pick_chunks(rows_pad / 256, p.phi_npb / kFwdKS);
    p.phi_adj_kc = pick_chunks(pts_pad / 256, (rows_pad / 8) / kAdjKS);
    const size_t part = 8 * static_cast<size_t>(kPhiObj) *
                        std::max<size_t>(static_cast<size_t>(p.phi_fwd_kc) * n_obs, static_cast<size_t>(p.phi_adj_kc) * p.P);
    if ((st = device_alloc(p, reinterpret_cast<void**>(&p.phi_gforms), static_cast<size_t>(p.phi_npb) * kKStepB)) != CUI_OK ||
        (st = device_alloc(p, reinterpret_cast<void**>(&p.phi_uforms), static_cast<size_t>(rows_pad / 8) * kKStepB)) != CUI_OK ||
        (st = device_alloc(p, reinterpret_cast<void**>(&p.phi_part), part)) != CUI_OK)
        return st;
    int smem_optin = 0;
    if ((e = cudaDeviceGetAttribute(&smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, p.device)) != cudaSuccess)
        return check_cuda(e, "cudaDeviceGetAttribute");
    const size_t sf = PhiCfg<kFwdKS, kFwdNS>::SMEM, sa = PhiCfg<kAdjKS, kAdjNS>::SMEM;
    if (std::max(sf, sa) > static_cast<size_t>(smem_optin))
        return set_error(CUI_ERR_UNSUPPORTED_SETUP, "shared memory too small for the folded-operator GEMM stages");
    if ((e = cudaFuncSetAttribute(phi_gemm_kernel<false, kFwdKS, kFwdNS>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  static_cast<int>(sf))) != cudaSuccess ||
        (e = cudaFuncSetAttribute(phi_gemm_kernel<true, kAdjKS, kAdjNS>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  static_cast<int>(sa))) != cudaSuccess ||
        (e = cudaFuncSetAttribute(phi_gemm_kernel<true, kAdjKS, kAdjNS, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  static_cast<int>(sa))) != cudaSuccess)
        return check_cuda(e, "cudaFuncSetAttribute");
    return CUI_OK;
}

}  // namespace

// Builds the folded operator once; a build that fails frees everything it allocated and leaves
// the plan as it was.
cui_status phi_prepare(Plan& p) {
    if (p.phi) return CUI_OK;
    if (!p.ws_status) {
        cui_status s = device_alloc(p, reinterpret_cast<void**>(&p.ws_status), sizeof(int));
        if (s != CUI_OK) return s;
        cudaError_t e = cudaMemset(p.ws_status, 0, sizeof(int));
        if (e != cudaSuccess) return check_cuda(e, "cudaMemset");
    }
    const size_t mark = p.allocations.size();
    const cui_status s = phi_build(p);
    if (s != CUI_OK) {
        release_since(p, mark);
        p.phi = p.phi_gforms = p.phi_uforms = nullptr;
        p.phi_part = nullptr;
        p.phi_bytes = 0;
        p.phi_reps = 0;
    }
    return s;
}

// Forward GEMM of objects [0, B) (B <= 64): B forms of gamma, then partials
// part[kc][b][row] of u; returns the chunk count the reduction adds.
cudaError_t launch_fwd_phi(Plan* p, const float2* gamma, int64_t ldg, int B, cudaStream_t st, int* n_kc) {
    forms_kernel<false><<<grid_1d((p->phi_npb + kFormsK8 - 1) / kFormsK8 * 256, 256), 256, 0, st>>>(gamma, ldg, B, p->P, p->phi_npb,
                                                                        reinterpret_cast<uint4*>(p->phi_gforms));
    count_launch();
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    PhiGemmArgs a;
    a.phi = p->phi; a.bf = p->phi_gforms; a.npb = p->phi_npb; a.nrb8 = p->phi_rows_pad / 8; a.n_kc = p->phi_fwd_kc;
    a.B = B; a.n_out = p->n_obs; a.part = p->phi_part; a.status = p->ws_status; a.wait_ns = p->wait_limit_ns;
    a.host_out = nullptr; a.host_ld = 0;
    if ((e = timing_begin(p, 0, st)) != cudaSuccess) return e;
    CUtensorMap unused;  // the forward's stages are contiguous runs (plain bulk copies)
    std::memset(&unused, 0, sizeof unused);
    phi_gemm_kernel<false, kFwdKS, kFwdNS>
        <<<dim3(p->phi_fwd_kc, static_cast<unsigned>(p->phi_rows_pad / 256)), kPhiThreads, PhiCfg<kFwdKS, kFwdNS>::SMEM, st>>>(
            a, unused);
    count_launch();
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    if ((e = timing_end(p, st)) != cudaSuccess) return e;
    *n_kc = p->phi_fwd_kc;
    return cudaSuccess;
}

// Adjoint GEMM of objects [0, B) (B <= 64): B forms of u, then partials part[kc][b][point].  With
// `host` (16-byte aligned FP64 columns, leading dimension ld_host) and one K chunk the GEMM writes
// the gradient there itself and *n_kc is 0: nothing is left to reduce.
cudaError_t launch_adj_phi(Plan* p, const float2* u, int64_t ldu, int B, cudaStream_t st, int* n_kc,
                           cui_complex64* host, int64_t ld_host) {
    const int64_t nrb8 = p->phi_rows_pad / 8;
    forms_kernel<true><<<grid_1d((nrb8 + kFormsK8 - 1) / kFormsK8 * 256, 256), 256, 0, st>>>(u, ldu, B, p->n_obs, nrb8,
                                                                 reinterpret_cast<uint4*>(p->phi_uforms));
    count_launch();
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    PhiGemmArgs a;
    a.phi = p->phi; a.bf = p->phi_uforms; a.npb = p->phi_npb; a.nrb8 = nrb8; a.n_kc = p->phi_adj_kc;
    a.B = B; a.n_out = p->P; a.part = p->phi_part; a.status = p->ws_status; a.wait_ns = p->wait_limit_ns;
    const bool to_host = host != nullptr && p->phi_adj_kc == 1 && (reinterpret_cast<uintptr_t>(host) & 15) == 0;
    a.host_out = to_host ? reinterpret_cast<double2*>(host) : nullptr;
    a.host_ld = ld_host;
    if ((e = timing_begin(p, 1, st)) != cudaSuccess) return e;
    CUtensorMap tmap;
    std::memcpy(&tmap, p->phi_tmap, sizeof tmap);
    const dim3 grid(static_cast<unsigned>(p->phi_npb / 32), p->phi_adj_kc);
    if (to_host)
        phi_gemm_kernel<true, kAdjKS, kAdjNS, true><<<grid, kPhiThreads, PhiCfg<kAdjKS, kAdjNS>::SMEM, st>>>(a, tmap);
    else
        phi_gemm_kernel<true, kAdjKS, kAdjNS><<<grid, kPhiThreads, PhiCfg<kAdjKS, kAdjNS>::SMEM, st>>>(a, tmap);
    count_launch();
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    if ((e = timing_end(p, st)) != cudaSuccess) return e;
    *n_kc = to_host ? 0 : p->phi_adj_kc;
    return cudaSuccess;
}

}  // namespace cui
