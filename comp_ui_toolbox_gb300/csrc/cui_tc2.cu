// Line-unit split-BF16 tensor-core (tcgen05) contractions of the Born operator
// for 2D setups with 4 grid points per element pitch.
//
// Table row of frequency f and depth z: T[o], o = x + 4*e' (x grid index,
// e' = E-1-e reversed element index; the lateral-offset table restated from
// setup_grid_symmetric.m:175-232).  Shifting the element by one moves the row
// window by 4 complex entries = 16 bytes, which is exactly the row pitch of a
// canonical no-swizzle K-major core matrix.  So the raw row, packed as bf16x2
// (re, im) words, *is* the forward's A operand over a whole grid line:
//     A[e'][x] = T[x + 4e']      descriptor LBO = 16 B, SBO = 128 B
// and no operand has to be expanded.  The adjoint contracts over elements
// (K = e') with rows = points of one residue class x = r + 4j, whose rows shift
// by one entry; it expands each residue into 16-byte "spread chunks" (chunk i =
// T[r+4i], T[r+4(i+1)], T[r+4(i+2)], T[r+4(i+3)]) with LBO = 64 B, SBO = 128 B.
//
// Columns of the B operand are (slot, object) pairs of one frequency: every
// incident wave of the frequency times a group of right-hand sides, so batched
// objects share each staged table row.  Complex arithmetic: K interleaves
// (re, im); B is stacked along N as [B1 hi | B2 hi | B1 lo | B2 lo] (NT columns
// each) with B1/B2 the two real forms that give Re and Im of the product.  Per
// K step one MMA with A hi (N = 4NT) and one with A lo (N = 2NT, accumulating
// onto the hi x hi columns) form hi*hi + lo*hi + hi*lo in FP32 tensor memory.
// Every accumulation chain covers 16 K steps and is then added into FP32
// registers (the forward) or multiplied into the gradient (the adjoint).
//
// Block: 8 producer warps (operand staging, tensor-memory read-out, epilogue),
// one warp whose lane 0 issues the MMAs and one whose lane 0 issues the bulk
// copies (table rows, incident-field and gamma segments) several stages ahead,
// so that no producer ever waits on global memory.  Stages are handed over with
// mbarriers; every wait has a wall-clock limit after which the block drains its
// asynchronous work, raises the plan's status word and returns.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <string>

#include "cui_internal.cuh"
#include "cui_tc.cuh"

namespace cui {
namespace {

constexpr int kProd = 256;                 // producer threads (warps 0-7)
constexpr int kThreads2 = kProd + 64;      // + the MMA warp and the bulk-copy warp
constexpr int kKC = 64;                    // forward: grid points per pipeline stage
constexpr int kChainChunks = 2;            // forward: stages per accumulation chain (2 x 8 K steps)
constexpr uint64_t kWaitLimitNs = 1000000000ull;  // 1 s per wait

__device__ __forceinline__ uint32_t pack2(float a, float b) {
    __nv_bfloat162 v = __floats2bfloat162_rn(a, b);
    return *reinterpret_cast<uint32_t*>(&v);
}

// hi/lo split of (a, b): hi = bf16(a, b), lo = bf16(a - hi, b - hi)
__device__ __forceinline__ void split(float a, float b, uint32_t& hi, uint32_t& lo) {
    hi = pack2(a, b);
    const float ha = __uint_as_float(hi << 16), hb = __uint_as_float(hi & 0xFFFF0000u);
    lo = pack2(a - ha, b - hb);
}

// (x, y) -> (-y, x) on a packed bf16x2 word: swap halves, negate the new low half
__device__ __forceinline__ uint32_t rot(uint32_t w) { return __byte_perm(w, 0, 0x1032) ^ 0x00008000u; }

__device__ __forceinline__ void sts128(uint32_t addr, uint32_t a, uint32_t b, uint32_t c, uint32_t d) {
    asm volatile("st.shared.v4.b32 [%0], {%1, %2, %3, %4};" ::"r"(addr), "r"(a), "r"(b), "r"(c), "r"(d) : "memory");
}

// wait by every lane of a producer warp; the result is made warp-uniform so that
// the warp-wide tcgen05.ld that follows is always executed by all 32 lanes
__device__ __forceinline__ bool warp_wait(uint32_t bar, uint32_t parity, volatile int* abort_flag, uint64_t ns) {
    const bool ok = tc::bar_wait_abortable(bar, parity, abort_flag, ns);
    return __all_sync(0xffffffffu, ok);
}

// named barrier over the 256 producer threads
__device__ __forceinline__ void producers_sync() { asm volatile("bar.sync 1, 256;" ::: "memory"); }

// byte offset of B row `row`, K group `g` (4 complex = 16 B) in a K-major stage
// whose 8-row groups are `sbo` bytes apart
__device__ __forceinline__ uint32_t b_off(int row, int g, int sbo) {
    return static_cast<uint32_t>((row >> 3) * sbo + g * 128 + (row & 7) * 16);
}

// ---------------------------------------------------------------------------
// band rows: tr[v][f][z][o], v = hi/lo of the packed (re, im) table entry
// ---------------------------------------------------------------------------
__global__ void row_kernel(const float2* __restrict__ table, uint32_t* __restrict__ tr, int64_t n_rows, int Nox,
                           int RowW, int64_t vstride) {
    const int64_t n = n_rows * RowW;
    for (int64_t idx = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; idx < n;
         idx += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const int64_t row = idx / RowW;
        const int o = static_cast<int>(idx - row * RowW);
        const float2 v = (o < Nox) ? table[row * Nox + o] : make_float2(0.f, 0.f);
        uint32_t hi, lo;
        split(v.x, v.y, hi, lo);
        tr[idx] = hi;
        tr[vstride + idx] = lo;
    }
}

// Column tiles of Bt objects (1, 2 or 4): the tile's NT columns split into Bt
// equal parts, part k holding object b0 + k with column c = k*NT/Bt + slot
// (ns <= NT/Bt).  Returns the slot index (-1: unused) and object.
template <int NT>
__device__ __forceinline__ int cols_per_object(int Bt) {
    return Bt == 4 ? NT / 4 : (Bt == 2 ? NT / 2 : NT);
}

template <int NT>
__device__ __forceinline__ void column(int c, int ns, int s0, int b0, int Bt, int B, const int* __restrict__ f_slot_list,
                                       int& slot, int& b) {
    const int per = cols_per_object<NT>(Bt);
    const int bl = c / per;
    const int sl = c - bl * per;
    b = b0 + bl;
    slot = (sl < ns && b < B) ? __ldg(f_slot_list + s0 + sl) : -1;
}

// ---------------------------------------------------------------------------
// Forward: D[e'][c] = sum over the block's grid lines and points x of
//   T_{f,z}[x + 4e'] q_c(x),   q_c = p_in[slot_c] * gamma[b_c]
// A = band row (M = 128 element rows), B = q (N = 4NT stacked rows), K = x.
// B1 = conj(q) = (q_re, -q_im) gives Re(T q), B2 = (q_im, q_re) gives Im(T q).
// The bulk-copy warp brings, per stage of 64 points, the incident-field
// segments of every slot of f and the gamma segments of the tile's objects
// ("raw" stages); producers multiply them, split to bf16 hi/lo and store B.
// ---------------------------------------------------------------------------
constexpr int kRawRow = 64 * 8 + 16;  // bytes per incident-field row of a raw stage (16 B pad: no bank conflicts)

struct Fwd2Args {
    const uint32_t* tr;
    int64_t tr_vstride;
    int RowW, RBW;
    const float2* p_fw;   // [F][Nz][nKC][ms][66]
    const float2* gamma;  // 16-byte aligned, even leading dimension
    int64_t ldg;
    const int* f_slot_ptr;
    const int* f_slot_list;
    int Nx, Nz, Ex, E, S, B, Bt, ms;  // ms: most slots of any frequency (rows of a raw stage)
    int64_t P;
    int lines_per_group, n_lines;
    float2* part;  // [groups][S][B][E]
    int* status;
    uint64_t wait_ns;  // limit of every wait for work (the drains keep kWaitLimitNs)
};

template <int NT>
struct FwdCfg {
    // 16-column tiles run three blocks per SM: two B stages, three raw stages, a quarter of tensor
    // memory and at most 64 registers a thread
    static constexpr bool THREE = NT <= 16;
    static constexpr int NS = NT >= 64 ? 2 : (NT >= 32 ? 3 : (THREE ? 2 : 4));  // B stages
    static constexpr int NR = THREE ? 3 : 4;     // raw stages
    static constexpr int STB = NT * 1024;        // 4NT rows x 64 points x 4 B
    static constexpr int SBO = 2048;             // 8-row groups: 16 K groups x 128 B
    // accumulators of 4NT columns
    static constexpr uint32_t TCOLS = NT >= 32 ? 512 : (THREE ? 128 : 256);
    static constexpr int NACC = TCOLS / (4 * NT);
    static constexpr int ITEMS = NT / 16;        // (4 points, column) items per producer
    static constexpr int LAG = NS - 1;           // read-out trails staging by LAG stages
};

template <int NT>
struct FwdLayout {
    int RS, oRaw, oBand, oBar;
    size_t total;
    __host__ __device__ FwdLayout(int ms, int Bt, int RBW) {
        using C = FwdCfg<NT>;
        RS = (ms * kRawRow + Bt * 512 + 15) & ~15;
        oRaw = C::NS * C::STB;
        oBand = oRaw + C::NR * RS;
        oBar = oBand + 16 * RBW;
        total = static_cast<size_t>(oBar) + 8 * (2 * C::NS + 2 * C::NR + 2 * C::NACC + 5) + 16;
    }
};

template <int NT>
__global__ void __launch_bounds__(kThreads2, FwdCfg<NT>::THREE ? 3 : 1) fwd_tc2_kernel(const Fwd2Args a) {
    using C = FwdCfg<NT>;
    extern __shared__ __align__(1024) unsigned char smem[];
    const FwdLayout<NT> L(a.ms, a.Bt, a.RBW);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    // the column tile varies fastest: the tiles of one line group and frequency run together and
    // share the table rows and incident-field segments through L2
    const int grp = blockIdx.y, f = blockIdx.z;
    const int s0 = a.f_slot_ptr[f], ns = a.f_slot_ptr[f + 1] - s0;
    const int b0 = blockIdx.x * a.Bt;
    const int line0 = grp * a.lines_per_group, line1 = min(line0 + a.lines_per_group, a.n_lines);
    if (ns == 0 || b0 >= a.B || line0 >= line1) return;  // uniform over the block
    // a block of an earlier launch gave up (status not yet read): skip the work, keep the error
    if (__syncthreads_or(tid == 0 && (*reinterpret_cast<volatile int*>(a.status) & 6) != 0)) return;
    const int nb = min(a.Bt, a.B - b0);
    const int nL = line1 - line0;
    const int nKC = (a.Nx + kKC - 1) / kKC;
    const int Q = nL * nKC;

    const uint32_t sB = tc::smem_u32(smem);
    const uint32_t sRaw = sB + L.oRaw, sBand = sB + L.oBand;
    const uint32_t bar0 = sB + L.oBar;
    const uint32_t FULL = bar0, EMPTY = bar0 + 8 * C::NS, RAWF = bar0 + 16 * C::NS, RAWE = RAWF + 8 * C::NR,
                   ACCF = RAWF + 16 * C::NR, ACCE = ACCF + 8 * C::NACC, BANDF = ACCE + 8 * C::NACC, BANDE = BANDF + 16,
                   DRAIN = BANDF + 32;
    uint32_t* tslot = reinterpret_cast<uint32_t*>(smem + L.oBar + 8 * (2 * C::NS + 2 * C::NR + 2 * C::NACC + 5));
    volatile int* abort_flag = reinterpret_cast<volatile int*>(tslot + 1);

    if (tid == 0) {
        for (int s = 0; s < C::NS; ++s) {
            tc::bar_init(FULL + 8 * s, kProd);
            tc::bar_init(EMPTY + 8 * s, 1);
        }
        for (int s = 0; s < C::NR; ++s) {
            tc::bar_init(RAWF + 8 * s, 1);
            tc::bar_init(RAWE + 8 * s, kProd);
        }
        for (int k = 0; k < C::NACC; ++k) {
            tc::bar_init(ACCF + 8 * k, 1);
            tc::bar_init(ACCE + 8 * k, kProd);
        }
        for (int k = 0; k < 2; ++k) {
            tc::bar_init(BANDF + 8 * k, 1);
            tc::bar_init(BANDE + 8 * k, 1);
        }
        tc::bar_init(DRAIN, 1);
        *abort_flag = 0;
    }
    if (tid < kProd) {  // zero the row buffers beyond the copied entries (read by rows e' >= E)
        const int tail = a.RBW - a.RowW;
        for (int i = tid; i < 4 * tail; i += kProd) {
            const int buf = i / tail, o = a.RowW + (i - buf * tail);
            *reinterpret_cast<uint32_t*>(smem + L.oBand + (static_cast<size_t>(buf) * a.RBW + o) * 4) = 0u;
        }
        tc::fence_async_smem();
    }
    if (warp == 8) tc::tmem_alloc(tc::smem_u32(tslot), C::TCOLS);
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = *tslot;
    int zero = 0;

    if (warp == 8) {
        if (lane == 0) {  // ---- MMA issue ----
            bool ok = true;
            constexpr uint32_t id_hi = tc::idesc_bf16(128, 4 * NT), id_lo = tc::idesc_bf16(128, 2 * NT);
            for (int q = 0; q < Q; ++q) {
                const int li = q / nKC, kc = q - li * nKC, bb = li & 1;
                if (kc == 0 && !(ok = tc::bar_wait_abortable(BANDF + 8 * bb, (li >> 1) & 1, abort_flag, a.wait_ns)))
                    break;
                const int s = q % C::NS;
                if (!(ok = tc::bar_wait_abortable(FULL + 8 * s, (q / C::NS) & 1, abort_flag, a.wait_ns))) break;
                const int k = q / kChainChunks, acc = static_cast<int>(static_cast<unsigned>(k) % C::NACC);
                const bool first = (q % kChainChunks) == 0;
                if (first && k >= C::NACC &&
                    !(ok = tc::bar_wait_abortable(ACCE + 8 * acc, ((static_cast<unsigned>(k) / C::NACC) - 1) & 1, abort_flag, a.wait_ns)))
                    break;
                tc::fence_after_sync();
                const uint32_t td = tmem + static_cast<uint32_t>(acc * 4 * NT);
                const int x0 = kc * kKC;
                const int nk = min(8, (a.Nx - x0) / 8);
                const uint32_t ahi = sBand + (bb * 2 + 0) * a.RBW * 4u + 4u * x0;
                const uint32_t alo = sBand + (bb * 2 + 1) * a.RBW * 4u + 4u * x0;
                const uint32_t bst = sB + s * C::STB;
                for (int ks = 0; ks < nk; ++ks) {
                    const uint64_t dh = tc::smem_desc(ahi + 32u * ks, 16, 128);
                    const uint64_t dl = tc::smem_desc(alo + 32u * ks, 16, 128);
                    const uint64_t db = tc::smem_desc(bst + 256u * ks, 128, C::SBO);
                    tc::mma_bf16(td, dh, db, id_hi, (first && ks == 0) ? 0u : 1u);
                    tc::mma_bf16(td, dl, db, id_lo, 1u);
                }
                tc::commit(EMPTY + 8 * s);
                if (q % kChainChunks == kChainChunks - 1 || q == Q - 1) tc::commit(ACCF + 8 * acc);
                if (kc == nKC - 1) tc::commit(BANDE + 8 * bb);
            }
            tc::commit(DRAIN);
            tc::bar_wait_abortable(DRAIN, 0, &zero, kWaitLimitNs);
            if (!ok) atomicOr(a.status, 2);
        }
    } else if (warp == 9) {
        if (lane == 0) {  // ---- bulk copies: table rows per line, raw inputs per stage ----
            bool ok = true;
            int last_raw[C::NR], last_band[2] = {-1, -1};
#pragma unroll
            for (int s = 0; s < C::NR; ++s) last_raw[s] = -1;
            auto band = [&](int li) {
                const int bb = li & 1;
                const uint32_t bytes = 4u * a.RowW;
                tc::bar_expect_tx(BANDF + 8 * bb, 2 * bytes);
                const int64_t row = static_cast<int64_t>(f) * a.Nz + (line0 + li);
                for (int v = 0; v < 2; ++v)
                    tc::bulk_g2s(sBand + (bb * 2 + v) * a.RBW * 4u, a.tr + v * a.tr_vstride + row * a.RowW, bytes,
                                 BANDF + 8 * bb);
                last_band[bb] = li >> 1;
            };
            band(0);
            if (nL > 1) band(1);
            const int bpos = min(nKC - 1, C::NR);
            for (int q = 0; q < Q; ++q) {
                const int li = q / nKC, kc = q - li * nKC;
                // rows of line li+1 go into the buffer of line li-1 once its MMAs are done
                if (kc == bpos && li >= 1 && li + 1 < nL) {
                    if (!(ok = tc::bar_wait_abortable(BANDE + 8 * ((li + 1) & 1), (((li + 1) >> 1) - 1) & 1, abort_flag,
                                                      a.wait_ns)))
                        break;
                    band(li + 1);
                }
                const int rs = q % C::NR;
                if (q >= C::NR &&
                    !(ok = tc::bar_wait_abortable(RAWE + 8 * rs, ((q / C::NR) - 1) & 1, abort_flag, a.wait_ns)))
                    break;
                const int x0 = kc * kKC;
                const uint32_t seg = 8u * min(kKC, a.Nx - x0);
                tc::bar_expect_tx(RAWF + 8 * rs, ns * kRawRow + nb * seg);
                const int64_t pt = static_cast<int64_t>(line0 + li) * a.Nx + x0;
                const uint32_t dst = sRaw + rs * L.RS;
                // every slot's segment of this stage in one copy
                tc::bulk_g2s(dst, a.p_fw + ((static_cast<int64_t>(f) * a.Nz + line0 + li) * nKC + kc) * a.ms * (kRawRow / 8),
                             ns * kRawRow, RAWF + 8 * rs);
                for (int bl = 0; bl < nb; ++bl)
                    tc::bulk_g2s(dst + a.ms * kRawRow + bl * 512, a.gamma + static_cast<int64_t>(b0 + bl) * a.ldg + pt, seg,
                                 RAWF + 8 * rs);
                last_raw[rs] = q / C::NR;
            }
            // every copy issued must have landed before the block may exit
            for (int s = 0; s < C::NR; ++s)
                if (last_raw[s] >= 0) tc::bar_wait_abortable(RAWF + 8 * s, last_raw[s] & 1, &zero, kWaitLimitNs);
            for (int k = 0; k < 2; ++k)
                if (last_band[k] >= 0) tc::bar_wait_abortable(BANDF + 8 * k, last_band[k] & 1, &zero, kWaitLimitNs);
            if (!ok) atomicOr(a.status, 2);
        }
    } else {
        // ---- producers: q = p_in * gamma -> B stages; accumulator read-out ----
        const int qd = warp & 3, h = warp >> 2;
        int cc[C::ITEMS], g4[C::ITEMS], prow[C::ITEMS], grow[C::ITEMS];
#pragma unroll
        for (int it = 0; it < C::ITEMS; ++it) {
            const int ib = warp + 8 * it, cb = ib % (NT / 8), gb = ib / (NT / 8);
            cc[it] = 8 * cb + (lane & 7);
            g4[it] = 4 * gb + (lane >> 3);
            const int per = cols_per_object<NT>(a.Bt);
            const int bl = cc[it] / per, sl = cc[it] - bl * per;
            const bool valid = sl < ns && bl < nb;
            prow[it] = valid ? sl * kRawRow + 32 * g4[it] : -1;
            grow[it] = valid ? a.ms * kRawRow + bl * 512 + 32 * g4[it] : -1;
        }
        float acc[NT];
#pragma unroll
        for (int c = 0; c < NT; ++c) acc[c] = 0.f;
        const uint32_t lane_addr = static_cast<uint32_t>(qd * 32) << 16;
        bool ok = true;
        for (int q = 0; q < Q + C::LAG && ok; ++q) {
            if (q < Q && NT == 64) {
                // 64-column tiles (4 objects x 16 slots): thread = (slot sl, 4-point group g4s), so each
                // slot's incident-field segment is read once and multiplied by the 4 objects' gamma
                const int rs = q % C::NR, s = q % C::NS;
                const int kc = q % nKC;
                const int sl = tid & 15, g4s = tid >> 4;
                if (!(ok = warp_wait(RAWF + 8 * rs, (q / C::NR) & 1, abort_flag, a.wait_ns))) break;
                const uint32_t raw = sRaw + rs * L.RS;
                const bool xin = kc * kKC + 4 * g4s < a.Nx;
                float4 pv[2], gv[4][2];
                if (xin && sl < ns) {
                    asm volatile("ld.shared.v4.f32 {%0, %1, %2, %3}, [%4];"
                                 : "=f"(pv[0].x), "=f"(pv[0].y), "=f"(pv[0].z), "=f"(pv[0].w)
                                 : "r"(raw + sl * kRawRow + 32 * g4s) : "memory");
                    asm volatile("ld.shared.v4.f32 {%0, %1, %2, %3}, [%4];"
                                 : "=f"(pv[1].x), "=f"(pv[1].y), "=f"(pv[1].z), "=f"(pv[1].w)
                                 : "r"(raw + sl * kRawRow + 32 * g4s + 16) : "memory");
                } else {
                    pv[0] = pv[1] = make_float4(0.f, 0.f, 0.f, 0.f);
                }
#pragma unroll
                for (int bl = 0; bl < 4; ++bl) {
                    if (xin && bl < nb) {
                        const uint32_t ga = raw + a.ms * kRawRow + bl * 512 + 32 * g4s;
                        asm volatile("ld.shared.v4.f32 {%0, %1, %2, %3}, [%4];"
                                     : "=f"(gv[bl][0].x), "=f"(gv[bl][0].y), "=f"(gv[bl][0].z), "=f"(gv[bl][0].w)
                                     : "r"(ga) : "memory");
                        asm volatile("ld.shared.v4.f32 {%0, %1, %2, %3}, [%4];"
                                     : "=f"(gv[bl][1].x), "=f"(gv[bl][1].y), "=f"(gv[bl][1].z), "=f"(gv[bl][1].w)
                                     : "r"(ga + 16) : "memory");
                    } else {
                        gv[bl][0] = gv[bl][1] = make_float4(0.f, 0.f, 0.f, 0.f);
                    }
                }
                tc::fence_async_smem();
                tc::bar_arrive(RAWE + 8 * rs);
                if (q >= C::NS && !(ok = warp_wait(EMPTY + 8 * s, ((q / C::NS) - 1) & 1, abort_flag, a.wait_ns))) break;
                const uint32_t bst = sB + s * C::STB;
                const float pr[4] = {pv[0].x, pv[0].z, pv[1].x, pv[1].z};
                const float pi[4] = {pv[0].y, pv[0].w, pv[1].y, pv[1].w};
#pragma unroll
                for (int bl = 0; bl < 4; ++bl) {
                    const float gr[4] = {gv[bl][0].x, gv[bl][0].z, gv[bl][1].x, gv[bl][1].z};
                    const float gi[4] = {gv[bl][0].y, gv[bl][0].w, gv[bl][1].y, gv[bl][1].w};
                    uint32_t h1[4], l1[4];
#pragma unroll
                    for (int t = 0; t < 4; ++t) {
                        const float qx = pr[t] * gr[t] - pi[t] * gi[t], qy = pr[t] * gi[t] + pi[t] * gr[t];
                        split(qx, -qy, h1[t], l1[t]);
                    }
                    const int c = bl * 16 + sl;
                    sts128(bst + b_off(c, g4s, C::SBO), h1[0], h1[1], h1[2], h1[3]);
                    sts128(bst + b_off(NT + c, g4s, C::SBO), rot(h1[0]), rot(h1[1]), rot(h1[2]), rot(h1[3]));
                    sts128(bst + b_off(2 * NT + c, g4s, C::SBO), l1[0], l1[1], l1[2], l1[3]);
                    sts128(bst + b_off(3 * NT + c, g4s, C::SBO), rot(l1[0]), rot(l1[1]), rot(l1[2]), rot(l1[3]));
                }
                tc::fence_async_smem();
                tc::bar_arrive(FULL + 8 * s);
            } else if (q < Q) {
                const int rs = q % C::NR, s = q % C::NS;
                const int kc = q % nKC;
                if (!(ok = warp_wait(RAWF + 8 * rs, (q / C::NR) & 1, abort_flag, a.wait_ns))) break;
                const uint32_t raw = sRaw + rs * L.RS;
                float4 pv[C::ITEMS][2], gv[C::ITEMS][2];
#pragma unroll
                for (int it = 0; it < C::ITEMS; ++it) {
                    const bool in = prow[it] >= 0 && kc * kKC + 4 * g4[it] < a.Nx;
                    if (in) {
                        asm volatile("ld.shared.v4.f32 {%0, %1, %2, %3}, [%4];"
                                     : "=f"(pv[it][0].x), "=f"(pv[it][0].y), "=f"(pv[it][0].z), "=f"(pv[it][0].w)
                                     : "r"(raw + prow[it]) : "memory");
                        asm volatile("ld.shared.v4.f32 {%0, %1, %2, %3}, [%4];"
                                     : "=f"(pv[it][1].x), "=f"(pv[it][1].y), "=f"(pv[it][1].z), "=f"(pv[it][1].w)
                                     : "r"(raw + prow[it] + 16) : "memory");
                        asm volatile("ld.shared.v4.f32 {%0, %1, %2, %3}, [%4];"
                                     : "=f"(gv[it][0].x), "=f"(gv[it][0].y), "=f"(gv[it][0].z), "=f"(gv[it][0].w)
                                     : "r"(raw + grow[it]) : "memory");
                        asm volatile("ld.shared.v4.f32 {%0, %1, %2, %3}, [%4];"
                                     : "=f"(gv[it][1].x), "=f"(gv[it][1].y), "=f"(gv[it][1].z), "=f"(gv[it][1].w)
                                     : "r"(raw + grow[it] + 16) : "memory");
                    } else {
                        pv[it][0] = pv[it][1] = gv[it][0] = gv[it][1] = make_float4(0.f, 0.f, 0.f, 0.f);
                    }
                }
                // the generic-proxy reads above must be ordered before the next bulk copy (async proxy) into the stage
                tc::fence_async_smem();
                tc::bar_arrive(RAWE + 8 * rs);
                if (q >= C::NS && !(ok = warp_wait(EMPTY + 8 * s, ((q / C::NS) - 1) & 1, abort_flag, a.wait_ns))) break;
                const uint32_t bst = sB + s * C::STB;
#pragma unroll
                for (int it = 0; it < C::ITEMS; ++it) {
                    const float pr[4] = {pv[it][0].x, pv[it][0].z, pv[it][1].x, pv[it][1].z};
                    const float pi[4] = {pv[it][0].y, pv[it][0].w, pv[it][1].y, pv[it][1].w};
                    const float gr[4] = {gv[it][0].x, gv[it][0].z, gv[it][1].x, gv[it][1].z};
                    const float gi[4] = {gv[it][0].y, gv[it][0].w, gv[it][1].y, gv[it][1].w};
                    uint32_t h1[4], l1[4];
#pragma unroll
                    for (int t = 0; t < 4; ++t) {
                        const float qx = pr[t] * gr[t] - pi[t] * gi[t], qy = pr[t] * gi[t] + pi[t] * gr[t];
                        split(qx, -qy, h1[t], l1[t]);  // B1 = (q_re, -q_im); B2 = rot(B1) = (q_im, q_re)
                    }
                    const int c = cc[it], g = g4[it];
                    sts128(bst + b_off(c, g, C::SBO), h1[0], h1[1], h1[2], h1[3]);
                    sts128(bst + b_off(NT + c, g, C::SBO), rot(h1[0]), rot(h1[1]), rot(h1[2]), rot(h1[3]));
                    sts128(bst + b_off(2 * NT + c, g, C::SBO), l1[0], l1[1], l1[2], l1[3]);
                    sts128(bst + b_off(3 * NT + c, g, C::SBO), rot(l1[0]), rot(l1[1]), rot(l1[2]), rot(l1[3]));
                }
                tc::fence_async_smem();
                tc::bar_arrive(FULL + 8 * s);
            }
            const int qr = q - C::LAG;
            if (qr >= 0 && (qr % kChainChunks == kChainChunks - 1 || qr == Q - 1)) {
                const int k = qr / kChainChunks, accs = static_cast<int>(static_cast<unsigned>(k) % C::NACC);
                if (!(ok = warp_wait(ACCF + 8 * accs, (static_cast<unsigned>(k) / C::NACC) & 1, abort_flag, a.wait_ns))) break;
                tc::fence_after_sync();
                const uint32_t col = tmem + lane_addr + static_cast<uint32_t>(accs * 4 * NT + h * NT);
#pragma unroll
                for (int jj = 0; jj < NT / 16; ++jj) {
                    float v1[16], v2[16];
                    tc::tmem_ld16(col + 16 * jj, v1);
                    tc::tmem_ld16(col + 2 * NT + 16 * jj, v2);
                    tc::tmem_wait_ld();
#pragma unroll
                    for (int u = 0; u < 16; ++u) acc[16 * jj + u] += v1[u] + v2[u];
                }
                tc::fence_before_sync();
                tc::bar_arrive(ACCE + 8 * accs);
            }
        }
        if (ok) {
            const int ep = qd * 32 + lane, e = a.Ex - 1 - ep;
            if (e >= 0) {
                float* out = reinterpret_cast<float*>(a.part);
#pragma unroll
                for (int c = 0; c < NT; ++c) {
                    int sl, b;
                    column<NT>(c, ns, s0, b0, a.Bt, a.B, a.f_slot_list, sl, b);
                    if (sl >= 0)
                        out[2 * (((static_cast<int64_t>(grp) * a.S + sl) * a.B + b) * a.E + e) + h] = acc[c];
                }
            }
        } else {
            atomicOr(a.status, 2);
        }
    }
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 8) {
        __syncwarp();
        tc::tmem_dealloc(tmem, C::TCOLS);
    }
}

// ---------------------------------------------------------------------------
// Adjoint of one grid line z, residue r (x = r + 4j) and frequency f:
//   Z[j][c] = sum_e' conj(T[r + 4(j + e')]) V[e'][c]
//   gamma_hat[b_c](x) += conj(p_in[slot_c](x)) Z[j][c]
// A = spread chunks of residue r (M = 128 point rows j, K = elements e'),
// expanded by the producers from the table row the bulk-copy warp brings;
// B = the V columns of the tile, split to bf16 hi/lo once per apply by
// vsplit_kernel straight into the shared-memory operand layout, so one bulk
// copy per frequency stages it.  B1 = (V_re, V_im) gives Re(conj(T) V),
// B2 = rot(B1) = (-V_im, V_re) gives -Im.  The epilogue reads the incident
// fields of the unit from the slot-major residue copy (p_ad[f][z][r][slot of
// f][j], one copy per unit) and keeps gamma_hat of its points in registers for
// the whole frequency chunk.  A block covers L grid lines (2 with 64-column
// tiles, whose single 128 KB B buffer is then reloaded once per 8 units, and
// with 16-column tiles, which run two blocks per SM with one 32 KB B buffer).
// ---------------------------------------------------------------------------

// V tiles in the B-operand layout: vs[f][tile][4NT rows x 2Epad bf16], rows
// [B1 hi | B2 hi | B1 lo | B2 lo], K-major core matrices (8 rows x 16 B), 8-row
// groups 32*Epad bytes apart -- byte-identical to what a block would stage.
template <int NT>
__global__ void vsplit_kernel(const float2* __restrict__ V, const int* __restrict__ f_slot_ptr,
                              const int* __restrict__ f_slot_list, uint32_t* __restrict__ vs, int F, int tiles, int Bt,
                              int B, int E, int Ex, int Epad) {
    const int64_t tile_words = 4ll * NT * Epad;  // 32-bit words of one tile: 4NT rows x 2Epad bf16
    const int64_t n = static_cast<int64_t>(F) * tiles * NT * (Epad / 4);
    const int SBOB = 32 * Epad;
    for (int64_t idx = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; idx < n;
         idx += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        int64_t t = idx;
        const int g = static_cast<int>(t % (Epad / 4)); t /= Epad / 4;
        const int c = static_cast<int>(t % NT); t /= NT;
        const int tile = static_cast<int>(t % tiles);
        const int f = static_cast<int>(t / tiles);
        const int s0 = f_slot_ptr[f], ns = f_slot_ptr[f + 1] - s0;
        int sl, b;
        column<NT>(c, ns, s0, tile * Bt, Bt, B, f_slot_list, sl, b);
        uint32_t hw[4], lw[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const int e = Ex - 1 - (4 * g + k);
            float2 v = make_float2(0.f, 0.f);
            if (sl >= 0 && e >= 0) v = V[(static_cast<int64_t>(sl) * B + b) * E + e];
            split(v.x, v.y, hw[k], lw[k]);
        }
        uint4* base = reinterpret_cast<uint4*>(vs + (static_cast<int64_t>(f) * tiles + tile) * tile_words);
        base[b_off(c, g, SBOB) / 16] = make_uint4(hw[0], hw[1], hw[2], hw[3]);
        base[b_off(NT + c, g, SBOB) / 16] = make_uint4(rot(hw[0]), rot(hw[1]), rot(hw[2]), rot(hw[3]));
        base[b_off(2 * NT + c, g, SBOB) / 16] = make_uint4(lw[0], lw[1], lw[2], lw[3]);
        base[b_off(3 * NT + c, g, SBOB) / 16] = make_uint4(rot(lw[0]), rot(lw[1]), rot(lw[2]), rot(lw[3]));
    }
}

struct Adj2Args {
    const uint32_t* tr;
    int64_t tr_vstride;
    int RowW, RBW;
    const float2* p_ad;  // [F][Nz][4][ms][Jp]
    int Jp;
    const uint32_t* vs;  // [F][tiles][tile bytes / 4] split V tiles (vsplit_kernel)
    int tiles;
    const int* f_slot_ptr;
    const int* f_slot_list;
    int Nx, Nz, Ex, E, Epad, B, Bt, F, fchunk, ms, L;
    int64_t P;
    float2* part;        // [nfc][B][P]
    int* status;
    uint64_t wait_ns;  // limit of every wait for work (the drains keep kWaitLimitNs)
};

template <int NT>
struct AdjCfg {
    // 16-column tiles run two blocks per SM, each with half of tensor memory, one V tile buffer
    // shared by two grid lines and at most 102 registers a thread
    static constexpr bool TWO = NT <= 16;
    static constexpr int NB = (NT >= 64 || TWO) ? 1 : 2;  // V tile buffers (128 KB each at 64 columns)
    static constexpr int NA = 3;                 // spread-chunk stages
    static constexpr int NP = TWO ? 2 : 3;       // incident-field stages
    static constexpr uint32_t TCOLS = TWO ? 256 : 512;
    static constexpr int NACC = TCOLS / (4 * NT);  // accumulators of 4NT columns: all of the block's tensor memory
    static constexpr int LAG = 2;                // shared roles: the epilogue trails the spreading by 2 units
    // 16/32-column tiles: warps 0-3 spread the A operand and warps 4-7 run the epilogues, each
    // group at its own pace (the epilogue of a unit may trail its MMAs by up to NACC units)
    static constexpr bool SPLIT = NT <= 32;
    static constexpr int MAXL = 2;               // grid lines per block, at most
    static constexpr int LINES = (NT >= 64 || TWO) ? MAXL : 1;
};

template <int NT>
struct AdjLayout {  // byte offsets of the dynamic shared memory
    int NCH, BB, AB, PS, oA, oP, oBand, oF, oBar;
    size_t total;
    __host__ __device__ AdjLayout(int Epad, int RBW, int ms, int Jp, int fchunk) {
        using C = AdjCfg<NT>;
        NCH = 128 + Epad;
        BB = 16 * NT * Epad;
        AB = 2 * NCH * 16;
        PS = ms * Jp * 8;
        oA = C::NB * BB;
        oP = oA + C::NA * AB;
        oBand = oP + C::NP * PS;
        oF = oBand + 16 * RBW;
        oBar = (oF + 4 * fchunk + 7) & ~7;
        total = static_cast<size_t>(oBar) + 8 * (2 * C::NB + 2 * C::NA + 2 * C::NP + 2 * C::NACC + 5) + 16;
    }
};

template <int NT>
__global__ void __launch_bounds__(kThreads2, AdjCfg<NT>::TWO ? 2 : 1) adj_tc2_kernel(const Adj2Args a) {
    using C = AdjCfg<NT>;
    extern __shared__ __align__(1024) unsigned char smem[];
    const AdjLayout<NT> L(a.Epad, a.RBW, a.ms, a.Jp, a.fchunk);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    // the column tile varies fastest: the tiles of one line and frequency chunk run together and
    // share the table rows and incident fields through L2
    const int tile = blockIdx.x, zb = blockIdx.y * a.L, fc = blockIdx.z;
    const int b0 = tile * a.Bt;
    const int nL = min(a.L, a.Nz - zb);
    if (b0 >= a.B || nL <= 0) return;  // uniform
    if (__syncthreads_or(tid == 0 && (*reinterpret_cast<volatile int*>(a.status) & 6) != 0)) return;
    const int f_lo = fc * a.fchunk, f_hi = min(f_lo + a.fchunk, a.F);

    const uint32_t sbase = tc::smem_u32(smem);
    const uint32_t sBv = sbase, sA = sbase + L.oA, sP = sbase + L.oP, sBand = sbase + L.oBand;
    int* sF = reinterpret_cast<int*>(smem + L.oF);
    const uint32_t bar0 = sbase + L.oBar;
    const uint32_t BFULL = bar0, BEMPTY = BFULL + 8 * C::NB, AFULL = BEMPTY + 8 * C::NB, AEMPTY = AFULL + 8 * C::NA,
                   PF = AEMPTY + 8 * C::NA, PE = PF + 8 * C::NP, ACCF = PE + 8 * C::NP, ACCE = ACCF + 8 * C::NACC,
                   BANDF = ACCE + 8 * C::NACC, BANDE = BANDF + 16, DRAIN = BANDF + 32;
    uint32_t* tslot =
        reinterpret_cast<uint32_t*>(smem + L.oBar + 8 * (2 * C::NB + 2 * C::NA + 2 * C::NP + 2 * C::NACC + 5));
    volatile int* abort_flag = reinterpret_cast<volatile int*>(tslot + 1);
    volatile int* nfa_s = reinterpret_cast<volatile int*>(tslot + 2);

    if (tid == 0) {
        for (int k = 0; k < C::NB; ++k) {
            tc::bar_init(BFULL + 8 * k, 1);
            tc::bar_init(BEMPTY + 8 * k, 1);
        }
        // with split roles, 4 warps spread (AFULL, BANDE) and 4 run the epilogue (PE, ACCE)
        const uint32_t n_role = C::SPLIT ? kProd / 2 : kProd;
        for (int k = 0; k < C::NACC; ++k) {
            tc::bar_init(ACCF + 8 * k, 1);
            tc::bar_init(ACCE + 8 * k, n_role);
        }
        for (int k = 0; k < 2; ++k) {
            tc::bar_init(BANDF + 8 * k, 1);
            tc::bar_init(BANDE + 8 * k, n_role);
        }
        for (int s = 0; s < C::NA; ++s) {
            tc::bar_init(AFULL + 8 * s, n_role);
            tc::bar_init(AEMPTY + 8 * s, 1);
        }
        for (int s = 0; s < C::NP; ++s) {
            tc::bar_init(PF + 8 * s, 1);
            tc::bar_init(PE + 8 * s, n_role);
        }
        tc::bar_init(DRAIN, 1);
        *abort_flag = 0;
        int n = 0;
        for (int f = f_lo; f < f_hi; ++f)
            if (a.f_slot_ptr[f + 1] > a.f_slot_ptr[f]) sF[n++] = f;
        *nfa_s = n;
    }
    if (tid < kProd) {
        const int tail = a.RBW - a.RowW;
        for (int i = tid; i < 4 * tail; i += kProd) {
            const int buf = i / tail, o = a.RowW + (i - buf * tail);
            *reinterpret_cast<uint32_t*>(smem + L.oBand + (static_cast<size_t>(buf) * a.RBW + o) * 4) = 0u;
        }
    }
    if (warp == 8) tc::tmem_alloc(tc::smem_u32(tslot), C::TCOLS);
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = *tslot;
    const int nfa = *nfa_s;
    const int upf = 4 * nL;  // units per frequency: lines x residues
    const int U = upf * nfa;
    const int nq = nL * nfa;  // table rows (frequency, line) in order
    const int NCH = L.NCH;
    const int SBOB = 32 * a.Epad;
    int zero = 0;

    if (warp == 8) {
        if (lane == 0) {  // ---- MMA issue ----
            bool ok = true;
            constexpr uint32_t id_hi = tc::idesc_bf16(128, 4 * NT), id_lo = tc::idesc_bf16(128, 2 * NT);
            const int ksteps = a.Epad / 8;
            for (int u = 0; u < U; ++u) {
                const int fi = u / upf, rem = u - fi * upf, zi = rem >> 2, r = rem & 3, kb = fi % C::NB;
                if (zi == 0 && r == 0 &&
                    !(ok = tc::bar_wait_abortable(BFULL + 8 * kb, (fi / C::NB) & 1, abort_flag, a.wait_ns)))
                    break;
                const int sa = u % C::NA;
                if (!(ok = tc::bar_wait_abortable(AFULL + 8 * sa, (u / C::NA) & 1, abort_flag, a.wait_ns))) break;
                const int acc = static_cast<int>(static_cast<unsigned>(u) % C::NACC);
                if (u >= C::NACC &&
                    !(ok = tc::bar_wait_abortable(ACCE + 8 * acc, ((static_cast<unsigned>(u) / C::NACC) - 1) & 1, abort_flag, a.wait_ns)))
                    break;
                tc::fence_after_sync();
                const uint32_t td = tmem + static_cast<uint32_t>(acc * 4 * NT);
                const uint32_t ah = sA + sa * L.AB, al = ah + NCH * 16, bv = sBv + kb * L.BB;
                for (int ks = 0; ks < ksteps; ++ks) {
                    const uint64_t dh = tc::smem_desc(ah + 128u * ks, 64, 128);
                    const uint64_t dl = tc::smem_desc(al + 128u * ks, 64, 128);
                    const uint64_t db = tc::smem_desc(bv + 256u * ks, 128, SBOB);
                    tc::mma_bf16(td, dh, db, id_hi, ks > 0 ? 1u : 0u);
                    tc::mma_bf16(td, dl, db, id_lo, 1u);
                }
                tc::commit(AEMPTY + 8 * sa);
                tc::commit(ACCF + 8 * acc);
                if (zi == nL - 1 && r == 3) tc::commit(BEMPTY + 8 * kb);
            }
            tc::commit(DRAIN);
            tc::bar_wait_abortable(DRAIN, 0, &zero, kWaitLimitNs);
            if (!ok) atomicOr(a.status, 4);
        }
    } else if (warp == 9) {
        if (lane == 0) {  // ---- bulk copies: V tiles per frequency, table rows per line, incident fields per unit ----
            bool ok = true;
            int last_p[C::NP], last_b[C::NB], last_band[2] = {-1, -1};
#pragma unroll
            for (int s = 0; s < C::NP; ++s) last_p[s] = -1;
#pragma unroll
            for (int s = 0; s < C::NB; ++s) last_b[s] = -1;
            auto band = [&](int q) {
                const int bb = q & 1;
                const uint32_t bytes = 4u * a.RowW;
                tc::bar_expect_tx(BANDF + 8 * bb, 2 * bytes);
                const int64_t row = static_cast<int64_t>(sF[q / nL]) * a.Nz + zb + q % nL;
                for (int v = 0; v < 2; ++v)
                    tc::bulk_g2s(sBand + (bb * 2 + v) * a.RBW * 4u, a.tr + v * a.tr_vstride + row * a.RowW, bytes,
                                 BANDF + 8 * bb);
                last_band[bb] = q >> 1;
            };
            auto vtile = [&](int fi) {
                const int kb = fi % C::NB;
                tc::bar_expect_tx(BFULL + 8 * kb, L.BB);
                tc::bulk_g2s(sBv + kb * L.BB, a.vs + (static_cast<int64_t>(sF[fi]) * a.tiles + blockIdx.x) * (L.BB / 4), L.BB,
                             BFULL + 8 * kb);
                last_b[kb] = fi / C::NB;
            };
            if (nq > 0) band(0);
            if (nq > 1) band(1);
            for (int fi = 0; fi < C::NB && fi < nfa; ++fi) vtile(fi);
            const uint32_t seg = 8u * a.Jp;
            for (int u = 0; u < U; ++u) {
                const int fi = u / upf, rem = u - fi * upf, zi = rem >> 2, r = rem & 3, q = fi * nL + zi;
                // V tile of frequency fi into the buffer of fi-NB once that frequency's MMAs are done
                if (zi == 0 && r == 0 && fi >= C::NB) {
                    if (!(ok = tc::bar_wait_abortable(BEMPTY + 8 * (fi % C::NB), ((fi / C::NB) - 1) & 1, abort_flag,
                                                      a.wait_ns)))
                        break;
                    vtile(fi);
                }
                // rows of table row q+1 go into the buffer of q-1 once the producers have spread it
                if (r == 0 && q >= 1 && q + 1 < nq) {
                    if (!(ok = tc::bar_wait_abortable(BANDE + 8 * ((q + 1) & 1), (((q + 1) >> 1) - 1) & 1, abort_flag,
                                                      a.wait_ns)))
                        break;
                    band(q + 1);
                }
                const int pu = u % C::NP;
                if (u >= C::NP &&
                    !(ok = tc::bar_wait_abortable(PE + 8 * pu, ((u / C::NP) - 1) & 1, abort_flag, a.wait_ns)))
                    break;
                const int f = sF[fi];
                const int ns = a.f_slot_ptr[f + 1] - a.f_slot_ptr[f];
                tc::bar_expect_tx(PF + 8 * pu, ns * seg);
                tc::bulk_g2s(sP + pu * L.PS, a.p_ad + ((static_cast<int64_t>(f) * a.Nz + zb + zi) * 4 + r) * a.ms * a.Jp,
                             ns * seg, PF + 8 * pu);
                last_p[pu] = u / C::NP;
            }
            // every copy issued must have landed before the block may exit
            for (int s = 0; s < C::NP; ++s)
                if (last_p[s] >= 0) tc::bar_wait_abortable(PF + 8 * s, last_p[s] & 1, &zero, kWaitLimitNs);
            for (int s = 0; s < C::NB; ++s)
                if (last_b[s] >= 0) tc::bar_wait_abortable(BFULL + 8 * s, last_b[s] & 1, &zero, kWaitLimitNs);
            for (int k = 0; k < 2; ++k)
                if (last_band[k] >= 0) tc::bar_wait_abortable(BANDF + 8 * k, last_band[k] & 1, &zero, kWaitLimitNs);
            if (!ok) atomicOr(a.status, 4);
        }
    } else {
        const int qd = warp & 3, h = warp >> 2;
        const int j = qd * 32 + lane;
        const uint32_t lane_addr = static_cast<uint32_t>(qd * 32) << 16;
        // columns per epilogue thread: half of the tile with shared roles, all of it with split roles
        constexpr int NH = C::SPLIT ? NT : NT / 2;
        // columns per pass: at most 16 and within one object (tiles of 16 or 32 columns hold at most
        // 2 objects, of 64 columns 4 objects of 16)
        constexpr int MW = C::SPLIT ? NT / 2 : (NH < 16 ? NH : 16);
        constexpr int NPS = NH / MW;                    // passes; pass ps holds one object of the tile
        const int hc = C::SPLIT ? 0 : h;                // column half of this thread's epilogue
        const int per = cols_per_object<NT>(a.Bt);
        float gx[C::MAXL][4][NPS], gy[C::MAXL][4][NPS];  // gamma_hat of x = r + 4j, line zi, pass object
#pragma unroll
        for (int zz = 0; zz < C::MAXL; ++zz)
#pragma unroll
            for (int rr = 0; rr < 4; ++rr)
#pragma unroll
                for (int ps = 0; ps < NPS; ++ps) gx[zz][rr][ps] = gy[zz][rr][ps] = 0.f;
        bool ok = true;
        // ---- spread chunks of residue r of unit `it` -> A stage (threads t0 .. t0 + nthr - 1) ----
        auto spread = [&](int it, int t0, int nthr) -> bool {
            const int fi = it / upf, rem = it - fi * upf, zi = rem >> 2, r = rem & 3, q = fi * nL + zi, bb = q & 1;
            if (r == 0 && !warp_wait(BANDF + 8 * bb, (q >> 1) & 1, abort_flag, a.wait_ns)) return false;
            const int sa = it % C::NA;
            if (it >= C::NA && !warp_wait(AEMPTY + 8 * sa, ((it / C::NA) - 1) & 1, abort_flag, a.wait_ns)) return false;
            const uint32_t as = sA + sa * L.AB;
            for (int idx = tid - t0; idx < 2 * NCH; idx += nthr) {
                const int v = idx >= NCH ? 1 : 0, i = idx - v * NCH;
                const uint32_t row = sBand + (bb * 2 + v) * a.RBW * 4u + 4u * (r + 4 * i);
                uint32_t w0, w1, w2, w3;
                asm volatile("ld.shared.b32 %0, [%1];" : "=r"(w0) : "r"(row) : "memory");
                asm volatile("ld.shared.b32 %0, [%1];" : "=r"(w1) : "r"(row + 16) : "memory");
                asm volatile("ld.shared.b32 %0, [%1];" : "=r"(w2) : "r"(row + 32) : "memory");
                asm volatile("ld.shared.b32 %0, [%1];" : "=r"(w3) : "r"(row + 48) : "memory");
                sts128(as + 16u * idx, w0, w1, w2, w3);
            }
            tc::fence_async_smem();  // orders these generic accesses before the MMAs and the next row copy
            tc::bar_arrive(AFULL + 8 * sa);
            if (r == 3) tc::bar_arrive(BANDE + 8 * bb);
            return true;
        };
        // ---- epilogue of unit ue: gamma_hat(x) += conj(p_in) * Z over this thread's columns ----
        auto epilogue = [&](int ue) -> bool {
            const int fi = ue / upf, rem = ue - fi * upf, zi = rem >> 2, r = rem & 3;
            const int accs = static_cast<int>(static_cast<unsigned>(ue) % C::NACC), pu = ue % C::NP;
            const int f = sF[fi];
            const int ns = a.f_slot_ptr[f + 1] - a.f_slot_ptr[f];
            const bool xin = r + 4 * j < a.Nx;
            if (!warp_wait(PF + 8 * pu, (ue / C::NP) & 1, abort_flag, a.wait_ns)) return false;
            float2 pv[NPS][MW];
#pragma unroll
            for (int ps = 0; ps < NPS; ++ps)
#pragma unroll
                for (int m = 0; m < MW; ++m) {
                    const int c = hc * NH + ps * MW + m, bl = c / per, sl = c - bl * per;
                    pv[ps][m] = make_float2(0.f, 0.f);  // unused columns contribute zero
                    if (sl < ns && b0 + bl < a.B && xin)
                        asm volatile("ld.shared.v2.f32 {%0, %1}, [%2];"
                                     : "=f"(pv[ps][m].x), "=f"(pv[ps][m].y)
                                     : "r"(sP + pu * L.PS + (sl * a.Jp + j) * 8) : "memory");
                }
            tc::fence_async_smem();  // generic reads before the next bulk copy into this stage
            tc::bar_arrive(PE + 8 * pu);
            if (!warp_wait(ACCF + 8 * accs, (static_cast<unsigned>(ue) / C::NACC) & 1, abort_flag, a.wait_ns)) return false;
            tc::fence_after_sync();
#pragma unroll
            for (int ps = 0; ps < NPS; ++ps) {
                const uint32_t col = tmem + lane_addr + static_cast<uint32_t>(accs * 4 * NT + hc * NH + ps * MW);
                float d0[MW], d1[MW], d2[MW], d3[MW];
                if constexpr (MW == 16) {
                    tc::tmem_ld16(col, d0);
                    tc::tmem_ld16(col + NT, d1);
                    tc::tmem_ld16(col + 2 * NT, d2);
                    tc::tmem_ld16(col + 3 * NT, d3);
                } else {
                    tc::tmem_ld8(col, d0);
                    tc::tmem_ld8(col + NT, d1);
                    tc::tmem_ld8(col + 2 * NT, d2);
                    tc::tmem_ld8(col + 3 * NT, d3);
                }
                tc::tmem_wait_ld();
                float sx = 0.f, sy = 0.f;
#pragma unroll
                for (int m = 0; m < MW; ++m) {
                    const float zr = d0[m] + d2[m], zi2 = -(d1[m] + d3[m]);
                    const float px = pv[ps][m].x, py = pv[ps][m].y;
                    sx = fmaf(px, zr, fmaf(py, zi2, sx));  // conj(p) * Z
                    sy = fmaf(px, zi2, fmaf(-py, zr, sy));
                }
#pragma unroll
                for (int zz = 0; zz < C::MAXL; ++zz)
#pragma unroll
                    for (int rr = 0; rr < 4; ++rr)
                        if (zz == zi && rr == r) {
                            gx[zz][rr][ps] += sx;
                            gy[zz][rr][ps] += sy;
                        }
            }
            tc::fence_before_sync();
            tc::bar_arrive(ACCE + 8 * accs);
            return true;
        };
        static_assert(C::LAG >= 1 && C::LAG <= C::NP, "the shared-role epilogue trails by LAG <= NP units");
        if constexpr (C::SPLIT) {
            if (h == 0) {
                for (int it = 0; it < U && ok; ++it) ok = spread(it, 0, kProd / 2);
            } else {
                for (int ue = 0; ue < U && ok; ++ue) ok = epilogue(ue);
            }
        } else {
            for (int it = 0; it < U + C::LAG && ok; ++it) {
                if (it < U) ok = spread(it, 0, kProd);
                if (ok && it >= C::LAG) ok = epilogue(it - C::LAG);
            }
        }
        if (!ok) atomicOr(a.status, 4);
        // every MMA has completed (the last epilogue waited on it) and every copy has been consumed:
        // the stage buffers from offset 0 now hold the partial gamma_hat of each (column half, pass),
        // sG[hc*NPS + ps][zi][x] (the host checks that it ends before the barriers)
        producers_sync();
        float2* sG = reinterpret_cast<float2*>(smem);
        const bool good = !*abort_flag;
        const bool has_epilogue = !C::SPLIT || h == 1;  // threads whose gx/gy hold sums
        if (good && has_epilogue) {
#pragma unroll
            for (int zz = 0; zz < C::MAXL; ++zz)
#pragma unroll
                for (int rr = 0; rr < 4; ++rr)
#pragma unroll
                    for (int ps = 0; ps < NPS; ++ps) {
                        const int x = rr + 4 * j;
                        if (zz < nL && x < a.Nx)
                            sG[((static_cast<size_t>(hc) * NPS + ps) * a.L + zz) * a.Nx + x] =
                                make_float2(gx[zz][rr][ps], gy[zz][rr][ps]);
                    }
        }
        producers_sync();
        if (good) {
            const int nb = min(a.Bt, a.B - b0);
            for (int idx = tid; idx < nb * nL * a.Nx; idx += kProd) {
                const int bl = idx / (nL * a.Nx), rest = idx - bl * (nL * a.Nx), zz = rest / a.Nx, x = rest - zz * a.Nx;
                float2 s = make_float2(0.f, 0.f);
                for (int k = 0; k < (C::SPLIT ? 1 : 2) * NPS; ++k) {  // (half, pass) slots of object bl's columns
                    const int c0 = (k / NPS) * NH + (k % NPS) * MW;
                    if (c0 / per == bl) {
                        const float2 v = sG[(static_cast<size_t>(k) * a.L + zz) * a.Nx + x];
                        s.x += v.x;
                        s.y += v.y;
                    }
                }
                a.part[(static_cast<int64_t>(fc) * a.B + b0 + bl) * a.P + static_cast<int64_t>(zb + zz) * a.Nx + x] = s;
            }
        }
    }
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 8) {
        __syncwarp();
        tc::tmem_dealloc(tmem, C::TCOLS);
    }
}

// incident fields, forward layout: p_fw[f][z][kc][sl][t] = p_in[slot sl of f][z][64kc + t] (zero padded)
__global__ void slot_major_fwd_kernel(const float2* __restrict__ p_in, const int* __restrict__ f_slot_ptr,
                                      const int* __restrict__ f_slot_list, float2* __restrict__ p_fw, int F, int Nz, int nKC,
                                      int ms, int Nx, int64_t P) {
    constexpr int W = kRawRow / 8;
    const int64_t n = static_cast<int64_t>(F) * Nz * nKC * ms * W;
    for (int64_t idx = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; idx < n;
         idx += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        int64_t t = idx;
        const int w = static_cast<int>(t % W); t /= W;
        const int sl = static_cast<int>(t % ms); t /= ms;
        const int kc = static_cast<int>(t % nKC); t /= nKC;
        const int z = static_cast<int>(t % Nz);
        const int f = static_cast<int>(t / Nz);
        const int s0 = f_slot_ptr[f], ns = f_slot_ptr[f + 1] - s0;
        const int x = kc * kKC + w;
        float2 v = make_float2(0.f, 0.f);
        if (sl < ns && w < kKC && x < Nx) v = p_in[static_cast<int64_t>(f_slot_list[s0 + sl]) * P + static_cast<int64_t>(z) * Nx + x];
        p_fw[idx] = v;
    }
}

// incident fields, adjoint layout: p_ad[f][z][r][sl][j] = p_in[slot sl of f][z][r + 4j] (zero padded)
__global__ void slot_major_adj_kernel(const float2* __restrict__ p_in, const int* __restrict__ f_slot_ptr,
                                      const int* __restrict__ f_slot_list, float2* __restrict__ p_ad, int F, int Nz, int ms,
                                      int Jp, int Nx, int64_t P) {
    const int64_t n = static_cast<int64_t>(F) * Nz * 4 * ms * Jp;
    for (int64_t idx = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; idx < n;
         idx += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        int64_t t = idx;
        const int j = static_cast<int>(t % Jp); t /= Jp;
        const int sl = static_cast<int>(t % ms); t /= ms;
        const int r = static_cast<int>(t % 4); t /= 4;
        const int z = static_cast<int>(t % Nz);
        const int f = static_cast<int>(t / Nz);
        const int s0 = f_slot_ptr[f], ns = f_slot_ptr[f + 1] - s0;
        const int x = r + 4 * j;
        float2 v = make_float2(0.f, 0.f);
        if (sl < ns && x < Nx) v = p_in[static_cast<int64_t>(f_slot_list[s0 + sl]) * P + static_cast<int64_t>(z) * Nx + x];
        p_ad[idx] = v;
    }
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
int tc2_rbw(const Plan* p) {  // entries of a shared-memory row buffer (both kernels' reach)
    const int need = std::max({p->RowW, 4 * 127 + p->Nx, 4 * (128 + p->Epad) + 12});
    return (need + 3) / 4 * 4;
}

struct Tile2 {
    int NT, Bt, tiles;
};

Tile2 tile2(const Plan* p, int B) {
    Tile2 t;
    const int ms = std::max(1, p->max_slots_per_f);
    if (B >= 2 && ms <= 8) {
        t.NT = 16, t.Bt = 2;
    } else if (B >= 2 && ms <= 16) {
        t.NT = 32, t.Bt = 2;
    } else {
        t.NT = ms <= 16 ? 16 : 32, t.Bt = 1;
    }
    t.tiles = (B + t.Bt - 1) / t.Bt;
    return t;
}

// column tiles of both kernels: 64 columns (4 objects x up to 16 waves, N = 256 per MMA) when the
// batch fills them, so that each staged table row feeds twice the columns; otherwise tile2
Tile2 tile_fwd(const Plan* p, int B) {
    if (p->tune_tile == 1) return tile2(p, B);  // the autotuner found the narrower tiles faster
    const int ms = std::max(1, p->max_slots_per_f);
    // (the adjoint's final gamma_hat of 2 lines x 4 column slots reuses its 16*64*Epad-byte V buffer)
    if (B >= 4 && ms >= 12 && ms <= 16 && p->Nx <= 16 * ((p->Ex + 15) / 16 * 16)) {
        Tile2 t;
        t.NT = 64, t.Bt = 4, t.tiles = (B + 3) / 4;
        return t;
    }
    return tile2(p, B);
}

template <int NT>
cudaError_t launch_fwd2(Plan* p, const float2* gamma, int64_t ldg, int B, const Tile2& t, cudaStream_t st,
                        int* groups_out) {
    cudaError_t e;
    // the bulk copies of gamma segments need 16-byte aligned rows
    if ((reinterpret_cast<uintptr_t>(gamma) & 15) != 0 || (ldg & 1) != 0) {
        if ((e = cudaMemcpy2DAsync(p->ws_galign, sizeof(float2) * p->P, gamma, sizeof(float2) * ldg, sizeof(float2) * p->P,
                                   B, cudaMemcpyDeviceToDevice, st)) != cudaSuccess)
            return e;
        gamma = p->ws_galign;
        ldg = p->P;
    }
    const int n_lines = p->Nz;
    const size_t slab = static_cast<size_t>(p->S) * B * p->E * sizeof(float2);
    const int target = p->tune_fwd_blocks > 0 ? p->tune_fwd_blocks : 8 * 152;  // blocks per launch
    int groups = std::max(1, std::min(n_lines, (target + p->F * t.tiles - 1) / (p->F * t.tiles)));
    groups = static_cast<int>(std::max<size_t>(1, std::min<size_t>(groups, p->ws_part_bytes / std::max<size_t>(slab, 1))));
    const int lpg = (n_lines + groups - 1) / groups;
    groups = (n_lines + lpg - 1) / lpg;  // every group holds at least one line
    Fwd2Args a;
    a.tr = p->tr; a.tr_vstride = p->tr_vstride; a.RowW = p->RowW; a.RBW = tc2_rbw(p);
    a.p_fw = p->p_fw; a.gamma = gamma; a.ldg = ldg;
    a.f_slot_ptr = p->f_slot_ptr; a.f_slot_list = p->f_slot_list;
    a.Nx = p->Nx; a.Nz = p->Nz; a.Ex = p->Ex; a.E = p->E; a.S = p->S; a.B = B; a.Bt = t.Bt;
    a.ms = p->ms; a.P = p->P;
    a.lines_per_group = lpg; a.n_lines = n_lines; a.part = p->ws_part; a.status = p->ws_status; a.wait_ns = p->wait_limit_ns;
    const size_t smem = FwdLayout<NT>(a.ms, a.Bt, a.RBW).total;
    if ((e = cudaFuncSetAttribute(fwd_tc2_kernel<NT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  static_cast<int>(smem))) != cudaSuccess)
        return e;
    if ((e = timing_begin(p, 0, st)) != cudaSuccess) return e;
    fwd_tc2_kernel<NT><<<dim3(t.tiles, groups, p->F), kThreads2, smem, st>>>(a);
    count_launch();
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    *groups_out = groups;
    return timing_end(p, st);
}

template <int NT>
cudaError_t launch_adj2(Plan* p, int B, const Tile2& t, cudaStream_t st, int* nfc_out) {
    const int Lz = AdjCfg<NT>::LINES;  // grid lines per block
    const int zblocks = (p->Nz + Lz - 1) / Lz;
    const size_t slab = static_cast<size_t>(B) * p->P * sizeof(float2);
    const int target = p->tune_adj_blocks > 0 ? p->tune_adj_blocks : 8 * 152;  // blocks per launch
    int nfc = std::max(1, std::min(p->F, (target + zblocks * t.tiles - 1) / (zblocks * t.tiles)));
    nfc = static_cast<int>(std::max<size_t>(1, std::min<size_t>(nfc, p->ws_part_bytes / std::max<size_t>(slab, 1))));
    const int fchunk = (p->F + nfc - 1) / nfc;
    nfc = (p->F + fchunk - 1) / fchunk;
    // V (unmixed data) -> split bf16 tiles in the B-operand layout, one per (frequency, column tile)
    const int64_t nv = static_cast<int64_t>(p->F) * t.tiles * NT * (p->Epad / 4);
    vsplit_kernel<NT><<<static_cast<int>(std::min<int64_t>((nv + 255) / 256, 152 * 32)), 256, 0, st>>>(
        p->ws_G, p->f_slot_ptr, p->f_slot_list, p->ws_vs, p->F, t.tiles, t.Bt, B, p->E, p->Ex, p->Epad);
    count_launch();
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    Adj2Args a;
    a.tr = p->tr; a.tr_vstride = p->tr_vstride; a.RowW = p->RowW; a.RBW = tc2_rbw(p);
    a.p_ad = p->p_ad; a.Jp = p->Jp; a.vs = p->ws_vs; a.tiles = t.tiles;
    a.f_slot_ptr = p->f_slot_ptr; a.f_slot_list = p->f_slot_list;
    a.Nx = p->Nx; a.Nz = p->Nz; a.Ex = p->Ex; a.E = p->E; a.Epad = p->Epad; a.B = B; a.Bt = t.Bt; a.F = p->F;
    a.fchunk = fchunk; a.ms = p->ms; a.L = Lz; a.P = p->P; a.part = p->ws_part; a.status = p->ws_status; a.wait_ns = p->wait_limit_ns;
    const AdjLayout<NT> L(a.Epad, a.RBW, a.ms, a.Jp, a.fchunk);
    {   // the final gamma_hat sums staged over the stage buffers must end before the barriers
        using C = AdjCfg<NT>;
        constexpr int NH = C::SPLIT ? NT : NT / 2, MW = C::SPLIT ? NT / 2 : (NH < 16 ? NH : 16);
        const size_t sg = sizeof(float2) * (C::SPLIT ? 1 : 2) * (NH / MW) * static_cast<size_t>(Lz) * p->Nx;
        if (sg > static_cast<size_t>(L.oBar)) return cudaErrorInvalidValue;
    }
    if ((e = cudaFuncSetAttribute(adj_tc2_kernel<NT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  static_cast<int>(L.total))) != cudaSuccess)
        return e;
    if ((e = timing_begin(p, 1, st)) != cudaSuccess) return e;
    adj_tc2_kernel<NT><<<dim3(t.tiles, zblocks, nfc), kThreads2, L.total, st>>>(a);
    count_launch();
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    *nfc_out = nfc;
    return timing_end(p, st);
}

// largest dynamic shared memory any launch of this plan can request
size_t tc2_smem_need(const Plan* p, int Epad, int RowW) {
    Plan q = *p;
    q.Epad = Epad;
    q.RowW = RowW;
    const int rbw = tc2_rbw(&q);
    const int ms = std::max(1, p->max_slots_per_f);
    const int Jp = ((p->Nx + 3) / 4 + 1) / 2 * 2;
    size_t need = 0;
    for (int B = 1; B <= std::min(p->max_objects, 4); ++B) {
        const Tile2 tf = tile_fwd(p, B);
        if (tf.NT == 64)
            need = std::max({need, FwdLayout<64>(ms, tf.Bt, rbw).total, AdjLayout<64>(Epad, rbw, ms, Jp, p->F).total});
        const Tile2 t = tile2(p, B);
        if (t.NT == 16)
            need = std::max({need, FwdLayout<16>(ms, t.Bt, rbw).total, AdjLayout<16>(Epad, rbw, ms, Jp, p->F).total});
        else
            need = std::max({need, FwdLayout<32>(ms, t.Bt, rbw).total, AdjLayout<32>(Epad, rbw, ms, Jp, p->F).total});
    }
    return need;
}

}  // namespace

bool tc2_supported(const Plan* p, std::string* why) {
    if (p->n_dims != 2) { *why = "line-unit kernels cover 2D setups"; return false; }
    if (p->ppx != 4) { *why = "line-unit kernels need 4 grid points per element pitch"; return false; }
    if (p->Ex > 128) { *why = "line-unit kernels cover up to 128 elements"; return false; }
    if (p->Nx % 8 != 0 || p->Nx > 512) { *why = "line-unit kernels need a lateral grid of 8..512 points, a multiple of 8"; return false; }
    if (p->max_slots_per_f > 32) { *why = "line-unit kernels cover up to 32 incident waves per frequency"; return false; }
    // the 32-column adjoint's final gamma_hat halves (2 x Nx) reuse its two V buffers (2 x 16 NT Epad bytes)
    if (16 * p->Nx > 32 * 16 * ((p->Ex + 15) / 16 * 16)) {
        *why = "lateral grid too wide for the element count of the line-unit kernels";
        return false;
    }
    int smem_optin = 0;
    if (cudaDeviceGetAttribute(&smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, p->device) != cudaSuccess) {
        *why = "cudaDeviceGetAttribute failed";
        return false;
    }
    const size_t need = tc2_smem_need(p, (p->Ex + 15) / 16 * 16, (p->Nox + 3) / 4 * 4);
    if (need > static_cast<size_t>(smem_optin)) { *why = "line-unit staging exceeds shared memory"; return false; }
    return true;
}

cui_status tc2_build(Plan& p) {
    p.Epad = (p.Ex + 15) / 16 * 16;
    p.RowW = (p.Nox + 3) / 4 * 4;
    p.Jp = ((p.Nx + 3) / 4 + 1) / 2 * 2;  // points per residue, even: 16-byte rows
    const int64_t n_rows = static_cast<int64_t>(p.F) * p.Nz * p.Noy;
    p.tr_vstride = n_rows * p.RowW;
    cui_status st = device_alloc(p, reinterpret_cast<void**>(&p.tr), sizeof(uint32_t) * 2 * p.tr_vstride);
    if (st != CUI_OK) return st;
    p.ms = std::max(1, p.max_slots_per_f);
    p.nKC = (p.Nx + kKC - 1) / kKC;
    const size_t fw_elems = static_cast<size_t>(p.F) * p.Nz * p.nKC * p.ms * (kRawRow / 8);
    const size_t ad_elems = static_cast<size_t>(p.F) * p.Nz * 4 * p.ms * p.Jp;
    if ((st = device_alloc(p, reinterpret_cast<void**>(&p.p_fw), sizeof(float2) * fw_elems)) != CUI_OK) return st;
    if ((st = device_alloc(p, reinterpret_cast<void**>(&p.p_ad), sizeof(float2) * ad_elems)) != CUI_OK) return st;
    if ((st = device_alloc(p, reinterpret_cast<void**>(&p.ws_galign), sizeof(float2) * p.P * p.max_objects)) != CUI_OK)
        return st;
    size_t vs_bytes = 0;  // split V tiles of the largest apply: F x tiles x 16 NT Epad bytes
    for (int B = 1; B <= p.max_objects; ++B) {
        const Tile2 t = tile_fwd(&p, B);
        vs_bytes = std::max(vs_bytes, static_cast<size_t>(p.F) * t.tiles * 16 * t.NT * p.Epad);
    }
    if ((st = device_alloc(p, reinterpret_cast<void**>(&p.ws_vs), vs_bytes)) != CUI_OK) return st;
    int blocks = static_cast<int>(std::min<int64_t>((p.tr_vstride + 255) / 256, 152 * 32));
    row_kernel<<<blocks, 256>>>(p.table, p.tr, n_rows, p.Nox, p.RowW, p.tr_vstride);
    count_launch();
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return check_cuda(e, "band rows");
    slot_major_fwd_kernel<<<152 * 16, 256>>>(p.p_in, p.f_slot_ptr, p.f_slot_list, p.p_fw, p.F, p.Nz, p.nKC, p.ms, p.Nx, p.P);
    count_launch();
    slot_major_adj_kernel<<<152 * 16, 256>>>(p.p_in, p.f_slot_ptr, p.f_slot_list, p.p_ad, p.F, p.Nz, p.ms, p.Jp, p.Nx, p.P);
    count_launch();
    if ((e = cudaGetLastError()) != cudaSuccess) return check_cuda(e, "slot-major incident fields");
    if ((e = cudaDeviceSynchronize()) != cudaSuccess) return check_cuda(e, "line-unit tables");
    p.tc_bytes += sizeof(uint32_t) * 2 * static_cast<size_t>(p.tr_vstride) + sizeof(float2) * (fw_elems + ad_elems) +
                  sizeof(float2) * p.P * p.max_objects + vs_bytes;
    p.tc2 = 1;
    return CUI_OK;
}

// Line-unit tables, built once; a build that fails frees what it allocated and leaves the plan as
// it was (the next switch starts over).
cui_status tc2_prepare(Plan& p) {
    if (p.tc2) return CUI_OK;
    const size_t mark = p.allocations.size();
    const size_t tc_bytes0 = p.tc_bytes;
    const cui_status s = tc2_build(p);
    if (s != CUI_OK) {
        release_since(p, mark);
        p.tr = nullptr;
        p.p_fw = p.p_ad = nullptr;
        p.ws_galign = nullptr;
        p.ws_vs = nullptr;
        p.tc_bytes = tc_bytes0;
    }
    return s;
}

cudaError_t launch_fwd_tc2(Plan* p, const float2* gamma, int64_t ldg, int B, cudaStream_t st, int* groups) {
    const Tile2 t = tile_fwd(p, B);
    if (t.NT == 64) return launch_fwd2<64>(p, gamma, ldg, B, t, st, groups);
    return t.NT == 16 ? launch_fwd2<16>(p, gamma, ldg, B, t, st, groups) : launch_fwd2<32>(p, gamma, ldg, B, t, st, groups);
}

cudaError_t launch_adj_tc2(Plan* p, int B, cudaStream_t st, int* nfc) {
    const Tile2 t = tile_fwd(p, B);  // the adjoint uses the forward's column tiles
    if (t.NT == 64) return launch_adj2<64>(p, B, t, st, nfc);
    return t.NT == 16 ? launch_adj2<16>(p, B, t, st, nfc) : launch_adj2<32>(p, B, t, st, nfc);
}

}  // namespace cui
