// FP32 Born operator kernels for sm_103a and the device apply entry points.
//
// The reference builds the matrix Phi_e = h_e .* p_in .* pref_e for every
// (measurement, mix, active element), writes it to global memory and hands
// it to cuBLAS (+scattering/combined_quick_gpu.cu:1099-1124, :902-921).  Here
// the element sum is taken out of the mixing:
//
//   forward   G[s, e]  = sum_p  h(f_s; o(p, e), z_p) * p_in[s, p] * gamma[p]
//             u[row]   = sum_{a in mix} pref[mix, f_row, a] * G[s_row, act[a]]
//   adjoint   V[s, e]  = sum_{rows of s} conj(pref[mix, f_row, pos(e)]) * u[row]
//             gh[p]    = sum_s conj(p_in[s, p]) * sum_e conj(h(f_s; o(p, e), z_p)) * V[s, e]
//
// with o(p, e) = i_x - e_x*ppp_x + (E_x-1)*ppp_x (and likewise in y) the
// signed lateral offset that indexes the lateral table.  Along one grid line
// (fixed z, y) and one residue r = i_x mod ppp_x the table entries form a
// Toeplitz band: h(r + ppp*j, e) = A_r[j - e + E_x - 1].  Each thread keeps a
// register window of KE (forward) or KJ (adjoint) consecutive band entries
// and slides it by one entry per step, so a step costs one shared-memory load
// of the band plus broadcast loads of the wave columns.  Table rows and
// incident-field rows are staged in shared memory per grid line; partial sums
// go to plan-owned scratch and are reduced in a fixed order (deterministic).
#include <cuda_runtime.h>
#include <cstdint>
#include <cstdio>
#include <algorithm>
#include <mutex>
#include <string>

#include "cui_internal.cuh"

namespace cui {

namespace {

constexpr int kPad = 8;  // zero padding on both ends of each staged band

__device__ __forceinline__ void cmac(float2& acc, float2 a, float2 b) {
    acc.x = fmaf(a.x, b.x, acc.x);
    acc.x = fmaf(-a.y, b.y, acc.x);
    acc.y = fmaf(a.x, b.y, acc.y);
    acc.y = fmaf(a.y, b.x, acc.y);
}

// acc += conj(a) * b
__device__ __forceinline__ void cmac_conj(float2& acc, float2 a, float2 b) {
    acc.x = fmaf(a.x, b.x, acc.x);
    acc.x = fmaf(a.y, b.y, acc.x);
    acc.y = fmaf(a.x, b.y, acc.y);
    acc.y = fmaf(-a.y, b.x, acc.y);
}

__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
    return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

struct LineGeom {
    int Nx, Ny, Nz, Ex, Ey, ppx, ppy, Nox, Noy;
    int64_t P;
    int E, S, F;
    int Ni, Nj_max;
};

// Stage table row (f, z, oy) into residue-major bands: band r holds
// A_r[i] = row[r + ppx*i] at sA[r*Ni + kPad + i]; entries outside the row are 0.
__device__ __forceinline__ void stage_band(float2* sA, const float2* __restrict__ row, const LineGeom& g) {
    const int n = g.ppx * g.Ni;
    for (int idx = threadIdx.x; idx < n; idx += blockDim.x) {
        const int r = idx / g.Ni;
        const int i = idx - r * g.Ni - kPad;
        const int o = r + g.ppx * i;
        sA[idx] = (i >= 0 && o < g.Nox) ? __ldg(row + o) : make_float2(0.f, 0.f);
    }
}

// Same bands with the entries of row (f, z, oy) computed in place (generated table, 3D setups).
__device__ __forceinline__ void stage_band_gen(float2* sA, const TableGen& t, int f, int z, int oy, const LineGeom& g) {
    const GenRow row = gen_row(t, f, z, oy);
    const int n = g.ppx * g.Ni;
    for (int idx = threadIdx.x; idx < n; idx += blockDim.x) {
        const int r = idx / g.Ni;
        const int i = idx - r * g.Ni - kPad;
        const int o = r + g.ppx * i;
        sA[idx] = (i >= 0 && o < g.Nox) ? gen_entry(t, row, o) : make_float2(0.f, 0.f);
    }
}

// Table row (f, z, oy) into the bands at sA: read from the stored table or generated.
template <bool GEN>
__device__ __forceinline__ void stage_row(float2* sA, const float2* __restrict__ table, int tab_f0, const TableGen& t,
                                          int f, int z, int oy, const LineGeom& g) {
    if constexpr (GEN)
        stage_band_gen(sA, t, f, z, oy, g);
    else
        stage_band(sA, table + ((static_cast<int64_t>(f - tab_f0) * g.Nz + z) * g.Noy + oy) * g.Nox, g);
}

// Skewed band layout of the FP32 contractions: entry n of the staged bands sits at n + n/16.  Their
// lanes read the bands one window (KJ or KE entries) apart; at an even window (the 2D arrays' 4)
// lanes 16/window apart would hit the same shared-memory bank, and one padding entry per 16 spreads
// them over all banks.
template <bool SKEW>
__device__ __forceinline__ int band_at(int n) { return SKEW ? n + (n >> 4) : n; }
__host__ __device__ constexpr size_t band_capacity(size_t n) { return n + (n >> 4) + 1; }

template <bool GEN, bool SKEW>
__device__ __forceinline__ void stage_row_at(float2* sA, int off, const float2* __restrict__ table, int tab_f0,
                                             const TableGen& t, int f, int z, int oy, const LineGeom& g) {
    const int n = g.ppx * g.Ni;
    if constexpr (GEN) {
        const GenRow row = gen_row(t, f, z, oy);
        for (int idx = threadIdx.x; idx < n; idx += blockDim.x) {
            const int r = idx / g.Ni;
            const int i = idx - r * g.Ni - kPad;
            const int o = r + g.ppx * i;
            sA[band_at<SKEW>(off + idx)] = (i >= 0 && o < g.Nox) ? gen_entry(t, row, o) : make_float2(0.f, 0.f);
        }
    } else {
        const float2* __restrict__ rowp = table + ((static_cast<int64_t>(f - tab_f0) * g.Nz + z) * g.Noy + oy) * g.Nox;
        for (int idx = threadIdx.x; idx < n; idx += blockDim.x) {
            const int r = idx / g.Ni;
            const int i = idx - r * g.Ni - kPad;
            const int o = r + g.ppx * i;
            sA[band_at<SKEW>(off + idx)] = (i >= 0 && o < g.Nox) ? __ldg(rowp + o) : make_float2(0.f, 0.f);
        }
    }
}

// ---------------------------------------------------------------------------
// dense forward: block = (line group x ey, frequency, object x column pass)
// ---------------------------------------------------------------------------
struct FwdArgs {
    LineGeom g;
    const float2* __restrict__ table;  // stored table (frequencies from tab_f0 on), or null when generated (gen)
    TableGen gen;
    int f_base, tab_f0;                // frequency of blockIdx.y = 0; first frequency the table holds
    const float2* __restrict__ p_in;
    const float2* __restrict__ gamma;
    int64_t ldg;
    const int* __restrict__ f_slot_ptr;
    const int* __restrict__ f_slot_list;
    int lines_per_group, n_lines;
    int n_eg, nseg, Js, ntask;
    int le;                     // lanes per element group; the 32/le lane groups split the j range
    int eyb, n_eyb;             // element rows (ey) per block, blocks per line group
    int B, npass;
    float2* __restrict__ part;  // [groups][S][B][E]
    const int* occ_sel;         // non-null: the occupancy pass's choice; 1 = the compacted forward runs instead
};

template <int NC, int KE, bool GEN>
__device__ __forceinline__ void fwd_dense_body(const FwdArgs& a) {
    if (a.occ_sel && *a.occ_sel != 0) return;  // uniform over the block
    extern __shared__ float4 smem_f4[];
    const LineGeom& g = a.g;
    const int EB = a.eyb;
    // lanes KE entries apart: the skewed band layout (band_at) at 4-entry windows (2d-plain forward
    // 0.208 -> 0.180 ms); the 3D forward's 2-entry windows measured slower with it (172.8 -> 180.6 ms)
    constexpr bool SKEW = (KE % 4) == 0;
    float2* sA = reinterpret_cast<float2*>(smem_f4);  // [EB][ppx * Ni] bands of the block's element rows
    float2* sQ = sA + band_capacity(static_cast<size_t>(EB) * g.ppx * g.Ni);  // [Nx][NC]
    float2* sR = sQ + g.Nx * NC;                     // [EB][Ex][NC]
    __shared__ int sSlot[NC];

    // a block covers EB element rows ey0 .. ey0+EB-1: each staged q line feeds all of them
    const int grp = blockIdx.x / a.n_eyb, ey0 = (blockIdx.x - grp * a.n_eyb) * EB;
    const int neb = min(EB, g.Ey - ey0);
    const int f = a.f_base + blockIdx.y;
    const int b = blockIdx.z / a.npass, cp = blockIdx.z - b * a.npass;
    const int s0 = a.f_slot_ptr[f];
    const int ns = a.f_slot_ptr[f + 1] - s0;
    const int c0 = cp * NC;
    if (c0 >= ns) return;  // uniform over the block
    const int nc = min(NC, ns - c0);
    if (threadIdx.x < NC) sSlot[threadIdx.x] = (threadIdx.x < nc) ? a.f_slot_list[s0 + c0 + threadIdx.x] : 0;

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    int r = 0, eg = 0, ek = 0, seg = 0;
    if (warp < a.ntask) {
        r = warp % g.ppx;
        int rest = warp / g.ppx;
        eg = rest % a.n_eg;
        rest /= a.n_eg;
        ek = rest % EB;
        seg = rest / EB;
    }
    const bool task_on = warp < a.ntask && ek < neb;
    // lane = (element group el, j sub-range sub): rows narrower than 32 windows of KE elements
    // keep every lane busy by splitting the task's j range among 32/le lane groups
    const int el = lane % a.le, sub = lane / a.le, nsub = 32 / a.le;
    const int e0 = (eg * a.le + el) * KE;
    const int Nj_r = (r < g.Nx) ? (g.Nx - r + g.ppx - 1) / g.ppx : 0;
    const int jlo0 = seg * a.Js, jhi0 = min(jlo0 + a.Js, Nj_r);
    const int jspan = (max(jhi0 - jlo0, 0) + nsub - 1) / nsub;
    const int jlo = jlo0 + sub * jspan, jhi = min(jlo + jspan, jhi0);
    const bool lane_on = task_on && (e0 < g.Ex) && (jlo < jhi);

    float2 acc[KE][NC];
#pragma unroll
    for (int t = 0; t < KE; ++t)
#pragma unroll
        for (int c = 0; c < NC; ++c) acc[t][c] = make_float2(0.f, 0.f);

    const int line0 = grp * a.lines_per_group;
    const int line1 = min(line0 + a.lines_per_group, a.n_lines);
    for (int line = line0; line < line1; ++line) {
        const int iy = line % g.Ny, z = line / g.Ny;
        const int64_t pt0 = (static_cast<int64_t>(z) * g.Ny + iy) * g.Nx;
        __syncthreads();
        for (int k = 0; k < neb; ++k) {
            const int oy = iy - (ey0 + k) * g.ppy + (g.Ey - 1) * g.ppy;
            stage_row_at<GEN, SKEW>(sA, k * g.ppx * g.Ni, a.table, a.tab_f0, a.gen, f, z, oy, g);
        }
        const float2* gam = a.gamma + static_cast<int64_t>(b) * a.ldg + pt0;
        for (int idx = threadIdx.x; idx < NC * g.Nx; idx += blockDim.x) {
            const int c = idx / g.Nx, x = idx - c * g.Nx;
            float2 q = make_float2(0.f, 0.f);
            if (c < nc) q = cmul(__ldg(a.p_in + static_cast<int64_t>(sSlot[c]) * g.P + pt0 + x), __ldg(gam + x));
            sQ[x * NC + c] = q;
        }
        __syncthreads();
        if (lane_on) {
            int base = ek * g.ppx * g.Ni + r * g.Ni + kPad + jlo - e0 + g.Ex - 1;  // in band r of row ek
            float2 win[KE];
#pragma unroll
            for (int t = 0; t < KE; ++t) win[t] = sA[band_at<SKEW>(base - t)];
            for (int j = jlo; j < jhi; ++j) {
                const float2* qx = sQ + (r + g.ppx * j) * NC;
                float2 q[NC];
#pragma unroll
                for (int c = 0; c < NC; ++c) q[c] = qx[c];
#pragma unroll
                for (int t = 0; t < KE; ++t)
#pragma unroll
                    for (int c = 0; c < NC; ++c) cmac(acc[t][c], win[t], q[c]);
#pragma unroll
                for (int t = KE - 1; t > 0; --t) win[t] = win[t - 1];
                ++base;
                win[0] = sA[band_at<SKEW>(base)];
            }
        }
    }

    // deterministic reduction over (residue, segment) tasks of the block
    __syncthreads();
    for (int idx = threadIdx.x; idx < EB * g.Ex * NC; idx += blockDim.x) sR[idx] = make_float2(0.f, 0.f);
    __syncthreads();
    for (int w = 0; w < a.ntask; ++w) {
        if (warp == w) {
            for (int sb = 0; sb < nsub; ++sb) {  // lane groups of one warp add to the same elements in turn
                if (sub == sb && lane_on) {
#pragma unroll
                    for (int t = 0; t < KE; ++t) {
                        const int e = e0 + t;
                        if (e < g.Ex) {
#pragma unroll
                            for (int c = 0; c < NC; ++c) {
                                float2 v = sR[(ek * g.Ex + e) * NC + c];
                                v.x += acc[t][c].x;
                                v.y += acc[t][c].y;
                                sR[(ek * g.Ex + e) * NC + c] = v;
                            }
                        }
                    }
                }
                __syncwarp();
            }
        }
        __syncthreads();
    }
    for (int idx = threadIdx.x; idx < neb * nc * g.Ex; idx += blockDim.x) {
        const int k = idx / (nc * g.Ex), rem = idx - k * (nc * g.Ex);
        const int c = rem / g.Ex, ex = rem - c * g.Ex;
        const int64_t o = ((static_cast<int64_t>(grp) * g.S + sSlot[c]) * a.B + b) * g.E + ex + g.Ex * (ey0 + k);
        a.part[o] = sR[(k * g.Ex + ex) * NC + c];
    }
}

template <int NC, int KE>
__global__ void __launch_bounds__(512) fwd_dense_kernel(const FwdArgs a) {
    fwd_dense_body<NC, KE, false>(a);
}

// Generated table: computing the entries while the accumulators stay live needs more registers than
// ptxas grants under a 512-thread bound (it settles at 64 and spills).  80 keeps two 384-thread
// blocks per SM (the 3D matrix array's shape); wider column and window counts get 128.
template <int NC, int KE>
__global__ void __maxnreg__(NC * KE >= 16 ? 128 : 80) fwd_gen_kernel(const FwdArgs a) {
    fwd_dense_body<NC, KE, true>(a);
}

// 3D setups read their (stored or streamed) table through the same register ceilings: on the 3D
// matrix array the forward then runs 4 % faster than under the 512-thread bound (187 vs 195 ms).
// 2D setups take them where the ceiling is 128 (wide column and window counts): 2d-batched FP32
// forward 891 -> 875 ms; narrower 2D shapes keep the 512-thread bound.
template <int NC, int KE>
__global__ void __maxnreg__(NC * KE >= 16 ? 128 : 80) fwd_dense3_kernel(const FwdArgs a) {
    fwd_dense_body<NC, KE, false>(a);
}

// G[s][b][e] = sum over line groups of the forward partials (skipped when the compacted forward ran)
// G = sum over the partials part[k][n] in order k = 0, 1, ...: `groups` of them written by the
// dense kernels, or `sparse_groups` by the compacted forward when the device chose it (occ_sel)
__global__ void reduce_groups_kernel(const float2* __restrict__ part, int groups, int64_t n, float2* __restrict__ G,
                                     const int* occ_sel = nullptr, int sparse_groups = 0) {
    if (occ_sel && *occ_sel != 0) groups = sparse_groups;
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        float2 s = make_float2(0.f, 0.f);
        for (int k = 0; k < groups; ++k) {
            const float2 v = part[k * n + i];
            s.x += v.x;
            s.y += v.y;
        }
        G[i] = s;
    }
}

// u[b][row] = sum_a pref[mix, fl, a] * G[slot][b][act[a]]  (one warp per (row, b))
struct MixArgs {
    const float2* __restrict__ G;
    const int* __restrict__ row_slot;
    const int* __restrict__ row_mix;
    const int* __restrict__ row_fl;
    const int* __restrict__ mix_nact;
    const int* __restrict__ mix_nf;
    const int64_t* __restrict__ mix_pref_off;
    const int* __restrict__ mix_act_off;
    const int* __restrict__ act;
    const float2* __restrict__ pref;
    int64_t n_obs;
    int B, E;
    float2* __restrict__ u;
    int64_t ldu;
};

__global__ void mix_kernel(const MixArgs a) {
    const int64_t wid = (blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (wid >= a.n_obs * a.B) return;
    const int64_t row = wid % a.n_obs;
    const int b = static_cast<int>(wid / a.n_obs);
    const int m = a.row_mix[row], fl = a.row_fl[row], s = a.row_slot[row];
    const int nact = a.mix_nact[m], nf = a.mix_nf[m];
    const float2* pr = a.pref + a.mix_pref_off[m] + fl;
    const int* ac = a.act + a.mix_act_off[m];
    const float2* Gs = a.G + (static_cast<int64_t>(s) * a.B + b) * a.E;
    float2 acc = make_float2(0.f, 0.f);
    for (int k = lane; k < nact; k += 32) cmac(acc, pr[static_cast<int64_t>(k) * nf], Gs[ac[k]]);
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        acc.x += __shfl_down_sync(0xffffffffu, acc.x, off);
        acc.y += __shfl_down_sync(0xffffffffu, acc.y, off);
    }
    if (lane == 0) a.u[b * a.ldu + row] = acc;
}

// V[s][b][e] = sum_{rows of s} conj(pref[mix, fl, pos(e)]) * u[b][row]
struct UnmixArgs {
    const float2* __restrict__ u;
    int64_t ldu;
    const int* __restrict__ slot_row_ptr;
    const int* __restrict__ slot_rows;
    const int* __restrict__ row_mix;
    const int* __restrict__ row_fl;
    const int* __restrict__ mix_nf;
    const int64_t* __restrict__ mix_pref_off;
    const int* __restrict__ pos;
    const float2* __restrict__ pref;
    int S, B, E;
    float2* __restrict__ V;
};

__global__ void unmix_kernel(const UnmixArgs a) {
    const int64_t n = static_cast<int64_t>(a.S) * a.B * a.E;
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const int e = static_cast<int>(i % a.E);
        const int64_t sb = i / a.E;
        const int b = static_cast<int>(sb % a.B);
        const int s = static_cast<int>(sb / a.B);
        float2 acc = make_float2(0.f, 0.f);
        for (int k = a.slot_row_ptr[s]; k < a.slot_row_ptr[s + 1]; ++k) {
            const int row = a.slot_rows[k];
            const int m = a.row_mix[row];
            const int ps = a.pos[static_cast<int64_t>(m) * a.E + e];
            if (ps >= 0) {
                const float2 p = a.pref[a.mix_pref_off[m] + a.row_fl[row] + static_cast<int64_t>(ps) * a.mix_nf[m]];
                cmac_conj(acc, p, a.u[b * a.ldu + row]);
            }
        }
        a.V[i] = acc;
    }
}

// ---------------------------------------------------------------------------
// Slot-tiled mixing for batched applies (B >= 8 objects, E <= 256 elements).
// Per slot s the mixing is a small complex product: u[rows of s][b] = P_s G[s]
// with P_s[row][e] = pref[mix, f_row, pos(e)] (0 where e is not active), and
// the unmixing its conjugate transpose V[s] = P_s^H u[rows of s].  A block
// takes one slot and up to 32 objects: it stages G[s] (forward) or the slot's
// rows of u (adjoint) and P_s in chunks of 32 rows in shared memory, lanes run
// over objects, and every sum runs in a fixed order.
// ---------------------------------------------------------------------------
constexpr int kMixBC = 32;   // objects per block
constexpr int kMixRC = 32;   // rows of P_s per chunk
constexpr int kMixEMax = 256;

struct MixTileArgs {
    const int* __restrict__ slot_row_ptr;
    const int* __restrict__ slot_rows;
    const int* __restrict__ row_mix;
    const int* __restrict__ row_fl;
    const int* __restrict__ mix_nact;
    const int* __restrict__ mix_nf;
    const int* __restrict__ mix_act_off;
    const int64_t* __restrict__ mix_pref_off;
    const int* __restrict__ act;
    const float2* __restrict__ pref;
    int B, E;
    const float2* __restrict__ G;  // forward input [S][B][E]
    float2* __restrict__ u;        // forward output, column b at b * ldu
    const float2* __restrict__ uin;  // adjoint input
    int64_t ldu;
    float2* __restrict__ V;        // adjoint output [S][B][E]
};

// P_s rows r0 .. r0+nk-1 of slot s into sP[k][e] (dense, zero-filled); sRow[k] = row index
__device__ void stage_prefactors(const MixTileArgs& a, int rbeg, int r0, int nk, float2* sP, int* sRow) {
    for (int i = threadIdx.x; i < nk * a.E; i += blockDim.x) sP[i] = make_float2(0.f, 0.f);
    if (threadIdx.x < nk) sRow[threadIdx.x] = a.slot_rows[rbeg + r0 + threadIdx.x];
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    for (int k = warp; k < nk; k += nw) {
        const int row = sRow[k], m = a.row_mix[row], fl = a.row_fl[row];
        const int nact = a.mix_nact[m], nf = a.mix_nf[m];
        const float2* pr = a.pref + a.mix_pref_off[m] + fl;
        const int* ac = a.act + a.mix_act_off[m];
        for (int ia = lane; ia < nact; ia += 32) sP[k * a.E + ac[ia]] = pr[static_cast<int64_t>(ia) * nf];
    }
    __syncthreads();
}

__global__ void __launch_bounds__(256) mix_tile_kernel(const MixTileArgs a) {
    extern __shared__ float4 smem_m4[];
    float2* sG = reinterpret_cast<float2*>(smem_m4);         // [E][kMixBC + 1]
    float2* sP = sG + a.E * (kMixBC + 1);                    // [kMixRC][E]
    __shared__ int sRow[kMixRC];
    const int s = blockIdx.x, b0 = blockIdx.y * kMixBC, nb = min(kMixBC, a.B - b0);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    for (int i = threadIdx.x; i < nb * a.E; i += blockDim.x) {
        const int bl = i / a.E, e = i - bl * a.E;
        sG[e * (kMixBC + 1) + bl] = a.G[(static_cast<int64_t>(s) * a.B + b0 + bl) * a.E + e];
    }
    const int rbeg = a.slot_row_ptr[s], nrows = a.slot_row_ptr[s + 1] - rbeg;
    for (int r0 = 0; r0 < nrows; r0 += kMixRC) {
        const int nk = min(kMixRC, nrows - r0);
        __syncthreads();  // previous chunk's readers are done (and sG is complete)
        stage_prefactors(a, rbeg, r0, nk, sP, sRow);
        for (int k = warp; k < nk; k += nw) {
            const float2* pk = sP + k * a.E;
            float2 acc = make_float2(0.f, 0.f);
            for (int e = 0; e < a.E; ++e) cmac(acc, pk[e], sG[e * (kMixBC + 1) + lane]);
            if (lane < nb) a.u[static_cast<int64_t>(b0 + lane) * a.ldu + sRow[k]] = acc;
        }
    }
}

__global__ void __launch_bounds__(256) unmix_tile_kernel(const MixTileArgs a) {
    extern __shared__ float4 smem_m4[];
    float2* sP = reinterpret_cast<float2*>(smem_m4);          // [kMixRC][E]; at the end [kMixBC][E + 1]
    float2* sU = sP + (kMixBC * (a.E + 1) > kMixRC * a.E ? kMixBC * (a.E + 1) : kMixRC * a.E);  // [kMixRC][kMixBC]
    __shared__ int sRow[kMixRC];
    const int s = blockIdx.x, b0 = blockIdx.y * kMixBC, nb = min(kMixBC, a.B - b0);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    constexpr int EJ = kMixEMax / 8;  // elements per warp (8 warps)
    float2 acc[EJ];
#pragma unroll
    for (int j = 0; j < EJ; ++j) acc[j] = make_float2(0.f, 0.f);
    const int rbeg = a.slot_row_ptr[s], nrows = a.slot_row_ptr[s + 1] - rbeg;
    for (int r0 = 0; r0 < nrows; r0 += kMixRC) {
        const int nk = min(kMixRC, nrows - r0);
        __syncthreads();
        stage_prefactors(a, rbeg, r0, nk, sP, sRow);
        for (int i = threadIdx.x; i < nk * kMixBC; i += blockDim.x) {
            const int k = i / kMixBC, bl = i - k * kMixBC;
            sU[i] = bl < nb ? a.uin[static_cast<int64_t>(b0 + bl) * a.ldu + sRow[k]] : make_float2(0.f, 0.f);
        }
        __syncthreads();
        for (int k = 0; k < nk; ++k) {
            const float2 uv = sU[k * kMixBC + lane];
            const float2* pk = sP + k * a.E;
#pragma unroll
            for (int j = 0; j < EJ; ++j) {
                const int e = warp + nw * j;
                if (e < a.E) cmac_conj(acc[j], pk[e], uv);
            }
        }
    }
    // transpose through shared memory so that V is written along e
    __syncthreads();
    float2* sV = sP;  // [kMixBC][E + 1]
#pragma unroll
    for (int j = 0; j < EJ; ++j) {
        const int e = warp + nw * j;
        if (e < a.E) sV[lane * (a.E + 1) + e] = acc[j];
    }
    __syncthreads();
    for (int i = threadIdx.x; i < nb * a.E; i += blockDim.x) {
        const int bl = i / a.E, e = i - bl * a.E;
        a.V[(static_cast<int64_t>(s) * a.B + b0 + bl) * a.E + e] = sV[bl * (a.E + 1) + e];
    }
}

size_t mix_tile_smem(int E) { return sizeof(float2) * (static_cast<size_t>(E) * (kMixBC + 1) + kMixRC * E); }
size_t unmix_tile_smem(int E) {
    return sizeof(float2) * (std::max<size_t>(static_cast<size_t>(kMixBC) * (E + 1), static_cast<size_t>(kMixRC) * E) +
                             kMixRC * kMixBC);
}

MixTileArgs mix_tile_args(const Plan* p, int B) {
    MixTileArgs m;
    m.slot_row_ptr = p->slot_row_ptr; m.slot_rows = p->slot_rows; m.row_mix = p->row_mix; m.row_fl = p->row_fl;
    m.mix_nact = p->mix_nact; m.mix_nf = p->mix_nf; m.mix_act_off = p->mix_act_off; m.mix_pref_off = p->mix_pref_off;
    m.act = p->act; m.pref = p->pref; m.B = B; m.E = p->E;
    m.G = nullptr; m.u = nullptr; m.uin = nullptr; m.ldu = 0; m.V = nullptr;
    return m;
}

// the slot-tiled kernels serve batches of 8 or more objects on arrays of up to 256 elements
bool use_mix_tile(const Plan* p, int B) { return B >= 8 && p->E <= kMixEMax; }

// ---------------------------------------------------------------------------
// dense adjoint: block = (grid line, frequency chunk, object)
// ---------------------------------------------------------------------------
struct AdjArgs {
    LineGeom g;
    const float2* __restrict__ table;  // stored table (frequencies from tab_f0 on), or null when generated (gen)
    TableGen gen;
    int fc_base, tab_f0;               // frequency chunk of blockIdx.y = 0; first frequency the table holds
    const float2* __restrict__ p_in;
    const float2* __restrict__ V;   // [S][B][E]
    const int* __restrict__ f_slot_ptr;
    const int* __restrict__ f_slot_list;
    int fchunk;
    int n_jg, nseg_e, Es, ntask;
    int lj, nsub;                   // lanes per j group; lane groups splitting the element range
    int B;
    int eyb;                        // element rows (ey) staged per synchronisation
    float2* __restrict__ part;      // [nfc][B][P]
};

template <int NC, int KJ, bool GEN>
__device__ __forceinline__ void adj_dense_body(const AdjArgs& a) {
    extern __shared__ float4 smem_f4[];
    const LineGeom& g = a.g;
    const int EB = a.eyb;
    // V rows padded to an odd number of columns: lane groups reading elements espan apart then hit
    // different banks
    constexpr int NCP = NC | 1;
    constexpr bool SKEW = (KJ % 2) == 0;
    float2* sA = reinterpret_cast<float2*>(smem_f4);  // [EB][ppx * Ni] bands of EB element rows (skewed)
    float2* sV = sA + band_capacity(static_cast<size_t>(EB) * g.ppx * g.Ni);  // [EB][Ex][NCP]
    float2* sR = sV + EB * g.Ex * NCP;               // [Nx]
    __shared__ int sSlot[NC];

    const int line = blockIdx.x;
    const int iy = line % g.Ny, z = line / g.Ny;
    const int fc = a.fc_base + blockIdx.y, b = blockIdx.z;
    const int64_t pt0 = (static_cast<int64_t>(z) * g.Ny + iy) * g.Nx;

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const bool task_on = warp < a.ntask;
    int r = 0, jg = 0, es = 0;
    if (task_on) {
        r = warp % g.ppx;
        const int rest = warp / g.ppx;
        jg = rest % a.n_jg;
        es = rest / a.n_jg;
    }
    // lane = (j group jl, element sub-range sub); lanes >= lj * nsub stay idle
    const int jl = lane % a.lj, sub = lane / a.lj;
    const int j0 = (jg * a.lj + jl) * KJ;
    const int Nj_r = (r < g.Nx) ? (g.Nx - r + g.ppx - 1) / g.ppx : 0;
    const int elo0 = es * a.Es, ehi0 = min(elo0 + a.Es, g.Ex);
    const int espan = (max(ehi0 - elo0, 0) + a.nsub - 1) / a.nsub;
    const int elo = elo0 + sub * espan, ehi = min(elo + espan, ehi0);
    const bool lane_on = task_on && sub < a.nsub && (j0 < Nj_r) && (elo < ehi);

    float2 gacc[KJ];
#pragma unroll
    for (int t = 0; t < KJ; ++t) gacc[t] = make_float2(0.f, 0.f);

    const int f_lo = fc * a.fchunk, f_hi = min(f_lo + a.fchunk, g.F);
    for (int f = f_lo; f < f_hi; ++f) {
        const int s0 = a.f_slot_ptr[f];
        const int ns = a.f_slot_ptr[f + 1] - s0;
        for (int c0 = 0; c0 < ns; c0 += NC) {
            const int nc = min(NC, ns - c0);
            float2 Z[KJ][NC];
#pragma unroll
            for (int t = 0; t < KJ; ++t)
#pragma unroll
                for (int c = 0; c < NC; ++c) Z[t][c] = make_float2(0.f, 0.f);
            // EB element rows per synchronisation: their table rows and V entries are staged together
            for (int ey0 = 0; ey0 < g.Ey; ey0 += EB) {
                const int neb = min(EB, g.Ey - ey0);
                __syncthreads();
                if (threadIdx.x < NC) sSlot[threadIdx.x] = (threadIdx.x < nc) ? a.f_slot_list[s0 + c0 + threadIdx.x] : 0;
                for (int k = 0; k < neb; ++k) {
                    const int oy = iy - (ey0 + k) * g.ppy + (g.Ey - 1) * g.ppy;
                    stage_row_at<GEN, SKEW>(sA, k * g.ppx * g.Ni, a.table, a.tab_f0, a.gen, f, z, oy, g);
                }
                __syncthreads();
                for (int idx = threadIdx.x; idx < neb * NC * g.Ex; idx += blockDim.x) {
                    const int k = idx / (NC * g.Ex), rem = idx - k * (NC * g.Ex);
                    const int c = rem / g.Ex, ex = rem - c * g.Ex;
                    sV[(k * g.Ex + ex) * NCP + c] = (c < nc)
                        ? __ldg(a.V + (static_cast<int64_t>(sSlot[c]) * a.B + b) * g.E + ex + g.Ex * (ey0 + k))
                        : make_float2(0.f, 0.f);
                }
                __syncthreads();
                if (lane_on) {
                    for (int k = 0; k < neb; ++k) {
                        const int a0 = k * g.ppx * g.Ni + r * g.Ni + kPad;  // band r of row k
                        const float2* sVk = sV + k * g.Ex * NCP;
                        int base = a0 + j0 - elo + g.Ex - 1;
                        float2 win[KJ];
#pragma unroll
                        for (int t = 0; t < KJ; ++t) win[t] = sA[band_at<SKEW>(base + t)];
                        for (int e = elo; e < ehi; ++e) {
                            const float2* vx = sVk + e * NCP;
                            float2 v[NC];
#pragma unroll
                            for (int c = 0; c < NC; ++c) v[c] = vx[c];
#pragma unroll
                            for (int t = 0; t < KJ; ++t)
#pragma unroll
                                for (int c = 0; c < NC; ++c) cmac_conj(Z[t][c], win[t], v[c]);
#pragma unroll
                            for (int t = KJ - 1; t > 0; --t) win[t] = win[t - 1];
                            --base;
                            win[0] = sA[band_at<SKEW>(base)];
                        }
                    }
                }
            }
            if (lane_on) {
#pragma unroll
                for (int t = 0; t < KJ; ++t) {
                    const int x = r + g.ppx * (j0 + t);
                    if (x < g.Nx) {
#pragma unroll
                        for (int c = 0; c < NC; ++c) {
                            if (c < nc) {
                                const float2 p = __ldg(a.p_in + static_cast<int64_t>(sSlot[c]) * g.P + pt0 + x);
                                cmac_conj(gacc[t], p, Z[t][c]);
                            }
                        }
                    }
                }
            }
        }
    }

    // deterministic reduction over element segments
    __syncthreads();
    for (int idx = threadIdx.x; idx < g.Nx; idx += blockDim.x) sR[idx] = make_float2(0.f, 0.f);
    __syncthreads();
    for (int w = 0; w < a.ntask; ++w) {
        if (warp == w) {
            for (int sb = 0; sb < a.nsub; ++sb) {  // lane groups of one warp add to the same points in turn
                if (sub == sb && lane_on) {
#pragma unroll
                    for (int t = 0; t < KJ; ++t) {
                        const int x = r + g.ppx * (j0 + t);
                        if (x < g.Nx) {
                            float2 v = sR[x];
                            v.x += gacc[t].x;
                            v.y += gacc[t].y;
                            sR[x] = v;
                        }
                    }
                }
                __syncwarp();
            }
        }
        __syncthreads();
    }
    float2* out = a.part + (static_cast<int64_t>(fc) * a.B + b) * g.P + pt0;
    for (int x = threadIdx.x; x < g.Nx; x += blockDim.x) out[x] = sR[x];
}

template <int NC, int KJ>
__global__ void __launch_bounds__(512) adj_dense_kernel(const AdjArgs a) {
    adj_dense_body<NC, KJ, false>(a);
}

// Generated table (see fwd_gen_kernel): 112 registers keep three 192-thread blocks per SM.
template <int NC, int KJ>
__global__ void __maxnreg__(NC * KJ >= 24 ? 128 : 112) adj_gen_kernel(const AdjArgs a) {
    adj_dense_body<NC, KJ, true>(a);
}

// 3D setups with a stored or streamed table (see fwd_dense3_kernel) and 2D setups where the ceiling is
// 128 (2d-batched FP32 adjoint 802 -> 713 ms, 2d-gradient 14.4 -> 13.2 ms; the single-wave 2d-plain
// adjoint is slower under a ceiling, 0.28 -> 0.36 ms, and keeps the bound).  The 3D windows of fewer
// than 24 accumulators take the lowest ceiling without spills: 64 registers below 16 accumulators (5
// blocks of 192 threads per SM), else 80 (4 blocks); the 3D array's <5,3> adjoint went from 195.2 ms
// (112 registers, 3 blocks) to 181.4 ms.
template <int NC, int KJ>
__global__ void __maxnreg__(NC * KJ >= 24 ? 128 : (NC * KJ >= 16 ? 80 : 64)) adj_dense3_kernel(const AdjArgs a) {
    adj_dense_body<NC, KJ, false>(a);
}

// gamma_hat[b][p] = sum over frequency chunks
__global__ void reduce_fchunks_kernel(const float2* __restrict__ part, int nfc, int B, int64_t P,
                                      float2* __restrict__ out, int64_t ldo) {
    const int64_t n = static_cast<int64_t>(B) * P;
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        float2 s = make_float2(0.f, 0.f);
        for (int k = 0; k < nfc; ++k) {
            const float2 v = part[k * n + i];
            s.x += v.x;
            s.y += v.y;
        }
        const int64_t b = i / P, p = i - b * P;
        out[b * ldo + p] = s;
    }
}

// Proximal-gradient (ISTA) step fused into the adjoint's final reduction:
//   v = gamma - step * sum_k part[k],   gamma <- v * max(0, 1 - step*lambda_b / |v|)
// (complex soft threshold, the proximal map of step*lambda_b*||gamma||_1).  Each
// element is read and written by one thread, so the update is in place.
__global__ void ista_reduce_kernel(const float2* __restrict__ part, int nfc, int B, int64_t P, float2* gamma, int64_t ldg,
                                   float step, const float* __restrict__ lambda) {
    const int64_t n = static_cast<int64_t>(B) * P;
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        float2 s = make_float2(0.f, 0.f);
        for (int k = 0; k < nfc; ++k) {
            const float2 v = part[k * n + i];
            s.x += v.x;
            s.y += v.y;
        }
        const int64_t b = i / P, pt = i - b * P;
        float2 g = gamma[b * ldg + pt];
        g.x = fmaf(-step, s.x, g.x);
        g.y = fmaf(-step, s.y, g.y);
        const float tau = step * lambda[b];
        const float mag = sqrtf(g.x * g.x + g.y * g.y);
        const float scale = (mag > tau) ? 1.f - tau / mag : 0.f;
        gamma[b * ldg + pt] = make_float2(g.x * scale, g.y * scale);
    }
}

// r = u_pred - u_meas in place; per-block partial sums of 0.5*|r|^2
constexpr int kLossBlocks = 128;

__global__ void residual_kernel(float2* __restrict__ r, int64_t ldr, const float2* __restrict__ um, int64_t ldu,
                                int64_t n_obs, float* __restrict__ loss_part) {
    const int b = blockIdx.y;
    float s = 0.f;
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n_obs;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        float2 v = r[b * ldr + i];
        const float2 w = um[b * ldu + i];
        v.x -= w.x;
        v.y -= w.y;
        r[b * ldr + i] = v;
        s = fmaf(v.x, v.x, s);
        s = fmaf(v.y, v.y, s);
    }
    __shared__ float red[32];
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) s += __shfl_down_sync(0xffffffffu, s, off);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x < 32) {
        s = (threadIdx.x < (blockDim.x >> 5)) ? red[threadIdx.x] : 0.f;
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) s += __shfl_down_sync(0xffffffffu, s, off);
        if (threadIdx.x == 0) loss_part[b * gridDim.x + blockIdx.x] = s;
    }
}

__global__ void loss_final_kernel(const float* __restrict__ part, int nblk, int B, float* __restrict__ loss) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= B) return;
    float s = 0.f;
    for (int k = 0; k < nblk; ++k) s += part[b * nblk + k];
    loss[b] = 0.5f * s;
}

// ---------------------------------------------------------------------------
// launch helpers
// ---------------------------------------------------------------------------
LineGeom geom_of(const Plan* p) {
    LineGeom g;
    g.Nx = p->Nx; g.Ny = p->Ny; g.Nz = p->Nz; g.Ex = p->Ex; g.Ey = p->Ey;
    g.ppx = p->ppx; g.ppy = p->ppy; g.Nox = p->Nox; g.Noy = p->Noy;
    g.P = p->P; g.E = p->E; g.S = p->S; g.F = p->F; g.Ni = p->Ni; g.Nj_max = p->Nj_max;
    return g;
}

// element rows (ey) whose table rows the FP32 adjoint stages together: all of them up to 8
// (one synchronisation per 8 rows instead of three per row on the 3D matrix array)
int adj_eyb(const Plan* p) { return std::min(p->Ey, 8); }

int pick_nc(int slots) {
    if (slots <= 1) return 1;
    if (slots <= 2) return 2;
    if (slots <= 4) return 4;
    if (slots <= 5) return 5;  // the 3D workload's 5 waves: 6 would waste 1 of 6 columns, 8 3 of 8
    if (slots <= 6) return 6;
    if (slots <= 8) return 8;
    if (slots <= 12) return 12;
    return 16;
}

constexpr int fwd_ke(int nc) { return nc >= 16 ? 2 : 4; }
constexpr int adj_kj(int nc) { return nc >= 12 ? 2 : 4; }

// Adjoint register-window length (points per lane) from k0 down to 1: the one that keeps most
// of a warp's lanes and their window slots busy over the n points of a residue, where the lanes
// form floor(32 / lj) groups of lj = ceil(n / k) lanes that split the element range (ties: the
// longer window).  The 2D arrays (128 points per residue) keep k0 = 4; the 3D matrix array
// (43 points per residue) takes 3: 2 groups of 15 lanes, 30 of 32 busy.
int adj_window(int n, int k0) {
    auto util = [n](int k) {
        const int lj = std::max(1, std::min(32, (n + k - 1) / k));
        const int groups = (n + lj * k - 1) / (lj * k);
        return static_cast<double>(n) / (static_cast<double>(groups) * lj * k) * (lj * (32 / lj)) / 32.0;
    };
    int best = k0;
    for (int k = k0 - 1; k >= 1; --k)
        if (util(k) > util(best) + 1e-9) best = k;
    return best;
}

struct FwdShape { int le, n_eg, nseg, Js, ntask, threads; };
struct AdjShape { int lj, nsub, n_jg, nseg_e, Es, ntask, threads; };

FwdShape fwd_shape(const Plan* p, int ke) {
    FwdShape s;
    s.le = 32;  // lanes per element group: the smallest power of two >= Ex / ke, at most 32
    while (s.le > 1 && (s.le / 2) * ke >= p->Ex) s.le /= 2;
    s.n_eg = (p->Ex + s.le * ke - 1) / (s.le * ke);
    const int base = p->ppx * s.n_eg * fwd_rows_per_block(p->Ey);
    s.nseg = std::max(1, 8 / base);
    s.nseg = std::min(s.nseg, std::max(1, p->Nj_max));
    s.Js = (p->Nj_max + s.nseg - 1) / s.nseg;
    s.ntask = base * s.nseg;
    s.threads = 32 * s.ntask;
    return s;
}

AdjShape adj_shape(const Plan* p, int kj) {
    AdjShape s;
    s.lj = std::max(1, std::min(32, (p->Nj_max + kj - 1) / kj));  // lanes per j group
    s.nsub = 32 / s.lj;
    s.n_jg = (p->Nj_max + s.lj * kj - 1) / (s.lj * kj);
    const int base = p->ppx * s.n_jg;
    s.nseg_e = std::max(1, 8 / base);
    s.nseg_e = std::min(s.nseg_e, p->Ex);
    s.Es = (p->Ex + s.nseg_e - 1) / s.nseg_e;
    s.ntask = base * s.nseg_e;
    s.threads = 32 * s.ntask;
    return s;
}

// Streamed table: the rows of frequencies f0 .. f0+nf-1 generated into the plan's chunk buffer
// (layout [nf][Nz][Noy][Nox], like the stored table).  Block = rows, thread = lateral offset.
__global__ void __launch_bounds__(256) table_chunk_kernel(const TableGen t, int f0, int n_rows, int Nz, int Noy,
                                                          float2* __restrict__ out, const int* skip) {
    // a forward's chunk is not needed when the occupancy pass chose the compacted forward, which
    // generates its own entries (uniform over the grid)
    if (skip && *skip != 0) return;
    for (int row = blockIdx.x; row < n_rows; row += gridDim.x) {
        const int oy = row % Noy, rz = row / Noy;
        const GenRow g = gen_row(t, f0 + rz / Nz, rz % Nz, oy);
        float2* o = out + static_cast<int64_t>(row) * t.Nox;
        for (int ox = threadIdx.x; ox < t.Nox; ox += blockDim.x) o[ox] = gen_entry(t, g, ox);
    }
}

cudaError_t stream_table_chunk(const Plan* p, int f0, int nf, cudaStream_t st, const int* skip = nullptr) {
    const int n_rows = nf * p->Nz * p->Noy;
    const int threads = std::min(256, (p->Nox + 31) / 32 * 32);
    table_chunk_kernel<<<std::min(n_rows, 152 * 16), threads, 0, st>>>(p->gen, f0, n_rows, p->Nz, p->Noy, p->stream_buf,
                                                                       skip);
    count_launch();
    return cudaGetLastError();
}

template <int NC, int KE>
cudaError_t launch_fwd_k(const Plan* p, const float2* gamma, int64_t ldg, int B, cudaStream_t st, const int* occ_sel) {
    const FwdShape sh = fwd_shape(p, KE);
    FwdArgs a;
    a.g = geom_of(p);
    a.table = p->table; a.gen = p->gen; a.f_base = 0; a.tab_f0 = 0;
    a.p_in = p->p_in; a.gamma = gamma; a.ldg = ldg;
    a.f_slot_ptr = p->f_slot_ptr; a.f_slot_list = p->f_slot_list;
    a.lines_per_group = p->fwd_lines_per_group; a.n_lines = p->Ny * p->Nz;
    a.n_eg = sh.n_eg; a.nseg = sh.nseg; a.Js = sh.Js; a.ntask = sh.ntask; a.le = sh.le;
    a.eyb = fwd_rows_per_block(p->Ey); a.n_eyb = (p->Ey + a.eyb - 1) / a.eyb;
    a.B = B; a.npass = (p->max_slots_per_f + NC - 1) / NC;
    a.part = p->ws_part;
    a.occ_sel = occ_sel;
    const size_t smem = fwd_smem_bytes(p, NC);
    void (*kern)(const FwdArgs) = p->table_mode == CUI_STORAGE_GENERATED ? fwd_gen_kernel<NC, KE>
                                  : p->n_dims == 3 || NC * KE >= 16       ? fwd_dense3_kernel<NC, KE>
                                                                          : fwd_dense_kernel<NC, KE>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
    if (e != cudaSuccess) return e;
    // streamed table: one chunk of frequencies at a time, generated into the chunk buffer and consumed
    // by the stored-table kernel before the next chunk overwrites it (stream order)
    const int fstep = p->table_mode == CUI_STORAGE_STREAMED ? p->stream_nf : p->F;
    for (int f0 = 0; f0 < p->F; f0 += fstep) {
        const int nf = std::min(fstep, p->F - f0);
        if (p->table_mode == CUI_STORAGE_STREAMED) {
            if ((e = stream_table_chunk(p, f0, nf, st, occ_sel)) != cudaSuccess) return e;
            a.table = p->stream_buf; a.f_base = f0; a.tab_f0 = f0;
        }
        kern<<<dim3(p->fwd_groups * a.n_eyb, nf, B * a.npass), sh.threads, smem, st>>>(a);
        count_launch();
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
    }
    return cudaSuccess;
}

template <int NC, int KJ>
cudaError_t launch_adj_k(const Plan* p, int B, cudaStream_t st) {
    const AdjShape sh = adj_shape(p, KJ);
    AdjArgs a;
    a.g = geom_of(p);
    a.table = p->table; a.gen = p->gen; a.fc_base = 0; a.tab_f0 = 0;
    a.p_in = p->p_in; a.V = p->ws_G;
    a.f_slot_ptr = p->f_slot_ptr; a.f_slot_list = p->f_slot_list;
    a.fchunk = p->adj_fchunk;
    a.n_jg = sh.n_jg; a.nseg_e = sh.nseg_e; a.Es = sh.Es; a.ntask = sh.ntask;
    a.lj = sh.lj; a.nsub = sh.nsub;
    a.B = B; a.eyb = adj_eyb(p); a.part = p->ws_part;
    const size_t smem = adj_smem_bytes(p, NC);
    void (*kern)(const AdjArgs) = p->table_mode == CUI_STORAGE_GENERATED ? adj_gen_kernel<NC, KJ>
                                  : p->n_dims == 3 || NC * KJ >= 24       ? adj_dense3_kernel<NC, KJ>
                                                                          : adj_dense_kernel<NC, KJ>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
    if (e != cudaSuccess) return e;
    if ((e = timing_begin(const_cast<Plan*>(p), 1, st)) != cudaSuccess) return e;
    if (p->table_mode == CUI_STORAGE_STREAMED) {
        // a streamed plan's frequency chunks are the adjoint's (adj_fchunk == stream_nf): chunk c is
        // generated, then contracted by the blocks of frequency chunk c
        for (int c = 0; c < p->adj_nfc; ++c) {
            const int f0 = c * p->adj_fchunk;
            if ((e = stream_table_chunk(p, f0, std::min(p->adj_fchunk, p->F - f0), st)) != cudaSuccess) return e;
            a.table = p->stream_buf; a.fc_base = c; a.tab_f0 = f0;
            kern<<<dim3(p->Ny * p->Nz, 1, B), sh.threads, smem, st>>>(a);
            count_launch();
            if ((e = cudaGetLastError()) != cudaSuccess) return e;
        }
    } else {
        kern<<<dim3(p->Ny * p->Nz, p->adj_nfc, B), sh.threads, smem, st>>>(a);
        count_launch();
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
    }
    return timing_end(const_cast<Plan*>(p), st);
}

// Forward window: the native one on rows of 32 x k0 elements or more; narrower rows (the 3D
// matrix array's 32, the 64-element arrays) take 2 and split the j range among lane groups, since
// the native window's registers would halve the resident blocks
constexpr int fwd_window(int nc, int ex) { return (ex < 32 * fwd_ke(nc) && fwd_ke(nc) > 2) ? 2 : fwd_ke(nc); }

template <int NC>
cudaError_t launch_fwd(const Plan* p, const float2* gamma, int64_t ldg, int B, cudaStream_t st, const int* occ_sel) {
    if (fwd_window(NC, p->Ex) == 2) return launch_fwd_k<NC, 2>(p, gamma, ldg, B, st, occ_sel);
    return launch_fwd_k<NC, fwd_ke(NC)>(p, gamma, ldg, B, st, occ_sel);
}

template <int NC>
cudaError_t launch_adj(const Plan* p, int B, cudaStream_t st) {
    constexpr int K0 = adj_kj(NC);
    switch (adj_window(p->Nj_max, K0)) {
        case 1: return launch_adj_k<NC, 1>(p, B, st);
        case 2: return launch_adj_k<NC, (K0 > 2 ? 2 : K0)>(p, B, st);
        case 3: return launch_adj_k<NC, (K0 > 3 ? 3 : K0)>(p, B, st);
        default: return launch_adj_k<NC, K0>(p, B, st);
    }
}

int grid_1d(int64_t n, int threads) {
    const int64_t b = (n + threads - 1) / threads;
    return static_cast<int>(std::min<int64_t>(std::max<int64_t>(b, 1), 152 * 32));
}

// ---------------------------------------------------------------------------
// occupancy compaction (FP32 forward): the reference's forward contracts only the grid points
// where some column of gamma is nonzero (operator_born.m:361, combined_quick_gpu.cu:457-499).
// A count / scan / scatter pass lists those points in ascending order and chooses, on the
// device, the compacted forward when they are few (n_occ <= limit) and the dense kernels
// otherwise; the kernel not chosen returns at once, so the choice needs no host round trip.
// ---------------------------------------------------------------------------
constexpr int kOccBlock = 1024;  // points per block of the count and scatter kernels (one per thread)

__device__ __forceinline__ bool occupied(const float2* __restrict__ g, int64_t ldg, int B, int64_t pt) {
    for (int b = 0; b < B; ++b) {
        const float2 v = g[static_cast<int64_t>(b) * ldg + pt];
        if (v.x != 0.f || v.y != 0.f) return true;
    }
    return false;
}

__global__ void __launch_bounds__(kOccBlock) occ_count_kernel(const float2* __restrict__ g, int64_t ldg, int B,
                                                              int64_t P, int* __restrict__ cnt) {
    const int64_t pt = static_cast<int64_t>(blockIdx.x) * kOccBlock + threadIdx.x;
    const int n = __syncthreads_count(pt < P && occupied(g, ldg, B, pt));
    if (threadIdx.x == 0) cnt[blockIdx.x] = n;
}

// one block: exclusive scan of the block counts into offsets; n_occ and the choice after them
__global__ void __launch_bounds__(1024) occ_scan_kernel(int* __restrict__ cnt, int nblk, int64_t limit) {
    __shared__ int warp_sum[32];
    const int tid = threadIdx.x, per = (nblk + 1023) / 1024;
    const int lo = min(nblk, tid * per), hi = min(nblk, lo + per);
    int mine = 0;
    for (int i = lo; i < hi; ++i) mine += cnt[i];
    // inclusive scan of the per-thread sums: warps, then the warp totals
    int v = mine;
    for (int d = 1; d < 32; d <<= 1) {
        const int o = __shfl_up_sync(0xffffffffu, v, d);
        if ((tid & 31) >= d) v += o;
    }
    if ((tid & 31) == 31) warp_sum[tid >> 5] = v;
    __syncthreads();
    if (tid < 32) {
        int w = warp_sum[tid];
        for (int d = 1; d < 32; d <<= 1) {
            const int o = __shfl_up_sync(0xffffffffu, w, d);
            if (tid >= d) w += o;
        }
        warp_sum[tid] = w;
    }
    __syncthreads();
    int run = v - mine + ((tid >> 5) ? warp_sum[(tid >> 5) - 1] : 0);  // exclusive prefix of this thread
    for (int i = lo; i < hi; ++i) {
        const int c = cnt[i];
        cnt[nblk + i] = run;
        run += c;
    }
    if (tid == 1023) {
        const int total = warp_sum[31];
        cnt[2 * nblk] = total;
        cnt[2 * nblk + 1] = (limit > 0 && total <= limit) ? 1 : 0;
    }
}

__global__ void __launch_bounds__(kOccBlock) occ_scatter_kernel(const float2* __restrict__ g, int64_t ldg, int B,
                                                                int64_t P, const int* __restrict__ cnt, int nblk,
                                                                int* __restrict__ idx) {
    if (cnt[2 * nblk + 1] == 0) return;  // the dense kernels run: no list needed
    __shared__ int warp_cnt[32];
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    const int64_t pt = static_cast<int64_t>(blockIdx.x) * kOccBlock + tid;
    const bool occ = pt < P && occupied(g, ldg, B, pt);
    const unsigned ballot = __ballot_sync(0xffffffffu, occ);
    if (lane == 0) warp_cnt[w] = __popc(ballot);
    __syncthreads();
    int before = 0;
    for (int k = 0; k < w; ++k) before += warp_cnt[k];
    if (occ) idx[cnt[nblk + blockIdx.x] + before + __popc(ballot & ((1u << lane) - 1u))] = static_cast<int>(pt);
}

struct SparseFwdArgs {
    LineGeom g;
    const float2* __restrict__ table;  // stored table, or null: entries generated (gen)
    TableGen gen;
    const float2* __restrict__ p_in;
    const float2* __restrict__ gamma;
    int64_t ldg;
    const int* __restrict__ f_slot_ptr;   // [F+1] slots of each frequency (CSR)
    const int* __restrict__ f_slot_list;  // [S]
    int n_sg;                          // slot groups per frequency (gridDim.x = F x n_sg)
    int S;
    const int* __restrict__ idx;
    const int* __restrict__ cnt;       // n_occ at [2 nblk], the choice at [2 nblk + 1]
    int nblk, B;
    int n_chunks;                      // point chunks: gridDim.z
    float2* __restrict__ part;         // [n_chunks][S][B][E] partial sums
};

constexpr int kSpThreads = 256;
constexpr int kSpMaxPerThread = 4;  // elements per thread: arrays of up to 1024 elements
constexpr int kSpSlots = 8;         // most slots of one frequency sharing each table entry

// part[c][s][b][e] = sum over chunk c of the occupied points p of h(f; o(p, e), z_p) p_in[s][p]
// gamma[b][p] for the slots s of frequency f: block per (frequency and group of up to 8 of its
// slots, object, point chunk), thread per element (up to 4).  The chunk's points are staged 256
// at a time with their grid coordinates and q = p_in gamma of every slot of the group; each table
// entry is loaded (or generated) once per point and element and applied to all the group's slots.
// Each staged batch is summed on its own and then added to the chunk's total (two-level
// summation), and the chunks are added in order by reduce_groups_kernel, so no accumulation
// chain runs over all points.
template <bool GEN, int SG>
__global__ void __launch_bounds__(kSpThreads) sparse_fwd_kernel(const SparseFwdArgs a) {
    if (a.cnt[2 * a.nblk + 1] == 0) return;  // the dense kernels run instead
    const LineGeom& g = a.g;
    const int f = blockIdx.x / a.n_sg, sg = blockIdx.x % a.n_sg;
    const int b = blockIdx.y, c = blockIdx.z;
    const int s_lo = a.f_slot_ptr[f] + sg * SG;
    const int ns = min(SG, a.f_slot_ptr[f + 1] - s_lo);
    if (ns <= 0) return;
    const int n_occ = a.cnt[2 * a.nblk];
    const int per = (n_occ + a.n_chunks - 1) / a.n_chunks;
    const int c0 = min(n_occ, c * per), c1 = min(n_occ, c0 + per);
    __shared__ float2 sq[SG][kSpThreads];
    __shared__ int sx[kSpThreads], sy[kSpThreads], sz[kSpThreads];
    __shared__ int slots[SG];
    if (threadIdx.x < SG) slots[threadIdx.x] = threadIdx.x < ns ? a.f_slot_list[s_lo + threadIdx.x] : 0;
    __syncthreads();
    float2 acc[kSpMaxPerThread][SG];
#pragma unroll
    for (int k = 0; k < kSpMaxPerThread; ++k)
#pragma unroll
        for (int j = 0; j < SG; ++j) acc[k][j] = make_float2(0.f, 0.f);
    const float2* gam = a.gamma + static_cast<int64_t>(b) * a.ldg;
    for (int t0 = c0; t0 < c1; t0 += kSpThreads) {
        const int t = t0 + threadIdx.x;
        if (t < c1) {
            const int pt = a.idx[t];
            const float2 gv = gam[pt];
            for (int j = 0; j < ns; ++j) sq[j][threadIdx.x] = cmul(a.p_in[static_cast<int64_t>(slots[j]) * g.P + pt], gv);
            const int x = pt % g.Nx, rest = pt / g.Nx;
            sx[threadIdx.x] = x;
            sy[threadIdx.x] = rest % g.Ny;
            sz[threadIdx.x] = rest / g.Ny;
        }
        __syncthreads();
        const int nt = min(kSpThreads, c1 - t0);
#pragma unroll
        for (int k = 0; k < kSpMaxPerThread; ++k) {
            const int e = threadIdx.x + k * kSpThreads;
            if (e >= g.E) break;
            const int ey = e / g.Ex, ex = e - ey * g.Ex;
            float2 bacc[SG];
#pragma unroll
            for (int j = 0; j < SG; ++j) bacc[j] = make_float2(0.f, 0.f);
            for (int i = 0; i < nt; ++i) {
                const int ox = sx[i] + (g.Ex - 1 - ex) * g.ppx, oy = sy[i] + (g.Ey - 1 - ey) * g.ppy;
                float2 h;
                if constexpr (GEN)
                    h = gen_entry(a.gen, gen_row(a.gen, f, sz[i], oy), ox);
                else
                    h = __ldg(a.table + ((static_cast<int64_t>(f) * g.Nz + sz[i]) * g.Noy + oy) * g.Nox + ox);
#pragma unroll
                for (int j = 0; j < SG; ++j)
                    if (j < ns) cmac(bacc[j], h, sq[j][i]);
            }
#pragma unroll
            for (int j = 0; j < SG; ++j) {
                acc[k][j].x += bacc[j].x;
                acc[k][j].y += bacc[j].y;
            }
        }
        __syncthreads();
    }
    const int64_t n = static_cast<int64_t>(a.S) * a.B * g.E;
#pragma unroll
    for (int k = 0; k < kSpMaxPerThread; ++k) {
        const int e = threadIdx.x + k * kSpThreads;
        if (e >= g.E) break;
#pragma unroll
        for (int j = 0; j < SG; ++j)
            if (j < ns) a.part[c * n + (static_cast<int64_t>(slots[j]) * a.B + b) * g.E + e] = acc[k][j];
    }
}

template <int SG>
void launch_sparse_fwd(bool gen, dim3 grid, const SparseFwdArgs& a, cudaStream_t st) {
    if (gen)
        sparse_fwd_kernel<true, SG><<<grid, kSpThreads, 0, st>>>(a);
    else
        sparse_fwd_kernel<false, SG><<<grid, kSpThreads, 0, st>>>(a);
}

// the occupancy pass and the compacted forward; returns the choice word the dense kernels read and
// the number of partials the compacted forward writes into the plan's partial-sum workspace
cudaError_t launch_occupancy(Plan* p, const float2* gamma, int64_t ldg, int B, cudaStream_t st, const int** sel,
                             int* sparse_groups) {
    *sel = nullptr;
    *sparse_groups = 0;
    if (!p->occ_idx || p->E > kSpThreads * kSpMaxPerThread) return cudaSuccess;
    // default limit: the compacted contraction gathers its table entries (stored) or generates them
    // one by one (streamed, generated), so it pays off below N_points/16 or N_points/32 occupied points
    const int64_t limit = p->occ_limit < 0 ? p->P / (p->table_mode == CUI_STORAGE_STORED ? 16 : 32) : p->occ_limit;
    if (limit == 0) return cudaSuccess;
    // point chunks: about four blocks per SM over (frequency and slot group, object, chunk), as many
    // as the workspace holds
    // slots per group, from {1, 2, 4, 8}: per (point, element) each group loads (about 16
    // instructions) or generates (about 220, cui_gen.cuh) the table entry once and spends about 4 on
    // each of its slots, padding included; the cheapest size wins, ties to the smaller (fewer registers)
    const int ms = std::max(1, p->max_slots_per_f);
    const int entry_cost = p->table_mode == CUI_STORAGE_STORED ? 16 : 220;
    int sgz = 1, best = ms * (entry_cost + 4);
    for (int cand = 2; cand <= kSpSlots; cand *= 2) {
        const int cost = (ms + cand - 1) / cand * (entry_cost + 4 * cand);
        if (cost < best) {
            best = cost;
            sgz = cand;
        }
    }
    const int n_sg = (ms + sgz - 1) / sgz;
    const int64_t fsg = static_cast<int64_t>(p->F) * n_sg * B;
    const int64_t per_group = static_cast<int64_t>(p->S) * B * p->E;
    const int64_t fit = static_cast<int64_t>(p->ws_part_bytes / (sizeof(float2) * std::max<int64_t>(1, per_group)));
    const int64_t want = (4 * 152 + fsg - 1) / fsg;
    const int chunks = static_cast<int>(std::max<int64_t>(1, std::min<int64_t>({want, fit, 64})));
    if (fit < 1) return cudaSuccess;
    occ_count_kernel<<<p->occ_nblk, kOccBlock, 0, st>>>(gamma, ldg, B, p->P, p->occ_cnt);
    occ_scan_kernel<<<1, 1024, 0, st>>>(p->occ_cnt, p->occ_nblk, limit);
    occ_scatter_kernel<<<p->occ_nblk, kOccBlock, 0, st>>>(gamma, ldg, B, p->P, p->occ_cnt, p->occ_nblk, p->occ_idx);
    SparseFwdArgs a;
    a.g = geom_of(p);
    a.table = p->table; a.gen = p->gen; a.p_in = p->p_in; a.gamma = gamma; a.ldg = ldg;
    a.f_slot_ptr = p->f_slot_ptr; a.f_slot_list = p->f_slot_list; a.n_sg = n_sg; a.S = p->S;
    a.idx = p->occ_idx; a.cnt = p->occ_cnt; a.nblk = p->occ_nblk; a.B = B;
    a.n_chunks = chunks; a.part = p->ws_part;
    // entries are generated where the table is not stored (the chunk buffer of a streamed plan is
    // refilled by the dense launch)
    const dim3 grid(static_cast<unsigned>(p->F * n_sg), B, chunks);
    const bool gen = p->table_mode != CUI_STORAGE_STORED;
    switch (sgz) {
        case 1: launch_sparse_fwd<1>(gen, grid, a, st); break;
        case 2: launch_sparse_fwd<2>(gen, grid, a, st); break;
        case 4: launch_sparse_fwd<4>(gen, grid, a, st); break;
        default: launch_sparse_fwd<kSpSlots>(gen, grid, a, st); break;
    }
    count_launch(4);
    *sel = p->occ_cnt + 2 * p->occ_nblk + 1;
    *sparse_groups = chunks;
    return cudaGetLastError();
}

// forward against the folded operator: 64-object GEMM passes, each reduced over its K chunks into u
cudaError_t run_forward_phi(Plan* p, const float2* gamma, int64_t ldg, int B, float2* u, int64_t ldu, cudaStream_t st) {
    for (int b0 = 0; b0 < B; b0 += 64) {
        const int nb = std::min(64, B - b0);
        int nkc = 1;
        cudaError_t e = launch_fwd_phi(p, gamma + static_cast<int64_t>(b0) * ldg, ldg, nb, st, &nkc);
        if (e != cudaSuccess) return e;
        reduce_fchunks_kernel<<<grid_1d(static_cast<int64_t>(nb) * p->n_obs, 256), 256, 0, st>>>(
            p->phi_part, nkc, nb, p->n_obs, u + static_cast<int64_t>(b0) * ldu, ldu);
        count_launch();
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
    }
    return cudaSuccess;
}

cudaError_t run_forward(Plan* p, const float2* gamma, int64_t ldg, int B, float2* u, int64_t ldu, cudaStream_t st) {
    cudaError_t e;
    if (p->precision == 2) return run_forward_phi(p, gamma, ldg, B, u, ldu, st);
    int groups = p->fwd_groups;
    const int* occ_sel = nullptr;
    int sparse_groups = 0;
    if (p->precision == 1 && p->tc2) {
        e = launch_fwd_tc2(p, gamma, ldg, B, st, &groups);
    } else if (p->precision == 1) {
        e = launch_fwd_tc(p, gamma, ldg, B, st);
    } else {
        // the forward's timed region (cui_born_timing_*) covers the occupancy pass, the compacted
        // contraction and the dense launches, whichever of the two contracts
        if ((e = timing_begin(p, 0, st)) != cudaSuccess) return e;
        if ((e = launch_occupancy(p, gamma, ldg, B, st, &occ_sel, &sparse_groups)) != cudaSuccess) return e;
        switch (pick_nc(p->max_slots_per_f)) {
            case 1: e = launch_fwd<1>(p, gamma, ldg, B, st, occ_sel); break;
            case 2: e = launch_fwd<2>(p, gamma, ldg, B, st, occ_sel); break;
            case 4: e = launch_fwd<4>(p, gamma, ldg, B, st, occ_sel); break;
            case 5: e = launch_fwd<5>(p, gamma, ldg, B, st, occ_sel); break;
            case 6: e = launch_fwd<6>(p, gamma, ldg, B, st, occ_sel); break;
            case 8: e = launch_fwd<8>(p, gamma, ldg, B, st, occ_sel); break;
            case 12: e = launch_fwd<12>(p, gamma, ldg, B, st, occ_sel); break;
            default: e = launch_fwd<16>(p, gamma, ldg, B, st, occ_sel); break;
        }
        if (e == cudaSuccess) e = timing_end(p, st);
    }
    if (e != cudaSuccess) return e;
    const int64_t n = static_cast<int64_t>(p->S) * B * p->E;
    reduce_groups_kernel<<<grid_1d(n, 256), 256, 0, st>>>(p->ws_part, groups, n, p->ws_G, occ_sel, sparse_groups);
    count_launch();
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    if (use_mix_tile(p, B)) {
        MixTileArgs t = mix_tile_args(p, B);
        t.G = p->ws_G; t.u = u; t.ldu = ldu;
        const size_t smem = mix_tile_smem(p->E);
        if ((e = cudaFuncSetAttribute(mix_tile_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      static_cast<int>(smem))) != cudaSuccess)
            return e;
        mix_tile_kernel<<<dim3(p->S, (B + kMixBC - 1) / kMixBC), 256, smem, st>>>(t);
        count_launch();
        return cudaGetLastError();
    }
    MixArgs m;
    m.G = p->ws_G; m.row_slot = p->row_slot; m.row_mix = p->row_mix; m.row_fl = p->row_fl;
    m.mix_nact = p->mix_nact; m.mix_nf = p->mix_nf; m.mix_pref_off = p->mix_pref_off; m.mix_act_off = p->mix_act_off;
    m.act = p->act; m.pref = p->pref; m.n_obs = p->n_obs; m.B = B; m.E = p->E; m.u = u; m.ldu = ldu;
    const int64_t warps = p->n_obs * B;
    const int64_t blocks = (warps * 32 + 255) / 256;
    mix_kernel<<<static_cast<unsigned>(blocks), 256, 0, st>>>(m);
    count_launch();
    return cudaGetLastError();
}

struct IstaArgs {
    float step;
    const float* lambda;  // [B] device
};

// final reduction of the adjoint's chunk partials part[nfc][B][P]: plain sum into g, or the ISTA update of g
cudaError_t finish_adjoint(Plan* p, const float2* part, int nfc, int B, float2* g, int64_t ldg, const IstaArgs* ista,
                           cudaStream_t st) {
    const int64_t m = static_cast<int64_t>(B) * p->P;
    if (ista)
        ista_reduce_kernel<<<grid_1d(m, 256), 256, 0, st>>>(part, nfc, B, p->P, g, ldg, ista->step, ista->lambda);
    else
        reduce_fchunks_kernel<<<grid_1d(m, 256), 256, 0, st>>>(part, nfc, B, p->P, g, ldg);
    count_launch();
    return cudaGetLastError();
}

// adjoint against the folded operator: 64-object GEMM passes straight from the observations
// (no unmixing: the mixes are inside the matrix)
cudaError_t run_adjoint_phi(Plan* p, const float2* u, int64_t ldu, int B, float2* g, int64_t ldg, cudaStream_t st,
                            const IstaArgs* ista, HostOut ho = HostOut{}) {
    if (ho.written) *ho.written = ho.host != nullptr && !ista;
    for (int b0 = 0; b0 < B; b0 += 64) {
        const int nb = std::min(64, B - b0);
        int nkc = 1;
        cudaError_t e = launch_adj_phi(p, u + static_cast<int64_t>(b0) * ldu, ldu, nb, st, &nkc,
                                       (ho.host && !ista) ? ho.host + static_cast<int64_t>(b0) * ho.ld : nullptr, ho.ld);
        if (e != cudaSuccess) return e;
        if (nkc == 0) continue;  // the GEMM wrote this pass's gradient to the host itself
        if (ho.written) *ho.written = false;
        IstaArgs is{};
        if (ista) is = IstaArgs{ista->step, ista->lambda + b0};
        if ((e = finish_adjoint(p, p->phi_part, nkc, nb, g + static_cast<int64_t>(b0) * ldg, ldg, ista ? &is : nullptr,
                                st)) != cudaSuccess)
            return e;
    }
    return cudaSuccess;
}

cudaError_t run_adjoint(Plan* p, const float2* u, int64_t ldu, int B, float2* g, int64_t ldg, cudaStream_t st,
                        const IstaArgs* ista = nullptr, HostOut ho = HostOut{}) {
    cudaError_t e;
    if (ho.written) *ho.written = false;
    if (p->precision == 2) return run_adjoint_phi(p, u, ldu, B, g, ldg, st, ista, ho);
    if (use_mix_tile(p, B)) {
        MixTileArgs t = mix_tile_args(p, B);
        t.uin = u; t.ldu = ldu; t.V = p->ws_G;
        const size_t smem = unmix_tile_smem(p->E);
        if ((e = cudaFuncSetAttribute(unmix_tile_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      static_cast<int>(smem))) != cudaSuccess)
            return e;
        unmix_tile_kernel<<<dim3(p->S, (B + kMixBC - 1) / kMixBC), 256, smem, st>>>(t);
    } else {
        UnmixArgs a;
        a.u = u; a.ldu = ldu; a.slot_row_ptr = p->slot_row_ptr; a.slot_rows = p->slot_rows;
        a.row_mix = p->row_mix; a.row_fl = p->row_fl; a.mix_nf = p->mix_nf; a.mix_pref_off = p->mix_pref_off;
        a.pos = p->pos; a.pref = p->pref; a.S = p->S; a.B = B; a.E = p->E; a.V = p->ws_G;
        const int64_t n = static_cast<int64_t>(p->S) * B * p->E;
        unmix_kernel<<<grid_1d(n, 256), 256, 0, st>>>(a);
    }
    count_launch();
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    if (p->precision == 1) {
        int nfc = p->adj_nfc;
        if (p->tc2) {
            if ((e = launch_adj_tc2(p, B, st, &nfc)) != cudaSuccess) return e;
        } else if ((e = launch_adj_tc(p, B, st)) != cudaSuccess) {
            return e;
        }
        return finish_adjoint(p, p->ws_part, nfc, B, g, ldg, ista, st);
    }
    switch (pick_nc(p->max_slots_per_f)) {
        case 1: e = launch_adj<1>(p, B, st); break;
        case 2: e = launch_adj<2>(p, B, st); break;
        case 4: e = launch_adj<4>(p, B, st); break;
        case 5: e = launch_adj<5>(p, B, st); break;
        case 6: e = launch_adj<6>(p, B, st); break;
        case 8: e = launch_adj<8>(p, B, st); break;
        case 12: e = launch_adj<12>(p, B, st); break;
        default: e = launch_adj<16>(p, B, st); break;
    }
    if (e != cudaSuccess) return e;
    return finish_adjoint(p, p->ws_part, p->adj_nfc, B, g, ldg, ista, st);
}

}  // namespace

bool launch_shapes_ok(const Plan* p, std::string* why) {
    const int nc = pick_nc(p->max_slots_per_f);
    const FwdShape f = fwd_shape(p, fwd_window(nc, p->Ex));
    const AdjShape a = adj_shape(p, adj_window(p->Nj_max, adj_kj(nc)));
    if (f.threads > 512 || a.threads > 512) {
        *why = "launch shape exceeds 512 threads (too many points per pitch or elements for these kernels)";
        return false;
    }
    return true;
}

cudaError_t timing_begin(Plan* p, int kind, cudaStream_t st) {
    if (!p->timing) return cudaSuccess;
    while (p->ev_pool.size() < 2 * (p->ev_used + 1)) {
        cudaEvent_t ev;
        cudaError_t e = cudaEventCreate(&ev);
        if (e != cudaSuccess) return e;
        p->ev_pool.push_back(ev);
    }
    if (p->ev_kind.size() < p->ev_used + 1) p->ev_kind.resize(p->ev_used + 1);
    p->ev_kind[p->ev_used] = kind;
    return cudaEventRecord(p->ev_pool[2 * p->ev_used], st);
}

cudaError_t timing_end(Plan* p, cudaStream_t st) {
    if (!p->timing) return cudaSuccess;
    cudaError_t e = cudaEventRecord(p->ev_pool[2 * p->ev_used + 1], st);
    ++p->ev_used;
    return e;
}

void timing_release(Plan* p) {
    for (cudaEvent_t ev : p->ev_pool) cudaEventDestroy(ev);
    p->ev_pool.clear();
    p->ev_kind.clear();
    p->ev_used = 0;
}

size_t fwd_smem_bytes(const Plan* p, int nc) {
    const size_t eb = fwd_rows_per_block(p->Ey);
    return sizeof(float2) * (band_capacity(eb * p->ppx * p->Ni) + static_cast<size_t>(p->Nx) * nc + eb * p->Ex * nc);
}

size_t adj_smem_bytes(const Plan* p, int nc) {
    const size_t eb = adj_eyb(p);
    return sizeof(float2) * (band_capacity(eb * p->ppx * p->Ni) + eb * p->Ex * (nc | 1) + static_cast<size_t>(p->Nx));
}

cui_status forward_device(Plan* p, const float2* gamma, int64_t ldg, int B, float2* u, int64_t ldu, cudaStream_t st) {
    return check_cuda(run_forward(p, gamma, ldg, B, u, ldu, st), "forward");
}

cui_status adjoint_device(Plan* p, const float2* u, int64_t ldu, int B, float2* g, int64_t ldg, cudaStream_t st,
                          HostOut ho) {
    return check_cuda(run_adjoint(p, u, ldu, B, g, ldg, st, nullptr, ho), "adjoint");
}

cui_status vjp_device(Plan* p, const float2* gamma, int64_t ldg, const float2* um, int64_t ldu, int B,
                      float2* grad, int64_t ldgr, float* loss, cudaStream_t st, HostOut ho, cudaEvent_t um_ready) {
    cudaError_t e = run_forward(p, gamma, ldg, B, p->ws_r, p->n_obs, st);
    if (e != cudaSuccess) return check_cuda(e, "vjp forward");
    if (um_ready && (e = cudaStreamWaitEvent(st, um_ready, 0)) != cudaSuccess) return check_cuda(e, "vjp wait");
    residual_kernel<<<dim3(kLossBlocks, B), 256, 0, st>>>(p->ws_r, p->n_obs, um, ldu, p->n_obs, p->ws_loss);
    count_launch();
    if ((e = cudaGetLastError()) != cudaSuccess) return check_cuda(e, "vjp residual");
    if (loss != nullptr) {
        loss_final_kernel<<<(B + 127) / 128, 128, 0, st>>>(p->ws_loss, kLossBlocks, B, loss);
        count_launch();
        if ((e = cudaGetLastError()) != cudaSuccess) return check_cuda(e, "vjp loss");
    }
    return check_cuda(run_adjoint(p, p->ws_r, p->n_obs, B, grad, ldgr, st, nullptr, ho), "vjp adjoint");
}

cui_status lasso_device(Plan* p, float2* gamma, int64_t ldg, const float2* um, int64_t ldu, int B, float step,
                        const float* lambda, int n_iter, float* loss, cudaStream_t st) {
    const IstaArgs ista{step, lambda};
    for (int it = 0; it < n_iter; ++it) {
        cudaError_t e = run_forward(p, gamma, ldg, B, p->ws_r, p->n_obs, st);
        if (e != cudaSuccess) return check_cuda(e, "lasso forward");
        residual_kernel<<<dim3(kLossBlocks, B), 256, 0, st>>>(p->ws_r, p->n_obs, um, ldu, p->n_obs, p->ws_loss);
        count_launch();
        if ((e = cudaGetLastError()) != cudaSuccess) return check_cuda(e, "lasso residual");
        if (loss != nullptr && it == n_iter - 1) {
            loss_final_kernel<<<(B + 127) / 128, 128, 0, st>>>(p->ws_loss, kLossBlocks, B, loss);
            count_launch();
            if ((e = cudaGetLastError()) != cudaSuccess) return check_cuda(e, "lasso loss");
        }
        if ((e = run_adjoint(p, p->ws_r, p->n_obs, B, gamma, ldg, st, &ista)) != cudaSuccess)
            return check_cuda(e, "lasso adjoint");
    }
    return CUI_OK;
}

size_t loss_workspace_floats(int max_objects) { return static_cast<size_t>(kLossBlocks) * max_objects; }

}  // namespace cui

// ---------------------------------------------------------------------------
// Forward apply that allocates nothing.
//
// Some callers cannot call cudaMalloc when they apply the operator: hosts
// that hand their plug-ins a fixed device-memory budget and forbid further
// allocations, and real-time loops that must not enter the allocator (which
// may synchronise the device) between frames.  cui_born_forward_static serves
// them: it reads the plan's tables like cui_born_forward but keeps its partial
// sums in a fixed file-scope device array instead of the plan's workspace, and
// it never allocates.  It runs the FP32 CUDA-core kernels whatever the plan's
// precision.  The array is kStaticScratchBytes large and is held by every GPU
// that loads the library until the process exits.
// ---------------------------------------------------------------------------
namespace cui {
namespace {

constexpr size_t kStaticScratchBytes = size_t(16) << 20;  // 16 MiB per device
static __device__ __align__(256) float2 g_static_scratch[kStaticScratchBytes / sizeof(float2)];

constexpr int kMaxDevices = 64;
std::mutex g_static_mu;
float2* g_static_ptr[kMaxDevices] = {};

// Device address of g_static_scratch on the current device.  The name of the
// array is only a host-side stand-in; kernels need this address.  Looked up
// once per device, on the first call on that device.
cudaError_t static_scratch(int device, float2** out) {
    if (device < 0 || device >= kMaxDevices) return cudaErrorInvalidDevice;  // rejected by the caller first
    std::lock_guard<std::mutex> lock(g_static_mu);
    if (!g_static_ptr[device]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_static_scratch);
        if (e != cudaSuccess) return e;
        g_static_ptr[device] = static_cast<float2*>(p);
    }
    *out = g_static_ptr[device];
    return cudaSuccess;
}

template <int NC, int KE>
cudaError_t launch_fwd_static_k(const Plan* p, const float2* gamma, int64_t ldg, int B, float2* part, int groups,
                                int lines_per_group, cudaStream_t st) {
    const FwdShape sh = fwd_shape(p, KE);
    FwdArgs a;
    a.g = geom_of(p);
    a.table = p->table; a.gen = p->gen; a.f_base = 0; a.tab_f0 = 0;
    a.p_in = p->p_in; a.gamma = gamma; a.ldg = ldg;
    a.f_slot_ptr = p->f_slot_ptr; a.f_slot_list = p->f_slot_list;
    a.lines_per_group = lines_per_group; a.n_lines = p->Ny * p->Nz;
    a.n_eg = sh.n_eg; a.nseg = sh.nseg; a.Js = sh.Js; a.ntask = sh.ntask; a.le = sh.le;
    a.eyb = fwd_rows_per_block(p->Ey); a.n_eyb = (p->Ey + a.eyb - 1) / a.eyb;
    a.B = B; a.npass = (p->max_slots_per_f + NC - 1) / NC;
    a.part = part;
    a.occ_sel = nullptr;
    const size_t smem = fwd_smem_bytes(p, NC);
    // a table that is not stored (generated or streamed) is generated inside the kernel here: the
    // chunk buffer of a streamed plan may be in use by work on another stream
    // the body cui_born_forward launches for this plan (register-capped for 3D plans and wide shapes)
    void (*kern)(const FwdArgs) = p->table_mode != CUI_STORAGE_STORED      ? fwd_gen_kernel<NC, KE>
                                  : p->n_dims == 3 || NC * KE >= 16         ? fwd_dense3_kernel<NC, KE>
                                                                            : fwd_dense_kernel<NC, KE>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
    if (e != cudaSuccess) return e;
    dim3 grid(groups * a.n_eyb, p->F, B * a.npass);
    kern<<<grid, sh.threads, smem, st>>>(a);
    count_launch();
    return cudaGetLastError();
}

// the register window cui_born_forward picks (fwd_window)
template <int NC>
cudaError_t launch_fwd_static(const Plan* p, const float2* gamma, int64_t ldg, int B, float2* part, int groups,
                              int lines_per_group, cudaStream_t st) {
    if (fwd_window(NC, p->Ex) == 2)
        return launch_fwd_static_k<NC, 2>(p, gamma, ldg, B, part, groups, lines_per_group, st);
    return launch_fwd_static_k<NC, fwd_ke(NC)>(p, gamma, ldg, B, part, groups, lines_per_group, st);
}

}  // namespace
}  // namespace cui

extern "C" cui_status cui_born_forward_static(cui_born_plan* plan, const cui_complex32* gamma, int64_t ld_gamma,
                                              int32_t n_objects, cui_complex32* u, int64_t ld_u, void* stream) {
    const cui::NvtxRange nvtx_range("cui_born_forward_static");
    using namespace cui;
    if (!plan) return set_error(CUI_ERR_INVALID_ARG, "plan is NULL");
    Plan* p = &plan->p;
    if (!gamma || !u || n_objects < 1 || ld_gamma < p->P || ld_u < p->n_obs)
        return set_error(CUI_ERR_INVALID_ARG, "invalid arguments to cui_born_forward_static");
    // scratch layout: `groups` partial sums [S][B][E] followed by the reduced element signals
    const size_t slab = sizeof(float2) * static_cast<size_t>(p->S) * n_objects * p->E;
    if (2 * slab > kStaticScratchBytes)
        return set_error(CUI_ERR_INVALID_ARG,
                         "cui_born_forward_static: slots x objects x elements x 16 B exceeds the 16 MiB static "
                         "scratch; use cui_born_forward or fewer objects per call");
    if (p->device < 0 || p->device >= kMaxDevices)
        return set_error(CUI_ERR_INVALID_ARG, "cui_born_forward_static: device index " + std::to_string(p->device) +
                                                  " beyond the " + std::to_string(kMaxDevices) +
                                                  " devices its scratch address table covers");
    // one grid z index per (object, pass over the frequency's slots): the launch limit is 65535
    const int64_t npass = (p->max_slots_per_f + pick_nc(p->max_slots_per_f) - 1) / pick_nc(p->max_slots_per_f);
    if (static_cast<int64_t>(n_objects) * npass > 65535)
        return set_error(CUI_ERR_INVALID_ARG, "cui_born_forward_static: objects x slot passes exceeds 65535 (the "
                                              "launch's z extent); use cui_born_forward or fewer objects per call");
    const int n_lines = p->Ny * p->Nz;
    int groups = static_cast<int>(std::min<size_t>(kStaticScratchBytes / slab - 1, static_cast<size_t>(p->fwd_groups)));
    groups = std::max(1, std::min(groups, n_lines));
    const int lines_per_group = (n_lines + groups - 1) / groups;
    groups = (n_lines + lines_per_group - 1) / lines_per_group;
    const DeviceGuard dev_guard(p->device);
    cudaError_t e = dev_guard.err;
    if (e != cudaSuccess) return check_cuda(e, "cudaSetDevice");
    float2* scratch = nullptr;
    if ((e = static_scratch(p->device, &scratch)) != cudaSuccess) return check_cuda(e, "cudaGetSymbolAddress");
    float2* part = scratch;
    float2* G = scratch + static_cast<size_t>(groups) * p->S * n_objects * p->E;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    switch (pick_nc(p->max_slots_per_f)) {
        case 1: e = launch_fwd_static<1>(p, reinterpret_cast<const float2*>(gamma), ld_gamma, n_objects, part, groups, lines_per_group, st); break;
        case 2: e = launch_fwd_static<2>(p, reinterpret_cast<const float2*>(gamma), ld_gamma, n_objects, part, groups, lines_per_group, st); break;
        case 4: e = launch_fwd_static<4>(p, reinterpret_cast<const float2*>(gamma), ld_gamma, n_objects, part, groups, lines_per_group, st); break;
        case 5: e = launch_fwd_static<5>(p, reinterpret_cast<const float2*>(gamma), ld_gamma, n_objects, part, groups, lines_per_group, st); break;
        case 6: e = launch_fwd_static<6>(p, reinterpret_cast<const float2*>(gamma), ld_gamma, n_objects, part, groups, lines_per_group, st); break;
        case 8: e = launch_fwd_static<8>(p, reinterpret_cast<const float2*>(gamma), ld_gamma, n_objects, part, groups, lines_per_group, st); break;
        case 12: e = launch_fwd_static<12>(p, reinterpret_cast<const float2*>(gamma), ld_gamma, n_objects, part, groups, lines_per_group, st); break;
        default: e = launch_fwd_static<16>(p, reinterpret_cast<const float2*>(gamma), ld_gamma, n_objects, part, groups, lines_per_group, st); break;
    }
    if (e != cudaSuccess) return check_cuda(e, "cui_born_forward_static");
    // every (group, slot, object, element) partial is written by the contraction, so nothing needs clearing
    const int64_t n = static_cast<int64_t>(p->S) * n_objects * p->E;
    reduce_groups_kernel<<<grid_1d(n, 256), 256, 0, st>>>(part, groups, n, G);
    count_launch();
    if ((e = cudaGetLastError()) != cudaSuccess) return check_cuda(e, "cui_born_forward_static reduce");
    MixArgs m;
    m.G = G; m.row_slot = p->row_slot; m.row_mix = p->row_mix; m.row_fl = p->row_fl;
    m.mix_nact = p->mix_nact; m.mix_nf = p->mix_nf; m.mix_pref_off = p->mix_pref_off; m.mix_act_off = p->mix_act_off;
    m.act = p->act; m.pref = p->pref; m.n_obs = p->n_obs; m.B = n_objects; m.E = p->E;
    m.u = reinterpret_cast<float2*>(u); m.ldu = ld_u;
    const int64_t blocks = (p->n_obs * n_objects * 32 + 255) / 256;
    mix_kernel<<<static_cast<unsigned>(blocks), 256, 0, st>>>(m);
    count_launch();
    return check_cuda(cudaGetLastError(), "cui_born_forward_static mix");
}
