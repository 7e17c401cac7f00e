// Received energies in the canonical basis: E[p] = ||Phi e_p||^2, the column
// norms the reference's energy_rx computes before its solvers normalise the
// operator (+scattering/operator_born.m:718-859, +regularization/+options/
// common.m:166-184).
//
// Per observation row (slot s, mix m, local frequency fl) and grid point p:
//   Phi[row, p] = p_in[s, p] * sum_{a in act(m)} pref[m][fl, a] * h(f_s; o(p, act_a), z_p)
// and E[p] = sum_rows |Phi[row, p]|^2 = sum_s |p_in[s, p]|^2 Q_s[p] with
// Q_s[p] = sum_{rows of s} |sum_a pref h|^2.  Slots of one frequency whose rows
// carry identical mixes share Q (the plan's energy groups: waves with a common
// receive mixing), so Q is formed once per group.  A block takes one grid line
// (y, z) and a chunk of groups; per group it stages the table rows of the
// frequency that the line's elements reach (E_y rows of N_ox entries) in shared
// memory (read from the stored table or generated there).  The group
// representative's terms (prefactor, table-row offset, end of row: built at
// plan creation in the order above) pass through shared memory in batches, so
// every thread reads each term as one broadcast and applies it to its PX points
// of the line; Q for the points stays in registers.  Then every slot of the
// group adds |p_in|^2 Q.  Partial sums per group chunk are reduced in a fixed
// order (deterministic).
#include <cuda_runtime.h>

#include <algorithm>

#include "cui_internal.cuh"

namespace cui {
namespace {

constexpr int kEnergyThreads = 128;
constexpr int kEnergyMaxPX = 8;    // points per thread: lateral lines of up to 1024 points
constexpr int kEnergyTerms = 1024; // terms per shared-memory batch (16 KB)

struct EnergyArgs {
    const float2* table;    // [F][Nz][Noy][Nox], or null when generated (gen)
    TableGen gen;
    const float2* p_in;     // [S][P]
    const int* slot_f;
    const int* egroup_ptr;
    const int* egroup_slots;
    const int* term_ptr;    // [n_groups + 1]
    const float4* terms;    // (pref re, pref im, bits of (offset << 1 | row end), 0)
    int Nx, Ny, Nz, Ex, Ey, ppx, ppy, Nox, Noy, n_groups, groups_per_chunk;
    int64_t P;
    float* part;            // [chunks][P]
};

template <bool GEN, int PX>
__global__ void __launch_bounds__(kEnergyThreads) energy_kernel(const EnergyArgs a) {
    extern __shared__ float4 sm_e4[];
    float4* sTerm = sm_e4;                                         // [kEnergyTerms]
    float2* sT = reinterpret_cast<float2*>(sm_e4 + kEnergyTerms);  // [Ey][Nox]
    const int line = blockIdx.x, chunk = blockIdx.y;
    const int iy = line % a.Ny, z = line / a.Ny;
    const int64_t pt0 = static_cast<int64_t>(line) * a.Nx;
    const int g_lo = chunk * a.groups_per_chunk, g_hi = min(g_lo + a.groups_per_chunk, a.n_groups);
    float E[PX];
#pragma unroll
    for (int k = 0; k < PX; ++k) E[k] = 0.f;
    for (int g = g_lo; g < g_hi; ++g) {
        const int gb = a.egroup_ptr[g], ge = a.egroup_ptr[g + 1];
        const int f = a.slot_f[a.egroup_slots[gb]];
        __syncthreads();  // the previous group's rows and terms are consumed
        for (int ey = 0; ey < a.Ey; ++ey) {  // row by row: independent loads (or one generator row each)
            const int oy = iy - ey * a.ppy + (a.Ey - 1) * a.ppy;
            float2* srow = sT + ey * a.Nox;
            if constexpr (GEN) {
                const GenRow r = gen_row(a.gen, f, z, oy);
                for (int ox = threadIdx.x; ox < a.Nox; ox += kEnergyThreads) srow[ox] = gen_entry(a.gen, r, ox);
            } else {
                const float2* row = a.table + ((static_cast<int64_t>(f) * a.Nz + z) * a.Noy + oy) * a.Nox;
#pragma unroll 4
                for (int ox = threadIdx.x; ox < a.Nox; ox += kEnergyThreads) srow[ox] = __ldg(row + ox);
            }
        }
        float Q[PX];
        float2 acc[PX];
#pragma unroll
        for (int k = 0; k < PX; ++k) {
            Q[k] = 0.f;
            acc[k] = make_float2(0.f, 0.f);
        }
        const int t0 = a.term_ptr[g], t1 = a.term_ptr[g + 1];
        for (int b0 = t0; b0 < t1; b0 += kEnergyTerms) {
            const int nb = min(kEnergyTerms, t1 - b0);
            if (b0 > t0) __syncthreads();  // the previous batch is consumed
            for (int i = threadIdx.x; i < nb; i += blockDim.x) sTerm[i] = __ldg(a.terms + b0 + i);
            __syncthreads();  // terms (and, for the first batch, the table rows) staged
            for (int i = 0; i < nb; ++i) {
                const float4 t = sTerm[i];
                const int info = __float_as_int(t.z);
                const float2* trow = sT + (info >> 1);
#pragma unroll
                for (int k = 0; k < PX; ++k) {
                    const int x = threadIdx.x + k * kEnergyThreads;
                    if (x < a.Nx) {
                        const float2 h = trow[x];
                        acc[k].x = fmaf(t.x, h.x, fmaf(-t.y, h.y, acc[k].x));
                        acc[k].y = fmaf(t.x, h.y, fmaf(t.y, h.x, acc[k].y));
                    }
                }
                if (info & 1) {  // end of an observation row: |sum_a pref h|^2
#pragma unroll
                    for (int k = 0; k < PX; ++k) {
                        Q[k] = fmaf(acc[k].x, acc[k].x, fmaf(acc[k].y, acc[k].y, Q[k]));
                        acc[k] = make_float2(0.f, 0.f);
                    }
                }
            }
        }
        for (int i = gb; i < ge; ++i) {  // every slot of the group: |p_in|^2 Q
            const float2* pin = a.p_in + static_cast<int64_t>(a.egroup_slots[i]) * a.P + pt0;
#pragma unroll
            for (int k = 0; k < PX; ++k) {
                const int x = threadIdx.x + k * kEnergyThreads;
                if (x < a.Nx) {
                    const float2 pv = __ldg(pin + x);
                    E[k] = fmaf(pv.x * pv.x + pv.y * pv.y, Q[k], E[k]);
                }
            }
        }
    }
#pragma unroll
    for (int k = 0; k < PX; ++k) {
        const int x = threadIdx.x + k * kEnergyThreads;
        if (x < a.Nx) a.part[static_cast<int64_t>(chunk) * a.P + pt0 + x] = E[k];
    }
}

__global__ void energy_reduce_kernel(const float* __restrict__ part, int chunks, int64_t P, float* __restrict__ out) {
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < P;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        float s = 0.f;
        for (int k = 0; k < chunks; ++k) s += part[k * P + i];
        out[i] = s;
    }
}

}  // namespace
}  // namespace cui

extern "C" cui_status cui_born_energy_rx(cui_born_plan* plan, float* energy, void* stream) {
    const cui::NvtxRange nvtx_range("cui_born_energy_rx");
    using namespace cui;
    if (!plan || !energy) return set_error(CUI_ERR_INVALID_ARG, "NULL argument");
    Plan& p = plan->p;
    if (p.Nx > kEnergyThreads * kEnergyMaxPX)
        return set_error(CUI_ERR_UNSUPPORTED_SETUP, "energy_rx covers lateral grid lines of up to 1024 points");
    const DeviceGuard dev_guard(p.device);
    cudaError_t e = dev_guard.err;
    if (e != cudaSuccess) return check_cuda(e, "cudaSetDevice");
    const int lines = p.Ny * p.Nz;
    const int64_t cap = static_cast<int64_t>(p.ws_part_bytes / (sizeof(float) * static_cast<size_t>(p.P)));
    const int64_t want = (8 * 152 + lines - 1) / lines;
    const int ng = p.n_egroups;
    const int chunks0 = static_cast<int>(std::max<int64_t>(1, std::min<int64_t>({want, static_cast<int64_t>(ng), cap})));
    const int gpc = std::max(1, (ng + chunks0 - 1) / chunks0);
    const int chunks = std::max(1, (ng + gpc - 1) / gpc);
    EnergyArgs a;
    a.table = p.table; a.gen = p.gen; a.p_in = p.p_in; a.slot_f = p.slot_f;
    a.egroup_ptr = p.egroup_ptr; a.egroup_slots = p.egroup_slots;
    a.term_ptr = p.egroup_term_ptr; a.terms = p.egroup_terms;
    a.Nx = p.Nx; a.Ny = p.Ny; a.Nz = p.Nz; a.Ex = p.Ex; a.Ey = p.Ey; a.ppx = p.ppx; a.ppy = p.ppy;
    a.Nox = p.Nox; a.Noy = p.Noy; a.n_groups = ng; a.groups_per_chunk = gpc; a.P = p.P;
    a.part = reinterpret_cast<float*>(p.ws_part);
    const size_t smem = sizeof(float4) * kEnergyTerms + sizeof(float2) * static_cast<size_t>(p.Ey) * p.Nox;
    const bool gen = p.table_mode != CUI_STORAGE_STORED;
    const int px = (p.Nx + kEnergyThreads - 1) / kEnergyThreads;
    void (*kern)(const EnergyArgs) = px <= 1 ? (gen ? energy_kernel<true, 1> : energy_kernel<false, 1>)
                                   : px <= 2 ? (gen ? energy_kernel<true, 2> : energy_kernel<false, 2>)
                                   : px <= 4 ? (gen ? energy_kernel<true, 4> : energy_kernel<false, 4>)
                                             : (gen ? energy_kernel<true, 8> : energy_kernel<false, 8>);
    if ((e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem))) != cudaSuccess)
        return check_cuda(e, "energy_rx shared memory");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    kern<<<dim3(lines, chunks), kEnergyThreads, smem, st>>>(a);
    count_launch();
    if ((e = cudaGetLastError()) != cudaSuccess) return check_cuda(e, "energy_rx");
    energy_reduce_kernel<<<static_cast<int>(std::min<int64_t>((p.P + 255) / 256, 152 * 32)), 256, 0, st>>>(
        a.part, chunks, p.P, energy);
    count_launch();
    return check_cuda(cudaGetLastError(), "energy_rx reduce");
}
