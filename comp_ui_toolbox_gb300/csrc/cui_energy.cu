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
// memory (read from the stored table or generated there), every thread forms Q for its points over the representative slot's
// rows and adds |p_in|^2 Q for each slot of the group.  Partial sums per group
// chunk are reduced in a fixed order (deterministic).
#include <cuda_runtime.h>

#include <algorithm>

#include "cui_internal.cuh"

namespace cui {
namespace {

constexpr int kEnergyThreads = 256;
constexpr int kEnergyMaxX = 4;  // points per thread: lateral lines of up to 1024 points

struct EnergyArgs {
    const float2* table;    // [F][Nz][Noy][Nox], or null when generated (gen)
    TableGen gen;
    const float2* p_in;     // [S][P]
    const int* slot_f;
    const int* egroup_ptr;
    const int* egroup_slots;
    const int* slot_row_ptr;
    const int* slot_rows;
    const int* row_mix;
    const int* row_fl;
    const int* mix_nact;
    const int* mix_nf;
    const int* mix_act_off;
    const int64_t* mix_pref_off;
    const int* act;
    const float2* pref;
    int Nx, Ny, Nz, Ex, Ey, ppx, ppy, Nox, Noy, n_groups, groups_per_chunk;
    int64_t P;
    float* part;            // [chunks][P]
};

template <bool GEN>
__global__ void __launch_bounds__(kEnergyThreads) energy_kernel(const EnergyArgs a) {
    extern __shared__ float2 sm_e[];
    float2* sT = sm_e;  // [Ey][Nox]
    const int line = blockIdx.x, chunk = blockIdx.y;
    const int iy = line % a.Ny, z = line / a.Ny;
    const int64_t pt0 = static_cast<int64_t>(line) * a.Nx;
    const int g_lo = chunk * a.groups_per_chunk, g_hi = min(g_lo + a.groups_per_chunk, a.n_groups);
    float E[kEnergyMaxX];
#pragma unroll
    for (int k = 0; k < kEnergyMaxX; ++k) E[k] = 0.f;
    for (int g = g_lo; g < g_hi; ++g) {
        const int gb = a.egroup_ptr[g], ge = a.egroup_ptr[g + 1];
        const int rep = a.egroup_slots[gb];
        const int f = a.slot_f[rep];
        __syncthreads();
        for (int idx = threadIdx.x; idx < a.Ey * a.Nox; idx += blockDim.x) {
            const int ey = idx / a.Nox, ox = idx - ey * a.Nox;
            const int oy = iy - ey * a.ppy + (a.Ey - 1) * a.ppy;
            if constexpr (GEN)
                sT[idx] = gen_entry(a.gen, gen_row(a.gen, f, z, oy), ox);
            else
                sT[idx] = a.table[((static_cast<int64_t>(f) * a.Nz + z) * a.Noy + oy) * a.Nox + ox];
        }
        __syncthreads();
        float Q[kEnergyMaxX];
#pragma unroll
        for (int k = 0; k < kEnergyMaxX; ++k) Q[k] = 0.f;
        for (int rr = a.slot_row_ptr[rep]; rr < a.slot_row_ptr[rep + 1]; ++rr) {
            const int row = a.slot_rows[rr];
            const int m = a.row_mix[row], fl = a.row_fl[row];
            const int nact = a.mix_nact[m], nf = a.mix_nf[m];
            const int* act = a.act + a.mix_act_off[m];
            const float2* pref = a.pref + a.mix_pref_off[m] + fl;
            float2 acc[kEnergyMaxX];
#pragma unroll
            for (int k = 0; k < kEnergyMaxX; ++k) acc[k] = make_float2(0.f, 0.f);
            for (int ia = 0; ia < nact; ++ia) {
                const int e = __ldg(act + ia);
                const int ey = a.Ey == 1 ? 0 : e / a.Ex, ex = e - ey * a.Ex;
                const float2 w = __ldg(pref + static_cast<int64_t>(ia) * nf);
                const float2* trow = sT + ey * a.Nox + (a.Ex - 1 - ex) * a.ppx;
#pragma unroll
                for (int k = 0; k < kEnergyMaxX; ++k) {
                    const int x = threadIdx.x + k * kEnergyThreads;
                    if (x < a.Nx) {
                        const float2 t = trow[x];
                        acc[k].x = fmaf(w.x, t.x, fmaf(-w.y, t.y, acc[k].x));
                        acc[k].y = fmaf(w.x, t.y, fmaf(w.y, t.x, acc[k].y));
                    }
                }
            }
#pragma unroll
            for (int k = 0; k < kEnergyMaxX; ++k) Q[k] = fmaf(acc[k].x, acc[k].x, fmaf(acc[k].y, acc[k].y, Q[k]));
        }
        for (int i = gb; i < ge; ++i) {  // every slot of the group: |p_in|^2 Q
            const float2* pin = a.p_in + static_cast<int64_t>(a.egroup_slots[i]) * a.P + pt0;
#pragma unroll
            for (int k = 0; k < kEnergyMaxX; ++k) {
                const int x = threadIdx.x + k * kEnergyThreads;
                if (x < a.Nx) {
                    const float2 pv = __ldg(pin + x);
                    E[k] = fmaf(pv.x * pv.x + pv.y * pv.y, Q[k], E[k]);
                }
            }
        }
    }
#pragma unroll
    for (int k = 0; k < kEnergyMaxX; ++k) {
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
    using namespace cui;
    if (!plan || !energy) return set_error(CUI_ERR_INVALID_ARG, "NULL argument");
    Plan& p = plan->p;
    if (p.Nx > kEnergyThreads * kEnergyMaxX)
        return set_error(CUI_ERR_UNSUPPORTED_SETUP, "energy_rx covers lateral grid lines of up to 1024 points");
    cudaError_t e = cudaSetDevice(p.device);
    if (e != cudaSuccess) return check_cuda(e, "cudaSetDevice");
    const int lines = p.Ny * p.Nz;
    const int64_t cap = static_cast<int64_t>(p.ws_part_bytes / (sizeof(float) * static_cast<size_t>(p.P)));
    const int64_t want = (8 * 152 + lines - 1) / lines;
    const int ng = p.n_egroups;
    const int chunks0 = static_cast<int>(std::max<int64_t>(1, std::min<int64_t>({want, static_cast<int64_t>(ng), cap})));
    const int gpc = std::max(1, (ng + chunks0 - 1) / chunks0);
    const int chunks = std::max(1, (ng + gpc - 1) / gpc);
    EnergyArgs a;
    a.table = p.table; a.gen = p.gen; a.p_in = p.p_in; a.slot_f = p.slot_f; a.slot_row_ptr = p.slot_row_ptr; a.slot_rows = p.slot_rows;
    a.egroup_ptr = p.egroup_ptr; a.egroup_slots = p.egroup_slots;
    a.row_mix = p.row_mix; a.row_fl = p.row_fl; a.mix_nact = p.mix_nact; a.mix_nf = p.mix_nf;
    a.mix_act_off = p.mix_act_off; a.mix_pref_off = p.mix_pref_off; a.act = p.act; a.pref = p.pref;
    a.Nx = p.Nx; a.Ny = p.Ny; a.Nz = p.Nz; a.Ex = p.Ex; a.Ey = p.Ey; a.ppx = p.ppx; a.ppy = p.ppy;
    a.Nox = p.Nox; a.Noy = p.Noy; a.n_groups = ng; a.groups_per_chunk = gpc; a.P = p.P;
    a.part = reinterpret_cast<float*>(p.ws_part);
    const size_t smem = sizeof(float2) * static_cast<size_t>(p.Ey) * p.Nox;
    void (*kern)(const EnergyArgs) = p.table_mode != CUI_STORAGE_STORED ? energy_kernel<true> : energy_kernel<false>;
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
