// Per-plan autotuner: times the contraction paths a plan can run for a given
// object count and keeps the faster one; on the split-BF16 line-unit path it
// then picks the launch shapes by a coordinate search over the column tiles
// (64 columns or the narrower 16/32-column tiles) and the block counts the
// forward's line groups and the adjoint's frequency chunks aim at, keeping
// each candidate only when it lowers the timed forward + adjoint pair.
//
// Candidates: the FP32 CUDA-core kernels and the split-BF16 tensor-core
// kernels (2D setups).  Both meet the operator's accuracy bound (relative L2
// <= 1e-5 against the FP64 oracle); which one is faster depends on how many
// incident waves share a frequency (the tensor-core tiles hold 16 or 32 wave x
// object columns, so a one-wave problem leaves most of a tile empty) and on
// the grid.  Scratch inputs are allocated, timed on the caller's stream and
// freed here, so the call belongs to plan set-up, before any stream capture.
#include <cuda_runtime.h>

#include <string>

#include "cui_internal.cuh"

namespace cui {
namespace {

// one forward + one adjoint apply of the plan's current path on scratch data
cui_status apply_pair(Plan* p, const float2* g, float2* u, float2* gh, int B, cudaStream_t st) {
    cui_status s = forward_device(p, g, p->P, B, u, p->n_obs, st);
    if (s != CUI_OK) return s;
    return adjoint_device(p, u, p->n_obs, B, gh, p->P, st);
}

cui_status time_path(Plan* p, const float2* g, float2* u, float2* gh, int B, cudaStream_t st, double* ms) {
    cui_status s = apply_pair(p, g, u, gh, B, st);  // warm-up (first use of a path's kernels)
    if (s != CUI_OK) return s;
    cudaEvent_t e0, e1;
    cudaError_t e = cudaEventCreate(&e0);
    if (e != cudaSuccess) return check_cuda(e, "cudaEventCreate");
    if ((e = cudaEventCreate(&e1)) != cudaSuccess) {
        cudaEventDestroy(e0);
        return check_cuda(e, "cudaEventCreate");
    }
    constexpr int kReps = 2;
    cudaEventRecord(e0, st);
    for (int r = 0; r < kReps && s == CUI_OK; ++r) s = apply_pair(p, g, u, gh, B, st);
    cudaEventRecord(e1, st);
    e = cudaEventSynchronize(e1);
    float t = 0.f;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&t, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (s != CUI_OK) return s;
    if (e != cudaSuccess) return check_cuda(e, "autotune timing");
    *ms = t / kReps;
    return CUI_OK;
}

}  // namespace
}  // namespace cui

extern "C" cui_status cui_born_autotune(cui_born_plan* plan, int32_t n_objects, int32_t* precision, double* ms,
                                        void* stream) {
    const cui::NvtxRange nvtx_range("cui_born_autotune");
    using namespace cui;
    if (!plan) return set_error(CUI_ERR_INVALID_ARG, "plan is NULL");
    Plan& p = plan->p;
    if (n_objects < 1 || n_objects > p.max_objects)
        return set_error(CUI_ERR_INVALID_ARG, "n_objects must be in [1, max_objects]");
    const DeviceGuard dev_guard(p.device);
    cudaError_t e = dev_guard.err;
    if (e != cudaSuccess) return check_cuda(e, "cudaSetDevice");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const size_t ng = static_cast<size_t>(p.P) * n_objects, nu = static_cast<size_t>(p.n_obs) * n_objects;
    float2 *g = nullptr, *u = nullptr, *gh = nullptr;
    if ((e = cudaMalloc(&g, ng * sizeof(float2))) != cudaSuccess) return check_cuda(e, "cudaMalloc");
    if ((e = cudaMalloc(&gh, ng * sizeof(float2))) != cudaSuccess) {
        cudaFree(g);
        return check_cuda(e, "cudaMalloc");
    }
    if ((e = cudaMalloc(&u, nu * sizeof(float2))) != cudaSuccess) {
        cudaFree(g);
        cudaFree(gh);
        return check_cuda(e, "cudaMalloc");
    }
    cudaMemsetAsync(g, 0, ng * sizeof(float2), st);
    const int32_t before = p.precision;
    p.tune_tile = p.tune_fwd_blocks = p.tune_adj_blocks = 0;  // every search starts from the rule
    double t[2] = {-1.0, -1.0};
    cui_status s = cui_born_set_precision(plan, CUI_PRECISION_FP32);
    if (s == CUI_OK) s = time_path(&p, g, u, gh, n_objects, st, &t[0]);
    std::string why;
    const bool tc_ok = (p.n_dims == 2) && (tc2_supported(&p, &why) || tc_supported(&p, &why));
    if (s == CUI_OK && tc_ok) {
        s = cui_born_set_precision(plan, CUI_PRECISION_BF16X3);
        if (s == CUI_OK) s = time_path(&p, g, u, gh, n_objects, st, &t[1]);
    }
    const int32_t best = (t[1] >= 0.0 && t[1] < t[0]) ? CUI_PRECISION_BF16X3 : CUI_PRECISION_FP32;
    if (s == CUI_OK) s = cui_born_set_precision(plan, best);
    if (s == CUI_OK && best == CUI_PRECISION_BF16X3 && p.tc2) {
        double t_best = t[1];
        auto trial = [&](int* field, int value) -> cui_status {
            const int old = *field;
            *field = value;
            double tv = 0.0;
            const cui_status s2 = time_path(&p, g, u, gh, n_objects, st, &tv);
            if (s2 == CUI_OK && tv < t_best)
                t_best = tv;
            else
                *field = old;
            return s2;
        };
        s = trial(&p.tune_tile, 1);
        for (int v : {4 * 152, 16 * 152, 32 * 152})
            if (s == CUI_OK) s = trial(&p.tune_fwd_blocks, v);
        for (int v : {4 * 152, 16 * 152, 32 * 152})
            if (s == CUI_OK) s = trial(&p.tune_adj_blocks, v);
        if (s == CUI_OK) t[1] = t_best;
    }
    cudaFree(g);
    cudaFree(gh);
    cudaFree(u);
    if (s != CUI_OK) {
        p.precision = before;
        p.tune_tile = p.tune_fwd_blocks = p.tune_adj_blocks = 0;
        return s;
    }
    if (precision) *precision = best;
    if (ms) {
        ms[0] = t[0];
        ms[1] = t[1];
    }
    return CUI_OK;
}

extern "C" cui_status cui_born_autotune_config(const cui_born_plan* plan, int32_t* narrow_tiles, int32_t* fwd_blocks,
                                               int32_t* adj_blocks) {
    if (!plan) return cui::set_error(CUI_ERR_INVALID_ARG, "plan is NULL");
    const cui::Plan& p = plan->p;
    if (narrow_tiles) *narrow_tiles = p.tune_tile;
    if (fwd_blocks) *fwd_blocks = p.tune_fwd_blocks;
    if (adj_blocks) *adj_blocks = p.tune_adj_blocks;
    return CUI_OK;
}

extern "C" cui_status cui_born_set_launch_shapes(cui_born_plan* plan, int32_t narrow_tiles, int32_t fwd_blocks,
                                                 int32_t adj_blocks) {
    if (!plan) return cui::set_error(CUI_ERR_INVALID_ARG, "plan is NULL");
    if ((narrow_tiles != 0 && narrow_tiles != 1) || fwd_blocks < 0 || adj_blocks < 0)
        return cui::set_error(CUI_ERR_INVALID_ARG, "narrow_tiles must be 0 or 1 and block counts >= 0");
    cui::Plan& p = plan->p;
    p.tune_tile = narrow_tiles;
    p.tune_fwd_blocks = fwd_blocks;
    p.tune_adj_blocks = adj_blocks;
    return CUI_OK;
}
