// Per-plan autotuner: times the contraction paths a plan can run for a given
// object count and keeps the faster one.
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
    using namespace cui;
    if (!plan) return set_error(CUI_ERR_INVALID_ARG, "plan is NULL");
    Plan& p = plan->p;
    if (n_objects < 1 || n_objects > p.max_objects)
        return set_error(CUI_ERR_INVALID_ARG, "n_objects must be in [1, max_objects]");
    cudaError_t e = cudaSetDevice(p.device);
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
    double t[2] = {-1.0, -1.0};
    cui_status s = cui_born_set_precision(plan, CUI_PRECISION_FP32);
    if (s == CUI_OK) s = time_path(&p, g, u, gh, n_objects, st, &t[0]);
    std::string why;
    const bool tc_ok = (p.n_dims == 2) && (tc2_supported(&p, &why) || tc_supported(&p, &why));
    if (s == CUI_OK && tc_ok) {
        s = cui_born_set_precision(plan, CUI_PRECISION_BF16X3);
        if (s == CUI_OK) s = time_path(&p, g, u, gh, n_objects, st, &t[1]);
    }
    cudaFree(g);
    cudaFree(gh);
    cudaFree(u);
    if (s != CUI_OK) {
        p.precision = before;
        return s;
    }
    const int32_t best = (t[1] >= 0.0 && t[1] < t[0]) ? CUI_PRECISION_BF16X3 : CUI_PRECISION_FP32;
    if ((s = cui_born_set_precision(plan, best)) != CUI_OK) return s;
    if (precision) *precision = best;
    if (ms) {
        ms[0] = t[0];
        ms[1] = t[1];
    }
    return CUI_OK;
}
