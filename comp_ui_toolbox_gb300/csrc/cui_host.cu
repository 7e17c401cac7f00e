// Host-buffer entry points with the MEX gateway's semantics.
//
// combined_quick_gpu converts its FP64 input to FP32 on the host, uploads
// it, runs the operator and converts the FP32 result back to FP64
// (+scattering/combined_quick_gpu.cu:700-780, :940-1006).  These entry points
// do the same around the device applies, in one of two ways:
//   * where the GPU reads pageable host memory through the host's page tables
//     (ATS over NVLink-C2C on Grace systems: cudaDevAttrPageableMemoryAccess and
//     cudaDevAttrPageableMemoryAccessUsesHostPageTables), a kernel reads the
//     caller's FP64 arrays and writes FP32 device columns, and another writes
//     the FP64 result straight into the caller's array: no host pass and no
//     staging copy;
//   * otherwise through pinned staging buffers that the plan allocates on first
//     use and keeps; the conversions run on all host cores, and the upload of
//     gamma overlaps the conversion of the measured data.
// The environment variable CUI_BORN_HOST_STAGING=1, read when a plan first
// uses a host entry point, selects the staging path.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "cui_internal.cuh"

namespace cui {
namespace {

bool host_direct(Plan& p) {
    if (p.host_direct < 0) {
        int pageable = 0, host_tables = 0;
        const char* env = std::getenv("CUI_BORN_HOST_STAGING");
        const bool staging = env && env[0] == '1';
        if (cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccess, p.device) != cudaSuccess) pageable = 0;
        if (cudaDeviceGetAttribute(&host_tables, cudaDevAttrPageableMemoryAccessUsesHostPageTables, p.device) !=
            cudaSuccess)
            host_tables = 0;
        p.host_direct = (!staging && pageable && host_tables) ? 1 : 0;
    }
    return p.host_direct == 1;
}

// FP64 host column-major (leading dimension ld) -> packed FP32 device columns; grid (row blocks, B)
__global__ void host_in_kernel(const cui_complex64* __restrict__ src, int64_t ld, int64_t rows, float2* __restrict__ dst) {
    const int b = blockIdx.y;
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < rows;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const cui_complex64 c = src[b * ld + i];
        dst[b * rows + i] = make_float2(static_cast<float>(c.re), static_cast<float>(c.im));
    }
}

// packed FP32 device columns -> FP64 host column-major, with streaming (evict-first) stores: the
// lines go out to host memory without being kept in L2 (172 GB/s into pageable host memory through
// the host page tables, against 97 GB/s with default stores); 16-byte stores when the caller's
// array is 16-byte aligned (every element then is), two 8-byte stores otherwise
template <bool A16>
__global__ void host_out_kernel(const float2* __restrict__ src, int64_t rows, cui_complex64* __restrict__ dst, int64_t ld) {
    const int b = blockIdx.y;
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < rows;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const float2 v = src[b * rows + i];
        cui_complex64* d = dst + b * ld + i;
        if (A16) {
            __stcs(reinterpret_cast<double2*>(d), make_double2(v.x, v.y));
        } else {
            __stcs(&d->re, static_cast<double>(v.x));
            __stcs(&d->im, static_cast<double>(v.y));
        }
    }
}

// the device kernels read and write the caller's arrays element by element: cui_complex64 and double
// arrays must have their types' 8-byte alignment (checked before any launch)
bool aligned8(const void* ptr) { return (reinterpret_cast<uintptr_t>(ptr) & 7) == 0; }

void launch_host_out(const float2* src, int64_t rows, int B, cui_complex64* dst, int64_t ld) {
    const dim3 grid(static_cast<unsigned>(std::min<int64_t>((rows + 255) / 256, 4 * 152)), static_cast<unsigned>(B));
    if ((reinterpret_cast<uintptr_t>(dst) & 15) == 0)
        host_out_kernel<true><<<grid, 256>>>(src, rows, dst, ld);
    else
        host_out_kernel<false><<<grid, 256>>>(src, rows, dst, ld);
}

__global__ void host_loss_kernel(const float* __restrict__ src, int B, double* __restrict__ dst) {
    for (int b = threadIdx.x; b < B; b += blockDim.x) dst[b] = src[b];
}

dim3 host_grid(int64_t rows, int B) {
    return dim3(static_cast<unsigned>(std::min<int64_t>((rows + 255) / 256, 4 * 152)), static_cast<unsigned>(B));
}

// device staging columns (both paths) and, for the staging path, the pinned host buffers
cui_status ensure_device_stage(Plan& p) {
    cudaError_t e;
    if (!p.in_stream && (e = cudaStreamCreateWithFlags(&p.in_stream, cudaStreamNonBlocking)) != cudaSuccess)
        return check_cuda(e, "cudaStreamCreate");
    if (!p.in_done && (e = cudaEventCreateWithFlags(&p.in_done, cudaEventDisableTiming)) != cudaSuccess)
        return check_cuda(e, "cudaEventCreate");
    // each buffer once; after a failed allocation the next call allocates the missing ones
    const size_t n = static_cast<size_t>(std::max<int64_t>(p.P, p.n_obs)) * p.max_objects;
    for (float2** d : {&p.d_stage_in, &p.d_stage_out, &p.d_stage_aux}) {
        if (*d) continue;
        const cui_status s = device_alloc(p, reinterpret_cast<void**>(d), n * sizeof(float2));
        if (s != CUI_OK) return s;
    }
    if (!p.d_stage_loss) return device_alloc(p, reinterpret_cast<void**>(&p.d_stage_loss), sizeof(float) * p.max_objects);
    return CUI_OK;
}

cui_status ensure_stage(Plan& p) {
    cui_status s = ensure_device_stage(p);
    if (s != CUI_OK) return s;
    const size_t n = static_cast<size_t>(std::max<int64_t>(p.P, p.n_obs)) * p.max_objects;
    for (float2** h : {&p.h_stage_in, &p.h_stage_out, &p.h_stage_aux}) {
        if (*h) continue;  // after a failed allocation the next call allocates the missing ones
        const cudaError_t e = cudaHostAlloc(reinterpret_cast<void**>(h), n * sizeof(float2), cudaHostAllocDefault);
        if (e != cudaSuccess) {
            *h = nullptr;
            return check_cuda(e, "cudaHostAlloc");
        }
    }
    p.h_stage_elems = n;
    return CUI_OK;
}

// fn(lo, hi) over [0, n) split across the host's cores (one thread below 64 Ki elements per core)
template <class Fn>
void parallel_for(int64_t n, Fn fn) {
    const int64_t per = int64_t(1) << 16;
    const int64_t cores = std::max(1u, std::thread::hardware_concurrency());
    const int nt = static_cast<int>(std::max<int64_t>(1, std::min<int64_t>(cores, n / per)));
    if (nt <= 1) {
        fn(int64_t(0), n);
        return;
    }
    std::vector<std::thread> ts;
    ts.reserve(nt);
    for (int t = 0; t < nt; ++t) ts.emplace_back(fn, n * t / nt, n * (t + 1) / nt);
    for (auto& t : ts) t.join();
}

// column-major FP64 (leading dimension ld) -> packed FP32
void pack(const cui_complex64* src, int64_t ld, int64_t rows, int B, float2* dst) {
    parallel_for(rows * B, [=](int64_t lo, int64_t hi) {
        for (int64_t k = lo; k < hi; ++k) {
            const int64_t b = k / rows, i = k - b * rows;
            const cui_complex64 c = src[b * ld + i];
            dst[k] = make_float2(static_cast<float>(c.re), static_cast<float>(c.im));
        }
    });
}

void unpack(const float2* src, int64_t rows, int B, cui_complex64* dst, int64_t ld) {
    parallel_for(rows * B, [=](int64_t lo, int64_t hi) {
        for (int64_t k = lo; k < hi; ++k) {
            const int64_t b = k / rows, i = k - b * rows;
            const float2 v = src[k];
            dst[b * ld + i].re = v.x;
            dst[b * ld + i].im = v.y;
        }
    });
}

}  // namespace
}  // namespace cui

extern "C" {

cui_status cui_born_combined_host(cui_born_plan* plan, int32_t mode, const cui_complex64* input, int64_t ld_in,
                                  int32_t n_objects, cui_complex64* output, int64_t ld_out) {
    const cui::NvtxRange nvtx_range("cui_born_combined_host");
    using namespace cui;
    if (!plan) return set_error(CUI_ERR_INVALID_ARG, "plan is NULL");
    Plan& p = plan->p;
    if (mode != 1 && mode != 2)
        return set_error(CUI_ERR_INVALID_ARG, "mode must be 1 (forward) or 2 (adjoint) (combined_quick_gpu:NoNumericScalarMode)");
    const int64_t rows_in = (mode == 1) ? p.P : p.n_obs;
    const int64_t rows_out = (mode == 1) ? p.n_obs : p.P;
    if (!input || !output || n_objects < 1 || n_objects > p.max_objects || ld_in < rows_in || ld_out < rows_out)
        return set_error(CUI_ERR_INVALID_ARG, "input must be a matrix with the operator's number of rows "
                                              "(combined_quick_gpu:NoValidDoubleMatrix)");
    if (!aligned8(input) || !aligned8(output))
        return set_error(CUI_ERR_INVALID_ARG, "host arrays must be 8-byte aligned (cui_complex64)");
    const DeviceGuard dev_guard(p.device);
    cudaError_t e = dev_guard.err;
    if (e != cudaSuccess) return check_cuda(e, "cudaSetDevice");
    if (host_direct(p)) {
        cui_status s = ensure_device_stage(p);
        if (s != CUI_OK) return s;
        host_in_kernel<<<host_grid(rows_in, n_objects), 256>>>(input, ld_in, rows_in, p.d_stage_in);
        count_launch();
        if ((e = cudaGetLastError()) != cudaSuccess) return check_cuda(e, "host input");
        bool written = false;  // the folded adjoint may write the caller's array itself
        s = (mode == 1) ? forward_device(&p, p.d_stage_in, rows_in, n_objects, p.d_stage_out, rows_out, 0)
                        : adjoint_device(&p, p.d_stage_in, rows_in, n_objects, p.d_stage_out, rows_out, 0,
                                         HostOut{output, ld_out, &written});
        if (s != CUI_OK) return s;
        if (!written) {
            launch_host_out(p.d_stage_out, rows_out, n_objects, output, ld_out);
            count_launch();
        }
        if ((e = cudaGetLastError()) != cudaSuccess) return check_cuda(e, "host output");
        return check_cuda(cudaStreamSynchronize(0), "synchronize");
    }
    cui_status s = ensure_stage(p);
    if (s != CUI_OK) return s;
    pack(input, ld_in, rows_in, n_objects, p.h_stage_in);
    const size_t bytes_in = sizeof(float2) * rows_in * n_objects;
    const size_t bytes_out = sizeof(float2) * rows_out * n_objects;
    if ((e = cudaMemcpyAsync(p.d_stage_in, p.h_stage_in, bytes_in, cudaMemcpyHostToDevice, 0)) != cudaSuccess)
        return check_cuda(e, "upload");
    s = (mode == 1) ? forward_device(&p, p.d_stage_in, rows_in, n_objects, p.d_stage_out, rows_out, 0)
                    : adjoint_device(&p, p.d_stage_in, rows_in, n_objects, p.d_stage_out, rows_out, 0);
    if (s != CUI_OK) return s;
    if ((e = cudaMemcpyAsync(p.h_stage_out, p.d_stage_out, bytes_out, cudaMemcpyDeviceToHost, 0)) != cudaSuccess)
        return check_cuda(e, "download");
    if ((e = cudaStreamSynchronize(0)) != cudaSuccess) return check_cuda(e, "synchronize");
    unpack(p.h_stage_out, rows_out, n_objects, output, ld_out);
    return CUI_OK;
}

cui_status cui_born_vjp_host(cui_born_plan* plan, const cui_complex64* gamma, int64_t ld_gamma,
                             const cui_complex64* u_meas, int64_t ld_u, int32_t n_objects, cui_complex64* grad,
                             int64_t ld_grad, double* loss) {
    const cui::NvtxRange nvtx_range("cui_born_vjp_host");
    using namespace cui;
    if (!plan) return set_error(CUI_ERR_INVALID_ARG, "plan is NULL");
    Plan& p = plan->p;
    if (!gamma || !u_meas || !grad || n_objects < 1 || n_objects > p.max_objects || ld_gamma < p.P ||
        ld_u < p.n_obs || ld_grad < p.P)
        return set_error(CUI_ERR_INVALID_ARG, "invalid arguments to cui_born_vjp_host");
    if (!aligned8(gamma) || !aligned8(u_meas) || !aligned8(grad) || (loss && !aligned8(loss)))
        return set_error(CUI_ERR_INVALID_ARG, "host arrays must be 8-byte aligned (cui_complex64, double)");
    const DeviceGuard dev_guard(p.device);
    cudaError_t e = dev_guard.err;
    if (e != cudaSuccess) return check_cuda(e, "cudaSetDevice");
    if (host_direct(p)) {
        cui_status s = ensure_device_stage(p);
        if (s != CUI_OK) return s;
        host_in_kernel<<<host_grid(p.P, n_objects), 256>>>(gamma, ld_gamma, p.P, p.d_stage_in);
        // the measured data are read on the plan's input stream while the forward runs; the previous
        // call's residual, the last reader of d_stage_aux, ended before that call returned
        host_in_kernel<<<host_grid(p.n_obs, n_objects), 256, 0, p.in_stream>>>(u_meas, ld_u, p.n_obs, p.d_stage_aux);
        count_launch(2);
        e = cudaGetLastError();
        if (e == cudaSuccess) e = cudaEventRecord(p.in_done, p.in_stream);
        // no return before the read of the caller's u_meas has ended
        struct InputGuard {
            cudaStream_t s;
            ~InputGuard() { cudaStreamSynchronize(s); }
        } input_guard{p.in_stream};
        if (e != cudaSuccess) return check_cuda(e, "host input");
        bool written = false;  // the folded adjoint may write the caller's gradient itself
        s = vjp_device(&p, p.d_stage_in, p.P, p.d_stage_aux, p.n_obs, n_objects, p.d_stage_out, p.P, p.d_stage_loss, 0,
                       HostOut{grad, ld_grad, &written}, p.in_done);
        if (s != CUI_OK) return s;
        if (!written) {
            launch_host_out(p.d_stage_out, p.P, n_objects, grad, ld_grad);
            count_launch();
        }
        if (loss) {
            host_loss_kernel<<<1, 128>>>(p.d_stage_loss, n_objects, loss);
            count_launch();
        }
        if ((e = cudaGetLastError()) != cudaSuccess) return check_cuda(e, "host output");
        return check_cuda(cudaStreamSynchronize(0), "synchronize");
    }
    cui_status s = ensure_stage(p);
    if (s != CUI_OK) return s;
    // gamma and u_meas share the input staging buffer: gamma first, then u_meas
    const int64_t ng = p.P * n_objects, nu = p.n_obs * n_objects;
    if (static_cast<size_t>(ng) > p.h_stage_elems || static_cast<size_t>(nu) > p.h_stage_elems)
        return set_error(CUI_ERR_INVALID_ARG, "staging buffer too small");
    pack(gamma, ld_gamma, p.P, n_objects, p.h_stage_in);
    if ((e = cudaMemcpyAsync(p.d_stage_in, p.h_stage_in, sizeof(float2) * ng, cudaMemcpyHostToDevice, 0)) != cudaSuccess)
        return check_cuda(e, "upload gamma");
    pack(u_meas, ld_u, p.n_obs, n_objects, p.h_stage_aux);  // overlaps the upload of gamma
    if ((e = cudaMemcpyAsync(p.d_stage_aux, p.h_stage_aux, sizeof(float2) * nu, cudaMemcpyHostToDevice, 0)) != cudaSuccess)
        return check_cuda(e, "upload u");
    s = vjp_device(&p, p.d_stage_in, p.P, p.d_stage_aux, p.n_obs, n_objects, p.d_stage_out, p.P, p.d_stage_loss, 0);
    if (s != CUI_OK) return s;
    if ((e = cudaMemcpyAsync(p.h_stage_out, p.d_stage_out, sizeof(float2) * ng, cudaMemcpyDeviceToHost, 0)) != cudaSuccess)
        return check_cuda(e, "download");
    std::vector<float> hl(n_objects);
    if (loss && (e = cudaMemcpyAsync(hl.data(), p.d_stage_loss, sizeof(float) * n_objects, cudaMemcpyDeviceToHost, 0)) !=
                    cudaSuccess)
        return check_cuda(e, "download loss");
    if ((e = cudaStreamSynchronize(0)) != cudaSuccess) return check_cuda(e, "synchronize");
    unpack(p.h_stage_out, p.P, n_objects, grad, ld_grad);
    if (loss)
        for (int b = 0; b < n_objects; ++b) loss[b] = hl[b];
    return CUI_OK;
}

}  // extern "C"

extern "C" cui_status cui_born_lasso_host(cui_born_plan* plan, const cui_complex64* u_meas, int64_t ld_u,
                                          int32_t n_objects, cui_complex64* gamma, int64_t ld_gamma,
                                          const float* lambda, float step, int32_t n_iter) {
    const cui::NvtxRange nvtx_range("cui_born_lasso_host");
    using namespace cui;
    if (!plan) return set_error(CUI_ERR_INVALID_ARG, "plan is NULL");
    Plan& p = plan->p;
    if (!u_meas || !gamma || !lambda || n_objects < 1 || n_objects > p.max_objects || ld_u < p.n_obs ||
        ld_gamma < p.P || n_iter < 0 || !(step > 0.f))
        return set_error(CUI_ERR_INVALID_ARG, "invalid arguments to cui_born_lasso_host");
    if (!aligned8(u_meas) || !aligned8(gamma))
        return set_error(CUI_ERR_INVALID_ARG, "host arrays must be 8-byte aligned (cui_complex64)");
    const DeviceGuard dev_guard(p.device);
    cudaError_t e = dev_guard.err;
    if (e != cudaSuccess) return check_cuda(e, "cudaSetDevice");
    const bool direct = host_direct(p);
    cui_status s = direct ? ensure_device_stage(p) : ensure_stage(p);
    if (s != CUI_OK) return s;
    const size_t ng = static_cast<size_t>(p.P) * n_objects, nu = static_cast<size_t>(p.n_obs) * n_objects;
    // thresholds in the loss slot of the device staging (one float per object)
    if ((e = cudaMemcpyAsync(p.d_stage_loss, lambda, sizeof(float) * n_objects, cudaMemcpyHostToDevice, 0)) !=
        cudaSuccess)
        return check_cuda(e, "upload lambda");
    if (direct) {
        host_in_kernel<<<host_grid(p.n_obs, n_objects), 256>>>(u_meas, ld_u, p.n_obs, p.d_stage_aux);
        host_in_kernel<<<host_grid(p.P, n_objects), 256>>>(gamma, ld_gamma, p.P, p.d_stage_in);
        count_launch(2);
        if ((e = cudaGetLastError()) != cudaSuccess) return check_cuda(e, "host input");
    } else {
        pack(u_meas, ld_u, p.n_obs, n_objects, p.h_stage_aux);
        pack(gamma, ld_gamma, p.P, n_objects, p.h_stage_in);
        if ((e = cudaMemcpyAsync(p.d_stage_aux, p.h_stage_aux, sizeof(float2) * nu, cudaMemcpyHostToDevice, 0)) !=
                cudaSuccess ||
            (e = cudaMemcpyAsync(p.d_stage_in, p.h_stage_in, sizeof(float2) * ng, cudaMemcpyHostToDevice, 0)) !=
                cudaSuccess)
            return check_cuda(e, "upload");
    }
    s = lasso_device(&p, p.d_stage_in, p.P, p.d_stage_aux, p.n_obs, n_objects, step, p.d_stage_loss, n_iter, nullptr, 0);
    if (s != CUI_OK) return s;
    if (direct) {
        launch_host_out(p.d_stage_in, p.P, n_objects, gamma, ld_gamma);
        count_launch();
        if ((e = cudaGetLastError()) != cudaSuccess) return check_cuda(e, "host output");
        return check_cuda(cudaStreamSynchronize(0), "synchronize");
    }
    if ((e = cudaMemcpyAsync(p.h_stage_out, p.d_stage_in, sizeof(float2) * ng, cudaMemcpyDeviceToHost, 0)) != cudaSuccess)
        return check_cuda(e, "download");
    if ((e = cudaStreamSynchronize(0)) != cudaSuccess) return check_cuda(e, "synchronize");
    unpack(p.h_stage_out, p.P, n_objects, gamma, ld_gamma);
    return CUI_OK;
}

extern "C" cui_status cui_born_host_path(cui_born_plan* plan, int32_t* direct) {
    using namespace cui;
    if (!plan || !direct) return set_error(CUI_ERR_INVALID_ARG, "NULL argument");
    const DeviceGuard dev_guard(plan->p.device);
    if (dev_guard.err != cudaSuccess) return check_cuda(dev_guard.err, "cudaSetDevice");
    *direct = host_direct(plan->p) ? 1 : 0;
    return CUI_OK;
}
