// Host stand-ins for the CUDA runtime and cuBLAS calls of the reference's MEX
// gateway (+scattering/combined_quick_gpu.cu), so that its host code runs
// unchanged on a machine without a GPU.
//
// TEST INFRASTRUCTURE ONLY (the oracle's reference runner).  "Device" memory is
// host memory; copies are memcpy; cudaMallocPitch pads rows to 512 bytes.  The
// gateway launches one kernel, compute_matrix_kernel (:1099-1124); its launch is
// executed here by host_compute_matrix, a restatement of that kernel's formula
//     Phi[p * N_f_mix + f] = (h_ref_row(shift[p])[f_seq[f]] * p_in_row(p)[f_meas[f]]) * pref[f]
// in FP32 complex arithmetic (cuCmulf), over the launch's grid.  cublasCgemm is a
// host complex GEMM (column-major, op N / T / C) whose inner products are summed in
// FP64 over the FP32 operands and rounded to FP32 once per call, as the output
// array is FP32; cuBLAS's own FP32 summation order is not specified, so the
// runner's outputs agree with a GPU run of the gateway to FP32 rounding, not bitwise.
#include <cuComplex.h>
#include <cublas_v2.h>
#include <cuda_runtime.h>

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <string>
#include <vector>

namespace {

struct LaunchCfg {
    dim3 grid, block;
    size_t shmem;
    void* stream;
};
// constructed on first use: nvcc's module constructor registers the kernel before this file's
// globals with constructors would be initialised
std::vector<LaunchCfg>& cfg_stack() {
    static std::vector<LaunchCfg> s;
    return s;
}
std::map<const void*, std::string>& kernels() {  // host stub -> device function name
    static std::map<const void*, std::string> k;
    return k;
}
int g_launches = 0;

void host_compute_matrix(dim3 grid, dim3 block, void** args) {
    cuComplex* phi = *static_cast<cuComplex**>(args[0]);
    const int n_f = *static_cast<int*>(args[1]);
    const int n_occ = *static_cast<int*>(args[2]);
    const char* h_ref = *static_cast<char**>(args[3]);
    const size_t pitch_h = *static_cast<size_t*>(args[4]);
    const int* shift = *static_cast<int**>(args[5]);
    const int* f_seq = *static_cast<int**>(args[6]);
    const char* p_in = *static_cast<char**>(args[7]);
    const size_t pitch_p = *static_cast<size_t*>(args[8]);
    const int* f_meas = *static_cast<int**>(args[9]);
    const cuComplex* pref = *static_cast<cuComplex**>(args[10]);
    for (unsigned by = 0; by < grid.y; ++by)
        for (unsigned bx = 0; bx < grid.x; ++bx)
            for (unsigned ty = 0; ty < block.y; ++ty)
                for (unsigned tx = 0; tx < block.x; ++tx) {
                    const int p = static_cast<int>(bx * block.x + tx), f = static_cast<int>(by * block.y + ty);
                    if (f >= n_f || p >= n_occ) continue;
                    const cuComplex h = reinterpret_cast<const cuComplex*>(h_ref + shift[p] * pitch_h)[f_seq[f]];
                    const cuComplex q = reinterpret_cast<const cuComplex*>(p_in + p * pitch_p)[f_meas[f]];
                    phi[static_cast<size_t>(p) * n_f + f] = cuCmulf(cuCmulf(h, q), pref[f]);
                }
}

}  // namespace

extern "C" {

// ---- registration and launch hooks of nvcc's host code ----------------------------
void** __cudaRegisterFatBinary(void*) {
    static void* handle = nullptr;
    return &handle;
}
void __cudaRegisterFatBinaryEnd(void**) {}
void __cudaUnregisterFatBinary(void**) {}
char __cudaInitModule(void**) { return 1; }
void __cudaRegisterFunction(void**, const char* hostFun, char*, const char* deviceName, int, uint3*, uint3*, dim3*,
                            dim3*, int*) {
    kernels()[hostFun] = deviceName;
}
unsigned __cudaPushCallConfiguration(dim3 gridDim, dim3 blockDim, size_t sharedMem, struct CUstream_st* stream) {
    cfg_stack().push_back(LaunchCfg{gridDim, blockDim, sharedMem, stream});
    return 0;
}
cudaError_t __cudaPopCallConfiguration(dim3* gridDim, dim3* blockDim, size_t* sharedMem, void* stream) {
    if (cfg_stack().empty()) return cudaErrorInvalidConfiguration;
    const LaunchCfg c = cfg_stack().back();
    cfg_stack().pop_back();
    *gridDim = c.grid;
    *blockDim = c.block;
    *sharedMem = c.shmem;
    *static_cast<void**>(stream) = c.stream;
    return cudaSuccess;
}
cudaError_t __cudaGetKernel(cudaKernel_t* kernel, const void* fun) {
    *kernel = reinterpret_cast<cudaKernel_t>(const_cast<void*>(fun));
    return cudaSuccess;
}
cudaError_t __cudaLaunchKernel(cudaKernel_t kernel, dim3 gridDim, dim3 blockDim, void** args, size_t, cudaStream_t) {
    auto it = kernels().find(reinterpret_cast<const void*>(kernel));
    if (it == kernels().end() || it->second.find("compute_matrix_kernel") == std::string::npos) {
        std::fprintf(stderr, "reference runner: unknown kernel launched\n");
        return cudaErrorInvalidDeviceFunction;
    }
    host_compute_matrix(gridDim, blockDim, args);
    ++g_launches;
    return cudaSuccess;
}

// ---- runtime API ------------------------------------------------------------------------
cudaError_t cudaSetDevice(int) { return cudaSuccess; }
cudaError_t cudaDeviceReset(void) { return cudaSuccess; }  // host stand-in: there is no device
cudaError_t cudaGetDeviceCount(int* n) {
    *n = 1;
    return cudaSuccess;
}
cudaError_t cudaGetDeviceProperties(cudaDeviceProp* prop, int) {
    std::memset(prop, 0, sizeof(*prop));
    std::snprintf(prop->name, sizeof prop->name, "host stand-in");
    return cudaSuccess;
}
cudaError_t cudaDriverGetVersion(int* v) {
    *v = 0;
    return cudaSuccess;
}
cudaError_t cudaRuntimeGetVersion(int* v) {
    *v = 0;
    return cudaSuccess;
}
cudaError_t cudaMemGetInfo(size_t* free_b, size_t* total_b) {
    *free_b = *total_b = size_t(1) << 34;
    return cudaSuccess;
}
cudaError_t cudaMalloc(void** p, size_t size) {
    *p = std::aligned_alloc(256, (size + 255) / 256 * 256 + 256);
    return *p ? cudaSuccess : cudaErrorMemoryAllocation;
}
cudaError_t cudaMallocPitch(void** p, size_t* pitch, size_t width, size_t height) {
    *pitch = (width + 511) / 512 * 512;
    return cudaMalloc(p, *pitch * (height ? height : 1));
}
cudaError_t cudaHostAlloc(void** p, size_t size, unsigned int) { return cudaMalloc(p, size); }
cudaError_t cudaFree(void* p) {
    std::free(p);
    return cudaSuccess;
}
cudaError_t cudaFreeHost(void* p) {
    std::free(p);
    return cudaSuccess;
}
cudaError_t cudaMemcpy(void* dst, const void* src, size_t count, cudaMemcpyKind) {
    std::memcpy(dst, src, count);
    return cudaSuccess;
}
cudaError_t cudaMemcpy2D(void* dst, size_t dpitch, const void* src, size_t spitch, size_t width, size_t height,
                         cudaMemcpyKind) {
    for (size_t r = 0; r < height; ++r)
        std::memcpy(static_cast<char*>(dst) + r * dpitch, static_cast<const char*>(src) + r * spitch, width);
    return cudaSuccess;
}
cudaError_t cudaMemset(void* p, int value, size_t count) {
    std::memset(p, value, count);
    return cudaSuccess;
}

// ---- cuBLAS ---------------------------------------------------------------------------
struct cublasContext {
    int unused;
};
cublasStatus_t cublasCreate_v2(cublasHandle_t* handle) {
    *handle = new cublasContext();
    return CUBLAS_STATUS_SUCCESS;
}
cublasStatus_t cublasDestroy_v2(cublasHandle_t handle) {
    delete handle;
    return CUBLAS_STATUS_SUCCESS;
}
// C = alpha op(A) op(B) + beta C, column-major
cublasStatus_t cublasCgemm_v2(cublasHandle_t, cublasOperation_t ta, cublasOperation_t tb, int m, int n, int k,
                              const cuComplex* alpha, const cuComplex* A, int lda, const cuComplex* B, int ldb,
                              const cuComplex* beta, cuComplex* C, int ldc) {
    auto get = [](const cuComplex* M, int ld, cublasOperation_t op, int i, int j) {
        // element (i, j) of op(M)
        if (op == CUBLAS_OP_N) return M[static_cast<size_t>(j) * ld + i];
        cuComplex v = M[static_cast<size_t>(i) * ld + j];
        if (op == CUBLAS_OP_C) v.y = -v.y;
        return v;
    };
    for (int j = 0; j < n; ++j)
        for (int i = 0; i < m; ++i) {
            double sr = 0.0, si = 0.0;
            for (int l = 0; l < k; ++l) {
                const cuComplex a = get(A, lda, ta, i, l), b = get(B, ldb, tb, l, j);
                sr += static_cast<double>(a.x) * b.x - static_cast<double>(a.y) * b.y;
                si += static_cast<double>(a.x) * b.y + static_cast<double>(a.y) * b.x;
            }
            cuComplex& c = C[static_cast<size_t>(j) * ldc + i];
            const double cr = c.x, ci = c.y;
            const double rr = alpha->x * sr - alpha->y * si + beta->x * cr - beta->y * ci;
            const double ri = alpha->x * si + alpha->y * sr + beta->x * ci + beta->y * cr;
            c.x = static_cast<float>(rr);
            c.y = static_cast<float>(ri);
        }
    return CUBLAS_STATUS_SUCCESS;
}

int ref_kernel_launches(void) { return g_launches; }

}  // extern "C"
