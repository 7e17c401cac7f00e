// Orthogonal matching pursuit on the device (+regularization/+algorithms/+greedy/omp.m:161-200).
//
// Per iteration k the reference
//   a) applies the adjoint to the residual            (omp.m:166-171)
//   b) selects the atom of largest magnitude          (:174)
//   c) extracts that column of the operator           (:177-185, a forward of a unit vector)
//   d) solves the normal equations on the atoms so far (:190-191)
//   e) recomputes the residual                         (:196-198)
// Here a) is cui_born_adjoint's path, b) a deterministic two-pass argmax, c) a
// direct evaluation of one column of Phi (sum over each row's active elements,
// no full forward apply), and d)-e) an orthonormal basis of the selected
// columns kept by classical Gram-Schmidt with one re-orthogonalisation: the
// residual of the least-squares fit is y minus its projection onto that basis,
// and the coefficients follow from the triangular factor at the end.  The host
// drives the iterations and reads one residual norm per iteration for the
// reference's stopping rule (relative RMSE, :215).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <complex>
#include <vector>

#include "cui_internal.cuh"

namespace cui {
namespace {

constexpr int kOmpThreads = 256;
constexpr int kOmpBlocks = 256;  // partial sums / maxima per reduction (fixed: deterministic order)

// keep (v, i) if it beats (bv, bi): larger value, ties to the smaller index (MATLAB's max)
__device__ __forceinline__ void keep_max(float& bv, int64_t& bi, float v, int64_t i) {
    if (v > bv || (v == bv && i < bi)) { bv = v; bi = i; }
}

__device__ void block_argmax(float best, int64_t bi, float* sv, int64_t* si) {
    sv[threadIdx.x] = best;
    si[threadIdx.x] = bi;
    __syncthreads();
    for (int off = blockDim.x / 2; off > 0; off >>= 1) {
        if (threadIdx.x < off) keep_max(sv[threadIdx.x], si[threadIdx.x], sv[threadIdx.x + off], si[threadIdx.x + off]);
        __syncthreads();
    }
}

// pass 1: per block the largest |g|^2 and its (smallest) index
__global__ void argmax_part_kernel(const float2* __restrict__ g, int64_t n, float* __restrict__ bval,
                                   int64_t* __restrict__ bidx) {
    __shared__ float sv[kOmpThreads];
    __shared__ int64_t si[kOmpThreads];
    float best = -1.f;
    int64_t bi = n;
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const float2 v = g[i];
        keep_max(best, bi, v.x * v.x + v.y * v.y, i);
    }
    block_argmax(best, bi, sv, si);
    if (threadIdx.x == 0) { bval[blockIdx.x] = sv[0]; bidx[blockIdx.x] = si[0]; }
}

// pass 2: one block over the partials -> atom
__global__ void argmax_final_kernel(const float* __restrict__ bval, const int64_t* __restrict__ bidx, int nb,
                                    int64_t* __restrict__ atom) {
    __shared__ float sv[kOmpThreads];
    __shared__ int64_t si[kOmpThreads];
    float best = -1.f;
    int64_t bi = INT64_MAX;
    for (int i = threadIdx.x; i < nb; i += blockDim.x) keep_max(best, bi, bval[i], bidx[i]);
    block_argmax(best, bi, sv, si);
    if (threadIdx.x == 0) *atom = si[0];
}

struct ColumnArgs {
    const float2* table;
    const float2* p_in;
    const int* slot_f;
    const int* row_slot;
    const int* row_mix;
    const int* row_fl;
    const int* mix_nact;
    const int* mix_nf;
    const int* mix_act_off;
    const int64_t* mix_pref_off;
    const int* act;
    const float2* pref;
    int Nx, Ny, Nz, Ex, Ey, ppx, ppy, Nox, Noy;
    int64_t P, n_obs;
    const int64_t* atom;  // device: the grid point whose column is extracted
    float2* col;          // [n_obs]
};

// col[row] = Phi[row, k] = p_in[s, k] * sum_a pref[m][fl, a] * h(f_s; o(k, act_a), z_k)
// with the lateral offsets o = (ix + (Ex-1-ex) ppx, iy + (Ey-1-ey) ppy) of the
// forward kernels' table rows.
__global__ void column_kernel(const ColumnArgs a) {
    const int64_t k = *a.atom;
    const int ix = static_cast<int>(k % a.Nx), iy = static_cast<int>((k / a.Nx) % a.Ny);
    const int iz = static_cast<int>(k / (static_cast<int64_t>(a.Nx) * a.Ny));
    for (int64_t row = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; row < a.n_obs;
         row += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const int s = a.row_slot[row], m = a.row_mix[row], fl = a.row_fl[row];
        const int f = a.slot_f[s];
        const int nact = a.mix_nact[m], nf = a.mix_nf[m];
        const int* act = a.act + a.mix_act_off[m];
        const float2* pref = a.pref + a.mix_pref_off[m] + fl;
        float2 acc = make_float2(0.f, 0.f);
        for (int ia = 0; ia < nact; ++ia) {
            const int e = act[ia];
            const int ey = e / a.Ex, ex = e - ey * a.Ex;
            const int ox = ix + (a.Ex - 1 - ex) * a.ppx, oy = iy + (a.Ey - 1 - ey) * a.ppy;
            const float2 h = a.table[((static_cast<int64_t>(f) * a.Nz + iz) * a.Noy + oy) * a.Nox + ox];
            const float2 w = pref[static_cast<int64_t>(ia) * nf];
            acc.x = fmaf(w.x, h.x, fmaf(-w.y, h.y, acc.x));
            acc.y = fmaf(w.x, h.y, fmaf(w.y, h.x, acc.y));
        }
        const float2 pv = a.p_in[static_cast<int64_t>(s) * a.P + k];
        a.col[row] = make_float2(pv.x * acc.x - pv.y * acc.y, pv.x * acc.y + pv.y * acc.x);
    }
}

// part[j][blk] = partial of sum_i conj(Q[j][i]) * v[i], j < nq  (grid: blocks x nq)
__global__ void dots_part_kernel(const float2* __restrict__ Q, int64_t ldq, const float2* __restrict__ v, int64_t n,
                                 float2* __restrict__ part) {
    const int j = blockIdx.y;
    const float2* q = Q + j * ldq;
    float2 s = make_float2(0.f, 0.f);
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const float2 a = q[i], b = v[i];
        s.x = fmaf(a.x, b.x, fmaf(a.y, b.y, s.x));
        s.y = fmaf(a.x, b.y, fmaf(-a.y, b.x, s.y));
    }
    __shared__ float2 sh[kOmpThreads];
    sh[threadIdx.x] = s;
    __syncthreads();
    for (int off = blockDim.x / 2; off > 0; off >>= 1) {
        if (threadIdx.x < off) {
            sh[threadIdx.x].x += sh[threadIdx.x + off].x;
            sh[threadIdx.x].y += sh[threadIdx.x + off].y;
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) part[static_cast<int64_t>(j) * gridDim.x + blockIdx.x] = sh[0];
}

// out[j] (+)= sum of the partials of dot j (one thread per dot, fixed order)
__global__ void dots_final_kernel(const float2* __restrict__ part, int nb, int nq, float2* __restrict__ out, int add) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= nq) return;
    float2 s = make_float2(0.f, 0.f);
    for (int b = 0; b < nb; ++b) {
        s.x += part[static_cast<int64_t>(j) * nb + b].x;
        s.y += part[static_cast<int64_t>(j) * nb + b].y;
    }
    if (add) { out[j].x += s.x; out[j].y += s.y; } else { out[j] = s; }
}

// v -= sum_j c[j] * Q[j]
__global__ void subtract_kernel(const float2* __restrict__ Q, int64_t ldq, const float2* __restrict__ c, int nq,
                                float2* __restrict__ v, int64_t n) {
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        float2 x = v[i];
        for (int j = 0; j < nq; ++j) {
            const float2 q = Q[j * ldq + i], w = c[j];
            x.x -= w.x * q.x - w.y * q.y;
            x.y -= w.x * q.y + w.y * q.x;
        }
        v[i] = x;
    }
}

// dst = v / ||v|| with ||v|| = sqrt(Re d), d = <v, v> (device); rkk = ||v||
__global__ void normalize_kernel(const float2* __restrict__ v, const float2* __restrict__ d, float2* __restrict__ dst,
                                 int64_t n, float2* __restrict__ rkk) {
    const float nrm = sqrtf(fmaxf(d->x, 0.f));
    const float inv = nrm > 0.f ? 1.f / nrm : 0.f;
    if (blockIdx.x == 0 && threadIdx.x == 0) *rkk = make_float2(nrm, 0.f);
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const float2 x = v[i];
        dst[i] = make_float2(x.x * inv, x.y * inv);
    }
}

struct OmpWork {
    float2 *g, *Q, *a, *r, *part, *c, *d, *R, *qy, *rr;
    float* bval;
    int64_t* bidx;
    int64_t* atom;
};

}  // namespace
}  // namespace cui

extern "C" cui_status cui_born_omp(cui_born_plan* plan, const cui_complex32* y, int32_t n_atoms_max, float rel_rmse,
                                   int64_t* atoms, cui_complex32* coefficients, float* rel_residuals,
                                   int32_t* n_atoms, void* stream) {
    using namespace cui;
    if (!plan || !y || !atoms || !coefficients || !n_atoms) return set_error(CUI_ERR_INVALID_ARG, "NULL argument");
    Plan& p = plan->p;
    const int64_t n = p.n_obs, P = p.P;
    const int kmax = static_cast<int>(std::min<int64_t>(n_atoms_max, n));
    if (kmax < 1) return set_error(CUI_ERR_INVALID_ARG, "n_atoms_max must be >= 1");
    cudaError_t e = cudaSetDevice(p.device);
    if (e != cudaSuccess) return check_cuda(e, "cudaSetDevice");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    // scratch for the whole solve, allocated per call (OMP is a host-driven loop with a
    // synchronisation per iteration, not a capturable entry point)
    OmpWork w{};
    const size_t bytes = sizeof(float2) * (P + static_cast<size_t>(n) * (kmax + 2) + static_cast<size_t>(kmax) * kOmpBlocks +
                                           3 * static_cast<size_t>(kmax) + static_cast<size_t>(kmax) * kmax + 4) +
                         (sizeof(float) + sizeof(int64_t)) * kOmpBlocks + sizeof(int64_t) + 16 * 16;
    char* base = nullptr;
    if ((e = cudaMalloc(&base, bytes)) != cudaSuccess) return check_cuda(e, "cudaMalloc (omp scratch)");
    char* cur = base;
    auto take = [&](size_t b) { char* q = cur; cur += (b + 15) / 16 * 16; return q; };
    w.g = reinterpret_cast<float2*>(take(sizeof(float2) * P));
    w.Q = reinterpret_cast<float2*>(take(sizeof(float2) * n * kmax));
    w.a = reinterpret_cast<float2*>(take(sizeof(float2) * n));
    w.r = reinterpret_cast<float2*>(take(sizeof(float2) * n));
    w.part = reinterpret_cast<float2*>(take(sizeof(float2) * kmax * kOmpBlocks));
    w.c = reinterpret_cast<float2*>(take(sizeof(float2) * kmax));
    w.d = reinterpret_cast<float2*>(take(sizeof(float2) * 2));
    w.R = reinterpret_cast<float2*>(take(sizeof(float2) * kmax * kmax));
    w.qy = reinterpret_cast<float2*>(take(sizeof(float2) * kmax));
    w.rr = reinterpret_cast<float2*>(take(sizeof(float2) * 2));
    w.bval = reinterpret_cast<float*>(take(sizeof(float) * kOmpBlocks));
    w.bidx = reinterpret_cast<int64_t*>(take(sizeof(int64_t) * kOmpBlocks));
    w.atom = reinterpret_cast<int64_t*>(take(sizeof(int64_t)));
    cui_status status = CUI_OK;
    auto fail = [&](cudaError_t err, const char* what) { status = check_cuda(err, what); };
    const int nb1 = static_cast<int>(std::min<int64_t>((n + kOmpThreads - 1) / kOmpThreads, kOmpBlocks));
    const int nbe = static_cast<int>(std::min<int64_t>((n + 255) / 256, 152 * 8));
    auto dots = [&](const float2* Qm, int nq, const float2* v, float2* out, int add) {
        dots_part_kernel<<<dim3(nb1, nq), kOmpThreads, 0, st>>>(Qm, n, v, n, w.part);
        dots_final_kernel<<<(nq + 127) / 128, 128, 0, st>>>(w.part, nb1, nq, out, add);
        count_launch(2);
    };
    ColumnArgs ca;
    ca.table = p.table; ca.p_in = p.p_in; ca.slot_f = p.slot_f; ca.row_slot = p.row_slot; ca.row_mix = p.row_mix;
    ca.row_fl = p.row_fl; ca.mix_nact = p.mix_nact; ca.mix_nf = p.mix_nf; ca.mix_act_off = p.mix_act_off;
    ca.mix_pref_off = p.mix_pref_off; ca.act = p.act; ca.pref = p.pref;
    ca.Nx = p.Nx; ca.Ny = p.Ny; ca.Nz = p.Nz; ca.Ex = p.Ex; ca.Ey = p.Ey; ca.ppx = p.ppx; ca.ppy = p.ppy;
    ca.Nox = p.Nox; ca.Noy = p.Noy; ca.P = P; ca.n_obs = n; ca.atom = w.atom; ca.col = w.a;
    const float2* yd = reinterpret_cast<const float2*>(y);

    std::vector<float2> qy_h(kmax), R_h(static_cast<size_t>(kmax) * kmax);
    int k = 0;
    do {
        if ((e = cudaMemcpyAsync(w.r, yd, sizeof(float2) * n, cudaMemcpyDeviceToDevice, st)) != cudaSuccess ||
            (e = cudaMemsetAsync(w.R, 0, sizeof(float2) * kmax * kmax, st)) != cudaSuccess) {
            fail(e, "omp init");
            break;
        }
        dots(w.r, 1, w.r, w.rr, 0);
        float2 yy;
        if ((e = cudaMemcpyAsync(&yy, w.rr, sizeof(float2), cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
            (e = cudaStreamSynchronize(st)) != cudaSuccess) {
            fail(e, "omp init");
            break;
        }
        const float y_norm = std::sqrt(std::max(yy.x, 0.f));
        for (k = 0; k < kmax;) {
            // a) adjoint of the residual, b) the atom of largest magnitude
            if ((status = adjoint_device(&p, w.r, n, 1, w.g, P, st)) != CUI_OK) break;
            argmax_part_kernel<<<kOmpBlocks, kOmpThreads, 0, st>>>(w.g, P, w.bval, w.bidx);
            argmax_final_kernel<<<1, kOmpThreads, 0, st>>>(w.bval, w.bidx, kOmpBlocks, w.atom);
            // c) the column of Phi at the atom
            column_kernel<<<nbe, 256, 0, st>>>(ca);
            count_launch(3);
            // d) orthogonalise against the basis, twice (CGS2): R[0:k, k] += Q^H a, a -= Q Q^H a
            for (int pass = 0; k > 0 && pass < 2; ++pass) {
                dots(w.Q, k, w.a, w.c, 0);
                subtract_kernel<<<nbe, 256, 0, st>>>(w.Q, n, w.c, k, w.a, n);
                // the partials of Q^H a are still in w.part: add them into column k of R
                dots_final_kernel<<<(k + 127) / 128, 128, 0, st>>>(w.part, nb1, k, w.R + static_cast<int64_t>(k) * kmax, 1);
                count_launch(2);
            }
            dots(w.a, 1, w.a, w.d, 0);
            normalize_kernel<<<nbe, 256, 0, st>>>(w.a, w.d, w.Q + static_cast<int64_t>(k) * n, n,
                                                  w.R + static_cast<int64_t>(k) * kmax + k);
            count_launch();
            // e) residual r -= <q_k, r> q_k ; qy_k = <q_k, y>
            dots(w.Q + static_cast<int64_t>(k) * n, 1, yd, w.qy + k, 0);
            dots(w.Q + static_cast<int64_t>(k) * n, 1, w.r, w.c, 0);
            subtract_kernel<<<nbe, 256, 0, st>>>(w.Q + static_cast<int64_t>(k) * n, n, w.c, 1, w.r, n);
            count_launch();
            dots(w.r, 1, w.r, w.rr, 0);
            float2 rr;
            int64_t at;
            if ((e = cudaMemcpyAsync(&rr, w.rr, sizeof(float2), cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
                (e = cudaMemcpyAsync(&at, w.atom, sizeof(int64_t), cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
                (e = cudaStreamSynchronize(st)) != cudaSuccess) {
                fail(e, "omp iteration");
                break;
            }
            atoms[k] = at;
            const float rel = (y_norm > 0.f) ? std::sqrt(std::max(rr.x, 0.f)) / y_norm : 0.f;
            if (rel_residuals) rel_residuals[k] = rel;
            ++k;
            if (rel <= rel_rmse) break;  // omp.m:215: stop once the relative RMSE is reached
        }
    } while (false);
    if (status == CUI_OK && k > 0) {
        // coefficients: R c = Q^H y, R upper triangular (column j at R + j*kmax), back-substituted in FP64
        e = cudaMemcpyAsync(R_h.data(), w.R, sizeof(float2) * kmax * kmax, cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaMemcpyAsync(qy_h.data(), w.qy, sizeof(float2) * kmax, cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) {
            fail(e, "omp coefficients");
        } else {
            std::vector<std::complex<double>> c(k);
            for (int i = k - 1; i >= 0; --i) {
                std::complex<double> s(qy_h[i].x, qy_h[i].y);
                for (int j = i + 1; j < k; ++j) {
                    const float2 rij = R_h[static_cast<size_t>(j) * kmax + i];
                    s -= std::complex<double>(rij.x, rij.y) * c[j];
                }
                const float2 rii = R_h[static_cast<size_t>(i) * kmax + i];
                c[i] = (rii.x != 0.f) ? s / std::complex<double>(rii.x, rii.y) : std::complex<double>(0.0, 0.0);
            }
            for (int i = 0; i < k; ++i) {
                coefficients[i].re = static_cast<float>(c[i].real());
                coefficients[i].im = static_cast<float>(c[i].imag());
            }
        }
    }
    *n_atoms = status == CUI_OK ? k : 0;
    cudaStreamSynchronize(st);  // the scratch may still be read by queued kernels after an error
    cudaFree(base);
    return status;
}
