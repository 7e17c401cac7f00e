// Greedy sparse recovery on the device: orthogonal matching pursuit
// (+regularization/+algorithms/+greedy/omp.m:161-200) and compressive sampling
// matching pursuit (+regularization/+algorithms/+greedy/cosamp.m:174-272).
//
// Per iteration OMP
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
//
// CoSaMP shares a)-c): the 2s largest proxy entries are 2s argmax passes that
// mask each winner, the union's new columns come from the same column kernel,
// and the least squares on the union is a Gram matrix (FP32 products, FP64
// sums) solved by a pivoted Cholesky on the host in FP64 with two steps of
// iterative refinement against device residuals.  Pruning and the support bookkeeping
// (at most 3s integers) stay on the host.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <complex>
#include <string>
#include <vector>

#include "cui_internal.cuh"

namespace cui {
namespace {

constexpr int kOmpThreads = 256;
constexpr int kOmpBlocks = 256;  // partial sums / maxima per reduction (fixed: deterministic order)
constexpr int kCosampMaxSparsity = 512;  // the host factorises Gram matrices of up to 3s x 3s
// relative pivot below which a column counts as dependent: the Gram matrix sums FP32 products
constexpr double kCosampPivotTol = 1e-6;

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

__device__ __forceinline__ float score(float2 v) { return v.x * v.x + v.y * v.y; }
__device__ __forceinline__ float score(float v) { return v; }

// pass 1: per block the largest score (|g|^2 of a complex entry, or the value of a
// real one) and its (smallest) index
template <typename T>
__global__ void argmax_part_kernel(const T* __restrict__ g, int64_t n, float* __restrict__ bval,
                                   int64_t* __restrict__ bidx) {
    __shared__ float sv[kOmpThreads];
    __shared__ int64_t si[kOmpThreads];
    float best = -1.f;
    int64_t bi = n;
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        keep_max(best, bi, score(g[i]), i);
    }
    block_argmax(best, bi, sv, si);
    if (threadIdx.x == 0) { bval[blockIdx.x] = sv[0]; bidx[blockIdx.x] = si[0]; }
}

// pass 2: one block over the partials -> atom; with `mask` the winner's score is
// set below every real score so that the next pass finds the runner-up
__global__ void argmax_final_kernel(const float* __restrict__ bval, const int64_t* __restrict__ bidx, int nb,
                                    int64_t* __restrict__ atom, float* __restrict__ mask, int64_t n) {
    __shared__ float sv[kOmpThreads];
    __shared__ int64_t si[kOmpThreads];
    float best = -1.f;
    int64_t bi = INT64_MAX;
    for (int i = threadIdx.x; i < nb; i += blockDim.x) keep_max(best, bi, bval[i], bidx[i]);
    block_argmax(best, bi, sv, si);
    if (threadIdx.x == 0) {
        *atom = si[0];
        if (mask && si[0] < n) mask[si[0]] = -2.f;  // si[0] == n: no finite score left
    }
}

struct ColumnArgs {
    const float2* table;  // stored table, or null: entries generated (streamed and generated 3D tables)
    TableGen gen;
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
    const int64_t* atom;  // device: the grid points whose columns are extracted (blockIdx.y)
    const int* slot;      // device: destination column of each (NULL: column blockIdx.y)
    float2* col;          // columns of n_obs values, leading dimension n_obs
};

// col[row] = Phi[row, k] = p_in[s, k] * sum_a pref[m][fl, a] * h(f_s; o(k, act_a), z_k)
// with the lateral offsets o = (ix + (Ex-1-ex) ppx, iy + (Ey-1-ey) ppy) of the
// forward kernels' table rows.
__global__ void column_kernel(const ColumnArgs a) {
    const int64_t k = a.atom[blockIdx.y];
    float2* col = a.col + static_cast<int64_t>(a.slot ? a.slot[blockIdx.y] : blockIdx.y) * a.n_obs;
    if (k < 0 || k >= a.P) {  // no atom (a proxy without finite entries): a zero column
        for (int64_t row = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; row < a.n_obs;
             row += static_cast<int64_t>(gridDim.x) * blockDim.x)
            col[row] = make_float2(0.f, 0.f);
        return;
    }
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
            const float2 h = a.table ? a.table[((static_cast<int64_t>(f) * a.Nz + iz) * a.Noy + oy) * a.Nox + ox]
                                     : gen_entry(a.gen, gen_row(a.gen, f, iz, oy), ox);
            const float2 w = pref[static_cast<int64_t>(ia) * nf];
            acc.x = fmaf(w.x, h.x, fmaf(-w.y, h.y, acc.x));
            acc.y = fmaf(w.x, h.y, fmaf(w.y, h.x, acc.y));
        }
        const float2 pv = a.p_in[static_cast<int64_t>(s) * a.P + k];
        col[row] = make_float2(pv.x * acc.x - pv.y * acc.y, pv.x * acc.y + pv.y * acc.x);
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

// G[i][j] += sum_r conj(c_i[r]) c_j[r] for the column pointers c_0..c_{K-1}, over
// 16 x 16 tiles (ti <= tj) of the upper triangle: grid (row blocks, tile pairs).
// Products and sums within a 128-row chunk in FP32, chunks summed in FP64;
// part[(pair, row block)][ty][tx] receives a row block's sums.
constexpr int kGramTile = 16, kGramRows = 128;
__global__ void __launch_bounds__(256) gram_part_kernel(const float2* const* __restrict__ colp, int K, int64_t n,
                                                        double2* __restrict__ part) {
    __shared__ float2 si[kGramRows][kGramTile + 1];
    __shared__ float2 sj[kGramRows][kGramTile + 1];
    // tile pair (ti, tj), ti <= tj, from the linear index over the upper triangle
    const int T = (K + kGramTile - 1) / kGramTile;
    int ti = 0, rem = blockIdx.y;
    while (rem >= T - ti) { rem -= T - ti; ++ti; }
    const int tj = ti + rem;
    const int tx = threadIdx.x % kGramTile, ty = threadIdx.x / kGramTile;
    double2 acc = make_double2(0.0, 0.0);
    const int64_t n_chunks = (n + kGramRows - 1) / kGramRows;
    for (int64_t ch = blockIdx.x; ch < n_chunks; ch += gridDim.x) {
        const int64_t r0 = ch * kGramRows;
        __syncthreads();
        for (int idx = threadIdx.x; idx < kGramRows * kGramTile; idx += blockDim.x) {
            const int c = idx / kGramRows, r = idx - c * kGramRows;
            const int ci = ti * kGramTile + c, cj = tj * kGramTile + c;
            const bool in = r0 + r < n;
            si[r][c] = (in && ci < K) ? colp[ci][r0 + r] : make_float2(0.f, 0.f);
            sj[r][c] = (in && cj < K) ? colp[cj][r0 + r] : make_float2(0.f, 0.f);
        }
        __syncthreads();
        float2 s = make_float2(0.f, 0.f);
#pragma unroll 8
        for (int r = 0; r < kGramRows; ++r) {
            const float2 a = si[r][ty], b = sj[r][tx];
            s.x = fmaf(a.x, b.x, fmaf(a.y, b.y, s.x));
            s.y = fmaf(a.x, b.y, fmaf(-a.y, b.x, s.y));
        }
        acc.x += s.x;
        acc.y += s.y;
    }
    part[(static_cast<int64_t>(blockIdx.y) * gridDim.x + blockIdx.x) * 256 + threadIdx.x] = acc;
}

// G (K x K, row-major, upper triangle) = sum over row blocks, fixed order, FP64
__global__ void gram_final_kernel(const double2* __restrict__ part, int K, int nbx, double2* __restrict__ G) {
    const int T = (K + kGramTile - 1) / kGramTile;
    int ti = 0, rem = blockIdx.x;
    while (rem >= T - ti) { rem -= T - ti; ++ti; }
    const int tj = ti + rem;
    const int i = ti * kGramTile + threadIdx.x / kGramTile, j = tj * kGramTile + threadIdx.x % kGramTile;
    double2 s = make_double2(0.0, 0.0);
    for (int b = 0; b < nbx; ++b) {
        const double2 v = part[(static_cast<int64_t>(blockIdx.x) * nbx + b) * 256 + threadIdx.x];
        s.x += v.x;
        s.y += v.y;
    }
    if (i < K && j < K && i <= j) G[static_cast<int64_t>(i) * K + j] = s;
}

// part[j][blk] = partial of <c_j, v> for the column pointers c_j (grid: blocks x nq)
__global__ void dots_list_part_kernel(const float2* const* __restrict__ colp, const float2* __restrict__ v, int64_t n,
                                      float2* __restrict__ part) {
    const float2* q = colp[blockIdx.y];
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
    if (threadIdx.x == 0) part[static_cast<int64_t>(blockIdx.y) * gridDim.x + blockIdx.x] = sh[0];
}

// out = v - sum_j c[j] * col_j  (out may alias v)
__global__ void subtract_list_kernel(const float2* const* __restrict__ colp, const float2* __restrict__ c, int nq,
                                     const float2* v, float2* out, int64_t n) {
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        float2 x = v[i];
        for (int j = 0; j < nq; ++j) {
            const float2 q = colp[j][i], w = c[j];
            x.x -= w.x * q.x - w.y * q.y;
            x.y -= w.x * q.y + w.y * q.x;
        }
        out[i] = x;
    }
}

// |g|^2 of every proxy entry
__global__ void mag2_kernel(const float2* __restrict__ g, int64_t n, float* __restrict__ m) {
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const float2 v = g[i];
        m[i] = v.x * v.x + v.y * v.y;
    }
}

ColumnArgs column_args(const Plan& p) {
    ColumnArgs ca{};
    ca.table = p.table; ca.gen = p.gen; ca.p_in = p.p_in; ca.slot_f = p.slot_f; ca.row_slot = p.row_slot; ca.row_mix = p.row_mix;
    ca.row_fl = p.row_fl; ca.mix_nact = p.mix_nact; ca.mix_nf = p.mix_nf; ca.mix_act_off = p.mix_act_off;
    ca.mix_pref_off = p.mix_pref_off; ca.act = p.act; ca.pref = p.pref;
    ca.Nx = p.Nx; ca.Ny = p.Ny; ca.Nz = p.Nz; ca.Ex = p.Ex; ca.Ey = p.Ey; ca.ppx = p.ppx; ca.ppy = p.ppy;
    ca.Nox = p.Nox; ca.Noy = p.Noy; ca.P = p.P; ca.n_obs = p.n_obs; ca.atom = nullptr; ca.slot = nullptr;
    ca.col = nullptr;
    return ca;
}

// Least squares through the normal equations G c = b (G = A^H A, Hermitian positive
// semidefinite, upper triangle given row-major), solved in FP64 by a Cholesky factorisation with
// diagonal pivoting.  Pivots that fall below tol x the largest diagonal mark columns that are
// linear combinations of the ones already taken (to the accuracy of a Gram matrix summed from
// FP32 products); they are left out with coefficient 0, which is the basic solution a
// column-pivoted QR -- MATLAB's A \ y of cosamp.m:244 -- gives for a rank-deficient A.
struct PivotedCholesky {
    int K = 0, r = 0;                      // size, numerical rank
    std::vector<int> perm;                 // perm[j]: column taken as pivot j
    std::vector<std::complex<double>> A;   // K x K: lower factor in columns 0..r-1

    void factor(const std::vector<std::complex<double>>& Gup, int n, double tol) {
        K = n;
        r = 0;
        perm.resize(K);
        A.assign(static_cast<size_t>(K) * K, {});
        double dmax = 0.0;
        for (int i = 0; i < K; ++i) {
            perm[i] = i;
            for (int j = i; j < K; ++j) {
                A[static_cast<size_t>(i) * K + j] = Gup[static_cast<size_t>(i) * K + j];
                A[static_cast<size_t>(j) * K + i] = std::conj(Gup[static_cast<size_t>(i) * K + j]);
            }
            dmax = std::max(dmax, Gup[static_cast<size_t>(i) * K + i].real());
        }
        auto at = [&](int i, int j) -> std::complex<double>& { return A[static_cast<size_t>(i) * K + j]; };
        for (int j = 0; j < K; ++j) {
            int p = j;
            for (int i = j + 1; i < K; ++i)
                if (at(i, i).real() > at(p, p).real()) p = i;
            if (!(at(p, p).real() > tol * dmax)) break;
            if (p != j) {  // symmetric swap of rows and columns j and p
                for (int c = 0; c < K; ++c) std::swap(at(j, c), at(p, c));
                for (int c = 0; c < K; ++c) std::swap(at(c, j), at(c, p));
                std::swap(perm[j], perm[p]);
            }
            const double l = std::sqrt(at(j, j).real());
            at(j, j) = l;
            for (int i = j + 1; i < K; ++i) at(i, j) /= l;
            for (int i = j + 1; i < K; ++i)
                for (int c = j + 1; c <= i; ++c) at(i, c) -= at(i, j) * std::conj(at(c, j));
            for (int i = j + 1; i < K; ++i)  // keep the trailing block Hermitian for the next pivot search
                for (int c = i + 1; c < K; ++c) at(i, c) = std::conj(at(c, i));
            r = j + 1;
        }
    }

    // x: right-hand side b on entry, coefficients c on return (0 for columns left out)
    void solve(std::vector<std::complex<double>>& x) const {
        std::vector<std::complex<double>> z(r);
        for (int i = 0; i < r; ++i) {  // L z = P b
            std::complex<double> v = x[perm[i]];
            for (int k = 0; k < i; ++k) v -= A[static_cast<size_t>(i) * K + k] * z[k];
            z[i] = v / A[static_cast<size_t>(i) * K + i].real();
        }
        for (int i = r - 1; i >= 0; --i) {  // L^H w = z
            std::complex<double> v = z[i];
            for (int k = i + 1; k < r; ++k) v -= std::conj(A[static_cast<size_t>(k) * K + i]) * z[k];
            z[i] = v / A[static_cast<size_t>(i) * K + i].real();
        }
        std::fill(x.begin(), x.end(), std::complex<double>());
        for (int i = 0; i < r; ++i) x[perm[i]] = z[i];
    }
};

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
    const cui::NvtxRange nvtx_range("cui_born_omp");
    using namespace cui;
    if (!plan || !y || !atoms || !coefficients || !n_atoms) return set_error(CUI_ERR_INVALID_ARG, "NULL argument");
    Plan& p = plan->p;
    const int64_t n = p.n_obs, P = p.P;
    const int kmax = static_cast<int>(std::min<int64_t>(n_atoms_max, n));
    if (kmax < 1) return set_error(CUI_ERR_INVALID_ARG, "n_atoms_max must be >= 1");
    const DeviceGuard dev_guard(p.device);
    cudaError_t e = dev_guard.err;
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
    ColumnArgs ca = column_args(p);
    ca.atom = w.atom;
    ca.col = w.a;
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
            argmax_part_kernel<float2><<<kOmpBlocks, kOmpThreads, 0, st>>>(w.g, P, w.bval, w.bidx);
            argmax_final_kernel<<<1, kOmpThreads, 0, st>>>(w.bval, w.bidx, kOmpBlocks, w.atom, nullptr, P);
            // c) the column of Phi at the atom
            column_kernel<<<dim3(nbe, 1), 256, 0, st>>>(ca);
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
            if (at < 0 || at >= P) {
                status = set_error(CUI_ERR_NUMERIC, "omp: the adjoint of the residual has no finite entry");
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

extern "C" cui_status cui_born_cosamp(cui_born_plan* plan, const cui_complex32* y, int32_t sparsity, int32_t n_iter_max,
                                      float rel_rmse, int64_t* atoms, cui_complex32* coefficients,
                                      float* rel_residuals, int32_t* n_iter, void* stream) {
    const cui::NvtxRange nvtx_range("cui_born_cosamp");
    using namespace cui;
    if (!plan || !y || !atoms || !coefficients || !n_iter) return set_error(CUI_ERR_INVALID_ARG, "NULL argument");
    *n_iter = 0;
    Plan& p = plan->p;
    const int64_t n = p.n_obs, P = p.P;
    const int s = sparsity;
    if (s < 1 || s > kCosampMaxSparsity)
        return set_error(CUI_ERR_INVALID_ARG, "sparsity must be in [1, " + std::to_string(kCosampMaxSparsity) + "]");
    if (2 * static_cast<int64_t>(s) > P) return set_error(CUI_ERR_INVALID_ARG, "2 * sparsity exceeds the grid points");
    if (3 * static_cast<int64_t>(s) > n)
        return set_error(CUI_ERR_INVALID_ARG, "3 * sparsity exceeds the observations (under-determined least squares)");
    const int iters = static_cast<int>(std::min<int64_t>(n_iter_max, n));
    if (iters < 1) return set_error(CUI_ERR_INVALID_ARG, "n_iter_max must be >= 1");
    const DeviceGuard dev_guard(p.device);
    cudaError_t e = dev_guard.err;
    if (e != cudaSuccess) return check_cuda(e, "cudaSetDevice");
    cudaStream_t st = static_cast<cudaStream_t>(stream);

    const int n_sel = 2 * s, n_slots = 3 * s, Kmax = n_slots + 1;
    const int Tmax = (Kmax + kGramTile - 1) / kGramTile, pairs_max = Tmax * (Tmax + 1) / 2;
    const int64_t n_chunks = (n + kGramRows - 1) / kGramRows;
    const int nb1 = static_cast<int>(std::min<int64_t>((n + kOmpThreads - 1) / kOmpThreads, kOmpBlocks));
    const int nbe = static_cast<int>(std::min<int64_t>((n + 255) / 256, 152 * 8));
    const int nbp = static_cast<int>(std::min<int64_t>((P + 255) / 256, 152 * 8));
    auto gram_blocks = [&](int pairs) {
        return static_cast<int>(std::max<int64_t>(1, std::min<int64_t>({(1216 + pairs - 1) / pairs, n_chunks, 304})));
    };
    // pairs * gram_blocks(pairs) <= 1216 + pairs - 1 for every pairs <= pairs_max
    const size_t gpart_elems = (1216 + static_cast<size_t>(pairs_max)) * 256;
    // scratch for the whole solve, allocated per call
    const size_t bytes = sizeof(float2) * (P + n * (static_cast<size_t>(n_slots) + 2) + Kmax + static_cast<size_t>(Kmax) * nb1) +
                         sizeof(float) * (P + kOmpBlocks) + sizeof(int64_t) * (kOmpBlocks + 2 * n_sel) +
                         sizeof(int) * n_sel + sizeof(float2*) * Kmax +
                         sizeof(double2) * (static_cast<size_t>(Kmax) * Kmax + gpart_elems) +
                         16 * 32;
    char* base = nullptr;
    if ((e = cudaMalloc(&base, bytes)) != cudaSuccess) return check_cuda(e, "cudaMalloc (cosamp scratch)");
    char* cur = base;
    auto take = [&](size_t b) { char* q = cur; cur += (b + 15) / 16 * 16; return q; };
    float2* g = reinterpret_cast<float2*>(take(sizeof(float2) * P));
    float* m = reinterpret_cast<float*>(take(sizeof(float) * P));
    float2* r = reinterpret_cast<float2*>(take(sizeof(float2) * n));
    float2* rt = reinterpret_cast<float2*>(take(sizeof(float2) * n));
    float2* cols = reinterpret_cast<float2*>(take(sizeof(float2) * n * n_slots));
    float2* coef = reinterpret_cast<float2*>(take(sizeof(float2) * Kmax));
    float2* dpart = reinterpret_cast<float2*>(take(sizeof(float2) * Kmax * nb1));
    float* bval = reinterpret_cast<float*>(take(sizeof(float) * kOmpBlocks));
    int64_t* bidx = reinterpret_cast<int64_t*>(take(sizeof(int64_t) * kOmpBlocks));
    int64_t* ident = reinterpret_cast<int64_t*>(take(sizeof(int64_t) * n_sel));
    int64_t* new_atoms = reinterpret_cast<int64_t*>(take(sizeof(int64_t) * n_sel));
    int* new_slots = reinterpret_cast<int*>(take(sizeof(int) * n_sel));
    const float2** colp = reinterpret_cast<const float2**>(take(sizeof(float2*) * Kmax));
    double2* G = reinterpret_cast<double2*>(take(sizeof(double2) * Kmax * Kmax));
    double2* gpart = reinterpret_cast<double2*>(take(sizeof(double2) * gpart_elems));
    float2* dout = reinterpret_cast<float2*>(take(sizeof(float2) * 2));
    const float2* yd = reinterpret_cast<const float2*>(y);
    ColumnArgs ca = column_args(p);
    ca.atom = new_atoms;
    ca.slot = new_slots;
    ca.col = cols;

    cui_status status = CUI_OK;
    std::vector<int64_t> support;                 // current atoms, the reference's order
    std::vector<std::complex<double>> kept;       // their coefficients
    std::vector<int> slot_of_support;
    std::vector<int> free_slots;
    for (int i = n_slots - 1; i >= 0; --i) free_slots.push_back(i);
    std::vector<int64_t> ident_h(n_sel);
    std::vector<const float2*> colp_h(Kmax);
    std::vector<double2> G_h;
    std::vector<float2> c_h(Kmax), d_h(Kmax);
    auto cuda_ok = [&](cudaError_t err, const char* what) {
        if (err == cudaSuccess) return true;
        status = check_cuda(err, what);
        return false;
    };
    // <colp[j], v> for j < k into d_h (host); the sums pass through `coef`, after its
    // readers in stream order
    auto dots_list = [&](int k, const float2* v) {
        dots_list_part_kernel<<<dim3(nb1, k), kOmpThreads, 0, st>>>(colp, v, n, dpart);
        dots_final_kernel<<<(k + 127) / 128, 128, 0, st>>>(dpart, nb1, k, coef, 0);
        count_launch(2);
        return cuda_ok(cudaMemcpyAsync(d_h.data(), coef, sizeof(float2) * k, cudaMemcpyDeviceToHost, st), "cosamp dots") &&
               cuda_ok(cudaStreamSynchronize(st), "cosamp dots");
    };
    // r_out = y - sum_j c[j] colp[j], c from the host
    auto residual = [&](int k, const std::vector<std::complex<double>>& c, float2* r_out) {
        for (int j = 0; j < k; ++j) c_h[j] = make_float2(static_cast<float>(c[j].real()), static_cast<float>(c[j].imag()));
        if (!cuda_ok(cudaMemcpyAsync(coef, c_h.data(), sizeof(float2) * k, cudaMemcpyHostToDevice, st), "cosamp coef"))
            return false;
        subtract_list_kernel<<<nbe, 256, 0, st>>>(colp, coef, k, yd, r_out, n);
        count_launch();
        return true;
    };

    if (cuda_ok(cudaMemcpyAsync(r, yd, sizeof(float2) * n, cudaMemcpyDeviceToDevice, st), "cosamp init")) {
        float2 yy{};
        dots_part_kernel<<<dim3(nb1, 1), kOmpThreads, 0, st>>>(r, n, r, n, dpart);
        dots_final_kernel<<<1, 128, 0, st>>>(dpart, nb1, 1, dout, 0);
        count_launch(2);
        if (cuda_ok(cudaMemcpyAsync(&yy, dout, sizeof(float2), cudaMemcpyDeviceToHost, st), "cosamp init") &&
            cuda_ok(cudaStreamSynchronize(st), "cosamp init")) {
            const double y_norm = std::sqrt(std::max(static_cast<double>(yy.x), 0.0));
            for (int it = 0; it < iters && status == CUI_OK; ++it) {
                // 1) proxy Phi^H r and its 2s largest magnitudes (stable: ties to the smaller index)
                if ((status = adjoint_device(&p, r, n, 1, g, P, st)) != CUI_OK) break;
                mag2_kernel<<<nbp, 256, 0, st>>>(g, P, m);
                for (int j = 0; j < n_sel; ++j) {
                    argmax_part_kernel<float><<<kOmpBlocks, kOmpThreads, 0, st>>>(m, P, bval, bidx);
                    argmax_final_kernel<<<1, kOmpThreads, 0, st>>>(bval, bidx, kOmpBlocks, ident + j, m, P);
                }
                count_launch(1 + 2 * n_sel);
                if (!cuda_ok(cudaMemcpyAsync(ident_h.data(), ident, sizeof(int64_t) * n_sel, cudaMemcpyDeviceToHost, st),
                             "cosamp select") ||
                    !cuda_ok(cudaStreamSynchronize(st), "cosamp select"))
                    break;
                bool finite = true;
                for (int j = 0; j < n_sel; ++j) finite = finite && ident_h[j] >= 0 && ident_h[j] < P;
                if (!finite) {
                    status = set_error(CUI_ERR_NUMERIC, "cosamp: the proxy has fewer than 2s finite entries");
                    break;
                }
                // 2) union with the support, ascending; columns of the new atoms into free slots
                std::vector<std::pair<int64_t, int>> uni;  // (atom, slot)
                for (size_t i = 0; i < support.size(); ++i) uni.emplace_back(support[i], slot_of_support[i]);
                std::vector<int64_t> na;
                std::vector<int> ns;
                for (int j = 0; j < n_sel; ++j) {
                    const int64_t a = ident_h[j];
                    bool have = false;
                    for (const auto& u : uni) have = have || u.first == a;
                    if (have) continue;
                    const int sl = free_slots.back();
                    free_slots.pop_back();
                    uni.emplace_back(a, sl);
                    na.push_back(a);
                    ns.push_back(sl);
                }
                std::sort(uni.begin(), uni.end());
                const int k = static_cast<int>(uni.size()), K = k + 1;
                if (!na.empty()) {
                    if (!cuda_ok(cudaMemcpyAsync(new_atoms, na.data(), sizeof(int64_t) * na.size(), cudaMemcpyHostToDevice, st),
                                 "cosamp columns") ||
                        !cuda_ok(cudaMemcpyAsync(new_slots, ns.data(), sizeof(int) * ns.size(), cudaMemcpyHostToDevice, st),
                                 "cosamp columns"))
                        break;
                    column_kernel<<<dim3(nbe, static_cast<unsigned>(na.size())), 256, 0, st>>>(ca);
                    count_launch();
                }
                // 3) least squares A \ y on the union: Gram matrix [A y]^H [A y] on the device
                for (int i = 0; i < k; ++i) colp_h[i] = cols + static_cast<int64_t>(uni[i].second) * n;
                colp_h[k] = yd;
                if (!cuda_ok(cudaMemcpyAsync(colp, colp_h.data(), sizeof(float2*) * K, cudaMemcpyHostToDevice, st),
                             "cosamp gram"))
                    break;
                const int T = (K + kGramTile - 1) / kGramTile, pairs = T * (T + 1) / 2, nbx = gram_blocks(pairs);
                gram_part_kernel<<<dim3(nbx, pairs), 256, 0, st>>>(colp, K, n, gpart);
                gram_final_kernel<<<pairs, 256, 0, st>>>(gpart, K, nbx, G);
                count_launch(2);
                G_h.resize(static_cast<size_t>(K) * K);
                if (!cuda_ok(cudaMemcpyAsync(G_h.data(), G, sizeof(double2) * K * K, cudaMemcpyDeviceToHost, st),
                             "cosamp gram") ||
                    !cuda_ok(cudaStreamSynchronize(st), "cosamp gram"))
                    break;
                std::vector<std::complex<double>> U(static_cast<size_t>(k) * k), c(k);
                for (int i = 0; i < k; ++i) {
                    for (int j = i; j < k; ++j)
                        U[static_cast<size_t>(i) * k + j] = {G_h[static_cast<size_t>(i) * K + j].x, G_h[static_cast<size_t>(i) * K + j].y};
                    c[i] = {G_h[static_cast<size_t>(i) * K + k].x, G_h[static_cast<size_t>(i) * K + k].y};
                }
                PivotedCholesky pc;
                pc.factor(U, k, kCosampPivotTol);
                pc.solve(c);
                // two steps of iterative refinement: c += (A^H A)^{-1} A^H (y - A c)
                bool ok = true;
                for (int ref = 0; ref < 2 && ok; ++ref) {
                    ok = residual(k, c, rt) && dots_list(k, rt);
                    if (!ok) break;
                    std::vector<std::complex<double>> d(k);
                    for (int i = 0; i < k; ++i) d[i] = {d_h[i].x, d_h[i].y};
                    pc.solve(d);
                    for (int i = 0; i < k; ++i) c[i] += d[i];
                }
                if (!ok) break;
                // 4) prune to the s largest |c| (stable descending over the ascending union)
                std::vector<int> order(k);
                for (int i = 0; i < k; ++i) order[i] = i;
                std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return std::abs(c[a]) > std::abs(c[b]); });
                support.assign(s, 0);
                slot_of_support.assign(s, 0);
                kept.assign(s, {});
                std::vector<char> keep(k, 0);
                for (int i = 0; i < s; ++i) {
                    support[i] = uni[order[i]].first;
                    slot_of_support[i] = uni[order[i]].second;
                    kept[i] = c[order[i]];
                    keep[order[i]] = 1;
                }
                for (int i = 0; i < k; ++i)
                    if (!keep[i]) free_slots.push_back(uni[i].second);
                // 5) residual with the pruned coefficients (not refitted) and its relative norm
                for (int i = 0; i < s; ++i) colp_h[i] = cols + static_cast<int64_t>(slot_of_support[i]) * n;
                if (!cuda_ok(cudaMemcpyAsync(colp, colp_h.data(), sizeof(float2*) * s, cudaMemcpyHostToDevice, st),
                             "cosamp residual") ||
                    !residual(s, kept, r))
                    break;
                dots_part_kernel<<<dim3(nb1, 1), kOmpThreads, 0, st>>>(r, n, r, n, dpart);
                dots_final_kernel<<<1, 128, 0, st>>>(dpart, nb1, 1, dout, 0);
                count_launch(2);
                float2 rr{};
                if (!cuda_ok(cudaMemcpyAsync(&rr, dout, sizeof(float2), cudaMemcpyDeviceToHost, st), "cosamp residual") ||
                    !cuda_ok(cudaStreamSynchronize(st), "cosamp residual"))
                    break;
                const float rel = y_norm > 0.0 ? static_cast<float>(std::sqrt(std::max(static_cast<double>(rr.x), 0.0)) / y_norm)
                                               : 0.f;
                if (rel_residuals) rel_residuals[it] = rel;
                *n_iter = it + 1;
                if (rel <= rel_rmse) break;  // cosamp.m:270
            }
        }
    }
    if (status == CUI_OK) {
        for (int i = 0; i < s; ++i) {
            atoms[i] = i < static_cast<int>(support.size()) ? support[i] : -1;
            const std::complex<double> v = i < static_cast<int>(kept.size()) ? kept[i] : std::complex<double>();
            coefficients[i].re = static_cast<float>(v.real());
            coefficients[i].im = static_cast<float>(v.imag());
        }
    } else {
        *n_iter = 0;
    }
    cudaStreamSynchronize(st);  // queued kernels may still read the scratch after an error
    cudaFree(base);
    return status;
}
