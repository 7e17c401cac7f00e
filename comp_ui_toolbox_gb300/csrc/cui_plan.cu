// Plan construction, C-ABI entry points and error handling of libcui_born.
//
// cui_born_plan_create replaces the per-call table handling of the reference
// MEX gateway (+scattering/combined_quick_gpu.cu:203-850): it validates the
// operator description, converts the tables to FP32 in the device layout
// described in cui_internal.cuh and uploads them once.  The applies then
// move only their own inputs and outputs.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdlib>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "cui_internal.cuh"

namespace cui {

size_t loss_workspace_floats(int max_objects);

namespace {
thread_local std::string g_last_error;
thread_local int g_injected = 0;  // number of the allocation that the injector failed last, not yet reported
std::atomic<int64_t> g_launches{0};
constexpr size_t kPartBudget = size_t(1) << 30;  // bytes of partial-sum scratch a plan may hold
}  // namespace

cui_status set_error(cui_status s, const std::string& msg) {
    if (s != CUI_OK) g_last_error = msg;
    return s;
}

cui_status check_cuda(cudaError_t e, const char* what) {
    if (e == cudaSuccess) return CUI_OK;
    if (e == cudaErrorMemoryAllocation) {
        std::string msg = std::string(what) + ": " + cudaGetErrorString(e);
        if (g_injected) msg += " (injected allocation failure " + std::to_string(g_injected) + ", CUI_BORN_FAIL_ALLOC)";
        g_injected = 0;
        return set_error(CUI_ERR_OOM, msg);
    }
    return set_error(CUI_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

void count_launch(int n) { g_launches.fetch_add(n, std::memory_order_relaxed); }

// Fault injection for the cleanup paths (tests): with CUI_BORN_FAIL_ALLOC=N in the environment, the
// N-th device allocation of each plan (counted over its whole life: creation, precision switches)
// fails as an out-of-memory error would, before cudaMalloc is called.
bool injected_alloc_failure(Plan& p) {
    const char* env = std::getenv("CUI_BORN_FAIL_ALLOC");
    ++p.n_device_allocs;
    const bool fail = env && env[0] && std::atoi(env) == p.n_device_allocs;
    if (fail) g_injected = p.n_device_allocs;
    return fail;
}

namespace {

template <typename T>
cudaError_t dalloc(Plan& p, T** ptr, size_t n) {
    if (injected_alloc_failure(p)) return cudaErrorMemoryAllocation;
    void* v = nullptr;
    cudaError_t e = cudaMalloc(&v, std::max<size_t>(n, 1) * sizeof(T));
    if (e == cudaSuccess) {
        p.allocations.push_back(v);
        *ptr = static_cast<T*>(v);
    }
    return e;
}

template <typename T>
cudaError_t upload(Plan& p, T** ptr, const std::vector<T>& h) {
    cudaError_t e = dalloc(p, ptr, h.size());
    if (e != cudaSuccess || h.empty()) return e;
    return cudaMemcpy(*ptr, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice);
}

void free_plan(Plan& p) {
    timing_release(&p);
    if (p.in_done) cudaEventDestroy(p.in_done);
    if (p.in_stream) cudaStreamDestroy(p.in_stream);
    p.in_done = nullptr;
    p.in_stream = nullptr;
    for (void* v : p.allocations) cudaFree(v);
    p.allocations.clear();
    if (p.h_stage_in) cudaFreeHost(p.h_stage_in);
    if (p.h_stage_out) cudaFreeHost(p.h_stage_out);
    if (p.h_stage_aux) cudaFreeHost(p.h_stage_aux);
    p.h_stage_in = p.h_stage_out = p.h_stage_aux = nullptr;
}

inline float2 to_f2(const cui_complex64& c) { return make_float2(static_cast<float>(c.re), static_cast<float>(c.im)); }

// Restatement of the symmetric-grid index map (setup_grid_symmetric.m:175-232):
// 1-based linear index into the reference element's transfer function for
// grid point (ix, iy, iz) and element (ex, ey), all 0-based here.  Returns 0
// when the mirrored subscript leaves the grid (the reference would fail).
int64_t reference_shift(const Plan& p, int ix, int iy, int iz, int ex, int ey) {
    auto one = [](int i1, int e1, int ppp, int N, int E) -> int {
        int s = i1 - e1 * ppp;                       // i - (e-1)*ppp with 1-based i, e
        if (s <= 0) s = (N - (E - 1) * ppp + 1) - s;  // mirror about the offset (:222, :226)
        return (s >= 1 && s <= N) ? s : 0;
    };
    const int sx = one(ix + 1, ex, p.ppx, p.Nx, p.Ex);
    if (!sx) return 0;
    int sy = 1;
    if (p.n_dims == 3) {
        sy = one(iy + 1, ey, p.ppy, p.Ny, p.Ey);
        if (!sy) return 0;
    }
    return (sx - 1) + static_cast<int64_t>(p.Nx) * ((sy - 1) + static_cast<int64_t>(p.Ny) * iz) + 1;
}

// grid point (ix, iy) realising lateral offset o = i - e*ppp + (E-1)*ppp:
// returns i and e (0-based), or false when no in-grid pair exists.
bool offset_pair(int o, int N, int E, int ppp, int* i, int* e) {
    int k = 0;  // k = (E-1) - e
    if (o > N - 1) k = (o - (N - 1) + ppp - 1) / ppp;
    if (k > E - 1) return false;
    const int ii = o - k * ppp;
    if (ii < 0 || ii >= N) return false;
    *i = ii;
    *e = (E - 1) - k;
    return true;
}

cui_status build_table(Plan& p, const cui_born_desc* d, std::vector<float2>& T) {
    const size_t row = static_cast<size_t>(p.Noy) * p.Nox;
    T.assign(static_cast<size_t>(p.F) * p.Nz * row, make_float2(0.f, 0.f));
    if (d->table_form == CUI_TABLE_LATERAL) {
        if (!d->h_lateral) return set_error(CUI_ERR_INVALID_ARG, "h_lateral is NULL");
        for (size_t i = 0; i < T.size(); ++i) {
            const cui_complex64 c = d->h_lateral[i];
            if (!std::isfinite(c.re) || !std::isfinite(c.im))
                return set_error(CUI_ERR_NUMERIC, "non-finite entry in h_lateral");
            T[i] = to_f2(c);
        }
        return CUI_OK;
    }
    if (d->table_form != CUI_TABLE_REFERENCE) return set_error(CUI_ERR_INVALID_ARG, "unknown table_form");
    if (!d->h_ref || !d->indices_grid_FOV_shift)
        return set_error(CUI_ERR_INVALID_ARG, "h_ref or indices_grid_FOV_shift is NULL");
    // 1) the index map must be the symmetric-grid lateral shift
    const int32_t* map = d->indices_grid_FOV_shift;
    for (int e = 0; e < p.E; ++e) {
        const int ex = e % p.Ex, ey = e / p.Ex;
        for (int64_t pt = 0; pt < p.P; ++pt) {
            const int ix = static_cast<int>(pt % p.Nx);
            const int iy = static_cast<int>((pt / p.Nx) % p.Ny);
            const int iz = static_cast<int>(pt / (static_cast<int64_t>(p.Nx) * p.Ny));
            const int64_t want = reference_shift(p, ix, iy, iz, ex, ey);
            if (want == 0)
                return set_error(CUI_ERR_UNSUPPORTED_SETUP,
                                 "symmetric index map leaves the FOV grid (FOV narrower than the array); "
                                 "pass the lateral table instead");
            if (map[static_cast<int64_t>(e) * p.P + pt] != want)
                return set_error(CUI_ERR_UNSUPPORTED_SETUP,
                                 "indices_grid_FOV_shift is not the symmetric-grid lateral shift "
                                 "(combined_quick_gpu:NoSymmetricGridsSetup)");
        }
    }
    // 2) gather the distinct entries: offset (ox, oy) at depth z
    for (int oy = 0; oy < p.Noy; ++oy) {
        int iy = 0, ey = 0;
        if (p.n_dims == 3 && !offset_pair(oy, p.Ny, p.Ey, p.ppy, &iy, &ey))
            return set_error(CUI_ERR_UNSUPPORTED_SETUP, "lateral offset (y) not realised on the grid");
        for (int ox = 0; ox < p.Nox; ++ox) {
            int ix = 0, ex = 0;
            if (!offset_pair(ox, p.Nx, p.Ex, p.ppx, &ix, &ex))
                return set_error(CUI_ERR_UNSUPPORTED_SETUP, "lateral offset (x) not realised on the grid");
            const int e = ex + p.Ex * ey;
            for (int z = 0; z < p.Nz; ++z) {
                const int64_t pt = ix + static_cast<int64_t>(p.Nx) * (iy + static_cast<int64_t>(p.Ny) * z);
                const int64_t src = static_cast<int64_t>(map[static_cast<int64_t>(e) * p.P + pt]) - 1;
                for (int f = 0; f < p.F; ++f) {
                    const cui_complex64 c = d->h_ref[src * p.F + f];
                    if (!std::isfinite(c.re) || !std::isfinite(c.im))
                        return set_error(CUI_ERR_NUMERIC, "non-finite entry in h_ref");
                    T[((static_cast<size_t>(f) * p.Nz + z) * p.Noy + oy) * p.Nox + ox] = to_f2(c);
                }
            }
        }
    }
    return CUI_OK;
}

}  // namespace

cui_status init_geometry(Plan& p, int n_dims, const int32_t* npts, const int32_t* nel, const int32_t* ppp, int F,
                         int W, int max_objects) {
    if (n_dims != 2 && n_dims != 3) return set_error(CUI_ERR_INVALID_ARG, "n_dims must be 2 or 3");
    if (max_objects < 1) return set_error(CUI_ERR_INVALID_ARG, "max_objects must be >= 1");
    for (int k = 0; k < n_dims; ++k)
        if (npts[k] < 1) return set_error(CUI_ERR_INVALID_ARG, "n_points_axis must be positive");
    for (int k = 0; k < n_dims - 1; ++k)
        if (nel[k] < 1 || ppp[k] < 1)
            return set_error(CUI_ERR_INVALID_ARG, "n_elements_axis / n_points_per_pitch must be positive");
    if (F < 1) return set_error(CUI_ERR_INVALID_ARG, "n_f_unique must be positive");
    if (W < 1) return set_error(CUI_ERR_INVALID_ARG, "no measurements");
    p.n_dims = n_dims;
    p.Nx = npts[0];
    p.Ny = (n_dims == 3) ? npts[1] : 1;
    p.Nz = npts[n_dims - 1];
    p.Ex = nel[0];
    p.Ey = (n_dims == 3) ? nel[1] : 1;
    p.ppx = ppp[0];
    p.ppy = (n_dims == 3) ? ppp[1] : 1;
    p.Nox = p.Nx + (p.Ex - 1) * p.ppx;
    p.Noy = (n_dims == 3) ? p.Ny + (p.Ey - 1) * p.ppy : 1;
    p.P = static_cast<int64_t>(p.Nx) * p.Ny * p.Nz;
    p.E = p.Ex * p.Ey;
    p.F = F;
    p.W = W;
    p.max_objects = max_objects;
    p.Nj_max = (p.Nx + p.ppx - 1) / p.ppx;
    p.Ni = 8 + p.Nj_max + p.Ex + 8;
    if (p.ppx > 16) return set_error(CUI_ERR_UNSUPPORTED_SETUP, "more than 16 grid points per pitch");
    if (p.P > (int64_t(1) << 31) - 1) return set_error(CUI_ERR_UNSUPPORTED_SETUP, "more than 2^31-1 grid points");
    return CUI_OK;
}

#define CUI_TRY(x) do { cudaError_t e_ = (x); if (e_ != cudaSuccess) return check_cuda(e_, #x); } while (0)

cui_status build_metadata(Plan& p, const std::vector<MeasIn>& ms, const std::vector<double2>* pref_scale,
                          std::vector<int>& meas_slot0) {
    std::vector<int> slot_f;
    meas_slot0.assign(p.W, 0);
    for (int w = 0; w < p.W; ++w) {
        const MeasIn& m = ms[w];
        if (m.n_f < 1 || !m.f_idx || m.n_mixes < 0 || (m.n_mixes > 0 && !m.mixes))
            return set_error(CUI_ERR_INVALID_ARG, "invalid measurement " + std::to_string(w));
        meas_slot0[w] = static_cast<int>(slot_f.size());
        for (int k = 0; k < m.n_f; ++k) {
            const int fg = m.f_idx[k] - 1;
            if (fg < 0 || fg >= p.F) return set_error(CUI_ERR_INVALID_ARG, "indices_f_to_unique out of range");
            slot_f.push_back(fg);
        }
    }
    p.S = static_cast<int>(slot_f.size());
    std::vector<int> f_slot_ptr(p.F + 1, 0), f_slot_list(p.S);
    for (int s = 0; s < p.S; ++s) f_slot_ptr[slot_f[s] + 1]++;
    for (int f = 0; f < p.F; ++f) f_slot_ptr[f + 1] += f_slot_ptr[f];
    {
        std::vector<int> fill(f_slot_ptr.begin(), f_slot_ptr.end() - 1);
        for (int s = 0; s < p.S; ++s) f_slot_list[fill[slot_f[s]]++] = s;
    }
    p.max_slots_per_f = 0;
    for (int f = 0; f < p.F; ++f) p.max_slots_per_f = std::max(p.max_slots_per_f, f_slot_ptr[f + 1] - f_slot_ptr[f]);

    std::vector<int> row_slot, row_mix, row_fl, mix_nact, mix_nf, mix_act_off, act, pos;
    std::vector<int64_t> mix_pref_off;
    std::vector<float2> pref;
    int mix_id = 0;
    for (int w = 0; w < p.W; ++w) {
        const MeasIn& m = ms[w];
        for (int k = 0; k < m.n_mixes; ++k, ++mix_id) {
            const cui_mix_desc& x = m.mixes[k];
            if (x.n_f < 0 || x.n_active < 0 || (x.n_f > 0 && !x.indices_f_to_unique) ||
                (x.n_active > 0 && (!x.indices_active || !x.prefactors)))
                return set_error(CUI_ERR_INVALID_ARG, "invalid mix " + std::to_string(k) + " of measurement " + std::to_string(w));
            mix_nact.push_back(x.n_active);
            mix_nf.push_back(x.n_f);
            mix_act_off.push_back(static_cast<int>(act.size()));
            mix_pref_off.push_back(static_cast<int64_t>(pref.size()));
            std::vector<int> mpos(p.E, -1);
            for (int a = 0; a < x.n_active; ++a) {
                const int e = x.indices_active[a] - 1;
                if (e < 0 || e >= p.E) return set_error(CUI_ERR_INVALID_ARG, "indices_active out of range");
                if (mpos[e] >= 0) return set_error(CUI_ERR_INVALID_ARG, "duplicate active element in a mix");
                mpos[e] = a;
                act.push_back(e);
            }
            pos.insert(pos.end(), mpos.begin(), mpos.end());
            std::vector<int> fm_of(x.n_f);
            for (int fl = 0; fl < x.n_f; ++fl) {
                const int fm = x.indices_f_to_unique[fl] - 1;
                if (fm < 0 || fm >= m.n_f) return set_error(CUI_ERR_INVALID_ARG, "mix indices_f_to_unique out of range");
                fm_of[fl] = fm;
                row_slot.push_back(meas_slot0[w] + fm);
                row_mix.push_back(mix_id);
                row_fl.push_back(fl);
            }
            for (int a = 0; a < x.n_active; ++a)
                for (int fl = 0; fl < x.n_f; ++fl) {
                    const cui_complex64 c = x.prefactors[static_cast<int64_t>(a) * x.n_f + fl];
                    if (!std::isfinite(c.re) || !std::isfinite(c.im))
                        return set_error(CUI_ERR_NUMERIC, "non-finite prefactor");
                    if (pref_scale) {
                        const double2 sc = (*pref_scale)[m.f_idx[fm_of[fl]] - 1];
                        pref.push_back(make_float2(static_cast<float>(sc.x * c.re - sc.y * c.im),
                                                   static_cast<float>(sc.x * c.im + sc.y * c.re)));
                    } else {
                        pref.push_back(to_f2(c));
                    }
                }
        }
    }
    p.n_mix = mix_id;
    p.n_obs = static_cast<int64_t>(row_slot.size());
    if (p.n_obs < 1) return set_error(CUI_ERR_INVALID_ARG, "the operator has no observations");
    std::vector<int> slot_row_ptr(p.S + 1, 0), slot_rows(p.n_obs);
    for (int64_t r = 0; r < p.n_obs; ++r) slot_row_ptr[row_slot[r] + 1]++;
    for (int s = 0; s < p.S; ++s) slot_row_ptr[s + 1] += slot_row_ptr[s];
    {
        std::vector<int> fill(slot_row_ptr.begin(), slot_row_ptr.end() - 1);
        for (int64_t r = 0; r < p.n_obs; ++r) slot_rows[fill[row_slot[r]]++] = static_cast<int>(r);
    }
    p.h_f_slot_ptr = f_slot_ptr;
    p.h_f_slot_list = f_slot_list;
    p.h_slot_f = slot_f;
    // device uploads happen in upload_metadata once the device is selected
    p.h_meta.row_slot.swap(row_slot);
    p.h_meta.row_mix.swap(row_mix);
    p.h_meta.row_fl.swap(row_fl);
    p.h_meta.mix_nact.swap(mix_nact);
    p.h_meta.mix_nf.swap(mix_nf);
    p.h_meta.mix_act_off.swap(mix_act_off);
    p.h_meta.act.swap(act);
    p.h_meta.pos.swap(pos);
    p.h_meta.mix_pref_off.swap(mix_pref_off);
    p.h_meta.pref.swap(pref);
    p.h_meta.slot_row_ptr.swap(slot_row_ptr);
    p.h_meta.slot_rows.swap(slot_rows);
    return CUI_OK;
}

cui_status select_device_and_shapes(Plan& p, int device) {
    const int n_lines = p.Ny * p.Nz;
    const int64_t gsz = static_cast<int64_t>(p.S) * p.max_objects * p.E * sizeof(float2);
    const int n_eyb = (p.Ey + fwd_rows_per_block(p.Ey) - 1) / fwd_rows_per_block(p.Ey);  // blocks per line group
    // about 2048 forward blocks, and at most 256 grid lines per group: each group is one FP32
    // accumulation chain per element, and the 3D array's 16384 lines in 4 groups left chains of
    // ~90k terms (partial sums are then added in a fixed order)
    int groups = std::max(1, std::min(n_lines, std::max((2048 + p.F * n_eyb - 1) / (p.F * n_eyb), (n_lines + 255) / 256)));
    groups = static_cast<int>(std::max<int64_t>(
        1, std::min<int64_t>(groups, std::max<int64_t>(1, static_cast<int64_t>(kPartBudget) / std::max<int64_t>(gsz, 1)))));
    p.fwd_lines_per_group = (n_lines + groups - 1) / groups;
    p.fwd_groups = (n_lines + p.fwd_lines_per_group - 1) / p.fwd_lines_per_group;
    const int64_t gpart = static_cast<int64_t>(p.max_objects) * p.P * sizeof(float2);
    int nfc = std::max(1, std::min(p.F, (4096 + n_lines - 1) / n_lines));
    nfc = static_cast<int>(std::max<int64_t>(
        1, std::min<int64_t>(nfc, std::max<int64_t>(1, static_cast<int64_t>(kPartBudget) / std::max<int64_t>(gpart, 1)))));
    p.adj_fchunk = (p.F + nfc - 1) / nfc;
    p.adj_nfc = (p.F + p.adj_fchunk - 1) / p.adj_fchunk;

    int n_dev = 0;
    if (cudaGetDeviceCount(&n_dev) != cudaSuccess || n_dev < 1)
        return set_error(CUI_ERR_NO_DEVICE, "no CUDA device (combined_quick_gpu:NoCUDADevices)");
    if (device < 0 || device >= n_dev)
        return set_error(CUI_ERR_NO_DEVICE, "invalid device index (combined_quick_gpu:InvalidCUDADevice)");
    p.device = device;
    CUI_TRY(cudaSetDevice(p.device));
    int smem_optin = 0;
    CUI_TRY(cudaDeviceGetAttribute(&smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, p.device));
    int nc = 1;
    while (nc < p.max_slots_per_f && nc < kMaxNC) nc = (nc < 8) ? nc * 2 : nc + 4;
    if (fwd_smem_bytes(&p, nc) + 1024 > static_cast<size_t>(smem_optin) ||
        adj_smem_bytes(&p, nc) + 1024 > static_cast<size_t>(smem_optin))
        return set_error(CUI_ERR_UNSUPPORTED_SETUP, "grid line too long for the shared-memory staging of these kernels");
    std::string why;
    if (!launch_shapes_ok(&p, &why)) return set_error(CUI_ERR_UNSUPPORTED_SETUP, why);
    return CUI_OK;
}

// Slots of one frequency whose observation rows carry identical mixes -- the same active
// elements and bitwise the same prefactors, row by row -- have the same per-row sums
// sum_a pref h in every column of Phi; only their incident fields differ.  The groups let the
// received energies form those sums once per group (waves that share a receive mixing).
static void energy_groups(const Plan& p, const HostMeta& h, std::vector<int>& gptr, std::vector<int>& gslots) {
    auto same_rows = [&](int s1, int s2) {
        const int b1 = h.slot_row_ptr[s1], n1 = h.slot_row_ptr[s1 + 1] - b1;
        const int b2 = h.slot_row_ptr[s2], n2 = h.slot_row_ptr[s2 + 1] - b2;
        if (n1 != n2) return false;
        for (int k = 0; k < n1; ++k) {
            const int r1 = h.slot_rows[b1 + k], r2 = h.slot_rows[b2 + k];
            const int m1 = h.row_mix[r1], m2 = h.row_mix[r2];
            const int na = h.mix_nact[m1];
            if (na != h.mix_nact[m2]) return false;
            if (m1 == m2 && h.row_fl[r1] == h.row_fl[r2]) continue;
            if (std::memcmp(&h.act[h.mix_act_off[m1]], &h.act[h.mix_act_off[m2]], sizeof(int) * na) != 0) return false;
            const int64_t o1 = h.mix_pref_off[m1] + h.row_fl[r1], o2 = h.mix_pref_off[m2] + h.row_fl[r2];
            const int nf1 = h.mix_nf[m1], nf2 = h.mix_nf[m2];
            for (int ia = 0; ia < na; ++ia)
                if (std::memcmp(&h.pref[o1 + static_cast<int64_t>(ia) * nf1], &h.pref[o2 + static_cast<int64_t>(ia) * nf2],
                                sizeof(float2)) != 0)
                    return false;
        }
        return true;
    };
    gptr.assign(1, 0);
    gslots.clear();
    for (int f = 0; f < p.F; ++f) {
        std::vector<std::vector<int>> groups;  // of this frequency, in first-seen order
        for (int i = p.h_f_slot_ptr[f]; i < p.h_f_slot_ptr[f + 1]; ++i) {
            const int s = p.h_f_slot_list[i];
            bool placed = false;
            for (auto& g : groups)
                if (same_rows(g[0], s)) {
                    g.push_back(s);
                    placed = true;
                    break;
                }
            if (!placed) groups.push_back({s});
        }
        for (const auto& g : groups) {
            gslots.insert(gslots.end(), g.begin(), g.end());
            gptr.push_back(static_cast<int>(gslots.size()));
        }
    }
}

// The terms of ||Phi e_p||^2 for each energy group's representative slot, in the order the energy
// kernel adds them: per observation row of the slot, per active element a, the element's table-row
// offset in the staged rows [E_y][N_ox] (e_y N_ox + (E_x - 1 - e_x) ppx) and the prefactor
// pref[mix][fl, a], packed as (re, im, bits of (offset << 1 | last term of the row), 0).
static void energy_terms(const Plan& p, const HostMeta& h, const std::vector<int>& gptr,
                         const std::vector<int>& gslots, std::vector<int>& tptr, std::vector<float4>& terms) {
    tptr.assign(1, 0);
    terms.clear();
    for (size_t g = 0; g + 1 < gptr.size(); ++g) {
        const int rep = gslots[gptr[g]];
        for (int rr = h.slot_row_ptr[rep]; rr < h.slot_row_ptr[rep + 1]; ++rr) {
            const int row = h.slot_rows[rr];
            const int m = h.row_mix[row], fl = h.row_fl[row];
            const int nact = h.mix_nact[m], nf = h.mix_nf[m];
            for (int ia = 0; ia < nact; ++ia) {
                const int e = h.act[h.mix_act_off[m] + ia];
                const int ey = p.Ey == 1 ? 0 : e / p.Ex, ex = e - ey * p.Ex;
                const int toff = ey * p.Nox + (p.Ex - 1 - ex) * p.ppx;
                const float2 w = h.pref[h.mix_pref_off[m] + static_cast<int64_t>(ia) * nf + fl];
                const int info = (toff << 1) | (ia == nact - 1 ? 1 : 0);
                float bits;
                std::memcpy(&bits, &info, sizeof bits);
                terms.push_back(make_float4(w.x, w.y, bits, 0.f));
            }
        }
        tptr.push_back(static_cast<int>(terms.size()));
    }
}

cui_status upload_metadata_and_workspace(Plan& p) {
    HostMeta& h = p.h_meta;
    CUI_TRY(upload(p, &p.f_slot_ptr, p.h_f_slot_ptr));
    CUI_TRY(upload(p, &p.slot_f, p.h_slot_f));
    CUI_TRY(upload(p, &p.f_slot_list, p.h_f_slot_list));
    CUI_TRY(upload(p, &p.row_slot, h.row_slot));
    CUI_TRY(upload(p, &p.row_mix, h.row_mix));
    CUI_TRY(upload(p, &p.row_fl, h.row_fl));
    CUI_TRY(upload(p, &p.mix_nact, h.mix_nact));
    CUI_TRY(upload(p, &p.mix_nf, h.mix_nf));
    CUI_TRY(upload(p, &p.mix_pref_off, h.mix_pref_off));
    CUI_TRY(upload(p, &p.mix_act_off, h.mix_act_off));
    CUI_TRY(upload(p, &p.act, h.act));
    CUI_TRY(upload(p, &p.pref, h.pref));
    CUI_TRY(upload(p, &p.pos, h.pos));
    CUI_TRY(upload(p, &p.slot_row_ptr, h.slot_row_ptr));
    CUI_TRY(upload(p, &p.slot_rows, h.slot_rows));
    {
        std::vector<int> gptr, gslots;
        energy_groups(p, h, gptr, gslots);
        p.n_egroups = static_cast<int>(gptr.size()) - 1;
        std::vector<int> tptr;
        std::vector<float4> terms;
        energy_terms(p, h, gptr, gslots, tptr, terms);
        CUI_TRY(upload(p, &p.egroup_term_ptr, tptr));
        CUI_TRY(upload(p, &p.egroup_terms, terms));
        CUI_TRY(upload(p, &p.egroup_ptr, gptr));
        CUI_TRY(upload(p, &p.egroup_slots, gslots));
    }
    {
        // channel-contraction entries per object (dense gamma): per slot, the rows it feeds or the
        // distinct elements they read, whichever is fewer, times the grid points
        int64_t ch = 0;
        std::vector<int> seen(p.E, -1);
        for (int s = 0; s < p.S; ++s) {
            int n_el = 0;
            const int r0 = h.slot_row_ptr[s], r1 = h.slot_row_ptr[s + 1];
            for (int i = r0; i < r1; ++i) {
                const int m = h.row_mix[h.slot_rows[i]];
                for (int a = 0; a < h.mix_nact[m]; ++a) {
                    const int e = h.act[h.mix_act_off[m] + a];
                    if (seen[e] != s) { seen[e] = s; ++n_el; }
                }
            }
            ch += std::min(r1 - r0, n_el);
        }
        p.channel_entries = ch * p.P;
    }
    p.h_meta = HostMeta();

    const int B = p.max_objects;
    const size_t part_fwd = static_cast<size_t>(p.fwd_groups) * p.S * B * p.E;
    const size_t part_adj = static_cast<size_t>(p.adj_nfc) * B * p.P;
    p.ws_part_bytes = std::max(part_fwd, part_adj) * sizeof(float2);
    CUI_TRY(dalloc(p, &p.ws_part, std::max(part_fwd, part_adj)));
    CUI_TRY(dalloc(p, &p.ws_G, static_cast<size_t>(p.S) * B * p.E));
    CUI_TRY(dalloc(p, &p.ws_r, static_cast<size_t>(p.n_obs) * B));
    CUI_TRY(dalloc(p, &p.ws_loss, loss_workspace_floats(B)));
    p.occ_nblk = static_cast<int>((p.P + 1023) / 1024);
    CUI_TRY(dalloc(p, &p.occ_idx, static_cast<size_t>(p.P)));
    CUI_TRY(dalloc(p, &p.occ_cnt, static_cast<size_t>(2 * p.occ_nblk + 2)));
    p.workspace_bytes = p.ws_part_bytes +
                        sizeof(float2) * (static_cast<size_t>(p.S) * B * p.E + static_cast<size_t>(p.n_obs) * B) +
                        sizeof(float) * loss_workspace_floats(B);
    return CUI_OK;
}

// frees the plan's allocations made since index `mark` (a failed build leaves nothing behind)
void release_since(Plan& p, size_t mark) {
    for (size_t i = mark; i < p.allocations.size(); ++i) cudaFree(p.allocations[i]);
    p.allocations.resize(std::min(mark, p.allocations.size()));
}

cui_status device_alloc(Plan& p, void** ptr, size_t bytes) {
    if (injected_alloc_failure(p)) return check_cuda(cudaErrorMemoryAllocation, "cudaMalloc");
    void* v = nullptr;
    cudaError_t e = cudaMalloc(&v, std::max<size_t>(bytes, 1));
    if (e != cudaSuccess) return check_cuda(e, "cudaMalloc");
    p.allocations.push_back(v);
    *ptr = v;
    return CUI_OK;
}

namespace {

cui_status create(const cui_born_desc* d, int32_t max_objects, Plan& p) {
    if (!d) return set_error(CUI_ERR_INVALID_ARG, "desc is NULL");
    cui_status st = init_geometry(p, d->n_dims, d->n_points_axis, d->n_elements_axis, d->n_points_per_pitch,
                                  d->n_f_unique, d->n_measurements, max_objects);
    if (st != CUI_OK) return st;
    if (!d->measurements) return set_error(CUI_ERR_INVALID_ARG, "no measurements");
    std::vector<MeasIn> ms(p.W);
    for (int w = 0; w < p.W; ++w) {
        const cui_measurement_desc& m = d->measurements[w];
        if (!m.p_incident) return set_error(CUI_ERR_INVALID_ARG, "invalid measurement " + std::to_string(w));
        ms[w] = MeasIn{m.n_f, m.indices_f_to_unique, m.n_mixes, m.mixes};
    }
    std::vector<int> meas_slot0;
    if ((st = build_metadata(p, ms, nullptr, meas_slot0)) != CUI_OK) return st;
    if ((st = select_device_and_shapes(p, d->device)) != CUI_OK) return st;

    std::vector<float2> T;
    if ((st = build_table(p, d, T)) != CUI_OK) return st;
    CUI_TRY(upload(p, &p.table, T));
    p.table_bytes = T.size() * sizeof(float2);
    std::vector<float2>().swap(T);
    std::vector<float2> pin(static_cast<size_t>(p.S) * p.P);
    for (int w = 0; w < p.W; ++w) {
        const cui_measurement_desc& m = d->measurements[w];
        for (int64_t pt = 0; pt < p.P; ++pt)
            for (int k = 0; k < m.n_f; ++k) {
                const cui_complex64 c = m.p_incident[pt * m.n_f + k];
                if (!std::isfinite(c.re) || !std::isfinite(c.im))
                    return set_error(CUI_ERR_NUMERIC, "non-finite entry in p_incident");
                pin[static_cast<size_t>(meas_slot0[w] + k) * p.P + pt] = to_f2(c);
            }
    }
    CUI_TRY(upload(p, &p.p_in, pin));
    p.incident_bytes = pin.size() * sizeof(float2);
    std::vector<float2>().swap(pin);
    return upload_metadata_and_workspace(p);
}
#undef CUI_TRY

bool valid_plan(const cui_born_plan* plan) { return plan != nullptr; }

cui_status check_apply(const cui_born_plan* plan, const void* in, int64_t ld_in, int64_t rows_in, int32_t B,
                       const void* out, int64_t ld_out, int64_t rows_out) {
    if (!valid_plan(plan)) return set_error(CUI_ERR_INVALID_ARG, "plan is NULL");
    if (B < 1 || B > plan->p.max_objects)
        return set_error(CUI_ERR_INVALID_ARG, "n_objects must be in [1, max_objects] (combined_quick_gpu:NoValidDoubleMatrix)");
    if (!in || !out) return set_error(CUI_ERR_INVALID_ARG, "NULL input or output");
    if (ld_in < rows_in || ld_out < rows_out)
        return set_error(CUI_ERR_INVALID_ARG, "leading dimension smaller than the number of rows");
    return CUI_OK;
}

}  // namespace
}  // namespace cui

using cui::set_error;

extern "C" {

cui_status cui_born_plan_create(const cui_born_desc* desc, int32_t max_objects, cui_born_plan** plan) {
    const cui::NvtxRange nvtx_range("cui_born_plan_create");
    if (!plan) return set_error(CUI_ERR_INVALID_ARG, "plan is NULL");
    *plan = nullptr;
    cui_born_plan* h = new (std::nothrow) cui_born_plan();
    if (!h) return set_error(CUI_ERR_OOM, "host allocation failed");
    const cui::DeviceGuard restore(-1);  // creation makes the plan's device current; the caller's is restored
    cui_status s;
    try {
        s = cui::create(desc, max_objects, h->p);
    } catch (const std::bad_alloc&) {
        s = set_error(CUI_ERR_OOM, "host allocation failed");
    }
    if (s != CUI_OK) {
        cui::free_plan(h->p);
        delete h;
        return s;
    }
    *plan = h;
    return CUI_OK;
}

cui_status cui_born_plan_destroy(cui_born_plan* plan) {
    if (!plan) return CUI_OK;
    const cui::DeviceGuard dev_guard(plan->p.device);
    cui::free_plan(plan->p);
    delete plan;
    return CUI_OK;
}

cui_status cui_born_plan_info(const cui_born_plan* plan, cui_born_info* info) {
    if (!plan || !info) return set_error(CUI_ERR_INVALID_ARG, "NULL argument");
    const cui::Plan& p = plan->p;
    info->n_points = p.P;
    info->n_observations = p.n_obs;
    info->n_elements = p.E;
    info->n_slots = p.S;
    info->n_f_unique = p.F;
    info->table_bytes = static_cast<int64_t>(p.table_bytes);
    info->incident_bytes = static_cast<int64_t>(p.incident_bytes);
    info->workspace_bytes = static_cast<int64_t>(p.workspace_bytes);
    info->contraction_macs = static_cast<int64_t>(p.S) * p.E * p.P;
    info->channel_macs = p.channel_entries;
    info->folded_bytes = static_cast<int64_t>(p.phi_bytes);
    info->folded_sums = p.phi_reps;
    info->device_allocations = p.n_device_allocs;
    return CUI_OK;
}

cui_status cui_born_size(const cui_born_plan* plan, int64_t* n_observations, int64_t* n_points) {
    if (!plan) return set_error(CUI_ERR_INVALID_ARG, "plan is NULL");
    if (n_observations) *n_observations = plan->p.n_obs;
    if (n_points) *n_points = plan->p.P;
    return CUI_OK;
}

cui_status cui_born_forward(cui_born_plan* plan, const cui_complex32* gamma, int64_t ld_gamma, int32_t n_objects,
                            cui_complex32* u, int64_t ld_u, void* stream) {
    const cui::NvtxRange nvtx_range("cui_born_forward");
    cui_status s = cui::check_apply(plan, gamma, ld_gamma, plan ? plan->p.P : 0, n_objects, u, ld_u,
                                    plan ? plan->p.n_obs : 0);
    if (s != CUI_OK) return s;
    const cui::DeviceGuard dev_guard(plan->p.device);
    return cui::forward_device(&plan->p, reinterpret_cast<const float2*>(gamma), ld_gamma, n_objects,
                               reinterpret_cast<float2*>(u), ld_u, static_cast<cudaStream_t>(stream));
}

cui_status cui_born_adjoint(cui_born_plan* plan, const cui_complex32* u, int64_t ld_u, int32_t n_objects,
                            cui_complex32* gamma_hat, int64_t ld_gamma, void* stream) {
    const cui::NvtxRange nvtx_range("cui_born_adjoint");
    cui_status s = cui::check_apply(plan, u, ld_u, plan ? plan->p.n_obs : 0, n_objects, gamma_hat, ld_gamma,
                                    plan ? plan->p.P : 0);
    if (s != CUI_OK) return s;
    const cui::DeviceGuard dev_guard(plan->p.device);
    return cui::adjoint_device(&plan->p, reinterpret_cast<const float2*>(u), ld_u, n_objects,
                               reinterpret_cast<float2*>(gamma_hat), ld_gamma, static_cast<cudaStream_t>(stream));
}

cui_status cui_born_vjp(cui_born_plan* plan, const cui_complex32* gamma, int64_t ld_gamma, const cui_complex32* u_meas,
                        int64_t ld_u, int32_t n_objects, cui_complex32* grad, int64_t ld_grad, float* loss, void* stream) {
    const cui::NvtxRange nvtx_range("cui_born_vjp");
    cui_status s = cui::check_apply(plan, gamma, ld_gamma, plan ? plan->p.P : 0, n_objects, grad, ld_grad,
                                    plan ? plan->p.P : 0);
    if (s != CUI_OK) return s;
    if (!u_meas || ld_u < plan->p.n_obs) return set_error(CUI_ERR_INVALID_ARG, "invalid u_meas");
    const cui::DeviceGuard dev_guard(plan->p.device);
    return cui::vjp_device(&plan->p, reinterpret_cast<const float2*>(gamma), ld_gamma,
                           reinterpret_cast<const float2*>(u_meas), ld_u, n_objects, reinterpret_cast<float2*>(grad),
                           ld_grad, loss, static_cast<cudaStream_t>(stream));
}

cui_status cui_born_lasso(cui_born_plan* plan, const cui_complex32* u_meas, int64_t ld_u, int32_t n_objects,
                          cui_complex32* gamma, int64_t ld_gamma, const float* lambda, float step, int32_t n_iter,
                          float* loss, void* stream) {
    const cui::NvtxRange nvtx_range("cui_born_lasso");
    cui_status s = cui::check_apply(plan, gamma, ld_gamma, plan ? plan->p.P : 0, n_objects, gamma, ld_gamma,
                                    plan ? plan->p.P : 0);
    if (s != CUI_OK) return s;
    if (!u_meas || ld_u < plan->p.n_obs) return set_error(CUI_ERR_INVALID_ARG, "invalid u_meas");
    if (!lambda) return set_error(CUI_ERR_INVALID_ARG, "lambda is NULL");
    if (n_iter < 0 || !(step > 0.f)) return set_error(CUI_ERR_INVALID_ARG, "n_iter must be >= 0 and step > 0");
    const cui::DeviceGuard dev_guard(plan->p.device);
    return cui::lasso_device(&plan->p, reinterpret_cast<float2*>(gamma), ld_gamma, reinterpret_cast<const float2*>(u_meas),
                             ld_u, n_objects, step, lambda, n_iter, loss, static_cast<cudaStream_t>(stream));
}

cui_status cui_born_timing_enable(cui_born_plan* plan, int32_t enable) {
    if (!plan) return set_error(CUI_ERR_INVALID_ARG, "plan is NULL");
    plan->p.timing = enable != 0;
    return CUI_OK;
}

cui_status cui_born_timing_read(cui_born_plan* plan, cui_born_timing* out) {
    if (!plan || !out) return set_error(CUI_ERR_INVALID_ARG, "NULL argument");
    cui::Plan& p = plan->p;
    *out = cui_born_timing{0, 0, 0.0, 0.0};
    const cui::DeviceGuard dev_guard(p.device);
    for (size_t i = 0; i < p.ev_used; ++i) {
        cudaError_t e = cudaEventSynchronize(p.ev_pool[2 * i + 1]);
        if (e != cudaSuccess) return cui::check_cuda(e, "cudaEventSynchronize");
        float ms = 0.f;
        if ((e = cudaEventElapsedTime(&ms, p.ev_pool[2 * i], p.ev_pool[2 * i + 1])) != cudaSuccess)
            return cui::check_cuda(e, "cudaEventElapsedTime");
        if (p.ev_kind[i] == 0) {
            out->n_forward++;
            out->ms_forward += ms;
        } else {
            out->n_adjoint++;
            out->ms_adjoint += ms;
        }
    }
    p.ev_used = 0;
    return CUI_OK;
}

const char* cui_status_string(cui_status status) {
    switch (status) {
        case CUI_OK: return "CUI_OK";
        case CUI_ERR_INVALID_ARG: return "CUI_ERR_INVALID_ARG";
        case CUI_ERR_UNSUPPORTED_SETUP: return "CUI_ERR_UNSUPPORTED_SETUP";
        case CUI_ERR_OOM: return "CUI_ERR_OOM";
        case CUI_ERR_CUDA: return "CUI_ERR_CUDA";
        case CUI_ERR_TIMEOUT: return "CUI_ERR_TIMEOUT";
        case CUI_ERR_NUMERIC: return "CUI_ERR_NUMERIC";
        case CUI_ERR_NO_DEVICE: return "CUI_ERR_NO_DEVICE";
    }
    return "CUI_ERR_UNKNOWN";
}

const char* cui_last_error(void) { return cui::g_last_error.c_str(); }

int64_t cui_launch_count(void) { return cui::g_launches.load(std::memory_order_relaxed); }

}  // extern "C"
