// Internal declarations shared by the translation units of libcui_born.
//
// Device layout of a plan (all FP32 complex as float2):
//   table   [F][Nz][Noy][Nox]  lateral-offset transfer-function table; row (f, z, oy)
//                              is contiguous in ox.  No_d = N_d + (E_d-1)*ppp_d.
//                              Not stored when generated (cui_gen.cuh).
//   p_in    [S][P]             incident field of each slot (measurement, unique
//                              frequency), points in column-major grid order.
//   rows    [n_obs]            observation -> (slot, mix, local frequency).
//   mixes                      active-element lists, prefactors [n_f x n_act]
//                              (column-major) and the element -> position map.
// The forward contraction produces element signals G[S][B][E]; mixing turns
// them into observations.  The adjoint unmixes observations into V[S][B][E]
// and contracts back onto the grid.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>
#include <cstddef>
#include <string>
#include <vector>

#include "../../include/cui_born.h"
#include "cui_gen.cuh"

#include <nvtx3/nvToolsExt.h>

namespace cui {

// Column chunk width of the FP32 contraction kernels: the number of slots
// (incident waves sharing one frequency) one thread block processes per pass.
constexpr int kMaxNC = 16;

// Observation-row and mixing metadata built on the host before upload.
struct HostMeta {
    std::vector<int> row_slot, row_mix, row_fl, mix_nact, mix_nf, mix_act_off, act, pos, slot_row_ptr, slot_rows;
    std::vector<int64_t> mix_pref_off;
    std::vector<float2> pref;
};

// One measurement as seen by the metadata builder (both descriptor forms).
struct MeasIn {
    int n_f;
    const int32_t* f_idx;         // 1-based global frequency indices
    int n_mixes;
    const cui_mix_desc* mixes;
};

struct Plan {
    int device = 0;
    int n_dims = 2;
    int Nx = 1, Ny = 1, Nz = 1;     // grid points (Ny = 1 in 2D)
    int Ex = 1, Ey = 1;             // elements per lateral axis (Ey = 1 in 2D)
    int ppx = 1, ppy = 1;           // points per pitch
    int Nox = 1, Noy = 1;           // lateral offsets (Noy = 1 in 2D)
    int64_t P = 0;                  // grid points
    int E = 0;                      // elements
    int F = 0;                      // global unique frequencies
    int S = 0;                      // slots
    int W = 0;                      // measurements
    int n_mix = 0;                  // mixes over all measurements
    int64_t n_obs = 0;              // observations
    int max_objects = 1;
    int max_slots_per_f = 0;

    // device tables
    float2* table = nullptr;        // null unless the table is stored
    int table_mode = CUI_STORAGE_STORED;  // or CUI_STORAGE_GENERATED / CUI_STORAGE_STREAMED (3D setup form)
    TableGen gen{};                 // generator parameters (device arrays) when not stored
    float2* stream_buf = nullptr;   // streamed: table rows of stream_nf frequencies, [stream_nf][Nz][Noy][Nox]
    int stream_nf = 0;              // frequencies per streamed chunk (= adj_fchunk)
    float2* p_in = nullptr;
    int* f_slot_ptr = nullptr;      // [F+1] CSR of slots per global frequency
    int* f_slot_list = nullptr;     // [S]
    int* slot_f = nullptr;          // [S] global frequency of each slot
    int* row_slot = nullptr;        // [n_obs]
    int* row_mix = nullptr;         // [n_obs]
    int* row_fl = nullptr;          // [n_obs]
    int* mix_nact = nullptr;        // [n_mix]
    int* mix_nf = nullptr;          // [n_mix]
    int64_t* mix_pref_off = nullptr;// [n_mix]
    int* mix_act_off = nullptr;     // [n_mix]
    int* act = nullptr;             // concatenated active lists (0-based)
    float2* pref = nullptr;         // concatenated prefactors
    int* pos = nullptr;             // [n_mix][E] position of element in mix or -1
    int* slot_row_ptr = nullptr;    // [S+1] CSR of observations per slot
    int* slot_rows = nullptr;       // [n_obs]
    // slots of one frequency whose rows carry identical mixes (active elements and prefactors),
    // as CSR over groups: they differ only in their incident fields (received energies)
    int n_egroups = 0;
    int* egroup_ptr = nullptr;      // [n_egroups + 1]
    int* egroup_slots = nullptr;    // [S], the first slot of a group is its representative
    int* egroup_term_ptr = nullptr; // [n_egroups + 1] CSR of the representative's energy terms
    float4* egroup_terms = nullptr; // (pref re, pref im, bits of (table-row offset << 1 | row end), 0)

    // workspace (sized for max_objects at creation; shared by all applies)
    float2* ws_part = nullptr;      // forward / adjoint partial sums
    size_t ws_part_bytes = 0;
    float2* ws_G = nullptr;         // [S][B][E] element signals / unmixed data
    float2* ws_r = nullptr;         // [B][n_obs] residual of the VJP
    float* ws_loss = nullptr;       // [B] loss partial sums
    // occupancy compaction of the FP32 forward (points where any column of gamma is nonzero)
    int* occ_idx = nullptr;         // [P] occupied points, ascending
    int* occ_cnt = nullptr;         // [2 * occ_nblk + 2]: per-block counts, offsets, then n_occ and the choice
    int occ_nblk = 0;               // 1024-point blocks
    int64_t occ_limit = -1;         // compact when n_occ <= occ_limit (-1: P / 16 stored, P / 32 otherwise; 0: never)

    // launch geometry chosen at creation
    int fwd_groups = 1;             // line groups of the dense forward
    int fwd_lines_per_group = 1;
    int adj_fchunk = 1;             // frequencies per adjoint block
    int adj_nfc = 1;                // adjoint frequency chunks
    int Nj_max = 1;                 // steps per residue along x
    int Ni = 1;                     // staged table entries per residue
    size_t table_bytes = 0, incident_bytes = 0, workspace_bytes = 0;
    int64_t channel_entries = 0;     // sum over slots of min(rows, distinct active elements) x points

    // host-side pinned staging for the FP64 host entry points
    float2* h_stage_in = nullptr;
    float2* h_stage_out = nullptr;
    float2* h_stage_aux = nullptr;   // second input staging buffer (measured data of the host VJP)
    size_t h_stage_elems = 0;
    int host_direct = -1;            // host entry points: kernels read/write the caller's buffers (-1: not probed)
    float2* d_stage_in = nullptr;   // device copies for the host entry points
    float2* d_stage_out = nullptr;
    float2* d_stage_aux = nullptr;
    float* d_stage_loss = nullptr;
    // the host VJP reads the measured data on this stream while the forward runs on the caller's
    cudaStream_t in_stream = nullptr;  // non-blocking: no implicit order against the legacy stream
    cudaEvent_t in_done = nullptr;     // recorded after that read; the residual waits on it

    // host copies kept after creation (launch planning, table builders)
    std::vector<int> h_f_slot_ptr, h_f_slot_list, h_slot_f;
    HostMeta h_meta;                 // emptied once uploaded

    // contraction path: 0 = FP32 CUDA cores, 1 = split-BF16 tensor cores over (slot, element)
    // (cui_tc.cu, cui_tc2.cu), 2 = split-BF16 GEMMs against the folded operator (cui_phi.cu)
    int precision = 0;
    uint32_t* tb = nullptr;          // band arrays [4][F][Nz][Noy][ppx][Nb] of packed bf16x2
    int64_t tb_vstride = 0;
    int Nb = 0;                      // band entries per residue
    int Epad = 0;                    // elements rounded up to a multiple of 8
    int Jpad = 0;                    // points per residue rounded up to a multiple of 8
    size_t tc_bytes = 0;
    // line-unit tensor-core kernels (cui_tc2.cu; 2D, 4 grid points per pitch):
    // raw band rows [2][F][Nz][RowW] of packed bf16x2 (re, im), hi then lo
    int tc2 = 0;                     // 1 when the plan runs the line-unit kernels
    // launch shapes picked by cui_born_autotune (0: the rule): column tiles of at most 32 columns
    // instead of 64 (1), and the block counts the forward's line groups and the adjoint's frequency
    // chunks aim at
    int tune_tile = 0;
    int tune_fwd_blocks = 0;
    int tune_adj_blocks = 0;
    uint32_t* tr = nullptr;
    int64_t tr_vstride = 0;          // entries per variant
    int RowW = 0;                    // entries per row (lateral offsets rounded up to 4, zero padded)
    // incident fields re-laid so that one bulk copy brings every slot of a frequency:
    //   p_fw [F][Nz][nKC][ms][66]  forward: 64-point segments (+2 pad) of each slot of f
    //   p_ad [F][Nz][4][ms][Jp]    adjoint: residue classes x = r + 4j of each slot of f
    float2* p_fw = nullptr;
    float2* p_ad = nullptr;
    int Jp = 0;                      // points per residue class, rounded up to even
    int nKC = 0;                     // 64-point segments per grid line
    int ms = 0;                      // slot rows per frequency in both layouts (most slots of any frequency)
    float2* ws_galign = nullptr;     // [max_objects][P] aligned copy of a misaligned gamma (forward)
    uint32_t* ws_vs = nullptr;       // split-BF16 V tiles of the adjoint [F][tiles][tile bytes / 4]
    int* ws_status = nullptr;        // device status word (bounded waits that gave up)
    // wall-clock limit of every bounded wait of the tensor-core kernels (a wait that runs out
    // raises the status word); the waits that drain in-flight copies keep a fixed 1 s
    uint64_t wait_limit_ns = 1000000000ull;

    // folded operator (cui_phi.cu, precision 2): observation x point matrix in split bf16,
    // 16-byte pieces per (row, 8-point block, component, half), rows padded to 256 and points
    // to 256; B forms of one 64-object pass of gamma and of u; chunk partial sums
    uint8_t* phi = nullptr;
    size_t phi_bytes = 0;
    int64_t phi_rows_pad = 0;
    int64_t phi_npb = 0;             // 8-point blocks
    uint64_t phi_tmap[16] = {};      // the adjoint's tensor map over the folded matrix (a CUtensorMap, 128 B)
    int64_t phi_reps = 0;            // distinct element sums the build formed
    int phi_fwd_kc = 1, phi_adj_kc = 1;
    uint8_t* phi_gforms = nullptr;
    uint8_t* phi_uforms = nullptr;
    float2* phi_part = nullptr;

    // per-kernel timing (diagnostics): event pairs around contraction launches
    bool timing = false;
    std::vector<cudaEvent_t> ev_pool;
    std::vector<int> ev_kind;        // 0 forward, 1 adjoint; pair i uses ev_pool[2i], ev_pool[2i+1]
    size_t ev_used = 0;

    std::vector<void*> allocations;  // every device allocation (freed on destroy)
    int n_device_allocs = 0;         // device allocations attempted so far (fault injection counts them)
};

// Makes a device current for the scope of an entry point and restores the caller's current device
// on return, so that calling the library never changes which device the caller's own CUDA calls use.
// DeviceGuard(-1) only restores (plan creation selects the device itself once it is validated).
// NVTX range over one entry point, named after it: visible in a profiler's timeline, a no-op (one
// branch on an unset pointer) when no tool has injected an NVTX implementation
struct NvtxRange {
    explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
    NvtxRange(const NvtxRange&) = delete;
    NvtxRange& operator=(const NvtxRange&) = delete;
};

struct DeviceGuard {
    int prev = -1;
    cudaError_t err = cudaSuccess;
    explicit DeviceGuard(int device) {
        if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
        if (device >= 0 && device != prev) err = cudaSetDevice(device);
    }
    ~DeviceGuard() {
        int now = -1;
        if (prev >= 0 && cudaGetDevice(&now) == cudaSuccess && now != prev) cudaSetDevice(prev);
    }
    DeviceGuard(const DeviceGuard&) = delete;
    DeviceGuard& operator=(const DeviceGuard&) = delete;
};

// error state (thread-local message) ------------------------------------
cui_status set_error(cui_status s, const std::string& msg);
cui_status check_cuda(cudaError_t e, const char* what);
void count_launch(int n = 1);

// plan construction stages shared by both descriptor forms -----------------
cui_status init_geometry(Plan& p, int n_dims, const int32_t* npts, const int32_t* nel, const int32_t* ppp, int F,
                         int W, int max_objects);
// pref_scale (optional, per global frequency) multiplies every prefactor
cui_status build_metadata(Plan& p, const std::vector<MeasIn>& ms, const std::vector<double2>* pref_scale,
                          std::vector<int>& meas_slot0);
cui_status select_device_and_shapes(Plan& p, int device);
cui_status upload_metadata_and_workspace(Plan& p);
cui_status device_alloc(Plan& p, void** ptr, size_t bytes);
// fault injection of device allocations (CUI_BORN_FAIL_ALLOC=N: the plan's N-th allocation fails)
void release_since(Plan& p, size_t mark);  // frees the plan's allocations made since index `mark`
bool injected_alloc_failure(Plan& p);
// table cache (cui_cache.cu): canonical key of the setup fields the device tables depend on,
// its file path under `dir` (the incident fields alone when the table is not stored), and
// loading / storing p.table (when stored) and p.p_in
cui_status setup_key(const cui_born_setup_desc* d, std::vector<unsigned char>& key);
uint64_t key_hash(const std::vector<unsigned char>& key);
std::string cache_path(const char* dir, const std::vector<unsigned char>& key, bool incident_only);
cui_status cache_load(const std::string& path, const std::vector<unsigned char>& key, Plan& p, bool* hit);
cui_status cache_store(const std::string& path, const std::vector<unsigned char>& key, const Plan& p);

// apply entry points used by the host wrappers ----------------------------
cui_status forward_device(Plan* p, const float2* gamma, int64_t ldg, int B, float2* u, int64_t ldu,
                          cudaStream_t st);
// With `host` (FP64 host columns, leading dimension ld_host) the folded path may write the result
// there itself; *host_written then says it did (else the result is in g as usual).
struct HostOut {
    cui_complex64* host = nullptr;
    int64_t ld = 0;
    bool* written = nullptr;
};
cui_status adjoint_device(Plan* p, const float2* u, int64_t ldu, int B, float2* g, int64_t ldg,
                          cudaStream_t st, HostOut ho = HostOut{});
// n_iter proximal-gradient LASSO iterations, gamma updated in place (no allocation, no synchronisation)
cui_status lasso_device(Plan* p, float2* gamma, int64_t ldg, const float2* um, int64_t ldu, int B, float step,
                        const float* lambda, int n_iter, float* loss, cudaStream_t st);
// um_ready: an event the residual waits on before it reads um (null: um is ready on st)
cui_status vjp_device(Plan* p, const float2* gamma, int64_t ldg, const float2* um, int64_t ldu, int B,
                      float2* grad, int64_t ldgr, float* loss, cudaStream_t st, HostOut ho = HostOut{},
                      cudaEvent_t um_ready = nullptr);

// shared-memory bytes the contraction kernels request
size_t fwd_smem_bytes(const Plan* p, int nc);
// element rows (ey) one FP32 forward block covers: the staged wave columns of a grid line feed
// this many table rows (the 2D arrays have one)
inline int fwd_rows_per_block(int Ey) { return Ey < 4 ? Ey : 4; }
size_t adj_smem_bytes(const Plan* p, int nc);
bool launch_shapes_ok(const Plan* p, std::string* why);
// tensor-core path
bool tc_supported(const Plan* p, std::string* why);
cui_status tc_prepare(Plan& p);
cudaError_t launch_adj_tc(Plan* p, int B, cudaStream_t st);
cudaError_t launch_fwd_tc(Plan* p, const float2* gamma, int64_t ldg, int B, cudaStream_t st);
// line-unit tensor-core kernels: launch the contraction and report how many
// partial-sum slabs (line groups / frequency chunks) the reduction must add
bool tc2_supported(const Plan* p, std::string* why);
cui_status tc2_prepare(Plan& p);
cudaError_t launch_fwd_tc2(Plan* p, const float2* gamma, int64_t ldg, int B, cudaStream_t st, int* groups);
cudaError_t launch_adj_tc2(Plan* p, int B, cudaStream_t st, int* nfc);

// folded operator (split-BF16 GEMMs against the stored observation x point matrix)
size_t phi_matrix_bytes(const Plan* p);
bool phi_supported(const Plan* p, std::string* why);
cui_status phi_prepare(Plan& p);
cudaError_t launch_fwd_phi(Plan* p, const float2* gamma, int64_t ldg, int B, cudaStream_t st, int* n_kc);
cudaError_t launch_adj_phi(Plan* p, const float2* u, int64_t ldu, int B, cudaStream_t st, int* n_kc,
                           cui_complex64* host = nullptr, int64_t ld_host = 0);

// timing hooks around a contraction launch (no-ops unless timing is enabled)
cudaError_t timing_begin(Plan* p, int kind, cudaStream_t st);
cudaError_t timing_end(Plan* p, cudaStream_t st);
void timing_release(Plan* p);

}  // namespace cui

struct cui_born_plan {
    cui::Plan p;
};
