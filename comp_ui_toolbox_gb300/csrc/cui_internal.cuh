// Internal declarations shared by the translation units of libcui_born.
//
// Device layout of a plan (all FP32 complex as float2):
//   table   [F][Nz][Noy][Nox]  lateral-offset transfer-function table; row (f, z, oy)
//                              is contiguous in ox.  No_d = N_d + (E_d-1)*ppp_d.
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

namespace cui {

// Column chunk width of the FP32 contraction kernels: the number of slots
// (incident waves sharing one frequency) one thread block processes per pass.
constexpr int kMaxNC = 16;

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
    float2* table = nullptr;
    float2* p_in = nullptr;
    int* f_slot_ptr = nullptr;      // [F+1] CSR of slots per global frequency
    int* f_slot_list = nullptr;     // [S]
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

    // workspace (sized for max_objects at creation; shared by all applies)
    float2* ws_part = nullptr;      // forward / adjoint partial sums
    size_t ws_part_bytes = 0;
    float2* ws_G = nullptr;         // [S][B][E] element signals / unmixed data
    float2* ws_r = nullptr;         // [B][n_obs] residual of the VJP
    int* ws_occ = nullptr;          // [P] occupied points (sparse forward)
    int* ws_occ_count = nullptr;    // [2] occupied-point count, spare
    float* ws_loss = nullptr;       // [B] loss partial sums

    // launch geometry chosen at creation
    int fwd_groups = 1;             // line groups of the dense forward
    int fwd_lines_per_group = 1;
    int adj_fchunk = 1;             // frequencies per adjoint block
    int adj_nfc = 1;                // adjoint frequency chunks
    int Nj_max = 1;                 // steps per residue along x
    int Ni = 1;                     // staged table entries per residue
    size_t table_bytes = 0, incident_bytes = 0, workspace_bytes = 0;

    // host-side pinned staging for the FP64 host entry points
    float2* h_stage_in = nullptr;
    float2* h_stage_out = nullptr;
    size_t h_stage_elems = 0;
    float2* d_stage_in = nullptr;   // device copies for the host entry points
    float2* d_stage_out = nullptr;
    float2* d_stage_aux = nullptr;
    float* d_stage_loss = nullptr;

    std::vector<void*> allocations;  // every device allocation (freed on destroy)
};

// error state (thread-local message) ------------------------------------
cui_status set_error(cui_status s, const std::string& msg);
cui_status check_cuda(cudaError_t e, const char* what);
void count_launch(int n = 1);

// apply entry points used by the host wrappers ----------------------------
cui_status forward_device(Plan* p, const float2* gamma, int64_t ldg, int B, float2* u, int64_t ldu,
                          cudaStream_t st);
cui_status adjoint_device(Plan* p, const float2* u, int64_t ldu, int B, float2* g, int64_t ldg,
                          cudaStream_t st);
cui_status vjp_device(Plan* p, const float2* gamma, int64_t ldg, const float2* um, int64_t ldu, int B,
                      float2* grad, int64_t ldgr, float* loss, cudaStream_t st);

// shared-memory bytes the contraction kernels request
size_t fwd_smem_bytes(const Plan* p, int nc);
size_t adj_smem_bytes(const Plan* p, int nc);
bool launch_shapes_ok(const Plan* p, std::string* why);

}  // namespace cui

struct cui_born_plan {
    cui::Plan p;
};
