/*
 * cui_born.h -- C-ABI of the GB300 Born scattering operator.
 *
 * Drop-in for the reference toolbox's MEX path (mschiffn/comp_ui_toolbox):
 *   output = scattering.combined_quick_gpu( operator_born, mode, input )
 * (+scattering/combined_quick_gpu.m:11, +scattering/combined_quick_gpu.cu:66-1094),
 * called from operator_born.forward_scalar / adjoint_scalar
 * (+scattering/operator_born.m:217, :286).
 *
 * The MEX function re-reads every operator table from MATLAB and uploads it
 * on each call.  Here the tables are uploaded once into a persistent plan
 * (cui_born_plan_create) and every apply only moves its input and output.
 *
 * Conventions
 *   - complex numbers are interleaved (re, im): cui_complex64 matches
 *     MATLAB's mxComplexDouble, cui_complex32 matches cuComplex / float2;
 *   - matrices are column-major with an explicit leading dimension;
 *   - index arrays copied from MATLAB are 1-based, as MATLAB stores them;
 *   - `stream` is a cudaStream_t passed as void* (0 = legacy default stream);
 *   - device applies are asynchronous on `stream`, allocate nothing and do
 *     not synchronise; one plan serves one stream at a time (its workspace
 *     is shared by all applies of the plan).
 *   - no function ever calls cudaDeviceReset (the reference does on any CUDA
 *     error, +scattering/combined_quick_gpu.h:38-42).
 */
#ifndef CUI_BORN_H
#define CUI_BORN_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes.  The MEX shim maps them onto the reference's error IDs
 * (+scattering/combined_quick_gpu.cu:201, :228, :374, :385, :397, :414,
 * :421, :428 and combined_quick_gpu.h:43). */
typedef enum {
    CUI_OK = 0,
    CUI_ERR_INVALID_ARG = 1,       /* combined_quick_gpu:NoValidDoubleMatrix, :NumberArguments, :NoNumericScalarMode */
    CUI_ERR_UNSUPPORTED_SETUP = 2, /* combined_quick_gpu:NoSymmetricGridsSetup (index map is not a lateral shift) */
    CUI_ERR_OOM = 3,               /* device or host allocation failed */
    CUI_ERR_CUDA = 4,              /* adjoint_quick_gpu:ErrorCUDA */
    CUI_ERR_TIMEOUT = 5,           /* a bounded device-side wait gave up */
    CUI_ERR_NUMERIC = 6,           /* non-finite table entries */
    CUI_ERR_NO_DEVICE = 7          /* combined_quick_gpu:NoCUDADevices / :InvalidCUDADevice */
} cui_status;

typedef struct { double re, im; } cui_complex64;
typedef struct { float re, im; } cui_complex32;

typedef struct cui_born_plan cui_born_plan;

/* One mixed voltage signal of a pulse-echo measurement
 * (sequence.settings(m).rx(mix), sequence.prefactors{m}(mix)). */
typedef struct {
    int32_t n_f;                          /* number of frequencies of the mix */
    const int32_t* indices_f_to_unique;   /* [n_f] 1-based into the measurement's unique frequencies
                                             (settings(m).indices_f_to_unique{mix}, read at .cu:313) */
    int32_t n_active;                     /* number of active elements */
    const int32_t* indices_active;        /* [n_active] 1-based element indices (rx(mix).indices_active, .cu:309) */
    const cui_complex64* prefactors;      /* [n_f x n_active] column-major (prefactors{m}(mix).samples.values, .cu:352) */
} cui_mix_desc;

/* One sequential pulse-echo measurement (incident wave). */
typedef struct {
    int32_t n_f;                          /* unique frequencies of the measurement */
    const int32_t* indices_f_to_unique;   /* [n_f] 1-based into the global unique frequencies
                                             (sequence.indices_f_to_unique{m}, .cu:278) */
    const cui_complex64* p_incident;      /* [n_f x N_points] column-major
                                             (incident_waves(m).p_incident.samples.values, .cu:817-823) */
    int32_t n_mixes;
    const cui_mix_desc* mixes;
} cui_measurement_desc;

typedef enum {
    /* sequence.h_ref.samples.values [n_f_unique x N_points] plus
     * setup.indices_grid_FOV_shift [N_points x N_elements] (1-based), exactly
     * what the MEX reads (.cu:231, :382-391).  The plan checks that the map
     * is the symmetric-grid lateral shift (setup_grid_symmetric.m:175-232)
     * and stores the distinct entries as a lateral-offset table. */
    CUI_TABLE_REFERENCE = 0,
    /* The lateral-offset table itself: entry (f, z, [o_y,] o_x) is the
     * transfer function of an element at signed lateral grid offset
     * i_d - e_d*ppp_d = o_d - (E_d-1)*ppp_d, depth index z; column-major
     * [No_x x (No_y) x N_z x n_f_unique], No_d = N_d + (E_d-1)*ppp_d. */
    CUI_TABLE_LATERAL = 1
} cui_table_form;

/* Everything combined_quick_gpu reads from the operator (.cu:203-393). */
typedef struct {
    int32_t n_dims;                 /* 2 or 3 (FOV grid dimensions) */
    int32_t n_points_axis[3];       /* FOV grid points: lateral axes then axial (FOV.shape.grid.N_points_axis) */
    int32_t n_elements_axis[2];     /* array elements per lateral axis (xdc_array.N_elements_axis) */
    int32_t n_points_per_pitch[2];  /* setup.N_points_per_pitch_axis */
    int32_t n_f_unique;             /* rows of h_ref (.cu:394) */
    int32_t table_form;             /* cui_table_form */
    const cui_complex64* h_ref;                 /* CUI_TABLE_REFERENCE */
    const int32_t* indices_grid_FOV_shift;      /* CUI_TABLE_REFERENCE */
    const cui_complex64* h_lateral;             /* CUI_TABLE_LATERAL */
    int32_t n_measurements;         /* selected measurements (indices_measurement_sel, .cu:238) */
    const cui_measurement_desc* measurements;
    int32_t device;                 /* CUDA device (options.momentary.gpu.index, .cu:378) */
} cui_born_desc;

/* Work and storage figures of a plan (bytes and complex multiply-adds). */
typedef struct {
    int64_t n_points;               /* N_points */
    int64_t n_observations;         /* rows of the forward output (sequence.size(1)) */
    int64_t n_elements;
    int64_t n_slots;                /* (measurement, unique frequency) pairs */
    int64_t n_f_unique;
    int64_t table_bytes;            /* device bytes of the lateral table */
    int64_t incident_bytes;         /* device bytes of all incident fields */
    int64_t workspace_bytes;        /* device scratch owned by the plan */
    int64_t contraction_macs;       /* complex MACs of one dense apply per object: sum_slots E*P */
    int64_t channel_macs;           /* channel-contraction entries per object and dense apply:
                                       sum_slots min(rows of the slot, distinct active elements) * P
                                       (the element sum folded into the receive mixes) */
    int64_t folded_bytes;           /* device bytes of the folded operator (0 until built) */
    int64_t folded_sums;            /* distinct element sums the folded build formed */
    int64_t device_allocations;     /* device allocations the plan has attempted so far (the count
                                       CUI_BORN_FAIL_ALLOC=N refers to: the N-th of them fails) */
} cui_born_info;

/* ---- setup form: tables built on the device ---------------------------------
 * Instead of the precomputed tables, the caller describes the discretised
 * setup; the plan computes the lateral transfer-function table (distances and
 * phases in FP64, the rest in FP32; setup.m:1216-1281, greens_function.m:88/103,
 * on.m:64-70, raised_cosine.m:106-119), the incident fields
 * (sequence.m:813-844) and the prefactors -dV k~^2 R (setup.m:759,
 * sequence.m:623) on the GPU. */
typedef enum { CUI_ABSORPTION_NONE = 0, CUI_ABSORPTION_TIME_CAUSAL = 1 } cui_absorption_kind;

typedef struct {
    int32_t kind;          /* cui_absorption_kind */
    double c;              /* none: c_0; time_causal: c_ref (m/s) */
    double constant_db;    /* time_causal: absorption constant (dB/cm), time_causal.m:82 */
    double slope_db;       /* time_causal: slope (dB/(MHz^y cm)), time_causal.m:83 */
    double exponent;       /* time_causal: y */
    double f_ref;          /* time_causal: reference frequency (Hz) */
    int32_t dispersion;    /* time_causal: nonzero = causal dispersion, time_causal.m:124-136 */
} cui_absorption_desc;

/* One incident wave (sequential pulse-echo measurement) of the setup form. */
typedef struct {
    int32_t n_f;                          /* unique frequencies of the wave */
    const int32_t* indices_f_to_unique;   /* [n_f] 1-based into f_unique */
    const cui_complex64* v_d;             /* [n_f x N_elements] column-major normal velocities
                                             (settings(m).v_d_unique, tx.m:284; zero = inactive) */
    int32_t n_mixes;
    const cui_mix_desc* mixes;            /* here `prefactors` holds the receive responses R
                                             (DFT of the mixer impulse responses); the plan
                                             multiplies them by -dV k~(f)^2 */
} cui_wave_desc;

typedef struct {
    int32_t n_dims;                 /* 2 or 3 */
    int32_t n_points_axis[3];       /* FOV grid points: lateral axes then axial */
    double delta_axis[3];           /* FOV grid spacing (m) */
    double z_start;                 /* axial position of the FOV's near edge (m); rows at z_start + (k+1/2) dz */
    int32_t n_elements_axis[2];
    double pitch_axis[2];           /* element pitch (m); must be an integer multiple of the lateral spacing */
    double width_axis[2];           /* element face width (m) */
    int32_t n_face_axis[2];         /* quadrature points across each face axis */
    cui_absorption_desc absorption;
    double aa_tx_beta, aa_rx_beta;  /* raised-cosine roll-off of the anti-aliasing filters; < 0 = off */
    int32_t n_f_unique;
    const double* f_unique;         /* [n_f_unique] global unique frequencies (Hz) */
    int32_t n_measurements;
    const cui_wave_desc* waves;
    int32_t device;
    /* Face weights (face.m:234-285 compute_weights; applied in setup.m:1241-1269): the lateral
       table sums w_q(f) G(k~(f), |r - r_q|) over the face's quadrature points q, with
       w_q(f) = a_q exp(-j k_lens(f) t_q), the same on every element.  Zero-initialised fields
       give uniform weights (a_q = 1, t_q = 0), the table of the fields above alone. */
    const double* face_apodization;  /* [n_face_axis[0] x n_face_axis[1]] apodization a_q at the face
                                        points, first axis fastest: the face's apodization function
                                        evaluated at the normalised positions 2 (r_q - r_c) / width
                                        (face.m:210-217); NULL = uniform (apodization/uniform.m) */
    double lens_focus_axis[2];       /* axial focus (m) per face axis of the lens thickness profile
                                        t_q (thickness/focus_axial.m); 0 or +inf = not focused along
                                        that axis */
    double lens_c;                   /* speed of sound of the lens (m/s), lossless (lens.m's default
                                        absorption model); 0 = 1540 */
} cui_born_setup_desc;

/* ---- plan lifetime ------------------------------------------------------ */
/* Validates the descriptor, converts every table to FP32 in the device
 * layout and uploads it.  Replaces the per-call host conversion and uploads
 * of .cu:520-850.  `max_objects` bounds the number of columns of one apply
 * (it sizes the plan's workspace). */
cui_status cui_born_plan_create(const cui_born_desc* desc, int32_t max_objects, cui_born_plan** plan);
/* Same plan from the setup form (tables computed on the device). */
cui_status cui_born_plan_create_setup(const cui_born_setup_desc* desc, int32_t max_objects, cui_born_plan** plan);
/* Same, through an on-disk cache of the two device-built arrays (the lateral
 * table and the incident fields), keyed like compute_or_load_hash
 * (+auxiliary/compute_or_load_hash.m:65-185): the file
 * `cache_dir`/cui_born_<cui_born_setup_hash>.tables is loaded when it exists,
 * else the arrays are computed and stored there (written to a temporary name,
 * then renamed).  A file whose stored setup differs from `desc` is a hash
 * collision: CUI_ERR_INVALID_ARG, as in the reference (:90-107).  `*loaded`
 * (may be NULL) = 1 loaded, 0 computed and stored, -1 computed but not stored
 * (the plan is still returned; cui_last_error() says why). */
cui_status cui_born_plan_create_setup_cached(const cui_born_setup_desc* desc, int32_t max_objects,
                                             const char* cache_dir, cui_born_plan** plan, int32_t* loaded);
/* Hash of the setup fields the device tables depend on -- grid, array, faces,
 * medium, anti-aliasing, frequencies, each wave's frequency map and normal
 * velocities; not the receive mixes or the device -- as 16 hex digits and a
 * NUL in `hex17`.  Host only (no GPU). */
cui_status cui_born_setup_hash(const cui_born_setup_desc* desc, char* hex17);
/* Storage of the lateral transfer-function table of a setup-form plan (no
 * counterpart in the reference, which always holds h_ref: operator.m:76-88).
 *   CUI_STORAGE_STORED: built once at creation ([F][Nz][Noy][Nox] FP32), read by
 *     every apply.
 *   CUI_STORAGE_STREAMED (3D setups): never stored whole; every apply regenerates
 *     it one chunk of frequencies at a time into a chunk buffer (about 512 MiB;
 *     the environment variable CUI_BORN_STREAM_FREQUENCIES caps the frequencies
 *     per chunk) that the contraction kernels read before the next chunk
 *     replaces it.  table_bytes is the buffer's size.
 *   CUI_STORAGE_GENERATED (3D setups): never stored at all; the contraction and
 *     received-energy kernels compute each entry where they stage it.  No table
 *     memory (table_bytes 0), at about 1.5x the apply time of the other two.
 * Generated entries are formed in FP32 with the distance and the phase range
 * reduction in FP32 pairs (relative entry error below 1e-6; the stored table
 * keeps distances and phases in FP64, the rest in FP32, entry error below 4e-7).  Streamed and generated plans run the
 * FP32 CUDA-core kernels only (cui_born_set_precision(BF16X3) is
 * CUI_ERR_UNSUPPORTED_SETUP); their received energies, the Phi columns of
 * cui_born_omp / cui_born_cosamp and cui_born_forward_static generate the
 * entries in the kernel.  Their incident
 * fields are stored, built from transmit-table chunks of a few frequencies.
 *   CUI_STORAGE_AUTO: stored, unless the table and the incident fields would not
 *     fit in the device's free memory; then streamed (3D; generated if not even
 *     the chunk buffer fits) or CUI_ERR_OOM (2D).
 * cui_born_plan_create_setup uses CUI_STORAGE_AUTO. */
typedef enum {
    CUI_STORAGE_AUTO = 0,
    CUI_STORAGE_STORED = 1,
    CUI_STORAGE_GENERATED = 2,
    CUI_STORAGE_STREAMED = 3
} cui_table_storage;
/* `cache_dir` (may be NULL) and `loaded` (may be NULL) as in
 * cui_born_plan_create_setup_cached; a streamed or generated plan caches only
 * the incident fields, in `cache_dir`/cui_born_<hash>.incident. */
cui_status cui_born_plan_create_setup_ex(const cui_born_setup_desc* desc, int32_t max_objects, int32_t storage,
                                         const char* cache_dir, cui_born_plan** plan, int32_t* loaded);
/* The storage a plan uses (CUI_STORAGE_STORED, _STREAMED or _GENERATED). */
cui_status cui_born_plan_table_storage(const cui_born_plan* plan, int32_t* storage);
cui_status cui_born_plan_destroy(cui_born_plan* plan);
cui_status cui_born_plan_info(const cui_born_plan* plan, cui_born_info* info);

/* combined_scalar mode 0 (+scattering/operator.m:1042-1045): operator size. */
cui_status cui_born_size(const cui_born_plan* plan, int64_t* n_observations, int64_t* n_points);

/* ---- device applies (FP32, device pointers) ------------------------------
 * Forward, mode 1 (.cu:902-909; operator_born.m:332-470):
 *   u[:, b] = Phi * gamma[:, b],  gamma: N_points x n_objects, u: N_obs x n_objects.
 * Rows of u are ordered measurement -> mix -> frequency (.cu:978). */
cui_status cui_born_forward(cui_born_plan* plan, const cui_complex32* gamma, int64_t ld_gamma,
                            int32_t n_objects, cui_complex32* u, int64_t ld_u, void* stream);

/* Forward that allocates nothing.  No counterpart in the reference: its MEX
 * allocates device memory on every call.  Same operation and arguments as
 * cui_born_forward, for callers that must not allocate device memory when
 * they apply the operator: plug-in hosts that hand a plug-in a fixed
 * device-memory budget and refuse further allocations, and real-time loops
 * that must not enter the allocator (and its possible synchronisation)
 * between frames.  It always runs the FP32 CUDA-core kernels, whatever
 * cui_born_set_precision chose for the plan.  Partial sums live in a 16 MiB
 * file-scope device array that each GPU loading the library holds until
 * exit, so slots x n_objects x elements x 16 B must not exceed 16 MiB, and
 * n_objects x (slot passes of the widest frequency) must not exceed 65535
 * (else CUI_ERR_INVALID_ARG).  The first call on a device looks up the
 * array's device address (cudaGetSymbolAddress) and keeps it for devices 0-63
 * (a plan on a higher device index: CUI_ERR_INVALID_ARG).  All calls share the
 * array: calls that overlap on the GPU (other streams, other plans, other
 * threads) race. */
cui_status cui_born_forward_static(cui_born_plan* plan, const cui_complex32* gamma, int64_t ld_gamma,
                                   int32_t n_objects, cui_complex32* u, int64_t ld_u, void* stream);

/* Adjoint, mode 2 (.cu:914-921; operator_born.m:480-596):
 *   gamma_hat[:, b] = Phi^H * u[:, b]. */
cui_status cui_born_adjoint(cui_born_plan* plan, const cui_complex32* u, int64_t ld_u,
                            int32_t n_objects, cui_complex32* gamma_hat, int64_t ld_gamma, void* stream);

/* Vector-Jacobian product of the data-fidelity term used by the
 * reference's solvers (operator.m:717 -> omp.m:170, spgl1.m:154):
 *   r = Phi*gamma - u_meas,  loss[b] = 0.5*||r[:, b]||^2,  grad = Phi^H r.
 * `loss` is a device pointer to n_objects floats (may be NULL). */
cui_status cui_born_vjp(cui_born_plan* plan, const cui_complex32* gamma, int64_t ld_gamma,
                        const cui_complex32* u_meas, int64_t ld_u, int32_t n_objects,
                        cui_complex32* grad, int64_t ld_grad, float* loss, void* stream);

/* Proximal-gradient (ISTA) LASSO iterations of the data-fidelity term above,
 * the solver loop the reference drives through combined_scalar
 * (+scattering/operator.m:717, lq_minimization :601-790):
 *   r = Phi*gamma - u_meas;  gamma <- S(gamma - step * Phi^H r, step * lambda[b])
 * with the complex soft threshold S(v, t) = v * max(0, 1 - t/|v|), n_iter times,
 * gamma (device, n_points x n_objects) updated in place.  `lambda` is a device
 * array of n_objects floats; `step` should not exceed 1/||Phi||^2.  `loss`
 * (device, may be NULL) receives 0.5*||r||^2 of the last iteration's iterate.
 * Every launch goes to `stream` and nothing is allocated or synchronised, so a
 * caller may capture the iterations of one or many plans into a CUDA graph. */
cui_status cui_born_lasso(cui_born_plan* plan, const cui_complex32* u_meas, int64_t ld_u, int32_t n_objects,
                          cui_complex32* gamma, int64_t ld_gamma, const float* lambda, float step, int32_t n_iter,
                          float* loss, void* stream);

/* Received energies in the canonical basis, energy_rx of the reference
 * (+scattering/operator_born.m:718-859, energy_rx_canonical; used to normalise
 * the operator before a solve, +regularization/+options/common.m:166-184):
 *   energy[p] = sum over observations of |Phi[row, p]|^2 = ||Phi e_p||^2,
 * p = 0..N_points-1, written to the device array `energy` (N_points floats).
 * TGC is the identity.  Allocates nothing; launches only on `stream`. */
cui_status cui_born_energy_rx(cui_born_plan* plan, float* energy, void* stream);

/* Orthogonal matching pursuit on one measured column, omp.m of the reference
 * (+regularization/+algorithms/+greedy/omp.m:161-200, reached through
 * +scattering/operator.m:601-790 with op_A = combined_scalar):
 *   per iteration the atom maximising |Phi^H r| (ties to the smaller index),
 *   the least-squares coefficients of y on the atoms so far, and the residual
 *   r = y - Phi_sel c; stops after n_atoms_max atoms or once ||r|| / ||y||
 *   <= rel_rmse (omp.m:215).
 * `y` is a device array of N_obs values.  Host outputs: `atoms` (n_atoms_max
 * grid-point indices, 0-based), `coefficients` (n_atoms_max), `rel_residuals`
 * (n_atoms_max, may be NULL: ||r|| / ||y|| after each atom), `*n_atoms` the
 * number of atoms taken.  The least squares is kept as an orthonormal basis of
 * the selected columns (Gram-Schmidt, twice); the columns come straight from
 * the tables, not from a forward apply.  Allocates device scratch of about
 * (n_atoms_max + 3) * N_obs + N_points complex values per call and
 * synchronises `stream` once per iteration. */
cui_status cui_born_omp(cui_born_plan* plan, const cui_complex32* y, int32_t n_atoms_max, float rel_rmse,
                        int64_t* atoms, cui_complex32* coefficients, float* rel_residuals, int32_t* n_atoms,
                        void* stream);

/* Compressive sampling matching pursuit on one measured column, cosamp.m of the
 * reference (+regularization/+algorithms/+greedy/cosamp.m:174-272):
 *   per iteration the 2s largest entries of |Phi^H r| (ties to the smaller
 *   index), their union with the current s atoms, the least-squares fit of y on
 *   the union, pruning to the s largest coefficient magnitudes, and the
 *   residual r = y - Phi_s c_s with the pruned coefficients (not refitted);
 *   stops after n_iter_max iterations or once ||r|| / ||y|| <= rel_rmse (:270).
 * s = `sparsity`, 1 <= s <= 512, 2s <= N_points, 3s <= N_obs (else
 * CUI_ERR_INVALID_ARG).  `y` is a device array of N_obs values.  Host outputs:
 * `atoms` and `coefficients` (s each: the final support in the reference's
 * order, largest coefficient first), `rel_residuals` (n_iter_max, may be NULL),
 * `*n_iter` the iterations run.  The least squares is a device Gram matrix
 * (FP64 sums) solved by a diagonally pivoted Cholesky in FP64 with two
 * refinement steps; columns that are dependent to the Gram matrix's accuracy
 * get coefficient 0, as the basic solution of the reference's pivoted-QR
 * A \ y (cosamp.m:244) does for a rank-deficient A.  Allocates
 * device scratch of about (3s + 2) * N_obs + 2 * N_points values per call and
 * synchronises `stream` a few times per iteration. */
cui_status cui_born_cosamp(cui_born_plan* plan, const cui_complex32* y, int32_t sparsity, int32_t n_iter_max,
                           float rel_rmse, int64_t* atoms, cui_complex32* coefficients, float* rel_residuals,
                           int32_t* n_iter, void* stream);

/* ---- host applies (FP64, MEX semantics) ----------------------------------
 * output = combined_quick_gpu(operator_born, mode, input): mode 1 forward
 * (input N_points x n_objects), mode 2 adjoint (input N_obs x n_objects).
 * Host buffers in MATLAB's interleaved complex double; FP64 <-> FP32
 * conversion and host <-> device copies happen inside, synchronously.  Where
 * the GPU reads pageable host memory through the host's page tables (Grace
 * systems: ATS over NVLink-C2C), kernels read the caller's arrays and write
 * the result into them directly; elsewhere the data pass through pinned
 * staging buffers the plan keeps (also selected by CUI_BORN_HOST_STAGING=1). */
cui_status cui_born_combined_host(cui_born_plan* plan, int32_t mode, const cui_complex64* input,
                                  int64_t ld_in, int32_t n_objects, cui_complex64* output, int64_t ld_out);

/* Host LASSO: n_iter proximal-gradient iterations (as cui_born_lasso) on host FP64
 * buffers: u_meas [N_obs x n_objects] (ld_u), gamma [N_points x n_objects]
 * (ld_gamma) the start iterate on entry and the result on return, lambda [n_objects]
 * thresholds in host memory.  Synchronous.  The MEX form of the solver loop that
 * lq_minimization (operator.m:601-790) drives through combined_scalar (:717). */
cui_status cui_born_lasso_host(cui_born_plan* plan, const cui_complex64* u_meas, int64_t ld_u, int32_t n_objects,
                               cui_complex64* gamma, int64_t ld_gamma, const float* lambda, float step,
                               int32_t n_iter);

/* How the host entry points move data: *direct = 1 when kernels read and write
 * the caller's FP64 arrays through the host's page tables (GPUs with
 * cudaDevAttrPageableMemoryAccessUsesHostPageTables, such as Grace systems), 0
 * when the data pass through the plan's pinned staging buffers (also forced by
 * CUI_BORN_HOST_STAGING=1 before the first host call). */
cui_status cui_born_host_path(cui_born_plan* plan, int32_t* direct);

/* Host VJP: same as cui_born_vjp with host FP64 buffers; loss may be NULL.
 * Synchronous.  With the direct path, u_meas is read on a non-blocking stream
 * the plan owns while the forward runs; the call returns only after that read
 * has ended (also on errors), so the caller may free u_meas on return. */
cui_status cui_born_vjp_host(cui_born_plan* plan, const cui_complex64* gamma, int64_t ld_gamma,
                             const cui_complex64* u_meas, int64_t ld_u, int32_t n_objects,
                             cui_complex64* grad, int64_t ld_grad, double* loss);

/* ---- precision ------------------------------------------------------------
 * CUI_PRECISION_FP32: FP32 CUDA-core contractions (default).
 * CUI_PRECISION_BF16X3: the forward and adjoint contractions over (slot,
 * element) run on the tcgen05 tensor cores with every operand split into
 * bf16 hi + lo and the three products hi*hi + hi*lo + lo*hi accumulated in
 * FP32 (2D setups, <= 128 elements).  Switching to BF16X3 builds the split
 * band tables once (allocates).
 * CUI_PRECISION_BF16X3_FOLDED: the same split-BF16 arithmetic as two tcgen05
 * GEMMs against the operator folded over its receive mixes and stored in
 * device memory: one row per observation (w, m, f), sum over the mix's active
 * elements of prefactor x table entry x incident field, the reference's
 * per-element Phi matrices (combined_quick_gpu.cu:1099-1124) summed over e.
 * It does min(mixes, active elements) / active elements of the element
 * contraction's multiply-adds and reads 8 bytes per observation x grid point
 * and apply direction (per 64-column pass); it needs a stored table and that
 * much free device memory (CUI_ERR_UNSUPPORTED_SETUP otherwise).  Switching
 * to it builds the matrix once (allocates).  Objects are applied 64 at a time. */
typedef enum {
    CUI_PRECISION_FP32 = 0,
    CUI_PRECISION_BF16X3 = 1,
    CUI_PRECISION_BF16X3_FOLDED = 2
} cui_precision;

cui_status cui_born_set_precision(cui_born_plan* plan, int32_t precision);

/* Autotuner (no counterpart in the reference, whose MEX has one path): times one
 * forward + adjoint apply of each path this plan can run for `n_objects`
 * columns -- the FP32 CUDA-core kernels and, for 2D setups, the split-BF16
 * tensor-core kernels -- on `stream` and keeps the faster (as
 * cui_born_set_precision would).  Both paths meet the operator's accuracy bound.
 * When the split-BF16 line-unit kernels win, it then searches their launch
 * shapes (column tiles, blocks per launch; cui_born_autotune_config) one at a
 * time and keeps each that lowers the timed pair; `ms[1]` is the tuned time.
 * Allocates and frees scratch buffers and synchronises: call it at set-up,
 * before any stream capture.  `precision` (may be NULL) receives the choice,
 * `ms` (may be NULL) the two times in ms (FP32, BF16X3; -1 when not run). */
cui_status cui_born_autotune(cui_born_plan* plan, int32_t n_objects, int32_t* precision, double* ms, void* stream);
/* Launch shapes the last cui_born_autotune picked for the split-BF16 line-unit
 * kernels (0 everywhere: the built-in rule): `narrow_tiles` 1 when column tiles
 * of at most 32 columns replaced the 64-column tiles, and the block counts the
 * forward's line groups (`fwd_blocks`) and the adjoint's frequency chunks
 * (`adj_blocks`) aim at.  Any pointer may be NULL. */
cui_status cui_born_autotune_config(const cui_born_plan* plan, int32_t* narrow_tiles, int32_t* fwd_blocks,
                                    int32_t* adj_blocks);
/* Sets those launch shapes directly (0 everywhere restores the rule), e.g. to
 * reuse a choice cui_born_autotune made on an earlier run.  Every combination
 * gives results within the operator's accuracy bound. */
cui_status cui_born_set_launch_shapes(cui_born_plan* plan, int32_t narrow_tiles, int32_t fwd_blocks,
                                      int32_t adj_blocks);

/* ---- diagnostics ----------------------------------------------------------- */
/* Device time of the two contraction kernels, from CUDA events recorded on
 * the launching stream around each launch while timing is enabled. */
typedef struct {
    int64_t n_forward;      /* forward contraction launches since the last read */
    int64_t n_adjoint;      /* adjoint contraction launches since the last read */
    double ms_forward;      /* summed device time of those launches (ms) */
    double ms_adjoint;
} cui_born_timing;

cui_status cui_born_timing_enable(cui_born_plan* plan, int32_t enable);
/* Wall-clock limit of every wait of the tensor-core kernels for an operand stage or an
 * accumulator (no counterpart in the reference, whose kernels do not wait): a block
 * whose wait runs out stops, drains its copies and MMAs (those drains keep a fixed
 * 1 s limit), frees its tensor memory and raises the plan's status word, which
 * cui_born_plan_status reports as CUI_ERR_TIMEOUT; blocks of later launches skip
 * their work until the status is read.  nanoseconds = 0 restores the default of
 * 1 s; otherwise 1 ns to 60 s. */
cui_status cui_born_set_wait_limit(cui_born_plan* plan, int64_t nanoseconds);
/* Occupancy compaction of the FP32 forward (operator_born.m:361, combined_quick_gpu.cu:457-499:
 * the reference contracts only the grid points where some column of gamma is nonzero).  Every
 * FP32 forward first lists those points on the device; when there are at most max_points of
 * them it contracts over the list (work proportional to their number), otherwise it runs the
 * dense kernels.  The choice is made on the device (no synchronisation).  max_points = -1
 * selects the default, N_points / 16 with a stored table and N_points / 32 with
 * a streamed or generated one; 0 turns the compaction off.  The split-BF16 paths
 * always contract densely. */
cui_status cui_born_set_occupancy_limit(cui_born_plan* plan, int64_t max_points);
/* Reads and clears the plan's device status word; CUI_ERR_TIMEOUT when a
 * bounded device-side wait gave up since the last call. */
cui_status cui_born_plan_status(cui_born_plan* plan, int32_t* device_status);
/* Waits for the recorded events, returns the sums and clears them. */
cui_status cui_born_timing_read(cui_born_plan* plan, cui_born_timing* out);

const char* cui_status_string(cui_status status);
/* Message of the last failing call on this thread (empty if none). */
const char* cui_last_error(void);
/* Number of kernel launches issued by this process (all plans). */
int64_t cui_launch_count(void);

#ifdef __cplusplus
}
#endif

#endif /* CUI_BORN_H */
