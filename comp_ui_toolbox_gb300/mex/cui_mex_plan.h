/* Plan building and caching shared by the MEX gateways (cui_born_mex.c, cui_lasso_mex.c).
 *
 * Reads the operator_born properties the reference's gateway reads
 * (+scattering/combined_quick_gpu.cu:203-393, :817-823) plus the grid geometry the
 * plan needs (setup.FOV.shape.grid.N_points_axis, setup.xdc_array.N_elements_axis,
 * setup.N_points_per_pitch_axis), validates them with the reference's error
 * identifiers, and keeps one plan per MEX file: MATLAB loads every MEX file as its
 * own shared library, so each gateway that includes this header has its own cache.
 * The cached plan is rebuilt when the operator changes -- detected by a 64-bit hash
 * over every array the plan is built from (sizes, index maps, prefactors, h_ref and
 * the incident fields: one pass over them, about 1 s per 8 GB) -- or when a call has
 * more objects than the plan was built for.  mexAtExit destroys it. */
#ifndef CUI_MEX_PLAN_H
#define CUI_MEX_PLAN_H

#include <stddef.h>
#include <stdint.h>
#include <string.h>

#include "cui_born.h"
#include "mex.h"

static cui_born_plan* g_cui_plan = NULL;
static uint64_t g_cui_plan_key = 0;
static int32_t g_cui_plan_objects = 0;

static void cui_mex_cleanup(void) {
    if (g_cui_plan) cui_born_plan_destroy(g_cui_plan);
    g_cui_plan = NULL;
    g_cui_plan_key = 0;
    g_cui_plan_objects = 0;
}

/* the reference's error identifier for a library status */
static const char* cui_mex_error_id(cui_status st) {
    switch (st) {
        case CUI_ERR_INVALID_ARG: return "combined_quick_gpu:NoValidDoubleMatrix";
        case CUI_ERR_UNSUPPORTED_SETUP: return "combined_quick_gpu:NoSymmetricGridsSetup";
        case CUI_ERR_NO_DEVICE: return "combined_quick_gpu:InvalidCUDADevice";
        default: return "adjoint_quick_gpu:ErrorCUDA";
    }
}

static void cui_mex_fail(cui_status st, const char* what) {
    mexErrMsgIdAndTxt(cui_mex_error_id(st), "%s: %s: %s", what, cui_status_string(st), cui_last_error());
}

static mxArray* cui_mex_prop(const mxArray* o, mwIndex i, const char* name) {
    mxArray* p = o ? mxGetProperty(o, i, name) : NULL;
    if (!p) mexErrMsgIdAndTxt("combined_quick_gpu:NoOperatorBorn", "operator_born has no property %s", name);
    return p;
}

static const mxComplexDouble* cui_mex_complex(const mxArray* a, const char* what) {
    if (!(mxIsDouble(a) && mxIsComplex(a)))
        mexErrMsgIdAndTxt("combined_quick_gpu:NoComplexDoubles", "%s must be complex doubles!", what);
    return mxGetComplexDoubles(a);
}

/* 1-based doubles -> int32 (mxMalloc'ed; MATLAB frees it when the MEX call returns) */
static int32_t* cui_mex_index(const mxArray* a) {
    const size_t n = mxGetNumberOfElements(a);
    const double* d = mxGetDoubles(a);
    int32_t* v = (int32_t*)mxMalloc((n ? n : 1) * sizeof(int32_t));
    if (!d && n) mexErrMsgIdAndTxt("combined_quick_gpu:NoOperatorBorn", "index arrays must be real doubles");
    for (size_t i = 0; i < n; ++i) v[i] = (int32_t)d[i];
    return v;
}

static uint64_t cui_mex_hash(uint64_t h, const void* data, size_t bytes) {
    const unsigned char* c = (const unsigned char*)data;
    size_t i = 0;
    for (; i + 8 <= bytes; i += 8) {
        uint64_t w;
        memcpy(&w, c + i, 8);
        h = (h ^ w) * 0x100000001b3ull;
        h ^= h >> 29;
    }
    for (; i < bytes; ++i) h = (h ^ c[i]) * 0x100000001b3ull;
    return h;
}

/* The plan for operator `op` and `n_objects` columns: the cached one when the operator's arrays
 * hash to the cached key and it holds enough objects, else a new one.  Every failure raises the
 * reference's error identifiers (combined_quick_gpu.cu:201-441). */
static cui_born_plan* cui_mex_plan(const mxArray* op, int32_t n_objects) {
    if (!(mxIsClass(op, "scattering.operator_born") && mxIsScalar(op)))
        mexErrMsgIdAndTxt("combined_quick_gpu:NoOperatorBorn", "operator_born must be a single scattering.operator_born!");
    mxArray* seq = cui_mex_prop(op, 0, "sequence");
    mxArray* setup = cui_mex_prop(seq, 0, "setup");
    if (!mxIsClass(setup, "scattering.sequences.setups.setup_grid_symmetric"))
        mexErrMsgIdAndTxt("combined_quick_gpu:NoSymmetricGridsSetup",
                          "sequence.setup must be scattering.sequences.setups.setup_grid_symmetric!");
    mxArray* gpu = cui_mex_prop(cui_mex_prop(cui_mex_prop(op, 0, "options"), 0, "momentary"), 0, "gpu");
    if (!mxIsClass(gpu, "scattering.options.gpu_active"))
        mexErrMsgIdAndTxt("combined_quick_gpu:NoScatteringOptionsGPUActive",
                          "options.momentary.gpu must be scattering.options.gpu_active!");
    const int32_t device = (int32_t)mxGetScalar(cui_mex_prop(gpu, 0, "index"));  /* .cu:378 */
    mxArray* grid = cui_mex_prop(cui_mex_prop(cui_mex_prop(setup, 0, "FOV"), 0, "shape"), 0, "grid");
    mxArray* xdc = cui_mex_prop(setup, 0, "xdc_array");
    mxArray* h_ref = cui_mex_prop(cui_mex_prop(cui_mex_prop(seq, 0, "h_ref"), 0, "samples"), 0, "values");
    mxArray* shift = cui_mex_prop(setup, 0, "indices_grid_FOV_shift");
    mxArray* sel = cui_mex_prop(op, 0, "indices_measurement_sel");
    mxArray* settings = cui_mex_prop(seq, 0, "settings");
    mxArray* f_to_unique = cui_mex_prop(seq, 0, "indices_f_to_unique");
    mxArray* prefactors = cui_mex_prop(seq, 0, "prefactors");
    mxArray* incident = cui_mex_prop(op, 0, "incident_waves");
    mxArray* npa = cui_mex_prop(grid, 0, "N_points_axis");
    mxArray* nea = cui_mex_prop(xdc, 0, "N_elements_axis");
    mxArray* ppp = cui_mex_prop(setup, 0, "N_points_per_pitch_axis");

    cui_born_desc d;
    memset(&d, 0, sizeof d);
    d.n_dims = (int32_t)mxGetNumberOfElements(npa);
    if (d.n_dims < 2 || d.n_dims > 3 || (int32_t)mxGetNumberOfElements(nea) != d.n_dims - 1 ||
        (int32_t)mxGetNumberOfElements(ppp) != d.n_dims - 1)
        mexErrMsgIdAndTxt("combined_quick_gpu:NoSymmetricGridsSetup", "a 2D or 3D regular grid and array are required");
    for (int k = 0; k < d.n_dims; ++k) d.n_points_axis[k] = (int32_t)mxGetDoubles(npa)[k];
    for (int k = 0; k < d.n_dims - 1; ++k) {
        d.n_elements_axis[k] = (int32_t)mxGetDoubles(nea)[k];
        d.n_points_per_pitch[k] = (int32_t)mxGetDoubles(ppp)[k];
    }
    d.n_f_unique = (int32_t)mxGetM(h_ref);
    d.table_form = CUI_TABLE_REFERENCE;
    d.h_ref = (const cui_complex64*)cui_mex_complex(h_ref, "operator_born.sequence.h_ref");
    d.indices_grid_FOV_shift = cui_mex_index(shift);
    d.n_measurements = (int32_t)mxGetNumberOfElements(sel);
    d.device = device;
    cui_measurement_desc* ms = (cui_measurement_desc*)mxCalloc(d.n_measurements ? d.n_measurements : 1, sizeof *ms);
    uint64_t key = 1469598103934665603ull;
    key = cui_mex_hash(key, &d, offsetof(cui_born_desc, h_ref));
    key = cui_mex_hash(key, &device, sizeof device);
    key = cui_mex_hash(key, d.h_ref, 2 * sizeof(double) * mxGetNumberOfElements(h_ref));
    key = cui_mex_hash(key, d.indices_grid_FOV_shift, sizeof(int32_t) * mxGetNumberOfElements(shift));
    for (int32_t s = 0; s < d.n_measurements; ++s) {
        const mwIndex m = (mwIndex)mxGetDoubles(sel)[s] - 1;  /* .cu:250 */
        mxArray* f2u = mxGetCell(f_to_unique, m);
        mxArray* pin = cui_mex_prop(cui_mex_prop(cui_mex_prop(incident, m, "p_incident"), 0, "samples"), 0, "values");
        mxArray* rx = cui_mex_prop(settings, m, "rx");
        mxArray* pm = mxGetCell(prefactors, m);
        mxArray* mixmap = cui_mex_prop(settings, m, "indices_f_to_unique");
        if (!f2u || !pm) mexErrMsgIdAndTxt("combined_quick_gpu:NoOperatorBorn", "measurement %d is incomplete", (int)m + 1);
        ms[s].n_f = (int32_t)mxGetM(f2u);
        ms[s].indices_f_to_unique = cui_mex_index(f2u);
        ms[s].p_incident = (const cui_complex64*)cui_mex_complex(pin, "operator_born.incident_waves.p_incident");
        ms[s].n_mixes = (int32_t)mxGetNumberOfElements(rx);
        key = cui_mex_hash(key, &ms[s].n_f, sizeof ms[s].n_f);
        key = cui_mex_hash(key, ms[s].indices_f_to_unique, sizeof(int32_t) * ms[s].n_f);
        key = cui_mex_hash(key, ms[s].p_incident, 2 * sizeof(double) * mxGetNumberOfElements(pin));
        cui_mix_desc* mx = (cui_mix_desc*)mxCalloc(ms[s].n_mixes ? ms[s].n_mixes : 1, sizeof *mx);
        for (int32_t k = 0; k < ms[s].n_mixes; ++k) {
            mxArray* act = cui_mex_prop(rx, k, "indices_active");
            mxArray* pv = cui_mex_prop(cui_mex_prop(pm, k, "samples"), 0, "values");
            mxArray* fm = mxGetCell(mixmap, k);
            if (!fm) mexErrMsgIdAndTxt("combined_quick_gpu:NoOperatorBorn", "mix %d has no frequency map", (int)k + 1);
            mx[k].n_f = (int32_t)mxGetM(pv);
            mx[k].indices_f_to_unique = cui_mex_index(fm);
            mx[k].n_active = (int32_t)mxGetNumberOfElements(act);
            mx[k].indices_active = cui_mex_index(act);
            mx[k].prefactors = (const cui_complex64*)cui_mex_complex(pv, "operator_born.sequence.prefactors");
            key = cui_mex_hash(key, &mx[k].n_f, sizeof mx[k].n_f);
            key = cui_mex_hash(key, &mx[k].n_active, sizeof mx[k].n_active);
            key = cui_mex_hash(key, mx[k].indices_f_to_unique, sizeof(int32_t) * mx[k].n_f);
            key = cui_mex_hash(key, mx[k].indices_active, sizeof(int32_t) * mx[k].n_active);
            key = cui_mex_hash(key, mx[k].prefactors, 2 * sizeof(double) * (size_t)mx[k].n_f * mx[k].n_active);
        }
        ms[s].mixes = mx;
    }
    d.measurements = ms;
    if (g_cui_plan && g_cui_plan_key == key && n_objects <= g_cui_plan_objects) return g_cui_plan;
    cui_mex_cleanup();
    const int32_t max_objects = n_objects > 64 ? n_objects : 64;
    cui_born_plan* plan = NULL;
    const cui_status st = cui_born_plan_create(&d, max_objects, &plan);
    if (st != CUI_OK) cui_mex_fail(st, "building the Born plan");
    g_cui_plan = plan;
    g_cui_plan_key = key;
    g_cui_plan_objects = max_objects;
    mexAtExit(cui_mex_cleanup);
    return plan;
}

/* the input as interleaved complex doubles: real input is promoted, as the reference does
 * (combined_quick_gpu.cu:424-437) */
static const cui_complex64* cui_mex_complex_input(const mxArray* a) {
    if (mxIsComplex(a)) return (const cui_complex64*)mxGetComplexDoubles(a);
    const size_t n = mxGetNumberOfElements(a);
    const double* re = mxGetDoubles(a);
    cui_complex64* c = (cui_complex64*)mxMalloc((n ? n : 1) * sizeof *c);
    for (size_t i = 0; i < n; ++i) {
        c[i].re = re[i];
        c[i].im = 0.0;
    }
    return c;
}

#endif /* CUI_MEX_PLAN_H */
