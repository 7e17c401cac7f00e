/* output = cui_born_mex(operator_born, mode, input)
 *
 * Drop-in MEX gateway for the reference's scattering.combined_quick_gpu (calling syntax
 * +scattering/combined_quick_gpu.m:11; gateway +scattering/combined_quick_gpu.cu:66-1094):
 *   mode 1: input = gamma (N_points x N_objects, real or complex double)  -> output = u
 *           (N_observations x N_objects, complex double)
 *   mode 2: input = u (N_observations x N_objects)                          -> output = gamma_hat
 *           (N_points x N_objects, complex double)
 * Argument checks and error identifiers follow the reference (.cu:201-441); mode must be 1 or
 * 2 (the reference treats every value but 1 as the adjoint).  The plan is cached across calls
 * (cui_mex_plan.h) and applied through cui_born_combined_host (FP64 in and out, FP32 on the
 * device).
 *
 * Build: mex -R2018a cui_born_mex.c -I<repo>/include -L<repo>/comp_ui_toolbox_gb300 -lcui_born */
#include "cui_mex_plan.h"

void mexFunction(int nlhs, mxArray* plhs[], int nrhs, const mxArray* prhs[]) {
    if (nrhs != 3 || nlhs != 1)
        mexErrMsgIdAndTxt("combined_quick_gpu:NumberArguments", "combined_quick_gpu requires 3 inputs and 1 output.");
    if (!(mxIsNumeric(prhs[1]) && mxIsScalar(prhs[1]) && !mxIsComplex(prhs[1])))
        mexErrMsgIdAndTxt("combined_quick_gpu:NoNumericScalarMode", "mode must be a real-valued numeric scalar!");
    const double mode_d = mxGetScalar(prhs[1]);
    if (mode_d != 1.0 && mode_d != 2.0)
        mexErrMsgIdAndTxt("combined_quick_gpu:NoNumericScalarMode", "mode must be 1 (forward) or 2 (adjoint)!");
    const int32_t mode = (int32_t)mode_d;
    const mxArray* in = prhs[2];
    const int32_t n_objects = (int32_t)mxGetN(in);
    cui_born_plan* plan = cui_mex_plan(prhs[0], n_objects > 0 ? n_objects : 1);
    int64_t n_obs = 0, n_points = 0;
    cui_status st = cui_born_size(plan, &n_obs, &n_points);
    if (st != CUI_OK) cui_mex_fail(st, "cui_born_size");
    const int64_t rows_in = mode == 1 ? n_points : n_obs, rows_out = mode == 1 ? n_obs : n_points;
    if (!(mxIsDouble(in) && mxGetNumberOfDimensions(in) == 2 && (int64_t)mxGetM(in) == rows_in && !mxIsEmpty(in)))
        mexErrMsgIdAndTxt("combined_quick_gpu:NoValidDoubleMatrix", "input must be a double matrix with %lld rows!",
                          (long long)rows_in);
    mwSize dims[2];
    dims[0] = (mwSize)rows_out;
    dims[1] = (mwSize)n_objects;
    plhs[0] = mxCreateNumericArray(2, dims, mxDOUBLE_CLASS, mxCOMPLEX);
    st = cui_born_combined_host(plan, mode, cui_mex_complex_input(in), rows_in, n_objects,
                                (cui_complex64*)mxGetComplexDoubles(plhs[0]), rows_out);
    if (st != CUI_OK) cui_mex_fail(st, mode == 1 ? "forward" : "adjoint");
}
