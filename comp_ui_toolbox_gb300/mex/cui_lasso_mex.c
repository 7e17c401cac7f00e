/* gamma = cui_lasso_mex(operator_born, u, lambda, step, n_iter, gamma0)
 *
 * The solver loop of lq_minimization (operator.m:601-790), which drives the Born operator
 * through combined_scalar (:717), run on the device: n_iter proximal-gradient LASSO
 * iterations gamma <- S(gamma - step * Phi^H (Phi gamma - u), step * lambda) per column from
 * gamma0 (cui_born_lasso_host).  u: N_observations x N_objects, gamma0: N_points x N_objects,
 * lambda: scalar or one value per column.  Same plan cache and error identifiers as
 * cui_born_mex.c (each MEX file holds its own cached plan).
 *
 * Build: mex -R2018a cui_lasso_mex.c -I<repo>/include -L<repo>/comp_ui_toolbox_gb300 -lcui_born */
#include "cui_mex_plan.h"

void mexFunction(int nlhs, mxArray* plhs[], int nrhs, const mxArray* prhs[]) {
    if (nrhs != 6 || nlhs != 1)
        mexErrMsgIdAndTxt("combined_quick_gpu:NumberArguments", "cui_lasso_mex requires 6 inputs and 1 output.");
    const mxArray *u = prhs[1], *lam = prhs[2], *g0 = prhs[5];
    const int32_t n_objects = (int32_t)mxGetN(u);
    cui_born_plan* plan = cui_mex_plan(prhs[0], n_objects > 0 ? n_objects : 1);
    int64_t n_obs = 0, n_points = 0;
    cui_status st = cui_born_size(plan, &n_obs, &n_points);
    if (st != CUI_OK) cui_mex_fail(st, "cui_born_size");
    if (!(mxIsDouble(u) && (int64_t)mxGetM(u) == n_obs && !mxIsEmpty(u)) ||
        !(mxIsDouble(g0) && (int64_t)mxGetM(g0) == n_points && (int32_t)mxGetN(g0) == n_objects))
        mexErrMsgIdAndTxt("combined_quick_gpu:NoValidDoubleMatrix",
                          "u must be N_observations x N_objects and gamma0 N_points x N_objects doubles!");
    const size_t n_lam = mxGetNumberOfElements(lam);
    if (!(mxIsDouble(lam) && !mxIsComplex(lam) && (n_lam == 1 || n_lam == (size_t)n_objects)) ||
        !mxIsScalar(prhs[3]) || !mxIsScalar(prhs[4]))
        mexErrMsgIdAndTxt("combined_quick_gpu:NoValidDoubleMatrix", "lambda, step and n_iter must be real scalars!");
    float* lf = (float*)mxMalloc(sizeof(float) * (size_t)n_objects);
    for (int32_t b = 0; b < n_objects; ++b) lf[b] = (float)mxGetDoubles(lam)[n_lam == 1 ? 0 : b];
    mwSize dims[2];
    dims[0] = (mwSize)n_points;
    dims[1] = (mwSize)n_objects;
    plhs[0] = mxCreateNumericArray(2, dims, mxDOUBLE_CLASS, mxCOMPLEX);
    cui_complex64* g = (cui_complex64*)mxGetComplexDoubles(plhs[0]);
    memcpy(g, cui_mex_complex_input(g0), sizeof(cui_complex64) * (size_t)n_points * n_objects);
    st = cui_born_lasso_host(plan, cui_mex_complex_input(u), n_obs, n_objects, g, n_points, lf,
                             (float)mxGetScalar(prhs[3]), (int32_t)mxGetScalar(prhs[4]));
    if (st != CUI_OK) cui_mex_fail(st, "lasso");
}
