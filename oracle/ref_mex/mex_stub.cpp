// In-memory MATLAB MEX runtime for running the reference's MEX gateway
// (+scattering/combined_quick_gpu.cu, mexFunction :66-1094) outside MATLAB.
//
// TEST INFRASTRUCTURE ONLY.  The oracle's reference runner (oracle/ref_runner.py)
// builds the operator_born object the gateway reads (combined_quick_gpu.cu:203-393,
// :817-823) as a tree of nodes -- object arrays with a class name and named
// properties, cell arrays, and double matrices (real or interleaved complex,
// column-major) -- through the ref_* functions below, then calls ref_call, which
// runs mexFunction and returns the output matrix or the error identifier that
// mexErrMsgIdAndTxt raised.  mxGetProperty returns the stored node instead of a
// copy; the gateway never writes into its inputs.
#include <csetjmp>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <memory>
#include <string>
#include <vector>

#include "mex.h"

struct mxArray_tag {
    enum Kind { OBJECT, CELL, DOUBLE } kind = DOUBLE;
    std::string cls;                                     // OBJECT: class name
    std::vector<std::map<std::string, mxArray*>> props;  // OBJECT: properties per element
    std::vector<mxArray*> cells;                          // CELL
    size_t m = 0, n = 0;                                  // DOUBLE: rows, columns
    bool complex_ = false;
    std::vector<double> data;                             // DOUBLE: m*n (real) or 2*m*n (interleaved)
};

namespace {

std::vector<std::unique_ptr<mxArray>> g_arena;
std::jmp_buf g_jmp;
bool g_in_call = false;
char g_err_id[256];
char g_err_msg[512];
bool g_verbose = false;
void (*g_at_exit)(void) = nullptr;

mxArray* fresh() {
    g_arena.emplace_back(new mxArray());
    return g_arena.back().get();
}

size_t numel(const mxArray* a) {
    if (!a) return 0;
    switch (a->kind) {
        case mxArray::OBJECT: return a->props.size();
        case mxArray::CELL: return a->cells.size();
        default: return a->m * a->n;
    }
}

[[noreturn]] void fail(const char* id, const char* msg) {
    std::snprintf(g_err_id, sizeof g_err_id, "%s", id);
    std::snprintf(g_err_msg, sizeof g_err_msg, "%s", msg);
    if (g_in_call) std::longjmp(g_jmp, 1);
    std::fprintf(stderr, "mex error outside a call: %s: %s\n", id, msg);
    std::abort();
}

}  // namespace

extern "C" {

// ---- the MEX API used by the gateway -------------------------------------------
mxArray* mxGetProperty(const mxArray* pa, mwIndex index, const char* name) {
    if (!pa || pa->kind != mxArray::OBJECT || index >= pa->props.size()) return nullptr;
    auto it = pa->props[index].find(name);
    return it == pa->props[index].end() ? nullptr : it->second;
}

mxArray* mxGetCell(const mxArray* pa, mwIndex index) {
    if (!pa || pa->kind != mxArray::CELL || index >= pa->cells.size()) return nullptr;
    return pa->cells[index];
}

mxDouble* mxGetDoubles(const mxArray* pa) {
    if (!pa || pa->kind != mxArray::DOUBLE || pa->complex_) return nullptr;
    return const_cast<double*>(pa->data.data());
}

mxComplexDouble* mxGetComplexDoubles(const mxArray* pa) {
    if (!pa || pa->kind != mxArray::DOUBLE || !pa->complex_) return nullptr;
    return reinterpret_cast<mxComplexDouble*>(const_cast<double*>(pa->data.data()));
}

double mxGetScalar(const mxArray* pa) {
    if (!pa || pa->kind != mxArray::DOUBLE || pa->data.empty()) return 0.0;
    return pa->data[0];
}

size_t mxGetNumberOfElements(const mxArray* pa) { return numel(pa); }

size_t mxGetM(const mxArray* pa) {
    if (!pa) return 0;
    return pa->kind == mxArray::DOUBLE ? pa->m : (numel(pa) ? 1 : 0);
}

size_t mxGetN(const mxArray* pa) {
    if (!pa) return 0;
    return pa->kind == mxArray::DOUBLE ? pa->n : numel(pa);
}

mwSize mxGetNumberOfDimensions(const mxArray*) { return 2; }

bool mxIsClass(const mxArray* pa, const char* name) {
    if (!pa) return false;
    if (pa->kind == mxArray::DOUBLE) return std::strcmp(name, "double") == 0;
    if (pa->kind == mxArray::CELL) return std::strcmp(name, "cell") == 0;
    return pa->cls == name;
}

bool mxIsScalar(const mxArray* pa) { return numel(pa) == 1; }
bool mxIsDouble(const mxArray* pa) { return pa && pa->kind == mxArray::DOUBLE; }
bool mxIsComplex(const mxArray* pa) { return pa && pa->kind == mxArray::DOUBLE && pa->complex_; }
bool mxIsNumeric(const mxArray* pa) { return pa && pa->kind == mxArray::DOUBLE; }
bool mxIsEmpty(const mxArray* pa) { return numel(pa) == 0; }

mxArray* mxDuplicateArray(const mxArray* pa) {
    mxArray* d = fresh();
    *d = *pa;
    return d;
}

int mxMakeArrayComplex(mxArray* pa) {
    if (!pa || pa->kind != mxArray::DOUBLE) return 0;
    if (pa->complex_) return 1;
    std::vector<double> c(2 * pa->data.size(), 0.0);
    for (size_t i = 0; i < pa->data.size(); ++i) c[2 * i] = pa->data[i];
    pa->data.swap(c);
    pa->complex_ = true;
    return 1;
}

mxArray* mxCreateNumericArray(mwSize ndim, const mwSize* dims, mxClassID classid, mxComplexity flag) {
    if (ndim != 2 || classid != mxDOUBLE_CLASS) fail("ref_mex:Unsupported", "only 2-D double arrays are supported");
    mxArray* a = fresh();
    a->kind = mxArray::DOUBLE;
    a->m = dims[0];
    a->n = dims[1];
    a->complex_ = flag == mxCOMPLEX;
    a->data.assign((a->complex_ ? 2 : 1) * a->m * a->n, 0.0);
    return a;
}

void* mxMalloc(size_t n) { return std::malloc(n ? n : 1); }
void* mxCalloc(size_t n, size_t size) { return std::calloc(n ? n : 1, size ? size : 1); }
void* mxRealloc(void* ptr, size_t size) { return std::realloc(ptr, size ? size : 1); }
void mxFree(void* ptr) { std::free(ptr); }

void mexErrMsgIdAndTxt(const char* id, const char* fmt, ...) {
    char msg[512];
    va_list ap;
    va_start(ap, fmt);
    std::vsnprintf(msg, sizeof msg, fmt, ap);
    va_end(ap);
    fail(id, msg);
}

int mexAtExit(void (*fn)(void)) {
    g_at_exit = fn;
    return 0;
}

int mexPrintf(const char* fmt, ...) {
    if (!g_verbose) return 0;
    va_list ap;
    va_start(ap, fmt);
    const int r = std::vprintf(fmt, ap);
    va_end(ap);
    return r;
}

// ---- the runner's builder API ----------------------------------------------------
mxArray* ref_new_object(const char* cls, size_t n) {
    mxArray* a = fresh();
    a->kind = mxArray::OBJECT;
    a->cls = cls;
    a->props.resize(n);
    return a;
}

mxArray* ref_new_cell(size_t n) {
    mxArray* a = fresh();
    a->kind = mxArray::CELL;
    a->cells.assign(n, nullptr);
    return a;
}

// column-major m x n doubles; `data` holds m*n values, or 2*m*n interleaved (re, im) when complex
mxArray* ref_new_double(size_t m, size_t n, int is_complex, const double* data) {
    mxArray* a = fresh();
    a->kind = mxArray::DOUBLE;
    a->m = m;
    a->n = n;
    a->complex_ = is_complex != 0;
    const size_t k = (a->complex_ ? 2 : 1) * m * n;
    a->data.assign(data, data + k);
    return a;
}

int ref_set_prop(mxArray* obj, size_t index, const char* name, mxArray* value) {
    if (!obj || obj->kind != mxArray::OBJECT || index >= obj->props.size()) return 1;
    obj->props[index][name] = value;
    return 0;
}

int ref_set_cell(mxArray* cell, size_t index, mxArray* value) {
    if (!cell || cell->kind != mxArray::CELL || index >= cell->cells.size()) return 1;
    cell->cells[index] = value;
    return 0;
}

// Runs the gateway with nrhs (<= 16) inputs and one output, as MATLAB would: returns 0 and the
// output node, or 1 with the error identifier and message of mexErrMsgIdAndTxt.  ref_call is the
// three-input form output = combined_quick_gpu(operator, mode, input).
int ref_call_args(const mxArray* const* args, int nrhs, mxArray** out, char* err_id, size_t err_id_len, char* err_msg,
                  size_t err_msg_len) {
    const mxArray* prhs[16] = {nullptr};
    for (int i = 0; i < nrhs && i < 16; ++i) prhs[i] = args[i];
    mxArray* plhs[1] = {nullptr};
    g_err_id[0] = g_err_msg[0] = '\0';
    g_in_call = true;
    if (setjmp(g_jmp) == 0) {
        mexFunction(1, plhs, nrhs, prhs);
        g_in_call = false;
        *out = plhs[0];
        return 0;
    }
    g_in_call = false;
    std::snprintf(err_id, err_id_len, "%s", g_err_id);
    std::snprintf(err_msg, err_msg_len, "%s", g_err_msg);
    *out = nullptr;
    return 1;
}

int ref_call(const mxArray* op, const mxArray* mode, const mxArray* input, int nrhs, mxArray** out, char* err_id,
             size_t err_id_len, char* err_msg, size_t err_msg_len) {
    const mxArray* args[3] = {op, mode, input};
    return ref_call_args(args, nrhs, out, err_id, err_id_len, err_msg, err_msg_len);
}

int ref_dims(const mxArray* a, size_t* m, size_t* n, int* is_complex) {
    if (!a || a->kind != mxArray::DOUBLE) return 1;
    *m = a->m;
    *n = a->n;
    *is_complex = a->complex_ ? 1 : 0;
    return 0;
}

int ref_read(const mxArray* a, double* out) {
    if (!a || a->kind != mxArray::DOUBLE) return 1;
    std::memcpy(out, a->data.data(), sizeof(double) * a->data.size());
    return 0;
}

void ref_reset(void) { g_arena.clear(); }
// what MATLAB does when the MEX file is cleared: the function registered by mexAtExit runs
void ref_clear_mex(void) {
    if (g_at_exit) g_at_exit();
    g_at_exit = nullptr;
}
void ref_verbose(int on) { g_verbose = on != 0; }

}  // extern "C"
