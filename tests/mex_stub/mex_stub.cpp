// Implementation of the mx/mex stand-in declared in mex.h (test support).
#include "mex.h"

#include <cstdarg>
#include <cstdio>

bool mxIsSparse(const mxArray *a) { return a && a->kind == mxArray::Sparse; }
bool mxIsDouble(const mxArray *a) { return a && (a->kind == mxArray::Dense || a->kind == mxArray::Sparse); }
bool mxIsComplex(const mxArray *a) { return a && a->complex; }
bool mxIsCell(const mxArray *a) { return a && a->kind == mxArray::Cell; }
bool mxIsStruct(const mxArray *a) { return a && a->kind == mxArray::Struct; }
bool mxIsChar(const mxArray *a) { return a && a->kind == mxArray::Char; }
bool mxIsEmpty(const mxArray *a) { return !a || a->m == 0 || a->n == 0; }
size_t mxGetM(const mxArray *a) { return a->m; }
size_t mxGetN(const mxArray *a) { return a->n; }
size_t mxGetNumberOfElements(const mxArray *a) { return a->m * a->n; }
mwIndex *mxGetJc(const mxArray *a) { return const_cast<mwIndex *>(a->jc.data()); }
mwIndex *mxGetIr(const mxArray *a) { return const_cast<mwIndex *>(a->ir.data()); }
mxDouble *mxGetDoubles(const mxArray *a) { return a->complex ? nullptr : const_cast<double *>(a->re.data()); }
mxComplexDouble *mxGetComplexDoubles(const mxArray *a) {
    return a->complex ? const_cast<mxComplexDouble *>(a->cx.data()) : nullptr;
}
mxArray *mxGetCell(const mxArray *a, mwIndex i) { return i < a->cells.size() ? a->cells[i] : nullptr; }
mxArray *mxGetField(const mxArray *a, mwIndex, const char *name) {
    auto it = a->fields.find(name);
    return it == a->fields.end() ? nullptr : it->second;
}
int mxGetString(const mxArray *a, char *buf, mwSize len) {
    if (!a || a->kind != mxArray::Char || a->str.size() + 1 > len) return 1;
    for (size_t i = 0; i < a->str.size(); ++i) buf[i] = a->str[i];
    buf[a->str.size()] = 0;
    return 0;
}
double mxGetScalar(const mxArray *a) { return a->complex ? a->cx[0].real : a->re[0]; }
mxArray *mxCreateDoubleMatrix(mwSize m, mwSize n, mxComplexity c) {
    mxArray *a = new mxArray;
    a->m = m; a->n = n; a->complex = (c == mxCOMPLEX);
    if (a->complex) a->cx.assign(m * n, mxComplexDouble{0, 0}); else a->re.assign(m * n, 0.0);
    return a;
}
void mexErrMsgIdAndTxt(const char *id, const char *fmt, ...) {
    char buf[2048];
    va_list ap;
    va_start(ap, fmt);
    std::vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    throw MexError{id, buf};            // like MATLAB: control does not return to the caller
}
static void (*g_exit)(void) = nullptr;
int mexAtExit(void (*fn)(void)) { g_exit = fn; return 0; }
void stub_run_atexit() { if (g_exit) g_exit(); }
