// Host-only stand-in for the handful of MATLAB mx/mex API functions the
// spinach_powder_gpu gateway uses (R2018a interleaved-complex API), so the
// gateway's argument marshalling can be compiled and tested without MATLAB.
#pragma once
#include <cstddef>
#include <cstdint>
#include <map>
#include <string>
#include <vector>

typedef size_t mwIndex;
typedef size_t mwSize;
typedef double mxDouble;
struct mxComplexDouble { double real, imag; };
enum mxComplexity { mxREAL = 0, mxCOMPLEX = 1 };

struct mxArray {
    enum Kind { Dense, Sparse, Cell, Struct, Char } kind = Dense;
    size_t m = 0, n = 0;
    bool complex = false;
    std::vector<double> re;
    std::vector<mxComplexDouble> cx;
    std::vector<mwIndex> jc, ir;
    std::vector<mxArray *> cells;
    std::map<std::string, mxArray *> fields;
    std::string str;
};

struct MexError {
    std::string id, msg;
};

bool mxIsSparse(const mxArray *a);
bool mxIsDouble(const mxArray *a);
bool mxIsComplex(const mxArray *a);
bool mxIsCell(const mxArray *a);
bool mxIsStruct(const mxArray *a);
bool mxIsChar(const mxArray *a);
bool mxIsEmpty(const mxArray *a);
size_t mxGetM(const mxArray *a);
size_t mxGetN(const mxArray *a);
size_t mxGetNumberOfElements(const mxArray *a);
mwIndex *mxGetJc(const mxArray *a);
mwIndex *mxGetIr(const mxArray *a);
mxDouble *mxGetDoubles(const mxArray *a);
mxComplexDouble *mxGetComplexDoubles(const mxArray *a);
mxArray *mxGetCell(const mxArray *a, mwIndex i);
mxArray *mxGetField(const mxArray *a, mwIndex i, const char *name);
int mxGetString(const mxArray *a, char *buf, mwSize len);
double mxGetScalar(const mxArray *a);
mxArray *mxCreateDoubleMatrix(mwSize m, mwSize n, mxComplexity c);
void mexErrMsgIdAndTxt(const char *id, const char *fmt, ...);
int mexAtExit(void (*fn)(void));

void mexFunction(int nlhs, mxArray *plhs[], int nrhs, const mxArray *prhs[]);
