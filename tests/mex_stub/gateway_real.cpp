// Drives spinach_powder_gpu.cpp through the mx stand-in and the REAL engine
// library (libspinach_gpu.so) on one GPU.  Inputs come from binary files
// written by tests/test_gpu_mex_gateway.py; the outputs of three calls go to
// binary files the test compares with the Python binding's runs:
//   out_a.bin   [fid, fids] = spinach_powder_gpu(I,Q,R,rho0,coil,grid,dt,nsteps,opts)
//               (one coil column, double precision, per-orientation FIDs)
//   out_b.bin   fid = spinach_powder_gpu(I,Q,R,rho0,[coil coil2],grid,dt,nsteps)
//               (two detection channels: a 2 x (nsteps+1) matrix)
//   out_c.bin   fid with opts.precision = 'single'
// File formats: a CSC matrix is int64 n, int64 nnz, int64 colptr[n+1],
// int64 rowidx[nnz], double values[2*nnz] (interleaved complex); a dense
// array is int64 count, double values[count].
#include <cstdint>
#include <cstdio>
#include <string>
#include <vector>

#include "mex.h"

void stub_run_atexit();

namespace {

std::string g_dir;

FILE *open_in(const std::string &name) {
    FILE *f = std::fopen((g_dir + "/" + name).c_str(), "rb");
    if (!f) {
        std::printf("FAIL: cannot open %s\n", name.c_str());
        std::exit(2);
    }
    return f;
}

template <class T> void rd(FILE *f, T *p, size_t count) {
    if (std::fread(p, sizeof(T), count, f) != count) {
        std::printf("FAIL: short read\n");
        std::exit(2);
    }
}

mxArray *read_csc(const std::string &name) {
    FILE *f = open_in(name);
    int64_t n = 0, nnz = 0;
    rd(f, &n, 1);
    rd(f, &nnz, 1);
    std::vector<int64_t> cp(n + 1), ri(nnz);
    std::vector<double> v(2 * nnz);
    rd(f, cp.data(), cp.size());
    rd(f, ri.data(), ri.size());
    rd(f, v.data(), v.size());
    std::fclose(f);
    mxArray *a = new mxArray;
    a->kind = mxArray::Sparse;
    a->m = a->n = (size_t)n;
    a->complex = true;
    a->jc.assign(cp.begin(), cp.end());
    a->ir.assign(ri.begin(), ri.end());
    a->cx.resize(nnz);
    for (int64_t p = 0; p < nnz; ++p) a->cx[p] = mxComplexDouble{v[2 * p], v[2 * p + 1]};
    return a;
}

std::vector<double> read_dense(const std::string &name) {
    FILE *f = open_in(name);
    int64_t count = 0;
    rd(f, &count, 1);
    std::vector<double> v(count);
    rd(f, v.data(), v.size());
    std::fclose(f);
    return v;
}

mxArray *real_column(const std::vector<double> &v) {
    mxArray *a = new mxArray;
    a->m = v.size();
    a->n = 1;
    a->re = v;
    return a;
}

// complex dense matrix from interleaved column-major values
mxArray *complex_matrix(const std::vector<double> &v, size_t m, size_t n) {
    mxArray *a = new mxArray;
    a->m = m;
    a->n = n;
    a->complex = true;
    a->cx.resize(m * n);
    for (size_t i = 0; i < m * n; ++i) a->cx[i] = mxComplexDouble{v[2 * i], v[2 * i + 1]};
    return a;
}

void write_out(const std::string &name, const mxArray *a) {
    FILE *f = std::fopen((g_dir + "/" + name).c_str(), "wb");
    const int64_t dims[2] = {(int64_t)a->m, (int64_t)a->n};
    std::fwrite(dims, sizeof(int64_t), 2, f);
    for (const mxComplexDouble &c : a->cx) {
        std::fwrite(&c.real, sizeof(double), 1, f);
        std::fwrite(&c.imag, sizeof(double), 1, f);
    }
    std::fclose(f);
}

bool call(int nlhs, mxArray **plhs, int nrhs, const mxArray **prhs, const char *what) {
    try {
        mexFunction(nlhs, plhs, nrhs, prhs);
        return true;
    } catch (const MexError &e) {
        std::printf("FAIL %s: %s %s\n", what, e.id.c_str(), e.msg.c_str());
        return false;
    }
}

}  // namespace

int main(int argc, char **argv) {
    if (argc < 2) {
        std::printf("usage: gateway_real <dir>\n");
        return 2;
    }
    g_dir = argv[1];
    const std::vector<double> meta = read_dense("meta.bin");     // n, n_orient, dt, nsteps, n_terms
    const size_t n = (size_t)meta[0], no = (size_t)meta[1];
    const double dt = meta[2];
    const size_t nsteps = (size_t)meta[3], nterms = (size_t)meta[4];
    const std::vector<double> rkm = read_dense("rkm.bin");        // 3 per term, 1-based k, m
    mxArray *I = read_csc("I.bin");
    mxArray *R = read_csc("R.bin");
    mxArray *Q = new mxArray;
    Q->kind = mxArray::Cell;
    Q->m = 1;
    Q->n = 2;
    for (int r = 1; r <= 2; ++r) {
        mxArray *c = new mxArray;
        c->kind = mxArray::Cell;
        c->m = c->n = 2 * r + 1;
        c->cells.assign(c->m * c->n, nullptr);
        Q->cells.push_back(c);
    }
    for (size_t t = 0; t < nterms; ++t) {
        const int r = (int)rkm[3 * t], k = (int)rkm[3 * t + 1], m = (int)rkm[3 * t + 2];
        mxArray *c = Q->cells[r - 1];
        c->cells[(k - 1) + (m - 1) * c->m] = read_csc("Q" + std::to_string(t) + ".bin");   // column-major cell
    }
    const std::vector<double> rho0 = read_dense("rho0.bin"), coils = read_dense("coils.bin");
    mxArray *rho = complex_matrix(rho0, n, 1);
    mxArray *coil1 = complex_matrix(std::vector<double>(coils.begin(), coils.begin() + 2 * n), n, 1);
    mxArray *coil2 = complex_matrix(coils, n, 2);
    const std::vector<double> g = read_dense("grid.bin");        // 4 x no, row by row
    mxArray *grid = new mxArray;
    grid->kind = mxArray::Struct;
    grid->m = grid->n = 1;
    const char *names[4] = {"alphas", "betas", "gammas", "weights"};
    for (int i = 0; i < 4; ++i)
        grid->fields[names[i]] = real_column(std::vector<double>(g.begin() + i * no, g.begin() + (i + 1) * no));
    mxArray *dta = real_column({dt});
    mxArray *nst = real_column({(double)nsteps});
    mxArray *opts = new mxArray;
    opts->kind = mxArray::Struct;
    opts->m = opts->n = 1;
    mxArray *dbl = new mxArray;
    dbl->kind = mxArray::Char;
    dbl->m = dbl->n = 1;
    dbl->str = "double";
    opts->fields["precision"] = dbl;
    int fails = 0;
    {
        const mxArray *in[9] = {I, Q, R, rho, coil1, grid, dta, nst, opts};
        mxArray *out[2] = {nullptr, nullptr};
        if (call(2, out, 9, in, "per-orientation")) {
            write_out("out_a_fid.bin", out[0]);
            write_out("out_a_fids.bin", out[1]);
        } else {
            ++fails;
        }
    }
    {
        const mxArray *in[8] = {I, Q, R, rho, coil2, grid, dta, nst};
        mxArray *out[1] = {nullptr};
        if (call(1, out, 8, in, "two channels")) write_out("out_b_fid.bin", out[0]);
        else ++fails;
    }
    {
        mxArray *single = new mxArray(*dbl);
        single->str = "single";
        mxArray *o2 = new mxArray(*opts);
        o2->fields["precision"] = single;
        const mxArray *in[9] = {I, Q, R, rho, coil1, grid, dta, nst, o2};
        mxArray *out[1] = {nullptr};
        if (call(1, out, 9, in, "single precision")) write_out("out_c_fid.bin", out[0]);
        else ++fails;
    }
    stub_run_atexit();                 // releases the engine handle as MATLAB's mexAtExit would
    if (fails == 0) std::printf("PASS\n");
    return fails == 0 ? 0 : 1;
}
