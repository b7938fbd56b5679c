// MATLAB MEX gateway to the GB300 powder-FID engine.
//
//   fid          = spinach_powder_gpu(I, Q, R, rho0, coil, grid, dt, nsteps)
//                  (coil with several columns: one FID row per column, as
//                  evolution(...,'multichannel') returns; rho0 with one
//                  column per orientation: per-orientation initial states)
//   [fid, fids]  = spinach_powder_gpu(I, Q, R, rho0, coil, grid, dt, nsteps, opts)
//
// I, Q     the outputs of [I,Q]=hamiltonian(spin_system) (kernel/hamiltonian.m:44):
//          I sparse dim x dim, Q a 1x2 cell {Q1 (3x3 cell), Q2 (5x5 cell)} of sparse
//          matrices; empty entries are skipped as orientation.m:45-52 does.
// R        relaxation(spin_system) (diagonal sparse) or [].
// rho0     initial state, coil detection state (dense or sparse columns).
// grid     struct with alphas, betas, gammas, weights (a kernel/grids/*.mat file).
// dt       1/parameters.sweep,  nsteps  parameters.npoints-1  (acquire.m:70-71).
// opts     optional struct: precision ('double' default, or 'single');
//          pulse_op (sparse dim x dim) and nloops run experiments/cpmg.m
//          instead of acquire.m: npoints = nsteps+1 per half-echo, fid
//          npoints*(1+2*nloops) x 1; pulse_op and sequence = 'eseem' run
//          experiments/esr_dipolar/eseem.m with timestep = dt and
//          npoints = nsteps+1 (fid (nsteps+1) x 1), sequence = 'oopeseem'
//          the out-of-phase echo of oopeseem.m; ex_prob, ex_pump and
//          sequence = 'deer' run experiments/esr_dipolar/deer_3p_hard_deer.m
//          ('brief') with stepsize = dt, nsteps pump positions and the probe
//          coil as coil (fid the (nsteps+1) x 1 DEER trace); pulse_ops (cell of
//          sparse dim x dim) and program (n x 6: kind 0 = pulse / 1 =
//          evolution, pulse index (1-based), angle, nsteps, dt, record) run a
//          pulse program (dt and nsteps of the call are then unused; fid the
//          recorded segments' FIDs, concatenated).
// fid      (nsteps+1) x 1 complex: sum_n weights(n) fid_n (powder.m:280-287).
// fids     (nsteps+1) x n_orient complex, the sum_up=false output (powder.m:291-297).
//
// Conventions follow etc/mex/prune_cpu.cpp: -R2018a interleaved complex API,
// 0-based mwIndex CSC arrays, inputs read-only, outputs from mxCreate*, and a
// grumble() that reports errors through mexErrMsgIdAndTxt.  Because
// mexErrMsgIdAndTxt does not return, every call runs in a scope whose RAII
// owners are released before the error is raised.  The engine handle (one
// CUDA context and stream) persists across calls and is released by mexAtExit.
#include "mex.h"

#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "spinach_gpu.h"

namespace {

spx_handle *g_handle = nullptr;

void release_handle() {
    if (g_handle) spx_destroy(g_handle);
    g_handle = nullptr;
}

struct CscCopy {
    std::vector<int64_t> colptr, rowidx;
    std::vector<double> values;
    spx_csc view{};
};

struct GatewayError {
    std::string id, msg;
};

void fill_csc(const mxArray *A, int64_t n, const char *name, CscCopy &out) {
    if (!mxIsSparse(A) || !mxIsDouble(A))
        throw GatewayError{"Spinach:spinach_powder_gpu:input", std::string(name) + " must be a sparse double matrix."};
    if ((int64_t)mxGetM(A) != n || (int64_t)mxGetN(A) != n)
        throw GatewayError{"Spinach:spinach_powder_gpu:input", std::string(name) + " has the wrong dimension."};
    const mwIndex *jc = mxGetJc(A);
    const mwIndex *ir = mxGetIr(A);
    const int64_t nnz = (int64_t)jc[n];
    out.colptr.assign(jc, jc + n + 1);
    out.rowidx.assign(ir, ir + nnz);
    out.values.assign(2 * (size_t)nnz, 0.0);
    if (mxIsComplex(A)) {
        const mxComplexDouble *v = mxGetComplexDoubles(A);
        for (int64_t p = 0; p < nnz; ++p) {
            out.values[2 * p] = v[p].real;
            out.values[2 * p + 1] = v[p].imag;
        }
    } else {
        const mxDouble *v = mxGetDoubles(A);
        for (int64_t p = 0; p < nnz; ++p) out.values[2 * p] = v[p];
    }
    out.view.n = n;
    out.view.colptr = out.colptr.data();
    out.view.rowidx = out.rowidx.data();
    out.view.values = out.values.data();
}

// Columns of a dim x ncol double array (dense or sparse, real or complex) as
// interleaved complex, column after column.
std::vector<double> columns(const mxArray *A, int64_t n, int64_t ncol, const char *name) {
    if (!mxIsDouble(A) || (int64_t)mxGetM(A) != n || (int64_t)mxGetN(A) != ncol)
        throw GatewayError{"Spinach:spinach_powder_gpu:input", std::string(name) + " must be a double array with dim rows."};
    std::vector<double> out(2 * (size_t)n * (size_t)ncol, 0.0);
    if (mxIsSparse(A)) {
        const mwIndex *jc = mxGetJc(A), *ir = mxGetIr(A);
        for (int64_t c = 0; c < ncol; ++c) {
            double *col = out.data() + 2 * (size_t)n * (size_t)c;
            if (mxIsComplex(A)) {
                const mxComplexDouble *v = mxGetComplexDoubles(A);
                for (mwIndex p = jc[c]; p < jc[c + 1]; ++p) { col[2 * ir[p]] = v[p].real; col[2 * ir[p] + 1] = v[p].imag; }
            } else {
                const mxDouble *v = mxGetDoubles(A);
                for (mwIndex p = jc[c]; p < jc[c + 1]; ++p) col[2 * ir[p]] = v[p];
            }
        }
    } else if (mxIsComplex(A)) {
        const mxComplexDouble *v = mxGetComplexDoubles(A);
        for (size_t i = 0; i < (size_t)n * (size_t)ncol; ++i) { out[2 * i] = v[i].real; out[2 * i + 1] = v[i].imag; }
    } else {
        const mxDouble *v = mxGetDoubles(A);
        for (size_t i = 0; i < (size_t)n * (size_t)ncol; ++i) out[2 * i] = v[i];
    }
    return out;
}

std::vector<double> grid_field(const mxArray *g, const char *name, int64_t &count) {
    const mxArray *f = mxGetField(g, 0, name);
    if (!f || !mxIsDouble(f) || mxIsComplex(f) || mxIsSparse(f))
        throw GatewayError{"Spinach:spinach_powder_gpu:grid", std::string("grid.") + name + " must be a real double vector."};
    const int64_t n = (int64_t)mxGetNumberOfElements(f);
    if (count >= 0 && n != count)
        throw GatewayError{"Spinach:spinach_powder_gpu:grid", "grid fields must have equal lengths."};
    count = n;
    const mxDouble *v = mxGetDoubles(f);
    return std::vector<double>(v, v + n);
}

double scalar(const mxArray *A, const char *name) {
    if (!mxIsDouble(A) || mxIsComplex(A) || mxGetNumberOfElements(A) != 1)
        throw GatewayError{"Spinach:spinach_powder_gpu:input", std::string(name) + " must be a real scalar."};
    return mxGetScalar(A);
}

// static grumble(): argument-count and type checks (etc/mex/prune_cpu.cpp:199-223 style)
void grumble(int nlhs, int nrhs, const mxArray *prhs[]) {
    if (nrhs < 8 || nrhs > 9)
        throw GatewayError{"Spinach:spinach_powder_gpu:nrhs", "eight or nine input arguments are required."};
    if (nlhs > 2) throw GatewayError{"Spinach:spinach_powder_gpu:nlhs", "at most two outputs are returned."};
    if (!mxIsCell(prhs[1]) || mxGetNumberOfElements(prhs[1]) != 2)
        throw GatewayError{"Spinach:spinach_powder_gpu:Q", "Q must be the 1x2 cell returned by hamiltonian()."};
    if (!mxIsStruct(prhs[5])) throw GatewayError{"Spinach:spinach_powder_gpu:grid", "grid must be a struct."};
    if (nrhs == 9 && !mxIsStruct(prhs[8]))
        throw GatewayError{"Spinach:spinach_powder_gpu:opts", "opts must be a struct."};
}

void run(int nlhs, mxArray *plhs[], int nrhs, const mxArray *prhs[]) {
    grumble(nlhs, nrhs, prhs);
    const int64_t n = (int64_t)mxGetM(prhs[0]);
    CscCopy I;
    fill_csc(prhs[0], n, "I", I);
    // non-empty rotational-basis terms Q{r}{k,m}
    std::vector<CscCopy> terms;
    std::vector<int32_t> rank, kk, mm;
    terms.reserve(34);
    for (int r = 1; r <= 2; ++r) {
        const mxArray *Qr = mxGetCell(prhs[1], r - 1);
        if (!Qr || !mxIsCell(Qr) || (int)mxGetM(Qr) != 2 * r + 1 || (int)mxGetN(Qr) != 2 * r + 1)
            throw GatewayError{"Spinach:spinach_powder_gpu:Q", "Q{r} must be a (2r+1)x(2r+1) cell."};
        for (int m = 0; m < 2 * r + 1; ++m)
            for (int k = 0; k < 2 * r + 1; ++k) {
                const mxArray *A = mxGetCell(Qr, (mwIndex)(k + m * (2 * r + 1)));   // column-major {k,m}
                if (!A || !mxIsSparse(A) || mxGetJc(A)[mxGetN(A)] == 0) continue;
                terms.emplace_back();
                fill_csc(A, n, "Q{r}{k,m}", terms.back());
                rank.push_back(r);
                kk.push_back(k);
                mm.push_back(m);
            }
    }
    std::vector<spx_csc> qv;
    for (auto &t : terms) qv.push_back(t.view);
    CscCopy R;
    const bool have_R = !mxIsEmpty(prhs[2]);
    if (have_R) fill_csc(prhs[2], n, "R", R);
    // rho0 with one column per orientation: the per-orientation initial states
    // of powder.m:244-254 ('aniso_eq' or a function handle, evaluated by the caller)
    const int64_t nrho = (int64_t)mxGetN(prhs[3]);
    const std::vector<double> rho0s = columns(prhs[3], n, nrho, "rho0");
    const std::vector<double> rho0(rho0s.begin(), rho0s.begin() + 2 * n);
    // several coil columns = several detection channels (evolution.m 'multichannel')
    const int64_t nchan = (int64_t)mxGetN(prhs[4]);
    if (nchan < 1 || nchan > 8)
        throw GatewayError{"Spinach:spinach_powder_gpu:coil", "coil must have 1 to 8 columns."};
    if (nchan > 1 && nlhs > 1)
        throw GatewayError{"Spinach:spinach_powder_gpu:nlhs", "per-orientation FIDs need a single coil column."};
    const std::vector<double> coils = columns(prhs[4], n, nchan, "coil");
    const std::vector<double> coil(coils.begin(), coils.begin() + 2 * n);
    int64_t no = -1;
    const std::vector<double> al = grid_field(prhs[5], "alphas", no);
    const std::vector<double> be = grid_field(prhs[5], "betas", no);
    const std::vector<double> ga = grid_field(prhs[5], "gammas", no);
    const std::vector<double> wt = grid_field(prhs[5], "weights", no);
    const double dt = scalar(prhs[6], "dt");
    const double ns = scalar(prhs[7], "nsteps");
    if (ns < 0 || ns != (double)(int64_t)ns)
        throw GatewayError{"Spinach:spinach_powder_gpu:nsteps", "nsteps must be a non-negative integer."};
    const int64_t nsteps = (int64_t)ns;
    spx_options opt{};
    opt.precision = SPX_FP64;
    CscCopy pulse;
    int32_t nloops = 0;                 // > 0: a CPMG echo train (experiments/cpmg.m)
    bool eseem = false;                 // a two-pulse echo (experiments/esr_dipolar/eseem.m)
    bool out_of_phase = false;          // its 45-degree first pulse (experiments/esr_dipolar/oopeseem.m)
    bool deer = false;                  // three-pulse DEER (experiments/esr_dipolar/deer_3p_hard_deer.m)
    CscCopy pump;
    std::vector<CscCopy> prog_pulses;   // a pulse program: its operators and operations
    std::vector<spx_seq_op> prog;
    bool program = false;
    if (nrhs == 9 && mxGetField(prhs[8], 0, "program")) {
        program = true;
        const mxArray *pg = mxGetField(prhs[8], 0, "program");
        const mxArray *pc = mxGetField(prhs[8], 0, "pulse_ops");
        if (!mxIsDouble(pg) || mxIsComplex(pg) || mxIsSparse(pg) || mxGetN(pg) != 6)
            throw GatewayError{"Spinach:spinach_powder_gpu:program", "opts.program must be a real n x 6 matrix."};
        const size_t np = pc ? mxGetNumberOfElements(pc) : 0;
        if (pc && !mxIsCell(pc))
            throw GatewayError{"Spinach:spinach_powder_gpu:program", "opts.pulse_ops must be a cell array."};
        prog_pulses.resize(np);
        for (size_t k = 0; k < np; ++k) fill_csc(mxGetCell(pc, (mwIndex)k), n, "opts.pulse_ops", prog_pulses[k]);
        const size_t m = mxGetM(pg);
        const mxDouble *v = mxGetDoubles(pg);
        for (size_t i = 0; i < m; ++i) {
            spx_seq_op q{};
            const double kind = v[i], idx = v[i + m], steps = v[i + 3 * m];
            if (kind != 0.0 && kind != 1.0)
                throw GatewayError{"Spinach:spinach_powder_gpu:program", "program kinds are 0 (pulse) and 1 (evolution)."};
            q.kind = kind == 0.0 ? SPX_SEQ_PULSE : SPX_SEQ_EVOLVE;
            if (q.kind == SPX_SEQ_PULSE && (idx < 1 || idx > (double)np || idx != (double)(int32_t)idx))
                throw GatewayError{"Spinach:spinach_powder_gpu:program", "pulse index out of range."};
            if (q.kind == SPX_SEQ_EVOLVE && (steps < 0 || steps != (double)(int64_t)steps))
                throw GatewayError{"Spinach:spinach_powder_gpu:program", "evolution steps must be non-negative integers."};
            q.pulse = q.kind == SPX_SEQ_PULSE ? (int32_t)idx - 1 : 0;
            q.angle = v[i + 2 * m];
            q.nsteps = q.kind == SPX_SEQ_EVOLVE ? (int64_t)steps : 0;
            q.dt = v[i + 4 * m];
            q.record = v[i + 5 * m] != 0.0;
            prog.push_back(q);
        }
        if (nlhs > 1)
            throw GatewayError{"Spinach:spinach_powder_gpu:nlhs", "a pulse program returns the powder signal only."};
    }
    if (nrhs == 9 && !program) {
        const mxArray *po = mxGetField(prhs[8], 0, "pulse_op");
        const mxArray *nl = mxGetField(prhs[8], 0, "nloops");
        const mxArray *sq = mxGetField(prhs[8], 0, "sequence");
        if (sq) {
            char buf[16] = {0};
            if (!mxIsChar(sq) || mxGetString(sq, buf, sizeof buf) != 0 ||
                (std::strcmp(buf, "eseem") != 0 && std::strcmp(buf, "oopeseem") != 0 &&
                 std::strcmp(buf, "cpmg") != 0 && std::strcmp(buf, "deer") != 0))
                throw GatewayError{"Spinach:spinach_powder_gpu:sequence",
                                   "opts.sequence must be 'cpmg', 'eseem', 'oopeseem' or 'deer'."};
            out_of_phase = std::strcmp(buf, "oopeseem") == 0;
            eseem = out_of_phase || std::strcmp(buf, "eseem") == 0;
            deer = std::strcmp(buf, "deer") == 0;
        }
        if (deer) {
            const mxArray *xp = mxGetField(prhs[8], 0, "ex_prob");
            const mxArray *xu = mxGetField(prhs[8], 0, "ex_pump");
            if (!xp || !xu || po || nl)
                throw GatewayError{"Spinach:spinach_powder_gpu:sequence",
                                   "DEER takes opts.ex_prob and opts.ex_pump, and no opts.pulse_op or opts.nloops."};
            if (nsteps < 1)
                throw GatewayError{"Spinach:spinach_powder_gpu:nsteps", "DEER needs a positive nsteps."};
            fill_csc(xp, n, "opts.ex_prob", pulse);
            fill_csc(xu, n, "opts.ex_pump", pump);
            if (nlhs > 1)
                throw GatewayError{"Spinach:spinach_powder_gpu:nlhs", "DEER returns the powder trace only."};
        } else if (eseem) {
            if (!po || nl)
                throw GatewayError{"Spinach:spinach_powder_gpu:sequence", "an echo takes opts.pulse_op and no opts.nloops."};
            fill_csc(po, n, "opts.pulse_op", pulse);
            if (nlhs > 1)
                throw GatewayError{"Spinach:spinach_powder_gpu:nlhs", "an echo returns the powder signal only."};
        } else if ((po == nullptr) != (nl == nullptr)) {
            throw GatewayError{"Spinach:spinach_powder_gpu:cpmg", "opts.pulse_op and opts.nloops go together."};
        }
        if (po && !eseem && !deer) {
            fill_csc(po, n, "opts.pulse_op", pulse);
            const double v = scalar(nl, "opts.nloops");
            if (v < 1 || v != (double)(int32_t)v)
                throw GatewayError{"Spinach:spinach_powder_gpu:cpmg", "opts.nloops must be a positive integer."};
            nloops = (int32_t)v;
            if (nlhs > 1)
                throw GatewayError{"Spinach:spinach_powder_gpu:nlhs", "a CPMG train returns the powder FID only."};
        }
    }
    if (nrhs == 9) {
        const mxArray *p = mxGetField(prhs[8], 0, "precision");
        if (p) {
            char buf[16] = {0};
            if (!mxIsChar(p) || mxGetString(p, buf, sizeof buf) != 0)
                throw GatewayError{"Spinach:spinach_powder_gpu:opts", "opts.precision must be 'single' or 'double'."};
            if (std::strcmp(buf, "single") == 0) opt.precision = SPX_FP32;
            else if (std::strcmp(buf, "double") != 0)
                throw GatewayError{"Spinach:spinach_powder_gpu:opts", "opts.precision must be 'single' or 'double'."};
        }
    }
    if (!g_handle) {
        spx_status st = spx_create(&g_handle, 0);
        if (st != SPX_OK)
            throw GatewayError{"Spinach:spinach_powder_gpu:device", std::string("GPU engine unavailable: ") + spx_status_string(st)};
        mexAtExit(release_handle);
    }
    spx_status st = spx_upload_system(g_handle, &I.view, (int32_t)rank.size(), rank.data(), kk.data(), mm.data(),
                                      qv.data(), have_R ? &R.view : nullptr, rho0.data(), coil.data());
    if (st == SPX_OK && nchan > 1) st = spx_upload_coils(g_handle, (int32_t)nchan, coils.data());
    if (st == SPX_OK && nrho > 1) {
        if (nrho != no)
            throw GatewayError{"Spinach:spinach_powder_gpu:rho0", "rho0 needs one column, or one per grid orientation."};
        st = spx_set_initial_states(g_handle, nrho, rho0s.data());
    }
    if (st != SPX_OK)
        throw GatewayError{"Spinach:spinach_powder_gpu:upload", std::string(spx_status_string(st)) + ": " + spx_last_error(g_handle)};
    if (program) {
        int64_t npts = 0;
        for (const auto &q : prog)
            if (q.kind == SPX_SEQ_EVOLVE && q.record) npts += q.nsteps + 1;
        std::vector<spx_csc> views;
        for (auto &c : prog_pulses) views.push_back(c.view);
        std::vector<double> fid(2 * (size_t)std::max<int64_t>(npts, 1));
        st = spx_run_sequence(g_handle, no, al.data(), be.data(), ga.data(), wt.data(), (int32_t)views.size(),
                              views.data(), (int32_t)prog.size(), prog.data(), &opt, fid.data(), nullptr);
        if (st != SPX_OK)
            throw GatewayError{"Spinach:spinach_powder_gpu:run", std::string(spx_status_string(st)) + ": " + spx_last_error(g_handle)};
        plhs[0] = mxCreateDoubleMatrix((mwSize)npts, 1, mxCOMPLEX);
        mxComplexDouble *out = mxGetComplexDoubles(plhs[0]);
        for (int64_t i = 0; i < npts; ++i) { out[i].real = fid[2 * i]; out[i].imag = fid[2 * i + 1]; }
        return;
    }
    if (deer) {
        std::vector<double> fid(2 * (size_t)(nsteps + 1));
        st = spx_run_deer(g_handle, no, al.data(), be.data(), ga.data(), wt.data(), dt, nsteps, &pulse.view,
                          &pump.view, &opt, fid.data(), nullptr);
        if (st != SPX_OK)
            throw GatewayError{"Spinach:spinach_powder_gpu:run", std::string(spx_status_string(st)) + ": " + spx_last_error(g_handle)};
        plhs[0] = mxCreateDoubleMatrix((mwSize)(nsteps + 1), 1, mxCOMPLEX);
        mxComplexDouble *out = mxGetComplexDoubles(plhs[0]);
        for (int64_t i = 0; i <= nsteps; ++i) { out[i].real = fid[2 * i]; out[i].imag = fid[2 * i + 1]; }
        return;
    }
    if (eseem) {
        std::vector<double> fid(2 * (size_t)(nsteps + 1));
        st = (out_of_phase ? spx_run_oopeseem : spx_run_eseem)(g_handle, no, al.data(), be.data(), ga.data(),
                                                               wt.data(), dt, nsteps + 1, &pulse.view, &opt,
                                                               fid.data(), nullptr);
        if (st != SPX_OK)
            throw GatewayError{"Spinach:spinach_powder_gpu:run", std::string(spx_status_string(st)) + ": " + spx_last_error(g_handle)};
        plhs[0] = mxCreateDoubleMatrix((mwSize)(nsteps + 1), 1, mxCOMPLEX);
        mxComplexDouble *out = mxGetComplexDoubles(plhs[0]);
        for (int64_t i = 0; i <= nsteps; ++i) { out[i].real = fid[2 * i]; out[i].imag = fid[2 * i + 1]; }
        return;
    }
    if (nloops > 0) {
        const int64_t npts = (nsteps + 1) * (1 + 2 * (int64_t)nloops);
        std::vector<double> fid(2 * (size_t)npts);
        st = spx_run_cpmg(g_handle, no, al.data(), be.data(), ga.data(), wt.data(), dt, nsteps + 1, nloops,
                          &pulse.view, &opt, fid.data(), nullptr);
        if (st != SPX_OK)
            throw GatewayError{"Spinach:spinach_powder_gpu:run", std::string(spx_status_string(st)) + ": " + spx_last_error(g_handle)};
        plhs[0] = mxCreateDoubleMatrix((mwSize)npts, 1, mxCOMPLEX);
        mxComplexDouble *out = mxGetComplexDoubles(plhs[0]);
        for (int64_t i = 0; i < npts; ++i) { out[i].real = fid[2 * i]; out[i].imag = fid[2 * i + 1]; }
        return;
    }
    // one channel: (nsteps+1) x 1 like powder(); several: one row per channel
    plhs[0] = nchan == 1 ? mxCreateDoubleMatrix((mwSize)(nsteps + 1), 1, mxCOMPLEX)
                         : mxCreateDoubleMatrix((mwSize)nchan, (mwSize)(nsteps + 1), mxCOMPLEX);
    double *per = nullptr;
    std::vector<double> per_buf;
    if (nlhs > 1) {
        per_buf.assign(2 * (size_t)(nsteps + 1) * (size_t)no, 0.0);
        per = per_buf.data();
    }
    std::vector<double> fid(2 * (size_t)(nsteps + 1) * (size_t)nchan);
    st = spx_run_powder(g_handle, no, al.data(), be.data(), ga.data(), wt.data(), dt, nsteps, &opt, fid.data(), per);
    if (st != SPX_OK)
        throw GatewayError{"Spinach:spinach_powder_gpu:run", std::string(spx_status_string(st)) + ": " + spx_last_error(g_handle)};
    mxComplexDouble *out = mxGetComplexDoubles(plhs[0]);
    for (int64_t c = 0; c < nchan; ++c)             // engine: channel-major; MATLAB: column-major
        for (int64_t i = 0; i <= nsteps; ++i) {
            const size_t src = (size_t)c * (nsteps + 1) + i, dst = (size_t)c + (size_t)i * nchan;
            out[dst].real = fid[2 * src];
            out[dst].imag = fid[2 * src + 1];
        }
    if (nlhs > 1) {
        plhs[1] = mxCreateDoubleMatrix((mwSize)(nsteps + 1), (mwSize)no, mxCOMPLEX);
        mxComplexDouble *o2 = mxGetComplexDoubles(plhs[1]);
        for (size_t i = 0; i < (size_t)(nsteps + 1) * (size_t)no; ++i) { o2[i].real = per[2 * i]; o2[i].imag = per[2 * i + 1]; }
    }
}

}  // namespace

void mexFunction(int nlhs, mxArray *plhs[], int nrhs, const mxArray *prhs[]) {
    // mexErrMsgIdAndTxt does not return: the message is copied into static
    // storage and every owner of run() is destroyed before it is raised.
    static char id[128], msg[1024];
    bool failed = false;
    try {
        run(nlhs, plhs, nrhs, prhs);
    } catch (const GatewayError &e) {
        std::snprintf(id, sizeof id, "%s", e.id.c_str());
        std::snprintf(msg, sizeof msg, "%s", e.msg.c_str());
        failed = true;
    } catch (const std::exception &e) {
        std::snprintf(id, sizeof id, "%s", "Spinach:spinach_powder_gpu:internal");
        std::snprintf(msg, sizeof msg, "%s", e.what());
        failed = true;
    }
    if (failed) mexErrMsgIdAndTxt(id, "%s", msg);
}
