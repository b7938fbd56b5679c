// Drives spinach_powder_gpu.cpp through the mx stand-in and the recording
// engine: argument marshalling, Q{r}{k,m} enumeration, real->complex and
// sparse->dense conversion, options and error identifiers.
#include <cmath>
#include <cstdio>
#include <string>
#include <vector>

#include "mex.h"

struct Recorded {
    int64_t n;
    std::vector<int64_t> I_colptr, I_rowidx;
    std::vector<double> I_values;
    std::vector<int> rank, k, m;
    std::vector<std::vector<double>> Q_values;
    bool have_R;
    std::vector<double> R_values, rho0, coil, coils, states, grid;
    int nchan;
    double dt;
    int64_t nsteps, n_orient;
    int precision;
    bool want_per;
    int fail_run;
    std::vector<double> pulse, pump;
    int64_t npoints;
    int nloops;
};
extern Recorded g_rec;
void stub_run_atexit();

static int failures = 0;
#define CHECK(c) do { if (!(c)) { std::printf("FAIL line %d: %s\n", __LINE__, #c); ++failures; } } while (0)

static mxArray *sparse(size_t n, const std::vector<size_t> &rows, const std::vector<size_t> &cols,
                       const std::vector<double> &re, const std::vector<double> &im) {
    mxArray *a = new mxArray;
    a->kind = mxArray::Sparse; a->m = n; a->n = n; a->complex = !im.empty();
    a->jc.assign(n + 1, 0);
    for (size_t c : cols) a->jc[c + 1]++;
    for (size_t c = 0; c < n; ++c) a->jc[c + 1] += a->jc[c];
    std::vector<size_t> fill(a->jc.begin(), a->jc.end() - 1);
    a->ir.assign(rows.size(), 0);
    if (a->complex) a->cx.assign(rows.size(), mxComplexDouble{0, 0}); else a->re.assign(rows.size(), 0);
    for (size_t p = 0; p < rows.size(); ++p) {
        size_t q = fill[cols[p]]++;
        a->ir[q] = rows[p];
        if (a->complex) a->cx[q] = mxComplexDouble{re[p], im[p]}; else a->re[q] = re[p];
    }
    return a;
}
static mxArray *empty_sparse(size_t n) { return sparse(n, {}, {}, {}, {}); }
static mxArray *cell(size_t m, size_t n) {
    mxArray *a = new mxArray; a->kind = mxArray::Cell; a->m = m; a->n = n; a->cells.assign(m * n, nullptr); return a;
}
static mxArray *dense(std::vector<double> v) {
    mxArray *a = new mxArray; a->m = v.size(); a->n = 1; a->re = v; return a;
}
static mxArray *scalar(double v) { return dense({v}); }
static mxArray *str(const char *s) { mxArray *a = new mxArray; a->kind = mxArray::Char; a->m = 1; a->n = 1; a->str = s; return a; }
static mxArray *strct() { mxArray *a = new mxArray; a->kind = mxArray::Struct; a->m = 1; a->n = 1; return a; }

int main() {
    const size_t n = 4;
    mxArray *I = sparse(n, {0, 1, 3}, {0, 1, 2}, {1.5, -2.0, 0.25}, {});
    mxArray *Q = cell(1, 2);
    Q->cells[0] = cell(3, 3);
    Q->cells[1] = cell(5, 5);
    for (auto &c : Q->cells[0]->cells) c = empty_sparse(n);
    for (auto &c : Q->cells[1]->cells) c = empty_sparse(n);
    Q->cells[0]->cells[0 + 2 * 3] = sparse(n, {1}, {2}, {3.0}, {4.0});      // Q{1}{1,3}
    Q->cells[1]->cells[2 + 0 * 5] = sparse(n, {0, 3}, {3, 0}, {5.0, 6.0}, {});   // Q{2}{3,1}
    Q->cells[1]->cells[2 + 4 * 5] = sparse(n, {2}, {2}, {7.0}, {-1.0});   // Q{2}{3,5}
    mxArray *R = sparse(n, {0, 1, 2, 3}, {0, 1, 2, 3}, {0, -1, -2, -3}, {});
    mxArray *rho0 = sparse(n, {2}, {0}, {0.5}, {});
    rho0->n = 1; rho0->jc.assign({0, 1});
    mxArray *coil = new mxArray; coil->m = n; coil->n = 1; coil->complex = true;
    coil->cx = {{0, 0}, {1, 2}, {0, 0}, {3, -4}};
    mxArray *grid = strct();
    grid->fields["alphas"] = dense({0, 0, 0});
    grid->fields["betas"] = dense({0.1, 0.2, 0.3});
    grid->fields["gammas"] = dense({1, 2, 3});
    grid->fields["weights"] = dense({0.2, 0.3, 0.5});
    mxArray *opts = strct();
    opts->fields["precision"] = str("single");
    const mxArray *prhs[9] = {I, Q, R, rho0, coil, grid, scalar(1e-5), scalar(5), opts};
    mxArray *plhs[2] = {nullptr, nullptr};
    mexFunction(2, plhs, 9, prhs);
    CHECK(g_rec.n == 4);
    CHECK((g_rec.I_colptr == std::vector<int64_t>{0, 1, 2, 3, 3}));
    CHECK((g_rec.I_rowidx == std::vector<int64_t>{0, 1, 3}));
    CHECK((g_rec.I_values == std::vector<double>{1.5, 0, -2.0, 0, 0.25, 0}));
    CHECK((g_rec.rank == std::vector<int>{1, 2, 2}));
    CHECK((g_rec.k == std::vector<int>{0, 2, 2}));
    CHECK((g_rec.m == std::vector<int>{2, 0, 4}));
    CHECK(g_rec.Q_values.size() == 3 && (g_rec.Q_values[0] == std::vector<double>{3.0, 4.0}));
    CHECK((g_rec.Q_values[1] == std::vector<double>{6.0, 0.0, 5.0, 0.0}));
    CHECK(g_rec.have_R && g_rec.R_values.size() == 8 && g_rec.R_values[6] == -3.0);
    CHECK((g_rec.rho0 == std::vector<double>{0, 0, 0, 0, 0.5, 0, 0, 0}));
    CHECK((g_rec.coil == std::vector<double>{0, 0, 1, 2, 0, 0, 3, -4}));
    CHECK(g_rec.n_orient == 3 && g_rec.grid[5] == 0.2 && g_rec.grid[11] == 0.5);
    CHECK(g_rec.dt == 1e-5 && g_rec.nsteps == 5 && g_rec.precision == 1 - 1 && g_rec.want_per);
    CHECK(plhs[0] && plhs[0]->m == 6 && plhs[0]->n == 1 && plhs[0]->complex);
    CHECK(plhs[0]->cx[3].real == 3.0 && plhs[0]->cx[3].imag == -1.5);
    CHECK(plhs[1] && plhs[1]->m == 6 && plhs[1]->n == 3 && plhs[1]->cx[6 + 2].real == 102.0);
    // default precision is double, one output
    const mxArray *p8[8] = {I, Q, mxCreateDoubleMatrix(0, 0, mxREAL), dense({0, 1, 0, 0}), coil, grid, scalar(2e-5), scalar(0)};
    mxArray *o1[1] = {nullptr};
    mexFunction(1, o1, 8, p8);
    CHECK(g_rec.precision == 1 && !g_rec.have_R && !g_rec.want_per && o1[0]->m == 1);
    // two coil columns: spx_upload_coils gets both, the FIDs come back as rows
    mxArray *coil2 = new mxArray; coil2->m = n; coil2->n = 2; coil2->complex = true;
    coil2->cx = {{0, 0}, {1, 2}, {0, 0}, {3, -4}, {5, 0}, {0, 0}, {0, 0}, {0, 1}};
    const mxArray *pc[8] = {I, Q, R, rho0, coil2, grid, scalar(1e-5), scalar(5)};
    mxArray *oc[1] = {nullptr};
    mexFunction(1, oc, 8, pc);
    CHECK(g_rec.nchan == 2 && g_rec.coils.size() == 16 && g_rec.coils[8] == 5.0 && g_rec.coils[15] == 1.0);
    CHECK((g_rec.coil == std::vector<double>{0, 0, 1, 2, 0, 0, 3, -4}));
    CHECK(oc[0] && oc[0]->m == 2 && oc[0]->n == 6);
    CHECK(oc[0]->cx[2 * 3 + 1].real == 1003.0 && oc[0]->cx[2 * 3].real == 3.0);
    // error identifiers
    auto expect = [&](int nl, int nr, const mxArray **pr, const char *id) {
        mxArray *o[2] = {nullptr, nullptr};
        try {
            mexFunction(nl, o, nr, pr);
            std::printf("FAIL: no error for %s\n", id);
            ++failures;
        } catch (const MexError &e) {
            if (e.id != id) { std::printf("FAIL: got %s, want %s\n", e.id.c_str(), id); ++failures; }
        }
    };
    expect(1, 3, prhs, "Spinach:spinach_powder_gpu:nrhs");
    const mxArray *badq[8] = {I, grid, R, rho0, coil, grid, scalar(1e-5), scalar(5)};
    expect(1, 8, badq, "Spinach:spinach_powder_gpu:Q");
    const mxArray *badn[8] = {I, Q, R, rho0, coil, grid, scalar(1e-5), scalar(2.5)};
    expect(1, 8, badn, "Spinach:spinach_powder_gpu:nsteps");
    // one rho0 column per orientation: spx_set_initial_states gets all three
    mxArray *rho3 = new mxArray; rho3->m = n; rho3->n = 3;
    rho3->re = {1, 0, 0, 0, 0, 2, 0, 0, 0, 0, 3, 0};
    const mxArray *pr3[8] = {I, Q, R, rho3, coil, grid, scalar(1e-5), scalar(5)};
    mxArray *or3[1] = {nullptr};
    mexFunction(1, or3, 8, pr3);
    CHECK(g_rec.states.size() == 24 && g_rec.states[0] == 1.0 && g_rec.states[2 * 5] == 2.0 && g_rec.states[2 * 10] == 3.0);
    CHECK((g_rec.rho0 == std::vector<double>{1, 0, 0, 0, 0, 0, 0, 0}));
    mxArray *rho2 = new mxArray; rho2->m = n; rho2->n = 2; rho2->re = {1, 0, 0, 0, 0, 2, 0, 0};
    const mxArray *pr2[8] = {I, Q, R, rho2, coil, grid, scalar(1e-5), scalar(5)};
    expect(1, 8, pr2, "Spinach:spinach_powder_gpu:rho0");
    // opts.pulse_op + opts.nloops: the CPMG train (experiments/cpmg.m)
    mxArray *copt = strct();
    copt->fields["pulse_op"] = sparse(n, {0, 1}, {1, 0}, {0.5, 0.5}, {0.0, -0.25});
    copt->fields["nloops"] = scalar(2);
    const mxArray *pcp[9] = {I, Q, R, rho0, coil, grid, scalar(1e-5), scalar(5), copt};
    mxArray *ocp[1] = {nullptr};
    mexFunction(1, ocp, 9, pcp);
    CHECK(g_rec.npoints == 6 && g_rec.nloops == 2 && g_rec.precision == 1 && g_rec.dt == 1e-5);
    CHECK((g_rec.pulse == std::vector<double>{0.5, -0.25, 0.5, 0.0}));
    CHECK(ocp[0] && ocp[0]->m == 30 && ocp[0]->n == 1 && ocp[0]->cx[7].real == 14.0 && ocp[0]->cx[7].imag == 1.0);
    expect(2, 9, pcp, "Spinach:spinach_powder_gpu:nlhs");
    mxArray *copt2 = strct();
    copt2->fields["pulse_op"] = copt->fields["pulse_op"];
    copt2->fields["nloops"] = scalar(0);
    const mxArray *pcp2[9] = {I, Q, R, rho0, coil, grid, scalar(1e-5), scalar(5), copt2};
    expect(1, 9, pcp2, "Spinach:spinach_powder_gpu:cpmg");
    mxArray *copt3 = strct();
    copt3->fields["nloops"] = scalar(1);
    const mxArray *pcp3[9] = {I, Q, R, rho0, coil, grid, scalar(1e-5), scalar(5), copt3};
    expect(1, 9, pcp3, "Spinach:spinach_powder_gpu:cpmg");
    // opts.pulse_op + opts.sequence = 'eseem': the two-pulse echo
    mxArray *eopt = strct();
    eopt->fields["pulse_op"] = copt->fields["pulse_op"];
    eopt->fields["sequence"] = str("eseem");
    eopt->fields["precision"] = str("single");
    const mxArray *pe[9] = {I, Q, R, rho0, coil, grid, scalar(2e-8), scalar(7), eopt};
    mxArray *oe[1] = {nullptr};
    mexFunction(1, oe, 9, pe);
    CHECK(g_rec.npoints == 8 && g_rec.nloops == -1 && g_rec.precision == 0 && g_rec.dt == 2e-8);
    CHECK(oe[0] && oe[0]->m == 8 && oe[0]->n == 1 && oe[0]->cx[5].real == 15.0 && oe[0]->cx[5].imag == -1.0);
    expect(2, 9, pe, "Spinach:spinach_powder_gpu:nlhs");
    mxArray *eoop = strct();
    eoop->fields["pulse_op"] = copt->fields["pulse_op"];
    eoop->fields["sequence"] = str("oopeseem");
    const mxArray *peo[9] = {I, Q, R, rho0, coil, grid, scalar(2e-8), scalar(7), eoop};
    mxArray *oeo[1] = {nullptr};
    mexFunction(1, oeo, 9, peo);
    CHECK(g_rec.nloops == -4 && g_rec.npoints == 8 && g_rec.precision == 1);
    CHECK(oeo[0] && oeo[0]->m == 8 && oeo[0]->cx[5].real == 15.0);
    mxArray *eopt2 = strct();
    eopt2->fields["pulse_op"] = copt->fields["pulse_op"];
    eopt2->fields["sequence"] = str("hahn");
    const mxArray *pe2[9] = {I, Q, R, rho0, coil, grid, scalar(2e-8), scalar(7), eopt2};
    expect(1, 9, pe2, "Spinach:spinach_powder_gpu:sequence");
    mxArray *eopt3 = strct();
    eopt3->fields["sequence"] = str("eseem");
    const mxArray *pe3[9] = {I, Q, R, rho0, coil, grid, scalar(2e-8), scalar(7), eopt3};
    expect(1, 9, pe3, "Spinach:spinach_powder_gpu:sequence");
    // opts.ex_prob + opts.ex_pump + opts.sequence = 'deer': three-pulse DEER
    mxArray *dopt = strct();
    dopt->fields["ex_prob"] = copt->fields["pulse_op"];
    dopt->fields["ex_pump"] = sparse(n, {2}, {3}, {0.25}, {});
    dopt->fields["sequence"] = str("deer");
    const mxArray *pd[9] = {I, Q, R, rho0, coil, grid, scalar(4e-9), scalar(6), dopt};
    mxArray *od[1] = {nullptr};
    mexFunction(1, od, 9, pd);
    CHECK(g_rec.nloops == -3 && g_rec.nsteps == 6 && g_rec.dt == 4e-9 && g_rec.precision == 1);
    CHECK(g_rec.pump.size() == 2 && g_rec.pump[0] == 0.25);
    CHECK(od[0] && od[0]->m == 7 && od[0]->n == 1 && od[0]->cx[2].real == 14.0 && od[0]->cx[2].imag == 0.5);
    expect(2, 9, pd, "Spinach:spinach_powder_gpu:nlhs");
    const mxArray *pd0[9] = {I, Q, R, rho0, coil, grid, scalar(4e-9), scalar(0), dopt};
    expect(1, 9, pd0, "Spinach:spinach_powder_gpu:nsteps");
    mxArray *dopt2 = strct();
    dopt2->fields["ex_prob"] = copt->fields["pulse_op"];
    dopt2->fields["sequence"] = str("deer");
    const mxArray *pd2[9] = {I, Q, R, rho0, coil, grid, scalar(4e-9), scalar(6), dopt2};
    expect(1, 9, pd2, "Spinach:spinach_powder_gpu:sequence");
    // opts.pulse_ops + opts.program: a pulse program (hp_acquire with an echo)
    mxArray *popt = strct();
    mxArray *pops = cell(1, 2);
    pops->cells[0] = copt->fields["pulse_op"];
    pops->cells[1] = sparse(n, {2}, {3}, {0.75}, {});
    popt->fields["pulse_ops"] = pops;
    mxArray *pg = new mxArray; pg->m = 3; pg->n = 6;
    pg->re = {0, 1, 1,   1, 0, 0,   1.5, 0, 0,   0, 1, 9,   0, 4e-5, 1e-5,   0, 0, 1};   // column-major
    popt->fields["program"] = pg;
    const mxArray *pp[9] = {I, Q, R, rho0, coil, grid, scalar(1e-5), scalar(5), popt};
    mxArray *op_[1] = {nullptr};
    mexFunction(1, op_, 9, pp);
    CHECK(g_rec.nloops == -2 && g_rec.npoints == 3 && g_rec.precision == 1);
    CHECK((g_rec.grid == std::vector<double>{0, 0, 1.5, 0, 0, 0,  1, 0, 0, 1, 4e-5, 0,  1, 0, 0, 9, 1e-5, 1}));
    CHECK(g_rec.pulse.size() == 6 && g_rec.pulse[4] == 0.75);
    CHECK(op_[0] && op_[0]->m == 10 && op_[0]->n == 1 && op_[0]->cx[3].real == 15.0 && op_[0]->cx[3].imag == 2.0);
    mxArray *pg2 = new mxArray; pg2->m = 1; pg2->n = 6; pg2->re = {0, 3, 1.0, 0, 0, 0};         // pulse 3 of 2
    mxArray *popt2 = strct();
    popt2->fields["pulse_ops"] = pops;
    popt2->fields["program"] = pg2;
    const mxArray *pp2[9] = {I, Q, R, rho0, coil, grid, scalar(1e-5), scalar(5), popt2};
    expect(1, 9, pp2, "Spinach:spinach_powder_gpu:program");
    expect(2, 9, pp, "Spinach:spinach_powder_gpu:nlhs");
    mxArray *o2[2] = {nullptr, nullptr};
    expect(2, 8, pc, "Spinach:spinach_powder_gpu:nlhs");
    (void)o2;
    g_rec.fail_run = 1;
    expect(1, 8, p8, "Spinach:spinach_powder_gpu:run");
    stub_run_atexit();
    std::printf(failures ? "FAILED %d\n" : "PASS\n", failures);
    return failures ? 1 : 0;
}
