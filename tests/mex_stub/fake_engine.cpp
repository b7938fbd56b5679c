// Recording stand-in for the engine's C ABI (test support): stores what the
// gateway passed and returns a deterministic FID, so the gateway's marshalling
// is checked without a GPU.
#include <cstring>
#include <string>
#include <vector>

#include "spinach_gpu.h"

struct spx_handle { int dummy; };

struct Recorded {
    int64_t n = 0;
    std::vector<int64_t> I_colptr, I_rowidx;
    std::vector<double> I_values;
    std::vector<int> rank, k, m;
    std::vector<std::vector<double>> Q_values;
    bool have_R = false;
    std::vector<double> R_values, rho0, coil, coils, states, grid;
    int nchan = 1;
    double dt = 0;
    int64_t nsteps = 0, n_orient = 0;
    int precision = -1;
    bool want_per = false;
    int fail_run = 0;
    std::vector<double> pulse, pump;
    int64_t npoints = 0;
    int nloops = 0;
} g_rec;

static spx_handle g_h;

extern "C" {
spx_status spx_create(spx_handle **h, int) { *h = &g_h; return SPX_OK; }
spx_status spx_destroy(spx_handle *) { return SPX_OK; }
spx_status spx_upload_system(spx_handle *, const spx_csc *I, int32_t nt, const int32_t *rank, const int32_t *k,
                             const int32_t *m, const spx_csc *Q, const spx_csc *R, const double *rho0,
                             const double *coil) {
    const int64_t n = I->n;
    g_rec.n = n;
    g_rec.I_colptr.assign(I->colptr, I->colptr + n + 1);
    g_rec.I_rowidx.assign(I->rowidx, I->rowidx + I->colptr[n]);
    g_rec.I_values.assign(I->values, I->values + 2 * I->colptr[n]);
    g_rec.rank.assign(rank, rank + nt);
    g_rec.k.assign(k, k + nt);
    g_rec.m.assign(m, m + nt);
    g_rec.Q_values.clear();
    for (int t = 0; t < nt; ++t) g_rec.Q_values.emplace_back(Q[t].values, Q[t].values + 2 * Q[t].colptr[n]);
    g_rec.have_R = R != nullptr;
    if (R) g_rec.R_values.assign(R->values, R->values + 2 * R->colptr[n]);
    g_rec.rho0.assign(rho0, rho0 + 2 * n);
    g_rec.coil.assign(coil, coil + 2 * n);
    g_rec.nchan = 1;
    g_rec.coils.clear();
    g_rec.states.clear();
    return SPX_OK;
}
spx_status spx_set_initial_states(spx_handle *, int64_t n_states, const double *states) {
    g_rec.states.assign(states, states + 2 * g_rec.n * n_states);
    return SPX_OK;
}
spx_status spx_upload_coils(spx_handle *, int32_t nchan, const double *coils) {
    g_rec.nchan = nchan;
    g_rec.coils.assign(coils, coils + 2 * g_rec.n * nchan);
    return SPX_OK;
}
spx_status spx_run_powder(spx_handle *, int64_t no, const double *a, const double *b, const double *g,
                          const double *w, double dt, int64_t nsteps, const spx_options *opt, double *fid,
                          double *per) {
    if (g_rec.fail_run) return SPX_ERR_SERIES;
    g_rec.n_orient = no;
    g_rec.grid.clear();
    for (int64_t i = 0; i < no; ++i) { g_rec.grid.push_back(a[i]); g_rec.grid.push_back(b[i]);
                                       g_rec.grid.push_back(g[i]); g_rec.grid.push_back(w[i]); }
    g_rec.dt = dt;
    g_rec.nsteps = nsteps;
    g_rec.precision = opt ? opt->precision : -1;
    g_rec.want_per = per != nullptr;
    for (int c = 0; c < g_rec.nchan; ++c)
        for (int64_t i = 0; i <= nsteps; ++i) {
            fid[2 * (c * (nsteps + 1) + i)] = (double)i + 1000.0 * c;
            fid[2 * (c * (nsteps + 1) + i) + 1] = -0.5 * i;
        }
    if (per)
        for (int64_t o = 0; o < no; ++o)
            for (int64_t i = 0; i <= nsteps; ++i) {
                per[2 * (o * (nsteps + 1) + i)] = 100.0 * o + i;
                per[2 * (o * (nsteps + 1) + i) + 1] = 1.0;
            }
    return SPX_OK;
}
spx_status spx_run_cpmg(spx_handle *, int64_t no, const double *, const double *, const double *, const double *,
                        double dt, int64_t npoints, int32_t nloops, const spx_csc *P, const spx_options *opt,
                        double *fid, double *) {
    g_rec.n_orient = no;
    g_rec.dt = dt;
    g_rec.npoints = npoints;
    g_rec.nloops = nloops;
    g_rec.precision = opt ? opt->precision : -1;
    g_rec.pulse.assign(P->values, P->values + 2 * P->colptr[P->n]);
    for (int64_t i = 0; i < npoints * (1 + 2 * nloops); ++i) { fid[2 * i] = 2.0 * i; fid[2 * i + 1] = 1.0; }
    return SPX_OK;
}
spx_status spx_run_sequence(spx_handle *, int64_t no, const double *, const double *, const double *,
                            const double *, int32_t n_pulse, const spx_csc *P, int32_t n_ops, const spx_seq_op *ops,
                            const spx_options *opt, double *fid, double *) {
    g_rec.n_orient = no;
    g_rec.precision = opt ? opt->precision : -1;
    g_rec.nloops = -2;
    g_rec.npoints = n_ops;
    g_rec.pulse.clear();
    for (int k = 0; k < n_pulse; ++k) g_rec.pulse.insert(g_rec.pulse.end(), P[k].values, P[k].values + 2 * P[k].colptr[P[k].n]);
    g_rec.grid.clear();
    int64_t npts = 0;
    for (int i = 0; i < n_ops; ++i) {
        g_rec.grid.push_back(ops[i].kind);
        g_rec.grid.push_back(ops[i].pulse);
        g_rec.grid.push_back(ops[i].angle);
        g_rec.grid.push_back((double)ops[i].nsteps);
        g_rec.grid.push_back(ops[i].dt);
        g_rec.grid.push_back(ops[i].record);
        if (ops[i].kind == SPX_SEQ_EVOLVE && ops[i].record) npts += ops[i].nsteps + 1;
    }
    for (int64_t i = 0; i < npts; ++i) { fid[2 * i] = 5.0 * i; fid[2 * i + 1] = 2.0; }
    return SPX_OK;
}
spx_status spx_run_eseem(spx_handle *, int64_t no, const double *, const double *, const double *, const double *,
                         double dt, int64_t npoints, const spx_csc *P, const spx_options *opt, double *fid,
                         double *) {
    g_rec.n_orient = no;
    g_rec.dt = dt;
    g_rec.npoints = npoints;
    g_rec.nloops = -1;
    g_rec.precision = opt ? opt->precision : -1;
    g_rec.pulse.assign(P->values, P->values + 2 * P->colptr[P->n]);
    for (int64_t i = 0; i < npoints; ++i) { fid[2 * i] = 3.0 * i; fid[2 * i + 1] = -1.0; }
    return SPX_OK;
}
spx_status spx_run_oopeseem(spx_handle *h, int64_t no, const double *a, const double *b, const double *c,
                            const double *w, double dt, int64_t npoints, const spx_csc *P, const spx_options *opt,
                            double *fid, double *per) {
    spx_run_eseem(h, no, a, b, c, w, dt, npoints, P, opt, fid, per);
    g_rec.nloops = -4;
    return SPX_OK;
}
spx_status spx_run_deer(spx_handle *, int64_t no, const double *, const double *, const double *, const double *,
                        double dt, int64_t nsteps, const spx_csc *Pp, const spx_csc *Pu, const spx_options *opt,
                        double *fid, double *) {
    g_rec.n_orient = no;
    g_rec.dt = dt;
    g_rec.nsteps = nsteps;
    g_rec.nloops = -3;
    g_rec.precision = opt ? opt->precision : -1;
    g_rec.pulse.assign(Pp->values, Pp->values + 2 * Pp->colptr[Pp->n]);
    g_rec.pump.assign(Pu->values, Pu->values + 2 * Pu->colptr[Pu->n]);
    for (int64_t i = 0; i <= nsteps; ++i) { fid[2 * i] = 7.0 * i; fid[2 * i + 1] = 0.5; }
    return SPX_OK;
}
spx_status spx_run_powder_device(spx_handle *, int64_t, const double *, const double *, const double *,
                                 const double *, double, int64_t, const spx_options *, double *) {
    return SPX_ERR_UNSUPPORTED;
}
spx_status spx_synchronize(spx_handle *) { return SPX_OK; }
void *spx_get_stream(spx_handle *) { return nullptr; }
spx_status spx_get_stats(spx_handle *, spx_stats *s) { std::memset(s, 0, sizeof *s); return SPX_OK; }
const char *spx_status_string(spx_status s) { return s == SPX_OK ? "success" : "fake failure"; }
const char *spx_last_error(const spx_handle *) { return "recorded"; }
const char *spx_version(void) { return "fake"; }
}
