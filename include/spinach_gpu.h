/*
 * spinach_gpu.h -- C ABI of the GB300 powder-FID engine.
 *
 * Replaces, on one GPU, the static powder path of Spinach:
 *   [fid,grid] = powder(spin_system, @acquire, parameters, assumptions)
 *     kernel/contexts/powder.m:99-309   (orientation loop and weighted sum)
 *     kernel/orientation.m:29-57        (H = I + sum D(k,m) Q{r}{k,m}, Hermitised)
 *     kernel/relaxation.m:72-93         (R, added as L = H + 1i*R, acquire.m:48)
 *     experiments/acquire.m:42-73       (dt = 1/sweep, nsteps = npoints-1)
 *     kernel/evolution.m:503-587        (observable: fid(n) = coil'*rho(n))
 *     kernel/propagator.m / krylov.m / step.m  (action of exp(-1i*L*dt))
 *
 * The caller (a MATLAB MEX gateway, Python ctypes, C or C++) passes the
 * matrices that kernel/hamiltonian.m returns once per powder call: the
 * isotropic part I and the non-empty rotational-basis terms Q{r}{k,m}, all
 * in MATLAB's own sparse layout (CSC, 0-based row indices, interleaved
 * complex double).  Inputs are read-only and owned by the caller; every
 * output buffer is caller-allocated.  No C++ exception crosses this ABI;
 * every entry point returns an spx_status.
 *
 * Threading: one handle per host thread.  A handle owns one CUDA stream and
 * its device buffers; calls on one handle are serialised by the caller.
 */
#ifndef SPINACH_GPU_H
#define SPINACH_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    SPX_OK = 0,
    SPX_ERR_INVALID_ARGUMENT = 1,   /* bad sizes, NULL pointers, non-finite input */
    SPX_ERR_NO_SYSTEM = 2,          /* spx_run_powder before spx_upload_system */
    SPX_ERR_CUDA = 3,               /* a CUDA runtime call failed */
    SPX_ERR_UNSUPPORTED = 4,        /* input outside this engine's scope */
    SPX_ERR_SERIES = 5,             /* the device series did not converge (status word set) */
    SPX_ERR_NORM = 6,               /* |L*dt| too large (kernel/step.m:230-233 analogue) */
    SPX_ERR_OUT_OF_MEMORY = 7,
    SPX_ERR_INTERNAL = 8
} spx_status;

typedef enum { SPX_FP32 = 0, SPX_FP64 = 1 } spx_precision;

/* One sparse matrix in MATLAB CSC layout (mxGetJc / mxGetIr / mxGetComplexDoubles). */
typedef struct {
    int64_t n;                 /* rows == columns */
    const int64_t *colptr;     /* n+1 entries, colptr[0] == 0 */
    const int64_t *rowidx;     /* colptr[n] entries, 0-based */
    const double *values;      /* 2*colptr[n] doubles, interleaved (re, im) */
} spx_csc;

/* Run options.  Zero-initialise and set what you need; zeros mean "auto". */
typedef struct {
    int32_t precision;         /* spx_precision: storage/arithmetic of the propagation */
    int32_t chunk_steps;       /* time steps covered by one series expansion, 0 = auto */
    int32_t threads;           /* CTA size, 0 = auto; up to 512 (FP32 with at most two 32-row slices per warp: 768) */
    int32_t cluster;           /* CTAs sharing one orientation (1, 2, 4, 8), 0 = auto:
                                  the smallest whose per-CTA share of L fits shared memory */
    double series_tol;         /* truncation tolerance of the series, 0 = auto */
    double chunk_target;       /* series argument s*M*dt one expansion covers, 0 = auto
                                  (the autotuned value, else the largest that fits) */
    int32_t lanczos_its;       /* Lanczos steps of the per-orientation spectral bound,
                                  0 = 32, else 2..48 (fewer: looser, cheaper bounds) */
    int32_t flags;             /* SPX_FLAG_* bits, 0 = defaults */
} spx_options;

/*
 * FP32 runs of spx_run_powder and spx_run_powder_device re-run
 * SPX_FP32_CHECKED_ORIENTATIONS orientations of the grid (evenly spaced) in
 * FP64 on a second stream while the FP32 run proceeds on the other SMs, and
 * report the largest relative 2-norm error of their FIDs in
 * spx_stats.fp32_rel_error and the error it implies for the powder FID in
 * spx_stats.fp32_powder_error.  When the error of what the caller receives
 * (the powder FID, and every orientation's FID when fids_per_orient is
 * given) exceeds half of SPX_FP32_ERROR_BAR (a margin for an estimate drawn
 * from two orientations), spx_run_powder runs the whole grid again in FP64
 * and returns that result (spx_stats.promoted_fp64 = 1);
 * spx_run_powder_device only reports the errors.
 */
#define SPX_FP32_ERROR_BAR 1e-5
#define SPX_FP32_CHECKED_ORIENTATIONS 2
#define SPX_FLAG_NO_FP32_CHECK 1   /* skip the FP64 check of an FP32 run */
#define SPX_FLAG_NO_PROMOTE 2      /* report the check, never re-run in FP64 */

/* Statistics of the last spx_run_powder* call on a handle. */
typedef struct {
    int64_t n_orientations;
    int64_t nsteps;
    int64_t matvecs;           /* Liouvillian actions executed, summed over orientations */
    int64_t orientations_failed;
    int32_t chunk_steps;
    int32_t max_terms;         /* largest series length used by any orientation */
    int32_t threads;
    int32_t precision;
    double kernel_ms;          /* propagation kernel, CUDA events on the handle stream */
    double reduce_ms;          /* powder summation kernel */
    double min_half_width;     /* smallest / largest spectral half-width seen (rad/s) */
    double max_half_width;
    int64_t dim;
    int64_t nnz;               /* stored Liouvillian non-zeros (diagonal included) */
    int64_t ell_entries;       /* padded sliced-ELL entries (off-diagonal) */
    int32_t value_streams;     /* per-non-zero value streams combined per orientation */
    int32_t real_offdiag;      /* 1 if off-diagonal Liouvillian values are real */
    int32_t cluster;           /* CTAs that shared one orientation (thread-block cluster size) */
    int32_t smem_bytes;        /* dynamic shared memory of each CTA */
    int32_t channels;          /* detection channels of the run */
    int32_t retries;           /* 1 if spx_run_powder re-ran after a device status
                                  (wider series table and the safe spectral bound) */
    int32_t fp32_checked;      /* orientations of the last FP32 run that were also run in
                                  FP64 to measure its error (0: not measured) */
    int64_t kernel_launches;   /* run kernels this handle has launched since spx_create
                                  (propagation, powder sums, pulses, echo forms, checks;
                                  spx_build_system's construction kernels not included) */
    double fp32_rel_error;     /* largest relative 2-norm error ||f32 - f64|| / ||f64|| of
                                  the checked orientations' FIDs (0 when not measured) */
    int32_t promoted_fp64;     /* 1 if spx_run_powder found the FP32 error above the
                                  bar and returned an FP64 re-run instead */
    int32_t reserved;
    double fp32_powder_error;  /* the error those imply for the powder FID, two parts in
                                  quadrature: the checked orientations' running relative
                                  error weighted by the powder FID's intensity over time,
                                  and their rms error norm summed as independent errors
                                  over the grid weights (0 when not measured) */
} spx_stats;

typedef struct spx_handle spx_handle;

/* Create a handle bound to CUDA device `device` (cudaSetDevice semantics). */
spx_status spx_create(spx_handle **handle, int device);

/* Release every device buffer and the stream of a handle.  NULL is a no-op. */
spx_status spx_destroy(spx_handle *handle);

/*
 * Builds I and Q{r}{k,m} on the GPU from the interaction content and uploads
 * the system (replaces [I,Q]=hamiltonian(assume(spin_system,...)) of
 * kernel/hamiltonian.m:59-790 with kernel/operators/superop.m:36-185, followed
 * by spx_upload_system).
 *   mults[n_spins]       spin multiplicities (2..8)
 *   basis_keys[dim]      basis states as mixed-radix keys sum_s code_s*radix[s],
 *                        code_s = l*l+l-m of spin s (kernel/indexing/lm2lin.m),
 *                        strictly ascending; radix[s] = prod_{s'>s} mults[s']^2
 *   rank/k/m[n_terms]    the anisotropic terms (as spx_upload_system)
 *   mono_*[n_mono]       monomials coef * [T(code_a)@spin_a T(code_b)@spin_b, .]:
 *                        mono_term 0 = isotropic part, t = anisotropic term t-1;
 *                        mono_spins/mono_codes two per monomial (spin -1: none);
 *                        mono_coefs interleaved complex
 *   r_diag[dim]          diagonal relaxation superoperator (real) or NULL
 *   rho0, coil           as spx_upload_system
 *   build_ms             device time of the construction (may be NULL)
 * Coefficients equal in every monomial of a term may be summed by the caller;
 * entries whose contributions cancel (to 1e-14 of their magnitudes) are dropped.
 */
spx_status spx_build_system(spx_handle *handle, int32_t n_spins, const int32_t *mults, int64_t dim,
                            const int64_t *basis_keys, const int64_t *radix, int32_t n_terms, const int32_t *rank,
                            const int32_t *k, const int32_t *m, int64_t n_mono, const int32_t *mono_term,
                            const int32_t *mono_spins, const int32_t *mono_codes, const double *mono_coefs,
                            const double *r_diag, const double *rho0, const double *coil, double *build_ms);

/*
 * Upload one spin system: the isotropic part I, n_terms rotational-basis
 * terms Q{rank}{k,m} (rank 1 or 2, 0-based k, m in 0..2*rank), the
 * relaxation superoperator R (diagonal; may be NULL for no relaxation), and
 * the initial state rho0 and detection state coil (2*n doubles each,
 * interleaved complex).  Replaces any previously uploaded system.
 * The Liouvillian of an orientation is L = (H+H')/2 + 1i*R with
 * H = I + sum_t D^{rank_t}(alpha,beta,gamma)(k_t,m_t) Q_t.
 */
spx_status spx_upload_system(spx_handle *handle, const spx_csc *I,
                             int32_t n_terms, const int32_t *rank,
                             const int32_t *k, const int32_t *m,
                             const spx_csc *Q, const spx_csc *R,
                             const double *rho0, const double *coil);

/*
 * Powder-averaged FID over an orientation grid (host buffers).  alphas,
 * betas, gammas, weights: n_orient doubles.  fid: 2*(nsteps+1) doubles
 * (interleaved complex), fid = sum_n weights(n) * fid_n.  fids_per_orient:
 * optional (NULL to skip), 2*(nsteps+1)*n_orient doubles, orientation-major
 * (the parameters.sum_up=false output of powder.m:291-297).
 */
spx_status spx_run_powder(spx_handle *handle, int64_t n_orient,
                          const double *alphas, const double *betas,
                          const double *gammas, const double *weights,
                          double dt, int64_t nsteps, const spx_options *opt,
                          double *fid, double *fids_per_orient);

/*
 * Same computation with every array already in device memory of the
 * handle's device (inputs n_orient doubles each; d_fid 2*(nsteps+1)
 * doubles).  Work is enqueued on the handle's stream and the call returns
 * without synchronising; spx_stats timings are filled at the next
 * synchronising call (spx_synchronize, spx_run_powder, spx_get_stats).
 */
spx_status spx_run_powder_device(spx_handle *handle, int64_t n_orient,
                                 const double *d_alphas, const double *d_betas,
                                 const double *d_gammas, const double *d_weights,
                                 double dt, int64_t nsteps, const spx_options *opt,
                                 double *d_fid);

/*
 * Powder run that allocates nothing (no counterpart in the reference).
 *
 * For callers that cannot allocate device memory while they run: a host that
 * reserves all GPU memory up front (for example a MATLAB session whose
 * gpuArray pool already holds it, or instrument software that budgets memory
 * at start-up) and code that must not trigger the implicit device-wide
 * synchronisation a cudaMalloc/cudaFree can cause.  Uses the system already
 * uploaded on the handle (with its detection channels and per-orientation
 * initial states, if set); the grid (d_alphas, d_betas, d_gammas, d_weights:
 * n_orient doubles each) and d_fid (2*(nsteps+1) doubles per channel, channel
 * by channel) are caller-owned device memory.  Every intermediate lives in one static device array of
 * SPX_NOALLOC_SCRATCH_BYTES per GPU (held from library load until process
 * exit); runs needing more return SPX_ERR_UNSUPPORTED before any work is
 * queued (a 1156-dimensional system over 2048 steps fits about 1.8k
 * orientations in FP32 and 0.9k in FP64: the Bessel tables of the 152 CTAs
 * take about 35 MB of the array).  Chunks are capped at 64 steps.  The
 * first call on a device (and the first after the device's context was reset)
 * looks up the array's address.  The call waits for its stream before it
 * returns, so it cannot be captured into a CUDA graph.  Calls share the
 * array, which keeps the last call's contents: calls that overlap on the GPU
 * (other threads or handles on the same device) race.  If an orientation fails
 * its series checks the call returns SPX_ERR_SERIES and d_fid holds no usable
 * result: unlike spx_run_powder it does not retry with conservative bounds,
 * and it leaves the handle's spx_stats as they were.
 */
#define SPX_NOALLOC_SCRATCH_BYTES (64u * 1024u * 1024u)
spx_status spx_run_powder_noalloc(spx_handle *handle, int64_t n_orient,
                                  const double *d_alphas, const double *d_betas,
                                  const double *d_gammas, const double *d_weights,
                                  double dt, int64_t nsteps, int32_t precision,
                                  double *d_fid);

/*
 * Orientation surrogate (no counterpart in the reference; the features follow
 * kernel/utilities/spher_harmon.m).  A multilayer perceptron over the
 * (lmax+1)^2 real spherical harmonics of (beta, gamma): `layers` hidden layers
 * of `hidden` GELU units and n_out linear outputs, FP32 master weights with
 * BF16 copies used in every product (FP32 accumulation).  Parameters are laid
 * out layer by layer as W (out x in, row-major) then b (out).  Every pointer
 * named d_* is device memory of the surrogate's device; h_* is host memory.
 */
typedef struct spx_surrogate spx_surrogate;
spx_status spx_surrogate_create(spx_surrogate **s, int device, int32_t lmax,
                                int32_t hidden, int32_t layers, int32_t n_out,
                                uint64_t seed);
spx_status spx_surrogate_destroy(spx_surrogate *s);
int64_t spx_surrogate_num_params(const spx_surrogate *s);
/* n x (lmax+1)^2 features, row-major: per l, Re Y_l0 then Re/Im Y_lm, m = 1..l. */
spx_status spx_surrogate_features(spx_surrogate *s, int64_t n, const double *d_beta,
                                  const double *d_gamma, float *d_features);
/* Full-batch Adam on the mean squared error against d_targets (n x n_out),
 * cosine-decayed learning rate; h_loss_per_epoch may be NULL. */
spx_status spx_surrogate_train(spx_surrogate *s, int64_t n, const double *d_beta,
                               const double *d_gamma, const float *d_targets,
                               int32_t epochs, float lr, float *h_loss_per_epoch);
spx_status spx_surrogate_predict(spx_surrogate *s, int64_t n, const double *d_beta,
                                 const double *d_gamma, float *d_out);
/* One forward and backward pass: loss and the gradient of every parameter. */
spx_status spx_surrogate_gradients(spx_surrogate *s, int64_t n, const double *d_beta,
                                   const double *d_gamma, const float *d_targets,
                                   float *h_grad, float *h_loss);
spx_status spx_surrogate_get_params(spx_surrogate *s, float *h_params);
spx_status spx_surrogate_set_params(spx_surrogate *s, const float *h_params);
const char *spx_surrogate_last_error(const spx_surrogate *s);

/*
 * Pulse programs on the evolution core.  A program is a list of operations:
 *   SPX_SEQ_PULSE   state <- exp(-1i*angle*pulse_ops[pulse]) state
 *                   (kernel/step.m with a commutation superoperator)
 *   SPX_SEQ_EVOLVE  nsteps steps of dt under the orientation's Liouvillian
 *                   (kernel/evolution.m); record != 0 appends the powder FID
 *                   coil'*rho at steps 0..nsteps to fid
 * Every orientation starts from rho0 (or its own state after
 * spx_set_initial_states); fid receives sum over recorded segments of
 * (nsteps+1) complex values; fids_per_orient (or NULL) the same for every
 * orientation, orientation-major (powder.m sum_up = false).  Needs one coil.
 */
enum { SPX_SEQ_PULSE = 0, SPX_SEQ_EVOLVE = 1 };
typedef struct spx_seq_op {
    int32_t kind;       /* SPX_SEQ_PULSE or SPX_SEQ_EVOLVE */
    int32_t pulse;      /* PULSE: index into pulse_ops */
    double angle;       /* PULSE: rotation angle (rad) */
    int64_t nsteps;     /* EVOLVE: number of steps */
    double dt;          /* EVOLVE: time step (s) */
    int32_t record;     /* EVOLVE: append this segment's FID */
    int32_t reserved;
} spx_seq_op;

spx_status spx_run_sequence(spx_handle *handle, int64_t n_orient, const double *alphas, const double *betas,
                            const double *gammas, const double *weights, int32_t n_pulse, const spx_csc *pulse_ops,
                            int32_t n_ops, const spx_seq_op *ops, const spx_options *opt, double *fid,
                            double *fids_per_orient);

/*
 * CPMG echo train on the same evolution core (experiments/cpmg.m): a hard
 * 90-degree pulse exp(-1i*(pi/2)*pulse_op) on rho0, npoints-1 steps of
 * acquisition, then nloops times a 180-degree pulse and 2*npoints-1 steps;
 * fid receives the concatenated powder FIDs, npoints*(1 + 2*nloops) complex
 * values.  pulse_op is the pulse's commutation superoperator in the basis of
 * the uploaded system (operator(spin_system,'Lx',...) in Spinach).  Needs one
 * coil; per-orientation initial states (spx_set_initial_states) are used
 * when set.  A program on spx_run_sequence; fids_per_orient (or NULL) as
 * there.
 */
spx_status spx_run_cpmg(spx_handle *handle, int64_t n_orient, const double *alphas, const double *betas,
                        const double *gammas, const double *weights, double dt, int64_t npoints, int32_t nloops,
                        const spx_csc *pulse_op, const spx_options *opt, double *fid, double *fids_per_orient);

/*
 * Two-pulse echo (experiments/esr_dipolar/eseem.m): a 90-degree pulse
 * exp(-1i*(pi/2)*pulse_op) on rho0, a trajectory of npoints-1 steps of
 * timestep/2, a 180-degree pulse on every state of it and the refocusing of
 * state n by n more steps; fid[n] = coil' * that state, powder-summed
 * (npoints complex values); fids_per_orient (or NULL) receives every
 * orientation's echoes, orientation-major.  Needs one coil and the single
 * rho0; the dimension is limited to 8192.
 */
spx_status spx_run_eseem(spx_handle *handle, int64_t n_orient, const double *alphas, const double *betas,
                         const double *gammas, const double *weights, double timestep, int64_t npoints,
                         const spx_csc *pulse_op, const spx_options *opt, double *fid, double *fids_per_orient);

/*
 * Out-of-phase two-pulse echo (experiments/esr_dipolar/oopeseem.m): as
 * spx_run_eseem with a 45-degree first pulse exp(-1i*(pi/4)*pulse_op).
 */
spx_status spx_run_oopeseem(spx_handle *handle, int64_t n_orient, const double *alphas, const double *betas,
                            const double *gammas, const double *weights, double timestep, int64_t npoints,
                            const spx_csc *pulse_op, const spx_options *opt, double *fid, double *fids_per_orient);

/*
 * Three-pulse DEER with hard pulses (experiments/esr_dipolar/
 * deer_3p_hard_deer.m, 'brief' output; replaces the orientation loop of
 * powder.m:226-287 around it): a 90-degree pulse exp(-1i*(pi/2)*ex_prob) on
 * rho0, a trajectory of nsteps steps of stepsize, a 180-degree pump pulse
 * exp(-1i*pi*ex_pump) on every state of it, the refocusing of state j by
 * nsteps-j more steps, a 180-degree probe pulse and nsteps more steps;
 * fid[j] = coil' * that state / norm(coil, 2), powder-summed, j = 0..nsteps
 * (nsteps+1 complex values; the coil is the probe coil).  fids_per_orient
 * (or NULL) receives every orientation's trace, orientation-major.  Needs one
 * coil and the single rho0; the dimension is limited to 8192.
 */
spx_status spx_run_deer(spx_handle *handle, int64_t n_orient, const double *alphas, const double *betas,
                        const double *gammas, const double *weights, double stepsize, int64_t nsteps,
                        const spx_csc *ex_prob, const spx_csc *ex_pump, const spx_options *opt, double *fid,
                        double *fids_per_orient);

/*
 * Per-orientation initial states (kernel/contexts/powder.m:244-254: the
 * 'aniso_eq' equilibrium or a function-handle rho0 evaluated at every grid
 * point).  states holds n_states Liouville vectors, orientation after
 * orientation, interleaved complex; later runs must use grids of exactly
 * n_states orientations and start orientation n from state n.  n_states = 0
 * returns to the single rho0 of spx_upload_system (which also clears them).
 */
spx_status spx_set_initial_states(spx_handle *handle, int64_t n_states, const double *states);

/*
 * Several detection states at once (kernel/evolution.m 'multichannel',
 * evolution.m:589-673: one FID row per coil column).  coils holds nchan
 * (1..8) columns of the Liouville dimension, column-major, interleaved
 * complex; it replaces the coil of spx_upload_system.  With nchan > 1 the
 * columns may hold at most 32 non-zeros together (SPX_ERR_UNSUPPORTED
 * otherwise).  Runs then return nchan FIDs: fid holds nchan*(nsteps+1)
 * complex values, channel by channel, and fids_per_orient / d_fid scale the
 * same way.
 */
spx_status spx_upload_coils(spx_handle *handle, int32_t nchan, const double *coils);

/*
 * Autotuner (no counterpart in the reference, whose step.m/propagator.m pick
 * their branch from fixed tolerances).  Times candidate launch shapes -- CTAs
 * per orientation (1, 2, 4, 8), warps per CTA, series length per chunk -- on
 * one wave of the given device-resident orientations over at most 512 steps,
 * and keeps the fastest in the handle: later runs whose options leave
 * threads, cluster and chunk_target at 0 use it.  Results are cached per
 * system shape (dimension, ELL size, value streams, precision, spectral
 * scale) for the life of the process.  best (may be NULL) receives the chosen
 * options; spx_stats reports what a run used.
 */
spx_status spx_autotune(spx_handle *handle, int64_t n_orient, const double *d_alphas, const double *d_betas,
                        const double *d_gammas, double dt, int64_t nsteps, int32_t precision,
                        spx_options *best);

/*
 * Batched powders (no counterpart in the reference, which runs systems one
 * powder() call at a time).  Captures one powder run of each of n handles --
 * each with its own uploaded system, device-resident grid and output (the
 * arguments of spx_run_powder_device, one entry per handle) -- into one CUDA
 * graph whose per-system launches sit on parallel branches.  The handles'
 * buffers are sized at creation; the handles must not run anything else
 * while the batch exists.
 */
typedef struct spx_batch spx_batch;
spx_status spx_batch_create(spx_batch **batch, int32_t n, spx_handle *const *handles, const int64_t *n_orient,
                            const double *const *d_alphas, const double *const *d_betas,
                            const double *const *d_gammas, const double *const *d_weights, const double *dt,
                            const int64_t *nsteps, const spx_options *opts, double *const *d_fids);
/* One launch of the whole graph on stream (a cudaStream_t; NULL = the batch's own stream). */
spx_status spx_batch_launch(spx_batch *batch, void *stream);
/* Wait for the last launch and check every system's status; ms = graph time (may be NULL). */
spx_status spx_batch_synchronize(spx_batch *batch, double *ms);
spx_status spx_batch_destroy(spx_batch *batch);
/* Detail of the batch's last error; with batch NULL, why this thread's last spx_batch_create failed. */
const char *spx_batch_last_error(const spx_batch *batch);

/* Wait for all work on the handle's stream; returns the device status. */
spx_status spx_synchronize(spx_handle *handle);

/* The handle's cudaStream_t, for callers that time or order work around it. */
void *spx_get_stream(spx_handle *handle);

/* Statistics of the last run (synchronises). */
spx_status spx_get_stats(spx_handle *handle, spx_stats *stats);

/* Static text of a status code. */
const char *spx_status_string(spx_status status);

/* Detail of the last error on a handle (empty string if none). */
const char *spx_last_error(const spx_handle *handle);

/* Library version string. */
const char *spx_version(void);

#ifdef __cplusplus
}
#endif

#endif /* SPINACH_GPU_H */
