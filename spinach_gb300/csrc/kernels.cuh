// Device code of the GB300 powder-FID engine.
//
// One CTA -- or a thread-block cluster of 2-8 CTAs for systems whose share of
// L does not fit one SM -- owns one orientation at a time (persistent grid,
// orientations handed out by a work counter).  For each orientation it
//   1. forms the Wigner-D coefficients of its Euler angles in FP64
//      (kernel/utilities/wigner.m:45-77) and assembles the Hermitised
//      Liouvillian L = Ih + sum_t Re(D_t) S_t + Im(D_t) A_t + 1i R on the
//      shared sparsity pattern straight into shared memory
//      (kernel/orientation.m:38-57, kernel/contexts/powder.m:235,263,
//      experiments/acquire.m:48);
//   2. bounds the spectrum of the Hermitian part with a short Lanczos run
//      (clamped by Gershgorin discs) and rescales L to L~ = (L - c)/s;
//   3. tabulates Bessel coefficients J_k(s*j*dt) for one chunk of M steps;
//   4. propagates the state chunk by chunk with the Chebyshev expansion
//      exp(-1i*L*t) = e^{-1i c t} sum_k (2-d_k0) (-1i)^k J_k(s t) T_k(L~),
//      reading the detection moments mu_k = coil' T_k(L~) rho at every term
//      (fused coil projection, kernel/evolution.m:564 / krylov.m:154) and
//      reconstructing the M FID points of the chunk from them.
// This replaces the reference's per-step action of exp(-1i*L*dt)
// (kernel/propagator.m:34-211 followed by P*rho, or kernel/step.m:204-375);
// the series is exact to the chosen tolerance, so the FID is the same
// quantity the reference computes.
//
// FP32 mode stores Liouvillian values as hi+lo float pairs (about 48
// significant bits; on clusters of real values hi + a half-precision low part
// next to the column), keeps series coefficients and state vectors in
// (complex) float, and sums every matvec row with a Kahan-compensated
// accumulator in packed f32x2 (re, im) arithmetic, rounding the row value
// once: that is what keeps the phase from drifting over thousands of steps.
// FP64 mode stores everything in double.
#pragma once

#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <math_constants.h>
#include <stdint.h>

#include <type_traits>

namespace spx {

constexpr int kMaxCoef = 128;     // 1 + 2 * (number of rotational-basis terms)
constexpr int kMaxLanczos = 48;
constexpr int kRedSlots = 64;
constexpr int kMaxCluster = 8;    // portable cluster size

enum DeviceStatus : int {
    kDevOk = 0,
    kDevTableTooSmall = 1,   // series longer than the scratch table
    kDevDiverged = 2,        // state norm grew: spectral bound violated
    kDevNonFinite = 3,
    kDevTooManyRows = 4,
};

// FP32 shared-memory layouts.  Liouvillian values are stored compactly (hi
// + lo float pairs) and expanded into f32x2 operand pairs in registers:
//   ValR  real off-diagonal value (hi, lo)                          8 B
//   ValRP real off-diagonal value with its column (cluster launches) 8 B:
//         hi, the low part as a half in units u = 2^-24 / s, and the
//         column index, so the column array is not stored.  s is a power
//         of two with |v| s <= 1: before the rescale to L~ the system's
//         lo_scale (1 / a bound on every assembled off-diagonal entry),
//         after it 1 (an off-diagonal entry of the Hermitian L is at most
//         half its spectral width, so the entries of L~ are below 1).
//         |lo| <= ulp(hi) / 2 <= 2^-24 / s keeps lo / u within [-1, 1]; the
//         half holds 11 bits of it, about 35 bits in all.
//   ValC  complex value (re_hi, im_hi, re_lo, im_lo)               16 B
//   DgS   diagonal (re_hi, re_lo, im, 0)                           16 B
// Series coefficients are few and read by every row, so they stay pre-packed:
//   PackA  h = (re, re, -im, im) in float: a chunk-end sum of float-rounded
//          coefficients loses about as much as storing the chunk-end state
//          in float does, and drops two products per row and term (with the
//          diagonal's relaxation part summed without its own compensation,
//          c1 moved from 2.4e-7 to 2.7e-7 from FP64 and ran 3 % faster)
struct __align__(8) ValR { float hi, lo; };
struct __align__(8) ValRP { float hi; __half lo; uint16_t col; };
static_assert(sizeof(ValRP) == sizeof(ValR), "packed values keep the layout's size");
struct __align__(16) ValC { float rh, ih, rl, il; };
struct __align__(16) DgS { float rh, rl, im, pad; };
struct __align__(16) PackC { float4 h; };
typedef PackC PackA;

// ---------------------------------------------------------------------------
// Precision policies
// ---------------------------------------------------------------------------
template <bool F64, bool CPLX> struct Prec;
template <> struct Prec<false, false> { using Vec = float2;  using Val = ValR;   using Dg = DgS;     using Af = PackA;   using Real = float;  using Acc = float2; };
template <> struct Prec<false, true>  { using Vec = float2;  using Val = ValC;   using Dg = DgS;     using Af = PackA;   using Real = float;  using Acc = float2; };
template <> struct Prec<true, false>  { using Vec = double2; using Val = double;  using Dg = double2; using Af = double2; using Real = double; using Acc = double2; };
template <> struct Prec<true, true>   { using Vec = double2; using Val = double2; using Dg = double2; using Af = double2; using Real = double; using Acc = double2; };

static __device__ __forceinline__ void split(double v, float &hi, float &lo) {
    hi = (float)v;
    lo = (float)(v - (double)hi);
}
static __device__ __forceinline__ void pack(ValR &o, double re, double) { split(re, o.hi, o.lo); }
// writes the value in units 2^-24 / s (s: a power of two with |re| s <= 1),
// keeps the column
static __device__ __forceinline__ void pack_rp(ValRP &o, double re, double s) {
    o.hi = (float)re;
    const float l = (float)((re - (double)o.hi) * (16777216.0 * s));
    o.lo = __float2half_rn(fminf(fmaxf(l, -65504.f), 65504.f));
}
static __device__ __forceinline__ void pack(ValC &o, double re, double im) {
    split(re, o.rh, o.rl);
    split(im, o.ih, o.il);
}
static __device__ __forceinline__ void pack(DgS &o, double re, double im) {
    split(re, o.rh, o.rl);
    o.im = (float)im;
    o.pad = 0.f;
}
static __device__ __forceinline__ void pack(PackC &o, double re, double im) {
    const float r = (float)re, i = (float)im;
    o.h = make_float4(r, r, -i, i);
}
static __device__ __forceinline__ double2 unpack(const ValR &v) { return make_double2((double)v.hi + (double)v.lo, 0.0); }
// value of a packed entry stored in units u
static __device__ __forceinline__ double2 unpack_rp(const ValRP &v, float u) {
    return make_double2((double)v.hi + (double)(__half2float(v.lo) * u), 0.0);
}
// column of ELL entry e: from the column array, or from a packed value
template <class V>
static __device__ __forceinline__ int col_of(const uint16_t *s_col, const V *, int e) { return s_col[e]; }
static __device__ __forceinline__ int col_of(const uint16_t *, const ValRP *s_val, int e) { return s_val[e].col; }
static __device__ __forceinline__ double2 unpack(const ValC &v) {
    return make_double2((double)v.rh + (double)v.rl, (double)v.ih + (double)v.il);
}
static __device__ __forceinline__ double2 unpack(const DgS &v) { return make_double2((double)v.rh + (double)v.rl, (double)v.im); }
static __device__ __forceinline__ void pack(double &o, double re, double) { o = re; }
static __device__ __forceinline__ void pack(double2 &o, double re, double im) { o = make_double2(re, im); }

static __device__ __forceinline__ double2 unpack(const double &v) { return make_double2(v, 0.0); }
static __device__ __forceinline__ double2 unpack(const double2 &v) { return v; }

// y += v * x  (value times complex state; plain arithmetic, used outside the
// propagation loop and in the FP64 path)
static __device__ __forceinline__ void mac(float2 &y, const ValR &v, const float2 x) {
    y.x = fmaf(v.hi, x.x, y.x); y.y = fmaf(v.hi, x.y, y.y);
    y.x = fmaf(v.lo, x.x, y.x); y.y = fmaf(v.lo, x.y, y.y);
}
// packed entry in units u
static __device__ __forceinline__ void mac_rp(float2 &y, const ValRP &v, const float2 x, float u) {
    const float lo = __half2float(v.lo) * u;
    y.x = fmaf(v.hi, x.x, y.x); y.y = fmaf(v.hi, x.y, y.y);
    y.x = fmaf(lo, x.x, y.x); y.y = fmaf(lo, x.y, y.y);
}
static __device__ __forceinline__ void mac(float2 &y, const ValC &v, const float2 x) {
    // (re + i im) x = re*x + (-im*x.y, im*x.x)
    y.x = fmaf(v.rh, x.x, y.x); y.y = fmaf(v.rh, x.y, y.y);
    y.x = fmaf(-v.ih, x.y, y.x); y.y = fmaf(v.ih, x.x, y.y);
    y.x = fmaf(v.rl, x.x, y.x); y.y = fmaf(v.rl, x.y, y.y);
    y.x = fmaf(-v.il, x.y, y.x); y.y = fmaf(v.il, x.x, y.y);
}
static __device__ __forceinline__ void mac(double2 &y, const double &v, const double2 x) {
    y.x = fma(v, x.x, y.x); y.y = fma(v, x.y, y.y);
}
static __device__ __forceinline__ void mac(double2 &y, const double2 &v, const double2 x) {
    y.x = fma(v.x, x.x, y.x); y.x = fma(-v.y, x.y, y.x);
    y.y = fma(v.x, x.y, y.y); y.y = fma(v.y, x.x, y.y);
}
// the same for any stored value; u: units of a packed entry's low part
template <class V>
static __device__ __forceinline__ double2 value_of(const V &v, float) { return unpack(v); }
static __device__ __forceinline__ double2 value_of(const ValRP &v, float u) { return unpack_rp(v, u); }
template <class Y, class V, class X>
static __device__ __forceinline__ void mac_u(Y &y, const V &v, const X x, float) { mac(y, v, x); }
static __device__ __forceinline__ void mac_u(float2 &y, const ValRP &v, const float2 x, float u) { mac_rp(y, v, x, u); }

template <class V> __device__ __forceinline__ V vzero();
template <> __device__ __forceinline__ float2 vzero<float2>() { return make_float2(0.f, 0.f); }
template <> __device__ __forceinline__ double2 vzero<double2>() { return make_double2(0.0, 0.0); }

static __device__ __forceinline__ float2 tovec(double2 a, float2) { return make_float2((float)a.x, (float)a.y); }
static __device__ __forceinline__ double2 tovec(double2 a, double2) { return a; }
static __device__ __forceinline__ double2 tod(float2 a) { return make_double2(a.x, a.y); }
static __device__ __forceinline__ double2 tod(double2 a) { return a; }

// conj(a) * b accumulated
static __device__ __forceinline__ void cdot_acc(float2 &s, const float2 a, const float2 b) {
    s.x = fmaf(a.x, b.x, s.x); s.x = fmaf(a.y, b.y, s.x);
    s.y = fmaf(a.x, b.y, s.y); s.y = fmaf(-a.y, b.x, s.y);
}
static __device__ __forceinline__ void cdot_acc(double2 &s, const double2 a, const double2 b) {
    s.x = fma(a.x, b.x, s.x); s.x = fma(a.y, b.y, s.x);
    s.y = fma(a.x, b.y, s.y); s.y = fma(-a.y, b.x, s.y);
}

template <class V> __device__ __forceinline__ V warp_sum(V v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        v.x += __shfl_xor_sync(0xffffffffu, v.x, o);
        v.y += __shfl_xor_sync(0xffffffffu, v.y, o);
    }
    return v;
}

// ---------------------------------------------------------------------------
// Packed f32x2 arithmetic (sm_100+ PTX add/sub/mul/fma.rn.f32x2).  A complex
// float is one 64-bit register pair (re, im).  Inline PTX is never contracted
// or reassociated by the compiler, which the Kahan bookkeeping relies on.
// ---------------------------------------------------------------------------
typedef unsigned long long f2x;

static __device__ __forceinline__ f2x f2pk(float a, float b) {
    f2x r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a), "f"(b));
    return r;
}
static __device__ __forceinline__ float2 f2up(f2x v) {
    float2 r;
    asm("mov.b64 {%0, %1}, %2;" : "=f"(r.x), "=f"(r.y) : "l"(v));
    return r;
}
static __device__ __forceinline__ f2x add2(f2x a, f2x b) { f2x r; asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b)); return r; }
static __device__ __forceinline__ f2x sub2(f2x a, f2x b) { f2x r; asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b)); return r; }
static __device__ __forceinline__ f2x mul2(f2x a, f2x b) { f2x r; asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b)); return r; }
static __device__ __forceinline__ f2x fma2(f2x a, f2x b, f2x c) {
    f2x r;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r) : "l"(a), "l"(b), "l"(c));
    return r;
}
static __device__ __forceinline__ f2x swap2(f2x a) { const float2 f = f2up(a); return f2pk(f.y, f.x); }
static __device__ __forceinline__ f2x lo2(const float4 &v) { return f2pk(v.x, v.y); }
static __device__ __forceinline__ f2x hi2(const float4 &v) { return f2pk(v.z, v.w); }

// Kahan-compensated Y += P with the lost low-order part kept in L (Y + L is
// the sum), so that products of the values' low parts can be added into L
// directly (one accumulator per row fewer).
__device__ __forceinline__ void kahan_add2l(f2x &Y, f2x &L, f2x P) {
    const f2x y = add2(P, L);
    const f2x t = add2(Y, y);
    L = sub2(y, sub2(t, Y));
    Y = t;
}
// a * t for a packed complex coefficient (PackC/PackA layout)
static __device__ __forceinline__ f2x cmul_pk(const PackC &a, f2x T) {
    return fma2(hi2(a.h), swap2(T), mul2(lo2(a.h), T));
}

// FP64 helpers of the generic propagation loop
static __device__ __forceinline__ void cmac(double2 &y, const double &v, const double2 x) { mac(y, v, x); }
static __device__ __forceinline__ void cmac(double2 &y, const double2 &v, const double2 x) { mac(y, v, x); }
static __device__ __forceinline__ double2 recur(const double2 &y, double two, const double2 tp) {
    return make_double2(two * y.x - tp.x, two * y.y - tp.y);
}

// Block reduction in the value's own type (op 0 sum, 1 max, 2 min); red holds
// one value per warp.  Every thread of the block must call it.
template <class T> __device__ __forceinline__ T rmax(T a, T b) { return a > b ? a : b; }
template <class T> __device__ __forceinline__ T rmin(T a, T b) { return a < b ? a : b; }
template <int OP, class T>
static __device__ T block_reduce(T v, T *red) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const T u = __shfl_xor_sync(0xffffffffu, v, o);
        v = OP == 0 ? v + u : OP == 1 ? rmax(v, u) : rmin(v, u);
    }
    __syncthreads();
    if (lane == 0) red[warp] = v;
    __syncthreads();
    T r = red[0];
    for (int w = 1; w < nw; ++w) r = OP == 0 ? r + red[w] : OP == 1 ? rmax(r, red[w]) : rmin(r, red[w]);
    return r;
}

// ---------------------------------------------------------------------------
// Thread-block clusters (distributed shared memory).  A cluster of CL CTAs
// shares one orientation: each CTA owns a contiguous block of 32-row slices,
// keeps a full replica of the Chebyshev vectors and pushes the rows it
// computes into every peer's replica; hardware cluster barriers order the
// pushes before the next product reads them.
// ---------------------------------------------------------------------------
static __device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }
static __device__ __forceinline__ int cluster_rank() {
    uint32_t r;
    asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
    return (int)r;
}
static __device__ __forceinline__ uint32_t cluster_addr(uint32_t local, int rank) {
    uint32_t r;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(local), "r"(rank));
    return r;
}
static __device__ __forceinline__ void st_cluster(uint32_t a, unsigned long long v) {
    asm volatile("st.shared::cluster.u64 [%0], %1;" ::"r"(a), "l"(v) : "memory");
}
static __device__ __forceinline__ void st_cluster(uint32_t a, double v) {
    asm volatile("st.shared::cluster.f64 [%0], %1;" ::"r"(a), "d"(v) : "memory");
}
static __device__ __forceinline__ double ld_cluster_f64(uint32_t a) {
    double v;
    asm volatile("ld.shared::cluster.f64 %0, [%1];" : "=d"(v) : "r"(a) : "memory");
    return v;
}
static __device__ __forceinline__ int ld_cluster_s32(uint32_t a) {
    int v;
    asm volatile("ld.shared::cluster.s32 %0, [%1];" : "=r"(v) : "r"(a) : "memory");
    return v;
}
// all threads of all CTAs of the cluster; release/acquire orders shared::cluster stores
template <bool CLU> __device__ __forceinline__ void csync() {
    if constexpr (!CLU) {
        __syncthreads();
    } else {
        asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
    }
}
// write v at the same shared-memory location of every other CTA of the cluster
template <bool CLU> __device__ __forceinline__ void push_peers(const void *p, unsigned long long v, int crank, int cl) {
    if constexpr (CLU) {
        const uint32_t a = smem_u32(p);
        for (int j = 0; j < cl; ++j)
            if (j != crank) st_cluster(cluster_addr(a, j), v);
    }
}
template <bool CLU> __device__ __forceinline__ void push_peers(const float2 *p, float2 v, int crank, int cl) {
    if constexpr (CLU)
        push_peers<CLU>((const void *)p,
                        ((unsigned long long)__float_as_uint(v.y) << 32) | (unsigned long long)__float_as_uint(v.x),
                        crank, cl);
}
template <bool CLU> __device__ __forceinline__ void push_peers(const double2 *p, double2 v, int crank, int cl) {
    if constexpr (CLU) {
        push_peers<CLU>((const void *)p, (unsigned long long)__double_as_longlong(v.x), crank, cl);
        push_peers<CLU>((const void *)(reinterpret_cast<const double *>(p) + 1),
                        (unsigned long long)__double_as_longlong(v.y), crank, cl);
    }
}
// Block reduction followed by a cluster-wide one (op 0 sum, 1 max, 2 min).
// Partial results go to a double-buffered slot array in every CTA; all CTAs
// combine them in rank order, so every CTA gets bit-identical results.
template <bool CLU, int OP, class T = double>
__device__ T cluster_reduce(T v, double *red, double *cred, int &par, int crank, int cl) {
    const T b = block_reduce<OP>(v, reinterpret_cast<T *>(red));
    if constexpr (!CLU) {
        return b;
    } else {
        double *slot = cred + par * kMaxCluster;
        par ^= 1;
        if ((int)threadIdx.x < cl) st_cluster(cluster_addr(smem_u32(slot + crank), (int)threadIdx.x), (double)b);
        csync<CLU>();
        T r = (T)slot[0];
        for (int j = 1; j < cl; ++j) {
            const T u = (T)slot[j];
            r = OP == 0 ? r + u : OP == 1 ? rmax(r, u) : rmin(r, u);
        }
        return r;
    }
}

// ---------------------------------------------------------------------------
// System and run descriptors (device pointers)
// ---------------------------------------------------------------------------
struct DevSystem {
    int n;              // Liouville dimension
    int n_pad;          // nslices * 32
    int nslices;        // 32-row slices of the sliced-ELL layout
    int ell_len;        // padded off-diagonal entries
    const int *slice_off;       // nslices + 1 (entries)
    const uint16_t *ell_col;    // ell_len
    const double *ell_re;       // nstreams * ell_len
    const double *ell_im;       // nstreams * ell_len, or nullptr (real off-diagonal)
    const double2 *diag;        // nstreams * n_pad
    const int *stream_coef;     // nstreams: slot in the per-orientation coefficient vector
    int nstreams;
    int ncoef;                  // 1 + 2 * nterms
    int nterms;
    const int *term_rkm;        // 3 * nterms: rank, k, m (0-based k, m)
    const double2 *rho0;        // n_pad (sliced order)
    const double2 *rho0s;       // per-orientation initial states (n_orient x n_pad, sliced order) or null
    const double2 *coil;        // n_pad (sliced order)
    int ncoil;                  // 1..32: non-zero coil entries listed below; 0 or -1: use the dense coil
    const int *coil_rows;       // ncoil rows (sliced order)
    const double2 *coil_vals;   // ncoil values
    const int *coil_chan;       // ncoil detection channels (0 .. nchan-1)
    int nchan;                  // detection channels (evolution.m 'multichannel'); > 1 needs the listed coil
    double max_im_diag;         // largest |Im L_ii| (relaxation), rad/s
    double lo_scale;            // power of two, at most 1 / (a bound on every assembled off-diagonal entry)
};

struct DevRun {
    int n_orient;
    const double *alpha, *beta, *gamma;
    double dt;
    int nsteps;
    int M;              // largest time-step count per chunk (table height - 1)
    int fixed_chunk;    // 1: every orientation uses M; 0: choose per orientation
    double chunk_x;     // target series argument s*M*dt of one chunk
    int Kmax;           // width of the Bessel table
    double tol;         // series truncation tolerance
    int lanczos_its;
    int safe_bounds;    // 1: theta + beta Lanczos bound clamped by Gershgorin
    void *fids;         // n_orient * (nsteps + 1) complex (precision of the run)
    double *table;      // gridDim.x * Kmax * (M + 1) doubles, per-CTA scratch
    int *status;        // n_orient
    long long *matvecs; // n_orient
    double *halfwidth;  // n_orient
    int *kused;         // n_orient
    int *mused;         // n_orient: time steps per chunk used
    int cl;                 // CTAs per cluster (1: no cluster)
    double2 *state_out;     // or null: the state after the last step, n_orient x n_pad (sliced order)
    double2 *traj_out;      // or null: the state at every time step, n_orient x (nsteps+1) x n_pad (sliced order)
    int traj_m;             // trajectory outputs: steps per chunk (the fixed chunk length; 1 otherwise)
    int *next_orient;       // work counter (zeroed before the launch): single CTAs take
                            // orientations gridDim.x, gridDim.x + 1, ... as they finish
    int cl_slices[kMaxCluster + 1];   // slice boundaries of the CTAs' row blocks (cluster launches)
    int nsl_loc;            // largest slice count of one CTA (shared-memory sizing)
    int ell_loc;            // largest ELL entry count of one CTA
};

// ---------------------------------------------------------------------------
// Wigner D (Brink & Satchler convention, rows/cols from +l to -l), FP64.
// Written from the closed forms d^1 and d^2 of the small-d matrices.
// ---------------------------------------------------------------------------
static __device__ void wigner_element(int rank, int k, int m, double a, double b, double g,
                               double &re, double &im) {
    // projections: row k -> p = rank - k, column m -> q = rank - m
    const int p = rank - k, q = rank - m;
    const double cb = cos(b), sb = sin(b);
    double d = 0.0;
    if (rank == 1) {
        const double s2 = sqrt(0.5);
        const double t[3][3] = {{(1 + cb) / 2, -sb * s2, (1 - cb) / 2},
                                {sb * s2, cb, -sb * s2},
                                {(1 - cb) / 2, sb * s2, (1 + cb) / 2}};
        d = t[k][m];
    } else if (rank == 2) {
        const double c2 = cos(b / 2), s2 = sin(b / 2);
        const double c4 = c2 * c2 * c2 * c2, s4 = s2 * s2 * s2 * s2;
        const double r38 = sqrt(3.0 / 8.0), r32 = sqrt(1.5);
        const double t[5][5] = {
            {c4, -sb * (1 + cb) / 2, r38 * sb * sb, -sb * (1 - cb) / 2, s4},
            {sb * (1 + cb) / 2, (2 * cb - 1) * (1 + cb) / 2, -r32 * sb * cb, (2 * cb + 1) * (1 - cb) / 2, sb * (cb - 1) / 2},
            {r38 * sb * sb, r32 * sb * cb, (3 * cb * cb - 1) / 2, -r32 * sb * cb, r38 * sb * sb},
            {-sb * (cb - 1) / 2, (2 * cb + 1) * (1 - cb) / 2, r32 * sb * cb, (2 * cb - 1) * (1 + cb) / 2, -sb * (cb + 1) / 2},
            {s4, sb * (1 - cb) / 2, r38 * sb * sb, sb * (1 + cb) / 2, c4}};
        d = t[k][m];
    }
    // D(p,q) = exp(-i p a) d(p,q) exp(-i q g)
    const double ph = -(p * a + q * g);
    re = d * cos(ph);
    im = d * sin(ph);
}

// Spectral-bound helpers in FP32: the interval they feed is widened by Ritz
// residuals and 2% of its width, so FP32 digits suffice, and GB300's FP64
// division and transcendentals are two orders of magnitude slower.

// Sturm count: eigenvalues of the symmetric tridiagonal matrix below x.
static __device__ int sturm_count(const float *al, const float *be2, int m, float x) {
    int cnt = 0;
    float q = al[0] - x;
    if (q < 0.f) ++cnt;
    for (int i = 1; i < m; ++i) {
        const float den = (q == 0.f) ? 1e-30f : q;
        q = al[i] - x - be2[i - 1] / den;
        if (q < 0.f) ++cnt;
    }
    return cnt;
}

// Extreme eigenvalues of the tridiagonal matrix by one warp: each round
// evaluates the Sturm count at 32 interior points of the bracket
// (multisection), shrinking it 33-fold, until it is 1e-6 relative.  All lanes
// must call; all get the result.
static __device__ void tridiag_extremes_warp(const double *al_d, const double *be_d, int m, double &lo, double &hi,
                                             int lane) {
    float al[kMaxLanczos], be2[kMaxLanczos];
    float glo = CUDART_INF_F, ghi = -CUDART_INF_F;
    for (int i = 0; i < m; ++i) {
        al[i] = (float)al_d[i];
        be2[i] = (float)(be_d[i] * be_d[i]);
        float r = 0.f;
        if (i > 0) r += fabsf((float)be_d[i - 1]);
        if (i < m - 1) r += fabsf((float)be_d[i]);
        glo = fminf(glo, al[i] - r);
        ghi = fmaxf(ghi, al[i] + r);
    }
    for (int which = 0; which < 2; ++which) {
        const int target = which == 0 ? 1 : m;      // count >= target: right of the wanted eigenvalue
        float a = glo, b = ghi;
        for (int it = 0; it < 12 && b - a > 1e-6f * fmaxf(fabsf(a), fabsf(b)) + 1e-30f; ++it) {
            const float step = (b - a) * (1.f / 33.f);
            const bool right = sturm_count(al, be2, m, a + (lane + 1) * step) >= target;
            const unsigned mask = __ballot_sync(0xffffffffu, right);
            if (mask == 0u) {
                a = a + 32.f * step;
            } else {
                const int j = __ffs(mask) - 1;
                b = a + (j + 1) * step;
                a = a + j * step;
            }
        }
        if (which == 0) lo = b; else hi = a;
    }
}

// |last component| of the normalised eigenvector of the tridiagonal matrix for
// eigenvalue theta, by three steps of inverse iteration (Thomas algorithm).
static __device__ double ritz_last_component(const double *al_d, const double *be_d, int m, double theta_d) {
    if (m <= 1) return 1.0;
    float y[kMaxLanczos], c[kMaxLanczos], d[kMaxLanczos];
    const float theta = (float)theta_d;
    const float shift = theta + 1e-5f * (fabsf(theta) + 1e-30f);
    for (int i = 0; i < m; ++i) y[i] = 1.f;
    for (int it = 0; it < 3; ++it) {
        // solve (T - shift) x = y
        float den = (float)al_d[0] - shift;
        if (den == 0.f) den = 1e-30f;
        c[0] = (float)be_d[0] / den;
        d[0] = y[0] / den;
        for (int i = 1; i < m; ++i) {
            den = ((float)al_d[i] - shift) - (float)be_d[i - 1] * c[i - 1];
            if (den == 0.f) den = 1e-30f;
            c[i] = (i < m - 1) ? (float)be_d[i] / den : 0.f;
            d[i] = (y[i] - (float)be_d[i - 1] * d[i - 1]) / den;
        }
        y[m - 1] = d[m - 1];
        for (int i = m - 2; i >= 0; --i) y[i] = d[i] - c[i] * y[i + 1];
        float nrm = 0.f;
        for (int i = 0; i < m; ++i) nrm += y[i] * y[i];
        nrm = sqrtf(nrm);
        if (!(nrm > 0.f) || !isfinite(nrm)) return 1.0;
        const float inv = 1.f / nrm;
        for (int i = 0; i < m; ++i) y[i] *= inv;
    }
    return fabsf(y[m - 1]);
}

// ---------------------------------------------------------------------------
// Shared-memory layout of the propagation kernel
// ---------------------------------------------------------------------------
template <bool F64, bool CPLX>
struct SmemLayout {
    using P = Prec<F64, CPLX>;
    size_t coef, red, cred, alpha, beta, slice_off, ell_col, ell_val, diag, xa, xb, part, atau, mu, phase, rec, tco, tacc,
        total;
    __host__ __device__ static size_t align(size_t x) { return (x + 15) & ~size_t(15); }
    // n_pad: replicated vector length; nslices / ell_len: the slices and ELL
    // entries one CTA owns (all of them without a cluster)
    // traj_m > 1: trajectory outputs with chunks of traj_m steps (coefficients
    // and accumulators of the traj_m - 1 states inside a chunk)
    // packed: FP32 real values carry their columns (ValRP), no column array
    __host__ __device__ SmemLayout(int n_pad, int nslices, int ell_len, int Kmax, int M, int nthreads, int nchan = 1,
                                   int traj_m = 1, bool packed = false) {
        size_t o = 0;
        coef = o; o = align(o + sizeof(double) * kMaxCoef);
        red = o; o = align(o + sizeof(double) * kRedSlots);
        cred = o; o = align(o + sizeof(double) * 2 * kMaxCluster);
        alpha = o; o = align(o + sizeof(double) * kMaxLanczos);
        beta = o; o = align(o + sizeof(double) * kMaxLanczos);
        slice_off = o; o = align(o + sizeof(int) * (nslices + 1));
        ell_col = o; o = align(o + (packed ? 0 : sizeof(uint16_t) * ell_len));
        ell_val = o; o = align(o + sizeof(typename P::Val) * ell_len);    // sizeof(ValRP) == sizeof(ValR)
        diag = o; o = align(o + sizeof(typename P::Dg) * 32 * (size_t)nslices);
        xa = o; o = align(o + sizeof(typename P::Vec) * n_pad);
        xb = o; o = align(o + sizeof(typename P::Vec) * n_pad);
        part = o; o = align(o + sizeof(typename P::Vec) * 2 * (nthreads / 32));   // two terms in flight
        atau = o; o = align(o + sizeof(typename P::Af) * Kmax);
        mu = o; o = align(o + sizeof(typename P::Vec) * Kmax * nchan);
        phase = o; o = align(o + sizeof(typename P::Vec) * (M + 1));
        rec = o; o = align(o + sizeof(typename P::Vec) * (nthreads > M ? nthreads : M));
        const size_t tm1 = traj_m > 1 ? (size_t)(traj_m - 1) : 0;
        tco = o; o = align(o + sizeof(typename P::Vec) * tm1 * Kmax);
        tacc = o; o = align(o + sizeof(typename P::Vec) * tm1 * 32 * (size_t)nslices);
        total = o;
    }
};

// acc += a * t (FP64 propagation loop)
static __device__ __forceinline__ void acc_add64(double2 &acc, const double2 &a, const double2 t) { mac(acc, a, t); }

// Number of Chebyshev/Bessel terms after which |J_k(x)| * e^{k*lg} < tol
// (Debye-type bound (e x / 2k)^k / sqrt(2 pi k), conservative for k > x).
// Evaluated in FP32 (it only sizes the series; the exact tail is checked
// against the Bessel column itself).
static __device__ int series_terms(double x, double lg, double tol, int kcap) {
    if (!(x > 0.0)) return 1;
    const float ltol = (float)log(tol), xf = (float)x, lgf = (float)lg;
    int k = max(1, (int)ceil(x) + 1);
    while (k < kcap) {
        const float kf = (float)k;
        const float lt = -0.5f * __logf(6.2831853f * kf) + kf * __logf(2.7182818f * xf / (2.f * kf)) + kf * lgf;
        if (lt < ltol) break;
        ++k;
    }
    return k;
}

// Column j of the table T[k][j] = (2 - delta_k0) J_k(half * j * dt), k < K,
// by Miller's backward recurrence J_{k-1} = (2k/x) J_k - J_{k+1}, normalised
// with J_0 + 2 sum J_2k = 1; tiny arguments use the leading terms of the
// power series.
static __device__ void bessel_column(double *table, int M, int j, int K, double half, double dt) {
    double *col = table + j;
    const size_t ld = (size_t)(M + 1);
    const double x = half * j * dt;
    if (x < 1e-6) {
        for (int k = 0; k < K; ++k) col[k * ld] = 0.0;
        col[0] = 1.0 - 0.25 * x * x;
        if (K > 1) col[ld] = 2.0 * 0.5 * x;
        if (K > 2) col[2 * ld] = 2.0 * 0.125 * x * x;
        return;
    }
    const int kneed = min(K, series_terms(x, 0.0, 1e-40, K + 64) + 1);
    const int base = max(kneed, (int)ceil(x));
    int kst = base + 20 + (int)sqrt(160.0 * base);
    kst += kst & 1;
    const double two_over_x = 2.0 / x;                // one division per column
    // Above the stored range the recurrence only has to forget its start (the
    // error it carries there decays towards k = 0), and those terms add below
    // 1e-40 to the normalisation: it runs in float, rescaled well inside the
    // float range (one step grows a value at most kst * 2/x-fold, below 1e9
    // for the arguments x >= 1e-6 that reach it), and hands over to FP64 at
    // the first stored term.
    const float ftx = (float)two_over_x;
    float fjp1 = 0.f, fjk = 1e-30f;
    int k = kst;
    for (; k > kneed; --k) {
        const float fjm1 = ((float)k * ftx) * fjk - fjp1;
        fjp1 = fjk;
        fjk = fjm1;                                 // J_{k-1}, unnormalised
        if (fabsf(fjk) > 1e20f) { fjk *= 1e-20f; fjp1 *= 1e-20f; }
    }
    double jp1 = fjp1, jk = fjk, norm = 0.0;
    for (; k >= 1; --k) {
        const double jm1 = (k * two_over_x) * jk - jp1;
        jp1 = jk;
        jk = jm1;                                   // J_{k-1}, unnormalised, k-1 < kneed
        const int km1 = k - 1;
        if (km1 > 0 && (km1 & 1) == 0) norm += 2.0 * jk;
        col[km1 * ld] = jk;
    }
    norm += jk;                                     // + J_0
    const double inv = 1.0 / norm;
    col[0] = col[0] * inv;
    for (int k = 1; k < kneed; ++k) col[k * ld] = 2.0 * col[k * ld] * inv;
    for (int k = kneed; k < K; ++k) col[k * ld] = 0.0;
}

// Real part of a diagonal entry in the working precision
__device__ __forceinline__ float diag_re(const DgS &d) { return d.rh + d.rl; }
__device__ __forceinline__ double diag_re(const double2 &d) { return d.x; }

// Moment of one term from the per-warp partials in slot `part` (nwarps
// entries), by one warp: lane w takes warp w's partial, then a fixed
// butterfly sum.
template <class Vec>
__device__ __forceinline__ void reduce_term(const Vec *part, int nwarps, int lane, Vec *mu) {
    Vec q = vzero<Vec>();
    if (lane < nwarps) q = part[lane];
    q = warp_sum(q);
    if (lane == 0) *mu = q;
}

// Next orientation of a CTA or cluster: orientations below `first` (one per
// CTA or cluster) were handed out at launch, the counter numbers the rest.  In
// a cluster rank 0 draws and every CTA reads its choice.  All threads call.
template <bool CLU>
static __device__ int next_orientation(int *counter, int *slot, int first, int crank) {
    csync<CLU>();
    if (threadIdx.x == 0 && crank == 0) *slot = first + atomicAdd(counter, 1);
    csync<CLU>();
    if constexpr (CLU) return ld_cluster_s32(cluster_addr(smem_u32(slot), 0));
    return *slot;
}

// Moment coil' x from the few non-zero coil rows (lane i takes row i), one warp.
template <class Vec>
__device__ __forceinline__ void coil_moment(const Vec *x, int ncoil, const int *rows, const Vec *cv, int lane, Vec *mu) {
    Vec q = vzero<Vec>();
    if (lane < ncoil) cdot_acc(q, cv[lane], x[rows[lane]]);
    q = warp_sum(q);
    if (lane == 0) *mu = q;
}

// Several channels (evolution.m 'multichannel'): each channel's entries are
// summed separately; channel c's moment goes to mu[c * stride].  Kept out of
// line so the term loop's code stays the size of the one-channel case.
template <class Vec>
static __device__ __noinline__ void coil_moments(const Vec *x, int ncoil, const int *rows, const Vec *cv,
                                                 const int *chan, int nchan, int stride, int lane, Vec *mu) {
    Vec q = vzero<Vec>();
    if (lane < ncoil) cdot_acc(q, cv[lane], x[rows[lane]]);
    const int my = lane < ncoil ? chan[lane] : -1;
    for (int c = 0; c < nchan; ++c) {
        Vec qc = (my == c) ? q : vzero<Vec>();
        qc = warp_sum(qc);
        if (lane == 0) mu[c * stride] = qc;
    }
}

// Trajectory outputs with chunks of m steps (evolution.m 'trajectory'): the
// state j steps into a chunk is sum_k c_k(j) t_k, accumulated for j = 1..m-1
// as acc[(j-1) * stride] (+)= c[j-1] * t (c: term k's m-1 coefficients).  Out
// of line, so the term loop of the other runs keeps its size.
template <class Vec>
static __device__ __noinline__ void traj_accumulate(Vec *acc, int stride, const Vec *c, int m1, Vec t, bool init) {
    for (int j = 0; j < m1; ++j) {
        const Vec cj = c[j];
        Vec p;
        p.x = cj.x * t.x - cj.y * t.y;
        p.y = cj.x * t.y + cj.y * t.x;
        Vec &a = acc[(size_t)j * stride];
        if (init) {
            a = p;
        } else {
            a.x += p.x;
            a.y += p.y;
        }
    }
}

// ---------------------------------------------------------------------------
// The propagation kernel
// ---------------------------------------------------------------------------
// SC: the coil has at most 32 non-zeros (sys.ncoil > 0), read by one warp per
// term; the dense-coil projection is compiled out, which keeps the term loop
// small (6 % on c1).
// TRJ: trajectory outputs (the state at every step, run.traj_out); compiled
// into separate instantiations so that the other runs' term loop keeps its
// registers (the out-of-line accumulation calls cost c1 5 % when present).
// WIDE: up to 24 warps (80 registers a thread) instead of 16 (128); used with
// 2 rows per lane in FP32, where the rows' state fits (c1: 20 warps 60.2 ms,
// 16 warps with 3 rows per lane 63.8 ms per powder).  The minimum of one
// block per SM keeps ptxas from holding the 1- and 2-row kernels at 64
// registers with spills.
template <bool F64, bool CPLX, int RMAX, bool CLU, bool SC, bool TRJ, bool WIDE = false>
__global__ void __launch_bounds__(WIDE ? 768 : 512, 1)
powder_chebyshev_kernel(const DevSystem sys, const DevRun run) {
    using P = Prec<F64, CPLX>;
    using Vec = typename P::Vec;
    // cluster launches of FP32 real values keep each column in its value
    // (ValRP), which leaves room for larger systems per CTA
    constexpr bool PACKED = !F64 && !CPLX && CLU;
    constexpr bool FOLD = RMAX > 4 && !PACKED;     // see the FP32 term loop
    constexpr bool TPR64 = F64 && (RMAX > 4 || (CLU && RMAX == 4));   // see the FP64 term loop
    using Val = std::conditional_t<PACKED, ValRP, typename P::Val>;
    // units of a packed entry's low part before the rescale to L~ (exact:
    // lo_scale is a power of two)
    const float lo_unit = (float)(5.9604644775390625e-8 / sys.lo_scale);
    using Dg = typename P::Dg;
    using Real = typename P::Real;
    using Acc = typename P::Acc;
    using Af = typename P::Af;

    extern __shared__ __align__(16) unsigned char smem[];
    const SmemLayout<F64, CPLX> L(sys.n_pad, CLU ? run.nsl_loc : sys.nslices, CLU ? run.ell_loc : sys.ell_len,
                                  run.Kmax, run.M, blockDim.x, sys.nchan, TRJ ? run.traj_m : 1, PACKED);
    double *s_coef = reinterpret_cast<double *>(smem + L.coef);
    double *s_red = reinterpret_cast<double *>(smem + L.red);
    double *s_cred = reinterpret_cast<double *>(smem + L.cred);
    double *s_al = reinterpret_cast<double *>(smem + L.alpha);
    double *s_be = reinterpret_cast<double *>(smem + L.beta);
    int *s_soff = reinterpret_cast<int *>(smem + L.slice_off);
    uint16_t *s_col = reinterpret_cast<uint16_t *>(smem + L.ell_col);
    Val *s_val = reinterpret_cast<Val *>(smem + L.ell_val);
    Dg *s_diag = reinterpret_cast<Dg *>(smem + L.diag);
    Vec *s_xa = reinterpret_cast<Vec *>(smem + L.xa);
    Vec *s_xb = reinterpret_cast<Vec *>(smem + L.xb);
    Vec *s_part = reinterpret_cast<Vec *>(smem + L.part);
    Af *s_atau = reinterpret_cast<Af *>(smem + L.atau);
    Vec *s_mu = reinterpret_cast<Vec *>(smem + L.mu);
    Vec *s_phase = reinterpret_cast<Vec *>(smem + L.phase);
    Vec *s_rec = reinterpret_cast<Vec *>(smem + L.rec);
    Vec *s_tco = reinterpret_cast<Vec *>(smem + L.tco);      // trajectory: [k][j-1] coefficients
    Vec *s_tacc = reinterpret_cast<Vec *>(smem + L.tacc);    // trajectory: [j-1][local row] states
    __shared__ double s_scalar[8];
    __shared__ int s_int[4];
    __shared__ int s_crow[32];
    __shared__ Vec s_cval[32];
    __shared__ int s_cchan[32];
    constexpr bool scoil = SC;              // moments from the coil rows, no per-row projection

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nwarps = blockDim.x >> 5;
    const int n = sys.n;
    const int M = run.M;
    const int nsteps = run.nsteps;
    double *table = run.table + (size_t)blockIdx.x * run.Kmax * (M + 1);
    // This CTA's block of slices [sb, se): global rows row0 .. row0 + 32*nsl.
    const int CL = CLU ? run.cl : 1;
    const int crank = CLU ? cluster_rank() : 0;
    const int sb = CLU ? run.cl_slices[crank] : 0;
    const int se = CLU ? run.cl_slices[crank + 1] : sys.nslices;
    const int nsl = se - sb;
    const int row0 = sb * 32, nrow_loc = nsl * 32;
    const int eb = sys.slice_off[sb];
    const int ell_loc = sys.slice_off[se] - eb;
    int par = 0;              // cluster reduction buffer parity
    // Static pattern: copy once per CTA (offsets local, columns global).
    for (int i = tid; i <= nsl; i += blockDim.x) s_soff[i] = sys.slice_off[sb + i] - eb;
    if (scoil && tid < sys.ncoil) {
        s_crow[tid] = sys.coil_rows[tid];
        s_cval[tid] = tovec(sys.coil_vals[tid], Vec());
        s_cchan[tid] = sys.coil_chan ? sys.coil_chan[tid] : 0;
    }
    for (int e = tid; e < ell_loc; e += blockDim.x) {
        if constexpr (PACKED) s_val[e].col = sys.ell_col[eb + e];
        else s_col[e] = sys.ell_col[eb + e];
    }
    // Slices to warps, longest-processing-time first: slices are stored in
    // non-increasing width, each goes to the least-loaded warp with room, so a
    // warp's slices also come in non-increasing width.  Cost ~ width + 3, no
    // allowance for the detection moment the last warp folds every term (c1
    // on 20 warps: 60.0 ms per powder, 60.2 with a handicap of 6, 60.5 with
    // 12; c4: 194.8 ms against 198.1 with width + 5 and a handicap of 6).
    __shared__ short s_wsl[32 * 8];
    __shared__ int s_wcnt[32];
    __shared__ int s_wload[32];
    csync<CLU>();             // every CTA of the cluster has started before any remote access
    if (tid == 0) {
        for (int w = 0; w < nwarps; ++w) { s_wcnt[w] = 0; s_wload[w] = 0; }
        bool fits = true;
        for (int sl = 0; sl < nsl; ++sl) {
            const int cost = ((s_soff[sl + 1] - s_soff[sl]) >> 5) + 3;
            int best = -1;
            for (int w = 0; w < nwarps; ++w)
                if (s_wcnt[w] < RMAX && (best < 0 || s_wload[w] < s_wload[best])) best = w;
            if (best < 0) { fits = false; break; }
            s_wsl[best * RMAX + s_wcnt[best]] = (short)sl;
            ++s_wcnt[best];
            s_wload[best] += cost;
        }
        s_wload[0] = fits ? 1 : 0;          // reused as the "assignment fits" flag
    }
    __syncthreads();
    const bool assignment_ok = cluster_reduce<CLU, 2>(s_wload[0] != 0 ? 1.0 : 0.0, s_red, s_cred, par, crank, CL) > 0.5;
    const int rows_per_lane = s_wcnt[warp];

    // Each CTA (cluster) starts at its own index and then takes the next free
    // orientation from a global counter, since orientations differ in cost.
    __shared__ int s_next;
    for (int o = blockIdx.x / CL; o < run.n_orient;
         o = next_orientation<CLU>(run.next_orient, &s_next, (int)(gridDim.x / CL), crank)) {
        if (!assignment_ok) {                        // launch configuration error
            if (tid == 0 && crank == 0) run.status[o] = kDevTooManyRows;
            continue;
        }
        // ---- 1. rotational coefficients (FP64) --------------------------------
        __syncthreads();
        for (int t = tid; t < sys.nterms; t += blockDim.x) {
            double re, im;
            wigner_element(sys.term_rkm[3 * t], sys.term_rkm[3 * t + 1], sys.term_rkm[3 * t + 2],
                           run.alpha[o], run.beta[o], run.gamma[o], re, im);
            s_coef[1 + 2 * t] = re;
            s_coef[2 + 2 * t] = im;
        }
        if (tid == 0) s_coef[0] = 1.0;
        __syncthreads();

        // ---- 2. assemble L(Omega) in FP64, store in working precision ---------
        double gmax = -CUDART_INF, gmin = CUDART_INF;
        for (int e = tid; e < ell_loc; e += blockDim.x) {
            double re = 0.0, im = 0.0;
            for (int s = 0; s < sys.nstreams; ++s) {
                const double c = s_coef[sys.stream_coef[s]];
                re = fma(c, sys.ell_re[(size_t)s * sys.ell_len + eb + e], re);
                if (CPLX) im = fma(c, sys.ell_im[(size_t)s * sys.ell_len + eb + e], im);
            }
            if constexpr (PACKED) pack_rp(s_val[e], re, sys.lo_scale);
            else pack(s_val[e], re, im);
        }
        for (int i = tid; i < nrow_loc; i += blockDim.x) {
            double re = 0.0, im = 0.0;
            for (int s = 0; s < sys.nstreams; ++s) {
                const double c = s_coef[sys.stream_coef[s]];
                const double2 d = sys.diag[(size_t)s * sys.n_pad + row0 + i];
                re = fma(c, d.x, re);
                im = fma(c, d.y, im);
            }
            pack(s_diag[i], re, im);
        }
        __syncthreads();
        // Gershgorin interval of the Hermitian part (real diagonal + off-diagonal)
        for (int r = 0; r < rows_per_lane; ++r) {
            const int sl = s_wsl[warp * RMAX + r];
            const int lrow = sl * 32 + lane;
            if (row0 + lrow >= n) continue;
            const int off = s_soff[sl], w = (s_soff[sl + 1] - off) >> 5;
            double rad = 0.0;
            for (int c = 0; c < w; ++c) {
                const double2 v = value_of(s_val[off + c * 32 + lane], lo_unit);
                rad += CPLX ? sqrt(v.x * v.x + v.y * v.y) : fabs(v.x);
            }
            const double dr = unpack(s_diag[lrow]).x;
            gmax = fmax(gmax, dr + rad);
            gmin = fmin(gmin, dr - rad);
        }
        gmax = cluster_reduce<CLU, 1>(gmax, s_red, s_cred, par, crank, CL);
        gmin = cluster_reduce<CLU, 2>(gmin, s_red, s_cred, par, crank, CL);
        double imax = 0.0;
        for (int i = tid; i < nrow_loc && row0 + i < n; i += blockDim.x) imax = fmax(imax, fabs(unpack(s_diag[i]).y));
        imax = cluster_reduce<CLU, 1>(imax, s_red, s_cred, par, crank, CL);

        // ---- 3. Lanczos bounds on the Hermitian part ---------------------------
        // (in the working precision: the bounds are widened afterwards)
        Vec q_prev[RMAX], q_cur[RMAX];
        Real nrm2 = 0;
#pragma unroll
        for (int r = 0; r < RMAX; ++r) {
            const int row = (r < rows_per_lane) ? row0 + s_wsl[warp * RMAX + r] * 32 + lane : n;
            const bool own = row < n;
            // deterministic pseudo-random start vector in [0.63, 1.37]
            const Real v = own ? (Real)(1.0f + 0.37f * __sinf(1.7f * (float)(row % 4096) + 0.3f)) : (Real)0;
            q_cur[r].x = v;
            q_cur[r].y = 0;
            q_prev[r] = vzero<Vec>();
            nrm2 += v * v;
        }
        nrm2 = cluster_reduce<CLU, 0, Real>(nrm2, s_red, s_cred, par, crank, CL);
        {
            const Real inv = (Real)1 / sqrt(nrm2);
#pragma unroll
            for (int r = 0; r < RMAX; ++r) {
                if (r >= rows_per_lane) break;
                const int sl = s_wsl[warp * RMAX + r];
                q_cur[r].x *= inv; q_cur[r].y *= inv;
                s_xa[row0 + sl * 32 + lane] = q_cur[r];
                push_peers<CLU>(&s_xa[row0 + sl * 32 + lane], q_cur[r], crank, CL);
            }
        }
        int m_eff = 0;
        Real beta_prev = 0;
        const int lits = min(run.lanczos_its, min(kMaxLanczos, n));
        for (int j = 0; j < lits; ++j) {
            csync<CLU>();
            Vec wv[RMAX];
            Real alpha_p = 0;
#pragma unroll
            for (int r = 0; r < RMAX; ++r) {
                wv[r] = vzero<Vec>();
                if (r >= rows_per_lane) continue;
                const int sl = s_wsl[warp * RMAX + r];
                const int lrow = sl * 32 + lane;
                if (row0 + lrow >= n) continue;
                const int off = s_soff[sl], w = (s_soff[sl + 1] - off) >> 5;
                Vec y = vzero<Vec>();
                for (int c = 0; c < w; ++c) {
                    const int e = off + c * 32 + lane;
                    mac_u(y, s_val[e], s_xa[col_of(s_col, s_val, e)], lo_unit);
                }
                const Real dr = diag_re(s_diag[lrow]);
                y.x += dr * q_cur[r].x;
                y.y += dr * q_cur[r].y;
                y.x -= beta_prev * q_prev[r].x;
                y.y -= beta_prev * q_prev[r].y;
                wv[r] = y;
                alpha_p += q_cur[r].x * y.x + q_cur[r].y * y.y;
            }
            const Real alpha = cluster_reduce<CLU, 0, Real>(alpha_p, s_red, s_cred, par, crank, CL);
            Real b2 = 0;
#pragma unroll
            for (int r = 0; r < RMAX; ++r) {
                wv[r].x -= alpha * q_cur[r].x;
                wv[r].y -= alpha * q_cur[r].y;
                b2 += wv[r].x * wv[r].x + wv[r].y * wv[r].y;
            }
            const Real beta = sqrt(cluster_reduce<CLU, 0, Real>(b2, s_red, s_cred, par, crank, CL));
            if (tid == 0) { s_al[j] = (double)alpha; s_be[j] = (double)beta; }
            m_eff = j + 1;
            if (!(beta > (Real)1e-12 * (fabs(alpha) + (Real)1e-30))) break;   // invariant subspace
            const Real inv = (Real)1 / beta;
#pragma unroll
            for (int r = 0; r < RMAX; ++r) {
                q_prev[r] = q_cur[r];
                q_cur[r].x = wv[r].x * inv;
                q_cur[r].y = wv[r].y * inv;
                if (r < rows_per_lane) {
                    Vec *dstp = &s_xb[row0 + s_wsl[warp * RMAX + r] * 32 + lane];
                    *dstp = q_cur[r];
                    push_peers<CLU>(dstp, q_cur[r], crank, CL);
                }
            }
            Vec *t = s_xa; s_xa = s_xb; s_xb = t;
            beta_prev = beta;
        }
        __syncthreads();
        if (warp == 0) {
            double tlo, thi;
            tridiag_extremes_warp(s_al, s_be, m_eff, tlo, thi, lane);
            const double bl = fabs(s_be[m_eff - 1]);
            // Ritz vectors' last components: lane 0 for the top, lane 1 for the bottom
            double rr = 0.0;
            if (!run.safe_bounds && lane < 2) rr = bl * ritz_last_component(s_al, s_be, m_eff, lane == 0 ? thi : tlo);
            const double rhi = __shfl_sync(0xffffffffu, rr, 0), rlo = __shfl_sync(0xffffffffu, rr, 1);
          if (lane == 0) {
            double hi, lo;
            if (run.safe_bounds) {
                // the retry after a violated bound: Gershgorin discs (FP64), which
                // enclose the spectrum of the Hermitian part whatever Lanczos found
                hi = gmax;
                lo = gmin;
            } else {
                // Ritz value plus its residual |beta_m * y_m| and 2% of the width;
                // the propagation checks the norm and the host retries with the
                // safe bound if this was too tight
                const double wid = thi - tlo;
                hi = fmin(thi + rhi + 0.02 * wid, gmax);
                lo = fmax(tlo - rlo - 0.02 * wid, gmin);
            }
            if (!(hi >= lo)) { hi = gmax; lo = gmin; }
            const double width = hi - lo;
            const double scale = fmax(fabs(hi), fabs(lo));
            // the width must also cover the dissipative (imaginary) extent of L
            const double half = fmax(0.5 * width * 1.01 + 1e-9 * scale, imax) + 1e-30;
            s_scalar[0] = 0.5 * (hi + lo);   // centre c
            s_scalar[1] = half;              // half-width s
            // chunk length: about chunk_x series argument per chunk
            int Mo = M;
            if (!run.fixed_chunk) {
                const double target = run.chunk_x / (half * run.dt);
                Mo = (int)fmax(1.0, fmin((double)M, floor(target)));
            }
            Mo = min(Mo, nsteps + 1);
            s_int[2] = Mo;
            // series length for the chunk (x = s*Mo*dt) incl. growth from Im(L)
            const double x = half * Mo * run.dt;
            const double lg = 2.0 * imax / half;
            // bound first (Debye-type, loose for k ~ x), then the exact tail
            // from the Bessel column of the chunk end itself
            const int Kb = min(run.Kmax, max(2, series_terms(x, lg, run.tol, run.Kmax + 1)) + 2);
            bessel_column(table, Mo, Mo, Kb, half, run.dt);
            int K = 2;
            {
                // growth e^{k lg} of term k, stepped down from k = Kb-1 (one exp)
                double grow = exp((Kb - 1) * lg);
                const double shrink = exp(-lg);
                for (int k = Kb - 1; k >= 2; --k, grow *= shrink) {
                    if (fabs(table[(size_t)k * (Mo + 1) + Mo]) * grow > run.tol) { K = k + 1; break; }
                }
            }
            K = min(K + 2, Kb);
            if (Kb >= run.Kmax && series_terms(x, lg, run.tol, run.Kmax + 1) + 2 > run.Kmax && K >= Kb - 2) K = run.Kmax + 1;
            s_int[0] = K;
            s_int[1] = (K > run.Kmax) ? 1 : 0;
          }
        }
        csync<CLU>();
        // every CTA of a cluster takes rank 0's decisions, so their control flow
        // (and their cluster barriers) cannot diverge
        double cen = s_scalar[0], half = s_scalar[1];
        int K = s_int[0], Mo = s_int[2], too_small = s_int[1];
        if constexpr (CLU) {
            cen = ld_cluster_f64(cluster_addr(smem_u32(&s_scalar[0]), 0));
            half = ld_cluster_f64(cluster_addr(smem_u32(&s_scalar[1]), 0));
            K = ld_cluster_s32(cluster_addr(smem_u32(&s_int[0]), 0));
            too_small = ld_cluster_s32(cluster_addr(smem_u32(&s_int[1]), 0));
            Mo = ld_cluster_s32(cluster_addr(smem_u32(&s_int[2]), 0));
        }
        if (too_small) {
            if (tid == 0 && crank == 0) { run.status[o] = kDevTableTooSmall; run.kused[o] = K; run.halfwidth[o] = half; }
            continue;
        }

        // ---- 4. rescale to L~ = (L - c)/s -------------------------------------
        {
            const double inv = 1.0 / half;
            for (int e = tid; e < ell_loc; e += blockDim.x) {
                const double2 v = value_of(s_val[e], lo_unit);
                if constexpr (PACKED) pack_rp(s_val[e], v.x * inv, 1.0);      // L~ entries below 1
                else pack(s_val[e], v.x * inv, v.y * inv);
            }
            for (int i = tid; i < nrow_loc; i += blockDim.x) {
                const double2 d = unpack(s_diag[i]);
                pack(s_diag[i], (d.x - cen) * inv, d.y * inv);
            }
        }

        // ---- 5. Bessel table J_k(s j dt), j = 0..M --------------------------
        for (int j = tid; j < (CLU ? Mo + 1 : Mo); j += blockDim.x) bessel_column(table, Mo, j, K, half, run.dt);
        __syncthreads();
        // the last chunk only reaches j_last steps: its series can stop where the
        // Bessel column of j_last (times the growth from Im L) drops below tol
        const int nchunks = (nsteps + Mo) / Mo;      // ceil((nsteps+1)/Mo)
        if (warp == 0) {
            // one warp scans the column 32 terms at a time from the top
            const int j_last = nsteps - (nchunks - 1) * Mo;
            const double lg = 2.0 * imax / half;
            int kl = 2;
            for (int top = K - 1; top >= 2; top -= 32) {
                const int k = top - lane;
                const bool sig = k >= 2 && fabs(table[(size_t)k * (Mo + 1) + j_last]) * exp(k * lg) > run.tol;
                const unsigned m = __ballot_sync(0xffffffffu, sig);
                if (m) { kl = top - (__ffs(m) - 1) + 1; break; }
            }
            if (lane == 0) s_int[3] = min(K, kl + 2);
        }
        // series coefficients of one chunk (tau = M dt), centre phase folded in
        {
            const double tau = Mo * run.dt;
            const double pr = cos(-cen * tau), pi_ = sin(-cen * tau);
            for (int k = tid; k < K; k += blockDim.x) {
                const double jv = table[(size_t)k * (Mo + 1) + Mo];
                // (-i)^k * e^{-i c tau} * jv   (factor 2 for k>0 is already in the table)
                double re, im;
                switch (k & 3) {
                    case 0: re = pr; im = pi_; break;
                    case 1: re = pi_; im = -pr; break;
                    case 2: re = -pr; im = -pi_; break;
                    default: re = -pi_; im = pr; break;
                }
                pack(s_atau[k], re * jv, im * jv);
            }
            for (int j = tid; j < Mo; j += blockDim.x) {
                const double ph = -cen * j * run.dt;
                s_phase[j] = tovec(make_double2(cos(ph), sin(ph)), Vec());
            }
        }
        // trajectory outputs: coefficients of the states 1 .. Mo-1 steps into a chunk
        const int TM1 = TRJ ? Mo - 1 : 0;
        for (int q = tid; q < TM1 * K; q += blockDim.x) {
            const int k = q / TM1, j = 1 + q % TM1;
            const double tau = j * run.dt;
            const double pr = cos(-cen * tau), pi_ = sin(-cen * tau);
            const double jv = table[(size_t)k * (Mo + 1) + j];
            double re, im;
            switch (k & 3) {
                case 0: re = pr; im = pi_; break;
                case 1: re = pi_; im = -pr; break;
                case 2: re = -pr; im = -pi_; break;
                default: re = -pi_; im = pr; break;
            }
            s_tco[q] = tovec(make_double2(re * jv, im * jv), Vec());
        }
        csync<CLU>();             // coefficients and phases visible before the first term
        int K_last = s_int[3];
        if constexpr (CLU) K_last = ld_cluster_s32(cluster_addr(smem_u32(&s_int[3]), 0));

        // ---- 6. chunked Chebyshev propagation with fused coil projection -------
        // Each lane owns up to RMAX rows (one per 32-row slice of its warp); the
        // rows advance together, entry index outer and rows inner, so their
        // accumulations are independent dependency chains.  A lane's slices come
        // in non-increasing width, so entry c is shared by rows 0..seg-1 while
        // c < width of row seg-1: each segment runs with a compile-time row count.
        // With 6 rows per lane a row (below 2^16: columns are uint16) and its
        // ELL width share a register.
        [[maybe_unused]] int r_rw[RMAX], r_rowv[RMAX], r_wv[RMAX];
        int r_off[RMAX];
        int nr = 0;
#pragma unroll
        for (int r = 0; r < RMAX; ++r) {
            r_rw[r] = 0; r_rowv[r] = 0; r_wv[r] = 0; r_off[r] = 0;
            if (r < rows_per_lane) {
                const int sl = s_wsl[warp * RMAX + r];
                nr = r + 1;
                const int row = row0 + sl * 32 + lane, w = (s_soff[sl + 1] - s_soff[sl]) >> 5;
                if constexpr (FOLD) r_rw[r] = row | (w << 16);
                else { r_rowv[r] = row; r_wv[r] = w; }
                r_off[r] = s_soff[sl] + lane;
            }
        }
        auto r_row = [&](int r) { if constexpr (FOLD) return r_rw[r] & 0xffff; else return r_rowv[r]; };
        auto r_w = [&](int r) { if constexpr (FOLD) return (int)((unsigned)r_rw[r] >> 16); else return r_wv[r]; };
        Vec *fid_out = reinterpret_cast<Vec *>(run.fids) + (size_t)o * sys.nchan * (nsteps + 1);
        int status = kDevOk;
        [[maybe_unused]] Vec t_prev[RMAX], t_cur[RMAX], acc[RMAX], cc[RMAX];
        [[maybe_unused]] f2x tp[RMAX], tc[RMAX], ac[RMAX], cp[RMAX], crr[RMAX], cim[RMAX];
#pragma unroll
        for (int r = 0; r < RMAX; ++r) {
            const double2 x0 = r >= nr ? make_double2(0.0, 0.0)
                               : sys.rho0s ? sys.rho0s[(size_t)o * sys.n_pad + r_row(r)] : sys.rho0[r_row(r)];
            const double2 c0 = r < nr ? sys.coil[r_row(r)] : make_double2(0.0, 0.0);
            if constexpr (F64) {
                t_prev[r] = vzero<Vec>(); acc[r] = vzero<Vec>();
                t_cur[r] = tovec(x0, Vec());
                cc[r] = tovec(c0, Vec());
            } else {
                tp[r] = 0ull; ac[r] = 0ull; cp[r] = 0ull;
                tc[r] = f2pk((float)x0.x, (float)x0.y);
                // conj(c) * t = (cr tr + ci ti, cr ti - ci tr) = crr*t + cim*swap(t)
                crr[r] = f2pk((float)c0.x, (float)c0.x);
                cim[r] = f2pk((float)c0.y, -(float)c0.y);
            }
        }
        long long mv = 0;
        for (int a = 0; a < nchunks && status == kDevOk; ++a) {
            const bool last = (a + 1 == nchunks);
            // the last chunk also propagates the state when the caller wants it
            // (pulse sequences continue from it): its coefficients are those of
            // its own length j_last, from the same Bessel table
            const bool advance = !last || run.state_out != nullptr;
            const int Kc = last ? K_last : K;              // terms of this chunk
            if (TRJ) {
                // trajectory output ('trajectory' of evolution.m): the state entering chunk a
                double2 *tr = run.traj_out + ((size_t)o * (nsteps + 1) + (size_t)a * Mo) * sys.n_pad;
#pragma unroll
                for (int r = 0; r < RMAX; ++r) {
                    if (r < nr) {
                        double2 v;
                        if constexpr (F64) v = tod(t_cur[r]);
                        else v = tod(f2up(tc[r]));
                        tr[r_row(r)] = v;
                    }
                }
            }
            mv += Kc - 1;
            if (last && run.state_out && nchunks > 0) {
                const int j_last = nsteps - (nchunks - 1) * Mo;
                const double tau = j_last * run.dt;
                const double pr = cos(-cen * tau), pi_ = sin(-cen * tau);
                csync<CLU>();                              // the previous chunk's reads of the coefficients are done
                for (int k = tid; k < Kc; k += blockDim.x) {
                    const double jv = table[(size_t)k * (Mo + 1) + j_last];
                    double re, im;
                    switch (k & 3) {
                        case 0: re = pr; im = pi_; break;
                        case 1: re = pi_; im = -pr; break;
                        case 2: re = -pr; im = -pi_; break;
                        default: re = -pi_; im = pr; break;
                    }
                    pack(s_atau[k], re * jv, im * jv);
                }
                csync<CLU>();
            }
            double start_n2 = 0.0, end_n2 = 0.0;
            if constexpr (F64) {
                // k = 0: t0 = rho
                Vec mom = vzero<Vec>();
#pragma unroll
                for (int r = 0; r < RMAX; ++r) {
                    if (r < nr) {
                        s_xa[r_row(r)] = t_cur[r];
                        push_peers<CLU>(&s_xa[r_row(r)], t_cur[r], crank, CL);
                        if (!scoil) cdot_acc(mom, cc[r], t_cur[r]);
                        acc[r] = vzero<Vec>();
                        acc_add64(acc[r], s_atau[0], t_cur[r]);
                        if (TRJ && TM1 > 0) traj_accumulate(s_tacc + (r_row(r) - row0), nrow_loc, s_tco, TM1, t_cur[r], true);
                        start_n2 += t_cur[r].x * t_cur[r].x + t_cur[r].y * t_cur[r].y;
                        t_prev[r] = vzero<Vec>();
                    }
                }
                if (!scoil) {
                    mom = warp_sum(mom);
                    if (lane == 0) s_part[warp] = mom;
                }
                csync<CLU>();
                // k = 1 .. K-1: t_k = (k==1 ? 1 : 2) L~ t_{k-1} - t_{k-2}
                for (int k = 1; k < Kc; ++k) {
                    const Vec *src = (k & 1) ? s_xa : s_xb;
                    Vec *dst = (k & 1) ? s_xb : s_xa;
                    const Real two = (k == 1) ? (Real)1 : (Real)2;
                    // the last warp folds term k-1's partials while the others start term k;
                    // slot (k-1)&1 is rewritten only in term k+1, after the next barrier
                    if (warp == nwarps - 1) {
                        if (sys.nchan > 1) coil_moments(src, sys.ncoil, s_crow, s_cval, s_cchan, sys.nchan, run.Kmax, lane, &s_mu[k - 1]);
                        else if (scoil) coil_moment(src, sys.ncoil, s_crow, s_cval, lane, &s_mu[k - 1]);
                        else reduce_term(s_part + ((k - 1) & 1) * nwarps, nwarps, lane, &s_mu[k - 1]);
                    }
                    Acc y[RMAX];
#pragma unroll
                    for (int r = 0; r < RMAX; ++r) {
                        y[r] = vzero<Vec>();
                        if (r < nr) cmac(y[r], s_diag[r_row(r) - row0], t_cur[r]);
                    }
                    int c = 0;
#pragma unroll
                    for (int seg = RMAX; seg >= 1; --seg) {
                        if (seg <= nr) {
                            const int cend = r_w(seg - 1);
                            for (; c < cend; ++c) {
#pragma unroll
                                for (int r = 0; r < seg; ++r) {
                                    const int e = r_off[r] + c * 32;
                                    cmac(y[r], s_val[e], src[s_col[e]]);
                                }
                            }
                        }
                    }
                    mom = vzero<Vec>();
#pragma unroll
                    for (int r = 0; r < RMAX; ++r) {
                        if (r < nr) {
                            // t_{k-2}: with 6 rows per lane, or 4 on a cluster, read back
                            // from the buffer this term overwrites (its own row, written two
                            // terms earlier), which keeps the FP64 rows' state in registers
                            // (c4 FP64 on 2-CTA clusters: no spills, 1238 ms per powder
                            // against 1263; on one CTA with 4 rows the reload costs 0.5 %)
                            Vec tpv;
                            if constexpr (TPR64) tpv = (k == 1) ? vzero<Vec>() : dst[r_row(r)];
                            else tpv = t_prev[r];
                            const Vec tn = recur(y[r], two, tpv);
                            if constexpr (!TPR64) t_prev[r] = t_cur[r];
                            t_cur[r] = tn;
                            dst[r_row(r)] = tn;
                            push_peers<CLU>(&dst[r_row(r)], tn, crank, CL);
                            if (!scoil) cdot_acc(mom, cc[r], tn);
                            if (advance) acc_add64(acc[r], s_atau[k], tn);
                            if (TRJ && TM1 > 0) traj_accumulate(s_tacc + (r_row(r) - row0), nrow_loc, s_tco + k * TM1, TM1, tn, false);
                        }
                    }
                    if (!scoil) {
                        mom = warp_sum(mom);
                        if (lane == 0) s_part[(k & 1) * nwarps + warp] = mom;
                    }
                    csync<CLU>();
                }
#pragma unroll
                for (int r = 0; r < RMAX; ++r) {
                    if (r < nr) {
                        if (advance) t_cur[r] = acc[r];
                        end_n2 += t_cur[r].x * t_cur[r].x + t_cur[r].y * t_cur[r].y;
                    }
                }
            } else {
                // ---- FP32: packed (re, im) pairs, compensated row sums ----
                // Row sums are Kahan-compensated: Y the running sum, Lw its lost
                // low-order part, Lp the products of the values' low parts (with
                // 6 rows per lane folded into Lw); the row value Y + Lw + Lp is
                // rounded once.
                const f2x TWO = f2pk(2.f, 2.f), ONE = f2pk(1.f, 1.f);
                f2x MOM = 0ull;
#pragma unroll
                for (int r = 0; r < RMAX; ++r) {
                    if (r < nr) {
                        const f2x T = tc[r];
                        reinterpret_cast<f2x *>(s_xa)[r_row(r)] = T;
                        push_peers<CLU>(reinterpret_cast<f2x *>(s_xa) + r_row(r), T, crank, CL);
                        if (!scoil) {
                            MOM = fma2(crr[r], T, MOM);
                            MOM = fma2(cim[r], swap2(T), MOM);
                        }
                        ac[r] = cmul_pk(s_atau[0], T);
                        if (TRJ && TM1 > 0) traj_accumulate(s_tacc + (r_row(r) - row0), nrow_loc, s_tco, TM1, f2up(T), true);
                        cp[r] = 0ull;
                        tp[r] = 0ull;
                        const float2 t = f2up(T);
                        start_n2 += (double)t.x * t.x + (double)t.y * t.y;
                    }
                }
                if (!scoil) {
                    float2 m = warp_sum(f2up(MOM));
                    if (lane == 0) s_part[warp] = m;
                }
                csync<CLU>();
                for (int k = 1; k < Kc; ++k) {
                    const f2x *src = reinterpret_cast<const f2x *>((k & 1) ? s_xa : s_xb);
                    f2x *dst = reinterpret_cast<f2x *>((k & 1) ? s_xb : s_xa);
                    const f2x TW = (k == 1) ? ONE : TWO;
                    if (warp == nwarps - 1) {
                        // moment of term k-1, whose vector is this term's source
                        if (sys.nchan > 1)
                            coil_moments(reinterpret_cast<const Vec *>(src), sys.ncoil, s_crow, s_cval, s_cchan, sys.nchan,
                                         run.Kmax, lane, &s_mu[k - 1]);
                        else if (scoil) coil_moment(reinterpret_cast<const Vec *>(src), sys.ncoil, s_crow, s_cval, lane, &s_mu[k - 1]);
                        else reduce_term(s_part + ((k - 1) & 1) * nwarps, nwarps, lane, &s_mu[k - 1]);
                    }
                    // Y + Lw + Lp is a row's sum: Y the running sum, Lw its
                    // compensated low-order part, Lp the products of the values'
                    // low parts (packed values: in units of 2^-24).  With 6 or 8
                    // rows per lane those products go into Lw instead: one
                    // accumulator per row fewer keeps the rows' state in
                    // registers (c4: 195 ms per powder against 323 with spills),
                    // at the cost of a longer dependency chain per entry (c1 4 %
                    // slower, so fewer rows keep Lp).
                    f2x Y[RMAX], Lw[RMAX];
                    [[maybe_unused]] f2x Lp[RMAX];
#pragma unroll
                    for (int r = 0; r < RMAX; ++r) {
                        Y[r] = 0ull;
                        Lw[r] = 0ull;
                        if constexpr (!FOLD) Lp[r] = 0ull;
                        if (r < nr) {
                            const DgS d = s_diag[r_row(r) - row0];
                            const f2x X = tc[r];
                            Y[r] = mul2(f2pk(d.rh, d.rh), X);
                            // the relaxation (imaginary) part of the diagonal goes into
                            // the low-order sum, without a compensation step of its own
                            Lw[r] = fma2(f2pk(-d.im, d.im), swap2(X), Lw[r]);
                            if constexpr (FOLD) {
                                Lw[r] = fma2(f2pk(d.rl, d.rl), X, Lw[r]);
                            } else {
                                const float dl = PACKED ? d.rl * 16777216.f : d.rl;
                                Lp[r] = mul2(f2pk(dl, dl), X);
                            }
                        }
                    }
                    int c = 0;
#pragma unroll
                    for (int seg = RMAX; seg >= 1; --seg) {
                        if (seg <= nr) {
                            const int cend = r_w(seg - 1);
                            for (; c < cend; ++c) {
#pragma unroll
                                for (int r = 0; r < seg; ++r) {
                                    const int e = r_off[r] + c * 32;
                                    const f2x X = src[col_of(s_col, s_val, e)];
                                    if constexpr (CPLX) {
                                        const ValC v = s_val[e];
                                        const f2x XS = swap2(X);
                                        kahan_add2l(Y[r], Lw[r], mul2(f2pk(v.rh, v.rh), X));
                                        kahan_add2l(Y[r], Lw[r], mul2(f2pk(-v.ih, v.ih), XS));
                                        f2x &Ls = FOLD ? Lw[r] : Lp[r];
                                        Ls = fma2(f2pk(v.rl, v.rl), X, Ls);
                                        Ls = fma2(f2pk(-v.il, v.il), XS, Ls);
                                    } else {
                                        const Val v = s_val[e];
                                        kahan_add2l(Y[r], Lw[r], mul2(f2pk(v.hi, v.hi), X));
                                        float lo;
                                        if constexpr (PACKED) lo = __half2float(v.lo);
                                        else lo = v.lo;
                                        f2x &Ls = FOLD ? Lw[r] : Lp[r];
                                        Ls = fma2(f2pk(lo, lo), X, Ls);
                                    }
                                }
                            }
                        }
                    }
                    MOM = 0ull;
#pragma unroll
                    for (int r = 0; r < RMAX; ++r) {
                        if (r < nr) {
                            // t_k = TW * (Y + Lw) - t_{k-2}
                            f2x Lr = Lw[r];
                            if constexpr (PACKED) Lr = fma2(Lp[r], f2pk(5.9604644775390625e-8f, 5.9604644775390625e-8f), Lr);
                            else if constexpr (!FOLD) Lr = add2(Lp[r], Lr);
                            // t_{k-2} of this row: in a register, or (6 rows per
                            // lane) read back from the buffer term k overwrites
                            f2x TP;
                            if constexpr (FOLD) TP = (k == 1) ? 0ull : dst[r_row(r)];
                            else TP = tp[r];
                            const f2x T = sub2(fma2(TW, Y[r], mul2(TW, Lr)), TP);
                            if constexpr (!FOLD) tp[r] = tc[r];
                            tc[r] = T;
                            dst[r_row(r)] = T;
                            push_peers<CLU>(dst + r_row(r), T, crank, CL);
                            if (!scoil) {
                                MOM = fma2(crr[r], T, MOM);
                                MOM = fma2(cim[r], swap2(T), MOM);
                            }
                            if (advance) {
                                // Kahan-compensated chunk-end sum acc += a_k t_k
                                const f2x Yk = sub2(cmul_pk(s_atau[k], T), cp[r]);
                                const f2x S = add2(ac[r], Yk);
                                cp[r] = sub2(sub2(S, ac[r]), Yk);
                                ac[r] = S;
                            }
                            if (TRJ && TM1 > 0)
                                traj_accumulate(s_tacc + (r_row(r) - row0), nrow_loc, s_tco + k * TM1, TM1, f2up(T), false);
                        }
                    }
                    if (!scoil) {
                        float2 m = warp_sum(f2up(MOM));
                        if (lane == 0) s_part[(k & 1) * nwarps + warp] = m;
                    }
                    csync<CLU>();
                }
#pragma unroll
                for (int r = 0; r < RMAX; ++r) {
                    if (r < nr) {
                        if (advance) tc[r] = ac[r];
                        const float2 t = f2up(tc[r]);
                        end_n2 += (double)t.x * t.x + (double)t.y * t.y;
                    }
                }
            }
            if (TRJ && TM1 > 0) {
                // the states 1 .. Mo-1 steps into this chunk (up to the last step)
                const int jn = min(TM1, nsteps - a * Mo);
#pragma unroll
                for (int r = 0; r < RMAX; ++r) {
                    if (r < nr) {
                        for (int j = 1; j <= jn; ++j) {
                            const Vec v = s_tacc[(size_t)(j - 1) * nrow_loc + (r_row(r) - row0)];
                            run.traj_out[((size_t)o * (nsteps + 1) + (size_t)a * Mo + j) * sys.n_pad + r_row(r)] =
                                make_double2((double)v.x, (double)v.y);
                        }
                    }
                }
            }
            // moment of the last term (the others were folded inside the loop)
            if (warp == nwarps - 1) {
                if (sys.nchan > 1)
                    coil_moments(((Kc - 1) & 1) ? s_xb : s_xa, sys.ncoil, s_crow, s_cval, s_cchan, sys.nchan, run.Kmax, lane,
                                 &s_mu[Kc - 1]);
                else if (scoil) coil_moment(((Kc - 1) & 1) ? s_xb : s_xa, sys.ncoil, s_crow, s_cval, lane, &s_mu[Kc - 1]);
                else reduce_term(s_part + ((Kc - 1) & 1) * nwarps, nwarps, lane, &s_mu[Kc - 1]);
            }
            if (CLU && !scoil) {
                // rank 0 adds the peers' partial moments in rank order; the peers
                // rewrite theirs only after the next cluster barrier, which rank 0
                // reaches after this read
                csync<CLU>();
                if (crank == 0) {
                    for (int k = tid; k < Kc; k += blockDim.x) {
                        Vec v = s_mu[k];
                        for (int j = 1; j < CL; ++j) {
                            const uint32_t a = cluster_addr(smem_u32(&s_mu[k]), j);
                            if constexpr (F64) {
                                v.x += ld_cluster_f64(a);
                                v.y += ld_cluster_f64(a + 8);
                            } else {
                                float fx, fy;
                                asm volatile("ld.shared::cluster.v2.f32 {%0, %1}, [%2];" : "=f"(fx), "=f"(fy) : "r"(a) : "memory");
                                v.x += fx;
                                v.y += fy;
                            }
                        }
                        s_mu[k] = v;
                    }
                }
            }
            __syncthreads();
            // FID points of this chunk: f_j = ph_j * sum_k J_k(s j dt) (-i)^k mu_k
            if (!CLU || crank == 0) {
              // the moments turned by (-i)^k, in place (nothing reads them after)
              for (int q = tid; q < Kc * sys.nchan; q += blockDim.x) {
                  const int k = q % Kc;
                  Vec &m = s_mu[(q / Kc) * run.Kmax + k];
                  const Vec mu = m;
                  switch (k & 3) {
                      case 1: m.x = mu.y; m.y = -mu.x; break;
                      case 2: m.x = -mu.x; m.y = -mu.y; break;
                      case 3: m.x = -mu.y; m.y = mu.x; break;
                      default: break;
                  }
              }
              __syncthreads();
              for (int ch = 0; ch < sys.nchan; ++ch) {
                const Vec *mu_c = s_mu + ch * run.Kmax;
                Vec *out_c = fid_out + (size_t)ch * (nsteps + 1);
                if (ch > 0) __syncthreads();         // s_rec reused per channel
                const int parts = max(1, (int)blockDim.x / Mo);
                const int kper = (Kc + parts - 1) / parts;
                const size_t ld = (size_t)(Mo + 1);
                for (int jj = tid; jj < Mo * parts; jj += blockDim.x) {
                    const int j = jj % Mo, pidx = jj / Mo;
                    const int k0 = pidx * kper, k1 = min(Kc, k0 + kper);
                    // the Bessel table sits in global memory (L2): four
                    // independent loads per step keep its latency off the
                    // critical path, two accumulators the adds
                    const double *tcol = table + j;
                    Vec f = vzero<Vec>(), g = vzero<Vec>();
                    int k = k0;
                    for (; k + 4 <= k1; k += 4) {
                        const Real j0 = (Real)tcol[(size_t)k * ld], j1 = (Real)tcol[(size_t)(k + 1) * ld];
                        const Real j2 = (Real)tcol[(size_t)(k + 2) * ld], j3 = (Real)tcol[(size_t)(k + 3) * ld];
                        const Vec m0 = mu_c[k], m1 = mu_c[k + 1], m2 = mu_c[k + 2], m3 = mu_c[k + 3];
                        f.x += j0 * m0.x; f.y += j0 * m0.y;
                        g.x += j1 * m1.x; g.y += j1 * m1.y;
                        f.x += j2 * m2.x; f.y += j2 * m2.y;
                        g.x += j3 * m3.x; g.y += j3 * m3.y;
                    }
                    for (; k < k1; ++k) {
                        const Real jv = (Real)tcol[(size_t)k * ld];
                        f.x += jv * mu_c[k].x;
                        f.y += jv * mu_c[k].y;
                    }
                    f.x += g.x;
                    f.y += g.y;
                    s_rec[jj] = f;
                }
                __syncthreads();
                for (int j = tid; j < Mo; j += blockDim.x) {
                    Vec f = vzero<Vec>();
                    for (int pidx = 0; pidx < parts; ++pidx) {
                        const Vec g = s_rec[pidx * Mo + j];
                        f.x += g.x; f.y += g.y;
                    }
                    const Vec ph = s_phase[j];
                    Vec out;
                    out.x = ph.x * f.x - ph.y * f.y;
                    out.y = ph.x * f.y + ph.y * f.x;
                    const int nidx = a * Mo + j;
                    if (nidx <= nsteps) out_c[nidx] = out;
                }
              }
            }
            // guard against a violated spectral bound (the series would then
            // grow; a dissipative L can only shrink the state)
            end_n2 = cluster_reduce<CLU, 0>(end_n2, s_red, s_cred, par, crank, CL);
            start_n2 = cluster_reduce<CLU, 0>(start_n2, s_red, s_cred, par, crank, CL);
            if (!isfinite(end_n2)) status = kDevNonFinite;
            else if (end_n2 > 16.0 * start_n2 + 1e-300) status = kDevDiverged;
        }
        if (run.state_out) {
            // the state at the last step, each CTA its own rows
#pragma unroll
            for (int r = 0; r < RMAX; ++r) {
                if (r < nr) {
                    double2 v;
                    if constexpr (F64) v = tod(t_cur[r]);
                    else v = tod(f2up(tc[r]));
                    run.state_out[(size_t)o * sys.n_pad + r_row(r)] = v;
                }
            }
        }
        if (tid == 0 && crank == 0) {
            run.status[o] = status;
            run.kused[o] = K;
            run.mused[o] = Mo;
            run.halfwidth[o] = half;
            run.matvecs[o] = mv;
        }
        csync<CLU>();
    }
    csync<CLU>();             // no CTA leaves while a peer may still read its shared memory
}

// ---------------------------------------------------------------------------
// Weighted powder sum (kernel/contexts/powder.m:280-287) in FP64.
// Deterministic: each output point sums its orientations in grid order,
// split into fixed groups that are combined in fixed order.
// ---------------------------------------------------------------------------
template <class Vec>
__global__ void powder_partial_kernel(const Vec *__restrict__ fids, const double *__restrict__ w,
                                      int n_orient, int npts, int group, double2 *__restrict__ part) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int g = blockIdx.y;
    if (t >= npts) return;
    const int o0 = g * group, o1 = min(n_orient, o0 + group);
    double2 s = make_double2(0.0, 0.0);
    for (int o = o0; o < o1; ++o) {
        const double2 v = tod(fids[(size_t)o * npts + t]);
        s.x = fma(w[o], v.x, s.x);
        s.y = fma(w[o], v.y, s.y);
    }
    part[(size_t)g * npts + t] = s;
}

static __global__ void powder_combine_kernel(const double2 *__restrict__ part, int ngroups, int npts,
                                      double2 *__restrict__ out) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= npts) return;
    double2 s = make_double2(0.0, 0.0);
    for (int g = 0; g < ngroups; ++g) {
        const double2 v = part[(size_t)g * npts + t];
        s.x += v.x; s.y += v.y;
    }
    out[t] = s;
}

}  // namespace spx
