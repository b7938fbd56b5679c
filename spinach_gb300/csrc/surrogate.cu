// Orientation surrogate for the powder FID: a small MLP over real spherical
// harmonics of the orientation (beta, gamma) that predicts the coefficients of
// an orientation's FID in an SVD basis.  Training and inference run on the GPU
// in the kernels below (split-TF32 tensor-core products with FP32 accumulation
// and BF16 weights, GELU, Adam); one training step is captured once in a CUDA
// graph and replayed.
//
// Features follow kernel/utilities/spher_harmon.m (orthonormal Y_lm with the
// Condon-Shortley phase): for each l, Re Y_l0, then Re Y_lm and Im Y_lm for
// m = 1..l, (lmax+1)^2 real numbers per orientation.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <new>
#include <random>
#include <stdexcept>
#include <string>
#include <vector>

#include "spinach_gpu.h"

namespace {

struct SurErr : std::runtime_error {
    spx_status code;
    SurErr(spx_status c, const std::string &m) : std::runtime_error(m), code(c) {}
};

#define SUR_CUDA(call)                                                                              \
    do {                                                                                            \
        cudaError_t e_ = (call);                                                                    \
        if (e_ != cudaSuccess)                                                                      \
            throw SurErr(e_ == cudaErrorMemoryAllocation ? SPX_ERR_OUT_OF_MEMORY : SPX_ERR_CUDA,    \
                         std::string(#call) + ": " + cudaGetErrorString(e_));                      \
    } while (0)

constexpr int kMaxL = 16;
constexpr int kSplitRows = 256;   // samples per split-K slab of the weight gradients
constexpr int kMaxSplits = 32;

// ---------------------------------------------------------------------------
// Spherical-harmonic features
// ---------------------------------------------------------------------------
__global__ void sh_features_kernel(int64_t n, const double *__restrict__ beta, const double *__restrict__ gamma,
                                   int lmax, int nfeat, float *__restrict__ X) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double x = cos(beta[i]), st = sin(beta[i]), g = gamma[i];
    // orthonormal associated Legendre functions p_lm(x), Condon-Shortley phase included
    double pmm = 0.28209479177387814;   // sqrt(1/(4 pi))
    float *out = X + i * nfeat;
    double pm[kMaxL + 1][kMaxL + 1];
    for (int m = 0; m <= lmax; ++m) {
        if (m > 0) pmm = -sqrt((2.0 * m + 1.0) / (2.0 * m)) * st * pmm;
        pm[m][m] = pmm;
        if (m + 1 <= lmax) pm[m + 1][m] = sqrt(2.0 * m + 3.0) * x * pmm;
        for (int l = m + 2; l <= lmax; ++l) {
            const double a = sqrt((4.0 * l * l - 1.0) / ((double)l * l - (double)m * m));
            const double b = sqrt(((l - 1.0) * (l - 1.0) - (double)m * m) / (4.0 * (l - 1.0) * (l - 1.0) - 1.0));
            pm[l][m] = a * (x * pm[l - 1][m] - b * pm[l - 2][m]);
        }
    }
    int f = 0;
    for (int l = 0; l <= lmax; ++l) {
        out[f++] = (float)pm[l][0];
        for (int m = 1; m <= l; ++m) {
            double s, c;
            sincos(m * g, &s, &c);
            // spher_harmon.m: Y_lm = p_lm e^{i m gamma} (m > 0)
            out[f++] = (float)(pm[l][m] * c);
            out[f++] = (float)(pm[l][m] * s);
        }
    }
}

// ---------------------------------------------------------------------------
// C[i,j] (+)= sum_k A(i,k) B(k,j) on the tensor cores with FP32 accumulation.
// A(i,k) = TA ? A[k*lda+i] : A[i*lda+k];  B(k,j) = TB ? B[j*ldb+k] : B[k*ldb+j].
// Operands are split into TF32 pairs (x = hi + lo, each TF32, 22 significant
// bits together) and the products hi*hi + lo*hi (+ hi*lo for an FP32 B) run as
// mma.sync m16n8k8 TF32 instructions: FP32-level accuracy from the tensor
// pipe.  A BF16 B (the weights) is exact in TF32 and is not split.  64x64
// tiles, 16-deep slabs staged in shared memory (rows padded to 20 floats, so
// the fragment reads are conflict-free), four warps of 32x32; gridDim.z
// splits K into slabs that write their own copies of C.
// ---------------------------------------------------------------------------
__device__ __forceinline__ float tof(float v) { return v; }
__device__ __forceinline__ float tof(__nv_bfloat16 v) { return __bfloat162float(v); }

__device__ __forceinline__ uint32_t tf32_rna(float x) {
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
    return r;
}
__device__ __forceinline__ void split_tf32(float x, uint32_t &hi, uint32_t &lo) {
    hi = tf32_rna(x);
    lo = tf32_rna(x - __uint_as_float(hi));
}
__device__ __forceinline__ void mma_tf32(float (&d)[4], const uint32_t (&a)[4], const uint32_t (&b)[2]) {
    asm volatile(
        "mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 {%0, %1, %2, %3}, {%4, %5, %6, %7}, {%8, %9}, "
        "{%0, %1, %2, %3};"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

template <class T> struct IsF32 { static constexpr bool value = false; };
template <> struct IsF32<float> { static constexpr bool value = true; };

template <bool TA, bool TB, class BT>
__global__ void __launch_bounds__(128) gemm_kernel(int M, int N, int K, const float *__restrict__ A, int lda,
                                                   const BT *__restrict__ B, int ldb, float *__restrict__ C,
                                                   int ldc, int accumulate) {
    constexpr bool kSplitB = IsF32<BT>::value;
    __shared__ float As[64][20];     // [row of A][k]
    __shared__ float Bs[64][20];     // [column of B][k]
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int g = lane >> 2, t = lane & 3;                   // fragment row group and thread in group
    const int wm = (warp >> 1) * 32, wn = (warp & 1) * 32;
    const int i0 = blockIdx.y * 64, j0 = blockIdx.x * 64;
    // split-K: slab z covers k in [kb, ke) and writes its own copy of C
    const int kchunk = (((K + gridDim.z - 1) / gridDim.z) + 15) & ~15;
    const int kb = blockIdx.z * kchunk, ke = min(K, kb + kchunk);
    C += (int64_t)blockIdx.z * M * ldc;
    float acc[2][4][4] = {};
    for (int k0 = kb; k0 < ke; k0 += 16) {
        for (int q = threadIdx.x; q < 64 * 16; q += 128) {
            // consecutive threads follow the contiguous global index
            const int ai = TA ? q % 64 : q / 16, ak = TA ? q / 64 : q % 16;
            const int i = i0 + ai, k = k0 + ak;
            As[ai][ak] = (i < M && k < ke) ? (TA ? A[(int64_t)k * lda + i] : A[(int64_t)i * lda + k]) : 0.f;
            const int bj = TB ? q / 16 : q % 64, bk = TB ? q % 16 : q / 64;
            const int j = j0 + bj, k2 = k0 + bk;
            Bs[bj][bk] = (j < N && k2 < ke) ? (TB ? tof(B[(int64_t)j * ldb + k2]) : tof(B[(int64_t)k2 * ldb + j])) : 0.f;
        }
        __syncthreads();
#pragma unroll
        for (int ks = 0; ks < 16; ks += 8) {
            uint32_t ah[2][4], al[2][4], bh[4][2], bl[4][2];
#pragma unroll
            for (int mt = 0; mt < 2; ++mt) {
                const int r = wm + mt * 16 + g;
                split_tf32(As[r][ks + t], ah[mt][0], al[mt][0]);
                split_tf32(As[r + 8][ks + t], ah[mt][1], al[mt][1]);
                split_tf32(As[r][ks + t + 4], ah[mt][2], al[mt][2]);
                split_tf32(As[r + 8][ks + t + 4], ah[mt][3], al[mt][3]);
            }
#pragma unroll
            for (int nt = 0; nt < 4; ++nt) {
                const int cj = wn + nt * 8 + g;
                if constexpr (kSplitB) {
                    split_tf32(Bs[cj][ks + t], bh[nt][0], bl[nt][0]);
                    split_tf32(Bs[cj][ks + t + 4], bh[nt][1], bl[nt][1]);
                } else {
                    bh[nt][0] = __float_as_uint(Bs[cj][ks + t]);
                    bh[nt][1] = __float_as_uint(Bs[cj][ks + t + 4]);
                }
            }
#pragma unroll
            for (int mt = 0; mt < 2; ++mt)
#pragma unroll
                for (int nt = 0; nt < 4; ++nt) {
                    mma_tf32(acc[mt][nt], al[mt], bh[nt]);
                    if constexpr (kSplitB) mma_tf32(acc[mt][nt], ah[mt], bl[nt]);
                    mma_tf32(acc[mt][nt], ah[mt], bh[nt]);
                }
        }
        __syncthreads();
    }
    // accumulator fragment: c0 (g, 2t), c1 (g, 2t+1), c2 (g+8, 2t), c3 (g+8, 2t+1)
#pragma unroll
    for (int mt = 0; mt < 2; ++mt)
#pragma unroll
        for (int nt = 0; nt < 4; ++nt)
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const int i = i0 + wm + mt * 16 + g + (q >> 1) * 8;
                const int j = j0 + wn + nt * 8 + 2 * t + (q & 1);
                if (i < M && j < N) {
                    float *p = C + (int64_t)i * ldc + j;
                    *p = accumulate ? *p + acc[mt][nt][q] : acc[mt][nt][q];
                }
            }
}

__device__ __forceinline__ float gelu(float z) { return 0.5f * z * (1.f + erff(z * 0.70710678118654752f)); }
__device__ __forceinline__ float gelu_grad(float z) {
    return 0.5f * (1.f + erff(z * 0.70710678118654752f)) + z * 0.3989422804014327f * expf(-0.5f * z * z);
}

// Z += b (row broadcast); Y = gelu(Z) or Z
__global__ void bias_act_kernel(int64_t n, int cols, float *__restrict__ Z, const float *__restrict__ b,
                                float *__restrict__ Y, int act) {
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= n * cols) return;
    const float z = Z[t] + b[t % cols];
    Z[t] = z;
    Y[t] = act ? gelu(z) : z;
}

// dY = 2 (Y - T) / (n cols); loss += sum (Y - T)^2 / (n cols)
__global__ void mse_kernel(int64_t n, int cols, const float *__restrict__ Y, const float *__restrict__ T,
                           float *__restrict__ dY, float *__restrict__ loss) {
    __shared__ float red[256];
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const float inv = 1.f / (float)(n * cols);
    float e2 = 0.f;
    if (t < n * cols) {
        const float d = Y[t] - T[t];
        dY[t] = 2.f * d * inv;
        e2 = d * d * inv;
    }
    red[threadIdx.x] = e2;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) atomicAdd(loss, red[0]);
}

__global__ void gelu_bwd_kernel(int64_t count, const float *__restrict__ Z, float *__restrict__ dY) {
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t < count) dY[t] *= gelu_grad(Z[t]);
}

// db[j] = sum_i dZ[i, j]; block (32, 32): 32 columns, 32 row lanes summed in a fixed order
__global__ void col_sum_kernel(int64_t n, int cols, const float *__restrict__ dZ, float *__restrict__ db) {
    __shared__ float part[32][33];
    const int j = blockIdx.x * 32 + threadIdx.x;
    float s = 0.f;
    if (j < cols)
        for (int64_t i = threadIdx.y; i < n; i += 32) s += dZ[i * cols + j];
    part[threadIdx.y][threadIdx.x] = s;
    __syncthreads();
    if (threadIdx.y == 0 && j < cols) {
        float t = 0.f;
        for (int r = 0; r < 32; ++r) t += part[r][threadIdx.x];
        db[j] = t;
    }
}

// C = sum over split-K slabs (fixed order)
__global__ void split_reduce_kernel(int64_t count, int splits, const float *__restrict__ part, float *__restrict__ C) {
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= count) return;
    float s = 0.f;
    for (int z = 0; z < splits; ++z) s += part[(int64_t)z * count + t];
    C[t] = s;
}

// Adam with bias correction; the step counter and learning rate come from
// device memory so the whole training step can be replayed as one graph.
__global__ void adam_kernel(int64_t count, float *__restrict__ w, __nv_bfloat16 *__restrict__ wb,
                            const float *__restrict__ g, float *__restrict__ m, float *__restrict__ v,
                            const int *__restrict__ step, const float *__restrict__ lr_sched, int nsched) {
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= count) return;
    const int s = *step;
    const float lr = lr_sched[min(s, nsched - 1)];
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    const float gi = g[t];
    const float mi = b1 * m[t] + (1.f - b1) * gi;
    const float vi = b2 * v[t] + (1.f - b2) * gi * gi;
    m[t] = mi;
    v[t] = vi;
    const float c1 = 1.f - powf(b1, (float)(s + 1)), c2 = 1.f - powf(b2, (float)(s + 1));
    const float wn = w[t] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
    w[t] = wn;
    wb[t] = __float2bfloat16_rn(wn);
}

__global__ void step_kernel(int *step, const float *loss, float *hist, int nhist) {
    const int k = *step;
    if (k < nhist) hist[k] = *loss;
    *step = k + 1;
}

__global__ void to_bf16_kernel(int64_t count, const float *__restrict__ w, __nv_bfloat16 *__restrict__ wb) {
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t < count) wb[t] = __float2bfloat16_rn(w[t]);
}

template <class T>
struct Buf {
    T *p = nullptr;
    size_t n = 0;
    ~Buf() { if (p) cudaFree(p); }
    void reserve(size_t c) {
        if (c <= n && p) return;
        if (p) cudaFree(p);
        p = nullptr;
        SUR_CUDA(cudaMalloc(&p, std::max<size_t>(c, 1) * sizeof(T)));
        n = c;
    }
};

inline unsigned blocks(int64_t count, int per = 256) { return (unsigned)((count + per - 1) / per); }

}  // namespace

struct spx_surrogate {
    int device = 0;
    cudaStream_t stream = nullptr;
    int lmax = 0, nin = 0, hidden = 0, layers = 0, nout = 0;
    std::vector<int> din, dout;          // per dense layer
    std::vector<size_t> woff, boff;      // offsets in the parameter vector
    size_t nparam = 0;
    Buf<float> w, g, m, v;               // master weights, gradients, Adam moments
    Buf<__nv_bfloat16> wb;               // BF16 weights used by every product
    Buf<float> feat, dY, loss, lr, hist, split;
    Buf<int> step;
    std::vector<Buf<float>> Z, Y;        // per layer pre-activation / output
    int64_t cap = 0;                     // rows the activation buffers hold
    cudaGraphExec_t graph = nullptr;
    int64_t graph_n = -1;
    const float *graph_targets = nullptr;
    std::string err;
};

namespace {

void ensure_rows(spx_surrogate *s, int64_t n) {
    s->feat.reserve((size_t)n * s->nin);
    for (size_t l = 0; l < s->Z.size(); ++l) {
        s->Z[l].reserve((size_t)n * s->dout[l]);
        s->Y[l].reserve((size_t)n * s->dout[l]);
    }
    size_t mx = (size_t)s->nin;
    for (int d : s->dout) mx = std::max(mx, (size_t)d);
    s->dY.reserve((size_t)n * mx * 2);
    size_t wmax = 0;
    for (size_t l = 0; l < s->din.size(); ++l) wmax = std::max(wmax, (size_t)s->din[l] * s->dout[l]);
    s->split.reserve(wmax * kMaxSplits);
    s->cap = std::max(s->cap, n);
}

template <bool TA, bool TB, class BT>
void gemm(cudaStream_t st, int M, int N, int K, const float *A, int lda, const BT *B, int ldb, float *C, int ldc,
          bool acc) {
    dim3 grid((N + 63) / 64, (M + 63) / 64);
    gemm_kernel<TA, TB, BT><<<grid, 128, 0, st>>>(M, N, K, A, lda, B, ldb, C, ldc, acc ? 1 : 0);
}

// weight gradient dW[dd x di] = dZ^T X over n samples, split along the samples
void weight_grad(spx_surrogate *s, int dd, int di, int64_t n, const float *dZ, const float *X, float *dW) {
    const int splits = (int)std::min<int64_t>(kMaxSplits, std::max<int64_t>(1, n / kSplitRows));
    dim3 grid((di + 63) / 64, (dd + 63) / 64, splits);
    if (splits == 1) {
        gemm_kernel<true, false, float><<<grid, 128, 0, s->stream>>>(dd, di, (int)n, dZ, dd, X, di, dW, di, 0);
        return;
    }
    gemm_kernel<true, false, float><<<grid, 128, 0, s->stream>>>(dd, di, (int)n, dZ, dd, X, di, s->split.p, di, 0);
    const int64_t count = (int64_t)dd * di;
    split_reduce_kernel<<<blocks(count), 256, 0, s->stream>>>(count, splits, s->split.p, dW);
}

void features(spx_surrogate *s, int64_t n, const double *b, const double *g) {
    sh_features_kernel<<<blocks(n, 128), 128, 0, s->stream>>>(n, b, g, s->lmax, s->nin, s->feat.p);
}

// forward through every layer; the output is s->Y.back()
void forward(spx_surrogate *s, int64_t n) {
    const float *x = s->feat.p;
    for (size_t l = 0; l < s->din.size(); ++l) {
        const int di = s->din[l], dd = s->dout[l];
        gemm<false, true, __nv_bfloat16>(s->stream, (int)n, dd, di, x, di, s->wb.p + s->woff[l], di, s->Z[l].p, dd, false);
        const bool act = l + 1 < s->din.size();
        bias_act_kernel<<<blocks(n * dd), 256, 0, s->stream>>>(n, dd, s->Z[l].p, s->w.p + s->boff[l], s->Y[l].p,
                                                                 act ? 1 : 0);
        x = s->Y[l].p;
    }
}

// loss and gradients of every parameter (s->g) for targets T
void backward(spx_surrogate *s, int64_t n, const float *T) {
    const size_t L = s->din.size();
    float *dA = s->dY.p, *dB = s->dY.p + s->dY.n / 2;
    SUR_CUDA(cudaMemsetAsync(s->loss.p, 0, sizeof(float), s->stream));
    mse_kernel<<<blocks(n * s->nout), 256, 0, s->stream>>>(n, s->nout, s->Y[L - 1].p, T, dA, s->loss.p);
    for (size_t li = L; li-- > 0;) {
        const int di = s->din[li], dd = s->dout[li];
        if (li + 1 < L) gelu_bwd_kernel<<<blocks(n * dd), 256, 0, s->stream>>>(n * dd, s->Z[li].p, dA);
        const float *xin = li == 0 ? s->feat.p : s->Y[li - 1].p;
        // dW = dZ^T X,  db = column sums of dZ,  dX = dZ W
        weight_grad(s, dd, di, n, dA, xin, s->g.p + s->woff[li]);
        col_sum_kernel<<<dim3((dd + 31) / 32), dim3(32, 32), 0, s->stream>>>(n, dd, dA, s->g.p + s->boff[li]);
        if (li > 0) gemm<false, false, __nv_bfloat16>(s->stream, (int)n, di, dd, dA, dd, s->wb.p + s->woff[li], di, dB, di, false);
        std::swap(dA, dB);
    }
}

void train_step(spx_surrogate *s, int64_t n, const float *T, int nsched) {
    forward(s, n);
    backward(s, n, T);
    adam_kernel<<<blocks((int64_t)s->nparam), 256, 0, s->stream>>>((int64_t)s->nparam, s->w.p, s->wb.p, s->g.p, s->m.p,
                                                                  s->v.p, s->step.p, s->lr.p, nsched);
    step_kernel<<<1, 1, 0, s->stream>>>(s->step.p, s->loss.p, s->hist.p, nsched);
}

template <class F>
spx_status sur_guard(spx_surrogate *s, F f) {
    try {
        f();
        if (s) s->err.clear();
        return SPX_OK;
    } catch (const SurErr &e) {
        if (s) s->err = e.what();
        return e.code;
    } catch (const std::bad_alloc &) {
        if (s) s->err = "host allocation failed";
        return SPX_ERR_OUT_OF_MEMORY;
    } catch (const std::exception &e) {
        if (s) s->err = e.what();
        return SPX_ERR_INTERNAL;
    }
}

void init_params(spx_surrogate *s, uint64_t seed) {
    std::vector<float> h(s->nparam, 0.f);
    std::mt19937_64 rng(seed);
    for (size_t l = 0; l < s->din.size(); ++l) {
        const float bound = std::sqrt(6.0f / (float)s->din[l]);     // He-uniform for GELU layers
        std::uniform_real_distribution<float> U(-bound, bound);
        for (size_t t = 0; t < (size_t)s->din[l] * s->dout[l]; ++t) h[s->woff[l] + t] = U(rng);
    }
    SUR_CUDA(cudaMemcpy(s->w.p, h.data(), s->nparam * sizeof(float), cudaMemcpyHostToDevice));
    to_bf16_kernel<<<blocks((int64_t)s->nparam), 256, 0, s->stream>>>((int64_t)s->nparam, s->w.p, s->wb.p);
    SUR_CUDA(cudaMemsetAsync(s->m.p, 0, s->nparam * sizeof(float), s->stream));
    SUR_CUDA(cudaMemsetAsync(s->v.p, 0, s->nparam * sizeof(float), s->stream));
    SUR_CUDA(cudaStreamSynchronize(s->stream));
}

}  // namespace

extern "C" {

spx_status spx_surrogate_create(spx_surrogate **out, int device, int32_t lmax, int32_t hidden, int32_t layers,
                                int32_t n_out, uint64_t seed) {
    if (!out) return SPX_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    if (lmax < 0 || lmax > kMaxL || hidden < 1 || hidden > 4096 || layers < 1 || layers > 16 || n_out < 1 ||
        n_out > 4096)
        return SPX_ERR_INVALID_ARGUMENT;
    spx_surrogate *s = new (std::nothrow) spx_surrogate();
    if (!s) return SPX_ERR_OUT_OF_MEMORY;
    const spx_status st = sur_guard(s, [&] {
        SUR_CUDA(cudaSetDevice(device));
        s->device = device;
        SUR_CUDA(cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking));
        s->lmax = lmax;
        s->nin = (lmax + 1) * (lmax + 1);
        s->hidden = hidden;
        s->layers = layers;
        s->nout = n_out;
        int prev = s->nin;
        for (int l = 0; l < layers; ++l) { s->din.push_back(prev); s->dout.push_back(hidden); prev = hidden; }
        s->din.push_back(prev);
        s->dout.push_back(n_out);
        size_t off = 0;
        for (size_t l = 0; l < s->din.size(); ++l) {
            s->woff.push_back(off);
            off += (size_t)s->din[l] * s->dout[l];
            s->boff.push_back(off);
            off += (size_t)s->dout[l];
        }
        s->nparam = off;
        s->w.reserve(off); s->g.reserve(off); s->m.reserve(off); s->v.reserve(off); s->wb.reserve(off);
        s->loss.reserve(1);
        s->step.reserve(1);
        s->Z.resize(s->din.size());
        s->Y.resize(s->din.size());
        init_params(s, seed);
    });
    if (st != SPX_OK) {
        spx_surrogate_destroy(s);
        return st;
    }
    *out = s;
    return SPX_OK;
}

spx_status spx_surrogate_destroy(spx_surrogate *s) {
    if (!s) return SPX_OK;
    cudaSetDevice(s->device);
    if (s->stream) cudaStreamSynchronize(s->stream);
    if (s->graph) cudaGraphExecDestroy(s->graph);
    if (s->stream) cudaStreamDestroy(s->stream);
    delete s;
    return SPX_OK;
}

int64_t spx_surrogate_num_params(const spx_surrogate *s) { return s ? (int64_t)s->nparam : 0; }

spx_status spx_surrogate_features(spx_surrogate *s, int64_t n, const double *d_beta, const double *d_gamma,
                                  float *d_features) {
    if (!s || n < 1 || !d_beta || !d_gamma || !d_features) return SPX_ERR_INVALID_ARGUMENT;
    return sur_guard(s, [&] {
        SUR_CUDA(cudaSetDevice(s->device));
        sh_features_kernel<<<blocks(n, 128), 128, 0, s->stream>>>(n, d_beta, d_gamma, s->lmax, s->nin, d_features);
        SUR_CUDA(cudaGetLastError());
        SUR_CUDA(cudaStreamSynchronize(s->stream));
    });
}

spx_status spx_surrogate_train(spx_surrogate *s, int64_t n, const double *d_beta, const double *d_gamma,
                               const float *d_targets, int32_t epochs, float lr, float *loss_out) {
    if (!s || n < 1 || !d_beta || !d_gamma || !d_targets || epochs < 1 || !(lr > 0.f)) return SPX_ERR_INVALID_ARGUMENT;
    return sur_guard(s, [&] {
        SUR_CUDA(cudaSetDevice(s->device));
        ensure_rows(s, n);
        features(s, n, d_beta, d_gamma);
        // cosine-decayed learning rate per step, read by the Adam kernel
        std::vector<float> sched(epochs);
        for (int e = 0; e < epochs; ++e)
            sched[e] = lr * (0.02f + 0.98f * 0.5f * (1.f + std::cos(3.14159265358979f * e / epochs)));
        s->lr.reserve(epochs);
        s->hist.reserve(epochs);
        SUR_CUDA(cudaMemcpyAsync(s->lr.p, sched.data(), epochs * sizeof(float), cudaMemcpyHostToDevice, s->stream));
        SUR_CUDA(cudaMemsetAsync(s->step.p, 0, sizeof(int), s->stream));
        SUR_CUDA(cudaStreamSynchronize(s->stream));
        // one training step as a graph, replayed every epoch
        if (s->graph) { cudaGraphExecDestroy(s->graph); s->graph = nullptr; }
        cudaGraph_t g = nullptr;
        SUR_CUDA(cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal));
        train_step(s, n, d_targets, epochs);
        SUR_CUDA(cudaStreamEndCapture(s->stream, &g));
        const cudaError_t ie = cudaGraphInstantiate(&s->graph, g, 0);
        cudaGraphDestroy(g);
        SUR_CUDA(ie);
        for (int e = 0; e < epochs; ++e) SUR_CUDA(cudaGraphLaunch(s->graph, s->stream));
        if (loss_out)
            SUR_CUDA(cudaMemcpyAsync(loss_out, s->hist.p, epochs * sizeof(float), cudaMemcpyDeviceToHost, s->stream));
        SUR_CUDA(cudaStreamSynchronize(s->stream));
    });
}

spx_status spx_surrogate_predict(spx_surrogate *s, int64_t n, const double *d_beta, const double *d_gamma,
                                 float *d_out) {
    if (!s || n < 1 || !d_beta || !d_gamma || !d_out) return SPX_ERR_INVALID_ARGUMENT;
    return sur_guard(s, [&] {
        SUR_CUDA(cudaSetDevice(s->device));
        ensure_rows(s, n);
        features(s, n, d_beta, d_gamma);
        forward(s, n);
        SUR_CUDA(cudaMemcpyAsync(d_out, s->Y.back().p, (size_t)n * s->nout * sizeof(float), cudaMemcpyDeviceToDevice,
                                 s->stream));
        SUR_CUDA(cudaStreamSynchronize(s->stream));
    });
}

spx_status spx_surrogate_gradients(spx_surrogate *s, int64_t n, const double *d_beta, const double *d_gamma,
                                   const float *d_targets, float *h_grad, float *h_loss) {
    if (!s || n < 1 || !d_beta || !d_gamma || !d_targets || !h_grad) return SPX_ERR_INVALID_ARGUMENT;
    return sur_guard(s, [&] {
        SUR_CUDA(cudaSetDevice(s->device));
        ensure_rows(s, n);
        features(s, n, d_beta, d_gamma);
        forward(s, n);
        backward(s, n, d_targets);
        SUR_CUDA(cudaMemcpyAsync(h_grad, s->g.p, s->nparam * sizeof(float), cudaMemcpyDeviceToHost, s->stream));
        if (h_loss) SUR_CUDA(cudaMemcpyAsync(h_loss, s->loss.p, sizeof(float), cudaMemcpyDeviceToHost, s->stream));
        SUR_CUDA(cudaStreamSynchronize(s->stream));
    });
}

spx_status spx_surrogate_get_params(spx_surrogate *s, float *h_params) {
    if (!s || !h_params) return SPX_ERR_INVALID_ARGUMENT;
    return sur_guard(s, [&] {
        SUR_CUDA(cudaSetDevice(s->device));
        SUR_CUDA(cudaMemcpy(h_params, s->w.p, s->nparam * sizeof(float), cudaMemcpyDeviceToHost));
    });
}

spx_status spx_surrogate_set_params(spx_surrogate *s, const float *h_params) {
    if (!s || !h_params) return SPX_ERR_INVALID_ARGUMENT;
    return sur_guard(s, [&] {
        SUR_CUDA(cudaSetDevice(s->device));
        SUR_CUDA(cudaMemcpy(s->w.p, h_params, s->nparam * sizeof(float), cudaMemcpyHostToDevice));
        to_bf16_kernel<<<blocks((int64_t)s->nparam), 256, 0, s->stream>>>((int64_t)s->nparam, s->w.p, s->wb.p);
        SUR_CUDA(cudaMemsetAsync(s->m.p, 0, s->nparam * sizeof(float), s->stream));
        SUR_CUDA(cudaMemsetAsync(s->v.p, 0, s->nparam * sizeof(float), s->stream));
        SUR_CUDA(cudaStreamSynchronize(s->stream));
    });
}

const char *spx_surrogate_last_error(const spx_surrogate *s) { return s ? s->err.c_str() : "NULL surrogate"; }

}  // extern "C"
