// On-GPU construction of I and Q{r}{k,m} (see builder.h).
//
// Host: irreducible spherical tensor product tables per multiplicity
// (kernel/cache/ist_product_table.m semantics, computed here from the
// irr_sph_ten.m recursion), the monomials grouped by term, a bound of the raw
// contributions per column.  Device: one warp per (term, column) expands every
// monomial of the term on the column's basis state (left and right products,
// superop.m:139-145's rule that drops unit-state halves of a commutator),
// finds each output state by binary search over the sorted basis keys, sums
// duplicates in monomial order and writes the column in row order.  A count
// pass sizes the CSC arrays, a fill pass writes them.
#include "builder.h"

#include <algorithm>
#include <cmath>
#include <map>
#include <numeric>
#include <stdexcept>
#include <string>

namespace spx {
namespace {

#define BCHECK(call)                                                                                  \
    do {                                                                                              \
        cudaError_t e_ = (call);                                                                      \
        if (e_ != cudaSuccess) throw std::runtime_error(std::string("CUDA: ") + cudaGetErrorString(e_)); \
    } while (0)

constexpr int kMaxMult = 8;

// ---------------------------------------------------------------------------
// Product tables
// ---------------------------------------------------------------------------
using Mat = std::vector<double>;   // mult x mult, row-major

Mat matmul(const Mat &a, const Mat &b, int n) {
    Mat c(n * n, 0.0);
    for (int i = 0; i < n; ++i)
        for (int l = 0; l < n; ++l) {
            const double x = a[i * n + l];
            if (x == 0.0) continue;
            for (int j = 0; j < n; ++j) c[i * n + j] += x * b[l * n + j];
        }
    return c;
}

// Unnormalised T(l, m) ordered by code l*l + l - m (kernel/operators/irr_sph_ten.m:61-75).
std::vector<Mat> ist_matrices(int mult) {
    const double s = (mult - 1) / 2.0;
    Mat up(mult * mult, 0.0), dn(mult * mult, 0.0);
    for (int i = 0; i + 1 < mult; ++i) {
        const double mz = (mult - 1 - (i + 1)) - s;           // projection of state i+1
        up[i * mult + i + 1] = std::sqrt(s * (s + 1) - mz * (mz + 1));
        dn[(i + 1) * mult + i] = up[i * mult + i + 1];
    }
    std::vector<Mat> out;
    for (int l = 0; l < mult; ++l) {
        if (l == 0) {
            Mat e(mult * mult, 0.0);
            for (int i = 0; i < mult; ++i) e[i * mult + i] = 1.0;
            out.push_back(e);
            continue;
        }
        Mat t(mult * mult, 0.0);
        for (int i = 0; i < mult; ++i) t[i * mult + i] = 1.0;
        for (int p = 0; p < l; ++p) t = matmul(t, up, mult);
        const double f = ((l & 1) ? -1.0 : 1.0) * std::pow(2.0, -l / 2.0);
        for (auto &x : t) x *= f;
        out.push_back(t);
        for (int q = l - 1; q >= -l; --q) {
            const Mat a = matmul(dn, t, mult), b = matmul(t, dn, mult);
            const double g = std::sqrt((double)(l + q + 1) * (l - q));
            for (int i = 0; i < mult * mult; ++i) t[i] = (a[i] - b[i]) / g;
            out.push_back(t);
        }
    }
    return out;
}

// left[n][m][k] = <E_k, T_n E_m>, right[n][m][k] = <E_k, E_m T_n> (E = normalised T).
void product_tables(int mult, std::vector<double> &left, std::vector<double> &right) {
    const std::vector<Mat> T = ist_matrices(mult);
    const int d = mult * mult;
    std::vector<Mat> E(d);
    for (int k = 0; k < d; ++k) {
        double nrm = 0.0;
        for (double x : T[k]) nrm += x * x;
        nrm = std::sqrt(nrm);
        E[k] = T[k];
        for (auto &x : E[k]) x /= nrm;
    }
    left.assign((size_t)d * d * d, 0.0);
    right.assign((size_t)d * d * d, 0.0);
    for (int n = 0; n < d; ++n)
        for (int m = 0; m < d; ++m) {
            const Mat tl = matmul(T[n], E[m], mult), tr = matmul(E[m], T[n], mult);
            for (int k = 0; k < d; ++k) {
                double a = 0.0, b = 0.0;
                for (int i = 0; i < mult * mult; ++i) {
                    a += E[k][i] * tl[i];
                    b += E[k][i] * tr[i];
                }
                left[((size_t)n * d + m) * d + k] = std::fabs(a) < 1e-15 ? 0.0 : a;
                right[((size_t)n * d + m) * d + k] = std::fabs(b) < 1e-15 ? 0.0 : b;
            }
        }
}

// ---------------------------------------------------------------------------
// Device side
// ---------------------------------------------------------------------------
struct DevSpec {
    int64_t dim;
    int n_terms1;                       // 1 + anisotropic terms
    const int64_t *keys;
    const int64_t *radix;
    const int *spin_d;                  // states per spin (mult^2)
    const int *spin_base;               // table list base of the spin's multiplicity
    const int *tab_off;                 // per (base + (side*d + n)*d + m): offset, count
    const int *tab_cnt;
    const int *tab_k;
    const double *tab_v;
    const int *term_ptr;                // monomials of term t: term_ptr[t] .. term_ptr[t+1]
    const int4 *mono;                   // spin_a, code_a, spin_b, code_b (spin < 0: absent)
    const double2 *coef;
    const int64_t *out_off;             // fill pass: start of column (t, j) in the outputs
    int *count;                         // count pass: entries of column (t, j)
    int *out_row;
    double2 *out_val;
    int cap;                            // entries per warp in shared memory
    int *overflow;
};

__device__ __forceinline__ int find_key(const int64_t *keys, int64_t n, int64_t key) {
    int64_t lo = 0, hi = n - 1;
    while (lo <= hi) {
        const int64_t mid = (lo + hi) >> 1;
        const int64_t v = __ldg(keys + mid);
        if (v == key) return (int)mid;
        if (v < key) lo = mid + 1;
        else hi = mid - 1;
    }
    return -1;
}

__device__ __forceinline__ int code_of(int64_t key, const DevSpec &s, int spin) {
    return (int)((key / s.radix[spin]) % s.spin_d[spin]);
}

// Expands one monomial on basis state `key` (column j): calls emit(row, value)
// for every surviving output, left half then right half (negated).
template <class Emit>
__device__ __forceinline__ void expand(const DevSpec &s, int64_t key, int4 mo, double2 c, Emit emit) {
    const int na = mo.x >= 0 && mo.y != 0, nb = mo.z >= 0 && mo.w != 0;
    if (!na && !nb) return;                     // [E, .] = 0
    const int sa = na ? mo.x : mo.z, ca = na ? mo.y : mo.w;
    const int sb = (na && nb) ? mo.z : -1, cb = (na && nb) ? mo.w : 0;
    const int da = s.spin_d[sa], ma = code_of(key, s, sa);
    const int db = sb >= 0 ? s.spin_d[sb] : 1, mb = sb >= 0 ? code_of(key, s, sb) : 0;
    const int64_t ra = s.radix[sa], rb = sb >= 0 ? s.radix[sb] : 0;
    for (int side = 0; side < 2; ++side) {
        const int ia = s.spin_base[sa] + (side * da + ca) * da + ma;
        const int oa = s.tab_off[ia], cna = s.tab_cnt[ia];
        int ob = 0, cnb = 1;
        if (sb >= 0) {
            const int ib = s.spin_base[sb] + (side * db + cb) * db + mb;
            ob = s.tab_off[ib];
            cnb = s.tab_cnt[ib];
        }
        const bool in_zero = ma == 0 && mb == 0;
        for (int x = 0; x < cna; ++x) {
            const int ka = s.tab_k[oa + x];
            const double va = s.tab_v[oa + x];
            for (int y = 0; y < cnb; ++y) {
                const int kb = sb >= 0 ? s.tab_k[ob + y] : 0;
                const double vb = sb >= 0 ? s.tab_v[ob + y] : 1.0;
                if (in_zero || (ka == 0 && kb == 0)) continue;     // superop.m:139-145
                const int64_t k2 = key + (int64_t)(ka - ma) * ra + (sb >= 0 ? (int64_t)(kb - mb) * rb : 0);
                const int row = find_key(s.keys, s.dim, k2);
                if (row < 0) continue;                              // outside the basis
                const double p = (va * vb) * (side ? -1.0 : 1.0);
                emit(row, make_double2(c.x * p, c.y * p));
            }
        }
    }
}

template <bool FILL>
__global__ void build_kernel(DevSpec s) {
    extern __shared__ unsigned char bsm[];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5, wpb = blockDim.x >> 5;
    int *rows = reinterpret_cast<int *>(bsm + (size_t)wib * s.cap * 40);
    int *keep = rows + s.cap;
    double2 *vals = reinterpret_cast<double2 *>(keep + s.cap);
    double2 *sums = vals + s.cap;
    const int64_t nwork = s.dim * s.n_terms1;
    for (int64_t w = (int64_t)blockIdx.x * wpb + wib; w < nwork; w += (int64_t)gridDim.x * wpb) {
        const int t = (int)(w / s.dim);
        const int64_t j = w % s.dim;
        const int64_t key = s.keys[j];
        const int mb = s.term_ptr[t], me = s.term_ptr[t + 1];
        // A: raw contributions in monomial order
        int ne = 0;
        bool over = false;
        for (int base = mb; base < me; base += 32) {
            const int i = base + lane;
            int cnt = 0;
            if (i < me) expand(s, key, s.mono[i], s.coef[i], [&](int, double2) { ++cnt; });
            int pre = cnt;                              // inclusive scan over the warp
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int v = __shfl_up_sync(0xffffffffu, pre, o);
                if (lane >= o) pre += v;
            }
            const int tot = __shfl_sync(0xffffffffu, pre, 31);
            if (ne + tot > s.cap) { over = true; break; }
            int at = ne + pre - cnt;
            if (i < me)
                expand(s, key, s.mono[i], s.coef[i], [&](int row, double2 v) {
                    rows[at] = row;
                    vals[at] = v;
                    ++at;
                });
            ne += tot;
        }
        if (over) {
            if (lane == 0) atomicExch(s.overflow, 1);
            if (!FILL && lane == 0) s.count[w] = 0;
            continue;
        }
        __syncwarp();
        // B: first occurrence of each row sums its duplicates in order
        for (int e = lane; e < ne; e += 32) {
            const int r = rows[e];
            bool first = true;
            for (int q = 0; q < e && first; ++q) first = rows[q] != r;
            int kp = 0;
            if (first) {
                double2 acc = make_double2(0.0, 0.0);
                double mag = 0.0;
                for (int q = e; q < ne; ++q)
                    if (rows[q] == r) {
                        acc.x += vals[q].x;
                        acc.y += vals[q].y;
                        mag += fabs(vals[q].x) + fabs(vals[q].y);
                    }
                // exact cancellations (a state the operator commutes with) leave
                // at most a few rounding units of the summed magnitudes
                kp = (fabs(acc.x) + fabs(acc.y)) > 1e-14 * mag;
                sums[e] = acc;
            }
            keep[e] = kp;
        }
        __syncwarp();
        if (!FILL) {
            int c = 0;
            for (int e = lane; e < ne; e += 32) c += keep[e];
#pragma unroll
            for (int o = 16; o; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
            if (lane == 0) s.count[w] = c;
        } else {
            const int64_t off = s.out_off[w];
            const int room = s.count[w];                // what the count pass found
            for (int e = lane; e < ne; e += 32) {
                if (!keep[e]) continue;
                const int r = rows[e];
                int rank = 0;
                for (int q = 0; q < ne; ++q) rank += keep[q] && rows[q] < r;
                if (rank >= room) {
                    atomicExch(s.overflow, 2);
                    continue;
                }
                s.out_row[off + rank] = r;
                s.out_val[off + rank] = sums[e];
            }
        }
        __syncwarp();
    }
}

template <class T>
struct DBuf {
    T *p = nullptr;
    explicit DBuf(size_t n) {
        if (n) BCHECK(cudaMalloc(&p, n * sizeof(T)));
    }
    ~DBuf() {
        if (p) cudaFree(p);
    }
    DBuf(const DBuf &) = delete;
    DBuf &operator=(const DBuf &) = delete;
};

template <class T>
T *upload(DBuf<T> &b, const std::vector<T> &v, cudaStream_t st) {
    if (!v.empty()) BCHECK(cudaMemcpyAsync(b.p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, st));
    return b.p;
}

}  // namespace

std::vector<HostCsc> build_operators(const BuildSpec &sp, cudaStream_t stream, BuildInfo *info) {
    const int ns = sp.n_spins;
    const int64_t n = sp.dim;
    if (ns < 1 || !sp.mults || !sp.keys || !sp.radix) throw std::invalid_argument("empty spin system or basis");
    if (n < 1 || n > 65535) throw std::invalid_argument("basis dimension must be 1..65535");
    if (sp.n_terms < 0 || sp.n_mono < 0 || (sp.n_mono > 0 && (!sp.mono_term || !sp.mono_spins || !sp.mono_codes || !sp.mono_coefs)))
        throw std::invalid_argument("bad monomial arrays");
    std::vector<int> d(ns);
    for (int s = 0; s < ns; ++s) {
        if (sp.mults[s] < 2 || sp.mults[s] > kMaxMult) throw std::invalid_argument("multiplicity must be 2..8");
        d[s] = sp.mults[s] * sp.mults[s];
    }
    // radix: mixed-radix place values of the per-spin state codes (basis.m ordering)
    if (sp.radix[ns - 1] != 1) throw std::invalid_argument("radix of the last spin must be 1");
    for (int s = ns - 2; s >= 0; --s)
        if (sp.radix[s] != sp.radix[s + 1] * d[s + 1]) throw std::invalid_argument("radix does not match the multiplicities");
    const double span = (double)sp.radix[0] * d[0];
    if (span > 9.0e18) throw std::invalid_argument("basis keys overflow 64 bits");
    for (int64_t j = 0; j < n; ++j) {
        if (sp.keys[j] < 0 || (double)sp.keys[j] >= span) throw std::invalid_argument("basis key out of range");
        if (j && sp.keys[j] <= sp.keys[j - 1]) throw std::invalid_argument("basis keys must be strictly ascending");
    }
    // product tables of each multiplicity as compact (k, value) lists
    std::map<int, int> base_of;
    std::vector<int> tab_off, tab_cnt, tab_k, maxcnt_of;     // maxcnt per (base + side*d + n)
    std::vector<double> tab_v;
    std::vector<int> spin_base(ns);
    for (int s = 0; s < ns; ++s) {
        const int mult = sp.mults[s];
        auto it = base_of.find(mult);
        if (it == base_of.end()) {
            const int dd = mult * mult, base = (int)tab_off.size();
            std::vector<double> L, R;
            product_tables(mult, L, R);
            tab_off.resize(base + 2 * dd * dd);
            tab_cnt.resize(base + 2 * dd * dd);
            for (int side = 0; side < 2; ++side)
                for (int c = 0; c < dd; ++c)
                    for (int m = 0; m < dd; ++m) {
                        const std::vector<double> &T = side ? R : L;
                        const int idx = base + (side * dd + c) * dd + m;
                        tab_off[idx] = (int)tab_k.size();
                        for (int k = 0; k < dd; ++k) {
                            const double v = T[((size_t)c * dd + m) * dd + k];
                            if (v != 0.0) {
                                tab_k.push_back(k);
                                tab_v.push_back(v);
                            }
                        }
                        tab_cnt[idx] = (int)tab_k.size() - tab_off[idx];
                    }
            it = base_of.emplace(mult, base).first;
        }
        spin_base[s] = it->second;
    }
    auto max_out = [&](int spin, int side, int code) {
        int mx = 0;
        for (int m = 0; m < d[spin]; ++m) mx = std::max(mx, tab_cnt[spin_base[spin] + (side * d[spin] + code) * d[spin] + m]);
        return mx;
    };
    // monomials grouped by term (stable: the caller's order within a term)
    const int nt1 = 1 + sp.n_terms;
    std::vector<int> order((size_t)sp.n_mono);
    std::iota(order.begin(), order.end(), 0);
    for (int64_t i = 0; i < sp.n_mono; ++i) {
        if (sp.mono_term[i] < 0 || sp.mono_term[i] >= nt1) throw std::invalid_argument("monomial term index out of range");
        for (int f = 0; f < 2; ++f) {
            const int spn = sp.mono_spins[2 * i + f], code = sp.mono_codes[2 * i + f];
            if (spn < -1 || spn >= ns) throw std::invalid_argument("monomial spin index out of range");
            if (spn >= 0 && (code < 0 || code >= d[spn])) throw std::invalid_argument("monomial state code out of range");
        }
        if (sp.mono_spins[2 * i] >= 0 && sp.mono_spins[2 * i] == sp.mono_spins[2 * i + 1])
            throw std::invalid_argument("a monomial acts on two different spins");
        if (!std::isfinite(sp.mono_coefs[2 * i]) || !std::isfinite(sp.mono_coefs[2 * i + 1]))
            throw std::invalid_argument("non-finite monomial coefficient");
    }
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return sp.mono_term[a] < sp.mono_term[b]; });
    std::vector<int> term_ptr(nt1 + 1, 0);
    std::vector<int4> mono((size_t)sp.n_mono);
    std::vector<double2> coef((size_t)sp.n_mono);
    std::vector<int64_t> bound(nt1, 0);
    for (int64_t q = 0; q < sp.n_mono; ++q) {
        const int i = order[q];
        const int t = sp.mono_term[i];
        term_ptr[t + 1]++;
        int4 mo{sp.mono_spins[2 * i], sp.mono_codes[2 * i], sp.mono_spins[2 * i + 1], sp.mono_codes[2 * i + 1]};
        if (mo.x < 0) mo.y = 0;
        if (mo.z < 0) mo.w = 0;
        mono[q] = mo;
        coef[q] = make_double2(sp.mono_coefs[2 * i], sp.mono_coefs[2 * i + 1]);
        int64_t b = 0;
        for (int side = 0; side < 2; ++side)
            b += (int64_t)(mo.x >= 0 ? max_out(mo.x, side, mo.y) : 1) * (mo.z >= 0 ? max_out(mo.z, side, mo.w) : 1);
        bound[t] += b;
    }
    for (int t = 0; t < nt1; ++t) term_ptr[t + 1] += term_ptr[t];
    // entries per warp, a multiple of 4 so that the double2 arrays stay 16-byte aligned
    const int64_t cap = (std::max<int64_t>(32, *std::max_element(bound.begin(), bound.end())) + 3) / 4 * 4;
    int dev = 0;
    BCHECK(cudaGetDevice(&dev));
    int smem_optin = 0;
    BCHECK(cudaDeviceGetAttribute(&smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    if (cap * 40 > smem_optin)
        throw std::invalid_argument("too many contributions per column for shared memory (" + std::to_string(cap) + ")");
    const int wpb = (int)std::max<int64_t>(1, std::min<int64_t>(8, smem_optin / (cap * 40)));
    const size_t smem = (size_t)wpb * cap * 40;
    int sms = 0;
    BCHECK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));

    std::vector<int> spin_d(d.begin(), d.end());
    DBuf<int64_t> d_keys(n), d_radix(ns), d_off((size_t)n * nt1);
    DBuf<int> d_sd(ns), d_sb(ns), d_toff(tab_off.size()), d_tcnt(tab_cnt.size()), d_tk(std::max<size_t>(1, tab_k.size())),
        d_tptr(term_ptr.size()), d_count((size_t)n * nt1), d_over(1);
    DBuf<double> d_tv(std::max<size_t>(1, tab_v.size()));
    DBuf<int4> d_mono(std::max<size_t>(1, mono.size()));
    DBuf<double2> d_coef(std::max<size_t>(1, coef.size()));
    DevSpec ds{};
    ds.dim = n;
    ds.n_terms1 = nt1;
    ds.keys = upload(d_keys, std::vector<int64_t>(sp.keys, sp.keys + n), stream);
    ds.radix = upload(d_radix, std::vector<int64_t>(sp.radix, sp.radix + ns), stream);
    ds.spin_d = upload(d_sd, spin_d, stream);
    ds.spin_base = upload(d_sb, spin_base, stream);
    ds.tab_off = upload(d_toff, tab_off, stream);
    ds.tab_cnt = upload(d_tcnt, tab_cnt, stream);
    ds.tab_k = upload(d_tk, tab_k, stream);
    ds.tab_v = upload(d_tv, tab_v, stream);
    ds.term_ptr = upload(d_tptr, term_ptr, stream);
    ds.mono = upload(d_mono, mono, stream);
    ds.coef = upload(d_coef, coef, stream);
    ds.count = d_count.p;
    ds.cap = (int)cap;
    ds.overflow = d_over.p;
    BCHECK(cudaMemsetAsync(d_over.p, 0, sizeof(int), stream));
    BCHECK(cudaFuncSetAttribute(reinterpret_cast<const void *>(&build_kernel<false>),
                                cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    BCHECK(cudaFuncSetAttribute(reinterpret_cast<const void *>(&build_kernel<true>),
                                cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    const int64_t nwork = n * nt1;
    const int grid = (int)std::max<int64_t>(1, std::min<int64_t>((nwork + wpb - 1) / wpb, (int64_t)sms * 16));
    cudaEvent_t e0, e1;
    BCHECK(cudaEventCreate(&e0));
    BCHECK(cudaEventCreate(&e1));
    BCHECK(cudaEventRecord(e0, stream));
    build_kernel<false><<<grid, wpb * 32, smem, stream>>>(ds);
    BCHECK(cudaGetLastError());
    std::vector<int> count((size_t)nwork);
    int over = 0;
    BCHECK(cudaMemcpyAsync(count.data(), d_count.p, count.size() * sizeof(int), cudaMemcpyDeviceToHost, stream));
    BCHECK(cudaMemcpyAsync(&over, d_over.p, sizeof(int), cudaMemcpyDeviceToHost, stream));
    BCHECK(cudaStreamSynchronize(stream));
    if (over) throw std::runtime_error("column contribution bound exceeded");
    std::vector<int64_t> off((size_t)nwork);
    int64_t total = 0;
    for (int64_t w = 0; w < nwork; ++w) {
        off[w] = total;
        total += count[w];
    }
    DBuf<int> d_row(std::max<int64_t>(1, total));
    DBuf<double2> d_val(std::max<int64_t>(1, total));
    ds.out_off = upload(d_off, off, stream);
    ds.out_row = d_row.p;
    ds.out_val = d_val.p;
    build_kernel<true><<<grid, wpb * 32, smem, stream>>>(ds);
    BCHECK(cudaGetLastError());
    BCHECK(cudaEventRecord(e1, stream));
    BCHECK(cudaMemcpyAsync(&over, d_over.p, sizeof(int), cudaMemcpyDeviceToHost, stream));
    std::vector<int> rows((size_t)total);
    std::vector<double2> vals((size_t)total);
    if (total) {
        BCHECK(cudaMemcpyAsync(rows.data(), d_row.p, total * sizeof(int), cudaMemcpyDeviceToHost, stream));
        BCHECK(cudaMemcpyAsync(vals.data(), d_val.p, total * sizeof(double2), cudaMemcpyDeviceToHost, stream));
    }
    BCHECK(cudaStreamSynchronize(stream));
    if (over) throw std::runtime_error("count and fill passes disagree");
    float ms = 0.0f;
    BCHECK(cudaEventElapsedTime(&ms, e0, e1));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    std::vector<HostCsc> out(nt1);
    for (int t = 0; t < nt1; ++t) {
        HostCsc &A = out[t];
        const int64_t b0 = off[(size_t)t * n];
        const int64_t b1 = t + 1 < nt1 ? off[(size_t)(t + 1) * n] : total;
        A.colptr.resize(n + 1);
        for (int64_t j = 0; j < n; ++j) A.colptr[j] = off[(size_t)t * n + j] - b0;
        A.colptr[n] = b1 - b0;
        A.rowidx.resize(b1 - b0);
        A.values.resize(2 * (b1 - b0));
        for (int64_t p = b0; p < b1; ++p) {
            A.rowidx[p - b0] = rows[p];
            A.values[2 * (p - b0)] = vals[p].x;
            A.values[2 * (p - b0) + 1] = vals[p].y;
        }
    }
    if (info) {
        info->kernel_ms = ms;
        info->nnz = total;
        info->max_entries = (int)cap;
    }
    return out;
}

}  // namespace spx
