// On-GPU construction of the rotational-basis Liouvillian terms
// (kernel/hamiltonian.m:59-790 with kernel/operators/superop.m:36-185 for the
// spherical-tensor Liouville formalism): the isotropic part I and every
// Q{r}{k,m} as sums of commutation superoperators of one- and two-spin
// irreducible spherical tensor products, built column by column on the device.
#pragma once

#include <cstdint>
#include <vector>

#include <cuda_runtime.h>

namespace spx {

// A monomial is coef * [T(code_a) on spin_a * T(code_b) on spin_b, .] (the
// commutation superoperator); spin_b < 0 for a one-spin operator.  term 0 is
// the isotropic part, term t > 0 the t-th anisotropic term.
struct BuildSpec {
    int n_spins = 0;
    const int32_t *mults = nullptr;      // n_spins, 2..4
    int64_t dim = 0;
    const int64_t *keys = nullptr;       // dim basis keys, sum_s code_s * radix_s, ascending
    const int64_t *radix = nullptr;      // n_spins
    int n_terms = 0;                     // anisotropic terms (term indices 1..n_terms)
    int64_t n_mono = 0;
    const int32_t *mono_term = nullptr;  // n_mono, 0..n_terms
    const int32_t *mono_spins = nullptr; // 2 n_mono
    const int32_t *mono_codes = nullptr; // 2 n_mono
    const double *mono_coefs = nullptr;  // 2 n_mono, interleaved complex
};

// One built matrix in MATLAB's CSC layout (0-based, interleaved complex).
struct HostCsc {
    std::vector<int64_t> colptr, rowidx;
    std::vector<double> values;
};

// Statistics of the last build (device time of the two passes).
struct BuildInfo {
    float kernel_ms = 0.0f;
    int64_t nnz = 0;
    int max_entries = 0;        // bound of raw contributions per column
};

// Builds the 1 + n_terms matrices on `stream` (synchronises it).  Throws
// std::runtime_error with a message on bad input or CUDA failure.
std::vector<HostCsc> build_operators(const BuildSpec &spec, cudaStream_t stream, BuildInfo *info);

}  // namespace spx
