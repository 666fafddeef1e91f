// Device-side pre-verification of sieve survivors (this project's addition).
//
// The reference hands every modular survivor to its host pool, which tests
// gcd(a, b) = 1 and takes an exact square root with GMP (src/point_search.cpp:
// 28-60, src/exact_polynomial.cpp:25-42).  Here a kernel first drops the
// survivors that cannot be points, on the device, before the copy to the host:
//   - gcd(a, d) != 1;
//   - F(a, d) mod 2^64 is not a square mod 2^64;
//   - F(a, d) mod p is not a square mod p (0 counts as a square) for one of
//     the primes 3 .. 97, or for one of four primes just below 2^31 (Euler's
//     criterion).
// F(a, d) = sum c_i a^i d^(n-i), times d when the coefficient count is even,
// as the host's exact check evaluates it.  A point has F = y^2, so it passes
// every test: the filtered set still holds every point, and the host's exact
// check of what remains yields the same points.
#pragma once

#include <cuda_runtime.h>

#include <string>
#include <vector>

namespace rpg {

class Preverifier {
public:
    Preverifier() = default;
    ~Preverifier();
    Preverifier(const Preverifier &) = delete;
    Preverifier &operator=(const Preverifier &) = delete;

    // Coefficient residues of each curve (curve i = survivors tagged i),
    // uploaded on `stream`; device buffers grow and are kept across calls.
    void prepare(const std::vector<const std::vector<std::string> *> &curves, cudaStream_t stream);

    // Filter survivors [0, min(*count, capacity)) of the device arrays a, d
    // (and curve, or nullptr for curve 0) into out_a, out_d (out_curve), whose
    // count goes to *out_count (zeroed by the caller before the launch).  The
    // output order is unspecified.  curve_modular (optional, zeroed by the
    // caller) receives each curve's input survivor count.  Allocates nothing;
    // may be captured in a CUDA graph.
    void launch(const long long *a, const int *d, const int *curve, const unsigned long long *count,
                unsigned long long capacity, long long *out_a, int *out_d, int *out_curve,
                unsigned long long *out_count, unsigned long long *curve_modular, cudaStream_t stream) const;

    unsigned long long upload_bytes() const { return upload_bytes_; }

private:
    void release();
    void *curves_ = nullptr;       // device PreCurve[ncurves]
    void *coefs_ = nullptr;        // device PreCoef[ncoefs]
    std::size_t curves_cap_ = 0, coefs_cap_ = 0;
    int blocks_ = 0;
    unsigned long long upload_bytes_ = 0;
};

// Host restatement of the device test for one survivor (CPU tests compare it
// with the exact check on small boxes).
bool preverify_host(const std::vector<std::string> &coefficients, long long a, long long d);

}  // namespace rpg
