// ORACLE TEST INFRASTRUCTURE — not part of the product.
//
// Seeded synthetic inputs for the CPU restatement, drawn with the C++
// standard library generators the reference uses, so the oracle can make its
// own inputs without the product library:
//   random_vec  (reference src/linalg.cpp:44-48): std::mt19937 and
//               std::normal_distribution<double>(0, 1), one draw each for the
//               imaginary and then the real part of every entry (the order
//               GCC on x86-64 gives the reference's cx(dist(rng), dist(rng)));
//   gauge links theta_mu(s) ~ N(0, 1/beta) i.i.d., mu-major then site order,
//               U = exp(i theta).
// A generator object (orc_rng_*) keeps one std::mt19937 across several
// random_vec draws, as the reference's hierarchy set-up does with its rng
// (src/multigrid.cpp:435-484, 545-587).
#include <cmath>
#include <complex>
#include <cstdint>
#include <random>

namespace {

struct Rng {
    std::mt19937 gen;
    std::normal_distribution<double> unit{0.0, 1.0};
    explicit Rng(uint32_t seed) : gen(seed) {}
    void random_vec(long n, double* v) {
        for (long i = 0; i < n; ++i) {
            const double im = unit(gen);
            const double re = unit(gen);
            v[2 * i] = re;
            v[2 * i + 1] = im;
        }
    }
};

}  // namespace

extern "C" {

void* orc_rng_create(uint32_t seed) { return new Rng(seed); }

void orc_rng_random_vec(void* h, long n, double* v) { static_cast<Rng*>(h)->random_vec(n, v); }

void orc_rng_destroy(void* h) { delete static_cast<Rng*>(h); }

void orc_random_vec(long n, uint32_t seed, double* v) {
    Rng r(seed);
    r.random_vec(n, v);
}

void orc_gauge_normal(int L, double beta, uint32_t seed, double* U) {
    std::mt19937 gen(seed);
    std::normal_distribution<double> theta(0.0, std::sqrt(1.0 / beta));
    const long V = (long)L * L;
    for (long i = 0; i < 2 * V; ++i) {
        const std::complex<double> u = std::exp(std::complex<double>(0.0, theta(gen)));
        U[2 * i] = u.real();
        U[2 * i + 1] = u.imag();
    }
}

}  // extern "C"
