// Seeded synthetic inputs, drawn with the C++ standard library generators the
// reference uses so that a seed reproduces the reference's own numbers:
//   random_vec   (reference src/linalg.cpp:44-48): std::mt19937 and
//                std::normal_distribution<double>(0, 1).  The reference writes
//                cx(dist(rng), dist(rng)), whose argument evaluation order C++
//                leaves unspecified; GCC on x86-64 evaluates right to left, so
//                the reference's vectors draw the imaginary part first.  This
//                generator fixes that order explicitly (imaginary, then real),
//                so it reproduces the reference built by GCC on x86-64;
//   gauge links  theta_mu(s) ~ N(0, 1/beta) i.i.d., mu-major then site order,
//                U = exp(i theta)  (the reference's own GaugeField::randomise,
//                src/gauge.h:19-24, draws uniform phases instead).
#include <complex>
#include <cmath>
#include <cstdint>
#include <random>

#include "../../include/smg_gpu.h"

namespace {
using cxd = std::complex<double>;
}

extern "C" {

SMG_API smg_status smg_host_gauge_normal(int L, double beta, uint32_t seed, double* U) {
    if (L < 2 || !(beta > 0) || !U) return SMG_BAD_ARG;
    std::mt19937 rng(seed);
    std::normal_distribution<double> dist(0.0, std::sqrt(1.0 / beta));
    const int64_t V = (int64_t)L * L;
    for (int64_t i = 0; i < 2 * V; ++i) {
        double th = dist(rng);
        cxd u = std::exp(cxd(0.0, th));
        U[2 * i] = u.real();
        U[2 * i + 1] = u.imag();
    }
    return SMG_OK;
}

SMG_API smg_status smg_host_random_vec(int64_t n_complex, uint32_t seed, double* v) {
    if (n_complex < 0 || (!v && n_complex > 0)) return SMG_BAD_ARG;
    std::mt19937 rng(seed);
    std::normal_distribution<double> dist(0.0, 1.0);
    for (int64_t i = 0; i < n_complex; ++i) {
        double im = dist(rng);
        double re = dist(rng);
        v[2 * i] = re;
        v[2 * i + 1] = im;
    }
    return SMG_OK;
}

}  // extern "C"
