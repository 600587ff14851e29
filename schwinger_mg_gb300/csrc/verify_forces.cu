// verify_forces (reference src/hmc_forces.cpp:869-981): the analytic gauge and
// pseudofermion forces of the device against central finite differences of the
// actions, at the reference's 20 links, with its pseudofermion
// (eta = random_vec from std::mt19937(12345), phi = D^dag eta, or phi_o =
// M^dag eta_o on the even-odd path) and its step eps = 1e-5.  Host code over
// the library's own entry points: every action and force is computed on the
// device; each perturbed configuration is a fresh gauge handle.
#include <cmath>
#include <cstring>
#include <memory>
#include <random>
#include <vector>

#include "smg_internal.h"

namespace {

struct Gauge {
    smg_gauge* h = nullptr;
    ~Gauge() { smg_gauge_destroy(h); }
};
struct Dirac {
    smg_dirac* h = nullptr;
    ~Dirac() { smg_dirac_destroy(h); }
};
struct Fld {
    smg_field* h = nullptr;
    ~Fld() { smg_field_destroy(h); }
};

#define VF_TRY(x)                          \
    do {                                   \
        const smg_status s_ = (x);         \
        if (s_ != SMG_OK) return s_;       \
    } while (0)

// S_F of the pseudofermion phi for the links U (host [mu][s] complex)
smg_status fermion_action(smg_context* ctx, int L, const std::vector<double>& U, double mass, double r, double c_sw,
                          double mu_t, bool eo, const smg_field* phi, int max_iter, double tol, double* S) {
    Gauge g;
    VF_TRY(smg_gauge_create(ctx, L, U.data(), &g.h));
    Dirac d;
    VF_TRY(smg_dirac_create(g.h, mass, r, c_sw, mu_t, &d.h));
    Fld X;
    VF_TRY(smg_field_create(ctx, L, 1, SMG_F64, &X.h));
    smg_solve_result res{};
    smg_status st = eo ? smg_eo_cg_solve(d.h, phi, X.h, max_iter, tol, &res)
                       : smg_cg_solve(d.h, phi, X.h, max_iter, tol, &res);
    if (st != SMG_OK && st != SMG_NOT_CONVERGED) return st;  // the reference carries on after a warning
    double dot[2] = {0, 0};
    VF_TRY(smg_blas_dot(phi, X.h, dot));
    *S = dot[0];
    if (eo && c_sw != 0.0) {
        double ld = 0;
        VF_TRY(smg_eo_logdet_ee(d.h, &ld));
        *S -= 2.0 * ld;
    }
    return SMG_OK;
}

}  // namespace

extern "C" {

SMG_API smg_status smg_verify_forces(smg_gauge* g, double beta, double mass, double wilson_r, int max_iter, double tol,
                                     double c_sw, int use_eo, double err_threshold, double mu_t,
                                     smg_force_check* out) {
    if (!g || !out || max_iter < 1 || !(tol > 0)) return SMG_BAD_ARG;
    smg_context* ctx = g->ctx;
    const int L = g->g.L, V = L * L;
    const bool eo = use_eo != 0;
    const double eps = 1e-5;
    std::vector<double> U((size_t)4 * V);
    VF_TRY(smg_gauge_get(g, U.data()));
    Dirac d0;
    VF_TRY(smg_dirac_create(g, mass, wilson_r, c_sw, mu_t, &d0.h));
    std::vector<double> gf((size_t)2 * V), ff((size_t)2 * V);
    VF_TRY(smg_gauge_force(g, beta, gf.data()));

    // eta = random_vec(n, mt19937(12345)) (each entry's imaginary part drawn first), phi = D^dag eta
    // or, on the even-odd path, eta_o of the odd half and phi_o = M^dag eta_o
    std::mt19937 rng(12345);
    std::normal_distribution<double> dist(0.0, 1.0);
    const int n = eo ? V : 2 * V;  // complex entries drawn
    std::vector<double> eta((size_t)4 * V, 0.0);
    double* dst = eta.data() + (eo ? (size_t)2 * V : 0);  // odd half: the second half of the field
    for (int i = 0; i < n; ++i) {
        const double im = dist(rng);
        const double re = dist(rng);
        dst[2 * i] = re;
        dst[2 * i + 1] = im;
    }
    Fld feta, phi, X;
    VF_TRY(smg_field_create(ctx, L, 1, SMG_F64, &feta.h));
    VF_TRY(smg_field_create(ctx, L, 1, SMG_F64, &phi.h));
    VF_TRY(smg_field_create(ctx, L, 1, SMG_F64, &X.h));
    VF_TRY(smg_field_upload(feta.h, eta.data()));
    smg_solve_result res{};
    if (eo) {
        VF_TRY(smg_field_zero(phi.h));
        VF_TRY(smg_eo_apply(d0.h, SMG_EO_SCHUR_DAG, feta.h, phi.h));
        const smg_status st = smg_eo_cg_solve(d0.h, phi.h, X.h, max_iter, tol, &res);
        if (st != SMG_OK && st != SMG_NOT_CONVERGED) return st;
        VF_TRY(smg_eo_fermion_force(d0.h, X.h, ff.data()));
    } else {
        VF_TRY(smg_dirac_apply(d0.h, SMG_OP_DDAG, feta.h, phi.h));
        const smg_status st = smg_cg_solve(d0.h, phi.h, X.h, max_iter, tol, &res);
        if (st != SMG_OK && st != SMG_NOT_CONVERGED) return st;
        VF_TRY(smg_fermion_force(d0.h, X.h, ff.data()));
    }

    std::memset(out, 0, sizeof(*out));
    out->n_links = SMG_VERIFY_LINKS;
    double gmax_err = 0, fmax_err = 0, gmax_val = 0, fmax_val = 0;
    std::vector<double> Up = U, Um = U;
    for (int t = 0; t < SMG_VERIFY_LINKS; ++t) {
        const int mu = t % 2;
        const int s = (t * 7 + t / 2 * 13) % V;
        const size_t k = 2 * ((size_t)mu * V + s);
        // U_mu(s) times exp(+-i eps)
        const double ur = U[k], ui = U[k + 1], c = std::cos(eps), sn = std::sin(eps);
        Up[k] = ur * c - ui * sn;
        Up[k + 1] = ur * sn + ui * c;
        Um[k] = ur * c + ui * sn;
        Um[k + 1] = -ur * sn + ui * c;
        double sgp = 0, sgm = 0, sfp = 0, sfm = 0;
        {
            Gauge gp, gm;
            VF_TRY(smg_gauge_create(ctx, L, Up.data(), &gp.h));
            VF_TRY(smg_gauge_create(ctx, L, Um.data(), &gm.h));
            VF_TRY(smg_gauge_action(gp.h, beta, &sgp));
            VF_TRY(smg_gauge_action(gm.h, beta, &sgm));
        }
        VF_TRY(fermion_action(ctx, L, Up, mass, wilson_r, c_sw, mu_t, eo, phi.h, max_iter, tol, &sfp));
        VF_TRY(fermion_action(ctx, L, Um, mass, wilson_r, c_sw, mu_t, eo, phi.h, max_iter, tol, &sfm));
        Up[k] = Um[k] = ur;
        Up[k + 1] = Um[k + 1] = ui;
        const double gnum = -(sgp - sgm) / (2 * eps), fnum = -(sfp - sfm) / (2 * eps);
        const double gana = gf[(size_t)mu * V + s], fana = ff[(size_t)mu * V + s];
        out->mu[t] = mu;
        out->site[t] = s;
        out->gf_ana[t] = gana;
        out->gf_num[t] = gnum;
        out->ff_ana[t] = fana;
        out->ff_num[t] = fnum;
        gmax_err = std::fmax(gmax_err, std::fabs(gana - gnum));
        fmax_err = std::fmax(fmax_err, std::fabs(fana - fnum));
        gmax_val = std::fmax(gmax_val, std::fabs(gana));
        fmax_val = std::fmax(fmax_val, std::fabs(fana));
    }
    out->gauge_max_err = gmax_err;
    out->fermion_max_err = fmax_err;
    out->gauge_rel = gmax_err / std::fmax(gmax_val, 1e-30);
    out->fermion_rel = fmax_err / std::fmax(fmax_val, 1e-30);
    out->gauge_passed = out->gauge_rel < err_threshold ? 1 : 0;
    out->fermion_passed = out->fermion_rel < err_threshold ? 1 : 0;
    out->passed = out->gauge_passed && out->fermion_passed;
    return SMG_OK;
}

}  // extern "C"
