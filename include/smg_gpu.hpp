// smg_gpu.hpp — header-only C++ drop-in over the C ABI (smg_gpu.h) with the
// reference's own types and call shapes (cpviolator/Schwinger_MG):
//   cx, Vec, RVec, OpApply                  src/types.h:7-10
//   Lattice                                 src/lattice.h:4-42
//   GaugeField                              src/gauge.h:10-36
//   DiracOp::apply/apply_dag/apply_DdagD    src/dirac.h:115-152
//   CGResult, cg_solve                      src/solvers.h:25-39
//   FCGResult, fcg_solve, fcg_solve_mg      src/solvers.h:31-35, 57-84
//   MGConfig, build_full_mg                 src/config.h:19-30, src/mg_builder.h:6-11
//   MGHierarchy::precondition               src/multigrid.h:63
//   fermion_force, gauge_force, gauge_action  src/hmc.h:46-69
//   cg_solve_precond, cg_solve_x0(_precond)   src/solvers.h:41-53, 99-104
//   FGMRESResult, RitzPair, fgmres_solve_mg   src/solvers.h:13-23, 62-79
//   mr_smooth, richardson_smooth_op,
//   estimate_lambda_max                     src/smoother.h
//   MGHierarchy::set_symmetric              src/multigrid.h:62
//   MGHierarchy::rebuild                    src/multigrid.cpp:158-193 (rebuild_deeper_levels)
//   MGHierarchy::setup_deflation / deflation / deflation_rr / lowmode_solution
//                                           src/coarse_op.cpp:10-54, src/eigen_evolve.cpp:48, src/hmc.h:307
//   coarse_lowmode_force                    src/hmc_multiscale.cpp:237-276
//   verify_forces                           src/hmc_forces.cpp:869-981
//   hmc_trajectory, reversibility_test_plain, hmc_trajectory_mg_multiscale,
//   reversibility_test_mg_multiscale        src/hmc_trajectory.cpp:38-509, src/hmc_multiscale.cpp:340-1000
//   fermion_action(_precond) + fermion_force as a forward/backward pair
//                                           src/hmc.h (FermionActionResult)
// Host vectors keep the reference layout (Vec v[2*s + spin]); each call copies
// them to the device, runs the sm_103a kernels and copies results back.
// Failures throw smg::Error carrying the smg_status, where the reference
// asserts or prints a warning.
#pragma once

#include <array>
#include <complex>
#include <functional>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "smg_gpu.h"

namespace smg {

using cx = std::complex<double>;
using Vec = std::vector<cx>;
using RVec = std::vector<double>;
using OpApply = std::function<void(const Vec& src, Vec& dst)>;

struct Error : std::runtime_error {
    smg_status status;
    Error(smg_status s, const std::string& m) : std::runtime_error(m), status(s) {}
};

inline void check(smg_status s, smg_context* ctx, const char* where) {
    if (s == SMG_OK) return;
    std::string msg = std::string(where) + ": " + smg_status_string(s);
    if (ctx) msg += std::string(" (") + smg_last_error(ctx) + ")";
    throw Error(s, msg);
}

// One device + stream per host thread; created on first use.
inline smg_context* default_context() {
    static thread_local std::unique_ptr<smg_context, smg_status (*)(smg_context*)> ctx(
        [] {
            smg_context* c = nullptr;
            check(smg_context_create(0, nullptr, &c), nullptr, "smg_context_create");
            return c;
        }(),
        &smg_context_destroy);
    return ctx.get();
}

struct Lattice {
    int L, V, ndof, V_half;
    explicit Lattice(int L_) : L(L_), V(L_ * L_), ndof(2 * L_ * L_), V_half(L_ * L_ / 2) {}
};

class GaugeField {
   public:
    const Lattice& lat;
    std::array<Vec, 2> U;  // host copy, reference layout U[mu][s]

    explicit GaugeField(const Lattice& lat_) : lat(lat_) {
        U[0].assign(lat.V, 1.0);
        U[1].assign(lat.V, 1.0);
    }
    // Copies the host links to the device; call after changing U.
    void sync() const {
        std::vector<double> flat(4 * (size_t)lat.V);
        for (int mu = 0; mu < 2; ++mu)
            for (int s = 0; s < lat.V; ++s) {
                flat[2 * ((size_t)mu * lat.V + s)] = U[mu][s].real();
                flat[2 * ((size_t)mu * lat.V + s) + 1] = U[mu][s].imag();
            }
        smg_context* ctx = default_context();
        if (!h_) {
            smg_gauge* g = nullptr;
            check(smg_gauge_create(ctx, lat.L, flat.data(), &g), ctx, "smg_gauge_create");
            h_.reset(g);
        } else {
            check(smg_gauge_set(h_.get(), flat.data()), ctx, "smg_gauge_set");
        }
    }
    smg_gauge* handle() const {
        if (!h_) sync();
        return h_.get();
    }
    double avg_plaq() const {
        double v = 0;
        check(smg_gauge_avg_plaq(handle(), &v), default_context(), "smg_gauge_avg_plaq");
        return v;
    }
    // Copies the device links into the host copy U (after a device-side update such as an HMC step).
    void pull() {
        std::vector<double> flat(4 * (size_t)lat.V);
        check(smg_gauge_get(handle(), flat.data()), default_context(), "smg_gauge_get");
        for (int mu = 0; mu < 2; ++mu)
            for (int s = 0; s < lat.V; ++s)
                U[mu][s] = cx(flat[2 * ((size_t)mu * lat.V + s)], flat[2 * ((size_t)mu * lat.V + s) + 1]);
    }

   private:
    mutable std::unique_ptr<smg_gauge, smg_status (*)(smg_gauge*)> h_{nullptr, &smg_gauge_destroy};
};

// Device field of nrhs spinors with host-Vec transfers.
class DeviceField {
   public:
    DeviceField(int L, int nrhs, smg_precision p = SMG_F64) {
        smg_field* f = nullptr;
        check(smg_field_create(default_context(), L, nrhs, p, &f), default_context(), "smg_field_create");
        h_.reset(f);
    }
    void upload(const Vec& v) {
        check(smg_field_upload(h_.get(), reinterpret_cast<const double*>(v.data())), default_context(), "upload");
    }
    void download(Vec& v) const {
        check(smg_field_download(h_.get(), reinterpret_cast<double*>(v.data())), default_context(), "download");
    }
    smg_field* get() const { return h_.get(); }

   private:
    std::unique_ptr<smg_field, smg_status (*)(smg_field*)> h_{nullptr, &smg_field_destroy};
};

class DiracOp {
   public:
    const Lattice& lat;
    const GaugeField& gauge;
    double mass, r, c_sw, mu_t;

    DiracOp(const Lattice& lat_, const GaugeField& g_, double m_, double r_ = 1.0, double csw_ = 0.0,
            double mu_t_ = 0.0)
        : lat(lat_), gauge(g_), mass(m_), r(r_), c_sw(csw_), mu_t(mu_t_) {
        smg_dirac* d = nullptr;
        check(smg_dirac_create(gauge.handle(), mass, r, c_sw, mu_t, &d), default_context(), "smg_dirac_create");
        h_.reset(d);
    }
    // Recomputes the clover term after GaugeField::sync().
    void refresh() { check(smg_dirac_refresh(h_.get()), default_context(), "smg_dirac_refresh"); }

    void apply(const Vec& src, Vec& dst) const { run(SMG_OP_D, src, dst); }
    void apply_dag(const Vec& src, Vec& dst) const { run(SMG_OP_DDAG, src, dst); }
    void apply_DdagD(const Vec& src, Vec& dst) const { run(SMG_OP_DDAGD, src, dst); }
    void apply_g5D(const Vec& src, Vec& dst) const { run(SMG_OP_G5D, src, dst); }
    OpApply as_DdagD_op() const {
        return [this](const Vec& s, Vec& d) { apply_DdagD(s, d); };
    }
    smg_dirac* handle() const { return h_.get(); }

   private:
    void run(smg_operator op, const Vec& src, Vec& dst) const {
        DeviceField a(lat.L, 1), b(lat.L, 1);
        a.upload(src);
        check(smg_dirac_apply(h_.get(), op, a.get(), b.get()), default_context(), "smg_dirac_apply");
        dst.resize(src.size());
        b.download(dst);
    }
    std::unique_ptr<smg_dirac, smg_status (*)(smg_dirac*)> h_{nullptr, &smg_dirac_destroy};
};

struct CGResult {
    Vec solution;
    int iterations;
    double final_residual;
};
struct FCGResult {
    Vec solution;
    int iterations;
    double final_residual;
};

// cg_solve(A, n, rhs, max_iter, tol) with A = D^dag D of `D`
inline CGResult cg_solve(const DiracOp& D, int n, const Vec& rhs, int max_iter, double tol) {
    if (n != D.lat.ndof) throw Error(SMG_BAD_ARG, "cg_solve: n must be 2*V");
    DeviceField b(D.lat.L, 1), x(D.lat.L, 1);
    b.upload(rhs);
    smg_solve_result r{};
    smg_status s = smg_cg_solve(D.handle(), b.get(), x.get(), max_iter, tol, &r);
    if (s != SMG_OK && s != SMG_NOT_CONVERGED) check(s, default_context(), "smg_cg_solve");
    CGResult out{Vec(n), r.iterations, r.final_residual};
    x.download(out.solution);
    return out;
}

// mr_smooth(D, x, b, niter): x is the start vector and the result
inline void mr_smooth(const DiracOp& D, Vec& x, const Vec& b, int niter) {
    DeviceField fb(D.lat.L, 1), fx(D.lat.L, 1);
    fb.upload(b);
    fx.upload(x);
    check(smg_mr_smooth(D.handle(), fb.get(), fx.get(), niter), default_context(), "smg_mr_smooth");
    fx.download(x);
}

// richardson_smooth_op with A = D^dag D of `D`
inline void richardson_smooth(const DiracOp& D, Vec& x, const Vec& b, int niter, double omega) {
    DeviceField fb(D.lat.L, 1), fx(D.lat.L, 1);
    fb.upload(b);
    fx.upload(x);
    check(smg_richardson_smooth(D.handle(), fb.get(), fx.get(), niter, omega), default_context(),
          "smg_richardson_smooth");
    fx.download(x);
}

// estimate_lambda_max(A, n, niter) with A = D^dag D of `D`
inline double estimate_lambda_max(const DiracOp& D, int niter) {
    double l = 0;
    check(smg_estimate_lambda_max(D.handle(), niter, &l), default_context(), "smg_estimate_lambda_max");
    return l;
}

struct MGConfig {  // reference src/config.h:19-30
    int mg_levels = 2;
    int block_size = 4;
    int k_null = 4;
    int coarse_block = 0;  // 0 = 4 * k_null dofs, i.e. 4 coarse sites
    bool w_cycle = true;
    int pre_smooth = 3;
    int post_smooth = 3;
};

class MGHierarchy {
   public:
    MGHierarchy(const DiracOp& D, const smg_mg_params& p, const std::vector<Vec>* warm = nullptr) : D_(D) {
        std::vector<cx> flat;
        if (warm) {
            for (const Vec& v : *warm) flat.insert(flat.end(), v.begin(), v.end());
        }
        smg_mg* mg = nullptr;
        check(smg_mg_create(D.handle(), &p, warm ? reinterpret_cast<const double*>(flat.data()) : nullptr, &mg),
              default_context(), "smg_mg_create");
        h_.reset(mg);
    }
    Vec precondition(const Vec& b) {
        DeviceField fb(D_.lat.L, 1), fx(D_.lat.L, 1);
        fb.upload(b);
        check(smg_mg_precondition(h_.get(), fb.get(), fx.get()), default_context(), "smg_mg_precondition");
        Vec x(b.size());
        fx.download(x);
        return x;
    }
    // Richardson smoothing at omega = damping / lambda_max on every level but the coarsest
    void set_symmetric(double damping = 0.8) {
        check(smg_mg_set_symmetric(h_.get(), damping, nullptr), default_context(), "smg_mg_set_symmetric");
    }
    // MGHierarchy::rebuild_deeper_levels (src/multigrid.cpp:158-193) after the links changed
    void rebuild() { check(smg_mg_rebuild(h_.get()), default_context(), "smg_mg_rebuild"); }
    // the deflation part of setup_sparse_coarse (src/multigrid.cpp:754-794): TRLM eigenpairs of the
    // level-1 operator, the coarsest CG of a two-level hierarchy starting from the deflated guess
    smg_deflation_info setup_deflation(int n_defl, int n_kr = 0, int max_restarts = 100, double tol = 1e-10) {
        smg_deflation_info info{};
        const smg_status s = smg_mg_setup_deflation(h_.get(), n_defl, n_kr, max_restarts, tol, &info);
        if (s != SMG_NOT_CONVERGED) check(s, default_context(), "smg_mg_setup_deflation");
        return info;
    }
    // sparse_Ac.defl_vals / defl_vecs
    void deflation(std::vector<double>& vals, std::vector<Vec>& vecs) const {
        int n = 0;
        check(smg_mg_get_deflation(h_.get(), &n, nullptr, nullptr), default_context(), "smg_mg_get_deflation");
        int nx = 0, ny = 0, nd = 0;
        check(smg_mg_level_dims(h_.get(), 1, &nx, &ny, &nd), default_context(), "smg_mg_level_dims");
        const size_t dim = (size_t)nx * ny * nd;
        std::vector<cx> flat((size_t)n * dim);
        vals.resize(n);
        check(smg_mg_get_deflation(h_.get(), &n, vals.data(), reinterpret_cast<double*>(flat.data())),
              default_context(), "smg_mg_get_deflation");
        vecs.assign(n, Vec());
        for (int i = 0; i < n; ++i) vecs[i].assign(flat.begin() + i * dim, flat.begin() + (i + 1) * dim);
    }
    // evolve_coarse_deflation without forecasting (src/hmc_multiscale.cpp:278-331) after rebuild()
    double deflation_rr() {
        double r = 0;
        check(smg_mg_deflation_rr(h_.get(), &r), default_context(), "smg_mg_deflation_rr");
        return r;
    }
    // CoarseDeflState::lowmode_solution (src/hmc.h:312-323)
    Vec lowmode_solution(const Vec& phi) {
        DeviceField fb(D_.lat.L, 1), fx(D_.lat.L, 1);
        fb.upload(phi);
        check(smg_mg_lowmode_solution(h_.get(), fb.get(), fx.get()), default_context(), "smg_mg_lowmode_solution");
        Vec x(phi.size());
        fx.download(x);
        return x;
    }
    smg_mg* handle() const { return h_.get(); }

   private:
    const DiracOp& D_;
    std::unique_ptr<smg_mg, smg_status (*)(smg_mg*)> h_{nullptr, &smg_mg_destroy};
};

// build_full_mg(D, mcfg, scfg, rng, ...) with the rng given as its seed
inline std::unique_ptr<MGHierarchy> build_full_mg(const DiracOp& D, const MGConfig& mcfg, uint32_t seed,
                                                  const std::vector<Vec>* warm_start = nullptr) {
    smg_mg_params p;
    smg_mg_params_default(&p);
    p.n_levels = mcfg.mg_levels < 2 ? 2 : mcfg.mg_levels;
    p.block[0][0] = p.block[0][1] = mcfg.block_size;
    int cb = mcfg.coarse_block > 0 ? mcfg.coarse_block : 4 * mcfg.k_null;
    for (int l = 0; l < SMG_MAX_LEVELS - 1; ++l) {
        p.n_vec[l] = mcfg.k_null;
        if (l > 0) {
            p.block[l][0] = cb / mcfg.k_null;
            p.block[l][1] = 1;
        }
    }
    p.null_iters = warm_start ? 5 : 20;
    p.w_cycle = mcfg.w_cycle;
    p.pre_smooth = mcfg.pre_smooth;
    p.post_smooth = mcfg.post_smooth;
    p.seed = seed;
    return std::make_unique<MGHierarchy>(D, p, warm_start);
}

inline FCGResult fcg_solve_mg(const DiracOp& D, int n, const Vec& rhs, MGHierarchy& mg, int max_iter, double tol,
                              int truncation = 20) {
    if (n != D.lat.ndof) throw Error(SMG_BAD_ARG, "fcg_solve_mg: n must be 2*V");
    DeviceField b(D.lat.L, 1), x(D.lat.L, 1);
    b.upload(rhs);
    smg_solve_result r{};
    smg_status s = smg_gcr_solve(D.handle(), mg.handle(), b.get(), x.get(), max_iter, tol, truncation, 0, &r);
    if (s != SMG_OK && s != SMG_NOT_CONVERGED) check(s, default_context(), "smg_gcr_solve");
    FCGResult out{Vec(n), r.iterations, r.final_residual};
    x.download(out.solution);
    return out;
}

// cg_solve_precond / cg_solve_x0 / cg_solve_x0_precond (mg == nullptr: no
// preconditioner; x0 == nullptr or empty: start from zero)
inline CGResult cg_solve_x0_precond(const DiracOp& D, int n, const Vec& rhs, const Vec* x0, MGHierarchy* mg,
                                    int max_iter, double tol) {
    if (n != D.lat.ndof) throw Error(SMG_BAD_ARG, "cg_solve_precond: n must be 2*V");
    DeviceField b(D.lat.L, 1), x(D.lat.L, 1);
    b.upload(rhs);
    const bool use_x0 = x0 && !x0->empty();
    if (use_x0) x.upload(*x0);
    smg_solve_result r{};
    smg_status s = smg_cg_solve_precond(D.handle(), mg ? mg->handle() : nullptr, b.get(), x.get(), use_x0 ? 1 : 0,
                                        max_iter, tol, &r);
    if (s != SMG_OK && s != SMG_NOT_CONVERGED) check(s, default_context(), "smg_cg_solve_precond");
    CGResult out{Vec(n), r.iterations, r.final_residual};
    x.download(out.solution);
    return out;
}
inline CGResult cg_solve_precond(const DiracOp& D, int n, const Vec& rhs, MGHierarchy& mg, int max_iter,
                                 double tol) {
    return cg_solve_x0_precond(D, n, rhs, nullptr, &mg, max_iter, tol);
}
inline CGResult cg_solve_x0(const DiracOp& D, int n, const Vec& rhs, const Vec& x0, int max_iter, double tol) {
    return cg_solve_x0_precond(D, n, rhs, &x0, nullptr, max_iter, tol);
}

struct RitzPair {
    double value;
    Vec vector;  // not returned by the device solver: left empty
};
struct FGMRESResult {
    Vec solution;
    int iterations;
    double final_residual;
    std::vector<RitzPair> ritz_pairs;
};

inline FGMRESResult fgmres_solve_mg(const DiracOp& D, int n, const Vec& rhs, MGHierarchy* mg, int restart,
                                    int max_iter, double tol, int n_ritz_harvest = 4) {
    if (n != D.lat.ndof) throw Error(SMG_BAD_ARG, "fgmres_solve_mg: n must be 2*V");
    DeviceField b(D.lat.L, 1), x(D.lat.L, 1);
    b.upload(rhs);
    smg_solve_result r{};
    std::vector<double> vals(3 * (size_t)(n_ritz_harvest > 0 ? n_ritz_harvest : 1));
    int nr = 0;
    smg_status s = smg_fgmres_solve(D.handle(), mg ? mg->handle() : nullptr, b.get(), x.get(), restart, max_iter,
                                    tol, n_ritz_harvest, &r, vals.data(), &nr);
    if (s != SMG_OK && s != SMG_NOT_CONVERGED) check(s, default_context(), "smg_fgmres_solve");
    FGMRESResult out{Vec(n), r.iterations, r.true_residual, {}};
    x.download(out.solution);
    for (int i = 0; i < nr; ++i) out.ritz_pairs.push_back({vals[i], {}});
    return out;
}

// The pseudofermion action as a differentiable pair: forward solves
// X = (D^dag D)^-1 phi and returns S = Re <phi, X>; backward returns
// F = -dS/dtheta from the X kept by forward (chi = D X is recomputed).
class PseudofermionAction {
   public:
    PseudofermionAction(const DiracOp& D, MGHierarchy* mg = nullptr) : D_(D), mg_(mg), X_(D.lat.L, 1) {}
    double forward(const Vec& phi, int max_iter, double tol) {
        DeviceField fp(D_.lat.L, 1);
        fp.upload(phi);
        double S = 0;
        smg_solve_result r{};
        check(smg_fermion_action(D_.handle(), mg_ ? mg_->handle() : nullptr, fp.get(), X_.get(), max_iter, tol, &S,
                                 &r),
              default_context(), "smg_fermion_action");
        iterations = r.iterations;
        return S;
    }
    void backward(std::array<RVec, 2>& force) const {
        RVec flat(2 * (size_t)D_.lat.V);
        check(smg_fermion_force(D_.handle(), X_.get(), flat.data()), default_context(), "smg_fermion_force");
        force[0].assign(flat.begin(), flat.begin() + D_.lat.V);
        force[1].assign(flat.begin() + D_.lat.V, flat.end());
    }
    int iterations = 0;

   private:
    const DiracOp& D_;
    MGHierarchy* mg_;
    DeviceField X_;
};

inline void fermion_force(const DiracOp& D, const Vec& X, std::array<RVec, 2>& force) {
    DeviceField fx(D.lat.L, 1);
    fx.upload(X);
    RVec flat(2 * (size_t)D.lat.V);
    check(smg_fermion_force(D.handle(), fx.get(), flat.data()), default_context(), "smg_fermion_force");
    force[0].assign(flat.begin(), flat.begin() + D.lat.V);
    force[1].assign(flat.begin() + D.lat.V, flat.end());
}

// coarse_lowmode_force (src/hmc_multiscale.cpp:237-276) with mg's prolongator and deflation space
inline void coarse_lowmode_force(const DiracOp& D, MGHierarchy& mg, const Vec& phi, std::array<RVec, 2>& force,
                                 int smooth_iters = 0) {
    DeviceField fp(D.lat.L, 1);
    fp.upload(phi);
    RVec flat(2 * (size_t)D.lat.V);
    check(smg_coarse_lowmode_force(D.handle(), mg.handle(), fp.get(), smooth_iters, flat.data()), default_context(),
          "smg_coarse_lowmode_force");
    force[0].assign(flat.begin(), flat.begin() + D.lat.V);
    force[1].assign(flat.begin() + D.lat.V, flat.end());
}

inline void gauge_force(const GaugeField& g, double beta, std::array<RVec, 2>& force) {
    RVec flat(2 * (size_t)g.lat.V);
    check(smg_gauge_force(g.handle(), beta, flat.data()), default_context(), "smg_gauge_force");
    force[0].assign(flat.begin(), flat.begin() + g.lat.V);
    force[1].assign(flat.begin() + g.lat.V, flat.end());
}

inline double gauge_action(const GaugeField& g, double beta) {
    double v = 0;
    check(smg_gauge_action(g.handle(), beta, &v), default_context(), "smg_gauge_action");
    return v;
}

// verify_forces (src/hmc_forces.cpp:869-981): true when both forces pass; details in *check
inline bool verify_forces(const GaugeField& g, double beta, double mass, double wilson_r, int max_iter, double tol,
                          double c_sw = 0.0, bool use_eo = false, double err_threshold = 1e-4, double mu_t = 0.0,
                          smg_force_check* check_out = nullptr) {
    smg_force_check c{};
    check(smg_verify_forces(g.handle(), beta, mass, wilson_r, max_iter, tol, c_sw, use_eo ? 1 : 0, err_threshold,
                            mu_t, &c),
          default_context(), "smg_verify_forces");
    if (check_out) *check_out = c;
    return c.passed != 0;
}

// std::mt19937 with the reference's distributions, owned by the library (momenta, eta, Metropolis)
class Rng {
   public:
    explicit Rng(uint32_t seed) {
        smg_rng* r = nullptr;
        check(smg_rng_create(seed, &r), default_context(), "smg_rng_create");
        h_.reset(r);
    }
    smg_rng* get() const { return h_.get(); }

   private:
    std::unique_ptr<smg_rng, smg_status (*)(smg_rng*)> h_{nullptr, &smg_rng_destroy};
};

// hmc_trajectory (src/hmc_trajectory.cpp:38-235) on the device; g.U follows the device links
inline smg_hmc_result hmc_trajectory(GaugeField& g, double mass, double wilson_r, const smg_hmc_params& p, Rng& rng) {
    smg_hmc_result res{};
    check(smg_hmc_trajectory(g.handle(), mass, wilson_r, &p, rng.get(), &res), default_context(),
          "smg_hmc_trajectory");
    g.pull();
    return res;
}

// reversibility_test_plain (src/hmc_trajectory.cpp:416-509); the links are restored
inline smg_reversibility_result reversibility_test_plain(GaugeField& g, double mass, double wilson_r,
                                                         const smg_hmc_params& p, Rng& rng) {
    smg_reversibility_result res{};
    check(smg_hmc_reversibility(g.handle(), mass, wilson_r, &p, rng.get(), &res), default_context(),
          "smg_hmc_reversibility");
    return res;
}

// hmc_trajectory_mg_multiscale (src/hmc_multiscale.cpp:340-886): mg supplies the preconditioner, the
// prolongator and the deflation space and must be built on a DiracOp over g
inline smg_ms_result hmc_trajectory_mg_multiscale(GaugeField& g, double mass, double wilson_r,
                                                  const smg_ms_params& p, MGHierarchy& mg, Rng& rng) {
    smg_ms_result res{};
    check(smg_hmc_mg_multiscale(g.handle(), mass, wilson_r, &p, mg.handle(), rng.get(), &res), default_context(),
          "smg_hmc_mg_multiscale");
    g.pull();
    return res;
}

// reversibility_test_mg_multiscale (src/hmc_multiscale.cpp:963-1000); the links are restored
inline smg_reversibility_result reversibility_test_mg_multiscale(GaugeField& g, double mass, double wilson_r,
                                                                 const smg_ms_params& p, MGHierarchy& mg, Rng& rng) {
    smg_reversibility_result res{};
    check(smg_hmc_mg_multiscale_reversibility(g.handle(), mass, wilson_r, &p, mg.handle(), rng.get(), &res),
          default_context(), "smg_hmc_mg_multiscale_reversibility");
    return res;
}

}  // namespace smg
