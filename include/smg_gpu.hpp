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
//   cg_solve, cg_solve_x0, cg_solve_precond, cg_solve_x0_precond, fcg_solve,
//   fcg_solve_mg, fgmres_solve_generic, fgmres_solve_mg on OpApply
//                                           src/solvers.h:37-104
//   SolverConfig, build_full_mg(D, mcfg, scfg, rng, n_defl, verbose, warm)
//                                           src/config.h:33-40, src/mg_builder.h:6-11
//   Prolongator                             src/prolongator.h:14-142
//   SparseCoarseOp                          src/coarse_op.h:154-548
//   EvenOddDiracOp                          src/dirac.h:190-553
// An OpApply or preconditioner handed to the solvers must be one this header
// made (DiracOp::as_DdagD_op, MGHierarchy::as_precond): they name device
// objects, so the solve runs on the GPU.  Any other std::function is a host
// callback the device solvers cannot run; they throw smg::Error with
// SMG_UNSUPPORTED instead of falling back to the CPU.
// Host vectors keep the reference layout (Vec v[2*s + spin]); each call copies
// them to the device, runs the sm_103a kernels and copies results back.
// Failures throw smg::Error carrying the smg_status, where the reference
// asserts or prints a warning.
#pragma once

#include <array>
#include <complex>
#include <functional>
#include <memory>
#include <random>
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

struct Lattice {  // src/lattice.h:4-42
    int L, V, ndof, V_half;
    std::vector<int> even_sites;  // global index of the i-th even site ((x + y) % 2 == 0), lexicographic
    std::vector<int> odd_sites;
    std::vector<int> eo_index;  // index of a site within its parity's list
    explicit Lattice(int L_) : L(L_), V(L_ * L_), ndof(2 * L_ * L_), V_half(L_ * L_ / 2) {
        eo_index.resize(V);
        for (int s = 0; s < V; ++s) {
            std::vector<int>& list = parity(s) == 0 ? even_sites : odd_sites;
            eo_index[s] = (int)list.size();
            list.push_back(s);
        }
    }
    int idx(int x, int y) const { return ((x % L + L) % L) + L * ((y % L + L) % L); }
    int xp(int s) const { return idx(s % L + 1, s / L); }
    int xm(int s) const { return idx(s % L - 1, s / L); }
    int yp(int s) const { return idx(s % L, s / L + 1); }
    int ym(int s) const { return idx(s % L, s / L - 1); }
    int parity(int s) const { return ((s % L) + (s / L)) % 2; }
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

class DiracOp;

// The OpApply DiracOp::as_DdagD_op returns: A = D^dag D of a device operator.
struct DdagDOp {
    const DiracOp* D;
    void operator()(const Vec& src, Vec& dst) const;
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
    // DiracOp::as_DdagD_op (src/dirac.h:177): an OpApply the device solvers recognise
    OpApply as_DdagD_op() const { return DdagDOp{this}; }
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

inline void DdagDOp::operator()(const Vec& src, Vec& dst) const { D->apply_DdagD(src, dst); }

// The device operator behind an OpApply made by as_DdagD_op; anything else is a host callback.
inline const DiracOp& device_operator(const OpApply& A, const char* where) {
    if (const DdagDOp* t = A.target<DdagDOp>()) return *t->D;
    throw Error(SMG_UNSUPPORTED, std::string(where) +
                                     ": the operator must be DiracOp::as_DdagD_op(); host callbacks do not run on "
                                     "the device solvers");
}

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

struct SolverConfig {  // reference src/config.h:33-40
    double tol = 1e-10;
    int krylov = 30;
    int max_iter = 300;
    std::string eigensolver = "trlm";
    double feast_emax = 0.0;
    int n_defl = 0;
};

class MGHierarchy;

// The preconditioner MGHierarchy::as_precond returns (one MG cycle, MGHierarchy::precondition).
struct MGPrecond {
    MGHierarchy* mg;
    Vec operator()(const Vec& v) const;
};

// Move-only: the hierarchy owns device memory.  The reference's MGHierarchy copies (and then needs
// rebind_prolongator_lambdas); here a copy would be a second device hierarchy, so it is not offered.
class MGHierarchy {
   public:
    // built from caller-drawn start vectors: starts[l] holds the n_vec[l] start vectors of level l
    MGHierarchy(const DiracOp& D, const smg_mg_params& p, const std::vector<std::vector<Vec>>& starts) : D_(D) {
        std::vector<std::vector<cx>> flat(starts.size());
        std::vector<const double*> ptrs(starts.size(), nullptr);
        for (size_t l = 0; l < starts.size(); ++l) {
            for (const Vec& v : starts[l]) flat[l].insert(flat[l].end(), v.begin(), v.end());
            ptrs[l] = reinterpret_cast<const double*>(flat[l].data());
        }
        smg_mg* mg = nullptr;
        check(smg_mg_create_from_starts(D.handle(), &p, ptrs.data(), &mg), default_context(),
              "smg_mg_create_from_starts");
        h_.reset(mg);
    }
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
    // MGHierarchy::null_vecs_l0 (src/multigrid.h:50): the level-0 near-null vectors
    std::vector<Vec> null_vectors() const {
        int nx = 0, ny = 0, nd = 0;
        check(smg_mg_level_dims(h_.get(), 1, &nx, &ny, &nd), default_context(), "smg_mg_level_dims");
        const size_t n = (size_t)D_.lat.ndof;
        int k = 0;
        check(smg_mg_n_null_vectors(h_.get(), &k), default_context(), "smg_mg_n_null_vectors");
        std::vector<cx> flat((size_t)k * n);
        check(smg_mg_null_vectors(h_.get(), reinterpret_cast<double*>(flat.data())), default_context(),
              "smg_mg_null_vectors");
        std::vector<Vec> out(k);
        for (int i = 0; i < k; ++i) out[i].assign(flat.begin() + i * n, flat.begin() + (i + 1) * n);
        return out;
    }
    // the preconditioner std::function the reference's solvers take, recognised by the device solvers
    std::function<Vec(const Vec&)> as_precond() { return MGPrecond{this}; }
    smg_mg* handle() const { return h_.get(); }
    const DiracOp& dirac() const { return D_; }

   private:
    const DiracOp& D_;
    std::unique_ptr<smg_mg, smg_status (*)(smg_mg*)> h_{nullptr, &smg_mg_destroy};
};

inline Vec MGPrecond::operator()(const Vec& v) const { return mg->precondition(v); }

// The hierarchy behind a preconditioner made by as_precond (nullptr for an empty std::function, which
// means no preconditioner); anything else is a host callback.
inline MGHierarchy* device_precond(const std::function<Vec(const Vec&)>& M, const char* where) {
    if (!M) return nullptr;
    if (const MGPrecond* t = M.target<MGPrecond>()) return t->mg;
    throw Error(SMG_UNSUPPORTED, std::string(where) +
                                     ": the preconditioner must be MGHierarchy::as_precond(); host callbacks do not "
                                     "run on the device solvers");
}

// random_vec (src/linalg.cpp:44-48): each entry draws its imaginary part and then its real part from
// N(0, 1), the order GCC on x86-64 gives the reference's cx(dist(rng), dist(rng))
inline Vec random_vec(int n, std::mt19937& rng) {
    std::normal_distribution<double> dist(0.0, 1.0);
    Vec v(n);
    for (int i = 0; i < n; ++i) {
        const double im = dist(rng);
        const double re = dist(rng);
        v[i] = cx(re, im);
    }
    return v;
}

// build_full_mg (src/mg_builder.cpp:3-31): build_mg_hierarchy with the start vectors drawn from the
// caller's generator in the reference's order (level 0 unless warm_start, then every deeper level),
// null_iters = 20 (5 with warm_start), the reference's coarse blocking of resolved_coarse_block()
// consecutive coarse dofs as a (cb / k_null) x 1 aggregate, the coarsest level solved by CG to
// 1e-12 (at most 200 iterations), and with n_defl > 0 the TRLM deflation of the level-1 operator
// (setup_sparse_coarse, src/multigrid.cpp:754-794).  The FEAST null-space option is not available.
inline MGHierarchy build_full_mg(const DiracOp& D, const MGConfig& mcfg, const SolverConfig& scfg, std::mt19937& rng,
                                 int n_defl = 0, bool verbose = true, const std::vector<Vec>* warm_start = nullptr) {
    (void)verbose;
    if (scfg.eigensolver == "feast") throw Error(SMG_UNSUPPORTED, "build_full_mg: the FEAST null space is not built");
    const int levels = mcfg.mg_levels < 2 ? 2 : mcfg.mg_levels;
    const int cb = mcfg.coarse_block > 0 ? mcfg.coarse_block : 4 * mcfg.k_null;
    if (cb % mcfg.k_null) throw Error(SMG_UNSUPPORTED, "build_full_mg: coarse_block must be a multiple of k_null");
    smg_mg_params p;
    smg_mg_params_default(&p);
    p.n_levels = levels;
    p.block[0][0] = p.block[0][1] = mcfg.block_size;
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
    p.coarse_max_iter = 200;
    p.coarse_tol = 1e-12;
    std::vector<std::vector<Vec>> starts(levels - 1);
    int dim = D.lat.ndof, nx = D.lat.L, ny = D.lat.L;
    for (int l = 0; l < levels - 1; ++l) {
        if (l == 0 && warm_start) {
            starts[0] = *warm_start;
        } else {
            for (int i = 0; i < mcfg.k_null; ++i) starts[l].push_back(random_vec(dim, rng));
        }
        nx /= p.block[l][0];
        ny /= p.block[l][1];
        dim = nx * ny * mcfg.k_null;
    }
    MGHierarchy mg(D, p, starts);
    if (n_defl > 0) mg.setup_deflation(n_defl, 0, 100, 1e-10);
    return mg;
}

// build_full_mg with the generator given as its seed (the library draws the start vectors)
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

// ---- the reference's solver signatures on OpApply (src/solvers.h:37-104).  A must come from
// DiracOp::as_DdagD_op() and a preconditioner from MGHierarchy::as_precond() (an empty
// std::function: none); other callables are host code and make these throw SMG_UNSUPPORTED.
inline CGResult cg_solve(const OpApply& A, int n, const Vec& rhs, int max_iter, double tol) {
    return cg_solve(device_operator(A, "cg_solve"), n, rhs, max_iter, tol);
}
inline CGResult cg_solve_x0(const OpApply& A, int n, const Vec& rhs, const Vec& x0, int max_iter, double tol) {
    return cg_solve_x0_precond(device_operator(A, "cg_solve_x0"), n, rhs, &x0, nullptr, max_iter, tol);
}
inline CGResult cg_solve_precond(const OpApply& A, int n, const Vec& rhs, const std::function<Vec(const Vec&)>& precond,
                                 int max_iter, double tol) {
    return cg_solve_x0_precond(device_operator(A, "cg_solve_precond"), n, rhs, nullptr,
                               device_precond(precond, "cg_solve_precond"), max_iter, tol);
}
inline CGResult cg_solve_x0_precond(const OpApply& A, int n, const Vec& rhs, const Vec& x0,
                                    const std::function<Vec(const Vec&)>& precond, int max_iter, double tol) {
    return cg_solve_x0_precond(device_operator(A, "cg_solve_x0_precond"), n, rhs, &x0,
                               device_precond(precond, "cg_solve_x0_precond"), max_iter, tol);
}
// fcg_solve (src/solvers.cpp:223-300): truncated GCR; the device solver takes the MG preconditioner
inline FCGResult fcg_solve(const OpApply& A, int n, const Vec& rhs, const std::function<Vec(const Vec&)>& precond,
                           int max_iter, double tol, int trunc = 30) {
    MGHierarchy* mg = device_precond(precond, "fcg_solve");
    if (!mg) throw Error(SMG_UNSUPPORTED, "fcg_solve: the device GCR needs an MG preconditioner (as_precond)");
    return fcg_solve_mg(device_operator(A, "fcg_solve"), n, rhs, *mg, max_iter, tol, trunc);
}
inline FCGResult fcg_solve_mg(const OpApply& A, int n, const Vec& rhs, MGHierarchy& mg, int max_iter, double tol,
                              int truncation = 20) {
    return fcg_solve_mg(device_operator(A, "fcg_solve_mg"), n, rhs, mg, max_iter, tol, truncation);
}
inline FGMRESResult fgmres_solve_generic(const OpApply& A, int n, const Vec& rhs,
                                         const std::function<Vec(const Vec&)>& precond, int restart, int max_iter,
                                         double tol, int n_ritz_harvest = 4) {
    return fgmres_solve_mg(device_operator(A, "fgmres_solve_generic"), n, rhs,
                           device_precond(precond, "fgmres_solve_generic"), restart, max_iter, tol, n_ritz_harvest);
}
inline FGMRESResult fgmres_solve_mg(const OpApply& A, int n, const Vec& rhs, MGHierarchy& mg, int restart,
                                    int max_iter, double tol, int n_ritz_harvest = 4) {
    return fgmres_solve_mg(device_operator(A, "fgmres_solve_mg"), n, rhs, &mg, restart, max_iter, tol,
                           n_ritz_harvest);
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

// Prolongator (src/prolongator.h:14-142): geometric bx x by blocks, k_vec block vectors per block.
// build_from_vectors cuts the null vectors to blocks and orthonormalises them on the device;
// block_vecs then holds a host copy [block][k][2 * (lx + bx * ly) + spin].
class Prolongator {
   public:
    const Lattice& lat;
    int bx, by, nbx, nby, nblocks, k_vec, coarse_dim;
    std::vector<std::vector<Vec>> block_vecs;

    Prolongator(const Lattice& lat_, int bx_, int by_, int k_)
        : lat(lat_), bx(bx_), by(by_), nbx(lat_.L / bx_), nby(lat_.L / by_), nblocks(nbx * nby), k_vec(k_),
          coarse_dim(nblocks * k_) {
        if (lat.L % bx || lat.L % by) throw Error(SMG_BAD_ARG, "Prolongator: blocks must divide L");
        block_vecs.assign(nblocks, std::vector<Vec>(k_vec));
    }
    int block_fine_dim() const { return 2 * bx * by; }
    void build_from_vectors(const std::vector<Vec>& null_vecs) {
        if ((int)null_vecs.size() < k_vec) throw Error(SMG_BAD_ARG, "build_from_vectors: fewer than k vectors");
        std::vector<cx> flat;
        for (int i = 0; i < k_vec; ++i) flat.insert(flat.end(), null_vecs[i].begin(), null_vecs[i].end());
        smg_prolongator* P = nullptr;
        check(smg_prolongator_create(default_context(), lat.L, bx, by, k_vec, reinterpret_cast<const double*>(flat.data()),
                                     &P),
              default_context(), "smg_prolongator_create");
        h_.reset(P);
        std::vector<cx> bv((size_t)nblocks * k_vec * block_fine_dim());
        check(smg_prolongator_get_block_vecs(P, reinterpret_cast<double*>(bv.data())), default_context(),
              "smg_prolongator_get_block_vecs");
        for (int b = 0; b < nblocks; ++b)
            for (int k = 0; k < k_vec; ++k) {
                auto it = bv.begin() + ((size_t)b * k_vec + k) * block_fine_dim();
                block_vecs[b][k].assign(it, it + block_fine_dim());
            }
    }
    Vec prolong(const Vec& coarse) const {
        Vec fine(lat.ndof);
        check(smg_prolongator_prolong(handle(), reinterpret_cast<const double*>(coarse.data()),
                                      reinterpret_cast<double*>(fine.data())),
              default_context(), "smg_prolongator_prolong");
        return fine;
    }
    Vec restrict_vec(const Vec& fine) const {
        Vec coarse(coarse_dim);
        check(smg_prolongator_restrict(handle(), reinterpret_cast<const double*>(fine.data()),
                                       reinterpret_cast<double*>(coarse.data())),
              default_context(), "smg_prolongator_restrict");
        return coarse;
    }
    smg_prolongator* handle() const {
        if (!h_) throw Error(SMG_BAD_ARG, "Prolongator: build_from_vectors first");
        return h_.get();
    }

   private:
    std::unique_ptr<smg_prolongator, smg_status (*)(smg_prolongator*)> h_{nullptr, &smg_prolongator_destroy};
};

// SparseCoarseOp (src/coarse_op.h:154-548): the 9-point Galerkin operator P^dag A P on the coarse
// lattice, A = D^dag D given as DiracOp::as_DdagD_op().
class SparseCoarseOp {
   public:
    int nbx = 0, nby = 0, nblocks = 0, k_vec = 0, dim = 0;
    static constexpr int N_DIR = 9;

    void build(const Prolongator& P, const OpApply& A, int fine_dim) {
        const DiracOp& D = device_operator(A, "SparseCoarseOp::build");
        if (fine_dim != D.lat.ndof) throw Error(SMG_BAD_ARG, "SparseCoarseOp::build: fine_dim must be 2V");
        smg_coarse_op* op = nullptr;
        check(smg_coarse_op_create(P.handle(), D.handle(), &op), default_context(), "smg_coarse_op_create");
        h_.reset(op);
        nbx = P.nbx;
        nby = P.nby;
        nblocks = P.nblocks;
        k_vec = P.k_vec;
        dim = nblocks * k_vec;
    }
    // the neighbour of block b in direction dir (0 self, 1 +x, 2 -x, 3 +y, 4 -y, 5 +x+y, 6 +x-y,
    // 7 -x+y, 8 -x-y; src/coarse_op.h:205-222)
    int neighbour(int b, int dir) const {
        static constexpr int dx[] = {0, 1, -1, 0, 0, 1, 1, -1, -1}, dy[] = {0, 0, 0, 1, -1, 1, -1, 1, -1};
        return (b % nbx + dx[dir] + nbx) % nbx + ((b / nbx + dy[dir] + nby) % nby) * nbx;
    }
    static int reverse_dir(int dir) {
        static constexpr int rev[] = {0, 2, 1, 4, 3, 8, 7, 6, 5};
        return rev[dir];
    }
    // link[block][dir]: k_vec x k_vec matrices, row-major [ki * k_vec + kj]
    std::vector<std::array<Vec, N_DIR>> links() const {
        std::vector<cx> flat((size_t)nblocks * N_DIR * k_vec * k_vec);
        check(smg_coarse_op_get_links(handle(), reinterpret_cast<double*>(flat.data())), default_context(),
              "smg_coarse_op_get_links");
        std::vector<std::array<Vec, N_DIR>> out(nblocks);
        const size_t kk = (size_t)k_vec * k_vec;
        for (int b = 0; b < nblocks; ++b)
            for (int d = 0; d < N_DIR; ++d) out[b][d].assign(flat.begin() + (b * N_DIR + d) * kk,
                                                             flat.begin() + (b * N_DIR + d + 1) * kk);
        return out;
    }
    void apply_to(const Vec& src, Vec& dst) const {
        dst.resize(dim);
        check(smg_coarse_op_apply(handle(), reinterpret_cast<const double*>(src.data()),
                                  reinterpret_cast<double*>(dst.data())),
              default_context(), "smg_coarse_op_apply");
    }
    Vec apply(const Vec& src) const {
        Vec dst;
        apply_to(src, dst);
        return dst;
    }
    void setup_deflation(int n_ev, int n_kr = 0, int max_restarts = 100, double tol = 1e-10,
                         const std::string& solver = "trlm", double feast_emax = 0.0) {
        (void)feast_emax;
        if (solver != "trlm") throw Error(SMG_UNSUPPORTED, "SparseCoarseOp::setup_deflation: only TRLM is built");
        smg_deflation_info info{};
        const smg_status s = smg_coarse_op_setup_deflation(handle(), n_ev, n_kr, max_restarts, tol, &info);
        if (s != SMG_NOT_CONVERGED) check(s, default_context(), "smg_coarse_op_setup_deflation");
    }
    Vec solve(const Vec& b, int max_iter = 200, double cg_tol = 1e-12) const {
        Vec x(dim);
        const smg_status s = smg_coarse_op_solve(handle(), reinterpret_cast<const double*>(b.data()),
                                                 reinterpret_cast<double*>(x.data()), max_iter, cg_tol);
        if (s != SMG_NOT_CONVERGED) check(s, default_context(), "smg_coarse_op_solve");
        return x;
    }
    smg_coarse_op* handle() const {
        if (!h_) throw Error(SMG_BAD_ARG, "SparseCoarseOp: build first");
        return h_.get();
    }

   private:
    std::unique_ptr<smg_coarse_op, smg_status (*)(smg_coarse_op*)> h_{nullptr, &smg_coarse_op_destroy};
};

// EvenOddDiracOp (src/dirac.h:190-553) on host half vectors: a half vector holds 2 * V/2 complex
// values in the order of lat.even_sites / lat.odd_sites.
class EvenOddDiracOp {
   public:
    const DiracOp& D;
    const Lattice& lat;
    explicit EvenOddDiracOp(const DiracOp& D_) : D(D_), lat(D_.lat) {}

    void apply_eo(const Vec& src_e, Vec& dst_o) const { dst_o = run(SMG_EO_HOP_EO, &src_e, nullptr, 1); }
    void apply_oe(const Vec& src_o, Vec& dst_e) const { dst_e = run(SMG_EO_HOP_OE, nullptr, &src_o, 0); }
    void apply_schur(const Vec& src_o, Vec& dst_o) const { dst_o = run(SMG_EO_SCHUR, nullptr, &src_o, 1); }
    void apply_schur_dag(const Vec& src_o, Vec& dst_o) const { dst_o = run(SMG_EO_SCHUR_DAG, nullptr, &src_o, 1); }
    void apply_schur_dag_schur(const Vec& src_o, Vec& dst_o) const {
        dst_o = run(SMG_EO_SCHUR_DAG_SCHUR, nullptr, &src_o, 1);
    }
    Vec scatter(const Vec& half_e, const Vec& half_o) const {
        Vec full(lat.ndof, 0.0);
        for (int i = 0; i < lat.V_half; ++i) {
            if (!half_e.empty()) {
                full[2 * lat.even_sites[i]] = half_e[2 * i];
                full[2 * lat.even_sites[i] + 1] = half_e[2 * i + 1];
            }
            if (!half_o.empty()) {
                full[2 * lat.odd_sites[i]] = half_o[2 * i];
                full[2 * lat.odd_sites[i] + 1] = half_o[2 * i + 1];
            }
        }
        return full;
    }
    Vec gather_even(const Vec& full) const { return gather(full, lat.even_sites); }
    Vec gather_odd(const Vec& full) const { return gather(full, lat.odd_sites); }
    // full solution from x_o: x_e = -D_ee^-1 D_oe x_o (reconstruct_full) or D_ee^-1 (phi_e - D_oe x_o)
    Vec reconstruct_full(const Vec& x_o) const { return reconstruct_impl(x_o, nullptr); }
    Vec reconstruct(const Vec& x_o, const Vec& phi) const { return reconstruct_impl(x_o, &phi); }
    double log_det_ee() const {
        double v = 0;
        check(smg_eo_logdet_ee(D.handle(), &v), default_context(), "smg_eo_logdet_ee");
        return v;
    }

   private:
    Vec gather(const Vec& full, const std::vector<int>& sites) const {
        Vec h(2 * (size_t)lat.V_half);
        for (int i = 0; i < lat.V_half; ++i) {
            h[2 * i] = full[2 * sites[i]];
            h[2 * i + 1] = full[2 * sites[i] + 1];
        }
        return h;
    }
    Vec run(smg_eo_operator op, const Vec* half_e, const Vec* half_o, int out_odd) const {
        DeviceField a(lat.L, 1), b(lat.L, 1);
        a.upload(scatter(half_e ? *half_e : Vec(), half_o ? *half_o : Vec()));
        check(smg_eo_apply(D.handle(), op, a.get(), b.get()), default_context(), "smg_eo_apply");
        Vec full(lat.ndof);
        b.download(full);
        return out_odd ? gather_odd(full) : gather_even(full);
    }
    Vec reconstruct_impl(const Vec& x_o, const Vec* phi) const {
        DeviceField fx(lat.L, 1), fp(lat.L, 1);
        fx.upload(scatter(Vec(), x_o));
        if (phi) fp.upload(*phi);
        check(smg_eo_reconstruct(D.handle(), phi ? fp.get() : nullptr, fx.get()), default_context(),
              "smg_eo_reconstruct");
        Vec full(lat.ndof);
        fx.download(full);
        return full;
    }
};

}  // namespace smg
