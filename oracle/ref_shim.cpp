// ORACLE TEST INFRASTRUCTURE — not part of the product.
//
// A thin extern "C" shim over the reference's own C++ sources, compiled from
// the reference tree (see oracle/Makefile) into oracle/_ref/libsmg_ref.so.
// Tests and the benchmark's CPU-baseline leg call it through ctypes to obtain
// the reference's results on the same seeded inputs as the GPU path.  Every
// function below constructs the reference objects (Lattice, GaugeField,
// DiracOp, MGHierarchy, ...) and calls the reference routine named in its
// comment; nothing here re-implements reference arithmetic.
//
// Array conventions: complex numbers are interleaved doubles; a gauge field
// is U[mu][s] (2*V complex), a spinor is v[2*s+spin] (2*V complex), a force
// is F[mu][s] (2*V doubles).
#include <array>
#include <complex>
#include <cstring>
#include <random>
#include <vector>

#include "types.h"
#include "lattice.h"
#include "gauge.h"
#include "dirac.h"
#include "linalg.h"
#include "smoother.h"
#include "prolongator.h"
#include "coarse_op.h"
#include "multigrid.h"
#include "mg_builder.h"
#include "solvers.h"
#include "hmc.h"

namespace {

struct World {
    Lattice lat;
    GaugeField g;
    World(int L, const double* U) : lat(L), g(lat) {
        for (int mu = 0; mu < 2; ++mu)
            for (int s = 0; s < lat.V; ++s) g.U[mu][s] = cx(U[2 * (mu * lat.V + s)], U[2 * (mu * lat.V + s) + 1]);
    }
};

Vec to_vec(const double* p, int n) {
    Vec v(n);
    for (int i = 0; i < n; ++i) v[i] = cx(p[2 * i], p[2 * i + 1]);
    return v;
}
void from_vec(const Vec& v, double* p) {
    for (size_t i = 0; i < v.size(); ++i) {
        p[2 * i] = v[i].real();
        p[2 * i + 1] = v[i].imag();
    }
}

}  // namespace

extern "C" {

void ref_set_verbosity(int v) { g_verbosity = v; }

// random_vec (src/linalg.cpp:44-48): k vectors drawn one after another from
// one std::mt19937(seed)
void ref_random_vecs(int k, int n, unsigned seed, double* out) {
    std::mt19937 rng(seed);
    for (int i = 0; i < k; ++i) from_vec(random_vec(n, rng), out + (size_t)2 * n * i);
}

// DiracOp::compute_clover_field (src/dirac.h:26-52)
void ref_clover(int L, const double* U, double* F01) {
    World w(L, U);
    DiracOp D(w.lat, w.g, 0.0, 1.0, 1.0, 0.0);
    for (int s = 0; s < w.lat.V; ++s) F01[s] = D.clover_field[s];
}

// GaugeField::avg_plaq (src/gauge.h:32-36)
double ref_avg_plaq(int L, const double* U) {
    World w(L, U);
    return w.g.avg_plaq();
}

// op: 0 apply (dirac.h:115), 1 apply_dag (:120), 2 apply_DdagD (:136), 3 apply_g5D (:145)
void ref_dirac(int L, const double* U, double m, double r, double csw, double mu, int op, const double* src,
               double* dst) {
    World w(L, U);
    DiracOp D(w.lat, w.g, m, r, csw, mu);
    Vec s = to_vec(src, w.lat.ndof), d(w.lat.ndof);
    switch (op) {
        case 0: D.apply(s, d); break;
        case 1: D.apply_dag(s, d); break;
        case 2: D.apply_DdagD(s, d); break;
        default: D.apply_g5D(s, d); break;
    }
    from_vec(d, dst);
}

// cg_solve on D^dag D (src/solvers.cpp:75-78)
int ref_cg(int L, const double* U, double m, double r, double csw, double mu, const double* b, double* x,
           int max_iter, double tol, double* final_res) {
    World w(L, U);
    DiracOp D(w.lat, w.g, m, r, csw, mu);
    OpApply A = [&D](const Vec& s, Vec& d) { D.apply_DdagD(s, d); };
    CGResult res = cg_solve(A, w.lat.ndof, to_vec(b, w.lat.ndof), max_iter, tol);
    from_vec(res.solution, x);
    if (final_res) *final_res = res.final_residual;
    return res.iterations;
}

// gauge_force / gauge_action (src/hmc_forces.cpp:80-111)
void ref_gauge_force(int L, const double* U, double beta, double* F) {
    World w(L, U);
    std::array<RVec, 2> f;
    gauge_force(w.g, beta, f);
    for (int mu = 0; mu < 2; ++mu) std::memcpy(F + (size_t)mu * w.lat.V, f[mu].data(), sizeof(double) * w.lat.V);
}
double ref_gauge_action(int L, const double* U, double beta) {
    World w(L, U);
    return gauge_action(w.g, beta);
}

// fermion_force (src/hmc_forces.cpp:134-139)
void ref_fermion_force(int L, const double* U, double m, double r, double csw, double mu, const double* X,
                       double* F) {
    World w(L, U);
    DiracOp D(w.lat, w.g, m, r, csw, mu);
    std::array<RVec, 2> f;
    fermion_force(D, to_vec(X, w.lat.ndof), f);
    for (int mu_ = 0; mu_ < 2; ++mu_) std::memcpy(F + (size_t)mu_ * w.lat.V, f[mu_].data(), sizeof(double) * w.lat.V);
}

// verify_forces (src/hmc_forces.cpp:869-981); returns 1 on PASS
int ref_verify_forces(int L, const double* U, double beta, double m, double r, double csw, double mu, int max_iter,
                      double tol, int use_eo) {
    World w(L, U);
    return verify_forces(w.g, beta, m, r, max_iter, tol, csw, use_eo != 0, 1e-4, mu) ? 1 : 0;
}

// mr_smooth (src/smoother.cpp:9-23): x is updated in place
void ref_mr_smooth(int L, const double* U, double m, double r, double csw, double mu, const double* b, double* x,
                   int niter) {
    World w(L, U);
    DiracOp D(w.lat, w.g, m, r, csw, mu);
    Vec xv = to_vec(x, w.lat.ndof);
    mr_smooth(D, xv, to_vec(b, w.lat.ndof), niter);
    from_vec(xv, x);
}

// compute_near_null_space (src/multigrid.cpp:435-484), rng = std::mt19937(seed)
void ref_near_null_space(int L, const double* U, double m, double r, double csw, double mu, int k, int iters,
                         unsigned seed, double* out) {
    World w(L, U);
    DiracOp D(w.lat, w.g, m, r, csw, mu);
    std::mt19937 rng(seed);
    auto nv = compute_near_null_space(D, k, iters, rng);
    for (int i = 0; i < k; ++i) from_vec(nv[i], out + (size_t)2 * w.lat.ndof * i);
}

// Prolongator::build_from_vectors (src/prolongator.h:133-141); block_vecs out
// as [b][k][2*bx*by] complex
void ref_prolongator_build(int L, int bs, int k, const double* null_vecs, double* block_vecs) {
    Lattice lat(L);
    Prolongator P(lat, bs, bs, k);
    std::vector<Vec> nv(k);
    for (int i = 0; i < k; ++i) nv[i] = to_vec(null_vecs + (size_t)2 * lat.ndof * i, lat.ndof);
    P.build_from_vectors(nv);
    int bd = P.block_fine_dim();
    for (int b = 0; b < P.nblocks; ++b)
        for (int i = 0; i < k; ++i) from_vec(P.block_vecs[b][i], block_vecs + (size_t)2 * bd * (b * k + i));
}

static Prolongator make_P(const Lattice& lat, int bs, int k, const double* block_vecs) {
    Prolongator P(lat, bs, bs, k);
    int bd = P.block_fine_dim();
    for (int b = 0; b < P.nblocks; ++b)
        for (int i = 0; i < k; ++i) P.block_vecs[b][i] = to_vec(block_vecs + (size_t)2 * bd * (b * k + i), bd);
    return P;
}

// Prolongator::prolong / restrict_vec (src/prolongator.h:77-108)
void ref_prolong(int L, int bs, int k, const double* block_vecs, const double* coarse, double* fine) {
    Lattice lat(L);
    Prolongator P = make_P(lat, bs, k, block_vecs);
    from_vec(P.prolong(to_vec(coarse, P.coarse_dim)), fine);
}
void ref_restrict(int L, int bs, int k, const double* block_vecs, const double* fine, double* coarse) {
    Lattice lat(L);
    Prolongator P = make_P(lat, bs, k, block_vecs);
    from_vec(P.restrict_vec(to_vec(fine, lat.ndof)), coarse);
}

// SparseCoarseOp::build with A = D^dag D (src/coarse_op.h:241-279); links out as
// [block][dir][ki*k + kj] complex
void ref_sparse_coarse_build(int L, const double* U, double m, double r, double csw, double mu, int bs, int k,
                             const double* block_vecs, double* links) {
    World w(L, U);
    DiracOp D(w.lat, w.g, m, r, csw, mu);
    Prolongator P = make_P(w.lat, bs, k, block_vecs);
    SparseCoarseOp Ac;
    OpApply A = [&D](const Vec& s, Vec& d) { D.apply_DdagD(s, d); };
    Ac.build(P, A, w.lat.ndof);
    for (int b = 0; b < Ac.nblocks; ++b)
        for (int d = 0; d < SparseCoarseOp::N_DIR; ++d)
            from_vec(Ac.link[b][d], links + (size_t)2 * k * k * (b * SparseCoarseOp::N_DIR + d));
}

// SparseCoarseOp::apply_to (src/coarse_op.h:282-297)
void ref_sparse_coarse_apply(int nbx, int nby, int k, const double* links, const double* src, double* dst) {
    SparseCoarseOp Ac;
    Ac.nbx = nbx;
    Ac.nby = nby;
    Ac.nblocks = nbx * nby;
    Ac.k_vec = k;
    Ac.dim = Ac.nblocks * k;
    Ac.link.resize(Ac.nblocks);
    for (int b = 0; b < Ac.nblocks; ++b)
        for (int d = 0; d < SparseCoarseOp::N_DIR; ++d)
            Ac.link[b][d] = to_vec(links + (size_t)2 * k * k * (b * SparseCoarseOp::N_DIR + d), k * k);
    Vec out;
    Ac.apply_to(to_vec(src, Ac.dim), out);
    from_vec(out, dst);
}

// CoarseOp::build (dense Galerkin by probing, src/coarse_op.h:40-43); mat out
// column-major [j][i] complex
void ref_dense_coarse_build(int L, const double* U, double m, double r, double csw, double mu, int bs, int k,
                            const double* block_vecs, double* mat) {
    World w(L, U);
    DiracOp D(w.lat, w.g, m, r, csw, mu);
    Prolongator P = make_P(w.lat, bs, k, block_vecs);
    CoarseOp Ac;
    Ac.build(D, P);
    for (int j = 0; j < Ac.dim; ++j) from_vec(Ac.mat[j], mat + (size_t)2 * Ac.dim * j);
}

struct RefMGParams {
    int levels, block_size, k_null, coarse_block, null_iters, w_cycle, pre_smooth, post_smooth, n_defl;
};

static MGHierarchy ref_build(const DiracOp& D, const RefMGParams& p, unsigned seed,
                             const std::vector<Vec>* warm) {
    MGConfig mc;
    mc.mg_levels = p.levels;
    mc.block_size = p.block_size;
    mc.k_null = p.k_null;
    mc.coarse_block = p.coarse_block;
    mc.w_cycle = p.w_cycle != 0;
    mc.pre_smooth = p.pre_smooth;
    mc.post_smooth = p.post_smooth;
    std::mt19937 rng(seed);
    MGHierarchy mg = build_mg_hierarchy(D, p.levels, p.block_size, p.k_null, mc.resolved_coarse_block(),
                                        p.null_iters, rng, mc.w_cycle, p.pre_smooth, p.post_smooth, false, warm);
    if (p.n_defl > 0) {
        OpApply A = [&D](const Vec& s, Vec& d) { D.apply_DdagD(s, d); };
        mg.setup_sparse_coarse(A, D.lat.ndof, p.n_defl, 1e-12, 200, "trlm", 0.0);
    }
    mg.rebind_prolongator_lambdas();
    return mg;
}

// MGHierarchy::precondition (src/multigrid.cpp:155-157) of a hierarchy built by
// build_mg_hierarchy (:595-687).  With warm != nullptr and null_iters = 0 the
// hierarchy uses exactly those level-0 null vectors (after normalisation and
// the final Gram-Schmidt pass, :473-481).
void ref_mg_precondition(int L, const double* U, double m, double r, double csw, double mu, const RefMGParams* p,
                         unsigned seed, const double* warm_vecs, const double* b, double* out) {
    World w(L, U);
    DiracOp D(w.lat, w.g, m, r, csw, mu);
    std::vector<Vec> warm;
    if (warm_vecs)
        for (int i = 0; i < p->k_null; ++i) warm.push_back(to_vec(warm_vecs + (size_t)2 * w.lat.ndof * i, w.lat.ndof));
    MGHierarchy mg = ref_build(D, *p, seed, warm_vecs ? &warm : nullptr);
    from_vec(mg.precondition(to_vec(b, w.lat.ndof)), out);
}

// fcg_solve_mg (src/solvers.cpp:803-811): GCR on D^dag D preconditioned by the
// MG hierarchy; returns the iteration count
int ref_mg_gcr(int L, const double* U, double m, double r, double csw, double mu, const RefMGParams* p,
               unsigned seed, const double* warm_vecs, const double* b, double* x, int max_iter, double tol, int trunc,
               double* final_res) {
    World w(L, U);
    DiracOp D(w.lat, w.g, m, r, csw, mu);
    std::vector<Vec> warm;
    if (warm_vecs)
        for (int i = 0; i < p->k_null; ++i) warm.push_back(to_vec(warm_vecs + (size_t)2 * w.lat.ndof * i, w.lat.ndof));
    MGHierarchy mg = ref_build(D, *p, seed, warm_vecs ? &warm : nullptr);
    OpApply A = [&D](const Vec& s, Vec& d) { D.apply_DdagD(s, d); };
    FCGResult res = fcg_solve_mg(A, w.lat.ndof, to_vec(b, w.lat.ndof), mg, max_iter, tol, trunc);
    from_vec(res.solution, x);
    if (final_res) *final_res = res.final_residual;
    return res.iterations;
}

// null vectors actually used by a hierarchy (MGHierarchy::null_vecs_l0)
void ref_mg_null_vectors(int L, const double* U, double m, double r, double csw, double mu, const RefMGParams* p,
                         unsigned seed, double* out) {
    World w(L, U);
    DiracOp D(w.lat, w.g, m, r, csw, mu);
    MGHierarchy mg = ref_build(D, *p, seed, nullptr);
    for (int i = 0; i < p->k_null; ++i) from_vec(mg.null_vecs_l0[i], out + (size_t)2 * w.lat.ndof * i);
}

// The three-level hierarchy of build_mg_hierarchy (src/multigrid.cpp:595-687):
// level-0 null vectors (k x 2V), the level-1 CoarseProlongator block vectors
// (src/prolongator.h:149-228; [block][k][block_k]), the level-1 operator
// (levels[0].Ac, dense columns) and the level-2 operator (intermediate_Ac,
// dense columns).  Sizes: dim1 = (L/bs)^2 k, dim2 = dim1 / block_k * k.
void ref_mg3_export(int L, const double* U, double m, double r, double csw, double mu, const RefMGParams* p,
                    unsigned seed, double* null0, double* bv1, double* Ac1, double* Ac2) {
    World w(L, U);
    DiracOp D(w.lat, w.g, m, r, csw, mu);
    MGHierarchy mg = ref_build(D, *p, seed, nullptr);
    for (int i = 0; i < p->k_null; ++i) from_vec(mg.null_vecs_l0[i], null0 + (size_t)2 * w.lat.ndof * i);
    const CoarseProlongator& Pc = mg.coarse_prolongators.at(0);
    for (int b = 0; b < Pc.nblocks; ++b)
        for (int k = 0; k < Pc.k_vec; ++k)
            from_vec(Pc.block_vecs[b][k], bv1 + (size_t)2 * ((size_t)b * Pc.k_vec + k) * Pc.block_k);
    const CoarseOp& A1 = mg.levels[0].Ac;
    for (int j = 0; j < A1.dim; ++j) from_vec(A1.mat[j], Ac1 + (size_t)2 * A1.dim * j);
    const CoarseOp& A2 = mg.intermediate_Ac.at(0);
    for (int j = 0; j < A2.dim; ++j) from_vec(A2.mat[j], Ac2 + (size_t)2 * A2.dim * j);
}

// generate_pseudofermion (src/hmc_trajectory.cpp:32-36) with mt19937(seed)
void ref_pseudofermion(int L, const double* U, double m, double r, double csw, double mu, unsigned seed,
                       double* phi) {
    World w(L, U);
    DiracOp D(w.lat, w.g, m, r, csw, mu);
    std::mt19937 rng(seed);
    Vec p;
    generate_pseudofermion(D, rng, p);
    from_vec(p, phi);
}


struct RefMSParams {
    double beta, tau;
    int n_outer, n_inner, cg_maxiter;
    double cg_tol;
    int inner_smooth, outer_type;
    double c_sw, mu_t;
};

static MGMultiScaleParams ms_params(const RefMSParams* q) {
    MGMultiScaleParams mp;
    mp.beta = q->beta;
    mp.tau = q->tau;
    mp.n_outer = q->n_outer;
    mp.n_inner = q->n_inner;
    mp.cg_maxiter = q->cg_maxiter;
    mp.cg_tol = q->cg_tol;
    mp.inner_smooth = q->inner_smooth;
    mp.outer_type = static_cast<OuterIntegrator>(q->outer_type);
    mp.c_sw = q->c_sw;
    mp.mu_t = q->mu_t;
    return mp;
}

// A hierarchy with coarse deflation (build_mg_hierarchy + setup_sparse_coarse with TRLM,
// src/multigrid.cpp:754-794): its level-0 null vectors (k_null x ndof), the deflation pairs
// (n_defl values, n_defl x coarse-dim vectors), CoarseDeflState::lowmode_solution of phi and
// coarse_lowmode_force(D, cdefl, P, phi, smooth) (src/hmc_multiscale.cpp:237-276).
void ref_ms_setup(int L, const double* U, double m, double r, double csw, double mu, const RefMGParams* p,
                  unsigned seed, const double* phi, int smooth, double* null_out, double* vals_out, double* vecs_out,
                  double* lowmode_out, double* force_out) {
    World w(L, U);
    DiracOp D(w.lat, w.g, m, r, csw, mu);
    MGHierarchy mg = ref_build(D, *p, seed, nullptr);
    for (int i = 0; i < p->k_null; ++i) from_vec(mg.null_vecs_l0[i], null_out + (size_t)2 * w.lat.ndof * i);
    CoarseDeflState cdefl;
    cdefl.eigvecs = mg.sparse_Ac.defl_vecs;
    cdefl.eigvals = mg.sparse_Ac.defl_vals;
    const int cdim = mg.sparse_Ac.dim;
    for (size_t i = 0; i < cdefl.eigvals.size(); ++i) {
        vals_out[i] = cdefl.eigvals[i];
        from_vec(cdefl.eigvecs[i], vecs_out + (size_t)2 * cdim * i);
    }
    const Vec ph = to_vec(phi, w.lat.ndof);
    from_vec(cdefl.lowmode_solution(ph, mg.geo_prolongators[0]), lowmode_out);
    std::array<RVec, 2> f;
    coarse_lowmode_force(D, cdefl, mg.geo_prolongators[0], ph, f, smooth);
    for (int mu2 = 0; mu2 < 2; ++mu2)
        for (int s = 0; s < w.lat.V; ++s) force_out[mu2 * w.lat.V + s] = f[mu2][s];
}

// hmc_trajectory_mg_multiscale (src/hmc_multiscale.cpp:340-886) n_traj times from one
// std::mt19937(seed) with the hierarchy of ref_ms_setup as preconditioner, prolongator and
// deflation space; after an accepted trajectory the sparse coarse operator is rebuilt for the new
// links and the deflation pairs follow by evolve_coarse_deflation, as the MG-HMC driver does
// (src/mode_mg_hmc.cpp:280-288).  U is updated in place; per trajectory out[9 t + {0..8}] =
// accepted, dH, dKE, dSG, dSF, CG iterations, low-mode force evaluations, plaquette, max |dH| 0.
void ref_ms_trajectories(int L, double* U, double m, double r, const RefMGParams* p, unsigned mg_seed,
                         const RefMSParams* q, unsigned seed, int n_traj, double* out) {
    World w(L, U);
    DiracOp D(w.lat, w.g, m, r, q->c_sw, q->mu_t);
    MGHierarchy mg = ref_build(D, *p, mg_seed, nullptr);
    CoarseDeflState cdefl;
    cdefl.eigvecs = mg.sparse_Ac.defl_vecs;
    cdefl.eigvals = mg.sparse_Ac.defl_vals;
    auto& P = mg.geo_prolongators[0];
    std::function<Vec(const Vec&)> pre = [&mg](const Vec& b) -> Vec { return mg.precondition(b); };
    const MGMultiScaleParams mp = ms_params(q);
    std::mt19937 rng(seed);
    for (int t = 0; t < n_traj; ++t) {
        MGMultiScaleResult res = hmc_trajectory_mg_multiscale(w.g, w.lat, m, r, mp, cdefl, P, pre, rng);
        double* o = out + 9 * t;
        o[0] = res.accepted ? 1.0 : 0.0;
        o[1] = res.dH;
        o[2] = res.dKE;
        o[3] = res.dSG;
        o[4] = res.dSF;
        o[5] = res.highmode_cg_iters;
        o[6] = res.lowmode_force_evals;
        o[7] = w.g.avg_plaq();
        o[8] = 0.0;
        if (res.accepted) {
            DiracOp Dn(w.lat, w.g, m, r, q->c_sw, q->mu_t);
            OpApply An = [&Dn](const Vec& s, Vec& d) { Dn.apply_DdagD(s, d); };
            mg.sparse_Ac.build(P, An, w.lat.ndof);
            evolve_coarse_deflation(cdefl, mg.sparse_Ac, nullptr);
        }
    }
    for (int mu2 = 0; mu2 < 2; ++mu2)
        for (int s = 0; s < w.lat.V; ++s) {
            U[2 * (mu2 * w.lat.V + s)] = w.g.U[mu2][s].real();
            U[2 * (mu2 * w.lat.V + s) + 1] = w.g.U[mu2][s].imag();
        }
}

// reversibility_test_mg_multiscale (src/hmc_multiscale.cpp:963-1000) with the hierarchy of
// ref_ms_setup; out = {gauge_delta, mom_delta, dH_forward, dH_backward, total CG}
void ref_ms_reversibility(int L, const double* U, double m, double r, const RefMGParams* p, unsigned mg_seed,
                          const RefMSParams* q, unsigned seed, double* out) {
    World w(L, U);
    DiracOp D(w.lat, w.g, m, r, q->c_sw, q->mu_t);
    MGHierarchy mg = ref_build(D, *p, mg_seed, nullptr);
    CoarseDeflState cdefl;
    cdefl.eigvecs = mg.sparse_Ac.defl_vecs;
    cdefl.eigvals = mg.sparse_Ac.defl_vals;
    std::function<Vec(const Vec&)> pre = [&mg](const Vec& b) -> Vec { return mg.precondition(b); };
    std::mt19937 rng(seed);
    ReversibilityResult res =
        reversibility_test_mg_multiscale(w.g, w.lat, m, r, ms_params(q), cdefl, mg.geo_prolongators[0], pre, rng);
    out[0] = res.gauge_delta;
    out[1] = res.mom_delta;
    out[2] = res.dH_forward;
    out[3] = res.dH_backward;
    out[4] = res.total_cg;
}

// reversibility_test_plain (src/hmc_trajectory.cpp:416-509) with one std::mt19937(seed) and no
// preconditioner; out = {gauge_delta, mom_delta, dH_forward, dH_backward, total_cg}.  The links
// are restored by the reference itself.
void ref_hmc_reversibility(int L, const double* U, double mass, double r, double beta, double tau, int n_steps,
                           int omelyan, int cg_maxiter, double cg_tol, double c_sw, double mu_t, unsigned seed,
                           double* out) {
    World w(L, U);
    HMCParams hp{};
    hp.beta = beta;
    hp.tau = tau;
    hp.n_steps = n_steps;
    hp.cg_maxiter = cg_maxiter;
    hp.cg_tol = cg_tol;
    hp.use_mg = false;
    hp.c_sw = c_sw;
    hp.mu_t = mu_t;
    hp.omelyan = omelyan != 0;
    std::mt19937 rng(seed);
    ReversibilityResult res = reversibility_test_plain(w.g, w.lat, mass, r, hp, rng, nullptr);
    out[0] = res.gauge_delta;
    out[1] = res.mom_delta;
    out[2] = res.dH_forward;
    out[3] = res.dH_backward;
    out[4] = res.total_cg;
}

// hmc_trajectory (src/hmc_trajectory.cpp:38-235, full-lattice path, no
// preconditioner, no tracking) for n_traj trajectories threading one
// std::mt19937(seed).  U (2V complex) is updated in place; per trajectory
// out[8 t + {0..6}] = accepted, dH, dKE, dSG, dSF, total CG iterations,
// average plaquette after the trajectory.
void ref_hmc_trajectories(int L, double* U, double mass, double r, double beta, double tau, int n_steps,
                          int omelyan, int cg_maxiter, double cg_tol, double c_sw, double mu_t, int force_accept,
                          unsigned seed, int n_traj, double* out, int use_eo) {
    World w(L, U);
    HMCParams hp{};
    hp.beta = beta;
    hp.tau = tau;
    hp.n_steps = n_steps;
    hp.cg_maxiter = cg_maxiter;
    hp.cg_tol = cg_tol;
    hp.use_mg = false;
    hp.c_sw = c_sw;
    hp.mu_t = mu_t;
    hp.use_eo = use_eo != 0;
    hp.omelyan = omelyan != 0;
    hp.force_accept = force_accept != 0;
    std::mt19937 rng(seed);
    for (int t = 0; t < n_traj; ++t) {
        HMCResult res = hmc_trajectory(w.g, w.lat, mass, r, hp, rng);
        out[8 * t + 0] = res.accepted ? 1.0 : 0.0;
        out[8 * t + 1] = res.dH;
        out[8 * t + 2] = res.dKE;
        out[8 * t + 3] = res.dSG;
        out[8 * t + 4] = res.dSF;
        out[8 * t + 5] = res.total_cg_iters;
        out[8 * t + 6] = w.g.avg_plaq();
        out[8 * t + 7] = res.dLD;
    }
    for (int mu = 0; mu < 2; ++mu)
        for (int s = 0; s < w.lat.V; ++s) {
            U[2 * (mu * w.lat.V + s)] = w.g.U[mu][s].real();
            U[2 * (mu * w.lat.V + s) + 1] = w.g.U[mu][s].imag();
        }
}


// richardson_smooth_op (src/smoother.cpp:64-73) with A = D^dag D; x updated in place
void ref_richardson_smooth(int L, const double* U, double m, double r, double csw, double mu, const double* b,
                           double* x, int niter, double omega) {
    World w(L, U);
    DiracOp D(w.lat, w.g, m, r, csw, mu);
    OpApply A = [&D](const Vec& s, Vec& d) { D.apply_DdagD(s, d); };
    Vec xv = to_vec(x, w.lat.ndof);
    richardson_smooth_op(A, xv, to_vec(b, w.lat.ndof), niter, omega);
    from_vec(xv, x);
}

// estimate_lambda_max (src/smoother.cpp:43-60) of D^dag D
double ref_estimate_lambda_max(int L, const double* U, double m, double r, double csw, double mu, int niter) {
    World w(L, U);
    DiracOp D(w.lat, w.g, m, r, csw, mu);
    OpApply A = [&D](const Vec& s, Vec& d) { D.apply_DdagD(s, d); };
    return estimate_lambda_max(A, w.lat.ndof, niter);
}

// MGHierarchy::set_symmetric(damping) (src/multigrid.cpp:144-152) followed by
// precondition (:155-157); omega receives levels - 1 values
void ref_mg_precondition_sym(int L, const double* U, double m, double r, double csw, double mu,
                             const RefMGParams* p, unsigned seed, double damping, const double* b, double* out,
                             double* omega) {
    World w(L, U);
    DiracOp D(w.lat, w.g, m, r, csw, mu);
    MGHierarchy mg = ref_build(D, *p, seed, nullptr);
    mg.set_symmetric(damping);
    for (size_t l = 0; l + 1 < mg.levels.size(); ++l) omega[l] = mg.levels[l].richardson_omega;
    from_vec(mg.precondition(to_vec(b, w.lat.ndof)), out);
}

// cg_solve_core (src/solvers.cpp:16-72) through cg_solve / cg_solve_x0 /
// cg_solve_precond / cg_solve_x0_precond: with_mg != 0 builds the hierarchy
// (set_symmetric(damping) when damping > 0) as the preconditioner; x0 may be
// NULL.  Returns the iteration count.
int ref_cg_precond(int L, const double* U, double m, double r, double csw, double mu, int with_mg,
                   const RefMGParams* p, unsigned seed, double damping, const double* b, const double* x0,
                   double* x, int max_iter, double tol, double* final_res) {
    World w(L, U);
    DiracOp D(w.lat, w.g, m, r, csw, mu);
    OpApply A = [&D](const Vec& s, Vec& d) { D.apply_DdagD(s, d); };
    const int n = w.lat.ndof;
    Vec bv = to_vec(b, n);
    CGResult res;
    if (with_mg) {
        MGHierarchy mg = ref_build(D, *p, seed, nullptr);
        if (damping > 0) mg.set_symmetric(damping);
        auto precond = [&mg](const Vec& v) { return mg.precondition(v); };
        res = x0 ? cg_solve_x0_precond(A, n, bv, to_vec(x0, n), precond, max_iter, tol)
                 : cg_solve_precond(A, n, bv, precond, max_iter, tol);
    } else {
        res = x0 ? cg_solve_x0(A, n, bv, to_vec(x0, n), max_iter, tol) : cg_solve(A, n, bv, max_iter, tol);
    }
    from_vec(res.solution, x);
    if (final_res) *final_res = res.final_residual;
    return res.iterations;
}

// fgmres_solve_mg (src/solvers.cpp:776-787), or fgmres_solve_generic with the
// identity preconditioner when with_mg == 0.  ritz receives up to 3 *
// n_ritz_harvest values (RitzPair::value, list order), n_ritz their count.
int ref_fgmres(int L, const double* U, double m, double r, double csw, double mu, int with_mg,
               const RefMGParams* p, unsigned seed, const double* b, double* x, int restart, int max_iter,
               double tol, int n_ritz_harvest, double* final_res, double* ritz, int* n_ritz) {
    World w(L, U);
    DiracOp D(w.lat, w.g, m, r, csw, mu);
    OpApply A = [&D](const Vec& s, Vec& d) { D.apply_DdagD(s, d); };
    const int n = w.lat.ndof;
    FGMRESResult res;
    if (with_mg) {
        MGHierarchy mg = ref_build(D, *p, seed, nullptr);
        res = fgmres_solve_mg(A, n, to_vec(b, n), mg, restart, max_iter, tol, n_ritz_harvest);
    } else {
        auto identity = [](const Vec& v) { return v; };
        res = fgmres_solve_generic(A, n, to_vec(b, n), identity, restart, max_iter, tol, n_ritz_harvest);
    }
    from_vec(res.solution, x);
    if (final_res) *final_res = res.final_residual;
    *n_ritz = (int)res.ritz_pairs.size();
    for (size_t i = 0; i < res.ritz_pairs.size(); ++i) ritz[i] = res.ritz_pairs[i].value;
    return res.iterations;
}

// fermion_action (src/hmc_forces.cpp:113-119): S = Re <phi, X>, X = (D^dag D)^-1 phi by cg_solve
double ref_fermion_action(int L, const double* U, double m, double r, double csw, double mu, const double* phi,
                          int max_iter, double tol, double* X) {
    World w(L, U);
    DiracOp D(w.lat, w.g, m, r, csw, mu);
    FermionActionResult fa = fermion_action(D, to_vec(phi, w.lat.ndof), max_iter, tol);
    from_vec(fa.X, X);
    return fa.action;
}


// save_gauge (src/hmc_forces.cpp:18-35) and GaugeField::save (src/gauge.h:38-46)
int ref_save_gauge(int L, const double* U, double beta, double mass, const char* swng_path, const char* raw_path) {
    World w(L, U);
    bool ok = save_gauge(w.g, beta, mass, swng_path);
    ok = w.g.save(raw_path) && ok;
    return ok ? 1 : 0;
}

// load_gauge (src/hmc_forces.cpp:37-62): links into U, header fields into hdr[0..2]
// (beta, mass, avg_plaq); returns 1 on success
int ref_load_gauge(int L, const char* path, double* U, double* hdr) {
    Lattice lat(L);
    GaugeField g(lat);
    GaugeHeader h{};
    if (!load_gauge(g, h, path)) return 0;
    for (int mu = 0; mu < 2; ++mu)
        for (int s = 0; s < lat.V; ++s) {
            U[2 * (mu * lat.V + s)] = g.U[mu][s].real();
            U[2 * (mu * lat.V + s) + 1] = g.U[mu][s].imag();
        }
    hdr[0] = h.beta;
    hdr[1] = h.mass;
    hdr[2] = h.avg_plaq;
    return 1;
}


// EvenOddDiracOp (src/dirac.h:190-553) on half vectors of 2 * V/2 complex:
// op 0 apply_schur, 1 apply_schur_dag, 2 apply_schur_dag_schur, 3 apply_eo, 4 apply_oe
void ref_eo_apply(int L, const double* U, double m, double r, double csw, double mu, int op, const double* src,
                  double* dst) {
    World w(L, U);
    DiracOp D(w.lat, w.g, m, r, csw, mu);
    EvenOddDiracOp eo(D);
    const int nh = 2 * w.lat.V_half;
    Vec in = to_vec(src, nh), out(nh);
    if (op == 0) eo.apply_schur(in, out);
    else if (op == 1) eo.apply_schur_dag(in, out);
    else if (op == 2) eo.apply_schur_dag_schur(in, out);
    else if (op == 3) eo.apply_eo(in, out);
    else eo.apply_oe(in, out);
    from_vec(out, dst);
}

// reconstruct(x_o, phi) (src/dirac.h:527-540), or reconstruct_full(x_o) when phi is NULL
void ref_eo_reconstruct(int L, const double* U, double m, double r, double csw, double mu, const double* x_o,
                        const double* phi, double* full) {
    World w(L, U);
    DiracOp D(w.lat, w.g, m, r, csw, mu);
    EvenOddDiracOp eo(D);
    const int nh = 2 * w.lat.V_half;
    Vec x = phi ? eo.reconstruct(to_vec(x_o, nh), to_vec(phi, w.lat.ndof)) : eo.reconstruct_full(to_vec(x_o, nh));
    from_vec(x, full);
}

double ref_eo_logdet(int L, const double* U, double m, double r, double csw, double mu) {
    World w(L, U);
    DiracOp D(w.lat, w.g, m, r, csw, mu);
    return EvenOddDiracOp(D).log_det_ee();
}

// cg_solve on apply_schur_dag_schur (src/hmc_trajectory.cpp:70-104); returns iterations
int ref_eo_cg(int L, const double* U, double m, double r, double csw, double mu, const double* phi_o, double* x_o,
              int max_iter, double tol, double* final_res) {
    World w(L, U);
    DiracOp D(w.lat, w.g, m, r, csw, mu);
    EvenOddDiracOp eo(D);
    const int nh = 2 * w.lat.V_half;
    OpApply A = [&eo](const Vec& s, Vec& d) { eo.apply_schur_dag_schur(s, d); };
    CGResult res = cg_solve(A, nh, to_vec(phi_o, nh), max_iter, tol);
    from_vec(res.solution, x_o);
    if (final_res) *final_res = res.final_residual;
    return res.iterations;
}

// eo_fermion_force (src/hmc_forces.cpp:812-867) at x_o with y_o = M x_o
void ref_eo_force(int L, const double* U, double m, double r, double csw, double mu, const double* x_o,
                  double* F) {
    World w(L, U);
    DiracOp D(w.lat, w.g, m, r, csw, mu);
    EvenOddDiracOp eo(D);
    const int nh = 2 * w.lat.V_half;
    Vec x = to_vec(x_o, nh), y(nh);
    eo.apply_schur(x, y);
    std::array<RVec, 2> f;
    eo_fermion_force(D, eo, x, y, f);
    for (int mu_ = 0; mu_ < 2; ++mu_) std::memcpy(F + (size_t)mu_ * w.lat.V, f[mu_].data(), sizeof(double) * w.lat.V);
}


// DiracOp::apply_delta_D (src/dirac.h:159-174): (D(e^{i dt pi} U) - D(U)) v through the hopping terms
void ref_apply_delta_D(int L, const double* U, double m, double r, double csw, double mu, const double* pi,
                       double dt, const double* src, double* dst) {
    World w(L, U);
    DiracOp D(w.lat, w.g, m, r, csw, mu);
    std::array<RVec, 2> p;
    for (int mu_ = 0; mu_ < 2; ++mu_) p[mu_].assign(pi + (size_t)mu_ * w.lat.V, pi + (size_t)(mu_ + 1) * w.lat.V);
    Vec out(w.lat.ndof);
    D.apply_delta_D(to_vec(src, w.lat.ndof), out, p, dt);
    from_vec(out, dst);
}

}  // extern "C"
