// Hybrid Monte Carlo on the device (reference src/hmc_trajectory.cpp:32-409,
// src/hmc_multiscale.cpp:660-710, src/hmc_forces.cpp:64-111).
//
// The links, momenta, forces, pseudofermion and solutions stay in device
// memory for the whole trajectory; the host draws the random numbers with the
// reference's generator and distributions (momenta, eta, Metropolis) and runs
// the integrator schedule.  Momenta and forces are lexicographic [mu][s]
// doubles, as the reference's MomentumField and force arrays.
#include <algorithm>
#include <cmath>
#include <random>
#include <vector>

#include "mg_internal.h"
#include "reduce.cuh"
#include "smg_internal.h"

struct smg_rng {
    std::mt19937 gen;
};

smg_status smg_fermion_force_dev(smg_dirac* d, const smg_field* X, double* F_dev);
smg_status smg_gauge_force_dev(smg_gauge* gf, double beta, double* F_dev);
smg_status smg_eo_schur_internal(smg_dirac* d, bool dag, const smg_field* src, smg_field* dst, smg_field* tmp,
                                 double* norm2_dev);
smg_status smg_eo_force_dev(smg_dirac* d, const smg_field* X, smg_field* chi, smg_field* psi, double* W,
                            double* F_dev);
smg_status smg_eo_logdet_dev(smg_dirac* d, double* out_dev);

namespace {

constexpr double kOmelyanLambda = 0.1932;  // hmc_trajectory.cpp:355

// pi += scale * (f1 + f2)  (update_mom, hmc_trajectory.cpp:330-335); f2 may be null
__global__ void k_kick(double* __restrict__ pi, const double* __restrict__ f1, const double* __restrict__ f2,
                       double scale, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double f = f1 ? f1[i] : 0.0;
    if (f2) f += f2[i];
    pi[i] += scale * f;
}

// U_mu(s) *= exp(i * scale * pi_mu(s))  (update_gauge, hmc_trajectory.cpp:337-342)
__global__ void k_links_exp(cx<double>* __restrict__ U, const double* __restrict__ pi, double scale, Geom g) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= 2 * g.V) return;
    const int mu = i / g.V, s = i - mu * g.V;
    double sn, cs;
    sincos(scale * pi[i], &sn, &cs);
    cx<double>& u = U[(int64_t)mu * g.V + site_q(g, s % g.L, s / g.L)];
    u = u * mk(cs, sn);
}

// pi = -pi (the momentum flip between the two halves of reversibility_test_plain)
__global__ void k_negate(double* __restrict__ pi, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) pi[i] = -pi[i];
}

// F = gf + ff - fl (the outer force of hmc_trajectory_mg_multiscale, src/hmc_multiscale.cpp:498-503)
__global__ void k_outer_combine(double* __restrict__ F, const double* __restrict__ gf, const double* __restrict__ ff,
                                const double* __restrict__ fl, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) F[i] = gf[i] + ff[i] - fl[i];
}

// r = a - b, or x += b (a == nullptr) over n complex entries
__global__ void k_sub_add(cx<double>* __restrict__ out, const cx<double>* __restrict__ a,
                          const cx<double>* __restrict__ b, int64_t n) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    out[i] = a ? a[i] - b[i] : out[i] + b[i];
}

// sum of squares of n doubles (MomentumField::kinetic_energy without the 1/2)
__global__ void __launch_bounds__(256) k_sumsq(const double* __restrict__ a, int n, double* partials,
                                               unsigned int* ticket, double* out) {
    double v[1] = {0.0};
    for (int i = blockIdx.x * blockDim.y + threadIdx.y; i < n; i += gridDim.x * blockDim.y) v[0] += a[i] * a[i];
    block_reduce_finalise<1>(v, partials, ticket, 1, FinStore{out, 1});
}

// coarse_lowmode_force (src/hmc_multiscale.cpp:237-276): MR on D^dag D x = phi from x = 0, the
// low-mode solution of the residual added, MR again (smooth > 0; otherwise x is the low-mode
// solution of phi), then the fermion force of x into F (device [mu][s]); xl, rl, tl are
// single-RHS F64 scratch fields
smg_status lowmode_force_fields(smg_dirac* d, smg_mg* mg, const smg_field* phi, int smooth, smg_field* xl,
                                smg_field* rl, smg_field* tl, double* F) {
    smg_context* ctx = d->ctx;
    if (smooth <= 0) {
        SMG_TRY(smg_mg_lowmode_internal(mg, phi, xl));
        return smg_fermion_force_dev(d, xl, F);
    }
    const int64_t n = 2 * (int64_t)phi->g.V;
    const unsigned blocks = (unsigned)((n + 255) / 256);
    SMG_CUDA(ctx, cudaMemsetAsync(xl->data, 0, xl->bytes, ctx->stream));
    SMG_TRY(smg_mr_smooth(d, phi, xl, smooth));
    SMG_TRY(smg_dirac_apply(d, SMG_OP_DDAGD, xl, tl));
    k_sub_add<<<blocks, 256, 0, ctx->stream>>>((cx<double>*)rl->data, (const cx<double>*)phi->data,
                                               (const cx<double>*)tl->data, n);
    count_launch(ctx);
    SMG_TRY(smg_mg_lowmode_internal(mg, rl, tl));
    k_sub_add<<<blocks, 256, 0, ctx->stream>>>((cx<double>*)xl->data, nullptr, (const cx<double>*)tl->data, n);
    count_launch(ctx);
    SMG_CHECK_LAUNCH(ctx);
    SMG_TRY(smg_mr_smooth(d, phi, xl, smooth));
    return smg_fermion_force_dev(d, xl, F);
}

struct Hmc {
    smg_context* ctx = nullptr;
    smg_gauge* g = nullptr;
    smg_dirac* d = nullptr;
    smg_hmc_params p{};
    double mass = 0, r = 1;
    double* pi = nullptr;  // device [mu][s]
    double* gf = nullptr;
    double* ff = nullptr;
    double* scal = nullptr;  // device scalars
    cx<double>* U_old = nullptr;
    smg_field* phi = nullptr;
    smg_field* X = nullptr;
    smg_field* eta = nullptr;
    smg_field* chi = nullptr;  // even-odd force scratch
    smg_field* psi = nullptr;
    double* W = nullptr;
    bool eo = false;
    bool stale = false;  // links changed since the clover field and the FP32 links were formed
    int cg_iters = 0, solves = 0;
    smg_status warn = SMG_OK;
    // multi-timescale MG HMC: the hierarchy (preconditioner, prolongator, deflation space) and the
    // low-mode force's fields and forces
    smg_mg* mg = nullptr;
    bool mg_stale = false;  // links changed since the hierarchy's own Dirac operator was refreshed
    int inner_smooth = 0, n_inner = 1, lowmode_evals = 0;
    double *fl = nullptr, *fo = nullptr, *pi_save = nullptr;
    cx<double>* U_save = nullptr;
    smg_field *xl = nullptr, *rl = nullptr, *tl = nullptr;

    ~Hmc() {
        if (ctx) cudaStreamSynchronize(ctx->stream);
        for (void* q : {(void*)pi, (void*)gf, (void*)ff, (void*)scal, (void*)U_old, (void*)W, (void*)fl, (void*)fo,
                        (void*)pi_save, (void*)U_save})
            if (q) cudaFree(q);
        smg_field_destroy(xl);
        smg_field_destroy(rl);
        smg_field_destroy(tl);
        smg_field_destroy(phi);
        smg_field_destroy(X);
        smg_field_destroy(eta);
        smg_field_destroy(chi);
        smg_field_destroy(psi);
        smg_dirac_destroy(d);
    }

    int n2() const { return 2 * g->g.V; }

    smg_status refresh() {
        if (!stale) return SMG_OK;
        SMG_TRY(smg_gauge_ensure_f32(g));
        SMG_TRY(smg_dirac_refresh(d));
        stale = false;
        return SMG_OK;
    }

    // X = (D^dag D)^-1 phi with the current links; with a hierarchy, CG preconditioned by its cycle
    // (cg_solve_precond, src/hmc_multiscale.cpp:479-484)
    smg_status solve() {
        SMG_TRY(refresh());
        if (mg && mg_stale) {
            smg_dirac* md = smg_mg_dirac(mg);
            if (md != d) SMG_TRY(smg_dirac_refresh(md));
            mg_stale = false;
        }
        smg_solve_result res{};
        const smg_status st = mg                  ? smg_cg_solve_precond(d, mg, phi, X, 0, p.cg_maxiter, p.cg_tol, &res)
                              : eo                ? smg_eo_cg_solve(d, phi, X, p.cg_maxiter, p.cg_tol, &res)
                              : p.mixed_precision ? smg_cg_solve_mixed(d, phi, X, p.cg_maxiter, p.cg_tol, &res)
                                                  : smg_cg_solve(d, phi, X, p.cg_maxiter, p.cg_tol, &res);
        cg_iters += res.iterations;
        ++solves;
        // the reference warns and carries on when CG stops early (solvers.cpp:55-62)
        if (st == SMG_NOT_CONVERGED || st == SMG_BREAKDOWN) {
            warn = st;
            return SMG_OK;
        }
        return st;
    }

    smg_status fermion_force() {
        SMG_TRY(solve());
        if (eo) return smg_eo_force_dev(d, X, chi, psi, W, ff);
        return smg_fermion_force_dev(d, X, ff);
    }

    // -2 log det D_ee (even-odd path with clover; 0 otherwise)
    smg_status log_det_term(double* ld) {
        *ld = 0;
        if (!eo || p.c_sw == 0.0) return SMG_OK;
        SMG_TRY(refresh());
        SMG_TRY(smg_eo_logdet_dev(d, scal + 1));
        double h = 0;
        SMG_CUDA(ctx, cudaMemcpyAsync(&h, scal + 1, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
        SMG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        *ld = -2.0 * h;
        return SMG_OK;
    }

    smg_status gauge_force() {
        SMG_TRY(refresh());
        return smg_gauge_force_dev(g, p.beta, gf);
    }

    smg_status kick(const double* f1, const double* f2, double scale) {
        k_kick<<<(n2() + 255) / 256, 256, 0, ctx->stream>>>(pi, f1, f2, scale, n2());
        count_launch(ctx);
        SMG_CHECK_LAUNCH(ctx);
        return SMG_OK;
    }

    smg_status update_gauge(double scale) {
        k_links_exp<<<(n2() + 255) / 256, 256, 0, ctx->stream>>>(g->U64, pi, scale, g->g);
        count_launch(ctx);
        SMG_CHECK_LAUNCH(ctx);
        stale = true;
        mg_stale = true;
        return SMG_OK;
    }

    smg_status lowmode_force(double* F) {
        SMG_TRY(refresh());
        return lowmode_force_fields(d, mg, phi, inner_smooth, xl, rl, tl, F);
    }

    // compute_outer_force (src/hmc_multiscale.cpp:424-504): gauge + fermion - low-mode force
    smg_status outer_force(double* F) {
        SMG_TRY(gauge_force());
        SMG_TRY(solve());
        SMG_TRY(smg_fermion_force_dev(d, X, ff));
        SMG_TRY(lowmode_force(fl));
        k_outer_combine<<<(n2() + 255) / 256, 256, 0, ctx->stream>>>(F, gf, ff, fl, n2());
        count_launch(ctx);
        SMG_CHECK_LAUNCH(ctx);
        return SMG_OK;
    }

    // inner_integrator (src/hmc_multiscale.cpp:638-658): leapfrog on the low-mode force
    smg_status inner_lowmode(double dt_total) {
        const double dti = dt_total / n_inner;
        SMG_TRY(lowmode_force(fl));
        ++lowmode_evals;
        SMG_TRY(kick(fl, nullptr, 0.5 * dti));
        for (int i = 0; i < n_inner; ++i) {
            SMG_TRY(update_gauge(dti));
            SMG_TRY(lowmode_force(fl));
            ++lowmode_evals;
            SMG_TRY(kick(fl, nullptr, i < n_inner - 1 ? dti : 0.5 * dti));
        }
        return SMG_OK;
    }

    // fg_step (src/hmc_multiscale.cpp:737-779): force-gradient update of the expensive force by a
    // displaced gauge field, lambda = 1/6, xi = 1/72
    smg_status fg_step(double h) {
        const double om = 1.0 - 2.0 / 6.0, xi_h3 = 2.0 / 72.0 * h * h * h;
        const size_t ub = (size_t)n2() * sizeof(cx<double>), pb = (size_t)n2() * sizeof(double);
        SMG_CUDA(ctx, cudaMemcpyAsync(U_save, g->U64, ub, cudaMemcpyDeviceToDevice, ctx->stream));
        SMG_CUDA(ctx, cudaMemcpyAsync(pi_save, pi, pb, cudaMemcpyDeviceToDevice, ctx->stream));
        SMG_CUDA(ctx, cudaMemsetAsync(pi, 0, pb, ctx->stream));
        SMG_TRY(outer_force(fo));
        SMG_TRY(kick(fo, nullptr, xi_h3 / (om * h)));
        SMG_TRY(update_gauge(1.0));
        SMG_CUDA(ctx, cudaMemcpyAsync(pi, pi_save, pb, cudaMemcpyDeviceToDevice, ctx->stream));
        SMG_TRY(outer_force(fo));
        SMG_TRY(kick(fo, nullptr, om * h));
        SMG_CUDA(ctx, cudaMemcpyAsync(g->U64, U_save, ub, cudaMemcpyDeviceToDevice, ctx->stream));
        stale = true;
        mg_stale = true;
        return SMG_OK;
    }

    // the outer integrators of hmc_trajectory_mg_multiscale (src/hmc_multiscale.cpp:712-836)
    smg_status evolve_multiscale(int outer_type, int n_outer, double tau) {
        const double h = tau / n_outer;
        if (outer_type == SMG_OUTER_LEAPFROG) {
            SMG_TRY(outer_force(fo));
            SMG_TRY(kick(fo, nullptr, 0.5 * h));
            for (int o = 0; o < n_outer; ++o) {
                SMG_TRY(inner_lowmode(h));
                SMG_TRY(outer_force(fo));
                SMG_TRY(kick(fo, nullptr, o < n_outer - 1 ? h : 0.5 * h));
            }
        } else if (outer_type == SMG_OUTER_OMELYAN) {
            const double lam = kOmelyanLambda;
            SMG_TRY(outer_force(fo));
            SMG_TRY(kick(fo, nullptr, lam * h));
            for (int o = 0; o < n_outer; ++o) {
                SMG_TRY(inner_lowmode(0.5 * h));
                SMG_TRY(outer_force(fo));
                SMG_TRY(kick(fo, nullptr, (1.0 - 2.0 * lam) * h));
                SMG_TRY(inner_lowmode(0.5 * h));
                SMG_TRY(outer_force(fo));
                SMG_TRY(kick(fo, nullptr, o < n_outer - 1 ? 2.0 * lam * h : lam * h));
            }
        } else if (outer_type == SMG_OUTER_FGI) {
            const double lam = 1.0 / 6.0;
            SMG_TRY(outer_force(fo));
            SMG_TRY(kick(fo, nullptr, lam * h));
            for (int o = 0; o < n_outer; ++o) {
                SMG_TRY(inner_lowmode(0.5 * h));
                SMG_TRY(fg_step(h));
                SMG_TRY(inner_lowmode(0.5 * h));
                SMG_TRY(outer_force(fo));
                SMG_TRY(kick(fo, nullptr, o < n_outer - 1 ? 2.0 * lam * h : lam * h));
            }
        } else {  // FGI_QPQPQ
            const double lam = 1.0 / 6.0;
            SMG_TRY(inner_lowmode(lam * h));
            for (int o = 0; o < n_outer; ++o) {
                SMG_TRY(outer_force(fo));
                SMG_TRY(kick(fo, nullptr, 0.5 * h));
                SMG_TRY(fg_step(h));
                SMG_TRY(outer_force(fo));
                SMG_TRY(kick(fo, nullptr, 0.5 * h));
                SMG_TRY(inner_lowmode(o < n_outer - 1 ? 2.0 * lam * h : lam * h));
            }
        }
        return SMG_OK;
    }

    smg_status kinetic(double* ke) {
        ReduceLaunch rl = reduce_launch(n2(), 1);
        SMG_TRY(smg_reduce_reserve(ctx, rl.grid.x));
        k_sumsq<<<rl.grid, rl.block, 0, ctx->stream>>>(pi, n2(), ctx->red.partials, ctx->red.tickets, scal);
        count_launch(ctx);
        SMG_CHECK_LAUNCH(ctx);
        double h = 0;
        SMG_CUDA(ctx, cudaMemcpyAsync(&h, scal, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
        SMG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        *ke = 0.5 * h;
        return SMG_OK;
    }

    // S_F = Re <phi, (D^dag D)^-1 phi> with a fresh solve (hmc_trajectory.cpp:170-182)
    smg_status fermion_action(double* sf) {
        SMG_TRY(solve());
        double dot[2] = {0, 0};
        SMG_TRY(smg_blas_dot(phi, X, dot));
        *sf = dot[0];
        return SMG_OK;
    }

    // H = KE + S_G + S_F (+ -2 log det D_ee on the even-odd path) with the current links
    smg_status hamiltonian(double* ke, double* sg, double* sf, double* ld) {
        SMG_TRY(refresh());
        SMG_TRY(kinetic(ke));
        SMG_TRY(smg_gauge_action(g, p.beta, sg));
        SMG_TRY(fermion_action(sf));
        return log_det_term(ld);
    }

    smg_status evolve() { return p.n_inner > 0 ? evolve_nested() : evolve_plain(); }

    // plain_leapfrog_evolve (hmc_trajectory.cpp:243-409): gauge + fermion force at every kick
    smg_status evolve_plain() {
        const double dt = p.tau / p.n_steps;
        auto solve_force = [&]() -> smg_status {
            SMG_TRY(gauge_force());
            return fermion_force();
        };
        if (p.omelyan && !eo) {  // the reference's even-odd trajectory always uses leapfrog
            const double lam = kOmelyanLambda;
            SMG_TRY(solve_force());
            SMG_TRY(kick(gf, ff, lam * dt));
            for (int step = 0; step < p.n_steps; ++step) {
                SMG_TRY(update_gauge(0.5 * dt));
                SMG_TRY(solve_force());
                SMG_TRY(kick(gf, ff, (1.0 - 2.0 * lam) * dt));
                SMG_TRY(update_gauge(0.5 * dt));
                SMG_TRY(solve_force());
                SMG_TRY(kick(gf, ff, step < p.n_steps - 1 ? 2.0 * lam * dt : lam * dt));
            }
        } else {
            SMG_TRY(solve_force());
            SMG_TRY(kick(gf, ff, 0.5 * dt));
            for (int step = 0; step < p.n_steps - 1; ++step) {
                SMG_TRY(update_gauge(dt));
                SMG_TRY(solve_force());
                SMG_TRY(kick(gf, ff, dt));
            }
            SMG_TRY(update_gauge(dt));
            SMG_TRY(solve_force());
            SMG_TRY(kick(gf, ff, 0.5 * dt));
        }
        return SMG_OK;
    }

    // nested integrator (hmc_multiscale.cpp:660-710): the fermion force on the outer
    // steps, an inner leapfrog of n_inner steps on the gauge force between them
    smg_status evolve_nested() {
        const double h = p.tau / p.n_steps;
        auto inner = [&](double dt_total) -> smg_status {
            const int ni = p.n_inner;
            const double dti = dt_total / ni;
            SMG_TRY(gauge_force());
            SMG_TRY(kick(gf, nullptr, 0.5 * dti));
            for (int i = 0; i < ni; ++i) {
                SMG_TRY(update_gauge(dti));
                SMG_TRY(gauge_force());
                SMG_TRY(kick(gf, nullptr, i < ni - 1 ? dti : 0.5 * dti));
            }
            return SMG_OK;
        };
        if (p.omelyan) {
            const double lam = kOmelyanLambda;
            SMG_TRY(fermion_force());
            SMG_TRY(kick(ff, nullptr, lam * h));
            for (int o = 0; o < p.n_steps; ++o) {
                SMG_TRY(inner(0.5 * h));
                SMG_TRY(fermion_force());
                SMG_TRY(kick(ff, nullptr, (1.0 - 2.0 * lam) * h));
                SMG_TRY(inner(0.5 * h));
                SMG_TRY(fermion_force());
                SMG_TRY(kick(ff, nullptr, o < p.n_steps - 1 ? 2.0 * lam * h : lam * h));
            }
        } else {
            SMG_TRY(fermion_force());
            SMG_TRY(kick(ff, nullptr, 0.5 * h));
            for (int o = 0; o < p.n_steps; ++o) {
                SMG_TRY(inner(h));
                SMG_TRY(fermion_force());
                SMG_TRY(kick(ff, nullptr, o < p.n_steps - 1 ? h : 0.5 * h));
            }
        }
        return SMG_OK;
    }
};

smg_status hmc_check(smg_gauge* g, const smg_hmc_params* p) {
    smg_context* ctx = g->ctx;
    if (p->n_steps < 1 || p->n_inner < 0 || !(p->tau > 0) || p->cg_maxiter < 1 || !(p->cg_tol > 0))
        return smg_fail(ctx, SMG_BAD_ARG, "hmc: n_steps >= 1, n_inner >= 0, tau > 0, cg_maxiter >= 1, cg_tol > 0");
    if (p->use_eo && (p->mixed_precision || g->g.L % 2))
        return smg_fail(ctx, SMG_UNSUPPORTED, "hmc: the even-odd path runs FP64 solves on an even L");
    return SMG_OK;
}

// device state of one trajectory; the links at entry are kept in U_old
smg_status hmc_setup(Hmc& h, smg_gauge* g, double mass, double wilson_r, const smg_hmc_params* p) {
    smg_context* ctx = g->ctx;
    h.ctx = ctx;
    h.g = g;
    h.p = *p;
    h.mass = mass;
    h.r = wilson_r;
    const int V = g->g.V, L = g->g.L;
    const size_t fb = (size_t)2 * V * sizeof(double);
    SMG_CUDA(ctx, cudaMalloc(&h.pi, fb));
    SMG_CUDA(ctx, cudaMalloc(&h.gf, fb));
    SMG_CUDA(ctx, cudaMalloc(&h.ff, fb));
    SMG_CUDA(ctx, cudaMalloc(&h.scal, 64));
    SMG_CUDA(ctx, cudaMalloc(&h.U_old, (size_t)2 * V * sizeof(cx<double>)));
    SMG_CUDA(ctx, cudaMemcpyAsync(h.U_old, g->U64, (size_t)2 * V * sizeof(cx<double>), cudaMemcpyDeviceToDevice,
                                  ctx->stream));
    SMG_TRY(smg_field_create(ctx, L, 1, SMG_F64, &h.phi));
    SMG_TRY(smg_field_create(ctx, L, 1, SMG_F64, &h.X));
    SMG_TRY(smg_field_create(ctx, L, 1, SMG_F64, &h.eta));
    SMG_TRY(smg_dirac_create(g, mass, wilson_r, p->c_sw, p->mu_t, &h.d));
    h.eo = p->use_eo != 0;
    if (h.eo) {
        SMG_TRY(smg_field_create(ctx, L, 1, SMG_F64, &h.chi));
        SMG_TRY(smg_field_create(ctx, L, 1, SMG_F64, &h.psi));
        SMG_CUDA(ctx, cudaMalloc(&h.W, (size_t)V * sizeof(double)));
        SMG_CUDA(ctx, cudaMemsetAsync(h.phi->data, 0, h.phi->bytes, ctx->stream));
        SMG_CUDA(ctx, cudaMemsetAsync(h.eta->data, 0, h.eta->bytes, ctx->stream));
    }
    return SMG_OK;
}

// momenta: MomentumField::randomise (hmc_forces.cpp:64-69), mu-major then site order
smg_status hmc_draw_momenta(Hmc& h, smg_rng* rng) {
    smg_context* ctx = h.ctx;
    std::vector<double> pi_h((size_t)h.n2());
    std::normal_distribution<double> dist(0.0, 1.0);
    for (auto& v : pi_h) v = dist(rng->gen);
    SMG_CUDA(ctx, cudaMemcpyAsync(h.pi, pi_h.data(), pi_h.size() * sizeof(double), cudaMemcpyHostToDevice,
                                  ctx->stream));
    SMG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return SMG_OK;
}

smg_status hmc_draw_pseudofermion(Hmc& h, smg_rng* rng) {
    smg_context* ctx = h.ctx;
    const int V = h.g->g.V;
    if (h.eo) {
        // phi_o = M^dag eta_o, eta_o = random_vec(V, rng) on the odd sites
        // (generate_pseudofermion_eo, src/dirac.h:491-497); the odd half of a field is the
        // reference's half vector in order
        std::vector<double> eta_h((size_t)2 * V);
        std::normal_distribution<double> dist(0.0, 1.0);
        for (size_t i = 0; i < (size_t)V; ++i) {
            const double im = dist(rng->gen);
            const double re = dist(rng->gen);
            eta_h[2 * i] = re;
            eta_h[2 * i + 1] = im;
        }
        SMG_CUDA(ctx, cudaMemcpyAsync((char*)h.eta->data + h.eta->bytes / 2, eta_h.data(), h.eta->bytes / 2,
                                      cudaMemcpyHostToDevice, ctx->stream));
        SMG_TRY(smg_eo_schur_internal(h.d, true, h.eta, h.phi, h.chi, nullptr));
        SMG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        return SMG_OK;
    }
    // pseudofermion phi = D^dag eta, eta = random_vec(n, rng) (hmc_trajectory.cpp:32-36); the
    // reference's random_vec draws each entry's imaginary part first (GCC argument order)
    std::vector<double> eta_h((size_t)4 * V);
    std::normal_distribution<double> dist(0.0, 1.0);
    for (size_t i = 0; i < (size_t)2 * V; ++i) {
        const double im = dist(rng->gen);
        const double re = dist(rng->gen);
        eta_h[2 * i] = re;
        eta_h[2 * i + 1] = im;
    }
    SMG_TRY(smg_field_upload(h.eta, eta_h.data()));
    return smg_dirac_apply(h.d, SMG_OP_DDAG, h.eta, h.phi);
}

smg_status ms_check(smg_gauge* g, const smg_ms_params* p, smg_mg* mg) {
    smg_context* ctx = g->ctx;
    if (p->n_outer < 1 || p->n_inner < 1 || !(p->tau > 0) || p->cg_maxiter < 1 || !(p->cg_tol > 0) ||
        p->inner_smooth < 0 || p->outer_type < SMG_OUTER_LEAPFROG || p->outer_type > SMG_OUTER_FGI_QPQPQ)
        return smg_fail(ctx, SMG_BAD_ARG,
                        "multiscale hmc: n_outer, n_inner >= 1, tau > 0, cg_maxiter >= 1, cg_tol > 0, "
                        "inner_smooth >= 0, outer_type in [0, 3]");
    if (smg_mg_dirac(mg)->gauge != g)
        return smg_fail(ctx, SMG_BAD_ARG, "multiscale hmc: the hierarchy must be built on the trajectory's gauge field");
    return SMG_OK;
}

// the device state of a multi-timescale trajectory; mu_t as given (the reversibility test passes 0)
smg_status ms_setup(Hmc& h, smg_gauge* g, double mass, double wilson_r, const smg_ms_params* p, double mu_t,
                    smg_mg* mg) {
    smg_hmc_params hp{};
    smg_hmc_params_default(&hp);
    hp.beta = p->beta;
    hp.tau = p->tau;
    hp.n_steps = p->n_outer;
    hp.cg_maxiter = p->cg_maxiter;
    hp.cg_tol = p->cg_tol;
    hp.c_sw = p->c_sw;
    hp.mu_t = mu_t;
    SMG_TRY(hmc_setup(h, g, mass, wilson_r, &hp));
    smg_context* ctx = g->ctx;
    const int L = g->g.L;
    const size_t fb = (size_t)h.n2() * sizeof(double);
    h.mg = mg;
    h.mg_stale = true;
    h.inner_smooth = p->inner_smooth;
    h.n_inner = p->n_inner;
    SMG_CUDA(ctx, cudaMalloc(&h.fl, fb));
    SMG_CUDA(ctx, cudaMalloc(&h.fo, fb));
    SMG_CUDA(ctx, cudaMalloc(&h.pi_save, fb));
    SMG_CUDA(ctx, cudaMalloc(&h.U_save, (size_t)h.n2() * sizeof(cx<double>)));
    SMG_TRY(smg_field_create(ctx, L, 1, SMG_F64, &h.xl));
    SMG_TRY(smg_field_create(ctx, L, 1, SMG_F64, &h.rl));
    SMG_TRY(smg_field_create(ctx, L, 1, SMG_F64, &h.tl));
    return SMG_OK;
}

}  // namespace

// gauge_force into a device array (defined next to the kernel in gauge.cu)

extern "C" {

SMG_API smg_status smg_rng_create(uint32_t seed, smg_rng** out) {
    if (!out) return SMG_BAD_ARG;
    *out = new smg_rng{std::mt19937(seed)};
    return SMG_OK;
}

SMG_API smg_status smg_rng_destroy(smg_rng* rng) {
    delete rng;
    return SMG_OK;
}

SMG_API smg_status smg_rng_uniform(smg_rng* rng, double* out) {
    if (!rng || !out) return SMG_BAD_ARG;
    std::uniform_real_distribution<double> uniform(0.0, 1.0);
    *out = uniform(rng->gen);
    return SMG_OK;
}

SMG_API smg_status smg_rng_normal(smg_rng* rng, int64_t n, double* out) {
    if (!rng || n < 0 || (!out && n > 0)) return SMG_BAD_ARG;
    std::normal_distribution<double> dist(0.0, 1.0);
    for (int64_t i = 0; i < n; ++i) out[i] = dist(rng->gen);
    return SMG_OK;
}

SMG_API smg_status smg_hmc_params_default(smg_hmc_params* p) {
    if (!p) return SMG_BAD_ARG;
    *p = smg_hmc_params{};
    p->beta = 4.0;
    p->tau = 1.0;
    p->n_steps = 10;
    p->omelyan = 1;
    p->n_inner = 0;
    p->cg_maxiter = 10000;
    p->cg_tol = 1e-10;
    p->c_sw = 0.0;
    p->mu_t = 0.0;
    p->force_accept = 0;
    p->mixed_precision = 0;
    return SMG_OK;
}

SMG_API smg_status smg_hmc_trajectory(smg_gauge* g, double mass, double wilson_r, const smg_hmc_params* p,
                                      smg_rng* rng, smg_hmc_result* res) {
    if (!g || !p || !rng) return SMG_BAD_ARG;
    smg_context* ctx = g->ctx;
    SMG_TRY(hmc_check(g, p));
    const int V = g->g.V;
    Hmc h;
    SMG_TRY(hmc_setup(h, g, mass, wilson_r, p));
    SMG_TRY(hmc_draw_momenta(h, rng));
    SMG_TRY(hmc_draw_pseudofermion(h, rng));

    double KE0 = 0, SG0 = 0, SF0 = 0, LD0 = 0;
    SMG_TRY(h.hamiltonian(&KE0, &SG0, &SF0, &LD0));
    SMG_TRY(h.evolve());
    double KE1 = 0, SG1 = 0, SF1 = 0, LD1 = 0;
    SMG_TRY(h.hamiltonian(&KE1, &SG1, &SF1, &LD1));
    const double dH = (KE1 + SG1 + SF1 + LD1) - (KE0 + SG0 + SF0 + LD0);
    // Metropolis (hmc_trajectory.cpp:226-228): the uniform draw happens only when needed
    bool accept = p->force_accept != 0 || dH < 0;
    if (!accept) {
        std::uniform_real_distribution<double> uniform(0.0, 1.0);
        accept = uniform(rng->gen) < std::exp(-dH);
    }
    if (!accept) {
        SMG_CUDA(ctx, cudaMemcpyAsync(g->U64, h.U_old, (size_t)2 * V * sizeof(cx<double>), cudaMemcpyDeviceToDevice,
                                      ctx->stream));
        SMG_TRY(smg_gauge_ensure_f32(g));
    }
    double plaq = 0;
    SMG_TRY(smg_gauge_avg_plaq(g, &plaq));
    if (res) {
        res->accepted = accept ? 1 : 0;
        res->dH = dH;
        res->dKE = KE1 - KE0;
        res->dSG = SG1 - SG0;
        res->dSF = SF1 - SF0;
        res->total_cg_iters = h.cg_iters;
        res->solves = h.solves;
        res->plaquette = plaq;
        res->dLD = LD1 - LD0;
    }
    return SMG_OK;
}

SMG_API smg_status smg_coarse_lowmode_force(smg_dirac* d, smg_mg* mg, const smg_field* phi, int smooth_iters,
                                            double* force) {
    if (!d || !mg || !phi || !force || smooth_iters < 0) return SMG_BAD_ARG;
    smg_context* ctx = d->ctx;
    if (phi->prec != SMG_F64 || phi->nrhs != 1 || phi->g.L != d->gauge->g.L ||
        smg_mg_dirac(mg)->gauge->g.L != d->gauge->g.L)
        return smg_fail(ctx, SMG_BAD_ARG, "coarse_lowmode_force: single-RHS F64 phi on the hierarchy's lattice");
    const int L = phi->g.L;
    smg_field *xl = nullptr, *rl = nullptr, *tl = nullptr;
    double* F = nullptr;
    const size_t fb = (size_t)2 * phi->g.V * sizeof(double);
    smg_status st = smg_field_create(ctx, L, 1, SMG_F64, &xl);
    if (st == SMG_OK) st = smg_field_create(ctx, L, 1, SMG_F64, &rl);
    if (st == SMG_OK) st = smg_field_create(ctx, L, 1, SMG_F64, &tl);
    if (st == SMG_OK && cudaMalloc(&F, fb) != cudaSuccess) st = smg_fail(ctx, SMG_NO_MEMORY, "force buffer");
    if (st == SMG_OK) st = lowmode_force_fields(d, mg, phi, smooth_iters, xl, rl, tl, F);
    if (st == SMG_OK && cudaMemcpyAsync(force, F, fb, cudaMemcpyDeviceToHost, ctx->stream) != cudaSuccess)
        st = smg_fail(ctx, SMG_DEVICE_ERROR, "force copy");
    cudaStreamSynchronize(ctx->stream);
    if (F) cudaFree(F);
    smg_field_destroy(xl);
    smg_field_destroy(rl);
    smg_field_destroy(tl);
    return st;
}

SMG_API smg_status smg_ms_params_default(smg_ms_params* p) {
    if (!p) return SMG_BAD_ARG;
    *p = smg_ms_params{};
    p->beta = 4.0;
    p->tau = 1.0;
    p->n_outer = 4;
    p->n_inner = 5;
    p->cg_maxiter = 500;
    p->cg_tol = 1e-10;
    p->inner_smooth = 3;
    p->outer_type = SMG_OUTER_LEAPFROG;
    return SMG_OK;
}

SMG_API smg_status smg_hmc_mg_multiscale(smg_gauge* g, double mass, double wilson_r, const smg_ms_params* p,
                                         smg_mg* mg, smg_rng* rng, smg_ms_result* res) {
    if (!g || !p || !mg || !rng) return SMG_BAD_ARG;
    smg_context* ctx = g->ctx;
    SMG_TRY(ms_check(g, p, mg));
    Hmc h;
    SMG_TRY(ms_setup(h, g, mass, wilson_r, p, p->mu_t, mg));
    // momenta, then the pseudofermion twice (the first draw is overwritten,
    // src/hmc_multiscale.cpp:360-384)
    SMG_TRY(hmc_draw_momenta(h, rng));
    SMG_TRY(hmc_draw_pseudofermion(h, rng));
    SMG_TRY(hmc_draw_pseudofermion(h, rng));
    double KE0 = 0, SG0 = 0, SF0 = 0, LD0 = 0;
    SMG_TRY(h.hamiltonian(&KE0, &SG0, &SF0, &LD0));
    SMG_TRY(h.evolve_multiscale(p->outer_type, p->n_outer, p->tau));
    double KE1 = 0, SG1 = 0, SF1 = 0, LD1 = 0;
    SMG_TRY(h.hamiltonian(&KE1, &SG1, &SF1, &LD1));
    const double dH = (KE1 + SG1 + SF1) - (KE0 + SG0 + SF0);
    // Metropolis (src/hmc_multiscale.cpp:874-876)
    bool accept = dH < 0;
    if (!accept) {
        std::uniform_real_distribution<double> uniform(0.0, 1.0);
        accept = uniform(rng->gen) < std::exp(-dH);
    }
    if (!accept) {
        SMG_CUDA(ctx, cudaMemcpyAsync(g->U64, h.U_old, (size_t)h.n2() * sizeof(cx<double>), cudaMemcpyDeviceToDevice,
                                      ctx->stream));
        SMG_TRY(smg_gauge_ensure_f32(g));
    }
    // the hierarchy's Dirac operator follows the links the trajectory leaves
    if (smg_mg_dirac(mg) != h.d) SMG_TRY(smg_dirac_refresh(smg_mg_dirac(mg)));
    double plaq = 0;
    SMG_TRY(smg_gauge_avg_plaq(g, &plaq));
    if (res) {
        res->accepted = accept ? 1 : 0;
        res->dH = dH;
        res->dKE = KE1 - KE0;
        res->dSG = SG1 - SG0;
        res->dSF = SF1 - SF0;
        res->highmode_cg_iters = h.cg_iters;
        res->lowmode_force_evals = h.lowmode_evals;
        res->solves = h.solves;
        res->plaquette = plaq;
    }
    return SMG_OK;
}

SMG_API smg_status smg_hmc_mg_multiscale_reversibility(smg_gauge* g, double mass, double wilson_r,
                                                       const smg_ms_params* p, smg_mg* mg, smg_rng* rng,
                                                       smg_reversibility_result* res) {
    if (!g || !p || !mg || !rng || !res) return SMG_BAD_ARG;
    smg_context* ctx = g->ctx;
    SMG_TRY(ms_check(g, p, mg));
    Hmc h;
    // DiracOp(lat, gauge, mass, wilson_r, c_sw) of mg_ms_md_evolve: mu_t = 0 (src/hmc_multiscale.cpp:904)
    SMG_TRY(ms_setup(h, g, mass, wilson_r, p, 0.0, mg));
    SMG_TRY(hmc_draw_momenta(h, rng));
    SMG_TRY(hmc_draw_pseudofermion(h, rng));
    const int n2 = h.n2();
    // mg_ms_md_evolve runs FGI_QPQPQ as FGI (src/hmc_multiscale.cpp:933)
    const int outer = p->outer_type == SMG_OUTER_FGI_QPQPQ ? SMG_OUTER_FGI : p->outer_type;
    std::vector<double> pi0((size_t)n2), pi1((size_t)n2);
    SMG_CUDA(ctx, cudaMemcpyAsync(pi0.data(), h.pi, (size_t)n2 * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    double KE0 = 0, SG0 = 0, SF0 = 0, LD0 = 0, KE1 = 0, SG1 = 0, SF1 = 0, LD1 = 0, KE2 = 0, SG2 = 0, SF2 = 0, LD2 = 0;
    SMG_TRY(h.hamiltonian(&KE0, &SG0, &SF0, &LD0));
    SMG_TRY(h.evolve_multiscale(outer, p->n_outer, p->tau));
    SMG_TRY(h.hamiltonian(&KE1, &SG1, &SF1, &LD1));
    k_negate<<<(n2 + 255) / 256, 256, 0, ctx->stream>>>(h.pi, n2);
    count_launch(ctx);
    SMG_CHECK_LAUNCH(ctx);
    SMG_TRY(h.evolve_multiscale(outer, p->n_outer, p->tau));
    SMG_TRY(h.hamiltonian(&KE2, &SG2, &SF2, &LD2));
    std::vector<cx<double>> u0((size_t)n2), u1((size_t)n2);
    SMG_CUDA(ctx, cudaMemcpyAsync(u0.data(), h.U_old, (size_t)n2 * sizeof(cx<double>), cudaMemcpyDeviceToHost,
                                  ctx->stream));
    SMG_CUDA(ctx, cudaMemcpyAsync(u1.data(), g->U64, (size_t)n2 * sizeof(cx<double>), cudaMemcpyDeviceToHost,
                                  ctx->stream));
    SMG_CUDA(ctx, cudaMemcpyAsync(pi1.data(), h.pi, (size_t)n2 * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    SMG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    double un = 0, ud = 0, pn = 0, pd = 0;
    for (int i = 0; i < n2; ++i) {
        const double dr = u1[i].re - u0[i].re, di = u1[i].im - u0[i].im;
        un += u0[i].re * u0[i].re + u0[i].im * u0[i].im;
        ud += dr * dr + di * di;
        const double dp = pi1[i] + pi0[i];
        pn += pi0[i] * pi0[i];
        pd += dp * dp;
    }
    SMG_CUDA(ctx, cudaMemcpyAsync(g->U64, h.U_old, (size_t)n2 * sizeof(cx<double>), cudaMemcpyDeviceToDevice,
                                  ctx->stream));
    SMG_TRY(smg_gauge_ensure_f32(g));
    if (smg_mg_dirac(mg) != h.d) SMG_TRY(smg_dirac_refresh(smg_mg_dirac(mg)));
    SMG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    res->gauge_delta = std::sqrt(ud / std::max(un, 1e-30));
    res->mom_delta = std::sqrt(pd / std::max(pn, 1e-30));
    res->dH_forward = (KE1 + SG1 + SF1) - (KE0 + SG0 + SF0);
    res->dH_backward = (KE2 + SG2 + SF2) - (KE1 + SG1 + SF1);
    res->total_cg_iters = h.cg_iters;
    res->solves = h.solves;
    return SMG_OK;
}

SMG_API smg_status smg_hmc_reversibility(smg_gauge* g, double mass, double wilson_r, const smg_hmc_params* p,
                                         smg_rng* rng, smg_reversibility_result* res) {
    if (!g || !p || !rng || !res) return SMG_BAD_ARG;
    smg_context* ctx = g->ctx;
    SMG_TRY(hmc_check(g, p));
    const int n2 = 2 * g->g.V;
    Hmc h;
    SMG_TRY(hmc_setup(h, g, mass, wilson_r, p));
    // the reference draws the pseudofermion before the momenta here (hmc_trajectory.cpp:428-433)
    SMG_TRY(hmc_draw_pseudofermion(h, rng));
    SMG_TRY(hmc_draw_momenta(h, rng));
    std::vector<double> pi0((size_t)n2), pi1((size_t)n2);
    SMG_CUDA(ctx, cudaMemcpyAsync(pi0.data(), h.pi, (size_t)n2 * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));

    double KE0 = 0, SG0 = 0, SF0 = 0, LD0 = 0, KE1 = 0, SG1 = 0, SF1 = 0, LD1 = 0, KE2 = 0, SG2 = 0, SF2 = 0, LD2 = 0;
    SMG_TRY(h.hamiltonian(&KE0, &SG0, &SF0, &LD0));
    SMG_TRY(h.evolve());
    SMG_TRY(h.hamiltonian(&KE1, &SG1, &SF1, &LD1));
    k_negate<<<(n2 + 255) / 256, 256, 0, ctx->stream>>>(h.pi, n2);
    count_launch(ctx);
    SMG_CHECK_LAUNCH(ctx);
    SMG_TRY(h.evolve());
    SMG_TRY(h.hamiltonian(&KE2, &SG2, &SF2, &LD2));

    // relative differences of the links and of the flipped momenta (hmc_trajectory.cpp:484-503)
    std::vector<cx<double>> u0((size_t)n2), u1((size_t)n2);
    SMG_CUDA(ctx, cudaMemcpyAsync(u0.data(), h.U_old, (size_t)n2 * sizeof(cx<double>), cudaMemcpyDeviceToHost,
                                  ctx->stream));
    SMG_CUDA(ctx, cudaMemcpyAsync(u1.data(), g->U64, (size_t)n2 * sizeof(cx<double>), cudaMemcpyDeviceToHost,
                                  ctx->stream));
    SMG_CUDA(ctx, cudaMemcpyAsync(pi1.data(), h.pi, (size_t)n2 * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    SMG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    double un = 0, ud = 0, pn = 0, pd = 0;
    for (int i = 0; i < n2; ++i) {
        const double dr = u1[i].re - u0[i].re, di = u1[i].im - u0[i].im;
        un += u0[i].re * u0[i].re + u0[i].im * u0[i].im;
        ud += dr * dr + di * di;
        const double dp = -pi1[i] - pi0[i];
        pn += pi0[i] * pi0[i];
        pd += dp * dp;
    }
    // the links at entry are restored
    SMG_CUDA(ctx, cudaMemcpyAsync(g->U64, h.U_old, (size_t)n2 * sizeof(cx<double>), cudaMemcpyDeviceToDevice,
                                  ctx->stream));
    SMG_TRY(smg_gauge_ensure_f32(g));
    SMG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    res->gauge_delta = std::sqrt(ud / std::max(un, 1e-30));
    res->mom_delta = std::sqrt(pd / std::max(pn, 1e-30));
    res->dH_forward = (KE1 + SG1 + SF1 + LD1) - (KE0 + SG0 + SF0 + LD0);
    res->dH_backward = (KE2 + SG2 + SF2 + LD2) - (KE1 + SG1 + SF1 + LD1);
    res->total_cg_iters = h.cg_iters;
    res->solves = h.solves;
    return SMG_OK;
}

}  // extern "C"
