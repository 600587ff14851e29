/* ORACLE TEST INFRASTRUCTURE — not part of the product.
 *
 * Plain-C (C99 complex + OpenMP) restatement of the reference's Wilson-clover
 * Dirac operator and MG solve path.  Each function cites the reference
 * file:line it follows and keeps the reference's operation order, so on the
 * same inputs it reproduces the reference to rounding (exactly, where the
 * compiler does not contract multiply-adds).  Loaded only by tests/,
 * __graft_entry__.smoke() and bench.py's CPU-baseline leg. */
#include "smg_oracle.h"

#include <complex.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef double complex cxd;

/* ------------------------------------------------------------------ threads */
void orc_set_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}
int orc_get_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* ---------------------------------------------------------- lattice helpers */
/* Lattice::idx/xp/xm/yp/ym (reference src/lattice.h:19-24) */
static inline int l_idx(int L, int x, int y) { return ((x % L + L) % L) + L * ((y % L + L) % L); }
static inline int l_xp(int L, int s) { return l_idx(L, s % L + 1, s / L); }
static inline int l_xm(int L, int s) { return l_idx(L, s % L - 1, s / L); }
static inline int l_yp(int L, int s) { return l_idx(L, s % L, s / L + 1); }
static inline int l_ym(int L, int s) { return l_idx(L, s % L, s / L - 1); }

static inline cxd ld(const double* p, long i) { return p[2 * i] + I * p[2 * i + 1]; }
static inline void st(double* p, long i, cxd z) {
    p[2 * i] = creal(z);
    p[2 * i + 1] = cimag(z);
}
static cxd* to_cx(const double* p, long n) {
    cxd* v = (cxd*)malloc(sizeof(cxd) * (size_t)n);
    for (long i = 0; i < n; ++i) v[i] = ld(p, i);
    return v;
}
static void from_cx(const cxd* v, long n, double* p) {
    for (long i = 0; i < n; ++i) st(p, i, v[i]);
}

/* ------------------------------------------------------------------- BLAS-1 */
/* dot = sum conj(a) b with separate re/im reductions (reference src/linalg.cpp:8-18) */
static cxd v_dot(const cxd* a, const cxd* b, long n) {
    double re = 0, im = 0;
#pragma omp parallel for reduction(+ : re, im) schedule(static) if (n > 4096)
    for (long i = 0; i < n; ++i) {
        cxd p = conj(a[i]) * b[i];
        re += creal(p);
        im += cimag(p);
    }
    return re + I * im;
}
static double v_norm(const cxd* v, long n) { return sqrt(creal(v_dot(v, v, n))); }
static void v_axpy(cxd a, const cxd* x, cxd* y, long n) { /* linalg.cpp:22-26 */
#pragma omp parallel for schedule(static) if (n > 4096)
    for (long i = 0; i < n; ++i) y[i] += a * x[i];
}
static void v_scale(cxd* v, cxd a, long n) { /* linalg.cpp:35-39 */
#pragma omp parallel for schedule(static) if (n > 4096)
    for (long i = 0; i < n; ++i) v[i] *= a;
}

/* --------------------------------------------------------------- gauge field */
typedef struct {
    int L, V;
    const cxd* U0;
    const cxd* U1;
    cxd* store;
} Gauge;

static Gauge g_make(int L, const double* U) {
    Gauge g;
    g.L = L;
    g.V = L * L;
    g.store = to_cx(U, 2L * g.V);
    g.U0 = g.store;
    g.U1 = g.store + g.V;
    return g;
}
static void g_free(Gauge* g) { free(g->store); }

/* GaugeField::plaq (reference src/gauge.h:26-30) */
static inline cxd g_plaq(const Gauge* g, int s) {
    int sp0 = l_xp(g->L, s), sp1 = l_yp(g->L, s);
    return g->U0[s] * g->U1[sp0] * conj(g->U0[sp1]) * conj(g->U1[s]);
}

double orc_avg_plaq(int L, const double* U) { /* gauge.h:32-36 */
    Gauge g = g_make(L, U);
    double s = 0;
#pragma omp parallel for reduction(+ : s) schedule(static)
    for (int i = 0; i < g.V; ++i) s += creal(g_plaq(&g, i));
    g_free(&g);
    return s / (L * L);
}

/* DiracOp::compute_clover_field (reference src/dirac.h:26-52) */
static void clover_field(const Gauge* g, double* F) {
    int L = g->L;
#pragma omp parallel for schedule(static)
    for (int s = 0; s < g->V; ++s) {
        int sxp = l_xp(L, s), sxm = l_xm(L, s), syp = l_yp(L, s), sym = l_ym(L, s);
        cxd P_ur = g->U0[s] * g->U1[sxp] * conj(g->U0[syp]) * conj(g->U1[s]);
        int sxmyp = l_yp(L, sxm);
        cxd P_ul = g->U1[s] * conj(g->U0[sxmyp]) * conj(g->U1[sxm]) * g->U0[sxm];
        int sxmym = l_ym(L, sxm);
        cxd P_ll = conj(g->U0[sxm]) * conj(g->U1[sxmym]) * g->U0[sxmym] * g->U1[sym];
        int sxpym = l_ym(L, sxp);
        cxd P_lr = conj(g->U1[sym]) * g->U0[sym] * g->U1[sxpym] * conj(g->U0[s]);
        cxd Q = P_ur + P_ul + P_ll + P_lr;
        F[s] = cimag(Q) / 4.0;
    }
}

void orc_clover(int L, const double* U, double* F01) {
    Gauge g = g_make(L, U);
    clover_field(&g, F01);
    g_free(&g);
}

/* ------------------------------------------------------------ Dirac operator */
typedef struct {
    Gauge g;
    double mass, r, csw, mu;
    double* F; /* clover field or NULL */
} Dirac;

static Dirac d_make(int L, const double* U, double m, double r, double csw, double mu) {
    Dirac d;
    d.g = g_make(L, U);
    d.mass = m;
    d.r = r;
    d.csw = csw;
    d.mu = mu;
    d.F = NULL;
    if (csw != 0.0) {
        d.F = (double*)malloc(sizeof(double) * (size_t)d.g.V);
        clover_field(&d.g, d.F);
    }
    return d;
}
static void d_free(Dirac* d) {
    g_free(&d->g);
    free(d->F);
}

/* accumulate_hops with unit scales (reference src/dirac.h:58-89) */
static inline void accumulate_hops(cxd* d0, cxd* d1, int s, const cxd* src, const Gauge* g, double r) {
    const int L = g->L;
    {
        int sf = l_xp(L, s);
        cxd u = g->U0[s];
        cxd up0 = u * src[2 * sf], up1 = u * src[2 * sf + 1];
        *d0 -= 0.5 * (r * up0 - up1);
        *d1 -= 0.5 * (-up0 + r * up1);
    }
    {
        int sb = l_xm(L, s);
        cxd ud = conj(g->U0[sb]);
        cxd udq0 = ud * src[2 * sb], udq1 = ud * src[2 * sb + 1];
        *d0 -= 0.5 * (r * udq0 + udq1);
        *d1 -= 0.5 * (udq0 + r * udq1);
    }
    {
        int sf = l_yp(L, s);
        cxd u = g->U1[s];
        cxd up0 = u * src[2 * sf], up1 = u * src[2 * sf + 1];
        *d0 -= 0.5 * (r * up0 + I * up1);
        *d1 -= 0.5 * (-I * up0 + r * up1);
    }
    {
        int sb = l_ym(L, s);
        cxd ud = conj(g->U1[sb]);
        cxd udq0 = ud * src[2 * sb], udq1 = ud * src[2 * sb + 1];
        *d0 -= 0.5 * (r * udq0 - I * udq1);
        *d1 -= 0.5 * (I * udq0 + r * udq1);
    }
}

/* DiracOp::apply_impl (reference src/dirac.h:93-113) */
static void apply_impl(const Dirac* D, const cxd* src, cxd* dst, double mu_eff) {
    const int V = D->g.V;
    const int has_clover = D->csw != 0.0, has_twist = mu_eff != 0.0;
#pragma omp parallel for schedule(static) if (V > 4096)
    for (int s = 0; s < V; ++s) {
        cxd s0 = src[2 * s], s1 = src[2 * s + 1];
        double diag = 2.0 * D->r + D->mass;
        cxd o0, o1;
        if (has_clover || has_twist) {
            double C = has_clover ? 0.5 * D->csw * D->F[s] : 0.0;
            cxd d0 = (diag + C) + I * mu_eff;
            cxd d1 = (diag - C) - I * mu_eff;
            o0 = d0 * s0;
            o1 = d1 * s1;
        } else {
            o0 = diag * s0;
            o1 = diag * s1;
        }
        accumulate_hops(&o0, &o1, s, src, &D->g, D->r);
        dst[2 * s] = o0;
        dst[2 * s + 1] = o1;
    }
}

/* apply (dirac.h:115), apply_dag = g5 D(-mu) g5 (dirac.h:120-134) */
static void d_apply(const Dirac* D, const cxd* src, cxd* dst) { apply_impl(D, src, dst, D->mu); }
static void d_apply_dag(const Dirac* D, const cxd* src, cxd* dst) {
    const int V = D->g.V;
    cxd* g5src = (cxd*)malloc(sizeof(cxd) * 2 * (size_t)V);
    cxd* g5dst = (cxd*)malloc(sizeof(cxd) * 2 * (size_t)V);
#pragma omp parallel for schedule(static) if (V > 4096)
    for (int s = 0; s < V; ++s) {
        g5src[2 * s] = src[2 * s];
        g5src[2 * s + 1] = -src[2 * s + 1];
    }
    apply_impl(D, g5src, g5dst, -D->mu);
#pragma omp parallel for schedule(static) if (V > 4096)
    for (int s = 0; s < V; ++s) {
        dst[2 * s] = g5dst[2 * s];
        dst[2 * s + 1] = -g5dst[2 * s + 1];
    }
    free(g5src);
    free(g5dst);
}
/* apply_DdagD (dirac.h:136-140) */
static void d_apply_DdagD(const Dirac* D, const cxd* src, cxd* dst) {
    cxd* tmp = (cxd*)malloc(sizeof(cxd) * 2 * (size_t)D->g.V);
    d_apply(D, src, tmp);
    d_apply_dag(D, tmp, dst);
    free(tmp);
}

void orc_dirac(int L, const double* U, double m, double r, double csw, double mu, int op, const double* src,
               double* dst) {
    Dirac D = d_make(L, U, m, r, csw, mu);
    long n = 2L * D.g.V;
    cxd* s = to_cx(src, n);
    cxd* d = (cxd*)malloc(sizeof(cxd) * (size_t)n);
    switch (op) {
        case 0: d_apply(&D, s, d); break;
        case 1: d_apply_dag(&D, s, d); break;
        case 2: d_apply_DdagD(&D, s, d); break;
        default: /* apply_g5D, dirac.h:145-152 */
            apply_impl(&D, s, d, D.mu);
            for (int q = 0; q < D.g.V; ++q) d[2 * q + 1] = -d[2 * q + 1];
            break;
    }
    from_cx(d, n, dst);
    free(s);
    free(d);
    d_free(&D);
}

/* -------------------------------------------------------------------- CG */
/* cg_solve_core without x0 / preconditioner (reference src/solvers.cpp:16-72) */
static int cg_core(const Dirac* D, const cxd* rhs, cxd* x, int max_iter, double tol, double* fres) {
    long n = 2L * D->g.V;
    double rhs_norm = v_norm(rhs, n);
    memset(x, 0, sizeof(cxd) * (size_t)n);
    if (rhs_norm < 1e-30) {
        if (fres) *fres = 0.0;
        return 0;
    }
    cxd* r = (cxd*)malloc(sizeof(cxd) * (size_t)n);
    cxd* p = (cxd*)malloc(sizeof(cxd) * (size_t)n);
    cxd* Ap = (cxd*)malloc(sizeof(cxd) * (size_t)n);
    memcpy(r, rhs, sizeof(cxd) * (size_t)n);
    memcpy(p, r, sizeof(cxd) * (size_t)n);
    cxd rz = v_dot(r, r, n);
    int iter = 0;
    while (iter < max_iter) {
        d_apply_DdagD(D, p, Ap);
        cxd pAp = v_dot(p, Ap, n);
        cxd alpha = rz / pAp;
#pragma omp parallel for schedule(static) if (n > 4096)
        for (long i = 0; i < n; ++i) {
            x[i] += alpha * p[i];
            r[i] -= alpha * Ap[i];
        }
        iter++;
        double rnorm = v_norm(r, n);
        if (rnorm / rhs_norm < tol) break;
        cxd rz_new = v_dot(r, r, n);
        cxd beta = rz_new / rz;
        rz = rz_new;
#pragma omp parallel for schedule(static) if (n > 4096)
        for (long i = 0; i < n; ++i) p[i] = r[i] + beta * p[i];
    }
    if (fres) *fres = v_norm(r, n) / rhs_norm;
    free(r);
    free(p);
    free(Ap);
    return iter;
}

int orc_cg(int L, const double* U, double m, double r, double csw, double mu, const double* b, double* x,
           int max_iter, double tol, double* final_res) {
    Dirac D = d_make(L, U, m, r, csw, mu);
    long n = 2L * D.g.V;
    cxd* bb = to_cx(b, n);
    cxd* xx = (cxd*)malloc(sizeof(cxd) * (size_t)n);
    int it = cg_core(&D, bb, xx, max_iter, tol, final_res);
    from_cx(xx, n, x);
    free(bb);
    free(xx);
    d_free(&D);
    return it;
}

/* ------------------------------------------------------- gauge force/action */
void orc_gauge_force(int L, const double* U, double beta, double* F) { /* hmc_forces.cpp:88-111 */
    Gauge g = g_make(L, U);
    const int V = g.V;
#pragma omp parallel for schedule(static)
    for (int s = 0; s < V; ++s) {
        {
            int sx = l_xp(L, s), sy = l_yp(L, s), smy = l_ym(L, s);
            int sxmy = l_ym(L, sx);
            cxd staple = g.U1[sx] * conj(g.U0[sy]) * conj(g.U1[s]) + conj(g.U1[sxmy]) * conj(g.U0[smy]) * g.U1[smy];
            F[s] = -beta * cimag(g.U0[s] * staple);
        }
        {
            int sy = l_yp(L, s), sx = l_xp(L, s), smx = l_xm(L, s);
            int symx = l_xm(L, sy);
            cxd staple = g.U0[sy] * conj(g.U1[sx]) * conj(g.U0[s]) + conj(g.U0[symx]) * conj(g.U1[smx]) * g.U0[smx];
            F[V + s] = -beta * cimag(g.U1[s] * staple);
        }
    }
    g_free(&g);
}

double orc_gauge_action(int L, const double* U, double beta) { /* hmc_forces.cpp:80-86 */
    Gauge g = g_make(L, U);
    double s = 0.0;
    for (int site = 0; site < g.V; ++site) s += creal(g_plaq(&g, site));
    g_free(&g);
    return -beta * s;
}

/* --------------------------------------------------------------- fermion force */
/* fermion_force = bilinear with chi = D X (reference src/hmc_forces.cpp:134-194)
 * plus the clover insertion in its final form (:409-492). */
void orc_fermion_force(int L, const double* U, double m, double r_, double csw, double mu, const double* Xh,
                       double* F) {
    Dirac D = d_make(L, U, m, r_, csw, mu);
    const int V = D.g.V;
    const double r = D.r;
    long n = 2L * V;
    cxd* X = to_cx(Xh, n);
    cxd* chi = (cxd*)malloc(sizeof(cxd) * (size_t)n);
    d_apply(&D, X, chi);
    const Gauge* g = &D.g;
#pragma omp parallel for schedule(static)
    for (int s = 0; s < V; ++s) {
        cxd chi_s0 = chi[2 * s], chi_s1 = chi[2 * s + 1];
        cxd x_s0 = X[2 * s], x_s1 = X[2 * s + 1];
        {
            int sf = l_xp(L, s);
            cxd u = g->U0[s], ud = conj(u);
            cxd ux0 = u * X[2 * sf], ux1 = u * X[2 * sf + 1];
            cxd fwd0 = r * ux0 - ux1, fwd1 = -ux0 + r * ux1;
            cxd c_fwd = conj(chi_s0) * fwd0 + conj(chi_s1) * fwd1;
            cxd udx0 = ud * x_s0, udx1 = ud * x_s1;
            cxd bwd0 = r * udx0 + udx1, bwd1 = udx0 + r * udx1;
            cxd c_bwd = conj(chi[2 * sf]) * bwd0 + conj(chi[2 * sf + 1]) * bwd1;
            F[s] = creal(I * c_bwd - I * c_fwd);
        }
        {
            int sf = l_yp(L, s);
            cxd u = g->U1[s], ud = conj(u);
            cxd ux0 = u * X[2 * sf], ux1 = u * X[2 * sf + 1];
            cxd fwd0 = r * ux0 + I * ux1, fwd1 = -I * ux0 + r * ux1;
            cxd c_fwd = conj(chi_s0) * fwd0 + conj(chi_s1) * fwd1;
            cxd udx0 = ud * x_s0, udx1 = ud * x_s1;
            cxd bwd0 = r * udx0 - I * udx1, bwd1 = I * udx0 + r * udx1;
            cxd c_bwd = conj(chi[2 * sf]) * bwd0 + conj(chi[2 * sf + 1]) * bwd1;
            F[V + s] = creal(I * c_bwd - I * c_fwd);
        }
    }
    if (csw != 0.0) {
        double* w = (double*)malloc(sizeof(double) * (size_t)V);
#pragma omp parallel for schedule(static)
        for (int s = 0; s < V; ++s) w[s] = creal(conj(chi[2 * s]) * X[2 * s] - conj(chi[2 * s + 1]) * X[2 * s + 1]);
#pragma omp parallel for schedule(static)
        for (int s = 0; s < V; ++s) {
            int sxp = l_xp(L, s), sxm = l_xm(L, s), syp = l_yp(L, s), sym = l_ym(L, s);
            int sxpym = l_ym(L, sxp), sxmyp = l_yp(L, sxm), sxpyp = l_yp(L, sxp);
            cxd P_UR_s = g->U0[s] * g->U1[sxp] * conj(g->U0[syp]) * conj(g->U1[s]);
            double re_P_fwd = creal(P_UR_s);
            double w_fwd = w[s] + w[sxp] + w[sxpyp] + w[syp];
            cxd P_UR_sym = g->U0[sym] * g->U1[sxpym] * conj(g->U0[s]) * conj(g->U1[sym]);
            double re_P_bwd = creal(P_UR_sym);
            double w_bwd = w[sym] + w[sxpym] + w[sxp] + w[s];
            F[s] += (csw / 4.0) * (re_P_fwd * w_fwd - re_P_bwd * w_bwd);
            cxd P_fwd_1 = g->U0[sxm] * g->U1[s] * conj(g->U0[sxmyp]) * conj(g->U1[sxm]);
            double re_P_fwd_1 = creal(P_fwd_1);
            double w_fwd_1 = w[sxm] + w[s] + w[syp] + w[sxmyp];
            double re_P_bwd_1 = creal(P_UR_s);
            double w_bwd_1 = w[s] + w[sxp] + w[sxpyp] + w[syp];
            F[V + s] += (csw / 4.0) * (re_P_fwd_1 * w_fwd_1 - re_P_bwd_1 * w_bwd_1);
        }
        free(w);
    }
    free(X);
    free(chi);
    d_free(&D);
}

/* ---------------------------------------------------------------- MR smoother */
/* mr_smooth (reference src/smoother.cpp:9-23) */
static void mr_smooth(const Dirac* D, cxd* x, const cxd* b, int niter) {
    long n = 2L * D->g.V;
    cxd* r = (cxd*)malloc(sizeof(cxd) * (size_t)n);
    cxd* Ar = (cxd*)malloc(sizeof(cxd) * (size_t)n);
    for (int it = 0; it < niter; ++it) {
        d_apply_DdagD(D, x, r);
#pragma omp parallel for schedule(static) if (n > 4096)
        for (long i = 0; i < n; ++i) r[i] = b[i] - r[i];
        d_apply_DdagD(D, r, Ar);
        cxd rAr = v_dot(Ar, r, n);
        cxd ArAr = v_dot(Ar, Ar, n);
        if (cabs(ArAr) < 1e-30) break;
        cxd omega = rAr / ArAr;
        v_axpy(omega, r, x, n);
    }
    free(r);
    free(Ar);
}

void orc_mr_smooth(int L, const double* U, double m, double r, double csw, double mu, const double* b, double* x,
                   int niter) {
    Dirac D = d_make(L, U, m, r, csw, mu);
    long n = 2L * D.g.V;
    cxd* bb = to_cx(b, n);
    cxd* xx = to_cx(x, n);
    mr_smooth(&D, xx, bb, niter);
    from_cx(xx, n, x);
    free(bb);
    free(xx);
    d_free(&D);
}

/* compute_near_null_space (reference src/multigrid.cpp:435-484); the k random
 * start vectors, which the reference draws with random_vec(n, rng), are given */
void orc_near_null_space(int L, const double* U, double m, double r, double csw, double mu, int k, int iters,
                         const double* init, double* out) {
    Dirac D = d_make(L, U, m, r, csw, mu);
    long n = 2L * D.g.V;
    cxd** nv = (cxd**)malloc(sizeof(cxd*) * (size_t)k);
    cxd* x_new = (cxd*)malloc(sizeof(cxd) * (size_t)n);
    for (int i = 0; i < k; ++i) {
        nv[i] = to_cx(init + 2 * n * i, n);
        double nrm = v_norm(nv[i], n);
        v_scale(nv[i], 1.0 / nrm, n);
        for (int it = 0; it < iters; ++it) {
            memset(x_new, 0, sizeof(cxd) * (size_t)n);
            mr_smooth(&D, x_new, nv[i], 5);
            for (int j = 0; j < i; ++j) {
                cxd proj = v_dot(nv[j], x_new, n);
                v_axpy(-proj, nv[j], x_new, n);
            }
            nrm = v_norm(x_new, n);
            if (nrm > 1e-14) {
                v_scale(x_new, 1.0 / nrm, n);
                memcpy(nv[i], x_new, sizeof(cxd) * (size_t)n);
            } else {
                break;
            }
        }
    }
    for (int i = 0; i < k; ++i) {
        for (int j = 0; j < i; ++j) {
            cxd proj = v_dot(nv[j], nv[i], n);
            v_axpy(-proj, nv[j], nv[i], n);
        }
        double nrm = v_norm(nv[i], n);
        if (nrm > 1e-14) v_scale(nv[i], 1.0 / nrm, n);
    }
    for (int i = 0; i < k; ++i) {
        from_cx(nv[i], n, out + 2 * n * i);
        free(nv[i]);
    }
    free(nv);
    free(x_new);
    d_free(&D);
}

/* ---------------------------------------------------------------- prolongator */
/* Prolongator block maps (reference src/prolongator.h:35-58): block
 * b = (x/bs) + nbx*(y/bs), local index (x%bs) + bs*(y%bs) */
typedef struct {
    int L, bs, k, nbx, nblocks, bdim;
    cxd* bv; /* [b][k][bdim] */
} Prol;

static inline int p_block(const Prol* P, int s) { return (s % P->L) / P->bs + P->nbx * ((s / P->L) / P->bs); }
static inline int p_local(const Prol* P, int s) { return (s % P->L) % P->bs + P->bs * ((s / P->L) % P->bs); }

static Prol p_make(int L, int bs, int k, const double* block_vecs) {
    Prol P;
    P.L = L;
    P.bs = bs;
    P.k = k;
    P.nbx = L / bs;
    P.nblocks = P.nbx * P.nbx;
    P.bdim = 2 * bs * bs;
    long tot = (long)P.nblocks * k * P.bdim;
    P.bv = block_vecs ? to_cx(block_vecs, tot) : (cxd*)calloc((size_t)tot, sizeof(cxd));
    return P;
}

/* orthonormalise_block (reference src/prolongator.h:111-130) */
static void p_orthonormalise_block(Prol* P, int b) {
    const int bd = P->bdim;
    for (int k = 0; k < P->k; ++k) {
        cxd* v = P->bv + ((long)b * P->k + k) * bd;
        for (int j = 0; j < k; ++j) {
            const cxd* u = P->bv + ((long)b * P->k + j) * bd;
            cxd proj = 0;
            for (int i = 0; i < bd; ++i) proj += conj(u[i]) * v[i];
            for (int i = 0; i < bd; ++i) v[i] -= proj * u[i];
        }
        double nn = 0;
        for (int i = 0; i < bd; ++i) nn += creal(v[i]) * creal(v[i]) + cimag(v[i]) * cimag(v[i]);
        nn = sqrt(nn);
        if (nn > 1e-14)
            for (int i = 0; i < bd; ++i) v[i] /= nn;
    }
}

/* build_from_vectors (reference src/prolongator.h:133-141) */
void orc_prolongator_build(int L, int bs, int k, const double* null_vecs, double* block_vecs) {
    Prol P = p_make(L, bs, k, NULL);
    const int V = L * L;
    for (int kk = 0; kk < k; ++kk) {
        const double* nv = null_vecs + (long)4 * V * kk;
        for (int s = 0; s < V; ++s) {
            int b = p_block(&P, s), loc = p_local(&P, s);
            cxd* v = P.bv + ((long)b * k + kk) * P.bdim;
            v[2 * loc] = ld(nv, 2L * s);
            v[2 * loc + 1] = ld(nv, 2L * s + 1);
        }
    }
#pragma omp parallel for schedule(static)
    for (int b = 0; b < P.nblocks; ++b) p_orthonormalise_block(&P, b);
    from_cx(P.bv, (long)P.nblocks * k * P.bdim, block_vecs);
    free(P.bv);
}

/* prolong (reference src/prolongator.h:77-90) */
static void p_prolong(const Prol* P, const cxd* coarse, cxd* fine) {
    const int V = P->L * P->L;
#pragma omp parallel for schedule(static) if (V > 4096)
    for (int s = 0; s < V; ++s) {
        int b = p_block(P, s), loc = p_local(P, s);
        cxd f0 = 0, f1 = 0;
        for (int k = 0; k < P->k; ++k) {
            cxd c = coarse[b * P->k + k];
            const cxd* v = P->bv + ((long)b * P->k + k) * P->bdim;
            f0 += c * v[2 * loc];
            f1 += c * v[2 * loc + 1];
        }
        fine[2 * s] = f0;
        fine[2 * s + 1] = f1;
    }
}

/* restrict_vec = P^dag (reference src/prolongator.h:94-108); block sites in
 * lexicographic order as block_sites lists them */
static void p_restrict(const Prol* P, const cxd* fine, cxd* coarse) {
    const int L = P->L, bs = P->bs;
#pragma omp parallel for schedule(static)
    for (int b = 0; b < P->nblocks; ++b) {
        int bx = b % P->nbx, by = b / P->nbx;
        for (int k = 0; k < P->k; ++k) coarse[b * P->k + k] = 0;
        for (int ly = 0; ly < bs; ++ly)
            for (int lx = 0; lx < bs; ++lx) {
                int s = (bx * bs + lx) + L * (by * bs + ly);
                int loc = lx + bs * ly;
                for (int k = 0; k < P->k; ++k) {
                    const cxd* v = P->bv + ((long)b * P->k + k) * P->bdim;
                    coarse[b * P->k + k] += conj(v[2 * loc]) * fine[2 * s] + conj(v[2 * loc + 1]) * fine[2 * s + 1];
                }
            }
    }
}

void orc_prolong(int L, int bs, int k, const double* block_vecs, const double* coarse, double* fine) {
    Prol P = p_make(L, bs, k, block_vecs);
    long nc = (long)P.nblocks * k, nf = 2L * L * L;
    cxd* c = to_cx(coarse, nc);
    cxd* f = (cxd*)malloc(sizeof(cxd) * (size_t)nf);
    p_prolong(&P, c, f);
    from_cx(f, nf, fine);
    free(c);
    free(f);
    free(P.bv);
}

void orc_restrict(int L, int bs, int k, const double* block_vecs, const double* fine, double* coarse) {
    Prol P = p_make(L, bs, k, block_vecs);
    long nc = (long)P.nblocks * k, nf = 2L * L * L;
    cxd* f = to_cx(fine, nf);
    cxd* c = (cxd*)malloc(sizeof(cxd) * (size_t)nc);
    p_restrict(&P, f, c);
    from_cx(c, nc, coarse);
    free(c);
    free(f);
    free(P.bv);
}

/* ----------------------------------------------------------- sparse coarse op */
/* SparseCoarseOp::neighbour / reverse_dir (reference src/coarse_op.h:205-229) */
static const int kDx[9] = {0, 1, -1, 0, 0, 1, 1, -1, -1};
static const int kDy[9] = {0, 0, 0, 1, -1, 1, -1, 1, -1};
static const int kRev[9] = {0, 2, 1, 4, 3, 8, 7, 6, 5};
static inline int c_neighbour(int nbx, int nby, int b, int dir) {
    int bxi = b % nbx, byi = b / nbx;
    int nx = (bxi + kDx[dir] + nbx) % nbx;
    int ny = (byi + kDy[dir] + nby) % nby;
    return nx + ny * nbx;
}

/* SparseCoarseOp::build by probing with A = D^dag D (reference src/coarse_op.h:241-279) */
void orc_sparse_coarse_build(int L, const double* U, double m, double r, double csw, double mu, int bs, int k,
                             const double* block_vecs, double* links) {
    Dirac D = d_make(L, U, m, r, csw, mu);
    Prol P = p_make(L, bs, k, block_vecs);
    const int nb = P.nblocks, dim = nb * k;
    long nf = 2L * L * L;
    cxd* lk = (cxd*)calloc((size_t)nb * 9 * k * k, sizeof(cxd));
    cxd* ej = (cxd*)calloc((size_t)dim, sizeof(cxd));
    cxd* fine = (cxd*)malloc(sizeof(cxd) * (size_t)nf);
    cxd* Afine = (cxd*)malloc(sizeof(cxd) * (size_t)nf);
    cxd* col = (cxd*)malloc(sizeof(cxd) * (size_t)dim);
    for (int J = 0; J < nb; ++J)
        for (int kj = 0; kj < k; ++kj) {
            int j = J * k + kj;
            ej[j] = 1.0;
            p_prolong(&P, ej, fine);
            d_apply_DdagD(&D, fine, Afine);
            p_restrict(&P, Afine, col);
            ej[j] = 0.0;
            for (int d = 0; d < 9; ++d) {
                int Ib = c_neighbour(P.nbx, P.nbx, J, d);
                int rd = kRev[d];
                for (int ki = 0; ki < k; ++ki) lk[(((long)Ib * 9 + rd) * k + ki) * k + kj] = col[Ib * k + ki];
            }
        }
    from_cx(lk, (long)nb * 9 * k * k, links);
    free(lk);
    free(ej);
    free(fine);
    free(Afine);
    free(col);
    free(P.bv);
    d_free(&D);
}

typedef struct {
    int nbx, nby, k, dim;
    const cxd* lk;
} Coarse;

/* SparseCoarseOp::apply_to (reference src/coarse_op.h:282-297) */
static void c_apply(const Coarse* A, const cxd* src, cxd* dst) {
    const int k = A->k, nb = A->nbx * A->nby;
#pragma omp parallel for schedule(static) if (nb > 256)
    for (int b = 0; b < nb; ++b) {
        for (int ki = 0; ki < k; ++ki) dst[b * k + ki] = 0;
        for (int d = 0; d < 9; ++d) {
            int n = c_neighbour(A->nbx, A->nby, b, d);
            const cxd* Lm = A->lk + ((long)b * 9 + d) * k * k;
            for (int ki = 0; ki < k; ++ki) {
                cxd sum = 0.0;
                for (int kj = 0; kj < k; ++kj) sum += Lm[ki * k + kj] * src[n * k + kj];
                dst[b * k + ki] += sum;
            }
        }
    }
}

void orc_sparse_coarse_apply(int nbx, int nby, int k, const double* links, const double* src, double* dst) {
    Coarse A;
    A.nbx = nbx;
    A.nby = nby;
    A.k = k;
    A.dim = nbx * nby * k;
    cxd* lk = to_cx(links, (long)nbx * nby * 9 * k * k);
    A.lk = lk;
    cxd* s = to_cx(src, A.dim);
    cxd* d = (cxd*)malloc(sizeof(cxd) * (size_t)A.dim);
    c_apply(&A, s, d);
    from_cx(d, A.dim, dst);
    free(lk);
    free(s);
    free(d);
}

/* SparseCoarseOp::solve without deflation vectors (reference src/coarse_op.h:492-547) */
static int c_cg(const Coarse* A, const cxd* b, cxd* x, int max_iter, double cg_tol) {
    const int dim = A->dim;
    double bnorm = v_norm(b, dim);
    memset(x, 0, sizeof(cxd) * (size_t)dim);
    if (bnorm < 1e-30) return 0;
    cxd* Ax = (cxd*)malloc(sizeof(cxd) * (size_t)dim);
    cxd* r = (cxd*)malloc(sizeof(cxd) * (size_t)dim);
    cxd* p = (cxd*)malloc(sizeof(cxd) * (size_t)dim);
    cxd* Ap = (cxd*)malloc(sizeof(cxd) * (size_t)dim);
    c_apply(A, x, Ax);
    for (int i = 0; i < dim; ++i) r[i] = b[i] - Ax[i];
    memcpy(p, r, sizeof(cxd) * (size_t)dim);
    cxd rr_val = v_dot(r, r, dim);
    int iter = 0;
    while (iter < max_iter) {
        c_apply(A, p, Ap);
        cxd pAp = v_dot(p, Ap, dim);
        if (cabs(pAp) < 1e-30) break;
        cxd alpha = rr_val / pAp;
#pragma omp parallel for schedule(static) if (dim > 4096)
        for (int i = 0; i < dim; ++i) {
            x[i] += alpha * p[i];
            r[i] -= alpha * Ap[i];
        }
        iter++;
        double rnorm = v_norm(r, dim);
        if (rnorm / bnorm < cg_tol) break;
        if (isnan(rnorm) || isinf(rnorm)) break;
        cxd rr_new = v_dot(r, r, dim);
        cxd beta = rr_new / rr_val;
        rr_val = rr_new;
#pragma omp parallel for schedule(static) if (dim > 4096)
        for (int i = 0; i < dim; ++i) p[i] = r[i] + beta * p[i];
    }
    free(Ax);
    free(r);
    free(p);
    free(Ap);
    return iter;
}

int orc_sparse_coarse_cg(int nbx, int nby, int k, const double* links, const double* b, double* x, int max_iter,
                         double tol) {
    Coarse A;
    A.nbx = nbx;
    A.nby = nby;
    A.k = k;
    A.dim = nbx * nby * k;
    cxd* lk = to_cx(links, (long)nbx * nby * 9 * k * k);
    A.lk = lk;
    cxd* bb = to_cx(b, A.dim);
    cxd* xx = (cxd*)malloc(sizeof(cxd) * (size_t)A.dim);
    int it = c_cg(&A, bb, xx, max_iter, tol);
    from_cx(xx, A.dim, x);
    free(lk);
    free(bb);
    free(xx);
    return it;
}

/* ----------------------------------------------------------- two-level MG */
typedef struct {
    const orc_mg2_params* p;
    Dirac D;
    Prol P;
    Coarse A;
    cxd* lk;
} MG2;

static MG2 mg2_make(const orc_mg2_params* p, const double* U, const double* block_vecs, const double* links) {
    MG2 m;
    m.p = p;
    m.D = d_make(p->L, U, p->m, p->r, p->csw, p->mu);
    m.P = p_make(p->L, p->bs, p->k, block_vecs);
    m.A.nbx = p->L / p->bs;
    m.A.nby = p->L / p->bs;
    m.A.k = p->k;
    m.A.dim = m.A.nbx * m.A.nby * p->k;
    m.lk = to_cx(links, (long)m.A.dim / p->k * 9 * p->k * p->k);
    m.A.lk = m.lk;
    return m;
}
static void mg2_free(MG2* m) {
    d_free(&m->D);
    free(m->P.bv);
    free(m->lk);
}

/* mg_cycle for two levels (reference src/multigrid.cpp:43-102): zero initial
 * guess, MR pre-smoothing (mr_smooth_op, smoother.cpp:26-40), residual,
 * restrict, coarsest solve, prolong, correct, MR post-smoothing */
static void mg2_cycle(const MG2* m, const cxd* b, cxd* x) {
    long n = 2L * m->D.g.V;
    int dimc = m->A.dim;
    memset(x, 0, sizeof(cxd) * (size_t)n);
    mr_smooth(&m->D, x, b, m->p->pre_smooth);
    cxd* Ax = (cxd*)malloc(sizeof(cxd) * (size_t)n);
    cxd* rc = (cxd*)malloc(sizeof(cxd) * (size_t)dimc);
    cxd* ec = (cxd*)malloc(sizeof(cxd) * (size_t)dimc);
    d_apply_DdagD(&m->D, x, Ax);
#pragma omp parallel for schedule(static) if (n > 4096)
    for (long i = 0; i < n; ++i) Ax[i] = b[i] - Ax[i];
    p_restrict(&m->P, Ax, rc);
    c_cg(&m->A, rc, ec, m->p->coarse_max_iter, m->p->coarse_tol);
    p_prolong(&m->P, ec, Ax);
#pragma omp parallel for schedule(static) if (n > 4096)
    for (long i = 0; i < n; ++i) x[i] += Ax[i];
    mr_smooth(&m->D, x, b, m->p->post_smooth);
    free(Ax);
    free(rc);
    free(ec);
}

void orc_mg2_precondition(const orc_mg2_params* p, const double* U, const double* block_vecs, const double* links,
                          const double* b, double* out) {
    MG2 m = mg2_make(p, U, block_vecs, links);
    long n = 2L * m.D.g.V;
    cxd* bb = to_cx(b, n);
    cxd* xx = (cxd*)malloc(sizeof(cxd) * (size_t)n);
    mg2_cycle(&m, bb, xx);
    from_cx(xx, n, out);
    free(bb);
    free(xx);
    mg2_free(&m);
}

/* fcg_solve = truncated GCR (reference src/solvers.cpp:223-300).  With
 * ref_coeff != 0 the orthogonalisation coefficient is the reference's
 * beta = dot(Az, AP_i) / ApAp_i (solvers.cpp:261), the complex conjugate of
 * the projection coefficient; with ref_coeff == 0 it is
 * beta = dot(AP_i, Az) / ApAp_i, which makes A p orthogonal to every stored
 * A p_i. */
int orc_mg2_gcr(const orc_mg2_params* p, const double* U, const double* block_vecs, const double* links,
                const double* bh, double* xh, int max_iter, double tol, int trunc, int ref_coeff,
                double* final_res) {
    MG2 m = mg2_make(p, U, block_vecs, links);
    long n = 2L * m.D.g.V;
    cxd* rhs = to_cx(bh, n);
    double rhs_norm = v_norm(rhs, n);
    cxd* x = (cxd*)calloc((size_t)n, sizeof(cxd));
    cxd* r = (cxd*)malloc(sizeof(cxd) * (size_t)n);
    memcpy(r, rhs, sizeof(cxd) * (size_t)n);
    cxd** Pd = (cxd**)calloc((size_t)trunc + 1, sizeof(cxd*));
    cxd** APd = (cxd**)calloc((size_t)trunc + 1, sizeof(cxd*));
    double* ApAp = (double*)calloc((size_t)trunc + 1, sizeof(double));
    int nd = 0, iter = 0;
    cxd* z = (cxd*)malloc(sizeof(cxd) * (size_t)n);
    cxd* Az = (cxd*)malloc(sizeof(cxd) * (size_t)n);
    if (rhs_norm >= 1e-30) {
        while (iter < max_iter) {
            double rnorm = v_norm(r, n);
            if (rnorm / rhs_norm < tol) break;
            mg2_cycle(&m, r, z);
            d_apply_DdagD(&m.D, z, Az);
            cxd* pp = (cxd*)malloc(sizeof(cxd) * (size_t)n);
            cxd* Ap = (cxd*)malloc(sizeof(cxd) * (size_t)n);
            memcpy(pp, z, sizeof(cxd) * (size_t)n);
            memcpy(Ap, Az, sizeof(cxd) * (size_t)n);
            for (int i = 0; i < nd; ++i) {
                cxd beta = (ref_coeff ? v_dot(Az, APd[i], n) : v_dot(APd[i], Az, n)) / ApAp[i];
#pragma omp parallel for schedule(static) if (n > 4096)
                for (long j = 0; j < n; ++j) {
                    pp[j] -= beta * Pd[i][j];
                    Ap[j] -= beta * APd[i][j];
                }
            }
            double ApAp_val = creal(v_dot(Ap, Ap, n));
            if (ApAp_val < 1e-30) {
                for (int i = 0; i < nd; ++i) {
                    free(Pd[i]);
                    free(APd[i]);
                }
                nd = 0;
                free(pp);
                free(Ap);
                continue;
            }
            cxd alpha = v_dot(Ap, r, n) / ApAp_val;
#pragma omp parallel for schedule(static) if (n > 4096)
            for (long j = 0; j < n; ++j) {
                x[j] += alpha * pp[j];
                r[j] -= alpha * Ap[j];
            }
            iter++;
            if (nd >= trunc) {
                free(Pd[0]);
                free(APd[0]);
                memmove(Pd, Pd + 1, sizeof(cxd*) * (size_t)(nd - 1));
                memmove(APd, APd + 1, sizeof(cxd*) * (size_t)(nd - 1));
                memmove(ApAp, ApAp + 1, sizeof(double) * (size_t)(nd - 1));
                nd--;
            }
            Pd[nd] = pp;
            APd[nd] = Ap;
            ApAp[nd] = ApAp_val;
            nd++;
        }
    }
    if (final_res) *final_res = rhs_norm >= 1e-30 ? v_norm(r, n) / rhs_norm : 0.0;
    from_cx(x, n, xh);
    for (int i = 0; i < nd; ++i) {
        free(Pd[i]);
        free(APd[i]);
    }
    free(Pd);
    free(APd);
    free(ApAp);
    free(z);
    free(Az);
    free(x);
    free(r);
    free(rhs);
    mg2_free(&m);
    return iter;
}

/* ------------------------------------------------------------ CPU timing */
/* Seconds for `reps` applications of D (op 0) or D^dag D (op 2) to each of
 * nrhs spinors, the Dirac operator built once outside the timed region. */
double orc_time_dirac(int L, const double* U, double m, double r, double csw, double mu, int op, int nrhs,
                      const double* src, double* dst, int reps) {
    Dirac D = d_make(L, U, m, r, csw, mu);
    long n = 2L * D.g.V;
    cxd* s = to_cx(src, n * nrhs);
    cxd* d = (cxd*)malloc(sizeof(cxd) * (size_t)(n * nrhs));
#ifdef _OPENMP
    double t0 = omp_get_wtime();
#endif
    for (int it = 0; it < reps; ++it)
        for (int j = 0; j < nrhs; ++j) {
            if (op == 2)
                d_apply_DdagD(&D, s + n * j, d + n * j);
            else
                d_apply(&D, s + n * j, d + n * j);
        }
#ifdef _OPENMP
    double t1 = omp_get_wtime();
#else
    double t0 = 0, t1 = 0;
#endif
    from_cx(d, n * nrhs, dst);
    free(s);
    free(d);
    d_free(&D);
    return t1 - t0;
}

/* Seconds for one CG solve on D^dag D (cg_core), Dirac built outside the timed region. */
double orc_time_cg(int L, const double* U, double m, double r, double csw, double mu, const double* b, double* x,
                   int max_iter, double tol, int* iters) {
    Dirac D = d_make(L, U, m, r, csw, mu);
    long n = 2L * D.g.V;
    cxd* bb = to_cx(b, n);
    cxd* xx = (cxd*)malloc(sizeof(cxd) * (size_t)n);
#ifdef _OPENMP
    double t0 = omp_get_wtime();
#endif
    int it = cg_core(&D, bb, xx, max_iter, tol, NULL);
#ifdef _OPENMP
    double t1 = omp_get_wtime();
#else
    double t0 = 0, t1 = 0;
#endif
    if (iters) *iters = it;
    from_cx(xx, n, x);
    free(bb);
    free(xx);
    d_free(&D);
    return t1 - t0;
}

/* ------------------------------------------------------------ N-level MG */
/* mg_cycle over a hierarchy of sparse stencil levels (reference
 * src/multigrid.cpp:43-102): MR pre-smoothing (mr_smooth_op,
 * src/smoother.cpp:26-40), residual, restriction, coarse cycle (twice with the
 * W-cycle when the next level is not the coarsest), prolongation, MR
 * post-smoothing; coarsest level by CG (src/coarse_op.h:492-547).  Level 0 is
 * D^dag D; level l >= 1 a 9-point stencil (SparseCoarseOp::apply_to).
 * Transfers l -> l+1 aggregate ax x ay sites with block vectors in the layout
 * [aggregate][i][loc * ndof_l + j] (Prolongator::block_vecs,
 * src/prolongator.h:23; CoarseProlongator for deeper levels). */

typedef struct {
    int nx, ny, ndof;     /* lattice and dofs of this level */
    int ax, ay, nc;       /* transfer to the next level */
    cxd* bv;              /* block vectors of the transfer, [agg][i][loc*ndof + j] */
    Coarse A;             /* operator of this level (l >= 1) */
    cxd* lk;
} NLevel;

typedef struct {
    const orc_mgN_params* p;
    Dirac D;
    int nl;
    NLevel lv[ORC_MAX_LEVELS];
} MGN;

static void n_restrict(const NLevel* L, const cxd* f, cxd* c) {
    const int nax = L->nx / L->ax, nay = L->ny / L->ay, m = L->ax * L->ay, nd = L->ndof;
#pragma omp parallel for schedule(static) if (nax * nay > 64)
    for (int B = 0; B < nax * nay; ++B) {
        const int x0 = (B % nax) * L->ax, y0 = (B / nax) * L->ay;
        for (int i = 0; i < L->nc; ++i) {
            const cxd* v = L->bv + ((long)B * L->nc + i) * m * nd;
            cxd acc = 0;
            for (int loc = 0; loc < m; ++loc) {
                int s = (x0 + loc % L->ax) + L->nx * (y0 + loc / L->ax);
                for (int j = 0; j < nd; ++j) acc += conj(v[loc * nd + j]) * f[(long)s * nd + j];
            }
            c[(long)B * L->nc + i] = acc;
        }
    }
}

static void n_prolong_add(const NLevel* L, const cxd* c, cxd* f) {
    const int nax = L->nx / L->ax, m = L->ax * L->ay, nd = L->ndof;
    const int ns = L->nx * L->ny;
#pragma omp parallel for schedule(static) if (ns > 256)
    for (int s = 0; s < ns; ++s) {
        const int x = s % L->nx, y = s / L->nx;
        const int B = x / L->ax + nax * (y / L->ay), loc = (x % L->ax) + L->ax * (y % L->ay);
        for (int j = 0; j < nd; ++j) {
            cxd acc = 0;
            for (int i = 0; i < L->nc; ++i) acc += c[(long)B * L->nc + i] * L->bv[((long)B * L->nc + i) * m * nd + loc * nd + j];
            f[(long)s * nd + j] += acc;
        }
    }
}

/* level-0 vectors are lexicographic v[2*s + spin], the same layout */
static void n_apply(const MGN* g, int l, const cxd* x, cxd* y) {
    if (l == 0)
        d_apply_DdagD(&g->D, x, y);
    else
        c_apply(&g->lv[l].A, x, y);
}

static long n_dim(const MGN* g, int l) { return (long)g->lv[l].nx * g->lv[l].ny * g->lv[l].ndof; }

/* mr_smooth_op with the residual recomputed every step, as the reference */
static void n_mr(const MGN* g, int l, cxd* x, const cxd* b, int niter) {
    long n = n_dim(g, l);
    cxd* r = (cxd*)malloc(sizeof(cxd) * (size_t)n);
    cxd* Ar = (cxd*)malloc(sizeof(cxd) * (size_t)n);
    for (int it = 0; it < niter; ++it) {
        n_apply(g, l, x, r);
#pragma omp parallel for schedule(static) if (n > 4096)
        for (long i = 0; i < n; ++i) r[i] = b[i] - r[i];
        n_apply(g, l, r, Ar);
        cxd rAr = v_dot(Ar, r, n), ArAr = v_dot(Ar, Ar, n);
        if (cabs(ArAr) < 1e-30) break;
        v_axpy(rAr / ArAr, r, x, n);
    }
    free(r);
    free(Ar);
}

static void n_cycle(const MGN* g, int l, const cxd* b, cxd* x) {
    const int last = g->nl - 1;
    long n = n_dim(g, l);
    if (l == last) {
        c_cg(&g->lv[l].A, b, x, g->p->coarse_max_iter, g->p->coarse_tol);
        return;
    }
    memset(x, 0, sizeof(cxd) * (size_t)n);
    n_mr(g, l, x, b, g->p->pre_smooth);
    cxd* r = (cxd*)malloc(sizeof(cxd) * (size_t)n);
    n_apply(g, l, x, r);
#pragma omp parallel for schedule(static) if (n > 4096)
    for (long i = 0; i < n; ++i) r[i] = b[i] - r[i];
    long nc = n_dim(g, l + 1);
    cxd* rc = (cxd*)malloc(sizeof(cxd) * (size_t)nc);
    cxd* ec = (cxd*)malloc(sizeof(cxd) * (size_t)nc);
    n_restrict(&g->lv[l], r, rc);
    n_cycle(g, l + 1, rc, ec);
    if (g->p->w_cycle && l + 1 < last) {
        cxd* Ae = (cxd*)malloc(sizeof(cxd) * (size_t)nc);
        cxd* e2 = (cxd*)malloc(sizeof(cxd) * (size_t)nc);
        n_apply(g, l + 1, ec, Ae);
        for (long i = 0; i < nc; ++i) Ae[i] = rc[i] - Ae[i];
        n_cycle(g, l + 1, Ae, e2);
        for (long i = 0; i < nc; ++i) ec[i] += e2[i];
        free(Ae);
        free(e2);
    }
    n_prolong_add(&g->lv[l], ec, x);
    n_mr(g, l, x, b, g->p->post_smooth);
    free(r);
    free(rc);
    free(ec);
}

static MGN n_make(const orc_mgN_params* p, const double* U) {
    MGN g;
    memset(&g, 0, sizeof(g));
    g.p = p;
    g.D = d_make(p->L, U, p->m, p->r, p->csw, p->mu);
    g.nl = p->n_levels;
    int nx = p->L, ny = p->L, nd = 2;
    for (int l = 0; l < g.nl; ++l) {
        NLevel* L = &g.lv[l];
        L->nx = nx;
        L->ny = ny;
        L->ndof = nd;
        if (l >= 1) {
            L->lk = to_cx(p->links[l], (long)nx * ny * 9 * nd * nd);
            L->A.nbx = nx;
            L->A.nby = ny;
            L->A.k = nd;
            L->A.dim = nx * ny * nd;
            L->A.lk = L->lk;
        }
        if (l < g.nl - 1) {
            L->ax = p->block[l][0];
            L->ay = p->block[l][1];
            L->nc = p->nc[l];
            L->bv = to_cx(p->block_vecs[l], (long)nx * ny * nd * L->nc);
            nx /= L->ax;
            ny /= L->ay;
            nd = L->nc;
        }
    }
    return g;
}

static void n_free(MGN* g) {
    d_free(&g->D);
    for (int l = 0; l < g->nl; ++l) {
        free(g->lv[l].bv);
        free(g->lv[l].lk);
    }
}

void orc_mgN_precondition(const orc_mgN_params* p, const double* U, const double* b, double* out) {
    MGN g = n_make(p, U);
    long n = n_dim(&g, 0);
    cxd* bb = to_cx(b, n);
    cxd* xx = (cxd*)malloc(sizeof(cxd) * (size_t)n);
    n_cycle(&g, 0, bb, xx);
    from_cx(xx, n, out);
    free(bb);
    free(xx);
    n_free(&g);
}

/* fcg_solve with the N-level preconditioner, projection coefficient; stops
 * after max_iter iterations or at tol; *seconds = wall time of the iterations */
int orc_mgN_gcr(const orc_mgN_params* p, const double* U, const double* bh, double* xh, int max_iter, double tol,
                int trunc, double* final_res, double* seconds) {
    MGN g = n_make(p, U);
    long n = n_dim(&g, 0);
    cxd* rhs = to_cx(bh, n);
    double rhs_norm = v_norm(rhs, n);
    cxd* x = (cxd*)calloc((size_t)n, sizeof(cxd));
    cxd* r = (cxd*)malloc(sizeof(cxd) * (size_t)n);
    memcpy(r, rhs, sizeof(cxd) * (size_t)n);
    cxd** Pd = (cxd**)calloc((size_t)trunc + 1, sizeof(cxd*));
    cxd** APd = (cxd**)calloc((size_t)trunc + 1, sizeof(cxd*));
    double* ApAp = (double*)calloc((size_t)trunc + 1, sizeof(double));
    cxd* z = (cxd*)malloc(sizeof(cxd) * (size_t)n);
    cxd* Az = (cxd*)malloc(sizeof(cxd) * (size_t)n);
    int nd = 0, iter = 0;
#ifdef _OPENMP
    double t0 = omp_get_wtime();
#endif
    while (rhs_norm >= 1e-30 && iter < max_iter) {
        if (v_norm(r, n) / rhs_norm < tol) break;
        n_cycle(&g, 0, r, z);
        d_apply_DdagD(&g.D, z, Az);
        cxd* pp = (cxd*)malloc(sizeof(cxd) * (size_t)n);
        cxd* Ap = (cxd*)malloc(sizeof(cxd) * (size_t)n);
        memcpy(pp, z, sizeof(cxd) * (size_t)n);
        memcpy(Ap, Az, sizeof(cxd) * (size_t)n);
        for (int i = 0; i < nd; ++i) {
            cxd beta = v_dot(APd[i], Az, n) / ApAp[i];
            const cxd* Pi = Pd[i];
            const cxd* APi = APd[i];
#pragma omp parallel for schedule(static) if (n > 4096)
            for (long j = 0; j < n; ++j) {
                pp[j] -= beta * Pi[j];
                Ap[j] -= beta * APi[j];
            }
        }
        double ApAp_val = creal(v_dot(Ap, Ap, n));
        if (ApAp_val < 1e-30) {
            for (int i = 0; i < nd; ++i) {
                free(Pd[i]);
                free(APd[i]);
            }
            nd = 0;
            free(pp);
            free(Ap);
            continue;
        }
        cxd alpha = v_dot(Ap, r, n) / ApAp_val;
#pragma omp parallel for schedule(static) if (n > 4096)
        for (long j = 0; j < n; ++j) {
            x[j] += alpha * pp[j];
            r[j] -= alpha * Ap[j];
        }
        iter++;
        if (nd >= trunc) {
            free(Pd[0]);
            free(APd[0]);
            memmove(Pd, Pd + 1, sizeof(cxd*) * (size_t)(nd - 1));
            memmove(APd, APd + 1, sizeof(cxd*) * (size_t)(nd - 1));
            memmove(ApAp, ApAp + 1, sizeof(double) * (size_t)(nd - 1));
            nd--;
        }
        Pd[nd] = pp;
        APd[nd] = Ap;
        ApAp[nd] = ApAp_val;
        nd++;
    }
#ifdef _OPENMP
    if (seconds) *seconds = omp_get_wtime() - t0;
#else
    if (seconds) *seconds = 0;
#endif
    if (final_res) *final_res = rhs_norm >= 1e-30 ? v_norm(r, n) / rhs_norm : 0.0;
    from_cx(x, n, xh);
    for (int i = 0; i < nd; ++i) {
        free(Pd[i]);
        free(APd[i]);
    }
    free(Pd);
    free(APd);
    free(ApAp);
    free(z);
    free(Az);
    free(x);
    free(r);
    free(rhs);
    n_free(&g);
    return iter;
}

/* ------------------------------------------------------ CPU hierarchy set-up */
/* The reference's hierarchy build (build_mg_hierarchy, src/multigrid.cpp:595-687)
 * restated on the CPU with a geometric ax x ay aggregate at every level (the
 * reference's CoarseProlongator linear blocking of 4k consecutive coarse dofs,
 * src/prolongator.h:149-228, is the 4 x 1 aggregate of coarse sites):
 *   - one std::mt19937(seed) draws every start vector, level by level, in
 *     random_vec order (compute_near_null_space / _generic draw from the rng
 *     they are given, src/multigrid.cpp:435-484, 545-587);
 *   - near-null vectors: per vector `iters` x (mr_smooth_op from x = 0 with
 *     the vector as right-hand side, Gram-Schmidt against the earlier ones,
 *     normalise), then a final Gram-Schmidt pass;
 *   - block vectors: the null vectors cut to aggregates and orthonormalised
 *     by modified Gram-Schmidt (orthonormalise_block, src/prolongator.h:111-130);
 *   - Galerkin operators formed directly instead of by probing
 *     (SparseCoarseOp::build, src/coarse_op.h:241-279):
 *       level 1:     A[b][d](i, j) = <D P e_{b,i}, D P e_{nb(b,d),j}>  (A = D^dag D)
 *       level l + 1: A[b][d](i, j) = <P e_{b,i}, A_l P e_{nb(b,d),j}>
 *     in the link layout [site][dir][i * nc + j] of SparseCoarseOp.
 * With chiral_split each null vector gives two block vectors, its upper and
 * lower chirality halves (spin 0 / 1 at level 0, the first / second half of
 * the coarse dofs deeper), ordered i = c * nvec + k. */

void* orc_rng_create(uint32_t seed);
void orc_rng_random_vec(void* h, long n, double* v);
void orc_rng_destroy(void* h);

typedef void (*op_fn)(const void* ctx, const cxd* x, cxd* y);

static void op_ddagd(const void* c, const cxd* x, cxd* y) { d_apply_DdagD((const Dirac*)c, x, y); }
static void op_coarse(const void* c, const cxd* x, cxd* y) { c_apply((const Coarse*)c, x, y); }

/* mr_smooth_op (reference src/smoother.cpp:26-40) */
static void mr_op(op_fn A, const void* ac, long n, cxd* x, const cxd* b, int niter, cxd* r, cxd* Ar) {
    for (int it = 0; it < niter; ++it) {
        A(ac, x, r);
#pragma omp parallel for schedule(static) if (n > 4096)
        for (long i = 0; i < n; ++i) r[i] = b[i] - r[i];
        A(ac, r, Ar);
        cxd rAr = v_dot(Ar, r, n), ArAr = v_dot(Ar, Ar, n);
        if (cabs(ArAr) < 1e-30) break;
        v_axpy(rAr / ArAr, r, x, n);
    }
}

/* compute_near_null_space_generic (reference src/multigrid.cpp:545-587) on
 * start vectors nv[0..k) that are overwritten with the result */
static void null_space_op(op_fn A, const void* ac, long n, int k, int iters, int mr_steps, cxd** nv) {
    cxd* x_new = (cxd*)malloc(sizeof(cxd) * (size_t)n);
    cxd* r = (cxd*)malloc(sizeof(cxd) * (size_t)n);
    cxd* Ar = (cxd*)malloc(sizeof(cxd) * (size_t)n);
    for (int i = 0; i < k; ++i) {
        v_scale(nv[i], 1.0 / v_norm(nv[i], n), n);
        for (int it = 0; it < iters; ++it) {
            memset(x_new, 0, sizeof(cxd) * (size_t)n);
            mr_op(A, ac, n, x_new, nv[i], mr_steps, r, Ar);
            for (int j = 0; j < i; ++j) v_axpy(-v_dot(nv[j], x_new, n), nv[j], x_new, n);
            double nrm = v_norm(x_new, n);
            if (!(nrm > 1e-14)) break;
            v_scale(x_new, 1.0 / nrm, n);
            memcpy(nv[i], x_new, sizeof(cxd) * (size_t)n);
        }
    }
    for (int i = 0; i < k; ++i) {
        for (int j = 0; j < i; ++j) v_axpy(-v_dot(nv[j], nv[i], n), nv[j], nv[i], n);
        double nrm = v_norm(nv[i], n);
        if (nrm > 1e-14) v_scale(nv[i], 1.0 / nrm, n);
    }
    free(x_new);
    free(r);
    free(Ar);
}

/* block vectors [agg][i][loc * nd + j] of ax x ay aggregates on an nx x ny
 * level with nd dofs per site (loc = (x % ax) + ax * (y % ay), agg =
 * (x / ax) + (nx / ax) * (y / ay)), orthonormalised per aggregate */
static cxd* block_vectors(int nx, int ny, int nd, int ax, int ay, int nvec, int split, cxd* const* nv) {
    const int nax = nx / ax, nagg = nax * (ny / ay), m = ax * ay, len = m * nd;
    const int nc = split ? 2 * nvec : nvec;
    cxd* bv = (cxd*)calloc((size_t)nagg * nc * len, sizeof(cxd));
#pragma omp parallel for schedule(static)
    for (int B = 0; B < nagg; ++B) {
        const int x0 = (B % nax) * ax, y0 = (B / nax) * ay;
        for (int k = 0; k < nvec; ++k)
            for (int loc = 0; loc < m; ++loc) {
                const long s = (x0 + loc % ax) + (long)nx * (y0 + loc / ax);
                for (int j = 0; j < nd; ++j) {
                    const cxd v = nv[k][s * nd + j];
                    if (split) {
                        const int chi = nd == 2 ? j : (j < nd / 2 ? 0 : 1);
                        bv[((long)B * nc + chi * nvec + k) * len + loc * nd + j] = v;
                    } else {
                        bv[((long)B * nc + k) * len + loc * nd + j] = v;
                    }
                }
            }
        for (int k = 0; k < nc; ++k) {
            cxd* v = bv + ((long)B * nc + k) * len;
            for (int j = 0; j < k; ++j) {
                const cxd* u = bv + ((long)B * nc + j) * len;
                cxd proj = 0;
                for (int e = 0; e < len; ++e) proj += conj(u[e]) * v[e];
                for (int e = 0; e < len; ++e) v[e] -= proj * u[e];
            }
            double nn = 0;
            for (int e = 0; e < len; ++e) nn += creal(v[e]) * creal(v[e]) + cimag(v[e]) * cimag(v[e]);
            nn = sqrt(nn);
            if (nn > 1e-14)
                for (int e = 0; e < len; ++e) v[e] /= nn;
        }
    }
    return bv;
}

/* one site of D applied to a field given by its values at the site and its
 * four neighbours (the arithmetic of apply_impl + accumulate_hops,
 * reference src/dirac.h:58-113) */
static void d_site(const Dirac* D, int s, const cxd* c, const cxd* xp, const cxd* xm, const cxd* yp,
                   const cxd* ym, cxd* out) {
    const int L = D->g.L;
    const double r = D->r;
    const double diag = 2.0 * D->r + D->mass;
    const double C = D->F ? 0.5 * D->csw * D->F[s] : 0.0;
    cxd d0 = ((diag + C) + I * D->mu) * c[0];
    cxd d1 = ((diag - C) - I * D->mu) * c[1];
    {
        cxd u = D->g.U0[s];
        cxd a0 = u * xp[0], a1 = u * xp[1];
        d0 -= 0.5 * (r * a0 - a1);
        d1 -= 0.5 * (-a0 + r * a1);
    }
    {
        cxd u = conj(D->g.U0[l_xm(L, s)]);
        cxd a0 = u * xm[0], a1 = u * xm[1];
        d0 -= 0.5 * (r * a0 + a1);
        d1 -= 0.5 * (a0 + r * a1);
    }
    {
        cxd u = D->g.U1[s];
        cxd a0 = u * yp[0], a1 = u * yp[1];
        d0 -= 0.5 * (r * a0 + I * a1);
        d1 -= 0.5 * (-I * a0 + r * a1);
    }
    {
        cxd u = conj(D->g.U1[l_ym(L, s)]);
        cxd a0 = u * ym[0], a1 = u * ym[1];
        d0 -= 0.5 * (r * a0 - I * a1);
        d1 -= 0.5 * (I * a0 + r * a1);
    }
    out[0] = d0;
    out[1] = d1;
}

static const int kDirOf[3][3] = {{8, 2, 7}, {4, 0, 3}, {6, 1, 5}}; /* [dx + 1][dy + 1] -> direction */

/* level-1 Galerkin operator from W_{B,i} = D P e_{B,i} on the (ax+2) x (ay+2)
 * frame around each aggregate; links [B][d][i * nc + j] */
static void galerkin0(const Dirac* D, int ax, int ay, int nc, const cxd* bv, cxd* lk) {
    const int L = D->g.L, nax = L / ax, nay = L / ay, nagg = nax * nay, m = ax * ay;
    const int fx = ax + 2, fy = ay + 2, nh = fx * fy;
    cxd* W = (cxd*)malloc(sizeof(cxd) * (size_t)nagg * nc * nh * 2);
    const cxd zero2[2] = {0, 0};
#pragma omp parallel for schedule(static)
    for (int B = 0; B < nagg; ++B) {
        const int x0 = (B % nax) * ax, y0 = (B / nax) * ay;
        for (int i = 0; i < nc; ++i) {
            const cxd* v = bv + ((long)B * nc + i) * m * 2;
            for (int h = 0; h < nh; ++h) {
                const int lx = h % fx - 1, ly = h / fx - 1;
                const int s = l_idx(L, x0 + lx, y0 + ly);
#define PV(X, Y) (((X) >= 0 && (X) < ax && (Y) >= 0 && (Y) < ay) ? v + 2 * ((X) + ax * (Y)) : zero2)
                d_site(D, s, PV(lx, ly), PV(lx + 1, ly), PV(lx - 1, ly), PV(lx, ly + 1), PV(lx, ly - 1),
                       W + (((long)B * nc + i) * nh + h) * 2);
#undef PV
            }
        }
    }
#pragma omp parallel for schedule(static)
    for (int B = 0; B < nagg; ++B) {
        const int Bx = B % nax, By = B / nax;
        for (int d = 0; d < 9; ++d) {
            const int dx = kDx[d], dy = kDy[d];
            const int B2 = (Bx + dx + nax) % nax + nax * ((By + dy + nay) % nay);
            const int hx0 = dx > 0 ? ax : 0, hx1 = dx < 0 ? 2 : fx;
            const int hy0 = dy > 0 ? ay : 0, hy1 = dy < 0 ? 2 : fy;
            for (int i = 0; i < nc; ++i) {
                const cxd* w1 = W + ((long)B * nc + i) * nh * 2;
                for (int j = 0; j < nc; ++j) {
                    const cxd* w2 = W + ((long)B2 * nc + j) * nh * 2;
                    cxd acc = 0;
                    for (int hy = hy0; hy < hy1; ++hy)
                        for (int hx = hx0; hx < hx1; ++hx) {
                            const int h1 = hx + fx * hy, h2 = (hx - dx * ax) + fx * (hy - dy * ay);
                            acc += conj(w1[2 * h1]) * w2[2 * h2] + conj(w1[2 * h1 + 1]) * w2[2 * h2 + 1];
                        }
                    lk[(((long)B * 9 + d) * nc + i) * nc + j] = acc;
                }
            }
        }
    }
    free(W);
}

/* Galerkin operator of a coarse level: A'[B][d'](i, j) = sum over the sites s
 * of B and directions d of V_B(s)^dag L[s][d] V_B2(nb(s, d)) */
static void galerkin_c(int nx, int ny, int nd, const cxd* lk, int ax, int ay, int nc, const cxd* bv, cxd* out) {
    const int nax = nx / ax, nay = ny / ay, nagg = nax * nay, m = ax * ay, len = m * nd;
    memset(out, 0, sizeof(cxd) * (size_t)nagg * 9 * nc * nc);
#pragma omp parallel
    {
        cxd* T = (cxd*)malloc(sizeof(cxd) * (size_t)nd * nc); /* T[ki][j] = sum_kj L(ki, kj) V_B2[j](loc2, kj) */
#pragma omp for schedule(static)
        for (int B = 0; B < nagg; ++B) {
            const int Bx = B % nax, By = B / nax;
            for (int loc = 0; loc < m; ++loc) {
                const int x = Bx * ax + loc % ax, y = By * ay + loc / ax;
                const long s = x + (long)nx * y;
                for (int d = 0; d < 9; ++d) {
                    const int x2 = (x + kDx[d] + nx) % nx, y2 = (y + kDy[d] + ny) % ny;
                    const int B2x = x2 / ax, B2y = y2 / ay;
                    int ddx = B2x - Bx, ddy = B2y - By;
                    if (ddx > 1) ddx -= nax;
                    if (ddx < -1) ddx += nax;
                    if (ddy > 1) ddy -= nay;
                    if (ddy < -1) ddy += nay;
                    const int dp = kDirOf[ddx + 1][ddy + 1];
                    const int B2 = B2x + nax * B2y, loc2 = (x2 % ax) + ax * (y2 % ay);
                    const cxd* Lm = lk + (s * 9 + d) * nd * nd;
                    for (int ki = 0; ki < nd; ++ki)
                        for (int j = 0; j < nc; ++j) {
                            const cxd* v2 = bv + ((long)B2 * nc + j) * len + loc2 * nd;
                            cxd acc = 0;
                            for (int kj = 0; kj < nd; ++kj) acc += Lm[ki * nd + kj] * v2[kj];
                            T[ki * nc + j] = acc;
                        }
                    cxd* Ao = out + ((long)B * 9 + dp) * nc * nc;
                    for (int i = 0; i < nc; ++i) {
                        const cxd* v1 = bv + ((long)B * nc + i) * len + loc * nd;
                        for (int j = 0; j < nc; ++j) {
                            cxd acc = 0;
                            for (int ki = 0; ki < nd; ++ki) acc += conj(v1[ki]) * T[ki * nc + j];
                            Ao[i * nc + j] += acc;
                        }
                    }
                }
            }
        }
        free(T);
    }
}

int orc_mgN_setup(const orc_mgN_setup_params* p, const double* U, double* const* block_vecs, double* const* links,
                  double* null0) {
    if (p->n_levels < 2 || p->n_levels > ORC_MAX_LEVELS) return -1;
    Dirac D = d_make(p->L, U, p->m, p->r, p->csw, p->mu);
    void* rng = orc_rng_create(p->seed);
    int nx = p->L, ny = p->L, nd = 2;
    cxd* lk_prev = NULL; /* operator of the current level l >= 1 */
    int rc = 0;
    for (int l = 0; l < p->n_levels - 1 && rc == 0; ++l) {
        const int ax = p->block[l][0], ay = p->block[l][1], k = p->nvec[l];
        const int nc = p->chiral_split ? 2 * k : k;
        const long n = (long)nx * ny * nd;
        if (ax < 1 || ay < 1 || nx % ax || ny % ay || nx / ax < 3 || ny / ay < 3) {
            rc = -2;
            break;
        }
        cxd** nv = (cxd**)malloc(sizeof(cxd*) * (size_t)k);
        double* h = (double*)malloc(sizeof(double) * 2 * (size_t)n);
        for (int i = 0; i < k; ++i) {
            orc_rng_random_vec(rng, n, h);
            nv[i] = to_cx(h, n);
        }
        free(h);
        Coarse A;
        if (l == 0) {
            null_space_op(op_ddagd, &D, n, k, p->null_iters, p->null_mr_steps, nv);
            if (null0)
                for (int i = 0; i < k; ++i) from_cx(nv[i], n, null0 + 2 * n * i);
        } else {
            A.nbx = nx;
            A.nby = ny;
            A.k = nd;
            A.dim = (int)n;
            A.lk = lk_prev;
            null_space_op(op_coarse, &A, n, k, p->null_iters, p->null_mr_steps, nv);
        }
        cxd* bv = block_vectors(nx, ny, nd, ax, ay, k, p->chiral_split, nv);
        for (int i = 0; i < k; ++i) free(nv[i]);
        free(nv);
        const int cx_ = nx / ax, cy_ = ny / ay;
        cxd* lk = (cxd*)malloc(sizeof(cxd) * (size_t)cx_ * cy_ * 9 * nc * nc);
        if (l == 0)
            galerkin0(&D, ax, ay, nc, bv, lk);
        else
            galerkin_c(nx, ny, nd, lk_prev, ax, ay, nc, bv, lk);
        from_cx(bv, n * nc, block_vecs[l]);
        from_cx(lk, (long)cx_ * cy_ * 9 * nc * nc, links[l + 1]);
        free(bv);
        free(lk_prev);
        lk_prev = lk;
        nx = cx_;
        ny = cy_;
        nd = nc;
    }
    free(lk_prev);
    orc_rng_destroy(rng);
    d_free(&D);
    return rc;
}
