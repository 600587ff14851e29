// Krylov solvers on A = D^dag D with every scalar kept on the device.
//
// CG (reference src/solvers.cpp:16-78).  One iteration is four kernels:
//   t  = D p            with ||t||^2 = <p, A p> fused into the epilogue
//   Ap = D^dag t
//   x += alpha p, r -= alpha Ap, ||r||^2      alpha = rr / pAp per rhs
//   p  = r + beta p                           beta = rr_new / rr
// The reduction finaliser of the update kernel applies the reference's stop
// rule (||r||/||b|| < tol after the update, solvers.cpp:55-59) per
// right-hand side; a stopped rhs gets alpha = beta = 0 from then on, so the
// remaining ones keep iterating in the same launches.  The host reads the
// number of active right-hand sides every `kCheckEvery` iterations only.
#include "smg_internal.h"
#include "reduce.cuh"

#include <algorithm>
#include <cmath>

smg_status smg_dslash(smg_dirac* d, bool dag, const smg_field* src, smg_field* dst, double* norm2_dev);
smg_status smg_norm2_dev(const smg_field* a, double* out_dev);

namespace {

constexpr int kCheckEvery = 8;

struct CgState {  // device arrays of length nrhs each
    double* rr = nullptr;
    double* pAp = nullptr;
    double* bnorm2 = nullptr;
    double* beta = nullptr;
    int* active = nullptr;
    int* iters = nullptr;
    int* flags = nullptr;     // bit 0: breakdown, bit 1: non-finite
    int* n_active = nullptr;  // scalar
    double tol2 = 0;
};

// single block; loops so any nrhs is covered
__global__ void k_cg_init(CgState s, int nrhs) {
    if (threadIdx.x == 0) *s.n_active = 0;
    __syncthreads();
    for (int j = threadIdx.x; j < nrhs; j += blockDim.x) {
        s.bnorm2[j] = s.rr[j];
        s.iters[j] = 0;
        s.flags[j] = 0;
        s.beta[j] = 0.0;
        int act = s.rr[j] >= 1e-60 ? 1 : 0;  // ||b|| < 1e-30 returns x = 0 (solvers.cpp:23)
        if (!isfinite(s.rr[j])) {
            act = 0;
            s.flags[j] |= 2;
        }
        s.active[j] = act;
        if (act) atomicAdd(s.n_active, 1);
    }
}

struct FinCgUpdate {
    CgState s;
    __device__ void operator()(int j, const double* sums) const {
        double rr_new = sums[0];
        if (!s.active[j]) { s.beta[j] = 0.0; return; }
        s.iters[j] += 1;
        if (!isfinite(rr_new)) {
            s.flags[j] |= 2;
            s.active[j] = 0;
            atomicSub(s.n_active, 1);
            s.beta[j] = 0.0;
            return;
        }
        if (rr_new < s.tol2 * s.bnorm2[j]) {
            s.active[j] = 0;
            atomicSub(s.n_active, 1);
            s.beta[j] = 0.0;
            s.rr[j] = rr_new;
            return;
        }
        s.beta[j] = rr_new / s.rr[j];
        s.rr[j] = rr_new;
    }
};

template <typename T>
__global__ void __launch_bounds__(256) k_cg_update(CgState s, cx<T>* __restrict__ x, cx<T>* __restrict__ r,
                                                   const cx<T>* __restrict__ p, const cx<T>* __restrict__ Ap,
                                                   int nsites, int nrhs, double* partials, unsigned int* ticket) {
    __shared__ T s_alpha[32];
    const int rhs = blockIdx.y * blockDim.x + threadIdx.x;
    if (threadIdx.y == 0) {
        T al = T(0);
        if (rhs < nrhs && s.active[rhs]) {
            double pap = s.pAp[rhs];
            if (pap > 0.0 && isfinite(pap)) al = (T)(s.rr[rhs] / pap);
        }
        s_alpha[threadIdx.x] = al;
    }
    __syncthreads();
    const T al = s_alpha[threadIdx.x];
    double v[1] = {0.0};
    if (rhs < nrhs) {
        for (int q = blockIdx.x * blockDim.y + threadIdx.y; q < nsites; q += gridDim.x * blockDim.y) {
#pragma unroll
            for (int sp = 0; sp < 2; ++sp) {
                int64_t i = sidx(q, rhs, sp, nrhs);
                cx<T> pi = p[i];
                cx<T> ri = r[i] - al * Ap[i];
                x[i] = x[i] + al * pi;
                r[i] = ri;
                v[0] += (double)norm2(ri);
            }
        }
    }
    block_reduce_finalise<1>(v, partials, ticket, nrhs, FinCgUpdate{s});
}

// breakdown guard before the update: pAp must be positive and finite
__global__ void k_cg_check_pap(CgState s, int nrhs) {
    int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= nrhs || !s.active[j]) return;
    double pap = s.pAp[j];
    if (!(pap > 0.0) || !isfinite(pap)) {
        s.flags[j] |= isfinite(pap) ? 1 : 2;
        s.active[j] = 0;
        atomicSub(s.n_active, 1);
    }
}

template <typename T>
__global__ void k_cg_p(const CgState s, const cx<T>* __restrict__ r, cx<T>* __restrict__ p, int nsites, int nrhs) {
    const int rhs = blockIdx.y * blockDim.x + threadIdx.x;
    const int q = blockIdx.x * blockDim.y + threadIdx.y;
    if (rhs >= nrhs || q >= nsites) return;
    const T be = (T)s.beta[rhs];
#pragma unroll
    for (int sp = 0; sp < 2; ++sp) {
        int64_t i = sidx(q, rhs, sp, nrhs);
        p[i] = r[i] + be * p[i];
    }
}

template <typename T>
__global__ void k_residual(const cx<T>* __restrict__ b, const cx<T>* __restrict__ Ax, cx<T>* __restrict__ r,
                           int64_t n) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) r[i] = b[i] - Ax[i];
}

struct FieldSet {
    std::vector<smg_field*> f;
    ~FieldSet() {
        for (auto* p : f) smg_field_destroy(p);
    }
    smg_status add(const smg_field* proto, smg_field** out) {
        SMG_TRY(smg_field_alloc_like(proto, proto->prec, out));
        f.push_back(*out);
        return SMG_OK;
    }
};

template <typename T>
smg_status cg_run(smg_dirac* d, const smg_field* b, smg_field* x, int max_iter, double tol, smg_solve_result* res) {
    smg_context* ctx = b->ctx;
    const int nrhs = b->nrhs;
    const int V = b->g.V;
    FieldSet fs;
    smg_field *r, *p, *t, *Ap;
    SMG_TRY(fs.add(b, &r));
    SMG_TRY(fs.add(b, &p));
    SMG_TRY(fs.add(b, &t));
    SMG_TRY(fs.add(b, &Ap));

    // device scalar block
    size_t nbytes = (size_t)nrhs * (5 * sizeof(double) + 3 * sizeof(int)) + 64;
    char* blk = nullptr;
    SMG_CUDA(ctx, cudaMallocAsync((void**)&blk, nbytes, ctx->stream));
    CgState s;
    s.rr = (double*)blk;
    s.pAp = s.rr + nrhs;
    s.bnorm2 = s.pAp + nrhs;
    s.beta = s.bnorm2 + nrhs;
    double* scratch_true = s.beta + nrhs;
    s.active = (int*)(scratch_true + nrhs);
    s.iters = s.active + nrhs;
    s.flags = s.iters + nrhs;
    s.n_active = (int*)(blk + nbytes - 16);
    s.tol2 = tol * tol;

    SMG_CUDA(ctx, cudaMemsetAsync(x->data, 0, x->bytes, ctx->stream));
    SMG_CUDA(ctx, cudaMemcpyAsync(r->data, b->data, b->bytes, cudaMemcpyDeviceToDevice, ctx->stream));
    SMG_CUDA(ctx, cudaMemcpyAsync(p->data, b->data, b->bytes, cudaMemcpyDeviceToDevice, ctx->stream));
    SMG_TRY(smg_norm2_dev(r, s.rr));
    k_cg_init<<<1, 256, 0, ctx->stream>>>(s, nrhs);
    count_launch(ctx);
    SMG_CHECK_LAUNCH(ctx);

    ReduceLaunch rl = reduce_launch(V, nrhs);
    SMG_TRY(smg_reduce_reserve(ctx, (size_t)rl.grid.x * nrhs * 3));
    SiteLaunch sl = site_launch(V, nrhs);
    SMG_TRY(smg_host_stage_reserve(ctx, 64));
    int* h_active = (int*)ctx->host_stage;

    int it = 0;
    bool done = false;
    // first check before any iteration (all-zero right-hand sides)
    SMG_CUDA(ctx, cudaMemcpyAsync(h_active, s.n_active, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    SMG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    done = (*h_active == 0);
    while (!done && it < max_iter) {
        int chunk = std::min(kCheckEvery, max_iter - it);
        for (int c = 0; c < chunk; ++c) {
            SMG_TRY(smg_dslash(d, false, p, t, s.pAp));
            SMG_TRY(smg_dslash(d, true, t, Ap, nullptr));
            k_cg_check_pap<<<(nrhs + 127) / 128, 128, 0, ctx->stream>>>(s, nrhs);
            k_cg_update<T><<<rl.grid, rl.block, 0, ctx->stream>>>(s, (cx<T>*)x->data, (cx<T>*)r->data,
                                                                 (const cx<T>*)p->data, (const cx<T>*)Ap->data, V,
                                                                 nrhs, ctx->red.partials, ctx->red.tickets);
            k_cg_p<T><<<sl.grid, sl.block, 0, ctx->stream>>>(s, (const cx<T>*)r->data, (cx<T>*)p->data, V, nrhs);
            count_launch(ctx, 3);
            SMG_CHECK_LAUNCH(ctx);
        }
        it += chunk;
        SMG_CUDA(ctx, cudaMemcpyAsync(h_active, s.n_active, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
        SMG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        done = (*h_active == 0);
    }

    // true residual ||b - A x|| / ||b|| with the operator of the field precision
    SMG_TRY(smg_dslash(d, false, x, t, nullptr));
    SMG_TRY(smg_dslash(d, true, t, Ap, nullptr));
    int64_t n = b->n_complex();
    k_residual<T><<<(unsigned)((n + 255) / 256), 256, 0, ctx->stream>>>((const cx<T>*)b->data,
                                                                      (const cx<T>*)Ap->data, (cx<T>*)r->data, n);
    count_launch(ctx);
    SMG_TRY(smg_norm2_dev(r, scratch_true));

    std::vector<double> h((size_t)nrhs * 5);
    std::vector<int> hi((size_t)nrhs * 3);
    SMG_CUDA(ctx, cudaMemcpyAsync(h.data(), blk, (size_t)nrhs * 5 * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    SMG_CUDA(ctx, cudaMemcpyAsync(hi.data(), s.active, (size_t)nrhs * 3 * sizeof(int), cudaMemcpyDeviceToHost,
                                  ctx->stream));
    SMG_CUDA(ctx, cudaFreeAsync(blk, ctx->stream));
    SMG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));

    smg_status st = SMG_OK;
    int worst_it = 0;
    double worst_rec = 0, worst_true = 0;
    for (int j = 0; j < nrhs; ++j) {
        double rr = h[j], b2 = h[2 * nrhs + j], tr = h[4 * nrhs + j];
        int active = hi[j], iters = hi[nrhs + j], flags = hi[2 * nrhs + j];
        double rec = b2 > 0 ? std::sqrt(rr / b2) : 0.0;
        double tru = b2 > 0 ? std::sqrt(tr / b2) : 0.0;
        worst_it = std::max(worst_it, iters);
        worst_rec = std::max(worst_rec, rec);
        worst_true = std::max(worst_true, tru);
        if (flags & 2) st = SMG_NONFINITE;
        else if ((flags & 1) && st == SMG_OK) st = SMG_BREAKDOWN;
        else if (active && st == SMG_OK) st = SMG_NOT_CONVERGED;
    }
    if (res) {
        res->iterations = worst_it;
        res->final_residual = worst_rec;
        res->true_residual = worst_true;
        res->operator_applications = worst_it + 1;
    }
    if (st != SMG_OK) smg_fail(ctx, st, "cg_solve: stopped before reaching the tolerance");
    return st;
}

}  // namespace

extern "C" {

SMG_API smg_status smg_cg_solve(smg_dirac* d, const smg_field* rhs, smg_field* x, int max_iter, double tol,
                                smg_solve_result* res) {
    if (!d || !rhs || !x) return SMG_BAD_ARG;
    smg_context* ctx = d->ctx;
    if (rhs == x) return smg_fail(ctx, SMG_BAD_ARG, "rhs and x must be distinct");
    SMG_TRY(smg_field_check_pair(rhs, x));
    if (rhs->g.L != d->gauge->g.L) return smg_fail(ctx, SMG_BAD_ARG, "field L differs from gauge L");
    if (max_iter < 0 || !(tol > 0)) return smg_fail(ctx, SMG_BAD_ARG, "max_iter >= 0 and tol > 0 required");
    if (rhs->prec == SMG_F64) return cg_run<double>(d, rhs, x, max_iter, tol, res);
    if (rhs->prec == SMG_F32) return cg_run<float>(d, rhs, x, max_iter, tol, res);
    return smg_fail(ctx, SMG_UNSUPPORTED, "cg_solve on F16 fields");
}

}  // extern "C"

// =====================================================================
// GCR (the reference's fcg_solve, src/solvers.cpp:223-300) on A = D^dag D,
// flexible in the preconditioner (one MG cycle per iteration).  Directions
// live in a ring of trunc + 1 (p, A p) buffer pairs; the pair that falls out
// of the window becomes the next iteration's work pair, so nothing is copied.
// All scalars stay on the device; the host reads the per-rhs residuals once
// per iteration to apply the stop rule.
// =====================================================================
#include "vec.cuh"

smg_status smg_mg_apply_internal(smg_mg* mg, const smg_field* b, smg_field* x);
smg_precision smg_mg_precision(const smg_mg* mg);
smg_status smg_mg_check_device_error(smg_mg* mg);

namespace {

struct GcrScalars {
    double* rr = nullptr;      // [rhs]
    double* bnorm2 = nullptr;  // [rhs]
    double* apr3 = nullptr;    // [rhs][3] of the current direction: <Ap, r> re, im, ||Ap||^2
    int* active = nullptr;     // [rhs]
    int* flags = nullptr;      // [rhs]
    double tol2 = 0;
};

// beta = (ref ? <Az, AP_i> : <AP_i, Az>) / ApAp_i;  p -= beta P_i, Ap -= beta AP_i
template <typename T>
__global__ void __launch_bounds__(256) k_gcr_orth(VecView<T> p, cx<T>* __restrict__ Ap, const cx<T>* __restrict__ Pi,
                                                  const cx<T>* __restrict__ APi, const double* __restrict__ dot,
                                                  const double* __restrict__ apap_i, int ref_coeff) {
    __shared__ cx<T> s_b[32];
    const int rhs = blockIdx.y * blockDim.x + threadIdx.x;
    if (threadIdx.y == 0) {
        cx<T> be = mk<T>(0, 0);
        if (rhs < p.nrhs) {
            double den = apap_i[3 * rhs + 2];
            // dot holds <AP_i, Az>; the reference's coefficient is its conjugate
            double re = dot[2 * rhs], im = ref_coeff ? -dot[2 * rhs + 1] : dot[2 * rhs + 1];
            if (den > 0) be = mk<T>((T)(re / den), (T)(im / den));
        }
        s_b[threadIdx.x] = be;
    }
    __syncthreads();
    const int s = blockIdx.x * blockDim.y + threadIdx.y;
    if (rhs >= p.nrhs || s >= p.nsites) return;
    const cx<T> be = s_b[threadIdx.x];
    const int64_t base = p.idx(s, rhs, 0);
    for (int d = 0; d < p.ndof; ++d) {
        p.p[base + d] = p.p[base + d] - be * Pi[base + d];
        Ap[base + d] = Ap[base + d] - be * APi[base + d];
    }
}

struct FinGcr {
    GcrScalars s;
    __device__ void operator()(int j, const double* sums) const {
        if (s.active[j]) s.rr[j] = sums[0];
    }
};

// alpha = <Ap, r> / ||Ap||^2; x += alpha p; r -= alpha Ap; ||r||^2
template <typename T>
__global__ void __launch_bounds__(256) k_gcr_update(GcrScalars sc, VecView<T> x, cx<T>* __restrict__ r,
                                                    const cx<T>* __restrict__ p, const cx<T>* __restrict__ Ap,
                                                    double* partials, unsigned int* ticket) {
    __shared__ cx<T> s_al[32];
    const int nrhs = x.nrhs;
    const int rhs = blockIdx.y * blockDim.x + threadIdx.x;
    if (threadIdx.y == 0) {
        cx<T> al = mk<T>(0, 0);
        if (rhs < nrhs && sc.active[rhs]) {
            double den = sc.apr3[3 * rhs + 2];
            if (den >= 1e-30 && isfinite(den))
                al = mk<T>((T)(sc.apr3[3 * rhs] / den), (T)(sc.apr3[3 * rhs + 1] / den));
        }
        s_al[threadIdx.x] = al;
    }
    __syncthreads();
    const cx<T> al = s_al[threadIdx.x];
    double v[1] = {0.0};
    if (rhs < nrhs) {
        for (int st = blockIdx.x * blockDim.y + threadIdx.y; st < x.nsites; st += gridDim.x * blockDim.y) {
            const int64_t base = x.idx(st, rhs, 0);
            for (int d = 0; d < x.ndof; ++d) {
                const cx<T> ri = r[base + d] - al * Ap[base + d];
                x.p[base + d] = x.p[base + d] + al * p[base + d];
                r[base + d] = ri;
                v[0] += (double)norm2(ri);
            }
        }
    }
    block_reduce_finalise<1>(v, partials, ticket, nrhs, FinGcr{sc});
}

template <typename T>
VecView<T> fv(const smg_field* f) {
    VecView<T> v;
    v.p = (cx<T>*)f->data;
    v.nsites = f->g.V;
    v.nrhs = f->nrhs;
    v.ndof = 2;
    return v;
}

template <typename T>
smg_status apply_A(smg_dirac* d, const smg_field* in, smg_field* tmp, smg_field* out) {
    SMG_TRY(smg_dslash(d, false, in, tmp, nullptr));
    return smg_dslash(d, true, tmp, out, nullptr);
}

template <typename T>
smg_status reduce_into(smg_context* ctx, VecView<T> a, const cx<T>* b, int mode, double* out) {
    ReduceLaunch rl = reduce_launch(a.nsites, a.nrhs);
    SMG_TRY(smg_reduce_reserve(ctx, (size_t)rl.grid.x * a.nrhs * 3));
    if (mode == VR_DOT)
        k_vreduce<T, VR_DOT><<<rl.grid, rl.block, 0, ctx->stream>>>(a, b, ctx->red.partials, ctx->red.tickets, out);
    else if (mode == VR_NORM)
        k_vreduce<T, VR_NORM><<<rl.grid, rl.block, 0, ctx->stream>>>(a, b, ctx->red.partials, ctx->red.tickets, out);
    else
        k_vreduce<T, VR_DOTNORM><<<rl.grid, rl.block, 0, ctx->stream>>>(a, b, ctx->red.partials, ctx->red.tickets, out);
    count_launch(ctx);
    SMG_CHECK_LAUNCH(ctx);
    return SMG_OK;
}

template <typename T>
smg_status gcr_run(smg_dirac* d, smg_mg* mg, const smg_field* b, smg_field* x, int max_iter, double tol, int trunc,
                   int ref_coeff, smg_solve_result* res) {
    smg_context* ctx = d->ctx;
    const int nrhs = b->nrhs, V = b->g.V;
    const int nbuf = trunc + 1;
    FieldSet fs;
    smg_field *r, *z, *Az, *tmp;
    SMG_TRY(fs.add(b, &r));
    SMG_TRY(fs.add(b, &z));
    SMG_TRY(fs.add(b, &Az));
    SMG_TRY(fs.add(b, &tmp));
    std::vector<smg_field*> P(nbuf), AP(nbuf);
    for (int i = 0; i < nbuf; ++i) {
        SMG_TRY(fs.add(b, &P[i]));
        SMG_TRY(fs.add(b, &AP[i]));
    }
    const bool mixed = mg && smg_mg_precision(mg) != b->prec;
    smg_field *rlo = nullptr, *zlo = nullptr;
    if (mixed) {
        SMG_TRY(smg_field_alloc_like(b, smg_mg_precision(mg), &rlo));
        fs.f.push_back(rlo);
        SMG_TRY(smg_field_alloc_like(b, smg_mg_precision(mg), &zlo));
        fs.f.push_back(zlo);
    }
    // scalar block: rr, bnorm2, true, dots (2), per buffer apr3 (3 each), ints
    const size_t nd_ = (size_t)nrhs * (5 + 3 * nbuf) + 64;
    double* blk = nullptr;
    SMG_CUDA(ctx, cudaMallocAsync(&blk, nd_ * sizeof(double) + (size_t)nrhs * 2 * sizeof(int) + 64, ctx->stream));
    SMG_CUDA(ctx, cudaMemsetAsync(blk, 0, nd_ * sizeof(double) + (size_t)nrhs * 2 * sizeof(int) + 64, ctx->stream));
    GcrScalars sc;
    sc.rr = blk;
    sc.bnorm2 = blk + nrhs;
    double* truev = blk + 2 * nrhs;
    double* dots = blk + 3 * nrhs;  // 2 * nrhs
    double* apr = blk + 5 * nrhs;   // nbuf * 3 * nrhs
    sc.active = (int*)(blk + nd_);
    sc.flags = sc.active + nrhs;
    sc.tol2 = tol * tol;
    auto apr_of = [&](int buf) { return apr + (size_t)buf * 3 * nrhs; };

    SMG_CUDA(ctx, cudaMemsetAsync(x->data, 0, x->bytes, ctx->stream));
    SMG_CUDA(ctx, cudaMemcpyAsync(r->data, b->data, b->bytes, cudaMemcpyDeviceToDevice, ctx->stream));
    SMG_TRY(reduce_into<T>(ctx, fv<T>(r), nullptr, VR_NORM, sc.rr));
    SMG_CUDA(ctx, cudaMemcpyAsync(sc.bnorm2, sc.rr, nrhs * sizeof(double), cudaMemcpyDeviceToDevice, ctx->stream));

    std::vector<double> h_rr(nrhs), h_b2(nrhs);
    std::vector<int> h_act(nrhs, 1);
    SMG_CUDA(ctx, cudaMemcpyAsync(h_b2.data(), sc.bnorm2, nrhs * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    SMG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    for (int j = 0; j < nrhs; ++j) h_act[j] = (h_b2[j] >= 1e-60 && std::isfinite(h_b2[j])) ? 1 : 0;
    bool nonfinite = false;
    for (int j = 0; j < nrhs; ++j)
        if (!std::isfinite(h_b2[j])) nonfinite = true;

    std::vector<int> ring;  // buffer indices of stored directions, oldest first
    int work = 0;           // buffer index of the current (p, Ap) pair
    std::vector<int> freeb;
    for (int i = 1; i < nbuf; ++i) freeb.push_back(i);
    int iter = 0;
    const ReduceLaunch rl = reduce_launch(V, nrhs);
    SMG_TRY(smg_reduce_reserve(ctx, (size_t)rl.grid.x * nrhs * 3));
    bool any_active = false;
    for (int j = 0; j < nrhs; ++j) any_active |= h_act[j] != 0;
    while (any_active && iter < max_iter) {
        SMG_CUDA(ctx, cudaMemcpyAsync(sc.active, h_act.data(), nrhs * sizeof(int), cudaMemcpyHostToDevice, ctx->stream));
        // z = M^-1 r
        if (!mg) {
            SMG_CUDA(ctx, cudaMemcpyAsync(z->data, r->data, r->bytes, cudaMemcpyDeviceToDevice, ctx->stream));
        } else if (!mixed) {
            SMG_TRY(smg_mg_apply_internal(mg, r, z));
        } else {
            // FP32 cycle on r / ||r||, then z = ||r|| * M^-1 (r / ||r||) in FP64
            VecView<float> rl32 = fv<float>(rlo);
            k_vconvert_scaled<float, T><<<vec_grid(V, nrhs), vec_block(nrhs), 0, ctx->stream>>>(
                rl32, (const cx<T>*)r->data, sc.rr, 1);
            SMG_TRY(smg_mg_apply_internal(mg, rlo, zlo));
            k_vconvert_scaled<T, float><<<vec_grid(V, nrhs), vec_block(nrhs), 0, ctx->stream>>>(
                fv<T>(z), (const cx<float>*)zlo->data, sc.rr, 0);
            count_launch(ctx, 2);
            SMG_CHECK_LAUNCH(ctx);
        }
        // p = z, Ap = A z, orthogonalised against the stored directions
        smg_field* p = P[work];
        smg_field* Ap = AP[work];
        SMG_TRY(apply_A<T>(d, z, tmp, Az));
        SMG_CUDA(ctx, cudaMemcpyAsync(p->data, z->data, z->bytes, cudaMemcpyDeviceToDevice, ctx->stream));
        SMG_CUDA(ctx, cudaMemcpyAsync(Ap->data, Az->data, Az->bytes, cudaMemcpyDeviceToDevice, ctx->stream));
        for (int slot : ring) {
            // <AP_i, Az> (classical Gram-Schmidt on Az, as solvers.cpp:260-267)
            SMG_TRY(reduce_into<T>(ctx, fv<T>(AP[slot]), (const cx<T>*)Az->data, VR_DOT, dots));
            k_gcr_orth<T><<<vec_grid(V, nrhs), vec_block(nrhs), 0, ctx->stream>>>(
                fv<T>(p), (cx<T>*)Ap->data, (const cx<T>*)P[slot]->data, (const cx<T>*)AP[slot]->data, dots,
                apr_of(slot), ref_coeff);
            count_launch(ctx);
            SMG_CHECK_LAUNCH(ctx);
        }
        // <Ap, r> and ||Ap||^2 into this buffer's scalar slot
        SMG_TRY(reduce_into<T>(ctx, fv<T>(Ap), (const cx<T>*)r->data, VR_DOTNORM, apr_of(work)));
        sc.apr3 = apr_of(work);
        k_gcr_update<T><<<rl.grid, rl.block, 0, ctx->stream>>>(sc, fv<T>(x), (cx<T>*)r->data, (const cx<T>*)p->data,
                                                               (const cx<T>*)Ap->data, ctx->red.partials,
                                                               ctx->red.tickets);
        count_launch(ctx);
        SMG_CHECK_LAUNCH(ctx);
        // host: stop rule and breakdown (||Ap||^2 < 1e-30 clears the history, solvers.cpp:272-276)
        std::vector<double> h_apr(3 * nrhs);
        SMG_CUDA(ctx, cudaMemcpyAsync(h_rr.data(), sc.rr, nrhs * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
        SMG_CUDA(ctx, cudaMemcpyAsync(h_apr.data(), apr_of(work), 3 * nrhs * sizeof(double), cudaMemcpyDeviceToHost,
                                      ctx->stream));
        SMG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        bool breakdown = false;
        for (int j = 0; j < nrhs; ++j)
            if (h_act[j] && !(h_apr[3 * j + 2] >= 1e-30)) breakdown = true;
        if (breakdown) {
            for (int slot : ring) freeb.push_back(slot);
            ring.clear();
            bool any_nan = false;
            for (int j = 0; j < nrhs; ++j)
                if (h_act[j] && !std::isfinite(h_apr[3 * j + 2])) any_nan = true;
            if (any_nan) {
                nonfinite = true;
                break;
            }
            continue;  // the reference retries without counting an iteration
        }
        ++iter;
        // store (p, Ap): the work pair joins the window, the oldest leaves it
        ring.push_back(work);
        if ((int)ring.size() > trunc) {
            freeb.push_back(ring.front());
            ring.erase(ring.begin());
        }
        work = freeb.back();
        freeb.pop_back();
        any_active = false;
        for (int j = 0; j < nrhs; ++j) {
            if (h_act[j]) {
                if (!std::isfinite(h_rr[j])) {
                    nonfinite = true;
                    h_act[j] = 0;
                } else if (h_rr[j] < tol * tol * h_b2[j]) {
                    h_act[j] = 0;
                }
            }
            any_active |= h_act[j] != 0;
        }
    }
    // true residual in the field precision
    SMG_TRY(apply_A<T>(d, x, tmp, Az));
    int64_t n = b->n_complex();
    k_residual<T><<<(unsigned)((n + 255) / 256), 256, 0, ctx->stream>>>((const cx<T>*)b->data, (const cx<T>*)Az->data,
                                                                      (cx<T>*)r->data, n);
    count_launch(ctx);
    SMG_TRY(reduce_into<T>(ctx, fv<T>(r), nullptr, VR_NORM, truev));
    std::vector<double> h_true(nrhs);
    SMG_CUDA(ctx, cudaMemcpyAsync(h_true.data(), truev, nrhs * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    SMG_CUDA(ctx, cudaMemcpyAsync(h_rr.data(), sc.rr, nrhs * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    SMG_CUDA(ctx, cudaFreeAsync(blk, ctx->stream));
    SMG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    double worst_rec = 0, worst_true = 0;
    bool notconv = false;
    for (int j = 0; j < nrhs; ++j) {
        if (h_b2[j] > 0 && std::isfinite(h_b2[j])) {
            worst_rec = std::max(worst_rec, std::sqrt(h_rr[j] / h_b2[j]));
            worst_true = std::max(worst_true, std::sqrt(h_true[j] / h_b2[j]));
        }
        if (h_act[j]) notconv = true;
    }
    if (res) {
        res->iterations = iter;
        res->final_residual = worst_rec;
        res->true_residual = worst_true;
        res->operator_applications = iter + 1;
    }
    if (mg) SMG_TRY(smg_mg_check_device_error(mg));
    if (nonfinite) return smg_fail(ctx, SMG_NONFINITE, "gcr_solve: non-finite residual");
    if (notconv) return smg_fail(ctx, SMG_NOT_CONVERGED, "gcr_solve: iteration limit reached");
    return SMG_OK;
}

}  // namespace

extern "C" {

SMG_API smg_status smg_gcr_solve(smg_dirac* d, smg_mg* mg, const smg_field* rhs, smg_field* x, int max_iter, double tol,
                                 int trunc, int reference_coefficient, smg_solve_result* res) {
    if (!d || !rhs || !x) return SMG_BAD_ARG;
    smg_context* ctx = d->ctx;
    if (rhs == x) return smg_fail(ctx, SMG_BAD_ARG, "rhs and x must be distinct");
    SMG_TRY(smg_field_check_pair(rhs, x));
    if (rhs->g.L != d->gauge->g.L) return smg_fail(ctx, SMG_BAD_ARG, "field L differs from gauge L");
    if (max_iter < 0 || !(tol > 0) || trunc < 1 || trunc > 256)
        return smg_fail(ctx, SMG_BAD_ARG, "max_iter >= 0, tol > 0 and trunc in [1, 256] required");
    if (rhs->prec == SMG_F64) return gcr_run<double>(d, mg, rhs, x, max_iter, tol, trunc, reference_coefficient, res);
    if (rhs->prec == SMG_F32) {
        if (mg && smg_mg_precision(mg) == SMG_F64)
            return smg_fail(ctx, SMG_UNSUPPORTED, "an F64 hierarchy needs F64 fields");
        return gcr_run<float>(d, mg, rhs, x, max_iter, tol, trunc, reference_coefficient, res);
    }
    return smg_fail(ctx, SMG_UNSUPPORTED, "gcr_solve on F16 fields");
}

}  // extern "C"
