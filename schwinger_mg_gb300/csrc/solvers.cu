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

struct CgState {      // device arrays of length nrhs each
    double* rr;
    double* pAp;
    double* bnorm2;
    double* beta;
    int* active;
    int* iters;
    int* flags;       // bit 0: breakdown, bit 1: non-finite
    int* n_active;    // scalar
    double tol2;
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
                int64_t i = ((int64_t)q * 2 + sp) * nrhs + rhs;
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
        int64_t i = ((int64_t)q * 2 + sp) * nrhs + rhs;
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
