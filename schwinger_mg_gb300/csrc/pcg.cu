// Preconditioned CG, the stand-alone fine smoothers and the pseudofermion
// action on A = D^dag D.
//
// PCG (the reference's cg_solve_core with a preconditioner and/or a start
// vector, src/solvers.cpp:16-72; cg_solve_precond, cg_solve_x0,
// cg_solve_x0_precond, :80-96).  One iteration:
//   t = D p with ||t||^2 = <p, A p> fused, Ap = D^dag t
//   alpha = rz / pAp; x += alpha p; r -= alpha Ap; ||r||^2 and the stop rule
//   z = M^-1 r (one MG cycle, or z = r)
//   rz' = <r, z>; beta = rz' / rz; p = z + beta p
// alpha and beta are complex as in the reference (the MG cycle is Hermitian
// only to rounding).  rz lives in two device slots used alternately, so
// the kernel that forms beta reads the old and the new value without a
// copy.  Every right-hand side stops on its own.
//
// Smoothers on the fine operator (src/smoother.cpp): mr_smooth (:9-23),
// richardson_smooth_op (:64-73) and estimate_lambda_max (:43-60).  The
// smoothers carry the residual recursively (r -= omega A r), one operator
// application per step where the reference recomputes r = b - A x.
//
// Pseudofermion action (fermion_action / fermion_action_precond,
// src/hmc_forces.cpp:113-131): X = (D^dag D)^-1 phi by PCG and
// S = Re <phi, X>; smg_fermion_force is the matching backward pass.
#include "krylov.cuh"

#include <algorithm>
#include <cmath>

smg_status smg_mg_apply_internal(smg_mg* mg, const smg_field* b, smg_field* x);
smg_status smg_mg_check_device_error(smg_mg* mg);
smg_status smg_mg_level0_L(const smg_mg* mg, int* L);

namespace {

struct PcgState {                 // device arrays, per rhs
    double* rz[2] = {nullptr, nullptr};  // [rhs][2] complex <r, z>, used alternately
    double* pAp = nullptr;
    double* rr = nullptr;
    double* bnorm2 = nullptr;
    int* active = nullptr;
    int* iters = nullptr;
    int* flags = nullptr;   // bit 0: breakdown, bit 1: non-finite
    int* n_active = nullptr;
    double tol2 = 0;
};

__global__ void k_pcg_init(PcgState s, int nrhs) {
    if (threadIdx.x == 0) *s.n_active = 0;
    __syncthreads();
    for (int j = threadIdx.x; j < nrhs; j += blockDim.x) {
        s.iters[j] = 0;
        s.flags[j] = 0;
        const double b2 = s.bnorm2[j];
        int act = b2 >= 1e-60 ? 1 : 0;  // ||b|| < 1e-30 returns x = 0 (solvers.cpp:22-23)
        if (!isfinite(b2)) {
            act = 0;
            s.flags[j] |= 2;
        }
        s.active[j] = act;
        if (act) atomicAdd(s.n_active, 1);
    }
}

// breakdown guard before the update: pAp must be positive and finite
__global__ void k_pcg_check_pap(PcgState s, int nrhs) {
    int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= nrhs || !s.active[j]) return;
    double pap = s.pAp[j];
    if (!(pap > 0.0) || !isfinite(pap)) {
        s.flags[j] |= isfinite(pap) ? 1 : 2;
        s.active[j] = 0;
        atomicSub(s.n_active, 1);
    }
}

struct FinPcg {
    PcgState s;
    __device__ void operator()(int j, const double* sums) const {
        if (!s.active[j]) return;
        const double rr = sums[0];
        s.iters[j] += 1;
        s.rr[j] = rr;
        if (!isfinite(rr)) {
            s.flags[j] |= 2;
            s.active[j] = 0;
            atomicSub(s.n_active, 1);
        } else if (rr < s.tol2 * s.bnorm2[j]) {  // ||r|| / ||b|| < tol (solvers.cpp:59)
            s.active[j] = 0;
            atomicSub(s.n_active, 1);
        }
    }
};

// alpha = rz / pAp; x += alpha p; r -= alpha Ap; ||r||^2 with the stop rule
template <typename T>
__global__ void __launch_bounds__(256) k_pcg_update(PcgState s, const double* __restrict__ rz, VecView<T> x,
                                                    cx<T>* __restrict__ r, const cx<T>* __restrict__ p,
                                                    const cx<T>* __restrict__ Ap, double* partials,
                                                    unsigned int* ticket) {
    __shared__ cx<T> s_al[32];
    const int rhs = blockIdx.y * blockDim.x + threadIdx.x;
    if (threadIdx.y == 0) {
        cx<T> al = mk<T>(0, 0);
        if (rhs < x.nrhs && s.active[rhs]) {
            const double pap = s.pAp[rhs];
            al = mk<T>((T)(rz[2 * rhs] / pap), (T)(rz[2 * rhs + 1] / pap));
        }
        s_al[threadIdx.x] = al;
    }
    __syncthreads();
    const cx<T> al = s_al[threadIdx.x];
    T v[1] = {T(0)};
    if (rhs < x.nrhs) {
        for (int st = blockIdx.x * blockDim.y + threadIdx.y; st < x.nsites; st += gridDim.x * blockDim.y) {
            const int64_t i = x.idx(st, rhs, 0);
#pragma unroll
            for (int d = 0; d < 2; ++d) {
                const cx<T> ri = r[i + d] - al * Ap[i + d];
                x.p[i + d] = x.p[i + d] + al * p[i + d];
                r[i + d] = ri;
                v[0] += norm2(ri);
            }
        }
    }
    block_reduce_finalise<1>(v, partials, ticket, x.nrhs, FinPcg{s});
}

// beta = rz_new / rz_old (0 for a stopped rhs); p = z + beta p
template <typename T>
__global__ void k_pcg_p(PcgState s, const double* __restrict__ rz_old, const double* __restrict__ rz_new,
                        VecView<T> p, const cx<T>* __restrict__ z) {
    const int rhs = blockIdx.y * blockDim.x + threadIdx.x;
    const int st = blockIdx.x * blockDim.y + threadIdx.y;
    if (rhs >= p.nrhs || st >= p.nsites) return;
    cx<T> be = mk<T>(0, 0);
    if (s.active[rhs]) {
        const double ar = rz_old[2 * rhs], ai = rz_old[2 * rhs + 1];
        const double br = rz_new[2 * rhs], bi = rz_new[2 * rhs + 1];
        const double den = ar * ar + ai * ai;
        if (den > 0) be = mk<T>((T)((br * ar + bi * ai) / den), (T)((bi * ar - br * ai) / den));
    }
    const int64_t i = p.idx(st, rhs, 0);
#pragma unroll
    for (int d = 0; d < 2; ++d) p.p[i + d] = z[i + d] + be * p.p[i + d];
}

template <typename T>
smg_status pcg_run(smg_dirac* d, smg_mg* mg, const smg_field* b, smg_field* x, bool use_x0, int max_iter,
                   double tol, smg_solve_result* res) {
    smg_context* ctx = d->ctx;
    const int nrhs = b->nrhs, V = b->g.V;
    FieldSet fs;
    smg_field *r, *z, *p, *t, *Ap;
    SMG_TRY(fs.add(b, &r));
    SMG_TRY(fs.add(b, &z));
    SMG_TRY(fs.add(b, &p));
    SMG_TRY(fs.add(b, &t));
    SMG_TRY(fs.add(b, &Ap));
    const size_t nd = (size_t)nrhs * 9 + 8;
    const size_t bytes = nd * sizeof(double) + (size_t)nrhs * 3 * sizeof(int) + 64;
    char* blk = nullptr;
    SMG_CUDA(ctx, cudaMallocAsync((void**)&blk, bytes, ctx->stream));
    SMG_CUDA(ctx, cudaMemsetAsync(blk, 0, bytes, ctx->stream));
    PcgState s;
    double* dp = (double*)blk;
    s.rz[0] = dp;
    s.rz[1] = dp + 2 * nrhs;
    s.pAp = dp + 4 * nrhs;
    s.rr = dp + 5 * nrhs;
    s.bnorm2 = dp + 6 * nrhs;
    double* truev = dp + 7 * nrhs;
    s.active = (int*)(dp + nd);
    s.iters = s.active + nrhs;
    s.flags = s.iters + nrhs;
    s.n_active = (int*)(blk + bytes - 16);
    s.tol2 = tol * tol;
    const VecView<T> xv = fv<T>(x), pv = fv<T>(p);
    SMG_TRY(reduce_into<T>(ctx, fv<T>(b), nullptr, VR_NORM, s.bnorm2));
    if (use_x0) {  // r = b - A x0
        SMG_TRY(apply_A<T>(d, x, t, Ap));
        const int64_t n = b->n_complex();
        k_residual<T><<<(unsigned)((n + 255) / 256), 256, 0, ctx->stream>>>(
            (const cx<T>*)b->data, (const cx<T>*)Ap->data, (cx<T>*)r->data, n);
        count_launch(ctx);
    } else {
        SMG_CUDA(ctx, cudaMemsetAsync(x->data, 0, x->bytes, ctx->stream));
        SMG_CUDA(ctx, cudaMemcpyAsync(r->data, b->data, b->bytes, cudaMemcpyDeviceToDevice, ctx->stream));
    }
    k_pcg_init<<<1, 256, 0, ctx->stream>>>(s, nrhs);
    count_launch(ctx);
    auto precondition = [&]() -> smg_status {
        if (mg) return smg_mg_apply_internal(mg, r, z);
        SMG_CUDA(ctx, cudaMemcpyAsync(z->data, r->data, r->bytes, cudaMemcpyDeviceToDevice, ctx->stream));
        return SMG_OK;
    };
    SMG_TRY(precondition());
    SMG_CUDA(ctx, cudaMemcpyAsync(p->data, z->data, z->bytes, cudaMemcpyDeviceToDevice, ctx->stream));
    int cur = 0;
    SMG_TRY(reduce_into<T>(ctx, fv<T>(r), (const cx<T>*)z->data, VR_DOT, s.rz[cur]));
    const ReduceLaunch rl = reduce_launch(V, nrhs);
    SMG_TRY(smg_reduce_reserve(ctx, (size_t)rl.grid.x * nrhs * 3));
    const dim3 vg = vec_grid(V, nrhs), vb = vec_block(nrhs);
    SMG_TRY(smg_host_stage_reserve(ctx, 64));
    int* h_active = (int*)ctx->host_stage;
    // with a preconditioner the cycle dominates an iteration: check every step
    const int check_every = mg ? 1 : 8;
    int it = 0;
    SMG_CUDA(ctx, cudaMemcpyAsync(h_active, s.n_active, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    SMG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    bool done = *h_active == 0;
    while (!done && it < max_iter) {
        const int chunk = std::min(check_every, max_iter - it);
        for (int c = 0; c < chunk; ++c) {
            SMG_TRY(smg_dslash(d, false, p, t, s.pAp));
            SMG_TRY(smg_dslash(d, true, t, Ap, nullptr));
            k_pcg_check_pap<<<(nrhs + 127) / 128, 128, 0, ctx->stream>>>(s, nrhs);
            k_pcg_update<T><<<rl.grid, rl.block, 0, ctx->stream>>>(s, s.rz[cur], xv, (cx<T>*)r->data,
                                                                  (const cx<T>*)p->data, (const cx<T>*)Ap->data,
                                                                  ctx->red.partials, ctx->red.tickets);
            count_launch(ctx, 2);
            SMG_CHECK_LAUNCH(ctx);
            SMG_TRY(precondition());
            SMG_TRY(reduce_into<T>(ctx, fv<T>(r), (const cx<T>*)z->data, VR_DOT, s.rz[1 - cur]));
            k_pcg_p<T><<<vg, vb, 0, ctx->stream>>>(s, s.rz[cur], s.rz[1 - cur], pv, (const cx<T>*)z->data);
            count_launch(ctx);
            SMG_CHECK_LAUNCH(ctx);
            cur = 1 - cur;
        }
        it += chunk;
        SMG_CUDA(ctx, cudaMemcpyAsync(h_active, s.n_active, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
        SMG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        done = *h_active == 0;
    }
    // true residual in the field precision
    SMG_TRY(apply_A<T>(d, x, t, Ap));
    const int64_t n = b->n_complex();
    k_residual<T><<<(unsigned)((n + 255) / 256), 256, 0, ctx->stream>>>((const cx<T>*)b->data,
                                                                      (const cx<T>*)Ap->data, (cx<T>*)r->data, n);
    count_launch(ctx);
    SMG_TRY(reduce_into<T>(ctx, fv<T>(r), nullptr, VR_NORM, truev));
    std::vector<double> h(nd);
    std::vector<int> hi((size_t)nrhs * 3);
    SMG_CUDA(ctx, cudaMemcpyAsync(h.data(), dp, nd * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    SMG_CUDA(ctx, cudaMemcpyAsync(hi.data(), s.active, hi.size() * sizeof(int), cudaMemcpyDeviceToHost,
                                  ctx->stream));
    SMG_CUDA(ctx, cudaFreeAsync(blk, ctx->stream));
    SMG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    smg_status st = SMG_OK;
    int worst_it = 0;
    double worst_rec = 0, worst_true = 0;
    for (int j = 0; j < nrhs; ++j) {
        const double b2 = h[6 * nrhs + j];
        const double rr = hi[nrhs + j] > 0 ? h[5 * nrhs + j] : b2;
        if (b2 > 0 && std::isfinite(b2)) {
            worst_rec = std::max(worst_rec, std::sqrt(rr / b2));
            worst_true = std::max(worst_true, std::sqrt(h[7 * nrhs + j] / b2));
        }
        worst_it = std::max(worst_it, hi[nrhs + j]);
        const int flags = hi[2 * nrhs + j];
        if (flags & 2) st = SMG_NONFINITE;
        else if ((flags & 1) && st == SMG_OK) st = SMG_BREAKDOWN;
        else if (hi[j] && st == SMG_OK) st = SMG_NOT_CONVERGED;
    }
    if (res) {
        res->iterations = worst_it;
        res->final_residual = worst_rec;
        res->true_residual = worst_true;
        res->operator_applications = worst_it + 1 + (use_x0 ? 1 : 0);
    }
    if (mg) SMG_TRY(smg_mg_check_device_error(mg));
    if (st != SMG_OK) smg_fail(ctx, st, "cg_solve_precond: stopped before reaching the tolerance");
    return st;
}

// MR (omega = 0) or Richardson (omega > 0) smoothing of x on A = D^dag D
template <typename T>
smg_status smooth_run(smg_dirac* d, const smg_field* b, smg_field* x, int niter, double omega) {
    smg_context* ctx = d->ctx;
    const int nrhs = b->nrhs, V = b->g.V;
    FieldSet fs;
    smg_field *r, *Ar, *t;
    SMG_TRY(fs.add(b, &r));
    SMG_TRY(fs.add(b, &Ar));
    SMG_TRY(fs.add(b, &t));
    double* sc = nullptr;
    SMG_CUDA(ctx, cudaMallocAsync((void**)&sc, (size_t)nrhs * 3 * sizeof(double), ctx->stream));
    SMG_TRY(apply_A<T>(d, x, t, Ar));
    const int64_t n = b->n_complex();
    k_residual<T><<<(unsigned)((n + 255) / 256), 256, 0, ctx->stream>>>((const cx<T>*)b->data,
                                                                      (const cx<T>*)Ar->data, (cx<T>*)r->data, n);
    count_launch(ctx);
    const VecView<T> xv = fv<T>(x);
    const dim3 vg = vec_grid(V, nrhs), vb = vec_block(nrhs);
    smg_status st = SMG_OK;
    for (int it = 0; it < niter && st == SMG_OK; ++it) {
        st = apply_A<T>(d, r, t, Ar);
        if (st != SMG_OK) break;
        if (omega > 0) {
            k_rich_update<T><<<vg, vb, 0, ctx->stream>>>(xv, (cx<T>*)r->data, (const cx<T>*)Ar->data, (T)omega);
            count_launch(ctx);
        } else {
            st = reduce_into<T>(ctx, fv<T>(Ar), (const cx<T>*)r->data, VR_DOTNORM, sc);
            if (st != SMG_OK) break;
            k_mr_update<T><<<vg, vb, 0, ctx->stream>>>(xv, (cx<T>*)r->data, (const cx<T>*)Ar->data, sc);
            count_launch(ctx);
        }
        if (cudaGetLastError() != cudaSuccess) st = smg_fail(ctx, SMG_DEVICE_ERROR, "smoother launch failed");
    }
    cudaFreeAsync(sc, ctx->stream);
    SMG_TRY(st);
    SMG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return SMG_OK;
}

smg_status check_solve_args(smg_dirac* d, const smg_field* rhs, const smg_field* x) {
    if (!d || !rhs || !x) return SMG_BAD_ARG;
    smg_context* ctx = d->ctx;
    if (rhs == x) return smg_fail(ctx, SMG_BAD_ARG, "rhs and x must be distinct");
    SMG_TRY(smg_field_check_pair(rhs, x));
    if (rhs->g.L != d->gauge->g.L) return smg_fail(ctx, SMG_BAD_ARG, "field L differs from gauge L");
    if (rhs->prec != SMG_F64 && rhs->prec != SMG_F32)
        return smg_fail(ctx, SMG_UNSUPPORTED, "F16 fields are not supported by the solvers");
    return SMG_OK;
}

}  // namespace

extern "C" {

SMG_API smg_status smg_cg_solve_precond(smg_dirac* d, smg_mg* mg, const smg_field* rhs, smg_field* x,
                                        int use_x0, int max_iter, double tol, smg_solve_result* res) {
    SMG_TRY(check_solve_args(d, rhs, x));
    smg_context* ctx = d->ctx;
    if (max_iter < 0 || !(tol > 0)) return smg_fail(ctx, SMG_BAD_ARG, "max_iter >= 0 and tol > 0 required");
    if (mg) {
        int L = 0;
        SMG_TRY(smg_mg_level0_L(mg, &L));
        if (L != rhs->g.L) return smg_fail(ctx, SMG_BAD_ARG, "field L differs from the hierarchy's");
    }
    if (rhs->prec == SMG_F64) return pcg_run<double>(d, mg, rhs, x, use_x0 != 0, max_iter, tol, res);
    return pcg_run<float>(d, mg, rhs, x, use_x0 != 0, max_iter, tol, res);
}

SMG_API smg_status smg_mr_smooth(smg_dirac* d, const smg_field* b, smg_field* x, int niter) {
    SMG_TRY(check_solve_args(d, b, x));
    if (niter < 0) return smg_fail(d->ctx, SMG_BAD_ARG, "niter >= 0 required");
    if (b->prec == SMG_F64) return smooth_run<double>(d, b, x, niter, 0.0);
    return smooth_run<float>(d, b, x, niter, 0.0);
}

SMG_API smg_status smg_richardson_smooth(smg_dirac* d, const smg_field* b, smg_field* x, int niter,
                                         double omega) {
    SMG_TRY(check_solve_args(d, b, x));
    if (niter < 0 || !(omega > 0) || !std::isfinite(omega))
        return smg_fail(d->ctx, SMG_BAD_ARG, "niter >= 0 and a finite omega > 0 required");
    if (b->prec == SMG_F64) return smooth_run<double>(d, b, x, niter, omega);
    return smooth_run<float>(d, b, x, niter, omega);
}

SMG_API smg_status smg_estimate_lambda_max(smg_dirac* d, int niter, double* lambda) {
    if (!d || !lambda || niter < 0) return SMG_BAD_ARG;
    smg_context* ctx = d->ctx;
    const int L = d->gauge->g.L;
    const int64_t n = (int64_t)2 * L * L;
    smg_field *v = nullptr, *Av = nullptr, *t = nullptr;
    FieldSet fs;
    SMG_TRY(smg_field_create(ctx, L, 1, SMG_F64, &v));
    fs.f.push_back(v);
    SMG_TRY(fs.add(v, &Av));
    SMG_TRY(fs.add(v, &t));
    std::vector<double> h(2 * n);
    SMG_TRY(smg_host_random_vec(n, 12345u, h.data()));  // std::mt19937 rng_local(12345) (smoother.cpp:45)
    SMG_TRY(smg_field_upload(v, h.data()));
    double* sc = nullptr;
    SMG_CUDA(ctx, cudaMallocAsync((void**)&sc, sizeof(double), ctx->stream));
    SMG_TRY(smg_host_stage_reserve(ctx, 64));
    VecView<double> vv = fv<double>(v);
    const dim3 vg = vec_grid(vv.nsites, 1), vb = vec_block(1);
    smg_status st = reduce_into<double>(ctx, vv, nullptr, VR_NORM, sc);
    if (st == SMG_OK) {
        k_vconvert_scaled<double, double><<<vg, vb, 0, ctx->stream>>>(vv, (const cx<double>*)v->data, sc, 1);
        count_launch(ctx);
    }
    double lam = 0;
    for (int i = 0; i < niter && st == SMG_OK; ++i) {
        st = apply_A<double>(d, v, t, Av);
        if (st != SMG_OK) break;
        st = reduce_into<double>(ctx, fv<double>(Av), nullptr, VR_NORM, sc);
        if (st != SMG_OK) break;
        if (cudaMemcpyAsync(ctx->host_stage, sc, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream) !=
                cudaSuccess ||
            cudaStreamSynchronize(ctx->stream) != cudaSuccess) {
            st = smg_fail(ctx, SMG_DEVICE_ERROR, "estimate_lambda_max: read-back failed");
            break;
        }
        lam = std::sqrt(ctx->host_stage[0]);
        if (lam < 1e-30) break;
        k_vconvert_scaled<double, double><<<vg, vb, 0, ctx->stream>>>(vv, (const cx<double>*)Av->data, sc, 1);
        count_launch(ctx);
    }
    cudaFreeAsync(sc, ctx->stream);
    SMG_TRY(st);
    *lambda = lam;
    return SMG_OK;
}

SMG_API smg_status smg_fermion_action(smg_dirac* d, smg_mg* mg, const smg_field* phi, smg_field* X, int max_iter,
                                      double tol, double* action, smg_solve_result* res) {
    SMG_TRY(check_solve_args(d, phi, X));
    smg_context* ctx = d->ctx;
    smg_solve_result r{};
    SMG_TRY(smg_cg_solve_precond(d, mg, phi, X, 0, max_iter, tol, &r));
    if (res) *res = r;
    if (action) {
        const int nrhs = phi->nrhs;
        double* dots = nullptr;
        SMG_CUDA(ctx, cudaMallocAsync((void**)&dots, (size_t)2 * nrhs * sizeof(double), ctx->stream));
        smg_status st = phi->prec == SMG_F64
                            ? reduce_into<double>(ctx, fv<double>(phi), (const cx<double>*)X->data, VR_DOT, dots)
                            : reduce_into<float>(ctx, fv<float>(phi), (const cx<float>*)X->data, VR_DOT, dots);
        std::vector<double> h(2 * nrhs);
        if (st == SMG_OK)
            st = cudaMemcpyAsync(h.data(), dots, h.size() * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream) ==
                         cudaSuccess
                     ? SMG_OK
                     : smg_fail(ctx, SMG_DEVICE_ERROR, "fermion_action: read-back failed");
        cudaFreeAsync(dots, ctx->stream);
        SMG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        SMG_TRY(st);
        for (int j = 0; j < nrhs; ++j) action[j] = h[2 * j];  // S = Re <phi, X>
    }
    return SMG_OK;
}

}  // extern "C"
