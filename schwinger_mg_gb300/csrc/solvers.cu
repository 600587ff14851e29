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
#include "krylov.cuh"

#include <algorithm>
#include <cstdlib>
#include <cmath>


smg_status smg_eo_schur_internal(smg_dirac* d, bool dag, const smg_field* src, smg_field* dst, smg_field* tmp,
                                 double* norm2_dev);

namespace {

constexpr int kCheckEvery = 8;

// SMG_CUDA_GRAPHS=0 in the environment launches the CG chunks kernel by kernel
bool chunk_graphs_enabled() {
    const char* e = std::getenv("SMG_CUDA_GRAPHS");
    return !(e && std::atoi(e) == 0);
}

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
    T v[1] = {T(0)};
    if (rhs < nrhs) {
        for (int q = blockIdx.x * blockDim.y + threadIdx.y; q < nsites; q += gridDim.x * blockDim.y) {
#pragma unroll
            for (int sp = 0; sp < 2; ++sp) {
                int64_t i = sidx(q, rhs, sp, nrhs);
                cx<T> pi = p[i];
                cx<T> ri = r[i] - al * Ap[i];
                x[i] = x[i] + al * pi;
                r[i] = ri;
                v[0] += norm2(ri);
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

// eo: CG on the Schur complement M^dag M (EvenOddDiracOp::apply_schur_dag_schur,
// src/dirac.h:441-447) over the odd halves of the fields, as the reference's
// e/o HMC runs cg_solve on half-lattice vectors (src/hmc_trajectory.cpp:70-104)
template <typename T>
smg_status cg_run(smg_dirac* d, const smg_field* b, smg_field* x, int max_iter, double tol, smg_solve_result* res,
                  bool eo = false) {
    smg_context* ctx = b->ctx;
    const int nrhs = b->nrhs;
    const int V = eo ? b->g.Vh : b->g.V;                   // sites the solver runs over
    const int64_t off = eo ? (int64_t)b->g.Vh * nrhs * 2 : 0;  // complex offset of the odd half
    FieldSet fs;
    smg_field *r, *p, *t, *Ap, *te = nullptr;
    SMG_TRY(fs.add(b, &r));
    SMG_TRY(fs.add(b, &p));
    SMG_TRY(fs.add(b, &t));
    SMG_TRY(fs.add(b, &Ap));
    if (eo) SMG_TRY(fs.add(b, &te));
    auto vp = [&](const smg_field* f) { return (cx<T>*)f->data + off; };
    auto half_view = [&](const smg_field* f) {
        VecView<T> v = fv<T>(f);
        v.p += off;
        v.nsites = V;
        return v;
    };
    auto apply_normal = [&](const smg_field* in, smg_field* out, double* n2) {
        return eo ? smg_eo_schur_internal(d, false, in, out, te, n2) : smg_dslash(d, false, in, out, n2);
    };
    auto apply_dag = [&](const smg_field* in, smg_field* out) {
        return eo ? smg_eo_schur_internal(d, true, in, out, te, nullptr) : smg_dslash(d, true, in, out, nullptr);
    };

    // device scalar block
    size_t nbytes = (size_t)nrhs * (5 * sizeof(double) + 3 * sizeof(int)) + 64;
    PoolBuf blk_buf;
    SMG_TRY(blk_buf.take(ctx, nbytes));
    char* blk = static_cast<char*>(blk_buf.p);
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
    SMG_TRY(reduce_into<T>(ctx, half_view(r), nullptr, VR_NORM, s.rr));
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
    auto body = [&](int n) -> smg_status {
        for (int c = 0; c < n; ++c) {
            SMG_TRY(apply_normal(p, t, s.pAp));
            SMG_TRY(apply_dag(t, Ap));
            k_cg_check_pap<<<(nrhs + 127) / 128, 128, 0, ctx->stream>>>(s, nrhs);
            k_cg_update<T><<<rl.grid, rl.block, 0, ctx->stream>>>(s, vp(x), vp(r), vp(p), vp(Ap), V, nrhs,
                                                                 ctx->red.partials, ctx->red.tickets);
            k_cg_p<T><<<sl.grid, sl.block, 0, ctx->stream>>>(s, vp(r), vp(p), V, nrhs);
            count_launch(ctx, 3);
            SMG_CHECK_LAUNCH(ctx);
        }
        return SMG_OK;
    };
    // After the first chunk (which also settles the stencil's launch shape), a full chunk of
    // kCheckEvery iterations is captured once as a CUDA graph and replayed: the kernels of a small
    // lattice run a few microseconds each, so launch overhead would otherwise dominate.
    cudaGraphExec_t gexec = nullptr;
    uint64_t graph_launches = 0;
    bool use_graph = chunk_graphs_enabled();
    while (!done && it < max_iter) {
        int chunk = std::min(kCheckEvery, max_iter - it);
        if (use_graph && it > 0 && chunk == kCheckEvery) {
            if (!gexec) {
                const uint64_t l0 = ctx->launches;
                cudaGraph_t graph = nullptr;
                smg_status st = SMG_OK;
                if (cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
                    st = body(kCheckEvery);
                    const cudaError_t e = cudaStreamEndCapture(ctx->stream, &graph);
                    if (st == SMG_OK && e == cudaSuccess && graph &&
                        cudaGraphInstantiate(&gexec, graph, 0) != cudaSuccess)
                        gexec = nullptr;
                    if (graph) cudaGraphDestroy(graph);
                }
                graph_launches = ctx->launches - l0;
                ctx->launches = l0;
                cudaGetLastError();
                if (!gexec) use_graph = false;  // capture failed: launch kernel by kernel
            }
            if (gexec) {
                SMG_CUDA(ctx, cudaGraphLaunch(gexec, ctx->stream));
                count_launch(ctx, (int)graph_launches);
            } else {
                SMG_TRY(body(chunk));
            }
        } else {
            SMG_TRY(body(chunk));
        }
        it += chunk;
        SMG_CUDA(ctx, cudaMemcpyAsync(h_active, s.n_active, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
        SMG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        done = (*h_active == 0);
    }

    if (gexec) cudaGraphExecDestroy(gexec);

    // true residual ||b - A x|| / ||b|| with the operator of the field precision
    SMG_TRY(apply_normal(x, t, nullptr));
    SMG_TRY(apply_dag(t, Ap));
    const int64_t n = (int64_t)V * nrhs * 2;
    k_residual<T><<<(unsigned)((n + 255) / 256), 256, 0, ctx->stream>>>(vp(b), vp(Ap), vp(r), n);
    count_launch(ctx);
    SMG_TRY(reduce_into<T>(ctx, half_view(r), nullptr, VR_NORM, scratch_true));

    std::vector<double> h((size_t)nrhs * 5);
    std::vector<int> hi((size_t)nrhs * 3);
    SMG_CUDA(ctx, cudaMemcpyAsync(h.data(), blk, (size_t)nrhs * 5 * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    SMG_CUDA(ctx, cudaMemcpyAsync(hi.data(), s.active, (size_t)nrhs * 3 * sizeof(int), cudaMemcpyDeviceToHost,
                                  ctx->stream));
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

SMG_API smg_status smg_eo_cg_solve(smg_dirac* d, const smg_field* rhs, smg_field* x, int max_iter, double tol,
                                   smg_solve_result* res) {
    if (!d || !rhs || !x) return SMG_BAD_ARG;
    smg_context* ctx = d->ctx;
    if (rhs == x) return smg_fail(ctx, SMG_BAD_ARG, "rhs and x must be distinct");
    SMG_TRY(smg_field_check_pair(rhs, x));
    if (rhs->g.L != d->gauge->g.L || rhs->g.L % 2) return smg_fail(ctx, SMG_BAD_ARG, "field L differs from gauge L");
    if (max_iter < 0 || !(tol > 0)) return smg_fail(ctx, SMG_BAD_ARG, "max_iter >= 0 and tol > 0 required");
    if (rhs->prec == SMG_F64) return cg_run<double>(d, rhs, x, max_iter, tol, res, true);
    if (rhs->prec == SMG_F32) return cg_run<float>(d, rhs, x, max_iter, tol, res, true);
    return smg_fail(ctx, SMG_UNSUPPORTED, "eo_cg_solve on F16 fields");
}

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
smg_status smg_mg_apply_internal(smg_mg* mg, const smg_field* b, smg_field* x);
smg_status smg_mg_graph_io(smg_mg* mg, const smg_field* proto, smg_field** in, smg_field** out);
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

// Classical Gram-Schmidt of the new direction against the stored window
// (solvers.cpp:260-267) in two passes over the fine fields:
//   k_gcr_multidot   <AP_i, Az> for up to kDotChunk stored directions at once
//   k_gcr_orth_all   p = z - sum_i beta_i P_i, Ap = Az - sum_i beta_i AP_i for
//                    up to kOrthChunk directions, fused with <Ap, r>, ||Ap||^2
constexpr int kDotChunk = 8;
constexpr int kOrthChunk = 32;

template <typename T>
struct DotPtrs {
    const cx<T>* ap[kDotChunk];
};

// per-block partials of <AP_i, Az> (block_partials<2 kDotChunk>); k_sum_partials finishes them
template <typename T>
__global__ void __launch_bounds__(256) k_gcr_multidot(VecView<T> az, DotPtrs<T> ptr, int ns, double* partials) {
    constexpr int K = 2 * kDotChunk;
    const int rhs = blockIdx.y * blockDim.x + threadIdx.x;
    T v[K];  // per-thread partials in the field precision (FP64 is scarce on this part)
#pragma unroll
    for (int k = 0; k < K; ++k) v[k] = T(0);
    if (rhs < az.nrhs) {
        for (int s = blockIdx.x * blockDim.y + threadIdx.y; s < az.nsites; s += gridDim.x * blockDim.y) {
            const Spinor<T> z = ld_spinor(az.p, s, rhs, az.nrhs);
#pragma unroll
            for (int i = 0; i < kDotChunk; ++i) {
                if (i < ns) {
                    const Spinor<T> a = ld_spinor(ptr.ap[i], s, rhs, az.nrhs);
                    const cx<T> c = cmulc(a.s0, z.s0) + cmulc(a.s1, z.s1);
                    v[2 * i] += c.re;
                    v[2 * i + 1] += c.im;
                }
            }
        }
    }
    block_partials<K>(v, partials, az.nrhs);
}

template <typename T>
struct OrthPtrs {
    const cx<T>* P[kOrthChunk];
    const cx<T>* AP[kOrthChunk];
    const double* apap[kOrthChunk];  // [rhs][3] scalar slot of each stored direction (||AP_i||^2 at 2)
};

// beta_i = (ref ? conj : id)(<AP_i, Az>) / ||AP_i||^2, dots[rhs * stride + 2 (i0 + i)] = <AP_i, Az>
template <typename T>
__global__ void __launch_bounds__(256) k_gcr_orth_all(VecView<T> p, cx<T>* Ap,
                                                      const cx<T>* z, const cx<T>* Az,
                                                      const cx<T>* __restrict__ r, OrthPtrs<T> ptr, int ns, int i0,
                                                      const double* __restrict__ dots, int stride, int ref_coeff,
                                                      int last, double* partials, unsigned int* ticket,
                                                      double* apr3) {
    __shared__ cx<T> s_b[kOrthChunk][32];
    const int nrhs = p.nrhs;
    const int rhs = blockIdx.y * blockDim.x + threadIdx.x;
    for (int i = threadIdx.y; i < ns; i += blockDim.y) {
        cx<T> be = mk<T>(0, 0);
        if (rhs < nrhs) {
            const double den = ptr.apap[i][3 * rhs + 2];
            const double re = dots[rhs * stride + 2 * (i0 + i)];
            const double im = dots[rhs * stride + 2 * (i0 + i) + 1];
            if (den > 0) be = mk<T>((T)(re / den), (T)((ref_coeff ? -im : im) / den));
        }
        s_b[i][threadIdx.x] = be;
    }
    __syncthreads();
    T v[3] = {T(0), T(0), T(0)};
    if (rhs < nrhs) {
        for (int s = blockIdx.x * blockDim.y + threadIdx.y; s < p.nsites; s += gridDim.x * blockDim.y) {
            Spinor<T> q = ld_spinor(z, s, rhs, nrhs);
            Spinor<T> aq = ld_spinor(Az, s, rhs, nrhs);
#pragma unroll 4
            for (int i = 0; i < ns; ++i) {
                const cx<T> be = s_b[i][threadIdx.x];
                const Spinor<T> pi = ld_spinor(ptr.P[i], s, rhs, nrhs);
                const Spinor<T> ai = ld_spinor(ptr.AP[i], s, rhs, nrhs);
                q.s0 = q.s0 - be * pi.s0;
                q.s1 = q.s1 - be * pi.s1;
                aq.s0 = aq.s0 - be * ai.s0;
                aq.s1 = aq.s1 - be * ai.s1;
            }
            st_spinor(p.p, s, rhs, nrhs, q);
            st_spinor(Ap, s, rhs, nrhs, aq);
            if (last) {
                const Spinor<T> rr = ld_spinor(r, s, rhs, nrhs);
                const cx<T> c = cmulc(aq.s0, rr.s0) + cmulc(aq.s1, rr.s1);
                v[0] += c.re;
                v[1] += c.im;
                v[2] += norm2(aq.s0) + norm2(aq.s1);
            }
        }
    }
    if (last) block_reduce_finalise<3>(v, partials, ticket, nrhs, FinStore{apr3, 3});
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
    T v[1] = {T(0)};
    if (rhs < nrhs) {
        for (int st = blockIdx.x * blockDim.y + threadIdx.y; st < x.nsites; st += gridDim.x * blockDim.y) {
            const int64_t base = x.idx(st, rhs, 0);
            const int ds = x.dstride();
            for (int d = 0; d < x.ndof; ++d) {
                const cx<T> ri = r[base + (int64_t)d * ds] - al * Ap[base + (int64_t)d * ds];
                x.p[base + (int64_t)d * ds] = x.p[base + (int64_t)d * ds] + al * p[base + (int64_t)d * ds];
                r[base + (int64_t)d * ds] = ri;
                v[0] += norm2(ri);
            }
        }
    }
    block_reduce_finalise<1>(v, partials, ticket, nrhs, FinGcr{sc});
}

// Workspace of one GCR solve: residual, preconditioned residual, A z, the
// D^dag D temporary, the ring of (p, A p) pairs and the device scalars.
template <typename T>
struct GcrWs {
    FieldSet fs;
    smg_field *r = nullptr, *z = nullptr, *Az = nullptr, *tmp = nullptr;
    std::vector<smg_field*> P, AP;
    double* blk = nullptr;
    smg_context* ctx = nullptr;
    GcrScalars sc;
    double* truev = nullptr;
    double* dots = nullptr;
    double* apr = nullptr;
    int nrhs = 0, nbuf = 0;
    PoolBuf blk_buf;
    double* apr_of(int buf) const { return apr + (size_t)buf * 3 * nrhs; }
    smg_status init(smg_context* c, const smg_field* proto, int trunc) {
        ctx = c;
        nrhs = proto->nrhs;
        nbuf = trunc + 1;
        SMG_TRY(fs.add(proto, &r));
        SMG_TRY(fs.add(proto, &z));
        SMG_TRY(fs.add(proto, &Az));
        SMG_TRY(fs.add(proto, &tmp));
        P.resize(nbuf);
        AP.resize(nbuf);
        for (int i = 0; i < nbuf; ++i) {
            SMG_TRY(fs.add(proto, &P[i]));
            SMG_TRY(fs.add(proto, &AP[i]));
        }
        const size_t nd_ = (size_t)nrhs * (3 + 5 * nbuf) + 64;
        const size_t bytes = nd_ * sizeof(double) + (size_t)nrhs * 2 * sizeof(int) + 64;
        SMG_TRY(blk_buf.take(ctx, bytes));
        blk = static_cast<double*>(blk_buf.p);
        SMG_CUDA(ctx, cudaMemsetAsync(blk, 0, bytes, ctx->stream));
        sc.rr = blk;
        sc.bnorm2 = blk + nrhs;
        truev = blk + 2 * nrhs;
        dots = blk + 3 * nrhs;                    // [rhs][nbuf][2]
        apr = blk + 3 * nrhs + 2 * nrhs * nbuf;  // nbuf * 3 * nrhs
        sc.active = (int*)(blk + nd_);
        sc.flags = sc.active + nrhs;
        return SMG_OK;
    }
};

struct GcrOut {
    int iterations = 0;
    bool nonfinite = false;
    std::vector<int> active;     // per rhs: still above tolerance
    std::vector<double> rr, b2;  // per rhs recursive ||r||^2 and ||b||^2
};

// The GCR iteration (fcg_solve, src/solvers.cpp:223-300) on fields of
// precision T from x = 0; the preconditioner is one MG cycle in the field
// precision (mg != nullptr) or the identity.
template <typename T>
smg_status gcr_core(smg_dirac* d, smg_mg* mg, GcrWs<T>& ws, const smg_field* b, smg_field* x, int max_iter, double tol,
                    int trunc, int ref_coeff, GcrOut& out) {
    // the residual and the preconditioned vector live in the captured cycle's own input and output
    // fields when the hierarchy has one, so a cycle copies neither (two 134 MB copies per cycle at
    // L = 512, 32 RHS in FP32)
    smg_field* rf = ws.r;
    smg_field* zf = ws.z;
    static const bool graph_io = [] {
        const char* e = std::getenv("SMG_GRAPH_IO");
        return !(e && std::atoi(e) == 0);
    }();
    if (mg && graph_io) {
        smg_field *gi = nullptr, *go = nullptr;
        SMG_TRY(smg_mg_graph_io(mg, ws.r, &gi, &go));
        if (gi && go) {
            rf = gi;
            zf = go;
        }
    }
    smg_context* ctx = d->ctx;
    const int nrhs = b->nrhs, V = b->g.V;
    GcrScalars& sc = ws.sc;
    sc.tol2 = tol * tol;
    SMG_CUDA(ctx, cudaMemsetAsync(x->data, 0, x->bytes, ctx->stream));
    SMG_CUDA(ctx, cudaMemcpyAsync(rf->data, b->data, b->bytes, cudaMemcpyDeviceToDevice, ctx->stream));
    SMG_TRY(reduce_into<T>(ctx, fv<T>(rf), nullptr, VR_NORM, sc.rr));
    SMG_CUDA(ctx, cudaMemcpyAsync(sc.bnorm2, sc.rr, nrhs * sizeof(double), cudaMemcpyDeviceToDevice, ctx->stream));
    out.rr.assign(nrhs, 0.0);
    out.b2.assign(nrhs, 0.0);
    out.active.assign(nrhs, 1);
    SMG_CUDA(ctx, cudaMemcpyAsync(out.b2.data(), sc.bnorm2, nrhs * sizeof(double), cudaMemcpyDeviceToHost,
                                  ctx->stream));
    SMG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    out.rr = out.b2;
    for (int j = 0; j < nrhs; ++j) {
        out.active[j] = (out.b2[j] >= 1e-60 && std::isfinite(out.b2[j])) ? 1 : 0;
        if (!std::isfinite(out.b2[j])) out.nonfinite = true;
    }
    std::vector<int> ring;  // buffer indices of stored directions, oldest first
    int work = 0;           // buffer index of the current (p, Ap) pair
    std::vector<int> freeb;
    for (int i = 1; i < ws.nbuf; ++i) freeb.push_back(i);
    int iter = 0;
    const ReduceLaunch rl = reduce_launch(V, nrhs);
    SMG_TRY(smg_reduce_reserve(ctx, (size_t)rl.grid.x * nrhs * 2 * kDotChunk));
    bool any_active = false;
    for (int j = 0; j < nrhs; ++j) any_active |= out.active[j] != 0;
    std::vector<double> h_apr(3 * nrhs);
    while (any_active && iter < max_iter) {
        SMG_CUDA(ctx, cudaMemcpyAsync(sc.active, out.active.data(), nrhs * sizeof(int), cudaMemcpyHostToDevice,
                                      ctx->stream));
        // z = M^-1 r
        if (!mg)
            SMG_CUDA(ctx, cudaMemcpyAsync(zf->data, rf->data, rf->bytes, cudaMemcpyDeviceToDevice, ctx->stream));
        else
            SMG_TRY(smg_mg_apply_internal(mg, rf, zf));
        // p = z, Ap = A z, orthogonalised against the stored directions
        smg_field* p = ws.P[work];
        smg_field* Ap = ws.AP[work];
        SMG_TRY(apply_A<T>(d, zf, ws.tmp, ws.Az));
        const int nring = (int)ring.size();
        // <AP_i, Az> for every stored direction, kDotChunk per pass over Az
        for (int c0 = 0; c0 < nring; c0 += kDotChunk) {
            DotPtrs<T> dp{};
            const int ns = std::min(kDotChunk, nring - c0);
            for (int i = 0; i < ns; ++i) dp.ap[i] = (const cx<T>*)ws.AP[ring[c0 + i]]->data;
            // every resident block streams Az and the AP_i; the 2 ns block partials per rhs are summed
            // by one warp each in a second kernel (a single finishing block would serialise them)
            k_gcr_multidot<T><<<rl.grid, rl.block, 0, ctx->stream>>>(fv<T>(ws.Az), dp, ns, ctx->red.partials);
            const int nwarp = nrhs * 2 * ns;
            k_sum_partials<<<(nwarp + 7) / 8, 256, 0, ctx->stream>>>(ctx->red.partials, (int)rl.grid.x, nrhs,
                                                                    2 * kDotChunk, 2 * ns, ws.dots + 2 * c0,
                                                                    2 * ws.nbuf);
            count_launch(ctx, 2);
            SMG_CHECK_LAUNCH(ctx);
        }
        // p and Ap in kOrthChunk passes; the last one also forms <Ap, r> and ||Ap||^2
        for (int c0 = 0; c0 == 0 || c0 < nring; c0 += kOrthChunk) {
            OrthPtrs<T> op{};
            const int ns = std::min(kOrthChunk, nring - c0);
            for (int i = 0; i < ns; ++i) {
                op.P[i] = (const cx<T>*)ws.P[ring[c0 + i]]->data;
                op.AP[i] = (const cx<T>*)ws.AP[ring[c0 + i]]->data;
                op.apap[i] = ws.apr_of(ring[c0 + i]);
            }
            const bool first = c0 == 0, last = c0 + kOrthChunk >= nring;
            k_gcr_orth_all<T><<<rl.grid, rl.block, 0, ctx->stream>>>(
                fv<T>(p), (cx<T>*)Ap->data, first ? (const cx<T>*)zf->data : (const cx<T>*)p->data,
                first ? (const cx<T>*)ws.Az->data : (const cx<T>*)Ap->data, (const cx<T>*)rf->data, op, ns, c0,
                ws.dots, 2 * ws.nbuf, ref_coeff, last ? 1 : 0, ctx->red.partials, ctx->red.tickets,
                ws.apr_of(work));
            count_launch(ctx);
            SMG_CHECK_LAUNCH(ctx);
        }
        sc.apr3 = ws.apr_of(work);
        k_gcr_update<T><<<rl.grid, rl.block, 0, ctx->stream>>>(sc, fv<T>(x), (cx<T>*)rf->data,
                                                               (const cx<T>*)p->data, (const cx<T>*)Ap->data,
                                                               ctx->red.partials, ctx->red.tickets);
        count_launch(ctx);
        SMG_CHECK_LAUNCH(ctx);
        // host: stop rule and breakdown (||Ap||^2 < 1e-30 clears the history, solvers.cpp:272-276)
        SMG_CUDA(ctx, cudaMemcpyAsync(out.rr.data(), sc.rr, nrhs * sizeof(double), cudaMemcpyDeviceToHost,
                                      ctx->stream));
        SMG_CUDA(ctx, cudaMemcpyAsync(h_apr.data(), ws.apr_of(work), 3 * nrhs * sizeof(double),
                                      cudaMemcpyDeviceToHost, ctx->stream));
        SMG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        bool breakdown = false;
        for (int j = 0; j < nrhs; ++j)
            if (out.active[j] && !(h_apr[3 * j + 2] >= 1e-30)) breakdown = true;
        if (breakdown) {
            for (int slot : ring) freeb.push_back(slot);
            ring.clear();
            bool any_nan = false;
            for (int j = 0; j < nrhs; ++j)
                if (out.active[j] && !std::isfinite(h_apr[3 * j + 2])) any_nan = true;
            if (any_nan) {
                out.nonfinite = true;
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
            if (out.active[j]) {
                if (!std::isfinite(out.rr[j])) {
                    out.nonfinite = true;
                    out.active[j] = 0;
                } else if (out.rr[j] < tol * tol * out.b2[j]) {
                    out.active[j] = 0;
                }
            }
            any_active |= out.active[j] != 0;
        }
    }
    out.iterations = iter;
    return SMG_OK;
}

template <typename T>
smg_status gcr_run(smg_dirac* d, smg_mg* mg, const smg_field* b, smg_field* x, int max_iter, double tol, int trunc,
                   int ref_coeff, smg_solve_result* res) {
    smg_context* ctx = d->ctx;
    const int nrhs = b->nrhs;
    GcrWs<T> ws;
    SMG_TRY(ws.init(ctx, b, trunc));
    GcrOut out;
    SMG_TRY(gcr_core<T>(d, mg, ws, b, x, max_iter, tol, trunc, ref_coeff, out));
    // true residual in the field precision
    SMG_TRY(apply_A<T>(d, x, ws.tmp, ws.Az));
    int64_t n = b->n_complex();
    k_residual<T><<<(unsigned)((n + 255) / 256), 256, 0, ctx->stream>>>((const cx<T>*)b->data,
                                                                      (const cx<T>*)ws.Az->data,
                                                                      (cx<T>*)ws.r->data, n);
    count_launch(ctx);
    SMG_TRY(reduce_into<T>(ctx, fv<T>(ws.r), nullptr, VR_NORM, ws.truev));
    std::vector<double> h_true(nrhs);
    SMG_CUDA(ctx, cudaMemcpyAsync(h_true.data(), ws.truev, nrhs * sizeof(double), cudaMemcpyDeviceToHost,
                                  ctx->stream));
    SMG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    double worst_rec = 0, worst_true = 0;
    bool notconv = false;
    for (int j = 0; j < nrhs; ++j) {
        if (out.b2[j] > 0 && std::isfinite(out.b2[j])) {
            worst_rec = std::max(worst_rec, std::sqrt(out.rr[j] / out.b2[j]));
            worst_true = std::max(worst_true, std::sqrt(h_true[j] / out.b2[j]));
        }
        if (out.active[j]) notconv = true;
    }
    if (res) {
        res->iterations = out.iterations;
        res->final_residual = worst_rec;
        res->true_residual = worst_true;
        res->operator_applications = out.iterations + 1;
    }
    if (mg) SMG_TRY(smg_mg_check_device_error(mg));
    if (out.nonfinite) return smg_fail(ctx, SMG_NONFINITE, "gcr_solve: non-finite residual");
    if (notconv) return smg_fail(ctx, SMG_NOT_CONVERGED, "gcr_solve: iteration limit reached");
    return SMG_OK;
}

// out(D) = mult[rhs] * in(S) per right-hand side (fine fields)
template <typename D, typename S>
__global__ void k_convert_mul(VecView<D> out, const cx<S>* __restrict__ in, const double* __restrict__ mult) {
    const int rhs = blockIdx.y * blockDim.x + threadIdx.x;
    const int s = blockIdx.x * blockDim.y + threadIdx.y;
    if (rhs >= out.nrhs || s >= out.nsites) return;
    const double f = mult[rhs];
    const int64_t base = out.idx(s, rhs, 0);
    for (int d = 0; d < out.ndof; ++d) {
        const cx<S> v = in[base + d];
        out.p[base + d] = mk<D>((D)((double)v.re * f), (D)((double)v.im * f));
    }
}

// y(D) += mult[rhs] * x(S) per right-hand side (fine fields)
template <typename D, typename S>
__global__ void k_axpy_mul(VecView<D> y, const cx<S>* __restrict__ x, const double* __restrict__ mult) {
    const int rhs = blockIdx.y * blockDim.x + threadIdx.x;
    const int s = blockIdx.x * blockDim.y + threadIdx.y;
    if (rhs >= y.nrhs || s >= y.nsites) return;
    const double f = mult[rhs];
    const int64_t base = y.idx(s, rhs, 0);
    for (int d = 0; d < y.ndof; ++d) {
        const cx<S> v = x[base + d];
        const cx<D> o = y.p[base + d];
        y.p[base + d] = mk<D>((D)((double)o.re + (double)v.re * f), (D)((double)o.im + (double)v.im * f));
    }
}

// Mixed precision: FP64 defect correction around an FP32 GCR preconditioned
// by the FP32 hierarchy.  Each outer step forms the true FP64 residual
// r = b - A x, solves A e = r / ||r|| in FP32 to kInnerTol (or further when
// that suffices for tol), and adds x += ||r|| e in FP64.  FP64 work is one
// D^dag D per outer step and the residual reductions.
constexpr double kInnerTol = 1e-5;

smg_status gcr_mixed(smg_dirac* d, smg_mg* mg, const smg_field* b, smg_field* x, int max_iter, double tol, int trunc,
                     int ref_coeff, smg_solve_result* res) {
    smg_context* ctx = d->ctx;
    const int nrhs = b->nrhs, V = b->g.V;
    FieldSet fs;
    smg_field *r64, *t64, *Ax64;
    SMG_TRY(fs.add(b, &r64));
    SMG_TRY(fs.add(b, &t64));
    SMG_TRY(fs.add(b, &Ax64));
    smg_field *r32 = nullptr, *e32 = nullptr;
    SMG_TRY(fs.add(b, SMG_F32, &r32));
    SMG_TRY(fs.add(b, SMG_F32, &e32));
    GcrWs<float> ws;
    SMG_TRY(ws.init(ctx, r32, trunc));
    PoolBuf sc_buf;  // [0, nrhs) ||r||^2, [nrhs, 2 nrhs) multipliers
    SMG_TRY(sc_buf.take(ctx, (size_t)2 * nrhs * sizeof(double)));
    double* sc = static_cast<double*>(sc_buf.p);
    std::vector<double> b2(nrhs), rr(nrhs), mult(nrhs);
    // x = 0, r = b
    SMG_CUDA(ctx, cudaMemsetAsync(x->data, 0, x->bytes, ctx->stream));
    SMG_CUDA(ctx, cudaMemcpyAsync(r64->data, b->data, b->bytes, cudaMemcpyDeviceToDevice, ctx->stream));
    SMG_TRY(reduce_into<double>(ctx, fv<double>(r64), nullptr, VR_NORM, sc));
    SMG_CUDA(ctx, cudaMemcpyAsync(b2.data(), sc, nrhs * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    SMG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    rr = b2;
    bool nonfinite = false;
    for (int j = 0; j < nrhs; ++j)
        if (!std::isfinite(b2[j])) nonfinite = true;
    int total = 0;
    smg_status st = SMG_OK;
    while (!nonfinite && total < max_iter) {
        bool any = false;
        double worst_ratio = 0;
        for (int j = 0; j < nrhs; ++j) {
            const bool act = b2[j] >= 1e-60 && rr[j] >= tol * tol * b2[j];
            mult[j] = act ? 1.0 / std::sqrt(rr[j]) : 0.0;  // a finished rhs gets a zero inner rhs
            if (act) {
                any = true;
                worst_ratio = std::max(worst_ratio, std::sqrt(rr[j] / b2[j]));
            }
        }
        if (!any) break;
        // inner tolerance: kInnerTol, or the reduction that reaches tol
        const double inner_tol = std::max(kInnerTol, 0.5 * tol / worst_ratio);
        SMG_CUDA(ctx, cudaMemcpyAsync(sc + nrhs, mult.data(), nrhs * sizeof(double), cudaMemcpyHostToDevice,
                                      ctx->stream));
        k_convert_mul<float, double><<<vec_grid(V, nrhs), vec_block(nrhs), 0, ctx->stream>>>(
            fv<float>(r32), (const cx<double>*)r64->data, sc + nrhs);
        count_launch(ctx);
        GcrOut out;
        SMG_TRY(gcr_core<float>(d, mg, ws, r32, e32, max_iter - total, inner_tol, trunc, ref_coeff, out));
        total += out.iterations;
        if (out.nonfinite) {
            nonfinite = true;
            break;
        }
        for (int j = 0; j < nrhs; ++j) mult[j] = mult[j] > 0 ? std::sqrt(rr[j]) : 0.0;
        SMG_CUDA(ctx, cudaMemcpyAsync(sc + nrhs, mult.data(), nrhs * sizeof(double), cudaMemcpyHostToDevice,
                                      ctx->stream));
        k_axpy_mul<double, float><<<vec_grid(V, nrhs), vec_block(nrhs), 0, ctx->stream>>>(
            fv<double>(x), (const cx<float>*)e32->data, sc + nrhs);
        count_launch(ctx);
        // true FP64 residual
        SMG_TRY(apply_A<double>(d, x, t64, Ax64));
        const int64_t n = b->n_complex();
        k_residual<double><<<(unsigned)((n + 255) / 256), 256, 0, ctx->stream>>>(
            (const cx<double>*)b->data, (const cx<double>*)Ax64->data, (cx<double>*)r64->data, n);
        count_launch(ctx);
        SMG_TRY(reduce_into<double>(ctx, fv<double>(r64), nullptr, VR_NORM, sc));
        SMG_CUDA(ctx, cudaMemcpyAsync(rr.data(), sc, nrhs * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
        SMG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        for (int j = 0; j < nrhs; ++j)
            if (!std::isfinite(rr[j])) nonfinite = true;
        if (out.iterations == 0) break;  // no progress possible
    }
    double worst = 0;
    bool notconv = false;
    for (int j = 0; j < nrhs; ++j) {
        if (b2[j] > 0 && std::isfinite(b2[j])) {
            const double rel = std::sqrt(rr[j] / b2[j]);
            worst = std::max(worst, rel);
            if (!(rel < tol)) notconv = true;
        }
    }
    if (res) {
        res->iterations = total;
        res->final_residual = worst;
        res->true_residual = worst;
        res->operator_applications = total + 1;
    }
    SMG_TRY(smg_mg_check_device_error(mg));
    if (nonfinite) st = smg_fail(ctx, SMG_NONFINITE, "gcr_solve: non-finite residual");
    else if (notconv) st = smg_fail(ctx, SMG_NOT_CONVERGED, "gcr_solve: iteration limit reached");
    return st;
}

// Mixed-precision CG: FP64 defect correction around the FP32 CG.  Each outer
// step forms the true FP64 residual r = b - A x, solves A e = r / ||r|| with
// the FP32 operator to kInnerTol (or further when that suffices for tol), and
// adds x += ||r|| e in FP64 (same scheme as the mixed GCR above).
smg_status cg_mixed(smg_dirac* d, const smg_field* b, smg_field* x, int max_iter, double tol, smg_solve_result* res) {
    smg_context* ctx = d->ctx;
    const int nrhs = b->nrhs, V = b->g.V;
    FieldSet fs;
    smg_field *r64, *t64, *Ax64;
    SMG_TRY(fs.add(b, &r64));
    SMG_TRY(fs.add(b, &t64));
    SMG_TRY(fs.add(b, &Ax64));
    smg_field *r32 = nullptr, *e32 = nullptr;
    SMG_TRY(fs.add(b, SMG_F32, &r32));
    SMG_TRY(fs.add(b, SMG_F32, &e32));
    SMG_TRY(smg_gauge_ensure_f32(d->gauge));
    PoolBuf sc_buf;  // [0, nrhs) ||r||^2, [nrhs, 2 nrhs) multipliers
    SMG_TRY(sc_buf.take(ctx, (size_t)2 * nrhs * sizeof(double)));
    double* sc = static_cast<double*>(sc_buf.p);
    std::vector<double> b2(nrhs), rr(nrhs), mult(nrhs);
    SMG_CUDA(ctx, cudaMemsetAsync(x->data, 0, x->bytes, ctx->stream));
    SMG_CUDA(ctx, cudaMemcpyAsync(r64->data, b->data, b->bytes, cudaMemcpyDeviceToDevice, ctx->stream));
    SMG_TRY(reduce_into<double>(ctx, fv<double>(r64), nullptr, VR_NORM, sc));
    SMG_CUDA(ctx, cudaMemcpyAsync(b2.data(), sc, nrhs * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    SMG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    rr = b2;
    bool nonfinite = false;
    for (int j = 0; j < nrhs; ++j)
        if (!std::isfinite(b2[j])) nonfinite = true;
    int total = 0;
    while (!nonfinite && total < max_iter) {
        bool any = false;
        double worst_ratio = 0;
        for (int j = 0; j < nrhs; ++j) {
            const bool act = b2[j] >= 1e-60 && rr[j] >= tol * tol * b2[j];
            mult[j] = act ? 1.0 / std::sqrt(rr[j]) : 0.0;
            if (act) {
                any = true;
                worst_ratio = std::max(worst_ratio, std::sqrt(rr[j] / b2[j]));
            }
        }
        if (!any) break;
        const double inner_tol = std::max(kInnerTol, 0.5 * tol / worst_ratio);
        SMG_CUDA(ctx, cudaMemcpyAsync(sc + nrhs, mult.data(), nrhs * sizeof(double), cudaMemcpyHostToDevice,
                                      ctx->stream));
        k_convert_mul<float, double><<<vec_grid(V, nrhs), vec_block(nrhs), 0, ctx->stream>>>(
            fv<float>(r32), (const cx<double>*)r64->data, sc + nrhs);
        count_launch(ctx);
        smg_solve_result ir{};
        const smg_status ist = cg_run<float>(d, r32, e32, max_iter - total, inner_tol, &ir);
        if (ist == SMG_NONFINITE) {
            nonfinite = true;
            break;
        }
        total += ir.iterations;
        for (int j = 0; j < nrhs; ++j) mult[j] = mult[j] > 0 ? std::sqrt(rr[j]) : 0.0;
        SMG_CUDA(ctx, cudaMemcpyAsync(sc + nrhs, mult.data(), nrhs * sizeof(double), cudaMemcpyHostToDevice,
                                      ctx->stream));
        k_axpy_mul<double, float><<<vec_grid(V, nrhs), vec_block(nrhs), 0, ctx->stream>>>(
            fv<double>(x), (const cx<float>*)e32->data, sc + nrhs);
        count_launch(ctx);
        SMG_TRY(apply_A<double>(d, x, t64, Ax64));
        const int64_t n = b->n_complex();
        k_residual<double><<<(unsigned)((n + 255) / 256), 256, 0, ctx->stream>>>(
            (const cx<double>*)b->data, (const cx<double>*)Ax64->data, (cx<double>*)r64->data, n);
        count_launch(ctx);
        SMG_TRY(reduce_into<double>(ctx, fv<double>(r64), nullptr, VR_NORM, sc));
        SMG_CUDA(ctx, cudaMemcpyAsync(rr.data(), sc, nrhs * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
        SMG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        for (int j = 0; j < nrhs; ++j)
            if (!std::isfinite(rr[j])) nonfinite = true;
        if (ir.iterations == 0) break;  // no progress possible
    }
    double worst = 0;
    bool notconv = false;
    for (int j = 0; j < nrhs; ++j) {
        if (b2[j] > 0 && std::isfinite(b2[j])) {
            const double rel = std::sqrt(rr[j] / b2[j]);
            worst = std::max(worst, rel);
            if (!(rel < tol)) notconv = true;
        }
    }
    if (res) {
        res->iterations = total;
        res->final_residual = worst;
        res->true_residual = worst;
        res->operator_applications = total + 1;
    }
    if (nonfinite) return smg_fail(ctx, SMG_NONFINITE, "cg_solve_mixed: non-finite residual");
    if (notconv) return smg_fail(ctx, SMG_NOT_CONVERGED, "cg_solve_mixed: iteration limit reached");
    return SMG_OK;
}

}  // namespace

extern "C" {

SMG_API smg_status smg_cg_solve_mixed(smg_dirac* d, const smg_field* rhs, smg_field* x, int max_iter, double tol,
                                      smg_solve_result* res) {
    if (!d || !rhs || !x) return SMG_BAD_ARG;
    smg_context* ctx = d->ctx;
    if (rhs == x) return smg_fail(ctx, SMG_BAD_ARG, "rhs and x must be distinct");
    SMG_TRY(smg_field_check_pair(rhs, x));
    if (rhs->prec != SMG_F64) return smg_fail(ctx, SMG_BAD_ARG, "cg_solve_mixed needs F64 fields");
    if (rhs->g.L != d->gauge->g.L) return smg_fail(ctx, SMG_BAD_ARG, "field L differs from gauge L");
    if (max_iter < 0 || !(tol > 0)) return smg_fail(ctx, SMG_BAD_ARG, "max_iter >= 0 and tol > 0 required");
    return cg_mixed(d, rhs, x, max_iter, tol, res);
}

SMG_API smg_status smg_gcr_solve(smg_dirac* d, smg_mg* mg, const smg_field* rhs, smg_field* x, int max_iter, double tol,
                                 int trunc, int reference_coefficient, smg_solve_result* res) {
    if (!d || !rhs || !x) return SMG_BAD_ARG;
    smg_context* ctx = d->ctx;
    if (rhs == x) return smg_fail(ctx, SMG_BAD_ARG, "rhs and x must be distinct");
    SMG_TRY(smg_field_check_pair(rhs, x));
    if (rhs->g.L != d->gauge->g.L) return smg_fail(ctx, SMG_BAD_ARG, "field L differs from gauge L");
    if (max_iter < 0 || !(tol > 0) || trunc < 1 || trunc > 256)
        return smg_fail(ctx, SMG_BAD_ARG, "max_iter >= 0, tol > 0 and trunc in [1, 256] required");
    if (rhs->prec == SMG_F64) {
        if (mg && smg_mg_precision(mg) == SMG_F32)
            return gcr_mixed(d, mg, rhs, x, max_iter, tol, trunc, reference_coefficient, res);
        return gcr_run<double>(d, mg, rhs, x, max_iter, tol, trunc, reference_coefficient, res);
    }
    if (rhs->prec == SMG_F32) {
        if (mg && smg_mg_precision(mg) == SMG_F64)
            return smg_fail(ctx, SMG_UNSUPPORTED, "an F64 hierarchy needs F64 fields");
        return gcr_run<float>(d, mg, rhs, x, max_iter, tol, trunc, reference_coefficient, res);
    }
    return smg_fail(ctx, SMG_UNSUPPORTED, "gcr_solve on F16 fields");
}

}  // extern "C"
