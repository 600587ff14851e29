// Restarted flexible GMRES on A = D^dag D with Ritz harvesting
// (the reference's fgmres_solve_generic / fgmres_solve_mg,
// src/solvers.cpp:555-800, 776-787), batched over right-hand sides.
//
// Every right-hand side runs its own Arnoldi process in the same launches:
// one MG cycle (or the identity) gives Z_k = M^-1 V_k, W = A Z_k is
// orthogonalised against V_0..V_k by two classical Gram-Schmidt passes
// (the reference uses two modified Gram-Schmidt passes; both leave W
// orthogonal to working precision), and a one-block kernel applies the
// Givens rotations to the new Hessenberg column per right-hand side and
// applies the stop rule |g_{k+1}| / ||b|| < tol.  A right-hand side that
// stops (tolerance, breakdown, end of its cycle) is masked out of the
// remaining steps of the cycle.  The host reads one counter per step.
//
// At the end of a cycle each right-hand side solves its triangular system,
// x += Z y, and harvests Ritz pairs: G = H~^dag H~ from the unreduced
// Hessenberg matrix is diagonalised on the host (cyclic complex Jacobi) and
// the n_ritz smallest pairs become unit vectors sum_j v_j Z_j kept in
// per-rhs slots (at most 3 n_ritz: the reference's list trims to n_ritz when
// it exceeds 2 n_ritz).  In later cycles Z_k += sum_p (<v_p, V_k> / theta_p) v_p
// for the stored pairs with theta_p > 1e-14.
//
// Quirks kept from the reference: a happy breakdown (H_{k+1,k} < 1e-14)
// ends the cycle before the rotations touch column k and without counting
// the step, and the cycle's final |g_kk| then reads zero; the outer loop
// stops on the true residual or the iteration budget.
#include "host_eig.h"
#include "krylov.cuh"

#include <algorithm>
#include <cmath>
#include <complex>
#include <numeric>

smg_status smg_mg_apply_internal(smg_mg* mg, const smg_field* b, smg_field* x);
smg_status smg_mg_check_device_error(smg_mg* mg);
smg_status smg_mg_level0_L(const smg_mg* mg, int* L);

namespace {

constexpr int kMdotChunk = 8;    // <X_i, w> per pass over w
constexpr int kAxpyChunk = 32;   // X_i per pass of w += sum_i c_i X_i
constexpr int kMaxRitz = 8;      // n_ritz_harvest limit (slots = 3 n_ritz)

template <typename T>
struct MdotPtrs {
    const cx<T>* x[kMdotChunk];
};

// out[rhs * stride + 2 (i0 + i) + {0, 1}] = <X_i, w>, i < ns
template <typename T>
__global__ void __launch_bounds__(256) k_fgm_mdot(VecView<T> w, MdotPtrs<T> ptr, int ns, int i0, double* partials,
                                                  unsigned int* ticket, double* out, int stride) {
    constexpr int K = 2 * kMdotChunk;
    const int rhs = blockIdx.y * blockDim.x + threadIdx.x;
    T v[K];
#pragma unroll
    for (int k = 0; k < K; ++k) v[k] = T(0);
    if (rhs < w.nrhs) {
        for (int s = blockIdx.x * blockDim.y + threadIdx.y; s < w.nsites; s += gridDim.x * blockDim.y) {
            const Spinor<T> z = ld_spinor(w.p, s, rhs, w.nrhs);
#pragma unroll
            for (int i = 0; i < kMdotChunk; ++i) {
                if (i < ns) {
                    const Spinor<T> a = ld_spinor(ptr.x[i], s, rhs, w.nrhs);
                    const cx<T> c = cmulc(a.s0, z.s0) + cmulc(a.s1, z.s1);
                    v[2 * i] += c.re;
                    v[2 * i + 1] += c.im;
                }
            }
        }
    }
    struct Fin {
        double* out;
        int stride, i0, nk;
        __device__ void operator()(int rhs, const double* s) const {
            for (int k = 0; k < nk; ++k) out[rhs * stride + 2 * i0 + k] = s[k];
        }
    };
    block_reduce_finalise<K>(v, partials, ticket, w.nrhs, Fin{out, stride, i0, 2 * ns});
}

template <typename T>
struct AxpyPtrs {
    const cx<T>* x[kAxpyChunk];
};

// Coefficients of w += sum_i c_i X_i, per rhs:
//   c_i = sgn * (coef[rhs * cstride + 2 (i0 + i)], ...) * (rscale ? rscale[rhs * sstride + i0 + i] : 1)
// and 0 where mask[rhs] == 0.
struct AxpyCoef {
    const double* coef = nullptr;
    int cstride = 0;
    const double* rscale = nullptr;
    int sstride = 0;
    const int* mask = nullptr;
    double sgn = 1.0;
};

// w (+)= sum_i c_i X_i over ns <= kAxpyChunk vectors; base (w itself or
// another field) is the starting value; with NORM, ||w||^2 per rhs into norm_out
template <typename T, bool NORM>
__global__ void __launch_bounds__(256) k_fgm_axpy(VecView<T> w, const cx<T>* base, AxpyPtrs<T> ptr, int ns, int i0,
                                                  AxpyCoef cf, double* partials, unsigned int* ticket,
                                                  double* norm_out) {
    __shared__ cx<T> s_c[kAxpyChunk][32];
    const int nrhs = w.nrhs;
    const int rhs = blockIdx.y * blockDim.x + threadIdx.x;
    for (int i = threadIdx.y; i < ns; i += blockDim.y) {
        cx<T> c = mk<T>(0, 0);
        if (rhs < nrhs && (!cf.mask || cf.mask[rhs])) {
            double sc = cf.sgn * (cf.rscale ? cf.rscale[rhs * cf.sstride + i0 + i] : 1.0);
            c = mk<T>((T)(sc * cf.coef[rhs * cf.cstride + 2 * (i0 + i)]),
                      (T)(sc * cf.coef[rhs * cf.cstride + 2 * (i0 + i) + 1]));
        }
        s_c[i][threadIdx.x] = c;
    }
    __syncthreads();
    T v[1] = {T(0)};
    if (rhs < nrhs) {
        for (int s = blockIdx.x * blockDim.y + threadIdx.y; s < w.nsites; s += gridDim.x * blockDim.y) {
            Spinor<T> q = ld_spinor(base, s, rhs, nrhs);
#pragma unroll 4
            for (int i = 0; i < ns; ++i) {
                const cx<T> c = s_c[i][threadIdx.x];
                const Spinor<T> a = ld_spinor(ptr.x[i], s, rhs, nrhs);
                q.s0 = q.s0 + c * a.s0;
                q.s1 = q.s1 + c * a.s1;
            }
            st_spinor(w.p, s, rhs, nrhs, q);
            if (NORM) v[0] += norm2(q.s0) + norm2(q.s1);
        }
    }
    if (NORM) block_reduce_finalise<1>(v, partials, ticket, nrhs, FinStore{norm_out, 1});
}

// w = w * f[rhs] (real per rhs)
template <typename T>
__global__ void k_fgm_scale(VecView<T> w, const double* __restrict__ f) {
    const int rhs = blockIdx.y * blockDim.x + threadIdx.x;
    const int s = blockIdx.x * blockDim.y + threadIdx.y;
    if (rhs >= w.nrhs || s >= w.nsites) return;
    const T a = (T)f[rhs];
    Spinor<T> q = ld_spinor(w.p, s, rhs, w.nrhs);
    q.s0 = a * q.s0;
    q.s1 = a * q.s1;
    st_spinor(w.p, s, rhs, w.nrhs, q);
}

struct FgmState {
    int nrhs = 0, m = 0, max_iter = 0, restart = 0;
    double tol = 0;
    double* H = nullptr;    // [rhs][k < m][j <= m] complex, rotated
    double* Hr = nullptr;   // same, unreduced (Ritz extraction)
    double* cs = nullptr;   // [rhs][m] complex
    double* sn = nullptr;   // [rhs][m] complex
    double* g = nullptr;    // [rhs][m + 1] complex
    double* y = nullptr;    // [rhs][m] complex
    double* d1 = nullptr;   // [rhs][m + 1] complex, first Gram-Schmidt pass
    double* d2 = nullptr;   // [rhs][m + 1] complex, second pass
    double* wn2 = nullptr;  // [rhs]
    double* b2 = nullptr;   // [rhs] ||b||^2
    double* r2 = nullptr;   // [rhs] ||b - A x||^2 at the last restart
    double* f = nullptr;    // [rhs] scale of the next Arnoldi vector
    int* kk = nullptr;      // [rhs] Arnoldi steps of the current cycle
    int* total = nullptr;   // [rhs] counted steps
    int* done = nullptr;    // [rhs]
    int* conv = nullptr;    // [rhs]
    int* cyc = nullptr;     // [rhs] still in this cycle's Arnoldi process
    int* mlen = nullptr;    // [rhs] length of this cycle
    int* flags = nullptr;   // [rhs] bit 1: non-finite
    int* n_cyc = nullptr;   // scalar
};

__device__ __forceinline__ double* hcol(double* H, int m, int rhs, int k) {
    return H + (size_t)2 * ((size_t)rhs * m + k) * (m + 1);
}

// Restart: ||b - A x|| in r2; opens a cycle for every right-hand side that is
// neither converged nor out of budget (solvers.cpp:571-590)
__global__ void k_fgm_restart(FgmState s) {
    if (threadIdx.x == 0) *s.n_cyc = 0;
    __syncthreads();
    for (int j = threadIdx.x; j < s.nrhs; j += blockDim.x) {
        s.kk[j] = 0;
        s.cyc[j] = 0;
        s.f[j] = 0.0;
        if (s.done[j]) continue;
        const double bn = sqrt(s.b2[j]);
        const double be = sqrt(s.r2[j]);
        if (!isfinite(be)) {
            s.flags[j] |= 2;
            s.done[j] = 1;
            continue;
        }
        if (s.total[j] >= s.max_iter) {
            s.done[j] = 1;
            continue;
        }
        if (be / bn < s.tol) {
            s.done[j] = 1;
            s.conv[j] = 1;
            continue;
        }
        s.mlen[j] = min(s.restart, s.max_iter - s.total[j]);
        double* g = s.g + (size_t)2 * j * (s.m + 1);
        for (int i = 0; i <= s.m; ++i) g[2 * i] = g[2 * i + 1] = 0.0;
        g[0] = be;
        s.f[j] = 1.0 / be;
        s.cyc[j] = 1;
        atomicAdd(s.n_cyc, 1);
    }
}

// Arnoldi column k of every rhs still in its cycle (solvers.cpp:614-668)
__global__ void k_fgm_arnoldi(FgmState s, int k) {
    const int m = s.m;
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < s.nrhs; j += gridDim.x * blockDim.x) {
        if (!s.cyc[j]) {
            s.f[j] = 0.0;
            continue;
        }
        double* col = hcol(s.H, m, j, k);
        double* raw = hcol(s.Hr, m, j, k);
        const double* d1 = s.d1 + (size_t)2 * j * (m + 1);
        const double* d2 = s.d2 + (size_t)2 * j * (m + 1);
        for (int i = 0; i <= k; ++i) {
            col[2 * i] = d1[2 * i] + d2[2 * i];
            col[2 * i + 1] = d1[2 * i + 1] + d2[2 * i + 1];
        }
        const double hn = sqrt(s.wn2[j]);
        col[2 * (k + 1)] = hn;
        col[2 * (k + 1) + 1] = 0.0;
        for (int i = 0; i <= 2 * (k + 1) + 1; ++i) raw[i] = col[i];
        if (!isfinite(hn)) {
            s.flags[j] |= 2;
            s.done[j] = 1;
            s.cyc[j] = 0;
            s.kk[j] = 0;
            s.f[j] = 0.0;
            atomicSub(s.n_cyc, 1);
            continue;
        }
        if (hn < 1e-14) {  // happy breakdown: the column stays unrotated, the step is not counted
            s.kk[j] = k + 1;
            s.cyc[j] = 0;
            s.f[j] = 0.0;
            atomicSub(s.n_cyc, 1);
            continue;
        }
        s.f[j] = 1.0 / hn;
        double* cs = s.cs + (size_t)2 * j * m;
        double* sn = s.sn + (size_t)2 * j * m;
        for (int i = 0; i < k; ++i) {  // [[conj(c), conj(s)], [-s, c]] on (h_i, h_i+1)
            const double hr = col[2 * i], hi = col[2 * i + 1];
            const double h1r = col[2 * i + 2], h1i = col[2 * i + 3];
            const double cr = cs[2 * i], ci = cs[2 * i + 1], sr = sn[2 * i], si = sn[2 * i + 1];
            col[2 * i] = (cr * hr + ci * hi) + (sr * h1r + si * h1i);
            col[2 * i + 1] = (cr * hi - ci * hr) + (sr * h1i - si * h1r);
            col[2 * i + 2] = -(sr * hr - si * hi) + (cr * h1r - ci * h1i);
            col[2 * i + 3] = -(sr * hi + si * hr) + (cr * h1i + ci * h1r);
        }
        const double ar = col[2 * k], ai = col[2 * k + 1];
        const double br = col[2 * k + 2], bi = col[2 * k + 3];
        const double a = sqrt(ar * ar + ai * ai), b = sqrt(br * br + bi * bi);
        const double den = sqrt(a * a + b * b);
        cs[2 * k] = ar / den;
        cs[2 * k + 1] = ai / den;
        sn[2 * k] = br / den;
        sn[2 * k + 1] = bi / den;
        double* g = s.g + (size_t)2 * j * (m + 1);
        const double gr = g[2 * k], gi = g[2 * k + 1];
        const double sr = sn[2 * k], si = sn[2 * k + 1], cr = cs[2 * k], ci = cs[2 * k + 1];
        g[2 * k + 2] = -(sr * gr - si * gi);
        g[2 * k + 3] = -(sr * gi + si * gr);
        g[2 * k] = cr * gr + ci * gi;
        g[2 * k + 1] = cr * gi - ci * gr;
        col[2 * k] = den;
        col[2 * k + 1] = 0.0;
        col[2 * k + 2] = 0.0;
        col[2 * k + 3] = 0.0;
        s.total[j] += 1;
        const double gn = sqrt(g[2 * k + 2] * g[2 * k + 2] + g[2 * k + 3] * g[2 * k + 3]);
        if (gn / sqrt(s.b2[j]) < s.tol || k + 1 >= s.mlen[j]) {
            s.kk[j] = k + 1;
            s.cyc[j] = 0;
            atomicSub(s.n_cyc, 1);
        }
    }
}

// y = H^-1 g on the leading kk x kk block (solvers.cpp:673-680); the cycle's
// stop test |g_kk| / ||b|| < tol (:748)
__global__ void k_fgm_solve(FgmState s) {
    const int m = s.m;
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < s.nrhs; j += gridDim.x * blockDim.x) {
        double* y = s.y + (size_t)2 * j * m;
        for (int i = 0; i < 2 * m; ++i) y[i] = 0.0;
        const int kk = s.kk[j];
        if (kk == 0) continue;
        const double* g = s.g + (size_t)2 * j * (m + 1);
        for (int i = kk - 1; i >= 0; --i) {
            double sr = g[2 * i], si = g[2 * i + 1];
            for (int c = i + 1; c < kk; ++c) {
                const double* col = hcol(s.H, m, j, c);
                const double hr = col[2 * i], hi = col[2 * i + 1];
                sr -= hr * y[2 * c] - hi * y[2 * c + 1];
                si -= hr * y[2 * c + 1] + hi * y[2 * c];
            }
            const double* col = hcol(s.H, m, j, i);
            const double dr = col[2 * i], di = col[2 * i + 1];
            const double dd = dr * dr + di * di;
            y[2 * i] = (sr * dr + si * di) / dd;
            y[2 * i + 1] = (si * dr - sr * di) / dd;
        }
        const double gn = sqrt(g[2 * kk] * g[2 * kk] + g[2 * kk + 1] * g[2 * kk + 1]);
        if (gn / sqrt(s.b2[j]) < s.tol) {
            s.done[j] = 1;
            s.conv[j] = 1;
        }
    }
}

// Ritz vectors: out slot tgt[rhs][p] = sum_j C[rhs][p][j] Z_j, with ||.||^2 per (rhs, p)
template <typename T>
struct RitzArgs {
    const cx<T>* Z[32];
    cx<T>* slot[3 * kMaxRitz];
    const double* C;   // [rhs][nh][m] complex
    const int* tgt;    // [rhs][nh], -1: none
    int nh, m, kmax;
};

template <typename T>
__global__ void __launch_bounds__(256) k_fgm_ritz_build(VecView<T> proto, RitzArgs<T> a, double* partials,
                                                        unsigned int* ticket, double* n2) {
    const int nrhs = proto.nrhs;
    const int rhs = blockIdx.y * blockDim.x + threadIdx.x;
    T v[kMaxRitz];
#pragma unroll
    for (int p = 0; p < kMaxRitz; ++p) v[p] = T(0);
    if (rhs < nrhs) {
        for (int p = 0; p < a.nh; ++p) {
            const int t = a.tgt[rhs * a.nh + p];
            if (t < 0) continue;
            const double* C = a.C + (size_t)2 * (rhs * a.nh + p) * a.m;
            for (int s = blockIdx.x * blockDim.y + threadIdx.y; s < proto.nsites; s += gridDim.x * blockDim.y) {
                Spinor<T> q;
                q.s0 = mk<T>(0, 0);
                q.s1 = mk<T>(0, 0);
                for (int j = 0; j < a.kmax; ++j) {
                    const cx<T> c = mk<T>((T)C[2 * j], (T)C[2 * j + 1]);
                    const Spinor<T> z = ld_spinor(a.Z[j], s, rhs, nrhs);
                    q.s0 = q.s0 + c * z.s0;
                    q.s1 = q.s1 + c * z.s1;
                }
                st_spinor(a.slot[t], s, rhs, nrhs, q);
#pragma unroll
                for (int pp = 0; pp < kMaxRitz; ++pp)
                    if (pp == p) v[pp] += norm2(q.s0) + norm2(q.s1);
            }
        }
    }
    block_reduce_finalise<kMaxRitz>(v, partials, ticket, nrhs, FinStore{n2, kMaxRitz});
}

// normalise each new Ritz vector (skipped when its norm is <= 1e-14)
template <typename T>
__global__ void k_fgm_ritz_scale(VecView<T> proto, RitzArgs<T> a, const double* __restrict__ n2) {
    const int rhs = blockIdx.y * blockDim.x + threadIdx.x;
    const int s = blockIdx.x * blockDim.y + threadIdx.y;
    if (rhs >= proto.nrhs || s >= proto.nsites) return;
    for (int p = 0; p < a.nh; ++p) {
        const int t = a.tgt[rhs * a.nh + p];
        if (t < 0) continue;
        const double nv = sqrt(n2[rhs * kMaxRitz + p]);
        if (!(nv > 1e-14)) continue;
        const T f = (T)(1.0 / nv);
        Spinor<T> q = ld_spinor(a.slot[t], s, rhs, proto.nrhs);
        q.s0 = f * q.s0;
        q.s1 = f * q.s1;
        st_spinor(a.slot[t], s, rhs, proto.nrhs, q);
    }
}


struct RitzPair {
    double value;
    int slot;
};

template <typename T>
smg_status fgmres_run(smg_dirac* d, smg_mg* mg, const smg_field* b, smg_field* x, int restart, int max_iter,
                      double tol, int nh, smg_solve_result* res, double* ritz_values, int* n_ritz) {
    smg_context* ctx = d->ctx;
    const int nrhs = b->nrhs, V = b->g.V, m = restart;
    FieldSet fs;
    std::vector<smg_field*> Vf(m + 1), Zf(m), Rf(3 * nh);
    smg_field* tmp = nullptr;
    for (auto& f : Vf) SMG_TRY(fs.add(b, &f));
    for (auto& f : Zf) SMG_TRY(fs.add(b, &f));
    for (auto& f : Rf) {  // unused slots enter the deflation sums with weight 0: keep them finite
        SMG_TRY(fs.add(b, &f));
        SMG_CUDA(ctx, cudaMemsetAsync(f->data, 0, f->bytes, ctx->stream));
    }
    SMG_TRY(fs.add(b, &tmp));
    // device scalars
    const size_t nH = (size_t)2 * nrhs * m * (m + 1);
    const size_t nd = 2 * nH + (size_t)2 * nrhs * (3 * m + 3 * (m + 1)) + (size_t)4 * nrhs +
                      (size_t)nrhs * 3 * kMaxRitz * 3 + (size_t)nrhs * kMaxRitz + (size_t)2 * nrhs * kMaxRitz * m + 64;
    const size_t ni = (size_t)nrhs * (7 + kMaxRitz) + 16;
    char* blk = nullptr;
    const size_t bytes = nd * sizeof(double) + ni * sizeof(int);
    SMG_CUDA(ctx, cudaMallocAsync((void**)&blk, bytes, ctx->stream));
    SMG_CUDA(ctx, cudaMemsetAsync(blk, 0, bytes, ctx->stream));
    struct Free {
        smg_context* c;
        char* p;
        ~Free() { cudaFreeAsync(p, c->stream); }
    } free_blk{ctx, blk};
    FgmState s;
    s.nrhs = nrhs;
    s.m = m;
    s.max_iter = max_iter;
    s.restart = restart;
    s.tol = tol;
    double* p = (double*)blk;
    auto take = [&](size_t n) {
        double* q = p;
        p += n;
        return q;
    };
    s.H = take(nH);
    s.Hr = take(nH);
    s.cs = take((size_t)2 * nrhs * m);
    s.sn = take((size_t)2 * nrhs * m);
    s.y = take((size_t)2 * nrhs * m);
    s.g = take((size_t)2 * nrhs * (m + 1));
    s.d1 = take((size_t)2 * nrhs * (m + 1));
    s.d2 = take((size_t)2 * nrhs * (m + 1));
    s.wn2 = take(nrhs);
    s.b2 = take(nrhs);
    s.r2 = take(nrhs);
    s.f = take(nrhs);
    const int nslot = 3 * nh;
    double* rdots = take((size_t)2 * nrhs * 3 * kMaxRitz);  // [rhs][slot] complex
    double* rinv = take((size_t)nrhs * 3 * kMaxRitz);       // [rhs][slot]
    double* rn2 = take((size_t)nrhs * kMaxRitz);             // [rhs][p]
    double* rC = take((size_t)2 * nrhs * kMaxRitz * m);      // [rhs][p][j] complex
    int* ip = (int*)(blk + nd * sizeof(double));
    s.kk = ip;
    s.total = ip + nrhs;
    s.done = ip + 2 * nrhs;
    s.conv = ip + 3 * nrhs;
    s.cyc = ip + 4 * nrhs;
    s.mlen = ip + 5 * nrhs;
    s.flags = ip + 6 * nrhs;
    int* rtgt = ip + 7 * nrhs;  // [rhs][p]
    s.n_cyc = ip + (ni - 4);
    const ReduceLaunch rl = reduce_launch(V, nrhs);
    SMG_TRY(smg_reduce_reserve(ctx, (size_t)rl.grid.x * nrhs * 2 * std::max(kMdotChunk, kMaxRitz)));
    const dim3 vg = vec_grid(V, nrhs), vb = vec_block(nrhs);
    const dim3 mgrid(std::min(rl.grid.x, 304u), rl.grid.y);
    SMG_TRY(smg_host_stage_reserve(ctx, 64));
    int* h_ncyc = (int*)ctx->host_stage;

    auto mdot = [&](const std::vector<const cx<T>*>& xs, const smg_field* w, double* out, int stride) -> smg_status {
        for (int c0 = 0; c0 < (int)xs.size(); c0 += kMdotChunk) {
            MdotPtrs<T> mp{};
            const int ns = std::min(kMdotChunk, (int)xs.size() - c0);
            for (int i = 0; i < ns; ++i) mp.x[i] = xs[c0 + i];
            k_fgm_mdot<T><<<mgrid, rl.block, 0, ctx->stream>>>(fv<T>(w), mp, ns, c0, ctx->red.partials,
                                                               ctx->red.tickets, out, stride);
            count_launch(ctx);
            SMG_CHECK_LAUNCH(ctx);
        }
        return SMG_OK;
    };
    // w += sum_i c_i X_i in kAxpyChunk passes; norm (optional) on the last pass
    auto axpy = [&](const std::vector<const cx<T>*>& xs, smg_field* w, AxpyCoef cf, double* norm) -> smg_status {
        const int n = (int)xs.size();
        for (int c0 = 0; c0 == 0 || c0 < n; c0 += kAxpyChunk) {
            AxpyPtrs<T> ap{};
            const int ns = std::max(0, std::min(kAxpyChunk, n - c0));
            for (int i = 0; i < ns; ++i) ap.x[i] = xs[c0 + i];
            const bool last = c0 + kAxpyChunk >= n;
            if (last && norm)
                k_fgm_axpy<T, true><<<rl.grid, rl.block, 0, ctx->stream>>>(fv<T>(w), (const cx<T>*)w->data, ap, ns,
                                                                           c0, cf, ctx->red.partials,
                                                                           ctx->red.tickets, norm);
            else
                k_fgm_axpy<T, false><<<rl.grid, rl.block, 0, ctx->stream>>>(fv<T>(w), (const cx<T>*)w->data, ap,
                                                                            ns, c0, cf, nullptr, nullptr, nullptr);
            count_launch(ctx);
            SMG_CHECK_LAUNCH(ctx);
        }
        return SMG_OK;
    };
    auto scale = [&](smg_field* w) {
        k_fgm_scale<T><<<vg, vb, 0, ctx->stream>>>(fv<T>(w), s.f);
        count_launch(ctx);
    };

    // per rhs Ritz lists (host) and slot occupancy
    std::vector<std::vector<RitzPair>> ritz(nrhs);
    std::vector<std::vector<int>> free_slots(nrhs);
    for (auto& fsl : free_slots)
        for (int i = nslot - 1; i >= 0; --i) fsl.push_back(i);
    std::vector<double> h_rinv((size_t)nrhs * 3 * kMaxRitz, 0.0);
    bool any_ritz = false;

    // x = 0, r = b
    SMG_CUDA(ctx, cudaMemsetAsync(x->data, 0, x->bytes, ctx->stream));
    SMG_TRY(reduce_into<T>(ctx, fv<T>(b), nullptr, VR_NORM, s.b2));
    SMG_CUDA(ctx, cudaMemcpyAsync(s.r2, s.b2, nrhs * sizeof(double), cudaMemcpyDeviceToDevice, ctx->stream));
    SMG_CUDA(ctx, cudaMemcpyAsync(Vf[0]->data, b->data, b->bytes, cudaMemcpyDeviceToDevice, ctx->stream));
    {
        // rhs with ||b|| < 1e-30 return x = 0 at once (solvers.cpp:565)
        std::vector<double> hb(nrhs);
        SMG_CUDA(ctx, cudaMemcpyAsync(hb.data(), s.b2, nrhs * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
        SMG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        std::vector<int> hd(nrhs), hc(nrhs), hf(nrhs);
        for (int j = 0; j < nrhs; ++j) {
            hd[j] = hb[j] < 1e-60 || !std::isfinite(hb[j]);
            hc[j] = hb[j] < 1e-60;
            hf[j] = std::isfinite(hb[j]) ? 0 : 2;
        }
        SMG_CUDA(ctx, cudaMemcpyAsync(s.done, hd.data(), nrhs * sizeof(int), cudaMemcpyHostToDevice, ctx->stream));
        SMG_CUDA(ctx, cudaMemcpyAsync(s.conv, hc.data(), nrhs * sizeof(int), cudaMemcpyHostToDevice, ctx->stream));
        SMG_CUDA(ctx, cudaMemcpyAsync(s.flags, hf.data(), nrhs * sizeof(int), cudaMemcpyHostToDevice, ctx->stream));
    }
    k_fgm_restart<<<1, 256, 0, ctx->stream>>>(s);
    count_launch(ctx);
    const int sb = std::min(256, ((nrhs + 31) / 32) * 32), sgrid = (nrhs + sb - 1) / sb;
    for (;;) {
        SMG_CUDA(ctx, cudaMemcpyAsync(h_ncyc, s.n_cyc, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
        SMG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        if (*h_ncyc == 0) break;
        scale(Vf[0]);  // V_0 = r / beta
        int kcols = 0;
        for (int k = 0; k < m; ++k) {
            // Z_k = M^-1 V_k
            if (mg)
                SMG_TRY(smg_mg_apply_internal(mg, Vf[k], Zf[k]));
            else
                SMG_CUDA(ctx, cudaMemcpyAsync(Zf[k]->data, Vf[k]->data, Vf[k]->bytes, cudaMemcpyDeviceToDevice,
                                              ctx->stream));
            if (any_ritz) {  // Z_k += sum_p <v_p, V_k> / theta_p v_p (solvers.cpp:606-612)
                std::vector<const cx<T>*> rs(nslot);
                for (int i = 0; i < nslot; ++i) rs[i] = (const cx<T>*)Rf[i]->data;
                SMG_TRY(mdot(rs, Vf[k], rdots, 2 * 3 * kMaxRitz));
                AxpyCoef cf;
                cf.coef = rdots;
                cf.cstride = 2 * 3 * kMaxRitz;
                cf.rscale = rinv;
                cf.sstride = 3 * kMaxRitz;
                cf.mask = s.cyc;
                SMG_TRY(axpy(rs, Zf[k], cf, nullptr));
            }
            // W = A Z_k in the V_{k+1} buffer, two Gram-Schmidt passes against V_0..V_k
            SMG_TRY(apply_A<T>(d, Zf[k], tmp, Vf[k + 1]));
            std::vector<const cx<T>*> vs(k + 1);
            for (int i = 0; i <= k; ++i) vs[i] = (const cx<T>*)Vf[i]->data;
            AxpyCoef cf;
            cf.cstride = 2 * (m + 1);
            cf.mask = s.cyc;
            cf.sgn = -1.0;
            SMG_TRY(mdot(vs, Vf[k + 1], s.d1, 2 * (m + 1)));
            cf.coef = s.d1;
            SMG_TRY(axpy(vs, Vf[k + 1], cf, nullptr));
            SMG_TRY(mdot(vs, Vf[k + 1], s.d2, 2 * (m + 1)));
            cf.coef = s.d2;
            SMG_TRY(axpy(vs, Vf[k + 1], cf, s.wn2));
            k_fgm_arnoldi<<<sgrid, sb, 0, ctx->stream>>>(s, k);
            count_launch(ctx);
            scale(Vf[k + 1]);
            SMG_CHECK_LAUNCH(ctx);
            kcols = k + 1;
            SMG_CUDA(ctx, cudaMemcpyAsync(h_ncyc, s.n_cyc, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
            SMG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
            if (*h_ncyc == 0) break;
        }
        // y = H^-1 g, x += Z y
        k_fgm_solve<<<sgrid, sb, 0, ctx->stream>>>(s);
        count_launch(ctx);
        {
            std::vector<const cx<T>*> zs(kcols);
            for (int i = 0; i < kcols; ++i) zs[i] = (const cx<T>*)Zf[i]->data;
            AxpyCoef cf;
            cf.coef = s.y;
            cf.cstride = 2 * m;
            SMG_TRY(axpy(zs, x, cf, nullptr));
        }
        // Ritz harvest (solvers.cpp:699-746)
        if (nh > 0) {
            std::vector<int> hkk(nrhs);
            std::vector<double> hH(nH);
            SMG_CUDA(ctx, cudaMemcpyAsync(hkk.data(), s.kk, nrhs * sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
            SMG_CUDA(ctx, cudaMemcpyAsync(hH.data(), s.Hr, nH * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
            SMG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
            std::vector<double> hC((size_t)2 * nrhs * kMaxRitz * m, 0.0);
            std::vector<int> htgt((size_t)nrhs * nh, -1);
            bool any_new = false;
            for (int j = 0; j < nrhs; ++j) {
                const int kk = hkk[j];
                if (kk < nh) continue;
                using C = std::complex<double>;
                auto Hraw = [&](int row, int col) {
                    const double* c = hH.data() + (size_t)2 * ((size_t)j * m + col) * (m + 1);
                    return C(c[2 * row], c[2 * row + 1]);
                };
                std::vector<C> G((size_t)kk * kk, C(0, 0));  // G(i, c) = sum_p conj(H(p, i)) H(p, c)
                for (int c = 0; c < kk; ++c)
                    for (int i = 0; i < kk; ++i) {
                        C acc(0, 0);
                        for (int pr = 0; pr <= kk; ++pr) acc += std::conj(Hraw(pr, i)) * Hraw(pr, c);
                        G[(size_t)c * kk + i] = acc;
                    }
                for (int i = 0; i < kk; ++i)
                    for (int c = i + 1; c < kk; ++c) {
                        C avg = 0.5 * (G[(size_t)c * kk + i] + std::conj(G[(size_t)i * kk + c]));
                        G[(size_t)c * kk + i] = avg;
                        G[(size_t)i * kk + c] = std::conj(avg);
                    }
                std::vector<double> ev;
                std::vector<C> evec;
                hermitian_eig(kk, G, ev, evec);
                for (int pp = 0; pp < nh; ++pp) {
                    const int slot = free_slots[j].back();
                    free_slots[j].pop_back();
                    htgt[(size_t)j * nh + pp] = slot;
                    ritz[j].push_back({ev[pp], slot});
                    double* Cp = hC.data() + (size_t)2 * ((size_t)j * nh + pp) * m;
                    for (int i = 0; i < kk; ++i) {
                        Cp[2 * i] = evec[(size_t)pp * kk + i].real();
                        Cp[2 * i + 1] = evec[(size_t)pp * kk + i].imag();
                    }
                }
                any_new = true;
            }
            if (any_new) {
                SMG_CUDA(ctx, cudaMemcpyAsync(rC, hC.data(), (size_t)2 * nrhs * nh * m * sizeof(double),
                                              cudaMemcpyHostToDevice, ctx->stream));
                SMG_CUDA(ctx, cudaMemcpyAsync(rtgt, htgt.data(), htgt.size() * sizeof(int), cudaMemcpyHostToDevice,
                                              ctx->stream));
                RitzArgs<T> ra{};
                for (int i = 0; i < kcols; ++i) ra.Z[i] = (const cx<T>*)Zf[i]->data;
                for (int i = 0; i < nslot; ++i) ra.slot[i] = (cx<T>*)Rf[i]->data;
                ra.C = rC;
                ra.tgt = rtgt;
                ra.nh = nh;
                ra.m = m;
                ra.kmax = kcols;
                k_fgm_ritz_build<T><<<rl.grid, rl.block, 0, ctx->stream>>>(fv<T>(b), ra, ctx->red.partials,
                                                                            ctx->red.tickets, rn2);
                k_fgm_ritz_scale<T><<<vg, vb, 0, ctx->stream>>>(fv<T>(b), ra, rn2);
                count_launch(ctx, 2);
                SMG_CHECK_LAUNCH(ctx);
                // keep the list bounded: beyond 2 n_ritz, the n_ritz smallest stay
                for (int j = 0; j < nrhs; ++j) {
                    auto& lst = ritz[j];
                    if ((int)lst.size() > 2 * nh) {
                        std::sort(lst.begin(), lst.end(),
                                  [](const RitzPair& u, const RitzPair& v) { return u.value < v.value; });
                        for (size_t i = nh; i < lst.size(); ++i) free_slots[j].push_back(lst[i].slot);
                        lst.resize(nh);
                    }
                    for (int i = 0; i < 3 * kMaxRitz; ++i) h_rinv[(size_t)j * 3 * kMaxRitz + i] = 0.0;
                    for (const auto& rp : lst)
                        if (rp.value > 1e-14) h_rinv[(size_t)j * 3 * kMaxRitz + rp.slot] = 1.0 / rp.value;
                }
                SMG_CUDA(ctx, cudaMemcpyAsync(rinv, h_rinv.data(), h_rinv.size() * sizeof(double),
                                              cudaMemcpyHostToDevice, ctx->stream));
                any_ritz = true;
            }
        }
        // restart: V_0 = b - A x, ||V_0||^2
        SMG_TRY(apply_A<T>(d, x, tmp, Vf[1]));
        {
            k_residual<T><<<(unsigned)((b->n_complex() + 255) / 256), 256, 0, ctx->stream>>>(
                (const cx<T>*)b->data, (const cx<T>*)Vf[1]->data, (cx<T>*)Vf[0]->data, b->n_complex());
            count_launch(ctx);
            SMG_TRY(reduce_into<T>(ctx, fv<T>(Vf[0]), nullptr, VR_NORM, s.r2));
        }
        k_fgm_restart<<<1, 256, 0, ctx->stream>>>(s);
        count_launch(ctx);
        SMG_CHECK_LAUNCH(ctx);
    }
    // results: the last restart holds ||b - A x||^2 of the final x for every rhs
    std::vector<double> hb(nrhs), hr(nrhs);
    std::vector<int> ht(nrhs), hcv(nrhs), hfl(nrhs);
    SMG_CUDA(ctx, cudaMemcpyAsync(hb.data(), s.b2, nrhs * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    SMG_CUDA(ctx, cudaMemcpyAsync(hr.data(), s.r2, nrhs * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    SMG_CUDA(ctx, cudaMemcpyAsync(ht.data(), s.total, nrhs * sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    SMG_CUDA(ctx, cudaMemcpyAsync(hfl.data(), s.flags, nrhs * sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    SMG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    int worst_it = 0;
    double worst = 0;
    bool nonfinite = false, notconv = false;
    for (int j = 0; j < nrhs; ++j) {
        worst_it = std::max(worst_it, ht[j]);
        if (hfl[j] & 2) nonfinite = true;
        if (hb[j] >= 1e-60 && std::isfinite(hb[j])) {
            const double rel = std::sqrt(hr[j] / hb[j]);
            worst = std::max(worst, rel);
            if (!(rel <= tol) && ht[j] >= max_iter) notconv = true;  // solvers.cpp:762-767
        }
        if (n_ritz) n_ritz[j] = (int)ritz[j].size();
        if (ritz_values)
            for (size_t i = 0; i < ritz[j].size(); ++i) ritz_values[(size_t)j * 3 * nh + i] = ritz[j][i].value;
    }
    if (res) {
        res->iterations = worst_it;
        res->final_residual = worst;
        res->true_residual = worst;
        res->operator_applications = worst_it;
    }
    if (mg) SMG_TRY(smg_mg_check_device_error(mg));
    if (nonfinite) return smg_fail(ctx, SMG_NONFINITE, "fgmres_solve: non-finite residual");
    if (notconv) return smg_fail(ctx, SMG_NOT_CONVERGED, "fgmres_solve: iteration limit reached");
    return SMG_OK;
}

}  // namespace

extern "C" {

SMG_API smg_status smg_fgmres_solve(smg_dirac* d, smg_mg* mg, const smg_field* rhs, smg_field* x, int restart,
                                    int max_iter, double tol, int n_ritz_harvest, smg_solve_result* res,
                                    double* ritz_values, int* n_ritz) {
    if (!d || !rhs || !x) return SMG_BAD_ARG;
    smg_context* ctx = d->ctx;
    if (rhs == x) return smg_fail(ctx, SMG_BAD_ARG, "rhs and x must be distinct");
    SMG_TRY(smg_field_check_pair(rhs, x));
    if (rhs->g.L != d->gauge->g.L) return smg_fail(ctx, SMG_BAD_ARG, "field L differs from gauge L");
    if (restart < 1 || restart > 32 || max_iter < 0 || !(tol > 0) || n_ritz_harvest < 0 ||
        n_ritz_harvest > kMaxRitz)
        return smg_fail(ctx, SMG_BAD_ARG, "fgmres_solve: 1 <= restart <= 32, 0 <= n_ritz_harvest <= 8, tol > 0");
    if (mg) {
        int L = 0;
        SMG_TRY(smg_mg_level0_L(mg, &L));
        if (L != rhs->g.L) return smg_fail(ctx, SMG_BAD_ARG, "field L differs from the hierarchy's");
    }
    if (rhs->prec == SMG_F64)
        return fgmres_run<double>(d, mg, rhs, x, restart, max_iter, tol, n_ritz_harvest, res, ritz_values, n_ritz);
    if (rhs->prec == SMG_F32)
        return fgmres_run<float>(d, mg, rhs, x, restart, max_iter, tol, n_ritz_harvest, res, ritz_values, n_ritz);
    return smg_fail(ctx, SMG_UNSUPPORTED, "fgmres_solve on F16 fields");
}

}  // extern "C"
