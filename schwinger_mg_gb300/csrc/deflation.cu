// Coarse-grid deflation on the device (reference src/coarse_op.h:168-200, 492-547,
// src/coarse_op.cpp:10-54, src/eigensolver_core.cpp:691-1057, src/eigen_evolve.cpp:48-105,
// src/hmc.h:307-324).
//
// The deflation space is the n lowest eigenpairs of the level-1 operator
// A_c = P^dag (D^dag D) P (or, on request, of a deeper coarse level's
// operator).  They are found by thick-restart Lanczos
// (Wu & Simon, SIAM J. Matrix Anal. Appl. 22 (2000) 602), the method of the
// reference's trlm_eigensolver without Chebyshev acceleration, with the same
// schedule: Krylov space n_kr, restart keeping
// min(n_conv + (n_kr - n_conv) / 2, n_kr - n_locked - 12) Ritz vectors, locking at
// 1e-15 and convergence at tol relative to the Ritz value, the start vector
// random_vec(dim, std::mt19937(42)).  Each Lanczos step is one FP64 coarse
// apply and two classical Gram-Schmidt passes against the whole Krylov basis
// (one multi-dot kernel and one multi-axpy kernel per pass); the small arrow /
// tridiagonal eigenproblem is solved on the host.
//
// The space is used three ways: the deflated initial guess of the coarsest CG
// (SparseCoarseOp::solve), the low-mode solution P (sum_i v_i v_i^dag / lambda_i) P^dag phi
// of the multi-timescale HMC (CoarseDeflState::lowmode_solution), and the
// Rayleigh-Ritz update after the coarse operator was rebuilt for new links
// (rr_evolve via evolve_coarse_deflation, src/hmc_multiscale.cpp:278-331).
#include <algorithm>
#include <cmath>
#include <complex>
#include <random>
#include <vector>

#include "host_eig.h"
#include "mg_internal.h"

namespace {

constexpr int kDotChunk = 8;   // Krylov vectors per multi-dot block
constexpr int kMaxGrid = 296;  // blocks of the reductions (two per SM)

// part[(chunk * 2 * kDotChunk + 2 kk + c) * G + g] = partial of <K_{chunk*8+kk}, r> (c = re, im)
__global__ void __launch_bounds__(256) k_mdot(const cx<double>* __restrict__ K, int64_t ld, int m,
                                              const cx<double>* __restrict__ r, int64_t n, double* __restrict__ part) {
    const int k0 = blockIdx.y * kDotChunk;
    double acc[2 * kDotChunk];
#pragma unroll
    for (int j = 0; j < 2 * kDotChunk; ++j) acc[j] = 0.0;
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x) {
        const cx<double> re = r[e];
#pragma unroll
        for (int kk = 0; kk < kDotChunk; ++kk) {
            if (k0 + kk < m) {
                const cx<double> v = K[(int64_t)(k0 + kk) * ld + e];
                acc[2 * kk] += v.re * re.re + v.im * re.im;
                acc[2 * kk + 1] += v.re * re.im - v.im * re.re;
            }
        }
    }
    __shared__ double sh[8][2 * kDotChunk];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int j = 0; j < 2 * kDotChunk; ++j) {
        double v = acc[j];
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if (lane == 0) sh[warp][j] = v;
    }
    __syncthreads();
    if (threadIdx.x < 2 * kDotChunk) {
        double v = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) v += sh[w][threadIdx.x];
        part[((int64_t)blockIdx.y * 2 * kDotChunk + threadIdx.x) * gridDim.x + blockIdx.x] = v;
    }
}

// out[k] = the sum of the per-block partials of <K_k, r> (fixed order)
__global__ void k_mdot_finish(const double* __restrict__ part, int G, int m, cx<double>* __restrict__ out) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= 2 * m) return;
    const int k = t >> 1, c = t & 1;
    const int row = (k / kDotChunk) * 2 * kDotChunk + 2 * (k % kDotChunk) + c;
    double v = 0.0;
    for (int g = 0; g < G; ++g) v += part[(int64_t)row * G + g];
    if (c == 0)
        out[k].re = v;
    else
        out[k].im = v;
}

// r -= sum_{k < m} c_k K_k
__global__ void __launch_bounds__(256) k_maxpy(const cx<double>* __restrict__ K, int64_t ld, int m,
                                               const cx<double>* __restrict__ c, cx<double>* __restrict__ r,
                                               int64_t n) {
    __shared__ cx<double> sc[128];
    for (int k = threadIdx.x; k < m; k += blockDim.x) sc[k] = c[k];
    __syncthreads();
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x) {
        cx<double> v = r[e];
        for (int k = 0; k < m; ++k) v = v - sc[k] * K[(int64_t)k * ld + e];
        r[e] = v;
    }
}

// beta = sqrt(nrm2.re); next = r / beta unless beta <= 1e-14 (then next is left as it was)
__global__ void __launch_bounds__(256) k_lanczos_next(const cx<double>* __restrict__ r,
                                                      const cx<double>* __restrict__ nrm2, cx<double>* __restrict__ next,
                                                      double* __restrict__ beta_out, int64_t n) {
    const double beta = sqrt(fmax(nrm2->re, 0.0));
    if (blockIdx.x == 0 && threadIdx.x == 0) *beta_out = beta;
    if (!(beta > 1e-14)) return;
    const double inv = 1.0 / beta;
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x)
        next[e] = inv * r[e];
}

// out_i = sum_{j < dim} Y(j, i) K_j for i < keep; Y column-major [i * dim + j]
__global__ void __launch_bounds__(256) k_rotate(const cx<double>* __restrict__ K, int64_t ld, int dim,
                                                const cx<double>* __restrict__ Y, int keep,
                                                cx<double>* __restrict__ out, int64_t n) {
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x) {
        for (int i = 0; i < keep; ++i) {
            cx<double> v = mk(0.0, 0.0);
            for (int j = 0; j < dim; ++j) v = v + Y[(int64_t)i * dim + j] * K[(int64_t)j * ld + e];
            out[(int64_t)i * ld + e] = v;
        }
    }
}

__global__ void k_to_f32(const cx<double>* __restrict__ a, cx<float>* __restrict__ b, int64_t n) {
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e < n) b[e] = mk((float)a[e].re, (float)a[e].im);
}

// ---- deflated initial guess for coarse vectors of nrhs right-hand sides ([site][dof][rhs])
// block (lanes, 256 / lanes): lane = rhs, rows stride over the entries e = site * ndof + dof
template <typename T>
__global__ void __launch_bounds__(256) k_defl_part(const cx<T>* __restrict__ V, int64_t dim, VecView<T> b,
                                                   double* __restrict__ part) {
    const int i = blockIdx.y, rhs = threadIdx.x, nrhs = b.nrhs;
    double re = 0.0, im = 0.0;
    if (rhs < nrhs) {
        const cx<T>* v = V + (int64_t)i * dim;
        for (int64_t e = (int64_t)blockIdx.x * blockDim.y + threadIdx.y; e < dim; e += (int64_t)gridDim.x * blockDim.y) {
            const cx<T> a = v[e], c = b.p[e * nrhs + rhs];
            re += (double)a.re * c.re + (double)a.im * c.im;
            im += (double)a.re * c.im - (double)a.im * c.re;
        }
    }
    __shared__ double sh[2][256];
    const int t = threadIdx.y * blockDim.x + threadIdx.x;
    sh[0][t] = re;
    sh[1][t] = im;
    __syncthreads();
    for (int s = blockDim.y >> 1; s > 0; s >>= 1) {
        if (threadIdx.y < s) {
            sh[0][t] += sh[0][t + s * blockDim.x];
            sh[1][t] += sh[1][t + s * blockDim.x];
        }
        __syncthreads();
    }
    if (threadIdx.y == 0 && rhs < nrhs) {
        const int64_t row = ((int64_t)i * nrhs + rhs) * 2;
        part[row * gridDim.x + blockIdx.x] = sh[0][t];
        part[(row + 1) * gridDim.x + blockIdx.x] = sh[1][t];
    }
}

// coef[i][rhs] = (sum of the partials) / lambda_i  (0 where lambda_i <= 1e-14)
__global__ void k_defl_coef(const double* __restrict__ part, int G, int nvec, int nrhs,
                            const double* __restrict__ inv, cx<double>* __restrict__ coef) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nvec * nrhs) return;
    const int i = t / nrhs;
    double re = 0.0, im = 0.0;
    for (int g = 0; g < G; ++g) {
        re += part[((int64_t)t * 2) * G + g];
        im += part[((int64_t)t * 2 + 1) * G + g];
    }
    coef[t] = mk(re * inv[i], im * inv[i]);
}

// x[e][rhs] = sum_i coef[i][rhs] v_i[e]
template <typename T>
__global__ void __launch_bounds__(256) k_defl_combine(const cx<T>* __restrict__ V, int64_t dim, int nvec,
                                                      const cx<double>* __restrict__ coef, VecView<T> x) {
    const int nrhs = x.nrhs;
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= dim * nrhs) return;
    const int64_t e = t / nrhs;
    const int rhs = (int)(t - e * nrhs);
    double re = 0.0, im = 0.0;
    for (int i = 0; i < nvec; ++i) {
        const cx<T> v = V[(int64_t)i * dim + e];
        const cx<double> c = coef[i * nrhs + rhs];
        re += c.re * v.re - c.im * v.im;
        im += c.re * v.im + c.im * v.re;
    }
    x.p[t] = mk((T)re, (T)im);
}

__global__ void k_fill_inv(const double* __restrict__ vals, double* __restrict__ inv, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) inv[i] = vals[i] > 1e-14 ? 1.0 / vals[i] : 0.0;
}

int grid_for(int64_t n, int cap = kMaxGrid) { return (int)std::max<int64_t>(1, std::min<int64_t>(cap, (n + 255) / 256)); }

// Dense helpers on device vector sets: K is [m][ld] complex doubles
struct Workspace {
    smg_context* ctx = nullptr;
    std::vector<void*> bufs;
    ~Workspace() {
        if (ctx) cudaStreamSynchronize(ctx->stream);
        for (void* p : bufs) cudaFree(p);
    }
    template <typename P>
    smg_status alloc(P** out, size_t count) {
        void* p = nullptr;
        if (cudaMalloc(&p, count * sizeof(P)) != cudaSuccess) return smg_fail(ctx, SMG_NO_MEMORY, "deflation workspace");
        bufs.push_back(p);
        *out = (P*)p;
        return SMG_OK;
    }
};

// c[0..m) = K[0..m)^dag r
smg_status multi_dot(smg_context* ctx, const cx<double>* K, int64_t ld, int m, const cx<double>* r, int64_t n,
                     double* part, cx<double>* c) {
    const int G = grid_for(n);
    const dim3 grid(G, (m + kDotChunk - 1) / kDotChunk);
    k_mdot<<<grid, 256, 0, ctx->stream>>>(K, ld, m, r, n, part);
    k_mdot_finish<<<(2 * m + 127) / 128, 128, 0, ctx->stream>>>(part, G, m, c);
    count_launch(ctx, 2);
    SMG_CHECK_LAUNCH(ctx);
    return SMG_OK;
}

size_t part_doubles(int m) { return (size_t)((m + kDotChunk - 1) / kDotChunk) * 2 * kDotChunk * kMaxGrid; }

smg_status ensure_storage(smg_context* ctx, MgDeflation& d, int cap, int64_t dim) {
    if (d.cap >= cap && d.dim == dim) return SMG_OK;
    cudaStreamSynchronize(ctx->stream);
    smg_defl_free(d);
    d.dim = dim;
    d.cap = cap;
    SMG_CUDA(ctx, cudaMalloc(&d.V64, (size_t)cap * dim * sizeof(cx<double>)));
    SMG_CUDA(ctx, cudaMalloc(&d.V32, (size_t)cap * dim * sizeof(cx<float>)));
    SMG_CUDA(ctx, cudaMalloc(&d.inv, (size_t)cap * sizeof(double)));
    SMG_CUDA(ctx, cudaMalloc(&d.coef, (size_t)cap * 32 * sizeof(cx<double>)));
    SMG_CUDA(ctx, cudaMalloc(&d.c_in, (size_t)dim * sizeof(cx<double>)));
    SMG_CUDA(ctx, cudaMalloc(&d.c_out, (size_t)dim * sizeof(cx<double>)));
    d.part_doubles = (size_t)cap * 32 * 2 * kMaxGrid;
    SMG_CUDA(ctx, cudaMalloc(&d.part, d.part_doubles * sizeof(double)));
    return SMG_OK;
}

// the FP32 copy and 1/lambda after the vectors or values changed
smg_status commit(smg_context* ctx, MgDeflation& d) {
    const int64_t n = (int64_t)d.n * d.dim;
    if (n > 0) {
        k_to_f32<<<(unsigned)((n + 255) / 256), 256, 0, ctx->stream>>>(d.V64, d.V32, n);
        count_launch(ctx);
    }
    double* vals = nullptr;
    SMG_CUDA(ctx, cudaMallocAsync(&vals, std::max<size_t>(1, d.vals.size()) * sizeof(double), ctx->stream));
    if (d.n > 0) {
        SMG_CUDA(ctx, cudaMemcpyAsync(vals, d.vals.data(), (size_t)d.n * sizeof(double), cudaMemcpyHostToDevice,
                                      ctx->stream));
        k_fill_inv<<<1, 128, 0, ctx->stream>>>(vals, d.inv, d.n);
        count_launch(ctx);
    }
    SMG_CUDA(ctx, cudaFreeAsync(vals, ctx->stream));
    SMG_CHECK_LAUNCH(ctx);
    SMG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return SMG_OK;
}

// trlm_eigensolver (src/eigensolver_core.cpp:691-1057, poly_deg = 0) on A_1 of the hierarchy
smg_status trlm(smg_mg* mg, int level, int n_ev, int n_kr, int max_restarts, double tol, cx<double>* vecs_out,
                std::vector<double>& vals_out, smg_deflation_info* info) {
    smg_context* ctx = smg_mg_ctx(mg);
    const int64_t n = smg_mg_level_dim(mg, level);
    Workspace ws;
    ws.ctx = ctx;
    cx<double>* K = nullptr;  // n_kr + 1 Krylov vectors
    cx<double>* r = nullptr;
    cx<double>* rot = nullptr;
    cx<double>* c = nullptr;
    cx<double>* Y = nullptr;
    double* ab = nullptr;  // device alpha[n_kr], beta[n_kr]
    double* part = nullptr;
    SMG_TRY(ws.alloc(&K, (size_t)(n_kr + 1) * n));
    SMG_TRY(ws.alloc(&r, (size_t)n));
    SMG_TRY(ws.alloc(&rot, (size_t)n_kr * n));
    SMG_TRY(ws.alloc(&c, (size_t)n_kr + 1));
    SMG_TRY(ws.alloc(&Y, (size_t)n_kr * n_kr));
    SMG_TRY(ws.alloc(&ab, (size_t)2 * n_kr));
    SMG_TRY(ws.alloc(&part, part_doubles(n_kr + 1)));
    SMG_CUDA(ctx, cudaMemsetAsync(K, 0, (size_t)(n_kr + 1) * n * sizeof(cx<double>), ctx->stream));
    {
        // kSpace[0] = random_vec(n, mt19937(42)) / norm (src/eigensolver_core.cpp:726-733); random_vec
        // draws each entry's imaginary part first
        std::mt19937 rng(42);
        std::normal_distribution<double> dist(0.0, 1.0);
        std::vector<cx<double>> h((size_t)n);
        double nrm = 0;
        for (auto& z : h) {
            const double im = dist(rng);
            const double re = dist(rng);
            z = mk(re, im);
            nrm += re * re + im * im;
        }
        const double inv = 1.0 / std::sqrt(nrm);
        for (auto& z : h) z = mk(z.re * inv, z.im * inv);
        SMG_CUDA(ctx, cudaMemcpyAsync(K, h.data(), (size_t)n * sizeof(cx<double>), cudaMemcpyHostToDevice,
                                      ctx->stream));
        SMG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    }
    std::vector<double> alpha(n_kr, 0.0), beta(n_kr, 0.0), residua(n_kr, 0.0);
    int num_locked = 0, num_converged = 0, num_keep = 0, iter = 0, restart = 0;
    bool converged = false;
    const int G = grid_for(n);
    for (restart = 0; restart < max_restarts && !converged; ++restart) {
        // Krylov extension from num_keep to n_kr (lanczosStep, src/eigensolver_core.cpp:816-851)
        for (int j = num_keep; j < n_kr; ++j) {
            cx<double>* vj = K + (int64_t)j * n;
            SMG_TRY(smg_mg_apply_f64(mg, level, vj, r));
            for (int pass = 0; pass < 2; ++pass) {
                SMG_TRY(multi_dot(ctx, K, n, j + 1, r, n, part, c));
                // alpha_j = Re <v_j, A v_j> before any orthogonalisation
                if (pass == 0)
                    SMG_CUDA(ctx, cudaMemcpyAsync(ab + j, (const double*)(c + j), sizeof(double),
                                                  cudaMemcpyDeviceToDevice, ctx->stream));
                k_maxpy<<<G, 256, 0, ctx->stream>>>(K, n, j + 1, c, r, n);
                count_launch(ctx);
            }
            SMG_TRY(multi_dot(ctx, r, n, 1, r, n, part, c + n_kr));
            k_lanczos_next<<<G, 256, 0, ctx->stream>>>(r, c + n_kr, K + (int64_t)(j + 1) * n, ab + n_kr + j, n);
            count_launch(ctx);
            SMG_CHECK_LAUNCH(ctx);
        }
        iter += n_kr - num_keep;
        if (num_keep < n_kr) {
            std::vector<double> h(2 * (size_t)n_kr);
            SMG_CUDA(ctx, cudaMemcpyAsync(h.data(), ab, h.size() * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
            SMG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
            for (int j = num_keep; j < n_kr; ++j) {
                alpha[j] = h[j];
                beta[j] = h[n_kr + j];
                if (!std::isfinite(alpha[j]) || !std::isfinite(beta[j]))
                    return smg_fail(ctx, SMG_NONFINITE, "deflation: Lanczos produced a non-finite coefficient");
            }
        }
        // arrow matrix (src/eigensolver_core.cpp:864-886)
        const int dim = n_kr - num_locked;
        const int arrow_pos = num_keep - num_locked;
        std::vector<std::complex<double>> A((size_t)dim * dim, 0.0);
        auto at = [&](int i, int j) -> std::complex<double>& { return A[(size_t)j * dim + i]; };
        for (int i = 0; i < dim; ++i) at(i, i) = alpha[i + num_locked];
        for (int i = 0; i < arrow_pos; ++i) {
            at(arrow_pos, i) = beta[i + num_locked];
            at(i, arrow_pos) = beta[i + num_locked];
        }
        for (int i = arrow_pos; i < dim - 1; ++i) {
            at(i + 1, i) = beta[i + num_locked];
            at(i, i + 1) = beta[i + num_locked];
        }
        std::vector<double> ev;
        std::vector<std::complex<double>> evec;  // evec[col * dim + row]
        hermitian_eig(dim, A, ev, evec);
        const double bl = beta[n_kr - 1];
        for (int i = 0; i < dim; ++i) {
            residua[i + num_locked] = std::abs(bl * evec[(size_t)i * dim + dim - 1].real());
            alpha[i + num_locked] = ev[i];
        }
        // locking and convergence (src/eigensolver_core.cpp:910-935)
        int iter_locked = 0, iter_converged = 0;
        for (int i = 1; i < dim; ++i) {
            if (residua[i + num_locked] < 1e-15 * std::abs(alpha[i + num_locked]))
                iter_locked = i;
            else
                break;
        }
        iter_converged = iter_locked;
        for (int i = iter_locked + 1; i < dim; ++i) {
            if (residua[i + num_locked] < tol * std::abs(alpha[i + num_locked]))
                iter_converged = i;
            else
                break;
        }
        int iter_keep = std::min(iter_converged + (n_kr - num_converged) / 2, n_kr - num_locked - 12);
        if (iter_keep < 1) iter_keep = 1;
        if (iter_keep > dim - 1) iter_keep = dim - 1;
        // thick restart: the leading Ritz vectors, then the last Lanczos vector (:941-962)
        {
            std::vector<cx<double>> yh((size_t)iter_keep * dim);
            for (int i = 0; i < iter_keep; ++i)
                for (int j = 0; j < dim; ++j) {
                    const std::complex<double> z = evec[(size_t)i * dim + j];
                    yh[(size_t)i * dim + j] = mk(z.real(), z.imag());
                }
            SMG_CUDA(ctx, cudaMemcpyAsync(Y, yh.data(), yh.size() * sizeof(cx<double>), cudaMemcpyHostToDevice,
                                          ctx->stream));
            k_rotate<<<G, 256, 0, ctx->stream>>>(K + (int64_t)num_locked * n, n, dim, Y, iter_keep, rot, n);
            count_launch(ctx);
            SMG_CHECK_LAUNCH(ctx);
            SMG_CUDA(ctx, cudaMemcpyAsync(K + (int64_t)num_locked * n, rot, (size_t)iter_keep * n * sizeof(cx<double>),
                                          cudaMemcpyDeviceToDevice, ctx->stream));
            if (num_locked + iter_keep != n_kr)
                SMG_CUDA(ctx, cudaMemcpyAsync(K + (int64_t)(num_locked + iter_keep) * n, K + (int64_t)n_kr * n,
                                              (size_t)n * sizeof(cx<double>), cudaMemcpyDeviceToDevice, ctx->stream));
            for (int i = 0; i < iter_keep; ++i) beta[i + num_locked] = bl * evec[(size_t)i * dim + dim - 1].real();
            SMG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        }
        num_converged = num_locked + iter_converged;
        num_keep = num_locked + iter_keep;
        num_locked += iter_locked;
        if (num_converged >= n_ev) converged = true;
    }
    // ascending order (the insertion sort of :981-989), the first n_ev pairs
    std::vector<int> perm(n_kr);
    for (int i = 0; i < n_kr; ++i) perm[i] = i;
    std::vector<double> a = alpha;
    if (converged) {
        for (int i = 1; i < n_kr; ++i) {
            int j = i;
            while (j > 0 && a[j - 1] > a[j]) {
                std::swap(a[j], a[j - 1]);
                std::swap(perm[j], perm[j - 1]);
                --j;
            }
        }
    }
    vals_out.assign(a.begin(), a.begin() + n_ev);
    for (int i = 0; i < n_ev; ++i)
        SMG_CUDA(ctx, cudaMemcpyAsync(vecs_out + (int64_t)i * n, K + (int64_t)perm[i] * n, (size_t)n * sizeof(cx<double>),
                                      cudaMemcpyDeviceToDevice, ctx->stream));
    SMG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if (info) {
        info->converged = converged ? 1 : 0;
        info->restarts = restart;
        info->iterations = iter;
        info->n_kr = n_kr;
    }
    return SMG_OK;
}

}  // namespace

void smg_defl_free(MgDeflation& d) {
    for (void* p : {(void*)d.V64, (void*)d.V32, (void*)d.inv, (void*)d.part, (void*)d.coef, (void*)d.c_in,
                    (void*)d.c_out})
        if (p) cudaFree(p);
    d = MgDeflation{};
}

template <typename T>
smg_status smg_defl_guess(smg_context* ctx, MgDeflation& d, VecView<T> b, VecView<T> x) {
    const int nrhs = b.nrhs;
    if (nrhs > 32 || (nrhs > 1 && !b.rhs_inner)) return smg_fail(ctx, SMG_UNSUPPORTED, "deflated guess: layout");
    int lanes = 1;
    while (lanes < nrhs) lanes *= 2;
    const dim3 block(lanes, 256 / lanes);
    const int64_t rows = (d.dim + block.y - 1) / block.y;
    const int G = (int)std::max<int64_t>(1, std::min<int64_t>(kMaxGrid, (rows + 3) / 4));
    const cx<T>* V = nullptr;
    if constexpr (std::is_same<T, double>::value)
        V = d.V64;
    else
        V = d.V32;
    k_defl_part<T><<<dim3(G, d.n), block, 0, ctx->stream>>>(V, d.dim, b, d.part);
    k_defl_coef<<<(d.n * nrhs + 127) / 128, 128, 0, ctx->stream>>>(d.part, G, d.n, nrhs, d.inv, d.coef);
    k_defl_combine<T><<<(unsigned)((d.dim * nrhs + 255) / 256), 256, 0, ctx->stream>>>(V, d.dim, d.n, d.coef, x);
    count_launch(ctx, 3);
    SMG_CHECK_LAUNCH(ctx);
    return SMG_OK;
}

template smg_status smg_defl_guess<float>(smg_context*, MgDeflation&, VecView<float>, VecView<float>);
template smg_status smg_defl_guess<double>(smg_context*, MgDeflation&, VecView<double>, VecView<double>);

// CoarseDeflState::lowmode_solution (src/hmc.h:312-323): x = P sum_i v_i (v_i^dag P^dag phi) / lambda_i
smg_status smg_mg_lowmode_internal(smg_mg* mg, const smg_field* phi, smg_field* x) {
    smg_context* ctx = smg_mg_ctx(mg);
    MgDeflation& d = smg_mg_defl(mg);
    if (d.n > 0 && d.level != 1)
        return smg_fail(ctx, SMG_UNSUPPORTED, "low-mode solution: the deflation space is not on level 1");
    if (d.n == 0) {
        SMG_CUDA(ctx, cudaMemsetAsync(x->data, 0, x->bytes, ctx->stream));
        return SMG_OK;
    }
    SMG_TRY(smg_mg_restrict0_f64(mg, phi, d.c_in));
    VecView<double> b, y;
    b.p = d.c_in;
    y.p = d.c_out;
    b.nsites = y.nsites = (int)d.dim;
    b.ndof = y.ndof = 1;
    b.nrhs = y.nrhs = 1;
    SMG_TRY(smg_defl_guess<double>(ctx, d, b, y));
    return smg_mg_prolong0_f64(mg, d.c_out, x);
}

extern "C" {

SMG_API smg_status smg_mg_setup_deflation_level(smg_mg* mg, int level, int n_ev, int n_kr, int max_restarts,
                                                double tol, smg_deflation_info* info) {
    if (!mg || n_ev < 0 || max_restarts < 0 || !(tol > 0)) return SMG_BAD_ARG;
    smg_context* ctx = smg_mg_ctx(mg);
    if (level < 1 || level >= smg_mg_nlevels(mg))
        return smg_fail(ctx, SMG_BAD_ARG, "deflation: level must be a coarse level of the hierarchy");
    const int64_t dim = smg_mg_level_dim(mg, level);
    MgDeflation& d = smg_mg_defl(mg);
    smg_mg_drop_cycle_graph(mg);
    if (n_ev == 0) {
        d.n = 0;
        d.vals.clear();
        if (info) *info = smg_deflation_info{1, 0, 0, 0};
        return SMG_OK;
    }
    // Krylov size of SparseCoarseOp::setup_deflation (src/coarse_op.cpp:40-44) and trlm_eigensolver (:705)
    if (n_kr <= 0) n_kr = (int)std::min<int64_t>(2 * n_ev + 10, dim);
    if (n_kr > dim) n_kr = (int)dim;
    if (n_kr < n_ev + 2) n_kr = (int)std::min<int64_t>(n_ev + 6, dim);
    if (n_kr < n_ev + 6) n_kr = (int)std::min<int64_t>(n_ev + 6, dim);
    if (n_ev > n_kr || n_kr > 120) return smg_fail(ctx, SMG_UNSUPPORTED, "deflation: n_ev <= n_kr <= 120 required");
    SMG_TRY(ensure_storage(ctx, d, n_ev, dim));
    d.n = 0;
    d.level = level;
    std::vector<double> vals;
    SMG_TRY(trlm(mg, level, n_ev, n_kr, max_restarts, tol, d.V64, vals, info));
    d.n = n_ev;
    d.vals = vals;
    SMG_TRY(commit(ctx, d));
    if (info && !info->converged) return SMG_NOT_CONVERGED;
    return SMG_OK;
}

SMG_API smg_status smg_mg_setup_deflation(smg_mg* mg, int n_ev, int n_kr, int max_restarts, double tol,
                                          smg_deflation_info* info) {
    return smg_mg_setup_deflation_level(mg, 1, n_ev, n_kr, max_restarts, tol, info);
}

SMG_API smg_status smg_mg_set_deflation(smg_mg* mg, int n, const double* vals, const double* vecs) {
    if (!mg || n < 0 || (n > 0 && (!vals || !vecs))) return SMG_BAD_ARG;
    smg_context* ctx = smg_mg_ctx(mg);
    if (smg_mg_nlevels(mg) < 2) return smg_fail(ctx, SMG_BAD_ARG, "deflation needs a coarse level");
    const int64_t dim = smg_mg_level_dim(mg, 1);
    MgDeflation& d = smg_mg_defl(mg);
    smg_mg_drop_cycle_graph(mg);
    d.level = 1;
    if (n > 0) {
        SMG_TRY(ensure_storage(ctx, d, n, dim));
        SMG_CUDA(ctx, cudaMemcpyAsync(d.V64, vecs, (size_t)n * dim * sizeof(cx<double>), cudaMemcpyHostToDevice,
                                      ctx->stream));
    }
    d.n = n;
    d.vals.assign(vals, vals + n);
    return commit(ctx, d);
}

SMG_API smg_status smg_mg_get_deflation(smg_mg* mg, int* n, double* vals, double* vecs) {
    if (!mg || !n) return SMG_BAD_ARG;
    smg_context* ctx = smg_mg_ctx(mg);
    MgDeflation& d = smg_mg_defl(mg);
    *n = d.n;
    if (vals) std::copy(d.vals.begin(), d.vals.end(), vals);
    if (vecs && d.n > 0) {
        SMG_CUDA(ctx, cudaMemcpyAsync(vecs, d.V64, (size_t)d.n * d.dim * sizeof(cx<double>), cudaMemcpyDeviceToHost,
                                      ctx->stream));
        SMG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    }
    return SMG_OK;
}

SMG_API smg_status smg_mg_deflation_rr(smg_mg* mg, double* max_residual) {
    if (!mg) return SMG_BAD_ARG;
    smg_context* ctx = smg_mg_ctx(mg);
    MgDeflation& d = smg_mg_defl(mg);
    const int k = d.n;
    if (k == 0) {
        if (max_residual) *max_residual = 0;
        return SMG_OK;
    }
    const int64_t n = d.dim;
    Workspace ws;
    ws.ctx = ctx;
    cx<double>* AV = nullptr;
    cx<double>* M = nullptr;
    cx<double>* Y = nullptr;
    cx<double>* out = nullptr;
    double* part = nullptr;
    SMG_TRY(ws.alloc(&AV, (size_t)k * n));
    SMG_TRY(ws.alloc(&M, (size_t)k * k + 1));
    SMG_TRY(ws.alloc(&Y, (size_t)k * k));
    SMG_TRY(ws.alloc(&out, (size_t)2 * k * n));
    SMG_TRY(ws.alloc(&part, part_doubles(k)));
    // rr_evolve (src/eigen_evolve.cpp:48-105): M_ij = v_i^dag A v_j, eigenpairs of M, rotated vectors
    for (int j = 0; j < k; ++j) SMG_TRY(smg_mg_apply_f64(mg, d.level, d.V64 + (int64_t)j * n, AV + (int64_t)j * n));
    for (int j = 0; j < k; ++j) SMG_TRY(multi_dot(ctx, d.V64, n, k, AV + (int64_t)j * n, n, part, M + (int64_t)j * k));
    std::vector<cx<double>> mh((size_t)k * k);
    SMG_CUDA(ctx, cudaMemcpyAsync(mh.data(), M, mh.size() * sizeof(cx<double>), cudaMemcpyDeviceToHost, ctx->stream));
    SMG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    std::vector<std::complex<double>> A((size_t)k * k);
    for (int j = 0; j < k; ++j)
        for (int i = 0; i <= j; ++i) {  // the upper triangle, mirrored (src/eigen_evolve.cpp:66-72)
            const cx<double> z = mh[(size_t)j * k + i];
            A[(size_t)j * k + i] = {z.re, z.im};
            A[(size_t)i * k + j] = {z.re, -z.im};
        }
    std::vector<double> ev;
    std::vector<std::complex<double>> evec;
    hermitian_eig(k, A, ev, evec);
    std::vector<cx<double>> yh((size_t)k * k);
    for (size_t i = 0; i < yh.size(); ++i) yh[i] = mk(evec[i].real(), evec[i].imag());
    SMG_CUDA(ctx, cudaMemcpyAsync(Y, yh.data(), yh.size() * sizeof(cx<double>), cudaMemcpyHostToDevice, ctx->stream));
    const int G = grid_for(n);
    k_rotate<<<G, 256, 0, ctx->stream>>>(d.V64, n, k, Y, k, out, n);
    k_rotate<<<G, 256, 0, ctx->stream>>>(AV, n, k, Y, k, out + (int64_t)k * n, n);
    count_launch(ctx, 2);
    SMG_CHECK_LAUNCH(ctx);
    SMG_CUDA(ctx, cudaMemcpyAsync(d.V64, out, (size_t)k * n * sizeof(cx<double>), cudaMemcpyDeviceToDevice,
                                  ctx->stream));
    d.vals = ev;
    if (max_residual) {
        // max_i ||A v_i - lambda_i v_i|| / ||A v_i|| (src/eigen_evolve.cpp:92-100)
        double worst = 0;
        for (int i = 0; i < k; ++i) {
            const cx<double>* av = out + (int64_t)(k + i) * n;
            SMG_TRY(multi_dot(ctx, av, n, 1, av, n, part, M));
            std::vector<cx<double>> coef = {mk(ev[i], 0.0)};
            SMG_CUDA(ctx, cudaMemcpyAsync(M + 1, coef.data(), sizeof(cx<double>), cudaMemcpyHostToDevice, ctx->stream));
            k_maxpy<<<G, 256, 0, ctx->stream>>>(d.V64 + (int64_t)i * n, n, 1, M + 1, (cx<double>*)av, n);
            count_launch(ctx);
            cx<double> h[2];
            SMG_CUDA(ctx, cudaMemcpyAsync(h, M, sizeof(cx<double>), cudaMemcpyDeviceToHost, ctx->stream));
            SMG_TRY(multi_dot(ctx, av, n, 1, av, n, part, M));
            SMG_CUDA(ctx, cudaMemcpyAsync(h + 1, M, sizeof(cx<double>), cudaMemcpyDeviceToHost, ctx->stream));
            SMG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
            worst = std::max(worst, std::sqrt(std::max(h[1].re, 0.0)) / std::max(std::sqrt(std::max(h[0].re, 0.0)), 1e-30));
        }
        *max_residual = worst;
    }
    return commit(ctx, d);
}

SMG_API smg_status smg_mg_lowmode_solution(smg_mg* mg, const smg_field* phi, smg_field* x) {
    if (!mg || !phi || !x) return SMG_BAD_ARG;
    smg_context* ctx = smg_mg_ctx(mg);
    smg_dirac* dd = smg_mg_dirac(mg);
    if (phi->prec != SMG_F64 || x->prec != SMG_F64 || phi->nrhs != 1 || x->nrhs != 1 ||
        phi->g.L != dd->gauge->g.L || x->g.L != dd->gauge->g.L)
        return smg_fail(ctx, SMG_BAD_ARG, "lowmode solution: single-RHS F64 fields of the hierarchy's lattice");
    return smg_mg_lowmode_internal(mg, phi, x);
}

}  // extern "C"
