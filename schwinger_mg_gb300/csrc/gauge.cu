// Gauge field on the device: storage, plaquette, Wilson gauge action and
// gauge force (reference src/gauge.h:10-36, src/hmc_forces.cpp:80-111).
#include "smg_internal.h"
#include "reduce.cuh"

namespace {

__device__ __forceinline__ cx<double> lk(const cx<double>* __restrict__ U, const Geom& g, int mu, int x, int y) {
    return U[(int64_t)mu * g.V + site_q(g, wrap(x, g.L), wrap(y, g.L))];
}

// host [mu][s] lexicographic  ->  device [mu][parity][cb]
__global__ void k_links_in(const cx<double>* __restrict__ host, cx<double>* __restrict__ U, Geom g) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= 2 * g.V) return;
    int mu = i / g.V, s = i - mu * g.V;
    int x = s % g.L, y = s / g.L;
    U[(int64_t)mu * g.V + site_q(g, x, y)] = host[i];
}

__global__ void k_links_out(const cx<double>* __restrict__ U, cx<double>* __restrict__ host, Geom g) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= 2 * g.V) return;
    int mu = i / g.V, s = i - mu * g.V;
    int x = s % g.L, y = s / g.L;
    host[i] = U[(int64_t)mu * g.V + site_q(g, x, y)];
}

__global__ void k_links_f32(const cx<double>* __restrict__ U, cx<float>* __restrict__ U32, int n) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) U32[i] = cvt<float>(U[i]);
}

// sum over sites of Re P(s), P(s) = U0(s) U1(s+x) U0*(s+y) U1*(s)  (gauge.h:26-30)
__global__ void k_plaq_sum(const cx<double>* __restrict__ U, Geom g, double* partials, unsigned int* ticket,
                           double* out) {
    double v[1] = {0.0};
    for (int s = blockIdx.x * blockDim.y + threadIdx.y; s < g.V; s += gridDim.x * blockDim.y) {
        int x = s % g.L, y = s / g.L;
        cx<double> P = lk(U, g, 0, x, y) * lk(U, g, 1, x + 1, y) * conj(lk(U, g, 0, x, y + 1)) *
                       conj(lk(U, g, 1, x, y));
        v[0] += P.re;
    }
    block_reduce_finalise<1>(v, partials, ticket, 1, FinStore{out, 1});
}

// gauge_force, hmc_forces.cpp:88-111; output lexicographic [mu][s]
__global__ void k_gauge_force(const cx<double>* __restrict__ U, Geom g, double beta, double* __restrict__ F) {
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= g.V) return;
    int x = s % g.L, y = s / g.L;
    {
        cx<double> staple = lk(U, g, 1, x + 1, y) * conj(lk(U, g, 0, x, y + 1)) * conj(lk(U, g, 1, x, y)) +
                            conj(lk(U, g, 1, x + 1, y - 1)) * conj(lk(U, g, 0, x, y - 1)) * lk(U, g, 1, x, y - 1);
        F[s] = -beta * (lk(U, g, 0, x, y) * staple).im;
    }
    {
        cx<double> staple = lk(U, g, 0, x, y + 1) * conj(lk(U, g, 1, x + 1, y)) * conj(lk(U, g, 0, x, y)) +
                            conj(lk(U, g, 0, x - 1, y + 1)) * conj(lk(U, g, 1, x - 1, y)) * lk(U, g, 0, x - 1, y);
        F[g.V + s] = -beta * (lk(U, g, 1, x, y) * staple).im;
    }
}

smg_status plaq_sum(smg_gauge* gf, double* out_host) {
    smg_context* ctx = gf->ctx;
    ReduceLaunch rl = reduce_launch(gf->g.V, 1);
    SMG_TRY(smg_reduce_reserve(ctx, rl.grid.x));
    SMG_TRY(smg_host_stage_reserve(ctx, sizeof(double)));
    double* dev = nullptr;
    SMG_CUDA(ctx, cudaMallocAsync(&dev, sizeof(double), ctx->stream));
    k_plaq_sum<<<rl.grid, rl.block, 0, ctx->stream>>>(gf->U64, gf->g, ctx->red.partials, ctx->red.tickets, dev);
    count_launch(ctx);
    SMG_CHECK_LAUNCH(ctx);
    SMG_CUDA(ctx, cudaMemcpyAsync(ctx->host_stage, dev, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    SMG_CUDA(ctx, cudaFreeAsync(dev, ctx->stream));
    SMG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    *out_host = ctx->host_stage[0];
    return SMG_OK;
}

}  // namespace

// gauge_force into a device array F[mu][s] (lexicographic)
smg_status smg_gauge_force_dev(smg_gauge* gf, double beta, double* F_dev) {
    smg_context* ctx = gf->ctx;
    k_gauge_force<<<(gf->g.V + 255) / 256, 256, 0, ctx->stream>>>(gf->U64, gf->g, beta, F_dev);
    count_launch(ctx);
    SMG_CHECK_LAUNCH(ctx);
    return SMG_OK;
}

smg_status smg_gauge_ensure_f32(smg_gauge* gf) {
    smg_context* ctx = gf->ctx;
    if (!gf->U32) SMG_CUDA(ctx, cudaMalloc(&gf->U32, (size_t)2 * gf->g.V * sizeof(cx<float>)));
    int n = 2 * gf->g.V;
    k_links_f32<<<(n + 255) / 256, 256, 0, ctx->stream>>>(gf->U64, gf->U32, n);
    count_launch(ctx);
    SMG_CHECK_LAUNCH(ctx);
    return SMG_OK;
}

extern "C" {

SMG_API smg_status smg_gauge_create(smg_context* ctx, int L, const double* U, smg_gauge** out) {
    if (!ctx || !out || !U) return SMG_BAD_ARG;
    *out = nullptr;
    if (L < 4 || (L & 1)) return smg_fail(ctx, SMG_BAD_ARG, "L must be even and >= 4");
    SMG_CUDA(ctx, cudaSetDevice(ctx->device));
    smg_gauge* gf = new smg_gauge();
    gf->ctx = ctx;
    gf->g = Geom{L, L / 2, L * L, L * L / 2};
    cudaError_t e = cudaMalloc(&gf->U64, (size_t)2 * gf->g.V * sizeof(cx<double>));
    if (e != cudaSuccess) {
        delete gf;
        return smg_fail(ctx, SMG_NO_MEMORY, "gauge allocation");
    }
    smg_status s = smg_gauge_set(gf, U);
    if (s != SMG_OK) {
        smg_gauge_destroy(gf);
        return s;
    }
    *out = gf;
    return SMG_OK;
}

SMG_API smg_status smg_gauge_destroy(smg_gauge* gf) {
    if (!gf) return SMG_OK;
    cudaSetDevice(gf->ctx->device);
    cudaStreamSynchronize(gf->ctx->stream);
    if (gf->U64) cudaFree(gf->U64);
    if (gf->U32) cudaFree(gf->U32);
    delete gf;
    return SMG_OK;
}

SMG_API smg_status smg_gauge_set(smg_gauge* gf, const double* U) {
    if (!gf || !U) return SMG_BAD_ARG;
    smg_context* ctx = gf->ctx;
    size_t bytes = (size_t)2 * gf->g.V * sizeof(cx<double>);
    cx<double>* tmp = nullptr;
    SMG_CUDA(ctx, cudaMallocAsync(&tmp, bytes, ctx->stream));
    SMG_CUDA(ctx, cudaMemcpyAsync(tmp, U, bytes, cudaMemcpyHostToDevice, ctx->stream));
    int n = 2 * gf->g.V;
    k_links_in<<<(n + 255) / 256, 256, 0, ctx->stream>>>(tmp, gf->U64, gf->g);
    count_launch(ctx);
    SMG_CHECK_LAUNCH(ctx);
    SMG_CUDA(ctx, cudaFreeAsync(tmp, ctx->stream));
    SMG_TRY(smg_gauge_ensure_f32(gf));
    return SMG_OK;
}

SMG_API smg_status smg_gauge_get(smg_gauge* gf, double* U) {
    if (!gf || !U) return SMG_BAD_ARG;
    smg_context* ctx = gf->ctx;
    size_t bytes = (size_t)2 * gf->g.V * sizeof(cx<double>);
    cx<double>* tmp = nullptr;
    SMG_CUDA(ctx, cudaMallocAsync(&tmp, bytes, ctx->stream));
    int n = 2 * gf->g.V;
    k_links_out<<<(n + 255) / 256, 256, 0, ctx->stream>>>(gf->U64, tmp, gf->g);
    count_launch(ctx);
    SMG_CHECK_LAUNCH(ctx);
    SMG_CUDA(ctx, cudaMemcpyAsync(U, tmp, bytes, cudaMemcpyDeviceToHost, ctx->stream));
    SMG_CUDA(ctx, cudaFreeAsync(tmp, ctx->stream));
    SMG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return SMG_OK;
}

SMG_API int smg_gauge_L(const smg_gauge* gf) { return gf ? gf->g.L : 0; }

SMG_API smg_status smg_gauge_avg_plaq(smg_gauge* gf, double* out) {
    if (!gf || !out) return SMG_BAD_ARG;
    double s = 0;
    SMG_TRY(plaq_sum(gf, &s));
    *out = s / gf->g.V;
    return SMG_OK;
}

SMG_API smg_status smg_gauge_action(smg_gauge* gf, double beta, double* out) {
    if (!gf || !out) return SMG_BAD_ARG;
    double s = 0;
    SMG_TRY(plaq_sum(gf, &s));
    *out = -beta * s;
    return SMG_OK;
}

SMG_API smg_status smg_gauge_force(smg_gauge* gf, double beta, double* force) {
    if (!gf || !force) return SMG_BAD_ARG;
    smg_context* ctx = gf->ctx;
    size_t bytes = (size_t)2 * gf->g.V * sizeof(double);
    double* dev = nullptr;
    SMG_CUDA(ctx, cudaMallocAsync(&dev, bytes, ctx->stream));
    k_gauge_force<<<(gf->g.V + 255) / 256, 256, 0, ctx->stream>>>(gf->U64, gf->g, beta, dev);
    count_launch(ctx);
    SMG_CHECK_LAUNCH(ctx);
    SMG_CUDA(ctx, cudaMemcpyAsync(force, dev, bytes, cudaMemcpyDeviceToHost, ctx->stream));
    SMG_CUDA(ctx, cudaFreeAsync(dev, ctx->stream));
    SMG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return SMG_OK;
}

}  // extern "C"
