// Spinor fields: allocation, host <-> device transfers with the even-odd
// permutation, precision conversion, and the BLAS-1 kernels
// (reference src/linalg.cpp:8-48).
#include "smg_internal.h"
#include "half.cuh"
#include "reduce.cuh"

namespace {

template <typename T>
__global__ void k_host_to_field(const cx<double>* __restrict__ host, cx<T>* __restrict__ out, Geom g,
                                int nrhs) {
    // one thread per (lexicographic site, rhs); coalesced reads of the host image
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    int64_t total = (int64_t)g.V * nrhs;
    if (i >= total) return;
    int rhs = (int)(i / g.V);
    int s = (int)(i - (int64_t)rhs * g.V);
    int x = s % g.L, y = s / g.L;
    int q = site_q(g, x, y);
    const cx<double>* h = host + ((int64_t)rhs * g.V + s) * 2;
    out[sidx(q, rhs, 0, nrhs)] = cvt<T>(h[0]);
    out[sidx(q, rhs, 1, nrhs)] = cvt<T>(h[1]);
}

template <typename T>
__global__ void k_field_to_host(const cx<T>* __restrict__ in, cx<double>* __restrict__ host, Geom g,
                                int nrhs) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    int64_t total = (int64_t)g.V * nrhs;
    if (i >= total) return;
    int rhs = (int)(i / g.V);
    int s = (int)(i - (int64_t)rhs * g.V);
    int x = s % g.L, y = s / g.L;
    int q = site_q(g, x, y);
    cx<double>* h = host + ((int64_t)rhs * g.V + s) * 2;
    h[0] = cvt<double>(in[sidx(q, rhs, 0, nrhs)]);
    h[1] = cvt<double>(in[sidx(q, rhs, 1, nrhs)]);
}

template <typename D, typename S>
__global__ void k_convert(const cx<S>* __restrict__ in, cx<D>* __restrict__ out, int64_t n) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = cvt<D>(in[i]);
}

// ---- BLAS-1: every kernel strides over sites; threadIdx.x is the rhs lane
template <typename T>
__global__ void k_dot(const cx<T>* __restrict__ a, const cx<T>* __restrict__ b, int nsites, int nrhs,
                      double* partials, unsigned int* ticket, double* out) {
    const int rhs = blockIdx.y * blockDim.x + threadIdx.x;
    T v[2] = {T(0), T(0)};
    if (rhs < nrhs) {
        for (int q = blockIdx.x * blockDim.y + threadIdx.y; q < nsites; q += gridDim.x * blockDim.y) {
#pragma unroll
            for (int sp = 0; sp < 2; ++sp) {
                int64_t i = sidx(q, rhs, sp, nrhs);
                cx<T> p = cmulc(a[i], b[i]);
                v[0] += p.re;
                v[1] += p.im;
            }
        }
    }
    block_reduce_finalise<2>(v, partials, ticket, nrhs, FinStore{out, 2});
}

template <typename T>
__global__ void k_norm2(const cx<T>* __restrict__ a, int nsites, int nrhs, double* partials,
                        unsigned int* ticket, double* out) {
    const int rhs = blockIdx.y * blockDim.x + threadIdx.x;
    T v[1] = {T(0)};
    if (rhs < nrhs) {
        for (int q = blockIdx.x * blockDim.y + threadIdx.y; q < nsites; q += gridDim.x * blockDim.y) {
            int64_t i0 = sidx(q, rhs, 0, nrhs);
            v[0] += norm2(a[i0]) + norm2(a[i0 + 1]);
        }
    }
    block_reduce_finalise<1>(v, partials, ticket, nrhs, FinStore{out, 1});
}

template <typename T>
__global__ void k_axpy(const double* __restrict__ alpha, const cx<T>* __restrict__ x, cx<T>* __restrict__ y,
                       int nsites, int nrhs) {
    const int rhs = blockIdx.y * blockDim.x + threadIdx.x;
    const int q = blockIdx.x * blockDim.y + threadIdx.y;
    if (rhs >= nrhs || q >= nsites) return;
    cx<T> a = mk<T>((T)alpha[2 * rhs], (T)alpha[2 * rhs + 1]);
#pragma unroll
    for (int sp = 0; sp < 2; ++sp) {
        int64_t i = sidx(q, rhs, sp, nrhs);
        y[i] = y[i] + a * x[i];
    }
}

template <typename T>
__global__ void k_scale(const double* __restrict__ alpha, cx<T>* __restrict__ v, int nsites, int nrhs) {
    const int rhs = blockIdx.y * blockDim.x + threadIdx.x;
    const int q = blockIdx.x * blockDim.y + threadIdx.y;
    if (rhs >= nrhs || q >= nsites) return;
    cx<T> a = mk<T>((T)alpha[2 * rhs], (T)alpha[2 * rhs + 1]);
#pragma unroll
    for (int sp = 0; sp < 2; ++sp) {
        int64_t i = sidx(q, rhs, sp, nrhs);
        v[i] = a * v[i];
    }
}

// F16 fields: one thread per (device site, rhs), a lane group of nrhs threads per site
__global__ void k_host_to_field_h(const cx<double>* __restrict__ host, __half2* __restrict__ out,
                                  float* __restrict__ scale, Geom g, int nrhs) {
    const int rhs = threadIdx.x;
    const int q = blockIdx.x * blockDim.y + threadIdx.y;
    const bool valid = q < g.V;
    Spinor<float> v;
    v.s0 = mk(0.f, 0.f);
    v.s1 = mk(0.f, 0.f);
    if (valid) {
        int x, y, p;
        site_coords(g, q, x, y, p);
        const cx<double>* h = host + ((int64_t)rhs * g.V + x + (int64_t)g.L * y) * 2;
        v.s0 = cvt<float>(h[0]);
        v.s1 = cvt<float>(h[1]);
    }
    st_spinor_h(out, scale, q, rhs, nrhs, blockDim.x, v, valid);
}

__global__ void k_field_h_to_host(const __half2* __restrict__ in, const float* __restrict__ scale,
                                  cx<double>* __restrict__ host, Geom g, int nrhs) {
    const int rhs = threadIdx.x;
    const int q = blockIdx.x * blockDim.y + threadIdx.y;
    if (q >= g.V) return;
    int x, y, p;
    site_coords(g, q, x, y, p);
    const Spinor<float> v = ld_spinor_h(in, scale, q, rhs, nrhs);
    cx<double>* h = host + ((int64_t)rhs * g.V + x + (int64_t)g.L * y) * 2;
    h[0] = cvt<double>(v.s0);
    h[1] = cvt<double>(v.s1);
}

size_t elem_bytes(smg_precision p) {
    switch (p) {
        case SMG_F64: return sizeof(cx<double>);
        case SMG_F32: return sizeof(cx<float>);
        case SMG_F16: return sizeof(__half2);
    }
    return 0;
}

// Host images go through a staging buffer from the context's pool (a DMA copy, then a layout kernel):
// allocating it per call put a device allocation and free into every upload and download.
smg_status transfer_in(smg_field* f, const double* host) {
    smg_context* ctx = f->ctx;
    SMG_CUDA(ctx, cudaSetDevice(ctx->device));
    const int64_t n = f->n_complex();
    const size_t nb = (size_t)n * sizeof(cx<double>);
    cx<double>* tmp = nullptr;
    SMG_TRY(smg_buf_take(ctx, nb, reinterpret_cast<void**>(&tmp)));
    SMG_CUDA(ctx, cudaMemcpyAsync(tmp, host, nb, cudaMemcpyHostToDevice, ctx->stream));
    int64_t total = (int64_t)f->g.V * f->nrhs;
    int blocks = (int)((total + 255) / 256);
    if (f->prec == SMG_F16) {
        const dim3 block(f->nrhs, 256 / f->nrhs);
        k_host_to_field_h<<<(f->g.V + block.y - 1) / block.y, block, 0, ctx->stream>>>(
            tmp, (__half2*)f->data, f->scale, f->g, f->nrhs);
    } else if (f->prec == SMG_F64)
        k_host_to_field<double><<<blocks, 256, 0, ctx->stream>>>(tmp, (cx<double>*)f->data, f->g, f->nrhs);
    else
        k_host_to_field<float><<<blocks, 256, 0, ctx->stream>>>(tmp, (cx<float>*)f->data, f->g, f->nrhs);
    count_launch(ctx);
    SMG_CHECK_LAUNCH(ctx);
    smg_buf_give(ctx, nb, tmp);  // later users are ordered after this work on the same stream
    return SMG_OK;
}

smg_status transfer_out(const smg_field* f, double* host, bool sync) {
    smg_context* ctx = f->ctx;
    SMG_CUDA(ctx, cudaSetDevice(ctx->device));
    const int64_t n = f->n_complex();
    const size_t nb = (size_t)n * sizeof(cx<double>);
    cx<double>* tmp = nullptr;
    SMG_TRY(smg_buf_take(ctx, nb, reinterpret_cast<void**>(&tmp)));
    int64_t total = (int64_t)f->g.V * f->nrhs;
    int blocks = (int)((total + 255) / 256);
    if (f->prec == SMG_F16) {
        const dim3 block(f->nrhs, 256 / f->nrhs);
        k_field_h_to_host<<<(f->g.V + block.y - 1) / block.y, block, 0, ctx->stream>>>(
            (const __half2*)f->data, f->scale, tmp, f->g, f->nrhs);
    } else if (f->prec == SMG_F64)
        k_field_to_host<double><<<blocks, 256, 0, ctx->stream>>>((const cx<double>*)f->data, tmp, f->g, f->nrhs);
    else
        k_field_to_host<float><<<blocks, 256, 0, ctx->stream>>>((const cx<float>*)f->data, tmp, f->g, f->nrhs);
    count_launch(ctx);
    SMG_CHECK_LAUNCH(ctx);
    SMG_CUDA(ctx, cudaMemcpyAsync(host, tmp, nb, cudaMemcpyDeviceToHost, ctx->stream));
    smg_buf_give(ctx, nb, tmp);
    if (sync) SMG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return SMG_OK;
}

}  // namespace

smg_status smg_field_check_pair(const smg_field* a, const smg_field* b) {
    if (!a || !b) return SMG_BAD_ARG;
    if (a->ctx != b->ctx)
        return smg_fail(a->ctx, SMG_BAD_ARG, "fields belong to different contexts");
    if (a->g.L != b->g.L || a->nrhs != b->nrhs || a->prec != b->prec)
        return smg_fail(a->ctx, SMG_BAD_ARG, "field shape or precision mismatch");
    return SMG_OK;
}

smg_status smg_field_alloc_like(const smg_field* proto, smg_precision prec, smg_field** out) {
    return smg_field_create(proto->ctx, proto->g.L, proto->nrhs, prec, out);
}

smg_status smg_field_take(const smg_field* proto, smg_precision prec, smg_field** out) {
    smg_context* ctx = proto->ctx;
    auto& pool = ctx->field_pool;
    for (size_t i = 0; i < pool.size(); ++i) {
        smg_field* f = pool[i];
        if (f->g.L == proto->g.L && f->nrhs == proto->nrhs && f->prec == prec) {
            pool.erase(pool.begin() + (std::ptrdiff_t)i);
            *out = f;
            return SMG_OK;
        }
    }
    return smg_field_create(ctx, proto->g.L, proto->nrhs, prec, out);
}

void smg_field_give(smg_field* f) {
    if (f) f->ctx->field_pool.push_back(f);
}

smg_status smg_buf_take(smg_context* ctx, size_t bytes, void** out) {
    auto& pool = ctx->buf_pool;
    for (size_t i = 0; i < pool.size(); ++i) {
        if (pool[i].first == bytes) {
            *out = pool[i].second;
            pool.erase(pool.begin() + (std::ptrdiff_t)i);
            return SMG_OK;
        }
    }
    SMG_CUDA(ctx, cudaMalloc(out, bytes));
    return SMG_OK;
}

void smg_buf_give(smg_context* ctx, size_t bytes, void* p) {
    if (p) ctx->buf_pool.emplace_back(bytes, p);
}

// Reduction helpers used by the solvers (results stay on the device).
smg_status smg_dot_dev(const smg_field* a, const smg_field* b, double* out_dev) {
    SMG_TRY(smg_field_check_pair(a, b));
    smg_context* ctx = a->ctx;
    ReduceLaunch rl = reduce_launch(a->g.V, a->nrhs);
    SMG_TRY(smg_reduce_reserve(ctx, (size_t)rl.grid.x * a->nrhs * 2));
    if (a->prec == SMG_F64)
        k_dot<double><<<rl.grid, rl.block, 0, ctx->stream>>>((const cx<double>*)a->data, (const cx<double>*)b->data,
                                                           a->g.V, a->nrhs, ctx->red.partials, ctx->red.tickets, out_dev);
    else if (a->prec == SMG_F32)
        k_dot<float><<<rl.grid, rl.block, 0, ctx->stream>>>((const cx<float>*)a->data, (const cx<float>*)b->data,
                                                          a->g.V, a->nrhs, ctx->red.partials, ctx->red.tickets, out_dev);
    else
        return smg_fail(ctx, SMG_UNSUPPORTED, "dot on F16 field");
    count_launch(ctx);
    SMG_CHECK_LAUNCH(ctx);
    return SMG_OK;
}

smg_status smg_norm2_dev(const smg_field* a, double* out_dev) {
    smg_context* ctx = a->ctx;
    ReduceLaunch rl = reduce_launch(a->g.V, a->nrhs);
    SMG_TRY(smg_reduce_reserve(ctx, (size_t)rl.grid.x * a->nrhs));
    if (a->prec == SMG_F64)
        k_norm2<double><<<rl.grid, rl.block, 0, ctx->stream>>>((const cx<double>*)a->data, a->g.V, a->nrhs,
                                                             ctx->red.partials, ctx->red.tickets, out_dev);
    else if (a->prec == SMG_F32)
        k_norm2<float><<<rl.grid, rl.block, 0, ctx->stream>>>((const cx<float>*)a->data, a->g.V, a->nrhs,
                                                            ctx->red.partials, ctx->red.tickets, out_dev);
    else
        return smg_fail(ctx, SMG_UNSUPPORTED, "norm on F16 field");
    count_launch(ctx);
    SMG_CHECK_LAUNCH(ctx);
    return SMG_OK;
}

smg_status smg_axpy_dev(const double* alpha_dev, const smg_field* x, smg_field* y) {
    SMG_TRY(smg_field_check_pair(x, y));
    smg_context* ctx = x->ctx;
    SiteLaunch sl = site_launch(x->g.V, x->nrhs);
    if (x->prec == SMG_F64)
        k_axpy<double><<<sl.grid, sl.block, 0, ctx->stream>>>(alpha_dev, (const cx<double>*)x->data,
                                                            (cx<double>*)y->data, x->g.V, x->nrhs);
    else if (x->prec == SMG_F32)
        k_axpy<float><<<sl.grid, sl.block, 0, ctx->stream>>>(alpha_dev, (const cx<float>*)x->data,
                                                           (cx<float>*)y->data, x->g.V, x->nrhs);
    else
        return smg_fail(ctx, SMG_UNSUPPORTED, "axpy on F16 field");
    count_launch(ctx);
    SMG_CHECK_LAUNCH(ctx);
    return SMG_OK;
}

extern "C" {

SMG_API smg_status smg_field_create(smg_context* ctx, int L, int nrhs, smg_precision prec, smg_field** out) {
    if (!ctx || !out) return SMG_BAD_ARG;
    *out = nullptr;
    if (L < 4 || (L & 1)) return smg_fail(ctx, SMG_BAD_ARG, "L must be even and >= 4");
    if (nrhs < 1 || nrhs > 2048) return smg_fail(ctx, SMG_BAD_ARG, "nrhs must be in [1, 2048]");
    if (prec != SMG_F64 && prec != SMG_F32 && prec != SMG_F16) return smg_fail(ctx, SMG_BAD_ARG, "precision");
    if (prec == SMG_F16 && !f16_nrhs_ok(nrhs))
        return smg_fail(ctx, SMG_BAD_ARG, "F16 fields need nrhs a power of two <= 32");
    SMG_CUDA(ctx, cudaSetDevice(ctx->device));
    smg_field* f = new smg_field();
    f->ctx = ctx;
    f->g = Geom{L, L / 2, L * L, L * L / 2};
    f->nrhs = nrhs;
    f->prec = prec;
    f->bytes = (size_t)f->n_complex() * elem_bytes(prec);
    cudaError_t e = cudaMalloc(&f->data, f->bytes);
    if (e != cudaSuccess) {
        delete f;
        return smg_fail(ctx, SMG_NO_MEMORY, std::string("field allocation: ") + cudaGetErrorString(e));
    }
    if (prec == SMG_F16) {
        e = cudaMalloc(&f->scale, (size_t)f->g.V * sizeof(float));
        if (e != cudaSuccess) {
            cudaFree(f->data);
            delete f;
            return smg_fail(ctx, SMG_NO_MEMORY, "field scale allocation");
        }
    }
    e = cudaMemsetAsync(f->data, 0, f->bytes, ctx->stream);
    if (e != cudaSuccess) {
        cudaFree(f->data);
        if (f->scale) cudaFree(f->scale);
        delete f;
        return smg_fail(ctx, SMG_DEVICE_ERROR, "field memset");
    }
    *out = f;
    return SMG_OK;
}

SMG_API smg_status smg_field_destroy(smg_field* f) {
    if (!f) return SMG_OK;
    cudaSetDevice(f->ctx->device);
    cudaStreamSynchronize(f->ctx->stream);
    if (f->data) cudaFree(f->data);
    if (f->scale) cudaFree(f->scale);
    delete f;
    return SMG_OK;
}

SMG_API smg_status smg_field_upload(smg_field* f, const double* host) {
    if (!f || !host) return SMG_BAD_ARG;
    SMG_TRY(transfer_in(f, host));
    return SMG_OK;
}

SMG_API smg_status smg_field_download(const smg_field* f, double* host) {
    if (!f || !host) return SMG_BAD_ARG;
    return transfer_out(f, host, true);
}

SMG_API smg_status smg_field_upload_async(smg_field* f, const double* host) {
    if (!f || !host) return SMG_BAD_ARG;
    return transfer_in(f, host);
}

SMG_API smg_status smg_field_download_async(const smg_field* f, double* host) {
    if (!f || !host) return SMG_BAD_ARG;
    return transfer_out(f, host, false);
}

SMG_API smg_status smg_field_zero(smg_field* f) {
    if (!f) return SMG_BAD_ARG;
    SMG_CUDA(f->ctx, cudaMemsetAsync(f->data, 0, f->bytes, f->ctx->stream));
    if (f->scale) SMG_CUDA(f->ctx, cudaMemsetAsync(f->scale, 0, (size_t)f->g.V * sizeof(float), f->ctx->stream));
    return SMG_OK;
}

SMG_API smg_status smg_field_copy(const smg_field* src, smg_field* dst) {
    if (!src || !dst) return SMG_BAD_ARG;
    smg_context* ctx = src->ctx;
    if (src->g.L != dst->g.L || src->nrhs != dst->nrhs || src->ctx != dst->ctx)
        return smg_fail(ctx, SMG_BAD_ARG, "copy: shape mismatch");
    const int64_t n = src->n_complex();
    if (src->prec == dst->prec) {
        SMG_CUDA(ctx, cudaMemcpyAsync(dst->data, src->data, src->bytes, cudaMemcpyDeviceToDevice, ctx->stream));
        if (src->scale)
            SMG_CUDA(ctx, cudaMemcpyAsync(dst->scale, src->scale, (size_t)src->g.V * sizeof(float),
                                          cudaMemcpyDeviceToDevice, ctx->stream));
        return SMG_OK;
    }
    int blocks = (int)((n + 255) / 256);
    if (src->prec == SMG_F64 && dst->prec == SMG_F32)
        k_convert<float, double><<<blocks, 256, 0, ctx->stream>>>((const cx<double>*)src->data, (cx<float>*)dst->data, n);
    else if (src->prec == SMG_F32 && dst->prec == SMG_F64)
        k_convert<double, float><<<blocks, 256, 0, ctx->stream>>>((const cx<float>*)src->data, (cx<double>*)dst->data, n);
    else
        return smg_fail(ctx, SMG_UNSUPPORTED, "copy: F16 conversion");
    count_launch(ctx);
    SMG_CHECK_LAUNCH(ctx);
    return SMG_OK;
}

SMG_API int smg_field_nrhs(const smg_field* f) { return f ? f->nrhs : 0; }
SMG_API int smg_field_L(const smg_field* f) { return f ? f->g.L : 0; }
SMG_API smg_precision smg_field_precision(const smg_field* f) { return f ? f->prec : SMG_F64; }
SMG_API void* smg_field_device_ptr(smg_field* f) { return f ? f->data : nullptr; }
SMG_API size_t smg_field_bytes(const smg_field* f) { return f ? f->bytes : 0; }

SMG_API smg_status smg_blas_dot(const smg_field* a, const smg_field* b, double* out) {
    if (!a || !b || !out) return SMG_BAD_ARG;
    smg_context* ctx = a->ctx;
    SMG_TRY(smg_host_stage_reserve(ctx, (size_t)a->nrhs * 2 * sizeof(double)));
    double* dev = nullptr;
    SMG_CUDA(ctx, cudaMallocAsync(&dev, (size_t)a->nrhs * 2 * sizeof(double), ctx->stream));
    SMG_TRY(smg_dot_dev(a, b, dev));
    SMG_CUDA(ctx, cudaMemcpyAsync(ctx->host_stage, dev, (size_t)a->nrhs * 2 * sizeof(double),
                                  cudaMemcpyDeviceToHost, ctx->stream));
    SMG_CUDA(ctx, cudaFreeAsync(dev, ctx->stream));
    SMG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    for (int i = 0; i < 2 * a->nrhs; ++i) out[i] = ctx->host_stage[i];
    return SMG_OK;
}

SMG_API smg_status smg_blas_norm(const smg_field* a, double* out) {
    if (!a || !out) return SMG_BAD_ARG;
    smg_context* ctx = a->ctx;
    SMG_TRY(smg_host_stage_reserve(ctx, (size_t)a->nrhs * sizeof(double)));
    double* dev = nullptr;
    SMG_CUDA(ctx, cudaMallocAsync(&dev, (size_t)a->nrhs * sizeof(double), ctx->stream));
    SMG_TRY(smg_norm2_dev(a, dev));
    SMG_CUDA(ctx, cudaMemcpyAsync(ctx->host_stage, dev, (size_t)a->nrhs * sizeof(double), cudaMemcpyDeviceToHost,
                                  ctx->stream));
    SMG_CUDA(ctx, cudaFreeAsync(dev, ctx->stream));
    SMG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    for (int i = 0; i < a->nrhs; ++i) out[i] = sqrt(ctx->host_stage[i]);
    return SMG_OK;
}

SMG_API smg_status smg_blas_axpy(const double* alpha, const smg_field* x, smg_field* y) {
    if (!alpha || !x || !y) return SMG_BAD_ARG;
    SMG_TRY(smg_field_check_pair(x, y));
    smg_context* ctx = x->ctx;
    double* dev = nullptr;
    SMG_CUDA(ctx, cudaMallocAsync(&dev, (size_t)x->nrhs * 2 * sizeof(double), ctx->stream));
    SMG_CUDA(ctx, cudaMemcpyAsync(dev, alpha, (size_t)x->nrhs * 2 * sizeof(double), cudaMemcpyHostToDevice,
                                  ctx->stream));
    SMG_TRY(smg_axpy_dev(dev, x, y));
    SMG_CUDA(ctx, cudaFreeAsync(dev, ctx->stream));
    return SMG_OK;
}

SMG_API smg_status smg_blas_scale(const double* alpha, smg_field* v) {
    if (!alpha || !v) return SMG_BAD_ARG;
    smg_context* ctx = v->ctx;
    double* dev = nullptr;
    SMG_CUDA(ctx, cudaMallocAsync(&dev, (size_t)v->nrhs * 2 * sizeof(double), ctx->stream));
    SMG_CUDA(ctx, cudaMemcpyAsync(dev, alpha, (size_t)v->nrhs * 2 * sizeof(double), cudaMemcpyHostToDevice,
                                  ctx->stream));
    SiteLaunch sl = site_launch(v->g.V, v->nrhs);
    if (v->prec == SMG_F64)
        k_scale<double><<<sl.grid, sl.block, 0, ctx->stream>>>(dev, (cx<double>*)v->data, v->g.V, v->nrhs);
    else if (v->prec == SMG_F32)
        k_scale<float><<<sl.grid, sl.block, 0, ctx->stream>>>(dev, (cx<float>*)v->data, v->g.V, v->nrhs);
    else
        return smg_fail(ctx, SMG_UNSUPPORTED, "scale on F16 field");
    count_launch(ctx);
    SMG_CHECK_LAUNCH(ctx);
    SMG_CUDA(ctx, cudaFreeAsync(dev, ctx->stream));
    return SMG_OK;
}

}  // extern "C"
