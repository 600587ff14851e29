// Internal definitions shared by the CUDA translation units of libsmg_gpu.
//
// Device data layout (all precisions):
//   site index   q = parity * Vh + cb, with cb = (x + L*y) / 2 for even L;
//                cb equals the reference's eo_index (src/lattice.h:28-41)
//   spinor       ((q * nrhs + rhs) * 2 + spin)  complex     -> both spin
//                components of one (site, rhs) are one 16-byte (FP32) or
//                32-byte (FP64) vector, and the RHS lanes of a warp read
//                consecutive vectors while sharing one link load
//   links        U[(mu * 2 + parity) * Vh + cb] complex
//   clover       C[q] = 0.5 * c_sw * F01 real (the diagonal shift of
//                src/dirac.h:102)
//   F16 fields   data as __half2 per complex, plus one float scale per
//                (site, rhs) covering both spin components
#pragma once

#include <cuda_runtime.h>
#include <cuda_fp16.h>
#include <cstdint>
#include <cstdio>
#include <string>
#include <vector>
#include <mutex>

#include "../../include/smg_gpu.h"

// ------------------------------------------------------------ complex type
template <typename T>
struct alignas(2 * sizeof(T)) cx {
    T re, im;
};

template <typename T>
__host__ __device__ __forceinline__ cx<T> mk(T a, T b) { cx<T> z; z.re = a; z.im = b; return z; }
template <typename T>
__host__ __device__ __forceinline__ cx<T> operator+(cx<T> a, cx<T> b) { return mk(a.re + b.re, a.im + b.im); }
template <typename T>
__host__ __device__ __forceinline__ cx<T> operator-(cx<T> a, cx<T> b) { return mk(a.re - b.re, a.im - b.im); }
template <typename T>
__host__ __device__ __forceinline__ cx<T> operator-(cx<T> a) { return mk(-a.re, -a.im); }
template <typename T>
__host__ __device__ __forceinline__ cx<T> operator*(cx<T> a, cx<T> b) {
    return mk(a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re);
}
template <typename T>
__host__ __device__ __forceinline__ cx<T> operator*(T s, cx<T> a) { return mk(s * a.re, s * a.im); }
template <typename T>
__host__ __device__ __forceinline__ cx<T> conj(cx<T> a) { return mk(a.re, -a.im); }
// conj(a) * b
template <typename T>
__host__ __device__ __forceinline__ cx<T> cmulc(cx<T> a, cx<T> b) {
    return mk(a.re * b.re + a.im * b.im, a.re * b.im - a.im * b.re);
}
// i * a
template <typename T>
__host__ __device__ __forceinline__ cx<T> times_i(cx<T> a) { return mk(-a.im, a.re); }
template <typename T>
__host__ __device__ __forceinline__ T norm2(cx<T> a) { return a.re * a.re + a.im * a.im; }

template <typename D, typename S>
__host__ __device__ __forceinline__ cx<D> cvt(cx<S> a) { return mk<D>((D)a.re, (D)a.im); }

// spinor element index: site q, right-hand side rhs, spin sp (spin innermost)
__host__ __device__ __forceinline__ int64_t sidx(int64_t q, int rhs, int sp, int nrhs) {
    return (q * nrhs + rhs) * 2 + sp;
}

// both spin components of one (site, rhs), loaded and stored as one vector
template <typename T>
struct alignas(4 * sizeof(T)) Spinor {
    cx<T> s0, s1;
};
template <typename T>
__device__ __forceinline__ Spinor<T> ld_spinor(const cx<T>* __restrict__ f, int64_t q, int rhs, int nrhs) {
    return reinterpret_cast<const Spinor<T>*>(f)[q * nrhs + rhs];
}
template <typename T>
__device__ __forceinline__ void st_spinor(cx<T>* __restrict__ f, int64_t q, int rhs, int nrhs, Spinor<T> v) {
    reinterpret_cast<Spinor<T>*>(f)[q * nrhs + rhs] = v;
}

// ------------------------------------------------------------ lattice geometry
struct Geom {
    int L, Lh, V, Vh;
};

__host__ __device__ __forceinline__ void site_coords(const Geom& g, int q, int& x, int& y, int& parity) {
    parity = q >= g.Vh ? 1 : 0;
    int cb = q - parity * g.Vh;
    y = cb / g.Lh;
    int xh = cb - y * g.Lh;
    x = 2 * xh + ((y + parity) & 1);
}
// device index q of the lexicographic site (x, y), coordinates already in range
__host__ __device__ __forceinline__ int site_q(const Geom& g, int x, int y) {
    int parity = (x + y) & 1;
    return parity * g.Vh + ((x + g.L * y) >> 1);
}
__host__ __device__ __forceinline__ int wrap(int a, int L) {
    return a < 0 ? a + L : (a >= L ? a - L : a);
}

// ------------------------------------------------------------ error handling
struct SmgError {
    smg_status status;
    std::string msg;
};

#define SMG_CUDA(ctx, call)                                                        \
    do {                                                                           \
        cudaError_t e__ = (call);                                                  \
        if (e__ != cudaSuccess) {                                                  \
            return smg_fail((ctx), e__ == cudaErrorMemoryAllocation ? SMG_NO_MEMORY \
                                                                   : SMG_DEVICE_ERROR, \
                            std::string(#call) + ": " + cudaGetErrorString(e__));  \
        }                                                                          \
    } while (0)

#define SMG_CHECK_LAUNCH(ctx)                                                      \
    do {                                                                           \
        cudaError_t e__ = cudaGetLastError();                                      \
        if (e__ != cudaSuccess)                                                    \
            return smg_fail((ctx), SMG_DEVICE_ERROR,                               \
                            std::string("kernel launch: ") + cudaGetErrorString(e__)); \
    } while (0)

#define SMG_TRY(call)                                                              \
    do {                                                                           \
        smg_status s__ = (call);                                                   \
        if (s__ != SMG_OK) return s__;                                             \
    } while (0)

// ------------------------------------------------------------ reduction scratch
// Per-context scratch for the two-stage reductions: per-block partial sums and
// one ticket counter per reduction slot ("last block finalises" pattern).
struct ReduceScratch {
    double* partials = nullptr;     // capacity doubles
    size_t capacity = 0;
    unsigned int* tickets = nullptr;  // kMaxTickets counters, kept at zero between launches
};
constexpr int kMaxTickets = 64;
constexpr int kMaxReduceBlocks = 1216;  // 152 SMs x 8

// ------------------------------------------------------------ objects
struct smg_context {
    int device = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    std::string last_error;
    uint64_t launches = 0;
    ReduceScratch red;
    double* host_stage = nullptr;   // pinned staging for scalar read-backs
    size_t host_stage_bytes = 0;
    int num_sms = 0;
    cudaEvent_t ev_begin = nullptr, ev_end = nullptr;
    // reduction buffers replaced by a larger one stay allocated until the
    // context is destroyed: a captured CUDA graph may still reference them
    std::vector<double*> retired;
    // stencil launch shape chosen by timing per (L, nrhs, precision): key -> variant
    std::vector<std::pair<uint64_t, int>> dslash_plans;
    // device memory of finished solves, kept for the next solve on this context and freed with it:
    // work fields by (L, nrhs, precision) and scalar buffers by size (stream order makes reuse safe)
    std::vector<smg_field*> field_pool;
    std::vector<std::pair<size_t, void*>> buf_pool;
};

struct smg_gauge {
    smg_context* ctx = nullptr;
    Geom g{};
    cx<double>* U64 = nullptr;  // [mu][parity][cb]
    cx<float>* U32 = nullptr;
};

// A Dirac handle reads its gauge handle's links at every apply, so the gauge
// must outlive it; destroying the Dirac handle touches only its own memory
// and context.
struct smg_dirac {
    smg_context* ctx = nullptr;
    smg_gauge* gauge = nullptr;
    double mass = 0, r = 1, c_sw = 0, mu_t = 0;
    double* C64 = nullptr;  // 0.5 * c_sw * F01 per device site (nullptr when c_sw == 0)
    float* C32 = nullptr;
    double* F01 = nullptr;  // F01 itself per device site
};

struct smg_field {
    smg_context* ctx = nullptr;
    Geom g{};
    int nrhs = 1;
    smg_precision prec = SMG_F64;
    void* data = nullptr;
    float* scale = nullptr;  // F16 only: one per site (largest component over its RHS)
    size_t bytes = 0;
    int64_t n_complex() const { return (int64_t)g.V * 2 * nrhs; }
};

// ------------------------------------------------------------ helpers
smg_status smg_fail(smg_context* ctx, smg_status s, const std::string& msg);
smg_status smg_reduce_reserve(smg_context* ctx, size_t doubles);
smg_status smg_host_stage_reserve(smg_context* ctx, size_t bytes);
inline void count_launch(smg_context* ctx, int n = 1) { ctx->launches += (uint64_t)n; }

// Launch shape for per-(site, rhs) kernels: x = rhs lanes, y = site rows.
struct SiteLaunch {
    dim3 grid, block;
    int rows;   // sites per block
    int lanes;  // rhs per block
};
inline SiteLaunch site_launch(int nsites, int nrhs, int threads = 256) {
    SiteLaunch s;
    s.lanes = nrhs < 32 ? nrhs : 32;
    s.rows = threads / s.lanes;
    if (s.rows < 1) s.rows = 1;
    s.block = dim3(s.lanes, s.rows, 1);
    s.grid = dim3((nsites + s.rows - 1) / s.rows, (nrhs + s.lanes - 1) / s.lanes, 1);
    return s;
}

// Internal entry points shared between translation units.
smg_status smg_dirac_apply_internal(smg_dirac* d, smg_operator op, const smg_field* src,
                                    smg_field* dst, double* norm2_out_dev);
smg_status smg_field_check_pair(const smg_field* a, const smg_field* b);
smg_status smg_field_alloc_like(const smg_field* proto, smg_precision prec, smg_field** out);
// a work field like proto in precision prec from the context's pool (allocated when none is free),
// and its return to the pool
smg_status smg_field_take(const smg_field* proto, smg_precision prec, smg_field** out);
void smg_field_give(smg_field* f);
// a device buffer of `bytes` from the context's pool, and its return
smg_status smg_buf_take(smg_context* ctx, size_t bytes, void** out);
void smg_buf_give(smg_context* ctx, size_t bytes, void* p);
smg_status smg_gauge_ensure_f32(smg_gauge* g);
