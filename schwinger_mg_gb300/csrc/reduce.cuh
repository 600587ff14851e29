// Two-stage block reductions with a "last block finalises" epilogue.
//
// Kernels that reduce run with blockDim = (lanes, rows), lanes a power of two
// <= 32 indexing right-hand sides, at most 256 threads per block.  Every
// thread contributes K doubles; the block sums them per lane (warp shuffles,
// then across warps), writes one partial per (rhs, k), and the block that
// finishes last sums the partials in a fixed order (deterministic run to run)
// and hands the totals to a finaliser functor `fin(rhs, const double* sums)`.
// Partials live in the context's scratch buffer:
//   partials[(rhs * K + k) * gridDim.x + blockIdx.x]
// and ticket[blockIdx.y] counts finished blocks; the last block puts it back
// to zero, so the scratch is ready for the next launch on the same stream.
#pragma once
#include "smg_internal.h"

constexpr int kReduceMaxThreads = 256;

struct FinStore {
    double* out;  // out[rhs * K + k] = total
    int K;
    __device__ void operator()(int rhs, const double* s) const {
        for (int k = 0; k < K; ++k) out[rhs * K + k] = s[k];
    }
};

template <int K, typename Fin>
__device__ __forceinline__ void block_reduce_finalise(double (&v)[K], double* __restrict__ partials,
                                                      unsigned int* __restrict__ ticket, int nrhs,
                                                      const Fin& fin) {
    __shared__ double s_rows[K][kReduceMaxThreads / 32][32];
    __shared__ double s_fin[K][32];
    __shared__ int s_last;

    const int lanes = blockDim.x;
    const int t = threadIdx.y * lanes + threadIdx.x;
    const int lane_id = t & 31;
    const int warp = t >> 5;
    const int nwarps = (blockDim.x * blockDim.y + 31) >> 5;
    const int rhs0 = blockIdx.y * lanes;

    // within a warp, lanes sharing threadIdx.x differ by multiples of `lanes`
#pragma unroll
    for (int k = 0; k < K; ++k) {
        double a = v[k];
        for (int off = 16; off >= lanes; off >>= 1) a += __shfl_xor_sync(0xffffffffu, a, off);
        v[k] = a;
    }
    if (lane_id < lanes) {
#pragma unroll
        for (int k = 0; k < K; ++k) s_rows[k][warp][lane_id] = v[k];
    }
    __syncthreads();
    if (t < lanes && rhs0 + t < nrhs) {
#pragma unroll
        for (int k = 0; k < K; ++k) {
            double a = 0.0;
            for (int w = 0; w < nwarps; ++w) a += s_rows[k][w][t];
            partials[((size_t)(rhs0 + t) * K + k) * gridDim.x + blockIdx.x] = a;
        }
        __threadfence();  // this thread's partials are visible before the block takes its ticket
    }
    __syncthreads();
    if (t == 0) {
        unsigned int prev = atomicAdd(ticket + blockIdx.y, 1u);
        s_last = (prev == gridDim.x - 1) ? 1 : 0;
    }
    __syncthreads();
    if (!s_last) return;
    __threadfence();
    // last block: with at most one (lane, k) pair per warp, one warp per pair with eight loads per
    // lane in flight (the short tail of few right-hand sides); otherwise each warp sums four pairs
    // at once with four blocks per pair in flight (16 independent loads per lane); fixed order,
    // deterministic
    const int npairs = lanes * K;
    const int nb = (int)gridDim.x;
    if (npairs <= nwarps) {
        if (warp < npairs) {
            const int l = warp / K, k = warp - l * K;
            double a = 0.0;
            if (rhs0 + l < nrhs) {
                const double* src = partials + ((size_t)(rhs0 + l) * K + k) * nb;
                double acc[8] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
                int b = lane_id;
                for (; b + 7 * 32 < nb; b += 8 * 32) {
#pragma unroll
                    for (int u = 0; u < 8; ++u) acc[u] += __ldcg(src + b + u * 32);
                }
#pragma unroll
                for (int u = 0; u < 8; ++u)
                    if (b + u * 32 < nb) acc[u] += __ldcg(src + b + u * 32);
                a = ((acc[0] + acc[1]) + (acc[2] + acc[3])) + ((acc[4] + acc[5]) + (acc[6] + acc[7]));
            }
            for (int off = 16; off >= 1; off >>= 1) a += __shfl_xor_sync(0xffffffffu, a, off);
            if (lane_id == 0) s_fin[k][l] = a;
        }
        __syncthreads();
        if (t < lanes && rhs0 + t < nrhs) {
            double sums[K];
#pragma unroll
            for (int k = 0; k < K; ++k) sums[k] = s_fin[k][t];
            fin(rhs0 + t, sums);
        }
        if (t == 0) ticket[blockIdx.y] = 0u;
        return;
    }
    for (int p0 = warp * 4; p0 < npairs; p0 += nwarps * 4) {
        const double* src[4];
        bool live[4];
        double acc[4][4];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const int p = p0 + q < npairs ? p0 + q : npairs - 1;
            const int l = p / K, k = p - l * K;
            live[q] = p0 + q < npairs && rhs0 + l < nrhs;
            src[q] = partials + ((size_t)(rhs0 + l) * K + k) * nb;
#pragma unroll
            for (int u = 0; u < 4; ++u) acc[q][u] = 0.0;
        }
        int b = lane_id;
        for (; b + 3 * 32 < nb; b += 4 * 32) {
#pragma unroll
            for (int q = 0; q < 4; ++q)
#pragma unroll
                for (int u = 0; u < 4; ++u)
                    if (live[q]) acc[q][u] += __ldcg(src[q] + b + u * 32);
        }
#pragma unroll
        for (int q = 0; q < 4; ++q)
#pragma unroll
            for (int u = 0; u < 4; ++u)
                if (live[q] && b + u * 32 < nb) acc[q][u] += __ldcg(src[q] + b + u * 32);
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            double a = (acc[q][0] + acc[q][1]) + (acc[q][2] + acc[q][3]);
            for (int off = 16; off >= 1; off >>= 1) a += __shfl_xor_sync(0xffffffffu, a, off);
            const int p = p0 + q, l = p / K, k = p - l * K;
            if (lane_id == 0 && p < npairs) s_fin[k][l] = live[q] ? a : 0.0;
        }
    }
    __syncthreads();
    if (t < lanes && rhs0 + t < nrhs) {
        double sums[K];
#pragma unroll
        for (int k = 0; k < K; ++k) sums[k] = s_fin[k][t];
        fin(rhs0 + t, sums);
    }
    if (t == 0) ticket[blockIdx.y] = 0u;
}

// First stage only: the block's partial per (rhs, k) into partials[(rhs * K + k) * gridDim.x + blockIdx.x],
// for a separate kernel to sum (k_sum_partials below) when a single finishing block would be slow.
template <int K, typename T>
__device__ __forceinline__ void block_partials(const T (&vin)[K], double* __restrict__ partials, int nrhs) {
    __shared__ double s_rows[K][kReduceMaxThreads / 32][32];
    const int lanes = blockDim.x;
    const int t = threadIdx.y * lanes + threadIdx.x;
    const int lane_id = t & 31, warp = t >> 5;
    const int nwarps = (blockDim.x * blockDim.y + 31) >> 5;
    const int rhs0 = blockIdx.y * lanes;
#pragma unroll
    for (int k = 0; k < K; ++k) {
        double a = (double)vin[k];
        for (int off = 16; off >= lanes; off >>= 1) a += __shfl_xor_sync(0xffffffffu, a, off);
        if (lane_id < lanes) s_rows[k][warp][lane_id] = a;
    }
    __syncthreads();
    if (t < lanes && rhs0 + t < nrhs) {
#pragma unroll
        for (int k = 0; k < K; ++k) {
            double a = 0.0;
            for (int w = 0; w < nwarps; ++w) a += s_rows[k][w][t];
            partials[((size_t)(rhs0 + t) * K + k) * gridDim.x + blockIdx.x] = a;
        }
    }
}

// Second stage: one warp per (rhs, k < nk) sums the nb block partials of block_partials<K> (lanes stride
// the blocks, eight loads in flight per lane, then a fixed shuffle tree: deterministic) into
// out[rhs * stride + k].  Launch with nrhs * nk warps.
static __global__ void __launch_bounds__(256) k_sum_partials(const double* __restrict__ partials, int nb, int nrhs, int K,
                                                      int nk, double* __restrict__ out, int stride) {
    const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (w >= nrhs * nk) return;
    const int rhs = w / nk, k = w - rhs * nk;
    const double* src = partials + ((size_t)rhs * K + k) * nb;
    double acc[8] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
    for (int b0 = 0; b0 < nb; b0 += 8 * 32) {
#pragma unroll
        for (int u = 0; u < 8; ++u) {
            const int b = b0 + u * 32 + lane;
            if (b < nb) acc[u] += __ldcg(src + b);
        }
    }
    double a = ((acc[0] + acc[1]) + (acc[2] + acc[3])) + ((acc[4] + acc[5]) + (acc[6] + acc[7]));
    for (int off = 16; off >= 1; off >>= 1) a += __shfl_xor_sync(0xffffffffu, a, off);
    if (lane == 0) out[rhs * stride + k] = a;
}

// FP32 per-thread partials: widened to FP64 once per thread, then reduced as above.
template <int K, typename Fin>
__device__ __forceinline__ void block_reduce_finalise(float (&v)[K], double* __restrict__ partials,
                                                      unsigned int* __restrict__ ticket, int nrhs, const Fin& fin) {
    double d[K];
#pragma unroll
    for (int k = 0; k < K; ++k) d[k] = (double)v[k];
    block_reduce_finalise<K>(d, partials, ticket, nrhs, fin);
}

// Launch shape for reducing kernels: lanes is a power of two <= 32, at most
// kReduceResidentBlocks blocks in all (kernels stride over the remaining sites).
constexpr int kReduceResidentBlocks = 152 * 4;
struct ReduceLaunch {
    dim3 grid, block;
    int lanes, rows;
};
inline ReduceLaunch reduce_launch(int nsites, int nrhs) {
    ReduceLaunch s;
    int lanes = 1;
    while (lanes * 2 <= nrhs && lanes < 32) lanes *= 2;
    s.lanes = lanes;
    s.rows = kReduceMaxThreads / lanes;
    const int by = (nrhs + lanes - 1) / lanes;
    // every block resident at once: the reducing kernels use 40-64 registers, so 4 blocks of
    // 256 threads per SM; more blocks would run as a second, partial wave
    const int cap = kReduceResidentBlocks / by > 0 ? kReduceResidentBlocks / by : 1;
    int bx = (nsites + s.rows - 1) / s.rows;
    if (bx > cap) bx = cap;
    if (bx < 1) bx = 1;
    s.block = dim3(lanes, s.rows, 1);
    s.grid = dim3(bx, by, 1);
    return s;
}
