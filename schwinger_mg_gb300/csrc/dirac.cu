// Wilson-clover Dirac operator on the device (reference src/dirac.h:8-183).
//
// One kernel applies D or D^dag to every right-hand side of a field:
//   D = (2r + m) + C(x) sigma3 + i mu sigma3
//       - 1/2 sum_mu [ (r - sigma_mu) U_mu(x) delta_{x+mu} + (r + sigma_mu) U_mu^dag(x-mu) delta_{x-mu} ]
// with sigma_0 -> sigma1, sigma_1 -> sigma2 as in accumulate_hops
// (dirac.h:58-89) and C = c_sw F01 / 2 (dirac.h:102).  D^dag = g5 D(-mu) g5
// (dirac.h:120-134) only flips the sign of the spin off-diagonal hopping
// terms and of mu, so it is the same kernel with DAG = true.  Optional
// epilogues fuse the reductions a solver step needs: ||out||^2 (CG's
// <p, D^dag D p> = ||D p||^2) and, for the MR smoother, <out, w> and ||out||^2.
#include "smg_internal.h"
#include "reduce.cuh"
#include "half.cuh"
#include "stencil.cuh"

#include <cstdlib>

namespace {

enum { EPI_NONE = 0, EPI_NORM = 1, EPI_MR = 2 };

template <typename T>
struct DslashArgs {
    const cx<T>* __restrict__ src = nullptr;
    cx<T>* __restrict__ dst = nullptr;
    const cx<T>* __restrict__ U = nullptr;  // [mu][parity][cb]
    const T* __restrict__ C = nullptr;      // clover shift per site or nullptr
    const cx<T>* __restrict__ w = nullptr;  // EPI_MR second field
    Geom g{};
    int nrhs = 1;
    int px = 0;  // EPI_NONE: 0 = a block walks one row; > 0 = a block is a px-wide patch of rows
    T diag = 0, mu_eff = 0, r = 0;
    double* partials = nullptr;
    unsigned int* ticket = nullptr;
    double* out = nullptr;
};

template <typename T, bool DAG, int EPI, bool R1>
__global__ void __launch_bounds__(256) k_dslash(DslashArgs<T> a) {
    constexpr int K = EPI == EPI_MR ? 3 : 1;
    const T half = T(0.5);
    const int nrhs = a.nrhs;
    const Geom g = a.g;
    T v[K];  // per-thread partials in the field precision (FP64 is scarce on this part)
#pragma unroll
    for (int k = 0; k < K; ++k) v[k] = T(0);

    // one (row y, position rem) work item: rem < L/2 even sites of the row, the rest odd sites
    auto site = [&](int y, int rem, int rhs) {
        const int p = rem >= g.Lh ? 1 : 0;
        const int xh = rem - p * g.Lh;
        const int x = 2 * xh + ((y + p) & 1);
        const int q = p * g.Vh + y * g.Lh + xh;
        const int op = (1 - p) * g.Vh;
        const int xp = x + 1 == g.L ? 0 : x + 1;
        const int xm = x == 0 ? g.L - 1 : x - 1;
        const int yp = y + 1 == g.L ? 0 : y + 1;
        const int ym = y == 0 ? g.L - 1 : y - 1;
        const int q_xp = op + ((xp + g.L * y) >> 1);
        const int q_xm = op + ((xm + g.L * y) >> 1);
        const int q_yp = op + ((x + g.L * yp) >> 1);
        const int q_ym = op + ((x + g.L * ym) >> 1);

        const cx<T> u0f = a.U[q];
        const cx<T> u0b = a.U[q_xm];
        const cx<T> u1f = a.U[g.V + q];
        const cx<T> u1b = a.U[g.V + q_ym];

        const Spinor<T> ps = ld_spinor(a.src, q, rhs, nrhs);
        const Spinor<T> pxp = ld_spinor(a.src, q_xp, rhs, nrhs);
        const Spinor<T> pxm = ld_spinor(a.src, q_xm, rhs, nrhs);
        const Spinor<T> pyp = ld_spinor(a.src, q_yp, rhs, nrhs);
        const Spinor<T> pym = ld_spinor(a.src, q_ym, rhs, nrhs);
        const cx<T> s0 = ps.s0, s1 = ps.s1;
        const T Cq = a.C ? a.C[q] : T(0);
        const cx<T> dg0 = mk<T>(a.diag + Cq, a.mu_eff);
        const cx<T> dg1 = mk<T>(a.diag - Cq, -a.mu_eff);
        cx<T> S0, S1;
        hop_sum<T, DAG, R1>(u0f, u0b, u1f, u1b, pxp, pxm, pyp, pym, a.r, S0, S1);
        const cx<T> d0 = dg0 * s0 - half * S0;
        const cx<T> d1 = dg1 * s1 - half * S1;
        Spinor<T> out;
        out.s0 = d0;
        out.s1 = d1;
        st_spinor(a.dst, q, rhs, nrhs, out);

        if (EPI == EPI_NORM) {
            v[0] += norm2(d0) + norm2(d1);
        } else if (EPI == EPI_MR) {
            const Spinor<T> wv = ld_spinor(a.w, q, rhs, nrhs);
            const cx<T> c = cmulc(d0, wv.s0) + cmulc(d1, wv.s1);
            v[0] += c.re;
            v[1] += c.im;
            v[2] += norm2(d0) + norm2(d1);
        }
    };

    if (EPI == EPI_NONE) {
        const int rhs = blockIdx.z * blockDim.x + threadIdx.x;
        if (a.px == 0) {
            // one item per thread: row = blockIdx.y, no index division
            const int rem = blockIdx.x * blockDim.y + threadIdx.y;
            if (rhs < nrhs && rem < g.L) site(blockIdx.y, rem, rhs);
        } else {
            // a block is a patch of px columns x (blockDim.y / px) rows holding both parities, so the
            // x and y neighbours of most of its sites are sites of the same block (L1 hits)
            const int x = blockIdx.x * a.px + (int)threadIdx.y % a.px;
            const int y = blockIdx.y * ((int)blockDim.y / a.px) + (int)threadIdx.y / a.px;
            const int p = (x + y) & 1;
            if (rhs < nrhs) site(y, p * g.Lh + (x >> 1), rhs);
        }
    } else {
        const int rhs = blockIdx.y * blockDim.x + threadIdx.x;
        if (rhs < nrhs) {
            // Work items walk rows with both parities interleaved (row y even
            // sites, row y odd sites, row y+1, ...), so the neighbour rows a
            // block reads were read moments ago by its predecessors and are still
            // in L2; walking all even sites before all odd ones streams every
            // spinor from DRAM twice once the field outgrows L2.
            for (int w = blockIdx.x * blockDim.y + threadIdx.y; w < g.V; w += gridDim.x * blockDim.y) {
                const int y = w / g.L;
                site(y, w - y * g.L, rhs);
            }
        }
    }
    if (EPI != EPI_NONE) block_reduce_finalise<K>(v, a.partials, a.ticket, nrhs, FinStore{a.out, K});
}

// ---------------------------------------------------------------- two RHS per thread
//
// The row kernel with every thread owning right-hand sides rhs and rhs + lanes (lanes = nrhs / 2):
// the index arithmetic and the link and clover loads of a site are shared by two right-hand sides,
// and each spinor load of a warp still covers 2 x lanes consecutive 16-byte vectors.
template <typename T, bool DAG>
__global__ void __launch_bounds__(256) k_dslash_r2(DslashArgs<T> a) {
    const T half = T(0.5);
    const Geom g = a.g;
    const int nrhs = a.nrhs, lanes = blockDim.x;
    const int rhs = threadIdx.x;
    const int rem = blockIdx.x * blockDim.y + threadIdx.y;
    const int y = blockIdx.y;
    if (rem >= g.L) return;
    const int p = rem >= g.Lh ? 1 : 0;
    const int xh = rem - p * g.Lh;
    const int x = 2 * xh + ((y + p) & 1);
    const int q = p * g.Vh + y * g.Lh + xh;
    const int op = (1 - p) * g.Vh;
    const int xp = x + 1 == g.L ? 0 : x + 1, xm = x == 0 ? g.L - 1 : x - 1;
    const int yp = y + 1 == g.L ? 0 : y + 1, ym = y == 0 ? g.L - 1 : y - 1;
    const int q_xp = op + ((xp + g.L * y) >> 1), q_xm = op + ((xm + g.L * y) >> 1);
    const int q_yp = op + ((x + g.L * yp) >> 1), q_ym = op + ((x + g.L * ym) >> 1);
    const cx<T> u0f = a.U[q], u0b = a.U[q_xm], u1f = a.U[g.V + q], u1b = a.U[g.V + q_ym];
    const T Cq = a.C ? a.C[q] : T(0);
    const cx<T> dg0 = mk<T>(a.diag + Cq, a.mu_eff), dg1 = mk<T>(a.diag - Cq, -a.mu_eff);
    Spinor<T> ps[2], pxp[2], pxm[2], pyp[2], pym[2];
#pragma unroll
    for (int k = 0; k < 2; ++k) {  // every load of both right-hand sides issued first
        const int rr = rhs + k * lanes;
        ps[k] = ld_spinor(a.src, q, rr, nrhs);
        pxp[k] = ld_spinor(a.src, q_xp, rr, nrhs);
        pxm[k] = ld_spinor(a.src, q_xm, rr, nrhs);
        pyp[k] = ld_spinor(a.src, q_yp, rr, nrhs);
        pym[k] = ld_spinor(a.src, q_ym, rr, nrhs);
    }
#pragma unroll
    for (int k = 0; k < 2; ++k) {
        cx<T> S0, S1;
        hop_sum<T, DAG, false>(u0f, u0b, u1f, u1b, pxp[k], pxm[k], pyp[k], pym[k], a.r, S0, S1);
        Spinor<T> o;
        o.s0 = dg0 * ps[k].s0 - half * S0;
        o.s1 = dg1 * ps[k].s1 - half * S1;
        st_spinor(a.dst, q, rhs + k * lanes, nrhs, o);
    }
}

// ---------------------------------------------------------------- tiled stencil
//
// The same operator for a CTA tile of TY rows x 2*TXH columns (TXH sites of
// each parity per row).  Both parity planes of the tile plus a one-site halo
// are staged in shared memory with 16-byte cp.async copies (the halo wraps
// periodically, which a TMA tile load cannot express), so every spinor is read
// from L2 about (TY+2)(TXH+2)/(TY TXH) times instead of five times; links and
// the clover term are read directly (one value per site shared by all RHS
// lanes).  Shared memory holds [parity][TY+2][TXH+2][rhs] spinors.
constexpr int kTileXH = 8;

__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

template <typename T, bool DAG>
__global__ void __launch_bounds__(256) k_dslash_tile(DslashArgs<T> a, int TY) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    Spinor<T>* sp = reinterpret_cast<Spinor<T>*>(smem_raw);
    const Geom g = a.g;
    const int nrhs = a.nrhs;
    const int X0 = blockIdx.x * kTileXH, y0 = blockIdx.y * TY;
    const int RW = kTileXH + 2, RH = TY + 2;
    const int tid = threadIdx.y * blockDim.x + threadIdx.x, nthr = blockDim.x * blockDim.y;
    // stage: every 16-byte chunk of [parity][row][col] sites, each nrhs spinors
    {
        const int site_bytes = nrhs * (int)sizeof(Spinor<T>);
        const int chunks_per_site = site_bytes / 16;
        const int total = 2 * RH * RW * chunks_per_site;
        for (int c = tid; c < total; c += nthr) {
            const int k = c % chunks_per_site;
            const int site = c / chunks_per_site;
            const int col = site % RW, rest = site / RW;
            const int row = rest % RH, par = rest / RH;
            const int y = wrap(y0 - 1 + row, g.L);
            const int xh = wrap(X0 - 1 + col, g.Lh);
            const char* src = reinterpret_cast<const char*>(a.src) +
                              ((int64_t)(par * g.Vh + y * g.Lh + xh) * site_bytes) + 16 * k;
            cp_async16(smem_raw + (int64_t)site * site_bytes + 16 * k, src);
        }
        cp_async_wait_all();
        __syncthreads();
    }
    const T half = T(0.5);
    const int rhs = threadIdx.x;
    if (rhs >= nrhs) return;
    auto S = [&](int par, int row, int col) -> const Spinor<T>& {
        return sp[((par * RH + row) * RW + col) * nrhs + rhs];
    };
    for (int it = threadIdx.y; it < 2 * TY * kTileXH; it += blockDim.y) {
        const int c = it % kTileXH, rest = it / kTileXH;
        const int r = rest % TY, p = rest / TY;
        const int y = y0 + r, xh = X0 + c;
        const int b = (y + p) & 1;
        const int x = 2 * xh + b;
        const int q = p * g.Vh + y * g.Lh + xh;
        const int op = 1 - p;
        const int xm = x == 0 ? g.L - 1 : x - 1;
        const int ym = y == 0 ? g.L - 1 : y - 1;
        const int q_xm = op * g.Vh + ((xm + g.L * y) >> 1);
        const int q_ym = op * g.Vh + ((x + g.L * ym) >> 1);
        const cx<T> u0f = a.U[q], u0b = a.U[q_xm];
        const cx<T> u1f = a.U[g.V + q], u1b = a.U[g.V + q_ym];
        const Spinor<T> ps = S(p, r + 1, c + 1);
        const Spinor<T> pxp = S(op, r + 1, c + 1 + b);
        const Spinor<T> pxm = S(op, r + 1, c + b);
        const Spinor<T> pyp = S(op, r + 2, c + 1);
        const Spinor<T> pym = S(op, r, c + 1);
        const T Cq = a.C ? a.C[q] : T(0);
        const cx<T> dg0 = mk<T>(a.diag + Cq, a.mu_eff);
        const cx<T> dg1 = mk<T>(a.diag - Cq, -a.mu_eff);
        cx<T> S0, S1;
        hop_sum<T, DAG, false>(u0f, u0b, u1f, u1b, pxp, pxm, pyp, pym, a.r, S0, S1);
        Spinor<T> o;
        o.s0 = dg0 * ps.s0 - half * S0;
        o.s1 = dg1 * ps.s1 - half * S1;
        st_spinor(a.dst, q, rhs, nrhs, o);
    }
}

// shared-memory bytes of a tile with TY rows
template <typename T>
size_t tile_smem(int TY, int nrhs) {
    return (size_t)2 * (TY + 2) * (kTileXH + 2) * nrhs * sizeof(Spinor<T>);
}

// ---------------------------------------------------------------- FP16 storage
//
// The row kernel with FP16 (per-site scaled) input and/or output fields and FP32
// arithmetic and links: the MG smoother's work vectors.  A thread owns NP pairs of
// adjacent right-hand sides of one site (2 NP consecutive two-spinors: one 16-byte
// load per pair and neighbour in FP16), a warp holds 32 / lanes sites of
// lanes = nrhs / (2 NP) threads, so an output site's scale is a shuffle reduction
// over its lane group.
struct DslashH {
    const cx<float>* __restrict__ src32 = nullptr;
    const __half2* __restrict__ src16 = nullptr;
    const float* __restrict__ src_scale = nullptr;
    cx<float>* __restrict__ dst32 = nullptr;
    __half2* __restrict__ dst16 = nullptr;
    float* __restrict__ dst_scale = nullptr;
    const cx<float>* __restrict__ U = nullptr;
    const float* __restrict__ C = nullptr;
    Geom g{};
    int nrhs = 1;
    float diag = 0, mu_eff = 0, r = 0;
    // NORM: ||out||^2 per block and rhs into part[(block * nrhs + rhs) * 2 + part_col]
    float* __restrict__ part = nullptr;
    int part_col = 0;
};

template <bool DAG, bool IN_H, bool OUT_H, bool R1, bool NORM, int NP>
__global__ void __launch_bounds__(256) k_dslash_h(DslashH a) {
    constexpr int NR = 2 * NP;
    const Geom g = a.g;
    const int nrhs = a.nrhs, lanes = blockDim.x;
    const int rhs0 = threadIdx.x * NR;
    const int rem = blockIdx.x * blockDim.y + threadIdx.y;
    const int y = blockIdx.y;
    const bool valid = rem < g.L;
    const int p = rem >= g.Lh ? 1 : 0;
    const int xh = rem - p * g.Lh;
    const int q = p * g.Vh + y * g.Lh + xh;
    Spinor<float> out[NR];
#pragma unroll
    for (int k = 0; k < NR; ++k) {
        out[k].s0 = mk(0.f, 0.f);
        out[k].s1 = mk(0.f, 0.f);
    }
    if (valid) {
        const int x = 2 * xh + ((y + p) & 1);
        const int op = (1 - p) * g.Vh;
        const int xp = x + 1 == g.L ? 0 : x + 1, xm = x == 0 ? g.L - 1 : x - 1;
        const int yp = y + 1 == g.L ? 0 : y + 1, ym = y == 0 ? g.L - 1 : y - 1;
        const int q_xp = op + ((xp + g.L * y) >> 1), q_xm = op + ((xm + g.L * y) >> 1);
        const int q_yp = op + ((x + g.L * yp) >> 1), q_ym = op + ((x + g.L * ym) >> 1);
        Spinor<float> ps[NR], pxp[NR], pxm[NR], pyp[NR], pym[NR];
        if (IN_H) {
            ld_pairs_h<NP>(a.src16, q, rhs0, nrhs, ps);
            ld_pairs_h<NP>(a.src16, q_xp, rhs0, nrhs, pxp);
            ld_pairs_h<NP>(a.src16, q_xm, rhs0, nrhs, pxm);
            ld_pairs_h<NP>(a.src16, q_yp, rhs0, nrhs, pyp);
            ld_pairs_h<NP>(a.src16, q_ym, rhs0, nrhs, pym);
        } else {
            ld_pairs_f<NP>(a.src32, q, rhs0, nrhs, ps);
            ld_pairs_f<NP>(a.src32, q_xp, rhs0, nrhs, pxp);
            ld_pairs_f<NP>(a.src32, q_xm, rhs0, nrhs, pxm);
            ld_pairs_f<NP>(a.src32, q_yp, rhs0, nrhs, pyp);
            ld_pairs_f<NP>(a.src32, q_ym, rhs0, nrhs, pym);
        }
        // FP16 input: the stored values are read unscaled and each neighbour's site scale is folded
        // into its link (and the centre's into the diagonal), the operator being linear in each; the
        // hopping term's 1/2 is folded into the links as well
        cx<float> u0f = a.U[q], u0b = a.U[q_xm], u1f = a.U[g.V + q], u1b = a.U[g.V + q_ym];
        const float Cq = a.C ? a.C[q] : 0.f;
        cx<float> dg0 = mk(a.diag + Cq, a.mu_eff), dg1 = mk(a.diag - Cq, -a.mu_eff);
        float hxp = 0.5f, hxm = 0.5f, hyp = 0.5f, hym = 0.5f;
        if (IN_H) {
            const float sq = a.src_scale[q];
            hxp *= a.src_scale[q_xp];
            hxm *= a.src_scale[q_xm];
            hyp *= a.src_scale[q_yp];
            hym *= a.src_scale[q_ym];
            dg0 = mk(dg0.re * sq, dg0.im * sq);
            dg1 = mk(dg1.re * sq, dg1.im * sq);
        }
        u0f = mk(u0f.re * hxp, u0f.im * hxp);
        u0b = mk(u0b.re * hxm, u0b.im * hxm);
        u1f = mk(u1f.re * hyp, u1f.im * hyp);
        u1b = mk(u1b.re * hym, u1b.im * hym);
#pragma unroll
        for (int k = 0; k < NR; ++k) {
            cx<float> S0, S1;
            hop_sum<float, DAG, R1>(u0f, u0b, u1f, u1b, pxp[k], pxm[k], pyp[k], pym[k], a.r, S0, S1);
            out[k].s0 = dg0 * ps[k].s0 - S0;
            out[k].s1 = dg1 * ps[k].s1 - S1;
        }
    }
    if (NORM) {
        // ||out||^2 of this block's sites per rhs: the rows of a warp by shuffles, the warps in shared memory
        __shared__ float s_n[8][32];
        float v[NR];
#pragma unroll
        for (int k = 0; k < NR; ++k) v[k] = valid ? norm2(out[k].s0) + norm2(out[k].s1) : 0.f;
#pragma unroll
        for (int k = 0; k < NR; ++k)
            for (int o = lanes; o < 32; o <<= 1) v[k] += __shfl_xor_sync(0xffffffffu, v[k], o);
        const int warp = (threadIdx.y * lanes + threadIdx.x) >> 5, nw = (blockDim.y * lanes) >> 5;
        if (((threadIdx.y * lanes) & 31) == 0) {  // the first row of each warp
#pragma unroll
            for (int k = 0; k < NR; ++k) s_n[warp][rhs0 + k] = v[k];
        }
        __syncthreads();
        if (threadIdx.y == 0) {
            float* pp = a.part + ((int64_t)blockIdx.y * gridDim.x + blockIdx.x) * nrhs * 2 + a.part_col;
#pragma unroll
            for (int k = 0; k < NR; ++k) {
                float t = 0.f;
                for (int w = 0; w < nw; ++w) t += s_n[w][rhs0 + k];
                pp[2 * (rhs0 + k)] = t;
            }
        }
    }
    if (OUT_H) {
        st_pairs_h<NP>(a.dst16, a.dst_scale, q, rhs0, nrhs, lanes, out, valid);
    } else if (valid) {
        float4* pd = reinterpret_cast<float4*>(a.dst32) + ((int64_t)q * nrhs + rhs0);
#pragma unroll
        for (int k = 0; k < NR; ++k) pd[k] = make_float4(out[k].s0.re, out[k].s0.im, out[k].s1.re, out[k].s1.im);
    }
}

// The MG smoother's FP16 -> FP16 stencil in its one production shape: 32 right-hand sides in two
// pairs per thread (8 threads per site, compile-time lane groups), r = 1, no twisted mass.  The spin
// projections of the four neighbours are formed on the packed FP16 pairs before conversion (one
// packed add, or a half swap and a packed fma for the +-i sigma_2 hops, where the generic kernel
// converts both spin components and adds in FP32); the extra rounding of that sum is of the size of
// the fields' own FP16 storage error.  The diagonal is real (the centre's site scale folded in).
__device__ __forceinline__ __half2 h2_of(unsigned u) { return *reinterpret_cast<const __half2*>(&u); }
__device__ __forceinline__ cx<float> cx_of(__half2 h) {
    const float2 f = __half22float2(h);
    return mk(f.x, f.y);
}
// s0 + s1, s0 - s1, s0 + i s1, s0 - i s1 on (re, im) FP16 pairs
__device__ __forceinline__ __half2 proj_add(__half2 s0, __half2 s1) { return __hadd2(s0, s1); }
__device__ __forceinline__ __half2 proj_sub(__half2 s0, __half2 s1) { return __hsub2(s0, s1); }
__device__ __forceinline__ __half2 proj_addi(__half2 s0, __half2 s1) {
    return __hfma2(__lowhigh2highlow(s1), __floats2half2_rn(-1.f, 1.f), s0);
}
__device__ __forceinline__ __half2 proj_subi(__half2 s0, __half2 s1) {
    return __hfma2(__lowhigh2highlow(s1), __floats2half2_rn(1.f, -1.f), s0);
}

template <bool DAG, bool NORM>
__global__ void __launch_bounds__(256) k_dslash_h32(DslashH a) {
    constexpr int NP = 2, NR = 4, LANES = 8, NRHS = 32;
    const Geom g = a.g;
    const int rhs0 = threadIdx.x * NR;
    const int rem = blockIdx.x * blockDim.y + threadIdx.y;
    const int y = blockIdx.y;
    const bool valid = rem < g.L;
    const int p = rem >= g.Lh ? 1 : 0;
    const int xh = rem - p * g.Lh;
    const int q = p * g.Vh + y * g.Lh + xh;
    Spinor<float> out[NR];
#pragma unroll
    for (int k = 0; k < NR; ++k) {
        out[k].s0 = mk(0.f, 0.f);
        out[k].s1 = mk(0.f, 0.f);
    }
    if (valid) {
        const int x = 2 * xh + ((y + p) & 1);
        const int op = (1 - p) * g.Vh;
        const int xp = x + 1 == g.L ? 0 : x + 1, xm = x == 0 ? g.L - 1 : x - 1;
        const int yp = y + 1 == g.L ? 0 : y + 1, ym = y == 0 ? g.L - 1 : y - 1;
        const int q_xp = op + ((xp + g.L * y) >> 1), q_xm = op + ((xm + g.L * y) >> 1);
        const int q_yp = op + ((x + g.L * yp) >> 1), q_ym = op + ((x + g.L * ym) >> 1);
        // a site's 32 two-spinors are 16 uint4 (one pair each); this thread's pairs 2 tx, 2 tx + 1
        const uint4* __restrict__ f = reinterpret_cast<const uint4*>(a.src16) + 2 * threadIdx.x;
        uint4 vc[NP], vxp[NP], vxm[NP], vyp[NP], vym[NP];
#pragma unroll
        for (int k = 0; k < NP; ++k) {
            vc[k] = __ldg(f + (int64_t)q * (NRHS / 2) + k);
            vxp[k] = __ldg(f + (int64_t)q_xp * (NRHS / 2) + k);
            vxm[k] = __ldg(f + (int64_t)q_xm * (NRHS / 2) + k);
            vyp[k] = __ldg(f + (int64_t)q_yp * (NRHS / 2) + k);
            vym[k] = __ldg(f + (int64_t)q_ym * (NRHS / 2) + k);
        }
        cx<float> u0f = a.U[q], u0b = a.U[q_xm], u1f = a.U[g.V + q], u1b = a.U[g.V + q_ym];
        const float Cq = a.C ? a.C[q] : 0.f;
        const float sq = a.src_scale[q];
        const float dg0 = (a.diag + Cq) * sq, dg1 = (a.diag - Cq) * sq;
        const float hxp = 0.5f * a.src_scale[q_xp], hxm = 0.5f * a.src_scale[q_xm];
        const float hyp = 0.5f * a.src_scale[q_yp], hym = 0.5f * a.src_scale[q_ym];
        u0f = mk(u0f.re * hxp, u0f.im * hxp);
        u0b = mk(u0b.re * hxm, u0b.im * hxm);
        u1f = mk(u1f.re * hyp, u1f.im * hyp);
        u1b = mk(u1b.re * hym, u1b.im * hym);
#pragma unroll
        for (int k = 0; k < NR; ++k) {
            const int j = k >> 1;
            const bool hi = k & 1;  // second right-hand side of the pair: words z (s0) and w (s1)
            const unsigned c0 = hi ? vc[j].z : vc[j].x, c1 = hi ? vc[j].w : vc[j].y;
            const __half2 xp0 = h2_of(hi ? vxp[j].z : vxp[j].x), xp1 = h2_of(hi ? vxp[j].w : vxp[j].y);
            const __half2 xm0 = h2_of(hi ? vxm[j].z : vxm[j].x), xm1 = h2_of(hi ? vxm[j].w : vxm[j].y);
            const __half2 yp0 = h2_of(hi ? vyp[j].z : vyp[j].x), yp1 = h2_of(hi ? vyp[j].w : vyp[j].y);
            const __half2 ym0 = h2_of(hi ? vym[j].z : vym[j].x), ym1 = h2_of(hi ? vym[j].w : vym[j].y);
            const cx<float> hxf = cx_of(DAG ? proj_add(xp0, xp1) : proj_sub(xp0, xp1));
            const cx<float> hxb = cx_of(DAG ? proj_sub(xm0, xm1) : proj_add(xm0, xm1));
            const cx<float> hyf = cx_of(DAG ? proj_subi(yp0, yp1) : proj_addi(yp0, yp1));
            const cx<float> hyb = cx_of(DAG ? proj_addi(ym0, ym1) : proj_subi(ym0, ym1));
            cx<float> S0, S1;
            hop_recon<float, DAG>(u0f, u0b, u1f, u1b, hxf, hxb, hyf, hyb, S0, S1);
            const cx<float> p0 = cx_of(h2_of(c0)), p1 = cx_of(h2_of(c1));
            out[k].s0 = mk(fmaf(dg0, p0.re, -S0.re), fmaf(dg0, p0.im, -S0.im));
            out[k].s1 = mk(fmaf(dg1, p1.re, -S1.re), fmaf(dg1, p1.im, -S1.im));
        }
    }
    if (NORM) {
        // ||out||^2 of this block's sites per rhs: the four sites of a warp by shuffles, the eight
        // warps in shared memory
        __shared__ float s_n[8][32];
        float v[NR];
#pragma unroll
        for (int k = 0; k < NR; ++k) {
            v[k] = valid ? norm2(out[k].s0) + norm2(out[k].s1) : 0.f;
            v[k] += __shfl_xor_sync(0xffffffffu, v[k], 8);
            v[k] += __shfl_xor_sync(0xffffffffu, v[k], 16);
        }
        const int warp = threadIdx.y >> 2;
        if ((threadIdx.y & 3) == 0) {
#pragma unroll
            for (int k = 0; k < NR; ++k) s_n[warp][rhs0 + k] = v[k];
        }
        __syncthreads();
        if (threadIdx.y == 0) {
            float* pp = a.part + ((int64_t)blockIdx.y * gridDim.x + blockIdx.x) * NRHS * 2 + a.part_col;
#pragma unroll
            for (int k = 0; k < NR; ++k) {
                float t = 0.f;
#pragma unroll
                for (int w = 0; w < 8; ++w) t += s_n[w][rhs0 + k];
                pp[2 * (rhs0 + k)] = t;
            }
        }
    }
    st_pairs_h<NP>(a.dst16, a.dst_scale, q, rhs0, NRHS, LANES, out, valid);
}

// right-hand-side pairs per thread of the FP16 stencil launches: two (four right-hand sides share a
// site's index, link and scale work) from 8 right-hand sides up (L = 512, 32 RHS: D 55.3 against
// 57.4 us, D^dag with the fused norm 66.0 against 71.2 us); SMG_DSLASH_H_NP=1 or 2 fixes it
int dslash_h_np(int nrhs) {
    static const int env = [] {
        const char* e = std::getenv("SMG_DSLASH_H_NP");
        return e ? std::atoi(e) : 0;
    }();
    const int np = env == 1 || env == 2 ? env : (nrhs >= 8 ? 2 : 1);
    return nrhs >= 4 * np ? np : 1;
}

// the specialised 32-RHS FP16 stencil (k_dslash_h32) where it applies; SMG_DSLASH_H32=0 keeps the
// generic kernel
bool dslash_h32_enabled() {
    static const bool on = [] {
        const char* e = std::getenv("SMG_DSLASH_H32");
        return !(e && std::atoi(e) == 0);
    }();
    return on;
}

struct HLaunch {
    dim3 grid, block;
};
HLaunch dslash_h_launch(int L, int nrhs) {
    const int np = dslash_h_np(nrhs), lanes = nrhs / (2 * np), rows = 256 / lanes;
    return {dim3((L + rows - 1) / rows, L), dim3(lanes, rows)};
}

// Sums of the stencil blocks' partials part[block][j] (j < ncol <= 96) in FP64 and a fixed order, in
// two passes: block g of the first sums the contiguous rows [g R, g R + R) with threads (row group,
// column j) and kDotsRows independent loads per thread; the second pass sums the per-block results
// of one column per block.
constexpr int kDotsRows = 8;  // rows per thread in the first pass
__global__ void __launch_bounds__(256) k_dots_stage(const float* __restrict__ part, int nblocks, int ncol, int R,
                                                    double* __restrict__ mid) {
    __shared__ double s[256];
    const int groups = blockDim.x / ncol;
    const int r = threadIdx.x / ncol, j = threadIdx.x - r * ncol;
    double acc = 0.0;
    if (r < groups) {
        const int b0 = blockIdx.x * R;
        const int b1 = b0 + R < nblocks ? b0 + R : nblocks;
        float v[kDotsRows];
#pragma unroll
        for (int u = 0; u < kDotsRows; ++u) {
            const int b = b0 + r + u * groups;
            v[u] = b < b1 ? part[(int64_t)b * ncol + j] : 0.f;
        }
#pragma unroll
        for (int u = 0; u < kDotsRows; ++u) acc += (double)v[u];
    }
    s[threadIdx.x] = acc;
    __syncthreads();
    if (threadIdx.x < ncol) {
        double t = 0.0;
        for (int q = 0; q < groups; ++q) t += s[q * ncol + threadIdx.x];
        mid[(int64_t)threadIdx.x * gridDim.x + blockIdx.x] = t;
    }
}

// the MR step's reductions per rhs from the two norm columns: out[3 rhs] = ||D r||^2 (= <A r, r> for
// A = D^dag D), out[3 rhs + 1] = 0, out[3 rhs + 2] = ||A r||^2, and the step's omega = out[3 rhs] /
// out[3 rhs + 2] as a float pair (0 when the denominator is not a usable number); one block per rhs
__global__ void __launch_bounds__(256) k_mr_norms_finish(const double* __restrict__ mid, int G,
                                                         double* __restrict__ out, float2* __restrict__ omega) {
    __shared__ double s[2][256];
    const int rhs = blockIdx.x;
    double a0 = 0.0, a1 = 0.0;
    for (int g = threadIdx.x; g < G; g += blockDim.x) {
        a0 += mid[(int64_t)(2 * rhs) * G + g];
        a1 += mid[(int64_t)(2 * rhs + 1) * G + g];
    }
    s[0][threadIdx.x] = a0;
    s[1][threadIdx.x] = a1;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) {
            s[0][threadIdx.x] += s[0][threadIdx.x + o];
            s[1][threadIdx.x] += s[1][threadIdx.x + o];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        const double num = s[0][0], den = s[1][0];
        out[3 * rhs] = num;
        out[3 * rhs + 1] = 0.0;
        out[3 * rhs + 2] = den;
        if (omega) omega[rhs] = make_float2((fabs(den) >= 1e-30 && isfinite(den)) ? (float)(num / den) : 0.f, 0.f);
    }
}

smg_status launch_dslash_h(smg_dirac* d, bool dag, const smg_field* src, smg_field* dst, float* part, int part_col) {
    smg_context* ctx = src->ctx;
    const int nrhs = src->nrhs;
    if (!f16_nrhs_ok(nrhs) || nrhs < 2)
        return smg_fail(ctx, SMG_UNSUPPORTED, "F16 stencil: nrhs a power of two from 2 to 32");
    if (src->prec == SMG_F64 || dst->prec == SMG_F64)
        return smg_fail(ctx, SMG_UNSUPPORTED, "dslash between F16 and F64 fields");
    if (!d->gauge->U32) return smg_fail(ctx, SMG_DEVICE_ERROR, "FP32 links missing");
    DslashH a;
    const bool ih = src->prec == SMG_F16, oh = dst->prec == SMG_F16;
    if (ih) {
        a.src16 = (const __half2*)src->data;
        a.src_scale = src->scale;
    } else {
        a.src32 = (const cx<float>*)src->data;
    }
    if (oh) {
        a.dst16 = (__half2*)dst->data;
        a.dst_scale = dst->scale;
    } else {
        a.dst32 = (cx<float>*)dst->data;
    }
    a.U = d->gauge->U32;
    a.C = d->C32;
    a.g = src->g;
    a.nrhs = nrhs;
    a.diag = (float)(2.0 * d->r + d->mass);
    a.mu_eff = (float)(dag ? -d->mu_t : d->mu_t);
    a.r = (float)d->r;
    a.part = part;
    a.part_col = part_col;
    const bool norm = part != nullptr;
    if (norm && !(ih && oh)) return smg_fail(ctx, SMG_UNSUPPORTED, "fused FP16 stencil norm: F16 fields");
    const HLaunch hl = dslash_h_launch(a.g.L, nrhs);
    const int np = dslash_h_np(nrhs);
    if (ih && oh && nrhs == 32 && np == 2 && d->r == 1.0 && a.mu_eff == 0.f && dslash_h32_enabled()) {
        if (dag) {
            if (norm) k_dslash_h32<true, true><<<hl.grid, hl.block, 0, ctx->stream>>>(a);
            else k_dslash_h32<true, false><<<hl.grid, hl.block, 0, ctx->stream>>>(a);
        } else {
            if (norm) k_dslash_h32<false, true><<<hl.grid, hl.block, 0, ctx->stream>>>(a);
            else k_dslash_h32<false, false><<<hl.grid, hl.block, 0, ctx->stream>>>(a);
        }
        count_launch(ctx);
        SMG_CHECK_LAUNCH(ctx);
        return SMG_OK;
    }
#define SMG_DH(DG, I, O, N)                                                                                         \
    do {                                                                                                            \
        if (np == 2) {                                                                                              \
            if (d->r == 1.0) k_dslash_h<DG, I, O, true, N, 2><<<hl.grid, hl.block, 0, ctx->stream>>>(a);           \
            else k_dslash_h<DG, I, O, false, N, 2><<<hl.grid, hl.block, 0, ctx->stream>>>(a);                     \
        } else {                                                                                                    \
            if (d->r == 1.0) k_dslash_h<DG, I, O, true, N, 1><<<hl.grid, hl.block, 0, ctx->stream>>>(a);           \
            else k_dslash_h<DG, I, O, false, N, 1><<<hl.grid, hl.block, 0, ctx->stream>>>(a);                     \
        }                                                                                                           \
    } while (0)
    if (norm) {
        if (dag) SMG_DH(true, true, true, true);
        else SMG_DH(false, true, true, true);
    } else if (dag) {
        if (ih && oh) SMG_DH(true, true, true, false);
        else if (ih) SMG_DH(true, true, false, false);
        else SMG_DH(true, false, true, false);
    } else {
        if (ih && oh) SMG_DH(false, true, true, false);
        else if (ih) SMG_DH(false, true, false, false);
        else SMG_DH(false, false, true, false);
    }
#undef SMG_DH
    count_launch(ctx);
    SMG_CHECK_LAUNCH(ctx);
    return SMG_OK;
}

// blocks of the FP16 stencil's grid (the size of the partial-sum buffer of the fused norms)
int dslash_h_blocks(int L, int nrhs) {
    const HLaunch hl = dslash_h_launch(L, nrhs);
    return (int)(hl.grid.x * hl.grid.y);
}

// the MR step's scalars from the norm partials of its two stencils (columns 0 and 1 of part):
// out3[rhs][3] = (||D r||^2, 0, ||D^dag D r||^2)
smg_status launch_mr_norms_finish(smg_context* ctx, int L, int nrhs, const float* part, double* out3, float* omega) {
    const int ncol = nrhs * 2, nblocks = dslash_h_blocks(L, nrhs);
    const int groups = 256 / ncol, R = groups * kDotsRows;  // rows per first-pass block
    const int G = (nblocks + R - 1) / R;
    SMG_TRY(smg_reduce_reserve(ctx, (size_t)G * ncol));
    k_dots_stage<<<G, groups * ncol, 0, ctx->stream>>>(part, nblocks, ncol, R, ctx->red.partials);
    k_mr_norms_finish<<<nrhs, 256, 0, ctx->stream>>>(ctx->red.partials, G, out3, reinterpret_cast<float2*>(omega));
    count_launch(ctx, 2);
    SMG_CHECK_LAUNCH(ctx);
    return SMG_OK;
}

// (D(e^{i dt pi} U) - D(U)) v through the hopping terms only (apply_delta_D, dirac.h:154-174): the
// forward hop's link is scaled by (e^{i dt pi_mu(x)} - 1), the backward hop's U^dag by
// (e^{-i dt pi_mu(x - mu)} - 1); pi is lexicographic [mu][s]
__global__ void k_delta_dslash(const cx<double>* __restrict__ src, cx<double>* __restrict__ dst,
                               const cx<double>* __restrict__ U, const double* __restrict__ pi, double dt, double r,
                               Geom g, int nrhs) {
    const int rhs = blockIdx.y * blockDim.x + threadIdx.x;
    const int q = blockIdx.x * blockDim.y + threadIdx.y;
    if (rhs >= nrhs || q >= g.V) return;
    int x, y, p;
    site_coords(g, q, x, y, p);
    const int xp = x + 1 == g.L ? 0 : x + 1, xm = x == 0 ? g.L - 1 : x - 1;
    const int yp = y + 1 == g.L ? 0 : y + 1, ym = y == 0 ? g.L - 1 : y - 1;
    const int q_xp = site_q(g, xp, y), q_xm = site_q(g, xm, y), q_yp = site_q(g, x, yp), q_ym = site_q(g, x, ym);
    auto phase_m1 = [&](double a) {  // e^{i a} - 1
        double sn, cs;
        sincos(a, &sn, &cs);
        return mk(cs - 1.0, sn);
    };
    const cx<double> u0f = phase_m1(dt * pi[x + g.L * y]) * U[q];
    const cx<double> u0b = phase_m1(-dt * pi[xm + g.L * y]) * conj(U[q_xm]);
    const cx<double> u1f = phase_m1(dt * pi[g.V + x + g.L * y]) * U[g.V + q];
    const cx<double> u1b = phase_m1(-dt * pi[g.V + x + g.L * ym]) * conj(U[g.V + q_ym]);
    const Spinor<double> pxp = ld_spinor(src, q_xp, rhs, nrhs), pxm = ld_spinor(src, q_xm, rhs, nrhs);
    const Spinor<double> pyp = ld_spinor(src, q_yp, rhs, nrhs), pym = ld_spinor(src, q_ym, rhs, nrhs);
    const cx<double> a0x = u0f * pxp.s0, a1x = u0f * pxp.s1;
    const cx<double> b0x = u0b * pxm.s0, b1x = u0b * pxm.s1;
    const cx<double> a0y = u1f * pyp.s0, a1y = u1f * pyp.s1;
    const cx<double> b0y = u1b * pym.s0, b1y = u1b * pym.s1;
    const cx<double> sr0 = (a0x + b0x) + (a0y + b0y);
    const cx<double> sr1 = (a1x + b1x) + (a1y + b1y);
    const cx<double> off0 = (b1x - a1x) + times_i(a1y - b1y);
    const cx<double> off1 = (b0x - a0x) - times_i(a0y - b0y);
    Spinor<double> o;
    o.s0 = -0.5 * (r * sr0 + off0);
    o.s1 = -0.5 * (r * sr1 + off1);
    st_spinor(dst, q, rhs, nrhs, o);
}

// F01(s) = Im(P_ur + P_ul + P_ll + P_lr) / 4   (dirac.h:26-52)
__device__ __forceinline__ cx<double> lkd(const cx<double>* __restrict__ U, const Geom& g, int mu, int x, int y) {
    return U[(int64_t)mu * g.V + site_q(g, wrap(x, g.L), wrap(y, g.L))];
}

__global__ void k_clover(const cx<double>* __restrict__ U, Geom g, double c_sw, double* __restrict__ F01,
                         double* __restrict__ C64, float* __restrict__ C32) {
    int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= g.V) return;
    int x, y, p;
    site_coords(g, q, x, y, p);
    cx<double> P_ur = lkd(U, g, 0, x, y) * lkd(U, g, 1, x + 1, y) * conj(lkd(U, g, 0, x, y + 1)) * conj(lkd(U, g, 1, x, y));
    cx<double> P_ul = lkd(U, g, 1, x, y) * conj(lkd(U, g, 0, x - 1, y + 1)) * conj(lkd(U, g, 1, x - 1, y)) *
                      lkd(U, g, 0, x - 1, y);
    cx<double> P_ll = conj(lkd(U, g, 0, x - 1, y)) * conj(lkd(U, g, 1, x - 1, y - 1)) * lkd(U, g, 0, x - 1, y - 1) *
                      lkd(U, g, 1, x, y - 1);
    cx<double> P_lr = conj(lkd(U, g, 1, x, y - 1)) * lkd(U, g, 0, x, y - 1) * lkd(U, g, 1, x + 1, y - 1) *
                      conj(lkd(U, g, 0, x, y));
    cx<double> Q = P_ur + P_ul + P_ll + P_lr;
    double f = Q.im / 4.0;
    F01[q] = f;
    double c = 0.5 * c_sw * f;
    C64[q] = c;
    C32[q] = (float)c;
}

__global__ void k_f01_out(const double* __restrict__ F01, Geom g, double* __restrict__ host) {
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= g.V) return;
    host[s] = F01[site_q(g, s % g.L, s / g.L)];
}

template <typename T>
__global__ void k_gamma5(cx<T>* __restrict__ v, int nsites, int nrhs) {
    int rhs = blockIdx.y * blockDim.x + threadIdx.x;
    int q = blockIdx.x * blockDim.y + threadIdx.y;
    if (rhs >= nrhs || q >= nsites) return;
    int64_t i = sidx(q, rhs, 1, nrhs);
    v[i] = -v[i];
}

constexpr int kTileSmemMax = 112 * 1024;

// both instantiations may use up to kTileSmemMax of dynamic shared memory (process-wide, set once)
template <typename T>
void ensure_tile_attr() {
    static std::once_flag once;
    std::call_once(once, [] {
        cudaFuncSetAttribute((const void*)k_dslash_tile<T, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             kTileSmemMax);
        cudaFuncSetAttribute((const void*)k_dslash_tile<T, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             kTileSmemMax);
    });
}

// the row kernel with the spin-projected hops when r = 1
template <typename T, bool DAG, int EPI>
void launch_row(smg_context* ctx, const DslashArgs<T>& a, dim3 grid, dim3 block) {
    if (a.r == T(1))
        k_dslash<T, DAG, EPI, true><<<grid, block, 0, ctx->stream>>>(a);
    else
        k_dslash<T, DAG, EPI, false><<<grid, block, 0, ctx->stream>>>(a);
}

// patch mapping of the row kernel: variant 4, 5, 6 = patches px = 2, 4, 8 sites wide and
// (256 / lanes) / px rows high, both parities
inline void patch_shape(int nrhs, int v, int& px, int& py) {
    const int lanes = nrhs < 32 ? nrhs : 32;
    const int sites = 256 / lanes;
    px = 1 << (v - 3);
    py = sites / px;
}

bool patch_ok(const Geom& g, int nrhs, int v) {
    const int lanes = nrhs < 32 ? nrhs : 32;
    int px, py;
    patch_shape(nrhs, v, px, py);
    return 256 % lanes == 0 && py >= 1 && px * py * lanes == 256 && g.L % px == 0 && g.L % py == 0;
}

template <typename T>
smg_status launch_patch(smg_context* ctx, DslashArgs<T> a, bool dag, int v) {
    const int lanes = a.nrhs < 32 ? a.nrhs : 32;
    int px, py;
    patch_shape(a.nrhs, v, px, py);
    a.px = px;
    const dim3 block(lanes, py * px), grid(a.g.L / px, a.g.L / py, (a.nrhs + lanes - 1) / lanes);
    if (dag)
        launch_row<T, true, EPI_NONE>(ctx, a, grid, block);
    else
        launch_row<T, false, EPI_NONE>(ctx, a, grid, block);
    count_launch(ctx);
    SMG_CHECK_LAUNCH(ctx);
    return SMG_OK;
}

// variant 7: two right-hand sides per thread (nrhs even, nrhs / 2 <= 32 lanes)
bool r2_ok(int nrhs) { return nrhs >= 2 && nrhs % 2 == 0 && nrhs / 2 <= 32 && 256 % (nrhs / 2) == 0; }

template <typename T>
smg_status launch_r2(smg_context* ctx, const DslashArgs<T>& a, bool dag) {
    const int lanes = a.nrhs / 2, rows = 256 / lanes;
    const dim3 block(lanes, rows), grid((a.g.L + rows - 1) / rows, a.g.L);
    if (dag)
        k_dslash_r2<T, true><<<grid, block, 0, ctx->stream>>>(a);
    else
        k_dslash_r2<T, false><<<grid, block, 0, ctx->stream>>>(a);
    count_launch(ctx);
    SMG_CHECK_LAUNCH(ctx);
    return SMG_OK;
}

// variant 0: one (site, rhs) per thread over rows; v in 1..3: the tiled kernel with TY = 2^v rows;
// v in 4..6: the row kernel on 2-D patches (patch_shape)
template <typename T>
smg_status launch_tile(smg_context* ctx, const DslashArgs<T>& a, bool dag, int v) {
    const int TY = 1 << v;
    const int nrhs = a.nrhs;
    const size_t sm = tile_smem<T>(TY, nrhs);
    const dim3 block(nrhs, 256 / nrhs), grid(a.g.Lh / kTileXH, a.g.L / TY);
    if (dag)
        k_dslash_tile<T, true><<<grid, block, sm, ctx->stream>>>(a, TY);
    else
        k_dslash_tile<T, false><<<grid, block, sm, ctx->stream>>>(a, TY);
    count_launch(ctx);
    SMG_CHECK_LAUNCH(ctx);
    return SMG_OK;
}

template <typename T>
bool tile_ok(const Geom& g, int nrhs, int v) {
    const int TY = 1 << v;
    return nrhs >= 4 && nrhs <= 32 && 256 % nrhs == 0 && g.Lh % kTileXH == 0 && g.L % TY == 0 &&
           (nrhs * sizeof(Spinor<T>)) % 16 == 0 && tile_smem<T>(TY, nrhs) <= (size_t)kTileSmemMax;
}

// The launch shape of the plain stencil is chosen once per (L, nrhs, precision)
// and context by timing every variant on the caller's own operands (a few
// launches each, CUDA events on the context's stream); the choice is cached.
// During CUDA-graph capture, or when nothing is cached yet for a capture, the
// row kernel runs.
template <typename T>
int dslash_variant(smg_context* ctx, const DslashArgs<T>& a, bool dag) {
    const uint64_t key = ((uint64_t)a.g.L << 24) ^ ((uint64_t)a.nrhs << 8) ^ (uint64_t)sizeof(T);
    for (const auto& kv : ctx->dslash_plans)
        if (kv.first == key) return kv.second;
    ensure_tile_attr<T>();
    if (const char* e = std::getenv("SMG_DSLASH_VARIANT")) {  // fixed choice, for measurements
        const int v = std::atoi(e);
        if (v == 0 || (v <= 3 && tile_ok<T>(a.g, a.nrhs, v)) || (v >= 4 && v <= 6 && patch_ok(a.g, a.nrhs, v)) ||
            (v == 7 && r2_ok(a.nrhs)))
            return v;
    }
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(ctx->stream, &cs) != cudaSuccess || cs != cudaStreamCaptureStatusNone) return 0;
    std::vector<int> cands{0};
    for (int v = 1; v <= 3; ++v)
        if (tile_ok<T>(a.g, a.nrhs, v)) cands.push_back(v);
    for (int v = 4; v <= 6; ++v)
        if (patch_ok(a.g, a.nrhs, v)) cands.push_back(v);
    if (r2_ok(a.nrhs)) cands.push_back(7);
    int best = 0;
    if (cands.size() > 1) {
        cudaEvent_t e0, e1;
        cudaEventCreate(&e0);
        cudaEventCreate(&e1);
        float best_ms = 1e30f;
        for (int v : cands) {
            auto run = [&]() {
                if (v == 0) {
                    const int lanes = a.nrhs < 32 ? a.nrhs : 32, rows = 256 / lanes;
                    const dim3 block(lanes, rows), grid((a.g.L + rows - 1) / rows, a.g.L, (a.nrhs + lanes - 1) / lanes);
                    if (dag)
                        launch_row<T, true, EPI_NONE>(ctx, a, grid, block);
                    else
                        launch_row<T, false, EPI_NONE>(ctx, a, grid, block);
                    count_launch(ctx);
                } else if (v <= 3) {
                    launch_tile<T>(ctx, a, dag, v);
                } else if (v <= 6) {
                    launch_patch<T>(ctx, a, dag, v);
                } else {
                    launch_r2<T>(ctx, a, dag);
                }
            };
            run();
            cudaEventRecord(e0, ctx->stream);
            for (int i = 0; i < 5; ++i) run();
            cudaEventRecord(e1, ctx->stream);
            cudaEventSynchronize(e1);
            float ms = 0;
            cudaEventElapsedTime(&ms, e0, e1);
            if (cudaGetLastError() == cudaSuccess && ms < best_ms) {
                best_ms = ms;
                best = v;
            }
        }
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
    }
    ctx->dslash_plans.push_back({key, best});
    return best;
}

template <typename T>
smg_status launch_dslash(smg_dirac* d, bool dag, int epi, const smg_field* src, smg_field* dst, const smg_field* w,
                         double* out_dev) {
    smg_context* ctx = src->ctx;
    DslashArgs<T> a;
    a.src = (const cx<T>*)src->data;
    a.dst = (cx<T>*)dst->data;
    if (sizeof(T) == 8) {
        a.U = (const cx<T>*)d->gauge->U64;
        a.C = (const T*)d->C64;
    } else {
        a.U = (const cx<T>*)d->gauge->U32;
        a.C = (const T*)d->C32;
    }
    a.w = w ? (const cx<T>*)w->data : nullptr;
    a.g = src->g;
    a.nrhs = src->nrhs;
    a.diag = (T)(2.0 * d->r + d->mass);
    a.mu_eff = (T)(dag ? -d->mu_t : d->mu_t);
    a.r = (T)d->r;
    a.partials = ctx->red.partials;
    a.ticket = ctx->red.tickets;
    a.out = out_dev;
    dim3 grid, block;
    if (epi == EPI_NONE) {
        const int variant = dslash_variant<T>(ctx, a, dag);
        if (variant == 7) return launch_r2<T>(ctx, a, dag);
        if (variant >= 4) return launch_patch<T>(ctx, a, dag, variant);
        if (variant > 0) return launch_tile<T>(ctx, a, dag, variant);

        // (row segment, row, rhs chunk) grid, one site and rhs per thread
        const int lanes = src->nrhs < 32 ? src->nrhs : 32;
        const int rows = 256 / lanes;
        block = dim3(lanes, rows, 1);
        grid = dim3((src->g.L + rows - 1) / rows, src->g.L, (src->nrhs + lanes - 1) / lanes);
    } else {
        ReduceLaunch rl = reduce_launch(src->g.V, src->nrhs);
        SMG_TRY(smg_reduce_reserve(ctx, (size_t)rl.grid.x * src->nrhs * 3));
        a.partials = ctx->red.partials;
        grid = rl.grid;
        block = rl.block;
    }
#define SMG_DS(DAG, EPI) launch_row<T, DAG, EPI>(ctx, a, grid, block)
    if (dag) {
        if (epi == EPI_NONE) SMG_DS(true, EPI_NONE);
        else if (epi == EPI_NORM) SMG_DS(true, EPI_NORM);
        else SMG_DS(true, EPI_MR);
    } else {
        if (epi == EPI_NONE) SMG_DS(false, EPI_NONE);
        else if (epi == EPI_NORM) SMG_DS(false, EPI_NORM);
        else SMG_DS(false, EPI_MR);
    }
#undef SMG_DS
    count_launch(ctx);
    SMG_CHECK_LAUNCH(ctx);
    return SMG_OK;
}

smg_status dslash_dispatch(smg_dirac* d, bool dag, int epi, const smg_field* src, smg_field* dst, const smg_field* w,
                           double* out_dev) {
    if (src->prec == SMG_F16 || dst->prec == SMG_F16) {
        if (epi != EPI_NONE) return smg_fail(src->ctx, SMG_UNSUPPORTED, "fused reductions on F16 fields");
        return launch_dslash_h(d, dag, src, dst, nullptr, 0);
    }
    if (src->prec != dst->prec) return smg_fail(src->ctx, SMG_BAD_ARG, "dslash between F32 and F64 fields");
    if (src->prec == SMG_F64) return launch_dslash<double>(d, dag, epi, src, dst, w, out_dev);
    if (src->prec == SMG_F32) return launch_dslash<float>(d, dag, epi, src, dst, w, out_dev);
    return smg_fail(src->ctx, SMG_UNSUPPORTED, "dslash on F16 field");
}

smg_status gamma5_inplace(smg_field* f) {
    smg_context* ctx = f->ctx;
    SiteLaunch sl = site_launch(f->g.V, f->nrhs);
    if (f->prec == SMG_F64)
        k_gamma5<double><<<sl.grid, sl.block, 0, ctx->stream>>>((cx<double>*)f->data, f->g.V, f->nrhs);
    else if (f->prec == SMG_F32)
        k_gamma5<float><<<sl.grid, sl.block, 0, ctx->stream>>>((cx<float>*)f->data, f->g.V, f->nrhs);
    else
        return smg_fail(ctx, SMG_UNSUPPORTED, "gamma5 on F16 field");
    count_launch(ctx);
    SMG_CHECK_LAUNCH(ctx);
    return SMG_OK;
}

smg_status check_op_fields(smg_dirac* d, const smg_field* src, const smg_field* dst) {
    if (!d || !src || !dst) return SMG_BAD_ARG;
    smg_context* ctx = d->ctx;
    if (src == dst) return smg_fail(ctx, SMG_BAD_ARG, "src and dst must be distinct fields");
    SMG_TRY(smg_field_check_pair(src, dst));
    if (src->ctx != ctx) return smg_fail(ctx, SMG_BAD_ARG, "field and operator belong to different contexts");
    if (src->g.L != d->gauge->g.L) return smg_fail(ctx, SMG_BAD_ARG, "field L differs from gauge L");
    return SMG_OK;
}

}  // namespace

// ---- internal entry points used by solvers, MG and forces
smg_status smg_dslash(smg_dirac* d, bool dag, const smg_field* src, smg_field* dst, double* norm2_dev) {
    return dslash_dispatch(d, dag, norm2_dev ? EPI_NORM : EPI_NONE, src, dst, nullptr, norm2_dev);
}
smg_status smg_dslash_mr(smg_dirac* d, bool dag, const smg_field* src, smg_field* dst, const smg_field* w,
                         double* out3_dev) {
    return dslash_dispatch(d, dag, EPI_MR, src, dst, w, out3_dev);
}
// FP16 stencil with ||out||^2 per block and rhs into part column part_col (see k_dslash_h)
smg_status smg_dslash_h_norm(smg_dirac* d, bool dag, const smg_field* src, smg_field* dst, float* part,
                             int part_col) {
    return launch_dslash_h(d, dag, src, dst, part, part_col);
}
smg_status smg_mr_norms_finish(smg_context* ctx, int L, int nrhs, const float* part, double* out3_dev,
                               float* omega_dev) {
    return launch_mr_norms_finish(ctx, L, nrhs, part, out3_dev, omega_dev);
}
int smg_dslash_h_blocks(int L, int nrhs) { return dslash_h_blocks(L, nrhs); }
// reduction scratch (doubles) the fused FP16 stencil norms use for a lattice and nrhs
size_t smg_dslash_h_dots_scratch(int L, int nrhs) {
    const int ncol = nrhs * 2, R = (256 / ncol) * kDotsRows;
    return (size_t)((dslash_h_blocks(L, nrhs) + R - 1) / R) * ncol;
}

smg_status smg_dirac_apply_internal(smg_dirac* d, smg_operator op, const smg_field* src, smg_field* dst,
                                    double* norm2_out_dev) {
    smg_context* ctx = src->ctx;
    switch (op) {
        case SMG_OP_D: return smg_dslash(d, false, src, dst, norm2_out_dev);
        case SMG_OP_DDAG: return smg_dslash(d, true, src, dst, norm2_out_dev);
        case SMG_OP_G5D:
            SMG_TRY(smg_dslash(d, false, src, dst, nullptr));
            return gamma5_inplace(dst);
        case SMG_OP_DDAGD: {
            smg_field* tmp = nullptr;
            SMG_TRY(smg_field_alloc_like(src, src->prec, &tmp));
            smg_status s = smg_dslash(d, false, src, tmp, nullptr);
            if (s == SMG_OK) s = smg_dslash(d, true, tmp, dst, norm2_out_dev);
            smg_field_destroy(tmp);
            return s;
        }
    }
    return smg_fail(ctx, SMG_BAD_ARG, "unknown operator");
}

extern "C" {

SMG_API smg_status smg_dirac_create(smg_gauge* gf, double mass, double r, double c_sw, double mu_t, smg_dirac** out) {
    if (!gf || !out) return SMG_BAD_ARG;
    *out = nullptr;
    smg_context* ctx = gf->ctx;
    smg_dirac* d = new smg_dirac();
    d->ctx = ctx;
    d->gauge = gf;
    d->mass = mass;
    d->r = r;
    d->c_sw = c_sw;
    d->mu_t = mu_t;
    size_t V = gf->g.V;
    if (cudaMalloc(&d->F01, V * sizeof(double)) != cudaSuccess) {
        delete d;
        return smg_fail(ctx, SMG_NO_MEMORY, "clover allocation");
    }
    if (c_sw != 0.0) {
        if (cudaMalloc(&d->C64, V * sizeof(double)) != cudaSuccess ||
            cudaMalloc(&d->C32, V * sizeof(float)) != cudaSuccess) {
            smg_dirac_destroy(d);
            return smg_fail(ctx, SMG_NO_MEMORY, "clover allocation");
        }
    }
    smg_status s = smg_dirac_refresh(d);
    if (s != SMG_OK) {
        smg_dirac_destroy(d);
        return s;
    }
    *out = d;
    return SMG_OK;
}

SMG_API smg_status smg_dirac_destroy(smg_dirac* d) {
    if (!d) return SMG_OK;
    cudaStreamSynchronize(d->ctx->stream);
    if (d->F01) cudaFree(d->F01);
    if (d->C64) cudaFree(d->C64);
    if (d->C32) cudaFree(d->C32);
    delete d;
    return SMG_OK;
}

SMG_API smg_status smg_dirac_refresh(smg_dirac* d) {
    if (!d) return SMG_BAD_ARG;
    smg_context* ctx = d->ctx;
    const Geom g = d->gauge->g;
    if (d->c_sw != 0.0) {
        k_clover<<<(g.V + 255) / 256, 256, 0, ctx->stream>>>(d->gauge->U64, g, d->c_sw, d->F01, d->C64, d->C32);
        count_launch(ctx);
        SMG_CHECK_LAUNCH(ctx);
    } else {
        SMG_CUDA(ctx, cudaMemsetAsync(d->F01, 0, (size_t)g.V * sizeof(double), ctx->stream));
    }
    return SMG_OK;
}

SMG_API smg_status smg_dirac_get_clover(smg_dirac* d, double* F01) {
    if (!d || !F01) return SMG_BAD_ARG;
    smg_context* ctx = d->ctx;
    const Geom g = d->gauge->g;
    double* tmp = nullptr;
    SMG_CUDA(ctx, cudaMallocAsync(&tmp, (size_t)g.V * sizeof(double), ctx->stream));
    k_f01_out<<<(g.V + 255) / 256, 256, 0, ctx->stream>>>(d->F01, g, tmp);
    count_launch(ctx);
    SMG_CHECK_LAUNCH(ctx);
    SMG_CUDA(ctx, cudaMemcpyAsync(F01, tmp, (size_t)g.V * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    SMG_CUDA(ctx, cudaFreeAsync(tmp, ctx->stream));
    SMG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return SMG_OK;
}

SMG_API smg_status smg_dirac_apply_delta(smg_dirac* d, const double* pi, double dt, const smg_field* src,
                                         smg_field* dst) {
    SMG_TRY(check_op_fields(d, src, dst));
    smg_context* ctx = d->ctx;
    if (!pi) return SMG_BAD_ARG;
    if (src->prec != SMG_F64) return smg_fail(ctx, SMG_UNSUPPORTED, "apply_delta_D on non-F64 fields");
    const Geom g = src->g;
    double* pd = nullptr;
    SMG_CUDA(ctx, cudaMallocAsync((void**)&pd, (size_t)2 * g.V * sizeof(double), ctx->stream));
    SMG_CUDA(ctx, cudaMemcpyAsync(pd, pi, (size_t)2 * g.V * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
    const SiteLaunch sl = site_launch(g.V, src->nrhs);
    k_delta_dslash<<<sl.grid, sl.block, 0, ctx->stream>>>((const cx<double>*)src->data, (cx<double>*)dst->data,
                                                          d->gauge->U64, pd, dt, d->r, g, src->nrhs);
    count_launch(ctx);
    SMG_CHECK_LAUNCH(ctx);
    SMG_CUDA(ctx, cudaFreeAsync(pd, ctx->stream));
    SMG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return SMG_OK;
}

SMG_API smg_status smg_dirac_apply(smg_dirac* d, smg_operator op, const smg_field* src, smg_field* dst) {
    SMG_TRY(check_op_fields(d, src, dst));
    return smg_dirac_apply_internal(d, op, src, dst, nullptr);
}

}  // extern "C"
