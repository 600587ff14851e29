// Batched coarse-operator apply on the 5th-generation tensor cores (tcgen05).
//
// The coarse operator is a 9-point stencil of Nc x Nc complex blocks
// (SparseCoarseOp::apply, src/coarse_op.h:154-297):
//     y[s](i, r) = sum_d sum_j L[s][d](i, j) x[nb(s, d)](j, r)
// for right-hand sides r.  With Nc = 16 and 32 right-hand sides each site is
// nine small complex GEMMs.  This kernel computes the transposed product
// y^T = sum_d x_nb^T L_d^T as real MMAs with BF16 operands and FP32
// accumulation:
//
//   A operand (M x K = 64 x 16, vectors):  row m = 2 r + c holds the real
//       (c = 0) or imaginary (c = 1) part of x(j, r) for K index j
//   B operand (N x K = 32 x 16, links):    row n = c' * 16 + i holds
//       Re L(i, j) (c' = 0) or Im L(i, j) (c' = 1) for K index j
//   D (M x N, FP32 in tensor memory):      D[2r + c][c' * 16 + i]
//
// and the epilogue forms Re y(i, r) = D[2r][i] - D[2r+1][16+i] and
// Im y(i, r) = D[2r][16+i] + D[2r+1][i] (the two rows sit in adjacent lanes
// of one warp).  The MMA is issued with M = 128: rows 64..127 read the next
// 2 KB of shared memory and are never read back, which keeps the accumulator
// in the plain one-lane-per-row layout.
//
// Source grouping.  A source tile x_t serves the three output sites of its
// row that reach it along x (dx = +1, 0, -1): one MMA with the three link
// blocks stacked along N (N = 96) accumulates into the three sites' adjacent
// 32-column accumulators.  A small MMA costs the same issue time for N up to
// 128, so a row of kW = 8 sites takes 3 x 10 MMAs instead of 72.  The links
// are pre-tiled once per hierarchy so that, for an output row y and a source
// row offset dy, block L[x][(dx, dy)] sits at position P = 3x + 4 + 2dx
// (mod 3 nx): the nine sites' blocks of a CTA strip for one dy form one
// contiguous run of 3 kW + 2 blocks and the stacked operand of source t is
// three consecutive blocks.
//
// Data movement (one CTA = a strip of kW sites along x, H rows):
//   * per output row and dy one 26 KB run of BF16 link blocks arrives by
//     cp.async.bulk (two when the run wraps around the lattice) into a ring
//     of kUnits units;
//   * each source row (kW + 2 sites with the x halo) is converted from the
//     FP32 vector [site][dof][rhs] layout into BF16 A tiles by four stager
//     warps and kept in a ring of four rows (output row y reads source rows
//     y-1, y, y+1);
//   * warp 10 issues the link copies, warp 11 the MMAs; the warp pairs (0, 1),
//     (4, 5), (8, 9) read the accumulators (TMEM lanes 0..63, which only warps
//     with warp % 4 = 0 or 1 may access; one 256-column slot per output row,
//     two slots), each pair a third of a row's sites, and write y with the
//     fused per-rhs reductions ||y||^2 and <y, w> of the FP32 kernels.  The
//     epilogue bounds the row rate, and the accumulator lanes tie it to two of
//     the SM's four schedulers, so it gets three warps on each of them.
// Every mbarrier wait is bounded (about one second of SM clock); on timeout
// the CTA raises *err = 2, waits (bounded) for its own bulk copies and MMAs,
// frees its tensor memory and returns.
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include <cstdlib>
#include <map>
#include <mutex>
#include <tuple>
#include <vector>

#include "half.cuh"
#include "smg_internal.h"

namespace {

constexpr int kNc = 16;                       // coarse dofs per site (the supported shape)
constexpr int kRhsTile = 32;                  // right-hand sides per CTA
constexpr int kW = 8;                         // output sites per row of a CTA strip
constexpr int kSrcSites = kW + 2;             // source sites per row (x halo)
constexpr int kRing = 4;                      // source rows resident
constexpr int kSboA = 272;                    // A tile: byte stride of 8-row groups (256 + 16 spreads banks)
constexpr int kTileA = 8 * kSboA;             // 64 rows x 16 K (BF16) = 2176 bytes
constexpr int kRowBytes = kSrcSites * kTileA;  // one source row
constexpr int kRingBytes = kRing * kRowBytes;
constexpr int kLinkDir = 1024;                // 32 x 16 BF16, K-major, no swizzle
constexpr int kLinkSite = 9 * kLinkDir;       // one site's nine blocks (HBM bytes per site)
constexpr int kRunBlocks = 3 * kW + 2;        // link blocks of one (output row, dy) run of a strip
constexpr int kUnitBytes = kRunBlocks * kLinkDir;
constexpr int kUnits = 5;                     // link runs resident
constexpr int kLinkBytes = kUnits * kUnitBytes;
constexpr int kAccCols = kW * 32;             // one output row of accumulators
constexpr int kTmemCols = 512;                // two row slots
// barriers: src_full[4], src_empty[4], unit_full[U], unit_empty[U], acc_full[2], acc_empty[2], final
constexpr int kBarSrcFull = 0;
constexpr int kBarSrcEmpty = kBarSrcFull + kRing;
constexpr int kBarUnitFull = kBarSrcEmpty + kRing;
constexpr int kBarUnitEmpty = kBarUnitFull + kUnits;
constexpr int kBarAccFull = kBarUnitEmpty + kUnits;
constexpr int kBarAccEmpty = kBarAccFull + 2;
constexpr int kBarFinal = kBarAccEmpty + 2;
constexpr int kNumBars = kBarFinal + 1;
constexpr int kBarOffset = kRingBytes + kLinkBytes;           // A-tile over-read (M = 128) lands in the link ring
constexpr int kMiscOffset = kBarOffset + kNumBars * 8;
constexpr int kThreads = 384;                                 // 12 warps (roles below)
// the apply: three epilogue warp pairs (0, 1), (4, 5), (8, 9) take output sites 0-2, 3-5, 6-7 of a row;
// the link producer and the MMA issuer are warps 10 and 11
constexpr int kApGroups = 3;
constexpr int kApSitesMax = 3;
constexpr int kProdWarp = 10, kMmaWarp = 11;
constexpr int kRedOffset = (kMiscOffset + 16 + 15) / 16 * 16;  // [half][32 rhs][3] doubles
constexpr int kSmemBytes = kRedOffset + kApGroups * kRhsTile * 3 * 8;
static_assert(kSmemBytes + 1024 <= 227 * 1024, "shared memory budget");
static_assert(kTileA % 16 == 0 && kRowBytes % 16 == 0 && kUnitBytes % 16 == 0, "16-byte alignment");
static_assert(2 * kAccCols <= kTmemCols, "tensor memory budget");

constexpr long long kWaitCycles = 2000000000ll;  // ~1 s at 2 GHz
constexpr long long kDrainCycles = 200000000ll;  // ~0.1 s

__device__ __forceinline__ int dir_dx(int d) { return d == 0 || d == 3 || d == 4 ? 0 : (d == 1 || d == 5 || d == 6 ? 1 : -1); }
__device__ __forceinline__ int dir_dy(int d) { return d <= 2 ? 0 : (d == 3 || d == 5 || d == 7 ? 1 : -1); }
__device__ __forceinline__ int wrapi(int a, int n) { return a < 0 ? a + n : (a >= n ? a - n : a); }

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// ------------------------------------------------------------ mbarrier / bulk copy
__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ bool mbar_try(uint32_t bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}\n"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    return ok != 0;
}
__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}
__device__ __forceinline__ void bulk_g2s(uint32_t dst, const void* src, uint32_t bytes, uint32_t bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
                 "l"(src), "r"(bytes), "r"(bar)
                 : "memory");
}
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// Wait for phase `parity` of a barrier.  Gives up when another thread of the
// CTA has raised the abort flag, or after kWaitCycles (then raises it).
__device__ __forceinline__ bool wait_bar(uint32_t bar, uint32_t parity, volatile int* abort_flag) {
    if (mbar_try(bar, parity)) return true;
    const long long t0 = clock64();
    for (int k = 1;; ++k) {
        if (mbar_try(bar, parity)) return true;
        if ((k & 31) == 0) {
            if (*abort_flag) return false;
            if (clock64() - t0 > kWaitCycles) {
                *abort_flag = 1;
                return false;
            }
        }
    }
}
// Bounded wait used while shutting down: ignores the abort flag.
__device__ __forceinline__ void drain_bar(uint32_t bar, uint32_t parity) {
    const long long t0 = clock64();
    while (!mbar_try(bar, parity))
        if (clock64() - t0 > kDrainCycles) return;
}

// ------------------------------------------------------------ tcgen05
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// Shared-memory matrix descriptor, no swizzle, K-major canonical layout:
// core matrices of 8 rows x 16 bytes; lbo = byte stride between the two core
// matrices along K, sbo = byte stride between 8-row groups.
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((addr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

// Instruction descriptor, kind::f16: D FP32, A and B BF16, both K-major, M = 128, N = n.
__host__ __device__ constexpr uint32_t idesc_bf16(uint32_t n) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((n >> 3) << 17) | ((128u >> 4) << 24);
}

__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc,
                                         uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(d_tmem),
        "l"(a), "l"(b), "r"(idesc), "r"(accumulate)
        : "memory");
}

// Source t (x = x0 - 1 + t) of a strip row feeds output sites t-2 (dx = +1),
// t-1 (dx = 0) and t (dx = -1) that lie in [0, kW): the first of them, their
// count, and the offset of their stacked link blocks inside a run.
struct SrcGroup {
    int first, count, run_off;
};
__device__ __forceinline__ SrcGroup src_group(int t) {
    const int lo = t - 2 < 0 ? 0 : t - 2, hi = t > kW - 1 ? kW - 1 : t;
    // block of (site i, dx) sits at run position 3 i + 4 + 2 dx - 2; the group's first block is
    // (lo, dx = t - 1 - lo)
    SrcGroup g;
    g.first = lo;
    g.count = hi - lo + 1;
    g.run_off = (3 * lo + 2 + 2 * (t - 1 - lo)) * kLinkDir;
    return g;
}
__device__ __forceinline__ void mma_commit(uint32_t bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}

// 32 consecutive FP32 columns of this thread's TMEM lane, waited for in the same asm block
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float (&v)[32]) {
    uint32_t r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
        "%15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];\n\t"
        "tcgen05.wait::ld.sync.aligned;"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
          "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
          "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr)
        : "memory");
#pragma unroll
    for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
    __nv_bfloat162 h = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<uint32_t*>(&h);
}

struct TcArgs {
    const uint8_t* links = nullptr;  // pre-tiled BF16 B operands, kLinkSite bytes per site
    const float2* x = nullptr;       // [site][dof][nrhs]
    float2* y = nullptr;
    const float2* w = nullptr;       // EPI 2
    // HIN: x and w in FP16 with FP32 scales, x = xh * xs[site * ssite + (rhs / 16) * shalf] (one scale
    // per site: ssite 1, shalf 0; one per site and half of the 32 rhs: ssite 2, shalf 1), w likewise
    const __half2* xh = nullptr;
    const float* xs = nullptr;
    const __half* wh = nullptr;
    const float* ws = nullptr;
    // HOUT: y in FP16 with one scale per site and rhs half (ys[2 site + rhs / 16], the half's largest
    // |re| or |im|)
    __half* yh = nullptr;
    float* ys = nullptr;
    int ssite = 1, shalf = 0;
    // EPI 2: omega[rhs] = <y, w> / ||y||^2 (0 when ||y||^2 < 1e-30 or not finite), the MR step size
    float2* omega = nullptr;
    double* partials = nullptr;
    unsigned int* tickets = nullptr;
    double* out = nullptr;
    const int* gate = nullptr;
    int* err = nullptr;
    int nx = 0, ny = 0, nrhs = 0, H = 0;
};

template <int EPI, bool HIN = false, bool HOUT = false>
__global__ void __launch_bounds__(kThreads, 1) k_coarse_apply_tc(TcArgs a) {
    if (a.gate && *a.gate == 0) return;  // every right-hand side of the solve has converged
    constexpr int K = EPI == 2 ? 3 : 1;
    extern __shared__ __align__(1024) uint8_t smem[];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int H = a.H, nx = a.nx, ny = a.ny, nrhs = a.nrhs;
    const int x0 = blockIdx.x * kW, y0 = blockIdx.y * H, rhs0 = blockIdx.z * kRhsTile;
    const uint32_t ring_a = smem_u32(smem);
    const uint32_t link_a = ring_a + kRingBytes;
    const uint32_t bar_a = ring_a + kBarOffset;
    int* misc = reinterpret_cast<int*>(smem + kMiscOffset);  // [0] TMEM base, [1] abort flag
    double* red = reinterpret_cast<double*>(smem + kRedOffset);
    volatile int* abort_flag = misc + 1;
    auto bar = [&](int i) { return bar_a + 8u * (uint32_t)i; };

    if (tid == 0) {
        for (int i = 0; i < kRing; ++i) {
            mbar_init(bar(kBarSrcFull + i), 128);
            mbar_init(bar(kBarSrcEmpty + i), 1);
        }
        for (int i = 0; i < kUnits; ++i) {
            mbar_init(bar(kBarUnitFull + i), 1);
            mbar_init(bar(kBarUnitEmpty + i), 1);
        }
        for (int i = 0; i < 2; ++i) {
            mbar_init(bar(kBarAccFull + i), 1);
            mbar_init(bar(kBarAccEmpty + i), 32 * 2 * kApGroups);
        }
        mbar_init(bar(kBarFinal), 1);
        misc[1] = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        fence_proxy_async();
    }
    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(misc)),
                     "r"(kTmemCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *reinterpret_cast<volatile uint32_t*>(misc);

    if (warp == kProdWarp) {
        // ---------------- link producer: per output row and dy one run of kRunBlocks blocks
        if (lane == 0) {
            const int ring3 = 3 * nx;  // blocks per (output row, dy) on the lattice
            int issued = 0;
            const int nunits = 3 * H;
            for (int u = 0; u < nunits; ++u) {
                const int slot = u % kUnits, use = u / kUnits;
                if (use > 0 && !wait_bar(bar(kBarUnitEmpty + slot), (use - 1) & 1, abort_flag)) break;
                const int r = u / 3, dyi = u - 3 * r;  // dy = dyi - 1
                const uint8_t* row = a.links + ((int64_t)(y0 + r) * 3 + dyi) * ring3 * kLinkDir;
                const int p0 = (3 * x0 + 2) % ring3;
                const int n1 = ring3 - p0 < kRunBlocks ? ring3 - p0 : kRunBlocks;
                const uint32_t dst = link_a + (uint32_t)(slot * kUnitBytes);
                mbar_expect_tx(bar(kBarUnitFull + slot), kUnitBytes);
                bulk_g2s(dst, row + (int64_t)p0 * kLinkDir, (uint32_t)(n1 * kLinkDir), bar(kBarUnitFull + slot));
                if (n1 < kRunBlocks)  // the run wraps around the lattice
                    bulk_g2s(dst + (uint32_t)(n1 * kLinkDir), row, (uint32_t)((kRunBlocks - n1) * kLinkDir),
                             bar(kBarUnitFull + slot));
                issued = u + 1;
            }
            // every issued copy has landed before the CTA can leave
            for (int u = issued > kUnits ? issued - kUnits : 0; u < issued; ++u)
                drain_bar(bar(kBarUnitFull + u % kUnits), (u / kUnits) & 1);
        }
        __syncwarp();
    } else if (warp == kMmaWarp) {
        // ---------------- MMA issuer: per output row, 3 dy x 10 source groups
        if (lane == 0) {
            bool ok = true;
            for (int r = 0; r < H && ok; ++r) {
                for (int lr = (r == 0 ? 0 : r + 2); lr <= r + 2 && ok; ++lr)
                    ok = wait_bar(bar(kBarSrcFull + lr % kRing), (lr / kRing) & 1, abort_flag);
                if (ok && r >= 2) ok = wait_bar(bar(kBarAccEmpty + (r & 1)), ((r >> 1) - 1) & 1, abort_flag);
                if (!ok) break;
                const uint32_t acc = tmem + (uint32_t)((r & 1) * kAccCols);
                for (int dyi = 0; dyi < 3 && ok; ++dyi) {
                    const int u = 3 * r + dyi, slot = u % kUnits;
                    ok = wait_bar(bar(kBarUnitFull + slot), (u / kUnits) & 1, abort_flag);
                    if (!ok) break;
                    tc_fence_after();
                    const int lr = r + dyi;  // source row y + dy, dy = dyi - 1
                    const uint32_t arow = ring_a + (uint32_t)((lr % kRing) * kRowBytes);
                    const uint32_t unit = link_a + (uint32_t)(slot * kUnitBytes);
#pragma unroll
                    for (int k = 0; k < kSrcSites; ++k) {
                        // the first run of a row starts every site with sources 2, 5, 8 (disjoint
                        // groups covering the row), then accumulates; later runs accumulate
                        const int t = dyi == 0 ? (k < 3 ? 2 + 3 * k : (k < 5 ? k - 3 : (k < 7 ? k - 2 : (k < 9 ? k - 1 : 9)))) : k;
                        const SrcGroup g = src_group(t);
                        const uint32_t accumulate = (dyi == 0 && k < 3) ? 0u : 1u;
                        mma_bf16(acc + (uint32_t)(32 * g.first), smem_desc(arow + (uint32_t)(t * kTileA), 128, kSboA),
                                 smem_desc(unit + (uint32_t)g.run_off, 128, 256), idesc_bf16(32u * (uint32_t)g.count),
                                 accumulate);
                    }
                    mma_commit(bar(kBarUnitEmpty + slot));  // this run of links is not read again
                }
                if (!ok) break;
                mma_commit(bar(kBarAccFull + (r & 1)));
                mma_commit(bar(kBarSrcEmpty + r % kRing));  // source row r is not read again
            }
            // all MMAs of this CTA have completed before tensor memory is freed
            mma_commit(bar(kBarFinal));
            drain_bar(bar(kBarFinal), 0);
        }
        __syncwarp();
    } else if ((warp & 3) < 2) {
        // ---------------- epilogue: TMEM lanes 0..63 hold the 64 useful rows and only warps with
        // warp % 4 = 0 (lanes 0-31) or 1 (lanes 32-63) may read them: the pairs (0, 1), (4, 5), (8, 9)
        // take sites 0-2, 3-5 and 6-7 of every output row
        const int half = warp >> 2;  // the pair's group
        const int sub = warp & 1;
        const int sbase = kApSitesMax * half, nsq = half < 2 ? kApSitesMax : kW - 2 * kApSitesMax;
        const int m = 32 * sub + lane;
        const int rhs = m >> 1, c = m & 1;
        double v[K];
#pragma unroll
        for (int k = 0; k < K; ++k) v[k] = 0.0;
        const int64_t rstride = 2ll * nrhs;  // floats between consecutive dofs
        const float* __restrict__ wbase = reinterpret_cast<const float*>(a.w);
        float* __restrict__ ybase = reinterpret_cast<float*>(a.y);
        // first entry of this thread's (rhs, re/im) for site q of the pair's half of output row r
        auto entry = [&](int r, int q) {
            return (((int64_t)x0 + sbase + q + (int64_t)nx * (y0 + r)) * kNc * nrhs + rhs0 + rhs) * 2 + c;
        };
        // EPI 2: w of site q of row r into wb[q].  Software-pipelined: row 0 is requested before the
        // first accumulator wait, row r + 1's site q right after row r's site q has used wb[q], so the
        // loads have a whole row of epilogue work to land instead of stalling every row
        float wb[kApSitesMax][kNc];
        auto load_w = [&](int r, int q) {
            const int64_t wi = entry(r, q);
            if (HIN) {
                const float sq = __ldcg(a.ws + ((x0 + sbase + q) + (int64_t)nx * (y0 + r)) * a.ssite +
                                        (rhs >> 4) * a.shalf);
#pragma unroll
                for (int k = 0; k < kNc; ++k) wb[q][k] = __half2float(__ldcg(a.wh + wi + k * rstride)) * sq;
            } else {
#pragma unroll
                for (int k = 0; k < kNc; ++k) wb[q][k] = __ldcg(wbase + wi + k * rstride);
            }
        };
        if (EPI == 2) {
#pragma unroll
            for (int q = 0; q < kApSitesMax; ++q)
                if (q < nsq) load_w(0, q);
        }
        for (int r = 0; r < H; ++r) {
            bool ok = wait_bar(bar(kBarAccFull + (r & 1)), (r >> 1) & 1, abort_flag);
            if (!__all_sync(0xffffffffu, ok)) break;
            tc_fence_after();
#pragma unroll
            for (int q = 0; q < kApSitesMax; ++q) {
                if (q >= nsq) break;
                const int i = sbase + q;
                float d[32];
                tmem_ld32(tmem + ((uint32_t)(32 * sub) << 16) + (uint32_t)((r & 1) * kAccCols + 32 * i), d);
                const int64_t base = entry(r, q);
                float o[kNc];
#pragma unroll
                for (int k = 0; k < kNc; ++k) {
                    const float other = __shfl_xor_sync(0xffffffffu, d[16 + k], 1);
                    o[k] = c == 0 ? d[k] - other : d[k] + other;
                }
                float s0 = 0.f, s1 = 0.f, s2 = 0.f;
#pragma unroll
                for (int k = 0; k < kNc; ++k) {
                    if (EPI == 1) {
                        s0 += o[k] * o[k];
                    } else if (EPI == 2) {
                        const float wc = wb[q][k];
                        s0 += o[k] * wc;  // Re <y, w>: yr wr + yi wi
                        if (!HOUT) {      // Im <y, w>: yr wi - yi wr (the FP16 MR step takes omega real:
                                          // <A r, r> is real for the Hermitian coarse operator)
                            const float wo = __shfl_xor_sync(0xffffffffu, wc, 1);
                            s1 += c == 0 ? o[k] * wo : -o[k] * wo;
                        }
                        s2 += o[k] * o[k];
                    }
                }
                if (EPI == 2 && r + 1 < H) load_w(r + 1, q);
                if (HOUT) {
                    // this warp holds the (site, rhs half sub) unit: its largest |re| or |im| is the scale
                    float mx = 0.f;
#pragma unroll
                    for (int k = 0; k < kNc; ++k) mx = fmaxf(mx, fabsf(o[k]));
                    mx = warp_max_nonneg(mx);
                    const float inv = mx > 0.f ? __fdividef(1.0f, mx) : 0.f;
#pragma unroll
                    for (int k = 0; k < kNc; ++k) a.yh[base + k * rstride] = __float2half_rn(o[k] * inv);
                    if (lane == 0) a.ys[2 * ((x0 + i) + (int64_t)nx * (y0 + r)) + sub] = mx;
                } else {
#pragma unroll
                    for (int k = 0; k < kNc; ++k) ybase[base + k * rstride] = o[k];
                }
                if (EPI == 1) {
                    v[0] += (double)s0;
                } else if (EPI == 2) {
                    v[0] += (double)s0;
                    v[1] += (double)s1;
                    v[K - 1] += (double)s2;
                }
            }
            tc_fence_before();
            mbar_arrive(bar(kBarAccEmpty + (r & 1)));
        }
        if (EPI != 0) {
#pragma unroll
            for (int k = 0; k < K; ++k) v[k] += __shfl_xor_sync(0xffffffffu, v[k], 1);
            if (c == 0)
#pragma unroll
                for (int k = 0; k < K; ++k) red[(half * kRhsTile + rhs) * K + k] = v[k];
        }
    } else if (warp < kProdWarp) {
        // ---------------- stagers (warps 2, 3, 6, 7): FP32 source rows -> BF16 A tiles
        const int st = (warp < 4 ? warp - 2 : warp - 4) * 32 + lane;  // 0..127
        for (int lr = 0; lr < H + 2; ++lr) {
            const int slot = lr % kRing, use = lr / kRing;
            if (use > 0 && !wait_bar(bar(kBarSrcEmpty + slot), (use - 1) & 1, abort_flag)) break;
            const int gy = wrapi(y0 - 1 + lr, ny);
            uint8_t* row = smem + slot * kRowBytes;
            constexpr int kItems = kSrcSites * 2 * 32;  // (site, 8-dof group, rhs)
            static_assert(kItems % 128 == 0, "stager items");
#pragma unroll
            for (int it = 0; it < kItems / 128; ++it) {
                const int item = st + it * 128;
                const int r = item & 31, g = (item >> 5) & 1, t = item >> 6;
                const int gx = wrapi(x0 - 1 + t, nx);
                const int64_t off = ((int64_t)(gx + (int64_t)nx * gy) * kNc + g * 8) * nrhs + rhs0 + r;
                float2 e[8];
                if (HIN) {
                    const float sc = __ldg(a.xs + (gx + (int64_t)nx * gy) * a.ssite + (r >> 4) * a.shalf);
#pragma unroll
                    for (int j = 0; j < 8; ++j) {
                        const float2 h = __half22float2(a.xh[off + (int64_t)j * nrhs]);
                        e[j] = make_float2(h.x * sc, h.y * sc);
                    }
                } else {
#pragma unroll
                    for (int j = 0; j < 8; ++j) e[j] = a.x[off + (int64_t)j * nrhs];
                }
                uint4 re, im;
                re.x = pack_bf16(e[0].x, e[1].x);
                re.y = pack_bf16(e[2].x, e[3].x);
                re.z = pack_bf16(e[4].x, e[5].x);
                re.w = pack_bf16(e[6].x, e[7].x);
                im.x = pack_bf16(e[0].y, e[1].y);
                im.y = pack_bf16(e[2].y, e[3].y);
                im.z = pack_bf16(e[4].y, e[5].y);
                im.w = pack_bf16(e[6].y, e[7].y);
                uint8_t* tile = row + t * kTileA;
                const int mr = 2 * r, mi = 2 * r + 1;
                *reinterpret_cast<uint4*>(tile + (mr >> 3) * kSboA + g * 128 + (mr & 7) * 16) = re;
                *reinterpret_cast<uint4*>(tile + (mi >> 3) * kSboA + g * 128 + (mi & 7) * 16) = im;
            }
            fence_proxy_async();
            mbar_arrive(bar(kBarSrcFull + slot));
        }
    }

    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == 1)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols) : "memory");
    const bool aborted = *abort_flag != 0;
    if (aborted && tid == 0 && a.err) atomicExch(a.err, 2);

    if (EPI != 0) {
        // per-rhs partials of this CTA, then the last CTA of this rhs tile sums them in block order
        const int nblk = gridDim.x * gridDim.y;
        const int blin = blockIdx.x + gridDim.x * blockIdx.y;
        __shared__ int s_last;
        if (tid < kRhsTile) {
#pragma unroll
            for (int k = 0; k < K; ++k)
                a.partials[((int64_t)(rhs0 + tid) * K + k) * nblk + blin] =
                    aborted ? 0.0
                            : (red[tid * K + k] + red[(kRhsTile + tid) * K + k]) + red[(2 * kRhsTile + tid) * K + k];
        }
        __threadfence();
        __syncthreads();
        if (tid == 0) s_last = atomicAdd(a.tickets + blockIdx.z, 1u) == (unsigned)(nblk - 1) ? 1 : 0;
        __syncthreads();
        if (s_last) {
            // each warp sums four (rhs, k) pairs at a time, lanes striding over the CTAs, so many
            // independent loads are in flight; the order is fixed (deterministic)
            __threadfence();
            constexpr int kPairs = kRhsTile * K;
            for (int p0 = warp * 4; p0 < kPairs; p0 += 4 * (kThreads / 32)) {
                double acc[4] = {0.0, 0.0, 0.0, 0.0};
                const double* src[4];
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    const int pq = p0 + q < kPairs ? p0 + q : kPairs - 1;
                    src[q] = a.partials + ((int64_t)(rhs0 + pq / K) * K + pq % K) * nblk;
                }
#pragma unroll 4
                for (int b = lane; b < nblk; b += 32) {
#pragma unroll
                    for (int q = 0; q < 4; ++q) acc[q] += __ldcg(src[q] + b);
                }
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    double v = acc[q];
                    for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
                    if (lane == 0 && p0 + q < kPairs)
                        a.out[(rhs0 + (p0 + q) / K) * K + (p0 + q) % K] = v;
                }
            }
            if (EPI == 2 && a.omega) {
                __syncthreads();  // this block's sums are in a.out
                if (tid < kRhsTile) {
                    const double* o3 = a.out + (int64_t)(rhs0 + tid) * K;
                    const double den = o3[K - 1];
                    float2 om = make_float2(0.f, 0.f);
                    if (fabs(den) >= 1e-30 && isfinite(den)) om = make_float2((float)(o3[0] / den), (float)(o3[1] / den));
                    a.omega[rhs0 + tid] = om;
                }
            }
            if (tid == 0) a.tickets[blockIdx.z] = 0u;
        }
    }
}

// B operands of every (site, direction): row n = c * 16 + i, K index j,
// value Re / Im of L[s][d](i, j) (stored [s][d][j][i]), rounded to BF16, in
// the run order of the source grouping: output row y, source row offset dy,
// position P = 3x + 4 + 2dx (mod 3 nx).  One thread writes one 16-byte
// core-matrix row (8 consecutive j).
__global__ void k_tile_links(const cx<double>* __restrict__ A, int nx, int64_t nsites, uint8_t* __restrict__ out) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nsites * 9 * 32 * 2) return;
    const int g = (int)(t & 1);
    const int n = (int)((t >> 1) & 31);
    const int64_t sd = t >> 6;  // site * 9 + d
    const int64_t site = sd / 9;
    const int d = (int)(sd - site * 9);
    const int x = (int)(site % nx), y = (int)(site / nx);
    const int cpart = n >> 4, i = n & 15;
    const cx<double>* blk = A + sd * kNc * kNc;
    float f[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        const cx<double> z = blk[(g * 8 + k) * kNc + i];
        f[k] = (float)(cpart == 0 ? z.re : z.im);
    }
    uint4 v;
    v.x = pack_bf16(f[0], f[1]);
    v.y = pack_bf16(f[2], f[3]);
    v.z = pack_bf16(f[4], f[5]);
    v.w = pack_bf16(f[6], f[7]);
    const int ring3 = 3 * nx;
    const int P = (3 * x + 4 + 2 * dir_dx(d)) % ring3;
    const int64_t block = ((int64_t)y * 3 + dir_dy(d) + 1) * ring3 + P;
    *reinterpret_cast<uint4*>(out + block * kLinkDir + (n >> 3) * 256 + g * 128 + (n & 7) * 16) = v;
}

// ------------------------------------------------------------ persistent coarsest CG
// The whole coarsest-level CG of 32 right-hand sides (SparseCoarseOp::solve without deflation,
// src/coarse_op.h:492-547) in one cooperative launch: every CTA owns the strip of kW x H sites of
// the apply above and keeps the apply's pipeline (link ring, staged source rows, tensor memory)
// across the iterations.  Per iteration k:
//   apply   the stagers form p_k = r_k + beta_{k-1} p_{k-1} on the fly for the source rows (FP16 r
//           and p_{k-1} of any CTA's sites, published before the last grid barrier) and stage it as
//           BF16; warps 0, 1, 4, 5, 8, 9 write p_k of the CTA's own sites (FP16) into the other p buffer,
//           then, as the apply's three epilogue pairs, A p_k (FP32) of the own sites with <A p_k, p_k>;
//   <A p_k, p_k> over the own sites per rhs, grid barrier, alpha_k = rr_k / <p_k, A p_k> from the
//           per-CTA partials summed in CTA order (identical, deterministic scalars in every CTA);
//   update  own sites: x += alpha p_k, r_{k+1} = r_k - alpha A p_k (FP16, new site scales), and
//           ||r_{k+1}||^2; grid barrier; beta_k, the per-rhs stop rule of the launched CG, and the
//           exit once no rhs is active.
// r and p are internal to the solve: FP16 dof-inner ([site][rhs][dof] __half2, the 16 dofs of a site
// and rhs are four 16-byte words) with one FP32 scale per site and half of the 32 rhs ([site][2]);
// b, x and A p keep the [site][dof][rhs] layout of the cycle.  The vector phases work on (site,
// half) units, one per warp: lane l takes rhs 16 h + l / 2 and dofs 8 (l & 1) .. 8 (l & 1) + 7, so
// that a warp's 16-byte accesses to r and p are one contiguous 1 KB and its accesses to b, x and
// A p two contiguous 128-byte runs per dof (whole 32-byte sectors: values other CTAs write are read
// past L1, ld.global.cg, and a half-used sector would cost a second L2 transfer).  Every phase issues
// its loads before its stores (the compiler may not move a load above a store to global memory that
// it cannot prove disjoint).  Every mbarrier and grid-barrier wait is bounded: a CTA
// that gives up raises the error word, which ends every other CTA's barrier wait.
struct CcgTcArgs {
    const uint8_t* links = nullptr;
    const float2* b = nullptr;           // [site][dof][32] right-hand side (FP32)
    float2* x = nullptr;                 // solution (FP32, [site][dof][32])
    __half2* r = nullptr;                // residual (FP16, dof-inner) and its scales [site][2]
    float* rs = nullptr;
    __half2* p[2] = {nullptr, nullptr};  // search directions (FP16, dof-inner), p_k in p[k & 1]
    float* ps[2] = {nullptr, nullptr};
    float2* Ap = nullptr;                // A p_k (FP32, [site][dof][32])
    double* part = nullptr;              // storage of the [2][32][nblk] FP32 per-CTA partial sums
    unsigned int* bar = nullptr;         // grid barrier: [0] arrivals, [1] generation
    int* err = nullptr;                  // 1 grid-barrier timeout, 2 mbarrier timeout
    int* iters = nullptr;                // iterations done (CTA 0)
    long long spin_limit = 0;
    double tol2 = 0;
    int nx = 0, ny = 0, H = 0, max_iter = 0;
};

constexpr int kCcgMaxCtas = 160;                    // partial sums: five loads per lane and rhs
// extra shared memory of the persistent CG after the apply's: scalars and reduction rows
constexpr int kCcgOffset = (kSmemBytes + 15) / 16 * 16;
constexpr int kCcgRr = kCcgOffset;                  // float [32]
constexpr int kCcgBn = kCcgRr + 32 * 4;             // float [32]
constexpr int kCcgSum = kCcgBn + 32 * 4;            // float [32]: the last grid-wide sums
constexpr int kCcgAlpha = kCcgSum + 32 * 4;         // float [32]
constexpr int kCcgBeta = kCcgAlpha + 32 * 4;        // float [32]
constexpr int kCcgAct = kCcgBeta + 32 * 4;          // int [32]
constexpr int kCcgWred = kCcgAct + 32 * 4;          // float [12][32]
constexpr int kCcgSmemBytes = kCcgWred + 12 * 32 * 4;
static_assert(kCcgSmemBytes + 1024 <= 227 * 1024, "shared memory budget (persistent CG)");

__device__ __forceinline__ float ccg_warp_max(float m) { return warp_max_nonneg(m); }
__device__ __forceinline__ float2 h2f(unsigned u) { return __half22float2(*reinterpret_cast<const __half2*>(&u)); }
__device__ __forceinline__ unsigned f2h(float re, float im) {
    const __half2 h = __floats2half2_rn(re, im);
    return *reinterpret_cast<const unsigned*>(&h);
}
__device__ __forceinline__ unsigned word_of(const uint4& w, int i) {
    return i == 0 ? w.x : (i == 1 ? w.y : (i == 2 ? w.z : w.w));
}
// the four 16-byte words of (site, rhs) of a dof-inner FP16 vector
__device__ __forceinline__ const uint4* h16_ptr(const __half2* v, int64_t site, int rhs) {
    return reinterpret_cast<const uint4*>(v) + (site * kRhsTile + rhs) * (kNc / 4);
}
__device__ __forceinline__ uint4* h16_ptr(__half2* v, int64_t site, int rhs) {
    return reinterpret_cast<uint4*>(v) + (site * kRhsTile + rhs) * (kNc / 4);
}

// grid-wide barrier of the co-resident grid; gives up after spin_limit polls or when *err is raised
__device__ __forceinline__ bool ccg_grid_barrier(unsigned int* bar, int* err, long long spin_limit) {
    __threadfence();
    __syncthreads();
    __shared__ int s_ok;
    if (threadIdx.x == 0) {
        int ok = 1;
        volatile unsigned int* vgen = bar + 1;
        volatile int* verr = err;
        if (*verr) {
            ok = 0;
        } else {
            const unsigned int gen = *vgen;
            __threadfence();
            const unsigned int nblk = gridDim.x * gridDim.y;
            if (atomicAdd(bar, 1u) == nblk - 1) {
                bar[0] = 0u;
                __threadfence();
                atomicAdd(bar + 1, 1u);
            } else {
                long long k = 0;
                while (*vgen == gen) {
                    if (*verr || ++k > spin_limit) {
                        atomicCAS(err, 0, 1);
                        ok = 0;
                        break;
                    }
                    __nanosleep(32);
                }
            }
            __threadfence();
        }
        s_ok = ok;
    }
    __syncthreads();
    return s_ok != 0;
}

// The same barrier in two halves, so that a CTA does work on its own data while the others arrive:
// ccg_barrier_arrive publishes this CTA's writes and counts it in (thread 0 keeps the generation it
// saw and whether it may wait); ccg_barrier_wait returns once every CTA has arrived, with the same
// bound and error flag as ccg_grid_barrier.  Between the two a CTA reads and writes only data no
// other CTA touches before the next barrier.
__device__ __forceinline__ void ccg_barrier_arrive(unsigned int* bar, int* err, unsigned int* s_gen, int* s_ok) {
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) {
        int ok = 1;
        volatile unsigned int* vgen = bar + 1;
        volatile int* verr = err;
        if (*verr) {
            ok = 0;
        } else {
            const unsigned int gen = *vgen;
            __threadfence();
            const unsigned int nblk = gridDim.x * gridDim.y;
            if (atomicAdd(bar, 1u) == nblk - 1) {
                bar[0] = 0u;
                __threadfence();
                atomicAdd(bar + 1, 1u);
            }
            *s_gen = gen;
        }
        *s_ok = ok;
    }
}
__device__ __forceinline__ bool ccg_barrier_wait(unsigned int* bar, int* err, long long spin_limit,
                                                 const unsigned int* s_gen, int* s_ok) {
    if (threadIdx.x == 0 && *s_ok) {
        volatile unsigned int* vgen = bar + 1;
        volatile int* verr = err;
        const unsigned int gen = *s_gen;
        long long k = 0;
        while (*vgen == gen) {
            if (*verr || ++k > spin_limit) {
                atomicCAS(err, 0, 1);
                *s_ok = 0;
                break;
            }
            __nanosleep(32);
        }
        __threadfence();
    }
    __syncthreads();
    return *s_ok != 0;
}

// out32[j] = sum over the grid's CTAs of part[j][cta] for the 32 rhs: warp w takes rhs w, w + 12,
// w + 24 with all its loads issued first, lanes stride the CTAs, then a fixed shuffle tree (the same
// order in every CTA).  The CG's scalars are FP32: the coarsest solve runs to a tolerance of a few
// per cent, and FP64 arithmetic, scarce on this part, put microseconds of latency on every sum.
__device__ __forceinline__ void ccg_sum_partials(const float* part, int nblk, float* out32) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    float v[3][5];
#pragma unroll
    for (int q = 0; q < 3; ++q) {
        const int j = warp + (kThreads / 32) * q;
#pragma unroll
        for (int u = 0; u < 5; ++u) {
            const int c = lane + 32 * u;
            v[q][u] = (j < 32 && c < nblk) ? __ldcg(part + (int64_t)j * nblk + c) : 0.f;
        }
    }
#pragma unroll
    for (int q = 0; q < 3; ++q) {
        const int j = warp + (kThreads / 32) * q;
        float s = ((v[q][0] + v[q][1]) + (v[q][2] + v[q][3])) + v[q][4];
        for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if (lane == 0 && j < 32) out32[j] = s;
    }
}

// this CTA's per-rhs partial part[rhs][blin] from the lanes' unit sums acc[h] (rhs 16 h + lane / 2,
// the two lanes of an rhs already combined; lanes with odd index hold copies)
__device__ __forceinline__ void ccg_publish(float* s_wred, const float (&acc)[2], float* part, int nblk, int blin) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if ((lane & 1) == 0) {
        s_wred[warp * 32 + (lane >> 1)] = acc[0];
        s_wred[warp * 32 + 16 + (lane >> 1)] = acc[1];
    }
    __syncthreads();
    if (threadIdx.x < 32) {
        float t = 0.f;
#pragma unroll
        for (int w = 0; w < kThreads / 32; ++w) t += s_wred[w * 32 + threadIdx.x];
        part[(int64_t)threadIdx.x * nblk + blin] = t;
    }
}

// 8 dofs (two 16-byte words) of a dof-inner FP16 vector as complex floats times a scale
__device__ __forceinline__ void h8_unpack(const uint4& w0, const uint4& w1, float s, float2 (&v)[8]) {
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        const float2 a = h2f(word_of(w0, j)), b = h2f(word_of(w1, j));
        v[j] = make_float2(a.x * s, a.y * s);
        v[4 + j] = make_float2(b.x * s, b.y * s);
    }
}
__device__ __forceinline__ void h8_pack(const float2 (&v)[8], float inv, uint4& w0, uint4& w1) {
    w0.x = f2h(v[0].x * inv, v[0].y * inv);
    w0.y = f2h(v[1].x * inv, v[1].y * inv);
    w0.z = f2h(v[2].x * inv, v[2].y * inv);
    w0.w = f2h(v[3].x * inv, v[3].y * inv);
    w1.x = f2h(v[4].x * inv, v[4].y * inv);
    w1.y = f2h(v[5].x * inv, v[5].y * inv);
    w1.z = f2h(v[6].x * inv, v[6].y * inv);
    w1.w = f2h(v[7].x * inv, v[7].y * inv);
}

__global__ void __launch_bounds__(kThreads, 1) k_ccg_tc(CcgTcArgs a) {
    extern __shared__ __align__(1024) uint8_t smem[];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int H = a.H, nx = a.nx, ny = a.ny;
    constexpr int nrhs = kRhsTile;
    const int x0 = blockIdx.x * kW, y0 = blockIdx.y * H;
    const int nblk = gridDim.x * gridDim.y, blin = blockIdx.x + gridDim.x * blockIdx.y;
    const int nunit = 2 * kW * H;  // (own site, rhs half) units
    const uint32_t ring_a = smem_u32(smem);
    const uint32_t link_a = ring_a + kRingBytes;
    const uint32_t bar_a = ring_a + kBarOffset;
    int* misc = reinterpret_cast<int*>(smem + kMiscOffset);  // [0] TMEM base, [1] abort flag
    float* s_rr = reinterpret_cast<float*>(smem + kCcgRr);
    float* s_bn = reinterpret_cast<float*>(smem + kCcgBn);
    float* s_sum = reinterpret_cast<float*>(smem + kCcgSum);
    float* s_alpha = reinterpret_cast<float*>(smem + kCcgAlpha);
    float* s_beta = reinterpret_cast<float*>(smem + kCcgBeta);
    int* s_act = reinterpret_cast<int*>(smem + kCcgAct);
    float* s_wred = reinterpret_cast<float*>(smem + kCcgWred);
    volatile int* abort_flag = misc + 1;
    __shared__ unsigned int s_gen[1];  // the split barrier's generation and go flag (thread 0)
    __shared__ int s_ok[1];
    auto bar = [&](int i) { return bar_a + 8u * (uint32_t)i; };
    float* part1 = reinterpret_cast<float*>(a.part);  // <A p, p> partials
    float* part2 = part1 + (int64_t)32 * nblk;         // ||r||^2 partials
    // unit u: own site u / 2 of the strip, rhs half u & 1; this lane's rhs and dof half
    const int lrhs = lane >> 1, dh = lane & 1;
    auto unit_site = [&](int u) {
        const int s = u >> 1;
        return (int64_t)(x0 + s % kW) + (int64_t)nx * (y0 + s / kW);
    };
    // [site][dof][rhs] index of (site, dof 8 dh, rhs) for b, x and A p
    auto e_of = [&](int64_t site, int rhs) { return (site * kNc + 8 * dh) * nrhs + rhs; };

    if (tid == 0) {
        for (int i = 0; i < kRing; ++i) {
            mbar_init(bar(kBarSrcFull + i), 128);
            mbar_init(bar(kBarSrcEmpty + i), 1);
        }
        for (int i = 0; i < kUnits; ++i) {
            mbar_init(bar(kBarUnitFull + i), 1);
            mbar_init(bar(kBarUnitEmpty + i), 1);
        }
        for (int i = 0; i < 2; ++i) {
            mbar_init(bar(kBarAccFull + i), 1);
            mbar_init(bar(kBarAccEmpty + i), 32 * 2 * kApGroups);
        }
        mbar_init(bar(kBarFinal), 1);
        misc[1] = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        fence_proxy_async();
    }
    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(misc)),
                     "r"(kTmemCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *reinterpret_cast<volatile uint32_t*>(misc);

    // ---- start: r = b (FP16), x = 0, p_{-1} = 0 in p[1], ||b||^2 per rhs
    {
        float acc[2] = {0.f, 0.f};
        for (int u = warp; u < nunit; u += kThreads / 32) {
            const int64_t site = unit_site(u);
            const int h = u & 1, rhs = 16 * h + lrhs;
            const int64_t e0 = e_of(site, rhs);
            float2 v[8];
#pragma unroll
            for (int j = 0; j < 8; ++j) v[j] = __ldcg(a.b + e0 + j * nrhs);
            float m = 0.f, n2 = 0.f;
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                m = fmaxf(m, fmaxf(fabsf(v[j].x), fabsf(v[j].y)));
                n2 += v[j].x * v[j].x + v[j].y * v[j].y;
            }
            m = ccg_warp_max(m);
            uint4 w0, w1;
            h8_pack(v, m > 0.f ? __fdividef(1.0f, m) : 0.f, w0, w1);
            uint4* rp = h16_ptr(a.r, site, rhs) + 2 * dh;
            uint4* pp = h16_ptr(a.p[1], site, rhs) + 2 * dh;
            __stcg(rp, w0);
            __stcg(rp + 1, w1);
            __stcg(pp, make_uint4(0u, 0u, 0u, 0u));
            __stcg(pp + 1, make_uint4(0u, 0u, 0u, 0u));
#pragma unroll
            for (int j = 0; j < 8; ++j) __stcg(a.x + e0 + j * nrhs, make_float2(0.f, 0.f));
            if (lane == 0) {
                __stcg(a.rs + 2 * site + h, m);
                __stcg(a.ps[1] + 2 * site + h, 0.f);
            }
            const float n2r = n2 + __shfl_xor_sync(0xffffffffu, n2, 1);  // the rhs's two lanes
            if (h) acc[1] += n2r;
            else acc[0] += n2r;
        }
        ccg_publish(s_wred, acc, part2, nblk, blin);
    }
    bool ok = ccg_grid_barrier(a.bar, a.err, a.spin_limit);
    if (ok) {
        ccg_sum_partials(part2, nblk, s_sum);
        __syncthreads();
        if (tid < 32) {
            const float rr = s_sum[tid];
            s_rr[tid] = rr;
            s_bn[tid] = rr;
            s_beta[tid] = 0.f;
            int act = (rr >= 1e-30f && isfinite(rr)) ? 1 : 0;
            if (act && rr < (float)a.tol2 * rr) act = 0;
            s_act[tid] = act;
        }
    }
    int iter = 0;
    int nact = ok ? __syncthreads_count(tid < 32 && s_act[tid]) : 0;
    int issued = 0;  // link units issued by the producer (lane 0 of warp 0)
    const int nunits = 3 * H;
    for (int k = 0; ok && nact > 0 && k < a.max_iter; ++k) {
        const __half2* __restrict__ pold = a.p[(k + 1) & 1];
        const float* __restrict__ psold = a.ps[(k + 1) & 1];
        __half2* __restrict__ pnew = a.p[k & 1];
        float* __restrict__ psnew = a.ps[k & 1];
        const int ub = k * nunits, sb = k * (H + 2), ab = k * H;  // unit, source-row and output-row bases
        // ================= apply: A p_k with the apply kernel's warp roles
        if (warp == kProdWarp) {
            if (lane == 0) {
                const int ring3 = 3 * nx;
                for (int u = 0; u < nunits; ++u) {
                    const int U = ub + u, slot = U % kUnits, use = U / kUnits;
                    if (use > 0 && !wait_bar(bar(kBarUnitEmpty + slot), (use - 1) & 1, abort_flag)) break;
                    const int r = u / 3, dyi = u - 3 * r;
                    const uint8_t* row = a.links + ((int64_t)(y0 + r) * 3 + dyi) * ring3 * kLinkDir;
                    const int p0 = (3 * x0 + 2) % ring3;
                    const int n1 = ring3 - p0 < kRunBlocks ? ring3 - p0 : kRunBlocks;
                    const uint32_t dst = link_a + (uint32_t)(slot * kUnitBytes);
                    mbar_expect_tx(bar(kBarUnitFull + slot), kUnitBytes);
                    bulk_g2s(dst, row + (int64_t)p0 * kLinkDir, (uint32_t)(n1 * kLinkDir), bar(kBarUnitFull + slot));
                    if (n1 < kRunBlocks)
                        bulk_g2s(dst + (uint32_t)(n1 * kLinkDir), row, (uint32_t)((kRunBlocks - n1) * kLinkDir),
                                 bar(kBarUnitFull + slot));
                    issued = U + 1;
                }
            }
            __syncwarp();
        } else if (warp == kMmaWarp) {
            if (lane == 0) {
                bool mok = true;
                for (int r = 0; r < H && mok; ++r) {
                    const int R = ab + r;
                    for (int lr = (r == 0 ? 0 : r + 2); lr <= r + 2 && mok; ++lr) {
                        const int S = sb + lr;
                        mok = wait_bar(bar(kBarSrcFull + S % kRing), (S / kRing) & 1, abort_flag);
                    }
                    if (mok && R >= 2) mok = wait_bar(bar(kBarAccEmpty + (R & 1)), ((R >> 1) - 1) & 1, abort_flag);
                    if (!mok) break;
                    const uint32_t acc = tmem + (uint32_t)((R & 1) * kAccCols);
                    for (int dyi = 0; dyi < 3 && mok; ++dyi) {
                        const int U = ub + 3 * r + dyi, slot = U % kUnits;
                        mok = wait_bar(bar(kBarUnitFull + slot), (U / kUnits) & 1, abort_flag);
                        if (!mok) break;
                        tc_fence_after();
                        const int S = sb + r + dyi;
                        const uint32_t arow = ring_a + (uint32_t)((S % kRing) * kRowBytes);
                        const uint32_t unit = link_a + (uint32_t)(slot * kUnitBytes);
#pragma unroll
                        for (int kk = 0; kk < kSrcSites; ++kk) {
                            const int t = dyi == 0 ? (kk < 3 ? 2 + 3 * kk : (kk < 5 ? kk - 3 : (kk < 7 ? kk - 2 : (kk < 9 ? kk - 1 : 9)))) : kk;
                            const SrcGroup g = src_group(t);
                            const uint32_t accumulate = (dyi == 0 && kk < 3) ? 0u : 1u;
                            mma_bf16(acc + (uint32_t)(32 * g.first), smem_desc(arow + (uint32_t)(t * kTileA), 128, kSboA),
                                     smem_desc(unit + (uint32_t)g.run_off, 128, 256),
                                     idesc_bf16(32u * (uint32_t)g.count), accumulate);
                        }
                        mma_commit(bar(kBarUnitEmpty + slot));
                    }
                    if (!mok) break;
                    mma_commit(bar(kBarAccFull + (R & 1)));
                    mma_commit(bar(kBarSrcEmpty + (sb + r) % kRing));
                }
                // the iteration's last two source rows are free once its MMAs complete
                if (mok) {
                    mma_commit(bar(kBarSrcEmpty + (sb + H) % kRing));
                    mma_commit(bar(kBarSrcEmpty + (sb + H + 1) % kRing));
                }
            }
            __syncwarp();
        } else if ((warp & 3) >= 2) {
            // stagers (warps 2, 3, 6, 7): p_k = r_k + beta p_{k-1} (FP16 inputs with scales) -> BF16 A tiles.  Item i of a
            // source row: site i / 128 of the row, rhs (i / 4) % 32, word i % 4 (dofs 4 (i % 4) ..
            // + 3): a warp's items are 8 rhs x 4 words of one site, 512 contiguous bytes of r and p
            const int st = (warp < 4 ? warp - 2 : warp - 4) * 32 + lane;
            constexpr int kItems = kSrcSites * 32 * 4;
            constexpr int kPer = kItems / 128;  // 10
            constexpr int kBatch = 10;
            for (int lr = 0; lr < H + 2; ++lr) {
                const int S = sb + lr, slot = S % kRing, use = S / kRing;
                if (use > 0 && !wait_bar(bar(kBarSrcEmpty + slot), (use - 1) & 1, abort_flag)) break;
                const int gy = wrapi(y0 - 1 + lr, ny);
                uint8_t* row = smem + slot * kRowBytes;
#pragma unroll
                for (int b0 = 0; b0 < kPer; b0 += kBatch) {
                    uint4 rv[kBatch], pv[kBatch];
                    float sr[kBatch], sp[kBatch];
#pragma unroll
                    for (int q = 0; q < kBatch; ++q) {  // the batch's loads first
                        const int i = st + 128 * (b0 + q);
                        const int t = i >> 7, r = (i >> 2) & 31, wq = i & 3;
                        const int64_t site = wrapi(x0 - 1 + t, nx) + (int64_t)nx * gy;
                        rv[q] = __ldcg(h16_ptr(a.r, site, r) + wq);
                        pv[q] = __ldcg(h16_ptr(pold, site, r) + wq);
                        sr[q] = __ldcg(a.rs + 2 * site + (r >> 4));
                        sp[q] = __ldcg(psold + 2 * site + (r >> 4)) * s_beta[r];
                    }
#pragma unroll
                    for (int q = 0; q < kBatch; ++q) {
                        const int i = st + 128 * (b0 + q);
                        const int t = i >> 7, r = (i >> 2) & 31, wq = i & 3;
                        float2 e[4];
#pragma unroll
                        for (int j = 0; j < 4; ++j) {
                            const float2 a2 = h2f(word_of(rv[q], j)), b2 = h2f(word_of(pv[q], j));
                            e[j] = make_float2(fmaf(sr[q], a2.x, sp[q] * b2.x), fmaf(sr[q], a2.y, sp[q] * b2.y));
                        }
                        const uint2 re = make_uint2(pack_bf16(e[0].x, e[1].x), pack_bf16(e[2].x, e[3].x));
                        const uint2 im = make_uint2(pack_bf16(e[0].y, e[1].y), pack_bf16(e[2].y, e[3].y));
                        uint8_t* tile = row + t * kTileA + (wq >> 1) * 128 + (wq & 1) * 8;
                        const int mr = 2 * r, mi = 2 * r + 1;
                        *reinterpret_cast<uint2*>(tile + (mr >> 3) * kSboA + (mr & 7) * 16) = re;
                        *reinterpret_cast<uint2*>(tile + (mi >> 3) * kSboA + (mi & 7) * 16) = im;
                    }
                }
                fence_proxy_async();
                mbar_arrive(bar(kBarSrcFull + slot));
            }
        } else {
            // warps 0, 1, 4, 5, 8, 9: p_k of the own sites -> p[k & 1] (FP16, scale per unit = its
            // largest |re| or |im|), then the epilogue; warp pw takes units pw, pw + 6, ..., four per
            // step with all four units' loads first
            const int pw = 2 * (warp >> 2) + (warp & 1);  // 0 .. 5
            constexpr int kPw = 6, kPq = 4;
            for (int u0 = pw; u0 < nunit; u0 += kPq * kPw) {
                uint4 rv[kPq][2], pv[kPq][2];
                float sr[kPq], sp[kPq];
#pragma unroll
                for (int q = 0; q < kPq; ++q) {
                    const int u = u0 + q * kPw < nunit ? u0 + q * kPw : u0;
                    const int64_t site = unit_site(u);
                    const int h = u & 1, rhs = 16 * h + lrhs;
                    const uint4* rp = h16_ptr(a.r, site, rhs) + 2 * dh;
                    const uint4* pp = h16_ptr(pold, site, rhs) + 2 * dh;
                    rv[q][0] = __ldcg(rp);
                    rv[q][1] = __ldcg(rp + 1);
                    pv[q][0] = __ldcg(pp);
                    pv[q][1] = __ldcg(pp + 1);
                    sr[q] = __ldcg(a.rs + 2 * site + h);
                    sp[q] = __ldcg(psold + 2 * site + h) * s_beta[rhs];
                }
#pragma unroll
                for (int q = 0; q < kPq; ++q) {
                    const int u = u0 + q * kPw;
                    if (u >= nunit) break;
                    const int64_t site = unit_site(u);
                    const int h = u & 1, rhs = 16 * h + lrhs;
                    float2 v[8], pr[8];
                    h8_unpack(rv[q][0], rv[q][1], sr[q], v);
                    h8_unpack(pv[q][0], pv[q][1], sp[q], pr);
                    float mx = 0.f;
#pragma unroll
                    for (int j = 0; j < 8; ++j) {
                        v[j] = make_float2(v[j].x + pr[j].x, v[j].y + pr[j].y);
                        mx = fmaxf(mx, fmaxf(fabsf(v[j].x), fabsf(v[j].y)));
                    }
                    mx = ccg_warp_max(mx);
                    uint4 w0, w1;
                    h8_pack(v, mx > 0.f ? __fdividef(1.0f, mx) : 0.f, w0, w1);
                    uint4* op = h16_ptr(pnew, site, rhs) + 2 * dh;
                    __stcg(op, w0);
                    __stcg(op + 1, w1);
                    if (lane == 0) __stcg(psnew + 2 * site + h, mx);
                }
            }
            // the six warps' own p_k is complete before the epilogue reads it back (named barrier 1)
            asm volatile("bar.sync 1, 192;" ::: "memory");
            {
                // epilogue: A p_k of the own sites to global memory and <A p_k, p_k> per rhs (p_k of
                // the row's sites requested before the row's accumulator wait); the pairs (0, 1),
                // (4, 5), (8, 9) take sites 0-2, 3-5 and 6-7 of every row
                const int half = warp >> 2;  // the pair's group
                const int sub = warp & 1;
                const int sbase = kApSitesMax * half, nsq = half < 2 ? kApSitesMax : kW - 2 * kApSitesMax;
                const int m = 32 * sub + lane;
                const int rhs = m >> 1, c = m & 1;
                const int64_t rstride = 2ll * nrhs;
                float* __restrict__ ybase = reinterpret_cast<float*>(a.Ap);
                float dot = 0.f;
                // p_k of site q of row r (16 dofs of this lane's rhs: four 16-byte words) and its scale
                auto load_p = [&](int r, int q, uint4 (&w)[4], float& sc) {
                    const int64_t site = (int64_t)x0 + sbase + (q < nsq ? q : 0) + (int64_t)nx * (y0 + r);
                    const uint4* pp = h16_ptr(pnew, site, rhs);
#pragma unroll
                    for (int w4 = 0; w4 < 4; ++w4) w[w4] = __ldcg(pp + w4);
                    sc = __ldcg(psnew + 2 * site + (rhs >> 4));
                };
                for (int r = 0; r < H; ++r) {
                    const int R = ab + r;
                    uint4 pw[2][4];  // sites q and q + 1 in flight
                    float psq[2];
                    load_p(r, 0, pw[0], psq[0]);
                    load_p(r, 1, pw[1], psq[1]);
                    const bool eok = wait_bar(bar(kBarAccFull + (R & 1)), (R >> 1) & 1, abort_flag);
                    if (!__all_sync(0xffffffffu, eok)) break;
                    tc_fence_after();
#pragma unroll
                    for (int q = 0; q < kApSitesMax; ++q) {
                        if (q >= nsq) break;
                        const int i = sbase + q;
                        float d[32];
                        tmem_ld32(tmem + ((uint32_t)(32 * sub) << 16) + (uint32_t)((R & 1) * kAccCols + 32 * i), d);
                        const int64_t base = (((int64_t)x0 + i + (int64_t)nx * (y0 + r)) * kNc * nrhs + rhs) * 2 + c;
                        float t = 0.f;
#pragma unroll
                        for (int kk = 0; kk < kNc; ++kk) {
                            const float other = __shfl_xor_sync(0xffffffffu, d[16 + kk], 1);
                            const float y = c == 0 ? d[kk] - other : d[kk] + other;
                            __stcg(ybase + base + kk * rstride, y);
                            const float2 p2 = h2f(word_of(pw[q & 1][kk >> 2], kk & 3));
                            t += y * (c == 0 ? p2.x : p2.y);
                        }
                        dot += psq[q & 1] * t;
                        if (q + 2 < nsq) load_p(r, q + 2, pw[q & 1], psq[q & 1]);
                    }
                    tc_fence_before();
                    mbar_arrive(bar(kBarAccEmpty + (R & 1)));
                }
                // Re <A p, p> of this warp's 16 rhs: the two lanes of an rhs combined
                dot += __shfl_xor_sync(0xffffffffu, dot, 1);
                if (c == 0) reinterpret_cast<float*>(smem + kRedOffset)[half * kRhsTile + rhs] = dot;
            }
        }
        tc_fence_before();
        __syncthreads();
        tc_fence_after();
        if (*abort_flag) {
            if (tid == 0) atomicCAS(a.err, 0, 2);
            break;
        }
        // ================= <A p_k, p_k>: the epilogue's per-warp sums as this CTA's partials
        if (tid < 32) {
            const float* ed = reinterpret_cast<const float*>(smem + kRedOffset);
            part1[(int64_t)tid * nblk + blin] = (ed[tid] + ed[kRhsTile + tid]) + ed[2 * kRhsTile + tid];
        }
        ok = ccg_grid_barrier(a.bar, a.err, a.spin_limit);
        if (!ok) break;
        ccg_sum_partials(part1, nblk, s_sum);
        __syncthreads();
        if (tid < 32) {
            float al = 0.f;
            const float pap = s_sum[tid];
            if (s_act[tid] && fabsf(pap) >= 1e-30f && isfinite(pap)) al = s_rr[tid] / pap;
            s_alpha[tid] = al;
        }
        __syncthreads();
        // ================= r update of the own sites: kUq units per step, all their loads first (x
        // moves in the second barrier's wait, below)
        {
            float acc[2] = {0.f, 0.f};
            constexpr int kW32 = kThreads / 32, kUq = 3;
            for (int u0 = warp; u0 < nunit; u0 += kUq * kW32) {
                uint4 rw[kUq][2];
                float2 av[kUq][8];
                float sr[kUq];
#pragma unroll
                for (int q = 0; q < kUq; ++q) {
                    const int u = u0 + q * kW32 < nunit ? u0 + q * kW32 : u0;
                    const int64_t site = unit_site(u);
                    const int h = u & 1, rhs = 16 * h + lrhs;
                    const int64_t e0 = e_of(site, rhs);
                    const uint4* rp = h16_ptr(a.r, site, rhs) + 2 * dh;
                    rw[q][0] = __ldcg(rp);
                    rw[q][1] = __ldcg(rp + 1);
#pragma unroll
                    for (int j = 0; j < 8; ++j) av[q][j] = __ldcg(a.Ap + e0 + j * nrhs);
                    sr[q] = __ldcg(a.rs + 2 * site + h);
                }
#pragma unroll
                for (int q = 0; q < kUq; ++q) {
                    const int u = u0 + q * kW32;
                    if (u >= nunit) break;
                    const int64_t site = unit_site(u);
                    const int h = u & 1, rhs = 16 * h + lrhs;
                    const float al = s_alpha[rhs];
                    float2 rv[8];
                    h8_unpack(rw[q][0], rw[q][1], sr[q], rv);
                    float mx = 0.f, n2 = 0.f;
#pragma unroll
                    for (int j = 0; j < 8; ++j) {
                        rv[j] = make_float2(rv[j].x - al * av[q][j].x, rv[j].y - al * av[q][j].y);
                        mx = fmaxf(mx, fmaxf(fabsf(rv[j].x), fabsf(rv[j].y)));
                        n2 += rv[j].x * rv[j].x + rv[j].y * rv[j].y;
                    }
                    mx = ccg_warp_max(mx);  // also orders every lane's scale read before lane 0's write
                    uint4 w0, w1;
                    h8_pack(rv, mx > 0.f ? __fdividef(1.0f, mx) : 0.f, w0, w1);
                    uint4* wp = h16_ptr(a.r, site, rhs) + 2 * dh;
                    __stcg(wp, w0);
                    __stcg(wp + 1, w1);
                    if (lane == 0) __stcg(a.rs + 2 * site + h, mx);
                    const float v = n2 + __shfl_xor_sync(0xffffffffu, n2, 1);  // the rhs's two lanes
                    if (h) acc[1] += v;
                    else acc[0] += v;
                }
            }
            ccg_publish(s_wred, acc, part2, nblk, blin);
        }
        // ================= x += alpha_k p_k of the own sites while the other CTAs arrive: x and
        // p_k's own-site entries are this CTA's alone until p_k's buffer is rewritten in iteration k + 2
        ccg_barrier_arrive(a.bar, a.err, s_gen, s_ok);
        {
            constexpr int kW32 = kThreads / 32, kXq = 3;
            for (int u0 = warp; u0 < nunit; u0 += kXq * kW32) {
                uint4 pw[kXq][2];
                float2 xv[kXq][8];
                float sp[kXq];
#pragma unroll
                for (int q = 0; q < kXq; ++q) {
                    const int u = u0 + q * kW32 < nunit ? u0 + q * kW32 : u0;
                    const int64_t site = unit_site(u);
                    const int h = u & 1, rhs = 16 * h + lrhs;
                    const int64_t e0 = e_of(site, rhs);
                    const uint4* pp = h16_ptr(pnew, site, rhs) + 2 * dh;
                    pw[q][0] = __ldcg(pp);
                    pw[q][1] = __ldcg(pp + 1);
#pragma unroll
                    for (int j = 0; j < 8; ++j) xv[q][j] = __ldcg(a.x + e0 + j * nrhs);
                    sp[q] = __ldcg(psnew + 2 * site + h);
                }
#pragma unroll
                for (int q = 0; q < kXq; ++q) {
                    const int u = u0 + q * kW32;
                    if (u >= nunit) break;
                    const int64_t site = unit_site(u);
                    const int h = u & 1, rhs = 16 * h + lrhs;
                    const int64_t e0 = e_of(site, rhs);
                    float2 pv[8];
                    h8_unpack(pw[q][0], pw[q][1], s_alpha[rhs] * sp[q], pv);
#pragma unroll
                    for (int j = 0; j < 8; ++j)
                        __stcg(a.x + e0 + j * nrhs, make_float2(xv[q][j].x + pv[j].x, xv[q][j].y + pv[j].y));
                }
            }
        }
        ok = ccg_barrier_wait(a.bar, a.err, a.spin_limit, s_gen, s_ok);
        if (!ok) break;
        // ================= beta_k and the stop rule (the launched CG's finaliser)
        ccg_sum_partials(part2, nblk, s_sum);
        __syncthreads();
        if (tid < 32) {
            const float rr_new = s_sum[tid];
            float be = 0.f;
            if (s_act[tid]) {
                if (!isfinite(rr_new) || rr_new < (float)a.tol2 * s_bn[tid]) {
                    s_act[tid] = 0;
                } else {
                    be = rr_new / s_rr[tid];
                    s_rr[tid] = rr_new;
                }
            }
            s_beta[tid] = be;
        }
        iter = k + 1;
        nact = __syncthreads_count(tid < 32 && s_act[tid]);
    }
    if (blin == 0 && tid == 0 && a.iters) *a.iters = iter;

    // ---- teardown: every issued bulk copy and MMA has completed before tensor memory is freed
    if (warp == kProdWarp && lane == 0)
        for (int U = issued > kUnits ? issued - kUnits : 0; U < issued; ++U)
            drain_bar(bar(kBarUnitFull + U % kUnits), (U / kUnits) & 1);
    if (warp == kMmaWarp && lane == 0) {
        mma_commit(bar(kBarFinal));
        drain_bar(bar(kBarFinal), 0);
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == 1)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols) : "memory");
    if (*abort_flag && tid == 0 && a.err) atomicCAS(a.err, 0, 2);
}

int rows_per_cta_rule(int nx, int ny, int nz) {
    int H = ny;
    while (H % 2 == 0 && H > 4 && (nx / kW) * (ny / H) * nz < 120) H /= 2;
    return H;
}

// Rows per CTA chosen by timing for a lattice and right-hand-side count (smg_coarse_tc_tune); the
// rule above until then.  Shared by every context of the process.
smg_status launch_tc(smg_context* ctx, const void* links, int nx, int ny, int nrhs, int H, const cx<float>* x,
                     cx<float>* y, int epi, const cx<float>* w, double* out, const int* gate, int* err,
                     const TcArgs* half_in = nullptr);

std::mutex g_rows_mu;
std::map<std::tuple<int, int, int>, int> g_rows;

int rows_per_cta(int nx, int ny, int nz) {
    std::lock_guard<std::mutex> lock(g_rows_mu);
    auto it = g_rows.find(std::make_tuple(nx, ny, nz));
    return it != g_rows.end() ? it->second : rows_per_cta_rule(nx, ny, nz);
}

}  // namespace

bool smg_coarse_tc_shape_ok(int nx, int ny, int ndof) { return ndof == kNc && nx % kW == 0 && nx > 0 && ny > 0; }

size_t smg_coarse_tc_link_bytes(int64_t nsites) { return (size_t)nsites * kLinkSite; }

smg_status smg_coarse_tc_tile_links(smg_context* ctx, const cx<double>* A64, int nx, int64_t nsites, void* out) {
    const int64_t n = nsites * 9 * 32 * 2;
    k_tile_links<<<(unsigned)((n + 255) / 256), 256, 0, ctx->stream>>>(A64, nx, nsites, static_cast<uint8_t*>(out));
    count_launch(ctx);
    SMG_CHECK_LAUNCH(ctx);
    // the apply kernels need more than the default 48 KB of dynamic shared memory
    SMG_CUDA(ctx, cudaFuncSetAttribute(k_coarse_apply_tc<0>, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemBytes));
    SMG_CUDA(ctx, cudaFuncSetAttribute(k_coarse_apply_tc<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemBytes));
    SMG_CUDA(ctx, cudaFuncSetAttribute(k_coarse_apply_tc<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemBytes));
    SMG_CUDA(ctx, cudaFuncSetAttribute(k_coarse_apply_tc<2, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       kSmemBytes));
    SMG_CUDA(ctx, cudaFuncSetAttribute(k_coarse_apply_tc<2, true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       kSmemBytes));
    SMG_CUDA(ctx, cudaFuncSetAttribute(k_ccg_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, kCcgSmemBytes));
    return SMG_OK;
}

// y = A x on nrhs (a multiple of 32) right-hand sides; epi 1 adds ||y||^2 and
// epi 2 <y, w> and ||y||^2 per rhs into out[rhs * K + k] (K = 1 or 3).
smg_status smg_coarse_tc_apply(smg_context* ctx, const void* links, int nx, int ny, int nrhs, const cx<float>* x,
                               cx<float>* y, int epi, const cx<float>* w, double* out, const int* gate, int* err) {
    if (!smg_coarse_tc_shape_ok(nx, ny, kNc) || nrhs % kRhsTile != 0 || nrhs / kRhsTile > kMaxTickets)
        return smg_fail(ctx, SMG_UNSUPPORTED, "tensor-core coarse apply: shape not supported");
    const int nz = nrhs / kRhsTile;
    return launch_tc(ctx, links, nx, ny, nrhs, rows_per_cta(nx, ny, nz), x, y, epi, w, out, gate, err);
}

// y = A x with x and w in FP16 with one FP32 scale per site ([site][dof][rhs] __half2, scales
// [site]) and the fused <y, w>, ||y||^2 per rhs; y in FP32
smg_status smg_coarse_tc_apply_h(smg_context* ctx, const void* links, int nx, int ny, int nrhs, const void* xh,
                                 const float* xs, cx<float>* y, const void* wh, const float* ws, double* out,
                                 const int* gate, int* err) {
    if (!smg_coarse_tc_shape_ok(nx, ny, kNc) || nrhs % kRhsTile != 0 || nrhs / kRhsTile > kMaxTickets || !xh ||
        !xs || !wh || !ws)
        return smg_fail(ctx, SMG_UNSUPPORTED, "tensor-core coarse apply on FP16 vectors: shape not supported");
    TcArgs h;
    h.xh = static_cast<const __half2*>(xh);
    h.xs = xs;
    h.wh = static_cast<const __half*>(wh);
    h.ws = ws;
    const int nz = nrhs / kRhsTile;
    return launch_tc(ctx, links, nx, ny, nrhs, rows_per_cta(nx, ny, nz), nullptr, y, 2, nullptr, out, gate, err, &h);
}

// Rows per CTA of the persistent coarsest CG: the fewest (smallest power-of-two divisor of ny, or ny)
// whose CTAs are all co-resident (one per SM); 0 when the shape does not fit.
int smg_coarse_cg_tc_rows(smg_context* ctx, int nx, int ny) {
    if (!smg_coarse_tc_shape_ok(nx, ny, kNc)) return 0;
    static int per_sm = -1;
    if (per_sm < 0) {
        int nb = 0;
        if (cudaFuncSetAttribute(k_ccg_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, kCcgSmemBytes) != cudaSuccess ||
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_ccg_tc, kThreads, kCcgSmemBytes) != cudaSuccess)
            nb = 0;
        per_sm = nb;
    }
    const int cap = per_sm * ctx->num_sms;
    for (int H = 1; H <= ny; H *= 2) {
        if (ny % H) break;
        if ((nx / kW) * (ny / H) <= cap && (nx / kW) * (ny / H) <= kCcgMaxCtas) return H;
    }
    return 0;
}

// The coarsest CG of 32 right-hand sides from x = 0 in one cooperative launch (k_ccg_tc): b and x
// FP32 [site][dof][32]; r, p0, p1 FP16 (__half2) with per-site scales rs, ps0, ps1; Ap FP32; part
// 64 * (CTAs) doubles; state: the grid-barrier words [0..1], the error word [2] and the iteration
// count [3] (ints).
smg_status smg_coarse_cg_tc(smg_context* ctx, const void* links, int nx, int ny, const cx<float>* b, cx<float>* x,
                            void* r, float* rs, void* p0, float* ps0, void* p1, float* ps1, cx<float>* Ap,
                            double* part, int* state, int max_iter, double tol, long long spin_limit) {
    const int H = smg_coarse_cg_tc_rows(ctx, nx, ny);
    if (H == 0) return smg_fail(ctx, SMG_UNSUPPORTED, "persistent coarsest CG: CTAs cannot be co-resident");
    CcgTcArgs a;
    a.links = static_cast<const uint8_t*>(links);
    a.b = reinterpret_cast<const float2*>(b);
    a.x = reinterpret_cast<float2*>(x);
    a.r = static_cast<__half2*>(r);
    a.rs = rs;
    a.p[0] = static_cast<__half2*>(p0);
    a.p[1] = static_cast<__half2*>(p1);
    a.ps[0] = ps0;
    a.ps[1] = ps1;
    a.Ap = reinterpret_cast<float2*>(Ap);
    a.part = part;
    a.bar = reinterpret_cast<unsigned int*>(state);
    a.err = state + 2;
    a.iters = state + 3;
    a.spin_limit = spin_limit;
    a.tol2 = tol * tol;
    a.nx = nx;
    a.ny = ny;
    a.H = H;
    a.max_iter = max_iter;
    SMG_CUDA(ctx, cudaMemsetAsync(state, 0, 2 * sizeof(int), ctx->stream));  // barrier words; errors stay raised
    void* args[] = {&a};
    SMG_CUDA(ctx, cudaLaunchCooperativeKernel((const void*)k_ccg_tc, dim3(nx / kW, ny / H), dim3(kThreads), args,
                                              kCcgSmemBytes, ctx->stream));
    count_launch(ctx);
    SMG_CHECK_LAUNCH(ctx);
    return SMG_OK;
}

// The MR step of an intermediate level on FP16 vectors with one scale per site and rhs half
// ([site][dof][rhs] __half2, scales [site][2]): y = A x in FP16 (same format), <y, x>, ||y||^2 per rhs
// into out[rhs * 3 + k] and omega[rhs] = <y, x> / ||y||^2
smg_status smg_coarse_tc_apply_mr16(smg_context* ctx, const void* links, int nx, int ny, int nrhs, const void* xh,
                                    const float* xs, void* yh, float* ys, double* out, float* omega, int* err) {
    if (!smg_coarse_tc_shape_ok(nx, ny, kNc) || nrhs != kRhsTile || !xh || !xs || !yh || !ys || !out || !omega)
        return smg_fail(ctx, SMG_UNSUPPORTED, "tensor-core MR apply on FP16 vectors: shape not supported");
    const int H = rows_per_cta(nx, ny, 1);
    const dim3 grid(nx / kW, ny / H, 1);
    TcArgs a;
    a.links = static_cast<const uint8_t*>(links);
    a.xh = static_cast<const __half2*>(xh);
    a.xs = xs;
    a.wh = static_cast<const __half*>(xh);
    a.ws = xs;
    a.yh = static_cast<__half*>(yh);
    a.ys = ys;
    a.ssite = 2;
    a.shalf = 1;
    a.omega = reinterpret_cast<float2*>(omega);
    a.err = err;
    a.nx = nx;
    a.ny = ny;
    a.nrhs = nrhs;
    a.H = H;
    SMG_TRY(smg_reduce_reserve(ctx, (size_t)grid.x * grid.y * nrhs * 3));
    a.partials = ctx->red.partials;
    a.tickets = ctx->red.tickets;
    a.out = out;
    k_coarse_apply_tc<2, true, true><<<grid, kThreads, kSmemBytes, ctx->stream>>>(a);
    count_launch(ctx);
    SMG_CHECK_LAUNCH(ctx);
    return SMG_OK;
}

// Times every rows-per-CTA choice H (the divisors ny, ny / 2, ... of the lattice height) for this
// lattice and right-hand-side count and keeps the fastest for later applies; x and y are scratch
// vectors of the shape.  Skipped inside stream capture and when the shape is already tuned.
smg_status smg_coarse_tc_tune(smg_context* ctx, const void* links, int nx, int ny, int nrhs, const cx<float>* x,
                              cx<float>* y) {
    if (!smg_coarse_tc_shape_ok(nx, ny, kNc) || nrhs % kRhsTile != 0 || nrhs / kRhsTile > kMaxTickets)
        return SMG_OK;
    const int nz = nrhs / kRhsTile;
    const auto key = std::make_tuple(nx, ny, nz);
    {
        std::lock_guard<std::mutex> lock(g_rows_mu);
        if (g_rows.count(key)) return SMG_OK;
    }
    // SMG_TC_ROWS=<H> fixes the rows per CTA for every shape it divides (for measurements, e.g. under a
    // profiler whose replay distorts the timing)
    if (const char* e = std::getenv("SMG_TC_ROWS")) {
        const int H = std::atoi(e);
        if (H > 0 && ny % H == 0) {
            SMG_TRY(smg_reduce_reserve(ctx, (size_t)(nx / kW) * (ny / H) * nrhs * 3));
            std::lock_guard<std::mutex> lock(g_rows_mu);
            g_rows[key] = H;
            return SMG_OK;
        }
    }
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    SMG_CUDA(ctx, cudaStreamIsCapturing(ctx->stream, &cs));
    if (cs != cudaStreamCaptureStatusNone) return SMG_OK;
    std::vector<int> cand;
    for (int H = ny;; H /= 2) {
        cand.push_back(H);
        if (H % 2) break;
    }
    cudaEvent_t e0, e1;
    SMG_CUDA(ctx, cudaEventCreate(&e0));
    SMG_CUDA(ctx, cudaEventCreate(&e1));
    int best = rows_per_cta_rule(nx, ny, nz);
    float best_ms = 1e30f;
    smg_status st = SMG_OK;
    for (int H : cand) {
        st = launch_tc(ctx, links, nx, ny, nrhs, H, x, y, 0, nullptr, nullptr, nullptr, nullptr);  // warm-up
        if (st != SMG_OK) break;
        cudaEventRecord(e0, ctx->stream);
        for (int rep = 0; rep < 3 && st == SMG_OK; ++rep)
            st = launch_tc(ctx, links, nx, ny, nrhs, H, x, y, 0, nullptr, nullptr, nullptr, nullptr);
        cudaEventRecord(e1, ctx->stream);
        if (st != SMG_OK || cudaEventSynchronize(e1) != cudaSuccess) break;
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        if (ms < best_ms) {
            best_ms = ms;
            best = H;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    SMG_TRY(st);
    SMG_CHECK_LAUNCH(ctx);
    // reduction scratch for the fused-epilogue applies of this shape, reserved outside any capture
    SMG_TRY(smg_reduce_reserve(ctx, (size_t)(nx / kW) * (ny / best) * nrhs * 3));
    std::lock_guard<std::mutex> lock(g_rows_mu);
    g_rows[key] = best;
    return SMG_OK;
}

namespace {

smg_status launch_tc(smg_context* ctx, const void* links, int nx, int ny, int nrhs, int H, const cx<float>* x,
                     cx<float>* y, int epi, const cx<float>* w, double* out, const int* gate, int* err,
                     const TcArgs* half_in) {
    const int nz = nrhs / kRhsTile;
    const dim3 grid(nx / kW, ny / H, nz);
    TcArgs a;
    if (half_in) {  // FP16 x and w with per-site scales (EPI 2 only)
        a.xh = half_in->xh;
        a.xs = half_in->xs;
        a.wh = half_in->wh;
        a.ws = half_in->ws;
    }
    a.links = static_cast<const uint8_t*>(links);
    a.x = reinterpret_cast<const float2*>(x);
    a.y = reinterpret_cast<float2*>(y);
    a.w = reinterpret_cast<const float2*>(w);
    a.gate = gate;
    a.err = err;
    a.nx = nx;
    a.ny = ny;
    a.nrhs = nrhs;
    a.H = H;
    if (epi != 0) {
        SMG_TRY(smg_reduce_reserve(ctx, (size_t)grid.x * grid.y * nrhs * 3));
        a.partials = ctx->red.partials;
        a.tickets = ctx->red.tickets;
        a.out = out;
    }
    if (half_in)
        k_coarse_apply_tc<2, true><<<grid, kThreads, kSmemBytes, ctx->stream>>>(a);
    else if (epi == 0)
        k_coarse_apply_tc<0><<<grid, kThreads, kSmemBytes, ctx->stream>>>(a);
    else if (epi == 1)
        k_coarse_apply_tc<1><<<grid, kThreads, kSmemBytes, ctx->stream>>>(a);
    else
        k_coarse_apply_tc<2><<<grid, kThreads, kSmemBytes, ctx->stream>>>(a);
    count_launch(ctx);
    SMG_CHECK_LAUNCH(ctx);
    return SMG_OK;
}

}  // namespace
