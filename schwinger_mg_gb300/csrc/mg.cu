// Aggregation multigrid for A = D^dag D on the device
// (reference src/multigrid.cpp, src/prolongator.h, src/coarse_op.h).
//
// Level 0 is the fine lattice (dof = 2 spins, device fields).  Level l >= 1 is
// a coarse lattice of nx_l x ny_l sites with Nc_l dofs per site whose operator
// is a 9-point stencil of Nc_l x Nc_l blocks (SparseCoarseOp,
// src/coarse_op.h:154-297).  The transfer from level l to l+1 aggregates
// ax x ay sites; its block vectors are stored V[agg][loc][dof][i] with the
// coarse dof i innermost, so prolongation reads one contiguous row per fine
// dof and restriction reads coalesced across i.
//
// Setup follows build_mg_hierarchy (src/multigrid.cpp:595-687): inverse
// iteration for the near-null vectors (:435-484, :545-587), block
// Gram-Schmidt (src/prolongator.h:111-130), then the Galerkin operator.  The
// level-0 Galerkin operator is formed directly: with W_{B,i} = D P_{B,i}
// (supported on block B plus a one-site halo),
//   A_c[B][d](i, j) = <P_{B,i}, D^dag D P_{B+d,j}> = sum_x conj(W_{B,i}(x)) W_{B+d,j}(x),
// which replaces the reference's probing with one fine D^dag D application
// per coarse dof (src/coarse_op.h:241-279).  Deeper Galerkin operators are
// triple products of the stencil blocks with the block vectors.
#include "smg_internal.h"
#include "vec.cuh"
#include "half.cuh"
#include "mg_internal.h"

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <random>
#include <type_traits>
#include <vector>

smg_status smg_dslash(smg_dirac* d, bool dag, const smg_field* src, smg_field* dst, double* norm2_dev);
smg_status smg_dslash_mr(smg_dirac* d, bool dag, const smg_field* src, smg_field* dst, const smg_field* w,
                         double* out3_dev);
smg_status smg_dslash_h_norm(smg_dirac* d, bool dag, const smg_field* src, smg_field* dst, float* part,
                             int part_col);
smg_status smg_mr_norms_finish(smg_context* ctx, int L, int nrhs, const float* part, double* out3_dev,
                               float* omega_dev);
int smg_dslash_h_blocks(int L, int nrhs);
size_t smg_dslash_h_dots_scratch(int L, int nrhs);
// tensor-core coarse apply (coarse_tc.cu)
bool smg_coarse_tc_shape_ok(int nx, int ny, int ndof);
size_t smg_coarse_tc_link_bytes(int64_t nsites);
smg_status smg_coarse_tc_tile_links(smg_context* ctx, const cx<double>* A64, int nx, int64_t nsites, void* out);
smg_status smg_coarse_tc_apply_h(smg_context* ctx, const void* links, int nx, int ny, int nrhs, const void* xh,
                                 const float* xs, cx<float>* y, const void* wh, const float* ws, double* out,
                                 const int* gate, int* err);
smg_status smg_coarse_tc_apply(smg_context* ctx, const void* links, int nx, int ny, int nrhs, const cx<float>* x,
                               cx<float>* y, int epi, const cx<float>* w, double* out, const int* gate, int* err);
smg_status smg_coarse_tc_tune(smg_context* ctx, const void* links, int nx, int ny, int nrhs, const cx<float>* x,
                              cx<float>* y);
int smg_coarse_cg_tc_rows(smg_context* ctx, int nx, int ny);
smg_status smg_coarse_tc_apply_mr16(smg_context* ctx, const void* links, int nx, int ny, int nrhs, const void* xh,
                                    const float* xs, void* yh, float* ys, double* out, float* omega, int* err);
smg_status smg_coarse_cg_tc(smg_context* ctx, const void* links, int nx, int ny, const cx<float>* b, cx<float>* x,
                            void* r, float* rs, void* p0, float* ps0, void* p1, float* ps1, cx<float>* Ap,
                            double* part, int* state, int max_iter, double tol, long long spin_limit);

namespace {

__constant__ int c_dx[9] = {0, 1, -1, 0, 0, 1, 1, -1, -1};
__constant__ int c_dy[9] = {0, 0, 0, 1, -1, 1, -1, 1, -1};

__host__ __device__ __forceinline__ int dir_of(int dx, int dy) {
    // inverse of (c_dx, c_dy): 0 self, 1 +x, 2 -x, 3 +y, 4 -y, 5 +x+y, 6 +x-y, 7 -x+y, 8 -x-y
    if (dy == 0) return dx == 0 ? 0 : (dx > 0 ? 1 : 2);
    if (dx == 0) return dy > 0 ? 3 : 4;
    if (dx > 0) return dy > 0 ? 5 : 6;
    return dy > 0 ? 7 : 8;
}

struct Level {
    int nx = 0, ny = 0, nsites = 0, ndof = 2;
    // transfer to level + 1
    int ax = 0, ay = 0, nvec = 0, nc_next = 0, nagg_x = 0, nagg_y = 0;
    cx<double>* V64 = nullptr;  // [agg][loc][dof][i]
    cx<float>* V32 = nullptr;
    // level 0 with the packed transfers: V in FP32 as pairs over the two spins of a site,
    // [agg][loc][i] = (Re V[loc][0][i], Re V[loc][1][i], Im V[loc][0][i], Im V[loc][1][i])
    float4* V32s = nullptr;
    // intermediate FP16 levels with the packed transfers: V as output pairs,
    // [agg][loc][dof][i/2] = (Re V[..][i], Re V[..][i+1], Im V[..][i], Im V[..][i+1]); V32s then pairs
    // adjacent dofs (2d, 2d+1) of a site instead of the two spins
    float4* V32o = nullptr;
    // operator of this level (l >= 1): [site][dir][j][i] = block(i, j)
    cx<double>* A64 = nullptr;
    cx<float>* A32 = nullptr;
    void* Atc = nullptr;  // BF16 links pre-tiled for the tensor-core apply (F32 hierarchies)
    double rich_omega = 0;  // > 0: Richardson smoothing with this omega (MGLevel::richardson_omega)
    int64_t vsize() const { return (int64_t)nagg_x * nagg_y * ax * ay * ndof * nc_next; }
    int64_t asize() const { return (int64_t)nsites * 9 * ndof * ndof; }
};

// ------------------------------------------------------------ level-0 kernels

// the level-0 shape the packed transfers serve: 4 x 4 aggregates and 8, 16 or 32 coarse dofs
inline bool packed_shape0(const Level& L) {
    return L.ax == 4 && L.ay == 4 && (L.nc_next == 8 || L.nc_next == 16 || L.nc_next == 32);
}

// the intermediate-level shape the packed FP16 transfers serve: 2 x 2 aggregates of 16-dof sites
// and 8, 16 or 32 coarse dofs
inline bool packed_shape_c16(const Level& L) {
    return L.ndof == 16 && L.ax == 2 && L.ay == 2 && (L.nc_next == 8 || L.nc_next == 16 || L.nc_next == 32);
}

// out[k] = (Re V[2k'][i], Re V[2k'+1][i], Im V[2k'][i], Im V[2k'+1][i]) in FP32 with k = k' nc + i:
// pairs of adjacent nc-entry rows of V64 [agg][loc][dof][i] (the two spins of a level-0 site, dofs
// (2d, 2d+1) of a coarse site), or of adjacent entries (nc = 1: output pairs); np = entries / 2
__global__ void k_pair_spins(const cx<double>* __restrict__ V, float4* __restrict__ out, int64_t np, int nc) {
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= np) return;
    const int64_t sl = k / nc;
    const int i = (int)(k - sl * nc);
    const cx<double> a = V[(2 * sl) * nc + i], b = V[(2 * sl + 1) * nc + i];
    out[k] = make_float4((float)a.re, (float)b.re, (float)a.im, (float)b.im);
}

// V[B][loc][sp][i] from null vector k: i = c * nvec + k with chirality c = sp
// (split) or i = k (no split)
__global__ void k_extract0(const cx<double>* __restrict__ nv, int k, Geom g, int bx, int by, int nvec, int nc,
                           int split, cx<double>* __restrict__ V) {
    int s = blockIdx.x * blockDim.x + threadIdx.x;  // lexicographic fine site
    if (s >= g.V) return;
    int x = s % g.L, y = s / g.L;
    int q = site_q(g, x, y);
    int nbx = g.L / bx;
    int B = (x / bx) + nbx * (y / by);
    int loc = (x % bx) + bx * (y % by);
    int m = bx * by;
    for (int sp = 0; sp < 2; ++sp) {
        cx<double> v = nv[sidx(q, 0, sp, 1)];
        if (split) {
            for (int c = 0; c < 2; ++c) {
                int i = c * nvec + k;
                V[(((int64_t)B * m + loc) * 2 + sp) * nc + i] = (c == sp) ? v : mk(0.0, 0.0);
            }
        } else {
            V[(((int64_t)B * m + loc) * 2 + sp) * nc + k] = v;
        }
    }
}

// coarse level: V[B][loc][j][i] from a coarse null vector (dof = ndof, lexicographic sites)
__global__ void k_extract_c(const cx<double>* __restrict__ nv, int k, int nx, int ny, int ndof, int ax, int ay,
                            int nvec, int nc, int split, cx<double>* __restrict__ V) {
    int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (int64_t)nx * ny * ndof) return;
    int s = (int)(t / ndof), j = (int)(t - (int64_t)s * ndof);
    int x = s % nx, y = s / nx;
    int B = (x / ax) + (nx / ax) * (y / ay);
    int loc = (x % ax) + ax * (y % ay);
    int m = ax * ay;
    cx<double> v = nv[(int64_t)s * ndof + j];
    if (split) {
        int chi = j < ndof / 2 ? 0 : 1;  // coarse dofs are chirality-major
        for (int c = 0; c < 2; ++c)
            V[(((int64_t)B * m + loc) * ndof + j) * nc + c * nvec + k] = (c == chi) ? v : mk(0.0, 0.0);
    } else {
        V[(((int64_t)B * m + loc) * ndof + j) * nc + k] = v;
    }
}

// Modified Gram-Schmidt of the nc block vectors of one aggregate
// (orthonormalise_block, src/prolongator.h:111-130): vectors of length
// len = (aggregate sites) * dof, element e at V[(B * len + e) * nc + i].
__global__ void k_block_orth(cx<double>* __restrict__ V, int len, int nc) {
    extern __shared__ cx<double> sv[];  // [len][nc]
    __shared__ double red[2][32];
    const int B = blockIdx.x;
    cx<double>* Vb = V + (int64_t)B * len * nc;
    for (int t = threadIdx.x; t < len * nc; t += blockDim.x) sv[t] = Vb[t];
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int i = 0; i < nc; ++i) {
        for (int j = 0; j < i; ++j) {
            double pr = 0, pi = 0;
            for (int e = threadIdx.x; e < len; e += blockDim.x) {
                cx<double> c = cmulc(sv[e * nc + j], sv[e * nc + i]);
                pr += c.re;
                pi += c.im;
            }
            for (int o = 16; o; o >>= 1) {
                pr += __shfl_xor_sync(0xffffffffu, pr, o);
                pi += __shfl_xor_sync(0xffffffffu, pi, o);
            }
            if (lane == 0) {
                red[0][warp] = pr;
                red[1][warp] = pi;
            }
            __syncthreads();
            double tr = 0, ti = 0;
            for (int w = 0; w < nw; ++w) {
                tr += red[0][w];
                ti += red[1][w];
            }
            const cx<double> proj = mk(tr, ti);
            for (int e = threadIdx.x; e < len; e += blockDim.x) sv[e * nc + i] = sv[e * nc + i] - proj * sv[e * nc + j];
            __syncthreads();
        }
        double nn = 0;
        for (int e = threadIdx.x; e < len; e += blockDim.x) nn += norm2(sv[e * nc + i]);
        for (int o = 16; o; o >>= 1) nn += __shfl_xor_sync(0xffffffffu, nn, o);
        if (lane == 0) red[0][warp] = nn;
        __syncthreads();
        double tot = 0;
        for (int w = 0; w < nw; ++w) tot += red[0][w];
        tot = sqrt(tot);
        if (tot > 1e-14)
            for (int e = threadIdx.x; e < len; e += blockDim.x) sv[e * nc + i] = (1.0 / tot) * sv[e * nc + i];
        __syncthreads();
    }
    for (int t = threadIdx.x; t < len * nc; t += blockDim.x) Vb[t] = sv[t];
}

// Coarse vectors are [site][dof][rhs] (right-hand side innermost); the
// transfer kernels run one thread per output element with the rhs fastest, so
// coarse reads and writes are coalesced and block-vector reads are shared by
// the rhs lanes of a warp.

// restriction, level 0: c[B][i][rhs] = sum_{loc,sp} conj(V[B][loc][sp][i]) f[q][rhs][sp]
template <typename T>
__global__ void k_restrict0(const cx<T>* __restrict__ V, const cx<T>* __restrict__ f, cx<T>* __restrict__ c, Geom g,
                            int bx, int by, int nc, int nrhs) {
    int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    int nbx = g.L / bx, nby = g.L / by;
    int64_t total = (int64_t)nbx * nby * nrhs * nc;
    if (t >= total) return;
    int rhs = (int)(t % nrhs);
    int64_t bi = t / nrhs;
    int i = (int)(bi % nc);
    int B = (int)(bi / nc);
    int x0 = (B % nbx) * bx, y0 = (B / nbx) * by;
    int m = bx * by;
    cx<T> acc = mk<T>(0, 0);
    for (int loc = 0; loc < m; ++loc) {
        int x = x0 + loc % bx, y = y0 + loc / bx;
        int q = site_q(g, x, y);
        Spinor<T> fv = ld_spinor(f, q, rhs, nrhs);
        const cx<T>* v = V + ((int64_t)B * m + loc) * 2 * nc;
        acc = acc + cmulc(v[i], fv.s0) + cmulc(v[nc + i], fv.s1);
    }
    c[t] = acc;  // t = (B * nc + i) * nrhs + rhs
}

// prolongation, level 0: f[q][rhs][sp] (+)= sum_i V[B][loc][sp][i] c[B][i][rhs]
template <typename T>
__global__ void k_prolong0(const cx<T>* __restrict__ V, const cx<T>* __restrict__ c, cx<T>* __restrict__ f, Geom g,
                           int bx, int by, int nc, int nrhs, int accumulate) {
    int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (int64_t)g.V * nrhs) return;
    int rhs = (int)(t % nrhs);
    int q = (int)(t / nrhs);
    int x, y, p;
    site_coords(g, q, x, y, p);
    int nbx = g.L / bx;
    int B = (x / bx) + nbx * (y / by);
    int loc = (x % bx) + bx * (y % by);
    int m = bx * by;
    const cx<T>* v = V + ((int64_t)B * m + loc) * 2 * nc;
    const cx<T>* cc = c + (int64_t)B * nc * nrhs + rhs;
    cx<T> f0 = mk<T>(0, 0), f1 = mk<T>(0, 0);
    for (int i = 0; i < nc; ++i) {
        cx<T> ci = cc[(int64_t)i * nrhs];
        f0 = f0 + ci * v[i];
        f1 = f1 + ci * v[nc + i];
    }
    Spinor<T> out;
    if (accumulate) {
        out = ld_spinor(f, q, rhs, nrhs);
        out.s0 = out.s0 + f0;
        out.s1 = out.s1 + f1;
    } else {
        out.s0 = f0;
        out.s1 = f1;
    }
    st_spinor(f, q, rhs, nrhs, out);
}

// coarse restriction: c'[B][i][rhs] = sum_{loc,j} conj(V[B][loc][j][i]) c[site][j][rhs]
template <typename T>
__global__ void k_restrict_c(const cx<T>* __restrict__ V, const cx<T>* __restrict__ c, cx<T>* __restrict__ cn, int nx,
                             int ax, int ay, int ndof, int nc, int nagg, int nrhs) {
    int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (int64_t)nagg * nrhs * nc) return;
    int rhs = (int)(t % nrhs);
    int64_t bi = t / nrhs;
    int i = (int)(bi % nc);
    int B = (int)(bi / nc);
    int nax = nx / ax;
    int x0 = (B % nax) * ax, y0 = (B / nax) * ay;
    int m = ax * ay;
    cx<T> acc = mk<T>(0, 0);
    for (int loc = 0; loc < m; ++loc) {
        int s = (x0 + loc % ax) + nx * (y0 + loc / ax);
        const cx<T>* cv = c + (int64_t)s * ndof * nrhs + rhs;
        const cx<T>* v = V + ((int64_t)B * m + loc) * ndof * nc;
        for (int j = 0; j < ndof; ++j) acc = acc + cmulc(v[j * nc + i], cv[(int64_t)j * nrhs]);
    }
    cn[t] = acc;  // t = (B * nc + i) * nrhs + rhs
}

// coarse prolongation: c[site][j][rhs] (+)= sum_i V[B][loc][j][i] c'[B][i][rhs]
template <typename T>
__global__ void k_prolong_c(const cx<T>* __restrict__ V, const cx<T>* __restrict__ cn, cx<T>* __restrict__ c, int nx,
                            int ny, int ax, int ay, int ndof, int nc, int nrhs, int accumulate) {
    int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (int64_t)nx * ny * nrhs * ndof) return;
    int rhs = (int)(t % nrhs);
    int64_t sj = t / nrhs;
    int j = (int)(sj % ndof);
    int s = (int)(sj / ndof);
    int x = s % nx, y = s / nx;
    int B = (x / ax) + (nx / ax) * (y / ay);
    int loc = (x % ax) + ax * (y % ay);
    int m = ax * ay;
    const cx<T>* v = V + (((int64_t)B * m + loc) * ndof + j) * nc;
    const cx<T>* cc = cn + (int64_t)B * nc * nrhs + rhs;
    cx<T> acc = mk<T>(0, 0);
    for (int i = 0; i < nc; ++i) acc = acc + v[i] * cc[(int64_t)i * nrhs];
    c[t] = accumulate ? c[t] + acc : acc;  // t = (s * ndof + j) * nrhs + rhs
}

// Aggregate-blocked transfers: one block per (aggregate, chunk of up to 32
// right-hand sides), threads (rhs lane, row).  Restriction reads every input
// value of the aggregate once and keeps the NC outputs of its rhs in
// registers (rows reduced through shared memory); prolongation keeps the NC
// coarse values of its rhs in registers and writes each output once.  Level 0
// inputs/outputs are fine spinors (dof = spin), coarse levels [site][dof][rhs].
struct TransferGeom {
    Geom g;            // level 0 only
    int nx = 0;        // coarse input/output lattice width (level >= 1)
    int ax = 0, ay = 0, nax = 0;
    int ndof = 2, nrhs = 1;
    int level0 = 0;
};

__device__ __forceinline__ int64_t transfer_site(const TransferGeom& t, int B, int loc) {
    const int x = (B % t.nax) * t.ax + loc % t.ax, y = (B / t.nax) * t.ay + loc / t.ax;
    return t.level0 ? (int64_t)site_q(t.g, x, y) : (int64_t)x + (int64_t)t.nx * y;
}
// element (site s, dof j, rhs) of a level-0 spinor field [q][rhs][spin] or a coarse vector [site][dof][rhs]
__device__ __forceinline__ int64_t transfer_idx(const TransferGeom& t, int64_t s, int j, int rhs) {
    return t.level0 ? (s * t.nrhs + rhs) * 2 + j : (s * t.ndof + j) * t.nrhs + rhs;
}

// fine/coarse vector readers for the restriction: plain, or FP16 with per-site scales
// (spinor() reads both spin components of a level-0 site and right-hand side in one access)
template <typename T>
struct InPlain {
    const cx<T>* __restrict__ p;
    __device__ __forceinline__ cx<T> operator()(int64_t idx, int64_t) const { return p[idx]; }
    __device__ __forceinline__ Spinor<T> spinor(int64_t q, int rhs, int nrhs) const { return ld_spinor(p, q, rhs, nrhs); }
};
struct InHalf {
    const __half2* __restrict__ p;
    const float* __restrict__ scale;
    __device__ __forceinline__ cx<float> operator()(int64_t idx, int64_t site) const {
        const float2 v = __half22float2(p[idx]);
        const float s = scale[site];
        return mk(v.x * s, v.y * s);
    }
    __device__ __forceinline__ Spinor<float> spinor(int64_t q, int rhs, int nrhs) const {
        return ld_spinor_h(p, scale, q, rhs, nrhs);
    }
};

// coarse vectors in FP16 with one scale per site and half of the 32 rhs ([site][dof][32] __half2,
// scales [site][2]): the intermediate-level MR smoother's residuals
struct InHalfC {
    const __half2* __restrict__ p;
    const float* __restrict__ scale;
    __device__ __forceinline__ cx<float> operator()(int64_t idx, int64_t site) const {
        const float2 v = __half22float2(p[idx]);
        const float s = scale[2 * site + ((idx & 31) >> 4)];
        return mk(v.x * s, v.y * s);
    }
    __device__ __forceinline__ Spinor<float> spinor(int64_t, int, int) const { return Spinor<float>{}; }
};

// One block per (aggregate, tile of `lanes` right-hand sides) stages the aggregate's ne = ax ay
// ndof input values of its right-hand sides and its block vectors in shared memory (every global
// load issued before any arithmetic), then each thread (rhs lane, row) forms whole outputs from
// shared memory: no cross-thread reduction, one barrier.
template <typename T, int NC, typename In = InPlain<T>>
__global__ void __launch_bounds__(256) k_restrict_agg(const cx<T>* __restrict__ V, In in,
                                                      cx<T>* __restrict__ out, TransferGeom t) {
    extern __shared__ unsigned char s_raw[];
    const int lanes = blockDim.x, rows = blockDim.y;
    const int B = blockIdx.x, m = t.ax * t.ay, nd = t.ndof, nrhs = t.nrhs, ne = m * nd;
    cx<T>* s_f = reinterpret_cast<cx<T>*>(s_raw);  // [ne][lanes]
    cx<T>* s_v = s_f + (int64_t)ne * lanes;        // [ne][NC]
    const int rhs = blockIdx.y * lanes + threadIdx.x;
    const bool live = rhs < nrhs;
    if (t.level0) {  // both spins of a site in one access
#pragma unroll 2
        for (int loc = threadIdx.y; loc < m; loc += rows) {
            Spinor<T> f;
            f.s0 = f.s1 = mk<T>(0, 0);
            if (live) f = in.spinor(transfer_site(t, B, loc), rhs, nrhs);
            s_f[(2 * loc) * lanes + threadIdx.x] = f.s0;
            s_f[(2 * loc + 1) * lanes + threadIdx.x] = f.s1;
        }
    } else {
#pragma unroll 4
        for (int e = threadIdx.y; e < ne; e += rows) {
            const int loc = e / nd, j = e - loc * nd;
            const int64_t s = transfer_site(t, B, loc);
            s_f[e * lanes + threadIdx.x] = live ? in(transfer_idx(t, s, j, rhs), s) : mk<T>(0, 0);
        }
    }
    const cx<T>* __restrict__ Vb = V + (int64_t)B * ne * NC;
    for (int k = threadIdx.y * lanes + threadIdx.x; k < ne * NC; k += lanes * rows) s_v[k] = Vb[k];
    __syncthreads();
    if (!live) return;
    if (NC == 2 * rows) {
        // two adjacent outputs per thread: one shared-memory read of the input per entry serves both,
        // and the two block-vector values are one 2 x 8-byte read
        const int i0 = 2 * threadIdx.y;
        cx<T> a0 = mk<T>(0, 0), a1 = mk<T>(0, 0);
#pragma unroll 8
        for (int e = 0; e < ne; ++e) {
            const cx<T> f = s_f[e * lanes + threadIdx.x];
            cx<T> v0, v1;
            if constexpr (std::is_same<T, float>::value) {  // s_v is 16-byte aligned, i0 even
                const float4 w = *reinterpret_cast<const float4*>(s_v + e * NC + i0);
                v0 = mk(w.x, w.y);
                v1 = mk(w.z, w.w);
            } else {
                v0 = s_v[e * NC + i0];
                v1 = s_v[e * NC + i0 + 1];
            }
            a0 = a0 + cmulc(v0, f);
            a1 = a1 + cmulc(v1, f);
        }
        out[((int64_t)B * NC + i0) * nrhs + rhs] = a0;
        out[((int64_t)B * NC + i0 + 1) * nrhs + rhs] = a1;
        return;
    }
    for (int i = threadIdx.y; i < NC; i += rows) {
        cx<T> acc = mk<T>(0, 0);
#pragma unroll 8
        for (int e = 0; e < ne; ++e) acc = acc + cmulc(s_v[e * NC + i], s_f[e * lanes + threadIdx.x]);
        out[((int64_t)B * NC + i) * nrhs + rhs] = acc;
    }
}

template <typename T, int NC>
__global__ void __launch_bounds__(256) k_prolong_agg(const cx<T>* __restrict__ V, const cx<T>* __restrict__ cin,
                                                     cx<T>* __restrict__ out, TransferGeom t, int accumulate) {
    extern __shared__ unsigned char s_raw[];
    const int lanes = blockDim.x, rows = blockDim.y;
    const int B = blockIdx.x, m = t.ax * t.ay, nd = t.ndof, nrhs = t.nrhs, ne = m * nd;
    cx<T>* s_c = reinterpret_cast<cx<T>*>(s_raw);  // [NC][lanes] (coarse levels)
    cx<T>* s_v = s_c + NC * lanes;                 // [ne][NC]
    const int rhs = blockIdx.y * lanes + threadIdx.x;
    const bool live = rhs < nrhs;
    const cx<T>* __restrict__ Vb = V + (int64_t)B * ne * NC;
    if (t.level0) {
        // the NC coarse values of this thread's rhs in registers, the block vectors in shared memory;
        // one fine site (both spins, one 2-spinor access) per step, two sites' previous values
        // requested before any arithmetic
        cx<T> c[NC];
#pragma unroll
        for (int i = 0; i < NC; ++i) c[i] = live ? cin[((int64_t)B * NC + i) * nrhs + rhs] : mk<T>(0, 0);
        for (int k = threadIdx.y * lanes + threadIdx.x; k < ne * NC; k += lanes * rows) s_v[k] = Vb[k];
        __syncthreads();
        if (!live) return;
        for (int l0 = threadIdx.y; l0 < m; l0 += 2 * rows) {
            const int l1 = l0 + rows;
            const int64_t q0 = transfer_site(t, B, l0), q1 = l1 < m ? transfer_site(t, B, l1) : 0;
            Spinor<T> p0, p1;
            p0.s0 = p0.s1 = p1.s0 = p1.s1 = mk<T>(0, 0);
            if (accumulate) {
                p0 = ld_spinor(out, q0, rhs, nrhs);
                if (l1 < m) p1 = ld_spinor(out, q1, rhs, nrhs);
            }
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int loc = h ? l1 : l0;
                if (loc >= m) break;
                cx<T> a0 = mk<T>(0, 0), a1 = mk<T>(0, 0);
#pragma unroll
                for (int i = 0; i < NC; ++i) {
                    a0 = a0 + s_v[(2 * loc) * NC + i] * c[i];
                    a1 = a1 + s_v[(2 * loc + 1) * NC + i] * c[i];
                }
                const Spinor<T>& pv = h ? p1 : p0;
                Spinor<T> o;
                o.s0 = accumulate ? pv.s0 + a0 : a0;
                o.s1 = accumulate ? pv.s1 + a1 : a1;
                st_spinor(out, h ? q1 : q0, rhs, nrhs, o);
            }
        }
        return;
    }
    for (int i = threadIdx.y; i < NC; i += rows)
        s_c[i * lanes + threadIdx.x] = live ? cin[((int64_t)B * NC + i) * nrhs + rhs] : mk<T>(0, 0);
    for (int k = threadIdx.y * lanes + threadIdx.x; k < ne * NC; k += lanes * rows) s_v[k] = Vb[k];
    __syncthreads();
    if (!live) return;
#pragma unroll 2
    for (int e = threadIdx.y; e < ne; e += rows) {
        const int loc = e / nd, j = e - loc * nd;
        const int64_t o = transfer_idx(t, transfer_site(t, B, loc), j, rhs);
        const cx<T> prev = accumulate ? out[o] : mk<T>(0, 0);
        cx<T> acc = mk<T>(0, 0);
#pragma unroll
        for (int i = 0; i < NC; ++i) acc = acc + s_v[e * NC + i] * s_c[i * lanes + threadIdx.x];
        out[o] = accumulate ? prev + acc : acc;
    }
}

// W[B][i][h][sp] = (D P_{B,i})(h) on the (bx+2) x (by+2) halo frame of block B
__global__ void k_W0(const cx<double>* __restrict__ V, const cx<double>* __restrict__ U, const double* __restrict__ C,
                     Geom g, int bx, int by, int nc, double diag, double mu, double r, cx<double>* __restrict__ W) {
    const int B = blockIdx.x;
    const int hx_n = bx + 2, hy_n = by + 2, nh = hx_n * hy_n;
    const int nbx = g.L / bx;
    const int x0 = (B % nbx) * bx, y0 = (B / nbx) * by;
    const int m = bx * by;
    for (int t = threadIdx.x; t < nh * nc; t += blockDim.x) {
        const int i = t % nc, h = t / nc;
        const int hx = h % hx_n, hy = h / hx_n;
        const int x = wrap(x0 - 1 + hx, g.L), y = wrap(y0 - 1 + hy, g.L);
        // P_{B,i} at block-frame coordinates (lx, ly); zero outside the block
        auto Pv = [&](int lx, int ly, int sp) -> cx<double> {
            if (lx < 0 || lx >= bx || ly < 0 || ly >= by) return mk(0.0, 0.0);
            return V[(((int64_t)B * m + lx + bx * ly) * 2 + sp) * nc + i];
        };
        const int lx = hx - 1, ly = hy - 1;
        const int q = site_q(g, x, y);
        const int q_xm = site_q(g, wrap(x - 1, g.L), y);
        const int q_ym = site_q(g, x, wrap(y - 1, g.L));
        const cx<double> u0f = U[q], u0b = U[q_xm], u1f = U[(int64_t)g.V + q], u1b = U[(int64_t)g.V + q_ym];
        const cx<double> a0x = u0f * Pv(lx + 1, ly, 0), a1x = u0f * Pv(lx + 1, ly, 1);
        const cx<double> b0x = cmulc(u0b, Pv(lx - 1, ly, 0)), b1x = cmulc(u0b, Pv(lx - 1, ly, 1));
        const cx<double> a0y = u1f * Pv(lx, ly + 1, 0), a1y = u1f * Pv(lx, ly + 1, 1);
        const cx<double> b0y = cmulc(u1b, Pv(lx, ly - 1, 0)), b1y = cmulc(u1b, Pv(lx, ly - 1, 1));
        const double Cq = C ? C[q] : 0.0;
        const cx<double> dg0 = mk(diag + Cq, mu), dg1 = mk(diag - Cq, -mu);
        const cx<double> sr0 = (a0x + b0x) + (a0y + b0y);
        const cx<double> sr1 = (a1x + b1x) + (a1y + b1y);
        const cx<double> off0 = (b1x - a1x) + times_i(a1y - b1y);
        const cx<double> off1 = (b0x - a0x) - times_i(a0y - b0y);
        const cx<double> w0 = dg0 * Pv(lx, ly, 0) - 0.5 * (r * sr0 + off0);
        const cx<double> w1 = dg1 * Pv(lx, ly, 1) - 0.5 * (r * sr1 + off1);
        cx<double>* o = W + (((int64_t)B * nc + i) * nh + h) * 2;
        o[0] = w0;
        o[1] = w1;
    }
}

// A[B][d][j][i] = sum_{x in halo(B) and halo(B+d)} conj(W_{B,i}(x)) W_{B+d,j}(x)
__global__ void k_galerkin0(const cx<double>* __restrict__ W, int nbx, int nby, int bx, int by, int nc,
                            cx<double>* __restrict__ A) {
    const int B = blockIdx.x, d = blockIdx.y;
    const int hx_n = bx + 2, hy_n = by + 2, nh = hx_n * hy_n;
    const int dx = c_dx[d], dy = c_dy[d];
    const int Bx = B % nbx, By = B / nbx;
    const int B2 = ((Bx + dx + nbx) % nbx) + nbx * ((By + dy + nby) % nby);
    const int hx_lo = dx > 0 ? bx : 0, hx_hi = dx < 0 ? 2 : hx_n;
    const int hy_lo = dy > 0 ? by : 0, hy_hi = dy < 0 ? 2 : hy_n;
    for (int t = threadIdx.x; t < nc * nc; t += blockDim.x) {
        const int i = t % nc, j = t / nc;
        const cx<double>* w1 = W + ((int64_t)B * nc + i) * nh * 2;
        const cx<double>* w2 = W + ((int64_t)B2 * nc + j) * nh * 2;
        cx<double> acc = mk(0.0, 0.0);
        for (int hy = hy_lo; hy < hy_hi; ++hy)
            for (int hx = hx_lo; hx < hx_hi; ++hx) {
                const int h1 = hx + hx_n * hy;
                const int h2 = (hx - dx * bx) + hx_n * (hy - dy * by);
                acc = acc + cmulc(w1[2 * h1], w2[2 * h2]) + cmulc(w1[2 * h1 + 1], w2[2 * h2 + 1]);
            }
        A[(((int64_t)B * 9 + d) * nc + j) * nc + i] = acc;
    }
}

// Galerkin of a coarse level: A'[B][d'](i', j') = sum_{loc, d} V_B(loc)^dag L[b][d] V_{B2}(loc2)
__global__ void k_galerkin_c(const cx<double>* __restrict__ Lk, const cx<double>* __restrict__ V, int nx, int ny, int ax,
                             int ay, int ndof, int nc, cx<double>* __restrict__ A) {
    extern __shared__ cx<double> sT[];  // [ndof][nc]
    const int B = blockIdx.x;
    const int nax = nx / ax, nay = ny / ay;
    const int Bx = B % nax, By = B / nax;
    const int m = ax * ay;
    // each thread owns (i', j') pairs; accumulators for 9 directions
    const int npair = nc * nc;
    constexpr int kMaxPairs = 4;  // pairs per thread (blockDim * 4 >= nc * nc)
    cx<double> acc[kMaxPairs][9];
    for (int a = 0; a < kMaxPairs; ++a)
        for (int d = 0; d < 9; ++d) acc[a][d] = mk(0.0, 0.0);
    for (int loc = 0; loc < m; ++loc) {
        const int x = Bx * ax + loc % ax, y = By * ay + loc / ax;
        const int s = x + nx * y;
        for (int d = 0; d < 9; ++d) {
            const int x2 = (x + c_dx[d] + nx) % nx, y2 = (y + c_dy[d] + ny) % ny;
            const int B2x = x2 / ax, B2y = y2 / ay;
            int ddx = B2x - Bx, ddy = B2y - By;
            if (ddx > 1) ddx -= nax;
            if (ddx < -1) ddx += nax;
            if (ddy > 1) ddy -= nay;
            if (ddy < -1) ddy += nay;
            const int dp = dir_of(ddx, ddy);
            const int B2 = B2x + nax * B2y;
            const int loc2 = (x2 % ax) + ax * (y2 % ay);
            // T(k, j') = sum_j L[s][d](k, j) V_{B2}[loc2][j][j']
            const cx<double>* Lsd = Lk + ((int64_t)s * 9 + d) * ndof * ndof;  // [j][k]
            const cx<double>* V2 = V + ((int64_t)B2 * m + loc2) * ndof * nc;  // [j][j']
            __syncthreads();
            for (int t = threadIdx.x; t < ndof * nc; t += blockDim.x) {
                const int k = t / nc, jp = t % nc;
                cx<double> sum = mk(0.0, 0.0);
                for (int j = 0; j < ndof; ++j) sum = sum + Lsd[j * ndof + k] * V2[j * nc + jp];
                sT[k * nc + jp] = sum;
            }
            __syncthreads();
            const cx<double>* V1 = V + ((int64_t)B * m + loc) * ndof * nc;  // [k][i']
            for (int a = 0; a < kMaxPairs; ++a) {
                const int t = threadIdx.x + a * blockDim.x;
                if (t >= npair) break;
                const int ip = t % nc, jp = t / nc;
                cx<double> sum = mk(0.0, 0.0);
                for (int k = 0; k < ndof; ++k) sum = sum + cmulc(V1[k * nc + ip], sT[k * nc + jp]);
                for (int dd = 0; dd < 9; ++dd)
                    if (dd == dp) acc[a][dd] = acc[a][dd] + sum;
            }
        }
    }
    for (int a = 0; a < kMaxPairs; ++a) {
        const int t = threadIdx.x + a * blockDim.x;
        if (t >= npair) break;
        const int ip = t % nc, jp = t / nc;
        for (int d = 0; d < 9; ++d) A[(((int64_t)B * 9 + d) * nc + jp) * nc + ip] = acc[a][d];
    }
}

// y[s][rhs][i] = sum_d sum_j A[s][d][j][i] x[nb(s,d)][rhs][j]; optional fused
// reductions <y, w> and ||y||^2 per rhs.  Threads: x = rhs lane, y = (site, i).
template <typename T, int EPI>
__global__ void __launch_bounds__(256) k_coarse_apply(const cx<T>* __restrict__ A, VecView<T> xin, cx<T>* __restrict__ y,
                                                      int nx, int ny, const cx<T>* __restrict__ w, double* partials,
                                                      unsigned int* ticket, double* out, const int* __restrict__ gate) {
    if (gate && *gate == 0) return;  // every right-hand side of the solve has converged
    constexpr int K = EPI == 2 ? 3 : 1;
    const int nc = xin.ndof, nrhs = xin.nrhs;
    const int rhs = blockIdx.y * blockDim.x + threadIdx.x;
    T v[K];  // per-thread partials in the field precision (FP64 is scarce on this part)
#pragma unroll
    for (int k = 0; k < K; ++k) v[k] = T(0);
    const int64_t nrow = (int64_t)xin.nsites * nc;
    if (rhs < nrhs) {
        for (int64_t row = (int64_t)blockIdx.x * blockDim.y + threadIdx.y; row < nrow;
             row += (int64_t)gridDim.x * blockDim.y) {
            const int s = (int)(row / nc), i = (int)(row - (int64_t)s * nc);
            const int x = s % nx, yy = s / nx;
            cx<T> acc = mk<T>(0, 0);
#pragma unroll 1
            for (int d = 0; d < 9; ++d) {
                const int xn = x + c_dx[d], yn = yy + c_dy[d];
                const int sn = (xn < 0 ? xn + nx : (xn >= nx ? xn - nx : xn)) +
                               nx * (yn < 0 ? yn + ny : (yn >= ny ? yn - ny : yn));
                const cx<T>* Ad = A + ((int64_t)s * 9 + d) * nc * nc + i;
                const cx<T>* xv = xin.p + (int64_t)sn * nc * nrhs + rhs;  // [site][dof][rhs]
                for (int j = 0; j < nc; ++j) acc = acc + Ad[(int64_t)j * nc] * xv[(int64_t)j * nrhs];
            }
            const int64_t o = ((int64_t)s * nc + i) * nrhs + rhs;
            y[o] = acc;
            if (EPI == 1) {
                v[0] += norm2(acc);
            } else if (EPI == 2) {
                const cx<T> c = cmulc(acc, w[o]);
                v[0] += c.re;
                v[1] += c.im;
                v[2] += norm2(acc);
            }
        }
    }
    if (EPI != 0) block_reduce_finalise<K>(v, partials, ticket, nrhs, FinStore{out, K});
}

// Single-RHS coarse apply: one thread per (site, i) row with the j loop
// unrolled, so each thread has all Nc link and vector loads of a direction in
// flight (the generic kernel's dependent j loop is latency-bound).
template <typename T, int EPI, int NC>
__global__ void __launch_bounds__(256) k_coarse_apply1(const cx<T>* __restrict__ A, VecView<T> xin,
                                                       cx<T>* __restrict__ y, int nx, int ny,
                                                       const cx<T>* __restrict__ w, double* partials,
                                                       unsigned int* ticket, double* out, const int* __restrict__ gate) {
    if (gate && *gate == 0) return;
    constexpr int K = EPI == 2 ? 3 : 1;
    T v[K];  // per-thread partials in the field precision (FP64 is scarce on this part)
#pragma unroll
    for (int k = 0; k < K; ++k) v[k] = T(0);
    const int64_t nrow = (int64_t)xin.nsites * NC;
    for (int64_t row = (int64_t)blockIdx.x * blockDim.y + threadIdx.y; row < nrow;
         row += (int64_t)gridDim.x * blockDim.y) {
        const int s = (int)(row / NC), i = (int)(row % NC);
        const int x = s % nx, yy = s / nx;
        cx<T> acc = mk<T>(0, 0);
#pragma unroll 3
        for (int d = 0; d < 9; ++d) {
            const int xn = x + c_dx[d], yn = yy + c_dy[d];
            const int sn = (xn < 0 ? xn + nx : (xn >= nx ? xn - nx : xn)) +
                           nx * (yn < 0 ? yn + ny : (yn >= ny ? yn - ny : yn));
            const cx<T>* Ad = A + ((int64_t)s * 9 + d) * NC * NC + i;
            const cx<T>* xv = xin.p + (int64_t)sn * NC;
#pragma unroll
            for (int j = 0; j < NC; ++j) acc = acc + Ad[j * NC] * xv[j];
        }
        y[row] = acc;
        if (EPI == 1) {
            v[0] += norm2(acc);
        } else if (EPI == 2) {
            const cx<T> c = cmulc(acc, w[row]);
            v[0] += c.re;
            v[1] += c.im;
            v[2] += norm2(acc);
        }
    }
    if (EPI != 0) block_reduce_finalise<K>(v, partials, ticket, 1, FinStore{out, K});
}

// Multi-RHS coarse apply, one coarse site per block iteration: for each of
// the 9 directions the Nc x Nc link block and the neighbour's Nc x R vector
// block (R right-hand sides of one lane chunk) are staged in shared memory,
// then thread (r, row) accumulates y(i, r) for i = row, row + rows, ...
// Rows of the staged vector block are padded by one complex so the RHS lanes
// of a warp hit distinct banks.  Epilogue reductions as k_coarse_apply.
template <typename T, int EPI, int NC>
__global__ void __launch_bounds__(256) k_coarse_apply_tiled(const cx<T>* __restrict__ A, VecView<T> xin,
                                                            cx<T>* __restrict__ y, int nx, int ny,
                                                            const cx<T>* __restrict__ w, double* partials,
                                                            unsigned int* ticket, double* out,
                                                            const int* __restrict__ gate) {
    if (gate && *gate == 0) return;  // every right-hand side of the solve has converged
    constexpr int K = EPI == 2 ? 3 : 1;
    constexpr int kPer = (NC + 7) / 8;  // outputs per thread; blockDim.y >= 8
    __shared__ cx<T> sA[NC * NC];       // [j][i]
    __shared__ cx<T> sX[32][NC + 1];    // [r][j]
    const int lanes = blockDim.x, rows = blockDim.y;
    const int nrhs = xin.nrhs;
    const int r0 = blockIdx.y * lanes;
    const int rhs = r0 + threadIdx.x;
    const int tid = threadIdx.y * lanes + threadIdx.x, nthr = lanes * rows;
    T v[K];  // per-thread partials in the field precision (FP64 is scarce on this part)
#pragma unroll
    for (int k = 0; k < K; ++k) v[k] = T(0);
    for (int s = blockIdx.x; s < xin.nsites; s += gridDim.x) {
        const int x = s % nx, yy = s / nx;
        cx<T> acc[kPer];
#pragma unroll
        for (int a = 0; a < kPer; ++a) acc[a] = mk<T>(0, 0);
        for (int d = 0; d < 9; ++d) {
            const int xn = x + c_dx[d], yn = yy + c_dy[d];
            const int sn = (xn < 0 ? xn + nx : (xn >= nx ? xn - nx : xn)) +
                           nx * (yn < 0 ? yn + ny : (yn >= ny ? yn - ny : yn));
            __syncthreads();
            const cx<T>* Ad = A + ((int64_t)s * 9 + d) * NC * NC;
            for (int t = tid; t < NC * NC; t += nthr) sA[t] = Ad[t];
            const cx<T>* Xn = xin.p + (int64_t)sn * NC * nrhs + r0;  // [site][dof][rhs]
            for (int t = tid; t < lanes * NC; t += nthr) {
                const int j = t / lanes, r = t - j * lanes;
                sX[r][j] = (r0 + r < nrhs) ? Xn[(int64_t)j * nrhs + r] : mk<T>(0, 0);
            }
            __syncthreads();
#pragma unroll
            for (int a = 0; a < kPer; ++a) {
                const int i = threadIdx.y + a * rows;
                if (i < NC) {
                    cx<T> sum = acc[a];
#pragma unroll
                    for (int j = 0; j < NC; ++j) sum = sum + sA[j * NC + i] * sX[threadIdx.x][j];
                    acc[a] = sum;
                }
            }
        }
        if (rhs < nrhs) {
#pragma unroll
            for (int a = 0; a < kPer; ++a) {
                const int i = threadIdx.y + a * rows;
                if (i < NC) {
                    const int64_t o = ((int64_t)s * NC + i) * nrhs + rhs;
                    y[o] = acc[a];
                    if (EPI == 1) {
                        v[0] += norm2(acc[a]);
                    } else if (EPI == 2) {
                        const cx<T> c = cmulc(acc[a], w[o]);
                        v[0] += c.re;
                        v[1] += c.im;
                        v[2] += norm2(acc[a]);
                    }
                }
            }
        }
    }
    if (EPI != 0) block_reduce_finalise<K>(v, partials, ticket, nrhs, FinStore{out, K});
}

// One thread per output entry y[s][i][rhs] (rhs fastest, so a warp's stores are contiguous): the
// 9 x NC link entries of column i are shared through L1 by the threads of the other right-hand
// sides, the neighbour vectors by the threads of the other output dofs.  No shared memory or
// barriers: every entry's 9 NC complex products run independently, which suits small NC and
// few right-hand sides, where the tiled kernel above leaves most threads idle between barriers.
template <typename T, int EPI, int NC>
__global__ void __launch_bounds__(256) k_coarse_apply_flat(const cx<T>* __restrict__ A, VecView<T> xin,
                                                           cx<T>* __restrict__ y, int nx, int ny,
                                                           const cx<T>* __restrict__ w, double* partials,
                                                           unsigned int* ticket, double* out,
                                                           const int* __restrict__ gate) {
    if (gate && *gate == 0) return;  // every right-hand side of the solve has converged
    constexpr int K = EPI == 2 ? 3 : 1;
    const int nrhs = xin.nrhs;
    const int rhs = blockIdx.y * blockDim.x + threadIdx.x;
    T v[K];
#pragma unroll
    for (int k = 0; k < K; ++k) v[k] = T(0);
    const int64_t items = (int64_t)xin.nsites * NC;
    if (rhs < nrhs)
        for (int64_t it = (int64_t)blockIdx.x * blockDim.y + threadIdx.y; it < items;
             it += (int64_t)gridDim.x * blockDim.y) {
            const int s = (int)(it / NC), i = (int)(it - (int64_t)s * NC);
            const int x = s % nx, yy = s / nx;
            cx<T> acc = mk<T>(0, 0);
#pragma unroll
            for (int d = 0; d < 9; ++d) {
                const int xn = x + c_dx[d], yn = yy + c_dy[d];
                const int sn = (xn < 0 ? xn + nx : (xn >= nx ? xn - nx : xn)) +
                               nx * (yn < 0 ? yn + ny : (yn >= ny ? yn - ny : yn));
                const cx<T>* Ad = A + ((int64_t)s * 9 + d) * NC * NC + i;      // [j][i]
                const cx<T>* Xn = xin.p + (int64_t)sn * NC * nrhs + rhs;      // [dof][rhs]
#pragma unroll
                for (int j = 0; j < NC; ++j) acc = acc + Ad[j * NC] * Xn[(int64_t)j * nrhs];
            }
            const int64_t o = ((int64_t)s * NC + i) * nrhs + rhs;
            y[o] = acc;
            if (EPI == 1) {
                v[0] += norm2(acc);
            } else if (EPI == 2) {
                const cx<T> c = cmulc(acc, w[o]);
                v[0] += c.re;
                v[1] += c.im;
                v[2] += norm2(acc);
            }
        }
    if (EPI != 0) block_reduce_finalise<K>(v, partials, ticket, nrhs, FinStore{out, K});
}

// The same operator with one thread per (coarse site, rhs) forming all NC outputs of its site: each
// neighbour value is loaded once for the NC outputs and the links of a (direction, j) as NC / 2
// 16-byte loads shared by the site's rhs lanes, against two 8-byte loads per multiply-add when
// every output entry has its own thread.
template <typename T, int EPI, int NC>
__global__ void __launch_bounds__(256) k_coarse_apply_site(const cx<T>* __restrict__ A, VecView<T> xin,
                                                           cx<T>* __restrict__ y, int nx, int ny,
                                                           const cx<T>* __restrict__ w, double* partials,
                                                           unsigned int* ticket, double* out,
                                                           const int* __restrict__ gate) {
    if (gate && *gate == 0) return;  // every right-hand side of the solve has converged
    constexpr int K = EPI == 2 ? 3 : 1;
    const int nrhs = xin.nrhs;
    const int rhs = blockIdx.y * blockDim.x + threadIdx.x;
    T v[K];
#pragma unroll
    for (int k = 0; k < K; ++k) v[k] = T(0);
    if (rhs < nrhs)
        for (int s = blockIdx.x * blockDim.y + threadIdx.y; s < xin.nsites; s += gridDim.x * blockDim.y) {
            const int x = s % nx, yy = s / nx;
            cx<T> acc[NC];
#pragma unroll
            for (int i = 0; i < NC; ++i) acc[i] = mk<T>(0, 0);
#pragma unroll 1
            for (int d = 0; d < 9; ++d) {
                const int xn = x + c_dx[d], yn = yy + c_dy[d];
                const int sn = (xn < 0 ? xn + nx : (xn >= nx ? xn - nx : xn)) +
                               nx * (yn < 0 ? yn + ny : (yn >= ny ? yn - ny : yn));
                const cx<T>* __restrict__ Ad = A + ((int64_t)s * 9 + d) * NC * NC;  // [j][i]
                const cx<T>* __restrict__ Xn = xin.p + (int64_t)sn * NC * nrhs + rhs;  // [dof][rhs]
                cx<T> xj[NC];
#pragma unroll
                for (int j = 0; j < NC; ++j) xj[j] = Xn[(int64_t)j * nrhs];
#pragma unroll
                for (int j = 0; j < NC; ++j) {
#pragma unroll
                    for (int i = 0; i < NC; ++i) acc[i] = acc[i] + Ad[j * NC + i] * xj[j];
                }
            }
#pragma unroll
            for (int i = 0; i < NC; ++i) {
                const int64_t o = ((int64_t)s * NC + i) * nrhs + rhs;
                y[o] = acc[i];
                if (EPI == 1) {
                    v[0] += norm2(acc[i]);
                } else if (EPI == 2) {
                    const cx<T> c = cmulc(acc[i], w[o]);
                    v[0] += c.re;
                    v[1] += c.im;
                    v[2] += norm2(acc[i]);
                }
            }
        }
    if (EPI != 0) block_reduce_finalise<K>(v, partials, ticket, nrhs, FinStore{out, K});
}

// one thread per (site, rhs) for few right-hand sides (k_coarse_apply_site); SMG_COARSE_SITE=0 keeps
// one thread per output entry (k_coarse_apply_flat)
bool coarse_site_on() {
    static const bool on = [] {
        const char* e = std::getenv("SMG_COARSE_SITE");
        return !(e && std::atoi(e) == 0);
    }();
    return on;
}

// ------------------------------------------------------------ persistent coarsest CG
// The whole coarsest-level CG of one right-hand side in one cooperative
// launch (SparseCoarseOp::solve without deflation, src/coarse_op.h:492-547).
// Per iteration: Ap = A p with the partial <p, Ap> of each block, barrier;
// x += alpha p, r -= alpha Ap with the partial ||r||^2, barrier; p = r + beta p,
// barrier.  Every block sums the per-block partials itself in block order, so
// all blocks take identical (deterministic) scalar decisions without a further
// barrier.  Every barrier wait is bounded; on timeout the kernel raises
// *err and returns.
struct CoarseCgArgs {
    const void* A = nullptr;
    const void* b = nullptr;
    void* x = nullptr;
    void* r = nullptr;
    void* p = nullptr;
    void* Ap = nullptr;
    int nx = 0, ny = 0, nsites = 0, max_iter = 0;
    double tol2 = 0;
    double* part = nullptr;        // [2][gridDim.x]
    unsigned int* bar = nullptr;   // [0] arrivals, [1] generation
    int* err = nullptr;            // 0 ok, 1 barrier timeout
    int* iters = nullptr;          // iterations done (written by block 0)
    long long spin_limit = 0;      // polls of a barrier wait before it gives up and raises err
};

constexpr long long kBarrierSpinLimit = 1ll << 22;  // x 256 ns sleep ~ 1 s

// a grid-wide barrier of a co-resident (cooperative) grid; a wait polls at most spin_limit times
// (spin_limit 0: it gives up at the first poll), then raises *err and the block returns false
__device__ __forceinline__ bool grid_barrier(unsigned int* bar, int* err, long long spin_limit) {
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
            const unsigned int arrived = atomicAdd(bar, 1u);
            if (arrived == gridDim.x - 1) {
                bar[0] = 0u;
                __threadfence();
                atomicAdd(bar + 1, 1u);
            } else {
                long long k = 0;
                while (*vgen == gen) {
                    if (*verr || ++k > spin_limit) {
                        atomicExch(err, 1);
                        ok = 0;
                        break;
                    }
                    __nanosleep(256);
                }
            }
            __threadfence();
        }
        s_ok = ok;
    }
    __syncthreads();
    return s_ok != 0;
}

// block sum of v (256 threads), result valid in every thread
__device__ __forceinline__ double block_sum256(double v) {
    __shared__ double s_w[8];
    for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    __syncthreads();
    if ((threadIdx.x & 31) == 0) s_w[threadIdx.x >> 5] = v;
    __syncthreads();
    double t = 0;
    for (int w = 0; w < 8; ++w) t += s_w[w];
    return t;
}

// every block sums part[0 .. gridDim.x) in order (identical result everywhere)
__device__ __forceinline__ double sum_partials(const double* part) {
    __shared__ double s_tot;
    if (threadIdx.x < 32) {
        double t = 0;
        for (int i = threadIdx.x; i < (int)gridDim.x; i += 32) t += __ldcg(part + i);
        for (int o = 16; o; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
        if (threadIdx.x == 0) s_tot = t;
    }
    __syncthreads();
    return s_tot;
}

// L2-coherent load of a complex written by another block during this kernel
__device__ __forceinline__ cx<float> ldcg_cx(const cx<float>* q) {
    float2 v = __ldcg(reinterpret_cast<const float2*>(q));
    return mk(v.x, v.y);
}
__device__ __forceinline__ cx<double> ldcg_cx(const cx<double>* q) {
    double2 v = __ldcg(reinterpret_cast<const double2*>(q));
    return mk(v.x, v.y);
}

template <typename T, int NC>
__global__ void __launch_bounds__(256) k_coarse_cg1(CoarseCgArgs a) {
    const cx<T>* A = (const cx<T>*)a.A;
    const cx<T>* b = (const cx<T>*)a.b;
    cx<T>* x = (cx<T>*)a.x;
    cx<T>* r = (cx<T>*)a.r;
    cx<T>* p = (cx<T>*)a.p;
    cx<T>* Ap = (cx<T>*)a.Ap;
    const int n = a.nsites * NC;
    const int stride = gridDim.x * blockDim.x;
    const int t0 = blockIdx.x * blockDim.x + threadIdx.x;
    double* part0 = a.part;              // <p, Ap> partials
    double* part1 = a.part + gridDim.x;  // ||r||^2 partials
    // x = 0, r = p = b (each element is owned by one thread for the whole solve)
    T loc_t = 0;  // per-thread partials in the field precision
    for (int e = t0; e < n; e += stride) {
        const cx<T> v = b[e];
        x[e] = mk<T>(0, 0);
        r[e] = v;
        p[e] = v;
        loc_t += norm2(v);
    }
    double loc = block_sum256((double)loc_t);
    if (threadIdx.x == 0) part1[blockIdx.x] = loc;
    if (!grid_barrier(a.bar, a.err, a.spin_limit)) return;
    double rr = sum_partials(part1);
    const double bnorm2 = rr;
    int it = 0;
    const bool solve = bnorm2 >= 1e-60 && isfinite(bnorm2);  // ||b|| < 1e-30 returns x = 0
    while (solve && it < a.max_iter) {
        // Ap = A p, partial <Ap, p>
        T pap_t = 0;
        for (int e = t0; e < n; e += stride) {
            const int s = e / NC, i = e - s * NC;
            const int xs = s % a.nx, ys = s / a.nx;
            cx<T> acc = mk<T>(0, 0);
#pragma unroll 3
            for (int d = 0; d < 9; ++d) {
                const int xn = xs + c_dx[d], yn = ys + c_dy[d];
                const int sn = (xn < 0 ? xn + a.nx : (xn >= a.nx ? xn - a.nx : xn)) +
                               a.nx * (yn < 0 ? yn + a.ny : (yn >= a.ny ? yn - a.ny : yn));
                const cx<T>* Ad = A + ((int64_t)s * 9 + d) * NC * NC + i;
                const cx<T>* pv = p + (int64_t)sn * NC;
#pragma unroll
                for (int j = 0; j < NC; ++j) acc = acc + Ad[j * NC] * ldcg_cx(pv + j);
            }
            Ap[e] = acc;
            pap_t += cmulc(acc, p[e]).re;
        }
        double pap = block_sum256((double)pap_t);
        if (threadIdx.x == 0) part0[blockIdx.x] = pap;
        if (!grid_barrier(a.bar, a.err, a.spin_limit)) return;
        pap = sum_partials(part0);
        if (!(fabs(pap) >= 1e-30) || !isfinite(pap)) break;  // coarse_op.h:522
        const T al = (T)(rr / pap);
        T rloc_t = 0;
        for (int e = t0; e < n; e += stride) {
            const cx<T> ri = r[e] - al * Ap[e];
            x[e] = x[e] + al * p[e];
            r[e] = ri;
            rloc_t += norm2(ri);
        }
        double rloc = block_sum256((double)rloc_t);
        if (threadIdx.x == 0) part1[blockIdx.x] = rloc;
        if (!grid_barrier(a.bar, a.err, a.spin_limit)) return;
        const double rr_new = sum_partials(part1);
        ++it;
        if (!isfinite(rr_new) || rr_new < a.tol2 * bnorm2) break;  // coarse_op.h:531-536
        const T be = (T)(rr_new / rr);
        rr = rr_new;
        for (int e = t0; e < n; e += stride) p[e] = r[e] + be * p[e];
        if (!grid_barrier(a.bar, a.err, a.spin_limit)) return;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) *a.iters = it;
}

template <typename D, typename S>
__global__ void k_cvt_flat(const cx<S>* __restrict__ in, cx<D>* __restrict__ out, int64_t n) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = cvt<D>(in[i]);
}

// coarsest-level CG scalars per rhs: rr, pAp (re, im, norm from the fused
// epilogue), bnorm2, active, and the update kernel's finaliser
struct CcgState {
    double* rr = nullptr;
    double* pap3 = nullptr;  // [rhs][3]: <Ap, p> re, im, ||Ap||^2
    double* bnorm2 = nullptr;
    double* beta = nullptr;
    int* active = nullptr;
    int* n_active = nullptr;
    double tol2 = 0;
};

// bnorm2 = ||b||^2: taken from rr = ||r0||^2 = ||b||^2 for a zero start, or already in place
// (have_bnorm) for a deflated start
__global__ void k_ccg_init(CcgState s, int nrhs, int have_bnorm) {
    if (threadIdx.x == 0) *s.n_active = 0;
    __syncthreads();
    for (int j = threadIdx.x; j < nrhs; j += blockDim.x) {
        if (!have_bnorm) s.bnorm2[j] = s.rr[j];
        s.beta[j] = 0.0;
        int act = (s.rr[j] >= 1e-60 && isfinite(s.rr[j]) && s.bnorm2[j] >= 1e-60) ? 1 : 0;
        if (act && s.rr[j] < s.tol2 * s.bnorm2[j]) act = 0;  // the initial guess already converged
        s.active[j] = act;
        if (act) atomicAdd(s.n_active, 1);
    }
}

struct FinCcg {
    CcgState s;
    __device__ void operator()(int j, const double* sums) const {
        double rr_new = sums[0];
        if (!s.active[j]) {
            s.beta[j] = 0.0;
            return;
        }
        if (!isfinite(rr_new) || rr_new < s.tol2 * s.bnorm2[j]) {
            s.active[j] = 0;
            atomicSub(s.n_active, 1);
            s.beta[j] = 0.0;
            return;
        }
        s.beta[j] = rr_new / s.rr[j];
        s.rr[j] = rr_new;
    }
};

// x += alpha p, r -= alpha Ap with alpha = rr / <p, Ap>; ||r||^2 -> finaliser
template <typename T>
__global__ void __launch_bounds__(256) k_ccg_update(CcgState s, VecView<T> x, cx<T>* __restrict__ r,
                                                    const cx<T>* __restrict__ p, const cx<T>* __restrict__ Ap,
                                                    double* partials, unsigned int* ticket) {
    if (*s.n_active == 0) return;  // read by every block before the finaliser can change it
    __shared__ T s_al[32];
    const int nrhs = x.nrhs;
    const int rhs = blockIdx.y * blockDim.x + threadIdx.x;
    if (threadIdx.y == 0) {
        T al = 0;
        if (rhs < nrhs && s.active[rhs]) {
            // <p, Ap> = conj(<Ap, p>) is real for Hermitian positive A
            double pap = s.pap3[3 * rhs];
            if (fabs(pap) >= 1e-30 && isfinite(pap)) al = (T)(s.rr[rhs] / pap);
        }
        s_al[threadIdx.x] = al;
    }
    __syncthreads();
    const T al = s_al[threadIdx.x];
    T v[1] = {T(0)};
    cx<T>* __restrict__ xp = x.p;
    if (rhs < nrhs) {
        // coarse vectors [site][dof][rhs]: entry (e = site * ndof + dof, rhs) at e * nrhs + rhs; four
        // entries per thread and pass with every load issued first
        constexpr int U = 4;
        const int64_t nel = (int64_t)x.nsites * x.ndof;
        for (int64_t e0 = ((int64_t)blockIdx.x * blockDim.y + threadIdx.y) * U; e0 < nel;
             e0 += (int64_t)gridDim.x * blockDim.y * U) {
            cx<T> rv[U], av[U], xv[U], pv[U];
#pragma unroll
            for (int u = 0; u < U; ++u)
                if (e0 + u < nel) {
                    const int64_t e = (e0 + u) * nrhs + rhs;
                    rv[u] = r[e];
                    av[u] = Ap[e];
                    xv[u] = xp[e];
                    pv[u] = p[e];
                }
#pragma unroll
            for (int u = 0; u < U; ++u)
                if (e0 + u < nel) {
                    const int64_t e = (e0 + u) * nrhs + rhs;
                    const cx<T> ri = rv[u] - al * av[u];
                    xp[e] = xv[u] + al * pv[u];
                    r[e] = ri;
                    v[0] += norm2(ri);
                }
        }
    }
    block_reduce_finalise<1>(v, partials, ticket, nrhs, FinCcg{s});
}

template <typename T>
__global__ void k_ccg_p(CcgState s, VecView<T> p, const cx<T>* __restrict__ r) {
    if (*s.n_active == 0) return;
    const int rhs = blockIdx.y * blockDim.x + threadIdx.x;
    const int st = blockIdx.x * blockDim.y + threadIdx.y;
    if (rhs >= p.nrhs || st >= p.nsites) return;
    const T be = (T)s.beta[rhs];
    const int64_t base = p.idx(st, rhs, 0);
    const int ds = p.dstride();
    for (int d = 0; d < p.ndof; ++d) p.p[base + (int64_t)d * ds] = r[base + (int64_t)d * ds] + be * p.p[base + (int64_t)d * ds];
}

// ---- the coarsest CG on FP16 vectors (coarse_half): r and p as __half2 [site][dof][rhs] with one
// FP32 scale per coarse site (the largest |re| or |im| of all its dofs and right-hand sides), x and
// A p in FP32, every arithmetic operation in FP32.  nrhs = 32, 16 dofs: a warp owns a site, lane =
// right-hand side, looping over the 16 dofs (128-byte accesses per dof), so the site maximum is a
// warp reduction; blocks of 8 warps walk the sites.
constexpr int kCgHalfDofs = 16;

__device__ __forceinline__ float warp_max(float m) { return warp_max_nonneg(m); }
__device__ __forceinline__ float absmax2(cx<float> z) { return fmaxf(fabsf(z.re), fabsf(z.im)); }
// the 16 dofs of (site, lane) in FP16 with the site maximum m (reduced over the warp)
__device__ __forceinline__ void st_site16(__half2* f, float* sc, int64_t e0, int site, const cx<float> (&v)[kCgHalfDofs],
                                          float m) {
    const float inv = m > 0.f ? __fdividef(1.0f, m) : 0.f;
#pragma unroll
    for (int d = 0; d < kCgHalfDofs; ++d) f[e0 + d * 32] = __floats2half2_rn(v[d].re * inv, v[d].im * inv);
    if (threadIdx.x == 0) sc[site] = m;
}

// r = p = b (FP16), x = 0, ||r||^2 per rhs into out
__global__ void __launch_bounds__(256) k_ccgh_init(const cx<float>* __restrict__ b, cx<float>* __restrict__ x,
                                                   __half2* __restrict__ r, float* __restrict__ rs,
                                                   __half2* __restrict__ p, float* __restrict__ ps, int nsites,
                                                   double* partials, unsigned int* ticket, double* out) {
    float n2 = 0.f;
    for (int site = blockIdx.x * blockDim.y + threadIdx.y; site < nsites; site += gridDim.x * blockDim.y) {
        const int64_t e0 = (int64_t)site * kCgHalfDofs * 32 + threadIdx.x;
        cx<float> v[kCgHalfDofs];
        float m = 0.f;
#pragma unroll
        for (int d = 0; d < kCgHalfDofs; ++d) {
            v[d] = b[e0 + d * 32];
            x[e0 + d * 32] = mk(0.f, 0.f);
            m = fmaxf(m, absmax2(v[d]));
            n2 += norm2(v[d]);
        }
        m = warp_max(m);
        st_site16(r, rs, e0, site, v, m);
        st_site16(p, ps, e0, site, v, m);
    }
    double v[1] = {(double)n2};
    block_reduce_finalise<1>(v, partials, ticket, 32, FinStore{out, 1});
}

// x += alpha p, r -= alpha A p with alpha = rr / <p, A p>; ||r||^2 -> finaliser
__global__ void __launch_bounds__(256) k_ccgh_update(CcgState s, cx<float>* __restrict__ x, __half2* __restrict__ r,
                                                     float* __restrict__ rs, const __half2* __restrict__ p,
                                                     const float* __restrict__ ps, const cx<float>* __restrict__ Ap,
                                                     int nsites, double* partials, unsigned int* ticket) {
    if (*s.n_active == 0) return;  // read by every block before the finaliser can change it
    const int rhs = threadIdx.x;
    float al = 0.f;
    if (s.active[rhs]) {
        const double pap = s.pap3[3 * rhs];  // <Ap, p>, real for Hermitian positive A
        if (fabs(pap) >= 1e-30 && isfinite(pap)) al = (float)(s.rr[rhs] / pap);
    }
    float n2 = 0.f;
    for (int site = blockIdx.x * blockDim.y + threadIdx.y; site < nsites; site += gridDim.x * blockDim.y) {
        const int64_t e0 = (int64_t)site * kCgHalfDofs * 32 + rhs;
        const float sr = rs[site], sp = ps[site];
        cx<float> rn[kCgHalfDofs];
        float m = 0.f;
#pragma unroll
        for (int d = 0; d < kCgHalfDofs; ++d) {
            const float2 rv = __half22float2(r[e0 + d * 32]);
            const float2 pv = __half22float2(p[e0 + d * 32]);
            const cx<float> av = Ap[e0 + d * 32];
            cx<float> xv = x[e0 + d * 32];
            xv.re += al * sp * pv.x;
            xv.im += al * sp * pv.y;
            x[e0 + d * 32] = xv;
            rn[d] = mk(sr * rv.x - al * av.re, sr * rv.y - al * av.im);
            m = fmaxf(m, absmax2(rn[d]));
            n2 += norm2(rn[d]);
        }
        m = warp_max(m);
        __syncwarp();  // every lane has read this site's scale before lane 0 replaces it
        st_site16(r, rs, e0, site, rn, m);
    }
    double v[1] = {(double)n2};
    block_reduce_finalise<1>(v, partials, ticket, 32, FinCcg{s});
}

// p = r + beta p
__global__ void __launch_bounds__(256) k_ccgh_p(CcgState s, const __half2* __restrict__ r, const float* __restrict__ rs,
                                                __half2* __restrict__ p, float* __restrict__ ps, int nsites) {
    if (*s.n_active == 0) return;
    const float be = (float)s.beta[threadIdx.x];
    for (int site = blockIdx.x * blockDim.y + threadIdx.y; site < nsites; site += gridDim.x * blockDim.y) {
        const int64_t e0 = (int64_t)site * kCgHalfDofs * 32 + threadIdx.x;
        const float sr = rs[site], sp = ps[site] * be;
        cx<float> pn[kCgHalfDofs];
        float m = 0.f;
#pragma unroll
        for (int d = 0; d < kCgHalfDofs; ++d) {
            const float2 rv = __half22float2(r[e0 + d * 32]);
            const float2 pv = __half22float2(p[e0 + d * 32]);
            pn[d] = mk(sr * rv.x + sp * pv.x, sr * rv.y + sp * pv.y);
            m = fmaxf(m, absmax2(pn[d]));
        }
        m = warp_max(m);
        __syncwarp();  // every lane has read this site's scale before lane 0 replaces it
        st_site16(p, ps, e0, site, pn, m);
    }
}

}  // namespace


// ---- the intermediate-level MR smoother on FP16 vectors (coarse_half): [site][16 dofs][32 rhs]
// __half2 with one FP32 scale per site and rhs half.  A warp owns a (site, half) unit: lane l takes
// rhs 16 h + l % 16 and dofs 8 (l / 16) .. + 7, so that each access instruction covers two
// contiguous 128-byte (FP32) or 64-byte (FP16) runs and the unit's scale is a warp maximum.
constexpr int kC16Dofs = 16;
constexpr int kC16MaxSteps = 8;  // MR steps one x pass combines
struct C16Unit {
    int64_t site;
    int h, rhs, d0;
};
__device__ __forceinline__ C16Unit c16_unit(int64_t u) {
    const int lane = threadIdx.x & 31;
    C16Unit c;
    c.site = u >> 1;
    c.h = (int)(u & 1);
    c.rhs = 16 * c.h + (lane & 15);
    c.d0 = 8 * (lane >> 4);
    return c;
}
__device__ __forceinline__ int64_t c16_idx(const C16Unit& c, int j) { return (c.site * kC16Dofs + c.d0 + j) * 32 + c.rhs; }
// stores the unit's 8 values of this lane with the unit's scale (the warp's largest |re| or |im|)
__device__ __forceinline__ void c16_store(const C16Unit& c, const cx<float> (&v)[8], __half2* __restrict__ out,
                                          float* __restrict__ os) {
    float m = 0.f;
#pragma unroll
    for (int j = 0; j < 8; ++j) m = fmaxf(m, fmaxf(fabsf(v[j].re), fabsf(v[j].im)));
    m = warp_max_nonneg(m);
    const float inv = m > 0.f ? __fdividef(1.0f, m) : 0.f;
#pragma unroll
    for (int j = 0; j < 8; ++j) out[c16_idx(c, j)] = __floats2half2_rn(v[j].re * inv, v[j].im * inv);
    if ((threadIdx.x & 31) == 0) os[2 * c.site + c.h] = m;
}

// r = b - y (y may be null: r = b), FP32 in, FP16 out; one warp per unit
__global__ void __launch_bounds__(256) k_c16_from(const cx<float>* __restrict__ b, const cx<float>* __restrict__ y,
                                                  __half2* __restrict__ r, float* __restrict__ rs, int nsites) {
    const int64_t u = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (u >= 2ll * nsites) return;
    const C16Unit c = c16_unit(u);
    cx<float> v[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) v[j] = b[c16_idx(c, j)];
    if (y) {
#pragma unroll
        for (int j = 0; j < 8; ++j) v[j] = v[j] - y[c16_idx(c, j)];
    }
    c16_store(c, v, r, rs);
}

// r' = r - omega Ar (all FP16), omega per rhs
__global__ void __launch_bounds__(256) k_c16_rupdate(const __half2* __restrict__ r, const float* __restrict__ rs,
                                                     const __half2* __restrict__ ar, const float* __restrict__ ars,
                                                     const float2* __restrict__ omega, __half2* __restrict__ ro,
                                                     float* __restrict__ ros, int nsites) {
    const int64_t u = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (u >= 2ll * nsites) return;
    const C16Unit c = c16_unit(u);
    const float2 om = omega[c.rhs];
    const float sr = rs[2 * c.site + c.h], sa = ars[2 * c.site + c.h];
    __half2 rv[8], av[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        rv[j] = r[c16_idx(c, j)];
        av[j] = ar[c16_idx(c, j)];
    }
    cx<float> v[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        const float2 a = __half22float2(rv[j]), y = __half22float2(av[j]);
        const float yr = sa * y.x, yi = sa * y.y;
        v[j] = mk(sr * a.x - (om.x * yr - om.y * yi), sr * a.y - (om.x * yi + om.y * yr));
    }
    c16_store(c, v, ro, ros);
}

// the MR residuals of one smoothing as a list of FP16 vectors
struct C16Ring {
    const __half2* r[kC16MaxSteps];
    const float* s[kC16MaxSteps];
};
// x (+)= sum_k omega_k r_k over n FP16 residuals (omega [k][32]); x FP32 [site][dof][32]; one warp per
// four (site, dof) rows of 32 rhs (lane = rhs, the rows of one site share its scales), every load of
// the four rows issued first: short-lived one-row warps left the kernel latency-bound
constexpr int kC16XRows = 4;
__global__ void __launch_bounds__(256) k_c16_xupdate(cx<float>* __restrict__ x, C16Ring ring, int n,
                                                     const float2* __restrict__ omega, int nsites, int zero) {
    const int lane = threadIdx.x & 31;
    const int64_t e0 = ((int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5)) * kC16XRows;
    if (e0 >= (int64_t)nsites * kC16Dofs) return;
    const int64_t site = e0 / kC16Dofs;  // kC16Dofs is a multiple of kC16XRows
    __half2 rv[kC16MaxSteps][kC16XRows];
    float sc[kC16MaxSteps];
    float2 om[kC16MaxSteps];
    cx<float> acc[kC16XRows];
#pragma unroll
    for (int k = 0; k < kC16MaxSteps; ++k)
        if (k < n) {
#pragma unroll
            for (int j = 0; j < kC16XRows; ++j) rv[k][j] = ring.r[k][(e0 + j) * 32 + lane];
            sc[k] = ring.s[k][2 * site + (lane >> 4)];
            om[k] = omega[k * 32 + lane];
        }
#pragma unroll
    for (int j = 0; j < kC16XRows; ++j) acc[j] = zero ? mk(0.f, 0.f) : x[(e0 + j) * 32 + lane];
#pragma unroll
    for (int k = 0; k < kC16MaxSteps; ++k)
        if (k < n) {
            const float wr = om[k].x * sc[k], wi = om[k].y * sc[k];  // omega_k times the scale
#pragma unroll
            for (int j = 0; j < kC16XRows; ++j) {
                const float2 a = __half22float2(rv[k][j]);
                acc[j] = mk(acc[j].re + wr * a.x - wi * a.y, acc[j].im + wr * a.y + wi * a.x);
            }
        }
#pragma unroll
    for (int j = 0; j < kC16XRows; ++j) x[(e0 + j) * 32 + lane] = acc[j];
}
// ====================================================================== host

struct CoarseWork {  // per level l >= 1, per precision
    void* b = nullptr;
    void* x = nullptr;
    void* r = nullptr;
    void* Ar = nullptr;
    void* e = nullptr;
    void* p = nullptr;
    // coarsest level with coarse_half: the CG's residual and search direction in FP16 (__half2
    // [site][dof][rhs]) with one FP32 scale per site
    void* rh = nullptr;
    void* ph = nullptr;
    float* rs = nullptr;
    float* ps = nullptr;
    // the persistent tensor-core CG (k_ccg_tc): the second search-direction buffer and the per-CTA
    // partial sums
    void* ph2 = nullptr;
    float* ps2 = nullptr;
    double* ccg_part = nullptr;
    // intermediate level with coarse_half: the MR residuals r_0 .. r_n of one smoothing and A r in
    // FP16 (scales per site and rhs half), the steps' MR scalars [step][rhs][3] and step sizes
    // [step][rhs], and the ring slot of the last smoothing's final residual
    std::vector<void*> r16;
    std::vector<float*> r16s;
    void* ar16 = nullptr;
    float* ar16s = nullptr;
    double* mr16_sc = nullptr;
    float* mr16_om = nullptr;
    int res16 = -1;
    // pre-smoothing x update left to the packed prolongation into this level:
    // x = (xp_zero ? 0 : x) + sum_{k < xp_n} omega_k r16[k]
    int xp_n = 0;
    bool xp_zero = false;
    // the pre-smoother's last residual left to the packed restriction: that MR step, or -1
    int rn_step = -1;
};

struct smg_mg {
    smg_context* ctx = nullptr;
    smg_dirac* dirac = nullptr;
    smg_mg_params p{};
    std::vector<Level> lv;
    std::vector<smg_field*> null0;  // level-0 null vectors, single-RHS F64 fields
    // workspace, rebuilt when nrhs or precision changes
    int work_nrhs = 0;
    smg_precision work_prec = SMG_F64;
    smg_field *f_r = nullptr, *f_Ar = nullptr, *f_t = nullptr;  // fine MR temps
    // FP16 smoother: residuals r_0 .. r_n of one smoothing (f_r aliases f_rs[0]), the field that
    // holds the last smoothing's final residual, the norm partials of its stencils and every step's
    // MR scalars [step][rhs][3]
    std::vector<smg_field*> f_rs;
    smg_field* f_res = nullptr;
    float* hdots = nullptr;
    double* mr_om = nullptr;
    float2* mr_omf = nullptr;  // each step's omega per rhs, as the update kernels read it
    // pre-smoothing x update left to the level-0 prolongation: x = (xp_zero ? 0 : x) +
    // sum_{k < xp_n} omega_k f_rs[xp_first + k]
    int xp_first = 0, xp_n = 0;
    bool xp_zero = false;
    double xp_omega = 0;
    // the pre-smoother's last residual r - omega A r left to the packed level-0 restriction: the step
    // (its r in f_rs[rn_step], A r in f_Ar, omega from mr_omf or rn_omega), or -1
    int rn_step = -1;
    double rn_omega = 0;
    std::vector<CoarseWork> cw;
    double* scal = nullptr;  // per-level scalar area
    size_t scal_doubles = 0;
    // CUDA graph of one cycle on internal input/output fields, per (nrhs, precision)
    bool capturing = false;
    bool use_graph = true;
    smg_field* g_in = nullptr;
    smg_field* g_out = nullptr;
    cudaGraphExec_t g_exec = nullptr;
    uint64_t g_launches = 0;
    uint64_t work_gen = 0;   // bumped whenever the workspace is reallocated
    uint64_t g_work_gen = 0; // workspace generation the graph was captured with
    // persistent coarsest CG: barrier words, error flag, iteration count, partials
    bool persistent = true;
    long long spin_limit = kBarrierSpinLimit;  // the grid barrier's wait bound (smg_mg_set_wait_limit)
    void* cg_state = nullptr;  // [0..1] barrier, [2] err, [3] iters (ints), doubles from byte 256
    // eigenpairs of the level-1 operator: the deflated initial guess of the coarsest CG when level 1
    // is the coarsest level, and the low-mode projector of the multi-timescale HMC
    MgDeflation defl;
    // during set-up only: caller-drawn start vectors per level (smg_mg_create_from_starts)
    const double* const* starts = nullptr;
};

namespace {

template <typename T>
const cx<T>* Vp(const Level& L);
template <>
const cx<double>* Vp<double>(const Level& L) { return L.V64; }
template <>
const cx<float>* Vp<float>(const Level& L) { return L.V32; }
template <typename T>
const cx<T>* Ap(const Level& L);
template <>
const cx<double>* Ap<double>(const Level& L) { return L.A64; }
template <>
const cx<float>* Ap<float>(const Level& L) { return L.A32; }

int blocks_for(int64_t n, int t = 256) { return (int)((n + t - 1) / t); }

// --- fine-level helpers on smg_field
template <typename T>
VecView<T> fview(const smg_field* f) {
    VecView<T> v;
    v.p = (cx<T>*)f->data;
    v.nsites = f->g.V;
    v.nrhs = f->nrhs;
    v.ndof = 2;
    return v;
}

// a single-RHS vector viewed as a flat array of single-dof sites, so the
// elementwise and reduction kernels get one thread per complex entry
template <typename T>
VecView<T> flat(VecView<T> v) {
    if (v.nrhs == 1) {
        v.nsites *= v.ndof;
        v.ndof = 1;
    }
    return v;
}

template <typename T>
VecView<T> cview(void* p, const Level& L, int nrhs) {
    VecView<T> v;
    v.p = (cx<T>*)p;
    v.nsites = L.nsites;
    v.nrhs = nrhs;
    v.ndof = L.ndof;
    v.rhs_inner = 1;  // coarse vectors: [site][dof][rhs]
    return v;
}

template <typename T>
smg_status vreduce(smg_context* ctx, VecView<T> a, const cx<T>* b, int mode, double* out) {
    ReduceLaunch rl = reduce_launch(a.nsites, a.nrhs);
    SMG_TRY(smg_reduce_reserve(ctx, (size_t)rl.grid.x * a.nrhs * 3));
    if (mode == VR_DOT)
        k_vreduce<T, VR_DOT><<<rl.grid, rl.block, 0, ctx->stream>>>(a, b, ctx->red.partials, ctx->red.tickets, out);
    else if (mode == VR_NORM)
        k_vreduce<T, VR_NORM><<<rl.grid, rl.block, 0, ctx->stream>>>(a, b, ctx->red.partials, ctx->red.tickets, out);
    else
        k_vreduce<T, VR_DOTNORM><<<rl.grid, rl.block, 0, ctx->stream>>>(a, b, ctx->red.partials, ctx->red.tickets, out);
    count_launch(ctx);
    SMG_CHECK_LAUNCH(ctx);
    return SMG_OK;
}

template <typename T>
smg_status vaxpy(smg_context* ctx, VecView<T> y, const cx<T>* x, const double* coef, double sgn) {
    k_vaxpy<T><<<vec_grid(y.nsites, y.nrhs), vec_block(y.nrhs), 0, ctx->stream>>>(y, x, coef, sgn);
    count_launch(ctx);
    SMG_CHECK_LAUNCH(ctx);
    return SMG_OK;
}

template <typename T, int NC>
smg_status coarse_apply_tiled(smg_context* ctx, const Level& L, const cx<T>* A, VecView<T> x, cx<T>* y, int epi,
                              const cx<T>* w, double* out, const int* gate) {
    if constexpr (NC <= 16) {
    if (x.nrhs < 32 && coarse_site_on()) {  // few right-hand sides: one thread per (site, rhs)
        ReduceLaunch rl = reduce_launch(L.nsites, x.nrhs);
        SMG_TRY(smg_reduce_reserve(ctx, (size_t)rl.grid.x * x.nrhs * 3));
        double* part = epi ? ctx->red.partials : nullptr;
        unsigned int* tick = epi ? ctx->red.tickets : nullptr;
        if (epi == 0)
            k_coarse_apply_site<T, 0, NC><<<rl.grid, rl.block, 0, ctx->stream>>>(A, x, y, L.nx, L.ny, w, part, tick,
                                                                                out, gate);
        else if (epi == 1)
            k_coarse_apply_site<T, 1, NC><<<rl.grid, rl.block, 0, ctx->stream>>>(A, x, y, L.nx, L.ny, w, part, tick,
                                                                                out, gate);
        else
            k_coarse_apply_site<T, 2, NC><<<rl.grid, rl.block, 0, ctx->stream>>>(A, x, y, L.nx, L.ny, w, part, tick,
                                                                                out, gate);
        count_launch(ctx);
        SMG_CHECK_LAUNCH(ctx);
        return SMG_OK;
    }
    }
    if (x.nrhs < 32) {  // few right-hand sides: one thread per output entry
        ReduceLaunch rl = reduce_launch((int)((int64_t)L.nsites * NC), x.nrhs);
        SMG_TRY(smg_reduce_reserve(ctx, (size_t)rl.grid.x * x.nrhs * 3));
        double* part = epi ? ctx->red.partials : nullptr;
        unsigned int* tick = epi ? ctx->red.tickets : nullptr;
        if (epi == 0)
            k_coarse_apply_flat<T, 0, NC><<<rl.grid, rl.block, 0, ctx->stream>>>(A, x, y, L.nx, L.ny, w, part, tick,
                                                                                out, gate);
        else if (epi == 1)
            k_coarse_apply_flat<T, 1, NC><<<rl.grid, rl.block, 0, ctx->stream>>>(A, x, y, L.nx, L.ny, w, part, tick,
                                                                                out, gate);
        else
            k_coarse_apply_flat<T, 2, NC><<<rl.grid, rl.block, 0, ctx->stream>>>(A, x, y, L.nx, L.ny, w, part, tick,
                                                                                out, gate);
        count_launch(ctx);
        SMG_CHECK_LAUNCH(ctx);
        return SMG_OK;
    }
    ReduceLaunch rl = reduce_launch(L.nsites, x.nrhs);  // lanes = rhs lanes, rows = 256 / lanes >= 8
    SMG_TRY(smg_reduce_reserve(ctx, (size_t)rl.grid.x * x.nrhs * 3));
    if (epi == 0)
        k_coarse_apply_tiled<T, 0, NC><<<rl.grid, rl.block, 0, ctx->stream>>>(A, x, y, L.nx, L.ny, w, nullptr,
                                                                             nullptr, nullptr, gate);
    else if (epi == 1)
        k_coarse_apply_tiled<T, 1, NC><<<rl.grid, rl.block, 0, ctx->stream>>>(A, x, y, L.nx, L.ny, w,
                                                                             ctx->red.partials, ctx->red.tickets, out,
                                                                             gate);
    else
        k_coarse_apply_tiled<T, 2, NC><<<rl.grid, rl.block, 0, ctx->stream>>>(A, x, y, L.nx, L.ny, w,
                                                                             ctx->red.partials, ctx->red.tickets, out,
                                                                             gate);
    count_launch(ctx);
    SMG_CHECK_LAUNCH(ctx);
    return SMG_OK;
}

// the tensor-core kernel takes FP32 coarse vectors of 16 dofs, rhs innermost, in multiples of 32
bool tc_path(const smg_mg* mg, int l, int nrhs) {
    const Level& L = mg->lv[l];
    return L.Atc != nullptr && nrhs % 32 == 0 && nrhs / 32 <= kMaxTickets;
}

int* device_err(smg_mg* mg) { return mg->cg_state ? reinterpret_cast<int*>(static_cast<char*>(mg->cg_state) + 8) : nullptr; }

template <typename T>
smg_status coarse_apply(smg_mg* mg, int l, VecView<T> x, cx<T>* y, int epi, const cx<T>* w, double* out,
                        const int* gate = nullptr, int engine = -1) {
    smg_context* ctx = mg->ctx;
    const Level& L = mg->lv[l];
    if constexpr (std::is_same<T, float>::value) {
        // engine -1: tensor cores where the shape allows; 0: CUDA cores; 1: tensor cores
        if (engine != 0 && x.rhs_inner && tc_path(mg, l, x.nrhs))
            return smg_coarse_tc_apply(ctx, L.Atc, L.nx, L.ny, x.nrhs, x.p, y, epi, w, out, gate, device_err(mg));
        if (engine == 1) return smg_fail(ctx, SMG_UNSUPPORTED, "tensor-core coarse apply: shape not supported");
    }
    if (x.nrhs == 1 && (L.ndof == 8 || L.ndof == 16 || L.ndof == 32)) {
        ReduceLaunch rl = reduce_launch((int)((int64_t)L.nsites * L.ndof), 1);
        SMG_TRY(smg_reduce_reserve(ctx, (size_t)rl.grid.x * 3));
        double* pp = epi ? ctx->red.partials : nullptr;
        unsigned int* tk = epi ? ctx->red.tickets : nullptr;
#define SMG_CA1(NC)                                                                                                  \
    do {                                                                                                             \
        if (epi == 0)                                                                                                \
            k_coarse_apply1<T, 0, NC><<<rl.grid, rl.block, 0, ctx->stream>>>(Ap<T>(L), x, y, L.nx, L.ny, w, pp, tk,  \
                                                                            out, gate);                              \
        else if (epi == 1)                                                                                           \
            k_coarse_apply1<T, 1, NC><<<rl.grid, rl.block, 0, ctx->stream>>>(Ap<T>(L), x, y, L.nx, L.ny, w, pp, tk,  \
                                                                            out, gate);                              \
        else                                                                                                         \
            k_coarse_apply1<T, 2, NC><<<rl.grid, rl.block, 0, ctx->stream>>>(Ap<T>(L), x, y, L.nx, L.ny, w, pp, tk,  \
                                                                            out, gate);                              \
    } while (0)
        if (L.ndof == 8) SMG_CA1(8);
        else if (L.ndof == 16) SMG_CA1(16);
        else SMG_CA1(32);
#undef SMG_CA1
        count_launch(ctx);
        SMG_CHECK_LAUNCH(ctx);
        return SMG_OK;
    }
    // several right-hand sides: stage link and vector blocks in shared memory
    if (x.nrhs >= 8) {
        if (L.ndof == 8) return coarse_apply_tiled<T, 8>(ctx, L, Ap<T>(L), x, y, epi, w, out, gate);
        if (L.ndof == 16) return coarse_apply_tiled<T, 16>(ctx, L, Ap<T>(L), x, y, epi, w, out, gate);
        if (L.ndof == 32) return coarse_apply_tiled<T, 32>(ctx, L, Ap<T>(L), x, y, epi, w, out, gate);
    }
    ReduceLaunch rl = reduce_launch((int)((int64_t)L.nsites * L.ndof), x.nrhs);
    SMG_TRY(smg_reduce_reserve(ctx, (size_t)rl.grid.x * x.nrhs * 3));
    if (epi == 0) {
        k_coarse_apply<T, 0><<<rl.grid, rl.block, 0, ctx->stream>>>(Ap<T>(L), x, y, L.nx, L.ny, w, nullptr, nullptr,
                                                                  nullptr, gate);
    } else if (epi == 1) {
        k_coarse_apply<T, 1><<<rl.grid, rl.block, 0, ctx->stream>>>(Ap<T>(L), x, y, L.nx, L.ny, w, ctx->red.partials,
                                                                  ctx->red.tickets, out, gate);
    } else {
        k_coarse_apply<T, 2><<<rl.grid, rl.block, 0, ctx->stream>>>(Ap<T>(L), x, y, L.nx, L.ny, w, ctx->red.partials,
                                                                  ctx->red.tickets, out, gate);
    }
    count_launch(ctx);
    SMG_CHECK_LAUNCH(ctx);
    return SMG_OK;
}

// A_l x -> y for any level; level 0 is D^dag D via the fine temp field
template <typename T>
smg_status level_apply_fine(smg_mg* mg, smg_field* x, smg_field* y, const smg_field* w, double* out3) {
    SMG_TRY(smg_dslash(mg->dirac, false, x, mg->f_t, nullptr));
    if (w && x->nrhs < 4) return smg_dslash_mr(mg->dirac, true, mg->f_t, y, w, out3);
    SMG_TRY(smg_dslash(mg->dirac, true, mg->f_t, y, nullptr));
    // several RHS: the one-item-per-thread stencil plus a streaming <y, w>, ||y||^2 pass beats the
    // stencil with the reduction fused into its grid-stride loop
    if (w) return vreduce<T>(mg->ctx, fview<T>(y), (const cx<T>*)w->data, VR_DOTNORM, out3);
    return SMG_OK;
}

// scalar area layout: per level 16 * nrhs doubles (MR: 3, CG: rr, pap3, bnorm2, beta, ints)
double* lvl_scal(smg_mg* mg, int l) { return mg->scal + (size_t)l * 16 * mg->work_nrhs + 64; }

smg_status free_work(smg_mg* mg) {
    if (mg->f_rs.empty()) smg_field_destroy(mg->f_r);  // else f_r is f_rs[0]
    for (smg_field* f : mg->f_rs) smg_field_destroy(f);
    mg->f_rs.clear();
    mg->f_res = nullptr;
    smg_field_destroy(mg->f_Ar);
    smg_field_destroy(mg->f_t);
    mg->f_r = mg->f_Ar = mg->f_t = nullptr;
    if (mg->hdots) cudaFree(mg->hdots);
    mg->hdots = nullptr;
    if (mg->mr_om) cudaFree(mg->mr_om);
    mg->mr_om = nullptr;
    if (mg->mr_omf) cudaFree(mg->mr_omf);
    mg->mr_omf = nullptr;
    for (auto& w : mg->cw) {
        for (void* p : {w.b, w.x, w.r, w.Ar, w.e, w.p, w.rh, w.ph, (void*)w.rs, (void*)w.ps, w.ph2, (void*)w.ps2,
                        (void*)w.ccg_part, w.ar16, (void*)w.ar16s, (void*)w.mr16_sc, (void*)w.mr16_om})
            if (p) cudaFree(p);
        for (void* p : w.r16) cudaFree(p);
        for (float* p : w.r16s) cudaFree(p);
    }
    mg->cw.clear();
    if (mg->scal) cudaFree(mg->scal);
    mg->scal = nullptr;
    if (mg->cg_state) cudaFree(mg->cg_state);
    mg->cg_state = nullptr;
    mg->work_nrhs = 0;
    return SMG_OK;
}

template <typename T, int NC>
smg_status coarse_cg_persistent(smg_mg* mg, int l, void* x, const void* b) {
    smg_context* ctx = mg->ctx;
    const Level& L = mg->lv[l];
    CoarseWork& w = mg->cw[l];
    static int blocks_per_sm = -1;  // per template instance
    if (blocks_per_sm < 0) {
        int nb = 0;
        SMG_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_coarse_cg1<T, NC>, 256, 0));
        blocks_per_sm = nb;
    }
    const int n = L.nsites * NC;
    int grid = blocks_per_sm * ctx->num_sms;
    const int need = (n + 255) / 256;
    if (grid > need) grid = need;
    if (grid > kMaxReduceBlocks) grid = kMaxReduceBlocks;
    if (grid < 1) return smg_fail(ctx, SMG_UNSUPPORTED, "coarsest CG kernel cannot be resident");
    CoarseCgArgs a;
    a.A = Ap<T>(L);
    a.b = b;
    a.x = x;
    a.r = w.r;
    a.p = w.p;
    a.Ap = w.Ar;
    a.nx = L.nx;
    a.ny = L.ny;
    a.nsites = L.nsites;
    a.max_iter = mg->p.coarse_max_iter;
    a.tol2 = mg->p.coarse_tol * mg->p.coarse_tol;
    char* st = static_cast<char*>(mg->cg_state);
    a.bar = reinterpret_cast<unsigned int*>(st);
    a.err = reinterpret_cast<int*>(st) + 2;
    a.iters = reinterpret_cast<int*>(st) + 3;
    a.part = reinterpret_cast<double*>(st + 256);
    a.spin_limit = mg->spin_limit;
    // barrier words back to zero; a raised error flag stays raised until read
    SMG_CUDA(ctx, cudaMemsetAsync(st, 0, 2 * sizeof(unsigned int), ctx->stream));
    void* args[] = {&a};
    SMG_CUDA(ctx, cudaLaunchCooperativeKernel((const void*)k_coarse_cg1<T, NC>, dim3(grid), dim3(256), args, 0,
                                              ctx->stream));
    count_launch(ctx);
    return SMG_OK;
}

// the fine smoother's work vectors are FP16 for F32 cycles of hierarchies that ask for it, when the
// right-hand sides fit the FP16 writers (power-of-two lane groups) and the aggregate restriction
// the coarsest level keeps its CG vectors in FP16 (coarse_half) on the tensor-core path with 32
// right-hand sides (one site-block of 16 dofs x 16 right-hand-side pairs per CTA in the update kernels)
bool coarse_half_level(const smg_mg* mg, int l, int nrhs, smg_precision prec) {
    return mg->p.coarse_half && prec == SMG_F32 && l == (int)mg->lv.size() - 1 && nrhs == 32 &&
           mg->lv[l].ndof == 16 && tc_path(mg, l, nrhs);
}

// an intermediate level of a coarse_half hierarchy smooths with MR on FP16 vectors (the tensor-core
// apply reading and writing them) when its smoother is MR and the cycle has 32 right-hand sides
bool mr16_level(const smg_mg* mg, int l, int nrhs, smg_precision prec) {
    return mg->p.coarse_half && prec == SMG_F32 && l >= 1 && l < (int)mg->lv.size() - 1 && nrhs == 32 &&
           mg->lv[l].ndof == 16 && tc_path(mg, l, nrhs) && !(mg->lv[l].rich_omega > 0) &&
           std::max(mg->p.pre_smooth, mg->p.post_smooth) <= kC16MaxSteps;
}

// the coarsest CG of a coarse_half level runs as one persistent cooperative launch (k_ccg_tc) when the
// hierarchy is not batched next to other streams (its CTAs must be co-resident) and the launch shape
// fits the GPU; SMG_CCG_PERSISTENT=0 keeps the per-iteration kernels
bool ccg_tc_level(const smg_mg* mg, int l) {
    static const bool on = [] {
        const char* e = std::getenv("SMG_CCG_PERSISTENT");
        return !(e && std::atoi(e) == 0);
    }();
    const Level& L = mg->lv[l];
    return on && mg->persistent && smg_coarse_cg_tc_rows(mg->ctx, L.nx, L.ny) > 0;
}

bool half_smoother(const smg_mg* mg, int nrhs, smg_precision prec) {
    const int nc = mg->lv[0].nc_next;
    return mg->p.smoother_half && prec == SMG_F32 && nrhs >= 8 && f16_nrhs_ok(nrhs) &&
           (nc == 8 || nc == 16 || nc == 32);
}

smg_status ensure_work(smg_mg* mg, int nrhs, smg_precision prec) {
    if (mg->work_nrhs == nrhs && mg->work_prec == prec && mg->f_t) return SMG_OK;
    smg_context* ctx = mg->ctx;
    SMG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    free_work(mg);
    const int L = mg->lv[0].nx;
    const smg_precision wp = half_smoother(mg, nrhs, prec) ? SMG_F16 : prec;
    if (wp == SMG_F16) {
        const int nsteps = std::max(1, std::max(mg->p.pre_smooth, mg->p.post_smooth));
        mg->f_rs.assign(nsteps + 1, nullptr);
        for (auto& f : mg->f_rs) SMG_TRY(smg_field_create(ctx, L, nrhs, wp, &f));
        mg->f_r = mg->f_rs[0];
        SMG_CUDA(ctx, cudaMalloc(&mg->hdots, (size_t)smg_dslash_h_blocks(L, nrhs) * nrhs * 2 * sizeof(float)));
        SMG_CUDA(ctx, cudaMalloc(&mg->mr_om, (size_t)nsteps * 3 * nrhs * sizeof(double)));
        SMG_CUDA(ctx, cudaMemsetAsync(mg->mr_om, 0, (size_t)nsteps * 3 * nrhs * sizeof(double), ctx->stream));
        SMG_CUDA(ctx, cudaMalloc(&mg->mr_omf, (size_t)nsteps * nrhs * sizeof(float2)));
        SMG_CUDA(ctx, cudaMemsetAsync(mg->mr_omf, 0, (size_t)nsteps * nrhs * sizeof(float2), ctx->stream));
        SMG_TRY(smg_reduce_reserve(ctx, smg_dslash_h_dots_scratch(L, nrhs)));  // before any capture
    } else {
        SMG_TRY(smg_field_create(ctx, L, nrhs, wp, &mg->f_r));
    }
    SMG_TRY(smg_field_create(ctx, L, nrhs, wp, &mg->f_Ar));
    SMG_TRY(smg_field_create(ctx, L, nrhs, wp, &mg->f_t));
    size_t es = prec == SMG_F64 ? sizeof(cx<double>) : sizeof(cx<float>);
    mg->cw.resize(mg->lv.size());
    for (size_t l = 1; l < mg->lv.size(); ++l) {
        size_t bytes = (size_t)mg->lv[l].nsites * nrhs * mg->lv[l].ndof * es;
        CoarseWork& w = mg->cw[l];
        for (void** p : {&w.b, &w.x, &w.r, &w.Ar, &w.e, &w.p}) {
            SMG_CUDA(ctx, cudaMalloc(p, bytes));
            SMG_CUDA(ctx, cudaMemsetAsync(*p, 0, bytes, ctx->stream));
        }
        if (coarse_half_level(mg, (int)l, nrhs, prec)) {
            const size_t hb = (size_t)mg->lv[l].nsites * nrhs * mg->lv[l].ndof * sizeof(__half2);
            // one scale per site (per-iteration kernels) or per site and half of the 32 rhs (k_ccg_tc)
            const size_t sb = (size_t)mg->lv[l].nsites * 2 * sizeof(float);
            SMG_CUDA(ctx, cudaMalloc(&w.rh, hb));
            SMG_CUDA(ctx, cudaMalloc(&w.ph, hb));
            SMG_CUDA(ctx, cudaMalloc((void**)&w.rs, sb));
            SMG_CUDA(ctx, cudaMalloc((void**)&w.ps, sb));
            SMG_CUDA(ctx, cudaMemsetAsync(w.rs, 0, sb, ctx->stream));
            SMG_CUDA(ctx, cudaMemsetAsync(w.ps, 0, sb, ctx->stream));
            if (ccg_tc_level(mg, (int)l)) {
                SMG_CUDA(ctx, cudaMalloc(&w.ph2, hb));
                SMG_CUDA(ctx, cudaMalloc((void**)&w.ps2, sb));
                const Level& Lc = mg->lv[l];
                const size_t nblk = (size_t)(Lc.nx / 8) * (Lc.ny / smg_coarse_cg_tc_rows(ctx, Lc.nx, Lc.ny));
                SMG_CUDA(ctx, cudaMalloc((void**)&w.ccg_part, 64 * nblk * sizeof(double)));
            }
        }
        if (mr16_level(mg, (int)l, nrhs, prec)) {
            const size_t hb = (size_t)mg->lv[l].nsites * nrhs * mg->lv[l].ndof * sizeof(__half2);
            const size_t sb = (size_t)mg->lv[l].nsites * 2 * sizeof(float);
            const int nsteps = std::max(1, std::max(mg->p.pre_smooth, mg->p.post_smooth));
            w.r16.assign(nsteps + 1, nullptr);
            w.r16s.assign(nsteps + 1, nullptr);
            for (int k = 0; k <= nsteps; ++k) {
                SMG_CUDA(ctx, cudaMalloc(&w.r16[k], hb));
                SMG_CUDA(ctx, cudaMalloc((void**)&w.r16s[k], sb));
            }
            SMG_CUDA(ctx, cudaMalloc(&w.ar16, hb));
            SMG_CUDA(ctx, cudaMalloc((void**)&w.ar16s, sb));
            SMG_CUDA(ctx, cudaMalloc((void**)&w.mr16_sc, (size_t)nsteps * nrhs * 3 * sizeof(double)));
            SMG_CUDA(ctx, cudaMalloc((void**)&w.mr16_om, (size_t)nsteps * nrhs * sizeof(float2)));
        }
    }
    if (!mg->cg_state) {
        SMG_CUDA(ctx, cudaMalloc(&mg->cg_state, 256 + 2 * kMaxReduceBlocks * sizeof(double)));
        SMG_CUDA(ctx, cudaMemsetAsync(mg->cg_state, 0, 256, ctx->stream));
    }
    mg->scal_doubles = (size_t)mg->lv.size() * 16 * nrhs + 128;
    SMG_CUDA(ctx, cudaMalloc(&mg->scal, mg->scal_doubles * sizeof(double)));
    SMG_CUDA(ctx, cudaMemsetAsync(mg->scal, 0, mg->scal_doubles * sizeof(double), ctx->stream));
    mg->work_nrhs = nrhs;
    mg->work_prec = prec;
    mg->work_gen++;
    // launch shape of the tensor-core coarse applies, timed once per lattice and nrhs
    if (prec == SMG_F32)
        for (size_t l = 1; l < mg->lv.size(); ++l)
            if (tc_path(mg, (int)l, nrhs))
                SMG_TRY(smg_coarse_tc_tune(ctx, mg->lv[l].Atc, mg->lv[l].nx, mg->lv[l].ny, nrhs,
                                           (const cx<float>*)mg->cw[l].x, (cx<float>*)mg->cw[l].Ar));
    return SMG_OK;
}

// ------------------------------------------------------------ MR smoothers

// ------------------------------------------------------------ FP16 smoother work vectors
//
// One thread per (fine site, pair of right-hand sides rhs and rhs + lanes); a block is
// (lanes = nrhs / 2, 256 / lanes sites), so the threads of a site are one lane group of a warp
// (FP16 writers reduce the site scale across it).

// r16 = b - Ax (Ax16 optional: r16 = b)
__global__ void __launch_bounds__(256) k_sub_h(const cx<float>* __restrict__ b, const __half2* __restrict__ ax,
                                               const float* __restrict__ axs, __half2* __restrict__ r,
                                               float* __restrict__ rs, int nsites, int nrhs) {
    const int lanes = blockDim.x, rhs = threadIdx.x;
    const int s = blockIdx.x * blockDim.y + threadIdx.y;
    const bool valid = s < nsites;
    Spinor<float> v[2];
#pragma unroll
    for (int k = 0; k < 2; ++k) {
        v[k].s0 = mk(0.f, 0.f);
        v[k].s1 = mk(0.f, 0.f);
        if (valid) {
            v[k] = ld_spinor(b, s, rhs + k * lanes, nrhs);
            if (ax) {
                const Spinor<float> a = ld_spinor_h(ax, axs, s, rhs + k * lanes, nrhs);
                v[k].s0 = v[k].s0 - a.s0;
                v[k].s1 = v[k].s1 - a.s1;
            }
        }
    }
    st_spinor2_h(r, rs, s, rhs, nrhs, lanes, v[0], v[1], valid);
}

// The MR steps of the FP16 smoother keep every residual r_0 .. r_n (a ring of FP16 fields) and
// leave x alone until the end, where one pass adds sum_k omega_k r_k: the FP32 x is read and
// written once per smoothing instead of once per step.  omega_k per rhs is the step's MR value,
// ||D r||^2 / ||A r||^2 as the norm-finishing kernel stored it, or a fixed Richardson omega.
constexpr int kMaxMrSteps = 16;  // residuals one x pass combines

// r_out = r_in - omega A r (FP16 fields); a thread owns one pair of adjacent right-hand sides
__global__ void __launch_bounds__(256) k_mr_rupdate_h(const __half2* __restrict__ r, const float* __restrict__ rs,
                                                      const __half2* __restrict__ ar, const float* __restrict__ ars,
                                                      __half2* __restrict__ ro, float* __restrict__ ros,
                                                      const float2* __restrict__ om, float omega, int nsites,
                                                      int nrhs) {
    const int lanes = blockDim.x, rhs0 = 2 * threadIdx.x;
    const int s = blockIdx.x * blockDim.y + threadIdx.y;
    const bool valid = s < nsites;
    Spinor<float> rn[2];
    rn[0].s0 = rn[0].s1 = rn[1].s0 = rn[1].s1 = mk(0.f, 0.f);
    if (valid) {
        Spinor<float> rv[2], av[2];
        ld_pairs_h<1>(r, s, rhs0, nrhs, rv);
        ld_pairs_h<1>(ar, s, rhs0, nrhs, av);
        const float sr = rs[s], sa = ars[s];
        const float4 o = om ? __ldg(reinterpret_cast<const float4*>(om + rhs0)) : make_float4(omega, 0.f, omega, 0.f);
#pragma unroll
        for (int k = 0; k < 2; ++k) {
            const cx<float> oa = k == 0 ? mk(o.x * sa, o.y * sa) : mk(o.z * sa, o.w * sa);
            rn[k].s0 = sr * rv[k].s0 - oa * av[k].s0;
            rn[k].s1 = sr * rv[k].s1 - oa * av[k].s1;
        }
    }
    st_pairs_h<1>(ro, ros, s, rhs0, nrhs, lanes, rn, valid);
}

struct ResidualRing {
    const __half2* r[kMaxMrSteps];
    const float* s[kMaxMrSteps];
};

// x = (x_zero ? 0 : x) + sum_{k < n} omega_k r_k, omega_k = om[k * nrhs + rhs] or fixed
__global__ void __launch_bounds__(256) k_mr_xupdate_h(cx<float>* __restrict__ x, ResidualRing ring, int n,
                                                      const float2* __restrict__ om, float omega, int x_zero,
                                                      int nsites, int nrhs) {
    const int rhs0 = 2 * threadIdx.x;
    const int s = blockIdx.x * blockDim.y + threadIdx.y;
    if (s >= nsites) return;
    Spinor<float> xv[2];
    if (x_zero) {
        xv[0].s0 = xv[0].s1 = xv[1].s0 = xv[1].s1 = mk(0.f, 0.f);
    } else {
        ld_pairs_f<1>(x, s, rhs0, nrhs, xv);
    }
    for (int k = 0; k < n; ++k) {
        Spinor<float> rv[2];
        ld_pairs_h<1>(ring.r[k], s, rhs0, nrhs, rv);
        const float sr = ring.s[k][s];
        const float4 o =
            om ? __ldg(reinterpret_cast<const float4*>(om + (size_t)k * nrhs + rhs0)) : make_float4(omega, 0.f, omega, 0.f);
#pragma unroll
        for (int j = 0; j < 2; ++j) {
            const cx<float> os = j == 0 ? mk(o.x * sr, o.y * sr) : mk(o.z * sr, o.w * sr);
            xv[j].s0 = xv[j].s0 + os * rv[j].s0;
            xv[j].s1 = xv[j].s1 + os * rv[j].s1;
        }
    }
    float4* px = reinterpret_cast<float4*>(x) + ((int64_t)s * nrhs + rhs0);
    px[0] = make_float4(xv[0].s0.re, xv[0].s0.im, xv[0].s1.re, xv[0].s1.im);
    px[1] = make_float4(xv[1].s0.re, xv[1].s0.im, xv[1].s1.re, xv[1].s1.im);
}

// asynchronous global -> shared copies (no registers held while in flight)
__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async8(void* smem, const void* gmem) {
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

// Packed FP32 pairs for the level-0 transfers: fma.rn.f32x2 does two independent FP32 FMAs in one
// instruction, so a complex multiply-add costs two instructions instead of four.  A pair is a
// 64-bit register (low half first).
using f32x2 = unsigned long long;
__device__ __forceinline__ f32x2 f2_pack(float lo, float hi) {
    f32x2 r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(lo), "f"(hi));
    return r;
}
__device__ __forceinline__ float2 f2_unpack(f32x2 v) {
    float2 r;
    asm("mov.b64 {%0, %1}, %2;" : "=f"(r.x), "=f"(r.y) : "l"(v));
    return r;
}
__device__ __forceinline__ f32x2 f2_fma(f32x2 a, f32x2 b, f32x2 c) {
    f32x2 d;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
    return d;
}

// The level-0 transfers of the FP16 smoother for aggregates of 4 x 4 sites and tiles of 32
// right-hand sides (lane = rhs).  The block vectors of an aggregate are V[e][i], e = 2 loc + spin,
// i < NC, as the generic transfer kernels read them.
constexpr int kAggSites0 = 16;

// Restriction out_i = sum_e conj(V[e][i]) r_e of an FP16 residual with per-site scales (the
// generic kernel with the InHalf reader, k_restrict_agg): one warp per aggregate, the lane's 16
// two-spinors in registers, the warp's block vectors staged in shared memory as output pairs
// [e][i/2] = (Re V[e][i], Re V[e][i+1], Im V[e][i], Im V[e][i+1]) so that one broadcast 16-byte read
// feeds four packed FMAs.  FUSED restricts r - omega A r of the last MR step, formed from that step's
// FP16 r and A r (scales per site, omega per rhs) in place of the stored r_n.
template <int NC, bool FUSED>
__global__ void __launch_bounds__(128) k_restrict0_h(const cx<float>* __restrict__ V, const __half2* __restrict__ r,
                                                     const float* __restrict__ rs, cx<float>* __restrict__ out,
                                                     TransferGeom t, int nagg, const __half2* __restrict__ ar,
                                                     const float* __restrict__ ars, const float2* __restrict__ om,
                                                     float omega) {
    constexpr int ne = 2 * kAggSites0, NP = NC / 2;
    __shared__ float4 s_v[4][ne * NP];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int B = blockIdx.x * 4 + w;
    if (B >= nagg) return;  // whole warps; the kernel has no block barrier
    const int nrhs = t.nrhs, rhs = blockIdx.y * 32 + lane;
    const int x0 = (B % t.nax) * 4, y0 = (B / t.nax) * 4;
    const int myq = site_q(t.g, x0 + (lane & 3), y0 + ((lane >> 2) & 3));  // lanes 16..31 repeat 0..15
    const float mys = __ldg(rs + myq);
    // FUSED: the input is the last MR step's r - omega A r, formed here from r and A r (the step's
    // k_mr_rupdate_h, whose output only this restriction would read)
    const float mya = FUSED ? __ldg(ars + myq) : 0.f;
    const float2 o = FUSED ? (om ? __ldg(om + rhs) : make_float2(omega, 0.f)) : make_float2(0.f, 0.f);
    uint2 raw[kAggSites0], rawa[FUSED ? kAggSites0 : 1];
#pragma unroll
    for (int s = 0; s < kAggSites0; ++s) {
        const int q = __shfl_sync(0xffffffffu, myq, s);
        raw[s] = __ldg(reinterpret_cast<const uint2*>(r) + ((int64_t)q * nrhs + rhs));
        if constexpr (FUSED) rawa[s] = __ldg(reinterpret_cast<const uint2*>(ar) + ((int64_t)q * nrhs + rhs));
    }
    // float4 k of the aggregate's block vectors holds V entries 2k, 2k+1 = (e, i), (e, i + 1), i even
    const float4* __restrict__ Vb = reinterpret_cast<const float4*>(V + (int64_t)B * ne * NC);
#pragma unroll
    for (int k = lane; k < ne * NP; k += 32) {
        const float4 a = __ldg(Vb + k);
        s_v[w][k] = make_float4(a.x, a.z, a.y, a.w);
    }
    __syncwarp();
    f32x2 accr[NP], acci[NP];  // (Re out_i, Re out_i+1), (Im out_i, Im out_i+1)
#pragma unroll
    for (int p = 0; p < NP; ++p) accr[p] = acci[p] = 0ull;
#pragma unroll
    for (int s = 0; s < kAggSites0; ++s) {
        const float sc = __shfl_sync(0xffffffffu, mys, s);
        const float2 f0 = __half22float2(*reinterpret_cast<const __half2*>(&raw[s].x));
        const float2 f1 = __half22float2(*reinterpret_cast<const __half2*>(&raw[s].y));
        float oar = 0.f, oai = 0.f;
        float2 a0 = make_float2(0.f, 0.f), a1 = make_float2(0.f, 0.f);
        if constexpr (FUSED) {
            const float sa = __shfl_sync(0xffffffffu, mya, s);
            oar = o.x * sa;
            oai = o.y * sa;
            a0 = __half22float2(*reinterpret_cast<const __half2*>(&rawa[s].x));
            a1 = __half22float2(*reinterpret_cast<const __half2*>(&rawa[s].y));
        }
#pragma unroll
        for (int j = 0; j < 2; ++j) {
            float fr = (j ? f1.x : f0.x) * sc, fi = (j ? f1.y : f0.y) * sc;
            if constexpr (FUSED) {  // r - (omega s_a) A r, as k_mr_rupdate_h forms it
                const float2 a = j ? a1 : a0;
                fr -= oar * a.x - oai * a.y;
                fi -= oar * a.y + oai * a.x;
            }
            const f32x2 FR = f2_pack(fr, fr), FI = f2_pack(fi, fi), FRn = f2_pack(-fr, -fr);
            const float4* __restrict__ vrow = &s_v[w][(2 * s + j) * NP];
#pragma unroll
            for (int p = 0; p < NP; ++p) {
                const float4 v = vrow[p];
                const f32x2 VR = f2_pack(v.x, v.y), VI = f2_pack(v.z, v.w);
                accr[p] = f2_fma(VR, FR, accr[p]);  // Re conj(v) f = Re v Re f + Im v Im f
                accr[p] = f2_fma(VI, FI, accr[p]);
                acci[p] = f2_fma(VR, FI, acci[p]);  // Im conj(v) f = Re v Im f - Im v Re f
                acci[p] = f2_fma(VI, FRn, acci[p]);
            }
        }
    }
#pragma unroll
    for (int p = 0; p < NP; ++p) {
        const float2 re = f2_unpack(accr[p]), im = f2_unpack(acci[p]);
        out[((int64_t)B * NC + 2 * p) * nrhs + rhs] = mk(re.x, im.x);
        out[((int64_t)B * NC + 2 * p + 1) * nrhs + rhs] = mk(re.y, im.y);
    }
}

// Prolongation with the pre-smoothing update folded in:
//   x(site, spin) = [x] + sum_{k < n} omega_k r_k + sum_i V[e][i] c_i
// (the generic kernel k_prolong_agg after k_mr_xupdate_h).  One block of four warps per aggregate,
// warp w on the aggregate's row w (four sites); the block vectors staged in shared memory as pairs
// over the two spins of a site, [loc][i] = (Re V[2 loc][i], Re V[2 loc + 1][i], Im V[2 loc][i],
// Im V[2 loc + 1][i]) (the level's V32s copy), the coarse values as [i][lane], and the lane's x
// values held as (Re spin 0, Re spin 1), (Im spin 0, Im spin 1) pairs.  The residuals' loads go
// out kRingChunk at a time.
constexpr int kRingChunk = 4;

template <int NC>
__global__ void __launch_bounds__(128) k_prolong0_ring(const float4* __restrict__ Vs, const cx<float>* __restrict__ cin,
                                                       cx<float>* __restrict__ x, TransferGeom t, ResidualRing ring,
                                                       int n, const float2* __restrict__ om, float omega,
                                                       int accumulate) {
    constexpr int S = 4;
    __shared__ float4 s_v[kAggSites0 * NC];
    __shared__ float2 s_c[NC * 32];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int B = blockIdx.x;
    const int nrhs = t.nrhs, rhs = blockIdx.y * 32 + lane;
    const int myq = site_q(t.g, (B % t.nax) * 4 + (lane & 3), (B / t.nax) * 4 + w);  // lanes repeat mod 4
    // the aggregate's spin-paired block vectors and the tile's coarse values go to shared memory by
    // asynchronous copies that hold no registers while the residuals' loads are in flight
    const float4* __restrict__ vsrc = Vs + (int64_t)B * kAggSites0 * NC;
#pragma unroll
    for (int k = threadIdx.x; k < kAggSites0 * NC; k += 128) cp_async16(&s_v[k], vsrc + k);
    const float2* __restrict__ c2 = reinterpret_cast<const float2*>(cin) + (int64_t)B * NC * nrhs + rhs;
#pragma unroll
    for (int i = w; i < NC; i += 4) cp_async8(&s_c[i * 32 + lane], c2 + (int64_t)i * nrhs);
    int q[S];
#pragma unroll
    for (int s = 0; s < S; ++s) q[s] = __shfl_sync(0xffffffffu, myq, s);
    f32x2 xr[S], xi[S];
    float4* __restrict__ px = reinterpret_cast<float4*>(x);  // one float4 = both spins of (site, rhs)
    if (accumulate) {
#pragma unroll
        for (int s = 0; s < S; ++s) {
            const float4 v = px[(int64_t)q[s] * nrhs + rhs];
            xr[s] = f2_pack(v.x, v.z);
            xi[s] = f2_pack(v.y, v.w);
        }
    } else {
#pragma unroll
        for (int s = 0; s < S; ++s) xr[s] = xi[s] = 0ull;
    }
    for (int k0 = 0; k0 < n; k0 += kRingChunk) {
        uint2 raw[kRingChunk][S];
        float scl[kRingChunk];
        float2 o[kRingChunk];
#pragma unroll
        for (int j = 0; j < kRingChunk; ++j) {
            if (k0 + j < n) {
                const int k = k0 + j;
                o[j] = om ? __ldg(om + (int64_t)k * nrhs + rhs) : make_float2(omega, 0.f);
                scl[j] = __ldg(ring.s[k] + myq);
                const uint2* __restrict__ rk = reinterpret_cast<const uint2*>(ring.r[k]);
#pragma unroll
                for (int s = 0; s < S; ++s) raw[j][s] = __ldg(rk + ((int64_t)q[s] * nrhs + rhs));
            }
        }
#pragma unroll
        for (int j = 0; j < kRingChunk; ++j) {
            if (k0 + j < n) {
#pragma unroll
                for (int s = 0; s < S; ++s) {
                    const float sc = __shfl_sync(0xffffffffu, scl[j], s);
                    const float orr = o[j].x * sc, oi = o[j].y * sc;
                    const float2 a = __half22float2(*reinterpret_cast<const __half2*>(&raw[j][s].x));
                    const float2 b = __half22float2(*reinterpret_cast<const __half2*>(&raw[j][s].y));
                    const f32x2 RR = f2_pack(a.x, b.x), RI = f2_pack(a.y, b.y);
                    // (omega s) r: Re = o_r r_r - o_i r_i, Im = o_r r_i + o_i r_r
                    xr[s] = f2_fma(f2_pack(orr, orr), RR, xr[s]);
                    xr[s] = f2_fma(f2_pack(-oi, -oi), RI, xr[s]);
                    xi[s] = f2_fma(f2_pack(orr, orr), RI, xi[s]);
                    xi[s] = f2_fma(f2_pack(oi, oi), RR, xi[s]);
                }
            }
        }
    }
    cp_async_wait_all();
    __syncthreads();
#pragma unroll
    for (int i = 0; i < NC; ++i) {
        const float2 c = s_c[i * 32 + lane];
        const f32x2 CR = f2_pack(c.x, c.x), CI = f2_pack(c.y, c.y), CIn = f2_pack(-c.y, -c.y);
#pragma unroll
        for (int s = 0; s < S; ++s) {
            const float4 v = s_v[(S * w + s) * NC + i];
            const f32x2 VR = f2_pack(v.x, v.y), VI = f2_pack(v.z, v.w);
            xr[s] = f2_fma(VR, CR, xr[s]);  // Re v c = Re v Re c - Im v Im c
            xr[s] = f2_fma(VI, CIn, xr[s]);
            xi[s] = f2_fma(VR, CI, xi[s]);  // Im v c = Re v Im c + Im v Re c
            xi[s] = f2_fma(VI, CR, xi[s]);
        }
    }
#pragma unroll
    for (int s = 0; s < S; ++s) {
        const float2 re = f2_unpack(xr[s]), im = f2_unpack(xi[s]);
        px[(int64_t)q[s] * nrhs + rhs] = make_float4(re.x, im.x, re.y, im.y);
    }
}

// The transfers of an intermediate FP16 level (coarse_half MR smoother) for 2 x 2 aggregates of
// 16-dof sites and 32 rhs (lane = rhs): vectors [site][dof][32], FP16 residuals with one scale per
// site and rhs half, block vectors V[agg][loc][dof][i].
constexpr int kAggSitesC = 4;

// Restriction out_i = sum_e conj(V[e][i]) r_e of the FP16 residual (the generic kernel with the
// InHalfC reader): one warp per aggregate, the lane's 64 FP16 inputs in registers, the block vectors
// (the level's output-pair copy V32o) staged in shared memory by asynchronous copies.
template <int NC, bool FUSED>
__global__ void __launch_bounds__(NC == 32 ? 64 : 128) k_restrict_c16p(const float4* __restrict__ Vo,
                                                                       const __half2* __restrict__ r,
                                                                       const float* __restrict__ rs,
                                                                       cx<float>* __restrict__ out, TransferGeom t,
                                                                       int nagg, const __half2* __restrict__ ar,
                                                                       const float* __restrict__ ars,
                                                                       const float2* __restrict__ om) {
    constexpr int WPB = NC == 32 ? 2 : 4, NE = kAggSitesC * kC16Dofs, NP = NC / 2;
    __shared__ float4 s_v[WPB][NE * NP];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int B = blockIdx.x * WPB + w;
    if (B >= nagg) return;  // whole warps; the kernel has no block barrier
    const float4* __restrict__ src = Vo + (int64_t)B * NE * NP;
#pragma unroll 4
    for (int k = lane; k < NE * NP; k += 32) cp_async16(&s_v[w][k], src + k);
    const int bx = (B % t.nax) * 2, by = (B / t.nax) * 2;
    // FUSED: the input is the last MR step's r - omega A r (k_c16_rupdate's arithmetic), formed here
    __half2 raw[kAggSitesC][kC16Dofs], rawa[FUSED ? kAggSitesC : 1][FUSED ? kC16Dofs : 1];
    float sc[kAggSitesC], sca[kAggSitesC];
    const float2 o = FUSED ? __ldg(om + lane) : make_float2(0.f, 0.f);
#pragma unroll
    for (int l = 0; l < kAggSitesC; ++l) {
        const int64_t site = (int64_t)(bx + (l & 1)) + (int64_t)t.nx * (by + (l >> 1));
        sc[l] = __ldg(rs + 2 * site + (lane >> 4));
        sca[l] = FUSED ? __ldg(ars + 2 * site + (lane >> 4)) : 0.f;
        const __half2* __restrict__ rp = r + site * kC16Dofs * 32 + lane;
#pragma unroll
        for (int d = 0; d < kC16Dofs; ++d) raw[l][d] = rp[d * 32];
        if constexpr (FUSED) {
            const __half2* __restrict__ ap = ar + site * kC16Dofs * 32 + lane;
#pragma unroll
            for (int d = 0; d < kC16Dofs; ++d) rawa[l][d] = ap[d * 32];
        }
    }
    cp_async_wait_all();
    __syncwarp();
    f32x2 accr[NP], acci[NP];  // (Re out_i, Re out_i+1), (Im out_i, Im out_i+1)
#pragma unroll
    for (int p = 0; p < NP; ++p) accr[p] = acci[p] = 0ull;
#pragma unroll
    for (int l = 0; l < kAggSitesC; ++l) {
#pragma unroll
        for (int d = 0; d < kC16Dofs; ++d) {
            const float2 f = __half22float2(raw[l][d]);
            float fr = f.x * sc[l], fi = f.y * sc[l];
            if constexpr (FUSED) {
                const float2 y = __half22float2(rawa[l][d]);
                const float yr = sca[l] * y.x, yi = sca[l] * y.y;
                fr -= o.x * yr - o.y * yi;
                fi -= o.x * yi + o.y * yr;
            }
            const f32x2 FR = f2_pack(fr, fr), FI = f2_pack(fi, fi), FRn = f2_pack(-fr, -fr);
            const float4* __restrict__ vrow = &s_v[w][(l * kC16Dofs + d) * NP];
#pragma unroll
            for (int p = 0; p < NP; ++p) {
                const float4 v = vrow[p];
                const f32x2 VR = f2_pack(v.x, v.y), VI = f2_pack(v.z, v.w);
                accr[p] = f2_fma(VR, FR, accr[p]);
                accr[p] = f2_fma(VI, FI, accr[p]);
                acci[p] = f2_fma(VR, FI, acci[p]);
                acci[p] = f2_fma(VI, FRn, acci[p]);
            }
        }
    }
#pragma unroll
    for (int p = 0; p < NP; ++p) {
        const float2 re = f2_unpack(accr[p]), im = f2_unpack(acci[p]);
        out[((int64_t)B * NC + 2 * p) * 32 + lane] = mk(re.x, im.x);
        out[((int64_t)B * NC + 2 * p + 1) * 32 + lane] = mk(re.y, im.y);
    }
}

// Prolongation into an intermediate FP16 level with its pre-smoothing x pass folded in:
//   x(site, dof) = [x] + sum_{k < n} omega_k r_k + sum_i V[loc][dof][i] c_i
// (k_prolong_agg after k_c16_xupdate).  One block of eight warps per aggregate, warp w on site w / 2
// and dofs 8 (w % 2) .. + 7; the block vectors (the level's dof-paired copy V32s) and the coarse
// values staged by asynchronous copies; the lane's x values held as pairs over dofs (2d, 2d + 1).
template <int NC>
__global__ void __launch_bounds__(256) k_prolong_c16p(const float4* __restrict__ Vs, const cx<float>* __restrict__ cin,
                                                      cx<float>* __restrict__ x, TransferGeom t, C16Ring ring, int n,
                                                      const float2* __restrict__ om, int accumulate) {
    constexpr int DP = 4;  // dof pairs per warp
    __shared__ float4 s_v[kAggSitesC * (kC16Dofs / 2) * NC];
    __shared__ float2 s_c[NC * 32];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int B = blockIdx.x, loc = w >> 1, dh = w & 1;
    const float4* __restrict__ vsrc = Vs + (int64_t)B * kAggSitesC * (kC16Dofs / 2) * NC;
#pragma unroll
    for (int k = threadIdx.x; k < kAggSitesC * (kC16Dofs / 2) * NC; k += 256) cp_async16(&s_v[k], vsrc + k);
    const float2* __restrict__ c2 = reinterpret_cast<const float2*>(cin) + (int64_t)B * NC * 32;
#pragma unroll
    for (int k = threadIdx.x; k < NC * 32; k += 256) cp_async8(&s_c[k], c2 + k);
    const int64_t site = (int64_t)((B % t.nax) * 2 + (loc & 1)) + (int64_t)t.nx * ((B / t.nax) * 2 + (loc >> 1));
    const int64_t row0 = site * kC16Dofs + 8 * dh;  // first (site, dof) row of the warp
    f32x2 xr[DP], xi[DP];
    float2* __restrict__ px = reinterpret_cast<float2*>(x);
    if (accumulate) {
#pragma unroll
        for (int p = 0; p < DP; ++p) {
            const float2 a = px[(row0 + 2 * p) * 32 + lane], b = px[(row0 + 2 * p + 1) * 32 + lane];
            xr[p] = f2_pack(a.x, b.x);
            xi[p] = f2_pack(a.y, b.y);
        }
    } else {
#pragma unroll
        for (int p = 0; p < DP; ++p) xr[p] = xi[p] = 0ull;
    }
#pragma unroll
    for (int k0 = 0; k0 < kC16MaxSteps; k0 += kRingChunk) {  // compile-time ring indices
        if (k0 >= n) break;
        __half2 raw[kRingChunk][2 * DP];
        float scl[kRingChunk];
        float2 o[kRingChunk];
#pragma unroll
        for (int j = 0; j < kRingChunk; ++j) {
            if (k0 + j < n) {
                const int k = k0 + j;
                o[j] = __ldg(om + k * 32 + lane);
                scl[j] = __ldg(ring.s[k] + 2 * site + (lane >> 4));
                const __half2* __restrict__ rk = ring.r[k] + row0 * 32 + lane;
#pragma unroll
                for (int d = 0; d < 2 * DP; ++d) raw[j][d] = rk[d * 32];
            }
        }
#pragma unroll
        for (int j = 0; j < kRingChunk; ++j) {
            if (k0 + j < n) {
                const float wr = o[j].x * scl[j], wi = o[j].y * scl[j];
                const f32x2 WR = f2_pack(wr, wr), WI = f2_pack(wi, wi), WIn = f2_pack(-wi, -wi);
#pragma unroll
                for (int p = 0; p < DP; ++p) {
                    const float2 a = __half22float2(raw[j][2 * p]), b = __half22float2(raw[j][2 * p + 1]);
                    const f32x2 RR = f2_pack(a.x, b.x), RI = f2_pack(a.y, b.y);
                    xr[p] = f2_fma(WR, RR, xr[p]);  // Re (w r) = w_r r_r - w_i r_i
                    xr[p] = f2_fma(WIn, RI, xr[p]);
                    xi[p] = f2_fma(WR, RI, xi[p]);  // Im (w r) = w_r r_i + w_i r_r
                    xi[p] = f2_fma(WI, RR, xi[p]);
                }
            }
        }
    }
    cp_async_wait_all();
    __syncthreads();
    const float4* __restrict__ vw = s_v + (loc * (kC16Dofs / 2) + DP * dh) * NC;
#pragma unroll
    for (int i = 0; i < NC; ++i) {
        const float2 c = s_c[i * 32 + lane];
        const f32x2 CR = f2_pack(c.x, c.x), CI = f2_pack(c.y, c.y), CIn = f2_pack(-c.y, -c.y);
#pragma unroll
        for (int p = 0; p < DP; ++p) {
            const float4 v = vw[p * NC + i];
            const f32x2 VR = f2_pack(v.x, v.y), VI = f2_pack(v.z, v.w);
            xr[p] = f2_fma(VR, CR, xr[p]);
            xr[p] = f2_fma(VI, CIn, xr[p]);
            xi[p] = f2_fma(VR, CI, xi[p]);
            xi[p] = f2_fma(VI, CR, xi[p]);
        }
    }
#pragma unroll
    for (int p = 0; p < DP; ++p) {
        const float2 re = f2_unpack(xr[p]), im = f2_unpack(xi[p]);
        px[(row0 + 2 * p) * 32 + lane] = make_float2(re.x, im.x);
        px[(row0 + 2 * p + 1) * 32 + lane] = make_float2(re.y, im.y);
    }
}

// launch shape of the pair kernels: (nrhs / 2 lanes, 256 / lanes sites)
dim3 pair_block(int nrhs) { return dim3(nrhs / 2, 512 / nrhs); }
dim3 pair_grid(int nsites, int nrhs) { return dim3((nsites + 512 / nrhs - 1) / (512 / nrhs)); }

smg_status mr_xupdate_h(smg_mg* mg, smg_field* x, int first, int n, bool x_zero, double omega) {
    smg_context* ctx = mg->ctx;
    const int V = x->g.V, nrhs = x->nrhs;
    if (n == 0) {
        if (x_zero) SMG_CUDA(ctx, cudaMemsetAsync(x->data, 0, x->bytes, ctx->stream));
        return SMG_OK;
    }
    ResidualRing ring{};
    for (int k = 0; k < n; ++k) {
        ring.r[k] = (const __half2*)mg->f_rs[first + k]->data;
        ring.s[k] = mg->f_rs[first + k]->scale;
    }
    const float2* om = omega > 0 ? nullptr : mg->mr_omf + (size_t)first * nrhs;
    k_mr_xupdate_h<<<pair_grid(V, nrhs), pair_block(nrhs), 0, ctx->stream>>>((cx<float>*)x->data, ring, n, om,
                                                                             (float)omega, x_zero ? 1 : 0, V, nrhs);
    count_launch(ctx);
    SMG_CHECK_LAUNCH(ctx);
    return SMG_OK;
}

// One MR (omega <= 0) or Richardson (fixed omega) step of the FP16 smoother on r_it = f_rs[it]:
// t = D r (||t||^2 fused), A r = D^dag t (||A r||^2 fused), the step's omega, and r_{it+1} when
// write_next.  For A = D^dag D, <A r, r> = ||D r||^2, so MR's omega = ||D r||^2 / ||A r||^2.
smg_status mr_step_h(smg_mg* mg, int it, double omega, bool write_next) {
    smg_context* ctx = mg->ctx;
    smg_field *r = mg->f_rs[it], *Ar = mg->f_Ar, *t = mg->f_t;
    const int V = r->g.V, nrhs = r->nrhs;
    const bool mr = !(omega > 0);
    double* sc = mg->mr_om + (size_t)it * 3 * nrhs;
    float2* om = mg->mr_omf + (size_t)it * nrhs;
    SMG_TRY(smg_dslash_h_norm(mg->dirac, false, r, t, mr ? mg->hdots : nullptr, 0));
    SMG_TRY(smg_dslash_h_norm(mg->dirac, true, t, Ar, mr ? mg->hdots : nullptr, 1));
    if (mr) SMG_TRY(smg_mr_norms_finish(ctx, r->g.L, nrhs, mg->hdots, sc, reinterpret_cast<float*>(om)));
    if (write_next) {
        smg_field* rn = mg->f_rs[it + 1];
        k_mr_rupdate_h<<<pair_grid(V, nrhs), pair_block(nrhs), 0, ctx->stream>>>(
            (const __half2*)r->data, r->scale, (const __half2*)Ar->data, Ar->scale, (__half2*)rn->data, rn->scale,
            mr ? om : nullptr, (float)omega, V, nrhs);
        count_launch(ctx);
    }
    SMG_CHECK_LAUNCH(ctx);
    return SMG_OK;
}

// mr_fine / smooth_fine with FP16 residuals, A r and D r (x and b FP32).  keep_residual: the last
// step also writes r_n = b - A x (the residual the cycle restricts after pre-smoothing).  defer_x:
// the last x pass is left to the caller (mg->xp_*), which folds it into the prolongation.
smg_status smooth_fine_half(smg_mg* mg, smg_field* x, const smg_field* b, int niter, bool x_is_zero, double omega,
                            bool keep_residual, bool defer_x = false, bool defer_last_residual = false) {
    smg_context* ctx = mg->ctx;
    smg_field *r0 = mg->f_rs[0], *Ar = mg->f_Ar, *t = mg->f_t;
    const int V = b->g.V, nrhs = b->nrhs;
    if ((int)mg->f_rs.size() < niter + 1) return smg_fail(ctx, SMG_BAD_ARG, "FP16 smoother: too few residual fields");
    const dim3 blk(nrhs / 2, 512 / nrhs), grd((V + blk.y - 1) / blk.y);
    if (x_is_zero) {
        k_sub_h<<<grd, blk, 0, ctx->stream>>>((const cx<float>*)b->data, nullptr, nullptr, (__half2*)r0->data,
                                              r0->scale, V, nrhs);
    } else {
        SMG_TRY(smg_dslash(mg->dirac, false, x, t, nullptr));
        SMG_TRY(smg_dslash(mg->dirac, true, t, Ar, nullptr));
        k_sub_h<<<grd, blk, 0, ctx->stream>>>((const cx<float>*)b->data, (const __half2*)Ar->data, Ar->scale,
                                              (__half2*)r0->data, r0->scale, V, nrhs);
    }
    count_launch(ctx);
    int first = 0;  // first residual not yet added into x
    bool zero = x_is_zero;
    const bool fuse_last = defer_last_residual && keep_residual && niter > 0;
    for (int it = 0; it < niter; ++it) {
        SMG_TRY(mr_step_h(mg, it, omega, it + 1 < niter || (keep_residual && !fuse_last)));
        if (it + 1 - first == kMaxMrSteps) {
            SMG_TRY(mr_xupdate_h(mg, x, first, it + 1 - first, zero, omega));
            first = it + 1;
            zero = false;
        }
    }
    if (defer_x) {
        mg->xp_first = first;
        mg->xp_n = niter - first;
        mg->xp_zero = zero;
        mg->xp_omega = omega;
    } else {
        SMG_TRY(mr_xupdate_h(mg, x, first, niter - first, zero, omega));
    }
    mg->f_res = fuse_last ? nullptr : mg->f_rs[niter];
    mg->rn_step = fuse_last ? niter - 1 : -1;
    mg->rn_omega = omega;
    return SMG_OK;
}

TransferGeom transfer_geom(const smg_mg* mg, int l, int nrhs);
dim3 transfer_block(int nrhs);

// the pre-smoother's last residual update folded into the packed level-0 restriction;
// SMG_FUSE_LAST_RESIDUAL=0 keeps it as its own kernel
bool fuse_last_residual_on() {
    static const bool on = [] {
        const char* e = std::getenv("SMG_FUSE_LAST_RESIDUAL");
        return !(e && std::atoi(e) == 0);
    }();
    return on;
}

// the transfers with packed FMAs: SMG_TRANSFER_PACKED=0 keeps the generic kernels and separate x passes
bool transfer_packed_on() {
    static const bool on = [] {
        const char* e = std::getenv("SMG_TRANSFER_PACKED");
        return !(e && std::atoi(e) == 0);
    }();
    return on;
}

// the level-0 transfers with packed FMAs (k_restrict0_h, k_prolong0_ring) serve the FP16 smoother
// with 4 x 4 aggregates, 8, 16 or 32 coarse dofs and whole tiles of 32 rhs
bool transfer0_packed(const smg_mg* mg) {
    const bool on = transfer_packed_on();
    const Level& L = mg->lv[0];
    return on && mg->lv.size() > 1 && packed_shape0(L) && mg->work_nrhs % 32 == 0 && mg->f_r &&
           mg->f_r->prec == SMG_F16 && L.V32 && L.V32s;
}

// the restriction of the pre-smoother's final residual: f_res, or, when the last MR step left it to
// this kernel (mg->rn_step >= 0), r - omega A r of that step formed on the fly
smg_status restrict0_packed(smg_mg* mg, void* out) {
    smg_context* ctx = mg->ctx;
    const Level& L = mg->lv[0];
    const int nagg = mg->lv[1].nsites, nrhs = mg->work_nrhs;
    const TransferGeom t = transfer_geom(mg, 0, nrhs);
    const dim3 grid((nagg + 3) / 4, nrhs / 32), block(128);
    cx<float>* o = (cx<float>*)out;
    const bool fused = mg->rn_step >= 0;
    const smg_field* r = fused ? mg->f_rs[mg->rn_step] : mg->f_res;
    const __half2* rp = (const __half2*)r->data;
    const __half2* arp = fused ? (const __half2*)mg->f_Ar->data : nullptr;
    const float* ars = fused ? mg->f_Ar->scale : nullptr;
    const float2* om = fused && !(mg->rn_omega > 0) ? mg->mr_omf + (size_t)mg->rn_step * nrhs : nullptr;
    const float omega = (float)mg->rn_omega;
    mg->rn_step = -1;
#define SMG_R0(NC)                                                                                                  \
    do {                                                                                                            \
        if (fused)                                                                                                  \
            k_restrict0_h<NC, true><<<grid, block, 0, ctx->stream>>>(L.V32, rp, r->scale, o, t, nagg, arp, ars, om, \
                                                                     omega);                                        \
        else                                                                                                        \
            k_restrict0_h<NC, false><<<grid, block, 0, ctx->stream>>>(L.V32, rp, r->scale, o, t, nagg, nullptr,     \
                                                                      nullptr, nullptr, 0.f);                       \
    } while (0)
    if (L.nc_next == 8) SMG_R0(8);
    else if (L.nc_next == 16) SMG_R0(16);
    else SMG_R0(32);
#undef SMG_R0
    count_launch(ctx);
    SMG_CHECK_LAUNCH(ctx);
    return SMG_OK;
}

// x = (pending x pass) + P e, consuming mg->xp_*
smg_status prolong0_packed(smg_mg* mg, const void* coarse, smg_field* x) {
    smg_context* ctx = mg->ctx;
    const Level& L = mg->lv[0];
    const int nagg = mg->lv[1].nsites, nrhs = mg->work_nrhs;
    const TransferGeom t = transfer_geom(mg, 0, nrhs);
    ResidualRing ring{};
    for (int k = 0; k < mg->xp_n; ++k) {
        ring.r[k] = (const __half2*)mg->f_rs[mg->xp_first + k]->data;
        ring.s[k] = mg->f_rs[mg->xp_first + k]->scale;
    }
    const double omega = mg->xp_omega;
    const float2* om = omega > 0 ? nullptr : mg->mr_omf + (size_t)mg->xp_first * nrhs;
    const int acc = mg->xp_zero ? 0 : 1;
    const dim3 grid(nagg, nrhs / 32), block(128);
    const cx<float>* c = (const cx<float>*)coarse;
    cx<float>* xp = (cx<float>*)x->data;
#define SMG_P0(NC) \
    k_prolong0_ring<NC><<<grid, block, 0, ctx->stream>>>(L.V32s, c, xp, t, ring, mg->xp_n, om, (float)omega, acc)
    if (L.nc_next == 8) SMG_P0(8);
    else if (L.nc_next == 16) SMG_P0(16);
    else SMG_P0(32);
#undef SMG_P0
    mg->xp_n = 0;
    count_launch(ctx);
    SMG_CHECK_LAUNCH(ctx);
    return SMG_OK;
}


// dynamic shared memory of the aggregate transfer kernels: staged inputs (restriction: ne x lanes,
// prolongation: NC x lanes) and the aggregate's block vectors (ne x NC)
template <typename T>
size_t transfer_smem(const Level& L, int lanes, bool restrict_in) {
    const int64_t ne = (int64_t)L.ax * L.ay * L.ndof;
    return (size_t)(((restrict_in ? ne : L.nc_next) * lanes + ne * L.nc_next) * sizeof(cx<T>));
}
// above the default 48 KB the kernel instance must opt in (once per instance)
template <typename K>
void transfer_smem_attr(K kernel, size_t bytes, std::once_flag& once) {
    if (bytes > 48 * 1024)
        std::call_once(once, [kernel] {
            cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
        });
}

// restriction of the FP16 fine residual (k_restrict_agg with an FP16 reader)
smg_status restrict_half(smg_mg* mg, const smg_field* r, void* out) {
    smg_context* ctx = mg->ctx;
    const Level& L = mg->lv[0];
    const Level& N = mg->lv[1];
    const int nrhs = mg->work_nrhs;
    const int nc = L.nc_next;
    TransferGeom t = transfer_geom(mg, 0, nrhs);
    const dim3 block = transfer_block(nrhs);
    const dim3 grid(N.nsites, (nrhs + block.x - 1) / block.x);
    const size_t sm = transfer_smem<float>(L, (int)block.x, true);
    const InHalf in{(const __half2*)r->data, r->scale};
    if (nc == 8)
        k_restrict_agg<float, 8, InHalf><<<grid, block, sm, ctx->stream>>>(L.V32, in, (cx<float>*)out, t);
    else if (nc == 16)
        k_restrict_agg<float, 16, InHalf><<<grid, block, sm, ctx->stream>>>(L.V32, in, (cx<float>*)out, t);
    else
        k_restrict_agg<float, 32, InHalf><<<grid, block, sm, ctx->stream>>>(L.V32, in, (cx<float>*)out, t);
    count_launch(ctx);
    SMG_CHECK_LAUNCH(ctx);
    return SMG_OK;
}

// Fine MR on D^dag D (reference mr_smooth_op, src/smoother.cpp:26-40): on
// entry x holds the initial guess; x_is_zero skips r = b - A x.  The residual
// is updated recursively, r -= omega A r.
template <typename T>
smg_status mr_fine(smg_mg* mg, smg_field* x, const smg_field* b, int niter, bool x_is_zero) {
    smg_context* ctx = mg->ctx;
    smg_field *r = mg->f_r, *Ar = mg->f_Ar;
    const int64_t n = b->n_complex();
    if (x_is_zero) {
        SMG_CUDA(ctx, cudaMemsetAsync(x->data, 0, x->bytes, ctx->stream));
        SMG_CUDA(ctx, cudaMemcpyAsync(r->data, b->data, b->bytes, cudaMemcpyDeviceToDevice, ctx->stream));
    } else {
        SMG_TRY(level_apply_fine<T>(mg, x, Ar, nullptr, nullptr));
        k_vsub<T><<<blocks_for(n), 256, 0, ctx->stream>>>((cx<T>*)r->data, (const cx<T>*)b->data,
                                                        (const cx<T>*)Ar->data, n);
        count_launch(ctx);
    }
    double* sc = lvl_scal(mg, 0);
    for (int it = 0; it < niter; ++it) {
        SMG_TRY(level_apply_fine<T>(mg, r, Ar, r, sc));
        const VecView<T> xv = flat(fview<T>(x));
        k_mr_update<T><<<vec_grid(xv.nsites, xv.nrhs), vec_block(xv.nrhs), 0, ctx->stream>>>(
            xv, (cx<T>*)r->data, (const cx<T>*)Ar->data, sc);
        count_launch(ctx);
        SMG_CHECK_LAUNCH(ctx);
    }
    return SMG_OK;
}

// Coarse MR on the level-l stencil operator; b, x, r, Ar from the level's work
template <typename T>
smg_status mr_coarse(smg_mg* mg, int l, void* x, const void* b, int niter, bool x_is_zero) {
    smg_context* ctx = mg->ctx;
    const Level& L = mg->lv[l];
    CoarseWork& w = mg->cw[l];
    const int nrhs = mg->work_nrhs;
    VecView<T> xv = cview<T>(x, L, nrhs), rv = cview<T>(w.r, L, nrhs);
    const int64_t n = xv.n();
    const size_t bytes = (size_t)n * sizeof(cx<T>);
    if (x_is_zero) {
        SMG_CUDA(ctx, cudaMemsetAsync(x, 0, bytes, ctx->stream));
        SMG_CUDA(ctx, cudaMemcpyAsync(w.r, b, bytes, cudaMemcpyDeviceToDevice, ctx->stream));
    } else {
        SMG_TRY(coarse_apply<T>(mg, l, xv, (cx<T>*)w.Ar, 0, nullptr, nullptr));
        k_vsub<T><<<blocks_for(n), 256, 0, ctx->stream>>>((cx<T>*)w.r, (const cx<T>*)b, (const cx<T>*)w.Ar, n);
        count_launch(ctx);
    }
    double* sc = lvl_scal(mg, l);
    for (int it = 0; it < niter; ++it) {
        SMG_TRY(coarse_apply<T>(mg, l, rv, (cx<T>*)w.Ar, 2, (const cx<T>*)w.r, sc));
        const VecView<T> xf = flat(xv);
        k_mr_update<T><<<vec_grid(xf.nsites, xf.nrhs), vec_block(xf.nrhs), 0, ctx->stream>>>(
            xf, (cx<T>*)w.r, (const cx<T>*)w.Ar, sc);
        count_launch(ctx);
        SMG_CHECK_LAUNCH(ctx);
    }
    return SMG_OK;
}

// Richardson smoothing (richardson_smooth_op, src/smoother.cpp:64-73) with the
// level's fixed omega; same entry state and residual contract as the MR
// smoothers above, so the cycle picks either per level (mg_cycle,
// src/multigrid.cpp:57-61, 95-98).
template <typename T>
smg_status smooth_fine(smg_mg* mg, smg_field* x, const smg_field* b, int niter, bool x_is_zero,
                       bool keep_residual = true) {
    const double om = mg->lv[0].rich_omega;
    if (mg->f_r->prec == SMG_F16) return smooth_fine_half(mg, x, b, niter, x_is_zero, om, keep_residual);
    if (!(om > 0)) return mr_fine<T>(mg, x, b, niter, x_is_zero);
    smg_context* ctx = mg->ctx;
    smg_field *r = mg->f_r, *Ar = mg->f_Ar;
    const int64_t n = b->n_complex();
    if (x_is_zero) {
        SMG_CUDA(ctx, cudaMemsetAsync(x->data, 0, x->bytes, ctx->stream));
        SMG_CUDA(ctx, cudaMemcpyAsync(r->data, b->data, b->bytes, cudaMemcpyDeviceToDevice, ctx->stream));
    } else {
        SMG_TRY(level_apply_fine<T>(mg, x, Ar, nullptr, nullptr));
        k_vsub<T><<<blocks_for(n), 256, 0, ctx->stream>>>((cx<T>*)r->data, (const cx<T>*)b->data,
                                                        (const cx<T>*)Ar->data, n);
        count_launch(ctx);
    }
    for (int it = 0; it < niter; ++it) {
        SMG_TRY(level_apply_fine<T>(mg, r, Ar, nullptr, nullptr));
        const VecView<T> xv = flat(fview<T>(x));
        k_rich_update<T><<<vec_grid(xv.nsites, xv.nrhs), vec_block(xv.nrhs), 0, ctx->stream>>>(
            xv, (cx<T>*)r->data, (const cx<T>*)Ar->data, (T)om);
        count_launch(ctx);
        SMG_CHECK_LAUNCH(ctx);
    }
    return SMG_OK;
}

// Coarse MR (mr_smooth_op, src/smoother.cpp:26-40) on FP16 work vectors (mr16_level): r_0 = b - A x
// (or b) in FP16, then per step A r_k in FP16 with <A r_k, r_k>, ||A r_k||^2 and omega_k from the
// tensor-core apply, r_{k+1} = r_k - omega_k A r_k, and x += sum_k omega_k r_k once at the end (x and
// all arithmetic FP32).  The final residual stays in the ring slot res16 for the restriction.
smg_status mr_coarse_half(smg_mg* mg, int l, void* x, const void* b, int niter, bool x_is_zero, bool defer_x = false,
                          bool defer_last_residual = false) {
    smg_context* ctx = mg->ctx;
    const Level& L = mg->lv[l];
    CoarseWork& w = mg->cw[l];
    const int nrhs = mg->work_nrhs;
    const int ugrid = (int)((2ll * L.nsites + 7) / 8);  // one warp per (site, rhs half), 8 warps per block
    const cx<float>* y = nullptr;
    if (!x_is_zero) {
        SMG_TRY(coarse_apply<float>(mg, l, cview<float>(x, L, nrhs), (cx<float>*)w.Ar, 0, nullptr, nullptr));
        y = (const cx<float>*)w.Ar;
    }
    k_c16_from<<<ugrid, 256, 0, ctx->stream>>>((const cx<float>*)b, y, (__half2*)w.r16[0], w.r16s[0], L.nsites);
    count_launch(ctx);
    for (int it = 0; it < niter; ++it) {
        double* sc = w.mr16_sc + (size_t)it * nrhs * 3;
        float* om = w.mr16_om + (size_t)it * nrhs * 2;
        SMG_TRY(smg_coarse_tc_apply_mr16(ctx, L.Atc, L.nx, L.ny, nrhs, w.r16[it], w.r16s[it], w.ar16, w.ar16s, sc, om,
                                         device_err(mg)));
        if (defer_last_residual && it + 1 == niter) break;  // the restriction forms r - omega A r itself
        k_c16_rupdate<<<ugrid, 256, 0, ctx->stream>>>((const __half2*)w.r16[it], w.r16s[it], (const __half2*)w.ar16,
                                                      w.ar16s, (const float2*)om, (__half2*)w.r16[it + 1],
                                                      w.r16s[it + 1], L.nsites);
        count_launch(ctx);
        SMG_CHECK_LAUNCH(ctx);
    }
    w.rn_step = defer_last_residual && niter > 0 ? niter - 1 : -1;
    if (defer_x) {  // the packed prolongation into this level adds the steps (k_prolong_c16p)
        w.xp_n = niter;
        w.xp_zero = x_is_zero;
    } else if (niter > 0) {
        C16Ring ring{};
        for (int k = 0; k < niter; ++k) {
            ring.r[k] = (const __half2*)w.r16[k];
            ring.s[k] = w.r16s[k];
        }
        const int64_t rows = (int64_t)L.nsites * kC16Dofs;
        const int64_t warps = rows / kC16XRows;
        k_c16_xupdate<<<(unsigned)((warps + 7) / 8), 256, 0, ctx->stream>>>((cx<float>*)x, ring, niter, (const float2*)w.mr16_om, L.nsites,
                                                      x_is_zero ? 1 : 0);
        count_launch(ctx);
    } else if (x_is_zero) {
        SMG_CUDA(ctx, cudaMemsetAsync(x, 0, (size_t)L.nsites * nrhs * L.ndof * sizeof(cx<float>), ctx->stream));
    }
    w.res16 = niter;
    SMG_CHECK_LAUNCH(ctx);
    return SMG_OK;
}

// restriction of an intermediate level's FP16 residual (k_restrict_agg with the InHalfC reader)
smg_status restrict_c16(smg_mg* mg, int l, void* out) {
    smg_context* ctx = mg->ctx;
    const Level& L = mg->lv[l];
    const Level& N = mg->lv[l + 1];
    CoarseWork& w = mg->cw[l];
    const int nrhs = mg->work_nrhs;
    const int nc = L.nc_next;
    if (nc != 8 && nc != 16 && nc != 32) return smg_fail(ctx, SMG_UNSUPPORTED, "FP16 restriction: coarse dofs");
    TransferGeom t = transfer_geom(mg, l, nrhs);
    const dim3 block = transfer_block(nrhs);
    const dim3 grid(N.nsites, (nrhs + block.x - 1) / block.x);
    const size_t sm = transfer_smem<float>(L, (int)block.x, true);
    const InHalfC in{(const __half2*)w.r16[w.res16], w.r16s[w.res16]};
#define SMG_RC(NC)                                                                                           \
    do {                                                                                                     \
        static std::once_flag once;                                                                          \
        transfer_smem_attr(k_restrict_agg<float, NC, InHalfC>, sm, once);                                    \
        k_restrict_agg<float, NC, InHalfC><<<grid, block, sm, ctx->stream>>>(L.V32, in, (cx<float>*)out, t); \
    } while (0)
    if (nc == 8) SMG_RC(8);
    else if (nc == 16) SMG_RC(16);
    else SMG_RC(32);
#undef SMG_RC
    count_launch(ctx);
    SMG_CHECK_LAUNCH(ctx);
    return SMG_OK;
}

// the packed transfers of an intermediate FP16 level (k_restrict_c16p, k_prolong_c16p)
bool transfer_c16_packed(const smg_mg* mg, int l) {
    const Level& L = mg->lv[l];
    return transfer_packed_on() && l + 1 < (int)mg->lv.size() && packed_shape_c16(L) && L.V32s && L.V32o &&
           !mg->cw[l].r16.empty() && mr16_level(mg, l, mg->work_nrhs, SMG_F32);
}

smg_status restrict_c16_packed(smg_mg* mg, int l, void* out) {
    smg_context* ctx = mg->ctx;
    const Level& L = mg->lv[l];
    CoarseWork& w = mg->cw[l];
    const int nagg = mg->lv[l + 1].nsites;
    const TransferGeom t = transfer_geom(mg, l, 32);
    // the last MR step's r - omega A r formed in the kernel when that step left it (rn_step >= 0)
    const bool fused = w.rn_step >= 0;
    const int slot = fused ? w.rn_step : w.res16;
    const __half2* r = (const __half2*)w.r16[slot];
    const float* rs = w.r16s[slot];
    const __half2* ar = fused ? (const __half2*)w.ar16 : nullptr;
    const float* ars = fused ? w.ar16s : nullptr;
    const float2* om = fused ? (const float2*)w.mr16_om + (size_t)w.rn_step * 32 : nullptr;
    w.rn_step = -1;
    cx<float>* o = (cx<float>*)out;
#define SMG_RC16(NC, G, B)                                                                                         \
    do {                                                                                                           \
        if (fused)                                                                                                 \
            k_restrict_c16p<NC, true><<<G, B, 0, ctx->stream>>>(L.V32o, r, rs, o, t, nagg, ar, ars, om);          \
        else                                                                                                       \
            k_restrict_c16p<NC, false><<<G, B, 0, ctx->stream>>>(L.V32o, r, rs, o, t, nagg, nullptr, nullptr,      \
                                                                 nullptr);                                         \
    } while (0)
    if (L.nc_next == 8) SMG_RC16(8, (nagg + 3) / 4, 128);
    else if (L.nc_next == 16) SMG_RC16(16, (nagg + 3) / 4, 128);
    else SMG_RC16(32, (nagg + 1) / 2, 64);
#undef SMG_RC16
    count_launch(ctx);
    SMG_CHECK_LAUNCH(ctx);
    return SMG_OK;
}

// x = (pending x pass of level l) + P e, consuming cw[l].xp_*
smg_status prolong_c16_packed(smg_mg* mg, int l, const void* coarse, void* x) {
    smg_context* ctx = mg->ctx;
    const Level& L = mg->lv[l];
    CoarseWork& w = mg->cw[l];
    const int nagg = mg->lv[l + 1].nsites;
    const TransferGeom t = transfer_geom(mg, l, 32);
    C16Ring ring{};
    for (int k = 0; k < w.xp_n; ++k) {
        ring.r[k] = (const __half2*)w.r16[k];
        ring.s[k] = w.r16s[k];
    }
    const float2* om = (const float2*)w.mr16_om;
    const int acc = w.xp_zero ? 0 : 1;
    const cx<float>* c = (const cx<float>*)coarse;
    cx<float>* xp = (cx<float>*)x;
    if (L.nc_next == 8)
        k_prolong_c16p<8><<<nagg, 256, 0, ctx->stream>>>(L.V32s, c, xp, t, ring, w.xp_n, om, acc);
    else if (L.nc_next == 16)
        k_prolong_c16p<16><<<nagg, 256, 0, ctx->stream>>>(L.V32s, c, xp, t, ring, w.xp_n, om, acc);
    else
        k_prolong_c16p<32><<<nagg, 256, 0, ctx->stream>>>(L.V32s, c, xp, t, ring, w.xp_n, om, acc);
    w.xp_n = 0;
    count_launch(ctx);
    SMG_CHECK_LAUNCH(ctx);
    return SMG_OK;
}

template <typename T>
smg_status smooth_coarse(smg_mg* mg, int l, void* x, const void* b, int niter, bool x_is_zero) {
    const double om = mg->lv[l].rich_omega;
    if (std::is_same<T, float>::value && !mg->cw[l].r16.empty() && mr16_level(mg, l, mg->work_nrhs, SMG_F32))
        return mr_coarse_half(mg, l, x, b, niter, x_is_zero);
    if (!(om > 0)) return mr_coarse<T>(mg, l, x, b, niter, x_is_zero);
    smg_context* ctx = mg->ctx;
    const Level& L = mg->lv[l];
    CoarseWork& w = mg->cw[l];
    const int nrhs = mg->work_nrhs;
    VecView<T> xv = cview<T>(x, L, nrhs), rv = cview<T>(w.r, L, nrhs);
    const int64_t n = xv.n();
    const size_t bytes = (size_t)n * sizeof(cx<T>);
    if (x_is_zero) {
        SMG_CUDA(ctx, cudaMemsetAsync(x, 0, bytes, ctx->stream));
        SMG_CUDA(ctx, cudaMemcpyAsync(w.r, b, bytes, cudaMemcpyDeviceToDevice, ctx->stream));
    } else {
        SMG_TRY(coarse_apply<T>(mg, l, xv, (cx<T>*)w.Ar, 0, nullptr, nullptr));
        k_vsub<T><<<blocks_for(n), 256, 0, ctx->stream>>>((cx<T>*)w.r, (const cx<T>*)b, (const cx<T>*)w.Ar, n);
        count_launch(ctx);
    }
    for (int it = 0; it < niter; ++it) {
        SMG_TRY(coarse_apply<T>(mg, l, rv, (cx<T>*)w.Ar, 0, nullptr, nullptr));
        const VecView<T> xf = flat(xv);
        k_rich_update<T><<<vec_grid(xf.nsites, xf.nrhs), vec_block(xf.nrhs), 0, ctx->stream>>>(
            xf, (cx<T>*)w.r, (const cx<T>*)w.Ar, (T)om);
        count_launch(ctx);
        SMG_CHECK_LAUNCH(ctx);
    }
    return SMG_OK;
}

// Coarsest solve: CG from x = 0 to coarse_tol (SparseCoarseOp::solve without
// deflation, src/coarse_op.h:492-547); the host checks progress every 8 steps
// coarse_cg with the residual and search direction in FP16 (coarse_half): the same iteration, stop
// rule and per-rhs masks, the tensor-core apply reading p in FP16 for A p and <A p, p>
smg_status coarse_cg_half(smg_mg* mg, int l, void* x, const void* b) {
    smg_context* ctx = mg->ctx;
    const Level& L = mg->lv[l];
    CoarseWork& w = mg->cw[l];
    const int nrhs = mg->work_nrhs;
    double* sc = lvl_scal(mg, l);
    CcgState s;
    s.rr = sc;
    s.pap3 = sc + nrhs;
    s.bnorm2 = sc + 4 * nrhs;
    s.beta = sc + 5 * nrhs;
    s.active = (int*)(sc + 6 * nrhs);
    s.n_active = (int*)(sc + 7 * nrhs);
    s.tol2 = mg->p.coarse_tol * mg->p.coarse_tol;
    const dim3 blk(32, 8);  // lane = rhs, one site per warp
    const int grid = std::min((L.nsites + 7) / 8, 4 * ctx->num_sms);
    SMG_TRY(smg_reduce_reserve(ctx, (size_t)grid * nrhs));
    __half2 *rh = (__half2*)w.rh, *ph = (__half2*)w.ph;
    k_ccgh_init<<<grid, blk, 0, ctx->stream>>>((const cx<float>*)b, (cx<float>*)x, rh, w.rs, ph, w.ps, L.nsites,
                                               ctx->red.partials, ctx->red.tickets, s.rr);
    k_ccg_init<<<1, 256, 0, ctx->stream>>>(s, nrhs, 0);
    count_launch(ctx, 2);
    SMG_TRY(smg_host_stage_reserve(ctx, 64));
    int* h_act = (int*)ctx->host_stage;
    int it = 0;
    while (it < mg->p.coarse_max_iter) {
        int chunk = std::min(8, mg->p.coarse_max_iter - it);
        for (int c = 0; c < chunk; ++c) {
            SMG_TRY(smg_coarse_tc_apply_h(ctx, L.Atc, L.nx, L.ny, nrhs, ph, w.ps, (cx<float>*)w.Ar, ph, w.ps, s.pap3,
                                          s.n_active, device_err(mg)));
            k_ccgh_update<<<grid, blk, 0, ctx->stream>>>(s, (cx<float>*)x, rh, w.rs, ph, w.ps, (const cx<float>*)w.Ar,
                                                         L.nsites, ctx->red.partials, ctx->red.tickets);
            k_ccgh_p<<<grid, blk, 0, ctx->stream>>>(s, rh, w.rs, ph, w.ps, L.nsites);
            count_launch(ctx, 2);
            SMG_CHECK_LAUNCH(ctx);
        }
        it += chunk;
        if (mg->capturing) continue;  // inside a graph: the gated kernels finish the budget as no-ops
        SMG_CUDA(ctx, cudaMemcpyAsync(h_act, s.n_active, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
        SMG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        if (*h_act == 0) break;
    }
    return SMG_OK;
}

template <typename T>
smg_status coarse_cg(smg_mg* mg, int l, void* x, const void* b) {
    smg_context* ctx = mg->ctx;
    const Level& L = mg->lv[l];
    if (std::is_same<T, float>::value && coarse_half_level(mg, l, mg->work_nrhs, SMG_F32) && mg->cw[l].rh &&
        !(l == mg->defl.level && mg->defl.n > 0)) {
        CoarseWork& w = mg->cw[l];
        if (w.ph2 && ccg_tc_level(mg, l))
            return smg_coarse_cg_tc(mg->ctx, L.Atc, L.nx, L.ny, (const cx<float>*)b, (cx<float>*)x, w.rh, w.rs, w.ph,
                                    w.ps, w.ph2, w.ps2, (cx<float>*)w.Ar, w.ccg_part, (int*)mg->cg_state,
                                    mg->p.coarse_max_iter, mg->p.coarse_tol, mg->spin_limit);
        return coarse_cg_half(mg, l, x, b);
    }
    if (mg->persistent && mg->work_nrhs == 1 && !(l == mg->defl.level && mg->defl.n > 0)) {
        if (L.ndof == 8) return coarse_cg_persistent<T, 8>(mg, l, x, b);
        if (L.ndof == 16) return coarse_cg_persistent<T, 16>(mg, l, x, b);
        if (L.ndof == 32) return coarse_cg_persistent<T, 32>(mg, l, x, b);
    }
    CoarseWork& w = mg->cw[l];
    const int nrhs = mg->work_nrhs;
    VecView<T> xv = cview<T>(x, L, nrhs), pv = cview<T>(w.p, L, nrhs), rv = cview<T>(w.r, L, nrhs);
    const size_t bytes = (size_t)xv.n() * sizeof(cx<T>);
    const bool deflated = l == mg->defl.level && mg->defl.n > 0;
    double* sc = lvl_scal(mg, l);
    CcgState s;
    s.rr = sc;
    s.pap3 = sc + nrhs;
    s.bnorm2 = sc + 4 * nrhs;
    s.beta = sc + 5 * nrhs;
    s.active = (int*)(sc + 6 * nrhs);
    s.n_active = (int*)(sc + 7 * nrhs);
    s.tol2 = mg->p.coarse_tol * mg->p.coarse_tol;
    if (deflated) {
        // SparseCoarseOp::solve (src/coarse_op.h:492-520): CG from x0 = sum_i v_i (v_i^dag b) / lambda_i
        SMG_TRY(smg_defl_guess<T>(ctx, mg->defl, cview<T>((void*)b, L, nrhs), xv));
        SMG_TRY(coarse_apply<T>(mg, l, xv, (cx<T>*)w.Ar, 0, nullptr, nullptr));
        k_vsub<T><<<blocks_for(xv.n()), 256, 0, ctx->stream>>>((cx<T>*)w.r, (const cx<T>*)b, (const cx<T>*)w.Ar,
                                                             xv.n());
        count_launch(ctx);
        SMG_CHECK_LAUNCH(ctx);
        SMG_CUDA(ctx, cudaMemcpyAsync(w.p, w.r, bytes, cudaMemcpyDeviceToDevice, ctx->stream));
        // the stopping test is relative to ||b|| as in the reference
        SMG_TRY(vreduce<T>(ctx, flat(cview<T>((void*)b, L, nrhs)), nullptr, VR_NORM, s.bnorm2));
    } else {
        SMG_CUDA(ctx, cudaMemsetAsync(x, 0, bytes, ctx->stream));
        SMG_CUDA(ctx, cudaMemcpyAsync(w.r, b, bytes, cudaMemcpyDeviceToDevice, ctx->stream));
        SMG_CUDA(ctx, cudaMemcpyAsync(w.p, b, bytes, cudaMemcpyDeviceToDevice, ctx->stream));
    }
    SMG_TRY(vreduce<T>(ctx, flat(rv), nullptr, VR_NORM, s.rr));
    k_ccg_init<<<1, 256, 0, ctx->stream>>>(s, nrhs, deflated ? 1 : 0);
    count_launch(ctx);
    const VecView<T> xf = flat(xv), pf = flat(pv);
    ReduceLaunch rl = reduce_launch(xf.nsites, nrhs);
    if (rl.grid.x > 148) rl.grid.x = 148;  // fewer partials for the finishing block (k_ccg_update strides)
    SMG_TRY(smg_reduce_reserve(ctx, (size_t)rl.grid.x * nrhs * 3));
    SMG_TRY(smg_host_stage_reserve(ctx, 64));
    int* h_act = (int*)ctx->host_stage;
    int it = 0;
    while (it < mg->p.coarse_max_iter) {
        int chunk = std::min(8, mg->p.coarse_max_iter - it);
        for (int c = 0; c < chunk; ++c) {
            SMG_TRY(coarse_apply<T>(mg, l, pv, (cx<T>*)w.Ar, 2, (const cx<T>*)w.p, s.pap3, s.n_active));
            k_ccg_update<T><<<rl.grid, rl.block, 0, ctx->stream>>>(s, xf, (cx<T>*)w.r, (const cx<T>*)w.p,
                                                                   (const cx<T>*)w.Ar, ctx->red.partials,
                                                                   ctx->red.tickets);
            k_ccg_p<T><<<vec_grid(pf.nsites, nrhs), vec_block(nrhs), 0, ctx->stream>>>(s, pf, (const cx<T>*)w.r);
            count_launch(ctx, 2);
            SMG_CHECK_LAUNCH(ctx);
        }
        it += chunk;
        if (mg->capturing) continue;  // inside a graph: the gated kernels finish the budget as no-ops
        SMG_CUDA(ctx, cudaMemcpyAsync(h_act, s.n_active, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
        SMG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        if (*h_act == 0) break;
    }
    return SMG_OK;
}

TransferGeom transfer_geom(const smg_mg* mg, int l, int nrhs) {
    const Level& L = mg->lv[l];
    TransferGeom t;
    t.level0 = l == 0 ? 1 : 0;
    if (l == 0) t.g = mg->null0[0]->g;
    t.nx = L.nx;
    t.ax = L.ax;
    t.ay = L.ay;
    t.nax = L.nx / L.ax;
    t.ndof = L.ndof;
    t.nrhs = nrhs;
    return t;
}

dim3 transfer_block(int nrhs) {
    int lanes = 1;
    while (lanes * 2 <= nrhs && lanes < 32) lanes *= 2;
    return dim3(lanes, 256 / lanes);
}

template <typename T>
smg_status restrict_to(smg_mg* mg, int l, const void* fine_or_coarse, void* out) {
    smg_context* ctx = mg->ctx;
    const Level& L = mg->lv[l];
    const Level& N = mg->lv[l + 1];
    const int nrhs = mg->work_nrhs;
    const int nc = L.nc_next;
    if ((nc == 8 || nc == 16 || nc == 32) && nrhs >= 8) {  // few rhs: one thread per output below
        TransferGeom t = transfer_geom(mg, l, nrhs);
        const dim3 block = transfer_block(nrhs);
        const dim3 grid(N.nsites, (nrhs + block.x - 1) / block.x);
        const size_t sm = transfer_smem<T>(L, (int)block.x, true);
#define SMG_RA(NC)                                                                                         \
    do {                                                                                                   \
        static std::once_flag once;                                                                        \
        transfer_smem_attr(k_restrict_agg<T, NC>, sm, once);                                               \
        k_restrict_agg<T, NC><<<grid, block, sm, ctx->stream>>>(Vp<T>(L), InPlain<T>{(const cx<T>*)fine_or_coarse}, \
                                                               (cx<T>*)out, t);                            \
    } while (0)
        if (nc == 8) SMG_RA(8);
        else if (nc == 16) SMG_RA(16);
        else SMG_RA(32);
#undef SMG_RA
    } else {
        int64_t total = (int64_t)N.nsites * nrhs * nc;
        if (l == 0)
            k_restrict0<T><<<blocks_for(total), 256, 0, ctx->stream>>>(Vp<T>(L), (const cx<T>*)fine_or_coarse,
                                                                      (cx<T>*)out, mg->null0[0]->g, L.ax, L.ay, nc,
                                                                      nrhs);
        else
            k_restrict_c<T><<<blocks_for(total), 256, 0, ctx->stream>>>(Vp<T>(L), (const cx<T>*)fine_or_coarse,
                                                                       (cx<T>*)out, L.nx, L.ax, L.ay, L.ndof, nc,
                                                                       N.nsites, nrhs);
    }
    count_launch(ctx);
    SMG_CHECK_LAUNCH(ctx);
    return SMG_OK;
}

template <typename T>
smg_status prolong_to(smg_mg* mg, int l, const void* coarse, void* out, int accumulate) {
    smg_context* ctx = mg->ctx;
    const Level& L = mg->lv[l];
    const Level& N = mg->lv[l + 1];
    const int nrhs = mg->work_nrhs;
    const int nc = L.nc_next;
    if ((nc == 8 || nc == 16 || nc == 32) && nrhs >= 8) {  // few rhs: one thread per output below
        TransferGeom t = transfer_geom(mg, l, nrhs);
        const dim3 block = transfer_block(nrhs);
        const dim3 grid(N.nsites, (nrhs + block.x - 1) / block.x);
        const size_t sm = transfer_smem<T>(L, (int)block.x, false);
#define SMG_PA(NC)                                                                                         \
    do {                                                                                                   \
        static std::once_flag once;                                                                        \
        transfer_smem_attr(k_prolong_agg<T, NC>, sm, once);                                                \
        k_prolong_agg<T, NC><<<grid, block, sm, ctx->stream>>>(Vp<T>(L), (const cx<T>*)coarse, (cx<T>*)out, t, \
                                                              accumulate);                                 \
    } while (0)
        if (nc == 8) SMG_PA(8);
        else if (nc == 16) SMG_PA(16);
        else SMG_PA(32);
#undef SMG_PA
    } else if (l == 0) {
        const Geom g = mg->null0[0]->g;
        k_prolong0<T><<<blocks_for((int64_t)g.V * nrhs), 256, 0, ctx->stream>>>(
            Vp<T>(L), (const cx<T>*)coarse, (cx<T>*)out, g, L.ax, L.ay, nc, nrhs, accumulate);
    } else {
        int64_t total = (int64_t)L.nsites * nrhs * L.ndof;
        k_prolong_c<T><<<blocks_for(total), 256, 0, ctx->stream>>>(Vp<T>(L), (const cx<T>*)coarse, (cx<T>*)out, L.nx,
                                                                  L.ny, L.ax, L.ay, L.ndof, nc, nrhs, accumulate);
    }
    count_launch(ctx);
    SMG_CHECK_LAUNCH(ctx);
    return SMG_OK;
}

// mg_cycle (reference src/multigrid.cpp:43-102) at a coarse level l >= 1:
// b = cw[l].b, result in x
template <typename T>
smg_status cycle_coarse(smg_mg* mg, int l, void* x, const void* b) {
    const int last = (int)mg->lv.size() - 1;
    if (l == last) return coarse_cg<T>(mg, l, x, b);
    smg_context* ctx = mg->ctx;
    const Level& L = mg->lv[l];
    const int nrhs = mg->work_nrhs;
    // packed FP16-level transfers: the pre-smoothing x pass is folded into the prolongation
    const bool packed = std::is_same<T, float>::value && transfer_c16_packed(mg, l);
    if (packed)
        SMG_TRY(mr_coarse_half(mg, l, x, b, mg->p.pre_smooth, true, true, fuse_last_residual_on()));
    else
        SMG_TRY(smooth_coarse<T>(mg, l, x, b, mg->p.pre_smooth, true));
    // residual of the smoothed x is in cw[l].r (or, FP16, in the ring slot cw[l].res16)
    CoarseWork& nw = mg->cw[l + 1];
    if (packed)
        SMG_TRY(restrict_c16_packed(mg, l, nw.b));
    else if (std::is_same<T, float>::value && !mg->cw[l].r16.empty() && mr16_level(mg, l, nrhs, SMG_F32))
        SMG_TRY(restrict_c16(mg, l, nw.b));
    else
        SMG_TRY(restrict_to<T>(mg, l, mg->cw[l].r, nw.b));
    SMG_TRY(cycle_coarse<T>(mg, l + 1, nw.x, nw.b));
    if (mg->p.w_cycle && l + 1 < last) {
        const Level& N = mg->lv[l + 1];
        const int64_t nn = (int64_t)N.nsites * nrhs * N.ndof;
        const size_t nb = (size_t)nn * sizeof(cx<T>);
        SMG_CUDA(ctx, cudaMemcpyAsync(nw.e, nw.x, nb, cudaMemcpyDeviceToDevice, ctx->stream));
        SMG_TRY(coarse_apply<T>(mg, l + 1, cview<T>(nw.e, N, nrhs), (cx<T>*)nw.Ar, 0, nullptr, nullptr));
        k_vsub<T><<<blocks_for(nn), 256, 0, ctx->stream>>>((cx<T>*)nw.b, (const cx<T>*)nw.b, (const cx<T>*)nw.Ar, nn);
        count_launch(ctx);
        SMG_TRY(cycle_coarse<T>(mg, l + 1, nw.x, nw.b));
        k_vadd<T><<<blocks_for(nn), 256, 0, ctx->stream>>>((cx<T>*)nw.x, (const cx<T>*)nw.e, nn);
        count_launch(ctx);
    }
    if (packed)
        SMG_TRY(prolong_c16_packed(mg, l, nw.x, x));
    else
        SMG_TRY(prolong_to<T>(mg, l, nw.x, x, 1));
    (void)L;
    return smooth_coarse<T>(mg, l, x, b, mg->p.post_smooth, false);
}

// mg_cycle at the fine level: x = M^-1 b for fine fields of precision T
template <typename T>
smg_status cycle_fine(smg_mg* mg, smg_field* x, const smg_field* b) {
    smg_context* ctx = mg->ctx;
    const int last = (int)mg->lv.size() - 1;
    // packed level-0 transfers: the pre-smoothing x pass is folded into the prolongation
    const bool packed = std::is_same<T, float>::value && transfer0_packed(mg);
    if (packed)
        SMG_TRY(smooth_fine_half(mg, x, b, mg->p.pre_smooth, true, mg->lv[0].rich_omega, true, true,
                                 fuse_last_residual_on()));
    else
        SMG_TRY(smooth_fine<T>(mg, x, b, mg->p.pre_smooth, true));
    CoarseWork& nw = mg->cw[1];
    if (packed)
        SMG_TRY(restrict0_packed(mg, nw.b));
    else if (mg->f_r->prec == SMG_F16)
        SMG_TRY(restrict_half(mg, mg->f_res, nw.b));
    else
        SMG_TRY(restrict_to<T>(mg, 0, mg->f_r->data, nw.b));
    SMG_TRY(cycle_coarse<T>(mg, 1, nw.x, nw.b));
    if (mg->p.w_cycle && 1 < last) {
        const Level& N = mg->lv[1];
        const int nrhs = mg->work_nrhs;
        const int64_t nn = (int64_t)N.nsites * nrhs * N.ndof;
        SMG_CUDA(ctx, cudaMemcpyAsync(nw.e, nw.x, (size_t)nn * sizeof(cx<T>), cudaMemcpyDeviceToDevice, ctx->stream));
        SMG_TRY(coarse_apply<T>(mg, 1, cview<T>(nw.e, N, nrhs), (cx<T>*)nw.Ar, 0, nullptr, nullptr));
        k_vsub<T><<<blocks_for(nn), 256, 0, ctx->stream>>>((cx<T>*)nw.b, (const cx<T>*)nw.b, (const cx<T>*)nw.Ar, nn);
        count_launch(ctx);
        SMG_TRY(cycle_coarse<T>(mg, 1, nw.x, nw.b));
        k_vadd<T><<<blocks_for(nn), 256, 0, ctx->stream>>>((cx<T>*)nw.x, (const cx<T>*)nw.e, nn);
        count_launch(ctx);
    }
    if (packed)
        SMG_TRY(prolong0_packed(mg, nw.x, x));
    else
        SMG_TRY(prolong_to<T>(mg, 0, nw.x, x->data, 1));
    return smooth_fine<T>(mg, x, b, mg->p.post_smooth, false, false);
}

// ------------------------------------------------------------ setup

// inverse iteration for one level's near-null vectors (multigrid.cpp:435-484
// at level 0, :545-587 at coarse levels); vecs hold the start vectors on entry
smg_status null_space_fine(smg_mg* mg, std::vector<smg_field*>& vecs) {
    smg_context* ctx = mg->ctx;
    const int k = (int)vecs.size();
    SMG_TRY(ensure_work(mg, 1, SMG_F64));
    smg_field* xn = nullptr;
    SMG_TRY(smg_field_create(ctx, vecs[0]->g.L, 1, SMG_F64, &xn));
    double* sc = mg->scal;  // [0..1] norm, [2..3] dot
    SMG_TRY(smg_host_stage_reserve(ctx, 64));
    auto norm_of = [&](smg_field* f, double* hv) -> smg_status {
        SMG_TRY(vreduce<double>(ctx, flat(fview<double>(f)), nullptr, VR_NORM, sc));
        SMG_CUDA(ctx, cudaMemcpyAsync(ctx->host_stage, sc, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
        SMG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        *hv = std::sqrt(ctx->host_stage[0]);
        return SMG_OK;
    };
    auto scale_by = [&](smg_field* f, double s) -> smg_status {
        double a[2] = {s, 0.0};
        return smg_blas_scale(a, f);
    };
    auto ortho = [&](smg_field* v, int upto) -> smg_status {
        for (int j = 0; j < upto; ++j) {
            SMG_TRY(vreduce<double>(ctx, flat(fview<double>(vecs[j])), (const cx<double>*)v->data, VR_DOT, sc + 2));
            SMG_TRY(vaxpy<double>(ctx, flat(fview<double>(v)), (const cx<double>*)vecs[j]->data, sc + 2, -1.0));
        }
        return SMG_OK;
    };
    for (int i = 0; i < k; ++i) {
        double nv;
        SMG_TRY(norm_of(vecs[i], &nv));
        SMG_TRY(scale_by(vecs[i], 1.0 / nv));
        for (int it = 0; it < mg->p.null_iters; ++it) {
            SMG_TRY(mr_fine<double>(mg, xn, vecs[i], mg->p.null_mr_steps, true));
            SMG_TRY(ortho(xn, i));
            SMG_TRY(norm_of(xn, &nv));
            if (nv > 1e-14) {
                SMG_TRY(scale_by(xn, 1.0 / nv));
                SMG_CUDA(ctx, cudaMemcpyAsync(vecs[i]->data, xn->data, xn->bytes, cudaMemcpyDeviceToDevice,
                                              ctx->stream));
            } else {
                break;
            }
        }
    }
    for (int i = 0; i < k; ++i) {
        SMG_TRY(ortho(vecs[i], i));
        double nv;
        SMG_TRY(norm_of(vecs[i], &nv));
        if (nv > 1e-14) SMG_TRY(scale_by(vecs[i], 1.0 / nv));
    }
    smg_field_destroy(xn);
    return SMG_OK;
}

smg_status null_space_coarse(smg_mg* mg, int l, std::vector<cx<double>*>& vecs) {
    smg_context* ctx = mg->ctx;
    const Level& L = mg->lv[l];
    const int k = (int)vecs.size();
    SMG_TRY(ensure_work(mg, 1, SMG_F64));
    CoarseWork& w = mg->cw[l];
    double* sc = mg->scal;
    SMG_TRY(smg_host_stage_reserve(ctx, 64));
    auto view = [&](void* p) { return flat(cview<double>(p, L, 1)); };
    auto norm_of = [&](void* f, double* hv) -> smg_status {
        SMG_TRY(vreduce<double>(ctx, view(f), nullptr, VR_NORM, sc));
        SMG_CUDA(ctx, cudaMemcpyAsync(ctx->host_stage, sc, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
        SMG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        *hv = std::sqrt(ctx->host_stage[0]);
        return SMG_OK;
    };
    auto scale_by = [&](void* f, double s) -> smg_status {
        double a[2] = {s - 1.0, 0.0};  // y += (s - 1) y
        SMG_CUDA(ctx, cudaMemcpyAsync(sc + 8, a, sizeof(a), cudaMemcpyHostToDevice, ctx->stream));
        return vaxpy<double>(ctx, view(f), (const cx<double>*)f, sc + 8, 1.0);
    };
    auto ortho = [&](void* v, int upto) -> smg_status {
        for (int j = 0; j < upto; ++j) {
            SMG_TRY(vreduce<double>(ctx, view(vecs[j]), (const cx<double>*)v, VR_DOT, sc + 2));
            SMG_TRY(vaxpy<double>(ctx, view(v), (const cx<double>*)vecs[j], sc + 2, -1.0));
        }
        return SMG_OK;
    };
    const size_t bytes = (size_t)L.nsites * L.ndof * sizeof(cx<double>);
    for (int i = 0; i < k; ++i) {
        double nv;
        SMG_TRY(norm_of(vecs[i], &nv));
        SMG_TRY(scale_by(vecs[i], 1.0 / nv));
        for (int it = 0; it < mg->p.null_iters; ++it) {
            SMG_TRY(mr_coarse<double>(mg, l, w.x, vecs[i], mg->p.null_mr_steps, true));
            SMG_TRY(ortho(w.x, i));
            SMG_TRY(norm_of(w.x, &nv));
            if (nv > 1e-14) {
                SMG_TRY(scale_by(w.x, 1.0 / nv));
                SMG_CUDA(ctx, cudaMemcpyAsync(vecs[i], w.x, bytes, cudaMemcpyDeviceToDevice, ctx->stream));
            } else {
                break;
            }
        }
    }
    for (int i = 0; i < k; ++i) {
        SMG_TRY(ortho(vecs[i], i));
        double nv;
        SMG_TRY(norm_of(vecs[i], &nv));
        if (nv > 1e-14) SMG_TRY(scale_by(vecs[i], 1.0 / nv));
    }
    return SMG_OK;
}

smg_status make_f32_copies(smg_mg* mg) {
    smg_context* ctx = mg->ctx;
    for (size_t l = 0; l < mg->lv.size(); ++l) {
        Level& L = mg->lv[l];
        if (L.V64) {
            int64_t n = L.vsize();
            if (!L.V32) SMG_CUDA(ctx, cudaMalloc(&L.V32, n * sizeof(cx<float>)));
            k_cvt_flat<float, double><<<blocks_for(n), 256, 0, ctx->stream>>>(L.V64, L.V32, n);
            count_launch(ctx);
            const int64_t np = n / 2;
            if ((l == 0 && mg->p.smoother_half && packed_shape0(L)) ||
                (l >= 1 && mg->p.coarse_half && packed_shape_c16(L))) {
                if (!L.V32s) SMG_CUDA(ctx, cudaMalloc(&L.V32s, np * sizeof(float4)));
                k_pair_spins<<<blocks_for(np), 256, 0, ctx->stream>>>(L.V64, L.V32s, np, L.nc_next);
                count_launch(ctx);
            }
            if (l >= 1 && mg->p.coarse_half && packed_shape_c16(L)) {
                if (!L.V32o) SMG_CUDA(ctx, cudaMalloc(&L.V32o, np * sizeof(float4)));
                k_pair_spins<<<blocks_for(np), 256, 0, ctx->stream>>>(L.V64, L.V32o, np, 1);
                count_launch(ctx);
            }
        }
        if (L.A64) {
            int64_t n = L.asize();
            if (!L.A32) SMG_CUDA(ctx, cudaMalloc(&L.A32, n * sizeof(cx<float>)));
            k_cvt_flat<float, double><<<blocks_for(n), 256, 0, ctx->stream>>>(L.A64, L.A32, n);
            count_launch(ctx);
            if (mg->p.precision == SMG_F32 && mg->p.tensor_cores && smg_coarse_tc_shape_ok(L.nx, L.ny, L.ndof)) {
                if (!L.Atc) SMG_CUDA(ctx, cudaMalloc(&L.Atc, smg_coarse_tc_link_bytes(L.nsites)));
                SMG_TRY(smg_coarse_tc_tile_links(ctx, L.A64, L.nx, L.nsites, L.Atc));
            }
        }
    }
    SMG_CHECK_LAUNCH(ctx);
    return SMG_OK;
}

smg_status validate(smg_context* ctx, int L, const smg_mg_params* p) {
    if (p->n_levels < 2 || p->n_levels > SMG_MAX_LEVELS)
        return smg_fail(ctx, SMG_BAD_ARG, "n_levels must be in [2, SMG_MAX_LEVELS]");
    int nx = L, ny = L, ndof = 2;
    for (int l = 0; l < p->n_levels - 1; ++l) {
        int ax = p->block[l][0], ay = p->block[l][1];
        if (ax < 1 || ay < 1 || nx % ax || ny % ay)
            return smg_fail(ctx, SMG_BAD_ARG, "aggregate size must divide the level's lattice");
        if (l == 0 && (ax < 2 || ay < 2)) return smg_fail(ctx, SMG_BAD_ARG, "level-0 aggregates must be >= 2 x 2");
        nx /= ax;
        ny /= ay;
        if (nx < 3 || ny < 3) return smg_fail(ctx, SMG_BAD_ARG, "every coarse lattice must be at least 3 x 3");
        int nvec = p->n_vec[l];
        int nc = p->chiral_split ? 2 * nvec : nvec;
        if (nvec < 1 || nc > 64) return smg_fail(ctx, SMG_BAD_ARG, "coarse dofs per site must be in [1, 64]");
        if (nc > ax * ay * ndof) return smg_fail(ctx, SMG_BAD_ARG, "more block vectors than aggregate dofs");
        if (p->chiral_split && l > 0 && (ndof % 2))
            return smg_fail(ctx, SMG_BAD_ARG, "chirality split needs a chirality-split parent level");
        ndof = nc;
    }
    if (p->precision != SMG_F64 && p->precision != SMG_F32)
        return smg_fail(ctx, SMG_BAD_ARG, "MG precision must be F64 or F32");
    if (p->pre_smooth < 0 || p->post_smooth < 0 || p->null_iters < 0 || p->null_mr_steps < 0 ||
        p->coarse_max_iter < 0)
        return smg_fail(ctx, SMG_BAD_ARG, "negative iteration count");
    return SMG_OK;
}

// level-0 block vectors from the null vectors in mg->null0: cut to aggregates (with the chirality
// split when asked) and orthonormalised per aggregate (Prolongator::build_from_vectors,
// src/prolongator.h:133-141)
smg_status block_vectors0(smg_mg* mg) {
    smg_context* ctx = mg->ctx;
    const Geom g = mg->null0[0]->g;
    Level& L = mg->lv[0];
    if (!L.V64) SMG_CUDA(ctx, cudaMalloc(&L.V64, L.vsize() * sizeof(cx<double>)));
    SMG_CUDA(ctx, cudaMemsetAsync(L.V64, 0, L.vsize() * sizeof(cx<double>), ctx->stream));
    for (int k = 0; k < L.nvec; ++k) {
        k_extract0<<<blocks_for(g.V), 256, 0, ctx->stream>>>((const cx<double>*)mg->null0[k]->data, k, g, L.ax, L.ay,
                                                            L.nvec, L.nc_next, mg->p.chiral_split, L.V64);
        count_launch(ctx);
    }
    const int len = L.ax * L.ay * 2, nc = L.nc_next;
    const int nagg = L.nagg_x * L.nagg_y;
    size_t smem = (size_t)len * nc * sizeof(cx<double>);
    if (smem > 200 * 1024) return smg_fail(ctx, SMG_UNSUPPORTED, "aggregate too large for block Gram-Schmidt");
    SMG_CUDA(ctx, cudaFuncSetAttribute(k_block_orth, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    k_block_orth<<<nagg, 128, smem, ctx->stream>>>(L.V64, len, nc);
    count_launch(ctx);
    SMG_CHECK_LAUNCH(ctx);
    return SMG_OK;
}

// the level-1 Galerkin operator A_1 = P^dag D^dag D P from the level-0 block vectors: W = D P on
// the block halos, then the 9 blocks of every coarse site
smg_status galerkin0(smg_mg* mg) {
    smg_context* ctx = mg->ctx;
    smg_dirac* d = mg->dirac;
    const Geom g = d->gauge->g;
    const Level& L = mg->lv[0];
    const int nc = L.nc_next, nagg = L.nagg_x * L.nagg_y;
    const int nh = (L.ax + 2) * (L.ay + 2);
    cx<double>* W = nullptr;
    SMG_CUDA(ctx, cudaMallocAsync(&W, (size_t)nagg * nc * nh * 2 * sizeof(cx<double>), ctx->stream));
    k_W0<<<nagg, 256, 0, ctx->stream>>>(L.V64, d->gauge->U64, d->C64, g, L.ax, L.ay, nc, 2.0 * d->r + d->mass,
                                       d->mu_t, d->r, W);
    count_launch(ctx);
    Level& N = mg->lv[1];
    if (!N.A64) SMG_CUDA(ctx, cudaMalloc(&N.A64, N.asize() * sizeof(cx<double>)));
    k_galerkin0<<<dim3(nagg, 9), 256, 0, ctx->stream>>>(W, L.nagg_x, L.nagg_y, L.ax, L.ay, nc, N.A64);
    count_launch(ctx);
    SMG_CHECK_LAUNCH(ctx);
    SMG_CUDA(ctx, cudaFreeAsync(W, ctx->stream));
    return SMG_OK;
}

// level geometry of a hierarchy from its parameters and the fine lattice size
void set_geometry(smg_mg* mg, int Lfine) {
    const smg_mg_params& P = mg->p;
    const int nlev = P.n_levels;
    mg->lv.resize(nlev);
    mg->lv[0].nx = mg->lv[0].ny = Lfine;
    mg->lv[0].nsites = Lfine * Lfine;
    mg->lv[0].ndof = 2;
    for (int l = 0; l < nlev - 1; ++l) {
        Level& L = mg->lv[l];
        L.ax = P.block[l][0];
        L.ay = P.block[l][1];
        L.nvec = P.n_vec[l];
        L.nc_next = P.chiral_split ? 2 * L.nvec : L.nvec;
        L.nagg_x = L.nx / L.ax;
        L.nagg_y = L.ny / L.ay;
        Level& N = mg->lv[l + 1];
        N.nx = L.nagg_x;
        N.ny = L.nagg_y;
        N.nsites = N.nx * N.ny;
        N.ndof = L.nc_next;
    }
}

smg_status build(smg_mg* mg, const double* warm) {
    smg_context* ctx = mg->ctx;
    const smg_mg_params& P = mg->p;
    const Geom g = mg->dirac->gauge->g;
    const int nlev = P.n_levels;
    set_geometry(mg, g.L);
    std::mt19937 rng(P.seed);
    std::normal_distribution<double> dist(0.0, 1.0);
    auto draw = [&](int64_t n, std::vector<double>& h) {  // random_vec order (linalg.cpp:44-48, GCC x86-64)
        h.resize(2 * n);
        for (int64_t i = 0; i < n; ++i) {
            double im = dist(rng);
            double re = dist(rng);
            h[2 * i] = re;
            h[2 * i + 1] = im;
        }
    };
    // ---- level 0 null vectors
    const Level& L0 = mg->lv[0];
    const int k0 = L0.nvec;
    std::vector<double> h;
    for (int i = 0; i < k0; ++i) {
        smg_field* f = nullptr;
        SMG_TRY(smg_field_create(ctx, g.L, 1, SMG_F64, &f));
        mg->null0.push_back(f);
        if (warm) {
            SMG_TRY(smg_field_upload(f, warm + (size_t)4 * g.V * i));
        } else if (mg->starts && mg->starts[0]) {
            SMG_TRY(smg_field_upload(f, mg->starts[0] + (size_t)4 * g.V * i));
        } else {
            draw((int64_t)2 * g.V, h);
            SMG_TRY(smg_field_upload(f, h.data()));
        }
    }
    SMG_TRY(null_space_fine(mg, mg->null0));
    // ---- level 0 prolongator and Galerkin operator
    SMG_TRY(block_vectors0(mg));
    SMG_TRY(galerkin0(mg));
    // ---- deeper levels
    for (int l = 1; l < nlev - 1; ++l) {
        Level& L = mg->lv[l];
        const int dim = L.nsites * L.ndof;
        std::vector<cx<double>*> vecs(L.nvec, nullptr);
        for (int i = 0; i < L.nvec; ++i) {
            SMG_CUDA(ctx, cudaMalloc(&vecs[i], (size_t)dim * sizeof(cx<double>)));
            const double* src = nullptr;
            if (mg->starts && mg->starts[l]) {
                src = mg->starts[l] + (size_t)2 * dim * i;
            } else {
                draw(dim, h);
                src = h.data();
            }
            SMG_CUDA(ctx, cudaMemcpy(vecs[i], src, (size_t)dim * sizeof(cx<double>), cudaMemcpyHostToDevice));
        }
        smg_status st = null_space_coarse(mg, l, vecs);
        if (st == SMG_OK) {
            SMG_CUDA(ctx, cudaMalloc(&L.V64, L.vsize() * sizeof(cx<double>)));
            SMG_CUDA(ctx, cudaMemsetAsync(L.V64, 0, L.vsize() * sizeof(cx<double>), ctx->stream));
            for (int k = 0; k < L.nvec; ++k) {
                k_extract_c<<<blocks_for(dim), 256, 0, ctx->stream>>>(vecs[k], k, L.nx, L.ny, L.ndof, L.ax, L.ay,
                                                                     L.nvec, L.nc_next, P.chiral_split, L.V64);
                count_launch(ctx);
            }
            const int len = L.ax * L.ay * L.ndof, nc = L.nc_next, nagg = L.nagg_x * L.nagg_y;
            size_t smem = (size_t)len * nc * sizeof(cx<double>);
            if (smem > 200 * 1024) st = smg_fail(ctx, SMG_UNSUPPORTED, "aggregate too large for block Gram-Schmidt");
            if (st == SMG_OK) {
                cudaFuncSetAttribute(k_block_orth, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
                k_block_orth<<<nagg, 128, smem, ctx->stream>>>(L.V64, len, nc);
                count_launch(ctx);
                Level& N = mg->lv[l + 1];
                SMG_CUDA(ctx, cudaMalloc(&N.A64, N.asize() * sizeof(cx<double>)));
                size_t sm2 = (size_t)L.ndof * nc * sizeof(cx<double>);
                int threads = 256;
                while (threads * 4 < nc * nc) threads *= 2;
                cudaFuncSetAttribute(k_galerkin_c, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm2);
                k_galerkin_c<<<nagg, threads, sm2, ctx->stream>>>(L.A64, L.V64, L.nx, L.ny, L.ax, L.ay, L.ndof, nc,
                                                                  N.A64);
                count_launch(ctx);
                SMG_CHECK_LAUNCH(ctx);
            }
        }
        cudaStreamSynchronize(ctx->stream);
        for (auto* p : vecs) cudaFree(p);
        SMG_TRY(st);
    }
    SMG_TRY(make_f32_copies(mg));
    SMG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return SMG_OK;
}

// The Galerkin operators of every level recomputed from the current links with the existing
// prolongators (MGHierarchy::rebuild_deeper_levels with the level-0 rebuild it assumes,
// src/multigrid.cpp:158-193); the FP32 and tensor-core copies are refreshed in place, so a captured
// cycle stays valid.
smg_status rebuild_operators(smg_mg* mg) {
    smg_context* ctx = mg->ctx;
    const int nlev = (int)mg->lv.size();
    SMG_TRY(galerkin0(mg));
    for (int l = 1; l < nlev - 1; ++l) {
        Level& L = mg->lv[l];
        const int nc = L.nc_next, nagg = L.nagg_x * L.nagg_y;
        const size_t sm2 = (size_t)L.ndof * nc * sizeof(cx<double>);
        int threads = 256;
        while (threads * 4 < nc * nc) threads *= 2;
        SMG_CUDA(ctx, cudaFuncSetAttribute(k_galerkin_c, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm2));
        k_galerkin_c<<<nagg, threads, sm2, ctx->stream>>>(L.A64, L.V64, L.nx, L.ny, L.ax, L.ay, L.ndof, nc,
                                                          mg->lv[l + 1].A64);
        count_launch(ctx);
        SMG_CHECK_LAUNCH(ctx);
    }
    SMG_TRY(make_f32_copies(mg));
    SMG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return SMG_OK;
}

void destroy_levels(smg_mg* mg) {
    for (auto& L : mg->lv) {
        for (void* p : {(void*)L.V64, (void*)L.V32, (void*)L.V32s, (void*)L.V32o, (void*)L.A64, (void*)L.A32, L.Atc})
            if (p) cudaFree(p);
    }
    mg->lv.clear();
    for (auto* f : mg->null0) smg_field_destroy(f);
    mg->null0.clear();
}

}  // namespace

namespace {

// The captured cycle goes; its input and output fields stay (a solver may hold them as its own
// residual and preconditioned vector, smg_mg_graph_io) until the hierarchy goes or the shape changes.
void drop_graph(smg_mg* mg) {
    if (mg->g_exec) cudaGraphExecDestroy(mg->g_exec);
    mg->g_exec = nullptr;
}
void free_graph_io(smg_mg* mg) {
    smg_field_destroy(mg->g_in);
    smg_field_destroy(mg->g_out);
    mg->g_in = mg->g_out = nullptr;
}

// One cycle from mg->g_in to mg->g_out captured as a CUDA graph.  The
// coarsest CG runs its full iteration budget inside the graph; its kernels
// return at once after every right-hand side has converged.
template <typename T>
smg_status capture_cycle(smg_mg* mg, const smg_field* proto) {
    smg_context* ctx = mg->ctx;
    drop_graph(mg);
    SMG_TRY(ensure_work(mg, proto->nrhs, proto->prec));
    const bool keep_io = mg->g_in && mg->g_out && mg->g_in->g.L == proto->g.L && mg->g_in->nrhs == proto->nrhs &&
                         mg->g_in->prec == proto->prec;
    if (!keep_io) {
        free_graph_io(mg);
        SMG_TRY(smg_field_alloc_like(proto, proto->prec, &mg->g_in));
        SMG_TRY(smg_field_alloc_like(proto, proto->prec, &mg->g_out));
    }
    SMG_TRY(smg_reduce_reserve(ctx, (size_t)kMaxReduceBlocks * proto->nrhs * 3 + 1024));
    SMG_TRY(smg_host_stage_reserve(ctx, 64));
    SMG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    const uint64_t l0 = ctx->launches;
    cudaGraph_t graph = nullptr;
    mg->capturing = true;
    SMG_CUDA(ctx, cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
    smg_status st = cycle_fine<T>(mg, mg->g_out, mg->g_in);
    cudaError_t e = cudaStreamEndCapture(ctx->stream, &graph);
    mg->capturing = false;
    mg->g_launches = ctx->launches - l0;
    ctx->launches = l0;
    if (st != SMG_OK) {
        if (graph) cudaGraphDestroy(graph);
        return st;
    }
    if (e != cudaSuccess || !graph)
        return smg_fail(ctx, SMG_DEVICE_ERROR, std::string("cycle capture: ") + cudaGetErrorString(e));
    e = cudaGraphInstantiate(&mg->g_exec, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) {
        mg->g_exec = nullptr;
        return smg_fail(ctx, SMG_DEVICE_ERROR, std::string("cycle graph: ") + cudaGetErrorString(e));
    }
    mg->g_work_gen = mg->work_gen;
    return SMG_OK;
}

template <typename T>
smg_status cycle_graph(smg_mg* mg, const smg_field* b, smg_field* x) {
    smg_context* ctx = mg->ctx;
    const bool stale = !mg->g_exec || !mg->g_in || mg->g_in->nrhs != b->nrhs || mg->g_in->prec != b->prec ||
                       mg->work_nrhs != b->nrhs || mg->work_prec != b->prec || mg->g_work_gen != mg->work_gen;
    if (stale) SMG_TRY(capture_cycle<T>(mg, b));
    // a caller that holds the graph's own input and output fields (smg_mg_graph_io) needs no copies
    if (b != mg->g_in)
        SMG_CUDA(ctx, cudaMemcpyAsync(mg->g_in->data, b->data, b->bytes, cudaMemcpyDeviceToDevice, ctx->stream));
    SMG_CUDA(ctx, cudaGraphLaunch(mg->g_exec, ctx->stream));
    ctx->launches += mg->g_launches;
    if (x != mg->g_out)
        SMG_CUDA(ctx, cudaMemcpyAsync(x->data, mg->g_out->data, x->bytes, cudaMemcpyDeviceToDevice, ctx->stream));
    return SMG_OK;
}

}  // namespace

// ---- internal entries used by the GCR solver
// The captured cycle's input and output fields for right-hand sides shaped like proto (capturing the
// cycle first if needed), or null when the hierarchy runs its cycle without a graph: a solver that
// keeps its residual in *in and its preconditioned vector in *out saves two field copies per cycle.
// They stay valid until the hierarchy is destroyed or runs a cycle of another shape or precision.
smg_status smg_mg_graph_io(smg_mg* mg, const smg_field* proto, smg_field** in, smg_field** out) {
    *in = *out = nullptr;
    if (!mg->use_graph || (proto->prec != SMG_F64 && proto->prec != SMG_F32)) return SMG_OK;
    const bool stale = !mg->g_exec || !mg->g_in || mg->g_in->nrhs != proto->nrhs || mg->g_in->prec != proto->prec ||
                       mg->g_in->g.L != proto->g.L || mg->work_nrhs != proto->nrhs || mg->work_prec != proto->prec ||
                       mg->g_work_gen != mg->work_gen;
    if (stale) {
        const smg_status st =
            proto->prec == SMG_F64 ? capture_cycle<double>(mg, proto) : capture_cycle<float>(mg, proto);
        if (st != SMG_OK) {
            if (st != SMG_DEVICE_ERROR || mg->g_exec) return st;
            cudaGetLastError();  // capture failed: the cycle runs kernel by kernel
            drop_graph(mg);
            mg->use_graph = false;
            return SMG_OK;
        }
    }
    *in = mg->g_in;
    *out = mg->g_out;
    return SMG_OK;
}

smg_status smg_mg_apply_internal(smg_mg* mg, const smg_field* b, smg_field* x) {
    if (b->prec != SMG_F64 && b->prec != SMG_F32)
        return smg_fail(mg->ctx, SMG_UNSUPPORTED, "MG cycle on F16 fields");
    if (mg->use_graph) {
        smg_status st = b->prec == SMG_F64 ? cycle_graph<double>(mg, b, x) : cycle_graph<float>(mg, b, x);
        if (st != SMG_DEVICE_ERROR || mg->g_exec) return st;
        // capture or instantiation failed: run the cycle with direct launches from now on
        cudaGetLastError();
        drop_graph(mg);
        mg->use_graph = false;
    }
    SMG_TRY(ensure_work(mg, b->nrhs, b->prec));
    if (b->prec == SMG_F64) return cycle_fine<double>(mg, x, b);
    return cycle_fine<float>(mg, x, b);
}

smg_precision smg_mg_precision(const smg_mg* mg) { return mg->p.precision; }

// The grid-barrier coarsest CG needs every block of its grid resident at once,
// which kernels of other streams on the same GPU can prevent; a hierarchy
// shared with concurrent streams uses the host-checked CG instead.
void smg_mg_set_persistent_internal(smg_mg* mg, bool on) { mg->persistent = on; }

smg_status smg_mg_level0_L(const smg_mg* mg, int* L) {
    *L = mg->lv[0].nx;
    return SMG_OK;
}

namespace {

// estimate_lambda_max (src/smoother.cpp:43-60) of the level-l operator in
// FP64: niter power steps from random_vec(dim, std::mt19937(12345)), with
// lambda = ||A v|| of the last step.  Level-l vectors use the reference's
// dof order (fine: 2 * site + spin, coarse: site * ndof + j).
smg_status lambda_max_level(smg_mg* mg, int l, int niter, double* out) {
    smg_context* ctx = mg->ctx;
    SMG_TRY(ensure_work(mg, 1, SMG_F64));
    const Level& L = mg->lv[l];
    const int64_t dim = (int64_t)L.nsites * L.ndof;
    std::vector<double> h(2 * dim);
    SMG_TRY(smg_host_random_vec(dim, 12345u, h.data()));
    double* sc = lvl_scal(mg, l);
    SMG_TRY(smg_host_stage_reserve(ctx, 64));
    VecView<double> v, Av;
    smg_field* fv0 = mg->f_r;
    smg_field* fAv = mg->f_Ar;
    if (l == 0) {
        SMG_TRY(smg_field_upload(fv0, h.data()));
        v = flat(fview<double>(fv0));
        Av = flat(fview<double>(fAv));
    } else {
        CoarseWork& w = mg->cw[l];
        SMG_CUDA(ctx, cudaMemcpyAsync(w.x, h.data(), h.size() * sizeof(double), cudaMemcpyHostToDevice,
                                      ctx->stream));
        v = flat(cview<double>(w.x, L, 1));
        Av = flat(cview<double>(w.Ar, L, 1));
    }
    auto scale_into = [&](VecView<double> dst, const cx<double>* src) {
        k_vconvert_scaled<double, double><<<vec_grid(dst.nsites, 1), vec_block(1), 0, ctx->stream>>>(dst, src, sc,
                                                                                                    1);
        count_launch(ctx);
    };
    SMG_TRY(vreduce<double>(ctx, v, nullptr, VR_NORM, sc));
    scale_into(v, v.p);
    double lam = 0;
    for (int i = 0; i < niter; ++i) {
        if (l == 0)
            SMG_TRY(level_apply_fine<double>(mg, fv0, fAv, nullptr, nullptr));
        else
            SMG_TRY(coarse_apply<double>(mg, l, cview<double>(v.p, L, 1), Av.p, 0, nullptr, nullptr));
        SMG_TRY(vreduce<double>(ctx, Av, nullptr, VR_NORM, sc));
        SMG_CUDA(ctx, cudaMemcpyAsync(ctx->host_stage, sc, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
        SMG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        lam = std::sqrt(ctx->host_stage[0]);
        if (lam < 1e-30) break;
        scale_into(v, Av.p);
    }
    SMG_CHECK_LAUNCH(ctx);
    *out = lam;
    return SMG_OK;
}

}  // namespace

// Reads (and clears) the persistent coarsest CG's error flag: SMG_TIMEOUT if a
// bounded grid-barrier wait ran out since the last check.  Synchronises.
smg_status smg_mg_check_device_error(smg_mg* mg) {
    if (!mg->cg_state) return SMG_OK;
    smg_context* ctx = mg->ctx;
    int err = 0;
    SMG_CUDA(ctx, cudaMemcpyAsync(&err, static_cast<char*>(mg->cg_state) + 8, sizeof(int), cudaMemcpyDeviceToHost,
                                  ctx->stream));
    SMG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if (err) {
        SMG_CUDA(ctx, cudaMemsetAsync(static_cast<char*>(mg->cg_state) + 8, 0, sizeof(int), ctx->stream));
        return smg_fail(ctx, SMG_TIMEOUT,
                        err == 2 ? "tensor-core coarse apply: a pipeline wait ran out"
                                 : "coarsest CG: a grid-barrier wait ran out");
    }
    return SMG_OK;
}

// ------------------------------------------------------------ level-1 helpers for deflation.cu

MgDeflation& smg_mg_defl(smg_mg* mg) { return mg->defl; }
smg_context* smg_mg_ctx(smg_mg* mg) { return mg->ctx; }
smg_dirac* smg_mg_dirac(smg_mg* mg) { return mg->dirac; }
int smg_mg_nlevels(const smg_mg* mg) { return (int)mg->lv.size(); }
int64_t smg_mg_level_dim(const smg_mg* mg, int l) { return (int64_t)mg->lv[l].nsites * mg->lv[l].ndof; }
void smg_mg_drop_cycle_graph(smg_mg* mg) {
    cudaStreamSynchronize(mg->ctx->stream);
    drop_graph(mg);
}

smg_status smg_mg_apply_f64(smg_mg* mg, int l, const cx<double>* x, cx<double>* y) {
    return coarse_apply<double>(mg, l, cview<double>((void*)x, mg->lv[l], 1), y, 0, nullptr, nullptr);
}

smg_status smg_mg_restrict0_f64(smg_mg* mg, const smg_field* fine, cx<double>* coarse) {
    smg_context* ctx = mg->ctx;
    const Level& L = mg->lv[0];
    const int64_t total = (int64_t)mg->lv[1].nsites * L.nc_next;
    k_restrict0<double><<<blocks_for(total), 256, 0, ctx->stream>>>(L.V64, (const cx<double>*)fine->data, coarse,
                                                                   mg->null0[0]->g, L.ax, L.ay, L.nc_next, 1);
    count_launch(ctx);
    SMG_CHECK_LAUNCH(ctx);
    return SMG_OK;
}

smg_status smg_mg_prolong0_f64(smg_mg* mg, const cx<double>* coarse, smg_field* fine) {
    smg_context* ctx = mg->ctx;
    const Level& L = mg->lv[0];
    const Geom g = mg->null0[0]->g;
    k_prolong0<double><<<blocks_for((int64_t)g.V), 256, 0, ctx->stream>>>(L.V64, coarse, (cx<double>*)fine->data, g,
                                                                         L.ax, L.ay, L.nc_next, 1, 0);
    count_launch(ctx);
    SMG_CHECK_LAUNCH(ctx);
    return SMG_OK;
}

extern "C" {

SMG_API smg_status smg_mg_params_default(smg_mg_params* p) {
    if (!p) return SMG_BAD_ARG;
    std::memset(p, 0, sizeof(*p));
    p->n_levels = 2;
    for (int l = 0; l < SMG_MAX_LEVELS - 1; ++l) {
        p->block[l][0] = l == 0 ? 4 : 4;
        p->block[l][1] = l == 0 ? 4 : 1;
        p->n_vec[l] = 4;
    }
    p->chiral_split = 0;
    p->null_iters = 20;
    p->null_mr_steps = 5;
    p->pre_smooth = 3;
    p->post_smooth = 3;
    p->w_cycle = 1;
    p->coarse_max_iter = 200;
    p->coarse_tol = 1e-12;
    p->precision = SMG_F64;
    p->seed = 42;
    p->tensor_cores = 1;
    return SMG_OK;
}

SMG_API smg_status smg_mg_create(smg_dirac* d, const smg_mg_params* p, const double* warm_start, smg_mg** out) {
    if (!d || !p || !out) return SMG_BAD_ARG;
    *out = nullptr;
    smg_context* ctx = d->ctx;
    SMG_TRY(validate(ctx, d->gauge->g.L, p));
    smg_mg* mg = new smg_mg();
    mg->ctx = ctx;
    mg->dirac = d;
    mg->p = *p;
    // SMG_CUDA_GRAPHS=0 launches the cycle kernel by kernel (for tools that cannot follow graph replays)
    if (const char* e = std::getenv("SMG_CUDA_GRAPHS")) mg->use_graph = std::atoi(e) != 0;
    smg_status st = build(mg, warm_start);
    if (st != SMG_OK) {
        cudaStreamSynchronize(ctx->stream);
        free_work(mg);
        destroy_levels(mg);
        delete mg;
        return st;
    }
    *out = mg;
    return SMG_OK;
}

SMG_API smg_status smg_mg_create_from_starts(smg_dirac* d, const smg_mg_params* p, const double* const* start_vecs,
                                             smg_mg** out) {
    if (!d || !p || !out || !start_vecs) return SMG_BAD_ARG;
    *out = nullptr;
    smg_context* ctx = d->ctx;
    SMG_TRY(validate(ctx, d->gauge->g.L, p));
    for (int l = 0; l < p->n_levels - 1; ++l)
        if (!start_vecs[l]) return smg_fail(ctx, SMG_BAD_ARG, "start vectors missing for a level");
    smg_mg* mg = new smg_mg();
    mg->ctx = ctx;
    mg->dirac = d;
    mg->p = *p;
    if (const char* e = std::getenv("SMG_CUDA_GRAPHS")) mg->use_graph = std::atoi(e) != 0;
    mg->starts = start_vecs;
    smg_status st = build(mg, nullptr);
    mg->starts = nullptr;
    if (st != SMG_OK) {
        cudaStreamSynchronize(ctx->stream);
        free_work(mg);
        destroy_levels(mg);
        delete mg;
        return st;
    }
    *out = mg;
    return SMG_OK;
}

// ---- standalone prolongator and coarse operator (Prolongator, src/prolongator.h:14-142, and
// SparseCoarseOp, src/coarse_op.h:154-548): each holds a two-level hierarchy shell whose level 0
// carries the block vectors (and, for the coarse operator, level 1 the Galerkin operator)
struct smg_prolongator {
    smg_mg* mg = nullptr;
};
struct smg_coarse_op {
    smg_mg* mg = nullptr;
};

namespace {
smg_mg* shell_mg(smg_context* ctx, smg_dirac* d, int L, int bx, int by, int k) {
    smg_mg* mg = new smg_mg();
    mg->ctx = ctx;
    mg->dirac = d;
    smg_mg_params_default(&mg->p);
    mg->p.n_levels = 2;
    mg->p.block[0][0] = bx;
    mg->p.block[0][1] = by;
    mg->p.n_vec[0] = k;
    mg->p.null_iters = 0;
    mg->p.w_cycle = 0;
    mg->p.precision = SMG_F64;
    mg->p.tensor_cores = 0;
    mg->use_graph = false;
    mg->persistent = false;
    set_geometry(mg, L);
    return mg;
}
}  // namespace

SMG_API smg_status smg_prolongator_create(smg_context* ctx, int L, int bx, int by, int k, const double* null_vecs,
                                          smg_prolongator** out) {
    if (!ctx || !null_vecs || !out) return SMG_BAD_ARG;
    *out = nullptr;
    if (L < 2 || (L & 1) || bx < 2 || by < 2 || L % bx || L % by || L / bx < 3 || L / by < 3)
        return smg_fail(ctx, SMG_BAD_ARG, "prolongator: blocks must divide L into at least 3 x 3 blocks");
    if (k < 1 || k > 64 || k > 2 * bx * by) return smg_fail(ctx, SMG_BAD_ARG, "prolongator: k in [1, min(64, 2 bx by)]");
    smg_mg* mg = shell_mg(ctx, nullptr, L, bx, by, k);
    smg_status st = SMG_OK;
    for (int i = 0; i < k && st == SMG_OK; ++i) {
        smg_field* f = nullptr;
        st = smg_field_create(ctx, L, 1, SMG_F64, &f);
        if (st == SMG_OK) {
            mg->null0.push_back(f);
            st = smg_field_upload(f, null_vecs + (size_t)4 * L * L * i);
        }
    }
    if (st == SMG_OK) st = block_vectors0(mg);
    if (st == SMG_OK) st = cudaStreamSynchronize(ctx->stream) == cudaSuccess ? SMG_OK : SMG_DEVICE_ERROR;
    if (st != SMG_OK) {
        smg_mg_destroy(mg);
        return st;
    }
    *out = new smg_prolongator{mg};
    return SMG_OK;
}

SMG_API smg_status smg_prolongator_destroy(smg_prolongator* P) {
    if (!P) return SMG_OK;
    smg_mg_destroy(P->mg);
    delete P;
    return SMG_OK;
}

SMG_API smg_status smg_prolongator_get_block_vecs(smg_prolongator* P, double* block_vecs) {
    if (!P) return SMG_BAD_ARG;
    return smg_mg_get_prolongator(P->mg, 0, block_vecs);
}

SMG_API smg_status smg_prolongator_prolong(smg_prolongator* P, const double* coarse, double* fine) {
    if (!P) return SMG_BAD_ARG;
    return smg_mg_prolong_host(P->mg, 0, coarse, fine);
}

SMG_API smg_status smg_prolongator_restrict(smg_prolongator* P, const double* fine, double* coarse) {
    if (!P) return SMG_BAD_ARG;
    return smg_mg_restrict_host(P->mg, 0, fine, coarse);
}

SMG_API smg_status smg_coarse_op_create(const smg_prolongator* P, smg_dirac* d, smg_coarse_op** out) {
    if (!P || !d || !out) return SMG_BAD_ARG;
    *out = nullptr;
    const smg_mg* pm = P->mg;
    smg_context* ctx = pm->ctx;
    if (d->ctx != ctx) return smg_fail(ctx, SMG_BAD_ARG, "coarse operator: prolongator and operator contexts differ");
    if (d->gauge->g.L != pm->lv[0].nx) return smg_fail(ctx, SMG_BAD_ARG, "coarse operator: lattice sizes differ");
    const Level& L0 = pm->lv[0];
    smg_mg* mg = shell_mg(ctx, d, L0.nx, L0.ax, L0.ay, L0.nvec);
    smg_status st = SMG_OK;
    Level& L = mg->lv[0];
    const size_t vb = (size_t)L.vsize() * sizeof(cx<double>);
    if (cudaMalloc(&L.V64, vb) != cudaSuccess) st = smg_fail(ctx, SMG_DEVICE_ERROR, "cudaMalloc");
    if (st == SMG_OK && cudaMemcpyAsync(L.V64, L0.V64, vb, cudaMemcpyDeviceToDevice, ctx->stream) != cudaSuccess)
        st = smg_fail(ctx, SMG_DEVICE_ERROR, "cudaMemcpyAsync");
    if (st == SMG_OK) {  // transfers need a level-0 geometry field
        smg_field* f = nullptr;
        st = smg_field_create(ctx, L.nx, 1, SMG_F64, &f);
        if (st == SMG_OK) mg->null0.push_back(f);
    }
    if (st == SMG_OK) st = galerkin0(mg);
    if (st == SMG_OK) st = cudaStreamSynchronize(ctx->stream) == cudaSuccess ? SMG_OK : SMG_DEVICE_ERROR;
    if (st != SMG_OK) {
        smg_mg_destroy(mg);
        return st;
    }
    *out = new smg_coarse_op{mg};
    return SMG_OK;
}

SMG_API smg_status smg_coarse_op_destroy(smg_coarse_op* A) {
    if (!A) return SMG_OK;
    smg_mg_destroy(A->mg);
    delete A;
    return SMG_OK;
}

SMG_API smg_status smg_coarse_op_dims(smg_coarse_op* A, int* nbx, int* nby, int* k) {
    if (!A) return SMG_BAD_ARG;
    return smg_mg_level_dims(A->mg, 1, nbx, nby, k);
}

SMG_API smg_status smg_coarse_op_get_links(smg_coarse_op* A, double* links) {
    if (!A) return SMG_BAD_ARG;
    return smg_mg_get_coarse_op(A->mg, 1, links);
}

SMG_API smg_status smg_coarse_op_apply(smg_coarse_op* A, const double* in, double* out) {
    if (!A) return SMG_BAD_ARG;
    return smg_mg_coarse_apply_host(A->mg, 1, in, out);
}

SMG_API smg_status smg_coarse_op_solve(smg_coarse_op* A, const double* b, double* x, int max_iter, double tol) {
    if (!A || !b || !x || max_iter < 0 || !(tol > 0)) return SMG_BAD_ARG;
    smg_mg* mg = A->mg;
    smg_context* ctx = mg->ctx;
    SMG_TRY(ensure_work(mg, 1, SMG_F64));
    const Level& L = mg->lv[1];
    CoarseWork& w = mg->cw[1];
    const size_t nb = (size_t)L.nsites * L.ndof * sizeof(cx<double>);
    mg->p.coarse_max_iter = max_iter;
    mg->p.coarse_tol = tol;
    SMG_CUDA(ctx, cudaMemcpyAsync(w.b, b, nb, cudaMemcpyHostToDevice, ctx->stream));
    SMG_TRY(coarse_cg<double>(mg, 1, w.x, w.b));
    SMG_CUDA(ctx, cudaMemcpyAsync(x, w.x, nb, cudaMemcpyDeviceToHost, ctx->stream));
    SMG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return smg_mg_check_device_error(mg);
}

SMG_API smg_status smg_coarse_op_setup_deflation(smg_coarse_op* A, int n_ev, int n_kr, int max_restarts, double tol,
                                                 smg_deflation_info* info) {
    if (!A) return SMG_BAD_ARG;
    return smg_mg_setup_deflation(A->mg, n_ev, n_kr, max_restarts, tol, info);
}

SMG_API smg_status smg_mg_destroy(smg_mg* mg) {
    if (!mg) return SMG_OK;
    cudaStreamSynchronize(mg->ctx->stream);
    drop_graph(mg);
    free_graph_io(mg);
    free_work(mg);
    destroy_levels(mg);
    smg_defl_free(mg->defl);
    delete mg;
    return SMG_OK;
}

SMG_API smg_status smg_mg_level_dims(smg_mg* mg, int level, int* nx, int* ny, int* ndof) {
    if (!mg || level < 0 || level >= (int)mg->lv.size()) return SMG_BAD_ARG;
    if (nx) *nx = mg->lv[level].nx;
    if (ny) *ny = mg->lv[level].ny;
    if (ndof) *ndof = mg->lv[level].ndof;
    return SMG_OK;
}

SMG_API smg_status smg_mg_null_vectors(smg_mg* mg, double* out) {
    if (!mg || !out) return SMG_BAD_ARG;
    const size_t per = (size_t)4 * mg->lv[0].nsites;
    for (size_t i = 0; i < mg->null0.size(); ++i) SMG_TRY(smg_field_download(mg->null0[i], out + per * i));
    return SMG_OK;
}

SMG_API smg_status smg_mg_set_wait_limit(smg_mg* mg, long long spins) {
    if (!mg) return SMG_BAD_ARG;
    mg->spin_limit = spins < 0 ? kBarrierSpinLimit : spins;
    drop_graph(mg);  // a captured cycle holds the old bound in its kernel arguments
    return SMG_OK;
}

SMG_API smg_status smg_mg_n_null_vectors(smg_mg* mg, int* k) {
    if (!mg || !k) return SMG_BAD_ARG;
    *k = (int)mg->null0.size();
    return SMG_OK;
}

SMG_API smg_status smg_mg_get_prolongator(smg_mg* mg, int level, double* block_vecs) {
    if (!mg || !block_vecs || level < 0 || level >= (int)mg->lv.size() - 1) return SMG_BAD_ARG;
    smg_context* ctx = mg->ctx;
    const Level& L = mg->lv[level];
    const int64_t n = L.vsize();
    std::vector<std::complex<double>> h(n);
    SMG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    SMG_CUDA(ctx, cudaMemcpy(h.data(), L.V64, n * sizeof(cx<double>), cudaMemcpyDeviceToHost));
    // device [agg][loc][dof][i] -> reference [agg][i][loc * dof_per_site + dof]
    const int m = L.ax * L.ay, nd = L.ndof, nc = L.nc_next, nagg = L.nagg_x * L.nagg_y;
    auto* o = reinterpret_cast<std::complex<double>*>(block_vecs);
    for (int B = 0; B < nagg; ++B)
        for (int loc = 0; loc < m; ++loc)
            for (int j = 0; j < nd; ++j)
                for (int i = 0; i < nc; ++i)
                    o[((int64_t)B * nc + i) * m * nd + loc * nd + j] = h[(((int64_t)B * m + loc) * nd + j) * nc + i];
    return SMG_OK;
}

SMG_API smg_status smg_mg_get_coarse_op(smg_mg* mg, int level, double* links) {
    if (!mg || !links || level < 1 || level >= (int)mg->lv.size()) return SMG_BAD_ARG;
    smg_context* ctx = mg->ctx;
    const Level& L = mg->lv[level];
    const int64_t n = L.asize();
    std::vector<std::complex<double>> h(n);
    SMG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    SMG_CUDA(ctx, cudaMemcpy(h.data(), L.A64, n * sizeof(cx<double>), cudaMemcpyDeviceToHost));
    const int nc = L.ndof;
    auto* o = reinterpret_cast<std::complex<double>*>(links);
    for (int64_t sd = 0; sd < (int64_t)L.nsites * 9; ++sd)
        for (int i = 0; i < nc; ++i)
            for (int j = 0; j < nc; ++j) o[sd * nc * nc + i * nc + j] = h[sd * nc * nc + j * nc + i];
    return SMG_OK;
}

SMG_API smg_status smg_mg_precondition(smg_mg* mg, const smg_field* b, smg_field* x) {
    if (!mg || !b || !x) return SMG_BAD_ARG;
    SMG_TRY(smg_field_check_pair(b, x));
    if (b == x) return smg_fail(mg->ctx, SMG_BAD_ARG, "b and x must be distinct");
    if (b->g.L != mg->lv[0].nx) return smg_fail(mg->ctx, SMG_BAD_ARG, "field L differs from the hierarchy's");
    SMG_TRY(smg_mg_apply_internal(mg, b, x));
    return smg_mg_check_device_error(mg);
}

SMG_API smg_status smg_mg_prolong_host(smg_mg* mg, int level, const double* coarse, double* fine) {
    if (!mg || !coarse || !fine || level < 0 || level >= (int)mg->lv.size() - 1) return SMG_BAD_ARG;
    smg_context* ctx = mg->ctx;
    SMG_TRY(ensure_work(mg, 1, SMG_F64));
    const Level& L = mg->lv[level];
    const Level& N = mg->lv[level + 1];
    CoarseWork& nw = mg->cw[level + 1];
    const size_t cb = (size_t)N.nsites * N.ndof * sizeof(cx<double>);
    SMG_CUDA(ctx, cudaMemcpyAsync(nw.x, coarse, cb, cudaMemcpyHostToDevice, ctx->stream));
    if (level == 0) {
        SMG_TRY(prolong_to<double>(mg, 0, nw.x, mg->f_t->data, 0));
        return smg_field_download(mg->f_t, fine);
    }
    SMG_TRY(prolong_to<double>(mg, level, nw.x, mg->cw[level].x, 0));
    const size_t fb = (size_t)L.nsites * L.ndof * sizeof(cx<double>);
    SMG_CUDA(ctx, cudaMemcpyAsync(fine, mg->cw[level].x, fb, cudaMemcpyDeviceToHost, ctx->stream));
    SMG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return SMG_OK;
}

SMG_API smg_status smg_mg_restrict_host(smg_mg* mg, int level, const double* fine, double* coarse) {
    if (!mg || !coarse || !fine || level < 0 || level >= (int)mg->lv.size() - 1) return SMG_BAD_ARG;
    smg_context* ctx = mg->ctx;
    SMG_TRY(ensure_work(mg, 1, SMG_F64));
    const Level& L = mg->lv[level];
    const Level& N = mg->lv[level + 1];
    CoarseWork& nw = mg->cw[level + 1];
    if (level == 0) {
        SMG_TRY(smg_field_upload(mg->f_t, fine));
        SMG_TRY(restrict_to<double>(mg, 0, mg->f_t->data, nw.b));
    } else {
        const size_t fb = (size_t)L.nsites * L.ndof * sizeof(cx<double>);
        SMG_CUDA(ctx, cudaMemcpyAsync(mg->cw[level].x, fine, fb, cudaMemcpyHostToDevice, ctx->stream));
        SMG_TRY(restrict_to<double>(mg, level, mg->cw[level].x, nw.b));
    }
    const size_t cb = (size_t)N.nsites * N.ndof * sizeof(cx<double>);
    SMG_CUDA(ctx, cudaMemcpyAsync(coarse, nw.b, cb, cudaMemcpyDeviceToHost, ctx->stream));
    SMG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return SMG_OK;
}

SMG_API smg_status smg_mg_time_coarse_solve(smg_mg* mg, int reps, double* ms, int* iters) {
    if (!mg || !ms || reps < 1 || mg->work_nrhs < 1 || mg->lv.size() < 2) return SMG_BAD_ARG;
    smg_context* ctx = mg->ctx;
    const int l = (int)mg->lv.size() - 1;
    CoarseWork& w = mg->cw[l];
    cudaEvent_t e0, e1;
    SMG_CUDA(ctx, cudaEventCreate(&e0));
    SMG_CUDA(ctx, cudaEventCreate(&e1));
    smg_status st = SMG_OK;
    for (int pass = 0; pass < 2 && st == SMG_OK; ++pass) {  // pass 0 warms up
        SMG_CUDA(ctx, cudaEventRecord(e0, ctx->stream));
        for (int i = 0; i < (pass ? reps : 1) && st == SMG_OK; ++i)
            st = mg->work_prec == SMG_F64 ? coarse_cg<double>(mg, l, w.x, w.b) : coarse_cg<float>(mg, l, w.x, w.b);
        SMG_CUDA(ctx, cudaEventRecord(e1, ctx->stream));
    }
    SMG_CUDA(ctx, cudaEventSynchronize(e1));
    float f = 0;
    SMG_CUDA(ctx, cudaEventElapsedTime(&f, e0, e1));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    SMG_TRY(st);
    SMG_TRY(smg_mg_check_device_error(mg));
    *ms = (double)f / reps;
    if (iters) {
        *iters = -1;
        if (mg->work_prec == SMG_F32 && coarse_half_level(mg, l, mg->work_nrhs, SMG_F32) && w.ph2 && ccg_tc_level(mg, l))
            SMG_CUDA(ctx, cudaMemcpy(iters, static_cast<int*>(mg->cg_state) + 3, sizeof(int), cudaMemcpyDeviceToHost));
    }
    return SMG_OK;
}

SMG_API smg_status smg_mg_time_coarse_apply(smg_mg* mg, int level, int nrhs, int reps, double* ms, double* bytes) {
    if (!mg || !ms || level < 1 || level >= (int)mg->lv.size() || nrhs < 1 || reps < 1) return SMG_BAD_ARG;
    smg_context* ctx = mg->ctx;
    const smg_precision prec = mg->p.precision;
    SMG_TRY(ensure_work(mg, nrhs, prec));
    const Level& L = mg->lv[level];
    CoarseWork& w = mg->cw[level];
    cudaEvent_t e0, e1;
    SMG_CUDA(ctx, cudaEventCreate(&e0));
    SMG_CUDA(ctx, cudaEventCreate(&e1));
    smg_status st = SMG_OK;
    for (int pass = 0; pass < 2 && st == SMG_OK; ++pass) {  // pass 0 warms up
        SMG_CUDA(ctx, cudaEventRecord(e0, ctx->stream));
        for (int i = 0; i < reps && st == SMG_OK; ++i) {
            if (prec == SMG_F64)
                st = coarse_apply<double>(mg, level, cview<double>(w.x, L, nrhs), (cx<double>*)w.Ar, 0, nullptr,
                                          nullptr);
            else
                st = coarse_apply<float>(mg, level, cview<float>(w.x, L, nrhs), (cx<float>*)w.Ar, 0, nullptr,
                                         nullptr);
        }
        SMG_CUDA(ctx, cudaEventRecord(e1, ctx->stream));
    }
    SMG_CUDA(ctx, cudaEventSynchronize(e1));
    float f = 0;
    SMG_CUDA(ctx, cudaEventElapsedTime(&f, e0, e1));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    SMG_TRY(st);
    SMG_TRY(smg_mg_check_device_error(mg));
    *ms = (double)f / reps;
    // compulsory bytes: the links once, the input and output vectors once
    const double es = prec == SMG_F64 ? 16.0 : 8.0;
    const double link_bytes = (prec == SMG_F32 && tc_path(mg, level, nrhs))
                                  ? (double)smg_coarse_tc_link_bytes(L.nsites)
                                  : es * (double)L.nsites * 9 * L.ndof * L.ndof;
    if (bytes) *bytes = link_bytes + es * 2.0 * L.nsites * L.ndof * nrhs;
    return SMG_OK;
}

// The fine smoother's kernels of one MR step on FP16 work vectors, each launched `reps` times on
// the context's stream and timed with CUDA events: [0] t = D r with ||t||^2 fused (FP16 -> FP16),
// [1] A r = D^dag t with ||A r||^2 fused plus the two small kernels that finish the MR scalars,
// [2] r' = r - omega A r, [3] the x pass that adds omega_k r_k of a whole smoothing (pre_smooth
// residuals).  r is made from b (F32, the hierarchy's nrhs); bytes[] are each kernel's compulsory
// HBM bytes.
SMG_API smg_status smg_mg_time_smoother(smg_mg* mg, const smg_field* b, int reps, double* ms, double* bytes) {
    if (!mg || !b || !ms || reps < 1) return SMG_BAD_ARG;
    smg_context* ctx = mg->ctx;
    if (b->prec != SMG_F32 || b->g.L != mg->lv[0].nx)
        return smg_fail(ctx, SMG_BAD_ARG, "smoother timing: b must be an F32 field of the hierarchy's lattice");
    const int V = b->g.V, nrhs = b->nrhs;
    if (!half_smoother(mg, nrhs, SMG_F32))
        return smg_fail(ctx, SMG_UNSUPPORTED, "smoother timing: the hierarchy has no FP16 smoother for this nrhs");
    SMG_TRY(ensure_work(mg, nrhs, SMG_F32));
    const int nx = std::max(1, mg->p.pre_smooth);
    smg_field* x = nullptr;
    SMG_TRY(smg_field_create(ctx, b->g.L, nrhs, SMG_F32, &x));
    SMG_CUDA(ctx, cudaMemsetAsync(x->data, 0, x->bytes, ctx->stream));
    // a smoothing's residuals from b, so every field the timed kernels read holds real data
    SMG_TRY(smooth_fine_half(mg, x, b, nx, true, 0.0, true));
    smg_field *r = mg->f_rs[0], *Ar = mg->f_Ar, *t = mg->f_t, *rn = mg->f_rs[1];
    double* sc = mg->mr_om;
    const dim3 blk = pair_block(nrhs), grd = pair_grid(V, nrhs);
    cudaEvent_t ev[5];
    for (auto& e : ev) SMG_CUDA(ctx, cudaEventCreate(&e));
    smg_status st = SMG_OK;
    for (int pass = 0; pass < 2 && st == SMG_OK; ++pass) {  // pass 0 warms up
        SMG_CUDA(ctx, cudaEventRecord(ev[0], ctx->stream));
        for (int i = 0; i < reps && st == SMG_OK; ++i) st = smg_dslash_h_norm(mg->dirac, false, r, t, mg->hdots, 0);
        SMG_CUDA(ctx, cudaEventRecord(ev[1], ctx->stream));
        for (int i = 0; i < reps && st == SMG_OK; ++i) {
            st = smg_dslash_h_norm(mg->dirac, true, t, Ar, mg->hdots, 1);
            if (st == SMG_OK)
                st = smg_mr_norms_finish(ctx, b->g.L, nrhs, mg->hdots, sc, reinterpret_cast<float*>(mg->mr_omf));
        }
        SMG_CUDA(ctx, cudaEventRecord(ev[2], ctx->stream));
        for (int i = 0; i < reps; ++i) {
            k_mr_rupdate_h<<<grd, blk, 0, ctx->stream>>>((const __half2*)r->data, r->scale, (const __half2*)Ar->data,
                                                         Ar->scale, (__half2*)rn->data, rn->scale, mg->mr_omf, 0.f, V,
                                                         nrhs);
            count_launch(ctx);
        }
        SMG_CUDA(ctx, cudaEventRecord(ev[3], ctx->stream));
        for (int i = 0; i < reps && st == SMG_OK; ++i) st = mr_xupdate_h(mg, x, 0, nx, false, 0.0);
        SMG_CUDA(ctx, cudaEventRecord(ev[4], ctx->stream));
    }
    SMG_CUDA(ctx, cudaEventSynchronize(ev[4]));
    for (int k = 0; k < 4; ++k) {
        float f = 0;
        SMG_CUDA(ctx, cudaEventElapsedTime(&f, ev[k], ev[k + 1]));
        ms[k] = (double)f / reps;
    }
    for (auto& e : ev) cudaEventDestroy(e);
    smg_field_destroy(x);
    SMG_TRY(st);
    SMG_CHECK_LAUNCH(ctx);
    if (bytes) {
        // per site: an FP16 two-spinor is 8 B per rhs plus a 4 B scale per field; links 2 x 8 B; clover 4 B
        const double n = (double)V;
        bytes[0] = n * (16.0 * nrhs + 8 + 16 + 4);              // r in, t out, links, clover
        bytes[1] = n * (16.0 * nrhs + 8 + 16 + 4);              // t in, A r out, links, clover
        bytes[2] = n * (24.0 * nrhs + 12);                      // r, A r in, r' out
        bytes[3] = n * (32.0 * nrhs + nx * (8.0 * nrhs + 4));   // x in and out (FP32), the residuals in
    }
    return SMG_OK;
}

SMG_API smg_status smg_mg_coarse_apply_batch(smg_mg* mg, int level, int nrhs, int engine, const float* in,
                                             const float* w, float* out, double* dots) {
    if (!mg || !in || !out || level < 1 || level >= (int)mg->lv.size() || nrhs < 1 || engine < 0 || engine > 1)
        return SMG_BAD_ARG;
    smg_context* ctx = mg->ctx;
    if (mg->p.precision != SMG_F32) return smg_fail(ctx, SMG_UNSUPPORTED, "coarse_apply_batch needs an F32 hierarchy");
    if (engine == 1 && !tc_path(mg, level, nrhs))
        return smg_fail(ctx, SMG_UNSUPPORTED, "tensor-core coarse apply: shape not supported");
    SMG_TRY(ensure_work(mg, nrhs, SMG_F32));
    const Level& L = mg->lv[level];
    CoarseWork& cw = mg->cw[level];
    const size_t b = (size_t)L.nsites * L.ndof * nrhs * sizeof(cx<float>);
    const int K = w ? 3 : 1;
    cx<float>* wdev = nullptr;
    double* ddev = nullptr;
    SMG_CUDA(ctx, cudaMemcpyAsync(cw.x, in, b, cudaMemcpyHostToDevice, ctx->stream));
    if (w) {
        SMG_CUDA(ctx, cudaMemcpyAsync(cw.r, w, b, cudaMemcpyHostToDevice, ctx->stream));
        wdev = (cx<float>*)cw.r;
    }
    if (dots) {
        SMG_CUDA(ctx, cudaMallocAsync((void**)&ddev, (size_t)nrhs * K * sizeof(double), ctx->stream));
        SMG_CUDA(ctx, cudaMemsetAsync(ddev, 0, (size_t)nrhs * K * sizeof(double), ctx->stream));
    }
    const int epi = dots ? (w ? 2 : 1) : 0;
    smg_status st = coarse_apply<float>(mg, level, cview<float>(cw.x, L, nrhs), (cx<float>*)cw.Ar, epi, wdev, ddev,
                                        nullptr, engine);
    if (st == SMG_OK) {
        SMG_CUDA(ctx, cudaMemcpyAsync(out, cw.Ar, b, cudaMemcpyDeviceToHost, ctx->stream));
        if (dots)
            SMG_CUDA(ctx, cudaMemcpyAsync(dots, ddev, (size_t)nrhs * K * sizeof(double), cudaMemcpyDeviceToHost,
                                          ctx->stream));
    }
    if (ddev) cudaFreeAsync(ddev, ctx->stream);
    SMG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    SMG_TRY(st);
    return smg_mg_check_device_error(mg);
}

SMG_API smg_status smg_mg_coarse_apply_host(smg_mg* mg, int level, const double* in, double* out) {
    if (!mg || !in || !out || level < 1 || level >= (int)mg->lv.size()) return SMG_BAD_ARG;
    smg_context* ctx = mg->ctx;
    SMG_TRY(ensure_work(mg, 1, SMG_F64));
    const Level& L = mg->lv[level];
    CoarseWork& w = mg->cw[level];
    const size_t b = (size_t)L.nsites * L.ndof * sizeof(cx<double>);
    SMG_CUDA(ctx, cudaMemcpyAsync(w.x, in, b, cudaMemcpyHostToDevice, ctx->stream));
    SMG_TRY(coarse_apply<double>(mg, level, cview<double>(w.x, L, 1), (cx<double>*)w.Ar, 0, nullptr, nullptr));
    SMG_CUDA(ctx, cudaMemcpyAsync(out, w.Ar, b, cudaMemcpyDeviceToHost, ctx->stream));
    SMG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return SMG_OK;
}

SMG_API smg_status smg_mg_estimate_lambda_max(smg_mg* mg, int level, int niter, double* lambda) {
    if (!mg || !lambda || niter < 0 || level < 0 || level >= (int)mg->lv.size()) return SMG_BAD_ARG;
    return lambda_max_level(mg, level, niter, lambda);
}

SMG_API smg_status smg_mg_set_symmetric(smg_mg* mg, double damping, double* omega) {
    if (!mg || !std::isfinite(damping)) return SMG_BAD_ARG;
    const int nl = (int)mg->lv.size();
    std::vector<double> om(nl - 1, 0.0);
    if (damping > 0) {
        for (int l = 0; l + 1 < nl; ++l) {
            double lmax = 0;
            SMG_TRY(lambda_max_level(mg, l, 30, &lmax));
            if (!(lmax > 0) || !std::isfinite(lmax))
                return smg_fail(mg->ctx, SMG_BREAKDOWN, "set_symmetric: lambda_max estimate is not positive");
            om[l] = damping / lmax;
        }
    }
    for (int l = 0; l + 1 < nl; ++l) mg->lv[l].rich_omega = om[l];
    drop_graph(mg);  // a captured cycle holds the old smoother
    if (omega)
        for (int l = 0; l + 1 < nl; ++l) omega[l] = om[l];
    return SMG_OK;
}

SMG_API smg_status smg_mg_rebuild(smg_mg* mg) {
    if (!mg) return SMG_BAD_ARG;
    return rebuild_operators(mg);
}

}  // extern "C"
