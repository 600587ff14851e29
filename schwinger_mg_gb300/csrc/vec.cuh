// Generic vector kernels for fine and coarse MG vectors.
//
// Fine MG vectors (smg_field) have the layout [site][rhs][dof] with the two
// spin components innermost.  Coarse MG vectors have the layout
// [site][dof][rhs] with the right-hand side innermost, so a warp of RHS lanes
// reads consecutive addresses for every dof and a dof row of all RHS is one
// contiguous tile (the B operand of the coarse-operator contraction).  For one
// right-hand side both layouts are the same array.  All per-right-hand-side
// scalars live in device memory; kernels that need a derived coefficient
// (alpha, omega, beta) compute it once per block from those scalars, so no
// host round trip sits between solver steps.
#pragma once
#include "reduce.cuh"
#include "smg_internal.h"

template <typename T>
struct VecView {
    cx<T>* p = nullptr;
    int nsites = 0, nrhs = 1, ndof = 2;
    int rhs_inner = 0;  // 0: [site][rhs][dof] (fine), 1: [site][dof][rhs] (coarse)
    __host__ __device__ int64_t n() const { return (int64_t)nsites * nrhs * ndof; }
    __host__ __device__ int64_t idx(int64_t site, int rhs, int dof) const {
        return rhs_inner ? (site * ndof + dof) * nrhs + rhs : (site * nrhs + rhs) * ndof + dof;
    }
    // distance between consecutive dofs of one (site, rhs)
    __host__ __device__ int dstride() const { return rhs_inner ? nrhs : 1; }
};

// per-rhs scalar slots used by the MG kernels (device memory)
struct MrScalars {  // MR step: <Ar, r> (re, im) and <Ar, Ar>
    double* s;      // [rhs][3]
};

enum { VR_DOT = 0, VR_NORM = 1, VR_DOTNORM = 2 };

// <a, b> (K=2), ||a||^2 (K=1), or <a, b> and ||a||^2 (K=3) per rhs
template <typename T, int MODE>
__global__ void __launch_bounds__(256) k_vreduce(VecView<T> a, const cx<T>* __restrict__ b, double* partials,
                                                 unsigned int* ticket, double* out) {
    constexpr int K = MODE == VR_DOT ? 2 : (MODE == VR_NORM ? 1 : 3);
    const int rhs = blockIdx.y * blockDim.x + threadIdx.x;
    T v[K];  // per-thread partials in the field precision (FP64 is scarce on this part)
#pragma unroll
    for (int k = 0; k < K; ++k) v[k] = T(0);
    if (rhs < a.nrhs && a.ndof == 2 && !a.rhs_inner) {
        // fine fields: one 2-spinor vector per (site, rhs), four sites per pass with every load issued first
        const Spinor<T>* __restrict__ ap = reinterpret_cast<const Spinor<T>*>(a.p);
        const Spinor<T>* __restrict__ bp = reinterpret_cast<const Spinor<T>*>(b);
        const int stride = gridDim.x * blockDim.y;
        T r0 = 0, r1 = 0, r2 = 0;
        for (int s0 = blockIdx.x * blockDim.y + threadIdx.y; s0 < a.nsites; s0 += 4 * stride) {
            Spinor<T> xa[4], xb[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const int s = s0 + u * stride;
                if (s < a.nsites) {
                    xa[u] = ap[(int64_t)s * a.nrhs + rhs];
                    if (MODE != VR_NORM) xb[u] = bp[(int64_t)s * a.nrhs + rhs];
                }
            }
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                if (s0 + u * stride >= a.nsites) continue;
                if (MODE != VR_NORM) {
                    const cx<T> c = cmulc(xa[u].s0, xb[u].s0) + cmulc(xa[u].s1, xb[u].s1);
                    r0 += c.re;
                    r1 += c.im;
                }
                if (MODE != VR_DOT) r2 += norm2(xa[u].s0) + norm2(xa[u].s1);
            }
        }
        if (MODE == VR_DOT) {
            v[0] = r0;
            v[1] = r1;
        } else if (MODE == VR_NORM) {
            v[0] = r2;
        } else {
            v[0] = r0;
            v[1] = r1;
            v[2] = r2;
        }
    } else if (rhs < a.nrhs) {
        for (int s = blockIdx.x * blockDim.y + threadIdx.y; s < a.nsites; s += gridDim.x * blockDim.y) {
            const int64_t base = a.idx(s, rhs, 0);
            const int ds = a.dstride();
            T r0 = 0, r1 = 0, r2 = 0;
            for (int d = 0; d < a.ndof; ++d) {
                cx<T> x = a.p[base + (int64_t)d * ds];
                if (MODE != VR_NORM) {
                    cx<T> c = cmulc(x, b[base + (int64_t)d * ds]);
                    r0 += c.re;
                    r1 += c.im;
                }
                if (MODE != VR_DOT) r2 += norm2(x);
            }
            if (MODE == VR_DOT) {
                v[0] += r0;
                v[1] += r1;
            } else if (MODE == VR_NORM) {
                v[0] += r2;
            } else {
                v[0] += r0;
                v[1] += r1;
                v[2] += r2;
            }
        }
    }
    block_reduce_finalise<K>(v, partials, ticket, a.nrhs, FinStore{out, K});
}

// y = y + sgn * coef[rhs] * x with coef a complex per rhs (interleaved doubles)
template <typename T>
__global__ void k_vaxpy(VecView<T> y, const cx<T>* __restrict__ x, const double* __restrict__ coef, double sgn) {
    const int rhs = blockIdx.y * blockDim.x + threadIdx.x;
    const int s = blockIdx.x * blockDim.y + threadIdx.y;
    if (rhs >= y.nrhs || s >= y.nsites) return;
    const cx<T> a = mk<T>((T)(sgn * coef[2 * rhs]), (T)(sgn * coef[2 * rhs + 1]));
    const int64_t base = y.idx(s, rhs, 0);
    const int ds = y.dstride();
    for (int d = 0; d < y.ndof; ++d) y.p[base + (int64_t)d * ds] = y.p[base + (int64_t)d * ds] + a * x[base + (int64_t)d * ds];
}

// MR step (reference src/smoother.cpp:26-40):  omega = <Ar, r> / <Ar, Ar>,
// x += omega r, r -= omega Ar.  sc[rhs*3 + {0,1,2}] = re<Ar,r>, im<Ar,r>, <Ar,Ar>.
// A step with |<Ar,Ar>| < 1e-30 leaves x and r unchanged (the reference breaks).
template <typename T>
__global__ void __launch_bounds__(256) k_mr_update(VecView<T> x, cx<T>* __restrict__ r, const cx<T>* __restrict__ Ar,
                                                   const double* __restrict__ sc) {
    __shared__ cx<T> s_om[32];
    const int rhs = blockIdx.y * blockDim.x + threadIdx.x;
    if (threadIdx.y == 0) {
        cx<T> om = mk<T>(0, 0);
        if (rhs < x.nrhs) {
            double den = sc[3 * rhs + 2];
            if (fabs(den) >= 1e-30 && isfinite(den)) om = mk<T>((T)(sc[3 * rhs] / den), (T)(sc[3 * rhs + 1] / den));
        }
        s_om[threadIdx.x] = om;
    }
    __syncthreads();
    const int s = blockIdx.x * blockDim.y + threadIdx.y;
    if (rhs >= x.nrhs || s >= x.nsites) return;
    const cx<T> om = s_om[threadIdx.x];
    const int64_t base = x.idx(s, rhs, 0);
    const int ds = x.dstride();
    for (int d = 0; d < x.ndof; ++d) {
        const cx<T> ri = r[base + (int64_t)d * ds];
        x.p[base + (int64_t)d * ds] = x.p[base + (int64_t)d * ds] + om * ri;
        r[base + (int64_t)d * ds] = ri - om * Ar[base + (int64_t)d * ds];
    }
}

// Richardson step with a fixed real omega (reference src/smoother.cpp:64-73):
// x += omega r, r -= omega Ar.  The residual is carried recursively, so a step
// costs one operator application as in the reference, which recomputes
// r = b - A x instead.
template <typename T>
__global__ void k_rich_update(VecView<T> x, cx<T>* __restrict__ r, const cx<T>* __restrict__ Ar, T omega) {
    const int rhs = blockIdx.y * blockDim.x + threadIdx.x;
    const int s = blockIdx.x * blockDim.y + threadIdx.y;
    if (rhs >= x.nrhs || s >= x.nsites) return;
    const int64_t base = x.idx(s, rhs, 0);
    const int ds = x.dstride();
    for (int d = 0; d < x.ndof; ++d) {
        const cx<T> ri = r[base + (int64_t)d * ds];
        x.p[base + (int64_t)d * ds] = x.p[base + (int64_t)d * ds] + omega * ri;
        r[base + (int64_t)d * ds] = ri - omega * Ar[base + (int64_t)d * ds];
    }
}

// r = b - Ax
template <typename T>
__global__ void k_vsub(cx<T>* __restrict__ r, const cx<T>* __restrict__ b, const cx<T>* __restrict__ Ax, int64_t n) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) r[i] = b[i] - Ax[i];
}

// y += x
template <typename T>
__global__ void k_vadd(cx<T>* __restrict__ y, const cx<T>* __restrict__ x, int64_t n) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) y[i] = y[i] + x[i];
}

// out = in * scale[rhs] (real) with precision conversion; used to move a
// residual between FP64 and the preconditioner precision with normalisation
template <typename D, typename S>
__global__ void k_vconvert_scaled(VecView<D> out, const cx<S>* __restrict__ in, const double* __restrict__ scale,
                                  int invert) {
    const int rhs = blockIdx.y * blockDim.x + threadIdx.x;
    const int s = blockIdx.x * blockDim.y + threadIdx.y;
    if (rhs >= out.nrhs || s >= out.nsites) return;
    double f = 1.0;
    if (scale) {
        double sv = scale[rhs];
        f = invert ? (sv > 0 ? 1.0 / sqrt(sv) : 0.0) : sqrt(sv);
    }
    const int64_t base = out.idx(s, rhs, 0);
    const int ds = out.dstride();
    for (int d = 0; d < out.ndof; ++d) {
        cx<S> v = in[base + (int64_t)d * ds];
        out.p[base + (int64_t)d * ds] = mk<D>((D)((double)v.re * f), (D)((double)v.im * f));
    }
}

inline dim3 vec_block(int nrhs) {
    int lanes = nrhs < 32 ? nrhs : 32;
    return dim3(lanes, 256 / lanes);
}
inline dim3 vec_grid(int nsites, int nrhs) {
    dim3 b = vec_block(nrhs);
    return dim3((nsites + b.y - 1) / b.y, (nrhs + b.x - 1) / b.x);
}
