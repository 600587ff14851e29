// Helpers shared by the Krylov solvers (CG, PCG, GCR, FGMRES) and the fine
// smoothers: temporaries shaped like a right-hand-side field, the fine-field
// vector view, A = D^dag D as two stencil passes, and the per-rhs reductions.
#pragma once
#include "smg_internal.h"
#include "reduce.cuh"
#include "vec.cuh"

#include <vector>

smg_status smg_dslash(smg_dirac* d, bool dag, const smg_field* src, smg_field* dst, double* norm2_dev);
smg_status smg_norm2_dev(const smg_field* a, double* out_dev);

namespace {

template <typename T>
__global__ void k_residual(const cx<T>* __restrict__ b, const cx<T>* __restrict__ Ax, cx<T>* __restrict__ r,
                           int64_t n) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) r[i] = b[i] - Ax[i];
}

// a solver's work fields, taken from the context's pool and given back when the solver returns
struct FieldSet {
    std::vector<smg_field*> f;
    ~FieldSet() {
        for (auto* p : f) smg_field_give(p);
    }
    smg_status add(const smg_field* proto, smg_field** out) { return add(proto, proto->prec, out); }
    smg_status add(const smg_field* proto, smg_precision prec, smg_field** out) {
        SMG_TRY(smg_field_take(proto, prec, out));
        f.push_back(*out);
        return SMG_OK;
    }
};

// a device buffer from the context's pool for the life of a solve
struct PoolBuf {
    smg_context* ctx = nullptr;
    size_t bytes = 0;
    void* p = nullptr;
    ~PoolBuf() {
        if (ctx) smg_buf_give(ctx, bytes, p);
    }
    smg_status take(smg_context* c, size_t b) {
        ctx = c;
        bytes = b;
        return smg_buf_take(c, b, &p);
    }
};

template <typename T>
VecView<T> fv(const smg_field* f) {
    VecView<T> v;
    v.p = (cx<T>*)f->data;
    v.nsites = f->g.V;
    v.nrhs = f->nrhs;
    v.ndof = 2;
    return v;
}

template <typename T>
smg_status apply_A(smg_dirac* d, const smg_field* in, smg_field* tmp, smg_field* out) {
    SMG_TRY(smg_dslash(d, false, in, tmp, nullptr));
    return smg_dslash(d, true, tmp, out, nullptr);
}

template <typename T>
smg_status reduce_into(smg_context* ctx, VecView<T> a, const cx<T>* b, int mode, double* out) {
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

}  // namespace
