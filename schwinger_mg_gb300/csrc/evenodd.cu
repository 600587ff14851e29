// Even-odd (Schur complement) preconditioned Wilson-clover operator and its
// force (reference EvenOddDiracOp, src/dirac.h:190-553; eo_fermion_force,
// schur_deriv_plus, logdet_ee_force, src/hmc_forces.cpp:571-867).
//
// Fields keep the device layout of the full operator: sites ordered parity
// half by parity half, q = p V/2 + (x + L y)/2.  Within a half this is the
// reference's even_sites / odd_sites order (eo_index[s] = (x + L y)/2), so a
// half-lattice vector of the reference is one contiguous half of a field and
// the solver kernels run on it with V/2 sites and an offset base pointer.
//
// With D = Diag + H (H the hopping part), the Schur complement on odd sites is
//   M x_o = Diag_oo x_o - H_oe Diag_ee^-1 H_eo x_o  (apply_schur, src/dirac.h:407-423),
// applied as two stencil kernels over one parity each:
//   EEINV   t_e = Diag_ee^-1 (H x_o)(e)
//   SCHUR   y_o = Diag_oo x_o - (H t_e)(o)            (optionally ||y_o||^2)
// M^dag = g5 M(-mu) g5 is the same pair with the spin off-diagonal hopping
// sign and the twist flipped (g5 commutes with the spin-diagonal Diag).
//
// Force, F = -dS/dtheta for S = phi_o^dag (M^dag M)^-1 phi_o - 2 log det Diag_ee:
// with x_o = (M^dag M)^-1 phi_o, y_o = M x_o, psi = (Diag_ee^-1 H x_o, x_o),
// chi = (Diag_ee(-mu)^-1 g5 H g5 y_o, y_o):
//   F_mu(s) = -Hbil_mu(s; chi, psi) + Ins_mu(s; W),
//   W = (c_sw/4) Re(chi^dag sigma3 psi) + (c_sw/4) [d0/(d0^2+mu^2) - d1/(d1^2+mu^2)]_even
// where Hbil is the hopping bilinear (hopping_force_bilinear) and Ins the
// plaquette insertion of a clover weight (clover_deriv_insert); the factors
// are those of eo_fermion_force (2 x schur_deriv_plus + logdet_ee_force).
#include "krylov.cuh"
#include "stencil.cuh"

#include <cmath>

namespace {

enum { EO_HOP = 0, EO_EEINV = 1, EO_RECON = 2, EO_SCHUR = 3 };

template <typename T>
struct EoArgs {
    const cx<T>* __restrict__ hop_src = nullptr;  // full field; the other parity's half is read
    const cx<T>* __restrict__ z = nullptr;        // full field; same-parity term (SCHUR: x_o, RECON: phi_e or none)
    cx<T>* __restrict__ out = nullptr;            // full field; the output parity's half is written
    const cx<T>* __restrict__ U = nullptr;
    const T* __restrict__ C = nullptr;
    Geom g{};
    int nrhs = 1;
    int p = 0;  // output parity
    T diag = 0, mu_eff = 0, r = 0;
    double* partials = nullptr;
    unsigned int* ticket = nullptr;
    double* norm = nullptr;
};

// one output parity; EPI: ||out||^2 per rhs
template <typename T, bool DAG, int MODE, bool EPI>
__global__ void __launch_bounds__(256) k_eo(EoArgs<T> a) {
    const T half = T(0.5);
    const Geom g = a.g;
    const int nrhs = a.nrhs;
    T v[1] = {T(0)};
    auto site = [&](int y, int xh, int rhs) {
        const int p = a.p;
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
        const cx<T> u0f = a.U[q], u0b = a.U[q_xm];
        const cx<T> u1f = a.U[g.V + q], u1b = a.U[g.V + q_ym];
        const Spinor<T> pxp = ld_spinor(a.hop_src, q_xp, rhs, nrhs);
        const Spinor<T> pxm = ld_spinor(a.hop_src, q_xm, rhs, nrhs);
        const Spinor<T> pyp = ld_spinor(a.hop_src, q_yp, rhs, nrhs);
        const Spinor<T> pym = ld_spinor(a.hop_src, q_ym, rhs, nrhs);
        // (H psi)(q) = -1/2 S, apply_hop (src/dirac.h:197-249)
        cx<T> S0, S1;
        hop_sum<T, DAG, false>(u0f, u0b, u1f, u1b, pxp, pxm, pyp, pym, a.r, S0, S1);
        const cx<T> h0 = -half * S0;
        const cx<T> h1 = -half * S1;
        const T Cq = a.C ? a.C[q] : T(0);
        const cx<T> dg0 = mk<T>(a.diag + Cq, a.mu_eff);
        const cx<T> dg1 = mk<T>(a.diag - Cq, -a.mu_eff);
        Spinor<T> o;
        if (MODE == EO_HOP) {
            o.s0 = h0;
            o.s1 = h1;
        } else if (MODE == EO_SCHUR) {
            const Spinor<T> zq = ld_spinor(a.z, q, rhs, nrhs);
            o.s0 = dg0 * zq.s0 - h0;
            o.s1 = dg1 * zq.s1 - h1;
        } else {
            cx<T> t0 = h0, t1 = h1;
            if (MODE == EO_RECON) {
                if (a.z) {
                    const Spinor<T> zq = ld_spinor(a.z, q, rhs, nrhs);
                    t0 = zq.s0 - h0;
                    t1 = zq.s1 - h1;
                } else {
                    t0 = -h0;
                    t1 = -h1;
                }
            }
            const T n0 = T(1) / norm2(dg0), n1 = T(1) / norm2(dg1);
            o.s0 = n0 * cmulc(dg0, t0);  // t / dg = conj(dg) t / |dg|^2
            o.s1 = n1 * cmulc(dg1, t1);
        }
        st_spinor(a.out, q, rhs, nrhs, o);
        if (EPI) v[0] += norm2(o.s0) + norm2(o.s1);
    };
    if (!EPI) {
        const int rhs = blockIdx.z * blockDim.x + threadIdx.x;
        const int xh = blockIdx.x * blockDim.y + threadIdx.y;
        if (rhs < nrhs && xh < g.Lh) site(blockIdx.y, xh, rhs);
    } else {
        const int rhs = blockIdx.y * blockDim.x + threadIdx.x;
        if (rhs < nrhs)
            for (int w = blockIdx.x * blockDim.y + threadIdx.y; w < g.Vh; w += gridDim.x * blockDim.y) {
                const int y = w / g.Lh;
                site(y, w - y * g.Lh, rhs);
            }
        block_reduce_finalise<1>(v, a.partials, a.ticket, nrhs, FinStore{a.norm, 1});
    }
}

template <typename T>
smg_status launch_eo(smg_dirac* d, bool dag, int mode, int p, const smg_field* hop_src, const smg_field* z,
                     smg_field* out, double* norm) {
    smg_context* ctx = d->ctx;
    EoArgs<T> a;
    a.hop_src = (const cx<T>*)hop_src->data;
    a.z = z ? (const cx<T>*)z->data : nullptr;
    a.out = (cx<T>*)out->data;
    if (sizeof(T) == 8) {
        a.U = (const cx<T>*)d->gauge->U64;
        a.C = (const T*)d->C64;
    } else {
        if (!d->gauge->U32) return smg_fail(ctx, SMG_DEVICE_ERROR, "FP32 links missing");
        a.U = (const cx<T>*)d->gauge->U32;
        a.C = (const T*)d->C32;
    }
    a.g = hop_src->g;
    a.nrhs = hop_src->nrhs;
    a.p = p;
    a.diag = (T)(2.0 * d->r + d->mass);
    a.mu_eff = (T)(dag ? -d->mu_t : d->mu_t);
    a.r = (T)d->r;
    a.norm = norm;
    const int nrhs = a.nrhs;
    if (!norm) {
        const int lanes = nrhs < 32 ? nrhs : 32, rows = 256 / lanes;
        const dim3 block(lanes, rows), grid((a.g.Lh + rows - 1) / rows, a.g.L, (nrhs + lanes - 1) / lanes);
#define SMG_EO(DAG, MODE) k_eo<T, DAG, MODE, false><<<grid, block, 0, ctx->stream>>>(a)
        if (dag) {
            if (mode == EO_HOP) SMG_EO(true, EO_HOP);
            else if (mode == EO_EEINV) SMG_EO(true, EO_EEINV);
            else if (mode == EO_RECON) SMG_EO(true, EO_RECON);
            else SMG_EO(true, EO_SCHUR);
        } else {
            if (mode == EO_HOP) SMG_EO(false, EO_HOP);
            else if (mode == EO_EEINV) SMG_EO(false, EO_EEINV);
            else if (mode == EO_RECON) SMG_EO(false, EO_RECON);
            else SMG_EO(false, EO_SCHUR);
        }
#undef SMG_EO
    } else {
        if (mode != EO_SCHUR) return smg_fail(ctx, SMG_BAD_ARG, "even-odd norm epilogue: Schur kernel only");
        const ReduceLaunch rl = reduce_launch(a.g.Vh, nrhs);
        SMG_TRY(smg_reduce_reserve(ctx, (size_t)rl.grid.x * nrhs));
        a.partials = ctx->red.partials;
        a.ticket = ctx->red.tickets;
        if (dag)
            k_eo<T, true, EO_SCHUR, true><<<rl.grid, rl.block, 0, ctx->stream>>>(a);
        else
            k_eo<T, false, EO_SCHUR, true><<<rl.grid, rl.block, 0, ctx->stream>>>(a);
    }
    count_launch(ctx);
    SMG_CHECK_LAUNCH(ctx);
    return SMG_OK;
}

smg_status eo_dispatch(smg_dirac* d, bool dag, int mode, int p, const smg_field* hop_src, const smg_field* z,
                       smg_field* out, double* norm) {
    if (hop_src->prec == SMG_F64) return launch_eo<double>(d, dag, mode, p, hop_src, z, out, norm);
    if (hop_src->prec == SMG_F32) return launch_eo<float>(d, dag, mode, p, hop_src, z, out, norm);
    return smg_fail(d->ctx, SMG_UNSUPPORTED, "even-odd operator on F16 fields");
}

// ---------------------------------------------------------------- force

// W(q) = (c_sw/4) Re(chi^dag sigma3 psi)(q) + (c_sw/4) [d0/(d0^2+mu^2) - d1/(d1^2+mu^2)] on even sites
__global__ void k_eo_weight(const cx<double>* __restrict__ chi, const cx<double>* __restrict__ psi,
                            const double* __restrict__ C, Geom g, double diag, double mu, double c_sw,
                            double* __restrict__ W) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= g.V) return;
    const cx<double> c0 = chi[2 * q], c1 = chi[2 * q + 1];
    const cx<double> p0 = psi[2 * q], p1 = psi[2 * q + 1];
    double w = 0.25 * c_sw * (cmulc(c0, p0).re - cmulc(c1, p1).re);
    if (q < g.Vh && C) {
        const double Cq = C[q];
        const double d0 = diag + Cq, d1 = diag - Cq, m2 = mu * mu;
        w += 0.25 * c_sw * (d0 / (d0 * d0 + m2) - d1 / (d1 * d1 + m2));
    }
    W[q] = w;
}

__device__ __forceinline__ int qof(const Geom& g, int x, int y) { return site_q(g, wrap(x, g.L), wrap(y, g.L)); }

// F[mu][s] (lexicographic) = -Hbil_mu(s; chi, psi) + Ins_mu(s; W)
__global__ void k_eo_force(const cx<double>* __restrict__ chi, const cx<double>* __restrict__ psi,
                           const cx<double>* __restrict__ U, const double* __restrict__ W, Geom g, double r,
                           int with_clover, double* __restrict__ F) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= g.V) return;
    const int x = s % g.L, y = s / g.L;
    const int q = qof(g, x, y), qxp = qof(g, x + 1, y), qyp = qof(g, x, y + 1);
    const cx<double> c0 = chi[2 * q], c1 = chi[2 * q + 1];
    const cx<double> x0 = psi[2 * q], x1 = psi[2 * q + 1];
    double f[2];
    for (int mu = 0; mu < 2; ++mu) {  // hopping_force_bilinear (src/hmc_forces.cpp:540-569)
        const int qf = mu == 0 ? qxp : qyp;
        const cx<double> u = U[(int64_t)mu * g.V + q];
        const cx<double> ux0 = u * psi[2 * qf], ux1 = u * psi[2 * qf + 1];
        const cx<double> udx0 = cmulc(u, x0), udx1 = cmulc(u, x1);
        cx<double> fwd0, fwd1, bwd0, bwd1;
        if (mu == 0) {
            fwd0 = r * ux0 - ux1;
            fwd1 = r * ux1 - ux0;
            bwd0 = r * udx0 + udx1;
            bwd1 = udx0 + r * udx1;
        } else {
            fwd0 = r * ux0 + times_i(ux1);
            fwd1 = r * ux1 - times_i(ux0);
            bwd0 = r * udx0 - times_i(udx1);
            bwd1 = times_i(udx0) + r * udx1;
        }
        const cx<double> cf = cmulc(c0, fwd0) + cmulc(c1, fwd1);
        const cx<double> cb = cmulc(chi[2 * qf], bwd0) + cmulc(chi[2 * qf + 1], bwd1);
        f[mu] = -(cf.im - cb.im);  // -Re(i c_bwd - i c_fwd)
    }
    if (with_clover) {  // clover_deriv_insert (src/hmc_forces.cpp:501-534)
        auto L0 = [&](int xx, int yy) { return U[qof(g, xx, yy)]; };
        auto L1 = [&](int xx, int yy) { return U[(int64_t)g.V + qof(g, xx, yy)]; };
        auto Wq = [&](int xx, int yy) { return W[qof(g, xx, yy)]; };
        const double pf = (L0(x, y) * L1(x + 1, y) * conj(L0(x, y + 1)) * conj(L1(x, y))).re;
        const double pb = (L0(x, y - 1) * L1(x + 1, y - 1) * conj(L0(x, y)) * conj(L1(x, y - 1))).re;
        const double pf1 = (L0(x - 1, y) * L1(x, y) * conj(L0(x - 1, y + 1)) * conj(L1(x - 1, y))).re;
        const double wf = Wq(x, y) + Wq(x + 1, y) + Wq(x + 1, y + 1) + Wq(x, y + 1);
        const double wb = Wq(x, y - 1) + Wq(x + 1, y - 1) + Wq(x + 1, y) + Wq(x, y);
        const double wf1 = Wq(x - 1, y) + Wq(x, y) + Wq(x, y + 1) + Wq(x - 1, y + 1);
        f[0] += pf * wf - pb * wb;
        f[1] += pf1 * wf1 - pf * wf;
    }
    F[s] = f[0];
    F[(int64_t)g.V + s] = f[1];
}

// Re log det Diag_ee = sum_e 1/2 log(d0^2 + mu^2) + 1/2 log(d1^2 + mu^2)  (log_det_ee, src/dirac.h:511-521)
__global__ void k_logdet(const double* __restrict__ C, Geom g, double diag, double mu, double* partials,
                         unsigned int* ticket, double* out) {
    double v[1] = {0.0};
    const double m2 = mu * mu;
    for (int e = blockIdx.x * blockDim.y + threadIdx.y; e < g.Vh; e += gridDim.x * blockDim.y) {
        const double Cq = C ? C[e] : 0.0;
        const double d0 = diag + Cq, d1 = diag - Cq;
        v[0] += 0.5 * log(d0 * d0 + m2) + 0.5 * log(d1 * d1 + m2);
    }
    block_reduce_finalise<1>(v, partials, ticket, 1, FinStore{out, 1});
}

smg_status check_eo_fields(smg_dirac* d, const smg_field* a, const smg_field* b) {
    if (!d || !a || !b) return SMG_BAD_ARG;
    smg_context* ctx = d->ctx;
    if (a == b) return smg_fail(ctx, SMG_BAD_ARG, "src and dst must be distinct fields");
    SMG_TRY(smg_field_check_pair(a, b));
    if (a->g.L != d->gauge->g.L) return smg_fail(ctx, SMG_BAD_ARG, "field L differs from gauge L");
    if (a->g.L % 2) return smg_fail(ctx, SMG_BAD_ARG, "even-odd operators need an even L");
    return SMG_OK;
}

}  // namespace

// ---- internal entry points (solvers, HMC)

// dst_o = M x_o (dag: M^dag x_o) with the even half of tmp as the scratch
// half-vector; norm2_dev (optional) receives ||dst_o||^2 per rhs
smg_status smg_eo_schur_internal(smg_dirac* d, bool dag, const smg_field* src, smg_field* dst, smg_field* tmp,
                                 double* norm2_dev) {
    SMG_TRY(eo_dispatch(d, dag, EO_EEINV, 0, src, nullptr, tmp, nullptr));
    return eo_dispatch(d, dag, EO_SCHUR, 1, tmp, src, dst, norm2_dev);
}

// x_e = Diag_ee^-1 (phi_e - H x_o) into the even half of x (reconstruct, src/dirac.h:527-540);
// phi == nullptr: x_e = -Diag_ee^-1 H x_o (reconstruct_full, :499-508)
smg_status smg_eo_reconstruct_internal(smg_dirac* d, const smg_field* phi, smg_field* x) {
    return eo_dispatch(d, false, EO_RECON, 0, x, phi, x, nullptr);
}

// log det Diag_ee into out_dev (one double)
smg_status smg_eo_logdet_dev(smg_dirac* d, double* out_dev) {
    smg_context* ctx = d->ctx;
    const Geom g = d->gauge->g;
    const ReduceLaunch rl = reduce_launch(g.Vh, 1);
    SMG_TRY(smg_reduce_reserve(ctx, (size_t)rl.grid.x));
    k_logdet<<<rl.grid, rl.block, 0, ctx->stream>>>(d->c_sw != 0.0 ? d->C64 : nullptr, g, 2.0 * d->r + d->mass,
                                                    d->mu_t, ctx->red.partials, ctx->red.tickets, out_dev);
    count_launch(ctx);
    SMG_CHECK_LAUNCH(ctx);
    return SMG_OK;
}

// F (device, [mu][s] lexicographic) = e/o force at x_o = odd half of X; chi and psi are
// full-field scratch (single rhs, F64), W is V doubles of scratch
smg_status smg_eo_force_dev(smg_dirac* d, const smg_field* X, smg_field* chi, smg_field* psi, double* W,
                            double* F_dev) {
    smg_context* ctx = d->ctx;
    const Geom g = X->g;
    const size_t hb = X->bytes / 2;
    // psi = (Diag_ee^-1 H x_o, x_o); chi = (Diag_ee(-mu)^-1 g5 H g5 y_o, y_o = M x_o)
    SMG_CUDA(ctx, cudaMemcpyAsync((char*)psi->data + hb, (const char*)X->data + hb, hb, cudaMemcpyDeviceToDevice,
                                  ctx->stream));
    SMG_TRY(eo_dispatch(d, false, EO_EEINV, 0, psi, nullptr, psi, nullptr));
    SMG_TRY(eo_dispatch(d, false, EO_SCHUR, 1, psi, psi, chi, nullptr));
    SMG_TRY(eo_dispatch(d, true, EO_EEINV, 0, chi, nullptr, chi, nullptr));
    k_eo_weight<<<(g.V + 255) / 256, 256, 0, ctx->stream>>>((const cx<double>*)chi->data,
                                                            (const cx<double>*)psi->data, d->C64, g,
                                                            2.0 * d->r + d->mass, d->mu_t, d->c_sw, W);
    k_eo_force<<<(g.V + 255) / 256, 256, 0, ctx->stream>>>((const cx<double>*)chi->data,
                                                           (const cx<double>*)psi->data, d->gauge->U64, W, g, d->r,
                                                           d->c_sw != 0.0 ? 1 : 0, F_dev);
    count_launch(ctx, 2);
    SMG_CHECK_LAUNCH(ctx);
    return SMG_OK;
}

extern "C" {

SMG_API smg_status smg_eo_reconstruct(smg_dirac* d, const smg_field* phi, smg_field* x) {
    if (!d || !x) return SMG_BAD_ARG;
    if (phi) SMG_TRY(check_eo_fields(d, phi, x));
    if (x->g.L != d->gauge->g.L || x->g.L % 2) return smg_fail(d->ctx, SMG_BAD_ARG, "field L differs from gauge L");
    return smg_eo_reconstruct_internal(d, phi, x);
}

SMG_API smg_status smg_eo_logdet_ee(smg_dirac* d, double* logdet) {
    if (!d || !logdet) return SMG_BAD_ARG;
    smg_context* ctx = d->ctx;
    double* dv = nullptr;
    SMG_CUDA(ctx, cudaMallocAsync((void**)&dv, sizeof(double), ctx->stream));
    smg_status s = smg_eo_logdet_dev(d, dv);
    if (s == SMG_OK && cudaMemcpyAsync(logdet, dv, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream) != cudaSuccess)
        s = smg_fail(ctx, SMG_DEVICE_ERROR, "eo_logdet_ee: read-back failed");
    cudaFreeAsync(dv, ctx->stream);
    SMG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return s;
}

SMG_API smg_status smg_eo_fermion_force(smg_dirac* d, const smg_field* X, double* force) {
    if (!d || !X || !force) return SMG_BAD_ARG;
    smg_context* ctx = d->ctx;
    if (X->prec != SMG_F64 || X->nrhs != 1)
        return smg_fail(ctx, SMG_BAD_ARG, "eo_fermion_force needs a single-RHS F64 field");
    if (X->g.L != d->gauge->g.L || X->g.L % 2) return smg_fail(ctx, SMG_BAD_ARG, "field L differs from gauge L");
    const Geom g = X->g;
    smg_field *chi = nullptr, *psi = nullptr;
    SMG_TRY(smg_field_alloc_like(X, SMG_F64, &chi));
    smg_status s = smg_field_alloc_like(X, SMG_F64, &psi);
    double* dev = nullptr;
    if (s == SMG_OK && cudaMallocAsync((void**)&dev, (size_t)3 * g.V * sizeof(double), ctx->stream) != cudaSuccess)
        s = smg_fail(ctx, SMG_NO_MEMORY, "eo_fermion_force scratch");
    if (s == SMG_OK) s = smg_eo_force_dev(d, X, chi, psi, dev + 2 * (size_t)g.V, dev);
    if (s == SMG_OK &&
        cudaMemcpyAsync(force, dev, (size_t)2 * g.V * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream) !=
            cudaSuccess)
        s = smg_fail(ctx, SMG_DEVICE_ERROR, "eo_fermion_force: read-back failed");
    if (dev) cudaFreeAsync(dev, ctx->stream);
    cudaStreamSynchronize(ctx->stream);
    smg_field_destroy(chi);
    smg_field_destroy(psi);
    return s;
}

SMG_API smg_status smg_eo_apply(smg_dirac* d, smg_eo_operator op, const smg_field* src, smg_field* dst) {
    SMG_TRY(check_eo_fields(d, src, dst));
    smg_context* ctx = d->ctx;
    switch (op) {
        case SMG_EO_SCHUR:
        case SMG_EO_SCHUR_DAG: {
            smg_field* tmp = nullptr;
            SMG_TRY(smg_field_alloc_like(src, src->prec, &tmp));
            smg_status s = smg_eo_schur_internal(d, op == SMG_EO_SCHUR_DAG, src, dst, tmp, nullptr);
            smg_field_destroy(tmp);
            return s;
        }
        case SMG_EO_SCHUR_DAG_SCHUR: {
            smg_field *tmp = nullptr, *mid = nullptr;
            SMG_TRY(smg_field_alloc_like(src, src->prec, &tmp));
            smg_status s = smg_field_alloc_like(src, src->prec, &mid);
            if (s == SMG_OK) s = smg_eo_schur_internal(d, false, src, mid, tmp, nullptr);
            if (s == SMG_OK) s = smg_eo_schur_internal(d, true, mid, dst, tmp, nullptr);
            smg_field_destroy(tmp);
            smg_field_destroy(mid);
            return s;
        }
        case SMG_EO_HOP_EO:  // apply_eo: the even half of src hopped onto the odd half of dst
            return eo_dispatch(d, false, EO_HOP, 1, src, nullptr, dst, nullptr);
        case SMG_EO_HOP_OE:  // apply_oe: the odd half of src hopped onto the even half of dst
            return eo_dispatch(d, false, EO_HOP, 0, src, nullptr, dst, nullptr);
    }
    return smg_fail(ctx, SMG_BAD_ARG, "unknown even-odd operator");
}

}  // extern "C"
