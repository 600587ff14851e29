// Pseudofermion force: the hand-written adjoint of S = phi^dag (D^dag D)^-1 phi.
//
// With X = (D^dag D)^-1 phi and chi = D X, the force on link (mu, s) is
// (reference src/hmc_forces.cpp:134-194 and 198-495)
//   F_mu(s) = Im(c_fwd) - Im(c_bwd)                                 hopping
//           + c_sw/4 [Re P_fwd * sum_fwd w - Re P_bwd * sum_bwd w]  clover
// with w(x) = Re(chi_0^* X_0 - chi_1^* X_1)(x).  chi is never stored: each
// thread block stages X and the links of its tile plus a two-site halo in
// shared memory, recomputes chi = D X and w on the tile plus a one-site halo,
// and forms both force components of every tile site from shared memory.
// Output is lexicographic F[mu][s] (reference src/hmc.h:34).
#include "smg_internal.h"

namespace {

constexpr int TX = 16, TY = 8;
constexpr int RX = TX + 4, RY = TY + 4;  // X / link region, origin (-2, -2)
constexpr int CX = TX + 2, CY = TY + 2;  // chi / w region, origin (-1, -1)

struct ForceArgs {
    const cx<double>* __restrict__ X = nullptr;  // single-RHS F64 field, device layout
    const cx<double>* __restrict__ U = nullptr;
    const double* __restrict__ C = nullptr;      // clover shift or nullptr
    double* __restrict__ F = nullptr;            // [mu][s] lexicographic
    Geom g{};
    double diag = 0, mu = 0, r = 0, c_sw = 0;
};

__device__ __forceinline__ int pmod(int a, int L) {
    int m = a % L;
    return m < 0 ? m + L : m;
}

__global__ void __launch_bounds__(TX* TY) k_fermion_force(ForceArgs a) {
    __shared__ cx<double> sX[RY * RX][2];
    __shared__ cx<double> sU[2][RY * RX];
    __shared__ double sC[CY * CX];
    __shared__ cx<double> sChi[CY * CX][2];
    __shared__ double sW[CY * CX];

    const Geom g = a.g;
    const int x0 = blockIdx.x * TX, y0 = blockIdx.y * TY;
    const int tid = threadIdx.y * TX + threadIdx.x;
    const int nthr = TX * TY;

    for (int i = tid; i < RX * RY; i += nthr) {
        int rx = i % RX, ry = i / RX;
        int gx = pmod(x0 - 2 + rx, g.L), gy = pmod(y0 - 2 + ry, g.L);
        int q = site_q(g, gx, gy);
        sX[i][0] = a.X[(int64_t)q * 2 + 0];
        sX[i][1] = a.X[(int64_t)q * 2 + 1];
        sU[0][i] = a.U[q];
        sU[1][i] = a.U[(int64_t)g.V + q];
    }
    for (int i = tid; i < CX * CY; i += nthr) {
        int cxx = i % CX, cyy = i / CX;
        int gx = pmod(x0 - 1 + cxx, g.L), gy = pmod(y0 - 1 + cyy, g.L);
        sC[i] = a.C ? a.C[site_q(g, gx, gy)] : 0.0;
    }
    __syncthreads();

    // chi = D X on the tile plus a one-site halo (dirac.h:93-113)
    const double half = 0.5, r = a.r;
    for (int i = tid; i < CX * CY; i += nthr) {
        int cxx = i % CX, cyy = i / CX;
        int c = (cyy + 1) * RX + (cxx + 1);  // index in the X / link frame
        cx<double> u0f = sU[0][c], u0b = sU[0][c - 1], u1f = sU[1][c], u1b = sU[1][c - RX];
        cx<double> a0x = u0f * sX[c + 1][0], a1x = u0f * sX[c + 1][1];
        cx<double> b0x = cmulc(u0b, sX[c - 1][0]), b1x = cmulc(u0b, sX[c - 1][1]);
        cx<double> a0y = u1f * sX[c + RX][0], a1y = u1f * sX[c + RX][1];
        cx<double> b0y = cmulc(u1b, sX[c - RX][0]), b1y = cmulc(u1b, sX[c - RX][1]);
        cx<double> dg0 = mk(a.diag + sC[i], a.mu), dg1 = mk(a.diag - sC[i], -a.mu);
        cx<double> sr0 = (a0x + b0x) + (a0y + b0y);
        cx<double> sr1 = (a1x + b1x) + (a1y + b1y);
        cx<double> off0 = (b1x - a1x) + times_i(a1y - b1y);
        cx<double> off1 = (b0x - a0x) - times_i(a0y - b0y);
        cx<double> c0 = dg0 * sX[c][0] - half * (r * sr0 + off0);
        cx<double> c1 = dg1 * sX[c][1] - half * (r * sr1 + off1);
        sChi[i][0] = c0;
        sChi[i][1] = c1;
        sW[i] = cmulc(c0, sX[c][0]).re - cmulc(c1, sX[c][1]).re;
    }
    __syncthreads();

    const int tx = threadIdx.x, ty = threadIdx.y;
    const int gx = x0 + tx, gy = y0 + ty;
    if (gx >= g.L || gy >= g.L) return;
    const int c = (ty + 2) * RX + (tx + 2);  // X / link frame
    const int k = (ty + 1) * CX + (tx + 1);  // chi / w frame
    const cx<double> X0 = sX[c][0], X1 = sX[c][1];
    const cx<double> ch0 = sChi[k][0], ch1 = sChi[k][1];
    double F0, F1;
    {   // mu = 0, hmc_forces.cpp:154-170
        cx<double> u = sU[0][c];
        cx<double> ux0 = u * sX[c + 1][0], ux1 = u * sX[c + 1][1];
        cx<double> fwd0 = r * ux0 - ux1, fwd1 = r * ux1 - ux0;
        cx<double> c_fwd = cmulc(ch0, fwd0) + cmulc(ch1, fwd1);
        cx<double> udx0 = cmulc(u, X0), udx1 = cmulc(u, X1);
        cx<double> bwd0 = r * udx0 + udx1, bwd1 = udx0 + r * udx1;
        cx<double> c_bwd = cmulc(sChi[k + 1][0], bwd0) + cmulc(sChi[k + 1][1], bwd1);
        F0 = c_fwd.im - c_bwd.im;
    }
    {   // mu = 1, hmc_forces.cpp:172-188
        cx<double> u = sU[1][c];
        cx<double> ux0 = u * sX[c + RX][0], ux1 = u * sX[c + RX][1];
        cx<double> fwd0 = r * ux0 + times_i(ux1), fwd1 = r * ux1 - times_i(ux0);
        cx<double> c_fwd = cmulc(ch0, fwd0) + cmulc(ch1, fwd1);
        cx<double> udx0 = cmulc(u, X0), udx1 = cmulc(u, X1);
        cx<double> bwd0 = r * udx0 - times_i(udx1), bwd1 = times_i(udx0) + r * udx1;
        cx<double> c_bwd = cmulc(sChi[k + CX][0], bwd0) + cmulc(sChi[k + CX][1], bwd1);
        F1 = c_fwd.im - c_bwd.im;
    }
    if (a.c_sw != 0.0) {  // clover insertion, hmc_forces.cpp:409-492
        // plaq(s) = U0(s) U1(s+x) U0*(s+y) U1*(s)
        cx<double> P_s = sU[0][c] * sU[1][c + 1] * conj(sU[0][c + RX]) * conj(sU[1][c]);
        // plaq(s-y)
        cx<double> P_sym = sU[0][c - RX] * sU[1][c - RX + 1] * conj(sU[0][c]) * conj(sU[1][c - RX]);
        // plaq(s-x)
        cx<double> P_sxm = sU[0][c - 1] * sU[1][c] * conj(sU[0][c - 1 + RX]) * conj(sU[1][c - 1]);
        double w_s = sW[k], w_xp = sW[k + 1], w_yp = sW[k + CX], w_xpyp = sW[k + 1 + CX];
        double w_ym = sW[k - CX], w_xpym = sW[k + 1 - CX], w_xm = sW[k - 1], w_xmyp = sW[k - 1 + CX];
        double w_fwd = w_s + w_xp + w_xpyp + w_yp;
        double w_bwd = w_ym + w_xpym + w_xp + w_s;
        F0 += (a.c_sw / 4.0) * (P_s.re * w_fwd - P_sym.re * w_bwd);
        double w_fwd1 = w_xm + w_s + w_yp + w_xmyp;
        F1 += (a.c_sw / 4.0) * (P_sxm.re * w_fwd1 - P_s.re * w_fwd);
    }
    const int s = gx + g.L * gy;
    a.F[s] = F0;
    a.F[(int64_t)g.V + s] = F1;
}

}  // namespace

// Device-side force into a device array F[mu][s] (lexicographic).
smg_status smg_fermion_force_dev(smg_dirac* d, const smg_field* X, double* F_dev) {
    smg_context* ctx = d->ctx;
    ForceArgs a;
    a.X = (const cx<double>*)X->data;
    a.U = d->gauge->U64;
    a.C = d->C64;
    a.F = F_dev;
    a.g = X->g;
    a.diag = 2.0 * d->r + d->mass;
    a.mu = d->mu_t;
    a.r = d->r;
    a.c_sw = d->c_sw;
    dim3 block(TX, TY);
    dim3 grid((X->g.L + TX - 1) / TX, (X->g.L + TY - 1) / TY);
    k_fermion_force<<<grid, block, 0, ctx->stream>>>(a);
    count_launch(ctx);
    SMG_CHECK_LAUNCH(ctx);
    return SMG_OK;
}

extern "C" {

SMG_API smg_status smg_fermion_force(smg_dirac* d, const smg_field* X, double* force) {
    if (!d || !X || !force) return SMG_BAD_ARG;
    smg_context* ctx = d->ctx;
    if (X->prec != SMG_F64 || X->nrhs != 1)
        return smg_fail(ctx, SMG_BAD_ARG, "fermion_force needs a single-RHS F64 field");
    if (X->g.L != d->gauge->g.L) return smg_fail(ctx, SMG_BAD_ARG, "field L differs from gauge L");
    size_t bytes = (size_t)2 * X->g.V * sizeof(double);
    double* dev = nullptr;
    SMG_CUDA(ctx, cudaMallocAsync(&dev, bytes, ctx->stream));
    smg_status s = smg_fermion_force_dev(d, X, dev);
    if (s != SMG_OK) {
        cudaFreeAsync(dev, ctx->stream);
        return s;
    }
    SMG_CUDA(ctx, cudaMemcpyAsync(force, dev, bytes, cudaMemcpyDeviceToHost, ctx->stream));
    SMG_CUDA(ctx, cudaFreeAsync(dev, ctx->stream));
    SMG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return SMG_OK;
}

}  // extern "C"
