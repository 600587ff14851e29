// The four Wilson hops of one site (reference accumulate_hops, src/dirac.h:58-89).
//
// With a = U psi(x+mu) and b = U^dag(x-mu) psi(x-mu) per spin component, the
// hopping part of D is -1/2 S with
//   S0 = r (a0x + b0x + a0y + b0y) + sgn [(b1x - a1x) + i (a1y - b1y)]
//   S1 = r (a1x + b1x + a1y + b1y) + sgn [(b0x - a0x) - i (a0y - b0y)]
// (sgn = +1 for D, -1 for D^dag = g5 D(-mu) g5).  For r = 1 the spin factors
// r -+ sigma_mu are twice rank-one projectors, so each hop needs one complex
// link product on a projected half spinor instead of two:
//   D:     S0 = A_xf + B_xb + A_yf + B_yb,   S1 = (B_xb - A_xf) + i (B_yb - A_yf)
//          A_xf = U (p0 - p1), B_xb = U^dag (m0 + m1), A_yf = U (p0 + i p1), B_yb = U^dag (m0 - i m1)
//   D^dag: S0 likewise with the projections' signs of p1, m1 flipped,
//          S1 = (A_xf - B_xb) + i (A_yf - B_yb).
#pragma once
#include "smg_internal.h"

// r = 1: the projected half spinors h (one per hop) times their links, rebuilt into the two spin
// components of the hopping sum
template <typename T, bool DAG>
__device__ __forceinline__ void hop_recon(cx<T> u0f, cx<T> u0b, cx<T> u1f, cx<T> u1b, cx<T> hxf, cx<T> hxb,
                                          cx<T> hyf, cx<T> hyb, cx<T>& S0, cx<T>& S1) {
    const cx<T> A_xf = u0f * hxf, B_xb = cmulc(u0b, hxb);
    const cx<T> A_yf = u1f * hyf, B_yb = cmulc(u1b, hyb);
    S0 = (A_xf + B_xb) + (A_yf + B_yb);
    S1 = DAG ? (A_xf - B_xb) + times_i(A_yf - B_yb) : (B_xb - A_xf) + times_i(B_yb - A_yf);
}

template <typename T, bool DAG, bool R1>
__device__ __forceinline__ void hop_sum(cx<T> u0f, cx<T> u0b, cx<T> u1f, cx<T> u1b, const Spinor<T>& pxp,
                                        const Spinor<T>& pxm, const Spinor<T>& pyp, const Spinor<T>& pym, T r,
                                        cx<T>& S0, cx<T>& S1) {
    if (R1) {
        const cx<T> hxf = DAG ? pxp.s0 + pxp.s1 : pxp.s0 - pxp.s1;
        const cx<T> hxb = DAG ? pxm.s0 - pxm.s1 : pxm.s0 + pxm.s1;
        const cx<T> hyf = DAG ? pyp.s0 - times_i(pyp.s1) : pyp.s0 + times_i(pyp.s1);
        const cx<T> hyb = DAG ? pym.s0 + times_i(pym.s1) : pym.s0 - times_i(pym.s1);
        hop_recon<T, DAG>(u0f, u0b, u1f, u1b, hxf, hxb, hyf, hyb, S0, S1);
    } else {
        const T sgn = DAG ? T(-1) : T(1);
        const cx<T> a0x = u0f * pxp.s0, a1x = u0f * pxp.s1;
        const cx<T> b0x = cmulc(u0b, pxm.s0), b1x = cmulc(u0b, pxm.s1);
        const cx<T> a0y = u1f * pyp.s0, a1y = u1f * pyp.s1;
        const cx<T> b0y = cmulc(u1b, pym.s0), b1y = cmulc(u1b, pym.s1);
        const cx<T> sr0 = (a0x + b0x) + (a0y + b0y), sr1 = (a1x + b1x) + (a1y + b1y);
        const cx<T> off0 = (b1x - a1x) + times_i(a1y - b1y);
        const cx<T> off1 = (b0x - a0x) - times_i(a0y - b0y);
        S0 = r * sr0 + sgn * off0;
        S1 = r * sr1 + sgn * off1;
    }
}
