// lbm_pair.cuh — the contracted collisions on two cells at once with the
// packed f32x2 arithmetic of sm_100-class GPUs (__fadd2_rn, __fmul2_rn,
// __ffma2_rn): one instruction does the same IEEE operation on both halves of
// a float2, so a thread's cells are collided in pairs at half the issue
// count.  Each half computes exactly what collide_fast / collide_dev compute
// for one cell with every a * b + c written as one fma; the per-cell results
// are those of the scalar fast path up to the contraction choices the
// compiler makes there (both are LBM_FAST arithmetic).
#pragma once

#include "lbm_common.cuh"

namespace lbmk {

__device__ __forceinline__ float2 bc2(float a) { return make_float2(a, a); }
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
// a - b as one fused operation: b * (-1) is exact, so this rounds once.
__device__ __forceinline__ float2 sub2(float2 a, float2 b) { return __ffma2_rn(b, bc2(-1.f), a); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 rcp2(float2 a) {
    return make_float2(Ar<true>::rcp(a.x), Ar<true>::rcp(a.y));
}

// f_eq of the four direction pairs (i, opp(i)) around a common P + -Q split:
// the rest population and f_eq = RW (base + k2 (c.u)^2) +- RW k1 (c.u), the
// shape shared by the plain and the deviation forms.
// Guo source of a pair: S_i = gw_i (kcF_i - uF + cF4_i (c_i.u)); for opp(i)
// c.u and c.F change sign, so S_opp = gw_i (-kcF_i - uF + cF4_i (c_i.u)).

// Plain populations (collide_fast on two cells).
__device__ __forceinline__ void collide_fast_x2(const Consts<float>& c, const float2 (&f)[9],
                                                float2 (&out)[9]) {
    const float2 rho = add2(add2(add2(add2(f[0], f[1]), add2(f[2], f[3])),
                                 add2(add2(f[4], f[5]), add2(f[6], f[7]))), f[8]);
    float2 mx = add2(add2(sub2(f[1], f[3]), sub2(f[5], f[6])), sub2(f[8], f[7]));
    float2 my = sub2(add2(sub2(f[2], f[4]), add2(f[5], f[6])), add2(f[7], f[8]));
    if (c.force) { mx = add2(mx, bc2(c.hfx)); my = add2(my, bc2(c.hfy)); }
    const float2 inv = rcp2(rho);
    const float2 ux = mul2(mx, inv), uy = mul2(my, inv);
    const float2 base = fma2(fma2(ux, ux, mul2(uy, uy)), bc2(c.k3), bc2(1.f));
    const float2 rw0 = mul2(rho, bc2(c.wt[0])), rw1 = mul2(rho, bc2(c.wt[1])),
                 rw5 = mul2(rho, bc2(c.wt[5]));
    const float2 rk1 = mul2(rw1, bc2(c.k1)), rk5 = mul2(rw5, bc2(c.k1));
    const float2 d = add2(ux, uy), e = sub2(uy, ux);
    float2 feq[9];
    feq[0] = mul2(rw0, base);
    {
        const float2 A = mul2(rw1, fma2(bc2(c.k2), mul2(ux, ux), base)), B = mul2(rk1, ux);
        feq[1] = add2(A, B); feq[3] = sub2(A, B);
    }
    {
        const float2 A = mul2(rw1, fma2(bc2(c.k2), mul2(uy, uy), base)), B = mul2(rk1, uy);
        feq[2] = add2(A, B); feq[4] = sub2(A, B);
    }
    {
        const float2 A = mul2(rw5, fma2(bc2(c.k2), mul2(d, d), base)), B = mul2(rk5, d);
        feq[5] = add2(A, B); feq[7] = sub2(A, B);
    }
    {
        const float2 A = mul2(rw5, fma2(bc2(c.k2), mul2(e, e), base)), B = mul2(rk5, e);
        feq[6] = add2(A, B); feq[8] = sub2(A, B);
    }
    if (c.collision == LBM_COLLISION_TRT) {
#pragma unroll
        for (int i = 0; i < 9; ++i) {
            const float2 fsw = f[OPP(i)];
            const float2 eqsw = (i == 0) ? feq[0] : fsw;
            const float2 om = fma2(sub2(sub2(f[i], fsw), sub2(feq[i], eqsw)), bc2(c.omega_m),
                                   mul2(sub2(add2(f[i], fsw), add2(feq[i], eqsw)), bc2(c.omega_p)));
            out[i] = fma2(om, bc2(c.trt_scale), f[i]);
        }
    } else {
#pragma unroll
        for (int i = 0; i < 9; ++i) out[i] = fma2(sub2(f[i], feq[i]), bc2(c.bgk_factor), f[i]);
    }
    if (c.force) {
        const float2 uF = mul2(bc2(c.k1), fma2(ux, bc2(c.fx), mul2(uy, bc2(c.fy))));
        const float2 v[5] = {bc2(0.f), ux, uy, d, e};
#pragma unroll
        for (int i = 1; i < 9; ++i) {
            // c_i.u of directions 1, 2, 5, 6 is v[1..4]; of their opposites its
            // negation.  An opposite's kcF and cF4 are the exact negations of
            // its partner's (the host computes them from the negated c_i) and
            // w_i is shared, so four constants of each kind and two gw values
            // serve all eight directions (fewer registers where the constants
            // come from memory).
            const int p = (i == 1 || i == 3) ? 1 : (i == 2 || i == 4) ? 2 : (i == 5 || i == 7) ? 3 : 4;
            const int r = p == 1 ? 1 : p == 2 ? 2 : p == 3 ? 5 : 6;
            const bool opp = i == 3 || i == 4 || i == 7 || i == 8;
            const float kc = opp ? -c.kcF[r] : c.kcF[r];
            out[i] = fma2(bc2(c.gw[i < 5 ? 1 : 5]), fma2(v[p], bc2(c.cF4[r]), sub2(bc2(kc), uF)), out[i]);
        }
        out[0] = fma2(bc2(c.gw[0]), sub2(bc2(c.kcF[0]), uF), out[0]);
    }
}

// Deviation variables G_i = s (f_i - w_i) (collide_dev on two cells).
__device__ __forceinline__ void collide_dev_x2_general(const Consts<float>& c,
                                                       const float2 (&G)[9], float2 (&out)[9]) {
    const float2 DR = add2(add2(add2(add2(G[0], G[1]), add2(G[2], G[3])),
                                add2(add2(G[4], G[5]), add2(G[6], G[7]))), G[8]);
    float2 jx = add2(add2(sub2(G[1], G[3]), sub2(G[5], G[6])), sub2(G[8], G[7]));
    float2 jy = sub2(add2(sub2(G[2], G[4]), add2(G[5], G[6])), add2(G[7], G[8]));
    if (c.force) { jx = add2(jx, bc2(c.shfx)); jy = add2(jy, bc2(c.shfy)); }
    const float2 RS = add2(bc2(c.dscale), DR);             // s * rho
    const float2 inv = rcp2(RS);
    const float2 ux = mul2(jx, inv), uy = mul2(jy, inv);
    const float2 u2k3 = mul2(bc2(c.k3), fma2(ux, ux, mul2(uy, uy)));
    const float2 rs0 = mul2(RS, bc2(c.wt[0])), rs1 = mul2(RS, bc2(c.wt[1])),
                 rs5 = mul2(RS, bc2(c.wt[5]));
    const float2 wd0 = mul2(DR, bc2(c.wt[0])), wd1 = mul2(DR, bc2(c.wt[1])),
                 wd5 = mul2(DR, bc2(c.wt[5]));
    const float2 d = add2(ux, uy), e = sub2(uy, ux);
    float2 geq[9];
    geq[0] = fma2(rs0, u2k3, wd0);
    {
        const float2 A = fma2(bc2(c.k2), mul2(ux, ux), u2k3), B = mul2(bc2(c.k1), ux);
        geq[1] = fma2(rs1, add2(A, B), wd1); geq[3] = fma2(rs1, sub2(A, B), wd1);
    }
    {
        const float2 A = fma2(bc2(c.k2), mul2(uy, uy), u2k3), B = mul2(bc2(c.k1), uy);
        geq[2] = fma2(rs1, add2(A, B), wd1); geq[4] = fma2(rs1, sub2(A, B), wd1);
    }
    {
        const float2 A = fma2(bc2(c.k2), mul2(d, d), u2k3), B = mul2(bc2(c.k1), d);
        geq[5] = fma2(rs5, add2(A, B), wd5); geq[7] = fma2(rs5, sub2(A, B), wd5);
    }
    {
        const float2 A = fma2(bc2(c.k2), mul2(e, e), u2k3), B = mul2(bc2(c.k1), e);
        geq[6] = fma2(rs5, add2(A, B), wd5); geq[8] = fma2(rs5, sub2(A, B), wd5);
    }
    if (c.collision == LBM_COLLISION_TRT) {
#pragma unroll
        for (int i = 0; i < 9; ++i) {
            const float2 gsw = G[OPP(i)];
            const float2 eqsw = (i == 0) ? geq[0] : gsw;
            const float2 om = fma2(sub2(sub2(G[i], gsw), sub2(geq[i], eqsw)), bc2(c.omega_m),
                                   mul2(sub2(add2(G[i], gsw), add2(geq[i], eqsw)), bc2(c.omega_p)));
            out[i] = fma2(om, bc2(c.trt_scale), G[i]);
        }
    } else {
#pragma unroll
        for (int i = 0; i < 9; ++i) out[i] = fma2(sub2(G[i], geq[i]), bc2(c.bgk_factor), G[i]);
    }
    if (c.force) {
        const float2 uF = mul2(bc2(c.k1), fma2(ux, bc2(c.fx), mul2(uy, bc2(c.fy))));
        const float2 v[5] = {bc2(0.f), ux, uy, d, e};
#pragma unroll
        for (int i = 1; i < 9; ++i) {
            // the shared constants of collide_fast_x2
            const int p = (i == 1 || i == 3) ? 1 : (i == 2 || i == 4) ? 2 : (i == 5 || i == 7) ? 3 : 4;
            const int r = p == 1 ? 1 : p == 2 ? 2 : p == 3 ? 5 : 6;
            const bool opp = i == 3 || i == 4 || i == 7 || i == 8;
            const float kc = opp ? -c.kcF[r] : c.kcF[r];
            out[i] = fma2(bc2(c.sgw[i < 5 ? 1 : 5]), fma2(v[p], bc2(c.cF4[r]), sub2(bc2(kc), uF)), out[i]);
        }
        out[0] = fma2(bc2(c.sgw[0]), sub2(bc2(c.kcF[0]), uF), out[0]);
    }
}

// BGK (with Guo forcing when a force is set) of deviation variables on two
// cells, folded: out_i = G_i - omega (G_i - G_eq_i) + S_i is written as
// keep G_i + (omega G_eq_i + S_i), and omega G_eq_i + S_i of a direction pair
// (i, opp(i)) is even +- odd (PairConsts), so a pair costs one quadratic
// term, two multiply-adds for the even part, one for the odd part and two
// for the outputs.  The constants come as float2 pairs from the parameter
// space.  Every term is of the size of the deviation, so the roundings stay
// far below the 16-bit storage's own.  (Plain f32 populations keep the
// general form: folded, keep f_i and omega f_eq_i are of the size of f_i,
// and their roundings shift the mass step after step.)
__device__ __forceinline__ void collide_bgk_folded_x2(const Consts<float>& c, const float2 (&G)[9],
                                                      float2 (&out)[9]) {
    const PairConsts& k = c.pk;
    const float2 s13 = add2(G[1], G[3]), d13 = sub2(G[1], G[3]);
    const float2 s24 = add2(G[2], G[4]), d24 = sub2(G[2], G[4]);
    const float2 s57 = add2(G[5], G[7]), d57 = sub2(G[5], G[7]);
    const float2 s68 = add2(G[6], G[8]), d68 = sub2(G[6], G[8]);
    const float2 D = add2(add2(G[0], s13), add2(add2(s24, s57), s68));
    float2 jx = sub2(add2(d13, d57), d68);            // c_x: 1, 5, 8 minus 3, 6, 7
    float2 jy = add2(add2(d24, d57), d68);            // c_y: 2, 5, 6 minus 4, 7, 8
    if (c.force) {
        jx = add2(jx, k.shfx);
        jy = add2(jy, k.shfy);
    }
    const float2 RS = add2(k.dscale, D);               // s rho
    const float2 inv = rcp2(RS);
    const float2 ux = mul2(jx, inv), uy = mul2(jy, inv);
    const float2 ux2 = mul2(ux, ux), uy2 = mul2(uy, uy);
    const float2 t3 = fma2(k.k3, ux2, mul2(k.k3, uy2));     // k3 u^2
    const float2 d = add2(ux, uy), e = sub2(uy, ux);         // c.u of directions 5 and 6
    float2 b0 = mul2(k.ow[0], D), b1 = mul2(k.ow[1], D), b5 = mul2(k.ow[2], D);
    if (c.force) {
        const float2 uF = fma2(ux, k.k1fx, mul2(uy, k.k1fy));
        b0 = fma2(k.nsgw[0], uF, b0);
        b1 = fma2(k.nsgw[1], uF, b1);
        b5 = fma2(k.nsgw[2], uF, b5);
    }
    const float2 a0 = mul2(k.ow[0], RS), a1 = mul2(k.ow[1], RS), a5 = mul2(k.ow[2], RS);
    const float2 a1k = mul2(k.owk[1], RS), a5k = mul2(k.owk[2], RS);
    out[0] = fma2(G[0], k.keep, fma2(a0, t3, b0));
    // one direction pair: cu = c_i.u, q = (c_i.u)^2, a / ak / b of its class
    auto pair = [&](int i, int o, float2 cu, float2 q, float2 a, float2 ak, float2 b) {
        float2 ee = fma2(a, fma2(k.k2, q, t3), b);
        float2 oo;
        if (c.force) {
            ee = fma2(k.sgwcF4[i], cu, ee);
            oo = fma2(ak, cu, k.so[i]);
        } else {
            oo = mul2(ak, cu);
        }
        out[i] = fma2(G[i], k.keep, add2(ee, oo));
        out[o] = fma2(G[o], k.keep, sub2(ee, oo));
    };
    pair(1, 3, ux, ux2, a1, a1k, b1);
    pair(2, 4, uy, uy2, a1, a1k, b1);
    pair(5, 7, d, mul2(d, d), a5, a5k, b5);
    pair(6, 8, e, mul2(e, e), a5, a5k, b5);
}

// The deviation collision on cell pairs: BGK folded, TRT general.
#ifndef LBM_FOLDED_BGK
#define LBM_FOLDED_BGK 1
#endif
__device__ __forceinline__ void collide_dev_x2(const Consts<float>& c, const float2 (&G)[9],
                                               float2 (&out)[9]) {
    if (LBM_FOLDED_BGK && c.collision != LBM_COLLISION_TRT) collide_bgk_folded_x2(c, G, out);
    else collide_dev_x2_general(c, G, out);
}

}  // namespace lbmk
