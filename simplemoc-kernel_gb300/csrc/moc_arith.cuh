// moc_arith.cuh — the per-(segment, group) attenuation arithmetic, shared by the
// single-problem sweep (moc_sweep.cu) and the batching form (moc_batch.cu).
//
// src/cpu/kernel.c:200-332: for one segment of length ds through a cell with total cross
// section s and quadratic source coefficients (q0, q1 mu, q2 mu^2), tau = s ds, the angular
// flux leaves as psi' = psi (1 - e) + the source terms and the tally gets FI. Divisions by
// powers of s become products with one reciprocal; 25 FP32 operations and two MUFU
// operations (ex2, rcp) per segment and group.
#pragma once

#include "moc_device.cuh"
#include "moc_internal.h"

namespace moc {

struct TableRef {
    const float2 *tab;
    int n;
    float dx, max;
};

// One group. x = (sigT, q0, q1*mu, q2*mu2); pm gets p = exp(-tau) (the product of the
// affine psi map that the long-track split composes).
template <int EK>
__device__ __forceinline__ void attenuate_one(const float4 &x, float ds, float weight,
                                              const TableRef &tr, float &psi, float &tal,
                                              float &pm)
{
    const float s = x.x, a0 = x.y, a1 = x.z, a2 = x.w;
    const float ps = psi;
    const float tau = __fmul_rn(s, ds);  // kept exact: the table index depends on it
    const float tt = tau * tau;
    float e, p, tme, cub3;                 // cub3 = (tau(tau(tau-3)+6) - 6e) / 3
    if constexpr (EK == EXPK_STABLE) {
        const ExpTerms u = exp_terms_stable(tau);
        e = u.e;
        p = u.p;
        tme = u.tme;
        cub3 = u.cub * (1.0f / 3.0f);
    } else {
        if constexpr (EK == EXPK_TABLE) {
            e = table_lookup(tr.tab, tr.n, tr.dx, tr.max, tau);
            p = 1.0f - e;
        } else {
            p = ex2_approx(tau * -1.44269504088896341f);
            e = 1.0f - p;
        }
        tme = tau - e;
        // (tau(tau(tau-3)+6) - 6e)/3 = tau^2 (tau/3 - 1) + 2 (tau - e)
        cub3 = fmaf(tt, fmaf(tau, 1.0f / 3.0f, -1.0f), tme + tme);
    }
    // (q0 tau + (s psi - q0) e)/s^2 == q0 (tau - e)/s^2 + psi e/s exactly, so FI and
    // psi' share e/s and (tau - e)/s^2; 2e/s^3 = 2 (e/s) / s^2.
    const float rs = rcp_approx(s);
    const float rs2 = rs * rs;
    const float e1 = e * rs, t2 = tme * rs2;
    const float reuse = fmaf(e1 + e1, rs2, fmaf(tau, -2.0f, tt));
    float fi = fmaf(a0, t2, ps * e1);
    fi = fmaf(a1, reuse, fi);
    fi = fmaf(a2 * cub3, rs2 * rs2, fi);
    tal = weight * fi;
    float pn = fmaf(a1, t2, a0 * e1);
    pn = fmaf(a2, reuse, pn);
    psi = fmaf(ps, p, pn);
    pm = p;
}

// attenuate_one for two groups at once, on the packed FP32 pipe (fma/mul/add
// .rn.f32x2: one instruction, two lanes, each rounded exactly as the scalar instruction).
// Every packed operation stands for the same scalar operation of the one-group form, and
// 1 - x and a - b are written fma(x, -1, 1) and fma(b, -1, a), which round once to the same
// value, so both forms give identical bits.
// x0 = (sigT_a, sigT_b, q0_a, q0_b), x1 = (q1mu_a, q1mu_b, q2mu2_a, q2mu2_b).
template <int EK>
__device__ __forceinline__ void attenuate_pair(const float4 &x0, const float4 &x1, float ds,
                                               float weight, const TableRef &tr,
                                               float &psi0, float &psi1, float &tal0,
                                               float &tal1, float &pm0, float &pm1)
{
    const float2 one = make_float2(1.0f, 1.0f), mone = make_float2(-1.0f, -1.0f);
    const float2 s = make_float2(x0.x, x0.y), a0 = make_float2(x0.z, x0.w);
    const float2 a1 = make_float2(x1.x, x1.y), a2 = make_float2(x1.z, x1.w);
    const float2 ps = make_float2(psi0, psi1);
    const float2 tau = __fmul2_rn(s, make_float2(ds, ds));
    const float2 tt = __fmul2_rn(tau, tau);
    float2 e, p, tme, cub3;
    if constexpr (EK == EXPK_STABLE) {
        const ExpTerms2 u = exp_terms_stable2(tau);
        e = u.e;
        p = u.p;
        tme = u.tme;
        cub3 = __fmul2_rn(u.cub, make_float2(1.0f / 3.0f, 1.0f / 3.0f));
    } else {
        if constexpr (EK == EXPK_TABLE) {
            e = make_float2(table_lookup(tr.tab, tr.n, tr.dx, tr.max, tau.x),
                            table_lookup(tr.tab, tr.n, tr.dx, tr.max, tau.y));
            p = __ffma2_rn(e, mone, one);
        } else {
            const float2 m = __fmul2_rn(
                tau, make_float2(-1.44269504088896341f, -1.44269504088896341f));
            p = make_float2(ex2_approx(m.x), ex2_approx(m.y));
            e = __ffma2_rn(p, mone, one);
        }
        tme = __ffma2_rn(e, mone, tau);
        cub3 = __ffma2_rn(tt,
                          __ffma2_rn(tau, make_float2(1.0f / 3.0f, 1.0f / 3.0f), mone),
                          __fadd2_rn(tme, tme));
    }
    const float2 rs = make_float2(rcp_approx(s.x), rcp_approx(s.y));
    const float2 rs2 = __fmul2_rn(rs, rs);
    const float2 e1 = __fmul2_rn(e, rs), t2 = __fmul2_rn(tme, rs2);
    const float2 reuse = __ffma2_rn(__fadd2_rn(e1, e1), rs2,
                                    __ffma2_rn(tau, make_float2(-2.0f, -2.0f), tt));
    float2 fi = __ffma2_rn(a0, t2, __fmul2_rn(ps, e1));
    fi = __ffma2_rn(a1, reuse, fi);
    fi = __ffma2_rn(__fmul2_rn(a2, cub3), __fmul2_rn(rs2, rs2), fi);
    const float2 tl = __fmul2_rn(make_float2(weight, weight), fi);
    float2 pn = __ffma2_rn(a1, t2, __fmul2_rn(a0, e1));
    pn = __ffma2_rn(a2, reuse, pn);
    const float2 pv = __ffma2_rn(ps, p, pn);
    psi0 = pv.x;
    psi1 = pv.y;
    tal0 = tl.x;
    tal1 = tl.y;
    pm0 = p.x;
    pm1 = p.y;
}

// VEC groups of one lane. PAIRS (VEC even): x holds the groups in the pair layout, two
// float4 per pair of groups, (sigT_a, sigT_b, q0_a, q0_b) and (q1mu_a, q1mu_b, q2mu2_a,
// q2mu2_b), and each pair goes through the packed arithmetic with its operands already in
// adjacent registers. Otherwise x holds one float4 per group.
template <int VEC, int EK, bool PAIRS>
__device__ __forceinline__ void attenuate_row(const float4 (&x)[VEC], float ds, float weight,
                                              const TableRef &tr, Vec<VEC> &psi,
                                              Vec<VEC> &tally, Vec<VEC> &pmul)
{
    if constexpr (PAIRS) {
        static_assert(VEC % 2 == 0, "the pair layout holds whole pairs");
#pragma unroll
        for (int k = 0; k < VEC; k += 2)
            attenuate_pair<EK>(x[k], x[k + 1], ds, weight, tr, psi.v[k], psi.v[k + 1],
                               tally.v[k], tally.v[k + 1], pmul.v[k], pmul.v[k + 1]);
    } else {
#pragma unroll
        for (int k = 0; k < VEC; k++)
            attenuate_one<EK>(x[k], ds, weight, tr, psi.v[k], tally.v[k], pmul.v[k]);
    }
}

}  // namespace moc
