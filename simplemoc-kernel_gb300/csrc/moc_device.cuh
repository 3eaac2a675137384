// moc_device.cuh — device helpers shared by the sweep kernels (sm_103a).
//
// Vector loads of table rows, vector tally reductions (red.global.add.v4.f32, sm_90+),
// the exponential in its two evaluation modes, and the reciprocal.
#pragma once

#include <cstdint>
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

namespace moc {

// ------------------------------------------------------------------------------------
// Row vectors: VEC consecutive groups held by one lane.
// ------------------------------------------------------------------------------------
template <int VEC>
struct Vec {
    float v[VEC];
};

// Read-only row load through the non-coherent path, kept in L2 (rows are re-read by
// many segments). Requires 4*VEC-byte alignment.
template <int VEC>
__device__ __forceinline__ Vec<VEC> ld_row(const float *p)
{
    Vec<VEC> r;
    if constexpr (VEC == 4) {
        float4 x = __ldg(reinterpret_cast<const float4 *>(p));
        r.v[0] = x.x; r.v[1] = x.y; r.v[2] = x.z; r.v[3] = x.w;
    } else if constexpr (VEC == 2) {
        float2 x = __ldg(reinterpret_cast<const float2 *>(p));
        r.v[0] = x.x; r.v[1] = x.y;
    } else {
        r.v[0] = __ldg(p);
    }
    return r;
}

// Two consecutive float4 (32 bytes, 32-byte aligned) in one 256-bit read-only load.
__device__ __forceinline__ void ldg_2x4(const float4 *p, float4 &a, float4 &b)
{
    asm("ld.global.nc.v8.f32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
        : "=f"(a.x), "=f"(a.y), "=f"(a.z), "=f"(a.w), "=f"(b.x), "=f"(b.y), "=f"(b.z),
          "=f"(b.w)
        : "l"(p));
}

// Plain (coherent) row load/store for psi, which the sweep owns.
template <int VEC>
__device__ __forceinline__ Vec<VEC> ld_psi(const float *p, int n_valid)
{
    Vec<VEC> r;
    if (n_valid >= VEC) {
        if constexpr (VEC == 4) {
            float4 x = *reinterpret_cast<const float4 *>(p);
            r.v[0] = x.x; r.v[1] = x.y; r.v[2] = x.z; r.v[3] = x.w;
        } else if constexpr (VEC == 2) {
            float2 x = *reinterpret_cast<const float2 *>(p);
            r.v[0] = x.x; r.v[1] = x.y;
        } else {
            r.v[0] = *p;
        }
    } else {
#pragma unroll
        for (int k = 0; k < VEC; k++) r.v[k] = k < n_valid ? p[k] : 0.0f;
    }
    return r;
}

template <int VEC>
__device__ __forceinline__ void st_psi(float *p, const Vec<VEC> &r, int n_valid)
{
    if (n_valid >= VEC) {
        if constexpr (VEC == 4) {
            *reinterpret_cast<float4 *>(p) = make_float4(r.v[0], r.v[1], r.v[2], r.v[3]);
        } else if constexpr (VEC == 2) {
            *reinterpret_cast<float2 *>(p) = make_float2(r.v[0], r.v[1]);
        } else {
            *p = r.v[0];
        }
    } else {
#pragma unroll
        for (int k = 0; k < VEC; k++)
            if (k < n_valid) p[k] = r.v[k];
    }
}

// ------------------------------------------------------------------------------------
// Bulk copies (the TMA engine, untiled: cp.async.bulk) into shared memory, completed on
// an mbarrier. The issuing thread declares the bytes it expects (arrive.expect_tx) and
// starts the copy; the barrier's phase completes when every byte has landed. Addresses
// and sizes are multiples of 16 bytes.
// ------------------------------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_addr(const void *p)
{
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}

// Makes initialised barriers visible to the bulk-copy engine before its first use.
__device__ __forceinline__ void mbar_init_fence()
{
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ void bulk_g2s(uint32_t dst, const void *src, uint32_t bytes,
                                         uint32_t bar)
{
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
        ::"r"(dst), "l"(src), "r"(bytes), "r"(bar)
        : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity)
{
    uint32_t ok;
    asm volatile("{\n\t.reg .pred p;\n\t"
                 "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                 "selp.u32 %0, 1, 0, p;\n\t}"
                 : "=r"(ok)
                 : "r"(bar), "r"(parity)
                 : "memory");
    return ok != 0;
}

// Wait for the barrier's phase of the given parity, for at most limit SM clocks (each
// try_wait returns after a bounded, hardware-chosen time). false: the wait gave up.
__device__ __forceinline__ bool mbar_wait_bounded(uint32_t bar, uint32_t parity,
                                                  long long limit)
{
    if (mbar_try_wait(bar, parity)) return true;
    const long long t0 = clock64();
    while (!mbar_try_wait(bar, parity))
        if (clock64() - t0 > limit) return false;
    return true;
}

// Streaming load of a per-segment descriptor field (read once; evict first).
template <typename T>
__device__ __forceinline__ T ld_stream(const T *p)
{
    return __ldcs(p);
}

// ------------------------------------------------------------------------------------
// Tally reduction: fine_flux[cell][g0 .. g0+VEC) += t. Vector reductions are one L2
// atomic request per lane instead of VEC. Lanes whose row is only partly inside the
// group range fall back to scalar reductions so padding entries are never written.
// ------------------------------------------------------------------------------------
template <int VEC>
__device__ __forceinline__ void red_row(float *p, const Vec<VEC> &t, int n_valid)
{
    if (n_valid >= VEC) {
        if constexpr (VEC == 4) {
            asm volatile("red.global.add.v4.f32 [%0], {%1, %2, %3, %4};" ::"l"(p),
                         "f"(t.v[0]), "f"(t.v[1]), "f"(t.v[2]), "f"(t.v[3])
                         : "memory");
        } else if constexpr (VEC == 2) {
            asm volatile("red.global.add.v2.f32 [%0], {%1, %2};" ::"l"(p), "f"(t.v[0]),
                         "f"(t.v[1])
                         : "memory");
        } else {
            asm volatile("red.global.add.f32 [%0], %1;" ::"l"(p), "f"(t.v[0]) : "memory");
        }
    } else {
#pragma unroll
        for (int k = 0; k < VEC; k++)
            if (k < n_valid)
                asm volatile("red.global.add.f32 [%0], %1;" ::"l"(p + k), "f"(t.v[k])
                             : "memory");
    }
}

// Full-row reduction sent only where (unsigned) cell < lim: lim is R*I for a lane whose
// groups are all real and 0 for a lane past G, so the null cell (index R*I) and idle lanes
// send nothing. One compare and one predicated reduction, no branch.
template <int VEC>
__device__ __forceinline__ void red_row_if(float *p, const Vec<VEC> &t, int cell, int lim)
{
    if constexpr (VEC == 4) {
        asm volatile("{\n\t.reg .pred q;\n\tsetp.lt.u32 q, %5, %6;\n\t"
                     "@q red.global.add.v4.f32 [%0], {%1, %2, %3, %4};\n\t}"
                     ::"l"(p), "f"(t.v[0]), "f"(t.v[1]), "f"(t.v[2]), "f"(t.v[3]), "r"(cell),
                     "r"(lim)
                     : "memory");
    } else if constexpr (VEC == 2) {
        asm volatile("{\n\t.reg .pred q;\n\tsetp.lt.u32 q, %3, %4;\n\t"
                     "@q red.global.add.v2.f32 [%0], {%1, %2};\n\t}"
                     ::"l"(p), "f"(t.v[0]), "f"(t.v[1]), "r"(cell), "r"(lim)
                     : "memory");
    } else {
        asm volatile("{\n\t.reg .pred q;\n\tsetp.lt.u32 q, %2, %3;\n\t"
                     "@q red.global.add.f32 [%0], %1;\n\t}"
                     ::"l"(p), "f"(t.v[0]), "r"(cell), "r"(lim)
                     : "memory");
    }
}

// Compensated tally: hi[g] += t with an atomic that returns the value it added to, then
// the exact rounding error of that addition (Knuth's TwoSum on the returned value) is
// reduced into lo[g]. Every addition into hi is an FP32 round-to-nearest addition of the
// returned value and t, so hi_final + sum(errors) equals hi_start + sum(t) exactly; lo
// only carries second-order error. hi + lo is combined in FP64 at the end.
__device__ __forceinline__ float two_sum_err(float a, float b)
{
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    return __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

template <int VEC>
__device__ __forceinline__ void comp_row(float *hi, float *lo, const Vec<VEC> &t, int n_valid)
{
    Vec<VEC> old, err;
    bool done = false;
    if constexpr (VEC == 4) {
        if (n_valid >= 4) {
            asm volatile("atom.global.add.v4.f32 {%0, %1, %2, %3}, [%4], {%5, %6, %7, %8};"
                         : "=f"(old.v[0]), "=f"(old.v[1]), "=f"(old.v[2]), "=f"(old.v[3])
                         : "l"(hi), "f"(t.v[0]), "f"(t.v[1]), "f"(t.v[2]), "f"(t.v[3])
                         : "memory");
            done = true;
        }
    } else if constexpr (VEC == 2) {
        if (n_valid >= 2) {
            asm volatile("atom.global.add.v2.f32 {%0, %1}, [%2], {%3, %4};"
                         : "=f"(old.v[0]), "=f"(old.v[1])
                         : "l"(hi), "f"(t.v[0]), "f"(t.v[1])
                         : "memory");
            done = true;
        }
    }
    if (!done) {
#pragma unroll
        for (int k = 0; k < VEC; k++)
            old.v[k] = k < n_valid ? atomicAdd(hi + k, t.v[k]) : 0.0f;
    }
#pragma unroll
    for (int k = 0; k < VEC; k++) err.v[k] = two_sum_err(old.v[k], t.v[k]);
    red_row<VEC>(lo, err, n_valid);
}

// FP64 tally: acc[g] += (double) t, one red.global.add.f64 per group.
template <int VEC>
__device__ __forceinline__ void red_row_f64(double *acc, const Vec<VEC> &t, int n_valid)
{
#pragma unroll
    for (int k = 0; k < VEC; k++)
        if (k < n_valid)
            asm volatile("red.global.add.f64 [%0], %1;" ::"l"(acc + k), "d"((double)t.v[k])
                         : "memory");
}

// ------------------------------------------------------------------------------------
// Arithmetic helpers.
// ------------------------------------------------------------------------------------

// Hardware reciprocal approximation (MUFU.RCP), about 1 ulp.
__device__ __forceinline__ float rcp_approx(float x)
{
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

// Hardware base-2 exponential (MUFU.EX2), about 2 ulp; the unit splits its argument into
// integer and fraction itself.
__device__ __forceinline__ float ex2_approx(float x)
{
    float r;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

// The exponential terms of the attenuation, accurate for every tau >= 0:
//   e = 1 - exp(-tau), p = exp(-tau), tme = tau - e,
//   cub = tau(tau(tau-3)+6) - 6e.
// For small tau the direct forms cancel (tme ~ tau^2/2, cub ~ tau^4/4). Below tau = 2
// all four come from s4 = sum_{k>=4} (-1)^k tau^k / k! = tau^4 h(tau):
//   cub = 6 s4,  tme = tau^2 (1/2 - tau/6) + s4,  e = tau - tme,  p = 1 - e,
// none of which cancels there (tme <= tau^2/2, e >= 0.43 tau). h is a degree-6
// polynomial fitted to the series on [0, 2] for least maximum relative error (weighted
// least squares on Chebyshev points, reweighted by the error until it equioscillates):
// evaluated by FP32 Horner steps it is within 1.3e-7 of h, where the series itself
// through tau^16 gives 9.3e-8, in 6 fused multiply-adds instead of 12. From tau = 2 on,
// p = ex2.approx(-tau log2 e): rounding the argument costs p a relative error of about
// tau 2^-24 (2.4e-6 at tau = 40, where p is 4e-18), and p <= e^-2 there, so e = 1 - p,
// tme = tau - e and the cubic (which cancels at most ~5-fold) keep FP32 accuracy.
constexpr float H6_0 = 4.166666791e-02f, H6_1 = -8.333321661e-03f, H6_2 = 1.388796256e-03f,
                H6_3 = -1.981338719e-04f, H6_4 = 2.439518357e-05f, H6_5 = -2.442981440e-06f,
                H6_6 = 1.485006180e-07f;
struct ExpTerms {
    float e, p, tme, cub;
};

// The four terms from the series, valid (and used) below tau = 2.
__device__ __forceinline__ ExpTerms exp_terms_series(float tau)
{
    ExpTerms r;
    float h = fmaf(H6_6, tau, H6_5);
    h = fmaf(h, tau, H6_4);
    h = fmaf(h, tau, H6_3);
    h = fmaf(h, tau, H6_2);
    h = fmaf(h, tau, H6_1);
    h = fmaf(h, tau, H6_0);
    const float t2 = tau * tau;
    const float s4 = h * t2 * t2;
    r.cub = 6.0f * s4;
    r.tme = fmaf(t2, fmaf(tau, -1.0f / 6.0f, 0.5f), s4);
    r.e = tau - r.tme;
    r.p = 1.0f - r.e;
    return r;
}

// The four terms from the exponential, used from tau = 2 on.
__device__ __forceinline__ ExpTerms exp_terms_direct(float tau)
{
    ExpTerms r;
    r.p = ex2_approx(tau * -1.44269504088896341f);
    r.e = 1.0f - r.p;
    r.tme = tau - r.e;
    r.cub = fmaf(tau * tau, tau - 3.0f, 6.0f * r.tme);
    return r;
}

// The series is evaluated for every tau (a warp whose groups straddle tau = 2 would run
// both sides of a branch anyway); the exponential only where a lane has a group at
// tau >= 2, and the larger tau take its terms. (Far above 2 the unused series overflows
// to inf or NaN, which the selection drops.)
__device__ __forceinline__ ExpTerms exp_terms_stable(float tau)
{
    ExpTerms r = exp_terms_series(tau);
    if (tau >= 2.0f) r = exp_terms_direct(tau);
    return r;
}

// exp_terms_stable for two groups at once on the packed FP32 pipe: every packed operation
// stands for the scalar one above in the same order (a - b and 1 - x as fma(b, -1, a) and
// fma(x, -1, 1), which round once to the same value), so the terms are the scalar ones bit
// for bit.
struct ExpTerms2 {
    float2 e, p, tme, cub;
};

__device__ __forceinline__ ExpTerms2 exp_terms_stable2(float2 tau)
{
    ExpTerms2 r;
    const float2 one = make_float2(1.0f, 1.0f), mone = make_float2(-1.0f, -1.0f);
    auto c = [](float v) { return make_float2(v, v); };
    float2 h = __ffma2_rn(c(H6_6), tau, c(H6_5));
    h = __ffma2_rn(h, tau, c(H6_4));
    h = __ffma2_rn(h, tau, c(H6_3));
    h = __ffma2_rn(h, tau, c(H6_2));
    h = __ffma2_rn(h, tau, c(H6_1));
    h = __ffma2_rn(h, tau, c(H6_0));
    const float2 t2 = __fmul2_rn(tau, tau);
    const float2 s4 = __fmul2_rn(__fmul2_rn(h, t2), t2);
    r.cub = __fmul2_rn(c(6.0f), s4);
    r.tme = __ffma2_rn(t2, __ffma2_rn(tau, c(-1.0f / 6.0f), c(0.5f)), s4);
    r.e = __ffma2_rn(r.tme, mone, tau);
    r.p = __ffma2_rn(r.e, mone, one);
    const bool bx = tau.x >= 2.0f, by = tau.y >= 2.0f;
    if (bx || by) {
        const float2 m = __fmul2_rn(tau, c(-1.44269504088896341f));
        const float2 p = make_float2(ex2_approx(m.x), ex2_approx(m.y));
        // each term replaces the series' where tau >= 2 as soon as it is formed
        auto take = [bx, by](float2 &dst, float2 v) {
            if (bx) dst.x = v.x;
            if (by) dst.y = v.y;
        };
        const float2 e = __ffma2_rn(p, mone, one);
        const float2 tme = __ffma2_rn(e, mone, tau);
        take(r.p, p);
        take(r.e, e);
        take(r.tme, tme);
        take(r.cub, __ffma2_rn(__fmul2_rn(tau, tau), __fadd2_rn(tau, c(-3.0f)),
                               __fmul2_rn(c(6.0f), tme)));
    }
    return r;
}

// The reference's table lookup (src/cpu/kernel.c:337-361), rounded exactly as the
// reference's C rounds it: IEEE division, no contraction, truncating conversion.
// tab holds (slope, intercept) pairs in shared memory.
__device__ __forceinline__ float table_lookup(const float2 *tab, int n_points, float dx,
                                              float lookup_max, float x)
{
    if (x > lookup_max) return 1.0f;
    const float q = __fdiv_rn(x, dx);
    const float h = __fmul_rn(0.5f, dx);
    int n = __float2int_rz(__fadd_rn(q, h));
    n = n < 0 ? 0 : (n >= n_points ? n_points - 1 : n);  // never taken for x in domain
    const float2 si = tab[n];
    return __fadd_rn(__fmul_rn(si.x, x), si.y);
}

}  // namespace moc
