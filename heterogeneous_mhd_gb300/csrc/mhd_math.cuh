// Per-cell arithmetic of the MHD step in two policies.
//
//   EX = true  ("exact"): the reference's own evaluation order and types.
//       The reference is C on float data, so each double literal (2.0, 4.0,
//       0.9 ...) promotes its sub-expression to double; those promotions are
//       kept (type W = double) and every abXYc "a*X + b*Y + c" keeps its
//       +0 and 0*Y terms.  The translation unit that instantiates EX = true is
//       compiled with --fmad=false, so results equal the reference built with
//       -ffp-contract=off bit for bit.
//   EX = false ("fast"): the same algorithm in the working precision R with
//       FMA contraction and one reciprocal per division by rho or c.
//
// Every function names the reference lines it restates.
#pragma once
#include <cuda_runtime.h>
#include <type_traits>

namespace mhd {

template <typename R, bool EX>
using wide_t = typename std::conditional<EX, double, R>::type;

template <typename R>
__device__ __forceinline__ R rabs(R x)
{
    return fabs(x);
}
template <>
__device__ __forceinline__ float rabs<float>(float x)
{
    return fabsf(x);
}

// FAST-policy division, reciprocal and square root: the SFU approximations
// (a few ulp) in FP32, IEEE in FP64.
template <typename R>
__device__ __forceinline__ R fast_rcp(R x)
{
    return R(1) / x;
}
template <>
__device__ __forceinline__ float fast_rcp<float>(float x)
{
    return __fdividef(1.0f, x);
}
template <typename R>
__device__ __forceinline__ R fast_div(R x, R y)
{
    return x / y;
}
template <>
__device__ __forceinline__ float fast_div<float>(float x, float y)
{
    return __fdividef(x, y);
}
template <typename R>
__device__ __forceinline__ R fast_sqrt(R x)
{
    return sqrt(x);
}
template <>
__device__ __forceinline__ float fast_sqrt<float>(float x)
{
    float r;
    asm("sqrt.approx.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

// abXYc_matrix2D with c = 0 (C/includefunc_spu.h:73-84): a*X + b*Y + 0.
template <typename R, bool EX>
__device__ __forceinline__ R lin(R a, R x, R b, R y)
{
    if constexpr (EX)
        return (a * x + b * y) + R(0);
    else
        return a * x + b * y;
}

// c*X + 0*X + 0 (the "fr = c*wr" form of C/tvd1.c:40,43,58,84).
template <typename R, bool EX>
__device__ __forceinline__ R scale0(R c, R x)
{
    if constexpr (EX)
        return (c * x + R(0) * x) + R(0);
    else
        return c * x;
}

// Limiter of C/tvd1.c:71-81,97-107 and C/tvdb.c:72-76:
// 0 unless a*b > 0, else 2ab/(a+b) (in double in the reference).
template <typename R, bool EX>
__device__ __forceinline__ R vanleer(R a, R b)
{
    using W = wide_t<R, EX>;
    if constexpr (EX) {
        R r = R(0);
        if (a * b > R(0))
            r = R(W(2.0) * W(a) * W(b) / W(a + b));
        return r;
    } else {  // branch-free: quotient for every cell, then the select
        const R ab = a * b;
        const R q = fast_div(R(2) * ab, a + b);
        return (ab > R(0)) ? q : R(0);
    }
}

// mhdflux for one cell (C/mhdflux.c:21-46): flux v (before division by the
// pencil max c) and the cell's fast speed ci.  q = u record, f = cell-centred B.
template <typename R, bool EX>
__device__ __forceinline__ void cell_flux(const R q[5], const R f[3], R v[5], R& ci)
{
    using W = wide_t<R, EX>;
    const R gamma = R(5.0 / 3.0);
    if constexpr (EX) {
        R vx = q[1] / q[0];
        R mm = q[1] * q[1] + q[2] * q[2] + q[3] * q[3];
        R bb = f[0] * f[0] + f[1] * f[1] + f[2] * f[2];
        R ps = R((W(q[4]) - W(mm / q[0]) / W(2.0)) * (W(gamma) - W(1.0)) +
                 (W(2.0) - W(gamma)) * W(bb) / W(2.0));
        v[0] = q[1];
        v[1] = q[1] * vx + ps - f[0] * f[0];
        v[2] = q[2] * vx - f[1] * f[0];
        v[3] = q[3] * vx - f[2] * f[0];
        v[4] = (q[4] + ps) * vx - f[0] * (f[0] * q[1] + f[1] * q[2] + f[2] * q[3]) / q[0];
        R p = R(W(ps) - W(bb) / W(2.0));
        ci = R(fabs(W(vx)) + sqrt(fabs(W((bb + gamma * p) / q[0]))));
    } else {
        const R ri = fast_rcp(q[0]);
        const R vx = q[1] * ri;
        const R mm = q[1] * q[1] + q[2] * q[2] + q[3] * q[3];
        const R bb = f[0] * f[0] + f[1] * f[1] + f[2] * f[2];
        const R ps = (q[4] - R(0.5) * mm * ri) * (gamma - R(1)) + R(0.5) * (R(2) - gamma) * bb;
        v[0] = q[1];
        v[1] = q[1] * vx + ps - f[0] * f[0];
        v[2] = q[2] * vx - f[1] * f[0];
        v[3] = q[3] * vx - f[2] * f[0];
        v[4] = (q[4] + ps) * vx - f[0] * (f[0] * q[1] + f[1] * q[2] + f[2] * q[3]) * ri;
        const R p = ps - R(0.5) * bb;
        ci = rabs(vx) + fast_sqrt(rabs((bb + gamma * p) * ri));
    }
}

// Divide the flux by the pencil max when it is positive (C/mhdflux.c:48-57).
template <typename R, bool EX>
__device__ __forceinline__ void scale_flux(R v[5], R c)
{
    if (c > R(0)) {
        if constexpr (EX) {
#pragma unroll
            for (int q = 0; q < 5; q++)
                v[q] = v[q] / c;
        } else {
            const R rc = fast_rcp(c);
#pragma unroll
            for (int q = 0; q < 5; q++)
                v[q] = v[q] * rc;
        }
    }
}

// max_3num (C/calcfl.c:65-89), strict '>' comparisons.
template <typename R>
__device__ __forceinline__ R max3(R a, R b, R c)
{
    if (a > b)
        return (a > c) ? a : c;
    return (b > c) ? b : c;
}

// Per-cell speed of calcfl (C/calcfl.c:44-54), from the face values f = b(:,i,j,k).
template <typename R, bool EX>
__device__ __forceinline__ R cfl_speed(const R q[5], const R f[3])
{
    using W = wide_t<R, EX>;
    const R gamma = R(5.0 / 3.0);
    if constexpr (EX) {
        R t1 = R(fabs(W(q[1] / q[0])));
        R t2 = R(fabs(W(q[2] / q[0])));
        R t3 = R(fabs(W(q[3] / q[0])));
        R v = max3(t1, t2, t3);
        R mm = q[1] * q[1] + q[2] * q[2] + q[3] * q[3];
        R bb = f[0] * f[0] + f[1] * f[1] + f[2] * f[2];
        R ps = R((W(q[4]) - W(mm / q[0]) / W(2.0)) * (W(gamma) - W(1.0)) +
                 (W(2.0) - W(gamma)) * W(bb) / W(2.0));
        R p = R(W(ps) - W(bb) / W(2.0));
        return R(W(v) + sqrt(fabs(W(bb) * W(2.0) + W(gamma * p)) / W(q[0])));
    } else {
        const R ri = fast_rcp(q[0]);
        const R v = max3(rabs(q[1] * ri), rabs(q[2] * ri), rabs(q[3] * ri));
        const R mm = q[1] * q[1] + q[2] * q[2] + q[3] * q[3];
        const R bb = f[0] * f[0] + f[1] * f[1] + f[2] * f[2];
        const R ps = (q[4] - R(0.5) * mm * ri) * (gamma - R(1)) + R(0.5) * (R(2) - gamma) * bb;
        const R p = ps - R(0.5) * bb;
        return v + fast_sqrt(rabs(bb * R(2) + gamma * p) * ri);
    }
}

}  // namespace mhd
