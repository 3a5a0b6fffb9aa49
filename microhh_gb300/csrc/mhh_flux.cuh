// mhh_flux.cuh -- device helpers shared by the flux-form tendency kernels
// (mhh_tend_flux.cu): asynchronous plane copies and the
// advective face fluxes of src/advec_2i5.cxx:150-728 (6th-order
// interpolation with 5th-order upwind dissipation, lower orders next to the
// walls) and of the flux limiter (include/advec_monotonic.h:28-219).
#pragma once

#include "mhh_common.cuh"
#include "mhh_stencil.cuh"

namespace mhh
{
    // Asynchronous global -> shared copy of one element; a copy with
    // valid == false writes zero and reads nothing.
    template<typename TF>
    __device__ __forceinline__ void cp_async_el(TF* dst, const TF* src, bool valid)
    {
        const unsigned s = (unsigned)__cvta_generic_to_shared(dst);
        const int n = valid ? (int)sizeof(TF) : 0;
        if constexpr (sizeof(TF) == 4)
            asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;\n" :: "r"(s), "l"(src), "r"(n) : "memory");
        else
            asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;\n" :: "r"(s), "l"(src), "r"(n) : "memory");
    }
    __device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
    __device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;\n" ::: "memory"); }

    // Upwind-biased advective flux vel * phi at a face from the six values
    // around it (6th-order interpolation minus 5th-order dissipation).
    template<typename TF>
    __device__ __forceinline__ TF adv6(TF vel, TF a, TF b, TF c, TF d, TF e, TF f)
    {
        return vel*i6ws(a, b, c, d, e, f) - fabs(vel)*i5ws(a, b, c, d, e, f);
    }

    // Two advective fluxes at once in packed float pairs (one FP32x2
    // instruction per pair of operations): the x- and y-face fluxes of one
    // field, or the fluxes of two fields through one face.  Same arithmetic
    // as adv6 per component, fused differently.
    __device__ __forceinline__ float2 adv6x2(float2 vel, float2 a, float2 b, float2 c, float2 d, float2 e, float2 f)
    {
        const float2 one_m = make_float2(-1.f, -1.f);
        const float2 p1 = __fadd2_rn(c, d), p2 = __fadd2_rn(b, e), p3 = __fadd2_rn(a, f);
        const float2 m1 = __ffma2_rn(c, one_m, d), m2 = __ffma2_rn(b, one_m, e), m3 = __ffma2_rn(a, one_m, f);
        const float2 i6 = __ffma2_rn(p1, make_float2(37.f/60.f, 37.f/60.f),
                                     __ffma2_rn(p2, make_float2(-8.f/60.f, -8.f/60.f),
                                                __fmul2_rn(p3, make_float2(1.f/60.f, 1.f/60.f))));
        const float2 i5 = __ffma2_rn(m1, make_float2(10.f/60.f, 10.f/60.f),
                                     __ffma2_rn(m2, make_float2(-5.f/60.f, -5.f/60.f),
                                                __fmul2_rn(m3, make_float2(1.f/60.f, 1.f/60.f))));
        const float2 nav = make_float2(-fabsf(vel.x), -fabsf(vel.y));
        return __ffma2_rn(vel, i6, __fmul2_rn(nav, i5));
    }

    __device__ __forceinline__ float2 f2(float x, float y) { return make_float2(x, y); }
    __device__ __forceinline__ float2 sub2(float2 a, float2 b) { return __ffma2_rn(b, make_float2(-1.f, -1.f), a); }

    // Vertical advective fluxes of two fields (queues qa, qb) through the
    // same face with face velocities wf.x, wf.y (order as zadv).
    __device__ __forceinline__ float2 zadv2(const float (&qa)[6], const float (&qb)[6], float2 wf, int order)
    {
        if (order == 6)
            return adv6x2(wf, f2(qa[0], qb[0]), f2(qa[1], qb[1]), f2(qa[2], qb[2]), f2(qa[3], qb[3]),
                          f2(qa[4], qb[4]), f2(qa[5], qb[5]));
        if (order == 4)
            return f2(wf.x*i4ws(qa[1], qa[2], qa[3], qa[4]) - fabsf(wf.x)*i3ws(qa[1], qa[2], qa[3], qa[4]),
                      wf.y*i4ws(qb[1], qb[2], qb[3], qb[4]) - fabsf(wf.y)*i3ws(qb[1], qb[2], qb[3], qb[4]));
        if (order == 2) return f2(wf.x*i2(qa[2], qa[3]), wf.y*i2(qb[2], qb[3]));
        return f2(0.f, 0.f);
    }

    // Vertical advective flux through the face between queue entries 2 and 3
    // (queue entry q holds level m-2+q of the own column).
    template<typename TF>
    __device__ __forceinline__ TF zadv(const TF (&q)[6], TF wf, int order)
    {
        if (order == 6) return adv6(wf, q[0], q[1], q[2], q[3], q[4], q[5]);
        if (order == 4) return wf*i4ws(q[1], q[2], q[3], q[4]) - fabs(wf)*i3ws(q[1], q[2], q[3], q[4]);
        if (order == 2) return wf*i2(q[2], q[3]);
        return TF(0);
    }

    // Limited advective flux through the face between sm1 and sp1 (values
    // sm2, sm1 | sp1, sp2 along the flow axis); side as for flux_koren.
    template<typename TF>
    __device__ __forceinline__ TF lim_flux(TF vel, TF sm2, TF sm1, TF sp1, TF sp2, int side)
    {
        if (vel >= TF(0)) return side < 0 ? vel*sm1 : vel*koren_face(sm1, sm2, sp1);
        return side > 0 ? vel*sp1 : vel*koren_face(sp1, sp2, sm1);
    }

}
