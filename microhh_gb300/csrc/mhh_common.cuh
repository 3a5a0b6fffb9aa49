// mhh_common.cuh -- shared device types and helpers of the LES/DNS kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "mhh.h"

namespace mhh
{
    // Grid dimensions as kernel parameters (by value).
    struct Dims
    {
        int itot, jtot, ktot;
        int igc, jgc, kgc;
        int icells, jcells, kcells, ijcells;
        int istart, iend, jstart, jend, kstart, kend;
        long long ncells;
        double dx, dy, dxi, dyi, zsize;
        float fdxi, fdyi, fzsize;   // the same in float, so float kernels convert nothing
    };

    // 1/dx, 1/dy and zsize in the kernel's precision.
    template<typename TF> __device__ __forceinline__ TF dxi_of(const Dims& d);
    template<> __device__ __forceinline__ double dxi_of<double>(const Dims& d) { return d.dxi; }
    template<> __device__ __forceinline__ float dxi_of<float>(const Dims& d) { return d.fdxi; }
    template<typename TF> __device__ __forceinline__ TF dyi_of(const Dims& d);
    template<> __device__ __forceinline__ double dyi_of<double>(const Dims& d) { return d.dyi; }
    template<> __device__ __forceinline__ float dyi_of<float>(const Dims& d) { return d.fdyi; }
    template<typename TF> __device__ __forceinline__ TF zsize_of(const Dims& d);
    template<> __device__ __forceinline__ double zsize_of<double>(const Dims& d) { return d.zsize; }
    template<> __device__ __forceinline__ float zsize_of<float>(const Dims& d) { return d.fzsize; }

    // Vertical profiles of one precision (device pointers, kcells each).
    template<typename TF>
    struct Prof
    {
        const TF *z, *zh, *dz, *dzh, *dzi, *dzhi;
        const TF *rhoref, *rhorefh;
        const TF *thref, *threfh;
        const TF *zfac, *zfach;     // dzi/rhoref and dzhi/rhorefh
        // The reference potential temperature in the units the scalar is
        // stored in (thref minus the context's storage offset of theta).
        const TF *thb, *thbh;
    };

    __host__ __device__ inline long long ijk(const Dims& d, int i, int j, int k)
    {
        return (long long)i + (long long)j*d.icells + (long long)k*d.ijcells;
    }

    template<typename TF> __device__ __forceinline__ TF ld(const TF* p, long long n) { return __ldg(p + n); }

    template<typename TF> __device__ __forceinline__ TF sq(TF a) { return a*a; }

    // Stencil primitives, include/finite_difference.h:35-157.
    template<typename TF> __device__ __forceinline__ TF i2(TF a, TF b) { return TF(0.5)*(a + b); }
    template<typename TF> __device__ __forceinline__ TF i4ws(TF a, TF b, TF c, TF d)
    { return TF(7./12.)*(b + c) - TF(1./12.)*(a + d); }
    template<typename TF> __device__ __forceinline__ TF i3ws(TF a, TF b, TF c, TF d)
    { return TF(3./12.)*(c - b) - TF(1./12.)*(d - a); }
    template<typename TF> __device__ __forceinline__ TF i6ws(TF a, TF b, TF c, TF d, TF e, TF f)
    { return TF(37./60.)*(c + d) - TF(8./60.)*(b + e) + TF(1./60.)*(a + f); }
    template<typename TF> __device__ __forceinline__ TF i5ws(TF a, TF b, TF c, TF d, TF e, TF f)
    { return TF(10./60.)*(d - c) - TF(5./60.)*(e - b) + TF(1./60.)*(f - a); }

    // Face interpolations between a[c-s] and a[c] from a[c-3s] .. a[c+2s].
    template<typename TF> __device__ __forceinline__ TF f6(const TF* a, long long c, long long s)
    { return i6ws(ld(a, c-3*s), ld(a, c-2*s), ld(a, c-s), ld(a, c), ld(a, c+s), ld(a, c+2*s)); }
    template<typename TF> __device__ __forceinline__ TF f5(const TF* a, long long c, long long s)
    { return i5ws(ld(a, c-3*s), ld(a, c-2*s), ld(a, c-s), ld(a, c), ld(a, c+s), ld(a, c+2*s)); }
    template<typename TF> __device__ __forceinline__ TF f4(const TF* a, long long c, long long s)
    { return i4ws(ld(a, c-2*s), ld(a, c-s), ld(a, c), ld(a, c+s)); }
    template<typename TF> __device__ __forceinline__ TF f3(const TF* a, long long c, long long s)
    { return i3ws(ld(a, c-2*s), ld(a, c-s), ld(a, c), ld(a, c+s)); }
    template<typename TF> __device__ __forceinline__ TF f2(const TF* a, long long c, long long s)
    { return i2(ld(a, c-s), ld(a, c)); }

    // Monotone max of non-negative doubles through their bit patterns
    // (a NaN, bit pattern above +inf, wins, so a blow-up is reported).
    // A product rounded on its own in double, never contracted with a
    // following addition into an FMA.  The FP64 path uses it where the
    // reference's CPU build rounds large elementwise terms separately (u/dt
    // in the pressure right-hand side, the pressure gradient, the RK3
    // update): the level sums of the right-hand side feed the mean-mode
    // pressure solve, whose conditioning amplifies any difference in their
    // round-off.  In float the compiler may contract as usual.
    __device__ __forceinline__ double mulx(double a, double b) { return __dmul_rn(a, b); }
    __device__ __forceinline__ float mulx(float a, float b) { return a*b; }

    // Maximum that keeps a NaN of either operand.  fmax returns the other
    // operand when one is NaN, which would turn a blown-up field into a
    // finite CFL, diffusion number or divergence.
    template<typename T> __device__ __forceinline__ T max_nan(T a, T b) { return (a != a || a > b) ? a : b; }

    // Maximum of non-negative doubles on their bit patterns, which order like
    // the values.  A NaN is stored as the positive quiet NaN, whose pattern
    // is above that of +inf, so it survives every later maximum.
    __device__ __forceinline__ void atomic_max_nonneg(unsigned long long* dst, double v)
    {
        const unsigned long long bits = v != v ? 0x7ff8000000000000ull : (unsigned long long)__double_as_longlong(v);
        atomicMax(dst, bits);
    }

    // Exact float <-> double conversions on the integer pipe (IEEE 754
    // binary32/binary64 layouts): the FP64 pipe of this GPU is narrow and
    // its conversions would cost as much as the solve.  Zeros, subnormals,
    // infinities, NaNs and results outside the normal float range take the
    // hardware conversion.
    __device__ __forceinline__ double f2d_exact(float f)
    {
        const unsigned u = __float_as_uint(f);
        const unsigned e = (u >> 23) & 0xffu;
        if (e == 0u || e == 0xffu)
            return (u << 1) == 0u ? __hiloint2double(int(u & 0x80000000u), 0) : double(f);
        const unsigned hi = (u & 0x80000000u) | ((e + 896u) << 20) | ((u >> 3) & 0xfffffu);
        return __hiloint2double(int(hi), int(u << 29));
    }

    // Round to nearest, ties to even.
    __device__ __forceinline__ float d2f_rn(double x)
    {
        const unsigned hi = unsigned(__double2hiint(x)), lo = unsigned(__double2loint(x));
        const unsigned e = (hi >> 20) & 0x7ffu;
        if (e < 897u || e > 1150u) return float(x);
        const unsigned r = (((hi & 0x7fffffffu) << 3) | (lo >> 29)) - (896u << 23);
        const unsigned rem = lo & 0x1fffffffu;
        const unsigned up = (rem > 0x10000000u || (rem == 0x10000000u && (r & 1u))) ? 1u : 0u;
        return __uint_as_float((hi & 0x80000000u) | (r + up));
    }

    // A double of the 2-D surface state in the compute type CT, and back.
    template<typename CT> __device__ __forceinline__ CT from_d(double x);
    template<> __device__ __forceinline__ double from_d<double>(double x) { return x; }
    template<> __device__ __forceinline__ float from_d<float>(double x) { return d2f_rn(x); }
    template<typename CT> __device__ __forceinline__ double to_d(CT x);
    template<> __device__ __forceinline__ double to_d<double>(double x) { return x; }
    template<> __device__ __forceinline__ double to_d<float>(float x) { return f2d_exact(x); }

    constexpr double KAPPA = 0.4;   // include/constants.h:28
    constexpr double GRAV = 9.81;   // include/constants.h:29
    constexpr double DSMALL = 1.e-9;
    constexpr double DBIG = 1.e9;
    constexpr int NZL_LUT = 10000;  // include/boundary.h:56
}

// Error convention of the C-ABI: 0 = ok; negative = mhh_status.
#define MHH_CUDA_TRY(call) do { cudaError_t e_ = (call); if (e_ != cudaSuccess) { mhh_set_last_error(cudaGetErrorString(e_)); return MHH_ERR_CUDA; } } while (0)
void mhh_set_last_error(const char* msg);
