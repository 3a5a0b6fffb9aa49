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
    __device__ __forceinline__ void atomic_max_nonneg(unsigned long long* dst, double v)
    {
        atomicMax(dst, (unsigned long long)__double_as_longlong(v));
    }

    constexpr double KAPPA = 0.4;   // include/constants.h:28
    constexpr double GRAV = 9.81;   // include/constants.h:29
    constexpr double DSMALL = 1.e-9;
    constexpr double DBIG = 1.e9;
    constexpr int NZL_LUT = 10000;  // include/boundary.h:56
}

// Error convention of the C-ABI: 0 = ok; negative = mhh_status.
#define MHH_CUDA_TRY(call) do { cudaError_t e_ = (call); if (e_ != cudaSuccess) { mhh_set_last_error(cudaGetErrorString(e_)); return MHH_ERR_CUDA; } } while (0)
void mhh_set_last_error(const char* msg);
