// mhh_batchable.cuh -- kernels that run either for one context or for many
// contexts (ensemble members, served jobs) in one launch.
//
// A kernel of the substep is written as a body over a parameter struct P and
// a block position (VBlock) instead of blockIdx / gridDim.  Two entry points
// wrap the same body: k_one<P, BODY>(P) for a launch of one context, and
// k_many<P, BODY>(const P*, BatchMap) for a launch over many contexts, where
// the contexts' grids are laid end to end in x: context m owns the blocks
// [start[m], start[m+1]) and decomposes its local block index into its own
// (gx, gy, gz) grid.  A body therefore runs with the same parameters and
// block positions in both, and gives the same results bit for bit.
//
// launch_body() is the one launch site.  Normally it launches k_one.  While
// a batch plan records a context's substep (BatchRecorder), it appends the
// launch (the k_many symbol, the grid, block, shared memory and the bytes of
// P) to the recording instead; the plan then groups equal k_many symbols of
// the same stage into one launch.
#pragma once

#include <cstring>
#include <vector>

#include "mhh_common.cuh"

namespace mhh
{
    struct VBlock
    {
        int x, y, z;
        int gx, gy, gz;
    };

    __device__ __forceinline__ VBlock vblock_self()
    {
        VBlock b;
        b.x = blockIdx.x; b.y = blockIdx.y; b.z = blockIdx.z;
        b.gx = gridDim.x; b.gy = gridDim.y; b.gz = gridDim.z;
        return b;
    }

    // Block map of a launch over n contexts (device arrays).
    struct BatchMap
    {
        const int* start;     // n + 1 prefix sums of the contexts' block counts
        const int4* grid;     // (gx, gy, gz, 0) of each context
        int n;
    };

    // The context of this block and its block position within the context.
    __device__ __forceinline__ int batch_find(const BatchMap& m, VBlock& vb)
    {
        const int b = blockIdx.x;
        int lo = 0, hi = m.n - 1;
        while (lo < hi)
        {
            const int mid = (lo + hi + 1) >> 1;
            if (__ldg(m.start + mid) <= b) lo = mid; else hi = mid - 1;
        }
        const int4 g = __ldg(m.grid + lo);
        const int local = b - __ldg(m.start + lo);
        vb.gx = g.x; vb.gy = g.y; vb.gz = g.z;
        vb.x = local % g.x;
        vb.y = (local / g.x) % g.y;
        vb.z = local / (g.x*g.y);
        return lo;
    }

    template<class P, void (*BODY)(const P&, const VBlock&), int MAXT, int MINB>
    __global__ void __launch_bounds__(MAXT, MINB) k_one(P p)
    {
        BODY(p, vblock_self());
    }

    // The context's parameters are copied to shared memory first: the body
    // reads them as often as it reads kernel parameters, and from global
    // memory each read would be a load instruction of its own.
    template<class P, void (*BODY)(const P&, const VBlock&), int MAXT, int MINB>
    __global__ void __launch_bounds__(MAXT, MINB) k_many(const P* __restrict__ ps, BatchMap map)
    {
        static_assert(sizeof(P) % 4 == 0, "parameter structs are word-sized");
        __shared__ __align__(16) unsigned int pbuf[sizeof(P)/4];
        VBlock vb;
        const int m = batch_find(map, vb);
        const unsigned int* src = reinterpret_cast<const unsigned int*>(ps + m);
        const int tid = threadIdx.x + blockDim.x*(threadIdx.y + blockDim.y*threadIdx.z);
        const int nt = blockDim.x*blockDim.y*blockDim.z;
        for (int q = tid; q < (int)(sizeof(P)/4); q += nt) pbuf[q] = __ldg(src + q);
        __syncthreads();
        BODY(*reinterpret_cast<const P*>(pbuf), vb);
    }

    // One recorded launch of one context.
    struct RecordedLaunch
    {
        const void* fn;                       // the k_many entry point
        dim3 grid, block;
        size_t smem;
        std::vector<unsigned char> params;    // the bytes of P
    };

    // While set (host thread-local), launch_body records instead of launching.
    struct BatchRecorder
    {
        std::vector<RecordedLaunch> launches;
    };
    BatchRecorder*& batch_recorder();

    // Dynamic shared memory above 48 KB needs the attribute on each entry point.
    template<class P, void (*BODY)(const P&, const VBlock&), int MAXT, int MINB>
    void set_smem_limit(size_t smem)
    {
        if (smem <= 48*1024) return;
        static const bool one = cudaFuncSetAttribute(k_one<P, BODY, MAXT, MINB>,
            cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) == cudaSuccess;
        static const bool many = cudaFuncSetAttribute(k_many<P, BODY, MAXT, MINB>,
            cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) == cudaSuccess;
        (void)one; (void)many;
    }

    template<class P, void (*BODY)(const P&, const VBlock&), int MAXT, int MINB = 1>
    void launch_body(dim3 grid, dim3 block, size_t smem, cudaStream_t s, const P& p)
    {
        set_smem_limit<P, BODY, MAXT, MINB>(smem);
        if (BatchRecorder* r = batch_recorder())
        {
            RecordedLaunch l;
            l.fn = reinterpret_cast<const void*>(k_many<P, BODY, MAXT, MINB>);
            l.grid = grid; l.block = block; l.smem = smem;
            l.params.resize(sizeof(P));
            std::memcpy(l.params.data(), &p, sizeof(P));
            r->launches.push_back(std::move(l));
            return;
        }
        k_one<P, BODY, MAXT, MINB><<<grid, block, smem, s>>>(p);
    }
}
