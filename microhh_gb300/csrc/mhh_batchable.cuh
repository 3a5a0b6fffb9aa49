// mhh_batchable.cuh -- kernels that run either for one context or for many
// contexts (ensemble members, served jobs) in one launch.
//
// A kernel of the substep is written as a body over a parameter struct P and
// a block position (VBlock) instead of blockIdx / gridDim.  Two entry points
// wrap the same body: k_one<P, BODY>(P) for a launch of one context, and
// k_many<P, BODY>(ManyArgs<P>) for a launch over up to ManyArgs<P>::NMAX
// contexts, where the contexts' grids are laid end to end in x: context m
// owns the blocks [start[m], start[m+1]) and decomposes its local block
// index into its own (gx, gy, gz) grid.  A body therefore runs with the same
// parameters and block positions in both, and gives the same results bit for
// bit.  k_one takes P by value and runs the body on a local copy; k_many
// takes the contexts' structs as up to 32 KB of __grid_constant__ kernel
// parameters and copies its block's struct to shared memory first.
//
// launch_body() is the one launch site.  Normally it launches k_one.  While
// a batch plan records a context's substep (BatchRecorder), it appends the
// launch (the k_many symbol, the grid, block, shared memory and the bytes of
// P) to the recording instead; the plan then groups equal k_many symbols of
// the same stage into one launch.  A group of one context launches k_one
// with its own grid: k_many's parameter struct is sized for NMAX contexts,
// and the launch of a 32 KB parameter block costs more than its one body.
#pragma once

#include <cstddef>
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

    // Parameters of a launch over n <= NMAX contexts: the block offsets
    // (n + 1 prefix sums of the contexts' block counts), the contexts' grids
    // and their parameter structs.
    template<class P>
    struct ManyArgs
    {
        static constexpr int NMAX_FIT = (32000 - 32) / (int)(sizeof(P) + sizeof(int) + sizeof(int4));
        static constexpr int NMAX = NMAX_FIT < 1 ? 1 : (NMAX_FIT > 128 ? 128 : NMAX_FIT);
        int4 grid[NMAX];
        P p[NMAX];
        int start[NMAX + 1];
        int n;
    };

    // The context of this block and its block position within the context.
    template<class P>
    __device__ __forceinline__ int batch_find(const ManyArgs<P>& a, VBlock& vb)
    {
        const int b = blockIdx.x;
        int lo = 0, hi = a.n - 1;
        while (lo < hi)
        {
            const int mid = (lo + hi + 1) >> 1;
            if (a.start[mid] <= b) lo = mid; else hi = mid - 1;
        }
        const int4 g = a.grid[lo];
        const int local = b - a.start[lo];
        vb.gx = g.x; vb.gy = g.y; vb.gz = g.z;
        vb.x = local % g.x;
        vb.y = (local / g.x) % g.y;
        vb.z = local / (g.x*g.y);
        return lo;
    }

    // The body binds a reference to a local copy of the parameter: bound to
    // the kernel parameter itself, the reference made the compiler treat the
    // parameter as addressable memory, which cost the flux-form tendency
    // kernel 5% more instructions and time than a kernel whose body reads a
    // local struct.
    template<class P, void (*BODY)(const P&, const VBlock&), int MAXT, int MINB>
    __global__ void __launch_bounds__(MAXT, MINB) k_one(P p)
    {
        const P q = p;
        BODY(q, vblock_self());
    }

    // The block's parameters are staged in shared memory before the body
    // runs: read through a run-time index into the parameter space they would
    // be loads the compiler may not hoist across the body's global stores,
    // which changes where it contracts products into FMAs and so the last bit
    // of float results.  From shared memory the body compiles to the same
    // arithmetic as in k_one.
    template<class P, void (*BODY)(const P&, const VBlock&), int MAXT, int MINB>
    __global__ void __launch_bounds__(MAXT, MINB) k_many(const __grid_constant__ ManyArgs<P> a)
    {
        static_assert(sizeof(P) % 4 == 0, "parameter structs are word-sized");
        __shared__ __align__(16) unsigned int pbuf[sizeof(P)/4];
        VBlock vb;
        const int m = batch_find(a, vb);
        const unsigned int* src = reinterpret_cast<const unsigned int*>(&a.p[m]);
        const int tid = threadIdx.x + blockDim.x*(threadIdx.y + blockDim.y*threadIdx.z);
        const int nt = blockDim.x*blockDim.y*blockDim.z;
        for (int q = tid; q < (int)(sizeof(P)/4); q += nt) pbuf[q] = src[q];
        __syncthreads();
        BODY(*reinterpret_cast<const P*>(pbuf), vb);
    }

    // One recorded launch of one context, with the layout of the k_many
    // parameter struct it would join.
    struct RecordedLaunch
    {
        const void* fn;                       // the k_many entry point
        const void* fn_one;                   // the k_one entry point
        dim3 grid, block;
        size_t smem;
        std::vector<unsigned char> params;    // the bytes of P
        int nmax;                             // ManyArgs<P>::NMAX
        size_t args_size, off_grid, off_p, off_start, off_n;
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
            l.fn_one = reinterpret_cast<const void*>(k_one<P, BODY, MAXT, MINB>);
            l.grid = grid; l.block = block; l.smem = smem;
            l.params.resize(sizeof(P));
            std::memcpy(l.params.data(), &p, sizeof(P));
            using A = ManyArgs<P>;
            l.nmax = A::NMAX;
            l.args_size = sizeof(A);
            l.off_grid = offsetof(A, grid); l.off_p = offsetof(A, p);
            l.off_start = offsetof(A, start); l.off_n = offsetof(A, n);
            r->launches.push_back(std::move(l));
            return;
        }
        k_one<P, BODY, MAXT, MINB><<<grid, block, smem, s>>>(p);
    }
}
