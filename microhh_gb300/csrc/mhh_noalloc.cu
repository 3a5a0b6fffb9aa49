// mhh_noalloc.cu -- maximum absolute divergence without any device
// allocation.
//
// Some callers must not allocate device memory once they are set up.
// Examples are a host that charges every device allocation against a fixed
// HBM budget, and code that runs where a cudaMalloc/cudaFree pair could
// synchronise the device in the middle of its work.  For them
// mhh_pres_2_get_divergence_noalloc computes what mhh_pres_2_get_divergence
// computes (src/pres_2.cxx:97-105, :389-422: max over the interior of
// |rho (du/dx + dv/dy) + d(rhoh w)/dz dzi|, in double).  Its scratch is the
// file-scope device array below, not memory of the context or of an
// allocator.
//
// The reduction has two stages, as the reference's reduce_interior
// (src/tools.cu:137-330): one maximum per (j, k) row, then the maximum of the
// rows.  The row maxima take jtot*ktot doubles of the array, so
// jtot*ktot <= MHH_NOALLOC_DIV_MAX_ROWS (262144, i.e. 2 MiB); larger grids
// are rejected with MHH_ERR_ARG.  Every slot that is read is first written in
// the same call, so nothing has to be cleared between calls; the array keeps
// the previous call's values until they are overwritten.
//
// The first call on each device looks up the array's device address
// (cudaGetSymbolAddress, with that device current) and keeps it.  CUDA loads
// a library's kernels lazily by default, so that first call can also load
// this file's module, which places the 2 MiB array in device memory and may
// synchronise the device.  Callers therefore make one warm-up call during
// their own set-up, before any stream capture; later calls allocate nothing
// and do not load anything.  All calls on one device share the array: calls
// that overlap in time (other host threads, or other streams whose work is
// not ordered with this call) race on it and must be serialised by the
// caller.  A NaN anywhere in u, v or w gives a NaN maximum, reported as
// MHH_ERR_NONFINITE.
#include <cmath>
#include <mutex>

#include "mhh_kernels.cuh"

namespace mhh
{
    namespace
    {
        constexpr int MHH_NOALLOC_DIV_MAX_ROWS = 262144;
        constexpr int NOALLOC_MAX_DEVICES = 64;

        // Row maxima [0, MAX_ROWS), then the final maximum at MAX_ROWS.
        static __device__ __align__(256) double g_div_scratch[MHH_NOALLOC_DIV_MAX_ROWS + 32];

        std::mutex g_setup_mutex;
        double* g_scratch_ptr[NOALLOC_MAX_DEVICES] = {};

        int fail_na(int code, const char* msg) { mhh_set_last_error(msg); return code; }

        // Device address of the scratch array on the current device, looked up
        // once per device.
        int scratch_address(double** out)
        {
            int dev = -1;
            if (cudaGetDevice(&dev) != cudaSuccess) return fail_na(MHH_ERR_CUDA, "cudaGetDevice failed");
            if (dev < 0 || dev >= NOALLOC_MAX_DEVICES) return fail_na(MHH_ERR_UNSUPPORTED, "device ordinal out of range");
            std::lock_guard<std::mutex> lock(g_setup_mutex);
            if (!g_scratch_ptr[dev])
            {
                void* p = nullptr;
                const cudaError_t rc = cudaGetSymbolAddress(&p, g_div_scratch);
                if (rc != cudaSuccess || !p) return fail_na(MHH_ERR_CUDA, cudaGetErrorString(rc));
                g_scratch_ptr[dev] = static_cast<double*>(p);
            }
            *out = g_scratch_ptr[dev];
            return MHH_OK;
        }
    }

    // One block per interior (j, k) row: the row's maximum |divergence|.
    template<typename TF>
    __global__ void __launch_bounds__(128)
    k_div_rows(Dims d, Prof<TF> pr, const TF* __restrict__ u, const TF* __restrict__ v,
               const TF* __restrict__ w, double* __restrict__ rows)
    {
        const int j = d.jstart + blockIdx.x;
        const int k = d.kstart + blockIdx.y;
        const long long ii = 1, jj = d.icells, kk = d.ijcells;
        double val = 0.;
        for (int i = d.istart + threadIdx.x; i < d.iend; i += blockDim.x)
        {
            const long long c = ijk(d, i, j, k);
            const double div = double(ld(pr.rhoref, k))*(double(ld(u, c+ii)-ld(u, c))*d.dxi + double(ld(v, c+jj)-ld(v, c))*d.dyi)
                             + (double(ld(pr.rhorefh, k+1))*double(ld(w, c+kk)) - double(ld(pr.rhorefh, k))*double(ld(w, c)))*double(ld(pr.dzi, k));
            val = max_nan(val, fabs(div));
        }
        for (int o=16; o>0; o>>=1)
            val = max_nan(val, __shfl_xor_sync(0xffffffffu, val, o));
        __shared__ double sm[4];
        const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
        if (lane == 0) sm[warp] = val;
        __syncthreads();
        if (threadIdx.x == 0)
            rows[blockIdx.x + (long long)blockIdx.y*gridDim.x] = max_nan(max_nan(sm[0], sm[1]), max_nan(sm[2], sm[3]));
    }

    // One block: the maximum of n row maxima into *out.
    __global__ void __launch_bounds__(1024)
    k_rows_max(const double* __restrict__ rows, int n, double* __restrict__ out)
    {
        double val = 0.;
        for (int q = threadIdx.x; q < n; q += blockDim.x)
            val = max_nan(val, rows[q]);
        for (int o=16; o>0; o>>=1)
            val = max_nan(val, __shfl_xor_sync(0xffffffffu, val, o));
        __shared__ double sm[32];
        const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
        if (lane == 0) sm[warp] = val;
        __syncthreads();
        if (warp == 0)
        {
            val = sm[lane];
            for (int o=16; o>0; o>>=1)
                val = max_nan(val, __shfl_xor_sync(0xffffffffu, val, o));
            if (lane == 0) *out = val;
        }
    }

    template<typename TF>
    static void launch_div_noalloc(const Dims& d, const Prof<TF>& pr, const mhh_fields* f, double* scratch,
                                   cudaStream_t s)
    {
        dim3 grid(d.jtot, d.ktot);
        k_div_rows<TF><<<grid, 128, 0, s>>>(d, pr, static_cast<const TF*>(f->u), static_cast<const TF*>(f->v),
                                            static_cast<const TF*>(f->w), scratch);
        k_rows_max<<<1, 1024, 0, s>>>(scratch, d.jtot*d.ktot, scratch + MHH_NOALLOC_DIV_MAX_ROWS);
        count_launch(2);
    }
}

using namespace mhh;

extern "C" int mhh_pres_2_get_divergence_noalloc(mhh_ctx* ctx, const mhh_fields* f, double* div, cudaStream_t stream)
{
    if (!ctx || !f || !div || !f->u || !f->v || !f->w) return fail_na(MHH_ERR_ARG, "NULL argument");
    const Dims& d = ctx_dims(ctx);
    if ((long long)d.jtot*d.ktot > MHH_NOALLOC_DIV_MAX_ROWS)
        return fail_na(MHH_ERR_ARG, "grid too large for the no-allocation divergence: jtot*ktot must be <= 262144");
    if (d.ktot > 65535) return fail_na(MHH_ERR_ARG, "ktot must be <= 65535");
    double* scratch = nullptr;
    int rc = scratch_address(&scratch);
    if (rc) return rc;
    if (ctx_precision(ctx) == MHH_FP64) launch_div_noalloc<double>(d, ctx_prof_double(ctx), f, scratch, stream);
    else launch_div_noalloc<float>(d, ctx_prof_float(ctx), f, scratch, stream);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail_na(MHH_ERR_CUDA, cudaGetErrorString(e));
    double v = 0.;
    e = cudaMemcpyAsync(&v, scratch + MHH_NOALLOC_DIV_MAX_ROWS, sizeof(double), cudaMemcpyDeviceToHost, stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
    if (e != cudaSuccess) return fail_na(MHH_ERR_CUDA, cudaGetErrorString(e));
    *div = v;
    if (!std::isfinite(v)) return fail_na(MHH_ERR_NONFINITE, "reduction is not finite");
    return MHH_OK;
}
