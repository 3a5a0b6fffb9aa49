// mhh_pres.cu -- the Pres_2 Poisson solve on the GPU without cuFFT:
// divergence of the predicted velocity, hand-written real FFTs along x and y
// (halfcomplex layout, so the spectral solve is the reference's), a Thomas
// solve per spectral column in double, inverse FFTs and the scatter back into
// the ghost-cell layout.
//
// FFT: two real sequences x, y of length n are transformed together as
// z = x + i y with a mixed-radix (4, 2, 3, 5, 7) Stockham autosort FFT in
// shared memory (ping-pong buffers, one barrier per stage), then separated by
// Hermitian symmetry into FFTW's halfcomplex order r_0 .. r_{n/2},
// i_{(n+1)/2-1} .. i_1 (the convention of src/fft.cxx:145-206).
#include <cmath>
#include <cstring>
#include <vector>

#include "mhh_kernels.cuh"

namespace mhh
{
    template<typename TF> struct C2;
    template<> struct C2<double> { using T = double2; };
    template<> struct C2<float> { using T = float2; };

    template<typename T2> __device__ __forceinline__ T2 cmul(T2 a, T2 b)
    {
        T2 r; r.x = a.x*b.x - a.y*b.y; r.y = a.x*b.y + a.y*b.x; return r;
    }
    template<typename T2> __device__ __forceinline__ T2 cadd(T2 a, T2 b) { T2 r; r.x = a.x + b.x; r.y = a.y + b.y; return r; }
    template<typename T2> __device__ __forceinline__ T2 csub(T2 a, T2 b) { T2 r; r.x = a.x - b.x; r.y = a.y - b.y; return r; }

    template<typename TF> __device__ __forceinline__ const TF* twtab(const FftPlan& pl);
    template<> __device__ __forceinline__ const double* twtab<double>(const FftPlan& pl) { return pl.tw_d; }
    template<> __device__ __forceinline__ const float* twtab<float>(const FftPlan& pl) { return pl.tw_f; }

    template<typename TF>
    __device__ __forceinline__ typename C2<TF>::T tw(const TF* t, int e)
    {
        typename C2<TF>::T r; r.x = __ldg(t + 2*e); r.y = __ldg(t + 2*e + 1); return r;
    }

    // All Stockham stages for P sequences of length n held in buf[0] (complex,
    // [P][n]); returns the buffer index that holds the natural-order result.
    template<typename TF>
    __device__ int stockham(const FftPlan& pl, typename C2<TF>::T* buf0, typename C2<TF>::T* buf1, int P)
    {
        using T2 = typename C2<TF>::T;
        const TF* tt = twtab<TF>(pl);
        const int n = pl.n;
        T2* src = buf0;
        T2* dst = buf1;
        int which = 0;
        int p = 1;
        for (int s=0; s<pl.nfac; ++s)
        {
            const int R = pl.fac[s];
            const int T = n / R;
            const int step = n / (p*R);
            const int nitem = P*T;
            for (int it = threadIdx.x; it < nitem; it += blockDim.x)
            {
                const int seq = it / T;
                const int i = it - seq*T;
                const int k = i % p;
                const T2* x = src + seq*n;
                T2* y = dst + seq*n;
                const int j = (i - k)*R + k;
                if (R == 2)
                {
                    T2 u0 = x[i], u1 = cmul(x[i + T], tw<TF>(tt, k*step));
                    y[j] = cadd(u0, u1);
                    y[j + p] = csub(u0, u1);
                }
                else if (R == 4)
                {
                    T2 u0 = x[i];
                    T2 u1 = cmul(x[i +   T], tw<TF>(tt, (1*k*step) % n));
                    T2 u2 = cmul(x[i + 2*T], tw<TF>(tt, (2*k*step) % n));
                    T2 u3 = cmul(x[i + 3*T], tw<TF>(tt, (3*k*step) % n));
                    const T2 a = cadd(u0, u2), b = csub(u0, u2);
                    const T2 c = cadd(u1, u3), e = csub(u1, u3);
                    // v_r = sum_q u_q (-i)^(q r)
                    T2 v1, v3;
                    v1.x = b.x + e.y; v1.y = b.y - e.x;   // b - i e
                    v3.x = b.x - e.y; v3.y = b.y + e.x;   // b + i e
                    y[j] = cadd(a, c);
                    y[j + p] = v1;
                    y[j + 2*p] = csub(a, c);
                    y[j + 3*p] = v3;
                }
                else if (R == 3)
                {
                    T2 u0 = x[i];
                    T2 u1 = cmul(x[i +   T], tw<TF>(tt, (1*k*step) % n));
                    T2 u2 = cmul(x[i + 2*T], tw<TF>(tt, (2*k*step) % n));
                    const TF s3 = TF(0.86602540378443864676);
                    const T2 t1 = cadd(u1, u2), t4 = csub(u1, u2);
                    T2 t2; t2.x = u0.x - TF(0.5)*t1.x; t2.y = u0.y - TF(0.5)*t1.y;
                    // v1 = t2 - i s3 t4, v2 = t2 + i s3 t4
                    T2 v1, v2;
                    v1.x = t2.x + s3*t4.y; v1.y = t2.y - s3*t4.x;
                    v2.x = t2.x - s3*t4.y; v2.y = t2.y + s3*t4.x;
                    y[j] = cadd(u0, t1);
                    y[j + p] = v1;
                    y[j + 2*p] = v2;
                }
                else
                {
                    // General small radix (5, 7): direct DFT with table twiddles.
                    T2 u[7];
                    for (int q=0; q<R; ++q)
                        u[q] = q ? cmul(x[i + q*T], tw<TF>(tt, (int)(((long long)q*k*step) % n))) : x[i];
                    for (int r=0; r<R; ++r)
                    {
                        T2 acc = u[0];
                        for (int q=1; q<R; ++q)
                            acc = cadd(acc, cmul(u[q], tw<TF>(tt, (int)(((long long)q*r*T) % n))));
                        y[j + r*p] = acc;
                    }
                }
            }
            __syncthreads();
            T2* t = src; src = dst; dst = t;
            which ^= 1;
            p *= R;
        }
        return which;
    }

    // Element j of real sequence s sits at base(s) + j*stride:
    //   rows (x):    base = s*n,                         stride = 1
    //   columns (y): base = (s / itot)*itot*n + s % itot, stride = itot
    struct SeqLayout
    {
        int rows;       // 1: contiguous rows; 0: strided columns
        int itot;       // columns per slab (y layout)
        long long nseq; // number of real sequences
    };

    __device__ __forceinline__ long long seq_base(const SeqLayout& L, long long s, int n)
    {
        if (L.rows) return s*(long long)n;
        return (s / L.itot)*(long long)L.itot*n + (s % L.itot);
    }

    // Shared-memory index of element j of local real sequence ls (2P x n, [ls][j]).
    template<typename TF, bool INV>
    __global__ void __launch_bounds__(256)
    k_fft(FftPlan pl, TF* __restrict__ data, SeqLayout L, int P, TF scale)
    {
        using T2 = typename C2<TF>::T;
        extern __shared__ __align__(16) unsigned char smem_raw[];
        const int n = pl.n;
        T2* buf0 = reinterpret_cast<T2*>(smem_raw);
        T2* buf1 = buf0 + (size_t)P*n;
        const long long s0 = (long long)blockIdx.x*2*P;     // first real sequence of this block
        const int nloc = (int)min((long long)2*P, L.nseq - s0);

        // 1. Load 2P real sequences into buf1 viewed as real [2P][n].
        TF* r1 = reinterpret_cast<TF*>(buf1);
        const int tot = 2*P*n;
        if (L.rows)
        {
            for (int e = threadIdx.x; e < tot; e += blockDim.x)
            {
                const int ls = e / n, j = e - ls*n;
                r1[e] = ls < nloc ? data[seq_base(L, s0 + ls, n) + j] : TF(0);
            }
        }
        else
        {
            // Consecutive threads take consecutive columns of one row.
            for (int e = threadIdx.x; e < tot; e += blockDim.x)
            {
                const int j = e / (2*P), ls = e - j*(2*P);
                r1[ls*n + j] = ls < nloc ? data[seq_base(L, s0 + ls, n) + (long long)j*L.itot] : TF(0);
            }
        }
        __syncthreads();

        // 2. Complex input: z = x + i y (forward) or conj(X + i Y) (inverse).
        for (int e = threadIdx.x; e < P*n; e += blockDim.x)
        {
            const int q = e / n, k = e - q*n;
            const TF* hx = r1 + (2*q)*n;
            const TF* hy = r1 + (2*q+1)*n;
            T2 z;
            if (!INV)
            {
                z.x = hx[k]; z.y = hy[k];
            }
            else
            {
                const int kk = k <= n/2 ? k : n - k;
                const TF sg = k <= n/2 ? TF(1) : TF(-1);
                const bool real_only = (kk == 0) || (2*kk == n);
                const TF xr = hx[kk], yr = hy[kk];
                const TF xi = real_only ? TF(0) : sg*hx[n - kk];
                const TF yi = real_only ? TF(0) : sg*hy[n - kk];
                // Z = (xr - yi) + i (xi + yr); store conj(Z).
                z.x = xr - yi;
                z.y = -(xi + yr);
            }
            buf0[e] = z;
        }
        __syncthreads();

        // 3. FFT.
        const int which = stockham<TF>(pl, buf0, buf1, P);
        T2* res = which ? buf1 : buf0;
        TF* rout = reinterpret_cast<TF*>(which ? buf0 : buf1);

        // 4. Real outputs into the other buffer, [2P][n].
        for (int e = threadIdx.x; e < P*n; e += blockDim.x)
        {
            const int q = e / n, k = e - q*n;
            TF* ox = rout + (2*q)*n;
            TF* oy = rout + (2*q+1)*n;
            if (!INV)
            {
                if (k <= n/2)
                {
                    const T2 a = res[q*n + k], b = res[q*n + (n - k) % n];
                    const TF xr = TF(0.5)*(a.x + b.x), xi = TF(0.5)*(a.y - b.y);
                    const TF yr = TF(0.5)*(a.y + b.y), yi = TF(-0.5)*(a.x - b.x);
                    ox[k] = xr; oy[k] = yr;
                    if (k > 0 && k < n - k) { ox[n - k] = xi; oy[n - k] = yi; }
                }
            }
            else
            {
                const T2 a = res[q*n + k];
                ox[k] = a.x*scale;
                oy[k] = -a.y*scale;
            }
        }
        __syncthreads();

        // 5. Store.
        if (L.rows)
        {
            for (int e = threadIdx.x; e < tot; e += blockDim.x)
            {
                const int ls = e / n, j = e - ls*n;
                if (ls < nloc) data[seq_base(L, s0 + ls, n) + j] = rout[e];
            }
        }
        else
        {
            for (int e = threadIdx.x; e < tot; e += blockDim.x)
            {
                const int j = e / (2*P), ls = e - j*(2*P);
                if (ls < nloc) data[seq_base(L, s0 + ls, n) + (long long)j*L.itot] = rout[ls*n + j];
            }
        }
    }

    template<typename TF>
    static int pairs_per_block(int n, bool rows)
    {
        // Two complex buffers of P*n each within 96 KB; columns want at least
        // 16 (float) or 8 (double) adjacent sequences for coalescing.
        const size_t per = 2*sizeof(typename C2<TF>::T)*(size_t)n;
        int P = (int)((96*1024) / per);
        const int want = rows ? 4 : (sizeof(TF) == 4 ? 8 : 4);
        if (P > want) P = want;
        if (P < 1) P = 1;
        return P;
    }

    template<typename TF>
    static void launch_fft(const FftPlan& pl, TF* data, SeqLayout L, bool inverse, TF scale, cudaStream_t s)
    {
        const int n = pl.n;
        if (n == 1) return;
        const int P = pairs_per_block<TF>(n, L.rows != 0);
        const size_t smem = 2*sizeof(typename C2<TF>::T)*(size_t)P*n;
        const long long nblk = (L.nseq + 2*P - 1) / (2*P);
        if (inverse)
        {
            cudaFuncSetAttribute(k_fft<TF, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            k_fft<TF, true><<<(unsigned)nblk, 256, smem, s>>>(pl, data, L, P, scale);
        }
        else
        {
            cudaFuncSetAttribute(k_fft<TF, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            k_fft<TF, false><<<(unsigned)nblk, 256, smem, s>>>(pl, data, L, P, scale);
        }
        count_launch();
    }

    template<typename TF>
    void launch_fft_x(const FftPlan& pl, TF* data, int nrows, bool inverse, double scale, cudaStream_t s)
    {
        SeqLayout L; L.rows = 1; L.itot = 0; L.nseq = nrows;
        launch_fft<TF>(pl, data, L, inverse, TF(scale), s);
    }

    template<typename TF>
    void launch_fft_y(const FftPlan& pl, TF* data, int itot, int jtot, int ktot, bool inverse, double scale, cudaStream_t s)
    {
        SeqLayout L; L.rows = 0; L.itot = itot; L.nseq = (long long)itot*ktot;
        launch_fft<TF>(pl, data, L, inverse, TF(scale), s);
        (void)jtot;
    }

    int fft_plan_init(FftPlan* pl, int n)
    {
        std::memset(pl, 0, sizeof(*pl));
        pl->n = n;
        int r = n;
        const int radices[] = {4, 2, 3, 5, 7};
        for (int q=0; q<5 && r>1; ++q)
            while (r % radices[q] == 0 && pl->nfac < 16) { pl->fac[pl->nfac++] = radices[q]; r /= radices[q]; }
        if (r != 1) return MHH_ERR_UNSUPPORTED;
        std::vector<double> td(2*(size_t)n);
        std::vector<float> tf(2*(size_t)n);
        const long double twopi = 6.283185307179586476925286766559005768L;
        for (int k=0; k<n; ++k)
        {
            const long double ang = -twopi*(long double)k/(long double)n;
            td[2*k] = (double)cosl(ang); td[2*k+1] = (double)sinl(ang);
            tf[2*k] = (float)td[2*k]; tf[2*k+1] = (float)td[2*k+1];
        }
        if (cudaMalloc(&pl->tw_d, sizeof(double)*2*n) != cudaSuccess) return MHH_ERR_CUDA;
        if (cudaMalloc(&pl->tw_f, sizeof(float)*2*n) != cudaSuccess) return MHH_ERR_CUDA;
        cudaMemcpy(pl->tw_d, td.data(), sizeof(double)*2*n, cudaMemcpyHostToDevice);
        cudaMemcpy(pl->tw_f, tf.data(), sizeof(float)*2*n, cudaMemcpyHostToDevice);
        return MHH_OK;
    }

    void fft_plan_free(FftPlan* pl)
    {
        if (pl->tw_d) cudaFree(pl->tw_d);
        if (pl->tw_f) cudaFree(pl->tw_f);
        pl->tw_d = nullptr; pl->tw_f = nullptr;
    }

    // ---------------------------------------------------------------------
    // Right-hand side, src/pres_2.cxx:155-196: divergence of ut + u/dt into
    // the packed itot*jtot*ktot array (the periodic fill of ut and vt is done
    // by the caller before).
    // ---------------------------------------------------------------------
    template<typename TF>
    __global__ void k_pres_in(Dims d, Prof<TF> pr, const TF* __restrict__ u, const TF* __restrict__ v, const TF* __restrict__ w,
                              const TF* __restrict__ ut, const TF* __restrict__ vt, const TF* __restrict__ wt,
                              TF* __restrict__ pk, TF dti)
    {
        const int i = blockIdx.x*blockDim.x + threadIdx.x;
        const int j = blockIdx.y*blockDim.y + threadIdx.y;
        const int k = blockIdx.z;
        if (i >= d.itot || j >= d.jtot) return;
        const long long c = ijk(d, i + d.igc, j + d.jgc, k + d.kgc);
        const long long ii = 1, jj = d.icells, kk = d.ijcells;
        const int kg = k + d.kgc;
        const TF rho = ld(pr.rhoref, kg);
        pk[i + (long long)j*d.itot + (long long)k*d.itot*d.jtot] =
              rho*((ld(ut, c+ii) + ld(u, c+ii)*dti) - (ld(ut, c) + ld(u, c)*dti))*TF(d.dxi)
            + rho*((ld(vt, c+jj) + ld(v, c+jj)*dti) - (ld(vt, c) + ld(v, c)*dti))*TF(d.dyi)
            + (ld(pr.rhorefh, kg+1)*(ld(wt, c+kk) + ld(w, c+kk)*dti)
             - ld(pr.rhorefh, kg  )*(ld(wt, c   ) + ld(w, c   )*dti))*ld(pr.dzi, kg);
    }

    template<typename TF>
    void launch_pres_in(const Dims& d, const Prof<TF>& pr, const TF* u, const TF* v, const TF* w,
                        const TF* ut, const TF* vt, const TF* wt, TF* pk, double dti, cudaStream_t s)
    {
        dim3 block(32, 8);
        dim3 grid((d.itot + 31)/32, (d.jtot + 7)/8, d.ktot);
        k_pres_in<TF><<<grid, block, 0, s>>>(d, pr, u, v, w, ut, vt, wt, pk, TF(dti));
        count_launch();
    }

    // ---------------------------------------------------------------------
    // Tridiagonal solve per spectral column in double, src/pres_2.cxx:200-326:
    // b = dz^2 rho (bmati + bmatj) - (a + c), b[0] += a[0]; the top row gets
    // -c for the mean mode (p = 0 at the top) and +c otherwise (dp/dz = 0);
    // right-hand side dz^2 p; Thomas algorithm.  The forward sweep keeps c/den
    // and the swept right-hand side in `work` (two doubles per cell).
    // ---------------------------------------------------------------------
    template<typename TF>
    __global__ void __launch_bounds__(128)
    k_tdma(int itot, int jtot, int ktot, const double* __restrict__ bmati, const double* __restrict__ bmatj,
           const double* __restrict__ a, const double* __restrict__ c, const double* __restrict__ dz2,
           const double* __restrict__ dz2rho, TF* __restrict__ pk, double* __restrict__ work)
    {
        const int i = blockIdx.x*blockDim.x + threadIdx.x;
        const int j = blockIdx.y;
        if (i >= itot) return;
        const long long ij = i + (long long)j*itot;
        const long long kk = (long long)itot*jtot;
        const double lam = bmati[i] + bmatj[j];
        const bool mean_mode = (i == 0 && j == 0);
        double* wc = work;
        double* wp = work + kk*ktot;

        double b = dz2rho[0]*lam - (a[0] + c[0]);
        b += a[0];
        if (ktot == 1) b += mean_mode ? -c[0] : c[0];
        double den = b;
        double pprev = (dz2[0]*double(pk[ij])) / den;
        wp[ij] = pprev;
        for (int k=1; k<ktot; ++k)
        {
            double bk = dz2rho[k]*lam - (a[k] + c[k]);
            if (k == ktot-1) bk += mean_mode ? -c[k] : c[k];
            const double w3 = c[k-1] / den;
            den = bk - a[k]*w3;
            double pkk = dz2[k]*double(pk[ij + k*kk]);
            pkk -= a[k]*pprev;
            pkk /= den;
            wc[ij + k*kk] = w3;
            wp[ij + k*kk] = pkk;
            pprev = pkk;
        }
        double x = pprev;
        pk[ij + (ktot-1)*kk] = TF(x);
        for (int k=ktot-2; k>=0; --k)
        {
            x = wp[ij + k*kk] - wc[ij + (k+1)*kk]*x;
            pk[ij + k*kk] = TF(x);
        }
    }

    template<typename TF>
    void launch_tdma(const Dims& d, const PresWork& pw, TF* pk, cudaStream_t s)
    {
        dim3 grid((d.itot + 127)/128, d.jtot);
        k_tdma<TF><<<grid, 128, 0, s>>>(d.itot, d.jtot, d.ktot, pw.bmati, pw.bmatj, pw.a, pw.c, pw.dz2, pw.dz2rho, pk, pw.work);
        count_launch();
    }

    // Packed solution back into the ghost layout with the bottom ghost level
    // p[kstart-1] = p[kstart], src/pres_2.cxx:330-358 (the periodic fill
    // follows separately).
    template<typename TF>
    __global__ void k_pres_scatter(Dims d, const TF* __restrict__ pk, TF* __restrict__ p)
    {
        const int i = blockIdx.x*blockDim.x + threadIdx.x;
        const int j = blockIdx.y*blockDim.y + threadIdx.y;
        const int k = blockIdx.z;
        if (i >= d.itot || j >= d.jtot) return;
        const TF val = pk[i + (long long)j*d.itot + (long long)k*d.itot*d.jtot];
        const long long c = ijk(d, i + d.igc, j + d.jgc, k + d.kgc);
        p[c] = val;
        if (k == 0) p[c - d.ijcells] = val;
    }

    template<typename TF>
    void launch_pres_scatter(const Dims& d, const TF* pk, TF* p, cudaStream_t s)
    {
        dim3 block(32, 8);
        dim3 grid((d.itot + 31)/32, (d.jtot + 7)/8, d.ktot);
        k_pres_scatter<TF><<<grid, block, 0, s>>>(d, pk, p);
        count_launch();
    }

#define MHH_PRES_INST(TF) \
    template void launch_pres_in<TF>(const Dims&, const Prof<TF>&, const TF*, const TF*, const TF*, const TF*, const TF*, const TF*, TF*, double, cudaStream_t); \
    template void launch_fft_x<TF>(const FftPlan&, TF*, int, bool, double, cudaStream_t); \
    template void launch_fft_y<TF>(const FftPlan&, TF*, int, int, int, bool, double, cudaStream_t); \
    template void launch_tdma<TF>(const Dims&, const PresWork&, TF*, cudaStream_t); \
    template void launch_pres_scatter<TF>(const Dims&, const TF*, TF*, cudaStream_t);

    MHH_PRES_INST(double)
    MHH_PRES_INST(float)
}
