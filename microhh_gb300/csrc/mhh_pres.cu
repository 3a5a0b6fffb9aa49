// mhh_pres.cu -- the Pres_2 Poisson solve on the GPU without cuFFT:
// divergence of the predicted velocity, hand-written real FFTs along x and y
// (halfcomplex layout, so the spectral solve is the reference's), a Thomas
// solve per spectral column (in double; in the float form in float where the
// column's forward sweep damps), inverse FFTs and the scatter back into the
// ghost-cell layout.
//
// FFT: two real sequences x, y of length n are transformed together as
// z = x + i y with a mixed-radix (4, 2, 3, 5, 7) Stockham autosort FFT in
// shared memory (ping-pong buffers, one barrier per stage), or for n = 128,
// 256 and 512 with a warp-synchronous schedule (one warp per sequence), then
// separated by Hermitian symmetry into FFTW's halfcomplex order r_0 ..
// r_{n/2}, i_{(n+1)/2-1} .. i_1 (the convention of src/fft.cxx:145-206).
#include <cmath>
#include <cstring>
#include <vector>

#include "mhh_kernels.cuh"
#include "mhh_batchable.cuh"

namespace mhh
{
    template<typename TF> struct C2;
    template<> struct C2<double> { using T = double2; };
    template<> struct C2<float> { using T = float2; };

    // a + b rounded once and never contracted with a preceding product.
    __device__ __forceinline__ double add_rn(double a, double b) { return __dadd_rn(a, b); }
    __device__ __forceinline__ float add_rn(float a, float b) { return __fadd_rn(a, b); }

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

    // Radix-R butterfly (R = 5 or 7, a compile-time constant) of one item of
    // a run-time-plan stage: the inputs x[i + q*T] times the stage twiddles
    // w^(q*k*step) (an index below n), then a direct DFT whose twiddles
    // w^(q*r*T) are w^(((q*r) mod R)*T).
    template<typename TF, int R>
    __device__ __forceinline__ void radix_gen(const typename C2<TF>::T* __restrict__ x, typename C2<TF>::T* __restrict__ y,
                                              const TF* __restrict__ tt, int i, int T, int k, int step, int j, int p)
    {
        using T2 = typename C2<TF>::T;
        T2 u[R];
        u[0] = x[i];
        #pragma unroll
        for (int q=1; q<R; ++q) u[q] = cmul(x[i + q*T], tw<TF>(tt, q*k*step));
        T2 wr[R];
        #pragma unroll
        for (int m=0; m<R; ++m) wr[m] = tw<TF>(tt, m*T);
        #pragma unroll
        for (int r=0; r<R; ++r)
        {
            T2 acc = u[0];
            #pragma unroll
            for (int q=1; q<R; ++q) acc = cadd(acc, cmul(u[q], wr[(q*r) % R]));
            y[j + r*p] = acc;
        }
    }

    // Quotient and remainder of a / b for 0 <= a < 2^20 and b >= 1 from a
    // float reciprocal rb ~ 1/b: the float quotient is within one of the
    // exact one, and one correction step in either direction makes it exact
    // (a run-time integer division costs several times more).
    __device__ __forceinline__ int div_rcp(int a, int b, float rb, int& rem)
    {
        int q = __float2int_rz(__int2float_rn(a)*rb);
        int r = a - q*b;
        if (r < 0) { --q; r += b; }
        else if (r >= b) { ++q; r -= b; }
        rem = r;
        return q;
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
            const float rT = 1.f/(float)T, rp = 1.f/(float)p;
            for (int it = threadIdx.x; it < nitem; it += blockDim.x)
            {
                int i, k;
                const int seq = div_rcp(it, T, rT, i);
                div_rcp(i, p, rp, k);
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
                    // q*k*step < R*p*step = n: no reduction modulo n.
                    T2 u0 = x[i];
                    T2 u1 = cmul(x[i +   T], tw<TF>(tt, 1*k*step));
                    T2 u2 = cmul(x[i + 2*T], tw<TF>(tt, 2*k*step));
                    T2 u3 = cmul(x[i + 3*T], tw<TF>(tt, 3*k*step));
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
                    T2 u1 = cmul(x[i +   T], tw<TF>(tt, 1*k*step));
                    T2 u2 = cmul(x[i + 2*T], tw<TF>(tt, 2*k*step));
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
                else if (R == 5) radix_gen<TF, 5>(x, y, tt, i, T, k, step, j, p);
                else radix_gen<TF, 7>(x, y, tt, i, T, k, step, j, p);
            }
            __syncthreads();
            T2* t = src; src = dst; dst = t;
            which ^= 1;
            p *= R;
        }
        return which;
    }


    // ---- fixed-length transforms -----------------------------------------
    // For the common lengths the radices are compile-time constants (8 first,
    // then 4, 2, 3, 5), so all index arithmetic folds into shifts and
    // multiplications and each stage is unrolled.
    __host__ __device__ constexpr int fixed_radix(int n, int s)
    {
        int r = n;
        for (int q=0; q<=s; ++q)
        {
            int f = 0;
            const int cand[5] = {8, 4, 2, 3, 5};
            for (int t=0; t<5 && !f; ++t) if (r % cand[t] == 0) f = cand[t];
            if (q == s) return f;
            r /= f;
        }
        return 0;
    }

    template<typename T2>
    __device__ __forceinline__ T2 mul_mi(T2 a) { T2 r; r.x = a.y; r.y = -a.x; return r; }   // -i a

    // Radix-8 DFT (forward, w = exp(-2 pi i/8)) of u[0..7] in place.
    template<typename TF, typename T2>
    __device__ __forceinline__ void dft8(T2* u)
    {
        const TF h = TF(0.70710678118654752440);
        // Stage 1: pairs (q, q+4)
        T2 a0 = cadd(u[0], u[4]), a4 = csub(u[0], u[4]);
        T2 a1 = cadd(u[1], u[5]), a5 = csub(u[1], u[5]);
        T2 a2 = cadd(u[2], u[6]), a6 = csub(u[2], u[6]);
        T2 a3 = cadd(u[3], u[7]), a7 = csub(u[3], u[7]);
        // twiddles w^q on the odd half: a5 *= w, a6 *= w^2 = -i, a7 *= w^3
        T2 t5; t5.x = h*(a5.x + a5.y); t5.y = h*(a5.y - a5.x);
        T2 t6 = mul_mi<T2>(a6);
        T2 t7; t7.x = h*(a7.y - a7.x); t7.y = -h*(a7.x + a7.y);
        // Stage 2: radix-4 on (a0,a1,a2,a3) and (a4,t5,t6,t7)
        T2 b0 = cadd(a0, a2), b2 = csub(a0, a2), b1 = cadd(a1, a3), b3 = mul_mi<T2>(csub(a1, a3));
        T2 c0 = cadd(a4, t6), c2 = csub(a4, t6), c1 = cadd(t5, t7), c3 = mul_mi<T2>(csub(t5, t7));
        u[0] = cadd(b0, b1); u[4] = csub(b0, b1);
        u[2] = cadd(b2, b3); u[6] = csub(b2, b3);
        u[1] = cadd(c0, c1); u[5] = csub(c0, c1);
        u[3] = cadd(c2, c3); u[7] = csub(c2, c3);
    }

    // Radix-R butterfly of u[0..R-1] in place (forward), for the stage with
    // sub-length T = N/R (general radices take their twiddles from tws).
    template<typename TF, int N, int R, int T>
    __device__ __forceinline__ void radix_bfly(typename C2<TF>::T* u, const typename C2<TF>::T* __restrict__ tws)
    {
        using T2 = typename C2<TF>::T;
        if (R == 8) dft8<TF, T2>(u);
        else if (R == 4)
        {
            const T2 a = cadd(u[0], u[2]), b = csub(u[0], u[2]);
            const T2 c = cadd(u[1], u[3]), e = mul_mi<T2>(csub(u[1], u[3]));
            u[0] = cadd(a, c); u[2] = csub(a, c); u[1] = cadd(b, e); u[3] = csub(b, e);
        }
        else if (R == 2)
        {
            const T2 a = u[0];
            u[0] = cadd(a, u[1]); u[1] = csub(a, u[1]);
        }
        else if (R == 3)
        {
            const TF s3 = TF(0.86602540378443864676);
            const T2 t1 = cadd(u[1], u[2]), t4 = csub(u[1], u[2]);
            T2 t2; t2.x = u[0].x - TF(0.5)*t1.x; t2.y = u[0].y - TF(0.5)*t1.y;
            u[0] = cadd(u[0], t1);
            u[1].x = t2.x + s3*t4.y; u[1].y = t2.y - s3*t4.x;
            u[2].x = t2.x - s3*t4.y; u[2].y = t2.y + s3*t4.x;
        }
        else
        {
            T2 v[R];
            #pragma unroll
            for (int r=0; r<R; ++r)
            {
                T2 acc = u[0];
                #pragma unroll
                for (int q=1; q<R; ++q) acc = cadd(acc, cmul(u[q], tws[(q*r*T) % N]));
                v[r] = acc;
            }
            #pragma unroll
            for (int r=0; r<R; ++r) u[r] = v[r];
        }
    }

    // Shared-memory position of complex element idx of a stage buffer: with
    // SWZ one element of padding per 16, so that the strided writes of the
    // first stages (element i*R + r of thread i) spread over all banks.
    template<bool SWZ> __device__ __forceinline__ int swz(int idx) { return SWZ ? idx + (idx >> 4) : idx; }

    // Stockham stages S.. of P sequences of length N, sequence q at
    // src + q*SS (SS >= N: a padded stride keeps column stores free of bank
    // conflicts).
    template<typename TF, int N, int P, int S, int PACC, int SS = N, bool SWZ = false>
    struct FixedStages
    {
        using T2 = typename C2<TF>::T;
        static __device__ __forceinline__ void run(T2*& src, T2*& dst, const T2* __restrict__ tws)
        {
            constexpr int R = fixed_radix(N, S);
            constexpr int T = N / R;
            constexpr int step = N / (PACC*R);
            constexpr int NITEM = P*T;
            for (int it = threadIdx.x; it < NITEM; it += blockDim.x)
            {
                const int seq = it / T;
                const int i = it - seq*T;
                const int k = i % PACC;
                const int xb = seq*SS + i;
                const int j = seq*SS + (i - k)*R + k;
                T2 u[R];
                u[0] = src[swz<SWZ>(xb)];
                #pragma unroll
                for (int q=1; q<R; ++q)
                    u[q] = (PACC == 1) ? src[swz<SWZ>(xb + q*T)] : cmul(src[swz<SWZ>(xb + q*T)], tws[(q*k*step) % N]);
                radix_bfly<TF, N, R, T>(u, tws);
                #pragma unroll
                for (int r=0; r<R; ++r) dst[swz<SWZ>(j + r*PACC)] = u[r];
            }
            __syncthreads();
            T2* t = src; src = dst; dst = t;
            FixedStages<TF, N, P, S+1, PACC*R, SS, SWZ>::run(src, dst, tws);
        }
    };

    template<typename TF, int N, int P, int S, int SS, bool SWZ>
    struct FixedStages<TF, N, P, S, N, SS, SWZ>
    {
        using T2 = typename C2<TF>::T;
        static __device__ __forceinline__ void run(T2*&, T2*&, const T2*) {}
    };

    // Right-hand side of the Poisson equation at interior cell (i, j, k)
    // (indices without ghosts), src/pres_2.cxx:155-196: the divergence of the
    // velocity that the tendencies would give after dt.
    template<typename TF>
    __device__ __forceinline__ TF pres_rhs_at(const Dims& d, const Prof<TF>& pr, const TF* __restrict__ u,
                                              const TF* __restrict__ v, const TF* __restrict__ w,
                                              const TF* __restrict__ ut, const TF* __restrict__ vt,
                                              const TF* __restrict__ wt, long long c, int kg, TF dti)
    {
        const long long ii = 1, jj = d.icells, kk = d.ijcells;
        const TF rho = ld(pr.rhoref, kg);
        const TF du = (ld(ut, c+ii) + mulx(ld(u, c+ii), dti)) - (ld(ut, c) + mulx(ld(u, c), dti));
        const TF dv = (ld(vt, c+jj) + mulx(ld(v, c+jj), dti)) - (ld(vt, c) + mulx(ld(v, c), dti));
        const TF dw = mulx(ld(pr.rhorefh, kg+1), ld(wt, c+kk) + mulx(ld(w, c+kk), dti))
                    - mulx(ld(pr.rhorefh, kg  ), ld(wt, c   ) + mulx(ld(w, c   ), dti));
        return mulx(mulx(rho, du), dxi_of<TF>(d)) + mulx(mulx(rho, dv), dyi_of<TF>(d)) + mulx(dw, ld(pr.dzi, kg));
    }

    template<typename TF>
    __device__ __forceinline__ TF pres_rhs(const Dims& d, const Prof<TF>& pr, const TF* __restrict__ u,
                                           const TF* __restrict__ v, const TF* __restrict__ w,
                                           const TF* __restrict__ ut, const TF* __restrict__ vt,
                                           const TF* __restrict__ wt, int i, int j, int k, TF dti)
    {
        return pres_rhs_at(d, pr, u, v, w, ut, vt, wt, ijk(d, i + d.igc, j + d.jgc, k + d.kgc), k + d.kgc, dti);
    }

    // Per-sequence offsets of a tile of nloc <= 16 real sequences starting at
    // s0, computed once per tile by its first threads (the callers
    // synchronise before use): the base of each sequence in data (sb), and
    // for the fused x transforms the ghost-layout offset of the row's first
    // interior cell (sc) and its level k (sk).  Keeps the 64-bit divisions
    // by itot or jtot out of the per-element loops.
    struct TileIdx
    {
        long long sb[16];
        long long sc[16];
        int sk[16];
    };

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

    template<typename TF>
    __device__ __forceinline__ void tile_index(TileIdx& ti, const SeqLayout& L, const FftFuse<TF>& fz, long long s0,
                                               int nloc, int n, bool fused)
    {
        const int ls = threadIdx.x;
        if (ls < nloc)
        {
            const long long s = s0 + ls;
            ti.sb[ls] = seq_base(L, s, n);
            if (fused)
            {
                const int kr = (int)(s / fz.d.jtot), jr = (int)(s - (long long)kr*fz.d.jtot);
                ti.sc[ls] = ijk(fz.d, fz.d.igc, jr + fz.d.jgc, kr + fz.d.kgc);
                ti.sk[ls] = kr;
            }
        }
    }

    template<typename TF>
    __device__ __forceinline__ void fft_cp_async(TF* dst, const TF* src, bool valid)
    {
        const unsigned s = (unsigned)__cvta_generic_to_shared(dst);
        const int nb = valid ? (int)sizeof(TF) : 0;
        if constexpr (sizeof(TF) == 4)
            asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;\n" :: "r"(s), "l"(src), "r"(nb) : "memory");
        else
            asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;\n" :: "r"(s), "l"(src), "r"(nb) : "memory");
    }

    // One block transforms 2P real sequences: load them into shared memory,
    // pack pairs as complex, FFT, separate into halfcomplex (forward) or take
    // real and imaginary parts (inverse), store.  NFIX > 0 selects the
    // fixed-length path (NFIX = n, PFIX = P); NFIX = 0 the run-time plan.
    // The float transform with the fused right-hand side keeps five blocks
    // per SM (at most 51 registers): its batched loads need the residency to
    // cover the latency of HBM.
    // ---- warp-synchronous schedule for n = 64 R (R = 2, 4, 8) --------------
    // For n = 128, 256 and 512 one warp transforms one complex sequence with
    // a single block-wide dependency (its input tile): a decimation-in-
    // frequency radix-R stage splits the sequence into R 64-point
    // sub-sequences,
    //   s_r[i] = wn^(i r) DFT_R,q(z[i + 64 q])[r],  X[R K + r] = DFT64(s_r)[K],
    // and each 64-point transform runs as 8 x 8 within the warp:
    //   A[t][k1] = w64^(t k1) DFT8_m(s_r[t + 8 m])[k1],
    //   X_r[k1 + 8 k2] = DFT8_t(A[t][k1])[k2].
    // The exchanges between the three passes go through the warp's own
    // shared-memory region with __syncwarp (an 8 x 8 transpose among eight
    // lanes is 16 shared accesses per lane; with __shfl_xor_sync it is 24
    // shuffles and 48 selects), so a tile needs block barriers only after its
    // load and before its store, against one per stage in the Stockham
    // schedule.  The last pass writes its result over the warp's own real
    // input, which no other warp reads.
    //
    // Positions within a sub-sequence block: rows of eight complex elements,
    // row index XOR (r & 1) and column index XOR row, so that eight lanes
    // reading a row or a column, and the sub-blocks a warp touches at once,
    // spread over all banks.
    __device__ __forceinline__ int warp_pos(int r, int row, int col)
    {
        return r*64 + ((row ^ (r & 1)) << 3) + (col ^ row);
    }

    // Twiddles of the schedule, n = 64 R entries in shared memory: wn^(i r)
    // at (r-1)*64 + i for r = 1..R-1, i = 0..63, then w64^(t k1) = wn^(R t k1)
    // at (R-1)*64 + k1*8 + t.
    template<typename TF, int R>
    __device__ __forceinline__ void warp_twiddles(typename C2<TF>::T* tw, const TF* __restrict__ twt)
    {
        using T2 = typename C2<TF>::T;
        constexpr int N = 64*R, B = (R - 1)*64;
        for (int e = threadIdx.x; e < N; e += blockDim.x)
        {
            const int idx = e < B ? ((e & 63)*((e >> 6) + 1)) % N : (R*(e & 7)*((e - B) >> 3)) % N;
            T2 w; w.x = twt[2*idx]; w.y = twt[2*idx + 1];
            tw[e] = w;
        }
    }

    // Complex input element k of the pair (hx, hy): z = x + i y (forward) or
    // the conjugated halfcomplex pair (inverse), as in the first Stockham
    // stage.
    template<typename TF, bool INV, int N>
    __device__ __forceinline__ typename C2<TF>::T pair_in(const TF* __restrict__ hx, const TF* __restrict__ hy, int k)
    {
        typename C2<TF>::T u;
        if (!INV)
        {
            u.x = hx[k]; u.y = hy[k];
        }
        else
        {
            const int kk = k <= N/2 ? k : N - k;
            const bool real_only = (kk == 0) || (2*kk == N);
            const TF sg = k <= N/2 ? TF(1) : TF(-1);
            const int km = real_only ? kk : N - kk;
            const TF xr = hx[kk], yr = hy[kk];
            const TF xi = real_only ? TF(0) : sg*hx[km];
            const TF yi = real_only ? TF(0) : sg*hy[km];
            u.x = xr - yi;
            u.y = -(xi + yr);
        }
        return u;
    }

    // Position of X[k] in the result of fft_warp: natural order, or with
    // SWAP the sub-sequence index r = k mod R and the next octal digit k1
    // exchanged (pass 3 then stores lane-consecutive elements; the column
    // stores read pairs of adjacent k, which this order keeps in different
    // banks).
    template<int R, bool SWAP> __device__ __forceinline__ int warp_res(int k)
    {
        if (!SWAP) return k;
        const int r = k % R, k1 = (k / R) & 7, k2 = k / (8*R);
        return r*8 + k1 + 8*R*k2;
    }

    // The transform of complex sequence q (warp q; q < P) of a tile whose
    // 2P real sequences sit at rin + s*ns.  work holds P regions of 64 R
    // complex elements at stride ss.  On return (after __syncwarp) X[k] of
    // sequence q is at element warp_res<R, SWAP>(k) of
    // reinterpret_cast<T2*>(rin + 2q*ns).
    template<typename TF, bool INV, bool SWAP, int R>
    __device__ __forceinline__ void fft_warp(TF* rin, int ns, typename C2<TF>::T* work, int ss,
                                             const typename C2<TF>::T* __restrict__ tw, int P)
    {
        using T2 = typename C2<TF>::T;
        constexpr int N = 64*R, NPAIR = 8*R;
        const int q = threadIdx.x >> 5, lane = threadIdx.x & 31;
        if (q >= P) return;
        const TF* hx = rin + (2*q)*ns;
        const TF* hy = hx + ns;
        T2* z = work + q*ss;
        // Pass 1: radix R over stride 64, twiddles wn^(i r).
        #pragma unroll
        for (int h=0; h<2; ++h)
        {
            const int i = lane + 32*h;
            T2 u[R];
            #pragma unroll
            for (int b=0; b<R; ++b) u[b] = pair_in<TF, INV, N>(hx, hy, i + 64*b);
            radix_bfly<TF, N, R, 64>(u, tw);
            #pragma unroll
            for (int r=1; r<R; ++r) u[r] = cmul(u[r], tw[(r - 1)*64 + i]);
            #pragma unroll
            for (int r=0; r<R; ++r) z[warp_pos(r, i >> 3, i & 7)] = u[r];
        }
        __syncwarp();
        // Pass 2: radix 8 over m within each sub-sequence, twiddles w64^(t k1),
        // in place (a lane's writes are the elements it read).
        #pragma unroll
        for (int h=0; h<(NPAIR + 31)/32; ++h)
        {
            const int pp = lane + 32*h, r = pp >> 3, t = pp & 7;
            if (pp < NPAIR)
            {
                T2 a[8];
                #pragma unroll
                for (int m=0; m<8; ++m) a[m] = z[warp_pos(r, m, t)];
                dft8<TF, T2>(a);
                #pragma unroll
                for (int k1=1; k1<8; ++k1) a[k1] = cmul(a[k1], tw[(R - 1)*64 + k1*8 + t]);
                #pragma unroll
                for (int k1=0; k1<8; ++k1) z[warp_pos(r, k1, t)] = a[k1];
            }
        }
        __syncwarp();
        // Pass 3: radix 8 over t; X[r + R k1 + 8 R k2] at warp_res over the
        // warp's real input (read only by this warp, in pass 1).
        T2* out = reinterpret_cast<T2*>(rin + (2*q)*ns);
        #pragma unroll
        for (int h=0; h<(NPAIR + 31)/32; ++h)
        {
            const int pp = lane + 32*h, r = pp >> 3, k1 = pp & 7;
            if (pp < NPAIR)
            {
                T2 a[8];
                #pragma unroll
                for (int t=0; t<8; ++t) a[t] = z[warp_pos(r, k1, t)];
                dft8<TF, T2>(a);
                #pragma unroll
                for (int k2=0; k2<8; ++k2) out[SWAP ? pp + 8*R*k2 : r + R*k1 + 8*R*k2] = a[k2];
            }
        }
        __syncwarp();
    }

    // Lengths that run the warp-synchronous schedule.
    __host__ __device__ constexpr bool warp_len(int n) { return n == 128 || n == 256 || n == 512; }

    template<typename TF> struct FftP { FftPlan pl; TF* data; SeqLayout L; int Prt; TF scale; FftFuse<TF> fz; };
    template<typename TF, int FUSE> struct FftOcc { static constexpr int v = (FUSE == 1 && sizeof(TF) == 4) ? 5 : 1; };

    template<typename TF, bool INV, int NFIX, int PFIX, int FUSE>
    __device__ __forceinline__ void fft_body(const FftP<TF>& A, const VBlock& vb)
    {
        const FftPlan& pl = A.pl;
        TF* __restrict__ data = A.data;
        const SeqLayout& L = A.L;
        const int Prt = A.Prt;
        const TF scale = A.scale;
        const FftFuse<TF>& fz = A.fz;
        using T2 = typename C2<TF>::T;
        extern __shared__ __align__(16) unsigned char smem_raw[];
        const int n = NFIX ? NFIX : pl.n;
        const int P = NFIX ? PFIX : Prt;
        // Each buffer holds P complex sequences plus P elements of padding:
        // viewed as 2P real sequences, the column (y) layout strides them by
        // n + 1 so that a warp reading one element of 16+ sequences hits
        // distinct banks.
        T2* buf0 = reinterpret_cast<T2*>(smem_raw);
        T2* buf1 = buf0 + (size_t)P*n + P;
        T2* tws = buf1 + (size_t)P*n + P;  // twiddle table (fixed path)
        const int ns = L.rows ? n : n + 1;  // real-sequence stride in shared memory
        const long long s0 = (long long)vb.x*2*P;
        const int nloc = (int)min((long long)2*P, L.nseq - s0);

        constexpr bool WARP = warp_len(NFIX);
        if constexpr (WARP) warp_twiddles<TF, NFIX/64>(tws, twtab<TF>(pl));
        else if (NFIX)
        {
            const TF* tt = twtab<TF>(pl);
            for (int e = threadIdx.x; e < n; e += blockDim.x)
            { T2 w; w.x = tt[2*e]; w.y = tt[2*e+1]; tws[e] = w; }
        }

        // 1. Load 2P real sequences into buf1 viewed as real [2P][n], with
        //    asynchronous copies so that all of a thread's loads are in
        //    flight together (a missing sequence reads as zero).
        __shared__ TileIdx ti;
        tile_index<TF>(ti, L, fz, s0, nloc, n, FUSE != 0);
        __syncthreads();
        TF* r1 = reinterpret_cast<TF*>(buf1);
        const int tot = 2*P*n;
        if (FUSE == 1)
        {
            // Rows of the pressure right-hand side computed in place of
            // loading them.  Unrolled so that the loads of several elements
            // are in flight together.
            // RB elements per thread at a time with all their loads issued
            // before the arithmetic (twelve loads each), so that the
            // latency of HBM is covered by the loads of several elements.
            const int kgc = fz.d.kgc;
            constexpr int RB = 4;
            const long long ii = 1, jj = fz.d.icells, kk = fz.d.ijcells;
            for (int e0 = threadIdx.x; e0 < tot; e0 += RB*blockDim.x)
            {
                TF vals[RB][12];
                int kgs[RB];
                #pragma unroll
                for (int b=0; b<RB; ++b)
                {
                    const int e = e0 + b*blockDim.x;
                    const int ls = e / n, i = e - ls*n;
                    const bool ok = e < tot && ls < nloc;
                    // A masked element reads the first interior cell (a valid
                    // address) and is stored as zero below.
                    const long long c = ok ? ti.sc[ls] + i : ti.sc[0];
                    kgs[b] = (ok ? ti.sk[ls] : ti.sk[0]) + kgc;
                    vals[b][0] = ld(fz.ut, c+ii); vals[b][1] = ld(fz.u, c+ii);
                    vals[b][2] = ld(fz.ut, c);    vals[b][3] = ld(fz.u, c);
                    vals[b][4] = ld(fz.vt, c+jj); vals[b][5] = ld(fz.v, c+jj);
                    vals[b][6] = ld(fz.vt, c);    vals[b][7] = ld(fz.v, c);
                    vals[b][8] = ld(fz.wt, c+kk); vals[b][9] = ld(fz.w, c+kk);
                    vals[b][10] = ld(fz.wt, c);   vals[b][11] = ld(fz.w, c);
                }
                #pragma unroll
                for (int b=0; b<RB; ++b)
                {
                    const int e = e0 + b*blockDim.x;
                    if (e < tot)
                    {
                        const int ls = e / n, i = e - ls*n;
                        const TF* x = vals[b];
                        const int kg = kgs[b];
                        const TF rho = ld(fz.pr.rhoref, kg);
                        const TF dti = fz.dti;
                        // The operation order of src/pres_2.cxx:184-191
                        // (products not contracted in double).
                        const TF du = (x[0] + mulx(x[1], dti)) - (x[2] + mulx(x[3], dti));
                        const TF dv = (x[4] + mulx(x[5], dti)) - (x[6] + mulx(x[7], dti));
                        const TF dw = mulx(ld(fz.pr.rhorefh, kg+1), x[8] + mulx(x[9], dti))
                                    - mulx(ld(fz.pr.rhorefh, kg  ), x[10] + mulx(x[11], dti));
                        const TF val = mulx(mulx(rho, du), dxi_of<TF>(fz.d)) + mulx(mulx(rho, dv), dyi_of<TF>(fz.d))
                                     + mulx(dw, ld(fz.pr.dzi, kg));
                        r1[ls*ns + i] = ls < nloc ? val : TF(0);
                    }
                }
            }
        }
        else if (L.rows)
        {
            for (int e = threadIdx.x; e < tot; e += blockDim.x)
            {
                const int ls = e / n, j = e - ls*n;
                const bool ok = ls < nloc;
                fft_cp_async(r1 + ls*ns + j, ok ? data + ti.sb[ls] + j : data, ok);
            }
        }
        else if (NFIX && (256 % (2*(PFIX ? PFIX : 1))) == 0)
        {
            // Columns: with 2P dividing the block size every thread keeps
            // one sequence (ls) and walks its elements.
            const int ls = threadIdx.x % (2*P);
            const bool ok = ls < nloc;
            const TF* src = data + (ok ? ti.sb[ls] : 0);
            const long long st = (long long)(blockDim.x/(2*P))*L.itot;
            const TF* sp = src + (long long)(threadIdx.x/(2*P))*L.itot;
            for (int j = threadIdx.x/(2*P); j < n; j += blockDim.x/(2*P), sp += st)
                fft_cp_async(r1 + ls*ns + j, ok ? sp : data, ok);
        }
        else
        {
            for (int e = threadIdx.x; e < tot; e += blockDim.x)
            {
                const int j = e / (2*P), ls = e - j*(2*P);
                const bool ok = ls < nloc;
                fft_cp_async(r1 + ls*ns + j, ok ? data + ti.sb[ls] + (long long)j*L.itot : data, ok);
            }
        }
        asm volatile("cp.async.commit_group;\n" ::: "memory");
        asm volatile("cp.async.wait_group 0;\n" ::: "memory");
        __syncthreads();

        // 2-3. With n = 128, 256 or 512 the warp-synchronous schedule, whose
        //      result is the natural order over each sequence pair's real
        //      input.
        T2* res;
        T2* other;
        if constexpr (WARP)
        {
            fft_warp<TF, INV, false, NFIX/64>(r1, ns, buf0, n, tws, P);
            __syncthreads();
            res = nullptr; other = buf0;
        }
        else
        {
        // 2. Complex input: z = x + i y (forward) or conj(X + i Y) (inverse).
        for (int e = threadIdx.x; e < P*n; e += blockDim.x)
        {
            const int q = e / n, k = e - q*n;
            const TF* hx = r1 + (2*q)*ns;
            const TF* hy = r1 + (2*q+1)*ns;
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
                z.x = xr - yi;
                z.y = -(xi + yr);
            }
            buf0[e] = z;
        }
        __syncthreads();

        // 3. FFT.
        if (NFIX)
        {
            T2* src = buf0;
            T2* dst = buf1;
            FixedStages<TF, (NFIX ? NFIX : 1), (PFIX ? PFIX : 1), 0, 1>::run(src, dst, tws);
            res = src; other = dst;
        }
        else
        {
            const int which = stockham<TF>(pl, buf0, buf1, P);
            res = which ? buf1 : buf0;
            other = which ? buf0 : buf1;
        }
        }
        TF* rout = reinterpret_cast<TF*>(other);

        // 4. Real outputs into the other buffer, [2P][n].
        for (int e = threadIdx.x; e < P*n; e += blockDim.x)
        {
            const int q = e / n, k = e - q*n;
            TF* ox = rout + (2*q)*ns;
            TF* oy = rout + (2*q+1)*ns;
            const T2* rq = WARP ? reinterpret_cast<const T2*>(r1 + (2*q)*ns) : res + q*n;
            if (!INV)
            {
                if (k <= n/2)
                {
                    const T2 a = rq[k], b = rq[(n - k) % n];
                    const TF xr = TF(0.5)*(a.x + b.x), xi = TF(0.5)*(a.y - b.y);
                    const TF yr = TF(0.5)*(a.y + b.y), yi = TF(-0.5)*(a.x - b.x);
                    ox[k] = xr; oy[k] = yr;
                    if (k > 0 && k < n - k) { ox[n - k] = xi; oy[n - k] = yi; }
                }
            }
            else
            {
                const T2 a = rq[k];
                ox[k] = a.x*scale;
                oy[k] = -a.y*scale;
            }
        }
        __syncthreads();

        // 5. Store (with FUSE == 2 straight into the ghost layout of p, with
        //    the bottom ghost level p[kstart-1] = p[kstart], src/pres_2.cxx:330-358).
        if (FUSE == 2)
        {
            for (int e = threadIdx.x; e < tot; e += blockDim.x)
            {
                const int ls = e / n, i = e - ls*n;
                if (ls < nloc)
                {
                    const TF val = fz.dcm ? add_rn(rout[ls*ns + i], fz.dcm[ti.sk[ls]]) : rout[ls*ns + i];
                    const long long c = ti.sc[ls] + i;
                    fz.p[c] = val;
                    if (ti.sk[ls] == 0) fz.p[c - fz.d.ijcells] = val;
                }
            }
        }
        else if (L.rows)
        {
            for (int e = threadIdx.x; e < tot; e += blockDim.x)
            {
                const int ls = e / n, j = e - ls*n;
                if (ls < nloc) data[ti.sb[ls] + j] = rout[ls*ns + j];
            }
        }
        else if (NFIX && (256 % (2*(PFIX ? PFIX : 1))) == 0)
        {
            const int ls = threadIdx.x % (2*P);
            if (ls < nloc)
            {
                const long long st = (long long)(blockDim.x/(2*P))*L.itot;
                TF* dp = data + ti.sb[ls] + (long long)(threadIdx.x/(2*P))*L.itot;
                for (int j = threadIdx.x/(2*P); j < n; j += blockDim.x/(2*P), dp += st)
                    *dp = rout[ls*ns + j];
            }
        }
        else
        {
            for (int e = threadIdx.x; e < tot; e += blockDim.x)
            {
                const int j = e / (2*P), ls = e - j*(2*P);
                if (ls < nloc) data[ti.sb[ls] + (long long)j*L.itot] = rout[ls*ns + j];
            }
        }
    }

    // ---- pipelined fixed-length transforms ----------------------------------
    // A persistent block loops over tiles of 2P real sequences.  While it
    // transforms tile t, the asynchronous copies of its next tile are already
    // in flight into a second input buffer, so the loads of HBM overlap the
    // shared-memory work of the stages (one tile per block left the memory
    // system idle between a block's load and its store).  The packing of two
    // real sequences into one complex one is folded into the first stage and
    // the separation into halfcomplex order into the store.
    //
    // Shared memory: two input buffers and one work buffer of P*SS + P
    // complex elements, plus the twiddle table.  Tile t's input buffer also
    // serves as the second stage buffer; the other input buffer receives
    // tile t + (the number of blocks).

    // Complex elements of one buffer of the pipelined kernel: P sequences at
    // stride SS (N for rows, N + 4 for columns) with the swizzle padding, and
    // at least the real input view of 2P sequences at stride NS.
    __host__ __device__ constexpr int fftp_buf(int N, int P, bool rows)
    {
        return (P*(rows ? N : N + 4)*17)/16 + 16 + P;
    }

    // First Stockham stage (radix R0, no twiddles) with the complex input
    // formed from the real sequences: z = x + i y (forward) or the
    // conjugated halfcomplex pair (inverse).  Real sequence s sits at
    // r + s*NS.
    template<typename TF, bool INV, int N, int P, int NS, int SS, bool SWZ>
    __device__ __forceinline__ void fft_first_stage(const TF* __restrict__ r, typename C2<TF>::T* __restrict__ y,
                                                    const typename C2<TF>::T* __restrict__ tws)
    {
        using T2 = typename C2<TF>::T;
        constexpr int R = fixed_radix(N, 0);
        constexpr int T = N / R;
        for (int it = threadIdx.x; it < P*T; it += blockDim.x)
        {
            const int seq = it / T, i = it - seq*T;
            const TF* hx = r + (2*seq)*NS;
            const TF* hy = hx + NS;
            T2 u[R];
            #pragma unroll
            for (int q=0; q<R; ++q)
            {
                const int k = i + q*T;
                if (!INV)
                {
                    u[q].x = hx[k]; u[q].y = hy[k];
                }
                else
                {
                    const int kk = k <= N/2 ? k : N - k;
                    const bool real_only = (kk == 0) || (2*kk == N);
                    const TF sg = k <= N/2 ? TF(1) : TF(-1);
                    const int km = real_only ? kk : N - kk;
                    const TF xr = hx[kk], yr = hy[kk];
                    const TF xi = real_only ? TF(0) : sg*hx[km];
                    const TF yi = real_only ? TF(0) : sg*hy[km];
                    u[q].x = xr - yi;
                    u[q].y = -(xi + yr);
                }
            }
            radix_bfly<TF, N, R, T>(u, tws);
            const int yb = seq*SS + i*R;
            #pragma unroll
            for (int q=0; q<R; ++q) y[swz<SWZ>(yb + q)] = u[q];
        }
        __syncthreads();
    }

    // Real output k of real sequence ls of a tile from the transformed pairs:
    // halfcomplex separation (forward) or real/imaginary parts (inverse).
    template<typename TF, bool INV, int N, int SS, bool SWZ>
    __device__ __forceinline__ TF fft_real_out(const typename C2<TF>::T* __restrict__ res, int ls, int k, TF scale)
    {
        using T2 = typename C2<TF>::T;
        const int qb = (ls >> 1)*SS;
        const bool yseq = ls & 1;
        if (INV)
        {
            const T2 a = res[swz<SWZ>(qb + k)];
            return yseq ? -a.y*scale : a.x*scale;
        }
        const int kk = k <= N/2 ? k : N - k;
        const T2 a = res[swz<SWZ>(qb + kk)], b = res[swz<SWZ>(qb + (kk == 0 ? 0 : N - kk))];
        if (k <= N/2) return yseq ? TF(0.5)*(a.y + b.y) : TF(0.5)*(a.x + b.x);
        return yseq ? TF(-0.5)*(a.x - b.x) : TF(0.5)*(a.y - b.y);
    }

    // The same from the result rq of the pair from fft_warp (yseq: the
    // pair's second real sequence).
    template<typename TF, bool INV, int N, bool SWAP>
    __device__ __forceinline__ TF fft_real_nat(const typename C2<TF>::T* __restrict__ rq, int yseq, int k, TF scale)
    {
        using T2 = typename C2<TF>::T;
        if (INV)
        {
            const T2 a = rq[warp_res<N/64, SWAP>(k)];
            return yseq ? -a.y*scale : a.x*scale;
        }
        const int kk = k <= N/2 ? k : N - k;
        const T2 a = rq[warp_res<N/64, SWAP>(kk)], b = rq[warp_res<N/64, SWAP>(kk == 0 ? 0 : N - kk)];
        if (k <= N/2) return yseq ? TF(0.5)*(a.y + b.y) : TF(0.5)*(a.x + b.x);
        return yseq ? TF(-0.5)*(a.x - b.x) : TF(0.5)*(a.y - b.y);
    }

    template<typename TF> struct FftpP { TF* data; SeqLayout L; TF scale; FftFuse<TF> fz; const TF* twt; long long ntiles; };

    template<typename TF, bool INV, int N, int P, int FUSE, bool ROWS>
    __device__ __forceinline__ void fftp_body(const FftpP<TF>& A, const VBlock& vb)
    {
        TF* __restrict__ data = A.data;
        const SeqLayout& L = A.L;
        const TF scale = A.scale;
        const FftFuse<TF>& fz = A.fz;
        const TF* __restrict__ twt = A.twt;
        const long long ntiles = A.ntiles;
        using T2 = typename C2<TF>::T;
        constexpr int NS = ROWS ? N : N + 1;      // real stride of the input view
        constexpr int SS = ROWS ? N : N + 4;      // complex stride of the stages
        constexpr int BUF = fftp_buf(N, P, ROWS);
        extern __shared__ __align__(16) unsigned char smem_raw[];
        T2* bufs = reinterpret_cast<T2*>(smem_raw);
        T2* work = bufs + BUF;
        T2* tws = bufs + 3*BUF;
        constexpr bool WARP = warp_len(N);
        if constexpr (WARP) warp_twiddles<TF, N/64>(tws, twt);
        else
            for (int e = threadIdx.x; e < N; e += blockDim.x)
            { T2 w; w.x = twt[2*e]; w.y = twt[2*e+1]; tws[e] = w; }

        // Asynchronous copies of tile t into input buffer b (a missing
        // sequence reads as zero).  Each thread computes the base of the
        // sequence it copies once per tile.
        auto issue = [&](long long t, T2* b)
        {
            TF* r = reinterpret_cast<TF*>(b);
            const long long s0 = t*2*P;
            const int nloc = (int)min((long long)2*P, L.nseq - s0);
            if (ROWS)
            {
                for (int e = threadIdx.x; e < 2*P*N; e += blockDim.x)
                {
                    const int ls = e / N, j = e - ls*N;
                    const bool ok = ls < nloc;
                    fft_cp_async(r + ls*NS + j, ok ? data + (s0 + ls)*(long long)N + j : data, ok);
                }
            }
            else
            {
                const int ls = threadIdx.x % (2*P);
                const bool ok = ls < nloc;
                const long long st = (long long)(blockDim.x/(2*P))*L.itot;
                const TF* sp = data + (ok ? seq_base(L, s0 + ls, N) : 0) + (long long)(threadIdx.x/(2*P))*L.itot;
                for (int j = threadIdx.x/(2*P); j < N; j += blockDim.x/(2*P), sp += st)
                    fft_cp_async(r + ls*NS + j, ok ? sp : data, ok);
            }
            asm volatile("cp.async.commit_group;\n" ::: "memory");
        };
        // Ghost-layout offsets of the current tile's rows (FUSE == 2),
        // written after the barrier that ends the previous tile and read
        // after the barriers of the stages.
        __shared__ TileIdx x;

        long long t = vb.x;
        int cur = 0;
        if (t < ntiles) issue(t, bufs);
        for (; t < ntiles; t += vb.gx)
        {
            T2* in = cur ? bufs + 2*BUF : bufs;
            asm volatile("cp.async.wait_group 0;\n" ::: "memory");
            __syncthreads();
            // The other input buffer was last read by the previous tile,
            // which every thread has finished (barrier above).
            if (t + vb.gx < ntiles) issue(t + vb.gx, cur ? bufs : bufs + 2*BUF);
            if (FUSE == 2)
            {
                const long long s0 = t*2*P;
                tile_index<TF>(x, L, fz, s0, (int)min((long long)2*P, L.nseq - s0), N, true);
            }

            const T2* res = work;
            TF* inr = reinterpret_cast<TF*>(in);
            if constexpr (WARP)
            {
                fft_warp<TF, INV, !ROWS, N/64>(inr, NS, work, SS, tws, P);
                __syncthreads();
            }
            else
            {
                // The swizzle pays off for rows; the padded column stride
                // already spreads the column stores.
                fft_first_stage<TF, INV, N, P, NS, SS, ROWS>(inr, work, tws);
                T2* src = work;
                T2* dst = in;
                FixedStages<TF, N, P, 1, fixed_radix(N, 0), SS, ROWS>::run(src, dst, tws);
                res = src;
            }
            // Real output k of real sequence ls of the tile.
            auto out_at = [&](int ls, int k) -> TF
            {
                if constexpr (WARP)
                    return fft_real_nat<TF, INV, N, !ROWS>(reinterpret_cast<const T2*>(inr + (ls & ~1)*NS), ls & 1, k, scale);
                else
                    return fft_real_out<TF, INV, N, SS, ROWS>(res, ls, k, scale);
            };

            const long long s0 = t*2*P;
            const int nloc = (int)min((long long)2*P, L.nseq - s0);
            if (FUSE == 2)
            {
                // Straight into the ghost layout of p, with the bottom ghost
                // level p[kstart-1] = p[kstart] (src/pres_2.cxx:330-358).
                for (int e = threadIdx.x; e < 2*P*N; e += blockDim.x)
                {
                    const int ls = e / N, i = e - ls*N;
                    if (ls < nloc)
                    {
                        TF val = out_at(ls, i);
                        if (fz.dcm) val = add_rn(val, fz.dcm[x.sk[ls]]);
                        const long long c = x.sc[ls] + i;
                        fz.p[c] = val;
                        if (x.sk[ls] == 0) fz.p[c - fz.d.ijcells] = val;
                    }
                }
            }
            else if (ROWS)
            {
                for (int e = threadIdx.x; e < 2*P*N; e += blockDim.x)
                {
                    const int ls = e / N, j = e - ls*N;
                    if (ls < nloc) data[(s0 + ls)*(long long)N + j] = out_at(ls, j);
                }
            }
            else
            {
                const int ls = threadIdx.x % (2*P);
                if (ls < nloc)
                {
                    const long long st = (long long)(blockDim.x/(2*P))*L.itot;
                    TF* dp = data + seq_base(L, s0 + ls, N) + (long long)(threadIdx.x/(2*P))*L.itot;
                    for (int j = threadIdx.x/(2*P); j < N; j += blockDim.x/(2*P), dp += st)
                        *dp = out_at(ls, j);
                }
            }
            cur ^= 1;
        }
        asm volatile("cp.async.wait_group 0;\n" ::: "memory");
    }

    template<typename TF, bool INV, int N, int P, int FUSE, bool ROWS>
    static void launch_fftp(const FftPlan& pl, TF* data, SeqLayout L, TF scale, const FftFuse<TF>& fz, cudaStream_t s)
    {
        using T2 = typename C2<TF>::T;
        // 8 pairs (16 columns, 64-byte rows of a tile) run with 512 threads;
        // the warp-synchronous schedule with one warp per pair.
        constexpr int NT = warp_len(N) ? 32*P : (P == 8 ? 512 : 256);
        const size_t smem = sizeof(T2)*((size_t)3*fftp_buf(N, P, ROWS) + N);
        const long long ntiles = (L.nseq + 2*P - 1) / (2*P);
        // Attribute and residency are set once per kernel, outside any stream
        // capture that a later call may be part of.
        using B = FftpP<TF>;
        constexpr auto body = fftp_body<TF, INV, N, P, FUSE, ROWS>;
        static const int resident = [&]
        {
            set_smem_limit<B, body, NT, 1>(smem);
            int per_sm = 0, dev = 0, sms = 0;
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_one<B, body, NT, 1>, NT, smem);
            cudaGetDevice(&dev);
            cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
            return (per_sm > 0 ? per_sm : 1)*(sms > 0 ? sms : 1);
        }();
        const long long nblk = ntiles < resident ? ntiles : resident;
        const TF* twt = sizeof(TF) == 8 ? reinterpret_cast<const TF*>(pl.tw_d) : reinterpret_cast<const TF*>(pl.tw_f);
        launch_body<B, body, NT, 1>(dim3((unsigned)nblk), dim3(NT), smem, s, B{data, L, scale, fz, twt, ntiles});
    }

    // Dynamic shared-memory limit of the run-time-plan FFT (two buffers of at
    // most 96 KB of sequences, plus padding).
    constexpr int FFT_GENERIC_SMEM = 100*1024;

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

    template<typename TF, bool INV, int NF, int PF, int FUSE>
    static void launch_fixed(const FftPlan& pl, TF* data, SeqLayout L, TF scale, const FftFuse<TF>& fz, cudaStream_t s)
    {
        const size_t smem = sizeof(typename C2<TF>::T)*((size_t)2*(PF*NF + PF) + NF);
        const long long nblk = (L.nseq + 2*PF - 1) / (2*PF);
        launch_body<FftP<TF>, fft_body<TF, INV, NF, PF, FUSE>, 256, FftOcc<TF, FUSE>::v>(
            dim3((unsigned)nblk), dim3(256), smem, s, FftP<TF>{pl, data, L, PF, scale, fz});
    }

    template<typename TF, bool INV, int NF>
    static bool try_fixed_n(const FftPlan& pl, TF* data, SeqLayout L, TF scale, const FftFuse<TF>& fz, cudaStream_t s)
    {
        if (pl.n != NF) return false;
        // Rows: 4 pairs per block; columns: 4 or 8 (float) pairs per block.
        constexpr int PR = (2*sizeof(typename C2<TF>::T)*4*NF <= 96*1024) ? 4 : 1;
        constexpr int PC = (sizeof(TF) == 4 && 2*sizeof(typename C2<TF>::T)*8*NF <= 96*1024) ? 8 : PR;
        // Pipelined transforms (three buffers) where they fit in 96 KB.
        constexpr bool PIPE_R = sizeof(typename C2<TF>::T)*(3*fftp_buf(NF, PR, true) + NF) <= 96*1024;
        constexpr bool PIPE_C = sizeof(typename C2<TF>::T)*(3*fftp_buf(NF, PR, false) + NF) <= 96*1024;
        constexpr bool PIPE_C8 = sizeof(TF) == 4 && sizeof(typename C2<TF>::T)*(3*fftp_buf(NF, 8, false) + NF) <= 200*1024;
        const bool pipe = fft_pipeline() != 0;
        if (L.rows)
        {
            if constexpr (!INV) { if (fz.mode == 1) { launch_fixed<TF, INV, NF, PR, 1>(pl, data, L, scale, fz, s); return true; } }
            else
            {
                if (fz.mode == 2)
                {
                    if (PIPE_R && pipe) launch_fftp<TF, INV, NF, PR, 2, true>(pl, data, L, scale, fz, s);
                    else launch_fixed<TF, INV, NF, PR, 2>(pl, data, L, scale, fz, s);
                    return true;
                }
            }
            if (PIPE_R && pipe) launch_fftp<TF, INV, NF, PR, 0, true>(pl, data, L, scale, fz, s);
            else launch_fixed<TF, INV, NF, PR, 0>(pl, data, L, scale, fz, s);
        }
        else if (PIPE_C8 && pipe && fft_column_pairs() == 8) launch_fftp<TF, INV, NF, 8, 0, false>(pl, data, L, scale, fz, s);
        else if (PIPE_C && pipe) launch_fftp<TF, INV, NF, PR, 0, false>(pl, data, L, scale, fz, s);
        else if (fft_column_pairs() == 4 || PC == PR) launch_fixed<TF, INV, NF, PR, 0>(pl, data, L, scale, fz, s);
        else launch_fixed<TF, INV, NF, PC, 0>(pl, data, L, scale, fz, s);
        return true;
    }

    template<typename TF, bool INV>
    static bool launch_fixed_any(const FftPlan& pl, TF* data, SeqLayout L, TF scale, const FftFuse<TF>& fz, cudaStream_t s)
    {
        return try_fixed_n<TF, INV, 512>(pl, data, L, scale, fz, s) || try_fixed_n<TF, INV, 256>(pl, data, L, scale, fz, s)
            || try_fixed_n<TF, INV, 128>(pl, data, L, scale, fz, s) || try_fixed_n<TF, INV, 64>(pl, data, L, scale, fz, s)
            || try_fixed_n<TF, INV, 32>(pl, data, L, scale, fz, s) || try_fixed_n<TF, INV, 1024>(pl, data, L, scale, fz, s)
            || try_fixed_n<TF, INV, 192>(pl, data, L, scale, fz, s) || try_fixed_n<TF, INV, 96>(pl, data, L, scale, fz, s)
            || try_fixed_n<TF, INV, 48>(pl, data, L, scale, fz, s) || try_fixed_n<TF, INV, 384>(pl, data, L, scale, fz, s)
            || try_fixed_n<TF, INV, 768>(pl, data, L, scale, fz, s) || try_fixed_n<TF, INV, 16>(pl, data, L, scale, fz, s);
    }

    template<typename TF, bool INV, int FUSE>
    static void launch_generic(const FftPlan& pl, TF* data, SeqLayout L, TF scale, const FftFuse<TF>& fz, cudaStream_t s)
    {
        const int n = pl.n;
        const int P = pairs_per_block<TF>(n, L.rows != 0);
        const size_t smem = 2*sizeof(typename C2<TF>::T)*((size_t)P*n + P);
        const long long nblk = (L.nseq + 2*P - 1) / (2*P);
        // The shared memory depends on n: the limit is set to the largest.
        set_smem_limit<FftP<TF>, fft_body<TF, INV, 0, 0, FUSE>, 256, FftOcc<TF, FUSE>::v>(FFT_GENERIC_SMEM);
        launch_body<FftP<TF>, fft_body<TF, INV, 0, 0, FUSE>, 256, FftOcc<TF, FUSE>::v>(
            dim3((unsigned)nblk), dim3(256), smem, s, FftP<TF>{pl, data, L, P, scale, fz});
    }

    template<typename TF>
    static void launch_fft(const FftPlan& pl, TF* data, SeqLayout L, bool inverse, TF scale, const FftFuse<TF>& fz,
                           cudaStream_t s)
    {
        const int n = pl.n;
        if (n == 1) return;
        count_launch();
        if (inverse ? launch_fixed_any<TF, true>(pl, data, L, scale, fz, s) : launch_fixed_any<TF, false>(pl, data, L, scale, fz, s))
            return;
        if (inverse)
        {
            if (L.rows && fz.mode == 2) launch_generic<TF, true, 2>(pl, data, L, scale, fz, s);
            else launch_generic<TF, true, 0>(pl, data, L, scale, fz, s);
        }
        else
        {
            if (L.rows && fz.mode == 1) launch_generic<TF, false, 1>(pl, data, L, scale, fz, s);
            else launch_generic<TF, false, 0>(pl, data, L, scale, fz, s);
        }
    }

    template<typename TF>
    void launch_fft_x(const FftPlan& pl, TF* data, int nrows, bool inverse, double scale, cudaStream_t s,
                      const FftFuse<TF>* fuse)
    {
        SeqLayout L; L.rows = 1; L.itot = 0; L.nseq = nrows;
        FftFuse<TF> fz;
        std::memset(&fz, 0, sizeof(fz));
        if (fuse) fz = *fuse;
        launch_fft<TF>(pl, data, L, inverse, TF(scale), fz, s);
    }

    template<typename TF>
    void launch_fft_y(const FftPlan& pl, TF* data, int itot, int jtot, int ktot, bool inverse, double scale, cudaStream_t s)
    {
        SeqLayout L; L.rows = 0; L.itot = itot; L.nseq = (long long)itot*ktot;
        FftFuse<TF> fz;
        std::memset(&fz, 0, sizeof(fz));
        launch_fft<TF>(pl, data, L, inverse, TF(scale), fz, s);
        (void)jtot;
    }

    int fft_plan_init(FftPlan* pl, int n, cudaStream_t s)
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
        if (cudaMallocAsync((void**)&pl->tw_d, sizeof(double)*2*n, s) != cudaSuccess) return MHH_ERR_CUDA;
        if (cudaMallocAsync((void**)&pl->tw_f, sizeof(float)*2*n, s) != cudaSuccess) return MHH_ERR_CUDA;
        cudaMemcpyAsync(pl->tw_d, td.data(), sizeof(double)*2*n, cudaMemcpyHostToDevice, s);
        cudaMemcpyAsync(pl->tw_f, tf.data(), sizeof(float)*2*n, cudaMemcpyHostToDevice, s);
        return cudaStreamSynchronize(s) == cudaSuccess ? MHH_OK : MHH_ERR_CUDA;
    }

    void fft_plan_free(FftPlan* pl, cudaStream_t s)
    {
        if (pl->tw_d) cudaFreeAsync(pl->tw_d, s);
        if (pl->tw_f) cudaFreeAsync(pl->tw_f, s);
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
        pk[i + (long long)j*d.itot + (long long)k*d.itot*d.jtot] = pres_rhs(d, pr, u, v, w, ut, vt, wt, i, j, k, dti);
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
    // right-hand side dz^2 p; Thomas algorithm.
    //
    // The elimination coefficients depend on the column only through
    // lambda = bmati[i] + bmatj[j], and bmati, bmatj are mirror-symmetric
    // (i and itot - i share a wave number), so the columns form groups of up
    // to four with identical coefficients.  den_k and c_k/den_k of every group
    // are computed once at set-up (k_tdma_table), rounded as the reference
    // rounds them.  The reference-order solve (k_tdma) then repeats the
    // reference's per-cell operations (a product, a difference and a division
    // forward, a product and a difference back) with one thread for the four
    // columns of a group: the mean mode's solve is ill-conditioned, so its
    // result follows every rounding of the sweep.  The rescaled solve
    // (k_tdma_col) needs two FMAs per cell, with one thread per column
    // (k_tdma_scaled: the same with four columns per thread).
    // ---------------------------------------------------------------------
    constexpr double TDMA_FLOAT_GAMMA = 0.999;

    __global__ void k_tdma_table(int niu, int nju, int ktot, const double* __restrict__ bmati,
                                 const double* __restrict__ bmatj, const double* __restrict__ a,
                                 const double* __restrict__ c, const double* __restrict__ dz2rho,
                                 const double* __restrict__ dz2, double* __restrict__ rtab,
                                 double* __restrict__ wtab, double* __restrict__ gtab, double* __restrict__ htab,
                                 float* __restrict__ stab, double* __restrict__ stabd,
                                 float* __restrict__ gftab, float* __restrict__ hftab,
                                 unsigned char* __restrict__ fmode)
    {
        const int iu = blockIdx.x*blockDim.x + threadIdx.x;
        const int ju = blockIdx.y;
        if (iu >= niu) return;
        const long long stride = (long long)niu*nju;
        const long long base = iu + (long long)ju*niu;
        const double lam = bmati[iu] + bmatj[ju];
        const bool mean_mode = (iu == 0 && ju == 0);
        // src/pres_2.cxx:266-326 and :200-263, products not contracted.
        double b = mulx(dz2rho[0], lam) - (a[0] + c[0]);
        b += a[0];
        if (ktot == 1) b += mean_mode ? -c[0] : c[0];
        double den = b;
        rtab[base] = den;
        for (int k=1; k<ktot; ++k)
        {
            double bk = mulx(dz2rho[k], lam) - (a[k] + c[k]);
            if (k == ktot-1) bk += mean_mode ? -c[k] : c[k];
            const double w3 = c[k-1]/den;
            wtab[base + (k-1)*stride] = w3;
            den = bk - mulx(a[k], w3);
            rtab[base + k*stride] = den;
        }
        wtab[base + (ktot-1)*stride] = 0.;
        // Rescaled recurrence: with s_k = dz2_k/den_k, y_k = s_k z_k and
        // x_k = s_k xi_k the sweeps become
        //   z_k = p_k - g_k z_{k-1},      g_k = a_k s_{k-1}/dz2_k,
        //   xi_k = z_k - h_k xi_{k+1},    h_k = c_k s_{k+1}/dz2_k,
        // and x_k = s_k xi_k: one FMA per cell and sweep.
        for (int k=0; k<ktot; ++k)
        {
            const double sk = dz2[k]/rtab[base + k*stride];
            stabd[base + k*stride] = sk;
            stab[base + k*stride] = float(sk);
            gtab[base + k*stride] = k ? a[k]*(dz2[k-1]/rtab[base + (k-1)*stride])/dz2[k] : 0.;
            htab[base + k*stride] = k < ktot-1 ? c[k]*(dz2[k+1]/rtab[base + (k+1)*stride])/dz2[k] : 0.;
        }
        // Float sweeps where the forward sweep damps: a rounding error of z_k
        // enters the next level multiplied by g_{k+1}, and as |g| -> 1 (small
        // |lambda| dz^2: the largest horizontal scales) the forward values
        // become running sums whose round-off grows with the level.  With
        // max |g| <= TDMA_FLOAT_GAMMA the float solve of a column stays
        // within about ten float roundings of its largest value (measured on
        // 256 uniform levels with random right-hand sides: 9 ulp at |g| =
        // 0.999, 4 ulp at 0.9).  The large backward factor h at the top
        // level (the Neumann row) multiplies a value that s scales down, and
        // adds no more.  The groups above the bound and the mean mode keep
        // FP64.
        double gam = 0.;
        for (int k=0; k<ktot; ++k)
        {
            const double g = gtab[base + k*stride], h = htab[base + k*stride];
            gftab[base + k*stride] = float(g);
            hftab[base + k*stride] = float(h);
            gam = fmax(gam, fabs(g));
        }
        fmode[base] = (!mean_mode && gam <= TDMA_FLOAT_GAMMA) ? 1 : 0;
    }

    // The k loops run in batches of levels (TDMA_KF forward, TDMA_KBK
    // backward, where the batch holds doubles): the loads of a batch do not
    // depend on the recurrence, so they are issued together and the few
    // threads of this kernel (one per column group) keep enough bytes in
    // flight to stream from HBM instead of waiting one level at a time.
    constexpr int TDMA_KF = 8;
    constexpr int TDMA_KBK = 4;

    // Output of column col at level k.  The mean mode (col 0) is not stored:
    // its level mean (X_00/jtot)/itot goes to dcm[k] and the column gets
    // zero, so that the inverse transforms carry only the other modes and the
    // large hydrostatic part of p stays out of their round-off; the inverse
    // x transform (or the scatter) adds the mean to every point.
    template<typename TF>
    __device__ __forceinline__ TF dc_out(TF val, int col, int k, int itot, int jtot, TF* __restrict__ dcm)
    {
        if (col != 0) return val;
        dcm[k] = TF((double(val) / jtot) / itot);
        return TF(0);
    }

    template<typename TF> struct TdmaP
    {
        int itot, jtot, ktot, niu, nju;
        const double *rtab, *wtab, *a, *dz2, *gtab, *htab;
        const float* stab;
        const double* stabd;
        TF* pk; double* work; TF* dcm;
        const float *gftab, *hftab;
        const unsigned char* fmode;
    };

    template<typename TF>
    __device__ __forceinline__ void tdma_body(const TdmaP<TF>& A, const VBlock& vb)
    {
        const int itot = A.itot, jtot = A.jtot, ktot = A.ktot, niu = A.niu, nju = A.nju;
        const double* __restrict__ rtab = A.rtab; const double* __restrict__ wtab = A.wtab;
        const double* __restrict__ a = A.a; const double* __restrict__ dz2 = A.dz2;
        TF* __restrict__ pk = A.pk; double* __restrict__ work = A.work; TF* __restrict__ dcm = A.dcm;
        const int iu = vb.x*blockDim.x + threadIdx.x;
        const int ju = vb.y;
        if (iu >= niu) return;
        const long long stride = (long long)niu*nju;
        const long long base = iu + (long long)ju*niu;
        const long long kk = (long long)itot*jtot;
        const int i1 = (iu == 0 || 2*iu == itot) ? -1 : itot - iu;
        const int j1 = (ju == 0 || 2*ju == jtot) ? -1 : jtot - ju;
        // The group's columns (i, j), (itot-i, j), (i, jtot-j), (itot-i, jtot-j);
        // a column that coincides with the first is masked out.  Column
        // offsets within a level are 32-bit (itot*jtot < 2^31 is checked at
        // set-up); level offsets are 64-bit pointers.
        const bool use[4] = {true, i1 >= 0, j1 >= 0, i1 >= 0 && j1 >= 0};
        const int ia = iu, ib = i1 >= 0 ? i1 : iu;
        const int ja = ju*itot, jb = (j1 >= 0 ? j1 : ju)*itot;
        const int col[4] = {ia + ja, ib + ja, ia + jb, ib + jb};

        // Forward sweep: y_k = (dz2_k p_k - a_k y_{k-1}) / den_k, rounded
        // after each operation as in src/pres_2.cxx:200-263.
        double y[4] = {0., 0., 0., 0.};
        for (int k0=0; k0<ktot; k0+=TDMA_KF)
        {
            const int nk = min(TDMA_KF, ktot - k0);
            double r[TDMA_KF];
            TF pv[TDMA_KF][4];
            #pragma unroll
            for (int b=0; b<TDMA_KF; ++b)
            {
                if (b < nk)
                {
                    const long long k = k0 + b;
                    r[b] = __ldg(&rtab[base + k*stride]);
                    const TF* row = pk + k*kk;
                    #pragma unroll
                    for (int q=0; q<4; ++q)
                        if (use[q]) pv[b][q] = row[col[q]];
                }
            }
            #pragma unroll
            for (int b=0; b<TDMA_KF; ++b)
            {
                if (b < nk)
                {
                    const int k = k0 + b;
                    const double dzk = dz2[k];
                    const double ak = a[k];
                    double* wrow = work + (long long)k*kk;
                    #pragma unroll
                    for (int q=0; q<4; ++q)
                    {
                        if (use[q])
                        {
                            double x = mulx(dzk, double(pv[b][q]));
                            if (k) x = x - mulx(ak, y[q]);
                            y[q] = x / r[b];
                            wrow[col[q]] = y[q];
                        }
                    }
                }
            }
        }
        // Back substitution: x_k = y_k - (c_k/den_k) x_{k+1}.
        {
            TF* row = pk + (long long)(ktot-1)*kk;
            #pragma unroll
            for (int q=0; q<4; ++q)
                if (use[q]) row[col[q]] = dc_out<TF>(TF(y[q]), col[q], ktot-1, itot, jtot, dcm);
        }
        for (int k0=ktot-2; k0>=0; k0-=TDMA_KBK)
        {
            const int nk = min(TDMA_KBK, k0 + 1);
            double r[TDMA_KBK];
            double wv[TDMA_KBK][4];
            #pragma unroll
            for (int b=0; b<TDMA_KBK; ++b)
            {
                if (b < nk)
                {
                    const long long k = k0 - b;
                    r[b] = __ldg(&wtab[base + k*stride]);
                    const double* wrow = work + k*kk;
                    #pragma unroll
                    for (int q=0; q<4; ++q)
                        if (use[q]) wv[b][q] = wrow[col[q]];
                }
            }
            #pragma unroll
            for (int b=0; b<TDMA_KBK; ++b)
            {
                if (b < nk)
                {
                    const int k = k0 - b;
                    const double w3 = r[b];
                    TF* row = pk + (long long)k*kk;
                    #pragma unroll
                    for (int q=0; q<4; ++q)
                    {
                        if (use[q])
                        {
                            y[q] = wv[b][q] - mulx(w3, y[q]);
                            row[col[q]] = dc_out<TF>(TF(y[q]), col[q], k, itot, jtot, dcm);
                        }
                    }
                }
            }
        }
    }

    template<typename TF> __device__ __forceinline__ double to_f64(TF v);
    template<> __device__ __forceinline__ double to_f64<float>(float v) { return f2d_exact(v); }
    template<> __device__ __forceinline__ double to_f64<double>(double v) { return v; }

    // Output x_k = s_k xi_k in the field precision: in float the product of
    // the rounded factors (the result is stored in float anyway).
    template<typename TF> __device__ __forceinline__ TF scale_out(double xi, float s, double sd);
    template<> __device__ __forceinline__ float scale_out<float>(double xi, float s, double) { return d2f_rn(xi)*s; }
    template<> __device__ __forceinline__ double scale_out<double>(double xi, float, double sd) { return xi*sd; }

    // The Thomas solve with the rescaled recurrence (coefficients from
    // k_tdma_table): in the float form the whole solve costs two FP64 FMAs
    // per cell, the elimination itself staying in double.
    template<typename TF>
    __device__ __forceinline__ void tdma_scaled_body(const TdmaP<TF>& A, const VBlock& vb)
    {
        const int itot = A.itot, jtot = A.jtot, ktot = A.ktot, niu = A.niu, nju = A.nju;
        const double* __restrict__ gtab = A.gtab; const double* __restrict__ htab = A.htab;
        const float* __restrict__ stab = A.stab; const double* __restrict__ stabd = A.stabd;
        TF* __restrict__ pk = A.pk; double* __restrict__ work = A.work; TF* __restrict__ dcm = A.dcm;
        const int iu = vb.x*blockDim.x + threadIdx.x;
        const int ju = vb.y;
        if (iu >= niu) return;
        const long long stride = (long long)niu*nju;
        const long long base = iu + (long long)ju*niu;
        const long long kk = (long long)itot*jtot;
        const int i1 = (iu == 0 || 2*iu == itot) ? -1 : itot - iu;
        const int j1 = (ju == 0 || 2*ju == jtot) ? -1 : jtot - ju;
        const bool use[4] = {true, i1 >= 0, j1 >= 0, i1 >= 0 && j1 >= 0};
        const int ia = iu, ib = i1 >= 0 ? i1 : iu;
        const int ja = ju*itot, jb = (j1 >= 0 ? j1 : ju)*itot;
        const int col[4] = {ia + ja, ib + ja, ia + jb, ib + jb};

        // Forward: z_k = p_k - g_k z_{k-1}.
        double z[4] = {0., 0., 0., 0.};
        for (int k0=0; k0<ktot; k0+=TDMA_KF)
        {
            const int nk = min(TDMA_KF, ktot - k0);
            double g[TDMA_KF];
            TF pv[TDMA_KF][4];
            #pragma unroll
            for (int b=0; b<TDMA_KF; ++b)
            {
                if (b < nk)
                {
                    const long long k = k0 + b;
                    g[b] = __ldg(&gtab[base + k*stride]);
                    const TF* row = pk + k*kk;
                    #pragma unroll
                    for (int q=0; q<4; ++q)
                        if (use[q]) pv[b][q] = row[col[q]];
                }
            }
            #pragma unroll
            for (int b=0; b<TDMA_KF; ++b)
            {
                if (b < nk)
                {
                    double* wrow = work + (long long)(k0 + b)*kk;
                    #pragma unroll
                    for (int q=0; q<4; ++q)
                    {
                        if (use[q])
                        {
                            z[q] = fma(-g[b], z[q], to_f64<TF>(pv[b][q]));
                            wrow[col[q]] = z[q];
                        }
                    }
                }
            }
        }
        // Backward: xi_k = z_k - h_k xi_{k+1}; x_k = s_k xi_k.
        {
            const long long k = ktot - 1;
            const float s = __ldg(&stab[base + k*stride]);
            const double sd = sizeof(TF) == 8 ? __ldg(&stabd[base + k*stride]) : 0.;
            TF* row = pk + k*kk;
            #pragma unroll
            for (int q=0; q<4; ++q)
                if (use[q]) row[col[q]] = dc_out<TF>(scale_out<TF>(z[q], s, sd), col[q], (int)k, itot, jtot, dcm);
        }
        for (int k0=ktot-2; k0>=0; k0-=TDMA_KBK)
        {
            const int nk = min(TDMA_KBK, k0 + 1);
            double h[TDMA_KBK], sd[TDMA_KBK];
            float s[TDMA_KBK];
            double zv[TDMA_KBK][4];
            #pragma unroll
            for (int b=0; b<TDMA_KBK; ++b)
            {
                if (b < nk)
                {
                    const long long k = k0 - b;
                    h[b] = __ldg(&htab[base + k*stride]);
                    s[b] = __ldg(&stab[base + k*stride]);
                    sd[b] = sizeof(TF) == 8 ? __ldg(&stabd[base + k*stride]) : 0.;
                    const double* wrow = work + k*kk;
                    #pragma unroll
                    for (int q=0; q<4; ++q)
                        if (use[q]) zv[b][q] = wrow[col[q]];
                }
            }
            #pragma unroll
            for (int b=0; b<TDMA_KBK; ++b)
            {
                if (b < nk)
                {
                    TF* row = pk + (long long)(k0 - b)*kk;
                    #pragma unroll
                    for (int q=0; q<4; ++q)
                    {
                        if (use[q])
                        {
                            z[q] = fma(-h[b], z[q], zv[b][q]);
                            row[col[q]] = dc_out<TF>(scale_out<TF>(z[q], s[b], sd[b]), col[q], k0 - b, itot, jtot, dcm);
                        }
                    }
                }
            }
        }
    }

    // The rescaled solve with one column per thread: the four columns that
    // share the coefficients of one eigenvalue (i, itot-i) x (j, jtot-j) sit
    // in four adjacent lanes, which read the same table entries in one
    // transaction.  Four times the threads of k_tdma_scaled, so that the FP64
    // recurrences and the loads of the next levels of other warps overlap.
    constexpr int TDC_KF = 8;
    constexpr int TDC_KB = 4;

    template<typename TF>
    __device__ __forceinline__ void tdma_col_fp64(const TdmaP<TF>& A, int col, long long base);

    // At most 64 registers, so that eight blocks (32 warps) fit on an SM:
    // the loads of one warp's next levels overlap the FP64 recurrences of
    // the others.
    template<typename TF>
    __device__ __forceinline__ void tdma_col_body(const TdmaP<TF>& A, const VBlock& vb)
    {
        const int itot = A.itot, jtot = A.jtot, niu = A.niu;
        const int t = vb.x*blockDim.x + threadIdx.x;
        const int iu = t >> 2, q = t & 3;
        const int ju = vb.y;
        if (iu >= niu) return;
        const int i1 = (iu == 0 || 2*iu == itot) ? -1 : itot - iu;
        const int j1 = (ju == 0 || 2*ju == jtot) ? -1 : jtot - ju;
        // Lane q holds column (q&1 ? itot-i : i, q&2 ? jtot-j : j); a mirror
        // that coincides with the first column has no lane.
        if (((q & 1) && i1 < 0) || ((q & 2) && j1 < 0)) return;
        const int col = ((q & 1) ? i1 : iu) + ((q & 2) ? j1 : ju)*itot;
        tdma_col_fp64<TF>(A, col, iu + (long long)ju*niu);
    }

    // One column's rescaled solve with the elimination in FP64 (forward
    // values in the FP64 work array).
    template<typename TF>
    __device__ __forceinline__ void tdma_col_fp64(const TdmaP<TF>& A, int col, long long base)
    {
        const int itot = A.itot, jtot = A.jtot, ktot = A.ktot;
        const double* __restrict__ gtab = A.gtab; const double* __restrict__ htab = A.htab;
        const float* __restrict__ stab = A.stab; const double* __restrict__ stabd = A.stabd;
        TF* __restrict__ pk = A.pk; double* __restrict__ work = A.work; TF* __restrict__ dcm = A.dcm;
        const long long stride = (long long)A.niu*A.nju;
        const long long kk = (long long)itot*jtot;

        // Forward: z_k = p_k - g_k z_{k-1}.
        double z = 0.;
        for (int k0=0; k0<ktot; k0+=TDC_KF)
        {
            const int nk = min(TDC_KF, ktot - k0);
            double g[TDC_KF];
            TF pv[TDC_KF];
            #pragma unroll
            for (int b=0; b<TDC_KF; ++b)
                if (b < nk)
                {
                    g[b] = __ldg(gtab + base + (long long)(k0 + b)*stride);
                    pv[b] = pk[col + (long long)(k0 + b)*kk];
                }
            #pragma unroll
            for (int b=0; b<TDC_KF; ++b)
                if (b < nk)
                {
                    z = fma(-g[b], z, to_f64<TF>(pv[b]));
                    work[col + (long long)(k0 + b)*kk] = z;
                }
        }
        // Backward: xi_k = z_k - h_k xi_{k+1}; x_k = s_k xi_k.
        {
            const long long k = ktot - 1;
            const float s = __ldg(stab + base + k*stride);
            const double sd = sizeof(TF) == 8 ? __ldg(stabd + base + k*stride) : 0.;
            pk[col + k*kk] = dc_out<TF>(scale_out<TF>(z, s, sd), col, (int)k, itot, jtot, dcm);
        }
        for (int k0=ktot-2; k0>=0; k0-=TDC_KB)
        {
            const int nk = min(TDC_KB, k0 + 1);
            double h[TDC_KB], sd[TDC_KB], zv[TDC_KB];
            float s[TDC_KB];
            #pragma unroll
            for (int b=0; b<TDC_KB; ++b)
                if (b < nk)
                {
                    const long long k = k0 - b;
                    h[b] = __ldg(htab + base + k*stride);
                    s[b] = __ldg(stab + base + k*stride);
                    sd[b] = sizeof(TF) == 8 ? __ldg(stabd + base + k*stride) : 0.;
                    zv[b] = work[col + k*kk];
                }
            #pragma unroll
            for (int b=0; b<TDC_KB; ++b)
                if (b < nk)
                {
                    z = fma(-h[b], z, zv[b]);
                    pk[col + (long long)(k0 - b)*kk] = dc_out<TF>(scale_out<TF>(z, s[b], sd[b]), col, k0 - b, itot, jtot, dcm);
                }
        }
    }

    // The rescaled solve in float for the column groups whose sweeps damp
    // (fmode, set with the tables), in FP64 for the others.  A float column
    // keeps its forward values in pk itself, where the backward sweep
    // overwrites them with the solution: 16 bytes per cell move instead of
    // 24 (float right-hand side and solution, FP64 work array), the tables
    // are read in float, no FP64 instruction runs, and the loads run sixteen
    // levels ahead of the recurrence.  Lanes as in k_tdma_col; a group's
    // four lanes take the same branch.
    constexpr int TDF_KF = 16;
    constexpr int TDF_KB = 8;

    __device__ __forceinline__ void tdma_mixed_body(const TdmaP<float>& A, const VBlock& vb)
    {
        const int itot = A.itot, jtot = A.jtot, ktot = A.ktot, niu = A.niu;
        const int t = vb.x*blockDim.x + threadIdx.x;
        const int iu = t >> 2, q = t & 3;
        const int ju = vb.y;
        if (iu >= niu) return;
        const int i1 = (iu == 0 || 2*iu == itot) ? -1 : itot - iu;
        const int j1 = (ju == 0 || 2*ju == jtot) ? -1 : jtot - ju;
        if (((q & 1) && i1 < 0) || ((q & 2) && j1 < 0)) return;
        const int col = ((q & 1) ? i1 : iu) + ((q & 2) ? j1 : ju)*itot;
        const long long base = iu + (long long)ju*niu;
        if (!A.fmode[base])
        {
            tdma_col_fp64<float>(A, col, base);
            return;
        }
        const float* __restrict__ gf = A.gftab; const float* __restrict__ hf = A.hftab;
        const float* __restrict__ stab = A.stab;
        float* __restrict__ pk = A.pk;
        const long long stride = (long long)niu*A.nju;
        const long long kk = (long long)itot*jtot;

        // Forward: z_k = p_k - g_k z_{k-1}, stored over p_k.
        float z = 0.f;
        for (int k0=0; k0<ktot; k0+=TDF_KF)
        {
            const int nk = min(TDF_KF, ktot - k0);
            float g[TDF_KF], pv[TDF_KF];
            #pragma unroll
            for (int b=0; b<TDF_KF; ++b)
                if (b < nk)
                {
                    g[b] = __ldg(gf + base + (long long)(k0 + b)*stride);
                    pv[b] = pk[col + (long long)(k0 + b)*kk];
                }
            #pragma unroll
            for (int b=0; b<TDF_KF; ++b)
                if (b < nk)
                {
                    z = fmaf(-g[b], z, pv[b]);
                    pk[col + (long long)(k0 + b)*kk] = z;
                }
        }
        // Backward: xi_k = z_k - h_k xi_{k+1}; x_k = s_k xi_k.
        pk[col + (long long)(ktot - 1)*kk] = z*__ldg(stab + base + (long long)(ktot - 1)*stride);
        float xi = z;
        for (int k0=ktot-2; k0>=0; k0-=TDF_KB)
        {
            const int nk = min(TDF_KB, k0 + 1);
            float h[TDF_KB], sv[TDF_KB], zv[TDF_KB];
            #pragma unroll
            for (int b=0; b<TDF_KB; ++b)
                if (b < nk)
                {
                    const long long k = k0 - b;
                    h[b] = __ldg(hf + base + k*stride);
                    sv[b] = __ldg(stab + base + k*stride);
                    zv[b] = pk[col + k*kk];
                }
            #pragma unroll
            for (int b=0; b<TDF_KB; ++b)
                if (b < nk)
                {
                    xi = fmaf(-h[b], xi, zv[b]);
                    pk[col + (long long)(k0 - b)*kk] = xi*sv[b];
                }
        }
    }

    int tdma_table(PresWork& pw, int itot, int jtot, int ktot, cudaStream_t s)
    {
        pw.niu = itot/2 + 1;
        pw.nju = jtot/2 + 1;
        const size_t n = (size_t)pw.niu*pw.nju*ktot;
        if (cudaMallocAsync((void**)&pw.rtab, sizeof(double)*n, s) != cudaSuccess) return MHH_ERR_CUDA;
        if (cudaMallocAsync((void**)&pw.wtab, sizeof(double)*n, s) != cudaSuccess) return MHH_ERR_CUDA;
        if (cudaMallocAsync((void**)&pw.gtab, sizeof(double)*n, s) != cudaSuccess) return MHH_ERR_CUDA;
        if (cudaMallocAsync((void**)&pw.htab, sizeof(double)*n, s) != cudaSuccess) return MHH_ERR_CUDA;
        if (cudaMallocAsync((void**)&pw.stab, sizeof(float)*n, s) != cudaSuccess) return MHH_ERR_CUDA;
        if (cudaMallocAsync((void**)&pw.stabd, sizeof(double)*n, s) != cudaSuccess) return MHH_ERR_CUDA;
        if (cudaMallocAsync((void**)&pw.gftab, sizeof(float)*n, s) != cudaSuccess) return MHH_ERR_CUDA;
        if (cudaMallocAsync((void**)&pw.hftab, sizeof(float)*n, s) != cudaSuccess) return MHH_ERR_CUDA;
        if (cudaMallocAsync((void**)&pw.fmode, (size_t)pw.niu*pw.nju, s) != cudaSuccess) return MHH_ERR_CUDA;
        dim3 grid((pw.niu + 127)/128, pw.nju);
        k_tdma_table<<<grid, 128, 0, s>>>(pw.niu, pw.nju, ktot, pw.bmati, pw.bmatj, pw.a, pw.c, pw.dz2rho, pw.dz2,
                                    pw.rtab, pw.wtab, pw.gtab, pw.htab, pw.stab, pw.stabd, pw.gftab, pw.hftab,
                                    pw.fmode);
        count_launch();
        return cudaStreamSynchronize(s) == cudaSuccess ? MHH_OK : MHH_ERR_CUDA;
    }

    template<typename TF>
    void launch_tdma(const Dims& d, const PresWork& pw, TF* pk, const KernelOpts& o, cudaStream_t s)
    {
        dim3 grid((pw.niu + 127)/128, pw.nju);
        TF* dcm = static_cast<TF*>(pw.dcm);
        int v = o.tdma < 0 ? (sizeof(TF) == 4 ? 3 : 0) : o.tdma;
        if (v == 3 && sizeof(TF) == 8) v = 1;
        const TdmaP<TF> A{d.itot, d.jtot, d.ktot, pw.niu, pw.nju, pw.rtab, pw.wtab, pw.a, pw.dz2, pw.gtab, pw.htab,
                          pw.stab, pw.stabd, pk, pw.work, dcm, pw.gftab, pw.hftab, pw.fmode};
        if constexpr (sizeof(TF) == 4)
        {
            if (v == 3)
            {
                dim3 gridc((4*pw.niu + 127)/128, pw.nju);
                launch_body<TdmaP<float>, tdma_mixed_body, 128, 8>(gridc, dim3(128), 0, s, A);
                count_launch();
                return;
            }
        }
        if (v == 1)
        {
            dim3 gridc((4*pw.niu + 127)/128, pw.nju);
            launch_body<TdmaP<TF>, tdma_col_body<TF>, 128, 8>(gridc, dim3(128), 0, s, A);
        }
        else if (v == 2)
            launch_body<TdmaP<TF>, tdma_scaled_body<TF>, 128>(grid, dim3(128), 0, s, A);
        else
            launch_body<TdmaP<TF>, tdma_body<TF>, 128>(grid, dim3(128), 0, s, A);
        count_launch();
    }

    // Packed solution back into the ghost layout with the bottom ghost level
    // p[kstart-1] = p[kstart], src/pres_2.cxx:330-358 (the periodic fill
    // follows separately).
    template<typename TF>
    __global__ void k_pres_scatter(Dims d, const TF* __restrict__ pk, const TF* __restrict__ dcm, TF* __restrict__ p)
    {
        const int i = blockIdx.x*blockDim.x + threadIdx.x;
        const int j = blockIdx.y*blockDim.y + threadIdx.y;
        const int k = blockIdx.z;
        if (i >= d.itot || j >= d.jtot) return;
        const TF val = add_rn(pk[i + (long long)j*d.itot + (long long)k*d.itot*d.jtot], dcm[k]);
        const long long c = ijk(d, i + d.igc, j + d.jgc, k + d.kgc);
        p[c] = val;
        if (k == 0) p[c - d.ijcells] = val;
    }

    template<typename TF>
    void launch_pres_scatter(const Dims& d, const TF* pk, const TF* dcm, TF* p, cudaStream_t s)
    {
        dim3 block(32, 8);
        dim3 grid((d.itot + 31)/32, (d.jtot + 7)/8, d.ktot);
        k_pres_scatter<TF><<<grid, block, 0, s>>>(d, pk, dcm, p);
        count_launch();
    }

#define MHH_PRES_INST(TF) \
    template void launch_pres_in<TF>(const Dims&, const Prof<TF>&, const TF*, const TF*, const TF*, const TF*, const TF*, const TF*, TF*, double, cudaStream_t); \
    template void launch_fft_x<TF>(const FftPlan&, TF*, int, bool, double, cudaStream_t, const FftFuse<TF>*); \
    template void launch_fft_y<TF>(const FftPlan&, TF*, int, int, int, bool, double, cudaStream_t); \
    template void launch_tdma<TF>(const Dims&, const PresWork&, TF*, const KernelOpts&, cudaStream_t); \
    template void launch_pres_scatter<TF>(const Dims&, const TF*, const TF*, TF*, cudaStream_t);

    MHH_PRES_INST(double)
    MHH_PRES_INST(float)
}
