// mhh_kernels.cuh -- launchers of the device kernels (host-side declarations).
#pragma once

#include "mhh_common.cuh"

namespace mhh
{
    void count_launch(int n = 1);
    long long launch_count();

    // Advection switch passed to launch_tendency for Advec_2i5 with the flux
    // limiter on the scalar (momentum as MHH_ADVEC_2I5).
    constexpr int ADVEC_2I5_LIM = 26;

    // Kernel choices of one call: variant switches (-1 = automatic) and the
    // level-chunk height of the marching kernels (0 = default 32).
    struct KernelOpts
    {
        int tend, visc, tdma;
        int tend_kchunk, visc_kchunk;
    };

    // Level-chunk height of a marching kernel with `tiles` blocks per chunk
    // row: the requested height, or for 0 64 where that gives eight blocks
    // per SM, else the largest of 32, 16, 8 that still gives two (small grids
    // get more, shorter chunks).
    int auto_kchunk(int requested, long long tiles, int ktot);

    // Read-only view of a context for kernels in other translation units.
    const Dims& ctx_dims(const mhh_ctx* c);
    int ctx_precision(const mhh_ctx* c);
    const Prof<double>& ctx_prof_double(const mhh_ctx* c);
    const Prof<float>& ctx_prof_float(const mhh_ctx* c);
    // Kernel variant of the LES tendencies: 0 = one thread per cell with
    // cached global loads, 1 = tiled shared-memory planes marching in k,
    // 2 = flux form (every face flux once) marching in k; -1 = automatic
    // (2 for float fields, 0 for double fields; the default).
    int tendency_variant();
    void set_tendency_variant(int v);

    template<typename TF>
    struct FieldList
    {
        int n;
        TF* p[8];
    };

    template<typename TF>
    struct GhostList
    {
        int n;
        TF* a[4];
        int bot_type[4], top_type[4];
        const TF* abot[4];
        const TF* agradbot[4];
        const TF* atop[4];
        const TF* agradtop[4];
    };

    template<typename TF>
    struct TendArgs
    {
        const TF *u, *v, *w, *s, *evisc;
        TF *ut, *vt, *wt, *st;
        const TF *u_fluxbot, *u_fluxtop, *v_fluxbot, *v_fluxtop, *s_fluxbot, *s_fluxtop;
        TF visc, svisc, tpri, fbody;
        double dxidxi, dyidyi;
        TF dxidxi_t, dyidyi_t;
    };

    template<typename TF> void launch_cyclic(const FieldList<TF>& fl, const Dims& d, int edges, cudaStream_t s);
    template<typename TF> void launch_cyclic2d(TF* a, const Dims& d, cudaStream_t s);
    template<typename TF> void launch_set_bc(TF* val, TF* grad, TF* flux, int type, double aval, double visc,
                                             int sfg, const Dims& d, cudaStream_t s);
    template<typename TF> void launch_ghost(const GhostList<TF>& gl, const Dims& d, const TF* dzh, cudaStream_t s);
    template<typename TF> void launch_viscosity(const Dims& d, const Prof<TF>& pr, const TF* u, const TF* v, const TF* w,
                                                const TF* th, TF* evisc, const TF* mlen2, const double* dudz,
                                                const double* dvdz, const double* dbdz, double cs, double tpr,
                                                double visc, int mason, bool surf, bool thermo, const KernelOpts& o,
                                                cudaStream_t s);
    template<typename TF> bool launch_viscosity_planes(const Dims& d, const Prof<TF>& pr, const TF* u, const TF* v,
                                                       const TF* w, const TF* th, TF* evisc, const TF* mlen2,
                                                       const double* dudz, const double* dvdz, const double* dbdz,
                                                       double tpr, bool surf, bool thermo, int kchunk, cudaStream_t s);
    // Viscosity kernel: 0 = per cell, 1 = shared-memory planes marching in k;
    // -1 = automatic (1 for float fields, 0 for double fields).
    int viscosity_variant();
    void set_viscosity_variant(int v);
    template<typename TF> void launch_tendency(const Dims& d, const Prof<TF>& pr, const TendArgs<TF>& a, int adv, int dif,
                                               bool surf, bool scal, bool buoy, bool force, const KernelOpts& o,
                                               cudaStream_t s);
    template<typename TF> void launch_tendency_les(const Dims& d, const Prof<TF>& pr, const TendArgs<TF>& a,
                                                   bool surf, bool scal, bool buoy, cudaStream_t s);
    // lim: the scalar is advected with the flux limiter.
    template<typename TF> void launch_tendency_flux(const Dims& d, const Prof<TF>& pr, const TendArgs<TF>& a,
                                                    bool surf, bool scal, bool buoy, bool lim, int kchunk,
                                                    cudaStream_t s);
    // Buffer-layer relaxation, src/buffer.cxx:37-59: prof holds, kcells each,
    // sigma(z) at full levels, sigma(zh) at half levels (zero below the
    // layer) and the u, v, s buffer profiles.
    template<typename TF> void launch_buffer(const Dims& d, const TF* prof, int kb, const TF* u, const TF* v,
                                             const TF* w, const TF* s, TF* ut, TF* vt, TF* wt, TF* st,
                                             cudaStream_t strm);
    template<typename TF> void launch_rk3(TF* a, TF* at, const Dims& d, int substep, double dt, cudaStream_t s);
    template<typename TF> void launch_presout_rk3(const Dims& d, const Prof<TF>& pr, const TF* p, TF* u, TF* v, TF* w,
                                                  TF* s, TF* ut, TF* vt, TF* wt, TF* st, int substep, double dt,
                                                  cudaStream_t strm);
    template<typename TF> void launch_reduce(int what, const Dims& d, const Prof<TF>& pr, const TF* u, const TF* v,
                                             const TF* w, const TF* ev, double tprfi, unsigned long long* out,
                                             cudaStream_t s);

    // ---- pressure solver (mhh_pres.cu) ----
    struct FftPlan
    {
        int n;
        int nfac;
        int fac[16];
        double* tw_d;     // exp(-2 pi i k/n), k < n, as (re, im) pairs (double)
        float* tw_f;      // the same in float
    };

    // Set-up and release on a stream: allocations are stream-ordered
    // (cudaMallocAsync / cudaFreeAsync), so neither synchronises the device.
    int fft_plan_init(FftPlan* pl, int n, cudaStream_t s);
    void fft_plan_free(FftPlan* pl, cudaStream_t s);

    struct PresWork
    {
        FftPlan px, py;
        void* pk;             // packed itot*jtot*ktot field (TF)
        double* bmati;        // itot
        double* bmatj;        // jtot
        double* a;            // ktot
        double* c;            // ktot
        double* dz2;          // ktot: dz^2
        double* dz2rho;       // ktot: dz^2 * rhoref
        double* work;         // itot*jtot*ktot doubles: forward-swept right-hand side
        double* rtab;         // (itot/2+1)*(jtot/2+1)*ktot: den per column group and level
        double* wtab;         // same shape: c_k/den_k, the back-substitution factor
        double* gtab;         // same shape: forward coefficient of the rescaled recurrence
        double* htab;         // same shape: backward coefficient of the rescaled recurrence
        float* stab;          // same shape: output scale dz^2/den in float
        double* stabd;        // same shape: output scale dz^2/den
        float* gftab;         // same shape: gtab in float
        float* hftab;         // same shape: htab in float
        unsigned char* fmode; // (itot/2+1)*(jtot/2+1): 1 where the group's recurrence may run in float
        void* dcm;            // ktot values (TF): each level's mean, (X_00/jtot)/itot
        int niu, nju;
    };

    // Tridiagonal kernel choice: 0 = the reference's operation order,
    // 1 = the rescaled recurrence (two FP64 FMAs per cell), 2 = the same with
    // four columns per thread, 3 = the rescaled recurrence in float for the
    // column groups whose sweeps damp (float fields only; 1 for double
    // fields); -1 = automatic (0 for double fields, 3 for float fields).
    int tdma_variant();
    void set_tdma_variant(int v);
    // Complex sequence pairs per block of the column (y) FFT: 4 or 8.
    int fft_column_pairs();
    int fft_pipeline();
    // 1 (default): the pressure right-hand side and the scatter into p are
    // fused into the x transforms; 0: separate kernels.
    int pres_fuse();
    void set_fft_column_pairs(int p);

    int tdma_table(PresWork& pw, int itot, int jtot, int ktot, cudaStream_t s);

    template<typename TF> void launch_pres_in(const Dims& d, const Prof<TF>& pr, const TF* u, const TF* v, const TF* w,
                                              const TF* ut, const TF* vt, const TF* wt, TF* pk, double dti, cudaStream_t s);
    // Work fused into the row (x) FFT: mode 1 computes the pressure
    // right-hand side in place of loading the forward transform's input;
    // mode 2 stores the inverse transform's output into the ghost layout of p.
    // With mode 2, dcm (if set) holds each level's mean, which the tridiagonal
    // solve took out of the mean mode; it is added to every stored point.
    template<typename TF>
    struct FftFuse
    {
        int mode;
        Dims d;
        Prof<TF> pr;
        const TF *u, *v, *w, *ut, *vt, *wt;
        TF dti;
        TF* p;
        const TF* dcm;
    };
    template<typename TF> void launch_fft_x(const FftPlan& pl, TF* data, int nrows, bool inverse, double scale, cudaStream_t s,
                                            const FftFuse<TF>* fuse = nullptr);
    template<typename TF> void launch_fft_y(const FftPlan& pl, TF* data, int itot, int jtot, int ktot, bool inverse,
                                            double scale, cudaStream_t s);
    template<typename TF> void launch_tdma(const Dims& d, const PresWork& pw, TF* pk, const KernelOpts& o, cudaStream_t s);
    template<typename TF> void launch_pres_scatter(const Dims& d, const TF* pk, const TF* dcm, TF* p, cudaStream_t s);

    // ---- surface layer (mhh_surface.cu) ----
    struct SurfWork
    {
        double *ustar, *obuk, *dudz, *dvdz, *dbdz, *dutot;
        double *fm, *fh, *phim, *phih;   // per-cell Monin-Obukhov functions of the last stability call
        double z0h;
        int* nobuk;
        float *zL, *f;
        double *mlen2;   // kcells: squared Smagorinsky mixing length per level
        float *mlen2f;   // the same in float
        double zsl;      // height of the first full level
        double thref_s, threfh_s;  // reference potential temperature at kstart (full, half)
        double thb_s, thbh_s;      // the same in the scalar's storage units
    };

    template<typename TF> void launch_surface(const Dims& d, const Prof<TF>& pr, const SurfWork& sw,
                                              const TF* u, const TF* v, const TF* s,
                                              TF* u_bot, TF* v_bot, TF* u_flux, TF* v_flux, TF* u_grad, TF* v_grad,
                                              TF* s_bot, TF* s_flux, TF* s_grad,
                                              int thermo, int thermo_bc, double z0m, double z0h, cudaStream_t st);
}
