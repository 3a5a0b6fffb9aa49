// mhh_capi.cu -- the C-ABI of include/mhh.h: context set-up (grid metrics,
// device profiles, all scratch) and the module entry points that the
// reference's Advec / Diff / Pres / Timeloop / Boundary classes would call.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "mhh_kernels.cuh"
#include "mhh_batchable.cuh"

namespace
{
    thread_local std::string g_last_error;
    std::atomic<long long> g_launches{0};

    // Live per-kernel timing: CUDA events recorded on the launching stream
    // around each kernel group, collected after a synchronisation.
    struct TimerEntry { std::string name; long long count = 0; double ms = 0.; };
    struct PendingPair { int idx; cudaEvent_t a, b; };
    bool g_timing = false;
    std::vector<TimerEntry> g_timers;
    std::vector<PendingPair> g_pending;
    std::vector<cudaEvent_t> g_event_pool;

    cudaEvent_t take_event()
    {
        if (!g_event_pool.empty()) { cudaEvent_t e = g_event_pool.back(); g_event_pool.pop_back(); return e; }
        cudaEvent_t e;
        cudaEventCreate(&e);
        return e;
    }

    int timer_index(const char* name)
    {
        for (size_t q=0; q<g_timers.size(); ++q) if (g_timers[q].name == name) return (int)q;
        g_timers.push_back(TimerEntry{name, 0, 0.});
        return (int)g_timers.size() - 1;
    }

    struct Timed
    {
        PendingPair pp;
        cudaStream_t s;
        bool on;
        Timed(const char* name, cudaStream_t st) : s(st), on(g_timing)
        {
            if (!on) return;
            pp.idx = timer_index(name);
            pp.a = take_event(); pp.b = take_event();
            cudaEventRecord(pp.a, s);
        }
        ~Timed()
        {
            if (!on) return;
            cudaEventRecord(pp.b, s);
            g_pending.push_back(pp);
        }
    };
}

void mhh_set_last_error(const char* msg) { g_last_error = msg ? msg : ""; }

namespace mhh
{
    void count_launch(int n) { g_launches += n; }
    static int g_tend_variant = -1;
    int tendency_variant() { return g_tend_variant; }
    void set_tendency_variant(int v) { g_tend_variant = v; }
    static int g_visc_variant = -1;
    int viscosity_variant() { return g_visc_variant; }
    void set_viscosity_variant(int v) { g_visc_variant = v; }
    static int g_tend_kchunk = 0, g_visc_kchunk = 0;
    static int g_fft_col_pairs = 8;
    static int g_pres_fuse = 1;
    int pres_fuse() { return g_pres_fuse; }
    int fft_column_pairs() { return g_fft_col_pairs; }
    static int g_fft_pipeline = 1;
    int fft_pipeline() { return g_fft_pipeline; }
    void set_fft_column_pairs(int p) { g_fft_col_pairs = p; }
    static int g_tdma_variant = -1;
    int tdma_variant() { return g_tdma_variant; }
    void set_tdma_variant(int v) { g_tdma_variant = v; }
    long long launch_count() { return g_launches.load(); }

    int auto_kchunk(int requested, long long tiles, int ktot)
    {
        if (requested > 0) return requested;
        static const int nsm = []
        {
            int dev = 0, n = 0;
            cudaGetDevice(&dev);
            cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
            return n > 0 ? n : 152;
        }();
        // 64 levels (fewer halo levels per chunk) while the grid still gives
        // eight blocks per SM; else 32, halved while it gives fewer than two.
        if (tiles*((ktot + 63)/64) >= 8LL*nsm) return 64;
        int kc = 32;
        while (kc > 8 && tiles*((ktot + kc - 1)/kc) < 2LL*nsm) kc /= 2;
        return kc;
    }

    // a += delta over a whole 3-D field (mhh_field_shift).
    template<typename TF>
    __global__ void k_shift(TF* __restrict__ a, long long n, TF delta)
    {
        for (long long q = blockIdx.x*(long long)blockDim.x + threadIdx.x; q < n; q += (long long)gridDim.x*blockDim.x)
            a[q] += delta;
    }

    template<typename TF>
    __global__ void k_pres_out(Dims d, Prof<TF> pr, const TF* __restrict__ p,
                               TF* __restrict__ ut, TF* __restrict__ vt, TF* __restrict__ wt)
    {
        const int i = d.istart + blockIdx.x*blockDim.x + threadIdx.x;
        const int j = d.jstart + blockIdx.y*blockDim.y + threadIdx.y;
        const int k = d.kstart + blockIdx.z;
        if (i >= d.iend || j >= d.jend) return;
        const long long c = ijk(d, i, j, k);
        const TF pc = ld(p, c);
        ut[c] -= mulx(pc - ld(p, c-1), dxi_of<TF>(d));
        vt[c] -= mulx(pc - ld(p, c-d.icells), dyi_of<TF>(d));
        wt[c] -= mulx(pc - ld(p, c-d.ijcells), ld(pr.dzhi, k));
    }
}

using namespace mhh;

struct mhh_ctx
{
    mhh_grid g;
    Dims d;
    int prec;
    mhh_physics phys;

    // Host profiles (double), device profiles (one precision).
    std::vector<double> h[14];
    void* dprof[14];
    Prof<double> pd;
    Prof<float> pf;
    // Storage offset of the scalar theta: FP32 contexts with thermodynamics
    // store theta - thref0 (0 elsewhere).
    double th0;

    PresWork pw;
    SurfWork sw;
    int surf_ready;
    // Per-context kernel choices (-2 = follow the process-wide option).
    int opt_tend, opt_visc, opt_tdma, opt_tend_kchunk, opt_visc_kchunk;
    size_t dev_bytes;               // device memory allocated by this context
    cudaStream_t setup;             // set-up and release stream (stream-ordered allocations)

    double* statbuf;              // 2*kcells: mean and variance profiles
    // Buffer layer: 5*kcells values in the field precision (sigma at full
    // and half levels, u, v, s profiles), the host copy in double, and the
    // first level the layer touches.
    void* bufprof;
    std::vector<double> hbuf;
    int buf_on, buf_kb, buf_set;   // buf_set: bits of the u, v, th profiles given
    int fluxlimit_s;               // Advec_2i5 advects the scalar with the flux limiter
    unsigned long long* red;      // device reduction word
    unsigned long long* red_host; // pinned host copy
    double dnmul2;                // Diff_2 multiplier
};

namespace mhh
{
    const Dims& ctx_dims(const mhh_ctx* c) { return c->d; }
    int ctx_precision(const mhh_ctx* c) { return c->prec; }
    const Prof<double>& ctx_prof_double(const mhh_ctx* c) { return c->pd; }
    const Prof<float>& ctx_prof_float(const mhh_ctx* c) { return c->pf; }
}

namespace
{
    enum { P_Z, P_ZH, P_DZ, P_DZH, P_DZI, P_DZHI, P_RHO, P_RHOH, P_TH, P_THH, P_ZF, P_ZFH, P_THB, P_THBH, NPROF };
    const char* prof_names[NPROF] = {"z", "zh", "dz", "dzh", "dzi", "dzhi", "rhoref", "rhorefh", "thref", "threfh",
                                     "zfac", "zfach", "thb", "thbh"};

    int fail(int code, const char* msg) { mhh_set_last_error(msg); return code; }

    template<typename TF> const Prof<TF>& prof(const mhh_ctx* c);
    template<> const Prof<double>& prof<double>(const mhh_ctx* c) { return c->pd; }
    template<> const Prof<float>& prof<float>(const mhh_ctx* c) { return c->pf; }

    int check_cuda(const char* where)
    {
        const cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess)
        {
            std::string m = std::string(where) + ": " + cudaGetErrorString(e);
            mhh_set_last_error(m.c_str());
            return MHH_ERR_CUDA;
        }
        return MHH_OK;
    }

    // src/grid.cxx:245-305, second order.
    void grid_metrics(mhh_ctx* c, const double* zin)
    {
        const Dims& d = c->d;
        for (auto& v : c->h) v.assign(d.kcells, 0.);
        auto& z = c->h[P_Z]; auto& zh = c->h[P_ZH]; auto& dz = c->h[P_DZ];
        auto& dzh = c->h[P_DZH]; auto& dzi = c->h[P_DZI]; auto& dzhi = c->h[P_DZHI];
        const int ks = d.kstart, ke = d.kend, kc = d.kcells;
        for (int k=0; k<d.ktot; ++k) z[k + ks] = zin[k];
        z[ks-1] = -z[ks];
        z[ke] = 2.*d.zsize - z[ke-1];
        for (int k=ks+1; k<ke; ++k) zh[k] = 0.5*(z[k-1] + z[k]);
        zh[ks] = 0.;
        zh[ke] = d.zsize;
        for (int k=1; k<kc; ++k) { dzh[k] = z[k] - z[k-1]; dzhi[k] = 1./dzh[k]; }
        dzh[ks-1] = dzh[ks+1]; dzhi[ks-1] = dzhi[ks+1];
        for (int k=1; k<kc-1; ++k) { dz[k] = zh[k+1] - zh[k]; dzi[k] = 1./dz[k]; }
        dz[ks-1] = dz[ks]; dzi[ks-1] = dzi[ks];
        dz[ke] = dz[ke-1]; dzi[ke] = dzi[ke-1];
        // Boussinesq base state, src/thermo_dry.cxx:547-559.
        for (int k=0; k<kc; ++k)
        {
            c->h[P_RHO][k] = 1.; c->h[P_RHOH][k] = 1.;
            c->h[P_TH][k] = c->phys.thref0; c->h[P_THH][k] = c->phys.thref0;
        }
        // Vertical flux-divergence factors of the flux-form tendency kernel.
        for (int k=0; k<kc; ++k)
        {
            c->h[P_ZF][k] = dzi[k]/c->h[P_RHO][k];
            c->h[P_ZFH][k] = dzhi[k]/c->h[P_RHOH][k];
        }
        // Reference profile in the scalar's storage units: the buoyancy
        // g/thref (theta - thref) becomes g/thref (theta_stored - thb).
        for (int k=0; k<kc; ++k)
        {
            c->h[P_THB][k] = c->h[P_TH][k] - c->th0;
            c->h[P_THBH][k] = c->h[P_THH][k] - c->th0;
        }
    }

    // Squared Smagorinsky mixing length per level: src/diff_smag2.cxx:176-180
    // (resolved walls), :213-265 (Mason, n = 2, with buoyancy), :108-140
    // (neutral, Mason n = 1).
    std::vector<double> mixing_length2(const mhh_ctx* c)
    {
        const Dims& d = c->d;
        const mhh_physics& p = c->phys;
        std::vector<double> m2(d.kcells, 0.);
        const double dx = c->d.dx, dy = c->d.dy;
        for (int k=d.kstart; k<d.kend; ++k)
        {
            const double mlen0 = p.cs*std::pow(dx*dy*c->h[P_DZ][k], 1./3.);
            double mlen = mlen0;
            if (p.surface && p.swmason)
            {
                const double n = p.thermo ? 2. : 1.;
                mlen = std::pow(1./(1./std::pow(mlen0, n) + 1./std::pow(KAPPA*(c->h[P_Z][k] + p.z0m), n)), 1./n);
            }
            m2[k] = mlen*mlen;
        }
        return m2;
    }

    template<typename TF>
    int upload_profiles(mhh_ctx* c)
    {
        const int kc = c->d.kcells;
        std::vector<TF> tmp(kc);
        for (int q=0; q<NPROF; ++q)
        {
            if (cudaMallocAsync(&c->dprof[q], sizeof(TF)*kc, c->setup) != cudaSuccess)
                return fail(MHH_ERR_CUDA, "cudaMallocAsync profiles");
            for (int k=0; k<kc; ++k) tmp[k] = TF(c->h[q][k]);
            cudaMemcpyAsync(c->dprof[q], tmp.data(), sizeof(TF)*kc, cudaMemcpyHostToDevice, c->setup);
            if (cudaStreamSynchronize(c->setup) != cudaSuccess) return fail(MHH_ERR_CUDA, "profiles");
        }
        Prof<TF> p;
        p.z = (const TF*)c->dprof[P_Z]; p.zh = (const TF*)c->dprof[P_ZH];
        p.dz = (const TF*)c->dprof[P_DZ]; p.dzh = (const TF*)c->dprof[P_DZH];
        p.dzi = (const TF*)c->dprof[P_DZI]; p.dzhi = (const TF*)c->dprof[P_DZHI];
        p.rhoref = (const TF*)c->dprof[P_RHO]; p.rhorefh = (const TF*)c->dprof[P_RHOH];
        p.thref = (const TF*)c->dprof[P_TH]; p.threfh = (const TF*)c->dprof[P_THH];
        p.zfac = (const TF*)c->dprof[P_ZF]; p.zfach = (const TF*)c->dprof[P_ZFH];
        p.thb = (const TF*)c->dprof[P_THB]; p.thbh = (const TF*)c->dprof[P_THBH];
        if constexpr (sizeof(TF) == 8) c->pd = *reinterpret_cast<Prof<double>*>(&p);
        else c->pf = *reinterpret_cast<Prof<float>*>(&p);
        return MHH_OK;
    }

    // The kernel choices of a call on context c.
    KernelOpts opts_of(const mhh_ctx* c)
    {
        KernelOpts o;
        o.tend = c->opt_tend != -2 ? c->opt_tend : tendency_variant();
        o.visc = c->opt_visc != -2 ? c->opt_visc : viscosity_variant();
        o.tdma = c->opt_tdma != -2 ? c->opt_tdma : tdma_variant();
        o.tend_kchunk = c->opt_tend_kchunk != -2 ? c->opt_tend_kchunk : g_tend_kchunk;
        o.visc_kchunk = c->opt_visc_kchunk != -2 ? c->opt_visc_kchunk : g_visc_kchunk;
        return o;
    }

    // Set-up allocations and copies go to the context's own stream with
    // stream-ordered allocation, so creating or destroying a context does not
    // synchronise the work of other contexts on the device.
    thread_local cudaStream_t g_setup = nullptr;

    template<typename T>
    int dalloc(T** p, size_t n, bool zero = true)
    {
        if (cudaMallocAsync((void**)p, sizeof(T)*(n ? n : 1), g_setup) != cudaSuccess)
            return fail(MHH_ERR_CUDA, "cudaMallocAsync scratch");
        if (zero) cudaMemsetAsync(*p, 0, sizeof(T)*(n ? n : 1), g_setup);
        return MHH_OK;
    }

    int upload(double* dst, const std::vector<double>& v)
    {
        cudaMemcpyAsync(dst, v.data(), sizeof(double)*v.size(), cudaMemcpyHostToDevice, g_setup);
        return cudaStreamSynchronize(g_setup) == cudaSuccess ? MHH_OK : fail(MHH_ERR_CUDA, "upload");
    }

    // Pressure-solver constants, src/pres_2.cxx:124-153.
    int setup_pres(mhh_ctx* c)
    {
        const Dims& d = c->d;
        const long long n = (long long)d.itot*d.jtot*d.ktot;
        int rc;
        if ((rc = fft_plan_init(&c->pw.px, d.itot, c->setup)) != MHH_OK) return fail(rc, "itot has a prime factor above 7");
        if ((rc = fft_plan_init(&c->pw.py, d.jtot, c->setup)) != MHH_OK) return fail(rc, "jtot has a prime factor above 7");
        const size_t tfb = c->prec == MHH_FP64 ? 8 : 4;
        if (cudaMallocAsync(&c->pw.pk, tfb*n, c->setup) != cudaSuccess) return fail(MHH_ERR_CUDA, "cudaMallocAsync pressure");
        if ((rc = dalloc(&c->pw.work, (size_t)n, false))) return rc;
        if (cudaMallocAsync(&c->pw.dcm, sizeof(double)*d.ktot, c->setup) != cudaSuccess) return fail(MHH_ERR_CUDA, "cudaMallocAsync pressure");
        if ((rc = dalloc(&c->pw.bmati, d.itot)) || (rc = dalloc(&c->pw.bmatj, d.jtot))) return rc;
        if ((rc = dalloc(&c->pw.a, d.ktot)) || (rc = dalloc(&c->pw.c, d.ktot))) return rc;
        if ((rc = dalloc(&c->pw.dz2, d.ktot)) || (rc = dalloc(&c->pw.dz2rho, d.ktot))) return rc;

        const double dxidxi = 1./(d.dx*d.dx), dyidyi = 1./(d.dy*d.dy);
        const double pi = std::acos(-1.);
        std::vector<double> bi(d.itot), bj(d.jtot), a(d.ktot), cc(d.ktot), dz2(d.ktot), dz2r(d.ktot);
        for (int j=0; j<d.jtot/2+1; ++j) bj[j] = 2.*(std::cos(2.*pi*(double)j/(double)d.jtot) - 1.)*dyidyi;
        for (int j=d.jtot/2+1; j<d.jtot; ++j) bj[j] = bj[d.jtot-j];
        for (int i=0; i<d.itot/2+1; ++i) bi[i] = 2.*(std::cos(2.*pi*(double)i/(double)d.itot) - 1.)*dxidxi;
        for (int i=d.itot/2+1; i<d.itot; ++i) bi[i] = bi[d.itot-i];
        const auto& dz = c->h[P_DZ]; const auto& dzhi = c->h[P_DZHI];
        const auto& rh = c->h[P_RHOH]; const auto& r = c->h[P_RHO];
        for (int k=0; k<d.ktot; ++k)
        {
            const int kg = k + d.kgc;
            a[k] = dz[kg]*rh[kg]*dzhi[kg];
            cc[k] = dz[kg]*rh[kg+1]*dzhi[kg+1];
            dz2[k] = dz[kg]*dz[kg];
            dz2r[k] = dz[kg]*dz[kg]*r[kg];
        }
        if ((rc = upload(c->pw.bmati, bi)) || (rc = upload(c->pw.bmatj, bj))) return rc;
        if ((rc = upload(c->pw.a, a)) || (rc = upload(c->pw.c, cc))) return rc;
        if ((rc = upload(c->pw.dz2, dz2)) || (rc = upload(c->pw.dz2rho, dz2r))) return rc;
        if ((rc = tdma_table(c->pw, d.itot, d.jtot, d.ktot, c->setup))) return fail(rc, "tridiagonal table");
        return MHH_OK;
    }

    // z/L lookup table, include/boundary_surface_kernels.h:77-130.
    double fm_host(double zsl, double z0m, double L)
    {
        auto phim_u = [](double z) { return std::pow(1. + 3.6*std::pow(std::fabs(z), 2./3.), -1./2.); };
        auto psim_u = [&](double z) { return 3.*std::log((1. + 1./phim_u(z))/2.); };
        auto psim_s = [](double z) { const double a = 1., b = 2./3., cc = 5., dd = 0.35;
                                     return -b*(z - (cc/dd))*std::exp(-dd*z) - a*z - (b*cc)/dd; };
        return L <= 0. ? KAPPA/(std::log(zsl/z0m) - psim_u(zsl/L) + psim_u(z0m/L))
                       : KAPPA/(std::log(zsl/z0m) - psim_s(zsl/L) + psim_s(z0m/L));
    }
    double fh_host(double zsl, double z0h, double L)
    {
        auto phih_u = [](double z) { return std::pow(1. + 7.9*std::pow(std::fabs(z), 2./3.), -1./2.); };
        auto psih_u = [&](double z) { return 3.*std::log((1. + 1./phih_u(z))/2.); };
        auto psih_s = [](double z) { const double a = 1., b = 2./3., cc = 5., dd = 0.35;
                                     return -b*(z - (cc/dd))*std::exp(-dd*z) - std::pow(1. + b*a*z, 1.5) - (b*cc)/dd + 1.; };
        return L <= 0. ? KAPPA/(std::log(zsl/z0h) - psih_u(zsl/L) + psih_u(z0h/L))
                       : KAPPA/(std::log(zsl/z0h) - psih_s(zsl/L) + psih_s(z0h/L));
    }

    void prepare_lut(std::vector<float>& zL, std::vector<float>& f, double zsl, double z0m, double z0h, int thermo_bc)
    {
        const int N = NZL_LUT;
        std::vector<double> zt(N);
        const double zLrange_min = -5., zL_max = 10., zL_min = -1.e4;
        double dzL = (zL_max - zLrange_min) / (9.*N/10. - 1.);
        zt[0] = -zL_max;
        for (int n=1; n<9*N/10; ++n) zt[n] = zt[n-1] + dzL;
        const double zLend = -(zL_min - zLrange_min);
        double r = 1.01, r0 = 1.e30;
        while (std::fabs((r - r0)/r0) > 1.e-10)
        {
            r0 = r;
            r = std::pow(1. - (zLend/dzL)*(1. - r), (1./(N/10.)));
        }
        for (int n=9*N/10; n<N; ++n) { zt[n] = zt[n-1] + dzL; dzL *= r; }
        zL.resize(N); f.resize(N);
        for (int n=0; n<N; ++n) zL[n] = (float)(-zt[N-n-1]);
        for (int n=0; n<N; ++n)
        {
            const double L = zsl/(double)zL[n];
            if (thermo_bc == MHH_BC_DIRICHLET)
                f[n] = (float)((double)zL[n]*std::pow(fm_host(zsl, z0m, L), 2)/fh_host(zsl, z0h, L));
            else
                f[n] = (float)((double)zL[n]*std::pow(fm_host(zsl, z0m, L), 3));
        }
    }

    int reduce_to_host(mhh_ctx* c, cudaStream_t s, double* out)
    {
        cudaMemcpyAsync(c->red_host, c->red, sizeof(unsigned long long), cudaMemcpyDeviceToHost, s);
        if (cudaStreamSynchronize(s) != cudaSuccess) return fail(MHH_ERR_CUDA, cudaGetErrorString(cudaGetLastError()));
        long long bits = (long long)*c->red_host;
        double v;
        std::memcpy(&v, &bits, sizeof(double));
        *out = v;
        if (!std::isfinite(v)) return fail(MHH_ERR_NONFINITE, "reduction is not finite");
        return MHH_OK;
    }

    template<typename TF> TF* T(void* p) { return static_cast<TF*>(p); }
    template<typename TF> const TF* CT(const void* p) { return static_cast<const TF*>(p); }

    template<typename TF>
    TendArgs<TF> tend_args(const mhh_ctx* c, const mhh_fields* f, const mhh_bcfields* bc)
    {
        TendArgs<TF> a{};
        a.u = CT<TF>(f->u); a.v = CT<TF>(f->v); a.w = CT<TF>(f->w); a.s = CT<TF>(f->s);
        a.evisc = CT<TF>(f->evisc);
        a.ut = T<TF>(f->ut); a.vt = T<TF>(f->vt); a.wt = T<TF>(f->wt); a.st = T<TF>(f->st);
        if (bc)
        {
            a.u_fluxbot = CT<TF>(bc->u_fluxbot); a.u_fluxtop = CT<TF>(bc->u_fluxtop);
            a.v_fluxbot = CT<TF>(bc->v_fluxbot); a.v_fluxtop = CT<TF>(bc->v_fluxtop);
            a.s_fluxbot = CT<TF>(bc->s_fluxbot); a.s_fluxtop = CT<TF>(bc->s_fluxtop);
        }
        a.visc = TF(c->phys.visc); a.svisc = TF(c->phys.svisc);
        a.tpri = TF(1)/TF(c->phys.tpr);
        a.dxidxi_t = TF(1./(c->d.dx*c->d.dx));
        a.dyidyi_t = TF(1./(c->d.dy*c->d.dy));
        a.fbody = TF(0);
        a.dxidxi = 1./(c->d.dx*c->d.dx);
        a.dyidyi = 1./(c->d.dy*c->d.dy);
        return a;
    }

    // ---------------------------------------------------------------------
    // Templated bodies
    // ---------------------------------------------------------------------
    template<typename TF>
    int pres_exec(mhh_ctx* c, const mhh_fields* f, double sub_dt, bool with_out, cudaStream_t s)
    {
        const Dims& d = c->d;
        const Prof<TF>& pr = prof<TF>(c);
        FieldList<TF> fl;
        TF* pk = T<TF>(c->pw.pk);
        if (pres_fuse() && d.itot > 1)
        {
            // The right-hand side is computed inside the forward x transform
            // and the inverse x transform stores into the ghost layout of p:
            // two field passes fewer each way.
            {
                Timed t("pres_in", s);
                fl.n = 1; fl.p[0] = T<TF>(f->ut); launch_cyclic(fl, d, MHH_EDGE_EW, s);
                fl.p[0] = T<TF>(f->vt); launch_cyclic(fl, d, MHH_EDGE_NS, s);
            }
            FftFuse<TF> fz;
            std::memset(&fz, 0, sizeof(fz));
            fz.d = d; fz.pr = pr;
            fz.u = CT<TF>(f->u); fz.v = CT<TF>(f->v); fz.w = CT<TF>(f->w);
            fz.ut = CT<TF>(f->ut); fz.vt = CT<TF>(f->vt); fz.wt = CT<TF>(f->wt);
            fz.dti = TF(1./sub_dt);
            fz.p = T<TF>(f->p);
            fz.dcm = static_cast<const TF*>(c->pw.dcm);
            fz.mode = 1;
            { Timed t("fft_x", s); launch_fft_x<TF>(c->pw.px, pk, d.jtot*d.ktot, false, 1., s, &fz); }
            { Timed t("fft_y", s); launch_fft_y<TF>(c->pw.py, pk, d.itot, d.jtot, d.ktot, false, 1., s); }
            { Timed t("tdma", s); launch_tdma<TF>(d, c->pw, pk, opts_of(c), s); }
            { Timed t("fft_y", s); launch_fft_y<TF>(c->pw.py, pk, d.itot, d.jtot, d.ktot, true, 1./d.jtot, s); }
            fz.mode = 2;
            { Timed t("fft_x", s); launch_fft_x<TF>(c->pw.px, pk, d.jtot*d.ktot, true, 1./d.itot, s, &fz); }
            {
                Timed t("pres_scatter", s);
                fl.p[0] = T<TF>(f->p); launch_cyclic(fl, d, MHH_EDGE_BOTH, s);
            }
        }
        else
        {
        {
            Timed t("pres_in", s);
            fl.n = 1; fl.p[0] = T<TF>(f->ut); launch_cyclic(fl, d, MHH_EDGE_EW, s);
            fl.p[0] = T<TF>(f->vt); launch_cyclic(fl, d, MHH_EDGE_NS, s);
            launch_pres_in<TF>(d, pr, CT<TF>(f->u), CT<TF>(f->v), CT<TF>(f->w), CT<TF>(f->ut), CT<TF>(f->vt), CT<TF>(f->wt),
                               pk, 1./sub_dt, s);
        }
        { Timed t("fft_x", s); launch_fft_x<TF>(c->pw.px, pk, d.jtot*d.ktot, false, 1., s); }
        { Timed t("fft_y", s); launch_fft_y<TF>(c->pw.py, pk, d.itot, d.jtot, d.ktot, false, 1., s); }
        { Timed t("tdma", s); launch_tdma<TF>(d, c->pw, pk, opts_of(c), s); }
        { Timed t("fft_y", s); launch_fft_y<TF>(c->pw.py, pk, d.itot, d.jtot, d.ktot, true, 1./d.jtot, s); }
        { Timed t("fft_x", s); launch_fft_x<TF>(c->pw.px, pk, d.jtot*d.ktot, true, 1./d.itot, s); }
        {
            Timed t("pres_scatter", s);
            launch_pres_scatter<TF>(d, pk, static_cast<const TF*>(c->pw.dcm), T<TF>(f->p), s);
            fl.p[0] = T<TF>(f->p); launch_cyclic(fl, d, MHH_EDGE_BOTH, s);
        }
        }
        if (with_out)
        {
            dim3 block(32, 8), grid((d.itot + 31)/32, (d.jtot + 7)/8, d.ktot);
            k_pres_out<TF><<<grid, block, 0, s>>>(d, pr, CT<TF>(f->p), T<TF>(f->ut), T<TF>(f->vt), T<TF>(f->wt));
            count_launch();
        }
        return check_cuda("pres_2");
    }

    template<typename TF>
    int viscosity(mhh_ctx* c, const mhh_fields* f, cudaStream_t s)
    {
        if (!f->evisc) return fail(MHH_ERR_ARG, "evisc is NULL");
        const bool surf = c->phys.surface != 0, thermo = c->phys.thermo != 0 && f->s;
        if (surf && !c->surf_ready) return fail(MHH_ERR_ARG, "surface layer not initialised");
        Timed t("viscosity", s);
        const TF* ml2 = sizeof(TF) == 8 ? reinterpret_cast<const TF*>(c->sw.mlen2) : reinterpret_cast<const TF*>(c->sw.mlen2f);
        launch_viscosity<TF>(c->d, prof<TF>(c), CT<TF>(f->u), CT<TF>(f->v), CT<TF>(f->w), CT<TF>(f->s), T<TF>(f->evisc),
                             ml2, c->sw.dudz, c->sw.dvdz, c->sw.dbdz, c->phys.cs, c->phys.tpr, c->phys.visc,
                             c->phys.swmason, surf, thermo, opts_of(c), s);
        return check_cuda("viscosity");
    }

    template<typename TF>
    int surface_exec(mhh_ctx* c, const mhh_fields* f, const mhh_bcfields* bc, int thermo_bc, cudaStream_t s)
    {
        if (!c->surf_ready) return fail(MHH_ERR_ARG, "surface layer not initialised");
        const int thermo = (c->phys.thermo && f->s) ? 1 : 0;
        Timed t("surface", s);
        launch_surface<TF>(c->d, prof<TF>(c), c->sw, CT<TF>(f->u), CT<TF>(f->v), CT<TF>(f->s),
                           T<TF>(bc->u_bot), T<TF>(bc->v_bot), T<TF>(bc->u_fluxbot), T<TF>(bc->v_fluxbot),
                           T<TF>(bc->u_gradbot), T<TF>(bc->v_gradbot),
                           T<TF>(bc->s_bot), T<TF>(bc->s_fluxbot), T<TF>(bc->s_gradbot),
                           thermo, thermo_bc, c->phys.z0m, c->phys.z0h, s);
        return check_cuda("surface");
    }

    template<typename TF>
    void ghost_all(mhh_ctx* c, const mhh_substep_config* cfg, const mhh_fields* f, const mhh_bcfields* bc,
                   bool momentum, cudaStream_t s)
    {
        GhostList<TF> gl{};
        auto add = [&](void* a, int bt, void* abot, void* agb, int tt, void* atop, void* agt)
        {
            const int q = gl.n++;
            gl.a[q] = T<TF>(a); gl.bot_type[q] = bt; gl.top_type[q] = tt;
            gl.abot[q] = CT<TF>(abot); gl.agradbot[q] = CT<TF>(agb);
            gl.atop[q] = CT<TF>(atop); gl.agradtop[q] = CT<TF>(agt);
        };
        if (momentum)
        {
            add(f->u, cfg->mbcbot, bc->u_bot, bc->u_gradbot, cfg->mbctop, bc->u_top, bc->u_gradtop);
            add(f->v, cfg->mbcbot, bc->v_bot, bc->v_gradbot, cfg->mbctop, bc->v_top, bc->v_gradtop);
        }
        if (f->s)
            add(f->s, cfg->sbcbot, bc->s_bot, bc->s_gradbot, cfg->sbctop, bc->s_top, bc->s_gradtop);
        if (gl.n) launch_ghost<TF>(gl, c->d, prof<TF>(c).dzh, s);
    }

    template<typename TF>
    int substep_begin(mhh_ctx* c, const mhh_substep_config* cfg, const mhh_fields* f, const mhh_bcfields* bc, cudaStream_t s)
    {
        {
            Timed t("boundaries", s);
            FieldList<TF> fl{};
            fl.p[fl.n++] = T<TF>(f->u); fl.p[fl.n++] = T<TF>(f->v); fl.p[fl.n++] = T<TF>(f->w);
            if (f->s) fl.p[fl.n++] = T<TF>(f->s);
            launch_cyclic(fl, c->d, MHH_EDGE_BOTH, s);
            ghost_all<TF>(c, cfg, f, bc, true, s);
        }
        if (cfg->diff == MHH_DIFF_SMAG2)
            return viscosity<TF>(c, f, s);
        return check_cuda("substep_begin");
    }

    template<typename TF>
    int substep_end(mhh_ctx* c, const mhh_substep_config* cfg, const mhh_fields* f, const mhh_bcfields* bc,
                    int substep, double dt, cudaStream_t s)
    {
        const Dims& d = c->d;
        const Prof<TF>& pr = prof<TF>(c);
        const bool surf = c->phys.surface != 0;
        if (surf)
        {
            int rc = surface_exec<TF>(c, f, bc, cfg->sbcbot, s);
            if (rc) return rc;
            Timed t("boundaries", s);
            ghost_all<TF>(c, cfg, f, bc, false, s);
        }
        TendArgs<TF> a = tend_args<TF>(c, f, bc);
        const bool force = cfg->swlspres != 0;
        a.fbody = TF(-1.*cfg->dpdx);
        const bool scal = f->s != nullptr;
        const bool buoy = scal && c->phys.thermo;
        {
            Timed t("tendency", s);
            const int adv = cfg->advec == MHH_ADVEC_2I5 && c->fluxlimit_s ? ADVEC_2I5_LIM : cfg->advec;
            launch_tendency<TF>(d, pr, a, adv, cfg->diff, surf, scal, buoy, force, opts_of(c), s);
            if (c->buf_on)
                launch_buffer<TF>(d, (const TF*)c->bufprof, c->buf_kb, CT<TF>(f->u), CT<TF>(f->v), CT<TF>(f->w),
                                  CT<TF>(f->s), T<TF>(f->ut), T<TF>(f->vt), T<TF>(f->wt), T<TF>(f->st), s);
        }
        const double cB[3] = {1./3., 15./16., 8./15.};
        int rc = pres_exec<TF>(c, f, cB[substep]*dt, false, s);
        if (rc) return rc;
        {
            Timed t("presout_rk3", s);
            launch_presout_rk3<TF>(d, pr, CT<TF>(f->p), T<TF>(f->u), T<TF>(f->v), T<TF>(f->w), T<TF>(f->s),
                                   T<TF>(f->ut), T<TF>(f->vt), T<TF>(f->wt), T<TF>(f->st), substep, dt, s);
        }
        return check_cuda("substep_end");
    }
}

#define DISPATCH(c, call) ((c)->prec == MHH_FP64 ? call<double> : call<float>)

extern "C" {

const char* mhh_last_error(void) { return g_last_error.c_str(); }

int mhh_set_option(const char* name, int value)
{
    if (!name) return fail(MHH_ERR_ARG, "NULL option");
    if (!std::strcmp(name, "tendency_kernel"))
    {
        if (value < -1 || value > 2) return fail(MHH_ERR_ARG, "tendency_kernel is -1, 0, 1 or 2");
        set_tendency_variant(value);
        return MHH_OK;
    }
    if (!std::strcmp(name, "viscosity_kernel"))
    {
        if (value < -1 || value > 1) return fail(MHH_ERR_ARG, "viscosity_kernel is -1, 0 or 1");
        set_viscosity_variant(value);
        return MHH_OK;
    }
    if (!std::strcmp(name, "tdma_kernel"))
    {
        if (value < -1 || value > 3) return fail(MHH_ERR_ARG, "tdma_kernel is -1, 0, 1, 2 or 3");
        set_tdma_variant(value);
        return MHH_OK;
    }
    if (!std::strcmp(name, "pres_fuse"))
    {
        if (value != 0 && value != 1) return fail(MHH_ERR_ARG, "pres_fuse is 0 or 1");
        g_pres_fuse = value;
        return MHH_OK;
    }
    if (!std::strcmp(name, "fft_pipeline"))
    {
        if (value != 0 && value != 1) return fail(MHH_ERR_ARG, "fft_pipeline is 0 or 1");
        g_fft_pipeline = value;
        return MHH_OK;
    }
    if (!std::strcmp(name, "fft_column_pairs"))
    {
        if (value != 4 && value != 8) return fail(MHH_ERR_ARG, "fft_column_pairs is 4 or 8");
        set_fft_column_pairs(value);
        return MHH_OK;
    }
    if (!std::strcmp(name, "tendency_kchunk") || !std::strcmp(name, "viscosity_kchunk"))
    {
        if (value != 0 && value != 4 && value != 8 && value != 16 && value != 32 && value != 64)
            return fail(MHH_ERR_ARG, "kchunk is 0 (default), 4, 8, 16, 32 or 64");
        (name[0] == 't' ? g_tend_kchunk : g_visc_kchunk) = value;
        return MHH_OK;
    }
    return fail(MHH_ERR_ARG, "unknown option");
}

int mhh_ctx_set_option(mhh_ctx* c, const char* name, int value)
{
    if (!c || !name) return fail(MHH_ERR_ARG, "NULL argument");
    const bool reset = value == -2;
    if (!std::strcmp(name, "tendency_kernel"))
    {
        if (!reset && (value < -1 || value > 2)) return fail(MHH_ERR_ARG, "tendency_kernel is -2, -1, 0, 1 or 2");
        c->opt_tend = value;
    }
    else if (!std::strcmp(name, "viscosity_kernel"))
    {
        if (!reset && (value < -1 || value > 1)) return fail(MHH_ERR_ARG, "viscosity_kernel is -2, -1, 0 or 1");
        c->opt_visc = value;
    }
    else if (!std::strcmp(name, "tdma_kernel"))
    {
        if (!reset && (value < -1 || value > 3)) return fail(MHH_ERR_ARG, "tdma_kernel is -2, -1, 0, 1, 2 or 3");
        c->opt_tdma = value;
    }
    else if (!std::strcmp(name, "tendency_kchunk") || !std::strcmp(name, "viscosity_kchunk"))
    {
        if (!reset && value != 0 && value != 4 && value != 8 && value != 16 && value != 32 && value != 64)
            return fail(MHH_ERR_ARG, "kchunk is -2, 0 (default), 4, 8, 16, 32 or 64");
        (name[0] == 't' ? c->opt_tend_kchunk : c->opt_visc_kchunk) = value;
    }
    else
        return fail(MHH_ERR_ARG, "unknown option");
    return MHH_OK;
}

int mhh_launch_count_add(long long n)
{
    mhh::count_launch((int)n);
    return MHH_OK;
}

int mhh_timing_enable(int on)
{
    g_timing = on != 0;
    return MHH_OK;
}

int mhh_timing_reset(void)
{
    for (auto& p : g_pending) { g_event_pool.push_back(p.a); g_event_pool.push_back(p.b); }
    g_pending.clear();
    g_timers.clear();
    return MHH_OK;
}

int mhh_timing_collect(void)
{
    for (auto& p : g_pending)
    {
        if (cudaEventSynchronize(p.b) != cudaSuccess) return fail(MHH_ERR_CUDA, "timing event");
        float ms = 0.f;
        cudaEventElapsedTime(&ms, p.a, p.b);
        g_timers[p.idx].ms += ms;
        g_timers[p.idx].count += 1;
        g_event_pool.push_back(p.a); g_event_pool.push_back(p.b);
    }
    g_pending.clear();
    return MHH_OK;
}

int mhh_timing_count(void) { return (int)g_timers.size(); }

int mhh_timing_get(int idx, const char** name, long long* count, double* total_ms)
{
    if (idx < 0 || idx >= (int)g_timers.size() || !name || !count || !total_ms) return fail(MHH_ERR_ARG, "bad timer index");
    *name = g_timers[idx].name.c_str();
    *count = g_timers[idx].count;
    *total_ms = g_timers[idx].ms;
    return MHH_OK;
}
long long mhh_launch_count(void) { return mhh::launch_count(); }

int mhh_ctx_create(const mhh_grid_desc* desc, const double* z, int precision, const mhh_physics* phys, mhh_ctx** out)
{
    if (!desc || !z || !phys || !out) return fail(MHH_ERR_ARG, "NULL argument");
    if (precision != MHH_FP64 && precision != MHH_FP32) return fail(MHH_ERR_ARG, "precision must be 64 or 32");
    if (desc->itot < 1 || desc->jtot < 1 || desc->ktot < 1 || desc->igc < 1 || desc->jgc < 1 || desc->kgc < 1 || desc->kgc > 2)
        return fail(MHH_ERR_ARG, "bad grid sizes or ghost cells (kgc must be 1 or 2)");
    if (desc->igc > desc->itot || desc->jgc > desc->jtot)
        return fail(MHH_ERR_ARG, "more ghost cells than interior cells");
    if ((desc->igc >= 3 || desc->jgc >= 3) && desc->ktot < 6)
        return fail(MHH_ERR_ARG, "the 5th-order scheme needs ktot >= 6");
    const double ncells = double(desc->itot + 2*desc->igc)*(desc->jtot + 2*desc->jgc)*(desc->ktot + 2);
    if (ncells > 4.0e9) return fail(MHH_ERR_ARG, "grid too large for 32-bit plane indexing");
    if (double(desc->itot + 2*desc->igc)*(desc->jtot + 2*desc->jgc) > 2.0e9)
        return fail(MHH_ERR_ARG, "horizontal plane too large for 32-bit indexing");

    size_t free0 = 0, total0 = 0;
    cudaMemGetInfo(&free0, &total0);
    mhh_ctx* c = new mhh_ctx();
    c->statbuf = nullptr;
    c->bufprof = nullptr;
    c->buf_on = 0;
    c->buf_kb = 0;
    c->buf_set = 0;
    c->fluxlimit_s = 0;
    c->opt_tend = c->opt_visc = c->opt_tdma = c->opt_tend_kchunk = c->opt_visc_kchunk = -2;
    c->dev_bytes = 0;
    if (cudaStreamCreateWithFlags(&c->setup, cudaStreamNonBlocking) != cudaSuccess)
    {
        delete c;
        return fail(MHH_ERR_CUDA, "cudaStreamCreate");
    }
    g_setup = c->setup;
    std::memset(c->dprof, 0, sizeof(c->dprof));
    std::memset(&c->pw, 0, sizeof(c->pw));
    std::memset(&c->sw, 0, sizeof(c->sw));
    c->prec = precision;
    c->phys = *phys;
    // Theta near 300 K keeps about 3e-5 K in float; stored as its difference
    // from the Boussinesq reference it keeps 1e-8 K in the boundary layer.
    // The buoyancy of the dry thermodynamics only needs theta - thref, so
    // the kernels see the offset through the thb profiles alone.
    c->th0 = (precision == MHH_FP32 && phys->thermo) ? phys->thref0 : 0.;
    Dims& d = c->d;
    d.itot = desc->itot; d.jtot = desc->jtot; d.ktot = desc->ktot;
    d.igc = desc->igc; d.jgc = desc->jgc; d.kgc = desc->kgc;
    d.icells = d.itot + 2*d.igc; d.jcells = d.jtot + 2*d.jgc; d.kcells = d.ktot + 2*d.kgc;
    d.ijcells = d.icells*d.jcells;
    d.ncells = (long long)d.ijcells*d.kcells;
    d.istart = d.igc; d.iend = d.itot + d.igc;
    d.jstart = d.jgc; d.jend = d.jtot + d.jgc;
    d.kstart = d.kgc; d.kend = d.ktot + d.kgc;
    d.dx = desc->xsize / d.itot; d.dy = desc->ysize / d.jtot;
    d.dxi = 1./d.dx; d.dyi = 1./d.dy;
    d.fdxi = float(d.dxi); d.fdyi = float(d.dyi); d.fzsize = float(desc->zsize);
    d.zsize = desc->zsize;

    mhh_grid& g = c->g;
    g.itot = d.itot; g.jtot = d.jtot; g.ktot = d.ktot; g.igc = d.igc; g.jgc = d.jgc; g.kgc = d.kgc;
    g.icells = d.icells; g.jcells = d.jcells; g.kcells = d.kcells; g.ijcells = d.ijcells;
    g.istart = d.istart; g.iend = d.iend; g.jstart = d.jstart; g.jend = d.jend; g.kstart = d.kstart; g.kend = d.kend;
    g.ncells = d.ncells; g.dx = d.dx; g.dy = d.dy; g.zsize = d.zsize; g.precision = precision;

    grid_metrics(c, z);
    int rc = precision == MHH_FP64 ? upload_profiles<double>(c) : upload_profiles<float>(c);
    if (!rc) rc = setup_pres(c);
    if (!rc) rc = dalloc(&c->red, 1);
    if (!rc) rc = dalloc(&c->statbuf, 2*(size_t)d.kcells);
    if (!rc && cudaMallocHost((void**)&c->red_host, sizeof(unsigned long long)) != cudaSuccess)
        rc = fail(MHH_ERR_CUDA, "cudaMallocHost");
    // Surface and viscosity arrays (always allocated; small).
    if (!rc) rc = dalloc(&c->sw.ustar, d.ijcells);
    if (!rc) rc = dalloc(&c->sw.obuk, d.ijcells);
    if (!rc) rc = dalloc(&c->sw.dudz, d.ijcells);
    if (!rc) rc = dalloc(&c->sw.dvdz, d.ijcells);
    if (!rc) rc = dalloc(&c->sw.dbdz, d.ijcells);
    if (!rc) rc = dalloc(&c->sw.dutot, d.ijcells);
    if (!rc) rc = dalloc(&c->sw.fm, d.ijcells);
    if (!rc) rc = dalloc(&c->sw.fh, d.ijcells);
    if (!rc) rc = dalloc(&c->sw.phim, d.ijcells);
    if (!rc) rc = dalloc(&c->sw.phih, d.ijcells);
    c->sw.z0h = phys->z0h;
    if (!rc) rc = dalloc(&c->sw.nobuk, d.ijcells);
    if (!rc) rc = dalloc(&c->sw.zL, NZL_LUT);
    if (!rc) rc = dalloc(&c->sw.f, NZL_LUT);
    if (!rc) rc = dalloc(&c->sw.mlen2, d.kcells);
    if (!rc) rc = upload(c->sw.mlen2, mixing_length2(c));
    if (!rc)
    {
        const std::vector<double> m2 = mixing_length2(c);
        std::vector<float> m2f(m2.begin(), m2.end());
        rc = dalloc(&c->sw.mlen2f, m2f.size());
        if (!rc)
        {
            cudaMemcpyAsync(c->sw.mlen2f, m2f.data(), sizeof(float)*m2f.size(), cudaMemcpyHostToDevice, c->setup);
            if (cudaStreamSynchronize(c->setup) != cudaSuccess) rc = fail(MHH_ERR_CUDA, "mixing length");
        }
    }
    c->sw.zsl = c->h[P_Z][d.kstart];
    c->sw.thref_s = c->h[P_TH][d.kstart];
    c->sw.threfh_s = c->h[P_THH][d.kstart];
    c->sw.thb_s = c->h[P_THB][d.kstart];
    c->sw.thbh_s = c->h[P_THBH][d.kstart];
    // Diff_2 multiplier, src/diff_2.cxx:143-155.
    {
        const double viscmax = phys->thermo ? std::max(phys->visc, phys->svisc) : phys->visc;
        double dn = 0.;
        for (int k=d.kstart; k<d.kend; ++k)
        {
            const double dzk = c->h[P_DZ][k];
            dn = std::max(dn, std::fabs(viscmax*(1./(d.dx*d.dx) + 1./(d.dy*d.dy) + 1./(dzk*dzk))));
        }
        c->dnmul2 = dn;
    }
    g_setup = nullptr;
    if (rc) { mhh_ctx_destroy(c); return rc; }
    if (cudaStreamSynchronize(c->setup) != cudaSuccess) { mhh_ctx_destroy(c); return fail(MHH_ERR_CUDA, "set-up failed"); }
    size_t free1 = 0, total1 = 0;
    cudaMemGetInfo(&free1, &total1);
    c->dev_bytes = free0 > free1 ? free0 - free1 : 0;
    *out = c;
    return MHH_OK;
}

int mhh_ctx_device_bytes(const mhh_ctx* c, size_t* bytes)
{
    if (!c || !bytes) return fail(MHH_ERR_ARG, "NULL argument");
    *bytes = c->dev_bytes;
    return MHH_OK;
}

int mhh_ctx_estimate_bytes(const mhh_grid_desc* g, int precision, size_t* bytes)
{
    if (!g || !bytes) return fail(MHH_ERR_ARG, "NULL argument");
    if (precision != MHH_FP64 && precision != MHH_FP32) return fail(MHH_ERR_ARG, "precision must be 64 or 32");
    const double tf = precision == MHH_FP64 ? 8. : 4.;
    const double icells = g->itot + 2*g->igc, jcells = g->jtot + 2*g->jgc, kcells = g->ktot + 2*g->kgc;
    const double ij = icells*jcells;
    const double n = double(g->itot)*g->jtot*g->ktot;
    const double groups = double(g->itot/2 + 1)*(g->jtot/2 + 1)*g->ktot;
    double b = 0.;
    b += 14.*kcells*tf;                         // profiles
    b += n*tf + n*8. + g->ktot*8.;              // packed pressure + work + level means
    b += groups*(8. + 8. + 8. + 8. + 4. + 8.); // elimination tables
    b += 2.*(g->itot + g->jtot)*(16. + 8.);    // twiddles
    b += 12.*ij*8. + ij*4. + 2.*10000*4.;      // surface layer
    b += 2.*kcells*8.;                          // mixing length
    // cudaMalloc granularity: about 40 allocations of up to 2 MiB each.
    b += 40.*2.*1024*1024;
    *bytes = (size_t)b;
    return MHH_OK;
}

int mhh_ctx_destroy(mhh_ctx* c)
{
    if (!c) return MHH_OK;
    // Stream-ordered release: the memory returns to the pool once the set-up
    // stream reaches it; the caller has finished its own work on the fields.
    for (auto& p : c->dprof) if (p) cudaFreeAsync(p, c->setup);
    fft_plan_free(&c->pw.px, c->setup); fft_plan_free(&c->pw.py, c->setup);
    void* ptrs[] = {c->pw.pk, c->pw.work, c->pw.dcm, c->pw.rtab, c->pw.wtab, c->pw.gtab, c->pw.htab, c->pw.stab, c->pw.stabd, c->pw.gftab, c->pw.hftab, c->pw.fmode, c->pw.bmati, c->pw.bmatj, c->pw.a, c->pw.c, c->pw.dz2, c->pw.dz2rho,
                    c->red, c->statbuf, c->bufprof, c->sw.fm, c->sw.fh, c->sw.phim, c->sw.phih, c->sw.ustar, c->sw.obuk, c->sw.dudz, c->sw.dvdz, c->sw.dbdz, c->sw.dutot,
                    c->sw.nobuk, c->sw.zL, c->sw.f, c->sw.mlen2, c->sw.mlen2f};
    for (void* p : ptrs) if (p) cudaFreeAsync(p, c->setup);
    if (c->red_host) cudaFreeHost(c->red_host);
    cudaStreamSynchronize(c->setup);
    cudaStreamDestroy(c->setup);
    delete c;
    return MHH_OK;
}

int mhh_ctx_get_grid(const mhh_ctx* c, mhh_grid* out)
{
    if (!c || !out) return fail(MHH_ERR_ARG, "NULL argument");
    *out = c->g;
    return MHH_OK;
}

int mhh_ctx_get_profile(const mhh_ctx* c, const char* name, double* out)
{
    if (!c || !name || !out) return fail(MHH_ERR_ARG, "NULL argument");
    for (int q=0; q<10; ++q)
        if (!std::strcmp(name, prof_names[q]))
        {
            std::memcpy(out, c->h[q].data(), sizeof(double)*c->h[q].size());
            return MHH_OK;
        }
    return fail(MHH_ERR_ARG, "unknown profile");
}

int mhh_ctx_scalar_offset(const mhh_ctx* c, double* offset)
{
    if (!c || !offset) return fail(MHH_ERR_ARG, "NULL argument");
    *offset = c->th0;
    return MHH_OK;
}

int mhh_field_shift(mhh_ctx* c, void* field, double delta, cudaStream_t s)
{
    if (!c || !field) return fail(MHH_ERR_ARG, "NULL argument");
    const long long n = c->d.ncells;
    const unsigned nb = (unsigned)std::min<long long>((n + 255)/256, 8LL*152);
    if (c->prec == MHH_FP64) k_shift<double><<<nb, 256, 0, s>>>((double*)field, n, delta);
    else k_shift<float><<<nb, 256, 0, s>>>((float*)field, n, float(delta));
    count_launch();
    return check_cuda("field_shift");
}

int mhh_boundary_cyclic(mhh_ctx* c, void* data, int edges, cudaStream_t s)
{
    if (!c || !data || edges < 1 || edges > 3) return fail(MHH_ERR_ARG, "bad argument");
    if (c->prec == MHH_FP64) { FieldList<double> fl{}; fl.n = 1; fl.p[0] = (double*)data; launch_cyclic(fl, c->d, edges, s); }
    else { FieldList<float> fl{}; fl.n = 1; fl.p[0] = (float*)data; launch_cyclic(fl, c->d, edges, s); }
    return check_cuda("cyclic");
}

int mhh_boundary_set_bc(mhh_ctx* c, void* val, void* grad, void* flux, int type, double aval, double visc,
                        int sfg, cudaStream_t s)
{
    if (!c || !val || !grad || !flux || type < 0 || type > 2) return fail(MHH_ERR_ARG, "bad argument");
    if (c->prec == MHH_FP64) launch_set_bc<double>((double*)val, (double*)grad, (double*)flux, type, aval, visc, sfg, c->d, s);
    else launch_set_bc<float>((float*)val, (float*)grad, (float*)flux, type, aval, visc, sfg, c->d, s);
    return check_cuda("set_bc");
}

int mhh_boundary_ghost_cells(mhh_ctx* c, void* a, int bt, const void* abot, const void* agb,
                             int tt, const void* atop, const void* agt, cudaStream_t s)
{
    if (!c || !a || !abot || !agb || !atop || !agt) return fail(MHH_ERR_ARG, "NULL argument");
    if (c->prec == MHH_FP64)
    {
        GhostList<double> gl{}; gl.n = 1; gl.a[0] = (double*)a; gl.bot_type[0] = bt; gl.top_type[0] = tt;
        gl.abot[0] = (const double*)abot; gl.agradbot[0] = (const double*)agb;
        gl.atop[0] = (const double*)atop; gl.agradtop[0] = (const double*)agt;
        launch_ghost<double>(gl, c->d, c->pd.dzh, s);
    }
    else
    {
        GhostList<float> gl{}; gl.n = 1; gl.a[0] = (float*)a; gl.bot_type[0] = bt; gl.top_type[0] = tt;
        gl.abot[0] = (const float*)abot; gl.agradbot[0] = (const float*)agb;
        gl.atop[0] = (const float*)atop; gl.agradtop[0] = (const float*)agt;
        launch_ghost<float>(gl, c->d, c->pf.dzh, s);
    }
    return check_cuda("ghost_cells");
}

int mhh_boundary_surface_init(mhh_ctx* c, int thermo_bc)
{
    if (!c) return fail(MHH_ERR_ARG, "NULL argument");
    if (thermo_bc != MHH_BC_FLUX && thermo_bc != MHH_BC_DIRICHLET)
        return fail(MHH_ERR_ARG, "surface model needs a flux or Dirichlet scalar BC");
    std::vector<float> zL, f;
    prepare_lut(zL, f, c->sw.zsl, c->phys.z0m, c->phys.z0h, thermo_bc);
    cudaStream_t s = c->setup;
    cudaMemcpyAsync(c->sw.zL, zL.data(), sizeof(float)*zL.size(), cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(c->sw.f, f.data(), sizeof(float)*f.size(), cudaMemcpyHostToDevice, s);
    const int n = c->d.ijcells;
    std::vector<double> obuk(n, DSMALL), ustar(n, 1e-2);
    cudaMemcpyAsync(c->sw.obuk, obuk.data(), sizeof(double)*n, cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(c->sw.ustar, ustar.data(), sizeof(double)*n, cudaMemcpyHostToDevice, s);
    cudaMemsetAsync(c->sw.nobuk, 0, sizeof(int)*n, s);
    cudaMemsetAsync(c->sw.dudz, 0, sizeof(double)*n, s);
    cudaMemsetAsync(c->sw.dvdz, 0, sizeof(double)*n, s);
    cudaMemsetAsync(c->sw.dbdz, 0, sizeof(double)*n, s);
    if (cudaStreamSynchronize(s) != cudaSuccess) return fail(MHH_ERR_CUDA, "surface_init");
    c->surf_ready = 1;
    return check_cuda("surface_init");
}

int mhh_boundary_surface_exec(mhh_ctx* c, const mhh_fields* f, const mhh_bcfields* bc, int thermo_bc, cudaStream_t s)
{
    if (!c || !f || !bc) return fail(MHH_ERR_ARG, "NULL argument");
    return c->prec == MHH_FP64 ? surface_exec<double>(c, f, bc, thermo_bc, s) : surface_exec<float>(c, f, bc, thermo_bc, s);
}

int mhh_boundary_surface_set(mhh_ctx* c, const char* name, const double* in)
{
    if (!c || !name || !in) return fail(MHH_ERR_ARG, "NULL argument");
    double* dst = nullptr;
    if (!std::strcmp(name, "dudz")) dst = c->sw.dudz;
    else if (!std::strcmp(name, "dvdz")) dst = c->sw.dvdz;
    else if (!std::strcmp(name, "dbdz")) dst = c->sw.dbdz;
    else if (!std::strcmp(name, "obuk")) dst = c->sw.obuk;
    else if (!std::strcmp(name, "ustar")) dst = c->sw.ustar;
    if (!dst) return fail(MHH_ERR_ARG, "unknown surface array");
    if (cudaMemcpy(dst, in, sizeof(double)*c->d.ijcells, cudaMemcpyHostToDevice) != cudaSuccess)
        return fail(MHH_ERR_CUDA, "cudaMemcpy");
    return MHH_OK;
}

int mhh_boundary_surface_get(mhh_ctx* c, const char* name, double* out)
{
    if (!c || !name || !out) return fail(MHH_ERR_ARG, "NULL argument");
    const double* src = nullptr;
    if (!std::strcmp(name, "ustar")) src = c->sw.ustar;
    else if (!std::strcmp(name, "obuk")) src = c->sw.obuk;
    else if (!std::strcmp(name, "dudz")) src = c->sw.dudz;
    else if (!std::strcmp(name, "dvdz")) src = c->sw.dvdz;
    else if (!std::strcmp(name, "dbdz")) src = c->sw.dbdz;
    if (!src) return fail(MHH_ERR_ARG, "unknown surface array");
    if (cudaMemcpy(out, src, sizeof(double)*c->d.ijcells, cudaMemcpyDeviceToHost) != cudaSuccess)
        return fail(MHH_ERR_CUDA, "cudaMemcpy");
    return MHH_OK;
}

static int tend_only(mhh_ctx* c, const mhh_fields* f, const mhh_bcfields* bc, int adv, int dif, bool buoy, bool force,
                     double fbody, cudaStream_t s)
{
    if (!c || !f || !f->u || !f->v || !f->w || !f->ut || !f->vt || !f->wt) return fail(MHH_ERR_ARG, "NULL field");
    const bool scal = f->s && f->st;
    const bool surf = dif == MHH_DIFF_SMAG2 && c->phys.surface;
    if (adv == MHH_ADVEC_2I5 && (c->d.igc < 3 || c->d.jgc < 3)) return fail(MHH_ERR_ARG, "Advec_2i5 needs 3 ghost cells");
    if (surf && !bc) return fail(MHH_ERR_ARG, "surface diffusion needs the boundary arrays");
    if (dif == MHH_DIFF_SMAG2 && !f->evisc) return fail(MHH_ERR_ARG, "evisc is NULL");
    if (buoy && !f->s) return fail(MHH_ERR_ARG, "buoyancy needs the scalar");
    if (adv == MHH_ADVEC_2I5 && c->fluxlimit_s) adv = ADVEC_2I5_LIM;
    if (c->prec == MHH_FP64)
    {
        TendArgs<double> a = tend_args<double>(c, f, bc); a.fbody = fbody;
        launch_tendency<double>(c->d, c->pd, a, adv, dif, surf, scal && !buoy, buoy, force, opts_of(c), s);
    }
    else
    {
        TendArgs<float> a = tend_args<float>(c, f, bc); a.fbody = float(fbody);
        launch_tendency<float>(c->d, c->pf, a, adv, dif, surf, scal && !buoy, buoy, force, opts_of(c), s);
    }
    return check_cuda("tendency");
}

int mhh_advec_2i5_exec(mhh_ctx* c, const mhh_fields* f, cudaStream_t s)
{ return tend_only(c, f, nullptr, MHH_ADVEC_2I5, 0, false, false, 0., s); }

int mhh_advec_2i5_set_fluxlimit(mhh_ctx* c, int limit_scalar)
{
    if (!c) return fail(MHH_ERR_ARG, "NULL argument");
    // The limiter's wall treatment needs four levels (src/advec_2i5.cxx
    // applies separate stencils at kstart, kstart+1, kend-2 and kend-1).
    if (limit_scalar && c->d.ktot < 4) return fail(MHH_ERR_ARG, "the flux limiter needs ktot >= 4");
    c->fluxlimit_s = limit_scalar ? 1 : 0;
    return MHH_OK;
}

int mhh_advec_2_exec(mhh_ctx* c, const mhh_fields* f, cudaStream_t s)
{ return tend_only(c, f, nullptr, MHH_ADVEC_2, 0, false, false, 0., s); }

int mhh_diff_smag2_exec(mhh_ctx* c, const mhh_fields* f, const mhh_bcfields* bc, cudaStream_t s)
{ return tend_only(c, f, bc, 0, MHH_DIFF_SMAG2, false, false, 0., s); }

int mhh_diff_2_exec(mhh_ctx* c, const mhh_fields* f, cudaStream_t s)
{ return tend_only(c, f, nullptr, 0, MHH_DIFF_2, false, false, 0., s); }

int mhh_thermo_dry_exec(mhh_ctx* c, const mhh_fields* f, cudaStream_t s)
{
    if (!c || !f || !f->s) return fail(MHH_ERR_ARG, "buoyancy needs the scalar");
    mhh_fields g = *f; g.st = nullptr;   // only wt changes
    return tend_only(c, &g, nullptr, 0, 0, true, false, 0., s);
}

int mhh_force_dpdx_exec(mhh_ctx* c, const mhh_fields* f, double dpdx, cudaStream_t s)
{
    if (!c || !f) return fail(MHH_ERR_ARG, "NULL argument");
    mhh_fields g = *f; g.s = nullptr; g.st = nullptr;
    return tend_only(c, &g, nullptr, 0, 0, false, true, -1.*dpdx, s);
}

int mhh_diff_smag2_exec_viscosity(mhh_ctx* c, const mhh_fields* f, const mhh_bcfields* bc, cudaStream_t s)
{
    (void)bc;
    if (!c || !f) return fail(MHH_ERR_ARG, "NULL argument");
    return c->prec == MHH_FP64 ? viscosity<double>(c, f, s) : viscosity<float>(c, f, s);
}

static int reduce(mhh_ctx* c, int what, const mhh_fields* f, double* out, cudaStream_t s)
{
    cudaMemsetAsync(c->red, 0, sizeof(unsigned long long), s);
    const double tprfi = 1./std::min(1., c->phys.tpr);
    if (c->prec == MHH_FP64)
        launch_reduce<double>(what, c->d, c->pd, (const double*)f->u, (const double*)f->v, (const double*)f->w,
                              (const double*)f->evisc, tprfi, c->red, s);
    else
        launch_reduce<float>(what, c->d, c->pf, (const float*)f->u, (const float*)f->v, (const float*)f->w,
                             (const float*)f->evisc, tprfi, c->red, s);
    int rc = check_cuda("reduce");
    if (rc) return rc;
    return reduce_to_host(c, s, out);
}

int mhh_advec_get_cfl(mhh_ctx* c, int scheme, const mhh_fields* f, double dt, double* cfl, cudaStream_t s)
{
    if (!c || !f || !cfl) return fail(MHH_ERR_ARG, "NULL argument");
    if (scheme == MHH_ADVEC_2I5 && (c->d.igc < 3 || c->d.jgc < 3)) return fail(MHH_ERR_ARG, "Advec_2i5 needs 3 ghost cells");
    double v;
    int rc = reduce(c, scheme == MHH_ADVEC_2I5 ? 0 : 1, f, &v, s);
    *cfl = v*dt;
    return rc;
}

int mhh_advec_get_time_limit(mhh_ctx* c, int scheme, const mhh_fields* f, unsigned long long idt, double dt,
                             unsigned long long* lim, cudaStream_t s)
{
    double cfl;
    int rc = mhh_advec_get_cfl(c, scheme, f, dt, &cfl, s);
    if (rc) return rc;
    cfl = std::max(1.e-5, cfl);
    *lim = (unsigned long long)((double)idt*c->phys.cflmax/cfl);
    return MHH_OK;
}

int mhh_diff_smag2_get_dn(mhh_ctx* c, const mhh_fields* f, double dt, double* dn, cudaStream_t s)
{
    if (!c || !f || !dn || !f->evisc) return fail(MHH_ERR_ARG, "NULL argument");
    double v;
    int rc = reduce(c, 2, f, &v, s);
    *dn = v*dt;
    return rc;
}

int mhh_diff_2_get_dn(mhh_ctx* c, double dt, double* dn)
{
    if (!c || !dn) return fail(MHH_ERR_ARG, "NULL argument");
    *dn = c->dnmul2*dt;
    return MHH_OK;
}

}

namespace mhh
{
    // Horizontal mean and variance of one level per block, in double (two
    // passes over the level: the mean, then the mean squared deviation).
    template<typename TF>
    __global__ void __launch_bounds__(256)
    k_profile(Dims d, const TF* __restrict__ a, double* __restrict__ mean, double* __restrict__ var)
    {
        const int k = blockIdx.x;
        const int n = d.itot*d.jtot;
        __shared__ double sm[8];
        __shared__ double m_sh;
        auto block_sum = [&](double v) -> double
        {
            for (int o=16; o>0; o>>=1) v += __shfl_xor_sync(0xffffffffu, v, o);
            if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = v;
            __syncthreads();
            double t = 0.;
            if (threadIdx.x == 0) { for (int q=0; q<8; ++q) t += sm[q]; }
            __syncthreads();
            return t;
        };
        double s = 0.;
        for (int q = threadIdx.x; q < n; q += blockDim.x)
        {
            const int j = q / d.itot, i = q - j*d.itot;
            s += double(a[ijk(d, i + d.istart, j + d.jstart, k)]);
        }
        s = block_sum(s);
        if (threadIdx.x == 0) m_sh = s/n;
        __syncthreads();
        const double m = m_sh;
        double v = 0.;
        for (int q = threadIdx.x; q < n; q += blockDim.x)
        {
            const int j = q / d.itot, i = q - j*d.itot;
            const double x = double(a[ijk(d, i + d.istart, j + d.jstart, k)]) - m;
            v += x*x;
        }
        v = block_sum(v);
        if (threadIdx.x == 0) { mean[k] = m; var[k] = v/n; }
    }
}

extern "C" {

static bool buffer_ready(const mhh_ctx* c, const mhh_fields* f)
{
    const int need = f->s ? 7 : 3;
    return (c->buf_set & need) == need;
}

static int upload_buffer(mhh_ctx* c)
{
    const size_t n = c->hbuf.size();
    const size_t tf = c->prec == MHH_FP64 ? 8 : 4;
    if (!c->bufprof && cudaMallocAsync(&c->bufprof, tf*n, c->setup) != cudaSuccess)
        return fail(MHH_ERR_CUDA, "cudaMallocAsync buffer");
    if (cudaStreamSynchronize(c->setup) != cudaSuccess) return fail(MHH_ERR_CUDA, "buffer allocation");
    cudaError_t e;
    if (c->prec == MHH_FP64)
        e = cudaMemcpy(c->bufprof, c->hbuf.data(), 8*n, cudaMemcpyHostToDevice);
    else
    {
        std::vector<float> f(c->hbuf.begin(), c->hbuf.end());
        e = cudaMemcpy(c->bufprof, f.data(), 4*n, cudaMemcpyHostToDevice);
    }
    return e == cudaSuccess ? MHH_OK : fail(MHH_ERR_CUDA, "upload buffer");
}

int mhh_buffer_setup(mhh_ctx* c, double zstart, double sigma, double beta)
{
    if (!c) return fail(MHH_ERR_ARG, "NULL argument");
    const Dims& d = c->d;
    const int kc = d.kcells;
    if (c->hbuf.empty()) c->hbuf.assign(5*(size_t)kc, 0.);
    // src/buffer.cxx:100-130: the layer starts at the first full (half)
    // level at or above zstart; sigma(z) = sigma ((z - zstart)/(zsize - zstart))^beta.
    int kb = d.kstart, kbh = d.kstart;
    for (int k=d.kstart; k<d.kend; ++k)
    {
        if (c->h[P_Z][k] < zstart) ++kb;
        if (c->h[P_ZH][k] < zstart) ++kbh;
    }
    if (kbh == d.kend) return fail(MHH_ERR_ARG, "Buffer is too close to the model top");
    const double zsizebuf = d.zsize - zstart;
    for (int k=0; k<kc; ++k)
    {
        c->hbuf[k] = k >= kb && k < d.kend ? sigma*std::pow((c->h[P_Z][k] - zstart)/zsizebuf, beta) : 0.;
        c->hbuf[kc + k] = k >= kbh && k < d.kend ? sigma*std::pow((c->h[P_ZH][k] - zstart)/zsizebuf, beta) : 0.;
    }
    c->buf_kb = std::min(kb, kbh);
    c->buf_on = 1;
    return upload_buffer(c);
}

int mhh_buffer_set_profile(mhh_ctx* c, const char* name, const double* prof)
{
    if (!c || !name || !prof) return fail(MHH_ERR_ARG, "NULL argument");
    if (!c->buf_on) return fail(MHH_ERR_ARG, "buffer layer not set up");
    int q = -1;
    if (!std::strcmp(name, "u")) q = 2;
    else if (!std::strcmp(name, "v")) q = 3;
    else if (!std::strcmp(name, "th")) q = 4;
    if (q < 0) return fail(MHH_ERR_ARG, "buffer profiles are u, v and th");
    const int kc = c->d.kcells;
    // Profiles are physical values; theta's is stored with the scalar's offset.
    const double off = q == 4 ? c->th0 : 0.;
    for (int k=0; k<kc; ++k) c->hbuf[(size_t)q*kc + k] = prof[k] - off;
    c->buf_set |= 1 << (q - 2);
    return upload_buffer(c);
}

int mhh_buffer_exec(mhh_ctx* c, const mhh_fields* f, cudaStream_t s)
{
    if (!c || !f) return fail(MHH_ERR_ARG, "NULL argument");
    if (!c->buf_on) return MHH_OK;
    if (!buffer_ready(c, f)) return fail(MHH_ERR_ARG, "buffer profiles of u, v (and th) not set");
    if (c->prec == MHH_FP64)
        launch_buffer<double>(c->d, (const double*)c->bufprof, c->buf_kb, (const double*)f->u, (const double*)f->v,
                              (const double*)f->w, (const double*)f->s, (double*)f->ut, (double*)f->vt, (double*)f->wt,
                              (double*)f->st, s);
    else
        launch_buffer<float>(c->d, (const float*)c->bufprof, c->buf_kb, (const float*)f->u, (const float*)f->v,
                             (const float*)f->w, (const float*)f->s, (float*)f->ut, (float*)f->vt, (float*)f->wt,
                             (float*)f->st, s);
    return check_cuda("buffer");
}

int mhh_stats_profile(mhh_ctx* c, const void* field, double* mean, double* var, cudaStream_t s)
{
    if (!c || !field || !mean || !var) return fail(MHH_ERR_ARG, "NULL argument");
    const Dims& d = c->d;
    if (c->prec == MHH_FP64) k_profile<double><<<d.kcells, 256, 0, s>>>(d, (const double*)field, c->statbuf, c->statbuf + d.kcells);
    else k_profile<float><<<d.kcells, 256, 0, s>>>(d, (const float*)field, c->statbuf, c->statbuf + d.kcells);
    count_launch();
    int rc = check_cuda("stats_profile");
    if (rc) return rc;
    cudaMemcpyAsync(mean, c->statbuf, sizeof(double)*d.kcells, cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(var, c->statbuf + d.kcells, sizeof(double)*d.kcells, cudaMemcpyDeviceToHost, s);
    if (cudaStreamSynchronize(s) != cudaSuccess) return fail(MHH_ERR_CUDA, "stats_profile");
    return MHH_OK;
}

int mhh_pres_2_exec(mhh_ctx* c, const mhh_fields* f, double sub_dt, cudaStream_t s)
{
    if (!c || !f || !f->p) return fail(MHH_ERR_ARG, "NULL argument");
    return c->prec == MHH_FP64 ? pres_exec<double>(c, f, sub_dt, true, s) : pres_exec<float>(c, f, sub_dt, true, s);
}

int mhh_pres_2_get_divergence(mhh_ctx* c, const mhh_fields* f, double* div, cudaStream_t s)
{
    if (!c || !f || !div) return fail(MHH_ERR_ARG, "NULL argument");
    return reduce(c, 3, f, div, s);
}

int mhh_fft_forward(mhh_ctx* c, void* data, cudaStream_t s)
{
    if (!c || !data) return fail(MHH_ERR_ARG, "NULL argument");
    const Dims& d = c->d;
    if (c->prec == MHH_FP64)
    {
        launch_fft_x<double>(c->pw.px, (double*)data, d.jtot*d.ktot, false, 1., s);
        launch_fft_y<double>(c->pw.py, (double*)data, d.itot, d.jtot, d.ktot, false, 1., s);
    }
    else
    {
        launch_fft_x<float>(c->pw.px, (float*)data, d.jtot*d.ktot, false, 1., s);
        launch_fft_y<float>(c->pw.py, (float*)data, d.itot, d.jtot, d.ktot, false, 1., s);
    }
    return check_cuda("fft_forward");
}

int mhh_fft_backward(mhh_ctx* c, void* data, cudaStream_t s)
{
    if (!c || !data) return fail(MHH_ERR_ARG, "NULL argument");
    const Dims& d = c->d;
    if (c->prec == MHH_FP64)
    {
        launch_fft_y<double>(c->pw.py, (double*)data, d.itot, d.jtot, d.ktot, true, 1., s);
        launch_fft_x<double>(c->pw.px, (double*)data, d.jtot*d.ktot, true, 1., s);
    }
    else
    {
        launch_fft_y<float>(c->pw.py, (float*)data, d.itot, d.jtot, d.ktot, true, 1., s);
        launch_fft_x<float>(c->pw.px, (float*)data, d.jtot*d.ktot, true, 1., s);
    }
    return check_cuda("fft_backward");
}

int mhh_timeloop_rk3(mhh_ctx* c, void* a, void* at, int substep, double dt, cudaStream_t s)
{
    if (!c || !a || !at || substep < 0 || substep > 2) return fail(MHH_ERR_ARG, "bad argument");
    if (c->prec == MHH_FP64) launch_rk3<double>((double*)a, (double*)at, c->d, substep, dt, s);
    else launch_rk3<float>((float*)a, (float*)at, c->d, substep, dt, s);
    return check_cuda("rk3");
}

int mhh_substep_begin(mhh_ctx* c, const mhh_substep_config* cfg, const mhh_fields* f, const mhh_bcfields* bc,
                      cudaStream_t s)
{
    if (!c || !cfg || !f || !bc) return fail(MHH_ERR_ARG, "NULL argument");
    return c->prec == MHH_FP64 ? substep_begin<double>(c, cfg, f, bc, s) : substep_begin<float>(c, cfg, f, bc, s);
}

int mhh_substep_end(mhh_ctx* c, const mhh_substep_config* cfg, const mhh_fields* f, const mhh_bcfields* bc,
                    int substep, double dt, cudaStream_t s)
{
    if (!c || !cfg || !f || !bc || !f->p || substep < 0 || substep > 2) return fail(MHH_ERR_ARG, "bad argument");
    if (cfg->advec == MHH_ADVEC_2I5 && (c->d.igc < 3 || c->d.jgc < 3)) return fail(MHH_ERR_ARG, "Advec_2i5 needs 3 ghost cells");
    if (cfg->diff == MHH_DIFF_SMAG2 && !f->evisc) return fail(MHH_ERR_ARG, "evisc is NULL");
    if (c->buf_on && !buffer_ready(c, f)) return fail(MHH_ERR_ARG, "buffer profiles of u, v (and th) not set");
    return c->prec == MHH_FP64 ? substep_end<double>(c, cfg, f, bc, substep, dt, s)
                               : substep_end<float>(c, cfg, f, bc, substep, dt, s);
}

}

// ---------------------------------------------------------------------------
// Batched substeps: many contexts, one launch per stage.
//
// The plan records, for every context and substep, the launches of
// mhh_substep_begin/end (launch_body appends them instead of launching,
// mhh_batchable.cuh).  Stage i of a substep is the i-th launch of every
// context; equal kernels (the same k_many entry point and block shape) of a
// stage form one launch over all their contexts, with the contexts' grids
// laid end to end.  Each context's kernels run with the same parameters and
// block positions as in its own substep, so the results are the same bit for
// bit.  The recording runs inside a stream capture on a scratch stream that
// is then discarded: a launch that cannot be batched (it does not go through
// launch_body) is caught by the launch count and the plan is refused.
// ---------------------------------------------------------------------------
namespace mhh
{
    BatchRecorder*& batch_recorder()
    {
        thread_local BatchRecorder* r = nullptr;
        return r;
    }
}

struct mhh_batch
{
    struct Group
    {
        int stage;
        const void* fn;
        dim3 block;
        size_t smem;
        int nmem;
        dim3 grid;
        std::vector<unsigned char> args;   // ManyArgs (k_many), or P of one context (k_one)
    };
    int n;
    std::vector<Group> groups[3];
    // Groups of one stage (different contexts) run side by side: the extra
    // groups of a stage go to their own streams, forked from and joined into
    // the caller's stream.
    std::vector<cudaStream_t> side;
    std::vector<cudaEvent_t> events;    // [0] fork, [1..] joins
};

namespace
{
    void batch_free(mhh_batch* b)
    {
        for (auto st : b->side) cudaStreamDestroy(st);
        for (auto e : b->events) cudaEventDestroy(e);
        delete b;
    }

    // The launches of one substep of context c (nothing runs).
    int record_substep(mhh_ctx* c, const mhh_substep_config* cfg, const mhh_fields* f, const mhh_bcfields* bc,
                       int substep, double dt, cudaStream_t scratch, std::vector<mhh::RecordedLaunch>& out)
    {
        mhh::BatchRecorder rec;
        const bool timing = g_timing;
        g_timing = false;
        const long long n0 = launch_count();
        if (cudaStreamBeginCapture(scratch, cudaStreamCaptureModeThreadLocal) != cudaSuccess)
        {
            g_timing = timing;
            return fail(MHH_ERR_CUDA, "batch: stream capture");
        }
        mhh::batch_recorder() = &rec;
        int rc = mhh_substep_begin(c, cfg, f, bc, scratch);
        if (!rc) rc = mhh_substep_end(c, cfg, f, bc, substep, dt, scratch);
        mhh::batch_recorder() = nullptr;
        cudaGraph_t g = nullptr;
        cudaStreamEndCapture(scratch, &g);
        if (g) cudaGraphDestroy(g);
        cudaGetLastError();
        g_timing = timing;
        const long long counted = launch_count() - n0;
        mhh_launch_count_add(-counted);
        if (rc) return rc;
        if (counted != (long long)rec.launches.size())
            return fail(MHH_ERR_UNSUPPORTED, "batch: a kernel of this configuration cannot run batched");
        out = std::move(rec.launches);
        return MHH_OK;
    }
}

extern "C" {

int mhh_batch_create(int n, mhh_ctx* const* ctx, const mhh_substep_config* cfg, const mhh_fields* f,
                     const mhh_bcfields* bc, const double* dt, mhh_batch** out)
{
    if (n < 1 || !ctx || !cfg || !f || !bc || !dt || !out) return fail(MHH_ERR_ARG, "NULL argument");
    for (int m=0; m<n; ++m)
        if (!ctx[m] || ctx[m]->prec != ctx[0]->prec) return fail(MHH_ERR_ARG, "batch: contexts of one precision");
    cudaStream_t scratch = nullptr;
    if (cudaStreamCreateWithFlags(&scratch, cudaStreamNonBlocking) != cudaSuccess) return fail(MHH_ERR_CUDA, "stream");
    mhh_batch* b = new mhh_batch();
    b->n = n;
    int rc = MHH_OK;
    for (int q=0; q<3 && !rc; ++q)
    {
        std::vector<std::vector<mhh::RecordedLaunch>> rec(n);
        for (int m=0; m<n && !rc; ++m)
            rc = record_substep(ctx[m], &cfg[m], &f[m], &bc[m], q, dt[m], scratch, rec[m]);
        if (rc) break;
        const size_t nstage = rec[0].size();
        for (int m=1; m<n; ++m)
            if (rec[m].size() != nstage) { rc = fail(MHH_ERR_UNSUPPORTED, "batch: contexts with different stages"); break; }
        for (size_t st=0; st<nstage && !rc; ++st)
        {
            // Contexts of this stage grouped by entry point and block shape.
            std::vector<int> done(n, 0);
            for (int m0=0; m0<n && !rc; ++m0)
            {
                if (done[m0]) continue;
                const mhh::RecordedLaunch& L0 = rec[m0][st];
                std::vector<int> mem;
                for (int m=m0; m<n; ++m)
                {
                    const mhh::RecordedLaunch& L = rec[m][st];
                    if (!done[m] && L.fn == L0.fn && L.block.x == L0.block.x && L.block.y == L0.block.y
                        && L.block.z == L0.block.z && L.params.size() == L0.params.size())
                    { mem.push_back(m); done[m] = 1; }
                }
                // One launch per chunk of at most nmax contexts (the kernel
                // parameter space holds their parameter structs).
                const size_t psz = L0.params.size();
                for (size_t c0=0; c0<mem.size() && !rc; c0 += (size_t)L0.nmax)
                {
                    const size_t nc = std::min(mem.size() - c0, (size_t)L0.nmax);
                    mhh_batch::Group g{};
                    g.stage = (int)st;
                    g.fn = L0.fn; g.block = L0.block; g.nmem = (int)nc;
                    if (nc == 1)
                    {
                        const mhh::RecordedLaunch& L = rec[mem[c0]][st];
                        g.fn = L.fn_one; g.grid = L.grid; g.smem = L.smem; g.args = L.params;
                        b->groups[q].push_back(std::move(g));
                        continue;
                    }
                    g.args.assign(L0.args_size, 0);
                    unsigned char* A = g.args.data();
                    long long total = 0;
                    for (size_t q2=0; q2<nc; ++q2)
                    {
                        const mhh::RecordedLaunch& L = rec[mem[c0 + q2]][st];
                        std::memcpy(A + L0.off_p + q2*psz, L.params.data(), psz);
                        const int4 gr = make_int4((int)L.grid.x, (int)L.grid.y, (int)L.grid.z, 0);
                        std::memcpy(A + L0.off_grid + q2*sizeof(int4), &gr, sizeof(int4));
                        const int st0 = (int)total;
                        std::memcpy(A + L0.off_start + q2*sizeof(int), &st0, sizeof(int));
                        total += (long long)L.grid.x*L.grid.y*L.grid.z;
                        g.smem = std::max(g.smem, L.smem);
                    }
                    if (total <= 0 || total > 0x7fffffffLL) { rc = fail(MHH_ERR_UNSUPPORTED, "batch: grid too large"); break; }
                    const int tot = (int)total, ncs = (int)nc;
                    std::memcpy(A + L0.off_start + nc*sizeof(int), &tot, sizeof(int));
                    std::memcpy(A + L0.off_n, &ncs, sizeof(int));
                    g.grid = dim3((unsigned)tot);
                    b->groups[q].push_back(std::move(g));
                }
            }
        }
    }
    cudaStreamDestroy(scratch);
    // Side streams for the largest number of groups in one stage.
    size_t width = 1;
    for (int q=0; q<3 && !rc; ++q)
        for (size_t a=0; a<b->groups[q].size(); )
        {
            size_t e = a;
            while (e < b->groups[q].size() && b->groups[q][e].stage == b->groups[q][a].stage) ++e;
            width = std::max(width, e - a);
            a = e;
        }
    for (size_t w=1; w<width && !rc; ++w)
    {
        cudaStream_t st;
        if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess) { rc = fail(MHH_ERR_CUDA, "stream"); break; }
        b->side.push_back(st);
    }
    for (size_t w=0; w<width && !rc; ++w)
    {
        cudaEvent_t e;
        if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) { rc = fail(MHH_ERR_CUDA, "event"); break; }
        b->events.push_back(e);
    }
    if (!rc && cudaDeviceSynchronize() != cudaSuccess) rc = fail(MHH_ERR_CUDA, "batch: set-up");
    if (rc) { batch_free(b); return rc; }
    *out = b;
    return MHH_OK;
}

int mhh_batch_substep(mhh_batch* b, int substep, cudaStream_t s)
{
    if (!b || substep < 0 || substep > 2) return fail(MHH_ERR_ARG, "bad argument");
    auto launch = [&](const mhh_batch::Group& g, cudaStream_t st)
    {
        void* args[] = {(void*)g.args.data()};
        return cudaLaunchKernel(g.fn, g.grid, g.block, args, g.smem, st) == cudaSuccess;
    };
    const auto& gs = b->groups[substep];
    for (size_t a=0; a<gs.size(); )
    {
        size_t e = a;
        while (e < gs.size() && gs[e].stage == gs[a].stage) ++e;
        bool ok = true;
        if (e - a == 1) ok = launch(gs[a], s);
        else
        {
            ok = cudaEventRecord(b->events[0], s) == cudaSuccess;
            for (size_t g=a+1; g<e && ok; ++g)
            {
                cudaStream_t st = b->side[g - a - 1];
                ok = cudaStreamWaitEvent(st, b->events[0], 0) == cudaSuccess && launch(gs[g], st)
                     && cudaEventRecord(b->events[g - a], st) == cudaSuccess;
            }
            ok = ok && launch(gs[a], s);
            for (size_t g=a+1; g<e && ok; ++g) ok = cudaStreamWaitEvent(s, b->events[g - a], 0) == cudaSuccess;
        }
        if (!ok) return fail(MHH_ERR_CUDA, "batch: launch");
        a = e;
    }
    count_launch((int)gs.size());
    return check_cuda("batch substep");
}

int mhh_batch_launches(const mhh_batch* b, int substep, int* nlaunch)
{
    if (!b || !nlaunch || substep < 0 || substep > 2) return fail(MHH_ERR_ARG, "bad argument");
    *nlaunch = (int)b->groups[substep].size();
    return MHH_OK;
}

int mhh_batch_destroy(mhh_batch* b)
{
    if (!b) return MHH_OK;
    cudaDeviceSynchronize();
    batch_free(b);
    return MHH_OK;
}

}
