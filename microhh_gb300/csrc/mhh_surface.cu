// mhh_surface.cu -- Monin-Obukhov surface layer on the GPU, after
// src/boundary_surface.cxx:836-994 and include/boundary_surface_kernels.h
// (lookup-table Obukhov-length solver with homogeneous z0m/z0h, noslip
// momentum, flux or Dirichlet scalar).  All 2-D arithmetic is in double; the
// z/L lookup table and the Richardson-number interpolation stay in float as in
// the reference, with the float operations rounded one by one so that they
// match the CPU bit for bit.
#include "mhh_kernels.cuh"

namespace mhh
{
    __device__ __forceinline__ double phim_unstable(double z) { return pow(1. + 3.6*pow(fabs(z), 2./3.), -1./2.); }
    __device__ __forceinline__ double phih_unstable(double z) { return pow(1. + 7.9*pow(fabs(z), 2./3.), -1./2.); }
    __device__ __forceinline__ double phim(double z) { return z <= 0. ? phim_unstable(z) : 1. + 5.*z; }
    __device__ __forceinline__ double phih(double z) { return z <= 0. ? phih_unstable(z) : (1. + 4.*z)*(1. + 4.*z); }
    __device__ __forceinline__ double psim_unstable(double z) { return 3.*log((1. + 1./phim_unstable(z))/2.); }
    __device__ __forceinline__ double psih_unstable(double z) { return 3.*log((1. + 1./phih_unstable(z))/2.); }
    __device__ __forceinline__ double psim_stable(double z)
    {
        const double a = 1., b = 2./3., c = 5., d = 0.35;
        return -b*(z - (c/d))*exp(-d*z) - a*z - (b*c)/d;
    }
    __device__ __forceinline__ double psih_stable(double z)
    {
        const double a = 1., b = 2./3., c = 5., d = 0.35;
        return -b*(z - (c/d))*exp(-d*z) - pow(1. + b*a*z, 1.5) - (b*c)/d + 1.;
    }
    // include/monin_obukhov.h:137-152
    __device__ __forceinline__ double most_fm(double zsl, double z0m, double L)
    {
        return L <= 0. ? KAPPA/(log(zsl/z0m) - psim_unstable(zsl/L) + psim_unstable(z0m/L))
                       : KAPPA/(log(zsl/z0m) - psim_stable  (zsl/L) + psim_stable  (z0m/L));
    }
    __device__ __forceinline__ double most_fh(double zsl, double z0h, double L)
    {
        return L <= 0. ? KAPPA/(log(zsl/z0h) - psih_unstable(zsl/L) + psih_unstable(z0h/L))
                       : KAPPA/(log(zsl/z0h) - psih_stable  (zsl/L) + psih_stable  (z0h/L));
    }

    // include/boundary_surface_kernels.h:282-298, with the search kept inside
    // the table.
    __device__ double find_zL(const float* zL, const float* f, int* np, float Ri)
    {
        int n = *np;
        if (__fsub_rn(f[n], Ri) > 0.f)
            while (n > 0 && __fsub_rn(f[n-1], Ri) > 0.f) --n;
        else
            while (__fsub_rn(f[n], Ri) < 0.f && n < NZL_LUT-1) ++n;
        *np = n;
        if (n == 0 || n == NZL_LUT-1) return (double)zL[n];
        const float num = __fsub_rn(Ri, f[n-1]);
        const float den = __fsub_rn(f[n], f[n-1]);
        const float dz = __fsub_rn(zL[n], zL[n-1]);
        return (double)__fadd_rn(zL[n-1], __fmul_rn(__fdiv_rn(num, den), dz));
    }

    // Filtered wind speed, include/boundary_surface_kernels.h:132-178 (interior).
    template<typename TF>
    __global__ void k_dutot(Dims d, const TF* __restrict__ u, const TF* __restrict__ v,
                            const TF* __restrict__ ubot, const TF* __restrict__ vbot, double* __restrict__ dutot)
    {
        const int i = d.istart + blockIdx.x*blockDim.x + threadIdx.x;
        const int j = d.jstart + blockIdx.y*blockDim.y + threadIdx.y;
        if (i >= d.iend || j >= d.jend) return;
        const long long ii = 1, jj = d.icells;
        const long long ij = i + j*jj;
        const long long c = ij + (long long)d.kstart*d.ijcells;
        auto U = [&](long long q) { return double(u[q]); };
        auto V = [&](long long q) { return double(v[q]); };
        const double uf = (1./9)*(
              0.5*U(c-ii-jj) + U(c-jj) + U(c+ii-jj) + 0.5*U(c+2*ii-jj)
            + 0.5*U(c-ii   ) + U(c   ) + U(c+ii   ) + 0.5*U(c+2*ii   )
            + 0.5*U(c-ii+jj) + U(c+jj) + U(c+ii+jj) + 0.5*U(c+2*ii+jj));
        const double vf = (1./9)*(
              0.5*V(c-ii-jj) + V(c-ii) + V(c-ii+jj) + 0.5*V(c-ii+2*jj)
            + 0.5*V(c   -jj) + V(c   ) + V(c   +jj) + 0.5*V(c   +2*jj)
            + 0.5*V(c+ii-jj) + V(c+ii) + V(c+ii+jj) + 0.5*V(c+ii+2*jj));
        const double du2 = sq(uf - 0.5*(double(ubot[ij]) + double(ubot[ij+ii])))
                         + sq(vf - 0.5*(double(vbot[ij]) + double(vbot[ij+jj])));
        dutot[ij] = fmax(pow(du2, 0.5), 1.e-1);
    }

    // The Monin-Obukhov functions of one cell, each evaluated once: the
    // similarity function phi of the stability branch feeds both the
    // integrated psi and the gradient (include/monin_obukhov.h:40-152).
    struct MostCell { double fm, fh, phim, phih; };

    __device__ __forceinline__ MostCell most_cell(double zsl, double z0m, double z0h, double L)
    {
        MostCell r;
        const double zeta = zsl/L;
        if (L <= 0.)
        {
            const double pm_s = phim_unstable(zeta), pm_0 = phim_unstable(z0m/L);
            const double ph_s = phih_unstable(zeta), ph_0 = phih_unstable(z0h/L);
            const double psim_s = 3.*log((1. + 1./pm_s)/2.), psim_0 = 3.*log((1. + 1./pm_0)/2.);
            const double psih_s = 3.*log((1. + 1./ph_s)/2.), psih_0 = 3.*log((1. + 1./ph_0)/2.);
            r.fm = KAPPA/(log(zsl/z0m) - psim_s + psim_0);
            r.fh = KAPPA/(log(zsl/z0h) - psih_s + psih_0);
            r.phim = zeta <= 0. ? pm_s : 1. + 5.*zeta;
            r.phih = zeta <= 0. ? ph_s : (1. + 4.*zeta)*(1. + 4.*zeta);
        }
        else
        {
            r.fm = KAPPA/(log(zsl/z0m) - psim_stable(zeta) + psim_stable(z0m/L));
            r.fh = KAPPA/(log(zsl/z0h) - psih_stable(zeta) + psih_stable(z0h/L));
            r.phim = phim(zeta);
            r.phih = phih(zeta);
        }
        return r;
    }

    // Obukhov length and friction velocity, src/boundary_surface.cxx:55-160
    // (all cells; the neutral branch when there is no thermodynamics).
    template<typename TF>
    __global__ void k_stability(Dims d, SurfWork sw, const TF* __restrict__ s, const TF* __restrict__ s_bot,
                                const TF* __restrict__ s_flux, double zsl, double z0m, double thref_s, double threfh_s,
                                int thermo, int thermo_bc)
    {
        const int n = blockIdx.x*blockDim.x + threadIdx.x;
        if (n >= d.ijcells) return;
        const double du = sw.dutot[n];
        double L;
        if (!thermo)
            L = -DBIG;
        else if (thermo_bc == MHH_BC_FLUX)
        {
            const double bfluxbot = GRAV/threfh_s*double(s_flux[n]);
            const float Ri = (float)(-KAPPA*bfluxbot*zsl/(du*du*du));
            L = zsl/find_zL(sw.zL, sw.f, &sw.nobuk[n], Ri);
        }
        else
        {
            const double b = GRAV/thref_s*(double(s[n + (long long)d.kstart*d.ijcells]) - thref_s);
            const double bbot = GRAV/threfh_s*(double(s_bot[n]) - threfh_s);
            const double db_ref = GRAV/thref_s*(thref_s - threfh_s);
            const double db = b - bbot + db_ref;
            const float Ri = (float)(KAPPA*db*zsl/(du*du));
            L = zsl/find_zL(sw.zL, sw.f, &sw.nobuk[n], Ri);
        }
        // zsl/L and z0/L of a large |L| can reach zero; the branch choice
        // follows the sign of L exactly as the separate functions do.
        const MostCell mc = most_cell(zsl, z0m, sw.z0h, L);
        sw.obuk[n] = L;
        sw.ustar[n] = du*mc.fm;
        sw.fm[n] = mc.fm; sw.fh[n] = mc.fh; sw.phim[n] = mc.phim; sw.phih[n] = mc.phih;
    }

    // Momentum fluxes, src/boundary_surface.cxx:163-190 (interior).
    template<typename TF>
    __global__ void k_surfm(Dims d, SurfWork sw, const TF* __restrict__ u, const TF* __restrict__ v,
                            const TF* __restrict__ ubot, const TF* __restrict__ vbot,
                            TF* __restrict__ uflux, TF* __restrict__ vflux, double zsl, double z0m)
    {
        const int i = d.istart + blockIdx.x*blockDim.x + threadIdx.x;
        const int j = d.jstart + blockIdx.y*blockDim.y + threadIdx.y;
        if (i >= d.iend || j >= d.jend) return;
        const long long ii = 1, jj = d.icells;
        const long long ij = i + j*jj;
        const long long c = ij + (long long)d.kstart*d.ijcells;
        const double fc = sw.ustar[ij]*sw.fm[ij];
        uflux[ij] = TF(-(double(u[c]) - double(ubot[ij]))*0.5*(sw.ustar[ij-ii]*sw.fm[ij-ii] + fc));
        vflux[ij] = TF(-(double(v[c]) - double(vbot[ij]))*0.5*(sw.ustar[ij-jj]*sw.fm[ij-jj] + fc));
    }

    // Surface gradients of u and v and the scalar surface value, gradient or
    // flux, src/boundary_surface.cxx:255-338 (all cells).
    template<typename TF>
    __global__ void k_surf_grads(Dims d, SurfWork sw, const TF* __restrict__ u, const TF* __restrict__ v,
                                 const TF* __restrict__ ubot, const TF* __restrict__ vbot,
                                 TF* __restrict__ ugrad, TF* __restrict__ vgrad,
                                 const TF* __restrict__ s, TF* __restrict__ sbot, TF* __restrict__ sgrad,
                                 TF* __restrict__ sflux, double zsl, double z0h, int thermo, int thermo_bc)
    {
        const int n = blockIdx.x*blockDim.x + threadIdx.x;
        if (n >= d.ijcells) return;
        const long long c = n + (long long)d.kstart*d.ijcells;
        ugrad[n] = TF((double(u[c]) - double(ubot[n]))/zsl);
        vgrad[n] = TF((double(v[c]) - double(vbot[n]))/zsl);
        if (thermo)
        {
            const double th = double(s[c]);
            if (thermo_bc == MHH_BC_DIRICHLET)
            {
                sflux[n] = TF(-(th - double(sbot[n]))*sw.ustar[n]*sw.fh[n]);
                sgrad[n] = TF((th - double(sbot[n]))/zsl);
            }
            else
            {
                const double bot = double(sflux[n])/(sw.ustar[n]*sw.fh[n]) + th;
                sbot[n] = TF(bot);
                sgrad[n] = TF((th - bot)/zsl);
            }
        }
    }

    // Monin-Obukhov gradients for the next viscosity, include/boundary_surface_kernels.h:180-238.
    template<typename TF>
    __global__ void k_duvdz(Dims d, SurfWork sw, const TF* __restrict__ u, const TF* __restrict__ v,
                            const TF* __restrict__ ubot, const TF* __restrict__ vbot, const TF* __restrict__ sflux,
                            double zsl, double z0m, double threfh_s, int thermo)
    {
        const int i = d.istart + blockIdx.x*blockDim.x + threadIdx.x;
        const int j = d.jstart + blockIdx.y*blockDim.y + threadIdx.y;
        if (i >= d.iend || j >= d.jend) return;
        const long long ii = 1, jj = d.icells;
        const long long ij = i + j*jj;
        const long long c = ij + (long long)d.kstart*d.ijcells;
        const double du_c = 0.5*((double(u[c]) - double(ubot[ij])) + (double(u[c+ii]) - double(ubot[ij+ii])));
        const double dv_c = 0.5*((double(v[c]) - double(vbot[ij])) + (double(v[c+jj]) - double(vbot[ij+jj])));
        const double us = sw.ustar[ij];
        const double fmv = sw.fm[ij];
        const double ufb = -du_c*us*fmv;
        const double vfb = -dv_c*us*fmv;
        const double ph = sw.phim[ij];
        sw.dudz[ij] = -ufb/(KAPPA*zsl*us)*ph;
        sw.dvdz[ij] = -vfb/(KAPPA*zsl*us)*ph;
        if (thermo)
        {
            const double bfb = GRAV/threfh_s*double(sflux[ij]);
            sw.dbdz[ij] = -bfb/(KAPPA*zsl*us)*sw.phih[ij];
        }
    }

    template<typename TF>
    void launch_surface(const Dims& d, const Prof<TF>& pr, const SurfWork& sw,
                        const TF* u, const TF* v, const TF* s,
                        TF* u_bot, TF* v_bot, TF* u_flux, TF* v_flux, TF* u_grad, TF* v_grad,
                        TF* s_bot, TF* s_flux, TF* s_grad,
                        int thermo, int thermo_bc, double z0m, double z0h, cudaStream_t st)
    {
        const double zsl = sw.zsl, thref_s = sw.thref_s, threfh_s = sw.threfh_s;
        dim3 b2(32, 8), g2((d.itot + 31)/32, (d.jtot + 7)/8);
        const int nb = (d.ijcells + 255)/256;
        k_dutot<TF><<<g2, b2, 0, st>>>(d, u, v, u_bot, v_bot, sw.dutot);
        launch_cyclic2d<double>(sw.dutot, d, st);
        k_stability<TF><<<nb, 256, 0, st>>>(d, sw, s, s_bot, s_flux, zsl, z0m, thref_s, threfh_s, thermo, thermo_bc);
        k_surfm<TF><<<g2, b2, 0, st>>>(d, sw, u, v, u_bot, v_bot, u_flux, v_flux, zsl, z0m);
        launch_cyclic2d<TF>(u_flux, d, st);
        launch_cyclic2d<TF>(v_flux, d, st);
        k_surf_grads<TF><<<nb, 256, 0, st>>>(d, sw, u, v, u_bot, v_bot, u_grad, v_grad, s, s_bot, s_grad, s_flux,
                                             zsl, z0h, thermo, thermo_bc);
        k_duvdz<TF><<<g2, b2, 0, st>>>(d, sw, u, v, u_bot, v_bot, s_flux, zsl, z0m, threfh_s, thermo);
        count_launch(5);
    }

    template void launch_surface<double>(const Dims&, const Prof<double>&, const SurfWork&, const double*, const double*,
        const double*, double*, double*, double*, double*, double*, double*, double*, double*, double*,
        int, int, double, double, cudaStream_t);
    template void launch_surface<float>(const Dims&, const Prof<float>&, const SurfWork&, const float*, const float*,
        const float*, float*, float*, float*, float*, float*, float*, float*, float*, float*,
        int, int, double, double, cudaStream_t);
}
