// mhh_surface.cu -- Monin-Obukhov surface layer on the GPU, after
// src/boundary_surface.cxx:836-994 and include/boundary_surface_kernels.h
// (lookup-table Obukhov-length solver with homogeneous z0m/z0h, noslip
// momentum, flux or Dirichlet scalar).  The 2-D fields are stored in double;
// the Obukhov length and the similarity functions are computed in the field
// precision (double for the FP64 path, float for the FP32 form, which keeps
// the float form off the slow FP64 pipe).  The z/L lookup table and the
// Richardson-number interpolation stay in float as in the reference, with the
// float operations rounded one by one so that they match the CPU bit for bit.
#include "mhh_kernels.cuh"
#include "mhh_batchable.cuh"

namespace mhh
{
    // Monin-Obukhov similarity functions, include/monin_obukhov.h:40-152, in
    // the compute type CT (double for the FP64 path, float for the FP32 form).
    template<typename CT> __device__ __forceinline__ CT phim_unstable(CT z)
    { return pow(CT(1) + CT(3.6)*pow(fabs(z), CT(2./3.)), CT(-1./2.)); }
    template<typename CT> __device__ __forceinline__ CT phih_unstable(CT z)
    { return pow(CT(1) + CT(7.9)*pow(fabs(z), CT(2./3.)), CT(-1./2.)); }
    template<typename CT> __device__ __forceinline__ CT phim(CT z) { return z <= CT(0) ? phim_unstable(z) : CT(1) + CT(5)*z; }
    template<typename CT> __device__ __forceinline__ CT phih(CT z) { return z <= CT(0) ? phih_unstable(z) : (CT(1) + CT(4)*z)*(CT(1) + CT(4)*z); }
    template<typename CT> __device__ __forceinline__ CT psim_stable(CT z)
    {
        const CT a = 1, b = CT(2)/CT(3), c = 5, d = CT(0.35);
        return -b*(z - (c/d))*exp(-d*z) - a*z - (b*c)/d;
    }
    template<typename CT> __device__ __forceinline__ CT psih_stable(CT z)
    {
        const CT a = 1, b = CT(2)/CT(3), c = 5, d = CT(0.35);
        return -b*(z - (c/d))*exp(-d*z) - pow(CT(1) + b*a*z, CT(1.5)) - (b*c)/d + CT(1);
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

    // Everything the surface-layer kernels of one context read and write.
    template<typename TF> struct SurfP
    {
        Dims d; SurfWork sw;
        const TF *u, *v, *s;
        TF *u_bot, *v_bot, *u_flux, *v_flux, *u_grad, *v_grad, *s_bot, *s_flux, *s_grad;
        double zsl, z0m, z0h, thref_s, threfh_s, thb_s, thbh_s;
        int thermo, thermo_bc;
    };

    // Filtered wind speed, include/boundary_surface_kernels.h:132-178
    // (interior), in the field precision.
    template<typename TF>
    __device__ __forceinline__ void dutot_body(const SurfP<TF>& P, const VBlock& vb)
    {
        const Dims& d = P.d;
        const TF* __restrict__ u = P.u; const TF* __restrict__ v = P.v;
        const TF* __restrict__ ubot = P.u_bot; const TF* __restrict__ vbot = P.v_bot;
        double* __restrict__ dutot = P.sw.dutot;
        const int i = d.istart + vb.x*blockDim.x + threadIdx.x;
        const int j = d.jstart + vb.y*blockDim.y + threadIdx.y;
        if (i >= d.iend || j >= d.jend) return;
        const long long ii = 1, jj = d.icells;
        const long long ij = i + j*jj;
        const long long c = ij + (long long)d.kstart*d.ijcells;
        using CT = TF;
        auto U = [&](long long q) { return CT(u[q]); };
        auto V = [&](long long q) { return CT(v[q]); };
        const CT h = CT(0.5);
        const CT uf = CT(1./9)*(
              h*U(c-ii-jj) + U(c-jj) + U(c+ii-jj) + h*U(c+2*ii-jj)
            + h*U(c-ii   ) + U(c   ) + U(c+ii   ) + h*U(c+2*ii   )
            + h*U(c-ii+jj) + U(c+jj) + U(c+ii+jj) + h*U(c+2*ii+jj));
        const CT vf = CT(1./9)*(
              h*V(c-ii-jj) + V(c-ii) + V(c-ii+jj) + h*V(c-ii+2*jj)
            + h*V(c   -jj) + V(c   ) + V(c   +jj) + h*V(c   +2*jj)
            + h*V(c+ii-jj) + V(c+ii) + V(c+ii+jj) + h*V(c+ii+2*jj));
        const CT du2 = sq(uf - h*(CT(ubot[ij]) + CT(ubot[ij+ii])))
                     + sq(vf - h*(CT(vbot[ij]) + CT(vbot[ij+jj])));
        dutot[ij] = to_d<CT>(fmax(pow(du2, CT(0.5)), CT(1.e-1)));
    }

    // The Monin-Obukhov functions of one cell, each evaluated once: the
    // similarity function phi of the stability branch feeds both the
    // integrated psi and the gradient (include/monin_obukhov.h:40-152).
    template<typename CT> struct MostCell { CT fm, fh, phim, phih; };

    template<typename CT>
    __device__ __forceinline__ MostCell<CT> most_cell(CT zsl, CT z0m, CT z0h, CT L)
    {
        MostCell<CT> r;
        const CT kappa = CT(KAPPA);
        const CT zeta = zsl/L;
        if (L <= CT(0))
        {
            const CT pm_s = phim_unstable(zeta), pm_0 = phim_unstable(z0m/L);
            const CT ph_s = phih_unstable(zeta), ph_0 = phih_unstable(z0h/L);
            const CT psim_s = CT(3)*log((CT(1) + CT(1)/pm_s)/CT(2)), psim_0 = CT(3)*log((CT(1) + CT(1)/pm_0)/CT(2));
            const CT psih_s = CT(3)*log((CT(1) + CT(1)/ph_s)/CT(2)), psih_0 = CT(3)*log((CT(1) + CT(1)/ph_0)/CT(2));
            r.fm = kappa/(log(zsl/z0m) - psim_s + psim_0);
            r.fh = kappa/(log(zsl/z0h) - psih_s + psih_0);
            r.phim = zeta <= CT(0) ? pm_s : CT(1) + CT(5)*zeta;
            r.phih = zeta <= CT(0) ? ph_s : (CT(1) + CT(4)*zeta)*(CT(1) + CT(4)*zeta);
        }
        else
        {
            r.fm = kappa/(log(zsl/z0m) - psim_stable(zeta) + psim_stable(z0m/L));
            r.fh = kappa/(log(zsl/z0h) - psih_stable(zeta) + psih_stable(z0h/L));
            r.phim = phim(zeta);
            r.phih = phih(zeta);
        }
        return r;
    }

    // Obukhov length and friction velocity, src/boundary_surface.cxx:55-160
    // (all cells; the neutral branch when there is no thermodynamics).
    template<typename TF>
    __device__ __forceinline__ void stability_body(const SurfP<TF>& P, const VBlock& vb)
    {
        const Dims& d = P.d;
        const SurfWork& sw = P.sw;
        const TF* __restrict__ s = P.s; const TF* __restrict__ s_bot = P.s_bot; const TF* __restrict__ s_flux = P.s_flux;
        const double zsl = P.zsl, z0m = P.z0m, thref_s = P.thref_s, threfh_s = P.threfh_s;
        const double thb_s = P.thb_s, thbh_s = P.thbh_s;
        const int thermo = P.thermo, thermo_bc = P.thermo_bc;
        const int n = vb.x*blockDim.x + threadIdx.x;
        if (n >= d.ijcells) return;
        using CT = TF;
        const CT du = from_d<CT>(sw.dutot[n]);
        const CT zs = CT(zsl);
        CT L;
        if (!thermo)
            L = CT(-DBIG);
        else if (thermo_bc == MHH_BC_FLUX)
        {
            const CT bfluxbot = CT(GRAV)/CT(threfh_s)*CT(s_flux[n]);
            const float Ri = (float)(CT(-KAPPA)*bfluxbot*zs/(du*du*du));
            L = zs/CT(find_zL(sw.zL, sw.f, &sw.nobuk[n], Ri));
        }
        else
        {
            // theta - thref in the scalar's storage units (thb = thref - offset).
            const CT b = CT(GRAV)/CT(thref_s)*(CT(s[n + (long long)d.kstart*d.ijcells]) - CT(thb_s));
            const CT bbot = CT(GRAV)/CT(threfh_s)*(CT(s_bot[n]) - CT(thbh_s));
            const CT db_ref = CT(GRAV)/CT(thref_s)*(CT(thref_s) - CT(threfh_s));
            const CT db = b - bbot + db_ref;
            const float Ri = (float)(CT(KAPPA)*db*zs/(du*du));
            L = zs/CT(find_zL(sw.zL, sw.f, &sw.nobuk[n], Ri));
        }
        const MostCell<CT> mc = most_cell<CT>(zs, CT(z0m), CT(sw.z0h), L);
        sw.obuk[n] = to_d<CT>(L);
        sw.ustar[n] = to_d<CT>(du*mc.fm);
        sw.fm[n] = to_d<CT>(mc.fm); sw.fh[n] = to_d<CT>(mc.fh);
        sw.phim[n] = to_d<CT>(mc.phim); sw.phih[n] = to_d<CT>(mc.phih);
    }

    // Momentum fluxes, src/boundary_surface.cxx:163-190 (interior).
    template<typename TF>
    __device__ __forceinline__ void surfm_body(const SurfP<TF>& P, const VBlock& vb)
    {
        const Dims& d = P.d;
        const SurfWork& sw = P.sw;
        const TF* __restrict__ u = P.u; const TF* __restrict__ v = P.v;
        const TF* __restrict__ ubot = P.u_bot; const TF* __restrict__ vbot = P.v_bot;
        TF* __restrict__ uflux = P.u_flux; TF* __restrict__ vflux = P.v_flux;
        const int i = d.istart + vb.x*blockDim.x + threadIdx.x;
        const int j = d.jstart + vb.y*blockDim.y + threadIdx.y;
        if (i >= d.iend || j >= d.jend) return;
        const long long ii = 1, jj = d.icells;
        const long long ij = i + j*jj;
        const long long c = ij + (long long)d.kstart*d.ijcells;
        using CT = TF;
        auto D = [&](const double* a, long long q) { return from_d<CT>(a[q]); };
        const CT fc = D(sw.ustar, ij)*D(sw.fm, ij);
        uflux[ij] = -(CT(u[c]) - CT(ubot[ij]))*CT(0.5)*(D(sw.ustar, ij-ii)*D(sw.fm, ij-ii) + fc);
        vflux[ij] = -(CT(v[c]) - CT(vbot[ij]))*CT(0.5)*(D(sw.ustar, ij-jj)*D(sw.fm, ij-jj) + fc);
    }

    // Surface gradients of u and v and the scalar surface value, gradient or
    // flux, src/boundary_surface.cxx:255-338 (all cells).
    template<typename TF>
    __device__ __forceinline__ void surf_grads_body(const SurfP<TF>& P, const VBlock& vb)
    {
        const Dims& d = P.d;
        const SurfWork& sw = P.sw;
        const TF* __restrict__ u = P.u; const TF* __restrict__ v = P.v;
        const TF* __restrict__ ubot = P.u_bot; const TF* __restrict__ vbot = P.v_bot;
        TF* __restrict__ ugrad = P.u_grad; TF* __restrict__ vgrad = P.v_grad;
        const TF* __restrict__ s = P.s; TF* __restrict__ sbot = P.s_bot; TF* __restrict__ sgrad = P.s_grad;
        TF* __restrict__ sflux = P.s_flux;
        const double zsl = P.zsl;
        const int thermo = P.thermo, thermo_bc = P.thermo_bc;
        const int n = vb.x*blockDim.x + threadIdx.x;
        if (n >= d.ijcells) return;
        const long long c = n + (long long)d.kstart*d.ijcells;
        using CT = TF;
        const CT z = CT(zsl);
        ugrad[n] = (CT(u[c]) - CT(ubot[n]))/z;
        vgrad[n] = (CT(v[c]) - CT(vbot[n]))/z;
        if (thermo)
        {
            const CT th = CT(s[c]);
            const CT us = from_d<CT>(sw.ustar[n]), fh = from_d<CT>(sw.fh[n]);
            if (thermo_bc == MHH_BC_DIRICHLET)
            {
                sflux[n] = -(th - CT(sbot[n]))*us*fh;
                sgrad[n] = (th - CT(sbot[n]))/z;
            }
            else
            {
                const CT bot = CT(sflux[n])/(us*fh) + th;
                sbot[n] = bot;
                sgrad[n] = (th - bot)/z;
            }
        }
    }

    // Monin-Obukhov gradients for the next viscosity, include/boundary_surface_kernels.h:180-238.
    template<typename TF>
    __device__ __forceinline__ void duvdz_body(const SurfP<TF>& P, const VBlock& vb)
    {
        const Dims& d = P.d;
        const SurfWork& sw = P.sw;
        const TF* __restrict__ u = P.u; const TF* __restrict__ v = P.v;
        const TF* __restrict__ ubot = P.u_bot; const TF* __restrict__ vbot = P.v_bot;
        const TF* __restrict__ sflux = P.s_flux;
        const double zsl = P.zsl, threfh_s = P.threfh_s;
        const int thermo = P.thermo;
        const int i = d.istart + vb.x*blockDim.x + threadIdx.x;
        const int j = d.jstart + vb.y*blockDim.y + threadIdx.y;
        if (i >= d.iend || j >= d.jend) return;
        const long long ii = 1, jj = d.icells;
        const long long ij = i + j*jj;
        const long long c = ij + (long long)d.kstart*d.ijcells;
        using CT = TF;
        const CT du_c = CT(0.5)*((CT(u[c]) - CT(ubot[ij])) + (CT(u[c+ii]) - CT(ubot[ij+ii])));
        const CT dv_c = CT(0.5)*((CT(v[c]) - CT(vbot[ij])) + (CT(v[c+jj]) - CT(vbot[ij+jj])));
        const CT us = from_d<CT>(sw.ustar[ij]);
        const CT fmv = from_d<CT>(sw.fm[ij]);
        const CT ufb = -du_c*us*fmv;
        const CT vfb = -dv_c*us*fmv;
        const CT ph = from_d<CT>(sw.phim[ij]);
        const CT kz = CT(KAPPA)*CT(zsl);
        sw.dudz[ij] = to_d<CT>(-ufb/(kz*us)*ph);
        sw.dvdz[ij] = to_d<CT>(-vfb/(kz*us)*ph);
        if (thermo)
        {
            const CT bfb = CT(GRAV)/CT(threfh_s)*CT(sflux[ij]);
            sw.dbdz[ij] = to_d<CT>(-bfb/(kz*us)*from_d<CT>(sw.phih[ij]));
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
        const SurfP<TF> P{d, sw, u, v, s, u_bot, v_bot, u_flux, v_flux, u_grad, v_grad, s_bot, s_flux, s_grad,
                          zsl, z0m, z0h, thref_s, threfh_s, sw.thb_s, sw.thbh_s, thermo, thermo_bc};
        launch_body<SurfP<TF>, dutot_body<TF>, 256>(g2, b2, 0, st, P);
        launch_cyclic2d<double>(sw.dutot, d, st);
        launch_body<SurfP<TF>, stability_body<TF>, 256>(dim3(nb), dim3(256), 0, st, P);
        launch_body<SurfP<TF>, surfm_body<TF>, 256>(g2, b2, 0, st, P);
        launch_cyclic2d<TF>(u_flux, d, st);
        launch_cyclic2d<TF>(v_flux, d, st);
        launch_body<SurfP<TF>, surf_grads_body<TF>, 256>(dim3(nb), dim3(256), 0, st, P);
        launch_body<SurfP<TF>, duvdz_body<TF>, 256>(g2, b2, 0, st, P);
        count_launch(5);
    }

    template void launch_surface<double>(const Dims&, const Prof<double>&, const SurfWork&, const double*, const double*,
        const double*, double*, double*, double*, double*, double*, double*, double*, double*, double*,
        int, int, double, double, cudaStream_t);
    template void launch_surface<float>(const Dims&, const Prof<float>&, const SurfWork&, const float*, const float*,
        const float*, float*, float*, float*, float*, float*, float*, float*, float*, float*,
        int, int, double, double, cudaStream_t);
}
