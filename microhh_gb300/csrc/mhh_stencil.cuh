// mhh_stencil.cuh -- per-cell tendency terms of the LES/DNS time step.
//
// Each function returns the contribution of one term at one interior cell of
// the ghost-cell layout; the kernels in mhh_stencil.cu sum them.  The
// arithmetic follows the reference CPU kernels cited per function.
#pragma once

#include "mhh_common.cuh"

namespace mhh
{
    // Order of the vertical flux through half level kf for a field at full
    // levels (walls at kstart and kend carry no flux; 2nd order next to them,
    // then 4th order; 6th order inside), src/advec_2i5.cxx:219-299.
    __device__ __forceinline__ int face_order_full(const Dims& d, int kf)
    {
        if (kf <= d.kstart || kf >= d.kend) return 0;
        if (kf == d.kstart+1 || kf == d.kend-1) return 2;
        if (kf == d.kstart+2 || kf == d.kend-2) return 4;
        return 6;
    }

    // Order of the flux of w through full level k, src/advec_2i5.cxx:515-578.
    __device__ __forceinline__ int face_order_w(const Dims& d, int k)
    {
        if (k == d.kstart || k == d.kend-1) return 2;
        if (k == d.kstart+1 || k == d.kend-2) return 4;
        return 6;
    }

    // Upwind-biased flux a_face * wf through the face below cell c.
    template<typename TF>
    __device__ __forceinline__ TF vflux(const TF* a, long long c, long long kk, TF wf, int order)
    {
        if (order == 6) return wf*f6(a, c, kk) - fabs(wf)*f5(a, c, kk);
        if (order == 4) return wf*f4(a, c, kk) - fabs(wf)*f3(a, c, kk);
        return wf*f2(a, c, kk);
    }

    // Horizontal 6th-order flux divergence plus 5th-order dissipation of a
    // along x and y with face velocities ue, uw (x) and vn, vs (y).
    template<typename TF>
    __device__ __forceinline__ TF hadv_2i5(const TF* a, long long c, long long jj,
                                           TF ue, TF uw, TF vn, TF vs, TF dxi, TF dyi)
    {
        return - (ue*f6(a, c+1, 1LL) - uw*f6(a, c, 1LL))*dxi
               + (fabs(ue)*f5(a, c+1, 1LL) - fabs(uw)*f5(a, c, 1LL))*dxi
               - (vn*f6(a, c+jj, jj) - vs*f6(a, c, jj))*dyi
               + (fabs(vn)*f5(a, c+jj, jj) - fabs(vs)*f5(a, c, jj))*dyi;
    }

    // ---- Advec_2i5, src/advec_2i5.cxx:150-728 ----------------------------

    template<typename TF>
    __device__ __forceinline__ TF advec_2i5_u(const Dims& d, const Prof<TF>& pr, const TF* u, const TF* v, const TF* w,
                                              long long c, int k, TF dxi, TF dyi)
    {
        const long long ii = 1, jj = d.icells, kk = d.ijcells;
        TF t = hadv_2i5(u, c, jj,
                        i2(ld(u, c), ld(u, c+ii)), i2(ld(u, c-ii), ld(u, c)),
                        i2(ld(v, c-ii+jj), ld(v, c+jj)), i2(ld(v, c-ii), ld(v, c)), dxi, dyi);
        const int ot = face_order_full(d, k+1), ob = face_order_full(d, k);
        const TF ftop = ot ? ld(pr.rhorefh, k+1)*vflux(u, c+kk, kk, i2(ld(w, c-ii+kk), ld(w, c+kk)), ot) : TF(0);
        const TF fbot = ob ? ld(pr.rhorefh, k  )*vflux(u, c   , kk, i2(ld(w, c-ii   ), ld(w, c   )), ob) : TF(0);
        return t - (ftop - fbot) / ld(pr.rhoref, k) * ld(pr.dzi, k);
    }

    template<typename TF>
    __device__ __forceinline__ TF advec_2i5_v(const Dims& d, const Prof<TF>& pr, const TF* u, const TF* v, const TF* w,
                                              long long c, int k, TF dxi, TF dyi)
    {
        const long long ii = 1, jj = d.icells, kk = d.ijcells;
        TF t = hadv_2i5(v, c, jj,
                        i2(ld(u, c+ii-jj), ld(u, c+ii)), i2(ld(u, c-jj), ld(u, c)),
                        i2(ld(v, c), ld(v, c+jj)), i2(ld(v, c-jj), ld(v, c)), dxi, dyi);
        const int ot = face_order_full(d, k+1), ob = face_order_full(d, k);
        const TF ftop = ot ? ld(pr.rhorefh, k+1)*vflux(v, c+kk, kk, i2(ld(w, c-jj+kk), ld(w, c+kk)), ot) : TF(0);
        const TF fbot = ob ? ld(pr.rhorefh, k  )*vflux(v, c   , kk, i2(ld(w, c-jj   ), ld(w, c   )), ob) : TF(0);
        return t - (ftop - fbot) / ld(pr.rhoref, k) * ld(pr.dzi, k);
    }

    // Only for kstart < k < kend.
    template<typename TF>
    __device__ __forceinline__ TF advec_2i5_w(const Dims& d, const Prof<TF>& pr, const TF* u, const TF* v, const TF* w,
                                              long long c, int k, TF dxi, TF dyi)
    {
        const long long ii = 1, jj = d.icells, kk = d.ijcells;
        TF t = hadv_2i5(w, c, jj,
                        i2(ld(u, c+ii-kk), ld(u, c+ii)), i2(ld(u, c-kk), ld(u, c)),
                        i2(ld(v, c+jj-kk), ld(v, c+jj)), i2(ld(v, c-kk), ld(v, c)), dxi, dyi);
        const TF ftop = ld(pr.rhoref, k  )*vflux(w, c+kk, kk, i2(ld(w, c), ld(w, c+kk)), face_order_w(d, k));
        const TF fbot = ld(pr.rhoref, k-1)*vflux(w, c   , kk, i2(ld(w, c-kk), ld(w, c)), face_order_w(d, k-1));
        return t - (ftop - fbot) / ld(pr.rhorefh, k) * ld(pr.dzhi, k);
    }

    template<typename TF>
    __device__ __forceinline__ TF advec_2i5_s(const Dims& d, const Prof<TF>& pr, const TF* s, const TF* u, const TF* v,
                                              const TF* w, long long c, int k, TF dxi, TF dyi)
    {
        const long long ii = 1, jj = d.icells, kk = d.ijcells;
        TF t = hadv_2i5(s, c, jj, ld(u, c+ii), ld(u, c), ld(v, c+jj), ld(v, c), dxi, dyi);
        const int ot = face_order_full(d, k+1), ob = face_order_full(d, k);
        const TF ftop = ot ? ld(pr.rhorefh, k+1)*vflux(s, c+kk, kk, ld(w, c+kk), ot) : TF(0);
        const TF fbot = ob ? ld(pr.rhorefh, k  )*vflux(s, c   , kk, ld(w, c   ), ob) : TF(0);
        return t - (ftop - fbot) / ld(pr.rhoref, k) * ld(pr.dzi, k);
    }

    // ---- Flux limiter, include/advec_monotonic.h:28-219 -----------------
    // Koren (1993): the face value is the upwind value plus half the limited
    // upwind difference, phi(r) = max(0, min(2r, (1 + 2r)/3, 2)), r the ratio
    // of the downwind to the upwind difference; the denominator keeps at
    // least machine epsilon (of TF) in magnitude.

    template<typename TF> __device__ __forceinline__ TF tf_epsilon();
    template<> __device__ __forceinline__ double tf_epsilon<double>() { return 2.220446049250313080847e-16; }  // 2^-52
    template<> __device__ __forceinline__ float tf_epsilon<float>() { return 1.1920928955078125e-7f; }        // 2^-23

    template<typename TF>
    __device__ __forceinline__ TF koren_face(TF up, TF upup, TF down)
    {
        const TF dd = up - upup;
        const TF ad = fabs(dd);
        // max(a, b) as (a < b ? b : a), min(a, b) as (b < a ? b : a).
        const TF denom = copysign(TF(1), dd)*(ad < tf_epsilon<TF>() ? tf_epsilon<TF>() : ad);
        const TF two_r = TF(2)*(down - up)/denom;
        const TF third = TF(1./3.)*(TF(1) + two_r);
        const TF lim = TF(2) < third ? TF(2) : third;
        const TF lo = lim < two_r ? lim : two_r;
        const TF phi = TF(0) < lo ? lo : TF(0);
        return up + TF(0.5)*phi*(up - upup);
    }

    // Limited flux vel * a through the low-side face of cell c along stride
    // st.  side -1: first face above the bottom wall (upward flow carries the
    // upwind value unlimited); +1: last face below the top wall (likewise
    // for downward flow); 0: elsewhere.
    template<typename TF>
    __device__ __forceinline__ TF flux_koren(const TF* a, long long c, long long st, TF vel, int side)
    {
        if (vel >= TF(0))
            return side < 0 ? vel*ld(a, c-st) : vel*koren_face(ld(a, c-st), ld(a, c-2*st), ld(a, c));
        return side > 0 ? vel*ld(a, c) : vel*koren_face(ld(a, c), ld(a, c+st), ld(a, c-st));
    }

    // Scalar advection with the limiter in x, y and z; no flux through the
    // walls (advec_s_lim, include/advec_monotonic.h:101-219; ktot >= 4).
    template<typename TF>
    __device__ __forceinline__ TF advec_2i5_s_lim(const Dims& d, const Prof<TF>& pr, const TF* s, const TF* u,
                                                  const TF* v, const TF* w, long long c, int k, TF dxi, TF dyi)
    {
        const long long jj = d.icells, kk = d.ijcells;
        auto side = [&](int kf) { return kf == d.kstart+1 ? -1 : (kf == d.kend-1 ? 1 : 0); };
        const int sidet = side(k+1), sideb = side(k);
        const TF ftop = k+1 < d.kend ? flux_koren(s, c+kk, kk, ld(w, c+kk), sidet) : TF(0);
        const TF fbot = k > d.kstart ? flux_koren(s, c, kk, ld(w, c), sideb) : TF(0);
        return - (flux_koren(s, c+1, 1LL, ld(u, c+1), 0) - flux_koren(s, c, 1LL, ld(u, c), 0))*dxi
               - (flux_koren(s, c+jj, jj, ld(v, c+jj), 0) - flux_koren(s, c, jj, ld(v, c), 0))*dyi
               - (ld(pr.rhorefh, k+1)*ftop - ld(pr.rhorefh, k)*fbot) / ld(pr.rhoref, k) * ld(pr.dzi, k);
    }

    // ---- Advec_2, src/advec_2.cxx:80-202 ---------------------------------

    template<typename TF>
    __device__ __forceinline__ TF advec_2_u(const Dims& d, const Prof<TF>& pr, const TF* u, const TF* v, const TF* w,
                                            long long c, int k, TF dxi, TF dyi)
    {
        const long long ii = 1, jj = d.icells, kk = d.ijcells;
        return - (i2(ld(u, c), ld(u, c+ii))*i2(ld(u, c), ld(u, c+ii)) - i2(ld(u, c-ii), ld(u, c))*i2(ld(u, c-ii), ld(u, c)))*dxi
               - (i2(ld(v, c-ii+jj), ld(v, c+jj))*i2(ld(u, c), ld(u, c+jj)) - i2(ld(v, c-ii), ld(v, c))*i2(ld(u, c-jj), ld(u, c)))*dyi
               - (ld(pr.rhorefh, k+1)*i2(ld(w, c-ii+kk), ld(w, c+kk))*i2(ld(u, c), ld(u, c+kk))
                - ld(pr.rhorefh, k  )*i2(ld(w, c-ii), ld(w, c))*i2(ld(u, c-kk), ld(u, c))) / ld(pr.rhoref, k)*ld(pr.dzi, k);
    }

    template<typename TF>
    __device__ __forceinline__ TF advec_2_v(const Dims& d, const Prof<TF>& pr, const TF* u, const TF* v, const TF* w,
                                            long long c, int k, TF dxi, TF dyi)
    {
        const long long ii = 1, jj = d.icells, kk = d.ijcells;
        return - (i2(ld(u, c+ii-jj), ld(u, c+ii))*i2(ld(v, c), ld(v, c+ii)) - i2(ld(u, c-jj), ld(u, c))*i2(ld(v, c-ii), ld(v, c)))*dxi
               - (i2(ld(v, c), ld(v, c+jj))*i2(ld(v, c), ld(v, c+jj)) - i2(ld(v, c-jj), ld(v, c))*i2(ld(v, c-jj), ld(v, c)))*dyi
               - (ld(pr.rhorefh, k+1)*i2(ld(w, c-jj+kk), ld(w, c+kk))*i2(ld(v, c), ld(v, c+kk))
                - ld(pr.rhorefh, k  )*i2(ld(w, c-jj), ld(w, c))*i2(ld(v, c-kk), ld(v, c))) / ld(pr.rhoref, k)*ld(pr.dzi, k);
    }

    template<typename TF>
    __device__ __forceinline__ TF advec_2_w(const Dims& d, const Prof<TF>& pr, const TF* u, const TF* v, const TF* w,
                                            long long c, int k, TF dxi, TF dyi)
    {
        const long long ii = 1, jj = d.icells, kk = d.ijcells;
        return - (i2(ld(u, c+ii-kk), ld(u, c+ii))*i2(ld(w, c), ld(w, c+ii)) - i2(ld(u, c-kk), ld(u, c))*i2(ld(w, c-ii), ld(w, c)))*dxi
               - (i2(ld(v, c+jj-kk), ld(v, c+jj))*i2(ld(w, c), ld(w, c+jj)) - i2(ld(v, c-kk), ld(v, c))*i2(ld(w, c-jj), ld(w, c)))*dyi
               - (ld(pr.rhoref, k  )*i2(ld(w, c), ld(w, c+kk))*i2(ld(w, c), ld(w, c+kk))
                - ld(pr.rhoref, k-1)*i2(ld(w, c-kk), ld(w, c))*i2(ld(w, c-kk), ld(w, c))) / ld(pr.rhorefh, k)*ld(pr.dzhi, k);
    }

    template<typename TF>
    __device__ __forceinline__ TF advec_2_s(const Dims& d, const Prof<TF>& pr, const TF* s, const TF* u, const TF* v,
                                            const TF* w, long long c, int k, TF dxi, TF dyi)
    {
        const long long ii = 1, jj = d.icells, kk = d.ijcells;
        return - (ld(u, c+ii)*i2(ld(s, c), ld(s, c+ii)) - ld(u, c)*i2(ld(s, c-ii), ld(s, c)))*dxi
               - (ld(v, c+jj)*i2(ld(s, c), ld(s, c+jj)) - ld(v, c)*i2(ld(s, c-jj), ld(s, c)))*dyi
               - (ld(pr.rhorefh, k+1)*ld(w, c+kk)*i2(ld(s, c), ld(s, c+kk))
                - ld(pr.rhorefh, k  )*ld(w, c   )*i2(ld(s, c-kk), ld(s, c))) / ld(pr.rhoref, k)*ld(pr.dzi, k);
    }

    // ---- Smagorinsky diffusion, include/diff_kernels.h:144-484 -------------
    // With the surface model (surf) the levels kstart and kend-1 take the wall
    // flux from the 2-D flux arrays instead of the ghost cells.

    template<typename TF>
    __device__ __forceinline__ TF diff_smag2_u(const Dims& d, const Prof<TF>& pr, const TF* u, const TF* v, const TF* w,
                                               const TF* ev, const TF* fbot_a, const TF* ftop_a, bool surf,
                                               long long c, long long ij, int k, TF dxi, TF dyi, TF visc)
    {
        const long long ii = 1, jj = d.icells, kk = d.ijcells;
        const TF e_e = ld(ev, c) + visc;
        const TF e_w = ld(ev, c-ii) + visc;
        const TF e_n = TF(0.25)*(ld(ev, c-ii) + ld(ev, c) + ld(ev, c-ii+jj) + ld(ev, c+jj)) + visc;
        const TF e_s = TF(0.25)*(ld(ev, c-ii-jj) + ld(ev, c-jj) + ld(ev, c-ii) + ld(ev, c)) + visc;
        TF ftop, fbot;
        if (surf && k == d.kend-1) ftop = -ld(pr.rhorefh, k+1)*ld(ftop_a, ij);
        else
        {
            const TF e_t = TF(0.25)*(ld(ev, c-ii) + ld(ev, c) + ld(ev, c-ii+kk) + ld(ev, c+kk)) + visc;
            ftop = ld(pr.rhorefh, k+1)*e_t*((ld(u, c+kk)-ld(u, c))*ld(pr.dzhi, k+1) + (ld(w, c+kk)-ld(w, c-ii+kk))*dxi);
        }
        if (surf && k == d.kstart) fbot = -ld(pr.rhorefh, k)*ld(fbot_a, ij);
        else
        {
            const TF e_b = TF(0.25)*(ld(ev, c-ii-kk) + ld(ev, c-kk) + ld(ev, c-ii) + ld(ev, c)) + visc;
            fbot = ld(pr.rhorefh, k)*e_b*((ld(u, c)-ld(u, c-kk))*ld(pr.dzhi, k) + (ld(w, c)-ld(w, c-ii))*dxi);
        }
        return (e_e*(ld(u, c+ii)-ld(u, c))*dxi - e_w*(ld(u, c)-ld(u, c-ii))*dxi)*TF(2)*dxi
             + (e_n*((ld(u, c+jj)-ld(u, c))*dyi + (ld(v, c+jj)-ld(v, c-ii+jj))*dxi)
              - e_s*((ld(u, c)-ld(u, c-jj))*dyi + (ld(v, c)-ld(v, c-ii))*dxi))*dyi
             + (ftop - fbot)/ld(pr.rhoref, k)*ld(pr.dzi, k);
    }

    template<typename TF>
    __device__ __forceinline__ TF diff_smag2_v(const Dims& d, const Prof<TF>& pr, const TF* u, const TF* v, const TF* w,
                                               const TF* ev, const TF* fbot_a, const TF* ftop_a, bool surf,
                                               long long c, long long ij, int k, TF dxi, TF dyi, TF visc)
    {
        const long long ii = 1, jj = d.icells, kk = d.ijcells;
        const TF e_e = TF(0.25)*(ld(ev, c-jj) + ld(ev, c) + ld(ev, c+ii-jj) + ld(ev, c+ii)) + visc;
        const TF e_w = TF(0.25)*(ld(ev, c-ii-jj) + ld(ev, c-ii) + ld(ev, c-jj) + ld(ev, c)) + visc;
        const TF e_n = ld(ev, c) + visc;
        const TF e_s = ld(ev, c-jj) + visc;
        TF ftop, fbot;
        if (surf && k == d.kend-1) ftop = -ld(pr.rhorefh, k+1)*ld(ftop_a, ij);
        else
        {
            const TF e_t = TF(0.25)*(ld(ev, c-jj) + ld(ev, c) + ld(ev, c+kk-jj) + ld(ev, c+kk)) + visc;
            ftop = ld(pr.rhorefh, k+1)*e_t*((ld(v, c+kk)-ld(v, c))*ld(pr.dzhi, k+1) + (ld(w, c+kk)-ld(w, c-jj+kk))*dyi);
        }
        if (surf && k == d.kstart) fbot = -ld(pr.rhorefh, k)*ld(fbot_a, ij);
        else
        {
            const TF e_b = TF(0.25)*(ld(ev, c-kk-jj) + ld(ev, c-kk) + ld(ev, c-jj) + ld(ev, c)) + visc;
            fbot = ld(pr.rhorefh, k)*e_b*((ld(v, c)-ld(v, c-kk))*ld(pr.dzhi, k) + (ld(w, c)-ld(w, c-jj))*dyi);
        }
        return (e_e*((ld(v, c+ii)-ld(v, c))*dxi + (ld(u, c+ii)-ld(u, c+ii-jj))*dyi)
              - e_w*((ld(v, c)-ld(v, c-ii))*dxi + (ld(u, c)-ld(u, c-jj))*dyi))*dxi
             + (e_n*(ld(v, c+jj)-ld(v, c))*dyi - e_s*(ld(v, c)-ld(v, c-jj))*dyi)*TF(2)*dyi
             + (ftop - fbot)/ld(pr.rhoref, k)*ld(pr.dzi, k);
    }

    // Only for kstart < k < kend.
    template<typename TF>
    __device__ __forceinline__ TF diff_smag2_w(const Dims& d, const Prof<TF>& pr, const TF* u, const TF* v, const TF* w,
                                               const TF* ev, long long c, int k, TF dxi, TF dyi, TF visc)
    {
        const long long ii = 1, jj = d.icells, kk = d.ijcells;
        const TF e_e = TF(0.25)*(ld(ev, c-kk) + ld(ev, c) + ld(ev, c+ii-kk) + ld(ev, c+ii)) + visc;
        const TF e_w = TF(0.25)*(ld(ev, c-ii-kk) + ld(ev, c-ii) + ld(ev, c-kk) + ld(ev, c)) + visc;
        const TF e_n = TF(0.25)*(ld(ev, c-kk) + ld(ev, c) + ld(ev, c+jj-kk) + ld(ev, c+jj)) + visc;
        const TF e_s = TF(0.25)*(ld(ev, c-jj-kk) + ld(ev, c-jj) + ld(ev, c-kk) + ld(ev, c)) + visc;
        const TF e_t = ld(ev, c) + visc;
        const TF e_b = ld(ev, c-kk) + visc;
        const TF dzhik = ld(pr.dzhi, k);
        return (e_e*((ld(w, c+ii)-ld(w, c))*dxi + (ld(u, c+ii)-ld(u, c+ii-kk))*dzhik)
              - e_w*((ld(w, c)-ld(w, c-ii))*dxi + (ld(u, c)-ld(u, c-kk))*dzhik))*dxi
             + (e_n*((ld(w, c+jj)-ld(w, c))*dyi + (ld(v, c+jj)-ld(v, c+jj-kk))*dzhik)
              - e_s*((ld(w, c)-ld(w, c-jj))*dyi + (ld(v, c)-ld(v, c-kk))*dzhik))*dyi
             + (ld(pr.rhoref, k)*e_t*(ld(w, c+kk)-ld(w, c))*ld(pr.dzi, k)
              - ld(pr.rhoref, k-1)*e_b*(ld(w, c)-ld(w, c-kk))*ld(pr.dzi, k-1)) / ld(pr.rhorefh, k)*TF(2)*dzhik;
    }

    template<typename TF>
    __device__ __forceinline__ TF diff_smag2_s(const Dims& d, const Prof<TF>& pr, const TF* a, const TF* ev,
                                               const TF* fbot_a, const TF* ftop_a, bool surf,
                                               long long c, long long ij, int k, TF dxidxi, TF dyidyi,
                                               TF tpri, TF visc)
    {
        const long long ii = 1, jj = d.icells, kk = d.ijcells;
        const TF e_e = TF(0.5)*(ld(ev, c) + ld(ev, c+ii))*tpri + visc;
        const TF e_w = TF(0.5)*(ld(ev, c-ii) + ld(ev, c))*tpri + visc;
        const TF e_n = TF(0.5)*(ld(ev, c) + ld(ev, c+jj))*tpri + visc;
        const TF e_s = TF(0.5)*(ld(ev, c-jj) + ld(ev, c))*tpri + visc;
        TF ftop, fbot;
        if (surf && k == d.kend-1) ftop = -ld(pr.rhorefh, k+1)*ld(ftop_a, ij);
        else
        {
            const TF e_t = TF(0.5)*(ld(ev, c) + ld(ev, c+kk))*tpri + visc;
            ftop = ld(pr.rhorefh, k+1)*e_t*(ld(a, c+kk)-ld(a, c))*ld(pr.dzhi, k+1);
        }
        if (surf && k == d.kstart) fbot = -ld(pr.rhorefh, k)*ld(fbot_a, ij);
        else
        {
            const TF e_b = TF(0.5)*(ld(ev, c-kk) + ld(ev, c))*tpri + visc;
            fbot = ld(pr.rhorefh, k)*e_b*(ld(a, c)-ld(a, c-kk))*ld(pr.dzhi, k);
        }
        return (e_e*(ld(a, c+ii)-ld(a, c)) - e_w*(ld(a, c)-ld(a, c-ii)))*dxidxi
             + (e_n*(ld(a, c+jj)-ld(a, c)) - e_s*(ld(a, c)-ld(a, c-jj)))*dyidyi
             + (ftop - fbot)/ld(pr.rhoref, k)*ld(pr.dzi, k);
    }

    // ---- Diff_2, src/diff_2.cxx:38-86 ------------------------------------
    // (dxidxi and dyidyi are double in the reference even for float fields;
    // here they take the kernel's precision so that float kernels stay off
    // the FP64 pipe.)

    template<typename TF>
    __device__ __forceinline__ TF diff_2_c(const Dims& d, const Prof<TF>& pr, const TF* a, long long c, int k,
                                           TF dxidxi, TF dyidyi, TF visc)
    {
        const long long ii = 1, jj = d.icells, kk = d.ijcells;
        const TF ac = ld(a, c);
        return visc*(((ld(a, c+ii)-ac) - (ac-ld(a, c-ii)))*dxidxi
                   + ((ld(a, c+jj)-ac) - (ac-ld(a, c-jj)))*dyidyi
                   + ((ld(a, c+kk)-ac)*ld(pr.dzhi, k+1) - (ac-ld(a, c-kk))*ld(pr.dzhi, k))*ld(pr.dzi, k));
    }

    template<typename TF>
    __device__ __forceinline__ TF diff_2_w(const Dims& d, const Prof<TF>& pr, const TF* w, long long c, int k,
                                           TF dxidxi, TF dyidyi, TF visc)
    {
        const long long ii = 1, jj = d.icells, kk = d.ijcells;
        const TF wc = ld(w, c);
        return visc*(((ld(w, c+ii)-wc) - (wc-ld(w, c-ii)))*dxidxi
                   + ((ld(w, c+jj)-wc) - (wc-ld(w, c-jj)))*dyidyi
                   + ((ld(w, c+kk)-wc)*ld(pr.dzi, k) - (wc-ld(w, c-kk))*ld(pr.dzi, k-1))*ld(pr.dzhi, k));
    }
}
