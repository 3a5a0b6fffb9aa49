// mhh_stencil.cu -- grid-point kernels of the LES/DNS time step: periodic and
// wall ghost cells, Smagorinsky viscosity, the fused tendency kernel
// (advection + diffusion + buoyancy + forcing), the pressure-gradient + RK3
// update and the CFL / diffusion-number / divergence reductions.
#include <type_traits>

#include "mhh_kernels.cuh"
#include "mhh_batchable.cuh"
#include "mhh_stencil.cuh"

namespace mhh
{
    // ---------------------------------------------------------------------
    // Periodic ghost cells, src/boundary_cyclic.cxx:370-440.  A ghost cell
    // (i,j) takes the interior value at the periodic image of (i,j); this
    // equals the reference's east-west-then-north-south copy, corners
    // included, and reads interior cells only.
    // ---------------------------------------------------------------------
    template<typename TF> struct CyclicP { FieldList<TF> fl; Dims d; int edges; };

    template<typename TF>
    __device__ __forceinline__ void cyclic_body(const CyclicP<TF>& P, const VBlock& vb)
    {
        const FieldList<TF>& fl = P.fl;
        const Dims& d = P.d;
        const int edges = P.edges;
        const int nghost_i = 2*d.igc, nghost_j = 2*d.jgc;
        // Work items: the ghost columns (all j) and the ghost rows: interior i
        // when the columns are filled too, every i for a north-south-only fill
        // (src/boundary_cyclic.cxx:404-422 copies whole rows).
        const int rowlen = (edges & 1) ? d.itot : d.icells;
        const int row0 = (edges & 1) ? d.istart : 0;
        const long long ncol = (long long)nghost_i*d.jcells;
        const long long nrow = (long long)nghost_j*rowlen;
        const long long nitem = ((edges & 1) ? ncol : 0) + ((edges & 2) ? nrow : 0);
        const int k = vb.y;
        for (long long n = vb.x*(long long)blockDim.x + threadIdx.x; n < nitem; n += (long long)vb.gx*blockDim.x)
        {
            int i, j;
            long long m = n;
            if ((edges & 1) && m < ncol)
            {
                j = (int)(m / nghost_i);
                const int g = (int)(m % nghost_i);
                i = g < d.igc ? g : d.iend + (g - d.igc);
            }
            else
            {
                if (edges & 1) m -= ncol;
                const int g = (int)(m / rowlen);
                i = row0 + (int)(m % rowlen);
                j = g < d.jgc ? g : d.jend + (g - d.jgc);
            }
            int si = i, sj = j;
            if (edges & 1)
            {
                if (i < d.istart) si = i + d.itot;
                else if (i >= d.iend) si = i - d.itot;
            }
            if (edges & 2)
            {
                if (j < d.jstart) sj = j + d.jtot;
                else if (j >= d.jend) sj = j - d.jtot;
            }
            const long long dst = ijk(d, i, j, k), src = ijk(d, si, sj, k);
            for (int f=0; f<fl.n; ++f)
                fl.p[f][dst] = fl.p[f][src];
        }
    }

    template<typename TF>
    void launch_cyclic(const FieldList<TF>& fl, const Dims& d, int edges, cudaStream_t s)
    {
        const long long nitem = 2LL*d.igc*d.jcells + 2LL*d.jgc*d.icells;
        const int threads = 128;
        int bx = (int)((nitem + threads - 1) / threads);
        if (bx > 64) bx = 64;
        dim3 grid(bx, d.kcells);
        launch_body<CyclicP<TF>, cyclic_body<TF>, 128>(grid, dim3(threads), 0, s, CyclicP<TF>{fl, d, edges});
        count_launch();
    }

    // Periodic fill of a 2-D array (icells*jcells).
    template<typename TF> struct Cyclic2P { TF* a; Dims d; };

    template<typename TF>
    __device__ __forceinline__ void cyclic2d_body(const Cyclic2P<TF>& P, const VBlock& vb)
    {
        TF* a = P.a;
        const Dims& d = P.d;
        const int n = vb.x*blockDim.x + threadIdx.x;
        if (n >= d.ijcells) return;
        const int i = n % d.icells, j = n / d.icells;
        if (i >= d.istart && i < d.iend && j >= d.jstart && j < d.jend) return;
        int si = i, sj = j;
        if (i < d.istart) si += d.itot; else if (i >= d.iend) si -= d.itot;
        if (j < d.jstart) sj += d.jtot; else if (j >= d.jend) sj -= d.jtot;
        a[n] = a[si + sj*d.icells];
    }

    template<typename TF>
    void launch_cyclic2d(TF* a, const Dims& d, cudaStream_t s)
    {
        launch_body<Cyclic2P<TF>, cyclic2d_body<TF>, 256>(dim3((d.ijcells + 255)/256), dim3(256), 0, s, Cyclic2P<TF>{a, d});
        count_launch();
    }

    // ---------------------------------------------------------------------
    // Homogeneous boundary values, src/boundary.cxx:50-100.
    // ---------------------------------------------------------------------
    template<typename TF>
    __global__ void k_set_bc(TF* val, TF* grad, TF* flux, int type, TF aval, TF visc, int set_flux_grad, int n)
    {
        const int q = blockIdx.x*blockDim.x + threadIdx.x;
        if (q >= n) return;
        if (type == MHH_BC_DIRICHLET) val[q] = aval;
        else if (type == MHH_BC_NEUMANN) { grad[q] = aval; if (set_flux_grad) flux[q] = -aval*visc; }
        else if (type == MHH_BC_FLUX) { flux[q] = aval; if (set_flux_grad) grad[q] = -aval/visc; }
    }

    template<typename TF>
    void launch_set_bc(TF* val, TF* grad, TF* flux, int type, double aval, double visc, int sfg, const Dims& d, cudaStream_t s)
    {
        k_set_bc<TF><<<(d.ijcells + 255)/256, 256, 0, s>>>(val, grad, flux, type, TF(aval), TF(visc), sfg, d.ijcells);
        count_launch();
    }

    // ---------------------------------------------------------------------
    // Wall ghost levels, 2nd order, src/boundary.cxx:700-760.
    // ---------------------------------------------------------------------
    template<typename TF> struct GhostP { GhostList<TF> gl; Dims d; const TF* dzh; };

    template<typename TF>
    __device__ __forceinline__ void ghost_body(const GhostP<TF>& P, const VBlock& vb)
    {
        const GhostList<TF>& gl = P.gl;
        const Dims& d = P.d;
        const TF* dzh = P.dzh;
        const int n = vb.x*blockDim.x + threadIdx.x;
        if (n >= d.ijcells) return;
        const TF dzhb = dzh[d.kstart], dzht = dzh[d.kend];
        for (int f=0; f<gl.n; ++f)
        {
            TF* a = gl.a[f];
            const long long cb = n + (long long)d.kstart*d.ijcells;
            const long long ct = n + (long long)(d.kend-1)*d.ijcells;
            if (gl.bot_type[f] == MHH_BC_DIRICHLET)
                a[cb - d.ijcells] = TF(2)*gl.abot[f][n] - a[cb];
            else
                a[cb - d.ijcells] = -gl.agradbot[f][n]*dzhb + a[cb];
            if (gl.top_type[f] == MHH_BC_DIRICHLET)
                a[ct + d.ijcells] = TF(2)*gl.atop[f][n] - a[ct];
            else
                a[ct + d.ijcells] = gl.agradtop[f][n]*dzht + a[ct];
        }
    }

    template<typename TF>
    void launch_ghost(const GhostList<TF>& gl, const Dims& d, const TF* dzh, cudaStream_t s)
    {
        launch_body<GhostP<TF>, ghost_body<TF>, 256>(dim3((d.ijcells + 255)/256), dim3(256), 0, s, GhostP<TF>{gl, d, dzh});
        count_launch();
    }

    // ---------------------------------------------------------------------
    // Smagorinsky viscosity: strain rate (include/diff_kernels.h:34-142),
    // N2 of the dry thermodynamics (src/thermo_dry.cxx:64-75) and the eddy
    // viscosity (src/diff_smag2.cxx:47-269) in one pass; evisc holds the
    // result at interior cells.
    // ---------------------------------------------------------------------
    template<typename TF> struct ViscP
    {
        Dims d; Prof<TF> pr;
        const TF *u, *v, *w, *th;
        TF* evisc;
        const TF* mlen2;
        const double *dudz, *dvdz, *dbdz;
        TF cs, tpr, visc; int mason;
    };

    template<typename TF, bool SURF, bool THERMO>
    __device__ __forceinline__ void viscosity_body(const ViscP<TF>& P, const VBlock& vb)
    {
        const Dims& d = P.d;
        const Prof<TF>& pr = P.pr;
        const TF* __restrict__ u = P.u; const TF* __restrict__ v = P.v; const TF* __restrict__ w = P.w;
        const TF* __restrict__ th = P.th;
        TF* __restrict__ evisc = P.evisc;
        const TF* __restrict__ mlen2 = P.mlen2;
        const double* __restrict__ dudz = P.dudz; const double* __restrict__ dvdz = P.dvdz;
        const double* __restrict__ dbdz = P.dbdz;
        const TF cs = P.cs, tpr = P.tpr, visc = P.visc;
        const int mason = P.mason;
        const int i = d.istart + vb.x*blockDim.x + threadIdx.x;
        const int j = d.jstart + vb.y*blockDim.y + threadIdx.y;
        const int k = d.kstart + vb.z;
        if (i >= d.iend || j >= d.jend) return;
        const long long ii = 1, jj = d.icells, kk = d.ijcells;
        const long long c = ijk(d, i, j, k);
        const long long ij = i + (long long)j*jj;
        const TF dxi = dxi_of<TF>(d), dyi = dyi_of<TF>(d);

        TF acc = sq((ld(u, c+ii)-ld(u, c))*dxi)
               + sq((ld(v, c+jj)-ld(v, c))*dyi)
               + sq((ld(w, c+kk)-ld(w, c))*ld(pr.dzi, k))
               + TF(0.125)*sq((ld(u, c      )-ld(u, c   -jj))*dyi + (ld(v, c      )-ld(v, c-ii   ))*dxi)
               + TF(0.125)*sq((ld(u, c+ii   )-ld(u, c+ii-jj))*dyi + (ld(v, c+ii   )-ld(v, c      ))*dxi)
               + TF(0.125)*sq((ld(u, c   +jj)-ld(u, c      ))*dyi + (ld(v, c   +jj)-ld(v, c-ii+jj))*dxi)
               + TF(0.125)*sq((ld(u, c+ii+jj)-ld(u, c+ii   ))*dyi + (ld(v, c+ii+jj)-ld(v, c   +jj))*dxi);
        if (SURF && k == d.kstart)
        {
            acc += TF(0.5)*sq(TF(dudz[ij]))
                 + TF(0.125)*sq((ld(w, c      )-ld(w, c-ii   ))*dxi)
                 + TF(0.125)*sq((ld(w, c+ii   )-ld(w, c      ))*dxi)
                 + TF(0.125)*sq((ld(w, c   +kk)-ld(w, c-ii+kk))*dxi)
                 + TF(0.125)*sq((ld(w, c+ii+kk)-ld(w, c   +kk))*dxi)
                 + TF(0.5)*sq(TF(dvdz[ij]))
                 + TF(0.125)*sq((ld(w, c      )-ld(w, c-jj   ))*dyi)
                 + TF(0.125)*sq((ld(w, c+jj   )-ld(w, c      ))*dyi)
                 + TF(0.125)*sq((ld(w, c   +kk)-ld(w, c-jj+kk))*dyi)
                 + TF(0.125)*sq((ld(w, c+jj+kk)-ld(w, c   +kk))*dyi);
        }
        else
        {
            const TF dzb = ld(pr.dzhi, k), dzt = ld(pr.dzhi, k+1);
            acc += TF(0.125)*sq((ld(u, c      )-ld(u, c   -kk))*dzb + (ld(w, c      )-ld(w, c-ii   ))*dxi)
                 + TF(0.125)*sq((ld(u, c+ii   )-ld(u, c+ii-kk))*dzb + (ld(w, c+ii   )-ld(w, c      ))*dxi)
                 + TF(0.125)*sq((ld(u, c   +kk)-ld(u, c      ))*dzt + (ld(w, c   +kk)-ld(w, c-ii+kk))*dxi)
                 + TF(0.125)*sq((ld(u, c+ii+kk)-ld(u, c+ii   ))*dzt + (ld(w, c+ii+kk)-ld(w, c   +kk))*dxi)
                 + TF(0.125)*sq((ld(v, c      )-ld(v, c   -kk))*dzb + (ld(w, c      )-ld(w, c-jj   ))*dyi)
                 + TF(0.125)*sq((ld(v, c+jj   )-ld(v, c+jj-kk))*dzb + (ld(w, c+jj   )-ld(w, c      ))*dyi)
                 + TF(0.125)*sq((ld(v, c   +kk)-ld(v, c      ))*dzt + (ld(w, c   +kk)-ld(w, c-jj+kk))*dyi)
                 + TF(0.125)*sq((ld(v, c+jj+kk)-ld(v, c+jj   ))*dzt + (ld(w, c+jj+kk)-ld(w, c   +kk))*dyi);
        }
        const TF s2 = TF(2)*acc + TF(DSMALL);

        // The squared mixing length is precomputed per level (and with the
        // Mason wall correction per level and column when z0m is uniform).
        const TF ml2 = mlen2[k];
        TF ev;
        if (THERMO)
        {
            TF n2;
            if (SURF && k == d.kstart)
                n2 = TF(dbdz[ij]);
            else
                n2 = TF(GRAV)/ld(pr.thref, k)*TF(0.5)*(ld(th, c+kk) - ld(th, c-kk))*ld(pr.dzi, k);
            TF ratio = n2 / s2 / tpr;
            ratio = fmin(ratio, TF(1.-DSMALL));
            ev = ml2*sqrt(s2)*sqrt(TF(1)-ratio);
        }
        else if (SURF)
            ev = ml2*sqrt(s2);
        else
        {
            // Van Driest wall damping of the neutral resolved-wall case,
            // src/diff_smag2.cxx:74-101.
            const long long cb = ijk(d, i, j, d.kstart), ct = ijk(d, i, j, d.kend);
            const TF dzhb = ld(pr.dzhi, d.kstart), dzht = ld(pr.dzhi, d.kend);
            const TF utb = pow(sq(visc*(ld(u, cb)-ld(u, cb-kk))*dzhb) + sq(visc*(ld(v, cb)-ld(v, cb-kk))*dzhb), TF(0.25));
            const TF utt = pow(sq(visc*(ld(u, ct)-ld(u, ct-kk))*dzht) + sq(visc*(ld(v, ct)-ld(v, ct-kk))*dzht), TF(0.25));
            const TF zk = ld(pr.z, k);
            const TF fb = TF(1) - exp(-(zk*utb)/(TF(26)*visc));
            const TF ft = TF(1) - exp(-((zsize_of<TF>(d) - zk)*utt)/(TF(26)*visc));
            const TF fac = fmin(fb, ft);
            ev = sq(fac)*ml2*sqrt(s2);
        }
        evisc[c] = ev;
    }

    // Mirror of the eddy viscosity over resolved walls, src/diff_smag2.cxx:195-207.
    template<typename TF>
    struct MirrorP { TF* evisc; Dims d; };

    template<typename TF>
    __device__ __forceinline__ void evisc_mirror_body(const MirrorP<TF>& P, const VBlock& vb)
    {
        TF* evisc = P.evisc;
        const Dims& d = P.d;
        const int n = vb.x*blockDim.x + threadIdx.x;
        if (n >= d.ijcells) return;
        const long long cb = n + (long long)d.kstart*d.ijcells;
        const long long ct = n + (long long)(d.kend-1)*d.ijcells;
        evisc[cb - d.ijcells] = evisc[cb];
        evisc[ct + d.ijcells] = evisc[ct];
    }

    template<typename TF>
    void launch_viscosity(const Dims& d, const Prof<TF>& pr, const TF* u, const TF* v, const TF* w, const TF* th,
                          TF* evisc, const TF* mlen2, const double* dudz, const double* dvdz, const double* dbdz,
                          double cs, double tpr, double visc, int mason, bool surf, bool thermo, const KernelOpts& o,
                          cudaStream_t s)
    {
        dim3 block(32, 8);
        dim3 grid((d.itot + 31)/32, (d.jtot + 7)/8, d.ktot);
        // Automatic choice (-1): the plane-staged kernel in both precisions
        // (in double it keeps the reference's evisc expression).
        const int var = o.visc < 0 ? 1 : o.visc;
        const bool planes = var == 1 && launch_viscosity_planes<TF>(d, pr, u, v, w, th, evisc, mlen2, dudz, dvdz, dbdz,
                                                                    tpr, surf, thermo, o.visc_kchunk, s);
        if (!planes)
        {
            const ViscP<TF> P{d, pr, u, v, w, th, evisc, mlen2, dudz, dvdz, dbdz, TF(cs), TF(tpr), TF(visc), mason};
            if (surf && thermo) launch_body<ViscP<TF>, viscosity_body<TF, true, true>, 256>(grid, block, 0, s, P);
            else if (surf) launch_body<ViscP<TF>, viscosity_body<TF, true, false>, 256>(grid, block, 0, s, P);
            else if (thermo) launch_body<ViscP<TF>, viscosity_body<TF, false, true>, 256>(grid, block, 0, s, P);
            else launch_body<ViscP<TF>, viscosity_body<TF, false, false>, 256>(grid, block, 0, s, P);
            count_launch();
        }
        if (!surf)
        {
            launch_body<MirrorP<TF>, evisc_mirror_body<TF>, 256>(dim3((d.ijcells + 255)/256), dim3(256), 0, s,
                                                               MirrorP<TF>{evisc, d});
            count_launch();
        }
        FieldList<TF> fl; fl.n = 1; fl.p[0] = evisc;
        launch_cyclic(fl, d, 3, s);
    }

    // ---------------------------------------------------------------------
    // Fused tendency kernel: every term a substep adds to ut, vt, wt and st
    // before the pressure solve (thermo buoyancy, advection, diffusion,
    // large-scale pressure force), one interior cell per thread.
    // ---------------------------------------------------------------------
    template<typename TF> struct TendP { Dims d; Prof<TF> pr; TendArgs<TF> a; };

    template<typename TF, int ADV, int DIF, bool SURF, bool SCAL, bool BUOY, bool FORCE>
    __device__ __forceinline__ void tendency_body(const TendP<TF>& P, const VBlock& vb)
    {
        const Dims& d = P.d;
        const Prof<TF>& pr = P.pr;
        const TendArgs<TF>& a = P.a;
        const int i = d.istart + vb.x*blockDim.x + threadIdx.x;
        const int j = d.jstart + vb.y*blockDim.y + threadIdx.y;
        const int k = d.kstart + vb.z;
        if (i >= d.iend || j >= d.jend) return;
        const long long c = ijk(d, i, j, k);
        const long long ij = i + (long long)j*d.icells;
        const TF dxi = dxi_of<TF>(d), dyi = dyi_of<TF>(d);
        const TF* u = a.u; const TF* v = a.v; const TF* w = a.w;

        constexpr bool A2I5 = ADV == MHH_ADVEC_2I5 || ADV == ADVEC_2I5_LIM;
        // u
        {
            TF t = TF(0);
            if (A2I5) t += advec_2i5_u(d, pr, u, v, w, c, k, dxi, dyi);
            else if (ADV == MHH_ADVEC_2) t += advec_2_u(d, pr, u, v, w, c, k, dxi, dyi);
            if (DIF == MHH_DIFF_SMAG2) t += diff_smag2_u(d, pr, u, v, w, a.evisc, a.u_fluxbot, a.u_fluxtop, SURF, c, ij, k, dxi, dyi, a.visc);
            else if (DIF == MHH_DIFF_2) t += diff_2_c(d, pr, u, c, k, a.dxidxi_t, a.dyidyi_t, a.visc);
            if (FORCE) t += a.fbody;
            a.ut[c] += t;
        }
        // v
        {
            TF t = TF(0);
            if (A2I5) t += advec_2i5_v(d, pr, u, v, w, c, k, dxi, dyi);
            else if (ADV == MHH_ADVEC_2) t += advec_2_v(d, pr, u, v, w, c, k, dxi, dyi);
            if (DIF == MHH_DIFF_SMAG2) t += diff_smag2_v(d, pr, u, v, w, a.evisc, a.v_fluxbot, a.v_fluxtop, SURF, c, ij, k, dxi, dyi, a.visc);
            else if (DIF == MHH_DIFF_2) t += diff_2_c(d, pr, v, c, k, a.dxidxi_t, a.dyidyi_t, a.visc);
            a.vt[c] += t;
        }
        // w (half levels above the wall)
        if (k > d.kstart)
        {
            TF t = TF(0);
            if (BUOY) t += TF(GRAV)/ld(pr.threfh, k)*(i2(ld(a.s, c-d.ijcells), ld(a.s, c)) - ld(pr.thbh, k));
            if (A2I5) t += advec_2i5_w(d, pr, u, v, w, c, k, dxi, dyi);
            else if (ADV == MHH_ADVEC_2) t += advec_2_w(d, pr, u, v, w, c, k, dxi, dyi);
            if (DIF == MHH_DIFF_SMAG2) t += diff_smag2_w(d, pr, u, v, w, a.evisc, c, k, dxi, dyi, a.visc);
            else if (DIF == MHH_DIFF_2) t += diff_2_w(d, pr, w, c, k, a.dxidxi_t, a.dyidyi_t, a.visc);
            a.wt[c] += t;
        }
        // scalar
        if (SCAL)
        {
            TF t = TF(0);
            if (ADV == ADVEC_2I5_LIM) t += advec_2i5_s_lim(d, pr, a.s, u, v, w, c, k, dxi, dyi);
            else if (ADV == MHH_ADVEC_2I5) t += advec_2i5_s(d, pr, a.s, u, v, w, c, k, dxi, dyi);
            else if (ADV == MHH_ADVEC_2) t += advec_2_s(d, pr, a.s, u, v, w, c, k, dxi, dyi);
            if (DIF == MHH_DIFF_SMAG2)
                t += diff_smag2_s(d, pr, a.s, a.evisc, a.s_fluxbot, a.s_fluxtop, SURF, c, ij, k,
                                  a.dxidxi_t, a.dyidyi_t, a.tpri, a.svisc);
            else if (DIF == MHH_DIFF_2) t += diff_2_c(d, pr, a.s, c, k, a.dxidxi_t, a.dyidyi_t, a.svisc);
            a.st[c] += t;
        }
    }

    template<typename TF, int ADV, int DIF, bool SURF, bool SCAL, bool BUOY, bool FORCE>
    static void launch_tend_t(const Dims& d, const Prof<TF>& pr, const TendArgs<TF>& a, cudaStream_t s)
    {
        dim3 block(32, 8);
        dim3 grid((d.itot + 31)/32, (d.jtot + 7)/8, d.ktot);
        launch_body<TendP<TF>, tendency_body<TF, ADV, DIF, SURF, SCAL, BUOY, FORCE>, 256>(grid, block, 0, s, TendP<TF>{d, pr, a});
        count_launch();
    }

    // Advec_2i5 with the limited scalar: only the combinations with a scalar.
    template<typename TF, int DIF>
    static void launch_tend_lim(const Dims& d, const Prof<TF>& pr, const TendArgs<TF>& a,
                                bool surf, bool buoy, bool force, cudaStream_t s)
    {
        const int mask = (surf ? 4 : 0) | (buoy ? 2 : 0) | (force ? 1 : 0);
        switch (mask)
        {
#define MHH_TEND_CASE(M) case M: launch_tend_t<TF, ADVEC_2I5_LIM, DIF, ((M) & 4) != 0, true, ((M) & 2) != 0, ((M) & 1) != 0>(d, pr, a, s); break;
            MHH_TEND_CASE(0) MHH_TEND_CASE(1) MHH_TEND_CASE(2) MHH_TEND_CASE(3)
            MHH_TEND_CASE(4) MHH_TEND_CASE(5) MHH_TEND_CASE(6) MHH_TEND_CASE(7)
#undef MHH_TEND_CASE
        }
    }

    template<typename TF, int ADV, int DIF>
    static void launch_tend_b(const Dims& d, const Prof<TF>& pr, const TendArgs<TF>& a,
                              bool surf, bool scal, bool buoy, bool force, cudaStream_t s)
    {
        // One instantiation per combination of the four switches.
        const int mask = (surf ? 8 : 0) | (scal ? 4 : 0) | (buoy ? 2 : 0) | (force ? 1 : 0);
        switch (mask)
        {
#define MHH_TEND_CASE(M) case M: launch_tend_t<TF, ADV, DIF, ((M) & 8) != 0, ((M) & 4) != 0, ((M) & 2) != 0, ((M) & 1) != 0>(d, pr, a, s); break;
            MHH_TEND_CASE(0) MHH_TEND_CASE(1) MHH_TEND_CASE(2) MHH_TEND_CASE(3)
            MHH_TEND_CASE(4) MHH_TEND_CASE(5) MHH_TEND_CASE(6) MHH_TEND_CASE(7)
            MHH_TEND_CASE(8) MHH_TEND_CASE(9) MHH_TEND_CASE(10) MHH_TEND_CASE(11)
            MHH_TEND_CASE(12) MHH_TEND_CASE(13) MHH_TEND_CASE(14) MHH_TEND_CASE(15)
#undef MHH_TEND_CASE
        }
    }

    template<typename TF>
    void launch_tendency(const Dims& d, const Prof<TF>& pr, const TendArgs<TF>& a, int adv, int dif,
                         bool surf, bool scal, bool buoy, bool force, const KernelOpts& o, cudaStream_t s)
    {
        // The LES combination can run in the tiled kernel (mhh_tend_tiled.cu)
        // or in the flux-form kernel (mhh_tend_flux.cu).
        // Automatic choice (-1): the flux form in both precisions (in double
        // it agrees with the per-cell kernel, which keeps the reference's
        // operation order, to round-off: both are held to 1e-12 against the
        // reference).
        // The limited scalar (adv == ADVEC_2I5_LIM) runs in the flux-form or
        // the per-cell kernel; the tiled kernel hands it to the flux form.
        const int var = o.tend < 0 ? 2 : o.tend;
        const bool lim = adv == ADVEC_2I5_LIM && scal;
        if (adv == ADVEC_2I5_LIM && !scal) adv = MHH_ADVEC_2I5;
        if (var >= 1 && (adv == MHH_ADVEC_2I5 || lim) && dif == MHH_DIFF_SMAG2 && !force && d.igc >= 3 && d.jgc >= 3)
        {
            if (var == 2 || lim) launch_tendency_flux<TF>(d, pr, a, surf, scal, buoy, lim, o.tend_kchunk, s);
            else launch_tendency_les<TF>(d, pr, a, surf, scal, buoy, s);
            return;
        }
        if (lim)
        {
            if (dif == MHH_DIFF_SMAG2) launch_tend_lim<TF, MHH_DIFF_SMAG2>(d, pr, a, surf, buoy, force, s);
            else if (dif == MHH_DIFF_2) launch_tend_lim<TF, MHH_DIFF_2>(d, pr, a, surf, buoy, force, s);
            else launch_tend_lim<TF, 0>(d, pr, a, surf, buoy, force, s);
            return;
        }
        // With scalar work requested but no scalar pointer, or buoyancy without
        // a scalar, fall back to the switches the arguments support.
        if (adv == MHH_ADVEC_2I5)
        {
            if (dif == MHH_DIFF_SMAG2) launch_tend_b<TF, MHH_ADVEC_2I5, MHH_DIFF_SMAG2>(d, pr, a, surf, scal, buoy, force, s);
            else if (dif == MHH_DIFF_2) launch_tend_b<TF, MHH_ADVEC_2I5, MHH_DIFF_2>(d, pr, a, surf, scal, buoy, force, s);
            else launch_tend_b<TF, MHH_ADVEC_2I5, 0>(d, pr, a, surf, scal, buoy, force, s);
        }
        else if (adv == MHH_ADVEC_2)
        {
            if (dif == MHH_DIFF_SMAG2) launch_tend_b<TF, MHH_ADVEC_2, MHH_DIFF_SMAG2>(d, pr, a, surf, scal, buoy, force, s);
            else if (dif == MHH_DIFF_2) launch_tend_b<TF, MHH_ADVEC_2, MHH_DIFF_2>(d, pr, a, surf, scal, buoy, force, s);
            else launch_tend_b<TF, MHH_ADVEC_2, 0>(d, pr, a, surf, scal, buoy, force, s);
        }
        else
        {
            if (dif == MHH_DIFF_SMAG2) launch_tend_b<TF, 0, MHH_DIFF_SMAG2>(d, pr, a, surf, scal, buoy, force, s);
            else if (dif == MHH_DIFF_2) launch_tend_b<TF, 0, MHH_DIFF_2>(d, pr, a, surf, scal, buoy, force, s);
            else launch_tend_b<TF, 0, 0>(d, pr, a, surf, scal, buoy, force, s);
        }
    }

    // ---------------------------------------------------------------------
    // RK3, src/timeloop.cxx:250-286: a += cB*dt*at; at *= cA(next), or zero
    // at over all cells (ghosts included) after the last substep.
    // ---------------------------------------------------------------------
    template<typename TF>
    __global__ void k_rk3(TF* __restrict__ a, TF* __restrict__ at, Dims d, TF cbdt, TF ca, int last)
    {
        const long long n = blockIdx.x*(long long)blockDim.x + threadIdx.x;
        if (n >= d.ncells) return;
        const int i = (int)(n % d.icells);
        const int j = (int)((n / d.icells) % d.jcells);
        const int k = (int)(n / d.ijcells);
        const bool interior = i >= d.istart && i < d.iend && j >= d.jstart && j < d.jend && k >= d.kstart && k < d.kend;
        if (interior)
        {
            const TF t = at[n];
            a[n] = a[n] + mulx(cbdt, t);
            at[n] = last ? TF(0) : t*ca;
        }
        else if (last)
            at[n] = TF(0);
    }

    // ---------------------------------------------------------------------
    // Buffer (damping) layer, src/buffer.cxx:37-59: at -= sigma(z) (a - abuf)
    // for u, v, s at the full levels and w (towards zero) at the half levels
    // inside the layer; levels with sigma = 0 are below it and untouched.
    // ---------------------------------------------------------------------
    template<typename TF> struct BufferP
    {
        Dims d; const TF* prof; int kb;
        const TF *u, *v, *w, *s;
        TF *ut, *vt, *wt, *st;
    };

    template<typename TF>
    __device__ __forceinline__ void buffer_body(const BufferP<TF>& P, const VBlock& vb)
    {
        const Dims& d = P.d;
        const TF* __restrict__ prof = P.prof;
        const int kb = P.kb;
        const TF* __restrict__ u = P.u; const TF* __restrict__ v = P.v; const TF* __restrict__ w = P.w;
        const TF* __restrict__ s = P.s;
        TF* __restrict__ ut = P.ut; TF* __restrict__ vt = P.vt; TF* __restrict__ wt = P.wt; TF* __restrict__ st = P.st;
        const int i = d.istart + vb.x*blockDim.x + threadIdx.x;
        const int j = d.jstart + vb.y*blockDim.y + threadIdx.y;
        const int k = kb + vb.z;
        if (i >= d.iend || j >= d.jend || k >= d.kend) return;
        const int kc = d.kcells;
        const TF sf = prof[k], sh = prof[kc + k];
        const long long c = ijk(d, i, j, k);
        if (sf != TF(0))
        {
            ut[c] -= sf*(u[c] - prof[2*kc + k]);
            vt[c] -= sf*(v[c] - prof[3*kc + k]);
            if (s) st[c] -= sf*(s[c] - prof[4*kc + k]);
        }
        if (sh != TF(0)) wt[c] -= sh*(w[c] - TF(0));
    }

    template<typename TF>
    void launch_buffer(const Dims& d, const TF* prof, int kb, const TF* u, const TF* v, const TF* w, const TF* s,
                       TF* ut, TF* vt, TF* wt, TF* st, cudaStream_t strm)
    {
        if (kb >= d.kend) return;
        dim3 block(32, 8), grid((d.itot + 31)/32, (d.jtot + 7)/8, d.kend - kb);
        launch_body<BufferP<TF>, buffer_body<TF>, 256>(grid, block, 0, strm, BufferP<TF>{d, prof, kb, u, v, w, s, ut, vt, wt, st});
        count_launch();
    }

    template<typename TF>
    void launch_rk3(TF* a, TF* at, const Dims& d, int substep, double dt, cudaStream_t s)
    {
        const double cA[3] = {0., -5./9., -153./128.};
        const double cB[3] = {1./3., 15./16., 8./15.};
        const int sn = (substep + 1) % 3;
        const long long n = d.ncells;
        k_rk3<TF><<<(unsigned)((n + 255)/256), 256, 0, s>>>(a, at, d, TF(cB[substep]*dt), TF(cA[sn]), sn == 0);
        count_launch();
    }

    // ---------------------------------------------------------------------
    // Pressure gradient (src/pres_2.cxx:364-387) fused with the RK3 update
    // of all prognostic fields (src/timeloop.cxx:250-286).  One thread per
    // cell of the full ghost layout so that the tendencies' ghost cells are
    // zeroed after the last substep as on the CPU.
    // ---------------------------------------------------------------------
    template<typename TF> struct PresoutP
    {
        Dims d; Prof<TF> pr; const TF* p;
        TF *u, *v, *w, *s, *ut, *vt, *wt, *st;
        TF cbdt, ca; int last;
    };

    template<typename TF, bool SCAL>
    __device__ __forceinline__ void presout_rk3_body(const PresoutP<TF>& P, const VBlock& vb)
    {
        const Dims& d = P.d;
        const Prof<TF>& pr = P.pr;
        const TF* __restrict__ p = P.p;
        TF* __restrict__ u = P.u; TF* __restrict__ v = P.v; TF* __restrict__ w = P.w; TF* __restrict__ s = P.s;
        TF* __restrict__ ut = P.ut; TF* __restrict__ vt = P.vt; TF* __restrict__ wt = P.wt; TF* __restrict__ st = P.st;
        const TF cbdt = P.cbdt, ca = P.ca;
        const int last = P.last;
        const int i = vb.x*blockDim.x + threadIdx.x;
        const int j = vb.y*blockDim.y + threadIdx.y;
        const int k = vb.z;
        if (i >= d.icells || j >= d.jcells) return;
        const long long c = ijk(d, i, j, k);
        const bool interior = i >= d.istart && i < d.iend && j >= d.jstart && j < d.jend && k >= d.kstart && k < d.kend;
        if (interior)
        {
            const TF pc = ld(p, c);
            // src/pres_2.cxx:380-382 and src/timeloop.cxx:264 (products not
            // contracted in double).
            TF tu = ut[c] - mulx(pc - ld(p, c-1), dxi_of<TF>(d));
            TF tv = vt[c] - mulx(pc - ld(p, c-d.icells), dyi_of<TF>(d));
            TF tw = wt[c] - mulx(pc - ld(p, c-d.ijcells), ld(pr.dzhi, k));
            u[c] = u[c] + mulx(cbdt, tu); v[c] = v[c] + mulx(cbdt, tv); w[c] = w[c] + mulx(cbdt, tw);
            ut[c] = last ? TF(0) : tu*ca;
            vt[c] = last ? TF(0) : tv*ca;
            wt[c] = last ? TF(0) : tw*ca;
            if (SCAL)
            {
                const TF ts = st[c];
                s[c] = s[c] + mulx(cbdt, ts);
                st[c] = last ? TF(0) : ts*ca;
            }
        }
        else if (last)
        {
            ut[c] = TF(0); vt[c] = TF(0); wt[c] = TF(0);
            if (SCAL) st[c] = TF(0);
        }
    }

    // Float fields with an even row length: two adjacent cells (i even) per
    // thread with 8-byte loads and stores, half the memory instructions of
    // the per-cell kernel.  A ghost cell of the pair keeps its values (or is
    // zeroed after the last substep); the arithmetic per cell is that of
    // k_presout_rk3.
    template<bool SCAL>
    __device__ __forceinline__ void presout_rk3_x2_body(const PresoutP<float>& P, const VBlock& vb)
    {
        const Dims& d = P.d;
        const Prof<float>& pr = P.pr;
        const float* __restrict__ p = P.p;
        float* __restrict__ u = P.u; float* __restrict__ v = P.v; float* __restrict__ w = P.w; float* __restrict__ s = P.s;
        float* __restrict__ ut = P.ut; float* __restrict__ vt = P.vt; float* __restrict__ wt = P.wt;
        float* __restrict__ st = P.st;
        const float cbdt = P.cbdt, ca = P.ca;
        const int last = P.last;
        const int i = 2*(vb.x*blockDim.x + threadIdx.x);
        const int j = vb.y*blockDim.y + threadIdx.y;
        const int k = vb.z;
        if (i >= d.icells || j >= d.jcells) return;
        const long long c = ijk(d, i, j, k);
        const bool row_in = j >= d.jstart && j < d.jend && k >= d.kstart && k < d.kend;
        const bool in0 = row_in && i >= d.istart && i < d.iend;
        const bool in1 = row_in && i+1 >= d.istart && i+1 < d.iend;
        if (!in0 && !in1)
        {
            if (last)
            {
                const float2 z = make_float2(0.f, 0.f);
                *reinterpret_cast<float2*>(ut + c) = z; *reinterpret_cast<float2*>(vt + c) = z;
                *reinterpret_cast<float2*>(wt + c) = z;
                if (SCAL) *reinterpret_cast<float2*>(st + c) = z;
            }
            return;
        }
        auto ld2 = [](const float* a, long long n) { return __ldg(reinterpret_cast<const float2*>(a + n)); };
        const float2 pc = ld2(p, c);
        const float pw = i > 0 ? __ldg(p + c - 1) : 0.f;
        const float2 ps = ld2(p, c - d.icells), pb = ld2(p, c - d.ijcells);
        const float dxi = dxi_of<float>(d), dyi = dyi_of<float>(d), dzhi = __ldg(pr.dzhi + k);
        float2 tu = *reinterpret_cast<const float2*>(ut + c), tv = *reinterpret_cast<const float2*>(vt + c);
        float2 tw = *reinterpret_cast<const float2*>(wt + c);
        float2 uu = *reinterpret_cast<const float2*>(u + c), vv = *reinterpret_cast<const float2*>(v + c);
        float2 ww = *reinterpret_cast<const float2*>(w + c);
        // Cell 0 (i) and cell 1 (i+1).
        const float tu0 = tu.x - (pc.x - pw)*dxi, tu1 = tu.y - (pc.y - pc.x)*dxi;
        const float tv0 = tv.x - (pc.x - ps.x)*dyi, tv1 = tv.y - (pc.y - ps.y)*dyi;
        const float tw0 = tw.x - (pc.x - pb.x)*dzhi, tw1 = tw.y - (pc.y - pb.y)*dzhi;
        if (in0) { uu.x += cbdt*tu0; vv.x += cbdt*tv0; ww.x += cbdt*tw0; }
        if (in1) { uu.y += cbdt*tu1; vv.y += cbdt*tv1; ww.y += cbdt*tw1; }
        *reinterpret_cast<float2*>(u + c) = uu; *reinterpret_cast<float2*>(v + c) = vv;
        *reinterpret_cast<float2*>(w + c) = ww;
        tu.x = in0 ? (last ? 0.f : tu0*ca) : (last ? 0.f : tu.x);
        tu.y = in1 ? (last ? 0.f : tu1*ca) : (last ? 0.f : tu.y);
        tv.x = in0 ? (last ? 0.f : tv0*ca) : (last ? 0.f : tv.x);
        tv.y = in1 ? (last ? 0.f : tv1*ca) : (last ? 0.f : tv.y);
        tw.x = in0 ? (last ? 0.f : tw0*ca) : (last ? 0.f : tw.x);
        tw.y = in1 ? (last ? 0.f : tw1*ca) : (last ? 0.f : tw.y);
        *reinterpret_cast<float2*>(ut + c) = tu; *reinterpret_cast<float2*>(vt + c) = tv;
        *reinterpret_cast<float2*>(wt + c) = tw;
        if (SCAL)
        {
            float2 ts = *reinterpret_cast<const float2*>(st + c);
            float2 ss = *reinterpret_cast<const float2*>(s + c);
            if (in0) ss.x += cbdt*ts.x;
            if (in1) ss.y += cbdt*ts.y;
            *reinterpret_cast<float2*>(s + c) = ss;
            ts.x = last ? 0.f : (in0 ? ts.x*ca : ts.x);
            ts.y = last ? 0.f : (in1 ? ts.y*ca : ts.y);
            *reinterpret_cast<float2*>(st + c) = ts;
        }
    }

    template<typename TF>
    void launch_presout_rk3(const Dims& d, const Prof<TF>& pr, const TF* p, TF* u, TF* v, TF* w, TF* s,
                            TF* ut, TF* vt, TF* wt, TF* st, int substep, double dt, cudaStream_t strm)
    {
        const double cA[3] = {0., -5./9., -153./128.};
        const double cB[3] = {1./3., 15./16., 8./15.};
        const int sn = (substep + 1) % 3;
        dim3 block(32, 8);
        const PresoutP<TF> prm{d, pr, p, u, v, w, s, ut, vt, wt, st, TF(cB[substep]*dt), TF(cA[sn]), sn == 0};
        if constexpr (sizeof(TF) == 4)
        {
            if (d.icells % 2 == 0 && d.ijcells % 2 == 0)
            {
                dim3 grid((d.icells/2 + 31)/32, (d.jcells + 7)/8, d.kcells);
                if (s) launch_body<PresoutP<float>, presout_rk3_x2_body<true>, 256>(grid, block, 0, strm, prm);
                else launch_body<PresoutP<float>, presout_rk3_x2_body<false>, 256>(grid, block, 0, strm, prm);
                count_launch();
                return;
            }
        }
        dim3 grid((d.icells + 31)/32, (d.jcells + 7)/8, d.kcells);
        if (s) launch_body<PresoutP<TF>, presout_rk3_body<TF, true>, 256>(grid, block, 0, strm, prm);
        else launch_body<PresoutP<TF>, presout_rk3_body<TF, false>, 256>(grid, block, 0, strm, prm);
        count_launch();
    }

    // ---------------------------------------------------------------------
    // Max reductions: CFL of Advec_2i5 (src/advec_2i5.cxx:59-148) and
    // Advec_2 (src/advec_2.cxx:50-80), diffusion number of Diff_smag2
    // (include/diff_kernels.h:486-511), divergence (src/pres_2.cxx:389-422).
    // The diffusion number and the divergence are computed per cell in
    // double.  The CFL terms are evaluated in the field precision, as in the
    // reference, and their maximum is taken in that precision before the one
    // conversion per block: a maximum commutes with the exact float-to-double
    // conversion, so the result is the same as a maximum over doubles.
    template<typename TF, int WHAT>
    __global__ void __launch_bounds__(256)
    k_reduce(Dims d, Prof<TF> pr, const TF* __restrict__ u, const TF* __restrict__ v, const TF* __restrict__ w,
             const TF* __restrict__ ev, double tprfi, unsigned long long* out)
    {
        using RT = typename std::conditional<(WHAT <= 1), TF, double>::type;
        const int i = d.istart + blockIdx.x*blockDim.x + threadIdx.x;
        const int j = d.jstart + blockIdx.y*blockDim.y + threadIdx.y;
        const int k = d.kstart + blockIdx.z;
        RT val = 0;
        if (i < d.iend && j < d.jend)
        {
            const long long ii = 1, jj = d.icells, kk = d.ijcells;
            const long long c = ijk(d, i, j, k);
            if constexpr (WHAT == 0)
            {
                // CFL 2i5: w interpolated with 2nd/4th/6th order by level.
                const int ord = face_order_w(d, k);
                TF wc;
                if (ord == 2) wc = f2(w, c+kk, kk);
                else if (ord == 4) wc = f4(w, c+kk, kk);
                else wc = f6(w, c+kk, kk);
                val = fabs(f6(u, c+ii, ii))*dxi_of<TF>(d) + fabs(f6(v, c+jj, jj))*dyi_of<TF>(d) + fabs(wc)*ld(pr.dzi, k);
            }
            else if constexpr (WHAT == 1)
            {
                val = fabs(i2(ld(u, c), ld(u, c+ii)))*dxi_of<TF>(d) + fabs(i2(ld(v, c), ld(v, c+jj)))*dyi_of<TF>(d)
                    + fabs(i2(ld(w, c), ld(w, c+kk)))*ld(pr.dzi, k);
            }
            else if constexpr (WHAT == 2)
            {
                const double dzi = double(ld(pr.dzi, k));
                val = fabs(double(ld(ev, c))*tprfi*(d.dxi*d.dxi + d.dyi*d.dyi + dzi*dzi));
            }
            else
            {
                const double div = double(ld(pr.rhoref, k))*(double(ld(u, c+ii)-ld(u, c))*d.dxi + double(ld(v, c+jj)-ld(v, c))*d.dyi)
                                 + (double(ld(pr.rhorefh, k+1))*double(ld(w, c+kk)) - double(ld(pr.rhorefh, k))*double(ld(w, c)))*double(ld(pr.dzi, k));
                val = fabs(div);
            }
        }
        // Block max (NaN kept), then one atomic per block.
        for (int o=16; o>0; o>>=1)
            val = max_nan(val, __shfl_xor_sync(0xffffffffu, val, o));
        __shared__ RT sm[8];
        const int lane = (threadIdx.x + threadIdx.y*blockDim.x) & 31;
        const int warp = (threadIdx.x + threadIdx.y*blockDim.x) >> 5;
        if (lane == 0) sm[warp] = val;
        __syncthreads();
        if (warp == 0)
        {
            val = lane < (int)(blockDim.x*blockDim.y/32) ? sm[lane] : RT(0);
            for (int o=16; o>0; o>>=1)
                val = max_nan(val, __shfl_xor_sync(0xffffffffu, val, o));
            if (lane == 0) atomic_max_nonneg(out, double(val));
        }
    }

    template<typename TF>
    void launch_reduce(int what, const Dims& d, const Prof<TF>& pr, const TF* u, const TF* v, const TF* w,
                       const TF* ev, double tprfi, unsigned long long* out, cudaStream_t s)
    {
        dim3 block(32, 8);
        dim3 grid((d.itot + 31)/32, (d.jtot + 7)/8, d.ktot);
        if (what == 0) k_reduce<TF, 0><<<grid, block, 0, s>>>(d, pr, u, v, w, ev, tprfi, out);
        else if (what == 1) k_reduce<TF, 1><<<grid, block, 0, s>>>(d, pr, u, v, w, ev, tprfi, out);
        else if (what == 2) k_reduce<TF, 2><<<grid, block, 0, s>>>(d, pr, u, v, w, ev, tprfi, out);
        else k_reduce<TF, 3><<<grid, block, 0, s>>>(d, pr, u, v, w, ev, tprfi, out);
        count_launch();
    }

#define MHH_INSTANTIATE(TF) \
    template void launch_cyclic<TF>(const FieldList<TF>&, const Dims&, int, cudaStream_t); \
    template void launch_cyclic2d<TF>(TF*, const Dims&, cudaStream_t); \
    template void launch_set_bc<TF>(TF*, TF*, TF*, int, double, double, int, const Dims&, cudaStream_t); \
    template void launch_ghost<TF>(const GhostList<TF>&, const Dims&, const TF*, cudaStream_t); \
    template void launch_viscosity<TF>(const Dims&, const Prof<TF>&, const TF*, const TF*, const TF*, const TF*, TF*, \
        const TF*, const double*, const double*, const double*, double, double, double, int, bool, bool, const KernelOpts&, cudaStream_t); \
    template void launch_tendency<TF>(const Dims&, const Prof<TF>&, const TendArgs<TF>&, int, int, bool, bool, bool, bool, const KernelOpts&, cudaStream_t); \
    template void launch_rk3<TF>(TF*, TF*, const Dims&, int, double, cudaStream_t); \
    template void launch_buffer<TF>(const Dims&, const TF*, int, const TF*, const TF*, const TF*, const TF*, TF*, TF*, TF*, TF*, cudaStream_t); \
    template void launch_presout_rk3<TF>(const Dims&, const Prof<TF>&, const TF*, TF*, TF*, TF*, TF*, TF*, TF*, TF*, TF*, int, double, cudaStream_t); \
    template void launch_reduce<TF>(int, const Dims&, const Prof<TF>&, const TF*, const TF*, const TF*, const TF*, double, unsigned long long*, cudaStream_t);

    MHH_INSTANTIATE(double)
    MHH_INSTANTIATE(float)
}
