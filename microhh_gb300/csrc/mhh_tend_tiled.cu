// mhh_tend_tiled.cu -- the LES tendency kernel (Advec_2i5 + Smagorinsky
// diffusion + dry buoyancy, optionally with the Monin-Obukhov wall fluxes),
// blocked for the GPU: a block owns a 32 x 8 tile of columns and marches
// upward through a chunk of levels.  The horizontal neighbourhoods come from
// shared-memory planes (u, v at k-1 and k; w at k and k+1; s at k; evisc at
// k-1, k, k+1, with a 3-cell halo), the vertical 7-point neighbourhoods of the
// thread's own column from register queues.  Every plane is loaded once per
// level, so a field is read from DRAM about once per substep.
//
// The arithmetic per term is that of mhh_stencil.cuh (and through it of
// src/advec_2i5.cxx:150-728, include/diff_kernels.h:144-484 and
// src/thermo_dry.cxx:165-181).
#include "mhh_kernels.cuh"
#include "mhh_batchable.cuh"
#include "mhh_stencil.cuh"

namespace mhh
{
    namespace
    {
        constexpr int TX = 32, TY = 8, H = 3;
        constexpr int PW = TX + 2*H;           // plane width
        constexpr int PH = TY + 2*H;           // plane height
        constexpr int PS = PW*PH;              // plane size
        constexpr int NPLANE = 10;
        constexpr int KCHUNK = 32;
    }

    template<typename TF>
    __device__ __forceinline__ void load_plane(TF* dst, const TF* __restrict__ src, const Dims& d,
                                               int i0, int j0, int k, int tid)
    {
        const long long base = (long long)k*d.ijcells;
        for (int e = tid; e < PS; e += TX*TY)
        {
            const int pj = e / PW, pi = e - pj*PW;
            const int i = i0 - H + pi, j = j0 - H + pj;
            dst[e] = (i < d.icells && j < d.jcells) ? __ldg(src + base + i + (long long)j*d.icells) : TF(0);
        }
    }

    // Upwind-biased flux a_face * wf through the face between queue entries
    // B-1 and B (queue entry m holds level k-3+m); `order` is uniform across
    // the block because all threads are at the same level.
    template<int B, typename TF>
    __device__ __forceinline__ TF qflux(const TF (&q)[7], TF wf, int order)
    {
        if (order == 6)
            return wf*i6ws(q[B-3], q[B-2], q[B-1], q[B], q[B+1], q[B+2])
                 - fabs(wf)*i5ws(q[B-3], q[B-2], q[B-1], q[B], q[B+1], q[B+2]);
        if (order == 4)
            return wf*i4ws(q[B-2], q[B-1], q[B], q[B+1])
                 - fabs(wf)*i3ws(q[B-2], q[B-1], q[B], q[B+1]);
        return wf*i2(q[B-1], q[B]);
    }

    // Two blocks per SM for float; double needs the full register file.
    template<typename TF> struct LesOcc { static constexpr int v = sizeof(TF) == 4 ? 2 : 1; };

    template<typename TF> struct TendLesP { Dims d; Prof<TF> pr; TendArgs<TF> a; };

    template<typename TF, bool SURF, bool SCAL, bool BUOY>
    __device__ __forceinline__ void tend_les_body(const TendLesP<TF>& P, const VBlock& vb)
    {
        const Dims& d = P.d;
        const Prof<TF>& pr = P.pr;
        const TendArgs<TF>& a = P.a;
        extern __shared__ __align__(16) unsigned char smem_raw[];
        TF* sm = reinterpret_cast<TF*>(smem_raw);
        // Plane slots: 0,1 u; 2,3 v; 4,5 w; 6 s; 7,8,9 evisc (addressed by
        // offset arithmetic so that nothing is indexed through local memory).
        #define PU(q) (sm + (0 + (q))*PS)
        #define PV(q) (sm + (2 + (q))*PS)
        #define PWW(q) (sm + (4 + (q))*PS)
        #define PE(q) (sm + (7 + (q))*PS)
        TF* ps = sm + 6*PS;

        const int tx = threadIdx.x, ty = threadIdx.y, tid = tx + ty*TX;
        const int i0 = d.istart + vb.x*TX;
        const int j0 = d.jstart + vb.y*TY;
        const int i = i0 + tx, j = j0 + ty;
        const bool active = i < d.iend && j < d.jend;
        const int k0 = d.kstart + vb.z*KCHUNK;
        const int k1 = min(k0 + KCHUNK, d.kend);

        const TF* __restrict__ u = a.u;
        const TF* __restrict__ v = a.v;
        const TF* __restrict__ w = a.w;
        const TF* __restrict__ s = a.s;
        const TF* __restrict__ ev = a.evisc;
        const long long col = (long long)min(i, d.icells-1) + (long long)min(j, d.jcells-1)*d.icells;
        const int pc = (ty + H)*PW + (tx + H);      // own cell in a plane

        auto colval = [&](const TF* f, int k) -> TF
        {
            const int kc = k < 0 ? 0 : (k > d.kcells-1 ? d.kcells-1 : k);
            return __ldg(f + col + (long long)kc*d.ijcells);
        };

        // Register queues of the own column: q[m] holds level k-3+m.
        TF qu[7], qv[7], qw[7], qs[7];
        #pragma unroll
        for (int m=0; m<6; ++m)
        {
            qu[m+1] = colval(u, k0-3+m);
            qv[m+1] = colval(v, k0-3+m);
            qw[m+1] = colval(w, k0-3+m);
            if (SCAL || BUOY) qs[m+1] = colval(s, k0-3+m);
        }

        // Planes that the first level finds in place.
        // Slots are rotated at the top of each level: u and v flip to the
        // other slot, w's level k+1 becomes level k, evisc advances by one.
        int cu = 0, cv = 0, cw = 0, ce = 0;
        load_plane(PU(0), u, d, i0, j0, k0-1, tid);
        load_plane(PV(0), v, d, i0, j0, k0-1, tid);
        load_plane(PWW(1), w, d, i0, j0, k0, tid);
        load_plane(PE(0), ev, d, i0, j0, k0-1, tid);
        load_plane(PE(1), ev, d, i0, j0, k0, tid);

        const TF dxi = dxi_of<TF>(d), dyi = dyi_of<TF>(d);
        const TF dxidxi = a.dxidxi_t, dyidyi = a.dyidyi_t;
        const TF visc = a.visc, svisc = a.svisc, tpri = a.tpri;
        const long long ij = col;
        TF ufb = 0, uft = 0, vfb = 0, vft = 0, sfb = 0, sft = 0;
        if (SURF && active)
        {
            ufb = a.u_fluxbot[ij]; uft = a.u_fluxtop[ij];
            vfb = a.v_fluxbot[ij]; vft = a.v_fluxtop[ij];
            if (SCAL) { sfb = a.s_fluxbot[ij]; sft = a.s_fluxtop[ij]; }
        }

        for (int k = k0; k < k1; ++k)
        {
            // Rotate: u, v current <- the other slot; w current <- old k+1; evisc shifts.
            cu ^= 1; cv ^= 1; cw ^= 1; ce = (ce + 1) % 3;
            // New planes: u(k), v(k), w(k+1), s(k), evisc(k+1).
            load_plane(PU(cu), u, d, i0, j0, k, tid);
            load_plane(PV(cv), v, d, i0, j0, k, tid);
            load_plane(PWW(cw ^ 1), w, d, i0, j0, k+1, tid);
            if (SCAL) load_plane(ps, s, d, i0, j0, k, tid);
            load_plane(PE((ce + 1) % 3), ev, d, i0, j0, k+1, tid);
            #pragma unroll
            for (int m=0; m<6; ++m) { qu[m] = qu[m+1]; qv[m] = qv[m+1]; qw[m] = qw[m+1]; qs[m] = qs[m+1]; }
            qu[6] = colval(u, k+3); qv[6] = colval(v, k+3); qw[6] = colval(w, k+3);
            if (SCAL || BUOY) qs[6] = colval(s, k+3);
            __syncthreads();

            if (active)
            {
                const TF* U = PU(cu) + pc;          // u(k)
                const TF* Um = PU(cu ^ 1) + pc;     // u(k-1)
                const TF* V = PV(cv) + pc;
                const TF* Vm = PV(cv ^ 1) + pc;
                const TF* W0 = PWW(cw) + pc;        // w(k)
                const TF* W1 = PWW(cw ^ 1) + pc;    // w(k+1)
                const TF* S = ps + pc;
                const TF* Em = PE((ce + 2) % 3) + pc;   // evisc(k-1)
                const TF* E0 = PE(ce) + pc;             // evisc(k)
                const TF* E1 = PE((ce + 1) % 3) + pc;   // evisc(k+1)
                #define X(P, di, dj) (P)[(dj)*PW + (di)]
                const long long c = col + (long long)k*d.ijcells;
                const TF rho = pr.rhoref[k], rhoh = pr.rhorefh[k], rhoh1 = pr.rhorefh[k+1];
                const TF dzik = pr.dzi[k], dzhik = pr.dzhi[k], dzhik1 = pr.dzhi[k+1];
                const int ot = face_order_full(d, k+1), ob = face_order_full(d, k);
                const bool bot = SURF && k == d.kstart, top = SURF && k == d.kend-1;

                auto hadv = [&](const TF* P, TF ue, TF uw, TF vn, TF vs) -> TF
                {
                    return - (ue*i6ws(X(P,-2,0), X(P,-1,0), X(P,0,0), X(P,1,0), X(P,2,0), X(P,3,0))
                            - uw*i6ws(X(P,-3,0), X(P,-2,0), X(P,-1,0), X(P,0,0), X(P,1,0), X(P,2,0)))*dxi
                           + (fabs(ue)*i5ws(X(P,-2,0), X(P,-1,0), X(P,0,0), X(P,1,0), X(P,2,0), X(P,3,0))
                            - fabs(uw)*i5ws(X(P,-3,0), X(P,-2,0), X(P,-1,0), X(P,0,0), X(P,1,0), X(P,2,0)))*dxi
                           - (vn*i6ws(X(P,0,-2), X(P,0,-1), X(P,0,0), X(P,0,1), X(P,0,2), X(P,0,3))
                            - vs*i6ws(X(P,0,-3), X(P,0,-2), X(P,0,-1), X(P,0,0), X(P,0,1), X(P,0,2)))*dyi
                           + (fabs(vn)*i5ws(X(P,0,-2), X(P,0,-1), X(P,0,0), X(P,0,1), X(P,0,2), X(P,0,3))
                            - fabs(vs)*i5ws(X(P,0,-3), X(P,0,-2), X(P,0,-1), X(P,0,0), X(P,0,1), X(P,0,2)))*dyi;
                };

                // ---- u ----
                {
                    TF t = hadv(U, i2(X(U,0,0), X(U,1,0)), i2(X(U,-1,0), X(U,0,0)),
                                   i2(X(V,-1,1), X(V,0,1)), i2(X(V,-1,0), X(V,0,0)));
                    const TF ftop = ot ? rhoh1*qflux<4>(qu, i2(X(W1,-1,0), X(W1,0,0)), ot) : TF(0);
                    const TF fbot = ob ? rhoh*qflux<3>(qu, i2(X(W0,-1,0), X(W0,0,0)), ob) : TF(0);
                    t -= (ftop - fbot) / rho * dzik;
                    // diffusion
                    const TF e_e = X(E0,0,0) + visc, e_w = X(E0,-1,0) + visc;
                    const TF e_n = TF(0.25)*(X(E0,-1,0) + X(E0,0,0) + X(E0,-1,1) + X(E0,0,1)) + visc;
                    const TF e_s = TF(0.25)*(X(E0,-1,-1) + X(E0,0,-1) + X(E0,-1,0) + X(E0,0,0)) + visc;
                    TF dt, db;
                    if (top) dt = -rhoh1*uft;
                    else
                    {
                        const TF e_t = TF(0.25)*(X(E0,-1,0) + X(E0,0,0) + X(E1,-1,0) + X(E1,0,0)) + visc;
                        dt = rhoh1*e_t*((qu[4]-qu[3])*dzhik1 + (X(W1,0,0)-X(W1,-1,0))*dxi);
                    }
                    if (bot) db = -rhoh*ufb;
                    else
                    {
                        const TF e_b = TF(0.25)*(X(Em,-1,0) + X(Em,0,0) + X(E0,-1,0) + X(E0,0,0)) + visc;
                        db = rhoh*e_b*((qu[3]-qu[2])*dzhik + (X(W0,0,0)-X(W0,-1,0))*dxi);
                    }
                    t += (e_e*(X(U,1,0)-X(U,0,0))*dxi - e_w*(X(U,0,0)-X(U,-1,0))*dxi)*TF(2)*dxi
                       + (e_n*((X(U,0,1)-X(U,0,0))*dyi + (X(V,0,1)-X(V,-1,1))*dxi)
                        - e_s*((X(U,0,0)-X(U,0,-1))*dyi + (X(V,0,0)-X(V,-1,0))*dxi))*dyi
                       + (dt - db)/rho*dzik;
                    a.ut[c] += t;
                }
                // ---- v ----
                {
                    TF t = hadv(V, i2(X(U,1,-1), X(U,1,0)), i2(X(U,0,-1), X(U,0,0)),
                                   i2(X(V,0,0), X(V,0,1)), i2(X(V,0,-1), X(V,0,0)));
                    const TF ftop = ot ? rhoh1*qflux<4>(qv, i2(X(W1,0,-1), X(W1,0,0)), ot) : TF(0);
                    const TF fbot = ob ? rhoh*qflux<3>(qv, i2(X(W0,0,-1), X(W0,0,0)), ob) : TF(0);
                    t -= (ftop - fbot) / rho * dzik;
                    const TF e_e = TF(0.25)*(X(E0,0,-1) + X(E0,0,0) + X(E0,1,-1) + X(E0,1,0)) + visc;
                    const TF e_w = TF(0.25)*(X(E0,-1,-1) + X(E0,-1,0) + X(E0,0,-1) + X(E0,0,0)) + visc;
                    const TF e_n = X(E0,0,0) + visc, e_s = X(E0,0,-1) + visc;
                    TF dt, db;
                    if (top) dt = -rhoh1*vft;
                    else
                    {
                        const TF e_t = TF(0.25)*(X(E0,0,-1) + X(E0,0,0) + X(E1,0,-1) + X(E1,0,0)) + visc;
                        dt = rhoh1*e_t*((qv[4]-qv[3])*dzhik1 + (X(W1,0,0)-X(W1,0,-1))*dyi);
                    }
                    if (bot) db = -rhoh*vfb;
                    else
                    {
                        const TF e_b = TF(0.25)*(X(Em,0,-1) + X(Em,0,0) + X(E0,0,-1) + X(E0,0,0)) + visc;
                        db = rhoh*e_b*((qv[3]-qv[2])*dzhik + (X(W0,0,0)-X(W0,0,-1))*dyi);
                    }
                    t += (e_e*((X(V,1,0)-X(V,0,0))*dxi + (X(U,1,0)-X(U,1,-1))*dyi)
                        - e_w*((X(V,0,0)-X(V,-1,0))*dxi + (X(U,0,0)-X(U,0,-1))*dyi))*dxi
                       + (e_n*(X(V,0,1)-X(V,0,0))*dyi - e_s*(X(V,0,0)-X(V,0,-1))*dyi)*TF(2)*dyi
                       + (dt - db)/rho*dzik;
                    a.vt[c] += t;
                }
                // ---- w (half levels above the wall) ----
                if (k > d.kstart)
                {
                    const TF rhom = pr.rhoref[k-1];
                    TF t = TF(0);
                    if (BUOY) t += TF(GRAV)/pr.threfh[k]*(i2(qs[2], qs[3]) - pr.thbh[k]);
                    t += hadv(W0, i2(X(Um,1,0), X(U,1,0)), i2(X(Um,0,0), X(U,0,0)),
                                  i2(X(Vm,0,1), X(V,0,1)), i2(X(Vm,0,0), X(V,0,0)));
                    const TF ftop = rho *qflux<4>(qw, i2(qw[3], qw[4]), face_order_w(d, k));
                    const TF fbot = rhom*qflux<3>(qw, i2(qw[2], qw[3]), face_order_w(d, k-1));
                    t -= (ftop - fbot) / rhoh * dzhik;
                    const TF e_e = TF(0.25)*(X(Em,0,0) + X(E0,0,0) + X(Em,1,0) + X(E0,1,0)) + visc;
                    const TF e_w = TF(0.25)*(X(Em,-1,0) + X(E0,-1,0) + X(Em,0,0) + X(E0,0,0)) + visc;
                    const TF e_n = TF(0.25)*(X(Em,0,0) + X(E0,0,0) + X(Em,0,1) + X(E0,0,1)) + visc;
                    const TF e_s = TF(0.25)*(X(Em,0,-1) + X(E0,0,-1) + X(Em,0,0) + X(E0,0,0)) + visc;
                    const TF e_t = X(E0,0,0) + visc, e_b = X(Em,0,0) + visc;
                    t += (e_e*((X(W0,1,0)-X(W0,0,0))*dxi + (X(U,1,0)-X(Um,1,0))*dzhik)
                        - e_w*((X(W0,0,0)-X(W0,-1,0))*dxi + (X(U,0,0)-X(Um,0,0))*dzhik))*dxi
                       + (e_n*((X(W0,0,1)-X(W0,0,0))*dyi + (X(V,0,1)-X(Vm,0,1))*dzhik)
                        - e_s*((X(W0,0,0)-X(W0,0,-1))*dyi + (X(V,0,0)-X(Vm,0,0))*dzhik))*dyi
                       + (rho*e_t*(qw[4]-qw[3])*dzik - rhom*e_b*(qw[3]-qw[2])*pr.dzi[k-1]) / rhoh*TF(2)*dzhik;
                    a.wt[c] += t;
                }
                // ---- scalar ----
                if (SCAL)
                {
                    TF t = hadv(S, X(U,1,0), X(U,0,0), X(V,0,1), X(V,0,0));
                    const TF ftop = ot ? rhoh1*qflux<4>(qs, qw[4], ot) : TF(0);
                    const TF fbot = ob ? rhoh*qflux<3>(qs, qw[3], ob) : TF(0);
                    t -= (ftop - fbot) / rho * dzik;
                    const TF e_e = TF(0.5)*(X(E0,0,0) + X(E0,1,0))*tpri + svisc;
                    const TF e_w = TF(0.5)*(X(E0,-1,0) + X(E0,0,0))*tpri + svisc;
                    const TF e_n = TF(0.5)*(X(E0,0,0) + X(E0,0,1))*tpri + svisc;
                    const TF e_s = TF(0.5)*(X(E0,0,-1) + X(E0,0,0))*tpri + svisc;
                    TF dt, db;
                    if (top) dt = -rhoh1*sft;
                    else
                    {
                        const TF e_t = TF(0.5)*(X(E0,0,0) + X(E1,0,0))*tpri + svisc;
                        dt = rhoh1*e_t*(qs[4]-qs[3])*dzhik1;
                    }
                    if (bot) db = -rhoh*sfb;
                    else
                    {
                        const TF e_b = TF(0.5)*(X(Em,0,0) + X(E0,0,0))*tpri + svisc;
                        db = rhoh*e_b*(qs[3]-qs[2])*dzhik;
                    }
                    t += (e_e*(X(S,1,0)-X(S,0,0)) - e_w*(X(S,0,0)-X(S,-1,0)))*dxidxi
                       + (e_n*(X(S,0,1)-X(S,0,0)) - e_s*(X(S,0,0)-X(S,0,-1)))*dyidyi
                       + (dt - db)/rho*dzik;
                    a.st[c] += t;
                }
                #undef X
            }
            __syncthreads();
        }
        #undef PU
        #undef PV
        #undef PWW
        #undef PE
    }

    template<typename TF, bool SURF, bool SCAL, bool BUOY>
    static void launch_les_t(const Dims& d, const Prof<TF>& pr, const TendArgs<TF>& a, cudaStream_t s)
    {
        const size_t smem = sizeof(TF)*NPLANE*PS;
        dim3 block(TX, TY);
        dim3 grid((d.itot + TX - 1)/TX, (d.jtot + TY - 1)/TY, (d.ktot + KCHUNK - 1)/KCHUNK);
        launch_body<TendLesP<TF>, tend_les_body<TF, SURF, SCAL, BUOY>, TX*TY, LesOcc<TF>::v>(grid, block, smem, s,
                                                                                     TendLesP<TF>{d, pr, a});
        count_launch();
    }

    // Advec_2i5 + Diff_smag2 (+ buoyancy) in the tiled kernel; igc, jgc >= 3.
    template<typename TF>
    void launch_tendency_les(const Dims& d, const Prof<TF>& pr, const TendArgs<TF>& a, bool surf, bool scal,
                             bool buoy, cudaStream_t s)
    {
        const int mask = (surf ? 4 : 0) | (scal ? 2 : 0) | (buoy ? 1 : 0);
        switch (mask)
        {
            case 0: launch_les_t<TF, false, false, false>(d, pr, a, s); break;
            case 1: launch_les_t<TF, false, false, true >(d, pr, a, s); break;
            case 2: launch_les_t<TF, false, true,  false>(d, pr, a, s); break;
            case 3: launch_les_t<TF, false, true,  true >(d, pr, a, s); break;
            case 4: launch_les_t<TF, true,  false, false>(d, pr, a, s); break;
            case 5: launch_les_t<TF, true,  false, true >(d, pr, a, s); break;
            case 6: launch_les_t<TF, true,  true,  false>(d, pr, a, s); break;
            default: launch_les_t<TF, true, true,  true >(d, pr, a, s); break;
        }
    }

    template void launch_tendency_les<double>(const Dims&, const Prof<double>&, const TendArgs<double>&, bool, bool, bool, cudaStream_t);
    template void launch_tendency_les<float>(const Dims&, const Prof<float>&, const TendArgs<float>&, bool, bool, bool, cudaStream_t);
}
