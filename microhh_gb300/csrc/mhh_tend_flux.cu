// mhh_tend_flux.cu -- the LES tendency kernel in flux form (Advec_2i5 +
// Smagorinsky diffusion + dry buoyancy, optionally with the Monin-Obukhov
// wall fluxes).
//
// Every face flux is computed once.  A block owns a 32 x 8 tile of columns
// and marches upward through a chunk of levels.  Its 33 x 9 face threads
// compute, per level, the total (diffusive minus advective) flux through the
// x- and y-faces of the u, v, w and s control volumes into shared memory; the
// 32 x 8 cell threads add the flux differences, with the vertical faces of
// their own column kept in registers (the top face of one level is the bottom
// face of the next).  The shear stresses are shared between the fields whose
// faces coincide: tau_xy at (i-1/2, j-1/2) is the y-flux of u and the x-flux
// of v, tau_xz at (i-1/2, k+1/2) the x-flux of w and the z-flux of u, and
// tau_yz likewise for w and v.
//
// Iteration m handles u, v, s at full level m and w at half level m+1, so the
// horizontal faces of w and the vertical faces of u, v, s lie on the same
// half level and share tau_xz and tau_yz.  The planes of each level (u, v, w,
// s and the eddy viscosity with a 3-cell halo) are staged in shared memory
// by cp.async two levels ahead of their use; the 7-point vertical
// neighbourhoods of the own column come from register queues.
//
// The arithmetic per face is that of the reference's kernels:
// src/advec_2i5.cxx:150-728 (6th-order interpolation with 5th-order upwind
// dissipation, lower orders next to the walls), include/diff_kernels.h:144-484
// (Smagorinsky fluxes; wall fluxes from the surface model) and
// src/thermo_dry.cxx:165-181 (buoyancy); with LIM the scalar's advective
// fluxes are those of the flux limiter (include/advec_monotonic.h:28-219).
// The sum of all fluxes is formed
// before it is added to the tendency, so the result differs from the
// reference's term-by-term accumulation by round-off only.
#include "mhh_kernels.cuh"
#include "mhh_stencil.cuh"
#include "mhh_flux.cuh"
#include "mhh_batchable.cuh"

namespace mhh
{
    namespace
    {
        constexpr int FTX = 32, FTY = 8, FH = 3;
        constexpr int FPW = 40;                 // plane row (FTX + 2*FH, padded)
        constexpr int FPH = FTY + 2*FH;         // plane rows
        constexpr int FPS = FPW*FPH;            // plane size
        constexpr int NFX = FTX + 1, NFY = FTY + 1;
        constexpr int NTHR = 320;
        constexpr int FKCHUNK_MAX = 64;
        // Plane slots: u 4, v 4, w 3, s 3, evisc 4; level l of a field lives
        // in slot base + l % n.  Planes are prefetched two levels ahead.
        constexpr int SU = 0, SV = 4, SW = 8, SS = 11, SE = 14, NSLOT = 18;
        constexpr int NGX = FTY*NFX;            // x-faces per level and field
        constexpr int NGY = NFY*FTX;            // y-faces per level and field
        constexpr int NEL1 = FPS - NTHR;        // threads that copy a second element

        template<typename TF> struct FluxOcc { static constexpr int v = sizeof(TF) == 4 ? 2 : 1; };

        constexpr int NPROF = 8;                // per-level constants staged in shared memory
        constexpr int PLEV = FKCHUNK_MAX + 2;   // levels m0 .. m0+kchunk+1

        template<typename TF>
        size_t flux_smem() { return sizeof(TF)*(size_t(NSLOT)*FPS + 2*4*(NGX + NGY) + NPROF*PLEV); }
    }

    template<typename TF> struct TendFluxP { Dims d; Prof<TF> pr; TendArgs<TF> a; int kchunk; };

    template<typename TF, bool SURF, bool SCAL, bool BUOY, bool LIM>
    __device__ __forceinline__ void tend_flux_body(const TendFluxP<TF>& P, const VBlock& vb)
    {
        const Dims& d = P.d;
        const Prof<TF>& pr = P.pr;
        const TendArgs<TF>& a = P.a;
        const int kchunk = P.kchunk;
        extern __shared__ __align__(16) unsigned char smem_raw[];
        TF* sm = reinterpret_cast<TF*>(smem_raw);
        TF* gbase = sm + NSLOT*FPS;     // [2 buffers][NGX][4 fields] then [2][NGY][4]
        TF* prof = gbase + 2*4*(NGX + NGY);   // [NPROF][PLEV]

        // Warps 0-8 own the face rows fy = 0..8 (fx = lane); warp 9 owns the
        // last face column fx = 32 of the rows fy = 0..7.  A warp thus reads
        // one contiguous plane row.
        const int tid = threadIdx.x;
        const int warp = tid >> 5, lane = tid & 31;
        const int fx = warp < NFY ? lane : FTX;
        const int fy = warp < NFY ? warp : lane;
        const bool face = warp < NFY || lane < FTY;
        const bool face_x = face && fy < FTY;
        const bool face_y = face && fx < FTX;
        const int i0 = d.istart + vb.x*FTX;
        const int j0 = d.jstart + vb.y*FTY;
        const int i = i0 + fx, j = j0 + fy;
        const bool cell = fx < FTX && fy < FTY && i < d.iend && j < d.jend;
        const int k0 = d.kstart + vb.z*kchunk;
        const int k1 = min(k0 + kchunk, d.kend);
        const int pc = (min(fy, FTY) + FH)*FPW + (fx + FH);   // own (i, j) in a plane
        const int gxi = fy*NFX + fx, gyi = fy*FTX + fx;

        // The (at most) two plane elements this thread copies per plane.
        const int e0 = tid, e1 = tid + NTHR;
        int go0, go1;
        bool v0, v1;
        {
            const int pj = e0 / FPW, pi = e0 - pj*FPW;
            const int gi = i0 - FH + pi, gj = j0 - FH + pj;
            v0 = gi < d.icells && gj < d.jcells;
            go0 = v0 ? gi + gj*d.icells : 0;
        }
        {
            const int pj = e1 / FPW, pi = e1 - pj*FPW;
            const int gi = i0 - FH + pi, gj = j0 - FH + pj;
            v1 = tid < NEL1 && gi < d.icells && gj < d.jcells;
            go1 = v1 ? gi + gj*d.icells : 0;
        }
        auto plane = [&](int slot, const TF* f, int l)
        {
            if (l > d.kcells - 1) return;
            TF* dst = sm + slot*FPS;
            const TF* src = f + (long long)l*d.ijcells;
            cp_async_el(dst + e0, v0 ? src + go0 : f, v0);
            if (tid < NEL1) cp_async_el(dst + e1, v1 ? src + go1 : f, v1);
        };

        const TF* __restrict__ u = a.u;
        const TF* __restrict__ v = a.v;
        const TF* __restrict__ w = a.w;
        const TF* __restrict__ s = a.s;
        const TF* __restrict__ ev = a.evisc;
        const long long col = cell ? (long long)i + (long long)j*d.icells : 0;
        auto colval = [&](const TF* f, int l) -> TF
        {
            l = l < 0 ? 0 : (l > d.kcells-1 ? d.kcells-1 : l);
            return __ldg(f + col + (long long)l*d.ijcells);
        };

        // Per-level constants of the chunk: index l - m0 for level l.
        const int m0 = k0 - 1;
        for (int q = tid; q < kchunk + 2; q += NTHR)
        {
            const int l = min(m0 + q, d.kcells - 1);
            prof[0*PLEV + q] = pr.dzhi[l];
            prof[1*PLEV + q] = pr.rhorefh[l];
            prof[2*PLEV + q] = pr.rhoref[l];
            prof[3*PLEV + q] = pr.dzi[l];
            prof[4*PLEV + q] = TF(GRAV)/pr.threfh[l];
            prof[7*PLEV + q] = pr.thbh[l];
            prof[5*PLEV + q] = pr.zfac[l];
            prof[6*PLEV + q] = pr.zfach[l];
        }

        // Planes of the first three iterations (m0 .. m0+2).
        for (int l = m0; l <= m0+3; ++l)
        {
            plane(SU + l%4, u, l); plane(SV + l%4, v, l); plane(SE + l%4, ev, l);
            if (l > m0) plane(SW + l%3, w, l);
            if (SCAL && l < m0+3) plane(SS + l%3, s, l);
        }
        cp_async_commit();

        // Register queues of the own column: u, v, s hold levels m-2 .. m+3,
        // w holds m-1 .. m+4.
        TF qu[6], qv[6], qw[6], qs[6];
        if (cell)
        {
            #pragma unroll
            for (int q=0; q<6; ++q)
            {
                qu[q] = colval(u, m0-2+q);
                qv[q] = colval(v, m0-2+q);
                qw[q] = colval(w, m0-1+q);
                qs[q] = (SCAL || BUOY) ? colval(s, m0-2+q) : TF(0);
            }
        }
        TF ufb = 0, uft = 0, vfb = 0, vft = 0, sfb = 0, sft = 0;
        if (SURF && cell)
        {
            ufb = a.u_fluxbot[col]; uft = a.u_fluxtop[col];
            vfb = a.v_fluxbot[col]; vft = a.v_fluxtop[col];
            if (SCAL) { sfb = a.s_fluxbot[col]; sft = a.s_fluxtop[col]; }
        }

        const TF dxi = dxi_of<TF>(d), dyi = dyi_of<TF>(d);
        const TF visc = a.visc, svisc = a.svisc, tpri = a.tpri;
        TF gzu_b = 0, gzv_b = 0, gzw_b = 0, gzs_b = 0;

        cp_async_wait_all();
        __syncthreads();

        for (int m = m0; m < k1; ++m)
        {
            const int buf = (m - m0) & 1;
            TF* gx = gbase + buf*4*NGX;
            TF* gy = gbase + 2*4*NGX + buf*4*NGY;
            const TF* U0 = sm + (SU + m%4)*FPS + pc;
            const TF* U1 = sm + (SU + (m+1)%4)*FPS + pc;
            const TF* V0 = sm + (SV + m%4)*FPS + pc;
            const TF* V1 = sm + (SV + (m+1)%4)*FPS + pc;
            const TF* W1 = sm + (SW + (m+1)%3)*FPS + pc;
            const TF* S0 = sm + (SS + m%3)*FPS + pc;
            const TF* E0 = sm + (SE + m%4)*FPS + pc;
            const TF* E1 = sm + (SE + (m+1)%4)*FPS + pc;
            #define PL(P, dx, dy) (P)[(dy)*FPW + (dx)]

            const bool write = cell && m >= k0;
            const bool wlev = m+1 > d.kstart && m+1 < d.kend;
            const long long c = col + (long long)m*d.ijcells;
            // Early loads: the tendencies this iteration updates and the queue
            // entries of the next iteration.
            TF tu = 0, tv = 0, tw = 0, ts = 0;
            if (write)
            {
                tu = a.ut[c]; tv = a.vt[c];
                if (wlev) tw = a.wt[c + d.ijcells];
                if (SCAL) ts = a.st[c];
            }
            TF nu = 0, nv = 0, nw = 0, ns = 0;
            if (cell)
            {
                nu = colval(u, m+4); nv = colval(v, m+4); nw = colval(w, m+5);
                if (SCAL || BUOY) ns = colval(s, m+4);
            }

            const int lq = m + 1 - m0;      // index of level m+1 in prof
            const TF dzhi1 = prof[0*PLEV + lq];

            // ---- faces: shear stresses and total fluxes ----
            TF txz = 0, tyz = 0;
            if (face)
            {
                const TF txy = (TF(0.25)*(PL(E0,-1,-1) + PL(E0,0,-1) + PL(E0,-1,0) + PL(E0,0,0)) + visc)
                             * ((PL(U0,0,0) - PL(U0,0,-1))*dyi + (PL(V0,0,0) - PL(V0,-1,0))*dxi);
                if constexpr (sizeof(TF) == 4)
                {
                    // tau_xz and tau_yz in one packed pair.
                    const float2 e = __ffma2_rn(__fadd2_rn(__fadd2_rn(f2(PL(E0,-1,0), PL(E0,0,-1)), f2(PL(E0,0,0), PL(E0,0,0))),
                                                           __fadd2_rn(f2(PL(E1,-1,0), PL(E1,0,-1)), f2(PL(E1,0,0), PL(E1,0,0)))),
                                                f2(0.25f, 0.25f), f2(visc, visc));
                    const float2 g = __ffma2_rn(sub2(f2(PL(U1,0,0), PL(V1,0,0)), f2(PL(U0,0,0), PL(V0,0,0))), f2(dzhi1, dzhi1),
                                                __fmul2_rn(sub2(f2(PL(W1,0,0), PL(W1,0,0)), f2(PL(W1,-1,0), PL(W1,0,-1))),
                                                           f2(dxi, dyi)));
                    const float2 t = __fmul2_rn(e, g);
                    txz = t.x; tyz = t.y;
                }
                else
                {
                    txz = (TF(0.25)*(PL(E0,-1,0) + PL(E0,0,0) + PL(E1,-1,0) + PL(E1,0,0)) + visc)
                        * ((PL(U1,0,0) - PL(U0,0,0))*dzhi1 + (PL(W1,0,0) - PL(W1,-1,0))*dxi);
                    tyz = (TF(0.25)*(PL(E0,0,-1) + PL(E0,0,0) + PL(E1,0,-1) + PL(E1,0,0)) + visc)
                        * ((PL(V1,0,0) - PL(V0,0,0))*dzhi1 + (PL(W1,0,0) - PL(W1,0,-1))*dyi);
                }
                if constexpr (sizeof(TF) == 4)
                {
                    // Float form: the x- and y-face advective fluxes of each
                    // field in packed pairs (both computed by every face
                    // thread; the plane holds the stencils of the edge faces).
                    const float2 Au = adv6x2(make_float2(i2(PL(U0,-1,0), PL(U0,0,0)), i2(PL(V0,-1,0), PL(V0,0,0))),
                                             make_float2(PL(U0,-3,0), PL(U0,0,-3)), make_float2(PL(U0,-2,0), PL(U0,0,-2)),
                                             make_float2(PL(U0,-1,0), PL(U0,0,-1)), make_float2(PL(U0,0,0), PL(U0,0,0)),
                                             make_float2(PL(U0,1,0), PL(U0,0,1)), make_float2(PL(U0,2,0), PL(U0,0,2)));
                    const float2 Av = adv6x2(make_float2(i2(PL(U0,0,-1), PL(U0,0,0)), i2(PL(V0,0,-1), PL(V0,0,0))),
                                             make_float2(PL(V0,-3,0), PL(V0,0,-3)), make_float2(PL(V0,-2,0), PL(V0,0,-2)),
                                             make_float2(PL(V0,-1,0), PL(V0,0,-1)), make_float2(PL(V0,0,0), PL(V0,0,0)),
                                             make_float2(PL(V0,1,0), PL(V0,0,1)), make_float2(PL(V0,2,0), PL(V0,0,2)));
                    const float2 Aw = adv6x2(make_float2(i2(PL(U0,0,0), PL(U1,0,0)), i2(PL(V0,0,0), PL(V1,0,0))),
                                             make_float2(PL(W1,-3,0), PL(W1,0,-3)), make_float2(PL(W1,-2,0), PL(W1,0,-2)),
                                             make_float2(PL(W1,-1,0), PL(W1,0,-1)), make_float2(PL(W1,0,0), PL(W1,0,0)),
                                             make_float2(PL(W1,1,0), PL(W1,0,1)), make_float2(PL(W1,2,0), PL(W1,0,2)));
                    float2 As = make_float2(0.f, 0.f);
                    if (SCAL)
                    {
                        if (LIM)
                            As = make_float2(lim_flux(PL(U0,0,0), PL(S0,-2,0), PL(S0,-1,0), PL(S0,0,0), PL(S0,1,0), 0),
                                             lim_flux(PL(V0,0,0), PL(S0,0,-2), PL(S0,0,-1), PL(S0,0,0), PL(S0,0,1), 0));
                        else
                            As = adv6x2(make_float2(PL(U0,0,0), PL(V0,0,0)),
                                        make_float2(PL(S0,-3,0), PL(S0,0,-3)), make_float2(PL(S0,-2,0), PL(S0,0,-2)),
                                        make_float2(PL(S0,-1,0), PL(S0,0,-1)), make_float2(PL(S0,0,0), PL(S0,0,0)),
                                        make_float2(PL(S0,1,0), PL(S0,0,1)), make_float2(PL(S0,2,0), PL(S0,0,2)));
                    }
                    // Normal diffusive fluxes of u (x) and v (y), and of s in
                    // x and y, in packed pairs.
                    const float2 eo = f2(PL(E0,-1,0), PL(E0,0,-1));
                    const float2 h2 = f2(dxi, dyi);
                    const float2 Duv = __fmul2_rn(__fmul2_rn(__fadd2_rn(eo, f2(visc, visc)), f2(2.f, 2.f)),
                                                  __fmul2_rn(sub2(f2(PL(U0,0,0), PL(V0,0,0)), f2(PL(U0,-1,0), PL(V0,0,-1))), h2));
                    float2 Ds = f2(0.f, 0.f);
                    if (SCAL)
                        Ds = __fmul2_rn(__ffma2_rn(__fmul2_rn(__fadd2_rn(eo, f2(PL(E0,0,0), PL(E0,0,0))), f2(0.5f, 0.5f)),
                                                   f2(tpri, tpri), f2(svisc, svisc)),
                                        __fmul2_rn(sub2(f2(PL(S0,0,0), PL(S0,0,0)), f2(PL(S0,-1,0), PL(S0,0,-1))), h2));
                    // The four fields' fluxes of a face are adjacent: one
                    // 16-byte store per face.
                    if (face_x)
                        reinterpret_cast<float4*>(gx)[gxi] = make_float4(Duv.x - Au.x, txy - Av.x, txz - Aw.x,
                                                                         SCAL ? Ds.x - As.x : 0.f);
                    if (face_y)
                        reinterpret_cast<float4*>(gy)[gyi] = make_float4(txy - Au.y, Duv.y - Av.y, tyz - Aw.y,
                                                                         SCAL ? Ds.y - As.y : 0.f);
                }
                else
                {
                    if (face_x)
                    {
                        // u at the cell centre i-1.
                        {
                            const TF uw = i2(PL(U0,-1,0), PL(U0,0,0));
                            const TF A = adv6(uw, PL(U0,-3,0), PL(U0,-2,0), PL(U0,-1,0), PL(U0,0,0), PL(U0,1,0), PL(U0,2,0));
                            const TF D = TF(2)*(PL(E0,-1,0) + visc)*(PL(U0,0,0) - PL(U0,-1,0))*dxi;
                            gx[(gxi)*4 + 0] = D - A;
                        }
                        // v at (i-1/2, j-1/2).
                        {
                            const TF uw = i2(PL(U0,0,-1), PL(U0,0,0));
                            const TF A = adv6(uw, PL(V0,-3,0), PL(V0,-2,0), PL(V0,-1,0), PL(V0,0,0), PL(V0,1,0), PL(V0,2,0));
                            gx[(gxi)*4 + 1] = txy - A;
                        }
                        // w at (i-1/2, m+1/2).
                        {
                            const TF uw = i2(PL(U0,0,0), PL(U1,0,0));
                            const TF A = adv6(uw, PL(W1,-3,0), PL(W1,-2,0), PL(W1,-1,0), PL(W1,0,0), PL(W1,1,0), PL(W1,2,0));
                            gx[(gxi)*4 + 2] = txz - A;
                        }
                        if (SCAL)
                        {
                            const TF uw = PL(U0,0,0);
                            const TF A = LIM ? lim_flux(uw, PL(S0,-2,0), PL(S0,-1,0), PL(S0,0,0), PL(S0,1,0), 0)
                                             : adv6(uw, PL(S0,-3,0), PL(S0,-2,0), PL(S0,-1,0), PL(S0,0,0), PL(S0,1,0), PL(S0,2,0));
                            const TF D = (TF(0.5)*(PL(E0,-1,0) + PL(E0,0,0))*tpri + svisc)*(PL(S0,0,0) - PL(S0,-1,0))*dxi;
                            gx[(gxi)*4 + 3] = D - A;
                        }
                    }
                    if (face_y)
                    {
                        // u at (i-1/2, j-1/2).
                        {
                            const TF vs = i2(PL(V0,-1,0), PL(V0,0,0));
                            const TF A = adv6(vs, PL(U0,0,-3), PL(U0,0,-2), PL(U0,0,-1), PL(U0,0,0), PL(U0,0,1), PL(U0,0,2));
                            gy[(gyi)*4 + 0] = txy - A;
                        }
                        // v at the cell centre j-1.
                        {
                            const TF vs = i2(PL(V0,0,-1), PL(V0,0,0));
                            const TF A = adv6(vs, PL(V0,0,-3), PL(V0,0,-2), PL(V0,0,-1), PL(V0,0,0), PL(V0,0,1), PL(V0,0,2));
                            const TF D = TF(2)*(PL(E0,0,-1) + visc)*(PL(V0,0,0) - PL(V0,0,-1))*dyi;
                            gy[(gyi)*4 + 1] = D - A;
                        }
                        // w at (j-1/2, m+1/2).
                        {
                            const TF vs = i2(PL(V0,0,0), PL(V1,0,0));
                            const TF A = adv6(vs, PL(W1,0,-3), PL(W1,0,-2), PL(W1,0,-1), PL(W1,0,0), PL(W1,0,1), PL(W1,0,2));
                            gy[(gyi)*4 + 2] = tyz - A;
                        }
                        if (SCAL)
                        {
                            const TF vs = PL(V0,0,0);
                            const TF A = LIM ? lim_flux(vs, PL(S0,0,-2), PL(S0,0,-1), PL(S0,0,0), PL(S0,0,1), 0)
                                             : adv6(vs, PL(S0,0,-3), PL(S0,0,-2), PL(S0,0,-1), PL(S0,0,0), PL(S0,0,1), PL(S0,0,2));
                            const TF D = (TF(0.5)*(PL(E0,0,-1) + PL(E0,0,0))*tpri + svisc)*(PL(S0,0,0) - PL(S0,0,-1))*dyi;
                            gy[(gyi)*4 + 3] = D - A;
                        }
                    }
                }
            }

            // ---- vertical faces of the own column ----
            TF gzu_t = 0, gzv_t = 0, gzw_t = 0, gzs_t = 0, buoy = 0;
            if (cell)
            {
                const int kf = m + 1;
                const int ot = face_order_full(d, kf);
                const TF rhoh1 = prof[1*PLEV + lq];
                // u and v: diffusive flux from the shear stress of the same
                // face, or the surface model's flux at the walls.
                const TF du = (SURF && kf == d.kstart) ? -ufb : ((SURF && kf == d.kend) ? -uft : txz);
                const TF dv = (SURF && kf == d.kstart) ? -vfb : ((SURF && kf == d.kend) ? -vft : tyz);
                if constexpr (sizeof(TF) == 4)
                {
                    const float2 A = zadv2(qu, qv, f2(i2(PL(W1,-1,0), PL(W1,0,0)), i2(PL(W1,0,-1), PL(W1,0,0))), ot);
                    const float2 g = __fmul2_rn(f2(rhoh1, rhoh1), sub2(f2(du, dv), A));
                    gzu_t = g.x; gzv_t = g.y;
                }
                else
                {
                    gzu_t = rhoh1*(du - zadv(qu, i2(PL(W1,-1,0), PL(W1,0,0)), ot));
                    gzv_t = rhoh1*(dv - zadv(qv, i2(PL(W1,0,-1), PL(W1,0,0)), ot));
                }
                // Float form, interior levels: the vertical advective fluxes of
                // w (through full level kf) and of s (through half level kf),
                // both 6th/5th order, in one packed pair.
                bool paired = false;
                float2 aws = make_float2(0.f, 0.f);
                if constexpr (sizeof(TF) == 4 && SCAL && !LIM)
                {
                    if (ot == 6 && kf < d.kend && face_order_w(d, kf) == 6)
                    {
                        aws = adv6x2(f2(i2(qw[2], qw[3]), qw[2]), f2(qw[0], qs[0]), f2(qw[1], qs[1]), f2(qw[2], qs[2]),
                                     f2(qw[3], qs[3]), f2(qw[4], qs[4]), f2(qw[5], qs[5]));
                        paired = true;
                    }
                }
                if (SCAL)
                {
                    const TF ds = (SURF && kf == d.kstart) ? -sfb : ((SURF && kf == d.kend) ? -sft
                                : (TF(0.5)*(PL(E0,0,0) + PL(E1,0,0))*tpri + svisc)*(qs[3] - qs[2])*dzhi1);
                    TF as;
                    if (paired) as = aws.y;
                    else if (LIM)
                    {
                        const int side = kf == d.kstart+1 ? -1 : (kf == d.kend-1 ? 1 : 0);
                        as = ot ? lim_flux(qw[2], qs[1], qs[2], qs[3], qs[4], side) : TF(0);
                    }
                    else as = zadv(qs, qw[2], ot);
                    gzs_t = rhoh1*(ds - as);
                }
                // w: the full level kf between w(kf) and w(kf+1).
                if (kf < d.kend)
                {
                    const int ow = face_order_w(d, kf);
                    const TF dw = TF(2)*(PL(E1,0,0) + visc)*(qw[3] - qw[2])*prof[3*PLEV + lq];
                    TF aw;
                    if (paired) aw = aws.x;
                    else if (ow == 6) aw = adv6(i2(qw[2], qw[3]), qw[0], qw[1], qw[2], qw[3], qw[4], qw[5]);
                    else if (ow == 4) aw = i2(qw[2], qw[3])*i4ws(qw[1], qw[2], qw[3], qw[4])
                                         - fabs(i2(qw[2], qw[3]))*i3ws(qw[1], qw[2], qw[3], qw[4]);
                    else aw = i2(qw[2], qw[3])*i2(qw[2], qw[3]);
                    gzw_t = prof[2*PLEV + lq]*(dw - aw);
                }
                if (BUOY && wlev)
                    buoy = prof[4*PLEV + lq]*(i2(qs[2], qs[3]) - prof[7*PLEV + lq]);
            }
            #undef PL

            // The planes of iteration m+1 were issued two iterations ago; the
            // last iteration's group may stay in flight.
            asm volatile("cp.async.wait_group 1;\n" ::: "memory");
            __syncthreads();

            // Planes first used by iteration m+3 into the slots that
            // iteration m freed.
            if (m + 3 < k1)
            {
                plane(SU + (m+4)%4, u, m+4);
                plane(SV + (m+4)%4, v, m+4);
                plane(SW + (m+4)%3, w, m+4);
                plane(SE + (m+4)%4, ev, m+4);
                if (SCAL) plane(SS + (m+3)%3, s, m+3);
            }
            cp_async_commit();

            if (write)
            {
                const int gx0 = gxi, gy0 = gyi;
                const TF zf = prof[5*PLEV + lq - 1];
                if constexpr (sizeof(TF) == 4)
                {
                    // The four fields' face fluxes in one 16-byte load per face;
                    // u/v and w/s in packed pairs.
                    const float4 xa = reinterpret_cast<const float4*>(gx)[gx0];
                    const float4 xb = reinterpret_cast<const float4*>(gx)[gx0 + 1];
                    const float4 ya = reinterpret_cast<const float4*>(gy)[gy0];
                    const float4 yb = reinterpret_cast<const float4*>(gy)[gy0 + FTX];
                    {
                        const float2 dgx = sub2(f2(xb.x, xb.y), f2(xa.x, xa.y));
                        const float2 dgy = sub2(f2(yb.x, yb.y), f2(ya.x, ya.y));
                        const float2 dgz = sub2(f2(gzu_t, gzv_t), f2(gzu_b, gzv_b));
                        const float2 t = __ffma2_rn(dgz, f2(zf, zf), __ffma2_rn(dgy, f2(dyi, dyi),
                                                    __ffma2_rn(dgx, f2(dxi, dxi), f2(tu, tv))));
                        a.ut[c] = t.x; a.vt[c] = t.y;
                    }
                    if constexpr (SCAL)
                    {
                        const float2 dgx = sub2(f2(xb.z, xb.w), f2(xa.z, xa.w));
                        const float2 dgy = sub2(f2(yb.z, yb.w), f2(ya.z, ya.w));
                        const float2 dgz = sub2(f2(gzw_t, gzs_t), f2(gzw_b, gzs_b));
                        const float2 t = __ffma2_rn(dgz, f2(prof[6*PLEV + lq], zf), __ffma2_rn(dgy, f2(dyi, dyi),
                                                    __ffma2_rn(dgx, f2(dxi, dxi), f2(tw + buoy, ts))));
                        if (wlev) a.wt[c + d.ijcells] = t.x;
                        a.st[c] = t.y;
                    }
                    else if (wlev)
                        a.wt[c + d.ijcells] = tw + (xb.z - xa.z)*dxi + (yb.z - ya.z)*dyi
                                                 + (gzw_t - gzw_b)*prof[6*PLEV + lq] + buoy;
                }
                else
                {
                    a.ut[c] = tu + (gx[(gx0 + 1)*4 + 0] - gx[(gx0)*4 + 0])*dxi
                                 + (gy[(gy0 + FTX)*4 + 0] - gy[(gy0)*4 + 0])*dyi + (gzu_t - gzu_b)*zf;
                    a.vt[c] = tv + (gx[(gx0 + 1)*4 + 1] - gx[(gx0)*4 + 1])*dxi
                                 + (gy[(gy0 + FTX)*4 + 1] - gy[(gy0)*4 + 1])*dyi + (gzv_t - gzv_b)*zf;
                    if (wlev)
                        a.wt[c + d.ijcells] = tw + (gx[(gx0 + 1)*4 + 2] - gx[(gx0)*4 + 2])*dxi
                                                 + (gy[(gy0 + FTX)*4 + 2] - gy[(gy0)*4 + 2])*dyi
                                                 + (gzw_t - gzw_b)*prof[6*PLEV + lq] + buoy;
                    if (SCAL)
                        a.st[c] = ts + (gx[(gx0 + 1)*4 + 3] - gx[(gx0)*4 + 3])*dxi
                                     + (gy[(gy0 + FTX)*4 + 3] - gy[(gy0)*4 + 3])*dyi + (gzs_t - gzs_b)*zf;
                }
            }

            gzu_b = gzu_t; gzv_b = gzv_t; gzw_b = gzw_t; gzs_b = gzs_t;
            #pragma unroll
            for (int q=0; q<5; ++q) { qu[q] = qu[q+1]; qv[q] = qv[q+1]; qw[q] = qw[q+1]; qs[q] = qs[q+1]; }
            qu[5] = nu; qv[5] = nv; qw[5] = nw; qs[5] = ns;
        }
        cp_async_wait_all();
    }

    template<typename TF, bool SURF, bool SCAL, bool BUOY, bool LIM = false>
    static void launch_flux_t(const Dims& d, const Prof<TF>& pr, const TendArgs<TF>& a, int kchunk, cudaStream_t s)
    {
        const size_t smem = flux_smem<TF>();
        kchunk = min(auto_kchunk(kchunk, (long long)((d.itot + FTX - 1)/FTX)*((d.jtot + FTY - 1)/FTY), d.ktot),
                     FKCHUNK_MAX);
        dim3 grid((d.itot + FTX - 1)/FTX, (d.jtot + FTY - 1)/FTY, (d.ktot + kchunk - 1)/kchunk);
        launch_body<TendFluxP<TF>, tend_flux_body<TF, SURF, SCAL, BUOY, LIM>, NTHR, FluxOcc<TF>::v>(
            grid, dim3(NTHR), smem, s, TendFluxP<TF>{d, pr, a, kchunk});
        count_launch();
    }

    // Advec_2i5 + Diff_smag2 (+ buoyancy) in flux form; igc, jgc >= 3.
    template<typename TF>
    void launch_tendency_flux(const Dims& d, const Prof<TF>& pr, const TendArgs<TF>& a, bool surf, bool scal,
                              bool buoy, bool lim, int kchunk, cudaStream_t s)
    {
        if (lim && scal)
        {
            if (surf && buoy) launch_flux_t<TF, true, true, true, true>(d, pr, a, kchunk, s);
            else if (surf) launch_flux_t<TF, true, true, false, true>(d, pr, a, kchunk, s);
            else if (buoy) launch_flux_t<TF, false, true, true, true>(d, pr, a, kchunk, s);
            else launch_flux_t<TF, false, true, false, true>(d, pr, a, kchunk, s);
            return;
        }
        const int mask = (surf ? 4 : 0) | (scal ? 2 : 0) | (buoy ? 1 : 0);
        switch (mask)
        {
            case 0: launch_flux_t<TF, false, false, false>(d, pr, a, kchunk, s); break;
            case 1: launch_flux_t<TF, false, false, true >(d, pr, a, kchunk, s); break;
            case 2: launch_flux_t<TF, false, true,  false>(d, pr, a, kchunk, s); break;
            case 3: launch_flux_t<TF, false, true,  true >(d, pr, a, kchunk, s); break;
            case 4: launch_flux_t<TF, true,  false, false>(d, pr, a, kchunk, s); break;
            case 5: launch_flux_t<TF, true,  false, true >(d, pr, a, kchunk, s); break;
            case 6: launch_flux_t<TF, true,  true,  false>(d, pr, a, kchunk, s); break;
            default: launch_flux_t<TF, true, true,  true >(d, pr, a, kchunk, s); break;
        }
    }

    template void launch_tendency_flux<double>(const Dims&, const Prof<double>&, const TendArgs<double>&, bool, bool, bool, bool, int, cudaStream_t);
    template void launch_tendency_flux<float>(const Dims&, const Prof<float>&, const TendArgs<float>&, bool, bool, bool, bool, int, cudaStream_t);
}
