// mhh_visc_planes.cu -- Smagorinsky eddy viscosity with every shear term of
// the strain rate computed once.
//
// The strain rate of include/diff_kernels.h:34-142 sums, per cell, three
// squared normal gradients and the squared shear of the 12 edges around the
// cell (4 each in the xy, xz and yz planes, weight 1/8).  Each edge is shared
// by four cells, so here it is computed once: a block owns a 32 x 8 tile of
// columns and marches upward through a chunk of levels; its 33 x 9 edge
// threads compute per level the xy edges of the level and the xz and yz
// edges of the half level above into shared memory, and the 32 x 8 cell
// threads add the twelve edges and the normal gradients.  The edges of the
// half level below come from the previous level's buffer.
//
// The planes u, v, w of the levels m and m+1 (1-cell halo) are staged in
// shared memory by cp.async two levels ahead of their use; theta comes from
// a register queue of the own column.  N^2 follows src/thermo_dry.cxx:64-75
// and the eddy viscosity src/diff_smag2.cxx:148-269.  At the first level with
// the surface model the vertical shear of u and v is the model's dudz, dvdz
// and the edge terms keep only the w gradients (include/diff_kernels.h:57-103);
// that level is computed from the planes directly.
#include "mhh_kernels.cuh"
#include "mhh_batchable.cuh"

namespace mhh
{
    namespace
    {
        constexpr int VTX = 32, VTY = 8, VH = 1;
        constexpr int VPW = VTX + 2*VH;         // 34
        constexpr int VPH = VTY + 2*VH;         // 10
        constexpr int VPS = VPW*VPH;            // 340
        constexpr int VNX = VTX + 1, VNY = VTY + 1;
        constexpr int VNT = 320;
        constexpr int VKCHUNK_MAX = 64;
        // Plane slots: u, v, w 4 each; level l of a field in slot base + l % 4.
        constexpr int VSU = 0, VSV = 4, VSW = 8, VNSLOT = 12;
        constexpr int VNEL1 = VPS - VNT;        // threads that copy a second element
        // Edge buffers: xy [VNY][VNX] for two levels (written and read in the
        // same iteration); xz [VTY][VNX] and yz [VNY][VTX] for three half
        // levels (an iteration reads the half levels below and above its
        // level while the next one writes the following half level).
        constexpr int NXY = VNY*VNX, NXZ = VTY*VNX, NYZ = VNY*VTX;

        constexpr int VPLEV = VKCHUNK_MAX + 2;  // per-level constants of levels m0 .. m0+kchunk+1

        template<typename TF>
        size_t visc_smem() { return sizeof(TF)*(size_t(VNSLOT)*VPS + 2*NXY + 3*(NXZ + NYZ) + 5*VPLEV); }

        // The eddy viscosity from S^2 and N^2, src/diff_smag2.cxx:171-174:
        // mlen^2 sqrt(S^2) sqrt(1 - min(N^2/(S^2 Pr), 1 - 1e-9)).  In double the
        // reference's operation order.  In float, where 1 - 1e-9 rounds to 1,
        // the same value as mlen^2 sqrt(S^2 - N^2/Pr) for N^2/Pr < S^2 and 0
        // otherwise, without the two divisions.
        template<typename TF>
        __device__ __forceinline__ TF evisc_of(TF ml2, TF s2, TF n2, TF tpr, TF tpri)
        {
            if constexpr (sizeof(TF) == 8)
            {
                TF ratio = n2 / s2 / tpr;
                ratio = fmin(ratio, TF(1.-DSMALL));
                return ml2*sqrt(s2)*sqrt(TF(1) - ratio);
            }
            else
            {
                const TF t = n2*tpri;
                return t < s2 ? ml2*sqrt(s2 - t) : TF(0);
            }
        }
    }

    template<typename TF>
    __device__ __forceinline__ void cp_async_v(TF* dst, const TF* src, bool valid)
    {
        const unsigned s = (unsigned)__cvta_generic_to_shared(dst);
        const int n = valid ? (int)sizeof(TF) : 0;
        if constexpr (sizeof(TF) == 4)
            asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;\n" :: "r"(s), "l"(src), "r"(n) : "memory");
        else
            asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;\n" :: "r"(s), "l"(src), "r"(n) : "memory");
    }

    template<typename TF> struct ViscPlanesP
    {
        Dims d; Prof<TF> pr;
        const TF *u, *v, *w, *th;
        TF* evisc;
        const TF* mlen2;
        const double *dudz, *dvdz, *dbdz;
        TF tpr; int kchunk;
    };

    template<typename TF, bool SURF, bool THERMO>
    __device__ __forceinline__ void visc_planes_body(const ViscPlanesP<TF>& P, const VBlock& vb)
    {
        const Dims& d = P.d;
        const Prof<TF>& pr = P.pr;
        const TF* __restrict__ u = P.u; const TF* __restrict__ v = P.v; const TF* __restrict__ w = P.w;
        const TF* __restrict__ th = P.th;
        TF* __restrict__ evisc = P.evisc;
        const TF* __restrict__ mlen2 = P.mlen2;
        const double* __restrict__ dudz = P.dudz; const double* __restrict__ dvdz = P.dvdz;
        const double* __restrict__ dbdz = P.dbdz;
        const TF tpr = P.tpr;
        const int kchunk = P.kchunk;
        extern __shared__ __align__(16) unsigned char smem_raw[];
        TF* sm = reinterpret_cast<TF*>(smem_raw);
        TF* exy = sm + VNSLOT*VPS;          // [2][NXY], by iteration parity
        TF* exz = exy + 2*NXY;              // [3][NXZ], by half level % 3
        TF* eyz = exz + 3*NXZ;              // [3][NYZ], by half level % 3
        TF* lev = eyz + 3*NYZ;              // [5][VPLEV]: dzhi, dzi, g/thref, mlen2, spare

        // Warps 0-8 own the edge rows ey = 0..8 (ex = lane); warp 9 owns the
        // last edge column ex = 32 of the rows ey = 0..8.
        const int tid = threadIdx.x;
        const int warp = tid >> 5, lane = tid & 31;
        const int ex = warp < VNY ? lane : VTX;
        const int ey = warp < VNY ? warp : lane;
        const bool edge = warp < VNY || lane < VNY;
        const int i0 = d.istart + vb.x*VTX, j0 = d.jstart + vb.y*VTY;
        const int i = i0 + ex, j = j0 + ey;
        const bool cell = ex < VTX && ey < VTY && i < d.iend && j < d.jend;
        const int k0 = d.kstart + vb.z*kchunk;
        const int k1 = min(k0 + kchunk, d.kend);
        const int pc = (min(ey, VTY) + VH)*VPW + (ex + VH);

        const int e0 = tid, e1 = tid + VNT;
        int go0, go1;
        bool v0, v1;
        {
            const int pj = e0 / VPW, pi = e0 - pj*VPW;
            const int gi = i0 - VH + pi, gj = j0 - VH + pj;
            v0 = gi < d.icells && gj < d.jcells;
            go0 = v0 ? gi + gj*d.icells : 0;
        }
        {
            const int pj = e1 / VPW, pi = e1 - pj*VPW;
            const int gi = i0 - VH + pi, gj = j0 - VH + pj;
            v1 = tid < VNEL1 && gi < d.icells && gj < d.jcells;
            go1 = v1 ? gi + gj*d.icells : 0;
        }
        auto plane = [&](int slot, const TF* f, int l)
        {
            if (l > d.kcells - 1) return;
            TF* dst = sm + slot*VPS;
            const TF* src = f + (long long)l*d.ijcells;
            cp_async_v(dst + e0, v0 ? src + go0 : f, v0);
            if (tid < VNEL1) cp_async_v(dst + e1, v1 ? src + go1 : f, v1);
        };

        // Iteration m uses the planes of m and m+1; the loop starts one level
        // below the chunk to produce the edges of the chunk's bottom half level.
        const int m0 = k0 - 1;
        for (int q = tid; q < kchunk + 2; q += VNT)
        {
            const int l = min(m0 + q, d.kcells - 1);
            lev[0*VPLEV + q] = pr.dzhi[l];
            lev[1*VPLEV + q] = pr.dzi[l];
            lev[2*VPLEV + q] = TF(GRAV)/pr.thref[l];
            lev[3*VPLEV + q] = mlen2[l];
        }
        for (int l = m0; l <= m0 + 3; ++l) { plane(VSU + l%4, u, l); plane(VSV + l%4, v, l); plane(VSW + l%4, w, l); }
        asm volatile("cp.async.commit_group;\n" ::: "memory");

        const long long col = cell ? (long long)i + (long long)j*d.icells : 0;
        // Theta queue of the own column: levels m-1, m, m+1.
        TF tq0 = 0, tq1 = 0, tq2 = 0;
        if (THERMO && cell)
        {
            tq0 = __ldg(th + col + (long long)(m0-1 < 0 ? 0 : m0-1)*d.ijcells);
            tq1 = __ldg(th + col + (long long)m0*d.ijcells);
            tq2 = __ldg(th + col + (long long)(m0+1)*d.ijcells);
        }
        const TF dxi = dxi_of<TF>(d), dyi = dyi_of<TF>(d);
        const TF tpri = TF(1)/tpr;

        asm volatile("cp.async.wait_group 0;\n" ::: "memory");
        __syncthreads();

        for (int m = m0; m < k1; ++m)
        {
            const int lq = m - m0;           // index of level m in lev
            const int b = (m - m0) & 1;      // xy buffer of this iteration
            const int bt = (m + 1) % 3;      // xz, yz buffer of half level m+1
            const int bb = m % 3;            // xz, yz buffer of half level m
            const TF* U0 = sm + (VSU + m%4)*VPS + pc;
            const TF* U1 = sm + (VSU + (m+1)%4)*VPS + pc;
            const TF* V0 = sm + (VSV + m%4)*VPS + pc;
            const TF* V1 = sm + (VSV + (m+1)%4)*VPS + pc;
            const TF* W0 = sm + (VSW + m%4)*VPS + pc;
            const TF* W1 = sm + (VSW + (m+1)%4)*VPS + pc;
            #define Q(P, dx, dy) (P)[(dy)*VPW + (dx)]

            TF thn = 0;
            if (THERMO && cell && m + 2 < d.kcells) thn = __ldg(th + col + (long long)(m+2)*d.ijcells);

            // ---- edges: xy at level m, xz and yz at half level m+1 ----
            if (edge)
            {
                const TF dzt = lev[0*VPLEV + lq + 1];
                exy[b*NXY + ey*VNX + ex] = sq((Q(U0,0,0) - Q(U0,0,-1))*dyi + (Q(V0,0,0) - Q(V0,-1,0))*dxi);
                if constexpr (sizeof(TF) == 4)
                {
                    // The xz and yz edges in one packed pair.
                    const float2 m1 = make_float2(-1.f, -1.f);
                    const float2 g = __ffma2_rn(__ffma2_rn(make_float2(Q(U0,0,0), Q(V0,0,0)), m1, make_float2(Q(U1,0,0), Q(V1,0,0))),
                                                make_float2(dzt, dzt),
                                                __fmul2_rn(__ffma2_rn(make_float2(Q(W1,-1,0), Q(W1,0,-1)), m1,
                                                                      make_float2(Q(W1,0,0), Q(W1,0,0))),
                                                           make_float2(dxi, dyi)));
                    const float2 g2 = __fmul2_rn(g, g);
                    if (ey < VTY) exz[bt*NXZ + ey*VNX + ex] = g2.x;
                    if (ex < VTX) eyz[bt*NYZ + ey*VTX + ex] = g2.y;
                }
                else
                {
                    if (ey < VTY)
                        exz[bt*NXZ + ey*VNX + ex] = sq((Q(U1,0,0) - Q(U0,0,0))*dzt + (Q(W1,0,0) - Q(W1,-1,0))*dxi);
                    if (ex < VTX)
                        eyz[bt*NYZ + ey*VTX + ex] = sq((Q(V1,0,0) - Q(V0,0,0))*dzt + (Q(W1,0,0) - Q(W1,0,-1))*dyi);
                }
            }

            // Normal gradients and, at the surface level, the special terms,
            // read before the barrier that releases the planes.
            TF acc = 0;
            const bool write = cell && m >= k0;
            if (write)
            {
                const TF dzi = lev[1*VPLEV + lq];
                acc = sq((Q(U0,1,0) - Q(U0,0,0))*dxi)
                    + sq((Q(V0,0,1) - Q(V0,0,0))*dyi)
                    + sq((Q(W1,0,0) - Q(W0,0,0))*dzi);
                if (SURF && m == d.kstart)
                {
                    acc += TF(0.5)*sq(TF(dudz[col]))
                         + TF(0.125)*sq((Q(W0,0,0) - Q(W0,-1,0))*dxi)
                         + TF(0.125)*sq((Q(W0,1,0) - Q(W0,0,0))*dxi)
                         + TF(0.125)*sq((Q(W1,0,0) - Q(W1,-1,0))*dxi)
                         + TF(0.125)*sq((Q(W1,1,0) - Q(W1,0,0))*dxi)
                         + TF(0.5)*sq(TF(dvdz[col]))
                         + TF(0.125)*sq((Q(W0,0,0) - Q(W0,0,-1))*dyi)
                         + TF(0.125)*sq((Q(W0,0,1) - Q(W0,0,0))*dyi)
                         + TF(0.125)*sq((Q(W1,0,0) - Q(W1,0,-1))*dyi)
                         + TF(0.125)*sq((Q(W1,0,1) - Q(W1,0,0))*dyi);
                }
            }
            #undef Q

            // The planes of iteration m+1 were issued two iterations ago; the
            // last iteration's group may stay in flight.
            asm volatile("cp.async.wait_group 1;\n" ::: "memory");
            __syncthreads();
            // Planes first used by iteration m+3 into the slot that iteration
            // m freed.
            if (m + 3 < k1)
            {
                plane(VSU + (m+4)%4, u, m+4);
                plane(VSV + (m+4)%4, v, m+4);
                plane(VSW + (m+4)%4, w, m+4);
            }
            asm volatile("cp.async.commit_group;\n" ::: "memory");

            if (write)
            {
                const TF* xy = exy + b*NXY + ey*VNX + ex;
                if (!(SURF && m == d.kstart))
                {
                    const TF* zt = exz + bt*NXZ + ey*VNX + ex;
                    const TF* zb = exz + bb*NXZ + ey*VNX + ex;
                    const TF* yt = eyz + bt*NYZ + ey*VTX + ex;
                    const TF* yb = eyz + bb*NYZ + ey*VTX + ex;
                    if constexpr (sizeof(TF) == 4)
                    {
                        // Sums of the xy / xz / yz edge groups: three of the
                        // four-term sums in packed pairs.
                        const float2 s1 = __fadd2_rn(__fadd2_rn(make_float2(xy[0], zb[0]), make_float2(xy[1], zb[1])),
                                                     __fadd2_rn(make_float2(xy[VNX], zt[0]), make_float2(xy[VNX+1], zt[1])));
                        const TF sy = (yb[0] + yb[VTX]) + (yt[0] + yt[VTX]);
                        acc += TF(0.125)*s1.x + (TF(0.125)*s1.y + TF(0.125)*sy);
                    }
                    else
                    {
                        acc += TF(0.125)*(xy[0] + xy[1] + xy[VNX] + xy[VNX+1]);
                        acc += TF(0.125)*(zb[0] + zb[1] + zt[0] + zt[1])
                             + TF(0.125)*(yb[0] + yb[VTX] + yt[0] + yt[VTX]);
                    }
                }
                else
                    acc += TF(0.125)*(xy[0] + xy[1] + xy[VNX] + xy[VNX+1]);
                const TF s2 = TF(2)*acc + TF(DSMALL);
                const TF ml2 = lev[3*VPLEV + lq];
                TF ev;
                if (THERMO)
                {
                    TF n2;
                    if (SURF && m == d.kstart) n2 = TF(dbdz[col]);
                    else n2 = lev[2*VPLEV + lq]*TF(0.5)*(tq2 - tq0)*lev[1*VPLEV + lq];
                    ev = evisc_of<TF>(ml2, s2, n2, tpr, tpri);
                }
                else
                    ev = ml2*sqrt(s2);
                evisc[col + (long long)m*d.ijcells] = ev;
            }
            if (THERMO) { tq0 = tq1; tq1 = tq2; tq2 = thn; }
        }
        asm volatile("cp.async.wait_all;\n" ::: "memory");
    }

    template<typename TF, bool SURF, bool THERMO>
    static void launch_vp_t(const Dims& d, const Prof<TF>& pr, const TF* u, const TF* v, const TF* w, const TF* th,
                            TF* evisc, const TF* mlen2, const double* dudz, const double* dvdz, const double* dbdz,
                            double tpr, int kchunk, cudaStream_t s)
    {
        const size_t smem = visc_smem<TF>();
        kchunk = min(auto_kchunk(kchunk, (long long)((d.itot + VTX - 1)/VTX)*((d.jtot + VTY - 1)/VTY), d.ktot),
                     VKCHUNK_MAX);
        dim3 grid((d.itot + VTX - 1)/VTX, (d.jtot + VTY - 1)/VTY, (d.ktot + kchunk - 1)/kchunk);
        launch_body<ViscPlanesP<TF>, visc_planes_body<TF, SURF, THERMO>, VNT>(grid, dim3(VNT), smem, s,
            ViscPlanesP<TF>{d, pr, u, v, w, th, evisc, mlen2, dudz, dvdz, dbdz, TF(tpr), kchunk});
        count_launch();
    }

    // The edge-once viscosity for the surface-model and thermo cases; returns
    // false for the neutral resolved-wall case (Van Driest damping), which
    // stays on the per-cell kernel.
    template<typename TF>
    bool launch_viscosity_planes(const Dims& d, const Prof<TF>& pr, const TF* u, const TF* v, const TF* w,
                                 const TF* th, TF* evisc, const TF* mlen2, const double* dudz, const double* dvdz,
                                 const double* dbdz, double tpr, bool surf, bool thermo, int kchunk, cudaStream_t s)
    {
        if (surf && thermo) launch_vp_t<TF, true, true>(d, pr, u, v, w, th, evisc, mlen2, dudz, dvdz, dbdz, tpr, kchunk, s);
        else if (surf) launch_vp_t<TF, true, false>(d, pr, u, v, w, th, evisc, mlen2, dudz, dvdz, dbdz, tpr, kchunk, s);
        else if (thermo) launch_vp_t<TF, false, true>(d, pr, u, v, w, th, evisc, mlen2, dudz, dvdz, dbdz, tpr, kchunk, s);
        else return false;
        return true;
    }

    template bool launch_viscosity_planes<double>(const Dims&, const Prof<double>&, const double*, const double*,
        const double*, const double*, double*, const double*, const double*, const double*, const double*, double,
        bool, bool, int, cudaStream_t);
    template bool launch_viscosity_planes<float>(const Dims&, const Prof<float>&, const float*, const float*,
        const float*, const float*, float*, const float*, const double*, const double*, const double*, double,
        bool, bool, int, cudaStream_t);
}
