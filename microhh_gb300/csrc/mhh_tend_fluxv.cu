// mhh_tend_fluxv.cu -- the float form's LES tendency kernel (Advec_2i5 +
// Smagorinsky diffusion + dry buoyancy, optionally with the Monin-Obukhov
// wall fluxes and the flux limiter on the scalar), in flux form with the
// four fields' planes interleaved.
//
// The decomposition is that of k_tend_flux (mhh_tend_flux.cu): a block owns
// a 32 x 8 tile of columns and marches up a chunk of levels; its 33 x 9 face
// threads compute every x- and y-face flux of u, v, w and s once per level
// into shared memory, the 32 x 8 cell threads add the differences, and the
// vertical faces of the own column stay in registers.  What differs is the
// layout of the staged planes: iteration m reads u, v and s at full level m
// and w at half level m+1, and each plane point holds exactly these four
// values, {u_m, v_m, w_m+1, s_m}, as one float4.  The six-point stencil of
// all four fields along x or along y is then six 16-byte shared loads
// (eleven for both directions, the centre shared), and the packed FP32x2
// arithmetic pairs fields whose values arrive in adjacent registers: u with
// v and w with s, through the same face.  The eddy viscosity has a plane of
// its own.  Each thread stages one field of the interleaved plane, so that
// the copies of a warp fill 32 consecutive words (no bank conflicts).
//
// The arithmetic per face is that of the reference's kernels:
// src/advec_2i5.cxx:150-728, include/diff_kernels.h:144-484 and
// src/thermo_dry.cxx:165-181 (with LIM the scalar's advective fluxes are
// those of include/advec_monotonic.h:28-219); the sum of all fluxes is
// formed before it is added to the tendency, so the result differs from the
// reference's term-by-term accumulation by round-off only.
#include "mhh_kernels.cuh"
#include "mhh_stencil.cuh"
#include "mhh_flux.cuh"

namespace mhh
{
    namespace
    {
        constexpr int VTX = 32, VTY = 8, VH = 3;
        constexpr int VPW = 40;                 // plane row (VTX + 2*VH, padded)
        constexpr int VPH = VTY + 2*VH;         // plane rows
        constexpr int VPS = VPW*VPH;            // plane points (560)
        constexpr int VNFX = VTX + 1, VNFY = VTY + 1;
        constexpr int VNTHR = 320;
        constexpr int VKMAX = 64;
        constexpr int VNGX = VTY*VNFX;          // x-faces per level
        constexpr int VNGY = VNFY*VTX;          // y-faces per level
        constexpr int VNEL1 = VPS - VNTHR;      // threads that copy a second viscosity point
        constexpr int VNPROF = 8;
        constexpr int VPLEV = VKMAX + 2;
        // Staging of the interleaved plane: thread t copies field t % 4 of the
        // points t/4 + 80 c, c = 0..6 (80 points are two plane rows).
        constexpr int VCOPY = VPS/(VNTHR/4);    // 7
        static_assert(VCOPY*(VNTHR/4) == VPS, "plane points must split evenly");
        static_assert(VNTHR/4 == 2*VPW, "one copy round spans two plane rows");

        // Shared memory: 4 interleaved planes, 2 x (x-faces + y-faces) float4
        // flux buffers, then 4 viscosity planes and the per-level constants.
        size_t fluxv_smem()
        {
            return sizeof(float4)*(4*VPS + 2*(VNGX + VNGY)) + sizeof(float)*(4*VPS + VNPROF*VPLEV);
        }

        __device__ __forceinline__ float2 lo2(const float4& a) { return make_float2(a.x, a.y); }
        __device__ __forceinline__ float2 hi2(const float4& a) { return make_float2(a.z, a.w); }
    }

    template<bool SURF, bool SCAL, bool BUOY, bool LIM>
    __global__ void __launch_bounds__(VNTHR, 2)
    k_tend_fluxv(Dims d, Prof<float> pr, TendArgs<float> a, int kchunk)
    {
        extern __shared__ __align__(16) unsigned char smem_raw[];
        float4* P = reinterpret_cast<float4*>(smem_raw);          // [4][VPS]
        float4* G = P + 4*VPS;                                     // [2][VNGX] then [2][VNGY]
        float* E = reinterpret_cast<float*>(G + 2*(VNGX + VNGY));  // [4][VPS]
        float* prof = E + 4*VPS;                                   // [VNPROF][VPLEV]

        // Warps 0-8 own the face rows fy = 0..8 (fx = lane); warp 9 owns the
        // last face column fx = 32 of the rows fy = 0..7.
        const int tid = threadIdx.x;
        const int warp = tid >> 5, lane = tid & 31;
        const int fx = warp < VNFY ? lane : VTX;
        const int fy = warp < VNFY ? warp : lane;
        const bool face = warp < VNFY || lane < VTY;
        const bool face_x = face && fy < VTY;
        const bool face_y = face && fx < VTX;
        const int i0 = d.istart + blockIdx.x*VTX;
        const int j0 = d.jstart + blockIdx.y*VTY;
        const int i = i0 + fx, j = j0 + fy;
        const bool cell = fx < VTX && fy < VTY && i < d.iend && j < d.jend;
        const int k0 = d.kstart + blockIdx.z*kchunk;
        const int k1 = min(k0 + kchunk, d.kend);
        const int pc = (min(fy, VTY) + VH)*VPW + (fx + VH);
        const int gxi = fy*VNFX + fx, gyi = fy*VTX + fx;

        const float* __restrict__ u = a.u;
        const float* __restrict__ v = a.v;
        const float* __restrict__ w = a.w;
        const float* __restrict__ s = a.s;
        const float* __restrict__ ev = a.evisc;

        // Interleaved-plane copies of this thread: field cf of the points
        // cp0 + 80 c, i.e. plane rows cpj + 2 c at column cpi.  In a tile
        // whose halo lies inside the field (all but the last tiles in x and
        // y) every copy is valid and needs no predicate; the others check
        // each point.
        const int cf = tid & 3, cp0 = tid >> 2;
        const int cpj = cp0 / VPW, cpi = cp0 - cpj*VPW;
        const int cgi = i0 - VH + cpi, cgj = j0 - VH + cpj;
        const bool full = i0 - VH + VPW <= d.icells && j0 - VH + VPH <= d.jcells;
        const bool cuse = cf != 3 || SCAL;
        const float* csrc = cf == 0 ? u : cf == 1 ? v : cf == 2 ? w : (SCAL ? s : u);
        const float* cbase = csrc + (cgi < d.icells ? cgi + cgj*d.icells : 0);
        const int cstep = 2*d.icells;
        float* cdst = reinterpret_cast<float*>(P) + 4*cp0 + cf;
        // Viscosity-plane copies: points tid and tid + VNTHR.
        int go0, go1;
        bool v0, v1;
        {
            const int pj = tid / VPW, pi = tid - pj*VPW;
            const int gi = i0 - VH + pi, gj = j0 - VH + pj;
            v0 = gi < d.icells && gj < d.jcells;
            go0 = v0 ? gi + gj*d.icells : 0;
        }
        {
            const int e1 = tid + VNTHR;
            const int pj = e1 / VPW, pi = e1 - pj*VPW;
            const int gi = i0 - VH + pi, gj = j0 - VH + pj;
            v1 = tid < VNEL1 && gi < d.icells && gj < d.jcells;
            go1 = v1 ? gi + gj*d.icells : 0;
        }
        // Planes of iteration l: {u_l, v_l, w_l+1, s_l} and evisc_l.
        auto plane = [&](int slot, int l)
        {
            if (l > d.kcells - 1) return;
            const int lf = cf == 2 ? l + 1 : l;
            // w of the level above the top reads as zero (never used).
            const bool lok = cuse && lf <= d.kcells - 1;
            const float* src = cbase + (long long)lf*d.ijcells;
            float* dst = cdst + slot*4*VPS;
            float* de = E + slot*VPS;
            const float* se = ev + (long long)l*d.ijcells;
            if (full)
            {
                #pragma unroll
                for (int c=0; c<VCOPY; ++c)
                    cp_async_el(dst + 4*(VNTHR/4)*c, lok ? src + c*cstep : csrc, lok);
                cp_async_el(de + tid, se + go0, true);
                if (tid < VNEL1) cp_async_el(de + tid + VNTHR, se + go1, true);
            }
            else
            {
                const bool lc = lok && cgi < d.icells;
                #pragma unroll
                for (int c=0; c<VCOPY; ++c)
                {
                    const bool ok = lc && cgj + 2*c < d.jcells;
                    cp_async_el(dst + 4*(VNTHR/4)*c, ok ? src + c*cstep : csrc, ok);
                }
                cp_async_el(de + tid, v0 ? se + go0 : ev, v0);
                if (tid < VNEL1) cp_async_el(de + tid + VNTHR, v1 ? se + go1 : ev, v1);
            }
        };

        const long long col = cell ? (long long)i + (long long)j*d.icells : 0;
        auto colval = [&](const float* f, int l) -> float
        {
            l = l < 0 ? 0 : (l > d.kcells-1 ? d.kcells-1 : l);
            return __ldg(f + col + (long long)l*d.ijcells);
        };

        // Per-level constants of the chunk: index l - m0 for level l.
        const int m0 = k0 - 1;
        for (int q = tid; q < kchunk + 2; q += VNTHR)
        {
            const int l = min(m0 + q, d.kcells - 1);
            prof[0*VPLEV + q] = pr.dzhi[l];
            prof[1*VPLEV + q] = pr.rhorefh[l];
            prof[2*VPLEV + q] = pr.rhoref[l];
            prof[3*VPLEV + q] = pr.dzi[l];
            prof[4*VPLEV + q] = float(GRAV)/pr.threfh[l];
            prof[5*VPLEV + q] = pr.zfac[l];
            prof[6*VPLEV + q] = pr.zfach[l];
            prof[7*VPLEV + q] = pr.thbh[l];
        }

        // Planes of the first four iterations (m0 .. m0+3).
        for (int l = m0; l <= m0+3; ++l) plane(l & 3, l);
        cp_async_commit();

        // Register queues of the own column: u, v, s hold levels m-2 .. m+3,
        // w holds m-1 .. m+4.
        float qu[6], qv[6], qw[6], qs[6];
        if (cell)
        {
            #pragma unroll
            for (int q=0; q<6; ++q)
            {
                qu[q] = colval(u, m0-2+q);
                qv[q] = colval(v, m0-2+q);
                qw[q] = colval(w, m0-1+q);
                qs[q] = (SCAL || BUOY) ? colval(s, m0-2+q) : 0.f;
            }
        }

        const float dxi = d.fdxi, dyi = d.fdyi;
        const float visc = a.visc, svisc = a.svisc, tpri = a.tpri;
        float gzu_b = 0, gzv_b = 0, gzw_b = 0, gzs_b = 0;

        cp_async_wait_all();
        __syncthreads();

        for (int m = m0; m < k1; ++m)
        {
            const int buf = (m - m0) & 1;
            float4* gx = G + buf*VNGX;
            float4* gy = G + 2*VNGX + buf*VNGY;
            const float4* Pm = P + (m & 3)*VPS + pc;
            const float4* Pn = P + ((m+1) & 3)*VPS + pc;
            const float* Em = E + (m & 3)*VPS + pc;
            const float* En = E + ((m+1) & 3)*VPS + pc;

            const bool write = cell && m >= k0;
            const bool wlev = m+1 > d.kstart && m+1 < d.kend;
            const long long c = col + (long long)m*d.ijcells;
            // Early loads: the tendencies this iteration updates and the queue
            // entries of the next iteration.
            float tu = 0, tv = 0, tw = 0, ts = 0;
            if (write)
            {
                tu = a.ut[c]; tv = a.vt[c];
                if (wlev) tw = a.wt[c + d.ijcells];
                if (SCAL) ts = a.st[c];
            }
            float nu = 0, nv = 0, nw = 0, ns = 0;
            if (cell)
            {
                nu = colval(u, m+4); nv = colval(v, m+4); nw = colval(w, m+5);
                if (SCAL || BUOY) ns = colval(s, m+4);
            }

            const int lq = m + 1 - m0;      // index of level m+1 in prof
            const float dzhi1 = prof[0*VPLEV + lq];

            // ---- faces: shear stresses and total fluxes ----
            // x3 = the own point, x2 = (i-1, j), y2 = (i, j-1); un = u, v at m+1.
            float4 x2 = make_float4(0.f, 0.f, 0.f, 0.f), x3 = x2, y2 = x2;
            float e00 = 0.f, e1_00 = 0.f;
            float txz = 0, tyz = 0;
            if (face)
            {
                x2 = Pm[-1]; x3 = Pm[0]; y2 = Pm[-VPW];
                const float2 un = *reinterpret_cast<const float2*>(Pn);
                e00 = Em[0]; e1_00 = En[0];
                const float em10 = Em[-1], e0m1 = Em[-VPW], em1m1 = Em[-VPW-1];
                const float e1m10 = En[-1], e10m1 = En[-VPW];
                const float txy = (0.25f*(em1m1 + e0m1 + em10 + e00) + visc)
                                * ((x3.x - y2.x)*dyi + (x3.y - x2.y)*dxi);
                {
                    // tau_xz and tau_yz in one packed pair.
                    const float2 e = __ffma2_rn(__fadd2_rn(__fadd2_rn(f2(em10, e0m1), f2(e00, e00)),
                                                           __fadd2_rn(f2(e1m10, e10m1), f2(e1_00, e1_00))),
                                                f2(0.25f, 0.25f), f2(visc, visc));
                    const float2 g = __ffma2_rn(sub2(un, lo2(x3)), f2(dzhi1, dzhi1),
                                                __fmul2_rn(sub2(f2(x3.z, x3.z), f2(x2.z, y2.z)), f2(dxi, dyi)));
                    const float2 t = __fmul2_rn(e, g);
                    txz = t.x; tyz = t.y;
                }
                if (face_x)
                {
                    const float4 x0 = Pm[-3], x1 = Pm[-2], x4 = Pm[1], x5 = Pm[2];
                    // u at the cell centre i-1 and v at (i-1/2, j-1/2): one pair.
                    const float2 Auv = adv6x2(f2(0.5f*(x2.x + x3.x), 0.5f*(y2.x + x3.x)),
                                              lo2(x0), lo2(x1), lo2(x2), lo2(x3), lo2(x4), lo2(x5));
                    // w at (i-1/2, m+1/2) and s at i-1/2.
                    float2 Aws;
                    const float wv = 0.5f*(x3.x + un.x);
                    if (SCAL && !LIM)
                        Aws = adv6x2(f2(wv, x3.x), hi2(x0), hi2(x1), hi2(x2), hi2(x3), hi2(x4), hi2(x5));
                    else
                        Aws = f2(adv6(wv, x0.z, x1.z, x2.z, x3.z, x4.z, x5.z),
                                 (SCAL && LIM) ? lim_flux(x3.x, x1.w, x2.w, x3.w, x4.w, 0) : 0.f);
                    const float Du = 2.f*(em10 + visc)*(x3.x - x2.x)*dxi;
                    const float Ds = SCAL ? (0.5f*(em10 + e00)*tpri + svisc)*(x3.w - x2.w)*dxi : 0.f;
                    const float2 f01 = sub2(f2(Du, txy), Auv);
                    const float2 f23 = sub2(f2(txz, Ds), Aws);
                    gx[gxi] = make_float4(f01.x, f01.y, f23.x, SCAL ? f23.y : 0.f);
                }
                if (face_y)
                {
                    const float4 y0 = Pm[-3*VPW], y1 = Pm[-2*VPW], y4 = Pm[VPW], y5 = Pm[2*VPW];
                    // u at (i-1/2, j-1/2) and v at the cell centre j-1.
                    const float2 Auv = adv6x2(f2(0.5f*(x2.y + x3.y), 0.5f*(y2.y + x3.y)),
                                              lo2(y0), lo2(y1), lo2(y2), lo2(x3), lo2(y4), lo2(y5));
                    float2 Aws;
                    const float wv = 0.5f*(x3.y + un.y);
                    if (SCAL && !LIM)
                        Aws = adv6x2(f2(wv, x3.y), hi2(y0), hi2(y1), hi2(y2), hi2(x3), hi2(y4), hi2(y5));
                    else
                        Aws = f2(adv6(wv, y0.z, y1.z, y2.z, x3.z, y4.z, y5.z),
                                 (SCAL && LIM) ? lim_flux(x3.y, y1.w, y2.w, x3.w, y4.w, 0) : 0.f);
                    const float Dv = 2.f*(e0m1 + visc)*(x3.y - y2.y)*dyi;
                    const float Ds = SCAL ? (0.5f*(e0m1 + e00)*tpri + svisc)*(x3.w - y2.w)*dyi : 0.f;
                    const float2 f01 = sub2(f2(txy, Dv), Auv);
                    const float2 f23 = sub2(f2(tyz, Ds), Aws);
                    gy[gyi] = make_float4(f01.x, f01.y, f23.x, SCAL ? f23.y : 0.f);
                }
            }

            // ---- vertical faces of the own column ----
            float gzu_t = 0, gzv_t = 0, gzw_t = 0, gzs_t = 0, buoy = 0;
            if (cell)
            {
                const int kf = m + 1;
                const int ot = face_order_full(d, kf);
                const float rhoh1 = prof[1*VPLEV + lq];
                // u and v: diffusive flux from the shear stress of the same
                // face, or the surface model's flux at the walls (read only
                // at the wall levels, to keep registers free).
                const bool wb = SURF && kf == d.kstart, wt = SURF && kf == d.kend;
                const float du = wb ? -a.u_fluxbot[col] : (wt ? -a.u_fluxtop[col] : txz);
                const float dv = wb ? -a.v_fluxbot[col] : (wt ? -a.v_fluxtop[col] : tyz);
                {
                    const float2 A = zadv2(qu, qv, f2(0.5f*(x2.z + x3.z), 0.5f*(y2.z + x3.z)), ot);
                    const float2 g = __fmul2_rn(f2(rhoh1, rhoh1), sub2(f2(du, dv), A));
                    gzu_t = g.x; gzv_t = g.y;
                }
                // Interior levels: the vertical advective fluxes of w (through
                // full level kf) and of s (through half level kf), both
                // 6th/5th order, in one packed pair.
                bool paired = false;
                float2 aws = make_float2(0.f, 0.f);
                if constexpr (SCAL && !LIM)
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
                    const float ds = wb ? -a.s_fluxbot[col] : (wt ? -a.s_fluxtop[col]
                                   : (0.5f*(e00 + e1_00)*tpri + svisc)*(qs[3] - qs[2])*dzhi1);
                    float as;
                    if (paired) as = aws.y;
                    else if (LIM)
                    {
                        const int side = kf == d.kstart+1 ? -1 : (kf == d.kend-1 ? 1 : 0);
                        as = ot ? lim_flux(qw[2], qs[1], qs[2], qs[3], qs[4], side) : 0.f;
                    }
                    else as = zadv(qs, qw[2], ot);
                    gzs_t = rhoh1*(ds - as);
                }
                // w: the full level kf between w(kf) and w(kf+1).
                if (kf < d.kend)
                {
                    const int ow = face_order_w(d, kf);
                    const float dw = 2.f*(e1_00 + visc)*(qw[3] - qw[2])*prof[3*VPLEV + lq];
                    float aw;
                    if (paired) aw = aws.x;
                    else if (ow == 6) aw = adv6(i2(qw[2], qw[3]), qw[0], qw[1], qw[2], qw[3], qw[4], qw[5]);
                    else if (ow == 4) aw = i2(qw[2], qw[3])*i4ws(qw[1], qw[2], qw[3], qw[4])
                                         - fabsf(i2(qw[2], qw[3]))*i3ws(qw[1], qw[2], qw[3], qw[4]);
                    else aw = i2(qw[2], qw[3])*i2(qw[2], qw[3]);
                    gzw_t = prof[2*VPLEV + lq]*(dw - aw);
                }
                if (BUOY && wlev)
                    buoy = prof[4*VPLEV + lq]*(i2(qs[2], qs[3]) - prof[7*VPLEV + lq]);
            }

            // The planes of iteration m+1 were issued two iterations ago; the
            // last iteration's group may stay in flight.
            asm volatile("cp.async.wait_group 1;\n" ::: "memory");
            __syncthreads();

            // Planes first used by iteration m+4 into the slot iteration m freed.
            if (m + 3 < k1) plane(m & 3, m + 4);
            cp_async_commit();

            if (write)
            {
                const float zf = prof[5*VPLEV + lq - 1];
                // The four fields' face fluxes in one 16-byte load per face;
                // u/v and w/s in packed pairs.
                const float4 xa = gx[gxi], xb = gx[gxi + 1];
                const float4 ya = gy[gyi], yb = gy[gyi + VTX];
                {
                    const float2 dgx = sub2(lo2(xb), lo2(xa));
                    const float2 dgy = sub2(lo2(yb), lo2(ya));
                    const float2 dgz = sub2(f2(gzu_t, gzv_t), f2(gzu_b, gzv_b));
                    const float2 t = __ffma2_rn(dgz, f2(zf, zf), __ffma2_rn(dgy, f2(dyi, dyi),
                                                __ffma2_rn(dgx, f2(dxi, dxi), f2(tu, tv))));
                    a.ut[c] = t.x; a.vt[c] = t.y;
                }
                if constexpr (SCAL)
                {
                    const float2 dgx = sub2(hi2(xb), hi2(xa));
                    const float2 dgy = sub2(hi2(yb), hi2(ya));
                    const float2 dgz = sub2(f2(gzw_t, gzs_t), f2(gzw_b, gzs_b));
                    const float2 t = __ffma2_rn(dgz, f2(prof[6*VPLEV + lq], zf), __ffma2_rn(dgy, f2(dyi, dyi),
                                                __ffma2_rn(dgx, f2(dxi, dxi), f2(tw + buoy, ts))));
                    if (wlev) a.wt[c + d.ijcells] = t.x;
                    a.st[c] = t.y;
                }
                else if (wlev)
                    a.wt[c + d.ijcells] = tw + (xb.z - xa.z)*dxi + (yb.z - ya.z)*dyi
                                             + (gzw_t - gzw_b)*prof[6*VPLEV + lq] + buoy;
            }

            gzu_b = gzu_t; gzv_b = gzv_t; gzw_b = gzw_t; gzs_b = gzs_t;
            #pragma unroll
            for (int q=0; q<5; ++q) { qu[q] = qu[q+1]; qv[q] = qv[q+1]; qw[q] = qw[q+1]; qs[q] = qs[q+1]; }
            qu[5] = nu; qv[5] = nv; qw[5] = nw; qs[5] = ns;
        }
        cp_async_wait_all();
    }

    template<bool SURF, bool SCAL, bool BUOY, bool LIM = false>
    static void launch_fluxv_t(const Dims& d, const Prof<float>& pr, const TendArgs<float>& a, int kchunk, cudaStream_t s)
    {
        const size_t smem = fluxv_smem();
        // The shared-memory limit is set once per kernel, outside any stream
        // capture that a later call may be part of.
        static const bool attr = cudaFuncSetAttribute(k_tend_fluxv<SURF, SCAL, BUOY, LIM>,
            cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) == cudaSuccess;
        (void)attr;
        kchunk = min(auto_kchunk(kchunk, (long long)((d.itot + VTX - 1)/VTX)*((d.jtot + VTY - 1)/VTY), d.ktot), VKMAX);
        dim3 grid((d.itot + VTX - 1)/VTX, (d.jtot + VTY - 1)/VTY, (d.ktot + kchunk - 1)/kchunk);
        k_tend_fluxv<SURF, SCAL, BUOY, LIM><<<grid, VNTHR, smem, s>>>(d, pr, a, kchunk);
        count_launch();
    }

    // Advec_2i5 + Diff_smag2 (+ buoyancy) in flux form on float fields with
    // interleaved planes; igc, jgc >= 3.
    void launch_tendency_fluxv(const Dims& d, const Prof<float>& pr, const TendArgs<float>& a, bool surf, bool scal,
                               bool buoy, bool lim, int kchunk, cudaStream_t s)
    {
        if (lim && scal)
        {
            if (surf && buoy) launch_fluxv_t<true, true, true, true>(d, pr, a, kchunk, s);
            else if (surf) launch_fluxv_t<true, true, false, true>(d, pr, a, kchunk, s);
            else if (buoy) launch_fluxv_t<false, true, true, true>(d, pr, a, kchunk, s);
            else launch_fluxv_t<false, true, false, true>(d, pr, a, kchunk, s);
            return;
        }
        const int mask = (surf ? 4 : 0) | (scal ? 2 : 0) | (buoy ? 1 : 0);
        switch (mask)
        {
            case 0: launch_fluxv_t<false, false, false>(d, pr, a, kchunk, s); break;
            case 1: launch_fluxv_t<false, false, true >(d, pr, a, kchunk, s); break;
            case 2: launch_fluxv_t<false, true,  false>(d, pr, a, kchunk, s); break;
            case 3: launch_fluxv_t<false, true,  true >(d, pr, a, kchunk, s); break;
            case 4: launch_fluxv_t<true,  false, false>(d, pr, a, kchunk, s); break;
            case 5: launch_fluxv_t<true,  false, true >(d, pr, a, kchunk, s); break;
            case 6: launch_fluxv_t<true,  true,  false>(d, pr, a, kchunk, s); break;
            default: launch_fluxv_t<true, true,  true >(d, pr, a, kchunk, s); break;
        }
    }
}
