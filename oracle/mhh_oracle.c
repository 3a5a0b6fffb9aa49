/*
 * mhh_oracle.c -- CPU oracle (TEST INFRASTRUCTURE ONLY; see mhh_oracle.h).
 *
 * A plain-C FP64 restatement of the MicroHH 2nd-order LES/DNS time step.
 * Every routine cites the reference file:line whose arithmetic it follows
 * (paths relative to the MicroHH source tree).  Loops keep the reference's
 * index space (ghost-cell layout ijk = i + j*icells + k*ijcells) so that the
 * fields can be compared cell by cell with the reference and with the GPU.
 *
 * Build: -O2 -ffp-contract=off (no fast-math), optionally -fopenmp.
 */
#include "mhh_oracle.h"
#include "orc_fft.h"

#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

#define KAPPA 0.4     /* include/constants.h:28 */
#define GRAV  9.81    /* include/constants.h:29 */
#define DSMALL 1.e-9  /* include/constants.h:97 */
#define DBIG   1.e9   /* include/constants.h:98 */
#define DHUGE  1.e30  /* include/constants.h:99 */
#define ZL_MAX 10.    /* include/constants.h:55 */
#define ZL_MIN -1.e4  /* include/constants.h:56 */
#define NZL_LUT 10000 /* include/boundary.h:56 */

static inline double sq(double a) { return a*a; }
static inline double dmax(double a, double b) { return a > b ? a : b; }
static inline double dmin(double a, double b) { return a < b ? a : b; }

/* ------------------------------------------------------------------------ */
/* Stencil primitives, include/finite_difference.h:35-157                    */
/* ------------------------------------------------------------------------ */
static inline double i2(double a, double b) { return 0.5*(a + b); }
static inline double i4ws(double a, double b, double c, double d)
{ return (7./12.)*(b + c) - (1./12.)*(a + d); }
static inline double i3ws(double a, double b, double c, double d)
{ return (3./12.)*(c - b) - (1./12.)*(d - a); }
static inline double i6ws(double a, double b, double c, double d, double e, double f)
{ return (37./60.)*(c + d) - (8./60.)*(b + e) + (1./60.)*(a + f); }
static inline double i5ws(double a, double b, double c, double d, double e, double f)
{ return (10./60.)*(d - c) - (5./60.)*(e - b) + (1./60.)*(f - a); }

/* Interpolations of field a to the face between a[c-s] and a[c], using the
   six points a[c-3s] .. a[c+2s]. */
static inline double f6(const double* a, long c, long s)
{ return i6ws(a[c-3*s], a[c-2*s], a[c-s], a[c], a[c+s], a[c+2*s]); }
static inline double f5(const double* a, long c, long s)
{ return i5ws(a[c-3*s], a[c-2*s], a[c-s], a[c], a[c+s], a[c+2*s]); }
static inline double f4(const double* a, long c, long s)
{ return i4ws(a[c-2*s], a[c-s], a[c], a[c+s]); }
static inline double f3(const double* a, long c, long s)
{ return i3ws(a[c-2*s], a[c-s], a[c], a[c+s]); }
static inline double f2(const double* a, long c, long s)
{ return i2(a[c-s], a[c]); }

/* ------------------------------------------------------------------------ */
/* Model state                                                               */
/* ------------------------------------------------------------------------ */
typedef struct
{
    int itot, jtot, ktot;
    int igc, jgc, kgc;
    int icells, jcells, kcells, ijcells;
    long ncells;
    int istart, iend, jstart, jend, kstart, kend;
    double xsize, ysize, zsize, dx, dy;
    double *z, *zh, *dz, *dzh, *dzi, *dzhi;
} grid_t;

typedef struct
{
    double *fld_bot, *fld_top, *grad_bot, *grad_top, *flux_bot, *flux_top;
} bc2d_t;

struct orc_model
{
    orc_params p;
    grid_t g;

    double *u, *v, *w, *th;
    double *ut, *vt, *wt, *tht;
    double *pp, *evisc, *tmp;
    double *rhoref, *rhorefh, *thref, *threfh;

    bc2d_t bu, bv, bth;

    /* surface layer (include/boundary_surface.h) */
    double *ustar, *obuk, *z0m, *z0h, *dudz, *dvdz, *dbdz, *dutot;
    int *nobuk;
    float *zL_sl, *f_sl;

    /* pressure solver */
    double *bmati, *bmatj, *pa, *pc, *work3d, *bb, *work2d, *fftbuf;

    /* buffer layer (src/buffer.cxx) */
    double *bufu, *bufv, *bufth;

    /* time loop */
    int substep, iteration;
    unsigned long itime, idt, idtlim, idtmax;
    double dt;
    double dnmul2;  /* Diff_2 constant diffusion multiplier */
};

#define IJK(g,i,j,k) ((long)(i) + (long)(j)*(g)->icells + (long)(k)*(g)->ijcells)

static double* alloc0(long n) { return (double*)calloc((size_t)(n > 0 ? n : 1), sizeof(double)); }

/* ------------------------------------------------------------------------ */
/* Grid, src/grid.cxx:105-193 (init) and :245-305 (calculate, 2nd order)     */
/* ------------------------------------------------------------------------ */
static void grid_init(grid_t* g, const orc_params* p, const double* zin)
{
    g->itot = p->itot; g->jtot = p->jtot; g->ktot = p->ktot;
    /* Advec_2i5 asks for (3,3,1) ghost cells, (3,3,2) with a flux-limited
       scalar (src/advec_2i5.cxx:36-46); all other modules on this path need
       (1,1,1). */
    g->igc = (p->advec == ORC_ADVEC_2I5) ? 3 : 1;
    g->jgc = g->igc;
    g->kgc = (p->advec == ORC_ADVEC_2I5 && p->fluxlimit_s) ? 2 : 1;
    g->icells = g->itot + 2*g->igc;
    g->jcells = g->jtot + 2*g->jgc;
    g->kcells = g->ktot + 2*g->kgc;
    g->ijcells = g->icells*g->jcells;
    g->ncells = (long)g->ijcells*g->kcells;
    g->istart = g->igc; g->iend = g->itot + g->igc;
    g->jstart = g->jgc; g->jend = g->jtot + g->jgc;
    g->kstart = g->kgc; g->kend = g->ktot + g->kgc;
    g->xsize = p->xsize; g->ysize = p->ysize; g->zsize = p->zsize;

    const int kc = g->kcells;
    g->z = alloc0(kc); g->zh = alloc0(kc); g->dz = alloc0(kc);
    g->dzh = alloc0(kc); g->dzi = alloc0(kc); g->dzhi = alloc0(kc);

    g->dx = g->xsize / g->itot;
    g->dy = g->ysize / g->jtot;

    for (int k=0; k<g->ktot; ++k)
        g->z[k + g->kstart] = zin[k];

    const int ks = g->kstart, ke = g->kend;
    g->z[ks-1] = -g->z[ks];
    g->z[ke]   = 2.*g->zsize - g->z[ke-1];
    for (int k=ks+1; k<ke; ++k)
        g->zh[k] = 0.5*(g->z[k-1] + g->z[k]);
    g->zh[ks] = 0.;
    g->zh[ke] = g->zsize;

    for (int k=1; k<kc; ++k)
    {
        g->dzh[k]  = g->z[k] - g->z[k-1];
        g->dzhi[k] = 1./g->dzh[k];
    }
    g->dzh[ks-1]  = g->dzh[ks+1];
    g->dzhi[ks-1] = g->dzhi[ks+1];

    for (int k=1; k<kc-1; ++k)
    {
        g->dz[k]  = g->zh[k+1] - g->zh[k];
        g->dzi[k] = 1./g->dz[k];
    }
    g->dz[ks-1]  = g->dz[ks];
    g->dzi[ks-1] = g->dzi[ks];
    g->dz[ke]    = g->dz[ke-1];
    g->dzi[ke]   = g->dzi[ke-1];
}

/* ------------------------------------------------------------------------ */
/* Periodic ghost cells, src/boundary_cyclic.cxx:370-470 (serial branch)     */
/* ------------------------------------------------------------------------ */
enum { EDGE_EW = 1, EDGE_NS = 2, EDGE_BOTH = 3 };

static void cyclic3d(const grid_t* g, double* a, int edge)
{
    if (edge & EDGE_EW)
    {
        #pragma omp parallel for
        for (int k=0; k<g->kcells; ++k)
            for (int j=0; j<g->jcells; ++j)
                for (int i=0; i<g->igc; ++i)
                {
                    a[IJK(g, i, j, k)] = a[IJK(g, g->iend - g->igc + i, j, k)];
                    a[IJK(g, g->iend + i, j, k)] = a[IJK(g, g->istart + i, j, k)];
                }
    }
    if (edge & EDGE_NS)
    {
        #pragma omp parallel for
        for (int k=0; k<g->kcells; ++k)
            for (int j=0; j<g->jgc; ++j)
                for (int i=0; i<g->icells; ++i)
                {
                    a[IJK(g, i, j, k)] = a[IJK(g, i, g->jend - g->jgc + j, k)];
                    a[IJK(g, i, g->jend + j, k)] = a[IJK(g, i, g->jstart + j, k)];
                }
    }
}

/* West ghosts copy from the east interior before east ghosts copy from the
   west interior; with igc <= itot the two sets never overlap, so doing both
   in one sweep matches the reference's two-sweep order. */
static void cyclic2d(const grid_t* g, double* a)
{
    for (int j=0; j<g->jcells; ++j)
        for (int i=0; i<g->igc; ++i)
        {
            a[i + j*g->icells] = a[g->iend - g->igc + i + j*g->icells];
            a[g->iend + i + j*g->icells] = a[g->istart + i + j*g->icells];
        }
    for (int j=0; j<g->jgc; ++j)
        for (int i=0; i<g->icells; ++i)
        {
            a[i + j*g->icells] = a[i + (g->jend - g->jgc + j)*g->icells];
            a[i + (g->jend + j)*g->icells] = a[i + (g->jstart + j)*g->icells];
        }
}

/* ------------------------------------------------------------------------ */
/* Boundary values, src/boundary.cxx:50-100 (set_bc) and :615-700            */
/* (set_values), src/boundary_surface.cxx:755-790 (surface override)         */
/* ------------------------------------------------------------------------ */
static void fill2d(const grid_t* g, double* a, double v)
{
    for (int n=0; n<g->ijcells; ++n) a[n] = v;
}

static void set_bc(const grid_t* g, bc2d_t* b, int bot, int type, double aval,
                   double visc, int set_flux_grad)
{
    double* fld  = bot ? b->fld_bot  : b->fld_top;
    double* grad = bot ? b->grad_bot : b->grad_top;
    double* flux = bot ? b->flux_bot : b->flux_top;
    if (type == ORC_BC_DIRICHLET)
        fill2d(g, fld, aval);
    else if (type == ORC_BC_NEUMANN)
    {
        fill2d(g, grad, aval);
        if (set_flux_grad) fill2d(g, flux, -aval*visc);
    }
    else if (type == ORC_BC_FLUX)
    {
        fill2d(g, flux, aval);
        if (set_flux_grad) fill2d(g, grad, -aval/visc);
    }
}

static void set_boundary_values(orc_model* m)
{
    const orc_params* p = &m->p;
    const grid_t* g = &m->g;
    const int sfg = (p->surface == 0);
    set_bc(g, &m->bu, 1, p->mbcbot, p->ubot, p->visc, 1);
    set_bc(g, &m->bv, 1, p->mbcbot, p->vbot, p->visc, 1);
    set_bc(g, &m->bu, 0, p->mbctop, p->utop, p->visc, 1);
    set_bc(g, &m->bv, 0, p->mbctop, p->vtop, p->visc, 1);
    if (p->thermo)
    {
        set_bc(g, &m->bth, 1, p->sbcbot, p->sbot, p->svisc, sfg);
        set_bc(g, &m->bth, 0, p->sbctop, p->stop, p->svisc, sfg);
    }
    if (p->surface)
    {
        /* The surface model forces a Dirichlet bottom for u and v. */
        fill2d(g, m->bu.fld_bot, p->ubot);
        fill2d(g, m->bv.fld_bot, p->vbot);
    }
}

/* 2nd-order ghost cells, src/boundary.cxx:700-760. */
static void ghost_bot(const grid_t* g, double* a, int type, const bc2d_t* b)
{
    const int ks = g->kstart;
    #pragma omp parallel for
    for (int j=0; j<g->jcells; ++j)
        for (int i=0; i<g->icells; ++i)
        {
            const long ij = i + (long)j*g->icells;
            const long ijk = IJK(g, i, j, ks);
            if (type == ORC_BC_DIRICHLET)
                a[ijk - g->ijcells] = 2.*b->fld_bot[ij] - a[ijk];
            else
                a[ijk - g->ijcells] = -b->grad_bot[ij]*g->dzh[ks] + a[ijk];
        }
}

static void ghost_top(const grid_t* g, double* a, int type, const bc2d_t* b)
{
    const int ke = g->kend;
    #pragma omp parallel for
    for (int j=0; j<g->jcells; ++j)
        for (int i=0; i<g->icells; ++i)
        {
            const long ij = i + (long)j*g->icells;
            const long ijk = IJK(g, i, j, ke-1);
            if (type == ORC_BC_DIRICHLET)
                a[ijk + g->ijcells] = 2.*b->fld_top[ij] - a[ijk];
            else
                a[ijk + g->ijcells] = b->grad_top[ij]*g->dzh[ke] + a[ijk];
        }
}

/* src/boundary.cxx:933-998 */
static void set_ghost_cells(orc_model* m)
{
    const orc_params* p = &m->p;
    const grid_t* g = &m->g;
    ghost_bot(g, m->u, p->mbcbot, &m->bu);
    ghost_top(g, m->u, p->mbctop, &m->bu);
    ghost_bot(g, m->v, p->mbcbot, &m->bv);
    ghost_top(g, m->v, p->mbctop, &m->bv);
    if (p->thermo)
    {
        ghost_bot(g, m->th, p->sbcbot, &m->bth);
        ghost_top(g, m->th, p->sbctop, &m->bth);
    }
}

void orc_set_cyclic_and_ghost(orc_model* m)
{
    /* src/boundary.cxx:450-461 then :933-998 */
    cyclic3d(&m->g, m->u, EDGE_BOTH);
    cyclic3d(&m->g, m->v, EDGE_BOTH);
    cyclic3d(&m->g, m->w, EDGE_BOTH);
    if (m->p.thermo) cyclic3d(&m->g, m->th, EDGE_BOTH);
    set_ghost_cells(m);
}

/* ------------------------------------------------------------------------ */
/* Advec_2i5, src/advec_2i5.cxx:150-728                                      */
/*                                                                           */
/* Horizontal fluxes: 6th-order interpolation plus |U|-weighted 5th-order    */
/* dissipation at all levels.  Vertical fluxes: the same in the interior,    */
/* reduced to 4th/3rd then 2nd order at the two levels next to a wall and    */
/* zero at the wall (w = 0).                                                 */
/* ------------------------------------------------------------------------ */

/* Vertical upwind flux of field a through the face below cell centre c
   (face index kf), transported with velocity wf.  `order` is the largest
   interpolation order the level allows (2, 4 or 6). */
static inline double vflux(const double* a, long c, long kk, double wf, int order)
{
    if (order == 6)
        return wf*f6(a, c, kk) - fabs(wf)*f5(a, c, kk);
    if (order == 4)
        return wf*f4(a, c, kk) - fabs(wf)*f3(a, c, kk);
    return wf*f2(a, c, kk);
}

/* Order of the flux through face kf (half level) for a field at full levels.
   Faces kstart and kend are walls (no flux); the faces right next to them
   use 2nd order, the next ones 4th order (src/advec_2i5.cxx:219-299). */
static inline int face_order_full(const grid_t* g, int kf)
{
    if (kf <= g->kstart || kf >= g->kend) return 0;
    if (kf == g->kstart+1 || kf == g->kend-1) return 2;
    if (kf == g->kstart+2 || kf == g->kend-2) return 4;
    return 6;
}

/* Order of the w-flux through the full-level face k (between half levels
   k and k+1), src/advec_2i5.cxx:515-578. */
static inline int face_order_w(const grid_t* g, int k)
{
    if (k == g->kstart || k == g->kend-1) return 2;
    if (k == g->kstart+1 || k == g->kend-2) return 4;
    return 6;
}

static void advec_2i5_u(orc_model* m)
{
    const grid_t* g = &m->g;
    const double* u = m->u; const double* v = m->v; const double* w = m->w;
    double* ut = m->ut;
    const long ii = 1, jj = g->icells, kk = g->ijcells;
    const double dxi = 1./g->dx, dyi = 1./g->dy;
    #pragma omp parallel for
    for (int k=g->kstart; k<g->kend; ++k)
        for (int j=g->jstart; j<g->jend; ++j)
            for (int i=g->istart; i<g->iend; ++i)
            {
                const long c = IJK(g, i, j, k);
                const double ue = i2(u[c], u[c+ii]), uw = i2(u[c-ii], u[c]);
                const double vn = i2(v[c-ii+jj], v[c+jj]), vs = i2(v[c-ii], v[c]);
                double t =
                    - (ue*f6(u, c+ii, ii) - uw*f6(u, c, ii))*dxi
                    + (fabs(ue)*f5(u, c+ii, ii) - fabs(uw)*f5(u, c, ii))*dxi
                    - (vn*f6(u, c+jj, jj) - vs*f6(u, c, jj))*dyi
                    + (fabs(vn)*f5(u, c+jj, jj) - fabs(vs)*f5(u, c, jj))*dyi;

                const double wt_ = i2(w[c-ii+kk], w[c+kk]), wb = i2(w[c-ii], w[c]);
                const int ot = face_order_full(g, k+1), ob = face_order_full(g, k);
                const double ftop = ot ? m->rhorefh[k+1]*vflux(u, c+kk, kk, wt_, ot) : 0.;
                const double fbot = ob ? m->rhorefh[k  ]*vflux(u, c   , kk, wb , ob) : 0.;
                t -= (ftop - fbot) / m->rhoref[k] * g->dzi[k];
                ut[c] += t;
            }
}

static void advec_2i5_v(orc_model* m)
{
    const grid_t* g = &m->g;
    const double* u = m->u; const double* v = m->v; const double* w = m->w;
    double* vt = m->vt;
    const long ii = 1, jj = g->icells, kk = g->ijcells;
    const double dxi = 1./g->dx, dyi = 1./g->dy;
    #pragma omp parallel for
    for (int k=g->kstart; k<g->kend; ++k)
        for (int j=g->jstart; j<g->jend; ++j)
            for (int i=g->istart; i<g->iend; ++i)
            {
                const long c = IJK(g, i, j, k);
                const double ue = i2(u[c+ii-jj], u[c+ii]), uw = i2(u[c-jj], u[c]);
                const double vn = i2(v[c], v[c+jj]), vs = i2(v[c-jj], v[c]);
                double t =
                    - (ue*f6(v, c+ii, ii) - uw*f6(v, c, ii))*dxi
                    + (fabs(ue)*f5(v, c+ii, ii) - fabs(uw)*f5(v, c, ii))*dxi
                    - (vn*f6(v, c+jj, jj) - vs*f6(v, c, jj))*dyi
                    + (fabs(vn)*f5(v, c+jj, jj) - fabs(vs)*f5(v, c, jj))*dyi;

                const double wt_ = i2(w[c-jj+kk], w[c+kk]), wb = i2(w[c-jj], w[c]);
                const int ot = face_order_full(g, k+1), ob = face_order_full(g, k);
                const double ftop = ot ? m->rhorefh[k+1]*vflux(v, c+kk, kk, wt_, ot) : 0.;
                const double fbot = ob ? m->rhorefh[k  ]*vflux(v, c   , kk, wb , ob) : 0.;
                t -= (ftop - fbot) / m->rhoref[k] * g->dzi[k];
                vt[c] += t;
            }
}

static void advec_2i5_w(orc_model* m)
{
    const grid_t* g = &m->g;
    const double* u = m->u; const double* v = m->v; const double* w = m->w;
    double* wt = m->wt;
    const long ii = 1, jj = g->icells, kk = g->ijcells;
    const double dxi = 1./g->dx, dyi = 1./g->dy;
    #pragma omp parallel for
    for (int k=g->kstart+1; k<g->kend; ++k)
        for (int j=g->jstart; j<g->jend; ++j)
            for (int i=g->istart; i<g->iend; ++i)
            {
                const long c = IJK(g, i, j, k);
                const double ue = i2(u[c+ii-kk], u[c+ii]), uw = i2(u[c-kk], u[c]);
                const double vn = i2(v[c+jj-kk], v[c+jj]), vs = i2(v[c-kk], v[c]);
                double t =
                    - (ue*f6(w, c+ii, ii) - uw*f6(w, c, ii))*dxi
                    + (fabs(ue)*f5(w, c+ii, ii) - fabs(uw)*f5(w, c, ii))*dxi
                    - (vn*f6(w, c+jj, jj) - vs*f6(w, c, jj))*dyi
                    + (fabs(vn)*f5(w, c+jj, jj) - fabs(vs)*f5(w, c, jj))*dyi;

                /* Faces of the w cell are the full levels k (top) and k-1 (bottom). */
                const double wtf = i2(w[c], w[c+kk]), wbf = i2(w[c-kk], w[c]);
                const double ftop = m->rhoref[k  ]*vflux(w, c+kk, kk, wtf, face_order_w(g, k  ));
                const double fbot = m->rhoref[k-1]*vflux(w, c   , kk, wbf, face_order_w(g, k-1));
                t -= (ftop - fbot) / m->rhorefh[k] * g->dzhi[k];
                wt[c] += t;
            }
}

static void advec_2i5_s(orc_model* m, double* st, const double* s)
{
    const grid_t* g = &m->g;
    const double* u = m->u; const double* v = m->v; const double* w = m->w;
    const long ii = 1, jj = g->icells, kk = g->ijcells;
    const double dxi = 1./g->dx, dyi = 1./g->dy;
    #pragma omp parallel for
    for (int k=g->kstart; k<g->kend; ++k)
        for (int j=g->jstart; j<g->jend; ++j)
            for (int i=g->istart; i<g->iend; ++i)
            {
                const long c = IJK(g, i, j, k);
                const double ue = u[c+ii], uw = u[c];
                const double vn = v[c+jj], vs = v[c];
                double t =
                    - (ue*f6(s, c+ii, ii) - uw*f6(s, c, ii))*dxi
                    + (fabs(ue)*f5(s, c+ii, ii) - fabs(uw)*f5(s, c, ii))*dxi
                    - (vn*f6(s, c+jj, jj) - vs*f6(s, c, jj))*dyi
                    + (fabs(vn)*f5(s, c+jj, jj) - fabs(vs)*f5(s, c, jj))*dyi;

                const int ot = face_order_full(g, k+1), ob = face_order_full(g, k);
                const double ftop = ot ? m->rhorefh[k+1]*vflux(s, c+kk, kk, w[c+kk], ot) : 0.;
                const double fbot = ob ? m->rhorefh[k  ]*vflux(s, c   , kk, w[c]   , ob) : 0.;
                t -= (ftop - fbot) / m->rhoref[k] * g->dzi[k];
                st[c] += t;
            }
}

/* Flux limiter of Koren (1993), include/advec_monotonic.h:28-99: the face
   value is the upwind value plus half the limited upwind difference,
   phi(r) = max(0, min(2r, (1 + 2r)/3, 2)), with r the ratio of the downwind
   to the upwind difference (its denominator kept at least machine epsilon
   in magnitude). */
static inline double koren_face(double up, double upup, double down)
{
    const double d = up - upup;
    const double denom = copysign(1., d)*dmax(fabs(d), DBL_EPSILON);
    const double two_r = 2.*(down - up)/denom;
    const double phi = dmax(0., dmin(two_r, dmin((1./3.)*(1. + two_r), 2.)));
    return up + 0.5*phi*(up - upup);
}

/* Limited flux vel * s through the face between a[c-st] and a[c] (the face
   of cell c on its low side, stride st).  side = -1: the first face above
   the bottom wall (upward flow takes the upwind value unlimited), +1: the
   last face below the top wall (likewise for downward flow), 0: interior. */
static inline double flux_koren(const double* a, long c, long st, double vel, int side)
{
    if (vel >= 0.)
        return side < 0 ? vel*a[c-st] : vel*koren_face(a[c-st], a[c-2*st], a[c]);
    return side > 0 ? vel*a[c] : vel*koren_face(a[c], a[c+st], a[c-st]);
}

/* Side argument of flux_koren for the face kf of a full-level field
   (interior faces kstart+1 .. kend-1; ktot >= 4). */
static inline int face_side_lim(const grid_t* g, int kf)
{
    return kf == g->kstart+1 ? -1 : (kf == g->kend-1 ? 1 : 0);
}

/* Scalar advection with the flux limiter, include/advec_monotonic.h:101-219
   (advec_s_lim): limited fluxes in x, y and z; no flux through the walls;
   the first face above the bottom and the last below the top are limited
   only for flow away from the wall. */
static void advec_2i5_s_lim(orc_model* m, double* st, const double* s)
{
    const grid_t* g = &m->g;
    const double* u = m->u; const double* v = m->v; const double* w = m->w;
    const long ii = 1, jj = g->icells, kk = g->ijcells;
    const double dxi = 1./g->dx, dyi = 1./g->dy;
    #pragma omp parallel for
    for (int k=g->kstart; k<g->kend; ++k)
    {
        /* No flux through the walls (faces kstart and kend). */
        const int top = k+1 < g->kend, bot = k > g->kstart;
        const int st_top = face_side_lim(g, k+1), st_bot = face_side_lim(g, k);
        for (int j=g->jstart; j<g->jend; ++j)
            for (int i=g->istart; i<g->iend; ++i)
            {
                const long c = IJK(g, i, j, k);
                const double ftop = top ? flux_koren(s, c+kk, kk, w[c+kk], st_top) : 0.;
                const double fbot = bot ? flux_koren(s, c, kk, w[c], st_bot) : 0.;
                st[c] +=
                    - (flux_koren(s, c+ii, ii, u[c+ii], 0) - flux_koren(s, c, ii, u[c], 0))*dxi
                    - (flux_koren(s, c+jj, jj, v[c+jj], 0) - flux_koren(s, c, jj, v[c], 0))*dyi
                    - (m->rhorefh[k+1]*ftop - m->rhorefh[k]*fbot) / m->rhoref[k] * g->dzi[k];
            }
    }
}

/* CFL of Advec_2i5, src/advec_2i5.cxx:59-148: the vertical interpolation of
   w to the cell centre is 2nd order at kstart and kend-1, 4th order at
   kstart+1 and kend-2 and 6th order elsewhere. */
static double cfl_2i5(orc_model* m)
{
    const grid_t* g = &m->g;
    const double* u = m->u; const double* v = m->v; const double* w = m->w;
    const long ii = 1, jj = g->icells, kk = g->ijcells;
    const double dxi = 1./g->dx, dyi = 1./g->dy;
    double cfl = 0.;
    #pragma omp parallel for reduction(max:cfl)
    for (int k=g->kstart; k<g->kend; ++k)
    {
        const int ord = face_order_w(g, k);
        for (int j=g->jstart; j<g->jend; ++j)
            for (int i=g->istart; i<g->iend; ++i)
            {
                const long c = IJK(g, i, j, k);
                double wc;
                if (ord == 2) wc = f2(w, c+kk, kk);
                else if (ord == 4) wc = f4(w, c+kk, kk);
                else wc = f6(w, c+kk, kk);
                const double val = fabs(f6(u, c+ii, ii))*dxi + fabs(f6(v, c+jj, jj))*dyi
                                 + fabs(wc)*g->dzi[k];
                cfl = dmax(cfl, val);
            }
    }
    return cfl;
}

/* ------------------------------------------------------------------------ */
/* Advec_2, src/advec_2.cxx:50-202                                           */
/* ------------------------------------------------------------------------ */
static void advec_2_uvw(orc_model* m)
{
    const grid_t* g = &m->g;
    const double* u = m->u; const double* v = m->v; const double* w = m->w;
    const long ii = 1, jj = g->icells, kk = g->ijcells;
    const double dxi = 1./g->dx, dyi = 1./g->dy;
    #pragma omp parallel for
    for (int k=g->kstart; k<g->kend; ++k)
        for (int j=g->jstart; j<g->jend; ++j)
            for (int i=g->istart; i<g->iend; ++i)
            {
                const long c = IJK(g, i, j, k);
                m->ut[c] +=
                    - (i2(u[c], u[c+ii])*i2(u[c], u[c+ii]) - i2(u[c-ii], u[c])*i2(u[c-ii], u[c]))*dxi
                    - (i2(v[c-ii+jj], v[c+jj])*i2(u[c], u[c+jj]) - i2(v[c-ii], v[c])*i2(u[c-jj], u[c]))*dyi
                    - (m->rhorefh[k+1]*i2(w[c-ii+kk], w[c+kk])*i2(u[c], u[c+kk])
                     - m->rhorefh[k  ]*i2(w[c-ii], w[c])*i2(u[c-kk], u[c])) / m->rhoref[k]*g->dzi[k];
                m->vt[c] +=
                    - (i2(u[c+ii-jj], u[c+ii])*i2(v[c], v[c+ii]) - i2(u[c-jj], u[c])*i2(v[c-ii], v[c]))*dxi
                    - (i2(v[c], v[c+jj])*i2(v[c], v[c+jj]) - i2(v[c-jj], v[c])*i2(v[c-jj], v[c]))*dyi
                    - (m->rhorefh[k+1]*i2(w[c-jj+kk], w[c+kk])*i2(v[c], v[c+kk])
                     - m->rhorefh[k  ]*i2(w[c-jj], w[c])*i2(v[c-kk], v[c])) / m->rhoref[k]*g->dzi[k];
                if (k > g->kstart)
                    m->wt[c] +=
                        - (i2(u[c+ii-kk], u[c+ii])*i2(w[c], w[c+ii]) - i2(u[c-kk], u[c])*i2(w[c-ii], w[c]))*dxi
                        - (i2(v[c+jj-kk], v[c+jj])*i2(w[c], w[c+jj]) - i2(v[c-kk], v[c])*i2(w[c-jj], w[c]))*dyi
                        - (m->rhoref[k  ]*i2(w[c], w[c+kk])*i2(w[c], w[c+kk])
                         - m->rhoref[k-1]*i2(w[c-kk], w[c])*i2(w[c-kk], w[c])) / m->rhorefh[k]*g->dzhi[k];
            }
}

static void advec_2_s(orc_model* m, double* st, const double* s)
{
    const grid_t* g = &m->g;
    const double* u = m->u; const double* v = m->v; const double* w = m->w;
    const long ii = 1, jj = g->icells, kk = g->ijcells;
    const double dxi = 1./g->dx, dyi = 1./g->dy;
    #pragma omp parallel for
    for (int k=g->kstart; k<g->kend; ++k)
        for (int j=g->jstart; j<g->jend; ++j)
            for (int i=g->istart; i<g->iend; ++i)
            {
                const long c = IJK(g, i, j, k);
                st[c] +=
                    - (u[c+ii]*i2(s[c], s[c+ii]) - u[c]*i2(s[c-ii], s[c]))*dxi
                    - (v[c+jj]*i2(s[c], s[c+jj]) - v[c]*i2(s[c-jj], s[c]))*dyi
                    - (m->rhorefh[k+1]*w[c+kk]*i2(s[c], s[c+kk])
                     - m->rhorefh[k  ]*w[c   ]*i2(s[c-kk], s[c])) / m->rhoref[k]*g->dzi[k];
            }
}

/* src/advec_2.cxx:50-80 */
static double cfl_2(orc_model* m)
{
    const grid_t* g = &m->g;
    const double* u = m->u; const double* v = m->v; const double* w = m->w;
    const long ii = 1, jj = g->icells, kk = g->ijcells;
    const double dxi = 1./g->dx, dyi = 1./g->dy;
    double cfl = 0.;
    #pragma omp parallel for reduction(max:cfl)
    for (int k=g->kstart; k<g->kend; ++k)
        for (int j=g->jstart; j<g->jend; ++j)
            for (int i=g->istart; i<g->iend; ++i)
            {
                const long c = IJK(g, i, j, k);
                cfl = dmax(cfl, fabs(i2(u[c], u[c+ii]))*dxi + fabs(i2(v[c], v[c+jj]))*dyi
                                + fabs(i2(w[c], w[c+kk]))*g->dzi[k]);
            }
    return cfl;
}

void orc_exec_advec(orc_model* m)
{
    if (m->p.advec == ORC_ADVEC_2I5)
    {
        advec_2i5_u(m);
        advec_2i5_v(m);
        advec_2i5_w(m);
        if (m->p.thermo && m->p.fluxlimit_s) advec_2i5_s_lim(m, m->tht, m->th);
        else if (m->p.thermo) advec_2i5_s(m, m->tht, m->th);
    }
    else
    {
        advec_2_uvw(m);
        if (m->p.thermo) advec_2_s(m, m->tht, m->th);
    }
}

#include "mhh_oracle_physics.inc"
