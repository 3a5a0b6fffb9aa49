/*
 * orc_fft.c -- real halfcomplex FFTs for the CPU oracle (TEST INFRASTRUCTURE
 * ONLY).  Shared by the C restatement (mhh_oracle.c) and by the reference
 * build in _ref/, which links it in place of FFTW.
 */
#include "orc_fft.h"

#include <math.h>
#include <stdlib.h>

/* ------------------------------------------------------------------------ */
/* Real FFT in FFTW's halfcomplex convention.                                */
/*                                                                           */
/* FFTW 3 (r2r R2HC / HC2R) is the reference's third-party transform         */
/* (src/fft.cxx:145-206); it is not in the source tree, so this restates its */
/* published definition: R2HC gives r_0 .. r_{n/2}, i_{(n+1)/2-1} .. i_1 of  */
/* the unnormalised DFT X_k = sum_j x_j exp(-2 pi i j k / n); HC2R is the     */
/* unnormalised inverse.  The complex transform is a recursive mixed-radix   */
/* Cooley-Tukey decimation in time; two real sequences share one complex     */
/* transform (x + i y) and are separated by Hermitian symmetry.               */
/* ------------------------------------------------------------------------ */
typedef struct { double re, im; } cpx;

typedef struct
{
    int n;
    int nfac;
    int fac[64];
    cpx* tw;   /* exp(-2 pi i k / n), k = 0..n-1, rounded from long double */
} fftplan;

static void fftplan_init(fftplan* pl, int n)
{
    pl->n = n;
    pl->nfac = 0;
    int r = n;
    const int radices[] = {4, 2, 3, 5};
    for (int q=0; q<4 && r>1; ++q)
        while (r % radices[q] == 0) { pl->fac[pl->nfac++] = radices[q]; r /= radices[q]; }
    for (int p=7; r>1; p+=2)
        while (r % p == 0) { pl->fac[pl->nfac++] = p; r /= p; }
    pl->tw = (cpx*)malloc(sizeof(cpx)*(size_t)n);
    const long double twopi = 6.283185307179586476925286766559005768L;
    for (int k=0; k<n; ++k)
    {
        const long double ang = -twopi*(long double)k/(long double)n;
        pl->tw[k].re = (double)cosl(ang);
        pl->tw[k].im = (double)sinl(ang);
    }
}

static void fftplan_free(fftplan* pl) { free(pl->tw); }

/* Output out[0..n) = DFT of in[0], in[s], in[2s], ... (length n/prod(prev)). */
static void fft_rec(const fftplan* pl, cpx* out, const cpx* in, long s, int fi, int len, int twstride, cpx* scratch)
{
    if (len == 1) { out[0] = in[0]; return; }
    const int p = pl->fac[fi];
    const int m = len / p;
    for (int q=0; q<p; ++q)
        fft_rec(pl, out + (long)q*m, in + (long)q*s, s*p, fi+1, m, twstride*p, scratch);
    /* Butterflies: out[u + q1*m] = sum_q2 w^(q2*(u+q1*m)) * sub_q2[u] */
    const int n = pl->n;
    for (int u=0; u<m; ++u)
    {
        for (int q=0; q<p; ++q)
        {
            const cpx a = out[u + (long)q*m];
            const int t = (int)(((long)q*u*twstride) % n);
            scratch[q].re = a.re*pl->tw[t].re - a.im*pl->tw[t].im;
            scratch[q].im = a.re*pl->tw[t].im + a.im*pl->tw[t].re;
        }
        for (int q1=0; q1<p; ++q1)
        {
            double re = scratch[0].re, im = scratch[0].im;
            for (int q2=1; q2<p; ++q2)
            {
                const int t = (int)(((long)q1*q2*m*twstride) % n);
                re += scratch[q2].re*pl->tw[t].re - scratch[q2].im*pl->tw[t].im;
                im += scratch[q2].re*pl->tw[t].im + scratch[q2].im*pl->tw[t].re;
            }
            out[u + (long)q1*m].re = re;
            out[u + (long)q1*m].im = im;
        }
    }
}

static void fft_forward_c(const fftplan* pl, cpx* out, const cpx* in, cpx* scratch)
{
    fft_rec(pl, out, in, 1, 0, pl->n, 1, scratch);
}

/* Two real sequences x, y (stride st) -> halfcomplex hx, hy (same places). */
static void r2hc_pair(const fftplan* pl, double* x, double* y, long st, cpx* zin, cpx* zout, cpx* scr)
{
    const int n = pl->n;
    for (int j=0; j<n; ++j) { zin[j].re = x[j*st]; zin[j].im = y ? y[j*st] : 0.; }
    fft_forward_c(pl, zout, zin, scr);
    for (int k=0; k<=n/2; ++k)
    {
        const cpx a = zout[k], b = zout[(n-k) % n];
        /* X_k = (Z_k + conj Z_{n-k})/2, Y_k = (Z_k - conj Z_{n-k})/(2i) */
        const double xr = 0.5*(a.re + b.re), xi = 0.5*(a.im - b.im);
        const double yr = 0.5*(a.im + b.im), yi = -0.5*(a.re - b.re);
        x[k*st] = xr;
        if (y) y[k*st] = yr;
        if (k > 0 && k < n-k)
        {
            x[(n-k)*st] = xi;
            if (y) y[(n-k)*st] = yi;
        }
    }
}

/* Halfcomplex hx, hy -> two real sequences (unnormalised inverse). */
static void hc2r_pair(const fftplan* pl, double* x, double* y, long st, cpx* zin, cpx* zout, cpx* scr)
{
    const int n = pl->n;
    /* Z_k = X_k + i Y_k; the inverse is conj(FFT(conj(Z))). */
    for (int k=0; k<n; ++k)
    {
        double xr, xi, yr, yi;
        const int kk_ = (k <= n/2) ? k : n-k;
        const double sgn = (k <= n/2) ? 1. : -1.;
        xr = x[kk_*st]; yr = y ? y[kk_*st] : 0.;
        if (kk_ == 0 || 2*kk_ == n) { xi = 0.; yi = 0.; }
        else { xi = sgn*x[(n-kk_)*st]; yi = y ? sgn*y[(n-kk_)*st] : 0.; }
        /* conj(Z_k) = (xr - yi) - i (xi + yr) */
        zin[k].re = xr - yi;
        zin[k].im = -(xi + yr);
    }
    fft_forward_c(pl, zout, zin, scr);
    for (int j=0; j<n; ++j)
    {
        x[j*st] = zout[j].re;
        if (y) y[j*st] = -zout[j].im;
    }
}

typedef struct { cpx *zin, *zout, *scr; } fftwork;

static void fftwork_init(fftwork* w, int n)
{
    w->zin = (cpx*)malloc(sizeof(cpx)*(size_t)n);
    w->zout = (cpx*)malloc(sizeof(cpx)*(size_t)n);
    w->scr = (cpx*)malloc(sizeof(cpx)*(size_t)(n + 64));
}
static void fftwork_free(fftwork* w) { free(w->zin); free(w->zout); free(w->scr); }

static void batch_transform(int n, int howmany, double* data, long stride, long dist, int inverse)
{
    if (n == 1) return;
    fftplan pl;
    fftplan_init(&pl, n);
    const int npairs = (howmany + 1)/2;
    #pragma omp parallel
    {
        fftwork w;
        fftwork_init(&w, n);
        #pragma omp for
        for (int q=0; q<npairs; ++q)
        {
            double* x = data + (long)(2*q)*dist;
            double* y = (2*q + 1 < howmany) ? data + (long)(2*q+1)*dist : NULL;
            if (inverse) hc2r_pair(&pl, x, y, stride, w.zin, w.zout, w.scr);
            else         r2hc_pair(&pl, x, y, stride, w.zin, w.zout, w.scr);
        }
        fftwork_free(&w);
    }
    fftplan_free(&pl);
}

void orcfft_r2hc(int n, int howmany, double* data, long stride, long dist)
{ batch_transform(n, howmany, data, stride, dist, 0); }
void orcfft_hc2r(int n, int howmany, double* data, long stride, long dist)
{ batch_transform(n, howmany, data, stride, dist, 1); }

