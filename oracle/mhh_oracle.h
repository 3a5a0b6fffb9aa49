/*
 * mhh_oracle.h -- CPU oracle for the MicroHH 2nd-order LES/DNS time step.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C, FP64 restatement of the
 * reference algorithm for the hot path (Advec_2i5 / Advec_2, Diff_smag2 /
 * Diff_2, Thermo_dry buoyancy, Pres_2 with x/y real FFTs and a Thomas solve
 * in z, the low-storage RK3 and the CFL / diffusion-number / divergence
 * reductions).  It is used by the tests, by __graft_entry__.smoke() and by
 * bench.py's CPU-baseline leg to compare against.  The product path never links,
 * loads or calls it.
 *
 * The same C API is exported by oracle/_ref/libmhh_ref.so, which is built
 * from the reference's own unchanged hot-path sources plus a stub host layer
 * (oracle/ref_harness); the golden fixtures under tests/golden were produced
 * by that build and pin this restatement.
 */
#ifndef MHH_ORACLE_H
#define MHH_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* Scheme switches (values mirror the reference's .ini strings). */
enum { ORC_ADVEC_2 = 2, ORC_ADVEC_2I5 = 25 };
enum { ORC_DIFF_2 = 2, ORC_DIFF_SMAG2 = 7 };
/* Boundary types, include/boundary.h Boundary_type. */
enum { ORC_BC_DIRICHLET = 0, ORC_BC_NEUMANN = 1, ORC_BC_FLUX = 2 };

typedef struct
{
    int itot, jtot, ktot;
    double xsize, ysize, zsize;

    int advec;        /* ORC_ADVEC_2 or ORC_ADVEC_2I5 */
    int diff;         /* ORC_DIFF_2 or ORC_DIFF_SMAG2 */
    int thermo;       /* 0: no scalars; 1: dry, Boussinesq, prognostic "th" */
    int surface;      /* 0: swboundary=default; 1: swboundary=surface (MOST) */

    int mbcbot, mbctop;       /* momentum BC types */
    int sbcbot, sbctop;       /* scalar BC types */
    double ubot, utop, vbot, vtop, sbot, stop;

    double visc, svisc;
    double cs, tpr, dnmax;
    int swmason;
    double cflmax;
    double thref0;

    int swlspres;     /* 0 off, 1 constant pressure gradient dpdx */
    double dpdx;

    double z0m, z0h;

    double dt, dtmax;
    int adaptivestep;

    int swbuffer;     /* 1: damping layer above buf_zstart ([buffer] swbuffer) */
    double buf_zstart, buf_sigma, buf_beta;
    int fluxlimit_s;  /* 1: th advected with the flux limiter ([advec] fluxlimit_list=th; 2i5 only) */
} orc_params;

typedef struct orc_model orc_model;

/* Creates a model.  z holds the ktot full-level heights (interior only). */
orc_model* orc_create(const orc_params* p, const double* z);
void orc_destroy(orc_model* m);

/* Number of cells of one 3-D field including ghost cells, and the ghost-cell
   counts (igc, jgc, kgc) the scheme selection implies. */
long orc_ncells(const orc_model* m);
void orc_dims(const orc_model* m, int* dims /* [igc,jgc,kgc,icells,jcells,kcells] */);

/* Copies a full ghost-layout 3-D field in or out.  Names: u v w th ut vt wt
   tht p evisc.  Returns 0 on success, -1 for an unknown name. */
int orc_set_field(orc_model* m, const char* name, const double* data);
int orc_get_field(const orc_model* m, const char* name, double* data);

/* Grid profiles of length kcells: z zh dz dzh dzi dzhi rhoref rhorefh. */
int orc_get_profile(const orc_model* m, const char* name, double* data);

/* 2-D surface arrays of length icells*jcells: ustar obuk dudz dvdz dbdz
   u_fluxbot v_fluxbot th_fluxbot u_gradbot v_gradbot th_gradbot. */
int orc_get_2d(const orc_model* m, const char* name, double* data);

/* Runs n RK3 substeps in the order of the reference's Model::exec time loop. */
void orc_run_substeps(orc_model* m, int n);

/* Diagnostics on the current fields, like the reference's status line. */
double orc_get_cfl(orc_model* m);
double orc_get_dn(orc_model* m);
double orc_get_div(orc_model* m);
double orc_get_dt(const orc_model* m);
int orc_get_substep(const orc_model* m);
unsigned long orc_get_itime(const orc_model* m);

/* Individual module calls, for per-operator parity tests. */
void orc_set_cyclic_and_ghost(orc_model* m);
void orc_exec_viscosity(orc_model* m);
void orc_exec_thermo(orc_model* m);
void orc_exec_boundary(orc_model* m);
void orc_exec_advec(orc_model* m);
void orc_exec_diff(orc_model* m);
void orc_exec_force(orc_model* m);
void orc_exec_buffer(orc_model* m);
/* Buffer profile of u, v or th (kcells values), the relaxation target of the
   damping layer (the initial profiles of the case). */
int orc_set_buffer_profile(orc_model* m, const char* name, const double* prof);
void orc_exec_pres(orc_model* m, double sub_dt);
void orc_exec_timeloop(orc_model* m);

/* Real halfcomplex transforms (FFTW R2HC / HC2R conventions, unnormalised)
   of `howmany` sequences of length n; element j of sequence s sits at
   data[s*dist + j*stride]. */
void orc_r2hc(int n, int howmany, double* data, long stride, long dist);
void orc_hc2r(int n, int howmany, double* data, long stride, long dist);

/* Number of OpenMP threads the oracle uses (1 when built without OpenMP). */
int orc_num_threads(void);

#ifdef __cplusplus
}
#endif
#endif
