/*
 * mhh.h -- C-ABI of the GB300 LES/DNS time step (libmhh_gb300.so).
 *
 * Plain C: device pointers, sizes and a cudaStream_t; no C++ or torch types.
 * Every entry point returns 0 on success or a negative mhh_status; the text
 * of the last error is available from mhh_last_error().  Nothing allocates
 * device memory except mhh_ctx_create (all scratch of the pressure solver,
 * the reductions and the surface layer lives in the context) and the
 * set-up call mhh_buffer_setup (the buffer layer's profiles).
 *
 * Fields use the reference's ghost-cell layout (include/grid.h:48-138):
 * element (i,j,k) of a 3-D field is at i + j*icells + k*ijcells, with the
 * interior at istart..iend-1, jstart..jend-1, kstart..kend-1.  2-D boundary
 * arrays have icells*jcells elements.  The element type is double for
 * MHH_FP64 contexts and float for MHH_FP32 contexts (the FP32 form keeps the
 * tridiagonal solve, the mean-mode pressure solve, the surface layer and all
 * reductions in double).
 *
 * Each entry point names the reference member function it replaces (paths
 * relative to the MicroHH source tree).
 */
#ifndef MHH_H
#define MHH_H

#include <stddef.h>
#include <cuda_runtime.h>

#ifdef __cplusplus
extern "C" {
#endif

enum mhh_status
{
    MHH_OK = 0,
    MHH_ERR_ARG = -1,         /* invalid argument (NULL pointer, bad size, bad switch) */
    MHH_ERR_CUDA = -2,        /* a CUDA call failed */
    MHH_ERR_UNSUPPORTED = -3, /* e.g. an FFT length with a prime factor above 7 */
    MHH_ERR_NONFINITE = -4,   /* a reduction returned NaN or inf; a model run with non-finite numbers */
    MHH_ERR_TIMEOUT = -5      /* a bounded device wait ran out */
};

enum mhh_precision { MHH_FP64 = 64, MHH_FP32 = 32 };
enum mhh_advec { MHH_ADVEC_2 = 2, MHH_ADVEC_2I5 = 25 };
enum mhh_diff { MHH_DIFF_NONE = 0, MHH_DIFF_2 = 2, MHH_DIFF_SMAG2 = 7 };
/* include/boundary.h:42 Boundary_type */
enum mhh_bc { MHH_BC_DIRICHLET = 0, MHH_BC_NEUMANN = 1, MHH_BC_FLUX = 2 };
/* src/boundary_cyclic.cxx:370 Edge */
enum mhh_edge { MHH_EDGE_EW = 1, MHH_EDGE_NS = 2, MHH_EDGE_BOTH = 3 };

typedef struct mhh_ctx mhh_ctx;

/* Grid description: the inputs of Grid<TF> (src/grid.cxx:47-100) plus the
   ghost-cell counts the schemes ask for (Advec_2i5: 3,3,1, or 3,3,2 with a
   flux-limited scalar; otherwise 1,1,1). */
typedef struct
{
    int itot, jtot, ktot;
    int igc, jgc, kgc;
    double xsize, ysize, zsize;
} mhh_grid_desc;

/* Derived grid data (mirrors Grid_data, include/grid.h:48-138). */
typedef struct
{
    int itot, jtot, ktot;
    int igc, jgc, kgc;
    int icells, jcells, kcells, ijcells;
    int istart, iend, jstart, jend, kstart, kend;
    long long ncells;
    double dx, dy, zsize;
    int precision;
} mhh_grid;

/* Physics constants the modules read from the .ini file. */
typedef struct
{
    double visc, svisc;        /* [fields] visc, svisc */
    double cs, tpr, dnmax;     /* [diff] cs, tPr, dnmax */
    int swmason;               /* [diff] swmason */
    double cflmax;             /* [advec] cflmax */
    double thref0;             /* [thermo] thref0 (Boussinesq) */
    int thermo;                /* 1: dry thermodynamics with prognostic scalar */
    int surface;               /* 1: swboundary=surface */
    double z0m, z0h;           /* [boundary] z0m, z0h (homogeneous roughness) */
} mhh_physics;

/* Device pointers of the prognostic state (ghost layout, ncells each). */
typedef struct
{
    void *u, *v, *w, *s;           /* s: the thermodynamic scalar (th) or NULL */
    void *ut, *vt, *wt, *st;       /* tendencies */
    void *evisc;                   /* eddy viscosity (Smagorinsky) or NULL */
    void *p;                       /* pressure (ghost layout) */
} mhh_fields;

/* 2-D boundary arrays (icells*jcells, device): bottom/top value, gradient and
   flux of u, v and s (Field3d fld_bot/grad_bot/flux_bot..., include/field3d.h). */
typedef struct
{
    void *u_bot, *u_top, *u_gradbot, *u_gradtop, *u_fluxbot, *u_fluxtop;
    void *v_bot, *v_top, *v_gradbot, *v_gradtop, *v_fluxbot, *v_fluxtop;
    void *s_bot, *s_top, *s_gradbot, *s_gradtop, *s_fluxbot, *s_fluxtop;
} mhh_bcfields;

/* ---------------------------------------------------------------------- */
/* Context                                                                 */
/* ---------------------------------------------------------------------- */

/* Grid<TF>::init + Grid<TF>::create/calculate (src/grid.cxx:105-305) and the
   device set-up of Pres_2 (src/pres_2.cu:221-245, FFT plans of
   src/pres.cu:208-285): computes the 2nd-order vertical metrics from the ktot
   full levels z, uploads them and allocates all scratch. */
int mhh_ctx_create(const mhh_grid_desc* desc, const double* z, int precision,
                   const mhh_physics* phys, mhh_ctx** out);
int mhh_ctx_destroy(mhh_ctx* ctx);
int mhh_ctx_get_grid(const mhh_ctx* ctx, mhh_grid* out);
/* Vertical profile (z zh dz dzh dzi dzhi rhoref rhorefh) to host, kcells doubles. */
int mhh_ctx_get_profile(const mhh_ctx* ctx, const char* name, double* out);
const char* mhh_last_error(void);
/* Kernels this library launched since load (for launch accounting). */
long long mhh_launch_count(void);
/* Adds n to that count: a driver that replays a captured CUDA graph adds the
   graph's kernel nodes per replay (no counterpart in the reference). */
int mhh_launch_count_add(long long n);
/* Device memory the context allocated (measured at creation), and an upper
   estimate of it from the grid alone, for admission by memory budget (no
   counterpart in the reference). */
int mhh_ctx_device_bytes(const mhh_ctx* ctx, size_t* bytes);
int mhh_ctx_estimate_bytes(const mhh_grid_desc* desc, int precision, size_t* bytes);

/* Process-wide kernel options (no counterpart in the reference; the
   reference picks kernel variants through its Kernel Launcher wisdom files):
   "tendency_kernel" 0 = one thread per cell, 1 = tiled planes marching in k,
   2 = flux form (each face flux computed once) marching in k, -1 = automatic
   (2; the default);
   "viscosity_kernel" 0 = one thread per cell, 1 = shared-memory planes
   marching in k, -1 = automatic (1; the default; the neutral resolved-wall
   case always runs per cell);
   "tdma_kernel" 0 = the Thomas recurrence in the reference's operation order,
   1 = the rescaled recurrence (two FP64 FMAs per cell) with one column per
   thread, 2 = the same with the four columns of one eigenvalue per thread,
   3 = the rescaled recurrence in float for the column groups whose forward
   sweep damps (max |g| <= 0.999) and in FP64 for the others (FP32 contexts;
   1 in FP64 contexts), -1 = automatic (0 for FP64 contexts, 3 for FP32
   contexts; the default). */
int mhh_set_option(const char* name, int value);
/* "fft_pipeline": 1 (the default) runs the fixed-length FFTs as persistent
   blocks that load their next tile while transforming the current one; 0
   runs one tile per block.  Both give identical results.
   "fft_column_pairs": complex sequence pairs per tile of the y FFT, 8 (the
   default: 16 adjacent columns, 512 threads per block, float fields; 256
   threads for the 512-point warp-synchronous schedule, one warp per pair)
   or 4.  "pres_fuse": 1 (the default) computes the Poisson
   right-hand side inside the forward x FFT and stores the inverse x FFT into
   the ghost layout of p; 0 runs them as separate kernels. */
/* "tendency_kchunk" / "viscosity_kchunk": levels per block of the marching
   kernels, 4, 8, 16, 32 or 64, or 0 (the default: 64 where the grid gives at
   least eight blocks per SM, else 32, halved down to 8 while the grid would
   give fewer than two blocks per SM). */
/* The same options for one context, overriding the process-wide value;
   -2 returns to it (no counterpart in the reference; used by the ensemble
   autotuner to pick variants and level chunks per grid size). */
int mhh_ctx_set_option(mhh_ctx* ctx, const char* name, int value);

/* Live per-kernel-group timing with CUDA events recorded on the launching
   stream (no counterpart in the reference, which has no event timing):
   enable, run, then collect (waits for the recorded events) and read the
   accumulated count and milliseconds per group. */
int mhh_timing_enable(int on);
int mhh_timing_reset(void);
int mhh_timing_collect(void);
int mhh_timing_count(void);
int mhh_timing_get(int idx, const char** name, long long* count, double* total_ms);

/* ---------------------------------------------------------------------- */
/* Boundaries                                                              */
/* ---------------------------------------------------------------------- */

/* Boundary_cyclic<TF>::exec (src/boundary_cyclic.cxx:370-440): periodic
   ghost cells of one 3-D field over all levels. */
int mhh_boundary_cyclic(mhh_ctx* ctx, void* data, int edges, cudaStream_t stream);

/* Boundary<TF>::set_values (src/boundary.cxx:615-700): fills the 2-D
   value/gradient/flux arrays of one field for a homogeneous BC. */
int mhh_boundary_set_bc(mhh_ctx* ctx, void* val, void* grad, void* flux, int bc_type,
                        double aval, double visc, int set_flux_grad, cudaStream_t stream);

/* Boundary<TF>::set_ghost_cells, 2nd order (src/boundary.cxx:700-760,
   :933-998) for one field: bottom and top ghost level from the BC types. */
int mhh_boundary_ghost_cells(mhh_ctx* ctx, void* a, int bot_type, const void* abot, const void* agradbot,
                             int top_type, const void* atop, const void* agradtop, cudaStream_t stream);

/* Boundary_surface<TF>::exec (src/boundary_surface.cxx:836-994), lookup-table
   Obukhov solver with homogeneous z0m/z0h (from mhh_physics), noslip momentum
   and a flux or Dirichlet scalar: updates the surface fluxes and gradients and
   the MO gradients kept in the context (used by the next Diff_smag2
   viscosity).  thermo_bc is the scalar's bottom BC type. */
int mhh_boundary_surface_exec(mhh_ctx* ctx, const mhh_fields* f, const mhh_bcfields* bc,
                              int thermo_bc, cudaStream_t stream);
/* Cold-start state of the surface layer (src/boundary_surface.cxx:545-580)
   and the z/L lookup table (include/boundary_surface_kernels.h:77-130). */
int mhh_boundary_surface_init(mhh_ctx* ctx, int thermo_bc);
/* Surface 2-D arrays to host (icells*jcells doubles): ustar obuk dudz dvdz dbdz;
   and back (restart, Boundary_surface<TF>::load, src/boundary_surface.cxx:584-643). */
int mhh_boundary_surface_set(mhh_ctx* ctx, const char* name, const double* in);
int mhh_boundary_surface_get(mhh_ctx* ctx, const char* name, double* out);

/* ---------------------------------------------------------------------- */
/* Advection                                                               */
/* ---------------------------------------------------------------------- */

/* Advec_2i5<TF>::exec (src/advec_2i5.cxx:995-1063): adds the 5th-order
   upwind advection tendencies to ut, vt, wt and st. */
int mhh_advec_2i5_exec(mhh_ctx* ctx, const mhh_fields* f, cudaStream_t stream);
/* Advec_2i5 with th in [advec] fluxlimit_list (src/advec_2i5.cxx:36-46,
   1047-1056; include/advec_monotonic.h:28-219): limit_scalar = 1 advects the
   scalar with the Koren flux limiter, in mhh_advec_2i5_exec and in the fused
   substep.  The reference then runs with kgc = 2 (the context accepts 1 or
   2); ktot >= 4. */
int mhh_advec_2i5_set_fluxlimit(mhh_ctx* ctx, int limit_scalar);
/* Advec_2<TF>::exec (src/advec_2.cxx:280-351). */
int mhh_advec_2_exec(mhh_ctx* ctx, const mhh_fields* f, cudaStream_t stream);
/* Advec_2i5<TF>::get_cfl / Advec_2<TF>::get_cfl (src/advec_2i5.cxx:953-971,
   src/advec_2.cxx:232-244): the CFL number times dt, in double; synchronises. */
int mhh_advec_get_cfl(mhh_ctx* ctx, int scheme, const mhh_fields* f, double dt, double* cfl, cudaStream_t stream);
/* Advec::get_time_limit (src/advec_2i5.cxx:974-992). */
int mhh_advec_get_time_limit(mhh_ctx* ctx, int scheme, const mhh_fields* f, unsigned long long idt,
                             double dt, unsigned long long* idt_lim, cudaStream_t stream);

/* ---------------------------------------------------------------------- */
/* Diffusion                                                               */
/* ---------------------------------------------------------------------- */

/* Diff_smag2<TF>::exec_viscosity (src/diff_smag2.cxx:473-607): strain rate,
   N2 of the dry thermodynamics, eddy viscosity, wall mirror and cyclic fill. */
int mhh_diff_smag2_exec_viscosity(mhh_ctx* ctx, const mhh_fields* f, const mhh_bcfields* bc, cudaStream_t stream);
/* Diff_smag2<TF>::exec (src/diff_smag2.cxx:380-471). */
int mhh_diff_smag2_exec(mhh_ctx* ctx, const mhh_fields* f, const mhh_bcfields* bc, cudaStream_t stream);
/* Diff_smag2<TF>::get_dn (src/diff_smag2.cxx:336-356); synchronises. */
int mhh_diff_smag2_get_dn(mhh_ctx* ctx, const mhh_fields* f, double dt, double* dn, cudaStream_t stream);
/* Diff_2<TF>::exec (src/diff_2.cxx:166-192). */
int mhh_diff_2_exec(mhh_ctx* ctx, const mhh_fields* f, cudaStream_t stream);
/* Diff_2<TF>::get_dn (src/diff_2.cxx:133-160): constant multiplier times dt. */
int mhh_diff_2_get_dn(mhh_ctx* ctx, double dt, double* dn);

/* ---------------------------------------------------------------------- */
/* Thermodynamics and forcing                                              */
/* ---------------------------------------------------------------------- */

/* Thermo_dry<TF>::exec, 2nd order (src/thermo_dry.cxx:610-627): buoyancy
   tendency on w. */
int mhh_thermo_dry_exec(mhh_ctx* ctx, const mhh_fields* f, cudaStream_t stream);
/* Force<TF>::exec with swlspres=dpdx (src/force.cxx:626-636). */
int mhh_force_dpdx_exec(mhh_ctx* ctx, const mhh_fields* f, double dpdx, cudaStream_t stream);

/* ---------------------------------------------------------------------- */
/* Pressure                                                                */
/* ---------------------------------------------------------------------- */

/* Storage offset of the scalar (potential temperature).  FP32 contexts with
   thermodynamics store theta - thref0 (the Boussinesq reference, so that the
   float keeps 1e-8 K of a boundary-layer fluctuation instead of 3e-5 K of
   300 K); FP64 contexts store theta itself (offset 0).  The 3-D scalar field
   and its boundary values passed to the entry points are in these storage
   units; profiles passed by name (mhh_buffer_set_profile) are physical.  No
   counterpart in the reference (its fields hold theta). */
int mhh_ctx_scalar_offset(const mhh_ctx* ctx, double* offset);
/* Adds delta to every cell (ghost cells included) of a 3-D field in the
   field precision; used to move the scalar between physical and storage
   units on the device. */
int mhh_field_shift(mhh_ctx* ctx, void* field, double delta, cudaStream_t stream);

/* Pres_2<TF>::exec (src/pres_2.cxx:65-94): divergence of the predicted
   velocity, x/y real FFTs (hand-written, no cuFFT), tridiagonal solve in z in
   double, inverse FFTs and the pressure gradient into ut, vt, wt. */
int mhh_pres_2_exec(mhh_ctx* ctx, const mhh_fields* f, double sub_dt, cudaStream_t stream);
/* Pres_2<TF>::check_divergence (src/pres_2.cxx:97-105, :389-422): maximum
   absolute divergence, in double; synchronises. */
int mhh_pres_2_get_divergence(mhh_ctx* ctx, const mhh_fields* f, double* div, cudaStream_t stream);

/* The same maximum absolute divergence without any device allocation (no
   counterpart in the reference).  For callers that must not allocate device
   memory after set-up, e.g. a host that charges every device allocation
   against a fixed HBM budget.  The scratch is a file-scope device array of
   the library: jtot*ktot <= 262144 (2 MiB of row maxima), larger grids return
   MHH_ERR_ARG.  The first call on each device looks up the array's address
   and, as CUDA loads kernels lazily, may load the module that holds the
   array (2 MiB of device memory, possibly a device synchronisation): make
   one warm-up call during set-up, before any stream capture.  Calls on one
   device share the array, so calls that overlap in time race and must be
   serialised by the caller.  A NaN in u, v or w returns MHH_ERR_NONFINITE.
   Synchronises the stream. */
int mhh_pres_2_get_divergence_noalloc(mhh_ctx* ctx, const mhh_fields* f, double* div, cudaStream_t stream);
/* Halfcomplex x/y transforms of a packed itot*jtot*ktot array in place
   (FFT<TF>::exec_forward / exec_backward, src/fft.cxx:337-452). */
int mhh_fft_forward(mhh_ctx* ctx, void* data, cudaStream_t stream);
int mhh_fft_backward(mhh_ctx* ctx, void* data, cudaStream_t stream);

/* Buffer<TF> damping layer (src/buffer.cxx:37-160, swupdate=false): setup
   from [buffer] zstart, sigma, beta; the relaxation targets of u, v and th
   (kcells each, the case's initial profiles; w relaxes to zero); exec adds
   -sigma(z) (a - abuf) to the tendencies above zstart.  Once set up, the
   fused substep applies it after advection and diffusion, as the reference's
   time loop does (src/model.cxx:416). */
int mhh_buffer_setup(mhh_ctx* ctx, double zstart, double sigma, double beta);
int mhh_buffer_set_profile(mhh_ctx* ctx, const char* name, const double* prof);
int mhh_buffer_exec(mhh_ctx* ctx, const mhh_fields* f, cudaStream_t stream);

/* Horizontal mean and variance (about the mean) of every level of a 3-D
   field, kcells values each, in double (Field3d_operators<TF>::
   calc_mean_profile, src/field3d_operators.cxx:46-67, with the variance of
   the statistics' second moments); synchronises. */
int mhh_stats_profile(mhh_ctx* ctx, const void* field, double* mean, double* var, cudaStream_t stream);

/* ---------------------------------------------------------------------- */
/* Time integration                                                        */
/* ---------------------------------------------------------------------- */

/* Timeloop<TF>::exec with rkorder=3 (src/timeloop.cxx:250-286, :358-387) for
   one field pair: a += cB[substep]*dt*at; at *= cA[substep+1], or at = 0
   over all cells after the last substep. */
int mhh_timeloop_rk3(mhh_ctx* ctx, void* a, void* at, int substep, double dt, cudaStream_t stream);

/* ---------------------------------------------------------------------- */
/* Fused substep (the GB300 path used by the C++ Model)                    */
/* ---------------------------------------------------------------------- */

/* Configuration of a whole substep. */
typedef struct
{
    int advec;                 /* mhh_advec */
    int diff;                  /* mhh_diff */
    int swlspres;              /* 1: constant pressure gradient */
    double dpdx;
    int mbcbot, mbctop;        /* momentum BC types */
    int sbcbot, sbctop;        /* scalar BC types */
} mhh_substep_config;

/* One RK3 substep in the order of src/model.cxx:356-505, split where the host
   may pick the time step (set_time_step needs this substep's viscosity):
   begin = periodic and wall ghost cells, Smagorinsky viscosity;
   end   = surface layer, ghost cells, advection + diffusion + buoyancy +
           forcing in one fused tendency kernel, pressure solve, and the
           pressure gradient fused with the RK3 update of all fields.
   dt is the full time step; substep is 0, 1 or 2.  Neither synchronises. */
int mhh_substep_begin(mhh_ctx* ctx, const mhh_substep_config* cfg, const mhh_fields* f,
                      const mhh_bcfields* bc, cudaStream_t stream);
int mhh_substep_end(mhh_ctx* ctx, const mhh_substep_config* cfg, const mhh_fields* f,
                    const mhh_bcfields* bc, int substep, double dt, cudaStream_t stream);

/* Batched substeps (no counterpart in the reference, which runs one
   simulation per process): n contexts of one precision -- ensemble members
   or served jobs, of uneven grid sizes -- advance a fused substep together
   with one kernel launch per stage over all of them (per group of contexts
   whose stage runs the same kernel, e.g. one group per FFT length).  Each
   context keeps its own fields; cfg, f, bc and dt are per context (dt is the
   fixed full time step).  Every context gets the kernels and parameters of
   its own mhh_substep_begin/end, so its results are the same bit for bit.
   mhh_batch_create records the contexts' substeps without running them and
   builds the launch parameters on the host (no device memory; the kernels
   take up to 32 KB of parameters per launch, larger groups are split into
   several launches); call it after one ordinary substep of every
   context (kernel attributes are set on first use) and outside any stream
   capture.  A configuration with a kernel that cannot run batched (the
   separate pressure right-hand-side and scatter kernels of the option
   pres_fuse = 0) returns MHH_ERR_UNSUPPORTED.
   mhh_batch_substep launches substep 0, 1 or 2 of all contexts on the
   stream; mhh_batch_launches gives its number of launches. */
typedef struct mhh_batch mhh_batch;
int mhh_batch_create(int n, mhh_ctx* const* ctx, const mhh_substep_config* cfg, const mhh_fields* f,
                     const mhh_bcfields* bc, const double* dt, mhh_batch** out);
int mhh_batch_substep(mhh_batch* b, int substep, cudaStream_t stream);
int mhh_batch_launches(const mhh_batch* b, int substep, int* nlaunch);
int mhh_batch_destroy(mhh_batch* b);

#ifdef __cplusplus
}
#endif
#endif
