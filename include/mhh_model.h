/*
 * mhh_model.h -- C entry points of the host layer (libmhh_host.so): a whole
 * LES/DNS model driven from reference-style .ini text, with host buffers in
 * and out.  This is the call a user of the framework makes; it corresponds to
 * Model<TF> (src/model.cxx:67-581) with the fields injected instead of read
 * from restart files.  Fields are passed in double in the ghost-cell layout
 * (kcells x jcells x icells) whatever the precision of the model.
 */
#ifndef MHH_MODEL_H
#define MHH_MODEL_H

#include "mhh.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct mhh_model mhh_model;

/* Model<TF>::Model + init + load_or_save (cold start), src/model.cxx:109-300;
   z holds the ktot full levels (the "z" of <case>_input.nc). */
int mhh_model_create(const char* ini_text, const double* z, int ktot, int precision, mhh_model** out);
int mhh_model_destroy(mhh_model* m);
const char* mhh_model_last_error(void);

/* Fields: u v w th ut vt wt tht p evisc. */
int mhh_model_set_field(mhh_model* m, const char* name, const double* data);
int mhh_model_get_field(mhh_model* m, const char* name, double* data);
/* The same with host buffers in the model's own precision (double for FP64,
   float for FP32), copied on the model's stream without a conversion;
   asynchronous for page-locked buffers (call mhh_model_synchronize). */
int mhh_model_set_field_native(mhh_model* m, const char* name, const void* data);
int mhh_model_get_field_native(mhh_model* m, const char* name, void* data);

/* The time loop of src/model.cxx:356-505: n RK3 steps or substeps.
   fused = 1: one fused tendency kernel and a fused pressure-gradient + RK3
   kernel per substep; fused = 0: the module-by-module call sequence.
   Every [time] outputiter iterations (default 20; 0 = every substep) the
   status check of src/model.cxx:842-872 computes the CFL number at the start
   of a step and stops with MHH_ERR_NONFINITE ("Simulation has non-finite
   numbers") when it is NaN, inf or outside [0, 10). */
int mhh_model_run_steps(mhh_model* m, int n, int fused);
int mhh_model_run_substeps(mhh_model* m, int n, int fused);

/* Status diagnostics, src/model.cxx:819-873 (after the periodic fill). */
int mhh_model_get_cfl(mhh_model* m, double* out);
int mhh_model_get_dn(mhh_model* m, double* out);
int mhh_model_get_div(mhh_model* m, double* out);
int mhh_model_get_dt(mhh_model* m, double* out);
int mhh_model_get_time(mhh_model* m, double* out);
int mhh_model_get_substep(mhh_model* m, int* out);
int mhh_model_get_grid(mhh_model* m, mhh_grid* out);
int mhh_model_get_profile(mhh_model* m, const char* name, double* out);
int mhh_model_get_surface(mhh_model* m, const char* name, double* out);

/* Restart files in the reference's formats, in directory dir (NULL: the
   working directory), named by iotime = itime / 10^iotimeprec s:
   u|v|w|th.%07d (interior, model precision), time.%07d (itime, idt as
   64-bit unsigned, iteration as 32-bit int), with the surface model
   dudz_mo|dvdz_mo|dbdz_mo.%07d (interior 2-D, double) and th_gradbot.%07d.
   Fields.save/load (src/fields.cxx:1244-1344), Timeloop.save/load
   (src/timeloop.cxx:446-529), Boundary_surface.save/load
   (src/boundary_surface.cxx:584-700).  Files are never overwritten. */
int mhh_model_save(mhh_model* m, const char* dir, int* iotime);
int mhh_model_load(mhh_model* m, const char* dir, int iotime);

/* Relaxation target of the buffer layer ([buffer] swbuffer=true) for u, v
   or th: kcells values in the ghost layout, the case's initial profiles
   (src/buffer.cxx:130-150).  u and v, and th with a thermo scheme, must be
   set before the first step. */
int mhh_model_set_buffer_profile(mhh_model* m, const char* name, const double* prof);

/* Streams and device access for batched drivers. */
int mhh_model_set_stream(mhh_model* m, cudaStream_t s);
int mhh_model_synchronize(mhh_model* m);
int mhh_model_get_device_fields(mhh_model* m, mhh_fields* f, mhh_bcfields* bc);
mhh_ctx* mhh_model_get_ctx(mhh_model* m);

#ifdef __cplusplus
}
#endif
#endif
