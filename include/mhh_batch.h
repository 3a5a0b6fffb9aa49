/*
 * mhh_batch.h -- batched ensembles and the serving loop (libmhh_host.so).
 *
 * Neither has a counterpart in the reference, which runs one simulation per
 * process.  Both drive models created with mhh_model_create (include/mhh_model.h)
 * and keep the results of every model identical to running it alone: the same
 * kernels with the same arguments run on the model's own stream.
 */
#ifndef MHH_BATCH_H
#define MHH_BATCH_H

#include "mhh_model.h"

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------------- */
/* Ensemble: many models of uneven sizes advanced together                  */
/* ---------------------------------------------------------------------- */

typedef struct mhh_ensemble mhh_ensemble;

enum mhh_ensemble_mode
{
    MHH_ENS_SEQUENTIAL = 0,  /* one member after another on one stream */
    MHH_ENS_STREAMS = 1,     /* every member on its own stream, substep by substep */
    MHH_ENS_GRAPHS = 2,      /* one CUDA-graph launch per RK3 substep for all members */
    MHH_ENS_BATCHED = 3      /* as GRAPHS, with one kernel launch per stage over all members of
                                one grid size (mhh_batch_substep), the sizes as parallel
                                branches; members whose kernels cannot run batched make this
                                an error */
};

int mhh_ensemble_create(mhh_ensemble** out);
/* Adds a model (borrowed: it must outlive the ensemble).  Graph mode needs a
   fixed time step (adaptivestep=false) in every member. */
int mhh_ensemble_add(mhh_ensemble* e, mhh_model* m);
/* Picks, per distinct grid size, the tendency and viscosity kernel variant and
   level chunk that run fastest, by timing a scratch model of that size, and
   sets them on the members' contexts (mhh_ctx_set_option).  The members'
   state is not touched.  A one-line summary of the choices goes to report. */
int mhh_ensemble_autotune(mhh_ensemble* e, char* report, int report_len);
/* n RK3 steps of every member in the given mode; does not synchronise.  In
   graph mode the first call runs one step eagerly and captures the next. */
int mhh_ensemble_run_steps(mhh_ensemble* e, int n, int mode);
int mhh_ensemble_synchronize(mhh_ensemble* e);
int mhh_ensemble_destroy(mhh_ensemble* e);

/* ---------------------------------------------------------------------- */
/* Server: simulation jobs admitted by device-memory budget                 */
/* ---------------------------------------------------------------------- */

typedef struct mhh_server mhh_server;

enum mhh_server_mode
{
    MHH_SERVE_FIFO = 0,      /* one job after another, in arrival order */
    MHH_SERVE_CONTINUOUS = 1 /* jobs admitted as memory and slots free up; their steps interleave */
};

/* budget_bytes: device memory the active jobs may hold (estimated from their
   grids before admission); max_active: concurrent jobs. */
int mhh_server_create(double budget_bytes, int max_active, mhh_server** out);
/* A job: the model's .ini text and full levels, its precision, the number of
   RK3 steps and its arrival time in seconds after the start of run.  keep = 1
   keeps u, v, w, th of the final state for mhh_server_get_result. */
int mhh_server_submit(mhh_server* s, const char* ini_text, const double* z, int ktot, int precision, int nsteps,
                      double arrival_s, int keep, int* job);
/* Initial field of a job (ghost layout, double), copied at submission. */
int mhh_server_set_initial(mhh_server* s, int job, const char* name, const double* data);
/* Runs every submitted job to completion in the given mode (a server can run
   its job list again in another mode; the jobs restart from their initial
   fields). */
int mhh_server_run(mhh_server* s, int mode);
/* Times of the last run, seconds after its start: arrival, admission, finish. */
int mhh_server_job_times(mhh_server* s, int job, double* arrival, double* admit, double* finish);
int mhh_server_get_result(mhh_server* s, int job, const char* name, double* data);
/* Largest sum of the admitted jobs' estimated device bytes during the last run. */
int mhh_server_peak_bytes(mhh_server* s, double* bytes);
/* Completed steps of the last run in the order the loop saw them: time
   (seconds after the start) and the cells the step advanced; count is the
   number of entries, at most max are written. */
int mhh_server_progress(mhh_server* s, double* times, double* cells, int max, int* count);
int mhh_server_destroy(mhh_server* s);
const char* mhh_batch_last_error(void);

#ifdef __cplusplus
}
#endif
#endif
