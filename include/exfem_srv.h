/*
 * exfem_srv.h — serving many site-response solves on one GPU.
 *
 * No counterpart in the reference (damian.par runs one problem per MPI job,
 * main.f90:42-53).  A server keeps a queue of submitted problems and steps
 * several of them at once, each in its own exfem_ctx on its own CUDA stream,
 * so their kernels overlap on the device (continuous batching):
 *   - admission by HBM footprint: a request is admitted when its estimated
 *     device bytes (exfem_gpu_estimate_bytes) fit the budget next to the
 *     requests already running and a slot is free; requests that fit may pass
 *     a larger one at the head, which is protected from starving;
 *   - device setup of admitted requests (exfem_gpu_create, init_explicit)
 *     runs on preparer threads so it never stalls the stepping;
 *   - requests may arrive as problem.in text: the same threads run the host
 *     mesher (include/exfem_host.h) before admission, so meshing overlaps
 *     the stepping of other requests;
 *   - the scheduler thread advances every running request by chunks of steps
 *     and collects the seismograms of finished ones, freeing their memory.
 * Each request computes exactly what exfem_gpu_run would compute for it
 * alone; the mix only changes when it runs.
 */
#ifndef EXFEM_SRV_H
#define EXFEM_SRV_H

#include "exfem_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct exfem_srv exfem_srv;

typedef struct exfem_srv_opts {
    size_t hbm_budget;    /* device bytes the server may hold (0: 90% of free memory) */
    int    max_active;    /* requests stepping at once (0: 16)                        */
    int    chunk_steps;   /* steps queued per request and scheduler round (0: 256)    */
    int    preparers;     /* threads running device setup (0: 4)                      */
    int    max_bypass;    /* admissions that may pass the head request (0: 8)         */
    exfem_opts solver;    /* options for every request's context                      */
} exfem_srv_opts;

/* Outcome and timings (seconds since exfem_srv_open) of one request. */
typedef struct exfem_srv_result {
    long long id;
    int       status;      /* EXFEM_OK or the request's EXFEM_E_* code             */
    int       nsteps, nelems, nrhs, nrecv, nsave;
    size_t    device_bytes;    /* bytes its context held                        */
    size_t    reserved_bytes;  /* footprint reserved at admission (upper bound)  */
    double    t_submit, t_admit, t_ready, t_done;
    double    t_meshed;        /* mesh built (deck requests; = t_submit otherwise) */
} exfem_srv_result;

void exfem_srv_default_opts(exfem_srv_opts *opts);
int  exfem_srv_open(const exfem_srv_opts *opts, exfem_srv **out);

/* Queue one problem for nsteps steps.  The mesh and problem are copied; the
 * caller may free them on return.  *id receives the request id. */
int  exfem_srv_submit(exfem_srv *srv, const exfem_mesh *mesh, const exfem_problem *prob, int nsteps,
                      long long *id);

/* Queue one problem given as problem.in text (the deck format of
 * include/exfem_host.h).  A preparer thread builds its mesh and problem as
 * the Fortran host's init_model would (explicit.f90:16-70), then it waits
 * for admission like any other request.  nsteps <= 0 runs the deck's own
 * step count.  Deck errors come back as the request's status. */
int  exfem_srv_submit_deck(exfem_srv *srv, const char *deck, int nsteps, long long *id);

/* Finished requests not reported before (up to cap), waiting up to wait_ms
 * for at least one.  Returns how many were written. */
int  exfem_srv_poll(exfem_srv *srv, exfem_srv_result *out, int cap, int wait_ms);

/* Seismograms of a finished request, out[rhs][save][recv][2] as
 * exfem_gpu_get_seismograms; releases the request's host copy. */
int  exfem_srv_fetch(exfem_srv *srv, long long id, double *out, size_t cap);

/* Counters: requests waiting (deck requests still meshing included), being
 * prepared, stepping, finished; bytes held. */
int  exfem_srv_stats(exfem_srv *srv, int *waiting, int *preparing, int *active, long long *finished,
                     size_t *bytes_held, int *peak_active);

const char *exfem_srv_last_error(const exfem_srv *srv);

/* Stops the threads, destroys every context still held. */
void exfem_srv_close(exfem_srv *srv);

#ifdef __cplusplus
}
#endif
#endif /* EXFEM_SRV_H */
