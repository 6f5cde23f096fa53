/*
 * exfem_gpu.h — C ABI of the GB300 (sm_103a) explicit time-stepping library.
 *
 * This is the drop-in boundary for the time loop of damian.par ("exfem"):
 * the Fortran host keeps problem.in parsing, quadtree meshing and seismogram
 * output and hands the finished model to this library instead of running
 * init_explicit()/run_explicit() (explicit.f90:79-159) itself.
 *
 * Conventions follow the reference's own FFI (io.h:1-39, io_utils.f90:14-286):
 * plain pointers and sizes, `extern "C"`, 1-based indices exactly as they sit
 * in the Fortran arrays and in mesh.bin (io.cpp:333-367).  The caller owns every
 * host array; the library copies what it needs to the device on create and only
 * writes into caller-provided buffers (no malloc hand-off as in
 * util_temps.m4:86-95).  Errors are negative status codes and a message string;
 * the library never calls exit() (compare io.cpp:29-35, pwaves.f90:32-35, 87-89).
 *
 * Threading: one host thread per context; distinct contexts may be used from
 * different threads, each runs on its own CUDA stream.
 */
#ifndef EXFEM_GPU_H
#define EXFEM_GPU_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------- */
#define EXFEM_OK               0
#define EXFEM_E_ARG           -1   /* bad argument / inconsistent sizes          */
#define EXFEM_E_MESH          -2   /* malformed mesh (non-hanging count != 4 ...) */
#define EXFEM_E_NOMEM         -3   /* device or host allocation failed            */
#define EXFEM_E_UNSUPPORTED   -4   /* grazing / post-critical wave, chained hanging */
#define EXFEM_E_CUDA          -5   /* CUDA runtime error                          */
#define EXFEM_E_NAN           -6   /* non-finite state detected by the watchdog   */
#define EXFEM_E_TIMEOUT       -7   /* bounded device wait ran out                 */
#define EXFEM_E_STATE         -8   /* call out of order (run before init ...)     */

/* ---- wave kinds (m_prob, model.f90:692-696) ------------------------------ */
#define EXFEM_WAVE_P   1           /* 'WAVEP ' */
#define EXFEM_WAVE_SV  2           /* 'WAVESV' */

/* ---- arithmetic forms ----------------------------------------------------- */
#define EXFEM_FP64          0      /* plain FP64, same update as explicit.f90:126-152 */
#define EXFEM_FP32_KAHAN    1      /* FP32 increment form, Kahan-compensated u      */

/* ---- FP64 kernel variants ------------------------------------------------ */
#define EXFEM_VARIANT_REFERENCE_ORDER 0  /* dense calck dgemv, element-order sums,
                                            no contraction: the oracle's rounding */
#define EXFEM_VARIANT_CLOSED_FORM     1  /* closed-form Q4 K.u with FMA (fewer
                                            FP64 operations, rounding differs)  */

/* ---- hanging-anchor reduction ---------------------------------------------- */
#define EXFEM_HANG_HALF     0      /* r_a += r_h/2 (communicator.f90:1232 twin)     */
#define EXFEM_HANG_LITERAL  1      /* text of model.f90:643-645 (oracle only)       */

/* One plane wave = one right-hand side.  Mirrors the PROBLEM: parameters that
 * init_wave() reads (model.f90:982-1001): m_wttoorigin = pparams(6),
 * m_wangle = pparams(7), m_wamp = pparams(8), m_wfreq = pparams(9). */
typedef struct exfem_wave {
    int    kind;       /* EXFEM_WAVE_P or EXFEM_WAVE_SV                          */
    double amp;        /* amplitude a (P) or b (SV)                              */
    double angle;      /* incidence angle [rad]                                  */
    double freq;       /* Ricker central frequency [Hz]                          */
    double t0;         /* time to origin [s]                                      */
} exfem_wave;

/* The mesh as mesh.bin stores it (io.cpp:333-367; model.f90:51-61). */
typedef struct exfem_mesh {
    int nelems;
    int nnodes;
    const int           *eptr;      /* [nelems+1], 1-based CSR offsets (m_eptr)       */
    const int           *eind;      /* [eptr[nelems]-1], 1-based node ids (m_eind)    */
    const unsigned char *ediv;      /* [eptr[nelems]-1], 1 = hanging slot (m_ediv)    */
    const double        *nodes;     /* [2*nnodes], (x, depth) pairs (m_nodes)          */
    const int           *ematprop;  /* [nelems], 1-based material id (m_ematprop)     */
} exfem_mesh;

/* Everything problem_setup()/init_wave()/recalculate_deltat() leave in the
 * model module (model.f90:21-101, 958-1106; communicator.f90:1629-1662). */
typedef struct exfem_problem {
    int           nmat;
    const double *matconst;   /* [5*nmat] (mu, lambda, rho, vp, vs) per material   */
    const int    *absorbing;  /* [nnodes] 0 none, 1 AB_ZDIR, 2 AB_XDIR            */
    int           nhanging;
    const int    *hanging;    /* [3*nhanging] (hanging, previous, next), 1-based   */
    int           nseismic;
    const int    *seismic;    /* [2*nseismic] (element, kind SE_*), 1-based        */
    double        deltat;     /* m_deltat                                           */
    int           nsteps;     /* m_nsteps                                           */
    int           io_interval;/* io_interval (receivers are sampled on these steps) */
    double        worigin[2]; /* m_worigin                                          */
    double        wbox[3];    /* DRM box: left, right, top (model.f90:205-207)       */
    double        walpha;     /* vp of the exterior material, m_wvelo(1)            */
    double        wbeta;      /* vs of the exterior material, m_wvelo(2)            */
    int           nrhs;
    const exfem_wave *waves;  /* [nrhs]                                            */
    int           nrecv;
    const double *recv_xy;    /* [2*nrecv] receiver points (find_highest output)    */
    const int    *recv_elem;  /* [nrecv] 1-based top element of each receiver       */
    /* Point source (setup_point_source, model.f90:1051-1078).  The y dof of
     * every listed node takes r(t) = amp exp(-t^2/(4 sigma)) (t^2 - 2 sigma) /
     * (8 sqrt(pi) sigma^2.5) at t = time - t0 (ricker, formulation.f90:53-59):
     *   EXFEM_POINT_FORCE (POINTN): added to the node's reaction after the
     *     element sums, before the anchor sums (point_reactions,
     *     model.f90:808-822; explicit.f90:144);
     *   EXFEM_POINT_DISP (POINTD): set as its displacement after each update,
     *     before the hanging-node averages, and at t = 0 and -dt for u and u-
     *     (point_displacements, model.f90:831-845; explicit.f90:93-94, 150).
     * Every right-hand side gets the same source.  Zero-initialised fields
     * mean no point source.  A problem with a point source and no DRM layer
     * (nseismic = 0) may pass waves = NULL: no free field is added anywhere. */
    int           point_kind;  /* 0 (none), EXFEM_POINT_FORCE or EXFEM_POINT_DISP */
    int           npoint;
    const int    *point_nodes; /* [npoint] 1-based node ids (hanging ones allowed) */
    double        point_amp, point_sigma, point_t0;   /* m_pointamp/sigma/start   */
} exfem_problem;

#define EXFEM_POINT_FORCE   1
#define EXFEM_POINT_DISP    2

typedef struct exfem_opts {
    int precision;     /* EXFEM_FP64 or EXFEM_FP32_KAHAN                          */
    int device;        /* CUDA device ordinal                                     */
    int use_graph;     /* 1: replay the step as a captured CUDA graph             */
    int graph_steps;   /* steps captured per graph (0 = library default)          */
    int block_threads; /* node-kernel block size (0 = default / autotuned)        */
    int rhs_per_thread;/* right-hand sides per thread in batched form (0 = auto)  */
    int reorder;       /* 1: renumber nodes/elements in Morton order on device    */
    int check_every;   /* non-finite watchdog period in steps (0 = off)           */
    int variant;       /* FP64: EXFEM_VARIANT_REFERENCE_ORDER (default) or
                          EXFEM_VARIANT_CLOSED_FORM.  FP32: 0 = direct gather
                          (default), 1 = shared-memory tiled step, 2 = tiles
                          streamed by bulk copies through a two-stage
                          shared-memory pipeline (persistent grid; needs nrhs
                          a multiple of 4, else the direct gather runs),
                          3 = element products on the tensor cores (tcgen05
                          kind::tf32 in 3xTF32; needs nrhs a multiple of 16,
                          else the direct gather runs), 4 = the direct
                          gather as a persistent grid (same results as 0),
                          5 = the direct gather reading every node's terms
                          through list pointers, which 0 and 4 do below
                          50,000 active nodes, instead of fixed-size node
                          records (same results as 0)                     */
    int index_bits;    /* FP32 direct gather: 0 = 32-bit indices when every
                          thread id and array index fits, else 64; 64 = always
                          64-bit (same results)                               */
    int pad_rhs;       /* FP32 form: 0 = pad the right-hand sides to an even
                          count (a multiple of 4 from 14) with zero-amplitude
                          waves when that aligns the state rows; 1 = never.
                          Same results; every output covers only the caller's
                          right-hand sides                                    */
    int wait_cycles;   /* bound of each device-side wait (the mbarrier waits
                          of FP32 variant 2), in SM clock cycles; 0 = the
                          library default, 2e9 (about 1 s at 2 GHz).  A wait
                          that runs out sets a watchdog flag; the kernel then
                          waits (with the default bound) for its own copies
                          in flight and returns, and exfem_gpu_sync reports
                          EXFEM_E_TIMEOUT.  The counterpart of the
                          reference's fatal mpi_abort path
                          (communicator.f90:144-156), as a status          */
    int tune;          /* FP32 direct gather: 1 = at exfem_gpu_init_explicit,
                          time every right-hand-sides-per-thread and block
                          shape on this context for a few steps from rest
                          (CUDA events on its stream) and keep the fastest,
                          unless rhs_per_thread or block_threads is set; the
                          state is then reset.  0 = the built-in choice.
                          Same results either way                         */
    int drm_inline;    /* FP32 form: 0 = the next step's DRM forces run on a
                          second stream beside the step kernel, into the
                          other of two force slots (default; a context
                          stepping alone: 4-20% less time per step on the
                          canyons and valleys of 1-16 RHS); 1 = inside the
                          hanging/receiver pass (the server's default: with
                          many requests stepping at once their kernels hide
                          that pass anyway, and the second streams measured
                          3% slower on a saturated burst).  Same results   */
    int serial_launch; /* FP32 form: 0 = the direct gather's step kernel is
                          launched as a programmatic dependent of the
                          hanging/receiver pass before it (its blocks start
                          while that pass runs, load the node records no
                          kernel writes, then wait for it; default); 1 = it
                          launches once that pass has finished.  Same
                          results                                         */
} exfem_opts;

typedef struct exfem_ctx exfem_ctx;

/* Fill *opts with defaults (FP64, device 0, graphs on, reorder on). */
void exfem_gpu_default_opts(exfem_opts *opts);

/* Build a device-resident model.  Replaces the state set up by init_model()
 * for the solver (explicit.f90:16-70) — the host passes what it computed.
 * Validates the mesh (elemallnhnodes' four non-hanging corners,
 * model.f90:166-171), precomputes the per-node lumped mass/damping
 * coefficients, the node-to-element gather lists and the DRM slots.
 * Returns EXFEM_E_UNSUPPORTED for grazing/post-critical waves, where the
 * reference would exit(1) (pwaves.f90:32-35, 87-89). */
int exfem_gpu_create(const exfem_mesh *mesh, const exfem_problem *prob,
                     const exfem_opts *opts, exfem_ctx **out);

/* init_explicit() (explicit.f90:79-109): zero state, assemble
 * m_full = sum_e(a2*c_e + a1*m_e) with the hanging-anchor reduction.
 * If mfull_out is non-NULL it receives m_full in the reference's dof order
 * (2*nnodes doubles, the content of mass.bin, io.cpp:409-429). */
int exfem_gpu_init_explicit(exfem_ctx *ctx, double *mfull_out);

/* run_explicit() (explicit.f90:111-159) for nsteps more steps (may be called
 * repeatedly; the total may not exceed the problem's nsteps).  Receivers are
 * sampled after every step with step % io_interval == 0 (save_step,
 * io_utils.f90:390).  Asynchronous: returns after queueing the work. */
int exfem_gpu_run(exfem_ctx *ctx, int nsteps);

/* Non-blocking: 0 when every queued step has finished, 1 while work is still
 * running, or a negative code (EXFEM_E_NAN when the watchdog tripped). */
int exfem_gpu_query(exfem_ctx *ctx);

/* Wait for queued work; returns EXFEM_E_NAN if the watchdog tripped. */
int exfem_gpu_sync(exfem_ctx *ctx);

/* Current displacement e_u of right-hand side `rhs` (0-based) in the
 * reference's dof order (2*nnodes doubles), as save_step would write it. */
int exfem_gpu_get_u(exfem_ctx *ctx, int rhs, double *u, size_t n);

/* Receiver traces: out[rhs][save][recv][2] (x, depth components), the FIELD
 * rows of sheet.txt (visualization.f90:307-354, io.cpp:862-876) including the
 * free field outside the DRM box (visu_field, visualization.f90:156-181).
 * *nsaved receives the number of stored samples per receiver. */
int exfem_gpu_get_seismograms(exfem_ctx *ctx, double *out, size_t cap, int *nsaved);

/* Displacement of right-hand side `rhs` at npoint arbitrary points for the
 * current step, as visu_field (visualization.f90:156-181) samples the ANIMAT
 * grid (visualize_solution, visualization.f90:192-284) from each step.bin:
 * out[2*i], out[2*i+1] = (x, depth) at (xy[2*i], xy[2*i+1]) inside the
 * 1-based element elem[i] (calcfieldat, formulation.f90:315-325), plus the
 * free field at time steps_done * dt outside the DRM box.  elem[i] = 0 (no
 * element holds the point) gives 0, as share_field fills unfound points
 * (communicator.f90:1580-1584).  Waits for the context's queued steps;
 * allocates device scratch for the points. */
int exfem_gpu_sample_points(exfem_ctx *ctx, int rhs, int npoint, const double *xy, const int *elem, double *out);

/* exfem_gpu_run() bracketed by CUDA events recorded on the context's own
 * stream; waits for completion and returns the device time in *ms.  A
 * measurement helper with no counterpart in the reference. */
int exfem_gpu_run_timed(exfem_ctx *ctx, int nsteps, double *ms);

/* Runs nsteps without graph capture, timing every launch with CUDA events on
 * the context's stream.  ms_out[k] receives the average duration of kernel
 * k, names_out[k] its name; returns the number of distinct kernels (at most
 * cap).  A measurement helper with no counterpart in the reference. */
int exfem_gpu_profile_kernels(exfem_ctx *ctx, int nsteps, double *ms_out, const char **names_out, int cap);

/* Size of the static scratch array behind exfem_gpu_step_noalloc, in
 * doubles (8 MiB; held by every device that loads the library). */
#define EXFEM_NOALLOC_SCRATCH_DOUBLES 1048576

/* One FP64 time step on buffers the caller owns, with no device allocation.
 * No counterpart in the reference.
 *
 * For hosts that keep the displacement state in device memory they manage
 * themselves and cannot let a library allocate: a host whose own pool or
 * arena hands out every device byte up front (a cudaMalloc from the library
 * would fall outside its budget, or fail once the arena holds the memory),
 * or a host with other work in flight on the device, which cudaFree would
 * stall, since cudaFree synchronizes the whole device.
 *
 * d_u, d_um: device arrays of u_i and u_{i-1}; d_unew receives u_{i+1}
 * (2*nnodes*nrhs doubles each, in the context's internal node order, the
 * layout exfem_gpu_run keeps; d_unew may alias d_um, the two-array rotation
 * of e_u/e_up).  `step` is the time index i+1 whose forcing is applied
 * (t = step*dt, explicit.f90:128).  The context must be EXFEM_FP64 with
 * variant EXFEM_VARIANT_REFERENCE_ORDER (EXFEM_E_ARG otherwise).
 *
 * Receivers are not sampled, so the NaN watchdog of exfem_gpu_run does not
 * run either: a diverging loop gets no EXFEM_E_NAN from this entry point.
 *
 * The element and DRM forces go through one static scratch array shared by
 * every call; the model must fit
 *   32 + 4*ceil(16*nseismic*nrhs / 4) + 8*nelems*nrhs
 *     <= EXFEM_NOALLOC_SCRATCH_DOUBLES
 * (EXFEM_E_ARG with a message otherwise).  The array keeps the last call's
 * contents; each call resets the counters it reads.  Calls that overlap on
 * the GPU (two contexts, two streams) race on it.  The first call on a
 * device looks up the array's device address with that device current.
 *
 * stream: the cudaStream_t the five launches are queued on, so they are
 * ordered after the caller's own writes of d_u/d_um and before its reads of
 * d_unew.  NULL queues them on the context's own stream, a non-blocking one
 * that does not wait for the legacy default stream (exfem_gpu_sync() waits
 * for it); a caller on the legacy default stream passes cudaStreamLegacy.
 * The caller's current device is the same on return as on entry. */
int exfem_gpu_step_noalloc(exfem_ctx *ctx, int step, const double *d_u, const double *d_um, double *d_unew,
                           void *stream);

/* Autotuner of the FP32 form (opts->precision must be EXFEM_FP32_KAHAN).
 * Times every candidate shape on this mesh and problem and writes the
 * fastest into opts: variant (0 direct gather, 4 the same as a persistent
 * grid, 1 shared-memory tiles, 2 bulk-copy pipeline when the right-hand sides
 * are a multiple of 4, 3 tensor-core step when they are a multiple of 16),
 * block_threads (128, 256, 512) and rhs_per_thread (1, 2, 4).  Each
 * candidate runs in a context of its own (one at a time: the device must
 * hold one more context of this problem), 3 warm-up steps and `steps` steps
 * timed with CUDA events (1 <= steps <= 1000); *ms_per_step (nullable)
 * receives the winner's time.  Results are cached in the process per
 * (elements, nodes, right-hand sides, device).  No counterpart in the
 * reference, whose element loop has one shape (explicit.f90:129-142). */
int exfem_gpu_autotune(const exfem_mesh *mesh, const exfem_problem *prob, exfem_opts *opts, int steps,
                       double *ms_per_step);

/* Steps taken so far. */
int exfem_gpu_steps_done(const exfem_ctx *ctx);

/* Number of kernel launches the library queued so far (its own kernels). */
long long exfem_gpu_launch_count(const exfem_ctx *ctx);

/* Bytes of device memory held by the context. */
size_t exfem_gpu_device_bytes(const exfem_ctx *ctx);

/* Contexts take their device memory from a stream-ordered pool per device
 * that keeps what destroyed contexts freed, so later contexts (a server's
 * next requests) reuse it without cudaMalloc/cudaFree.  This returns the
 * pool's unused memory on `device` to the driver (memory of live contexts
 * stays). */
int exfem_gpu_release_cached(int device);

/* Bytes the context has copied host -> device (the model's arrays at create,
 * sample points) and device -> host (seismograms, fields, status flags) so
 * far.  Either pointer may be NULL. */
int exfem_gpu_copy_bytes(const exfem_ctx *ctx, unsigned long long *h2d, unsigned long long *d2h);

/* Estimated device bytes a context for this mesh/problem/opts would hold
 * (used for admission by HBM footprint).  No device work. */
size_t exfem_gpu_estimate_bytes(const exfem_mesh *mesh, const exfem_problem *prob,
                                const exfem_opts *opts);

/* Last error message of the context (or of the last failed create when ctx is NULL). */
const char *exfem_gpu_last_error(const exfem_ctx *ctx);

void exfem_gpu_destroy(exfem_ctx *ctx);

#ifdef __cplusplus
}
#endif
#endif /* EXFEM_GPU_H */
