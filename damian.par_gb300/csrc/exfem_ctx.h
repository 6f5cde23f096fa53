// exfem_ctx.h — device context shared by the FP64 and FP32 kernel files.
#pragma once

#include <cuda_runtime.h>

#include <string>
#include <utility>
#include <vector>

#include "exfem_gpu.h"
#include "exfem_plan.h"

namespace exfem {

// Plane-wave constants as the kernels read them (pwaves.f90 module state).
struct DevWave {
    int kind;
    double alpha, beta, fp;
    double sine, cose, sinf, cosf;
    double amp0, wa1, wb1;
    double wui[6];
    double t0;
    double inv_alpha, inv_beta;   // 1/vp, 1/vs (FP32 free field only)
};

// Device arrays common to both arithmetic forms.
struct DevModel {
    int nn, ne, R, n_active, n_hang, ns, nrecv, nsave, io;
    int lg;                  // RHS group of the state layout (row_off): R, or the FP32 RHS per thread
    double dt, a1, a2, a3;
    double worigin_x, worigin_y;
    const int *econn;        // 4 per element
    const double *ecoef;     // 4 per element (FP64)
    const float *ecoef32;    // 4 per element (FP32), derived from ecoef2 (fp32_coef)
    const float *ecoef2;     // 2 per element: lam/12, mu/4 (FP32)
    const double *ekv;       // 6 per element: calck_values(mu, lambda)
    const double *emass;     // per element
    const int *edamp;        // per element, -1 or slot
    const double *edampv;    // 8 per slot
    const double *nxy;       // 2 per node (internal)
    const int *tptr, *tlist; // gather lists (active nodes)
    const int *dptr, *dlist; // DRM gather lists (active nodes)
    const double *inv_mfull; // 2 per active node
    const double *mfull;     // 2 per active node (m_full, divided by)
    const int *hang;         // 3 per hanging entry
    const int *s_elem, *s_kind;
    const int *rnode;        // 4 per receiver (corners; hanging ones read as anchor averages)
    const double *rw;        // 4 per receiver (shape-function weights)
    const int *rsoil;
    const double *rxy;       // 2 per receiver
    const DevWave *waves;    // R
    const int *ownptr, *ownlist;   // own element incidences, all nodes, element order
    const int *odptr, *odlist;     // own DRM incidences, all nodes, seismic order
    const int *lptr, *llist;       // anchor links (h, other anchor), m_hanging order
    // FP32 increment form
    const float *ncoef4;           // per active node: 1/m_full (x, y), -2 a2 C (x, y)
    const float *hcoef4;           // per hanging entry: -2 a2 C (x, y), a1 M + a2 C (x, y)
    float *fdrm32;                 // ns * 8 * R DRM forces (FP64 math, stored FP32)
    const int *tcorn;              // 4 per gather term: the corners of its element
    // the direct gather's fixed-size node records (build_node_slots; null in
    // the list form): 4 term entries and 1/m_full (negative: marked) per
    // active node, and with term corners 4 x 4 corners per active node
    const int *tslot4;
    const float *ninvm;
    const int *tcorn4;
    const double *drm_delay;       // ((s*4 + corner)*3 + term)*R + r: the DRM corners' free-field delays
    // point source (EXFEM_POINT_*; 0 = none)
    int point_kind, npoint;
    double point_amp, point_sigma, point_t0;
    const unsigned char *pflag;    // per internal node: 1 on a source node (or null)
    const int *pnodes;             // the source nodes (internal ids)
    // mutable state
    double *fdrm;            // ns * 16 * R DRM forces (stiffness part, mass part)
    double *seis;            // R * nsave * nrecv * 2
    int *d_step;             // steps completed (device counter)
    unsigned *d_blocks;      // last-block counter
    int *d_flag;             // watchdog flags
    int *d_drm_step;         // FP32 side-stream DRM: the last step whose forces are computed
    unsigned *d_drm_blocks;  // its last-block counter
};

struct Ctx {
    Plan plan;
    exfem_opts opts;
    int device = 0;
    int precision = EXFEM_FP64;
    cudaStream_t stream = nullptr;
    DevModel dm{};
    std::vector<void *> allocs;
    size_t bytes = 0;
    // bytes copied host -> device and device -> host so far
    unsigned long long h2d_bytes = 0, d2h_bytes = 0;
    // FP64 state: u[2] ping-pong + element forces
    double *u64[2] = {nullptr, nullptr};
    double *ef64 = nullptr;
    // FP32 state: u_hi[2] ping-pong and the increment D in FP32, each with a
    // bf16 Kahan compensation (stored as raw 16-bit words)
    float *uhi[2] = {nullptr, nullptr};
    unsigned short *ucomp = nullptr;
    float *udel[2] = {nullptr, nullptr};
    unsigned short *dcomp = nullptr;
    // shared-memory tiles of the FP32 step (see build_tiles)
    bool use_tiles = false;
    int tile_tn = 0, tile_n = 0, tile_hmax = 0, tile_rc = 0;
    size_t tile_smem = 0;
    const int *t_hptr = nullptr, *t_hlist = nullptr, *t_nslot = nullptr, *t_lslot = nullptr;
    const unsigned short *t_tslot = nullptr;
    // point source in the FP32 form: the active nodes it acts on and their
    // weights (1 on a source node, 1/2 per hanging source node anchored)
    const int *p32_node = nullptr;
    const float *p32_w = nullptr;
    int p32_n = 0;
    // bulk-copy pipeline of the FP32 step (variant 2): per-tile headers and
    // halo runs, node records, term records; persistent grid
    // tensor-core step of the FP32 form (variant 3): element tiles and the
    // split [Kmu; Klambda] operand
    bool use_mma = false;
    int mma_ntiles = 0;
    const int *mma_nptr = nullptr, *mma_eptr = nullptr, *mma_elist = nullptr;
    const unsigned char *mma_tj = nullptr;
    const float *mma_btile = nullptr;
    bool use_pipe = false;
    const void *p_hdr = nullptr, *p_runs = nullptr, *p_nrec = nullptr, *p_tpack = nullptr;
    int pipe_grid = 0, pipe_threads = 0, pipe_nstage = 0;
    unsigned pipe_stage = 0;
    unsigned pipe_off[6] = {0, 0, 0, 0, 0, 0};   // D, D_comp, u_comp, node records, slots, coefficients
    // The next step's DRM forces on a second stream (k_drm32 in the FP32
    // form, k_drm_ref_side in the reference-order FP64 form) while this step
    // runs, into the other of two force slots (see side_drm_next)
    bool drm_side = false;
    cudaStream_t side = nullptr;
    cudaEvent_t ev_step = nullptr, ev_fork = nullptr, ev_drm[2] = {nullptr, nullptr};
    // the events used while a graph is captured (an event last recorded in a
    // capture cannot be waited on outside it)
    cudaEvent_t cev_step = nullptr, cev_drm[2] = {nullptr, nullptr};
    float *fdrm_slot[2] = {nullptr, nullptr};
    double *fdrm64_slot[2] = {nullptr, nullptr};
    bool drm_wait[2] = {false, false};   // a k_drm32 into slot s that the main stream has not waited for
    bool ev_step_valid = false;          // ev_step marks the previous step's k_step32
    int parity = 0;          // index of the current u buffer
    int steps_done = 0;
    bool inited = false;
    long long launches = 0;
    cudaGraphExec_t graph = nullptr;
    int graph_steps = 0;
    int graph_parity = -1;
    int block_threads = 128;
    int persist_grid = 0;    // FP32 variant 4: blocks of the persistent step grid (0 until the first launch)
    int rhs_per_thread = 1;
    bool idx32 = true;   // k_step32 with 32-bit indices (every index below 2^32)
    int num_sms = 1;     // SMs of the context's device
    std::string err;
    // per-launch event marks while exfem_gpu_profile_kernels runs
    bool prof_on = false;
    std::vector<std::pair<const char *, cudaEvent_t>> marks;
};

// Work items per block for the free-field kernels (DRM forces, receivers).
// Their cost is FP64 arithmetic (travel times, Ricker pulses), and an SM's
// FP64 pipe is narrow: the same lanes spread over every SM, a few per SM,
// finish sooner than full warps packed on a few SMs.  At most `cap` items per
// block (the block's threads / lanes per item).
inline int spread_per_block(long long items, int nsm, int cap) {
    const long long per = (items + (nsm > 0 ? nsm : 1) - 1) / (nsm > 0 ? nsm : 1);
    return (int)(per < 1 ? 1 : (per > cap ? cap : per));
}
inline int spread_blocks(long long items, int per_block) {
    const long long b = (items + per_block - 1) / per_block;
    return (int)(b < 1 ? 1 : b);
}

// FP32 direct gather: whether each term carries a copy of its element's
// corners (16 B per term, one load less in the gather chain).  With few RHS
// the copy is most of a node's traffic and the corners come from econn:
// measured 12% faster with one RHS and, with a node's rows paired, 12% at
// four (0.55M-element valley); the copy is 1-2% faster from six.
constexpr bool f32_term_corners(int R) { return R > 4; }
// The same choice for the fixed-size node records (4 x 16 B per node in
// tcorn4).  With the records the chain without copies is slot record ->
// econn -> corner rows, one level longer, but the copies are most of a
// node's metadata.  Measured: copies 10-27% slower up to four RHS (the
// 1.5M-element valley at one, 0.52M- and 0.86M-element requests at two);
// econn 2-5% faster on the 6-, 8- and 12-RHS requests of the saturated burst
// and the 6-RHS canyon (0.6% less for the burst's requests alone, 0.5% on
// its makespan), and the copies 0.4-1.5% faster at 16.
constexpr bool f32_slot_corners(int R) { return R > 12; }

// FP32 direct gather: active nodes from which the fixed-size node records
// (build_node_slots) replace the list form.  A marked node's path is longer
// with them (its slot terms, then its lists), and a mesh this small runs in
// one partial wave of blocks, so its step lasts as long as its slowest warp:
// measured 5-8% slower with the records on 34K- and 36K-element requests,
// the same at 55K-74K, and 3-11% faster from 0.13M elements (the 1.5M-element
// valley: 7% at one RHS, 4% at 64).
constexpr int kSlotMinNodes = 50000;

// FP32 direct gather with several threads per node: whether the state is laid
// out in groups of one thread's right-hand sides (row_off), so that a thread's
// x and y values of a node are adjacent and move as one vector.  Measured 9 to
// 12% faster per step from 6 to 16 RHS on a 0.55M-element valley and on the
// served requests; no gain at 64.
constexpr bool f32_interleave(int R) { return R < 64; }

// FP32 form: right-hand-side counts up to which the next step's DRM forces
// run on a second stream beside the step (k_drm32) instead of inside the
// hanging/receiver pass, where the latency of their FP64 chains holds up every
// step of a mesh too small to hide it.
constexpr int kDrmSideMaxRhs = 64;

// Device memory of a context: a stream-ordered allocation on its stream from
// the library's memory pool for the device, which keeps what destroyed
// contexts freed for the next ones (no cudaMalloc, and no cudaFree, which
// waits for the whole device, once the pool has grown; see
// exfem_gpu_release_cached).  ctx_alloc records the block for free_all and
// counts it in the context's bytes; scratch_alloc does neither (free it with
// cudaFreeAsync on the context's stream).
cudaError_t ctx_alloc(Ctx &c, void **p, size_t bytes);
cudaError_t scratch_alloc(Ctx &c, void **p, size_t bytes);
int release_cached(int device);

// Records a profiling mark after a launch (no-op unless profiling).
void mark(Ctx &c, const char *kernel);

// Launchers of the reference-order FP64 file.
int f64ref_launch_drm_elem_node(Ctx &c, int par);
int f64_launch_hang(Ctx &c, double *unew, int mode);

// Launchers implemented by the FP32 file.
int f32_alloc(Ctx &c);
int f32_init(Ctx &c);
int f32_tune_in_place(Ctx &c);
int f32_launch_step(Ctx &c, int par);
int f32_launch_sample0(Ctx &c, int par);
// Side-stream DRM forces, shared by both forms.  side_create makes the
// stream and events.  side_drm_next, before step k's kernels (at parity
// `par`): makes the main stream wait for step k's forces (slot par) if a
// side launch made them, then queues `launch(stream)` for step k + 1's forces
// into slot par ^ 1 on the side stream, after step k - 1's reader of that
// slot (the main stream under exfem_gpu_profile_kernels, which times each
// launch alone).  side_mark, after the last kernel of step k that reads its
// slot.  side_join makes the main stream wait for any side launch it has not
// waited for (before a sync point, a graph replay or the end of a capture).
int side_create(Ctx &c);
template <class F>
int side_drm_next(Ctx &c, int par, F &&launch) {
    if (c.drm_wait[par]) {
        if (cudaStreamWaitEvent(c.stream, c.ev_drm[par], 0) != cudaSuccess) return EXFEM_E_CUDA;
        c.drm_wait[par] = false;
    }
    if (c.prof_on) {
        launch(c.stream);
        return EXFEM_OK;
    }
    if (c.ev_step_valid && cudaStreamWaitEvent(c.side, c.ev_step, 0) != cudaSuccess) return EXFEM_E_CUDA;
    launch(c.side);
    if (cudaEventRecord(c.ev_drm[par ^ 1], c.side) != cudaSuccess) return EXFEM_E_CUDA;
    c.drm_wait[par ^ 1] = true;
    return EXFEM_OK;
}
int side_mark(Ctx &c);
int side_join(Ctx &c);

// Launches kernel k on the context's stream as a programmatic dependent of
// the kernel before it (its blocks may start while that one drains and wait
// in pdl_wait), unless exfem_opts.serial_launch is set or the launches are
// being timed one by one.
template <typename... KArgs, typename... Args>
cudaError_t launch_dep(Ctx &c, void (*k)(KArgs...), unsigned grid, unsigned block, Args &&...args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(block);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = c.stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    const bool dep = c.opts.serial_launch == 0 && !c.prof_on;
    cfg.attrs = dep ? attr : nullptr;
    cfg.numAttrs = dep ? 1 : 0;
    return cudaLaunchKernelEx(&cfg, k, std::forward<Args>(args)...);
}
// bf16 <-> float on the host (round to nearest even), for tests and read-back.
float bf16_to_float(unsigned short h);

}  // namespace exfem

// The opaque handle of include/exfem_gpu.h.
struct exfem_ctx : exfem::Ctx {};
