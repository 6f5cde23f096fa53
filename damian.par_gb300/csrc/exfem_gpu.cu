// exfem_gpu.cu — C ABI (include/exfem_gpu.h) and the FP64 step kernels.
//
// One time step of run_explicit (explicit.f90:125-153) is four kernels:
//   k_drm       DRM effective forces of the boundary layer at t = (i)*dt
//               (additive_reactions -> wave_reactions, model.f90:745-800)
//   k_elem64    per-element localr = (a3 u - a1 u-)*m + a2 c*u- - K u
//               (explicit.f90:130-140) into an element-force buffer
//   k_node64    per non-hanging node: gather its element and DRM terms (terms
//               of a hanging node it anchors at weight 1/2: sum_reactanchors
//               in halving form), u+ = r / m_full (explicit.f90:143-148);
//               the gather replaces the element scatter and the MPI sums, so
//               no atomics are needed
//   k_hang      u_h = (u_a + u_b)/2 (set_dispshanging, model.f90:612-624) and
//               the in-loop receiver samples (visu_field) on save steps
// The step counter lives on the device so a captured CUDA graph of several
// steps can be replayed unchanged.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <mutex>
#include <new>
#include <string>
#include <vector>

#include "exfem_ctx.h"
#include "exfem_device.cuh"
#include "exfem_gpu.h"
#include "exfem_plan.h"

using namespace exfem;

namespace {

thread_local std::string g_create_err;

#define CK(call)                                                                              \
    do {                                                                                      \
        cudaError_t e_ = (call);                                                              \
        if (e_ != cudaSuccess) {                                                              \
            c.err = std::string(#call) + ": " + cudaGetErrorString(e_);                       \
            return EXFEM_E_CUDA;                                                              \
        }                                                                                     \
    } while (0)

__device__ __forceinline__ int read_step(const DevModel &m) { return *(volatile int *)m.d_step; }

// ---------------------------------------------------------------- DRM ----
// Free field at a boundary element's four corners, then multdrm for K and for
// the consistent mass (model.f90:766-798), in closed form.  Four threads per
// (boundary element, rhs): thread k evaluates the free field at corner k, the
// quad shares the values by shuffles, thread k stores forces 2k and 2k+1
// (launch: `ipb` items per block of 4 * ipb or more threads, a multiple of 32).
__global__ void k_drm(DevModel m, int ipb) {
    const int li = threadIdx.x >> 2;
    const long long w = (long long)blockIdx.x * ipb + li;
    const int k = (int)(threadIdx.x & 3);
    const bool valid = li < ipb && w < (long long)m.ns * m.R;
    int s = 0, r = 0, ie = 0;
    double ukx = 0.0, ukz = 0.0, akx = 0.0, akz = 0.0;
    if (valid) {
        s = (int)(w / m.R);
        r = (int)(w % m.R);
        int step = read_step(m) + 1;
        const DevWave wv = m.waves[r];
        double outt = (double)step * m.dt - wv.t0;   // timetransform(m_wttoorigin, i*dt)
        ie = m.s_elem[s];
        int x = m.econn[4 * ie + k];
        double ox = m.nxy[2 * x] - m.worigin_x, oz = m.nxy[2 * x + 1] - m.worigin_y;
        double ux[3], uz[3];
        planewave(wv, outt, ox, oz, ux, uz);
        ukx = ux[0]; ukz = uz[0];
        akx = ux[2]; akz = uz[2];
    }
    double u0[8], a0[8];
#pragma unroll
    for (int c = 0; c < 4; ++c) {
        u0[2 * c] = __shfl_sync(0xffffffffu, ukx, c, 4);
        u0[2 * c + 1] = __shfl_sync(0xffffffffu, ukz, c, 4);
        a0[2 * c] = __shfl_sync(0xffffffffu, akx, c, 4);
        a0[2 * c + 1] = __shfl_sync(0xffffffffu, akz, c, 4);
    }
    if (!valid) return;
    double kc[4] = {m.ecoef[4 * ie], m.ecoef[4 * ie + 1], m.ecoef[4 * ie + 2], m.ecoef[4 * ie + 3]};
    double p[8];
    drm_forces<double>(kc, m.emass[ie], drm_mask(m.s_kind[s]), u0, a0, p);
    m.fdrm[((size_t)s * 16 + 2 * k) * m.R + r] = p[2 * k];
    m.fdrm[((size_t)s * 16 + 2 * k + 1) * m.R + r] = p[2 * k + 1];
}

// ----------------------------------------------------------- elements ----
__global__ void __launch_bounds__(256) k_elem64(DevModel m, const double *__restrict__ u,
                                                const double *__restrict__ um, double *__restrict__ ef) {
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)m.ne * m.R) return;
    int e = (int)(t / m.R), r = (int)(t % m.R);
    const int4 c = reinterpret_cast<const int4 *>(m.econn)[e];
    const int cn[4] = {c.x, c.y, c.z, c.w};
    double ux[4], uy[4], vx[4], vy[4];
    if (m.R == 1) {
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            double2 a = reinterpret_cast<const double2 *>(u)[cn[k]];
            double2 b = reinterpret_cast<const double2 *>(um)[cn[k]];
            ux[k] = a.x; uy[k] = a.y; vx[k] = b.x; vy[k] = b.y;
        }
    } else {
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            size_t ix = ((size_t)cn[k] * 2) * m.R + r, iy = ix + m.R;
            ux[k] = u[ix]; uy[k] = u[iy]; vx[k] = um[ix]; vy[k] = um[iy];
        }
    }
    const double4 kc = reinterpret_cast<const double4 *>(m.ecoef)[e];
    double fx[4], fy[4];
    q4_ku<double>(kc.x, kc.y, kc.z, kc.w, ux, uy, fx, fy);
    double mass = m.emass[e];
    int ds = m.edamp[e];
    double lr[8];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        lr[2 * k] = (m.a3 * ux[k] - m.a1 * vx[k]) * mass;
        lr[2 * k + 1] = (m.a3 * uy[k] - m.a1 * vy[k]) * mass;
    }
    if (ds >= 0) {
        const double *dv = m.edampv + (size_t)ds * 8;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            lr[2 * k] = lr[2 * k] + m.a2 * dv[2 * k] * vx[k];
            lr[2 * k + 1] = lr[2 * k + 1] + m.a2 * dv[2 * k + 1] * vy[k];
        }
    }
#pragma unroll
    for (int k = 0; k < 4; ++k) { lr[2 * k] -= fx[k]; lr[2 * k + 1] -= fy[k]; }
    if (m.R == 1) {
        double4 *o = reinterpret_cast<double4 *>(ef + (size_t)e * 8);
        o[0] = make_double4(lr[0], lr[1], lr[2], lr[3]);
        o[1] = make_double4(lr[4], lr[5], lr[6], lr[7]);
    } else {
#pragma unroll
        for (int k = 0; k < 8; ++k) ef[((size_t)e * 8 + k) * m.R + r] = lr[k];
    }
}

// --------------------------------------------------------------- nodes ----
// Point force on the y dof (absolute_reactions, explicit.f90:144): the node's
// own, and half of each hanging source node it anchors (sum_reactanchors).
__device__ __forceinline__ void point_terms(const DevModel &m, int n, double &rx, double &ry) {
    (void)rx;
    if (m.point_kind != EXFEM_POINT_FORCE) return;
    const int step = read_step(m) + 1;
    if (m.pflag[n]) ry += point_value(m, step);
    for (int q = m.lptr[n]; q < m.lptr[n + 1]; ++q)
        if (m.pflag[m.llist[2 * q]]) ry += 0.5 * point_value(m, step);
}

__global__ void __launch_bounds__(256) k_node64(DevModel m, const double *__restrict__ ef,
                                                double *__restrict__ unew) {
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)m.n_active * m.R) return;
    int n = (int)(t / m.R), r = (int)(t % m.R);
    double rx = 0.0, ry = 0.0;
    for (int q = m.dptr[n]; q < m.dptr[n + 1]; ++q) {
        int ent = m.dlist[q];
        double w = (ent & 1) ? 0.5 : 1.0;
        int sc = ent >> 1;
        size_t base = ((size_t)(sc >> 2) * 16 + 2 * (sc & 3)) * m.R + r;
        rx += w * m.fdrm[base];
        ry += w * m.fdrm[base + m.R];
    }
    const int q0 = m.tptr[n], q1 = m.tptr[n + 1];
    if (m.R == 1) {
        for (int q = q0; q < q1; ++q) {
            int ent = __ldg(m.tlist + q);
            double w = (ent & 1) ? 0.5 : 1.0;
            int ec = ent >> 1;
            double2 v = reinterpret_cast<const double2 *>(ef)[(size_t)(ec >> 2) * 4 + (ec & 3)];
            rx += w * v.x;
            ry += w * v.y;
        }
        point_terms(m, n, rx, ry);
        double2 im = reinterpret_cast<const double2 *>(m.inv_mfull)[n];
        double uy = ry * im.y;
        if (m.point_kind == EXFEM_POINT_DISP && m.pflag[n]) uy = point_value(m, read_step(m) + 1);
        reinterpret_cast<double2 *>(unew)[n] = make_double2(rx * im.x, uy);
    } else {
        for (int q = q0; q < q1; ++q) {
            int ent = __ldg(m.tlist + q);
            double w = (ent & 1) ? 0.5 : 1.0;
            int ec = ent >> 1;
            size_t base = ((size_t)(ec >> 2) * 8 + 2 * (ec & 3)) * m.R + r;
            rx += w * ef[base];
            ry += w * ef[base + m.R];
        }
        point_terms(m, n, rx, ry);
        double uy = ry * m.inv_mfull[2 * n + 1];
        if (m.point_kind == EXFEM_POINT_DISP && m.pflag[n]) uy = point_value(m, read_step(m) + 1);
        unew[((size_t)n * 2) * m.R + r] = rx * m.inv_mfull[2 * n];
        unew[((size_t)n * 2 + 1) * m.R + r] = uy;
    }
}

inline int nblocks(long long work, int threads) { return (int)std::max<long long>(1, (work + threads - 1) / threads); }

// A prescribed point displacement v on the y dof of every source node.
__global__ void k_point_set64(DevModel m, double *u, double v) {
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)m.npoint * m.R) return;
    const int n = m.pnodes[t / m.R], r = (int)(t % m.R);
    u[((size_t)n * 2 + 1) * m.R + r] = v;
}

// visu_field at arbitrary points: FP64 rows (u64) or FP32 hi - comp (uh, uc).
__global__ void k_sample_points(DevModel m, const double *__restrict__ u64, const float *__restrict__ uh,
                                const unsigned short *__restrict__ uc, int rhs, int np, const int *__restrict__ node,
                                const double *__restrict__ w, const int *__restrict__ soil,
                                const double *__restrict__ xy, double time, double *__restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= np) return;
    double fx = 0.0, fy = 0.0;
    if (node[4 * (size_t)i] >= 0) {
        for (int k = 0; k < 4; ++k) {
            const size_t bx = state_at(m, (size_t)node[4 * (size_t)i + k], 0, rhs);
            const size_t by = state_at(m, (size_t)node[4 * (size_t)i + k], 1, rhs);
            double vx, vy;
            if (u64) {
                vx = u64[bx];
                vy = u64[by];
            } else {
                vx = (double)uh[bx] - (double)__bfloat162float(__ushort_as_bfloat16(uc[bx]));
                vy = (double)uh[by] - (double)__bfloat162float(__ushort_as_bfloat16(uc[by]));
            }
            const double wk = w[4 * (size_t)i + k];
            fx = fx + wk * vx;
            fy = fy + wk * vy;
        }
        if (soil[i]) {
            const DevWave wv = m.waves[rhs];
            double dx, dz;
            planewave_u(wv, time - wv.t0, xy[2 * (size_t)i] - m.worigin_x, xy[2 * (size_t)i + 1] - m.worigin_y, dx, dz);
            fx = fx + dx;
            fy = fy + dz;
        }
    }
    out[2 * (size_t)i] = fx;
    out[2 * (size_t)i + 1] = fy;
}

// One right-hand side of the state in internal dof order (2 per node): the
// FP64 value, or u_hi - u_comp in FP64 for the FP32 form.
__global__ void k_extract_rhs(DevModel m, const double *__restrict__ u64, const float *__restrict__ uh,
                              const unsigned short *__restrict__ uc, int rhs, long long ndof,
                              double *__restrict__ out) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= ndof) return;
    const size_t k = state_at(m, (size_t)(i >> 1), (int)(i & 1), rhs);
    out[i] = u64 ? u64[k] : (double)uh[k] - (double)__bfloat162float(__ushort_as_bfloat16(uc[k]));
}

int launch_step64(Ctx &c, int par) {
    DevModel &m = c.dm;
    double *u = c.u64[par], *um = c.u64[par ^ 1];
    if (c.opts.variant == EXFEM_VARIANT_REFERENCE_ORDER) {
        if (f64ref_launch_drm_elem_node(c, par)) { c.err = cudaGetErrorString(cudaGetLastError()); return EXFEM_E_CUDA; }
    } else {
        const int T = c.block_threads;
        if (m.ns > 0) {
            const long long W = (long long)m.ns * m.R;
            const int ipb = spread_per_block(W, c.num_sms, 32);
            k_drm<<<spread_blocks(W, ipb), 128, 0, c.stream>>>(m, ipb);
            c.launches++;
            mark(c, "k_drm");
        }
        k_elem64<<<nblocks((long long)m.ne * m.R, T), T, 0, c.stream>>>(m, u, um, c.ef64);
        mark(c, "k_elem64");
        k_node64<<<nblocks((long long)m.n_active * m.R, T), T, 0, c.stream>>>(m, c.ef64, um);
        mark(c, "k_node64");
        c.launches += 2;
        CK(cudaGetLastError());
    }
    if (f64_launch_hang(c, um, 0)) { c.err = cudaGetErrorString(cudaGetLastError()); return EXFEM_E_CUDA; }
    return EXFEM_OK;
}

int launch_sample0_64(Ctx &c, int par) {
    c.drm_wait[0] = c.drm_wait[1] = false;   // step 1's forces come from this launch, into slot 0
    c.ev_step_valid = false;
    if (f64_launch_hang(c, c.u64[par], 1)) { c.err = cudaGetErrorString(cudaGetLastError()); return EXFEM_E_CUDA; }
    return EXFEM_OK;
}

template <typename T, typename A>
int upload(Ctx &c, const std::vector<T, A> &v, const T **dst) {
    if (v.empty()) { *dst = nullptr; return EXFEM_OK; }
    void *p = nullptr;
    CK(ctx_alloc(c, &p, v.size() * sizeof(T)));
    CK(cudaMemcpyAsync(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, c.stream));
    c.h2d_bytes += v.size() * sizeof(T);
    *dst = static_cast<const T *>(p);
    return EXFEM_OK;
}

template <typename T>
int dalloc(Ctx &c, size_t n, T **dst) {
    void *p = nullptr;
    if (n == 0) n = 1;
    CK(ctx_alloc(c, &p, n * sizeof(T)));
    *dst = static_cast<T *>(p);
    return EXFEM_OK;
}

#define TRY(x)                   \
    do {                         \
        int rc_ = (x);           \
        if (rc_) return rc_;     \
    } while (0)

int setup_device(Ctx &c) {
    Plan &P = c.plan;
    DevModel &m = c.dm;
    m.nn = P.nn; m.ne = P.ne; m.R = P.R; m.n_active = P.n_active; m.n_hang = P.n_hang;
    m.lg = P.R;   // plain layout; the FP32 direct gather may group it (f32_alloc)
    m.ns = (int)P.s_elem.size(); m.nrecv = P.nrecv; m.nsave = P.nsave; m.io = P.io;
    m.dt = P.dt; m.a1 = P.a1; m.a2 = P.a2; m.a3 = P.a3;
    m.worigin_x = P.worigin[0]; m.worigin_y = P.worigin[1];
    TRY(upload(c, P.econn, &m.econn));
    TRY(upload(c, P.emass, &m.emass));
    // arrays only the FP64 kernels read (the FP32 step folds mass, damping
    // and the operator into its own per-node and per-term arrays)
    m.ekv = nullptr; m.mfull = nullptr; m.ownptr = nullptr; m.ownlist = nullptr;
    m.odptr = nullptr; m.odlist = nullptr; m.edamp = nullptr; m.edampv = nullptr;
    m.ecoef = nullptr; m.inv_mfull = nullptr;
    if (c.precision == EXFEM_FP64) {
        TRY(upload(c, P.ekv, &m.ekv));
        TRY(upload(c, P.mfull_int, &m.mfull));
        TRY(upload(c, P.ownptr, &m.ownptr));
        TRY(upload(c, P.ownlist, &m.ownlist));
        TRY(upload(c, P.odptr, &m.odptr));
        TRY(upload(c, P.odlist, &m.odlist));
        TRY(upload(c, P.edamp, &m.edamp));
        TRY(upload(c, P.edampv, &m.edampv));
        TRY(upload(c, P.ecoef, &m.ecoef));
        TRY(upload(c, P.inv_mfull, &m.inv_mfull));
    }
    TRY(upload(c, P.lptr, &m.lptr));
    TRY(upload(c, P.llist, &m.llist));
    TRY(upload(c, P.tptr, &m.tptr));
    TRY(upload(c, P.tlist, &m.tlist));
    TRY(upload(c, P.dptr, &m.dptr));
    TRY(upload(c, P.dlist, &m.dlist));
    TRY(upload(c, P.hang, &m.hang));
    TRY(upload(c, P.s_elem, &m.s_elem));
    TRY(upload(c, P.s_kind, &m.s_kind));
    TRY(upload(c, P.rnode, &m.rnode));
    TRY(upload(c, P.rw, &m.rw));
    TRY(upload(c, P.rsoil, &m.rsoil));
    TRY(upload(c, P.rxy, &m.rxy));
    std::vector<DevWave> dw(P.R);
    for (int r = 0; r < P.R; ++r) {
        const WaveConst &w = P.waves[r];
        DevWave &d = dw[r];
        d.kind = w.kind; d.alpha = w.alpha; d.beta = w.beta; d.fp = w.fp;
        d.sine = w.sine; d.cose = w.cose; d.sinf = w.sinf; d.cosf = w.cosf;
        d.amp0 = w.amp0; d.wa1 = w.wa1; d.wb1 = w.wb1;
        for (int k = 0; k < 6; ++k) d.wui[k] = w.wui[k];
        d.t0 = w.t0;
        d.inv_alpha = 1.0 / w.alpha;
        d.inv_beta = 1.0 / w.beta;
    }
    TRY(upload(c, dw, &m.waves));
    m.point_kind = P.point_kind;
    m.point_amp = P.point_amp;
    m.point_sigma = P.point_sigma;
    m.point_t0 = P.point_t0;
    m.pflag = nullptr;
    m.pnodes = nullptr;
    m.npoint = 0;
    if (P.point_kind != 0) {
        std::vector<int> pn;
        for (int n = 0; n < P.nn; ++n)
            if (P.pflag[n]) pn.push_back(n);
        TRY(upload(c, P.pflag, &m.pflag));
        m.npoint = (int)pn.size();
        if (!pn.empty()) TRY(upload(c, pn, &m.pnodes));
    }
    TRY(dalloc(c, (size_t)std::max(m.ns, 1) * 16 * P.R, &m.fdrm));
    TRY(dalloc(c, (size_t)P.R * P.nsave * std::max(P.nrecv, 1) * 2, &m.seis));
    int *ctr = nullptr;
    TRY(dalloc(c, 8, &ctr));
    m.d_step = ctr;
    m.d_flag = ctr + 1;
    m.d_blocks = reinterpret_cast<unsigned *>(ctr + 2);
    m.d_drm_step = ctr + 3;
    m.d_drm_blocks = reinterpret_cast<unsigned *>(ctr + 4);
    return EXFEM_OK;
}

int alloc_fp64(Ctx &c) {
    const Plan &P = c.plan;
    size_t nst = (size_t)P.nn * 2 * P.R;
    TRY(dalloc(c, nst, &c.u64[0]));
    TRY(dalloc(c, nst, &c.u64[1]));
    TRY(dalloc(c, (size_t)P.ne * 8 * P.R, &c.ef64));
    // the reference-order form runs the next step's DRM forces on a second
    // stream too (its slot 0 is the DRM force array every form has)
    c.drm_side = c.opts.variant == EXFEM_VARIANT_REFERENCE_ORDER && c.dm.ns > 0 && c.opts.drm_inline == 0;
    if (c.drm_side) {
        c.fdrm64_slot[0] = c.dm.fdrm;
        TRY(dalloc(c, (size_t)c.dm.ns * 16 * P.R, &c.fdrm64_slot[1]));
        TRY(side_create(c));
    }
    return EXFEM_OK;
}

void free_all(Ctx &c) {
    if (c.graph) { cudaGraphExecDestroy(c.graph); c.graph = nullptr; }
    if (c.side) {
        cudaStreamSynchronize(c.side);
        cudaStreamDestroy(c.side);
        c.side = nullptr;
    }
    for (cudaEvent_t *e : {&c.ev_step, &c.ev_fork, &c.ev_drm[0], &c.ev_drm[1], &c.cev_step, &c.cev_drm[0],
                           &c.cev_drm[1]})
        if (*e) { cudaEventDestroy(*e); *e = nullptr; }
    if (c.stream) {
        for (void *p : c.allocs) cudaFreeAsync(p, c.stream);   // back to the pool, in stream order
        cudaStreamSynchronize(c.stream);
        cudaStreamDestroy(c.stream);
        c.stream = nullptr;
    }
    c.allocs.clear();
}

}  // namespace

namespace exfem {

int side_create(Ctx &c) {
    CK(cudaStreamCreateWithFlags(&c.side, cudaStreamNonBlocking));
    for (cudaEvent_t *e : {&c.ev_step, &c.ev_fork, &c.ev_drm[0], &c.ev_drm[1], &c.cev_step, &c.cev_drm[0],
                           &c.cev_drm[1]})
        CK(cudaEventCreateWithFlags(e, cudaEventDisableTiming));
    return EXFEM_OK;
}

int side_mark(Ctx &c) {
    if (c.prof_on) return EXFEM_OK;
    CK(cudaEventRecord(c.ev_step, c.stream));
    c.ev_step_valid = true;
    return EXFEM_OK;
}

int side_join(Ctx &c) {
    for (int s = 0; s < 2; ++s)
        if (c.drm_wait[s]) {
            CK(cudaStreamWaitEvent(c.stream, c.ev_drm[s], 0));
            c.drm_wait[s] = false;
        }
    return EXFEM_OK;
}

}  // namespace exfem

namespace {

int launch_step(Ctx &c, int par) {
    return c.precision == EXFEM_FP64 ? launch_step64(c, par) : f32_launch_step(c, par);
}

// Capture `g` steps starting at parity 0 into a graph (g even keeps parity).
int capture_graph(Ctx &c, int g) {
    if (c.graph) { cudaGraphExecDestroy(c.graph); c.graph = nullptr; }
    cudaGraph_t graph = nullptr;
    CK(cudaStreamBeginCapture(c.stream, cudaStreamCaptureModeThreadLocal));
    long long before = c.launches;
    // The side stream (FP32 DRM forces) joins the capture through an event of
    // the main stream and rejoins it at the end.  Inside the graph the first
    // step waits for no earlier DRM launch: a replay starts only after the
    // host has made the main stream wait for them (f32_join_side).
    const bool w0 = c.drm_wait[0], w1 = c.drm_wait[1], sv = c.ev_step_valid;
    int rc = EXFEM_OK;
    if (c.drm_side) {
        cudaEventRecord(c.ev_fork, c.stream);
        cudaStreamWaitEvent(c.side, c.ev_fork, 0);
        c.drm_wait[0] = c.drm_wait[1] = false;
        c.ev_step_valid = false;
        std::swap(c.ev_step, c.cev_step);
        std::swap(c.ev_drm[0], c.cev_drm[0]);
        std::swap(c.ev_drm[1], c.cev_drm[1]);
    }
    int par = 0;
    for (int i = 0; i < g && rc == EXFEM_OK; ++i) {
        rc = launch_step(c, par);
        par ^= 1;
    }
    if (c.drm_side) {
        const int rj = side_join(c);
        if (!rc) rc = rj;
    }
    cudaError_t e = cudaStreamEndCapture(c.stream, &graph);
    if (c.drm_side) {
        std::swap(c.ev_step, c.cev_step);
        std::swap(c.ev_drm[0], c.cev_drm[0]);
        std::swap(c.ev_drm[1], c.cev_drm[1]);
    }
    c.drm_wait[0] = w0;
    c.drm_wait[1] = w1;
    c.ev_step_valid = sv;
    c.launches = before;   // captured launches are counted on replay
    if (rc) { if (graph) cudaGraphDestroy(graph); return rc; }
    if (e != cudaSuccess) { c.err = std::string("graph capture: ") + cudaGetErrorString(e); return EXFEM_E_CUDA; }
    e = cudaGraphInstantiate(&c.graph, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) { c.err = std::string("graph instantiate: ") + cudaGetErrorString(e); c.graph = nullptr; return EXFEM_E_CUDA; }
    c.graph_steps = g;
    return EXFEM_OK;
}

int launches_per_step(const Ctx &c) {
    // the reference-order FP64 variant and the FP32 form compute the next
    // step's DRM forces inside their hanging/receiver kernel
    if (c.precision == EXFEM_FP64)   // (drm,) elem, node, hang
        return (c.dm.ns > 0 && (c.opts.variant != EXFEM_VARIANT_REFERENCE_ORDER || c.drm_side) ? 1 : 0) + 3;
    return 2 + (c.p32_n > 0 ? 1 : 0) + (c.drm_side ? 1 : 0);   // step, (point,) hang, (side-stream DRM)
}

// Device side of exfem_gpu_create: stream, uploads, state buffers.
int create_device(Ctx &c, const exfem_mesh &mesh) {
    CK(cudaSetDevice(c.device));
    CK(cudaStreamCreateWithFlags(&c.stream, cudaStreamNonBlocking));
    CK(cudaDeviceGetAttribute(&c.num_sms, cudaDevAttrMultiProcessorCount, c.device));
    // node coordinates in internal order (free field at DRM corners)
    TRY(upload(c, c.plan.nxy, &c.dm.nxy));   // internal node coordinates
    TRY(setup_device(c));
    c.block_threads = c.opts.block_threads > 0 ? c.opts.block_threads : 128;
    TRY(c.precision == EXFEM_FP64 ? alloc_fp64(c) : f32_alloc(c));
    CK(cudaStreamSynchronize(c.stream));
    return EXFEM_OK;
}

}  // namespace

namespace exfem {
static std::mutex g_pool_mu;
static cudaMemPool_t g_pool[128] = {};

// The library's pool for a device, created on first use.  Its release
// threshold keeps every freed byte, so contexts created after others were
// destroyed reuse their memory.
static cudaError_t device_pool(int dev, cudaMemPool_t *out) {
    if (dev < 0 || dev >= 128) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(g_pool_mu);
    if (!g_pool[dev]) {
        cudaMemPoolProps props;
        std::memset(&props, 0, sizeof(props));
        props.allocType = cudaMemAllocationTypePinned;
        props.location.type = cudaMemLocationTypeDevice;
        props.location.id = dev;
        cudaMemPool_t pool = nullptr;
        cudaError_t e = cudaMemPoolCreate(&pool, &props);
        if (e != cudaSuccess) return e;
        uint64_t keep = UINT64_MAX;
        e = cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
        if (e != cudaSuccess) { cudaMemPoolDestroy(pool); return e; }
        g_pool[dev] = pool;
    }
    *out = g_pool[dev];
    return cudaSuccess;
}

int release_cached(int device) {
    cudaMemPool_t pool = nullptr;
    {
        if (device < 0 || device >= 128) return EXFEM_E_ARG;
        std::lock_guard<std::mutex> lock(g_pool_mu);
        pool = g_pool[device];
    }
    if (!pool) return EXFEM_OK;
    int prev = 0;
    if (cudaGetDevice(&prev) != cudaSuccess || cudaSetDevice(device) != cudaSuccess) return EXFEM_E_CUDA;
    const cudaError_t e = cudaMemPoolTrimTo(pool, 0);
    cudaSetDevice(prev);
    return e == cudaSuccess ? EXFEM_OK : EXFEM_E_CUDA;
}

cudaError_t scratch_alloc(Ctx &c, void **p, size_t bytes) {
    cudaMemPool_t pool = nullptr;
    cudaError_t e = device_pool(c.device, &pool);
    if (e != cudaSuccess) return e;
    return cudaMallocFromPoolAsync(p, bytes, pool, c.stream);
}

cudaError_t ctx_alloc(Ctx &c, void **p, size_t bytes) {
    cudaError_t e = scratch_alloc(c, p, bytes);
    if (e == cudaSuccess) {
        c.allocs.push_back(*p);
        c.bytes += bytes;
    }
    return e;
}

void mark(Ctx &c, const char *kernel) {
    if (!c.prof_on) return;
    cudaEvent_t ev = nullptr;
    if (cudaEventCreate(&ev) != cudaSuccess) return;
    cudaEventRecord(ev, c.stream);
    c.marks.push_back({kernel, ev});
}
}  // namespace exfem

extern "C" {

void exfem_gpu_default_opts(exfem_opts *o) {
    if (!o) return;
    std::memset(o, 0, sizeof(*o));
    o->precision = EXFEM_FP64;
    o->device = 0;
    o->use_graph = 1;
    o->graph_steps = 0;
    o->block_threads = 0;
    o->rhs_per_thread = 0;
    o->reorder = 1;
    o->check_every = 0;
    o->variant = EXFEM_VARIANT_REFERENCE_ORDER;
    o->index_bits = 0;
    o->pad_rhs = 0;
    o->wait_cycles = 0;
    o->tune = 0;
    o->drm_inline = 0;
    o->serial_launch = 0;
}

int exfem_gpu_create(const exfem_mesh *mesh, const exfem_problem *prob, const exfem_opts *opts, exfem_ctx **out) {
    g_create_err.clear();
    if (!out || !mesh || !prob) { g_create_err = "NULL argument"; return EXFEM_E_ARG; }
    *out = nullptr;
    exfem_opts o;
    if (opts) o = *opts;
    else exfem_gpu_default_opts(&o);
    if (o.precision != EXFEM_FP64 && o.precision != EXFEM_FP32_KAHAN) { g_create_err = "unknown precision"; return EXFEM_E_ARG; }
    if (o.variant < 0 || o.variant > (o.precision == EXFEM_FP32_KAHAN ? 5 : 1)) {
        g_create_err = "unknown kernel variant";
        return EXFEM_E_ARG;
    }
    if (o.index_bits != 0 && o.index_bits != 64) { g_create_err = "index_bits must be 0 or 64"; return EXFEM_E_ARG; }
    if (o.pad_rhs != 0 && o.pad_rhs != 1) { g_create_err = "pad_rhs must be 0 or 1"; return EXFEM_E_ARG; }
    if (o.wait_cycles < 0) { g_create_err = "wait_cycles must be >= 0"; return EXFEM_E_ARG; }
    if (o.tune != 0 && o.tune != 1) { g_create_err = "tune must be 0 or 1"; return EXFEM_E_ARG; }
    if (o.drm_inline != 0 && o.drm_inline != 1) { g_create_err = "drm_inline must be 0 or 1"; return EXFEM_E_ARG; }
    if (o.serial_launch != 0 && o.serial_launch != 1) {
        g_create_err = "serial_launch must be 0 or 1";
        return EXFEM_E_ARG;
    }
    const int max_bt = o.precision == EXFEM_FP64 ? 256 : 512;   // the kernels' __launch_bounds__
    if (o.block_threads < 0 || o.block_threads > max_bt || (o.block_threads % 32) != 0) {
        g_create_err = "block_threads must be a multiple of 32 in [0, " + std::to_string(max_bt) + "]";
        return EXFEM_E_ARG;
    }
    exfem_ctx *c = nullptr;
    try {
        c = new exfem_ctx();
    } catch (const std::bad_alloc &) {
        g_create_err = "host allocation failed";
        return EXFEM_E_NOMEM;
    }
    c->opts = o;
    c->precision = o.precision;
    c->device = o.device;
    int rc;
    try {
        const int r_int = (o.precision == EXFEM_FP32_KAHAN && o.pad_rhs == 0) ? padded_rhs(prob->nrhs) : 0;
        rc = build_plan(*mesh, *prob, o.reorder != 0, c->plan, c->err, r_int, o.precision == EXFEM_FP64);
    } catch (const std::bad_alloc &) {
        rc = EXFEM_E_NOMEM;
        c->err = "host allocation failed while preparing the model";
    }
    if (rc) { g_create_err = c->err; delete c; return rc; }
    rc = create_device(*c, *mesh);
    if (rc) {
        if (rc == EXFEM_E_CUDA && c->err.find("out of memory") != std::string::npos) rc = EXFEM_E_NOMEM;
        g_create_err = c->err;
        free_all(*c);
        delete c;
        return rc;
    }
    *out = c;
    return EXFEM_OK;
}

int exfem_gpu_init_explicit(exfem_ctx *ctx, double *mfull_out) {
    if (!ctx) return EXFEM_E_ARG;
    Ctx &c = *ctx;
    CK(cudaSetDevice(c.device));
    DevModel &m = c.dm;
    if (c.precision == EXFEM_FP64) {
        size_t nst = (size_t)c.plan.nn * 2 * c.plan.R;
        CK(cudaMemsetAsync(c.u64[0], 0, nst * sizeof(double), c.stream));
        CK(cudaMemsetAsync(c.u64[1], 0, nst * sizeof(double), c.stream));
        if (m.point_kind == EXFEM_POINT_DISP && m.npoint > 0) {   // explicit.f90:93-94
            const int nb = nblocks((long long)m.npoint * m.R, 128);
            k_point_set64<<<nb, 128, 0, c.stream>>>(m, c.u64[0], point_ricker(m.point_amp, m.point_sigma, 0.0 - m.point_t0));
            k_point_set64<<<nb, 128, 0, c.stream>>>(m, c.u64[1],
                                                    point_ricker(m.point_amp, m.point_sigma, -m.dt - m.point_t0));
            c.launches += 2;
            CK(cudaGetLastError());
        }
    } else {
        int rc = c.opts.tune ? f32_tune_in_place(c) : EXFEM_OK;
        if (!rc) rc = f32_init(c);
        if (rc) return rc;
    }
    CK(cudaMemsetAsync(m.seis, 0, sizeof(double) * (size_t)c.plan.R * c.plan.nsave * std::max(c.plan.nrecv, 1) * 2,
                       c.stream));
    CK(cudaMemsetAsync(m.d_step, 0, 8 * sizeof(int), c.stream));
    c.parity = 0;
    c.steps_done = 0;
    int rc = c.precision == EXFEM_FP64 ? launch_sample0_64(c, 0) : f32_launch_sample0(c, 0);
    if (rc) return rc;
    // the first side-stream DRM launch follows all of this (the counter reset,
    // the step-0 sample that computes step 1's forces and sets that counter)
    if (c.drm_side) {
        CK(cudaEventRecord(c.ev_step, c.stream));
        c.ev_step_valid = true;
    }
    if (mfull_out) std::memcpy(mfull_out, c.plan.mfull_ref.data(), sizeof(double) * c.plan.mfull_ref.size());
    c.inited = true;
    return EXFEM_OK;
}

int exfem_gpu_run(exfem_ctx *ctx, int nsteps) {
    if (!ctx) return EXFEM_E_ARG;
    Ctx &c = *ctx;
    if (!c.inited) { c.err = "exfem_gpu_run before exfem_gpu_init_explicit"; return EXFEM_E_STATE; }
    if (nsteps < 0 || nsteps > c.plan.nsteps - c.steps_done) {
        c.err = "nsteps exceeds the steps left in the problem";
        return EXFEM_E_ARG;
    }
    CK(cudaSetDevice(c.device));
    int left = nsteps;
    if (c.opts.use_graph) {
        int g = c.opts.graph_steps > 0 ? c.opts.graph_steps : 16;
        g += g & 1;
        if (left >= g) {
            if (!c.graph || c.graph_steps != g) {
                int rc = capture_graph(c, g);
                if (rc) return rc;
            }
            // the graph was captured from parity 0: align first
            if (c.parity == 1) {
                int rc = launch_step(c, c.parity);
                if (rc) return rc;
                c.parity ^= 1;
                --left;
                c.steps_done++;
            }
            while (left >= g) {
                if (c.drm_side) {
                    int rj = side_join(c);
                    if (rj) return rj;
                }
                CK(cudaGraphLaunch(c.graph, c.stream));
                if (c.drm_side) {   // the replay joined its side work; later side launches follow it
                    CK(cudaEventRecord(c.ev_step, c.stream));
                    c.ev_step_valid = true;
                }
                c.launches += (long long)g * launches_per_step(c);
                left -= g;
                c.steps_done += g;
            }
        }
    }
    while (left > 0) {
        int rc = launch_step(c, c.parity);
        if (rc) return rc;
        c.parity ^= 1;
        --left;
        c.steps_done++;
    }
    // the main stream covers the last side-stream launch (sync, query, events)
    return c.drm_side ? side_join(c) : EXFEM_OK;
}

int exfem_gpu_sync(exfem_ctx *ctx) {
    if (!ctx) return EXFEM_E_ARG;
    Ctx &c = *ctx;
    CK(cudaSetDevice(c.device));
    CK(cudaStreamSynchronize(c.stream));
    int flag = 0;
    CK(cudaMemcpy(&flag, c.dm.d_flag, sizeof(int), cudaMemcpyDeviceToHost));
    c.d2h_bytes += sizeof(int);
    // a timed-out wait leaves the state incomplete, so it is reported first
    if (flag & 2) { c.err = "a bounded device wait timed out"; return EXFEM_E_TIMEOUT; }
    if (flag & 1) { c.err = "non-finite receiver sample (the run diverged)"; return EXFEM_E_NAN; }
    return EXFEM_OK;
}

int exfem_gpu_query(exfem_ctx *ctx) {
    if (!ctx) return EXFEM_E_ARG;
    Ctx &c = *ctx;
    CK(cudaSetDevice(c.device));
    cudaError_t e = cudaStreamQuery(c.stream);
    if (e == cudaErrorNotReady) return 1;
    if (e != cudaSuccess) { c.err = cudaGetErrorString(e); return EXFEM_E_CUDA; }
    int flag = 0;
    CK(cudaMemcpy(&flag, c.dm.d_flag, sizeof(int), cudaMemcpyDeviceToHost));
    c.d2h_bytes += sizeof(int);
    if (flag & 2) { c.err = "a bounded device wait timed out"; return EXFEM_E_TIMEOUT; }
    if (flag & 1) { c.err = "non-finite receiver sample (the run diverged)"; return EXFEM_E_NAN; }
    return EXFEM_OK;
}

int exfem_gpu_get_u(exfem_ctx *ctx, int rhs, double *u, size_t n) {
    if (!ctx || !u) return EXFEM_E_ARG;
    Ctx &c = *ctx;
    const Plan &P = c.plan;
    if (rhs < 0 || rhs >= P.R_user || n < (size_t)2 * P.nn) { c.err = "bad rhs or buffer too small"; return EXFEM_E_ARG; }
    CK(cudaSetDevice(c.device));
    // the right-hand side is gathered on the device, so only its 2 * nn
    // values cross to the host (not the whole batched state)
    const long long ndof = 2LL * P.nn;
    std::vector<double> in((size_t)ndof);
    double *d = nullptr;
    CK(scratch_alloc(c, reinterpret_cast<void **>(&d), (size_t)ndof * sizeof(double)));
    const bool f64 = c.precision == EXFEM_FP64;
    k_extract_rhs<<<nblocks(ndof, 256), 256, 0, c.stream>>>(c.dm, f64 ? c.u64[c.parity] : nullptr,
                                                            f64 ? nullptr : c.uhi[c.parity], c.ucomp, rhs,
                                                            ndof, d);
    c.launches++;
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(in.data(), d, (size_t)ndof * sizeof(double), cudaMemcpyDeviceToHost, c.stream);
    cudaFreeAsync(d, c.stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c.stream);
    if (e != cudaSuccess) { c.err = std::string("get_u: ") + cudaGetErrorString(e); return EXFEM_E_CUDA; }
    c.d2h_bytes += (size_t)ndof * sizeof(double);
    for (int i = 0; i < P.nn; ++i) {
        int rn = P.ref_of_node[i];
        u[2 * (size_t)rn] = in[2 * (size_t)i];
        u[2 * (size_t)rn + 1] = in[2 * (size_t)i + 1];
    }
    return EXFEM_OK;
}

int exfem_gpu_get_seismograms(exfem_ctx *ctx, double *out, size_t cap, int *nsaved) {
    if (!ctx) return EXFEM_E_ARG;
    Ctx &c = *ctx;
    const Plan &P = c.plan;
    // right-hand side r's samples are block r (r-major): the caller's are the
    // first R_user blocks, any padding follows them
    size_t need = (size_t)P.R_user * P.nsave * P.nrecv * 2;
    if (nsaved) *nsaved = c.steps_done / P.io + 1;
    if (!out) return EXFEM_OK;
    if (cap < need) { c.err = "seismogram buffer too small"; return EXFEM_E_ARG; }
    CK(cudaSetDevice(c.device));
    CK(cudaStreamSynchronize(c.stream));
    if (need) CK(cudaMemcpy(out, c.dm.seis, need * sizeof(double), cudaMemcpyDeviceToHost));
    c.d2h_bytes += need * sizeof(double);
    return EXFEM_OK;
}

int exfem_gpu_run_timed(exfem_ctx *ctx, int nsteps, double *ms) {
    if (!ctx || !ms) return EXFEM_E_ARG;
    Ctx &c = *ctx;
    CK(cudaSetDevice(c.device));
    cudaEvent_t a, b;
    CK(cudaEventCreate(&a));
    CK(cudaEventCreate(&b));
    cudaEventRecord(a, c.stream);
    int rc = exfem_gpu_run(ctx, nsteps);
    cudaEventRecord(b, c.stream);
    cudaError_t e = cudaEventSynchronize(b);
    float f = 0.f;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&f, a, b);
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    if (rc) return rc;
    if (e != cudaSuccess) { c.err = cudaGetErrorString(e); return EXFEM_E_CUDA; }
    *ms = f;
    return EXFEM_OK;
}

int exfem_gpu_profile_kernels(exfem_ctx *ctx, int nsteps, double *ms_out, const char **names_out, int cap) {
    if (!ctx || !ms_out || !names_out || cap <= 0) return EXFEM_E_ARG;
    Ctx &c = *ctx;
    if (!c.inited) { c.err = "profile before exfem_gpu_init_explicit"; return EXFEM_E_STATE; }
    if (nsteps < 1 || nsteps > c.plan.nsteps - c.steps_done) { c.err = "nsteps exceeds the steps left"; return EXFEM_E_ARG; }
    CK(cudaSetDevice(c.device));
    CK(cudaStreamSynchronize(c.stream));
    c.prof_on = true;
    c.marks.clear();
    mark(c, "start");
    int rc = EXFEM_OK;
    for (int i = 0; i < nsteps && rc == EXFEM_OK; ++i) {
        rc = launch_step(c, c.parity);
        c.parity ^= 1;
        c.steps_done++;
    }
    c.prof_on = false;
    cudaError_t e = cudaStreamSynchronize(c.stream);
    std::vector<std::string> names;
    std::vector<double> tot;
    std::vector<int> cnt;
    for (size_t k = 1; k < c.marks.size() && e == cudaSuccess; ++k) {
        float f = 0.f;
        cudaEventElapsedTime(&f, c.marks[k - 1].second, c.marks[k].second);
        std::string n = c.marks[k].first;
        size_t j = 0;
        while (j < names.size() && names[j] != n) ++j;
        if (j == names.size()) { names.push_back(n); tot.push_back(0); cnt.push_back(0); }
        tot[j] += f;
        cnt[j]++;
    }
    for (auto &pr : c.marks) cudaEventDestroy(pr.second);
    c.marks.clear();
    if (rc) return rc;
    if (e != cudaSuccess) { c.err = cudaGetErrorString(e); return EXFEM_E_CUDA; }
    int n = (int)std::min<size_t>(names.size(), (size_t)cap);
    static thread_local std::vector<std::string> keep;
    keep = names;
    for (int k = 0; k < n; ++k) {
        ms_out[k] = tot[k] / cnt[k];
        names_out[k] = keep[k].c_str();
    }
    return n;
}

int exfem_gpu_sample_points(exfem_ctx *ctx, int rhs, int npoint, const double *xy, const int *elem, double *out) {
    if (!ctx) return EXFEM_E_ARG;
    Ctx &c = *ctx;
    if (!c.inited) { c.err = "exfem_gpu_sample_points before exfem_gpu_init_explicit"; return EXFEM_E_STATE; }
    if (rhs < 0 || rhs >= c.plan.R_user || npoint < 0 || (npoint > 0 && (!xy || !elem || !out))) {
        c.err = "bad sample_points arguments";
        return EXFEM_E_ARG;
    }
    if (npoint == 0) return EXFEM_OK;
    std::vector<int> node, soil;
    std::vector<double> w;
    if (int rc = point_weights(c.plan, npoint, xy, elem, node, w, soil, c.err)) return rc;
    CK(cudaSetDevice(c.device));
    // one scratch block: corners, soil flags, weights, points, output
    const size_t n = (size_t)npoint;
    const size_t bytes = n * (16 + 4) + n * (32 + 16 + 16) + 64;
    void *buf = nullptr;
    CK(scratch_alloc(c, &buf, bytes));
    char *b = static_cast<char *>(buf);
    double *d_w = reinterpret_cast<double *>(b);
    double *d_xy = d_w + 4 * n;
    double *d_out = d_xy + 2 * n;
    int *d_node = reinterpret_cast<int *>(d_out + 2 * n);
    int *d_soil = d_node + 4 * n;
    cudaError_t e = cudaMemcpyAsync(d_w, w.data(), 32 * n, cudaMemcpyHostToDevice, c.stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_xy, xy, 16 * n, cudaMemcpyHostToDevice, c.stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_node, node.data(), 16 * n, cudaMemcpyHostToDevice, c.stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_soil, soil.data(), 4 * n, cudaMemcpyHostToDevice, c.stream);
    const double time = c.plan.dt * (double)c.steps_done;
    if (e == cudaSuccess) {
        const bool f64 = c.precision == EXFEM_FP64;
        k_sample_points<<<nblocks((long long)npoint, 128), 128, 0, c.stream>>>(
            c.dm, f64 ? c.u64[c.parity] : nullptr, f64 ? nullptr : c.uhi[c.parity], f64 ? nullptr : c.ucomp, rhs,
            npoint, d_node, d_w, d_soil, d_xy, time, d_out);
        c.launches++;
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(out, d_out, 16 * n, cudaMemcpyDeviceToHost, c.stream);
    cudaFreeAsync(buf, c.stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c.stream);
    c.h2d_bytes += n * (32 + 16 + 16 + 4);
    c.d2h_bytes += n * 16;
    if (e != cudaSuccess) { c.err = std::string("sample_points: ") + cudaGetErrorString(e); return EXFEM_E_CUDA; }
    return EXFEM_OK;
}

int exfem_gpu_steps_done(const exfem_ctx *ctx) { return ctx ? ctx->steps_done : 0; }
long long exfem_gpu_launch_count(const exfem_ctx *ctx) { return ctx ? ctx->launches : 0; }
size_t exfem_gpu_device_bytes(const exfem_ctx *ctx) { return ctx ? ctx->bytes : 0; }

int exfem_gpu_release_cached(int device) { return exfem::release_cached(device); }

int exfem_gpu_copy_bytes(const exfem_ctx *ctx, unsigned long long *h2d, unsigned long long *d2h) {
    if (!ctx) return EXFEM_E_ARG;
    if (h2d) *h2d = ctx->h2d_bytes;
    if (d2h) *d2h = ctx->d2h_bytes;
    return EXFEM_OK;
}

size_t exfem_gpu_estimate_bytes(const exfem_mesh *mesh, const exfem_problem *prob, const exfem_opts *opts) {
    // An upper bound of what exfem_gpu_create and init_explicit allocate
    // (the sum over the allocations of setup_device, alloc_fp64/f32_alloc).
    if (!mesh || !prob) return 0;
    const size_t nn = (size_t)std::max(mesh->nnodes, 0), ne = (size_t)std::max(mesh->nelems, 0);
    const bool pad = opts && opts->precision == EXFEM_FP32_KAHAN && opts->pad_rhs == 0;
    const size_t R = (size_t)std::max(pad ? padded_rhs(prob->nrhs) : prob->nrhs, 1);
    const size_t nh = (size_t)std::max(prob->nhanging, 0);
    const size_t ns = (size_t)std::max(prob->nseismic, 0), nr = (size_t)std::max(prob->nrecv, 0);
    const size_t nsave = prob->io_interval > 0 ? (size_t)(prob->nsteps / prob->io_interval + 1) : 1;
    size_t nabs = 0;
    if (prob->absorbing)
        for (size_t i = 0; i < nn; ++i) nabs += prob->absorbing[i] != 0;
    const bool f64 = !opts || opts->precision == EXFEM_FP64;
    size_t b = 16 * nn;                                            // node coordinates
    b += ne * (16 + 8);                                            // conn, mass
    if (f64) {
        b += ne * (48 + 4 + 32 + 16);                              // calck values, damp slot, coef, own list
        b += 64 * std::min(ne, 4 * nabs + 4);                      // dashpot values of boundary elements
        b += 2 * 4 * (nn + 1) + 32 * nn;                           // own and DRM-own pointers, m_full, 1/m_full
    }
    b += 3 * 4 * (nn + 1) + 16 * nh + 12 * nh;                     // link, gather and DRM pointers, links, hanging
    b += 4 * (4 * ne + 4 * nh);                                    // gather lists (own + hanging halves)
    b += ns * (16 + 8 + 32) + nr * (16 + 32 + 4 + 16) + R * 192;   // DRM lists, receivers, waves
    b += 2 * 16 * std::max(ns, (size_t)1) * R * 8;                  // DRM forces (two slots with the second stream)
    b += R * nsave * std::max(nr, (size_t)1) * 16 + 16;            // seismograms, counters
    if (f64) b += R * (nn * 32 + ne * 64);                          // u ping-pong, element forces
    else b += nn * 16 + 16 * std::max(nh, (size_t)1) + ne * 16 + 64 * std::max(ns, (size_t)1) * R + 96 * ns * R +
              R * nn * 2 * (4 + 4 + 2 + 4 + 2);                     // FP32 state
    if (!f64 && opts->variant >= 1) {
        // tiles: every halo entry is a node or a corner/anchor of one of its terms
        const size_t H = nn + 16 * (ne + nh) + nh;
        b += 8 * (nn + 2) + 12 * H + 8 * (4 * ne + 4 * nh) + 4 * nn + 4 * nh;
    }
    if (!f64) b += 20 * nn + 8 * ne;                                // node slot records, the two stored coefficients
    // the direct gather's term corners: per term (list form) or 4 per node (slot records)
    if (!f64 && (f32_term_corners(R) || f32_slot_corners(R))) b += std::max(16 * (4 * ne + 4 * nh), 64 * nn);
    if (prob->point_kind) b += nn + 4 * (size_t)std::max(prob->npoint, 0) + 1024;   // source flags and nodes
    return b + 64 * 1024;
}

const char *exfem_gpu_last_error(const exfem_ctx *ctx) {
    if (!ctx) return g_create_err.c_str();
    return ctx->err.c_str();
}

void exfem_gpu_destroy(exfem_ctx *ctx) {
    if (!ctx) return;
    cudaSetDevice(ctx->device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    free_all(*ctx);
    delete ctx;
}

}  // extern "C"
