// exfem_f64ref_nofma.cu — FP64 step kernels in the reference's operation order.
//
// This translation unit is compiled with -fmad=false: every product and sum
// rounds separately, as the reference's Fortran (and the CPU oracle) does, so
// the per-element terms, the per-dof sums and the update reproduce
// run_explicit (explicit.f90:125-153) operation for operation:
//   * localr = (a3 u - a1 u-)*m; localr += a2*c*u-; then the
//     dgemv('N',8,8,-1,K,8,u,1,1,localr,1) of explicit.f90:139-140 column by
//     column with K = calck(mu, lambda) (formulation.f90:276-313);
//   * each dof sums its DRM terms (seismic order, K part then mass part,
//     model.f90:794-798) and then its element terms in element order;
//   * anchors add half of each hanging node's sum in m_hanging order
//     (sum_reactanchors, halving form), then u = r / m_full (explicit.f90:148).
// The only differences left are the exp() of the free field (CUDA vs the host
// libm, ulp level).
#include <cuda_runtime.h>

#include <algorithm>
#include <mutex>
#include <string>

#include "exfem_ctx.h"
#include "exfem_device.cuh"

namespace exfem {

namespace {



// calcsqm (formulation.f90:256-268) entry (i, j): same component only,
// 4 on the diagonal, 2 for edge-adjacent corners, 1 for the opposite corner.
__device__ __forceinline__ double sqm(int i, int j) {
    if ((i & 1) != (j & 1)) return 0.0;
    int d = ((j >> 1) - (i >> 1)) & 3;
    double v = (d == 0) ? 4.0 : (d == 2 ? 1.0 : 2.0);
    return v / 9.0;
}

// One thread per (boundary element, rhs): wave_reactions with the dense
// multdrm loops (formulation.f90:378-393).  Stores the stiffness part and
// the mass part separately (each is added to the reactions on its own).
// Sixteen threads per (DRM element, rhs).  Thread 4c + q evaluates term q of
// the free field (incident, reflected P, reflected SV; q = 3 idles) at the
// element's corner c: its FP64 Ricker pulse is the cost.  Shuffles give every
// thread the corner values, summed term by term in planewave's order, and
// thread o < 8 forms row o of both multdrm products.  For each row it applies
// exactly the updates of the reference's loop over (i, j), in the same order,
// so every force is bit for bit the one-thread result.  Block `b` holds items
// [b * ipb, (b + 1) * ipb) (ipb <= threads / 16, threads a multiple of 32);
// every thread of the block must call it (warp shuffles).  The forces depend
// on time only: `step` is the step they are for.
__device__ __forceinline__ void drm_ref_items(const DevModel &m, int ipb, long long b, int step) {
    const int li = threadIdx.x >> 4;
    const long long w = b * ipb + li;
    const int l = (int)(threadIdx.x & 15), corner = l >> 2, term = l & 3;
    const bool valid = li < ipb && w < (long long)m.ns * m.R;
    int s = 0, r = 0, ie = 0;
    double p0x = 0.0, p0z = 0.0, p2x = 0.0, p2z = 0.0;   // columns u and ddu of this term
    if (valid) {
        s = (int)(w / m.R);
        r = (int)(w % m.R);
        ie = m.s_elem[s];
        if (term < 3) {
            const DevWave wv = m.waves[r];
            double outt = (double)step * m.dt - wv.t0;
            int x = m.econn[4 * ie + corner];
            double ox = m.nxy[2 * x] - m.worigin_x, oz = m.nxy[2 * x + 1] - m.worigin_y;
            double px[3], pz[3];
            pw_term(wv, term, outt, ox, oz, px, pz);
            p0x = px[0]; p0z = pz[0];
            p2x = px[2]; p2z = pz[2];
        }
    }
    double u0[8], a0[8];
#pragma unroll
    for (int c = 0; c < 4; ++c) {
        double v[4][3];
#pragma unroll
        for (int q = 0; q < 3; ++q) {
            v[0][q] = __shfl_sync(0xffffffffu, p0x, 4 * c + q, 16);
            v[1][q] = __shfl_sync(0xffffffffu, p0z, 4 * c + q, 16);
            v[2][q] = __shfl_sync(0xffffffffu, p2x, 4 * c + q, 16);
            v[3][q] = __shfl_sync(0xffffffffu, p2z, 4 * c + q, 16);
        }
        u0[2 * c] = v[0][0] + v[0][1] + v[0][2];
        u0[2 * c + 1] = v[1][0] + v[1][1] + v[1][2];
        a0[2 * c] = v[2][0] + v[2][1] + v[2][2];
        a0[2 * c + 1] = v[3][0] + v[3][1] + v[3][2];
    }
    if (!valid || l >= 8) return;
    const int o = l;
    unsigned e = drm_mask(m.s_kind[s]);
    double K[64];
    {
        const double2 *kv2 = reinterpret_cast<const double2 *>(m.ekv + (size_t)ie * 6);
        const double2 a = kv2[0], b = kv2[1], c6 = kv2[2];
        const double kv[6] = {a.x, a.y, b.x, b.y, c6.x, c6.y};
        calck(kv, K);
    }
    double pk = 0.0, pm = 0.0;
    for (int i = 0; i < 8; ++i)
        for (int j = 0; j < 8; ++j)
            if (((e >> j) & 1u) && !((e >> i) & 1u)) {
                if (i == o) {
                    pk = pk - K[j * 8 + o] * u0[j];
                    pm = pm - sqm(o, j) * a0[j];
                }
                if (j == o) {
                    pk = pk + K[i * 8 + o] * u0[i];
                    pm = pm + sqm(o, i) * a0[i];
                }
            }
    m.fdrm[((size_t)s * 16 + o) * m.R + r] = pk;
    m.fdrm[((size_t)s * 16 + 8 + o) * m.R + r] = pm * m.emass[ie];
}

// DRM forces of the current step (read from the device step counter), on
// their own: the step without allocation, whose counters are its own.
__global__ void k_drm_ref(DevModel m, int ipb) {
    drm_ref_items(m, ipb, blockIdx.x, *(volatile int *)m.d_step + 1);
}

// The DRM forces of the step after the last one computed, on the context's
// second stream (the same items as in k_hang_ref, so the same bits): the step
// comes from the launches' own counter, which only they advance (in their
// stream's order), not from the step counter, which the main stream's
// hanging pass advances at the same time.  Writes m.fdrm (the slot the
// caller picked); the last block advances the counter.
__global__ void __launch_bounds__(128) k_drm_ref_side(DevModel m, int ipb) {
    const int step = *(volatile int *)m.d_drm_step + 1;
    drm_ref_items(m, ipb, blockIdx.x, step);
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        const unsigned prev = atomicAdd(m.d_drm_blocks, 1u);
        if (prev == gridDim.x - 1) {
            *m.d_drm_step = step;
            *m.d_drm_blocks = 0u;
            __threadfence();
        }
    }
}

__global__ void __launch_bounds__(128) k_elem_ref(DevModel m, const double *__restrict__ u,
                                                  const double *__restrict__ um, double *__restrict__ ef) {
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)m.ne * m.R) return;
    int e = (int)(t / m.R), r = (int)(t % m.R);
    const int4 c = reinterpret_cast<const int4 *>(m.econn)[e];
    const int cn[4] = {c.x, c.y, c.z, c.w};
    double lu[8], lp[8];
    const size_t R = m.R;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        size_t ix = ((size_t)cn[k] * 2) * R + r;
        lu[2 * k] = u[ix]; lu[2 * k + 1] = u[ix + R];
        lp[2 * k] = um[ix]; lp[2 * k + 1] = um[ix + R];
    }
    double mass = m.emass[e];
    double lr[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) lr[k] = (m.a3 * lu[k] - m.a1 * lp[k]) * mass;
    int ds = m.edamp[e];
    if (ds >= 0) {
        const double *dv = m.edampv + (size_t)ds * 8;
#pragma unroll
        for (int k = 0; k < 8; ++k) lr[k] = lr[k] + m.a2 * dv[k] * lp[k];
    }
    double K[64];
    {
        const double2 *kv2 = reinterpret_cast<const double2 *>(m.ekv + (size_t)e * 6);
        const double2 a = kv2[0], b = kv2[1], c6 = kv2[2];
        const double kv[6] = {a.x, a.y, b.x, b.y, c6.x, c6.y};
        calck(kv, K);
    }
#pragma unroll
    for (int col = 0; col < 8; ++col) {
        double temp = -1.0 * lu[col];
#pragma unroll
        for (int row = 0; row < 8; ++row) lr[row] = lr[row] + temp * K[col * 8 + row];
    }
    if (R == 1) {
        double4 *o = reinterpret_cast<double4 *>(ef + (size_t)e * 8);
        o[0] = make_double4(lr[0], lr[1], lr[2], lr[3]);
        o[1] = make_double4(lr[4], lr[5], lr[6], lr[7]);
    } else {
#pragma unroll
        for (int k = 0; k < 8; ++k) ef[((size_t)e * 8 + k) * R + r] = lr[k];
    }
}

// Sum of one node's own terms in the reference order: DRM (additive_reactions,
// explicit.f90:128), elements (129-142), then a point force on its y dof
// (absolute_reactions, 144) at step `step`.
__device__ __forceinline__ void own_sum(const DevModel &m, int n, int r, const double *__restrict__ ef, int step,
                                        double &rx, double &ry) {
    const size_t R = m.R;
    rx = 0.0;
    ry = 0.0;
    for (int q = m.odptr[n]; q < m.odptr[n + 1]; ++q) {
        int sc = m.odlist[q];
        size_t b = ((size_t)(sc >> 2) * 16 + 2 * (sc & 3)) * R + r;
        rx = rx + m.fdrm[b];
        ry = ry + m.fdrm[b + R];
        rx = rx + m.fdrm[b + 8 * R];
        ry = ry + m.fdrm[b + 9 * R];
    }
    for (int q = m.ownptr[n]; q < m.ownptr[n + 1]; ++q) {
        int ec = __ldg(m.ownlist + q);
        size_t b = ((size_t)(ec >> 2) * 8 + 2 * (ec & 3)) * R + r;
        rx = rx + ef[b];
        ry = ry + ef[b + R];
    }
    if (m.point_kind == EXFEM_POINT_FORCE && m.pflag[n]) ry = ry + point_value(m, step);
}

__global__ void __launch_bounds__(128) k_node_ref(DevModel m, const double *__restrict__ ef, double *__restrict__ unew) {
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)m.n_active * m.R) return;
    int n = (int)(t / m.R), r = (int)(t % m.R);
    const int step = *(volatile int *)m.d_step + 1;
    double rx, ry;
    own_sum(m, n, r, ef, step, rx, ry);
    for (int q = m.lptr[n]; q < m.lptr[n + 1]; ++q) {
        double hx, hy;
        own_sum(m, m.llist[2 * q], r, ef, step, hx, hy);
        rx = rx + hx / 2.0;
        ry = ry + hy / 2.0;
    }
    const size_t R = m.R;
    unew[((size_t)n * 2) * R + r] = rx / m.mfull[2 * n];
    double uy = ry / m.mfull[2 * n + 1];
    if (m.point_kind == EXFEM_POINT_DISP && m.pflag[n]) uy = point_value(m, step);   // explicit.f90:150
    unew[((size_t)n * 2 + 1) * R + r] = uy;
}

// u at a receiver corner.  A hanging corner is read as set_dispshanging's
// (u_a + u_b)/2, because the blocks writing hanging nodes run beside the
// receiver blocks; `rows` reads its own row instead (the step-0 sample, where
// a prescribed point displacement may differ from the average).
__device__ __forceinline__ void load_u64(const DevModel &m, const double *u, int node, int r, bool rows, double &vx,
                                         double &vy) {
    const size_t R = m.R;
    if (node < m.n_active || rows) {
        vx = u[((size_t)node * 2) * R + r];
        vy = u[((size_t)node * 2 + 1) * R + r];
    } else {   // hanging corner: set_dispshanging value (u_a + u_b)/2
        int i = node - m.n_active;
        int a = m.hang[3 * i + 1], b = m.hang[3 * i + 2];
        vx = (u[((size_t)a * 2) * R + r] + u[((size_t)b * 2) * R + r]) / 2.0;
        vy = (u[((size_t)a * 2 + 1) * R + r] + u[((size_t)b * 2 + 1) * R + r]) / 2.0;
    }
}

// Hanging nodes (set_dispshanging) and receiver samples (visu_field,
// visualization.f90:156-181): blocks [0, nb_hang) do the hanging nodes, the
// rest sample the receivers on save steps.  mode 1 records the step-0 sample.
// Hanging nodes, receivers, and (reference-order variant) the DRM forces of
// the next step, which depend on time only: blocks [0, nb_hang) hanging
// nodes, then nb_recv receiver blocks (ipb items each), then the DRM blocks
// (ipb_drm items each).  mode 1: the step-0 receiver sample and the DRM
// forces of step 1.  (In the element kernel's launch instead, the DRM blocks
// slowed the elements by what they saved here: both wait on the FP64 pipe.)
__global__ void __launch_bounds__(128) k_hang_ref(DevModel m, double *__restrict__ unew, int nb_hang, int mode, int ipb,
                                                  int nb_recv, int ipb_drm) {
    int step = (mode == 1) ? 0 : *(volatile int *)m.d_step + 1;
    const size_t R = m.R;
    // the step-0 sample computes step 1's DRM forces: the side-stream DRM
    // launches continue from there
    if (mode == 1 && blockIdx.x == 0 && threadIdx.x == 0) *m.d_drm_step = 1;
    if ((int)blockIdx.x >= nb_hang + nb_recv) {
        drm_ref_items(m, ipb_drm, (long long)blockIdx.x - nb_hang - nb_recv, step + 1);
    } else if ((int)blockIdx.x < nb_hang) {
        long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
        if (mode == 0 && t < (long long)m.n_hang * m.R) {
            int i = (int)(t / m.R), r = (int)(t % m.R);
            int h = m.hang[3 * i], a = m.hang[3 * i + 1], b = m.hang[3 * i + 2];
            for (int d = 0; d < 2; ++d)
                unew[((size_t)h * 2 + d) * R + r] = (unew[((size_t)a * 2 + d) * R + r] + unew[((size_t)b * 2 + d) * R + r]) / 2.0;
        }
    } else if (step % m.io == 0) {
        // four threads per (receiver, rhs): thread q < 3 evaluates free-field
        // term q (the FP64 Ricker pulses are the cost), thread 0 interpolates
        // and adds the terms in planewave_u's order; `ipb` items per block
        const int li = threadIdx.x >> 2;
        const long long wq = (long long)(blockIdx.x - nb_hang) * ipb + li;
        const int q = (int)(threadIdx.x & 3);
        const bool valid = li < ipb && wq < (long long)m.nrecv * m.R;
        const int slot = step / m.io;
        int i = 0, r = 0;
        bool soil = false;
        double px = 0.0, pz = 0.0;
        if (valid) {
            i = (int)(wq % m.nrecv);
            r = (int)(wq / m.nrecv);
            soil = m.rsoil[i] != 0;
            if (soil && q < 3) {
                const DevWave wv = m.waves[r];
                double time = m.dt * (double)slot * (double)m.io;
                pw_term_u(wv, q, time - wv.t0, m.rxy[2 * i] - m.worigin_x, m.rxy[2 * i + 1] - m.worigin_y, px, pz);
            }
        }
        double tx[3], tz[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            tx[k] = __shfl_sync(0xffffffffu, px, k, 4);
            tz[k] = __shfl_sync(0xffffffffu, pz, k, 4);
        }
        if (valid && q == 0) {
            double fx = 0.0, fy = 0.0;
            for (int k = 0; k < 4; ++k) {
                double vx, vy;
                load_u64(m, unew, m.rnode[4 * i + k], r, mode == 1, vx, vy);
                double w = m.rw[4 * i + k];
                fx = fx + w * vx;
                fy = fy + w * vy;
            }
            if (soil) {
                const double dx = tx[0] + tx[1] + tx[2], dz = tz[0] + tz[1] + tz[2];
                fx = fx + dx;
                fy = fy + dz;
            }
            size_t o = (((size_t)r * m.nsave + slot) * m.nrecv + i) * 2;
            m.seis[o] = fx;
            m.seis[o + 1] = fy;
            if (!isfinite(fx) || !isfinite(fy)) atomicOr(m.d_flag, 1);
        }
    }
    if (mode == 0) {   // last block advances the device step counter
        __syncthreads();
        if (threadIdx.x == 0) {
            __threadfence();
            unsigned prev = atomicAdd(m.d_blocks, 1u);
            if (prev == gridDim.x - 1) {
                *m.d_step = *m.d_step + 1;
                *m.d_blocks = 0u;
                __threadfence();
            }
        }
    }
}

inline int nblocks(long long work, int threads) { return (int)std::max<long long>(1, (work + threads - 1) / threads); }

}  // namespace

int f64ref_launch_drm_elem_node(Ctx &c, int par) {
    DevModel m = c.dm;
    double *u = c.u64[par], *um = c.u64[par ^ 1];
    const int T = 128;
    // This step's DRM forces came from the previous step's k_hang_ref (or for
    // step 1 from the step-0 sample), or, with the second stream, from a
    // k_drm_ref_side into slot `par` while the previous step ran; the next
    // step's go into the other slot beside this step (side_drm_next).
    if (c.drm_side) {
        m.fdrm = c.fdrm64_slot[par];
        DevModel md = c.dm;
        md.fdrm = c.fdrm64_slot[par ^ 1];
        const long long WD = (long long)md.ns * md.R;   // sixteen threads per (DRM element, rhs)
        const int ipd = spread_per_block(WD, c.num_sms, T / 16);
        const int rc = side_drm_next(c, par, [&](cudaStream_t st) {
            k_drm_ref_side<<<spread_blocks(WD, ipd), T, 0, st>>>(md, ipd);
            mark(c, "k_drm_ref_side");
        });
        if (rc) return rc;
        c.launches++;
    }
    k_elem_ref<<<nblocks((long long)m.ne * m.R, T), T, 0, c.stream>>>(m, u, um, c.ef64);
    mark(c, "k_elem_ref");
    k_node_ref<<<nblocks((long long)m.n_active * m.R, T), T, 0, c.stream>>>(m, c.ef64, um);
    mark(c, "k_node_ref");
    c.launches += 2;
    if (c.drm_side && side_mark(c)) return EXFEM_E_CUDA;   // k_node_ref was the slot's reader
    return cudaGetLastError() == cudaSuccess ? EXFEM_OK : EXFEM_E_CUDA;
}

// Hanging + receivers for both FP64 variants, plus the next step's DRM forces
// for the reference-order one; mode 1 = step-0 sample (and step 1's forces).
int f64_launch_hang(Ctx &c, double *unew, int mode) {
    DevModel &m = c.dm;
    const int T = 128;
    int nbh = mode == 1 ? 0 : (int)std::max<long long>(1, ((long long)m.n_hang * m.R + T - 1) / T);
    const long long WR = (long long)m.nrecv * m.R;   // four threads per (receiver, rhs)
    const int ipb = spread_per_block(WR, c.num_sms, T / 4);
    const int nbr = WR > 0 ? spread_blocks(WR, ipb) : 0;
    // (with the second stream the DRM forces of steps 2 and on come from there)
    const bool drm = c.opts.variant == EXFEM_VARIANT_REFERENCE_ORDER && m.ns > 0 && (mode == 1 || !c.drm_side);
    const long long WD = drm ? (long long)m.ns * m.R : 0;   // sixteen threads per (DRM element, rhs)
    const int ipd = spread_per_block(WD, c.num_sms, T / 16);
    const int nbd = WD > 0 ? spread_blocks(WD, ipd) : 0;
    if (nbh + nbr + nbd == 0) return EXFEM_OK;
    k_hang_ref<<<nbh + nbr + nbd, T, 0, c.stream>>>(m, unew, nbh, mode, ipb, nbr, ipd);
    c.launches++;
    mark(c, "k_hang_ref");
    return cudaGetLastError() == cudaSuccess ? EXFEM_OK : EXFEM_E_CUDA;
}

}  // namespace exfem

// ---------------------------------------------------------------------------
// Step without allocation (exfem_gpu_step_noalloc).
//
// Callers that keep the displacement state in device memory they manage
// themselves and may not call cudaMalloc/cudaFree inside their time loop get
// one FP64 step of their buffers here.  The per-step scratch — element forces,
// DRM forces and the two step counters — lives in this file-scope array
// instead of memory the library allocates.  Every device that loads the
// library holds the array until the process exits.
namespace exfem {
namespace {

constexpr size_t kNoallocScratchDoubles = EXFEM_NOALLOC_SCRATCH_DOUBLES;
constexpr size_t kNoallocHeadDoubles = 32;   // counters, padded to 256 bytes

__device__ __align__(256) double g_noalloc_scratch[kNoallocScratchDoubles];

// Device address of g_noalloc_scratch per device, looked up once per device
// with that device current (host code only sees a stand-in for the symbol).
std::mutex g_noalloc_mu;
double *g_noalloc_addr[128] = {nullptr};

// Resets the counters a step reads: device step = step - 1, flags, blocks.
__global__ void k_noalloc_prep(int *counters, int step) {
    counters[0] = step - 1;
    counters[1] = 0;
    counters[2] = 0;
}

}  // namespace

}  // namespace exfem

namespace {

// Puts the caller's current device back when the entry point returns.
struct DeviceRestore {
    int prev = -1;
    ~DeviceRestore() {
        if (prev >= 0) cudaSetDevice(prev);
    }
};

}  // namespace

extern "C" int exfem_gpu_step_noalloc(exfem_ctx *ctx, int step, const double *d_u, const double *d_um,
                                      double *d_unew, void *stream) {
    using namespace exfem;
    if (!ctx || !d_u || !d_um || !d_unew) return EXFEM_E_ARG;
    Ctx &c = *ctx;
    if (c.precision != EXFEM_FP64) { c.err = "exfem_gpu_step_noalloc needs an EXFEM_FP64 context"; return EXFEM_E_ARG; }
    if (c.opts.variant != EXFEM_VARIANT_REFERENCE_ORDER) {
        c.err = "exfem_gpu_step_noalloc runs the reference-order kernels only: create the context with "
                "variant = EXFEM_VARIANT_REFERENCE_ORDER";
        return EXFEM_E_ARG;
    }
    if (step < 1) { c.err = "step must be >= 1 (the time index i of explicit.f90:125)"; return EXFEM_E_ARG; }
    if (c.device < 0 || c.device >= 128) { c.err = "device ordinal out of range"; return EXFEM_E_ARG; }
    const Plan &P = c.plan;
    const size_t ns = P.s_elem.size();
    // 32 head doubles, the DRM forces rounded up to 4 doubles (the element
    // forces' double4 stores stay 32-byte aligned), then the element forces
    const size_t ef_off = kNoallocHeadDoubles + ((ns * 16 * (size_t)P.R + 3) & ~(size_t)3);
    const size_t need = ef_off + (size_t)P.ne * 8 * P.R;
    if (need > kNoallocScratchDoubles) {
        c.err = "exfem_gpu_step_noalloc: the model needs " + std::to_string(need) +
                " doubles of scratch (32 + 16*nseismic*nrhs rounded up to a multiple of 4 + 8*nelems*nrhs); "
                "the static limit is EXFEM_NOALLOC_SCRATCH_DOUBLES = " + std::to_string(kNoallocScratchDoubles);
        return EXFEM_E_ARG;
    }
    DeviceRestore restore;
    cudaError_t e = cudaGetDevice(&restore.prev);
    if (e != cudaSuccess) { restore.prev = -1; c.err = cudaGetErrorString(e); return EXFEM_E_CUDA; }
    if (restore.prev == c.device) restore.prev = -1;   // nothing to put back
    e = cudaSetDevice(c.device);
    if (e != cudaSuccess) { c.err = cudaGetErrorString(e); return EXFEM_E_CUDA; }
    double *base = nullptr;
    {
        std::lock_guard<std::mutex> lock(g_noalloc_mu);
        if (!g_noalloc_addr[c.device]) {
            void *p = nullptr;
            e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
            if (e != cudaSuccess || !p) {
                c.err = std::string("cudaGetSymbolAddress(g_noalloc_scratch): ") + cudaGetErrorString(e);
                return EXFEM_E_CUDA;
            }
            g_noalloc_addr[c.device] = static_cast<double *>(p);
        }
        base = g_noalloc_addr[c.device];
    }
    cudaStream_t st = stream ? static_cast<cudaStream_t>(stream) : c.stream;
    DevModel m = c.dm;
    int *counters = reinterpret_cast<int *>(base);
    m.d_step = counters;
    m.d_flag = counters + 1;
    m.d_blocks = reinterpret_cast<unsigned *>(counters + 2);
    m.fdrm = base + kNoallocHeadDoubles;
    m.nrecv = 0;   // receivers (and with them the NaN watchdog) stay with exfem_gpu_run
    double *ef = base + ef_off;
    const int T = 128;
    k_noalloc_prep<<<1, 1, 0, st>>>(counters, step);
    if (m.ns > 0) {
        const long long W = (long long)m.ns * m.R;
        const int ipb = spread_per_block(W, c.num_sms, 8);
        k_drm_ref<<<spread_blocks(W, ipb), 128, 0, st>>>(m, ipb);
    }
    k_elem_ref<<<nblocks((long long)m.ne * m.R, T), T, 0, st>>>(m, d_u, d_um, ef);
    k_node_ref<<<nblocks((long long)m.n_active * m.R, T), T, 0, st>>>(m, ef, d_unew);
    int nbh = (int)std::max<long long>(1, ((long long)m.n_hang * m.R + T - 1) / T);
    k_hang_ref<<<nbh, T, 0, st>>>(m, d_unew, nbh, 0, 1, 0, 1);
    e = cudaGetLastError();
    if (e != cudaSuccess) { c.err = cudaGetErrorString(e); return EXFEM_E_CUDA; }
    c.launches += 4 + (m.ns > 0 ? 1 : 0);
    return EXFEM_OK;
}
