// exfem_f32.cu — FP32 increment form with Kahan-compensated state.
//
// The central-difference update of explicit.f90:135-148,
//   (a1 M + a2 C) u+ = f - K u + 2 a1 M u - a1 M u- + a2 C u-,
// rewritten for the increment D = u - u- (exact algebra):
//   D+ = D + delta,  delta = (f - K u - 2 a2 C D) / m_full,   u+ = u + D+.
// delta holds only the small physical terms, so FP32 keeps its relative
// precision; D and u are each accumulated with a Kahan compensation term
// (true value = hi - comp).  Without the compensation on D its rounding
// random-walks (about sqrt(steps) * 2^-24 of the peak); the compensations are
// stored as bf16 (FP32's exponent range, 8 extra bits), so the state stays at
// 12 bytes per dof: u_hi 4 + u_comp 2 + D 4 + D_comp 2.
// Anchors of hanging nodes add half of each hanging node's term
// (sum_reactanchors, halving form); in the increment form that carries
// D_h ((u_b - u_a)/2 + (D_h - D_a)) because the hanging node's mass acts on
// its own displacement and increment.  Templates, masses, dashpots, hanging
// weights and dt stay FP64 on the host and are rounded once.
//
// One step is three kernels:
//   k_drm32    DRM effective forces in FP64, stored FP32
//   k_step32   per (non-hanging node, group of right-hand sides): gather the
//              closed-form Q4 forces of its elements from u_hi, the DRM terms,
//              the dashpot and anchor terms, update D and u (fused; no
//              element buffer)
//   k_hang32   hanging nodes = anchor averages; receivers in FP64
// State layout: value (node n, dof d, rhs r) at (n*2 + d)*R + r, so a warp
// reads R contiguous values per (node, dof) and one set of mesh metadata
// serves every right-hand side.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "exfem_ctx.h"
#include "exfem_device.cuh"

namespace exfem {

namespace {

#define CK(call)                                                                  \
    do {                                                                          \
        cudaError_t e_ = (call);                                                  \
        if (e_ != cudaSuccess) {                                                  \
            c.err = std::string(#call) + ": " + cudaGetErrorString(e_);           \
            return EXFEM_E_CUDA;                                                  \
        }                                                                         \
    } while (0)

template <int N>
struct Vec;
template <>
struct Vec<1> {
    using T = float;
    __device__ static void load(const float *p, float *v) { v[0] = __ldg(p); }
    __device__ static void load_cg(const float *p, float *v) { v[0] = *p; }
    __device__ static void store(float *p, const float *v) { *p = v[0]; }
};
template <>
struct Vec<2> {
    __device__ static void load(const float *p, float *v) {
        float2 a = __ldg(reinterpret_cast<const float2 *>(p));
        v[0] = a.x; v[1] = a.y;
    }
    __device__ static void load_cg(const float *p, float *v) {
        float2 a = *reinterpret_cast<const float2 *>(p);
        v[0] = a.x; v[1] = a.y;
    }
    __device__ static void store(float *p, const float *v) { *reinterpret_cast<float2 *>(p) = make_float2(v[0], v[1]); }
};
template <>
struct Vec<4> {
    __device__ static void load(const float *p, float *v) {
        float4 a = __ldg(reinterpret_cast<const float4 *>(p));
        v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w;
    }
    __device__ static void load_cg(const float *p, float *v) {
        float4 a = *reinterpret_cast<const float4 *>(p);
        v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w;
    }
    __device__ static void store(float *p, const float *v) {
        *reinterpret_cast<float4 *>(p) = make_float4(v[0], v[1], v[2], v[3]);
    }
};

// RPT floats from shared memory.
template <int N>
struct VecS;
template <>
struct VecS<1> {
    __device__ static void load(const float *p, float *v) { v[0] = *p; }
};
template <>
struct VecS<2> {
    __device__ static void load(const float *p, float *v) {
        float2 a = *reinterpret_cast<const float2 *>(p);
        v[0] = a.x; v[1] = a.y;
    }
};
template <>
struct VecS<4> {
    __device__ static void load(const float *p, float *v) {
        float4 a = *reinterpret_cast<const float4 *>(p);
        v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w;
    }
};

// RPT bf16 values (raw 16-bit words) <-> float.
template <int N>
struct Half;
template <>
struct Half<1> {
    __device__ static void load(const unsigned short *p, float *v) {
        v[0] = __bfloat162float(__ushort_as_bfloat16(*p));
    }
    __device__ static void store(unsigned short *p, const float *v) {
        *p = __bfloat16_as_ushort(__float2bfloat16_rn(v[0]));
    }
};
template <>
struct Half<2> {
    __device__ static void load(const unsigned short *p, float *v) {
        unsigned w = *reinterpret_cast<const unsigned *>(p);
        v[0] = __bfloat162float(__ushort_as_bfloat16((unsigned short)(w & 0xffffu)));
        v[1] = __bfloat162float(__ushort_as_bfloat16((unsigned short)(w >> 16)));
    }
    __device__ static void store(unsigned short *p, const float *v) {
        unsigned lo = __bfloat16_as_ushort(__float2bfloat16_rn(v[0]));
        unsigned hi = __bfloat16_as_ushort(__float2bfloat16_rn(v[1]));
        *reinterpret_cast<unsigned *>(p) = lo | (hi << 16);
    }
};
template <>
struct Half<4> {
    __device__ static void load(const unsigned short *p, float *v) {
        uint2 w = *reinterpret_cast<const uint2 *>(p);
        v[0] = __bfloat162float(__ushort_as_bfloat16((unsigned short)(w.x & 0xffffu)));
        v[1] = __bfloat162float(__ushort_as_bfloat16((unsigned short)(w.x >> 16)));
        v[2] = __bfloat162float(__ushort_as_bfloat16((unsigned short)(w.y & 0xffffu)));
        v[3] = __bfloat162float(__ushort_as_bfloat16((unsigned short)(w.y >> 16)));
    }
    __device__ static void store(unsigned short *p, const float *v) {
        unsigned a = __bfloat16_as_ushort(__float2bfloat16_rn(v[0]));
        unsigned b = __bfloat16_as_ushort(__float2bfloat16_rn(v[1]));
        unsigned c = __bfloat16_as_ushort(__float2bfloat16_rn(v[2]));
        unsigned d = __bfloat16_as_ushort(__float2bfloat16_rn(v[3]));
        *reinterpret_cast<uint2 *>(p) = make_uint2(a | (b << 16), c | (d << 16));
    }
};

__device__ __forceinline__ float bf2f(unsigned short h) { return __bfloat162float(__ushort_as_bfloat16(h)); }
__device__ __forceinline__ unsigned short f2bf(float f) { return __bfloat16_as_ushort(__float2bfloat16_rn(f)); }

__device__ __forceinline__ int read_step(const DevModel &m) { return *(volatile int *)m.d_step; }

// DRM forces (model.f90:745-800) for the FP32 form: travel times in FP64,
// the Ricker terms and the boundary/exterior split in FP32.
__global__ void k_drm32(DevModel m) {
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)m.ns * m.R) return;
    int s = (int)(t / m.R), r = (int)(t % m.R);
    int step = read_step(m) + 1;
    const DevWave &w = m.waves[r];
    double outt = (double)step * m.dt - w.t0;
    int ie = m.s_elem[s];
    float u0[8], a0[8];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        int x = m.econn[4 * ie + k];
        planewave32(w, outt, m.nxy[2 * x] - m.worigin_x, m.nxy[2 * x + 1] - m.worigin_y, &u0[2 * k], &a0[2 * k]);
    }
    const float4 k4 = reinterpret_cast<const float4 *>(m.ecoef32)[ie];
    float kc[4] = {k4.x, k4.y, k4.z, k4.w};
    float p[8];
    drm_forces<float>(kc, (float)m.emass[ie], drm_mask(m.s_kind[s]), u0, a0, p);
#pragma unroll
    for (int k = 0; k < 8; ++k) m.fdrm32[((size_t)s * 8 + k) * m.R + r] = p[k];
}

// The fused step for one non-hanging node and RPT right-hand sides.
template <int RPT>
__global__ void __launch_bounds__(512) k_step32(DevModel m, const float *__restrict__ uh, float *__restrict__ uhn,
                                                unsigned short *__restrict__ uc, float *__restrict__ dh,
                                                unsigned short *__restrict__ dc) {
    const int G = m.R / RPT;
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)m.n_active * G) return;
    const int n = (int)(t / G);
    const int r0 = (int)(t % G) * RPT;
    const size_t R = m.R;
    const size_t bn = ((size_t)n * 2) * R + r0;
    // Ask L2 for this node's own streaming state (read only after the
    // gather) so its DRAM latency overlaps the gather instead of following
    // it.  Measured on the 64-RHS valley: 8% faster at 4 and 1 right-hand
    // sides per thread, slower at 2, where it is left out.
    if (RPT != 2) {
        asm volatile("prefetch.global.L2 [%0];" ::"l"(dh + bn));
        asm volatile("prefetch.global.L2 [%0];" ::"l"(dh + bn + R));
        asm volatile("prefetch.global.L2 [%0];" ::"l"(dc + bn));
        asm volatile("prefetch.global.L2 [%0];" ::"l"(dc + bn + R));
        asm volatile("prefetch.global.L2 [%0];" ::"l"(uc + bn));
        asm volatile("prefetch.global.L2 [%0];" ::"l"(uc + bn + R));
        asm volatile("prefetch.global.L2 [%0];" ::"l"(uh + bn));
        asm volatile("prefetch.global.L2 [%0];" ::"l"(uh + bn + R));
    }
    float ax[RPT], ay[RPT];
#pragma unroll
    for (int j = 0; j < RPT; ++j) { ax[j] = 0.f; ay[j] = 0.f; }
    // DRM terms (hanging corners at half weight in their anchors)
    for (int q = m.dptr[n]; q < m.dptr[n + 1]; ++q) {
        int ent = __ldg(m.dlist + q);
        float w = (ent & 1) ? 0.5f : 1.0f;
        int sc = ent >> 1;
        size_t b = ((size_t)(sc >> 2) * 8 + 2 * (sc & 3)) * R + r0;
        float fx[RPT], fy[RPT];
        Vec<RPT>::load_cg(m.fdrm32 + b, fx);
        Vec<RPT>::load_cg(m.fdrm32 + b + R, fy);
#pragma unroll
        for (int j = 0; j < RPT; ++j) { ax[j] += w * fx[j]; ay[j] += w * fy[j]; }
    }
    // element terms: -K_e u_e at this node's corner (and its hanging nodes' at 1/2)
    const int4 *econn4 = reinterpret_cast<const int4 *>(m.econn);
    const float4 *coef4 = reinterpret_cast<const float4 *>(m.ecoef32);
    for (int q = m.tptr[n]; q < m.tptr[n + 1]; ++q) {
        int ent = __ldg(m.tlist + q);
        float w = (ent & 1) ? 0.5f : 1.0f;
        int ec = ent >> 1;
        int e = ec >> 2, c = ec & 3;
        int4 cn = __ldg(econn4 + e);
        float4 k = __ldg(coef4 + e);
        const int cc[4] = {cn.x, cn.y, cn.z, cn.w};
        float ux[4][RPT], uy[4][RPT];
#pragma unroll
        for (int v = 0; v < 4; ++v) {
            size_t b = ((size_t)cc[v] * 2) * R + r0;
            Vec<RPT>::load(uh + b, ux[v]);
            Vec<RPT>::load(uh + b + R, uy[v]);
        }
#pragma unroll
        for (int j = 0; j < RPT; ++j) {
            float vx[4] = {ux[0][j], ux[1][j], ux[2][j], ux[3][j]};
            float vy[4] = {uy[0][j], uy[1][j], uy[2][j], uy[3][j]};
            float fx, fy;
            q4_ku_corner<float>(k.x, k.y, k.z, k.w, vx, vy, c, fx, fy);
            ax[j] -= w * fx;
            ay[j] -= w * fy;
        }
    }
    // dashpot term -2 a2 C D (zero away from the absorbing boundary)
    const float4 nc = __ldg(reinterpret_cast<const float4 *>(m.ncoef4) + n);
    float dx[RPT], dy[RPT];
    Vec<RPT>::load_cg(dh + bn, dx);
    Vec<RPT>::load_cg(dh + bn + R, dy);
    if (nc.z != 0.f || nc.w != 0.f) {
#pragma unroll
        for (int j = 0; j < RPT; ++j) { ax[j] += nc.z * dx[j]; ay[j] += nc.w * dy[j]; }
    }
    float unx[RPT], uny[RPT];
    Vec<RPT>::load(uh + bn, unx);
    Vec<RPT>::load(uh + bn + R, uny);
    // hanging nodes this node anchors:
    //   1/2 [ -2 a2 C_h D_h + D_h,mass ((u_b - u_n)/2 + (D_h - D_n)) ]
    // (D_b - D_n = 2 (D_h - D_n); D_h is read instead of D_b because the
    // other anchor's thread rewrites D_b in place during this kernel, while
    // D_h changes only in k_hang32)
    for (int q = m.lptr[n]; q < m.lptr[n + 1]; ++q) {
        int h = __ldg(m.llist + 2 * q), b = __ldg(m.llist + 2 * q + 1);
        float4 hc = __ldg(reinterpret_cast<const float4 *>(m.hcoef4) + (h - m.n_active));
        size_t bh = ((size_t)h * 2) * R + r0, bb = ((size_t)b * 2) * R + r0;
        float hx[RPT], hy[RPT], ubx[RPT], uby[RPT];
        Vec<RPT>::load_cg(dh + bh, hx);
        Vec<RPT>::load_cg(dh + bh + R, hy);
        Vec<RPT>::load(uh + bb, ubx);
        Vec<RPT>::load(uh + bb + R, uby);
#pragma unroll
        for (int j = 0; j < RPT; ++j) {
            ax[j] += 0.5f * (hc.x * hx[j] + hc.z * (0.5f * (ubx[j] - unx[j]) + (hx[j] - dx[j])));
            ay[j] += 0.5f * (hc.y * hy[j] + hc.w * (0.5f * (uby[j] - uny[j]) + (hy[j] - dy[j])));
        }
    }
    // delta = r / m_full; D+ = D + delta and u+ = u + D+, both Kahan-compensated
    float dcx[RPT], dcy[RPT], ucx[RPT], ucy[RPT], ox[RPT], oy[RPT];
    Half<RPT>::load(dc + bn, dcx);
    Half<RPT>::load(dc + bn + R, dcy);
    Half<RPT>::load(uc + bn, ucx);
    Half<RPT>::load(uc + bn + R, ucy);
#pragma unroll
    for (int j = 0; j < RPT; ++j) {
        float yx = ax[j] * nc.x - dcx[j], yy = ay[j] * nc.y - dcy[j];
        float tx = dx[j] + yx, ty = dy[j] + yy;
        dcx[j] = (tx - dx[j]) - yx;
        dcy[j] = (ty - dy[j]) - yy;
        dx[j] = tx;
        dy[j] = ty;
        float vx = tx - ucx[j], vy = ty - ucy[j];
        float sx = unx[j] + vx, sy = uny[j] + vy;
        ucx[j] = (sx - unx[j]) - vx;
        ucy[j] = (sy - uny[j]) - vy;
        ox[j] = sx;
        oy[j] = sy;
    }
    Vec<RPT>::store(dh + bn, dx);
    Vec<RPT>::store(dh + bn + R, dy);
    Half<RPT>::store(dc + bn, dcx);
    Half<RPT>::store(dc + bn + R, dcy);
    Half<RPT>::store(uc + bn, ucx);
    Half<RPT>::store(uc + bn + R, ucy);
    Vec<RPT>::store(uhn + bn, ox);
    Vec<RPT>::store(uhn + bn + R, oy);
}

// Tiled variant of k_step32: a block owns `tn` consecutive active nodes (a
// compact Morton patch) and a chunk of `rc` right-hand sides.  It first copies
// the u_hi rows of the patch's halo (every node its terms read) into shared
// memory with coalesced vector loads, then each thread gathers its element
// terms from shared memory through the host-computed halo slots.  The update
// itself is the one of k_step32.
struct TileArgs {
    const int *hptr, *hlist, *nslot, *lslot;
    const unsigned short *tslot;
    int tn, rc;
};

template <int RPT>
__global__ void __launch_bounds__(512) k_tile32(DevModel m, TileArgs ta, const float *__restrict__ uh,
                                                float *__restrict__ uhn, unsigned short *__restrict__ uc,
                                                float *__restrict__ dh, unsigned short *__restrict__ dc) {
    extern __shared__ float sm[];
    const int RC = ta.rc, G = RC / RPT, row = 2 * RC;
    const int tile = blockIdx.x, rbase = blockIdx.y * RC;
    const int h0 = ta.hptr[tile], nhalo = ta.hptr[tile + 1] - h0;
    const size_t R = m.R;
    const int ln = threadIdx.x / G, g = threadIdx.x - (threadIdx.x / G) * G;
    const int n = tile * ta.tn + ln;
    const bool valid = (ln < ta.tn) && (n < m.n_active);
    const int rl = g * RPT, r0 = rbase + rl;
    const size_t bn = ((size_t)n * 2) * R + r0;
    if (valid && RPT != 2) {   // the node's own streaming state, as in k_step32
        asm volatile("prefetch.global.L2 [%0];" ::"l"(dh + bn));
        asm volatile("prefetch.global.L2 [%0];" ::"l"(dh + bn + R));
        asm volatile("prefetch.global.L2 [%0];" ::"l"(dc + bn));
        asm volatile("prefetch.global.L2 [%0];" ::"l"(dc + bn + R));
        asm volatile("prefetch.global.L2 [%0];" ::"l"(uc + bn));
        asm volatile("prefetch.global.L2 [%0];" ::"l"(uc + bn + R));
    }
    // halo rows -> shared memory
    if ((RC & 3) == 0) {
        const int per = row >> 2;
        for (int i = threadIdx.x; i < nhalo * per; i += blockDim.x) {
            int h = i / per, k = (i - h * per) << 2;
            int d = k >= RC ? 1 : 0, rr = k - d * RC;
            float4 v = __ldg(reinterpret_cast<const float4 *>(uh + ((size_t)__ldg(ta.hlist + h0 + h) * 2 + d) * R + rbase + rr));
            *reinterpret_cast<float4 *>(sm + h * row + k) = v;
        }
    } else {
        for (int i = threadIdx.x; i < nhalo * row; i += blockDim.x) {
            int h = i / row, k = i - h * row;
            int d = k >= RC ? 1 : 0, rr = k - d * RC;
            sm[h * row + k] = __ldg(uh + ((size_t)__ldg(ta.hlist + h0 + h) * 2 + d) * R + rbase + rr);
        }
    }
    __syncthreads();
    if (!valid) return;
    float ax[RPT], ay[RPT];
#pragma unroll
    for (int j = 0; j < RPT; ++j) { ax[j] = 0.f; ay[j] = 0.f; }
    for (int q = m.dptr[n]; q < m.dptr[n + 1]; ++q) {
        int ent = __ldg(m.dlist + q);
        float w = (ent & 1) ? 0.5f : 1.0f;
        int sc = ent >> 1;
        size_t b = ((size_t)(sc >> 2) * 8 + 2 * (sc & 3)) * R + r0;
        float fx[RPT], fy[RPT];
        Vec<RPT>::load_cg(m.fdrm32 + b, fx);
        Vec<RPT>::load_cg(m.fdrm32 + b + R, fy);
#pragma unroll
        for (int j = 0; j < RPT; ++j) { ax[j] += w * fx[j]; ay[j] += w * fy[j]; }
    }
    const float4 *coef4 = reinterpret_cast<const float4 *>(m.ecoef32);
    const ushort4 *slots = reinterpret_cast<const ushort4 *>(ta.tslot);
    for (int q = m.tptr[n]; q < m.tptr[n + 1]; ++q) {
        int ent = __ldg(m.tlist + q);
        float w = (ent & 1) ? 0.5f : 1.0f;
        int ec = ent >> 1;
        int e = ec >> 2, c = ec & 3;
        float4 k = __ldg(coef4 + e);
        ushort4 sl = __ldg(slots + q);
        const int ss[4] = {sl.x, sl.y, sl.z, sl.w};
        float ux[4][RPT], uy[4][RPT];
#pragma unroll
        for (int v = 0; v < 4; ++v) {
            VecS<RPT>::load(sm + ss[v] * row + rl, ux[v]);
            VecS<RPT>::load(sm + ss[v] * row + RC + rl, uy[v]);
        }
#pragma unroll
        for (int j = 0; j < RPT; ++j) {
            float vx[4] = {ux[0][j], ux[1][j], ux[2][j], ux[3][j]};
            float vy[4] = {uy[0][j], uy[1][j], uy[2][j], uy[3][j]};
            float fx, fy;
            q4_ku_corner<float>(k.x, k.y, k.z, k.w, vx, vy, c, fx, fy);
            ax[j] -= w * fx;
            ay[j] -= w * fy;
        }
    }
    const float4 nc = __ldg(reinterpret_cast<const float4 *>(m.ncoef4) + n);
    float dx[RPT], dy[RPT];
    Vec<RPT>::load_cg(dh + bn, dx);
    Vec<RPT>::load_cg(dh + bn + R, dy);
    if (nc.z != 0.f || nc.w != 0.f) {
#pragma unroll
        for (int j = 0; j < RPT; ++j) { ax[j] += nc.z * dx[j]; ay[j] += nc.w * dy[j]; }
    }
    const int ns_ = __ldg(ta.nslot + n);
    float unx[RPT], uny[RPT];
    VecS<RPT>::load(sm + ns_ * row + rl, unx);
    VecS<RPT>::load(sm + ns_ * row + RC + rl, uny);
    for (int q = m.lptr[n]; q < m.lptr[n + 1]; ++q) {
        int h = __ldg(m.llist + 2 * q);
        int sb = __ldg(ta.lslot + q);
        float4 hc = __ldg(reinterpret_cast<const float4 *>(m.hcoef4) + (h - m.n_active));
        size_t bh = ((size_t)h * 2) * R + r0;
        float hx[RPT], hy[RPT], ubx[RPT], uby[RPT];
        Vec<RPT>::load_cg(dh + bh, hx);
        Vec<RPT>::load_cg(dh + bh + R, hy);
        VecS<RPT>::load(sm + sb * row + rl, ubx);
        VecS<RPT>::load(sm + sb * row + RC + rl, uby);
#pragma unroll
        for (int j = 0; j < RPT; ++j) {
            ax[j] += 0.5f * (hc.x * hx[j] + hc.z * (0.5f * (ubx[j] - unx[j]) + (hx[j] - dx[j])));
            ay[j] += 0.5f * (hc.y * hy[j] + hc.w * (0.5f * (uby[j] - uny[j]) + (hy[j] - dy[j])));
        }
    }
    float dcx[RPT], dcy[RPT], ucx[RPT], ucy[RPT], ox[RPT], oy[RPT];
    Half<RPT>::load(dc + bn, dcx);
    Half<RPT>::load(dc + bn + R, dcy);
    Half<RPT>::load(uc + bn, ucx);
    Half<RPT>::load(uc + bn + R, ucy);
#pragma unroll
    for (int j = 0; j < RPT; ++j) {
        float yx = ax[j] * nc.x - dcx[j], yy = ay[j] * nc.y - dcy[j];
        float tx = dx[j] + yx, ty = dy[j] + yy;
        dcx[j] = (tx - dx[j]) - yx;
        dcy[j] = (ty - dy[j]) - yy;
        dx[j] = tx;
        dy[j] = ty;
        float vx = tx - ucx[j], vy = ty - ucy[j];
        float sx = unx[j] + vx, sy = uny[j] + vy;
        ucx[j] = (sx - unx[j]) - vx;
        ucy[j] = (sy - uny[j]) - vy;
        ox[j] = sx;
        oy[j] = sy;
    }
    Vec<RPT>::store(dh + bn, dx);
    Vec<RPT>::store(dh + bn + R, dy);
    Half<RPT>::store(dc + bn, dcx);
    Half<RPT>::store(dc + bn + R, dcy);
    Half<RPT>::store(uc + bn, ucx);
    Half<RPT>::store(uc + bn + R, ucy);
    Vec<RPT>::store(uhn + bn, ox);
    Vec<RPT>::store(uhn + bn + R, oy);
}

// u of one node in FP64 (u_hi - comp); hanging corners read as anchor averages.
__device__ __forceinline__ void load_u32(const DevModel &m, const float *uh, const unsigned short *uc, int node,
                                         int r, double &vx, double &vy) {
    const size_t R = m.R;
    auto val = [&](int x, int d) {
        size_t i = ((size_t)x * 2 + d) * R + r;
        return (double)uh[i] - (double)bf2f(uc[i]);
    };
    if (node < m.n_active) {
        vx = val(node, 0);
        vy = val(node, 1);
    } else {
        int i = node - m.n_active;
        int a = m.hang[3 * i + 1], b = m.hang[3 * i + 2];
        vx = (val(a, 0) + val(b, 0)) / 2.0;
        vy = (val(a, 1) + val(b, 1)) / 2.0;
    }
}

// Hanging nodes (anchor averages of u_hi, comp and D) and receivers.
__global__ void __launch_bounds__(256) k_hang32(DevModel m, float *__restrict__ uhn,
                                                unsigned short *__restrict__ uc, float *__restrict__ dh,
                                                unsigned short *__restrict__ dc, int nb_hang, int mode) {
    int step = (mode == 1) ? 0 : read_step(m) + 1;
    const size_t R = m.R;
    if ((int)blockIdx.x < nb_hang) {
        long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
        if (mode == 0 && t < (long long)m.n_hang * m.R) {
            int i = (int)(t / m.R), r = (int)(t % m.R);
            int h = m.hang[3 * i], a = m.hang[3 * i + 1], b = m.hang[3 * i + 2];
#pragma unroll
            for (int d = 0; d < 2; ++d) {
                size_t ih = ((size_t)h * 2 + d) * R + r, ia = ((size_t)a * 2 + d) * R + r,
                       ib = ((size_t)b * 2 + d) * R + r;
                uhn[ih] = 0.5f * (uhn[ia] + uhn[ib]);
                uc[ih] = f2bf(0.5f * (bf2f(uc[ia]) + bf2f(uc[ib])));
                dh[ih] = 0.5f * (dh[ia] + dh[ib]);
                dc[ih] = f2bf(0.5f * (bf2f(dc[ia]) + bf2f(dc[ib])));
            }
        }
    } else if (step % m.io == 0) {
        long long t = (long long)(blockIdx.x - nb_hang) * blockDim.x + threadIdx.x;
        if (t < (long long)m.nrecv * m.R) {
            int i = (int)(t % m.nrecv), r = (int)(t / m.nrecv);
            int slot = step / m.io;
            double fx = 0.0, fy = 0.0;
            for (int k = 0; k < 4; ++k) {
                double vx, vy;
                load_u32(m, uhn, uc, m.rnode[4 * i + k], r, vx, vy);
                double w = m.rw[4 * i + k];
                fx += w * vx;
                fy += w * vy;
            }
            if (m.rsoil[i]) {
                const DevWave wv = m.waves[r];
                double time = m.dt * (double)slot * (double)m.io;
                double ddx, ddz;
                planewave_u(wv, time - wv.t0, m.rxy[2 * i] - m.worigin_x, m.rxy[2 * i + 1] - m.worigin_y, ddx, ddz);
                fx += ddx;
                fy += ddz;
            }
            size_t o = (((size_t)r * m.nsave + slot) * m.nrecv + i) * 2;
            m.seis[o] = fx;
            m.seis[o + 1] = fy;
            if (!isfinite(fx) || !isfinite(fy)) atomicOr(m.d_flag, 1);
        }
    }
    if (mode == 0) {   // the last block advances the device step counter
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

template <typename T>
int upload32(Ctx &c, const std::vector<T> &v, const T **dst) {
    if (v.empty()) { *dst = nullptr; return EXFEM_OK; }
    void *p = nullptr;
    CK(cudaMalloc(&p, v.size() * sizeof(T)));
    c.allocs.push_back(p);
    c.bytes += v.size() * sizeof(T);
    CK(cudaMemcpyAsync(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, c.stream));
    *dst = static_cast<const T *>(p);
    return EXFEM_OK;
}

template <typename T>
int alloc32(Ctx &c, size_t n, T **dst) {
    void *p = nullptr;
    if (n == 0) n = 1;
    CK(cudaMalloc(&p, n * sizeof(T)));
    c.allocs.push_back(p);
    c.bytes += n * sizeof(T);
    *dst = static_cast<T *>(p);
    return EXFEM_OK;
}

}  // namespace

// Right-hand sides per thread: the largest of 4, 2, 1 dividing R (or the
// requested one when it divides R).
static int pick_rpt(const Ctx &c) {
    int R = c.plan.R;
    int want = c.opts.rhs_per_thread;
    if (want == 1 || want == 2 || want == 4) return (R % want == 0) ? want : 1;
    if (R % 4 == 0 && R >= 32) return 4;
    if (R % 2 == 0 && R >= 16) return 2;
    return 1;
}

int f32_alloc(Ctx &c) {
    const Plan &P = c.plan;
    DevModel &m = c.dm;
    // per active node: 1/m_full (x, y), -2 a2 C (x, y)
    std::vector<float> nc((size_t)4 * P.n_active);
    for (int n = 0; n < P.n_active; ++n) {
        nc[4 * (size_t)n] = (float)P.inv_mfull[2 * (size_t)n];
        nc[4 * (size_t)n + 1] = (float)P.inv_mfull[2 * (size_t)n + 1];
        nc[4 * (size_t)n + 2] = (float)(-2.0 * P.a2 * P.ndamp[2 * (size_t)n]);
        nc[4 * (size_t)n + 3] = (float)(-2.0 * P.a2 * P.ndamp[2 * (size_t)n + 1]);
    }
    std::vector<float> hc((size_t)4 * std::max(P.n_hang, 1), 0.f);
    for (int i = 0; i < P.n_hang; ++i) {
        int h = P.hang[3 * (size_t)i];
        hc[4 * (size_t)i] = (float)(-2.0 * P.a2 * P.ndamp[2 * (size_t)h]);
        hc[4 * (size_t)i + 1] = (float)(-2.0 * P.a2 * P.ndamp[2 * (size_t)h + 1]);
        hc[4 * (size_t)i + 2] = (float)(P.a1 * P.nmass[h] + P.a2 * P.ndamp[2 * (size_t)h]);
        hc[4 * (size_t)i + 3] = (float)(P.a1 * P.nmass[h] + P.a2 * P.ndamp[2 * (size_t)h + 1]);
    }
    int rc;
    if ((rc = upload32(c, nc, &m.ncoef4))) return rc;
    if ((rc = upload32(c, hc, &m.hcoef4))) return rc;
    if ((rc = upload32(c, P.ecoef32, &m.ecoef32))) return rc;
    if ((rc = alloc32(c, (size_t)std::max(m.ns, 1) * 8 * P.R, &m.fdrm32))) return rc;
    size_t nst = (size_t)P.nn * 2 * P.R;
    if ((rc = alloc32(c, nst, &c.uhi[0]))) return rc;
    if ((rc = alloc32(c, nst, &c.uhi[1]))) return rc;
    if ((rc = alloc32(c, nst, &c.ucomp))) return rc;
    if ((rc = alloc32(c, nst, &c.udel[0]))) return rc;
    if ((rc = alloc32(c, nst, &c.dcomp))) return rc;
    c.rhs_per_thread = pick_rpt(c);
    if (c.opts.block_threads <= 0) c.block_threads = 256;
    // shared-memory tiles (variant 1; variant 0, the default, is the direct gather)
    c.use_tiles = false;
    if (c.opts.variant == 1) {
        const int R = P.R, rpt = c.rhs_per_thread;
        const int chunk = R <= 64 ? R : ((R % 64 == 0) ? 64 : 0);
        if (chunk > 0 && chunk % rpt == 0) {
            int G = chunk / rpt;
            int tn = std::max(1, c.block_threads / G);
            Tiles T;
            std::string terr;
            if (build_tiles(P, tn, T, terr) == EXFEM_OK) {
                size_t smem = (size_t)T.hmax * 2 * chunk * sizeof(float);
                int dev_smem = 0;
                cudaDeviceGetAttribute(&dev_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, c.device);
                if (smem <= (size_t)dev_smem && tn * G <= 512) {
                    if ((rc = upload32(c, T.hptr, &c.t_hptr)) ||
                        (rc = upload32(c, T.hlist, &c.t_hlist)) ||
                        (rc = upload32(c, T.tslot, &c.t_tslot)) ||
                        (rc = upload32(c, T.nslot, &c.t_nslot)))
                        return rc;
                    if (!T.lslot.empty() && (rc = upload32(c, T.lslot, &c.t_lslot))) return rc;
                    c.tile_tn = tn;
                    c.tile_n = T.ntiles;
                    c.tile_hmax = T.hmax;
                    c.tile_rc = chunk;
                    c.tile_smem = smem;
                    c.use_tiles = true;
                    CK(cudaFuncSetAttribute(k_tile32<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
                    CK(cudaFuncSetAttribute(k_tile32<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
                    CK(cudaFuncSetAttribute(k_tile32<4>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
                }
            }
        }
    }
    return EXFEM_OK;
}

int f32_init(Ctx &c) {
    size_t nst = (size_t)c.plan.nn * 2 * c.plan.R;
    CK(cudaMemsetAsync(c.uhi[0], 0, nst * sizeof(float), c.stream));
    CK(cudaMemsetAsync(c.uhi[1], 0, nst * sizeof(float), c.stream));
    CK(cudaMemsetAsync(c.ucomp, 0, nst * sizeof(unsigned short), c.stream));
    CK(cudaMemsetAsync(c.udel[0], 0, nst * sizeof(float), c.stream));
    CK(cudaMemsetAsync(c.dcomp, 0, nst * sizeof(unsigned short), c.stream));
    return EXFEM_OK;
}

int f32_launch_step(Ctx &c, int par) {
    DevModel &m = c.dm;
    float *uh = c.uhi[par], *uhn = c.uhi[par ^ 1];
    if (m.ns > 0) {
        k_drm32<<<nblocks((long long)m.ns * m.R, 64), 64, 0, c.stream>>>(m);
        c.launches++;
        mark(c, "k_drm32");
    }
    const int T = c.block_threads;
    const int rpt = c.rhs_per_thread;
    long long work = (long long)m.n_active * (m.R / rpt);
    if (c.use_tiles) {
        TileArgs ta{c.t_hptr, c.t_hlist, c.t_nslot, c.t_lslot, c.t_tslot, c.tile_tn, c.tile_rc};
        dim3 grid(c.tile_n, m.R / c.tile_rc);
        int threads = c.tile_tn * (c.tile_rc / rpt);
        switch (rpt) {
            case 4: k_tile32<4><<<grid, threads, c.tile_smem, c.stream>>>(m, ta, uh, uhn, c.ucomp, c.udel[0], c.dcomp); break;
            case 2: k_tile32<2><<<grid, threads, c.tile_smem, c.stream>>>(m, ta, uh, uhn, c.ucomp, c.udel[0], c.dcomp); break;
            default: k_tile32<1><<<grid, threads, c.tile_smem, c.stream>>>(m, ta, uh, uhn, c.ucomp, c.udel[0], c.dcomp); break;
        }
        c.launches++;
        mark(c, "k_tile32");
    } else {
    switch (rpt) {
        case 4: k_step32<4><<<nblocks(work, T), T, 0, c.stream>>>(m, uh, uhn, c.ucomp, c.udel[0], c.dcomp); break;
        case 2: k_step32<2><<<nblocks(work, T), T, 0, c.stream>>>(m, uh, uhn, c.ucomp, c.udel[0], c.dcomp); break;
        default: k_step32<1><<<nblocks(work, T), T, 0, c.stream>>>(m, uh, uhn, c.ucomp, c.udel[0], c.dcomp); break;
    }
    c.launches++;
    mark(c, "k_step32");
    }
    const int TH = 256;
    int nbh = (int)std::max<long long>(1, ((long long)m.n_hang * m.R + TH - 1) / TH);
    int nbr = (int)(((long long)m.nrecv * m.R + TH - 1) / TH);
    k_hang32<<<nbh + nbr, TH, 0, c.stream>>>(m, uhn, c.ucomp, c.udel[0], c.dcomp, nbh, 0);
    c.launches++;
    mark(c, "k_hang32");
    CK(cudaGetLastError());
    return EXFEM_OK;
}

int f32_launch_sample0(Ctx &c, int par) {
    DevModel &m = c.dm;
    const int TH = 256;
    int nbr = (int)(((long long)m.nrecv * m.R + TH - 1) / TH);
    if (nbr > 0) {
        k_hang32<<<nbr, TH, 0, c.stream>>>(m, c.uhi[par], c.ucomp, c.udel[0], c.dcomp, 0, 1);
        c.launches++;
    }
    CK(cudaGetLastError());
    return EXFEM_OK;
}

int f32_get_u(Ctx &c, int rhs, std::vector<double> &out) {
    const Plan &P = c.plan;
    size_t nst = (size_t)P.nn * 2 * P.R;
    std::vector<float> hi(nst);
    std::vector<unsigned short> co(nst);
    CK(cudaMemcpy(hi.data(), c.uhi[c.parity], nst * sizeof(float), cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(co.data(), c.ucomp, nst * sizeof(unsigned short), cudaMemcpyDeviceToHost));
    out.resize((size_t)P.nn * 2);
    for (int i = 0; i < P.nn; ++i)
        for (int d = 0; d < 2; ++d) {
            size_t k = ((size_t)i * 2 + d) * P.R + rhs;
            out[2 * (size_t)i + d] = (double)hi[k] - (double)bf16_to_float(co[k]);
        }
    return EXFEM_OK;
}

float bf16_to_float(unsigned short h) {
    unsigned w = (unsigned)h << 16;
    float f;
    std::memcpy(&f, &w, sizeof(f));
    return f;
}

}  // namespace exfem
