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
// D_h ((u_h - u_a) + (D_h - D_a)) because the hanging node's mass acts on
// its own displacement and increment (read from its row, which holds the
// anchor average after every step and a prescribed displacement at t = 0).  Templates, masses, dashpots, hanging
// weights and dt stay FP64 on the host and are rounded once.
//
// One step is two kernels (three with a point source):
//   k_step32   per (non-hanging node, group of right-hand sides): gather the
//              closed-form Q4 forces of its elements from u_hi, the DRM terms,
//              the dashpot and anchor terms, update D and u (fused; no
//              element buffer)
//   k_point32  (point sources) the source term at its nodes
//   k_hang32   hanging nodes = anchor averages; receivers in FP64; and the
//              next step's DRM effective forces (travel times FP64, stored
//              FP32), which depend on time only
// State layout: a node's 2R values are contiguous, so one set of mesh
// metadata serves every right-hand side.  Within them (row_off) the RHS form
// groups of m.lg, each group's x row, then its y row: lg = R (plain:
// (n*2 + d)*R + r), or lg = RHS per thread for the direct gather with
// several threads per node, whose x and y values then sit side by side.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <type_traits>
#include <vector>

#include "exfem_ctx.h"
#include "exfem_device.cuh"
#include "exfem_tc.cuh"

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

// Eight floats (a paired node row at four RHS per thread) as one 32-byte
// access; the address is 32-byte aligned.
template <>
struct Vec<8> {
    __device__ static void load(const float *p, float *v) {
        asm volatile("ld.global.nc.v8.f32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
                     : "=f"(v[0]), "=f"(v[1]), "=f"(v[2]), "=f"(v[3]), "=f"(v[4]), "=f"(v[5]), "=f"(v[6]), "=f"(v[7])
                     : "l"(p));
    }
    __device__ static void load_cg(const float *p, float *v) {
        asm volatile("ld.global.v8.f32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
                     : "=f"(v[0]), "=f"(v[1]), "=f"(v[2]), "=f"(v[3]), "=f"(v[4]), "=f"(v[5]), "=f"(v[6]), "=f"(v[7])
                     : "l"(p) : "memory");
    }
    __device__ static void store(float *p, const float *v) {
        asm volatile("st.global.v8.f32 [%0], {%1, %2, %3, %4, %5, %6, %7, %8};"
                     :: "l"(p), "f"(v[0]), "f"(v[1]), "f"(v[2]), "f"(v[3]), "f"(v[4]), "f"(v[5]), "f"(v[6]), "f"(v[7])
                     : "memory");
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

template <>
struct Half<8> {
    __device__ static void load(const unsigned short *p, float *v) {
        uint4 w = *reinterpret_cast<const uint4 *>(p);
        const unsigned u[4] = {w.x, w.y, w.z, w.w};
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            v[2 * k] = __bfloat162float(__ushort_as_bfloat16((unsigned short)(u[k] & 0xffffu)));
            v[2 * k + 1] = __bfloat162float(__ushort_as_bfloat16((unsigned short)(u[k] >> 16)));
        }
    }
    __device__ static void store(unsigned short *p, const float *v) {
        unsigned u[4];
#pragma unroll
        for (int k = 0; k < 4; ++k)
            u[k] = (unsigned)__bfloat16_as_ushort(__float2bfloat16_rn(v[2 * k])) |
                   ((unsigned)__bfloat16_as_ushort(__float2bfloat16_rn(v[2 * k + 1])) << 16);
        *reinterpret_cast<uint4 *>(p) = make_uint4(u[0], u[1], u[2], u[3]);
    }
};

// A thread's x and y values of a node (or of a DRM corner's force pair) for
// RPT right-hand sides: at p and p + R in the plain layout; PAIR: at p and
// p + RPT in the layout grouped by RPT (row_off), where they move as one
// vector of 2 RPT values (8, 16 or 32 bytes, aligned: p is a multiple of
// 2 RPT).
template <int RPT, bool PAIR>
struct XY {
    template <typename I>
    __device__ static void load(const float *p, I R, float *x, float *y) {
        if constexpr (PAIR) {
            float t[2 * RPT];
            Vec<2 * RPT>::load(p, t);
#pragma unroll
            for (int j = 0; j < RPT; ++j) { x[j] = t[j]; y[j] = t[RPT + j]; }
        } else {
            Vec<RPT>::load(p, x);
            Vec<RPT>::load(p + R, y);
        }
    }
    template <typename I>
    __device__ static void load_cg(const float *p, I R, float *x, float *y) {
        if constexpr (PAIR) {
            float t[2 * RPT];
            Vec<2 * RPT>::load_cg(p, t);
#pragma unroll
            for (int j = 0; j < RPT; ++j) { x[j] = t[j]; y[j] = t[RPT + j]; }
        } else {
            Vec<RPT>::load_cg(p, x);
            Vec<RPT>::load_cg(p + R, y);
        }
    }
    template <typename I>
    __device__ static void store(float *p, I R, const float *x, const float *y) {
        if constexpr (PAIR) {
            float t[2 * RPT];
#pragma unroll
            for (int j = 0; j < RPT; ++j) { t[j] = x[j]; t[RPT + j] = y[j]; }
            Vec<2 * RPT>::store(p, t);
        } else {
            Vec<RPT>::store(p, x);
            Vec<RPT>::store(p + R, y);
        }
    }
    template <typename I>
    __device__ static void load_half(const unsigned short *p, I R, float *x, float *y) {
        if constexpr (PAIR) {
            float t[2 * RPT];
            Half<2 * RPT>::load(p, t);
#pragma unroll
            for (int j = 0; j < RPT; ++j) { x[j] = t[j]; y[j] = t[RPT + j]; }
        } else {
            Half<RPT>::load(p, x);
            Half<RPT>::load(p + R, y);
        }
    }
    template <typename I>
    __device__ static void store_half(unsigned short *p, I R, const float *x, const float *y) {
        if constexpr (PAIR) {
            float t[2 * RPT];
#pragma unroll
            for (int j = 0; j < RPT; ++j) { t[j] = x[j]; t[RPT + j] = y[j]; }
            Half<2 * RPT>::store(p, t);
        } else {
            Half<RPT>::store(p, x);
            Half<RPT>::store(p + R, y);
        }
    }
};

__device__ __forceinline__ float bf2f(unsigned short h) { return __bfloat162float(__ushort_as_bfloat16(h)); }
__device__ __forceinline__ unsigned short f2bf(float f) { return __bfloat16_as_ushort(__float2bfloat16_rn(f)); }

__device__ __forceinline__ int read_step(const DevModel &m) { return *(volatile int *)m.d_step; }


// DRM forces (model.f90:745-800) of step `step` for the FP32 form: travel
// times in FP64, the Ricker terms and the boundary/exterior split in FP32.
// They depend on time only, so the hanging/receiver pass of step k computes
// those of step k + 1 in extra blocks of its own launch (and the step-0 sample
// those of step 1).  Four threads per (boundary element, rhs): thread k
// evaluates the free field at corner k, the quad shares the values, thread k
// stores forces 2k and 2k+1; block `b` holds items [b * ipb, (b + 1) * ipb)
// (ipb <= threads / 4, threads a multiple of 32).  Every thread of the block
// must call it (warp shuffles).
__device__ __forceinline__ void drm32_items(const DevModel &m, int ipb, long long b, int step) {
    const int li = threadIdx.x >> 2;
    const long long w = b * ipb + li;
    const int k = (int)(threadIdx.x & 3);
    const bool valid = li < ipb && w < (long long)m.ns * m.R;
    int s = 0, r = 0, ie = 0;
    float uk[2] = {0.f, 0.f}, ak[2] = {0.f, 0.f};
    if (valid) {
        s = (int)(w / m.R);
        r = (int)(w % m.R);
        const DevWave &wv = m.waves[r];
        double outt = (double)step * m.dt - wv.t0;
        ie = m.s_elem[s];
        const double *dl = m.drm_delay + ((size_t)s * 4 + k) * 3 * m.R + r;
        const double v[3] = {dl[0], dl[m.R], dl[2 * (size_t)m.R]};
        planewave32_at(wv, outt, v, uk, ak);
    }
    float u0[8], a0[8];
#pragma unroll
    for (int c = 0; c < 4; ++c) {
        u0[2 * c] = __shfl_sync(0xffffffffu, uk[0], c, 4);
        u0[2 * c + 1] = __shfl_sync(0xffffffffu, uk[1], c, 4);
        a0[2 * c] = __shfl_sync(0xffffffffu, ak[0], c, 4);
        a0[2 * c + 1] = __shfl_sync(0xffffffffu, ak[1], c, 4);
    }
    if (!valid) return;
    const float4 k4 = reinterpret_cast<const float4 *>(m.ecoef32)[ie];
    float kc[4] = {k4.x, k4.y, k4.z, k4.w};
    float p[8];
    drm_forces<float>(kc, (float)m.emass[ie], drm_mask(m.s_kind[s]), u0, a0, p);
    m.fdrm32[((size_t)s * 8 + 2 * k) * m.R + row_off(m, 0, r)] = p[2 * k];
    m.fdrm32[((size_t)s * 8 + 2 * k) * m.R + row_off(m, 1, r)] = p[2 * k + 1];
}

// The DRM forces of the step after the last one computed (the side-stream
// form): that step comes from the launch's own counter, which only these
// launches advance (they run in order on one stream), not from the step
// counter, which the main stream's hanging pass advances concurrently.
// Writes m.fdrm32 (the slot the caller picked); the last block advances the
// counter.
__global__ void __launch_bounds__(256) k_drm32(DevModel m, int ipb) {
    const int step = *(volatile int *)m.d_drm_step + 1;
    drm32_items(m, ipb, blockIdx.x, step);
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

// Per gather term, a copy of its element's four corners (the direct gather's
// tcorn), built on the device from the term list and the element corners
// rather than on the host and copied over: 16 bytes per term, 98 MB on the
// 64-RHS valley.
__global__ void k_term_corners(const int *__restrict__ tlist, const int *__restrict__ econn, int *__restrict__ tcorn,
                               long long nterms) {
    const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= nterms) return;
    const int e = (__ldg(tlist + q) >> 1) >> 2;
    reinterpret_cast<int4 *>(tcorn)[q] = __ldg(reinterpret_cast<const int4 *>(econn) + e);
}

// An element's four FP32 coefficients from its two stored values, with the
// operations and roundings of fp32_coef (exfem_plan.h).
__device__ __forceinline__ float4 coef_from2(float2 k2) {
    const float B = __fmul_rn(3.f, k2.x);
    return make_float4(__fadd_rn(B, __fmul_rn(2.f, k2.y)), B, k2.y, __fadd_rn(k2.x, k2.y));
}

// ecoef32 from ecoef2, once per context (8 bytes per element uploaded
// instead of 16).
__global__ void k_coef32(const float *__restrict__ ecoef2, float *__restrict__ ecoef32, int ne) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= ne) return;
    reinterpret_cast<float4 *>(ecoef32)[e] = coef_from2(reinterpret_cast<const float2 *>(ecoef2)[e]);
}

// The direct gather's node slot records (build_node_slots, in the same
// words): per active node its first four tlist entries (-1 past the last)
// and 1/m_full, or -1 on a node with more than four terms, DRM terms,
// anchored hanging nodes, a dashpot or unequal x and y coefficients.
__global__ void k_node_slots(const int *__restrict__ tptr, const int *__restrict__ tlist, const int *__restrict__ dptr,
                             const int *__restrict__ lptr, const float *__restrict__ ncoef4, int n_active,
                             int *__restrict__ slot4, float *__restrict__ invm) {
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= n_active) return;
    const int q0 = tptr[n], nt = tptr[n + 1] - q0;
    int4 s;
    s.x = nt > 0 ? tlist[q0] : -1;
    s.y = nt > 1 ? tlist[q0 + 1] : -1;
    s.z = nt > 2 ? tlist[q0 + 2] : -1;
    s.w = nt > 3 ? tlist[q0 + 3] : -1;
    reinterpret_cast<int4 *>(slot4)[n] = s;
    const float4 c = reinterpret_cast<const float4 *>(ncoef4)[n];
    const bool mark = nt > 4 || dptr[n + 1] > dptr[n] || lptr[n + 1] > lptr[n] || c.z != 0.f || c.w != 0.f ||
                      __float_as_uint(c.x) != __float_as_uint(c.y) || !(c.x > 0.f);
    invm[n] = mark ? -1.f : c.x;
}

// The slot form's corner copies: for slot j of active node n (an entry, or
// -1), the four corners of its element at tcorn4[4 * (4n + j)], from the slot
// records and the element corners (an empty slot gets -1s, never read).
__global__ void k_slot_corners(const int *__restrict__ slot4, const int *__restrict__ econn, int *__restrict__ tcorn4,
                               long long nslots) {
    const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= nslots) return;
    const int ent = __ldg(slot4 + q);
    reinterpret_cast<int4 *>(tcorn4)[q] =
        ent < 0 ? make_int4(-1, -1, -1, -1) : __ldg(reinterpret_cast<const int4 *>(econn) + ((ent >> 1) >> 2));
}

// Free-field delays of the DRM corners, once per context (see
// planewave32_delays): thread per (DRM element, corner, rhs).
__global__ void k_drm_delays32(DevModel m, double *__restrict__ out) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)m.ns * 4 * m.R) return;
    const int r = (int)(t % m.R);
    const long long sk = t / m.R;
    const int k = (int)(sk & 3), s = (int)(sk >> 2);
    const int x = m.econn[4 * m.s_elem[s] + k];
    double v[3];
    planewave32_delays(m.waves[r], m.nxy[2 * x] - m.worigin_x, m.nxy[2 * x + 1] - m.worigin_y, v);
    for (int q = 0; q < 3; ++q) out[((size_t)s * 4 + k) * 3 * m.R + (size_t)q * m.R + r] = v[q];
}

// The rest of a node's step once its DRM and element terms are in (ax, ay):
// the dashpot term, the hanging nodes it anchors, and the Kahan-compensated
// increment update of D and u (shared by the direct gather and the
// tensor-core step).
// SLOT: the node's record came from the fixed-size slots (build_node_slots):
// an unmarked node (invm > 0) has 1/m_full = invm in x and y, no dashpot and
// anchors no hanging node, so it reads neither ncoef4 nor the anchor list.
template <int RPT, bool PAIR, typename I, bool SLOT = false>
__device__ __forceinline__ void node_update(const DevModel &m, int n, I bn, I R, I roff, float (&ax)[RPT],
                                            float (&ay)[RPT], const float *__restrict__ uh,
                                            float *__restrict__ uhn, unsigned short *__restrict__ uc,
                                            float *__restrict__ dh, unsigned short *__restrict__ dc,
                                            float invm = -1.f) {
    // dashpot term -2 a2 C D (zero away from the absorbing boundary)
    const bool plain = SLOT && invm > 0.f;
    const float4 nc = plain ? make_float4(invm, invm, 0.f, 0.f) : __ldg(reinterpret_cast<const float4 *>(m.ncoef4) + n);
    float dx[RPT], dy[RPT];
    XY<RPT, PAIR>::load_cg(dh + bn, R, dx, dy);
    if (nc.z != 0.f || nc.w != 0.f) {
#pragma unroll
        for (int j = 0; j < RPT; ++j) { ax[j] += nc.z * dx[j]; ay[j] += nc.w * dy[j]; }
    }
    float unx[RPT], uny[RPT];
    XY<RPT, PAIR>::load(uh + bn, R, unx, uny);
    // hanging nodes this node anchors:
    //   1/2 [ -2 a2 C_h D_h + D_h,mass ((u_h - u_n) + (D_h - D_n)) ]
    // (u_h, D_h from the hanging node's rows, which change only in k_hang32;
    // the other anchor's row is rewritten in place during this kernel)
    for (int q = plain ? 0 : m.lptr[n]; q < (plain ? 0 : m.lptr[n + 1]); ++q) {
        int h = __ldg(m.llist + 2 * q);
        float4 hc = __ldg(reinterpret_cast<const float4 *>(m.hcoef4) + (h - m.n_active));
        I bh = ((I)h * 2) * R + roff;
        float hx[RPT], hy[RPT], uhx[RPT], uhy[RPT];
        XY<RPT, PAIR>::load_cg(dh + bh, R, hx, hy);
        XY<RPT, PAIR>::load(uh + bh, R, uhx, uhy);
#pragma unroll
        for (int j = 0; j < RPT; ++j) {
            ax[j] += 0.5f * (hc.x * hx[j] + hc.z * ((uhx[j] - unx[j]) + (hx[j] - dx[j])));
            ay[j] += 0.5f * (hc.y * hy[j] + hc.w * ((uhy[j] - uny[j]) + (hy[j] - dy[j])));
        }
    }
    // delta = r / m_full; D+ = D + delta and u+ = u + D+, both Kahan-compensated
    float dcx[RPT], dcy[RPT], ucx[RPT], ucy[RPT], ox[RPT], oy[RPT];
    XY<RPT, PAIR>::load_half(dc + bn, R, dcx, dcy);
    XY<RPT, PAIR>::load_half(uc + bn, R, ucx, ucy);
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
    XY<RPT, PAIR>::store(dh + bn, R, dx, dy);
    XY<RPT, PAIR>::store_half(dc + bn, R, dcx, dcy);
    XY<RPT, PAIR>::store_half(uc + bn, R, ucx, ucy);
    XY<RPT, PAIR>::store(uhn + bn, R, ox, oy);
}

// One element term of a node's gather: -K_e u_e at the node's corner c of
// element e (weight 1/2 for a hanging node's term carried by its anchor),
// ent = ((e*4 + c) << 1) | half, cn = the element's corners.
// k: the element's coefficients (ecoef32, or coef_from2 of ecoef2).
template <int RPT, bool PAIR, typename I>
__device__ __forceinline__ void gather_term(int ent, int4 cn, float4 k, I R, I roff, const float *__restrict__ uh,
                                            float (&ax)[RPT], float (&ay)[RPT]) {
    float w = (ent & 1) ? 0.5f : 1.0f;
    int c = (ent >> 1) & 3;
    const int cc[4] = {cn.x, cn.y, cn.z, cn.w};
    float ux[4][RPT], uy[4][RPT];
#pragma unroll
    for (int v = 0; v < 4; ++v) {
        I b = ((I)cc[v] * 2) * R + roff;
        XY<RPT, PAIR>::load(uh + b, R, ux[v], uy[v]);
    }
    const Q4Fold<float> f = q4_fold<float>(k.x, k.y, k.z, k.w, c, w);
#pragma unroll
    for (int j = 0; j < RPT; ++j) {
        float vx[4] = {ux[0][j], ux[1][j], ux[2][j], ux[3][j]};
        float vy[4] = {uy[0][j], uy[1][j], uy[2][j], uy[3][j]};
        q4_corner_acc<float>(f, vx, vy, ax[j], ay[j]);
    }
}

// The fused step for one non-hanging node and RPT right-hand sides.  The
// corners of each term's element come from the per-term copy m.tcorn, loaded
// beside the term itself (not from econn after it), so the gather chain is
// term -> corner u_hi.  I32: every thread id and array index fits in 32 bits
// (checked on the host), so the index arithmetic is 32-bit and a power-of-two
// thread count per node splits by shift and mask; this kernel is sensitive to
// its instruction count (64-bit indices cost 7% on the 64-RHS valley).
// TC: corners from the per-term copy m.tcorn (16 B per term) or, without it,
// from the element's econn entry after the term (a longer chain, but econn is
// shared by the element's four nodes through the caches); f32_term_corners
// picks by RHS count.
// PAIR: the state is grouped by RPT (m.lg == RPT, row_off; with RPT == R
// that is the plain layout), so the thread's x and y values of a node are
// adjacent and load and store as one vector (XY).
// SLOT: the node's first four terms and its 1/m_full come from its
// fixed-size slot record (m.tslot4, m.ninvm; build_node_slots), loaded with
// nothing before them, and with TC the corners of those terms from m.tcorn4
// (4 per node); only a marked node (invm < 0) reads its DRM list, its terms
// past the fourth (corners from econn), ncoef4 and its anchor list.  The terms
// are added in the same order as the list form, so results are bit-identical.
// WAIT: the tile's threads wait for the previous kernel (pdl_wait) after
// loading their slot records, which no kernel writes (k_step32; the
// persistent form waits once before its first tile).
template <int RPT, bool I32, bool TC, bool PAIR, bool SLOT, bool WAIT>
__device__ __forceinline__ void step32_tile(const DevModel &m, unsigned tile, const float *__restrict__ uh,
                                            float *__restrict__ uhn, unsigned short *__restrict__ uc,
                                            float *__restrict__ dh, unsigned short *__restrict__ dc) {
    using I = typename std::conditional<I32, unsigned, size_t>::type;
    const int G = m.R / RPT;
    int n, r0;
    if (I32) {
        const unsigned t = tile * blockDim.x + threadIdx.x;
        if (t >= (unsigned)m.n_active * (unsigned)G) return;
        if ((G & (G - 1)) == 0) {
            n = (int)(t >> (__ffs(G) - 1));
            r0 = (int)(t & (unsigned)(G - 1)) * RPT;
        } else {
            n = (int)(t / (unsigned)G);
            r0 = (int)(t % (unsigned)G) * RPT;
        }
    } else {
        const long long t = (long long)tile * blockDim.x + threadIdx.x;
        if (t >= (long long)m.n_active * G) return;
        n = (int)(t / G);
        r0 = (int)(t % G) * RPT;
    }
    const I R = m.R;
    // PAIR: the state is grouped by RPT (m.lg == RPT), so this thread's
    // values of a node start at 2 r0 and its y row follows its x row
    const I roff = PAIR ? 2 * (I)r0 : (I)r0;
    const I bn = ((I)n * 2) * R + roff;
    int4 s4 = make_int4(-1, -1, -1, -1);
    float invm = -1.f;
    if constexpr (SLOT) {
        s4 = __ldg(reinterpret_cast<const int4 *>(m.tslot4) + n);
        invm = __ldg(m.ninvm + n);
    }
    if constexpr (WAIT) pdl_wait();
    // Ask L2 for the node's own streaming state (read only after the
    // gather) so its DRAM latency overlaps the gather instead of following
    // it.  A block's nodes are consecutive, so their rows are one range per
    // array: one thread asks for the four ranges with bulk prefetches (needs
    // 16-byte aligned ranges of the 2-byte arrays: R a multiple of 4).  This
    // takes the per-thread address work out of every warp (6% on the 64-RHS
    // valley); otherwise each thread prefetches its own lines, which measured
    // 8% faster at 4 and 1 right-hand sides per thread and slower at 2.
    // Paired rows (one or two RHS, a node per thread) gain nothing from
    // either form: measured the same with per-thread, bulk or no prefetches.
    if ((m.R & 3) == 0) {
        if (threadIdx.x == 0) {
            const long long tb = (long long)tile * blockDim.x;
            const int na = (int)(tb / G);
            const int nz = (int)min((long long)m.n_active, (tb + blockDim.x - 1) / G + 1);
            const size_t e0 = (size_t)na * 2 * m.R, cnt = (size_t)(nz - na) * 2 * m.R;
            asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(dh + e0), "r"((unsigned)(cnt * 4)) : "memory");
            asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(uh + e0), "r"((unsigned)(cnt * 4)) : "memory");
            asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(dc + e0), "r"((unsigned)(cnt * 2)) : "memory");
            asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(uc + e0), "r"((unsigned)(cnt * 2)) : "memory");
        }
    } else if (RPT != 2 && !PAIR) {
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
    if (!SLOT || invm < 0.f) {
        for (int q = m.dptr[n]; q < m.dptr[n + 1]; ++q) {
            int ent = __ldg(m.dlist + q);
            float w = (ent & 1) ? 0.5f : 1.0f;
            int sc = ent >> 1;
            I b = ((I)(sc >> 2) * 8 + 2 * (sc & 3)) * R + roff;
            float fx[RPT], fy[RPT];
            XY<RPT, PAIR>::load_cg(m.fdrm32 + b, R, fx, fy);
#pragma unroll
            for (int j = 0; j < RPT; ++j) { ax[j] += w * fx[j]; ay[j] += w * fy[j]; }
        }
    }
    // element terms: -K_e u_e at this node's corner (and its hanging nodes' at 1/2)
    if constexpr (SLOT) {
        const int sl[4] = {s4.x, s4.y, s4.z, s4.w};
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            if (sl[j] < 0) continue;   // only trailing slots are empty
            const int e = (sl[j] >> 1) >> 2;
            int4 cn;
            if constexpr (TC) cn = __ldg(reinterpret_cast<const int4 *>(m.tcorn4) + ((I)n * 4 + j));
            else cn = __ldg(reinterpret_cast<const int4 *>(m.econn) + e);
            // the two stored coefficients (8 B per element, not 16)
            const float4 k = coef_from2(__ldg(reinterpret_cast<const float2 *>(m.ecoef2) + e));
            gather_term<RPT, PAIR, I>(sl[j], cn, k, R, roff, uh, ax, ay);
        }
        if (invm < 0.f) {
            for (int q = m.tptr[n] + 4; q < m.tptr[n + 1]; ++q) {
                const int ent = __ldg(m.tlist + q), e = (ent >> 1) >> 2;
                gather_term<RPT, PAIR, I>(ent, __ldg(reinterpret_cast<const int4 *>(m.econn) + e),
                                          __ldg(reinterpret_cast<const float4 *>(m.ecoef32) + e), R, roff, uh, ax, ay);
            }
        }
    } else {
        for (int q = m.tptr[n]; q < m.tptr[n + 1]; ++q) {
            const int ent = __ldg(m.tlist + q), e = (ent >> 1) >> 2;
            int4 cn;
            if constexpr (TC) cn = __ldg(reinterpret_cast<const int4 *>(m.tcorn) + q);
            else cn = __ldg(reinterpret_cast<const int4 *>(m.econn) + e);
            gather_term<RPT, PAIR, I>(ent, cn, __ldg(reinterpret_cast<const float4 *>(m.ecoef32) + e), R, roff, uh,
                                      ax, ay);
        }
    }
    node_update<RPT, PAIR, I, SLOT>(m, n, bn, R, roff, ax, ay, uh, uhn, uc, dh, dc, invm);
}

template <int RPT, bool I32, bool TC = true, bool PAIR = false, bool SLOT = false>
__global__ void __launch_bounds__(512) k_step32(DevModel m, const float *__restrict__ uh, float *__restrict__ uhn,
                                                unsigned short *__restrict__ uc, float *__restrict__ dh,
                                                unsigned short *__restrict__ dc) {
    step32_tile<RPT, I32, TC, PAIR, SLOT, true>(m, blockIdx.x, uh, uhn, uc, dh, dc);
}

// The same step as a persistent kernel (variant 4): a grid of as many blocks
// as fit on the device at once, each striding over the block-sized tiles of
// (node, RHS group) threads that k_step32 gives one block each.
template <int RPT, bool I32, bool TC = true, bool PAIR = false, bool SLOT = false>
__global__ void __launch_bounds__(512) k_step32p(DevModel m, const float *__restrict__ uh, float *__restrict__ uhn,
                                                 unsigned short *__restrict__ uc, float *__restrict__ dh,
                                                 unsigned short *__restrict__ dc, unsigned ntiles) {
    pdl_wait();
    for (unsigned tile = blockIdx.x; tile < ntiles; tile += gridDim.x)
        step32_tile<RPT, I32, TC, PAIR, SLOT, false>(m, tile, uh, uhn, uc, dh, dc);
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
        const Q4Fold<float> f = q4_fold<float>(k.x, k.y, k.z, k.w, c, w);
#pragma unroll
        for (int j = 0; j < RPT; ++j) {
            float vx[4] = {ux[0][j], ux[1][j], ux[2][j], ux[3][j]};
            float vy[4] = {uy[0][j], uy[1][j], uy[2][j], uy[3][j]};
            q4_corner_acc<float>(f, vx, vy, ax[j], ay[j]);
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
        float hx[RPT], hy[RPT], uhx[RPT], uhy[RPT];
        Vec<RPT>::load_cg(dh + bh, hx);
        Vec<RPT>::load_cg(dh + bh + R, hy);
        VecS<RPT>::load(sm + sb * row + rl, uhx);
        VecS<RPT>::load(sm + sb * row + RC + rl, uhy);
#pragma unroll
        for (int j = 0; j < RPT; ++j) {
            ax[j] += 0.5f * (hc.x * hx[j] + hc.z * ((uhx[j] - unx[j]) + (hx[j] - dx[j])));
            ay[j] += 0.5f * (hc.y * hy[j] + hc.w * ((uhy[j] - uny[j]) + (hy[j] - dy[j])));
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

// ---- bulk-copy pipeline (variant 2) ----------------------------------------
//
// A persistent kernel.  Each block walks tiles t = blockIdx.x, + gridDim.x,
// ...  A tile is `tn` consecutive active nodes over all R right-hand sides,
// and everything its update reads lies in a few contiguous runs of HBM:
//   - the u_hi rows of its halo, merged into runs of consecutive node ids;
//   - its own D, D_comp and u_comp rows;
//   - its node records, 32 bytes per node in node order: 1/m_full and
//     -2 a2 C (float4), then (first term in the tile | terms << 16, halo slot
//     of the node, DRM start | count << 24, anchor-link start | count << 24);
//   - its term records, packed per tile: the halo slots of the element's
//     corners as ushort4 (the node's corner in bits 14-15 of the first) for an
//     even number of terms, then the element's (A, B, C, D) times the term's
//     weight as float4 (a power of two: the sums are those of k_step32, bit
//     for bit).
// Warp 0 is the producer.  Its lanes issue those runs as cp.async.bulk copies
// into a shared-memory stage, one halo run per lane; the copies complete on
// the stage's "full" mbarrier, whose byte count lane 0 sets with
// arrive.expect_tx.  The other warps are consumers: each thread waits on
// "full", updates one (node, RPT right-hand sides) from shared memory, stores
// to HBM from registers, and each warp arrives on the stage's "empty" mbarrier,
// which the producer waits on before it refills the stage.  With S stages the
// producer runs S - 1 tiles ahead, and it loads the next tile's header and
// runs while it issues the current one.  Consumers read HBM only for DRM
// forces and hanging-node D (boundary-layer and anchor nodes).
// Every wait is bounded in time.  A warp that times out sets bit 2 of the
// watchdog flag and leaves; the producer then waits (bounded again) for the
// copies it issued before it leaves, so no copy outlives its block.
struct PipeArgs {
    const int4 *hdr;        // per tile: (halo nodes, terms, term-pack offset in 16 B, runs)
    const int2 *runs;       // per tile: PIPE_RUNS (first node, count), count 0 past the last
    const int4 *nrec;       // per active node: 2 int4 (node record)
    const int4 *tpack;      // term records, per tile
    const int *lslot;       // per anchor link: halo slot of the hanging node
    int tn, ntiles, nstage;
    unsigned stage_bytes;   // one stage; regions at the offsets below
    unsigned off_dh, off_dc, off_uc, off_nrec, off_ts, off_tk;
    long long wait_cycles;  // bound of each pipeline wait (exfem_opts.wait_cycles)
};

constexpr int PIPE_RUNS = 64;
constexpr int PIPE_MAX_STAGES = 4;
constexpr long long PIPE_WAIT_CYCLES = 2000000000LL;   // default bound: about 1 s at 2 GHz
// Bounds below this poll with mbarrier.test_wait, which returns at once;
// longer ones use try_wait, which may suspend the thread for a while (and so
// could outlast a short bound on its own).
constexpr long long PIPE_POLL_BELOW = 1000000LL;

__device__ __forceinline__ unsigned smem_addr(const void *p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ bool mbar_try_wait(unsigned bar, unsigned parity) {
    unsigned ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    return ok != 0;
}

__device__ __forceinline__ bool mbar_test_wait(unsigned bar, unsigned parity) {
    unsigned ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    return ok != 0;
}

// Waits for the phase with the given parity to complete, for at most
// `budget` SM cycles (and 2^26 polls); false on timeout.
__device__ __forceinline__ bool mbar_wait_bounded(unsigned bar, unsigned parity, long long budget) {
    const long long t0 = clock64();
    const bool poll = budget < PIPE_POLL_BELOW;
    for (int it = 0; it < (1 << 26); ++it) {
        if (poll ? mbar_test_wait(bar, parity) : mbar_try_wait(bar, parity)) return true;
        if (clock64() - t0 > budget) break;
    }
    return false;
}

__device__ __forceinline__ void bulk_g2s(unsigned dst, const void *src, unsigned bytes, unsigned bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                 ::"r"(dst), "l"(src), "r"(bytes), "r"(bar)
                 : "memory");
}

__device__ __forceinline__ int warp_excl_scan(int v, int lane, int &total) {
    int x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    total = __shfl_sync(0xffffffffu, x, 31);
    return x - v;
}

// Warp 0 of a k_pipe32 block: issues every tile's copies.
__device__ __forceinline__ void pipe_produce(const DevModel &m, const PipeArgs &pa, unsigned char *stage0,
                                             unsigned long long *full, unsigned long long *empty,
                                             const float *uh, const float *dh, const unsigned short *dc,
                                             const unsigned short *uc) {
    const int lane = threadIdx.x & 31;
    const unsigned R = (unsigned)m.R;
    const int NS = pa.nstage;
    int t = blockIdx.x;
    if (t >= pa.ntiles) return;
    int4 h = __ldg(pa.hdr + t);
    int2 ra = __ldg(pa.runs + (size_t)t * PIPE_RUNS + lane);
    int2 rb = __ldg(pa.runs + (size_t)t * PIPE_RUNS + 32 + lane);
    int k = 0;
    bool ok = true;
    for (; t < pa.ntiles; t += gridDim.x, ++k) {
        // the next tile's header and runs load while this one is issued
        const int tnext = t + gridDim.x;
        int4 h2 = h;
        int2 ra2 = ra, rb2 = rb;
        if (tnext < pa.ntiles) {
            h2 = __ldg(pa.hdr + tnext);
            ra2 = __ldg(pa.runs + (size_t)tnext * PIPE_RUNS + lane);
            rb2 = __ldg(pa.runs + (size_t)tnext * PIPE_RUNS + 32 + lane);
        }
        const int s = k % NS;
        if (k >= NS) {
            const bool w = mbar_wait_bounded(smem_addr(empty + s), (unsigned)(k / NS - 1) & 1u, pa.wait_cycles);
            if (!__all_sync(0xffffffffu, w)) { ok = false; break; }
            // the consumers' reads of the stage (generic proxy) come before the refill (async proxy)
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        }
        int tota, totb;
        const int offa = warp_excl_scan(ra.y, lane, tota);
        const int offb = tota + warp_excl_scan(rb.y, lane, totb);
        const unsigned base = smem_addr(stage0 + (size_t)s * pa.stage_bytes);
        const unsigned bar = smem_addr(full + s);
        const int n0 = t * pa.tn;
        const unsigned cnt = (unsigned)min(pa.tn, m.n_active - n0);
        const unsigned nt = (unsigned)h.y, ntev = (nt + 1u) & ~1u;
        if (lane == 0) {
            const unsigned bytes = (unsigned)h.x * 8u * R + cnt * (16u * R + 32u) + ntev * 8u + nt * 16u;
            asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
        }
        __syncwarp();
        if (ra.y > 0) bulk_g2s(base + (unsigned)offa * 8u * R, uh + (size_t)ra.x * 2 * R, (unsigned)ra.y * 8u * R, bar);
        if (rb.y > 0) bulk_g2s(base + (unsigned)offb * 8u * R, uh + (size_t)rb.x * 2 * R, (unsigned)rb.y * 8u * R, bar);
        const size_t o = (size_t)n0 * 2 * R;
        if (lane == 0) bulk_g2s(base + pa.off_dh, dh + o, cnt * 8u * R, bar);
        if (lane == 1) bulk_g2s(base + pa.off_dc, dc + o, cnt * 4u * R, bar);
        if (lane == 2) bulk_g2s(base + pa.off_uc, uc + o, cnt * 4u * R, bar);
        if (lane == 3) bulk_g2s(base + pa.off_nrec, pa.nrec + 2 * (size_t)n0, cnt * 32u, bar);
        if (lane == 4 && nt > 0) bulk_g2s(base + pa.off_ts, pa.tpack + h.z, ntev * 8u, bar);
        if (lane == 5 && nt > 0) bulk_g2s(base + pa.off_tk, pa.tpack + h.z + ntev / 2, nt * 16u, bar);
        h = h2;
        ra = ra2;
        rb = rb2;
    }
    if (!ok && lane == 0) atomicOr(m.d_flag, 2);
    // Copies that may still be in flight (the last NS tiles issued): the
    // producer leaves only once they have landed, so no copy outlives the
    // block even when the consumers gave up early.  Always the default bound:
    // a short caller bound must not cut this wait.
    if (lane == 0)
        for (int j = max(0, k - NS); j < k; ++j)
            mbar_wait_bounded(smem_addr(full + j % NS), (unsigned)(j / NS) & 1u, PIPE_WAIT_CYCLES);
    __syncwarp();
}

template <int RPT>
__global__ void __launch_bounds__(544) k_pipe32(DevModel m, PipeArgs pa, const float *__restrict__ uh,
                                                float *__restrict__ uhn, unsigned short *__restrict__ uc,
                                                float *__restrict__ dh, unsigned short *__restrict__ dc) {
    extern __shared__ __align__(128) unsigned char smraw[];
    // [0, 64): full mbarriers, [64, 128): empty mbarriers; stages from byte 128
    unsigned long long *full = reinterpret_cast<unsigned long long *>(smraw);
    unsigned long long *empty = full + PIPE_MAX_STAGES;
    unsigned char *stage0 = smraw + 128;
    const int NS = pa.nstage;
    const int lane = threadIdx.x & 31;
    if (threadIdx.x == 0) {
        const unsigned ncons = (blockDim.x >> 5) - 1;
        for (int s = 0; s < NS; ++s) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(full + s)));
            asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(empty + s)), "r"(ncons));
        }
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    if (threadIdx.x < 32) {
        pipe_produce(m, pa, stage0, full, empty, uh, dh, dc, uc);
        return;
    }
    const int R = m.R, G = R / RPT, row = 2 * R;
    const int ct = threadIdx.x - 32;
    const int ln = ct / G, g = ct - ln * G;
    const int rl = g * RPT, r0 = rl;
    int k = 0;
    for (int t = blockIdx.x; t < pa.ntiles; t += gridDim.x, ++k) {
        const int s = k % NS;
        const bool w = mbar_wait_bounded(smem_addr(full + s), (unsigned)(k / NS) & 1u, pa.wait_cycles);
        if (!__all_sync(0xffffffffu, w)) {
            if (lane == 0) atomicOr(m.d_flag, 2);
            return;
        }
        const unsigned char *st = stage0 + (size_t)s * pa.stage_bytes;
        const float *sh = reinterpret_cast<const float *>(st);
        const int n = t * pa.tn + ln;
        if (ln < pa.tn && n < m.n_active) {
            const size_t bn = ((size_t)n * 2) * R + r0;
            const int so = ln * row + rl;   // own row offset in the D region
            const float *sd = reinterpret_cast<const float *>(st + pa.off_dh);
            const unsigned short *sdc = reinterpret_cast<const unsigned short *>(st + pa.off_dc);
            const unsigned short *suc = reinterpret_cast<const unsigned short *>(st + pa.off_uc);
            const int4 *snr = reinterpret_cast<const int4 *>(st + pa.off_nrec);
            const uint2 *sts = reinterpret_cast<const uint2 *>(st + pa.off_ts);
            const float4 *stk = reinterpret_cast<const float4 *>(st + pa.off_tk);
            const int4 meta = snr[2 * ln + 1];
            const int tb = meta.x & 0xffff, tc = (int)((unsigned)meta.x >> 16);
            const int dbeg = meta.z & 0xffffff, dcnt = (int)((unsigned)meta.z >> 24);
            const int lbeg = meta.w & 0xffffff, lcnt = (int)((unsigned)meta.w >> 24);
            float ax[RPT], ay[RPT];
#pragma unroll
            for (int j = 0; j < RPT; ++j) { ax[j] = 0.f; ay[j] = 0.f; }
            for (int q = dbeg; q < dbeg + dcnt; ++q) {
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
            for (int q = tb; q < tb + tc; ++q) {
                const uint2 sl = sts[q];
                const float4 kc = stk[q];
                const int c = (int)((sl.x >> 14) & 3u);
                const int ss[4] = {(int)(sl.x & 0x3fffu), (int)(sl.x >> 16), (int)(sl.y & 0xffffu), (int)(sl.y >> 16)};
                float ux[4][RPT], uy[4][RPT];
#pragma unroll
                for (int v = 0; v < 4; ++v) {
                    VecS<RPT>::load(sh + ss[v] * row + rl, ux[v]);
                    VecS<RPT>::load(sh + ss[v] * row + R + rl, uy[v]);
                }
                const Q4Fold<float> f = q4_fold<float>(kc.x, kc.y, kc.z, kc.w, c, 1.0f);
#pragma unroll
                for (int j = 0; j < RPT; ++j) {
                    float vx[4] = {ux[0][j], ux[1][j], ux[2][j], ux[3][j]};
                    float vy[4] = {uy[0][j], uy[1][j], uy[2][j], uy[3][j]};
                    q4_corner_acc<float>(f, vx, vy, ax[j], ay[j]);
                }
            }
            const int4 nci = snr[2 * ln];
            const float4 nc = make_float4(__int_as_float(nci.x), __int_as_float(nci.y), __int_as_float(nci.z),
                                          __int_as_float(nci.w));
            float dx[RPT], dy[RPT];
            VecS<RPT>::load(sd + so, dx);
            VecS<RPT>::load(sd + so + R, dy);
            if (nc.z != 0.f || nc.w != 0.f) {
#pragma unroll
                for (int j = 0; j < RPT; ++j) { ax[j] += nc.z * dx[j]; ay[j] += nc.w * dy[j]; }
            }
            float unx[RPT], uny[RPT];
            VecS<RPT>::load(sh + meta.y * row + rl, unx);
            VecS<RPT>::load(sh + meta.y * row + R + rl, uny);
            for (int q = lbeg; q < lbeg + lcnt; ++q) {
                int hn = __ldg(m.llist + 2 * q);
                int sb = __ldg(pa.lslot + q);
                float4 hc = __ldg(reinterpret_cast<const float4 *>(m.hcoef4) + (hn - m.n_active));
                size_t bh = ((size_t)hn * 2) * R + r0;
                float hx[RPT], hy[RPT], uhx[RPT], uhy[RPT];
                Vec<RPT>::load_cg(dh + bh, hx);
                Vec<RPT>::load_cg(dh + bh + R, hy);
                VecS<RPT>::load(sh + sb * row + rl, uhx);
                VecS<RPT>::load(sh + sb * row + R + rl, uhy);
#pragma unroll
                for (int j = 0; j < RPT; ++j) {
                    ax[j] += 0.5f * (hc.x * hx[j] + hc.z * ((uhx[j] - unx[j]) + (hx[j] - dx[j])));
                    ay[j] += 0.5f * (hc.y * hy[j] + hc.w * ((uhy[j] - uny[j]) + (hy[j] - dy[j])));
                }
            }
            float dcx[RPT], dcy[RPT], ucx[RPT], ucy[RPT], ox[RPT], oy[RPT];
            Half<RPT>::load(sdc + so, dcx);
            Half<RPT>::load(sdc + so + R, dcy);
            Half<RPT>::load(suc + so, ucx);
            Half<RPT>::load(suc + so + R, ucy);
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
        __syncwarp();
        if (lane == 0) asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(empty + s)) : "memory");
    }
}

// ---- tensor-core step (variant 3) ------------------------------------------
// The element products K_e u_e of the batched form on the 5th-generation
// tensor cores (tcgen05, kind::tf32).  A block owns a tile of at most kMmaTn
// consecutive active nodes (closed early where their terms would read more
// than kMmaEmax distinct elements) and kMmaRc right-hand sides.  With
// K_e = mu_e Kmu + lambda_e Klambda (calck is linear in (mu, lambda),
// formulation.f90:276-313), every distinct element of the tile's terms
// (at most kMmaEmax) contributes one row per right-hand side: its 8 corner
// dofs u_e relative to corner 0 (K has the rigid translations in its null
// space, so K (u_e - u_0) = K u_e, and the differences are small).  The rows
// meet B = [Kmu; Klambda] (16 x 8) in 128 x 16 x 8 MMAs, 8 elements x 16
// right-hand sides each, in 3xTF32: A_hi B_hi + A_hi B_lo + A_lo B_hi, with
// hi = tf32(x) and lo = tf32(x - hi), which holds FP32-level accuracy.  One
// thread issues every MMA of the tile and commits them to an mbarrier; the
// four warps read D = (Kmu u_e, Klambda u_e) back from TMEM, scale by
// (mu_e, lambda_e) into per-element corner forces in shared memory (over the
// A tiles, which the MMAs no longer read), and then each thread finishes a
// node for four right-hand sides: its DRM terms, its element terms (the
// forces of its corner, at weight 1 or 1/2), and node_update.  The plain
// state layout (value of node n, dof d, rhs r at (n*2 + d)*R + r).
struct MmaArgs {
    const int *nptr;              // per tile: first active node
    const int *eptr, *elist;      // per tile: its distinct elements
    const unsigned char *tj;      // per gather term: its element's index in the tile
    const float *btile;           // [Kmu; Klambda] split into tf32 hi then lo, 128 floats each, K-major layout
    long long wait_cycles;        // bound of the MMA completion wait
};

constexpr int kMmaRc = 16;        // right-hand sides per block
constexpr int kMmaTn = 32;        // nodes per tile
constexpr int kMmaEmax = 64;      // elements per tile (8 MMA row chunks of 8 elements x 16 RHS)
constexpr int kMmaThreads = 256;  // kMmaTn nodes x kMmaRc / 2 right-hand sides per thread
constexpr unsigned kMmaTmemCols = 128;   // 8 chunks x 16 FP32 columns
constexpr unsigned kMmaAbytes = kMmaEmax * kMmaRc * 32;   // one A tile (hi or lo)
constexpr unsigned kMmaSmem = 1024 + 2 * kMmaAbytes;       // B hi/lo, A hi, A lo

__global__ void __launch_bounds__(kMmaThreads) k_mma32(DevModel m, MmaArgs ma, const float *__restrict__ uh,
                                                       float *__restrict__ uhn, unsigned short *__restrict__ uc,
                                                       float *__restrict__ dh, unsigned short *__restrict__ dc) {
    extern __shared__ __align__(128) unsigned char smtc[];   // 16-byte alignment suffices without swizzle
    __shared__ __align__(8) unsigned long long mbar;
    __shared__ uint32_t tslot;
    unsigned char *sAhi = smtc + 1024, *sAlo = sAhi + kMmaAbytes;
    float *sF = reinterpret_cast<float *>(sAhi);   // after the MMAs: force (j*8 + k)*kMmaRc + r
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    // the RHS chunks of a tile are adjacent blocks, so they meet the tile's
    // metadata and the same state rows in L2 together
    const int nch = m.R / kMmaRc;
    const int tile = (int)(blockIdx.x / nch), rbase = (int)(blockIdx.x % nch) * kMmaRc;
    const size_t R = (size_t)m.R;
    const int e0 = __ldg(ma.eptr + tile), ne_t = __ldg(ma.eptr + tile + 1) - e0;
    const int nchunk = (ne_t + 7) >> 3;
    for (int i = tid; i < 64; i += kMmaThreads)
        reinterpret_cast<float4 *>(smtc)[i] = __ldg(reinterpret_cast<const float4 *>(ma.btile) + i);
    // every load of the thread's rows first (at most four rows a thread), then
    // the differences, splits and stores
    constexpr int kRowsPerThread = kMmaEmax * kMmaRc / kMmaThreads;
    float ux[kRowsPerThread][4], uy[kRowsPerThread][4];
#pragma unroll
    for (int i = 0; i < kRowsPerThread; ++i) {
        const int row = tid + i * kMmaThreads, j = row >> 4, r = row & 15;
        if (row < nchunk * 128 && j < ne_t) {
            const int4 cn = __ldg(reinterpret_cast<const int4 *>(m.econn) + __ldg(ma.elist + e0 + j));
            const int cc[4] = {cn.x, cn.y, cn.z, cn.w};
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const size_t b = (size_t)cc[q] * 2 * R + rbase + r;
                ux[i][q] = __ldg(uh + b);
                uy[i][q] = __ldg(uh + b + R);
            }
        } else {
#pragma unroll
            for (int q = 0; q < 4; ++q) { ux[i][q] = 0.f; uy[i][q] = 0.f; }
        }
    }
#pragma unroll
    for (int i = 0; i < kRowsPerThread; ++i) {
        const int row = tid + i * kMmaThreads;
        if (row >= nchunk * 128) continue;
        float v[8];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            v[2 * q] = ux[i][q] - ux[i][0];
            v[2 * q + 1] = uy[i][q] - uy[i][0];
        }
        float hi[8], lo[8];
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            hi[k] = tc_tf32(v[k]);
            lo[k] = tc_tf32(v[k] - hi[k]);
        }
        const unsigned o = tc_kmaj_off(row, 0);
        *reinterpret_cast<float4 *>(sAhi + o) = make_float4(hi[0], hi[1], hi[2], hi[3]);
        *reinterpret_cast<float4 *>(sAhi + o + kTcLbo) = make_float4(hi[4], hi[5], hi[6], hi[7]);
        *reinterpret_cast<float4 *>(sAlo + o) = make_float4(lo[0], lo[1], lo[2], lo[3]);
        *reinterpret_cast<float4 *>(sAlo + o + kTcLbo) = make_float4(lo[4], lo[5], lo[6], lo[7]);
    }
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(&mbar)));
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) tc_alloc(smem_addr(&tslot), kMmaTmemCols);
    // the A and B tiles (generic-proxy stores) become visible to the MMAs
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tbase = tslot;
    if (tid == 0) {
        const uint32_t idesc = tc_idesc_tf32(128, 16);
        const unsigned sb = smem_addr(smtc);
        const uint64_t bh = tc_smem_desc(sb), bl = tc_smem_desc(sb + 512);
        for (int c = 0; c < nchunk; ++c) {
            const uint64_t ah = tc_smem_desc(smem_addr(sAhi) + 4096u * c);
            const uint64_t al = tc_smem_desc(smem_addr(sAlo) + 4096u * c);
            const uint32_t d = tbase + 16u * c;
            tc_mma_tf32(d, ah, bh, idesc, 0);
            tc_mma_tf32(d, ah, bl, idesc, 1);
            tc_mma_tf32(d, al, bh, idesc, 1);
        }
        tc_commit(smem_addr(&mbar));
    }
    bool ok = mbar_wait_bounded(smem_addr(&mbar), 0u, ma.wait_cycles);
    if (!ok) {
        if (lane == 0) atomicOr(m.d_flag, 2);
        // the MMAs must have finished before their TMEM is freed
        ok = mbar_wait_bounded(smem_addr(&mbar), 0u, PIPE_WAIT_CYCLES);
    }
    tc_fence_after();
    const bool all_ok = __syncthreads_and(ok ? 1 : 0) != 0;
    if (all_ok) {
        // warp w reads TMEM lanes 32 (w % 4) .. + 31 of every other chunk
        const int quarter = warp & 3;
        for (int c = warp >> 2; c < nchunk; c += kMmaThreads / 128) {
            float d[16];
            tc_ld16(tbase + ((uint32_t)(32 * quarter) << 16) + 16u * c, d);
            const int row = c * 128 + 32 * quarter + lane, j = row >> 4, r = row & 15;
            if (j < ne_t) {
                const float4 k4 = __ldg(reinterpret_cast<const float4 *>(m.ecoef32) + __ldg(ma.elist + e0 + j));
                const float mu = 4.f * k4.z, lam = 4.f * k4.y;   // ecoef32 = ((l+2m)/4, l/4, m/4, (l+3m)/12)
#pragma unroll
                for (int k = 0; k < 8; ++k) sF[(j * 8 + k) * kMmaRc + r] = mu * d[k] + lam * d[8 + k];
            }
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) tc_dealloc(tbase, kMmaTmemCols);
    if (!all_ok) return;
    constexpr int RPT = kMmaRc * kMmaTn / kMmaThreads;   // right-hand sides per thread
    constexpr int TPN = kMmaRc / RPT;                     // threads per node
    const int n = __ldg(ma.nptr + tile) + tid / TPN;
    if (n >= __ldg(ma.nptr + tile + 1)) return;
    const int r0 = (tid % TPN) * RPT;
    const size_t roff = (size_t)rbase + r0;
    const size_t bn = ((size_t)n * 2) * R + roff;
    float ax[RPT], ay[RPT];
#pragma unroll
    for (int j = 0; j < RPT; ++j) { ax[j] = 0.f; ay[j] = 0.f; }
    for (int q = m.dptr[n]; q < m.dptr[n + 1]; ++q) {
        int ent = __ldg(m.dlist + q);
        float w = (ent & 1) ? 0.5f : 1.0f;
        int sc = ent >> 1;
        size_t b = ((size_t)(sc >> 2) * 8 + 2 * (sc & 3)) * R + roff;
        float fx[RPT], fy[RPT];
        XY<RPT, false>::load_cg(m.fdrm32 + b, R, fx, fy);
#pragma unroll
        for (int j = 0; j < RPT; ++j) { ax[j] += w * fx[j]; ay[j] += w * fy[j]; }
    }
    for (int q = m.tptr[n]; q < m.tptr[n + 1]; ++q) {
        const int ent = __ldg(m.tlist + q);
        const float w = (ent & 1) ? 0.5f : 1.0f;
        const int c = (ent >> 1) & 3, j = __ldg(ma.tj + q);
        const float *fx = sF + (j * 8 + 2 * c) * kMmaRc + r0, *fy = fx + kMmaRc;
#pragma unroll
        for (int k = 0; k < RPT; ++k) {
            ax[k] -= w * fx[k];
            ay[k] -= w * fy[k];
        }
    }
    node_update<RPT, false, size_t>(m, n, bn, R, roff, ax, ay, uh, uhn, uc, dh, dc);
}

// Point source in the FP32 form, after the step kernel and before k_hang32
// (the force enters delta linearly, so the step kernels stay untouched).
//   POINTN: the y dof of node p32_node[i] gets w_i f(t) / m_full added to D+
//           and to u+ (point_reactions before sum_reactanchors: a hanging
//           source node gives each anchor half its force).
//   POINTD: u+ = f(t) on the source node's y dof, D+ = f(t) - u, with u the
//           displacement before the step (point_displacements after the
//           update, explicit.f90:150).
// Values are recombined and re-split (hi - comp) in FP64.
__global__ void k_point32(DevModel m, const int *__restrict__ pn, const float *__restrict__ pw, int np,
                          float *__restrict__ uhn, unsigned short *__restrict__ uc, float *__restrict__ dh,
                          unsigned short *__restrict__ dc) {
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)np * m.R) return;
    const int i = (int)(t / m.R), r = (int)(t % m.R);
    const int n = pn[i];
    const size_t iy = state_at(m, (size_t)n, 1, r);
    const double f = point_value(m, read_step(m) + 1);
    const double u1 = (double)uhn[iy] - (double)bf2f(uc[iy]);
    const double d1 = (double)dh[iy] - (double)bf2f(dc[iy]);
    double u2, d2;
    if (m.point_kind == EXFEM_POINT_FORCE) {
        const double dp = (double)pw[i] * f * (double)reinterpret_cast<const float4 *>(m.ncoef4)[n].y;
        u2 = u1 + dp;
        d2 = d1 + dp;
    } else {
        u2 = f;
        d2 = f - (u1 - d1);
    }
    const float uh2 = (float)u2, dh2 = (float)d2;
    uhn[iy] = uh2;
    uc[iy] = f2bf((float)((double)uh2 - u2));
    dh[iy] = dh2;
    dc[iy] = f2bf((float)((double)dh2 - d2));
}

// A prescribed displacement at t = 0 and -dt on every source node (hanging
// ones included): u = v0, D = v0 - vm (explicit.f90:93-94).
__global__ void k_point_init32(DevModel m, float *__restrict__ uh, unsigned short *__restrict__ uc,
                               float *__restrict__ dh, unsigned short *__restrict__ dc, double v0, double vm) {
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)m.npoint * m.R) return;
    const int n = m.pnodes[t / m.R], r = (int)(t % m.R);
    const size_t iy = state_at(m, (size_t)n, 1, r);
    const double d = v0 - vm;
    const float uh2 = (float)v0, dh2 = (float)d;
    uh[iy] = uh2;
    uc[iy] = f2bf((float)((double)uh2 - v0));
    dh[iy] = dh2;
    dc[iy] = f2bf((float)((double)dh2 - d));
}

// u of one node in FP64 (u_hi - comp); hanging corners read as anchor averages.
// (rows: read a hanging corner's own row, for the step-0 sample.)
__device__ __forceinline__ void load_u32(const DevModel &m, const float *uh, const unsigned short *uc, int node,
                                         int r, bool rows, double &vx, double &vy) {
    auto val = [&](int x, int d) {
        size_t i = state_at(m, (size_t)x, d, r);
        return (double)uh[i] - (double)bf2f(uc[i]);
    };
    if (node < m.n_active || rows) {
        vx = val(node, 0);
        vy = val(node, 1);
    } else {
        int i = node - m.n_active;
        int a = m.hang[3 * i + 1], b = m.hang[3 * i + 2];
        vx = (val(a, 0) + val(b, 0)) / 2.0;
        vy = (val(a, 1) + val(b, 1)) / 2.0;
    }
}

// Hanging nodes (anchor averages of u_hi, comp and D), receivers, and the
// DRM forces of the next step.  Blocks [0, nb_hang) hanging nodes, then
// nb_recv receiver blocks (ipb items each), then the DRM blocks (ipb_drm
// items each).  mode 1: the step-0 receiver sample and the DRM forces of
// step 1.
__global__ void __launch_bounds__(256) k_hang32(DevModel m, const float *__restrict__ uho, float *__restrict__ uhn,
                                                unsigned short *__restrict__ uc, float *__restrict__ dh,
                                                unsigned short *__restrict__ dc, int nb_hang, int mode, int ipb,
                                                int nb_recv, int ipb_drm) {
    // the next step kernel (a programmatic dependent of this one) may launch
    // now and load its static records while this pass runs
    pdl_trigger();
    int step = (mode == 1) ? 0 : read_step(m) + 1;
    // the step-0 sample computes step 1's DRM forces: the side-stream DRM
    // launches continue from there
    if (mode == 1 && blockIdx.x == 0 && threadIdx.x == 0) *m.d_drm_step = 1;
    // the DRM blocks, whose FP64/exp chains are the longest, take the lowest
    // block indices so that they are scheduled first
    const int nb_drm = (int)gridDim.x - nb_hang - nb_recv;
    const int bx = (int)blockIdx.x - nb_drm;
    if (bx < 0) {
        drm32_items(m, ipb_drm, blockIdx.x, step + 1);
    } else if (bx < nb_hang) {
        long long t = (long long)bx * blockDim.x + threadIdx.x;
        if (mode == 0 && t < (long long)m.n_hang * m.R) {
            int i = (int)(t / m.R), r = (int)(t % m.R);
            int h = m.hang[3 * i], a = m.hang[3 * i + 1], b = m.hang[3 * i + 2];
            // A prescribed point displacement at t = 0 (explicit.f90:93) is
            // the one hanging value that is not its anchors' average, so at
            // the first step the increment of such a node is new - old.
            const bool from_row = m.point_kind == EXFEM_POINT_DISP && step == 1 && m.pflag[h];
            // every input of both dofs is loaded before the first store (the
            // stores could alias the anchors' rows for all the compiler knows,
            // which would serialise the two dofs' round trips)
            size_t ih[2], ia[2], ib[2];
            float ua[2], ub[2], da[2], db[2];
            unsigned short uca[2], ucb[2], dca[2], dcb[2];
            double u_old[2];
#pragma unroll
            for (int d = 0; d < 2; ++d) {
                ih[d] = state_at(m, (size_t)h, d, r);
                ia[d] = state_at(m, (size_t)a, d, r);
                ib[d] = state_at(m, (size_t)b, d, r);
                u_old[d] = (double)uho[ih[d]] - (double)bf2f(uc[ih[d]]);   // the row before this step
                ua[d] = uhn[ia[d]]; ub[d] = uhn[ib[d]];
                uca[d] = uc[ia[d]]; ucb[d] = uc[ib[d]];
                da[d] = dh[ia[d]]; db[d] = dh[ib[d]];
                dca[d] = dc[ia[d]]; dcb[d] = dc[ib[d]];
            }
#pragma unroll
            for (int d = 0; d < 2; ++d) {
                const float un = 0.5f * (ua[d] + ub[d]);
                const unsigned short ucn = f2bf(0.5f * (bf2f(uca[d]) + bf2f(ucb[d])));
                uhn[ih[d]] = un;
                uc[ih[d]] = ucn;
                if (from_row) {
                    const double dn = ((double)un - (double)bf2f(ucn)) - u_old[d];
                    const float dnf = (float)dn;
                    dh[ih[d]] = dnf;
                    dc[ih[d]] = f2bf((float)((double)dnf - dn));
                } else {
                    dh[ih[d]] = 0.5f * (da[d] + db[d]);
                    dc[ih[d]] = f2bf(0.5f * (bf2f(dca[d]) + bf2f(dcb[d])));
                }
            }
        }
    } else if (step % m.io == 0) {
        // four threads per (receiver, rhs): thread q < 3 evaluates free-field
        // term q (the FP64 Ricker pulses are the cost), thread 0 interpolates
        // and adds the terms in planewave_u's order; `ipb` items per block
        const int li = threadIdx.x >> 2;
        const long long wq = (long long)(bx - nb_hang) * ipb + li;
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
                load_u32(m, uhn, uc, m.rnode[4 * i + k], r, mode == 1, vx, vy);
                double w = m.rw[4 * i + k];
                fx += w * vx;
                fy += w * vy;
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

template <typename T, typename A>
int upload32(Ctx &c, const std::vector<T, A> &v, const T **dst) {
    if (v.empty()) { *dst = nullptr; return EXFEM_OK; }
    void *p = nullptr;
    CK(ctx_alloc(c, &p, v.size() * sizeof(T)));
    CK(cudaMemcpyAsync(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, c.stream));
    c.h2d_bytes += v.size() * sizeof(T);
    *dst = static_cast<const T *>(p);
    return EXFEM_OK;
}

template <typename T>
int alloc32(Ctx &c, size_t n, T **dst) {
    void *p = nullptr;
    if (n == 0) n = 1;
    CK(ctx_alloc(c, &p, n * sizeof(T)));
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
    // measured on canyons and valleys of 3e4-9e5 elements: two per thread
    // beats one from R = 4 (the per-term metadata and fold are shared), four
    // pays off from R = 16.  At R = 2 and 4 a thread per node makes the
    // node's x and y rows one 16- or 32-byte vector (k_step32's PAIR form):
    // 17% faster per step than two threads per node on the 1.5M-element
    // valley at R = 2, 12% on a 0.55M-element valley at R = 4.
    if (R % 4 == 0 && (R >= 16 || R == 4)) return 4;
    if (R % 2 == 0) return 2;
    return 1;
}

// Tiles, their headers and halo runs, node and term records for k_pipe32,
// and the stage layout.  Leaves c.use_pipe false when the model does not fit
// the record formats or shared memory.
static int pipe_setup(Ctx &c) {
    const Plan &P = c.plan;
    const int R = P.R, rpt = c.rhs_per_thread, G = R / rpt;
    const int tn = c.block_threads / G;
    if (tn < 1) return EXFEM_OK;
    const int consumers = (tn * G + 31) / 32 * 32;
    if (consumers > 512) return EXFEM_OK;
    Tiles T;
    std::string terr;
    if (build_tiles(P, tn, T, terr) != EXFEM_OK) return EXFEM_OK;
    PipePack pk;
    if (!build_pipe_pack(P, T, PIPE_RUNS, pk, terr)) return EXFEM_OK;
    const int tmax = pk.tmax;
    // stage: halo rows | D | D_comp | u_comp | node records | slots | coefficients
    const unsigned Ru = (unsigned)R, tnu = (unsigned)tn;
    const unsigned tmev = (unsigned)((tmax + 1) & ~1);
    unsigned off[6];
    off[0] = (unsigned)T.hmax * 8u * Ru;
    off[1] = off[0] + tnu * 8u * Ru;
    off[2] = off[1] + tnu * 4u * Ru;
    off[3] = off[2] + tnu * 4u * Ru;
    off[4] = off[3] + tnu * 32u;
    off[5] = off[4] + (tmev * 8u + 15u) / 16u * 16u;
    const unsigned stage = (off[5] + (unsigned)tmax * 16u + 127u) / 128u * 128u;
    int dev_smem = 0, nsm = 0;
    cudaDeviceGetAttribute(&dev_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, c.device);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, c.device);
    int ns = 0;
    for (int k = PIPE_MAX_STAGES; k >= 2 && !ns; --k)
        if (128 + (size_t)k * stage <= (size_t)dev_smem) ns = k;
    if (!ns || stage >= (1u << 20)) return EXFEM_OK;
    const size_t smem = 128 + (size_t)ns * stage;
    const int threads = 32 + consumers;
    int per_sm = 0, rc;
    switch (rpt) {
        case 4:
            CK(cudaFuncSetAttribute(k_pipe32<4>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
            CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_pipe32<4>, threads, smem));
            break;
        case 2:
            CK(cudaFuncSetAttribute(k_pipe32<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
            CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_pipe32<2>, threads, smem));
            break;
        default:
            CK(cudaFuncSetAttribute(k_pipe32<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
            CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_pipe32<1>, threads, smem));
            break;
    }
    if (per_sm < 1) return EXFEM_OK;
    const int *d = nullptr;
    if ((rc = upload32(c, pk.hdr, &d))) return rc;
    c.p_hdr = d;
    if ((rc = upload32(c, pk.runs, &d))) return rc;
    c.p_runs = d;
    if ((rc = upload32(c, pk.nrec, &d))) return rc;
    c.p_nrec = d;
    if ((rc = upload32(c, pk.tpack, &d))) return rc;
    c.p_tpack = d;
    if (!T.lslot.empty() && (rc = upload32(c, T.lslot, &c.t_lslot))) return rc;
    c.tile_tn = tn;
    c.tile_n = T.ntiles;
    c.tile_hmax = T.hmax;
    c.tile_smem = smem;
    c.pipe_stage = stage;
    c.pipe_nstage = ns;
    c.pipe_threads = threads;
    for (int k = 0; k < 6; ++k) c.pipe_off[k] = off[k];
    c.pipe_grid = std::min(T.ntiles, per_sm * std::max(nsm, 1));
    c.use_pipe = true;
    return EXFEM_OK;
}

static int mma_setup(Ctx &c) {
    const Plan &P = c.plan;
    MmaTiles T;
    std::string why;
    if (!build_mma_tiles(P, kMmaTn, kMmaEmax, T, why)) return EXFEM_OK;   // the direct gather runs
    int rc;
    if ((rc = upload32(c, T.nptr, &c.mma_nptr)) || (rc = upload32(c, T.eptr, &c.mma_eptr)) ||
        (rc = upload32(c, T.elist, &c.mma_elist)) ||
        (rc = upload32(c, T.tj, &c.mma_tj)) || (rc = upload32(c, tc_b_operand_q4(), &c.mma_btile)))
        return rc;
    CK(cudaFuncSetAttribute(k_mma32, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kMmaSmem));
    if ((long long)T.ntiles * (P.R / kMmaRc) >= (1LL << 31)) return EXFEM_OK;   // grid limit: the direct gather runs
    c.mma_ntiles = T.ntiles;
    c.rhs_per_thread = kMmaRc * kMmaTn / kMmaThreads;
    c.block_threads = kMmaThreads;
    c.use_mma = true;
    return EXFEM_OK;
}

int f32_alloc(Ctx &c) {
    const Plan &P = c.plan;
    DevModel &m = c.dm;
    // per active node: 1/m_full (x, y), -2 a2 C (x, y)
    const pvec<float> nc = node_coef32(P);
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
    // the FP32 coefficients: two per element uploaded, the four derived on
    // the device (the same operations as the plan's ecoef32)
    if ((rc = upload32(c, P.ecoef2, &m.ecoef2))) return rc;
    {
        float *k4 = nullptr;
        if ((rc = alloc32(c, 4 * (size_t)std::max(P.ne, 1), &k4))) return rc;
        if (P.ne > 0) {
            k_coef32<<<nblocks(P.ne, 256), 256, 0, c.stream>>>(m.ecoef2, k4, P.ne);
            c.launches++;
            CK(cudaGetLastError());
        }
        m.ecoef32 = k4;
    }
    // with few right-hand sides the next step's DRM forces run beside this
    // step on a second stream, into the other of two force slots
    c.drm_side = m.ns > 0 && P.R <= kDrmSideMaxRhs && c.opts.drm_inline == 0;
    const size_t slot = (size_t)std::max(m.ns, 1) * 8 * P.R;
    if ((rc = alloc32(c, slot * (c.drm_side ? 2 : 1), &m.fdrm32))) return rc;
    if (c.drm_side) {
        c.fdrm_slot[0] = m.fdrm32;
        c.fdrm_slot[1] = m.fdrm32 + slot;
        if ((rc = side_create(c))) return rc;
    }
    m.drm_delay = nullptr;
    if (m.ns > 0) {
        double *dd = nullptr;
        if ((rc = alloc32(c, (size_t)m.ns * 12 * P.R, &dd))) return rc;
        k_drm_delays32<<<nblocks((long long)m.ns * 4 * P.R, 128), 128, 0, c.stream>>>(m, dd);
        c.launches++;
        CK(cudaGetLastError());
        m.drm_delay = dd;
    }
    size_t nst = (size_t)P.nn * 2 * P.R;
    if ((rc = alloc32(c, nst, &c.uhi[0]))) return rc;
    if ((rc = alloc32(c, nst, &c.uhi[1]))) return rc;
    if ((rc = alloc32(c, nst, &c.ucomp))) return rc;
    if ((rc = alloc32(c, nst, &c.udel[0]))) return rc;
    if ((rc = alloc32(c, nst, &c.dcomp))) return rc;
    // point source: the active nodes it acts on, with their weights
    c.p32_n = 0;
    if (P.point_kind != 0) {
        std::vector<float> w(P.n_active, 0.f);
        for (int n = 0; n < P.n_active; ++n) {
            if (P.pflag[n]) w[n] += 1.f;
            if (P.point_kind == EXFEM_POINT_FORCE)
                for (int q = P.lptr[n]; q < P.lptr[n + 1]; ++q)
                    if (P.pflag[P.llist[2 * (size_t)q]]) w[n] += 0.5f;
        }
        std::vector<int> pn;
        std::vector<float> pw;
        for (int n = 0; n < P.n_active; ++n)
            if (w[n] != 0.f) { pn.push_back(n); pw.push_back(w[n]); }
        if (!pn.empty()) {
            if ((rc = upload32(c, pn, &c.p32_node))) return rc;
            if ((rc = upload32(c, pw, &c.p32_w))) return rc;
            c.p32_n = (int)pn.size();
        }
    }
    c.rhs_per_thread = pick_rpt(c);
    {
        // 32-bit indices in k_step32: thread ids (grid rounded up to a block)
        // and the largest state and DRM-force element index
        const unsigned long long lim = 1ull << 32;
        const unsigned long long threads = (unsigned long long)P.n_active * (P.R / c.rhs_per_thread) + 1024;
        const unsigned long long state = (unsigned long long)P.nn * 2 * P.R;
        const unsigned long long drm = (unsigned long long)std::max(m.ns, 1) * 8 * P.R;
        c.idx32 = c.opts.index_bits != 64 && threads < lim && state < lim && drm < lim;
    }
    // default block: 256, and 128 for the direct gather from four RHS
    // (measured on 0.1M- and 0.55M-element valleys: 1-3% faster than 256 on
    // the larger mesh, within 2% either way on the smaller)
    if (c.opts.block_threads <= 0)
        c.block_threads = (P.R >= 4 && (c.opts.variant == 0 || c.opts.variant == 4 || c.opts.variant == 5)) ? 128 : 256;
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
    // bulk-copy pipeline (variant 2): needs 16-byte rows (R a multiple of 4)
    // and at least two stages in shared memory; otherwise the direct gather runs
    c.use_pipe = false;
    if (c.opts.variant == 2 && P.R % 4 == 0) {
        if ((rc = pipe_setup(c))) return rc;
    }
    // tensor-core step (variant 3): R a multiple of kMmaRc and every tile
    // within kMmaEmax elements; otherwise the direct gather runs
    c.use_mma = false;
    if (c.opts.variant == 3 && P.R % kMmaRc == 0) {
        if ((rc = mma_setup(c))) return rc;
    }
    // the direct gather with several threads per node groups the state by
    // the thread's RHS (the tiled variants read the plain layout)
    const bool direct = !c.use_tiles && !c.use_pipe && !c.use_mma;
    m.lg = (direct && c.rhs_per_thread < P.R && f32_interleave(P.R)) ? c.rhs_per_thread : P.R;
    // the direct gather's fixed-size node records from kSlotMinNodes active
    // nodes (variant 5: the list form always)
    m.tslot4 = nullptr;
    m.ninvm = nullptr;
    m.tcorn4 = nullptr;
    if (direct && c.opts.variant != 5 && P.n_active >= kSlotMinNodes) {
        // built on the device from the lists and node coefficients already
        // there (build_node_slots states the same records on the host)
        if ((long long)P.ne * 8 <= (1ll << 31) - 1 && P.n_active > 0) {
            int *s4 = nullptr;
            float *iv = nullptr;
            if ((rc = alloc32(c, 4 * (size_t)P.n_active, &s4)) || (rc = alloc32(c, (size_t)P.n_active, &iv))) return rc;
            k_node_slots<<<nblocks(P.n_active, 256), 256, 0, c.stream>>>(m.tptr, m.tlist, m.dptr, m.lptr, m.ncoef4,
                                                                        P.n_active, s4, iv);
            c.launches++;
            CK(cudaGetLastError());
            m.tslot4 = s4;
            m.ninvm = iv;
            if (f32_slot_corners(P.R)) {
                const long long ns4 = 4 * (long long)P.n_active;
                int *tc = nullptr;
                if ((rc = alloc32(c, 4 * (size_t)std::max<long long>(ns4, 1), &tc))) return rc;
                if (ns4 > 0) {
                    k_slot_corners<<<nblocks(ns4, 256), 256, 0, c.stream>>>(m.tslot4, m.econn, tc, ns4);
                    c.launches++;
                    CK(cudaGetLastError());
                }
                m.tcorn4 = tc;
            }
        }
    }
    // the direct gather's per-term corner copies in the list form (with few
    // RHS k_step32 reads the corners from econn)
    m.tcorn = nullptr;
    if (direct && !m.tslot4 && f32_term_corners(P.R)) {
        const long long nt = (long long)P.tlist.size();
        int *tc = nullptr;
        if ((rc = alloc32(c, 4 * (size_t)std::max<long long>(nt, 1), &tc))) return rc;
        if (nt > 0) {
            k_term_corners<<<nblocks(nt, 256), 256, 0, c.stream>>>(m.tlist, m.econn, tc, nt);
            c.launches++;
            CK(cudaGetLastError());
        }
        m.tcorn = tc;
    }
    return EXFEM_OK;
}

// The direct gather's shape: right-hand sides per thread and block size,
// with what depends on them (the state's RHS grouping and the index width).
static void f32_set_shape(Ctx &c, int rpt, int block) {
    const Plan &P = c.plan;
    c.rhs_per_thread = rpt;
    c.block_threads = block;
    c.dm.lg = (rpt < P.R && f32_interleave(P.R)) ? rpt : P.R;
    const unsigned long long lim = 1ull << 32;
    const unsigned long long threads = (unsigned long long)P.n_active * (P.R / rpt) + 1024;
    const unsigned long long state = (unsigned long long)P.nn * 2 * P.R;
    const unsigned long long drm = (unsigned long long)std::max(c.dm.ns, 1) * 8 * P.R;
    c.idx32 = c.opts.index_bits != 64 && threads < lim && state < lim && drm < lim;
}

// exfem_opts.tune: before the state is set up, time every shape of the
// direct gather (RHS per thread 1, 2, 4 dividing R; blocks of 128, 256, 512)
// on the context itself for a few steps from the zero state, and keep the
// fastest.  The steps run from step 1 again for every shape (device counter
// reset), at most min(nsteps, 4) of them, so the receiver slots they write
// stay inside the seismogram buffer; init_explicit then clears it all.
int f32_tune_in_place(Ctx &c) {
    if (c.use_tiles || c.use_pipe || c.use_mma || c.opts.rhs_per_thread > 0 || c.opts.block_threads > 0)
        return EXFEM_OK;
    const int nst = std::min(c.plan.nsteps, 4);
    if (nst < 2) return EXFEM_OK;
    cudaEvent_t a = nullptr, b = nullptr;
    CK(cudaEventCreate(&a));
    CK(cudaEventCreate(&b));
    int best_rpt = c.rhs_per_thread, best_bt = c.block_threads, rc = EXFEM_OK;
    float best = -1.f;
    for (int rpt : {1, 2, 4}) {
        if (c.plan.R % rpt) continue;
        for (int bt : {128, 256, 512}) {
            f32_set_shape(c, rpt, bt);
            if ((rc = f32_init(c))) break;
            if (cudaMemsetAsync(c.dm.d_step, 0, 8 * sizeof(int), c.stream) != cudaSuccess) { rc = EXFEM_E_CUDA; break; }
            if (c.drm_side && (rc = side_mark(c))) break;   // side launches follow the reset
            int par = 0;
            if ((rc = f32_launch_step(c, par))) break;   // warm-up step
            par ^= 1;
            cudaEventRecord(a, c.stream);
            for (int i = 1; i < nst && rc == EXFEM_OK; ++i) {
                rc = f32_launch_step(c, par);
                par ^= 1;
            }
            if (!rc) rc = side_join(c);   // the side stream is idle before the next shape resets the counters
            cudaEventRecord(b, c.stream);
            float ms = 0.f;
            if (rc || cudaEventSynchronize(b) != cudaSuccess || cudaEventElapsedTime(&ms, a, b) != cudaSuccess) {
                if (!rc) rc = EXFEM_E_CUDA;
                break;
            }
            if (best < 0.f || ms < best) { best = ms; best_rpt = rpt; best_bt = bt; }
        }
        if (rc) break;
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    if (rc) { if (c.err.empty()) c.err = "shape tuning failed"; return rc; }
    f32_set_shape(c, best_rpt, best_bt);
    return EXFEM_OK;
}

int f32_init(Ctx &c) {
    size_t nst = (size_t)c.plan.nn * 2 * c.plan.R;
    CK(cudaMemsetAsync(c.uhi[0], 0, nst * sizeof(float), c.stream));
    CK(cudaMemsetAsync(c.uhi[1], 0, nst * sizeof(float), c.stream));
    CK(cudaMemsetAsync(c.ucomp, 0, nst * sizeof(unsigned short), c.stream));
    CK(cudaMemsetAsync(c.udel[0], 0, nst * sizeof(float), c.stream));
    CK(cudaMemsetAsync(c.dcomp, 0, nst * sizeof(unsigned short), c.stream));
    const DevModel &m = c.dm;
    if (m.point_kind == EXFEM_POINT_DISP && m.npoint > 0) {
        const double v0 = point_ricker(m.point_amp, m.point_sigma, 0.0 - m.point_t0);
        const double vm = point_ricker(m.point_amp, m.point_sigma, -m.dt - m.point_t0);
        k_point_init32<<<nblocks((long long)m.npoint * m.R, 128), 128, 0, c.stream>>>(m, c.uhi[0], c.ucomp, c.udel[0],
                                                                                      c.dcomp, v0, vm);
        c.launches++;
        CK(cudaGetLastError());
    }
    return EXFEM_OK;
}

// k_step32 with 32- or 64-bit indices as the context allows.
template <int RPT, bool TC, bool PAIR, bool SLOT>
static cudaError_t step32(Ctx &c, const DevModel &m, int nb, int T, const float *uh, float *uhn) {
    if (c.opts.variant == 4) {   // persistent: the blocks that fit at once stride over the tiles
        if (c.persist_grid <= 0) {
            int per = 0;
            if (c.idx32) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_step32p<RPT, true, TC, PAIR, SLOT>, T, 0);
            else cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_step32p<RPT, false, TC, PAIR, SLOT>, T, 0);
            c.persist_grid = std::max(1, per) * c.num_sms;
        }
        const int g = std::min(nb, c.persist_grid);
        if (c.idx32)
            return launch_dep(c, k_step32p<RPT, true, TC, PAIR, SLOT>, g, T, m, uh, uhn, c.ucomp, c.udel[0], c.dcomp,
                              (unsigned)nb);
        return launch_dep(c, k_step32p<RPT, false, TC, PAIR, SLOT>, g, T, m, uh, uhn, c.ucomp, c.udel[0], c.dcomp,
                          (unsigned)nb);
    }
    if (c.idx32) return launch_dep(c, k_step32<RPT, true, TC, PAIR, SLOT>, nb, T, m, uh, uhn, c.ucomp, c.udel[0], c.dcomp);
    return launch_dep(c, k_step32<RPT, false, TC, PAIR, SLOT>, nb, T, m, uh, uhn, c.ucomp, c.udel[0], c.dcomp);
}

// The direct gather's kernel for the context's shape: RHS per thread, term
// corners (copies or econn), paired rows, slot records or lists.
template <bool SLOT>
static int step32_pick(Ctx &c, const DevModel &m, int nb, int T, const float *uh, float *uhn) {
    const int rpt = c.rhs_per_thread;
    // rows paired when the state is grouped by the thread's RHS (or a thread
    // holds the whole node)
    const bool pair = m.lg == rpt;
    const bool tc = SLOT ? m.tcorn4 != nullptr : m.tcorn != nullptr;
    cudaError_t e = cudaSuccess;
    if (!tc) {   // few RHS (f32_term_corners, f32_slot_corners): corners from econn
        // below 64 RHS the direct gather's state is always grouped by the
        // thread's RHS (f32_alloc), so these rows are always paired
        static_assert(f32_term_corners(63) && f32_slot_corners(63) && f32_interleave(63),
                      "econn corners only below 64 RHS, with grouped rows");
        if (!pair) {
            c.err = "internal: few-RHS step on the plain layout";
            return EXFEM_E_STATE;
        }
        switch (rpt) {
            case 4: e = step32<4, false, true, SLOT>(c, m, nb, T, uh, uhn); break;
            case 2: e = step32<2, false, true, SLOT>(c, m, nb, T, uh, uhn); break;
            default: e = step32<1, false, true, SLOT>(c, m, nb, T, uh, uhn); break;
        }
    } else {
        switch (rpt) {
            case 4:
                if (pair) e = step32<4, true, true, SLOT>(c, m, nb, T, uh, uhn);
                else e = step32<4, true, false, SLOT>(c, m, nb, T, uh, uhn);
                break;
            case 2:
                if (pair) e = step32<2, true, true, SLOT>(c, m, nb, T, uh, uhn);
                else e = step32<2, true, false, SLOT>(c, m, nb, T, uh, uhn);
                break;
            default:
                if (pair) e = step32<1, true, true, SLOT>(c, m, nb, T, uh, uhn);
                else e = step32<1, true, false, SLOT>(c, m, nb, T, uh, uhn);
                break;
        }
    }
    if (e != cudaSuccess) {
        c.err = std::string("step kernel launch: ") + cudaGetErrorString(e);
        return EXFEM_E_CUDA;
    }
    return EXFEM_OK;
}

int f32_launch_step(Ctx &c, int par) {
    DevModel m = c.dm;
    float *uh = c.uhi[par], *uhn = c.uhi[par ^ 1];
    // This step's DRM forces came from the previous step's k_hang32 (or for
    // step 1 from the step-0 sample).  With few RHS they come instead from a
    // k_drm32 on the side stream, into slot `par` of two: step k reads slot
    // (k - 1) & 1, and while it runs the side stream computes step k + 1's
    // forces into the other slot, once step k - 1 (which read that slot) is
    // done.  Under exfem_gpu_profile_kernels it runs on the main stream, so the
    // per-launch marks time it alone.
    if (c.drm_side) {
        m.fdrm32 = c.fdrm_slot[par];
        DevModel md = c.dm;
        md.fdrm32 = c.fdrm_slot[par ^ 1];
        const long long WD = (long long)md.ns * md.R;   // four threads per (DRM element, rhs)
        const int ipd = spread_per_block(WD, c.num_sms, 64);
        const int rc = side_drm_next(c, par, [&](cudaStream_t st) {
            k_drm32<<<spread_blocks(WD, ipd), 256, 0, st>>>(md, ipd);
            mark(c, "k_drm32");
        });
        if (rc) { c.err = "side-stream DRM launch failed"; return rc; }
        c.launches++;
    }
    const int T = c.block_threads;
    const int rpt = c.rhs_per_thread;
    long long work = (long long)m.n_active * (m.R / rpt);
    if (c.use_mma) {
        MmaArgs ma{c.mma_nptr, c.mma_eptr, c.mma_elist, c.mma_tj, c.mma_btile,
                   c.opts.wait_cycles > 0 ? (long long)c.opts.wait_cycles : PIPE_WAIT_CYCLES};
        k_mma32<<<(unsigned)c.mma_ntiles * (unsigned)(m.R / kMmaRc), kMmaThreads, kMmaSmem, c.stream>>>(
            m, ma, uh, uhn, c.ucomp, c.udel[0], c.dcomp);
        c.launches++;
        mark(c, "k_mma32");
    } else if (c.use_pipe) {
        PipeArgs pa{static_cast<const int4 *>(c.p_hdr), static_cast<const int2 *>(c.p_runs),
                    static_cast<const int4 *>(c.p_nrec), static_cast<const int4 *>(c.p_tpack), c.t_lslot,
                    c.tile_tn, c.tile_n, c.pipe_nstage, c.pipe_stage,
                    c.pipe_off[0], c.pipe_off[1], c.pipe_off[2], c.pipe_off[3], c.pipe_off[4], c.pipe_off[5],
                    c.opts.wait_cycles > 0 ? (long long)c.opts.wait_cycles : PIPE_WAIT_CYCLES};
        const int threads = c.pipe_threads;
        switch (rpt) {
            case 4: k_pipe32<4><<<c.pipe_grid, threads, c.tile_smem, c.stream>>>(m, pa, uh, uhn, c.ucomp, c.udel[0], c.dcomp); break;
            case 2: k_pipe32<2><<<c.pipe_grid, threads, c.tile_smem, c.stream>>>(m, pa, uh, uhn, c.ucomp, c.udel[0], c.dcomp); break;
            default: k_pipe32<1><<<c.pipe_grid, threads, c.tile_smem, c.stream>>>(m, pa, uh, uhn, c.ucomp, c.udel[0], c.dcomp); break;
        }
        c.launches++;
        mark(c, "k_pipe32");
    } else if (c.use_tiles) {
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
    const int nb = nblocks(work, T);
    const int rc = m.tslot4 ? step32_pick<true>(c, m, nb, T, uh, uhn) : step32_pick<false>(c, m, nb, T, uh, uhn);
    if (rc) return rc;
    c.launches++;
    mark(c, c.opts.variant == 4 ? "k_step32p" : "k_step32");
    }
    if (c.drm_side) {   // the side stream's next launch may overwrite the slot this step read
        int rc = side_mark(c);
        // The next step's forces (queued on the side stream above) are
        // waited for here, before this step's hanging pass, not just before
        // the next step kernel: that kernel is a programmatic dependent of
        // the hanging pass and follows it with no event wait in between, so
        // its order after the forces rests on the hanging pass's ordinary
        // launch.  (With the FP64 element kernel launched as a programmatic
        // dependent directly after such an event wait, its step read wrong
        // DRM forces: seismograms off by up to 94%.)
        if (!rc) rc = side_join(c);
        if (rc) return rc;
    }
    if (c.p32_n > 0) {
        k_point32<<<nblocks((long long)c.p32_n * m.R, 128), 128, 0, c.stream>>>(m, c.p32_node, c.p32_w, c.p32_n, uhn,
                                                                               c.ucomp, c.udel[0], c.dcomp);
        c.launches++;
        mark(c, "k_point32");
    }
    const int TH = 256;
    int nbh = (int)std::max<long long>(1, ((long long)m.n_hang * m.R + TH - 1) / TH);
    const long long WR = (long long)m.nrecv * m.R;   // four threads per (receiver, rhs)
    const int ipb = spread_per_block(WR, c.num_sms, TH / 4);
    const int nbr = WR > 0 ? spread_blocks(WR, ipb) : 0;
    const long long WD = c.drm_side ? 0 : (long long)m.ns * m.R;   // four threads per (DRM element, rhs)
    const int ipd = spread_per_block(WD, c.num_sms, TH / 4);
    const int nbd = WD > 0 ? spread_blocks(WD, ipd) : 0;
    // an ordinary launch: as a programmatic dependent of the step kernel
    // (its blocks resident early, waiting) it measured up to 10% slower on
    // one-wave meshes; it lets the next step kernel launch early (pdl_trigger)
    k_hang32<<<nbh + nbr + nbd, TH, 0, c.stream>>>(m, uh, uhn, c.ucomp, c.udel[0], c.dcomp, nbh, 0, ipb, nbr, ipd);
    c.launches++;
    mark(c, "k_hang32");
    CK(cudaGetLastError());
    return EXFEM_OK;
}

int f32_launch_sample0(Ctx &c, int par) {
    DevModel m = c.dm;
    if (c.drm_side) m.fdrm32 = c.fdrm_slot[0];   // step 1 reads slot 0
    c.drm_wait[0] = c.drm_wait[1] = false;
    c.ev_step_valid = false;
    const int TH = 256;
    const long long WR = (long long)m.nrecv * m.R;   // four threads per (receiver, rhs)
    const int ipb = spread_per_block(WR, c.num_sms, TH / 4);
    const int nbr = WR > 0 ? spread_blocks(WR, ipb) : 0;
    const long long WD = (long long)m.ns * m.R;      // DRM forces of step 1
    const int ipd = spread_per_block(WD, c.num_sms, TH / 4);
    const int nbd = WD > 0 ? spread_blocks(WD, ipd) : 0;
    if (nbr + nbd > 0) {
        k_hang32<<<nbr + nbd, TH, 0, c.stream>>>(m, c.uhi[par], c.uhi[par], c.ucomp, c.udel[0], c.dcomp, 0, 1, ipb,
                                                  nbr, ipd);
        c.launches++;
    }
    CK(cudaGetLastError());
    return EXFEM_OK;
}

float bf16_to_float(unsigned short h) {
    unsigned w = (unsigned)h << 16;
    float f;
    std::memcpy(&f, &w, sizeof(f));
    return f;
}

}  // namespace exfem
