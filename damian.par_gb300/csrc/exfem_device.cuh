// exfem_device.cuh — device functions shared by the kernels.
#pragma once

#include <cuda_runtime.h>

#include "exfem_ctx.h"

// Programmatic dependent launch (griddepcontrol): pdl_wait blocks the thread
// until the grids this one depends on have completed and their writes are
// visible (at once in a grid launched without the attribute); pdl_trigger
// lets the next grid of the stream launch once every block of this one has
// issued it or exited.  A kernel launched as a programmatic dependent touches
// nothing an earlier kernel writes, and writes nothing an earlier kernel
// reads, before its pdl_wait.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

namespace exfem {

// Offset of (dof d, rhs r) within a node's 2R state values, or within a DRM
// corner's force pair.  The right-hand sides form groups of m.lg, and each
// group holds its x row, then its y row.  lg = R is the plain layout (every
// RHS's x, then every RHS's y); lg = the FP32 direct gather's RHS per thread
// puts a thread's x and y values of a node side by side, so that it loads
// and stores them as one vector.
__host__ __device__ __forceinline__ size_t row_off(const DevModel &m, int d, int r) {
    const int g = r / m.lg;
    return (size_t)g * 2 * m.lg + (size_t)d * m.lg + (size_t)(r - g * m.lg);
}
__host__ __device__ __forceinline__ size_t state_at(const DevModel &m, size_t n, int d, int r) {
    return n * 2 * (size_t)m.R + row_off(m, d, r);
}

// Q4 square plane-strain stiffness applied to one element's corner
// displacements, K(mu, lambda) u with K = calck(mu, lambda)
// (formulation.f90:276-313).  The bilinear field is split into its modes
// c1 = d/dxi, c2 = d/deta, c3 = xi*eta per component; the fully integrated
// energy of the square element is
//   2(l+2m)(c1x^2 + c2y^2) + 4 l c1x c2y + 2 m (c2x + c1y)^2 + (2/3)(l+3m)(c3x^2 + c3y^2)
// (modes scaled by 1/4), whose gradient gives the eight nodal forces with
// about 34 operations instead of the 64 multiply-adds of the dense 8x8 product.
// k = ((l+2m)/4, l/4, m/4, (l+3m)/12); corners in CSR order TL, TR, BR, BL.
template <typename T>
__host__ __device__ __forceinline__ void q4_ku(T A, T B, T C, T D, const T ux[4], const T uy[4], T fx[4], T fy[4]) {
    T px = ux[2] - ux[0], qx = ux[1] - ux[3];
    T c1x = px + qx, c2x = px - qx, c3x = (ux[0] + ux[2]) - (ux[1] + ux[3]);
    T py = uy[2] - uy[0], qy = uy[1] - uy[3];
    T c1y = py + qy, c2y = py - qy, c3y = (uy[0] + uy[2]) - (uy[1] + uy[3]);
    T F1 = A * c1x + B * c2y;
    T F2 = A * c2y + B * c1x;
    T S = C * (c2x + c1y);
    T Gx = D * c3x, Gy = D * c3y;
    T ax = F1 + S, bx = F1 - S;
    fx[0] = Gx - ax; fx[1] = bx - Gx; fx[2] = ax + Gx; fx[3] = -(bx + Gx);
    T ay = S + F2, by = S - F2;
    fy[0] = Gy - ay; fy[1] = by - Gy; fy[2] = ay + Gy; fy[3] = -(by + Gy);
}

// Force of corner `c` only (the node-centric gather needs one corner).
template <typename T>
__host__ __device__ __forceinline__ void q4_ku_corner(T A, T B, T C, T D, const T ux[4], const T uy[4], int c, T &fx, T &fy) {
    T px = ux[2] - ux[0], qx = ux[1] - ux[3];
    T c1x = px + qx, c2x = px - qx, c3x = (ux[0] + ux[2]) - (ux[1] + ux[3]);
    T py = uy[2] - uy[0], qy = uy[1] - uy[3];
    T c1y = py + qy, c2y = py - qy, c3y = (uy[0] + uy[2]) - (uy[1] + uy[3]);
    T F1 = A * c1x + B * c2y;
    T F2 = A * c2y + B * c1x;
    T S = C * (c2x + c1y);
    T Gx = D * c3x, Gy = D * c3y;
    // corner sign pattern of (P, Q, G): TL(-,-,+) TR(+,-,-) BR(+,+,+) BL(-,+,-)
    T sP = (c == 1 || c == 2) ? T(1) : T(-1);
    T sQ = (c >= 2) ? T(1) : T(-1);
    T sG = (c == 0 || c == 2) ? T(1) : T(-1);
    fx = sP * F1 + sQ * S + sG * Gx;
    fy = sP * S + sQ * F2 + sG * Gy;
}

// calck (formulation.f90:276-313), column-major k[col*8+row].  Its 64 entries
// are six values with signs, kv = (3m+l)/3, (m+l)/4, (3m+2l)/6, (m-l)/4,
// (3m+l)/6, l/6 (calck_values, exfem_plan.h), computed once per element on
// the host with the formula's operations, as the reference computes m_kmat
// once per material (explicit.f90:139).  Negation is exact, so every entry
// is the formula's own rounding.
__host__ __device__ __forceinline__ void calck(const double kv[6], double k[64]) {
    const double v[64] = {
        kv[0], kv[1], -kv[2], -kv[3], -kv[4], -kv[1], kv[5], kv[3],
        kv[1], kv[0], kv[3], kv[5], -kv[1], -kv[4], -kv[3], -kv[2],
        -kv[2], kv[3], kv[0], -kv[1], kv[5], -kv[3], -kv[4], kv[1],
        -kv[3], kv[5], -kv[1], kv[0], kv[3], -kv[2], kv[1], -kv[4],
        -kv[4], -kv[1], kv[5], kv[3], kv[0], kv[1], -kv[2], -kv[3],
        -kv[1], -kv[4], -kv[3], -kv[2], kv[1], kv[0], kv[3], kv[5],
        kv[5], -kv[3], -kv[4], kv[1], -kv[2], kv[3], kv[0], -kv[1],
        kv[3], -kv[2], kv[1], -kv[4], -kv[3], kv[5], -kv[1], kv[0]};
#pragma unroll
    for (int i = 0; i < 64; ++i) k[i] = v[i];
}

__host__ __device__ __forceinline__ float q4fma(float a, float b, float c) { return fmaf(a, b, c); }
__host__ __device__ __forceinline__ double q4fma(double a, double b, double c) { return fma(a, b, c); }

// q4_ku_corner folded for accumulation.  With s = c2x + c1y,
//   fx = sP A c1x + sP B c2y + sQ C s + sG D c3x
//   fy = sP C s + sQ A c2y + sQ B c1x + sG D c3y,
// so one (element, corner, weight w) term of a node's force sum, -w (fx, fy),
// is 8 multiply-adds on the modes with 7 coefficients scaled by -w and the
// corner's signs, computed once per term (the FP32 kernels' form).
template <typename T>
struct Q4Fold {
    T a0, a1, a2, a3;   // c1x, c2y, s, c3x (and c3y) into x
    T b0, b1, b2;       // s, c2y, c1x into y
};

template <typename T>
__host__ __device__ __forceinline__ Q4Fold<T> q4_fold(T A, T B, T C, T D, int c, T w) {
    const T sP = (c == 1 || c == 2) ? -w : w;
    const T sQ = (c >= 2) ? -w : w;
    const T sG = (c == 0 || c == 2) ? -w : w;
    return Q4Fold<T>{sP * A, sP * B, sQ * C, sG * D, sP * C, sQ * A, sQ * B};
}

// ax += -w fx, ay += -w fy for the folded term f.
template <typename T>
__host__ __device__ __forceinline__ void q4_corner_acc(const Q4Fold<T> &f, const T ux[4], const T uy[4], T &ax,
                                                       T &ay) {
    T px = ux[2] - ux[0], qx = ux[1] - ux[3];
    T c1x = px + qx, c2x = px - qx, c3x = (ux[0] + ux[2]) - (ux[1] + ux[3]);
    T py = uy[2] - uy[0], qy = uy[1] - uy[3];
    T c1y = py + qy, c2y = py - qy, c3y = (uy[0] + uy[2]) - (uy[1] + uy[3]);
    T s = c2x + c1y;
    ax = q4fma(f.a3, c3x, q4fma(f.a2, s, q4fma(f.a1, c2y, q4fma(f.a0, c1x, ax))));
    ay = q4fma(f.a3, c3y, q4fma(f.b2, c1x, q4fma(f.b1, c2y, q4fma(f.b0, s, ay))));
}

// Consistent mass (calcsqm/9, formulation.f90:256-268) times v for one
// component: weights 4 (self), 2 (edge neighbours), 1 (opposite corner).
template <typename T>
__host__ __device__ __forceinline__ void q4_msq(const T v[4], T out[4]) {
    for (int k = 0; k < 4; ++k)
        out[k] = (T(4) * v[k] + T(2) * v[(k + 1) & 3] + v[(k + 2) & 3] + T(2) * v[(k + 3) & 3]) / T(9);
}

// The point-source pulse, ricker (formulation.f90:53-59), in its operation
// order: amp * exp(-t^2/(4 sigma)) (t^2 - 2 sigma) / (8 sqrt(pi) sigma^2.5).
__host__ __device__ __forceinline__ double point_ricker(double amp, double sigma, double t) {
    double r = exp(-(t * t) / (4.0 * sigma)) * (t * t - 2.0 * sigma) /
               (8.0 * sqrt(3.14159265358979323846) * pow(sigma, 2.5));
    return r * amp;
}

// The source's value at step `step` (time step * dt).
__device__ __forceinline__ double point_value(const DevModel &m, int step) {
    return point_ricker(m.point_amp, m.point_sigma, (double)step * m.dt - m.point_t0);
}

// One Ricker term with its first two time derivatives (pwaves.f90:157-169).
__host__ __device__ __forceinline__ void ricker3(double fp, double d, double out[3]) {
    double q = fp * d;
    double v2 = q * q;
    double e = exp(v2);
    out[0] = (1.0 - 2.0 * v2) / e;
    out[1] = (2.0 * v2 - 3.0) * (fp * fp) * d / e;
    out[2] = -2.0 * (4.0 * (v2 * v2) - 12.0 * v2 + 3.0) * (fp * fp) / e;
}

// planewave (pwaves.f90:100-217): u[comp][col], comp x/z, col u/du/ddu.
__host__ __device__ __forceinline__ void planewave(const DevWave &w, double t, double x1, double x3, double ux[3],
                                          double uz[3]) {
    double v0;
    if (w.kind == EXFEM_WAVE_P) v0 = (x1 * w.sine - x3 * w.cose) / w.alpha;
    else v0 = (x1 * w.sinf - x3 * w.cosf) / w.beta;
    double v1 = (x1 * w.sine + x3 * w.cose) / w.alpha;
    double v2 = (x1 * w.sinf + x3 * w.cosf) / w.beta;
    double r0[3], r1[3], r2[3];
    ricker3(w.fp, t - v0, r0);
    ricker3(w.fp, t - v1, r1);
    ricker3(w.fp, t - v2, r2);
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        double ipx = r0[c] * w.wui[0] * w.amp0, ipz = r0[c] * w.wui[1] * w.amp0;
        double rpx = r1[c] * w.wui[2] * w.wa1, rpz = r1[c] * w.wui[3] * w.wa1;
        double rsx = r2[c] * w.wui[4] * w.wb1, rsz = r2[c] * w.wui[5] * w.wb1;
        ux[c] = ipx + rpx + rsx;
        uz[c] = ipz + rpz + rsz;
    }
}

// One term of planewave: m = 0 incident, 1 reflected P, 2 reflected SV.
// pw_term gives the term's parts px[c], pz[c] of ux[c], uz[c] with planewave's
// arithmetic, so planewave's ux[c] is px_0[c] + px_1[c] + px_2[c] summed in
// that order; pw_term_u gives the displacement column alone, as planewave_u
// computes it.  Threads evaluating the terms in parallel reproduce the
// one-thread values bit for bit.
__host__ __device__ __forceinline__ double pw_delay(const DevWave &w, int m, double x1, double x3) {
    if (m == 0) {
        if (w.kind == EXFEM_WAVE_P) return (x1 * w.sine - x3 * w.cose) / w.alpha;
        return (x1 * w.sinf - x3 * w.cosf) / w.beta;
    }
    if (m == 1) return (x1 * w.sine + x3 * w.cose) / w.alpha;
    return (x1 * w.sinf + x3 * w.cosf) / w.beta;
}
__host__ __device__ __forceinline__ void pw_term(const DevWave &w, int m, double t, double x1, double x3,
                                              double px[3], double pz[3]) {
    double r[3];
    ricker3(w.fp, t - pw_delay(w, m, x1, x3), r);
    const double amp = m == 0 ? w.amp0 : (m == 1 ? w.wa1 : w.wb1);
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        px[c] = r[c] * w.wui[2 * m] * amp;
        pz[c] = r[c] * w.wui[2 * m + 1] * amp;
    }
}
// Displacement of one term (the column planewave_u sums).
__host__ __device__ __forceinline__ void pw_term_u(const DevWave &w, int m, double t, double x1, double x3,
                                                double &px, double &pz) {
    const double q = w.fp * (t - pw_delay(w, m, x1, x3));
    const double sq = q * q;
    const double r = (1.0 - 2.0 * sq) / exp(sq);
    const double amp = m == 0 ? w.amp0 : (m == 1 ? w.wa1 : w.wb1);
    px = r * w.wui[2 * m] * amp;
    pz = r * w.wui[2 * m + 1] * amp;
}

// Displacement column only.
__host__ __device__ __forceinline__ void planewave_u(const DevWave &w, double t, double x1, double x3, double &ux,
                                            double &uz) {
    double v0;
    if (w.kind == EXFEM_WAVE_P) v0 = (x1 * w.sine - x3 * w.cose) / w.alpha;
    else v0 = (x1 * w.sinf - x3 * w.cosf) / w.beta;
    double v1 = (x1 * w.sine + x3 * w.cose) / w.alpha;
    double v2 = (x1 * w.sinf + x3 * w.cosf) / w.beta;
    double q0 = w.fp * (t - v0), q1 = w.fp * (t - v1), q2 = w.fp * (t - v2);
    double s0 = q0 * q0, s1 = q1 * q1, s2 = q2 * q2;
    double r0 = (1.0 - 2.0 * s0) / exp(s0), r1 = (1.0 - 2.0 * s1) / exp(s1), r2 = (1.0 - 2.0 * s2) / exp(s2);
    ux = r0 * w.wui[0] * w.amp0 + r1 * w.wui[2] * w.wa1 + r2 * w.wui[4] * w.wb1;
    uz = r0 * w.wui[1] * w.amp0 + r1 * w.wui[3] * w.wa1 + r2 * w.wui[5] * w.wb1;
}

// DRM exterior masks of wave_reactions (model.f90:778-793), bit k = dof k.
__host__ __device__ __forceinline__ unsigned drm_mask(int kind) {
    switch (kind) {
        case 2: return 0xC3u;   // SE_SVERL: T T F F F F T T
        case 4: return 0x3Cu;   // SE_SVERR: F F T T T T F F
        case 1: return 0xF0u;   // SE_SHORI: F F F F T T T T
        case 6: return 0xF3u;   // SE_CORNL: T T F F T T T T
        case 5: return 0xFCu;   // SE_CORNR: F F T T T T T T
        default: return 0u;
    }
}

// Effective DRM forces of one boundary element (wave_reactions,
// model.f90:745-800, with multdrm formulation.f90:378-393 for K and for the
// consistent mass): p = -K_be u0_e on boundary dofs, +K_eb u0_b on exterior
// dofs, plus the same with M_cons*mass on the free-field acceleration.
template <typename T>
__host__ __device__ __forceinline__ void drm_forces(const T k[4], T mass, unsigned e, const T u0[8], const T a0[8],
                                                    T p[8]) {
    T uex[4], uey[4], ubx[4], uby[4];
#pragma unroll
    for (int c = 0; c < 4; ++c) {
        bool ex = (e >> (2 * c)) & 1u, ey = (e >> (2 * c + 1)) & 1u;
        uex[c] = ex ? u0[2 * c] : T(0);       ubx[c] = ex ? T(0) : u0[2 * c];
        uey[c] = ey ? u0[2 * c + 1] : T(0);   uby[c] = ey ? T(0) : u0[2 * c + 1];
    }
    T kex[4], key[4], kbx[4], kby[4];
    q4_ku<T>(k[0], k[1], k[2], k[3], uex, uey, kex, key);
    q4_ku<T>(k[0], k[1], k[2], k[3], ubx, uby, kbx, kby);
    T aex[4], aey[4], abx[4], aby[4];
#pragma unroll
    for (int c = 0; c < 4; ++c) {
        bool ex = (e >> (2 * c)) & 1u, ey = (e >> (2 * c + 1)) & 1u;
        aex[c] = ex ? a0[2 * c] : T(0);       abx[c] = ex ? T(0) : a0[2 * c];
        aey[c] = ey ? a0[2 * c + 1] : T(0);   aby[c] = ey ? T(0) : a0[2 * c + 1];
    }
    T mex[4], mey[4], mbx[4], mby[4];
    q4_msq<T>(aex, mex); q4_msq<T>(aey, mey); q4_msq<T>(abx, mbx); q4_msq<T>(aby, mby);
#pragma unroll
    for (int c = 0; c < 4; ++c) {
        bool ex = (e >> (2 * c)) & 1u, ey = (e >> (2 * c + 1)) & 1u;
        T pkx = ex ? kbx[c] : -kex[c], pky = ey ? kby[c] : -key[c];
        T pmx = ex ? mbx[c] : -mex[c], pmy = ey ? mby[c] : -mey[c];
        p[2 * c] = pkx + pmx * mass;
        p[2 * c + 1] = pky + pmy * mass;
    }
}

// Free-field displacement and acceleration for the FP32 form: the travel
// time t - (x sin + z cos)/v is formed in FP64 (the subtraction cancels), the
// Ricker terms in FP32.  Relative error ~1e-7, the size of storing the forces
// in FP32.
// The FP32 free field's three travel-time delays at (x1, x3): incident,
// reflected P, reflected SV.  They do not depend on time, so the FP32 DRM pass
// reads them precomputed per (DRM corner, rhs) instead of redoing this FP64
// arithmetic every step.
__host__ __device__ __forceinline__ void planewave32_delays(const DevWave &w, double x1, double x3, double v[3]) {
    if (w.kind == EXFEM_WAVE_P) v[0] = (x1 * w.sine - x3 * w.cose) * w.inv_alpha;
    else v[0] = (x1 * w.sinf - x3 * w.cosf) * w.inv_beta;
    v[1] = (x1 * w.sine + x3 * w.cose) * w.inv_alpha;
    v[2] = (x1 * w.sinf + x3 * w.cosf) * w.inv_beta;
}
// planewave32 from its delays.
__host__ __device__ __forceinline__ void planewave32_at(const DevWave &w, double t, const double v[3], float u[2],
                                                        float a[2]) {
    const float fp2 = (float)(w.fp * w.fp);
    const float amp[3] = {(float)w.amp0, (float)w.wa1, (float)w.wb1};
    u[0] = u[1] = a[0] = a[1] = 0.f;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        float q = (float)(w.fp * (t - v[k]));
        float s2 = q * q;
        float e = expf(-s2);
        float r0 = (1.f - 2.f * s2) * e;
        float r2 = -2.f * ((4.f * s2 - 12.f) * s2 + 3.f) * fp2 * e;
        float ax = (float)w.wui[2 * k] * amp[k], az = (float)w.wui[2 * k + 1] * amp[k];
        u[0] += r0 * ax;
        u[1] += r0 * az;
        a[0] += r2 * ax;
        a[1] += r2 * az;
    }
}
__host__ __device__ __forceinline__ void planewave32(const DevWave &w, double t, double x1, double x3, float u[2],
                                                     float a[2]) {
    double v[3];
    planewave32_delays(w, x1, x3, v);
    planewave32_at(w, t, v, u, a);
}

}  // namespace exfem
