// exfem_tc.cuh — the 5th-generation tensor-core (tcgen05) pieces of the
// tensor-core FP32 step: TMEM allocation, shared-memory matrix descriptors,
// the kind::tf32 MMA with its commit to an mbarrier, and the TMEM read-back.
//
// Operand layout: K-major, no swizzle.  A row-major tile of `rows` x 8 tf32
// values (32 bytes a row) is stored as 8-row x 16-byte core matrices: the two
// core matrices of a row group (K values 0-3 and 4-7) are 128 bytes apart
// (the descriptor's leading-dimension offset) and row groups are 256 bytes
// apart (its stride-dimension offset).  Element (row, k) is at byte
// tc_kmaj_off(row, k).  D (M = 128 rows, N = 16 columns, FP32) lives in TMEM:
// row i in lane i, column j in column base + j.
#pragma once

#include <cstdint>
#include <cstring>
#include <vector>

#include "exfem_device.cuh"

namespace exfem {

constexpr unsigned kTcLbo = 128;   // bytes between the K-adjacent core matrices of a row group
constexpr unsigned kTcSbo = 256;   // bytes between row groups

__device__ __forceinline__ unsigned tc_kmaj_off(int row, int k) {
    return (unsigned)((row >> 3) * kTcSbo + (k >> 2) * kTcLbo + (row & 7) * 16 + (k & 3) * 4);
}

// Shared-memory matrix descriptor: start address, leading and stride byte
// offsets (each >> 4), descriptor version 1, base offset 0, no swizzle.
__device__ __forceinline__ uint64_t tc_smem_desc(unsigned saddr) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr >> 4) & 0x3FFFu);
    d |= (uint64_t)((kTcLbo >> 4) & 0x3FFFu) << 16;
    d |= (uint64_t)((kTcSbo >> 4) & 0x3FFFu) << 32;
    d |= (uint64_t)1 << 46;
    return d;
}

// Instruction descriptor of kind::tf32: D in FP32, A and B tf32, both K-major,
// N >> 3 and M >> 4.
__host__ __device__ constexpr uint32_t tc_idesc_tf32(int M, int N) {
    return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

// TMEM columns: the whole warp calls alloc/dealloc; the base address is
// written to shared memory at `slot`.
__device__ __forceinline__ void tc_alloc(unsigned slot_saddr, unsigned ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(slot_saddr), "r"(ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tc_dealloc(uint32_t taddr, unsigned ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// D[tmem] (+)= A[smem] * B[smem]^T, M x N x 8, issued by one thread.
__device__ __forceinline__ void tc_mma_tf32(uint32_t d_tmem, uint64_t a_desc, uint64_t b_desc, uint32_t idesc,
                                            int accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
        "l"(a_desc), "l"(b_desc), "r"(idesc), "r"(accumulate)
        : "memory");
}

// Arrives on the mbarrier once every MMA this thread issued has completed.
__device__ __forceinline__ void tc_commit(unsigned mbar_saddr) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar_saddr)
                 : "memory");
}

// 16 consecutive FP32 columns of this thread's lane (the warp reads lanes
// 32*(warp % 4) .. +31: taddr carries that lane base in bits 16-31).
__device__ __forceinline__ void tc_ld16(uint32_t taddr, float (&v)[16]) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int j = 0; j < 16; ++j) v[j] = __uint_as_float(r[j]);
}

// Round to tf32 (nearest, ties away): the value the tensor core multiplies.
__device__ __forceinline__ float tc_tf32(float x) {
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
    return __uint_as_float(r);
}

// [Kmu; Klambda] of the square Q4 element (the stiffness for (mu, lambda) =
// (1, 0) and (0, 1), from the closed form of q4_fold/q4_corner_acc in FP64:
// row 2c + d is the force on corner c, dof d, for unit corner dofs), split
// into tf32 hi and lo parts and laid out as the K-major operand tile.
inline std::vector<float> tc_b_operand_q4() {
    auto tf32 = [](double x) {   // round to nearest, ties away, to a 10-bit mantissa
        float f = (float)x;
        uint32_t u;
        std::memcpy(&u, &f, 4);
        u = (u + 0x1000u) & 0xFFFFE000u;
        std::memcpy(&f, &u, 4);
        return f;
    };
    std::vector<float> out(256, 0.f);
    for (int part = 0; part < 2; ++part) {     // mu, lambda
        const double mu = part == 0 ? 1.0 : 0.0, lam = part == 0 ? 0.0 : 1.0;
        const double A = (lam + 2 * mu) / 4, B = lam / 4, Cc = mu / 4, D = (lam + 3 * mu) / 12;
        for (int c = 0; c < 4; ++c)
            for (int j = 0; j < 8; ++j) {
                double ux[4] = {0, 0, 0, 0}, uy[4] = {0, 0, 0, 0};
                (j & 1 ? uy : ux)[j >> 1] = 1.0;
                double ax = 0.0, ay = 0.0;
                q4_corner_acc<double>(q4_fold<double>(A, B, Cc, D, c, 1.0), ux, uy, ax, ay);
                for (int d = 0; d < 2; ++d) {
                    const double kv = -(d == 0 ? ax : ay);   // K[2c + d][j]
                    const int n = part * 8 + 2 * c + d;
                    const float hi = tf32(kv), lo = tf32(kv - (double)hi);
                    const int off = ((n >> 3) * (int)kTcSbo + (j >> 2) * (int)kTcLbo + (n & 7) * 16 + (j & 3) * 4) / 4;
                    out[off] = hi;
                    out[128 + off] = lo;
                }
            }
    }
    return out;
}

}  // namespace exfem
