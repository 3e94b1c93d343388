// Wake potentials of a batch on the tensor cores (included by batch.cu).
//
// For bunches sharing a mesh size n and an impedance, the wake of step k is
// the product of one Toeplitz matrix with their profiles of step k-1:
//     wake[b][x] = s_b * sum_m T[x][m] P[b][m],  T[x][m] = w[(x-m) mod nmax]
// (the unnormalised irfft of the impedance, src/PS/ElectricField.cpp:
// 186-253).  k_wake_tc computes D[x][b] = sum_m T[x][m] P[b][m] with
// tcgen05.mma kind::tf32 in three products per K step, T_hi P_hi + T_hi P_lo
// + T_lo P_hi, where v = v_hi + v_lo and v_hi keeps the 19 leading bits of
// v (so it is exact in TF32); the products accumulate in FP32 in tensor
// memory.  The dropped T_lo P_lo term and the TF32 rounding of the lo
// parts are below 2^-20 of each product: FP32-level accuracy.
//
// One CTA (4 warps) per tile of 128 mesh rows x 64 bunches; K in chunks of
// 32 (128 bytes of TF32 per row) staged in shared memory in the 128-byte
// swizzled K-major layout (8-row atoms of 1024 bytes; the 16-byte chunk c
// of row r sits at chunk c ^ (r & 7)); one thread issues the MMAs and
// commits them to an mbarrier that every thread waits on (bounded) before
// the chunk is overwritten.  The accumulator (128 lanes x 64 columns of
// FP32) is read back with tcgen05.ld, one 32-lane slice per warp.
#pragma once

#include <cstring>

#include "vfps_internal.cuh"

namespace {

constexpr int TC_M = 128;         // mesh rows per tile (TMEM lanes)
constexpr int TC_N = 64;          // bunches per tile (TMEM columns)
constexpr int TC_K = 32;          // K of one staged chunk (128 bytes)
constexpr int TC_THREADS = 128;
constexpr uint32_t TC_A_BYTES = TC_M * TC_K * 4;   // 16 KiB per plane
constexpr uint32_t TC_B_BYTES = TC_N * TC_K * 4;   //  8 KiB per plane
// A_hi, A_lo, B_hi, B_lo (1024-byte aligned), then the barrier, the TMEM
// address and the tile's bunch table; +1024 to align the dynamic base
constexpr uint32_t TC_SMEM = 1024 + 2 * TC_A_BYTES + 2 * TC_B_BYTES + 1024;

// one tile of bunches sharing n and the impedance
struct TcGroup {
    uint32_t n;          // mesh size
    uint32_t t_off;      // T_hi at t_off, T_lo at t_off + n * n
    uint32_t nbt;        // bunches in this tile (<= TC_N)
    uint32_t list_off;   // their indices: list[list_off .. + nbt)
};

__host__ __device__ inline float tf32_hi(float v)
{
#ifdef __CUDA_ARCH__
    return __uint_as_float(__float_as_uint(v) & 0xFFFFE000u);
#else
    uint32_t u;
    std::memcpy(&u, &v, 4);
    u &= 0xFFFFE000u;
    float h;
    std::memcpy(&h, &u, 4);
    return h;
#endif
}

// shared-memory matrix descriptor: K-major, 128-byte swizzle, 8-row atoms
// 1024 bytes apart (stride byte offset), descriptor version 1
__device__ __forceinline__ uint64_t sdesc_sw128(uint32_t saddr)
{
    uint64_t d = uint64_t((saddr >> 4) & 0x3FFFu);
    d |= uint64_t(1) << 16;                 // leading byte offset (unused)
    d |= uint64_t(1024 >> 4) << 32;         // stride byte offset
    d |= uint64_t(1) << 46;                 // version
    d |= uint64_t(2) << 61;                 // SWIZZLE_128B
    return d;
}

// instruction descriptor: D F32, A and B TF32, both K-major, M x N
__host__ __device__ constexpr uint32_t idesc_tf32(int m, int n)
{
    return (1u << 4) | (2u << 7) | (2u << 10)
           | (uint32_t(n >> 3) << 17) | (uint32_t(m >> 4) << 24);
}

__device__ __forceinline__ void tc_mma_tf32(uint32_t d, uint64_t a,
                                            uint64_t b, uint32_t idesc,
                                            uint32_t acc)
{
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}"
        :: "r"(d), "l"(a), "l"(b), "r"(idesc), "r"(acc) : "memory");
}

__device__ __forceinline__ void tc_commit(uint64_t* bar)
{
    asm volatile(
        "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster"
        ".b64 [%0];" :: "r"(smem_addr(bar)) : "memory");
}

__device__ __forceinline__ void tc_fence_before()
{
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}

__device__ __forceinline__ void tc_fence_after()
{
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

// 16 columns of this warp's 32 lanes: v[j] = D[lane][col + j]
__device__ __forceinline__ void tc_ld16(uint32_t taddr, float* v)
{
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
        "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]),
          "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]), "=r"(r[9]),
          "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]),
          "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int j = 0; j < 16; j++) {
        v[j] = __uint_as_float(r[j]);
    }
}

// store the 16-byte chunk c of row r of a swizzled K-major tile
__device__ __forceinline__ void sw128_store(uint8_t* tile, int r, int c,
                                            float4 v)
{
    *reinterpret_cast<float4*>(tile + r * 128 + ((c ^ (r & 7)) << 4)) = v;
}

__global__ void __launch_bounds__(TC_THREADS)
k_wake_tc(const BDev* __restrict__ bd, const TcGroup* __restrict__ groups,
          const uint32_t* __restrict__ list,
          const float* __restrict__ tplanes, const float* __restrict__ pin,
          float* __restrict__ wake, int* __restrict__ status)
{
    extern __shared__ uint8_t tc_raw[];
    const TcGroup G = groups[blockIdx.y];
    const int n = int(G.n);
    const int x0 = int(blockIdx.x) * TC_M;
    if (x0 >= n) {
        return;    // the whole CTA, before any barrier or allocation
    }
    uint8_t* base = reinterpret_cast<uint8_t*>(
        (reinterpret_cast<uintptr_t>(tc_raw) + 1023) & ~uintptr_t(1023));
    uint8_t* a_hi = base;
    uint8_t* a_lo = a_hi + TC_A_BYTES;
    uint8_t* b_hi = a_lo + TC_A_BYTES;
    uint8_t* b_lo = b_hi + TC_B_BYTES;
    uint64_t* bar = reinterpret_cast<uint64_t*>(b_lo + TC_B_BYTES);
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bar + 1);
    uint32_t* poff = tmem_slot + 4;                  // [TC_N]
    float* scale = reinterpret_cast<float*>(poff + TC_N);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int nbt = int(G.nbt);

    if (tid < TC_N) {
        if (tid < nbt) {
            const BDev B = bd[list[G.list_off + tid]];
            poff[tid] = B.prof_off;
            scale[tid] = B.wakescale;
        } else {
            poff[tid] = 0;
            scale[tid] = 0.f;
        }
    }
    if (tid == 0) {
        mbar_init(bar, 1);
        mbar_fence_init();
    }
    if (warp == 0) {
        asm volatile(
            "tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
            :: "r"(smem_addr(tmem_slot)), "r"(uint32_t(TC_N)) : "memory");
        asm volatile(
            "tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;"
            ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *reinterpret_cast<volatile uint32_t*>(tmem_slot);

    const float* t_hi = tplanes + G.t_off;
    const float* t_lo = t_hi + size_t(n) * n;
    const uint32_t idesc = idesc_tf32(TC_M, TC_N);
    const int nchunks = n / TC_K;
    bool ok = true;
    for (int kc = 0; kc < nchunks && ok; kc++) {
        const int m0 = kc * TC_K;
        // A: 128 rows x 8 chunks of 16 bytes, hi and lo planes
        for (int i = tid; i < TC_M * 8; i += TC_THREADS) {
            const int r = i >> 3, c = i & 7;
            const int x = x0 + r;
            float4 h = make_float4(0.f, 0.f, 0.f, 0.f), l = h;
            if (x < n) {
                h = *reinterpret_cast<const float4*>(
                    t_hi + size_t(x) * n + m0 + 4 * c);
                l = *reinterpret_cast<const float4*>(
                    t_lo + size_t(x) * n + m0 + 4 * c);
            }
            sw128_store(a_hi, r, c, h);
            sw128_store(a_lo, r, c, l);
        }
        // B: 64 bunch rows x 8 chunks, split into hi and lo here
        for (int i = tid; i < TC_N * 8; i += TC_THREADS) {
            const int j = i >> 3, c = i & 7;
            float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
            if (j < nbt) {
                v = *reinterpret_cast<const float4*>(pin + poff[j] + m0
                                                     + 4 * c);
            }
            const float4 h = make_float4(tf32_hi(v.x), tf32_hi(v.y),
                                         tf32_hi(v.z), tf32_hi(v.w));
            const float4 l = make_float4(v.x - h.x, v.y - h.y, v.z - h.z,
                                         v.w - h.w);
            sw128_store(b_hi, j, c, h);
            sw128_store(b_lo, j, c, l);
        }
        // the tensor cores read shared memory through the async proxy
        fence_proxy_async();
        tc_fence_before();
        __syncthreads();
        tc_fence_after();
        if (tid == 0) {
            const uint32_t sa_hi = smem_addr(a_hi), sa_lo = smem_addr(a_lo);
            const uint32_t sb_hi = smem_addr(b_hi), sb_lo = smem_addr(b_lo);
#pragma unroll
            for (int kk = 0; kk < TC_K / 8; kk++) {
                // 8 TF32 of K = 32 bytes further into each 128-byte row
                const uint32_t o = uint32_t(kk) * 32u;
                const uint32_t acc = (kc > 0 || kk > 0) ? 1u : 0u;
                tc_mma_tf32(tmem, sdesc_sw128(sa_hi + o),
                            sdesc_sw128(sb_hi + o), idesc, acc);
                tc_mma_tf32(tmem, sdesc_sw128(sa_hi + o),
                            sdesc_sw128(sb_lo + o), idesc, 1u);
                tc_mma_tf32(tmem, sdesc_sw128(sa_lo + o),
                            sdesc_sw128(sb_hi + o), idesc, 1u);
            }
            tc_commit(bar);
        }
        // all MMAs of this chunk done before its operands are overwritten
        bool done = mbar_wait_bounded(bar, uint32_t(kc & 1), WAIT_NS);
        if (!done) {
            atomicCAS(status, 0, VFPS_ERR_TIMEOUT);
            mbar_wait_bounded(bar, uint32_t(kc & 1), WAIT_NS);
        }
        ok = __syncthreads_and(done) != 0;   // the same for every thread
    }
    tc_fence_after();
    if (ok) {
        // warp w reads lanes 32w..32w+31 (rows x0 + 32w + lane)
        const int x = x0 + 32 * warp + lane;
        const uint32_t ta = tmem + (uint32_t(32 * warp) << 16);
#pragma unroll
        for (int c0 = 0; c0 < TC_N; c0 += 16) {
            float v[16];
            tc_ld16(ta + uint32_t(c0), v);
            if (x < n) {
#pragma unroll
                for (int j = 0; j < 16; j++) {
                    if (c0 + j < nbt) {
                        wake[poff[c0 + j] + x] = __fmul_rn(scale[c0 + j],
                                                           v[j]);
                    }
                }
            }
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) {
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;"
                     :: "r"(tmem), "r"(uint32_t(TC_N)) : "memory");
    }
}

}  // namespace
