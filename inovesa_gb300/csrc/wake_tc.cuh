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
// One CTA (4 warps) per tile of 128 mesh rows x 16 bunches, K in chunks of
// 32 (128 bytes of TF32 per row).  The T operand is constant: the host
// stores each (row tile, chunk) as the byte image of its shared-memory
// tile (hi plane, then lo plane, 128-byte swizzled K-major: 8-row atoms of
// 1024 bytes, the 16-byte chunk c of row r at chunk c ^ (r & 7)), so one
// bulk copy of 32 KiB stages a chunk, up to six chunks in flight.  The
// profiles (the B operand) are split into hi and lo and swizzled by the
// CTA's threads, all chunks at once.  One thread issues the MMAs of a chunk
// as it lands and commits them to that stage's mbarrier, which frees the
// stage for the chunk as many stages further on; every wait is bounded.  The
// accumulator (128 lanes x 16 columns of FP32) is read back with
// tcgen05.ld, one 32-lane slice per warp.
#pragma once

#include <cstring>

#include "vfps_internal.cuh"

namespace {

constexpr int TC_M = 128;         // mesh rows per tile (TMEM lanes)
constexpr int TC_N = 16;          // bunches per tile (TMEM columns)
constexpr int TC_K = 32;          // K of one chunk (128 bytes)
constexpr int TC_THREADS = 128;
constexpr int TC_MAX_STAGES = 6;  // T chunks in flight, at most
constexpr int TC_MAX_N = 1024;    // widest mesh (shared memory of B)
constexpr uint32_t TC_TMEM_COLS = 32;              // smallest allocation
constexpr uint32_t TC_A_BYTES = TC_M * TC_K * 4;   // 16 KiB per plane
constexpr uint32_t TC_B_BYTES = TC_N * TC_K * 4;   //  2 KiB per plane
constexpr uint32_t TC_IMG_FLOATS = TC_M * TC_K;    // floats of one plane

constexpr uint32_t TC_SMEM_MAX = 232448;          // per CTA (227 KiB)

// T chunks in flight for an n-row mesh: as many stages as fit next to all
// of B (at most TC_MAX_STAGES, at most the number of chunks)
__host__ __device__ constexpr int tc_stages(int n)
{
    const int nkc = n / TC_K;
    const int room = int((TC_SMEM_MAX - 1536 - uint32_t(nkc) * 2 * TC_B_BYTES)
                         / (2 * TC_A_BYTES));
    const int s = room < TC_MAX_STAGES ? room : TC_MAX_STAGES;
    return s < nkc ? s : nkc;
}

// dynamic shared memory of an n-row mesh: +1024 to align the base, the T
// stages (hi, lo), every B chunk (hi, lo), barriers and the tile's bunch
// table
__host__ __device__ constexpr uint32_t tc_smem(int n)
{
    return 1024 + uint32_t(tc_stages(n)) * 2 * TC_A_BYTES
           + uint32_t(n / TC_K) * 2 * TC_B_BYTES + 512;
}

// one tile of bunches sharing n and the impedance
struct TcGroup {
    uint32_t n;          // mesh size (a multiple of TC_K, at most TC_MAX_N)
    uint32_t t_off;      // the T images: [row tile][chunk][hi, lo plane]
    uint32_t nbt;        // bunches in this tile (<= TC_N)
    uint32_t list_off;   // their profile offsets and wake scalings (bits):
                         // list[list_off .. + nbt)
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
k_wake_tc(const TcGroup* __restrict__ groups,
          const uint2* __restrict__ list,
          const float* __restrict__ tplanes, const float* __restrict__ pin,
          float* __restrict__ wake, int* __restrict__ status)
{
    extern __shared__ uint8_t tc_raw[];
    const TcGroup G = groups[blockIdx.y];
    const int n = int(G.n);
    const int mt = int(blockIdx.x);
    const int x0 = mt * TC_M;
    if (x0 >= n) {
        return;    // the whole CTA, before any barrier or allocation
    }
    const int nkc = n / TC_K;
    const int stages = tc_stages(n);
    uint8_t* base = reinterpret_cast<uint8_t*>(
        (reinterpret_cast<uintptr_t>(tc_raw) + 1023) & ~uintptr_t(1023));
    uint8_t* a_st = base;                                  // [stage][hi, lo]
    uint8_t* b_ch = a_st + stages * 2 * TC_A_BYTES;        // [chunk][hi, lo]
    uint64_t* full = reinterpret_cast<uint64_t*>(b_ch
                                                 + nkc * 2 * TC_B_BYTES);
    uint64_t* empty = full + TC_MAX_STAGES;
    uint64_t* done = empty + TC_MAX_STAGES;
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(done + 1);
    uint32_t* poff = tmem_slot + 4;                  // [TC_N]
    float* scale = reinterpret_cast<float*>(poff + TC_N);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int nbt = int(G.nbt);
    // this row tile's T images: chunk kc at img + kc * 2 planes
    const float* img = tplanes + G.t_off
                       + size_t(mt) * nkc * 2 * TC_IMG_FLOATS;

    if (tid < TC_N) {
        if (tid < nbt) {
            const uint2 e = list[G.list_off + tid];
            poff[tid] = e.x;
            scale[tid] = __uint_as_float(e.y);
        } else {
            poff[tid] = 0;
            scale[tid] = 0.f;
        }
    }
    int issued[TC_MAX_STAGES] = {};     // thread 0: loads per stage
    if (tid == 0) {
        for (int s = 0; s < stages; s++) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        mbar_init(done, 1);
        mbar_fence_init();
        // the first chunks of T while the profiles are split
        for (int s = 0; s < stages; s++) {
            mbar_arrive_expect_tx(&full[s], 2 * TC_A_BYTES);
            tma_load_1d(a_st + s * 2 * TC_A_BYTES,
                        img + size_t(s) * 2 * TC_IMG_FLOATS, 2 * TC_A_BYTES,
                        &full[s]);
            issued[s]++;
        }
    }
    if (warp == 0) {
        asm volatile(
            "tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
            :: "r"(smem_addr(tmem_slot)), "r"(TC_TMEM_COLS) : "memory");
        asm volatile(
            "tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;"
            ::: "memory");
    }
    __syncthreads();   // poff for the profile loads below
    // B: every chunk of the tile's profiles, split into hi and lo; 8
    // loads per thread in flight at a time
    {
        const int q4 = n >> 2;                 // float4 per profile
        const int total = TC_N * q4;
        for (int i0 = 0; i0 < total; i0 += 8 * TC_THREADS) {
            float4 v[8];
#pragma unroll
            for (int u = 0; u < 8; u++) {
                const int i = i0 + u * TC_THREADS + tid;
                const int j = i / q4, q = i - j * q4;
                v[u] = make_float4(0.f, 0.f, 0.f, 0.f);
                if (i < total && j < nbt) {
                    v[u] = *reinterpret_cast<const float4*>(pin + poff[j]
                                                            + 4 * q);
                }
            }
#pragma unroll
            for (int u = 0; u < 8; u++) {
                const int i = i0 + u * TC_THREADS + tid;
                if (i < total) {
                    const int j = i / q4, q = i - j * q4;
                    const int kc = q >> 3, c = q & 7;
                    const float4 h = make_float4(
                        tf32_hi(v[u].x), tf32_hi(v[u].y), tf32_hi(v[u].z),
                        tf32_hi(v[u].w));
                    const float4 l = make_float4(
                        v[u].x - h.x, v[u].y - h.y, v[u].z - h.z,
                        v[u].w - h.w);
                    uint8_t* t = b_ch + kc * 2 * TC_B_BYTES;
                    sw128_store(t, j, c, h);
                    sw128_store(t + TC_B_BYTES, j, c, l);
                }
            }
        }
    }
    // the tensor cores read shared memory through the async proxy
    fence_proxy_async();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *reinterpret_cast<volatile uint32_t*>(tmem_slot);

    bool ok = true;    // thread 0: every chunk arrived in time
    if (tid == 0) {
        const uint32_t idesc = idesc_tf32(TC_M, TC_N);
        int consumed[TC_MAX_STAGES] = {};
        for (int kc = 0; kc < nkc; kc++) {
            const int s = kc % stages;
            if (!mbar_wait_bounded(&full[s], uint32_t(consumed[s] & 1),
                                   WAIT_NS)) {
                ok = false;
                break;
            }
            consumed[s]++;
            tc_fence_after();
            const uint32_t sa_hi = smem_addr(a_st + s * 2 * TC_A_BYTES);
            const uint32_t sa_lo = sa_hi + TC_A_BYTES;
            const uint32_t sb_hi = smem_addr(b_ch + kc * 2 * TC_B_BYTES);
            const uint32_t sb_lo = sb_hi + TC_B_BYTES;
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
            tc_commit(&empty[s]);
            // the previous chunk's stage takes the chunk `stages` after it
            // once its products are done
            const int kp = kc - 1;
            if (kp >= 0 && kp + stages < nkc) {
                const int sp = kp % stages;
                if (!mbar_wait_bounded(&empty[sp],
                                       uint32_t((kp / stages) & 1),
                                       WAIT_NS)) {
                    ok = false;
                    break;
                }
                mbar_arrive_expect_tx(&full[sp], 2 * TC_A_BYTES);
                tma_load_1d(a_st + sp * 2 * TC_A_BYTES,
                            img + size_t(kp + stages) * 2 * TC_IMG_FLOATS,
                            2 * TC_A_BYTES, &full[sp]);
                issued[sp]++;
            }
        }
        // every product issued so far completes before done arrives
        tc_commit(done);
        if (!ok) {
            atomicCAS(status, 0, VFPS_ERR_TIMEOUT);
            // the copies still in flight land before the CTA ends
            for (int s = 0; s < stages; s++) {
                while (consumed[s] < issued[s]) {
                    mbar_wait_bounded(&full[s], uint32_t(consumed[s] & 1),
                                      WAIT_NS);
                    consumed[s]++;
                }
            }
        }
    }
    bool fin = mbar_wait_bounded(done, 0u, WAIT_NS);
    if (!fin && tid == 0) {
        atomicCAS(status, 0, VFPS_ERR_TIMEOUT);
    }
    const bool all = __syncthreads_and(fin && ok) != 0;
    tc_fence_after();
    if (all) {
        // warp w reads lanes 32w..32w+31 (rows x0 + 32w + lane)
        const int x = x0 + 32 * warp + lane;
        const uint32_t ta = tmem + (uint32_t(32 * warp) << 16);
        float v[16];
        tc_ld16(ta, v);
        if (x < n) {
#pragma unroll
            for (int j = 0; j < 16; j++) {
                if (j < nbt) {
                    wake[poff[j] + x] = __fmul_rn(scale[j], v[j]);
                }
            }
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) {
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;"
                     :: "r"(tmem), "r"(TC_TMEM_COLS) : "memory");
    }
}

}  // namespace
