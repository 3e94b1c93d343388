// Device side of the batched solver step (included by batch.cu only).
//
//  k_bwake   one CTA per bunch (per 128-row block of wider meshes): the
//            wake potential of every mesh row as the Toeplitz sum
//            wake[x] = s sum_m P[m] w[(x-m) mod nmax]  of the previous
//            step's profile P (w built once per impedance in FP64), the
//            charge integral (compensated FP32), this step's
//            renormalisation factor, both y-kick stencils of every row and
//            the step counter.
//  k_bmaps0  chain 0 (the reference's loop, src/main.cpp:1034-1044) for
//            meshes up to 512 rows: a persistent kernel whose CTAs walk
//            consecutive tiles of mesh rows through a ring of staged rows
//            in shared memory (TMA bulk copies one tile ahead); rows are
//            y-kicked in place once, the drift x-kick and Fokker-Planck
//            stage reads them from the ring, new rows and projections go
//            straight to HBM.  One CTA barrier per tile.
//  k_bmaps0w  chain 0 for wider meshes: tiles staged with their halo in
//            double-buffered shared memory (TMA bulk copies), y-kicks fused
//            in registers, drift x-kick as a column-wise sliding window,
//            Fokker-Planck, new rows and their projections.
//  k_bmaps1  chain 1 (rotation, wake y-kick, Fokker-Planck).
#pragma once

#include <cfloat>

#include "vfps_internal.cuh"

namespace {

constexpr int THREADS = 256;
constexpr int ROWPAD = 16;     // extra floats per rotated row (chain 1)
constexpr int TPAD = 4;        // zero floats on each side of a t3 row
constexpr int APAD = 8;        // zero floats left of a staged row (chain 0)
constexpr uint64_t WAIT_NS = 1000000000ull;  // bounded TMA waits (1 s)

struct __align__(16) BDev {     // 96 bytes: vector loads of its fields
    uint32_t n, it, chain, flags;  // flags: F_*
    uint32_t dens_off, prof_off, tab_off, st_off;
    uint32_t fp_off, wt_off, nmax, rot_h;
    int32_t renorm, halo_lo, halo_hi;
    uint32_t dw_off;               // drift, Fokker-Planck planes (ring kernels)
    float wakescale, fillset, dq, dp;
    float zbq, zbp, cs, sn;
};

struct __align__(16) Tile {
    uint32_t bunch, x0, rows, pad;
};
static_assert(sizeof(BDev) == 96 && sizeof(Tile) == 16,
              "host and device share these layouts");

// CSR power recording of the batched step (src/PS/ElectricField.cpp:
// 133-184): the power of a profile P is the quadratic form
//   sum_{m,m'} P[m] P[m'] K(m - m'),
//   K(d) = df sum_{i <= nmax/2} dq^2 c(f_i) Re Z[i] cos(2 pi i d / nmax),
// c the cutoff factor 1 - exp(-(f/fc)^2) (1 without a cutoff): the same
// number as the reference's sum of its spectrum over the half spectrum of
// the padded profile, as one Toeplitz product and a dot product
constexpr uint32_t NO_CSR = 0xffffffffu;
struct CsrRec {
    const float* k;              // K(d) for d = 1-n .. n-1, per table
    const uint32_t* off;         // per bunch: its table (NO_CSR: none)
    float* power;                // ring [cap][nb]
    unsigned long long* steps;   // ring [cap]: the step in each slot
    uint32_t every;              // record steps with step % every == 0
    uint32_t cap;                // (every == 0: no recording)
    uint32_t nb;                 // bunches (the power ring's row length)
    float2* part;                // [nb][CSR_MAXBLK]: blocks' sums (hi, lo)
    unsigned* done;              // [nb]: blocks of the step that are done
};
// most k_bwake blocks of one bunch (1024 rows in blocks of 128)
constexpr int CSR_MAXBLK = 8;

// the beam of a bunch: bunches of one beam share a padded profile (their
// buckets spacing mesh cells apart, src/PS/ElectricField.cpp:255-263), so
// each one's wake carries the others' fields
struct BeamDev {
    uint32_t first;    // its members in the member list
    uint32_t count;    // 1: the bunch alone
    int32_t bucket;    // bucket number of the bunch
    uint32_t spacing;  // mesh cells between neighbouring buckets
};

// log2 of seg = n / 8 lanes per row (n a power of two): the lane splits
// below are shifts and masks instead of divisions by a runtime value
__device__ __forceinline__ int lg_seg(int n)
{
    return __ffs(n) - 4;
}

// one kick stencil: tap j reads cell i + shift0 + j with weight w[j]
// (dropped taps have weight 0)
struct RowStencil {
    int shift0;
    float w[4];
};

// per mesh row of chain 0: combined shift of the two y-kicks and their
// weights (built by k_bwake once per step; 48 bytes, three 16-byte loads)
struct __align__(16) RowInfo {
    int s;      // sa + sb
    int sb;     // shift of the second (RF) kick
    float a[4]; // wake kick weights (times the renormalisation factor)
    float b[4]; // RF kick weights
    int pad[2];
};

// per mesh row of chain 0 for the fast ring kernel (k_bmaps0f): both
// y-kicks as one 7-tap stencil, out[y] = sum_k c[k] t1[y + s + k], with
// s = sa + sb and c[k] = sum_{i+j=k} a[i] b[j] (the wake kick's weights a,
// times the renormalisation factor, then the RF kick's b).  The same
// product of the two kicks except at the energy edges, where the
// reference drops the first kick's values that land off the mesh before
// the second kick (the composite keeps them: they carry the density of
// the outermost cells, about 1e-8 of the peak on a +-6 sigma mesh)
struct __align__(16) RowInfo7 {
    int s;
    float c[7];
};
static_assert(sizeof(RowInfo7) == 32, "two 16-byte loads per row");

// F_Y7: the bunch runs on k_bmaps0f (k_bwake writes RowInfo7 records)
enum { F_WAKE = 1, F_FP = 2, F_CLAMP = 4, F_Y7 = 8 };
enum { TAB_WS = 0, TAB_Q = 1, TAB_P = 2, TAB_COUNT = 3 };
enum { ST_RF = 0, ST_DRIFT = 1, ST_COUNT = 2 };

using namespace vfps::dev;

__host__ __device__ inline size_t align16(size_t v)
{
    return (v + 15) & ~size_t(15);
}

// rows of a k_bwake block of an n-row mesh: meshes up to 256 rows are one
// block, wider ones blocks of 128 rows (a block's wake sum costs its rows
// times n; measured, one block beats two for 256 rows and four blocks beat
// two for 512)
__host__ __device__ inline int wake_block_rows(int n)
{
    return n <= 256 ? n : 128;
}

// staged row of chain 0: APAD zeros, the n mesh values, APAD + 16 zeros
// (the y-kick windows reach past the row by the kick shift)
__host__ __device__ inline int astride0(int n) { return n + 2 * APAD + 16; }

// byte offsets of the regions of k_bmaps0w's dynamic shared memory; the
// host sizes each region for the largest tile of the batch
struct Smem0 {
    uint32_t a[2];  // staging buffers (TMA targets)
    uint32_t b;     // y-kicked rows [nr][n]
    uint32_t t;     // t3 rows [rows][n + 2 TPAD]
    uint32_t s;     // RowInfo [nr]
    uint32_t part;  // projection partials [rows][8]
    uint32_t bar;   // two mbarriers
    uint32_t pads;  // per staging buffer: mesh size of its row layout and
                    // the number of leading rows with zero pads
    uint32_t a_floats;  // capacity of one staging buffer
    uint32_t total;
};

__device__ __forceinline__ RowStencil make_stencil(float offset, uint32_t n,
                                                   int it)
{
    const KickStencil s = kick_stencil(offset, n, it);
    RowStencil r;
    bool any = false;
#pragma unroll
    for (int j = 0; j < 4; j++) {
        r.w[j] = s.valid[j] ? s.w[j] : 0.f;
        any = any || s.valid[j];
    }
    r.shift0 = any ? s.shift[0] : 0;
    return r;
}

// ----------------------------------------------------------------- wake
// Compensated FP32 sums (float-float: value = hi + lo).  A product of two
// floats splits exactly into hi + lo with one FMA; additions use Knuth's
// two-sum, whose error term is exact, so a + b and b + a give the same
// bits.  About 48 significant bits: far finer than the reference's FP32
// charge integral, and on this GPU much cheaper than FP64 arithmetic.
struct FF {
    float hi, lo;
};

__device__ __forceinline__ FF ff_prod(float a, float b)
{
    const float p = __fmul_rn(a, b);
    return FF{p, fmaf(a, b, -p)};
}

__device__ __forceinline__ FF ff_add(FF a, FF b)
{
    const float s = __fadd_rn(a.hi, b.hi);
    const float v = __fsub_rn(s, a.hi);
    float e = __fadd_rn(__fsub_rn(a.hi, __fsub_rn(s, v)), __fsub_rn(b.hi, v));
    e = __fadd_rn(e, __fadd_rn(a.lo, b.lo));
    const float hi = __fadd_rn(s, e);
    return FF{hi, __fsub_rn(e, __fsub_rn(hi, s))};
}

// Toeplitz sum wake[x] = sum_m w[x - m] P[m] over rows x0 <= x < x0 + R
// of a CTA of THREADS threads, from W[k + k/8] = w[x0 + k - (n-1)] (one pad
// entry per 8 puts the lanes below on 32 banks).  Thread = (group g of 8
// consecutive rows, slice q of the m range); the 8 rows read W at
// consecutive places, so stepping m slides a register window by one: 2
// shared loads (P broadcast, W) per 8 multiply-adds, the same trip count in
// every lane.  Writes the partial sums partial[q][x - x0] (Q = THREADS /
// (R/8) slices; n and R powers of two, 64 <= R <= n <= 2048, R <= 8
// THREADS); the caller sums them after a barrier.
__device__ __forceinline__ void toeplitz_partials(const float* P,
                                                  const float* W,
                                                  float* partial, int n,
                                                  int R)
{
    const int G = R >> 3;                    // <= THREADS
    const int Q = THREADS / G;
    const int q = threadIdx.x / G;
    const int g = threadIdx.x % G;
    const int span = n / Q;
    const int m0 = q * span;
    const int x = 8 * g;
    int bidx = x - m0 + n - 1;   // W index of (row x, m0)
    float w[8], acc[8];
#pragma unroll
    for (int j = 0; j < 8; j++) {
        const int k = bidx + j;
        w[j] = W[k + (k >> 3)];
        acc[j] = 0.f;
    }
#pragma unroll 8   // a whole turn of the 8-register window: no moves
    for (int m = m0; m < m0 + span; m++) {
        const float pm = P[m];
#pragma unroll
        for (int j = 0; j < 8; j++) {
            acc[j] = fmaf(pm, w[j], acc[j]);
        }
#pragma unroll
        for (int j = 7; j > 0; j--) {
            w[j] = w[j - 1];
        }
        bidx--;
        const int k = bidx > 0 ? bidx : 0;
        w[0] = W[k + (k >> 3)];
    }
    // two 16-byte stores (partial starts 16-byte aligned: 13n bytes into
    // the shared memory for n >= 64): a stride of 8 floats between lanes
    // costs 8 wavefronts per store instead of 8 scalar 8-way conflicts
    float4* pr = reinterpret_cast<float4*>(partial + size_t(q) * R + x);
    pr[0] = make_float4(acc[0], acc[1], acc[2], acc[3]);
    pr[1] = make_float4(acc[4], acc[5], acc[6], acc[7]);
}

// W[k + k/8] = w[(delta + k - (n-1)) mod nmax] for k < R + n - 1 (the
// layout that toeplitz_partials reads for R rows): the field at distance
// delta + x - m of a source cell m on row x (delta: the first row of the
// block plus the distance between two bunches' buckets in the padded
// profile, 0 for the rows of a bunch's own field from row 0)
__device__ __forceinline__ void load_toeplitz(const float* __restrict__ w,
                                              int nmax, int n, float* W,
                                              long long delta, int R)
{
    // one 64-bit remainder per thread, then each step of k adds THREADS
    // mod nmax to the index, and one subtraction reduces it
    long long b = (delta + threadIdx.x - (n - 1)) % nmax;
    b += b < 0 ? nmax : 0;
    int base = static_cast<int>(b);
    const int step = THREADS % nmax;
    for (int k = threadIdx.x; k < R + n - 1; k += THREADS) {
        W[k + (k >> 3)] = w[base];
        base += step;
        base -= base >= nmax ? nmax : 0;
    }
}

// The unscaled wake on rows x0 <= x < x0 + R of a bunch in beam Mb: the
// fields of every member of the beam (the bunch included) at their bucket
// distances, from the members' profiles in pin, into acc[x - x0] (each
// thread sums the rows it owns).  W, partial, Pm: scratch as for
// toeplitz_partials (Pm holds one member's profile of n cells).
__device__ __forceinline__ void beam_wake_rows(
    const BDev* __restrict__ bd, const BeamDev* __restrict__ beams,
    const uint32_t* __restrict__ members, const BeamDev& Mb,
    const float* __restrict__ w, int nmax, int n, int x0, int R,
    const float* __restrict__ pin, float* W, float* partial, float* Pm,
    float* acc)
{
    const int Q = THREADS / (R >> 3);
    for (int x = threadIdx.x; x < R; x += THREADS) {
        acc[x] = 0.f;
    }
    for (uint32_t k = 0; k < Mb.count; k++) {
        const uint32_t b2 = members[Mb.first + k];
        const BDev B2 = bd[b2];
        const long long delta = (long long)(Mb.bucket - beams[b2].bucket)
                                * Mb.spacing;
        __syncthreads();   // the previous member's W, Pm, partial read
        for (int i = threadIdx.x; i < n; i += THREADS) {
            Pm[i] = pin[B2.prof_off + i];
        }
        load_toeplitz(w, nmax, n, W, delta + x0, R);
        __syncthreads();
        toeplitz_partials(Pm, W, partial, n, R);
        __syncthreads();
        for (int x = threadIdx.x; x < R; x += THREADS) {
            float sum = 0.f;
            for (int q = 0; q < Q; q++) {
                sum += partial[size_t(q) * R + x];
            }
            acc[x] += sum;   // read back by this thread only
        }
    }
}

// One CTA per block of rows of a bunch (wake_block_rows; wblk: bunch and
// first row of each CTA): wake potential of the previous step's profile on
// the block's rows, charge integral, renormalisation factor and, for chain 0,
// both y-kick stencils of the block's rows.  Every CTA of a bunch sums the
// whole profile's charge (the same bits); the first one stores it.  The
// step number is the CTA's own 64-bit counter, which it advances once per
// step (the steps run in stream order, and no other CTA touches it), so no
// CTA waits for another or contends for a shared counter.
__global__ void __launch_bounds__(THREADS)
k_bwake(const BDev* __restrict__ bd, const uint2* __restrict__ wblk,
        const float* __restrict__ tabs,
        const float* __restrict__ wt, const RowStencil* __restrict__ st,
        const float* __restrict__ pin, float* __restrict__ wake,
        RowInfo* __restrict__ rinfo, RowInfo7* __restrict__ rinfo7,
        float* __restrict__ factor,
        double* __restrict__ filling, unsigned long long* __restrict__ tickets,
        const BeamDev* __restrict__ beams,
        const uint32_t* __restrict__ members, CsrRec csr,
        int* __restrict__ status, int wake_ready, int block_per_bunch)
{
    extern __shared__ float4 wsm4[];
    float* P = reinterpret_cast<float*>(wsm4);      // [n]
    __shared__ float2 red[32];
    __shared__ unsigned long long ticket_s;
    // one block per bunch (no mesh wider than a block): CTA i is bunch i,
    // and its record loads do not wait for the block list
    const uint2 blk = block_per_bunch ? make_uint2(blockIdx.x, 0u)
                                      : wblk[blockIdx.x];
    const uint32_t b = blk.x;
    const BDev B = bd[b];
    const int n = int(B.n);
    const int xr0 = int(blk.y);                   // first row of the block
    const int R = wake_block_rows(n);             // rows of the block
    // W[k + k/8] = w[(k - (n-1)) mod nmax] for k < 2n - 1: one pad entry
    // per 8 puts the 32 lanes of the wake sum (rows 8 apart) on 32 banks
    float* W = P + n;
    const bool has_wake = B.flags & F_WAKE;
    // wake_ready: the tensor-core kernel has written this step's wake
    const bool sum_here = has_wake && !wake_ready;
    // the bunch's own field (a coupled beam reloads it per member; not
    // waiting for the beam record keeps this load off its latency)
    if (sum_here) {
        load_toeplitz(wt + B.wt_off, int(B.nmax), n, W, xr0, R);
    }
    const BeamDev Mb = beams[b];
    const bool coupled = Mb.count > 1;
    // loads for the later phases, issued now
    const float* ws = tabs + B.tab_off + TAB_WS * n;
    const int x0 = threadIdx.x;
    const float ws0 = x0 < n ? ws[x0] : 0.f;
    const RowStencil* rf = st + B.st_off + ST_RF * n;
    RowStencil sb0 = {};
    if (B.chain == 0 && x0 < R) {
        sb0 = rf[xr0 + x0];
    }
    // the profile's lines into L2 ahead of their loads after the wait (a
    // hint: the previous maps kernel's writes still land in L2 after it,
    // so the loads read them either way)
    for (int i = 32 * threadIdx.x; i < n; i += 32 * THREADS) {
        prefetch_l2(pin + B.prof_off + i);
    }
    // the records and tables above do not change between steps; launched
    // as a programmatic dependent of the previous step's maps kernel, the
    // CTA reads them while that kernel ends, and waits for it here before
    // it reads the profiles or writes anything.  Then the maps kernel that
    // follows may start its prologue
    pdl_wait();
    pdl_trigger();
    if (threadIdx.x == 0) {
        ticket_s = tickets[blockIdx.x]++;
    }
    for (int i = threadIdx.x; i < n; i += THREADS) {
        P[i] = pin[B.prof_off + i];
    }
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    // charge integral (src/PS/PhaseSpace.cpp:200-239), compensated:
    // per-warp sums now, the block total after the barrier that ends the
    // wake sum
    {
        FF a = x0 < n ? ff_prod(P[x0], ws0) : FF{0.f, 0.f};
        for (int i = x0 + THREADS; i < n; i += THREADS) {
            a = ff_add(a, ff_prod(P[i], ws[i]));
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const FF t{__shfl_down_sync(0xffffffffu, a.hi, o),
                       __shfl_down_sync(0xffffffffu, a.lo, o)};
            a = ff_add(a, t);
        }
        if (lane == 0) {
            red[warp] = make_float2(a.hi, a.lo);
        }
    }
    float* partial = W + 2 * n + (n >> 2);   // [Q][R], Q R = 8 THREADS
    const int Q = THREADS / (R >> 3);
    float* acc = partial + 8 * THREADS;      // coupled beams: wake [R]
    float* Pm = acc + n;                     // and a member's profile [n]
    if (sum_here && !coupled) {
        toeplitz_partials(P, W, partial, n, R);
    } else if (sum_here) {
        beam_wake_rows(bd, beams, members, Mb, wt + B.wt_off, int(B.nmax), n,
                       xr0, R, pin, W, partial, Pm, acc);
    }
    __syncthreads();   // partial sums, per-warp integrals and ticket_s
    FF tot = FF{0.f, 0.f};
    if (lane < (THREADS >> 5)) {
        const float2 r = red[lane];
        tot = FF{r.x, r.y};
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {   // same bits in every thread
        const FF t{__shfl_xor_sync(0xffffffffu, tot.hi, o),
                   __shfl_xor_sync(0xffffffffu, tot.lo, o)};
        tot = ff_add(tot, t);
    }
    const unsigned step = static_cast<unsigned>(ticket_s);
    const bool renorm_now = B.renorm > 0 && (step % unsigned(B.renorm)) == 0;
    float fac = 1.f;
    if (renorm_now && B.fillset > 0) {
        const double a = double(tot.hi) + double(tot.lo);
        fac = static_cast<float>(double(B.fillset) / a);
    } else if (renorm_now) {
        fac = 0.f;
    }
    if (threadIdx.x == 0 && xr0 == 0) {
        filling[b] = double(tot.hi) + double(tot.lo);
        factor[b] = fac;
        if (B.fillset > 0 && !(tot.hi > 0.f)) {
            atomicCAS(status, 0, VFPS_ERR_NUMERIC);
        }
    }
    // wake potential of every row and, for chain 0, both y-kick stencils
    // of the row for this step, the renormalisation factor folded into the
    // first (both kicks are linear)
    const bool chain0 = B.chain == 0;
    for (int xl = threadIdx.x; xl < R; xl += THREADS) {
        const int x = xr0 + xl;
        float v = 0.f;
        if (sum_here) {
            float sum = 0.f;
            if (coupled) {
                sum = acc[xl];
            } else {
                for (int k = 0; k < Q; k++) {
                    sum += partial[size_t(k) * R + xl];
                }
            }
            v = __fmul_rn(B.wakescale, sum);
            wake[B.prof_off + x] = v;
        } else if (has_wake) {
            v = wake[B.prof_off + x];
        } else {
            wake[B.prof_off + x] = 0.f;
        }
        if (!chain0) {
            continue;
        }
        RowStencil sa;
        if (has_wake) {
            sa = make_stencil(v, B.n, int(B.it));
        } else {
            sa.shift0 = 0;
            sa.w[0] = 1.f;
            sa.w[1] = sa.w[2] = sa.w[3] = 0.f;
        }
        const RowStencil sb = xl == x0 ? sb0 : rf[x];
        if (B.flags & F_Y7) {
            RowInfo7 r7;
            r7.s = sa.shift0 + sb.shift0;
            float a[4];
#pragma unroll
            for (int j = 0; j < 4; j++) {
                a[j] = sa.w[j] * fac;
            }
#pragma unroll
            for (int k = 0; k < 7; k++) {
                float c = 0.f;
#pragma unroll
                for (int i = 0; i < 4; i++) {
                    if (k - i >= 0 && k - i < 4) {
                        c = fmaf(a[i], sb.w[k - i], c);
                    }
                }
                r7.c[k] = c;
            }
            rinfo7[B.prof_off + x] = r7;
            continue;
        }
        RowInfo ri;
        ri.s = sa.shift0 + sb.shift0;
        ri.sb = sb.shift0;
#pragma unroll
        for (int j = 0; j < 4; j++) {
            ri.a[j] = sa.w[j] * fac;
            ri.b[j] = sb.w[j];
        }
        ri.pad[0] = ri.pad[1] = 0;
        rinfo[B.prof_off + x] = ri;
    }
    // CSR power of this step's profile (recording steps only; the same
    // decision in every CTA): the block's rows' part of the quadratic form
    // P^T T_K P; the bunch's last block to finish adds the parts in block
    // order
    if (csr.every == 0 || step % csr.every != 0) {
        return;
    }
    const uint32_t koff = csr.off[b];
    if (koff == NO_CSR) {
        return;
    }
    __syncthreads();   // W and the partial sums of the wake are free
    // W[k + k/8] = K(xr0 + k - (n-1)) for k < R + n - 1 (the table holds
    // K(d) for d = 1-n .. n-1)
    for (int k = threadIdx.x; k < R + n - 1; k += THREADS) {
        W[k + (k >> 3)] = csr.k[koff + xr0 + k];
    }
    __syncthreads();
    toeplitz_partials(P, W, partial, n, R);
    __syncthreads();
    FF dot = FF{0.f, 0.f};
    for (int xl = threadIdx.x; xl < R; xl += THREADS) {
        float v = 0.f;
        for (int q = 0; q < Q; q++) {
            v += partial[size_t(q) * R + xl];
        }
        dot = ff_add(dot, ff_prod(P[xr0 + xl], v));
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const FF t{__shfl_down_sync(0xffffffffu, dot.hi, o),
                   __shfl_down_sync(0xffffffffu, dot.lo, o)};
        dot = ff_add(dot, t);
    }
    __syncthreads();   // red[] was read by every thread above
    if (lane == 0) {
        red[warp] = make_float2(dot.hi, dot.lo);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        FF tot = FF{0.f, 0.f};
        for (int w2 = 0; w2 < (THREADS >> 5); w2++) {
            tot = ff_add(tot, FF{red[w2].x, red[w2].y});
        }
        const int nblk = n / R;
        bool last = true;
        if (nblk > 1) {
            // publish this block's part, then count it (the last block
            // sees every part: each was written before its count)
            csr.part[size_t(b) * CSR_MAXBLK + xr0 / R] =
                make_float2(tot.hi, tot.lo);
            __threadfence();
            last = atomicAdd(csr.done + b, 1u) == unsigned(nblk - 1);
            if (last) {
                __threadfence();
                tot = FF{0.f, 0.f};
                for (int r = 0; r < nblk; r++) {
                    const float2 v = __ldcg(csr.part
                                            + size_t(b) * CSR_MAXBLK + r);
                    tot = ff_add(tot, FF{v.x, v.y});
                }
                csr.done[b] = 0u;   // for the next recording step
            }
        }
        if (last) {
            const uint32_t slot = (step / csr.every) % csr.cap;
            csr.power[size_t(slot) * csr.nb + b] = tot.hi + tot.lo;
            if (b == 0) {
                csr.steps[slot] = step;
            }
        }
    }
}

// ------------------------------------------------------ potential well
// Per chain-0 bunch: offsets of the RF kick (per row) and of the drift (per
// column) in pwtab, and the energy scale T of the state below
struct PwDev {
    uint32_t off;  // rf offsets [n], then drift offsets [n]
    float T;       // slip0 / (dq dp); 0: no potential-well state
    uint32_t chain;
    float pad;
};

// float offsets of the regions of k_potential_well's dynamic shared memory
// for a mesh of n rows (every region grows with n, so the layout of the
// largest mesh of a batch covers the others)
struct PwSmem {
    size_t P, W, partial, F, Phi, G, D, RF, WS, M, S, acc, Pm, total;
};

__host__ __device__ inline PwSmem pw_smem(size_t n)
{
    PwSmem L;
    L.P = 0;                          // profile [n]
    L.W = L.P + n;                    // Toeplitz table [2n + n/4]
    L.partial = L.W + 2 * n + n / 4;  // partial sums [8 THREADS]
    L.F = L.partial + 8 * THREADS;    // row kicks [n]
    L.Phi = L.F + n;                  // their integral [n]
    L.G = L.Phi + n;                  // integral of the drift offsets [n]
    L.D = L.G + n;                    // drift offsets [n]
    L.RF = L.D + n;                   // RF offsets [n]
    L.WS = L.RF + n;                  // Simpson weights [n]
    L.M = L.WS + n;                   // row maxima [n]
    L.S = L.M + n;                    // row sums [n]
    L.acc = L.S + n;                  // a beam's wake [n]
    L.Pm = L.acc + n;                 // and one member's profile [n]
    L.total = L.Pm + n;
    return L;
}

// block-wide trapezoid integral: out[0] = 0, out[i] = out[i-1] +
// (f[i-1] + f[i]) / 2; each thread sums a run of consecutive entries
__device__ void block_trapezoid(const float* f, float* out, int n,
                                float* scratch32)
{
    const int per = (n + THREADS - 1) / THREADS;
    const int i0 = threadIdx.x * per;
    const int i1 = min(n, i0 + per);
    float run = 0.f;
    for (int i = max(i0, 1); i < i1; i++) {
        run += 0.5f * (f[i - 1] + f[i]);
    }
    // exclusive scan of the per-thread sums: within warps, then warps
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    float inc = run;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const float v = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) {
            inc += v;
        }
    }
    if (lane == 31) {
        scratch32[warp] = inc;
    }
    __syncthreads();
    float base = 0.f;
    for (int w = 0; w < warp; w++) {
        base += scratch32[w];
    }
    float acc = base + inc - run;
    for (int i = i0; i < i1; i++) {
        if (i > 0) {
            acc += 0.5f * (f[i - 1] + f[i]);
        }
        out[i] = acc;
    }
    __syncthreads();
}

__device__ float block_max(float v, float* scratch32)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) {
        scratch32[warp] = v;
    }
    __syncthreads();
    float m = scratch32[0];
    for (int w = 1; w < (THREADS >> 5); w++) {
        m = fmaxf(m, scratch32[w]);
    }
    return m;
}

__device__ float block_sum_f(float v, float* scratch32)
{
    v = warp_sum_f(v);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) {
        scratch32[warp] = v;
    }
    __syncthreads();
    float t = 0.f;
    for (int w = 0; w < (THREADS >> 5); w++) {
        t += scratch32[w];
    }
    return t;
}

// The stationary state of the chain-0 step (y-kicks of the wake and the
// RF, drift, Fokker-Planck) below the instability threshold, and of the
// rotation chain (rotation, wake kick, Fokker-Planck): a function of
// the step's invariant, exp(-E / T) with
//   E(x, y) = Phi(x) + G(y) + F(x) d(y) / 2,
// F = -(rf + wake) the y-kick of row x (cells per step), Phi its integral
// over x, d the drift offset of column y, G its integral over y, and T =
// slip0 / (dq dp) the scale at which the Fokker-Planck term holds the
// energy spread at one unit.  Phi + G is the Haissinski potential well
// (the continuous-time invariant); the cross term is the first correction
// of the split step (kick, then drift) to it.  The wake depends on the
// profile, so the profile iterates to a fixed point (mixing `mix` of each
// new profile into the old one).  For the rotation chain, rf and d are the
// linear kick and drift of the rotation's angle (its quadratic potential
// and kinetic term) and only the wake kick enters the cross term, with the
// opposite sign (the rotation conserves the radial invariant exactly; the
// wake kick follows it).  One CTA per bunch.  Writes the density normalised
// to the bunch's filling and the last relative L1 change of the profile.
// pass < 0: every iteration in this launch (bunches on their own).
// pass >= 0 (a batch with coupled beams): iteration `pass` only; the wake
// of each member sums the fields of its beam's profiles of the previous
// pass (pin), the bunch's mixed profile goes to pout, and the last pass
// (iters, or 0 without a wake) writes the density.
__global__ void __launch_bounds__(THREADS)
k_potential_well(const BDev* __restrict__ bd, const PwDev* __restrict__ pw,
                 const float* __restrict__ pwtab,
                 const float* __restrict__ tabs,
                 const float* __restrict__ wt,
                 const BeamDev* __restrict__ beams,
                 const uint32_t* __restrict__ members,
                 const float* __restrict__ pin, float* __restrict__ pout,
                 float* __restrict__ dens, float* __restrict__ change,
                 int* __restrict__ status, int iters, float mix, int pass)
{
    const BDev B = bd[blockIdx.x];
    const PwDev Z = pw[blockIdx.x];
    if (!(Z.T > 0.f)) {
        return;
    }
    const bool has_wake = B.flags & F_WAKE;
    const int last = has_wake ? iters : 0;   // without a wake: one pass
    // half the row factor of the split-step term: the whole y-kick after
    // the kick-drift step (chain 0); for the rotation chain only the wake
    // kick, -(F + rf), with the sign of a kick after the rotation
    const float hsign = Z.chain == 0 ? 0.5f : -0.5f;
    const bool hrf = Z.chain != 0;
    if (pass > last) {
        return;   // this bunch's state is written already
    }
    extern __shared__ float4 pwsm4[];
    __shared__ float scratch[32];
    const int n = int(B.n);
    const PwSmem L = pw_smem(size_t(n));
    uint32_t dyn_bytes;
    asm("mov.u32 %0, %%dynamic_smem_size;" : "=r"(dyn_bytes));
    if (L.total * sizeof(float) > dyn_bytes) {   // the launch's layout
        if (threadIdx.x == 0) {
            atomicCAS(status, 0, VFPS_ERR_INVALID_ARGUMENT);
        }
        return;
    }
    float* base = reinterpret_cast<float*>(pwsm4);
    float* P = base + L.P;
    float* W = base + L.W;
    float* partial = base + L.partial;
    float* F = base + L.F;
    float* Phi = base + L.Phi;
    float* G = base + L.G;
    float* D = base + L.D;
    float* RF = base + L.RF;
    float* WS = base + L.WS;
    float* M = base + L.M;
    float* S = base + L.S;
    float* acc = base + L.acc;
    float* Pm = base + L.Pm;
    const float* ws = tabs + B.tab_off + TAB_WS * n;
    for (int i = threadIdx.x; i < n; i += THREADS) {
        RF[i] = pwtab[Z.off + i];
        D[i] = pwtab[Z.off + n + i];
        WS[i] = ws[i];
        P[i] = pass > 0 ? pin[B.prof_off + i] : 0.f;
    }
    if (has_wake && pass < 0) {
        load_toeplitz(wt + B.wt_off, int(B.nmax), n, W, 0, n);
    }
    __syncthreads();
    block_trapezoid(D, G, n, scratch);
    {
        float gmin = 3.4e38f;
        for (int i = threadIdx.x; i < n; i += THREADS) {
            gmin = fminf(gmin, G[i]);
        }
        gmin = -block_max(-gmin, scratch);
        for (int i = threadIdx.x; i < n; i += THREADS) {
            G[i] -= gmin;
        }
        __syncthreads();
    }
    const float fill = B.fillset > 0 ? B.fillset : 1.f;
    const float invT = 1.f / Z.T;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int Q = THREADS / (n >> 3);
    float delta = 0.f;
    bool changed = false;   // delta holds a change of this launch
    const int it0 = pass < 0 ? 0 : pass;
    const int it1 = pass < 0 ? last : pass;
    for (int it = it0; it <= it1; it++) {
        // row kicks of the current profile (the first pass: RF only)
        const bool wk = has_wake && it > 0;
        if (wk && pass < 0) {
            toeplitz_partials(P, W, partial, n, n);
        } else if (wk) {
            beam_wake_rows(bd, beams, members, beams[blockIdx.x],
                           wt + B.wt_off, int(B.nmax), n, 0, n, pin, W,
                           partial, Pm, acc);
        }
        __syncthreads();
        for (int x = threadIdx.x; x < n; x += THREADS) {
            float wake = 0.f;
            if (wk) {
                float sum = 0.f;
                if (pass < 0) {
                    for (int k = 0; k < Q; k++) {
                        sum += partial[size_t(k) * n + x];
                    }
                } else {
                    sum = acc[x];
                }
                wake = __fmul_rn(B.wakescale, sum);
            }
            F[x] = -(RF[x] + wake);
        }
        __syncthreads();
        block_trapezoid(F, Phi, n, scratch);
        // per row: maximum of the exponent and the Simpson sum over y
        for (int x = warp; x < n; x += THREADS >> 5) {
            const float phi = Phi[x];
            const float hf = hsign * (hrf ? F[x] + RF[x] : F[x]);
            float m = -3.4e38f;
            for (int y = lane; y < n; y += 32) {
                m = fmaxf(m, -(phi + G[y] + hf * D[y]) * invT);
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
            }
            float sum = 0.f;
            for (int y = lane; y < n; y += 32) {
                sum += WS[y] * expf(-(phi + G[y] + hf * D[y]) * invT - m);
            }
            sum = warp_sum_f(sum);
            if (lane == 0) {
                M[x] = m;
                S[x] = sum;
            }
        }
        __syncthreads();
        float mloc = -3.4e38f;
        for (int x = threadIdx.x; x < n; x += THREADS) {
            mloc = fmaxf(mloc, M[x]);
        }
        const float mx = block_max(mloc, scratch);
        float mass = 0.f;
        for (int x = threadIdx.x; x < n; x += THREADS) {
            mass += WS[x] * S[x] * expf(M[x] - mx);
        }
        mass = block_sum_f(mass, scratch);
        const float scale = fill / mass;
        if (it == last) {
            // the state: exp(-E / T) scaled to the filling
            float* out = dens + B.dens_off;
            for (int x = warp; x < n; x += THREADS >> 5) {
                const float phi = Phi[x];
                const float hf = hsign * (hrf ? F[x] + RF[x] : F[x]);
                for (int y = lane; y < n; y += 32) {
                    out[size_t(x) * n + y] =
                        scale * expf(-(phi + G[y] + hf * D[y]) * invT - mx);
                }
            }
            break;
        }
        // new profile, its change against the current one, mixing
        float dsum = 0.f, psum = 0.f;
        for (int x = threadIdx.x; x < n; x += THREADS) {
            const float r = scale * S[x] * expf(M[x] - mx);
            dsum += fabsf(r - P[x]);
            psum += fabsf(P[x]);
            P[x] = it == 0 ? r : fmaf(mix, r - P[x], P[x]);
            if (pass >= 0) {
                pout[B.prof_off + x] = P[x];
            }
        }
        dsum = block_sum_f(dsum, scratch);
        psum = block_sum_f(psum, scratch);
        delta = psum > 0.f ? dsum / psum : 1.f;
        changed = true;
        __syncthreads();
    }
    if (threadIdx.x == 0 && (changed || pass < 0)) {
        change[blockIdx.x] = delta;
    }
}

// t2[i] = sum_j a_j c[AL + i + j], the first y-kick of 11 positions from
// a window whose first input sits at c[AL]
template <int AL>
__device__ __forceinline__ void first_kick(const float* c, const RowInfo& ri,
                                           float* t2)
{
#pragma unroll
    for (int i = 0; i < 11; i++) {
        float v = ri.a[0] * c[AL + i];
        v = fmaf(ri.a[1], c[AL + i + 1], v);
        v = fmaf(ri.a[2], c[AL + i + 2], v);
        v = fmaf(ri.a[3], c[AL + i + 3], v);
        t2[i] = v;
    }
}

// per-thread column constants of the Fokker-Planck stage: the thread owns
// the 8 energy cells y0..y0+7 of its rows (5 weights each for the offsets
// -2..2) and their Simpson weights
struct FpCols {
    float f[8][5];
    float wsr[8];
};

__device__ __forceinline__ void load_fp_cols(const BDev& B,
                                             const float* __restrict__ fp5,
                                             const float* __restrict__ ws,
                                             FpCols& c)
{
    const int n = int(B.n);
    const int y0 = 8 * (threadIdx.x % (n >> 3));
    const bool has_fp = B.flags & F_FP;
#pragma unroll
    for (int k = 0; k < 8; k++) {
        c.wsr[k] = ws[y0 + k];
#pragma unroll
        for (int o = 0; o < 5; o++) {
            c.f[k][o] = has_fp ? fp5[B.fp_off + (y0 + k) * 5 + o]
                               : (o == 2 ? 1.f : 0.f);
        }
    }
}

// Fokker-Planck (5 weights per column for offsets -2..2), output rows and
// their projections.  T holds t3 rows with TPAD zeros on both sides.
__device__ __forceinline__ void fp_and_store(
    const float* __restrict__ T, int rows, int n, int x0, const BDev& B,
    const FpCols& cc, float* __restrict__ dout, float* __restrict__ pout,
    float* part)
{
    const int seg = n >> 3;               // threads per row
    const int lg = lg_seg(n);
    const int rp = THREADS >> lg;         // rows in parallel
    const int l = threadIdx.x & (seg - 1);
    const int rl = threadIdx.x >> lg;
    const int y0 = 8 * l;
    const int stride = n + 2 * TPAD;
    {
        const auto& f = cc.f;
        const auto& wsr = cc.wsr;
        // every lane runs the same number of iterations (the shuffles
        // below need the whole warp); rows past the tile are predicated off
        for (int rbase = 0; rbase < rows; rbase += rp) {
            const int r = rbase + rl;
            const bool valid = r < rows;
            const float4* src = reinterpret_cast<const float4*>(
                T + size_t(valid ? r : 0) * stride + y0);
            float win[16];
#pragma unroll
            for (int c = 0; c < 4; c++) {
                const float4 v = src[c];
                win[4 * c] = v.x;
                win[4 * c + 1] = v.y;
                win[4 * c + 2] = v.z;
                win[4 * c + 3] = v.w;
            }
            float out[8];
            float pp = 0.f;
#pragma unroll
            for (int k = 0; k < 8; k++) {
                float v = f[k][0] * win[k + 2];
                v = fmaf(f[k][1], win[k + 3], v);
                v = fmaf(f[k][2], win[k + 4], v);
                v = fmaf(f[k][3], win[k + 5], v);
                v = fmaf(f[k][4], win[k + 6], v);
                out[k] = v;
                pp = fmaf(v, wsr[k], pp);
            }
            if (valid) {
                float4* dst = reinterpret_cast<float4*>(
                    dout + B.dens_off + size_t(x0 + r) * n + y0);
                dst[0] = make_float4(out[0], out[1], out[2], out[3]);
                dst[1] = make_float4(out[4], out[5], out[6], out[7]);
            }
            // reduce the row's partial sums (groups of seg lanes)
            const int width = seg < 32 ? seg : 32;
            for (int o = width >> 1; o > 0; o >>= 1) {
                pp += __shfl_xor_sync(0xffffffffu, pp, o);
            }
            if (valid && (l & (width - 1)) == 0) {
                part[r * 8 + (l >> 5)] = pp;
            }
        }
    }
    __syncthreads();
    const int groups = seg < 32 ? 1 : seg / 32;
    for (int r = threadIdx.x; r < rows; r += THREADS) {
        float s = 0.f;
        for (int g = 0; g < groups; g++) {
            s += part[r * 8 + g];
        }
        pout[B.prof_off + x0 + r] = s;
    }
}

// --------------------------------------------------------------- chain 0
// Before the bulk copies of a tile land in a staging buffer: zero the
// slots of rows off the mesh, and the pad columns of every row that does
// not hold zero pads yet for this mesh size.  `pads` describes the buffer:
// pads[0] = the mesh size its row layout follows, pads[1] = how many
// leading rows have zero pads in that layout (shared memory starts with
// arbitrary contents, and a short tail tile prepares fewer rows than a
// later full tile reads).  Called by all threads.
__device__ __forceinline__ void prepare_slots(const BDev& B, const Tile& t,
                                              float* A, const int* pads)
{
    const int n = int(B.n);
    const int as = astride0(n);
    const int nr = int(t.rows) + B.halo_lo + B.halo_hi;
    const int first = int(t.x0) - B.halo_lo;
    const volatile int* pv = pads;
    const int ready = pv[0] == n ? pv[1] : 0;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const float4 z = make_float4(0.f, 0.f, 0.f, 0.f);
    for (int r = warp; r < nr; r += THREADS / 32) {
        const int x = first + r;
        float4* row = reinterpret_cast<float4*>(A + size_t(r) * as);
        if (unsigned(x) >= unsigned(n)) {
            for (int j = lane; j < as / 4; j += 32) {
                row[j] = z;
            }
        } else if (r >= ready) {
            // APAD/4 float4 left of the data, (APAD + 16)/4 right of it
            for (int j = lane; j < (2 * APAD + 16) / 4; j += 32) {
                row[j < APAD / 4 ? j : n / 4 + j] = z;
            }
        }
    }
}

// after prepare_slots (and a barrier): every row of the tile now has zero
// pads in the layout of its mesh size (thread 0 only)
__device__ __forceinline__ void note_slots(const BDev& B, const Tile& t,
                                           int* pads)
{
    const int n = int(B.n);
    const int nr = int(t.rows) + B.halo_lo + B.halo_hi;
    const int ready = pads[0] == n ? pads[1] : 0;
    pads[0] = n;
    pads[1] = nr > ready ? nr : ready;
}

// issue the bulk copies of a tile's mesh rows (warp 0; lane 0 arms the
// barrier with the byte count first)
__device__ __forceinline__ void issue_tile(const BDev& B, const Tile& t,
                                           const float* __restrict__ din,
                                           float* A, uint64_t* bar)
{
    const int n = int(B.n);
    const int as = astride0(n);
    const int first = int(t.x0) - B.halo_lo;
    const int lo = max(0, first);
    const int hi = min(n, int(t.x0 + t.rows) + B.halo_hi);
    const uint32_t row_bytes = uint32_t(n) * 4u;
    const int lane = threadIdx.x & 31;
    if (lane == 0) {
        fence_proxy_async();
        mbar_arrive_expect_tx(bar, uint32_t(hi - lo) * row_bytes);
    }
    __syncwarp();
    for (int x = lo + lane; x < hi; x += 32) {
        tma_load_1d(A + size_t(x - first) * as + APAD,
                    din + B.dens_off + size_t(x) * n, row_bytes, bar);
    }
}

__global__ void __launch_bounds__(THREADS, 2)
k_bmaps0w(const BDev* __restrict__ bd, const Tile* __restrict__ tiles,
         uint32_t ntiles, const float* __restrict__ tabs,
         const RowStencil* __restrict__ st, const float* __restrict__ fp5,
         const RowInfo* __restrict__ rinfo,
         const float* __restrict__ din, float* __restrict__ dout,
         float* __restrict__ pout, int* __restrict__ status, Smem0 L)
{
    extern __shared__ float4 smem4[];
    char* base = reinterpret_cast<char*>(smem4);
    float* const A0 = reinterpret_cast<float*>(base + L.a[0]);
    float* const A1 = reinterpret_cast<float*>(base + L.a[1]);
    float* Bs = reinterpret_cast<float*>(base + L.b);
    float* T = reinterpret_cast<float*>(base + L.t);
    RowInfo* S = reinterpret_cast<RowInfo*>(base + L.s);
    float* part = reinterpret_cast<float*>(base + L.part);
    uint64_t* bar = reinterpret_cast<uint64_t*>(base + L.bar);
    int* pads = reinterpret_cast<int*>(base + L.pads);   // [2][2]

    if (threadIdx.x == 0) {
        mbar_init(&bar[0], 1);
        mbar_init(&bar[1], 1);
        mbar_fence_init();
        for (int i = 0; i < 4; i++) {
            pads[i] = i & 1 ? 0 : -1;
        }
    }
    __syncthreads();

    // each CTA walks a contiguous chunk of the tile list (tiles of a bunch
    // are adjacent), so per-bunch column constants stay in registers; the
    // chunks differ by at most one tile
    const uint32_t t_begin = uint32_t(uint64_t(blockIdx.x) * ntiles
                                      / gridDim.x);
    const uint32_t t_end = uint32_t(uint64_t(blockIdx.x + 1) * ntiles
                                    / gridDim.x);
    uint32_t tid = t_begin;
    if (tid < t_end) {
        const Tile t = tiles[tid];
        const BDev B = bd[t.bunch];
        prepare_slots(B, t, A0, &pads[0]);
        __syncthreads();
        if (threadIdx.x == 0) {
            note_slots(B, t, &pads[0]);
        }
        if (threadIdx.x < 32) {
            issue_tile(B, t, din, A0, &bar[0]);
        }
    }
    int bad = 0;
    uint32_t cached = 0xffffffffu;   // bunch of the register caches
    FpCols fpc;
    RowStencil dcol;                 // drift stencil of this thread's column
    for (uint32_t k = 0; tid < t_end; tid++, k++) {
        const int cur = int(k & 1);
        const Tile t = tiles[tid];
        const BDev B = bd[t.bunch];
        const int n = int(B.n);
        const int x0 = int(t.x0);
        const int rows = int(t.rows);
        const int hlo = B.halo_lo, hhi = B.halo_hi;
        const int nr = rows + hlo + hhi;
        const int as = astride0(n);
        float* A = cur ? A1 : A0;
        if (t.bunch != cached) {
            cached = t.bunch;
            load_fp_cols(B, fp5, tabs + B.tab_off + TAB_WS * n, fpc);
            if (n <= THREADS) {
                dcol = st[B.st_off + ST_DRIFT * n + threadIdx.x % n];
            }
        }

        // prefetch the next tile into the other buffer: its last reader
        // (the previous tile) finished at the barrier that ended the loop
        const uint32_t nxt = tid + 1;
        if (nxt < t_end) {
            const Tile tn = tiles[nxt];
            const BDev Bn = bd[tn.bunch];
            prepare_slots(Bn, tn, cur ? A0 : A1, &pads[2 * (cur ^ 1)]);
            if (threadIdx.x < 32) {
                issue_tile(Bn, tn, din, cur ? A0 : A1, &bar[cur ^ 1]);
            }
        }

        // per staged row: both y-kick stencils of this step
        {
            for (int r = threadIdx.x; r < nr; r += THREADS) {
                const int x = x0 - hlo + r;
                RowInfo ri;
                if (unsigned(x) < unsigned(n)) {
                    ri = rinfo[B.prof_off + x];
                } else {
                    ri.s = 0;
                    ri.sb = 0;
#pragma unroll
                    for (int j = 0; j < 4; j++) {
                        ri.a[j] = 0.f;
                        ri.b[j] = 0.f;
                    }
                }
                S[r] = ri;
            }
        }

        // wait for this tile's rows (bounded: a wait that runs out flags
        // VFPS_ERR_TIMEOUT and keeps waiting a bounded time more).  A CTA
        // whose wait ran out stops walking its tiles: the next tile's
        // copies, already issued, get one bounded wait, and the kernel
        // reports the timeout after about one wait limit
        if (!mbar_wait_bounded(&bar[cur], (k >> 1) & 1, WAIT_NS)) {
            bad = 1;
            mbar_wait_bounded(&bar[cur], (k >> 1) & 1, WAIT_NS);
        }
        if (__syncthreads_or(bad)) {
            bad = 1;
            if (nxt < t_end) {
                mbar_wait_bounded(&bar[cur ^ 1], ((k + 1) >> 1) & 1,
                                  WAIT_NS);
            }
            break;
        }
        if (threadIdx.x == 0 && nxt < t_end) {
            const Tile tn = tiles[nxt];
            note_slots(bd[tn.bunch], tn, &pads[2 * (cur ^ 1)]);
        }

        // both y-kicks: t2 = K_wake(t1) (zero off the mesh), t1' = K_rf(t2).
        // The 14 inputs of 8 outputs start at mesh position y0 + s; they
        // are read as five aligned float4 and picked at the row alignment.
        {
            const int seg = n >> 3;
            const int lg = lg_seg(n);
            const int rp = THREADS >> lg;
            const int l = threadIdx.x & (seg - 1);
            const int rl = threadIdx.x >> lg;
            const int y0 = 8 * l;
            for (int r = rl; r < nr; r += rp) {
                const RowInfo ri = S[r];
                const float* arow = A + size_t(r) * as;
                const int start = APAD + y0 + ri.s;
                float t2[11];
                if (start >= 0 && (start & ~3) + 20 <= as) {
                    const float4* src = reinterpret_cast<const float4*>(
                        arow + (start & ~3));
                    float c[20];
#pragma unroll
                    for (int q = 0; q < 5; q++) {
                        const float4 v = src[q];
                        c[4 * q] = v.x;
                        c[4 * q + 1] = v.y;
                        c[4 * q + 2] = v.z;
                        c[4 * q + 3] = v.w;
                    }
                    switch (start & 3) {
                    case 0: first_kick<0>(c, ri, t2); break;
                    case 1: first_kick<1>(c, ri, t2); break;
                    case 2: first_kick<2>(c, ri, t2); break;
                    default: first_kick<3>(c, ri, t2); break;
                    }
                } else {
                    // window beyond the padded row: off the mesh, zero
                    float c[14];
#pragma unroll
                    for (int q = 0; q < 14; q++) {
                        const int p = start + q;
                        c[q] = (p >= 0 && p < as) ? arow[p] : 0.f;
                    }
                    first_kick<0>(c, ri, t2);
                }
                const int q0 = y0 + ri.sb;    // mesh position of t2[0]
                if (q0 < 0 || q0 + 10 >= n) {
#pragma unroll
                    for (int i = 0; i < 11; i++) {
                        if (unsigned(q0 + i) >= unsigned(n)) {
                            t2[i] = 0.f;
                        }
                    }
                }
                float out[8];
#pragma unroll
                for (int q = 0; q < 8; q++) {
                    float v = ri.b[0] * t2[q];
                    v = fmaf(ri.b[1], t2[q + 1], v);
                    v = fmaf(ri.b[2], t2[q + 2], v);
                    v = fmaf(ri.b[3], t2[q + 3], v);
                    out[q] = v;
                }
                float4* dst = reinterpret_cast<float4*>(Bs + size_t(r) * n + y0);
                dst[0] = make_float4(out[0], out[1], out[2], out[3]);
                dst[1] = make_float4(out[4], out[5], out[6], out[7]);
            }
        }
        __syncthreads();

        // drift x-kick (per-column stencil), sliding window along x; t3
        // into T with TPAD zero columns on both sides
        const int tstride = n + 2 * TPAD;
        {
            const RowStencil* dr = st + B.st_off + ST_DRIFT * n;
            const int cols = n < THREADS ? n : THREADS;
            const int groups = THREADS / cols;
            const int col = threadIdx.x % cols;
            const int g = threadIdx.x / cols;
            const int chunk = (rows + groups - 1) / groups;
            const int rb = g * chunk;
            const int re = min(rows, rb + chunk);
            for (int y = col; y < n && rb < re; y += cols) {
                const RowStencil s = n <= THREADS ? dcol : dr[y];
                const float* cp = Bs + y;
                const int src = rb + hlo + s.shift0;   // staged row of tap 0
                float w0 = cp[size_t(src) * n];
                float w1 = cp[size_t(src + 1) * n];
                float w2 = cp[size_t(src + 2) * n];
                float w3 = cp[size_t(src + 3) * n];
                for (int r = rb; r < re; r++) {
                    float v = s.w[0] * w0;
                    v = fmaf(s.w[1], w1, v);
                    v = fmaf(s.w[2], w2, v);
                    v = fmaf(s.w[3], w3, v);
                    T[size_t(r) * tstride + TPAD + y] = v;
                    w0 = w1;
                    w1 = w2;
                    w2 = w3;
                    if (r + 1 < re) {
                        w3 = cp[size_t(src + (r - rb) + 4) * n];
                    }
                }
            }
            for (int i = threadIdx.x; i < rows * 2 * TPAD; i += THREADS) {
                const int r = i / (2 * TPAD), q = i % (2 * TPAD);
                T[size_t(r) * tstride + (q < TPAD ? q : n + q)] = 0.f;
            }
        }
        __syncthreads();

        // Fokker-Planck, output rows, projections
        fp_and_store(T, rows, n, x0, B, fpc, dout, pout, part);
        __syncthreads();
    }
    if (bad && threadIdx.x == 0) {
        atomicCAS(status, 0, VFPS_ERR_TIMEOUT);
    }
}

// ------------------------------------------- chain 0, meshes up to 256
// Lane mapping of the row stages: the n cells of a row are served by
// seg = n/8 consecutive lanes of one warp; lane l owns the two groups of 4
// columns that start at 4l and n/2 + 4l, so that the lanes of a row read
// and write consecutive 16-byte words (no shared-memory bank conflicts).
// Staged rows live in a ring of RB slots (twice the rows a tile reads) of
// RS floats: APAD zeros, the row, zeros; a tile's rows get the slots after
// the rows staged before it, and consecutive tiles of a bunch share their
// halo rows.  The drift and Fokker-Planck planes of the tile's bunch sit
// next to the ring (one bulk copy per distinct table).
constexpr int RTHREADS = 128;

struct SmemR {
    uint32_t ring;  // RB slots of RS floats
    uint32_t s;     // RowInfo of the new rows of one tile
    uint32_t tab;   // drift and Fokker-Planck planes of a bunch [10][n]
    uint32_t bar;   // three mbarriers (two for the rows, one for tab)
    uint32_t rb;    // ring slots: twice the rows a tile reads
    uint32_t rs;    // floats per slot
    uint32_t part;  // k_bmaps0f, 512/1024 rows: the parts' row sums
    uint32_t total;
};

// t2[i] = sum_j a_j c[AL + i + j] for the 7 positions the second kick of
// 4 cells reads
template <int AL>
__device__ __forceinline__ void kick7(const float* c, const RowInfo& ri,
                                      float* t2)
{
    // output pairs in packed FP32 (each component rounds like fmaf)
#pragma unroll
    for (int i = 0; i < 6; i += 2) {
        float2 v = __fmul2_rn(make_float2(ri.a[0], ri.a[0]),
                              make_float2(c[AL + i], c[AL + i + 1]));
#pragma unroll
        for (int j = 1; j < 4; j++) {
            v = __ffma2_rn(make_float2(ri.a[j], ri.a[j]),
                           make_float2(c[AL + i + j], c[AL + i + j + 1]), v);
        }
        t2[i] = v.x;
        t2[i + 1] = v.y;
    }
    float v = ri.a[0] * c[AL + 6];
    v = fmaf(ri.a[1], c[AL + 7], v);
    v = fmaf(ri.a[2], c[AL + 8], v);
    v = fmaf(ri.a[3], c[AL + 9], v);
    t2[6] = v;
}

// Both y-kicks of the 4 cells y..y+3 of a staged row (mesh value of
// column y at row[APAD + y]): t2 = K_wake(t1), zero off the mesh, then
// K_rf(t2).  The 10 inputs start at mesh column y + s.
__device__ __forceinline__ float4 ykick4(const float* row, int as, int n,
                                         int y, const RowInfo& ri)
{
    const int start = APAD + y + ri.s;
    float t2[7];
    if (start >= 0 && (start & ~3) + 16 <= as) {
        const float4* src = reinterpret_cast<const float4*>(row + (start & ~3));
        float c[16];
        const float4 v0 = src[0], v1 = src[1], v2 = src[2];
        c[0] = v0.x; c[1] = v0.y; c[2] = v0.z; c[3] = v0.w;
        c[4] = v1.x; c[5] = v1.y; c[6] = v1.z; c[7] = v1.w;
        c[8] = v2.x; c[9] = v2.y; c[10] = v2.z; c[11] = v2.w;
        switch (start & 3) {
        case 0: kick7<0>(c, ri, t2); break;
        case 1: kick7<1>(c, ri, t2); break;
        case 2: kick7<2>(c, ri, t2); break;
        default: {
            const float4 v3 = src[3];
            c[12] = v3.x; c[13] = v3.y; c[14] = v3.z; c[15] = v3.w;
            kick7<3>(c, ri, t2);
            break;
        }
        }
    } else {
        // window beyond the padded row: those cells are off the mesh
        float c[10];
#pragma unroll
        for (int q = 0; q < 10; q++) {
            const int p = start + q;
            c[q] = (p >= 0 && p < as) ? row[p] : 0.f;
        }
        kick7<0>(c, ri, t2);
    }
    const int q0 = y + ri.sb;    // mesh column of t2[0]
    if (q0 < 0 || q0 + 6 >= n) {
#pragma unroll
        for (int i = 0; i < 7; i++) {
            if (unsigned(q0 + i) >= unsigned(n)) {
                t2[i] = 0.f;
            }
        }
    }
    float o[4];
#pragma unroll
    for (int q = 0; q < 4; q += 2) {
        float2 v = __fmul2_rn(make_float2(ri.b[0], ri.b[0]),
                              make_float2(t2[q], t2[q + 1]));
#pragma unroll
        for (int i = 1; i < 4; i++) {
            v = __ffma2_rn(make_float2(ri.b[i], ri.b[i]),
                           make_float2(t2[q + i], t2[q + i + 1]), v);
        }
        o[q] = v.x;
        o[q + 1] = v.y;
    }
    return make_float4(o[0], o[1], o[2], o[3]);
}

// ring slot of mesh row x: (x - xref + pref) mod rb, where xref is the
// lowest row the tile reads (its first row less the halo) and pref < rb
// that row's slot, kept as off = pref - xref; a tile reads fewer than rb
// rows above xref, so one conditional subtraction reduces the sum (rb need
// not be a power of two)
struct RingMap {
    int off;
    __device__ __forceinline__ static RingMap at(int xref, int pref)
    {
        return RingMap{pref - xref};
    }
    __device__ __forceinline__ int slot(int x, int rb) const
    {
        const int s = x + off;
        return s >= rb ? s - rb : s;
    }
};

// bulk copies of the mesh rows among [lo, hi) into their slots, and of
// their y-kick stencils into S[x - lo] (warp 0).  The rows part arms the
// barrier with the byte count of both parts first (lane 0); the stencils
// part may follow later, the barrier's phase completes when both have
// landed.
template <typename Rec>
__device__ __forceinline__ void issue_rows(const BDev& B, int lo, int hi,
                                           const RingMap& m, float* ring,
                                           int rb, int rs,
                                           const float* __restrict__ din,
                                           const Rec* __restrict__ rinfo,
                                           Rec* S, uint64_t* bar,
                                           bool rows = true,
                                           bool stencils = true)
{
    const int n = int(B.n);
    // the rows inside the mesh; none when a short last tile's new rows lie
    // all beyond the mesh end (the previous tile's halo reached past it)
    const int a = max(lo, 0), e = max(min(hi, n), a);
    const uint32_t row_bytes = uint32_t(n) * 4u;
    const uint32_t ri_bytes = uint32_t(e - a) * uint32_t(sizeof(Rec));
    const int lane = threadIdx.x & 31;
    if (lane == 0) {
        if (rows) {
            fence_proxy_async();
            mbar_arrive_expect_tx(bar,
                                  uint32_t(e - a) * row_bytes + ri_bytes);
        }
        if (stencils && e > a) {
            tma_load_1d(S + (a - lo), rinfo + B.prof_off + a, ri_bytes, bar);
        }
    }
    if (rows) {
        __syncwarp();
        for (int x = a + lane; x < e; x += 32) {
            tma_load_1d(ring + size_t(m.slot(x, rb)) * rs + APAD,
                        din + B.dens_off + size_t(x) * n, row_bytes, bar);
        }
    }
}

// Drift x-kick of two output rows and 4 columns from the ring: tap j of
// output row X reads staged row X + shift + j.  The 5 staged rows stream
// through registers (tap j of the first row and tap j - 1 of the second
// share row j).
__device__ __forceinline__ void drift2(const float* ring, const RingMap& m,
                                       int rb, int rs, int X0, int y,
                                       const float* __restrict__ W, int n,
                                       float* d0, float* d1)
{
    const int4 sh = *(reinterpret_cast<const int4*>(W + 4 * n + y));
    if (sh.x == sh.y && sh.y == sh.z && sh.z == sh.w) {
        // packed FP32 (two lanes of 4 columns per instruction; each
        // component rounds like fmaf / a plain product)
        float4 wp = make_float4(0.f, 0.f, 0.f, 0.f);
        float2 a0 = make_float2(0.f, 0.f), b0 = a0, a1 = a0, b1 = a0;
#pragma unroll
        for (int j = 0; j < 5; j++) {
            const float4 v = *reinterpret_cast<const float4*>(
                ring + size_t(m.slot(X0 + sh.x + j, rb)) * rs + APAD + y);
            const float2 va = make_float2(v.x, v.y);
            const float2 vb = make_float2(v.z, v.w);
            float4 wj = wp;
            if (j < 4) {
                wj = *(reinterpret_cast<const float4*>(W + j * n + y));
            }
            const float2 wa = make_float2(wj.x, wj.y);
            const float2 wb = make_float2(wj.z, wj.w);
            const float2 pa = make_float2(wp.x, wp.y);
            const float2 pb = make_float2(wp.z, wp.w);
            if (j == 0) {
                a0 = __fmul2_rn(wa, va);
                b0 = __fmul2_rn(wb, vb);
            } else if (j < 4) {
                a0 = __ffma2_rn(wa, va, a0);
                b0 = __ffma2_rn(wb, vb, b0);
            }
            if (j == 1) {
                a1 = __fmul2_rn(pa, va);
                b1 = __fmul2_rn(pb, vb);
            } else if (j > 1) {
                a1 = __ffma2_rn(pa, va, a1);
                b1 = __ffma2_rn(pb, vb, b1);
            }
            wp = wj;
        }
        d0[0] = a0.x;
        d0[1] = a0.y;
        d0[2] = b0.x;
        d0[3] = b0.y;
        d1[0] = a1.x;
        d1[1] = a1.y;
        d1[2] = b1.x;
        d1[3] = b1.y;
    } else {
        // a shift boundary inside the 4 columns: column by column
        const int shv[4] = {sh.x, sh.y, sh.z, sh.w};
#pragma unroll
        for (int c = 0; c < 4; c++) {
            float q[5];
#pragma unroll
            for (int j = 0; j < 5; j++) {
                q[j] = ring[size_t(m.slot(X0 + shv[c] + j, rb)) * rs + APAD
                            + y + c];
            }
            const float w0 = W[y + c], w1 = W[n + y + c],
                        w2 = W[2 * n + y + c], w3 = W[3 * n + y + c];
            float v = w0 * q[0];
            v = fmaf(w1, q[1], v);
            v = fmaf(w2, q[2], v);
            v = fmaf(w3, q[3], v);
            d0[c] = v;
            float u = w0 * q[1];
            u = fmaf(w1, q[2], u);
            u = fmaf(w2, q[3], u);
            u = fmaf(w3, q[4], u);
            d1[c] = u;
        }
    }
}

// Fokker-Planck of two rows (d0, d1: their 8 lane cells after the drift,
// group A then group B) with the neighbours' cells taken by shuffles
// within the row's seg lanes; the weights of a group's 4 columns come as
// 5 planes F[o][y] (offsets -2..2).  Stores the rows (where valid) and
// returns their Simpson-weighted partial sums (in units of h03: the
// weights alternate 2, 4 along the row, 1 at both ends).
__device__ __forceinline__ void fp_rows2(const float* d0, const float* d1,
                                         int l, int seg, int n,
                                         const float* __restrict__ F,
                                         float* o0, float* o1, bool v0,
                                         bool v1, float& p0, float& p1)
{
    const int lp = (l + 1) & (seg - 1), lm = (l + seg - 1) & (seg - 1);
    const bool first = l == 0, last = l == seg - 1;
    // columns 2, 3 of the left lane's group A (group A's left neighbours,
    // and group B's on lane 0) and columns 0, 1 of the right lane's group B
    // (group B's right neighbours, and group A's on the last lane)
    float la[2][2], rb_[2][2];
#pragma unroll
    for (int r = 0; r < 2; r++) {
        const float* d = r ? d1 : d0;
        la[r][0] = __shfl_sync(0xffffffffu, d[2], lm, seg);
        la[r][1] = __shfl_sync(0xffffffffu, d[3], lm, seg);
        rb_[r][0] = __shfl_sync(0xffffffffu, d[4], lp, seg);
        rb_[r][1] = __shfl_sync(0xffffffffu, d[5], lp, seg);
    }
    float pe[2] = {0.f, 0.f}, po[2] = {0.f, 0.f};
#pragma unroll
    for (int g = 0; g < 2; g++) {
        const int y = g * (n >> 1) + 4 * l;
        float f[5][4];
#pragma unroll
        for (int o = 0; o < 5; o++) {
            const float4 v = *(reinterpret_cast<const float4*>(
                F + o * n + y));
            f[o][0] = v.x; f[o][1] = v.y; f[o][2] = v.z; f[o][3] = v.w;
        }
#pragma unroll
        for (int r = 0; r < 2; r++) {
            const float* d = (r ? d1 : d0) + 4 * g;
            float w[8];
            if (g == 0) {
                const float rA0 = __shfl_sync(0xffffffffu, d[0], lp, seg);
                const float rA1 = __shfl_sync(0xffffffffu, d[1], lp, seg);
                w[0] = first ? 0.f : la[r][0];
                w[1] = first ? 0.f : la[r][1];
                w[6] = last ? rb_[r][0] : rA0;
                w[7] = last ? rb_[r][1] : rA1;
            } else {
                const float lB2 = __shfl_sync(0xffffffffu, d[2], lm, seg);
                const float lB3 = __shfl_sync(0xffffffffu, d[3], lm, seg);
                w[0] = first ? la[r][0] : lB2;
                w[1] = first ? la[r][1] : lB3;
                w[6] = last ? 0.f : rb_[r][0];
                w[7] = last ? 0.f : rb_[r][1];
            }
#pragma unroll
            for (int c = 0; c < 4; c++) {
                w[2 + c] = d[c];
            }
            float out[4];
#pragma unroll
            for (int c = 0; c < 4; c++) {
                float v = f[0][c] * w[c];
                v = fmaf(f[1][c], w[c + 1], v);
                v = fmaf(f[2][c], w[c + 2], v);
                v = fmaf(f[3][c], w[c + 3], v);
                v = fmaf(f[4][c], w[c + 4], v);
                out[c] = v;
            }
            if (r ? v1 : v0) {
                *reinterpret_cast<float4*>((r ? o1 : o0) + y) =
                    make_float4(out[0], out[1], out[2], out[3]);
            }
            // Simpson weights along the row: even columns 2, odd 4, with
            // column 0 (lane 0, group A) and n - 1 (last lane, group B) 1
            float e = out[0] + out[2], od = out[1] + out[3];
            if (g == 0 && first) {
                e -= 0.5f * out[0];
            }
            if (g == 1 && last) {
                od -= 0.75f * out[3];
            }
            pe[r] += e;
            po[r] += od;
        }
    }
    p0 = fmaf(4.f, po[0], 2.f * pe[0]);
    p1 = fmaf(4.f, po[1], 2.f * pe[1]);
}

// Drift x-kick of one output row and 4 columns from the ring: tap j of row
// X reads staged row X + shift + j (the same taps and order as drift2's
// first row).
__device__ __forceinline__ void drift1(const float* ring, const RingMap& m,
                                       int rb, int rs, int X, int y,
                                       const float* __restrict__ W, int n,
                                       float* d)
{
    const int4 sh = *(reinterpret_cast<const int4*>(W + 4 * n + y));
    if (sh.x == sh.y && sh.y == sh.z && sh.z == sh.w) {
        // packed FP32 (each component rounds like fmaf / a plain product)
        float2 a = make_float2(0.f, 0.f), c = a;
#pragma unroll
        for (int j = 0; j < 4; j++) {
            const float4 v = *reinterpret_cast<const float4*>(
                ring + size_t(m.slot(X + sh.x + j, rb)) * rs + APAD + y);
            const float4 w = *(reinterpret_cast<const float4*>(
                W + j * n + y));
            const float2 va = make_float2(v.x, v.y);
            const float2 vb = make_float2(v.z, v.w);
            const float2 wa = make_float2(w.x, w.y);
            const float2 wb = make_float2(w.z, w.w);
            if (j == 0) {
                a = __fmul2_rn(wa, va);
                c = __fmul2_rn(wb, vb);
            } else {
                a = __ffma2_rn(wa, va, a);
                c = __ffma2_rn(wb, vb, c);
            }
        }
        d[0] = a.x;
        d[1] = a.y;
        d[2] = c.x;
        d[3] = c.y;
    } else {
        // a shift boundary inside the 4 columns: column by column
        const int shv[4] = {sh.x, sh.y, sh.z, sh.w};
#pragma unroll
        for (int q = 0; q < 4; q++) {
            float t[4];
#pragma unroll
            for (int j = 0; j < 4; j++) {
                t[j] = ring[size_t(m.slot(X + shv[q] + j, rb)) * rs + APAD
                            + y + q];
            }
            float v = W[y + q] * t[0];
            v = fmaf(W[n + y + q], t[1], v);
            v = fmaf(W[2 * n + y + q], t[2], v);
            v = fmaf(W[3 * n + y + q], t[3], v);
            d[q] = v;
        }
    }
}

// Fokker-Planck of one row whose 32 lanes own G groups of 4 columns each
// (group g: columns g n/G + 4l .. +3), neighbours by shuffles; the
// neighbour of group g left of lane 0 is group g-1 on lane 31 and right of
// lane 31 group g+1 on lane 0 (none beyond the mesh).  Stores the row
// (valid) and returns its Simpson-weighted sum in units of h03 (as
// fp_rows2).
template <int G>
__device__ __forceinline__ float fp_row(const float (&d)[G][4], int l, int n,
                                        const float* __restrict__ F,
                                        float* o, bool valid)
{
    const int lp = (l + 1) & 31, lm = (l + 31) & 31;
    const bool first = l == 0, last = l == 31;
    float L0[G], L1[G], R0[G], R1[G];
#pragma unroll
    for (int g = 0; g < G; g++) {
        L0[g] = __shfl_sync(0xffffffffu, d[g][2], lm);
        L1[g] = __shfl_sync(0xffffffffu, d[g][3], lm);
        R0[g] = __shfl_sync(0xffffffffu, d[g][0], lp);
        R1[g] = __shfl_sync(0xffffffffu, d[g][1], lp);
    }
    const int gw = n / G;
    float pe = 0.f, po = 0.f;
#pragma unroll
    for (int g = 0; g < G; g++) {
        const int y = g * gw + 4 * l;
        float f[5][4];
#pragma unroll
        for (int q = 0; q < 5; q++) {
            const float4 v = *(reinterpret_cast<const float4*>(
                F + q * n + y));
            f[q][0] = v.x;
            f[q][1] = v.y;
            f[q][2] = v.z;
            f[q][3] = v.w;
        }
        float w[8];
        w[0] = first ? (g > 0 ? L0[g > 0 ? g - 1 : 0] : 0.f) : L0[g];
        w[1] = first ? (g > 0 ? L1[g > 0 ? g - 1 : 0] : 0.f) : L1[g];
        w[6] = last ? (g < G - 1 ? R0[g < G - 1 ? g + 1 : g] : 0.f) : R0[g];
        w[7] = last ? (g < G - 1 ? R1[g < G - 1 ? g + 1 : g] : 0.f) : R1[g];
#pragma unroll
        for (int c = 0; c < 4; c++) {
            w[2 + c] = d[g][c];
        }
        float out[4];
#pragma unroll
        for (int c = 0; c < 4; c++) {
            float v = f[0][c] * w[c];
            v = fmaf(f[1][c], w[c + 1], v);
            v = fmaf(f[2][c], w[c + 2], v);
            v = fmaf(f[3][c], w[c + 3], v);
            v = fmaf(f[4][c], w[c + 4], v);
            out[c] = v;
        }
        if (valid) {
            *reinterpret_cast<float4*>(o + y) =
                make_float4(out[0], out[1], out[2], out[3]);
        }
        // Simpson weights along the row: even columns 2, odd 4, column 0
        // and n - 1 one
        float e = out[0] + out[2], od = out[1] + out[3];
        if (g == 0 && first) {
            e -= 0.5f * out[0];
        }
        if (g == G - 1 && last) {
            od -= 0.75f * out[3];
        }
        pe += e;
        po += od;
    }
    return fmaf(4.f, po, 2.f * pe);
}

// G = 2: meshes up to 256 rows, n/8 lanes per row, two rows per pass;
// G = 4: 512-row meshes, 32 lanes (one warp) per row, one row per pass
template <int G, int NT>
__global__ void __launch_bounds__(NT, G == 2 ? 4 : 2)
k_bmaps0(const BDev* __restrict__ bd, const Tile* __restrict__ tiles,
         uint32_t ntiles, const float* __restrict__ tabs,
         const float* __restrict__ dwt, const RowInfo* __restrict__ rinfo,
         const float* __restrict__ din, float* __restrict__ dout,
         float* __restrict__ pout, int* __restrict__ status, SmemR L)
{
    extern __shared__ float4 smem4[];
    char* base = reinterpret_cast<char*>(smem4);
    float* ring = reinterpret_cast<float*>(base + L.ring);
    RowInfo* S = reinterpret_cast<RowInfo*>(base + L.s);
    float* T = reinterpret_cast<float*>(base + L.tab);
    uint64_t* bar = reinterpret_cast<uint64_t*>(base + L.bar);
    const int rb = int(L.rb), rs = int(L.rs);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

    // the ring starts zero: slots are written only in
    // [APAD, n + 2 APAD + 16)
    {
        float4* r4 = reinterpret_cast<float4*>(ring);
        const float4 z = make_float4(0.f, 0.f, 0.f, 0.f);
        for (int i = threadIdx.x; i < rb * rs / 4; i += NT) {
            r4[i] = z;
        }
    }
    if (threadIdx.x == 0) {
        mbar_init(&bar[0], 1);
        mbar_init(&bar[1], 1);
        mbar_init(&bar[2], 1);
        mbar_fence_init();
    }
    fence_proxy_async();
    __syncthreads();

    // each CTA walks a contiguous chunk of the tile list: tiles of a bunch
    // are adjacent and in row order, so consecutive tiles share halo rows;
    // the chunks differ by at most one tile (no CTA left idle while others
    // carry a whole extra tile)
    const uint32_t t_begin = uint32_t(uint64_t(blockIdx.x) * ntiles
                                      / gridDim.x);
    const uint32_t t_end = uint32_t(uint64_t(blockIdx.x + 1) * ntiles
                                    / gridDim.x);

    // ring state of the current and of the next tile: slot mapping and the
    // new rows [lo, hi) staged for it
    RingMap mc{0}, mn{0};
    int lo_c = 0, hi_c = 0, lo_n = 0, hi_n = 0;
    int front = 0;   // ring position after the last staged row
    // the drift and Fokker-Planck planes in T: those of table tab_off
    // (bunches of one lattice share a table), a copy in flight while
    // tab_wait, completing phase tab_ph of bar[2]
    uint32_t tab_off = 0xffffffffu, tab_ph = 0;
    bool tab_wait = false;
    auto load_tab = [&](const BDev& Bt) {
        const uint32_t bytes = 10u * Bt.n * 4u;
        if (threadIdx.x == 0) {
            fence_proxy_async();
            mbar_arrive_expect_tx(&bar[2], bytes);
            tma_load_1d(T, dwt + Bt.dw_off, bytes, &bar[2]);
        }
        tab_off = Bt.dw_off;
        tab_wait = true;
    };
    if (t_begin < t_end) {
        const Tile t = tiles[t_begin];
        const BDev B = bd[t.bunch];
        load_tab(B);   // constant tables: before the wait below
        lo_c = int(t.x0) - B.halo_lo;
        hi_c = int(t.x0 + t.rows) + B.halo_hi;
        mc = RingMap::at(lo_c, 0);
        front = hi_c - lo_c;
        // the first tile's density rows already while the stencil kernel
        // runs: the previous step wrote them and had completed before that
        // kernel started
        if (warp == 0) {
            issue_rows(B, lo_c, hi_c, mc, ring, rb, rs, din, rinfo, S,
                       &bar[0], true, false);
        }
    }
    // this step's stencils are complete
    pdl_wait();
    if (t_begin < t_end && warp == 0) {
        const BDev B = bd[tiles[t_begin].bunch];
        issue_rows(B, lo_c, hi_c, mc, ring, rb, rs, din, rinfo, S, &bar[0],
                   false, true);
    }
    int bad = 0;
    for (uint32_t k = 0, tid = t_begin; tid < t_end; tid++, k++) {
        const Tile t = tiles[tid];
        const BDev B = bd[t.bunch];
        const int n = int(B.n);
        const int x0 = int(t.x0);
        const int rows = int(t.rows);
        const int seg = n / (4 * G);   // lanes per row
        const int l = threadIdx.x % seg;
        const int rl = threadIdx.x / seg;
        const int rp = NT / seg;
        const int as = astride0(n);

        // stage 1: both y-kicks of the new rows, in place
        {
            const int m = hi_c - lo_c;
            if (!mbar_wait_bounded(&bar[k & 1], (k >> 1) & 1, WAIT_NS)) {
                bad = 1;
                mbar_wait_bounded(&bar[k & 1], (k >> 1) & 1, WAIT_NS);
            }
            // lanes of one row: a segment of seg lanes of this warp
            const unsigned rmask = seg == 32 ? 0xffffffffu
                : (((1u << seg) - 1u) << (lane & ~(seg - 1)));
            const float4 z = make_float4(0.f, 0.f, 0.f, 0.f);
            for (int i = rl; i < m; i += rp) {
                const int x = lo_c + i;
                float* row = ring + size_t(mc.slot(x, rb)) * rs;
                // zeros right of the row: the slot may have held a longer
                // row of another bunch (rows as long as the slots leave
                // the zeros of the ring's start there)
                if (n + 2 * APAD + 16 < rs) {
                    for (int j = l; j < (APAD + 16) / 4; j += seg) {
                        reinterpret_cast<float4*>(row + APAD + n)[j] = z;
                    }
                }
                const int gw = n / G;   // columns per lane group
                if (unsigned(x) < unsigned(n)) {
                    const RowInfo ri = S[i];
                    __syncwarp(rmask);
                    float4 o[G];
#pragma unroll
                    for (int g = 0; g < G; g++) {
                        o[g] = ykick4(row, as, n, g * gw + 4 * l, ri);
                    }
                    __syncwarp(rmask);
#pragma unroll
                    for (int g = 0; g < G; g++) {
                        *reinterpret_cast<float4*>(row + APAD + g * gw
                                                   + 4 * l) = o[g];
                    }
                } else {
#pragma unroll
                    for (int g = 0; g < G; g++) {
                        reinterpret_cast<float4*>(row + APAD + g * gw)[l] = z;
                    }
                }
            }
        }
        // the in-place writes precede later bulk copies into these slots.
        // A wait of this CTA that ran out (here or on the tables) ends its
        // walk: no further copies are issued, the one of the tables still
        // in flight gets one more bounded wait, and the kernel reports
        // VFPS_ERR_TIMEOUT after about one wait limit instead of one per
        // remaining tile
        fence_proxy_async();
        if (__syncthreads_or(bad)) {
            bad = 1;
            if (tab_wait) {
                mbar_wait_bounded(&bar[2], tab_ph, WAIT_NS);
            }
            break;
        }

        // stage the next tile's new rows: their slots hold no row that this
        // tile still reads (the ring holds two tiles with their halos)
        if (tid + 1 < t_end) {
            const Tile tn = tiles[tid + 1];
            const BDev Bn = bd[tn.bunch];
            const bool cont = tn.bunch == t.bunch
                              && int(tn.x0) == x0 + rows;
            hi_n = int(tn.x0 + tn.rows) + Bn.halo_hi;
            const int xr = int(tn.x0) - Bn.halo_lo;   // lowest row it reads
            if (cont) {
                // the same slots, referred to the next tile's lowest row
                mn = RingMap::at(xr, mc.slot(xr, rb));
                lo_n = hi_c;
            } else {
                lo_n = xr;
                mn = RingMap::at(xr, front);
            }
            front = mn.slot(hi_n, rb);
            if (warp == 0) {
                issue_rows(Bn, lo_n, hi_n, mn, ring, rb, rs, din, rinfo, S,
                           &bar[(k + 1) & 1]);
            }
        }

        // this tile's drift and Fokker-Planck planes in T (a new table is
        // copied in after the barrier above, which ends the last tile's
        // reads of the old one)
        if (B.dw_off != tab_off) {
            load_tab(B);
        }
        if (tab_wait) {
            if (!mbar_wait_bounded(&bar[2], tab_ph, WAIT_NS)) {
                bad = 1;
                mbar_wait_bounded(&bar[2], tab_ph, WAIT_NS);
            }
            tab_ph ^= 1u;
            tab_wait = false;
        }

        // drift x-kick, Fokker-Planck, output rows and projections, two
        // rows per lane segment
        if constexpr (G == 2) {
            const float* W = T;                   // drift planes [5][n]
            const float* F = W + 5 * n;           // Fokker-Planck [5][n]
            const float h03 = tabs[B.tab_off + TAB_WS * n];
            const int hw = seg >> 1;
            for (int rbase = 0; rbase < rows; rbase += 2 * rp) {
                const int r0 = rbase + 2 * rl;
                const bool v0 = r0 < rows, v1 = r0 + 1 < rows;
                const int X0 = x0 + (v0 ? r0 : 0);
                float d0[8], d1[8];
                drift2(ring, mc, rb, rs, X0, 4 * l, W, n, d0, d1);
                drift2(ring, mc, rb, rs, X0, (n >> 1) + 4 * l, W, n, d0 + 4,
                       d1 + 4);
                float* o0 = dout + B.dens_off + size_t(X0) * n;
                float pa, pb;
                fp_rows2(d0, d1, l, seg, n, F, o0, o0 + n, v0, v1, pa, pb);
                // row sums of both rows in one butterfly: the lower half of
                // the segment sums row r0, the upper half row r0 + 1
                const bool up = (l & hw) != 0;
                float v = (up ? pb : pa)
                          + __shfl_xor_sync(0xffffffffu, up ? pa : pb, hw);
                for (int o = hw >> 1; o > 0; o >>= 1) {
                    v += __shfl_xor_sync(0xffffffffu, v, o);
                }
                if ((l & (hw - 1)) == 0 && (up ? v1 : v0)) {
                    pout[B.prof_off + X0 + (up ? 1 : 0)] = h03 * v;
                }
            }
        } else {
            // one row per warp and pass, G groups of 4 columns per lane
            const float* W = T;                   // drift planes [5][n]
            const float* F = W + 5 * n;           // Fokker-Planck [5][n]
            const float h03 = tabs[B.tab_off + TAB_WS * n];
            const int gw = n / G;
            for (int rbase = 0; rbase < rows; rbase += rp) {
                const int r = rbase + rl;
                const bool valid = r < rows;
                const int X = x0 + (valid ? r : 0);
                float d[G][4];
#pragma unroll
                for (int g = 0; g < G; g++) {
                    drift1(ring, mc, rb, rs, X, g * gw + 4 * l, W, n, d[g]);
                }
                float* o = dout + B.dens_off + size_t(X) * n;
                float v = fp_row<G>(d, l, n, F, o, valid);
#pragma unroll
                for (int q = 16; q > 0; q >>= 1) {
                    v += __shfl_xor_sync(0xffffffffu, v, q);
                }
                if (l == 0 && valid) {
                    pout[B.prof_off + X] = h03 * v;
                }
            }
        }
        mc = mn;
        lo_c = lo_n;
        hi_c = hi_n;
    }
    if (bad && threadIdx.x == 0) {
        atomicCAS(status, 0, VFPS_ERR_TIMEOUT);
    }
}

// --------------------------------------------------------------- chain 1
struct Smem1 {
    size_t a, b, s, part, cols, total;
};

// A = staged rows [nr][n + 8] (4 zero columns each side, 16-byte aligned
// rows), B = rotated rows [rows][n + ROWPAD] (pre-shifted by the wake
// kick), S = RowStencil[rows], part = [rows][8], cols = sin(-a) p[y] and
// cos(-a) p[y] [2][n]; t3 reuses A.
__host__ __device__ inline Smem1 smem1(int n, int nr, int rows)
{
    Smem1 L;
    L.a = 0;
    const size_t a_rows = size_t(nr) * (n + 8);
    const size_t t_rows = size_t(rows) * (n + 2 * TPAD);
    L.b = align16(L.a + sizeof(float) * (a_rows > t_rows ? a_rows : t_rows));
    L.s = align16(L.b + sizeof(float) * size_t(rows) * (n + ROWPAD));
    L.part = align16(L.s + sizeof(RowStencil) * rows);
    L.cols = align16(L.part + sizeof(float) * size_t(rows) * 8);
    L.total = align16(L.cols + sizeof(float) * 2 * size_t(n));
    return L;
}

// Lagrange weights (calcCoefficiants, src/SM/SourceMap.cpp:142-170) of two
// fractions at once, in packed FP32: each component rounds as the scalar
// form's fmul / fadd / fsub (a - b computed as a + (-b), the same bits)
template <int IT>
__device__ __forceinline__ void coefficients2(float2* ic, float2 f)
{
    const float2 one = make_float2(1.f, 1.f);
    const float2 mone = make_float2(-1.f, -1.f);
    if (IT == 2) {
        ic[0] = __fadd2_rn(one, make_float2(-f.x, -f.y));
        ic[1] = f;
    } else if (IT == 3) {
        const float2 half = make_float2(0.5f, 0.5f);
        ic[0] = __fmul2_rn(__fmul2_rn(f, __fadd2_rn(f, mone)), half);
        const float2 ff = __fmul2_rn(f, f);
        ic[1] = __fadd2_rn(one, make_float2(-ff.x, -ff.y));
        ic[2] = __fmul2_rn(__fmul2_rn(f, __fadd2_rn(f, one)), half);
    } else {
        const float2 fm1 = __fadd2_rn(f, mone);
        const float2 fm2 = __fadd2_rn(f, make_float2(-2.f, -2.f));
        const float2 fp1 = __fadd2_rn(f, one);
        const float2 tmf = __fadd2_rn(make_float2(2.f, 2.f),
                                      make_float2(-f.x, -f.y));
        const float s6 = static_cast<float>(-1. / 6.);
        const float p6 = static_cast<float>(1. / 6.);
        ic[0] = __fmul2_rn(__fmul2_rn(__fmul2_rn(fm1, fm2), f),
                           make_float2(s6, s6));
        ic[1] = __fmul2_rn(__fmul2_rn(__fmul2_rn(fp1, fm1), fm2),
                           make_float2(0.5f, 0.5f));
        ic[2] = __fmul2_rn(__fmul2_rn(__fmul2_rn(tmf, f), fp1),
                           make_float2(0.5f, 0.5f));
        ic[3] = __fmul2_rn(__fmul2_rn(__fmul2_rn(f, fp1), fm1),
                           make_float2(p6, p6));
    }
}

// The rotation (src/SM/RotationMap.cpp:97-260) of a tile's rows from the
// staged rows A ([nr][n + 8], 4 zero columns each side) into Bs
// ([rows][n + ROWPAD], slot j of row r holds mesh column j + the row's
// wake kick shift), for interpolation with IT points per axis (the
// reference's calcCoefficiants, src/SM/SourceMap.cpp:142-170) and, when
// CLAMP, the CPU path's clamp to the 2x2 nearest taps.  A warp per row;
// each lane computes the slots j and j + 32 together: their source
// coordinates, Lagrange weights and tap sums in packed FP32 (each
// component rounds as the scalar operation), their taps and clamps one
// by one.  NC: the mesh size as a constant (0: the bunch's).
template <int IT, bool CLAMP, int NC>
__device__ __forceinline__ void rotate_rows(
    const BDev& B, int x0, int rows, int hlo, const float* __restrict__ tabs,
    const float* __restrict__ din, float fac, const float* A, float* Bs,
    const RowStencil* S, const float* snp, const float* csp)
{
    const int n = NC ? NC : int(B.n);
    const int astride = n + 8;
    const int bstride = n + ROWPAD;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    constexpr int NW = THREADS / 32;
    constexpr int h = (IT - 1) / 2;
    const float* qv = tabs + B.tab_off + TAB_Q * n;
    const float cell0 = CLAMP ? din[B.dens_off] * fac : 0.f;
    const float inv_dq = 1.f / B.dq, inv_dp = 1.f / B.dp;
    const float2 idq2 = make_float2(inv_dq, inv_dq);
    const float2 idp2 = make_float2(inv_dp, inv_dp);
    const float2 zbq2 = make_float2(B.zbq, B.zbq);
    const float2 zbp2 = make_float2(B.zbp, B.zbp);
    // staged row of tap i1 of base x1: x1 + i1 - h - (x0 - hlo)
    const int row0 = hlo - h - x0;
    for (int r = warp; r < rows; r += NW) {
        const float q = qv[x0 + r];
        const float cq = __fmul_rn(B.cs, q), sq = __fmul_rn(B.sn, q);
        const float2 cq2 = make_float2(cq, cq), sq2 = make_float2(sq, sq);
        const int sh = S[r].shift0;
        float* brow = Bs + size_t(r) * bstride;
        for (int j = lane; j < bstride; j += 64) {
            const int jb = j + 32;
            const bool hasb = jb < bstride;
            const int ya = j + sh, yb = jb + sh;   // mesh columns
            const bool ina = unsigned(ya) < unsigned(n);
            const bool inb = hasb && unsigned(yb) < unsigned(n);
            const int ca = ina ? ya : 0, cb = inb ? yb : 0;
            const float2 sn2 = make_float2(-snp[ca], -snp[cb]);
            const float2 cs2 = make_float2(csp[ca], csp[cb]);
            const float2 x1r = __ffma2_rn(__fadd2_rn(cq2, sn2), idq2, zbq2);
            const float2 y1r = __ffma2_rn(__fadd2_rn(sq2, cs2), idp2, zbp2);
            int x1a = 0, y1a = 0, x1b = 0, y1b = 0;
            float2 xf, yf;
            const bool oka = base_index(x1r.x, n, &x1a, &xf.x)
                             & base_index(y1r.x, n, &y1a, &yf.x) & ina;
            const bool okb = base_index(x1r.y, n, &x1b, &xf.y)
                             & base_index(y1r.y, n, &y1b, &yf.y) & inb;
            float2 icq[4], icp[4];
            coefficients2<IT>(icq, xf);
            coefficients2<IT>(icp, yf);
            float ta[IT][IT], tb[IT][IT];
            // the taps of each slot (a slot without a source cell reads
            // none: zeros)
            {
                const float* sa = A + size_t(x1a + row0) * astride
                                  + (y1a - h + 4);
                const float* sb = A + size_t(x1b + row0) * astride
                                  + (y1b - h + 4);
#pragma unroll
                for (int i1 = 0; i1 < IT; i1++) {
#pragma unroll
                    for (int j1 = 0; j1 < IT; j1++) {
                        ta[i1][j1] = oka ? sa[i1 * astride + j1] : 0.f;
                        tb[i1][j1] = okb ? sb[i1 * astride + j1] : 0.f;
                    }
                }
            }
            float2 v = make_float2(0.f, 0.f);
#pragma unroll
            for (int i1 = 0; i1 < IT; i1++) {
                float2 rv = make_float2(0.f, 0.f);
#pragma unroll
                for (int j1 = 0; j1 < IT; j1++) {
                    rv = __ffma2_rn(make_float2(ta[i1][j1], tb[i1][j1]),
                                    icp[j1], rv);
                }
                v = __ffma2_rn(rv, icq[i1], v);
            }
            float va = oka ? v.x : 0.f, vb = okb ? v.y : 0.f;
            if (CLAMP) {
                // 2x2 nearest taps; taps off the mesh read cell (0,0),
                // as the CPU path's clamp does
                auto clamp1 = [&](float val, bool ok, bool in, int x1,
                                  int y1, const float (&tap)[IT][IT]) {
                    float hi = FLT_MIN, lo = FLT_MAX;
#pragma unroll
                    for (int i1 = 1; i1 <= 2; i1++) {
#pragma unroll
                        for (int j1 = 1; j1 <= 2; j1++) {
                            const int i0 = x1 + i1 - h, j0 = y1 + j1 - h;
                            const bool inm = ok
                                && unsigned(i0) < unsigned(n)
                                && unsigned(j0) < unsigned(n);
                            const float sv = inm ? tap[i1 < IT ? i1 : 0]
                                                      [j1 < IT ? j1 : 0]
                                                 : cell0;
                            hi = (hi < sv) ? sv : hi;
                            lo = (sv < lo) ? sv : lo;
                        }
                    }
                    const float tmin = (val < hi) ? val : hi;
                    const float c = (tmin < lo) ? lo : tmin;
                    return in ? c : 0.f;
                };
                va = clamp1(va, oka, ina, x1a, y1a, ta);
                vb = clamp1(vb, okb, inb, x1b, y1b, tb);
            }
            brow[j] = va;
            if (hasb) {
                brow[jb] = vb;
            }
        }
    }
}

// Chain 1 (the rotation scheme: RotationMap, wake kick, Fokker-Planck) on
// a tile of rows, one CTA per tile.  Warps own whole rows in every stage:
//  staging   the tile's rows with the rotation's halo, 16-byte loads, times
//            the renormalisation factor;
//  rotation  (src/SM/RotationMap.cpp:97-260) every output cell from the
//            16 taps of its source cell's neighbourhood; the source
//            coordinates (cos q - sin p)/dq + zbq and (sin q + cos p)/dp
//            + zbp from per-row and per-column products and the
//            reciprocals of dq and dp (the reference divides; the base
//            cell can differ where a coordinate lies within one rounding
//            of an integer); truncation toward zero, off-mesh bases give
//            0, taps off the mesh read the zero halo; with clamping the
//            result is held within the 2x2 nearest taps as the CPU path
//            does.  Rows are written pre-shifted by the row's wake kick;
//  wake kick, Fokker-Planck, new rows and projections.
__global__ void __launch_bounds__(THREADS, 3)
k_bmaps1(const BDev* __restrict__ bd, const Tile* __restrict__ tiles,
         const float* __restrict__ tabs, const float* __restrict__ fp5,
         const float* __restrict__ wake, const float* __restrict__ factor,
         const float* __restrict__ din, float* __restrict__ dout,
         float* __restrict__ pout)
{
    extern __shared__ float4 smem4[];
    char* base = reinterpret_cast<char*>(smem4);
    const Tile t = tiles[blockIdx.x];
    const BDev B = bd[t.bunch];
    const int n = int(B.n);
    const int x0 = int(t.x0);
    const int rows = int(t.rows);
    const int hlo = B.halo_lo, hhi = B.halo_hi;
    const int nr = rows + hlo + hhi;
    const Smem1 L = smem1(n, nr, rows);
    float* A = reinterpret_cast<float*>(base + L.a);
    float* Bs = reinterpret_cast<float*>(base + L.b);
    RowStencil* S = reinterpret_cast<RowStencil*>(base + L.s);
    float* part = reinterpret_cast<float*>(base + L.part);
    float* snp = reinterpret_cast<float*>(base + L.cols);
    float* csp = snp + n;
    const int it = int(B.it);
    const float fac = factor[t.bunch];
    const int astride = n + 8;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    constexpr int NW = THREADS / 32;

    // wake kick of the tile rows; the rotation's column products
    for (int r = threadIdx.x; r < rows; r += THREADS) {
        RowStencil sa;
        if (B.flags & F_WAKE) {
            sa = make_stencil(wake[B.prof_off + x0 + r], B.n, it);
        } else {
            sa.shift0 = 0;
            sa.w[0] = 1.f;
            sa.w[1] = sa.w[2] = sa.w[3] = 0.f;
        }
        S[r] = sa;
    }
    {
        const float* pv = tabs + B.tab_off + TAB_P * n;
        for (int y = threadIdx.x; y < n; y += THREADS) {
            const float p = pv[y];
            snp[y] = __fmul_rn(B.sn, p);
            csp[y] = __fmul_rn(B.cs, p);
        }
    }
    // stage rows x0-hlo .. x0+rows+hhi with 4 zero columns on each side
    {
        const float* src = din + B.dens_off;
        const float4 z = make_float4(0.f, 0.f, 0.f, 0.f);
        const int nq = n >> 2;
        for (int r = warp; r < nr; r += NW) {
            const int x = x0 - hlo + r;
            float4* arow = reinterpret_cast<float4*>(A + size_t(r) * astride);
            const bool in = unsigned(x) < unsigned(n);
            const float4* srow = reinterpret_cast<const float4*>(
                src + size_t(in ? x : 0) * n);
            for (int c = lane; c < nq; c += 32) {
                float4 v = z;
                if (in) {
                    v = __ldg(srow + c);
                    v.x *= fac;
                    v.y *= fac;
                    v.z *= fac;
                    v.w *= fac;
                }
                arow[1 + c] = v;
            }
            if (lane == 0) {
                arow[0] = z;
                arow[1 + nq] = z;
            }
        }
    }
    __syncthreads();

    // rotation of the tile rows, each output written pre-shifted by its
    // row's wake kick shift (the interpolation order and the clamp are
    // the bunch's: one instance each, chosen once per tile)
    {
        const bool clamp = B.flags & F_CLAMP;
        // 256-row meshes (the benchmark's) with the mesh size a constant
        if (n == 256) {
            switch (it) {
            case 2:
                rotate_rows<2, false, 256>(B, x0, rows, hlo, tabs, din, fac,
                                           A, Bs, S, snp, csp);
                break;
            case 3:
                rotate_rows<3, false, 256>(B, x0, rows, hlo, tabs, din, fac,
                                           A, Bs, S, snp, csp);
                break;
            default:
                if (clamp) {
                    rotate_rows<4, true, 256>(B, x0, rows, hlo, tabs, din,
                                              fac, A, Bs, S, snp, csp);
                } else {
                    rotate_rows<4, false, 256>(B, x0, rows, hlo, tabs, din,
                                               fac, A, Bs, S, snp, csp);
                }
                break;
            }
        } else {
            switch (it) {
            case 2:
                rotate_rows<2, false, 0>(B, x0, rows, hlo, tabs, din, fac, A,
                                         Bs, S, snp, csp);
                break;
            case 3:
                rotate_rows<3, false, 0>(B, x0, rows, hlo, tabs, din, fac, A,
                                         Bs, S, snp, csp);
                break;
            default:
                if (clamp) {
                    rotate_rows<4, true, 0>(B, x0, rows, hlo, tabs, din, fac,
                                            A, Bs, S, snp, csp);
                } else {
                    rotate_rows<4, false, 0>(B, x0, rows, hlo, tabs, din,
                                             fac, A, Bs, S, snp, csp);
                }
                break;
            }
        }
    }
    __syncthreads();

    // wake y-kick: t3[x][y] = sum_j w_j t2[x][y + shift0 + j], the row of
    // Bs already starts at shift0; t3 goes to A with TPAD zero columns.
    // Lane segments of n/8 lanes own 8 columns of a row each.
    float* T = A;
    const int tstride = n + 2 * TPAD;
    {
        const int seg = n >> 3;
        const int lg = lg_seg(n);
        const int rp = THREADS >> lg;
        const int l = threadIdx.x & (seg - 1);
        const int y = 8 * l;
        for (int r = threadIdx.x >> lg; r < rows; r += rp) {
            const RowStencil s = S[r];
            const float4* br = reinterpret_cast<const float4*>(
                Bs + size_t(r) * (n + ROWPAD) + y);
            const float4 v0 = br[0], v1 = br[1], v2 = br[2];
            const float c[12] = {v0.x, v0.y, v0.z, v0.w, v1.x, v1.y,
                                 v1.z, v1.w, v2.x, v2.y, v2.z, v2.w};
            float o[8];
#pragma unroll
            for (int k = 0; k < 8; k++) {
                float a = s.w[0] * c[k];
                a = fmaf(s.w[1], c[k + 1], a);
                a = fmaf(s.w[2], c[k + 2], a);
                a = fmaf(s.w[3], c[k + 3], a);
                o[k] = a;
            }
            float* trow = T + size_t(r) * tstride;
            reinterpret_cast<float4*>(trow + TPAD + y)[0] =
                make_float4(o[0], o[1], o[2], o[3]);
            reinterpret_cast<float4*>(trow + TPAD + y)[1] =
                make_float4(o[4], o[5], o[6], o[7]);
            if (l == 0) {
                reinterpret_cast<float4*>(trow)[0] =
                    make_float4(0.f, 0.f, 0.f, 0.f);
                reinterpret_cast<float4*>(trow + TPAD + n)[0] =
                    make_float4(0.f, 0.f, 0.f, 0.f);
            }
        }
    }
    __syncthreads();
    FpCols fpc;
    load_fp_cols(B, fp5, tabs + B.tab_off + TAB_WS * n, fpc);
    fp_and_store(T, rows, n, x0, B, fpc, dout, pout, part);
}

// ------------------------------------------------------------- set-up
// warp per packed row: profile of the current density
__global__ void k_bproject(const BDev* __restrict__ bd,
                           const uint32_t* __restrict__ row_bunch,
                           const float* __restrict__ tabs,
                           const float* __restrict__ dens,
                           float* __restrict__ prof, uint32_t total_rows)
{
    const uint32_t r = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (r >= total_rows) {
        return;
    }
    const BDev B = bd[row_bunch[r]];
    const uint32_t x = r - B.prof_off;
    if (x >= B.n) {
        return;
    }
    const float* src = dens + B.dens_off + size_t(x) * B.n;
    const float* ws = tabs + B.tab_off + TAB_WS * B.n;
    float acc = 0.f;
    for (uint32_t y = lane; y < B.n; y += 32) {
        acc = fmaf(src[y], ws[y], acc);
    }
    acc = warp_sum_f(acc);
    if (lane == 0) {
        prof[r] = acc;
    }
}

// block per bunch: filling = sum proj ws (FP64); optionally normalise
__global__ void k_bintegrate(const BDev* __restrict__ bd,
                             const float* __restrict__ tabs,
                             const float* __restrict__ prof,
                             float* __restrict__ dens,
                             double* __restrict__ filling, int normalize)
{
    __shared__ double red[32];
    __shared__ float s_f;
    const BDev B = bd[blockIdx.x];
    const float* ws = tabs + B.tab_off + TAB_WS * B.n;
    double acc = 0;
    for (uint32_t i = threadIdx.x; i < B.n; i += blockDim.x) {
        acc += double(prof[B.prof_off + i]) * double(ws[i]);
    }
    acc = block_sum(acc, red);
    if (threadIdx.x == 0) {
        if (!normalize) {
            filling[blockIdx.x] = acc;
        }
        s_f = B.fillset > 0
                  ? static_cast<float>(double(B.fillset) / filling[blockIdx.x])
                  : 0.f;
    }
    __syncthreads();
    if (normalize) {
        const float f = s_f;
        float* d = dens + B.dens_off;
        const size_t cells = size_t(B.n) * B.n;
        for (size_t i = threadIdx.x; i < cells; i += blockDim.x) {
            d[i] = B.fillset > 0 ? d[i] * f : 0.f;
        }
    }
}

__global__ void k_bgauss(const BDev* __restrict__ bd,
                         const uint32_t* __restrict__ goff,
                         const float* __restrict__ g, float* __restrict__ dens)
{
    const BDev B = bd[blockIdx.y];
    const size_t cells = size_t(B.n) * B.n;
    const float* gx = g + goff[blockIdx.y];
    const float* gy = gx + B.n;
    for (size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x; i < cells;
         i += size_t(gridDim.x) * blockDim.x) {
        dens[B.dens_off + i] = __fmul_rn(gx[i / B.n], gy[i % B.n]);
    }
}

}  // namespace
