// k_bmaps0f: chain 0 (the reference's loop, src/main.cpp:1034-1044:
// wake kick, RF kick, drift, Fokker-Planck) for meshes of 64, 128, 256,
// 512 and 1024 rows whose lattice has the regular form of the benchmark's
// scans (checked on the host, fast_ring_ok): every aligned group of 4
// energy columns has one drift shift (1024 rows: at most two adjacent
// ones), and the Fokker-Planck stencil of the lower half of the energy
// axis spans offsets -2..1, that of the upper half -1..2 (the cubic
// stencil of a mesh centred on the reference energy, whose last lower
// column may take the upper form and reach -2..2; two-sided stencils and
// no Fokker-Planck fit too).  Other lattices run on k_bmaps0 / k_bmaps0w.
//
// Included by batch.cu after batch_kernels.cuh (shares its ring, tiles and
// bulk-copy helpers).  Per tile of rows, as k_bmaps0:
//  stage 1  both y-kicks of the tile's new staged rows as one 7-tap
//           stencil (RowInfo7), in place in the ring: a row's shift is
//           the same for all its lanes, so the window alignment and the
//           bounds test are warp-uniform branches;
//  stage 2  each segment of n/8 lanes walks a contiguous run of the
//           tile's output rows with a sliding window of 4 staged rows per
//           group of 4 columns in registers (one new row per output row),
//           the drift weights in registers for the whole tile, the drift
//           in packed FP32, Fokker-Planck with 4 taps (neighbour columns
//           by shuffles), the new row to HBM and its Simpson sum; the row
//           sums of 4 output rows leave in one reduce-scatter.
// 512- and 1024-row meshes: stage 1 gives a row to one warp (n/128 column
// groups per lane); in stage 2 a group of n/256 warps walks the rows, one
// warp per part of 256 columns (two groups per lane, as a 256-row mesh),
// each warp computing the drift of the columns past its part that its
// Fokker-Planck stencils reach from 2-column windows of its own; the
// parts' row sums meet in shared memory and are stored after the tile's
// next barrier.  1024 rows: 5-row drift windows (a group spanning two
// shifts reads one more row) and 256-thread CTAs.
#pragma once

namespace {

// 4 outputs y..y+3 of the composite y-kick from the 16-byte aligned
// window src (AL: offset of column y + s in it)
template <int AL>
__device__ __forceinline__ float4 ykick7(const float* src, const float (&c)[7])
{
    const float4* s4 = reinterpret_cast<const float4*>(src);
    float v[16];
    const float4 v0 = s4[0], v1 = s4[1], v2 = s4[2];
    v[0] = v0.x; v[1] = v0.y; v[2] = v0.z; v[3] = v0.w;
    v[4] = v1.x; v[5] = v1.y; v[6] = v1.z; v[7] = v1.w;
    v[8] = v2.x; v[9] = v2.y; v[10] = v2.z; v[11] = v2.w;
    if (AL == 3) {
        const float4 v3 = s4[3];
        v[12] = v3.x; v[13] = v3.y; v[14] = v3.z; v[15] = v3.w;
    } else {
        v[12] = v[13] = v[14] = v[15] = 0.f;
    }
    float o[4];
#pragma unroll
    for (int q = 0; q < 4; q++) {
        float a = c[0] * v[AL + q];
#pragma unroll
        for (int k = 1; k < 7; k++) {
            a = fmaf(c[k], v[AL + q + k], a);
        }
        o[q] = a;
    }
    return make_float4(o[0], o[1], o[2], o[3]);
}

// the same with every read bounds-checked against the staged row [0, as)
__device__ __forceinline__ float4 ykick7_checked(const float* row, int start,
                                                 int as, const float (&c)[7])
{
    float v[10];
#pragma unroll
    for (int q = 0; q < 10; q++) {
        const int p = start + q;
        v[q] = (p >= 0 && p < as) ? row[p] : 0.f;
    }
    float o[4];
#pragma unroll
    for (int q = 0; q < 4; q++) {
        float a = c[0] * v[q];
#pragma unroll
        for (int k = 1; k < 7; k++) {
            a = fmaf(c[k], v[q + k], a);
        }
        o[q] = a;
    }
    return make_float4(o[0], o[1], o[2], o[3]);
}

// ykick7 on G column groups STEP floats apart
template <int AL, int G, int STEP>
__device__ __forceinline__ void ykick7_groups(const float* src,
                                              const float (&c)[7],
                                              float4 (&o)[G])
{
#pragma unroll
    for (int g = 0; g < G; g++) {
        o[g] = ykick7<AL>(src + g * STEP, c);
    }
}

// drift x-kick of 4 columns: tap j of the output reads window row r[j]
// (packed FP32: two columns per instruction, each component rounded like
// fmaf / a plain product)
__device__ __forceinline__ float4 drift4(const float4& r0, const float4& r1,
                                         const float4& r2, const float4& r3,
                                         const float4 (&w)[4])
{
    float2 lo = __fmul2_rn(make_float2(w[0].x, w[0].y),
                           make_float2(r0.x, r0.y));
    float2 hi = __fmul2_rn(make_float2(w[0].z, w[0].w),
                           make_float2(r0.z, r0.w));
    lo = __ffma2_rn(make_float2(w[1].x, w[1].y), make_float2(r1.x, r1.y), lo);
    hi = __ffma2_rn(make_float2(w[1].z, w[1].w), make_float2(r1.z, r1.w), hi);
    lo = __ffma2_rn(make_float2(w[2].x, w[2].y), make_float2(r2.x, r2.y), lo);
    hi = __ffma2_rn(make_float2(w[2].z, w[2].w), make_float2(r2.z, r2.w), hi);
    lo = __ffma2_rn(make_float2(w[3].x, w[3].y), make_float2(r3.x, r3.y), lo);
    hi = __ffma2_rn(make_float2(w[3].z, w[3].w), make_float2(r3.z, r3.w), hi);
    return make_float4(lo.x, lo.y, hi.x, hi.y);
}

// the same for 2 columns (the operations of drift4's first pair)
__device__ __forceinline__ float2 drift2(const float2& r0, const float2& r1,
                                         const float2& r2, const float2& r3,
                                         const float2 (&w)[4])
{
    float2 v = __fmul2_rn(w[0], r0);
    v = __ffma2_rn(w[1], r1, v);
    v = __ffma2_rn(w[2], r2, v);
    v = __ffma2_rn(w[3], r3, v);
    return v;
}

template <int V>
struct IntC {
    static constexpr int value = V;
};

// Fokker-Planck of 4 columns with 4 taps: out[c] = sum_o F_o[c] w[c + o]
// (w: the 7 drift values the taps reach, F_o: weight planes)
__device__ __forceinline__ float4 fp4(const float (&w)[7], const float4& f0,
                                      const float4& f1, const float4& f2,
                                      const float4& f3)
{
    const float a0[4] = {f0.x, f0.y, f0.z, f0.w};
    const float a1[4] = {f1.x, f1.y, f1.z, f1.w};
    const float a2[4] = {f2.x, f2.y, f2.z, f2.w};
    const float a3[4] = {f3.x, f3.y, f3.z, f3.w};
    float o[4];
#pragma unroll
    for (int c = 0; c < 4; c++) {
        float v = a0[c] * w[c];
        v = fmaf(a1[c], w[c + 1], v);
        v = fmaf(a2[c], w[c + 2], v);
        v = fmaf(a3[c], w[c + 3], v);
        o[c] = v;
    }
    return make_float4(o[0], o[1], o[2], o[3]);
}

// issue_rows with the row copies spread over the CTA's warps (row i of the
// new rows from lane i / warps of warp i % warps), so that no warp issues
// them all.  A copy may complete before thread 0 has set the expected
// bytes: the barrier's phase still waits for that thread's arrival
template <int NT>
__device__ __forceinline__ void issue_rows_cta(const BDev& B, int lo, int hi,
                                               const RingMap& m, float* ring,
                                               int rb, int rs,
                                               const float* __restrict__ din,
                                               const RowInfo7* __restrict__ rinfo,
                                               RowInfo7* S, uint64_t* bar)
{
    const int n = int(B.n);
    const int a = max(lo, 0), e = max(min(hi, n), a);
    const uint32_t row_bytes = uint32_t(n) * 4u;
    const uint32_t ri_bytes = uint32_t(e - a) * uint32_t(sizeof(RowInfo7));
    if (threadIdx.x == 0) {
        fence_proxy_async();
        mbar_arrive_expect_tx(bar, uint32_t(e - a) * row_bytes + ri_bytes);
        if (e > a) {
            tma_load_1d(S + (a - lo), rinfo + B.prof_off + a, ri_bytes, bar);
        }
    }
    constexpr int NW = NT / 32;
    const int i = (threadIdx.x >> 5) + NW * (threadIdx.x & 31);
    for (int x = a + i; x < e; x += NT) {
        tma_load_1d(ring + size_t(m.slot(x, rb)) * rs + APAD,
                    din + B.dens_off + size_t(x) * n, row_bytes, bar);
    }
}

// meshes of 512 and 1024 rows: rows in parts of 256 columns, one warp each
// in stage 2; 1024-row lattices take a 5-row drift window (groups of 4
// columns may span two drift shifts) and an 11-plane table
template <int N>
struct RingShape {
    static constexpr bool HALF = N > 256;
    static constexpr int PARTS = HALF ? N / 256 : 1;
    static constexpr int WIN = N >= 1024 ? 5 : 4;
    // drift planes, the shift, 5 Fokker-Planck planes
    static constexpr int TAB_PLANES = WIN + 1 + 5;
};

// N: the mesh size of every bunch of the tile list (64, 128, 256, 512 or
// 1024; the lane mapping, strides and shuffle widths are constants)
template <int NT, int N>
__global__ void __launch_bounds__(NT, N >= 1024 ? 1 : (N > 256 ? 2 : 3))
k_bmaps0f(const BDev* __restrict__ bd, const Tile* __restrict__ tiles,
          uint32_t ntiles, const float* __restrict__ tabs,
          const float* __restrict__ dwt, const RowInfo7* __restrict__ rinfo,
          const float* __restrict__ din, float* __restrict__ dout,
          float* __restrict__ pout, int* __restrict__ status, SmemR L)
{
    constexpr bool HALF = RingShape<N>::HALF;
    constexpr int PARTS = RingShape<N>::PARTS;
    constexpr int WIN = RingShape<N>::WIN;
    constexpr int TAB_PLANES = RingShape<N>::TAB_PLANES;
    extern __shared__ float4 smem4[];
    char* base = reinterpret_cast<char*>(smem4);
    float* ring = reinterpret_cast<float*>(base + L.ring);
    RowInfo7* S = reinterpret_cast<RowInfo7*>(base + L.s);
    float* T = reinterpret_cast<float*>(base + L.tab);
    uint64_t* bar = reinterpret_cast<uint64_t*>(base + L.bar);
    // 512, 1024 rows: the parts' row sums of a tile, [2 tiles][PARTS][rb/2]
    float* part = reinterpret_cast<float*>(base + L.part);
    const int rb = int(L.rb);
    constexpr int rs = N + 2 * APAD + 16;   // astride0(N), the ring's L.rs
    const int ring_floats = rb * rs;
    const int lane = threadIdx.x & 31;

    // the ring starts zero: slots are written only in [APAD, n + APAD)
    {
        float4* r4 = reinterpret_cast<float4*>(ring);
        const float4 z = make_float4(0.f, 0.f, 0.f, 0.f);
        for (int i = threadIdx.x; i < ring_floats / 4; i += NT) {
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

    // a contiguous chunk of the tile list per CTA (chunks differ by at
    // most one tile)
    const uint32_t t_begin = uint32_t(uint64_t(blockIdx.x) * ntiles
                                      / gridDim.x);
    const uint32_t t_end = uint32_t(uint64_t(blockIdx.x + 1) * ntiles
                                    / gridDim.x);

    RingMap mc{0}, mn{0};
    int lo_c = 0, hi_c = 0, lo_n = 0, hi_n = 0;
    int front = 0;
    uint32_t tab_off = 0xffffffffu, tab_ph = 0;
    bool tab_wait = false;
    auto load_tab = [&](const BDev& Bt) {
        const uint32_t bytes = uint32_t(TAB_PLANES) * Bt.n * 4u;
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
        load_tab(B);
        lo_c = int(t.x0) - B.halo_lo;
        hi_c = int(t.x0 + t.rows) + B.halo_hi;
        mc = RingMap::at(lo_c, 0);
        front = hi_c - lo_c;
        // the first tile's density rows while the stencil kernel runs
        if (threadIdx.x < 32) {
            issue_rows(B, lo_c, hi_c, mc, ring, rb, rs, din, rinfo, S,
                       &bar[0], true, false);
        }
    }
    // this step's stencils are complete
    pdl_wait();
    if (t_begin < t_end && threadIdx.x < 32) {
        const BDev B = bd[tiles[t_begin].bunch];
        issue_rows(B, lo_c, hi_c, mc, ring, rb, rs, din, rinfo, S, &bar[0],
                   false, true);
    }
    int bad = 0;
    // the previous tile's row sums (512 and 1024 rows: one part per warp of
    // a row, added in part order and stored after a barrier)
    int prev_off = 0, prev_rows = 0;
    float prev_h03 = 0.f;
    auto store_halves = [&](int buf) {
        const float* p0 = part + buf * PARTS * (rb >> 1);
        for (int i = threadIdx.x; i < prev_rows; i += NT) {
            float v = p0[i];
#pragma unroll
            for (int q = 1; q < PARTS; q++) {
                v += p0[i + q * (rb >> 1)];
            }
            pout[prev_off + i] = prev_h03 * v;
        }
    };
    for (uint32_t k = 0, tid = t_begin; tid < t_end; tid++, k++) {
        const Tile t = tiles[tid];
        const BDev B = bd[t.bunch];
        constexpr int n = N;
        const int x0 = int(t.x0);
        const int rows = int(t.rows);
        constexpr int G1 = HALF ? N / 128 : 2;   // column groups per lane
        constexpr int seg = N / (4 * G1);    // lanes per row (stage 1)
        const int l = threadIdx.x & (seg - 1);
        const int rl = threadIdx.x / seg;    // segment
        constexpr int rp = NT / seg;         // segments
        constexpr int as = N + 2 * APAD + 16;
        const int yA = 4 * l, yB = (n >> 1) + 4 * l;

        // stage 1: both y-kicks of the new rows, in place
        {
            const int m = hi_c - lo_c;
            if (!mbar_wait_bounded(&bar[k & 1], (k >> 1) & 1, WAIT_NS)) {
                bad = 1;
                mbar_wait_bounded(&bar[k & 1], (k >> 1) & 1, WAIT_NS);
            }
            const unsigned rmask = seg == 32 ? 0xffffffffu
                : (((1u << seg) - 1u) << (lane & ~(seg - 1)));
            const float4 z = make_float4(0.f, 0.f, 0.f, 0.f);
            for (int i = rl; i < m; i += rp) {
                const int x = lo_c + i;
                float* row = ring + size_t(mc.slot(x, rb)) * rs;
                // (every row of the list has n columns: the zeros right of
                // a staged row, written when the ring was cleared, stay)
                if (unsigned(x) < unsigned(n)) {
                    const float4 q0 = reinterpret_cast<const float4*>(S + i)[0];
                    const float4 q1 = reinterpret_cast<const float4*>(S + i)[1];
                    const int s = __float_as_int(q0.x);
                    const float c[7] = {q0.y, q0.z, q0.w, q1.x, q1.y, q1.z,
                                        q1.w};
                    // lane l's groups start at 4l + g n/G1
                    constexpr int STEP = N / G1;
                    float4 o[G1];
                    // the window of every lane inside the staged row: the
                    // lowest starts at APAD + s, the highest ends 16 floats
                    // after its aligned start APAD + n - 4 + (s & ~3)
                    if (s >= -APAD && s <= APAD + 7) {
                        const float* w0 = row + APAD + (s & ~3) + yA;
                        switch (s & 3) {
                        case 0:
                            ykick7_groups<0, G1, STEP>(w0, c, o);
                            break;
                        case 1:
                            ykick7_groups<1, G1, STEP>(w0, c, o);
                            break;
                        case 2:
                            ykick7_groups<2, G1, STEP>(w0, c, o);
                            break;
                        default:
                            ykick7_groups<3, G1, STEP>(w0, c, o);
                            break;
                        }
                    } else {
#pragma unroll
                        for (int g = 0; g < G1; g++) {
                            o[g] = ykick7_checked(row, APAD + yA + g * STEP
                                                  + s, as, c);
                        }
                    }
                    __syncwarp(rmask);
#pragma unroll
                    for (int g = 0; g < G1; g++) {
                        *reinterpret_cast<float4*>(row + APAD + yA
                                                   + g * STEP) = o[g];
                    }
                } else {
#pragma unroll
                    for (int g = 0; g < G1; g++) {
                        *reinterpret_cast<float4*>(row + APAD + yA
                                                   + g * (N / G1)) = z;
                    }
                }
            }
        }
        // the in-place writes precede later bulk copies into these slots.
        // A wait that ran out (here or on the tables) ends the CTA's walk:
        // no further copies are issued, the tables' copy still in flight
        // gets one more bounded wait, and the kernel reports
        // VFPS_ERR_TIMEOUT after about one wait limit
        fence_proxy_async();
        if (__syncthreads_or(bad)) {
            bad = 1;
            if (tab_wait) {
                mbar_wait_bounded(&bar[2], tab_ph, WAIT_NS);
            }
            break;
        }
        if constexpr (HALF) {
            if (k > 0) {
                store_halves((k - 1) & 1);
            }
        }

        // stage the next tile's new rows: their slots hold no row that this
        // tile still reads (the ring holds two tiles with their halos)
        if (tid + 1 < t_end) {
            const Tile tn = tiles[tid + 1];
            const BDev Bn = bd[tn.bunch];
            const bool cont = tn.bunch == t.bunch
                              && int(tn.x0) == x0 + rows;
            hi_n = int(tn.x0 + tn.rows) + Bn.halo_hi;
            const int xr = int(tn.x0) - Bn.halo_lo;
            if (cont) {
                mn = RingMap::at(xr, mc.slot(xr, rb));
                lo_n = hi_c;
            } else {
                lo_n = xr;
                mn = RingMap::at(xr, front);
            }
            front = mn.slot(hi_n, rb);
            // (spread over the warps where a row is one warp's; the parts of
            // 512 and 1024 rows were measured faster with warp 0 alone)
            if constexpr (HALF) {
                if (threadIdx.x < 32) {
                    issue_rows(Bn, lo_n, hi_n, mn, ring, rb, rs, din, rinfo,
                               S, &bar[(k + 1) & 1]);
                }
            } else {
                issue_rows_cta<NT>(Bn, lo_n, hi_n, mn, ring, rb, rs, din,
                                   rinfo, S, &bar[(k + 1) & 1]);
            }
        }

        // this tile's drift and Fokker-Planck planes in T
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

        // stage 2: drift, Fokker-Planck, new rows, projections.  Segment rl
        // walks output rows [ra, ra + per) of the tile in steps of 4 (every
        // segment makes the same number of steps, so the shuffles see whole
        // warps; rows past the tile are computed and dropped)
        if constexpr (!HALF) {
            const float* W = T;             // drift weights [4][n], shift [n]
            const float* F = T + 5 * n;     // Fokker-Planck planes [5][n]
            const float h03 = tabs[B.tab_off + TAB_WS * n];
            const int shA = __float_as_int(W[4 * n + yA]);
            const int shB = __float_as_int(W[4 * n + yB]);
            float4 wA[4], wB[4];
#pragma unroll
            for (int j = 0; j < 4; j++) {
                wA[j] = *reinterpret_cast<const float4*>(W + j * n + yA);
                wB[j] = *reinterpret_cast<const float4*>(W + j * n + yB);
            }
            // the Fokker-Planck weights (plane o, column y); the compiler
            // keeps them in registers across the rows
            auto fw = [&](int o, int y) {
                return *reinterpret_cast<const float4*>(F + o * n + y);
            };
            const int per = (rows + rp - 1) / rp;
            const int ra = rl * per;
            const int xend = x0 + min(rows, ra + per);
            // window row offsets in the ring (floats), advanced by one slot
            // per output row (segments past the tile's rows start further
            // on: reduced modulo the ring)
            auto slot0 = [&](int x) {
                // x + off lies in [-rb, 2 rb): one step reduces it
                const int q = x + mc.off;
                return q < 0 ? q + rb : (q >= rb ? q - rb : q);
            };
            int oA = slot0(x0 + ra + shA) * rs + APAD + yA;
            int oB = slot0(x0 + ra + shB) * rs + APAD + yB;
            auto next = [&](int& o) {
                o += rs;
                o -= o >= ring_floats ? ring_floats : 0;
            };
            float4 a0, a1, a2, a3, b0, b1, b2, b3;
            a0 = *reinterpret_cast<const float4*>(ring + oA);
            b0 = *reinterpret_cast<const float4*>(ring + oB);
            next(oA);
            next(oB);
            a1 = *reinterpret_cast<const float4*>(ring + oA);
            b1 = *reinterpret_cast<const float4*>(ring + oB);
            next(oA);
            next(oB);
            a2 = *reinterpret_cast<const float4*>(ring + oA);
            b2 = *reinterpret_cast<const float4*>(ring + oB);
            next(oA);
            next(oB);
            const float f4a = F[4 * n + yA + 3];
            const int lp = (l + 1) & (seg - 1), lm = (l + seg - 1) & (seg - 1);
            const bool first = l == 0, last = l == seg - 1;
            const int hs = seg >> 1, qs = seg >> 2;
            float* obase = dout + B.dens_off;
            // one output row X from the window rows r0..r3 of each group
            // (the newest, r3, loaded here): its Simpson-weighted row sum
            // (in units of h03) is returned
            auto one = [&](int X, const float4& r0, const float4& r1,
                           const float4& r2, float4& r3, const float4& s0,
                           const float4& s1, const float4& s2, float4& s3) {
                r3 = *reinterpret_cast<const float4*>(ring + oA);
                s3 = *reinterpret_cast<const float4*>(ring + oB);
                next(oA);
                next(oB);
                const float4 dA = drift4(r0, r1, r2, r3, wA);
                const float4 dB = drift4(s0, s1, s2, s3, wB);
                // neighbour columns: A's left (lane l-1's A2, A3) and right
                // (lane l+1's A0; the last lane takes lane 0's B0), B's
                // left (lane l-1's B3; lane 0 takes the last lane's A3)
                // and right (lane l+1's B0, B1).  Beyond the mesh edges the
                // wrapped values meet zero weights (rows 0, 1, n-2, n-1 of
                // the Fokker-Planck stencil are zero)
                const float aL2 = __shfl_sync(0xffffffffu, dA.z, lm, seg);
                const float aL3 = __shfl_sync(0xffffffffu, dA.w, lm, seg);
                const float aR0 = __shfl_sync(0xffffffffu, dA.x, lp, seg);
                const float bL3 = __shfl_sync(0xffffffffu, dB.w, lm, seg);
                const float bR0 = __shfl_sync(0xffffffffu, dB.x, lp, seg);
                const float bR1 = __shfl_sync(0xffffffffu, dB.y, lp, seg);
                const float wa[7] = {aL2, aL3, dA.x, dA.y, dA.z, dA.w,
                                     last ? bR0 : aR0};
                const float wb[7] = {first ? aL3 : bL3, dB.x, dB.y, dB.z,
                                     dB.w, bR0, bR1};
                // lower half: offsets -2..1 (planes 0..3); upper half:
                // -1..2 (planes 1..4)
                float4 fA = fp4(wa, fw(0, yA), fw(1, yA), fw(2, yA),
                                fw(3, yA));
                // offset +2 of the lower half's columns: zero but in its
                // last column (n/2 - 1, the last lane's 4th), whose +2
                // neighbour n/2 + 1 is lane 0's B1 (bR1 there; elsewhere
                // bR1 meets the zero weight)
                fA.w = fmaf(f4a, bR1, fA.w);
                const float4 fB = fp4(wb, fw(1, yB), fw(2, yB), fw(3, yB),
                                      fw(4, yB));
                if (X < xend) {
                    float* o = obase + size_t(X) * n;
                    *reinterpret_cast<float4*>(o + yA) = fA;
                    *reinterpret_cast<float4*>(o + yB) = fB;
                }
                // Simpson weights along the row: even columns 2, odd 4,
                // columns 0 and n - 1 one
                float e = (fA.x + fA.z) + (fB.x + fB.z);
                float od = (fA.y + fA.w) + (fB.y + fB.w);
                if (first) {
                    e -= 0.5f * fA.x;
                }
                if (last) {
                    od -= 0.75f * fB.w;
                }
                return fmaf(4.f, od, 2.f * e);
            };
            // the row sums of 4 consecutive output rows X..X+3 (partials
            // p0..p3 of every lane): reduce-scatter over the segment, the
            // row's sum stored by one lane
            auto flush = [&](int X, float p0, float p1, float p2, float p3) {
                const bool u1 = (l & hs) != 0;
                float k0 = u1 ? p2 : p0, k1 = u1 ? p3 : p1;
                const float s0 = u1 ? p0 : p2, s1 = u1 ? p1 : p3;
                k0 += __shfl_xor_sync(0xffffffffu, s0, hs, seg);
                k1 += __shfl_xor_sync(0xffffffffu, s1, hs, seg);
                const bool u2 = (l & qs) != 0;
                float v = u2 ? k1 : k0;
                v += __shfl_xor_sync(0xffffffffu, u2 ? k0 : k1, qs, seg);
                for (int o = qs >> 1; o > 0; o >>= 1) {
                    v += __shfl_xor_sync(0xffffffffu, v, o, seg);
                }
                const int r = (u1 ? 2 : 0) + (u2 ? 1 : 0);
                if ((l & (qs - 1)) == 0 && X + r < xend) {
                    pout[B.prof_off + X + r] = h03 * v;
                }
            };
            for (int X = x0 + ra; X < x0 + ra + per; X += 4) {
                const float p0 = one(X, a0, a1, a2, a3, b0, b1, b2, b3);
                const float p1 = one(X + 1, a1, a2, a3, a0, b1, b2, b3, b0);
                const float p2 = one(X + 2, a2, a3, a0, a1, b2, b3, b0, b1);
                const float p3 = one(X + 3, a3, a0, a1, a2, b3, b0, b1, b2);
                flush(X, p0, p1, p2, p3);
            }
        } else {
            // PARTS warps per run of output rows: warp h of a group takes
            // the part of columns [256h, 256h + 256), its lane l the groups
            // at 256h + 4l (A) and 256h + 128 + 4l (B); the parts of the
            // lower half take the stencil's lower form (offsets -2..1,
            // planes 0..3), those of the upper half the upper form (-1..2,
            // planes 1..4).  The columns just left and right of its part
            // that a warp's stencils reach come from two 2-column windows
            // of the same staged rows, C (256h - 2, 256h - 1) and D
            // (256h + 256, 256h + 257), with the same drift arithmetic as
            // their own warps', so no value crosses between warps (at the
            // mesh edges C and D repeat columns 0, 1 or n - 2, n - 1, which
            // meet the zero stencils of those columns).  With two parts
            // each has one inner edge: one window, the edge lanes' mesh
            // edge neighbours wrapped around the warp.  WIN staged rows
            // per window: 4, or 5 where a group of 4 columns spans two
            // drift shifts (its table holds 5 planes from the group's
            // lowest shift, with a zero where a column's stencil ends)
            const float* W = T;                     // drift [WIN][n], shift
            const float* F = T + (WIN + 1) * n;     // Fokker-Planck [5][n]
            const float h03 = tabs[B.tab_off + TAB_WS * n];
            const int h = rl % PARTS;
            constexpr int groups = rp / PARTS;
            const int per = (rows + groups - 1) / groups;
            const int ra = (rl / PARTS) * per;
            const int xend = x0 + min(rows, ra + per);
            float* psum = part + (k & 1) * PARTS * (rb >> 1)
                          + h * (rb >> 1) - x0;
            auto slot0 = [&](int x) {
                // x + off lies in [-rb, 2 rb): one step reduces it
                const int q = x + mc.off;
                return q < 0 ? q + rb : (q >= rb ? q - rb : q);
            };
            auto next = [&](int& o) {
                o += rs;
                o -= o >= ring_floats ? ring_floats : 0;
            };
            const bool first = h == 0 && l == 0;
            const bool last = h == PARTS - 1 && l == 31;
            const bool lfirst = l == 0, llast = l == 31;
            const int lm = (l + 31) & 31, lp = (l + 1) & 31;
            float* obase = dout + B.dens_off;
            constexpr bool TWO = PARTS == 2;
            auto walk = [&](auto lc) {
                constexpr bool LOWER = decltype(lc)::value != 0;
                constexpr int P0 = LOWER ? 0 : 1;   // first Fokker-Planck plane
                const int yA = 256 * h + 4 * l;
                const int yB = yA + 128;
                const int yC = TWO ? (LOWER ? 256 * h + 256 : 256 * h - 2)
                                   : (h == 0 ? 0 : 256 * h - 2);
                const int yD = TWO ? yC
                                   : (h == PARTS - 1 ? n - 2 : 256 * h + 256);
                const int shA = __float_as_int(W[WIN * n + yA]);
                const int shB = __float_as_int(W[WIN * n + yB]);
                const int shC = __float_as_int(W[WIN * n + yC]);
                const int shD = __float_as_int(W[WIN * n + yD]);
                float4 wA[WIN], wB[WIN];
                float2 wC[WIN], wD[WIN];
#pragma unroll
                for (int j = 0; j < WIN; j++) {
                    wA[j] = *reinterpret_cast<const float4*>(W + j * n + yA);
                    wB[j] = *reinterpret_cast<const float4*>(W + j * n + yB);
                    wC[j] = *reinterpret_cast<const float2*>(W + j * n + yC);
                    wD[j] = *reinterpret_cast<const float2*>(W + j * n + yD);
                }
                auto fw = [&](int o, int y) {
                    return *reinterpret_cast<const float4*>(F + o * n + y);
                };
                int oA = slot0(x0 + ra + shA) * rs + APAD + yA;
                int oB = slot0(x0 + ra + shB) * rs + APAD + yB;
                int oC = slot0(x0 + ra + shC) * rs + APAD + yC;
                int oD = slot0(x0 + ra + shD) * rs + APAD + yD;
                // the windows: slots 0..WIN-2 loaded here, the newest row
                // by one()
                float4 a[WIN], bw[WIN];
                float2 c[WIN];
                [[maybe_unused]] float2 dd[WIN];   // not with two parts
                auto load = [&](int j) {
                    a[j] = *reinterpret_cast<const float4*>(ring + oA);
                    bw[j] = *reinterpret_cast<const float4*>(ring + oB);
                    c[j] = *reinterpret_cast<const float2*>(ring + oC);
                    next(oA);
                    next(oB);
                    next(oC);
                    if constexpr (!TWO) {
                        dd[j] = *reinterpret_cast<const float2*>(ring + oD);
                        next(oD);
                    }
                };
#pragma unroll
                for (int j = 0; j < WIN - 1; j++) {
                    load(j);
                }
                // offset +2 of the lower half: zero but in its last column
                // n/2 - 1 (the last lane's 4th of B in the last lower
                // part), whose neighbour n/2 + 1 is D's second column
                const float f4b = LOWER ? F[4 * n + yB + 3] : 0.f;
                // output row X from window slots S0 .. S0 + WIN - 1 (mod
                // WIN), the newest of them loaded here
                auto one = [&](int X, auto sc) -> float {
                    constexpr int S0 = decltype(sc)::value;
                    constexpr int S1 = (S0 + 1) % WIN, S2 = (S0 + 2) % WIN,
                                  S3 = (S0 + 3) % WIN;
                    constexpr int SN = (S0 + WIN - 1) % WIN;
                    load(SN);
                    const float4 wa4[4] = {wA[0], wA[1], wA[2], wA[3]};
                    const float4 wb4[4] = {wB[0], wB[1], wB[2], wB[3]};
                    const float2 wc2[4] = {wC[0], wC[1], wC[2], wC[3]};
                    const float2 wd2[4] = {wD[0], wD[1], wD[2], wD[3]};
                    float4 dA = drift4(a[S0], a[S1], a[S2], a[S3], wa4);
                    float4 dB = drift4(bw[S0], bw[S1], bw[S2], bw[S3], wb4);
                    float2 dC = drift2(c[S0], c[S1], c[S2], c[S3], wc2);
                    float2 dD = dC;
                    if constexpr (!TWO) {
                        dD = drift2(dd[S0], dd[S1], dd[S2], dd[S3], wd2);
                    }
                    if constexpr (WIN == 5) {
                        // the fifth tap: one more packed FMA per pair (a
                        // zero weight where a column's stencil ends at the
                        // fourth, which keeps its sum's bits)
                        const float4 r4 = a[SN], s4 = bw[SN];
                        float2 lo = __ffma2_rn(make_float2(wA[4].x, wA[4].y),
                                               make_float2(r4.x, r4.y),
                                               make_float2(dA.x, dA.y));
                        float2 hi = __ffma2_rn(make_float2(wA[4].z, wA[4].w),
                                               make_float2(r4.z, r4.w),
                                               make_float2(dA.z, dA.w));
                        dA = make_float4(lo.x, lo.y, hi.x, hi.y);
                        lo = __ffma2_rn(make_float2(wB[4].x, wB[4].y),
                                        make_float2(s4.x, s4.y),
                                        make_float2(dB.x, dB.y));
                        hi = __ffma2_rn(make_float2(wB[4].z, wB[4].w),
                                        make_float2(s4.z, s4.w),
                                        make_float2(dB.z, dB.w));
                        dB = make_float4(lo.x, lo.y, hi.x, hi.y);
                        dC = __ffma2_rn(wC[4], c[SN], dC);
                        if constexpr (!TWO) {
                            dD = __ffma2_rn(wD[4], dd[SN], dD);
                        } else {
                            dD = dC;
                        }
                    }
                    float4 fA, fB;
                    if constexpr (LOWER) {
                        // A: left lane l-1's A2, A3 (lane 0: C), right lane
                        // l+1's A0 (lane 31: lane 0's B0); B: left lane
                        // l-1's B2, B3 (lane 0: lane 31's A2, A3), right
                        // lane l+1's B0 (lane 31: D's first column)
                        const float aL2 = __shfl_sync(0xffffffffu, dA.z, lm);
                        const float aL3 = __shfl_sync(0xffffffffu, dA.w, lm);
                        const float aR0 = __shfl_sync(0xffffffffu, dA.x, lp);
                        const float bL2 = __shfl_sync(0xffffffffu, dB.z, lm);
                        const float bL3 = __shfl_sync(0xffffffffu, dB.w, lm);
                        const float bR0 = __shfl_sync(0xffffffffu, dB.x, lp);
                        // (two parts: lane 0's left neighbours are lane
                        // 31's A2, A3, meeting the zero stencils of
                        // columns 0, 1)
                        const float wa[7] = {(lfirst && !TWO) ? dC.x : aL2,
                                             (lfirst && !TWO) ? dC.y : aL3,
                                             dA.x, dA.y, dA.z, dA.w,
                                             llast ? bR0 : aR0};
                        const float wb[7] = {lfirst ? aL2 : bL2,
                                             lfirst ? aL3 : bL3, dB.x, dB.y,
                                             dB.z, dB.w, llast ? dD.x : bR0};
                        fA = fp4(wa, fw(P0, yA), fw(P0 + 1, yA),
                                 fw(P0 + 2, yA), fw(P0 + 3, yA));
                        fB = fp4(wb, fw(P0, yB), fw(P0 + 1, yB),
                                 fw(P0 + 2, yB), fw(P0 + 3, yB));
                        fB.w = fmaf(f4b, dD.y, fB.w);
                    } else {
                        // A: left lane l-1's A3 (lane 0: C's second
                        // column), right lane l+1's A0, A1 (lane 31: lane
                        // 0's B0, B1); B: left lane l-1's B3 (lane 0: lane
                        // 31's A3), right lane l+1's B0, B1 (lane 31: D)
                        const float aL3 = __shfl_sync(0xffffffffu, dA.w, lm);
                        const float aR0 = __shfl_sync(0xffffffffu, dA.x, lp);
                        const float aR1 = __shfl_sync(0xffffffffu, dA.y, lp);
                        const float bL3 = __shfl_sync(0xffffffffu, dB.w, lm);
                        const float bR0 = __shfl_sync(0xffffffffu, dB.x, lp);
                        const float bR1 = __shfl_sync(0xffffffffu, dB.y, lp);
                        const float wa[7] = {lfirst ? dC.y : aL3, dA.x, dA.y,
                                             dA.z, dA.w, llast ? bR0 : aR0,
                                             llast ? bR1 : aR1};
                        // (two parts: lane 31's right neighbours are lane
                        // 0's B0, B1, meeting the zero stencils of columns
                        // n - 2, n - 1)
                        const float wb[7] = {lfirst ? aL3 : bL3, dB.x, dB.y,
                                             dB.z, dB.w,
                                             (llast && !TWO) ? dD.x : bR0,
                                             (llast && !TWO) ? dD.y : bR1};
                        fA = fp4(wa, fw(P0, yA), fw(P0 + 1, yA),
                                 fw(P0 + 2, yA), fw(P0 + 3, yA));
                        fB = fp4(wb, fw(P0, yB), fw(P0 + 1, yB),
                                 fw(P0 + 2, yB), fw(P0 + 3, yB));
                    }
                    if (X < xend) {
                        float* o = obase + size_t(X) * n;
                        *reinterpret_cast<float4*>(o + yA) = fA;
                        *reinterpret_cast<float4*>(o + yB) = fB;
                    }
                    // Simpson weights: even columns 2, odd 4, columns 0
                    // and n - 1 one
                    float e = (fA.x + fA.z) + (fB.x + fB.z);
                    float od = (fA.y + fA.w) + (fB.y + fB.w);
                    if (first) {
                        e -= 0.5f * fA.x;
                    }
                    if (last) {
                        od -= 0.75f * fB.w;
                    }
                    return fmaf(4.f, od, 2.f * e);
                };
                // the part's sums of 4 output rows: reduce-scatter over
                // the warp, one lane stores a row's
                auto flush = [&](int X, float p0, float p1, float p2,
                                 float p3) {
                    const bool u1 = (l & 16) != 0;
                    float k0 = u1 ? p2 : p0, k1 = u1 ? p3 : p1;
                    const float s0 = u1 ? p0 : p2, s1 = u1 ? p1 : p3;
                    k0 += __shfl_xor_sync(0xffffffffu, s0, 16);
                    k1 += __shfl_xor_sync(0xffffffffu, s1, 16);
                    const bool u2 = (l & 8) != 0;
                    float v = u2 ? k1 : k0;
                    v += __shfl_xor_sync(0xffffffffu, u2 ? k0 : k1, 8);
                    v += __shfl_xor_sync(0xffffffffu, v, 4);
                    v += __shfl_xor_sync(0xffffffffu, v, 2);
                    v += __shfl_xor_sync(0xffffffffu, v, 1);
                    const int r = (u1 ? 2 : 0) + (u2 ? 1 : 0);
                    if ((l & 7) == 0 && X + r < xend) {
                        psum[X + r] = v;
                    }
                };
                for (int X = x0 + ra; X < x0 + ra + per; X += 4) {
                    const float p0 = one(X, IntC<0>{});
                    const float p1 = one(X + 1, IntC<1>{});
                    const float p2 = one(X + 2, IntC<2>{});
                    const float p3 = one(X + 3, IntC<3>{});
                    flush(X, p0, p1, p2, p3);
                    if constexpr (WIN == 5) {
                        // 5 slots, 4 rows per step: slots 4, 0, 1, 2 hold
                        // the next step's first 4 rows; move them to 0..3
                        a[3] = a[2];
                        a[2] = a[1];
                        a[1] = a[0];
                        a[0] = a[4];
                        bw[3] = bw[2];
                        bw[2] = bw[1];
                        bw[1] = bw[0];
                        bw[0] = bw[4];
                        c[3] = c[2];
                        c[2] = c[1];
                        c[1] = c[0];
                        c[0] = c[4];
                        if constexpr (!TWO) {
                            dd[3] = dd[2];
                            dd[2] = dd[1];
                            dd[1] = dd[0];
                            dd[0] = dd[4];
                        }
                    }
                }
            };
            if (h < PARTS / 2) {
                walk(IntC<1>{});
            } else {
                walk(IntC<0>{});
            }
            prev_off = int(B.prof_off) + x0;
            prev_rows = rows;
            prev_h03 = h03;
        }
        mc = mn;
        lo_c = lo_n;
        hi_c = hi_n;
    }
    if constexpr (HALF) {
        // the last tile's row sums (after a wait that ran out, none)
        bad = __syncthreads_or(bad);
        if (!bad && prev_rows > 0) {
            store_halves((t_end - t_begin - 1) & 1);
        }
    }
    if (bad && threadIdx.x == 0) {
        atomicCAS(status, 0, VFPS_ERR_TIMEOUT);
    }
    // the next step's k_bwake may launch once every CTA is here
    pdl_trigger();
}

}  // namespace
