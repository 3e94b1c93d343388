// Batched solver step: many independent single-bunch simulations advanced
// by ONE fused kernel per step (no reference counterpart; each bunch
// follows the reference solver step, src/main.cpp:948-1053).
//
// Work unit = a tile of TX consecutive mesh rows (x) of one bunch.  A CTA
//   1. reads the previous step's profile of its bunch (n floats) and
//      evaluates the wake potential of the rows it needs as the Toeplitz
//      sum  wake[x] = s sum_m P[m] w[(x-m) mod nmax]  (w built once per
//      impedance in FP64), so no separate wake launch and no grid-wide
//      synchronisation is needed;
//   2. stages rows [x0-halo, x0+TX+halo) of the density in shared memory
//      (the halo covers the reach of the 2-D stage: drift x-kick or
//      rotation; it is computed on the host from the actual stencils);
//   3. chain 0: wake y-kick, RF y-kick (all staged rows), drift x-kick,
//      Fokker-Planck (tile rows); chain 1: rotation, wake y-kick,
//      Fokker-Planck;
//   4. writes its rows and their x projections (the next step's profile).
// Densities and profiles are double-buffered; a step counter in device
// memory drives the renormalisation cadence.  Steps are captured in CUDA
// graphs.  Out-of-mesh taps are dropped as in the reference; a tap that
// would leave the staged rows (it cannot, by construction of the halo)
// is dropped and flagged in the context's device status word.
#include <algorithm>
#include <cfloat>
#include <cstdlib>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <map>
#include <mutex>

#include "vfps_internal.cuh"

namespace {

using vfps::DevBuf;

constexpr int THREADS = 256;

struct BDev {
    uint32_t n, it, chain, flags;  // flags: 1 wake, 2 fp, 4 clamp
    uint32_t dens_off, prof_off, tab_off, fp_off;
    uint32_t wt_off, nmax, ip, rot_h;
    int32_t renorm, halo_lo, halo_hi, pad;
    float wakescale, fillset, dq, dp;
    float zbq, zbp, cs, sn;
};

struct Tile {
    uint32_t bunch, x0, rows, pad;
};

enum { F_WAKE = 1, F_FP = 2, F_CLAMP = 4 };
enum { TAB_WS = 0, TAB_Q = 1, TAB_P = 2, TAB_RF = 3, TAB_DRIFT = 4,
       TAB_COUNT = 5 };

// ----------------------------------------------------------- device
using namespace vfps::dev;

struct RowStencil {
    int shift0;   // tap j reads cell i + shift0 + j
    float w[4];   // 0 for dropped taps
};

__device__ __forceinline__ RowStencil make_stencil(float offset, uint32_t n,
                                                   int it)
{
    const KickStencil s = kick_stencil(offset, n, it);
    RowStencil r;
    r.shift0 = s.shift[0];
#pragma unroll
    for (int j = 0; j < 4; j++) {
        r.w[j] = s.valid[j] ? s.w[j] : 0.f;
    }
    return r;
}

// byte offsets of the dynamic shared memory regions (16-byte aligned)
struct SmemLayout {
    size_t p, w, s, a, b, total;
};

__host__ __device__ inline size_t align16(size_t v) { return (v + 15) & ~size_t(15); }

__host__ __device__ inline SmemLayout smem_layout(int n, int nr)
{
    SmemLayout L;
    L.p = 0;
    L.w = align16(L.p + sizeof(float) * n);
    L.s = align16(L.w + sizeof(float) * nr);
    L.a = align16(L.s + sizeof(RowStencil) * nr);
    L.b = align16(L.a + sizeof(float) * size_t(nr) * n);
    L.total = align16(L.b + sizeof(float) * size_t(nr) * n);
    return L;
}

// y-kick of one staged row: out[y] = sum_j w_j in[y + shift0 + j]
__device__ __forceinline__ void ykick_rows(const float* __restrict__ in,
                                           float* __restrict__ out,
                                           const RowStencil* st, int nrows,
                                           int n)
{
    const int cols = n < THREADS ? n : THREADS;
    const int lanes = THREADS / cols;
    const int col = threadIdx.x % cols;
    const int rl = threadIdx.x / cols;
    if (rl >= lanes) {
        return;
    }
    for (int r = rl; r < nrows; r += lanes) {
        const RowStencil s = st[r];
        const float* src = in + size_t(r) * n;
        float* dst = out + size_t(r) * n;
        for (int y = col; y < n; y += cols) {
            float v = 0.f;
#pragma unroll
            for (int j = 0; j < 4; j++) {
                const int ys = y + s.shift0 + j;
                if (unsigned(ys) < unsigned(n)) {
                    v = fmaf(src[ys], s.w[j], v);
                }
            }
            dst[y] = v;
        }
    }
}

__global__ void __launch_bounds__(THREADS)
k_bstep(const BDev* __restrict__ bd, const Tile* __restrict__ tiles,
        const float* __restrict__ tabs, const float* __restrict__ fpw,
        const int* __restrict__ fpo, const float* __restrict__ wt,
        const float* __restrict__ din, float* __restrict__ dout,
        const float* __restrict__ pin, float* __restrict__ pout,
        float* __restrict__ wake_out, double* __restrict__ filling,
        unsigned* __restrict__ counters, int* __restrict__ status,
        uint32_t ntiles)
{
    extern __shared__ float4 smem4[];
    float* smem = reinterpret_cast<float*>(smem4);
    __shared__ double red[32];
    __shared__ float s_factor;
    __shared__ int s_bad;

    const Tile t = tiles[blockIdx.x];
    const BDev B = bd[t.bunch];
    const int n = int(B.n);
    const int x0 = int(t.x0);
    const int rows = int(t.rows);
    const unsigned step = *((volatile unsigned*)counters);
    const float* ws = tabs + B.tab_off + TAB_WS * n;
    const bool chain0 = B.chain == 0;
    // rows staged from the input
    const int r0 = max(0, x0 - B.halo_lo);
    const int r1 = min(n, x0 + rows + B.halo_hi);
    const int nr = r1 - r0;
    // wake rows: staged rows (chain 0) or tile rows (chain 1)
    const int w0 = chain0 ? r0 : x0;
    const int w1 = chain0 ? r1 : x0 + rows;

    // shared layout (see smem_layout)
    const SmemLayout L = smem_layout(n, nr);
    char* base = reinterpret_cast<char*>(smem);
    float* P = reinterpret_cast<float*>(base + L.p);    // [n] profile
    float* W = reinterpret_cast<float*>(base + L.w);    // wake rows
    RowStencil* S = reinterpret_cast<RowStencil*>(base + L.s);
    float* bufA = reinterpret_cast<float*>(base + L.a);
    float* bufB = reinterpret_cast<float*>(base + L.b);

    if (threadIdx.x == 0) {
        s_bad = 0;
    }
    for (int i = threadIdx.x; i < n; i += THREADS) {
        P[i] = pin[B.prof_off + i];
    }
    __syncthreads();

    // charge integral (FP64) for the renormalisation and the report
    const bool renorm_now = B.renorm > 0 && (step % unsigned(B.renorm)) == 0;
    if (renorm_now || x0 == 0) {
        double acc = 0;
        for (int i = threadIdx.x; i < n; i += THREADS) {
            acc += double(P[i]) * double(ws[i]);
        }
        acc = block_sum(acc, red);
        if (threadIdx.x == 0) {
            float f = 1.f;
            if (renorm_now) {
                f = B.fillset > 0 ? static_cast<float>(double(B.fillset) / acc)
                                  : 0.f;
            }
            s_factor = f;
            if (x0 == 0) {
                filling[t.bunch] = acc;
            }
            if (B.fillset > 0 && !(acc > 0)) {
                atomicCAS(status, 0, VFPS_ERR_NUMERIC);
            }
        }
    } else if (threadIdx.x == 0) {
        s_factor = 1.f;
    }

    // wake potential of rows w0..w1: one warp per row
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (B.flags & F_WAKE) {
        const float* w = wt + B.wt_off;
        const int nmax = int(B.nmax);
        for (int x = w0 + warp; x < w1; x += THREADS / 32) {
            float acc = 0.f;
            for (int m = lane; m < n; m += 32) {
                int d = x - m;
                d += (d < 0) ? nmax : 0;
                acc = fmaf(P[m], __ldg(w + d), acc);
            }
            acc = warp_sum_f(acc);
            if (lane == 0) {
                const float v = __fmul_rn(B.wakescale, acc);
                W[x - w0] = v;
                if (x >= x0 && x < x0 + rows) {
                    wake_out[B.prof_off + x] = v;
                }
            }
        }
    }
    __syncthreads();

    // stage the input rows
    const float factor = s_factor;
    {
        const float4* src = reinterpret_cast<const float4*>(
            din + B.dens_off + size_t(r0) * n);
        float4* dst = reinterpret_cast<float4*>(bufA);
        const int cnt = nr * n / 4;
        for (int i = threadIdx.x; i < cnt; i += THREADS) {
            float4 v = __ldg(src + i);
            v.x *= factor;
            v.y *= factor;
            v.z *= factor;
            v.w *= factor;
            dst[i] = v;
        }
    }
    __syncthreads();

    const int it = int(B.it);
    float* cur = bufA;    // holds the state after the last stage
    float* other = bufB;
    int cur_r0 = r0;      // first row held in cur
    int cur_nr = nr;

    if (chain0) {
        // wake y-kick t1 -> t2 on staged rows
        if (B.flags & F_WAKE) {
            for (int r = threadIdx.x; r < nr; r += THREADS) {
                S[r] = make_stencil(W[r0 + r - w0], B.n, it);
            }
            __syncthreads();
            ykick_rows(cur, other, S, nr, n);
            __syncthreads();
            float* tmp = cur;
            cur = other;
            other = tmp;
        }
        // RF y-kick t2 -> t1
        {
            const float* rf = tabs + B.tab_off + TAB_RF * n;
            for (int r = threadIdx.x; r < nr; r += THREADS) {
                S[r] = make_stencil(rf[r0 + r], B.n, it);
            }
            __syncthreads();
            ykick_rows(cur, other, S, nr, n);
            __syncthreads();
            float* tmp = cur;
            cur = other;
            other = tmp;
        }
        // drift x-kick t1 -> t3 on the tile rows (column stencils)
        {
            const float* dr = tabs + B.tab_off + TAB_DRIFT * n;
            const int cols = n < THREADS ? n : THREADS;
            const int lanes = THREADS / cols;
            const int col = threadIdx.x % cols;
            const int rl = threadIdx.x / cols;
            if (rl < lanes) {
                for (int y = col; y < n; y += cols) {
                    const RowStencil s = make_stencil(dr[y], B.n, it);
                    for (int r = rl; r < rows; r += lanes) {
                        const int x = x0 + r;
                        float v = 0.f;
#pragma unroll
                        for (int j = 0; j < 4; j++) {
                            const int xs = x + s.shift0 + j;
                            if (unsigned(xs) < unsigned(n) && s.w[j] != 0.f) {
                                if (xs >= r0 && xs < r1) {
                                    v = fmaf(cur[size_t(xs - r0) * n + y],
                                             s.w[j], v);
                                } else {
                                    s_bad = 1;
                                }
                            }
                        }
                        other[size_t(r) * n + y] = v;
                    }
                }
            }
            __syncthreads();
            float* tmp = cur;
            cur = other;
            other = tmp;
            cur_r0 = x0;
            cur_nr = rows;
        }
    } else {
        // rotation t1 -> t2 on the tile rows
        const float* qv = tabs + B.tab_off + TAB_Q * n;
        const float* pv = tabs + B.tab_off + TAB_P * n;
        const int h = int(B.rot_h);
        const bool clamp = B.flags & F_CLAMP;
        for (int i = threadIdx.x; i < rows * n; i += THREADS) {
            const int r = i / n, y0 = i % n;
            const int xo = x0 + r;
            const float q = qv[xo], p = pv[y0];
            const float x1r = fadd(fdiv(fsub(fmul(B.cs, q), fmul(B.sn, p)),
                                        B.dq), B.zbq);
            const float y1r = fadd(fdiv(fadd(fmul(B.sn, q), fmul(B.cs, p)),
                                        B.dp), B.zbp);
            int x1 = 0, y1 = 0;
            float xf, yf;
            const bool ok = base_index(x1r, B.n, &x1, &xf)
                            & base_index(y1r, B.n, &y1, &yf);
            float v = 0.f;
            if (ok) {
                float icq[4], icp[4];
                coefficients(icq, xf, it);
                coefficients(icp, yf, it);
                for (int i1 = 0; i1 < it; i1++) {
                    const int i0 = x1 + i1 - h;
                    if (unsigned(i0) >= unsigned(n)) {
                        continue;
                    }
                    if (i0 < r0 || i0 >= r1) {
                        s_bad = 1;
                        continue;
                    }
                    const float* srow = cur + size_t(i0 - r0) * n;
                    float rv = 0.f;
                    for (int j1 = 0; j1 < it; j1++) {
                        const int j0 = y1 + j1 - h;
                        if (unsigned(j0) < unsigned(n)) {
                            rv = fmaf(srow[j0], icp[j1], rv);
                        }
                    }
                    v = fmaf(rv, icq[i1], v);
                }
            }
            if (clamp) {
                float hi = FLT_MIN, lo = FLT_MAX;
                for (int i1 = 1; i1 <= 2; i1++) {
                    for (int j1 = 1; j1 <= 2; j1++) {
                        const int i0 = x1 + i1 - h, j0 = y1 + j1 - h;
                        const bool inm = ok && unsigned(i0) < unsigned(n)
                                         && unsigned(j0) < unsigned(n)
                                         && i0 >= r0 && i0 < r1;
                        // taps off the mesh read cell (0,0) of the bunch
                        const float sv = inm ? cur[size_t(i0 - r0) * n + j0]
                                             : din[B.dens_off] * factor;
                        hi = (hi < sv) ? sv : hi;
                        lo = (sv < lo) ? sv : lo;
                    }
                }
                const float tmin = (v < hi) ? v : hi;
                v = (tmin < lo) ? lo : tmin;
            }
            other[size_t(r) * n + y0] = v;
        }
        __syncthreads();
        float* tmp = cur;
        cur = other;
        other = tmp;
        cur_r0 = x0;
        cur_nr = rows;
        // wake y-kick t2 -> t3 on the tile rows
        if (B.flags & F_WAKE) {
            for (int r = threadIdx.x; r < rows; r += THREADS) {
                S[r] = make_stencil(W[r], B.n, it);
            }
            __syncthreads();
            ykick_rows(cur, other, S, rows, n);
            __syncthreads();
            tmp = cur;
            cur = other;
            other = tmp;
        }
    }
    (void)cur_r0;
    (void)cur_nr;

    // Fokker-Planck t3 -> t1 (tile rows), per-y stencils
    if (B.flags & F_FP) {
        const int ip = int(B.ip);
        const int cols = n < THREADS ? n : THREADS;
        const int lanes = THREADS / cols;
        const int col = threadIdx.x % cols;
        const int rl = threadIdx.x / cols;
        if (rl < lanes) {
            for (int y = col; y < n; y += cols) {
                float wv[4];
                int ov[4];
#pragma unroll
                for (int j = 0; j < 4; j++) {
                    wv[j] = j < ip ? fpw[B.fp_off + y * 4 + j] : 0.f;
                    ov[j] = j < ip ? fpo[B.fp_off + y * 4 + j] : 0;
                }
                for (int r = rl; r < rows; r += lanes) {
                    const float* src = cur + size_t(r) * n;
                    float v = 0.f;
#pragma unroll
                    for (int j = 0; j < 4; j++) {
                        v = fmaf(src[y + ov[j]], wv[j], v);
                    }
                    other[size_t(r) * n + y] = v;
                }
            }
        }
        __syncthreads();
        float* tmp = cur;
        cur = other;
        other = tmp;
    }

    // write rows and their projections: one warp per row
    for (int r = warp; r < rows; r += THREADS / 32) {
        const float* src = cur + size_t(r) * n;
        float* dst = dout + B.dens_off + size_t(x0 + r) * n;
        float acc = 0.f;
        for (int y = lane * 4; y < n; y += 128) {
            const float4 v = *reinterpret_cast<const float4*>(src + y);
            *reinterpret_cast<float4*>(dst + y) = v;
            acc = fmaf(v.x, ws[y], acc);
            acc = fmaf(v.y, ws[y + 1], acc);
            acc = fmaf(v.z, ws[y + 2], acc);
            acc = fmaf(v.w, ws[y + 3], acc);
        }
        acc = warp_sum_f(acc);
        if (lane == 0) {
            pout[B.prof_off + x0 + r] = acc;
        }
    }

    // step counter: the last CTA to finish advances it
    __syncthreads();
    if (threadIdx.x == 0) {
        if (s_bad) {
            atomicCAS(status, 0, VFPS_ERR_INVALID_ARGUMENT);
        }
        __threadfence();
        const unsigned ticket = atomicAdd(counters + 1, 1u);
        if (ticket == ntiles - 1) {
            counters[1] = 0;
            counters[0] = step + 1;
            __threadfence();
        }
    }
}

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
                         const float* __restrict__ g, float* __restrict__ dens)
{
    const BDev B = bd[blockIdx.y];
    const size_t cells = size_t(B.n) * B.n;
    const float* gx = g + 2 * size_t(B.tab_off) / TAB_COUNT;
    const float* gy = gx + B.n;
    for (size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x; i < cells;
         i += size_t(gridDim.x) * blockDim.x) {
        dens[B.dens_off + i] = __fmul_rn(gx[i / B.n], gy[i % B.n]);
    }
}

}  // namespace

// ================================================================== host
struct vfps_batch {
    vfps_ctx* ctx = nullptr;
    int device = 0;
    uint32_t nb = 0;
    std::vector<vfps_bunch_desc> desc;
    std::vector<BDev> hb;
    std::vector<Tile> htiles;
    size_t cells = 0, rows = 0;
    DevBuf<BDev> bd;
    DevBuf<Tile> tiles;
    DevBuf<float> tabs, fpw, wt;
    DevBuf<int> fpo;
    DevBuf<uint32_t> row_bunch;
    DevBuf<float> dens[2], prof[2];
    DevBuf<float> wake;
    DevBuf<double> filling;
    DevBuf<unsigned> counters;
    int cur = 0;               // buffer holding the current state
    size_t smem = 0;
    int tile_rows = 0;
    cudaGraphExec_t graph[2] = {nullptr, nullptr};  // 1 step from buffer i
    cudaGraphExec_t graph8[2] = {nullptr, nullptr}; // 8 steps from buffer i
};

namespace {

std::vector<float> simpson(uint32_t n, float delta)
{
    std::vector<float> ws(n);
    const float h03 = delta / 3.f;
    float dc = 1;
    ws[0] = h03;
    for (uint32_t x = 1; x + 1 < n; x++) {
        ws[x] = h03 * (3.f + dc);
        dc = -dc;
    }
    ws[n - 1] = h03;
    return ws;
}

// KickMap::updateSM for one offset: first valid tap shift and tap reach
void stencil_reach(float offset, uint32_t n, int it, int* lo, int* hi)
{
    const float poffs = static_cast<float>(n / 2) + offset;
    const float t = std::trunc(poffs);
    if (!(t >= 0) || !(t < static_cast<float>(n))) {
        return;
    }
    const int jd = static_cast<int>(t);
    const int h = (it - 1) / 2;
    for (int j = 0; j < it; j++) {
        const int j0 = jd + j - h;
        if (j0 >= 0 && j0 < int(n)) {
            const int s = j0 - int(n / 2);
            *lo = std::min(*lo, s);
            *hi = std::max(*hi, s);
        }
    }
}

void launch_step(vfps_batch* b, int from)
{
    const int to = 1 - from;
    k_bstep<<<static_cast<unsigned>(b->htiles.size()), THREADS, b->smem,
              b->ctx->stream>>>(
        b->bd.p, b->tiles.p, b->tabs.p, b->fpw.p, b->fpo.p, b->wt.p,
        b->dens[from].p, b->dens[to].p, b->prof[from].p, b->prof[to].p,
        b->wake.p, b->filling.p, b->counters.p, b->ctx->d_status,
        static_cast<uint32_t>(b->htiles.size()));
    VFPS_LAUNCHED();
}

void build_tiles(vfps_batch* b, int tile_cells)
{
    b->htiles.clear();
    size_t smem = 0;
    int max_rows = 0;
    for (uint32_t i = 0; i < b->nb; i++) {
        const BDev& B = b->hb[i];
        const int n = int(B.n);
        int tx = std::max(1, tile_cells / n);
        tx = std::min(tx, n);
        max_rows = std::max(max_rows, tx);
        for (int x0 = 0; x0 < n; x0 += tx) {
            const int rows = std::min(tx, n - x0);
            b->htiles.push_back({i, uint32_t(x0), uint32_t(rows), 0});
        }
        const int nr = std::min(n, tx + B.halo_lo + B.halo_hi);
        smem = std::max(smem, smem_layout(n, nr).total);
    }
    b->smem = smem;
    b->tile_rows = max_rows;
}

void destroy_graphs(vfps_batch* b)
{
    for (int i = 0; i < 2; i++) {
        if (b->graph[i]) {
            cudaGraphExecDestroy(b->graph[i]);
            b->graph[i] = nullptr;
        }
        if (b->graph8[i]) {
            cudaGraphExecDestroy(b->graph8[i]);
            b->graph8[i] = nullptr;
        }
    }
}

cudaGraphExec_t capture(vfps_batch* b, int from, int steps)
{
    cudaGraph_t g;
    VFPS_CUDA(cudaStreamBeginCapture(b->ctx->stream,
                                     cudaStreamCaptureModeThreadLocal));
    int f = from;
    for (int s = 0; s < steps; s++) {
        launch_step(b, f);
        f = 1 - f;
    }
    VFPS_CUDA(cudaStreamEndCapture(b->ctx->stream, &g));
    cudaGraphExec_t ex;
    VFPS_CUDA(cudaGraphInstantiate(&ex, g, 0));
    VFPS_CUDA(cudaGraphDestroy(g));
    return ex;
}

void setup_kernel(vfps_batch* b)
{
    VFPS_REQUIRE(b->smem <= 227 * 1024,
                 "tile of the largest mesh does not fit in shared memory");
    VFPS_CUDA(cudaFuncSetAttribute(k_bstep,
                                   cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   static_cast<int>(b->smem)));
    b->tiles.alloc(b->htiles.size());
    VFPS_CUDA(cudaMemcpy(b->tiles.p, b->htiles.data(),
                         b->htiles.size() * sizeof(Tile),
                         cudaMemcpyHostToDevice));
    destroy_graphs(b);
    for (int i = 0; i < 2; i++) {
        b->graph[i] = capture(b, i, 1);
        b->graph8[i] = capture(b, i, 8);
    }
}

// Autotuner: time candidate tile sizes on the real batch (state restored
// afterwards) and keep the fastest; results are cached per mesh mix.
std::mutex g_tune_mu;
std::map<std::string, int> g_tune_cache;

int autotune(vfps_batch* b)
{
    std::string key;
    for (auto& B : b->hb) {
        key += std::to_string(B.n) + "/" + std::to_string(B.chain) + "/"
               + std::to_string(B.halo_lo + B.halo_hi) + ",";
    }
    {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        auto it = g_tune_cache.find(key);
        if (it != g_tune_cache.end()) {
            return it->second;
        }
    }
    // save state
    DevBuf<float> sd(b->dens[b->cur].n), sp(b->prof[b->cur].n);
    cudaStream_t st = b->ctx->stream;
    VFPS_CUDA(cudaMemcpyAsync(sd.p, b->dens[b->cur].p, sd.bytes(),
                              cudaMemcpyDeviceToDevice, st));
    VFPS_CUDA(cudaMemcpyAsync(sp.p, b->prof[b->cur].p, sp.bytes(),
                              cudaMemcpyDeviceToDevice, st));
    unsigned saved_ctr[2];
    VFPS_CUDA(cudaMemcpyAsync(saved_ctr, b->counters.p, sizeof(saved_ctr),
                              cudaMemcpyDeviceToHost, st));
    VFPS_CUDA(cudaStreamSynchronize(st));
    const int cands[] = {2048, 4096, 8192, 16384};
    int best = 4096;
    float best_ms = 1e30f;
    cudaEvent_t e0, e1;
    VFPS_CUDA(cudaEventCreate(&e0));
    VFPS_CUDA(cudaEventCreate(&e1));
    for (int c : cands) {
        build_tiles(b, c);
        if (b->smem > 227 * 1024) {
            continue;
        }
        VFPS_CUDA(cudaFuncSetAttribute(
            k_bstep, cudaFuncAttributeMaxDynamicSharedMemorySize,
            static_cast<int>(b->smem)));
        b->tiles.alloc(b->htiles.size());
        VFPS_CUDA(cudaMemcpy(b->tiles.p, b->htiles.data(),
                             b->htiles.size() * sizeof(Tile),
                             cudaMemcpyHostToDevice));
        int from = b->cur;
        for (int w = 0; w < 3; w++) {
            launch_step(b, from);
            from = 1 - from;
        }
        VFPS_CUDA(cudaEventRecord(e0, st));
        for (int s = 0; s < 10; s++) {
            launch_step(b, from);
            from = 1 - from;
        }
        VFPS_CUDA(cudaEventRecord(e1, st));
        VFPS_CUDA(cudaEventSynchronize(e1));
        float ms = 0;
        VFPS_CUDA(cudaEventElapsedTime(&ms, e0, e1));
        if (ms < best_ms) {
            best_ms = ms;
            best = c;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    VFPS_CUDA(cudaMemcpyAsync(b->dens[b->cur].p, sd.p, sd.bytes(),
                              cudaMemcpyDeviceToDevice, st));
    VFPS_CUDA(cudaMemcpyAsync(b->prof[b->cur].p, sp.p, sp.bytes(),
                              cudaMemcpyDeviceToDevice, st));
    VFPS_CUDA(cudaMemcpyAsync(b->counters.p, saved_ctr, sizeof(saved_ctr),
                              cudaMemcpyHostToDevice, st));
    VFPS_CUDA(cudaStreamSynchronize(st));
    {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        g_tune_cache[key] = best;
    }
    return best;
}

thread_local std::string g_batch_error;

template <typename F>
int bguard(vfps_ctx* ctx, F&& f)
{
    try {
        if (ctx) {
            VFPS_CUDA(cudaSetDevice(ctx->device));
        }
        f();
        return VFPS_OK;
    } catch (const vfps::Error& e) {
        if (ctx) {
            ctx->last_error = e.what();
        }
        return e.code;
    } catch (const std::bad_alloc&) {
        if (ctx) {
            ctx->last_error = "host allocation failed";
        }
        return VFPS_ERR_OUT_OF_MEMORY;
    } catch (const std::exception& e) {
        if (ctx) {
            ctx->last_error = e.what();
        }
        return VFPS_ERR_INVALID_ARGUMENT;
    }
}

void project_all(vfps_batch* b, int buf)
{
    const unsigned total = static_cast<unsigned>(b->rows);
    k_bproject<<<(total * 32 + 255) / 256, 256, 0, b->ctx->stream>>>(
        b->bd.p, b->row_bunch.p, b->tabs.p, b->dens[buf].p, b->prof[buf].p,
        total);
    VFPS_LAUNCHED();
}

void integrate_all(vfps_batch* b, int buf, int normalize)
{
    k_bintegrate<<<b->nb, 256, 0, b->ctx->stream>>>(
        b->bd.p, b->tabs.p, b->prof[buf].p, b->dens[buf].p, b->filling.p,
        normalize);
    VFPS_LAUNCHED();
}

// state after loading densities: the PhaseSpace(data) constructor
// (project, integrate) followed by the solver's initial renormalisation
// (src/main.cpp:527-532) for bunches with renormalize >= 0.
void prepare_state(vfps_batch* b, bool normalize_initial)
{
    project_all(b, b->cur);
    integrate_all(b, b->cur, 0);
    if (normalize_initial) {
        project_all(b, b->cur);
        integrate_all(b, b->cur, 1);
    }
}

}  // namespace

extern "C" int vfps_batch_create(vfps_ctx* ctx, uint32_t nb,
                                 const vfps_bunch_desc* desc,
                                 const vfps_impedance* const* imps,
                                 uint32_t nimp, const float* data,
                                 vfps_batch** out)
{
    if (!ctx || !desc || !out) {
        return VFPS_ERR_INVALID_ARGUMENT;
    }
    *out = nullptr;
    return bguard(ctx, [&] {
        VFPS_REQUIRE(nb >= 1, "a batch needs at least one bunch");
        auto b = std::make_unique<vfps_batch>();
        b->ctx = ctx;
        b->device = ctx->device;
        b->nb = nb;
        b->desc.assign(desc, desc + nb);
        b->hb.resize(nb);
        std::vector<float> tabs, fpw, wt, gauss;
        std::vector<int> fpo;
        std::vector<uint32_t> row_bunch;
        std::vector<uint32_t> wt_off(nimp, 0xffffffffu);
        size_t dens_off = 0, prof_off = 0;
        bool any_renorm = false;
        for (uint32_t i = 0; i < nb; i++) {
            const vfps_bunch_desc& d = desc[i];
            const uint32_t n = d.n;
            VFPS_REQUIRE(n >= 8 && n % 8 == 0 && n <= 4096,
                         "batched meshes need n a multiple of 8, 8..4096");
            VFPS_REQUIRE(d.it >= 2 && d.it <= 4,
                         "batched interpolation points must be 2..4");
            VFPS_REQUIRE(d.chain == 0 || d.chain == 1, "chain must be 0 or 1");
            VFPS_REQUIRE(!d.clamp || (d.chain == 1 && d.it == 4),
                         "clamping needs the cubic rotation chain");
            VFPS_REQUIRE(d.e1 <= 0 || d.derivation == 3 || d.derivation == 4,
                         "derivation must be 3 or 4");
            BDev& B = b->hb[i];
            std::memset(&B, 0, sizeof(B));
            B.n = n;
            B.it = d.it;
            B.chain = d.chain;
            B.dens_off = static_cast<uint32_t>(dens_off);
            B.prof_off = static_cast<uint32_t>(prof_off);
            B.tab_off = static_cast<uint32_t>(tabs.size());
            B.renorm = d.renormalize;
            B.fillset = 1.f;
            any_renorm = any_renorm || d.renormalize >= 0;
            const auto ax = vfps::make_axis(n, float(d.axes[0]),
                                            float(d.axes[1]), float(d.axes[2]));
            const auto ay = vfps::make_axis(n, float(d.axes[3]),
                                            float(d.axes[4]), float(d.axes[5]));
            B.dq = ax.delta;
            B.dp = ay.delta;
            B.zbq = ax.zerobin;
            B.zbp = ay.zerobin;
            // tables: ws, q, p, rf offsets, drift offsets
            const auto ws = simpson(n, ax.delta);
            std::vector<float> rf(n, 0.f), drift(n, 0.f);
            if (d.chain == 0) {
                const float bl2phase = static_cast<float>(d.rf_bl2phase);
                if (d.rf_linear) {
                    const float ang = static_cast<float>(d.rf_angle);
                    for (uint32_t x = 0; x < n; x++) {
                        rf[x] = std::tan(ang) * (ax.zerobin - float(x));
                        rf[x] += std::tan(ang) * 0.f / bl2phase / ax.delta;
                    }
                } else {
                    const float rp = float(d.rf_revpart), v = float(d.rf_vrf),
                                v0 = float(d.rf_v0), ph = float(d.rf_phase);
                    for (uint32_t x = 0; x < n; x++) {
                        rf[x] = rp * (-1.f * v * std::sin(ax.v[x] * bl2phase + ph)
                                      + v0)
                                / ay.delta / ay.scale;
                    }
                }
                const float e0 = float(d.e0);
                for (uint32_t y = 0; y < n; y++) {
                    float o = 0;
                    for (int s = 0; s < d.nslip && s < 3; s++) {
                        o += float(d.slip[s]) * ay.v[y]
                             * std::pow(ay.v[y] * ay.scale / e0, float(s));
                    }
                    drift[y] = o / ax.delta;
                }
                int lo = 0, hi = 0;
                for (uint32_t y = 0; y < n; y++) {
                    stencil_reach(drift[y], n, d.it, &lo, &hi);
                }
                B.halo_lo = std::max(0, -lo);
                B.halo_hi = std::max(0, hi);
            } else {
                const float ang = static_cast<float>(d.angle);
                B.cs = std::cos(-ang);
                B.sn = std::sin(-ang);
                const int h = (d.it - 1) / 2;
                B.rot_h = h;
                int lo = 0, hi = 0;
                for (uint32_t x0 = 0; x0 < n; x0++) {
                    for (uint32_t y0 = 0; y0 < n; y0++) {
                        // same float operations as the kernel
                        volatile float a = B.cs * ax.v[x0];
                        volatile float c = B.sn * ay.v[y0];
                        volatile float e = a - c;
                        volatile float f = e / ax.delta;
                        const float x1r = f + ax.zerobin;
                        const float t = std::trunc(x1r);
                        if (!(t >= 0) || !(t < float(n))) {
                            continue;
                        }
                        const int x1 = int(t);
                        for (int i1 = 0; i1 < d.it; i1++) {
                            const int i0 = x1 + i1 - h;
                            if (i0 >= 0 && i0 < int(n)) {
                                lo = std::min(lo, i0 - int(x0));
                                hi = std::max(hi, i0 - int(x0));
                            }
                        }
                    }
                }
                B.halo_lo = std::max(0, -lo) + 1;
                B.halo_hi = std::max(0, hi) + 1;
            }
            tabs.insert(tabs.end(), ws.begin(), ws.end());
            tabs.insert(tabs.end(), ax.v.begin(), ax.v.end());
            tabs.insert(tabs.end(), ay.v.begin(), ay.v.end());
            tabs.insert(tabs.end(), rf.begin(), rf.end());
            tabs.insert(tabs.end(), drift.begin(), drift.end());
            // Fokker-Planck stencils via a throw-away plain map on the host
            // formulas (src/SM/FokkerPlanckMap.cpp:11-118)
            B.fp_off = static_cast<uint32_t>(fpw.size());
            std::vector<float> w4(size_t(n) * 4, 0.f);
            std::vector<int> o4(size_t(n) * 4, 0);
            if (d.e1 > 0) {
                B.flags |= F_FP;
                B.ip = d.derivation;
                const float e1 = float(d.e1);
                const float e1_2d = e1 / (2.f * ay.delta);
                const float e1_6d = e1 / (6.f * ay.delta);
                const float e1_d2 = e1 / (ay.delta * ay.delta);
                const bool damp = d.fptype != 0 && d.fptype != 2;
                const bool diff = d.fptype != 0 && d.fptype != 1;
                std::vector<uint32_t> idx(size_t(n) * 4, 0);
                if (d.derivation == 3) {
                    for (uint32_t j = 1; j + 1 < n; j++) {
                        float W[3] = {0, 1, 0};
                        if (damp) {
                            const float pos = ay.v[j];
                            W[0] += -e1_2d * pos;
                            W[1] += e1;
                            W[2] += e1_2d * pos;
                        }
                        if (diff) {
                            W[0] += e1_d2;
                            W[1] += -2.f * e1_d2;
                            W[2] += e1_d2;
                        }
                        for (int k = 0; k < 3; k++) {
                            idx[j * 4 + k] = j - 1 + k;
                            w4[j * 4 + k] = W[k];
                        }
                    }
                } else {
                    for (uint32_t j = 2; float(j) < ay.zerobin; j++) {
                        const float pos = ay.v[j];
                        float W[4] = {0, 0, 1, 0};
                        if (damp) {
                            W[0] += e1_6d * 1.f * pos;
                            W[1] += e1_6d * -6.f * pos;
                            W[2] += e1 + e1_6d * 3.f * pos;
                            W[3] += e1_6d * 2.f * pos;
                        }
                        if (diff) {
                            W[1] += e1_d2;
                            W[2] += -2.f * e1_d2;
                            W[3] += e1_d2;
                        }
                        for (int k = 0; k < 4; k++) {
                            idx[j * 4 + k] = j - 2 + k;
                            w4[j * 4 + k] = W[k];
                        }
                    }
                    for (uint32_t j = uint32_t(ay.zerobin); j + 2 < n; j++) {
                        const float pos = ay.v[j];
                        float W[4] = {0, 1, 0, 0};
                        if (damp) {
                            W[0] += e1_6d * -2.f * pos;
                            W[1] += e1 + e1_6d * -3.f * pos;
                            W[2] += e1_6d * 6.f * pos;
                            W[3] += e1_6d * -1.f * pos;
                        }
                        if (diff) {
                            W[0] += e1_d2;
                            W[1] += -2.f * e1_d2;
                            W[2] += e1_d2;
                        }
                        for (int k = 0; k < 4; k++) {
                            idx[j * 4 + k] = j - 1 + k;
                            w4[j * 4 + k] = W[k];
                        }
                    }
                    for (uint32_t j : {0u, 1u, n - 2, n - 1}) {
                        for (int k = 0; k < 4; k++) {
                            idx[j * 4 + k] = 0;
                            w4[j * 4 + k] = 0;
                        }
                    }
                }
                for (uint32_t y = 0; y < n; y++) {
                    for (int k = 0; k < 4; k++) {
                        o4[y * 4 + k] = int(idx[y * 4 + k]) - int(y);
                    }
                }
            }
            fpw.insert(fpw.end(), w4.begin(), w4.end());
            fpo.insert(fpo.end(), o4.begin(), o4.end());
            // wake
            if (d.wakescaling != 0) {
                VFPS_REQUIRE(imps && d.impedance >= 0
                                 && uint32_t(d.impedance) < nimp
                                 && imps[d.impedance],
                             "bunch names a missing impedance");
                const vfps_impedance* z = imps[d.impedance];
                VFPS_REQUIRE(z->nfreqs >= 2 * size_t(n),
                             "impedance needs at least 2n frequencies");
                if (wt_off[d.impedance] == 0xffffffffu) {
                    wt_off[d.impedance] = static_cast<uint32_t>(wt.size());
                    wt.resize(wt.size() + z->nfreqs, 0.f);
                }
                B.flags |= F_WAKE;
                B.wt_off = wt_off[d.impedance];
                B.nmax = static_cast<uint32_t>(z->nfreqs);
                B.wakescale = static_cast<float>(d.wakescaling)
                              / static_cast<float>(z->nfreqs);
            }
            // Gaussian start (src/PS/PhaseSpace.cpp:471-484)
            const double zoom2 = d.zoom * d.zoom;
            const float c = 0.398942280401432677939946059934381868f;
            for (const auto* a : {&ax, &ay}) {
                for (uint32_t k = 0; k < n; k++) {
                    gauss.push_back(static_cast<float>(
                        double(c) * std::exp((-0.5) * double(a->v[k])
                                             * double(a->v[k]) / zoom2)));
                }
            }
            for (uint32_t x = 0; x < n; x++) {
                row_bunch.push_back(i);
            }
            dens_off += (size_t(n) * n + 63) & ~size_t(63);
            prof_off += (n + 31) & ~31u;
            row_bunch.resize(prof_off, i);
        }
        VFPS_REQUIRE(dens_off < (size_t(1) << 32),
                     "batch exceeds 2^32 cells per buffer");
        b->cells = dens_off;
        b->rows = prof_off;
        cudaStream_t st = ctx->stream;
        b->bd.alloc(nb);
        VFPS_CUDA(cudaMemcpy(b->bd.p, b->hb.data(), nb * sizeof(BDev),
                             cudaMemcpyHostToDevice));
        b->tabs.alloc(tabs.size());
        VFPS_CUDA(cudaMemcpy(b->tabs.p, tabs.data(), tabs.size() * 4,
                             cudaMemcpyHostToDevice));
        b->fpw.alloc(fpw.size());
        VFPS_CUDA(cudaMemcpy(b->fpw.p, fpw.data(), fpw.size() * 4,
                             cudaMemcpyHostToDevice));
        b->fpo.alloc(fpo.size());
        VFPS_CUDA(cudaMemcpy(b->fpo.p, fpo.data(), fpo.size() * 4,
                             cudaMemcpyHostToDevice));
        b->wt.alloc(std::max<size_t>(wt.size(), 1));
        for (uint32_t k = 0; k < nimp; k++) {
            if (wt_off[k] != 0xffffffffu) {
                // Toeplitz kernel of impedance k (FP64 build)
                vfps::launch_wake_table_raw(ctx, imps[k]->z.p,
                                            imps[k]->nfreqs,
                                            b->wt.p + wt_off[k]);
            }
        }
        b->row_bunch.alloc(row_bunch.size());
        VFPS_CUDA(cudaMemcpy(b->row_bunch.p, row_bunch.data(),
                             row_bunch.size() * 4, cudaMemcpyHostToDevice));
        for (int k = 0; k < 2; k++) {
            b->dens[k].alloc(b->cells);
            b->prof[k].alloc(b->rows);
            VFPS_CUDA(cudaMemsetAsync(b->dens[k].p, 0, b->dens[k].bytes(), st));
            VFPS_CUDA(cudaMemsetAsync(b->prof[k].p, 0, b->prof[k].bytes(), st));
        }
        b->wake.alloc(b->rows);
        VFPS_CUDA(cudaMemsetAsync(b->wake.p, 0, b->wake.bytes(), st));
        b->filling.alloc(nb);
        b->counters.alloc(2);
        VFPS_CUDA(cudaMemsetAsync(b->counters.p, 0, b->counters.bytes(), st));
        b->cur = 0;
        if (data) {
            for (uint32_t i = 0; i < nb; i++) {
                const size_t n2 = size_t(b->hb[i].n) * b->hb[i].n;
                size_t src = 0;
                for (uint32_t k = 0; k < i; k++) {
                    src += size_t(b->hb[k].n) * b->hb[k].n;
                }
                VFPS_CUDA(cudaMemcpyAsync(b->dens[0].p + b->hb[i].dens_off,
                                          data + src, n2 * 4,
                                          cudaMemcpyHostToDevice, st));
            }
            prepare_state(b.get(), any_renorm);
        } else {
            DevBuf<float> g(gauss.size());
            VFPS_CUDA(cudaMemcpyAsync(g.p, gauss.data(), gauss.size() * 4,
                                      cudaMemcpyHostToDevice, st));
            dim3 grid(64, nb);
            k_bgauss<<<grid, 256, 0, st>>>(b->bd.p, g.p, b->dens[0].p);
            VFPS_LAUNCHED();
            // createFromProjections: project, integrate, normalize
            project_all(b.get(), 0);
            integrate_all(b.get(), 0, 0);
            integrate_all(b.get(), 0, 1);
            // end of the constructor: project, integrate
            project_all(b.get(), 0);
            integrate_all(b.get(), 0, 0);
            if (any_renorm) {
                project_all(b.get(), 0);
                integrate_all(b.get(), 0, 1);
            }
            VFPS_CUDA(cudaStreamSynchronize(st));
        }
        VFPS_CUDA(cudaStreamSynchronize(st));
        const char* forced = std::getenv("VFPS_TILE_CELLS");
        const int tile_cells = forced ? std::atoi(forced) : autotune(b.get());
        build_tiles(b.get(), tile_cells);
        setup_kernel(b.get());
        VFPS_CUDA(cudaStreamSynchronize(st));
        *out = b.release();
    });
}

extern "C" int vfps_batch_step(vfps_batch* b, uint64_t nsteps)
{
    if (!b) {
        return VFPS_ERR_INVALID_ARGUMENT;
    }
    return bguard(b->ctx, [&] {
        cudaStream_t st = b->ctx->stream;
        while (nsteps >= 8) {
            VFPS_CUDA(cudaGraphLaunch(b->graph8[b->cur], st));
            nsteps -= 8;   // 8 steps return to the same buffer
        }
        while (nsteps > 0) {
            VFPS_CUDA(cudaGraphLaunch(b->graph[b->cur], st));
            b->cur = 1 - b->cur;
            nsteps--;
        }
    });
}

namespace {

void copy_packed(vfps_batch* b, float* host, bool to_host, bool profiles)
{
    cudaStream_t st = b->ctx->stream;
    size_t src = 0;
    for (uint32_t i = 0; i < b->nb; i++) {
        const BDev& B = b->hb[i];
        const size_t cnt = profiles ? B.n : size_t(B.n) * B.n;
        float* dev = profiles ? b->prof[b->cur].p + B.prof_off
                              : b->dens[b->cur].p + B.dens_off;
        if (to_host) {
            VFPS_CUDA(cudaMemcpyAsync(host + src, dev, cnt * 4,
                                      cudaMemcpyDeviceToHost, st));
        } else {
            VFPS_CUDA(cudaMemcpyAsync(dev, host + src, cnt * 4,
                                      cudaMemcpyHostToDevice, st));
        }
        src += cnt;
    }
}

bool contiguous(const vfps_batch* b)
{
    // one copy suffices when the packed layout has no padding
    size_t off = 0;
    for (const auto& B : b->hb) {
        if (B.dens_off != off) {
            return false;
        }
        off += size_t(B.n) * B.n;
    }
    return off == b->cells;
}

}  // namespace

extern "C" int vfps_batch_run(vfps_batch* b, const float* density_in,
                              uint64_t nsteps, float* density_out,
                              float* profiles_out, float* filling_out)
{
    if (!b) {
        return VFPS_ERR_INVALID_ARGUMENT;
    }
    return bguard(b->ctx, [&] {
        cudaStream_t st = b->ctx->stream;
        if (density_in) {
            if (contiguous(b)) {
                VFPS_CUDA(cudaMemcpyAsync(b->dens[b->cur].p, density_in,
                                          b->cells * 4,
                                          cudaMemcpyHostToDevice, st));
            } else {
                copy_packed(b, const_cast<float*>(density_in), false, false);
            }
            project_all(b, b->cur);
        }
        while (nsteps >= 8) {
            VFPS_CUDA(cudaGraphLaunch(b->graph8[b->cur], st));
            nsteps -= 8;
        }
        while (nsteps > 0) {
            VFPS_CUDA(cudaGraphLaunch(b->graph[b->cur], st));
            b->cur = 1 - b->cur;
            nsteps--;
        }
        if (density_out) {
            if (contiguous(b)) {
                VFPS_CUDA(cudaMemcpyAsync(density_out, b->dens[b->cur].p,
                                          b->cells * 4,
                                          cudaMemcpyDeviceToHost, st));
            } else {
                copy_packed(b, density_out, true, false);
            }
        }
        if (profiles_out) {
            copy_packed(b, profiles_out, true, true);
        }
        if (filling_out) {
            std::vector<double> f(b->nb);
            VFPS_CUDA(cudaMemcpyAsync(f.data(), b->filling.p, b->nb * 8,
                                      cudaMemcpyDeviceToHost, st));
            VFPS_CUDA(cudaStreamSynchronize(st));
            for (uint32_t i = 0; i < b->nb; i++) {
                filling_out[i] = static_cast<float>(f[i]);
            }
        }
        VFPS_CUDA(cudaStreamSynchronize(st));
    });
}

extern "C" int vfps_batch_layout(const vfps_batch* b, uint32_t i,
                                 size_t* density_offset,
                                 size_t* profile_offset)
{
    if (!b || i >= b->nb) {
        return VFPS_ERR_INVALID_ARGUMENT;
    }
    size_t d = 0, p = 0;
    for (uint32_t k = 0; k < i; k++) {
        d += size_t(b->hb[k].n) * b->hb[k].n;
        p += b->hb[k].n;
    }
    if (density_offset) {
        *density_offset = d;
    }
    if (profile_offset) {
        *profile_offset = p;
    }
    return VFPS_OK;
}

extern "C" int vfps_batch_download(vfps_batch* b, float* density)
{
    if (!b || !density) {
        return VFPS_ERR_INVALID_ARGUMENT;
    }
    return bguard(b->ctx, [&] {
        copy_packed(b, density, true, false);
        VFPS_CUDA(cudaStreamSynchronize(b->ctx->stream));
    });
}

extern "C" int vfps_batch_upload(vfps_batch* b, const float* density)
{
    if (!b || !density) {
        return VFPS_ERR_INVALID_ARGUMENT;
    }
    return bguard(b->ctx, [&] {
        copy_packed(b, const_cast<float*>(density), false, false);
        project_all(b, b->cur);
        integrate_all(b, b->cur, 0);
        VFPS_CUDA(cudaStreamSynchronize(b->ctx->stream));
    });
}

extern "C" int vfps_batch_get_profiles(vfps_batch* b, float* profiles)
{
    if (!b || !profiles) {
        return VFPS_ERR_INVALID_ARGUMENT;
    }
    return bguard(b->ctx, [&] {
        copy_packed(b, profiles, true, true);
        VFPS_CUDA(cudaStreamSynchronize(b->ctx->stream));
    });
}

extern "C" int vfps_batch_get_filling(vfps_batch* b, double* filling)
{
    if (!b || !filling) {
        return VFPS_ERR_INVALID_ARGUMENT;
    }
    return bguard(b->ctx, [&] {
        VFPS_CUDA(cudaMemcpyAsync(filling, b->filling.p, b->nb * 8,
                                  cudaMemcpyDeviceToHost, b->ctx->stream));
        VFPS_CUDA(cudaStreamSynchronize(b->ctx->stream));
    });
}

extern "C" int vfps_batch_get_wake(vfps_batch* b, float* wake)
{
    if (!b || !wake) {
        return VFPS_ERR_INVALID_ARGUMENT;
    }
    return bguard(b->ctx, [&] {
        size_t dst = 0;
        for (uint32_t i = 0; i < b->nb; i++) {
            VFPS_CUDA(cudaMemcpyAsync(wake + dst, b->wake.p + b->hb[i].prof_off,
                                      b->hb[i].n * 4, cudaMemcpyDeviceToHost,
                                      b->ctx->stream));
            dst += b->hb[i].n;
        }
        VFPS_CUDA(cudaStreamSynchronize(b->ctx->stream));
    });
}

extern "C" int vfps_batch_info(const vfps_batch* b, uint32_t* launches,
                               uint32_t* tile_rows)
{
    if (!b) {
        return VFPS_ERR_INVALID_ARGUMENT;
    }
    if (launches) {
        *launches = 1;  // one fused kernel per solver step
    }
    if (tile_rows) {
        *tile_rows = static_cast<uint32_t>(b->tile_rows);
    }
    return VFPS_OK;
}

extern "C" int vfps_batch_destroy(vfps_batch* b)
{
    if (!b) {
        return VFPS_OK;
    }
    cudaSetDevice(b->device);
    destroy_graphs(b);
    delete b;
    return VFPS_OK;
}
