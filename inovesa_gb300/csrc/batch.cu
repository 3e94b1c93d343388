// Batched solver step: many bunch simulations advanced together (no
// reference counterpart; every bunch follows the reference solver step,
// src/main.cpp:948-1053).  One step is k_bwake and, per tile list, one
// maps kernel:
//
//  k_bwake   per bunch: the wake potential of every mesh row as the
//            Toeplitz sum  wake[x] = s sum_m P[m] w[(x-m) mod nmax]  of the
//            previous step's profiles P of its beam (w built once per
//            impedance in FP64), the charge integral (compensated FP32),
//            the renormalisation factor of this step, the y-kick stencils
//            of chain-0 rows and a step ticket.
//  k_bmaps0  chain 0 (main.cpp's loop) for meshes up to 256 rows and for
//            512-row meshes (template: 2 or 4 column groups per lane): a
//            persistent kernel streaming rows through a ring in shared
//            memory (launched as a programmatic dependent of k_bwake).
//  k_bmaps0w  chain 0 for 1024-row meshes on a tile of TX mesh rows: wake
//            y-kick and RF y-kick fused in registers, drift x-kick,
//            Fokker-Planck, the new rows and their projections.
//  k_bmaps1  chain 1 (rotation, wake y-kick, Fokker-Planck).
//
// Layout in HBM: densities packed bunch after bunch ([x][y], y contiguous,
// 256-byte aligned), double-buffered; profiles/wakes packed per row.
// Inside a CTA the staged rows live in shared memory: the input rows of the
// tile plus a halo that covers the reach of the 2-D stage (computed on the
// host from all tap positions); halo rows outside the mesh are zero rows,
// which is exactly the reference's "taps outside the mesh are dropped".
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <map>
#include <mutex>
#include <string>

#include "vfps_internal.cuh"

#include "batch_kernels.cuh"
#include "ring_fast.cuh"
#include "wake_tc.cuh"

using vfps::DevBuf;

// ================================================================== host
enum {
    TL_RING = 0, TL_ROT = 1, TL_WIDE = 2, TL_RING4 = 3, TL_RINGF = 4,
    TL_RINGF128 = 5, TL_RINGF64 = 6, TL_RINGF512 = 7, TL_RINGF1024 = 8,
    TL_COUNT = 9
};
constexpr int RING_MAX_N = 256;   // widest mesh of the ring kernel, G = 2
constexpr int RING4_N = 512;      // the mesh of the ring kernel, G = 4
constexpr int RTHREADS4 = 256;    // its CTA: 8 warps, one row each
constexpr int RINGF_WIDE_N = 1024;  // the widest mesh of the fast kernel
constexpr int RTHREADSF1024 = 256;  // its CTA: two rows of 4 parts at once

struct vfps_batch {
    vfps_ctx* ctx = nullptr;
    int device = 0;
    uint32_t nb = 0;
    std::vector<vfps_bunch_desc> desc;
    std::vector<BDev> hb;
    // tile lists: TL_RINGF, TL_RINGF128, TL_RINGF64, TL_RINGF512,
    // TL_RINGF1024 (chain 0, n = 256, 128, 64, 512, 1024, regular
    // lattices: the fast ring kernel), TL_RING (the other chain-0 meshes up
    // to 256 rows), TL_RING4 (the other chain-0 meshes of 512 rows), TL_ROT
    // (chain 1), TL_WIDE (the other chain-0 meshes of 1024 rows)
    std::vector<Tile> htiles[TL_COUNT];
    size_t cells = 0, rows = 0;
    uint32_t max_n = 0;
    DevBuf<BDev> bd;
    DevBuf<Tile> tiles[TL_COUNT];
    DevBuf<float> tabs, fp5, wt, dwt;
    DevBuf<RowStencil> st;
    DevBuf<PwDev> pw;          // potential-well state: per bunch
    DevBuf<float> pwtab;       // raw RF and drift offsets (potential well)
    DevBuf<uint32_t> row_bunch;
    DevBuf<float> dens[2], prof[2];
    DevBuf<float> wake, factor;
    DevBuf<RowInfo> rinfo;     // chain-0 y-kick stencils of every row
    DevBuf<RowInfo7> rinfo7;   // the same as one 7-tap stencil (F_Y7)
    DevBuf<double> filling;
    // k_bwake's CTAs: (bunch, first row) of each block of rows
    DevBuf<uint2> wblk;
    uint32_t nwblk = 0;
    // step counters: one per k_bwake CTA, which advances its own once per
    // step (no two CTAs share one)
    DevBuf<unsigned long long> tickets;
    int cur = 0;               // buffer holding the current state
    size_t smem[TL_COUNT] = {};
    SmemR layoutR{};           // shared-memory regions of k_bmaps0
    Smem0 layout0{};           // shared-memory regions of k_bmaps0w
    unsigned gridR = 0;        // persistent CTAs of k_bmaps0
    SmemR layoutR4{};          // the same for the 512-row ring kernel
    unsigned gridR4 = 0;
    SmemR layoutRF[5] = {};    // the same for the fast ring kernel, per
    unsigned gridRF[5] = {};   // mesh size 256, 128, 64, 512, 1024
    unsigned grid0 = 0;        // persistent CTAs of k_bmaps0w
    int tile_cells = 0;
    int tile_rows = 0;
    // wake potentials on the tensor cores (k_wake_tc) instead of inside
    // k_bwake: Toeplitz planes per (impedance, mesh size) and bunch tiles
    int wake_tc = 0;
    DevBuf<BeamDev> beams;     // per bunch: its beam (default: alone)
    DevBuf<uint32_t> members;  // bunches grouped by beam
    bool coupled = false;      // some beam has more than one bunch
    // CSR power recording (vfps_batch_set_csr)
    DevBuf<float> csrk;        // K tables
    DevBuf<uint32_t> csroff;   // per bunch: its table or NO_CSR
    DevBuf<float> csrpow;      // ring [cap][nb]
    DevBuf<unsigned long long> csrsteps;   // ring [cap]
    DevBuf<float2> csrpart;    // [nb][CSR_MAXBLK] blocks' parts of a step
    DevBuf<unsigned> csrdone;  // [nb] blocks done (reset by the last)
    uint32_t csr_every = 0, csr_cap = 0;
    DevBuf<float> tplanes;
    DevBuf<TcGroup> tcg;
    DevBuf<uint2> tclist;      // per tile member: profile offset, scaling
    uint32_t tc_groups = 0;
    bool tc_ok = true;     // every wake mesh fits the tensor-core kernel
    uint32_t tc_n = 0;     // the widest of them
    uint32_t tc_smem = 0;  // k_wake_tc's shared memory for all of them
    // a second stream for the maps kernels of the other mesh classes, which
    // run next to the first ring kernel (fork after k_bwake, join before
    // the step ends)
    cudaStream_t side = nullptr;
    cudaEvent_t fork = nullptr, join = nullptr;
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

// KickMap::updateSM (src/SM/KickMap.cpp:339-389) for one offset, in the
// kernel's stencil form (host copy of make_stencil)
RowStencil host_stencil(float offset, uint32_t n, int it)
{
    RowStencil r;
    r.shift0 = 0;
    for (int j = 0; j < 4; j++) {
        r.w[j] = 0.f;
    }
    const float poffs = static_cast<float>(n / 2) + offset;
    const float t = std::trunc(poffs);
    if (!(t >= 0) || !(t < static_cast<float>(n))) {
        return r;
    }
    const int jd = static_cast<int>(t);
    const float f = poffs - t;
    float c[4] = {0, 0, 0, 0};
    switch (it) {
    case 1:
        c[0] = 1.f;
        break;
    case 2:
        c[0] = 1.f - f;
        c[1] = f;
        break;
    case 3:
        c[0] = f * (f - 1.f) * 0.5f;
        c[1] = 1.f - f * f;
        c[2] = f * (f + 1.f) * 0.5f;
        break;
    default:
        c[0] = (f - 1.f) * (f - 2.f) * f * static_cast<float>(-1. / 6.);
        c[1] = (f + 1.f) * (f - 1.f) * (f - 2.f) * 0.5f;
        c[2] = (2.f - f) * f * (f + 1.f) * 0.5f;
        c[3] = f * (f + 1.f) * (f - 1.f) * static_cast<float>(1. / 6.);
        break;
    }
    const int h = (it - 1) / 2;
    bool any = false;
    for (int j = 0; j < it; j++) {
        const int j0 = jd + j - h;
        if (j0 >= 0 && j0 < int(n)) {
            r.w[j] = c[j];
            any = true;
        }
    }
    r.shift0 = any ? jd - h - int(n / 2) : 0;
    return r;
}

// One solver step of every bunch.  ev (optional, 4 events): recorded
// before k_bwake and after k_bwake, the chain-0 kernels and k_bmaps1.
void launch_step(vfps_batch* b, int from, cudaEvent_t* ev = nullptr)
{
    const int to = 1 - from;
    cudaStream_t st = b->ctx->stream;
    auto mark = [&](int i) {
        if (ev) {
            VFPS_CUDA(cudaEventRecord(ev[i], st));
        }
    };
    // P[n], padded W[2n + n/4], partial sums [Q][n] with Q n = 8 THREADS,
    // a coupled beam's wake [n] and member profile [n]
    const size_t wsm = (5 * size_t(b->max_n) + b->max_n / 4 + 8 * THREADS)
                       * sizeof(float);
    mark(0);
    const bool tc = b->wake_tc && b->tc_groups > 0;
    if (tc) {
        const dim3 grid((b->tc_n + TC_M - 1) / TC_M, b->tc_groups);
        k_wake_tc<<<grid, TC_THREADS, b->tc_smem, st>>>(
            b->tcg.p, b->tclist.p, b->tplanes.p, b->prof[from].p,
            b->wake.p, b->ctx->d_status);
        VFPS_LAUNCHED();
    }
    {
        // a programmatic dependent of the previous step's maps kernel (when
        // that is the last kernel on this stream): the launch overlaps that
        // kernel's end, and k_bwake waits for it before it reads or writes
        // anything the maps kernel touches
        cudaLaunchAttribute at[1];
        at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
        at[0].val.programmaticStreamSerializationAllowed = 1;
        cudaLaunchConfig_t c = {};
        c.gridDim = dim3(b->nwblk);
        c.blockDim = dim3(THREADS);
        c.dynamicSmemBytes = wsm;
        c.stream = st;
        c.attrs = at;
        c.numAttrs = tc ? 0 : 1;
        VFPS_CUDA(cudaLaunchKernelEx(
            &c, k_bwake, (const BDev*)b->bd.p, (const uint2*)b->wblk.p,
            (const float*)b->tabs.p, (const float*)b->wt.p,
            (const RowStencil*)b->st.p, (const float*)b->prof[from].p,
            b->wake.p, b->rinfo.p, b->rinfo7.p, b->factor.p, b->filling.p,
            b->tickets.p, (const BeamDev*)b->beams.p,
            (const uint32_t*)b->members.p,
            CsrRec{b->csrk.p, b->csroff.p, b->csrpow.p, b->csrsteps.p,
                   b->csr_every, b->csr_cap, b->nb, b->csrpart.p,
                   b->csrdone.p},
            b->ctx->d_status, tc ? 1 : 0, b->nwblk == b->nb ? 1 : 0));
    }
    VFPS_LAUNCHED();
    mark(1);
    // programmatic dependent launch of the first ring kernel: its CTAs zero
    // their rings, set up their barriers and start the bulk copies of their
    // first density rows while k_bwake runs, then wait for it to finish
    // (griddepcontrol.wait) before they read its stencils or write device
    // memory.  (The fast ring kernel lets the next k_bwake launch only at
    // its end: k_bwake CTAs launched earlier crowd onto the SMs that finish
    // first, which was measured slower.)
    cudaLaunchAttribute pdl[1];
    pdl[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    pdl[0].val.programmaticStreamSerializationAllowed = 1;
    // the maps kernels of a batch with several mesh classes: the first on
    // this stream, the others on the side stream, all after k_bwake, so
    // that each fills the SMs the others leave free (no kernel's tail
    // idles the GPU); sequential when the kernels are timed one by one
    int classes = 0;
    for (int c : {TL_RINGF, TL_RINGF128, TL_RINGF64, TL_RINGF512,
                  TL_RINGF1024, TL_RING, TL_RING4, TL_WIDE, TL_ROT}) {
        classes += b->htiles[c].empty() ? 0 : 1;
    }
    const bool forked = !ev && classes > 1;
    if (forked) {
        VFPS_CUDA(cudaEventRecord(b->fork, st));
        VFPS_CUDA(cudaStreamWaitEvent(b->side, b->fork, 0));
    }
    bool first_ring = true;
    bool first = true;   // the next maps kernel is the step's first
    auto next_stream = [&]() {
        const cudaStream_t s = first || !forked ? st : b->side;
        first = false;
        return s;
    };
    auto ring_launch = [&](auto kernel, int list, unsigned grid, int threads,
                           const SmemR& layout, auto rinfo) {
        if (b->htiles[list].empty()) {
            return;
        }
        cudaLaunchConfig_t c = {};
        c.gridDim = dim3(grid);
        c.blockDim = dim3(threads);
        c.dynamicSmemBytes = b->smem[list];
        c.stream = next_stream();
        c.attrs = pdl;
        c.numAttrs = first_ring ? 1 : 0;
        first_ring = false;
        VFPS_CUDA(cudaLaunchKernelEx(
            &c, kernel, (const BDev*)b->bd.p, (const Tile*)b->tiles[list].p,
            static_cast<uint32_t>(b->htiles[list].size()),
            (const float*)b->tabs.p, (const float*)b->dwt.p,
            rinfo, (const float*)b->dens[from].p,
            b->dens[to].p, b->prof[to].p, b->ctx->d_status, layout));
        VFPS_LAUNCHED();
    };
    ring_launch(k_bmaps0f<RTHREADS, 256>, TL_RINGF, b->gridRF[0], RTHREADS,
                b->layoutRF[0], (const RowInfo7*)b->rinfo7.p);
    ring_launch(k_bmaps0f<RTHREADS, 128>, TL_RINGF128, b->gridRF[1],
                RTHREADS, b->layoutRF[1], (const RowInfo7*)b->rinfo7.p);
    ring_launch(k_bmaps0f<RTHREADS, 64>, TL_RINGF64, b->gridRF[2], RTHREADS,
                b->layoutRF[2], (const RowInfo7*)b->rinfo7.p);
    ring_launch(k_bmaps0f<RTHREADS, 512>, TL_RINGF512, b->gridRF[3],
                RTHREADS, b->layoutRF[3], (const RowInfo7*)b->rinfo7.p);
    ring_launch(k_bmaps0f<RTHREADSF1024, 1024>, TL_RINGF1024, b->gridRF[4],
                RTHREADSF1024, b->layoutRF[4], (const RowInfo7*)b->rinfo7.p);
    ring_launch(k_bmaps0<2, RTHREADS>, TL_RING, b->gridR, RTHREADS,
                b->layoutR, (const RowInfo*)b->rinfo.p);
    ring_launch(k_bmaps0<4, RTHREADS4>, TL_RING4, b->gridR4, RTHREADS4,
                b->layoutR4, (const RowInfo*)b->rinfo.p);
    if (!b->htiles[TL_WIDE].empty()) {
        k_bmaps0w<<<b->grid0, THREADS, b->smem[TL_WIDE], next_stream()>>>(
            b->bd.p, b->tiles[TL_WIDE].p,
            static_cast<uint32_t>(b->htiles[TL_WIDE].size()), b->tabs.p,
            b->st.p, b->fp5.p, b->rinfo.p, b->dens[from].p,
            b->dens[to].p, b->prof[to].p, b->ctx->d_status, b->layout0);
        VFPS_LAUNCHED();
    }
    mark(2);
    if (!b->htiles[TL_ROT].empty()) {
        k_bmaps1<<<static_cast<unsigned>(b->htiles[TL_ROT].size()), THREADS,
                   b->smem[TL_ROT], next_stream()>>>(
            b->bd.p, b->tiles[TL_ROT].p, b->tabs.p, b->fp5.p, b->wake.p,
            b->factor.p, b->dens[from].p, b->dens[to].p, b->prof[to].p);
        VFPS_LAUNCHED();
    }
    if (forked) {
        VFPS_CUDA(cudaEventRecord(b->join, b->side));
        VFPS_CUDA(cudaStreamWaitEvent(st, b->join, 0));
    }
    mark(3);
}

// persistent grid of a kernel: as many CTAs as fit on the device with
// `smem` bytes each, at most one per tile
template <typename K>
unsigned persistent_grid(vfps_batch* b, K kernel, int threads, size_t smem,
                         size_t ntiles)
{
    int per_sm = 0;
    if (smem <= 227 * 1024
        && cudaFuncSetAttribute(kernel,
                                cudaFuncAttributeMaxDynamicSharedMemorySize,
                                static_cast<int>(smem)) == cudaSuccess
        && cudaOccupancyMaxActiveBlocksPerMultiprocessor(
               &per_sm, kernel, threads, smem) == cudaSuccess) {
        per_sm = std::max(per_sm, 1);
    } else {
        per_sm = 1;
    }
    return static_cast<unsigned>(
        std::min<size_t>(ntiles, size_t(per_sm) * b->ctx->sm_count));
}

void build_tiles(vfps_batch* b, int tile_cells)
{
    for (int c = 0; c < TL_COUNT; c++) {
        b->htiles[c].clear();
        b->smem[c] = 0;
    }
    int max_rows = 0;
    // regions sized for the largest tile of each kernel
    size_t a_floats = 0, b_floats = 0, t_floats = 0, s_rows = 0, p_rows = 0;
    int ring_rows = 0, ring_n = 0, ring4_rows = 0;
    int ringf_rows[5] = {0, 0, 0, 0, 0};
    for (uint32_t i = 0; i < b->nb; i++) {
        const BDev& B = b->hb[i];
        const int n = int(B.n);
        const int c = B.chain == 1 ? TL_ROT
                      : (n <= RING_MAX_N
                             ? ((B.flags & F_Y7)
                                    ? (n == 256 ? TL_RINGF
                                                : (n == 128 ? TL_RINGF128
                                                            : TL_RINGF64))
                                    : TL_RING)
                             : (n == RING4_N ? ((B.flags & F_Y7)
                                                    ? TL_RINGF512
                                                    : TL_RING4)
                                             : ((B.flags & F_Y7)
                                                    ? TL_RINGF1024
                                                    : TL_WIDE)));
        const int fk = c == TL_RINGF ? 0
                       : c == TL_RINGF128 ? 1
                       : c == TL_RINGF64 ? 2
                       : c == TL_RINGF512 ? 3
                       : c == TL_RINGF1024 ? 4 : -1;
        int tx = std::max(4, tile_cells / n);
        if (c == TL_RING || c == TL_RING4 || fk >= 0) {
            // the ring holds two tiles with their halos: at most 32 staged
            // rows per tile keeps it at 64 slots or fewer
            tx = std::min(tx, std::max(4, 32 - B.halo_lo - B.halo_hi));
        }
        tx = std::min(tx, n);
        max_rows = std::max(max_rows, tx);
        for (int x0 = 0; x0 < n; x0 += tx) {
            const int rows = std::min(tx, n - x0);
            b->htiles[c].push_back({i, uint32_t(x0), uint32_t(rows), 0});
        }
        const int nr = tx + B.halo_lo + B.halo_hi;
        if (c == TL_RING) {
            ring_rows = std::max(ring_rows, nr);
            ring_n = std::max(ring_n, n);
        } else if (fk >= 0) {
            ringf_rows[fk] = std::max(ringf_rows[fk], nr);
        } else if (c == TL_RING4) {
            ring4_rows = std::max(ring4_rows, nr);
        } else if (c == TL_WIDE) {
            a_floats = std::max(a_floats, size_t(nr) * astride0(n));
            b_floats = std::max(b_floats, size_t(nr) * n);
            t_floats = std::max(t_floats, size_t(tx) * (n + 2 * TPAD));
            s_rows = std::max(s_rows, size_t(nr));
            p_rows = std::max(p_rows, size_t(tx));
        } else {
            b->smem[TL_ROT] = std::max(b->smem[TL_ROT],
                                       smem1(n, nr, tx).total);
        }
    }
    size_t o = 0;
    auto take = [&](uint32_t* at, size_t bytes) {
        *at = static_cast<uint32_t>(o);
        o = align16(o + bytes);
    };
    // the ring holds the staged rows of two tiles with their halos
    // parts: the fast kernel's row parts on 512- and 1024-row meshes
    // (their sums of two tiles), planes: the drift and Fokker-Planck table
    auto ring_layout = [&](SmemR& L, int rows, int n, size_t rec,
                           int parts = 0, int planes = 10) {
        const int rb = 2 * rows;
        L.rb = static_cast<uint32_t>(rb);
        L.rs = static_cast<uint32_t>(astride0(n));
        o = 0;
        take(&L.ring, size_t(rb) * L.rs * 4);
        take(&L.s, size_t(rows) * rec);
        take(&L.tab, size_t(planes) * n * 4);
        take(&L.part, size_t(parts) * rb * 4);
        take(&L.bar, 3 * sizeof(uint64_t));
        L.total = static_cast<uint32_t>(o);
        return o;
    };
    const int flist[5] = {TL_RINGF, TL_RINGF128, TL_RINGF64, TL_RINGF512,
                          TL_RINGF1024};
    const int fn[5] = {256, 128, 64, 512, 1024};
    for (int k = 0; k < 5; k++) {
        const int c = flist[k];
        if (b->htiles[c].empty()) {
            continue;
        }
        b->smem[c] = ring_layout(b->layoutRF[k], ringf_rows[k], fn[k],
                                 sizeof(RowInfo7),
                                 fn[k] > RING_MAX_N ? fn[k] / 256 : 0,
                                 fn[k] == RINGF_WIDE_N ? 11 : 10);
        const size_t nt = b->htiles[c].size();
        b->gridRF[k] =
            k == 0 ? persistent_grid(b, k_bmaps0f<RTHREADS, 256>, RTHREADS,
                                     b->smem[c], nt)
            : k == 1 ? persistent_grid(b, k_bmaps0f<RTHREADS, 128>, RTHREADS,
                                       b->smem[c], nt)
            : k == 2 ? persistent_grid(b, k_bmaps0f<RTHREADS, 64>, RTHREADS,
                                       b->smem[c], nt)
            : k == 3 ? persistent_grid(b, k_bmaps0f<RTHREADS, 512>, RTHREADS,
                                       b->smem[c], nt)
                     : persistent_grid(b, k_bmaps0f<RTHREADSF1024, 1024>,
                                       RTHREADSF1024, b->smem[c], nt);
    }
    if (!b->htiles[TL_RING].empty()) {
        b->smem[TL_RING] = ring_layout(b->layoutR, ring_rows, ring_n,
                                       sizeof(RowInfo));
        b->gridR = persistent_grid(b, k_bmaps0<2, RTHREADS>, RTHREADS,
                                   b->smem[TL_RING],
                                   b->htiles[TL_RING].size());
    }
    if (!b->htiles[TL_RING4].empty()) {
        b->smem[TL_RING4] = ring_layout(b->layoutR4, ring4_rows, RING4_N,
                                        sizeof(RowInfo));
        b->gridR4 = persistent_grid(b, k_bmaps0<4, RTHREADS4>, RTHREADS4,
                                    b->smem[TL_RING4],
                                    b->htiles[TL_RING4].size());
    }
    if (!b->htiles[TL_WIDE].empty()) {
        Smem0& L = b->layout0;
        o = 0;
        take(&L.a[0], a_floats * 4);
        take(&L.a[1], a_floats * 4);
        take(&L.b, b_floats * 4);
        take(&L.t, t_floats * 4);
        take(&L.s, s_rows * sizeof(RowInfo));
        take(&L.part, p_rows * 8 * 4);
        take(&L.bar, 2 * sizeof(uint64_t));
        take(&L.pads, 4 * sizeof(int));
        L.a_floats = static_cast<uint32_t>(a_floats);
        L.total = static_cast<uint32_t>(o);
        b->smem[TL_WIDE] = o;
        b->grid0 = persistent_grid(b, k_bmaps0w, THREADS, o,
                                   b->htiles[TL_WIDE].size());
    }
    b->tile_cells = tile_cells;
    b->tile_rows = max_rows;
}

bool tiles_fit(const vfps_batch* b)
{
    for (int c = 0; c < TL_COUNT; c++) {
        if (b->smem[c] > 227 * 1024) {
            return false;
        }
    }
    return true;
}

void upload_tiles(vfps_batch* b)
{
    VFPS_REQUIRE(tiles_fit(b),
                 "tile of the largest mesh does not fit in shared memory");
    VFPS_CUDA(cudaFuncSetAttribute(k_bmaps0f<RTHREADS, 256>,
                                   cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   static_cast<int>(std::max<size_t>(
                                       b->smem[TL_RINGF], 1))));
    VFPS_CUDA(cudaFuncSetAttribute(k_bmaps0f<RTHREADS, 128>,
                                   cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   static_cast<int>(std::max<size_t>(
                                       b->smem[TL_RINGF128], 1))));
    VFPS_CUDA(cudaFuncSetAttribute(k_bmaps0f<RTHREADS, 64>,
                                   cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   static_cast<int>(std::max<size_t>(
                                       b->smem[TL_RINGF64], 1))));
    VFPS_CUDA(cudaFuncSetAttribute(k_bmaps0f<RTHREADS, 512>,
                                   cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   static_cast<int>(std::max<size_t>(
                                       b->smem[TL_RINGF512], 1))));
    VFPS_CUDA(cudaFuncSetAttribute(k_bmaps0f<RTHREADSF1024, 1024>,
                                   cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   static_cast<int>(std::max<size_t>(
                                       b->smem[TL_RINGF1024], 1))));
    VFPS_CUDA(cudaFuncSetAttribute(k_bmaps0<2, RTHREADS>,
                                   cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   static_cast<int>(std::max<size_t>(
                                       b->smem[TL_RING], 1))));
    VFPS_CUDA(cudaFuncSetAttribute(k_bmaps0<4, RTHREADS4>,
                                   cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   static_cast<int>(std::max<size_t>(
                                       b->smem[TL_RING4], 1))));
    VFPS_CUDA(cudaFuncSetAttribute(k_bmaps0w,
                                   cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   static_cast<int>(std::max<size_t>(
                                       b->smem[TL_WIDE], 1))));
    VFPS_CUDA(cudaFuncSetAttribute(k_bmaps1,
                                   cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   static_cast<int>(std::max<size_t>(
                                       b->smem[TL_ROT], 1))));
    for (int c = 0; c < TL_COUNT; c++) {
        b->tiles[c].alloc(std::max<size_t>(b->htiles[c].size(), 1));
        if (!b->htiles[c].empty()) {
            VFPS_CUDA(cudaMemcpy(b->tiles[c].p, b->htiles[c].data(),
                                 b->htiles[c].size() * sizeof(Tile),
                                 cudaMemcpyHostToDevice));
        }
    }
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

void make_graphs(vfps_batch* b)
{
    destroy_graphs(b);
    for (int i = 0; i < 2; i++) {
        b->graph[i] = capture(b, i, 1);
        b->graph8[i] = capture(b, i, 8);
    }
}

// Autotuner: time candidate tile sizes on the batch itself (its state is
// saved and restored) and keep the fastest; cached per mesh mix.
std::mutex g_tune_mu;
std::map<std::string, int> g_tune_cache;

int autotune(vfps_batch* b)
{
    std::string key;
    for (auto& B : b->hb) {
        key += std::to_string(B.n) + "/" + std::to_string(B.chain) + "/"
               + std::to_string(B.halo_lo) + "/" + std::to_string(B.halo_hi)
               + ",";
    }
    {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        auto it = g_tune_cache.find(key);
        if (it != g_tune_cache.end()) {
            return it->second;
        }
    }
    cudaStream_t st = b->ctx->stream;
    DevBuf<float> sd(b->dens[b->cur].n), sp(b->prof[b->cur].n);
    VFPS_CUDA(cudaMemcpyAsync(sd.p, b->dens[b->cur].p, sd.bytes(),
                              cudaMemcpyDeviceToDevice, st));
    VFPS_CUDA(cudaMemcpyAsync(sp.p, b->prof[b->cur].p, sp.bytes(),
                              cudaMemcpyDeviceToDevice, st));
    DevBuf<unsigned long long> saved(b->tickets.n);
    VFPS_CUDA(cudaMemcpyAsync(saved.p, b->tickets.p, saved.bytes(),
                              cudaMemcpyDeviceToDevice, st));
    VFPS_CUDA(cudaStreamSynchronize(st));
    const int cands[] = {2048, 3072, 4096, 6144, 8192, 12288};
    int best = 4096;
    float best_ms = 1e30f;
    cudaEvent_t e0, e1;
    VFPS_CUDA(cudaEventCreate(&e0));
    VFPS_CUDA(cudaEventCreate(&e1));
    for (int c : cands) {
        build_tiles(b, c);
        if (!tiles_fit(b)) {
            continue;
        }
        upload_tiles(b);
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
    VFPS_CUDA(cudaMemcpyAsync(b->tickets.p, saved.p, saved.bytes(),
                              cudaMemcpyDeviceToDevice, st));
    VFPS_CUDA(cudaStreamSynchronize(st));
    {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        g_tune_cache[key] = best;
    }
    return best;
}

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

// the state after loading densities: the PhaseSpace(data) constructor
// (project, integrate) and the solver's initial renormalisation
// (src/main.cpp:527-532) for bunches with renormalize >= 0
void prepare_state(vfps_batch* b, bool normalize_initial)
{
    project_all(b, b->cur);
    integrate_all(b, b->cur, 0);
    if (normalize_initial) {
        project_all(b, b->cur);
        integrate_all(b, b->cur, 1);
    }
}

// Fokker-Planck stencils (src/SM/FokkerPlanckMap.cpp:11-118) as 5 weights
// per energy cell for the offsets -2..2
std::vector<float> fp_weights(const vfps::Axis& ay, float e1, int fptype,
                              int derivation)
{
    const uint32_t n = ay.n;
    std::vector<float> w5(size_t(n) * 5, 0.f);
    const float e1_2d = e1 / (2.f * ay.delta);
    const float e1_6d = e1 / (6.f * ay.delta);
    const float e1_d2 = e1 / (ay.delta * ay.delta);
    const bool damp = fptype != 0 && fptype != 2;
    const bool diff = fptype != 0 && fptype != 1;
    auto put = [&](uint32_t y, int first, const float* W, int cnt) {
        for (int k = 0; k < cnt; k++) {
            w5[size_t(y) * 5 + (first + k + 2)] = W[k];
        }
    };
    if (derivation == 3) {
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
            put(j, -1, W, 3);
        }
        return w5;
    }
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
        put(j, -2, W, 4);
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
        for (int k = 0; k < 5; k++) {
            w5[size_t(j) * 5 + k] = 0.f;
        }
        put(j, -1, W, 4);
    }
    for (uint32_t j : {0u, 1u, n - 2, n - 1}) {
        for (int k = 0; k < 5; k++) {
            w5[size_t(j) * 5 + k] = 0.f;
        }
    }
    return w5;
}

// The lattice forms k_bmaps0f takes: the drift shifts of every aligned
// group of 4 energy columns differ by at most `spread` (0: one window of 4
// rows per group; 1: the 5-row window of 1024-row meshes), and the
// Fokker-Planck stencils of the lower half of the energy columns
// reach offsets -2..1 only, those of the upper half -1..2 only (4 taps),
// except the last column of the lower half, which may reach -2..2 (the
// reference starts its upper stencils at the truncated centre, which is
// that column on a mesh centred on the reference energy)
bool fast_ring_ok(const std::vector<RowStencil>& dr,
                  const std::vector<float>& w5, uint32_t n, int spread)
{
    for (uint32_t y = 0; y < n; y += 4) {
        int lo = dr[y].shift0, hi = dr[y].shift0;
        for (uint32_t c = 1; c < 4; c++) {
            lo = std::min(lo, dr[y + c].shift0);
            hi = std::max(hi, dr[y + c].shift0);
        }
        if (hi - lo > spread) {
            return false;
        }
    }
    for (uint32_t y = 0; y < n; y++) {
        if (y + 1 != n / 2 && w5[size_t(y) * 5 + (y < n / 2 ? 4 : 0)] != 0.f) {
            return false;
        }
    }
    return true;
}

// VFPS_RING_KERNEL=classic keeps every chain-0 mesh up to 256 rows on
// k_bmaps0 (the two kernels side by side in tests and profiles)
bool fast_ring_off()
{
    const char* v = std::getenv("VFPS_RING_KERNEL");
    return v && std::string(v) == "classic";
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
        std::vector<float> tabs, fp5, wt, gauss, dwt, pwtab;
        std::vector<PwDev> pws;
        std::map<std::string, uint32_t> dw_seen;
        std::vector<RowStencil> sts;
        std::vector<uint32_t> row_bunch, goff;
        std::vector<uint32_t> wt_off(nimp, 0xffffffffu);
        size_t dens_off = 0, prof_off = 0;
        bool any_renorm = false;
        for (uint32_t i = 0; i < nb; i++) {
            const vfps_bunch_desc& d = desc[i];
            const uint32_t n = d.n;
            VFPS_REQUIRE(n >= 64 && n <= 1024 && (n & (n - 1)) == 0,
                         "batched meshes must be a power of two, 64..1024 "
                         "(wider meshes run on the plain path)");
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
            B.st_off = static_cast<uint32_t>(sts.size());
            B.fp_off = static_cast<uint32_t>(fp5.size());
            B.renorm = d.renormalize;
            B.fillset = 1.f;
            if (d.clamp) {
                B.flags |= F_CLAMP;
            }
            any_renorm = any_renorm || d.renormalize >= 0;
            b->max_n = std::max(b->max_n, n);
            const auto ax = vfps::make_axis(n, float(d.axes[0]),
                                            float(d.axes[1]), float(d.axes[2]));
            const auto ay = vfps::make_axis(n, float(d.axes[3]),
                                            float(d.axes[4]), float(d.axes[5]));
            B.dq = ax.delta;
            B.dp = ay.delta;
            B.zbq = ax.zerobin;
            B.zbp = ay.zerobin;
            const auto ws = simpson(n, ax.delta);
            tabs.insert(tabs.end(), ws.begin(), ws.end());
            tabs.insert(tabs.end(), ax.v.begin(), ax.v.end());
            tabs.insert(tabs.end(), ay.v.begin(), ay.v.end());
            // RF (per row) and drift (per column) stencils
            std::vector<RowStencil> rf(n), dr(n);
            PwDev pwd{};
            if (d.chain == 0) {
                // their raw offsets for the potential-well state
                pwd.off = static_cast<uint32_t>(pwtab.size());
                pwd.T = static_cast<float>(d.slip[0])
                        / (ax.delta * ay.delta);
                pwtab.resize(pwtab.size() + 2 * size_t(n), 0.f);
                const float bl2phase = static_cast<float>(d.rf_bl2phase);
                for (uint32_t x = 0; x < n; x++) {
                    float o;
                    if (d.rf_linear) {
                        // src/SM/RFKickMap.cpp:59-68 (static phase)
                        const float ang = static_cast<float>(d.rf_angle);
                        o = std::tan(ang) * (ax.zerobin - float(x));
                        o += std::tan(ang) * 0.f / bl2phase / ax.delta;
                    } else {
                        // src/SM/RFKickMap.cpp:69-78
                        o = float(d.rf_revpart)
                            * (-1.f * float(d.rf_vrf)
                                   * std::sin(ax.v[x] * bl2phase
                                              + float(d.rf_phase))
                               + float(d.rf_v0))
                            / ay.delta / ay.scale;
                    }
                    rf[x] = host_stencil(o, n, d.it);
                    pwtab[pwd.off + x] = o;
                }
                // src/SM/DriftMap.cpp:21-30
                const float e0 = float(d.e0);
                int lo = 0, hi = 0;
                for (uint32_t y = 0; y < n; y++) {
                    float o = 0;
                    for (int s = 0; s < d.nslip && s < 3; s++) {
                        o += float(d.slip[s]) * ay.v[y]
                             * std::pow(ay.v[y] * ay.scale / e0, float(s));
                    }
                    o /= ax.delta;
                    dr[y] = host_stencil(o, n, d.it);
                    pwtab[pwd.off + n + y] = o;
                    lo = std::min(lo, dr[y].shift0);
                    hi = std::max(hi, dr[y].shift0 + 3);
                }
                B.halo_lo = std::max(0, -lo);
                B.halo_hi = std::max(0, hi);
            } else {
                const float ang = static_cast<float>(d.angle);
                // the potential-well state of the rotation chain: the
                // linear kick and drift of the rotation's angle (both axes
                // in units of the spreads)
                pwd.off = static_cast<uint32_t>(pwtab.size());
                pwd.T = ang / (ax.delta * ay.delta);
                pwd.chain = 1;
                pwtab.resize(pwtab.size() + 2 * size_t(n), 0.f);
                for (uint32_t x = 0; x < n; x++) {
                    pwtab[pwd.off + x] = std::tan(ang) * (ax.zerobin
                                                          - float(x));
                }
                for (uint32_t y = 0; y < n; y++) {
                    pwtab[pwd.off + n + y] = ang * ay.v[y] / ax.delta;
                }
                B.cs = std::cos(-ang);
                B.sn = std::sin(-ang);
                const int h = (d.it - 1) / 2;
                B.rot_h = h;
                int lo = 0, hi = 0;
                for (uint32_t x0 = 0; x0 < n; x0++) {
                    for (uint32_t y0 = 0; y0 < n; y0++) {
                        // the kernel's float operations, unfused
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
                        lo = std::min(lo, x1 - h - int(x0));
                        hi = std::max(hi, x1 - h + 3 - int(x0));
                    }
                }
                B.halo_lo = std::max(0, -lo) + 1;
                B.halo_hi = std::max(0, hi) + 1;
            }
            sts.insert(sts.end(), rf.begin(), rf.end());
            sts.insert(sts.end(), dr.begin(), dr.end());
            pws.push_back(pwd);
            if (d.chain == 0) {
                std::vector<float> w5(size_t(n) * 5, 0.f);
                if (d.e1 > 0) {
                    w5 = fp_weights(ay, float(d.e1), d.fptype, d.derivation);
                } else {
                    for (uint32_t y = 0; y < n; y++) {
                        w5[size_t(y) * 5 + 2] = 1.f;
                    }
                }
                // 1024 rows: the fast kernel's 5-row window (a group of 4
                // columns may span two drift shifts)
                const bool win5 = n == RINGF_WIDE_N;
                if ((n <= RING_MAX_N || n == RING4_N || win5)
                    && fast_ring_ok(dr, w5, n, win5 ? 1 : 0)
                    && !fast_ring_off()) {
                    B.flags |= F_Y7;
                }
                // drift stencils as planes for 16-byte loads: w[j][y] for
                // j < 4, then shift0[y] (int bits), then the Fokker-Planck
                // weights as planes F[o][y] for the offsets -2..2 (the
                // identity without Fokker-Planck).  The 5-row window's
                // table: planes j < 5 of the taps from the group's lowest
                // shift (a column one shift higher has a zero in plane 0,
                // the others a zero in plane 4), the group's lowest shift
                // for every column
                std::vector<float> tab;
                const bool t5 = win5 && (B.flags & F_Y7);
                tab.reserve(size_t(n) * (t5 ? 11 : 10));
                std::vector<int> gshift(n);
                for (uint32_t y = 0; y < n; y++) {
                    gshift[y] = dr[y].shift0;
                    if (t5) {
                        const uint32_t g = y & ~3u;
                        gshift[y] = std::min(std::min(dr[g].shift0,
                                                      dr[g + 1].shift0),
                                             std::min(dr[g + 2].shift0,
                                                      dr[g + 3].shift0));
                    }
                }
                for (int j = 0; j < (t5 ? 5 : 4); j++) {
                    for (uint32_t y = 0; y < n; y++) {
                        const int k = j - (dr[y].shift0 - gshift[y]);
                        tab.push_back(k >= 0 && k < 4 ? dr[y].w[k] : 0.f);
                    }
                }
                for (uint32_t y = 0; y < n; y++) {
                    float f;
                    std::memcpy(&f, &gshift[y], sizeof(f));
                    tab.push_back(f);
                }
                for (int o = 0; o < 5; o++) {
                    for (uint32_t y = 0; y < n; y++) {
                        tab.push_back(w5[size_t(y) * 5 + o]);
                    }
                }
                if (t5) {
                    // the fifth row of a window lies one past the rows the
                    // stencils read: one more staged row below the tile
                    B.halo_hi += 1;
                }
                // bunches of a scan share these tables: one copy each, so
                // that a ring kernel's CTA stages a shared one only once
                std::string key(reinterpret_cast<const char*>(tab.data()),
                                tab.size() * sizeof(float));
                auto it = dw_seen.find(key);
                if (it != dw_seen.end()) {
                    B.dw_off = it->second;
                } else {
                    B.dw_off = static_cast<uint32_t>(dwt.size());
                    dw_seen.emplace(std::move(key), B.dw_off);
                    dwt.insert(dwt.end(), tab.begin(), tab.end());
                }
            }
            if (d.e1 > 0) {
                B.flags |= F_FP;
                const auto w5 = fp_weights(ay, float(d.e1), d.fptype,
                                           d.derivation);
                fp5.insert(fp5.end(), w5.begin(), w5.end());
            } else {
                fp5.insert(fp5.end(), size_t(n) * 5, 0.f);
            }
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
                // src/PS/ElectricField.cpp:56-58
                B.wakescale = static_cast<float>(d.wakescaling)
                              / static_cast<float>(z->nfreqs);
            }
            // Gaussian start (src/PS/PhaseSpace.cpp:471-484)
            goff.push_back(static_cast<uint32_t>(gauss.size()));
            const double zoom2 = d.zoom * d.zoom;
            const float c = 0.398942280401432677939946059934381868f;
            for (const auto* a : {&ax, &ay}) {
                for (uint32_t k = 0; k < n; k++) {
                    gauss.push_back(static_cast<float>(
                        double(c) * std::exp((-0.5) * double(a->v[k])
                                             * double(a->v[k]) / zoom2)));
                }
            }
            row_bunch.resize(prof_off + n, i);
            dens_off += (size_t(n) * n + 63) & ~size_t(63);
            prof_off += (n + 31) & ~31u;
            row_bunch.resize(prof_off, i);
        }
        VFPS_REQUIRE(dens_off < (size_t(1) << 32),
                     "batch exceeds 2^32 cells per buffer");
        b->cells = dens_off;
        b->rows = prof_off;
        cudaStream_t st = ctx->stream;
        auto put = [&](auto& dst, const auto& src) {
            dst.alloc(std::max<size_t>(src.size(), 1));
            if (!src.empty()) {
                VFPS_CUDA(cudaMemcpy(dst.p, src.data(),
                                     src.size() * sizeof(src[0]),
                                     cudaMemcpyHostToDevice));
            }
        };
        put(b->bd, b->hb);
        {
            // k_bwake: one CTA per block of rows
            std::vector<uint2> wblk;
            for (uint32_t i = 0; i < nb; i++) {
                const uint32_t n = b->hb[i].n;
                const uint32_t R = static_cast<uint32_t>(
                    wake_block_rows(static_cast<int>(n)));
                for (uint32_t x0 = 0; x0 < n; x0 += R) {
                    wblk.push_back(make_uint2(i, x0));
                }
            }
            b->nwblk = static_cast<uint32_t>(wblk.size());
            put(b->wblk, wblk);
        }
        put(b->tabs, tabs);
        put(b->st, sts);
        put(b->fp5, fp5);
        put(b->dwt, dwt);
        put(b->pw, pws);
        put(b->pwtab, pwtab);
        {
            std::vector<BeamDev> beams(nb);
            std::vector<uint32_t> members(nb);
            for (uint32_t i = 0; i < nb; i++) {
                beams[i] = BeamDev{i, 1u, 0, 0u};
                members[i] = i;
            }
            put(b->beams, beams);
            put(b->members, members);
        }
        {
            const std::vector<uint32_t> none(nb, NO_CSR);
            put(b->csroff, none);
            b->csrk.alloc(1);
            b->csrpow.alloc(1);
            b->csrsteps.alloc(1);
            b->csrpart.alloc(size_t(nb) * CSR_MAXBLK);
            b->csrdone.alloc(nb);
            VFPS_CUDA(cudaMemset(b->csrdone.p, 0, b->csrdone.bytes()));
        }
        b->wt.alloc(std::max<size_t>(wt.size(), 1));
        for (uint32_t k = 0; k < nimp; k++) {
            if (wt_off[k] != 0xffffffffu) {
                // Toeplitz kernel of impedance k (built in FP64)
                vfps::launch_wake_table_raw(ctx, imps[k]->z.p,
                                            imps[k]->nfreqs,
                                            b->wt.p + wt_off[k]);
            }
        }
        // Toeplitz planes T[x][m] = w[(x - m) mod nmax] of every (impedance,
        // mesh size) pair (hi and lo parts for the tensor cores) and the
        // bunch tiles that share them
        {
            std::vector<float> wt_host(wt.size());
            VFPS_CUDA(cudaStreamSynchronize(ctx->stream));
            if (!wt.empty()) {
                VFPS_CUDA(cudaMemcpy(wt_host.data(), b->wt.p,
                                     wt.size() * sizeof(float),
                                     cudaMemcpyDeviceToHost));
            }
            std::vector<float> tp;
            std::vector<TcGroup> groups;
            std::vector<uint2> tl;
            std::map<std::pair<uint32_t, uint32_t>, uint32_t> t_at;
            std::map<std::pair<uint32_t, uint32_t>, std::vector<uint32_t>>
                members;
            for (uint32_t i = 0; i < nb; i++) {
                const BDev& B = b->hb[i];
                if (!(B.flags & F_WAKE)) {
                    continue;
                }
                const auto key = std::make_pair(B.wt_off, B.n);
                members[key].push_back(i);
                if (t_at.count(key)) {
                    continue;
                }
                t_at[key] = static_cast<uint32_t>(tp.size());
                const uint32_t nn = B.n, nmax = B.nmax;
                if (nn % TC_K != 0 || nn > uint32_t(TC_MAX_N)) {
                    b->tc_ok = false;   // no tensor-core wake for this batch
                    continue;
                }
                b->tc_n = std::max(b->tc_n, nn);
                b->tc_smem = std::max(b->tc_smem, tc_smem(int(nn)));
                const float* w = wt_host.data() + B.wt_off;
                // the shared-memory images of every (row tile, chunk):
                // T[x][m] at row r = x mod 128, chunk c of 4, element e,
                // stored at r * 32 + 4 (c ^ (r & 7)) + e; hi plane, then lo
                const uint32_t mtn = (nn + TC_M - 1) / TC_M, nkc = nn / TC_K;
                const size_t at0 = tp.size();
                tp.resize(at0 + size_t(mtn) * nkc * 2 * TC_IMG_FLOATS, 0.f);
                for (uint32_t mt = 0; mt < mtn; mt++) {
                    for (uint32_t kc = 0; kc < nkc; kc++) {
                        float* hi = tp.data() + at0
                                    + (size_t(mt) * nkc + kc) * 2
                                          * TC_IMG_FLOATS;
                        float* lo = hi + TC_IMG_FLOATS;
                        for (uint32_t r = 0; r < uint32_t(TC_M); r++) {
                            const uint32_t x = mt * TC_M + r;
                            if (x >= nn) {
                                break;
                            }
                            for (uint32_t k = 0; k < uint32_t(TC_K); k++) {
                                const uint32_t m = kc * TC_K + k;
                                const float v = w[(x + nmax - m) % nmax];
                                const float h = tf32_hi(v);
                                const uint32_t at =
                                    r * TC_K + 4 * ((k / 4) ^ (r & 7)) + k % 4;
                                hi[at] = h;
                                lo[at] = v - h;
                            }
                        }
                    }
                }
            }
            for (const auto& kv : members) {
                const auto& idx = kv.second;
                for (size_t j = 0; j < idx.size(); j += TC_N) {
                    TcGroup g;
                    g.n = kv.first.second;
                    g.t_off = t_at[kv.first];
                    g.nbt = static_cast<uint32_t>(
                        std::min<size_t>(TC_N, idx.size() - j));
                    g.list_off = static_cast<uint32_t>(tl.size());
                    for (size_t u = j; u < j + g.nbt; u++) {
                        const BDev& Bm = b->hb[idx[u]];
                        uint32_t sc;
                        std::memcpy(&sc, &Bm.wakescale, sizeof(sc));
                        tl.push_back(make_uint2(Bm.prof_off, sc));
                    }
                    groups.push_back(g);
                }
            }
            b->tc_groups = static_cast<uint32_t>(groups.size());
            put(b->tplanes, tp);
            put(b->tcg, groups);
            put(b->tclist, tl);
            if (b->tc_ok && b->tc_n > 0) {
                VFPS_CUDA(cudaFuncSetAttribute(
                    k_wake_tc, cudaFuncAttributeMaxDynamicSharedMemorySize,
                    static_cast<int>(b->tc_smem)));
            }
        }
        put(b->row_bunch, row_bunch);
        for (int k = 0; k < 2; k++) {
            b->dens[k].alloc(b->cells);
            b->prof[k].alloc(b->rows);
            VFPS_CUDA(cudaMemsetAsync(b->dens[k].p, 0, b->dens[k].bytes(), st));
            VFPS_CUDA(cudaMemsetAsync(b->prof[k].p, 0, b->prof[k].bytes(), st));
        }
        b->wake.alloc(b->rows);
        b->rinfo.alloc(b->rows);
        VFPS_CUDA(cudaMemsetAsync(b->rinfo.p, 0, b->rinfo.bytes(), st));
        b->rinfo7.alloc(b->rows);
        VFPS_CUDA(cudaMemsetAsync(b->rinfo7.p, 0, b->rinfo7.bytes(), st));
        VFPS_CUDA(cudaMemsetAsync(b->wake.p, 0, b->wake.bytes(), st));
        b->factor.alloc(nb);
        b->filling.alloc(nb);
        b->tickets.alloc(b->nwblk);
        VFPS_CUDA(cudaMemsetAsync(b->tickets.p, 0, b->tickets.bytes(), st));
        VFPS_CUDA(cudaStreamCreateWithFlags(&b->side, cudaStreamNonBlocking));
        VFPS_CUDA(cudaEventCreateWithFlags(&b->fork,
                                           cudaEventDisableTiming));
        VFPS_CUDA(cudaEventCreateWithFlags(&b->join,
                                           cudaEventDisableTiming));
        b->cur = 0;
        if (data) {
            size_t src = 0;
            for (uint32_t i = 0; i < nb; i++) {
                const size_t n2 = size_t(b->hb[i].n) * b->hb[i].n;
                VFPS_CUDA(cudaMemcpyAsync(b->dens[0].p + b->hb[i].dens_off,
                                          data + src, n2 * 4,
                                          cudaMemcpyHostToDevice, st));
                src += n2;
            }
            prepare_state(b.get(), any_renorm);
        } else {
            DevBuf<float> g(gauss.size());
            DevBuf<uint32_t> go(goff.size());
            VFPS_CUDA(cudaMemcpyAsync(g.p, gauss.data(), gauss.size() * 4,
                                      cudaMemcpyHostToDevice, st));
            VFPS_CUDA(cudaMemcpyAsync(go.p, goff.data(), goff.size() * 4,
                                      cudaMemcpyHostToDevice, st));
            dim3 grid(64, nb);
            k_bgauss<<<grid, 256, 0, st>>>(b->bd.p, go.p, g.p, b->dens[0].p);
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
        upload_tiles(b.get());
        make_graphs(b.get());
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

// per-bunch arrays of n rows (profiles, wakes) without gaps between bunches
bool rows_packed(const vfps_batch* b)
{
    size_t off = 0;
    for (const auto& B : b->hb) {
        if (B.prof_off != off) {
            return false;
        }
        off += B.n;
    }
    return true;
}

void copy_packed(vfps_batch* b, float* host, bool to_host, bool profiles,
                 const float* src_dev = nullptr)
{
    cudaStream_t st = b->ctx->stream;
    if (profiles && rows_packed(b)) {
        // one copy instead of one per bunch (small copies into pageable
        // memory each cost a staged, synchronous transfer)
        const float* dev = src_dev ? src_dev : b->prof[b->cur].p;
        size_t rows = 0;
        for (const auto& B : b->hb) {
            rows += B.n;
        }
        if (to_host) {
            VFPS_CUDA(cudaMemcpyAsync(host, dev, rows * 4,
                                      cudaMemcpyDeviceToHost, st));
        } else {
            VFPS_CUDA(cudaMemcpyAsync(const_cast<float*>(dev), host, rows * 4,
                                      cudaMemcpyHostToDevice, st));
        }
        return;
    }
    size_t off = 0;
    for (uint32_t i = 0; i < b->nb; i++) {
        const BDev& B = b->hb[i];
        const size_t cnt = profiles ? B.n : size_t(B.n) * B.n;
        float* dev = profiles ? (src_dev ? const_cast<float*>(src_dev)
                                         : b->prof[b->cur].p) + B.prof_off
                              : b->dens[b->cur].p + B.dens_off;
        if (to_host) {
            VFPS_CUDA(cudaMemcpyAsync(host + off, dev, cnt * 4,
                                      cudaMemcpyDeviceToHost, st));
        } else {
            VFPS_CUDA(cudaMemcpyAsync(dev, host + off, cnt * 4,
                                      cudaMemcpyHostToDevice, st));
        }
        off += cnt;
    }
}

bool contiguous(const vfps_batch* b)
{
    size_t off = 0;
    for (const auto& B : b->hb) {
        if (B.dens_off != off) {
            return false;
        }
        off += size_t(B.n) * B.n;
    }
    return off == b->cells;
}

void run_steps(vfps_batch* b, uint64_t nsteps)
{
    cudaStream_t st = b->ctx->stream;
    while (nsteps >= 8) {
        VFPS_CUDA(cudaGraphLaunch(b->graph8[b->cur], st));
        nsteps -= 8;
    }
    while (nsteps > 0) {
        VFPS_CUDA(cudaGraphLaunch(b->graph[b->cur], st));
        b->cur = 1 - b->cur;
        nsteps--;
    }
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
        run_steps(b, nsteps);
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
        copy_packed(b, wake, true, true, b->wake.p);
        VFPS_CUDA(cudaStreamSynchronize(b->ctx->stream));
    });
}

extern "C" int vfps_batch_potential_well(vfps_batch* b, uint32_t iterations,
                                         float mix, float* change)
{
    if (!b || iterations > 100000 || !(mix > 0.f) || mix > 1.f) {
        return VFPS_ERR_INVALID_ARGUMENT;
    }
    return bguard(b->ctx, [&] {
        cudaStream_t st = b->ctx->stream;
        const size_t smem = pw_smem(b->max_n).total * sizeof(float);
        VFPS_CUDA(cudaFuncSetAttribute(
            k_potential_well, cudaFuncAttributeMaxDynamicSharedMemorySize,
            static_cast<int>(smem)));
        DevBuf<float> ch(b->nb);
        VFPS_CUDA(cudaMemsetAsync(ch.p, 0, ch.bytes(), st));
        if (!b->coupled) {
            // bunches on their own: every iteration in one launch
            k_potential_well<<<b->nb, THREADS, smem, st>>>(
                b->bd.p, b->pw.p, b->pwtab.p, b->tabs.p, b->wt.p,
                b->beams.p, b->members.p, nullptr, nullptr,
                b->dens[b->cur].p, ch.p, b->ctx->d_status,
                static_cast<int>(iterations), mix, -1);
            VFPS_LAUNCHED();
        } else {
            // coupled beams: one launch per iteration, the members'
            // profiles of the previous pass in one buffer, the new ones
            // in the other
            DevBuf<float> pa(b->rows), pb(b->rows);
            VFPS_CUDA(cudaMemsetAsync(pa.p, 0, pa.bytes(), st));
            VFPS_CUDA(cudaMemsetAsync(pb.p, 0, pb.bytes(), st));
            for (uint32_t it = 0; it <= iterations; it++) {
                k_potential_well<<<b->nb, THREADS, smem, st>>>(
                    b->bd.p, b->pw.p, b->pwtab.p, b->tabs.p, b->wt.p,
                    b->beams.p, b->members.p, (it & 1) ? pb.p : pa.p,
                    (it & 1) ? pa.p : pb.p, b->dens[b->cur].p, ch.p,
                    b->ctx->d_status, static_cast<int>(iterations), mix,
                    static_cast<int>(it));
                VFPS_LAUNCHED();
            }
            VFPS_CUDA(cudaStreamSynchronize(st));   // before pa, pb go
        }
        // profiles and filling of the new state (as after an upload)
        project_all(b, b->cur);
        integrate_all(b, b->cur, 0);
        if (change) {
            VFPS_CUDA(cudaMemcpyAsync(change, ch.p, ch.bytes(),
                                      cudaMemcpyDeviceToHost, st));
        }
        VFPS_CUDA(cudaStreamSynchronize(st));
    });
}

extern "C" int vfps_batch_info(const vfps_batch* b, uint32_t* launches,
                               uint32_t* tile_rows)
{
    if (!b) {
        return VFPS_ERR_INVALID_ARGUMENT;
    }
    if (launches) {
        // wake kernel + one map kernel per chain present
        *launches = (b->wake_tc && b->tc_groups > 0) ? 2 : 1;
        for (int c = 0; c < TL_COUNT; c++) {
            *launches += b->htiles[c].empty() ? 0 : 1;
        }
    }
    if (tile_rows) {
        *tile_rows = static_cast<uint32_t>(b->tile_rows);
    }
    return VFPS_OK;
}

extern "C" int vfps_batch_kernel_tiles(const vfps_batch* b, uint32_t* tiles,
                                       uint32_t count)
{
    if (!b || (count && !tiles)) {
        return VFPS_ERR_INVALID_ARGUMENT;
    }
    const int order[] = {TL_RINGF, TL_RING, TL_RING4, TL_WIDE, TL_ROT};
    for (uint32_t k = 0; k < count && k < 5; k++) {
        tiles[k] = static_cast<uint32_t>(b->htiles[order[k]].size());
    }
    if (count > 0) {   // the fast ring kernel: every mesh size
        tiles[0] += static_cast<uint32_t>(b->htiles[TL_RINGF128].size()
                                          + b->htiles[TL_RINGF64].size()
                                          + b->htiles[TL_RINGF512].size()
                                          + b->htiles[TL_RINGF1024].size());
    }
    return VFPS_OK;
}

extern "C" int vfps_batch_kernel_times(vfps_batch* b, uint32_t nsteps,
                                       float* ms)
{
    if (!b || !ms || nsteps == 0) {
        return VFPS_ERR_INVALID_ARGUMENT;
    }
    return bguard(b->ctx, [&] {
        cudaEvent_t ev[4];
        for (auto& e : ev) {
            VFPS_CUDA(cudaEventCreate(&e));
        }
        double acc[3] = {0, 0, 0};
        for (uint32_t s = 0; s < nsteps; s++) {
            launch_step(b, b->cur, ev);
            b->cur = 1 - b->cur;
            VFPS_CUDA(cudaEventSynchronize(ev[3]));
            for (int k = 0; k < 3; k++) {
                float t = 0;
                VFPS_CUDA(cudaEventElapsedTime(&t, ev[k], ev[k + 1]));
                acc[k] += t;
            }
        }
        for (auto& e : ev) {
            cudaEventDestroy(e);
        }
        for (int k = 0; k < 3; k++) {
            ms[k] = static_cast<float>(acc[k] / nsteps);
        }
    });
}

extern "C" int vfps_batch_set_beams(vfps_batch* b, const uint32_t* beam,
                                    const uint32_t* bucket,
                                    uint32_t spacing_bins,
                                    const float* filling)
{
    if (!b || !beam || !bucket) {
        return VFPS_ERR_INVALID_ARGUMENT;
    }
    return bguard(b->ctx, [&] {
        const uint32_t nb = b->nb;
        std::map<uint32_t, std::vector<uint32_t>> groups;
        for (uint32_t i = 0; i < nb; i++) {
            if (beam[i] != 0) {
                groups[beam[i]].push_back(i);
            }
            VFPS_REQUIRE(!filling || filling[i] >= 0.f,
                         "fillings must not be negative");
        }
        std::vector<BeamDev> beams(nb);
        std::vector<uint32_t> members;
        bool coupled = false;
        for (uint32_t i = 0; i < nb; i++) {
            if (beam[i] == 0) {
                beams[i] = BeamDev{static_cast<uint32_t>(members.size()), 1u,
                                   static_cast<int32_t>(bucket[i]),
                                   spacing_bins};
                members.push_back(i);
            }
        }
        for (const auto& g : groups) {
            const auto& idx = g.second;
            const BDev& B0 = b->hb[idx[0]];
            for (uint32_t j : idx) {
                const BDev& B = b->hb[j];
                VFPS_REQUIRE(B.n == B0.n && B.wt_off == B0.wt_off
                                 && B.nmax == B0.nmax
                                 && (B.flags & F_WAKE) == (B0.flags & F_WAKE)
                                 && B.wakescale == B0.wakescale,
                             "bunches of one beam need the same mesh, "
                             "impedance and wake scaling");
            }
            const uint32_t first = static_cast<uint32_t>(members.size());
            for (uint32_t j : idx) {
                beams[j] = BeamDev{first, static_cast<uint32_t>(idx.size()),
                                   static_cast<int32_t>(bucket[j]),
                                   spacing_bins};
            }
            members.insert(members.end(), idx.begin(), idx.end());
            coupled = coupled || idx.size() > 1;
        }
        cudaStream_t st = b->ctx->stream;
        VFPS_CUDA(cudaStreamSynchronize(st));
        VFPS_CUDA(cudaMemcpy(b->beams.p, beams.data(), nb * sizeof(BeamDev),
                             cudaMemcpyHostToDevice));
        VFPS_CUDA(cudaMemcpy(b->members.p, members.data(),
                             nb * sizeof(uint32_t), cudaMemcpyHostToDevice));
        b->coupled = coupled;
        if (filling) {
            // the reference's filling_set: normalise every bunch to it
            // (src/PS/PhaseSpace.cpp:342-372)
            for (uint32_t i = 0; i < nb; i++) {
                b->hb[i].fillset = filling[i];
            }
            VFPS_CUDA(cudaMemcpy(b->bd.p, b->hb.data(), nb * sizeof(BDev),
                                 cudaMemcpyHostToDevice));
            project_all(b, b->cur);
            integrate_all(b, b->cur, 0);
            integrate_all(b, b->cur, 1);
            project_all(b, b->cur);
            integrate_all(b, b->cur, 0);
        }
        if (coupled && b->wake_tc) {
            b->wake_tc = 0;   // the tensor-core sum has no coupling
        }
        make_graphs(b);
        VFPS_CUDA(cudaStreamSynchronize(st));
    });
}

extern "C" int vfps_batch_set_csr(vfps_batch* b,
                                  const vfps_impedance* const* imps,
                                  uint32_t nimp, const int32_t* impedance,
                                  const double* fc, const double* freq_scale,
                                  uint32_t every, uint32_t capacity)
{
    if (!b || (every > 0 && (!imps || !impedance || !fc || !freq_scale
                             || capacity == 0))) {
        return VFPS_ERR_INVALID_ARGUMENT;
    }
    return bguard(b->ctx, [&] {
        cudaStream_t st = b->ctx->stream;
        VFPS_CUDA(cudaStreamSynchronize(st));
        const uint32_t nb = b->nb;
        std::vector<uint32_t> off(nb, NO_CSR);
        std::vector<float> tabs;
        if (every > 0) {
            // one K table per (impedance, mesh, dq, cutoff, frequency scale)
            std::map<std::string, uint32_t> seen;
            std::vector<std::vector<float>> re(nimp);
            for (uint32_t i = 0; i < nb; i++) {
                if (impedance[i] < 0) {
                    continue;
                }
                const uint32_t k = static_cast<uint32_t>(impedance[i]);
                VFPS_REQUIRE(k < nimp && imps[k], "bunch names a missing "
                             "CSR impedance");
                const vfps_impedance* z = imps[k];
                const BDev& B = b->hb[i];
                const size_t nmax = z->nfreqs;
                VFPS_REQUIRE(nmax >= B.n, "CSR impedance needs at least n "
                             "frequencies");
                const double dq = double(B.dq);
                std::string key(reinterpret_cast<const char*>(&k), 4);
                key.append(reinterpret_cast<const char*>(&B.n), 4);
                key.append(reinterpret_cast<const char*>(&B.dq), 4);
                key.append(reinterpret_cast<const char*>(&fc[i]), 8);
                key.append(reinterpret_cast<const char*>(&freq_scale[i]), 8);
                auto it = seen.find(key);
                if (it != seen.end()) {
                    off[i] = it->second;
                    continue;
                }
                if (re[k].empty()) {
                    std::vector<float> zz(2 * nmax);
                    VFPS_CUDA(cudaMemcpy(zz.data(), z->z.p, zz.size() * 4,
                                         cudaMemcpyDeviceToHost));
                    re[k].resize(nmax);
                    for (size_t f = 0; f < nmax; f++) {
                        re[k][f] = zz[2 * f];
                    }
                }
                // the frequency ruler 0 .. 1/dq over nmax points
                // (src/PS/ElectricField.cpp:133-184)
                const double df = (1.0 / dq) / double(nmax - 1);
                std::vector<double> c(nmax / 2 + 1);
                for (size_t f = 0; f <= nmax / 2; f++) {
                    double r = dq * dq;
                    if (fc[i] > 0) {
                        const double u = freq_scale[i] * df * double(f)
                                         / fc[i];
                        r *= 1.0 - std::exp(-u * u);
                    }
                    c[f] = r * double(re[k][f]);
                }
                const uint32_t n = B.n;
                off[i] = static_cast<uint32_t>(tabs.size());
                seen.emplace(key, off[i]);
                const double two_pi = 6.283185307179586476925286766559;
                for (int64_t d = 1 - int64_t(n); d < int64_t(n); d++) {
                    double sum = 0;
                    for (size_t f = 0; f <= nmax / 2; f++) {
                        // the angle reduced exactly before the cosine
                        const int64_t r = (d * int64_t(f)) % int64_t(nmax);
                        sum += c[f] * std::cos(two_pi * double(r)
                                               / double(nmax));
                    }
                    tabs.push_back(static_cast<float>(df * sum));
                }
            }
            b->csrk.alloc(std::max<size_t>(tabs.size(), 1));
            if (!tabs.empty()) {
                VFPS_CUDA(cudaMemcpy(b->csrk.p, tabs.data(), tabs.size() * 4,
                                     cudaMemcpyHostToDevice));
            }
            b->csrpow.alloc(size_t(capacity) * nb);
            VFPS_CUDA(cudaMemset(b->csrpow.p, 0, b->csrpow.bytes()));
            b->csrsteps.alloc(capacity);
            VFPS_CUDA(cudaMemset(b->csrsteps.p, 0xff, b->csrsteps.bytes()));
        }
        VFPS_CUDA(cudaMemcpy(b->csroff.p, off.data(), nb * 4,
                             cudaMemcpyHostToDevice));
        b->csr_every = every;
        b->csr_cap = every > 0 ? capacity : 0;
        make_graphs(b);
        VFPS_CUDA(cudaStreamSynchronize(st));
    });
}

extern "C" int vfps_batch_get_csr(vfps_batch* b, float* power,
                                  uint64_t* steps)
{
    if (!b || !power || !steps || b->csr_every == 0) {
        return VFPS_ERR_INVALID_ARGUMENT;
    }
    return bguard(b->ctx, [&] {
        cudaStream_t st = b->ctx->stream;
        VFPS_CUDA(cudaMemcpyAsync(power, b->csrpow.p,
                                  size_t(b->csr_cap) * b->nb * 4,
                                  cudaMemcpyDeviceToHost, st));
        VFPS_CUDA(cudaMemcpyAsync(steps, b->csrsteps.p,
                                  size_t(b->csr_cap) * 8,
                                  cudaMemcpyDeviceToHost, st));
        VFPS_CUDA(cudaStreamSynchronize(st));
    });
}

extern "C" int vfps_batch_set_wake_mode(vfps_batch* b, int mode)
{
    if (!b || (mode != 0 && mode != 1)
        || (mode == 1 && (b->coupled || !b->tc_ok))) {
        return VFPS_ERR_INVALID_ARGUMENT;
    }
    return bguard(b->ctx, [&] {
        VFPS_CUDA(cudaStreamSynchronize(b->ctx->stream));
        b->wake_tc = mode;
        make_graphs(b);
    });
}

extern "C" int vfps_batch_destroy(vfps_batch* b)
{
    if (!b) {
        return VFPS_OK;
    }
    cudaSetDevice(b->device);
    destroy_graphs(b);
    if (b->fork) {
        cudaEventDestroy(b->fork);
    }
    if (b->join) {
        cudaEventDestroy(b->join);
    }
    if (b->side) {
        cudaStreamDestroy(b->side);
    }
    delete b;
    return VFPS_OK;
}
