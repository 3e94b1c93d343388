// Plain (one map per launch) SourceMap kernels.  Weights are evaluated in
// registers from the source coordinate -- the reference's per-cell
// (index, weight) tables (8 B per tap) are never materialised.
//
//  k_rotation  RotationMap::genHInfo + apply (src/SM/RotationMap.cpp:97-260)
//  k_kick_y    KickMap y-kick, one CTA per mesh row (src/SM/KickMap.cpp:244-266)
//  k_kick_x    KickMap x-kick (src/SM/KickMap.cpp:221-242)
//  k_fp        FokkerPlanckMap::apply (src/SM/FokkerPlanckMap.cpp:170-213)
#include <algorithm>
#include <cfloat>

#include "vfps_internal.cuh"

namespace vfps {
namespace {

using namespace dev;

__global__ void k_rotation(const float* __restrict__ in,
                           float* __restrict__ out, uint32_t n,
                           const float* __restrict__ qv,
                           const float* __restrict__ pv, float dq, float dp,
                           float zbq, float zbp, float cs, float sn, int it,
                           int clamp)
{
    const uint32_t y0 = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t x0 = blockIdx.y;
    if (y0 >= n) {
        return;
    }
    const size_t nxy = size_t(n) * n;
    const float* src = in + blockIdx.z * nxy;
    const float q = qv[x0], p = pv[y0];
    const float x1r = fadd(fdiv(fsub(fmul(cs, q), fmul(sn, p)), dq), zbq);
    const float y1r = fadd(fdiv(fadd(fmul(sn, q), fmul(cs, p)), dp), zbp);
    int x1 = 0, y1 = 0;
    float xf, yf;
    const bool okx = base_index(x1r, n, &x1, &xf);
    const bool oky = base_index(y1r, n, &y1, &yf);
    const bool ok = okx && oky;
    float value = 0.f;
    float icq[4], icp[4];
    const int h = (it - 1) / 2;
    if (ok) {
        coefficients(icq, xf, it);
        coefficients(icp, yf, it);
        for (int i1 = 0; i1 < it; i1++) {
            const int i0 = x1 + i1 - h;
            for (int j1 = 0; j1 < it; j1++) {
                const int j0 = y1 + j1 - h;
                if (i0 >= 0 && i0 < int(n) && j0 >= 0 && j0 < int(n)) {
                    value = fadd(value, fmul(__ldg(src + size_t(i0) * n + j0),
                                             fmul(icq[i1], icp[j1])));
                }
            }
        }
    }
    if (clamp) {
        // src/SM/RotationMap.cpp:159-172: range of the 2x2 nearest taps,
        // starting from FLT_MIN / FLT_MAX; taps off the mesh read cell 0.
        float ceil_v = FLT_MIN, flor_v = FLT_MAX;
        for (int i1 = 1; i1 <= 2; i1++) {
            for (int j1 = 1; j1 <= 2; j1++) {
                const int i0 = x1 + i1 - h, j0 = y1 + j1 - h;
                const bool in_mesh = ok && i0 >= 0 && i0 < int(n) && j0 >= 0
                                     && j0 < int(n);
                const float v = __ldg(src + (in_mesh ? size_t(i0) * n + j0 : 0));
                ceil_v = (ceil_v < v) ? v : ceil_v;
                flor_v = (v < flor_v) ? v : flor_v;
            }
        }
        const float t = (value < ceil_v) ? value : ceil_v;
        value = (t < flor_v) ? flor_v : t;
    }
    out[blockIdx.z * nxy + size_t(x0) * n + y0] = value;
}

// The reference's CPU KickMap never clamps (its interpol_clamp flag only
// prints a notice, src/SM/KickMap.cpp:42-44), so the kick kernels follow
// that path and take no clamp argument.

// one CTA per (bunch, row x); offsets[b*n + x] in mesh units
__global__ void k_kick_y(const float* __restrict__ in, float* __restrict__ out,
                         const float* __restrict__ offsets, uint32_t n, int it)
{
    const uint32_t row = blockIdx.x;
    const KickStencil s = kick_stencil(offsets[row], n, it);
    const float* src = in + size_t(row) * n;
    float* dst = out + size_t(row) * n;
    for (uint32_t y = threadIdx.x; y < n; y += blockDim.x) {
        float value = 0.f;
        for (int j = 0; j < it; j++) {
            const int ys = int(y) + s.shift[j];
            if (s.valid[j] && ys >= 0 && ys < int(n)) {
                value = fadd(value, fmul(__ldg(src + ys), s.w[j]));
            }
        }
        dst[y] = value;
    }
}

// thread per cell; offsets[y] shared by all bunches
__global__ void k_kick_x(const float* __restrict__ in, float* __restrict__ out,
                         const float* __restrict__ offsets, uint32_t n, int it)
{
    const uint32_t y = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t x = blockIdx.y;
    if (y >= n) {
        return;
    }
    const size_t nxy = size_t(n) * n;
    const float* src = in + blockIdx.z * nxy;
    const KickStencil s = kick_stencil(offsets[y], n, it);
    float value = 0.f;
    for (int j = 0; j < it; j++) {
        const int xs = int(x) + s.shift[j];
        if (s.valid[j] && xs >= 0 && xs < int(n)) {
            value = fadd(value, fmul(__ldg(src + size_t(xs) * n + y), s.w[j]));
        }
    }
    out[blockIdx.z * nxy + size_t(x) * n + y] = value;
}

// thread per cell; stencil table idx/w [n][ip] shared by every row
__global__ void k_fp(const float* __restrict__ in, float* __restrict__ out,
                     const uint32_t* __restrict__ idx,
                     const float* __restrict__ w, uint32_t n, int ip)
{
    const uint32_t y = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t x = blockIdx.y;
    if (y >= n) {
        return;
    }
    const size_t row = (blockIdx.z * size_t(n) + x) * n;
    float value = 0.f;
    for (int j = 0; j < ip; j++) {
        value = fadd(value, fmul(__ldg(in + row + idx[y * ip + j]),
                                 w[y * ip + j]));
    }
    out[row + y] = value;
}

// ------------------------------------------------ row-sweep forms
// Meshes whose side is a multiple of 4 (up to PLAIN_V4_MAX) take these
// instead of the thread-per-cell kernels above: 16-byte row sweeps in and
// out, the stencils computed once per thread for its 4 columns and kept
// in registers, and rows staged in shared memory where a stencil reads
// along the row.  Every output is the same sum in the same order as the
// kernels above; a tap outside the mesh reads a zero pad instead of being
// skipped, and adds fmul(0, w) = +-0 (an exact no-op, because the sum is
// never -0).

// one output group: taps j < it of the aligned window v (AL: offset of
// the first tap of the first output)
template <int AL>
__device__ __forceinline__ float4 kick_row4(const float4 (&v4)[3],
                                            const float (&w)[4], int it)
{
    const float v[12] = {v4[0].x, v4[0].y, v4[0].z, v4[0].w,
                         v4[1].x, v4[1].y, v4[1].z, v4[1].w,
                         v4[2].x, v4[2].y, v4[2].z, v4[2].w};
    float o[4];
#pragma unroll
    for (int c = 0; c < 4; c++) {
        float value = 0.f;
#pragma unroll
        for (int j = 0; j < 4; j++) {
            if (j < it) {
                value = fadd(value, fmul(v[AL + c + j], w[j]));
            }
        }
        o[c] = value;
    }
    return make_float4(o[0], o[1], o[2], o[3]);
}

// y-kick, one CTA per (bunch, row): the row in shared memory between zero
// pads of kick_pad(n) floats (a valid tap lies at most n/2 + 3 columns
// away), the stencil uniform over the row, 4 outputs per thread from 3
// aligned 16-byte reads (the window's alignment is the same for the whole
// row)
__host__ __device__ inline int kick_pad(uint32_t n)
{
    return int(((n / 2 + 3) & ~3u) + 16);
}

__global__ void k_kick_y4(const float* __restrict__ in,
                          float* __restrict__ out,
                          const float* __restrict__ offsets, uint32_t n,
                          int it)
{
    extern __shared__ float4 row4[];
    const uint32_t row = blockIdx.x;
    const KickStencil s = kick_stencil(offsets[row], n, it);
    const int pad4 = kick_pad(n) / 4, n4 = int(n / 4);
    const float4* src = reinterpret_cast<const float4*>(in + size_t(row) * n);
    float4* dst = reinterpret_cast<float4*>(out + size_t(row) * n);
    const float4 z = make_float4(0.f, 0.f, 0.f, 0.f);
    const bool any = s.valid[0] || s.valid[1] || s.valid[2] || s.valid[3];
    if (!any) {   // no tap inside the mesh: the row is zero
        for (int i = threadIdx.x; i < n4; i += blockDim.x) {
            dst[i] = z;
        }
        return;
    }
    for (int i = threadIdx.x; i < 2 * pad4 + n4; i += blockDim.x) {
        const int k = i - pad4;
        row4[i] = (k >= 0 && k < n4) ? __ldg(src + k) : z;
    }
    __syncthreads();
    // shift[0] lies in [-n/2 - 3, n/2): every window inside the pads
    const int s0 = s.shift[0];
    const int al = s0 & 3;
    const int b4 = pad4 + ((s0 - al) >> 2);
    for (int i = threadIdx.x; i < n4; i += blockDim.x) {
        const float4 v[3] = {row4[b4 + i], row4[b4 + i + 1],
                             row4[b4 + i + 2]};
        float4 o;
        switch (al) {
        case 0: o = kick_row4<0>(v, s.w, it); break;
        case 1: o = kick_row4<1>(v, s.w, it); break;
        case 2: o = kick_row4<2>(v, s.w, it); break;
        default: o = kick_row4<3>(v, s.w, it); break;
        }
        dst[i] = o;
    }
}

// the x-kick's stencils of every column, tap-major: shift[j][y], w[j][y]
// (the same function the kernels evaluate, computed once per set of
// offsets)
__global__ void k_kick_table(const float* __restrict__ offsets, uint32_t n,
                             int it, int* __restrict__ shift,
                             float* __restrict__ w)
{
    const uint32_t y = blockIdx.x * blockDim.x + threadIdx.x;
    if (y >= n) {
        return;
    }
    const KickStencil s = kick_stencil(offsets[y], n, it);
#pragma unroll
    for (int j = 0; j < 4; j++) {
        shift[j * n + y] = s.shift[j];
        w[j * n + y] = s.w[j];
    }
}

// x-kick: a CTA per block of rows of one bunch; each thread owns 4
// columns (their stencils, one per column, loaded from the table in
// 16-byte words) and sweeps the rows with 16-byte reads where the 4
// columns take the same shifts, column by column otherwise
__global__ void k_kick_x4(const float* __restrict__ in,
                          float* __restrict__ out,
                          const int* __restrict__ shtab,
                          const float* __restrict__ wtab, uint32_t n,
                          int it, int rows)
{
    const int n4 = int(n / 4);
    const size_t nxy = size_t(n) * n;
    const float* src = in + blockIdx.y * nxy;
    float* dst = out + blockIdx.y * nxy;
    const int xa = blockIdx.x * rows;
    const int xe = min(int(n), xa + rows);
    for (int g = threadIdx.x; g < n4; g += blockDim.x) {
        KickStencil s[4];
#pragma unroll
        for (int j = 0; j < 4; j++) {
            const int4 sh = __ldg(reinterpret_cast<const int4*>(
                                      shtab + size_t(j) * n) + g);
            const float4 wv = __ldg(reinterpret_cast<const float4*>(
                                        wtab + size_t(j) * n) + g);
            s[0].shift[j] = sh.x;
            s[1].shift[j] = sh.y;
            s[2].shift[j] = sh.z;
            s[3].shift[j] = sh.w;
            s[0].w[j] = wv.x;
            s[1].w[j] = wv.y;
            s[2].w[j] = wv.z;
            s[3].w[j] = wv.w;
        }
        bool same = true;
#pragma unroll
        for (int j = 0; j < 4; j++) {
            same = same && s[1].shift[j] == s[0].shift[j]
                   && s[2].shift[j] == s[0].shift[j]
                   && s[3].shift[j] == s[0].shift[j];
        }
        for (int x = xa; x < xe; x++) {
            float o[4] = {0.f, 0.f, 0.f, 0.f};
            if (same) {
#pragma unroll
                for (int j = 0; j < 4; j++) {
                    const int xs = x + s[0].shift[j];
                    if (j < it && xs >= 0 && xs < int(n)) {
                        const float4 v = __ldg(reinterpret_cast<const float4*>(
                            src + size_t(xs) * n) + g);
                        o[0] = fadd(o[0], fmul(v.x, s[0].w[j]));
                        o[1] = fadd(o[1], fmul(v.y, s[1].w[j]));
                        o[2] = fadd(o[2], fmul(v.z, s[2].w[j]));
                        o[3] = fadd(o[3], fmul(v.w, s[3].w[j]));
                    }
                }
            } else {
#pragma unroll
                for (int c = 0; c < 4; c++) {
#pragma unroll
                    for (int j = 0; j < 4; j++) {
                        const int xs = x + s[c].shift[j];
                        if (j < it && xs >= 0 && xs < int(n)) {
                            o[c] = fadd(o[c], fmul(__ldg(src + size_t(xs) * n
                                                         + 4 * g + c),
                                                   s[c].w[j]));
                        }
                    }
                }
            }
            reinterpret_cast<float4*>(dst + size_t(x) * n)[g] =
                make_float4(o[0], o[1], o[2], o[3]);
        }
    }
}

// Fokker-Planck: a CTA per block of rows of one bunch, the rows staged in
// shared memory by 16-byte reads; each thread owns 4 columns, whose
// stencils (ip <= 4 taps: column index and weight, tap-major tables
// [4][n]) it reads with 16-byte loads before the rows arrive
__global__ void k_fp4(const float* __restrict__ in, float* __restrict__ out,
                      const uint32_t* __restrict__ idx4,
                      const float* __restrict__ w4, uint32_t n, int ip,
                      int rows)
{
    extern __shared__ float4 blk4[];
    const float* blk = reinterpret_cast<const float*>(blk4);
    const int n4 = int(n / 4);
    const int xa = blockIdx.x * rows;
    const int nr = min(int(n) - xa, rows);
    const size_t base = (blockIdx.y * size_t(n) + xa) * n;
    // this thread's first group's stencils (one group per thread when
    // n <= 1024)
    uint4 ixv[4];
    float4 wtv[4];
    const int g0 = threadIdx.x < n4 ? threadIdx.x : 0;
#pragma unroll
    for (int j = 0; j < 4; j++) {
        ixv[j] = __ldg(reinterpret_cast<const uint4*>(idx4 + size_t(j) * n)
                       + g0);
        wtv[j] = __ldg(reinterpret_cast<const float4*>(w4 + size_t(j) * n)
                       + g0);
    }
    const float4* src = reinterpret_cast<const float4*>(in + base);
    for (int i = threadIdx.x; i < nr * n4; i += blockDim.x) {
        blk4[i] = __ldg(src + i);
    }
    __syncthreads();
    float4* dst = reinterpret_cast<float4*>(out + base);
    for (int g = threadIdx.x; g < n4; g += blockDim.x) {
        if (g != g0) {
#pragma unroll
            for (int j = 0; j < 4; j++) {
                ixv[j] = __ldg(reinterpret_cast<const uint4*>(
                                   idx4 + size_t(j) * n) + g);
                wtv[j] = __ldg(reinterpret_cast<const float4*>(
                                   w4 + size_t(j) * n) + g);
            }
        }
        uint32_t ix[4][4];
        float wt[4][4];
#pragma unroll
        for (int j = 0; j < 4; j++) {
            ix[0][j] = ixv[j].x;
            ix[1][j] = ixv[j].y;
            ix[2][j] = ixv[j].z;
            ix[3][j] = ixv[j].w;
            wt[0][j] = wtv[j].x;
            wt[1][j] = wtv[j].y;
            wt[2][j] = wtv[j].z;
            wt[3][j] = wtv[j].w;
        }
        for (int r = 0; r < nr; r++) {
            const float* rowp = blk + size_t(r) * n;
            float o[4];
#pragma unroll
            for (int c = 0; c < 4; c++) {
                float value = 0.f;
#pragma unroll
                for (int j = 0; j < 4; j++) {
                    if (j < ip) {
                        value = fadd(value, fmul(rowp[ix[c][j]], wt[c][j]));
                    }
                }
                o[c] = value;
            }
            dst[size_t(r) * n4 + g] = make_float4(o[0], o[1], o[2], o[3]);
        }
    }
}

// DynamicRFKickMap::apply (src/SM/DynamicRFKickMap.cpp:79-109 and
// RFKickMap::_calcKick, src/SM/RFKickMap.cpp:59-83): the modulation of
// apply number `step` -- phase = syncphase + N(0,1) phasenoise + modampl
// sin(2 pi modtimeincrement step), amplitude = 1 + N(0,1) amplnoise, the
// normals drawn by Box-Muller from Philox(step, seed) -- and the RF kick
// offsets of every row with it (identical for every bunch).
__global__ void k_dynrf(DynRf d, uint64_t step, const float* __restrict__ q,
                        float xcenter, float dq, float dp, float pscale,
                        uint32_t n, uint32_t nb, float* __restrict__ offset,
                        float* __restrict__ log)
{
    const uint32_t ctr[4] = {uint32_t(step), uint32_t(step >> 32), 0u, 0u};
    const uint32_t key[2] = {d.seed, 0x5EED0001u};
    uint32_t r[4];
    philox4x32_10(ctr, key, r);
    // uniforms in (0, 1]
    const float u1 = (float(r[0] >> 8) + 1.f) * (1.f / 16777216.f);
    const float u2 = (float(r[1] >> 8) + 1.f) * (1.f / 16777216.f);
    const float rad = sqrtf(-2.f * logf(u1));
    float sn, cs;
    sincospif(2.f * u2, &sn, &cs);
    const float n1 = rad * cs, n2 = rad * sn;
    const float mod = d.modampl
        * static_cast<float>(sin(d.modtimedelta * double(step)));
    const float phase = d.syncphase + n1 * d.phasenoise + mod;
    const float ampl = 1.f + n2 * d.amplnoise;
    if (blockIdx.x == 0 && threadIdx.x == 0 && log) {
        log[0] = phase;
        log[1] = ampl;
    }
    for (uint32_t x = blockIdx.x * blockDim.x + threadIdx.x; x < n;
         x += gridDim.x * blockDim.x) {
        float o;
        if (d.linear) {
            const float phaseoffs = d.syncphase - phase;
            const float ta = tanf(d.angle);
            o = __fmul_rn(ta, __fsub_rn(xcenter, float(x)));
            o = __fadd_rn(o, __fdiv_rn(__fdiv_rn(__fmul_rn(ta, phaseoffs),
                                                 d.bl2phase), dq));
            o = __fmul_rn(o, ampl);
        } else {
            const float arg = __fadd_rn(__fmul_rn(q[x], d.bl2phase), phase);
            const float v = __fadd_rn(__fmul_rn(-ampl * d.v_rf, sinf(arg)),
                                      d.v0);
            o = __fdiv_rn(__fdiv_rn(__fmul_rn(d.revolutionpart, v), dp),
                          pscale);
        }
        for (uint32_t b = 0; b < nb; b++) {
            offset[size_t(b) * n + x] = o;
        }
    }
}

}  // namespace

void launch_dynrf(vfps_map* m)
{
    const vfps_ps* in = m->in;
    const uint32_t n = in->n;
    float* log = m->dyn_step < m->dyn_cap ? m->dyn_log.p + 2 * m->dyn_step
                                          : nullptr;
    k_dynrf<<<(n + 127) / 128, 128, 0, in->ctx->stream>>>(
        m->dyn, m->dyn_step, m->axis_q.p, in->ax[0].zerobin, in->ax[0].delta,
        in->ax[1].delta, in->ax[1].scale, n, in->nb, m->offset.p, log);
    VFPS_LAUNCHED();
    m->dyn_step++;
}

void launch_rotation(const vfps_map* m)
{
    const vfps_ps* in = m->in;
    const uint32_t n = in->n;
    dim3 grid((n + 127) / 128, n, in->nb);
    k_rotation<<<grid, 128, 0, in->ctx->stream>>>(
        in->data.p, m->out->data.p, n, in->axisv[0].p, in->axisv[1].p,
        in->ax[0].delta, in->ax[1].delta, in->ax[0].zerobin, in->ax[1].zerobin,
        m->cs, m->sn, m->it, m->clamp);
    VFPS_LAUNCHED();
}

// the row-sweep forms: sides that are a multiple of 4, up to this size
// (shared memory of the y-kick's padded row and of k_fp4's rows: 32 KiB at
// most, within the default limit)
constexpr uint32_t PLAIN_V4_MAX = 4096;

bool plain_v4(uint32_t n)
{
    return n % 4 == 0 && n <= PLAIN_V4_MAX;
}

// rows per CTA of k_kick_x4 and k_fp4: one, unless the meshes give more
// than 4 CTAs per SM (152 SMs) with one; at most 8
int plain_rows(uint32_t n, uint32_t nb)
{
    const size_t per = size_t(n) * nb / (4 * 152);
    return int(std::max<size_t>(1, std::min<size_t>(8, per)));
}

void launch_kick(const vfps_map* m, const float* offset)
{
    const vfps_ps* in = m->in;
    const uint32_t n = in->n;
    const int t4 = int(std::min<uint32_t>(256, ((n / 4 + 31) / 32) * 32));
    const bool v4 = plain_v4(n) && !m->cells;
    if (v4 && m->axis == VFPS_AXIS_Y) {
        const size_t smem = (2 * size_t(kick_pad(n)) + n) * sizeof(float);
        k_kick_y4<<<in->nb * n, t4, smem, in->ctx->stream>>>(
            in->data.p, m->out->data.p, offset, n, m->it);
    } else if (v4) {
        if (!m->xtab_valid) {
            m->xshift.alloc(size_t(4) * n);
            m->xweight.alloc(size_t(4) * n);
            k_kick_table<<<(n + 127) / 128, 128, 0, in->ctx->stream>>>(
                offset, n, m->it, m->xshift.p, m->xweight.p);
            VFPS_LAUNCHED();
            m->xtab_valid = true;
        }
        const int rows = plain_rows(n, in->nb);
        dim3 grid((n + rows - 1) / rows, in->nb);
        k_kick_x4<<<grid, t4, 0, in->ctx->stream>>>(
            in->data.p, m->out->data.p, m->xshift.p, m->xweight.p, n, m->it,
            rows);
    } else if (m->axis == VFPS_AXIS_Y) {
        const int threads = n >= 256 ? 256 : ((n + 31) / 32) * 32;
        k_kick_y<<<in->nb * n, threads, 0, in->ctx->stream>>>(
            in->data.p, m->out->data.p, offset, n, m->it);
    } else {
        dim3 grid((n + 127) / 128, n, in->nb);
        k_kick_x<<<grid, 128, 0, in->ctx->stream>>>(
            in->data.p, m->out->data.p, offset, n, m->it);
    }
    VFPS_LAUNCHED();
}

void launch_fp(const vfps_map* m)
{
    const vfps_ps* in = m->in;
    const uint32_t n = in->n;
    if (plain_v4(n) && m->ip <= 4 && !m->cells) {
        // at most 8 rows of up to 1024 floats (32 KiB), fewer for wider
        // meshes
        const int rows = std::min(plain_rows(n, in->nb),
                                  int(std::max<uint32_t>(1, 8192 / n)));
        const int t4 = int(std::min<uint32_t>(256, ((n / 4 + 31) / 32) * 32));
        dim3 grid((n + rows - 1) / rows, in->nb);
        k_fp4<<<grid, t4, size_t(rows) * n * sizeof(float),
                in->ctx->stream>>>(in->data.p, m->out->data.p,
                                   m->fp_idx4.p, m->fp_w4.p, n, m->ip, rows);
        VFPS_LAUNCHED();
        return;
    }
    dim3 grid((n + 127) / 128, n, in->nb);
    k_fp<<<grid, 128, 0, in->ctx->stream>>>(in->data.p, m->out->data.p,
                                            m->fp_idx.p, m->fp_w.p, n, m->ip);
    VFPS_LAUNCHED();
}

}  // namespace vfps
