// PhaseSpace kernels: Gaussian start, x/y projections, integral,
// normalisation and moments (src/PS/PhaseSpace.cpp:200-372,457-501).
// Sums feeding the wake and the charge integral accumulate in FP64; the
// per-lane partial sums of at most 8 cells stay in FP32 so that the FP64
// pipe (slow on GB300) sees n/256 additions per row.
#include "vfps_internal.cuh"

namespace vfps {
namespace {

__global__ void k_fill_gaussian(float* __restrict__ data,
                                const float* __restrict__ gx,
                                const float* __restrict__ gy, uint32_t nb,
                                uint32_t n)
{
    const size_t nxy = size_t(n) * n;
    const size_t total = nxy * nb;
    for (size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x; i < total;
         i += size_t(gridDim.x) * blockDim.x) {
        const size_t c = i % nxy;
        data[i] = __fmul_rn(gx[c / n], gy[c % n]);
    }
}

// one warp per row: proj[row] = sum_y data[row][y] ws[y]
__global__ void k_project_x(const float* __restrict__ data,
                            const float* __restrict__ ws,
                            float* __restrict__ proj,
                            double* __restrict__ proj64, uint32_t rows,
                            uint32_t n)
{
    const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (warp >= rows) {
        return;
    }
    const float* r = data + size_t(warp) * n;
    double acc = 0;
    float part = 0;
    int cnt = 0;
    for (uint32_t y = lane; y < n; y += 32) {
        part = fmaf(r[y], ws[y], part);
        if (++cnt == 8) {
            acc += part;
            part = 0;
            cnt = 0;
        }
    }
    acc += part;
    acc = dev::warp_sum(acc);
    if (lane == 0) {
        proj[warp] = static_cast<float>(acc);
        if (proj64) {
            proj64[warp] = acc;
        }
    }
}

// thread per (bunch, y): proj[b][y] = sum_x data[b][x][y] ws[x]
__global__ void k_project_y(const float* __restrict__ data,
                            const float* __restrict__ ws,
                            float* __restrict__ proj, uint32_t n)
{
    const uint32_t y = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t b = blockIdx.y;
    if (y >= n) {
        return;
    }
    const float* d = data + size_t(b) * n * n + y;
    double acc = 0;
    float part = 0;
    for (uint32_t x = 0; x < n; x++) {
        part = fmaf(d[size_t(x) * n], ws[x], part);
        if ((x & 7) == 7) {
            acc += part;
            part = 0;
        }
    }
    acc += part;
    proj[size_t(b) * n + y] = static_cast<float>(acc);
}

// single block: filling[b] = sum_x proj64[b][x] ws[x]; filling[nb] = total
__global__ void k_integrate(const double* __restrict__ proj64,
                            const float* __restrict__ ws,
                            const float* __restrict__ fillset,
                            double* __restrict__ filling, uint32_t nb,
                            uint32_t n, int* status)
{
    __shared__ double scratch[32];
    double total = 0;
    for (uint32_t b = 0; b < nb; b++) {
        double acc = 0;
        for (uint32_t x = threadIdx.x; x < n; x += blockDim.x) {
            acc += proj64[size_t(b) * n + x] * double(ws[x]);
        }
        acc = dev::block_sum(acc, scratch);
        if (threadIdx.x == 0) {
            filling[b] = acc;
            total += acc;
            // watchdog: a populated bunch must keep a finite, positive charge
            if (fillset[b] > 0 && !(acc > 0) && status) {
                atomicCAS(status, 0, VFPS_ERR_NUMERIC);
            }
        }
    }
    if (threadIdx.x == 0) {
        filling[nb] = total;
    }
}

__global__ void k_normalize(float* __restrict__ data,
                            const float* __restrict__ fillset,
                            const double* __restrict__ filling, uint32_t nb,
                            size_t nxy)
{
    const size_t total = nxy * nb;
    for (size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x; i < total;
         i += size_t(gridDim.x) * blockDim.x) {
        const uint32_t b = static_cast<uint32_t>(i / nxy);
        const float fs = fillset[b];
        data[i] = fs > 0 ? data[i] * static_cast<float>(double(fs) / filling[b])
                         : 0.f;
    }
}

// one block per bunch: average, variance, rms of one axis
__global__ void k_moments(const float* __restrict__ proj,
                          const float* __restrict__ axisv,
                          const float* __restrict__ fillset,
                          const double* __restrict__ filling, float delta,
                          uint32_t nb, uint32_t n, float* __restrict__ mom)
{
    __shared__ double scratch[32];
    __shared__ double avg_s;
    const uint32_t b = blockIdx.x;
    const bool pop = fillset[b] > 0;
    double a = 0;
    for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) {
        a += double(proj[size_t(b) * n + i]) * double(axisv[i]);
    }
    a = dev::block_sum(a, scratch);
    if (threadIdx.x == 0) {
        avg_s = pop ? a * double(delta) / filling[b] : 0.0;
    }
    __syncthreads();
    const double avg = avg_s;
    double v = 0;
    for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) {
        const double d = double(axisv[i]) - avg;
        v += double(proj[size_t(b) * n + i]) * d * d;
    }
    v = dev::block_sum(v, scratch);
    if (threadIdx.x == 0) {
        const double var = pop ? v * double(delta) / filling[b] : 0.0;
        mom[0 * nb + b] = static_cast<float>(avg);
        mom[1 * nb + b] = static_cast<float>(var);
        mom[2 * nb + b] = static_cast<float>(sqrt(var));
    }
}

int grid_for(size_t total, int threads)
{
    const size_t blocks = (total + threads - 1) / threads;
    return static_cast<int>(blocks < 65535 * 16 ? blocks : 65535 * 16);
}

}  // namespace

void launch_fill_gaussian(vfps_ps* ps, const float* gx, const float* gy)
{
    const size_t total = size_t(ps->nb) * ps->n * ps->n;
    k_fill_gaussian<<<grid_for(total, 256), 256, 0, ps->ctx->stream>>>(
        ps->data.p, gx, gy, ps->nb, ps->n);
    VFPS_LAUNCHED();
}

void launch_project_x(vfps_ps* ps, const float* data)
{
    const uint32_t rows = ps->nb * ps->n;
    const int threads = 256;
    const int blocks = (rows * 32 + threads - 1) / threads;
    k_project_x<<<blocks, threads, 0, ps->ctx->stream>>>(
        data ? data : ps->data.p, ps->ws.p, ps->proj[0].p, ps->proj64.p, rows,
        ps->n);
    VFPS_LAUNCHED();
}

void launch_project_y(vfps_ps* ps)
{
    dim3 grid((ps->n + 127) / 128, ps->nb);
    k_project_y<<<grid, 128, 0, ps->ctx->stream>>>(ps->data.p, ps->ws.p,
                                                   ps->proj[1].p, ps->n);
    VFPS_LAUNCHED();
}

void launch_integrate(vfps_ps* ps)
{
    k_integrate<<<1, 256, 0, ps->ctx->stream>>>(ps->proj64.p, ps->ws.p,
                                                ps->fillset.p, ps->filling.p,
                                                ps->nb, ps->n,
                                                ps->ctx->d_status);
    VFPS_LAUNCHED();
}

void launch_normalize(vfps_ps* ps)
{
    const size_t nxy = size_t(ps->n) * ps->n;
    k_normalize<<<grid_for(nxy * ps->nb, 256), 256, 0, ps->ctx->stream>>>(
        ps->data.p, ps->fillset.p, ps->filling.p, ps->nb, nxy);
    VFPS_LAUNCHED();
}

void launch_moments(vfps_ps* ps, int axis)
{
    k_moments<<<ps->nb, 256, 0, ps->ctx->stream>>>(
        ps->proj[axis].p, ps->axisv[axis].p, ps->fillset.p, ps->filling.p,
        ps->ax[axis].delta, ps->nb, ps->n,
        ps->moments.p + size_t(axis) * 3 * ps->nb);
    VFPS_LAUNCHED();
}

}  // namespace vfps
