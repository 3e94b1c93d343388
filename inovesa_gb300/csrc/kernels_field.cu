// ElectricField kernels (src/PS/ElectricField.cpp:133-263).
//
// The reference computes the wake potential as c2r(Z * r2c(padded
// profile)) with unnormalised FFTW transforms, multiplying only the bins
// below nmax/2.  That is a circular convolution of the padded profile with
//   w[d] = Re Z_0 + 2 sum_{k=1}^{floor(nmax/2)-1} Re(Z_k e^{+2 pi i k d/nmax}),
// so the wake is the Toeplitz product  wake_b[x] = s sum_{b',m}
// proj_b'[m] w[(pos_b + x - pos_b' - m) mod nmax]  with s = wakescaling/nmax.
// w is built once per field in FP64; no FFT runs per step.
#include "vfps_internal.cuh"

namespace vfps {
namespace {

// w[d] in FP64 from the float impedance table, rounded to float at the end
__global__ void k_wake_table(const float* __restrict__ z, uint32_t nmax,
                             float* __restrict__ wtab)
{
    const uint32_t d = blockIdx.x * blockDim.x + threadIdx.x;
    if (d >= nmax) {
        return;
    }
    double acc = double(z[0]);
    const uint32_t kmax = nmax / 2;  // bins k < nmax/2 are multiplied
    double part = 0;
    for (uint32_t k = 1; k < kmax; k++) {
        const uint64_t r = (uint64_t(k) * d) % nmax;
        double s, c;
        sincospi(2.0 * double(r) / double(nmax), &s, &c);
        part += double(z[2 * k]) * c - double(z[2 * k + 1]) * s;
    }
    acc += 2.0 * part;
    wtab[d] = static_cast<float>(acc);
}

constexpr int FW = 8;   // warps per CTA of the wake and CSR sums

// wake[b][x] = scale * sum_{b2,m} proj[b2][m] w[(pos_b - pos_b2 + x - m) mod nmax]:
// a CTA per 32 outputs x of bunch b (one per lane), its warps splitting
// the source cells m in chunks of 32 (chunk c to warp c mod FW).  Each
// chunk's FP32 partial is added in FP64, the warps' sums in a fixed order
__global__ void __launch_bounds__(FW * 32)
k_wake(const float* __restrict__ proj, const float* __restrict__ wtab,
       const uint32_t* __restrict__ pos, float* __restrict__ wake,
       uint32_t nb, uint32_t n, uint32_t nmax, float scale)
{
    extern __shared__ float sp[];
    __shared__ double red[FW][32];
    const uint32_t b = blockIdx.y;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t x = blockIdx.x * 32 + lane;
    const long long nm = nmax;
    double acc = 0;
    for (uint32_t b2 = 0; b2 < nb; b2++) {
        __syncthreads();
        for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) {
            sp[i] = proj[size_t(b2) * n + i];
        }
        __syncthreads();
        if (x < n) {
            const long long base = (long long)pos[b] - (long long)pos[b2] + x;
            for (uint32_t m0 = 32u * warp; m0 < n; m0 += 32u * FW) {
                long long d0 = (base - (long long)m0) % nm;
                uint32_t d = static_cast<uint32_t>(d0 < 0 ? d0 + nm : d0);
                const uint32_t me = min(n, m0 + 32u);
                float part = 0.f;
                for (uint32_t m = m0; m < me; m++) {
                    part = fmaf(sp[m], __ldg(wtab + d), part);
                    d = (d == 0) ? nmax - 1 : d - 1;
                }
                acc += part;
            }
        }
    }
    red[warp][lane] = acc;
    __syncthreads();
    if (warp == 0 && x < n) {
        double sum = 0;
#pragma unroll
        for (int w = 0; w < FW; w++) {
            sum += red[w][lane];
        }
        wake[size_t(b) * n + x] = __fmul_rn(scale, static_cast<float>(sum));
    }
}

__global__ void k_pad(const float* __restrict__ proj,
                      const uint32_t* __restrict__ pos,
                      float* __restrict__ padded, uint32_t n)
{
    const uint32_t b = blockIdx.y;
    const uint32_t x = blockIdx.x * blockDim.x + threadIdx.x;
    if (x < n) {
        padded[pos[b] + x] = proj[size_t(b) * n + x];
    }
}

// one lane per frequency bin k <= nmax/2 (32 bins per CTA) of bunch
// blockIdx.y: FF_k = sum_m p[m] e^{-2 pi i k m / nmax}, spectrum = coef_k
// |FF_k|^2.  The warps split the source cells in chunks of 32 as in
// k_wake; the twiddles sit in shared memory when tw_smem is set
__global__ void __launch_bounds__(FW * 32)
k_csr(const float* __restrict__ proj, const float2* __restrict__ tw,
      const float* __restrict__ coef, float* __restrict__ spectrum,
      double* __restrict__ power, uint32_t n, uint32_t nmax, float fdelta,
      int tw_smem)
{
    extern __shared__ float4 csr_dyn[];
    float2* stw = reinterpret_cast<float2*>(csr_dyn);
    float* sp = reinterpret_cast<float*>(csr_dyn) + (tw_smem ? 2 * nmax : 0);
    __shared__ double red[2][FW][32];
    const uint32_t b = blockIdx.y;
    for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) {
        sp[i] = proj[size_t(b) * n + i];
    }
    if (tw_smem) {
        for (uint32_t i = threadIdx.x; i < nmax; i += blockDim.x) {
            stw[i] = tw[i];
        }
    }
    __syncthreads();
    const float2* T = tw_smem ? stw : tw;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t k = blockIdx.x * 32 + lane;
    double re = 0, im = 0;
    if (k <= nmax / 2) {
        for (uint32_t m0 = 32u * warp; m0 < n; m0 += 32u * FW) {
            uint32_t idx = static_cast<uint32_t>((uint64_t(m0) * k) % nmax);
            const uint32_t me = min(n, m0 + 32u);
            float pre = 0.f, pim = 0.f;
            for (uint32_t m = m0; m < me; m++) {
                const float2 t = T[idx];
                pre = fmaf(sp[m], t.x, pre);
                pim = fmaf(-sp[m], t.y, pim);
                idx += k;
                if (idx >= nmax) {
                    idx -= nmax;
                }
            }
            re += pre;
            im += pim;
        }
    }
    red[0][warp][lane] = re;
    red[1][warp][lane] = im;
    __syncthreads();
    if (warp == 0) {
        double pw = 0;
        if (k <= nmax / 2) {
            double R = 0, I = 0;
#pragma unroll
            for (int w = 0; w < FW; w++) {
                R += red[0][w][lane];
                I += red[1][w][lane];
            }
            const float sv = __fmul_rn(coef[k], static_cast<float>(R * R
                                                                 + I * I));
            spectrum[size_t(b) * nmax + k] = sv;
            pw = double(fdelta) * double(sv);
        }
        pw = dev::warp_sum(pw);
        if (lane == 0) {
            atomicAdd(power + b, pw);
        }
    }
}

__global__ void k_twiddle(float2* tw, uint32_t nmax)
{
    const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j < nmax) {
        double s, c;
        sincospi(2.0 * double(j) / double(nmax), &s, &c);
        tw[j] = make_float2(static_cast<float>(c), static_cast<float>(s));
    }
}

}  // namespace

void launch_wake_table(vfps_field* f)
{
    const uint32_t nmax = static_cast<uint32_t>(f->nmax);
    cudaStream_t st = f->ps->ctx->stream;
    k_wake_table<<<(nmax + 127) / 128, 128, 0, st>>>(f->z.p, nmax, f->wtab.p);
    VFPS_LAUNCHED();
    k_twiddle<<<(nmax + 127) / 128, 128, 0, st>>>(
        reinterpret_cast<float2*>(f->twiddle.p), nmax);
    VFPS_LAUNCHED();
}

void launch_wake_table_raw(vfps_ctx* ctx, const float* z, size_t nmax,
                           float* out)
{
    const uint32_t m = static_cast<uint32_t>(nmax);
    k_wake_table<<<(m + 127) / 128, 128, 0, ctx->stream>>>(z, m, out);
    VFPS_LAUNCHED();
}

void launch_wake(vfps_field* f)
{
    vfps_ps* ps = f->ps;
    const uint32_t n = ps->n;
    dim3 grid((n + 31) / 32, ps->nb);
    k_wake<<<grid, FW * 32, n * sizeof(float), ps->ctx->stream>>>(
        ps->proj[0].p, f->wtab.p, f->d_pos.p, f->wake.p, ps->nb, n,
        static_cast<uint32_t>(f->nmax), f->wakescale);
    VFPS_LAUNCHED();
}

void launch_pad(vfps_field* f)
{
    vfps_ps* ps = f->ps;
    VFPS_CUDA(cudaMemsetAsync(f->padded.p, 0, f->padded.bytes(),
                              ps->ctx->stream));
    dim3 grid((ps->n + 127) / 128, ps->nb);
    k_pad<<<grid, 128, 0, ps->ctx->stream>>>(ps->proj[0].p, f->d_pos.p,
                                             f->padded.p, ps->n);
    VFPS_LAUNCHED();
}

void launch_csr(vfps_field* f)
{
    vfps_ps* ps = f->ps;
    const uint32_t nmax = static_cast<uint32_t>(f->nmax);
    cudaStream_t st = ps->ctx->stream;
    VFPS_CUDA(cudaMemsetAsync(f->power.p, 0, f->power.bytes(), st));
    // twiddles in shared memory up to nmax = 4096 (32 KiB, with the
    // profile within the default 48 KiB)
    const int tw_smem = nmax <= 4096 ? 1 : 0;
    const size_t smem = (tw_smem ? size_t(nmax) * sizeof(float2) : 0)
                        + ps->n * sizeof(float);
    dim3 grid((nmax / 2 + 1 + 31) / 32, ps->nb);
    k_csr<<<grid, FW * 32, smem, st>>>(
        ps->proj[0].p, reinterpret_cast<const float2*>(f->twiddle.p),
        f->csr_coef.p, f->spectrum.p, f->power.p, ps->n, nmax, f->freq_delta,
        tw_smem);
    VFPS_LAUNCHED();
}

}  // namespace vfps
