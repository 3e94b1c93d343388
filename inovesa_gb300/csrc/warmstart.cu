// Learned warm start (no counterpart in the reference): a small network
// that proposes the equilibrium density of a bunch from its normalised
// current, gap ratio and damping time, trained on equilibria the solver
// itself produced.  Forward, backward and Adam kernels; every buffer is a
// device pointer owned by the caller (vfps_ws_net in vfps.h).
//
// Network (B samples, nin inputs, nh hidden units, nlat latent channels,
// npix output cells):
//   h1 = tanh(W1 x + b1)            W1 [nh][nin]
//   h2 = tanh(W2 h1 + b2)           W2 [nh][nh]
//   z  = W3 h2 + b3                 W3 [nlat][nh]
//   y  = bd + sum_k z_k Wd[k]       Wd [nlat][npix]: a transposed
//                                   convolution from a 1x1 latent map with
//                                   nlat channels to the full mesh
// Weights are read as BF16 (the Adam step keeps FP32 masters and writes
// the BF16 copies); all sums accumulate in FP32.  Loss: mean squared error
// against the target densities, L = sum (y - t)^2 / (B npix).
#include <algorithm>

#include <cuda_bf16.h>

#include "vfps_internal.cuh"

namespace {

constexpr int WS_THREADS = 256;
constexpr uint32_t WS_LAT = 32;   // latent channels (nlat must equal it)

__device__ __forceinline__ float bf(const __nv_bfloat16* w, size_t i)
{
    return __bfloat162float(w[i]);
}

// one CTA per sample: hidden layers and latent
__global__ void k_ws_mlp_fwd(vfps_ws_net N, const float* __restrict__ x,
                             float* __restrict__ h1, float* __restrict__ h2,
                             float* __restrict__ z)
{
    const uint32_t b = blockIdx.x;
    extern __shared__ float ws_s[];
    float* xs = ws_s;                 // [nin]
    float* a1 = xs + N.nin;           // [nh]
    float* a2 = a1 + N.nh;            // [nh]
    const auto* W1 = static_cast<const __nv_bfloat16*>(N.w1);
    const auto* W2 = static_cast<const __nv_bfloat16*>(N.w2);
    const auto* W3 = static_cast<const __nv_bfloat16*>(N.w3);
    for (uint32_t i = threadIdx.x; i < N.nin; i += blockDim.x) {
        xs[i] = x[size_t(b) * N.nin + i];
    }
    __syncthreads();
    for (uint32_t j = threadIdx.x; j < N.nh; j += blockDim.x) {
        float s = N.b1[j];
        for (uint32_t i = 0; i < N.nin; i++) {
            s = fmaf(bf(W1, size_t(j) * N.nin + i), xs[i], s);
        }
        a1[j] = tanhf(s);
        h1[size_t(b) * N.nh + j] = a1[j];
    }
    __syncthreads();
    for (uint32_t j = threadIdx.x; j < N.nh; j += blockDim.x) {
        float s = N.b2[j];
        for (uint32_t i = 0; i < N.nh; i++) {
            s = fmaf(bf(W2, size_t(j) * N.nh + i), a1[i], s);
        }
        a2[j] = tanhf(s);
        h2[size_t(b) * N.nh + j] = a2[j];
    }
    __syncthreads();
    for (uint32_t k = threadIdx.x; k < N.nlat; k += blockDim.x) {
        float s = N.b3[k];
        for (uint32_t i = 0; i < N.nh; i++) {
            s = fmaf(bf(W3, size_t(k) * N.nh + i), a2[i], s);
        }
        z[size_t(b) * N.nlat + k] = s;
    }
}

// y[b][p] = bd[p] + sum_k z[b][k] Wd[k][p]; with a target, also the loss
// gradient g = 2 (y - t) / (B npix) and per-CTA partial losses
__global__ void k_ws_decode(vfps_ws_net N, const float* __restrict__ z,
                            uint32_t B, const float* __restrict__ target,
                            float* __restrict__ y, float* __restrict__ g,
                            double* __restrict__ lpart)
{
    extern __shared__ float ws_s[];
    float* zs = ws_s;                 // [B][nlat]
    __shared__ double red[32];
    for (uint32_t i = threadIdx.x; i < B * N.nlat; i += blockDim.x) {
        zs[i] = z[i];
    }
    __syncthreads();
    const auto* Wd = static_cast<const __nv_bfloat16*>(N.wd);
    const float inv = 2.f / (float(B) * float(N.npix));
    double loss = 0;
    for (size_t p = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
         p < N.npix; p += size_t(gridDim.x) * blockDim.x) {
        float w[WS_LAT];
#pragma unroll
        for (uint32_t k = 0; k < WS_LAT; k++) {
            w[k] = bf(Wd, size_t(k) * N.npix + p);
        }
        const float bias = N.bd[p];
        for (uint32_t b = 0; b < B; b++) {
            float s = bias;
#pragma unroll
            for (uint32_t k = 0; k < WS_LAT; k++) {
                s = fmaf(zs[b * WS_LAT + k], w[k], s);
            }
            const size_t o = size_t(b) * N.npix + p;
            if (y) {
                y[o] = s;
            }
            if (target) {
                const float d = s - target[o];
                g[o] = inv * d;
                loss += double(d) * d;
            }
        }
    }
    if (target) {
        loss = vfps::dev::block_sum(loss, red);
        if (threadIdx.x == 0) {
            lpart[blockIdx.x] = loss;
        }
    }
}

// dWd[k][p] = sum_b z[b][k] g[b][p], dbd[p] = sum_b g[b][p]
__global__ void k_ws_decode_bwd_w(vfps_ws_net N, vfps_ws_net G,
                                  const float* __restrict__ z,
                                  const float* __restrict__ g, uint32_t B)
{
    extern __shared__ float ws_s[];
    float* zs = ws_s;
    for (uint32_t i = threadIdx.x; i < B * N.nlat; i += blockDim.x) {
        zs[i] = z[i];
    }
    __syncthreads();
    float* dWd = const_cast<float*>(static_cast<const float*>(G.wd));
    float* dbd = const_cast<float*>(G.bd);
    for (size_t p = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
         p < N.npix; p += size_t(gridDim.x) * blockDim.x) {
        float acc[WS_LAT];
#pragma unroll
        for (uint32_t k = 0; k < WS_LAT; k++) {
            acc[k] = 0.f;
        }
        float sb = 0.f;
        for (uint32_t b = 0; b < B; b++) {
            const float gv = g[size_t(b) * N.npix + p];
            sb += gv;
#pragma unroll
            for (uint32_t k = 0; k < WS_LAT; k++) {
                acc[k] = fmaf(zs[b * WS_LAT + k], gv, acc[k]);
            }
        }
#pragma unroll
        for (uint32_t k = 0; k < WS_LAT; k++) {
            dWd[size_t(k) * N.npix + p] = acc[k];
        }
        dbd[p] = sb;
    }
}

// dz[b][k] = sum_p Wd[k][p] g[b][p]: one CTA per (b, k)
__global__ void k_ws_decode_bwd_z(vfps_ws_net N, const float* __restrict__ g,
                                  float* __restrict__ dz)
{
    __shared__ double red[32];
    const uint32_t b = blockIdx.x / N.nlat, k = blockIdx.x % N.nlat;
    const auto* Wd = static_cast<const __nv_bfloat16*>(N.wd);
    float s = 0.f;
    double acc = 0;
    int cnt = 0;
    for (size_t p = threadIdx.x; p < N.npix; p += blockDim.x) {
        s = fmaf(bf(Wd, size_t(k) * N.npix + p), g[size_t(b) * N.npix + p],
                 s);
        if (++cnt == 32) {
            acc += s;
            s = 0.f;
            cnt = 0;
        }
    }
    acc += s;
    acc = vfps::dev::block_sum(acc, red);
    if (threadIdx.x == 0) {
        dz[blockIdx.x] = float(acc);
    }
}

// back through the MLP, one CTA per sample: per-sample deltas
//   d3 = dz, d2 = (W3^T d3) (1 - h2^2), d1 = (W2^T d2) (1 - h1^2)
__global__ void k_ws_mlp_bwd(vfps_ws_net N, const float* __restrict__ h1,
                             const float* __restrict__ h2,
                             const float* __restrict__ dz,
                             float* __restrict__ d1, float* __restrict__ d2)
{
    const uint32_t b = blockIdx.x;
    extern __shared__ float ws_s[];
    float* s3 = ws_s;                 // [nlat]
    float* s2 = s3 + N.nlat;          // [nh]
    const auto* W2 = static_cast<const __nv_bfloat16*>(N.w2);
    const auto* W3 = static_cast<const __nv_bfloat16*>(N.w3);
    for (uint32_t k = threadIdx.x; k < N.nlat; k += blockDim.x) {
        s3[k] = dz[size_t(b) * N.nlat + k];
    }
    __syncthreads();
    for (uint32_t i = threadIdx.x; i < N.nh; i += blockDim.x) {
        float s = 0.f;
        for (uint32_t k = 0; k < N.nlat; k++) {
            s = fmaf(bf(W3, size_t(k) * N.nh + i), s3[k], s);
        }
        const float a = h2[size_t(b) * N.nh + i];
        s2[i] = s * (1.f - a * a);
        d2[size_t(b) * N.nh + i] = s2[i];
    }
    __syncthreads();
    for (uint32_t i = threadIdx.x; i < N.nh; i += blockDim.x) {
        float s = 0.f;
        for (uint32_t j = 0; j < N.nh; j++) {
            s = fmaf(bf(W2, size_t(j) * N.nh + i), s2[j], s);
        }
        const float a = h1[size_t(b) * N.nh + i];
        d1[size_t(b) * N.nh + i] = s * (1.f - a * a);
    }
}

// dW[j][i] = sum_b d[b][j] a[b][i], db[j] = sum_b d[b][j]; one thread per
// weight (the layers are small)
__global__ void k_ws_outer(const float* __restrict__ d,
                           const float* __restrict__ a, uint32_t B,
                           uint32_t nout, uint32_t nin, float* __restrict__ dW,
                           float* __restrict__ db)
{
    const size_t t = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (t < size_t(nout) * nin) {
        const uint32_t j = uint32_t(t / nin), i = uint32_t(t % nin);
        float s = 0.f;
        for (uint32_t b = 0; b < B; b++) {
            s = fmaf(d[size_t(b) * nout + j], a[size_t(b) * nin + i], s);
        }
        dW[t] = s;
    } else if (t < size_t(nout) * nin + nout) {
        const uint32_t j = uint32_t(t - size_t(nout) * nin);
        float s = 0.f;
        for (uint32_t b = 0; b < B; b++) {
            s += d[size_t(b) * nout + j];
        }
        db[j] = s;
    }
}

// Adam (Kingma & Ba 2015) on FP32 masters; writes the BF16 copy
__global__ void k_ws_adam(float* __restrict__ w, const float* __restrict__ g,
                          float* __restrict__ m, float* __restrict__ v,
                          __nv_bfloat16* __restrict__ w16, size_t count,
                          float lr, float b1, float b2, float eps, float c1,
                          float c2)
{
    for (size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x; i < count;
         i += size_t(gridDim.x) * blockDim.x) {
        const float gi = g[i];
        const float mi = b1 * m[i] + (1.f - b1) * gi;
        const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
        m[i] = mi;
        v[i] = vi;
        const float wi = w[i] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
        w[i] = wi;
        if (w16) {
            w16[i] = __float2bfloat16_rn(wi);
        }
    }
}

int ws_check(const vfps_ws_net* n)
{
    if (!n || n->nin == 0 || n->nh == 0 || n->nlat != WS_LAT
        || n->npix == 0 || !n->w1 || !n->b1 || !n->w2 || !n->b2 || !n->w3
        || !n->b3 || !n->wd || !n->bd) {
        return VFPS_ERR_INVALID_ARGUMENT;
    }
    return VFPS_OK;
}

int launched(vfps_ctx* ctx)
{
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        ctx->last_error = cudaGetErrorString(e);
        return VFPS_ERR_CUDA;
    }
    return VFPS_OK;
}

}  // namespace

extern "C" int vfps_ws_forward(vfps_ctx* ctx, const vfps_ws_net* net,
                               const float* x, uint32_t B, float* h1,
                               float* h2, float* z, float* y,
                               const float* target, float* g, double* lpart,
                               uint32_t nparts)
{
    if (!ctx || ws_check(net) || !x || !h1 || !h2 || !z || B == 0
        || (target && (!g || !lpart || nparts == 0))) {
        return VFPS_ERR_INVALID_ARGUMENT;
    }
    if (cudaSetDevice(ctx->device) != cudaSuccess) {
        return VFPS_ERR_CUDA;
    }
    const vfps_ws_net N = *net;
    const size_t s1 = sizeof(float) * (N.nin + 2 * N.nh);
    k_ws_mlp_fwd<<<B, WS_THREADS, s1, ctx->stream>>>(N, x, h1, h2, z);
    int rc = launched(ctx);
    if (rc) {
        return rc;
    }
    const size_t s2 = sizeof(float) * size_t(B) * N.nlat;
    const uint32_t grid = target ? nparts
        : uint32_t((N.npix + WS_THREADS - 1) / WS_THREADS);
    k_ws_decode<<<grid, WS_THREADS, s2, ctx->stream>>>(N, z, B, target, y, g,
                                                      lpart);
    return launched(ctx);
}

extern "C" int vfps_ws_backward(vfps_ctx* ctx, const vfps_ws_net* net,
                                const vfps_ws_net* grad, const float* x,
                                uint32_t B, const float* h1, const float* h2,
                                const float* z, const float* g, float* dz,
                                float* d1, float* d2)
{
    if (!ctx || ws_check(net) || ws_check(grad) || !x || !h1 || !h2 || !z
        || !g || !dz || !d1 || !d2 || B == 0) {
        return VFPS_ERR_INVALID_ARGUMENT;
    }
    if (cudaSetDevice(ctx->device) != cudaSuccess) {
        return VFPS_ERR_CUDA;
    }
    const vfps_ws_net N = *net, G = *grad;
    cudaStream_t st = ctx->stream;
    const size_t sz = sizeof(float) * size_t(B) * N.nlat;
    k_ws_decode_bwd_w<<<(N.npix + WS_THREADS - 1) / WS_THREADS, WS_THREADS,
                        sz, st>>>(N, G, z, g, B);
    k_ws_decode_bwd_z<<<B * N.nlat, WS_THREADS, 0, st>>>(N, g, dz);
    k_ws_mlp_bwd<<<B, WS_THREADS, sizeof(float) * (N.nlat + N.nh), st>>>(
        N, h1, h2, dz, d1, d2);
    auto outer = [&](const float* d, const float* a, uint32_t nout,
                     uint32_t nin, const void* dW, const float* db) {
        const size_t tot = size_t(nout) * nin + nout;
        k_ws_outer<<<(tot + WS_THREADS - 1) / WS_THREADS, WS_THREADS, 0,
                     st>>>(d, a, B, nout, nin,
                           const_cast<float*>(static_cast<const float*>(dW)),
                           const_cast<float*>(db));
    };
    outer(dz, h2, N.nlat, N.nh, G.w3, G.b3);
    outer(d2, h1, N.nh, N.nh, G.w2, G.b2);
    outer(d1, x, N.nh, N.nin, G.w1, G.b1);
    return launched(ctx);
}

extern "C" int vfps_ws_adam(vfps_ctx* ctx, float* w, const float* g,
                            float* m, float* v, void* w_bf16, size_t count,
                            float lr, float beta1, float beta2, float eps,
                            uint32_t step)
{
    if (!ctx || !w || !g || !m || !v || count == 0 || step == 0) {
        return VFPS_ERR_INVALID_ARGUMENT;
    }
    if (cudaSetDevice(ctx->device) != cudaSuccess) {
        return VFPS_ERR_CUDA;
    }
    const float c1 = 1.f - powf(beta1, float(step));
    const float c2 = 1.f - powf(beta2, float(step));
    const size_t blocks = std::min<size_t>((count + WS_THREADS - 1)
                                           / WS_THREADS, 65535);
    k_ws_adam<<<unsigned(blocks), WS_THREADS, 0, ctx->stream>>>(
        w, g, m, v, static_cast<__nv_bfloat16*>(w_bf16), count, lr, beta1,
        beta2, eps, c1, c2);
    return launched(ctx);
}
