// Internal declarations of libvfps: objects behind the C ABI, RAII device
// buffers, error plumbing and device helpers shared by the kernels.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "vfps.h"

namespace vfps {

// ------------------------------------------------------------ errors
struct Error : std::runtime_error {
    int code;
    Error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

#define VFPS_CUDA(call)                                                   \
    do {                                                                  \
        cudaError_t e_ = (call);                                          \
        if (e_ != cudaSuccess) {                                          \
            throw ::vfps::Error(                                          \
                e_ == cudaErrorMemoryAllocation ? VFPS_ERR_OUT_OF_MEMORY  \
                                                : VFPS_ERR_CUDA,          \
                std::string(#call) + ": " + cudaGetErrorString(e_));      \
        }                                                                 \
    } while (0)

#define VFPS_REQUIRE(cond, msg)                                           \
    do {                                                                  \
        if (!(cond)) {                                                    \
            throw ::vfps::Error(VFPS_ERR_INVALID_ARGUMENT, (msg));        \
        }                                                                 \
    } while (0)

#define VFPS_LAUNCHED() VFPS_CUDA(cudaGetLastError())

// ----------------------------------------------------- device buffers
template <typename T>
struct DevBuf {
    T* p = nullptr;
    size_t n = 0;
    DevBuf() = default;
    explicit DevBuf(size_t count) { alloc(count); }
    DevBuf(const DevBuf&) = delete;
    DevBuf& operator=(const DevBuf&) = delete;
    DevBuf(DevBuf&& o) noexcept : p(o.p), n(o.n) { o.p = nullptr; o.n = 0; }
    DevBuf& operator=(DevBuf&& o) noexcept
    {
        if (this != &o) {
            release();
            p = o.p;
            n = o.n;
            o.p = nullptr;
            o.n = 0;
        }
        return *this;
    }
    ~DevBuf() { release(); }
    void alloc(size_t count)
    {
        release();
        if (count) {
            VFPS_CUDA(cudaMalloc(&p, count * sizeof(T)));
        }
        n = count;
    }
    void release() noexcept
    {
        if (p) {
            cudaFree(p);
        }
        p = nullptr;
        n = 0;
    }
    size_t bytes() const { return n * sizeof(T); }
    void swap(DevBuf& o) noexcept
    {
        std::swap(p, o.p);
        std::swap(n, o.n);
    }
};

// --------------------------------------------------------------- axis
// Ruler (inc/PS/Ruler.hpp:31-51) in float, as the reference keeps it.
struct Axis {
    uint32_t n = 0;
    float min = 0, max = 0, delta = 0, zerobin = 0, scale = 1;
    std::vector<float> v;
};
Axis make_axis(uint32_t n, float mn, float mx, float scale);

}  // namespace vfps

// ----------------------------------------------------- C ABI objects
struct vfps_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    std::string last_error;
    int* d_status = nullptr;   // device error word
    int sm_count = 0;
};

struct vfps_ps {
    vfps_ctx* ctx = nullptr;
    int device = 0;                  // own copy: destroy touches nothing else
    uint32_t nb = 0, n = 0;
    double charge = 0, current = 0;
    vfps::Axis ax[2];
    std::vector<float> filling_set;
    vfps::DevBuf<float> data;        // [nb][n][n]
    vfps::DevBuf<float> proj[2];     // [nb][n] per axis
    vfps::DevBuf<double> proj64;     // x projection, FP64
    vfps::DevBuf<float> ws;          // Simpson weights [n]
    vfps::DevBuf<float> axisv[2];    // axis values [n]
    vfps::DevBuf<float> fillset;     // [nb]
    vfps::DevBuf<double> filling;    // [nb] + integral at [nb]
    vfps::DevBuf<float> moments;     // [2][3][nb]: avg, var, rms
};

enum MapKind {
    MAP_ROTATION,
    MAP_KICK,
    MAP_FP,
    MAP_IDENTITY
};

// Counter-based generator Philox-4x32-10 (Salmon, Moraes, Dror, Shaw,
// "Parallel random numbers: as easy as 1, 2, 3", SC 2011): ten rounds of
// two 32x32->64-bit multiplications mixing a 128-bit counter under a
// 64-bit key bumped by the Weyl constants between rounds.
__host__ __device__ inline void philox4x32_10(const uint32_t ctr[4],
                                              const uint32_t key[2],
                                              uint32_t out[4])
{
    uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
    uint32_t k0 = key[0], k1 = key[1];
    for (int r = 0; r < 10; r++) {
        const uint64_t p0 = uint64_t(0xD2511F53u) * c0;
        const uint64_t p1 = uint64_t(0xCD9E8D57u) * c2;
        const uint32_t hi0 = uint32_t(p0 >> 32), lo0 = uint32_t(p0);
        const uint32_t hi1 = uint32_t(p1 >> 32), lo1 = uint32_t(p1);
        c0 = hi1 ^ c1 ^ k0;
        c1 = lo1;
        c2 = hi0 ^ c3 ^ k1;
        c3 = lo0;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    out[0] = c0;
    out[1] = c1;
    out[2] = c2;
    out[3] = c3;
}

// parameters of a DynamicRFKickMap (src/SM/DynamicRFKickMap.cpp:15-109)
struct DynRf {
    int linear = 1;
    float angle = 0, revolutionpart = 0, v_rf = 0, v0 = 0;
    float syncphase = 0, bl2phase = 0;
    float phasenoise = 0, amplnoise = 0;   // spreads / sqrt(revolutionpart)
    float modampl = 0;
    double modtimedelta = 0;               // 2 pi modtimeincrement
    uint32_t seed = 0;
};

// VFPS_PLAIN_KERNEL=cell keeps a plain kick or Fokker-Planck map created
// while it is set on the thread-per-cell kernels (the row-sweep forms and
// these side by side in tests)
inline bool plain_cells_env()
{
    const char* v = std::getenv("VFPS_PLAIN_KERNEL");
    return v && std::string(v) == "cell";
}

struct vfps_map {
    MapKind kind = MAP_IDENTITY;
    bool cells = plain_cells_env();
    int device = 0;
    vfps_ps* in = nullptr;
    vfps_ps* out = nullptr;
    int it = 4;
    int clamp = 0;
    // rotation
    float angle = 0, cs = 1, sn = 0;
    // kick
    int axis = 1;
    vfps::DevBuf<float> offset;      // x-kick: [n]; y-kick: [nb][n]
    const float* offset_src = nullptr;  // wake map: field's wake buffer
    vfps_field* field = nullptr;
    std::vector<float> host_offset;  // mirror for applyTo / getForce
    bool host_offset_valid = true;
    // x-kick: the stencils of the current offsets, tap-major [4][n] (the
    // row-sweep kernel reads them instead of evaluating them per row)
    mutable vfps::DevBuf<int> xshift;
    mutable vfps::DevBuf<float> xweight;
    mutable bool xtab_valid = false;
    // DynamicRFKickMap: per-step phase and amplitude drawn on the device
    bool dynrf = false;
    DynRf dyn;
    uint64_t dyn_step = 0;                 // applies so far
    vfps::DevBuf<float> dyn_log;           // [capacity][2] phase, ampl
    uint64_t dyn_cap = 0;
    vfps::DevBuf<float> axis_q;            // q axis values [n]
    // Fokker-Planck
    int ip = 0;
    int fptrack = 0;
    float e1 = 0;
    vfps::DevBuf<uint32_t> fp_idx;
    vfps::DevBuf<float> fp_w;
    vfps::DevBuf<uint32_t> fp_idx4;        // the same, tap-major [4][n]
    vfps::DevBuf<float> fp_w4;
    std::vector<uint32_t> h_fp_idx;
    std::vector<float> h_fp_w;
};

struct vfps_impedance {
    vfps_ctx* ctx = nullptr;
    int device = 0;
    size_t nfreqs = 0;
    double f_max = 0;
    vfps::DevBuf<float> z;           // interleaved re, im
};

struct vfps_field {
    vfps_ps* ps = nullptr;
    int device = 0;
    const vfps_impedance* imp = nullptr;
    vfps::DevBuf<float> z;           // private copy of the table
    size_t nmax = 0;
    uint32_t spacing = 0;
    std::vector<uint32_t> buckets;
    vfps::DevBuf<uint32_t> d_pos;    // bucket * spacing per bunch
    double f_rev = 0, revpart = 1;
    float wakescale = 0;             // wakescaling / nmax
    bool has_wake = false;
    vfps::DevBuf<float> wtab;        // Toeplitz kernel w[d], d in [0,nmax)
    vfps::DevBuf<float> wake;        // [nb][n]
    vfps::DevBuf<float> padded;      // [nmax]
    // CSR
    vfps::DevBuf<float> twiddle;     // [nmax] (cos, sin) pairs
    vfps::DevBuf<float> csr_coef;    // [nmax/2+1]
    vfps::DevBuf<float> spectrum;    // [nb][nmax]
    vfps::DevBuf<double> power;      // [nb]
    float csr_fc = -1;
    bool csr_ready = false;
    float freq_delta = 0;
    double freq_scale = 0;
    double factor4watts = 0;
};

// ----------------------------------------------------- launch wrappers
namespace vfps {

void set_status(vfps_ctx* ctx, int code);  // host-side helper

void launch_fill_gaussian(vfps_ps* ps, const float* gx, const float* gy);
void launch_project_x(vfps_ps* ps, const float* data);
void launch_project_y(vfps_ps* ps);
void launch_integrate(vfps_ps* ps);
void launch_normalize(vfps_ps* ps);
void launch_moments(vfps_ps* ps, int axis);

void launch_rotation(const vfps_map* m);
void launch_kick(const vfps_map* m, const float* offset);
void launch_dynrf(vfps_map* m);
void launch_fp(const vfps_map* m);

void launch_wake_table(vfps_field* f);
void launch_wake_table_raw(vfps_ctx* ctx, const float* z, size_t nmax,
                           float* out);
void launch_wake(vfps_field* f);
void launch_pad(vfps_field* f);
void launch_csr(vfps_field* f);

void launch_z_model(vfps_ctx* ctx, int model, size_t n, const double* prm,
                    float* out);
void launch_z_add(vfps_ctx* ctx, float* dst, const float* src, size_t n);

}  // namespace vfps

// ------------------------------------------------------ device helpers
// Float arithmetic with the reference's operation order and rounding
// (no contraction into FMA), so that stencils agree with its CPU build.
namespace vfps {
namespace dev {

__device__ __forceinline__ float fadd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float fsub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float fmul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float fdiv(float a, float b) { return __fdiv_rn(a, b); }

// calcCoefficiants (src/SM/SourceMap.cpp:142-170); x/2 == x*0.5 exactly.
__device__ __forceinline__ void coefficients(float* ic, float f, int it)
{
    switch (it) {
    case 1:
        ic[0] = 1.f;
        break;
    case 2:
        ic[0] = fsub(1.f, f);
        ic[1] = f;
        break;
    case 3:
        ic[0] = fmul(fmul(f, fsub(f, 1.f)), 0.5f);
        ic[1] = fsub(1.f, fmul(f, f));
        ic[2] = fmul(fmul(f, fadd(f, 1.f)), 0.5f);
        break;
    default:
        ic[0] = fmul(fmul(fmul(fsub(f, 1.f), fsub(f, 2.f)), f),
                     static_cast<float>(-1. / 6.));
        ic[1] = fmul(fmul(fmul(fadd(f, 1.f), fsub(f, 1.f)), fsub(f, 2.f)),
                     0.5f);
        ic[2] = fmul(fmul(fmul(fsub(2.f, f), f), fadd(f, 1.f)), 0.5f);
        ic[3] = fmul(fmul(fmul(f, fadd(f, 1.f)), fsub(f, 1.f)),
                     static_cast<float>(1. / 6.));
        break;
    }
}

// truncated base index of a source coordinate, as modf + static_cast<>
// to uint32 do on x86-64: values <= -1 and >= size are out of range.
__device__ __forceinline__ bool base_index(float v, uint32_t size, int* base,
                                           float* frac)
{
    const float t = truncf(v);
    *frac = v - t;  // exact
    if (!(t >= 0.f) || !(t < static_cast<float>(size))) {
        return false;
    }
    *base = static_cast<int>(t);
    return true;
}

// KickMap::updateSM (src/SM/KickMap.cpp:339-389) for one row/column:
// source index offset (tap j reads cell i + shift[j]) and weight, with
// dropped taps marked by weight 0 and valid = false.
struct KickStencil {
    int shift[4];
    float w[4];
    bool valid[4];
};

__device__ __forceinline__ KickStencil kick_stencil(float offset, uint32_t n,
                                                    int it)
{
    KickStencil s;
    const float poffs = fadd(static_cast<float>(n / 2), offset);
    int jd = 0;   // no valid tap when base_index fails
    float f;
    const bool ok = base_index(poffs, n, &jd, &f);
    float c[4] = {0.f, 0.f, 0.f, 0.f};
    if (ok) {
        coefficients(c, f, it);
    }
    const int h = (it - 1) / 2;
#pragma unroll
    for (int j = 0; j < 4; j++) {
        const int j0 = jd + j - h;
        s.valid[j] = ok && j < it && j0 >= 0 && j0 < static_cast<int>(n);
        s.w[j] = s.valid[j] ? c[j] : 0.f;
        s.shift[j] = j0 - static_cast<int>(n / 2);
    }
    return s;
}

// ---------------------------------------- mbarrier + TMA bulk copies
__device__ __forceinline__ uint32_t smem_addr(const void* p)
{
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;"
                 :: "r"(smem_addr(bar)), "r"(count) : "memory");
}

// make barrier initialisation visible to the async (TMA) proxy
__device__ __forceinline__ void mbar_fence_init()
{
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// order this thread's earlier generic shared-memory accesses before
// later async-proxy (TMA) writes to the same memory
__device__ __forceinline__ void fence_proxy_async()
{
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar,
                                                      uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;"
                 :: "r"(smem_addr(bar)), "r"(bytes) : "memory");
}

// bulk copy of `bytes` (multiple of 16, both addresses 16-byte aligned)
// from global to this CTA's shared memory, completing on `bar`
__device__ __forceinline__ void tma_load_1d(void* dst, const void* src,
                                            uint32_t bytes, uint64_t* bar)
{
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes"
        " [%0], [%1], %2, [%3];"
        :: "r"(smem_addr(dst)), "l"(src), "r"(bytes), "r"(smem_addr(bar))
        : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity)
{
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n"
        " mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        " selp.u32 %0, 1, 0, p;\n}"
        : "=r"(done) : "r"(smem_addr(bar)), "r"(parity) : "memory");
    return done != 0;
}

// Programmatic dependent launch: let the next kernel of the stream (one
// launched with programmatic stream serialisation) start its independent
// prologue, and wait until the previous kernel has completed and its
// memory is visible before reading or writing anything it touches.
__device__ __forceinline__ void pdl_trigger()
{
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

__device__ __forceinline__ void pdl_wait()
{
    asm volatile("griddepcontrol.wait;" ::: "memory");
}

// a hint to bring the 128-byte line of p into L2
__device__ __forceinline__ void prefetch_l2(const void* p)
{
    asm volatile("prefetch.global.L2 [%0];" ::"l"(p));
}

__device__ __forceinline__ uint64_t global_ns()
{
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// wait for phase `parity` of `bar` for at most timeout_ns; false if it
// gave up (the caller records an error instead of hanging)
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar,
                                                  uint32_t parity,
                                                  uint64_t timeout_ns)
{
    if (mbar_try_wait(bar, parity)) {
        return true;
    }
    const uint64_t t0 = global_ns();
    while (!mbar_try_wait(bar, parity)) {
        if (global_ns() - t0 > timeout_ns) {
            return false;
        }
    }
    return true;
}

__device__ __forceinline__ double warp_sum(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        v += __shfl_down_sync(0xffffffffu, v, o);
    }
    return v;
}

__device__ __forceinline__ float warp_sum_f(float v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        v += __shfl_down_sync(0xffffffffu, v, o);
    }
    return v;
}

// block-wide FP64 sum (blockDim multiple of 32, <= 1024); result valid in
// thread 0.
__device__ __forceinline__ double block_sum(double v, double* scratch32)
{
    v = warp_sum(v);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) {
        scratch32[warp] = v;
    }
    __syncthreads();
    v = 0;
    if (warp == 0) {
        const int nw = (blockDim.x + 31) >> 5;
        v = lane < nw ? scratch32[lane] : 0.0;
        v = warp_sum(v);
    }
    __syncthreads();
    return v;
}

}  // namespace dev
}  // namespace vfps
