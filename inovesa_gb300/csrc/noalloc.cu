// vfps_charge_noalloc: charge integrals of densities the caller already
// holds in device memory, computed without allocating anything.
//
// Who needs this.  Some callers may not allocate device memory at the
// moment they want the charge of a density: a host program that reserved
// its whole device-memory budget at start-up and hands the library only
// raw pointers into it; a pool allocator (PyTorch's caching allocator, a
// solver's own arena) that must be the only owner of the device's free
// memory; or a time-critical loop on one stream that cannot afford the
// device-wide synchronisation cudaMalloc/cudaFree may imply, which would
// stall every other stream of the process.  The PhaseSpace path
// (vfps_ps_create, then vfps_ps_update_x_projection and vfps_ps_integrate)
// owns device buffers, so it cannot serve them.
//
// What it computes.  For each of nb meshes [n][n] (row x = position, column
// y = energy): the x projection proj[x] = sum_y rho[x][y] ws[y] and the
// integral sum_x proj[x] ws[x] with the Simpson weights ws of spacing
// delta, in the same order of operations as vfps_ps_update_x_projection
// followed by vfps_ps_integrate (FP32 partial sums of at most 8 cells per
// lane, FP64 beyond), so both give the same numbers.
//
// Where the scratch lives.  The FP64 row projections and the per-mesh
// results go to one file-scope __device__ array of fixed size (below).
// Its address on a device is looked up once, by the first call made with
// that device current (cudaGetSymbolAddress); make that first call before
// any stream capture starts.  The address belongs to the device's CUDA
// context: it is remembered together with that context's unique id, and a
// call that finds another context current (the host program or a library
// reset the device with cudaDeviceReset and a new context came up) looks
// it up again, so that call is a set-up call too.  Calls whose nb * n rows
// or nb meshes exceed the scratch are rejected with
// VFPS_ERR_INVALID_ARGUMENT before anything is launched.
//
// The call makes the context's device current while it runs and gives the
// calling thread back the device that was current before (other entry
// points of the library leave the context's device current).
//
// Rules for callers.  Nothing in the scratch has to start at zero: each
// call writes every word it reads before reading it.  There is one scratch
// per device for the whole process, so two calls on the same device must
// not overlap in time (from two host threads, or two contexts on one
// device): they would overwrite each other's partial sums.  One call
// returns only after its results are in host memory, so calls made one
// after another from one thread never overlap.
#include <mutex>

#include "vfps_internal.cuh"

// 2^18 rows of FP64 projections (2 MiB) + one FP64 result per mesh
constexpr uint32_t NOALLOC_MAX_ROWS = 1u << 18;
constexpr uint32_t NOALLOC_MAX_MESHES = 4096;

static __device__ __align__(256) double
    g_noalloc_scratch[NOALLOC_MAX_ROWS + NOALLOC_MAX_MESHES];

namespace {

constexpr int NOALLOC_MAX_DEVICES = 64;
constexpr int NOALLOC_THREADS = 256;

std::mutex g_noalloc_mu;
double* g_noalloc_ptr[NOALLOC_MAX_DEVICES] = {};
// unique id of the context each cached address was looked up in
unsigned long long g_noalloc_ctx[NOALLOC_MAX_DEVICES] = {};

// cuCtxGetId of the driver (CUDA 12.0+), reached through the runtime so
// that the library does not link the driver library itself
using CtxGetIdFn = int (*)(void*, unsigned long long*);
CtxGetIdFn ctx_get_id()
{
    static CtxGetIdFn fn = [] {
        void* f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000,
                                             cudaEnableDefault, &q)
                != cudaSuccess
            || q != cudaDriverEntryPointSuccess) {
            f = nullptr;
        }
        return reinterpret_cast<CtxGetIdFn>(f);
    }();
    return fn;
}

// Simpson weight of index i, computed as the host table of the PhaseSpace
// path: h03 = delta / 3 at both ends, h03 * 4 at odd and h03 * 2 at even
// interior indices (float arithmetic, correctly rounded)
__device__ __forceinline__ float simpson_weight(uint32_t i, uint32_t n,
                                                float h03)
{
    if (i == 0 || i + 1 == n) {
        return h03;
    }
    return __fmul_rn(h03, (i & 1) ? 4.f : 2.f);
}

// one CTA per mesh: warps project rows into rows64, then the CTA reduces
// them with the Simpson weights into out[mesh]
__global__ void __launch_bounds__(NOALLOC_THREADS)
k_charge_noalloc(const float* __restrict__ density, uint32_t n, float delta,
                 double* __restrict__ rows64, double* __restrict__ out)
{
    __shared__ double red[32];
    const uint32_t b = blockIdx.x;
    const float h03 = __fdiv_rn(delta, 3.f);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int nwarps = NOALLOC_THREADS / 32;
    const float* mesh = density + size_t(b) * n * n;
    double* proj = rows64 + size_t(b) * n;
    for (uint32_t x = warp; x < n; x += nwarps) {
        const float* r = mesh + size_t(x) * n;
        double acc = 0;
        float part = 0;
        int cnt = 0;
        for (uint32_t y = lane; y < n; y += 32) {
            part = fmaf(r[y], simpson_weight(y, n, h03), part);
            if (++cnt == 8) {
                acc += part;
                part = 0;
                cnt = 0;
            }
        }
        acc += part;
        acc = vfps::dev::warp_sum(acc);
        if (lane == 0) {
            proj[x] = acc;
        }
    }
    __syncthreads();
    double acc = 0;
    for (uint32_t x = threadIdx.x; x < n; x += NOALLOC_THREADS) {
        acc += proj[x] * double(simpson_weight(x, n, h03));
    }
    acc = vfps::dev::block_sum(acc, red);
    if (threadIdx.x == 0) {
        out[b] = acc;
    }
}

int fail(vfps_ctx* ctx, int code, const char* msg)
{
    ctx->last_error = msg;
    return code;
}

// the scratch address on the current device: looked up on the first call
// in the device's current context (again after a device reset brought up
// a new context; every call when the context id is not available)
double* scratch_on(int device)
{
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    unsigned long long id = 0;
    const CtxGetIdFn get_id = ctx_get_id();
    const bool known = get_id && get_id(nullptr, &id) == 0 && id != 0;
    if (!g_noalloc_ptr[device] || !known || g_noalloc_ctx[device] != id) {
        void* p = nullptr;
        if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess) {
            g_noalloc_ptr[device] = nullptr;
            return nullptr;
        }
        g_noalloc_ptr[device] = static_cast<double*>(p);
        g_noalloc_ctx[device] = known ? id : 0;
    }
    return g_noalloc_ptr[device];
}

// makes a device current for the scope of one call and gives the calling
// thread its previous device back
struct DeviceScope {
    int prev = -1;
    bool ok = false;
    explicit DeviceScope(int device)
    {
        if (cudaGetDevice(&prev) != cudaSuccess) {
            prev = -1;
        }
        ok = cudaSetDevice(device) == cudaSuccess;
    }
    ~DeviceScope()
    {
        if (prev >= 0) {
            cudaSetDevice(prev);
        }
    }
};

}  // namespace

extern "C" int vfps_charge_noalloc(vfps_ctx* ctx, const float* density,
                                   uint32_t nb, uint32_t n, float delta,
                                   double* integrals)
{
    if (!ctx) {
        return VFPS_ERR_INVALID_ARGUMENT;
    }
    if (!density || !integrals || nb == 0 || n < 2) {
        return fail(ctx, VFPS_ERR_INVALID_ARGUMENT,
                    "vfps_charge_noalloc: null pointer, nb == 0 or n < 2");
    }
    if (nb > NOALLOC_MAX_MESHES || uint64_t(nb) * n > NOALLOC_MAX_ROWS) {
        return fail(ctx, VFPS_ERR_INVALID_ARGUMENT,
                    "vfps_charge_noalloc: nb * n exceeds the fixed scratch "
                    "(at most 262144 rows and 4096 meshes per call)");
    }
    if (ctx->device < 0 || ctx->device >= NOALLOC_MAX_DEVICES) {
        return fail(ctx, VFPS_ERR_INVALID_ARGUMENT,
                    "vfps_charge_noalloc: device index out of range");
    }
    const DeviceScope scope(ctx->device);
    if (!scope.ok) {
        return fail(ctx, VFPS_ERR_CUDA, "vfps_charge_noalloc: cudaSetDevice");
    }
    double* scratch = scratch_on(ctx->device);
    if (!scratch) {
        return fail(ctx, VFPS_ERR_CUDA,
                    "vfps_charge_noalloc: cudaGetSymbolAddress of the "
                    "scratch failed");
    }
    double* out = scratch + NOALLOC_MAX_ROWS;
    k_charge_noalloc<<<nb, NOALLOC_THREADS, 0, ctx->stream>>>(
        density, n, delta, scratch, out);
    if (cudaGetLastError() != cudaSuccess) {
        return fail(ctx, VFPS_ERR_CUDA, "vfps_charge_noalloc: launch failed");
    }
    if (cudaMemcpyAsync(integrals, out, sizeof(double) * nb,
                        cudaMemcpyDeviceToHost, ctx->stream) != cudaSuccess
        || cudaStreamSynchronize(ctx->stream) != cudaSuccess) {
        return fail(ctx, VFPS_ERR_CUDA,
                    "vfps_charge_noalloc: copy of the results failed");
    }
    return VFPS_OK;
}
