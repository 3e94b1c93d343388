// C ABI of libvfps: host logic of the PhaseSpace, SourceMap, Impedance and
// ElectricField objects.  Construction-time tables (axes, Simpson weights,
// static kick offsets, Fokker-Planck stencils, CSR weights) are computed on
// the host in float with the reference's order of operations; everything
// that runs per step is a kernel on the context's stream.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <fstream>
#include <limits>
#include <numeric>
#include <random>
#include <sstream>

#include "vfps_internal.cuh"

namespace {

thread_local std::string g_last_error;

void record(vfps_ctx* ctx, const std::string& msg)
{
    if (ctx) {
        ctx->last_error = msg;
    }
    g_last_error = msg;
}

template <typename F>
int guard(vfps_ctx* ctx, F&& f)
{
    try {
        if (ctx) {
            VFPS_CUDA(cudaSetDevice(ctx->device));
        }
        f();
        return VFPS_OK;
    } catch (const vfps::Error& e) {
        record(ctx, e.what());
        return e.code;
    } catch (const std::bad_alloc&) {
        record(ctx, "host allocation failed");
        return VFPS_ERR_OUT_OF_MEMORY;
    } catch (const std::exception& e) {
        record(ctx, e.what());
        return VFPS_ERR_INVALID_ARGUMENT;
    }
}

int null_arg(const char* what)
{
    g_last_error = std::string("null argument: ") + what;
    return VFPS_ERR_INVALID_ARGUMENT;
}

const double C_LIGHT = 2.99792458e8;            // inc/defines.hpp:48
const double EPS0 = 8.854187817e-12;            // inc/defines.hpp:51
const double Z0_PHYS = 1 / (EPS0 * C_LIGHT);    // inc/defines.hpp:54
const double Z0_IMP = 376.730313461;            // inc/Z/Impedance.hpp:94
const double PI = 3.14159265358979323846;

template <typename T>
void h2d(T* dst, const T* src, size_t count, vfps_ctx* ctx)
{
    VFPS_CUDA(cudaMemcpyAsync(dst, src, count * sizeof(T),
                              cudaMemcpyHostToDevice, ctx->stream));
    VFPS_CUDA(cudaStreamSynchronize(ctx->stream));
}

template <typename T>
void d2h(T* dst, const T* src, size_t count, vfps_ctx* ctx)
{
    VFPS_CUDA(cudaMemcpyAsync(dst, src, count * sizeof(T),
                              cudaMemcpyDeviceToHost, ctx->stream));
    VFPS_CUDA(cudaStreamSynchronize(ctx->stream));
}

// float -> uint32 cast of a truncated coordinate as on x86-64 (see
// base_index in vfps_internal.cuh)
bool host_base(float v, uint32_t size, uint32_t* out)
{
    if (!(v >= 0.f) || !(v < static_cast<float>(size))) {
        return false;
    }
    *out = static_cast<uint32_t>(v);
    return true;
}

}  // namespace

namespace vfps {

Axis make_axis(uint32_t n, float mn, float mx, float scale)
{
    // Ruler throws for min >= max (inc/PS/Ruler.hpp:41-43)
    VFPS_REQUIRE(mn < mx, "Tried to set up Ruler with min >= max.");
    VFPS_REQUIRE(n >= 2, "a mesh axis needs at least 2 points");
    Axis a;
    a.n = n;
    a.min = mn;
    a.max = mx;
    a.scale = scale;
    a.delta = (mx - mn) / static_cast<float>(n - 1);
    a.zerobin = ((mn + mx) / (mn - mx) + 1) * static_cast<float>(n - 1) / 2;
    a.v.resize(n);
    for (uint32_t i = 0; i < n; i++) {
        a.v[i] = mn + (static_cast<float>(i) * a.delta);
    }
    return a;
}

void set_status(vfps_ctx* ctx, int code)
{
    int zero = 0;
    VFPS_CUDA(cudaMemcpyAsync(ctx->d_status, code ? &code : &zero, sizeof(int),
                              cudaMemcpyHostToDevice, ctx->stream));
    VFPS_CUDA(cudaStreamSynchronize(ctx->stream));
}

}  // namespace vfps

using vfps::DevBuf;

/* ================================================================ context */
extern "C" int vfps_create(vfps_ctx** out, int device)
{
    if (!out) {
        return null_arg("ctx");
    }
    *out = nullptr;
    auto ctx = std::make_unique<vfps_ctx>();
    ctx->device = device;
    int rc = guard(ctx.get(), [&] {
        int count = 0;
        VFPS_CUDA(cudaGetDeviceCount(&count));
        VFPS_REQUIRE(device >= 0 && device < count, "no such CUDA device");
        VFPS_CUDA(cudaSetDevice(device));
        VFPS_CUDA(cudaStreamCreateWithFlags(&ctx->stream,
                                            cudaStreamNonBlocking));
        VFPS_CUDA(cudaMalloc(&ctx->d_status, sizeof(int)));
        VFPS_CUDA(cudaMemsetAsync(ctx->d_status, 0, sizeof(int), ctx->stream));
        VFPS_CUDA(cudaDeviceGetAttribute(&ctx->sm_count,
                                         cudaDevAttrMultiProcessorCount,
                                         device));
        VFPS_CUDA(cudaStreamSynchronize(ctx->stream));
    });
    if (rc != VFPS_OK) {
        g_last_error = ctx->last_error;
        if (ctx->stream) {
            cudaStreamDestroy(ctx->stream);
        }
        return rc;
    }
    *out = ctx.release();
    return VFPS_OK;
}

extern "C" int vfps_destroy(vfps_ctx* ctx)
{
    if (!ctx) {
        return VFPS_OK;
    }
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    cudaFree(ctx->d_status);
    cudaStreamDestroy(ctx->stream);
    delete ctx;
    return VFPS_OK;
}

extern "C" const char* vfps_last_error(const vfps_ctx* ctx)
{
    return ctx ? ctx->last_error.c_str() : g_last_error.c_str();
}

extern "C" int vfps_synchronize(vfps_ctx* ctx)
{
    if (!ctx) {
        return null_arg("ctx");
    }
    return guard(ctx, [&] { VFPS_CUDA(cudaStreamSynchronize(ctx->stream)); });
}

extern "C" void* vfps_stream(vfps_ctx* ctx)
{
    return ctx ? static_cast<void*>(ctx->stream) : nullptr;
}

extern "C" int vfps_device_status(vfps_ctx* ctx, int* code)
{
    if (!ctx || !code) {
        return null_arg("ctx/code");
    }
    return guard(ctx, [&] {
        d2h(code, ctx->d_status, 1, ctx);
        VFPS_CUDA(cudaMemsetAsync(ctx->d_status, 0, sizeof(int), ctx->stream));
        VFPS_CUDA(cudaStreamSynchronize(ctx->stream));
    });
}

namespace {
// The wait pattern of the persistent solver kernels on barriers that
// nothing arrives at: a CTA walks `tiles` tiles; at each, every thread
// waits for the tile's barrier phase, bounded by limit_ns, then waits once
// more (for a copy that might still land); the CTA then decides together
// (__syncthreads_or) and stops walking at the first tile whose wait ran
// out, records VFPS_ERR_TIMEOUT and returns (no copy in flight, no tensor
// memory held).  So the kernel ends after about two wait limits, not two
// per tile.
__global__ void k_wait_selftest(int* status, unsigned long long limit_ns,
                                int tiles)
{
    __shared__ uint64_t bar[2];
    if (threadIdx.x == 0) {
        vfps::dev::mbar_init(&bar[0], 1);
        vfps::dev::mbar_init(&bar[1], 1);
        vfps::dev::mbar_fence_init();
    }
    __syncthreads();
    int bad = 0;
    for (int k = 0; k < tiles; k++) {
        if (!vfps::dev::mbar_wait_bounded(&bar[k & 1], (k >> 1) & 1,
                                          limit_ns)) {
            bad = 1;
            vfps::dev::mbar_wait_bounded(&bar[k & 1], (k >> 1) & 1,
                                         limit_ns);
        }
        if (__syncthreads_or(bad)) {
            bad = 1;
            break;
        }
    }
    if (bad && threadIdx.x == 0) {
        atomicCAS(status, 0, VFPS_ERR_TIMEOUT);
    }
}
}  // namespace

extern "C" int vfps_selftest_wait_timeout(vfps_ctx* ctx, uint64_t limit_ns)
{
    if (!ctx) {
        return null_arg("ctx");
    }
    if (limit_ns == 0 || limit_ns > 1000000000ull) {
        ctx->last_error = "limit must be in (0, 1 s]";
        return VFPS_ERR_INVALID_ARGUMENT;
    }
    return guard(ctx, [&] {
        k_wait_selftest<<<1, 128, 0, ctx->stream>>>(ctx->d_status, limit_ns,
                                                     16);
        VFPS_LAUNCHED();
        VFPS_CUDA(cudaStreamSynchronize(ctx->stream));
    });
}

extern "C" int vfps_host_alloc(vfps_ctx* ctx, size_t bytes, void** ptr)
{
    if (!ctx || !ptr) {
        return null_arg("ctx/ptr");
    }
    return guard(ctx, [&] { VFPS_CUDA(cudaMallocHost(ptr, bytes)); });
}

extern "C" int vfps_host_free(vfps_ctx* ctx, void* ptr)
{
    if (!ctx) {
        return null_arg("ctx");
    }
    return guard(ctx, [&] { VFPS_CUDA(cudaFreeHost(ptr)); });
}

/* ============================================================ PhaseSpace */
namespace {

std::vector<float> simpson_weights(uint32_t n, float delta)
{
    // src/PS/PhaseSpace.cpp:486-501
    std::vector<float> ws(n);
    const float ca = 3;
    float dc = 1;
    const float h03 = delta / 3.f;
    ws[0] = h03;
    for (uint32_t x = 1; x + 1 < n; x++) {
        ws[x] = h03 * (ca + dc);
        dc = -dc;
    }
    ws[n - 1] = h03;
    return ws;
}

std::vector<float> gaussian(const vfps::Axis& a, double zoom)
{
    // src/PS/PhaseSpace.cpp:471-484 (exponent in double)
    const double zoom2 = zoom * zoom;
    const float c = 0.398942280401432677939946059934381868f;
    std::vector<float> g(a.n);
    for (uint32_t i = 0; i < a.n; i++) {
        g[i] = static_cast<float>(
            double(c) * std::exp((-0.5) * double(a.v[i]) * double(a.v[i])
                                 / zoom2));
    }
    return g;
}

void ps_alloc(vfps_ps* p)
{
    const size_t nxy = size_t(p->n) * p->n;
    p->data.alloc(nxy * p->nb);
    p->proj[0].alloc(size_t(p->nb) * p->n);
    p->proj[1].alloc(size_t(p->nb) * p->n);
    p->proj64.alloc(size_t(p->nb) * p->n);
    p->ws.alloc(p->n);
    p->axisv[0].alloc(p->n);
    p->axisv[1].alloc(p->n);
    p->fillset.alloc(p->nb);
    p->filling.alloc(p->nb + 1);
    p->moments.alloc(size_t(6) * p->nb);
    vfps_ctx* ctx = p->ctx;
    VFPS_CUDA(cudaMemsetAsync(p->proj[0].p, 0, p->proj[0].bytes(),
                              ctx->stream));
    VFPS_CUDA(cudaMemsetAsync(p->proj[1].p, 0, p->proj[1].bytes(),
                              ctx->stream));
    VFPS_CUDA(cudaMemsetAsync(p->proj64.p, 0, p->proj64.bytes(), ctx->stream));
    VFPS_CUDA(cudaMemsetAsync(p->filling.p, 0, p->filling.bytes(),
                              ctx->stream));
    VFPS_CUDA(cudaMemsetAsync(p->moments.p, 0, p->moments.bytes(),
                              ctx->stream));
    const auto ws = simpson_weights(p->n, p->ax[0].delta);
    h2d(p->ws.p, ws.data(), p->n, ctx);
    h2d(p->axisv[0].p, p->ax[0].v.data(), p->n, ctx);
    h2d(p->axisv[1].p, p->ax[1].v.data(), p->n, ctx);
    h2d(p->fillset.p, p->filling_set.data(), p->nb, ctx);
}

}  // namespace

extern "C" int vfps_ps_create(vfps_ctx* ctx, uint32_t nb, uint32_t n,
                              const double axes[6], double charge,
                              double current, const float* filling,
                              double zoom, const float* data, vfps_ps** ps)
{
    if (!ctx || !ps || !axes || !filling) {
        return null_arg("ctx/ps/axes/filling");
    }
    *ps = nullptr;
    return guard(ctx, [&] {
        VFPS_REQUIRE(nb >= 1, "a phase space needs at least one bunch");
        VFPS_REQUIRE(n >= 2, "mesh size must be at least 2");
        // src/PS/PhaseSpace.cpp:47-51
        float fsum = 0;
        for (uint32_t b = 0; b < nb; b++) {
            fsum += filling[b];
        }
        VFPS_REQUIRE(std::round(1e5 * fsum) == 1e5,
                     "Argument \"filling\" not normalized.");
        auto p = std::make_unique<vfps_ps>();
        p->ctx = ctx;
        p->device = ctx->device;
        p->nb = nb;
        p->n = n;
        p->charge = charge;
        p->current = current;
        p->ax[0] = vfps::make_axis(n, float(axes[0]), float(axes[1]),
                                   float(axes[2]));
        p->ax[1] = vfps::make_axis(n, float(axes[3]), float(axes[4]),
                                   float(axes[5]));
        p->filling_set.assign(filling, filling + nb);
        ps_alloc(p.get());
        const size_t nxy = size_t(n) * n;
        if (data) {
            h2d(p->data.p, data, nxy * nb, ctx);
        } else {
            const auto gx = gaussian(p->ax[0], zoom);
            const auto gy = gaussian(p->ax[1], zoom);
            DevBuf<float> g(2 * size_t(n));
            h2d(g.p, gx.data(), n, ctx);
            h2d(g.p + n, gy.data(), n, ctx);
            vfps::launch_fill_gaussian(p.get(), g.p, g.p + n);
            // createFromProjections: project, integrate, normalize
            vfps::launch_project_x(p.get(), nullptr);
            vfps::launch_integrate(p.get());
            vfps::launch_normalize(p.get());
            VFPS_CUDA(cudaStreamSynchronize(ctx->stream));
        }
        vfps::launch_project_x(p.get(), nullptr);
        vfps::launch_project_y(p.get());
        vfps::launch_integrate(p.get());
        VFPS_CUDA(cudaStreamSynchronize(ctx->stream));
        *ps = p.release();
    });
}

extern "C" int vfps_ps_copy(const vfps_ps* src, vfps_ps** ps)
{
    if (!src || !ps) {
        return null_arg("src/ps");
    }
    *ps = nullptr;
    vfps_ctx* ctx = src->ctx;
    return guard(ctx, [&] {
        auto p = std::make_unique<vfps_ps>();
        p->ctx = ctx;
        p->device = ctx->device;
        p->nb = src->nb;
        p->n = src->n;
        p->charge = src->charge;
        p->current = src->current;
        p->ax[0] = src->ax[0];
        p->ax[1] = src->ax[1];
        p->filling_set = src->filling_set;
        ps_alloc(p.get());
        VFPS_CUDA(cudaMemcpyAsync(p->data.p, src->data.p, src->data.bytes(),
                                  cudaMemcpyDeviceToDevice, ctx->stream));
        vfps::launch_project_x(p.get(), nullptr);
        vfps::launch_project_y(p.get());
        vfps::launch_integrate(p.get());
        VFPS_CUDA(cudaStreamSynchronize(ctx->stream));
        *ps = p.release();
    });
}

extern "C" int vfps_ps_destroy(vfps_ps* ps)
{
    if (!ps) {
        return VFPS_OK;
    }
    // device buffers are released with cudaFree, which waits for the
    // device; nothing else is dereferenced (other objects may be gone)
    cudaSetDevice(ps->device);
    delete ps;
    return VFPS_OK;
}

extern "C" int vfps_ps_swap(vfps_ps* a, vfps_ps* b)
{
    if (!a || !b) {
        return null_arg("a/b");
    }
    return guard(a->ctx, [&] {
        VFPS_REQUIRE(a->n == b->n && a->nb == b->nb,
                     "swap needs phase spaces of equal size");
        a->data.swap(b->data);
    });
}

extern "C" int vfps_ps_assign(vfps_ps* dst, const vfps_ps* src)
{
    if (!dst || !src) {
        return null_arg("dst/src");
    }
    return guard(dst->ctx, [&] {
        VFPS_REQUIRE(dst->n == src->n && dst->nb == src->nb,
                     "assignment needs phase spaces of equal size");
        if (dst != src) {
            VFPS_CUDA(cudaMemcpyAsync(dst->data.p, src->data.p,
                                      src->data.bytes(),
                                      cudaMemcpyDeviceToDevice,
                                      dst->ctx->stream));
            VFPS_CUDA(cudaStreamSynchronize(dst->ctx->stream));
        }
    });
}

extern "C" int vfps_ps_download(vfps_ps* ps, float* data)
{
    if (!ps || !data) {
        return null_arg("ps/data");
    }
    return guard(ps->ctx, [&] { d2h(data, ps->data.p, ps->data.n, ps->ctx); });
}

extern "C" int vfps_ps_upload(vfps_ps* ps, const float* data)
{
    if (!ps || !data) {
        return null_arg("ps/data");
    }
    return guard(ps->ctx, [&] { h2d(ps->data.p, data, ps->data.n, ps->ctx); });
}

extern "C" float* vfps_ps_device_data(vfps_ps* ps)
{
    return ps ? ps->data.p : nullptr;
}

extern "C" int vfps_ps_shape(const vfps_ps* ps, uint32_t* nb, uint32_t* n)
{
    if (!ps) {
        return null_arg("ps");
    }
    if (nb) {
        *nb = ps->nb;
    }
    if (n) {
        *n = ps->n;
    }
    return VFPS_OK;
}

extern "C" int vfps_ps_axis(const vfps_ps* ps, int axis, float* values,
                            float* delta, float* zerobin)
{
    if (!ps || (axis != 0 && axis != 1)) {
        return null_arg("ps/axis");
    }
    const vfps::Axis& a = ps->ax[axis];
    if (values) {
        std::copy(a.v.begin(), a.v.end(), values);
    }
    if (delta) {
        *delta = a.delta;
    }
    if (zerobin) {
        *zerobin = a.zerobin;
    }
    return VFPS_OK;
}

extern "C" int vfps_ps_update_x_projection(vfps_ps* ps)
{
    if (!ps) {
        return null_arg("ps");
    }
    return guard(ps->ctx, [&] { vfps::launch_project_x(ps, nullptr); });
}

extern "C" int vfps_ps_update_y_projection(vfps_ps* ps)
{
    if (!ps) {
        return null_arg("ps");
    }
    return guard(ps->ctx, [&] { vfps::launch_project_y(ps); });
}

extern "C" int vfps_ps_integrate(vfps_ps* ps)
{
    if (!ps) {
        return null_arg("ps");
    }
    return guard(ps->ctx, [&] { vfps::launch_integrate(ps); });
}

extern "C" int vfps_ps_normalize(vfps_ps* ps)
{
    if (!ps) {
        return null_arg("ps");
    }
    return guard(ps->ctx, [&] { vfps::launch_normalize(ps); });
}

extern "C" int vfps_ps_integrate_and_normalize(vfps_ps* ps)
{
    if (!ps) {
        return null_arg("ps");
    }
    return guard(ps->ctx, [&] {
        vfps::launch_integrate(ps);
        vfps::launch_normalize(ps);
    });
}

extern "C" int vfps_ps_variance(vfps_ps* ps, int axis)
{
    if (!ps || (axis != 0 && axis != 1)) {
        return null_arg("ps/axis");
    }
    return guard(ps->ctx, [&] { vfps::launch_moments(ps, axis); });
}

extern "C" int vfps_ps_get_projection(vfps_ps* ps, int axis, float* proj)
{
    if (!ps || !proj || (axis != 0 && axis != 1)) {
        return null_arg("ps/proj/axis");
    }
    return guard(ps->ctx,
                 [&] { d2h(proj, ps->proj[axis].p, ps->proj[axis].n, ps->ctx); });
}

extern "C" int vfps_ps_set_projection(vfps_ps* ps, int axis, uint32_t bunch,
                                      const float* proj)
{
    if (!ps || !proj || (axis != 0 && axis != 1)) {
        return null_arg("ps/proj/axis");
    }
    return guard(ps->ctx, [&] {
        VFPS_REQUIRE(bunch < ps->nb, "bunch index out of range");
        h2d(ps->proj[axis].p + size_t(bunch) * ps->n, proj, ps->n, ps->ctx);
        if (axis == 0) {
            std::vector<double> p64(proj, proj + ps->n);
            h2d(ps->proj64.p + size_t(bunch) * ps->n, p64.data(), ps->n,
                ps->ctx);
        }
    });
}

extern "C" int vfps_ps_get_filling(vfps_ps* ps, float* filling,
                                   double* integral)
{
    if (!ps) {
        return null_arg("ps");
    }
    return guard(ps->ctx, [&] {
        std::vector<double> f(ps->nb + 1);
        d2h(f.data(), ps->filling.p, ps->nb + 1, ps->ctx);
        if (filling) {
            for (uint32_t b = 0; b < ps->nb; b++) {
                filling[b] = static_cast<float>(f[b]);
            }
        }
        if (integral) {
            *integral = f[ps->nb];
        }
    });
}

extern "C" int vfps_ps_get_moments(vfps_ps* ps, int axis, float* average,
                                   float* variance, float* rms)
{
    if (!ps || (axis != 0 && axis != 1)) {
        return null_arg("ps/axis");
    }
    return guard(ps->ctx, [&] {
        std::vector<float> m(3 * size_t(ps->nb));
        d2h(m.data(), ps->moments.p + size_t(axis) * 3 * ps->nb, m.size(),
            ps->ctx);
        for (uint32_t b = 0; b < ps->nb; b++) {
            if (average) {
                average[b] = m[b];
            }
            if (variance) {
                variance[b] = m[ps->nb + b];
            }
            if (rms) {
                rms[b] = m[2 * ps->nb + b];
            }
        }
    });
}

/* ============================================================ SourceMaps */
namespace {

void check_pair(const vfps_ps* in, const vfps_ps* out)
{
    VFPS_REQUIRE(in && out, "map needs input and output phase spaces");
    VFPS_REQUIRE(in->n == out->n && in->nb == out->nb,
                 "map input and output must have the same size");
    VFPS_REQUIRE(in->ctx == out->ctx, "map input and output on one context");
}

void check_it(int it)
{
    VFPS_REQUIRE(it >= 1 && it <= 4, "interpolation points must be 1..4");
}

std::unique_ptr<vfps_map> new_kick(vfps_ps* in, vfps_ps* out, int it,
                                   int clamp, int axis)
{
    check_pair(in, out);
    check_it(it);
    VFPS_REQUIRE(axis == VFPS_AXIS_X || axis == VFPS_AXIS_Y, "bad axis");
    auto m = std::make_unique<vfps_map>();
    m->device = in->ctx->device;
    m->kind = MAP_KICK;
    m->in = in;
    m->out = out;
    m->it = it;
    m->clamp = clamp ? 1 : 0;
    m->axis = axis;
    const size_t count = (axis == VFPS_AXIS_X) ? in->n : size_t(in->nb) * in->n;
    m->offset.alloc(count);
    m->host_offset.assign(count, 0.f);
    h2d(m->offset.p, m->host_offset.data(), count, in->ctx);
    return m;
}

void upload_offset(vfps_map* m, const std::vector<float>& off)
{
    VFPS_REQUIRE(off.size() == m->offset.n, "offset has the wrong length");
    m->host_offset = off;
    m->host_offset_valid = true;
    m->xtab_valid = false;
    h2d(m->offset.p, off.data(), off.size(), m->in->ctx);
}

}  // namespace

extern "C" int vfps_rotation_map_create(vfps_ps* in, vfps_ps* out,
                                        uint32_t xsize, uint32_t ysize,
                                        float angle, int it, int clamp,
                                        uint32_t rotmapsize, vfps_map** map)
{
    if (!in || !out || !map) {
        return null_arg("in/out/map");
    }
    *map = nullptr;
    return guard(in->ctx, [&] {
        check_pair(in, out);
        check_it(it);
        VFPS_REQUIRE(xsize == in->n && ysize == in->n,
                     "RotationMap size must match the mesh");
        VFPS_REQUIRE(rotmapsize == 0 || rotmapsize == xsize * ysize,
                     "rotmapsize must be 0 or xsize*ysize");
        // src/SM/RotationMap.cpp:83-87
        VFPS_REQUIRE(!clamp || (it == VFPS_INTERP_CUBIC && rotmapsize > 0),
                     "Clamping only supportedwith cubic interpolationand "
                     "rotmapsize > 0.");
        auto m = std::make_unique<vfps_map>();
        m->device = in->ctx->device;
        m->kind = MAP_ROTATION;
        m->in = in;
        m->out = out;
        m->it = it;
        m->clamp = clamp ? 1 : 0;
        m->angle = angle;
        m->cs = std::cos(-angle);
        m->sn = std::sin(-angle);
        *map = m.release();
    });
}

extern "C" int vfps_kick_map_create(vfps_ps* in, vfps_ps* out, int it,
                                    int clamp, int axis, vfps_map** map)
{
    if (!in || !out || !map) {
        return null_arg("in/out/map");
    }
    *map = nullptr;
    return guard(in->ctx,
                 [&] { *map = new_kick(in, out, it, clamp, axis).release(); });
}

extern "C" int vfps_kick_map_set_offset(vfps_map* map, const float* offset,
                                        size_t count)
{
    if (!map || !offset) {
        return null_arg("map/offset");
    }
    return guard(map->in->ctx, [&] {
        VFPS_REQUIRE(map->kind == MAP_KICK && !map->field,
                     "not a kick map with settable offsets");
        upload_offset(map, std::vector<float>(offset, offset + count));
    });
}

extern "C" int vfps_kick_map_get_offset(vfps_map* map, float* offset,
                                        size_t count)
{
    if (!map || !offset) {
        return null_arg("map/offset");
    }
    return guard(map->in->ctx, [&] {
        VFPS_REQUIRE(map->kind == MAP_KICK, "not a kick map");
        const float* src = map->field ? map->field->wake.p : map->offset.p;
        const size_t n = map->field ? map->field->wake.n : map->offset.n;
        VFPS_REQUIRE(count == n, "offset has the wrong length");
        d2h(offset, src, n, map->in->ctx);
    });
}

extern "C" int vfps_drift_map_create(vfps_ps* in, vfps_ps* out,
                                     const float* slip, uint32_t nslip,
                                     float e0, int it, int clamp,
                                     vfps_map** map)
{
    if (!in || !out || !map || (nslip && !slip)) {
        return null_arg("in/out/map/slip");
    }
    *map = nullptr;
    return guard(in->ctx, [&] {
        auto m = new_kick(in, out, it, clamp, VFPS_AXIS_X);
        // src/SM/DriftMap.cpp:21-30
        const vfps::Axis& ax = in->ax[0];
        const vfps::Axis& ay = in->ax[1];
        std::vector<float> off(in->n);
        for (uint32_t y = 0; y < in->n; y++) {
            off[y] = 0;
            for (uint32_t i = 0; i < nslip; i++) {
                off[y] += slip[i] * ay.v[y]
                          * std::pow(ay.v[y] * ay.scale / e0,
                                     static_cast<float>(i));
            }
            off[y] /= ax.delta;
        }
        upload_offset(m.get(), off);
        *map = m.release();
    });
}

extern "C" int vfps_rf_kick_map_create_linear(vfps_ps* in, vfps_ps* out,
                                              float angle, float f_rf, int it,
                                              int clamp, vfps_map** map)
{
    if (!in || !out || !map) {
        return null_arg("in/out/map");
    }
    *map = nullptr;
    return guard(in->ctx, [&] {
        auto m = new_kick(in, out, it, clamp, VFPS_AXIS_Y);
        // src/SM/RFKickMap.cpp:15-32,59-68 with phase = syncphase = 0
        const vfps::Axis& ax = in->ax[0];
        const float bl2phase = static_cast<float>(
            double(ax.scale) / C_LIGHT * double(f_rf) * 2 * PI);
        const float phaseoffs = 0;
        const float xcenter = ax.zerobin;
        std::vector<float> off(size_t(in->nb) * in->n, 0.f);
        for (uint32_t x = 0; x < in->n; x++) {
            off[x] = std::tan(angle) * (xcenter - static_cast<float>(x));
            off[x] += std::tan(angle) * phaseoffs / bl2phase / ax.delta;
            off[x] *= 1.f;
        }
        for (uint32_t b = 1; b < in->nb; b++) {
            std::copy(off.begin(), off.begin() + in->n, off.begin() + b * in->n);
        }
        upload_offset(m.get(), off);
        *map = m.release();
    });
}

extern "C" int vfps_rf_kick_map_create(vfps_ps* in, vfps_ps* out,
                                       float revolutionpart, float v_rf,
                                       float f_rf, float v0, int it, int clamp,
                                       vfps_map** map)
{
    if (!in || !out || !map) {
        return null_arg("in/out/map");
    }
    *map = nullptr;
    return guard(in->ctx, [&] {
        auto m = new_kick(in, out, it, clamp, VFPS_AXIS_Y);
        // src/SM/RFKickMap.cpp:34-57,69-78
        const vfps::Axis& ax = in->ax[0];
        const vfps::Axis& ay = in->ax[1];
        const float syncphase = std::asin(v0 / v_rf);
        const float bl2phase = static_cast<float>(
            double(ax.scale) / C_LIGHT * double(f_rf) * 2 * PI);
        std::vector<float> off(size_t(in->nb) * in->n, 0.f);
        for (uint32_t x = 0; x < in->n; x++) {
            off[x] = revolutionpart
                     * (-1.f * v_rf * std::sin(ax.v[x] * bl2phase + syncphase)
                        + v0)
                     / ay.delta / ay.scale;
        }
        for (uint32_t b = 1; b < in->nb; b++) {
            std::copy(off.begin(), off.begin() + in->n, off.begin() + b * in->n);
        }
        upload_offset(m.get(), off);
        *map = m.release();
    });
}

extern "C" int vfps_dynamic_rf_kick_map_create(
    vfps_ps* in, vfps_ps* out, int linear, float angle, float revolutionpart,
    float v_rf, float f_rf, float v0, float phasespread, float amplspread,
    float modampl, double modtimeincrement, uint32_t steps, int it,
    int clamp, uint32_t seed, vfps_map** map)
{
    if (!in || !out || !map) {
        return null_arg("in/out/map");
    }
    *map = nullptr;
    return guard(in->ctx, [&] {
        VFPS_REQUIRE(revolutionpart > 0, "revolutionpart must be positive");
        VFPS_REQUIRE(linear || (v_rf != 0 && std::fabs(v0) <= std::fabs(v_rf)),
                     "sinusoidal RF needs |V0| <= |V_RF| != 0");
        auto m = new_kick(in, out, it, clamp, VFPS_AXIS_Y);
        const vfps::Axis& ax = in->ax[0];
        DynRf& d = m->dyn;
        d.linear = linear ? 1 : 0;
        d.angle = angle;
        d.revolutionpart = revolutionpart;
        d.v_rf = v_rf;
        d.v0 = v0;
        // src/SM/RFKickMap.cpp:15-57
        d.syncphase = linear ? 0.f : std::asin(v0 / v_rf);
        d.bl2phase = static_cast<float>(double(ax.scale) / C_LIGHT
                                        * double(f_rf) * 2 * PI);
        // src/SM/DynamicRFKickMap.cpp:31-38
        d.phasenoise = phasespread / std::sqrt(revolutionpart);
        d.amplnoise = amplspread / std::sqrt(revolutionpart);
        d.modampl = modampl;
        d.modtimedelta = 2 * PI * modtimeincrement;
        d.seed = seed;
        m->dynrf = true;
        m->dyn_cap = steps;
        m->dyn_log.alloc(std::max<size_t>(2 * size_t(steps), 2));
        m->axis_q.alloc(in->n);
        h2d(m->axis_q.p, ax.v.data(), in->n, in->ctx);
        m->host_offset_valid = false;
        *map = m.release();
    });
}

extern "C" int vfps_dynamic_rf_get_modulation(vfps_map* map, float* out,
                                              uint64_t* count)
{
    if (!map || !map->dynrf) {
        return null_arg("map (a dynamic RF kick map)");
    }
    return guard(map->in->ctx, [&] {
        const uint64_t c = std::min(map->dyn_step, map->dyn_cap);
        if (count) {
            *count = c;
        }
        if (out && c) {
            d2h(out, map->dyn_log.p, 2 * c, map->in->ctx);
        }
    });
}

extern "C" int vfps_philox4x32(const uint32_t* counter, const uint32_t* key,
                               uint32_t* out)
{
    if (!counter || !key || !out) {
        return VFPS_ERR_INVALID_ARGUMENT;
    }
    philox4x32_10(counter, key, out);
    return VFPS_OK;
}

extern "C" int vfps_fokker_planck_map_create(vfps_ps* in, vfps_ps* out,
                                             uint32_t xsize, uint32_t ysize,
                                             int fptype, int fptrack, float e1,
                                             int derivation, vfps_map** map)
{
    if (!in || !out || !map) {
        return null_arg("in/out/map");
    }
    *map = nullptr;
    return guard(in->ctx, [&] {
        check_pair(in, out);
        VFPS_REQUIRE(xsize == in->n && ysize == in->n,
                     "FokkerPlanckMap size must match the mesh");
        VFPS_REQUIRE(derivation == 3 || derivation == 4,
                     "derivation must be 3 (two-sided) or 4 (cubic)");
        VFPS_REQUIRE(fptype >= 0 && fptype <= 3, "bad FPType");
        auto m = std::make_unique<vfps_map>();
        m->device = in->ctx->device;
        m->kind = MAP_FP;
        m->in = in;
        m->out = out;
        m->ip = derivation;
        m->fptrack = fptrack;
        m->e1 = e1;
        // src/SM/FokkerPlanckMap.cpp:11-118
        const uint32_t n = in->n;
        const vfps::Axis& ay = in->ax[1];
        const int ip = derivation;
        std::vector<uint32_t> idx(size_t(n) * ip, 0);
        std::vector<float> w(size_t(n) * ip, 0.f);
        const float e1_2d = e1 / (2.f * ay.delta);
        const float e1_6d = e1 / (6.f * ay.delta);
        const float e1_d2 = e1 / (ay.delta * ay.delta);
        const bool damp = fptype != VFPS_FP_NONE
                          && fptype != VFPS_FP_DIFFUSION_ONLY;
        const bool diff = fptype != VFPS_FP_NONE
                          && fptype != VFPS_FP_DAMPING_ONLY;
        if (derivation == 3) {
            for (uint32_t j = 1; j + 1 < n; j++) {
                uint32_t* I = &idx[j * 3];
                float* W = &w[j * 3];
                I[0] = j - 1; W[0] = 0;
                I[1] = j;     W[1] = 1;
                I[2] = j + 1; W[2] = 0;
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
            }
        } else {
            const float ycenter = ay.zerobin;
            for (uint32_t j = 2; static_cast<float>(j) < ycenter; j++) {
                const float pos = ay.v[j];
                uint32_t* I = &idx[j * 4];
                float* W = &w[j * 4];
                I[0] = j - 2; W[0] = 0;
                I[1] = j - 1; W[1] = 0;
                I[2] = j;     W[2] = 1;
                I[3] = j + 1; W[3] = 0;
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
            }
            for (uint32_t j = static_cast<uint32_t>(ycenter); j + 2 < n; j++) {
                const float pos = ay.v[j];
                uint32_t* I = &idx[j * 4];
                float* W = &w[j * 4];
                I[0] = j - 1; W[0] = 0;
                I[1] = j;     W[1] = 1;
                I[2] = j + 1; W[2] = 0;
                I[3] = j + 2; W[3] = 0;
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
            }
            const uint32_t zero_rows[4] = {0u, 1u, n - 2, n - 1};
            for (uint32_t j : zero_rows) {
                if (j < n) {
                    for (int k = 0; k < 4; k++) {
                        idx[j * 4 + k] = 0;
                        w[j * 4 + k] = 0;
                    }
                }
            }
        }
        if (derivation == 3) {
            for (int k = 0; k < 3; k++) {
                idx[k] = 0;
                w[k] = 0;
                idx[(n - 1) * 3 + k] = 0;
                w[(n - 1) * 3 + k] = 0;
            }
        }
        m->h_fp_idx = idx;
        m->h_fp_w = w;
        m->fp_idx.alloc(idx.size());
        m->fp_w.alloc(w.size());
        h2d(m->fp_idx.p, idx.data(), idx.size(), in->ctx);
        h2d(m->fp_w.p, w.data(), w.size(), in->ctx);
        // the same tables tap-major [4][n] (a missing 4th tap: index 0,
        // weight 0) for the row-sweep kernel's 16-byte reads
        std::vector<uint32_t> it4(size_t(4) * n, 0u);
        std::vector<float> wt4(size_t(4) * n, 0.f);
        for (uint32_t y = 0; y < n; y++) {
            for (int k = 0; k < derivation; k++) {
                it4[size_t(k) * n + y] = idx[size_t(y) * derivation + k];
                wt4[size_t(k) * n + y] = w[size_t(y) * derivation + k];
            }
        }
        m->fp_idx4.alloc(it4.size());
        m->fp_w4.alloc(wt4.size());
        h2d(m->fp_idx4.p, it4.data(), it4.size(), in->ctx);
        h2d(m->fp_w4.p, wt4.data(), wt4.size(), in->ctx);
        *map = m.release();
    });
}

extern "C" int vfps_identity_map_create(vfps_ps* in, vfps_ps* out,
                                        vfps_map** map)
{
    if (!in || !out || !map) {
        return null_arg("in/out/map");
    }
    *map = nullptr;
    return guard(in->ctx, [&] {
        check_pair(in, out);
        auto m = std::make_unique<vfps_map>();
        m->device = in->ctx->device;
        m->kind = MAP_IDENTITY;
        m->in = in;
        m->out = out;
        *map = m.release();
    });
}

extern "C" int vfps_wake_potential_map_create(vfps_ps* in, vfps_ps* out,
                                              vfps_field* field, int it,
                                              int clamp, vfps_map** map)
{
    if (!in || !out || !map || !field) {
        return null_arg("in/out/map/field");
    }
    *map = nullptr;
    return guard(in->ctx, [&] {
        VFPS_REQUIRE(field->ps->n == in->n && field->ps->nb == in->nb,
                     "field and map meshes differ");
        auto m = new_kick(in, out, it, clamp, VFPS_AXIS_Y);
        m->field = field;
        m->offset_src = field->wake.p;
        m->host_offset_valid = false;
        *map = m.release();
    });
}

extern "C" int vfps_wake_map_update(vfps_map* map)
{
    if (!map) {
        return null_arg("map");
    }
    return guard(map->in->ctx, [&] {
        VFPS_REQUIRE(map->field, "not a wake kick map");
        vfps::launch_wake(map->field);
        map->host_offset_valid = false;
    });
}

extern "C" int vfps_map_apply(vfps_map* map)
{
    if (!map) {
        return null_arg("map");
    }
    return guard(map->in->ctx, [&] {
        switch (map->kind) {
        case MAP_ROTATION:
            vfps::launch_rotation(map);
            break;
        case MAP_KICK:
            if (map->dynrf) {
                vfps::launch_dynrf(map);
                map->host_offset_valid = false;
            }
            vfps::launch_kick(map, map->field ? map->offset_src
                                              : map->offset.p);
            break;
        case MAP_FP:
            vfps::launch_fp(map);
            break;
        case MAP_IDENTITY:
            if (map->in != map->out) {
                VFPS_CUDA(cudaMemcpyAsync(map->out->data.p, map->in->data.p,
                                          map->in->data.bytes(),
                                          cudaMemcpyDeviceToDevice,
                                          map->in->ctx->stream));
            }
            break;
        }
    });
}

namespace {
thread_local std::mt19937 g_prng{std::random_device{}()};
}

extern "C" int vfps_map_apply_to(vfps_map* map, float* pos, size_t count)
{
    if (!map || (count && !pos)) {
        return null_arg("map/pos");
    }
    return guard(map->in->ctx, [&] {
        const vfps_ps* ps = map->in;
        const uint32_t n = ps->n;
        switch (map->kind) {
        case MAP_ROTATION: {
            // src/SM/RotationMap.cpp:178-188
            const float zx = ps->ax[0].zerobin, zy = ps->ax[1].zerobin;
            for (size_t i = 0; i < count; i++) {
                float& px = pos[2 * i];
                float& py = pos[2 * i + 1];
                const float tx = map->cs * (px - zx) + map->sn * (py - zy) + zx;
                const float ty = map->cs * (py - zy) - map->sn * (px - zx) + zy;
                px = tx;
                py = ty;
            }
            break;
        }
        case MAP_KICK: {
            // src/SM/KickMap.cpp:280-303 (offsets of bunch 0)
            if (!map->host_offset_valid) {
                // the wake map's offsets live in its field, the others' in
                // the map (the dynamic RF map rewrites them every apply)
                const float* src = map->field ? map->field->wake.p
                                              : map->offset.p;
                const size_t cnt = map->field ? map->field->wake.n
                                              : map->offset.n;
                map->host_offset.resize(cnt);
                d2h(map->host_offset.data(), src, cnt, ps->ctx);
                map->host_offset_valid = true;
            }
            const auto& off = map->host_offset;
            for (size_t i = 0; i < count; i++) {
                float& along = map->axis == VFPS_AXIS_X ? pos[2 * i]
                                                        : pos[2 * i + 1];
                const float across = map->axis == VFPS_AXIS_X ? pos[2 * i + 1]
                                                              : pos[2 * i];
                float ip;
                const float f = std::modf(across, &ip);
                uint32_t k;
                if (host_base(ip, 0xffffffffu, &k) && k + 1 < n) {
                    along -= (1 - f) * off[k] + f * off[k + 1];
                }
                along = std::max(1.f, std::min(along, static_cast<float>(n - 1)));
            }
            break;
        }
        case MAP_FP: {
            // src/SM/FokkerPlanckMap.cpp:214-268
            const int ip = map->ip;
            if (map->fptrack == 1) {
                for (size_t i = 0; i < count; i++) {
                    float& py = pos[2 * i + 1];
                    uint32_t yi = std::min(static_cast<uint32_t>(
                                               std::max(0.f, std::floor(py))),
                                           n - 1);
                    float offset = 0;
                    for (int j = 0; j < ip; j++) {
                        const float dy = static_cast<float>(yi)
                                         - static_cast<float>(
                                             map->h_fp_idx[yi * ip + j]);
                        offset += dy * map->h_fp_w[yi * ip + j];
                    }
                    py = std::max(1.f, std::min(py + offset,
                                                static_cast<float>(n - 1)));
                }
            } else if (map->fptrack == 2) {
                std::vector<float> d(size_t(n) * n);
                d2h(d.data(), ps->data.p, d.size(), ps->ctx);
                for (size_t i = 0; i < count; i++) {
                    const float px = pos[2 * i];
                    float& py = pos[2 * i + 1];
                    const long xi = std::min(static_cast<long>(std::floor(px)),
                                             static_cast<long>(n) - 1);
                    const long yi = std::min(static_cast<long>(std::floor(py)),
                                             static_cast<long>(n) - 1);
                    if (xi < 0 || yi < 0) {
                        continue;
                    }
                    float offset = 0, charge = 0;
                    for (int j = 0; j < ip; j++) {
                        const uint32_t hi = map->h_fp_idx[yi * ip + j];
                        const float v = d[size_t(xi) * n + hi]
                                        * map->h_fp_w[yi * ip + j];
                        charge += v;
                        offset += v * (static_cast<long>(hi) - yi);
                    }
                    offset /= charge;
                    py = std::max(1.f, std::min(py + offset,
                                                static_cast<float>(n - 1)));
                }
            } else if (map->fptrack == 3) {
                std::normal_distribution<float> nd(
                    0.f, std::sqrt(2 * map->e1) / ps->ax[1].delta);
                for (size_t i = 0; i < count; i++) {
                    float& py = pos[2 * i + 1];
                    py -= py * map->e1 + nd(g_prng);
                }
            }
            break;
        }
        case MAP_IDENTITY:
            break;
        }
    });
}

extern "C" int vfps_map_destroy(vfps_map* map)
{
    if (!map) {
        return VFPS_OK;
    }
    cudaSetDevice(map->device);
    delete map;
    return VFPS_OK;
}

/* ============================================================= Impedance */
namespace {

std::unique_ptr<vfps_impedance> new_imp(vfps_ctx* ctx, size_t n, double fmax)
{
    VFPS_REQUIRE(n >= 2, "an impedance needs at least 2 frequencies");
    auto z = std::make_unique<vfps_impedance>();
    z->ctx = ctx;
    z->device = ctx->device;
    z->nfreqs = n;
    z->f_max = fmax;
    z->z.alloc(2 * n);
    VFPS_CUDA(cudaMemsetAsync(z->z.p, 0, z->z.bytes(), ctx->stream));
    return z;
}

void z_model(vfps_impedance* z, int model, std::vector<double> prm)
{
    prm.resize(7, 0.0);
    vfps::launch_z_model(z->ctx, model, z->nfreqs, prm.data(), z->z.p);
    VFPS_CUDA(cudaStreamSynchronize(z->ctx->stream));
}

// Impedance::readData (src/Z/Impedance.cpp:94-111): "lineno re im" rows; a
// repeated line number does not add an entry.
std::vector<float> read_impedance_file(const char* path)
{
    std::ifstream is(path);
    if (!is) {
        throw vfps::Error(VFPS_ERR_IO,
                          std::string("cannot open impedance file ") + path);
    }
    std::vector<float> z;
    size_t lineno;
    size_t old = std::numeric_limits<size_t>::max();
    float re, im;
    while (is >> lineno >> re >> im) {
        if (lineno != old) {
            z.push_back(re);
            z.push_back(im);
        }
        old = lineno;
    }
    return z;
}

}  // namespace

extern "C" int vfps_impedance_create(vfps_ctx* ctx, const float* zt,
                                     size_t nfreqs, double f_max,
                                     vfps_impedance** imp)
{
    if (!ctx || !imp || !zt) {
        return null_arg("ctx/imp/z");
    }
    *imp = nullptr;
    return guard(ctx, [&] {
        auto z = new_imp(ctx, nfreqs, f_max);
        h2d(z->z.p, zt, 2 * nfreqs, ctx);
        *imp = z.release();
    });
}

extern "C" int vfps_impedance_free_space_csr(vfps_ctx* ctx, size_t n,
                                             float f_rev, float f_max,
                                             vfps_impedance** imp)
{
    if (!ctx || !imp) {
        return null_arg("ctx/imp");
    }
    *imp = nullptr;
    return guard(ctx, [&] {
        auto z = new_imp(ctx, n, f_max);
        z_model(z.get(), 0, {double(f_rev), double(f_max)});
        *imp = z.release();
    });
}

extern "C" int vfps_impedance_parallel_plates_csr(vfps_ctx* ctx, size_t n,
                                                  float f0, float f_max,
                                                  double g,
                                                  vfps_impedance** imp)
{
    if (!ctx || !imp) {
        return null_arg("ctx/imp");
    }
    *imp = nullptr;
    return guard(ctx, [&] {
        VFPS_REQUIRE(g > 0, "parallel plates need a positive gap");
        auto z = new_imp(ctx, n, f_max);
        z_model(z.get(), 1, {double(f0), double(f_max), g, Z0_PHYS});
        *imp = z.release();
    });
}

extern "C" int vfps_impedance_resistive_wall(vfps_ctx* ctx, size_t n,
                                             float f0, float f_max, double L,
                                             double s, double xi, double b,
                                             vfps_impedance** imp)
{
    if (!ctx || !imp) {
        return null_arg("ctx/imp");
    }
    *imp = nullptr;
    return guard(ctx, [&] {
        auto z = new_imp(ctx, n, f_max);
        z_model(z.get(), 2, {double(f0), double(f_max), L, s, xi, b, Z0_IMP});
        *imp = z.release();
    });
}

extern "C" int vfps_impedance_const(vfps_ctx* ctx, size_t n, float f_max,
                                    float re, float im, vfps_impedance** imp)
{
    if (!ctx || !imp) {
        return null_arg("ctx/imp");
    }
    *imp = nullptr;
    return guard(ctx, [&] {
        auto z = new_imp(ctx, n, f_max);
        z_model(z.get(), 3, {double(re), double(im)});
        *imp = z.release();
    });
}

extern "C" int vfps_impedance_collimator(vfps_ctx* ctx, size_t n, float f_max,
                                         double outer, double inner,
                                         vfps_impedance** imp)
{
    const float re = static_cast<float>(Z0_IMP / PI * std::log(outer / inner));
    return vfps_impedance_const(ctx, n, f_max, re, 0.f, imp);
}

extern "C" int vfps_impedance_from_file(vfps_ctx* ctx, const char* path,
                                        double f_max, vfps_impedance** imp)
{
    if (!ctx || !imp || !path) {
        return null_arg("ctx/imp/path");
    }
    *imp = nullptr;
    return guard(ctx, [&] {
        const auto zt = read_impedance_file(path);
        auto z = new_imp(ctx, zt.size() / 2, f_max);
        h2d(z->z.p, zt.data(), zt.size(), ctx);
        *imp = z.release();
    });
}

extern "C" int vfps_make_impedance(vfps_ctx* ctx, size_t nfreqs, float fmax,
                                   double r_bend, double frev, double gap,
                                   int use_csr, double s, double xi,
                                   double inner_coll_radius,
                                   const char* impedance_file,
                                   vfps_impedance** imp)
{
    if (!ctx || !imp) {
        return null_arg("ctx/imp");
    }
    *imp = nullptr;
    return guard(ctx, [&] {
        // src/Z/ImpedanceFactory.cpp:21-84
        const double f0 = C_LIGHT / (2 * PI * r_bend);
        auto acc = new_imp(ctx, nfreqs, fmax);
        bool changed = false;
        auto add = [&](vfps_impedance* t) {
            vfps::launch_z_add(ctx, acc->z.p, t->z.p, nfreqs);
            VFPS_CUDA(cudaStreamSynchronize(ctx->stream));
            changed = true;
        };
        if (gap != 0) {
            if (use_csr) {
                auto t = new_imp(ctx, nfreqs, fmax);
                if (gap > 0) {
                    z_model(t.get(), 1, {double(float(f0)), double(fmax), gap,
                                         Z0_PHYS});
                } else {
                    z_model(t.get(), 0, {double(float(f0)), double(fmax)});
                }
                add(t.get());
            }
            const double radius = std::abs(gap / 2);
            if (s > 0 && xi >= -1) {
                auto t = new_imp(ctx, nfreqs, fmax);
                z_model(t.get(), 2, {double(float(frev)), double(fmax),
                                     C_LIGHT / frev, s, xi, radius, Z0_IMP});
                add(t.get());
            }
            if (0 < inner_coll_radius && inner_coll_radius < radius) {
                auto t = new_imp(ctx, nfreqs, fmax);
                z_model(t.get(), 3,
                        {double(static_cast<float>(
                             Z0_IMP / PI * std::log(radius / inner_coll_radius))),
                         0.0});
                add(t.get());
            }
        }
        if (impedance_file && impedance_file[0]) {
            const auto zt = read_impedance_file(impedance_file);
            VFPS_REQUIRE(zt.size() / 2 >= nfreqs,
                         "impedance file has fewer entries than nfreqs");
            auto t = new_imp(ctx, nfreqs, fmax);
            h2d(t->z.p, zt.data(), 2 * nfreqs, ctx);
            add(t.get());
        }
        if (changed) {
            *imp = acc.release();
        }
    });
}

extern "C" int vfps_impedance_add(vfps_impedance* dst,
                                  const vfps_impedance* rhs)
{
    if (!dst || !rhs) {
        return null_arg("dst/rhs");
    }
    return guard(dst->ctx, [&] {
        VFPS_REQUIRE(dst->nfreqs == rhs->nfreqs,
                     "impedances must have the same number of frequencies");
        vfps::launch_z_add(dst->ctx, dst->z.p, rhs->z.p, dst->nfreqs);
        VFPS_CUDA(cudaStreamSynchronize(dst->ctx->stream));
    });
}

extern "C" int vfps_impedance_copy(const vfps_impedance* src,
                                   vfps_impedance** imp)
{
    if (!src || !imp) {
        return null_arg("src/imp");
    }
    *imp = nullptr;
    return guard(src->ctx, [&] {
        auto z = new_imp(src->ctx, src->nfreqs, src->f_max);
        VFPS_CUDA(cudaMemcpyAsync(z->z.p, src->z.p, src->z.bytes(),
                                  cudaMemcpyDeviceToDevice, src->ctx->stream));
        VFPS_CUDA(cudaStreamSynchronize(src->ctx->stream));
        *imp = z.release();
    });
}

extern "C" int vfps_impedance_swap(vfps_impedance* a, vfps_impedance* b)
{
    if (!a || !b) {
        return null_arg("a/b");
    }
    return guard(a->ctx, [&] {
        VFPS_REQUIRE(a->nfreqs == b->nfreqs,
                     "swap needs impedances of equal size");
        a->z.swap(b->z);
    });
}

extern "C" int vfps_impedance_get(const vfps_impedance* imp, float* z,
                                  size_t* nfreqs, double* f_max)
{
    if (!imp) {
        return null_arg("imp");
    }
    return guard(imp->ctx, [&] {
        if (nfreqs) {
            *nfreqs = imp->nfreqs;
        }
        if (f_max) {
            *f_max = imp->f_max;
        }
        if (z) {
            d2h(z, imp->z.p, 2 * imp->nfreqs, imp->ctx);
        }
    });
}

extern "C" int vfps_impedance_destroy(vfps_impedance* imp)
{
    if (!imp) {
        return VFPS_OK;
    }
    cudaSetDevice(imp->device);
    delete imp;
    return VFPS_OK;
}

/* ========================================================= ElectricField */
extern "C" int vfps_field_create(vfps_ps* ps, const vfps_impedance* imp,
                                 const uint32_t* buckets,
                                 uint32_t spacing_bins, double f_rev,
                                 double revolutionpart, double wakescaling,
                                 vfps_field** field)
{
    if (!ps || !imp || !field) {
        return null_arg("ps/imp/field");
    }
    *field = nullptr;
    vfps_ctx* ctx = ps->ctx;
    return guard(ctx, [&] {
        VFPS_REQUIRE(imp->ctx == ctx, "impedance and phase space contexts");
        auto f = std::make_unique<vfps_field>();
        f->ps = ps;
        f->device = ctx->device;
        f->imp = imp;
        f->nmax = imp->nfreqs;
        f->spacing = spacing_bins;
        f->f_rev = f_rev;
        f->revpart = revolutionpart;
        f->buckets.assign(ps->nb, 0u);
        if (buckets) {
            f->buckets.assign(buckets, buckets + ps->nb);
        }
        std::vector<uint32_t> pos(ps->nb);
        for (uint32_t b = 0; b < ps->nb; b++) {
            const uint64_t p = uint64_t(f->buckets[b]) * spacing_bins;
            VFPS_REQUIRE(p + ps->n <= f->nmax,
                         "bunch profile does not fit into the padded buffer");
            pos[b] = static_cast<uint32_t>(p);
        }
        // ElectricField.cpp:56-58: wakescaling (float) / nmax
        f->wakescale = static_cast<float>(wakescaling)
                       / static_cast<float>(f->nmax);
        f->has_wake = wakescaling != 0;
        const size_t nmax = f->nmax;
        f->z.alloc(2 * nmax);
        VFPS_CUDA(cudaMemcpyAsync(f->z.p, imp->z.p, imp->z.bytes(),
                                  cudaMemcpyDeviceToDevice, ctx->stream));
        f->d_pos.alloc(ps->nb);
        h2d(f->d_pos.p, pos.data(), ps->nb, ctx);
        f->wtab.alloc(nmax);
        f->wake.alloc(size_t(ps->nb) * ps->n);
        f->padded.alloc(nmax);
        f->twiddle.alloc(2 * nmax);
        f->csr_coef.alloc(nmax / 2 + 1);
        f->spectrum.alloc(size_t(ps->nb) * nmax);
        f->power.alloc(ps->nb);
        VFPS_CUDA(cudaMemsetAsync(f->wake.p, 0, f->wake.bytes(), ctx->stream));
        VFPS_CUDA(cudaMemsetAsync(f->padded.p, 0, f->padded.bytes(),
                                  ctx->stream));
        VFPS_CUDA(cudaMemsetAsync(f->spectrum.p, 0, f->spectrum.bytes(),
                                  ctx->stream));
        VFPS_CUDA(cudaMemsetAsync(f->power.p, 0, f->power.bytes(),
                                  ctx->stream));
        vfps::launch_wake_table(f.get());
        // frequency ruler 0 .. 1/dq over nmax points, "Hertz" = c/qscale
        const float fmax_axis = 1 / ps->ax[0].delta;
        f->freq_delta = fmax_axis / static_cast<float>(nmax - 1);
        f->freq_scale = static_cast<float>(C_LIGHT / double(ps->ax[0].scale));
        const double f4wph = 2 * 1.0 * ps->current * ps->current / f_rev;
        f->factor4watts = f4wph * f->freq_scale;
        VFPS_CUDA(cudaStreamSynchronize(ctx->stream));
        *field = f.release();
    });
}

extern "C" int vfps_field_create_wake(vfps_ps* ps, const vfps_impedance* imp,
                                      const uint32_t* buckets,
                                      uint32_t spacing_bins, double f_rev,
                                      double revolutionpart, double ib,
                                      double e0, double sigma_delta, double dt,
                                      vfps_field** field)
{
    if (!ps) {
        return null_arg("ps");
    }
    // inc/PS/ElectricField.hpp:99-100
    const double ws = ib * dt * C_LIGHT / double(ps->ax[0].scale)
                      / (double(ps->ax[1].delta) * sigma_delta * e0);
    return vfps_field_create(ps, imp, buckets, spacing_bins, f_rev,
                             revolutionpart, static_cast<float>(ws), field);
}

extern "C" int vfps_field_pad_bunch_profiles(vfps_field* field)
{
    if (!field) {
        return null_arg("field");
    }
    return guard(field->ps->ctx, [&] { vfps::launch_pad(field); });
}

extern "C" int vfps_field_get_padded_profiles(vfps_field* field, float* padded)
{
    if (!field || !padded) {
        return null_arg("field/padded");
    }
    return guard(field->ps->ctx, [&] {
        d2h(padded, field->padded.p, field->nmax, field->ps->ctx);
    });
}

extern "C" int vfps_field_wake_potential(vfps_field* field)
{
    if (!field) {
        return null_arg("field");
    }
    return guard(field->ps->ctx, [&] { vfps::launch_wake(field); });
}

extern "C" int vfps_field_get_wake_potential(vfps_field* field, float* wake)
{
    if (!field || !wake) {
        return null_arg("field/wake");
    }
    return guard(field->ps->ctx, [&] {
        d2h(wake, field->wake.p, field->wake.n, field->ps->ctx);
    });
}

extern "C" int vfps_field_info(const vfps_field* field, float* wakescale,
                               size_t* nmax)
{
    if (!field) {
        return null_arg("field");
    }
    if (wakescale) {
        *wakescale = field->wakescale;
    }
    if (nmax) {
        *nmax = field->nmax;
    }
    return VFPS_OK;
}

extern "C" int vfps_field_update_csr(vfps_field* field, float fc)
{
    if (!field) {
        return null_arg("field");
    }
    vfps_ctx* ctx = field->ps->ctx;
    return guard(ctx, [&] {
        if (!field->csr_ready || field->csr_fc != fc) {
            // src/PS/ElectricField.cpp:167-179: renorm = dq^2
            // (1 - exp(-(f_i/fc)^2)), times Re Z[i]
            const size_t nmax = field->nmax;
            std::vector<float> zt(2 * nmax);
            d2h(zt.data(), field->z.p, 2 * nmax, ctx);
            const float dq = field->ps->ax[0].delta;
            const float scale_hz = static_cast<float>(field->freq_scale);
            std::vector<float> coef(nmax / 2 + 1);
            for (size_t i = 0; i <= nmax / 2; i++) {
                float renorm = dq * dq;
                const float fi = 0.f + static_cast<float>(i) * field->freq_delta;
                if (fc > 0) {
                    renorm *= (1 - std::exp(-std::pow(scale_hz * fi / fc, 2)));
                }
                coef[i] = renorm * zt[2 * i];
            }
            h2d(field->csr_coef.p, coef.data(), coef.size(), ctx);
            field->csr_fc = fc;
            field->csr_ready = true;
        }
        vfps::launch_csr(field);
    });
}

extern "C" int vfps_field_get_csr(vfps_field* field, float* spectrum,
                                  float* power, double* factor4watts)
{
    if (!field) {
        return null_arg("field");
    }
    return guard(field->ps->ctx, [&] {
        vfps_ctx* ctx = field->ps->ctx;
        if (spectrum) {
            d2h(spectrum, field->spectrum.p, field->spectrum.n, ctx);
        }
        if (power) {
            std::vector<double> p(field->ps->nb);
            d2h(p.data(), field->power.p, p.size(), ctx);
            for (size_t b = 0; b < p.size(); b++) {
                power[b] = static_cast<float>(p[b]);
            }
        }
        if (factor4watts) {
            *factor4watts = field->factor4watts;
        }
    });
}

extern "C" int vfps_field_destroy(vfps_field* field)
{
    if (!field) {
        return VFPS_OK;
    }
    cudaSetDevice(field->device);
    delete field;
    return VFPS_OK;
}
