// Impedance tables computed on the device in FP64, stored as complex float
// (impedance_t in the reference).  Models: FreeSpaceCSR
// (src/Z/FreeSpaceCSR.cpp:18-43), ParallelPlatesCSR
// (src/Z/ParallelPlatesCSR.cpp:25-70), ResistiveWall
// (src/Z/ResistiveWall.cpp:24-57), ConstImpedance (src/Z/ConstImpedance.cpp).
//
// ParallelPlatesCSR needs Ai, Ai', Bi, Bi' for u > 0 (Boost.Math in the
// reference).  Own implementation:
//   - Maclaurin series (Abramowitz & Stegun 10.4.2-10.4.5) for Ai, Ai' at
//     u <= 1.5 and for Bi, Bi' at u <= 12 (Bi's series has no
//     cancellation for u > 0);
//   - Ai, Ai' for u > 1.5 from DLMF 9.5.6,
//       Ai(u) = e^{-z}/pi Int_0^inf exp(-sqrt(u) t^2) cos(t^3/3) dt,
//     z = 2/3 u^{3/2}, with s = u^{1/4} t and the trapezoidal rule (step
//     1/8 on [0, 7]), which converges exponentially for this integrand;
//   - Bi, Bi' for u > 12 from the asymptotic series A&S 10.4.63/10.4.66.
// As in the reference, where Bi or Bi' overflows a double (Boost throws
// and the reference catches it) the sum over p ends.
#include "vfps_internal.cuh"

namespace vfps {
namespace {

__device__ void airy_series(double x, double* ai, double* aip, double* bi,
                            double* bip)
{
    const double c1 = 0.355028053887817239260;
    const double c2 = 0.258819403792806798405;
    const double x3 = x * x * x;
    double tf = 1.0, tg = x, f = 1.0, g = x, fp = 0.0, gp = 1.0;
    for (int k = 1; k < 2000; k++) {
        tf = tf * x3 / ((3.0 * k - 1.0) * (3.0 * k));
        tg = tg * x3 / ((3.0 * k) * (3.0 * k + 1.0));
        f += tf;
        g += tg;
        const double dfp = (x > 0) ? tf * (3.0 * k) / x : 0.0;
        const double dgp = (x > 0) ? tg * (3.0 * k + 1.0) / x : 0.0;
        fp += dfp;
        gp += dgp;
        if (tf <= 1e-18 * f && tg <= 1e-18 * g && dfp <= 1e-18 * fp
            && dgp <= 1e-18 * gp) {
            break;
        }
    }
    const double s3 = 1.7320508075688772935;
    *ai = c1 * f - c2 * g;
    *aip = c1 * fp - c2 * gp;
    *bi = s3 * (c1 * f + c2 * g);
    *bip = s3 * (c1 * fp + c2 * gp);
}

__device__ void airy_ai_integral(double x, double* ai, double* aip)
{
    const double h = 0.125;
    const double c = 3.0 * pow(x, 0.75);
    double j0 = 0, j2 = 0;
    for (int k = 0; k < 57; k++) {
        const double s = k * h;
        const double wk = (k == 0) ? 0.5 * h : h;
        const double e = exp(-s * s) * cos(s * s * s / c);
        j0 += wk * e;
        j2 += wk * s * s * e;
    }
    const double z = 2.0 / 3.0 * x * sqrt(x);
    const double pre = exp(-z) / 3.14159265358979323846;
    const double x14 = pow(x, 0.25);
    *ai = pre * j0 / x14;
    *aip = pre * (-x14 * j0 - 0.5 * j2 / (x14 * x14 * x14 * x14 * x14));
}

__device__ void airy_bi_asymptotic(double x, double* bi, double* bip)
{
    const double z = 2.0 / 3.0 * x * sqrt(x);
    double u = 1.0, su = 1.0, sv = 1.0, zk = 1.0;
    for (int k = 1; k < 40; k++) {
        u = u * ((6.0 * k - 5.0) * (6.0 * k - 3.0) * (6.0 * k - 1.0))
            / ((2.0 * k - 1.0) * 216.0 * k);
        const double v = -(6.0 * k + 1.0) / (6.0 * k - 1.0) * u;
        zk /= z;
        su += u * zk;
        sv += v * zk;
        if (fabs(u * zk) < 1e-18 && fabs(v * zk) < 1e-18) {
            break;
        }
    }
    const double ez = exp(z);
    const double x14 = pow(x, 0.25);
    const double rpi = 0.564189583547756286948;
    *bi = ez * rpi / x14 * su;
    *bip = x14 * ez * rpi * sv;
}

// returns false when Bi or Bi' overflows
__device__ bool airy(double x, double* ai, double* aip, double* bi,
                     double* bip)
{
    if (x <= 12.0) {
        airy_series(x, ai, aip, bi, bip);
    } else {
        airy_bi_asymptotic(x, bi, bip);
    }
    if (x > 1.5) {
        airy_ai_integral(x, ai, aip);
    }
    return isfinite(*bi) && isfinite(*bip);
}

const double C_LIGHT = 2.99792458e8;
const double PI = 3.14159265358979323846;

// prm: f0, f_max, g (f0 and f_max already rounded to float by the caller)
__global__ void k_z_parallel_plates(size_t nfreqs, double f0, double f_max,
                                    double g, double z0, float* out)
{
    const size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x + 1;
    if (i > nfreqs / 2) {
        return;
    }
    const double delta = f_max / f0 / (nfreqs - 1.0);
    const double r_bend = C_LIGHT / (2 * PI * f0);
    const double n = i * delta;
    const double m = n * pow(g / r_bend, 1.5);
    const uint32_t maxp = static_cast<uint32_t>(2 * m * pow(r_bend / g, 1.5)
                                                * f0 * g / C_LIGHT);
    const double b = pow(m, -4. / 3.);
    const double two23 = pow(2.0, 2. / 3.);
    double zr = 0, zi = 0;
    for (uint32_t p = 1; p <= maxp; p += 2) {
        const double u = PI * PI * p * p / two23 * b;
        double ai, aip, bi, bip;
        if (!airy(u, &ai, &aip, &bi, &bip)) {
            break;
        }
        // Ai'(Ai' - i Bi') + u Ai (Ai - i Bi)
        zr += aip * aip + u * ai * ai;
        zi += -(aip * bip + u * ai * bi);
    }
    const double fac = 4.0 * b * n * g / r_bend * PI * PI * pow(2.0, 1. / 3.)
                       * z0;
    out[2 * i] = static_cast<float>(zr * fac);
    out[2 * i + 1] = static_cast<float>(zi * fac);
}

// model 0 free space: prm f_rev, f_max; model 2 resistive wall: prm f0,
// f_max, L, s, xi, b, z0; model 3 const: prm re, im
__global__ void k_z_simple(int model, size_t n, double p0, double p1,
                           double p2, double p3, double p4, double p5,
                           double p6, float* out)
{
    const size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x;
    if (i >= n) {
        return;
    }
    double re = 0, im = 0;
    if (model == 0) {
        if (i <= n / 2) {
            const double delta = p1 / p0 / double(n - 1);
            const double a = pow(double(i) * delta, 1.0 / 3.0);
            re = double(306.3f) * a;
            im = double(176.9f) * a;
        }
    } else if (model == 2) {
        if (i <= n / 2) {
            const double mu_r = 1 + p4;
            const double z1 = static_cast<float>(
                sqrt(p6 * mu_r * p0 / p3 / PI / C_LIGHT) * p2 / 2 / p5);
            const double delta = double(static_cast<float>(p1 / p0))
                                 / (n - 1.0);
            const double a = sqrt(double(i) * delta);
            re = z1 * a;
            im = -z1 * a;
        }
    } else if (model == 3) {
        if (i < n / 2) {
            re = p0;
            im = p1;
        }
    }
    out[2 * i] = static_cast<float>(re);
    out[2 * i + 1] = static_cast<float>(im);
}

__global__ void k_z_add(float* dst, const float* src, size_t n2)
{
    const size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x;
    if (i < n2) {
        dst[i] = __fadd_rn(dst[i], src[i]);
    }
}

}  // namespace

// model: 0 free space, 1 parallel plates, 2 resistive wall, 3 const
void launch_z_model(vfps_ctx* ctx, int model, size_t n, const double* prm,
                    float* out)
{
    VFPS_CUDA(cudaMemsetAsync(out, 0, 2 * n * sizeof(float), ctx->stream));
    if (model == 1) {
        const size_t half = n / 2;
        if (half > 0) {
            k_z_parallel_plates<<<(half + 63) / 64, 64, 0, ctx->stream>>>(
                n, prm[0], prm[1], prm[2], prm[3], out);
        }
    } else {
        k_z_simple<<<(n + 255) / 256, 256, 0, ctx->stream>>>(
            model, n, prm[0], prm[1], prm[2], prm[3], prm[4], prm[5], prm[6],
            out);
    }
    VFPS_LAUNCHED();
}

void launch_z_add(vfps_ctx* ctx, float* dst, const float* src, size_t n)
{
    k_z_add<<<(2 * n + 255) / 256, 256, 0, ctx->stream>>>(dst, src, 2 * n);
    VFPS_LAUNCHED();
}

}  // namespace vfps
