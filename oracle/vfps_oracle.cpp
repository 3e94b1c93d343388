/*
 * vfps_oracle.cpp -- TEST INFRASTRUCTURE ONLY.
 *
 * This file is the checker, never the product: only tests/, the smoke test
 * and the CPU-baseline leg of bench.py load it.  It is a CPU restatement of
 * the Inovesa phase-space hot path (reference paths are relative to the
 * Inovesa source tree), templated on the arithmetic type:
 *
 *   T = float   mirrors the reference CPU build, in which every data type
 *               aliases float (inc/defines.hpp:31-43).  It is the timed CPU
 *               baseline ("port") and follows the reference's order of
 *               operations, including where the reference itself promotes
 *               to double.
 *   T = double  is the FP64 oracle the CUDA path is judged against.
 *
 * Build with -ffp-contract=off so that float results do not depend on
 * whether the compiler fuses multiply-adds (it does by default on aarch64).
 *
 * Parity of this restatement is pinned by the golden vectors of the
 * reference's own unit tests (test/TestRotationMap.cpp, test/TestKickMap.cpp,
 * test/TestPhaseSpace.cpp, test/TestElectricField.cpp, test/TestRuler.cpp,
 * test/TestImpedance.cpp, test/TestConstImpedance.cpp), extracted into
 * tests/golden/ by tests/golden/make_golden.py.  Parts with no reference
 * test (FokkerPlanck stencils, Drift/RF offsets, ParallelPlatesCSR,
 * ResistiveWall, CSR spectrum) follow the cited code line by line; the Airy
 * functions are checked against scipy.special.airy.
 *
 * The reference cannot be compiled here (Boost and FFTW3 are absent), so no
 * reference binary backs this file.
 */
#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdint>
#include <cstring>
#include <limits>
#include <numeric>
#include <thread>
#include <vector>

namespace vo {

typedef uint32_t u32;

/* ------------------------------------------------------------------ Ruler
 * inc/PS/Ruler.hpp:31-51: delta = (max-min)/(steps-1),
 * zerobin = ((min+max)/(min-max)+1)*(steps-1)/2, at(i) = min + i*delta. */
template <typename T>
struct Axis {
    u32 n = 0;
    T min = 0, max = 0, delta = 0, zerobin = 0, scale = 1;
    std::vector<T> v;
};

template <typename T>
Axis<T> make_axis(u32 n, T mn, T mx, T scale)
{
    Axis<T> a;
    a.n = n;
    a.min = mn;
    a.max = mx;
    a.scale = scale;
    a.delta = (mx - mn) / static_cast<T>(n - 1);
    a.zerobin = ((mn + mx) / (mn - mx) + 1) * static_cast<T>(n - 1) / 2;
    a.v.resize(n);
    for (u32 i = 0; i < n; i++) {
        a.v[i] = mn + (static_cast<T>(i) * a.delta);
    }
    return a;
}

/* float -> uint32 cast of an already truncated value, as done by
 * static_cast<meshindex_t>() on x86-64: negative values (<= -1) wrap to huge
 * numbers and therefore fail every "< size" test; -0 maps to 0. */
template <typename T>
inline bool base_index(T truncated, u32 size, u32* out)
{
    if (!(truncated >= 0) || !(truncated < static_cast<T>(size))) {
        return false;
    }
    *out = static_cast<u32>(truncated);
    return true;
}

/* ------------------------------------------------- interpolation weights
 * src/SM/SourceMap.cpp:142-170 (calcCoefficiants). */
template <typename T>
void coefficients(T* ic, T f, int it)
{
    switch (it) {
    case 1:
        ic[0] = 1;
        break;
    case 2:
        ic[0] = T(1) - f;
        ic[1] = f;
        break;
    case 3:
        ic[0] = f * (f - T(1)) / T(2);
        ic[1] = T(1) - f * f;
        ic[2] = f * (f + T(1)) / T(2);
        break;
    case 4:
        ic[0] = (f - T(1)) * (f - T(2)) * f * T(-1. / 6.);
        ic[1] = (f + T(1)) * (f - T(1)) * (f - T(2)) / T(2);
        ic[2] = (T(2) - f) * f * (f + T(1)) / T(2);
        ic[3] = f * (f + T(1)) * (f - T(1)) * T(1. / 6.);
        break;
    }
}

/* ------------------------------------------------------------ PhaseSpace */

/* src/PS/PhaseSpace.cpp:486-501: h/3*[1,4,2,4,...,(2|4),1]; for even n the
 * last interior weight is followed directly by 1 (not a Simpson rule). */
template <typename T>
void simpson_weights(u32 n, T delta, T* ws)
{
    const T ca = 3;
    T dc = 1;
    const T h03 = delta / T(3);
    ws[0] = h03;
    for (u32 x = 1; x + 1 < n; x++) {
        ws[x] = h03 * (ca + dc);
        dc = -dc;
    }
    ws[n - 1] = h03;
}

/* src/PS/PhaseSpace.cpp:471-484: 1/sqrt(2 pi) * exp(-x^2/(2 zoom^2)), with
 * the exponent evaluated in double as in the reference. */
template <typename T>
void gaussian(const Axis<T>& a, double zoom, T* out)
{
    const double zoom2 = zoom * zoom;
    const T c = static_cast<T>(0.398942280401432677939946059934381868L);
    for (u32 i = 0; i < a.n; i++) {
        out[i] = static_cast<T>(
            static_cast<double>(c)
            * std::exp((-0.5) * static_cast<double>(a.v[i])
                       * static_cast<double>(a.v[i]) / zoom2));
    }
}

/* src/PS/PhaseSpace.cpp:291-323 (updateXProjection, CPU branch). */
template <typename T>
void project_x(u32 nb, u32 n, const T* data, const T* ws, T* proj)
{
    for (u32 b = 0; b < nb; b++) {
        for (u32 x = 0; x < n; x++) {
            const T* row = data + (size_t(b) * n + x) * n;
            T acc = 0;
            for (u32 y = 0; y < n; y++) {
                acc = acc + row[y] * ws[y];
            }
            proj[size_t(b) * n + x] = acc;
        }
    }
}

/* src/PS/PhaseSpace.cpp:325-340 (updateYProjection): uses the x weights. */
template <typename T>
void project_y(u32 nb, u32 n, const T* data, const T* ws, T* proj)
{
    for (u32 b = 0; b < nb; b++) {
        for (u32 y = 0; y < n; y++) {
            T acc = 0;
            for (u32 x = 0; x < n; x++) {
                acc += data[(size_t(b) * n + x) * n + y] * ws[x];
            }
            proj[size_t(b) * n + y] = acc;
        }
    }
}

/* src/PS/PhaseSpace.cpp:200-239 (integrate, CPU branch). Returns the sum. */
template <typename T>
T integrate(u32 nb, u32 n, const T* proj, const T* ws, T* filling)
{
    for (u32 b = 0; b < nb; b++) {
        T acc = 0;
        for (u32 x = 0; x < n; x++) {
            acc = acc + proj[size_t(b) * n + x] * ws[x];
        }
        filling[b] = acc;
    }
    T total = 0;
    for (u32 b = 0; b < nb; b++) {
        total = total + filling[b];
    }
    return total;
}

/* src/PS/PhaseSpace.cpp:342-372 (normalize). */
template <typename T>
void normalize(u32 nb, u32 n, T* data, const T* filling_set, const T* filling)
{
    const size_t nxy = size_t(n) * n;
    for (u32 b = 0; b < nb; b++) {
        T* d = data + b * nxy;
        if (filling_set[b] > 0) {
            for (size_t i = 0; i < nxy; i++) {
                d[i] *= filling_set[b] / filling[b];
            }
        } else {
            for (size_t i = 0; i < nxy; i++) {
                d[i] = 0;
            }
        }
    }
}

/* src/PS/PhaseSpace.cpp:241-289 (average + variance) for one axis; the
 * squared deviation goes through std::pow(float,int), i.e. double. */
template <typename T>
void moments(u32 nb, u32 n, const T* axis_values, T delta, const T* proj,
             const T* filling_set, const T* filling, T* avg_out, T* var_out)
{
    for (u32 b = 0; b < nb; b++) {
        T avg = 0;
        if (filling_set[b] > 0) {
            for (u32 i = 0; i < n; i++) {
                avg += proj[size_t(b) * n + i] * axis_values[i];
            }
            avg *= delta / filling[b];
        }
        T var = 0;
        if (filling_set[b] > 0) {
            for (u32 i = 0; i < n; i++) {
                var += proj[size_t(b) * n + i]
                       * std::pow(static_cast<double>(axis_values[i] - avg), 2);
            }
            var *= delta / filling[b];
        }
        avg_out[b] = avg;
        var_out[b] = var;
    }
}

/* ------------------------------------------------------------ RotationMap
 * src/SM/RotationMap.cpp:190-260 (genHInfo) and :97-176 (apply, CPU
 * branch, with the clamp of :159-172).  Source coordinates are truncated
 * with std::modf; a base index outside the mesh yields an all-zero stencil;
 * single taps outside the mesh get index 0 and weight 0.  Each bunch is
 * rotated on its own (the reference handles bunch 0 only). */
template <typename T>
struct RotationTap {
    u32 index;
    T weight;
};

template <typename T>
void rotation_stencil(const Axis<T>& ax, const Axis<T>& ay, T cs, T sn,
                      int it, u32 x0, u32 y0, RotationTap<T>* taps)
{
    const int ip = it * it;
    T x1r = (cs * ax.v[x0] - sn * ay.v[y0]) / ax.delta + ax.zerobin;
    T y1r = (sn * ax.v[x0] + cs * ay.v[y0]) / ay.delta + ay.zerobin;
    T xi, yi;
    const T xf = std::modf(x1r, &xi);
    const T yf = std::modf(y1r, &yi);
    u32 x1, y1;
    if (base_index(xi, ax.n, &x1) && base_index(yi, ay.n, &y1)) {
        T icq[4], icp[4];
        coefficients(icq, xf, it);
        coefficients(icp, yf, it);
        for (int j1 = 0; j1 < it; j1++) {
            const long long j0 = (long long)y1 + j1 - (it - 1) / 2;
            for (int i1 = 0; i1 < it; i1++) {
                const long long i0 = (long long)x1 + i1 - (it - 1) / 2;
                RotationTap<T>& h = taps[i1 * it + j1];
                if (i0 >= 0 && i0 < ax.n && j0 >= 0 && j0 < ay.n) {
                    h.index = static_cast<u32>(i0 * ay.n + j0);
                    h.weight = icq[i1] * icp[j1];
                } else {
                    h.index = 0;
                    h.weight = 0;
                }
            }
        }
    } else {
        for (int i = 0; i < ip; i++) {
            taps[i].index = 0;
            taps[i].weight = 0;
        }
    }
}

template <typename T>
void rotation_apply(const Axis<T>& ax, const Axis<T>& ay, T angle, int it,
                    bool clamp, u32 nb, const T* in, T* out)
{
    const T cs = std::cos(-angle);
    const T sn = std::sin(-angle);
    const int ip = it * it;
    const size_t nxy = size_t(ax.n) * ay.n;
    std::vector<RotationTap<T>> taps(ip);
    for (u32 b = 0; b < nb; b++) {
        const T* src = in + b * nxy;
        T* dst = out + b * nxy;
        for (u32 x0 = 0; x0 < ax.n; x0++) {
            for (u32 y0 = 0; y0 < ay.n; y0++) {
                rotation_stencil(ax, ay, cs, sn, it, x0, y0, taps.data());
                T value = 0;
                for (int j = 0; j < ip; j++) {
                    value += src[taps[j].index] * taps[j].weight;
                }
                if (clamp) {
                    T ceil = std::numeric_limits<T>::min();
                    T flor = std::numeric_limits<T>::max();
                    for (int x = 1; x <= 2; x++) {
                        for (int y = 1; y <= 2; y++) {
                            ceil = std::max(ceil, src[taps[x * it + y].index]);
                            flor = std::min(flor, src[taps[x * it + y].index]);
                        }
                    }
                    value = std::max(std::min(ceil, value), flor);
                }
                dst[size_t(x0) * ay.n + y0] = value;
            }
        }
    }
}

/* --------------------------------------------------------------- KickMap
 * src/SM/KickMap.cpp:339-389 (updateSM): offset in mesh units -> per-row
 * stencil.  poffs = n/2 + offset, truncated with modf; taps outside [0,n)
 * become (n/2, 0); an out-of-range base gives an all-(n/2, 0) stencil. */
template <typename T>
void kick_stencils(u32 kd, int it, const T* offset, size_t count, u32* idx,
                   T* w)
{
    T smc[4];
    for (size_t i = 0; i < count; i++) {
        const T poffs = static_cast<T>(kd / 2) + offset[i];
        T qp_int;
        const T xip = std::modf(poffs, &qp_int);
        u32 jd;
        if (base_index(qp_int, kd, &jd)) {
            coefficients(smc, xip, it);
            for (int j1 = 0; j1 < it; j1++) {
                const long long j0 = (long long)jd + j1 - (it - 1) / 2;
                if (j0 >= 0 && j0 < kd) {
                    idx[i * it + j1] = static_cast<u32>(j0);
                    w[i * it + j1] = smc[j1];
                } else {
                    idx[i * it + j1] = kd / 2;
                    w[i * it + j1] = 0;
                }
            }
        } else {
            for (int j1 = 0; j1 < it; j1++) {
                idx[i * it + j1] = kd / 2;
                w[i * it + j1] = 0;
            }
        }
    }
}

/* src/SM/KickMap.cpp:194-271 (apply, CPU branch), square mesh.
 * y-kick: out[x][y] = sum_j in[x][y + idx_j - n/2] w_j, stencil of row x
 *         (of bunch b: row b*n + x; the reference indexes bunches > 0
 *         without the tap stride, :246,252 -- not reproduced);
 * x-kick: out[x][y] = sum_j in[x + idx_j - n/2][y] w_j, stencil of column y
 *         (shared by all bunches, as in the reference).
 * Taps that leave the mesh are dropped, not renormalised. */
template <typename T>
void kick_apply(int axis, u32 nb, u32 n, int it, const u32* idx, const T* w,
                const T* in, T* out)
{
    const size_t nxy = size_t(n) * n;
    const int32_t half = static_cast<int32_t>(n / 2);
    for (u32 b = 0; b < nb; b++) {
        const T* src = in + b * nxy;
        T* dst = out + b * nxy;
        if (axis == 0) {
            for (u32 x = 0; x < n; x++) {
                for (u32 y = 0; y < n; y++) {
                    T value = 0;
                    for (int j = 0; j < it; j++) {
                        const u32 xs = static_cast<u32>(
                            static_cast<int32_t>(x + idx[y * it + j]) - half);
                        if (xs < n) {
                            value += src[size_t(xs) * n + y] * w[y * it + j];
                        }
                    }
                    dst[size_t(x) * n + y] = value;
                }
            }
        } else {
            for (u32 x = 0; x < n; x++) {
                const size_t row = (size_t(b) * n + x) * it;
                for (u32 y = 0; y < n; y++) {
                    T value = 0;
                    for (int j = 0; j < it; j++) {
                        const u32 ys = static_cast<u32>(
                            static_cast<int32_t>(y + idx[row + j]) - half);
                        if (ys < n) {
                            value += src[size_t(x) * n + ys] * w[row + j];
                        }
                    }
                    dst[size_t(x) * n + y] = value;
                }
            }
        }
    }
}

/* src/SM/DriftMap.cpp:21-30: offset[y] = sum_i slip_i p (p dE/E0)^i / dq. */
template <typename T>
void drift_offsets(const Axis<T>& ax, const Axis<T>& ay, const T* slip,
                   int nslip, T e0, T* off)
{
    for (u32 y = 0; y < ay.n; y++) {
        off[y] = 0;
        for (int i = 0; i < nslip; i++) {
            off[y] += slip[i] * ay.v[y]
                      * std::pow(ay.v[y] * ay.scale / e0, static_cast<T>(i));
        }
        off[y] /= ax.delta;
    }
}

/* src/SM/RFKickMap.cpp:59-83 (_calcKick) with the static phase and unit
 * amplitude of the static maps; linear and sinusoidal forms. */
template <typename T>
void rf_offsets_linear(const Axis<T>& ax, T angle, T phaseoffs, T bl2phase,
                       T ampl, T* off)
{
    const T xcenter = ax.zerobin;
    for (u32 x = 0; x < ax.n; x++) {
        off[x] = std::tan(angle) * (xcenter - static_cast<T>(x));
        off[x] += std::tan(angle) * phaseoffs / bl2phase / ax.delta;
        off[x] *= ampl;
    }
}

template <typename T>
void rf_offsets_sin(const Axis<T>& ax, const Axis<T>& ay, T revpart, T v_rf,
                    T v0, T bl2phase, T phase, T ampl, T* off)
{
    for (u32 x = 0; x < ax.n; x++) {
        off[x] = revpart * (-ampl * v_rf * std::sin(ax.v[x] * bl2phase + phase)
                            + v0)
                 / ay.delta / ay.scale;
    }
}

/* ------------------------------------------------------- FokkerPlanckMap
 * src/SM/FokkerPlanckMap.cpp:11-118: one stencil per energy cell y, shared
 * by every x.  derivation 4 (cubic): taps (y-2..y+1) below trunc(zerobin),
 * (y-1..y+2) from there on; rows 0,1,n-2,n-1 are all zero.  derivation 3
 * (two-sided): taps (y-1..y+1); rows 0 and n-1 are zero.  fptype: 0 none,
 * 1 damping only, 2 diffusion only, 3 full. */
template <typename T>
int fp_stencils(const Axis<T>& ay, T e1, int fptype, int derivation,
                u32* idx, T* w)
{
    const u32 n = ay.n;
    const int ip = derivation;
    const T e1_2d = e1 / (T(2) * ay.delta);
    const T e1_6d = e1 / (T(6) * ay.delta);
    const T e1_d2 = e1 / (ay.delta * ay.delta);
    const T ycenter = ay.zerobin;
    const bool damp = fptype != 0 && fptype != 2;
    const bool diff = fptype != 0 && fptype != 1;
    for (u32 k = 0; k < n * (u32)ip; k++) {
        idx[k] = 0;
        w[k] = 0;
    }
    if (derivation == 3) {
        for (u32 j = 1; j + 1 < n; j++) {
            u32* I = idx + j * 3;
            T* W = w + j * 3;
            I[0] = j - 1; W[0] = 0;
            I[1] = j;     W[1] = 1;
            I[2] = j + 1; W[2] = 0;
            if (damp) {
                const T pos = ay.v[j];
                W[0] += -e1_2d * pos;
                W[1] += e1;
                W[2] += e1_2d * pos;
            }
            if (diff) {
                W[0] += e1_d2;
                W[1] += T(-2) * e1_d2;
                W[2] += e1_d2;
            }
        }
        return 0;
    }
    if (derivation != 4) {
        return -1;
    }
    for (u32 j = 2; static_cast<T>(j) < ycenter; j++) {
        const T pos = ay.v[j];
        u32* I = idx + j * 4;
        T* W = w + j * 4;
        I[0] = j - 2; W[0] = 0;
        I[1] = j - 1; W[1] = 0;
        I[2] = j;     W[2] = 1;
        I[3] = j + 1; W[3] = 0;
        if (damp) {
            W[0] += e1_6d * T(1) * pos;
            W[1] += e1_6d * T(-6) * pos;
            W[2] += e1 + e1_6d * T(3) * pos;
            W[3] += e1_6d * T(2) * pos;
        }
        if (diff) {
            W[1] += e1_d2;
            W[2] += T(-2) * e1_d2;
            W[3] += e1_d2;
        }
    }
    for (u32 j = static_cast<u32>(ycenter); j + 2 < n; j++) {
        const T pos = ay.v[j];
        u32* I = idx + j * 4;
        T* W = w + j * 4;
        I[0] = j - 1; W[0] = 0;
        I[1] = j;     W[1] = 1;
        I[2] = j + 1; W[2] = 0;
        I[3] = j + 2; W[3] = 0;
        if (damp) {
            W[0] += e1_6d * T(-2) * pos;
            W[1] += e1 + e1_6d * T(-3) * pos;
            W[2] += e1_6d * T(6) * pos;
            W[3] += e1_6d * T(-1) * pos;
        }
        if (diff) {
            W[0] += e1_d2;
            W[1] += T(-2) * e1_d2;
            W[2] += e1_d2;
        }
    }
    for (u32 j : {0u, 1u, n - 2, n - 1}) {
        for (int k = 0; k < 4; k++) {
            idx[j * 4 + k] = 0;
            w[j * 4 + k] = 0;
        }
    }
    return 0;
}

/* src/SM/FokkerPlanckMap.cpp:170-213 (apply, CPU branch). */
template <typename T>
void fp_apply(u32 nb, u32 n, int ip, const u32* idx, const T* w, const T* in,
              T* out)
{
    for (u32 b = 0; b < nb; b++) {
        for (u32 x = 0; x < n; x++) {
            const size_t offs = (size_t(b) * n + x) * n;
            for (u32 y = 0; y < n; y++) {
                T value = 0;
                for (int j = 0; j < ip; j++) {
                    value += in[offs + idx[y * ip + j]] * w[y * ip + j];
                }
                out[offs + y] = value;
            }
        }
    }
}

/* ------------------------------------------------------ Airy functions
 * Needed by ParallelPlatesCSR (src/Z/ParallelPlatesCSR.cpp:44-60), which
 * calls Boost.Math's airy_ai/bi(_prime) for u > 0.  Own implementation:
 *  - Ai, Ai' for x <= 1.5 and Bi, Bi' for x <= 12: Maclaurin series
 *    (Abramowitz & Stegun 10.4.2-10.4.5); Bi's series has no cancellation.
 *  - Ai, Ai' for x > 1.5: Ai(x) = e^-z/pi * Int_0^inf exp(-sqrt(x) t^2)
 *    cos(t^3/3) dt (DLMF 9.5.6), z = 2/3 x^1.5, substituted s = x^(1/4) t
 *    and summed with the trapezoidal rule (exponentially convergent for this
 *    analytic, Gaussian-damped integrand); Ai' by differentiating under the
 *    integral.
 *  - Bi, Bi' for x > 12: asymptotic expansions A&S 10.4.63 / 10.4.66.
 * Boost throws an overflow error when Bi or Bi' exceeds DBL_MAX, which the
 * reference catches to end the sum over p; *overflow reports that case. */
inline void airy_series(double x, double* ai, double* aip, double* bi,
                        double* bip)
{
    const double c1 = 0.355028053887817239260;
    const double c2 = 0.258819403792806798405;
    const double x3 = x * x * x;
    double tf = 1.0, tg = x;          /* f and g terms (A&S 10.4.3) */
    double f = 1.0, g = x;
    double fp = 0.0, gp = 1.0;        /* derivatives, term by term */
    for (int k = 1; k < 2000; k++) {
        tf = tf * x3 / ((3.0 * k - 1.0) * (3.0 * k));
        tg = tg * x3 / ((3.0 * k) * (3.0 * k + 1.0));
        f += tf;
        g += tg;
        const double dfp = (x > 0) ? tf * (3.0 * k) / x : 0.0;
        const double dgp = tg * (3.0 * k + 1.0) / (x > 0 ? x : 1.0);
        fp += dfp;
        gp += (x > 0) ? dgp : 0.0;
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

inline void airy_ai_integral(double x, double* ai, double* aip)
{
    const double h = 0.125;
    const int ns = 57; /* s in [0, 7]: exp(-49) is far below double eps */
    const double c = 3.0 * std::pow(x, 0.75);
    double j0 = 0, j2 = 0;
    for (int k = 0; k < ns; k++) {
        const double s = k * h;
        const double wk = (k == 0) ? 0.5 * h : h;
        const double e = std::exp(-s * s) * std::cos(s * s * s / c);
        j0 += wk * e;
        j2 += wk * s * s * e;
    }
    const double z = 2.0 / 3.0 * x * std::sqrt(x);
    const double pre = std::exp(-z) / 3.14159265358979323846;
    const double x14 = std::pow(x, 0.25);
    *ai = pre * j0 / x14;
    *aip = pre * (-x14 * j0 - 0.5 * j2 / (x14 * x14 * x14 * x14 * x14));
}

inline void airy_bi_asymptotic(double x, double* bi, double* bip)
{
    const double z = 2.0 / 3.0 * x * std::sqrt(x);
    double u = 1.0, su = 1.0, sv = 1.0, zk = 1.0;
    for (int k = 1; k < 40; k++) {
        u = u * ((6.0 * k - 5.0) * (6.0 * k - 3.0) * (6.0 * k - 1.0))
            / ((2.0 * k - 1.0) * 216.0 * k);
        const double v = -(6.0 * k + 1.0) / (6.0 * k - 1.0) * u;
        zk /= z;
        su += u * zk;
        sv += v * zk;
        if (std::fabs(u * zk) < 1e-18 && std::fabs(v * zk) < 1e-18) {
            break;
        }
    }
    const double ez = std::exp(z);
    const double x14 = std::pow(x, 0.25);
    const double rpi = 0.564189583547756286948; /* 1/sqrt(pi) */
    *bi = ez * rpi / x14 * su;
    *bip = x14 * ez * rpi * sv;
}

inline void airy(double x, double* ai, double* aip, double* bi, double* bip,
                 int* overflow)
{
    double sai, saip, sbi, sbip;
    if (x <= 12.0) {
        airy_series(x, &sai, &saip, &sbi, &sbip);
    } else {
        airy_bi_asymptotic(x, &sbi, &sbip);
        sai = saip = 0;
    }
    if (x > 1.5) {
        airy_ai_integral(x, &sai, &saip);
    }
    *ai = sai;
    *aip = saip;
    *bi = sbi;
    *bip = sbip;
    *overflow = !(std::isfinite(sbi) && std::isfinite(sbip));
}

/* ------------------------------------------------------------ Impedance
 * All constructors return tables of complex<float> (impedance_t), as the
 * reference stores them. */
typedef std::complex<float> zf;
const double C_LIGHT = 2.99792458e8;                 /* inc/defines.hpp:48 */
const double EPS0 = 8.854187817e-12;                 /* inc/defines.hpp:51 */
const double Z0_PHYS = 1 / (EPS0 * C_LIGHT);         /* inc/defines.hpp:54 */
const double Z0_IMP = 376.730313461;                 /* inc/Z/Impedance.hpp:94 */
const double PI = 3.14159265358979323846;

/* src/Z/FreeSpaceCSR.cpp:18-43 (float arithmetic as in the reference). */
inline void z_free_space(size_t n, float f_rev, float f_max, zf* out)
{
    const zf z0(306.3f, 176.9f);
    const float delta = f_max / f_rev / static_cast<float>(n - 1);
    for (size_t i = 0; i < n; i++) {
        out[i] = (i <= n / 2)
                     ? z0 * std::pow(static_cast<float>(i) * delta,
                                     static_cast<float>(1.0 / 3.0))
                     : zf(0, 0);
    }
}

/* src/Z/ParallelPlatesCSR.cpp:25-70 (double arithmetic, cast at the end).
 * f0 and f_max arrive as float parameters (frequency_t) in the reference. */
inline void z_parallel_plates(size_t nfreqs, float f0, float f_max, double g,
                              zf* out)
{
    for (size_t i = 0; i < nfreqs; i++) {
        out[i] = zf(0, 0);
    }
    const double delta = double(f_max) / double(f0) / (nfreqs - 1.0);
    const double r_bend = C_LIGHT / (2 * PI * double(f0));
    for (size_t i = 1; i <= nfreqs / 2; i++) {
        std::complex<double> Z = 0;
        const double n = i * delta;
        const double m = n * std::pow(g / r_bend, 3. / 2.);
        const uint32_t maxp = static_cast<uint32_t>(
            2 * m * std::pow(r_bend / g, 3. / 2.) * double(f0) * g / C_LIGHT);
        const double b = std::pow(m, -4. / 3.);
        for (uint32_t p = 1; p <= maxp; p += 2) {
            const double u = PI * PI * p * p / std::pow(2, 2. / 3.) * b;
            double ai, aip, bi, bip;
            int ovf;
            airy(u, &ai, &aip, &bi, &bip, &ovf);
            if (ovf) {
                break;
            }
            const std::complex<double> j(0, 1);
            Z += aip * (aip - j * bip) + u * ai * (ai - j * bi);
        }
        Z *= 4.0 * b * n * g / r_bend * PI * PI * std::pow(2, 1. / 3.)
             * Z0_PHYS;
        out[i] = zf(static_cast<float>(Z.real()), static_cast<float>(Z.imag()));
    }
}

/* src/Z/ResistiveWall.cpp:24-57. */
inline void z_resistive_wall(size_t n, float f0, float f_max, double L,
                             double s, double xi, double b, zf* out)
{
    const double mu_r = 1 + xi;
    const zf z1 = static_cast<float>(
                      std::sqrt(Z0_IMP * mu_r * double(f0) / s / PI / C_LIGHT)
                      * L / 2 / b)
                  * zf(1, -1);
    const float delta = static_cast<float>(double(f_max / f0) / (n - 1.0));
    for (size_t i = 0; i < n; i++) {
        out[i] = (i <= n / 2)
                     ? z1 * std::sqrt(static_cast<float>(i) * delta)
                     : zf(0, 0);
    }
}

/* src/Z/ConstImpedance.cpp:18-28: first n/2 entries Z, rest 0. */
inline void z_const(size_t n, zf z, zf* out)
{
    for (size_t i = 0; i < n; i++) {
        out[i] = (i < n / 2) ? z : zf(0, 0);
    }
}

/* src/Z/CollimatorImpedance.cpp:12-25. */
inline void z_collimator(size_t n, double outer, double inner, zf* out)
{
    z_const(n, zf(static_cast<float>(Z0_IMP / PI * std::log(outer / inner)),
                  0.0f),
            out);
}

/* ------------------------------------------------------------------ FFT
 * Own transforms (FFTW is absent): iterative radix-2 for powers of two,
 * direct DFT otherwise.  Unnormalised, sign -1 forward, +1 backward. */
template <typename T>
void dft(std::vector<std::complex<T>>& a, int sign)
{
    const size_t n = a.size();
    if (n == 0) {
        return;
    }
    if ((n & (n - 1)) != 0) {
        std::vector<std::complex<T>> r(n);
        for (size_t k = 0; k < n; k++) {
            std::complex<double> acc = 0;
            for (size_t j = 0; j < n; j++) {
                const double ph = sign * 2 * PI * double((k * j) % n) / n;
                acc += std::complex<double>(a[j]) *
                       std::complex<double>(std::cos(ph), std::sin(ph));
            }
            r[k] = std::complex<T>(acc);
        }
        a.swap(r);
        return;
    }
    for (size_t i = 1, j = 0; i < n; i++) {
        size_t bit = n >> 1;
        for (; j & bit; bit >>= 1) {
            j ^= bit;
        }
        j ^= bit;
        if (i < j) {
            std::swap(a[i], a[j]);
        }
    }
    for (size_t len = 2; len <= n; len <<= 1) {
        const double ang = sign * 2 * PI / double(len);
        for (size_t i = 0; i < n; i += len) {
            for (size_t k = 0; k < len / 2; k++) {
                const std::complex<T> wk(static_cast<T>(std::cos(ang * k)),
                                         static_cast<T>(std::sin(ang * k)));
                const std::complex<T> u = a[i + k];
                const std::complex<T> v = a[i + k + len / 2] * wk;
                a[i + k] = u + v;
                a[i + k + len / 2] = u - v;
            }
        }
    }
}

/* Real -> half spectrum (bins 0..n/2), like an FFTW r2c plan; bins above
 * n/2 are zero (the reference's form factor buffer is zero-initialised and
 * r2c never writes them). */
template <typename T>
void rfft(const T* x, size_t n, std::complex<T>* out)
{
    std::vector<std::complex<T>> a(n);
    for (size_t i = 0; i < n; i++) {
        a[i] = x[i];
    }
    dft(a, -1);
    for (size_t i = 0; i < n; i++) {
        out[i] = (i <= n / 2) ? a[i] : std::complex<T>(0, 0);
    }
}

/* Half spectrum -> real, unnormalised, like an FFTW c2r plan: uses bins
 * 0..n/2 with the imaginary parts of DC and Nyquist ignored. */
template <typename T>
void irfft(const std::complex<T>* h, size_t n, T* out)
{
    std::vector<std::complex<T>> a(n);
    for (size_t k = 0; k <= n / 2; k++) {
        a[k] = h[k];
    }
    a[0] = std::complex<T>(h[0].real(), 0);
    if (n % 2 == 0) {
        a[n / 2] = std::complex<T>(h[n / 2].real(), 0);
    }
    for (size_t k = 1; k < (n + 1) / 2; k++) {
        a[n - k] = std::conj(a[k]);
    }
    dft(a, +1);
    for (size_t i = 0; i < n; i++) {
        out[i] = a[i].real();
    }
}

/* -------------------------------------------------------- ElectricField
 * src/PS/ElectricField.cpp:255-263 (padBunchProfiles) and :186-253
 * (wakePotential, CPU branch): r2c of the padded profiles, Z*FF for the
 * bins below nmax/2 (the Nyquist bin stays 0), c2r, times wakescale, which
 * is the ElectricField's wakescaling/nmax (:56-58). */
template <typename T>
void wake_potential(u32 nb, u32 n, size_t nmax, const T* proj,
                    const u32* bucket, size_t spacing, const zf* Z,
                    T wakescale, T* wake, T* padded_out)
{
    std::vector<T> bp(nmax, T(0));
    for (u32 b = 0; b < nb; b++) {
        for (u32 x = 0; x < n; x++) {
            bp[bucket[b] * spacing + x] = proj[size_t(b) * n + x];
        }
    }
    std::vector<std::complex<T>> ff(nmax);
    rfft(bp.data(), nmax, ff.data());
    std::vector<std::complex<T>> loss(nmax / 2 + 1, std::complex<T>(0, 0));
    for (size_t i = 0; i < nmax / 2; i++) {
        loss[i] = std::complex<T>(T(Z[i].real()), T(Z[i].imag())) * ff[i];
    }
    std::vector<T> wpad(nmax);
    irfft(loss.data(), nmax, wpad.data());
    if (padded_out) {
        std::copy(wpad.begin(), wpad.end(), padded_out);
    }
    for (u32 b = 0; b < nb; b++) {
        for (u32 x = 0; x < n; x++) {
            wake[size_t(b) * n + x] = wakescale * wpad[bucket[b] * spacing + x];
        }
    }
}

/* src/PS/ElectricField.cpp:133-184 (updateCSR, CPU branch) for one bunch:
 * spectrum[i] = dq^2 (1-exp(-(f_i/fc)^2)) Re Z[i] |FF[i]|^2, power = sum of
 * spectrum * df.  freq_scale is the "Hertz" scale c/bl of the frequency
 * ruler (0 .. 1/dq over nmax points). */
template <typename T>
T csr(u32 n, size_t nmax, const T* proj, const zf* Z, T dq, T fc,
      T freq_scale, T* spectrum)
{
    std::vector<T> bp(nmax, T(0));
    for (u32 x = 0; x < n; x++) {
        bp[x] = proj[x];
    }
    std::vector<std::complex<T>> ff(nmax);
    rfft(bp.data(), nmax, ff.data());
    const Axis<T> faxis = make_axis<T>(static_cast<u32>(nmax), T(0),
                                       T(1) / dq, freq_scale);
    const T renorm0 = dq * dq;
    T intensity = 0;
    for (size_t i = 0; i < nmax; i++) {
        T renorm(renorm0);
        if (fc > 0) {
            renorm *= (1 - std::exp(-std::pow(
                               static_cast<double>(freq_scale * faxis.v[i]
                                                   / fc), 2)));
        }
        const T s = renorm * T(Z[i].real()) * std::norm(ff[i]);
        if (spectrum) {
            spectrum[i] = s;
        }
        intensity += faxis.delta * s;
    }
    return intensity;
}

/* ------------------------------------------------------------- solver loop
 * Independent single-bunch simulations stepped like the reference solver
 * loop.  chain 0 is src/main.cpp:948-1053: wake update, integrate (or
 * integrate+normalize), wake y-kick t1->t2, RF y-kick t2->t1, drift x-kick
 * t1->t3, Fokker-Planck t3->t1, x projection.  chain 1 is the rotation
 * scheme the reference tests use: wake update, integrate, rotation t1->t2,
 * wake y-kick t2->t3, Fokker-Planck t3->t1, x projection.  A missing wake or
 * FP term is an Identity map (inc/SM/Identity.hpp:29-54). */
}  // namespace vo

extern "C" {
typedef struct {
    int n;              /* mesh side */
    int chain;          /* 0 kick-drift (main.cpp loop), 1 rotation */
    int it;             /* interpolation points: 2, 3, 4 */
    int clamp;          /* rotation clamp (cubic only) */
    double qmin, qmax, qscale, pmin, pmax, pscale;
    double zoom;        /* start distribution zoom */
    double angle;       /* rotation angle per step (chain 1) */
    int rf_linear;      /* chain 0: 1 linear RF, 0 sinusoidal */
    double rf_angle;    /* linear RF angle */
    double rf_revpart, rf_vrf, rf_v0, rf_bl2phase, rf_phase;
    double slip[3];     /* drift slip terms */
    int nslip;
    double e0;          /* beam energy (eV) for the drift */
    double e1;          /* FP decrement; <= 0: no FP term */
    int fptype, derivation;
    double wakescaling; /* ElectricField wakescaling (before /nmax); 0: none */
    int renormalize;    /* >0 every n steps, 0 initial only, <0 never */
} oracle_bunch_desc;
}

namespace vo {

template <typename T>
struct Bunch {
    oracle_bunch_desc d;
    Axis<T> ax, ay;
    std::vector<T> ws;
    std::vector<T> t1, t2, t3;
    std::vector<T> proj;
    T filling_set = 1, filling = 0;
    std::vector<u32> rf_idx, drift_idx, fp_idx, wake_idx;
    std::vector<T> rf_w, drift_w, fp_w, wake_w;
    std::vector<T> wake;
    bool has_fp = false, has_wake = false;
    T wakescale = 0;
    long step = 0;
};

template <typename T>
struct Sim {
    std::vector<Bunch<T>> bunches;
    size_t nmax = 0;
    std::vector<zf> Z;
};

template <typename T>
void bunch_init(Bunch<T>& B, const oracle_bunch_desc& d, const T* data,
                size_t nmax)
{
    const u32 n = static_cast<u32>(d.n);
    B.d = d;
    B.ax = make_axis<T>(n, T(d.qmin), T(d.qmax), T(d.qscale));
    B.ay = make_axis<T>(n, T(d.pmin), T(d.pmax), T(d.pscale));
    B.ws.resize(n);
    simpson_weights<T>(n, B.ax.delta, B.ws.data());
    const size_t nxy = size_t(n) * n;
    B.t1.assign(nxy, T(0));
    B.t2.assign(nxy, T(0));
    B.t3.assign(nxy, T(0));
    B.proj.assign(n, T(0));
    B.filling_set = 1;
    /* PhaseSpace constructor, src/PS/PhaseSpace.cpp:17-134 */
    if (data) {
        std::copy(data, data + nxy, B.t1.begin());
    } else {
        std::vector<T> gx(n), gy(n);
        gaussian(B.ax, d.zoom, gx.data());
        gaussian(B.ay, d.zoom, gy.data());
        for (u32 x = 0; x < n; x++) {
            for (u32 y = 0; y < n; y++) {
                B.t1[size_t(x) * n + y] = gx[x] * gy[y];
            }
        }
        project_x<T>(1, n, B.t1.data(), B.ws.data(), B.proj.data());
        integrate<T>(1, n, B.proj.data(), B.ws.data(), &B.filling);
        normalize<T>(1, n, B.t1.data(), &B.filling_set, &B.filling);
    }
    project_x<T>(1, n, B.t1.data(), B.ws.data(), B.proj.data());
    integrate<T>(1, n, B.proj.data(), B.ws.data(), &B.filling);
    /* src/main.cpp:527-532: initial renormalisation */
    if (d.renormalize >= 0) {
        project_x<T>(1, n, B.t1.data(), B.ws.data(), B.proj.data());
        normalize<T>(1, n, B.t1.data(), &B.filling_set, &B.filling);
    }
    const int it = d.it;
    if (d.chain == 0) {
        std::vector<T> off(n);
        if (d.rf_linear) {
            rf_offsets_linear<T>(B.ax, T(d.rf_angle), T(0), T(d.rf_bl2phase),
                                 T(1), off.data());
        } else {
            rf_offsets_sin<T>(B.ax, B.ay, T(d.rf_revpart), T(d.rf_vrf),
                              T(d.rf_v0), T(d.rf_bl2phase), T(d.rf_phase), T(1),
                              off.data());
        }
        B.rf_idx.resize(size_t(n) * it);
        B.rf_w.resize(size_t(n) * it);
        kick_stencils<T>(n, it, off.data(), n, B.rf_idx.data(),
                         B.rf_w.data());
        T slip[3] = {T(d.slip[0]), T(d.slip[1]), T(d.slip[2])};
        drift_offsets<T>(B.ax, B.ay, slip, d.nslip, T(d.e0), off.data());
        B.drift_idx.resize(size_t(n) * it);
        B.drift_w.resize(size_t(n) * it);
        kick_stencils<T>(n, it, off.data(), n, B.drift_idx.data(),
                         B.drift_w.data());
    }
    B.has_fp = d.e1 > 0;
    if (B.has_fp) {
        B.fp_idx.resize(size_t(n) * d.derivation);
        B.fp_w.resize(size_t(n) * d.derivation);
        fp_stencils<T>(B.ay, T(d.e1), d.fptype, d.derivation, B.fp_idx.data(),
                       B.fp_w.data());
    }
    B.has_wake = d.wakescaling != 0 && nmax > 0;
    B.wakescale = static_cast<T>(static_cast<T>(d.wakescaling)
                                 / static_cast<T>(nmax));
    B.wake.assign(n, T(0));
    B.wake_idx.resize(size_t(n) * it);
    B.wake_w.resize(size_t(n) * it);
    B.step = 0;
}

template <typename T>
void bunch_step(Bunch<T>& B, size_t nmax, const zf* Z)
{
    const u32 n = static_cast<u32>(B.d.n);
    const int it = B.d.it;
    const u32 bucket0 = 0;
    if (B.has_wake) {
        wake_potential<T>(1, n, nmax, B.proj.data(), &bucket0, 0, Z,
                          B.wakescale, B.wake.data(), nullptr);
        kick_stencils<T>(n, it, B.wake.data(), n, B.wake_idx.data(),
                         B.wake_w.data());
    }
    if (B.d.renormalize > 0 && B.step % B.d.renormalize == 0) {
        integrate<T>(1, n, B.proj.data(), B.ws.data(), &B.filling);
        normalize<T>(1, n, B.t1.data(), &B.filling_set, &B.filling);
    } else {
        integrate<T>(1, n, B.proj.data(), B.ws.data(), &B.filling);
    }
    T* t1 = B.t1.data();
    T* t2 = B.t2.data();
    T* t3 = B.t3.data();
    const size_t nxy = size_t(n) * n;
    if (B.d.chain == 0) {
        if (B.has_wake) {
            kick_apply<T>(1, 1, n, it, B.wake_idx.data(), B.wake_w.data(), t1,
                          t2);
        } else {
            std::copy(t1, t1 + nxy, t2);
        }
        kick_apply<T>(1, 1, n, it, B.rf_idx.data(), B.rf_w.data(), t2, t1);
        kick_apply<T>(0, 1, n, it, B.drift_idx.data(), B.drift_w.data(), t1,
                      t3);
    } else {
        rotation_apply<T>(B.ax, B.ay, T(B.d.angle), it, B.d.clamp != 0, 1, t1,
                          t2);
        if (B.has_wake) {
            kick_apply<T>(1, 1, n, it, B.wake_idx.data(), B.wake_w.data(), t2,
                          t3);
        } else {
            std::copy(t2, t2 + nxy, t3);
        }
    }
    if (B.has_fp) {
        fp_apply<T>(1, n, B.d.derivation, B.fp_idx.data(), B.fp_w.data(), t3,
                    t1);
    } else {
        std::copy(t3, t3 + nxy, t1);
    }
    project_x<T>(1, n, t1, B.ws.data(), B.proj.data());
    B.step++;
}

template <typename T>
void sim_steps(Sim<T>& S, long nsteps, int nthreads)
{
    const size_t nb = S.bunches.size();
    if (nthreads <= 1 || nb <= 1) {
        for (size_t b = 0; b < nb; b++) {
            for (long s = 0; s < nsteps; s++) {
                bunch_step(S.bunches[b], S.nmax, S.Z.data());
            }
        }
        return;
    }
    std::vector<std::thread> pool;
    const size_t nt = std::min<size_t>(nthreads, nb);
    for (size_t t = 0; t < nt; t++) {
        pool.emplace_back([&S, t, nt, nb, nsteps]() {
            for (size_t b = t; b < nb; b += nt) {
                for (long s = 0; s < nsteps; s++) {
                    bunch_step(S.bunches[b], S.nmax, S.Z.data());
                }
            }
        });
    }
    for (auto& th : pool) {
        th.join();
    }
}

}  // namespace vo

/* ================================================================ C API */
using vo::u32;
using vo::zf;

#define OR_EXPORT extern "C" __attribute__((visibility("default")))

#define OR_BOTH(ret, name, params, call_f, call_d) \
    OR_EXPORT ret name##_f32 params { call_f; }    \
    OR_EXPORT ret name##_f64 params { call_d; }

template <typename T>
static vo::Axis<T> axis_from(u32 n, double mn, double mx, double scale)
{
    return vo::make_axis<T>(n, T(mn), T(mx), T(scale));
}

/* axis: values, delta and zerobin of a Ruler */
template <typename T>
static void ruler_impl(u32 n, double mn, double mx, T* values, T* delta,
                       T* zerobin)
{
    auto a = axis_from<T>(n, mn, mx, 1);
    if (values) {
        std::copy(a.v.begin(), a.v.end(), values);
    }
    *delta = a.delta;
    *zerobin = a.zerobin;
}
OR_EXPORT void oracle_ruler_f32(u32 n, double mn, double mx, float* v,
                                float* d, float* z)
{
    ruler_impl<float>(n, mn, mx, v, d, z);
}
OR_EXPORT void oracle_ruler_f64(u32 n, double mn, double mx, double* v,
                                double* d, double* z)
{
    ruler_impl<double>(n, mn, mx, v, d, z);
}

template <typename T>
static void simpson_impl(u32 n, double mn, double mx, T* ws)
{
    auto a = axis_from<T>(n, mn, mx, 1);
    vo::simpson_weights<T>(n, a.delta, ws);
}
OR_EXPORT void oracle_simpson_f32(u32 n, double mn, double mx, float* ws)
{
    simpson_impl<float>(n, mn, mx, ws);
}
OR_EXPORT void oracle_simpson_f64(u32 n, double mn, double mx, double* ws)
{
    simpson_impl<double>(n, mn, mx, ws);
}

/* PhaseSpace constructor: Gaussian (data==NULL) or copied data; fills the
 * density, both projections and the bunch populations. Returns 0, or -1
 * when the filling is not normalised (src/PS/PhaseSpace.cpp:47-51). */
template <typename T>
static int ps_init_impl(u32 nb, u32 n, const double* ax6, const T* filling_set,
                        double zoom, const T* data, T* out, T* projx, T* projy,
                        T* filling, T* integral)
{
    T fsum = 0;
    for (u32 b = 0; b < nb; b++) {
        fsum += filling_set[b];
    }
    if (std::round(1e5 * fsum) != 1e5) {
        return -1;
    }
    auto ax = axis_from<T>(n, ax6[0], ax6[1], ax6[2]);
    auto ay = axis_from<T>(n, ax6[3], ax6[4], ax6[5]);
    std::vector<T> ws(n);
    vo::simpson_weights<T>(n, ax.delta, ws.data());
    const size_t nxy = size_t(n) * n;
    if (data) {
        std::copy(data, data + nxy * nb, out);
    } else {
        std::vector<T> gx(n), gy(n);
        vo::gaussian(ax, zoom, gx.data());
        vo::gaussian(ay, zoom, gy.data());
        for (u32 b = 0; b < nb; b++) {
            for (u32 x = 0; x < n; x++) {
                for (u32 y = 0; y < n; y++) {
                    out[b * nxy + size_t(x) * n + y] = gx[x] * gy[y];
                }
            }
        }
        vo::project_x<T>(nb, n, out, ws.data(), projx);
        vo::integrate<T>(nb, n, projx, ws.data(), filling);
        vo::normalize<T>(nb, n, out, filling_set, filling);
    }
    vo::project_x<T>(nb, n, out, ws.data(), projx);
    vo::project_y<T>(nb, n, out, ws.data(), projy);
    *integral = vo::integrate<T>(nb, n, projx, ws.data(), filling);
    return 0;
}
OR_EXPORT int oracle_ps_init_f32(u32 nb, u32 n, const double* ax6,
                                 const float* fs, double zoom,
                                 const float* data, float* out, float* px,
                                 float* py, float* filling, float* integral)
{
    return ps_init_impl<float>(nb, n, ax6, fs, zoom, data, out, px, py,
                               filling, integral);
}
OR_EXPORT int oracle_ps_init_f64(u32 nb, u32 n, const double* ax6,
                                 const double* fs, double zoom,
                                 const double* data, double* out, double* px,
                                 double* py, double* filling, double* integral)
{
    return ps_init_impl<double>(nb, n, ax6, fs, zoom, data, out, px, py,
                                filling, integral);
}

OR_BOTH(void, oracle_project_x,
        (u32 nb, u32 n, const void* data, const void* ws, void* proj),
        vo::project_x<float>(nb, n, (const float*)data, (const float*)ws,
                             (float*)proj),
        vo::project_x<double>(nb, n, (const double*)data, (const double*)ws,
                              (double*)proj))
OR_BOTH(void, oracle_project_y,
        (u32 nb, u32 n, const void* data, const void* ws, void* proj),
        vo::project_y<float>(nb, n, (const float*)data, (const float*)ws,
                             (float*)proj),
        vo::project_y<double>(nb, n, (const double*)data, (const double*)ws,
                              (double*)proj))
OR_BOTH(void, oracle_integrate,
        (u32 nb, u32 n, const void* proj, const void* ws, void* filling,
         void* total),
        *(float*)total = vo::integrate<float>(nb, n, (const float*)proj,
                                              (const float*)ws,
                                              (float*)filling),
        *(double*)total = vo::integrate<double>(nb, n, (const double*)proj,
                                                (const double*)ws,
                                                (double*)filling))
OR_BOTH(void, oracle_normalize,
        (u32 nb, u32 n, void* data, const void* fset, const void* filling),
        vo::normalize<float>(nb, n, (float*)data, (const float*)fset,
                             (const float*)filling),
        vo::normalize<double>(nb, n, (double*)data, (const double*)fset,
                              (const double*)filling))
OR_BOTH(void, oracle_moments,
        (u32 nb, u32 n, const void* axis, double delta, const void* proj,
         const void* fset, const void* filling, void* avg, void* var),
        vo::moments<float>(nb, n, (const float*)axis, float(delta),
                           (const float*)proj, (const float*)fset,
                           (const float*)filling, (float*)avg, (float*)var),
        vo::moments<double>(nb, n, (const double*)axis, delta,
                            (const double*)proj, (const double*)fset,
                            (const double*)filling, (double*)avg,
                            (double*)var))

/* RotationMap construction + apply over nb bunches.  Returns -1 for the
 * invalid clamp configurations of src/SM/RotationMap.cpp:83-87. */
template <typename T>
static int rotation_impl(u32 nb, u32 n, const double* ax6, double angle,
                         int it, int clamp, long rotmapsize, const T* in,
                         T* out)
{
    if (clamp && !(it == 4 && rotmapsize > 0)) {
        return -1;
    }
    auto ax = axis_from<T>(n, ax6[0], ax6[1], ax6[2]);
    auto ay = axis_from<T>(n, ax6[3], ax6[4], ax6[5]);
    vo::rotation_apply<T>(ax, ay, T(angle), it, clamp != 0, nb, in, out);
    return 0;
}
OR_BOTH(int, oracle_rotation,
        (u32 nb, u32 n, const double* ax6, double angle, int it, int clamp,
         long rotmapsize, const void* in, void* out),
        return rotation_impl<float>(nb, n, ax6, angle, it, clamp, rotmapsize,
                                    (const float*)in, (float*)out),
        return rotation_impl<double>(nb, n, ax6, angle, it, clamp, rotmapsize,
                                     (const double*)in, (double*)out))

/* RotationMap::applyTo (src/SM/RotationMap.cpp:178-188), one particle */
template <typename T>
static void rotation_particle_impl(u32 n, const double* ax6, double angle,
                                   T* pos)
{
    auto ax = axis_from<T>(n, ax6[0], ax6[1], ax6[2]);
    auto ay = axis_from<T>(n, ax6[3], ax6[4], ax6[5]);
    const T cs = std::cos(-T(angle));
    const T sn = std::sin(-T(angle));
    const T x = cs * (pos[0] - ax.zerobin) + sn * (pos[1] - ay.zerobin)
                + ax.zerobin;
    const T y = cs * (pos[1] - ay.zerobin) - sn * (pos[0] - ax.zerobin)
                + ay.zerobin;
    pos[0] = x;
    pos[1] = y;
}
OR_BOTH(void, oracle_rotation_particle,
        (u32 n, const double* ax6, double angle, void* pos),
        rotation_particle_impl<float>(n, ax6, angle, (float*)pos),
        rotation_particle_impl<double>(n, ax6, angle, (double*)pos))

OR_BOTH(void, oracle_kick_stencils,
        (u32 kd, int it, const void* offset, size_t count, u32* idx, void* w),
        vo::kick_stencils<float>(kd, it, (const float*)offset, count, idx,
                                 (float*)w),
        vo::kick_stencils<double>(kd, it, (const double*)offset, count, idx,
                                  (double*)w))
OR_BOTH(void, oracle_kick_apply,
        (int axis, u32 nb, u32 n, int it, const u32* idx, const void* w,
         const void* in, void* out),
        vo::kick_apply<float>(axis, nb, n, it, idx, (const float*)w,
                              (const float*)in, (float*)out),
        vo::kick_apply<double>(axis, nb, n, it, idx, (const double*)w,
                               (const double*)in, (double*)out))

/* KickMap::applyTo (src/SM/KickMap.cpp:280-303), one particle. */
template <typename T>
static void kick_particle_impl(int axis, u32 n, const T* offset, T* pos)
{
    T& along = (axis == 0) ? pos[0] : pos[1];
    const T across = (axis == 0) ? pos[1] : pos[0];
    T ip;
    const T f = std::modf(across, &ip);
    u32 i = 0;
    const bool ok = vo::base_index(ip, 0xffffffffu, &i);
    if (ok && i + 1 < n) {
        along -= (1 - f) * offset[i] + f * offset[i + 1];
    }
    along = std::max(static_cast<T>(1), std::min(along, static_cast<T>(n - 1)));
}
OR_BOTH(void, oracle_kick_particle,
        (int axis, u32 n, const void* offset, void* pos),
        kick_particle_impl<float>(axis, n, (const float*)offset, (float*)pos),
        kick_particle_impl<double>(axis, n, (const double*)offset,
                                   (double*)pos))

template <typename T>
static void drift_offsets_impl(u32 n, const double* ax6, const double* slip,
                               int nslip, double e0, T* off)
{
    auto ax = axis_from<T>(n, ax6[0], ax6[1], ax6[2]);
    auto ay = axis_from<T>(n, ax6[3], ax6[4], ax6[5]);
    T s[3] = {T(slip[0]), T(nslip > 1 ? slip[1] : 0),
              T(nslip > 2 ? slip[2] : 0)};
    vo::drift_offsets<T>(ax, ay, s, nslip, T(e0), off);
}
OR_BOTH(void, oracle_drift_offsets,
        (u32 n, const double* ax6, const double* slip, int nslip, double e0,
         void* off),
        drift_offsets_impl<float>(n, ax6, slip, nslip, e0, (float*)off),
        drift_offsets_impl<double>(n, ax6, slip, nslip, e0, (double*)off))

template <typename T>
static void rf_offsets_impl(u32 n, const double* ax6, int linear,
                            double angle, double revpart, double vrf,
                            double v0, double bl2phase, double phase,
                            double ampl, T* off)
{
    auto ax = axis_from<T>(n, ax6[0], ax6[1], ax6[2]);
    auto ay = axis_from<T>(n, ax6[3], ax6[4], ax6[5]);
    if (linear) {
        vo::rf_offsets_linear<T>(ax, T(angle), T(0), T(bl2phase), T(ampl),
                                 off);
    } else {
        vo::rf_offsets_sin<T>(ax, ay, T(revpart), T(vrf), T(v0), T(bl2phase),
                              T(phase), T(ampl), off);
    }
}
OR_BOTH(void, oracle_rf_offsets,
        (u32 n, const double* ax6, int linear, double angle, double revpart,
         double vrf, double v0, double bl2phase, double phase, double ampl,
         void* off),
        rf_offsets_impl<float>(n, ax6, linear, angle, revpart, vrf, v0,
                               bl2phase, phase, ampl, (float*)off),
        rf_offsets_impl<double>(n, ax6, linear, angle, revpart, vrf, v0,
                                bl2phase, phase, ampl, (double*)off))

template <typename T>
static int fp_stencils_impl(u32 n, const double* ax6, double e1, int fptype,
                            int derivation, u32* idx, T* w)
{
    auto ay = axis_from<T>(n, ax6[3], ax6[4], ax6[5]);
    return vo::fp_stencils<T>(ay, T(e1), fptype, derivation, idx, w);
}
OR_BOTH(int, oracle_fp_stencils,
        (u32 n, const double* ax6, double e1, int fptype, int derivation,
         u32* idx, void* w),
        return fp_stencils_impl<float>(n, ax6, e1, fptype, derivation, idx,
                                       (float*)w),
        return fp_stencils_impl<double>(n, ax6, e1, fptype, derivation, idx,
                                        (double*)w))
OR_BOTH(void, oracle_fp_apply,
        (u32 nb, u32 n, int ip, const u32* idx, const void* w, const void* in,
         void* out),
        vo::fp_apply<float>(nb, n, ip, idx, (const float*)w, (const float*)in,
                            (float*)out),
        vo::fp_apply<double>(nb, n, ip, idx, (const double*)w,
                             (const double*)in, (double*)out))

OR_EXPORT void oracle_airy(double x, double* out4, int* overflow)
{
    vo::airy(x, out4, out4 + 1, out4 + 2, out4 + 3, overflow);
}

/* Impedance tables as interleaved (re, im) float pairs. */
OR_EXPORT void oracle_z_free_space(size_t n, float f_rev, float f_max,
                                   float* out)
{
    vo::z_free_space(n, f_rev, f_max, reinterpret_cast<zf*>(out));
}
OR_EXPORT void oracle_z_parallel_plates(size_t n, float f0, float f_max,
                                        double g, float* out)
{
    vo::z_parallel_plates(n, f0, f_max, g, reinterpret_cast<zf*>(out));
}
OR_EXPORT void oracle_z_resistive_wall(size_t n, float f0, float f_max,
                                       double L, double s, double xi,
                                       double b, float* out)
{
    vo::z_resistive_wall(n, f0, f_max, L, s, xi, b, reinterpret_cast<zf*>(out));
}
OR_EXPORT void oracle_z_const(size_t n, float re, float im, float* out)
{
    vo::z_const(n, zf(re, im), reinterpret_cast<zf*>(out));
}
OR_EXPORT void oracle_z_collimator(size_t n, double outer, double inner,
                                   float* out)
{
    vo::z_collimator(n, outer, inner, reinterpret_cast<zf*>(out));
}

/* makeImpedance (src/Z/ImpedanceFactory.cpp:21-84) without the file term.
 * Returns 0 if some impedance was added, 1 if the result is "no impedance". */
OR_EXPORT int oracle_make_impedance(size_t nfreqs, float fmax, double r_bend,
                                    double frev, double gap, int use_csr,
                                    double s, double xi, double coll,
                                    float* out)
{
    const double f0 = vo::C_LIGHT / (2 * vo::PI * r_bend);
    std::vector<zf> acc(nfreqs, zf(0, 0)), term(nfreqs);
    bool changed = false;
    auto add = [&]() {
        for (size_t i = 0; i < nfreqs; i++) {
            acc[i] += term[i];
        }
    };
    if (gap != 0) {
        if (use_csr) {
            changed = true;
            if (gap > 0) {
                vo::z_parallel_plates(nfreqs, float(f0), fmax, gap,
                                      term.data());
            } else {
                vo::z_free_space(nfreqs, float(f0), fmax, term.data());
            }
            add();
        }
        const double radius = std::abs(gap / 2);
        if (s > 0 && xi >= -1) {
            changed = true;
            vo::z_resistive_wall(nfreqs, float(frev), fmax,
                                 vo::C_LIGHT / frev, s, xi, radius,
                                 term.data());
            add();
        }
        if (0 < coll && coll < radius) {
            changed = true;
            vo::z_collimator(nfreqs, radius, coll, term.data());
            add();
        }
    }
    std::memcpy(out, acc.data(), nfreqs * sizeof(zf));
    return changed ? 0 : 1;
}

template <typename T>
static void wake_impl(u32 nb, u32 n, size_t nmax, const T* proj,
                      const u32* bucket, size_t spacing, const float* Z,
                      double wakescaling, T* wake, T* padded)
{
    const T ws = static_cast<T>(static_cast<T>(wakescaling)
                                / static_cast<T>(nmax));
    vo::wake_potential<T>(nb, n, nmax, proj, bucket, spacing,
                          reinterpret_cast<const zf*>(Z), ws, wake, padded);
}
OR_BOTH(void, oracle_wake_potential,
        (u32 nb, u32 n, size_t nmax, const void* proj, const u32* bucket,
         size_t spacing, const float* Z, double wakescaling, void* wake,
         void* padded),
        wake_impl<float>(nb, n, nmax, (const float*)proj, bucket, spacing, Z,
                         wakescaling, (float*)wake, (float*)padded),
        wake_impl<double>(nb, n, nmax, (const double*)proj, bucket, spacing, Z,
                          wakescaling, (double*)wake, (double*)padded))

OR_BOTH(void, oracle_csr,
        (u32 n, size_t nmax, const void* proj, const float* Z, double dq,
         double fc, double freq_scale, void* spectrum, void* power),
        *(float*)power = vo::csr<float>(n, nmax, (const float*)proj,
                                        reinterpret_cast<const zf*>(Z),
                                        float(dq), float(fc),
                                        float(freq_scale), (float*)spectrum),
        *(double*)power = vo::csr<double>(n, nmax, (const double*)proj,
                                          reinterpret_cast<const zf*>(Z), dq,
                                          fc, freq_scale, (double*)spectrum))

/* Real <-> half-spectrum transforms, for checking the FFT itself. */
OR_EXPORT void oracle_rfft_f64(const double* x, size_t n, double* out_ri)
{
    std::vector<std::complex<double>> o(n);
    vo::rfft(x, n, o.data());
    std::memcpy(out_ri, o.data(), n * sizeof(std::complex<double>));
}

/* --- solver loop over independent bunches --- */
template <typename T>
static void* sim_create_impl(int nb, const oracle_bunch_desc* descs,
                             const T* data, size_t nmax, const float* Z)
{
    auto* S = new vo::Sim<T>();
    S->nmax = nmax;
    if (Z && nmax) {
        const zf* z = reinterpret_cast<const zf*>(Z);
        S->Z.assign(z, z + nmax);
    }
    S->bunches.resize(nb);
    size_t off = 0;
    for (int b = 0; b < nb; b++) {
        vo::bunch_init<T>(S->bunches[b], descs[b], data ? data + off : nullptr,
                          Z ? nmax : 0);
        off += size_t(descs[b].n) * descs[b].n;
    }
    return S;
}
OR_EXPORT void* oracle_sim_create_f32(int nb, const oracle_bunch_desc* d,
                                      const float* data, size_t nmax,
                                      const float* Z)
{
    return sim_create_impl<float>(nb, d, data, nmax, Z);
}
OR_EXPORT void* oracle_sim_create_f64(int nb, const oracle_bunch_desc* d,
                                      const double* data, size_t nmax,
                                      const float* Z)
{
    return sim_create_impl<double>(nb, d, data, nmax, Z);
}
OR_EXPORT void oracle_sim_step_f32(void* s, long nsteps, int nthreads)
{
    vo::sim_steps(*static_cast<vo::Sim<float>*>(s), nsteps, nthreads);
}
OR_EXPORT void oracle_sim_step_f64(void* s, long nsteps, int nthreads)
{
    vo::sim_steps(*static_cast<vo::Sim<double>*>(s), nsteps, nthreads);
}
/* what: 0 density t1, 1 x projection, 2 wake potential, 3 filling */
template <typename T>
static void sim_get_impl(void* s, int b, int what, T* out)
{
    auto& B = static_cast<vo::Sim<T>*>(s)->bunches[b];
    switch (what) {
    case 0:
        std::copy(B.t1.begin(), B.t1.end(), out);
        break;
    case 1:
        std::copy(B.proj.begin(), B.proj.end(), out);
        break;
    case 2:
        std::copy(B.wake.begin(), B.wake.end(), out);
        break;
    case 3:
        *out = B.filling;
        break;
    }
}
OR_EXPORT void oracle_sim_get_f32(void* s, int b, int what, float* out)
{
    sim_get_impl<float>(s, b, what, out);
}
OR_EXPORT void oracle_sim_get_f64(void* s, int b, int what, double* out)
{
    sim_get_impl<double>(s, b, what, out);
}
OR_EXPORT void oracle_sim_destroy_f32(void* s)
{
    delete static_cast<vo::Sim<float>*>(s);
}
OR_EXPORT void oracle_sim_destroy_f64(void* s)
{
    delete static_cast<vo::Sim<double>*>(s);
}
