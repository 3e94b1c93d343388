/* C++ façade over the C ABI of vfps.h with the reference's class names and
 * constructor parameters, so that a solver loop written against
 * inc/PS/PhaseSpace.hpp, the map headers of inc/SM, inc/PS/ElectricField.hpp
 * and the impedance headers of inc/Z compiles against the GPU path with the
 * handle type (vfps::ctxptr_t instead of oclhptr_t) as the only change.
 *
 * Header only; link with libvfps.so.  Errors become exceptions as in the
 * reference: std::invalid_argument for VFPS_ERR_INVALID_ARGUMENT (bad
 * filling, bad clamp configuration, Ruler min >= max), std::runtime_error
 * for everything else.  Objects own their handles (move-only). */
#ifndef VFPS_HPP
#define VFPS_HPP

#include <cstdint>
#include <memory>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "vfps.h"

namespace vfps {

inline void check(int rc, const vfps_ctx* ctx)
{
    if (rc == VFPS_OK) {
        return;
    }
    const char* m = vfps_last_error(ctx);
    const std::string msg = m ? m : "vfps error";
    if (rc == VFPS_ERR_INVALID_ARGUMENT) {
        throw std::invalid_argument(msg);
    }
    throw std::runtime_error(msg + " (status " + std::to_string(rc) + ")");
}

/* one device and its in-order stream; stands in for oclhptr_t */
class Context {
public:
    explicit Context(int device = 0) { check(vfps_create(&h_, device), nullptr); }
    ~Context() { vfps_destroy(h_); }
    Context(const Context&) = delete;
    Context& operator=(const Context&) = delete;
    vfps_ctx* get() const { return h_; }
    void synchronize() { check(vfps_synchronize(h_), h_); }
    int deviceStatus()
    {
        int c = 0;
        check(vfps_device_status(h_, &c), h_);
        return c;
    }

private:
    vfps_ctx* h_ = nullptr;
};
using ctxptr_t = std::shared_ptr<Context>;

/* inc/PS/PhaseSpace.hpp:54-96; the static setSize becomes the n argument */
class PhaseSpace {
public:
    PhaseSpace(double qmin, double qmax, double qscale, double pmin,
               double pmax, double pscale, ctxptr_t ctx, double Fk,
               double Iz, const std::vector<float>& filling, double zoom,
               uint32_t n, const float* data = nullptr)
        : ctx_(std::move(ctx))
    {
        const double axes[6] = {qmin, qmax, qscale, pmin, pmax, pscale};
        check(vfps_ps_create(ctx_->get(), uint32_t(filling.size()), n, axes,
                             Fk, Iz, filling.data(), zoom, data, &h_),
              ctx_->get());
        check(vfps_ps_shape(h_, &nb_, &n_), ctx_->get());
    }
    PhaseSpace(const PhaseSpace& o) : ctx_(o.ctx_), nb_(o.nb_), n_(o.n_)
    {
        check(vfps_ps_copy(o.h_, &h_), ctx_->get());
    }
    PhaseSpace& operator=(const PhaseSpace& o)
    {
        check(vfps_ps_assign(h_, o.h_), ctx_->get());
        return *this;
    }
    ~PhaseSpace() { vfps_ps_destroy(h_); }
    vfps_ps* handle() const { return h_; }
    uint32_t nx() const { return n_; }
    uint32_t nb() const { return nb_; }
    size_t nxyb() const { return size_t(nb_) * n_ * n_; }

    void updateXProjection() { check(vfps_ps_update_x_projection(h_), c()); }
    void updateYProjection() { check(vfps_ps_update_y_projection(h_), c()); }
    void integrate() { check(vfps_ps_integrate(h_), c()); }
    void normalize() { check(vfps_ps_normalize(h_), c()); }
    void integrateAndNormalize()
    {
        check(vfps_ps_integrate_and_normalize(h_), c());
    }
    void variance(int axis) { check(vfps_ps_variance(h_, axis), c()); }
    std::vector<float> getData()
    {
        std::vector<float> d(nxyb());
        check(vfps_ps_download(h_, d.data()), c());
        return d;
    }
    void setData(const std::vector<float>& d)
    {
        if (d.size() != nxyb()) {
            throw std::invalid_argument("setData: wrong size");
        }
        check(vfps_ps_upload(h_, d.data()), c());
    }
    std::vector<float> getProjection(int axis)
    {
        std::vector<float> p(size_t(nb_) * n_);
        check(vfps_ps_get_projection(h_, axis, p.data()), c());
        return p;
    }
    std::vector<float> getBunchPopulation()
    {
        std::vector<float> f(nb_);
        check(vfps_ps_get_filling(h_, f.data(), nullptr), c());
        return f;
    }
    double getIntegral()
    {
        double v = 0;
        check(vfps_ps_get_filling(h_, nullptr, &v), c());
        return v;
    }
    float getDelta(int axis) const
    {
        float d = 0;
        check(vfps_ps_axis(h_, axis, nullptr, &d, nullptr), c());
        return d;
    }

private:
    vfps_ctx* c() const { return ctx_->get(); }
    ctxptr_t ctx_;
    vfps_ps* h_ = nullptr;
    uint32_t nb_ = 0, n_ = 0;
};
using psptr_t = std::shared_ptr<PhaseSpace>;

/* inc/SM/SourceMap.hpp:53-87 */
class SourceMap {
public:
    virtual ~SourceMap() { vfps_map_destroy(m_); }
    SourceMap(const SourceMap&) = delete;
    SourceMap& operator=(const SourceMap&) = delete;
    virtual void apply() { check(vfps_map_apply(m_), c()); }
    /* applyTo/applyToAll: pos = {x0, y0, x1, y1, ...} in mesh units */
    void applyToAll(std::vector<float>& pos)
    {
        check(vfps_map_apply_to(m_, pos.data(), pos.size() / 2), c());
    }
    vfps_map* handle() const { return m_; }

protected:
    SourceMap(psptr_t in, psptr_t out, ctxptr_t ctx)
        : in_(std::move(in)), out_(std::move(out)), ctx_(std::move(ctx)) {}
    vfps_ctx* c() const { return ctx_->get(); }
    psptr_t in_, out_;
    ctxptr_t ctx_;
    vfps_map* m_ = nullptr;
};

/* inc/SM/RotationMap.hpp:40-45 */
class RotationMap : public SourceMap {
public:
    RotationMap(psptr_t in, psptr_t out, uint32_t xsize, uint32_t ysize,
                float angle, int it, bool clamp, size_t rotmapsize,
                ctxptr_t ctx)
        : SourceMap(in, out, ctx)
    {
        check(vfps_rotation_map_create(in->handle(), out->handle(), xsize,
                                       ysize, angle, it, clamp,
                                       uint32_t(rotmapsize), &m_),
              c());
    }
};

/* inc/SM/KickMap.hpp:34-38 (axis 0: x-kick, 1: y-kick) */
class KickMap : public SourceMap {
public:
    KickMap(psptr_t in, psptr_t out, int it, bool clamp, int axis,
            ctxptr_t ctx)
        : SourceMap(in, out, ctx)
    {
        check(vfps_kick_map_create(in->handle(), out->handle(), it, clamp,
                                   axis, &m_),
              c());
    }
    void swapOffset(const std::vector<float>& offset)
    {
        check(vfps_kick_map_set_offset(m_, offset.data(), offset.size()),
              c());
    }

protected:
    explicit KickMap(psptr_t in, psptr_t out, ctxptr_t ctx)
        : SourceMap(in, out, ctx) {}
};

/* inc/SM/DriftMap.hpp:17-24 */
class DriftMap : public KickMap {
public:
    DriftMap(psptr_t in, psptr_t out, const std::vector<float>& slip,
             float E0, int it, bool clamp, ctxptr_t ctx)
        : KickMap(in, out, ctx)
    {
        check(vfps_drift_map_create(in->handle(), out->handle(), slip.data(),
                                    uint32_t(slip.size()), E0, it, clamp,
                                    &m_),
              c());
    }
};

/* inc/SM/RFKickMap.hpp:17-34: linear RF, or sinusoidal RF */
class RFKickMap : public KickMap {
public:
    RFKickMap(psptr_t in, psptr_t out, float angle, float f_RF, int it,
              bool clamp, ctxptr_t ctx)
        : KickMap(in, out, ctx)
    {
        check(vfps_rf_kick_map_create_linear(in->handle(), out->handle(),
                                             angle, f_RF, it, clamp, &m_),
              c());
    }
    RFKickMap(psptr_t in, psptr_t out, float revolutionpart, float V_RF,
              float f_RF, float V0, int it, bool clamp, ctxptr_t ctx)
        : KickMap(in, out, ctx)
    {
        check(vfps_rf_kick_map_create(in->handle(), out->handle(),
                                      revolutionpart, V_RF, f_RF, V0, it,
                                      clamp, &m_),
              c());
    }
};

/* inc/SM/FokkerPlanckMap.hpp:56-64 */
class FokkerPlanckMap : public SourceMap {
public:
    FokkerPlanckMap(psptr_t in, psptr_t out, uint32_t xsize, uint32_t ysize,
                    int fptype, int fptrack, float e1, int derivation,
                    ctxptr_t ctx)
        : SourceMap(in, out, ctx)
    {
        check(vfps_fokker_planck_map_create(in->handle(), out->handle(),
                                            xsize, ysize, fptype, fptrack,
                                            e1, derivation, &m_),
              c());
    }
};

/* inc/SM/Identity.hpp:29-34 */
class Identity : public SourceMap {
public:
    Identity(psptr_t in, psptr_t out, ctxptr_t ctx) : SourceMap(in, out, ctx)
    {
        check(vfps_identity_map_create(in->handle(), out->handle(), &m_),
              c());
    }
};

/* inc/Z/Impedance.hpp:29-113 and the model classes of inc/Z/ */
class Impedance {
public:
    Impedance(ctxptr_t ctx, vfps_impedance* h) : ctx_(std::move(ctx)), h_(h) {}
    Impedance(const Impedance& o) : ctx_(o.ctx_)
    {
        check(vfps_impedance_copy(o.h_, &h_), ctx_->get());
    }
    ~Impedance() { vfps_impedance_destroy(h_); }
    Impedance& operator+=(const Impedance& rhs)
    {
        check(vfps_impedance_add(h_, rhs.h_), ctx_->get());
        return *this;
    }
    size_t nFreqs() const
    {
        size_t n = 0;
        check(vfps_impedance_get(h_, nullptr, &n, nullptr), ctx_->get());
        return n;
    }
    std::vector<float> data() const   /* re, im interleaved */
    {
        std::vector<float> z(2 * nFreqs());
        check(vfps_impedance_get(h_, z.data(), nullptr, nullptr),
              ctx_->get());
        return z;
    }
    const vfps_impedance* handle() const { return h_; }

    static std::shared_ptr<Impedance> freeSpaceCSR(ctxptr_t c, size_t n,
                                                   float f_rev, float f_max)
    {
        vfps_impedance* h = nullptr;
        check(vfps_impedance_free_space_csr(c->get(), n, f_rev, f_max, &h),
              c->get());
        return std::make_shared<Impedance>(c, h);
    }
    static std::shared_ptr<Impedance> parallelPlatesCSR(ctxptr_t c, size_t n,
                                                        float f0,
                                                        float f_max,
                                                        double g)
    {
        vfps_impedance* h = nullptr;
        check(vfps_impedance_parallel_plates_csr(c->get(), n, f0, f_max, g,
                                                 &h),
              c->get());
        return std::make_shared<Impedance>(c, h);
    }
    static std::shared_ptr<Impedance> resistiveWall(ctxptr_t c, size_t n,
                                                    float f0, float f_max,
                                                    double L, double s,
                                                    double xi, double b)
    {
        vfps_impedance* h = nullptr;
        check(vfps_impedance_resistive_wall(c->get(), n, f0, f_max, L, s, xi,
                                            b, &h),
              c->get());
        return std::make_shared<Impedance>(c, h);
    }

private:
    ctxptr_t ctx_;
    vfps_impedance* h_ = nullptr;
};
using impptr_t = std::shared_ptr<Impedance>;

/* makeImpedance (inc/Z/ImpedanceFactory.hpp:35-46); nullptr when no
 * contribution is selected */
inline impptr_t makeImpedance(ctxptr_t c, size_t nfreqs, float fmax,
                              double R_bend, double frev, double gap,
                              bool use_csr = true, double s = 0,
                              double xi = 0, double collimator_radius = 0,
                              const std::string& impedance_file = "")
{
    vfps_impedance* h = nullptr;
    check(vfps_make_impedance(c->get(), nfreqs, fmax, R_bend, frev, gap,
                              use_csr, s, xi, collimator_radius,
                              impedance_file.empty() ? nullptr
                                                     : impedance_file.c_str(),
                              &h),
          c->get());
    return h ? std::make_shared<Impedance>(c, h) : nullptr;
}

/* inc/PS/ElectricField.hpp:49-103 */
class ElectricField {
public:
    /* CSR field (no wake potential) */
    ElectricField(psptr_t ps, impptr_t z, const std::vector<uint32_t>& buckets,
                  uint32_t spacing_bins, ctxptr_t ctx, double f_rev,
                  double revolutionpart)
        : ps_(std::move(ps)), z_(std::move(z)), ctx_(std::move(ctx))
    {
        check(vfps_field_create(ps_->handle(), z_->handle(), buckets.data(),
                                spacing_bins, f_rev, revolutionpart, 0.0,
                                &h_),
              ctx_->get());
    }
    /* field with wake potential */
    ElectricField(psptr_t ps, impptr_t z, const std::vector<uint32_t>& buckets,
                  uint32_t spacing_bins, ctxptr_t ctx, double f_rev,
                  double revolutionpart, double Ib, double E0, double sE,
                  double dt)
        : ps_(std::move(ps)), z_(std::move(z)), ctx_(std::move(ctx))
    {
        check(vfps_field_create_wake(ps_->handle(), z_->handle(),
                                     buckets.data(), spacing_bins, f_rev,
                                     revolutionpart, Ib, E0, sE, dt, &h_),
              ctx_->get());
    }
    ~ElectricField() { vfps_field_destroy(h_); }
    ElectricField(const ElectricField&) = delete;
    ElectricField& operator=(const ElectricField&) = delete;
    vfps_field* handle() const { return h_; }

    /* wakePotential(): computed on the device; returned to the host */
    std::vector<float> wakePotential()
    {
        check(vfps_field_wake_potential(h_), ctx_->get());
        return getWakePotentials();
    }
    std::vector<float> getWakePotentials()
    {
        std::vector<float> w(size_t(ps_->nb()) * ps_->nx());
        check(vfps_field_get_wake_potential(h_, w.data()), ctx_->get());
        return w;
    }
    /* updateCSR(fc): the CSR power of each bunch */
    std::vector<float> updateCSR(float fc)
    {
        check(vfps_field_update_csr(h_, fc), ctx_->get());
        return getCSRPower();
    }
    std::vector<float> getCSRPower()
    {
        std::vector<float> p(ps_->nb());
        check(vfps_field_get_csr(h_, nullptr, p.data(), nullptr),
              ctx_->get());
        return p;
    }

private:
    psptr_t ps_;
    impptr_t z_;
    ctxptr_t ctx_;
    vfps_field* h_ = nullptr;
};

/* inc/SM/WakePotentialMap.hpp:20-26 with WakeKickMap::update() */
class WakePotentialMap : public KickMap {
public:
    WakePotentialMap(psptr_t in, psptr_t out, ElectricField* field, int it,
                     bool clamp, ctxptr_t ctx)
        : KickMap(in, out, ctx)
    {
        check(vfps_wake_potential_map_create(in->handle(), out->handle(),
                                             field->handle(), it, clamp,
                                             &m_),
              c());
    }
    void update() { check(vfps_wake_map_update(m_), c()); }
};

}  // namespace vfps

#endif /* VFPS_HPP */
