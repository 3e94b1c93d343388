/*
 * vfps.h -- C ABI of the GB300 phase-space hot path (libvfps.so).
 *
 * Replaces the C++/OpenCL objects of Inovesa's solver step: PhaseSpace,
 * the SourceMap family, Impedance and ElectricField.  Every call returns a
 * status (VFPS_OK = 0); the message of the last failure on a context is
 * read with vfps_last_error().  Signatures use plain pointers and sizes
 * only.  Host arrays are float / double in the reference's layouts:
 * densities [bunch][x][y] with y contiguous, projections [bunch][cell],
 * impedances as interleaved (re, im) float pairs.
 *
 * One context owns one CUDA stream on one device.  All work of a context
 * is ordered on that stream; calls that return host data synchronise it.
 * Contexts are independent: use one per host thread.
 *
 * Reference paths below are relative to the Inovesa source tree.
 */
#ifndef VFPS_H
#define VFPS_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define VFPS_API __attribute__((visibility("default")))

/* ------------------------------------------------------------ status */
enum {
    VFPS_OK = 0,
    /* std::invalid_argument in the reference (bad sizes, clamp set-up,
     * unnormalised filling, ...) */
    VFPS_ERR_INVALID_ARGUMENT = 1,
    VFPS_ERR_CUDA = 2,            /* a CUDA call failed */
    VFPS_ERR_OUT_OF_MEMORY = 3,
    VFPS_ERR_NUMERIC = 4,         /* NaN / non-positive charge watchdog */
    VFPS_ERR_TIMEOUT = 5,         /* a bounded device wait gave up */
    VFPS_ERR_IO = 6               /* impedance file could not be read */
};

/* interpolation points, src: inc/SM/SourceMap.hpp:22-27 */
enum { VFPS_INTERP_NONE = 1, VFPS_INTERP_LINEAR = 2,
       VFPS_INTERP_QUADRATIC = 3, VFPS_INTERP_CUBIC = 4 };
/* kick direction, inc/SM/KickMap.hpp:29-31 */
enum { VFPS_AXIS_X = 0, VFPS_AXIS_Y = 1 };
/* Fokker-Planck variants, inc/SM/FokkerPlanckMap.hpp:47-63 */
enum { VFPS_FP_NONE = 0, VFPS_FP_DAMPING_ONLY = 1,
       VFPS_FP_DIFFUSION_ONLY = 2, VFPS_FP_FULL = 3 };
enum { VFPS_DERIVATION_TWO_SIDED = 3, VFPS_DERIVATION_CUBIC = 4 };

typedef struct vfps_ctx vfps_ctx;
typedef struct vfps_ps vfps_ps;
typedef struct vfps_map vfps_map;
typedef struct vfps_impedance vfps_impedance;
typedef struct vfps_field vfps_field;
typedef struct vfps_batch vfps_batch;

/* ----------------------------------------------------------- context
 * Replaces the OpenCL handler (src/CL/OpenCLHandler.cpp:23-92): one device,
 * one in-order stream. */
VFPS_API int vfps_create(vfps_ctx** ctx, int device);
VFPS_API int vfps_destroy(vfps_ctx* ctx);
VFPS_API const char* vfps_last_error(const vfps_ctx* ctx);
/* OCLH::flush / finish: wait for all queued work of the context. */
VFPS_API int vfps_synchronize(vfps_ctx* ctx);
/* The context's cudaStream_t, for callers that order their own work. */
VFPS_API void* vfps_stream(vfps_ctx* ctx);
/* Device-side error word (bounded waits, watchdogs); 0 = none.  Reading it
 * synchronises; *code is cleared afterwards. */
VFPS_API int vfps_device_status(vfps_ctx* ctx, int* code);
/* No reference counterpart: exercises the failure path of the solver
 * kernels' bounded waits without faulting the GPU.  One CTA walks 16
 * tiles the way the persistent solver kernels do, each tile waiting on a
 * barrier that nothing completes: the first wait gives up after limit_ns
 * (at most 1 s), one more bounded wait follows, the CTA stops walking and
 * sets the device status to VFPS_ERR_TIMEOUT, so the call ends after about
 * 2 * limit_ns; the context stays usable (read and clear the status with
 * vfps_device_status). */
VFPS_API int vfps_selftest_wait_timeout(vfps_ctx* ctx, uint64_t limit_ns);
/* Pinned host buffers for asynchronous copies (no reference counterpart). */
VFPS_API int vfps_host_alloc(vfps_ctx* ctx, size_t bytes, void** ptr);
VFPS_API int vfps_host_free(vfps_ctx* ctx, void* ptr);

/* -------------------------------------------------------- PhaseSpace
 * PhaseSpace(qmin,qmax,qscale,pmin,pmax,pscale,oclh,charge,current,
 *            filling,zoom,data), inc/PS/PhaseSpace.hpp:79-91 and
 * src/PS/PhaseSpace.cpp:17-134.  axes = {qmin, qmax, qscale, pmin, pmax,
 * pscale}; qscale is the "Meter" and pscale the "ElectronVolt" scale.
 * filling[nb] must sum to 1 (else VFPS_ERR_INVALID_ARGUMENT).  data ==
 * NULL creates the normalised Gaussian of width zoom, otherwise nb*n*n
 * values are copied.  The static PhaseSpace::setSize(n, nb)
 * (src/PS/PhaseSpace.cpp:428-443) becomes per-object sizes. */
VFPS_API int vfps_ps_create(vfps_ctx* ctx, uint32_t nb, uint32_t n,
                            const double axes[6], double charge,
                            double current, const float* filling,
                            double zoom, const float* data, vfps_ps** ps);
/* copy constructor, src/PS/PhaseSpace.cpp:168-178 */
VFPS_API int vfps_ps_copy(const vfps_ps* src, vfps_ps** ps);
VFPS_API int vfps_ps_destroy(vfps_ps* ps);
/* PhaseSpace::swap / operator= (src/PS/PhaseSpace.cpp:374-378,503-506):
 * exchange or copy the density only. */
VFPS_API int vfps_ps_swap(vfps_ps* a, vfps_ps* b);
VFPS_API int vfps_ps_assign(vfps_ps* dst, const vfps_ps* src);
/* getData() with a device->host copy / writing the density back
 * (syncCLMem, src/PS/PhaseSpace.cpp:381-414). */
VFPS_API int vfps_ps_download(vfps_ps* ps, float* data);
VFPS_API int vfps_ps_upload(vfps_ps* ps, const float* data);
/* Device pointer of the density (nb*n*n floats), for zero-copy callers. */
VFPS_API float* vfps_ps_device_data(vfps_ps* ps);
/* sizes and the axis rulers (inc/PS/Ruler.hpp:31-51): values[n], delta,
 * zerobin of axis 0 (q) or 1 (p) */
VFPS_API int vfps_ps_shape(const vfps_ps* ps, uint32_t* nb, uint32_t* n);
VFPS_API int vfps_ps_axis(const vfps_ps* ps, int axis, float* values,
                          float* delta, float* zerobin);
/* updateXProjection / updateYProjection, src/PS/PhaseSpace.cpp:291-340
 * (sums accumulated in FP64 on the device) */
VFPS_API int vfps_ps_update_x_projection(vfps_ps* ps);
VFPS_API int vfps_ps_update_y_projection(vfps_ps* ps);
/* integrate / normalize / integrateAndNormalize,
 * src/PS/PhaseSpace.cpp:200-239,342-372, inc/PS/PhaseSpace.hpp:222-226
 * (FP64 on the device) */
VFPS_API int vfps_ps_integrate(vfps_ps* ps);
VFPS_API int vfps_ps_normalize(vfps_ps* ps);
VFPS_API int vfps_ps_integrate_and_normalize(vfps_ps* ps);
/* variance(axis) (src/PS/PhaseSpace.cpp:241-289): average and variance
 * from the current projection of that axis. */
VFPS_API int vfps_ps_variance(vfps_ps* ps, int axis);
/* getProjection(axis) -> proj[nb*n]; setProjection(axis, bunch, proj) */
VFPS_API int vfps_ps_get_projection(vfps_ps* ps, int axis, float* proj);
VFPS_API int vfps_ps_set_projection(vfps_ps* ps, int axis, uint32_t bunch,
                                    const float* proj);
/* getBunchPopulation(), getIntegral() */
VFPS_API int vfps_ps_get_filling(vfps_ps* ps, float* filling,
                                 double* integral);
/* getMoment(axis,0|1) and getBunchLength()/getEnergySpread() (rms) */
VFPS_API int vfps_ps_get_moments(vfps_ps* ps, int axis, float* average,
                                 float* variance, float* rms);

/* ---------------------------------------------------------- SourceMaps
 * Every map binds its input and output PhaseSpace at construction
 * (inc/SM/SourceMap.hpp:53-72) and is applied with vfps_map_apply
 * (SourceMap::apply(), inc/SM/SourceMap.hpp:79).  The interpolation
 * weights are evaluated on the device; no per-cell table is stored. */

/* RotationMap(in,out,xsize,ysize,angle,it,clamp,rotmapsize,oclh),
 * inc/SM/RotationMap.hpp:40-45.  rotmapsize is 0 or xsize*ysize; clamping
 * needs cubic interpolation and rotmapsize > 0. */
VFPS_API int vfps_rotation_map_create(vfps_ps* in, vfps_ps* out,
                                      uint32_t xsize, uint32_t ysize,
                                      float angle, int it, int clamp,
                                      uint32_t rotmapsize, vfps_map** map);
/* KickMap(in,out,it,clamp,axis,oclh), inc/SM/KickMap.hpp:34-38; the
 * offsets start at 0.  As in the reference's CPU path, the clamp flag of a
 * kick map is accepted and has no effect (src/SM/KickMap.cpp:42-44,
 * :194-271); DriftMap, RFKickMap and WakePotentialMap inherit this. */
VFPS_API int vfps_kick_map_create(vfps_ps* in, vfps_ps* out, int it,
                                  int clamp, int axis, vfps_map** map);
/* KickMap::swapOffset (inc/SM/KickMap.hpp:54-55): count = n (x-kick) or
 * nb*n (y-kick, one row of offsets per bunch) values in mesh units. */
VFPS_API int vfps_kick_map_set_offset(vfps_map* map, const float* offset,
                                      size_t count);
/* KickMap::getForce (inc/SM/KickMap.hpp:47-48) */
VFPS_API int vfps_kick_map_get_offset(vfps_map* map, float* offset,
                                      size_t count);
/* DriftMap(in,out,slip,E0,it,clamp,oclh), inc/SM/DriftMap.hpp:17-24 */
VFPS_API int vfps_drift_map_create(vfps_ps* in, vfps_ps* out,
                                   const float* slip, uint32_t nslip,
                                   float e0, int it, int clamp,
                                   vfps_map** map);
/* RFKickMap, linear RF (inc/SM/RFKickMap.hpp:17-23) */
VFPS_API int vfps_rf_kick_map_create_linear(vfps_ps* in, vfps_ps* out,
                                            float angle, float f_rf, int it,
                                            int clamp, vfps_map** map);
/* RFKickMap, sinusoidal RF (inc/SM/RFKickMap.hpp:26-34) */
VFPS_API int vfps_rf_kick_map_create(vfps_ps* in, vfps_ps* out,
                                     float revolutionpart, float v_rf,
                                     float f_rf, float v0, int it, int clamp,
                                     vfps_map** map);
/* DynamicRFKickMap (src/SM/DynamicRFKickMap.cpp:15-109): an RF kick map
 * whose phase and amplitude change at every apply, phase = syncphase +
 * N(0,1) phasespread/sqrt(revolutionpart) + modampl sin(2 pi
 * modtimeincrement i), amplitude = 1 + N(0,1) amplspread/sqrt(
 * revolutionpart) for apply number i; linear = 1 uses the linear RF
 * (angle), 0 the sinusoidal RF (v_rf, v0).  The normals come from a
 * counter-based generator (Philox-4x32-10 keyed by seed, Box-Muller), so a
 * run is reproducible (the reference seeds std::mt19937 from
 * std::random_device).  The first `steps` modulations are logged for
 * vfps_dynamic_rf_get_modulation (the reference's getPastModulation). */
VFPS_API int vfps_dynamic_rf_kick_map_create(
    vfps_ps* in, vfps_ps* out, int linear, float angle, float revolutionpart,
    float v_rf, float f_rf, float v0, float phasespread, float amplspread,
    float modampl, double modtimeincrement, uint32_t steps, int it,
    int clamp, uint32_t seed, vfps_map** map);
/* out[2*count] = (phase, amplitude) of the applies so far (at most the
 * logged `steps`); either pointer may be NULL. */
VFPS_API int vfps_dynamic_rf_get_modulation(vfps_map* map, float* out,
                                            uint64_t* count);
/* The generator of the dynamic RF map (no counterpart in the reference):
 * Philox-4x32-10 of counter[4] under key[2] into out[4]. */
VFPS_API int vfps_philox4x32(const uint32_t* counter, const uint32_t* key,
                             uint32_t* out);
/* FokkerPlanckMap(in,out,xsize,ysize,fptype,fptrack,e1,derivation,oclh),
 * inc/SM/FokkerPlanckMap.hpp:56-64 */
VFPS_API int vfps_fokker_planck_map_create(vfps_ps* in, vfps_ps* out,
                                           uint32_t xsize, uint32_t ysize,
                                           int fptype, int fptrack, float e1,
                                           int derivation, vfps_map** map);
/* Identity(in,out,oclh), inc/SM/Identity.hpp:29-34 */
VFPS_API int vfps_identity_map_create(vfps_ps* in, vfps_ps* out,
                                      vfps_map** map);
/* WakePotentialMap(in,out,field,it,clamp,oclh),
 * inc/SM/WakePotentialMap.hpp:20-26 */
VFPS_API int vfps_wake_potential_map_create(vfps_ps* in, vfps_ps* out,
                                            vfps_field* field, int it,
                                            int clamp, vfps_map** map);
/* WakeKickMap::update (inc/SM/WakeKickMap.hpp:38,
 * src/SM/WakePotentialMap.cpp:34-50): wake potential -> kick offsets. */
VFPS_API int vfps_wake_map_update(vfps_map* map);
/* SourceMap::apply() */
VFPS_API int vfps_map_apply(vfps_map* map);
/* SourceMap::applyToAll(particles) (src/SM/SourceMap.cpp:111-117):
 * pos = {x0, y0, x1, y1, ...} in mesh coordinates, updated in place on the
 * host (particle tracking is for display, as in the reference). */
VFPS_API int vfps_map_apply_to(vfps_map* map, float* pos, size_t count);
VFPS_API int vfps_map_destroy(vfps_map* map);

/* ---------------------------------------------------------- Impedance
 * Impedance (inc/Z/Impedance.hpp:29-113): a complex table of nfreqs
 * entries over [0, f_max].  Model tables are computed on the device in
 * FP64 and stored as complex float. */
VFPS_API int vfps_impedance_create(vfps_ctx* ctx, const float* z,
                                   size_t nfreqs, double f_max,
                                   vfps_impedance** imp);
/* FreeSpaceCSR(n,f_rev,f_max), src/Z/FreeSpaceCSR.cpp:10-43 */
VFPS_API int vfps_impedance_free_space_csr(vfps_ctx* ctx, size_t n,
                                           float f_rev, float f_max,
                                           vfps_impedance** imp);
/* ParallelPlatesCSR(n,f0,f_max,g), src/Z/ParallelPlatesCSR.cpp:12-70 */
VFPS_API int vfps_impedance_parallel_plates_csr(vfps_ctx* ctx, size_t n,
                                                float f0, float f_max,
                                                double g,
                                                vfps_impedance** imp);
/* ResistiveWall(n,f0,f_max,L,s,xi,b), src/Z/ResistiveWall.cpp:11-57 */
VFPS_API int vfps_impedance_resistive_wall(vfps_ctx* ctx, size_t n,
                                           float f0, float f_max, double L,
                                           double s, double xi, double b,
                                           vfps_impedance** imp);
/* ConstImpedance(n,f_max,Z), src/Z/ConstImpedance.cpp:10-28 */
VFPS_API int vfps_impedance_const(vfps_ctx* ctx, size_t n, float f_max,
                                  float re, float im, vfps_impedance** imp);
/* CollimatorImpedance(n,f_max,outer,inner),
 * src/Z/CollimatorImpedance.cpp:12-25 */
VFPS_API int vfps_impedance_collimator(vfps_ctx* ctx, size_t n, float f_max,
                                       double outer, double inner,
                                       vfps_impedance** imp);
/* Impedance(datafile,f_max), src/Z/Impedance.cpp:53-59,94-111 */
VFPS_API int vfps_impedance_from_file(vfps_ctx* ctx, const char* path,
                                      double f_max, vfps_impedance** imp);
/* makeImpedance (src/Z/ImpedanceFactory.cpp:21-84).  *imp is NULL when no
 * contribution is selected (the reference returns nullptr). */
VFPS_API int vfps_make_impedance(vfps_ctx* ctx, size_t nfreqs, float fmax,
                                 double r_bend, double frev, double gap,
                                 int use_csr, double s, double xi,
                                 double inner_coll_radius,
                                 const char* impedance_file,
                                 vfps_impedance** imp);
/* operator+= (src/Z/Impedance.cpp:67-76) and copy constructor */
VFPS_API int vfps_impedance_add(vfps_impedance* dst,
                                const vfps_impedance* rhs);
VFPS_API int vfps_impedance_copy(const vfps_impedance* src,
                                 vfps_impedance** imp);
VFPS_API int vfps_impedance_swap(vfps_impedance* a, vfps_impedance* b);
/* nFreqs(), data(), getRuler()->max() */
VFPS_API int vfps_impedance_get(const vfps_impedance* imp, float* z,
                                size_t* nfreqs, double* f_max);
VFPS_API int vfps_impedance_destroy(vfps_impedance* imp);

/* ------------------------------------------------------- ElectricField
 * ElectricField(ps,impedance,bucketnumbers,spacing_bins,oclh,f_rev,
 * revolutionpart,wakescaling), inc/PS/ElectricField.hpp:49-56.
 * buckets[nb] are the bucket numbers of the bunches of ps.  wakescaling 0
 * gives a field without wake potential. */
VFPS_API int vfps_field_create(vfps_ps* ps, const vfps_impedance* imp,
                               const uint32_t* buckets, uint32_t spacing_bins,
                               double f_rev, double revolutionpart,
                               double wakescaling, vfps_field** field);
/* The wake-potential constructor (inc/PS/ElectricField.hpp:81-103):
 * wakescaling = Ib dt c / qscale / (dp sigma_delta E0). */
VFPS_API int vfps_field_create_wake(vfps_ps* ps, const vfps_impedance* imp,
                                    const uint32_t* buckets,
                                    uint32_t spacing_bins, double f_rev,
                                    double revolutionpart, double ib,
                                    double e0, double sigma_delta, double dt,
                                    vfps_field** field);
/* padBunchProfiles (src/PS/ElectricField.cpp:255-263) and
 * getPaddedBunchProfiles(): padded[nmax] */
VFPS_API int vfps_field_pad_bunch_profiles(vfps_field* field);
VFPS_API int vfps_field_get_padded_profiles(vfps_field* field,
                                            float* padded);
/* wakePotential() (src/PS/ElectricField.cpp:186-253): from the phase
 * space's current x projection; result stays on the device. */
VFPS_API int vfps_field_wake_potential(vfps_field* field);
/* getWakePotentials(): wake[nb*n] */
VFPS_API int vfps_field_get_wake_potential(vfps_field* field, float* wake);
/* getWakeScaling() (wakescaling/nmax), getNMax() */
VFPS_API int vfps_field_info(const vfps_field* field, float* wakescale,
                             size_t* nmax);
/* updateCSR(fc) (src/PS/ElectricField.cpp:133-184). */
VFPS_API int vfps_field_update_csr(vfps_field* field, float fc);
/* getCSRSpectrum() spectrum[nb*nmax] and getCSRPower() power[nb]; either
 * may be NULL.  factor4Watts (inc/PS/ElectricField.hpp:203-208) converts
 * the power to W. */
VFPS_API int vfps_field_get_csr(vfps_field* field, float* spectrum,
                                float* power, double* factor4watts);
VFPS_API int vfps_field_destroy(vfps_field* field);

/* ------------------------------------------------------------ batches
 * No reference counterpart: many independent single-bunch simulations
 * (current scans, uneven grid sizes) stepped together by fused kernels
 * captured in a CUDA graph.  Each bunch follows the reference solver step
 * (src/main.cpp:948-1053 for chain 0, the rotation scheme of
 * test/TestRotationMap.cpp for chain 1). */
typedef struct {
    uint32_t n;            /* mesh side of this bunch */
    int32_t chain;         /* 0: wake, RF y-kick, drift x-kick, FP
                              1: rotation, wake y-kick, FP */
    int32_t it;            /* interpolation points (2, 3, 4) */
    int32_t clamp;         /* rotation clamp (chain 1, cubic) */
    double axes[6];        /* qmin, qmax, qscale, pmin, pmax, pscale */
    double zoom;           /* width of the initial Gaussian */
    double angle;          /* chain 1: rotation per step */
    int32_t rf_linear;     /* chain 0: 1 linear, 0 sinusoidal RF */
    double rf_angle;       /* linear RF: angle per step */
    double rf_revpart, rf_vrf, rf_v0, rf_bl2phase, rf_phase;
    double slip[3];        /* drift slip terms (src/main.cpp:663-664) */
    int32_t nslip;
    double e0;             /* beam energy (eV) */
    double e1;             /* FP decrement 2/(fs td steps); <= 0: none */
    int32_t fptype, derivation;
    double wakescaling;    /* ElectricField wakescaling; 0: no wake */
    int32_t renormalize;   /* >0 every n steps, 0 once, <0 never */
    int32_t impedance;     /* index into the impedance list of the batch */
} vfps_bunch_desc;

/* imps[nimp]: impedance tables shared by the bunches that name them;
 * each table's nfreqs must be >= 2 n of its bunches.  data == NULL starts
 * every bunch from its Gaussian. */
VFPS_API int vfps_batch_create(vfps_ctx* ctx, uint32_t nb,
                               const vfps_bunch_desc* desc,
                               const vfps_impedance* const* imps,
                               uint32_t nimp, const float* data,
                               vfps_batch** batch);
/* Advance every bunch by nsteps solver steps (device only). */
VFPS_API int vfps_batch_step(vfps_batch* batch, uint64_t nsteps);
/* End-to-end: densities from host memory in, nsteps steps, densities
 * (and optionally profiles [total cells of all profiles] and fillings
 * [nb]) back to host memory.  Either input or output may be NULL. */
VFPS_API int vfps_batch_run(vfps_batch* batch, const float* density_in,
                            uint64_t nsteps, float* density_out,
                            float* profiles_out, float* filling_out);
/* Offsets of bunch b in the packed density/profile arrays. */
VFPS_API int vfps_batch_layout(const vfps_batch* batch, uint32_t b,
                               size_t* density_offset, size_t* profile_offset);
VFPS_API int vfps_batch_download(vfps_batch* batch, float* density);
VFPS_API int vfps_batch_upload(vfps_batch* batch, const float* density);
VFPS_API int vfps_batch_get_profiles(vfps_batch* batch, float* profiles);
VFPS_API int vfps_batch_get_filling(vfps_batch* batch, double* filling);
VFPS_API int vfps_batch_get_wake(vfps_batch* batch, float* wake);
/* Multi-bunch beams (src/main.cpp:248-321, src/PS/ElectricField.cpp:
 * 255-263): bunches with the same beam[i] > 0 share one padded profile,
 * bunch i at bucket[i] * spacing_bins, so each one's wake carries the
 * other members' fields (circular in the impedance's nfreqs, like the
 * reference's FFT); beam[i] == 0 leaves bunch i alone.  Members must share
 * mesh size, impedance and wake scaling (that of the beam's total
 * current).  filling[nb] (optional): each bunch's share of the charge
 * (the reference's filling_set); the current densities are normalised to
 * it.  The tensor-core wake (vfps_batch_set_wake_mode 1) has no coupling
 * and is switched off; the potential-well start uses each bunch's own
 * field only. */
VFPS_API int vfps_batch_set_beams(vfps_batch* batch, const uint32_t* beam,
                                  const uint32_t* bucket,
                                  uint32_t spacing_bins, const float* filling);
/* CSR power of every bunch at recording steps (updateCSR,
 * src/PS/ElectricField.cpp:133-184): the radiated power of the bunch's
 * profile at the start of a step, the reference's sum over the half
 * spectrum of the padded profile (its own impedance, cutoff and frequency
 * axis), computed as the quadratic form of the profile with a Toeplitz
 * kernel built once in FP64.  impedance[nb] indexes imps[nimp] (-1: no
 * CSR for that bunch); fc[nb] the cutoff frequency (<= 0: none);
 * freq_scale[nb] the "Hertz" scale of the frequency ruler (c / bunch
 * length).  Steps with step % every == 0 are recorded into a ring of
 * `capacity` slots; every == 0 switches recording off. */
VFPS_API int vfps_batch_set_csr(vfps_batch* batch,
                                const vfps_impedance* const* imps,
                                uint32_t nimp, const int32_t* impedance,
                                const double* fc, const double* freq_scale,
                                uint32_t every, uint32_t capacity);
/* The ring: power[capacity][nb] and steps[capacity], the step each slot
 * holds (UINT64_MAX: not written yet). */
VFPS_API int vfps_batch_get_csr(vfps_batch* batch, float* power,
                                uint64_t* steps);
/* Replace the density of every bunch with the stationary state of its
 * solver step below the instability threshold, and refresh profiles
 * and filling (as vfps_batch_upload does).  The reference names this
 * start only as an ignored option (HaissinskiIterations,
 * src/IO/ProgramOptions.cpp:270); here it is the Haissinski potential
 * well of the wake and RF kicks, written as a function of the invariant
 * of the discrete step (kick, then drift):
 *   density(x, y) ~ exp(-(Phi(x) + G(y) + F(x) d(y) / 2) / T),
 * F = -(rf + wake) the y-kick of row x, Phi its integral, d the drift
 * offset of column y, G its integral, T = slip0 / (dq dp).  The wake
 * depends on the profile: `iterations` fixed-point passes, each mixing
 * `mix` (0 < mix <= 1) of the new profile into the old.  Members of a
 * multi-bunch beam (vfps_batch_set_beams) iterate together: each pass
 * sums, in every member's wake, the fields of all members' profiles of
 * the previous pass at their bucket distances.  For the rotation chain
 * (chain 1), rf and d are the linear kick and drift of the rotation's
 * angle and only the wake kick enters the cross term, with the opposite
 * sign: E = Phi + G + wake(x) d(y) / 2.  change[nb] (optional) receives
 * the last relative L1 change of each profile (0 for bunches without a
 * wake). */
VFPS_API int vfps_batch_potential_well(vfps_batch* batch, uint32_t iterations,
                                       float mix, float* change);
/* kernel launches per solver step (for launch accounting) */
VFPS_API int vfps_batch_info(const vfps_batch* batch, uint32_t* launches,
                             uint32_t* tile_rows);
/* No reference counterpart.  Tiles each maps kernel of the batched step
 * walks, in the order: the fast chain-0 ring kernel (meshes up to 256 rows
 * with the regular lattice form), the chain-0 ring kernel for the other
 * meshes up to 256 rows, the 512-row ring kernel, the 1024-row kernel, the
 * rotation chain's kernel; tiles[count] receives the first count. */
VFPS_API int vfps_batch_kernel_tiles(const vfps_batch* batch, uint32_t* tiles,
                                     uint32_t count);
/* Advance every bunch by nsteps solver steps launched one kernel at a time
 * with CUDA events between the kernels, and return the mean duration per
 * step of each kernel in ms[3] (wake, chain-0 maps, chain-1 maps; 0 for a
 * chain the batch does not hold).  Profiling aid (no counterpart in the
 * reference): the state advances exactly as with vfps_batch_step. */
VFPS_API int vfps_batch_kernel_times(vfps_batch* batch, uint32_t nsteps,
                                     float* ms);

/* Where the batch computes the wake potentials (no counterpart in the
 * reference): mode 0 (default) on the CUDA cores inside the per-bunch wake
 * kernel; mode 1 as one Toeplitz x profiles product per group of bunches
 * sharing an impedance and mesh size, on the tensor cores (TF32 split into
 * three products, FP32 accumulation: FP32-level accuracy). */
VFPS_API int vfps_batch_set_wake_mode(vfps_batch* batch, int mode);

/* ---------------------------------------------------- learned warm start
 * No counterpart in the reference.  A small network proposes the
 * equilibrium density of a bunch from (normalised current, gap ratio,
 * damping time); the proposal enters through vfps_batch_upload (the
 * PhaseSpace data argument of the reference), and the solver judges it.
 *   h1 = tanh(W1 x + b1), h2 = tanh(W2 h1 + b2), z = W3 h2 + b3,
 *   y  = bd + sum_k z_k Wd[k]   (a transposed convolution from a 1x1 map
 *                                of nlat channels to the npix cells)
 * In a network the w* point to BF16 weights [out][in] (Wd [nlat][npix]);
 * in a gradient they point to FP32 arrays of the same shapes.  All
 * buffers are device memory owned by the caller; nlat must be 32. */
typedef struct vfps_ws_net {
    uint32_t nin, nh, nlat, npix;
    const void* w1;
    const float* b1;
    const void* w2;
    const float* b2;
    const void* w3;
    const float* b3;
    const void* wd;
    const float* bd;
} vfps_ws_net;
/* Forward pass of B samples x[B][nin]: keeps h1, h2 [B][nh] and z
 * [B][nlat] for the backward pass, writes y [B][npix] if y != NULL.  With
 * a target [B][npix]: also g = dL/dy of L = sum (y - t)^2 / (B npix), and
 * partial sums of (y - t)^2 in lpart[nparts] (add them up for the loss). */
VFPS_API int vfps_ws_forward(vfps_ctx* ctx, const vfps_ws_net* net,
                             const float* x, uint32_t B, float* h1,
                             float* h2, float* z, float* y,
                             const float* target, float* g, double* lpart,
                             uint32_t nparts);
/* Backward pass from g = dL/dy: all weight and bias gradients into grad
 * (FP32), with dz [B][nlat], d1, d2 [B][nh] as workspace. */
VFPS_API int vfps_ws_backward(vfps_ctx* ctx, const vfps_ws_net* net,
                              const vfps_ws_net* grad, const float* x,
                              uint32_t B, const float* h1, const float* h2,
                              const float* z, const float* g, float* dz,
                              float* d1, float* d2);
/* One Adam step (bias-corrected, step >= 1) on FP32 weights w with
 * moments m, v; writes the BF16 copy w_bf16 when it is not NULL. */
VFPS_API int vfps_ws_adam(vfps_ctx* ctx, float* w, const float* g, float* m,
                          float* v, void* w_bf16, size_t count, float lr,
                          float beta1, float beta2, float eps, uint32_t step);

/* ------------------------------------------------- no-allocation helper
 * No counterpart in the reference.  Charge integral of nb meshes [n][n]
 * that the caller already holds in device memory (density = device
 * pointer, e.g. vfps_ps_device_data): the Simpson x projection of every
 * row and its Simpson integral for mesh spacing delta (the q axis of the
 * mesh), the same numbers vfps_ps_update_x_projection followed by
 * vfps_ps_integrate give.  integrals[nb] is host memory; the call returns
 * after the results are there.
 *
 * It allocates nothing, for callers that may not allocate device memory
 * at that point: a program that reserved its whole device budget up front
 * and passes raw pointers into it, a pool allocator that must stay the
 * only owner of free device memory, or a time-critical loop that cannot
 * take the device-wide synchronisation cudaMalloc/cudaFree may cause.
 * Its scratch is one fixed __device__ array per device: at most 262144
 * rows (nb * n) and 4096 meshes per call, larger calls are rejected with
 * VFPS_ERR_INVALID_ARGUMENT.  The first call on a device looks up the
 * scratch address once and should come before any stream capture starts;
 * the address is tied to the device's context, so the first call after a
 * device reset (cudaDeviceReset by the host program or a library) looks it
 * up again and is a set-up call as well.  The call restores the calling
 * thread's current device before it returns.  Nothing in the scratch
 * needs to start at zero.  Calls on one device must not overlap in time
 * (from several host threads, or several contexts on one device): they
 * share the scratch and would race on it. */
VFPS_API int vfps_charge_noalloc(vfps_ctx* ctx, const float* density,
                                 uint32_t nb, uint32_t n, float delta,
                                 double* integrals);
VFPS_API int vfps_batch_destroy(vfps_batch* batch);

#ifdef __cplusplus
}
#endif
#endif /* VFPS_H */
