/* ax3d.hpp -- C++ host interface over the ax3d C-ABI (header only, C++17).
 *
 * ax3d::Domain mirrors the reference's Domain (SOLVER/src/core/domain/Domain.h:25-118):
 * the same loop bodies under the same names (updateNewmark, applySource, computeStiff,
 * coupleSolidFluid, record) and Newmark::solve's loop as solve(n), with errors raised as
 * std::runtime_error subclasses carrying the library's "Class::method || msg" text, the
 * way the reference throws.  The set-up calls take the packed arrays of include/ax3d.h;
 * the object owns the handle (ax3d_destroy on destruction) and is movable, not copyable.
 */
#pragma once

#include <complex>
#include <cstdint>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "ax3d.h"

namespace ax3d {

class Error : public std::runtime_error {
  public:
    Error(int code, const std::string &what) : std::runtime_error(what), code_(code) {}
    int code() const { return code_; }

  private:
    int code_;
};

inline void check(int rc) {
    if (rc == AX3D_OK) return;
    char buf[1024];
    ax3d_last_error(buf, sizeof buf);
    throw Error(rc, buf);
}

class Domain {
  public:
    explicit Domain(const ax3d_config &cfg) { check(ax3d_create(&cfg, &d_)); }
    ~Domain() {
        if (d_) ax3d_destroy(d_);
    }
    Domain(const Domain &) = delete;
    Domain &operator=(const Domain &) = delete;
    Domain(Domain &&o) noexcept : d_(std::exchange(o.d_, nullptr)) {}
    Domain &operator=(Domain &&o) noexcept {
        if (this != &o) {
            if (d_) ax3d_destroy(d_);
            d_ = std::exchange(o.d_, nullptr);
        }
        return *this;
    }
    ax3d_domain *handle() const { return d_; }

    // ---- set-up (Domain::addPoint / addElement / addSourceTerm / setSTF, recorders) ----
    int32_t addPoints(int32_t n, const int32_t *nr, const int8_t *kind, const uint8_t *axial,
                      const uint8_t *fluid_surface, const int32_t *ms_len, const float *ms_inv,
                      const int32_t *mf_len, const float *mf_inv, const int32_t *sf_len, const float *sf_normal,
                      const float *sf_normal_invmf) {
        int32_t first = -1;
        check(ax3d_add_points(d_, n, nr, kind, axial, fluid_surface, ms_len, ms_inv, mf_len, mf_inv, sf_len,
                              sf_normal, sf_normal_invmf, &first));
        return first;
    }
    int32_t addElements(int32_t n, const int32_t *points, const int8_t *material, const uint8_t *axial,
                        const uint8_t *in_3d, const float *geometry, const float *trig, const int64_t *moduli_ofs,
                        const float *moduli, const int8_t *att, const int64_t *att_ofs, const float *att_moduli) {
        int32_t first = -1;
        check(ax3d_add_elements(d_, n, points, material, axial, in_3d, geometry, trig, moduli_ofs, moduli, att,
                                att_ofs, att_moduli, &first));
        return first;
    }
    // force [25][norders][3] complex
    void addSourceTerm(int32_t elem, int32_t norders, const std::complex<float> *force) {
        check(ax3d_add_source(d_, elem, norders, reinterpret_cast<const float *>(force)));
    }
    void setSTF(const std::vector<float> &stf) { check(ax3d_set_stf(d_, (int32_t)stf.size(), stf.data())); }
    void addReceivers(int32_t n, const int32_t *elem, const float *phi, const float *weights) {
        check(ax3d_add_receivers(d_, n, elem, phi, weights));
    }
    void setReceiverDumps(int32_t n, const int32_t *flags) { check(ax3d_set_receiver_dumps(d_, n, flags)); }
    void addSurface(int32_t n, const int32_t *elem, const int32_t *side, int32_t interval) {
        check(ax3d_add_surface(d_, n, elem, side, interval));
    }
    void addOceanLoad(int32_t n, const int32_t *point, const int32_t *len, const float *vals) {
        check(ax3d_add_ocean_load(d_, n, point, len, vals));
    }
    void setPRT(int32_t n, const int32_t *elem, const int32_t *len, const float *x) {
        check(ax3d_set_prt(d_, n, elem, len, x));
    }
    void finalize() { check(ax3d_finalize(d_)); }

    // ---- the loop bodies (Domain.cpp:82-191) and Newmark::solve (Newmark.cpp:47-93) ----
    void updateNewmark() { check(ax3d_update_newmark(d_)); }
    void applySource(int32_t tstep) { check(ax3d_apply_source(d_, tstep)); }
    void computeStiff() { check(ax3d_compute_stiff(d_)); }
    void coupleSolidFluid() { check(ax3d_couple_solid_fluid(d_)); }
    void record(int32_t tstep) { check(ax3d_record(d_, tstep)); }
    void solve(int32_t nsteps) { check(ax3d_step(d_, nsteps)); }
    void resetZero() { check(ax3d_reset(d_)); }
    int32_t currentStep() const { return ax3d_current_step(d_); }

    // ---- fields and records ----
    int64_t fieldSize(int32_t phase) const { return ax3d_field_size(d_, phase); }
    std::vector<std::complex<float>> getField(int32_t which, int32_t phase) const {
        std::vector<std::complex<float>> v((size_t)fieldSize(phase));
        check(ax3d_get_field(d_, which, phase, reinterpret_cast<float *>(v.data())));
        return v;
    }
    void setField(int32_t which, int32_t phase, const std::vector<std::complex<float>> &v) {
        if ((int64_t)v.size() != fieldSize(phase)) throw Error(AX3D_ERR_ARG, "ax3d::Domain::setField || size");
        check(ax3d_set_field(d_, which, phase, reinterpret_cast<const float *>(v.data())));
    }
    // [nsteps][receivers][3] (s, phi, z)
    std::vector<float> seismograms(int32_t first, int32_t nsteps, int32_t nreceivers) const {
        std::vector<float> out((size_t)nsteps * nreceivers * 3);
        check(ax3d_read_seismograms(d_, first, nsteps, out.data()));
        return out;
    }
    // streamed transfers (host buffers pinned, untouched until syncFields)
    void setFieldAsync(int32_t which, int32_t phase, const std::complex<float> *in) {
        check(ax3d_set_field_async(d_, which, phase, reinterpret_cast<const float *>(in)));
    }
    void getFieldAsync(int32_t which, int32_t phase, std::complex<float> *out) {
        check(ax3d_get_field_async(d_, which, phase, reinterpret_cast<float *>(out)));
    }
    void syncFields() { check(ax3d_sync_fields(d_)); }

  private:
    ax3d_domain *d_ = nullptr;
};

}  // namespace ax3d
