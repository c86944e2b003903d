// ax3d_oracle_capi.cpp -- C entry points of the CPU oracle (TEST INFRASTRUCTURE ONLY).
//
// Mirrors include/ax3d.h with the prefixes axo_ (Real = float, the reference's default
// build) and axod_ (Real = double, the FP64 oracle).  Only tests, smoke() and the
// cpu_baseline leg of bench.py load this library.
#include <cstring>
#include <string>

#include "../include/ax3d.h"
#include "ax3d_oracle.hpp"
#include "ax3d_oracle_preloop.hpp"

namespace {
thread_local std::string g_err;
template <typename F>
int guard(F f) {
    try {
        return f();
    } catch (const std::exception &e) {
        g_err = e.what();
        return AX3D_ERR_ARG;
    }
}
}  // namespace

#define AXO_DEFINE(P, REAL)                                                                      \
    extern "C" {                                                                                 \
    typedef axo::Oracle<REAL> P##dom;                                                            \
    int P##create(const ax3d_config *c, void **out) {                                            \
        return guard([&] {                                                                       \
            if (!c || c->npol != 4) throw std::runtime_error("create || npol must be 4");        \
            auto *d = new P##dom();                                                              \
            d->config(c->dt, c->g_gll, c->g_glj, c->nsls, c->att_alpha, c->att_beta,             \
                      c->att_gamma, c->att_do_kappa != 0, c->kahan != 0, c->stability_interval); \
            *out = d;                                                                            \
            return 0;                                                                            \
        });                                                                                      \
    }                                                                                            \
    int P##add_points(void *d, int32_t n, const int32_t *nr, const int8_t *kind,                 \
                      const uint8_t *axial, const uint8_t *fs, const int32_t *msl,               \
                      const float *ms, const int32_t *mfl, const float *mf, const int32_t *sfl, \
                      const float *sfn, const float *sfni) {                                     \
        return guard([&] {                                                                       \
            static_cast<P##dom *>(d)->add_points(n, nr, kind, axial, fs, msl, ms, mfl, mf, sfl, \
                                                 sfn, sfni);                                     \
            return 0;                                                                            \
        });                                                                                      \
    }                                                                                            \
    int P##add_elements(void *d, int32_t n, const int32_t *pts, const int8_t *mat,               \
                        const uint8_t *ax, const uint8_t *in3d, const float *geo,                \
                        const float *trig, const int64_t *mofs, const float *mod,                \
                        const int8_t *att, const int64_t *aofs, const float *attm) {             \
        return guard([&] {                                                                       \
            static_cast<P##dom *>(d)->add_elements(n, pts, mat, ax, in3d, geo, trig, mofs, mod, \
                                                   att, aofs, attm);                             \
            return 0;                                                                            \
        });                                                                                      \
    }                                                                                            \
    int P##add_source(void *dv, int32_t elem, int32_t nord, const float *force) {                \
        return guard([&] {                                                                       \
            auto *d = static_cast<P##dom *>(dv);                                                 \
            if (elem < 0 || elem >= (int)d->elems.size())                                        \
                throw std::runtime_error("add_source || element out of range");                  \
            typename P##dom::Source s;                                                           \
            s.elem = elem;                                                                       \
            s.nord = nord;                                                                       \
            s.force.resize((size_t)25 * nord * 3);                                               \
            for (size_t i = 0; i < s.force.size(); i++)                                          \
                s.force[i] = std::complex<REAL>(force[2 * i], force[2 * i + 1]);                 \
            d->srcs.push_back(s);                                                                \
            return 0;                                                                            \
        });                                                                                      \
    }                                                                                            \
    int P##set_stf(void *dv, int32_t n, const float *stf) {                                      \
        auto *d = static_cast<P##dom *>(dv);                                                     \
        d->stf.assign(stf, stf + n);                                                             \
        return 0;                                                                                \
    }                                                                                            \
    int P##add_receivers(void *dv, int32_t n, const int32_t *elem, const float *phi,             \
                         const float *w) {                                                       \
        auto *d = static_cast<P##dom *>(dv);                                                     \
        for (int i = 0; i < n; i++) {                                                            \
            typename P##dom::Rec r;                                                              \
            r.elem = elem[i];                                                                    \
            r.phi = phi[i];                                                                      \
            for (int p = 0; p < 25; p++) r.w[p] = w[i * 25 + p];                                 \
            d->recs.push_back(r);                                                                \
        }                                                                                        \
        return 0;                                                                                \
    }                                                                                            \
    int P##add_ocean_load(void *dv, int32_t n, const int32_t *point, const int32_t *len,         \
                          const float *vals) {                                                   \
        return guard([&] {                                                                       \
            static_cast<P##dom *>(dv)->add_ocean_load(n, point, len, vals);                      \
            return 0;                                                                            \
        });                                                                                      \
    }                                                                                            \
    int P##add_surface(void *dv, int32_t n, const int32_t *elem, const int32_t *side,            \
                       int32_t interval) {                                                       \
        auto *d = static_cast<P##dom *>(dv);                                                     \
        if (interval < 1) return AX3D_ERR_ARG;                                                   \
        d->sf_interval = interval;                                                               \
        d->sf_elem.insert(d->sf_elem.end(), elem, elem + n);                                     \
        d->sf_side.insert(d->sf_side.end(), side, side + n);                                     \
        return 0;                                                                                \
    }                                                                                            \
    int64_t P##surface_record_size(void *d) {                                                    \
        return static_cast<P##dom *>(d)->surface_record_size();                                  \
    }                                                                                            \
    int P##read_surface(void *dv, int32_t first, int32_t n, double *out) {                       \
        auto *d = static_cast<P##dom *>(dv);                                                     \
        const size_t row = (size_t)d->surface_record_size();                                     \
        if (first < 0 || d->surf.size() < (size_t)(first + n) * row) return AX3D_ERR_ARG;        \
        for (size_t i = 0; i < (size_t)n * row; i++) {                                           \
            out[2 * i] = (double)d->surf[(size_t)first * row + i].real();                        \
            out[2 * i + 1] = (double)d->surf[(size_t)first * row + i].imag();                    \
        }                                                                                        \
        return 0;                                                                                \
    }                                                                                            \
    int P##finalize(void *d) {                                                                   \
        return guard([&] {                                                                       \
            static_cast<P##dom *>(d)->finalize();                                                \
            return 0;                                                                            \
        });                                                                                      \
    }                                                                                            \
    int64_t P##field_size(void *dv, int32_t phase) {                                             \
        auto *d = static_cast<P##dom *>(dv);                                                     \
        return phase == 0 ? (int64_t)d->su.size() : (int64_t)d->fu.size();                       \
    }                                                                                            \
    static std::vector<std::complex<REAL>> *P##pick(P##dom *d, int which, int phase) {           \
        if (phase == 0) {                                                                        \
            switch (which) {                                                                     \
                case 0: return &d->su;                                                           \
                case 1: return &d->sv;                                                           \
                case 2: return &d->sa;                                                           \
                case 3: return &d->ss;                                                           \
            }                                                                                    \
        } else {                                                                                 \
            switch (which) {                                                                     \
                case 0: return &d->fu;                                                           \
                case 1: return &d->fv;                                                           \
                case 2: return &d->fa;                                                           \
                case 3: return &d->fs;                                                           \
            }                                                                                    \
        }                                                                                        \
        return nullptr;                                                                          \
    }                                                                                            \
    int P##get_field(void *dv, int32_t which, int32_t phase, double *out) {                      \
        auto *v = P##pick(static_cast<P##dom *>(dv), which, phase);                              \
        if (!v) return AX3D_ERR_ARG;                                                             \
        for (size_t i = 0; i < v->size(); i++) {                                                 \
            out[2 * i] = (double)(*v)[i].real();                                                 \
            out[2 * i + 1] = (double)(*v)[i].imag();                                             \
        }                                                                                        \
        return 0;                                                                                \
    }                                                                                            \
    int P##set_field(void *dv, int32_t which, int32_t phase, const double *in) {                 \
        auto *v = P##pick(static_cast<P##dom *>(dv), which, phase);                              \
        if (!v) return AX3D_ERR_ARG;                                                             \
        for (size_t i = 0; i < v->size(); i++)                                                   \
            (*v)[i] = std::complex<REAL>((REAL)in[2 * i], (REAL)in[2 * i + 1]);                  \
        return 0;                                                                                \
    }                                                                                            \
    int P##set_field_async(void *dv, int32_t which, int32_t phase, const double *in) {           \
        auto *d = static_cast<P##dom *>(dv);                                                     \
        auto *v = P##pick(d, which, phase);                                                      \
        if (!v || d->queued.size() >= 2) return AX3D_ERR_ARG;                                    \
        std::vector<std::complex<REAL>> c(v->size());                                            \
        for (size_t i = 0; i < v->size(); i++)                                                   \
            c[i] = std::complex<REAL>((REAL)in[2 * i], (REAL)in[2 * i + 1]);                     \
        d->queued.emplace_back(v, std::move(c));                                                 \
        return 0;                                                                                \
    }                                                                                            \
    int P##get_field_async(void *dv, int32_t which, int32_t phase, double *out) {                \
        return P##get_field(dv, which, phase, out);                                              \
    }                                                                                            \
    int P##sync_fields(void *) { return 0; }                                                     \
    int P##update_newmark(void *d) {                                                             \
        return guard([&] {                                                                       \
            static_cast<P##dom *>(d)->update_newmark();                                          \
            return 0;                                                                            \
        });                                                                                      \
    }                                                                                            \
    int P##apply_source(void *d, int32_t t) {                                                    \
        return guard([&] {                                                                       \
            static_cast<P##dom *>(d)->apply_source(t);                                           \
            return 0;                                                                            \
        });                                                                                      \
    }                                                                                            \
    int P##compute_stiff(void *d) {                                                              \
        return guard([&] {                                                                       \
            static_cast<P##dom *>(d)->compute_stiff();                                           \
            return 0;                                                                            \
        });                                                                                      \
    }                                                                                            \
    int P##couple_solid_fluid(void *d) {                                                         \
        return guard([&] {                                                                       \
            static_cast<P##dom *>(d)->couple_solid_fluid();                                      \
            return 0;                                                                            \
        });                                                                                      \
    }                                                                                            \
    int P##record(void *d, int32_t t) {                                                          \
        return guard([&] {                                                                       \
            static_cast<P##dom *>(d)->record(t);                                                 \
            return 0;                                                                            \
        });                                                                                      \
    }                                                                                            \
    int P##step(void *d, int32_t n) {                                                            \
        return guard([&] { return static_cast<P##dom *>(d)->step(n); });                         \
    }                                                                                            \
    int P##read_seismograms(void *dv, int32_t first, int32_t n, double *out) {                   \
        auto *d = static_cast<P##dom *>(dv);                                                     \
        size_t nrec = d->recs.size();                                                            \
        size_t need = (size_t)(first + n) * nrec * 3;                                            \
        if (first < 0 || d->seis.size() < need) return AX3D_ERR_ARG;                             \
        for (size_t i = 0; i < (size_t)n * nrec * 3; i++)                                        \
            out[i] = (double)d->seis[(size_t)first * nrec * 3 + i];                              \
        return 0;                                                                                \
    }                                                                                            \
    int P##set_prt(void *dv, int32_t n, const int32_t *elem, const int32_t *len, const float *x) { \
        return guard([&] {                                                                       \
            static_cast<P##dom *>(dv)->set_prt(n, elem, len, x);                                 \
            return 0;                                                                            \
        });                                                                                      \
    }                                                                                            \
    int P##set_receiver_dumps(void *dv, int32_t n, const int32_t *flags) {                       \
        return guard([&] {                                                                       \
            static_cast<P##dom *>(dv)->set_receiver_dumps(n, flags);                             \
            return 0;                                                                            \
        });                                                                                      \
    }                                                                                            \
    int P##read_strain_curl(void *dv, int32_t which, int32_t first, int32_t n, double *out) {    \
        auto *d = static_cast<P##dom *>(dv);                                                     \
        const auto &v = which == 0 ? d->strain_rec : d->curl_rec;                                \
        size_t row = which == 0 ? (size_t)d->n_strain * 6 : (size_t)d->n_curl * 3;               \
        if (first < 0 || v.size() < (size_t)(first + n) * row) return AX3D_ERR_ARG;              \
        for (size_t i = 0; i < (size_t)n * row; i++) out[i] = (double)v[(size_t)first * row + i]; \
        return 0;                                                                                \
    }                                                                                            \
    int P##reset(void *d) {                                                                      \
        static_cast<P##dom *>(d)->reset();                                                       \
        return 0;                                                                                \
    }                                                                                            \
    int32_t P##current_step(void *d) { return static_cast<P##dom *>(d)->tstep; }                 \
    int P##set_wisdom_learning(void *dv, int32_t interval, float cutoff) {                       \
        auto *d = static_cast<P##dom *>(dv);                                                     \
        d->wis_interval = interval > 0 ? interval : 0;                                           \
        d->wis_cutoff = (REAL)cutoff;                                                            \
        return 0;                                                                                \
    }                                                                                            \
    int P##learn_wisdom(void *d, float cutoff) {                                                 \
        static_cast<P##dom *>(d)->learn_wisdom((REAL)cutoff);                                    \
        return 0;                                                                                \
    }                                                                                            \
    int P##get_wisdom(void *d, int32_t *out) {                                                   \
        auto v = static_cast<P##dom *>(d)->get_wisdom();                                         \
        std::copy(v.begin(), v.end(), out);                                                      \
        return 0;                                                                                \
    }                                                                                            \
    int P##destroy(void *d) {                                                                    \
        delete static_cast<P##dom *>(d);                                                         \
        return 0;                                                                                \
    }                                                                                            \
    }

AXO_DEFINE(axo_, float)
AXO_DEFINE(axod_, double)

extern "C" size_t axo_last_error(char *buf, size_t len) {
    if (buf && len) {
        size_t n = std::min(len - 1, g_err.size());
        std::memcpy(buf, g_err.data(), n);
        buf[n] = 0;
    }
    return g_err.size();
}

// ---- FP64 pre-loop (ax3d_oracle_preloop.hpp), the checker of ax3d_precompute_* ----
extern "C" int axo_pre_geometry(int32_t n, const double *nodes, const int8_t *etype, const int8_t *co,
                                const uint8_t *axial, const double *spectral, double *geo, double *ifact,
                                double *crds) {
    axo_pre::Spectral S;
    for (int i = 0; i < 5; i++) {
        S.xg[i] = spectral[i];
        S.wg[i] = spectral[5 + i];
        S.xj[i] = spectral[10 + i];
        S.wj[i] = spectral[15 + i];
    }
    for (int e = 0; e < n; e++) {
        double nd[2][4];
        for (int r = 0; r < 2; r++)
            for (int k = 0; k < 4; k++) nd[r][k] = nodes[(int64_t)e * 8 + r * 4 + k];
        axo_pre::quad_geometry(nd, etype[e], co[e], axial[e] != 0, S,
                               reinterpret_cast<double(*)[25]>(geo + (int64_t)e * 125), ifact + (int64_t)e * 25,
                               reinterpret_cast<double(*)[2]>(crds + (int64_t)e * 50));
    }
    return 0;
}

extern "C" int axo_pre_mass(int32_t n, const int32_t *rows, const double *ifact, const double *rho,
                            const double *vp, const uint8_t *fluid, double *mass) {
    int64_t o = 0;
    for (int e = 0; e < n; e++) {
        axo_pre::elemental_mass(rows[e], ifact + (int64_t)e * 25, rho + o, vp ? vp + o : nullptr, fluid[e] != 0,
                                mass + o);
        o += (int64_t)rows[e] * 25;
    }
    return 0;
}

// model values [8][rows][25] per element back to back (vpv, vph, vsv, vsh, eta, rho, qkappa,
// qmu); out moduli [k][rows][25] and att [2][rows][npa] per element back to back
extern "C" int axo_pre_elastic(int32_t n, const int32_t *rows, const double *ifact, const double *model,
                               int32_t iso, int32_t att, int32_t nsls, const double *w, const double *y,
                               double f_min, double f_max, double f_ref, int32_t do_kappa, double *mod,
                               double *attm) {
    axo_pre::AttFit fit{nsls, std::vector<double>(w, w + (att ? nsls : 0)),
                        std::vector<double>(y, y + (att ? nsls : 0)), f_min, f_max, f_ref, do_kappa != 0};
    int64_t mi = 0, mo = 0, ao = 0;
    const int km = iso ? 2 : 5, npa = att == 2 ? 4 : 25;
    for (int e = 0; e < n; e++) {
        const int64_t nv = (int64_t)rows[e] * 25;
        const double *m = model + mi;
        axo_pre::create_elastic(rows[e], ifact + (int64_t)e * 25, m, m + nv, m + 2 * nv, m + 3 * nv, m + 4 * nv,
                                m + 5 * nv, m + 6 * nv, m + 7 * nv, iso != 0, att, &fit, mod + mo,
                                att ? attm + ao : nullptr);
        mi += 8 * nv;
        mo += km * nv;
        ao += att ? 2 * (int64_t)rows[e] * npa : 0;
    }
    return 0;
}

#ifdef AX3D_ORACLE_FFT
// The CPU baseline's transforms alone, for the test that checks them against the exact
// DFT: two Hermitian columns (orders 0..nr/2, interleaved complex float) to two real
// columns of nr samples, and back (x 1/nr).
extern "C" int axf_c2r_pair(int32_t nr, const float *X1, const float *X2, float *x1, float *x2) {
    axfft::c2r_pair(reinterpret_cast<const axfft::cf *>(X1), reinterpret_cast<const axfft::cf *>(X2), 1, nr, x1, x2);
    return 0;
}
extern "C" int axf_r2c_pair(int32_t nr, const float *x1, const float *x2, float *X1, float *X2) {
    axfft::r2c_pair(x1, x2, nr, reinterpret_cast<axfft::cf *>(X1), reinterpret_cast<axfft::cf *>(X2), 1);
    return 0;
}
#endif
