// ax3d_oracle_preloop.hpp -- FP64 restatement of the reference's one-time pre-loop
// arithmetic (TEST INFRASTRUCTURE ONLY: the checker of ax3d_precompute_geometry,
// ax3d_precompute_mass and ax3d_precompute_elastic).
//
// Follows, for nPol = 4 and one element at a time:
//  * the geometric mappings: Mapping::sOrthogQ2 (SOLVER/src/preloop/spectral/mapping/
//    Mapping.cpp:48-53), SphericalMapping::mapping / jacobian (SphericalMapping.cpp:9-78),
//    LinearMapping (LinearMapping.cpp:8-44), SemiSphericalMapping (SemiSphericalMapping.cpp:
//    9-70), XMath::makeClose (SOLVER/src/preloop/utilities/XMath.cpp:9-16);
//  * Quad::createGraident and Quad::formIntegralFactor (SOLVER/src/preloop/mesh/Quad.cpp:
//    509-547), with SpectralConstants::getXiEta / getWeights (GLJ in xi on axial elements);
//  * Material::computeElementalMass (SOLVER/src/preloop/physics/material/Material.cpp:233-255)
//    without relabelling (mass Jacobian 1);
//  * Material::createElastic for isotropic / transversely isotropic elements (Material.cpp:
//    280-379): A = rho vph^2 iFact, C = rho vpv^2 iFact, L = rho vsv^2 iFact,
//    N = rho vsh^2 iFact, F = eta (A - 2 L), then with attenuation the Voigt split and
//    AttBuilder::createAttenuation1D/3D (SOLVER/src/preloop/physics/attenuation/
//    AttBuilder.cpp:17-129) with AttAxiSEM::computeAttFactors (AttAxiSEM.cpp:14-57) and
//    Quad::computeWeightsCG4 (Quad.cpp:438-466).
#pragma once

#include <cmath>
#include <cstdint>
#include <vector>

namespace axo_pre {

constexpr double PI = 3.14159265358979323846;

struct Spectral {
    double xg[5], wg[5], xj[5], wj[5];  // GLL and GLJ(0,1) nodes and weights
};

// Mapping::sOrthogQ2: rotation that brings side `co` to position 2
inline void q2(int co, double Q[2][2]) {
    static const double T[4][2][2] = {{{-1, 0}, {0, -1}}, {{0, -1}, {1, 0}}, {{1, 0}, {0, 1}}, {{0, 1}, {-1, 0}}};
    for (int i = 0; i < 2; i++)
        for (int j = 0; j < 2; j++) Q[i][j] = T[co][i][j];
}
inline int period(int p) { return ((p % 4) + 4) % 4; }
inline void make_close(double &a, double &b) {
    if (a - b > PI) b += 2. * PI;
    if (b - a > PI) a += 2. * PI;
}

// (s, z) and the Jacobian d(s, z)/d(xi, eta) at (xi, eta); etype 0 spherical, 1 linear,
// 2 semi-spherical; nodes[2][4] = (s, z) of the corners.
inline void map_jac(const double nodes[2][4], double xi, double eta, int etype, int co, double sz[2],
                    double J[2][2]) {
    if (etype == 1) {
        const double xip = 1. + xi, xim = 1. - xi, etap = 1. + eta, etam = 1. - eta;
        const double shp[4] = {xim * etam / 4., xip * etam / 4., xip * etap / 4., xim * etap / 4.};
        const double dxi[4] = {-etam / 4., etam / 4., etap / 4., -etap / 4.};
        const double deta[4] = {-xim / 4., -xip / 4., xip / 4., xim / 4.};
        for (int r = 0; r < 2; r++) {
            sz[r] = J[r][0] = J[r][1] = 0.;
            for (int k = 0; k < 4; k++) {
                sz[r] += nodes[r][k] * shp[k];
                J[r][0] += nodes[r][k] * dxi[k];
                J[r][1] += nodes[r][k] * deta[k];
            }
        }
        return;
    }
    double Q[2][2];
    q2(co, Q);
    double n2[2][4], r[4], t[4];
    for (int k = 0; k < 4; k++) {
        n2[0][k] = Q[0][0] * nodes[0][k] + Q[0][1] * nodes[1][k];
        n2[1][k] = Q[1][0] * nodes[0][k] + Q[1][1] * nodes[1][k];
        r[k] = std::sqrt(n2[0][k] * n2[0][k] + n2[1][k] * n2[1][k]);
        t[k] = std::atan2(n2[0][k], n2[1][k]);
    }
    const double x = Q[0][0] * xi + Q[0][1] * eta, y = Q[1][0] * xi + Q[1][1] * eta;
    const int i0 = period(co - 2), i1 = period(co - 1), i2 = period(co), i3 = period(co + 1);
    double t2 = t[i2], t3 = t[i3];
    make_close(t2, t3);
    const double r3 = r[i3];
    const double a_out = ((1. - x) * t3 + (1. + x) * t2) / 2.;
    double s2, z2, K[2][2];
    if (etype == 0) {
        double t0 = t[i0], t1 = t[i1];
        make_close(t0, t1);
        const double r0 = r[i0];
        const double a_in = ((1. - x) * t0 + (1. + x) * t1) / 2.;
        s2 = (1. + y) * r3 / 2. * std::sin(a_out) + (1. - y) * r0 / 2. * std::sin(a_in);
        z2 = (1. + y) * r3 / 2. * std::cos(a_out) + (1. - y) * r0 / 2. * std::cos(a_in);
        K[0][0] = (1. + y) * r3 * (t2 - t3) / 4. * std::cos(a_out) + (1. - y) * r0 * (t1 - t0) / 4. * std::cos(a_in);
        K[0][1] = .5 * (r3 * std::sin(a_out) - r0 * std::sin(a_in));
        K[1][0] = -(1. + y) * r3 * (t2 - t3) / 4. * std::sin(a_out) - (1. - y) * r0 * (t1 - t0) / 4. * std::sin(a_in);
        K[1][1] = .5 * (r3 * std::cos(a_out) - r0 * std::cos(a_in));
    } else {
        const double s0 = n2[0][i0], z0 = n2[1][i0], s1 = n2[0][i1], z1 = n2[1][i1];
        s2 = (1. + y) * r3 / 2. * std::sin(a_out) + (1. - y) / 2. * (((1. - x) * s0 + (1. + x) * s1) / 2.);
        z2 = (1. + y) * r3 / 2. * std::cos(a_out) + (1. - y) / 2. * (((1. - x) * z0 + (1. + x) * z1) / 2.);
        K[0][0] = ((1. - y) * (s1 - s0)) / 4. + ((1. + y) * r3 * (t2 - t3) * std::cos(a_out)) / 4.;
        K[0][1] = -((1. - x) * s0 + (1. + x) * s1) / 4. + r3 / 2. * std::sin(a_out);
        K[1][0] = ((1. - y) * (z1 - z0)) / 4. - ((1. + y) * r3 * (t2 - t3) * std::sin(a_out)) / 4.;
        K[1][1] = -((1. - x) * z0 + (1. + x) * z1) / 4. + r3 / 2. * std::cos(a_out);
    }
    // back: sz = Q^T sz2, J = Q^T K Q
    sz[0] = Q[0][0] * s2 + Q[1][0] * z2;
    sz[1] = Q[0][1] * s2 + Q[1][1] * z2;
    for (int i = 0; i < 2; i++)
        for (int j = 0; j < 2; j++) {
            double acc = 0.;
            for (int k = 0; k < 2; k++)
                for (int l = 0; l < 2; l++) acc += Q[k][i] * K[k][l] * Q[l][j];
            J[i][j] = acc;
        }
}

// Quad::createGraident + formIntegralFactor: geo[5][25] (dsdxii, dsdeta, dzdxii, dzdeta,
// inv_s), ifact[25], crds[25][2] (GLL point (s, z))
inline void quad_geometry(const double nodes[2][4], int etype, int co, bool axial, const Spectral &S,
                          double geo[5][25], double ifact[25], double crds[25][2]) {
    for (int ip = 0; ip < 5; ip++)
        for (int jp = 0; jp < 5; jp++) {
            const int k = ip * 5 + jp;
            const double xi = axial ? S.xj[ip] : S.xg[ip], eta = S.xg[jp];
            const double wxw = (axial ? S.wj[ip] : S.wg[ip]) * S.wg[jp];
            double sz[2], J[2][2];
            map_jac(nodes, xi, eta, etype, co, sz, J);
            const double det = J[0][0] * J[1][1] - J[0][1] * J[1][0];
            geo[0][k] = J[0][0] / det;
            geo[1][k] = -J[0][1] / det;
            geo[2][k] = -J[1][0] / det;
            geo[3][k] = J[1][1] / det;
            geo[4][k] = (axial && ip == 0) ? 0. : 1. / sz[0];
            if (axial)
                ifact[k] = ip == 0 ? wxw * J[0][0] * det : wxw * sz[0] / (1. + xi) * det;
            else
                ifact[k] = wxw * sz[0] * det;
            crds[k][0] = sz[0];
            crds[k][1] = sz[1];
        }
}

// Material::computeElementalMass: rho iFact (solid) or iFact / (rho vp^2) (fluid), per row
inline void elemental_mass(int rows, const double ifact[25], const double *rho, const double *vp, bool fluid,
                           double *mass) {
    for (int k = 0; k < rows; k++)
        for (int p = 0; p < 25; p++) {
            const int64_t i = (int64_t)k * 25 + p;
            const double m = fluid ? 1. / (rho[i] * vp[i] * vp[i]) : rho[i];
            mass[i] = m * ifact[p];
        }
}

// Quad::computeWeightsCG4
inline void cg4_weights(const double f[25], double w[4]) {
    auto F = [&](int a, int b) { return f[a * 5 + b]; };
    w[0] = (F(0, 0) + F(0, 1) + F(1, 0) + F(1, 1) + .5 * (F(0, 2) + F(1, 2) + F(2, 0) + F(2, 1)) + .25 * F(2, 2)) /
           F(1, 1);
    w[1] = (F(0, 3) + F(0, 4) + F(1, 3) + F(1, 4) + .5 * (F(0, 2) + F(1, 2) + F(2, 3) + F(2, 4)) + .25 * F(2, 2)) /
           F(1, 3);
    w[2] = (F(3, 0) + F(3, 1) + F(4, 0) + F(4, 1) + .5 * (F(2, 0) + F(2, 1) + F(3, 2) + F(4, 2)) + .25 * F(2, 2)) /
           F(3, 1);
    w[3] = (F(3, 3) + F(3, 4) + F(4, 3) + F(4, 4) + .5 * (F(2, 3) + F(2, 4) + F(3, 2) + F(4, 2)) + .25 * F(2, 2)) /
           F(3, 3);
}

struct AttFit {
    int nsls;
    std::vector<double> w, y;
    double f_min, f_max, f_ref;
    bool do_kappa;
};

// Material::createElastic (+ AttBuilder / AttAxiSEM) for one element of `rows` rows (1-D:
// 1, 3-D: nr): model values [rows][25]; out moduli [k][rows][25] (k = 2 isotropic: F = lambda,
// L = mu; 5: A, C, F, L, N); with att (1 full, 2 CG4) att_out [2][rows][npa] (dkappa, dmu).
inline void create_elastic(int rows, const double ifact[25], const double *vpv, const double *vph,
                           const double *vsv, const double *vsh, const double *eta, const double *rho,
                           const double *qk, const double *qm, bool iso, int att, const AttFit *fit,
                           double *mod, double *att_out) {
    const int n = rows * 25;
    std::vector<double> A(n), C(n), F(n), L(n), N(n);
    for (int i = 0; i < n; i++) {
        const double f = ifact[i % 25];
        A[i] = rho[i] * (vph[i] * vph[i] * f);
        C[i] = rho[i] * (vpv[i] * vpv[i] * f);
        L[i] = rho[i] * (vsv[i] * vsv[i] * f);
        N[i] = rho[i] * (vsh[i] * vsh[i] * f);
        F[i] = eta[i] * (A[i] - 2. * L[i]);
    }
    if (att) {
        // AttAxiSEM::computeAttFactors, the scalar part
        double ysum = 0.;
        for (int l = 0; l < fit->nsls; l++) ysum += fit->y[l];
        const double w0 = fit->f_ref * (2 * PI), w1 = std::sqrt(fit->f_min * fit->f_max) * (2. * PI);
        double fact = 0.;
        for (int l = 0; l < fit->nsls; l++) fact += fit->y[l] / ysum * fit->w[l] * fit->w[l] / (w1 * w1 + fit->w[l] * fit->w[l]);
        const double lw = std::log(w1 / w0);
        double wcg[4];
        cg4_weights(ifact, wcg);
        const int cgp[4] = {6, 8, 16, 18};
        const int npa = att == 2 ? 4 : 25;
        for (int k = 0; k < rows; k++) {
            double kp[25], mu[25], dkf[25], kfa[25], kfn[25], dmf[25], mfa[25], mfn[25];
            for (int p = 0; p < 25; p++) {
                const int i = k * 25 + p;
                kp[p] = (4. * A[i] + C[i] + 4. * F[i] - 4. * N[i]) / 9.;
                mu[p] = (A[i] + C[i] - 2. * F[i] + 6. * L[i] + 5. * N[i]) / 15.;
                A[i] -= kp[p] + 4. / 3. * mu[p];
                C[i] -= kp[p] + 4. / 3. * mu[p];
                F[i] -= kp[p] - 2. / 3. * mu[p];
                L[i] -= mu[p];
                N[i] -= mu[p];
                if (fit->do_kappa) {
                    kfn[p] = 1. + 2. * lw / PI * (1. / qk[i]);
                    dkf[p] = kfn[p] / (1. / ysum * qk[i] + (1. - fact));
                    kfa[p] = kfn[p] + dkf[p] * fact;
                } else {
                    dkf[p] = 0.;
                    kfa[p] = kfn[p] = 1.;
                }
                mfn[p] = 1. + 2. * lw / PI * (1. / qm[i]);
                dmf[p] = mfn[p] / (1. / ysum * qm[i] + (1. - fact));
                mfa[p] = mfn[p] + dmf[p] * fact;
            }
            double *dk = att_out + (int64_t)k * npa, *dm = att_out + (int64_t)rows * npa + (int64_t)k * npa;
            if (att == 2) {
                for (int c = 0; c < 4; c++) {
                    const int p = cgp[c];
                    dk[c] = wcg[c] * dkf[p] * kp[p];
                    dm[c] = wcg[c] * dmf[p] * mu[p];
                }
                for (int p = 0; p < 25; p++) {
                    kp[p] *= kfn[p];
                    mu[p] *= mfn[p];
                }
                for (int c = 0; c < 4; c++) {
                    const int p = cgp[c];
                    kp[p] *= 1. + wcg[c] * (kfa[p] / kfn[p] - 1.);
                    mu[p] *= 1. + wcg[c] * (mfa[p] / mfn[p] - 1.);
                }
            } else {
                for (int p = 0; p < 25; p++) {
                    dk[p] = dkf[p] * kp[p];
                    dm[p] = dmf[p] * mu[p];
                    kp[p] *= kfa[p];
                    mu[p] *= mfa[p];
                }
            }
            for (int p = 0; p < 25; p++) {
                const int i = k * 25 + p;
                A[i] += kp[p] + 4. / 3. * mu[p];
                C[i] += kp[p] + 4. / 3. * mu[p];
                F[i] += kp[p] - 2. / 3. * mu[p];
                L[i] += mu[p];
                N[i] += mu[p];
            }
        }
    }
    if (iso) {
        for (int i = 0; i < n; i++) {
            mod[i] = F[i];
            mod[n + i] = L[i];
        }
    } else {
        for (int i = 0; i < n; i++) {
            mod[i] = A[i];
            mod[n + i] = C[i];
            mod[2 * n + i] = F[i];
            mod[3 * n + i] = L[i];
            mod[4 * n + i] = N[i];
        }
    }
}

}  // namespace axo_pre
