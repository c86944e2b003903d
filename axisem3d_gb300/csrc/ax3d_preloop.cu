// ax3d_preloop.cu -- pre-loop on the GPU in FP64.
//
// Geometry and mass: Quad::createGraident and Quad::formIntegralFactor
// (SOLVER/src/preloop/mesh/Quad.cpp:509-547) over the spherical, linear and semi-spherical
// mappings (SOLVER/src/preloop/spectral/mapping/SphericalMapping.cpp:9-78,
// LinearMapping.cpp:8-44, SemiSphericalMapping.cpp:9-70, rotated by Mapping::sOrthogQ2,
// Mapping.cpp:48-53), and Material::computeElementalMass (Material.cpp:233-255); one thread
// per (element, GLL point) or (element, row, GLL point).
//
// Moduli: the elastic moduli of many elements at once, Material::createElastic (SOLVER/src/preloop/physics/material/Material.cpp:280-379)
// with the attenuation split of AttBuilder::createAttenuation1D/3D
// (SOLVER/src/preloop/physics/attenuation/AttBuilder.cpp:17-129), the per-sample factors of
// AttAxiSEM::computeAttFactors (AttAxiSEM.cpp:14-57) and the CG4 weights of
// Quad::computeWeightsCG4 (Quad.cpp:438-466).  One CTA per element, one thread per
// (sample, GLL point); the model values come in as FP32, everything is computed in FP64 and
// the moduli leave as FP32 in the layout ax3d_add_elements takes.
#include <algorithm>
#include <cmath>
#include <string>
#include <vector>

#include "../../include/ax3d.h"
#include "ax3d_common.cuh"

namespace ax3d {
namespace {

struct AttScalars {
    int on, cg4, do_kappa;
    double ysum, fact, lw;  // sum y, sum yd w^2 / (w1^2 + w^2), log(w1 / w0)
};

__device__ __forceinline__ int cg4_slot(int p) {
    return p == 6 ? 0 : p == 8 ? 1 : p == 16 ? 2 : p == 18 ? 3 : -1;
}

// CG4 weight of coarse point i from the element's integral factors
__device__ double cg4_weight(const double *f, int i) {
    auto F = [&](int a, int b) { return f[a * 5 + b]; };
    switch (i) {
        case 0:
            return (F(0, 0) + F(0, 1) + F(1, 0) + F(1, 1) + 0.5 * (F(0, 2) + F(1, 2) + F(2, 0) + F(2, 1)) +
                    0.25 * F(2, 2)) / F(1, 1);
        case 1:
            return (F(0, 3) + F(0, 4) + F(1, 3) + F(1, 4) + 0.5 * (F(0, 2) + F(1, 2) + F(2, 3) + F(2, 4)) +
                    0.25 * F(2, 2)) / F(1, 3);
        case 2:
            return (F(3, 0) + F(3, 1) + F(4, 0) + F(4, 1) + 0.5 * (F(2, 0) + F(2, 1) + F(3, 2) + F(4, 2)) +
                    0.25 * F(2, 2)) / F(3, 1);
        default:
            return (F(3, 3) + F(3, 4) + F(4, 3) + F(4, 4) + 0.5 * (F(2, 3) + F(2, 4) + F(3, 2) + F(4, 2)) +
                    0.25 * F(2, 2)) / F(3, 3);
    }
}

// in: [6 or 8][rows][25] per element at rofs (vpv, vph, vsv, vsh, eta, rho[, qkappa, qmu]);
// out moduli [nmod][rows][25] at mofs, attenuation moduli [2][rows][npa] at aofs
__global__ void __launch_bounds__(256)
    k_pre_elastic(int ne, const int32_t *__restrict__ rows, const int64_t *__restrict__ rofs,
                  const double *__restrict__ ifact, const float *__restrict__ vpv, const float *__restrict__ vph,
                  const float *__restrict__ vsv, const float *__restrict__ vsh, const float *__restrict__ eta,
                  const float *__restrict__ rho, const float *__restrict__ qk, const float *__restrict__ qm,
                  int iso, AttScalars S, float *__restrict__ mod, const int64_t *__restrict__ mofs,
                  float *__restrict__ attm, const int64_t *__restrict__ aofs) {
    const double pi = 3.14159265358979323846;
    for (int e = blockIdx.x; e < ne; e += gridDim.x) {
        const int nr = rows[e];
        const double *f = ifact + (int64_t)e * 25;
        const int npa = S.cg4 ? 4 : 25;
        for (int t = threadIdx.x; t < nr * 25; t += blockDim.x) {
            const int k = t / 25, p = t - k * 25;
            const int64_t i = rofs[e] + t;
            const double fi = f[p], r = rho[i];
            const double vh = vph[i], vv = vpv[i], sv = vsv[i], sh = vsh[i];
            double A = r * vh * vh * fi, C = r * vv * vv * fi, L = r * sv * sv * fi, N = r * sh * sh * fi;
            double F = (double)eta[i] * (A - 2.0 * L);
            if (S.on) {
                double kappa = (4.0 * A + C + 4.0 * F - 4.0 * N) / 9.0;
                double mu = (A + C - 2.0 * F + 6.0 * L + 5.0 * N) / 15.0;
                A -= kappa + 4.0 / 3.0 * mu;
                C -= kappa + 4.0 / 3.0 * mu;
                F -= kappa - 2.0 / 3.0 * mu;
                L -= mu;
                N -= mu;
                const double qkappa = qk[i], qmu = qm[i];
                double dkp = 0.0, kp_att = 1.0, kp_no = 1.0;
                if (S.do_kappa) {
                    kp_no = 1.0 + 2.0 * S.lw / pi / qkappa;
                    dkp = kp_no / (qkappa / S.ysum + (1.0 - S.fact));
                    kp_att = kp_no + dkp * S.fact;
                }
                const double mu_no = 1.0 + 2.0 * S.lw / pi / qmu;
                const double dmu = mu_no / (qmu / S.ysum + (1.0 - S.fact));
                const double mu_att = mu_no + dmu * S.fact;
                float *ao = attm + aofs[e];
                if (S.cg4) {
                    const int c = cg4_slot(p);
                    if (c >= 0) {
                        const double wc = cg4_weight(f, c);
                        ao[(int64_t)k * npa + c] = (float)(wc * dkp * kappa);
                        ao[(int64_t)nr * npa + (int64_t)k * npa + c] = (float)(wc * dmu * mu);
                        kappa = kappa * kp_no * (1.0 + wc * (kp_att / kp_no - 1.0));
                        mu = mu * mu_no * (1.0 + wc * (mu_att / mu_no - 1.0));
                    } else {
                        kappa *= kp_no;
                        mu *= mu_no;
                    }
                } else {
                    ao[(int64_t)k * npa + p] = (float)(dkp * kappa);
                    ao[(int64_t)nr * npa + (int64_t)k * npa + p] = (float)(dmu * mu);
                    kappa *= kp_att;
                    mu *= mu_att;
                }
                A += kappa + 4.0 / 3.0 * mu;
                C += kappa + 4.0 / 3.0 * mu;
                F += kappa - 2.0 / 3.0 * mu;
                L += mu;
                N += mu;
            }
            float *mo = mod + mofs[e];
            const int64_t plane = (int64_t)nr * 25;
            if (iso) {  // Isotropic1D / 3D take (F, L) = (lambda, mu)
                mo[t] = (float)F;
                mo[plane + t] = (float)L;
            } else {
                mo[t] = (float)A;
                mo[plane + t] = (float)C;
                mo[2 * plane + t] = (float)F;
                mo[3 * plane + t] = (float)L;
                mo[4 * plane + t] = (float)N;
            }
        }
    }
}

// (s, z) and d(s, z)/d(xi, eta) of one GLL point; etype 0 spherical, 1 linear, 2 semi-spherical
__device__ void map_jac(const double *nd, double xi, double eta, int etype, int co, double sz[2], double J[2][2]) {
    // nd: (s0..s3, z0..z3) of the corners
    if (etype == 1) {
        const double xp = 1.0 + xi, xm = 1.0 - xi, ep = 1.0 + eta, em = 1.0 - eta;
        const double shp[4] = {0.25 * xm * em, 0.25 * xp * em, 0.25 * xp * ep, 0.25 * xm * ep};
        const double dx[4] = {-0.25 * em, 0.25 * em, 0.25 * ep, -0.25 * ep};
        const double de[4] = {-0.25 * xm, -0.25 * xp, 0.25 * xp, 0.25 * xm};
        for (int c = 0; c < 2; c++) {
            double a = 0.0, b = 0.0, d = 0.0;
            for (int k = 0; k < 4; k++) {
                a += nd[4 * c + k] * shp[k];
                b += nd[4 * c + k] * dx[k];
                d += nd[4 * c + k] * de[k];
            }
            sz[c] = a;
            J[c][0] = b;
            J[c][1] = d;
        }
        return;
    }
    // rotation bringing the curved side to position 2: rows (q00, q01), (q10, q11)
    const double Q[4][4] = {{-1, 0, 0, -1}, {0, -1, 1, 0}, {1, 0, 0, 1}, {0, 1, -1, 0}};
    const double q00 = Q[co][0], q01 = Q[co][1], q10 = Q[co][2], q11 = Q[co][3];
    const int i0 = (co + 2) & 3, i1 = (co + 3) & 3, i2 = co & 3, i3 = (co + 1) & 3;
    auto rot = [&](int k, double &a, double &b) {
        a = q00 * nd[k] + q01 * nd[4 + k];
        b = q10 * nd[k] + q11 * nd[4 + k];
    };
    double s2n, z2n, s3n, z3n;
    rot(i2, s2n, z2n);
    rot(i3, s3n, z3n);
    const double pi = 3.14159265358979323846;
    double t2 = atan2(s2n, z2n), t3 = atan2(s3n, z3n);
    if (t2 - t3 > pi) t3 += 2.0 * pi;  // XMath::makeClose
    if (t3 - t2 > pi) t2 += 2.0 * pi;
    const double r3 = sqrt(s3n * s3n + z3n * z3n);
    const double x = q00 * xi + q01 * eta, y = q10 * xi + q11 * eta;
    const double ao = ((1.0 - x) * t3 + (1.0 + x) * t2) / 2.0;
    const double so = sin(ao), coo = cos(ao);
    double s2, z2, K00, K01, K10, K11;
    double s0n, z0n, s1n, z1n;
    rot(i0, s0n, z0n);
    rot(i1, s1n, z1n);
    if (etype == 0) {
        double t0 = atan2(s0n, z0n), t1 = atan2(s1n, z1n);
        if (t0 - t1 > pi) t1 += 2.0 * pi;
        if (t1 - t0 > pi) t0 += 2.0 * pi;
        const double r0 = sqrt(s0n * s0n + z0n * z0n);
        const double ai = ((1.0 - x) * t0 + (1.0 + x) * t1) / 2.0;
        const double si = sin(ai), ci = cos(ai);
        s2 = (1.0 + y) * r3 / 2.0 * so + (1.0 - y) * r0 / 2.0 * si;
        z2 = (1.0 + y) * r3 / 2.0 * coo + (1.0 - y) * r0 / 2.0 * ci;
        K00 = (1.0 + y) * r3 * (t2 - t3) / 4.0 * coo + (1.0 - y) * r0 * (t1 - t0) / 4.0 * ci;
        K01 = 0.5 * (r3 * so - r0 * si);
        K10 = -(1.0 + y) * r3 * (t2 - t3) / 4.0 * so - (1.0 - y) * r0 * (t1 - t0) / 4.0 * si;
        K11 = 0.5 * (r3 * coo - r0 * ci);
    } else {
        s2 = (1.0 + y) * r3 / 2.0 * so + (1.0 - y) / 2.0 * (((1.0 - x) * s0n + (1.0 + x) * s1n) / 2.0);
        z2 = (1.0 + y) * r3 / 2.0 * coo + (1.0 - y) / 2.0 * (((1.0 - x) * z0n + (1.0 + x) * z1n) / 2.0);
        K00 = ((1.0 - y) * (s1n - s0n)) / 4.0 + ((1.0 + y) * r3 * (t2 - t3) * coo) / 4.0;
        K01 = -((1.0 - x) * s0n + (1.0 + x) * s1n) / 4.0 + r3 / 2.0 * so;
        K10 = ((1.0 - y) * (z1n - z0n)) / 4.0 - ((1.0 + y) * r3 * (t2 - t3) * so) / 4.0;
        K11 = -((1.0 - x) * z0n + (1.0 + x) * z1n) / 4.0 + r3 / 2.0 * coo;
    }
    sz[0] = q00 * s2 + q10 * z2;  // Q^T (s2, z2)
    sz[1] = q01 * s2 + q11 * z2;
    // J = Q^T K Q
    const double KQ00 = K00 * q00 + K01 * q10, KQ01 = K00 * q01 + K01 * q11;
    const double KQ10 = K10 * q00 + K11 * q10, KQ11 = K10 * q01 + K11 * q11;
    J[0][0] = q00 * KQ00 + q10 * KQ10;
    J[0][1] = q00 * KQ01 + q10 * KQ11;
    J[1][0] = q01 * KQ00 + q11 * KQ10;
    J[1][1] = q01 * KQ01 + q11 * KQ11;
}

struct SpecNodes {
    double xg[5], wg[5], xj[5], wj[5];
};

// nodes [n][2][4]; out geo [n][5][25], ifact [n][25], crds [n][25][2]
__global__ void __launch_bounds__(256)
    k_pre_geometry(int n, const double *__restrict__ nodes, const int8_t *__restrict__ etype,
                   const int8_t *__restrict__ curved, const uint8_t *__restrict__ axial, SpecNodes S,
                   double *__restrict__ geo, double *__restrict__ ifact, double *__restrict__ crds) {
    const int64_t total = (int64_t)n * 25;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        const int e = (int)(t / 25), k = (int)(t - (int64_t)e * 25);
        const int ip = k / 5, jp = k - 5 * (k / 5);
        const bool ax = axial[e] != 0;
        const double xi = ax ? S.xj[ip] : S.xg[ip], eta = S.xg[jp];
        const double wxw = (ax ? S.wj[ip] : S.wg[ip]) * S.wg[jp];
        double sz[2], J[2][2];
        map_jac(nodes + (int64_t)e * 8, xi, eta, etype[e], curved[e], sz, J);
        const double det = J[0][0] * J[1][1] - J[0][1] * J[1][0];
        double *g = geo + (int64_t)e * 125;
        g[k] = J[0][0] / det;
        g[25 + k] = -J[0][1] / det;
        g[50 + k] = -J[1][0] / det;
        g[75 + k] = J[1][1] / det;
        g[100 + k] = (ax && ip == 0) ? 0.0 : 1.0 / sz[0];
        double f;
        if (ax)
            f = ip == 0 ? wxw * J[0][0] * det : wxw * sz[0] / (1.0 + xi) * det;
        else
            f = wxw * sz[0] * det;
        ifact[t] = f;
        crds[2 * t] = sz[0];
        crds[2 * t + 1] = sz[1];
    }
}

// Material::computeElementalMass: per (element, row, point) rho iFact, fluid iFact / (rho vp^2)
__global__ void k_pre_mass(int n, const int32_t *__restrict__ rows, const int64_t *__restrict__ rofs,
                           const double *__restrict__ ifact, const float *__restrict__ rho,
                           const float *__restrict__ vp, const uint8_t *__restrict__ fluid,
                           double *__restrict__ mass) {
    for (int e = blockIdx.x; e < n; e += gridDim.x) {
        const bool fl = fluid[e] != 0;
        for (int t = threadIdx.x; t < rows[e] * 25; t += blockDim.x) {
            const int64_t i = rofs[e] + t;
            const double r = rho[i];
            const double m = fl ? 1.0 / (r * ((double)vp[i] * (double)vp[i])) : r;
            mass[i] = m * ifact[(int64_t)e * 25 + t % 25];
        }
    }
}

// 3-D model sampling (Material::addVolumetric3D, Material.cpp:96-231, for the project's
// Gaussian-random model): the field rms sqrt(2 / M) sum_j cos(kr_j r + klR_j . n + phase_j) at
// every GLL point of every element on its nr slices phi_k = 2 pi k / nr (or one phi in 2-D
// mode), x = (s cos phi, s sin phi, z), r = |x|, n = x / r.  One thread per sample, FP64.
__global__ void __launch_bounds__(256)
    k_pre_gaussian_random(int n, const int32_t *__restrict__ rows, const int64_t *__restrict__ rofs,
                          const double *__restrict__ crds, int modes, const double *__restrict__ kr,
                          const double *__restrict__ klR, const double *__restrict__ ph, double amp,
                          double phi2d, int use_phi2d, double *__restrict__ out) {
    extern __shared__ double sm_modes[];  // kr, klR (3 x modes), phase
    for (int i = threadIdx.x; i < modes; i += blockDim.x) {
        sm_modes[i] = kr[i];
        sm_modes[modes + i] = klR[i];
        sm_modes[2 * modes + i] = klR[modes + i];
        sm_modes[3 * modes + i] = klR[2 * modes + i];
        sm_modes[4 * modes + i] = ph[i];
    }
    __syncthreads();
    const double two_pi = 6.28318530717958647692;
    for (int e = blockIdx.x; e < n; e += gridDim.x) {
        const int nr = rows[e];
        for (int t = threadIdx.x; t < nr * 25; t += blockDim.x) {
            const int k = t / 25, p = t - k * 25;
            const double s = crds[((int64_t)e * 25 + p) * 2], z = crds[((int64_t)e * 25 + p) * 2 + 1];
            const double phi = use_phi2d ? phi2d : two_pi * (double)k / (double)nr;
            double sp, cp;
            sincos(phi, &sp, &cp);
            const double x = s * cp, y = s * sp;
            const double r = sqrt(x * x + y * y + z * z);
            const double inv = 1.0 / fmax(r, 1e-9);
            const double nx = x * inv, ny = y * inv, nz = z * inv;
            double acc = 0.0;
            for (int j = 0; j < modes; j++)
                acc += cos(sm_modes[j] * r + nx * sm_modes[modes + j] + ny * sm_modes[2 * modes + j] +
                           nz * sm_modes[3 * modes + j] + sm_modes[4 * modes + j]);
            out[rofs[e] + t] = amp * acc;
        }
    }
}

template <typename T>
struct Dev {
    T *p = nullptr;
    ~Dev() { release(); }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
    }
    cudaError_t up(const T *h, size_t n) {
        cudaError_t e = cudaMalloc(&p, std::max<size_t>(n, 1) * sizeof(T));
        if (e == cudaSuccess && h && n) e = cudaMemcpy(p, h, n * sizeof(T), cudaMemcpyHostToDevice);
        return e;
    }
};

thread_local std::string g_pre_err;

}  // namespace
}  // namespace ax3d

extern "C" int ax3d_precompute_elastic(int32_t device, int32_t n_elem, const int32_t *rows, const double *ifact,
                                       const float *vpv, const float *vph, const float *vsv, const float *vsh,
                                       const float *eta, const float *rho, const float *qkappa, const float *qmu,
                                       int32_t isotropic, int32_t att, int32_t nsls, const double *w,
                                       const double *y, double f_min, double f_max, double f_ref,
                                       int32_t do_kappa, float *moduli, float *att_moduli) {
    using namespace ax3d;
    if (n_elem < 0 || (n_elem && (!rows || !ifact || !vpv || !vph || !vsv || !vsh || !eta || !rho || !moduli)) ||
        att < 0 || att > 2 || (att && (!qkappa || !qmu || !att_moduli || nsls < 1 || !w || !y))) {
        g_pre_err = "ax3d_precompute_elastic || bad argument";
        return AX3D_ERR_ARG;
    }
    AttScalars S{att != 0, att == AX3D_ATT_CG4, do_kappa != 0, 0.0, 0.0, 0.0};
    if (att) {
        // AttAxiSEM::computeAttFactors: the element-independent sums
        const double pi = 3.14159265358979323846;
        for (int l = 0; l < nsls; l++) S.ysum += y[l];
        const double w0 = f_ref * 2.0 * pi, w1 = std::sqrt(f_min * f_max) * 2.0 * pi;
        for (int l = 0; l < nsls; l++) S.fact += (y[l] / S.ysum) * w[l] * w[l] / (w1 * w1 + w[l] * w[l]);
        S.lw = std::log(w1 / w0);
    }
    std::vector<int64_t> rofs(n_elem), mofs(n_elem), aofs(n_elem);
    int64_t nrow = 0, nmod = 0, natt = 0;
    const int km = isotropic ? 2 : 5, npa = att == AX3D_ATT_CG4 ? 4 : 25;
    for (int e = 0; e < n_elem; e++) {
        if (rows[e] < 1) {
            g_pre_err = "ax3d_precompute_elastic || rows must be >= 1";
            return AX3D_ERR_ARG;
        }
        rofs[e] = nrow * 25;
        mofs[e] = nmod;
        aofs[e] = natt;
        nrow += rows[e];
        nmod += (int64_t)km * rows[e] * 25;
        natt += att ? (int64_t)2 * rows[e] * npa : 0;
    }
    const size_t nv = (size_t)nrow * 25;
    int prev_device = 0;
    cudaGetDevice(&prev_device);
    cudaError_t err = cudaSetDevice(device);
    Dev<int32_t> d_rows;
    Dev<int64_t> d_rofs, d_mofs, d_aofs;
    Dev<double> d_if;
    Dev<float> d_in[8], d_mod, d_att;
    const float *hin[8] = {vpv, vph, vsv, vsh, eta, rho, qkappa, qmu};
    if (err == cudaSuccess) err = d_rows.up(rows, n_elem);
    if (err == cudaSuccess) err = d_rofs.up(rofs.data(), n_elem);
    if (err == cudaSuccess) err = d_mofs.up(mofs.data(), n_elem);
    if (err == cudaSuccess) err = d_aofs.up(aofs.data(), n_elem);
    if (err == cudaSuccess) err = d_if.up(ifact, (size_t)n_elem * 25);
    for (int k = 0; k < 8 && err == cudaSuccess; k++) err = d_in[k].up(k < 6 || att ? hin[k] : nullptr, k < 6 || att ? nv : 1);
    if (err == cudaSuccess) err = d_mod.up(nullptr, nmod);
    if (err == cudaSuccess) err = d_att.up(nullptr, natt);
    if (err == cudaSuccess && n_elem > 0) {
        const int grid = std::min(n_elem, 152 * 16);
        k_pre_elastic<<<grid, 256>>>(n_elem, d_rows.p, d_rofs.p, d_if.p, d_in[0].p, d_in[1].p, d_in[2].p, d_in[3].p,
                                     d_in[4].p, d_in[5].p, d_in[6].p, d_in[7].p, isotropic != 0, S, d_mod.p,
                                     d_mofs.p, d_att.p, d_aofs.p);
        err = cudaGetLastError();
        if (err == cudaSuccess) err = cudaMemcpy(moduli, d_mod.p, nmod * sizeof(float), cudaMemcpyDeviceToHost);
        if (err == cudaSuccess && natt)
            err = cudaMemcpy(att_moduli, d_att.p, natt * sizeof(float), cudaMemcpyDeviceToHost);
    }
    // the device buffers are freed here, on `device`; then the caller's device is restored
    for (auto *d : {&d_in[0], &d_in[1], &d_in[2], &d_in[3], &d_in[4], &d_in[5], &d_in[6], &d_in[7], &d_mod, &d_att})
        d->release();
    d_rows.release();
    d_rofs.release();
    d_mofs.release();
    d_aofs.release();
    d_if.release();
    cudaSetDevice(prev_device);
    if (err != cudaSuccess) {
        g_pre_err = std::string("ax3d_precompute_elastic || CUDA: ") + cudaGetErrorString(err);
        return AX3D_ERR_CUDA;
    }
    return AX3D_OK;
}

extern "C" int ax3d_precompute_geometry(int32_t device, int32_t n_elem, const double *nodes, const int8_t *etype,
                                        const int8_t *curved_outer, const uint8_t *axial, const double *spectral,
                                        double *geometry, double *ifact, double *crds) {
    using namespace ax3d;
    if (n_elem < 0 || (n_elem && (!nodes || !etype || !curved_outer || !axial || !spectral || !geometry || !ifact ||
                                  !crds))) {
        g_pre_err = "ax3d_precompute_geometry || bad argument";
        return AX3D_ERR_ARG;
    }
    for (int e = 0; e < n_elem; e++)
        if (etype[e] < 0 || etype[e] > 2 || (etype[e] != 1 && (curved_outer[e] < 0 || curved_outer[e] > 3))) {
            g_pre_err = "ax3d_precompute_geometry || mapping type must be 0..2 and, for a curved mapping, curved "
                        "side 0..3";
            return AX3D_ERR_ARG;
        }
    if (n_elem == 0) return AX3D_OK;
    SpecNodes S;
    for (int i = 0; i < 5; i++) {
        S.xg[i] = spectral[i];
        S.wg[i] = spectral[5 + i];
        S.xj[i] = spectral[10 + i];
        S.wj[i] = spectral[15 + i];
    }
    int prev_device = 0;
    cudaGetDevice(&prev_device);
    cudaError_t err = cudaSetDevice(device);
    Dev<double> d_nodes, d_geo, d_if, d_crds;
    Dev<int8_t> d_et, d_co;
    Dev<uint8_t> d_ax;
    const size_t ne = (size_t)n_elem;
    if (err == cudaSuccess) err = d_nodes.up(nodes, ne * 8);
    if (err == cudaSuccess) err = d_et.up(etype, ne);
    if (err == cudaSuccess) err = d_co.up(curved_outer, ne);
    if (err == cudaSuccess) err = d_ax.up(axial, ne);
    if (err == cudaSuccess) err = d_geo.up(nullptr, ne * 125);
    if (err == cudaSuccess) err = d_if.up(nullptr, ne * 25);
    if (err == cudaSuccess) err = d_crds.up(nullptr, ne * 50);
    if (err == cudaSuccess) {
        int sms = 0;
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
        const int grid = (int)std::min<int64_t>(((int64_t)ne * 25 + 255) / 256, (int64_t)std::max(sms, 1) * 8);
        k_pre_geometry<<<grid, 256>>>(n_elem, d_nodes.p, d_et.p, d_co.p, d_ax.p, S, d_geo.p, d_if.p, d_crds.p);
        err = cudaGetLastError();
        if (err == cudaSuccess) err = cudaMemcpy(geometry, d_geo.p, ne * 125 * sizeof(double), cudaMemcpyDeviceToHost);
        if (err == cudaSuccess) err = cudaMemcpy(ifact, d_if.p, ne * 25 * sizeof(double), cudaMemcpyDeviceToHost);
        if (err == cudaSuccess) err = cudaMemcpy(crds, d_crds.p, ne * 50 * sizeof(double), cudaMemcpyDeviceToHost);
    }
    d_nodes.release();
    d_et.release();
    d_co.release();
    d_ax.release();
    d_geo.release();
    d_if.release();
    d_crds.release();
    cudaSetDevice(prev_device);
    if (err != cudaSuccess) {
        g_pre_err = std::string("ax3d_precompute_geometry || CUDA: ") + cudaGetErrorString(err);
        return AX3D_ERR_CUDA;
    }
    return AX3D_OK;
}

extern "C" int ax3d_precompute_mass(int32_t device, int32_t n_elem, const int32_t *rows, const double *ifact,
                                    const float *rho, const float *vp, const uint8_t *fluid, double *mass) {
    using namespace ax3d;
    if (n_elem < 0 || (n_elem && (!rows || !ifact || !rho || !fluid || !mass))) {
        g_pre_err = "ax3d_precompute_mass || bad argument";
        return AX3D_ERR_ARG;
    }
    std::vector<int64_t> rofs(n_elem);
    int64_t nrow = 0;
    bool any_fluid = false;
    for (int e = 0; e < n_elem; e++) {
        if (rows[e] < 1) {
            g_pre_err = "ax3d_precompute_mass || rows must be >= 1";
            return AX3D_ERR_ARG;
        }
        rofs[e] = nrow * 25;
        nrow += rows[e];
        any_fluid |= fluid[e] != 0;
    }
    if (any_fluid && !vp) {
        g_pre_err = "ax3d_precompute_mass || fluid elements need vp";
        return AX3D_ERR_ARG;
    }
    if (n_elem == 0) return AX3D_OK;
    const size_t nv = (size_t)nrow * 25;
    int prev_device = 0;
    cudaGetDevice(&prev_device);
    cudaError_t err = cudaSetDevice(device);
    Dev<int32_t> d_rows;
    Dev<int64_t> d_rofs;
    Dev<double> d_if, d_mass;
    Dev<float> d_rho, d_vp;
    Dev<uint8_t> d_fl;
    if (err == cudaSuccess) err = d_rows.up(rows, n_elem);
    if (err == cudaSuccess) err = d_rofs.up(rofs.data(), n_elem);
    if (err == cudaSuccess) err = d_if.up(ifact, (size_t)n_elem * 25);
    if (err == cudaSuccess) err = d_rho.up(rho, nv);
    if (err == cudaSuccess) err = d_vp.up(any_fluid ? vp : nullptr, any_fluid ? nv : 1);
    if (err == cudaSuccess) err = d_fl.up(fluid, n_elem);
    if (err == cudaSuccess) err = d_mass.up(nullptr, nv);
    if (err == cudaSuccess) {
        int sms = 0;
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
        const int grid = std::min(n_elem, std::max(sms, 1) * 16);
        k_pre_mass<<<grid, 256>>>(n_elem, d_rows.p, d_rofs.p, d_if.p, d_rho.p, d_vp.p, d_fl.p, d_mass.p);
        err = cudaGetLastError();
        if (err == cudaSuccess) err = cudaMemcpy(mass, d_mass.p, nv * sizeof(double), cudaMemcpyDeviceToHost);
    }
    d_rows.release();
    d_rofs.release();
    d_if.release();
    d_rho.release();
    d_vp.release();
    d_fl.release();
    d_mass.release();
    cudaSetDevice(prev_device);
    if (err != cudaSuccess) {
        g_pre_err = std::string("ax3d_precompute_mass || CUDA: ") + cudaGetErrorString(err);
        return AX3D_ERR_CUDA;
    }
    return AX3D_OK;
}

extern "C" int ax3d_sample_gaussian_random(int32_t device, int32_t n_elem, const int32_t *rows, const double *crds,
                                           int32_t modes, const double *kr, const double *klR, const double *phase,
                                           double rms, int32_t use_phi2d, double phi2d, double *out) {
    using namespace ax3d;
    if (n_elem < 0 || modes < 1 || modes > 4096 ||
        (n_elem && (!rows || !crds || !kr || !klR || !phase || !out))) {
        g_pre_err = "ax3d_sample_gaussian_random || bad argument";
        return AX3D_ERR_ARG;
    }
    std::vector<int64_t> rofs(n_elem);
    int64_t nrow = 0;
    for (int e = 0; e < n_elem; e++) {
        if (rows[e] < 1) {
            g_pre_err = "ax3d_sample_gaussian_random || rows must be >= 1";
            return AX3D_ERR_ARG;
        }
        rofs[e] = nrow * 25;
        nrow += rows[e];
    }
    if (n_elem == 0) return AX3D_OK;
    const size_t nv = (size_t)nrow * 25;
    int prev_device = 0;
    cudaGetDevice(&prev_device);
    cudaError_t err = cudaSetDevice(device);
    Dev<int32_t> d_rows;
    Dev<int64_t> d_rofs;
    Dev<double> d_crds, d_kr, d_kl, d_ph, d_out;
    if (err == cudaSuccess) err = d_rows.up(rows, n_elem);
    if (err == cudaSuccess) err = d_rofs.up(rofs.data(), n_elem);
    if (err == cudaSuccess) err = d_crds.up(crds, (size_t)n_elem * 50);
    if (err == cudaSuccess) err = d_kr.up(kr, modes);
    if (err == cudaSuccess) err = d_kl.up(klR, (size_t)3 * modes);
    if (err == cudaSuccess) err = d_ph.up(phase, modes);
    if (err == cudaSuccess) err = d_out.up(nullptr, nv);
    if (err == cudaSuccess) {
        int sms = 0;
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
        const int grid = std::min(n_elem, std::max(sms, 1) * 16);
        const double amp = rms * std::sqrt(2.0 / (double)modes);
        k_pre_gaussian_random<<<grid, 256, (size_t)5 * modes * sizeof(double)>>>(
            n_elem, d_rows.p, d_rofs.p, d_crds.p, modes, d_kr.p, d_kl.p, d_ph.p, amp, phi2d, use_phi2d != 0, d_out.p);
        err = cudaGetLastError();
        if (err == cudaSuccess) err = cudaMemcpy(out, d_out.p, nv * sizeof(double), cudaMemcpyDeviceToHost);
    }
    d_rows.release();
    d_rofs.release();
    d_crds.release();
    d_kr.release();
    d_kl.release();
    d_ph.release();
    d_out.release();
    cudaSetDevice(prev_device);
    if (err != cudaSuccess) {
        g_pre_err = std::string("ax3d_sample_gaussian_random || CUDA: ") + cudaGetErrorString(err);
        return AX3D_ERR_CUDA;
    }
    return AX3D_OK;
}

extern "C" size_t ax3d_precompute_last_error(char *buf, size_t n) {
    const std::string &s = ax3d::g_pre_err;
    if (buf && n) {
        const size_t k = std::min(n - 1, s.size());
        std::copy(s.begin(), s.begin() + k, buf);
        buf[k] = 0;
    }
    return s.size();
}
