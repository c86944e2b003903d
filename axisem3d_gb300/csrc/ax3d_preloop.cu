// ax3d_preloop.cu -- pre-loop on the GPU in FP64: the elastic moduli of many elements at
// once, Material::createElastic (SOLVER/src/preloop/physics/material/Material.cpp:280-379)
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

extern "C" size_t ax3d_precompute_last_error(char *buf, size_t n) {
    const std::string &s = ax3d::g_pre_err;
    if (buf && n) {
        const size_t k = std::min(n - 1, s.size());
        std::copy(s.begin(), s.begin() + k, buf);
        buf[k] = 0;
    }
    return s.size();
}
