// ax3d_elements.cu -- Fourier-space element stiffness kernels (Element::computeStiff of
// elements with 1D material) for sm_103a: one warp per (element, Fourier order); the
// order loop of SolidElement::displToStiff (SOLVER/src/core/element/SolidElement.cpp:
// 404-443) and FluidElement::displToStiff (FluidElement.cpp:333-355) is embarrassingly
// parallel there.  The physical-space (3D material) elements are in ax3d_phys.cu.
#include <algorithm>

#include "ax3d_elem_ops.cuh"
#include "ax3d_kernels.cuh"

namespace ax3d {



// SolidElement::computeStrain / computeCurl (SolidElement.cpp:219-345, no relabelling) at
// receivers with dump_strain / dump_curl.  One CTA of four warps per receiver: warp w takes
// orders w, w + 4, ...; lane p < 25 owns GLL point p: grad6 (strain) or grad9 (curl),
// rotated to RTZ, synthesised at the receiver's phi; the weighted sum is reduced in the CTA.
// list[i] = (receiver, strain slot or -1, curl slot or -1).
__global__ void __launch_bounds__(128)
    k_record_strain_curl(PointTable P, ElemTable T, const float2 *__restrict__ su, const int32_t *rec_elem,
                         const float *rec_phi, const float *rec_w, const int32_t *list, int n, float *strain_out,
                         int nst, float *curl_out, int ncu, int cap, const int32_t *tptr, int tofs) {
    __shared__ float2 sh[4][75];
    __shared__ float red[4][9];
    const int t = *tptr + tofs;
    if (t < 0 || t >= cap) return;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const bool active = lane < NPE;
    const int p = active ? lane : 0;
    for (int i = blockIdx.x; i < n; i += gridDim.x) {
        const int r = list[3 * i], sslot = list[3 * i + 1], cslot = list[3 * i + 2];
        const int e = rec_elem[r];
        const float phi = rec_phi[r];
        const int nr = T.nr[e], lim = nr / 2 - (nr % 2 == 0);
        const bool axial = T.flags[e] & EF_AXIAL;
        LaneOps L;
        L.init(p, axial);
        Geo g;
        g.load(T.geo + (int64_t)e * 125, p);
        const float *tr = T.trig + (int64_t)e * 100;
        const float s1 = tr[p], c1 = tr[25 + p], s2 = tr[50 + p], c2 = tr[75 + p];
        const int pt = T.pts[e * NPE + p];
        const int pnr = P.nr[pt], plim = pnr / 2 - (pnr % 2 == 0);  // scatterDisplToElement drops the Nyquist order
        const float2 *up = su + P.sofs[pt];
        float acc[9];
#pragma unroll
        for (int k = 0; k < 9; k++) acc[k] = 0.f;
        for (int a = warp; a <= lim; a += 4) {
            if (active)
#pragma unroll
                for (int c = 0; c < 3; c++)
                    sh[warp][c * 25 + lane] = a <= plim ? up[a * 3 + c] : make_float2(0.f, 0.f);
            __syncwarp();
            if (active) {
                float sn, cs;
                sincosf((float)a * phi, &sn, &cs);
                const float ex = a == 0 ? 1.f : 2.f * cs, ey = a == 0 ? 0.f : 2.f * sn;
                if (sslot >= 0) {
                    float2 e6[6];
                    grad6_lane(L, g, axial, a, sh[warp], e6);
                    spz_rtz(e6, s1, c1, s2, c2);
#pragma unroll
                    for (int k = 0; k < 6; k++) acc[k] += ex * e6[k].x - ey * e6[k].y;
                }
                if (cslot >= 0) {
                    float2 g9[9];
                    grad9_lane(L, g, axial, a, sh[warp], g9);
                    spz_rtz9(g9, s1, c1, s2, c2);
                    const float2 k0 = csub(g9[7], g9[5]), k1 = csub(g9[2], g9[6]), k2 = csub(g9[3], g9[1]);
                    acc[6] += ex * k0.x - ey * k0.y;
                    acc[7] += ex * k1.x - ey * k1.y;
                    acc[8] += ex * k2.x - ey * k2.y;
                }
            }
            __syncwarp();
        }
        const float w = active ? rec_w[(int64_t)r * NPE + lane] : 0.f;
        const bool use = active && fabsf(w) >= 1e-10f;  // SolidElement.cpp:262 skips tiny weights
#pragma unroll
        for (int k = 0; k < 9; k++) {
            float v = use ? w * acc[k] : 0.f;
            for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
            if (lane == 0) red[warp][k] = v;
        }
        __syncthreads();
        if (threadIdx.x < 9) {
            const int k = threadIdx.x;
            const float v = red[0][k] + red[1][k] + red[2][k] + red[3][k];
            if (k < 6 && sslot >= 0) strain_out[((int64_t)t * nst + sslot) * 6 + k] = v;
            if (k >= 6 && cslot >= 0) curl_out[((int64_t)t * ncu + cslot) * 3 + (k - 6)] = v;
        }
        __syncthreads();
    }
}

void launch_record_strain_curl(const PointTable &P, const ElemTable &T, const float2 *su, const int32_t *rec_elem,
                               const float *rec_phi, const float *rec_w, const int32_t *list, int n,
                               float *strain_out, int nst, float *curl_out, int ncu, int cap, const int32_t *tptr,
                               int tofs, cudaStream_t s) {
    if (n <= 0) return;
    k_record_strain_curl<<<std::min(n, 152 * 8), 128, 0, s>>>(P, T, su, rec_elem, rec_phi, rec_w, list, n,
                                                               strain_out, nst, curl_out, ncu, cap, tptr, tofs);
}

void set_g_matrices(const float *g_gll, const float *g_glj, cudaStream_t s) {
    cudaMemcpyToSymbolAsync(c_G, g_gll, 25 * sizeof(float), 0, cudaMemcpyHostToDevice, s);
    cudaMemcpyToSymbolAsync(c_G, g_glj, 25 * sizeof(float), 25 * sizeof(float),
                            cudaMemcpyHostToDevice, s);
    set_g_matrices_phys(g_gll, g_glj, s);
}

constexpr int FW_WARPS = 8;   // warps per CTA in the Fourier-space kernels
constexpr int QSCR = 14 * 25;  // per-warp scratch (float2) for grad/quad

// scatterDisplToElement (SolidPoint.cpp:175-195): orders above the point's Nu, and its
// Nyquist order, read as zero.
__device__ __forceinline__ void load_solid_u(const PointTable &P, const float2 *su, int pt, int a,
                                             float2 u[3]) {
    int pnr = P.nr[pt];
    int plim = pnr / 2 - (pnr % 2 == 0);
    if (a <= plim) {
        const float2 *s = su + P.sofs[pt] + (int64_t)a * 3;
        u[0] = s[0];
        u[1] = s[1];
        u[2] = s[2];
    } else {
        u[0] = u[1] = u[2] = make_float2(0.f, 0.f);
    }
}
__device__ __forceinline__ float2 load_fluid_u(const PointTable &P, const float2 *fu, int pt, int a) {
    int pnr = P.nr[pt];
    int plim = pnr / 2 - (pnr % 2 == 0);
    return a <= plim ? fu[P.fofs[pt] + a] : make_float2(0.f, 0.f);
}

// ------------------------------------------------------------------------------------
// Fourier-space solid elements: warp per (element, block of FW_OB orders)
// ------------------------------------------------------------------------------------
// A point's displacement block and order limit, read once per work item.
struct UPoint {
    const float2 *base;
    int plim;
    __device__ __forceinline__ void init(const PointTable &P, const float2 *u, int64_t ofs, int pt) {
        const int pnr = P.nr[pt];
        plim = pnr / 2 - (pnr % 2 == 0);
        base = u + ofs;
    }
};

__global__ void __launch_bounds__(FW_WARPS * 32)
    k_elem_fourier_solid(ElemTable T, PointTable P, const float2 *__restrict__ su,
                         const int2 *__restrict__ items, int nitems, SLS sls) {
    __shared__ float2 scr[FW_WARPS][QSCR];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    float2 *q = scr[warp];
    const bool active = lane < NPE;
    const int p = active ? lane : 0;
    for (int it = blockIdx.x * FW_WARPS + warp; it < nitems; it += gridDim.x * FW_WARPS) {
        const int e = items[it].x, a0 = items[it].y;
        const int flags = T.flags[e];
        const bool axial = flags & EF_AXIAL;
        const int nr = T.nr[e], nu = nr / 2, n = nu + 1, lim = nu - (nr % 2 == 0);
        const int a1 = min(a0 + FW_OB, n);
        const int mat = ef_mat(flags), att = ef_att(flags);
        const bool tiso = (mat == 1 || mat == 2);
        // the element's per-lane constants, kept over the item's orders
        LaneOps L;
        L.init(p, axial);
        Geo g;
        g.load(T.geo + (int64_t)e * 125, p);
        float s1 = 0.f, c1 = 0.f, s2 = 0.f, c2 = 0.f;
        if (tiso) {
            const float *tr = T.trig + (int64_t)e * 100;
            s1 = tr[p];
            c1 = tr[25 + p];
            s2 = tr[50 + p];
            c2 = tr[75 + p];
        }
        const float *md = T.moduli + T.mofs[e];
        const int npa = att == 2 ? 4 : NPE;
        const int qq = att == 2 ? cg4_index(p) : p;
        float dk = 0.f, dm = 0.f;
        if (att && qq >= 0) {
            const float *am = T.attm + T.aofs[e];
            dk = am[qq];
            dm = am[npa + qq];
        }
        const int pt = T.pts[e * NPE + p];
        UPoint up;
        up.init(P, su, P.sofs[pt], pt);
        float2 un[3] = {make_float2(0.f, 0.f), make_float2(0.f, 0.f), make_float2(0.f, 0.f)};
        if (active && a0 <= up.plim) {
            const float2 *s = up.base + (int64_t)a0 * 3;
            un[0] = s[0];
            un[1] = s[1];
            un[2] = s[2];
        }
        float2 *ef = T.ef + T.efofs[e] + (int64_t)p * n * 3;
        for (int a = a0; a < a1; a++) {
            if (active) {
                q[p] = un[0];
                q[25 + p] = un[1];
                q[50 + p] = un[2];
                // the next order's displacement is in flight while this one is worked on
                un[0] = un[1] = un[2] = make_float2(0.f, 0.f);
                if (a + 1 < a1 && a + 1 <= up.plim) {
                    const float2 *s = up.base + (int64_t)(a + 1) * 3;
                    un[0] = s[0];
                    un[1] = s[1];
                    un[2] = s[2];
                }
            }
            __syncwarp();
            float2 eps[6], sig[6];
#pragma unroll
            for (int c = 0; c < 6; c++) eps[c] = make_float2(0.f, 0.f);
            if (active && a <= lim) grad6_lane(L, g, axial, a, q, eps);
            __syncwarp();
            if (active) {
                if (tiso) spz_rtz(eps, s1, c1, s2, c2);
                elastic(mat, eps, sig, [&](int k) { return md[k * NPE + p]; });
                if (att && qq >= 0) {
                    float2 *mem = reinterpret_cast<float2 *>(T.mem + T.memofs[e]);
                    const int64_t sl = (int64_t)n * 6 * npa;
                    float2 *R = mem + (int64_t)a * 6 * npa + qq;
                    float2 *SR = R + sls.nsls * sl;
                    for (int l = 0; l < sls.nsls; l++)
#pragma unroll
                        for (int c = 0; c < 6; c++) sig[c] = csub(sig[c], R[l * sl + c * npa]);
                    sls_update(sls, R, SR, sl, (int64_t)npa, eps, dk, dm);
                }
                if (tiso) rtz_spz(sig, s1, c1, s2, c2);
            }
            float2 f[3];
            quad6_lane(L, g, axial, a, sig, q, active && a <= lim, f);
            if (active) {
                float2 *o = ef + (int64_t)a * 3;
                if (a <= lim) {
                    o[0] = f[0];
                    o[1] = f[1];
                    o[2] = f[2];
                } else {
                    o[0] = o[1] = o[2] = make_float2(0.f, 0.f);
                }
            }
            __syncwarp();  // the scratch is rewritten by the next order
        }
    }
}

// Fourier-space fluid elements (FluidElement.cpp:333-355 with Acoustic1D.cpp:8-16): warp
// per (element, block of FW_OB orders), as the solid kernel
__global__ void __launch_bounds__(FW_WARPS * 32)
    k_elem_fourier_fluid(ElemTable T, PointTable P, const float2 *__restrict__ fu,
                         const int2 *__restrict__ items, int nitems) {
    __shared__ float2 scr[FW_WARPS][QSCR];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    float2 *q = scr[warp];
    const bool active = lane < NPE;
    const int p = active ? lane : 0;
    for (int it = blockIdx.x * FW_WARPS + warp; it < nitems; it += gridDim.x * FW_WARPS) {
        const int e = items[it].x, a0 = items[it].y;
        const bool axial = T.flags[e] & EF_AXIAL;
        const int nr = T.nr[e], nu = nr / 2, n = nu + 1, lim = nu - (nr % 2 == 0);
        const int a1 = min(a0 + FW_OB, n);
        LaneOps L;
        L.init(p, axial);
        Geo g;
        g.load(T.geo + (int64_t)e * 125, p);
        const float K = active ? T.moduli[T.mofs[e] + p] : 0.f;
        const int pt = T.pts[e * NPE + p];
        UPoint up;
        up.init(P, fu, P.fofs[pt], pt);
        float2 un = (active && a0 <= up.plim) ? up.base[a0] : make_float2(0.f, 0.f);
        float2 *ef = T.ef + T.efofs[e] + (int64_t)p * n;
        for (int a = a0; a < a1; a++) {
            if (active) {
                q[p] = un;
                un = (a + 1 < a1 && a + 1 <= up.plim) ? up.base[a + 1] : make_float2(0.f, 0.f);
            }
            __syncwarp();
            float2 eps[3] = {make_float2(0.f, 0.f), make_float2(0.f, 0.f), make_float2(0.f, 0.f)};
            if (active && a <= lim) grad1_lane(L, g, axial, a, q, eps);
            __syncwarp();
            float2 sig[3];
#pragma unroll
            for (int c = 0; c < 3; c++) sig[c] = cscale(K, eps[c]);
            float2 f;
            quad1_lane(L, g, axial, a, sig, q, active && a <= lim, f);
            if (active) ef[a] = a <= lim ? f : make_float2(0.f, 0.f);
            __syncwarp();
        }
    }
}

// ------------------------------------------------------------------------------------
// Particle relabelling.  PRT_1D elements (1-D material, X per point) stay in Fourier space:
// warp per (element, order), grad9 -> RTZ -> undulated strain -> stress (+ SLS on the
// undulated strain) -> back -> SPZ -> quad9 (SolidElement.cpp:404-443); fluids likewise
// with the three-component gradient (FluidElement.cpp:333-355).  PRT elements always
// rotate to RTZ (mInTIso = mHasPRT).
// ------------------------------------------------------------------------------------
__global__ void __launch_bounds__(FW_WARPS * 32)
    k_elem_prt1_solid(ElemTable T, PointTable P, const float2 *__restrict__ su, const int2 *__restrict__ items,
                      int nitems, SLS sls) {
    __shared__ float2 scr[FW_WARPS][QSCR];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    float2 *q = scr[warp];
    const bool active = lane < NPE;
    const int p = active ? lane : 0;
    for (int it = blockIdx.x * FW_WARPS + warp; it < nitems; it += gridDim.x * FW_WARPS) {
        const int e = items[it].x, a = items[it].y;
        const int flags = T.flags[e];
        const bool axial = flags & EF_AXIAL;
        const int nr = T.nr[e], nu = nr / 2, n = nu + 1, lim = nu - (nr % 2 == 0);
        const int mat = ef_mat(flags), att = ef_att(flags);
        LaneOps L;
        L.init(p, axial);
        Geo g;
        g.load(T.geo + (int64_t)e * 125, p);
        if (active) {
            float2 u[3];
            load_solid_u(P, su, T.pts[e * NPE + p], a, u);
            q[p] = u[0];
            q[25 + p] = u[1];
            q[50 + p] = u[2];
        }
        __syncwarp();
        float2 g9[9], s9[9];
#pragma unroll
        for (int c = 0; c < 9; c++) g9[c] = s9[c] = make_float2(0.f, 0.f);
        if (active && a <= lim) grad9_lane(L, g, axial, a, q, g9);
        __syncwarp();
        if (active) {
            const float *tr = T.trig + (int64_t)e * 100;
            const float s1 = tr[p], c1 = tr[25 + p], s2 = tr[50 + p], c2 = tr[75 + p];
            spz_rtz9(g9, s1, c1, s2, c2);
            const float *xp = T.prtx + T.prtofs[e];
            auto xf = [&](int k) { return xp[k * NPE + p]; };
            float2 und[6], sig[6];
            prt_s2u(g9, und, xf);
            const float *md = T.moduli + T.mofs[e];
            elastic(mat, und, sig, [&](int k) { return md[k * NPE + p]; });
            if (att) {
                const int npa = att == 2 ? 4 : NPE;
                const int qq = att == 2 ? cg4_index(p) : p;
                if (qq >= 0) {
                    float2 *mem = reinterpret_cast<float2 *>(T.mem + T.memofs[e]);
                    const int64_t sl = (int64_t)n * 6 * npa;
                    float2 *R = mem + (int64_t)a * 6 * npa + qq;
                    float2 *SR = R + sls.nsls * sl;
                    for (int l = 0; l < sls.nsls; l++)
#pragma unroll
                        for (int c = 0; c < 6; c++) sig[c] = csub(sig[c], R[l * sl + c * npa]);
                    const float *am = T.attm + T.aofs[e];
                    sls_update(sls, R, SR, sl, (int64_t)npa, und, am[qq], am[npa + qq]);
                }
            }
            prt_u2s(sig, s9, xf);
            rtz_spz9(s9, s1, c1, s2, c2);
        }
        float2 f[3];
        quad9_lane(L, g, axial, a, s9, q, active && a <= lim, f);
        if (active) {
            float2 *ef = T.ef + T.efofs[e] + ((int64_t)p * n + a) * 3;
            const bool on = a <= lim;
            ef[0] = on ? f[0] : make_float2(0.f, 0.f);
            ef[1] = on ? f[1] : make_float2(0.f, 0.f);
            ef[2] = on ? f[2] : make_float2(0.f, 0.f);
        }
    }
}

__global__ void __launch_bounds__(FW_WARPS * 32)
    k_elem_prt1_fluid(ElemTable T, PointTable P, const float2 *__restrict__ fu, const int2 *__restrict__ items,
                      int nitems) {
    __shared__ float2 scr[FW_WARPS][QSCR];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    float2 *q = scr[warp];
    const bool active = lane < NPE;
    const int p = active ? lane : 0;
    for (int it = blockIdx.x * FW_WARPS + warp; it < nitems; it += gridDim.x * FW_WARPS) {
        const int e = items[it].x, a = items[it].y;
        const bool axial = T.flags[e] & EF_AXIAL;
        const int nr = T.nr[e], nu = nr / 2, n = nu + 1, lim = nu - (nr % 2 == 0);
        LaneOps L;
        L.init(p, axial);
        Geo g;
        g.load(T.geo + (int64_t)e * 125, p);
        if (active) q[p] = load_fluid_u(P, fu, T.pts[e * NPE + p], a);
        __syncwarp();
        float2 v[3] = {make_float2(0.f, 0.f), make_float2(0.f, 0.f), make_float2(0.f, 0.f)};
        if (active && a <= lim) grad1_lane(L, g, axial, a, q, v);
        __syncwarp();
        if (active) {
            const float *tr = T.trig + (int64_t)e * 100;
            const float s1 = tr[p], c1 = tr[25 + p];
            spz_rtz3(v, s1, c1);
            const float *xp = T.prtx + T.prtofs[e];
            auto xf = [&](int k) { return xp[k * NPE + p]; };
            prt_s2u_fluid(v, xf);
            const float K = T.moduli[T.mofs[e] + p];
#pragma unroll
            for (int c = 0; c < 3; c++) v[c] = cscale(K, v[c]);
            prt_u2s_fluid(v, xf);
            rtz_spz3(v, s1, c1);
        }
        float2 f;
        quad1_lane(L, g, axial, a, v, q, active && a <= lim, f);
        if (active) T.ef[T.efofs[e] + (int64_t)p * n + a] = a <= lim ? f : make_float2(0.f, 0.f);
    }
}

// PRT_3D elements (3-D material, X per sample): the gradient of every order, rotated to
// RTZ, goes to a Fourier-space scratch w [alpha][nc][25] (k_prt3_grad); k_prt3_fft
// (ax3d_phys.cu, on the element pass's transforms) takes it to the nr samples, relabels,
// computes the stress (+ SLS) and the relabelled-back stress per sample and transforms
// back into w (PRT_3D.cpp with FieldFFT's C2R / R2C x 1/nr); the divergence of every
// order follows (k_prt3_quad).
template <bool SOLID>
__global__ void __launch_bounds__(FW_WARPS * 32)
    k_prt3_grad(ElemTable T, PointTable P, const float2 *__restrict__ u, const int2 *__restrict__ items, int nitems) {
    constexpr int NC = SOLID ? 9 : 3;
    __shared__ float2 scr[FW_WARPS][QSCR];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    float2 *q = scr[warp];
    const bool active = lane < NPE;
    const int p = active ? lane : 0;
    for (int it = blockIdx.x * FW_WARPS + warp; it < nitems; it += gridDim.x * FW_WARPS) {
        const int e = items[it].x, a = items[it].y;
        const bool axial = T.flags[e] & EF_AXIAL;
        const int nr = T.nr[e], lim = nr / 2 - (nr % 2 == 0);
        LaneOps L;
        L.init(p, axial);
        Geo g;
        g.load(T.geo + (int64_t)e * 125, p);
        if (active) {
            if (SOLID) {
                float2 uu[3];
                load_solid_u(P, u, T.pts[e * NPE + p], a, uu);
                q[p] = uu[0];
                q[25 + p] = uu[1];
                q[50 + p] = uu[2];
            } else {
                q[p] = load_fluid_u(P, u, T.pts[e * NPE + p], a);
            }
        }
        __syncwarp();
        float2 v[NC];
#pragma unroll
        for (int c = 0; c < NC; c++) v[c] = make_float2(0.f, 0.f);
        if (active && a <= lim) {
            const float *tr = T.trig + (int64_t)e * 100;
            if constexpr (SOLID) {
                grad9_lane(L, g, axial, a, q, v);
                spz_rtz9(v, tr[p], tr[25 + p], tr[50 + p], tr[75 + p]);
            } else {
                grad1_lane(L, g, axial, a, q, v);
                spz_rtz3(v, tr[p], tr[25 + p]);
            }
        }
        __syncwarp();
        if (active) {
            float2 *w = T.w + T.wofs[e] + (int64_t)a * NC * NPE + p;
#pragma unroll
            for (int c = 0; c < NC; c++) w[c * NPE] = v[c];
        }
    }
}

template <bool SOLID>
__global__ void __launch_bounds__(FW_WARPS * 32)
    k_prt3_quad(ElemTable T, const int2 *__restrict__ items, int nitems) {
    constexpr int NC = SOLID ? 9 : 3;
    __shared__ float2 scr[FW_WARPS][QSCR];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    float2 *q = scr[warp];
    const bool active = lane < NPE;
    const int p = active ? lane : 0;
    for (int it = blockIdx.x * FW_WARPS + warp; it < nitems; it += gridDim.x * FW_WARPS) {
        const int e = items[it].x, a = items[it].y;
        const bool axial = T.flags[e] & EF_AXIAL;
        const int nr = T.nr[e], n = nr / 2 + 1, lim = nr / 2 - (nr % 2 == 0);
        LaneOps L;
        L.init(p, axial);
        Geo g;
        g.load(T.geo + (int64_t)e * 125, p);
        float2 v[NC];
#pragma unroll
        for (int c = 0; c < NC; c++) v[c] = make_float2(0.f, 0.f);
        if (active) {
            const float2 *w = T.w + T.wofs[e] + (int64_t)a * NC * NPE + p;
#pragma unroll
            for (int c = 0; c < NC; c++) v[c] = w[c * NPE];
            const float *tr = T.trig + (int64_t)e * 100;
            if constexpr (SOLID) rtz_spz9(v, tr[p], tr[25 + p], tr[50 + p], tr[75 + p]);
            else rtz_spz3(v, tr[p], tr[25 + p]);
        }
        if constexpr (SOLID) {
            float2 f[3];
            quad9_lane(L, g, axial, a, v, q, active && a <= lim, f);
            if (active) {
                float2 *ef = T.ef + T.efofs[e] + ((int64_t)p * n + a) * 3;
                const bool on = a <= lim;
                ef[0] = on ? f[0] : make_float2(0.f, 0.f);
                ef[1] = on ? f[1] : make_float2(0.f, 0.f);
                ef[2] = on ? f[2] : make_float2(0.f, 0.f);
            }
        } else {
            float2 f;
            quad1_lane(L, g, axial, a, v, q, active && a <= lim, f);
            if (active) T.ef[T.efofs[e] + (int64_t)p * n + a] = a <= lim ? f : make_float2(0.f, 0.f);
        }
    }
}

static int fw_blocks(int nitems) {
    const int b = (nitems + FW_WARPS - 1) / FW_WARPS;
    return b > 152 * 16 ? 152 * 16 : b;
}

void launch_elem_prt1(bool solid, const ElemTable &T, const PointTable &P, const float2 *u, const int2 *items,
                      int nitems, const SLS &sls, cudaStream_t s) {
    if (nitems <= 0) return;
    if (solid) k_elem_prt1_solid<<<fw_blocks(nitems), FW_WARPS * 32, 0, s>>>(T, P, u, items, nitems, sls);
    else k_elem_prt1_fluid<<<fw_blocks(nitems), FW_WARPS * 32, 0, s>>>(T, P, u, items, nitems);
}

void launch_elem_prt3(bool solid, const ElemTable &T, const PointTable &P, const float2 *u, const int2 *items,
                      int nitems, const int32_t *elems, int nelem, int lbuf_max, const PhysTables &X, const SLS &sls,
                      cudaStream_t s) {
    if (nitems <= 0 || nelem <= 0) return;
    if (solid) {
        k_prt3_grad<true><<<fw_blocks(nitems), FW_WARPS * 32, 0, s>>>(T, P, u, items, nitems);
        launch_prt3_fft(true, T, elems, nelem, lbuf_max, X, sls, s);
        k_prt3_quad<true><<<fw_blocks(nitems), FW_WARPS * 32, 0, s>>>(T, items, nitems);
    } else {
        k_prt3_grad<false><<<fw_blocks(nitems), FW_WARPS * 32, 0, s>>>(T, P, u, items, nitems);
        launch_prt3_fft(false, T, elems, nelem, lbuf_max, X, sls, s);
        k_prt3_quad<false><<<fw_blocks(nitems), FW_WARPS * 32, 0, s>>>(T, items, nitems);
    }
}

void launch_elem_fourier_solid(const ElemTable &T, const PointTable &P, const float2 *su,
                               const int2 *items, int nitems, const SLS &sls, cudaStream_t s) {
    if (nitems <= 0) return;
    int blocks = (nitems + FW_WARPS - 1) / FW_WARPS;
    if (blocks > 152 * 16) blocks = 152 * 16;
    k_elem_fourier_solid<<<blocks, FW_WARPS * 32, 0, s>>>(T, P, su, items, nitems, sls);
}
void launch_elem_fourier_fluid(const ElemTable &T, const PointTable &P, const float2 *fu,
                               const int2 *items, int nitems, cudaStream_t s) {
    if (nitems <= 0) return;
    int blocks = (nitems + FW_WARPS - 1) / FW_WARPS;
    if (blocks > 152 * 16) blocks = 152 * 16;
    k_elem_fourier_fluid<<<blocks, FW_WARPS * 32, 0, s>>>(T, P, fu, items, nitems);
}

void init_kernel_attributes() {
    init_phys_attributes();
}

}  // namespace ax3d
