// ax3d_elem_ops.cuh -- per-GLL-point element operators shared by the element kernels.
//
// One warp evaluates one Fourier order of one element: lane p (< 25) owns GLL point
// p = ipol * 5 + jpol.  The derivative matrices live in registers (the lane's rows and
// columns), the element's displacement / stress of that order in a per-warp shared
// scratch.  The arithmetic restates SOLVER/src/core/element/grad/Gradient.cpp:206-317
// (solid) and :26-82 (fluid); the axial L'Hopital terms use the linearity of G^T so
// that v = i*alpha*u combinations need no extra loads.
#pragma once

#include "ax3d_common.cuh"

namespace ax3d {

// G(i,j) = l_i'(xi_j); [0] = GLL, [1] = GLJ(0,1)
// Set once per device by set_g_matrices (each translation unit has its own copy;
// only the element kernels read it).
static __constant__ float c_G[2][25];

struct LaneOps {
    float gxc[5];  // G_xi[k][i]  (column i)  -> (G_xi^T u)(i,j)
    float gec[5];  // G_eta[k][j] (column j)  -> (u G_eta)(i,j)
    float gxr[5];  // G_xi[i][k]  (row i)     -> (G_xi X)(i,j)
    float ger[5];  // G_eta[j][k] (row j)     -> (Y G_eta^T)(i,j)
    int i, j;
    __device__ void init(int p, bool axial) { init_from(p, c_G[axial ? 1 : 0], c_G[0]); }
    // Gx: G of the xi direction (GLJ on axial elements), Ge: G of eta (GLL), both [25].
    __device__ void init_from(int p, const float *Gx, const float *Ge) {
        i = p / 5;
        j = p - 5 * (p / 5);
#pragma unroll
        for (int k = 0; k < 5; k++) {
            gxc[k] = Gx[k * 5 + i];
            gec[k] = Ge[k * 5 + j];
            gxr[k] = Gx[i * 5 + k];
            ger[k] = Ge[j * 5 + k];
        }
    }
};

struct Geo {
    float dsdxii, dsdeta, dzdxii, dzdeta, inv_s;
    __device__ void load(const float *g, int p) {
        dsdxii = g[p];
        dsdeta = g[25 + p];
        dzdxii = g[50 + p];
        dzdeta = g[75 + p];
        inv_s = g[100 + p];
    }
};

// (G_xi^T u)(i,j) and (u G_eta)(i,j) of a [25] complex field in shared memory
__device__ __forceinline__ void gu_ug(const LaneOps &L, const float2 *u, float2 &GU, float2 &UG) {
    GU = make_float2(0.f, 0.f);
    UG = make_float2(0.f, 0.f);
#pragma unroll
    for (int k = 0; k < 5; k++) {
        float2 a = u[k * 5 + L.j];
        float2 b = u[L.i * 5 + k];
        GU.x += L.gxc[k] * a.x;
        GU.y += L.gxc[k] * a.y;
        UG.x += b.x * L.gec[k];
        UG.y += b.y * L.gec[k];
    }
}

// computeGrad6 at one point for order alpha; su = [3][25] displacement of this order.
__device__ __forceinline__ void grad6_lane(const LaneOps &L, const Geo &g, bool axial, int alpha,
                                          const float2 *su, float2 eps[6]) {
    const int p = L.i * 5 + L.j;
    float2 GU0, UG0, GU1, UG1, GU2, UG2;
    gu_ug(L, su, GU0, UG0);
    gu_ug(L, su + 25, GU1, UG1);
    gu_ug(L, su + 50, GU2, UG2);
    const float a = (float)alpha;
    float2 u0 = su[p], u1 = su[25 + p], u2 = su[50 + p];
    float2 v0 = cadd(u0, cimul(a, u1));
    float2 v1 = csub(cimul(a, u0), u1);
    float2 v2 = cimul(a, u2);
    eps[0] = cadd(cscale(g.dzdeta, GU0), cscale(g.dzdxii, UG0));
    eps[1] = cscale(g.inv_s, v0);
    eps[2] = cadd(cscale(g.dsdeta, GU2), cscale(g.dsdxii, UG2));
    eps[3] = cadd(cadd(cscale(g.dsdeta, GU1), cscale(g.dsdxii, UG1)), cscale(g.inv_s, v2));
    eps[4] = cadd(cadd(cadd(cscale(g.dsdeta, GU0), cscale(g.dsdxii, UG0)), cscale(g.dzdeta, GU2)),
                  cscale(g.dzdxii, UG2));
    eps[5] = cadd(cadd(cscale(g.dzdeta, GU1), cscale(g.dzdxii, UG1)), cscale(g.inv_s, v1));
    if (axial && L.i == 0) {
        // row 0: += DzDeta * (G_xi^T v)(0,j)   (Gradient.cpp:245-248)
        float2 gv0 = cadd(GU0, cimul(a, GU1));
        float2 gv1 = csub(cimul(a, GU0), GU1);
        float2 gv2 = cimul(a, GU2);
        eps[1] = cadd(eps[1], cscale(g.dzdeta, gv0));
        eps[5] = cadd(eps[5], cscale(g.dzdeta, gv1));
        eps[3] = cadd(eps[3], cscale(g.dzdeta, gv2));
        if (alpha == 1) {  // Gradient.cpp:249-252
            float2 h0 = cadd(UG0, cimul(a, UG1));
            float2 h1 = csub(cimul(a, UG0), UG1);
            eps[1] = cadd(eps[1], cscale(g.dzdxii, h0));
            eps[5] = cadd(eps[5], cscale(g.dzdxii, h1));
        }
    }
}

// computeGrad9 at one point for order alpha (Gradient.cpp:84-152): g[3c + d] = d-th
// derivative (s, phi, z) of component c, with grad6's axial rows.
__device__ __forceinline__ void grad9_lane(const LaneOps &L, const Geo &g, bool axial, int alpha,
                                          const float2 *su, float2 g9[9]) {
    const int p = L.i * 5 + L.j;
    float2 GU[3], UG[3];
    gu_ug(L, su, GU[0], UG[0]);
    gu_ug(L, su + 25, GU[1], UG[1]);
    gu_ug(L, su + 50, GU[2], UG[2]);
    const float a = (float)alpha;
    float2 u0 = su[p], u1 = su[25 + p], u2 = su[50 + p];
    float2 v0 = cadd(u0, cimul(a, u1));
    float2 v1 = csub(cimul(a, u0), u1);
    float2 v2 = cimul(a, u2);
#pragma unroll
    for (int c = 0; c < 3; c++) {
        g9[3 * c] = cadd(cscale(g.dzdeta, GU[c]), cscale(g.dzdxii, UG[c]));
        g9[3 * c + 2] = cadd(cscale(g.dsdeta, GU[c]), cscale(g.dsdxii, UG[c]));
    }
    g9[1] = cscale(g.inv_s, v1);
    g9[4] = cscale(g.inv_s, v0);
    g9[7] = cscale(g.inv_s, v2);
    if (axial && L.i == 0) {
        g9[4] = cadd(g9[4], cscale(g.dzdeta, cadd(GU[0], cimul(a, GU[1]))));
        g9[1] = cadd(g9[1], cscale(g.dzdeta, csub(cimul(a, GU[0]), GU[1])));
        g9[7] = cadd(g9[7], cscale(g.dzdeta, cimul(a, GU[2])));
        if (alpha == 1) {
            g9[4] = cadd(g9[4], cscale(g.dzdxii, cadd(UG[0], cimul(a, UG[1]))));
            g9[1] = cadd(g9[1], cscale(g.dzdxii, csub(cimul(a, UG[0]), UG[1])));
        }
    }
}

// computeQuad6 at one point for order beta.  Each lane first writes its X, Y, g terms
// into the scratch q ([14][25] complex), then reads its neighbours'.  Must be called by
// all lanes of the warp (lanes >= 25 pass active = false).
__device__ __forceinline__ void quad6_lane(const LaneOps &L, const Geo &g, bool axial, int beta,
                                           const float2 sig[6], float2 *q, bool active,
                                           float2 f[3]) {
    const int p = L.i * 5 + L.j;
    const float b = -(float)beta;
    if (active) {
        float2 g0 = cadd(sig[1], cimul(b, sig[5]));
        float2 g1 = csub(cimul(b, sig[1]), sig[5]);
        float2 g2 = cimul(b, sig[3]);
        q[0 * 25 + p] = cadd(cscale(g.dzdeta, sig[0]), cscale(g.dsdeta, sig[4]));  // X0
        q[1 * 25 + p] = cadd(cscale(g.dzdeta, sig[5]), cscale(g.dsdeta, sig[3]));  // X1
        q[2 * 25 + p] = cadd(cscale(g.dzdeta, sig[4]), cscale(g.dsdeta, sig[2]));  // X2
        q[3 * 25 + p] = cadd(cscale(g.dzdxii, sig[0]), cscale(g.dsdxii, sig[4]));  // Y0
        q[4 * 25 + p] = cadd(cscale(g.dzdxii, sig[5]), cscale(g.dsdxii, sig[3]));  // Y1
        q[5 * 25 + p] = cadd(cscale(g.dzdxii, sig[4]), cscale(g.dsdxii, sig[2]));  // Y2
        q[6 * 25 + p] = g0;
        q[7 * 25 + p] = g1;
        q[8 * 25 + p] = g2;
        q[9 * 25 + p] = cscale(g.dzdeta, g0);   // DzDeta o g (axial column term)
        q[10 * 25 + p] = cscale(g.dzdeta, g1);
        q[11 * 25 + p] = cscale(g.dzdeta, g2);
        q[12 * 25 + p] = cscale(g.dzdxii, g0);  // DzDxii o g (axial, beta = 1)
        q[13 * 25 + p] = cscale(g.dzdxii, g1);
    }
    __syncwarp();
    if (active) {
#pragma unroll
        for (int c = 0; c < 3; c++) {
            float2 acc = make_float2(0.f, 0.f), acc2 = make_float2(0.f, 0.f);
            const float2 *X = q + c * 25, *Y = q + (3 + c) * 25;
#pragma unroll
            for (int k = 0; k < 5; k++) {
                float2 x = X[k * 5 + L.j];
                float2 y = Y[L.i * 5 + k];
                acc.x += L.gxr[k] * x.x;
                acc.y += L.gxr[k] * x.y;
                acc2.x += y.x * L.ger[k];
                acc2.y += y.y * L.ger[k];
            }
            f[c] = cadd(cadd(acc, acc2), cscale(g.inv_s, q[(6 + c) * 25 + p]));
            if (axial) {
                // += G_xi(:,0) * (DzDeta o g)(0,:)   (Gradient.cpp:300-303)
                f[c] = cadd(f[c], cscale(L.gxr[0], q[(9 + c) * 25 + L.j]));
                if (beta == 1 && L.i == 0 && c < 2) {  // Gradient.cpp:304-307
                    float2 h = make_float2(0.f, 0.f);
#pragma unroll
                    for (int k = 0; k < 5; k++) {
                        float2 t = q[(12 + c) * 25 + k];
                        h.x += t.x * L.ger[k];
                        h.y += t.y * L.ger[k];
                    }
                    f[c] = cadd(f[c], h);
                }
            }
        }
    }
    __syncwarp();
}

// computeQuad9 at one point for order beta (Gradient.cpp:154-212); same scratch use as
// quad6_lane.  sig9[3c + d] pairs with grad9's u_{c,d}.
__device__ __forceinline__ void quad9_lane(const LaneOps &L, const Geo &g, bool axial, int beta,
                                           const float2 sig[9], float2 *q, bool active, float2 f[3]) {
    const int p = L.i * 5 + L.j;
    const float b = -(float)beta;
    if (active) {
        const float2 g0 = cadd(sig[4], cimul(b, sig[1]));
        const float2 g1 = csub(cimul(b, sig[4]), sig[1]);
        const float2 g2 = cimul(b, sig[7]);
#pragma unroll
        for (int c = 0; c < 3; c++) {
            q[c * 25 + p] = cadd(cscale(g.dzdeta, sig[3 * c]), cscale(g.dsdeta, sig[3 * c + 2]));
            q[(3 + c) * 25 + p] = cadd(cscale(g.dzdxii, sig[3 * c]), cscale(g.dsdxii, sig[3 * c + 2]));
        }
        q[6 * 25 + p] = g0;
        q[7 * 25 + p] = g1;
        q[8 * 25 + p] = g2;
        q[9 * 25 + p] = cscale(g.dzdeta, g0);
        q[10 * 25 + p] = cscale(g.dzdeta, g1);
        q[11 * 25 + p] = cscale(g.dzdeta, g2);
        q[12 * 25 + p] = cscale(g.dzdxii, g0);
        q[13 * 25 + p] = cscale(g.dzdxii, g1);
    }
    __syncwarp();
    if (active) {
#pragma unroll
        for (int c = 0; c < 3; c++) {
            float2 acc = make_float2(0.f, 0.f), acc2 = make_float2(0.f, 0.f);
            const float2 *X = q + c * 25, *Y = q + (3 + c) * 25;
#pragma unroll
            for (int k = 0; k < 5; k++) {
                float2 x = X[k * 5 + L.j];
                float2 y = Y[L.i * 5 + k];
                acc.x += L.gxr[k] * x.x;
                acc.y += L.gxr[k] * x.y;
                acc2.x += y.x * L.ger[k];
                acc2.y += y.y * L.ger[k];
            }
            f[c] = cadd(cadd(acc, acc2), cscale(g.inv_s, q[(6 + c) * 25 + p]));
            if (axial) {
                f[c] = cadd(f[c], cscale(L.gxr[0], q[(9 + c) * 25 + L.j]));
                if (beta == 1 && L.i == 0 && c < 2) {
                    float2 h = make_float2(0.f, 0.f);
#pragma unroll
                    for (int k = 0; k < 5; k++) {
                        float2 t = q[(12 + c) * 25 + k];
                        h.x += t.x * L.ger[k];
                        h.y += t.y * L.ger[k];
                    }
                    f[c] = cadd(f[c], h);
                }
            }
        }
    }
    __syncwarp();
}

// computeGrad (scalar potential) at one point (Gradient.cpp:26-56); su = [25].
__device__ __forceinline__ void grad1_lane(const LaneOps &L, const Geo &g, bool axial, int alpha,
                                          const float2 *su, float2 eps[3]) {
    const int p = L.i * 5 + L.j;
    float2 GU, UG;
    gu_ug(L, su, GU, UG);
    const float a = (float)alpha;
    float2 v = cimul(a, su[p]);
    eps[0] = cadd(cscale(g.dzdeta, GU), cscale(g.dzdxii, UG));
    eps[1] = cscale(g.inv_s, v);
    eps[2] = cadd(cscale(g.dsdeta, GU), cscale(g.dsdxii, UG));
    if (axial && L.i == 0 && alpha > 0) eps[1] = cadd(eps[1], cscale(g.dzdeta, cimul(a, GU)));
}

// computeQuad (scalar) at one point (Gradient.cpp:58-82); scratch q = [5][25].
__device__ __forceinline__ void quad1_lane(const LaneOps &L, const Geo &g, bool axial, int beta,
                                           const float2 sig[3], float2 *q, bool active, float2 &f) {
    const int p = L.i * 5 + L.j;
    const float b = -(float)beta;
    if (active) {
        float2 gg = cimul(b, sig[1]);
        q[0 * 25 + p] = cadd(cscale(g.dzdeta, sig[0]), cscale(g.dsdeta, sig[2]));  // X
        q[1 * 25 + p] = cadd(cscale(g.dzdxii, sig[0]), cscale(g.dsdxii, sig[2]));  // Y
        q[2 * 25 + p] = gg;
        q[3 * 25 + p] = cscale(g.dzdeta, gg);
    }
    __syncwarp();
    if (active) {
        float2 acc = make_float2(0.f, 0.f), acc2 = make_float2(0.f, 0.f);
#pragma unroll
        for (int k = 0; k < 5; k++) {
            float2 x = q[k * 5 + L.j];
            float2 y = q[25 + L.i * 5 + k];
            acc.x += L.gxr[k] * x.x;
            acc.y += L.gxr[k] * x.y;
            acc2.x += y.x * L.ger[k];
            acc2.y += y.y * L.ger[k];
        }
        f = cadd(cadd(acc, acc2), cscale(g.inv_s, q[2 * 25 + p]));
        if (axial && beta > 0) f = cadd(f, cscale(L.gxr[0], q[3 * 25 + L.j]));
    }
    __syncwarp();
}

// CrdTransTIsoSolid::transformSPZ_RTZ / transformRTZ_SPZ (CrdTransTIsoSolid.cpp:14-42)
__device__ __forceinline__ void spz_rtz(float2 u[6], float s1, float c1, float s2, float c2) {
    float2 sum02 = cadd(u[0], u[2]);
    float2 dif02 = csub(u[0], u[2]);
    float2 u3 = u[3];
    u[0] = cscale(0.5f, csub(cadd(sum02, cscale(c2, dif02)), cscale(s2, u[4])));
    u[2] = csub(sum02, u[0]);
    u[4] = cadd(cscale(c2, u[4]), cscale(s2, dif02));
    u[3] = cadd(cscale(c1, u3), cscale(s1, u[5]));
    u[5] = csub(cscale(c1, u[5]), cscale(s1, u3));
}
__device__ __forceinline__ void rtz_spz(float2 u[6], float s1, float c1, float s2, float c2) {
    float2 sum02 = cadd(u[0], u[2]);
    float2 dif02 = cscale(0.5f, csub(u[0], u[2]));
    float2 u3 = u[3];
    u[0] = cadd(cadd(cscale(0.5f, sum02), cscale(c2, dif02)), cscale(s2, u[4]));
    u[2] = csub(sum02, u[0]);
    u[4] = csub(cscale(c2, u[4]), cscale(s2, dif02));
    u[3] = csub(cscale(c1, u3), cscale(s1, u[5]));
    u[5] = cadd(cscale(c1, u[5]), cscale(s1, u3));
}

// CrdTransTIsoSolid::transformSPZ_RTZ of a nine-component gradient (CrdTransTIsoSolid.cpp:44-66)
__device__ __forceinline__ void spz_rtz9(float2 u[9], float s1, float c1, float s2, float c2) {
    const float2 sum08 = cadd(u[0], u[8]), dif08 = csub(u[0], u[8]);
    const float2 sum26 = cadd(u[2], u[6]), dif26 = csub(u[2], u[6]);
    const float2 u1 = u[1], u3 = u[3];
    u[0] = cscale(0.5f, csub(cadd(sum08, cscale(c2, dif08)), cscale(s2, sum26)));
    u[2] = cscale(0.5f, cadd(cadd(dif26, cscale(c2, sum26)), cscale(s2, dif08)));
    u[6] = csub(u[2], dif26);
    u[8] = csub(sum08, u[0]);
    u[1] = csub(cscale(c1, u1), cscale(s1, u[7]));
    u[7] = cadd(cscale(c1, u[7]), cscale(s1, u1));
    u[3] = csub(cscale(c1, u3), cscale(s1, u[5]));
    u[5] = cadd(cscale(c1, u[5]), cscale(s1, u3));
}

// CrdTransTIsoSolid::transformRTZ_SPZ of a nine-component tensor (CrdTransTIsoSolid.cpp:68-90)
__device__ __forceinline__ void rtz_spz9(float2 u[9], float s1, float c1, float s2, float c2) {
    const float2 sum08 = cadd(u[0], u[8]), dif08 = csub(u[0], u[8]);
    const float2 sum26 = cadd(u[2], u[6]), dif26 = csub(u[2], u[6]);
    const float2 u1 = u[1], u3 = u[3];
    u[0] = cscale(0.5f, cadd(cadd(sum08, cscale(c2, dif08)), cscale(s2, sum26)));
    u[2] = cscale(0.5f, csub(cadd(dif26, cscale(c2, sum26)), cscale(s2, dif08)));
    u[6] = csub(u[2], dif26);
    u[8] = csub(sum08, u[0]);
    u[1] = cadd(cscale(c1, u1), cscale(s1, u[7]));
    u[7] = csub(cscale(c1, u[7]), cscale(s1, u1));
    u[3] = cadd(cscale(c1, u3), cscale(s1, u[5]));
    u[5] = csub(cscale(c1, u[5]), cscale(s1, u3));
}
// CrdTransTIsoFluid::transformSPZ_RTZ / transformRTZ_SPZ (CrdTransTIsoFluid.cpp:14-32)
__device__ __forceinline__ void spz_rtz3(float2 u[3], float s1, float c1) {
    const float2 u0 = u[0];
    u[0] = csub(cscale(c1, u0), cscale(s1, u[2]));
    u[2] = cadd(cscale(c1, u[2]), cscale(s1, u0));
}
__device__ __forceinline__ void rtz_spz3(float2 u[3], float s1, float c1) {
    const float2 u0 = u[0];
    u[0] = cadd(cscale(c1, u0), cscale(s1, u[2]));
    u[2] = csub(cscale(c1, u[2]), cscale(s1, u0));
}

// Elastic strain -> stress at one point / sample for real (T = float) or complex
// (T = float2) values.  Isotropic1D.cpp:9-26, TransverselyIsotropic1D.cpp:9-27,
// Anisotropic1D.cpp:9-54 (3D variants identical per sample).  mod(k) = modulus k.
__device__ __forceinline__ float vadd(float a, float b) { return a + b; }
__device__ __forceinline__ float2 vadd(float2 a, float2 b) { return cadd(a, b); }
__device__ __forceinline__ float vsub(float a, float b) { return a - b; }
__device__ __forceinline__ float2 vsub(float2 a, float2 b) { return csub(a, b); }
__device__ __forceinline__ float vmul(float s, float a) { return s * a; }
__device__ __forceinline__ float2 vmul(float s, float2 a) { return cscale(s, a); }
__device__ __forceinline__ float vneg(float a) { return -a; }
__device__ __forceinline__ float2 vneg(float2 a) { return make_float2(-a.x, -a.y); }

template <typename T, typename M>
__device__ __forceinline__ void elastic(int mat, const T e[6], T s[6], M mod) {
    if (mat == 0) {
        float lam = mod(0), mu = mod(1), mu2 = 2.f * mu;
        T sii = vmul(lam, vadd(vadd(e[0], e[1]), e[2]));
        s[0] = vadd(sii, vmul(mu2, e[0]));
        s[1] = vadd(sii, vmul(mu2, e[1]));
        s[2] = vadd(sii, vmul(mu2, e[2]));
        s[3] = vmul(mu, e[3]);
        s[4] = vmul(mu, e[4]);
        s[5] = vmul(mu, e[5]);
    } else if (mat == 1) {
        float A = mod(0), C = mod(1), F = mod(2), L = mod(3), N = mod(4), N2 = 2.f * N;
        T e01 = vadd(e[0], e[1]);
        T temp = vadd(vmul(A, e01), vmul(F, e[2]));
        s[0] = vsub(temp, vmul(N2, e[1]));
        s[1] = vsub(temp, vmul(N2, e[0]));
        s[2] = vadd(vmul(C, e[2]), vmul(F, e01));
        s[3] = vmul(L, e[3]);
        s[4] = vmul(L, e[4]);
        s[5] = vmul(N, e[5]);
    } else {
        // rows of the symmetric 6x6 in the 21-vector (C11..C16, C22..C26, ..., C66)
        const int idx[6][6] = {{0, 1, 2, 3, 4, 5},      {1, 6, 7, 8, 9, 10},
                               {2, 7, 11, 12, 13, 14},  {3, 8, 12, 15, 16, 17},
                               {4, 9, 13, 16, 18, 19},  {5, 10, 14, 17, 19, 20}};
#pragma unroll
        for (int r = 0; r < 6; r++) {
            T acc = vmul(mod(idx[r][0]), e[0]);
#pragma unroll
            for (int c = 1; c < 6; c++) acc = vadd(acc, vmul(mod(idx[r][c]), e[c]));
            s[r] = acc;
        }
    }
}

// Particle relabelling (PRT_1D.cpp, PRT_3D.cpp) at one point / sample, real or complex.
// x(k) = X component k there.  sph: nine RTZ gradient components; und: six undulated
// strain components (shear doubled).
template <typename T, typename XF>
__device__ __forceinline__ void prt_s2u(const T sph[9], T und[6], XF x) {
    const float x0 = x(0), x1 = x(1), x2 = x(2), x3 = x(3);
    und[0] = vadd(vmul(x0, sph[0]), vmul(x1, sph[2]));
    und[1] = vadd(vmul(x0, sph[4]), vmul(x2, sph[5]));
    und[2] = vmul(x3, sph[8]);
    und[3] = vadd(vadd(vmul(x0, sph[7]), vmul(x2, sph[8])), vmul(x3, sph[5]));
    und[4] = vadd(vadd(vmul(x0, sph[6]), vmul(x1, sph[8])), vmul(x3, sph[2]));
    und[5] = vadd(vadd(vmul(x0, vadd(sph[3], sph[1])), vmul(x1, sph[5])), vmul(x2, sph[2]));
}
template <typename T, typename XF>
__device__ __forceinline__ void prt_u2s(const T und[6], T sph[9], XF x) {
    const float x0 = x(0), x1 = x(1), x2 = x(2), x3 = x(3);
    sph[0] = vmul(x0, und[0]);
    sph[1] = vmul(x0, und[5]);
    sph[2] = vadd(vadd(vmul(x1, und[0]), vmul(x3, und[4])), vmul(x2, und[5]));
    sph[3] = sph[1];
    sph[4] = vmul(x0, und[1]);
    sph[5] = vadd(vadd(vmul(x2, und[1]), vmul(x3, und[3])), vmul(x1, und[5]));
    sph[6] = vmul(x0, und[4]);
    sph[7] = vmul(x0, und[3]);
    sph[8] = vadd(vadd(vmul(x3, und[2]), vmul(x2, und[3])), vmul(x1, und[4]));
}
template <typename T, typename XF>
__device__ __forceinline__ void prt_s2u_fluid(T s[3], XF x) {
    const float x0 = x(0), x1 = x(1), x2 = x(2), x3 = x(3);
    s[0] = vadd(vmul(x0, s[0]), vmul(x1, s[2]));
    s[1] = vadd(vmul(x0, s[1]), vmul(x2, s[2]));
    s[2] = vmul(x3, s[2]);
}
template <typename T, typename XF>
__device__ __forceinline__ void prt_u2s_fluid(T s[3], XF x) {
    const float x0 = x(0), x1 = x(1), x2 = x(2), x3 = x(3);
    s[2] = vadd(vadd(vmul(x1, s[0]), vmul(x2, s[1])), vmul(x3, s[2]));
    s[0] = vmul(x0, s[0]);
    s[1] = vmul(x0, s[1]);
}

// SLS memory-variable update at one attenuated point (Attenuation1D_Full.cpp:30-74,
// Attenuation3D_Full.cpp:23-50; CG4 variants identical at the four coarse points).
// R points at memvar[l=0][c=0] of this point, stride_l between SLS, stride_c between
// components; SR (stressR) likewise.  The caller has already subtracted sum R from
// the stress (applyToStress).
// As sls_update, with the old stressR (sr_old) already loaded by the caller.
template <typename T>
__device__ __forceinline__ void sls_update_from(const SLS &sls, T *R, T *SR, int64_t stride_l, int64_t stride_c,
                                                const T e[6], const T sr_old[6], float dk, float dmu) {
    const float third = (float)(1.0 / 3.0);
    float dk3 = 3.f * dk, dmu2 = 2.f * dmu;
    T e3 = vmul(third, vadd(vadd(e[0], e[1]), e[2]));
    T s[6];
    if (sls.do_kappa) {
        T sii3 = vmul(dk3, e3);
        s[0] = vadd(sii3, vmul(dmu2, vsub(e[0], e3)));
        s[1] = vadd(sii3, vmul(dmu2, vsub(e[1], e3)));
        s[2] = vadd(sii3, vmul(dmu2, vsub(e[2], e3)));
    } else {
        s[0] = vmul(dmu2, vsub(e[0], e3));
        s[1] = vmul(dmu2, vsub(e[1], e3));
        s[2] = vneg(vadd(s[0], s[1]));
    }
    s[3] = vmul(dmu, e[3]);
    s[4] = vmul(dmu, e[4]);
    s[5] = vmul(dmu, e[5]);
    for (int l = 0; l < sls.nsls; l++) {
#pragma unroll
        for (int c = 0; c < 6; c++) {
            T r = R[l * stride_l + c * stride_c];
            r = vadd(vmul(sls.a[l], r), vmul(sls.b[l], sr_old[c]));
            r = vadd(r, vmul(sls.g[l], s[c]));
            R[l * stride_l + c * stride_c] = r;
        }
    }
#pragma unroll
    for (int c = 0; c < 6; c++) SR[c * stride_c] = s[c];
}

template <typename T>
__device__ __forceinline__ void sls_update(const SLS &sls, T *R, T *SR, int64_t stride_l,
                                           int64_t stride_c, const T e[6], float dk, float dmu) {
    T sr_old[6];
#pragma unroll
    for (int c = 0; c < 6; c++) sr_old[c] = SR[c * stride_c];
    sls_update_from(sls, R, SR, stride_l, stride_c, e, sr_old, dk, dmu);
}

__device__ __forceinline__ int cg4_index(int p) {
    return p == 6 ? 0 : p == 8 ? 1 : p == 16 ? 2 : p == 18 ? 3 : -1;
}

}  // namespace ax3d
