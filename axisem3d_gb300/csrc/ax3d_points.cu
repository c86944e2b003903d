// ax3d_points.cu -- point kernels: assembly through gather lists, masks, mass, Newmark,
// solid-fluid coupling, source injection, receivers and the stability check.
//
// A "row" is one Fourier order of one point (3 complex for solid, 1 for fluid).  Every
// operation with a Fourier-space (1D) mass or coupling is row-local, so those kernels
// use one thread per row.  Points with a physical-space (3D) mass or coupling
// (Mass3D.cpp:13-57, SFCoupling3D.cpp:9-56) take one CTA each and transform their nr
// azimuthal samples with a direct DFT in shared memory.
#include <algorithm>

#include "ax3d_elem_ops.cuh"
#include "ax3d_kernels.cuh"

namespace ax3d {

constexpr int ROW_THREADS = 256;
constexpr int PT3_THREADS = 128;

__host__ __device__ inline int grid_for(int64_t n, int threads) {
    int64_t b = (n + threads - 1) / threads;
    return (int)(b < 1 ? 1 : (b > 152 * 32 ? 152 * 32 : b));
}

// ---------------- assembly: stiff -= element forces (gatherStiffFromElement) ----------------
// SolidPoint.cpp:197-209 / FluidPoint.cpp:184-195; references are in ascending element
// order so the sums round exactly like Domain::computeStiff's element loop.
__global__ void k_gather_solid(PointTable P, ElemTable T, float2 *__restrict__ ss) {
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < P.nsrows;
         r += (int64_t)gridDim.x * blockDim.x) {
        const int pt = P.srow_pt[r];
        if (P.gskip[pt]) continue;  // assembled by its element
        const int a = (int)(r - P.sofs[pt] / 3);
        const int nr = P.nr[pt], lim = nr / 2 - (nr % 2 == 0);
        float2 *s = ss + r * 3;
        if (a > lim) {
            s[0] = s[1] = s[2] = make_float2(0.f, 0.f);
            continue;
        }
        float2 s0 = s[0], s1 = s[1], s2 = s[2];
        for (int i = P.sg_ptr[pt]; i < P.sg_ptr[pt + 1]; i++) {
            const float2 *f = T.ef + P.sg_ref[i] + (int64_t)a * 3;
            s0 = csub(s0, f[0]);
            s1 = csub(s1, f[1]);
            s2 = csub(s2, f[2]);
        }
        s[0] = s0;
        s[1] = s1;
        s[2] = s2;
    }
}

__global__ void k_gather_fluid(PointTable P, ElemTable T, float2 *__restrict__ fs) {
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < P.nfrows;
         r += (int64_t)gridDim.x * blockDim.x) {
        const int pt = P.frow_pt[r];
        const int a = (int)(r - P.fofs[pt]);
        const int nr = P.nr[pt], lim = nr / 2 - (nr % 2 == 0);
        if (a > lim) {
            fs[r] = make_float2(0.f, 0.f);
            continue;
        }
        float2 s = fs[r];
        for (int i = P.fg_ptr[pt]; i < P.fg_ptr[pt + 1]; i++) s = csub(s, T.ef[P.fg_ref[i] + a]);
        fs[r] = s;
    }
}

void launch_gather(const PointTable &P, const ElemTable &T, const Fields &F, cudaStream_t s) {
    if (P.nsrows && P.sgather) k_gather_solid<<<grid_for(P.nsrows, ROW_THREADS), ROW_THREADS, 0, s>>>(P, T, F.ss);
    if (P.nfrows) k_gather_fluid<<<grid_for(P.nfrows, ROW_THREADS), ROW_THREADS, 0, s>>>(P, T, F.fs);
}

// ---------------- masks (SolidPoint.cpp:216-238, FluidPoint.cpp:197-207) ----------------
__device__ __forceinline__ void mask_solid_row(float2 v[3], int a, int nu, bool even, bool axial) {
    if (a == 0) {
        v[0].y = v[1].y = v[2].y = 0.f;
        if (axial) v[0] = v[1] = make_float2(0.f, 0.f);
    } else if (axial) {
        if (a == 1) {
            float2 s0 = v[0], s1 = v[1];
            // 0.5 (s0 - i s1), 0.5 (s1 + i s0)
            v[0] = cscale(0.5f, make_float2(s0.x + s1.y, s0.y - s1.x));
            v[1] = cscale(0.5f, make_float2(s1.x - s0.y, s1.y + s0.x));
            v[2] = make_float2(0.f, 0.f);
        } else {
            v[0] = v[1] = v[2] = make_float2(0.f, 0.f);
        }
    }
    if (even && a == nu) v[0] = v[1] = v[2] = make_float2(0.f, 0.f);
}
__device__ __forceinline__ void mask_fluid_row(float2 &v, int a, int nu, bool even, bool axial) {
    if (a == 0) v.y = 0.f;
    else if (axial) v = make_float2(0.f, 0.f);
    if (even && a == nu) v = make_float2(0.f, 0.f);
}

__device__ __forceinline__ void kahan_add(float2 &x, float2 &c, float2 d) {
    float2 y = csub(d, c);
    float2 t = cadd(x, y);
    c = csub(csub(t, x), y);
    x = t;
}

// Newmark update of one complex entry (SolidPoint.cpp:30-37)
__device__ __forceinline__ void newmark_entry(float2 &u, float2 &v, float2 &a, float2 &ku, float2 &kv,
                                              float2 acc, float dt, float hd, float hdd, int kahan) {
    if (kahan) {
        kahan_add(v, kv, cscale(hd, cadd(a, acc)));
        a = acc;
        kahan_add(u, ku, cadd(cscale(dt, v), cscale(hdd, a)));
    } else {
        v = cadd(v, cscale(hd, cadd(a, acc)));
        a = acc;
        u = cadd(u, cadd(cscale(dt, v), cscale(hdd, a)));
    }
}

// MassOcean1D::computeAccel (MassOcean1D.cpp:17-32) on one order: the radial component
// (s sin + z cos) takes 1/(m + m_ocean), the tangential ones 1/m.
__device__ __forceinline__ void ocean_accel_row(float2 (&s)[3], const float *__restrict__ o) {
    const float imz = o[0], imr = o[1], st = o[2], ct = o[3];
    float2 z = cadd(cscale(st, s[0]), cscale(ct, s[2]));
    float2 r = csub(cscale(ct, s[0]), cscale(st, s[2]));
    z = cscale(imz, z);
    r = cscale(imr, r);
    s[0] = cadd(cscale(st, z), cscale(ct, r));
    s[2] = csub(cscale(ct, z), cscale(st, r));
    s[1] = cscale(imr, s[1]);
}

// Row-local Newmark (points with a Mass1D or MassOcean1D), SolidPoint::updateNewmark.
__global__ void k_newmark_solid_rows(PointTable P, Fields F, float dt, float hd, float hdd, int kahan,
                                     int in_step) {
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < P.nsrows;
         r += (int64_t)gridDim.x * blockDim.x) {
        const int pt = P.srow_pt[r];
        const int ocl = P.oclen[pt];
        if (ocl > 1 || (ocl == 0 && P.mslen[pt] != 1)) continue;  // Mass3D / MassOcean3D: CTA kernel
        const int a = (int)(r - P.sofs[pt] / 3);
        const int nr = P.nr[pt], nu = nr / 2;
        const bool even = nr % 2 == 0, axial = P.axial[pt];
        const bool clear = !(in_step && P.gskip[pt] == 2);
        float2 s[3];
        const int64_t o = r * 3;
#pragma unroll
        for (int c = 0; c < 3; c++) s[c] = F.ss[o + c];
        mask_solid_row(s, a, nu, even, axial);
        if (ocl == 1) {
            ocean_accel_row(s, P.oc + P.ocofs[pt]);
        } else {
            const float im = P.ms[P.msofs[pt]];
#pragma unroll
            for (int c = 0; c < 3; c++) s[c] = cscale(im, s[c]);  // Mass1D::computeAccel
        }
        mask_solid_row(s, a, nu, even, axial);
#pragma unroll
        for (int c = 0; c < 3; c++) {
            float2 u = F.su[o + c], v = F.sv[o + c], ac = F.sa[o + c];
            float2 ku = kahan ? F.sku[o + c] : make_float2(0.f, 0.f);
            float2 kv = kahan ? F.skv[o + c] : make_float2(0.f, 0.f);
            newmark_entry(u, v, ac, ku, kv, s[c], dt, hd, hdd, kahan);
            F.su[o + c] = u;
            F.sv[o + c] = v;
            F.sa[o + c] = ac;
            if (kahan) {
                F.sku[o + c] = ku;
                F.skv[o + c] = kv;
            }
            if (clear) F.ss[o + c] = make_float2(0.f, 0.f);
        }
    }
}

// FluidPoint::updateNewmark (FluidPoint.cpp:23-44); free-surface fluid points reset.
__global__ void k_newmark_fluid_rows(PointTable P, Fields F, float dt, float hd, float hdd, int kahan) {
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < P.nfrows;
         r += (int64_t)gridDim.x * blockDim.x) {
        const int pt = P.frow_pt[r];
        if (P.fsurf[pt]) {
            F.fu[r] = F.fv[r] = F.fa[r] = F.fs[r] = make_float2(0.f, 0.f);
            if (kahan) F.fku[r] = F.fkv[r] = make_float2(0.f, 0.f);
            continue;
        }
        if (P.mflen[pt] != 1) continue;
        const int a = (int)(r - P.fofs[pt]);
        const int nr = P.nr[pt], nu = nr / 2;
        const bool even = nr % 2 == 0, axial = P.axial[pt];
        float2 s = F.fs[r];
        mask_fluid_row(s, a, nu, even, axial);
        s = cscale(P.mf[P.mfofs[pt]], s);
        mask_fluid_row(s, a, nu, even, axial);
        float2 u = F.fu[r], v = F.fv[r], ac = F.fa[r];
        float2 ku = kahan ? F.fku[r] : make_float2(0.f, 0.f);
        float2 kv = kahan ? F.fkv[r] : make_float2(0.f, 0.f);
        newmark_entry(u, v, ac, ku, kv, s, dt, hd, hdd, kahan);
        F.fu[r] = u;
        F.fv[r] = v;
        F.fa[r] = ac;
        if (kahan) {
            F.fku[r] = ku;
            F.fkv[r] = kv;
        }
        F.fs[r] = make_float2(0.f, 0.f);
    }
}

// ---------------- block-level small DFTs for 3D points ----------------
// x[k] (k < nr) of column c from X[a*stride + c] (a <= nu, order 0 real part only);
// weights 2 for 0 < a < nr/2, 1 for the Nyquist order of an even nr.
__device__ void blk_c2r(const float2 *X, int stride, int ncol, int nr, float *x /*[ncol][nr]*/) {
    const int nu = nr / 2;
    for (int t = threadIdx.x; t < ncol * nr; t += blockDim.x) {
        const int c = t / nr, k = t - c * nr;
        float acc = X[c].x;
        int m = 0;
        for (int a = 1; a <= nu; a++) {
            m += k;
            if (m >= nr) m -= nr;
            float s, co;
            sincospif(2.f * (float)m / (float)nr, &s, &co);
            const float w = (nr % 2 == 0 && a == nu) ? 1.f : 2.f;
            const float2 v = X[(int64_t)a * stride + c];
            acc += w * (v.x * co - v.y * s);
        }
        x[c * nr + k] = acc;
    }
}
// Y[a*stride + c] = (1/nr) sum_k x[c][k] e^{-i 2 pi k a / nr}, a = 0..nu
__device__ void blk_r2c(const float *x, int ncol, int nr, float2 *Y, int stride) {
    const int nu = nr / 2;
    const float inv = 1.f / (float)nr;
    for (int t = threadIdx.x; t < ncol * (nu + 1); t += blockDim.x) {
        const int c = t / (nu + 1), a = t - c * (nu + 1);
        float re = 0.f, im = 0.f;
        int m = 0;
        for (int k = 0; k < nr; k++) {
            float s, co;
            sincospif(2.f * (float)m / (float)nr, &s, &co);
            re += x[c * nr + k] * co;
            im -= x[c * nr + k] * s;
            m += a;
            if (m >= nr) m -= nr;
        }
        Y[(int64_t)a * stride + c] = make_float2(re * inv, im * inv);
    }
}

// Mass3D::computeAccel (or MassOcean3D::computeAccel, MassOcean3D.cpp:24-55, on the solid
// part) + Newmark for one point per CTA (solid and/or fluid part).
__global__ void __launch_bounds__(PT3_THREADS)
    k_newmark_3d(PointTable P, Fields F, const int32_t *__restrict__ pts, int n, float dt, float hd,
                 float hdd, int kahan) {
    extern __shared__ float sm3[];
    const int pt = pts[blockIdx.x];
    const int nr = P.nr[pt], nu = nr / 2, na = nu + 1;
    const bool even = nr % 2 == 0, axial = P.axial[pt];
    float2 *S = reinterpret_cast<float2 *>(sm3);  // [na][3]
    float *x = sm3 + 2 * 3 * na;                  // [3][nr]
    for (int phase = 0; phase < 2; phase++) {
        const int ncomp = phase == 0 ? 3 : 1;
        int64_t ofs;
        const float *im;
        const int ocl = P.oclen[pt];
        if (phase == 0) {
            if (P.kind[pt] == 1 || !(ocl > 1 || (ocl == 0 && P.mslen[pt] > 1))) continue;
            ofs = P.sofs[pt];
            im = P.ms + P.msofs[pt];
        } else {
            if (P.kind[pt] == 0 || P.mflen[pt] == 1) continue;
            ofs = P.fofs[pt];
            im = P.mf + P.mfofs[pt];
        }
        float2 *ss = phase == 0 ? F.ss : F.fs;
        float2 *su = phase == 0 ? F.su : F.fu, *sv = phase == 0 ? F.sv : F.fv, *sa = phase == 0 ? F.sa : F.fa;
        float2 *sku = phase == 0 ? F.sku : F.fku, *skv = phase == 0 ? F.skv : F.fkv;
        if (phase == 1 && P.fsurf[pt]) {
            for (int i = threadIdx.x; i < na; i += blockDim.x) {
                su[ofs + i] = sv[ofs + i] = sa[ofs + i] = ss[ofs + i] = make_float2(0.f, 0.f);
                if (kahan) sku[ofs + i] = skv[ofs + i] = make_float2(0.f, 0.f);
            }
            __syncthreads();
            continue;
        }
        for (int a = threadIdx.x; a < na; a += blockDim.x) {
            if (ncomp == 3) {
                float2 v[3] = {ss[ofs + a * 3], ss[ofs + a * 3 + 1], ss[ofs + a * 3 + 2]};
                mask_solid_row(v, a, nu, even, axial);
                S[a * 3] = v[0];
                S[a * 3 + 1] = v[1];
                S[a * 3 + 2] = v[2];
            } else {
                float2 v = ss[ofs + a];
                mask_fluid_row(v, a, nu, even, axial);
                S[a * 3] = v;
            }
        }
        __syncthreads();
        blk_c2r(S, 3, ncomp, nr, x);
        __syncthreads();
        if (phase == 0 && ocl > 1) {
            // a = f / m - (f . n') n', n' = unit normal * sqrt(m_ocean / (m (m + m_ocean)))
            const float *o = P.oc + P.ocofs[pt];
            for (int k = threadIdx.x; k < nr; k += blockDim.x) {
                const float m = o[4 * k], n0 = o[4 * k + 1], n1 = o[4 * k + 2], n2 = o[4 * k + 3];
                const float f0 = x[k], f1 = x[nr + k], f2 = x[2 * nr + k];
                const float fn = f0 * n0 + f1 * n1 + f2 * n2;
                x[k] = f0 * m - fn * n0;
                x[nr + k] = f1 * m - fn * n1;
                x[2 * nr + k] = f2 * m - fn * n2;
            }
        } else {
            for (int t = threadIdx.x; t < ncomp * nr; t += blockDim.x) x[t] *= im[t % nr];
        }
        __syncthreads();
        blk_r2c(x, ncomp, nr, S, 3);
        __syncthreads();
        for (int a = threadIdx.x; a < na; a += blockDim.x) {
            float2 v[3] = {S[a * 3], S[a * 3 + 1], S[a * 3 + 2]};
            if (ncomp == 3) mask_solid_row(v, a, nu, even, axial);
            else mask_fluid_row(v[0], a, nu, even, axial);
            for (int c = 0; c < ncomp; c++) {
                const int64_t o = ofs + (int64_t)a * ncomp + c;
                float2 u = su[o], vv = sv[o], ac = sa[o];
                float2 ku = kahan ? sku[o] : make_float2(0.f, 0.f);
                float2 kv = kahan ? skv[o] : make_float2(0.f, 0.f);
                newmark_entry(u, vv, ac, ku, kv, v[c], dt, hd, hdd, kahan);
                su[o] = u;
                sv[o] = vv;
                sa[o] = ac;
                if (kahan) {
                    sku[o] = ku;
                    skv[o] = kv;
                }
                ss[o] = make_float2(0.f, 0.f);
            }
        }
        __syncthreads();
    }
}

void launch_newmark(const PointTable &P, const Fields &F, float dt, float hd, float hdd, int kahan,
                    const int32_t *pts3d, int n3d, int in_step, cudaStream_t s) {
    if (P.nsrows)
        k_newmark_solid_rows<<<grid_for(P.nsrows, ROW_THREADS), ROW_THREADS, 0, s>>>(P, F, dt, hd, hdd, kahan,
                                                                                  in_step);
    if (P.nfrows)
        k_newmark_fluid_rows<<<grid_for(P.nfrows, ROW_THREADS), ROW_THREADS, 0, s>>>(P, F, dt, hd, hdd, kahan);
    if (n3d > 0)
        k_newmark_3d<<<n3d, PT3_THREADS, 48 * 1024, s>>>(P, F, pts3d, n3d, dt, hd, hdd, kahan);
}

// ---------------- solid-fluid coupling (SolidFluidPoint.cpp:106-110) ----------------
// SFCoupling1D.cpp:9-17, row-local; solid->fluid first, then fluid->solid.
__global__ void k_couple_1d(PointTable P, Fields F) {
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < P.nsrows;
         r += (int64_t)gridDim.x * blockDim.x) {
        const int pt = P.srow_pt[r];
        if (P.kind[pt] != 2 || P.sflen[pt] != 1) continue;
        const int a = (int)(r - P.sofs[pt] / 3);
        const float *n = P.sfn + P.sfofs[pt] * 3;
        const float *ni = P.sfni + P.sfofs[pt] * 3;
        const int64_t fr = P.fofs[pt] + a;
        float2 us = F.su[r * 3], uz = F.su[r * 3 + 2];
        float2 f = cadd(F.fs[fr], cadd(cscale(n[0], us), cscale(n[2], uz)));
        F.fs[fr] = f;
        F.ss[r * 3] = csub(F.ss[r * 3], cscale(ni[0], f));
        F.ss[r * 3 + 2] = csub(F.ss[r * 3 + 2], cscale(ni[2], f));
    }
}

// SFCoupling3D.cpp:9-56, one CTA per point.
__global__ void __launch_bounds__(PT3_THREADS) k_couple_3d(PointTable P, Fields F, const int32_t *__restrict__ pts) {
    extern __shared__ float sm3[];
    const int pt = pts[blockIdx.x];
    const int nr = P.nr[pt], nu = nr / 2, na = nu + 1;
    float2 *S = reinterpret_cast<float2 *>(sm3);  // [na][3]
    float *x = sm3 + 2 * 3 * na;                  // [3][nr]
    float *y = x + 3 * nr;                        // [nr]
    const float *n = P.sfn + P.sfofs[pt] * 3;
    const float *ni = P.sfni + P.sfofs[pt] * 3;
    const int64_t so = P.sofs[pt], fo = P.fofs[pt];
    // solid -> fluid
    for (int t = threadIdx.x; t < na * 3; t += blockDim.x) S[t] = F.su[so + t];
    __syncthreads();
    blk_c2r(S, 3, 3, nr, x);
    __syncthreads();
    for (int k = threadIdx.x; k < nr; k += blockDim.x)
        y[k] = n[k * 3] * x[k] + n[k * 3 + 1] * x[nr + k] + n[k * 3 + 2] * x[2 * nr + k];
    __syncthreads();
    blk_r2c(y, 1, nr, S, 3);
    __syncthreads();
    for (int a = threadIdx.x; a < na; a += blockDim.x) {
        F.fs[fo + a] = cadd(F.fs[fo + a], S[a * 3]);
    }
    __syncthreads();
    // fluid -> solid
    for (int a = threadIdx.x; a < na; a += blockDim.x) S[a * 3] = F.fs[fo + a];
    __syncthreads();
    blk_c2r(S, 3, 1, nr, y);
    __syncthreads();
    for (int t = threadIdx.x; t < 3 * nr; t += blockDim.x) {
        const int c = t / nr, k = t - c * nr;
        x[c * nr + k] = ni[k * 3 + c] * y[k];
    }
    __syncthreads();
    blk_r2c(x, 3, nr, S, 3);
    __syncthreads();
    for (int t = threadIdx.x; t < na * 3; t += blockDim.x) F.ss[so + t] = csub(F.ss[so + t], S[t]);
}

void launch_couple(const PointTable &P, const Fields &F, const int32_t *sf3d, int n3d, int n1d, cudaStream_t s) {
    if (P.nsrows && n1d > 0) k_couple_1d<<<grid_for(P.nsrows, ROW_THREADS), ROW_THREADS, 0, s>>>(P, F);
    if (n3d > 0) k_couple_3d<<<n3d, PT3_THREADS, 48 * 1024, s>>>(P, F, sf3d);
}

// ---------------- source (SourceTerm.cpp:29-35) ----------------
// The step index is read on the device (*tptr + tofs) so that one captured step serves
// every time step of a CUDA graph replay.
__global__ void k_source(PointTable P, ElemTable T, float2 *__restrict__ ss, const int32_t *src_elem,
                         const int32_t *src_nord, const int64_t *src_ofs, const float2 *force, int nsrc,
                         const float *stf, int nstf, const int32_t *tptr, int tofs) {
    const int tstep = *tptr + tofs;
    if (tstep < 0 || tstep >= nstf) return;  // beyond the source-time function: no force
    const float f = stf[tstep];
    for (int s = 0; s < nsrc; s++) {
        const int e = src_elem[s], nord = src_nord[s];
        for (int t = threadIdx.x; t < NPE * nord; t += blockDim.x) {
            const int p = t / nord, a = t - p * nord;
            const int pt = T.pts[e * NPE + p];
            if (a > P.nr[pt] / 2) continue;  // truncated to Nu_p + 1 rows
            const float2 *fc = force + src_ofs[s] + ((int64_t)p * nord + a) * 3;
            float2 *o = ss + P.sofs[pt] + (int64_t)a * 3;
#pragma unroll
            for (int c = 0; c < 3; c++) o[c] = cadd(o[c], cscale(f, fc[c]));
        }
        __syncthreads();  // sources may share points: apply them in order
    }
}

void launch_source(const PointTable &P, const ElemTable &T, const Fields &F, const int32_t *src_elem,
                   const int32_t *src_nord, const int64_t *src_ofs, const float2 *src_force, int nsrc,
                   const float *stf, int nstf, const int32_t *tptr, int tofs, cudaStream_t s) {
    if (nsrc <= 0) return;
    k_source<<<1, 128, 0, s>>>(P, T, F.ss, src_elem, src_nord, src_ofs, src_force, nsrc, stf, nstf, tptr, tofs);
}

// ---------------- receivers (SolidElement::computeGroundMotion, SolidElement.cpp:189-216) ----------------
__global__ void k_record(PointTable P, ElemTable T, const float2 *__restrict__ su, const int32_t *rec_elem,
                         const float *rec_phi, const float *rec_w, int nrec, float *out_base, int cap,
                         const int32_t *tptr, int tofs) {
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    const int t = *tptr + tofs;
    if (warp >= nrec || t < 0 || t >= cap) return;
    float *out = out_base + (size_t)t * nrec * 3;
    const int e = rec_elem[warp];
    const float phi = rec_phi[warp];
    const int nr = T.nr[e], lim = nr / 2 - (nr % 2 == 0);
    float o[3] = {0.f, 0.f, 0.f};
    if (lane < NPE) {
        const float w = rec_w[warp * NPE + lane];
        if (fabsf(w) >= 1e-10f) {
            const int pt = T.pts[e * NPE + lane];
            const int pnr = P.nr[pt], plim = pnr / 2 - (pnr % 2 == 0);
            const float2 *u = su + P.sofs[pt];
            float up[3] = {u[0].x, u[1].x, u[2].x};
            const int amax = min(lim, plim);
            for (int a = 1; a <= amax; a++) {
                float s, c;
                sincosf((float)a * phi, &s, &c);
#pragma unroll
                for (int k = 0; k < 3; k++) {
                    const float2 v = u[a * 3 + k];
                    up[k] += 2.f * c * v.x - 2.f * s * v.y;
                }
            }
#pragma unroll
            for (int k = 0; k < 3; k++) o[k] = w * up[k];
        }
    }
#pragma unroll
    for (int k = 0; k < 3; k++)
        for (int off = 16; off > 0; off >>= 1) o[k] += __shfl_down_sync(0xffffffffu, o[k], off);
    if (lane == 0) {
        out[warp * 3] = o[0];
        out[warp * 3 + 1] = o[1];
        out[warp * 3 + 2] = o[2];
    }
}

void launch_record(const PointTable &P, const ElemTable &T, const float2 *su, const int32_t *rec_elem,
                   const float *rec_phi, const float *rec_w, int nrec, float *out_base, int cap,
                   const int32_t *tptr, int tofs, cudaStream_t s) {
    if (nrec <= 0) return;
    const int threads = 128;
    const int blocks = (nrec * 32 + threads - 1) / threads;
    k_record<<<blocks, threads, 0, s>>>(P, T, su, rec_elem, rec_phi, rec_w, nrec, out_base, cap, tptr, tofs);
}

// ---------------- stability (Domain::checkStability, Domain.cpp:237-275) ----------------
// SurfaceRecorder::record with SolidElement::feedDispOnSide (SolidElement.cpp:354-390):
// when the step index t is a multiple of interval, record t / interval gets, per edge,
// [component][point q on the side][order a], a <= Nu_e; a point's rows 0..Nu_p are copied,
// the orders above them are zero.  Block per edge.
__global__ void k_record_surface(PointTable P, ElemTable T, const float2 *__restrict__ su, const int32_t *elem,
                                 const int32_t *side, const int64_t *rofs, int nedge, float2 *out_base,
                                 int64_t rowlen, int cap, const int32_t *tptr, int tofs, int interval) {
    const int t = *tptr + tofs;
    if (t < 0 || t % interval) return;
    const int rec = t / interval;
    if (rec >= cap) return;
    for (int i = blockIdx.x; i < nedge; i += gridDim.x) {
        const int e = elem[i], sd = side[i];
        const int n = T.nr[e] / 2 + 1;
        float2 *o = out_base + (int64_t)rec * rowlen + rofs[i];
        for (int idx = threadIdx.x; idx < 15 * n; idx += blockDim.x) {
            const int c = idx / (5 * n), rem = idx - c * 5 * n, q = rem / n, a = rem - q * n;
            const int ipol = sd == 1 ? 4 : sd == 3 ? 0 : q;
            const int jpol = sd == 0 ? 0 : sd == 2 ? 4 : q;
            const int pt = T.pts[e * NPE + ipol * 5 + jpol];
            o[idx] = a <= P.nr[pt] / 2 ? su[P.sofs[pt] + (int64_t)a * 3 + c] : make_float2(0.f, 0.f);
        }
    }
}

void launch_record_surface(const PointTable &P, const ElemTable &T, const float2 *su, const int32_t *elem,
                           const int32_t *side, const int64_t *rofs, int nedge, float2 *out_base, int64_t rowlen,
                           int cap, const int32_t *tptr, int tofs, int interval, cudaStream_t s) {
    if (nedge <= 0) return;
    k_record_surface<<<std::min(nedge, 152 * 8), 128, 0, s>>>(P, T, su, elem, side, rofs, nedge, out_base, rowlen,
                                                             cap, tptr, tofs, interval);
}

__global__ void k_stability(const float2 *__restrict__ su, int64_t ns, const float2 *__restrict__ fu, int64_t nf,
                            int32_t *flag, const int32_t *tptr, int interval) {
    if (interval <= 0 || (*tptr) % interval != 0) return;  // Newmark.cpp:68-70
    bool bad = false;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < ns + nf;
         i += (int64_t)gridDim.x * blockDim.x) {
        const float2 v = i < ns ? su[i] : fu[i - ns];
        if (!isfinite(v.x) || !isfinite(v.y)) bad = true;
    }
    if (__any_sync(0xffffffffu, bad) && (threadIdx.x & 31) == 0) atomicOr(flag, 1);
}

void launch_stability(const float2 *su, int64_t ns, const float2 *fu, int64_t nf, int32_t *flag,
                      const int32_t *tptr, int interval, cudaStream_t s) {
    if (ns + nf == 0) return;
    k_stability<<<grid_for(ns + nf, ROW_THREADS), ROW_THREADS, 0, s>>>(su, ns, fu, nf, flag, tptr, interval);
}

__global__ void k_advance(int32_t *tptr) { *tptr += 1; }

void launch_advance(int32_t *tptr, cudaStream_t s) { k_advance<<<1, 1, 0, s>>>(tptr); }

}  // namespace ax3d

namespace ax3d {

// ---------------- Nu wisdom (SolidPoint::learnWisdom, SolidPoint.cpp:240-272) ----------------
// One thread per point; per component the L2 norm, the Hilbert norm (order 0 halved) and,
// when the Hilbert norm is a new maximum, the smallest order whose tail energy is below
// h2 * cutoff^2.  Sums run over orders in increasing order (the oracle's order).
__device__ int wisdom_component(const float2 *u, int stride, int nu, float cutoff, float &maxh, int nu_old) {
    float l2 = 0.f;
    for (int a = 0; a <= nu; a++) {
        const float2 v = u[a * stride];
        l2 += v.x * v.x + v.y * v.y;
    }
    const float2 v0 = u[0];
    // Real h2norm = L2norm - .5 * |u_0|^2, the .5 being a double literal
    const float h2 = (float)((double)l2 - 0.5 * (double)(v0.x * v0.x + v0.y * v0.y));
    if (h2 <= maxh) return nu_old;
    maxh = h2;
    const float tol = h2 * cutoff * cutoff;
    float head = 0.f;
    for (int nn = 0; nn < nu; nn++) {
        const float2 v = u[nn * stride];
        head += v.x * v.x + v.y * v.y;
        if (l2 - head <= tol) return nn;
    }
    return nu;
}

__global__ void k_learn_wisdom(PointTable P, const float2 *__restrict__ su, const float2 *__restrict__ fu,
                               float *maxh, int32_t *nuw, float cutoff, const int32_t *tptr, int interval) {
    if (tptr && (interval <= 0 || (*tptr - 1) % interval != 0)) return;  // Domain::learnWisdom(tstep - 1)
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < P.n; p += gridDim.x * blockDim.x) {
        const int nu = P.nr[p] / 2;
        if (P.sofs[p] >= 0)
            for (int c = 0; c < 3; c++)
                nuw[p * 4 + c] = wisdom_component(su + P.sofs[p] + c, 3, nu, cutoff, maxh[p * 4 + c], nuw[p * 4 + c]);
        if (P.fofs[p] >= 0)
            nuw[p * 4 + 3] = wisdom_component(fu + P.fofs[p], 1, nu, cutoff, maxh[p * 4 + 3], nuw[p * 4 + 3]);
    }
}

void launch_learn_wisdom(const PointTable &P, const Fields &F, float *maxh, int32_t *nuw, float cutoff,
                         const int32_t *tptr, int interval, cudaStream_t s) {
    if (P.n <= 0) return;
    k_learn_wisdom<<<grid_for(P.n, ROW_THREADS), ROW_THREADS, 0, s>>>(P, F.su, F.fu, maxh, nuw, cutoff, tptr, interval);
}

}  // namespace ax3d
