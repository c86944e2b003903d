// ax3d_elements.cu -- element stiffness kernels (Element::computeStiff) for sm_103a.
//
// Fourier-space elements (1D material): one warp per (element, Fourier order); the order
//   loop of SolidElement::displToStiff (SOLVER/src/core/element/SolidElement.cpp:404-443)
//   is embarrassingly parallel there.
// Physical-space elements (3D material): one CTA per element.  The element's strain for
//   all orders is staged in shared memory, transformed to the nr azimuthal samples
//   (FieldFFT::transformF2P, SOLVER/src/core/element/fft/FieldFFT.cpp:19-25), turned
//   into stress with the SLS update per sample, transformed back (transformP2F, scaled
//   by 1/nr as SolverFFTW_N6::computeR2C, SolverFFTW_N6.cpp:45-49) and divergence-
//   projected, so the field makes one HBM round trip per step.  When the 150 columns
//   of an element do not fit in shared memory the GLL points are processed in chunks;
//   the divergence is linear in the stress, so chunk contributions add up.
//   The azimuthal transform is a register-tiled real DFT with a shared twiddle table,
//   exploiting cos/sin parity (k <-> nr - k) to halve the work.
#include "ax3d_elem_ops.cuh"
#include "ax3d_kernels.cuh"

namespace ax3d {



void set_g_matrices(const float *g_gll, const float *g_glj, cudaStream_t s) {
    cudaMemcpyToSymbolAsync(c_G, g_gll, 25 * sizeof(float), 0, cudaMemcpyHostToDevice, s);
    cudaMemcpyToSymbolAsync(c_G, g_glj, 25 * sizeof(float), 25 * sizeof(float),
                            cudaMemcpyHostToDevice, s);
}

constexpr int FW_WARPS = 8;   // warps per CTA in the Fourier-space kernels
constexpr int PH_THREADS = 256;
constexpr int PH_WARPS = PH_THREADS / 32;
constexpr int QSCR = 14 * 25;  // per-warp scratch (float2) for grad/quad
constexpr int KT = 8;          // DFT tile: samples (or orders) per thread
constexpr int CT = 4;          // DFT tile: columns per thread
constexpr size_t SMEM_MAX = 227 * 1024;

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
// Fourier-space solid elements: warp per (element, order)
// ------------------------------------------------------------------------------------
__global__ void __launch_bounds__(FW_WARPS * 32)
    k_elem_fourier_solid(ElemTable T, PointTable P, const float2 *__restrict__ su,
                         const int2 *__restrict__ items, int nitems, SLS sls) {
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
        const bool tiso = (mat == 1 || mat == 2);
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
        float2 eps[6], sig[6];
#pragma unroll
        for (int c = 0; c < 6; c++) eps[c] = make_float2(0.f, 0.f);
        if (active && a <= lim) grad6_lane(L, g, axial, a, q, eps);
        __syncwarp();
        if (active) {
            const float *tr = T.trig + (int64_t)e * 100;
            float s1 = 0.f, c1 = 0.f, s2 = 0.f, c2 = 0.f;
            if (tiso) {
                s1 = tr[p];
                c1 = tr[25 + p];
                s2 = tr[50 + p];
                c2 = tr[75 + p];
                spz_rtz(eps, s1, c1, s2, c2);
            }
            const float *md = T.moduli + T.mofs[e];
            elastic(mat, eps, sig, [&](int k) { return md[k * NPE + p]; });
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
                    sls_update(sls, R, SR, sl, (int64_t)npa, eps, am[qq], am[npa + qq]);
                }
            }
            if (tiso) rtz_spz(sig, s1, c1, s2, c2);
        }
        float2 f[3];
        quad6_lane(L, g, axial, a, sig, q, active && a <= lim, f);
        if (active) {
            float2 *ef = T.ef + T.efofs[e] + ((int64_t)p * n + a) * 3;
            if (a <= lim) {
                ef[0] = f[0];
                ef[1] = f[1];
                ef[2] = f[2];
            } else {
                ef[0] = ef[1] = ef[2] = make_float2(0.f, 0.f);
            }
        }
    }
}

// Fourier-space fluid elements (FluidElement.cpp:333-355 with Acoustic1D.cpp:8-16)
__global__ void __launch_bounds__(FW_WARPS * 32)
    k_elem_fourier_fluid(ElemTable T, PointTable P, const float2 *__restrict__ fu,
                         const int2 *__restrict__ items, int nitems) {
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
        float2 eps[3] = {make_float2(0.f, 0.f), make_float2(0.f, 0.f), make_float2(0.f, 0.f)};
        if (active && a <= lim) grad1_lane(L, g, axial, a, q, eps);
        __syncwarp();
        float2 sig[3];
        const float K = active ? T.moduli[T.mofs[e] + p] : 0.f;
#pragma unroll
        for (int c = 0; c < 3; c++) sig[c] = cscale(K, eps[c]);
        float2 f;
        quad1_lane(L, g, axial, a, sig, q, active && a <= lim, f);
        if (active) T.ef[T.efofs[e] + (int64_t)p * n + a] = a <= lim ? f : make_float2(0.f, 0.f);
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

// ------------------------------------------------------------------------------------
// Physical-space elements: CTA per element
// ------------------------------------------------------------------------------------
// Shared layout (bytes): tw[nr] float2 | F[n][ncolp] float2 | X[nr][ncolp] float,
// where the per-warp grad/quad scratch aliases X (X is dead in those phases).
__host__ __device__ inline int pad4(int x) { return (x + 3) & ~3; }

size_t phys_smem_bytes(int nr, int ncomp, int npts_chunk) {
    int n = nr / 2 + 1;
    int ncolp = pad4(ncomp * npts_chunk);
    size_t tw = (size_t)8 * ((nr + 1) & ~1);
    size_t F = (size_t)8 * n * ncolp;
    size_t X = (size_t)4 * nr * ncolp;
    size_t scr = (size_t)PH_WARPS * QSCR * 8;
    return tw + F + (X > scr ? X : scr);
}

int phys_points_per_chunk(int nr, int ncomp) {
    for (int nchunk = 1; nchunk <= NPE; nchunk++) {
        int P = (NPE + nchunk - 1) / nchunk;
        if (phys_smem_bytes(nr, ncomp, P) <= SMEM_MAX) return P;
    }
    return 0;  // does not fit even one point per pass
}

// C2R of ncolp columns: X[k][col] = Re F[0][col] + 2 sum_{a=1}^{lim} Re(F[a][col] e^{+i 2pi k a/nr})
__device__ void phys_c2r(const float2 *__restrict__ tw, const float2 *__restrict__ F,
                         float *__restrict__ X, int nr, int lim, int ncolp) {
    const int kh = nr / 2 + 1;  // k = 0 .. nr/2 computed, mirrors filled by parity
    const int nkb = (kh + KT - 1) / KT, ncb = ncolp / CT;
    for (int tile = threadIdx.x; tile < nkb * ncb; tile += blockDim.x) {
        const int kb = tile / ncb, cb = tile - kb * ncb;
        const int k0 = kb * KT, c0 = cb * CT;
        float cs[KT][CT], sn[KT][CT];
        int idx[KT], inc[KT];
#pragma unroll
        for (int t = 0; t < KT; t++) {
            idx[t] = 0;
            inc[t] = (k0 + t) % nr;
#pragma unroll
            for (int c = 0; c < CT; c++) cs[t][c] = sn[t][c] = 0.f;
        }
        for (int a = 1; a <= lim; a++) {
            const float4 f01 = *reinterpret_cast<const float4 *>(F + (int64_t)a * ncolp + c0);
            const float4 f23 = *reinterpret_cast<const float4 *>(F + (int64_t)a * ncolp + c0 + 2);
            const float fr[4] = {f01.x, f01.z, f23.x, f23.z};
            const float fi[4] = {f01.y, f01.w, f23.y, f23.w};
#pragma unroll
            for (int t = 0; t < KT; t++) {
                int m = idx[t] + inc[t];  // (k * a) mod nr, incrementally
                m = m >= nr ? m - nr : m;
                idx[t] = m;
                const float2 w = tw[m];
#pragma unroll
                for (int c = 0; c < CT; c++) {
                    cs[t][c] = fmaf(fr[c], w.x, cs[t][c]);
                    sn[t][c] = fmaf(fi[c], w.y, sn[t][c]);
                }
            }
        }
        float f0[CT];
#pragma unroll
        for (int c = 0; c < CT; c++) f0[c] = F[c0 + c].x;
#pragma unroll
        for (int t = 0; t < KT; t++) {
            const int k = k0 + t;
            if (k >= kh) break;
            float lo[CT], hi[CT];
#pragma unroll
            for (int c = 0; c < CT; c++) {
                lo[c] = f0[c] + 2.f * (cs[t][c] - sn[t][c]);
                hi[c] = f0[c] + 2.f * (cs[t][c] + sn[t][c]);
            }
            *reinterpret_cast<float4 *>(X + (int64_t)k * ncolp + c0) = make_float4(lo[0], lo[1], lo[2], lo[3]);
            const int km = nr - k;
            if (k > 0 && km != k)
                *reinterpret_cast<float4 *>(X + (int64_t)km * ncolp + c0) =
                    make_float4(hi[0], hi[1], hi[2], hi[3]);
        }
    }
}

// R2C of ncolp columns scaled by 1/nr, orders 0..lim:
// F[a] = (x_0 + sum_{k=1}^{(nr-1)/2} (x_k + x_{nr-k}) cos - i (x_k - x_{nr-k}) sin
//         + [nr even] (-1)^a x_{nr/2}) / nr
__device__ void phys_r2c(const float2 *__restrict__ tw, const float *__restrict__ X,
                         float2 *__restrict__ F, int nr, int lim, int ncolp) {
    const int k2 = (nr - 1) / 2;
    const int na = lim + 1;
    const int nab = (na + KT - 1) / KT, ncb = ncolp / CT;
    const float inv_nr = 1.f / (float)nr;
    for (int tile = threadIdx.x; tile < nab * ncb; tile += blockDim.x) {
        const int ab = tile / ncb, cb = tile - ab * ncb;
        const int a0 = ab * KT, c0 = cb * CT;
        float re[KT][CT], im[KT][CT];
        int idx[KT], inc[KT];
#pragma unroll
        for (int t = 0; t < KT; t++) {
            idx[t] = 0;
            inc[t] = (a0 + t) % nr;
#pragma unroll
            for (int c = 0; c < CT; c++) re[t][c] = im[t][c] = 0.f;
        }
        for (int k = 1; k <= k2; k++) {
            const float4 xl = *reinterpret_cast<const float4 *>(X + (int64_t)k * ncolp + c0);
            const float4 xh = *reinterpret_cast<const float4 *>(X + (int64_t)(nr - k) * ncolp + c0);
            const float sm[4] = {xl.x + xh.x, xl.y + xh.y, xl.z + xh.z, xl.w + xh.w};
            const float df[4] = {xl.x - xh.x, xl.y - xh.y, xl.z - xh.z, xl.w - xh.w};
#pragma unroll
            for (int t = 0; t < KT; t++) {
                int m = idx[t] + inc[t];  // (k * a) mod nr, incrementally in k
                m = m >= nr ? m - nr : m;
                idx[t] = m;
                const float2 w = tw[m];
#pragma unroll
                for (int c = 0; c < CT; c++) {
                    re[t][c] = fmaf(sm[c], w.x, re[t][c]);
                    im[t][c] = fmaf(df[c], w.y, im[t][c]);
                }
            }
        }
        const float4 x0 = *reinterpret_cast<const float4 *>(X + c0);
        const float x0v[4] = {x0.x, x0.y, x0.z, x0.w};
        float xn[4] = {0.f, 0.f, 0.f, 0.f};
        if (nr % 2 == 0) {
            const float4 t4 = *reinterpret_cast<const float4 *>(X + (int64_t)(nr / 2) * ncolp + c0);
            xn[0] = t4.x; xn[1] = t4.y; xn[2] = t4.z; xn[3] = t4.w;
        }
#pragma unroll
        for (int t = 0; t < KT; t++) {
            const int a = a0 + t;
            if (a >= na) break;
            const float sgn = (a & 1) ? -1.f : 1.f;
            float2 o[CT];
#pragma unroll
            for (int c = 0; c < CT; c++)
                o[c] = make_float2((x0v[c] + re[t][c] + sgn * xn[c]) * inv_nr, -im[t][c] * inv_nr);
            *reinterpret_cast<float4 *>(F + (int64_t)a * ncolp + c0) = make_float4(o[0].x, o[0].y, o[1].x, o[1].y);
            *reinterpret_cast<float4 *>(F + (int64_t)a * ncolp + c0 + 2) = make_float4(o[2].x, o[2].y, o[3].x, o[3].y);
        }
    }
}

// Twiddles (cos, sin)(2 pi m / nr), precomputed in FP64 on the host per distinct nr.
__device__ void fill_twiddles(float2 *tw, const ElemTable &T, int nr) {
    const float2 *src = T.twtab + T.twofs[nr];
    for (int m = threadIdx.x; m < nr; m += blockDim.x) tw[m] = src[m];
}

template <int NCOMP>
__device__ __forceinline__ void phys_layout(int nr, int P, float2 *&tw, float2 *&F, float *&X,
                                            float2 *&scr, int &ncolp, char *smem) {
    const int n = nr / 2 + 1;
    ncolp = pad4(NCOMP * P);
    tw = reinterpret_cast<float2 *>(smem);
    F = tw + ((nr + 1) & ~1);  // keep F 16-byte aligned
    X = reinterpret_cast<float *>(F + (int64_t)n * ncolp);
    scr = reinterpret_cast<float2 *>(X);
}

__global__ void __launch_bounds__(PH_THREADS)
    k_elem_phys_solid(ElemTable T, PointTable P, const float2 *__restrict__ su,
                      const int32_t *__restrict__ elems, int Pmax, SLS sls) {
    extern __shared__ __align__(16) char smem[];
    const int e = elems[blockIdx.x];
    const int flags = T.flags[e];
    const bool axial = flags & EF_AXIAL;
    const int nr = T.nr[e], nu = nr / 2, n = nu + 1, lim = nu - (nr % 2 == 0);
    const int mat = ef_mat(flags), att = ef_att(flags);
    const bool tiso = (mat == 1 || mat == 2);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    float2 *tw, *F, *scr;
    float *X;
    int ncolp;
    phys_layout<6>(nr, Pmax, tw, F, X, scr, ncolp, smem);
    fill_twiddles(tw, T, nr);
    float2 *q = scr + warp * QSCR;
    const bool active = lane < NPE;
    const int p = active ? lane : 0;
    LaneOps L;
    L.init(p, axial);
    Geo g;
    g.load(T.geo + (int64_t)e * 125, p);
    const float *tr = T.trig + (int64_t)e * 100;
    float s1 = 0.f, c1 = 0.f, s2 = 0.f, c2 = 0.f;
    if (tiso) {
        s1 = tr[p];
        c1 = tr[25 + p];
        s2 = tr[50 + p];
        c2 = tr[75 + p];
    }
    const int pt_me = T.pts[e * NPE + p];
    float2 *ef = T.ef + T.efofs[e];
    const float *md = T.moduli + T.mofs[e];
    const int npa = att == 2 ? 4 : NPE;
    float *mem = T.mem + (att ? T.memofs[e] : 0);
    const float *am = T.attm + (att ? T.aofs[e] : 0);
    const int64_t sl = (int64_t)nr * 6 * npa;

    for (int p0 = 0; p0 < NPE; p0 += Pmax) {
        const int Pc = min(Pmax, NPE - p0);
        const int ncol = 6 * Pc;
        const bool mine = active && p >= p0 && p < p0 + Pc;
        // ---- phase 1: strain (grad6 + rotation) of the chunk's points, all orders ----
        for (int a = warp; a < n; a += PH_WARPS) {
            if (active) {
                float2 u[3];
                load_solid_u(P, su, pt_me, a, u);
                q[p] = u[0];
                q[25 + p] = u[1];
                q[50 + p] = u[2];
            }
            __syncwarp();
            float2 eps[6];
#pragma unroll
            for (int c = 0; c < 6; c++) eps[c] = make_float2(0.f, 0.f);
            if (mine && a <= lim) {
                grad6_lane(L, g, axial, a, q, eps);
                if (tiso) spz_rtz(eps, s1, c1, s2, c2);
            }
            if (mine)
#pragma unroll
                for (int c = 0; c < 6; c++) F[(int64_t)a * ncolp + c * Pc + (p - p0)] = eps[c];
            for (int c = ncol + lane; c < ncolp; c += 32) F[(int64_t)a * ncolp + c] = make_float2(0.f, 0.f);
            __syncwarp();
        }
        __syncthreads();
        // ---- phase 2: C2R to nr samples ----
        phys_c2r(tw, F, X, nr, lim, ncolp);
        __syncthreads();
        // ---- phase 3: stress (+ SLS) per sample and point ----
        for (int t = threadIdx.x; t < nr * Pc; t += blockDim.x) {
            const int k = t / Pc, pp = t - k * Pc, pg = p0 + pp;
            float e6[6], s6[6];
#pragma unroll
            for (int c = 0; c < 6; c++) e6[c] = X[(int64_t)k * ncolp + c * Pc + pp];
            elastic(mat, e6, s6, [&](int m) { return md[((int64_t)m * nr + k) * NPE + pg]; });
            if (att) {
                const int qq = att == 2 ? cg4_index(pg) : pg;
                if (qq >= 0) {
                    float *R = mem + (int64_t)k * 6 * npa + qq;
                    float *SR = R + sls.nsls * sl;
                    for (int l = 0; l < sls.nsls; l++)
#pragma unroll
                        for (int c = 0; c < 6; c++) s6[c] -= R[l * sl + c * npa];
                    sls_update(sls, R, SR, sl, (int64_t)npa, e6, am[(int64_t)k * npa + qq],
                               am[(int64_t)nr * npa + (int64_t)k * npa + qq]);
                }
            }
#pragma unroll
            for (int c = 0; c < 6; c++) X[(int64_t)k * ncolp + c * Pc + pp] = s6[c];
        }
        __syncthreads();
        // ---- phase 4: R2C back to orders 0..lim ----
        phys_r2c(tw, X, F, nr, lim, ncolp);
        __syncthreads();
        // ---- phase 5: back-rotation + quad6, accumulate into the element force ----
        for (int a = warp; a < n; a += PH_WARPS) {
            float2 sig[6];
#pragma unroll
            for (int c = 0; c < 6; c++)
                sig[c] = (mine && a <= lim) ? F[(int64_t)a * ncolp + c * Pc + (p - p0)] : make_float2(0.f, 0.f);
            if (mine && tiso) rtz_spz(sig, s1, c1, s2, c2);
            float2 f[3];
            quad6_lane(L, g, axial, a, sig, q, active && a <= lim, f);
            if (active) {
                float2 *o = ef + ((int64_t)p * n + a) * 3;
                if (a > lim) f[0] = f[1] = f[2] = make_float2(0.f, 0.f);
                if (p0 == 0) {
                    o[0] = f[0];
                    o[1] = f[1];
                    o[2] = f[2];
                } else {
                    o[0] = cadd(o[0], f[0]);
                    o[1] = cadd(o[1], f[1]);
                    o[2] = cadd(o[2], f[2]);
                }
            }
        }
        __syncthreads();
    }
}

__global__ void __launch_bounds__(PH_THREADS)
    k_elem_phys_fluid(ElemTable T, PointTable P, const float2 *__restrict__ fu,
                      const int32_t *__restrict__ elems, int Pmax) {
    extern __shared__ __align__(16) char smem[];
    const int e = elems[blockIdx.x];
    const bool axial = T.flags[e] & EF_AXIAL;
    const int nr = T.nr[e], nu = nr / 2, n = nu + 1, lim = nu - (nr % 2 == 0);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    float2 *tw, *F, *scr;
    float *X;
    int ncolp;
    phys_layout<3>(nr, Pmax, tw, F, X, scr, ncolp, smem);
    fill_twiddles(tw, T, nr);
    float2 *q = scr + warp * QSCR;
    const bool active = lane < NPE;
    const int p = active ? lane : 0;
    LaneOps L;
    L.init(p, axial);
    Geo g;
    g.load(T.geo + (int64_t)e * 125, p);
    const int pt_me = T.pts[e * NPE + p];
    float2 *ef = T.ef + T.efofs[e];
    const float *md = T.moduli + T.mofs[e];
    for (int p0 = 0; p0 < NPE; p0 += Pmax) {
        const int Pc = min(Pmax, NPE - p0);
        const int ncol = 3 * Pc;
        const bool mine = active && p >= p0 && p < p0 + Pc;
        for (int a = warp; a < n; a += PH_WARPS) {
            if (active) q[p] = load_fluid_u(P, fu, pt_me, a);
            __syncwarp();
            float2 eps[3] = {make_float2(0.f, 0.f), make_float2(0.f, 0.f), make_float2(0.f, 0.f)};
            if (mine && a <= lim) grad1_lane(L, g, axial, a, q, eps);
            if (mine)
#pragma unroll
                for (int c = 0; c < 3; c++) F[(int64_t)a * ncolp + c * Pc + (p - p0)] = eps[c];
            for (int c = ncol + lane; c < ncolp; c += 32) F[(int64_t)a * ncolp + c] = make_float2(0.f, 0.f);
            __syncwarp();
        }
        __syncthreads();
        phys_c2r(tw, F, X, nr, lim, ncolp);
        __syncthreads();
        for (int t = threadIdx.x; t < nr * Pc; t += blockDim.x) {
            const int k = t / Pc, pp = t - k * Pc, pg = p0 + pp;
            const float K = md[(int64_t)k * NPE + pg];  // Acoustic3D.cpp:9-16
#pragma unroll
            for (int c = 0; c < 3; c++) X[(int64_t)k * ncolp + c * Pc + pp] *= K;
        }
        __syncthreads();
        phys_r2c(tw, X, F, nr, lim, ncolp);
        __syncthreads();
        for (int a = warp; a < n; a += PH_WARPS) {
            float2 sig[3];
#pragma unroll
            for (int c = 0; c < 3; c++)
                sig[c] = (mine && a <= lim) ? F[(int64_t)a * ncolp + c * Pc + (p - p0)] : make_float2(0.f, 0.f);
            float2 f;
            quad1_lane(L, g, axial, a, sig, q, active && a <= lim, f);
            if (active) {
                float2 *o = ef + (int64_t)p * n + a;
                if (a > lim) f = make_float2(0.f, 0.f);
                *o = (p0 == 0) ? f : cadd(*o, f);
            }
        }
        __syncthreads();
    }
}

void init_kernel_attributes() {
    cudaFuncSetAttribute(k_elem_phys_solid, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SMEM_MAX);
    cudaFuncSetAttribute(k_elem_phys_fluid, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SMEM_MAX);
}

void launch_elem_phys_solid(const ElemTable &T, const PointTable &P, const float2 *su,
                            const PhysBucket &b, const SLS &sls, cudaStream_t s) {
    if (b.count <= 0) return;
    k_elem_phys_solid<<<b.count, PH_THREADS, b.smem, s>>>(T, P, su, b.elems, b.npts_chunk, sls);
}
void launch_elem_phys_fluid(const ElemTable &T, const PointTable &P, const float2 *fu,
                            const PhysBucket &b, cudaStream_t s) {
    if (b.count <= 0) return;
    k_elem_phys_fluid<<<b.count, PH_THREADS, b.smem, s>>>(T, P, fu, b.elems, b.npts_chunk);
}

}  // namespace ax3d
