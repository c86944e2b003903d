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
constexpr int PH_THREADS = 512;
constexpr int PH_WARPS = PH_THREADS / 32;
constexpr int QSCR = 14 * 25;  // per-warp scratch (float2) for grad/quad
constexpr int CG = 16;         // DFT: column padding (warp tasks take 8 or 16 columns)
constexpr int RESEED = 8;      // DFT: exact twiddle reload interval
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
// Shared layout: tw[nr] float2 | F[n][SF] float2 | X[nr][SX] float.  The per-warp
// grad/quad scratch aliases X (X is dead in phases 1 and 5).  Column counts are padded
// to CG; SF = 2 (mod 16) and SX = 4 (mod 32) keep the row-wise vector stores of the
// transforms free of bank conflicts.
__host__ __device__ inline int round_up(int x, int m) { return (x + m - 1) / m * m; }
__host__ __device__ inline int stride_f(int ncolg) { return ncolg + 2; }                        // = 2 mod 16
__host__ __device__ inline int stride_x(int ncolg) { return ncolg + ((ncolg % 32) ? 20 : 4); }  // = 4 mod 32

size_t phys_smem_bytes(int nr, int ncomp, int npts_chunk) {
    const int n = nr / 2 + 1;
    const int ncolg = round_up(ncomp * npts_chunk, CG);
    const size_t tw = (size_t)8 * ((nr + 1) & ~1);
    const size_t F = (size_t)8 * n * stride_f(ncolg);
    const size_t X = (size_t)4 * nr * stride_x(ncolg);
    const size_t scr = (size_t)PH_WARPS * QSCR * 8;
    return tw + F + (X > scr ? X : scr);
}

int phys_points_per_chunk(int nr, int ncomp) {
    for (int nchunk = 1; nchunk <= NPE; nchunk++) {
        int P = (NPE + nchunk - 1) / nchunk;
        if (phys_smem_bytes(nr, ncomp, P) <= SMEM_MAX) return P;
    }
    return 0;  // does not fit even one point per pass
}

// C2R, lane = output sample: X[k][c] = Re F[0][c] + 2 sum_{a=1}^{lim} Re(F[a][c] w^{k a}),
// w = e^{i 2 pi / nr}, for k = 0..nr/2; the mirror sample nr - k follows from the parity of
// cos / sin.  Each warp task covers KL*32 samples x CG columns; F rows are read with
// broadcast vector loads, the twiddle w^{ka} is advanced by one complex rotation per
// order and reloaded exactly from the table every RESEED orders.
template <int KL, int CG>
__device__ __forceinline__ void c2r_task(const float2 *__restrict__ tw, const float2 *__restrict__ F, int SF,
                                         float *__restrict__ X, int SX, int nr, int lim, int kb, int c0, int lane) {
    const int kh = nr / 2 + 1;
    int k[KL], idx[KL];
    float2 w[KL], w1[KL];
    float cs[KL][CG], sn[KL][CG];
#pragma unroll
    for (int j = 0; j < KL; j++) {
        k[j] = kb * (32 * KL) + j * 32 + lane;
        const int kk = k[j] < kh ? k[j] : 0;
        idx[j] = kk;
        w1[j] = tw[kk];
        w[j] = w1[j];
#pragma unroll
        for (int c = 0; c < CG; c++) cs[j][c] = sn[j][c] = 0.f;
    }
    int step8[KL];
#pragma unroll
    for (int j = 0; j < KL; j++) step8[j] = (RESEED * (k[j] < kh ? k[j] : 0)) % nr;
    for (int a0 = 1; a0 <= lim; a0 += RESEED) {
        // exact twiddle w^{k a0} at the start of every block, rotations inside it
#pragma unroll
        for (int j = 0; j < KL; j++) w[j] = tw[idx[j]];
        const int aend = min(a0 + RESEED, lim + 1);
#pragma unroll 2
        for (int a = a0; a < aend; a++) {
            const float4 *fp = reinterpret_cast<const float4 *>(F + (int64_t)a * SF + c0);
#pragma unroll
            for (int q = 0; q < CG / 2; q++) {
                const float4 f = fp[q];
#pragma unroll
                for (int j = 0; j < KL; j++) {
                    cs[j][2 * q] = fmaf(f.x, w[j].x, cs[j][2 * q]);
                    sn[j][2 * q] = fmaf(f.y, w[j].y, sn[j][2 * q]);
                    cs[j][2 * q + 1] = fmaf(f.z, w[j].x, cs[j][2 * q + 1]);
                    sn[j][2 * q + 1] = fmaf(f.w, w[j].y, sn[j][2 * q + 1]);
                }
            }
#pragma unroll
            for (int j = 0; j < KL; j++) w[j] = cmul(w[j], w1[j]);
        }
#pragma unroll
        for (int j = 0; j < KL; j++) {
            idx[j] += step8[j];
            if (idx[j] >= nr) idx[j] -= nr;
        }
    }
    float f0[CG];
#pragma unroll
    for (int c = 0; c < CG; c++) f0[c] = F[c0 + c].x;
#pragma unroll
    for (int j = 0; j < KL; j++) {
        if (k[j] >= kh) continue;
        float4 *lo = reinterpret_cast<float4 *>(X + (int64_t)k[j] * SX + c0);
#pragma unroll
        for (int q = 0; q < CG / 4; q++)
            lo[q] = make_float4(f0[4 * q] + 2.f * (cs[j][4 * q] - sn[j][4 * q]),
                                f0[4 * q + 1] + 2.f * (cs[j][4 * q + 1] - sn[j][4 * q + 1]),
                                f0[4 * q + 2] + 2.f * (cs[j][4 * q + 2] - sn[j][4 * q + 2]),
                                f0[4 * q + 3] + 2.f * (cs[j][4 * q + 3] - sn[j][4 * q + 3]));
        const int km = nr - k[j];
        if (k[j] > 0 && km != k[j]) {
            float4 *hi = reinterpret_cast<float4 *>(X + (int64_t)km * SX + c0);
#pragma unroll
            for (int q = 0; q < CG / 4; q++)
                hi[q] = make_float4(f0[4 * q] + 2.f * (cs[j][4 * q] + sn[j][4 * q]),
                                    f0[4 * q + 1] + 2.f * (cs[j][4 * q + 1] + sn[j][4 * q + 1]),
                                    f0[4 * q + 2] + 2.f * (cs[j][4 * q + 2] + sn[j][4 * q + 2]),
                                    f0[4 * q + 3] + 2.f * (cs[j][4 * q + 3] + sn[j][4 * q + 3]));
        }
    }
}

// ---- mixed-radix FFT for ring sizes whose prime factors are all <= 13 -----------------
// (the FFT-friendly "lucky" sizes, PreloopFFTW.cpp:59-109).  Two real columns (2s, 2s+1)
// travel as one complex sequence z = x_2s + i x_2s+1; a self-sorting (Stockham) pass per
// radix, ping-ponging between the sample buffer X (viewed as complex [nr][SX/2]) and the
// order buffer F (viewed as complex [nr][ncolg/2]), one thread per (butterfly, sequence).
// Twiddles w^m come from the exact table; no recurrence.

constexpr int FFT_MIN = 16;   // below this the direct transform is as fast

// n / d for n < 2^32 by multiply-high (round-up method of Granlund and Montgomery)
struct FDiv {
    uint32_t m, s, d;
};
__device__ __forceinline__ FDiv make_fdiv(uint32_t d) {
    uint32_t s = 0;
    while ((1u << s) < d) s++;
    const uint64_t m = ((1ull << 32) * ((1ull << s) - d)) / d + 1;
    return FDiv{(uint32_t)m, s, d};
}
__device__ __forceinline__ uint32_t fdiv(uint32_t n, const FDiv &f) {
    if (f.d == 1) return n;
    const uint32_t t = __umulhi(n, f.m);
    return (t + ((n - t) >> 1)) >> (f.s - 1);
}

// true when every prime factor of n is at most 13
__host__ __device__ inline bool fft_size_ok(int n) {
    for (int p = 2; p <= 13; p++)
        while (n % p == 0) n /= p;
    return n == 1;
}

// v <- DFT_R(v) with e^{+2 pi i rk/R} (inv) or e^{-2 pi i rk/R}; cq/sq = cos/sin(2 pi q/R)
template <int R>
__device__ __forceinline__ void butterfly(float2 (&v)[R], bool inv, const float *cq, const float *sq) {
    if constexpr (R == 2) {
        const float2 a = v[0], b = v[1];
        v[0] = cadd(a, b);
        v[1] = make_float2(a.x - b.x, a.y - b.y);
    } else if constexpr (R == 4) {
        const float2 t0 = cadd(v[0], v[2]), t1 = make_float2(v[0].x - v[2].x, v[0].y - v[2].y);
        const float2 t2 = cadd(v[1], v[3]);
        const float2 d = make_float2(v[1].x - v[3].x, v[1].y - v[3].y);
        const float2 t3 = inv ? make_float2(-d.y, d.x) : make_float2(d.y, -d.x);  // +-i d
        v[0] = cadd(t0, t2);
        v[2] = make_float2(t0.x - t2.x, t0.y - t2.y);
        v[1] = cadd(t1, t3);
        v[3] = make_float2(t1.x - t3.x, t1.y - t3.y);
    } else {
        // odd R: out_k = v0 + sum_r (v_r + v_{R-r}) cos(2 pi rk/R) +- i (v_r - v_{R-r}) sin(..)
        constexpr int H = (R - 1) / 2;
        float2 sp[H], sm[H];
        float2 out0 = v[0];
#pragma unroll
        for (int r = 1; r <= H; r++) {
            sp[r - 1] = cadd(v[r], v[R - r]);
            sm[r - 1] = make_float2(v[r].x - v[R - r].x, v[r].y - v[R - r].y);
            out0 = cadd(out0, sp[r - 1]);
        }
        const float sg = inv ? 1.f : -1.f;
        float2 o[R];
        o[0] = out0;
#pragma unroll
        for (int k = 1; k <= H; k++) {
            float2 a = v[0], b = make_float2(0.f, 0.f);
#pragma unroll
            for (int r = 1; r <= H; r++) {
                const int q = (r * k) % R;
                a.x = fmaf(sp[r - 1].x, cq[q], a.x);
                a.y = fmaf(sp[r - 1].y, cq[q], a.y);
                b.x = fmaf(sm[r - 1].x, sq[q], b.x);
                b.y = fmaf(sm[r - 1].y, sq[q], b.y);
            }
            // i sg b = (-sg b.y, sg b.x)
            o[k] = make_float2(a.x - sg * b.y, a.y + sg * b.x);
            o[R - k] = make_float2(a.x + sg * b.y, a.y - sg * b.x);
        }
#pragma unroll
        for (int k = 0; k < R; k++) v[k] = o[k];
    }
}

// one Stockham pass of radix R over nseq sequences of length N (Ns = product of the
// radices already applied)
template <int R>
__device__ void fft_pass(const float2 *in, int Si, float2 *out, int So, int N, int Ns, int nseq,
                         const float2 *tw, bool inv, const FDiv &fseq) {
    const int m = N / R, step = N / (Ns * R);
    const FDiv fns = make_fdiv((uint32_t)Ns);
    constexpr bool ODD = (R % 2) == 1;
    float cq[ODD ? R : 1], sq[ODD ? R : 1];
    if constexpr (ODD) {
#pragma unroll
        for (int q = 0; q < R; q++) {
            const float2 w = tw[q * m];   // (cos, sin)(2 pi q / R)
            cq[q] = w.x;
            sq[q] = w.y;
        }
    }
    const int total = m * nseq;
    for (int t = threadIdx.x; t < total; t += blockDim.x) {
        const int j = (int)fdiv((uint32_t)t, fseq), s = t - j * nseq;
        const int jd = (int)fdiv((uint32_t)j, fns), jm = j - jd * Ns;
        float2 v[R];
#pragma unroll
        for (int r = 0; r < R; r++) v[r] = in[(int64_t)(j + r * m) * Si + s];
#pragma unroll
        for (int r = 1; r < R; r++) {
            float2 w = tw[jm * step * r];
            if (!inv) w.y = -w.y;
            v[r] = cmul(v[r], w);
        }
        butterfly<R>(v, inv, cq, sq);
        const int d = jd * Ns * R + jm;
#pragma unroll
        for (int r = 0; r < R; r++) out[(int64_t)(d + r * Ns) * So + s] = v[r];
    }
}

// all passes; returns the buffer holding the result (a or b)
__device__ int next_radix(int n) {
    return n % 4 == 0 ? 4 : n % 2 == 0 ? 2 : n % 3 == 0 ? 3 : n % 5 == 0 ? 5 : n % 7 == 0 ? 7 : n % 11 == 0 ? 11 : 13;
}

__device__ float2 *fft_run(float2 *a, int Sa, float2 *b, int Sb, int N, int nseq, const float2 *tw, bool inv,
                           const FDiv &fseq) {
    float2 *in = a, *out = b;
    int Si = Sa, So = Sb, Ns = 1;
    for (int rest = N; rest > 1;) {
        const int R = next_radix(rest);
        switch (R) {
            case 4: fft_pass<4>(in, Si, out, So, N, Ns, nseq, tw, inv, fseq); break;
            case 2: fft_pass<2>(in, Si, out, So, N, Ns, nseq, tw, inv, fseq); break;
            case 3: fft_pass<3>(in, Si, out, So, N, Ns, nseq, tw, inv, fseq); break;
            case 5: fft_pass<5>(in, Si, out, So, N, Ns, nseq, tw, inv, fseq); break;
            case 7: fft_pass<7>(in, Si, out, So, N, Ns, nseq, tw, inv, fseq); break;
            case 11: fft_pass<11>(in, Si, out, So, N, Ns, nseq, tw, inv, fseq); break;
            default: fft_pass<13>(in, Si, out, So, N, Ns, nseq, tw, inv, fseq); break;
        }
        __syncthreads();
        Ns *= R;
        rest /= R;
        float2 *tp = in;
        in = out;
        out = tp;
        const int ts = Si;
        Si = So;
        So = ts;
    }
    return in;
}

__device__ void copy_rows(const float2 *src, int Ss, float2 *dst, int Sd, int N, int nseq, const FDiv &fseq) {
    for (int t = threadIdx.x; t < N * nseq; t += blockDim.x) {
        const int k = (int)fdiv((uint32_t)t, fseq), s = t - k * nseq;
        dst[(int64_t)k * Sd + s] = src[(int64_t)k * Ss + s];
    }
}

// C2R by FFT: X[k][c] = Re F[0][c] + 2 sum_{a=1}^{lim} Re(F[a][c] w^{ka}) for all k < nr
__device__ void fft_c2r(const float2 *tw, float2 *F, int SF, float *X, int SX, int nr, int lim, int ncolg) {
    const int nseq = ncolg / 2, SZ = SX / 2;
    const FDiv fseq = make_fdiv((uint32_t)nseq);
    float2 *Zx = reinterpret_cast<float2 *>(X);
    // Hermitian extension of the column pair (2s, 2s+1), packed as A + i B
    for (int t = threadIdx.x; t < nr * nseq; t += blockDim.x) {
        const int k = (int)fdiv((uint32_t)t, fseq), s = t - k * nseq;
        float2 z = make_float2(0.f, 0.f);
        if (k == 0) {
            const float4 f = *reinterpret_cast<const float4 *>(F + 2 * s);
            z = make_float2(f.x, f.z);
        } else if (k <= lim) {
            const float4 f = *reinterpret_cast<const float4 *>(F + (int64_t)k * SF + 2 * s);
            z = make_float2(f.x - f.w, f.y + f.z);
        } else if (k >= nr - lim) {
            const float4 f = *reinterpret_cast<const float4 *>(F + (int64_t)(nr - k) * SF + 2 * s);
            z = make_float2(f.x + f.w, f.z - f.y);
        }
        Zx[(int64_t)k * SZ + s] = z;
    }
    __syncthreads();
    float2 *res = fft_run(Zx, SZ, F, nseq, nr, nseq, tw, true, fseq);
    if (res != Zx) {
        copy_rows(res, nseq, Zx, SZ, nr, nseq, fseq);
        __syncthreads();
    }
}

// R2C by FFT (after the stress phase): F[a][c] = (1/nr) sum_k X[k][c] w^{-ka}, a <= lim
__device__ void fft_r2c(const float2 *tw, float *X, int SX, float2 *F, int SF, int nr, int lim, int ncolg) {
    const int nseq = ncolg / 2, SZ = SX / 2;
    const FDiv fseq = make_fdiv((uint32_t)nseq);
    float2 *Zx = reinterpret_cast<float2 *>(X);
    float2 *res = fft_run(Zx, SZ, F, nseq, nr, nseq, tw, false, fseq);
    if (res != Zx) {
        copy_rows(res, nseq, Zx, SZ, nr, nseq, fseq);
        __syncthreads();
    }
    // split the packed spectra: A = (Z_a + conj Z_{nr-a}) / 2, B = (Z_a - conj Z_{nr-a}) / 2i
    const float h = 0.5f / (float)nr;
    for (int t = threadIdx.x; t < (lim + 1) * nseq; t += blockDim.x) {
        const int a = (int)fdiv((uint32_t)t, fseq), s = t - a * nseq;
        const float2 z1 = Zx[(int64_t)a * SZ + s];
        const float2 z2 = Zx[(int64_t)(a == 0 ? 0 : nr - a) * SZ + s];
        *reinterpret_cast<float4 *>(F + (int64_t)a * SF + 2 * s) =
            make_float4((z1.x + z2.x) * h, (z1.y - z2.y) * h, (z1.y + z2.y) * h, (z2.x - z1.x) * h);
    }
}

__device__ void phys_c2r(const float2 *tw, const float2 *F, int SF, float *X, int SX, int nr, int lim, int ncolg) {
    if (nr >= FFT_MIN && fft_size_ok(nr)) {
        fft_c2r(tw, const_cast<float2 *>(F), SF, X, SX, nr, lim, ncolg);
        return;
    }
    const int kh = nr / 2 + 1;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    if (kh >= 96) {
        const int ncg = ncolg / 8, nkb = (kh + 63) / 64;
        for (int t = warp; t < nkb * ncg; t += nw) c2r_task<2, 8>(tw, F, SF, X, SX, nr, lim, t / ncg, (t % ncg) * 8, lane);
    } else {
        const int ncg = ncolg / 16, nkb = (kh + 31) / 32;
        for (int t = warp; t < nkb * ncg; t += nw) c2r_task<1, 16>(tw, F, SF, X, SX, nr, lim, t / ncg, (t % ncg) * 16, lane);
    }
}

// In place: X[k] <- X[k] + X[nr-k], X[nr-k] <- X[k] - X[nr-k] for k = 1..(nr-1)/2.
__device__ void phys_fold(float *X, int SX, int nr, int ncolg) {
    const int k2 = (nr - 1) / 2;
    const int nq = ncolg / 4;
    for (int t = threadIdx.x; t < k2 * nq; t += blockDim.x) {
        const int k = 1 + t / nq, q = t - (k - 1) * nq;
        float4 *a = reinterpret_cast<float4 *>(X + (int64_t)k * SX) + q;
        float4 *b = reinterpret_cast<float4 *>(X + (int64_t)(nr - k) * SX) + q;
        const float4 x = *a, y = *b;
        *a = make_float4(x.x + y.x, x.y + y.y, x.z + y.z, x.w + y.w);
        *b = make_float4(x.x - y.x, x.y - y.y, x.z - y.z, x.w - y.w);
    }
}

// R2C (after phys_fold), lane = output order a = 0..lim, scaled by 1/nr:
// F[a] = (x_0 + sum_k s_k cos(k a t) + [nr even] (-1)^a x_{nr/2}, -sum_k d_k sin(k a t)) / nr.
template <int KL, int CG>
__device__ __forceinline__ void r2c_task(const float2 *__restrict__ tw, const float *__restrict__ X, int SX,
                                         float2 *__restrict__ F, int SF, int nr, int lim, int ab, int c0, int lane) {
    const int na = lim + 1, k2 = (nr - 1) / 2;
    int a[KL], idx[KL];
    float2 w[KL], w1[KL];
    float re[KL][CG], im[KL][CG];
#pragma unroll
    for (int j = 0; j < KL; j++) {
        a[j] = ab * (32 * KL) + j * 32 + lane;
        const int aa = a[j] < na ? a[j] : 0;
        idx[j] = aa;
        w1[j] = tw[aa];
        w[j] = w1[j];
#pragma unroll
        for (int c = 0; c < CG; c++) re[j][c] = im[j][c] = 0.f;
    }
    int step8[KL];
#pragma unroll
    for (int j = 0; j < KL; j++) step8[j] = (RESEED * (a[j] < na ? a[j] : 0)) % nr;
    for (int k0 = 1; k0 <= k2; k0 += RESEED) {
#pragma unroll
        for (int j = 0; j < KL; j++) w[j] = tw[idx[j]];
        const int kend = min(k0 + RESEED, k2 + 1);
#pragma unroll 2
        for (int k = k0; k < kend; k++) {
            const float4 *sp = reinterpret_cast<const float4 *>(X + (int64_t)k * SX + c0);
            const float4 *dp = reinterpret_cast<const float4 *>(X + (int64_t)(nr - k) * SX + c0);
#pragma unroll
            for (int q = 0; q < CG / 4; q++) {
                const float4 sv = sp[q], d = dp[q];
#pragma unroll
                for (int j = 0; j < KL; j++) {
                    re[j][4 * q] = fmaf(sv.x, w[j].x, re[j][4 * q]);
                    re[j][4 * q + 1] = fmaf(sv.y, w[j].x, re[j][4 * q + 1]);
                    re[j][4 * q + 2] = fmaf(sv.z, w[j].x, re[j][4 * q + 2]);
                    re[j][4 * q + 3] = fmaf(sv.w, w[j].x, re[j][4 * q + 3]);
                    im[j][4 * q] = fmaf(d.x, w[j].y, im[j][4 * q]);
                    im[j][4 * q + 1] = fmaf(d.y, w[j].y, im[j][4 * q + 1]);
                    im[j][4 * q + 2] = fmaf(d.z, w[j].y, im[j][4 * q + 2]);
                    im[j][4 * q + 3] = fmaf(d.w, w[j].y, im[j][4 * q + 3]);
                }
            }
#pragma unroll
            for (int j = 0; j < KL; j++) w[j] = cmul(w[j], w1[j]);
        }
#pragma unroll
        for (int j = 0; j < KL; j++) {
            idx[j] += step8[j];
            if (idx[j] >= nr) idx[j] -= nr;
        }
    }
    const float inv_nr = 1.f / (float)nr;
    float x0[CG], xn[CG];
#pragma unroll
    for (int c = 0; c < CG; c++) {
        x0[c] = X[c0 + c];
        xn[c] = (nr % 2 == 0) ? X[(int64_t)(nr / 2) * SX + c0 + c] : 0.f;
    }
#pragma unroll
    for (int j = 0; j < KL; j++) {
        if (a[j] >= na) continue;
        const float sgn = (a[j] & 1) ? -1.f : 1.f;
        float4 *o = reinterpret_cast<float4 *>(F + (int64_t)a[j] * SF + c0);
#pragma unroll
        for (int q = 0; q < CG / 2; q++)
            o[q] = make_float4((x0[2 * q] + re[j][2 * q] + sgn * xn[2 * q]) * inv_nr, -im[j][2 * q] * inv_nr,
                               (x0[2 * q + 1] + re[j][2 * q + 1] + sgn * xn[2 * q + 1]) * inv_nr,
                               -im[j][2 * q + 1] * inv_nr);
    }
}

__device__ void phys_r2c(const float2 *tw, float *X, int SX, float2 *F, int SF, int nr, int lim, int ncolg) {
    if (nr >= FFT_MIN && fft_size_ok(nr)) {
        fft_r2c(tw, X, SX, F, SF, nr, lim, ncolg);
        return;
    }
    phys_fold(X, SX, nr, ncolg);
    __syncthreads();
    const int na = lim + 1;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    if (na >= 96) {
        const int ncg = ncolg / 8, nab = (na + 63) / 64;
        for (int t = warp; t < nab * ncg; t += nw) r2c_task<2, 8>(tw, X, SX, F, SF, nr, lim, t / ncg, (t % ncg) * 8, lane);
    } else {
        const int ncg = ncolg / 16, nab = (na + 31) / 32;
        for (int t = warp; t < nab * ncg; t += nw) r2c_task<1, 16>(tw, X, SX, F, SF, nr, lim, t / ncg, (t % ncg) * 16, lane);
    }
}

// Twiddles (cos, sin)(2 pi m / nr), precomputed in FP64 on the host per distinct nr.
__device__ void fill_twiddles(float2 *tw, const ElemTable &T, int nr) {
    const float2 *src = T.twtab + T.twofs[nr];
    for (int m = threadIdx.x; m < nr; m += blockDim.x) tw[m] = src[m];
}

// Phase 3a of the physical-space solid kernel: SLS memory variables (Attenuation3D_Full
// / _CG4 applyToStress + updateMemoryVariables) with one thread per (sample, attenuated
// point, component): the loads of R and stressR are independent across threads and the
// dependent chain per thread is one load-update-store.  The sum of the old memory
// variables, which applyToStress subtracts from the stress, goes to dR[k][c][q] (the
// Fourier buffer, dead during this phase; 6 Pc nr floats fit in its n * SF complex).
__device__ __forceinline__ void sls_phase(const float *X, int SX, float *mem, const float *__restrict__ am,
                                          int64_t sl, int npa, int att, const SLS &sls, int nr, int Pc, int p0,
                                          float *dR) {
    // attenuated points: CG4 -> (6, 8, 16, 18) when inside this chunk; full -> all
    const int npts = att == 2 ? 4 : Pc;
    const int total = nr * npts * 6;
    const float third = (float)(1.0 / 3.0);
    for (int t = threadIdx.x; t < total; t += blockDim.x) {
        const int c = t % 6, r = t / 6, k = r / npts, j = r - k * npts;
        int pp, qq;
        if (att == 2) {
            const int pg = j < 2 ? 6 + 2 * j : 16 + 2 * (j - 2);
            if (pg < p0 || pg >= p0 + Pc) continue;
            pp = pg - p0;
            qq = j;
        } else {
            pp = j;
            qq = p0 + j;
        }
        float e[6];
#pragma unroll
        for (int i = 0; i < 6; i++) e[i] = X[(int64_t)k * SX + i * Pc + pp];
        float *R = mem + (int64_t)k * 6 * npa + (int64_t)c * npa + qq;
        float *SR = R + sls.nsls * sl;
        const float sr_old = *SR;
        const float dk = am[(int64_t)k * npa + qq], dmu = am[(int64_t)nr * npa + (int64_t)k * npa + qq];
        const float e3 = (e[0] + e[1] + e[2]) * third;
        float snew;
        if (c < 3) {
            if (sls.do_kappa) {
                snew = 3.f * dk * e3 + 2.f * dmu * (e[c] - e3);
            } else if (c < 2) {
                snew = 2.f * dmu * (e[c] - e3);
            } else {
                snew = -(2.f * dmu * (e[0] - e3) + 2.f * dmu * (e[1] - e3));
            }
        } else {
            snew = dmu * e[c];
        }
        float acc = 0.f;
        for (int l = 0; l < sls.nsls; l++) {
            const float r0 = R[l * sl];
            acc += r0;
            R[l * sl] = (sls.a[l] * r0 + sls.b[l] * sr_old) + sls.g[l] * snew;
        }
        *SR = snew;
        dR[((int64_t)k * 6 + c) * Pc + pp] = acc;
    }
}

// Phase 3b: strain -> stress at every (sample, point) of the chunk, in place in X, minus
// the memory-variable sum from phase 3a.  Each thread takes IT items and issues all their
// modulus loads before any arithmetic, so enough loads are in flight to keep HBM busy.
template <int MAT, int IT>
__device__ __forceinline__ void stress_phase(float *X, int SX, const float *__restrict__ md, int att,
                                             int nr, int Pc, int p0, const float *dR) {
    constexpr int NM = MAT == 0 ? 2 : MAT == 1 ? 5 : 21;
    const int total = nr * Pc;
    for (int t0 = threadIdx.x; t0 < total; t0 += blockDim.x * IT) {
        float mv[IT][NM];
#pragma unroll
        for (int i = 0; i < IT; i++) {
            const int t = t0 + i * blockDim.x;
            if (t < total) {
                const int k = t / Pc, pg = p0 + (t - k * Pc);
#pragma unroll
                for (int m = 0; m < NM; m++) mv[i][m] = __ldg(md + ((int64_t)m * nr + k) * NPE + pg);
            }
        }
#pragma unroll
        for (int i = 0; i < IT; i++) {
            const int t = t0 + i * blockDim.x;
            if (t >= total) break;
            const int k = t / Pc, pp = t - k * Pc, pg = p0 + pp;
            float e6[6], s6[6];
#pragma unroll
            for (int c = 0; c < 6; c++) e6[c] = X[(int64_t)k * SX + c * Pc + pp];
            elastic(MAT, e6, s6, [&](int m) { return mv[i][m]; });
            if (att && (att == 1 || cg4_index(pg) >= 0)) {
#pragma unroll
                for (int c = 0; c < 6; c++) s6[c] -= dR[((int64_t)k * 6 + c) * Pc + pp];
            }
#pragma unroll
            for (int c = 0; c < 6; c++) X[(int64_t)k * SX + c * Pc + pp] = s6[c];
        }
    }
}

struct PhysLayout {
    float2 *tw, *F, *scr;
    float *X;
    int ncolg, SF, SX;
    __device__ PhysLayout(char *smem, int nr, int ncomp, int Pmax) {
        const int n = nr / 2 + 1;
        ncolg = round_up(ncomp * Pmax, CG);
        SF = stride_f(ncolg);
        SX = stride_x(ncolg);
        tw = reinterpret_cast<float2 *>(smem);
        F = tw + ((nr + 1) & ~1);
        X = reinterpret_cast<float *>(F + (int64_t)n * SF);
        scr = reinterpret_cast<float2 *>(X);
    }
};

__global__ void __launch_bounds__(PH_THREADS, 1)
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
    PhysLayout S(smem, nr, 6, Pmax);
    float2 *tw = S.tw, *F = S.F;
    float *X = S.X;
    const int SF = S.SF, SX = S.SX;
    fill_twiddles(tw, T, nr);
    float2 *q = S.scr + warp * QSCR;
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
        const int ncolg = round_up(ncol, CG);
        const bool mine = active && p >= p0 && p < p0 + Pc;
        // ---- phase 1: strain (grad6 + rotation) of the chunk's points, all orders ----
        float2 un[3] = {make_float2(0.f, 0.f), make_float2(0.f, 0.f), make_float2(0.f, 0.f)};
        if (active && warp < n) load_solid_u(P, su, pt_me, warp, un);
        for (int a = warp; a < n; a += PH_WARPS) {
            if (active) {
                q[p] = un[0];
                q[25 + p] = un[1];
                q[50 + p] = un[2];
                if (a + PH_WARPS < n) load_solid_u(P, su, pt_me, a + PH_WARPS, un);  // prefetch
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
                for (int c = 0; c < 6; c++) F[(int64_t)a * SF + c * Pc + (p - p0)] = eps[c];
            for (int c = ncol + lane; c < ncolg; c += 32) F[(int64_t)a * SF + c] = make_float2(0.f, 0.f);
            __syncwarp();
        }
        __syncthreads();
        // ---- phase 2: C2R to nr samples ----
        phys_c2r(tw, F, SF, X, SX, nr, lim, ncolg);
        __syncthreads();
        // ---- phase 3: SLS update, then stress per sample and point ----
        float *dR = reinterpret_cast<float *>(F);  // nr * 6 * Pc floats (<= F size), F is dead here
        if (att) {
            sls_phase(X, SX, mem, am, sl, npa, att, sls, nr, Pc, p0, dR);
            __syncthreads();
        }
        if (mat == 0)
            stress_phase<0, 8>(X, SX, md, att, nr, Pc, p0, dR);
        else if (mat == 1)
            stress_phase<1, 4>(X, SX, md, att, nr, Pc, p0, dR);
        else
            stress_phase<2, 1>(X, SX, md, att, nr, Pc, p0, dR);
        __syncthreads();
        // ---- phase 4: R2C back to orders 0..lim ----
        phys_r2c(tw, X, SX, F, SF, nr, lim, ncolg);
        __syncthreads();
        // ---- phase 5: back-rotation + quad6, accumulate into the element force ----
        for (int a = warp; a < n; a += PH_WARPS) {
            float2 sig[6];
#pragma unroll
            for (int c = 0; c < 6; c++)
                sig[c] = (mine && a <= lim) ? F[(int64_t)a * SF + c * Pc + (p - p0)] : make_float2(0.f, 0.f);
            if (mine && tiso) rtz_spz(sig, s1, c1, s2, c2);
            float2 old[3] = {make_float2(0.f, 0.f), make_float2(0.f, 0.f), make_float2(0.f, 0.f)};
            float2 *o = ef + ((int64_t)p * n + a) * 3;
            if (active && p0 > 0) {  // issued before the divergence so the load overlaps it
                old[0] = o[0];
                old[1] = o[1];
                old[2] = o[2];
            }
            float2 f[3];
            quad6_lane(L, g, axial, a, sig, q, active && a <= lim, f);
            if (active) {
                if (a > lim) f[0] = f[1] = f[2] = make_float2(0.f, 0.f);
                o[0] = cadd(old[0], f[0]);
                o[1] = cadd(old[1], f[1]);
                o[2] = cadd(old[2], f[2]);
            }
        }
        __syncthreads();
    }
}

__global__ void __launch_bounds__(PH_THREADS, 1)
    k_elem_phys_fluid(ElemTable T, PointTable P, const float2 *__restrict__ fu,
                      const int32_t *__restrict__ elems, int Pmax) {
    extern __shared__ __align__(16) char smem[];
    const int e = elems[blockIdx.x];
    const bool axial = T.flags[e] & EF_AXIAL;
    const int nr = T.nr[e], nu = nr / 2, n = nu + 1, lim = nu - (nr % 2 == 0);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    PhysLayout S(smem, nr, 3, Pmax);
    float2 *tw = S.tw, *F = S.F;
    float *X = S.X;
    const int SF = S.SF, SX = S.SX;
    fill_twiddles(tw, T, nr);
    float2 *q = S.scr + warp * QSCR;
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
        const int ncolg = round_up(ncol, CG);
        const bool mine = active && p >= p0 && p < p0 + Pc;
        for (int a = warp; a < n; a += PH_WARPS) {
            if (active) q[p] = load_fluid_u(P, fu, pt_me, a);
            __syncwarp();
            float2 eps[3] = {make_float2(0.f, 0.f), make_float2(0.f, 0.f), make_float2(0.f, 0.f)};
            if (mine && a <= lim) grad1_lane(L, g, axial, a, q, eps);
            if (mine)
#pragma unroll
                for (int c = 0; c < 3; c++) F[(int64_t)a * SF + c * Pc + (p - p0)] = eps[c];
            for (int c = ncol + lane; c < ncolg; c += 32) F[(int64_t)a * SF + c] = make_float2(0.f, 0.f);
            __syncwarp();
        }
        __syncthreads();
        phys_c2r(tw, F, SF, X, SX, nr, lim, ncolg);
        __syncthreads();
        for (int t = threadIdx.x; t < nr * Pc; t += blockDim.x) {
            const int k = t / Pc, pp = t - k * Pc, pg = p0 + pp;
            const float K = md[(int64_t)k * NPE + pg];  // Acoustic3D.cpp:9-16
#pragma unroll
            for (int c = 0; c < 3; c++) X[(int64_t)k * SX + c * Pc + pp] *= K;
        }
        __syncthreads();
        phys_r2c(tw, X, SX, F, SF, nr, lim, ncolg);
        __syncthreads();
        for (int a = warp; a < n; a += PH_WARPS) {
            float2 sig[3];
#pragma unroll
            for (int c = 0; c < 3; c++)
                sig[c] = (mine && a <= lim) ? F[(int64_t)a * SF + c * Pc + (p - p0)] : make_float2(0.f, 0.f);
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
