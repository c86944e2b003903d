// ax3d_phys.cu -- physical-space element stiffness (3-D material) for sm_103a.
//
// Restates the 3-D branch of SolidElement::displToStiff and FluidElement::displToStiff
// (SOLVER/src/core/element/SolidElement.cpp:404-443, FluidElement.cpp:333-355): the
// gradient per Fourier order, FieldFFT::transformF2P to the nr azimuthal samples
// (FieldFFT.cpp:19-25; SolverFFTW_N6::computeC2R, unnormalised, SolverFFTW_N6.cpp:39-44),
// strain -> stress with the SLS memory variables at every sample, transformP2F
// (computeR2C then x 1/nr, SolverFFTW_N6.cpp:45-53) and the divergence per order.
//
// One CTA of 256 threads works on one element at a time; the grid is persistent over a
// bucket of elements of similar transform length, sized so that at least two CTAs are
// resident per SM and the HBM streams of one element overlap the arithmetic of another.
//
// Each pair of real strain columns (components 2s and 2s+1 of one GLL point) travels as
// one complex sequence z = a + i b of length L in shared memory, laid out
// [position][sequence] so that consecutive threads touch consecutive sequences.  The
// Hermitian spectra of a and b pack into z's spectrum as Z_k = A_k + i B_k and
// Z_{nr-k} = conj(A_k) + i conj(B_k).  The transforms run in place:
//  * mixed radix: decimation-in-frequency passes (radix 2, 3, 4, 5, 7, 11 and 13
//    butterflies in registers; a warp-cooperative symmetric direct DFT for a prime factor
//    above 13) take the spectrum in natural order to the samples in digit-reversed order.
//    The stress is computed there, with the sample index from a table, and
//    decimation-in-time passes take the reversed samples back to the natural spectrum.
//  * Bluestein (ring sizes with a large prime factor): the length-nr DFT as a chirp
//    convolution of smooth length M >= 2 nr - 1, with the same passes and the chirp
//    kernel's spectrum stored in digit-reversed order.
// All twiddles, chirps and kernel spectra are computed in FP64 on the host.
// When an element's sequences do not fit in one CTA's shared memory, a thread-block
// cluster of C CTAs (on C SMs) shares it: CTA r holds the sequences of GLL points
// [r Pc, (r + 1) Pc) and transforms them; the gradient and the divergence are split over
// the cluster by Fourier order and write / read the owning CTA's shared memory through
// distributed shared memory, so nothing leaves the chip between them.
#include <algorithm>
#include <cmath>
#include <complex>
#include <vector>

#include <cooperative_groups.h>

#include "ax3d_elem_ops.cuh"
#include "ax3d_kernels.cuh"

namespace cg = cooperative_groups;

namespace ax3d {

namespace {

constexpr int NT = 256;      // threads per CTA (512 for buckets of policy 2)
constexpr int WSCR = 125;    // per-warp grad / divergence scratch (float2)
constexpr int RESEED = 8;    // direct DFT: exact twiddle reload interval
constexpr int DIRECT_MAX = 257;  // largest prime handled by a direct pass
constexpr size_t SMEM_CAP = 227 * 1024;
constexpr size_t SMEM_TWO = 112 * 1024;  // two CTAs per SM
constexpr size_t SMEM_FOUR = 56 * 1024;  // four CTAs per SM
constexpr size_t SMEM_EIGHT = 27 * 1024; // eight CTAs per SM
constexpr int64_t PREFETCH_MAX = 1024 * 1024;  // largest per-element block asked of L2 ahead
constexpr int CLUSTER_MAX = 8;
constexpr int PLAN_BYTES = (sizeof(FftPlan) + 15) / 16 * 16;

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

__device__ __forceinline__ float2 conjf2(float2 a) { return make_float2(a.x, -a.y); }
// w_L^idx with the transform's sign (+1: e^{+i..}, -1: e^{-i..})
__device__ __forceinline__ float2 twv(const float2 *tw, int idx, int sg) {
    const float2 w = tw[idx];
    return sg > 0 ? w : make_float2(w.x, -w.y);
}

// The threads that share one set of sequences and the barrier between their passes.
struct Grp {
    int tid, n, warp, nwarp;
    bool cta;
    __device__ __forceinline__ void sync() const {
        if (cta)
            __syncthreads();
        else
            __syncwarp();
    }
};
__device__ __forceinline__ Grp grp_cta() {
    return Grp{(int)threadIdx.x, (int)blockDim.x, (int)(threadIdx.x >> 5), (int)(blockDim.x >> 5), true};
}

// v <- DFT_R(v) with e^{+2 pi i rk/R} (inv) or e^{-2 pi i rk/R}; cq/sq = cos/sin(2 pi q/R)
template <int R>
__device__ __forceinline__ void butterfly(float2 (&v)[R], bool inv, const float *cq, const float *sq) {
    if constexpr (R == 2) {
        const float2 a = v[0], b = v[1];
        v[0] = cadd(a, b);
        v[1] = csub(a, b);
    } else if constexpr (R == 4) {
        const float2 t0 = cadd(v[0], v[2]), t1 = csub(v[0], v[2]);
        const float2 t2 = cadd(v[1], v[3]), d = csub(v[1], v[3]);
        const float2 t3 = inv ? make_float2(-d.y, d.x) : make_float2(d.y, -d.x);  // +-i d
        v[0] = cadd(t0, t2);
        v[2] = csub(t0, t2);
        v[1] = cadd(t1, t3);
        v[3] = csub(t1, t3);
    } else {
        // odd R: out_k = v0 + sum_r (v_r + v_{R-r}) cos(2 pi rk/R) +- i (v_r - v_{R-r}) sin(..)
        constexpr int H = (R - 1) / 2;
        float2 sp[H], sm[H];
        float2 out0 = v[0];
#pragma unroll
        for (int r = 1; r <= H; r++) {
            sp[r - 1] = cadd(v[r], v[R - r]);
            sm[r - 1] = csub(v[r], v[R - r]);
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
                const int qk = (r * k) % R;
                a.x = fmaf(sp[r - 1].x, cq[qk], a.x);
                a.y = fmaf(sp[r - 1].y, cq[qk], a.y);
                b.x = fmaf(sm[r - 1].x, sq[qk], b.x);
                b.y = fmaf(sm[r - 1].y, sq[qk], b.y);
            }
            o[k] = make_float2(a.x - sg * b.y, a.y + sg * b.x);  // a + i sg b
            o[R - k] = make_float2(a.x + sg * b.y, a.y - sg * b.x);
        }
#pragma unroll
        for (int k = 0; k < R; k++) v[k] = o[k];
    }
}

// One in-place pass of radix R over ns sequences (row stride S) of length L; the pass
// works on blocks of length Ls with butterfly stride m = Ls / R.
//   DIF: butterfly, then output k of butterfly j times w_Ls^{jk}.
//   DIT: input k of butterfly j times w_Ls^{jk}, then butterfly.
template <int R>
__device__ __noinline__ void rad_pass(float2 *buf, int S, int ns, int L, int Ls, const float2 *tw, int sg, bool dit,
                                      const Grp g) {
    const int m = Ls / R, ts = L / Ls;
    const int total = (L / R) * ns;
    const FDiv fs = make_fdiv((uint32_t)ns), fm = make_fdiv((uint32_t)m);
    constexpr bool ODD = (R % 2) == 1;
    float cq[ODD ? R : 1], sq[ODD ? R : 1];
    if constexpr (ODD) {
#pragma unroll
        for (int qk = 0; qk < R; qk++) {
            const float2 w = tw[qk * (L / R)];
            cq[qk] = w.x;
            sq[qk] = w.y;
        }
    }
    // U butterflies per iteration, their shared-memory loads issued together (two for the
    // radices up to 5: four measured 0.4-3 % slower, the larger body costing instruction cache)
    constexpr int U = R <= 5 ? 2 : 1;
    const int64_t rs = (int64_t)m * S;
    for (int t0 = g.tid; t0 < total; t0 += g.n * U) {
        float2 v[U][R];
        float2 *p0[U];
        int jj[U];
#pragma unroll
        for (int uu = 0; uu < U; uu++) {
            const int t = min(t0 + uu * g.n, total - 1);
            const int bj = (int)fdiv((uint32_t)t, fs), s = t - bj * ns;
            const int b = (int)fdiv((uint32_t)bj, fm);
            jj[uu] = bj - b * m;
            p0[uu] = buf + (int64_t)(b * Ls + jj[uu]) * S + s;
#pragma unroll
            for (int r = 0; r < R; r++) v[uu][r] = p0[uu][r * rs];
        }
#pragma unroll
        for (int uu = 0; uu < U; uu++) {
            const int j = jj[uu];
            const bool ok = t0 + uu * g.n < total;
            if (dit) {
#pragma unroll
                for (int r = 1; r < R; r++) v[uu][r] = cmul(v[uu][r], twv(tw, j * r * ts, sg));
            }
            if constexpr (!ODD) {
                butterfly<R>(v[uu], sg > 0, cq, sq);
                if (!dit) {
#pragma unroll
                    for (int r = 1; r < R; r++) v[uu][r] = cmul(v[uu][r], twv(tw, j * r * ts, sg));
                }
                if (ok) {
#pragma unroll
                    for (int r = 0; r < R; r++) p0[uu][r * rs] = v[uu][r];
                }
            } else {
                // odd R: out_k = v0 + sum_r (v_r + v_{R-r}) cos(2 pi rk/R) +- i (v_r - v_{R-r})
                // sin(..); each pair (k, R - k) is stored as soon as it is formed (the
                // butterfly's inputs are all in registers, and only this thread owns them)
                constexpr int H = (R - 1) / 2;
                float2 sp[H], sm[H];
                float2 out0 = v[uu][0];
#pragma unroll
                for (int r = 1; r <= H; r++) {
                    sp[r - 1] = cadd(v[uu][r], v[uu][R - r]);
                    sm[r - 1] = csub(v[uu][r], v[uu][R - r]);
                    out0 = cadd(out0, sp[r - 1]);
                }
                const float2 x0 = v[uu][0];
                if (ok) p0[uu][0] = out0;
                const float sgf = sg > 0 ? 1.f : -1.f;
#pragma unroll
                for (int k = 1; k <= H; k++) {
                    float2 a = x0, bb = make_float2(0.f, 0.f);
#pragma unroll
                    for (int r = 1; r <= H; r++) {
                        const int qk = (r * k) % R;
                        a.x = fmaf(sp[r - 1].x, cq[qk], a.x);
                        a.y = fmaf(sp[r - 1].y, cq[qk], a.y);
                        bb.x = fmaf(sm[r - 1].x, sq[qk], bb.x);
                        bb.y = fmaf(sm[r - 1].y, sq[qk], bb.y);
                    }
                    float2 o1 = make_float2(a.x - sgf * bb.y, a.y + sgf * bb.x);  // a + i sg b
                    float2 o2 = make_float2(a.x + sgf * bb.y, a.y - sgf * bb.x);
                    if (!dit) {
                        o1 = cmul(o1, twv(tw, j * k * ts, sg));
                        o2 = cmul(o2, twv(tw, j * (R - k) * ts, sg));
                    }
                    if (ok) {
                        p0[uu][k * rs] = o1;
                        p0[uu][(R - k) * rs] = o2;
                    }
                }
            }
        }
    }
}

// One in-place pass of a prime radix p > 13 by the symmetric direct DFT.  A group of GS
// lanes owns one butterfly of SG sequences; lane gl computes outputs k = 1 + gl + GS q
// (q < KL) and p - k.  The group first replaces (v_r, v_{p-r}) by (v_r + v_{p-r},
// v_r - v_{p-r}) in place, then accumulates with twiddles advanced by complex rotation and
// reloaded exactly every RESEED orders, and writes after a warp barrier (only the group
// reads or writes its butterfly).
template <int GS, int KL, int SG>
__device__ __noinline__ void direct_pass(float2 *buf, int S, int ns, int L, int Ls, int p, const float2 *tw, int sg, bool dit,
                                         const Grp g) {
    const int H = (p - 1) >> 1, m = Ls / p, ts = L / Ls, ps = L / p;
    const int nsg = (ns + SG - 1) / SG;
    const int ntask = (L / Ls) * m * nsg;
    constexpr int GPW = 32 / GS;
    const int lane = threadIdx.x & 31, gi = lane / GS, gl = lane - gi * GS;
    const int warp = g.warp, nw = g.nwarp;
    const FDiv fn = make_fdiv((uint32_t)nsg), fm = make_fdiv((uint32_t)m);
    const int64_t rs = (int64_t)m * S;
    for (int t0 = warp * GPW; t0 < ntask; t0 += nw * GPW) {
        const int t = t0 + gi;
        const bool act = t < ntask;
        const int tt = act ? t : 0;
        const int bj = (int)fdiv((uint32_t)tt, fn), sgi = tt - bj * nsg;
        const int b = (int)fdiv((uint32_t)bj, fm), j = bj - b * m;
        const int s0 = sgi * SG;
        const int nv = act ? min(SG, ns - s0) : 0;
        float2 *base = buf + (int64_t)(b * Ls + j) * S + s0;
        // (DIT input twiddles and) sums / differences, in place
        for (int r = 1 + gl; r <= H; r += GS) {
            float2 wr = make_float2(1.f, 0.f), wm = make_float2(1.f, 0.f);
            if (dit) {
                wr = twv(tw, j * r * ts, sg);
                wm = twv(tw, j * (p - r) * ts, sg);
            }
#pragma unroll
            for (int s = 0; s < SG; s++) {
                if (s < nv) {
                    float2 a = base[r * rs + s], c = base[(p - r) * rs + s];
                    if (dit) {
                        a = cmul(a, wr);
                        c = cmul(c, wm);
                    }
                    base[r * rs + s] = cadd(a, c);
                    base[(p - r) * rs + s] = csub(a, c);
                }
            }
        }
        __syncwarp();
        float2 v0[SG], sum0[SG], ca[KL][SG], cb[KL][SG];
#pragma unroll
        for (int s = 0; s < SG; s++) {
            v0[s] = s < nv ? base[s] : make_float2(0.f, 0.f);
            sum0[s] = make_float2(0.f, 0.f);
#pragma unroll
            for (int qk = 0; qk < KL; qk++) ca[qk][s] = cb[qk][s] = make_float2(0.f, 0.f);
        }
        int idx[KL], step[KL];
        float2 w[KL], w1[KL];
#pragma unroll
        for (int qk = 0; qk < KL; qk++) {
            const int k = 1 + gl + GS * qk;
            const int kk = k <= H ? k : 0;
            idx[qk] = (kk * ps) % L;  // w_p^{k r} at r = 1
            step[qk] = (RESEED * kk * ps) % L;
            w1[qk] = tw[idx[qk]];
            w[qk] = w1[qk];
        }
        for (int r0 = 1; r0 <= H; r0 += RESEED) {
#pragma unroll
            for (int qk = 0; qk < KL; qk++) w[qk] = tw[idx[qk]];
            const int rend = min(r0 + RESEED, H + 1);
            for (int r = r0; r < rend; r++) {
                float2 sp[SG], sm[SG];
#pragma unroll
                for (int s = 0; s < SG; s++) {
                    sp[s] = s < nv ? base[r * rs + s] : make_float2(0.f, 0.f);
                    sm[s] = s < nv ? base[(p - r) * rs + s] : make_float2(0.f, 0.f);
                    sum0[s] = cadd(sum0[s], sp[s]);
                }
#pragma unroll
                for (int qk = 0; qk < KL; qk++) {
#pragma unroll
                    for (int s = 0; s < SG; s++) {
                        ca[qk][s].x = fmaf(w[qk].x, sp[s].x, ca[qk][s].x);
                        ca[qk][s].y = fmaf(w[qk].x, sp[s].y, ca[qk][s].y);
                        cb[qk][s].x = fmaf(w[qk].y, sm[s].x, cb[qk][s].x);
                        cb[qk][s].y = fmaf(w[qk].y, sm[s].y, cb[qk][s].y);
                    }
                    w[qk] = cmul(w[qk], w1[qk]);
                }
            }
#pragma unroll
            for (int qk = 0; qk < KL; qk++) {
                idx[qk] += step[qk];
                if (idx[qk] >= L) idx[qk] -= L;
            }
        }
        __syncwarp();
#pragma unroll
        for (int qk = 0; qk < KL; qk++) {
            const int k = 1 + gl + GS * qk;
            if (k > H) continue;
            float2 wk = make_float2(1.f, 0.f), wpk = make_float2(1.f, 0.f);
            if (!dit) {
                wk = twv(tw, j * k * ts, sg);
                wpk = twv(tw, j * (p - k) * ts, sg);
            }
#pragma unroll
            for (int s = 0; s < SG; s++) {
                if (s < nv) {
                    const float2 a = cadd(v0[s], ca[qk][s]), bb = cb[qk][s];
                    const float2 ib = sg > 0 ? make_float2(-bb.y, bb.x) : make_float2(bb.y, -bb.x);
                    float2 ok = cadd(a, ib), opk = csub(a, ib);
                    if (!dit) {
                        ok = cmul(ok, wk);
                        opk = cmul(opk, wpk);
                    }
                    base[k * rs + s] = ok;
                    base[(p - k) * rs + s] = opk;
                }
            }
        }
        if (gl == 0) {
#pragma unroll
            for (int s = 0; s < SG; s++)
                if (s < nv) base[s] = cadd(v0[s], sum0[s]);
        }
        __syncwarp();
    }
}

__device__ void run_pass(int R, float2 *buf, int S, int ns, int L, int Ls, const float2 *tw, int sg, bool dit,
                         const Grp g) {
    switch (R) {
        case 2: rad_pass<2>(buf, S, ns, L, Ls, tw, sg, dit, g); break;
        case 3: rad_pass<3>(buf, S, ns, L, Ls, tw, sg, dit, g); break;
        case 4: rad_pass<4>(buf, S, ns, L, Ls, tw, sg, dit, g); break;
        case 5: rad_pass<5>(buf, S, ns, L, Ls, tw, sg, dit, g); break;
        case 7: rad_pass<7>(buf, S, ns, L, Ls, tw, sg, dit, g); break;
        case 11: rad_pass<11>(buf, S, ns, L, Ls, tw, sg, dit, g); break;
        case 13: rad_pass<13>(buf, S, ns, L, Ls, tw, sg, dit, g); break;
        default: {
            // the narrowest group whose lanes cover the H = (R - 1) / 2 output pairs with at
            // most three outputs each (four for R above 193), two sequences per group: five
            // instantiations in all, so that CTAs of different rings on one SM share little
            // instruction cache (measured: 4.9 % faster on rings up to 91 samples than a
            // cost-model choice among 26 instantiations, 0.8 % on the full Nu 8-256 mix)
            const int H = (R - 1) / 2;
            if (H <= 12)
                direct_pass<4, 3, 2>(buf, S, ns, L, Ls, R, tw, sg, dit, g);
            else if (H <= 24)
                direct_pass<8, 3, 2>(buf, S, ns, L, Ls, R, tw, sg, dit, g);
            else if (H <= 48)
                direct_pass<16, 3, 2>(buf, S, ns, L, Ls, R, tw, sg, dit, g);
            else if (H <= 96)
                direct_pass<32, 3, 2>(buf, S, ns, L, Ls, R, tw, sg, dit, g);
            else
                direct_pass<32, 4, 2>(buf, S, ns, L, Ls, R, tw, sg, dit, g);
        }
    }
}

// All passes of a plan: DIF (natural -> reversed) or DIT (reversed -> natural).
__device__ void fft_passes(float2 *buf, int S, int ns, const FftPlan &pl, const float2 *tw, int sg, bool dit,
                           const Grp g) {
    const int L = pl.L;
    if (!dit) {
        int Ls = L;
        for (int i = 0; i < pl.nrad; i++) {
            run_pass(pl.rad[i], buf, S, ns, L, Ls, tw, sg, false, g);
            g.sync();
            Ls /= pl.rad[i];
        }
    } else {
        int Ls = 1;
        for (int i = pl.nrad - 1; i >= 0; i--) {
            Ls *= pl.rad[i];
            run_pass(pl.rad[i], buf, S, ns, L, Ls, tw, sg, true, g);
            g.sync();
        }
    }
}

// buf[pos] *= K[pos] over L positions; with save >= 0 the zero-frequency sum at position
// 0 is first kept in slot save (Rader).
__device__ void pointwise(float2 *buf, int S, int ns, int L, const float2 *__restrict__ K, int save, const Grp g) {
    const FDiv fs = make_fdiv((uint32_t)ns);
    for (int t = g.tid; t < L * ns; t += g.n) {
        const int pos = (int)fdiv((uint32_t)t, fs), s = t - pos * ns;
        const float2 v = buf[(int64_t)pos * S + s];
        if (save >= 0 && pos == 0) buf[(int64_t)save * S + s] = v;
        buf[(int64_t)pos * S + s] = cmul(v, __ldg(K + pos));
    }
    g.sync();
}

// spectrum -> samples: mixed radix leaves them digit-reversed, Bluestein natural (before the
// post-chirp h_k, which the stress phase applies), Rader in generator order (before the
// zero-frequency term, which the stress phase adds)
__device__ void transform_c2r(float2 *buf, int S, int ns, int nr, const FftPlan &pl, const float2 *tw,
                              const float2 *f2, const Grp g) {
    if (pl.kind == 0) {
        fft_passes(buf, S, ns, pl, tw, +1, false, g);
    } else {
        fft_passes(buf, S, ns, pl, tw, -1, false, g);
        pointwise(buf, S, ns, pl.L, f2 + pl.bc2r, pl.kind == 2 ? nr : -1, g);
        fft_passes(buf, S, ns, pl, tw, +1, true, g);
    }
}
// samples -> spectrum; scaled by 1/nr in the extraction (mixed radix) or in the kernel
// spectrum (Bluestein, Rader)
__device__ void transform_r2c(float2 *buf, int S, int ns, int nr, const FftPlan &pl, const float2 *tw,
                              const float2 *f2, const Grp g) {
    if (pl.kind == 0) {
        fft_passes(buf, S, ns, pl, tw, -1, true, g);
    } else {
        fft_passes(buf, S, ns, pl, tw, -1, false, g);
        pointwise(buf, S, ns, pl.L, f2 + pl.br2c, pl.kind == 2 ? nr - 1 : -1, g);
        fft_passes(buf, S, ns, pl, tw, +1, true, g);
    }
}

// Where an element's orders and samples live in its packed sequences.
struct Pk {
    int kind, nr;
    const float2 *chirp;  // kind 1
    const int32_t *ord;   // kind 2: order -> position (shared memory)
    float inv_nr;
};

// Hermitian packing of order a of the column pair (A, B) into sequence col.
__device__ __forceinline__ void zput(float2 *buf, int S, int col, int a, const Pk &k, float2 A, float2 B) {
    if (a == 0) {
        // only Re of order 0 enters the C2R
        buf[(int64_t)(k.kind == 2 ? k.nr - 1 : 0) * S + col] = make_float2(A.x, B.x);
        return;
    }
    float2 z1 = make_float2(A.x - B.y, A.y + B.x);  // A + i B
    float2 z2 = make_float2(A.x + B.y, B.x - A.y);  // conj(A) + i conj(B)
    int s1 = a, s2 = k.nr - a;
    if (k.kind == 1) {
        z1 = cmul(z1, __ldg(k.chirp + a));
        z2 = cmul(z2, __ldg(k.chirp + k.nr - a));
    } else if (k.kind == 2) {
        s1 = k.ord[a];
        s2 = k.ord[k.nr - a];
    }
    buf[(int64_t)s1 * S + col] = z1;
    buf[(int64_t)s2 * S + col] = z2;
}
// Order a of the column pair of sequence col from the transformed spectrum (x h).
__device__ __forceinline__ void zget(const float2 *buf, int S, int col, int a, const Pk &k, float h, float2 &A,
                                     float2 &B) {
    float2 z1, z2;
    if (k.kind == 2) {
        const float2 x0 = buf[(int64_t)k.nr * S + col];
        if (a == 0) {
            z1 = z2 = cscale(k.inv_nr, cadd(x0, buf[(int64_t)(k.nr - 1) * S + col]));
        } else {
            const float2 xs = cscale(k.inv_nr, x0);
            z1 = cadd(buf[(int64_t)k.ord[a] * S + col], xs);
            z2 = cadd(buf[(int64_t)k.ord[k.nr - a] * S + col], xs);
        }
    } else {
        z1 = buf[(int64_t)a * S + col];
        z2 = a == 0 ? z1 : buf[(int64_t)(k.nr - a) * S + col];
        if (k.kind == 1) {
            z1 = cmul(z1, conjf2(__ldg(k.chirp + a)));
            z2 = a == 0 ? z1 : cmul(z2, conjf2(__ldg(k.chirp + k.nr - a)));
        }
    }
    A = make_float2((z1.x + z2.x) * h, (z1.y - z2.y) * h);
    B = make_float2((z1.y + z2.y) * h, (z2.x - z1.x) * h);
}

// Sample of position pos in the transformed sequences: its azimuth index k, its slot,
// and (Bluestein) the chirp factor, (Rader) the zero-frequency slot to add.
struct SampleAt {
    int k, slot;
    float2 h;
    __device__ __forceinline__ SampleAt(int pos, const Pk &pk, const int32_t *rev) {
        h = make_float2(1.f, 0.f);
        if (pk.kind == 1) {
            k = slot = pos;
            h = __ldg(pk.chirp + pos);
        } else {
            k = rev[pos];
            slot = (pk.kind == 2 && pos == pk.nr - 1) ? pk.nr : pos;
        }
    }
};
__device__ __forceinline__ float2 sample_in(const float2 *buf, int S, int col, const SampleAt &sa, const Pk &pk) {
    float2 v = buf[(int64_t)sa.slot * S + col];
    if (pk.kind == 1) v = cmul(v, sa.h);
    if (pk.kind == 2) v = cadd(v, buf[(int64_t)(pk.nr - 1) * S + col]);
    return v;
}
__device__ __forceinline__ void sample_out(float2 *buf, int S, int col, const SampleAt &sa, const Pk &pk, float2 v) {
    buf[(int64_t)sa.slot * S + col] = pk.kind == 1 ? cmul(v, conjf2(sa.h)) : v;
}

// scatterDisplToElement (SolidPoint.cpp:175-195): orders above the point's Nu, and its
// Nyquist order, read as zero.  The point's block and order limit are read once.
struct USrc {
    const float2 *base;
    int plim;
    __device__ void init(const PointTable &P, const float2 *u, bool solid, int pt) {
        const int pnr = P.nr[pt];
        plim = pnr / 2 - (pnr % 2 == 0);
        base = u + (solid ? P.sofs[pt] : P.fofs[pt]);
    }
    __device__ __forceinline__ void load(bool solid, int a, float2 v[3]) const {
        v[0] = v[1] = v[2] = make_float2(0.f, 0.f);
        if (a > plim) return;
        if (solid) {
            const float2 *s = base + (int64_t)a * 3;
            v[0] = s[0];
            v[1] = s[1];
            v[2] = s[2];
        } else {
            v[0] = base[a];
        }
    }
};

// Ask L2 for slice `part` of `parts` of [ptr, ptr + bytes), ahead of a phase that reads it
// in scattered order.
__device__ __forceinline__ void prefetch_l2(const void *ptr, int64_t bytes, int part = 0, int parts = 1) {
    const char *c = static_cast<const char *>(ptr);
    const int64_t lo = bytes * part / parts, hi = bytes * (part + 1) / parts;
    const int64_t first = (reinterpret_cast<uintptr_t>(c) + lo) & 127;
    for (int64_t o = lo + (int64_t)threadIdx.x * 128 - first; o < hi; o += (int64_t)blockDim.x * 128)
        if (o >= lo) asm volatile("prefetch.global.L2 [%0];" ::"l"(c + o));
}

// Divergence of one Fourier order (computeQuad6, Gradient.cpp:267-317) with one
// component at a time through a 5 x 25 scratch.
__device__ __forceinline__ void quad6_split(const LaneOps &L, const Geo &g, bool axial, int beta,
                                            const float2 sig[6], float2 *q, bool active, float2 f[3]) {
    const int p = L.i * 5 + L.j;
    const float b = -(float)beta;
#pragma unroll
    for (int c = 0; c < 3; c++) {
        if (active) {
            float2 X, Y, gg;
            if (c == 0) {
                X = cadd(cscale(g.dzdeta, sig[0]), cscale(g.dsdeta, sig[4]));
                Y = cadd(cscale(g.dzdxii, sig[0]), cscale(g.dsdxii, sig[4]));
                gg = cadd(sig[1], cimul(b, sig[5]));
            } else if (c == 1) {
                X = cadd(cscale(g.dzdeta, sig[5]), cscale(g.dsdeta, sig[3]));
                Y = cadd(cscale(g.dzdxii, sig[5]), cscale(g.dsdxii, sig[3]));
                gg = csub(cimul(b, sig[1]), sig[5]);
            } else {
                X = cadd(cscale(g.dzdeta, sig[4]), cscale(g.dsdeta, sig[2]));
                Y = cadd(cscale(g.dzdxii, sig[4]), cscale(g.dsdxii, sig[2]));
                gg = cimul(b, sig[3]);
            }
            q[p] = X;
            q[25 + p] = Y;
            q[50 + p] = gg;
            q[75 + p] = cscale(g.dzdeta, gg);   // DzDeta o g (axial column term)
            q[100 + p] = cscale(g.dzdxii, gg);  // DzDxii o g (axial, beta = 1)
        }
        __syncwarp();
        if (active) {
            float2 acc = make_float2(0.f, 0.f), acc2 = make_float2(0.f, 0.f);
#pragma unroll
            for (int k = 0; k < 5; k++) {
                const float2 x = q[k * 5 + L.j], y = q[25 + L.i * 5 + k];
                acc.x += L.gxr[k] * x.x;
                acc.y += L.gxr[k] * x.y;
                acc2.x += y.x * L.ger[k];
                acc2.y += y.y * L.ger[k];
            }
            float2 fc = cadd(cadd(acc, acc2), cscale(g.inv_s, q[50 + p]));
            if (axial) {
                fc = cadd(fc, cscale(L.gxr[0], q[75 + L.j]));  // Gradient.cpp:300-303
                if (beta == 1 && L.i == 0 && c < 2) {            // Gradient.cpp:304-307
                    float2 h = make_float2(0.f, 0.f);
#pragma unroll
                    for (int k = 0; k < 5; k++) {
                        const float2 t = q[100 + k];
                        h.x += t.x * L.ger[k];
                        h.y += t.y * L.ger[k];
                    }
                    fc = cadd(fc, h);
                }
            }
            f[c] = fc;
        }
        __syncwarp();
    }
}

struct PhysSmem {
    float2 *tw, *buf, *wscr;
    int32_t *rev, *ord, *lst;
    FftPlan *pl;  // this element's plan
    __device__ PhysSmem(char *smem, int Lmax, int S) {
        pl = reinterpret_cast<FftPlan *>(smem);
        tw = reinterpret_cast<float2 *>(smem + PLAN_BYTES);
        rev = reinterpret_cast<int32_t *>(tw + Lmax);
        ord = rev + ((Lmax + 1) & ~1);
        lst = ord + ((Lmax + 1) & ~1);
        buf = reinterpret_cast<float2 *>(lst + 64);
        wscr = buf + (int64_t)Lmax * S;
    }
};

}  // namespace

size_t phys_smem_bytes(int Lmax, int nsq, int npts_chunk, int nthreads) {
    return (size_t)PLAN_BYTES + (size_t)8 * Lmax + (size_t)8 * ((Lmax + 1) & ~1) + 4 * 64 + (size_t)8 * Lmax * nsq * npts_chunk +
           (size_t)8 * (nthreads / 32) * WSCR;
}

// ------------------------------------------------------------------------------------
// Phases.  Each is a separate (not inlined) function so that registers are allocated per
// phase: the per-lane element operators live only in the gradient and divergence.
// ------------------------------------------------------------------------------------
namespace {

// Phase 1 of the first chunk: gradient (computeGrad6 / computeGrad, with the RTZ
// rotation for TI) of every order at all 25 points, warp per order and lane per point;
// points of the chunk go into the packed sequences, the others into the scratch.
template <bool SOLID>
__device__ __noinline__ void phase_grad(const ElemTable &T, const PointTable &P, const float2 *u, int e, int nr,
                                        bool axial, bool tiso, const Pk pk, float2 *buf, int S, int Pc, int crank,
                                        int C, float2 *q) {
    constexpr int NSQ = SOLID ? 3 : 2;
    constexpr int NC = SOLID ? 6 : 3;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const bool active = lane < NPE;
    const int p = active ? lane : 0;
    const int nu = nr / 2, n = nu + 1, lim = nu - (nr % 2 == 0);
    // sequences of point p live in cluster CTA p / Pc
    float2 *ob = cg::this_cluster().map_shared_rank(buf, p / Pc);
    const int col0 = NSQ * (p - (p / Pc) * Pc);
    LaneOps Lo;
    Lo.init(p, axial);
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
    USrc us;
    us.init(P, u, SOLID, T.pts[e * NPE + p]);
    // this CTA's orders: a = crank nw + warp + k C nw (nw warps per CTA); the displacement
    // of the next two of them is in flight while one is differentiated
    const int nwc = (int)(blockDim.x >> 5);
    const int a0 = crank * nwc + warp, da = C * nwc;
    float2 un[3], un2[3];
    if (active) {
        us.load(SOLID, a0, un);
        us.load(SOLID, a0 + da, un2);
    }
    for (int a = a0; a < n; a += da) {
        if (active) {
            q[p] = un[0];
            if (SOLID) {
                q[25 + p] = un[1];
                q[50 + p] = un[2];
            }
#pragma unroll
            for (int i = 0; i < 3; i++) un[i] = un2[i];
            us.load(SOLID, a + 2 * da, un2);
        }
        __syncwarp();
        if (active && a <= lim) {
            float2 eps[NC];
            if constexpr (SOLID) {
                grad6_lane(Lo, g, axial, a, q, eps);
                if (tiso) spz_rtz(eps, s1, c1, s2, c2);
            } else {
                grad1_lane(Lo, g, axial, a, q, eps);
            }
#pragma unroll
            for (int s = 0; s < NSQ; s++)
                zput(ob, S, col0 + s, a, pk, eps[2 * s], 2 * s + 1 < NC ? eps[2 * s + 1] : make_float2(0.f, 0.f));
        }
        __syncwarp();
    }
}

// Phase 3, points without memory variables: elastic stress at every sample.  Each thread
// takes IT items and issues all their modulus loads before any arithmetic.
template <int MAT>
__device__ __noinline__ void phase_stress(float2 *buf, int S, int nr, int ne_, const int32_t *lst, const int32_t *rev,
                                          const float *md, const Pk pk, int p0, const Grp g) {
    constexpr int NM = MAT == 0 ? 2 : MAT == 1 ? 5 : 21;
    constexpr int IT = MAT == 2 ? 1 : MAT == 1 ? 2 : 8;
    const int total = nr * ne_;
    const FDiv fe = make_fdiv((uint32_t)ne_);
    for (int t0 = g.tid; t0 < total; t0 += g.n * IT) {
        float mv[IT][NM];
        int kk[IT];
#pragma unroll
        for (int i = 0; i < IT; i++) {
            const int t = min(t0 + i * g.n, total - 1);
            const int pos = (int)fdiv((uint32_t)t, fe), pg = p0 + lst[t - pos * ne_];
            kk[i] = pk.kind == 1 ? pos : rev[pos];
#pragma unroll
            for (int mm = 0; mm < NM; mm++) mv[i][mm] = __ldg(md + ((int64_t)mm * nr + kk[i]) * NPE + pg);
        }
#pragma unroll
        for (int i = 0; i < IT; i++) {
            const int t = t0 + i * g.n;
            if (t >= total) break;
            const int pos = (int)fdiv((uint32_t)t, fe), pp = lst[t - pos * ne_];
            const SampleAt sa(pos, pk, rev);
            float2 zz[3];
#pragma unroll
            for (int s = 0; s < 3; s++) zz[s] = sample_in(buf, S, 3 * pp + s, sa, pk);
            const float e6[6] = {zz[0].x, zz[0].y, zz[1].x, zz[1].y, zz[2].x, zz[2].y};
            float s6[6];
            elastic(MAT, e6, s6, [&](int mm) { return mv[i][mm]; });
#pragma unroll
            for (int s = 0; s < 3; s++) sample_out(buf, S, 3 * pp + s, sa, pk, make_float2(s6[2 * s], s6[2 * s + 1]));
        }
    }
}

// Phase 3, attenuated points: elastic stress minus the memory variables (applyToStress),
// then updateMemoryVariables (Attenuation3D_Full.cpp:16-50, Attenuation3D_CG4.cpp:16-62).
// All loads of an item (moduli, every memory variable, stressR, the two attenuation
// moduli) are issued together and the memory variables stay in registers for the update,
// so an item costs one round trip to memory.  LMAX (>= nsls) bounds the registers held.
template <int MAT, int LMAX>
__device__ __noinline__ void phase_stress_att(float2 *buf, int S, int nr, int na_, const int32_t *lst,
                                              const int32_t *rev, const float *md, const Pk pk, int p0,
                                              int att, float *mem, const float *am, const SLS &sls, const Grp g) {
    constexpr int NM = MAT == 0 ? 2 : MAT == 1 ? 5 : 21;
    const int npa = att == 2 ? 4 : NPE;
    const int64_t sl = (int64_t)nr * 6 * npa;
    const int total = nr * na_;
    const int nsls = sls.nsls;
    const FDiv fa = make_fdiv((uint32_t)na_);
    const float third = (float)(1.0 / 3.0);
    for (int t = g.tid; t < total; t += g.n) {
        const int pos = (int)fdiv((uint32_t)t, fa), pp = lst[t - pos * na_], pg = p0 + pp;
        const int qq = att == 2 ? cg4_index(pg) : pg;
        const int k = pk.kind == 1 ? pos : rev[pos];
        float mv[NM], rv[LMAX][6], sr[6];
#pragma unroll
        for (int mm = 0; mm < NM; mm++) mv[mm] = __ldg(md + ((int64_t)mm * nr + k) * NPE + pg);
        float *R = mem + (int64_t)k * 6 * npa + qq;
#pragma unroll
        for (int l = 0; l < LMAX; l++)
#pragma unroll
            for (int c = 0; c < 6; c++) rv[l][c] = l < nsls ? R[l * sl + c * npa] : 0.f;
#pragma unroll
        for (int c = 0; c < 6; c++) sr[c] = R[nsls * sl + c * npa];
        const float dk = am[(int64_t)k * npa + qq], dm = am[(int64_t)nr * npa + (int64_t)k * npa + qq];
        const SampleAt sa(pos, pk, rev);
        float2 zz[3];
#pragma unroll
        for (int s = 0; s < 3; s++) zz[s] = sample_in(buf, S, 3 * pp + s, sa, pk);
        const float e6[6] = {zz[0].x, zz[0].y, zz[1].x, zz[1].y, zz[2].x, zz[2].y};
        float s6[6];
        elastic(MAT, e6, s6, [&](int mm) { return mv[mm]; });
        // applyToStress: sigma -= R_l, one solid after another
#pragma unroll
        for (int l = 0; l < LMAX; l++)
            if (l < nsls)
#pragma unroll
                for (int c = 0; c < 6; c++) s6[c] -= rv[l][c];
        // updateMemoryVariables: R_l <- a_l R_l + b_l stressR_old + g_l stressR_new
        const float dk3 = 3.f * dk, dmu2 = 2.f * dm;
        const float e3 = third * ((e6[0] + e6[1]) + e6[2]);
        float sn[6];
        if (sls.do_kappa) {
            const float sii3 = dk3 * e3;
            sn[0] = sii3 + dmu2 * (e6[0] - e3);
            sn[1] = sii3 + dmu2 * (e6[1] - e3);
            sn[2] = sii3 + dmu2 * (e6[2] - e3);
        } else {
            sn[0] = dmu2 * (e6[0] - e3);
            sn[1] = dmu2 * (e6[1] - e3);
            sn[2] = -(sn[0] + sn[1]);
        }
        sn[3] = dm * e6[3];
        sn[4] = dm * e6[4];
        sn[5] = dm * e6[5];
#pragma unroll
        for (int l = 0; l < LMAX; l++)
            if (l < nsls)
#pragma unroll
                for (int c = 0; c < 6; c++)
                    R[l * sl + c * npa] = (sls.a[l] * rv[l][c] + sls.b[l] * sr[c]) + sls.g[l] * sn[c];
#pragma unroll
        for (int c = 0; c < 6; c++) R[nsls * sl + c * npa] = sn[c];
#pragma unroll
        for (int s = 0; s < 3; s++) sample_out(buf, S, 3 * pp + s, sa, pk, make_float2(s6[2 * s], s6[2 * s + 1]));
    }
}

// Phase 3 of a fluid element: sigma_i = K d_i chi (Acoustic3D.cpp:9-16) at every sample.
__device__ __noinline__ void phase_stress_fluid(float2 *buf, int S, int nr, int pc, const int32_t *rev,
                                                const float *md, const Pk pk, int p0, const Grp g) {
    const FDiv fp = make_fdiv((uint32_t)pc);
    for (int t = g.tid; t < nr * pc; t += g.n) {
        const int pos = (int)fdiv((uint32_t)t, fp), pp = t - pos * pc;
        const SampleAt sa(pos, pk, rev);
        const float K = __ldg(md + (int64_t)sa.k * NPE + p0 + pp);
#pragma unroll
        for (int s = 0; s < 2; s++) sample_out(buf, S, 2 * pp + s, sa, pk, cscale(K, sample_in(buf, S, 2 * pp + s, sa, pk)));
    }
}

// Phase 6: divergence (computeQuad6 / computeQuad, after the TI back-rotation) of every
// order into the element force; the last chunk's stress spectra come from the packed
// sequences, the earlier chunks' from the scratch.
template <bool SOLID>
__device__ __noinline__ void phase_quad(const ElemTable &T, const PointTable &P, int e, int nr, bool axial,
                                        bool tiso, bool direct, bool rmw, const Pk pk, float hsc, float2 *buf, int S,
                                        int Pc, int crank, int C, float2 *q) {
    constexpr int NSQ = SOLID ? 3 : 2;
    constexpr int NC = SOLID ? 6 : 3;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const bool active = lane < NPE;
    const int p = active ? lane : 0;
    const int nu = nr / 2, n = nu + 1, lim = nu - (nr % 2 == 0);
    const float2 *ob = cg::this_cluster().map_shared_rank(buf, p / Pc);
    const int col0 = NSQ * (p - (p / Pc) * Pc);
    LaneOps Lo;
    Lo.init(p, axial);
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
    float2 *ef = T.ef + T.efofs[e];
    // direct assembly (gatherStiffFromElement, SolidPoint.cpp:197-209, for the point's only
    // element): stiff -= force up to the point's own Nyquist limit, its Nyquist row zeroed
    float2 *st = nullptr;
    int pnu = 0, plim = 0;
    if (SOLID && direct) {
        const int pt = T.pts[e * NPE + p];
        const int pnr = P.nr[pt];
        pnu = pnr / 2;
        plim = pnu - (pnr % 2 == 0);
        st = T.stiff + P.sofs[pt];
    }
    const int nwc = (int)(blockDim.x >> 5);
    for (int a = crank * nwc + warp; a < n; a += C * nwc) {
        float2 old[3] = {make_float2(0.f, 0.f), make_float2(0.f, 0.f), make_float2(0.f, 0.f)};
        const bool row = SOLID && direct && active && a <= pnu;
        if (rmw && row && a <= plim) {  // issued before the divergence so the loads overlap it
            old[0] = st[(int64_t)a * 3];
            old[1] = st[(int64_t)a * 3 + 1];
            old[2] = st[(int64_t)a * 3 + 2];
        }
        float2 sig[NC];
#pragma unroll
        for (int i = 0; i < NC; i++) sig[i] = make_float2(0.f, 0.f);
        if (active && a <= lim) {
#pragma unroll
            for (int s = 0; s < NSQ; s++) {
                float2 A, B;
                zget(ob, S, col0 + s, a, pk, hsc, A, B);
                sig[2 * s] = A;
                if (2 * s + 1 < NC) sig[2 * s + 1] = B;
            }
        }
        if constexpr (SOLID) {
            if (active && tiso) rtz_spz(sig, s1, c1, s2, c2);
            float2 f[3];
            quad6_split(Lo, g, axial, a, sig, q, active && a <= lim, f);
            if (a > lim) f[0] = f[1] = f[2] = make_float2(0.f, 0.f);
            if (direct) {
                if (row) {
                    float2 *o = st + (int64_t)a * 3;
                    const bool keep = a <= plim;
                    o[0] = keep ? csub(old[0], f[0]) : make_float2(0.f, 0.f);
                    o[1] = keep ? csub(old[1], f[1]) : make_float2(0.f, 0.f);
                    o[2] = keep ? csub(old[2], f[2]) : make_float2(0.f, 0.f);
                }
            } else if (active) {
                float2 *o = ef + ((int64_t)p * n + a) * 3;
                o[0] = f[0];
                o[1] = f[1];
                o[2] = f[2];
            }
        } else {
            float2 f;
            quad1_lane(Lo, g, axial, a, sig, q, active && a <= lim, f);
            if (active) ef[(int64_t)p * n + a] = a <= lim ? f : make_float2(0.f, 0.f);
        }
    }
}

}  // namespace

// ------------------------------------------------------------------------------------
// The kernel: SOLID = 6 strain components (3 sequences per point), else the fluid's 3
// potential-gradient components (2 sequences per point).
// ------------------------------------------------------------------------------------
template <bool SOLID, int NTT>
__global__ void __launch_bounds__(NTT, NTT == 64 ? 8 : NTT == 128 ? 4 : NTT == 256 ? 2 : 1)
    k_elem_phys(const __grid_constant__ ElemTable T, const __grid_constant__ PointTable P,
                const float2 *__restrict__ u, const int32_t *__restrict__ elems, int count, int Pc, int Lmax,
                const __grid_constant__ PhysTables X, const __grid_constant__ SLS sls, int overwrite) {
    constexpr int NSQ = SOLID ? 3 : 2;
    extern __shared__ __align__(16) char smem[];
    cg::cluster_group cl = cg::this_cluster();
    const int crank = (int)cl.block_rank(), C = (int)cl.num_blocks();
    // a barrier over the cluster (with its shared-memory fence) only when there is one
    auto csync = [&]() {
        if (C > 1)
            cl.sync();
        else
            __syncthreads();
    };
    const int S = NSQ * Pc;
    PhysSmem sm(smem, Lmax, S);
    float2 *tw = sm.tw, *buf = sm.buf;
    float2 *q = sm.wscr + (threadIdx.x >> 5) * WSCR;
    // this CTA's GLL points
    const int p0 = crank * Pc, pc = min(Pc, NPE - p0), ns = NSQ * pc;

    int have_nr = -1;  // ring size whose plan and tables the shared memory holds
    for (int ei = blockIdx.x / C; ei < count; ei += gridDim.x / C) {
        const int e = elems[ei];
        const int flags = T.flags[e];
        const bool axial = flags & EF_AXIAL;
        const int nr = T.nr[e];
        const int mat = ef_mat(flags), att = SOLID ? ef_att(flags) : 0;
        const bool tiso = SOLID && (mat == 1 || mat == 2);
        csync();  // the whole cluster is done with the previous element's sequences
        // the plan and its tables in shared memory (the transform passes read them once per
        // pass), loaded only when the ring size changes: bucket lists are sorted by it
        const bool reload = nr != have_nr;
        if (reload) {
            if (threadIdx.x < (int)(sizeof(FftPlan) / 4))
                reinterpret_cast<int32_t *>(sm.pl)[threadIdx.x] =
                    reinterpret_cast<const int32_t *>(X.plans + nr)[threadIdx.x];
            __syncthreads();
        }
        have_nr = nr;
        const FftPlan &pl = *sm.pl;
        const int L = pl.L, Lb = pl.Lbuf;
        const bool blue = pl.kind == 1;
        Pk pk;
        pk.kind = pl.kind;
        pk.nr = nr;
        pk.chirp = X.f2 + pl.chirp;
        pk.ord = sm.ord;
        pk.inv_nr = 1.f / (float)nr;
        const float hsc = pl.kind == 0 ? 0.5f / (float)nr : 0.5f;
        const float *md = T.moduli + T.mofs[e];
        if (reload) {
            for (int m = threadIdx.x; m < L; m += blockDim.x) tw[m] = X.f2[pl.tw + m];
            if (!blue)
                for (int m = threadIdx.x; m < nr; m += blockDim.x) sm.rev[m] = X.i32[pl.rev + m];
            if (pl.kind == 2)
                for (int m = threadIdx.x; m < nr; m += blockDim.x) sm.ord[m] = X.i32[pl.ord + m];
        }
        // positions the packing does not write: the Nyquist order (even nr) and the
        // Bluestein padding [nr, Lb)
        if (nr % 2 == 0)
            for (int s = threadIdx.x; s < ns; s += blockDim.x) buf[(int64_t)(nr / 2) * S + s] = make_float2(0.f, 0.f);
        if (blue)
            for (int t = threadIdx.x; t < (Lb - nr) * ns; t += blockDim.x)
                buf[(int64_t)(nr + t / ns) * S + t % ns] = make_float2(0.f, 0.f);
        __syncthreads();  // the order table is read by the packing in phase 1
        // ---- phase 1: Hermitian-packed strain spectra (this CTA's orders, all points) ----
        phase_grad<SOLID>(T, P, u, e, nr, axial, tiso, pk, buf, S, Pc, crank, C, q);
        if constexpr (SOLID) {
            // the stress phase's moduli and memory variables, asked of L2 while the C2R
            // runs; each CTA of a cluster asks for its share
            const int nm = mat == 0 ? 2 : mat == 1 ? 5 : 21;
            const int npa = att == 2 ? 4 : NPE;
            const int64_t sb = (int64_t)4 * nr * (NPE * nm + (att ? (sls.nsls + 1) * 6 * npa + 2 * npa : 0));
            if (sb <= PREFETCH_MAX) {
                prefetch_l2(md, (int64_t)4 * NPE * nr * nm, crank, C);
                if (att) {
                    prefetch_l2(T.mem + T.memofs[e], (int64_t)4 * (sls.nsls + 1) * nr * 6 * npa, crank, C);
                    prefetch_l2(T.attm + T.aofs[e], (int64_t)4 * 2 * nr * npa, crank, C);
                }
            }
        }
        csync();
        // ---- phases 2-4: the CTA's points, all its threads on each pass ----
        {
            const Grp g = grp_cta();
            const int gp0 = 0, gpc = pc;
            float2 *gbuf = buf;
            const int gns = ns;
            int32_t *lst = sm.lst;
            // the group's point lists: elastic-only and attenuated
            if (g.tid == 0) {
                int ne_ = 0, na_ = 0;
                for (int pp = 0; pp < gpc; pp++) {
                    const int pg = p0 + gp0 + pp;
                    if (att == 1 || (att == 2 && cg4_index(pg) >= 0))
                        lst[32 + na_++] = pp;
                    else
                        lst[ne_++] = pp;
                }
                lst[30] = ne_;
                lst[31] = na_;
            }
            g.sync();
            // ---- phase 2: to the nr azimuthal samples ----
            transform_c2r(gbuf, S, gns, nr, pl, tw, X.f2, g);
            // ---- phase 3: stress at every sample (SLS where attenuated) ----
            const int gpg = p0 + gp0;  // global index of the group's first point
            if constexpr (SOLID) {
                const int ne_ = lst[30], na_ = lst[31];
                if (ne_ > 0) {
                    if (mat == 0)
                        phase_stress<0>(gbuf, S, nr, ne_, lst, sm.rev, md, pk, gpg, g);
                    else if (mat == 1)
                        phase_stress<1>(gbuf, S, nr, ne_, lst, sm.rev, md, pk, gpg, g);
                    else
                        phase_stress<2>(gbuf, S, nr, ne_, lst, sm.rev, md, pk, gpg, g);
                }
                if (na_ > 0) {
                    float *mem = T.mem + T.memofs[e];
                    const float *am = T.attm + T.aofs[e];
                    if (sls.nsls <= 3) {
                        if (mat == 0)
                            phase_stress_att<0, 3>(gbuf, S, nr, na_, lst + 32, sm.rev, md, pk, gpg, att, mem, am, sls, g);
                        else if (mat == 1)
                            phase_stress_att<1, 3>(gbuf, S, nr, na_, lst + 32, sm.rev, md, pk, gpg, att, mem, am, sls, g);
                        else
                            phase_stress_att<2, 3>(gbuf, S, nr, na_, lst + 32, sm.rev, md, pk, gpg, att, mem, am, sls, g);
                    } else {
                        if (mat == 0)
                            phase_stress_att<0, 8>(gbuf, S, nr, na_, lst + 32, sm.rev, md, pk, gpg, att, mem, am, sls, g);
                        else if (mat == 1)
                            phase_stress_att<1, 8>(gbuf, S, nr, na_, lst + 32, sm.rev, md, pk, gpg, att, mem, am, sls, g);
                        else
                            phase_stress_att<2, 8>(gbuf, S, nr, na_, lst + 32, sm.rev, md, pk, gpg, att, mem, am, sls, g);
                    }
                }
            } else {
                phase_stress_fluid(gbuf, S, nr, gpc, sm.rev, md, pk, gpg, g);
            }
            if (blue)
                for (int t = g.tid; t < (Lb - nr) * gns; t += g.n)
                    gbuf[(int64_t)(nr + t / gns) * S + t % gns] = make_float2(0.f, 0.f);
            g.sync();
            // ---- phase 4: back to orders 0..lim ----
            transform_r2c(gbuf, S, gns, nr, pl, tw, X.f2, g);
        }
        csync();
        // ---- phase 5: divergence of this CTA's orders, all points, into the element force ----
        phase_quad<SOLID>(T, P, e, nr, axial, tiso, (flags & EF_DIRECT) != 0, !overwrite || (flags & EF_SOURCE), pk, hsc,
                          buf, S, Pc, crank, C, q);
    }
    csync();  // no CTA leaves while a peer may still read its shared memory
}

// PRT_3D elements (PRT_3D.cpp, with FieldFFT's C2R / R2C x 1/nr) on the element pass's
// transforms.  k_prt3_grad leaves the relabelled-frame gradient spectra of every order in the
// Fourier-space scratch w [alpha][nc][25]; here one CTA per (element, chunk of Pc points)
// packs each point's nc columns in pairs into complex sequences, transforms them to the nr
// samples, relabels (X), computes the stress (+ SLS) and relabels back at every sample, and
// transforms back into w, orders 0..nr/2; k_prt3_quad takes the divergence.
template <bool SOLID>
__global__ void __launch_bounds__(NT, 2)
    k_prt3_fft(const __grid_constant__ ElemTable T, const int32_t *__restrict__ elems, int nchunk, int Pc, int Lmax,
               const __grid_constant__ PhysTables X, const __grid_constant__ SLS sls) {
    constexpr int NC = SOLID ? 9 : 3;
    constexpr int NSQ = (NC + 1) / 2;
    extern __shared__ __align__(16) char smem[];
    const int S = NSQ * Pc;
    PhysSmem sm(smem, Lmax, S);
    float2 *buf = sm.buf;
    const int e = elems[blockIdx.x / nchunk], p0 = (blockIdx.x % nchunk) * Pc;
    const int pc = min(Pc, NPE - p0), ns = NSQ * pc;
    const int flags = T.flags[e];
    const int nr = T.nr[e], nu = nr / 2, lim = nu - (nr % 2 == 0);
    const Grp g = grp_cta();
    if (threadIdx.x < (int)(sizeof(FftPlan) / 4))
        reinterpret_cast<int32_t *>(sm.pl)[threadIdx.x] = reinterpret_cast<const int32_t *>(X.plans + nr)[threadIdx.x];
    __syncthreads();
    const FftPlan &pl = *sm.pl;
    const int L = pl.L, Lb = pl.Lbuf;
    const bool blue = pl.kind == 1;
    for (int m = threadIdx.x; m < L; m += blockDim.x) sm.tw[m] = X.f2[pl.tw + m];
    if (!blue)
        for (int m = threadIdx.x; m < nr; m += blockDim.x) sm.rev[m] = X.i32[pl.rev + m];
    if (pl.kind == 2)
        for (int m = threadIdx.x; m < nr; m += blockDim.x) sm.ord[m] = X.i32[pl.ord + m];
    Pk pk;
    pk.kind = pl.kind;
    pk.nr = nr;
    pk.chirp = X.f2 + pl.chirp;
    pk.ord = sm.ord;
    pk.inv_nr = 1.f / (float)nr;
    const float hsc = pl.kind == 0 ? 0.5f / (float)nr : 0.5f;
    // positions the packing does not write: the Nyquist order (even nr), the Bluestein padding
    if (nr % 2 == 0)
        for (int t = threadIdx.x; t < ns; t += blockDim.x) buf[(int64_t)nu * S + t] = make_float2(0.f, 0.f);
    if (blue)
        for (int t = threadIdx.x; t < (Lb - nr) * ns; t += blockDim.x)
            buf[(int64_t)(nr + t / ns) * S + t % ns] = make_float2(0.f, 0.f);
    __syncthreads();  // the order table is read by the packing
    float2 *w = T.w + T.wofs[e] + p0;
    // orders 0..lim of column pair (2s, 2s + 1) of point pp -> sequence NSQ pp + s
    for (int t = threadIdx.x; t < (lim + 1) * ns; t += blockDim.x) {
        const int a = t / ns, col = t - a * ns, pp = col / NSQ, sq = col - pp * NSQ;
        const float2 *wa = w + (int64_t)a * NC * NPE + pp;
        const float2 A = wa[2 * sq * NPE];
        const float2 B = 2 * sq + 1 < NC ? wa[(2 * sq + 1) * NPE] : make_float2(0.f, 0.f);
        zput(buf, S, col, a, pk, A, B);
    }
    __syncthreads();
    transform_c2r(buf, S, ns, nr, pl, sm.tw, X.f2, g);
    const float *xp = T.prtx + T.prtofs[e];
    const float *md = T.moduli + T.mofs[e];
    for (int t = threadIdx.x; t < nr * pc; t += blockDim.x) {
        const int pos = t / pc, pp = t - pos * pc, p = p0 + pp;
        const SampleAt sa(pos, pk, sm.rev);
        const int k = sa.k;
        float v[2 * NSQ];
#pragma unroll
        for (int sq = 0; sq < NSQ; sq++) {
            const float2 z = sample_in(buf, S, NSQ * pp + sq, sa, pk);
            v[2 * sq] = z.x;
            v[2 * sq + 1] = z.y;
        }
        auto xf = [&](int m) { return xp[((int64_t)m * nr + k) * NPE + p]; };
        if constexpr (SOLID) {
            float und[6], sig[6];
            prt_s2u(v, und, xf);
            elastic(ef_mat(flags), und, sig, [&](int m) { return md[((int64_t)m * nr + k) * NPE + p]; });
            const int att = ef_att(flags);
            if (att) {
                const int npa = att == 2 ? 4 : NPE;
                const int qq = att == 2 ? cg4_index(p) : p;
                if (qq >= 0) {
                    float *mem = T.mem + T.memofs[e];
                    const int64_t sl = (int64_t)nr * 6 * npa;
                    float *R = mem + (int64_t)k * 6 * npa + qq;
                    float *SR = R + sls.nsls * sl;
                    for (int l = 0; l < sls.nsls; l++)
#pragma unroll
                        for (int c = 0; c < 6; c++) sig[c] -= R[l * sl + c * npa];
                    const float *am = T.attm + T.aofs[e];
                    sls_update(sls, R, SR, sl, (int64_t)npa, und, am[(int64_t)k * npa + qq],
                               am[(int64_t)nr * npa + (int64_t)k * npa + qq]);
                }
            }
            prt_u2s(sig, v, xf);
            v[9] = 0.f;
        } else {
            prt_s2u_fluid(v, xf);
            const float K = md[(int64_t)k * NPE + p];
#pragma unroll
            for (int c = 0; c < 3; c++) v[c] *= K;
            prt_u2s_fluid(v, xf);
            v[3] = 0.f;
        }
#pragma unroll
        for (int sq = 0; sq < NSQ; sq++) sample_out(buf, S, NSQ * pp + sq, sa, pk, make_float2(v[2 * sq], v[2 * sq + 1]));
    }
    if (blue) {
        __syncthreads();
        for (int t = threadIdx.x; t < (Lb - nr) * ns; t += blockDim.x)
            buf[(int64_t)(nr + t / ns) * S + t % ns] = make_float2(0.f, 0.f);
    }
    __syncthreads();
    transform_r2c(buf, S, ns, nr, pl, sm.tw, X.f2, g);
    // orders 0..nr/2 (x 1/nr) back into w (the divergence drops the Nyquist order)
    for (int t = threadIdx.x; t < (nu + 1) * ns; t += blockDim.x) {
        const int a = t / ns, col = t - a * ns, pp = col / NSQ, sq = col - pp * NSQ;
        float2 A, B;
        zget(buf, S, col, a, pk, hsc, A, B);
        float2 *wa = w + (int64_t)a * NC * NPE + pp;
        wa[2 * sq * NPE] = A;
        if (2 * sq + 1 < NC) wa[(2 * sq + 1) * NPE] = B;
    }
}

// ------------------------------------------------------------------------------------
// host side
// ------------------------------------------------------------------------------------
void set_g_matrices_phys(const float *g_gll, const float *g_glj, cudaStream_t s) {
    cudaMemcpyToSymbolAsync(c_G, g_gll, 25 * sizeof(float), 0, cudaMemcpyHostToDevice, s);
    cudaMemcpyToSymbolAsync(c_G, g_glj, 25 * sizeof(float), 25 * sizeof(float), cudaMemcpyHostToDevice, s);
}

void init_phys_attributes() {
    cudaFuncSetAttribute(k_elem_phys<true, NT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SMEM_CAP);
    cudaFuncSetAttribute(k_elem_phys<false, NT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SMEM_CAP);
    cudaFuncSetAttribute(k_elem_phys<true, 2 * NT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SMEM_CAP);
    cudaFuncSetAttribute(k_elem_phys<false, 2 * NT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SMEM_CAP);
    cudaFuncSetAttribute(k_elem_phys<true, NT / 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SMEM_CAP);
    cudaFuncSetAttribute(k_elem_phys<false, NT / 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SMEM_CAP);
    cudaFuncSetAttribute(k_elem_phys<true, NT / 4>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SMEM_CAP);
    cudaFuncSetAttribute(k_elem_phys<false, NT / 4>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SMEM_CAP);
    cudaFuncSetAttribute(k_prt3_fft<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SMEM_CAP);
    cudaFuncSetAttribute(k_prt3_fft<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SMEM_CAP);
}

// Points per CTA of the PRT_3D transform pass for sequences of Lmax buffer positions: all 25
// if they fit two CTAs per SM, else the most that do, else the most that fit one CTA per SM;
// 0 if not even one point fits.
int prt3_points_per_cta(bool solid, int Lmax) {
    const int nsq = solid ? 5 : 2;
    for (size_t cap : {SMEM_TWO, SMEM_CAP})
        for (int pc = NPE; pc >= 1; pc--)
            if (phys_smem_bytes(Lmax, nsq, pc, NT) <= cap) return pc;
    return 0;
}

void launch_prt3_fft(bool solid, const ElemTable &T, const int32_t *elems, int nelem, int Lmax, const PhysTables &X,
                     const SLS &sls, cudaStream_t s) {
    const int pc = prt3_points_per_cta(solid, Lmax);
    if (nelem <= 0 || pc <= 0) return;
    const int nchunk = (NPE + pc - 1) / pc;
    const size_t smem = phys_smem_bytes(Lmax, solid ? 5 : 2, pc, NT);
    if (solid)
        k_prt3_fft<true><<<nelem * nchunk, NT, smem, s>>>(T, elems, nchunk, pc, Lmax, X, sls);
    else
        k_prt3_fft<false><<<nelem * nchunk, NT, smem, s>>>(T, elems, nchunk, pc, Lmax, X, sls);
}

namespace {

std::vector<int> prime_factors(int n) {
    std::vector<int> f;
    for (int p = 2; n > 1; p++)
        while (n % p == 0) {
            f.push_back(p);
            n /= p;
        }
    return f;
}

// DIF radix order: prime factors above 13 first (direct passes), then radix 4, one
// radix 2, and the odd radices in descending order.
std::vector<int> radices(int L) {
    std::vector<int> f = prime_factors(L), big, odd, out;
    int n2 = 0;
    for (int x : f) {
        if (x == 2)
            n2++;
        else if (x > 13)
            big.push_back(x);
        else
            odd.push_back(x);
    }
    std::sort(odd.rbegin(), odd.rend());
    out = big;
    for (int i = 0; i < n2 / 2; i++) out.push_back(4);
    if (n2 % 2) out.push_back(2);
    out.insert(out.end(), odd.begin(), odd.end());
    return out;
}

// modelled cost of one length-L transform of one sequence: issued instructions per point
// and pass (a radix-R butterfly in registers, or for a prime above 13 the direct pass's
// (R - 1) / 2 multiply-accumulate steps of about 3.3 instructions per point each)
double pass_cost(int L) {
    double c = 0;
    for (int r : radices(L)) c += (double)L * (r == 2 ? 12 : r == 4 ? 15 : r <= 13 ? r + 8 : 1.65 * r + 12);
    return c;
}
bool smooth13(int n) {
    for (int p : prime_factors(n))
        if (p > 13) return false;
    return true;
}

// position -> frequency index after the DIF passes
std::vector<int32_t> digit_reversal(const std::vector<int> &rad, int L) {
    std::vector<int32_t> pos2k(L);
    for (int k = 0; k < L; k++) {
        int pos = 0, rem = k, Ls = L;
        for (int r : rad) {
            const int d = rem % r;
            rem /= r;
            Ls /= r;
            pos += d * Ls;
        }
        pos2k[pos] = k;
    }
    return pos2k;
}

using cd = std::complex<double>;
// exact (FP64) DFT with e^{-2 pi i nk/L} by recursive mixed radix
void dft64(std::vector<cd> &x) {
    const int L = (int)x.size();
    if (L <= 1) return;
    int r = 2;
    while (L % r) r++;
    const int m = L / r;
    std::vector<std::vector<cd>> sub(r, std::vector<cd>(m));
    for (int j = 0; j < m; j++)
        for (int q = 0; q < r; q++) sub[q][j] = x[j * r + q];
    for (auto &s : sub) dft64(s);
    for (int k = 0; k < L; k++) {
        cd acc = 0;
        for (int q = 0; q < r; q++) acc += sub[q][k % m] * std::polar(1.0, -2.0 * M_PI * (double)(q * k % L) / L);
        x[k] = acc;
    }
}

}  // namespace

FftTables build_fft_tables(const std::vector<char> &used) {
    FftTables T;
    const int nmax = (int)used.size() - 1;
    T.plans.assign(std::max(nmax + 1, 1), FftPlan{});
    std::vector<int> tw_ofs;  // by length
    auto twiddles = [&](int L) -> int64_t {
        if ((int)tw_ofs.size() <= L) tw_ofs.resize(L + 1, -1);
        if (tw_ofs[L] >= 0) return tw_ofs[L];
        tw_ofs[L] = (int)T.f2.size();
        for (int m = 0; m < L; m++) {
            const double th = 2.0 * M_PI * (double)m / (double)L;
            T.f2.push_back(make_float2((float)std::cos(th), (float)std::sin(th)));
        }
        return tw_ofs[L];
    };
    // FP64 kernel spectrum of the cyclic sequence b (length M), / scale, digit-reversed
    auto kernel_spectrum = [&](std::vector<cd> b, const std::vector<int32_t> &rv, double scale) -> int64_t {
        dft64(b);
        const int64_t ofs = (int64_t)T.f2.size();
        for (size_t pos = 0; pos < b.size(); pos++) {
            const cd v = b[rv[pos]] / scale;
            T.f2.push_back(make_float2((float)v.real(), (float)v.imag()));
        }
        return ofs;
    };
    for (int nr = 1; nr <= nmax; nr++) {
        if (!used[nr]) continue;
        FftPlan pl{};
        const std::vector<int> fac = prime_factors(nr);
        const int bigp = fac.empty() ? 1 : fac.back();
        // candidates: mixed radix (direct passes for primes up to DIRECT_MAX), Bluestein
        // (the cheapest 13-smooth M in [2 nr - 1, 1.3 (2 nr - 1)]) and, for a prime nr,
        // Rader over the length nr - 1
        const double c_mixed = bigp <= DIRECT_MAX ? pass_cost(nr) : 1e300;
        int M = 0;
        double c_blue = 1e300;
        if (nr > 2 && !smooth13(nr)) {
            const int lo = 2 * nr - 1;
            for (int m = lo; m <= lo + lo * 3 / 10; m++) {
                if (!smooth13(m)) continue;
                const double c = 2.0 * pass_cost(m) + 16.0 * m;
                if (c < c_blue) {
                    c_blue = c;
                    M = m;
                }
            }
        }
        const bool prime = nr > 13 && fac.size() == 1;
        double c_rader = 1e300;
        if (prime) {
            int big1 = 1;
            for (int x : prime_factors(nr - 1)) big1 = std::max(big1, x);
            if (big1 <= DIRECT_MAX) c_rader = 2.0 * pass_cost(nr - 1) + 16.0 * nr;
        }
        pl.kind = c_rader < std::min(c_mixed, c_blue) ? 2 : c_blue < c_mixed ? 1 : 0;
        pl.L = pl.kind == 0 ? nr : pl.kind == 1 ? M : nr - 1;
        pl.Lbuf = pl.kind == 2 ? nr + 1 : pl.L;
        const std::vector<int> rad = radices(pl.L);
        if ((int)rad.size() > FFT_MAXRAD) throw std::runtime_error("ax3d_finalize || ring size has too many factors");
        pl.nrad = (int)rad.size();
        for (size_t i = 0; i < rad.size(); i++) pl.rad[i] = rad[i];
        pl.tw = twiddles(pl.L);
        const std::vector<int32_t> rv = digit_reversal(rad, pl.L);
        if (pl.kind == 0) {
            pl.rev = (int64_t)T.i32.size();
            T.i32.insert(T.i32.end(), rv.begin(), rv.end());
        } else if (pl.kind == 1) {
            // h_n = e^{i pi n^2 / nr}, n^2 reduced mod 2 nr exactly
            std::vector<cd> h(nr);
            for (int nn = 0; nn < nr; nn++) {
                const int64_t r2 = ((int64_t)nn * nn) % (2 * (int64_t)nr);
                h[nn] = std::polar(1.0, M_PI * (double)r2 / (double)nr);
            }
            pl.chirp = (int64_t)T.f2.size();
            for (auto &z : h) T.f2.push_back(make_float2((float)z.real(), (float)z.imag()));
            // C2R kernel conj(h_m), R2C kernel h_m (with 1/nr), |m| < nr, cyclic in M
            for (int which = 0; which < 2; which++) {
                std::vector<cd> b(M, 0.0);
                for (int m = 0; m < nr; m++) {
                    const cd v = which == 0 ? std::conj(h[m]) : h[m];
                    b[m] = v;
                    if (m > 0) b[M - m] = v;
                }
                (which == 0 ? pl.bc2r : pl.br2c) = kernel_spectrum(b, rv, which == 0 ? M : (double)M * nr);
            }
        } else {
            // Rader with the smallest primitive root g: order a = g^-m at position m, order 0
            // at position nr - 1; sample k = g^q at position q, sample 0 at position nr
            const int P = nr - 1;
            std::vector<int> pf1 = prime_factors(P);
            pf1.erase(std::unique(pf1.begin(), pf1.end()), pf1.end());
            int g = 2;
            for (;; g++) {
                bool ok = true;
                for (int q : pf1) {
                    int64_t r = 1, b = g, ex = P / q;
                    for (; ex; ex >>= 1, b = b * b % nr)
                        if (ex & 1) r = r * b % nr;
                    if (r == 1) ok = false;
                }
                if (ok) break;
            }
            std::vector<int32_t> gpow(P), ord(nr), samp(nr);
            for (int q = 0, x = 1; q < P; q++, x = (int)((int64_t)x * g % nr)) gpow[q] = x;
            ord[0] = nr - 1;
            for (int q = 0; q < P; q++) ord[gpow[q]] = (P - q) % P;
            for (int q = 0; q < P; q++) samp[q] = gpow[q];
            samp[P] = 0;
            pl.rev = (int64_t)T.i32.size();
            T.i32.insert(T.i32.end(), samp.begin(), samp.end());
            pl.ord = (int64_t)T.i32.size();
            T.i32.insert(T.i32.end(), ord.begin(), ord.end());
            // C2R kernel w^{g^j}, R2C kernel w^{-g^{-j}} (with 1/nr), w = e^{2 pi i / nr}
            std::vector<cd> bc(P), br(P);
            for (int j = 0; j < P; j++) {
                bc[j] = std::polar(1.0, 2.0 * M_PI * (double)gpow[j] / nr);
                br[j] = std::polar(1.0, -2.0 * M_PI * (double)gpow[(P - j) % P] / nr);
            }
            pl.bc2r = kernel_spectrum(bc, rv, (double)P);
            pl.br2c = kernel_spectrum(br, rv, (double)P * nr);
        }
        T.plans[nr] = pl;
    }
    if (T.f2.empty()) T.f2.push_back(make_float2(1.f, 0.f));
    if (T.i32.empty()) T.i32.push_back(0);
    return T;
}

// Points per CTA, cluster size, threads per CTA and shared memory of a bucket.
//   Policy 0: 256-thread CTAs; all 25 points in one CTA when two CTAs per SM fit, else the
//             smallest cluster whose CTAs fit (two per SM if possible).
//   Policy 1: 256-thread CTAs; the smallest cluster whose CTAs fit the whole shared memory
//             of an SM (one CTA per SM for rings up to ~360 samples, fewer clusters above).
//   Policy 2: as policy 0 while all points fit two CTAs per SM; larger rings take 512-thread
//             CTAs with the whole shared memory of an SM (16 warps per SM as two 256-thread
//             CTAs give), in the smallest cluster that fits: no cluster up to ~360 samples.
//   Policy 3: as policy 2, except that rings whose 25 points fit a quarter of an SM's shared
//             memory take 128-thread CTAs, four per SM (16 warps per SM over four elements
//             in flight instead of two: short rings spend most of their time in barriers).
//   Policy 4: as policy 3, except that rings whose 25 points fit an eighth of an SM's shared
//             memory (up to ~41 samples for a solid, ~60 for a fluid) take 64-thread CTAs,
//             eight per SM (the same 16 warps over eight elements in flight).
void size_phys_bucket(PhysBucket &b, bool solid, int policy) {
    const int nsq = solid ? 3 : 2;
    b.npts_chunk = 0;
    b.nt = NT;
    if (policy == 4) {
        const size_t sm = phys_smem_bytes(b.L_max, nsq, NPE, NT / 4);
        if (sm <= SMEM_EIGHT) {
            b.npts_chunk = NPE;
            b.csize = 1;
            b.smem = sm;
            b.nt = NT / 4;
            return;
        }
        policy = 3;
    }
    if (policy == 3) {
        const size_t sm = phys_smem_bytes(b.L_max, nsq, NPE, NT / 2);
        if (sm <= SMEM_FOUR) {
            b.npts_chunk = NPE;
            b.csize = 1;
            b.smem = sm;
            b.nt = NT / 2;
            return;
        }
        policy = 2;
    }
    if (policy == 2 && phys_smem_bytes(b.L_max, nsq, NPE, NT) > SMEM_TWO) {
        for (int pc = NPE; pc >= 1; pc--) {
            const size_t sm = phys_smem_bytes(b.L_max, nsq, pc, 2 * NT);
            const int C = (NPE + pc - 1) / pc;
            if (sm <= SMEM_CAP && C <= CLUSTER_MAX) {
                b.npts_chunk = pc;
                b.csize = C;
                b.smem = sm;
                b.nt = 2 * NT;
                return;
            }
        }
    }
    const std::vector<size_t> caps = policy == 1 ? std::vector<size_t>{SMEM_CAP} : std::vector<size_t>{SMEM_TWO, SMEM_CAP};
    for (size_t cap : caps) {
        for (int pc = NPE; pc >= 1; pc--) {
            const size_t sm = phys_smem_bytes(b.L_max, nsq, pc, NT);
            const int C = (NPE + pc - 1) / pc;
            if (sm <= cap && C <= CLUSTER_MAX) {
                b.npts_chunk = pc;
                b.csize = C;
                b.smem = sm;
                return;
            }
        }
    }
}

namespace {
cudaLaunchConfig_t phys_config(const PhysBucket &b, cudaLaunchAttribute *at, cudaStream_t s) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)std::max(b.grid, b.csize));
    cfg.blockDim = dim3((unsigned)b.nt);
    cfg.dynamicSmemBytes = b.smem;
    cfg.stream = s;
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = (unsigned)b.csize;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    return cfg;
}
// the instantiation of a bucket: solid or fluid, 64, 128, 256 or 512 threads
template <typename F>
void with_kernel(bool solid, int nt, F f) {
    if (solid)
        nt > NT        ? f(k_elem_phys<true, 2 * NT>)
        : nt == NT / 4 ? f(k_elem_phys<true, NT / 4>)
        : nt < NT      ? f(k_elem_phys<true, NT / 2>)
                       : f(k_elem_phys<true, NT>);
    else
        nt > NT        ? f(k_elem_phys<false, 2 * NT>)
        : nt == NT / 4 ? f(k_elem_phys<false, NT / 4>)
        : nt < NT      ? f(k_elem_phys<false, NT / 2>)
                       : f(k_elem_phys<false, NT>);
}
}  // namespace

int phys_grid(const PhysBucket &b, bool solid, int num_sms) {
    cudaLaunchAttribute at[1];
    int ncl = 0;
    cudaLaunchConfig_t cfg = phys_config(b, at, nullptr);
    with_kernel(solid, b.nt, [&](auto k) { cudaOccupancyMaxActiveClusters(&ncl, k, &cfg); });
    if (ncl <= 0) ncl = std::max(1, num_sms / b.csize);
    return b.csize * std::max(1, std::min(b.count, ncl));
}

void launch_elem_phys(bool solid, const ElemTable &T, const PointTable &P, const float2 *u, const PhysBucket &b,
                      const PhysTables &X, const SLS &sls, bool overwrite, cudaStream_t s) {
    if (b.count <= 0) return;
    cudaLaunchAttribute at[1];
    cudaLaunchConfig_t cfg = phys_config(b, at, s);
    with_kernel(solid, b.nt, [&](auto k) {
        cudaLaunchKernelEx(&cfg, k, T, P, u, (const int32_t *)b.elems, b.count, b.npts_chunk, b.L_max, X, sls,
                           (int)overwrite);
    });
}

}  // namespace ax3d
