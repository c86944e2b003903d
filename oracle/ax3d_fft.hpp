// ax3d_fft.hpp -- O(n log n) FP32 transforms for the timed CPU baseline (TEST
// INFRASTRUCTURE ONLY: the CPU port that bench.py times beside the GPU path; the checker
// keeps the exact double DFT of ax3d_oracle.hpp).
//
// The reference transforms with FFTW 3.3 plans (SolverFFTW_N6.cpp:15-53, FieldFFT.cpp:19-57:
// fftwf_plan_many_dft_c2r / _r2c over the 150 strain / stress columns of an element,
// unnormalised C2R that reads only Re of order 0, R2C followed by x 1/nr).  FFTW is not on
// this image, so the same transforms are written here from published methods:
//  * complex transforms of length n by the Stockham autosort formulation of the mixed-radix
//    Cooley-Tukey algorithm (natural order in and out, one pass per radix; as given by
//    Govindaraju et al., "High performance discrete Fourier transforms on graphics
//    processors", SC 2008), radix 4, 2, 3, 5 butterflies written out and any other prime
//    radix up to 31 as a direct DFT of its length;
//  * lengths with a prime factor above 31 by Bluestein's chirp-z algorithm (Bluestein 1970)
//    over the cheapest 7-smooth length M >= 2 n - 1;
//  * two real sequences per complex transform (z = a + i b; A_k = (Z_k + conj Z_{n-k}) / 2,
//    B_k = (Z_k - conj Z_{n-k}) / 2i), the usual substitute for a dedicated real FFT.
// Twiddles, chirps and kernel spectra are computed in double once per length and rounded to
// float.  Plans are cached per thread.
#pragma once

#include <cmath>
#include <complex>
#include <map>
#include <memory>
#include <vector>

namespace axfft {

using cf = std::complex<float>;

struct Plan {
    int n = 0;
    bool blue = false;
    // Stockham stages: radix and the offset of its twiddles in tw (per stage Ns x R values)
    std::vector<int> rad, twofs;
    std::vector<cf> tw;                    // e^{+2 pi i (j mod Ns) r / (Ns R)}
    std::vector<std::vector<float>> dftc;  // generic radix: cos(2 pi q / R) per stage
    std::vector<std::vector<float>> dfts;
    // Bluestein
    int M = 0;
    const Plan *sub = nullptr;
    std::vector<cf> chirp;           // h_j = e^{+i pi j^2 / n}
    std::vector<cf> kern_p, kern_m;  // FFT_M of the kernel conj(h) (sign +) / h (sign -), / M
};

inline std::vector<int> factors(int n) {
    std::vector<int> f;
    for (int p = 2; n > 1; p++)
        while (n % p == 0) {
            f.push_back(p);
            n /= p;
        }
    return f;
}

inline bool smooth(int n, int lim) {
    for (int p : factors(n))
        if (p > lim) return false;
    return true;
}

// radices of a smooth length: 4s first, then a 2, then the odd primes
inline std::vector<int> radices(int n) {
    std::vector<int> f = factors(n), out;
    int n2 = 0;
    std::vector<int> odd;
    for (int x : f) (x == 2 ? n2++ : (odd.push_back(x), 0));
    for (int i = 0; i < n2 / 2; i++) out.push_back(4);
    if (n2 % 2) out.push_back(2);
    out.insert(out.end(), odd.begin(), odd.end());
    return out;
}

const Plan &plan(int n);

inline void build_stockham(Plan &P, int n) {
    P.rad = radices(n);
    int Ns = 1;
    for (int R : P.rad) {
        P.twofs.push_back((int)P.tw.size());
        for (int j = 0; j < Ns; j++)
            for (int r = 0; r < R; r++) {
                const double th = 2.0 * M_PI * (double)(j * r) / (double)(Ns * R);
                P.tw.push_back(cf((float)std::cos(th), (float)std::sin(th)));
            }
        std::vector<float> c(R), s(R);
        for (int q = 0; q < R; q++) {
            c[q] = (float)std::cos(2.0 * M_PI * q / R);
            s[q] = (float)std::sin(2.0 * M_PI * q / R);
        }
        P.dftc.push_back(c);
        P.dfts.push_back(s);
        Ns *= R;
    }
}

// v <- DFT_R(v) with e^{sg 2 pi i q k / R}
template <int R>
inline void bfly(cf *v, float sg) {
    if constexpr (R == 2) {
        const cf a = v[0], b = v[1];
        v[0] = a + b;
        v[1] = a - b;
    } else if constexpr (R == 3) {
        const float c1 = -0.5f, s1 = sg * 0.86602540378443864676f;
        const cf t = v[1] + v[2], d = v[1] - v[2];
        const cf a = v[0] + c1 * t, b(-s1 * d.imag(), s1 * d.real());
        v[0] = v[0] + t;
        v[1] = a + b;
        v[2] = a - b;
    } else if constexpr (R == 4) {
        const cf t0 = v[0] + v[2], t1 = v[0] - v[2], t2 = v[1] + v[3], d = v[1] - v[3];
        const cf t3 = sg > 0 ? cf(-d.imag(), d.real()) : cf(d.imag(), -d.real());
        v[0] = t0 + t2;
        v[2] = t0 - t2;
        v[1] = t1 + t3;
        v[3] = t1 - t3;
    } else if constexpr (R == 5) {
        const float c1 = 0.30901699437494742410f, c2 = -0.80901699437494742410f;
        const float s1 = sg * 0.95105651629515357212f, s2 = sg * 0.58778525229247312917f;
        const cf a1 = v[1] + v[4], b1 = v[1] - v[4], a2 = v[2] + v[3], b2 = v[2] - v[3];
        const cf r1 = v[0] + c1 * a1 + c2 * a2, r2 = v[0] + c2 * a1 + c1 * a2;
        const cf i1 = s1 * b1 + s2 * b2, i2 = s2 * b1 - s1 * b2;
        v[0] = v[0] + a1 + a2;
        v[1] = r1 + cf(-i1.imag(), i1.real());
        v[4] = r1 - cf(-i1.imag(), i1.real());
        v[2] = r2 + cf(-i2.imag(), i2.real());
        v[3] = r2 - cf(-i2.imag(), i2.real());
    }
}

// generic odd prime radix: symmetric direct DFT
inline void bfly_generic(cf *v, int R, const float *c, const float *s, float sg) {
    cf o[32];
    const int H = (R - 1) / 2;
    cf sp[16], sm[16];
    cf out0 = v[0];
    for (int r = 1; r <= H; r++) {
        sp[r] = v[r] + v[R - r];
        sm[r] = v[r] - v[R - r];
        out0 += sp[r];
    }
    o[0] = out0;
    for (int k = 1; k <= H; k++) {
        cf a = v[0], b = 0.f;
        for (int r = 1; r <= H; r++) {
            const int q = (r * k) % R;
            a += c[q] * sp[r];
            b += s[q] * sm[r];
        }
        const cf ib = sg > 0 ? cf(-b.imag(), b.real()) : cf(b.imag(), -b.real());
        o[k] = a + ib;
        o[R - k] = a - ib;
    }
    for (int k = 0; k < R; k++) v[k] = o[k];
}

// one Stockham stage: x (length n) -> y
template <int R>
inline void stage(const cf *__restrict x, cf *__restrict y, int n, int Ns, const cf *tw, float sg) {
    const int nb = n / R;
    for (int j = 0; j < nb; j++) {
        const int jm = j % Ns;
        cf v[R];
        for (int r = 0; r < R; r++) {
            const cf w = tw[jm * R + r];
            v[r] = x[j + r * nb] * (sg > 0 ? w : std::conj(w));
        }
        bfly<R>(v, sg);
        const int o = (j - jm) * R + jm;
        for (int r = 0; r < R; r++) y[o + r * Ns] = v[r];
    }
}

inline void stage_generic(const cf *__restrict x, cf *__restrict y, int n, int Ns, int R, const cf *tw,
                          const float *c, const float *s, float sg) {
    const int nb = n / R;
    cf v[32];
    for (int j = 0; j < nb; j++) {
        const int jm = j % Ns;
        for (int r = 0; r < R; r++) {
            const cf w = tw[jm * R + r];
            v[r] = x[j + r * nb] * (sg > 0 ? w : std::conj(w));
        }
        bfly_generic(v, R, c, s, sg);
        const int o = (j - jm) * R + jm;
        for (int r = 0; r < R; r++) y[o + r * Ns] = v[r];
    }
}

// In-place complex transform of length P.n with e^{sg 2 pi i jk / n}, unnormalised; `work`
// holds at least 2 max(n, M) values.
inline void fft(const Plan &P, cf *x, cf *work, int sg) {
    const float s = sg > 0 ? 1.f : -1.f;
    if (P.blue) {
        const int n = P.n, M = P.M;
        cf *a = work, *w2 = work + M;
        for (int j = 0; j < n; j++) a[j] = x[j] * (sg > 0 ? P.chirp[j] : std::conj(P.chirp[j]));
        for (int j = n; j < M; j++) a[j] = 0.f;
        fft(*P.sub, a, w2, -1);
        const std::vector<cf> &K = sg > 0 ? P.kern_p : P.kern_m;
        for (int j = 0; j < M; j++) a[j] *= K[j];
        fft(*P.sub, a, w2, +1);
        for (int k = 0; k < n; k++) x[k] = a[k] * (sg > 0 ? P.chirp[k] : std::conj(P.chirp[k]));
        return;
    }
    cf *src = x, *dst = work;
    int Ns = 1;
    for (size_t i = 0; i < P.rad.size(); i++) {
        const int R = P.rad[i];
        const cf *tw = P.tw.data() + P.twofs[i];
        switch (R) {
            case 2: stage<2>(src, dst, P.n, Ns, tw, s); break;
            case 3: stage<3>(src, dst, P.n, Ns, tw, s); break;
            case 4: stage<4>(src, dst, P.n, Ns, tw, s); break;
            case 5: stage<5>(src, dst, P.n, Ns, tw, s); break;
            default: stage_generic(src, dst, P.n, Ns, R, tw, P.dftc[i].data(), P.dfts[i].data(), s);
        }
        std::swap(src, dst);
        Ns *= R;
    }
    if (src != x)
        for (int k = 0; k < P.n; k++) x[k] = src[k];
}

inline const Plan &plan(int n) {
    thread_local std::map<int, std::unique_ptr<Plan>> cache;
    auto it = cache.find(n);
    if (it != cache.end()) return *it->second;
    auto P = std::make_unique<Plan>();
    P->n = n;
    if (n <= 1 || smooth(n, 31)) {
        build_stockham(*P, n);
    } else {
        P->blue = true;
        int M = 2 * n - 1;
        while (!smooth(M, 7)) M++;
        P->M = M;
        P->sub = &plan(M);
        P->chirp.resize(n);
        for (int j = 0; j < n; j++) {
            const long long r2 = (long long)j * j % (2LL * n);
            const double th = M_PI * (double)r2 / (double)n;
            P->chirp[j] = cf((float)std::cos(th), (float)std::sin(th));
        }
        // kernel b_m = e^{-sg i pi m^2 / n}, |m| < n, cyclic in M; its spectrum (sign -1) / M
        for (int which = 0; which < 2; which++) {
            std::vector<std::complex<double>> b(M, 0.0);
            const double sgn = which == 0 ? -1.0 : 1.0;  // kern_p: sg = +1 -> e^{-i..}
            for (int m = 0; m < n; m++) {
                const long long r2 = (long long)m * m % (2LL * n);
                const std::complex<double> v = std::polar(1.0, sgn * M_PI * (double)r2 / (double)n);
                b[m] = v;
                if (m > 0) b[M - m] = v;
            }
            // exact DFT of b in double (once per length), angles from a table of e^{-2 pi i q / M}
            std::vector<std::complex<double>> e(M);
            for (int q = 0; q < M; q++) e[q] = std::polar(1.0, -2.0 * M_PI * (double)q / (double)M);
            std::vector<cf> &K = which == 0 ? P->kern_p : P->kern_m;
            K.resize(M);
            for (int k = 0; k < M; k++) {
                std::complex<double> acc = 0.0;
                for (int j = 0, q = 0; j < M; j++, q = (q + k) % M) acc += b[j] * e[q];
                acc /= (double)M;
                K[k] = cf((float)acc.real(), (float)acc.imag());
            }
        }
    }
    const Plan &ref = *P;
    cache.emplace(n, std::move(P));
    return ref;
}

inline std::vector<cf> &scratch(size_t n) {
    thread_local std::vector<cf> w;
    if (w.size() < n) w.resize(n);
    return w;
}

// C2R of two Hermitian columns (orders 0..nr/2 at stride `st`), FFTW's conventions:
// unnormalised, only Re of order 0 (and of the Nyquist order of an even nr) enters.
inline void c2r_pair(const cf *X1, const cf *X2, int st, int nr, float *x1, float *x2) {
    const Plan &P = plan(nr);
    std::vector<cf> &w = scratch(3 * (size_t)std::max(nr, P.M) + 4);
    cf *z = w.data(), *work = z + std::max(nr, P.M);
    const int nu = nr / 2;
    z[0] = cf(X1[0].real(), X2[0].real());
    for (int a = 1; a <= nu; a++) {
        const cf A = X1[(size_t)a * st], B = X2[(size_t)a * st];
        if (2 * a == nr) {
            z[a] = cf(A.real(), B.real());
        } else {
            z[a] = cf(A.real() - B.imag(), A.imag() + B.real());            // A + i B
            z[nr - a] = cf(A.real() + B.imag(), B.real() - A.imag());       // conj(A) + i conj(B)
        }
    }
    fft(P, z, work, +1);
    for (int k = 0; k < nr; k++) {
        x1[k] = z[k].real();
        x2[k] = z[k].imag();
    }
}

// R2C of two real columns scaled by 1/nr: orders 0..nr/2 at stride `st`.
inline void r2c_pair(const float *x1, const float *x2, int nr, cf *X1, cf *X2, int st) {
    const Plan &P = plan(nr);
    std::vector<cf> &w = scratch(3 * (size_t)std::max(nr, P.M) + 4);
    cf *z = w.data(), *work = z + std::max(nr, P.M);
    for (int k = 0; k < nr; k++) z[k] = cf(x1[k], x2[k]);
    fft(P, z, work, -1);
    const float h = 0.5f / (float)nr;
    for (int a = 0; a <= nr / 2; a++) {
        const cf p = z[a], q = std::conj(z[a == 0 ? 0 : nr - a]);
        const cf s = p + q, d = p - q;
        X1[(size_t)a * st] = cf(s.real() * h, s.imag() * h);
        X2[(size_t)a * st] = cf(d.imag() * h, -d.real() * h);  // (p - q) / 2i
    }
}

}  // namespace axfft
