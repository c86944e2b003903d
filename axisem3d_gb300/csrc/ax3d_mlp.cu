// ax3d_mlp.cu -- the Nu network: inference and training kernels.
//
// A 16 -> 128 -> 128 -> 128 -> 1 perceptron with GELU, small enough that one CTA holds a
// 64-sample tile's whole forward and backward pass in shared memory: the activations
// (BF16), the pre-activations (FP32, for GELU'), one weight matrix at a time (BF16) and
// the back-propagated errors (BF16).  Products of two BF16 values are exact in FP32 and
// are accumulated in FP32.  Each tile writes its parameter gradient to its own slot; one
// pass then sums the slots in tile order and applies Adam, so results do not depend on
// scheduling.  The per-tile GEMMs -- the three forward layers (64 x 128 x K), the two
// hidden backward products (64 x 128 x 128) and the two hidden weight gradients
// (128 x 128 x 64) -- run on the tensor cores as warp-level BF16 mma.sync (m16n8k16, FP32
// accumulators), their operands read from shared memory with ldmatrix (transposed where
// the stored layout is k-major); the small first-layer weight gradient and the output
// layer stay on the CUDA cores.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <string>

#include "../../include/ax3d.h"
#include "ax3d_kernels.cuh"

namespace {

constexpr int NI = AX3D_MLP_NIN, NH = AX3D_MLP_NHID;
constexpr int TB = 64;       // samples per CTA
constexpr int NT = 256;      // threads per CTA
constexpr int HP = NH + 8;   // BF16 row pitch of activations and weights in shared memory

// FP32 master parameters
constexpr int OW1 = 0, OB1 = OW1 + NH * NI, OW2 = OB1 + NH, OB2 = OW2 + NH * NH, OW3 = OB2 + NH,
              OB3 = OW3 + NH * NH, OW4 = OB3 + NH, OB4 = OW4 + NH, NP = OB4 + 1;
static_assert(NP == AX3D_MLP_NPARAM, "parameter count");
constexpr int NPP = (NP + 3) & ~3;   // per-tile gradient slot stride (16-byte rows)

// BF16 weight copies: transposed [in][out] for the forward pass (T*), as stored
// [out][in] for the backward pass (N*)
constexpr int T1 = 0, T2 = T1 + NI * NH, T3 = T2 + NH * NH, N2 = T3 + NH * NH, N3 = N2 + NH * NH,
              N4 = N3 + NH * NH, NB = N4 + NH;

// shared memory (bytes)
constexpr int S_X = 0;                        // bf16 [TB][NI]        features
constexpr int S_H = S_X + TB * NI * 2;        // bf16 3 x [TB][HP]    h1, h2, h3
constexpr int S_Z = S_H + 3 * TB * HP * 2;    // f32  3 x [TB][NH]    z1, z2, z3
constexpr int S_W = S_Z + 3 * TB * NH * 4;    // bf16 [NH][HP]        one weight matrix
constexpr int S_D = S_W + NH * HP * 2;        // bf16 2 x [TB][HP]    dz (ping-pong)
constexpr int S_Y = S_D + 2 * TB * HP * 2;    // f32  [TB]            dy
constexpr int S_E = S_Y + TB * 4;             // f32  [TB]            squared errors
constexpr int S_V = S_E + TB * 4;             // f32  [NH]            w4
constexpr int SMEM = S_V + NH * 4;
static_assert(S_H % 16 == 0 && S_Z % 16 == 0 && S_W % 16 == 0 && S_D % 16 == 0, "alignment");
static_assert(SMEM <= 227 * 1024, "shared memory");

__device__ __forceinline__ float bf_lo(uint32_t v) { return __uint_as_float(v << 16); }
__device__ __forceinline__ float bf_hi(uint32_t v) { return __uint_as_float(v & 0xffff0000u); }
__device__ __forceinline__ uint16_t to_bf(float f) {
    return __bfloat16_as_ushort(__float2bfloat16_rn(f));
}
__device__ __forceinline__ void unpack8(const uint4 &u, float *f) {
    f[0] = bf_lo(u.x); f[1] = bf_hi(u.x); f[2] = bf_lo(u.y); f[3] = bf_hi(u.y);
    f[4] = bf_lo(u.z); f[5] = bf_hi(u.z); f[6] = bf_lo(u.w); f[7] = bf_hi(u.w);
}
__device__ __forceinline__ uint4 pack8(const float *f) {
    uint4 u;
    u.x = (uint32_t)to_bf(f[0]) | ((uint32_t)to_bf(f[1]) << 16);
    u.y = (uint32_t)to_bf(f[2]) | ((uint32_t)to_bf(f[3]) << 16);
    u.z = (uint32_t)to_bf(f[4]) | ((uint32_t)to_bf(f[5]) << 16);
    u.w = (uint32_t)to_bf(f[6]) | ((uint32_t)to_bf(f[7]) << 16);
    return u;
}
// gelu(z) = z Phi(z); gelu'(z) = Phi(z) + z phi(z)
__device__ __forceinline__ float gelu(float z) {
    return 0.5f * z * (1.f + erff(z * 0.70710678118654752f));
}
__device__ __forceinline__ float dgelu(float z) {
    return 0.5f * (1.f + erff(z * 0.70710678118654752f)) +
           z * 0.39894228040143268f * expf(-0.5f * z * z);
}

// rows x 128 BF16 from global (row-major, 256 B per row) into sW with pitch HP
__device__ __forceinline__ void load_w(uint16_t *sW, const uint16_t *g, int rows, int tid) {
    for (int i = tid; i < rows * (NH / 8); i += NT) {
        const int r = i >> 4, c = i & 15;
        *reinterpret_cast<uint4 *>(sW + r * HP + c * 8) =
            __ldg(reinterpret_cast<const uint4 *>(g + r * NH + c * 8));
    }
}

// ---- tensor-core tiles: mma.sync m16n8k16, BF16 inputs, FP32 accumulators ----
__device__ __forceinline__ uint32_t smem_addr(const void *p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}
// four 8x8 BF16 matrices; lane l gives the address of row l % 8 of matrix l / 8
__device__ __forceinline__ void ldsm4(uint32_t (&r)[4], const void *p) {
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
                 : "r"(smem_addr(p)));
}
__device__ __forceinline__ void ldsm4t(uint32_t (&r)[4], const void *p) {
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0,%1,%2,%3}, [%4];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
                 : "r"(smem_addr(p)));
}
// d += a (16x16, row) * b (16x8, col)
__device__ __forceinline__ void mma_bf16(float (&d)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// Warp w of 8 computes rows m0 = (w % 4) 16 .. +16 and columns n0 = (w / 4) 64 .. +64 of
// out[b][c] = sum_r in[b][r] sW[r][c] (in: [64][K] pitch IP; sW: [K][128] pitch HP).
// acc[nt][i]: column n0 + 8 nt + 2 (lane % 4) + (i & 1), row m0 + lane / 4 + 8 (i >> 1).
template <int K, int IP>
__device__ __forceinline__ void mma_rows(const uint16_t *in, const uint16_t *sW, float (&acc)[8][4]) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int m0 = (w & 3) * 16, n0 = (w >> 2) * 64;
    const int q = lane >> 3, i = lane & 7;
#pragma unroll
    for (int nt = 0; nt < 8; nt++)
#pragma unroll
        for (int c = 0; c < 4; c++) acc[nt][c] = 0.f;
#pragma unroll
    for (int k0 = 0; k0 < K; k0 += 16) {
        uint32_t a[4];
        // matrices: (rows 0-7, k 0-7), (rows 8-15, k 0-7), (rows 0-7, k 8-15), (rows 8-15, k 8-15)
        ldsm4(a, in + (m0 + i + 8 * (q & 1)) * IP + k0 + 8 * (q >> 1));
#pragma unroll
        for (int np = 0; np < 4; np++) {
            // B of two n-tiles from the k-major sW: (k 0-7, n), (k 8-15, n), (k 0-7, n+8), (k 8-15, n+8)
            uint32_t b[4];
            ldsm4t(b, sW + (k0 + i + 8 * (q & 1)) * HP + n0 + 16 * np + 8 * (q >> 1));
            mma_bf16(acc[2 * np], a, b[0], b[1]);
            mma_bf16(acc[2 * np + 1], a, b[2], b[3]);
        }
    }
}

// forward layer: z = W in + b, out = bf16(gelu(z)); z kept for the backward pass
template <int K, int IP, bool KEEPZ>
__device__ __forceinline__ void dense_fwd(const uint16_t *in, const uint16_t *sW, const float *bias,
                                          float *sZ, uint16_t *out, int tid) {
    float acc[8][4];
    mma_rows<K, IP>(in, sW, acc);
    const int lane = tid & 31, w = tid >> 5;
    const int r0 = (w & 3) * 16 + (lane >> 2), c0 = (w >> 2) * 64 + 2 * (lane & 3);
#pragma unroll
    for (int nt = 0; nt < 8; nt++) {
        const int c = c0 + 8 * nt;
        const float b0 = __ldg(bias + c), b1 = __ldg(bias + c + 1);
#pragma unroll
        for (int h = 0; h < 2; h++) {
            const int b = r0 + 8 * h;
            const float z0 = acc[nt][2 * h] + b0, z1 = acc[nt][2 * h + 1] + b1;
            if (KEEPZ) *reinterpret_cast<float2 *>(sZ + b * NH + c) = make_float2(z0, z1);
            *reinterpret_cast<uint32_t *>(out + b * HP + c) =
                (uint32_t)to_bf(gelu(z0)) | ((uint32_t)to_bf(gelu(z1)) << 16);
        }
    }
}

// backward through one hidden layer: dh = W^T dz (sW holds W as [out][in], which is the
// k-major [k][n] operand of dh[b][in] = sum_out dz[b][out] W[out][in]),
// dz_prev = bf16(dh * gelu'(z_prev))
__device__ __forceinline__ void dense_bwd(const uint16_t *dz, const uint16_t *sW, const float *zprev,
                                          uint16_t *dzprev, int tid) {
    float acc[8][4];
    mma_rows<NH, HP>(dz, sW, acc);
    const int lane = tid & 31, w = tid >> 5;
    const int r0 = (w & 3) * 16 + (lane >> 2), c0 = (w >> 2) * 64 + 2 * (lane & 3);
#pragma unroll
    for (int nt = 0; nt < 8; nt++) {
        const int c = c0 + 8 * nt;
#pragma unroll
        for (int h = 0; h < 2; h++) {
            const int b = r0 + 8 * h;
            const float2 z = *reinterpret_cast<const float2 *>(zprev + b * NH + c);
            *reinterpret_cast<uint32_t *>(dzprev + b * HP + c) =
                (uint32_t)to_bf(acc[nt][2 * h] * dgelu(z.x)) | ((uint32_t)to_bf(acc[nt][2 * h + 1] * dgelu(z.y)) << 16);
        }
    }
}

// weight gradient of a 128 x 128 layer over the tile: P[j][k] = sum_b dz[b][j] h[b][k];
// bias gradient P_b[j] = sum_b dz[b][j].  Warp w computes rows j0 = (w % 4) 32 .. +32 and
// columns k0 = (w / 4) 64 .. +64; both operands are stored [b][.], so A = dz^T comes in
// through transposed ldmatrix and B = h as in the forward layers.
__device__ __forceinline__ void wgrad(const uint16_t *dz, const uint16_t *h, float *P, float *Pb,
                                      int tid) {
    const int lane = tid & 31, w = tid >> 5;
    const int j0 = (w & 3) * 32, n0 = (w >> 2) * 64;
    const int q = lane >> 3, i = lane & 7;
    float acc[2][8][4];
#pragma unroll
    for (int mt = 0; mt < 2; mt++)
#pragma unroll
        for (int nt = 0; nt < 8; nt++)
#pragma unroll
            for (int c = 0; c < 4; c++) acc[mt][nt][c] = 0.f;
#pragma unroll
    for (int b0 = 0; b0 < TB; b0 += 16) {
        uint32_t a[2][4];
#pragma unroll
        for (int mt = 0; mt < 2; mt++)
            // (j 0-7, b 0-7), (j 8-15, b 0-7), (j 0-7, b 8-15), (j 8-15, b 8-15) of the [b][j] store
            ldsm4t(a[mt], dz + (b0 + i + 8 * (q >> 1)) * HP + j0 + 16 * mt + 8 * (q & 1));
#pragma unroll
        for (int np = 0; np < 4; np++) {
            uint32_t bb[4];
            ldsm4t(bb, h + (b0 + i + 8 * (q & 1)) * HP + n0 + 16 * np + 8 * (q >> 1));
#pragma unroll
            for (int mt = 0; mt < 2; mt++) {
                mma_bf16(acc[mt][2 * np], a[mt], bb[0], bb[1]);
                mma_bf16(acc[mt][2 * np + 1], a[mt], bb[2], bb[3]);
            }
        }
    }
#pragma unroll
    for (int mt = 0; mt < 2; mt++)
#pragma unroll
        for (int nt = 0; nt < 8; nt++)
#pragma unroll
            for (int hh = 0; hh < 2; hh++) {
                const int j = j0 + 16 * mt + (lane >> 2) + 8 * hh, k = n0 + 8 * nt + 2 * (lane & 3);
                *reinterpret_cast<float2 *>(P + j * NH + k) = make_float2(acc[mt][nt][2 * hh], acc[mt][nt][2 * hh + 1]);
            }
    if (tid < NH) {
        float s = 0.f;
        for (int b = 0; b < TB; b++) s += __uint_as_float((uint32_t)dz[b * HP + tid] << 16);
        Pb[tid] = s;
    }
}

// One 64-sample tile per CTA.  TRAIN: forward, loss, backward and the tile's gradient
// slot partial[tile]; else forward only, y to y_out.
template <bool TRAIN>
__global__ void __launch_bounds__(NT, 1)
k_mlp(const float *__restrict__ x, const float *__restrict__ tgt, int n,
      const float *__restrict__ master, const uint16_t *__restrict__ wb, float *__restrict__ y_out,
      float *__restrict__ partial, float *__restrict__ ploss) {
    extern __shared__ __align__(16) unsigned char smem[];
    uint16_t *sX = reinterpret_cast<uint16_t *>(smem + S_X);
    uint16_t *sH = reinterpret_cast<uint16_t *>(smem + S_H);
    float *sZ = reinterpret_cast<float *>(smem + S_Z);
    uint16_t *sW = reinterpret_cast<uint16_t *>(smem + S_W);
    uint16_t *sD = reinterpret_cast<uint16_t *>(smem + S_D);
    float *sY = reinterpret_cast<float *>(smem + S_Y);
    float *sE = reinterpret_cast<float *>(smem + S_E);
    float *sV = reinterpret_cast<float *>(smem + S_V);
    uint16_t *h1 = sH, *h2 = sH + TB * HP, *h3 = sH + 2 * TB * HP;
    float *z1 = sZ, *z2 = sZ + TB * NH, *z3 = sZ + 2 * TB * NH;
    uint16_t *d0 = sD, *d1 = sD + TB * HP;
    const int tid = threadIdx.x;
    const int64_t b0 = (int64_t)blockIdx.x * TB;
    const int nb = (int)((int64_t)n - b0 < TB ? (int64_t)n - b0 : TB);

    // features (rows past the batch are zero) and W1^T
    for (int i = tid; i < TB * NI; i += NT) {
        const int b = i / NI;
        sX[i] = to_bf(b < nb ? __ldg(x + b0 * NI + i) : 0.f);
    }
    if (tid < NH) sV[tid] = __uint_as_float((uint32_t)__ldg(wb + N4 + tid) << 16);
    load_w(sW, wb + T1, NI, tid);
    __syncthreads();
    dense_fwd<NI, NI, TRAIN>(sX, sW, master + OB1, z1, h1, tid);
    __syncthreads();
    load_w(sW, wb + T2, NH, tid);
    __syncthreads();
    dense_fwd<NH, HP, TRAIN>(h1, sW, master + OB2, z2, h2, tid);
    __syncthreads();
    load_w(sW, wb + T3, NH, tid);
    __syncthreads();
    dense_fwd<NH, HP, TRAIN>(h2, sW, master + OB3, z3, h3, tid);
    __syncthreads();

    // output: four threads per sample, fixed reduction order
    {
        const int b = tid >> 2, q = tid & 3;
        float s = 0.f;
#pragma unroll 8
        for (int k = q * 32; k < q * 32 + 32; k++)
            s = fmaf(__uint_as_float((uint32_t)h3[b * HP + k] << 16), sV[k], s);
        s += __shfl_xor_sync(0xffffffffu, s, 1);
        s += __shfl_xor_sync(0xffffffffu, s, 2);
        if (q == 0) {
            const float yv = s + __ldg(master + OB4);
            if (TRAIN) {
                const float e = b < nb ? yv - __ldg(tgt + b0 + b) : 0.f;
                sY[b] = 2.f * e / (float)n;
                sE[b] = e * e;
            } else if (b < nb) {
                y_out[b0 + b] = yv;
            }
        }
    }
    if (!TRAIN) return;
    __syncthreads();

    float *P = partial + (int64_t)blockIdx.x * NPP;
    if (tid == 0) {
        float s = 0.f;
        for (int b = 0; b < TB; b++) s += sE[b];
        ploss[blockIdx.x] = s;
    }
    // output layer: dz3 = bf16(w4 dy gelu'(z3)); dw4, db4
    {
        const int tc = tid & 15, tb = tid >> 4;
#pragma unroll
        for (int bb = 0; bb < 4; bb++) {
            const int b = tb * 4 + bb;
            float d[8];
#pragma unroll
            for (int c = 0; c < 8; c++)
                d[c] = sV[tc * 8 + c] * sY[b] * dgelu(z3[b * NH + tc * 8 + c]);
            *reinterpret_cast<uint4 *>(d0 + b * HP + tc * 8) = pack8(d);
        }
        if (tid < NH) {
            float s = 0.f;
            for (int b = 0; b < TB; b++)
                s = fmaf(sY[b], __uint_as_float((uint32_t)h3[b * HP + tid] << 16), s);
            P[OW4 + tid] = s;
        } else if (tid == NH) {
            float s = 0.f;
            for (int b = 0; b < TB; b++) s += sY[b];
            P[OB4] = s;
        }
    }
    load_w(sW, wb + N3, NH, tid);
    __syncthreads();
    dense_bwd(d0, sW, z2, d1, tid);       // dz2
    wgrad(d0, h2, P + OW3, P + OB3, tid); // dW3, db3
    __syncthreads();
    load_w(sW, wb + N2, NH, tid);
    __syncthreads();
    dense_bwd(d1, sW, z1, d0, tid);       // dz1
    wgrad(d1, h1, P + OW2, P + OB2, tid); // dW2, db2
    __syncthreads();
    // dW1 [128][16]: two threads per output row, 8 inputs each; db1
    {
        const int j = tid >> 1, k0 = (tid & 1) * 8;
        float acc[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
        for (int b = 0; b < TB; b++) {
            const float d = __uint_as_float((uint32_t)d0[b * HP + j] << 16);
            float xv[8];
            unpack8(*reinterpret_cast<const uint4 *>(sX + b * NI + k0), xv);
#pragma unroll
            for (int c = 0; c < 8; c++) acc[c] = fmaf(d, xv[c], acc[c]);
        }
        float4 *p = reinterpret_cast<float4 *>(P + OW1 + j * NI + k0);
        p[0] = make_float4(acc[0], acc[1], acc[2], acc[3]);
        p[1] = make_float4(acc[4], acc[5], acc[6], acc[7]);
        if (tid < NH) {
            float s = 0.f;
            for (int b = 0; b < TB; b++) s += __uint_as_float((uint32_t)d0[b * HP + tid] << 16);
            P[OB1 + tid] = s;
        }
    }
}

// BF16 copies of parameter p's value w
__device__ __forceinline__ void store_bf(uint16_t *wb, int p, float w) {
    const uint16_t v = to_bf(w);
    if (p < OB1) {
        wb[T1 + (p % NI) * NH + p / NI] = v;
    } else if (p >= OW2 && p < OB2) {
        const int q = p - OW2;
        wb[T2 + (q % NH) * NH + q / NH] = v;
        wb[N2 + q] = v;
    } else if (p >= OW3 && p < OB3) {
        const int q = p - OW3;
        wb[T3 + (q % NH) * NH + q / NH] = v;
        wb[N3 + q] = v;
    } else if (p >= OW4 && p < OB4) {
        wb[N4 + p - OW4] = v;
    }
}

__global__ void k_mlp_refresh(const float *__restrict__ master, uint16_t *__restrict__ wb) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p < NP) store_bf(wb, p, master[p]);
}

// gradient = sum of the tile slots in tile order; optional Adam step (step count on device)
__global__ void k_mlp_reduce(const float *__restrict__ partial, int ntiles, float *__restrict__ grad,
                             float *__restrict__ master, float *__restrict__ m1,
                             float *__restrict__ m2, uint16_t *__restrict__ wb,
                             const int *__restrict__ step, float lr, int update) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= NP) return;
    float g = 0.f;
    for (int t = 0; t < ntiles; t++) g += partial[(int64_t)t * NPP + p];
    if (grad) grad[p] = g;
    if (!update) return;
    const int t = *step + 1;
    const float a = 0.9f * m1[p] + 0.1f * g;
    const float b = 0.999f * m2[p] + 0.001f * g * g;
    m1[p] = a;
    m2[p] = b;
    const float c1 = 1.f - powf(0.9f, (float)t), c2 = 1.f - powf(0.999f, (float)t);
    const float w = master[p] - lr * (a / c1) / (sqrtf(b / c2) + 1e-8f);
    master[p] = w;
    store_bf(wb, p, w);
}

__global__ void k_mlp_finish(const float *__restrict__ ploss, int ntiles, int n,
                             float *__restrict__ loss, int *__restrict__ step, int update) {
    if (threadIdx.x != 0) return;
    float s = 0.f;
    for (int t = 0; t < ntiles; t++) s += ploss[t];
    if (loss) *loss = s / (float)n;
    if (update) *step += 1;
}

}  // namespace

struct ax3d_mlp {
    int device = 0;
    int max_tiles = 0;
    float *master = nullptr, *m1 = nullptr, *m2 = nullptr, *partial = nullptr, *ploss = nullptr;
    uint16_t *wb = nullptr;
    int *step = nullptr;
};

namespace {

int fail(int code, const std::string &msg) {
    ax3d::set_last_error(msg);
    return code;
}

int cuda_fail(cudaError_t e, const char *where) {
    return fail(AX3D_ERR_CUDA, std::string(where) + " || " + cudaGetErrorString(e));
}

#define MLP_CK(call, where)                                  \
    do {                                                     \
        cudaError_t e_ = (call);                             \
        if (e_ != cudaSuccess) return cuda_fail(e_, where);  \
    } while (0)

void release(ax3d_mlp *m) {
    cudaFree(m->master);
    cudaFree(m->m1);
    cudaFree(m->m2);
    cudaFree(m->partial);
    cudaFree(m->ploss);
    cudaFree(m->wb);
    cudaFree(m->step);
}

int launch_train(ax3d_mlp *m, const float *x, const float *t, int n, cudaStream_t s,
                 const char *where) {
    if (!m || !x || !t || n < 1 || (int64_t)n > (int64_t)m->max_tiles * TB)
        return fail(AX3D_ERR_ARG, std::string(where) + " || bad arguments or n above max_batch");
    MLP_CK(cudaSetDevice(m->device), where);
    const int ntiles = (n + TB - 1) / TB;
    k_mlp<true><<<ntiles, NT, SMEM, s>>>(x, t, n, m->master, m->wb, nullptr, m->partial, m->ploss);
    MLP_CK(cudaGetLastError(), where);
    return AX3D_OK;
}

}  // namespace

extern "C" {

int ax3d_mlp_create(int32_t max_batch, int32_t device, ax3d_mlp **out) {
    if (!out || max_batch < 1) return fail(AX3D_ERR_ARG, "ax3d_mlp_create || bad arguments");
    *out = nullptr;
    MLP_CK(cudaSetDevice(device), "ax3d_mlp_create");
    int optin = 0;
    MLP_CK(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, device),
           "ax3d_mlp_create");
    if (optin < SMEM)
        return fail(AX3D_ERR_UNSUPPORTED, "ax3d_mlp_create || device shared memory too small");
    MLP_CK(cudaFuncSetAttribute(k_mlp<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM),
           "ax3d_mlp_create");
    MLP_CK(cudaFuncSetAttribute(k_mlp<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM),
           "ax3d_mlp_create");
    auto *m = new ax3d_mlp();
    m->device = device;
    m->max_tiles = (int)(((int64_t)max_batch + TB - 1) / TB);
    cudaError_t e = cudaSuccess;
    auto alloc = [&](void **p, size_t bytes) {
        if (e == cudaSuccess) e = cudaMalloc(p, bytes);
        if (e == cudaSuccess) e = cudaMemset(*p, 0, bytes);
    };
    alloc((void **)&m->master, NP * sizeof(float));
    alloc((void **)&m->m1, NP * sizeof(float));
    alloc((void **)&m->m2, NP * sizeof(float));
    alloc((void **)&m->partial, (size_t)m->max_tiles * NPP * sizeof(float));
    alloc((void **)&m->ploss, (size_t)m->max_tiles * sizeof(float));
    alloc((void **)&m->wb, NB * sizeof(uint16_t));
    alloc((void **)&m->step, sizeof(int));
    if (e != cudaSuccess) {
        release(m);
        delete m;
        return e == cudaErrorMemoryAllocation ? fail(AX3D_ERR_NOMEM, "ax3d_mlp_create || out of memory")
                                              : cuda_fail(e, "ax3d_mlp_create");
    }
    *out = m;
    return AX3D_OK;
}

int ax3d_mlp_set_params(ax3d_mlp *m, const float *params, int64_t n) {
    if (!m || !params || n != NP) return fail(AX3D_ERR_ARG, "ax3d_mlp_set_params || bad arguments");
    MLP_CK(cudaSetDevice(m->device), "ax3d_mlp_set_params");
    MLP_CK(cudaMemcpy(m->master, params, NP * sizeof(float), cudaMemcpyHostToDevice),
           "ax3d_mlp_set_params");
    MLP_CK(cudaMemset(m->m1, 0, NP * sizeof(float)), "ax3d_mlp_set_params");
    MLP_CK(cudaMemset(m->m2, 0, NP * sizeof(float)), "ax3d_mlp_set_params");
    MLP_CK(cudaMemset(m->step, 0, sizeof(int)), "ax3d_mlp_set_params");
    k_mlp_refresh<<<(NP + 255) / 256, 256>>>(m->master, m->wb);
    MLP_CK(cudaGetLastError(), "ax3d_mlp_set_params");
    MLP_CK(cudaDeviceSynchronize(), "ax3d_mlp_set_params");
    return AX3D_OK;
}

int ax3d_mlp_get_params(ax3d_mlp *m, float *params, int64_t n) {
    if (!m || !params || n != NP) return fail(AX3D_ERR_ARG, "ax3d_mlp_get_params || bad arguments");
    MLP_CK(cudaSetDevice(m->device), "ax3d_mlp_get_params");
    MLP_CK(cudaDeviceSynchronize(), "ax3d_mlp_get_params");
    MLP_CK(cudaMemcpy(params, m->master, NP * sizeof(float), cudaMemcpyDeviceToHost),
           "ax3d_mlp_get_params");
    return AX3D_OK;
}

int ax3d_mlp_forward(ax3d_mlp *m, const float *d_x, int32_t n, float *d_y, void *stream) {
    if (!m || !d_x || !d_y || n < 0) return fail(AX3D_ERR_ARG, "ax3d_mlp_forward || bad arguments");
    if (n == 0) return AX3D_OK;
    MLP_CK(cudaSetDevice(m->device), "ax3d_mlp_forward");
    const int ntiles = (n + TB - 1) / TB;
    k_mlp<false><<<ntiles, NT, SMEM, (cudaStream_t)stream>>>(d_x, nullptr, n, m->master, m->wb, d_y,
                                                            nullptr, nullptr);
    MLP_CK(cudaGetLastError(), "ax3d_mlp_forward");
    return AX3D_OK;
}

int ax3d_mlp_gradient(ax3d_mlp *m, const float *d_x, const float *d_t, int32_t n, float *d_grad,
                      float *d_loss, void *stream) {
    if (!d_grad) return fail(AX3D_ERR_ARG, "ax3d_mlp_gradient || d_grad is NULL");
    cudaStream_t s = (cudaStream_t)stream;
    int rc = launch_train(m, d_x, d_t, n, s, "ax3d_mlp_gradient");
    if (rc != AX3D_OK) return rc;
    const int ntiles = (n + TB - 1) / TB;
    k_mlp_reduce<<<(NP + 255) / 256, 256, 0, s>>>(m->partial, ntiles, d_grad, m->master, m->m1, m->m2,
                                                   m->wb, m->step, 0.f, 0);
    k_mlp_finish<<<1, 32, 0, s>>>(m->ploss, ntiles, n, d_loss, m->step, 0);
    MLP_CK(cudaGetLastError(), "ax3d_mlp_gradient");
    return AX3D_OK;
}

int ax3d_mlp_train_step(ax3d_mlp *m, const float *d_x, const float *d_t, int32_t n, float lr,
                        float *d_loss, void *stream) {
    cudaStream_t s = (cudaStream_t)stream;
    int rc = launch_train(m, d_x, d_t, n, s, "ax3d_mlp_train_step");
    if (rc != AX3D_OK) return rc;
    const int ntiles = (n + TB - 1) / TB;
    k_mlp_reduce<<<(NP + 255) / 256, 256, 0, s>>>(m->partial, ntiles, nullptr, m->master, m->m1,
                                                   m->m2, m->wb, m->step, lr, 1);
    k_mlp_finish<<<1, 32, 0, s>>>(m->ploss, ntiles, n, d_loss, m->step, 1);
    MLP_CK(cudaGetLastError(), "ax3d_mlp_train_step");
    return AX3D_OK;
}

int ax3d_mlp_destroy(ax3d_mlp *m) {
    if (!m) return AX3D_OK;
    cudaSetDevice(m->device);
    cudaDeviceSynchronize();
    release(m);
    delete m;
    return AX3D_OK;
}

}  // extern "C"
