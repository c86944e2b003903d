// ax3d_noalloc.cu -- element stiffness + assembly that allocates no device memory.
//
// For callers that cannot call cudaMalloc themselves or let a library do so: for
// example a host code that runs inside a pre-sized memory pool or arena (every device
// byte handed out by its own allocator), or one that must not allocate between set-up
// and the end of a run.  They own and pass every input and output buffer; the element
// forces that sit between the element pass and the assembly pass -- scratch that
// ax3d_compute_stiff keeps in a buffer allocated by ax3d_finalize -- live here in one
// file-scope __device__ array of fixed size instead.
//
// Scope: Fourier-space isotropic solid elements (Isotropic1D, no attenuation) sharing GLL
// points, one Fourier order count Nu for all points (nr = 2 Nu + 1).  Arithmetic as
// SolidElement::displToStiff + gatherStiffFromElement (SolidElement.cpp:43-65, 404-443;
// SolidPoint.cpp:197-209), with the same per-point operators as the domain path.
#include <cstdint>
#include <cstring>
#include <mutex>
#include <string>

#include "../../include/ax3d.h"
#include "ax3d_elem_ops.cuh"
#include "ax3d_kernels.cuh"

namespace {

using namespace ax3d;

// The scratch: element forces [elem][25][Nu+1][3] complex.  Every device that loads the
// library holds it until the process exits.
constexpr size_t NOALLOC_SCRATCH_BYTES = (size_t)AX3D_NOALLOC_SCRATCH_MIB << 20;
static __device__ __align__(256) float2 g_noalloc_scratch[NOALLOC_SCRATCH_BYTES / sizeof(float2)];

// Per-device set-up, done once with that device current: the device address of
// g_noalloc_scratch (host code only holds a host-side stand-in for the symbol, which no
// kernel may be given), the SM count, and the two kernels loaded.  Guarded by a mutex, so
// two host threads making their first call on one device do not race on the slot.
constexpr int MAX_DEVICES = 64;
struct DevSetup {
    float2 *scratch = nullptr;
    int sms = 0;
};
DevSetup g_dev[MAX_DEVICES];
std::mutex g_dev_mu;

struct GMats {
    float g[2][25];  // [0] GLL, [1] GLJ(0,1); passed by value, so no copy to the device is needed
};

__global__ void __launch_bounds__(256)
    k_noalloc_elem(GMats G, int nelem, int nu, const int32_t *__restrict__ pts, const uint8_t *__restrict__ axial,
                   const float *__restrict__ geo, const float *__restrict__ lm, const float2 *__restrict__ u,
                   float2 *__restrict__ ef) {
    __shared__ float2 scr[8][14 * 25];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    float2 *q = scr[warp];
    const bool active = lane < NPE;
    const int p = active ? lane : 0;
    const int na = nu + 1;
    const int64_t nitems = (int64_t)nelem * na;
    for (int64_t it = (int64_t)blockIdx.x * 8 + warp; it < nitems; it += (int64_t)gridDim.x * 8) {
        const int e = (int)(it / na), a = (int)(it - (int64_t)e * na);
        const bool ax = axial[e] != 0;
        LaneOps L;
        L.init_from(p, G.g[ax ? 1 : 0], G.g[0]);
        Geo g;
        g.load(geo + (int64_t)e * 125, p);
        if (active) {
            const float2 *s = u + ((int64_t)pts[e * NPE + p] * na + a) * 3;
            q[p] = s[0];
            q[25 + p] = s[1];
            q[50 + p] = s[2];
        }
        __syncwarp();
        float2 eps[6], sig[6];
#pragma unroll
        for (int c = 0; c < 6; c++) eps[c] = make_float2(0.f, 0.f);
        if (active) grad6_lane(L, g, ax, a, q, eps);
        __syncwarp();
        if (active) {
            const float *m = lm + (int64_t)e * 50;
            elastic(0, eps, sig, [&](int k) { return m[k * NPE + p]; });
        }
        float2 f[3];
        quad6_lane(L, g, ax, a, sig, q, active, f);
        if (active) {
            float2 *o = ef + (((int64_t)e * NPE + p) * na + a) * 3;
            o[0] = f[0];
            o[1] = f[1];
            o[2] = f[2];
        }
    }
}

__global__ void k_noalloc_gather(int npoints, int nu, const int32_t *__restrict__ gptr,
                                 const int32_t *__restrict__ gref, const float2 *__restrict__ ef,
                                 float2 *__restrict__ stiff) {
    const int na = nu + 1;
    const int64_t rows = (int64_t)npoints * na;
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < rows; r += (int64_t)gridDim.x * blockDim.x) {
        const int pt = (int)(r / na), a = (int)(r - (int64_t)pt * na);
        float2 *s = stiff + r * 3;
        float2 s0 = s[0], s1 = s[1], s2 = s[2];
        for (int i = gptr[pt]; i < gptr[pt + 1]; i++) {
            const float2 *f = ef + ((int64_t)gref[i] * na + a) * 3;
            s0 = csub(s0, f[0]);
            s1 = csub(s1, f[1]);
            s2 = csub(s2, f[2]);
        }
        s[0] = s0;
        s[1] = s1;
        s[2] = s2;
    }
}

int fail(int code, const std::string &m) {
    ax3d::set_last_error(m);  // read back with ax3d_last_error
    return code;
}

// Resolves the scratch address and SM count of the current device and forces the module
// (the scratch array and both kernels) onto it, under lazy module loading too: after this
// the entry point touches no allocator of its own.
int device_setup(DevSetup &out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return fail(AX3D_ERR_CUDA, std::string("cudaGetDevice || ") + cudaGetErrorString(e));
    if (dev < 0 || dev >= MAX_DEVICES)
        return fail(AX3D_ERR_UNSUPPORTED, "ax3d_compute_stiff_iso1d_noalloc || device index");
    std::lock_guard<std::mutex> lk(g_dev_mu);
    DevSetup &d = g_dev[dev];
    if (!d.scratch) {
        cudaFuncAttributes fa;
        e = cudaFuncGetAttributes(&fa, k_noalloc_elem);
        if (e == cudaSuccess) e = cudaFuncGetAttributes(&fa, k_noalloc_gather);
        if (e != cudaSuccess)
            return fail(AX3D_ERR_CUDA, std::string("cudaFuncGetAttributes || ") + cudaGetErrorString(e));
        int sms = 0;
        e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (e != cudaSuccess)
            return fail(AX3D_ERR_CUDA, std::string("cudaDeviceGetAttribute || ") + cudaGetErrorString(e));
        void *ptr = nullptr;
        e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
        if (e != cudaSuccess)
            return fail(AX3D_ERR_CUDA, std::string("cudaGetSymbolAddress || ") + cudaGetErrorString(e));
        d.sms = sms > 0 ? sms : 1;
        d.scratch = static_cast<float2 *>(ptr);
    }
    out = d;
    return AX3D_OK;
}

}  // namespace

extern "C" {

int ax3d_compute_stiff_iso1d_noalloc(int32_t nelem, int32_t nu, const int32_t *d_points,
                                     const uint8_t *d_axial, const float *d_geometry,
                                     const float *d_lambda_mu, int32_t npoints,
                                     const int32_t *d_gather_ptr, const int32_t *d_gather_ref,
                                     const float *d_displ, float *d_stiff, const double *g_gll,
                                     const double *g_glj, void *stream) {
    if (nelem < 0 || nu < 0 || npoints < 0)
        return fail(AX3D_ERR_ARG, "ax3d_compute_stiff_iso1d_noalloc || negative size");
    // set-up first, so that a call with nelem = 0 at start-up loads everything
    DevSetup d;
    int rc = device_setup(d);
    if (rc != AX3D_OK) return rc;
    if (nelem == 0 || npoints == 0) return AX3D_OK;
    if (!d_points || !d_axial || !d_geometry || !d_lambda_mu || !d_gather_ptr || !d_gather_ref || !d_displ ||
        !d_stiff || !g_gll || !g_glj)
        return fail(AX3D_ERR_ARG, "ax3d_compute_stiff_iso1d_noalloc || null argument");
    if (((uintptr_t)d_displ | (uintptr_t)d_stiff) & 7)
        return fail(AX3D_ERR_ARG, "ax3d_compute_stiff_iso1d_noalloc || d_displ and d_stiff must be 8-byte aligned "
                                  "(complex float pairs)");
    const size_t need = (size_t)nelem * NPE * ((size_t)nu + 1) * 3 * sizeof(float2);
    if (need > NOALLOC_SCRATCH_BYTES)
        return fail(AX3D_ERR_ARG, "ax3d_compute_stiff_iso1d_noalloc || element forces need " + std::to_string(need) +
                                      " bytes, more than the " + std::to_string(NOALLOC_SCRATCH_BYTES) +
                                      "-byte static scratch (nelem * 25 * (nu + 1) * 24 bytes)");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    GMats G;
    for (int i = 0; i < 25; i++) {
        G.g[0][i] = (float)g_gll[i];
        G.g[1][i] = (float)g_glj[i];
    }
    const int64_t items = (int64_t)nelem * (nu + 1);
    int blocks = (int)std::min<int64_t>((items + 7) / 8, (int64_t)d.sms * 16);
    k_noalloc_elem<<<blocks, 256, 0, s>>>(G, nelem, nu, d_points, d_axial, d_geometry, d_lambda_mu,
                                           reinterpret_cast<const float2 *>(d_displ), d.scratch);
    const int64_t rows = (int64_t)npoints * (nu + 1);
    blocks = (int)std::min<int64_t>((rows + 255) / 256, (int64_t)d.sms * 32);
    k_noalloc_gather<<<blocks, 256, 0, s>>>(npoints, nu, d_gather_ptr, d_gather_ref, d.scratch,
                                             reinterpret_cast<float2 *>(d_stiff));
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail(AX3D_ERR_CUDA, std::string("launch || ") + cudaGetErrorString(e));
    return AX3D_OK;
}

}  // extern "C"
