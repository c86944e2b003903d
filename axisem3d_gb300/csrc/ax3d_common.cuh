// ax3d_common.cuh -- shared device-side definitions of the GB300 time-stepping path.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace ax3d {

constexpr int NP = 5;    // GLL points per edge (nPol = 4)
constexpr int NPE = 25;  // GLL points per element
// Fourier orders per work item of the Fourier-space element kernels: a warp keeps the
// element's operators, geometry and moduli in registers over FW_OB consecutive orders
// and loads the next order's displacement while it works on the current one
constexpr int FW_OB = 8;

// element flag bits
constexpr int EF_AXIAL = 1;
constexpr int EF_IN3D = 2;
constexpr int EF_FLUID = 4;
constexpr int EF_DIRECT = 1 << 12;  // owns all its points: assembles into their stiffness itself
constexpr int EF_SOURCE = 1 << 13;  // carries a source term (its points' stiffness is not zero before assembly)
__host__ __device__ inline int ef_mat(int f) { return (f >> 4) & 15; }
__host__ __device__ inline int ef_att(int f) { return (f >> 8) & 3; }

// Device view of the element table (structure of arrays).
struct ElemTable {
    const int32_t *pts;     // [E][25]
    const int32_t *flags;   // [E]
    const int32_t *nr;      // [E] nr_e = max nr of the element's points
    const float *geo;       // [E][5][25] dsdxii, dsdeta, dzdxii, dzdeta, inv_s
    const float *trig;      // [E][4][25] sin t, cos t, sin 2t, cos 2t
    const int64_t *mofs;    // [E] float offset into moduli
    const float *moduli;
    const int64_t *aofs;    // [E] float offset into att_moduli
    const float *attm;
    const int64_t *memofs;  // [E] float offset into mem (memory variables + stressR)
    float *mem;
    const int64_t *efofs;   // [E] complex offset into ef (element forces, [l][alpha][ncomp])
    float2 *ef;
    float2 *stiff;          // solid point stiffness, written directly by EF_DIRECT elements
    const int64_t *prtofs;  // [E] float offset into prtx (particle relabelling X, [4][len][25])
    const float *prtx;
    const int64_t *wofs;    // [E] complex offset into w (PRT_3D Fourier strain / stress, [alpha][nc][25])
    float2 *w;
};

// Device view of the point table.
struct PointTable {
    int32_t n;
    const int32_t *nr;
    const int8_t *kind;
    const uint8_t *axial;
    const uint8_t *fsurf;
    const int64_t *sofs;   // complex offset of the solid block ([alpha][3]), -1 if none
    const int64_t *fofs;   // complex offset of the fluid block ([alpha]), -1 if none
    const int32_t *mslen;  // solid inverse mass length (1 or nr), 0 if none
    const int64_t *msofs;
    const float *ms;
    const int32_t *mflen;
    const int64_t *mfofs;
    const float *mf;
    // ocean load on the solid part (MassOcean1D / MassOcean3D): oclen 0 none, 1 -> four
    // values (1/(m + m_ocean), 1/m, sin theta, cos theta), nr -> nr x (1/m, scaled normal s,
    // phi, z); replaces the solid mass
    const int32_t *oclen;
    const int64_t *ocofs;
    const float *oc;
    const int32_t *sflen;  // solid-fluid coupling length (1 or nr), 0 if none
    const int64_t *sfofs;  // row offset into sfn/sfni ([row][3])
    const float *sfn;
    const float *sfni;
    // gather lists (CSR, ascending element order): complex offsets of (element, local) blocks
    const int32_t *sg_ptr;
    const int64_t *sg_ref;
    const int32_t *fg_ptr;
    const int64_t *fg_ref;
    const uint8_t *gskip;   // nonzero: the point's only element assembles it directly (2: and,
                            // inside ax3d_step, overwrites its stiffness, so the Newmark update
                            // need not clear it)
    int32_t sgather;        // some solid point needs the gather
    // row -> point maps (a row = one Fourier order of one point)
    int64_t nsrows, nfrows;
    const int32_t *srow_pt;
    const int32_t *frow_pt;
};

struct Fields {
    float2 *su, *sv, *sa, *ss, *sku, *skv;  // solid [rows][3]
    float2 *fu, *fv, *fa, *fs, *fku, *fkv;  // fluid [rows]
};

struct SLS {
    int nsls;
    float a[8], b[8], g[8];
    int do_kappa;
};

__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ float2 cscale(float s, float2 a) { return make_float2(s * a.x, s * a.y); }
__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
    return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
// i * alpha * a
__device__ __forceinline__ float2 cimul(float alpha, float2 a) { return make_float2(-alpha * a.y, alpha * a.x); }

}  // namespace ax3d
