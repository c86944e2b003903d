// ax3d_kernels.cuh -- launch interface of the GB300 kernels (host side).
#pragma once

#include <string>

#include "ax3d_common.cuh"

namespace ax3d {

struct PhysBucket {
    int32_t *elems = nullptr;  // device list of element indices
    int count = 0;
    int nr_max = 0;
    int npts_chunk = 25;       // GLL points per pass (shared-memory budget)
    size_t smem = 0;
};

// Sets the text ax3d_last_error returns on this thread.
void set_last_error(const std::string &msg);

void set_g_matrices(const float *g_gll, const float *g_glj, cudaStream_t s);

size_t phys_smem_bytes(int nr, int ncomp, int npts_chunk);
int phys_points_per_chunk(int nr, int ncomp);
void init_kernel_attributes();

void launch_elem_fourier_solid(const ElemTable &T, const PointTable &P, const float2 *su,
                               const int2 *items, int nitems, const SLS &sls, cudaStream_t s);
void launch_elem_fourier_fluid(const ElemTable &T, const PointTable &P, const float2 *fu,
                               const int2 *items, int nitems, cudaStream_t s);
void launch_elem_phys_solid(const ElemTable &T, const PointTable &P, const float2 *su,
                            const PhysBucket &b, const SLS &sls, cudaStream_t s);
void launch_elem_phys_fluid(const ElemTable &T, const PointTable &P, const float2 *fu,
                            const PhysBucket &b, cudaStream_t s);

void launch_gather(const PointTable &P, const ElemTable &T, const Fields &F, cudaStream_t s);
void launch_newmark(const PointTable &P, const Fields &F, float dt, float half_dt,
                    float half_dt_dt, int kahan, const int32_t *pts3d, int n3d, cudaStream_t s);
void launch_couple(const PointTable &P, const Fields &F, const int32_t *sf3d, int n3d,
                   cudaStream_t s);
void launch_source(const PointTable &P, const ElemTable &T, const Fields &F,
                   const int32_t *src_elem, const int32_t *src_nord, const int64_t *src_ofs,
                   const float2 *src_force, int nsrc, const float *stf, int nstf,
                   const int32_t *tptr, int tofs, cudaStream_t s);
void launch_record(const PointTable &P, const ElemTable &T, const float2 *su,
                   const int32_t *rec_elem, const float *rec_phi, const float *rec_w, int nrec,
                   float *out_base, int cap, const int32_t *tptr, int tofs, cudaStream_t s);
void launch_stability(const float2 *su, int64_t ns, const float2 *fu, int64_t nf,
                      int32_t *flag, const int32_t *tptr, int interval, cudaStream_t s);
void launch_advance(int32_t *tptr, cudaStream_t s);
// tptr == nullptr: learn now; otherwise only when (*tptr - 1) % interval == 0
void launch_learn_wisdom(const PointTable &P, const Fields &F, float *maxh, int32_t *nuw, float cutoff,
                         const int32_t *tptr, int interval, cudaStream_t s);

}  // namespace ax3d
