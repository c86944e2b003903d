// ax3d_kernels.cuh -- launch interface of the GB300 kernels (host side).
#pragma once

#include <string>
#include <vector>

#include "ax3d_common.cuh"

namespace ax3d {

// Transform plan of one ring size nr (device table indexed by nr).
//   kind 0: in-place mixed radix of length L = nr;
//   kind 1: Bluestein chirp convolution of smooth length L >= 2 nr - 1;
//   kind 2: Rader (prime nr): cyclic convolution of length L = nr - 1 over the
//           generator-ordered spectrum, plus two slots for the zero-frequency terms.
constexpr int FFT_MAXRAD = 12;
struct FftPlan {
    int32_t kind = 0, L = 1, nrad = 0, Lbuf = 1;  // Lbuf: buffer positions per sequence
    int32_t rad[FFT_MAXRAD] = {};  // radices of L in decimation-in-frequency order
    int64_t tw = 0;                // L twiddles (cos, sin)(2 pi m / L) in the float2 table
    int64_t rev = 0;               // kinds 0, 2: position -> sample map (nr int32)
    int64_t ord = 0;               // kind 2: order -> position map (nr int32)
    int64_t chirp = 0;             // kind 1: h_n = e^{i pi n^2 / nr}, n < nr
    int64_t bc2r = 0, br2c = 0;    // kinds 1, 2: kernel spectra (L float2, digit-reversed)
};
struct FftTables {
    std::vector<FftPlan> plans;
    std::vector<float2> f2;
    std::vector<int32_t> i32;
};
// Device view of the transform tables.
struct PhysTables {
    const FftPlan *plans = nullptr;
    const float2 *f2 = nullptr;
    const int32_t *i32 = nullptr;
};

struct PhysBucket {
    int32_t *elems = nullptr;  // device list of element indices
    int count = 0;
    int L_max = 0;             // longest transform in the bucket
    int n_max = 0;             // most Fourier orders in the bucket
    int npts_chunk = 25;       // GLL points per CTA (shared-memory budget)
    int csize = 1;             // CTAs per cluster sharing one element
    int nt = 256;              // threads per CTA (256, or 512 with a whole SM's shared memory)
    size_t smem = 0;
    int grid = 0;              // persistent CTAs (a multiple of csize)
};

// Sets the text ax3d_last_error returns on this thread.
void set_last_error(const std::string &msg);

void set_g_matrices(const float *g_gll, const float *g_glj, cudaStream_t s);

void init_kernel_attributes();
void init_phys_attributes();
void set_g_matrices_phys(const float *g_gll, const float *g_glj, cudaStream_t s);
// FP64 plans, twiddles, chirps and kernel spectra for every used ring size (used[nr] != 0)
FftTables build_fft_tables(const std::vector<char> &used);
size_t phys_smem_bytes(int Lmax, int nsq, int npts_chunk, int nthreads = 256);
void size_phys_bucket(PhysBucket &b, bool solid, int policy = 0);
int phys_grid(const PhysBucket &b, bool solid, int num_sms);

void launch_elem_fourier_solid(const ElemTable &T, const PointTable &P, const float2 *su,
                               const int2 *items, int nitems, const SLS &sls, cudaStream_t s);
void launch_elem_fourier_fluid(const ElemTable &T, const PointTable &P, const float2 *fu,
                               const int2 *items, int nitems, cudaStream_t s);
// overwrite: the point stiffness of direct-assembly elements without a source term is known
// to be zero (the Newmark update just cleared it), so they store -force instead of
// subtracting
void launch_elem_phys(bool solid, const ElemTable &T, const PointTable &P, const float2 *u, const PhysBucket &b,
                      const PhysTables &X, const SLS &sls, bool overwrite, cudaStream_t s);

void launch_gather(const PointTable &P, const ElemTable &T, const Fields &F, cudaStream_t s);
// in_step: stiffness rows that direct elements overwrite later in the step are not cleared
void launch_newmark(const PointTable &P, const Fields &F, float dt, float half_dt, float half_dt_dt, int kahan,
                    const int32_t *pts3d, int n3d, int in_step, cudaStream_t s);
// n1d: solid-fluid points with a 1-D coupling (none: the row kernel is not launched)
void launch_couple(const PointTable &P, const Fields &F, const int32_t *sf3d, int n3d, int n1d, cudaStream_t s);
void launch_source(const PointTable &P, const ElemTable &T, const Fields &F,
                   const int32_t *src_elem, const int32_t *src_nord, const int64_t *src_ofs,
                   const float2 *src_force, int nsrc, const float *stf, int nstf,
                   const int32_t *tptr, int tofs, cudaStream_t s);
// particle relabelling: PRT_1D elements in Fourier space, PRT_3D elements through the
// Fourier scratch T.w (lbuf_max = longest transform buffer among them, sizing k_prt3_fft's
// shared memory)
void launch_elem_prt1(bool solid, const ElemTable &T, const PointTable &P, const float2 *u, const int2 *items,
                      int nitems, const SLS &sls, cudaStream_t s);
void launch_elem_prt3(bool solid, const ElemTable &T, const PointTable &P, const float2 *u, const int2 *items,
                      int nitems, const int32_t *elems, int nelem, int lbuf_max, const PhysTables &X, const SLS &sls,
                      cudaStream_t s);
// PRT_3D transform pass (k_prt3_fft) and the points per CTA it takes for sequences of Lmax
// buffer positions (0: not even one fits in shared memory)
void launch_prt3_fft(bool solid, const ElemTable &T, const int32_t *elems, int nelem, int Lmax, const PhysTables &X,
                     const SLS &sls, cudaStream_t s);
int prt3_points_per_cta(bool solid, int Lmax);
void launch_record_strain_curl(const PointTable &P, const ElemTable &T, const float2 *su, const int32_t *rec_elem,
                               const float *rec_phi, const float *rec_w, const int32_t *list, int n,
                               float *strain_out, int nst, float *curl_out, int ncu, int cap, const int32_t *tptr,
                               int tofs, cudaStream_t s);
void launch_record(const PointTable &P, const ElemTable &T, const float2 *su,
                   const int32_t *rec_elem, const float *rec_phi, const float *rec_w, int nrec,
                   float *out_base, int cap, const int32_t *tptr, int tofs, cudaStream_t s);
void launch_record_surface(const PointTable &P, const ElemTable &T, const float2 *su, const int32_t *elem,
                           const int32_t *side, const int64_t *rofs, int nedge, float2 *out_base, int64_t rowlen,
                           int cap, const int32_t *tptr, int tofs, int interval, cudaStream_t s);
void launch_stability(const float2 *su, int64_t ns, const float2 *fu, int64_t nf,
                      int32_t *flag, const int32_t *tptr, int interval, cudaStream_t s);
void launch_advance(int32_t *tptr, cudaStream_t s);
// tptr == nullptr: learn now; otherwise only when (*tptr - 1) % interval == 0
void launch_learn_wisdom(const PointTable &P, const Fields &F, float *maxh, int32_t *nuw, float cutoff,
                         const int32_t *tptr, int interval, cudaStream_t s);

}  // namespace ax3d
