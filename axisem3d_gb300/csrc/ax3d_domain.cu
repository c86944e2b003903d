// ax3d_domain.cu -- host runtime behind include/ax3d.h: the GB300 Domain.
//
// Mirrors the reference's Domain (SOLVER/src/core/domain/Domain.h:20-125): it owns the
// points, elements, source terms, source-time function and receivers, and runs the
// Newmark::solve loop body (SOLVER/src/core/newmark/Newmark.cpp:47-93) on one CUDA
// stream.  Set-up data arrive as structure-of-arrays host buffers, are validated and
// packed once in ax3d_finalize (the counterpart of Mesh::release), and stay resident in
// HBM for the whole run.  There is no CPU fallback: a failed CUDA call is an error.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <deque>
#include <map>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/ax3d.h"
#include "ax3d_kernels.cuh"

namespace {

thread_local std::string g_err;

struct Error : std::runtime_error {
    int code;
    Error(int c, const std::string &m) : std::runtime_error(m), code(c) {}
};

#define CK(call)                                                                                 \
    do {                                                                                         \
        cudaError_t e_ = (call);                                                                 \
        if (e_ != cudaSuccess)                                                                   \
            throw Error(AX3D_ERR_CUDA, std::string(#call) + " || " + cudaGetErrorString(e_)); \
    } while (0)

template <typename T>
struct DevBuf {
    T *p = nullptr;
    size_t n = 0;
    void alloc(size_t count) {
        free();
        n = count;
        if (count) CK(cudaMalloc(&p, count * sizeof(T)));
    }
    void upload(const std::vector<T> &v, cudaStream_t s) {
        alloc(v.size());
        if (n) CK(cudaMemcpyAsync(p, v.data(), n * sizeof(T), cudaMemcpyHostToDevice, s));
    }
    void zero(cudaStream_t s) {
        if (n) CK(cudaMemsetAsync(p, 0, n * sizeof(T), s));
    }
    void free() {
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
    }
    ~DevBuf() { free(); }
};

int n_moduli(int mat) {
    switch (mat) {
        case AX3D_MAT_ISO: return 2;
        case AX3D_MAT_TISO: return 5;
        case AX3D_MAT_ANISO: return 21;
        case AX3D_MAT_ACOUSTIC: return 1;
    }
    throw Error(AX3D_ERR_ARG, "ax3d_add_elements || unknown material");
}

}  // namespace

struct ax3d_domain {
    // ---------------- configuration ----------------
    int device = 0;
    double dt = 0.;
    float g_gll[25], g_glj[25];
    ax3d::SLS sls{};
    int kahan = 0;
    int stab_interval = 0;
    cudaStream_t stream = nullptr;
    // side streams for the physical-space buckets, forked from / joined into `stream`
    static constexpr int NSIDE = 3;
    cudaStream_t side[NSIDE] = {};
    cudaEvent_t ev_fork = nullptr, ev_join[NSIDE] = {};
    bool finalized = false;
    int tstep = 1;

    // ---------------- host staging ----------------
    std::vector<int32_t> p_nr;
    std::vector<int8_t> p_kind;
    std::vector<uint8_t> p_axial, p_fsurf;
    std::vector<int32_t> p_mslen, p_mflen, p_sflen;
    std::vector<int64_t> p_msofs, p_mfofs, p_sfofs;
    std::vector<float> p_ms, p_mf, p_sfn, p_sfni;
    std::vector<int32_t> oc_pt, oc_len;  // ocean load rows as added
    std::vector<float> oc_vals;

    std::vector<int32_t> e_pts, e_flags, e_nr;
    std::vector<float> e_geo, e_trig;
    std::vector<uint8_t> e_hastrig;
    std::vector<int32_t> e_prtlen;  // particle relabelling: 0 none, 1 PRT_1D, nr PRT_3D
    std::vector<int64_t> e_prtofs;
    std::vector<float> e_prtx;
    std::vector<int64_t> e_mofs, e_aofs;
    std::vector<float> e_mod, e_attm;

    std::vector<int32_t> s_elem, s_nord;
    std::vector<int64_t> s_ofs;
    std::vector<float> s_force;  // complex interleaved
    std::vector<float> stf;

    std::vector<int32_t> r_elem;
    std::vector<float> r_phi, r_w;

    // ---------------- device ----------------
    DevBuf<int32_t> d_pnr, d_mslen, d_mflen, d_sflen, d_sg_ptr, d_fg_ptr, d_srow, d_frow;
    DevBuf<int8_t> d_pkind;
    DevBuf<uint8_t> d_paxial, d_pfsurf, d_gskip;
    DevBuf<int64_t> d_sofs, d_fofs, d_msofs, d_mfofs, d_sfofs, d_sg_ref, d_fg_ref;
    DevBuf<float> d_ms, d_mf, d_sfn, d_sfni, d_oc;
    DevBuf<int32_t> d_oclen;
    DevBuf<int64_t> d_ocofs;
    DevBuf<int32_t> d_epts, d_eflags, d_enr;
    DevBuf<float> d_geo, d_trig, d_mod, d_attm, d_mem;
    DevBuf<int64_t> d_mofs, d_aofs, d_memofs, d_efofs;
    DevBuf<float2> d_ef, d_f2;
    DevBuf<int32_t> d_i32;
    DevBuf<ax3d::FftPlan> d_plans;
    ax3d::PhysTables X{};
    DevBuf<float2> d_su, d_sv, d_sa, d_ss, d_sku, d_skv, d_fu, d_fv, d_fa, d_fs, d_fku, d_fkv;
    DevBuf<int2> d_items_s, d_items_f, d_items_p1s, d_items_p1f, d_items_p3s, d_items_p3f;
    DevBuf<int32_t> d_p3s, d_p3f;
    DevBuf<int64_t> d_prtofs, d_wofs;
    DevBuf<float> d_prtx;
    DevBuf<float2> d_w;
    int nitems_p1s = 0, nitems_p1f = 0, nitems_p3s = 0, nitems_p3f = 0, n_p3s = 0, n_p3f = 0;
    int lbuf_p3s = 1, lbuf_p3f = 1;  // longest transform buffer of the PRT_3D elements
    std::vector<ax3d::PhysBucket> buckets_s, buckets_f;
    std::vector<DevBuf<int32_t>> bucket_lists;
    // the bucket schedule: geometric step of the transform length between buckets, shared
    // memory policy (0: two CTAs per SM where they fit; 1: one CTA per SM, fewer clusters)
    // and side streams used; set at ax3d_finalize, changed by ax3d_autotune
    // the bucket schedule without ax3d_autotune / ax3d_set_schedule: policy 3 with merged
    // launches.  Policy 4 (64-thread CTAs for the shortest rings) gains on learned-Nu
    // domains with three side streams but loses on others there (concurrent persistent
    // launches of different CTA sizes contend for the SMs: element pass of 100,000 elements
    // at Nu 4-40 11.9 ms against 9.6 ms for this default), so it is left to the autotuner
    struct Schedule {
        double ratio = 1.12;
        int policy = 3, nside = NSIDE, merge = 1;
    } sched;
    std::vector<int32_t> phys3_s_list, phys3_f_list;  // physical-space elements
    std::vector<int32_t> lbuf_of_nr;                   // buffer length of each ring size's plan
    int num_sms = 0;
    DevBuf<int32_t> d_pts3d, d_sf3d;
    int n_pts3d = 0, n_sf3d = 0, n_sf1d = 0;
    DevBuf<int32_t> d_selem, d_snord;
    DevBuf<int64_t> d_sofs_src;
    DevBuf<float2> d_sforce;
    DevBuf<float> d_stf;
    DevBuf<int32_t> d_relem;
    DevBuf<float> d_rphi, d_rw, d_seis;
    int seis_cap = 0;
    // dump_strain / dump_curl receivers: list of (receiver, strain slot, curl slot)
    std::vector<int32_t> r_dump;
    int n_strain = 0, n_curl = 0, n_sclist = 0;
    DevBuf<int32_t> d_sclist;
    DevBuf<float> d_strain, d_curl;
    // whole-surface recorder: edges (element, side), record every sf_interval steps
    std::vector<int32_t> sf_elem, sf_side;
    int sf_interval = 1;
    int64_t sf_row = 0;  // complex values per record
    int sf_cap = 0;      // records the buffer holds
    DevBuf<int32_t> d_sfe, d_sfs;
    DevBuf<int64_t> d_sfrofs;
    DevBuf<float2> d_surf;
    DevBuf<int32_t> d_flag;
    DevBuf<int32_t> d_tstep, d_targ;  // step counter (1-based) and explicit step index
    DevBuf<float> d_wis_max;          // [P][4] largest Hilbert norm per component (s, phi, z, fluid)
    DevBuf<int32_t> d_wis_nu;         // [P][4] Nu wisdom per component
    int wis_interval = 0;
    float wis_cutoff = 0.f;
    int32_t h_targ = 0;
    bool use_graphs = true;
    cudaGraphExec_t graph_execs[2] = {};  // one per displacement buffer

    ax3d::ElemTable T{};
    ax3d::PointTable P{};
    ax3d::Fields F{};
    int64_t nsolid = 0, nfluid = 0;  // complex sizes
    int nitems_s = 0, nitems_f = 0;

    // ---------------- phase timers ----------------
    bool timers = false;
    double t_ms[AX3D_NTIMERS] = {};
    int64_t t_launch[AX3D_NTIMERS] = {};
    struct Mark {
        int phase;
        cudaEvent_t a, b;
    };
    std::vector<Mark> marks;
    std::vector<cudaEvent_t> pool;
    int open_phase = -1;
    cudaEvent_t open_ev = nullptr;

    cudaEvent_t get_event() {
        if (!pool.empty()) {
            cudaEvent_t e = pool.back();
            pool.pop_back();
            return e;
        }
        cudaEvent_t e;
        CK(cudaEventCreate(&e));
        return e;
    }
    void tbegin(int ph) {
        if (!timers) return;
        open_phase = ph;
        open_ev = get_event();
        CK(cudaEventRecord(open_ev, stream));
    }
    void tend(int nlaunch) {
        if (open_phase < 0) return;
        cudaEvent_t b = get_event();
        CK(cudaEventRecord(b, stream));
        marks.push_back({open_phase, open_ev, b});
        t_launch[open_phase] += nlaunch;
        open_phase = -1;
    }
    void collect_timers() {  // stream already synchronised
        for (auto &m : marks) {
            float ms = 0.f;
            CK(cudaEventElapsedTime(&ms, m.a, m.b));
            t_ms[m.phase] += ms;
            pool.push_back(m.a);
            pool.push_back(m.b);
        }
        marks.clear();
    }

    // ---- asynchronous field transfers: two input staging slots, one output ----
    // The solid displacement is double-buffered instead (buffer su_cur is the field): a queued
    // displacement is copied straight into the other buffer and step() switches to it, and
    // reads come straight from the live buffer; one captured graph per buffer.
    struct Queued {
        int which, phase, slot;  // slot < 0: displacement buffer -1 - slot
    };
    cudaStream_t cp_in = nullptr, cp_out = nullptr;
    DevBuf<float2> stage_in[2], stage_out, d_su_alt;
    cudaEvent_t ev_in_ready[2] = {}, ev_in_free[2] = {}, ev_out_ready = nullptr, ev_out_free = nullptr;
    cudaEvent_t ev_su_ready[2] = {}, ev_su_read[2] = {}, ev_main = nullptr;
    std::deque<Queued> queued;
    int next_slot = 0, su_cur = 0;
    float2 *su_buf(int k) { return k ? d_su_alt.p : d_su.p; }
    bool su_async(int which, int phase) const { return which == AX3D_FIELD_DISPL && phase == AX3D_PHASE_SOLID; }
    // main-stream work that writes the live displacement waits for reads of it in flight
    void guard_su() {
        if (cp_in) CK(cudaStreamWaitEvent(stream, ev_su_read[su_cur], 0));
    }

    void init_async() {
        if (cp_in) return;
        CK(cudaStreamCreateWithFlags(&cp_in, cudaStreamNonBlocking));
        CK(cudaStreamCreateWithFlags(&cp_out, cudaStreamNonBlocking));
        for (int k = 0; k < 2; k++) {
            CK(cudaEventCreateWithFlags(&ev_in_ready[k], cudaEventDisableTiming));
            CK(cudaEventCreateWithFlags(&ev_in_free[k], cudaEventDisableTiming));
            CK(cudaEventRecord(ev_in_free[k], stream));
        }
        CK(cudaEventCreateWithFlags(&ev_out_ready, cudaEventDisableTiming));
        CK(cudaEventCreateWithFlags(&ev_out_free, cudaEventDisableTiming));
        CK(cudaEventRecord(ev_out_free, stream));
        d_su_alt.alloc(std::max<int64_t>(nsolid, 1));
        CK(cudaEventCreateWithFlags(&ev_main, cudaEventDisableTiming));
        for (int k = 0; k < 2; k++) {
            CK(cudaEventCreateWithFlags(&ev_su_ready[k], cudaEventDisableTiming));
            CK(cudaEventCreateWithFlags(&ev_su_read[k], cudaEventDisableTiming));
            CK(cudaEventRecord(ev_su_read[k], stream));
        }
    }
    // staging for fields other than the solid displacement, allocated on first use
    void init_staging() {
        if (stage_out.p) return;
        const int64_t n = std::max<int64_t>(std::max(nsolid, nfluid), 1);
        stage_in[0].alloc(n);
        stage_in[1].alloc(n);
        stage_out.alloc(n);
    }
    // host -> staging slot on the input copy stream; consumed by the next step()
    void set_field_async(int which, int phase, const float *in) {
        need_final();
        field(which, phase);  // validates
        init_async();
        if (queued.size() >= 2) throw Error(AX3D_ERR_STATE, "ax3d_set_field_async || two inputs already queued");
        if (su_async(which, phase)) {
            // the buffer after every queued displacement, flipped
            int planned = su_cur;
            for (const Queued &q : queued)
                if (q.slot < 0) planned = -1 - q.slot;
            const int target = 1 - planned;
            CK(cudaStreamWaitEvent(cp_in, ev_su_read[target], 0));
            CK(cudaMemcpyAsync(su_buf(target), in, nsolid * sizeof(float2), cudaMemcpyHostToDevice, cp_in));
            CK(cudaEventRecord(ev_su_ready[target], cp_in));
            queued.push_back({which, phase, -1 - target});
            return;
        }
        init_staging();
        const int slot = next_slot;
        next_slot ^= 1;
        CK(cudaStreamWaitEvent(cp_in, ev_in_free[slot], 0));
        CK(cudaMemcpyAsync(stage_in[slot].p, in, fsize(phase) * sizeof(float2), cudaMemcpyHostToDevice, cp_in));
        CK(cudaEventRecord(ev_in_ready[slot], cp_in));
        queued.push_back({which, phase, slot});
    }
    // the oldest queued input replaces its field, ordered on the main stream
    void apply_queued_input() {
        if (queued.empty()) {
            guard_su();
            return;
        }
        const Queued q = queued.front();
        queued.pop_front();
        if (q.slot < 0) {
            su_cur = -1 - q.slot;
            F.su = su_buf(su_cur);
            CK(cudaStreamWaitEvent(stream, ev_su_ready[su_cur], 0));
            guard_su();
            return;
        }
        guard_su();
        CK(cudaStreamWaitEvent(stream, ev_in_ready[q.slot], 0));
        CK(cudaMemcpyAsync(field(q.which, q.phase), stage_in[q.slot].p, fsize(q.phase) * sizeof(float2),
                           cudaMemcpyDeviceToDevice, stream));
        CK(cudaEventRecord(ev_in_free[q.slot], stream));
    }
    // field -> staging (main stream, so it sees every step enqueued before), then staging ->
    // host on the output copy stream while later steps run
    void get_field_async(int which, int phase, float *out) {
        need_final();
        float2 *src = field(which, phase);
        init_async();
        if (su_async(which, phase)) {
            CK(cudaEventRecord(ev_main, stream));
            CK(cudaStreamWaitEvent(cp_out, ev_main, 0));
            CK(cudaMemcpyAsync(out, src, nsolid * sizeof(float2), cudaMemcpyDeviceToHost, cp_out));
            CK(cudaEventRecord(ev_su_read[su_cur], cp_out));
            return;
        }
        init_staging();
        CK(cudaStreamWaitEvent(stream, ev_out_free, 0));
        CK(cudaMemcpyAsync(stage_out.p, src, fsize(phase) * sizeof(float2), cudaMemcpyDeviceToDevice, stream));
        CK(cudaEventRecord(ev_out_ready, stream));
        CK(cudaStreamWaitEvent(cp_out, ev_out_ready, 0));
        CK(cudaMemcpyAsync(out, stage_out.p, fsize(phase) * sizeof(float2), cudaMemcpyDeviceToHost, cp_out));
        CK(cudaEventRecord(ev_out_free, cp_out));
    }
    void sync_fields() {
        if (!cp_in) return;
        CK(cudaStreamSynchronize(cp_in));
        CK(cudaStreamSynchronize(cp_out));
        CK(cudaStreamSynchronize(stream));
    }

    ~ax3d_domain() {
        if (cp_in) {
            cudaStreamSynchronize(cp_in);
            cudaStreamSynchronize(cp_out);
            for (int k = 0; k < 2; k++) {
                cudaEventDestroy(ev_in_ready[k]);
                cudaEventDestroy(ev_in_free[k]);
            }
            cudaEventDestroy(ev_out_ready);
            cudaEventDestroy(ev_out_free);
            cudaEventDestroy(ev_main);
            for (int k = 0; k < 2; k++) {
                cudaEventDestroy(ev_su_ready[k]);
                cudaEventDestroy(ev_su_read[k]);
            }
            cudaStreamDestroy(cp_in);
            cudaStreamDestroy(cp_out);
        }
        for (auto &m : marks) {
            cudaEventDestroy(m.a);
            cudaEventDestroy(m.b);
        }
        for (auto e : pool) cudaEventDestroy(e);
        drop_graph();
        for (int k = 0; k < NSIDE; k++) {
            if (ev_join[k]) cudaEventDestroy(ev_join[k]);
            if (side[k]) cudaStreamDestroy(side[k]);
        }
        if (ev_fork) cudaEventDestroy(ev_fork);
        if (stream) cudaStreamDestroy(stream);
    }

    // ================================================================
    void add_points(int n, const int32_t *nr, const int8_t *kind, const uint8_t *axial,
                    const uint8_t *fsurf, const int32_t *msl, const float *ms, const int32_t *mfl,
                    const float *mf, const int32_t *sfl, const float *sfn, const float *sfni) {
        if (finalized) throw Error(AX3D_ERR_STATE, "ax3d_add_points || domain already finalized");
        if (n < 0 || !nr || !kind || !axial || !msl || !mfl)
            throw Error(AX3D_ERR_ARG, "ax3d_add_points || null argument");
        int64_t om = 0, of = 0, osf = 0;
        for (int i = 0; i < n; i++) {
            const int r = nr[i], k = kind[i];
            if (r < 1) throw Error(AX3D_ERR_ARG, "ax3d_add_points || nr must be >= 1");
            if (k < 0 || k > 2) throw Error(AX3D_ERR_ARG, "ax3d_add_points || bad point kind");
            const bool hasS = k != AX3D_POINT_FLUID, hasF = k != AX3D_POINT_SOLID;
            const int ls = msl[i], lf = mfl[i], lsf = sfl ? sfl[i] : 0;
            if (hasS ? !(ls == 1 || ls == r) : ls != 0)
                throw Error(AX3D_ERR_ARG, "ax3d_add_points || solid mass length must be 1 or nr");
            if (hasF ? !(lf == 1 || lf == r) : lf != 0)
                throw Error(AX3D_ERR_ARG, "ax3d_add_points || fluid mass length must be 1 or nr");
            if (k == AX3D_POINT_SOLID_FLUID ? !(lsf == 1 || lsf == r) : lsf != 0)
                throw Error(AX3D_ERR_ARG, "ax3d_add_points || coupling length must be 1 or nr");
            p_nr.push_back(r);
            p_kind.push_back((int8_t)k);
            p_axial.push_back(axial[i] ? 1 : 0);
            p_fsurf.push_back(fsurf && fsurf[i] ? 1 : 0);
            p_mslen.push_back(ls);
            p_msofs.push_back((int64_t)p_ms.size());
            if (ls) p_ms.insert(p_ms.end(), ms + om, ms + om + ls);
            om += ls;
            p_mflen.push_back(lf);
            p_mfofs.push_back((int64_t)p_mf.size());
            if (lf) p_mf.insert(p_mf.end(), mf + of, mf + of + lf);
            of += lf;
            p_sflen.push_back(lsf);
            p_sfofs.push_back((int64_t)p_sfn.size() / 3);
            if (lsf) {
                p_sfn.insert(p_sfn.end(), sfn + osf * 3, sfn + (osf + lsf) * 3);
                p_sfni.insert(p_sfni.end(), sfni + osf * 3, sfni + (osf + lsf) * 3);
            }
            osf += lsf;
        }
    }

    void add_elements(int n, const int32_t *pts, const int8_t *mat, const uint8_t *axial,
                      const uint8_t *in3d, const float *geo, const float *trig, const int64_t *mofs,
                      const float *mod, const int8_t *att, const int64_t *aofs, const float *attm) {
        if (finalized) throw Error(AX3D_ERR_STATE, "ax3d_add_elements || domain already finalized");
        if (n < 0 || !pts || !mat || !axial || !in3d || !geo || !mofs || !mod)
            throw Error(AX3D_ERR_ARG, "ax3d_add_elements || null argument");
        const int npts = (int)p_nr.size();
        for (int e = 0; e < n; e++) {
            int nr = -1;
            bool any_solid = false, any_fluid = false;
            for (int l = 0; l < 25; l++) {
                const int p = pts[(int64_t)e * 25 + l];
                if (p < 0 || p >= npts) throw Error(AX3D_ERR_ARG, "ax3d_add_elements || point index out of range");
                nr = std::max(nr, p_nr[p]);  // Element.cpp:13-18
                any_solid |= p_kind[p] != AX3D_POINT_FLUID;
                any_fluid |= p_kind[p] != AX3D_POINT_SOLID;
                e_pts.push_back(p);
            }
            const int m = mat[e];
            const int km = n_moduli(m);
            const bool fluid = m == AX3D_MAT_ACOUSTIC;
            for (int l = 0; l < 25; l++) {
                const int p = pts[(int64_t)e * 25 + l];
                if (fluid && p_kind[p] == AX3D_POINT_SOLID)
                    throw Error(AX3D_ERR_ARG, "ax3d_add_elements || fluid element on a solid-only point");
                if (!fluid && p_kind[p] == AX3D_POINT_FLUID)
                    throw Error(AX3D_ERR_ARG, "ax3d_add_elements || solid element on a fluid-only point");
            }
            const int a = (fluid || !att) ? 0 : att[e];
            if (a < 0 || a > 2) throw Error(AX3D_ERR_ARG, "ax3d_add_elements || bad attenuation kind");
            if (a && sls.nsls <= 0) throw Error(AX3D_ERR_ARG, "ax3d_add_elements || attenuation without SLS");
            if ((m == AX3D_MAT_TISO || m == AX3D_MAT_ANISO) && !trig)
                throw Error(AX3D_ERR_ARG, "ax3d_add_elements || TISO/ANISO need theta tables");
            const bool e3d = in3d[e] != 0;
            int flags = (axial[e] ? ax3d::EF_AXIAL : 0) | (e3d ? ax3d::EF_IN3D : 0) |
                        (fluid ? ax3d::EF_FLUID : 0) | (m << 4) | (a << 8);
            e_flags.push_back(flags);
            e_nr.push_back(nr);
            e_geo.insert(e_geo.end(), geo + (int64_t)e * 125, geo + (int64_t)e * 125 + 125);
            if (trig)
                e_trig.insert(e_trig.end(), trig + (int64_t)e * 100, trig + (int64_t)e * 100 + 100);
            else
                e_trig.insert(e_trig.end(), 100, 0.f);
            e_hastrig.push_back(trig ? 1 : 0);
            const int64_t mlen = (int64_t)km * 25 * (e3d ? nr : 1);
            e_mofs.push_back((int64_t)e_mod.size());
            e_mod.insert(e_mod.end(), mod + mofs[e], mod + mofs[e] + mlen);
            const int npa = a == AX3D_ATT_CG4 ? 4 : 25;
            const int64_t alen = a ? 2LL * npa * (e3d ? nr : 1) : 0;
            if (a && (!aofs || !attm)) throw Error(AX3D_ERR_ARG, "ax3d_add_elements || attenuation moduli missing");
            e_aofs.push_back((int64_t)e_attm.size());
            if (alen) e_attm.insert(e_attm.end(), attm + aofs[e], attm + aofs[e] + alen);
        }
    }

    // ================================================================
    void finalize() {
        if (finalized) throw Error(AX3D_ERR_STATE, "ax3d_finalize || already finalized");
        CK(cudaSetDevice(device));
        CK(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
        for (int k = 0; k < NSIDE; k++) {
            CK(cudaStreamCreateWithFlags(&side[k], cudaStreamNonBlocking));
            CK(cudaEventCreateWithFlags(&ev_join[k], cudaEventDisableTiming));
        }
        CK(cudaEventCreateWithFlags(&ev_fork, cudaEventDisableTiming));
        ax3d::init_kernel_attributes();
        ax3d::set_g_matrices(g_gll, g_glj, stream);
        const int np = (int)p_nr.size(), ne = (int)e_nr.size();
        // point field offsets and row maps
        std::vector<int64_t> sofs(np, -1), fofs(np, -1);
        std::vector<int32_t> srow, frow;
        for (int p = 0; p < np; p++) {
            const int na = p_nr[p] / 2 + 1;
            if (p_kind[p] != AX3D_POINT_FLUID) {
                sofs[p] = nsolid;
                nsolid += (int64_t)na * 3;
                srow.insert(srow.end(), na, p);
            }
            if (p_kind[p] != AX3D_POINT_SOLID) {
                fofs[p] = nfluid;
                nfluid += na;
                frow.insert(frow.end(), na, p);
            }
        }
        // element force buffer, memory variables, gather lists, work items, buckets
        std::vector<int64_t> efofs(ne), memofs(ne);
        int64_t efsize = 0, memsize = 0;
        std::vector<std::vector<int64_t>> sref(np), fref(np);
        std::vector<int2> items_s, items_f;
        std::vector<int32_t> phys3_s, phys3_f;
        std::vector<int2> items_p1s, items_p1f, items_p3s, items_p3f;
        std::vector<int32_t> p3s, p3f;
        std::vector<int64_t> wofs(ne, 0);
        int64_t wsize = 0;
        e_prtlen.resize(ne, 0);
        e_prtofs.resize(ne, 0);
        int nr_max = 1;
        for (int e = 0; e < ne; e++) {
            const int nr = e_nr[e], n = nr / 2 + 1, flags = e_flags[e];
            nr_max = std::max(nr_max, nr);
            const bool fluid = flags & ax3d::EF_FLUID, e3d = flags & ax3d::EF_IN3D;
            const int nc = fluid ? 1 : 3;
            efofs[e] = efsize;
            for (int l = 0; l < 25; l++) {
                const int p = e_pts[(int64_t)e * 25 + l];
                (fluid ? fref : sref)[p].push_back(efsize + (int64_t)l * n * nc);
            }
            efsize += (int64_t)25 * n * nc;
            const int a = ax3d::ef_att(flags), npa = a == AX3D_ATT_CG4 ? 4 : 25;
            memofs[e] = memsize;
            if (a) memsize += (int64_t)(sls.nsls + 1) * 6 * npa * (e3d ? nr : 2 * n);
            if (e_prtlen[e] && e3d) {
                (fluid ? p3f : p3s).push_back(e);
                for (int al = 0; al < n; al++) (fluid ? items_p3f : items_p3s).push_back(make_int2(e, al));
                wofs[e] = wsize;
                wsize += (int64_t)n * (fluid ? 3 : 9) * 25;
            } else if (e_prtlen[e]) {
                for (int al = 0; al < n; al++) (fluid ? items_p1f : items_p1s).push_back(make_int2(e, al));
            } else if (e3d) {
                (fluid ? phys3_f : phys3_s).push_back(e);
            } else {
                for (int al = 0; al < n; al += ax3d::FW_OB) (fluid ? items_f : items_s).push_back(make_int2(e, al));
            }
        }
        // physical-space solid elements that own all their points (solid points of no other
        // element) subtract their forces straight into the point stiffness; the gather
        // skips those points
        std::vector<uint8_t> p_gskip(np, 0);
        for (int e = 0; e < ne; e++) {
            if ((e_flags[e] & ax3d::EF_FLUID) || !(e_flags[e] & ax3d::EF_IN3D) || e_prtlen[e]) continue;
            bool own = true;
            for (int l = 0; l < 25 && own; l++) {
                const int p = e_pts[(int64_t)e * 25 + l];
                own = p_kind[p] == AX3D_POINT_SOLID && sref[p].size() == 1;
            }
            if (!own) continue;
            e_flags[e] |= ax3d::EF_DIRECT;
            if (std::find(s_elem.begin(), s_elem.end(), e) != s_elem.end()) e_flags[e] |= ax3d::EF_SOURCE;
            const uint8_t g = (e_flags[e] & ax3d::EF_SOURCE) ? 1 : 2;
            for (int l = 0; l < 25; l++) p_gskip[e_pts[(int64_t)e * 25 + l]] = g;
        }
        int32_t sgather = 0;
        for (int p = 0; p < np; p++)
            if (p_kind[p] != AX3D_POINT_FLUID && !p_gskip[p]) sgather = 1;
        std::vector<int32_t> sg_ptr(np + 1, 0), fg_ptr(np + 1, 0);
        std::vector<int64_t> sg_ref, fg_ref;
        for (int p = 0; p < np; p++) {
            sg_ptr[p + 1] = sg_ptr[p] + (int32_t)sref[p].size();
            fg_ptr[p + 1] = fg_ptr[p] + (int32_t)fref[p].size();
            sg_ref.insert(sg_ref.end(), sref[p].begin(), sref[p].end());
            fg_ref.insert(fg_ref.end(), fref[p].begin(), fref[p].end());
        }
        // transform plans (FP64 tables) for every ring size of a 3D element, then
        // geometric buckets of the transform length so shared memory is sized per bucket
        std::vector<char> used(nr_max + 1, 0);
        for (int e = 0; e < ne; e++)
            if (e_flags[e] & ax3d::EF_IN3D) used[e_nr[e]] = 1;
        ax3d::FftTables ft = ax3d::build_fft_tables(used);
        phys3_s_list = phys3_s;
        phys3_f_list = phys3_f;
        lbuf_of_nr.assign(ft.plans.size(), 1);
        for (size_t k = 0; k < ft.plans.size(); k++) lbuf_of_nr[k] = ft.plans[k].Lbuf;
        for (int e : p3s) lbuf_p3s = std::max(lbuf_p3s, lbuf_of_nr[e_nr[e]]);
        for (int e : p3f) lbuf_p3f = std::max(lbuf_p3f, lbuf_of_nr[e_nr[e]]);
        if ((!p3s.empty() && ax3d::prt3_points_per_cta(true, lbuf_p3s) == 0) ||
            (!p3f.empty() && ax3d::prt3_points_per_cta(false, lbuf_p3f) == 0))
            throw Error(AX3D_ERR_ARG, "ax3d_set_prt || a PRT_3D element's ring is too long for one CTA's shared memory");
        // ocean load per point (GLLPoint.cpp:57-72 picks MassOcean1D / MassOcean3D)
        std::vector<int32_t> p_oclen(np, 0);
        std::vector<int64_t> p_ocofs(np, 0);
        {
            int64_t o = 0;
            for (size_t i = 0; i < oc_pt.size(); i++) {
                p_oclen[oc_pt[i]] = oc_len[i];
                p_ocofs[oc_pt[i]] = o;
                o += 4 * (int64_t)oc_len[i];
            }
        }
        // 3D points (Mass3D, MassOcean3D) and 3D couplings
        std::vector<int32_t> pts3d, sf3d;
        for (int p = 0; p < np; p++) {
            if ((p_mslen[p] > 1) || (p_mflen[p] > 1) || (p_oclen[p] > 1)) pts3d.push_back(p);
            if (p_sflen[p] > 1) sf3d.push_back(p);
            if (p_kind[p] == AX3D_POINT_SOLID_FLUID && p_sflen[p] == 1) n_sf1d++;
        }
        // sources
        for (size_t s = 0; s < s_elem.size(); s++)
            if (e_flags[s_elem[s]] & ax3d::EF_FLUID)
                throw Error(AX3D_ERR_ARG, "ax3d_add_source || source in a fluid element");

        cudaStream_t st = stream;
        d_pnr.upload(p_nr, st);
        d_pkind.upload(p_kind, st);
        d_paxial.upload(p_axial, st);
        d_pfsurf.upload(p_fsurf, st);
        d_sofs.upload(sofs, st);
        d_fofs.upload(fofs, st);
        d_mslen.upload(p_mslen, st);
        d_msofs.upload(p_msofs, st);
        d_ms.upload(p_ms.empty() ? std::vector<float>{0.f} : p_ms, st);
        d_oclen.upload(p_oclen, st);
        d_ocofs.upload(p_ocofs, st);
        d_oc.upload(oc_vals.empty() ? std::vector<float>{0.f} : oc_vals, st);
        d_mflen.upload(p_mflen, st);
        d_mfofs.upload(p_mfofs, st);
        d_mf.upload(p_mf.empty() ? std::vector<float>{0.f} : p_mf, st);
        d_sflen.upload(p_sflen, st);
        d_sfofs.upload(p_sfofs, st);
        d_sfn.upload(p_sfn.empty() ? std::vector<float>{0.f} : p_sfn, st);
        d_sfni.upload(p_sfni.empty() ? std::vector<float>{0.f} : p_sfni, st);
        d_sg_ptr.upload(sg_ptr, st);
        d_gskip.upload(p_gskip.empty() ? std::vector<uint8_t>{0} : p_gskip, st);
        d_fg_ptr.upload(fg_ptr, st);
        d_sg_ref.upload(sg_ref.empty() ? std::vector<int64_t>{0} : sg_ref, st);
        d_fg_ref.upload(fg_ref.empty() ? std::vector<int64_t>{0} : fg_ref, st);
        d_srow.upload(srow.empty() ? std::vector<int32_t>{0} : srow, st);
        d_frow.upload(frow.empty() ? std::vector<int32_t>{0} : frow, st);
        d_epts.upload(e_pts, st);
        d_eflags.upload(e_flags, st);
        d_enr.upload(e_nr, st);
        d_geo.upload(e_geo, st);
        d_trig.upload(e_trig, st);
        d_mofs.upload(e_mofs, st);
        d_mod.upload(e_mod.empty() ? std::vector<float>{0.f} : e_mod, st);
        d_aofs.upload(e_aofs, st);
        d_attm.upload(e_attm.empty() ? std::vector<float>{0.f} : e_attm, st);
        d_memofs.upload(memofs, st);
        d_mem.alloc(std::max<int64_t>(memsize, 1));
        d_mem.zero(st);
        d_efofs.upload(efofs, st);
        d_ef.alloc(std::max<int64_t>(efsize, 1));
        d_ef.zero(st);
        d_plans.upload(ft.plans, st);
        d_f2.upload(ft.f2, st);
        d_i32.upload(ft.i32, st);
        X.plans = d_plans.p;
        X.f2 = d_f2.p;
        X.i32 = d_i32.p;
        for (auto *b : {&d_su, &d_sv, &d_sa, &d_ss}) {
            b->alloc(std::max<int64_t>(nsolid, 1));
            b->zero(st);
        }
        for (auto *b : {&d_fu, &d_fv, &d_fa, &d_fs}) {
            b->alloc(std::max<int64_t>(nfluid, 1));
            b->zero(st);
        }
        if (kahan) {
            for (auto *b : {&d_sku, &d_skv}) { b->alloc(std::max<int64_t>(nsolid, 1)); b->zero(st); }
            for (auto *b : {&d_fku, &d_fkv}) { b->alloc(std::max<int64_t>(nfluid, 1)); b->zero(st); }
        }
        d_items_p1s.upload(items_p1s.empty() ? std::vector<int2>{make_int2(0, 0)} : items_p1s, st);
        d_items_p1f.upload(items_p1f.empty() ? std::vector<int2>{make_int2(0, 0)} : items_p1f, st);
        d_items_p3s.upload(items_p3s.empty() ? std::vector<int2>{make_int2(0, 0)} : items_p3s, st);
        d_items_p3f.upload(items_p3f.empty() ? std::vector<int2>{make_int2(0, 0)} : items_p3f, st);
        nitems_p1s = (int)items_p1s.size();
        nitems_p1f = (int)items_p1f.size();
        nitems_p3s = (int)items_p3s.size();
        nitems_p3f = (int)items_p3f.size();
        d_p3s.upload(p3s.empty() ? std::vector<int32_t>{0} : p3s, st);
        d_p3f.upload(p3f.empty() ? std::vector<int32_t>{0} : p3f, st);
        n_p3s = (int)p3s.size();
        n_p3f = (int)p3f.size();
        d_prtofs.upload(e_prtofs, st);
        d_prtx.upload(e_prtx.empty() ? std::vector<float>{0.f} : e_prtx, st);
        d_wofs.upload(wofs, st);
        d_w.alloc(std::max<int64_t>(wsize, 1));
        d_w.zero(st);
        d_items_s.upload(items_s, st);
        d_items_f.upload(items_f, st);
        nitems_s = (int)items_s.size();
        nitems_f = (int)items_f.size();
        CK(cudaDeviceGetAttribute(&num_sms, cudaDevAttrMultiProcessorCount, device));
        build_buckets(sched, st);
        n_pts3d = (int)pts3d.size();
        n_sf3d = (int)sf3d.size();
        d_pts3d.upload(pts3d.empty() ? std::vector<int32_t>{0} : pts3d, st);
        d_sf3d.upload(sf3d.empty() ? std::vector<int32_t>{0} : sf3d, st);
        // sources, stf, receivers
        d_selem.upload(s_elem.empty() ? std::vector<int32_t>{0} : s_elem, st);
        d_snord.upload(s_nord.empty() ? std::vector<int32_t>{0} : s_nord, st);
        d_sofs_src.upload(s_ofs.empty() ? std::vector<int64_t>{0} : s_ofs, st);
        {
            std::vector<float2> f(s_force.size() / 2);
            for (size_t i = 0; i < f.size(); i++) f[i] = make_float2(s_force[2 * i], s_force[2 * i + 1]);
            d_sforce.upload(f.empty() ? std::vector<float2>{make_float2(0.f, 0.f)} : f, st);
        }
        d_stf.upload(stf.empty() ? std::vector<float>{0.f} : stf, st);
        d_relem.upload(r_elem.empty() ? std::vector<int32_t>{0} : r_elem, st);
        d_rphi.upload(r_phi.empty() ? std::vector<float>{0.f} : r_phi, st);
        d_rw.upload(r_w.empty() ? std::vector<float>{0.f} : r_w, st);
        if (!sf_elem.empty()) {
            std::vector<int64_t> rofs(sf_elem.size());
            sf_row = 0;
            for (size_t i = 0; i < sf_elem.size(); i++) {
                rofs[i] = sf_row;
                sf_row += (int64_t)15 * (e_nr[sf_elem[i]] / 2 + 1);
            }
            d_sfe.upload(sf_elem, st);
            d_sfs.upload(sf_side, st);
            d_sfrofs.upload(rofs, st);
            sf_cap = std::max<int>(((int)stf.size() + sf_interval - 1) / sf_interval, 1);
            d_surf.alloc((size_t)sf_cap * sf_row);
            d_surf.zero(st);
        }
        seis_cap = std::max<int>((int)stf.size(), 1);
        d_seis.alloc((size_t)seis_cap * std::max<size_t>(r_elem.size(), 1) * 3);
        d_seis.zero(st);
        {
            std::vector<int32_t> list;
            n_strain = n_curl = 0;
            for (size_t r = 0; r < r_dump.size(); r++) {
                if (!r_dump[r]) continue;
                if (e_prtlen[r_elem[r]])
                    throw Error(AX3D_ERR_ARG, "ax3d_set_receiver_dumps || strain / curl receivers in relabelled "
                                              "elements are not supported");
                if (!e_hastrig[r_elem[r]])  // Receiver.cpp:49-51 forces the RTZ transform
                    throw Error(AX3D_ERR_ARG, "ax3d_set_receiver_dumps || strain / curl receivers need theta tables");
                list.push_back((int32_t)r);
                list.push_back((r_dump[r] & 1) ? n_strain++ : -1);
                list.push_back((r_dump[r] & 2) ? n_curl++ : -1);
            }
            n_sclist = (int)list.size() / 3;
            d_sclist.upload(list.empty() ? std::vector<int32_t>{0} : list, st);
            d_strain.alloc((size_t)seis_cap * std::max(n_strain, 1) * 6);
            d_strain.zero(st);
            d_curl.alloc((size_t)seis_cap * std::max(n_curl, 1) * 3);
            d_curl.zero(st);
        }
        d_flag.alloc(1);
        d_flag.zero(st);
        d_tstep.alloc(1);
        d_targ.alloc(1);
        reset_wisdom(st);
        tstep = 1;
        CK(cudaMemcpyAsync(d_tstep.p, &tstep, sizeof(int32_t), cudaMemcpyHostToDevice, st));

        P.n = np;
        P.nr = d_pnr.p;
        P.kind = d_pkind.p;
        P.axial = d_paxial.p;
        P.fsurf = d_pfsurf.p;
        P.sofs = d_sofs.p;
        P.fofs = d_fofs.p;
        P.mslen = d_mslen.p;
        P.msofs = d_msofs.p;
        P.ms = d_ms.p;
        P.oclen = d_oclen.p;
        P.ocofs = d_ocofs.p;
        P.oc = d_oc.p;
        P.mflen = d_mflen.p;
        P.mfofs = d_mfofs.p;
        P.mf = d_mf.p;
        P.sflen = d_sflen.p;
        P.sfofs = d_sfofs.p;
        P.sfn = d_sfn.p;
        P.sfni = d_sfni.p;
        P.sg_ptr = d_sg_ptr.p;
        P.gskip = d_gskip.p;
        P.sgather = sgather;
        P.sg_ref = d_sg_ref.p;
        P.fg_ptr = d_fg_ptr.p;
        P.fg_ref = d_fg_ref.p;
        P.nsrows = nsolid / 3;
        P.nfrows = nfluid;
        P.srow_pt = d_srow.p;
        P.frow_pt = d_frow.p;
        T.pts = d_epts.p;
        T.flags = d_eflags.p;
        T.nr = d_enr.p;
        T.geo = d_geo.p;
        T.trig = d_trig.p;
        T.mofs = d_mofs.p;
        T.moduli = d_mod.p;
        T.aofs = d_aofs.p;
        T.attm = d_attm.p;
        T.memofs = d_memofs.p;
        T.mem = d_mem.p;
        T.efofs = d_efofs.p;
        T.ef = d_ef.p;
        T.prtofs = d_prtofs.p;
        T.prtx = d_prtx.p;
        T.wofs = d_wofs.p;
        T.w = d_w.p;
        T.stiff = d_ss.p;
        F.su = d_su.p; F.sv = d_sv.p; F.sa = d_sa.p; F.ss = d_ss.p; F.sku = d_sku.p; F.skv = d_skv.p;
        F.fu = d_fu.p; F.fv = d_fv.p; F.fa = d_fa.p; F.fs = d_fs.p; F.fku = d_fku.p; F.fkv = d_fkv.p;
        CK(cudaStreamSynchronize(st));
        finalized = true;
        tstep = 1;
    }

    void need_final() const {
        if (!finalized) throw Error(AX3D_ERR_STATE, "ax3d || domain not finalized");
    }

    // ================= Domain loop bodies =================
    void update_newmark(bool in_step = false) {
        if (!in_step) guard_su();  // inside a step, apply_queued_input has waited already
        const double half_dt = 0.5 * dt, half_dt_dt = half_dt * dt;
        ax3d::launch_newmark(P, F, (float)dt, (float)half_dt, (float)half_dt_dt, kahan, d_pts3d.p, n_pts3d,
                             in_step, stream);
    }
    // explicit step index for the fine-grained entry points (the step loop reads d_tstep)
    void set_targ(int t) {
        h_targ = t;
        CK(cudaMemcpyAsync(d_targ.p, &h_targ, sizeof(int32_t), cudaMemcpyHostToDevice, stream));
    }
    void apply_source(int t) {
        if (s_elem.empty()) return;
        if (t < 0 || t >= (int)stf.size()) throw Error(AX3D_ERR_ARG, "ax3d_apply_source || step out of range");
        set_targ(t);
        ax3d::launch_source(P, T, F, d_selem.p, d_snord.p, d_sofs_src.p, d_sforce.p, (int)s_elem.size(),
                            d_stf.p, (int)stf.size(), d_targ.p, 0, stream);
    }
    // Physical-space buckets of a schedule: elements grouped by the geometric step of their
    // transform buffer length, each bucket with its own shared-memory size, points per CTA,
    // cluster size and persistent grid.
    void build_buckets(const Schedule &sc, cudaStream_t st) {
        std::map<int, std::vector<int32_t>> phys[2];  // keyed by bucket id
        for (int fl = 0; fl < 2; fl++)
            for (int e : fl ? phys3_f_list : phys3_s_list) {
                const int b = (int)std::floor(std::log((double)lbuf_of_nr[e_nr[e]]) / std::log(sc.ratio));
                phys[fl][b].push_back(e);
            }
        // size every bucket; with `merge`, buckets of one launch shape (CTAs per cluster,
        // threads per CTA) then become one persistent launch over their elements, longest
        // transforms first, its shared memory laid out for the longest and its points per CTA
        // the fewest of the merged buckets
        struct Sized {
            ax3d::PhysBucket b;
            std::vector<int32_t> elems;
        };
        std::vector<Sized> sized[2];
        for (int fl = 0; fl < 2; fl++)
            for (auto &kv : phys[fl]) {
                Sized z;
                z.b.count = (int)kv.second.size();
                for (int e : kv.second) {
                    z.b.L_max = std::max(z.b.L_max, lbuf_of_nr[e_nr[e]]);
                    z.b.n_max = std::max(z.b.n_max, e_nr[e] / 2 + 1);
                }
                ax3d::size_phys_bucket(z.b, !fl, sc.policy);
                if (z.b.npts_chunk <= 0)
                    throw Error(AX3D_ERR_UNSUPPORTED, "ax3d_finalize || nr too large for the physical-space kernel");
                z.elems = kv.second;
                // ring sizes together (the kernel keeps one ring's plan and tables loaded)
                std::stable_sort(z.elems.begin(), z.elems.end(),
                                 [&](int32_t a, int32_t b) { return e_nr[a] > e_nr[b]; });
                sized[fl].push_back(z);
            }
        if (sc.merge)
            for (int fl = 0; fl < 2; fl++) {
                std::map<std::pair<int, int>, Sized> byshape;
                for (auto &z : sized[fl]) {
                    auto key = std::make_pair(z.b.csize, z.b.nt);
                    auto it = byshape.find(key);
                    if (it == byshape.end()) {
                        byshape[key] = z;
                        continue;
                    }
                    Sized &m = it->second;
                    m.elems.insert(m.elems.end(), z.elems.begin(), z.elems.end());
                    m.b.count += z.b.count;
                    m.b.L_max = std::max(m.b.L_max, z.b.L_max);
                    m.b.n_max = std::max(m.b.n_max, z.b.n_max);
                    m.b.npts_chunk = std::min(m.b.npts_chunk, z.b.npts_chunk);
                    m.b.smem = std::max(m.b.smem, z.b.smem);
                }
                sized[fl].clear();
                for (auto &kv : byshape) {
                    Sized z = kv.second;
                    std::stable_sort(z.elems.begin(), z.elems.end(), [&](int32_t a, int32_t b) {
                        const int la = lbuf_of_nr[e_nr[a]], lb = lbuf_of_nr[e_nr[b]];
                        return la != lb ? la > lb : e_nr[a] > e_nr[b];
                    });
                    z.b.smem = ax3d::phys_smem_bytes(z.b.L_max, fl ? 2 : 3, z.b.npts_chunk, z.b.nt);
                    sized[fl].push_back(z);
                }
            }
        bucket_lists.clear();
        bucket_lists.resize(sized[0].size() + sized[1].size());
        buckets_s.clear();
        buckets_f.clear();
        size_t bi = 0;
        for (int fl = 0; fl < 2; fl++) {
            auto &dst = fl ? buckets_f : buckets_s;
            for (auto &z : sized[fl]) {
                z.b.grid = ax3d::phys_grid(z.b, !fl, num_sms);
                bucket_lists[bi].upload(z.elems, st);
                z.b.elems = bucket_lists[bi].p;
                bi++;
                dst.push_back(z.b);
            }
        }
        sched = sc;
    }
    // ---- autotuner: the bucket schedule from timed trials on this domain's own elements ----
    // Candidates: transform-length steps between buckets {1.06, 1.12, 1.25} x shared-memory
    // policy {two CTAs per SM; one CTA per SM; two per SM for small rings and one 512-thread
    // CTA per SM above; as the last with four 128-thread CTAs per SM for short rings, and
    // with eight 64-thread CTAs per SM for the shortest} x side streams {1, NSIDE}.  Each trial
    // times `trials` element passes (after one untimed pass) with CUDA events on the domain's
    // stream; the point stiffness and the memory variables the passes change are saved
    // before and put back after every trial.  The choice is cached per process under the
    // device name and the histogram of transform buffer lengths, so a second domain of the
    // same shape takes it without trials.
    static std::map<std::string, Schedule> &tune_cache() {
        static std::map<std::string, Schedule> c;
        return c;
    }
    std::string tune_key() const {
        cudaDeviceProp prop;
        CK(cudaGetDeviceProperties(&prop, device));
        std::map<int, int64_t> hist;
        for (int fl = 0; fl < 2; fl++)
            for (int e : fl ? phys3_f_list : phys3_s_list) hist[lbuf_of_nr[e_nr[e]] * 2 + fl]++;
        std::string k = prop.name;
        for (auto &kv : hist) k += " " + std::to_string(kv.first) + ":" + std::to_string(kv.second);
        return k;
    }
    std::string autotune(int trials) {
        need_final();
        if (phys3_s_list.empty() && phys3_f_list.empty()) return "no physical-space elements: nothing to tune";
        const std::string key = tune_key();
        auto hit = tune_cache().find(key);
        char buf[256];
        if (hit != tune_cache().end()) {
            build_buckets(hit->second, stream);
            drop_graph();
            snprintf(buf, sizeof buf, "cached: ratio %.2f, policy %d, side streams %d, merged %d", hit->second.ratio,
                     hit->second.policy, hit->second.nside, hit->second.merge);
            return buf;
        }
        trials = std::max(1, trials);
        // save what an element pass changes
        DevBuf<float2> save_ss, save_fs;
        DevBuf<float> save_mem;
        save_ss.alloc(std::max<int64_t>(nsolid, 1));
        save_fs.alloc(std::max<int64_t>(nfluid, 1));
        save_mem.alloc(std::max<int64_t>(d_mem.n, 1));
        auto copy = [&](void *dst, const void *src, size_t bytes) {
            if (bytes) CK(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToDevice, stream));
        };
        copy(save_ss.p, d_ss.p, (size_t)nsolid * sizeof(float2));
        copy(save_fs.p, d_fs.p, (size_t)nfluid * sizeof(float2));
        copy(save_mem.p, d_mem.p, (size_t)d_mem.n * sizeof(float));
        cudaEvent_t a = get_event(), b = get_event();
        const bool was_timers = timers;
        timers = false;
        const Schedule start = sched;
        Schedule best = start;
        float best_ms = 1e30f;
        std::string log;
        std::vector<Schedule> cands;
        for (double ratio : {1.06, 1.12, 1.25})
            for (int policy : {0, 1, 2})
                for (int nside : {1, (int)NSIDE}) cands.push_back(Schedule{ratio, policy, nside, 0});
        for (int policy : {0, 2, 3, 4})
            for (int nside : {1, (int)NSIDE}) cands.push_back(Schedule{1.12, policy, nside, 1});
        for (int nside : {1, (int)NSIDE}) cands.push_back(Schedule{1.12, 3, nside, 0});
        for (const Schedule &sc : cands) {
                {
                    build_buckets(sc, stream);
                    launch_elements(false);  // untimed: first launch of this shape
                    CK(cudaEventRecord(a, stream));
                    for (int t = 0; t < trials; t++) launch_elements(false);
                    CK(cudaEventRecord(b, stream));
                    CK(cudaEventSynchronize(b));
                    float ms = 0.f;
                    CK(cudaEventElapsedTime(&ms, a, b));
                    ms /= trials;
                    snprintf(buf, sizeof buf, " %.2f/%d/%d%s:%.2f", sc.ratio, sc.policy, sc.nside, sc.merge ? "m" : "", ms);
                    log += buf;
                    if (ms < best_ms) {
                        best_ms = ms;
                        best = sc;
                    }
                    copy(d_ss.p, save_ss.p, (size_t)nsolid * sizeof(float2));
                    copy(d_fs.p, save_fs.p, (size_t)nfluid * sizeof(float2));
                    copy(d_mem.p, save_mem.p, (size_t)d_mem.n * sizeof(float));
                }
        }
        build_buckets(best, stream);
        drop_graph();
        CK(cudaStreamSynchronize(stream));
        pool.push_back(a);
        pool.push_back(b);
        timers = was_timers;
        tune_cache()[key] = best;
        snprintf(buf, sizeof buf,
                 "chose ratio %.2f, policy %d, side streams %d, merged %d (%.2f ms per element pass); trials ms:",
                 best.ratio, best.policy, best.nside, best.merge, best_ms);
        return std::string(buf) + log;
    }
    // Element stiffness (Domain::computeStiff's element loop).  The physical-space buckets
    // go round-robin, longest transforms first, over side streams forked from and joined
    // back into the main stream, so one bucket's tail overlaps the next bucket's start;
    // a graph capture of the step records the same fork and join.
    void launch_elements(bool overwrite) {
        ax3d::launch_elem_fourier_solid(T, P, F.su, d_items_s.p, nitems_s, sls, stream);
        ax3d::launch_elem_fourier_fluid(T, P, F.fu, d_items_f.p, nitems_f, stream);
        ax3d::launch_elem_prt1(true, T, P, F.su, d_items_p1s.p, nitems_p1s, sls, stream);
        ax3d::launch_elem_prt1(false, T, P, F.fu, d_items_p1f.p, nitems_p1f, sls, stream);
        ax3d::launch_elem_prt3(true, T, P, F.su, d_items_p3s.p, nitems_p3s, d_p3s.p, n_p3s, lbuf_p3s, X, sls, stream);
        ax3d::launch_elem_prt3(false, T, P, F.fu, d_items_p3f.p, nitems_p3f, d_p3f.p, n_p3f, lbuf_p3f, X, sls, stream);
        const int nb = (int)(buckets_s.size() + buckets_f.size());
        if (nb == 0) return;
        if (nb == 1) {
            for (auto &b : buckets_s) ax3d::launch_elem_phys(true, T, P, F.su, b, X, sls, overwrite, stream);
            for (auto &b : buckets_f) ax3d::launch_elem_phys(false, T, P, F.fu, b, X, sls, overwrite, stream);
            return;
        }
        const int ns = std::max(1, std::min(sched.nside, NSIDE));
        CK(cudaEventRecord(ev_fork, stream));
        for (int k = 0; k < ns; k++) CK(cudaStreamWaitEvent(side[k], ev_fork, 0));
        int i = 0;
        for (auto it = buckets_s.rbegin(); it != buckets_s.rend(); ++it)
            ax3d::launch_elem_phys(true, T, P, F.su, *it, X, sls, overwrite, side[i++ % ns]);
        for (auto it = buckets_f.rbegin(); it != buckets_f.rend(); ++it)
            ax3d::launch_elem_phys(false, T, P, F.fu, *it, X, sls, overwrite, side[i++ % ns]);
        for (int k = 0; k < ns; k++) {
            CK(cudaEventRecord(ev_join[k], side[k]));
            CK(cudaStreamWaitEvent(stream, ev_join[k], 0));
        }
    }
    void compute_stiff() {
        launch_elements(false);
        ax3d::launch_gather(P, T, F, stream);
    }
    void couple() { ax3d::launch_couple(P, F, d_sf3d.p, n_sf3d, n_sf1d, stream); }
    void record(int t) {
        if (t < 0) throw Error(AX3D_ERR_ARG, "ax3d_record || negative step");
        if (r_elem.empty() && sf_elem.empty()) return;
        set_targ(t);
        if (!r_elem.empty()) {
            if (t >= seis_cap) grow_seis(t + 1);
            ax3d::launch_record(P, T, F.su, d_relem.p, d_rphi.p, d_rw.p, (int)r_elem.size(), d_seis.p, seis_cap,
                                d_targ.p, 0, stream);
            ax3d::launch_record_strain_curl(P, T, F.su, d_relem.p, d_rphi.p, d_rw.p, d_sclist.p, n_sclist,
                                            d_strain.p, n_strain, d_curl.p, n_curl, seis_cap, d_targ.p, 0, stream);
        }
        if (!sf_elem.empty()) {
            if (t / sf_interval >= sf_cap) grow_surf(t / sf_interval + 1);
            ax3d::launch_record_surface(P, T, F.su, d_sfe.p, d_sfs.p, d_sfrofs.p, (int)sf_elem.size(), d_surf.p, sf_row,
                                        sf_cap, d_targ.p, 0, sf_interval, stream);
        }
    }
    void grow_surf(int need) {
        const int cap = std::max(need, sf_cap * 2);
        DevBuf<float2> nb;
        nb.alloc((size_t)cap * sf_row);
        nb.zero(stream);
        CK(cudaMemcpyAsync(nb.p, d_surf.p, (size_t)sf_cap * sf_row * sizeof(float2), cudaMemcpyDeviceToDevice,
                           stream));
        CK(cudaStreamSynchronize(stream));
        std::swap(nb.p, d_surf.p);
        std::swap(nb.n, d_surf.n);
        sf_cap = cap;
        drop_graph();  // the captured step holds the old buffer address
    }
    void grow_seis(int need) {
        int cap = std::max(need, seis_cap * 2);
        DevBuf<float> nb;
        nb.alloc((size_t)cap * r_elem.size() * 3);
        nb.zero(stream);
        CK(cudaMemcpyAsync(nb.p, d_seis.p, (size_t)seis_cap * r_elem.size() * 3 * sizeof(float),
                           cudaMemcpyDeviceToDevice, stream));
        CK(cudaStreamSynchronize(stream));
        std::swap(nb.p, d_seis.p);
        std::swap(nb.n, d_seis.n);
        for (int which = 0; which < 2; which++) {
            DevBuf<float> &buf = which ? d_curl : d_strain;
            const size_t row = which ? (size_t)std::max(n_curl, 1) * 3 : (size_t)std::max(n_strain, 1) * 6;
            DevBuf<float> nc;
            nc.alloc((size_t)cap * row);
            nc.zero(stream);
            CK(cudaMemcpyAsync(nc.p, buf.p, (size_t)seis_cap * row * sizeof(float), cudaMemcpyDeviceToDevice,
                               stream));
            CK(cudaStreamSynchronize(stream));
            std::swap(nc.p, buf.p);
            std::swap(nc.n, buf.n);
        }
        seis_cap = cap;
        drop_graph();  // the captured step holds the old buffer address
    }
    // mMaxDisplWisdom = -1, mNuWisdom = Nu (SolidPoint.cpp:9-17, FluidPoint.cpp:9-17)
    void reset_wisdom(cudaStream_t st) {
        const int np = (int)p_nr.size();
        std::vector<float> mx((size_t)np * 4, -1.f);
        std::vector<int32_t> nu((size_t)np * 4);
        for (int p = 0; p < np; p++)
            for (int c = 0; c < 4; c++) nu[(size_t)p * 4 + c] = p_nr[p] / 2;
        d_wis_max.upload(mx.empty() ? std::vector<float>{0.f} : mx, st);
        d_wis_nu.upload(nu.empty() ? std::vector<int32_t>{0} : nu, st);
        drop_graph();
    }
    std::vector<int32_t> get_wisdom() {
        const int np = (int)p_nr.size();
        std::vector<int32_t> nu((size_t)np * 4);
        CK(cudaMemcpyAsync(nu.data(), d_wis_nu.p, nu.size() * sizeof(int32_t), cudaMemcpyDeviceToHost, stream));
        CK(cudaStreamSynchronize(stream));
        std::vector<int32_t> out(np, 0);
        for (int p = 0; p < np; p++) {
            int m = 0;
            if (p_kind[p] != AX3D_POINT_FLUID)
                m = std::max({nu[(size_t)p * 4], nu[(size_t)p * 4 + 1], nu[(size_t)p * 4 + 2]});
            if (p_kind[p] != AX3D_POINT_SOLID) m = std::max(m, nu[(size_t)p * 4 + 3]);
            out[p] = m;
        }
        return out;
    }
    void drop_graph() {
        for (auto &g : graph_execs) {
            if (g) cudaGraphExecDestroy(g);
            g = nullptr;
        }
    }
    // One time step of Newmark::solve with the step index read on the device (d_tstep),
    // so the same launches serve every step; used directly or captured as a CUDA graph.
    void enqueue_step() {
        const int nrow = (P.nsrows > 0) + (P.nfrows > 0);
        tbegin(AX3D_TIMER_POINTS);
        update_newmark(true);
        tend(nrow + (n_pts3d > 0));
        if (!s_elem.empty()) {
            tbegin(AX3D_TIMER_SOURCE);
            ax3d::launch_source(P, T, F, d_selem.p, d_snord.p, d_sofs_src.p, d_sforce.p, (int)s_elem.size(),
                                d_stf.p, (int)stf.size(), d_tstep.p, -1, stream);
            tend(1);
        }
        tbegin(AX3D_TIMER_ELEMENTS);
        launch_elements(true);  // the Newmark update above cleared the point stiffness
        tend(n_elem_launches());
        tbegin(AX3D_TIMER_ASSEMBLE);
        ax3d::launch_gather(P, T, F, stream);
        tend((P.nsrows > 0 && P.sgather) + (P.nfrows > 0));
        tbegin(AX3D_TIMER_COUPLE);
        couple();
        tend((P.nsrows > 0 && n_sf1d > 0) + (n_sf3d > 0));
        if (!r_elem.empty()) {
            tbegin(AX3D_TIMER_RECORD);
            ax3d::launch_record(P, T, F.su, d_relem.p, d_rphi.p, d_rw.p, (int)r_elem.size(), d_seis.p, seis_cap,
                                d_tstep.p, -1, stream);
            ax3d::launch_record_strain_curl(P, T, F.su, d_relem.p, d_rphi.p, d_rw.p, d_sclist.p, n_sclist,
                                            d_strain.p, n_strain, d_curl.p, n_curl, seis_cap, d_tstep.p, -1, stream);
            tend(1 + (n_sclist > 0));
        }
        if (!sf_elem.empty()) {
            tbegin(AX3D_TIMER_RECORD);
            ax3d::launch_record_surface(P, T, F.su, d_sfe.p, d_sfs.p, d_sfrofs.p, (int)sf_elem.size(), d_surf.p, sf_row,
                                        sf_cap, d_tstep.p, -1, sf_interval, stream);
            tend(1);
        }
        if (wis_interval > 0) {
            tbegin(AX3D_TIMER_OTHER);
            ax3d::launch_learn_wisdom(P, F, d_wis_max.p, d_wis_nu.p, wis_cutoff, d_tstep.p, wis_interval, stream);
            tend(1);
        }
        if (stab_interval > 0) {
            tbegin(AX3D_TIMER_OTHER);
            ax3d::launch_stability(F.su, nsolid, F.fu, nfluid, d_flag.p, d_tstep.p, stab_interval, stream);
            tend(1);
        }
        ax3d::launch_advance(d_tstep.p, stream);
    }
    int n_elem_launches() const {
        return (nitems_s > 0) + (nitems_f > 0) + (nitems_p1s > 0) + (nitems_p1f > 0) + 3 * (n_p3s > 0) +
               3 * (n_p3f > 0) + (int)buckets_s.size() + (int)buckets_f.size();
    }
    int step(int nsteps) {
        need_final();
        cudaEvent_t s0 = nullptr, s1 = nullptr;
        if (timers) {
            s0 = get_event();
            CK(cudaEventRecord(s0, stream));
        }
        if (!r_elem.empty() && tstep - 1 + nsteps > seis_cap) grow_seis(tstep - 1 + nsteps);
        if (!sf_elem.empty() && nsteps > 0 && (tstep - 2 + nsteps) / sf_interval >= sf_cap)
            grow_surf((tstep - 2 + nsteps) / sf_interval + 1);
        apply_queued_input();
        if (timers || !use_graphs) {
            // phase timers need events between the phases: plain launches
            for (int s = 0; s < nsteps; s++) enqueue_step();
        } else {
            cudaGraphExec_t &graph_exec = graph_execs[su_cur];
            if (!graph_exec) {
                cudaGraph_t g = nullptr;
                CK(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
                enqueue_step();
                CK(cudaStreamEndCapture(stream, &g));
                CK(cudaGraphInstantiate(&graph_exec, g, 0));
                CK(cudaGraphDestroy(g));
            }
            for (int s = 0; s < nsteps; s++) CK(cudaGraphLaunch(graph_exec, stream));
        }
        tstep += nsteps;
        if (timers) {
            s1 = get_event();
            CK(cudaEventRecord(s1, stream));
            marks.push_back({AX3D_TIMER_STEP, s0, s1});
        }
        CK(cudaGetLastError());
        int32_t flag = 0;
        CK(cudaMemcpyAsync(&flag, d_flag.p, sizeof(int32_t), cudaMemcpyDeviceToHost, stream));
        CK(cudaStreamSynchronize(stream));
        if (timers) collect_timers();
        if (flag) throw Error(AX3D_ERR_UNSTABLE, "Domain::checkStability || Simulation blew up.");
        return AX3D_OK;
    }

    float2 *field(int which, int phase) {
        if (phase == AX3D_PHASE_SOLID) {
            switch (which) {
                case AX3D_FIELD_DISPL: return F.su;
                case AX3D_FIELD_VELOC: return F.sv;
                case AX3D_FIELD_ACCEL: return F.sa;
                case AX3D_FIELD_STIFF: return F.ss;
            }
        } else if (phase == AX3D_PHASE_FLUID) {
            switch (which) {
                case AX3D_FIELD_DISPL: return F.fu;
                case AX3D_FIELD_VELOC: return F.fv;
                case AX3D_FIELD_ACCEL: return F.fa;
                case AX3D_FIELD_STIFF: return F.fs;
            }
        }
        throw Error(AX3D_ERR_ARG, "ax3d_get_field || bad field or phase");
    }
    int64_t fsize(int phase) const { return phase == AX3D_PHASE_SOLID ? nsolid : nfluid; }

    void reset() {
        need_final();
        sync_fields();
        queued.clear();
        su_cur = 0;
        F.su = d_su.p;
        if (d_su_alt.p) d_su_alt.zero(stream);
        for (auto *b : {&d_su, &d_sv, &d_sa, &d_ss, &d_fu, &d_fv, &d_fa, &d_fs, &d_ef}) b->zero(stream);
        if (kahan)
            for (auto *b : {&d_sku, &d_skv, &d_fku, &d_fkv}) b->zero(stream);
        d_mem.zero(stream);
        d_seis.zero(stream);
        d_strain.zero(stream);
        d_curl.zero(stream);
        if (!sf_elem.empty()) d_surf.zero(stream);
        d_flag.zero(stream);
        reset_wisdom(stream);
        tstep = 1;
        CK(cudaMemcpyAsync(d_tstep.p, &tstep, sizeof(int32_t), cudaMemcpyHostToDevice, stream));
        CK(cudaStreamSynchronize(stream));
    }
};

namespace ax3d {
void set_last_error(const std::string &msg) { g_err = msg; }
}  // namespace ax3d

// ================================================================ C ABI
namespace {
template <typename F>
int guard(F f) {
    try {
        f();
        return AX3D_OK;
    } catch (const Error &e) {
        g_err = e.what();
        return e.code;
    } catch (const std::bad_alloc &) {
        g_err = "ax3d || out of host memory";
        return AX3D_ERR_NOMEM;
    } catch (const std::exception &e) {
        g_err = e.what();
        return AX3D_ERR_ARG;
    }
}
}  // namespace

extern "C" {

int ax3d_create(const ax3d_config *cfg, ax3d_domain **out) {
    return guard([&] {
        if (!cfg || !out) throw Error(AX3D_ERR_ARG, "ax3d_create || null argument");
        if (cfg->npol != 4) throw Error(AX3D_ERR_UNSUPPORTED, "ax3d_create || only nPol = 4 is built");
        if (!(cfg->dt > 0.)) throw Error(AX3D_ERR_ARG, "ax3d_create || dt must be positive");
        if (!cfg->g_gll || !cfg->g_glj) throw Error(AX3D_ERR_ARG, "ax3d_create || G matrices missing");
        if (cfg->nsls < 0 || cfg->nsls > 8) throw Error(AX3D_ERR_ARG, "ax3d_create || nsls must be in [0, 8]");
        int ndev = 0;
        CK(cudaGetDeviceCount(&ndev));
        if (cfg->device < 0 || cfg->device >= ndev) throw Error(AX3D_ERR_ARG, "ax3d_create || bad device");
        auto *d = new ax3d_domain();
        d->device = cfg->device;
        d->dt = cfg->dt;
        for (int i = 0; i < 25; i++) {
            d->g_gll[i] = (float)cfg->g_gll[i];
            d->g_glj[i] = (float)cfg->g_glj[i];
        }
        d->sls.nsls = cfg->nsls;
        for (int i = 0; i < cfg->nsls; i++) {
            d->sls.a[i] = (float)cfg->att_alpha[i];
            d->sls.b[i] = (float)cfg->att_beta[i];
            d->sls.g[i] = (float)cfg->att_gamma[i];
        }
        d->sls.do_kappa = cfg->att_do_kappa != 0;
        d->kahan = cfg->kahan != 0;
        d->stab_interval = cfg->stability_interval;
        *out = d;
    });
}

int ax3d_add_points(ax3d_domain *d, int32_t n, const int32_t *nr, const int8_t *kind, const uint8_t *axial,
                    const uint8_t *fluid_surface, const int32_t *mass_solid_len, const float *mass_solid_inv,
                    const int32_t *mass_fluid_len, const float *mass_fluid_inv, const int32_t *sf_len,
                    const float *sf_normal, const float *sf_normal_invmf, int32_t *first) {
    return guard([&] {
        if (!d) throw Error(AX3D_ERR_ARG, "ax3d_add_points || null domain");
        int32_t f0 = (int32_t)d->p_nr.size();
        d->add_points(n, nr, kind, axial, fluid_surface, mass_solid_len, mass_solid_inv, mass_fluid_len,
                      mass_fluid_inv, sf_len, sf_normal, sf_normal_invmf);
        if (first) *first = f0;
    });
}

int ax3d_add_elements(ax3d_domain *d, int32_t n, const int32_t *points, const int8_t *material,
                      const uint8_t *axial, const uint8_t *in_3d, const float *geometry, const float *trig,
                      const int64_t *moduli_ofs, const float *moduli, const int8_t *att, const int64_t *att_ofs,
                      const float *att_moduli, int32_t *first) {
    return guard([&] {
        if (!d) throw Error(AX3D_ERR_ARG, "ax3d_add_elements || null domain");
        int32_t f0 = (int32_t)d->e_nr.size();
        d->add_elements(n, points, material, axial, in_3d, geometry, trig, moduli_ofs, moduli, att, att_ofs,
                        att_moduli);
        if (first) *first = f0;
    });
}

int ax3d_add_source(ax3d_domain *d, int32_t elem, int32_t norders, const float *force) {
    return guard([&] {
        if (!d || !force) throw Error(AX3D_ERR_ARG, "ax3d_add_source || null argument");
        if (d->finalized) throw Error(AX3D_ERR_STATE, "ax3d_add_source || domain already finalized");
        if (elem < 0 || elem >= (int)d->e_nr.size()) throw Error(AX3D_ERR_ARG, "ax3d_add_source || element out of range");
        if (norders < 1) throw Error(AX3D_ERR_ARG, "ax3d_add_source || norders must be >= 1");
        d->s_elem.push_back(elem);
        d->s_nord.push_back(norders);
        d->s_ofs.push_back((int64_t)d->s_force.size() / 2);
        d->s_force.insert(d->s_force.end(), force, force + (size_t)25 * norders * 3 * 2);
    });
}

int ax3d_set_stf(ax3d_domain *d, int32_t nsteps, const float *stf) {
    return guard([&] {
        if (!d || (nsteps > 0 && !stf) || nsteps < 0) throw Error(AX3D_ERR_ARG, "ax3d_set_stf || bad argument");
        if (d->finalized) throw Error(AX3D_ERR_STATE, "ax3d_set_stf || domain already finalized");
        d->stf.assign(stf, stf + nsteps);
    });
}

int ax3d_add_receivers(ax3d_domain *d, int32_t n, const int32_t *elem, const float *phi, const float *weights) {
    return guard([&] {
        if (!d || n < 0 || (n && (!elem || !phi || !weights))) throw Error(AX3D_ERR_ARG, "ax3d_add_receivers || bad argument");
        if (d->finalized) throw Error(AX3D_ERR_STATE, "ax3d_add_receivers || domain already finalized");
        for (int i = 0; i < n; i++) {
            if (elem[i] < 0 || elem[i] >= (int)d->e_nr.size())
                throw Error(AX3D_ERR_ARG, "ax3d_add_receivers || element out of range");
            if (d->e_flags[elem[i]] & ax3d::EF_FLUID)
                throw Error(AX3D_ERR_ARG, "ax3d_add_receivers || receiver in a fluid element");
        }
        d->r_elem.insert(d->r_elem.end(), elem, elem + n);
        d->r_phi.insert(d->r_phi.end(), phi, phi + n);
        d->r_w.insert(d->r_w.end(), weights, weights + (size_t)n * 25);
    });
}

int ax3d_add_surface(ax3d_domain *d, int32_t n, const int32_t *elem, const int32_t *side, int32_t interval) {
    return guard([&] {
        if (!d || n < 0 || (n && (!elem || !side)) || interval < 1)
            throw Error(AX3D_ERR_ARG, "ax3d_add_surface || bad argument");
        if (d->finalized) throw Error(AX3D_ERR_STATE, "ax3d_add_surface || domain already finalized");
        if (!d->sf_elem.empty() && interval != d->sf_interval)
            throw Error(AX3D_ERR_ARG, "ax3d_add_surface || one record interval per domain");
        for (int i = 0; i < n; i++) {
            if (elem[i] < 0 || elem[i] >= (int)d->e_nr.size())
                throw Error(AX3D_ERR_ARG, "ax3d_add_surface || element out of range");
            if (d->e_flags[elem[i]] & ax3d::EF_FLUID)
                throw Error(AX3D_ERR_ARG, "ax3d_add_surface || surface edge on a fluid element");
            if (side[i] < 0 || side[i] > 3) throw Error(AX3D_ERR_ARG, "ax3d_add_surface || side must be 0..3");
        }
        d->sf_interval = interval;
        d->sf_elem.insert(d->sf_elem.end(), elem, elem + n);
        d->sf_side.insert(d->sf_side.end(), side, side + n);
    });
}

int ax3d_add_ocean_load(ax3d_domain *d, int32_t n, const int32_t *point, const int32_t *len, const float *vals) {
    return guard([&] {
        if (!d || n < 0 || (n && (!point || !len || !vals)))
            throw Error(AX3D_ERR_ARG, "ax3d_add_ocean_load || bad argument");
        if (d->finalized) throw Error(AX3D_ERR_STATE, "ax3d_add_ocean_load || domain already finalized");
        std::vector<char> seen(d->p_nr.size(), 0);
        for (int32_t p : d->oc_pt) seen[p] = 1;
        int64_t o = 0;
        for (int i = 0; i < n; i++) {
            const int p = point[i];
            if (p < 0 || p >= (int)d->p_nr.size()) throw Error(AX3D_ERR_ARG, "ax3d_add_ocean_load || point out of range");
            if (d->p_kind[p] == AX3D_POINT_FLUID)
                throw Error(AX3D_ERR_ARG, "MassOcean3D::checkCompatibility || Fluid point with ocean load.");
            if (!(len[i] == 1 || len[i] == d->p_nr[p]))
                throw Error(AX3D_ERR_ARG, "MassOcean3D::checkCompatibility || Incompatible size.");
            if (seen[p]) throw Error(AX3D_ERR_ARG, "ax3d_add_ocean_load || point already has an ocean load");
            seen[p] = 1;
            o += 4 * (int64_t)len[i];
        }
        d->oc_pt.insert(d->oc_pt.end(), point, point + n);
        d->oc_len.insert(d->oc_len.end(), len, len + n);
        d->oc_vals.insert(d->oc_vals.end(), vals, vals + o);
    });
}

int ax3d_finalize(ax3d_domain *d) {
    return guard([&] {
        if (!d) throw Error(AX3D_ERR_ARG, "ax3d_finalize || null domain");
        d->finalize();
    });
}

int64_t ax3d_field_size(const ax3d_domain *d, int32_t phase) { return d ? d->fsize(phase) : -1; }

int ax3d_get_field(ax3d_domain *d, int32_t which, int32_t phase, float *out) {
    return guard([&] {
        if (!d || !out) throw Error(AX3D_ERR_ARG, "ax3d_get_field || null argument");
        d->need_final();
        float2 *src = d->field(which, phase);
        CK(cudaMemcpyAsync(out, src, d->fsize(phase) * sizeof(float2), cudaMemcpyDeviceToHost, d->stream));
        CK(cudaStreamSynchronize(d->stream));
    });
}

int ax3d_set_field(ax3d_domain *d, int32_t which, int32_t phase, const float *in) {
    return guard([&] {
        if (!d || !in) throw Error(AX3D_ERR_ARG, "ax3d_set_field || null argument");
        d->need_final();
        float2 *dst = d->field(which, phase);
        if (d->su_async(which, phase)) d->guard_su();
        CK(cudaMemcpyAsync(dst, in, d->fsize(phase) * sizeof(float2), cudaMemcpyHostToDevice, d->stream));
        CK(cudaStreamSynchronize(d->stream));
    });
}

int ax3d_set_field_async(ax3d_domain *d, int32_t which, int32_t phase, const float *in) {
    return guard([&] {
        if (!d || !in) throw Error(AX3D_ERR_ARG, "ax3d_set_field_async || null argument");
        d->set_field_async(which, phase, in);
    });
}

int ax3d_get_field_async(ax3d_domain *d, int32_t which, int32_t phase, float *out) {
    return guard([&] {
        if (!d || !out) throw Error(AX3D_ERR_ARG, "ax3d_get_field_async || null argument");
        d->get_field_async(which, phase, out);
    });
}

int ax3d_sync_fields(ax3d_domain *d) {
    return guard([&] {
        if (!d) throw Error(AX3D_ERR_ARG, "ax3d_sync_fields || null domain");
        d->sync_fields();
    });
}

#define AX3D_SIMPLE(name, body)                  \
    int name {                                   \
        return guard([&] {                       \
            if (!d) throw Error(AX3D_ERR_ARG, #name " || null domain"); \
            d->need_final();                     \
            body;                                \
            CK(cudaGetLastError());              \
            CK(cudaStreamSynchronize(d->stream)); \
        });                                      \
    }

AX3D_SIMPLE(ax3d_update_newmark(ax3d_domain *d), d->update_newmark())
AX3D_SIMPLE(ax3d_apply_source(ax3d_domain *d, int32_t tstep), d->apply_source(tstep))
AX3D_SIMPLE(ax3d_compute_stiff(ax3d_domain *d), d->compute_stiff())
AX3D_SIMPLE(ax3d_couple_solid_fluid(ax3d_domain *d), d->couple())
AX3D_SIMPLE(ax3d_record(ax3d_domain *d, int32_t tstep), d->record(tstep))

int ax3d_step(ax3d_domain *d, int32_t nsteps) {
    return guard([&] {
        if (!d || nsteps < 0) throw Error(AX3D_ERR_ARG, "ax3d_step || bad argument");
        d->step(nsteps);
    });
}

int ax3d_read_seismograms(ax3d_domain *d, int32_t first, int32_t nsteps, float *out) {
    return guard([&] {
        if (!d || !out || first < 0 || nsteps < 0) throw Error(AX3D_ERR_ARG, "ax3d_read_seismograms || bad argument");
        d->need_final();
        if (first + nsteps > d->seis_cap) throw Error(AX3D_ERR_ARG, "ax3d_read_seismograms || steps not recorded");
        const size_t row = d->r_elem.size() * 3;
        CK(cudaMemcpyAsync(out, d->d_seis.p + (size_t)first * row, (size_t)nsteps * row * sizeof(float),
                           cudaMemcpyDeviceToHost, d->stream));
        CK(cudaStreamSynchronize(d->stream));
    });
}

int ax3d_set_prt(ax3d_domain *d, int32_t n, const int32_t *elem, const int32_t *len, const float *x) {
    return guard([&] {
        if (!d || n < 0 || (n && (!elem || !len || !x))) throw Error(AX3D_ERR_ARG, "ax3d_set_prt || bad argument");
        if (d->finalized) throw Error(AX3D_ERR_STATE, "ax3d_set_prt || domain already finalized");
        const int ne = (int)d->e_nr.size();
        d->e_prtlen.resize(ne, 0);
        d->e_prtofs.resize(ne, 0);
        for (int i = 0; i < n; i++) {
            const int e = elem[i];
            if (e < 0 || e >= ne) throw Error(AX3D_ERR_ARG, "ax3d_set_prt || element out of range");
            const bool e3d = d->e_flags[e] & ax3d::EF_IN3D, fluid = d->e_flags[e] & ax3d::EF_FLUID;
            if (len[i] != (e3d ? d->e_nr[e] : 1))
                throw Error(AX3D_ERR_ARG, fluid ? "FluidElement::FluidElement || Particle Relabelling and Elasticity "
                                                  "are generated in different spaces."
                                                : "SolidElement::SolidElement || Particle Relabelling and Elasticity "
                                                  "are generated in different spaces.");
            if (!d->e_hastrig[e]) throw Error(AX3D_ERR_ARG, "ax3d_set_prt || relabelled elements need theta tables");
        }
        int64_t o = 0;
        for (int i = 0; i < n; i++) {
            const int e = elem[i];
            const int64_t sz = (int64_t)4 * len[i] * 25;
            d->e_prtlen[e] = len[i];
            d->e_prtofs[e] = (int64_t)d->e_prtx.size();
            d->e_prtx.insert(d->e_prtx.end(), x + o, x + o + sz);
            o += sz;
        }
    });
}

int ax3d_set_receiver_dumps(ax3d_domain *d, int32_t n, const int32_t *flags) {
    return guard([&] {
        if (!d || n < 0 || (n && !flags)) throw Error(AX3D_ERR_ARG, "ax3d_set_receiver_dumps || bad argument");
        if (d->finalized) throw Error(AX3D_ERR_STATE, "ax3d_set_receiver_dumps || domain already finalized");
        if (n != (int)d->r_elem.size())
            throw Error(AX3D_ERR_ARG, "ax3d_set_receiver_dumps || one flag per receiver added");
        for (int i = 0; i < n; i++)
            if (flags[i] < 0 || flags[i] > 3) throw Error(AX3D_ERR_ARG, "ax3d_set_receiver_dumps || flags must be 0..3");
        d->r_dump.assign(flags, flags + n);
    });
}

int ax3d_read_strain_curl(ax3d_domain *d, int32_t which, int32_t first, int32_t nsteps, float *out) {
    return guard([&] {
        if (!d || !out || first < 0 || nsteps < 0 || which < 0 || which > 1)
            throw Error(AX3D_ERR_ARG, "ax3d_read_strain_curl || bad argument");
        d->need_final();
        if (first + nsteps > d->seis_cap) throw Error(AX3D_ERR_ARG, "ax3d_read_strain_curl || steps not recorded");
        const size_t row = which ? (size_t)d->n_curl * 3 : (size_t)d->n_strain * 6;
        const float *src = which ? d->d_curl.p : d->d_strain.p;
        if (row == 0 || nsteps == 0) return;
        CK(cudaMemcpyAsync(out, src + (size_t)first * row, (size_t)nsteps * row * sizeof(float),
                           cudaMemcpyDeviceToHost, d->stream));
        CK(cudaStreamSynchronize(d->stream));
    });
}

int64_t ax3d_surface_record_size(const ax3d_domain *d) { return d && d->finalized ? d->sf_row : -1; }

int ax3d_read_surface(ax3d_domain *d, int32_t first, int32_t count, float *out) {
    return guard([&] {
        if (!d || !out || first < 0 || count < 0) throw Error(AX3D_ERR_ARG, "ax3d_read_surface || bad argument");
        d->need_final();
        if (d->sf_elem.empty()) throw Error(AX3D_ERR_STATE, "ax3d_read_surface || no surface recorder");
        if (first + count > d->sf_cap) throw Error(AX3D_ERR_ARG, "ax3d_read_surface || records not taken");
        CK(cudaMemcpyAsync(out, d->d_surf.p + (size_t)first * d->sf_row, (size_t)count * d->sf_row * sizeof(float2),
                           cudaMemcpyDeviceToHost, d->stream));
        CK(cudaStreamSynchronize(d->stream));
    });
}

int ax3d_reset(ax3d_domain *d) {
    return guard([&] {
        if (!d) throw Error(AX3D_ERR_ARG, "ax3d_reset || null domain");
        d->reset();
    });
}

int32_t ax3d_current_step(const ax3d_domain *d) { return d ? d->tstep : -1; }

int ax3d_set_wisdom_learning(ax3d_domain *d, int32_t interval, float cutoff) {
    return guard([&] {
        if (!d) throw Error(AX3D_ERR_ARG, "ax3d_set_wisdom_learning || null domain");
        if (interval > 0 && !(cutoff > 0.f)) throw Error(AX3D_ERR_ARG, "ax3d_set_wisdom_learning || cutoff must be > 0");
        d->wis_interval = interval > 0 ? interval : 0;
        d->wis_cutoff = cutoff;
        d->drop_graph();
    });
}

int ax3d_learn_wisdom(ax3d_domain *d, float cutoff) {
    return guard([&] {
        if (!d) throw Error(AX3D_ERR_ARG, "ax3d_learn_wisdom || null domain");
        d->need_final();
        if (!(cutoff > 0.f)) throw Error(AX3D_ERR_ARG, "ax3d_learn_wisdom || cutoff must be > 0");
        ax3d::launch_learn_wisdom(d->P, d->F, d->d_wis_max.p, d->d_wis_nu.p, cutoff, nullptr, 0, d->stream);
        CK(cudaGetLastError());
        CK(cudaStreamSynchronize(d->stream));
    });
}

int ax3d_get_wisdom(ax3d_domain *d, int32_t *nu_wisdom) {
    return guard([&] {
        if (!d || !nu_wisdom) throw Error(AX3D_ERR_ARG, "ax3d_get_wisdom || null argument");
        d->need_final();
        auto v = d->get_wisdom();
        std::copy(v.begin(), v.end(), nu_wisdom);
    });
}

int ax3d_enable_timers(ax3d_domain *d, int32_t enable) {
    return guard([&] {
        if (!d) throw Error(AX3D_ERR_ARG, "ax3d_enable_timers || null domain");
        d->timers = enable != 0;
    });
}

int ax3d_set_schedule(ax3d_domain *d, double ratio, int32_t policy, int32_t nside, int32_t merge) {
    return guard([&] {
        if (!d) throw Error(AX3D_ERR_ARG, "ax3d_set_schedule || null domain");
        if (!(ratio > 1.0 && ratio < 4.0) || policy < 0 || policy > 4 || nside < 1)
            throw Error(AX3D_ERR_ARG, "ax3d_set_schedule || ratio in (1, 4), policy 0..4, nside >= 1");
        d->need_final();
        CK(cudaSetDevice(d->device));
        ax3d_domain::Schedule sc;
        sc.ratio = ratio;
        sc.policy = policy;
        sc.nside = nside;
        sc.merge = merge != 0;
        d->build_buckets(sc, d->stream);
        d->drop_graph();
        CK(cudaStreamSynchronize(d->stream));
    });
}

int ax3d_autotune(ax3d_domain *d, int32_t trials, char *report, size_t len) {
    return guard([&] {
        if (!d) throw Error(AX3D_ERR_ARG, "ax3d_autotune || null domain");
        CK(cudaSetDevice(d->device));
        const std::string r = d->autotune(trials);
        if (report && len) {
            const size_t n = std::min(len - 1, r.size());
            std::memcpy(report, r.data(), n);
            report[n] = 0;
        }
    });
}

int ax3d_read_timers(ax3d_domain *d, double *ms, int64_t *launches) {
    return guard([&] {
        if (!d) throw Error(AX3D_ERR_ARG, "ax3d_read_timers || null domain");
        for (int i = 0; i < AX3D_NTIMERS; i++) {
            if (ms) ms[i] = d->t_ms[i];
            if (launches) launches[i] = d->t_launch[i];
            d->t_ms[i] = 0.;
            d->t_launch[i] = 0;
        }
    });
}

int ax3d_destroy(ax3d_domain *d) {
    delete d;
    return AX3D_OK;
}

size_t ax3d_last_error(char *buf, size_t len) {
    if (buf && len) {
        size_t n = std::min(len - 1, g_err.size());
        std::memcpy(buf, g_err.data(), n);
        buf[n] = 0;
    }
    return g_err.size();
}

}  // extern "C"
