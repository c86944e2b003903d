/*
 * ax3d.h -- C-ABI of the GB300 time-stepping path for AxiSEM3D (nPol = 4).
 *
 * The reference has no FFI for this path: it sits behind C++ virtual
 * interfaces that Mesh::release populates (SOLVER/src/core/domain/Domain.h:31-40,
 * SOLVER/src/core/element/Element.h:20, SOLVER/src/core/point/Point.h:17-51) and
 * is driven by Newmark::solve (SOLVER/src/core/newmark/Newmark.cpp:47-93).  Each
 * entry point below names the reference interface it replaces.  All calls take
 * plain host pointers and sizes; nothing here exposes CUDA or torch types.
 *
 * Data model (host FP32 unless stated; "complex" = two interleaved floats):
 *   point p      : nr_p azimuthal samples, Nu_p = nr_p / 2 Fourier orders stored
 *                  as (Nu_p + 1) complex values per component.  Solid fields are
 *                  laid out per point as [alpha][3] complex (s, phi, z); fluid
 *                  fields as [alpha] complex.  Points are concatenated in the
 *                  order they were added.
 *   element e    : 25 GLL points, row-major (ipol * 5 + jpol).  nr_e is the
 *                  maximum nr of its points (SOLVER/src/core/element/Element.cpp:13-18).
 *
 * Errors: every function returns AX3D_OK (0) or an AX3D_ERR_* code; the text
 * of the last error on the calling thread is returned by ax3d_last_error.
 * The reference throws std::runtime_error("Class::method || msg") and aborts
 * (SOLVER/src/axisem.cpp:193-204); here the same conditions return a code.
 */
#ifndef AX3D_H
#define AX3D_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define AX3D_NPOL 4
#define AX3D_NPE 25

enum {
    AX3D_OK = 0,
    AX3D_ERR_ARG = 1,        /* invalid argument or size */
    AX3D_ERR_STATE = 2,      /* call out of order (e.g. step before finalize) */
    AX3D_ERR_CUDA = 3,       /* CUDA runtime error */
    AX3D_ERR_UNSTABLE = 4,   /* non-finite displacement (Domain::checkStability) */
    AX3D_ERR_NOMEM = 5,
    AX3D_ERR_UNSUPPORTED = 6,
    AX3D_ERR_TIMEOUT = 7     /* a bounded device wait gave up */
};

/* point kinds (GLLPoint::release, SOLVER/src/preloop/mesh/GLLPoint.cpp:48-128) */
enum { AX3D_POINT_SOLID = 0, AX3D_POINT_FLUID = 1, AX3D_POINT_SOLID_FLUID = 2 };

/* element materials (Material::createElastic / createAcoustic,
   SOLVER/src/preloop/physics/material/Material.cpp:257-519) */
enum {
    AX3D_MAT_ISO = 0,      /* 2 moduli: lambda (=F), mu (=L)                       */
    AX3D_MAT_TISO = 1,     /* 5 moduli: A, C, F, L, N (Love)                        */
    AX3D_MAT_ANISO = 2,    /* 21 moduli: C11..C16, C22..C26, C33..C36, C44..C46, C55, C56, C66 */
    AX3D_MAT_ACOUSTIC = 3  /* 1 modulus: K = integral factor / rho (fluid element)  */
};

/* attenuation (AttBuilder::createAttenuation1D/3D,
   SOLVER/src/preloop/physics/attenuation/AttBuilder.cpp:17-129) */
enum { AX3D_ATT_NONE = 0, AX3D_ATT_FULL = 1, AX3D_ATT_CG4 = 2 };

/* which field for get/set */
enum { AX3D_FIELD_DISPL = 0, AX3D_FIELD_VELOC = 1, AX3D_FIELD_ACCEL = 2, AX3D_FIELD_STIFF = 3 };
enum { AX3D_PHASE_SOLID = 0, AX3D_PHASE_FLUID = 1 };

typedef struct ax3d_config {
    int32_t npol;                 /* must be 4 (SOLVER/src/global.h:26-33) */
    double dt;                    /* time step, cast to float in the update like Newmark */
    const double *g_gll;          /* [25] G(i,j) = l_i'(xi_j), GLL nodes, row-major     */
    const double *g_glj;          /* [25] the same on GLJ(0,1) nodes (axial xi)         */
    int32_t nsls;                 /* number of standard linear solids, 0 = elastic      */
    const double *att_alpha;      /* [nsls] SLS factors (AttAxiSEM::computeAttFactors)  */
    const double *att_beta;       /* [nsls]                                             */
    const double *att_gamma;      /* [nsls]                                             */
    int32_t att_do_kappa;         /* ATTENUATION_QKAPPA                                 */
    int32_t kahan;                /* 1: compensated sums in the Newmark update          */
    int32_t stability_interval;   /* steps between non-finite checks, <= 0: never       */
    int32_t device;               /* CUDA device ordinal (ignored by the CPU oracle)    */
} ax3d_config;

typedef struct ax3d_domain ax3d_domain;

/* Creates an empty domain.  Replaces `new Domain` + SpectralConstants/Gradient
   static set-up (SOLVER/src/axisem.cpp:40-60, Gradient::setGMat Gradient.cpp:324-329). */
int ax3d_create(const ax3d_config *cfg, ax3d_domain **out);

/* Bulk Domain::addPoint (Domain.h:31-40) of typed points as GLLPoint::release builds them
   (GLLPoint.cpp:48-128).  Per point: nr, kind (AX3D_POINT_*), axial, fluid_surface
   (fluid point on the free surface, FluidPoint.cpp:25-28).
   Inverse masses: mass_*_len[p] is 0 (no such phase), 1 (Mass1D) or nr (Mass3D); the
   values are concatenated in mass_*_inv.  Solid-fluid coupling (kind == SOLID_FLUID):
   sf_len[p] is 1 (SFCoupling1D) or nr (SFCoupling3D); sf_normal holds the unassembled
   normal [len][3] and sf_normal_invmf the assembled normal / fluid mass [len][3]
   (SFCoupling1D uses components 0 and 2 of row 0).  Returns the index of the first
   point in *first. */
int ax3d_add_points(ax3d_domain *d, int32_t n, const int32_t *nr, const int8_t *kind,
                    const uint8_t *axial, const uint8_t *fluid_surface,
                    const int32_t *mass_solid_len, const float *mass_solid_inv,
                    const int32_t *mass_fluid_len, const float *mass_fluid_inv,
                    const int32_t *sf_len, const float *sf_normal,
                    const float *sf_normal_invmf, int32_t *first);

/* Bulk Domain::addElement of SolidElement / FluidElement as Quad::release builds them
   (SOLVER/src/preloop/mesh/Quad.cpp:378-420).
   points   [n][25] point indices (ipol * 5 + jpol)
   material AX3D_MAT_*; in_3d = 1 for physical-space (3D) material, 0 for Fourier-space (1D)
   geometry [n][5][25]: dsdxii, dsdeta, dzdxii, dzdeta, inv_s (Quad::createGraident,
            Quad.cpp:509-525), cast from FP64
   trig     [n][4][25]: sin(theta), cos(theta), sin(2 theta), cos(2 theta) of the GLL
            points (CrdTransTIsoSolid.cpp:7-12); read for TISO and ANISO only; may be NULL
            when no element needs it
   moduli   concatenated, moduli_ofs[e] floats into it: 1D [k][25]; 3D [k][nr_e][25]
   att      AX3D_ATT_*; att_moduli concatenated, att_ofs[e] floats into it:
            1D FULL [2][25] (dkappa, dmu); 1D CG4 [2][4]; 3D FULL [2][nr_e][25];
            3D CG4 [2][nr_e][4].  CG4 points are (1,1), (1,3), (3,1), (3,3).
   Returns the index of the first element in *first. */
int ax3d_add_elements(ax3d_domain *d, int32_t n, const int32_t *points,
                      const int8_t *material, const uint8_t *axial, const uint8_t *in_3d,
                      const float *geometry, const float *trig,
                      const int64_t *moduli_ofs, const float *moduli,
                      const int8_t *att, const int64_t *att_ofs, const float *att_moduli,
                      int32_t *first);

/* Domain::addSourceTerm of a SourceTerm (SourceTerm.cpp:13-27): force [25][norders][3]
   complex, truncated per point to Nu_p + 1 orders like the SourceTerm constructor. */
int ax3d_add_source(ax3d_domain *d, int32_t elem, int32_t norders, const float *force);

/* Domain::setSTF (SourceTimeFunction.h:11-24): one factor per time step. */
int ax3d_set_stf(ax3d_domain *d, int32_t nsteps, const float *stf);

/* Receivers (PointwiseRecorder, SOLVER/src/core/output/pointwise/PointwiseRecorder.cpp:62-144):
   element index, azimuth phi and Lagrange weights [n][25] (Receiver::computeInterpFact).
   Each step records (s, phi, z) displacement via Element::computeGroundMotion. */
int ax3d_add_receivers(ax3d_domain *d, int32_t n, const int32_t *elem, const float *phi,
                       const float *weights);

/* Whole-surface recorder (SurfaceRecorder::addElement / record,
   SOLVER/src/core/output/surface/SurfaceRecorder.cpp:22-104): the Fourier displacement of
   the 5 GLL points on side side[i] (0: jpol = 0, 1: ipol = nPol, 2: jpol = nPol, 3: ipol = 0)
   of solid element elem[i], recorded when the step index is a multiple of interval.  One
   record holds, per edge in the order given, [component][point on the side][order] for
   orders 0..Nu_e (Nu_e = element nr / 2); orders a point does not hold are zero
   (SolidElement::feedDispOnSide, SolidElement.cpp:354-390).  Before ax3d_finalize. */
int ax3d_add_surface(ax3d_domain *d, int32_t n, const int32_t *elem, const int32_t *side, int32_t interval);

/* Ocean load on the solid part of n points (GLLPoint::release, GLLPoint.cpp:57-72), replacing
   the mass given to ax3d_add_points.  len[i] = 1: MassOcean1D (MassOcean1D.cpp), four values
   1/(m + m_ocean), 1/m, sin theta, cos theta (theta = colatitude of the point); len[i] = nr:
   MassOcean3D (MassOcean3D.cpp), nr rows of four values 1/m, and the unit surface normal
   (s, phi, z) scaled by sqrt(m_ocean / (m (m + m_ocean))).  Values back to back.  For a
   point with nr = 1 a length of 1 is the MassOcean1D form (one sample never varies).  Fluid
   points and other lengths are rejected with the reference's messages.  Before
   ax3d_finalize. */
int ax3d_add_ocean_load(ax3d_domain *d, int32_t n, const int32_t *point, const int32_t *len, const float *vals);

/* Ends set-up (Mesh::release + Domain::initializeRecorders): checks sizes, builds the
   gather lists and element buckets, uploads everything. */
int ax3d_finalize(ax3d_domain *d);

/* Number of complex values in the solid or fluid field arrays. */
int64_t ax3d_field_size(const ax3d_domain *d, int32_t phase);

/* Copy a whole field (all points, concatenated) to / from the host. */
int ax3d_get_field(ax3d_domain *d, int32_t which, int32_t phase, float *out);
int ax3d_set_field(ax3d_domain *d, int32_t which, int32_t phase, const float *in);

/* The Domain loop bodies, one call each (Domain.cpp:82-191), for fine-grained parity. */
int ax3d_update_newmark(ax3d_domain *d);                /* Domain::updateNewmark      */
int ax3d_apply_source(ax3d_domain *d, int32_t tstep);   /* Domain::applySource(tstep) */
int ax3d_compute_stiff(ax3d_domain *d);                 /* Domain::computeStiff       */
int ax3d_couple_solid_fluid(ax3d_domain *d);            /* Domain::coupleSolidFluid   */
int ax3d_record(ax3d_domain *d, int32_t tstep);         /* Domain::record(tstep, t)   */

/* nsteps iterations of Newmark::solve's loop body (Newmark.cpp:47-93) starting at the
   internal step counter: update, source, stiffness, solid-fluid coupling, record,
   stability check every stability_interval steps.  Returns AX3D_ERR_UNSTABLE if a
   non-finite displacement was found. */
int ax3d_step(ax3d_domain *d, int32_t nsteps);

/* Recorded (s, phi, z) displacement [nsteps][nrec][3] for steps first..first+nsteps-1. */
int ax3d_read_seismograms(ax3d_domain *d, int32_t first, int32_t nsteps, float *out);

/* Particle relabelling (PRT_1D / PRT_3D, core/element/prt; created by
   Relabelling::createPRT for Quad::releaseSolid / releaseFluid, Quad.cpp:386-420): for n
   elements, len[i] = 1 (1-D element: X [4][25]) or nr_e (3-D element: X [4][nr_e][25]),
   X back to back.  The element's strain goes through grad9 (fluid: the potential
   gradient), RTZ, the relabelling and back (SolidElement.cpp:404-443,
   FluidElement.cpp:333-355).  A length that does not match the element's space is
   rejected with the reference's message; theta tables are required.  Before ax3d_finalize. */
int ax3d_set_prt(ax3d_domain *d, int32_t n, const int32_t *elem, const int32_t *len, const float *x);

/* Pre-loop on the GPU (FP64): elastic moduli of n_elem elements at once, as
   Material::createElastic (Material.cpp:280-379) builds them, with the attenuation split
   of AttBuilder (AttBuilder.cpp:17-129, AttAxiSEM.cpp:14-57) and the CG4 weights of
   Quad::computeWeightsCG4 (Quad.cpp:438-466).  Stateless: runs on `device`, host buffers in
   and out.  rows[e] = 1 (1-D element) or nr_e (3-D); ifact [n_elem][25] (FP64); vpv, vph,
   vsv, vsh, eta, rho and, with attenuation, qkappa, qmu: [sum rows][25], element after
   element.  isotropic != 0 writes (lambda, mu) = (F, L), else (A, C, F, L, N): moduli
   [nmod][rows][25] per element, back to back, in the layout ax3d_add_elements takes; att =
   AX3D_ATT_FULL / AX3D_ATT_CG4 also writes att_moduli [2][rows][npa] per element (dkappa,
   dmu; npa = 25 or 4) from the SLS fit (w, y over nsls) and f_min, f_max, f_ref.  Errors:
   ax3d_precompute_last_error. */
int ax3d_precompute_elastic(int32_t device, int32_t n_elem, const int32_t *rows, const double *ifact,
                            const float *vpv, const float *vph, const float *vsv, const float *vsh,
                            const float *eta, const float *rho, const float *qkappa, const float *qmu,
                            int32_t isotropic, int32_t att, int32_t nsls, const double *w, const double *y,
                            double f_min, double f_max, double f_ref, int32_t do_kappa, float *moduli,
                            float *att_moduli);
/* Quad::createGraident + Quad::formIntegralFactor (Quad.cpp:509-547) for many elements on
   `device`, FP64: nodes [n][2][4] ((s0..s3), (z0..z3) of the corners in the reference's node
   order), etype [n] (0 spherical, 1 linear, 2 semi-spherical mapping), curved_outer [n]
   (0..3, the curved side; ignored for linear), axial [n]; spectral [20] = GLL nodes, GLL weights, GLJ(0,1) nodes,
   GLJ weights (SpectralConstants, nPol = 4).  Out: geometry [n][5][25] (dsdxii, dsdeta,
   dzdxii, dzdeta, inv_s), ifact [n][25], crds [n][25][2] (s, z of every GLL point). */
int ax3d_precompute_geometry(int32_t device, int32_t n_elem, const double *nodes, const int8_t *etype,
                             const int8_t *curved_outer, const uint8_t *axial, const double *spectral,
                             double *geometry, double *ifact, double *crds);
/* Material::computeElementalMass (Material.cpp:233-255) without relabelling for many
   elements on `device`, FP64: rows [n] (1 or nr), ifact [n][25], rho and (fluid elements) vp
   as [rows][25] per element back to back, fluid [n].  Out: mass [rows][25] per element,
   rho iFact for solids and iFact / (rho vp^2) for fluids. */
int ax3d_precompute_mass(int32_t device, int32_t n_elem, const int32_t *rows, const double *ifact,
                         const float *rho, const float *vp, const uint8_t *fluid, double *mass);
/* 3-D model sampling of the project's Gaussian-random volumetric model (no counterpart in
   the reference, whose tomography models are data tables; the step is
   Material::addVolumetric3D, Material.cpp:96-231) on `device`, FP64: for every element (rows
   [n] slices, GLL coordinates crds [n][25][2] = (s, z)) and slice phi_k = 2 pi k / rows (or
   phi2d for every slice when use_phi2d), the value rms sqrt(2 / modes) sum_j cos(kr_j r +
   klR_j . n + phase_j) with x = (s cos phi, s sin phi, z), r = |x|, n = x / r; klR is
   [3][modes].  out: [rows][25] per element back to back. */
int ax3d_sample_gaussian_random(int32_t device, int32_t n_elem, const int32_t *rows, const double *crds,
                                int32_t modes, const double *kr, const double *klR, const double *phase,
                                double rms, int32_t use_phi2d, double phi2d, double *out);
size_t ax3d_precompute_last_error(char *buf, size_t n);

/* Strain and curl at receivers (PointwiseRecorder::record, PointwiseRecorder.cpp:96-130;
   SolidElement::computeStrain / computeCurl, SolidElement.cpp:219-345): flags[i] for each
   receiver added so far, bit 0 dump_strain, bit 1 dump_curl (the STATIONS keywords,
   ReceiverCollection.cpp:58-72).  Before ax3d_finalize. */
int ax3d_set_receiver_dumps(ax3d_domain *d, int32_t n, const int32_t *flags);

/* Strain (which = 0: six RTZ components per flagged receiver) or curl (which = 1: three)
   of steps first..first+nsteps-1, recorded with the seismograms; [step][receiver][k] in
   the order of the flagged receivers. */
int ax3d_read_strain_curl(ax3d_domain *d, int32_t which, int32_t first, int32_t nsteps, float *out);

/* Asynchronous field transfers for callers that stream one state per step (inputs in,
   results out) without serialising the copies with the steps.  Host buffers should be
   pinned and must stay untouched until ax3d_sync_fields.
   ax3d_set_field_async: copies `in` into one of two device staging slots on a copy stream;
   each ax3d_step call first replaces the field with the oldest queued input (at most two
   queued; a third is rejected).  ax3d_get_field_async: snapshots the field on the step
   stream (after every step enqueued before it) and copies the snapshot to `out` on a second
   copy stream while later steps run.  ax3d_sync_fields waits for every queued copy. */
int ax3d_set_field_async(ax3d_domain *d, int32_t which, int32_t phase, const float *in);
int ax3d_get_field_async(ax3d_domain *d, int32_t which, int32_t phase, float *out);
int ax3d_sync_fields(ax3d_domain *d);

/* Complex values in one whole-surface record: sum over edges of 15 (Nu_e + 1). */
int64_t ax3d_surface_record_size(const ax3d_domain *d);

/* Whole-surface records first..first+count-1 (record r = step index r * interval), complex
   interleaved: count x ax3d_surface_record_size values. */
int ax3d_read_surface(ax3d_domain *d, int32_t first, int32_t count, float *out);

/* Zero every field and memory variable (Domain::resetZero, Domain.cpp:67-74); the
   internal step counter restarts at 1. */
int ax3d_reset(ax3d_domain *d);

/* Current internal step counter (next step to run, 1-based like Newmark::solve). */
int32_t ax3d_current_step(const ax3d_domain *d);

/* Nu wisdom (Domain::learnWisdom, Domain.cpp:384-402; SolidPoint::learnWisdom,
   SolidPoint.cpp:240-272; FluidPoint::learnWisdom, FluidPoint.cpp:209-229).
   ax3d_set_wisdom_learning: during ax3d_step, learn every `interval` steps (at step index
   tstep - 1 divisible by interval, as Newmark.cpp:89) with tail-energy cutoff `cutoff`;
   interval <= 0 switches learning off.  ax3d_learn_wisdom runs one learning pass now.
   ax3d_get_wisdom writes, per point, the smallest Fourier order holding the tail energy
   below cutoff^2 of the largest Hilbert norm seen so far (max over components and over
   the solid and fluid parts, SolidPoint::getNuWisdom). */
int ax3d_set_wisdom_learning(ax3d_domain *d, int32_t interval, float cutoff);
int ax3d_learn_wisdom(ax3d_domain *d, float cutoff);
int ax3d_get_wisdom(ax3d_domain *d, int32_t *nu_wisdom);

/* Time-loop phase timers: the reference's _MEASURE_TIMELOOP timers (Domain.h:111-118,
   reported by Domain::reportCost, Domain.cpp:349-382).  When enabled, ax3d_step brackets
   every phase with CUDA events on the domain's stream.  ax3d_read_timers fills
   ms[AX3D_NTIMERS] (accumulated device milliseconds) and launches[AX3D_NTIMERS]
   (kernel launches) indexed by AX3D_TIMER_*, and resets the accumulators. */
enum {
    AX3D_TIMER_STEP = 0,      /* whole ax3d_step calls             */
    AX3D_TIMER_ELEMENTS = 1,  /* Domain::computeStiff element loop */
    AX3D_TIMER_POINTS = 2,    /* Domain::updateNewmark             */
    AX3D_TIMER_ASSEMBLE = 3,  /* gatherStiffFromElement            */
    AX3D_TIMER_COUPLE = 4,    /* Domain::coupleSolidFluid          */
    AX3D_TIMER_SOURCE = 5,    /* Domain::applySource               */
    AX3D_TIMER_RECORD = 6,    /* Domain::record                    */
    AX3D_TIMER_OTHER = 7,     /* stability checks                  */
    AX3D_NTIMERS = 8
};
int ax3d_enable_timers(ax3d_domain *d, int32_t enable);
/* No counterpart in the reference, whose element cost table (Domain.cpp:349-382) weights
   the METIS partition instead (Mesh.cpp:412-588).  After ax3d_finalize: chooses the
   schedule of the physical-space element buckets -- the step of transform length between
   buckets, the shared-memory policy (see ax3d_set_schedule), the side streams and whether
   buckets of one launch shape merge into one launch -- from timed element passes on this domain's own
   elements (`trials` timed passes per candidate; the fields are left as they were), then
   recaptures the step.  The choice is cached for the process under the device name and the
   domain's histogram of transform lengths; a later domain of the same shape takes it
   without trials.  `report` (len bytes, may be NULL) receives the choice and the times. */
int ax3d_autotune(ax3d_domain *d, int32_t trials, char *report, size_t len);
/* No counterpart in the reference.  After ax3d_finalize: sets the bucket schedule by hand --
   ratio (> 1) between the transform lengths of neighbouring buckets, shared-memory policy
   (0: 256-thread CTAs, two per SM where they fit; 1: 256-thread CTAs with an SM's whole
   shared memory; 2: as 0 for rings that fit two per SM, 512-thread CTAs with an SM's whole
   shared memory above; 3: as 2, with 128-thread CTAs four per SM for the rings that fit a
   quarter of an SM's shared memory; 4: as 3, with 64-thread CTAs eight per SM for the rings
   that fit an eighth), side streams (1..3) and merge (nonzero: the buckets of one launch
   shape -- CTAs per cluster, threads per CTA -- run as one persistent launch over their
   elements, longest transforms first) -- and recaptures the step. */
int ax3d_set_schedule(ax3d_domain *d, double ratio, int32_t policy, int32_t nside, int32_t merge);
int ax3d_read_timers(ax3d_domain *d, double *ms, int64_t *launches);

int ax3d_destroy(ax3d_domain *d);

/* Size of the static device scratch of ax3d_compute_stiff_iso1d_noalloc, in MiB. */
#define AX3D_NOALLOC_SCRATCH_MIB 32

/* No counterpart in the reference.  Element stiffness plus assembly, stiff -= K u, for
   callers that cannot allocate device memory (a code that hands out every device byte
   from its own pre-sized pool, or one that must not allocate once a run has started):
   nothing is allocated, every pointer below is the caller's device buffer, and the element
   forces between the element pass and the assembly pass live in one static __device__
   array of AX3D_NOALLOC_SCRATCH_MIB MiB that every GPU loading the library holds until
   the process exits.
   Scope: Fourier-space isotropic solid elements without attenuation, all points with the
   same nu (nr = 2 nu + 1); layouts as the domain path:
     d_points    [nelem][25] point indices      d_axial     [nelem] 1 for axial elements
     d_geometry  [nelem][5][25] (ax3d_add_elements)  d_lambda_mu [nelem][2][25]
     d_gather_ptr[npoints + 1], d_gather_ref: CSR of (element * 25 + local point) per point,
                 ascending element order (the order the reference's element loop sums in)
     d_displ, d_stiff [npoints][nu + 1][3] complex
     g_gll, g_glj host [25] G matrices (as ax3d_config).
   d_displ and d_stiff must be 8-byte aligned (AX3D_ERR_ARG otherwise).
   Runs asynchronously on `stream` (a cudaStream_t, NULL = default stream).  Returns
   AX3D_ERR_ARG without launching when nelem * 25 * (nu + 1) * 24 bytes exceeds the
   scratch.  Set-up: the first call on a device, with that device current, loads the
   scratch array and the two kernels onto it (even under lazy module loading) and looks up
   the scratch's device address (cudaGetSymbolAddress) and the SM count; a call with
   nelem = 0 does only this.  Make one such call per device at start-up, before the
   caller's pool takes the device memory and before any stream capture; later calls then
   allocate nothing.  All calls share the one scratch: calls that overlap on the GPU (two
   streams, two threads) race and must be serialised by the caller.  The scratch keeps the
   last call's contents; every entry a call reads is written by the same call first. */
int ax3d_compute_stiff_iso1d_noalloc(int32_t nelem, int32_t nu, const int32_t *d_points,
                                     const uint8_t *d_axial, const float *d_geometry,
                                     const float *d_lambda_mu, int32_t npoints,
                                     const int32_t *d_gather_ptr, const int32_t *d_gather_ref,
                                     const float *d_displ, float *d_stiff, const double *g_gll,
                                     const double *g_glj, void *stream);

/* ---- Learned Fourier order: the Nu network ------------------------------------------
   No counterpart in the reference, whose Fourier-order field comes from NU_TYPE rules or
   from a wisdom file of an earlier run (NuWisdom.cpp:19-86, Domain.cpp:384-440).  A fixed
   multilayer perceptron maps AX3D_MLP_NIN per-element features to one value:
     h1 = gelu(W1 x + b1), h2 = gelu(W2 h1 + b2), h3 = gelu(W3 h2 + b3), y = w4 . h3 + b4
   with AX3D_MLP_NHID hidden units and gelu(z) = z Phi(z) (erf form).  Precision: weights,
   the features and the hidden activations are BF16 (round to nearest even), products are
   accumulated in FP32, biases and y are FP32; parameters are kept as an FP32 master copy
   that Adam (beta1 0.9, beta2 0.999, eps 1e-8) updates.  Loss: mean squared error over
   the n samples of a call.  Gradients are summed in a fixed order (per 64-sample tile,
   then over tiles), so repeated calls give identical bits.
   Parameter vector (FP32, AX3D_MLP_NPARAM values): W1 [128][16], b1 [128], W2 [128][128],
   b2 [128], W3 [128][128], b3 [128], w4 [128], b4 [1]  (W[j][k]: output j, input k).
   Device pointers are the caller's (for example torch tensors); calls run asynchronously
   on `stream` (a cudaStream_t, NULL = default stream). */
#define AX3D_MLP_NIN 16
#define AX3D_MLP_NHID 128
#define AX3D_MLP_NPARAM 35329
typedef struct ax3d_mlp ax3d_mlp;
/* max_batch: the largest n of a gradient / training call (inference takes any n). */
int ax3d_mlp_create(int32_t max_batch, int32_t device, ax3d_mlp **out);
/* Copies AX3D_MLP_NPARAM host values in (and resets Adam's moments and step count). */
int ax3d_mlp_set_params(ax3d_mlp *m, const float *params, int64_t n);
int ax3d_mlp_get_params(ax3d_mlp *m, float *params, int64_t n);
/* d_x [n][16] FP32 features -> d_y [n] FP32. */
int ax3d_mlp_forward(ax3d_mlp *m, const float *d_x, int32_t n, float *d_y, void *stream);
/* Gradient of the loss w.r.t. the parameters into d_grad [AX3D_MLP_NPARAM] (FP32) and
   the loss into d_loss [1]; no update.  d_t [n] targets. */
int ax3d_mlp_gradient(ax3d_mlp *m, const float *d_x, const float *d_t, int32_t n, float *d_grad,
                      float *d_loss, void *stream);
/* One Adam step on the mini-batch (d_x, d_t) with learning rate lr; the batch loss
   (before the update) goes to d_loss [1] when d_loss is not NULL. */
int ax3d_mlp_train_step(ax3d_mlp *m, const float *d_x, const float *d_t, int32_t n, float lr,
                        float *d_loss, void *stream);
int ax3d_mlp_destroy(ax3d_mlp *m);

/* Text of the last error on this thread (always NUL terminated); returns its length. */
size_t ax3d_last_error(char *buf, size_t len);

#ifdef __cplusplus
}
#endif

#endif /* AX3D_H */
